"""bench.py's reference arm (the oracle on the host cores) keeps the JSON contract
on every workload, at small sizes, without a GPU."""
import json
import subprocess
import sys

import pytest

from conftest import ROOT

ARGS = {
    "segments": ["--n", "20000", "--ref-sample", "20"],
    "plate": ["--n", "100000", "--ref-sample", "20"],
    "ompl": ["--n", "20000", "--ref-sample", "40"],
    "disentangled": ["--n", "100000", "--ref-sample", "20"],
    "contacts": ["--n", "64", "--ref-sample", "32"],
    "keyconf": ["--n", "256", "--ref-sample", "32"],
    "touch": ["--n", "64", "--ref-sample", "16"],
    "visibility": ["--n", "64", "--ref-sample", "160"],
}


def _run(workload, extra):
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", workload, "--steps", "2",
                        "--warmup", "1"] + extra, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


@pytest.mark.parametrize("workload", sorted(ARGS))
def test_reference_arm_line(workload):
    line = _run(workload, ARGS[workload])
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["steps"] == 2 and line["warmup"] == 1 and line["config"]["workload"]
    cpu = line["cpu_baseline"]
    assert cpu["value"] == line["value"] and cpu["unit"] == line["unit"] and cpu["kind"] == "port"
    assert cpu["cores"] >= 1 and cpu["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_narrow_reference_arm_is_unavailable():
    line = _run("narrow", [])
    assert line["impl"] == "reference" and "unavailable" in line
