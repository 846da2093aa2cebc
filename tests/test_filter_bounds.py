"""The FP32 filter's certified verdicts against the FP64 triangle test (CPU).

tests/harness/filter_bounds.cu drives pwf::tri_filter, pwf::sat_sep32 and
pwf::sat_sep32_obb (the code the kernels run) on millions of near-contact
triangle pairs; a certified verdict that differs from the FP64 Moeller test, or
a box test that separates touching triangles, is a failure.  The oriented boxes
are fitted as the BVH build fits them (pwm::jacobi_eigen3); besides the
triangles' own boxes, thick boxes are checked against the exact FP64 boxes, and
pairs moved (by bisection) to just inside their exact contact must never be
certified apart.  Built host-only with g++.
"""
import os
import subprocess

import pytest

from conftest import ROOT


def _cuda_include():
    for p in ("/usr/local/cuda/include", "/usr/local/cuda/targets/x86_64-linux/include",
              "/usr/local/cuda/targets/sbsa-linux/include"):
        if os.path.exists(os.path.join(p, "cuda_runtime.h")):
            return p
    pytest.skip("CUDA headers not found")


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("fb") / "filter_bounds")
    src = os.path.join(ROOT, "tests", "harness", "filter_bounds.cu")
    cmd = ["g++", "-O2", "-std=c++17", "-x", "c++", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "puzzletunneldiscovery_gb300", "csrc"), "-I", _cuda_include(), src, "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_certified_verdicts_match_fp64(harness, seed):
    r = subprocess.run([harness, "1500000", str(seed)], capture_output=True, text=True)
    fields = {}
    for line in r.stdout.strip().splitlines()[-3:]:
        fields.update(dict(zip(line.split()[0::2], map(int, line.split()[1::2]))))
    assert r.returncode == 0, r.stdout
    assert fields["filter_violations"] == 0 and fields["box_violations"] == 0
    assert fields["certified_hits"] > 100_000       # the filter does certify contacts
    assert fields["oriented_violations"] == 0
    assert fields["oriented_separations"] > 100_000 and fields["touching_cases"] > 500_000
