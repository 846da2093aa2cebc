"""The kernels' shortcut for runs of the reference's delta updates
(pwm::walk_delta / delta_try / delta_jump; unit_world.cc:463-470 is one update per step)
against the updates taken one at a time, bit for bit, on random and
adversarial step sizes: rounding ties inside a binade, dist on and next to
powers of two, dist an exact multiple of the step; and the filter frames'
slerp weights (a reciprocal instead of a division) within their stated error
of the reference's interpolation (CPU)."""
import os
import subprocess

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("dw") / "delta_walk")
    src = os.path.join(ROOT, "tests", "harness", "delta_walk.cc")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "puzzletunneldiscovery_gb300", "csrc"), src, "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_walk_delta_equals_single_updates(harness, seed):
    r = subprocess.run([harness, "20000", str(seed)], capture_output=True, text=True)
    f = r.stdout.split()
    fields = dict(zip(f[0::2], map(int, f[1::2])))
    assert r.returncode == 0 and fields["mismatches"] == 0, r.stdout
    assert fields["jumped"] > fields["walks"] // 2       # the shortcuts are taken
    assert fields["tried"] > fields["walks"] // 2
    assert fields["ties"] > 1000                         # and the tie fallback is exercised
    assert fields["interpolations"] > 100_000            # the filter frames' slerp weights were compared
