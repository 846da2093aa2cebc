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


@pytest.fixture(scope="module")
def dis_harness(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("db") / "disentangled_bounds")
    src = os.path.join(ROOT, "tests", "harness", "disentangled_bounds.cc")
    cmd = ["g++", "-O2", "-std=c++17", "-x", "c++", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "puzzletunneldiscovery_gb300", "csrc"), "-I", _cuda_include(), src, "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


@pytest.mark.parametrize("seed", [1, 2])
def test_disentangled_fp32_verdicts_match_fp64(dis_harness, seed):
    """pwf::boxes_disjoint32 (isDisentangled in FP32, unit_world.cc:249-264) never
    certifies a verdict that differs from the FP64 test, on states bisected to
    within 1e-17 of the boxes' contact and at growing distances from it."""
    r = subprocess.run([dis_harness, "200000", str(seed), "1"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    f = r.stdout.split()
    wrong, cert, und, states, far_und, far = (int(f[i]) for i in (1, 3, 5, 7, 9, 11))
    assert wrong == 0 and states > 3_000_000 and cert > 1_000_000
    # states within about 1e-3 (relative) of contact stay undecided; states away from it do not
    assert far_und / far < 0.02, r.stdout


def test_disentangled_check_has_teeth(dis_harness):
    """The same run without the error bound certifies wrong verdicts."""
    r = subprocess.run([dis_harness, "50000", "3", "0"], capture_output=True, text=True)
    f = r.stdout.split()
    assert int(f[1]) > 100, r.stdout
