"""The C ABI library loads, exports every declared entry point, and its host-only
helpers agree bit for bit with the oracle (CPU; no GPU compute)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _declared():
    names = set()
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        src = open(os.path.join(ROOT, "include", h)).read()
        names |= set(re.findall(r"PW_API[^;]*?\b(pw_[a-z0-9_]+)\s*\(", src, flags=re.S))
    return names


def test_header_and_binding_agree():
    from puzzletunneldiscovery_gb300 import _lib
    assert _declared() == set(_lib.EXPORTS)


def test_library_exports_every_symbol(built_lib):
    L = ctypes.CDLL(built_lib)
    for name in _declared():
        assert hasattr(L, name), name


def test_host_state_math_bit_exact(built_lib, oracle_mod):
    import puzzletunneldiscovery_gb300 as pw
    from puzzletunneldiscovery_gb300 import workloads as W
    q0, q1 = W.segment_batch(200, -2, 2, 0.4, seed=5)
    for a, b in zip(q0, q1):
        assert pw.distance(a, b) == oracle_mod.distance(a, b)
        for tau in (0.0, 0.25, 0.999, 1.0):
            assert (pw.interpolate(a, b, tau) == oracle_mod.interpolate(a, b, tau)).all()
    a, b = q0[0], q1[0]
    K = oracle_mod.segment_steps(a, b, 0.001)
    for k in (0, 1, K // 2, K - 1):
        s, tau, n = pw.segment_step_state(a, b, 0.001, k)
        s2, tau2 = oracle_mod.segment_state(a, b, 0.001, k)
        assert n == K and (s == s2).all() and tau == tau2


def test_nearly_identical_rotations_take_linear_branch(built_lib, oracle_mod):
    import puzzletunneldiscovery_gb300 as pw
    a = np.array([0.1, 0.2, 0.3, 1.0, 0.0, 0.0, 0.0])
    b = np.array([0.2, 0.2, 0.3, 1.0, 1e-17, 0.0, 0.0])
    for tau in (0.3, 0.7):
        assert (pw.interpolate(a, b, tau) == oracle_mod.interpolate(a, b, tau)).all()
    c = b.copy()
    c[3:] = -c[3:]                         # the same rotation, opposite sign: d < 0 path
    assert (pw.interpolate(a, c, 0.4) == oracle_mod.interpolate(a, c, 0.4)).all()


def test_world_create_reports_errors_without_device(built_lib):
    import torch
    from puzzletunneldiscovery_gb300 import _lib
    L = _lib.load()
    h = ctypes.c_void_p()
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    rc = L.pw_world_create(ctypes.byref(h), 0)
    assert rc in (_lib.PW_ERR_CUDA, _lib.PW_ERR_INVALID_ARG)
    assert L.pw_last_error()
    assert L.pw_world_destroy(None) == _lib.PW_OK


def test_unitworld_refuses_cpu(built_lib):
    import torch
    import puzzletunneldiscovery_gb300 as pw
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError):
        pw.UnitWorld()


_NULL_OK = {"pw_last_error", "pw_world_destroy", "pw_mlp_destroy", "pw_mlp_num_params"}

_NULL_PROBE = r"""
import ctypes, json, sys
sys.path.insert(0, sys.argv[1])
from puzzletunneldiscovery_gb300 import _lib
L = _lib.load()
out = {}
for name in _lib.EXPORTS:
    if name in %r:
        continue
    fn = getattr(L, name)
    args = []
    for t in fn.argtypes:
        if t in (ctypes.c_int, ctypes.c_int64, ctypes.c_uint64, ctypes.c_int32):
            args.append(t(1))
        elif t in (ctypes.c_double, ctypes.c_float):
            args.append(t(1.0))
        else:
            args.append(None)
    rc = fn(*args)
    out[name] = [int(rc), (L.pw_last_error() or b"").decode()]
print(json.dumps(out))
"""


def test_every_entry_point_rejects_null_arguments(built_lib):
    """Host-side fault injection without a device: every entry point, called with
    NULL for each pointer and size 1, returns an error status and leaves a
    message in pw_last_error instead of dereferencing anything.  Runs in a child
    process so that a missing check shows as a failed test, not a crashed run."""
    import json
    import subprocess
    import sys
    r = subprocess.run([sys.executable, "-c", _NULL_PROBE % (_NULL_OK,), ROOT], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    from puzzletunneldiscovery_gb300 import _lib
    assert set(res) == set(_lib.EXPORTS) - _NULL_OK
    for name, (rc, msg) in res.items():
        assert rc != _lib.PW_OK, name
        assert msg, name


@pytest.mark.parametrize("lang,std", [("c", "-std=c99"), ("c++", "-std=c++11")])
def test_headers_compile_standalone(lang, std, tmp_path):
    """The C-ABI headers are usable from plain C99 and C++11 callers (a cgo / JNI /
    ctypes binding compiles against them), with every warning enabled."""
    import shutil
    import subprocess
    cc = shutil.which("gcc" if lang == "c" else "g++")
    if cc is None:
        pytest.skip("no host compiler")
    src = tmp_path / ("use." + ("c" if lang == "c" else "cc"))
    src.write_text('#include "pw_collide.h"\n#include "pw_mlp.h"\n'
                   "int use(void) { return pw_last_error() != 0 ? PW_OK : PW_ERR_INTERNAL; }\n")
    r = subprocess.run([cc, "-fsyntax-only", std, "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                        str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_every_mesh_array_is_kept_on_a_partial_rebuild():
    """pw_world_set_perturbation rebuilds the env mesh and keeps the robot's device
    arrays: the keep list (mesh_arrays) must name every array the mesh build
    allocates, or the robot's would be freed while still in use."""
    src = open(os.path.join(ROOT, "puzzletunneldiscovery_gb300", "csrc", "pw_world.cu")).read()
    allocated = set(re.findall(r"walloc\(w, &m\.(\w+),", src))
    body = re.search(r"mesh_arrays\(const MeshDev &m\)\s*\{(.*?)\}", src, re.S).group(1)
    kept = set(re.findall(r"m\.(\w+)", body))
    assert allocated and allocated == kept, (allocated - kept, kept - allocated)
