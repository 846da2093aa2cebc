"""Generate the committed golden fixtures of tests/golden/.

Run where the reference checkout (read-only) is present: PW_REFERENCE_DIR
names it, by default a sibling of this repository named "reference".  Machines
without the checkout read only the files this script writes.

* alpha_puzzle.npz -- the reference's alpha puzzle (res/alpha/alpha_env-1.2.org.obj,
  res/alpha/alpha-1.2.org.obj) parsed by objio.load_obj, the OMPL robot centre
  the reference records for it (src/RL/aniconf12.py:17), the OMPL solution
  path (res/alpha/alpha-1.2.org.path, w-last), its w-first keys
  (alpha-1.2.org.w-first.npz) and the tunnel vertices (alpha-1.2.org.tunnel*.npz).
  Every one of those states is collision-free in the reference (it is a
  planner's solution), so they pin the oracle's "free" verdicts.
* alpha_rl.npz -- the mesh pair and states of src/RL/test_collide.py (see alpha_rl).
* fcl_kat.npz -- the triangle pair of sancheck/fclcontacts/main.cc:17-64
  (expected: collision) and the analytic intersection segment of that pair.
* torus_regression.npz -- seeded interlocking-tori states and segments with
  the oracle's verdicts / first-contact steps, a regression pin for both the
  oracle and the GPU path.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from puzzletunneldiscovery_gb300 import objio, workloads  # noqa: E402

REF = os.environ.get("PW_REFERENCE_DIR", os.path.join(os.path.dirname(ROOT), "reference"))


def alpha():
    A = os.path.join(REF, "res", "alpha")
    Ve, Fe = objio.load_obj(os.path.join(A, "alpha_env-1.2.org.obj"))
    Vr, Fr = objio.load_obj(os.path.join(A, "alpha-1.2.org.obj"))
    center = np.array([16.973146438598633, 1.2278236150741577, 10.204807281494141])
    path = np.loadtxt(os.path.join(A, "alpha-1.2.org.path"))
    keys = np.load(os.path.join(A, "alpha-1.2.org.w-first.npz"))["VS"]
    tun = np.load(os.path.join(A, "alpha-1.2.org.tunnel.npz"))["TUNNEL_V"]
    tun_more = np.load(os.path.join(A, "alpha-1.2.org.tunnel-more.npz"))["TUNNEL_V"]
    np.savez_compressed(os.path.join(HERE, "alpha_puzzle.npz"), Ve=Ve, Fe=Fe, Vr=Vr, Fr=Fr, center=center,
                        path_wlast=path, keys_wfirst=keys, tunnel=tun, tunnel_more=tun_more)


def alpha_rl():
    """res/alpha/env-1.2.obj + robot.obj and the states src/RL/test_collide.py:39-53
    checks on them (float32 as the script builds them): [0.04, 0, 0, .5, .5, .5, .5]
    and [0.7, 0, 0, .5, .5, .5, .5], both printed with "Expecting True", plus the
    script's x sweep [-0.8, 0.8) step 0.02 with the oracle's verdicts (a regression
    pin; the reference prints the sweep without expectations)."""
    A = os.path.join(REF, "res", "alpha")
    Ve, Fe = objio.load_obj(os.path.join(A, "env-1.2.obj"))
    Vr, Fr = objio.load_obj(os.path.join(A, "robot.obj"))
    expect_free = np.array([[0.04, 0, 0, 0.5, 0.5, 0.5, 0.5], [0.7, 0, 0, 0.5, 0.5, 0.5, 0.5]],
                           dtype=np.float32).astype(np.float64)
    sweep = np.array([[x, 0, 0, 0.5, 0.5, 0.5, 0.5] for x in np.arange(-0.8, 0.8, 0.02)],
                     dtype=np.float32).astype(np.float64)
    w = O.OracleWorld(Ve, Fe, Vr, Fr)
    np.savez_compressed(os.path.join(HERE, "alpha_rl.npz"), Ve=Ve, Fe=Fe, Vr=Vr, Fr=Fr, expect_free=expect_free,
                        sweep=sweep, sweep_valid=w.is_valid(sweep))


def fcl_kat():
    h = np.array([[0, 0, 0], [1, 0, 0], [0, 0, 1]], dtype=np.float64)
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], dtype=np.float64) + np.array([-0.49, -0.5, 0.5])
    np.savez(os.path.join(HERE, "fcl_kat.npz"), tri_h=h, tri_v=v, collide=np.array(True),
             isect=np.array([[0.0, 0.0, 0.5], [0.01, 0.0, 0.5]]))


def torus_regression():
    Ve, Fe, Vr, Fr = workloads.cfg_interlocking_tori()
    w = O.OracleWorld(Ve, Fe, Vr, Fr)
    s = w.scene_scale
    q = workloads.uniform_states(3000, -2.0, 2.0, s, seed=0)
    valid = w.is_valid(q)
    dis = w.is_disentangled(q)
    q0, q1 = workloads.segment_batch(300, -2.0, 2.0, s, seed=0)
    first, checks = w.segments_first_contact(q0, q1, 0.001, mode=0)
    tfirst, _ = w.segments_first_contact(q0, q1, 0.001, mode=1)
    np.savez_compressed(os.path.join(HERE, "torus_regression.npz"), states=q, valid=valid, disentangled=dis,
                        seg_from=q0, seg_to=q1, first=first, checks=checks, transition_first=tfirst,
                        delta=np.array(0.001))


if __name__ == "__main__":
    makers = {"alpha": alpha, "alpha_rl": alpha_rl, "fcl_kat": fcl_kat, "torus_regression": torus_regression}
    for name in (sys.argv[1:] or list(makers)):
        makers[name]()
    print("fixtures written to", HERE)
