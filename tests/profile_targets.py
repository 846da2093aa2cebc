"""Small, fixed workloads for ncu captures (not collected by pytest).

python tests/profile_targets.py states|segments|mlp|train|all [n]
"""
import sys, os
sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import torch
import puzzletunneldiscovery_gb300 as pw
from puzzletunneldiscovery_gb300 import workloads as W
what = sys.argv[1]
n = int(sys.argv[2]) if len(sys.argv) > 2 else 1_000_000
Ve, Fe, Vr, Fr = W.cfg_interlocking_tori()
uw = pw.UnitWorld(0)
uw.load_env_mesh(Ve, Fe); uw.load_robot_mesh(Vr, Fr); uw.scaleToUnit(); uw.angleModel(0, 0)
s = uw.scene_scale
if what == "all":
    # every kernel of the engine once, on small inputs (for a launch list)
    import numpy as np
    from puzzletunneldiscovery_gb300 import narrow as N, sampling as S
    from puzzletunneldiscovery_gb300.surrogate import Surrogate, select_top
    q = torch.from_numpy(W.uniform_states(n, -2, 2, s, seed=0)).cuda()
    uw.is_valid_states(q)
    uw.is_disentangled_states(q)
    q0, q1 = W.segment_batch(max(1, n // 10), -2, 2, s, seed=0)
    a, b = torch.from_numpy(q0).cuda(), torch.from_numpy(q1).cuda()
    uw.transit_states_to_with_contact(a, b, 0.001)
    uw.intersecting_segments(np.array([0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0]))
    ends = N.expand(q[:1000], 64, 0.01, 0.1, 5)
    N.crossings(q[:1000], ends, 64, torch.zeros((4, 3), dtype=torch.float64, device="cuda"), 0.0, 0.5)
    net = Surrogate(0, 1)
    sc = net.score(q)
    select_top(sc, q, max(1, n // 10))
    net.predict_mma(q[:65536])
    y = uw.is_valid_states(q[:65536])
    net.train_step(q[:65536], y, 1e-3)
    net.set_training_kernels(True)
    net.train_step(q[:65536], y, 1e-3)
    net.check()
    torch.cuda.synchronize()
    print("done")
    sys.exit(0)
if what in ("mlp", "train"):
    from puzzletunneldiscovery_gb300.surrogate import Surrogate, uniform_states_device
    net = Surrogate(0, 1)
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    q = uniform_states_device(n, -2, 2, s, g, torch.device("cuda", 0))
    if what == "mlp":
        for _ in range(3):
            p = net.predict(q)
        net.check()
    else:
        y = uw.is_valid_states(q[:65536])
        for _ in range(3):
            net.train_step(q[:65536], y, 1e-3)
    torch.cuda.synchronize()
    print("done")
    sys.exit(0)
if what == "states":
    q = torch.from_numpy(W.uniform_states(n, -2, 2, s, seed=0)).cuda()
    for _ in range(3):
        v = uw.is_valid_states(q)
else:
    q0, q1 = W.segment_batch(n, -2, 2, s, seed=0)
    a = torch.from_numpy(q0).cuda(); b = torch.from_numpy(q1).cuda()
    for _ in range(3):
        f = uw.first_contact_steps(a, b, 0.001)
torch.cuda.synchronize()
print("done", uw.last_stats())
