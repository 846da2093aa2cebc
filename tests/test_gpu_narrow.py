"""Narrow-passage search on the plate / torus-knot meshes: the crossing filter
on constructed cases, and a small search whose escapes are all exactly free
(re-checked by the oracle)."""
import numpy as np
import pytest
import torch

from puzzletunneldiscovery_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_crossing_filter_constructed_cases(built_lib):
    from puzzletunneldiscovery_gb300 import narrow as N
    dev = torch.device("cuda", 0)
    probes = torch.tensor([[0.0, 0.0, 0.0]], dtype=torch.float64, device=dev)
    root = torch.tensor([[0.1, 0.2, 0.1, 1, 0, 0, 0]], dtype=torch.float64, device=dev)
    ends = torch.tensor([[0.1, 0.2, -0.1, 1, 0, 0, 0],      # crosses inside
                         [0.9, 0.2, -0.1, 1, 0, 0, 0],      # crosses at x = 0.5: outside extent 0.4
                         [0.1, 0.2, 0.05, 1, 0, 0, 0],      # stays above
                         [0.1, 0.2, 0.1, 0, 1, 0, 0]],      # rotation only: the probe at the origin stays
                        dtype=torch.float64, device=dev)
    roots = root.expand(1, 7).contiguous()
    got = N.crossings(roots, ends, 4, probes, 0.0, 0.4).cpu().numpy().tolist()
    assert got == [True, False, False, False]
    # a probe off the origin: a half turn about x carries it through the plane
    probes = torch.tensor([[0.0, 0.0, 0.15]], dtype=torch.float64, device=dev)
    ends = torch.tensor([[0.1, 0.2, 0.1, 0, 1, 0, 0]], dtype=torch.float64, device=dev)
    assert N.crossings(roots, ends, 1, probes, 0.0, 0.4).cpu().numpy().tolist() == [True]


def test_small_search_escapes_are_free(built_lib, oracle_mod):
    import puzzletunneldiscovery_gb300 as pw
    from puzzletunneldiscovery_gb300 import narrow as N
    from puzzletunneldiscovery_gb300.surrogate import Surrogate
    Ve, Fe, Vr, Fr = W.cfg_plate_knot(n=120)
    uw = pw.UnitWorld(0)
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    s = uw.scene_scale
    gen = torch.Generator(device="cuda")
    gen.manual_seed(3)
    lo, hi = Ve.min(0) - 0.5, Ve.max(0) + 0.5
    roots = N.draw_free_roots(uw, 20000, lo, hi, gen)
    assert uw.is_valid_states(roots).all()
    probes = N.centre_line_probes(uw, 256, 16, every=8)
    extent = float(np.abs(Ve[:, :2]).max()) * s
    net = Surrogate(0, 9)
    search = N.NarrowPassageSearch(uw, net, probes, 0.0, extent, k=4096, retrain_labels=8192, seed=1)
    rep = search.run(roots, guided=True, roots_per_round=5000, keep_escapes=True)
    assert rep.crossing > 0 and rep.validated > 0
    assert rep.retrains >= 1
    plain = N.NarrowPassageSearch(uw, None, probes, 0.0, extent, k=4096, seed=1)
    prep = plain.run(roots, guided=False, roots_per_round=5000)
    assert prep.validated > 0
    ow = oracle_mod.OracleWorld(Ve, Fe, Vr, Fr)
    checked = 0
    for frm, to in rep.escape_states:
        f, t = frm.cpu().numpy(), to.cpu().numpy()
        for i in range(min(len(f), 40)):
            (lf, st, done, _, _), _, _ = ow.transit_state_to_with_contact(f[i], t[i], min(0.001, 0.5 * pw.distance(f[i], t[i])))
            assert done
            checked += 1
    assert rep.escapes == 0 or checked > 0
