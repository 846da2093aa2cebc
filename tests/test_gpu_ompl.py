"""OMPL's discrete motion check on the GPU (pw_ompl_check_motions and
pw_ompl_motion_states, the check behind OmplDriver::validateMotionPairs,
lib/pyse3ompl/ompldriver.cc:597-621) against the oracle's restatement of OMPL's
rule, on OMPL-frame states of the alpha puzzle: the checked states bit for bit,
the verdicts exactly, and the windowed batch path against per-state verdicts."""
import numpy as np
import pytest
import torch

from conftest import golden

pytestmark = pytest.mark.gpu

CDRES = 0.01


def _pair(O, Ve, Fe, Vr, Fr, center):
    import puzzletunneldiscovery_gb300 as pw
    uw = pw.UnitWorld()
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.enforceRobotCenter(center)
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    return uw, O.OracleWorld(Ve, Fe, Vr, Fr, center=np.asarray(center, dtype=np.float32))


@pytest.fixture(scope="module")
def alpha(oracle_mod, built_lib):
    g = golden("alpha_puzzle.npz")
    uw, ow = _pair(oracle_mod, g["Ve"], g["Fe"], g["Vr"], g["Fr"], g["center"].astype(np.float32))
    P = uw.translate_unit_to_ompl(uw.translate_to_unit_state(g["keys_wfirst"]))
    lo = P[:, :3].min(axis=0) - 20.0
    hi = P[:, :3].max(axis=0) + 20.0
    return uw, ow, P, lo, hi


def _motions(P, n, seed, sigma=2.0):
    """Consecutive keys, random key pairs with perturbed targets, and the edge
    cases of OMPL's rule: a motion to itself, a target written with the negated
    quaternion, and a translation with a rotation change below OMPL's 1e-9 cut."""
    rng = np.random.default_rng(seed)
    A = [P[:-1]]
    B = [P[1:]]
    i = rng.integers(0, len(P), n)
    j = rng.integers(0, len(P), n)
    Bj = P[j].copy()
    Bj[:, :3] += rng.normal(0.0, sigma, (n, 3))
    A.append(P[i])
    B.append(Bj)
    same = P[:3].copy()
    neg = P[3:6].copy()
    neg[:, 3:] = -neg[:, 3:]
    tiny = P[6:9].copy()
    tiny[:, 0] += 0.5
    A += [P[:3], P[3:6] + np.array([0.3, 0, 0, 0, 0, 0, 0]), P[6:9]]
    B += [same, neg, tiny]
    return np.concatenate(A), np.concatenate(B)


def _expected_checks(ok, counts):
    """States the passes check, given every state's verdict in listing order (the
    target, then k = 1 .. nd - 1): each target, then level by level while every
    state checked so far is free, level l of a motion with m = nd - 1 and
    T = floor(log2 m) holding the odd multiples of 2^(T - l) in 1 .. m."""
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
    total = 0
    for s, nd in zip(starts, counts):
        total += 1
        free = bool(ok[s])
        m = int(nd) - 1
        T = m.bit_length() - 1
        for e in range(T, -1, -1):
            if not free:
                break
            ks = np.arange(1 << e, m + 1, 2 << e)
            total += len(ks)
            free = bool(ok[s + ks].all())
    return total


def _oracle_states(O, uw, A, B, lo, hi, cdres):
    per = [O.ompl_motion_states(a, b, lo, hi, cdres) for a, b in zip(A, B)]
    counts = np.array([p.shape[0] for p in per])
    return uw.translate_ompl_to_unit(np.concatenate(per)), counts


def test_checked_states_match_the_oracle_bit_for_bit(alpha, oracle_mod):
    from puzzletunneldiscovery_gb300 import ompl_compat as OC
    uw, ow, P, lo, hi = alpha
    A, B = _motions(P, 300, seed=1)
    states, offs = OC.motion_states(uw, A, B, lo, hi, CDRES)
    want, counts = _oracle_states(oracle_mod, uw, A, B, lo, hi, CDRES)
    assert np.array_equal(np.diff(offs.cpu().numpy()), counts)
    assert counts.max() > 20 and counts.min() == 1
    got = states.cpu().numpy()
    assert got.shape == want.shape
    assert np.array_equal(got, want)


def test_verdicts_match_the_oracle(alpha, oracle_mod):
    from puzzletunneldiscovery_gb300 import ompl_compat as OC
    uw, ow, P, lo, hi = alpha
    A, B = _motions(P, 400, seed=2, sigma=4.0)
    got, checked = OC.check_motions_discrete(uw, A, B, lo, hi, CDRES)
    U, counts = _oracle_states(oracle_mod, uw, A, B, lo, hi, CDRES)
    ok = ow.is_valid(U).astype(bool)
    want = np.logical_and.reduceat(ok, np.concatenate([[0], np.cumsum(counts)[:-1]])).astype(np.int32)
    assert got.dtype == np.int32 and checked == _expected_checks(ok, counts) < counts.sum()
    assert np.array_equal(got, want)
    assert 0 < got.sum() < len(got)
    # the driver object gives the same answers once its bounds and resolution are set
    d = OC.OmplDriver(uw)
    with pytest.raises(RuntimeError):
        d.validate_motion_pairs(A, B)
    d.set_bb(lo, hi)
    d.set_cdres(CDRES)
    assert np.array_equal(d.validate_motion_pairs(A, B), got) and d.last_states_checked == checked
    assert np.array_equal(d.validate_states(B), ow.is_valid(uw.translate_ompl_to_unit(B)).astype(np.int32))


def test_windowed_batch_agrees_with_per_state_verdicts(alpha):
    """More than one window of states (4M) in the listing: every motion's verdict
    is the AND of the engine's verdicts on the states pw_ompl_motion_states lists
    for it, and the passes check exactly the states their early exits leave."""
    from puzzletunneldiscovery_gb300 import ompl_compat as OC
    uw, ow, P, lo, hi = alpha
    A, B = _motions(P, 12000, seed=3, sigma=6.0)
    cdres = 0.0007
    states, offs = OC.motion_states(uw, A, B, lo, hi, cdres)
    assert states.shape[0] > (1 << 22) + 1000
    ok = uw.is_valid_states(states).to(torch.int64)
    counts = torch.diff(offs)
    owner = torch.repeat_interleave(torch.arange(len(A), device=ok.device), counts)
    bad = torch.zeros(len(A), dtype=torch.int64, device=ok.device).index_add_(0, owner, 1 - ok)
    want = (bad == 0).to(torch.int32).cpu().numpy()
    got, checked = OC.check_motions_discrete(uw, A, B, lo, hi, cdres)
    assert checked == _expected_checks(ok.cpu().numpy(), counts.cpu().numpy())
    assert np.array_equal(got, want)
    assert 0 < got.sum() < len(got)


def test_arguments_and_edge_cases(alpha):
    from puzzletunneldiscovery_gb300 import _lib
    from puzzletunneldiscovery_gb300 import ompl_compat as OC
    uw, ow, P, lo, hi = alpha
    A, B = P[:5], P[1:6]
    for bad in (0.0, 1.0, -0.1, float("nan")):
        with pytest.raises(_lib.PwError):
            OC.check_motions_discrete(uw, A, B, lo, hi, bad)
    with pytest.raises(_lib.PwError):
        OC.check_motions_discrete(uw, A, B, hi, lo, CDRES)
    with pytest.raises(_lib.PwError):
        OC.check_motions_discrete(uw, A, B, lo, lo, CDRES)
    with pytest.raises(ValueError):
        OC.check_motions_discrete(uw, A, B, lo[:2], hi, CDRES)
    out, checked = OC.check_motions_discrete(uw, np.zeros((0, 7)), np.zeros((0, 7)), lo, hi, CDRES)
    assert out.shape == (0,) and checked == 0
    # a shorter second batch leaves the trailing rows 0, as the reference does
    full, _ = OC.check_motions_discrete(uw, P[:10], P[1:11], lo, hi, CDRES)
    short, _ = OC.check_motions_discrete(uw, P[:10], P[1:6], lo, hi, CDRES)
    assert short.shape == (10,) and np.array_equal(short[:5], full[:5]) and not short[5:].any()
    # a motion with a non-finite component is answered 0, the others are unaffected
    Bn = P[1:11].copy()
    Bn[4, 2] = np.nan
    An = P[:10].copy()
    An[7, 5] = np.inf
    nf, _ = OC.check_motions_discrete(uw, An, Bn, lo, hi, CDRES)
    keep = np.ones(10, bool)
    keep[[4, 7]] = False
    assert nf[4] == 0 and nf[7] == 0 and np.array_equal(nf[keep], full[keep])


def test_screening_with_the_ompl_rule(alpha, tmp_path):
    """screen_keyconf with an OmplDriver (the reference's screening worker,
    solve2.py:218-219) keeps exactly the lower-triangle pairs that
    validate_motion_pairs finds valid, across tasks and batches."""
    from puzzletunneldiscovery_gb300 import ompl_compat as OC
    from puzzletunneldiscovery_gb300 import screening as S
    uw, ow, P, lo, hi = alpha
    keys = P[:40]
    d = OC.OmplDriver(uw)
    d.set_bb(lo, hi)
    d.set_cdres(CDRES)
    ef, et = S.screen_keyconf(uw, keys, max_chunk_number=4, out_dir=str(tmp_path), batch=100, driver=d)
    r, c = np.tril_indices(len(keys) - S.RESERVED)
    r, c = r + S.RESERVED, c + S.RESERVED
    want = d.validate_motion_pairs(keys[r], keys[c]).astype(bool)
    assert np.array_equal(ef, r[want]) and np.array_equal(et, c[want])
    assert 0 < want.sum() <= len(want)
