"""The learned proposal on the GPU: forward, gradients and Adam against the CPU
oracle (oracle/mlp_oracle.py), and a trained network that beats uniform
sampling at finding free states.  Everything runs through libpwcollide.so.

Tolerances.  The device accumulates in FP32 in a different order from the
FP64 oracle, and a BF16 rounding of an activation can land on the other side
of a tie; both are far below these bounds:
  * probabilities: |p_dev - p_oracle| <= 2e-3 (absolute);
  * loss: relative 1e-3;
  * gradients: per parameter tensor, ||g_dev - g_oracle|| <= 2e-2 ||g_oracle||;
  * Adam: parameters after the step within 1e-6 relative of the oracle step
    applied to the device gradient.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mo():
    from oracle import mlp_oracle
    return mlp_oracle


def _net(seed=1):
    from puzzletunneldiscovery_gb300.surrogate import Surrogate
    return Surrogate(0, seed)


def _states(n, seed):
    from puzzletunneldiscovery_gb300 import workloads as W
    return W.uniform_states(n, -2.0, 2.0, 0.4, seed=seed)


def _tensors(mo, p):
    layers, ow5, ob5, n = mo.layout()
    out = []
    for l, (o, fin, ob) in enumerate(layers):
        out.append(("W%d" % (l + 1), slice(o, o + mo.H * fin)))
        out.append(("b%d" % (l + 1), slice(ob, ob + mo.H)))
    out.append(("w5", slice(ow5, ow5 + mo.H)))
    out.append(("b5", slice(ob5, ob5 + 1)))
    return out


def test_parameter_block_layout(built_lib, mo):
    net = _net()
    assert net.num_params == mo.layout()[3]
    p = net.params()
    W1 = p[:mo.H * mo.KIN].reshape(mo.H, mo.KIN)
    assert (W1[:, 9:] == 0).all() and np.abs(W1[:, :9]).max() > 0
    p2 = np.random.default_rng(0).normal(0, 0.05, p.shape).astype(np.float32)
    net.set_params(p2)
    assert (net.params() == p2).all()


@pytest.mark.parametrize("n", [1, 127, 4096, 70001])
def test_predict_matches_oracle(built_lib, mo, n):
    net = _net(2)
    q = _states(n, 10 + n)
    p = net.params().astype(np.float64)
    want = mo.predict(p, q)
    got = net.predict(torch.from_numpy(q).cuda()).cpu().numpy()
    assert got.shape == (n,)
    assert np.abs(got - want).max() <= 2e-3


@pytest.mark.parametrize("n", [1, 128, 129, 300000])
def test_tcgen05_forward_matches_mma_forward(built_lib, mo, n):
    """The fused tcgen05 kernel (pw_mlp_predict) and the layer-by-layer mma.sync
    kernels (pw_mlp_predict_mma) compute the same network: both against the
    oracle, and against each other, on tile-aligned and ragged batch sizes."""
    net = _net(7)
    q = _states(n, 40 + n)
    dq = torch.from_numpy(q).cuda()
    a = net.predict(dq)
    net.check()
    b = net.predict_mma(dq)
    logit = net.score(dq).cpu().numpy()
    a, b = a.cpu().numpy(), b.cpu().numpy()
    assert np.abs(a - b).max() <= 2e-3
    assert np.abs(1.0 / (1.0 + np.exp(-logit.astype(np.float64))) - a).max() <= 1e-6
    k = min(n, 2048)
    want = mo.predict(net.params().astype(np.float64), q[:k])
    assert np.abs(a[:k] - want).max() <= 2e-3


def test_tcgen05_forward_after_training_step(built_lib, mo):
    """Adam updates reach the swizzled weight images the tcgen05 kernel reads."""
    net = _net(8)
    q = torch.from_numpy(_states(65536, 50)).cuda()
    y = (q[:, :3].norm(dim=1) > 0.5).to(torch.uint8)
    net.predict(q)
    for _ in range(3):
        net.train_step(q, y, 1e-3)
    a = net.predict(q[:4096]).cpu().numpy()
    net.check()
    want = mo.predict(net.params().astype(np.float64), q[:4096].cpu().numpy())
    assert np.abs(a - want).max() <= 2e-3


@pytest.mark.parametrize("kernels", ["tcgen05", "mma"])
@pytest.mark.parametrize("n", [1000, 65536])
def test_gradients_match_oracle(built_lib, mo, n, kernels):
    """Both training paths (tcgen05 GEMMs with TMA-loaded operands, and the
    mma.sync GEMMs) give the oracle's gradients."""
    net = _net(3)
    net.set_training_kernels(kernels == "mma")
    q = _states(n, 20)
    y = (np.linalg.norm(q[:, :3], axis=1) > 0.5).astype(np.uint8)
    p = net.params().astype(np.float64)
    loss = net.gradients(torch.from_numpy(q).cuda(), torch.from_numpy(y).cuda())
    L, g = mo.gradients(p, q, y)
    assert abs(loss - L) <= 1e-3 * abs(L)
    gd = net.grads().astype(np.float64)
    for name, sl in _tensors(mo, p):
        ref = g[sl]
        err = np.linalg.norm(gd[sl] - ref)
        assert err <= 2e-2 * np.linalg.norm(ref) + 1e-9, (name, err, np.linalg.norm(ref))


def test_training_kernels_agree(built_lib, mo):
    """The two training paths give the same gradient, tensor by tensor, to
    BF16-rounding accuracy (ragged batch: 30000 rows is no multiple of 128)."""
    q = torch.from_numpy(_states(30000, 60)).cuda()
    y = (q[:, :3].norm(dim=1) > 0.45).to(torch.uint8)
    grads = []
    for mma in (False, True):
        net = _net(6)
        net.set_training_kernels(mma)
        net.gradients(q, y)
        grads.append(net.grads().astype(np.float64))
    p = _net(6).params().astype(np.float64)
    for name, sl in _tensors(mo, p):
        a, b = grads[0][sl], grads[1][sl]
        assert np.linalg.norm(a - b) <= 2e-2 * np.linalg.norm(b) + 1e-9, name


def test_adam_step_matches_oracle(built_lib, mo):
    net = _net(4)
    q = torch.from_numpy(_states(4096, 30)).cuda()
    y = (torch.rand(4096, device="cuda") < 0.5).to(torch.uint8)
    p0 = net.params().astype(np.float64)
    net.gradients(q, y)
    g = net.grads().astype(np.float64)
    net.train_step(q, y, 1e-3)
    p1 = net.params().astype(np.float64)
    want, _, _ = mo.adam(p0, g, np.zeros_like(p0), np.zeros_like(p0), 1, 1e-3)
    assert np.abs(p1 - want).max() <= 1e-6 * max(1.0, np.abs(want).max())


def test_checkpoint_resume_gives_the_same_next_step(built_lib, mo, tmp_path):
    """A torch.save checkpoint (parameters, Adam moments, step count) restores
    into a fresh network exactly, and the resumed network's next Adam step is
    the oracle step from the restored state (1e-6 relative, as above).  The
    moments matter: restoring the parameters alone gives a different step."""
    lr = 1e-3
    a = _net(11)
    for s in range(3):
        q = torch.from_numpy(_states(8192, 80 + s)).cuda()
        a.train_step(q, (q[:, :3].norm(dim=1) > 0.45).to(torch.uint8), lr)
    path = str(tmp_path / "net.pt")
    a.save(path)
    ck = torch.load(path, weights_only=True)
    assert ck["step"] == 3 and ck["m2"].abs().sum() > 0
    b = _net(99)
    b.load(path)
    assert np.array_equal(b.params(), ck["params"].numpy())
    st = b.adam_state()
    assert st["step"] == 3 and np.array_equal(st["m1"], ck["m1"].numpy()) and np.array_equal(st["m2"], ck["m2"].numpy())
    q = torch.from_numpy(_states(8192, 90)).cuda()
    y = (q[:, :3].norm(dim=1) > 0.45).to(torch.uint8)
    b.train_step(q, y, lr)
    pb = b.params().astype(np.float64)
    want, _, _ = mo.adam(ck["params"].numpy().astype(np.float64), b.grads().astype(np.float64),
                         ck["m1"].numpy().astype(np.float64), ck["m2"].numpy().astype(np.float64), 4, lr)
    tol = 1e-6 * max(1.0, np.abs(want).max())
    assert np.abs(pb - want).max() <= tol
    a.train_step(q, y, lr)
    assert np.abs(a.params().astype(np.float64) - pb).max() <= 2 * tol
    c = _net(99)
    c.set_params(ck["params"].numpy())
    c.train_step(q, y, lr)
    assert np.abs(c.params().astype(np.float64) - pb).max() > 100 * tol
    with pytest.raises(ValueError):
        b.load_state_dict({"format": "something else"})


def test_bounded_wait_runs_out_and_is_reported(built_lib):
    """The tcgen05 forward kernel's waits are bounded: a launch whose weight
    copies are withheld (nothing ever completes the stage it waits for) gives
    up after the limit, frees its tensor memory and returns; pw_mlp_check
    reports it, and the next launch gives the same probabilities as before."""
    import time
    from puzzletunneldiscovery_gb300 import _lib
    net = _net(2)
    q = torch.from_numpy(_states(4096, 70)).cuda()
    want = net.predict(q).clone()
    net.check()
    assert net._L.pw_mlp_withhold_next_weights(net._h) == _lib.PW_OK
    t0 = time.perf_counter()
    net.predict(q)
    with pytest.raises(_lib.PwError) as e:
        net.check()
    assert e.value.code == _lib.PW_ERR_INTERNAL and "gave up" in str(e.value)
    assert time.perf_counter() - t0 < 30.0
    got = net.predict(q)
    net.check()
    assert torch.equal(got, want)


def test_training_beats_uniform_sampling(built_lib):
    """The gain the network brings: after online training on exact labels, the
    top 10% of candidates it ranks are free far more often than uniform
    candidates, and every accepted sample is exactly free."""
    import puzzletunneldiscovery_gb300 as pw
    from puzzletunneldiscovery_gb300 import surrogate as S
    from puzzletunneldiscovery_gb300 import workloads as W
    Ve, Fe, Vr, Fr = W.cfg_interlocking_tori()
    uw = pw.UnitWorld(0)
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    dev = torch.device("cuda", 0)
    gen = torch.Generator(device=dev)
    gen.manual_seed(0)
    draw = lambda n: S.uniform_states_device(n, -2.0, 2.0, uw.scene_scale, gen, dev)  # noqa: E731
    net = _net(5)
    rep = S.train_online(uw, net, draw, 4 << 20, batch=65536, lr=1e-3, log_every=16)
    assert rep.losses[-1][1] < 0.6 * rep.losses[0][1]
    cand = draw(1 << 22)
    exact = uw.is_valid_states(cand)
    base = float(exact.float().mean())
    acc, g = S.guided_free_samples(uw, net, cand, top_frac=0.1)
    assert uw.is_valid_states(acc).all()          # no false-free sample
    assert g.precision >= min(0.99, base + 0.3)
    prec, rec = S.precision_recall(net.predict(cand), exact)
    assert prec > base + 0.2 and rec > 0.8


@pytest.mark.parametrize("n,k,lo", [(1, 1, 0.0), (1000, 100, 0.0), (1 << 20, 104857, 0.0), (300000, 300000, 0.0),
                                    (200000, 77777, -8.0), (65536, 3, -1.0)])
def test_select_top_is_exact(built_lib, n, k, lo):
    """pw_select_top keeps exactly the states scored at or above the k-th
    largest score, ties included (scores quantised so that ties occur;
    negative scores where lo < 0)."""
    from puzzletunneldiscovery_gb300.surrogate import select_top
    g = torch.Generator(device="cuda")
    g.manual_seed(n)
    score = lo + (torch.rand(n, device="cuda", generator=g) * 4096).floor() / 4096 * (1.0 - 2 * lo)
    q = torch.zeros((n, 7), dtype=torch.float64, device="cuda")
    q[:, 0] = torch.arange(n, device="cuda", dtype=torch.float64)
    out = select_top(score, q, k)
    kth = torch.topk(score, k).values.min()
    want = torch.nonzero(score >= kth).flatten()
    got = torch.sort(out[:, 0].long()).values
    assert got.shape[0] >= k
    assert torch.equal(got, want)
