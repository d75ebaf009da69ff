"""The learned refinement estimator on the GPU (adaptivemesh_gb300/csrc/estimator.cu).

* Forward pass of the BF16 tensor-core network equals the NumPy oracle (oracle/estimator_oracle.py,
  float64 with the same BF16 roundings) to FP32-accumulation differences: relative L2 <= 5e-3.
* Gradients of every parameter tensor equal the oracle's: relative L2 <= 2e-2 per tensor (the
  residual is FP32 summation order plus BF16 re-roundings of activations that sit on a rounding
  boundary).
* Tile features and plain-criterion indicators equal a NumPy restatement of the state they read.
* Adam training on Richardson-error samples lowers the loss; on a held-out configuration the
  network predicts log10 of the true error with a lower mean squared error than the plain indicator
  calibrated by a least-squares fit on the same samples, and its ranking captures at least 90% of
  the error share the ideal ranking does for a fixed refinement budget.
* Regrids by the plain criterion and by the network (judged by it) on a held-out configuration,
  followed by evolution, keep a consistent tree and finite constraints.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def random_params(eo, seed):
    rng = np.random.default_rng(seed)
    p = {}
    fan_in = {"W1": 81, "W2": 432, "W3": 1024, "W4": 32}
    for name, shape in eo.SIZES:
        if name.startswith("W"):
            p[name] = rng.uniform(-1, 1, shape) * np.sqrt(6.0 / fan_in[name])
        else:
            p[name] = rng.uniform(-0.1, 0.1, shape)
    p["W1"][81:] = 0.0
    return eo.pack(p).astype(np.float32)


def random_features(rng, b):
    x = np.empty((b, 3, 512), np.float32)
    x[:, 0] = rng.uniform(0.3, 1.0, (b, 512))
    x[:, 1] = rng.uniform(-1.0, 1.0, (b, 512))
    x[:, 2] = rng.uniform(-1.0, 1.0, (b, 512))
    return x


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-300))


def test_parameters_round_trip(am, torch_cuda):
    from oracle import estimator_oracle as eo
    est = am.Estimator(64, seed=5)
    p0 = est.get_params()
    assert p0.shape == (41313,) and np.isfinite(p0).all()
    assert np.all(eo.unpack(p0)["W1"][81:] == 0)
    p = random_params(eo, 1)
    est.set_params(p)
    assert np.array_equal(est.get_params(), p)
    est.close()


@pytest.mark.parametrize("b", [1, 37, 64, 130])
def test_forward_matches_oracle(am, torch_cuda, b):
    torch = torch_cuda
    from oracle import estimator_oracle as eo
    rng = np.random.default_rng(b)
    est = am.Estimator(64, seed=2)
    p = random_params(eo, b)
    est.set_params(p)
    x = random_features(rng, b)
    got = est.forward(torch.from_numpy(x).cuda()).cpu().numpy()
    want = eo.forward(p.astype(np.float64), x.astype(np.float64))["out"]
    err = rel_l2(got, want)
    print(f"\nforward b={b}: rel L2 {err:.2e}")
    assert err <= 5e-3
    est.close()


@pytest.mark.parametrize("b", [8, 64])
def test_gradients_match_oracle(am, torch_cuda, b):
    torch = torch_cuda
    from oracle import estimator_oracle as eo
    rng = np.random.default_rng(100 + b)
    est = am.Estimator(64, seed=3)
    p = random_params(eo, 7 + b)
    est.set_params(p)
    x = random_features(rng, b)
    t = rng.normal(-3.0, 1.0, b).astype(np.float32)
    g, loss = est.gradients(torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda())
    gw, lw = eo.gradients(p.astype(np.float64), x.astype(np.float64), t.astype(np.float64))
    assert abs(loss - lw) <= 1e-3 * lw
    gu, wu = eo.unpack(g), eo.unpack(gw)
    for name, _ in eo.SIZES:
        err = rel_l2(gu[name], wu[name])
        print(f"  grad {name}: rel L2 {err:.2e}")
        assert err <= 2e-2, name
    assert np.all(gu["W1"][81:] == 0)
    est.close()


def test_train_step_is_adam(am, torch_cuda):
    """One train_step equals one Adam step (beta 0.9 / 0.999, eps 1e-8, bias-corrected) applied to the
    gradients the library reports for the same batch."""
    torch = torch_cuda
    from oracle import estimator_oracle as eo
    rng = np.random.default_rng(9)
    est = am.Estimator(64, seed=4)
    p = random_params(eo, 11)
    est.set_params(p)
    x = torch.from_numpy(random_features(rng, 32)).cuda()
    t = torch.from_numpy(rng.normal(-2.0, 0.5, 32).astype(np.float32)).cuda()
    g, _ = est.gradients(x, t)
    est.train_step(x, t, 1e-3)
    got = est.get_params()
    m = 0.1 * g.astype(np.float64)
    v = 0.001 * g.astype(np.float64) ** 2
    want = p - 1e-3 * (m / 0.1) / (np.sqrt(v / 0.001) + 1e-8)
    want = eo.unpack(want)
    want["W1"][81:] = 0.0
    assert np.abs(got - eo.pack(want)).max() <= 2e-6 + 1e-5 * np.abs(p).max()
    est.close()


def features_restated(st, tensors, n, p):
    """NumPy restatement of the tile features and indicators from the state's chi, alpha and gt."""
    t = n + 2 * p
    r = n // 8
    used = st["used_slots"]
    pos, ch = st["positions"], st["children"]
    leaves = [s for s in range(used) if pos[s] != 0xFFFFFFFF and all(c == -1 for c in ch[8 * s:8 * s + 8])]
    chi = tensors["chi"].reshape(-1, t, t, t).astype(np.float64) + 1.0
    al = tensors["alpha"].reshape(-1, t, t, t).astype(np.float64) + 1.0
    gt = [g.reshape(-1, t, t, t).astype(np.float64) for g in tensors["gt"]]
    feats, ind = [], []
    for s in leaves:
        sl = np.s_[p:p + n, p:p + n, p:p + n]
        def cdiff(f, a):
            return 0.5 * (np.roll(f, -1, axis=2 - a) - np.roll(f, 1, axis=2 - a))[sl]
        dchi = np.sqrt(sum(cdiff(chi[s], a) ** 2 for a in range(3)))
        dal = np.sqrt(sum(cdiff(al[s], a) ** 2 for a in range(3)))
        g2 = sum(cdiff(g[s], a) ** 2 for g in gt for a in range(3))
        def pool(v, op=np.mean):
            return op(v.reshape(8, r, 8, r, 8, r), axis=(1, 3, 5)).reshape(512)
        f = np.stack([pool(chi[s][sl]), np.log10(pool(dchi + dal, np.max) + 1e-10) * 0.2 + 1.0,
                      np.log10(np.sqrt(pool(g2)) + 1e-10) * 0.2 + 1.0])
        feats.append(f)
        ind.append((dchi + dal).max())
    return leaves, np.array(feats), np.array(ind)


def test_tile_features_match_restatement(am, torch_cuda):
    from adaptivemesh_gb300 import estimator as E
    sim = E.build_sim(16, 32.0, E.binary_punctures(3), 2, mode=am.MODE_PLAIN)
    sim.timestep()
    sim.synchronize()
    feats, ind, slots = sim.tile_features()
    st = sim.state()
    t = 16 + 6
    used = st["used_slots"]
    def host(f):
        return sim.tensor(sim.NEW_STATE, f)[: used * t ** 3].cpu().numpy()
    tensors = {"chi": host(am.F_CHI), "alpha": host(am.F_ALPHA), "gt": [host(am.F_GXX + q) for q in range(6)]}
    leaves, want_f, want_i = features_restated(st, tensors, 16, 3)
    assert list(slots) == leaves
    got_f = feats.cpu().numpy()
    assert np.abs(got_f[:, 0] - want_f[:, 0]).max() <= 1e-5
    assert np.abs(got_f[:, 1:] - want_f[:, 1:]).max() <= 1e-3
    assert np.allclose(ind.cpu().numpy(), want_i, rtol=1e-4, atol=1e-7)
    sim.close()


@pytest.fixture(scope="module")
def trained(am, torch_cuda):
    """A network trained on four seeded binary Brill-Lindquist configurations, and a fifth held out."""
    torch = torch_cuda
    from adaptivemesh_gb300 import estimator as E
    fs, ts = [], []
    for seed in range(1, 5):
        f, t, _ = E.richardson_samples(seed)
        fs.append(f)
        ts.append(t)
    feats, targets = torch.cat(fs), torch.cat(ts)
    est = am.Estimator(64, seed=1)
    losses = E.train(est, feats, targets, epochs=150, batch=64, lr=2e-3)
    held = E.richardson_samples(5)
    yield est, losses, feats, targets, held
    est.close()


def test_training_lowers_the_loss(trained, torch_cuda):
    """The network's held-out error prediction, beside the plain indicator calibrated by a least-squares
    line log10(error) ~ a + b log10(indicator) fitted on the same training tiles."""
    torch = torch_cuda
    from adaptivemesh_gb300 import estimator as E
    est, losses, feats, targets, (fh, th, ih) = trained
    pred = est.forward(fh)
    mse = float(((pred - th) ** 2).mean())
    var = float(th.var())
    ind_train = torch.cat([E.richardson_samples(seed)[2] for seed in range(1, 5)])
    X = torch.stack([torch.ones_like(ind_train), torch.log10(ind_train + 1e-12)], 1).double()
    coef = torch.linalg.lstsq(X, targets.double()[:, None]).solution[:, 0]
    fit = coef[0] + coef[1] * torch.log10(ih.double() + 1e-12)
    mse_fit = float(((fit - th.double()) ** 2).mean())
    print(f"\n{feats.shape[0]} training tiles: loss {losses[0]:.3f} -> {losses[-1]:.3f}; held-out "
          f"{fh.shape[0]} tiles: MSE {mse:.3f} (network), {mse_fit:.3f} (calibrated plain indicator), "
          f"target variance {var:.3f}")
    assert losses[-1] < 0.5 * losses[0]
    assert mse < 0.5 * var
    assert mse < mse_fit   # the network's error prediction beats the calibrated plain indicator


def test_learned_ranking_captures_the_error(trained):
    """For a refinement budget of k leaves, the share of the held-out configuration's true
    (Richardson) error that the network's ranking captures, beside the plain criterion's."""
    from adaptivemesh_gb300 import estimator as E
    est, _, _, _, (fh, th, ih) = trained
    pred = est.forward(fh)
    n = fh.shape[0]
    for frac in (0.1, 0.25):
        k = max(1, int(frac * n))
        learned, plain = E.captured_error(pred, th, k), E.captured_error(ih, th, k)
        oracle_best = E.captured_error(th, th, k)
        print(f"\nbudget {k}/{n} leaves: captured error learned {learned:.3f}, plain {plain:.3f}, best {oracle_best:.3f}")
        assert learned >= 0.9 * oracle_best


def count_leaves(st):
    return sum(1 for s in range(st["used_slots"]) if st["positions"][s] != 0xFFFFFFFF
               and all(c == -1 for c in st["children"][8 * s:8 * s + 8]))


def test_regrid_plain_and_learned(am, trained, torch_cuda):
    """Regrid a held-out configuration by the plain criterion, by the network judged by it, and not
    at all, then evolve two root steps: the trees stay consistent and the constraints finite."""
    torch = torch_cuda
    from adaptivemesh_gb300 import estimator as E
    est = trained[0]
    punct = E.binary_punctures(5)
    out = {}
    for name, net in (("none", None), ("plain", None), ("learned", est)):
        sim = E.build_sim(8, 32.0, punct, 3)
        before = sim.constraint_norms(1.0)
        feats, ind, _ = sim.tile_features()
        leaves0 = count_leaves(sim.state())
        stats = {"refined": 0, "coarsened": 0, "overridden": 0, "leaves": leaves0}
        if name != "none":
            pred = est.forward(feats)
            params = am.Regrid(refine_threshold=float(torch.quantile(ind, 0.75)),
                               coarsen_threshold=float(torch.quantile(ind, 0.2)),
                               learned_refine=float(torch.quantile(pred, 0.75)),
                               learned_coarsen=float(torch.quantile(pred, 0.2)),
                               judge_factor=4.0, max_depth=5, min_depth=2)
            stats = sim.regrid(params, net)
            assert stats["leaves"] == count_leaves(sim.state()) and stats["refined"] > 0
            if net is None:
                assert stats["overridden"] == 0
        for _ in range(2):
            sim.timestep()
        sim.synchronize()
        after = sim.constraint_norms(1.0)
        out[name] = (stats, before, after)
        assert np.isfinite(after["H_l2"]) and np.isfinite(after["M_l2"])
        sim.close()
    for name, (stats, before, after) in out.items():
        print(f"\n{name}: {stats}, H_l2 {before['H_l2']:.3e} -> {after['H_l2']:.3e}, "
              f"M_l2 {before['M_l2']:.3e} -> {after['M_l2']:.3e}")
