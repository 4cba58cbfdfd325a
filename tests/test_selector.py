"""The learned plan selector: the perceptron kernels against the numpy oracle,
the measured dataset, and the selector's regret against exhaustive search and
against the default plan."""
import os

import numpy as np
import pytest

from oracle import mlp_oracle as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DATA = os.path.join(ROOT, "tests", "golden", "selector_timings.npz")
NIN, NH, NOUT = 18, 64, 16


def _rand_problem(seed, B=96, nin=NIN, nh=NH, nout=NOUT):
    rng = np.random.default_rng(seed)
    nparams = nin * nh + nh + nh * nh + nh + nh * nout + nout
    p = (rng.standard_normal(nparams) * 0.2).astype(np.float32)
    X = rng.random((B, nin), dtype=np.float32)
    T = rng.random((B, nout), dtype=np.float32)
    return p, X, T


def test_oracle_gradient_matches_finite_differences():
    p, X, T = _rand_problem(1, B=7, nin=5, nh=6, nout=4)
    p = p.astype(np.float64)
    _, g = M.loss_grad(p, X, T, 5, 6, 4)
    h = 1e-6
    for i in range(0, p.size, 3):
        e = np.zeros_like(p)
        e[i] = h
        fd = (M.loss_grad(p + e, X, T, 5, 6, 4)[0] - M.loss_grad(p - e, X, T, 5, 6, 4)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 + 1e-5 * abs(g[i])


def test_oracle_adam_reduces_loss():
    p, X, T = _rand_problem(2, B=32)
    l0, _ = M.loss_grad(p, X, T, NIN, NH, NOUT)
    _, l1 = M.train(p, X, T, NIN, NH, NOUT, steps=50, lr=3e-3)
    assert l1 < 0.5 * l0


def test_sample_shapes_follow_the_workload():
    from heffte_gb300 import selector
    shapes = selector.sample_shapes(2000)
    assert shapes == selector.sample_shapes(2000)
    sides = np.array([s for s, _, _ in shapes])
    assert sides.min() >= 32 and sides.max() <= 768
    rough = np.array([any(n % 7 == 0 or n % 11 == 0 for n in s) for s, _, _ in shapes])
    assert 0.17 < rough.mean() < 0.23
    for s, _, _ in shapes:
        for n in s:
            m = n
            for q in (2, 3, 5, 7, 11):
                while m % q == 0:
                    m //= q
            assert m == 1
    kinds = {k for _, k, _ in shapes}
    assert kinds == {0, 1, 2}
    precs = np.array([p for _, _, p in shapes])
    assert 0.4 < precs.mean() < 0.6
    assert max(s[0] * s[1] * s[2] for s, _, _ in shapes) <= 1 << 26


def test_features_and_candidates(gb):
    from heffte_gb300 import selector
    f = selector.features((64, 48, 35), gb.kind.r2c, 1)
    assert f.shape == (18,)
    assert f[4:8].tolist() == [0.0, 1.0, 0.0, 1.0]        # kind one-hot, precision
    assert f[8] == 1.0 and f[11] == 0.0 and f[14] == 0.0  # 64 is a power of two, 48 and 35 are not
    seen = set()
    for c in range(16):
        opts, v, t, r = selector.candidate(c)
        seen.add((opts.use_reorder, v, t, r))
    assert len(seen) == 16
    with pytest.raises(gb.HeffteError):
        selector.candidate(16)


@pytest.mark.skipif(not os.path.exists(DATA), reason="selector dataset not measured")
def test_dataset_matches_its_shapes(gb):
    from heffte_gb300 import selector
    d = np.load(DATA)
    shapes = selector.sample_shapes(len(d["X"]), seed=int(d["seed"]))
    assert [tuple(s) for s in d["sizes"].tolist()] == [s for s, _, _ in shapes]
    for i in range(0, len(shapes), 97):
        s, k, p = shapes[i]
        np.testing.assert_array_equal(d["X"][i], selector.features(s, k, p))
    T = d["T"]
    assert T.shape == (len(shapes), 16)
    assert np.all(np.isnan(T) | (T > 0))
    assert np.all(np.isfinite(np.nanmin(T, axis=1)))


# ---------------------------------------------------------------------------
# GPU: the CUDA kernels against the oracle, and the selector's regret
# ---------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("B", [1, 33, 2000])
def test_cuda_gradient_matches_oracle(gb, B):
    from heffte_gb300 import selector
    net = selector.Selector(hidden=NH, seed=3)
    p, X, T = _rand_problem(4, B=B)
    net.set_params(p)
    np.testing.assert_array_equal(net.params(), p)
    loss, g = net.loss_grad(X, T)
    lref, gref = M.loss_grad(p, X, T, NIN, NH, NOUT)
    assert abs(loss - lref) <= 1e-5 * abs(lref)
    assert np.linalg.norm(g - gref) <= 1e-5 * np.linalg.norm(gref)


@pytest.mark.gpu
def test_cuda_forward_matches_oracle(gb):
    from heffte_gb300 import selector
    net = selector.Selector(hidden=NH, seed=5)
    p, X, _ = _rand_problem(6, B=257)
    net.set_params(p)
    y = net.predict(X)
    yref, _ = M.forward(p, X, NIN, NH, NOUT)
    assert np.linalg.norm(y - yref) <= 1e-6 * np.linalg.norm(yref)


@pytest.mark.gpu
def test_cuda_adam_training_matches_oracle(gb):
    from heffte_gb300 import selector
    net = selector.Selector(hidden=NH, seed=7)
    p, X, T = _rand_problem(8, B=64)
    net.set_params(p)
    loss = net.train(X, T, steps=40, lr=1e-3)
    pref, lref = M.train(p, X, T, NIN, NH, NOUT, steps=40, lr=1e-3)
    assert abs(loss - lref) <= 1e-3 * abs(lref)
    assert np.max(np.abs(net.params() - pref)) <= 1e-4


@pytest.mark.gpu
def test_select_agrees_with_predict(gb):
    from heffte_gb300 import selector
    net = selector.Selector(hidden=NH, seed=9)
    for s, k, p in selector.sample_shapes(20, seed=11):
        x = selector.features(s, k, p)[None, :]
        assert net.select(s, k, p) == int(net.predict(x).argmin())


def _split(n, seed=0):
    idx = np.random.default_rng(seed).permutation(n)
    cut = int(0.8 * n)
    return idx[:cut], idx[cut:]


@pytest.mark.gpu
@pytest.mark.skipif(not os.path.exists(DATA), reason="selector dataset not measured")
def test_selector_regret_and_gain(gb):
    """Trained on 80% of the measured shapes, the selector's picks on the other
    20% are within 5% of exhaustive search and faster than the default plan
    (the options heFFTe's fixed rules give) and than the best single fixed
    candidate."""
    from heffte_gb300 import selector
    d = np.load(DATA)
    X, T = d["X"], selector.filled(d["T"])
    tr, te = _split(len(X))
    net = selector.Selector(hidden=NH, seed=1)
    net.train(X[tr], selector.targets(T[tr]), steps=4000, lr=2e-3)
    choice = net.choose(X[te])
    r_sel = selector.regret(T[te], choice)
    r_default = selector.regret(T[te], np.zeros(len(te), dtype=int))
    fixed = int(np.argmin(np.log(T[tr] / T[tr].min(axis=1, keepdims=True)).mean(axis=0)))
    r_fixed = selector.regret(T[te], np.full(len(te), fixed))
    print(f"held-out regret: selector {r_sel:.4f}, default plan {r_default:.4f}, best fixed candidate "
          f"{fixed} {r_fixed:.4f}")
    assert r_sel <= 0.05
    assert r_sel < r_default
    assert r_sel <= r_fixed


@pytest.mark.gpu
def test_plan_for_with_and_without_network(gb):
    """plan_for uses the network's pick, or exhaustive timing without one; both
    plans compute the same transform (numerics are untouched by the choice)."""
    import torch
    from heffte_gb300 import selector
    size, tkind, prec = (48, 40, 36), gb.kind.c2c, 0
    rng = np.random.default_rng(5)
    n = int(np.prod(size))
    x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
    from oracle import heffte_oracle as O
    ref = O.fft3d_c2c(x, size)
    c = selector.best_candidate(size, tkind, prec)
    assert 0 <= c < 16
    net = selector.Selector(hidden=NH, seed=1)
    for p in (selector.plan_for(size, tkind, prec), selector.plan_for(size, tkind, prec, net)):
        xin = torch.from_numpy(x).cuda()
        y = torch.empty_like(xin)
        p.forward(xin, y)
        assert O.rel_l2(y.cpu().numpy(), ref) <= 1e-6
