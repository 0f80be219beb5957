"""Pins the FP64 personalised-PageRank oracle (no reference code exists for
it): power iteration against the dense solve, the analytic adjoint against
brute-force central finite differences of the dense-solve loss, the rank-one
finite-difference shortcut against the brute force, and the identities the
gradient must satisfy."""
import numpy as np
import pytest

from oracle import ppr_oracle as pp


def _graph(V=40, E=260, seed=3, dangling=(5, 17)):
    rng = np.random.default_rng(seed)
    src = rng.integers(0, V, E)
    dst = rng.integers(0, V, E)
    keep = ~np.isin(src, dangling)  # vertices with no out-edges
    src, dst = src[keep], dst[keep]
    src = np.concatenate([src, [0, 0, 3]])  # a repeated edge and a self loop
    dst = np.concatenate([dst, [1, 1, 3]])
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    off = np.zeros(V + 1, np.int64)
    np.add.at(off, src + 1, 1)
    off = np.cumsum(off)
    w = rng.lognormal(0.0, 1.0, len(dst))
    K = 3
    T = pp.seeds_teleport(V, K, 4, rng).astype(np.float64)
    W = rng.standard_normal((V, K))
    return off, dst, w, T, W


def test_power_iteration_reaches_dense_solve():
    off, dst, w, T, W = _graph()
    R, it, res = pp.forward_iter(off, dst, w, T, tol=1e-13)
    assert res < 1e-13 and it < 400
    np.testing.assert_allclose(R, pp.forward_dense(off, dst, w, T), rtol=0, atol=1e-12)


def test_adjoint_matches_brute_force_central_differences():
    off, dst, w, T, W = _graph()
    gw, gT, L, R, Lam = pp.adjoint_dense(off, dst, w, T, W)
    assert L == pytest.approx(pp.loss(off, dst, w, T, W), rel=1e-13)
    h = 1e-5
    for e in range(0, len(w), 7):
        wp, wm = w.copy(), w.copy()
        wp[e] += h
        wm[e] -= h
        fd = (pp.loss(off, dst, wp, T, W) - pp.loss(off, dst, wm, T, W)) / (2 * h)
        assert abs(fd - gw[e]) <= 1e-7 * max(1.0, abs(fd)), (e, fd, gw[e])
    for v, k in [(0, 0), (9, 1), (33, 2)]:
        Tp, Tm = T.copy(), T.copy()
        Tp[v, k] += h
        Tm[v, k] -= h
        fd = (pp.loss(off, dst, w, Tp, W) - pp.loss(off, dst, w, Tm, W)) / (2 * h)
        assert abs(fd - gT[v, k]) <= 1e-8 * max(1.0, abs(fd))


def test_rank_one_finite_difference_equals_brute_force():
    off, dst, w, T, W = _graph()
    fd = pp.FiniteDifference(off, dst, w, T, W)
    L0 = pp.loss(off, dst, w, T, W)
    for e in (0, 1, 2, 50, len(w) - 1):
        for t in (1e-4, -1e-4, 0.3):
            wt = w.copy()
            wt[e] += t
            assert fd.delta_loss(e, t) == pytest.approx(pp.loss(off, dst, wt, T, W) - L0, rel=1e-9, abs=1e-14)


def test_gradient_identities():
    off, dst, w, T, W = _graph()
    gw, gT, L, _, _ = pp.adjoint_dense(off, dst, w, T, W)
    # L is linear in T: L = <dL/dT, T>
    assert np.sum(gT * T) == pytest.approx(L, rel=1e-12)
    # P is invariant to scaling one source's weights: sum_{e of u} w_e dL/dw_e = 0
    src = pp.sources(off)
    per_src = np.bincount(src, weights=w * gw, minlength=len(off) - 1)
    assert np.abs(per_src).max() <= 1e-12 * np.abs(w * gw).sum()
