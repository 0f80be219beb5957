"""Personalised PageRank forward and hand-written adjoint on the GPU
(gbx_ppr_forward / gbx_ppr_adjoint) against the FP64 oracle: the same number
of FP64 power-iteration sweeps, a dense FP64 solve, and FP64 central finite
differences (h = 1e-4) on 200 sampled edges of a 2,048-vertex graph (the
subgraph of an RMAT-20 edge list induced by vertices 0..2047). At full size
(RMAT-20, 2^24 edges, K = 64) the checks are size-independent identities.

Tolerances, written per check below:
  ranks vs FP64 with the same sweeps      relative L1 <= 1e-6 per column
  ranks vs the dense solve (converged)    relative L1 <= 5e-6 per column
  dL/dT vs the dense solve                relative L1 <= 1e-5
  dL/dw vs the dense solve                relative L1 <= 1e-4
  dL/dw vs central differences            |err| <= 1e-3 |fd| + 1e-4 max|fd|
"""
import numpy as np
import pytest

from graphblox_gb300 import _lib
from graphblox_gb300 import graph as gg
from oracle import ppr_oracle as pp

pytestmark = pytest.mark.gpu

D = 0.85
TOL = 1e-7


def _csr(V, src, dst):
    order = np.lexsort((dst, src))
    src, dst = src[order].astype(np.int64), dst[order].astype(np.uint32)
    off = np.zeros(V + 1, np.int64)
    np.add.at(off, src + 1, 1)
    return np.cumsum(off).astype(np.uint32), dst


def _device(V, off, dst):
    return gg.DeviceGraph.from_offsets(V, np.ascontiguousarray(off, np.uint32), np.ascontiguousarray(dst, np.uint32))


@pytest.fixture(scope="module")
def sub2048():
    s, d = gg.generate_rmat(20, 1 << 24, seed=7)
    m = (s < 2048) & (d < 2048)
    V = 2048
    off, dst = _csr(V, s[m], d[m])
    w = gg.generate_values(len(dst), 3, seed=11)
    rng = np.random.default_rng(5)
    K = 64
    T = pp.seeds_teleport(V, K, 32, rng)
    W = rng.standard_normal((V, K)).astype(np.float32)
    return V, off, dst, w, T, W


def _rel_l1_cols(a, ref):
    return (np.abs(a - ref).sum(axis=0) / np.abs(ref).sum(axis=0)).max()


def test_ppr_forward_matches_fp64(gbx, cuda_device, sub2048):
    V, off, dst, w, T, W = sub2048
    with _device(V, off, dst) as dg:
        st = gg.ppr_forward(dg, w, T, D, TOL)
    assert st.residual < TOL and 10 < st.iterations < 1000
    R64, _, _ = pp.forward_iter(off, dst, w, T, D, iterations=st.iterations)
    err = _rel_l1_cols(st.ranks.astype(np.float64), R64)
    print(f"ppr forward: {st.iterations} sweeps, rel L1 vs FP64 same sweeps {err:.2e}")
    assert err <= 1e-6
    Rd = pp.forward_dense(off, dst, w, T, D)
    err_d = _rel_l1_cols(st.ranks.astype(np.float64), Rd)
    print(f"ppr forward: rel L1 vs dense solve {err_d:.2e}")
    assert err_d <= 5e-6


def test_ppr_adjoint_matches_dense_solve(gbx, cuda_device, sub2048):
    V, off, dst, w, T, W = sub2048
    with _device(V, off, dst) as dg:
        R = gg.ppr_forward(dg, w, T, D, TOL).ranks
        adj = gg.ppr_adjoint(dg, w, R, W, D, TOL)
    gw, gT, L, _, _ = pp.adjoint_dense(off, dst, w, T, W, D)
    e_t = np.abs(adj.grad_teleport - gT).sum() / np.abs(gT).sum()
    e_w = np.abs(adj.grad_weights - gw).sum() / np.abs(gw).sum()
    print(f"ppr adjoint: {adj.iterations} sweeps, dL/dT rel L1 {e_t:.2e}, dL/dw rel L1 {e_w:.2e}, "
          f"loss {adj.loss:.9g} vs {L:.9g}")
    assert adj.residual < TOL
    assert e_t <= 1e-5
    assert e_w <= 1e-4
    # the loss is the FP64 dot of the FP32 ranks given to the adjoint
    assert adj.loss == pytest.approx(float(np.sum(W.astype(np.float64) * R.astype(np.float64))), rel=1e-12)
    assert adj.loss == pytest.approx(L, rel=1e-5, abs=1e-7)


def test_ppr_adjoint_matches_central_differences(gbx, cuda_device, sub2048):
    V, off, dst, w, T, W = sub2048
    with _device(V, off, dst) as dg:
        R = gg.ppr_forward(dg, w, T, D, TOL).ranks
        adj = gg.ppr_adjoint(dg, w, R, W, D, TOL, want_teleport=False)
    fd = pp.FiniteDifference(off, dst, w, T, W, D)
    rng = np.random.default_rng(9)
    edges = rng.choice(len(dst), 200, replace=False)
    ref = np.array([fd.central(int(e), 1e-4) for e in edges])
    got = adj.grad_weights[edges].astype(np.float64)
    err = np.abs(got - ref)
    bound = 1e-3 * np.abs(ref) + 1e-4 * np.abs(ref).max()
    print(f"ppr dL/dw vs FD on 200 edges: max err {err.max():.2e}, max |fd| {np.abs(ref).max():.2e}, "
          f"worst err/bound {(err / bound).max():.3f}")
    assert (err <= bound).all()


def test_ppr_autograd_function(gbx, cuda_device, sub2048):
    torch = pytest.importorskip("torch")
    from ppr_binding import personalised_pagerank

    V, off, dst, w, T, W = sub2048
    dev = torch.device("cuda:0")
    with _device(V, off, dst) as dg:
        wt = torch.tensor(w, device=dev, requires_grad=True)
        Tt = torch.tensor(T, device=dev, requires_grad=True)
        Wt = torch.tensor(W, device=dev)
        R = personalised_pagerank(wt, Tt, dg, D, TOL)
        loss = (R.double() * Wt.double()).sum()
        loss.backward()
        direct = gg.ppr_adjoint(dg, w, R.detach().cpu().numpy(), W, D, TOL)
    np.testing.assert_array_equal(wt.grad.cpu().numpy(), direct.grad_weights)
    np.testing.assert_array_equal(Tt.grad.cpu().numpy(), direct.grad_teleport)
    assert float(loss.detach()) == pytest.approx(direct.loss, rel=1e-12)


@pytest.mark.parametrize("K", [32, 128, 256])
def test_ppr_multigraph_dangling_and_widths(gbx, cuda_device, K):
    """Repeated edges, self loops, vertices without out-edges and without
    in-edges, rows long enough to be split, and each supported K."""
    rng = np.random.default_rng(K)
    V = 3000
    src = np.concatenate([rng.integers(0, V, 40000), np.full(1500, 7), np.full(700, 11)])
    dst = np.concatenate([rng.integers(0, V, 40000), rng.integers(0, V, 1500), np.full(700, 12)])
    keep = (src % 97 != 5) & (dst % 89 != 3)  # some vertices with no out- / in-edges
    src, dst = src[keep], dst[keep]
    src = np.concatenate([src, [4, 4, 4]])
    dst = np.concatenate([dst, [4, 9, 9]])
    off, dst = _csr(V, src, dst)
    w = rng.lognormal(0, 1, len(dst)).astype(np.float32)
    T = pp.seeds_teleport(V, K, 32, rng)
    W = rng.standard_normal((V, K)).astype(np.float32)
    with _device(V, off, dst) as dg:
        st = gg.ppr_forward(dg, w, T, D, TOL)
        adj = gg.ppr_adjoint(dg, w, st.ranks, W, D, TOL)
    gw, gT, L, Rd, _ = pp.adjoint_dense(off, dst, w, T, W, D)
    assert _rel_l1_cols(st.ranks.astype(np.float64), Rd) <= 5e-6
    assert np.abs(adj.grad_teleport - gT).sum() / np.abs(gT).sum() <= 1e-5
    assert np.abs(adj.grad_weights - gw).sum() / np.abs(gw).sum() <= 1e-4


def test_ppr_errors(gbx, cuda_device, sub2048):
    V, off, dst, w, T, W = sub2048
    with _device(V, off, dst) as dg:
        with pytest.raises(_lib.GbxError) as ei:
            gg.ppr_forward(dg, w, T[:, :48].copy(), D, TOL)
        assert ei.value.status == -1
        with pytest.raises(_lib.GbxError) as ei:
            gg.ppr_forward(dg, w, T, D, TOL, max_iterations=3)
        assert ei.value.status == -4
        with pytest.raises(_lib.GbxError) as ei:
            gg.ppr_forward(dg, w, T, 1.0, TOL)
        assert ei.value.status == -1


def test_ppr_rmat20_k64_identities(gbx, cuda_device):
    """The differentiable-PPR workload at full size: RMAT-20, 2^24 edges as
    generated (repeats kept), lognormal(0,1) weights, 64 teleport columns of
    32 seeds each, W ~ N(0,1), d = 0.85 to 1e-7 L1."""
    torch = pytest.importorskip("torch")
    V, E = 1 << 20, 1 << 24
    s, d = gg.generate_rmat(20, E, seed=1)
    off, dst = _csr(V, s, d)
    w = gg.generate_values(E, 3, seed=2)
    rng = np.random.default_rng(3)
    T = pp.seeds_teleport(V, 64, 32, rng)
    W = rng.standard_normal((V, 64)).astype(np.float32)
    dev = torch.device("cuda:0")
    with _device(V, off, dst) as dg:
        wt, Tt, Wt = (torch.from_numpy(a).to(dev) for a in (w, T, W))
        st = gg.ppr_forward(dg, wt, Tt, D, TOL)
        adj = gg.ppr_adjoint(dg, wt, st.ranks, Wt, D, TOL)
        R = st.ranks.double().cpu().numpy()
        gw = adj.grad_weights.double().cpu().numpy()
        gT = adj.grad_teleport.double().cpu().numpy()
    assert st.residual < TOL and adj.residual < TOL
    # teleport mass: each column sums to at most 1 and is positive
    col = R.sum(axis=0)
    assert (col > 0).all() and (col <= 1 + 1e-5).all()
    # L = <dL/dT, T> (L is linear in T)
    assert np.sum(gT * T) == pytest.approx(adj.loss, rel=2e-5)
    # scale invariance of each source's weights: sum_{e of u} w_e dL/dw_e = 0
    src = pp.sources(off)
    per_src = np.bincount(src, weights=w.astype(np.float64) * gw, minlength=V)
    assert np.abs(per_src).sum() <= 1e-4 * np.abs(w * gw).sum()
    # two columns against FP64 power iteration with the same sweep count
    R64, _, _ = pp.forward_iter(off, dst, w, T[:, :2], D, iterations=st.iterations)
    err = _rel_l1_cols(R[:, :2], R64)
    print(f"rmat20 K=64: {st.iterations} forward / {adj.iterations} adjoint sweeps, rel L1 cols 0-1 {err:.2e}")
    assert err <= 1e-6
