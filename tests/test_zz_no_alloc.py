"""gbx_pagerank_pull_noalloc: pull PageRank for callers that cannot allocate.

Some hosts cannot call cudaMalloc once they are running: their own allocator
took all device memory at start-up, or they must not grow the CUDA heap
while they serve. They use this entry point; its working memory is a fixed
device array inside libgbx.so. The tests call it through the C ABI twice in
a row on the same inputs and check both results against the allocating
entry point, gbx_pagerank_pull, and against the oracle's FP64 restatement of
the reference's recurrence, within the 1e-6 relative-L1 tolerance used for
PageRank everywhere else; the result fields (iterations, active_last,
error_total) are checked against gbx_pagerank_pull's when both stop at the
same iteration, else against the stop rule itself. One case runs at the
array's maximum size, 4,194,304 vertices (RMAT scale 22). This file is
collected last so that a failure here comes after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

REL_L1_TOL = 1e-6
# error_total is a mean of FP32 rank differences reduced in FP64; two FP32
# summation orders move each difference by a few ulps of the ranks
ERROR_TOTAL_RTOL = 1e-4
MAX_VERTICES = 1 << 22


def _graph(gbx, scale, seed):
    src, dst = gbx.generate_rmat(scale, (1 << scale) * 16, seed=seed)
    el = gbx.EdgeList(1 << scale, src, dst)
    return gbx.graph_csr_preprocessing(el, sort=1, dedup=True, directed=True, keep_weights=False)


def _device_inputs(g, dev):
    import torch

    V = g.num_vertices
    in_off = np.zeros(V + 1, np.uint32)
    in_off[1:] = np.cumsum(g.inverse_out_degree, dtype=np.uint64).astype(np.uint32)
    return (torch.from_numpy(in_off.view(np.int32)).to(dev),
            torch.from_numpy(np.ascontiguousarray(g.inverse_dest).view(np.int32)).to(dev),
            torch.from_numpy(np.ascontiguousarray(g.out_degree).view(np.int32)).to(dev))


def _noalloc(gbx, lib, V, d_off, d_src, d_deg, iters, eps, dev):
    import torch

    out = torch.full((V,), -1.0, dtype=torch.float32, device=dev)
    res = gbx._lib.PrResult()
    st = lib.gbx_pagerank_pull_noalloc(V, d_off.data_ptr(), d_src.data_ptr(), d_deg.data_ptr(), iters, eps,
                                       out.data_ptr(), C.byref(res), torch.cuda.current_stream().cuda_stream)
    assert st == 0, lib.gbx_last_error().decode()
    return out.cpu().numpy(), res


def _check(gbx, g, dev, cases):
    lib = gbx.load()
    V = g.num_vertices
    host = po.HostCSR(V, g.out_degree, g.edges_idx, g.dest)
    pull = po.HostCSR(V, g.inverse_out_degree, g.inverse_edges_idx, g.inverse_dest)
    d_off, d_src, d_deg = _device_inputs(g, dev)
    with gbx.DeviceGraph.from_graph_csr(g) as dg:
        refs = {(eps, iters): gbx.page_rank(dg, iters, eps) for eps, iters in set(cases)}
    for eps, iters in cases:
        ref = refs[(eps, iters)]
        for call in range(2):  # two calls in a row share (and reuse) the scratch array
            got, res = _noalloc(gbx, lib, V, d_off, d_src, d_deg, iters, eps, dev)
            ok, err, _ = po.fp32_close(got, np.asarray(ref.pageRanks), REL_L1_TOL)
            assert ok, f"call {call}: rel L1 {err:.3e} against gbx_pagerank_pull (epsilon {eps})"
            # the oracle in FP64, run for the iterations this call executed
            executed = res.iterations + 1 if (eps > 0 and res.iterations < iters) else iters
            r64, _, _ = po.pagerank(host, executed, 0.0, pull, fp64=True)
            ok, err, _ = po.fp32_close(got, r64, REL_L1_TOL)
            assert ok, f"call {call}: rel L1 {err:.3e} against the FP64 oracle (epsilon {eps})"
            if res.iterations == ref.iterations:
                assert res.active_last == ref.active_last
                assert res.error_total == pytest.approx(ref.error_total, rel=ERROR_TOTAL_RTOL, abs=1e-30)
            else:
                # The stop test |delta| >= epsilon works at the FP32 resolution of
                # the largest ranks, so another summation order stops at another
                # iteration; this call must still have stopped for the stated
                # reason: nothing moved by epsilon in its last iteration.
                assert eps > 0 and res.iterations < iters and res.active_last == 0
                assert 0.0 <= res.error_total < eps


def test_noalloc_pagerank_matches_allocating_entry_point(gbx, cuda_device):
    g = _graph(gbx, 14, 21)
    _check(gbx, g, cuda_device, [(0.0, 20), (1e-4, 100), (0.0, 20)])


def test_noalloc_pagerank_at_the_array_limit(gbx, cuda_device):
    """RMAT-22: exactly the largest vertex count the scratch array holds."""
    g = _graph(gbx, 22, 1)
    assert g.num_vertices == MAX_VERTICES
    _check(gbx, g, cuda_device, [(0.0, 20), (1e-4, 200)])


def test_noalloc_rejects_sizes_beyond_its_array(gbx, cuda_device):
    import torch

    lib = gbx.load()
    buf = torch.zeros(8, dtype=torch.int32, device=cuda_device)
    p = buf.data_ptr()
    st = lib.gbx_pagerank_pull_noalloc(MAX_VERTICES + 1, p, p, p, 20, 0.0, p, None, None)
    assert st == -1 and b"at most" in lib.gbx_last_error()
    st = lib.gbx_pagerank_pull_noalloc(4, p, p, p, 5000, 0.0, p, None, None)
    assert st == -1 and b"at most" in lib.gbx_last_error()
