"""gbx_pagerank_pull_noalloc: pull PageRank for callers that cannot allocate.

Callers that cannot call cudaMalloc (code inside stream capture, hosts whose
allocator owns all device memory) use this entry point; its working memory
is a fixed device array inside libgbx.so. The test calls it through the C
ABI twice in a row on the same inputs and checks both results against the
allocating entry point, gbx_pagerank_pull, within the 1e-6 relative-L1
tolerance used for PageRank everywhere else. This file is collected last so
that a failure here comes after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

REL_L1_TOL = 1e-6


def _graph(gbx):
    scale = 14
    src, dst = gbx.generate_rmat(scale, (1 << scale) * 16, seed=21)
    el = gbx.EdgeList(1 << scale, src, dst)
    return gbx.graph_csr_preprocessing(el, sort=1, dedup=True, directed=True, keep_weights=False)


def test_noalloc_pagerank_matches_allocating_entry_point(gbx, cuda_device):
    import torch

    lib = gbx.load()
    g = _graph(gbx)
    V = g.num_vertices
    in_off = np.zeros(V + 1, np.uint32)
    in_off[1:] = np.cumsum(g.inverse_out_degree, dtype=np.uint64).astype(np.uint32)
    d_off = torch.from_numpy(in_off.view(np.int32)).to(cuda_device)
    d_src = torch.from_numpy(np.ascontiguousarray(g.inverse_dest).view(np.int32)).to(cuda_device)
    d_deg = torch.from_numpy(np.ascontiguousarray(g.out_degree).view(np.int32)).to(cuda_device)
    with gbx.DeviceGraph.from_graph_csr(g) as dg:
        ref = gbx.page_rank(dg, 20, 0.0).pageRanks
        ref_eps = gbx.page_rank(dg, 100, 1e-4)
    for eps, iters, expect in ((0.0, 20, ref), (1e-4, 100, ref_eps.pageRanks), (0.0, 20, ref)):
        for _ in range(2):  # two calls in a row share (and reuse) the scratch array
            out = torch.full((V,), -1.0, dtype=torch.float32, device=cuda_device)
            res = gbx._lib.PrResult()
            st = lib.gbx_pagerank_pull_noalloc(V, d_off.data_ptr(), d_src.data_ptr(), d_deg.data_ptr(), iters,
                                               eps, out.data_ptr(), C.byref(res),
                                               torch.cuda.current_stream().cuda_stream)
            assert st == 0, lib.gbx_last_error().decode()
            got = out.cpu().numpy()
            ok, err, _ = po.fp32_close(got, expect, REL_L1_TOL)
            assert ok, f"rel L1 {err:.3e} against gbx_pagerank_pull (epsilon {eps})"
            if eps > 0:
                assert res.iterations == ref_eps.iterations


def test_noalloc_rejects_sizes_beyond_its_array(gbx, cuda_device):
    import torch

    lib = gbx.load()
    buf = torch.zeros(8, dtype=torch.int32, device=cuda_device)
    p = buf.data_ptr()
    st = lib.gbx_pagerank_pull_noalloc((1 << 22) + 1, p, p, p, 20, 0.0, p, None, None)
    assert st == -1 and b"at most" in lib.gbx_last_error()
    st = lib.gbx_pagerank_pull_noalloc(4, p, p, p, 5000, 0.0, p, None, None)
    assert st == -1 and b"at most" in lib.gbx_last_error()
