"""The scale-up generator and pipeline at a small size: gbx_generate_chung_lu
(on the GPU) is deterministic, gives the requested mean out-degree, local
fraction and a power-law tail, writes host and device memory alike; and the
graph it makes goes through the CSR build, BFS, PageRank to epsilon 1e-6
and CC with the oracle's results (bit-exact levels and labels, PR within
1e-6 relative L1 of FP64)."""
import numpy as np
import pytest

from graphblox_gb300 import _lib
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

V, MEAN = 200_000, 30
E = V * MEAN


@pytest.fixture(scope="module")
def edges(gbx, cuda_device):
    return gbx.generate_chung_lu(V, E, 2.1, 4096, 0.7, seed=5)


def test_generator_properties(gbx, cuda_device, edges):
    torch = pytest.importorskip("torch")
    s, d = edges
    assert s.max() < V and d.max() < V
    s2, d2 = gbx.generate_chung_lu(V, E, 2.1, 4096, 0.7, seed=5)
    np.testing.assert_array_equal(s, s2)
    np.testing.assert_array_equal(d, d2)
    ts = torch.empty(E, dtype=torch.int32, device="cuda:0")
    td = torch.empty(E, dtype=torch.int32, device="cuda:0")
    gbx.generate_chung_lu(V, E, 2.1, 4096, 0.7, seed=5, src=ts, dst=td)
    np.testing.assert_array_equal(ts.cpu().numpy().view(np.uint32), s)
    np.testing.assert_array_equal(td.cpu().numpy().view(np.uint32), d)
    # 70% local draws plus the global draws that land in the same window
    same = (s // 4096) == (d // 4096)
    assert 0.69 <= same.mean() <= 0.75
    deg = np.bincount(s, minlength=V)
    assert deg.mean() == MEAN
    assert np.sqrt(E) / 4 <= deg.max() <= 4 * np.sqrt(E)
    # heavy tail: the top 1% of vertices hold well over 1% of the edges
    top = np.sort(deg)[::-1][: V // 100].sum() / E
    assert top > 0.1
    with pytest.raises(_lib.GbxError):
        gbx.generate_chung_lu(V, E, 1.5, 4096, 0.7)


def test_pipeline_matches_oracle(gbx, cuda_device, edges):
    s, d = edges
    el = gbx.EdgeList(V, s, d)
    g = gbx.graph_csr_preprocessing(el, sort=0, directed=True, keep_weights=False)
    host = po.HostCSR(V, g.out_degree, g.edges_idx, g.dest)
    pull = po.HostCSR(V, g.inverse_out_degree, g.inverse_edges_idx, g.inverse_dest)
    rng = np.random.default_rng(1)
    roots = rng.choice(np.nonzero(g.out_degree)[0], 2, replace=False)
    with gbx.DeviceGraph.from_graph_csr(g, use_weights=False) as dg:
        dg.label_array = None
        for r in roots:
            st = gbx.breadth_first_search(dg, int(r), 2)
            dref, _, proc, it = po.bfs(host, int(r), pull)
            np.testing.assert_array_equal(st.distances, dref)
            assert (st.processed_nodes, st.iteration) == (proc, it)
        pr = gbx.page_rank(dg, 1000, 1e-6)
        n = pr.iterations + 1 if pr.iterations < 1000 else 1000
        r64, _, _ = po.pagerank(host, n, 0.0, pull, fp64=True)
        ok, err, _ = po.fp32_close(pr.pageRanks, r64, 1e-6)
        assert ok, err
    sym = gbx.EdgeList(V, np.concatenate([s, d]), np.concatenate([d, s]))
    gsym = gbx.graph_csr_preprocessing(sym, sort=0, directed=False, keep_weights=False)
    with gbx.DeviceGraph.from_graph_csr(gsym, use_weights=False) as dgs:
        comp, _ = gbx.connected_components(dgs, 1)
    cref = po.cc(po.HostCSR(V, gsym.out_degree, gsym.edges_idx, gsym.dest))
    np.testing.assert_array_equal(comp, cref)
