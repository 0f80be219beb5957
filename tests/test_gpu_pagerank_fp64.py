"""gbx_pagerank_pull_fp64, the FP64 yardstick the large-graph PageRank error
is reported against: it equals the oracle's FP64 restatement of the
reference's recurrence to 1e-12 relative L1 -- on RMAT graphs, on a star
whose hub row spans many warps' edge ranges, on rows left empty, and on a
graph without edges."""
import numpy as np
import pytest

from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def _fp64(gbx, g, iters):
    out = np.zeros(g.num_vertices, np.float64)
    with gbx.DeviceGraph.from_graph_csr(g, use_weights=False) as dg:
        gbx._lib.call("gbx_pagerank_pull_fp64", dg.handle, iters, out.ctypes.data, None)
    return out


def _oracle(g, iters):
    V = g.num_vertices
    host = po.HostCSR(V, g.out_degree, g.edges_idx, g.dest)
    pull = po.HostCSR(V, g.inverse_out_degree, g.inverse_edges_idx, g.inverse_dest)
    return po.pagerank(host, iters, 0.0, pull, fp64=True)[0]


def _build(gbx, V, s, d):
    return gbx.graph_csr_preprocessing(gbx.EdgeList(V, np.asarray(s, np.uint32), np.asarray(d, np.uint32)),
                                       sort=1, dedup=True, directed=True, keep_weights=False)


@pytest.mark.parametrize("scale,iters", [(10, 1), (14, 20), (16, 50)])
def test_rmat(gbx, cuda_device, scale, iters):
    V = 1 << scale
    s, d = gbx.generate_rmat(scale, V * 16, seed=scale)
    g = _build(gbx, V, s, d)
    got, want = _fp64(gbx, g, iters), _oracle(g, iters)
    assert po.rel_l1(got, want) <= 1e-12


def test_star_and_empty_rows(gbx, cuda_device):
    V = 100_000
    hub = 7
    s = np.concatenate([np.arange(V), np.full(V // 2, hub)])
    d = np.concatenate([np.full(V, hub), np.arange(0, V, 2)])
    g = _build(gbx, V, s, d)
    got, want = _fp64(gbx, g, 30), _oracle(g, 30)
    assert po.rel_l1(got, want) <= 1e-12


def test_no_edges(gbx, cuda_device):
    g = _build(gbx, 5, [], [])
    got = _fp64(gbx, g, 10)
    np.testing.assert_allclose(got, np.full(5, float(np.float32(1) - np.float32(0.85)) / 5), rtol=1e-15)
