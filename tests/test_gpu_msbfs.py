"""Multi-source bitmask BFS (gbx_bfs_multisource) against the oracle's BFS
from every source alone: distances, processed_nodes and iteration bit-exact,
edges_traversed equal to the single-source GPU BFS. Covers 1, 33, 100 and
256 sources, repeated sources, sources without out-edges, undirected graphs
(pull over the forward CSR), hub rows cut into chunks, traversals deeper than
the 32 level masks kept for the final pass (a long chain), and bad sources."""
import numpy as np
import pytest

from graphblox_gb300 import _lib
from oracle import pyoracle as po
from test_gpu_parity import _rmat_graph, host_views

pytestmark = pytest.mark.gpu


def _sources(g, n, seed):
    rng = np.random.default_rng(seed)
    nz = np.nonzero(g.out_degree)[0]
    src = rng.choice(nz, n, replace=False).astype(np.uint32)
    zero = np.nonzero(g.out_degree == 0)[0]
    if n >= 4:
        src[1] = src[0]                      # a repeated source
        if len(zero):
            src[2] = zero[0]                 # a source without out-edges
    return src


@pytest.mark.parametrize("n", [1, 33, 100, 256])
def test_multisource_directed_matches_oracle(gbx, cuda_device, n):
    g = _rmat_graph(gbx, 14, 16, 3)
    host, pull = host_views(g)
    src = _sources(g, n, n)
    with gbx.DeviceGraph.from_graph_csr(g) as dg:
        dg.label_array = None
        dist, res = gbx.bfs_multisource(dg, src)
        singles = [gbx.breadth_first_search(dg, int(s), 2) for s in src[:4]]
    assert dist.shape == (g.num_vertices, n)
    for i, s in enumerate(src):
        d_ref, _, proc, it = po.bfs(host, int(s), pull)
        np.testing.assert_array_equal(dist[:, i], d_ref, err_msg=f"source {i} ({s})")
        assert (res["processed_nodes"][i], res["iteration"][i]) == (proc, it), i
    for i, st in enumerate(singles):
        assert res["edges_traversed"][i] == st.edges_traversed


def test_multisource_undirected_and_hubs(gbx, cuda_device):
    g = _rmat_graph(gbx, 15, 16, 4, symmetric=True)
    assert int(g.out_degree.max()) > 1024  # hub rows are cut into chunks
    host, _ = host_views(g)
    src = _sources(g, 64, 9)
    src[5] = int(np.argmax(g.out_degree))  # the largest hub as a source
    with gbx.DeviceGraph.from_graph_csr(g, use_weights=False) as dg:
        dg.label_array = None
        dist, res = gbx.bfs_multisource(dg, src)
    for i, s in enumerate(src):
        d_ref, _, proc, it = po.bfs(host, int(s))
        np.testing.assert_array_equal(dist[:, i], d_ref, err_msg=f"source {i}")
        assert (res["processed_nodes"][i], res["iteration"][i]) == (proc, it)


def test_multisource_device_output_and_checks(gbx, cuda_device):
    torch = pytest.importorskip("torch")
    g = _rmat_graph(gbx, 12, 8, 5)
    src = _sources(g, 40, 2)
    with gbx.DeviceGraph.from_graph_csr(g) as dg:
        dg.label_array = None
        host_dist, _ = gbx.bfs_multisource(dg, src)
        dev = torch.zeros((g.num_vertices, 40), dtype=torch.int32, device="cuda:0")
        gbx.bfs_multisource(dg, src, distances=dev)
        np.testing.assert_array_equal(dev.cpu().numpy().view(np.uint32), host_dist)
        bad = src.copy()
        bad[7] = g.num_vertices
        with pytest.raises(_lib.GbxError) as ei:
            gbx.bfs_multisource(dg, bad)
        assert ei.value.status == -1
        with pytest.raises(_lib.GbxError) as ei:
            gbx.bfs_multisource(dg, np.zeros(257, np.uint32))
        assert ei.value.status == -1


@pytest.mark.parametrize("n", [5, 64, 256])
def test_multisource_deeper_than_the_stored_levels(gbx, cuda_device, n):
    """An RMAT-10 graph with a 90-vertex chain hanging off vertex 0 (and a
    shortcut into its middle): sources near the chain's start run past the
    32 stored level masks, so their late levels take the bit-by-bit path."""
    V0, chain = 1 << 10, 90
    src, dst = gbx.generate_rmat(10, V0 * 8, seed=12)
    c = np.arange(V0, V0 + chain, dtype=np.uint32)
    src = np.concatenate([src, [0], c[:-1], [c[10]]]).astype(np.uint32)
    dst = np.concatenate([dst, [c[0]], c[1:], [c[60]]]).astype(np.uint32)
    el = gbx.EdgeList(V0 + chain, src, dst)
    g = gbx.graph_csr_preprocessing(el, sort=1, dedup=True, directed=True, keep_weights=False)
    host, pull = host_views(g)
    rng = np.random.default_rng(n)
    srcs = np.concatenate([[0, V0, V0 + 5, V0 + 40], rng.choice(np.nonzero(g.out_degree)[0], n - 4)])
    srcs = srcs[:n].astype(np.uint32)
    with gbx.DeviceGraph.from_graph_csr(g) as dg:
        dg.label_array = None
        dist, res = gbx.bfs_multisource(dg, srcs)
    assert int(dist.max()) > 40
    for i, s0 in enumerate(srcs):
        d_ref, _, proc, it = po.bfs(host, int(s0), pull)
        np.testing.assert_array_equal(dist[:, i], d_ref, err_msg=f"source {i} ({s0})")
        assert (res["processed_nodes"][i], res["iteration"][i]) == (proc, it), i
