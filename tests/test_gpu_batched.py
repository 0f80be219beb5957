"""Batched BFS and PageRank (gbx_bfs_batched / gbx_pr_batched): every graph
of a packed batch against the oracle run on that graph alone (BFS distances,
processed_nodes and iteration bit-exact; PageRank within 1e-6 relative L1 of
FP64) and against the single-graph GPU entry points. Covers graphs beyond the
shared-memory capacities (the global-scratch path), one-vertex and edgeless
graphs, repeated edges and self loops, undirected batches, and the input
checks."""
import numpy as np
import pytest

from graphblox_gb300 import _lib
from graphblox_gb300 import graph as gg
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def _host_csr(V, off, dest):
    off = off.astype(np.int64)
    return po.HostCSR(V, np.diff(off).astype(np.uint32), off[:-1].astype(np.uint32), dest)


def _check_parents(V, off, dest, dist, par, src, proc):
    reached = (dist > 0)
    reached[src] = True
    assert int(reached.sum()) == proc
    assert par[src] == src
    deg = np.diff(off.astype(np.int64))
    un = ~reached
    np.testing.assert_array_equal(par[un], np.where(deg[un] > 0, -deg[un], -1))
    vs = np.nonzero(reached)[0]
    vs = vs[vs != src]
    ps = par[vs].astype(np.int64)
    assert ((ps >= 0) & (ps < V)).all()
    np.testing.assert_array_equal(dist[ps].astype(np.int64) + 1, dist[vs])
    # every (parent, child) pair is an edge
    edge_keys = np.repeat(np.arange(V, dtype=np.int64), deg) * V + dest.astype(np.int64)
    assert np.isin(ps * V + vs, edge_keys).all()


def _graphs():
    gl = gg.generate_rmat_batch(48, seed=3, scale_lo=4, scale_hi=11, ef_lo=2, ef_hi=16)
    rng = np.random.default_rng(1)
    gl.append((1, np.zeros(0, np.uint32), np.zeros(0, np.uint32)))             # one vertex, no edges
    gl.append((5, np.zeros(0, np.uint32), np.zeros(0, np.uint32)))             # edgeless
    gl.append((4, np.array([0, 0, 1, 2, 2], np.uint32), np.array([1, 1, 2, 2, 3], np.uint32)))  # repeats, loop
    chain = np.arange(699, dtype=np.uint32)
    gl.append((700, chain, chain + 1))                                          # 700 levels
    star = np.zeros(3000, np.uint32)
    gl.append((3001, np.concatenate([star, np.arange(1, 3001, dtype=np.uint32)]),
               np.concatenate([np.arange(1, 3001, dtype=np.uint32), star])))    # hub, both directions
    # beyond both shared-memory capacities (131072-vertex bitmaps, 53248 PR contributions)
    s, d = gg.generate_rmat(18, 1 << 20, seed=9)
    gl.append((1 << 18, s, d))
    gl.append((60000, rng.integers(0, 60000, 400000).astype(np.uint32),
               rng.integers(0, 60000, 400000).astype(np.uint32)))
    return gl


@pytest.fixture(scope="module")
def packed():
    return gg.pack_graphs(_graphs())


def test_batched_bfs_matches_oracle_and_single_graph(gbx, cuda_device, packed):
    G = packed.num_graphs
    rng = np.random.default_rng(7)
    sources = np.array([0 if g % 3 else int(rng.integers(0, packed.graph(g)[0])) for g in range(G)], np.uint32)
    with gg.GraphBatch(packed) as b:
        dist = np.zeros(b.num_vertices, np.uint32)
        par = np.zeros(b.num_vertices, np.int32)
        dist, par, res = b.bfs(sources, dist, par)
    vb = packed.vertex_base.astype(np.int64)
    for g in range(G):
        V, off, dest, ioff, isrc = packed.graph(g)
        sl = slice(vb[g], vb[g + 1])
        fwd, pull = _host_csr(V, off, dest), _host_csr(V, ioff, isrc)
        d_ref, _, proc, it = po.bfs(fwd, int(sources[g]), pull)
        np.testing.assert_array_equal(dist[sl], d_ref, err_msg=f"graph {g}")
        assert (res["processed_nodes"][g], res["iteration"][g]) == (proc, it), g
        assert res["depth"][g] + 2 == it
        _check_parents(V, off, dest, dist[sl], par[sl], int(sources[g]), proc)
        if g % 6 == 0 or V > 50000:
            with gg.DeviceGraph.from_offsets(V, off, dest, in_offsets=ioff, in_src=isrc) as dg:
                st = gg.breadth_first_search(dg, int(sources[g]), 2, map_source=False)
            np.testing.assert_array_equal(dist[sl], st.distances)
            assert (st.processed_nodes, st.iteration, st.edges_traversed) == \
                (res["processed_nodes"][g], res["iteration"][g], res["edges_traversed"][g])


@pytest.mark.parametrize("iters,eps", [(30, 0.0), (100, 1e-4)])
def test_batched_pagerank_matches_fp64(gbx, cuda_device, packed, iters, eps):
    with gg.GraphBatch(packed) as b:
        ranks, res = b.page_rank(iters, eps)
    vb = packed.vertex_base.astype(np.int64)
    worst = 0.0
    for g in range(packed.num_graphs):
        V, off, dest, ioff, isrc = packed.graph(g)
        sl = slice(vb[g], vb[g + 1])
        fwd, pull = _host_csr(V, off, dest), _host_csr(V, ioff, isrc)
        _, it32, _ = po.pagerank(fwd, iters, eps, pull)
        it = int(res["iterations"][g])
        # the stop test |delta| >= eps sits on a threshold, so FP32 sums in
        # another order may stop one iteration apart; ranks are then compared
        # with FP64 run for the GPU's own iteration count
        assert abs(it - it32) <= 1, (g, it, it32)
        n = it + 1 if (eps > 0 and it < iters) else iters
        r64, _, _ = po.pagerank(fwd, n, 0.0, pull, fp64=True)
        ok, err, _ = po.fp32_close(ranks[sl], r64, 1e-6)
        worst = max(worst, err)
        assert ok, (g, err)
    print(f"batched PR ({iters} its, eps {eps}): worst rel L1 vs FP64 {worst:.2e}")


def test_batched_undirected(gbx, cuda_device):
    gl = []
    for V, s, d in gg.generate_rmat_batch(16, seed=5, scale_lo=5, scale_hi=10):
        gl.append((V, np.concatenate([s, d]), np.concatenate([d, s])))
    p = gg.pack_graphs(gl, inverse=False)
    src = np.zeros(p.num_graphs, np.uint32)
    with gg.GraphBatch(p) as b:
        dist, _, res = b.bfs(src)
        ranks, pres = b.page_rank(20, 0.0)
    vb = p.vertex_base.astype(np.int64)
    for g in range(p.num_graphs):
        V, off, dest, _, _ = p.graph(g)
        h = _host_csr(V, off, dest)
        d_ref, _, proc, it = po.bfs(h, 0)
        np.testing.assert_array_equal(dist[vb[g]:vb[g + 1]], d_ref)
        assert (res["processed_nodes"][g], res["iteration"][g]) == (proc, it)
        r64, _, _ = po.pagerank(h, 20, 0.0, fp64=True)
        assert po.fp32_close(ranks[vb[g]:vb[g + 1]], r64, 1e-6)[0]


def test_batched_input_checks(gbx, cuda_device):
    vb = np.array([0, 3, 5], np.uint32)
    off = np.array([0, 1, 2, 2, 3, 3], np.uint32)
    dest = np.array([1, 2, 2], np.uint32)  # graph 1 has 2 vertices: local id 2 is out of range
    h = _lib.vp()
    with pytest.raises(_lib.GbxError) as ei:
        _lib.call("gbx_batch_create", _lib.C.byref(h), 2, vb.ctypes.data, off.ctypes.data, dest.ctypes.data,
                  None, None, None)
    assert ei.value.status == -1
    dest[2] = 1
    # directed: the in-edge CSR in the same packing (0->1, 1->2 | 0->1)
    p = gg.PackedGraphs(vb, off, dest, np.array([0, 0, 1, 2, 2, 3], np.uint32), np.array([0, 1, 0], np.uint32))
    with gg.GraphBatch(p) as b:
        with pytest.raises(_lib.GbxError) as ei:
            b.bfs(np.array([0, 2], np.uint32))
        assert ei.value.status == -1
        d, _, res = b.bfs(np.array([0, 1], np.uint32))
        np.testing.assert_array_equal(d, [0, 1, 2, 0, 0])
        assert list(res["processed_nodes"]) == [3, 1]
