"""The single-step BFS entry points (the reference's topDownStepGraphCSR and
bottomUpStepGraphCSR, BFS.c:498-613) on the GPU: traversals driven step by
step from the host -- all top-down, all bottom-up, and the reference's
direction-optimising schedule -- reach the oracle's BFS levels exactly; mf
is the reference's sum of -parent over the claimed vertices; every top-down
parent is an in-neighbour one level up, and bottom-up parents are the first
frontier in-neighbour in pull order, as in the reference. The drop-in's
exported symbols are called with the reference's ArrayQueue / Bitmap
structs."""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as po
from test_gpu_integration import BFSStats, Built, _p
from conftest import load_golden

pytestmark = pytest.mark.gpu

u32 = C.c_uint32


def _graph(gbx, scale=13, seed=4):
    V = 1 << scale
    s, d = gbx.generate_rmat(scale, V * 12, seed=seed)
    g = gbx.graph_csr_preprocessing(gbx.EdgeList(V, s, d), sort=1, dedup=True, directed=True, keep_weights=False)
    return V, g


def _init(g, src):
    V = g.num_vertices
    par = np.where(g.out_degree > 0, -g.out_degree.astype(np.int64), -1).astype(np.int32)
    par[src] = src
    return par, np.zeros(V, np.uint32)


def _td(gbx, dg, frontier, par, dist):
    V = dg.num_vertices
    nxt = np.zeros(V, np.uint32)
    n, mf = u32(0), u32(0)
    gbx._lib.call("gbx_bfs_top_down_step", dg.handle, frontier.ctypes.data, len(frontier), par.ctypes.data,
             dist.ctypes.data, nxt.ctypes.data, V, C.byref(n), C.byref(mf), None)
    return nxt[:n.value].copy(), mf.value


def _bu(gbx, dg, bm, par, dist):
    nxt = np.zeros_like(bm)
    nf = u32(0)
    gbx._lib.call("gbx_bfs_bottom_up_step", dg.handle, bm.ctypes.data, nxt.ctypes.data, par.ctypes.data,
             dist.ctypes.data, C.byref(nf), None)
    return nxt, nf.value


def _bits(V, vs):
    bm = np.zeros((V + 31) // 32, np.uint32)
    np.bitwise_or.at(bm, np.asarray(vs, np.int64) >> 5, (np.uint32(1) << (np.asarray(vs, np.uint32) & 31)))
    return bm


def _members(V, bm):
    return np.nonzero(np.unpackbits(bm.view(np.uint8), bitorder="little")[:V])[0].astype(np.uint32)


def _oracle_levels(g, src):
    V = g.num_vertices
    host = po.HostCSR(V, g.out_degree, g.edges_idx, g.dest)
    pull = po.HostCSR(V, g.inverse_out_degree, g.inverse_edges_idx, g.inverse_dest)
    return po.bfs(host, src, pull)[0]


@pytest.mark.parametrize("schedule", ["push", "pull", "direction_optimising"])
def test_step_by_step_traversal_matches_oracle(gbx, cuda_device, schedule):
    V, g = _graph(gbx)
    src = int(np.argmax(g.out_degree))
    want = _oracle_levels(g, src)
    deg = g.out_degree.astype(np.int64)
    with gbx.DeviceGraph.from_graph_csr(g, use_weights=False) as dg:
        par, dist = _init(g, src)
        frontier = np.array([src], np.uint32)
        bu = schedule == "pull"
        mu, mf = g.num_edges, int(deg[src])
        for _ in range(64):
            if len(frontier) == 0:
                break
            if schedule == "direction_optimising":
                bu = mf > mu // 15  # the reference's alpha switch (BFS.c:374-402)
            if bu:
                nxt_bm, nf = _bu(gbx, dg, _bits(V, frontier), par, dist)
                new = _members(V, nxt_bm)
                assert nf == len(new)
                mf = int(np.maximum(deg[new], 1).sum())
            else:
                before = par.copy()
                new, mf = _td(gbx, dg, frontier, par, dist)
                mu -= mf
                assert len(np.unique(new)) == len(new)
                assert mf == int((-before[new].astype(np.int64)).sum())
            frontier = new
        assert len(frontier) == 0
    np.testing.assert_array_equal(dist, want)
    # parents: the source keeps itself; every reached vertex's parent is an
    # in-neighbour one level up; unreached vertices keep their negative marker
    reached = np.nonzero((dist > 0))[0]
    p = par[reached].astype(np.int64)
    assert np.all(p >= 0) and np.all(dist[p] + 1 == dist[reached])
    adj = set(zip(g.src.tolist(), g.dest.tolist()))
    assert all((int(a), int(b)) in adj for a, b in zip(p[:2000], reached[:2000]))


def test_bottom_up_parent_is_first_frontier_in_neighbour(gbx, cuda_device):
    V, g = _graph(gbx, 12, 9)
    src = int(np.argmax(g.out_degree))
    with gbx.DeviceGraph.from_graph_csr(g, use_weights=False) as dg:
        par, dist = _init(g, src)
        frontier, _ = _td(gbx, dg, np.array([src], np.uint32), par, dist)
        bm = _bits(V, frontier)
        before = par.copy()
        _, nf = _bu(gbx, dg, bm, par, dist)
    inb = set(frontier.tolist())
    found = 0
    for v in range(V):
        if before[v] >= 0:
            continue
        b, n = int(g.inverse_edges_idx[v]), int(g.inverse_out_degree[v])
        first = next((int(u) for u in g.inverse_dest[b:b + n] if int(u) in inb), None)
        if first is None:
            assert par[v] == before[v]
        else:
            found += 1
            assert par[v] == first and dist[v] == 2
    assert found == nf


def test_step_rejects_out_of_range_frontier(gbx, cuda_device):
    V, g = _graph(gbx, 10, 3)
    with gbx.DeviceGraph.from_graph_csr(g, use_weights=False) as dg:
        par, dist = _init(g, 0)
        with pytest.raises(RuntimeError):
            _td(gbx, dg, np.array([V + 5], np.uint32), par, dist)


class Bitmap(C.Structure):  # 01_host/include/structures/bitmap.h:23-30
    _fields_ = [("real_size", u32), ("size", u32), ("numSetBits", u32), ("bitarray", C.POINTER(u32))]


class ArrayQueue(C.Structure):  # 01_host/include/structures/arrayQueue.h:11-20
    _fields_ = [("head", u32), ("tail", u32), ("tail_next", u32), ("size", u32), ("queue", C.POINTER(u32)),
                ("q_bitmap", C.POINTER(Bitmap)), ("q_bitmap_next", C.POINTER(Bitmap))]


def test_dropin_step_symbols(gbx):
    """topDownStepGraphCSR / bottomUpStepGraphCSR of the drop-in, with the
    reference's structs: one top-down step from the source, then one
    bottom-up step, against the oracle's levels 1 and 2."""
    import graphblox_gb300._build as b

    lib = C.CDLL(str(b.PKG / "libgbx_graphblox_dw.so"))
    lib.topDownStepGraphCSR.restype = u32
    lib.bottomUpStepGraphCSR.restype = u32
    lib.newBFSStatsGraphCSR.restype = C.c_void_p
    fx = load_golden("v1000_e10000")
    bg = Built(fx, "dw", directed=True)
    V = bg.V
    src = int(np.argmax(fx["dw_out_degree"]))
    sp = C.cast(lib.newBFSStatsGraphCSR(C.byref(bg.g)), C.POINTER(BFSStats))
    stats = sp.contents
    stats.parents[src] = src
    qbuf = np.zeros(V, np.uint32)
    qbuf[0] = src
    q = ArrayQueue(0, 1, 1, V, _p(qbuf), None, None)
    mf = lib.topDownStepGraphCSR(C.byref(bg.g), C.byref(q), None, sp)
    n1 = q.tail_next - 1
    lvl1 = qbuf[1:1 + n1]
    host = po.HostCSR(V, fx["dw_out_degree"], fx["dw_edges_idx"], fx["dw_dest"])
    inv = po.build_csr(V, fx["dw_dest"], fx["dw_src"], None, sort_mode=1)
    want = po.bfs(host, src, inv)[0]
    assert sorted(lvl1.tolist()) == sorted(np.nonzero(want == 1)[0].tolist())
    deg = fx["dw_out_degree"].astype(np.int64)
    assert mf == int(np.maximum(deg[lvl1], 1).sum())
    words = (V + 31) // 32
    cur, nxt = _bits(V, lvl1), np.zeros(words, np.uint32)
    bc = Bitmap(V, words, 0, _p(cur))
    bn = Bitmap(V, words, 0, _p(nxt))
    nf = lib.bottomUpStepGraphCSR(C.byref(bg.g), C.byref(bc), C.byref(bn), sp)
    lvl2 = _members(V, nxt)
    assert nf == len(lvl2) and sorted(lvl2.tolist()) == sorted(np.nonzero(want == 2)[0].tolist())
    dist = np.ctypeslib.as_array(stats.distances, shape=(V,))
    assert np.all(dist[lvl2] == 2) and np.all(dist[lvl1] == 1)
    lib.freeBFSStats(sp)
