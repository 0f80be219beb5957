"""gbx_graph_create_csr / gbx_graph_create_offsets: a graph's upload enqueues
every copy of both directions before it checks either, then validates the
layout on the device. Covers the errors those checks report once the copies
are in flight (degree sum, runs past E, decreasing offsets, a failing
inverse after a good forward direction, in_src NULL), a weighted CSR whose
runs are out of vertex order (gathered into offset order on the device) with
SSSP, BFS and PageRank equal to the same graph given in vertex order, and a
graph without edges."""
import ctypes as C

import numpy as np
import pytest

from graphblox_gb300 import _lib
from test_gpu_parity import _rmat_graph

pytestmark = pytest.mark.gpu


def _u32(a):
    return np.ascontiguousarray(a, np.uint32)


def _create(gbx, V, E, idx, deg, dest, w=None, in_idx=None, in_deg=None, in_src=None, in_w=None):
    lib = gbx.load()
    keep = [None if a is None else np.ascontiguousarray(a) for a in (idx, deg, dest, w, in_idx, in_deg, in_src, in_w)]
    ptrs = [None if a is None else a.ctypes.data for a in keep]
    h = C.c_void_p()
    st = lib.gbx_graph_create_csr(C.byref(h), V, E, *ptrs, None)
    err = lib.gbx_last_error()
    if st == 0:
        lib.gbx_graph_destroy(h)
    return st, err


def test_create_reports_layout_errors(gbx, cuda_device):
    ok = dict(idx=_u32([0, 1]), deg=_u32([1, 1]), dest=_u32([1, 0]))
    assert _create(gbx, 2, 2, **ok)[0] == 0
    st, err = _create(gbx, 3, 3, _u32([0, 1, 2]), _u32([1, 1, 0]), _u32([1, 2, 0]))
    assert st == -1 and b"sum of degrees" in err
    st, err = _create(gbx, 2, 2, _u32([0, 2]), _u32([1, 1]), _u32([1, 0]))
    assert st == -1 and b"exceeds num_edges" in err
    # a good forward direction, then an inverse whose degrees do not sum to E
    st, err = _create(gbx, 2, 2, **ok, in_idx=_u32([0, 1]), in_deg=_u32([1, 0]), in_src=_u32([1, 0]))
    assert st == -1 and b"sum of degrees" in err
    st, err = _create(gbx, 2, 2, **ok, in_idx=_u32([0, 1]), in_deg=_u32([1, 1]))
    assert st == -1 and b"in_src is NULL" in err
    with pytest.raises(_lib.GbxError) as ei:
        gbx.DeviceGraph.from_offsets(3, _u32([0, 2, 1, 2]), _u32([1, 2]))
    assert ei.value.status == -1 and "non-decreasing" in str(ei.value)
    # the same device serves a good graph after the failures
    with gbx.DeviceGraph.from_offsets(3, _u32([0, 1, 2, 2]), _u32([1, 2])) as dg:
        st = gbx.breadth_first_search(dg, 0, 1)
        np.testing.assert_array_equal(st.distances, [0, 1, 2])


def _shuffle_runs(g, seed):
    """The same CSR with its rows' runs stored in a random order (edges_idx
    points at each run), forward and inverse."""
    rng = np.random.default_rng(seed)

    def shuffle(deg, idx, ids, w):
        V = deg.shape[0]
        order = rng.permutation(V)
        new_idx = np.zeros(V, np.uint32)
        pos = 0
        parts_i, parts_w = [], []
        for v in order:
            d = int(deg[v])
            new_idx[v] = pos
            parts_i.append(ids[idx[v]: idx[v] + d])
            if w is not None:
                parts_w.append(w[idx[v]: idx[v] + d])
            pos += d
        new_ids = np.concatenate(parts_i).astype(np.uint32)
        new_w = None if w is None else np.concatenate(parts_w).astype(np.float32)
        return new_idx, new_ids, new_w

    i, d, w = shuffle(g.out_degree, g.edges_idx, g.dest, g.weight)
    ii, idst, iw = shuffle(g.inverse_out_degree, g.inverse_edges_idx, g.inverse_dest, g.inverse_weight)
    return type(g)(g.num_vertices, g.num_edges, g.out_degree, i, d, g.src, w, g.label_array,
                   g.inverse_label_array, g.inverse_out_degree, ii, idst, iw)


def test_runs_out_of_vertex_order_are_gathered(gbx, cuda_device):
    g = _rmat_graph(gbx, 11, 8, 21, weights="int")
    gsh = _shuffle_runs(g, 5)
    assert np.any(np.diff(gsh.edges_idx[g.out_degree > 0].astype(np.int64)) < 0)
    roots = [int(r) for r in np.nonzero(g.out_degree)[0][:3]]
    with gbx.DeviceGraph.from_graph_csr(g) as a, gbx.DeviceGraph.from_graph_csr(gsh) as b:
        a.label_array = b.label_array = None
        for r in roots:
            sa, sb = gbx.sssp(a, r), gbx.sssp(b, r)
            np.testing.assert_array_equal(sa.distances, sb.distances)
            assert sa.edges_traversed == sb.edges_traversed
            ba, bb = gbx.breadth_first_search(a, r, 0), gbx.breadth_first_search(b, r, 0)
            np.testing.assert_array_equal(ba.distances, bb.distances)
        pa, pb = gbx.page_rank(a, 10, 0.0), gbx.page_rank(b, 10, 0.0)
        np.testing.assert_array_equal(pa.pageRanks, pb.pageRanks)


def test_graph_without_edges(gbx, cuda_device):
    V = 5
    z = np.zeros(V, np.uint32)
    assert _create(gbx, V, 0, z, z, np.zeros(1, np.uint32))[0] == 0
    with gbx.DeviceGraph.from_offsets(V, np.zeros(V + 1, np.uint32), np.zeros(0, np.uint32)) as dg:
        st = gbx.breadth_first_search(dg, 2, 2)
        assert st.processed_nodes == 1
