"""The cuda integration on the GPU: the reference's own entry points
(breadthFirstSearchGraphCSR, pageRankGraphCSR, SSSPGraphCSR,
connectedComponentsGraphCSR, triangleCountGraphCSR, SPMVGraphCSR) called with
the reference's structs -- struct Arguments and struct GraphCSR built here
with ctypes in the reference's layout -- against the golden outputs of the
reference host on the same graphs."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

u32, P = C.c_uint32, C.POINTER


class MT(C.Structure):
    _fields_ = [("mt", C.c_ulong * 624), ("mti", C.c_int)]


class Arguments(C.Structure):  # 01_host/include/config/graphConfig.h:18-63
    _fields_ = [(n, C.c_int) for n in ("wflag", "xflag", "sflag", "Sflag", "dflag")] + \
               [(n, u32) for n in ("binSize", "verbosity", "iterations", "trials")] + [("epsilon", C.c_double)] + \
               [(n, u32) for n in ("source", "algorithm", "datastructure", "pushpull", "sort", "lmode", "lmode_l2",
                                   "lmode_l3", "mmode", "symmetric", "weighted", "delta")] + \
               [(n, C.c_int) for n in ("pre_numThreads", "algo_numThreads", "ker_numThreads")] + \
               [("fnameb", C.c_char_p), ("fnamel", C.c_char_p), ("fnameb_format", u32), ("convert_format", u32),
                ("mt19937var", MT), ("cache_size", u32), ("kernel_name", C.c_char_p), ("cu_id", C.c_int),
                ("device_index", C.c_int), ("xclbin_path", C.c_char_p), ("overlay_path", C.c_char_p)] + \
               [(n, C.c_int) for n in ("ctrl_mode", "endian_read", "endian_write", "flush_cache", "bankGroupIndex")]


class Vertex(C.Structure):
    _fields_ = [("num_vertices", u32), ("out_degree", P(u32)), ("in_degree", P(u32)), ("edges_idx", P(u32))]


class EdgeList(C.Structure):
    _fields_ = [("num_edges", u32), ("num_vertices", u32), ("avg_degree", u32), ("max_weight", C.c_float),
                ("edges_array_weight", P(C.c_float)), ("edges_array_src", P(u32)), ("edges_array_dest", P(u32)),
                ("mask_array", P(u32)), ("label_array", P(u32)), ("inverse_label_array", P(u32))]


class GraphCSRdw(C.Structure):  # WEIGHTED 1, DIRECTED 1
    _fields_ = [("num_edges", u32), ("num_vertices", u32), ("avg_degree", u32), ("max_weight", C.c_float),
                ("vertices", P(Vertex)), ("sorted_edges_array", P(EdgeList)), ("inverse_vertices", P(Vertex)),
                ("inverse_sorted_edges_array", P(EdgeList))]


class GraphCSRu(C.Structure):  # WEIGHTED 0, DIRECTED 0
    _fields_ = [("num_edges", u32), ("num_vertices", u32), ("avg_degree", u32), ("vertices", P(Vertex)),
                ("sorted_edges_array", P(EdgeList))]


class BFSStats(C.Structure):
    _fields_ = [("distances", P(u32)), ("parents", P(C.c_int)), ("distances_DualOrder", P(u32)),
                ("parents_DualOrder", P(C.c_int)), ("processed_nodes", u32), ("num_vertices", u32),
                ("iteration", u32), ("time_total", C.c_double)]


class PageRankStats(C.Structure):
    _fields_ = [("damp", C.c_float), ("base_pr", C.c_float), ("iterations", u32), ("num_vertices", u32),
                ("activeVertices", u32), ("realRanks", P(u32)), ("pageRanks", P(C.c_float)),
                ("time_total", C.c_double), ("error_total", C.c_double)]


class SSSPStats(C.Structure):
    _fields_ = [("distances", P(u32)), ("parents", P(u32)), ("buckets_map", P(u32))] + \
               [(n, u32) for n in ("bucket_counter", "bucket_current", "buckets_total", "processed_nodes", "delta",
                                   "num_vertices")] + [("time_total", C.c_double)]


class CCStats(C.Structure):
    _fields_ = [("iterations", u32), ("neighbor_rounds", u32), ("arguments", C.c_void_p), ("num_vertices", u32),
                ("components", P(u32)), ("counts", P(u32)), ("labels", P(u32)), ("time_total", C.c_double)]


class TCStats(C.Structure):
    _fields_ = [("num_vertices", u32), ("counts", P(C.c_uint64)), ("total_counts", C.c_uint64),
                ("time_total", C.c_double)]


class SPMVStats(C.Structure):
    _fields_ = [("iterations", u32), ("arguments", C.c_void_p), ("num_vertices", u32),
                ("vector_output", P(C.c_float)), ("vector_input", P(C.c_float)), ("time_total", C.c_double)]


def _p(a, t=u32):
    return a.ctypes.data_as(P(t))


def _arr(ptr, n, dt):
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dt).copy()


class Built:
    """Reference-layout GraphCSR assembled from a golden fixture (keeps the
    backing arrays alive)."""

    def __init__(self, fx, variant, directed):
        self.keep = []
        V = int(fx[f"{variant}_num_vertices"])
        E = int(fx[f"{variant}_dest"].shape[0])
        deg = np.ascontiguousarray(fx[f"{variant}_out_degree"], np.uint32)
        idx = np.ascontiguousarray(fx[f"{variant}_edges_idx"], np.uint32)
        dest = np.ascontiguousarray(fx[f"{variant}_dest"], np.uint32)
        src = np.ascontiguousarray(fx[f"{variant}_src"], np.uint32)
        w = np.ascontiguousarray(fx.get(f"{variant}_weight", np.ones(E, np.float32)), np.float32)
        lab = np.arange(V, dtype=np.uint32)
        zeros = np.zeros(V, np.uint32)
        self.keep += [deg, idx, dest, src, w, lab, zeros]
        self.vert = Vertex(V, _p(deg), _p(zeros), _p(idx))
        self.el = EdgeList(E, V, E // V, float(w.max()) if E else 0.0, _p(w, C.c_float), _p(src), _p(dest),
                           _p(zeros), _p(lab), _p(lab))
        if directed:
            inv = po.build_csr(V, dest, src, w, sort_mode=1)
            self.keep += [inv.out_degree, inv.edges_idx, inv.dest, inv.src, inv.weight]
            self.ivert = Vertex(V, _p(inv.out_degree), _p(zeros), _p(inv.edges_idx))
            self.iel = EdgeList(E, V, E // V, 0.0, _p(inv.weight, C.c_float), _p(inv.src), _p(inv.dest), _p(zeros),
                                _p(lab), _p(lab))
            self.g = GraphCSRdw(E, V, E // V, float(w.max()) if E else 0.0, C.pointer(self.vert),
                                C.pointer(self.el), C.pointer(self.ivert), C.pointer(self.iel))
        else:
            self.g = GraphCSRu(E, V, E // V, C.pointer(self.vert), C.pointer(self.el))
        self.V, self.E = V, E


def _lib(gbx, name, gtype):
    import graphblox_gb300._build as b

    b.build_integration()
    lib = C.CDLL(str(b.PKG / f"libgbx_graphblox_{name}.so"))
    for fn, st in (("breadthFirstSearchGraphCSR", BFSStats), ("pageRankGraphCSR", PageRankStats),
                   ("SSSPGraphCSR", SSSPStats), ("connectedComponentsGraphCSR", CCStats),
                   ("triangleCountGraphCSR", TCStats), ("SPMVGraphCSR", SPMVStats)):
        f = getattr(lib, fn)
        f.restype = P(st)
        f.argtypes = [P(Arguments), P(gtype)]
    for fn in ("freeBFSStats", "freePageRankStats", "freeSSSPStats", "freeCCStats", "freeTCStats", "freeSPMVStats"):
        getattr(lib, fn).argtypes = [C.c_void_p]
    return lib


def _args(**kw):
    a = Arguments()
    a.iterations, a.epsilon, a.delta, a.trials = 20, 1e-4, 1, 1
    for k, v in kw.items():
        setattr(a, k, v)
    return a


@pytest.mark.parametrize("name", ["v51_e1021", "v1000_e10000", "v8192_e32768", "v300_e2730"])
def test_reference_entry_points_directed_weighted(gbx, cuda_device, name):
    fx = load_golden(name)
    b = Built(fx, "dw", directed=True)
    lib = _lib(gbx, "dw", GraphCSRdw)
    g = C.byref(b.g)
    for dist, meta in zip(fx["dw_bfs_distances"], fx["dw_bfs_meta"]):
        a = _args(source=int(meta[0]), pushpull=2)
        s = lib.breadthFirstSearchGraphCSR(C.byref(a), g)
        assert s, "NULL BFSStats"
        np.testing.assert_array_equal(_arr(s.contents.distances, b.V, np.uint32), dist)
        assert (s.contents.processed_nodes, s.contents.iteration) == (int(meta[2]), int(meta[3]))
        assert a.source == int(meta[1])  # BFS.c:153 side effect kept
        lib.freeBFSStats(s)
    a = _args(pushpull=0, iterations=20, epsilon=0.0)
    s = lib.pageRankGraphCSR(C.byref(a), g)
    assert po.fp32_close(_arr(s.contents.pageRanks, b.V, np.float32), fx["dw_pr20"], 1e-6)[0]
    lib.freePageRankStats(s)
    a = _args(source=1)
    s = lib.SSSPGraphCSR(C.byref(a), g)
    np.testing.assert_array_equal(_arr(s.contents.distances, b.V, np.uint32), fx["dw_sssp"])
    lib.freeSSSPStats(s)
    a = _args(pushpull=1)
    s = lib.connectedComponentsGraphCSR(C.byref(a), g)
    np.testing.assert_array_equal(_arr(s.contents.components, b.V, np.uint32), fx["dw_cc"])
    lib.freeCCStats(s)
    a = _args(pushpull=0, iterations=2)
    s = lib.SPMVGraphCSR(C.byref(a), g)
    assert po.fp32_close(_arr(s.contents.vector_output, b.V, np.float32), fx["dw_spmv_y"], 1e-6)[0]
    lib.freeSPMVStats(s)


@pytest.mark.parametrize("name", ["v51_e1021", "v8192_e32768", "graphbrew"])
def test_reference_entry_points_undirected(gbx, cuda_device, name):
    fx = load_golden(name)
    b = Built(fx, "u", directed=False)
    lib = _lib(gbx, "u", GraphCSRu)
    g = C.byref(b.g)
    a = _args(pushpull=1)
    s = lib.triangleCountGraphCSR(C.byref(a), g)
    assert s.contents.total_counts == int(fx["u_tc"])
    lib.freeTCStats(s)
    for dist, meta in zip(fx["u_bfs_distances"], fx["u_bfs_meta"]):
        a = _args(source=int(meta[0]), pushpull=2)
        s = lib.breadthFirstSearchGraphCSR(C.byref(a), g)
        np.testing.assert_array_equal(_arr(s.contents.distances, b.V, np.uint32), dist)
        assert (s.contents.processed_nodes, s.contents.iteration) == (int(meta[2]), int(meta[3]))
        lib.freeBFSStats(s)
    a = _args(pushpull=1)
    s = lib.connectedComponentsGraphCSR(C.byref(a), g)
    np.testing.assert_array_equal(_arr(s.contents.components, b.V, np.uint32), fx["u_cc"])
    lib.freeCCStats(s)


class BellmanFordStats(C.Structure):
    _fields_ = [("distances", P(u32)), ("parents", P(u32)), ("processed_nodes", u32), ("num_vertices", u32),
                ("time_total", C.c_double)]


class DFSStats(C.Structure):
    _fields_ = [("distances", P(u32)), ("parents", P(C.c_int)), ("processed_nodes", u32), ("num_vertices", u32),
                ("time_total", C.c_double)]


class Predecessor(C.Structure):
    _fields_ = [("nodes", P(u32)), ("degree", u32)]


class BCStats(C.Structure):
    _fields_ = [("stack", P(Predecessor)), ("distances", P(u32)), ("realRanks", P(u32)), ("parents", P(C.c_int)),
                ("sigma", P(C.c_int)), ("dependency", P(C.c_float)), ("betweennessCentrality", P(C.c_float)),
                ("predecessors", P(Predecessor)), ("iteration", u32), ("processed_nodes", u32),
                ("num_vertices", u32), ("time_total", C.c_double)]


def _seed_mt(a, seed=27491095):
    """initializeMersenneState (mt19937.c:55-67) into a.mt19937var."""
    for i in range(624):
        hi = seed & 0xFFFF0000
        seed = (69069 * seed + 1) & 0xFFFFFFFF
        a.mt19937var.mt[i] = hi | ((seed & 0xFFFF0000) >> 16)
        seed = (69069 * seed + 1) & 0xFFFFFFFF
    a.mt19937var.mti = 624


def _lib_more(gbx, name):
    import graphblox_gb300._build as b

    b.build_integration()
    lib = C.CDLL(str(b.PKG / f"libgbx_graphblox_{name}.so"))
    gtype = GraphCSRdw if name == "dw" else GraphCSRu
    for fn, st in (("bellmanFordGraphCSR", BellmanFordStats), ("depthFirstSearchGraphCSR", DFSStats),
                   ("betweennessCentralityGraphCSR", BCStats)):
        f = getattr(lib, fn)
        f.restype = P(st)
        f.argtypes = [P(Arguments), P(gtype)]
    for fn in ("freeBellmanFordStats", "freeDFSStats", "freeBetweennessCentralityStats"):
        getattr(lib, fn).argtypes = [C.c_void_p]
    return lib


@pytest.mark.parametrize("name", ["v300_e2730", "v1000_e10000", "v8192_e32768"])
def test_reference_bf_dfs_bc_directed_weighted(gbx, cuda_device, name):
    from conftest import load_bf_dfs_bc

    more = load_bf_dfs_bc()
    fx = load_golden(name)
    b = Built(fx, "dw", directed=True)
    lib = _lib_more(gbx, "dw")
    g = C.byref(b.g)
    key = f"{name}_dw"
    a = _args(source=1, pushpull=1)
    s = lib.bellmanFordGraphCSR(C.byref(a), g)
    assert s, "NULL BellmanFordStats"
    np.testing.assert_array_equal(_arr(s.contents.distances, b.V, np.uint32), more[f"{key}_bf_r1"])
    assert a.iterations == b.V - 1  # bellmanFord.c:449 side effect kept
    lib.freeBellmanFordStats(s)
    for r in (0, 1):
        a = _args(source=r)
        s = lib.depthFirstSearchGraphCSR(C.byref(a), g)
        np.testing.assert_array_equal(_arr(s.contents.distances, b.V, np.uint32), more[f"{key}_dfs_r{r}"])
        np.testing.assert_array_equal(_arr(s.contents.parents, b.V, np.int32), more[f"{key}_dfs_parents_r{r}"])
        assert s.contents.processed_nodes == int(more[f"{key}_dfs_processed_r{r}"])
        lib.freeDFSStats(s)
    roots = more[f"{key}_bc_roots"]
    a = _args(iterations=len(roots))
    _seed_mt(a)
    s = lib.betweennessCentralityGraphCSR(C.byref(a), g)
    assert s, "NULL BetweennessCentralityStats"
    bc = _arr(s.contents.betweennessCentrality, b.V, np.float32)
    np.testing.assert_array_equal(bc.view(np.uint32), more[f"{key}_bc"].view(np.uint32))
    np.testing.assert_array_equal(_arr(s.contents.distances, b.V, np.uint32), more[f"{key}_bc_distances"])
    np.testing.assert_array_equal(_arr(s.contents.sigma, b.V, np.int32), more[f"{key}_bc_sigma"])
    assert (s.contents.iteration, s.contents.processed_nodes) == (len(roots), int(more[f"{key}_bc_processed"]))
    reached = int(np.count_nonzero(more[f"{key}_bc_distances"] != 0xFFFFFFFF))
    stack = _arr(s.contents.stack.contents.nodes, b.V, np.uint32)[:reached]
    assert s.contents.stack.contents.degree == reached
    lv = more[f"{key}_bc_distances"][stack].astype(np.int64)
    assert np.all(np.diff(lv) >= 0) and stack[0] == roots[-1]
    lib.freeBetweennessCentralityStats(s)


@pytest.mark.parametrize("name", ["v51_e1021", "v8192_e32768", "graphbrew"])
def test_reference_bf_dfs_undirected(gbx, cuda_device, name):
    from conftest import load_bf_dfs_bc

    more = load_bf_dfs_bc()
    fx = load_golden(name)
    b = Built(fx, "u", directed=False)
    lib = _lib_more(gbx, "u")
    g = C.byref(b.g)
    key = f"{name}_u"
    a = _args(source=1, pushpull=1)
    s = lib.bellmanFordGraphCSR(C.byref(a), g)
    np.testing.assert_array_equal(_arr(s.contents.distances, b.V, np.uint32), more[f"{key}_bf_r1"])
    lib.freeBellmanFordStats(s)
    for r in (0, 1):
        a = _args(source=r)
        s = lib.depthFirstSearchGraphCSR(C.byref(a), g)
        np.testing.assert_array_equal(_arr(s.contents.parents, b.V, np.int32), more[f"{key}_dfs_parents_r{r}"])
        assert s.contents.processed_nodes == int(more[f"{key}_dfs_processed_r{r}"])
        lib.freeDFSStats(s)


def test_graph_rewritten_in_place_is_uploaded_again(gbx, cuda_device):
    """The drop-in caches the device copy of a GraphCSR; rewriting its
    weights in place (same pointers) between two SSSPGraphCSR calls must give
    the new graph's distances, and so must a different graph built at the
    same addresses (edges rewritten too)."""
    fx = load_golden("v1000_e10000")
    b = Built(fx, "dw", directed=True)
    lib = _lib(gbx, "dw", GraphCSRdw)
    g = C.byref(b.g)
    V = b.V
    src = int(np.argmax(fx["dw_out_degree"]))

    def sssp():
        a = _args(source=src)
        s = lib.SSSPGraphCSR(C.byref(a), g)
        assert s, "NULL SSSPStats"
        d = _arr(s.contents.distances, V, np.uint32)
        lib.freeSSSPStats(s)
        return d

    def oracle(weights):
        host = po.HostCSR(V, fx["dw_out_degree"], fx["dw_edges_idx"], fx["dw_dest"], weights)
        return po.sssp(host, src, 1)

    w = np.ctypeslib.as_array(b.el.edges_array_weight, shape=(b.E,))
    iw = np.ctypeslib.as_array(b.iel.edges_array_weight, shape=(b.E,))
    first = sssp()
    np.testing.assert_array_equal(first, oracle(w.copy()))
    # new integer weights, written into the same arrays (forward and inverse)
    rng = np.random.default_rng(3)
    neww = rng.integers(1, 50, b.E).astype(np.float32)
    w[:] = neww
    inv = po.build_csr(V, fx["dw_dest"], fx["dw_src"], neww, sort_mode=1)
    iw[:] = inv.weight
    second = sssp()
    np.testing.assert_array_equal(second, oracle(neww))
    assert not np.array_equal(first, second)
