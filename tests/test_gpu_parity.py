"""GPU parity: every kernel through the C ABI against the reference's golden
outputs (tests/golden) and the CPU oracle on the same seeded inputs.

Integer results (CSR, reordering, BFS levels and stats, SSSP distances, CC
labels, TC counts) must be bit-exact. PageRank and SpMV must be within 1e-6
relative L1 of the FP64 restatement (the tolerance the spec states).
"""
import numpy as np
import pytest

from conftest import GOLDEN_GRAPHS, REORDER_MODES, load_golden, load_reorder_modes
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

REL_L1_TOL = 1e-6
VARIANTS = [("u", True, True), ("dw", False, False), ("dwk", False, True)]


def _inputs(fx, variant, symmetric):
    src, dst = fx["src"], fx["dst"]
    w = fx.get("weight")
    if variant == "u":
        w = None
    elif w is None:
        w = np.ones(src.shape[0], np.float32)
    V = int(max(src.max(), dst.max())) + 1
    return V, src, dst, w


def gpu_graph(gbx, fx, variant, symmetric, dedup):
    V, src, dst, w = _inputs(fx, variant, symmetric)
    deg, idx, s, d, ww = gbx.csr_build(src, dst, w, num_vertices=V, symmetric=symmetric, dedup=dedup, sort=1)
    g = gbx.GraphCSR(V, int(s.shape[0]), deg, idx, d, s, ww, np.arange(V, dtype=np.uint32),
                     np.arange(V, dtype=np.uint32))
    if variant != "u":
        ideg, iidx, _, idst, iw = gbx.csr_build(d, s, ww, num_vertices=V, sort=1)
        g.inverse_out_degree, g.inverse_edges_idx, g.inverse_dest, g.inverse_weight = ideg, iidx, idst, iw
    return g


def host_views(g):
    host = po.HostCSR(g.num_vertices, g.out_degree, g.edges_idx, g.dest, g.weight, g.src)
    pull = None
    if g.inverse_dest is not None:
        pull = po.HostCSR(g.num_vertices, g.inverse_out_degree, g.inverse_edges_idx, g.inverse_dest,
                          g.inverse_weight)
    return host, pull


@pytest.mark.parametrize("name", GOLDEN_GRAPHS)
@pytest.mark.parametrize("variant,symmetric,dedup", VARIANTS)
def test_csr_build_golden(gbx, cuda_device, name, variant, symmetric, dedup):
    fx = load_golden(name)
    g = gpu_graph(gbx, fx, variant, symmetric, dedup)
    assert g.num_vertices == int(fx[f"{variant}_num_vertices"])
    np.testing.assert_array_equal(g.out_degree, fx[f"{variant}_out_degree"])
    np.testing.assert_array_equal(g.edges_idx, fx[f"{variant}_edges_idx"])
    np.testing.assert_array_equal(g.dest, fx[f"{variant}_dest"])
    np.testing.assert_array_equal(g.src, fx[f"{variant}_src"])
    if f"{variant}_weight" in fx:
        np.testing.assert_array_equal(g.weight, fx[f"{variant}_weight"])


@pytest.mark.parametrize("name", GOLDEN_GRAPHS)
@pytest.mark.parametrize("variant,symmetric,dedup", VARIANTS)
def test_degree_reorder_golden(gbx, cuda_device, name, variant, symmetric, dedup):
    fx = load_golden(name)
    g = gpu_graph(gbx, fx, variant, symmetric, dedup)
    el = gbx.EdgeList(g.num_vertices, g.src.copy(), g.dest.copy())
    gbx.degree_reorder(el, 1)
    np.testing.assert_array_equal(el.label_array, fx[f"{variant}_reorder_label"])
    np.testing.assert_array_equal(el.inverse_label_array[el.label_array],
                                  np.arange(g.num_vertices, dtype=np.uint32))
    deg, _, _, d, _ = gbx.csr_build(el.src, el.dst, num_vertices=g.num_vertices, sort=1)
    np.testing.assert_array_equal(d, fx[f"{variant}_reorder_dest"])
    np.testing.assert_array_equal(deg, fx[f"{variant}_reorder_out_degree"])


@pytest.mark.parametrize("name", GOLDEN_GRAPHS)
@pytest.mark.parametrize("variant,symmetric,dedup", VARIANTS)
def test_algorithms_golden(gbx, cuda_device, name, variant, symmetric, dedup):
    fx = load_golden(name)
    g = gpu_graph(gbx, fx, variant, symmetric, dedup)
    host, pull = host_views(g)
    with gbx.DeviceGraph.from_graph_csr(g, use_weights=(variant != "u")) as dg:
        for dist, meta in zip(fx[f"{variant}_bfs_distances"], fx[f"{variant}_bfs_meta"]):
            st = gbx.breadth_first_search(dg, int(meta[0]), pushpull=2)
            np.testing.assert_array_equal(st.distances, dist)
            assert (st.processed_nodes, st.iteration) == (int(meta[2]), int(meta[3]))
            for mode in (0, 1):
                st = gbx.breadth_first_search(dg, int(meta[0]), pushpull=mode)
                np.testing.assert_array_equal(st.distances, dist)
        pr = gbx.page_rank(dg, 20, 0.0)
        ref64, _, _ = po.pagerank(host, 20, 0.0, pull, fp64=True)
        assert po.fp32_close(pr.pageRanks, ref64, REL_L1_TOL)[0]
        assert po.fp32_close(pr.pageRanks, fx[f"{variant}_pr20"], REL_L1_TOL)[0]
        assert pr.iterations == 20
        st = gbx.sssp(dg, int(fx[f"{variant}_sssp_source"]), delta=1, map_source=False)
        np.testing.assert_array_equal(st.distances, fx[f"{variant}_sssp"])
        st = gbx.sssp(dg, int(fx[f"{variant}_sssp_source"]), delta=0, map_source=False)
        np.testing.assert_array_equal(st.distances, fx[f"{variant}_sssp"])
        for cv in (0, 1, 2):
            comp, _ = gbx.connected_components(dg, cv)
            np.testing.assert_array_equal(comp, fx[f"{variant}_cc"])
        x = fx[f"{variant}_spmv_x"]
        y = gbx.spmv(dg, x, iterations=2)
        y64 = po.spmv(host, x, None if variant == "u" else pull.weight, 0.0001, 2, pull=pull, fp64=True)
        assert po.fp32_close(y, y64, REL_L1_TOL)[0]
        assert po.fp32_close(y, fx[f"{variant}_spmv_y"], REL_L1_TOL)[0]
        if variant == "u":
            assert gbx.triangle_count(dg) == int(fx["u_tc"])


def _rmat_graph(gbx, scale, ef, seed, symmetric=False, weights=None):
    V = 1 << scale
    src, dst = gbx.generate_rmat(scale, V * ef, seed=seed)
    w = None
    if weights == "int":
        w = gbx.generate_values(src.shape[0], 0, 1, 255, seed=seed + 11)
    el = gbx.EdgeList(V, src, dst, w)
    if symmetric:
        el = gbx.EdgeList(V, np.concatenate([src, dst]), np.concatenate([dst, src]),
                          None if w is None else np.concatenate([w, w]))
    return gbx.graph_csr_preprocessing(el, sort=1, dedup=True, directed=not symmetric,
                                       keep_weights=w is not None)


@pytest.mark.parametrize("scale,ef,seed", [(14, 16, 1), (16, 16, 2)])
def test_rmat_directed(gbx, cuda_device, scale, ef, seed):
    g = _rmat_graph(gbx, scale, ef, seed, weights="int")
    host, pull = host_views(g)
    # CSR build against the oracle's sort/dedup of the same edge list
    src, dst = gbx.generate_rmat(scale, (1 << scale) * ef, seed=seed)
    w = gbx.generate_values(src.shape[0], 0, 1, 255, seed=seed + 11)
    ref = po.build_csr(1 << scale, src, dst, w, sort_mode=1, dedup=True)
    np.testing.assert_array_equal(g.dest, ref.dest)
    np.testing.assert_array_equal(g.edges_idx, ref.edges_idx)
    np.testing.assert_array_equal(g.weight, ref.weight)
    rng = np.random.default_rng(seed)
    roots = [0] + [int(r) for r in rng.choice(np.nonzero(g.out_degree)[0], 5)]
    with gbx.DeviceGraph.from_graph_csr(g) as dg:
        for r in roots:
            st = gbx.breadth_first_search(dg, r)
            d, _, proc, it = po.bfs(host, r, pull)
            np.testing.assert_array_equal(st.distances, d)
            assert (st.processed_nodes, st.iteration) == (proc, it)
            # parents form a BFS tree
            par = np.asarray(st.parents)
            reached = np.nonzero((d > 0))[0]
            assert np.all(d[par[reached]] == d[reached] - 1)
        for r in roots[:3]:
            st = gbx.sssp(dg, r)
            np.testing.assert_array_equal(st.distances, po.sssp(host, r, 64))
        pr = gbx.page_rank(dg, 20, 0.0)
        ref64, _, _ = po.pagerank(host, 20, 0.0, pull, fp64=True)
        assert po.fp32_close(pr.pageRanks, ref64, REL_L1_TOL)[0]
        x = gbx.generate_values(g.num_vertices, 2, seed=5)
        vals = gbx.generate_values(g.num_edges, 1, seed=6)
        y = gbx.spmv(dg, x, values=vals)
        y64 = po.spmv(host, x, vals, pull=pull, fp64=True)
        assert po.fp32_close(y, y64, REL_L1_TOL)[0]


@pytest.mark.parametrize("scale,ef,seed", [(14, 8, 3), (16, 16, 4)])
def test_rmat_symmetric(gbx, cuda_device, scale, ef, seed):
    g = _rmat_graph(gbx, scale, ef, seed, symmetric=True)
    host, _ = host_views(g)
    with gbx.DeviceGraph.from_graph_csr(g) as dg:
        ref = po.cc(host, 1)
        for cv in (0, 1, 2):
            comp, _ = gbx.connected_components(dg, cv)
            np.testing.assert_array_equal(comp, ref)
        assert gbx.triangle_count(dg) == po.triangle_count(host)
    # degree-ordered DAG: TC after degree reordering gives the same count;
    # the first count searches the rows for the prefix lengths, the second
    # builds the plan's per-edge prefix lengths and the third reads them
    el = gbx.EdgeList(g.num_vertices, g.src.copy(), g.dest.copy())
    gbx.degree_reorder(el, 1)
    g2 = gbx.graph_csr_preprocessing(el, sort=1, directed=False, keep_weights=False)
    tri = po.triangle_count(host)
    with gbx.DeviceGraph.from_graph_csr(g2) as dg2:
        assert [gbx.triangle_count(dg2) for _ in range(3)] == [tri, tri, tri]


def test_tc_asymmetric_simple_graphs(gbx, cuda_device):
    """Simple (no repeated neighbour) but not symmetric CSRs take the
    reference-multiplicity path: a directed RMAT graph, and a symmetric graph
    with one reverse edge removed."""
    g = _rmat_graph(gbx, 12, 8, 7)
    host, _ = host_views(g)
    with gbx.DeviceGraph.from_graph_csr(g, use_weights=False) as dg:
        assert gbx.triangle_count(dg) == po.triangle_count(host)
    gs = _rmat_graph(gbx, 12, 8, 7, symmetric=True)
    keep = np.ones(gs.num_edges, bool)
    keep[np.nonzero(gs.src < gs.dest)[0][len(gs.src) // 7]] = False  # drop one direction of one edge
    src, dst = gs.src[keep], gs.dest[keep]
    deg, idx, s, d, _ = gbx.csr_build(src, dst, num_vertices=gs.num_vertices, sort=1)
    g1 = gbx.GraphCSR(gs.num_vertices, int(s.shape[0]), deg, idx, d, s, None,
                      np.arange(gs.num_vertices, dtype=np.uint32), np.arange(gs.num_vertices, dtype=np.uint32))
    with gbx.DeviceGraph.from_graph_csr(g1) as dg:
        assert gbx.triangle_count(dg) == po.triangle_count(po.HostCSR(gs.num_vertices, deg, idx, d))


def test_edge_cases(gbx, cuda_device):
    # single vertex, no edges
    g = gbx.GraphCSR(1, 0, np.zeros(1, np.uint32), np.zeros(1, np.uint32), np.zeros(0, np.uint32),
                     np.zeros(0, np.uint32), None, np.zeros(1, np.uint32), np.zeros(1, np.uint32))
    with gbx.DeviceGraph.from_graph_csr(g) as dg:
        st = gbx.breadth_first_search(dg, 0)
        assert st.processed_nodes == 1 and st.distances[0] == 0
        pr = gbx.page_rank(dg, 5, 0.0)
        assert np.isclose(pr.pageRanks[0], np.float32(1.0) - np.float32(0.85))
        assert gbx.triangle_count(dg) == 0
        comp, _ = gbx.connected_components(dg, 1)
        assert comp[0] == 0
        with pytest.raises(gbx.GbxError):
            gbx.breadth_first_search(dg, 1, map_source=False)  # source out of range
    # isolated vertices, a degree-0 source, self loops and duplicates kept
    src = np.array([0, 0, 1, 1, 2, 2, 5, 5, 5], np.uint32)
    dst = np.array([1, 1, 2, 2, 0, 2, 5, 0, 1], np.uint32)
    V = 8
    deg, idx, s, d, _ = gbx.csr_build(src, dst, num_vertices=V, sort=1)
    ref = po.build_csr(V, src, dst, sort_mode=1)
    np.testing.assert_array_equal(d, ref.dest)
    g = gbx.GraphCSR(V, int(s.shape[0]), deg, idx, d, s, None, np.arange(V, dtype=np.uint32),
                     np.arange(V, dtype=np.uint32))
    host = po.HostCSR(V, deg, idx, d)
    with gbx.DeviceGraph.from_graph_csr(g) as dg:
        for r in range(V):
            st = gbx.breadth_first_search(dg, r)
            dd, par, proc, it = po.bfs(host, r)
            np.testing.assert_array_equal(st.distances, dd)
            assert (st.processed_nodes, st.iteration) == (proc, it)
            unreached = (dd == 0) & (np.arange(V) != r)
            np.testing.assert_array_equal(np.asarray(st.parents)[unreached], par[unreached])
        assert gbx.triangle_count(dg) == po.triangle_count(host)  # multiplicities and loops
        comp, _ = gbx.connected_components(dg, 2)
        np.testing.assert_array_equal(comp, po.cc(host, 2))


def _runs_reversed(deg, idx, ids, w):
    """The same CSR with every vertex's run stored in reverse vertex order
    (edges_idx no longer the prefix sum of the degrees)."""
    V = deg.shape[0]
    new_idx = np.zeros(V, np.uint32)
    parts, wparts, at = [], [], 0
    for v in range(V - 1, -1, -1):
        n = int(deg[v])
        if n:
            new_idx[v] = at
            parts.append(ids[idx[v]: idx[v] + n])
            if w is not None:
                wparts.append(w[idx[v]: idx[v] + n])
            at += n
    cat = np.concatenate(parts).astype(np.uint32)
    return new_idx, cat, (None if w is None else np.concatenate(wparts).astype(np.float32))


def test_layout_runs_out_of_vertex_order(gbx, cuda_device):
    g = _rmat_graph(gbx, 12, 8, 9, weights="int")
    host, pull = host_views(g)
    V = g.num_vertices
    fidx, fdest, fw = _runs_reversed(g.out_degree, g.edges_idx, g.dest, g.weight)
    iidx, idest, iw = _runs_reversed(g.inverse_out_degree, g.inverse_edges_idx, g.inverse_dest,
                                     g.inverse_weight)
    assert np.any(np.diff(fidx[g.out_degree > 0].astype(np.int64)) < 0)
    g2 = gbx.GraphCSR(V, g.num_edges, g.out_degree, fidx, fdest, g.src, fw, g.label_array,
                      g.inverse_label_array, g.inverse_out_degree, iidx, idest, iw)
    with gbx.DeviceGraph.from_graph_csr(g2) as dg:
        for r in (0, 5):
            d, _, proc, it = po.bfs(host, r, pull)
            st = gbx.breadth_first_search(dg, r)
            np.testing.assert_array_equal(st.distances, d)
            assert (st.processed_nodes, st.iteration) == (proc, it)
        np.testing.assert_array_equal(gbx.sssp(dg, 0, 64).distances, po.sssp(host, 0, 64))
        pr = gbx.page_rank(dg, 20, 0.0)
        ref64, _, _ = po.pagerank(host, 20, 0.0, pull, fp64=True)
        assert po.fp32_close(np.asarray(pr.pageRanks), ref64, REL_L1_TOL)[0]


def test_layout_run_past_edges_rejected(gbx, cuda_device):
    # vertex 0's run starts at 1 and holds two edges: it ends past E = 2
    g = gbx.GraphCSR(3, 2, np.array([2, 0, 0], np.uint32), np.array([1, 0, 0], np.uint32),
                     np.array([1, 2], np.uint32), np.array([0, 0], np.uint32), None,
                     np.arange(3, dtype=np.uint32), np.arange(3, dtype=np.uint32))
    with pytest.raises(gbx.GbxError) as e:
        gbx.DeviceGraph.from_graph_csr(g)
    assert e.value.status == -1


def test_device_resident_outputs(gbx, cuda_device):
    import torch

    g = _rmat_graph(gbx, 12, 8, 9)
    host, pull = host_views(g)
    with gbx.DeviceGraph.from_graph_csr(g) as dg:
        dist = torch.empty(g.num_vertices, dtype=torch.int32, device=cuda_device)
        st = gbx.breadth_first_search(dg, 0, distances=dist, parents=None)
        d, _, _, _ = po.bfs(host, 0, pull)
        np.testing.assert_array_equal(dist.cpu().numpy().view(np.uint32), d)
        ranks = torch.empty(g.num_vertices, dtype=torch.float32, device=cuda_device)
        gbx.page_rank(dg, 20, 0.0, ranks=ranks)
        ref64, _, _ = po.pagerank(host, 20, 0.0, pull, fp64=True)
        assert po.fp32_close(ranks.cpu().numpy(), ref64, REL_L1_TOL)[0]


def test_tuning_knobs_keep_results(gbx, cuda_device):
    """Every knob setting gives the oracle's integer results; the pull-engine
    threshold only reorders FP32 sums (PR, SpMV stay within the L1 bound)."""
    g = _rmat_graph(gbx, 15, 16, 12, weights="int")
    host, pull = host_views(g)
    x = gbx.generate_values(g.num_vertices, 2, seed=7)
    vals = gbx.generate_values(g.num_edges, 1, seed=8)
    ref_pr, _, _ = po.pagerank(host, 20, 0.0, pull, fp64=True)
    ref_y = po.spmv(host, x, vals, pull=pull, fp64=True)
    ref_bfs = po.bfs(host, 0, pull)
    ref_sssp = po.sssp(host, 0, 64)
    with gbx.DeviceGraph.from_graph_csr(g) as dg:
        assert dg.get_tuning("pull_heavy_min") == 4096
        for heavy in (64, 200, 1024, 4096, 1 << 20):
            dg.set_tuning("pull_heavy_min", heavy)
            assert dg.get_tuning("pull_heavy_min") == heavy
            pr = gbx.page_rank(dg, 20, 0.0)
            assert po.fp32_close(pr.pageRanks, ref_pr, REL_L1_TOL)[0], heavy
            y = gbx.spmv(dg, x, values=vals)
            assert po.fp32_close(y, ref_y, REL_L1_TOL)[0], heavy
        for alpha, beta in ((1, 1), (4, 18), (4096, 64)):
            dg.set_tuning("bfs_alpha", alpha)
            dg.set_tuning("bfs_beta", beta)
            st = gbx.breadth_first_search(dg, 0)
            np.testing.assert_array_equal(st.distances, ref_bfs[0])
            assert (st.processed_nodes, st.iteration) == ref_bfs[2:]
        for delta in (1, 100, 4096):
            dg.set_tuning("sssp_delta", delta)
            np.testing.assert_array_equal(gbx.sssp(dg, 0).distances, ref_sssp)
        tuned = dg.autotune(bfs=True, sssp=True, samples=2, pull=True)
        assert tuned["pull_heavy_min"] in (1024, 4096, 16384)
        assert tuned["bfs_alpha"] >= 1 and tuned["sssp_delta"] >= 1
        np.testing.assert_array_equal(gbx.breadth_first_search(dg, 0).distances, ref_bfs[0])
        assert po.fp32_close(gbx.page_rank(dg, 20, 0.0).pageRanks, ref_pr, REL_L1_TOL)[0]
        for key, bad in (("pull_heavy_min", 8), ("bfs_alpha", 0), ("no_such_knob", 1)):
            with pytest.raises(gbx.GbxError) as e:
                dg.set_tuning(key, bad)
            assert e.value.status == -1


def test_bfs_pull_over_forward_with_sinks(gbx, cuda_device):
    """No inverse CSR (the reference's DIRECTED 0 pull over out-edges) on a
    directed RMAT graph whose out-neighbours include sinks: the bottom-up
    frontier bitmap must then hold the frontier's out-degree-0 vertices too.
    Levels here depend on the direction schedule, so the reference's
    thresholds stay in place and the autotuner leaves them alone."""
    scale = 14
    src, dst = gbx.generate_rmat(scale, (1 << scale) * 8, seed=21)
    V = 1 << scale
    deg, idx, s, d, _ = gbx.csr_build(src, dst, num_vertices=V, dedup=True, sort=1)
    assert np.any(deg[d] == 0)  # some out-neighbour is a sink
    g = gbx.GraphCSR(V, int(s.shape[0]), deg, idx, d, s, None, np.arange(V, dtype=np.uint32),
                     np.arange(V, dtype=np.uint32))
    host = po.HostCSR(V, deg, idx, d)
    rng = np.random.default_rng(3)
    with gbx.DeviceGraph.from_graph_csr(g) as dg:
        tuned = dg.autotune(bfs=True, sssp=False, samples=2)
        assert (tuned["bfs_alpha"], tuned["bfs_beta"]) == (15, 18)
        for r in [0] + [int(x) for x in rng.choice(np.nonzero(deg)[0], 6)]:
            dd, _, proc, it = po.bfs(host, r, None)
            st = gbx.breadth_first_search(dg, r)
            np.testing.assert_array_equal(st.distances, dd)
            assert (st.processed_nodes, st.iteration) == (proc, it)


@pytest.mark.parametrize("delta", [1, 8, 64, 100, 200])
def test_sssp_bucket_widths(gbx, cuda_device, delta):
    """Weighted RMAT with hubs (rows longer than two work chunks): narrow
    buckets (many bucket moves, far pile refills) to wide ones; the distances
    are the unique fixed point whatever the schedule."""
    g = _rmat_graph(gbx, 16, 16, 31, weights="int")
    host, _ = host_views(g)
    assert int(g.out_degree.max()) > 2048
    rng = np.random.default_rng(delta)
    roots = [0] + [int(r) for r in rng.choice(np.nonzero(g.out_degree)[0], 3)]
    with gbx.DeviceGraph.from_graph_csr(g) as dg:
        for r in roots:
            st = gbx.sssp(dg, r, delta)
            np.testing.assert_array_equal(st.distances, po.sssp(host, r, 64))


def _bottom_up_levels(deg, idx, dest, V, source):
    """Pull-only BFS over out-edges (the reference's DIRECTED 0 bottom-up
    step, BFS.c:562-613, run from the first level): v joins level L+1 when
    one of its out-neighbours is in level L."""
    dist = np.zeros(V, np.int64)
    seen = np.zeros(V, bool)
    seen[source] = True
    frontier = np.zeros(V, bool)
    frontier[source] = True
    level = 0
    while True:
        nxt = np.zeros(V, bool)
        for v in np.nonzero(~seen)[0]:
            row = dest[idx[v]:idx[v] + deg[v]]
            if row.size and frontier[row].any():
                nxt[v] = True
        if not nxt.any():
            return dist, int(seen.sum())
        level += 1
        dist[nxt] = level
        seen |= nxt
        frontier = nxt


def test_bfs_pull_only_level_scan(gbx, cuda_device):
    """Mode 0 (bottom-up from the first step) on an asymmetric graph without
    an inverse CSR and with sinks: the first frontier bitmap comes from the
    level scan, where unreached vertices (level 0 in the output format) must
    not count as level-0 frontier."""
    scale = 10
    src, dst = gbx.generate_rmat(scale, (1 << scale) * 8, seed=23)
    V = 1 << scale
    deg, idx, s, d, _ = gbx.csr_build(src, dst, num_vertices=V, dedup=True, sort=1)
    assert np.any(deg[d] == 0)
    g = gbx.GraphCSR(V, int(s.shape[0]), deg, idx, d, s, None, np.arange(V, dtype=np.uint32),
                     np.arange(V, dtype=np.uint32))
    with gbx.DeviceGraph.from_graph_csr(g) as dg:
        for r in [0, 5, int(np.nonzero(deg)[0][-1])]:
            ref, reached = _bottom_up_levels(deg, idx, d, V, r)
            st = gbx.breadth_first_search(dg, r, 0)
            np.testing.assert_array_equal(np.asarray(st.distances).astype(np.int64), ref)
            assert st.processed_nodes == reached


@pytest.mark.parametrize("name", GOLDEN_GRAPHS)
@pytest.mark.parametrize("variant", ["u", "dw"])
def test_reorder_modes_golden(gbx, cuda_device, name, variant):
    """In/in+out degree, DBG, HUBSort, HUBCluster and Corder on the GPU
    against the reference's labels, on the CSR the reference reorders."""
    fx = load_golden(name)
    rm = load_reorder_modes()
    V = int(fx[f"{variant}_num_vertices"])
    for lm in REORDER_MODES:
        el = gbx.EdgeList(V, fx[f"{variant}_src"].copy(), fx[f"{variant}_dest"].copy())
        gbx.degree_reorder(el, lm)
        lab = rm[f"{name}_{variant}_l{lm}"]
        np.testing.assert_array_equal(el.label_array, lab, err_msg=f"lmode {lm}")
        np.testing.assert_array_equal(el.inverse_label_array[lab], np.arange(V, dtype=np.uint32))
        np.testing.assert_array_equal(el.src, lab[fx[f"{variant}_src"]])
        np.testing.assert_array_equal(el.dst, lab[fx[f"{variant}_dest"]])


@pytest.mark.parametrize("lmode", [1, 2, 3, 4, 5, 6, 7, 8, 9, 12, 13])
def test_reorder_modes_rmat(gbx, cuda_device, lmode):
    """Every mode on a deduplicated RMAT-16 edge list (hubs above all DBG
    thresholds, many degree-0 vertices) against the oracle."""
    src, dst = gbx.generate_rmat(16, (1 << 16) * 16, seed=41)
    V = 1 << 16
    _, _, s, d, _ = gbx.csr_build(src, dst, num_vertices=V, dedup=True, sort=1)
    rs, rd, rlab, rinv = po.degree_reorder(V, s, d, lmode=lmode)
    el = gbx.EdgeList(V, s.copy(), d.copy())
    gbx.degree_reorder(el, lmode)
    np.testing.assert_array_equal(el.label_array, rlab)
    np.testing.assert_array_equal(el.inverse_label_array, rinv)
    np.testing.assert_array_equal(el.src, rs)
    np.testing.assert_array_equal(el.dst, rd)


def test_relabel_explicit_and_rejected(gbx, cuda_device, tmp_path):
    """lmode 11: labels from the reference's label file; a label list that
    is not a permutation, and the non-reproducible random mode, are errors."""
    src, dst = gbx.generate_rmat(12, 1 << 15, seed=43)
    V = 1 << 12
    perm = np.random.default_rng(4).permutation(V).astype(np.uint32)
    f = tmp_path / "labels.txt"
    f.write_text("".join(f"{x}\n" for x in perm))
    el = gbx.relabel_from_file(gbx.EdgeList(V, src.copy(), dst.copy()), str(f))
    np.testing.assert_array_equal(el.src, perm[src])
    np.testing.assert_array_equal(el.dst, perm[dst])
    np.testing.assert_array_equal(el.label_array, perm)
    np.testing.assert_array_equal(el.inverse_label_array[perm], np.arange(V, dtype=np.uint32))
    # composition: a second relabelling maps the composed labels
    perm2 = np.roll(np.arange(V, dtype=np.uint32), 5)
    gbx.relabel(el, perm2)
    np.testing.assert_array_equal(el.label_array, perm2[perm])
    np.testing.assert_array_equal(el.src, perm2[perm[src]])
    bad = perm.copy()
    bad[7] = bad[8]
    with pytest.raises(gbx.GbxError) as e:
        gbx.relabel(gbx.EdgeList(V, src.copy(), dst.copy()), bad)
    assert e.value.status == -1
    with pytest.raises(gbx.GbxError) as e:
        gbx.degree_reorder(gbx.EdgeList(V, src.copy(), dst.copy()), 10)
    assert e.value.status == -6
