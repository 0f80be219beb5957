"""Bellman-Ford, DFS and betweenness centrality against the reference host
(tests/golden/bf_dfs_bc.npz) and the oracle.

CPU: the oracle's restatements (MT19937 root draw, Brandes, stack DFS, and
SSSP for Bellman-Ford's distances) reproduce the reference's outputs bit
for bit. GPU: gbx_betweenness / gbx_dfs / gbx_bellman_ford do too, on the
test graphs and on RMAT graphs with and without an inverse CSR.
"""
import numpy as np
import pytest

from conftest import GOLDEN_GRAPHS, load_bf_dfs_bc, load_golden
from oracle import pyoracle as po

FX = load_bf_dfs_bc()
VARIANTS = [("u", True, True), ("dw", False, False), ("dwk", False, True)]
BC_VARIANTS = [v for v in VARIANTS if v[0] != "u"]


def _host(fx, variant, with_weights=False):
    """The reference's CSR of <variant> from the fixture, its inverse built
    by the oracle for the DIRECTED build."""
    V = int(fx[f"{variant}_num_vertices"])
    w = fx.get(f"{variant}_weight") if with_weights else None
    g = po.HostCSR(V, fx[f"{variant}_out_degree"], fx[f"{variant}_edges_idx"], fx[f"{variant}_dest"], w,
                   fx[f"{variant}_src"])
    pull = None
    if variant != "u":
        pull = po.build_csr(V, g.dest, g.src, w, sort_mode=1)
    return g, pull


def _bits(a):
    return np.asarray(a, np.float32).view(np.uint32)


def _cheap_draw(g, n):
    """The reference draws 32-bit values until one names a vertex with an
    out-degree above the average: about n * 2^32 / (such vertices) draws.
    The draw is checked where that stays below ~1e8 draws; elsewhere the
    tests take the reference's recorded roots."""
    k = int(np.count_nonzero(np.asarray(g.out_degree) > g.num_edges // g.num_vertices))
    return k > 0 and n * (2.0 ** 32) / k <= 1e8


@pytest.mark.parametrize("name", GOLDEN_GRAPHS)
@pytest.mark.parametrize("variant,symmetric,dedup", BC_VARIANTS)
def test_oracle_betweenness(name, variant, symmetric, dedup):
    fx = load_golden(name)
    key = f"{name}_{variant}"
    g, pull = _host(fx, variant)
    roots = FX[f"{key}_bc_roots"]
    if _cheap_draw(g, len(roots)):
        np.testing.assert_array_equal(po.random_roots(g, len(roots)), roots)
    bc, dist, sig, dep, proc = po.betweenness(g, roots, pull)
    np.testing.assert_array_equal(_bits(bc), _bits(FX[f"{key}_bc"]))
    np.testing.assert_array_equal(dist, FX[f"{key}_bc_distances"])
    np.testing.assert_array_equal(sig, FX[f"{key}_bc_sigma"])
    np.testing.assert_array_equal(_bits(dep), _bits(FX[f"{key}_bc_dependency"]))
    assert proc == int(FX[f"{key}_bc_processed"])


@pytest.mark.parametrize("name", GOLDEN_GRAPHS)
@pytest.mark.parametrize("variant,symmetric,dedup", VARIANTS)
def test_oracle_dfs_and_bellman_ford(name, variant, symmetric, dedup):
    fx = load_golden(name)
    key = f"{name}_{variant}"
    g, _ = _host(fx, variant, with_weights=True)
    for r in (0, 1):
        if r >= g.num_vertices:
            continue
        d, p, n = po.dfs(g, r)
        np.testing.assert_array_equal(d, FX[f"{key}_dfs_r{r}"])
        np.testing.assert_array_equal(p, FX[f"{key}_dfs_parents_r{r}"])
        assert n == int(FX[f"{key}_dfs_processed_r{r}"])
    if g.num_vertices > 1:
        np.testing.assert_array_equal(po.sssp(g, 1, 64), FX[f"{key}_bf_r1"])


# ---------------------------------------------------------------------------- GPU


def _device_graph(gbx, fx, variant, with_weights=True):
    g, pull = _host(fx, variant, with_weights)
    V = g.num_vertices
    ident = np.arange(V, dtype=np.uint32)
    G = gbx.GraphCSR(V, g.num_edges, g.out_degree, g.edges_idx, g.dest, g.src, g.weight, ident, ident.copy())
    if pull is not None:
        G.inverse_out_degree, G.inverse_edges_idx = pull.out_degree, pull.edges_idx
        G.inverse_dest, G.inverse_weight = pull.dest, pull.weight
    return G, g, pull


def _min_parents(g, dist, source):
    """Smallest u with u->v and (uint32)((float)d[u] + w) == d[v]."""
    V = g.num_vertices
    src = np.repeat(np.arange(V, dtype=np.uint32), g.out_degree)
    # rows are in vertex order in these CSRs, so src lines up with dest
    w = g.weight if g.weight is not None else np.ones(g.num_edges, np.float32)
    du = dist[src]
    ok = du != 0x7FFFFFFF
    nd = (du.astype(np.float32) + w).astype(np.uint32)
    hit = ok & (nd == dist[g.dest]) & (g.dest != source)
    par = np.full(V, 0xFFFFFFFF, np.uint64)
    np.minimum.at(par, g.dest[hit], src[hit].astype(np.uint64))
    par[source] = source
    return par.astype(np.uint32)


@pytest.mark.gpu
@pytest.mark.parametrize("name", GOLDEN_GRAPHS)
@pytest.mark.parametrize("variant,symmetric,dedup", BC_VARIANTS)
def test_gpu_betweenness_golden(gbx, cuda_device, name, variant, symmetric, dedup):
    fx = load_golden(name)
    key = f"{name}_{variant}"
    G, g, _ = _device_graph(gbx, fx, variant)
    roots = FX[f"{key}_bc_roots"]
    with gbx.DeviceGraph.from_graph_csr(G) as dg:
        if _cheap_draw(g, len(roots)):
            np.testing.assert_array_equal(gbx.reference_roots(dg, len(roots)), roots)
        st = gbx.betweenness_centrality(dg, roots=roots)
    np.testing.assert_array_equal(_bits(st.betweennessCentrality), _bits(FX[f"{key}_bc"]))
    np.testing.assert_array_equal(st.distances, FX[f"{key}_bc_distances"])
    np.testing.assert_array_equal(st.sigma, FX[f"{key}_bc_sigma"])
    np.testing.assert_array_equal(_bits(st.dependency), _bits(FX[f"{key}_bc_dependency"]))
    assert st.processed_nodes == int(FX[f"{key}_bc_processed"])
    assert st.iteration == len(roots)


@pytest.mark.gpu
@pytest.mark.parametrize("name", GOLDEN_GRAPHS)
@pytest.mark.parametrize("variant,symmetric,dedup", VARIANTS)
def test_gpu_dfs_and_bellman_ford_golden(gbx, cuda_device, name, variant, symmetric, dedup):
    fx = load_golden(name)
    key = f"{name}_{variant}"
    G, g, _ = _device_graph(gbx, fx, variant)
    with gbx.DeviceGraph.from_graph_csr(G, use_weights=variant != "u") as dg:
        for r in (0, 1):
            if r >= g.num_vertices:
                continue
            st = gbx.depth_first_search(dg, r)
            np.testing.assert_array_equal(st.distances, FX[f"{key}_dfs_r{r}"])
            np.testing.assert_array_equal(st.parents, FX[f"{key}_dfs_parents_r{r}"])
            assert st.processed_nodes == int(FX[f"{key}_dfs_processed_r{r}"])
        if g.num_vertices > 1:
            bf = gbx.bellman_ford(dg, 1)
            np.testing.assert_array_equal(bf.distances, FX[f"{key}_bf_r1"])
            hw = g if variant != "u" else po.HostCSR(g.num_vertices, g.out_degree, g.edges_idx, g.dest, None, g.src)
            np.testing.assert_array_equal(bf.parents, _min_parents(hw, bf.distances, 1))


def _rmat(gbx, scale, ef, seed, directed, inverse, weights=False):
    V = 1 << scale
    src, dst = gbx.generate_rmat(scale, V * ef, seed=seed)
    w = gbx.generate_values(src.shape[0], 0, 1, 255, seed=seed + 3) if weights else None
    if not directed:
        src, dst = np.concatenate([src, dst]), np.concatenate([dst, src])
        w = None if w is None else np.concatenate([w, w])
    el = gbx.EdgeList(V, src, dst, w)
    return gbx.graph_csr_preprocessing(el, sort=1, dedup=True, directed=inverse, keep_weights=weights)


@pytest.mark.gpu
@pytest.mark.parametrize("directed,inverse", [(True, True), (True, False), (False, False)])
def test_gpu_betweenness_rmat(gbx, cuda_device, directed, inverse):
    """With an inverse CSR the successors are the forward rows; without one
    (pull over the forward CSR, as the reference's DIRECTED 0 build) the
    library builds the transpose."""
    g = _rmat(gbx, 12, 8, 21, directed, inverse)
    host = po.HostCSR(g.num_vertices, g.out_degree, g.edges_idx, g.dest, None, g.src)
    pull = None
    if inverse:
        pull = po.HostCSR(g.num_vertices, g.inverse_out_degree, g.inverse_edges_idx, g.inverse_dest)
    with gbx.DeviceGraph.from_graph_csr(g) as dg:
        roots = gbx.reference_roots(dg, 6)
        np.testing.assert_array_equal(roots, po.random_roots(host, 6))
        st = gbx.betweenness_centrality(dg, roots=roots)
        # accumulation into a caller array continues the sum
        again = gbx.betweenness_centrality(dg, roots=roots[:2], centrality=st.betweennessCentrality.copy())
    bc, dist, sig, dep, proc = po.betweenness(host, roots, pull)
    np.testing.assert_array_equal(_bits(st.betweennessCentrality), _bits(bc))
    np.testing.assert_array_equal(st.distances, dist)
    np.testing.assert_array_equal(st.sigma, sig)
    np.testing.assert_array_equal(_bits(st.dependency), _bits(dep))
    assert st.processed_nodes == proc
    bc2, *_ = po.betweenness(host, np.concatenate([roots, roots[:2]]), pull)
    np.testing.assert_array_equal(_bits(again.betweennessCentrality), _bits(bc2))


@pytest.mark.gpu
def test_gpu_dfs_and_bellman_ford_rmat(gbx, cuda_device):
    g = _rmat(gbx, 13, 8, 5, True, True, weights=True)
    host = po.HostCSR(g.num_vertices, g.out_degree, g.edges_idx, g.dest, g.weight, g.src)
    with gbx.DeviceGraph.from_graph_csr(g) as dg:
        for r in (0, 3, 77):
            st = gbx.depth_first_search(dg, r)
            d, p, n = po.dfs(host, r)
            np.testing.assert_array_equal(st.distances, d)
            np.testing.assert_array_equal(st.parents, p)
            assert st.processed_nodes == n
            bf = gbx.bellman_ford(dg, r)
            np.testing.assert_array_equal(bf.distances, po.sssp(host, r, 64))
            np.testing.assert_array_equal(bf.parents, _min_parents(host, bf.distances, r))


@pytest.mark.gpu
def test_gpu_bc_dfs_bf_reject_bad_sources(gbx, cuda_device):
    g = _rmat(gbx, 8, 4, 1, True, True)
    with gbx.DeviceGraph.from_graph_csr(g) as dg:
        V = dg.num_vertices
        for f in (lambda: gbx.depth_first_search(dg, V), lambda: gbx.bellman_ford(dg, V, map_source=False),
                  lambda: gbx.betweenness_centrality(dg, roots=[0, V])):
            with pytest.raises(gbx.GbxError) as e:
                f()
            assert e.value.status == -1
