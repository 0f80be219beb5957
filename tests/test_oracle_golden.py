"""The CPU oracle against the reference's golden vectors (no GPU).

Pins oracle/gbx_oracle.c to (a) the reference's own CSR text dumps in
03_data/TEST and (b) outputs of the reference host, both stored in
tests/golden/*.npz by tests/golden/make_golden.py.
"""
import numpy as np
import pytest

from conftest import GOLDEN_GRAPHS, REORDER_MODES, load_golden, load_reorder_modes
from oracle import pyoracle as po

VARIANTS = [("u", True, True), ("dw", False, False), ("dwk", False, True)]


def _inputs(fx, variant, symmetric):
    src, dst = fx["src"], fx["dst"]
    w = fx.get("weight")
    if variant == "u":
        w = None  # WEIGHTED 0 build ignores weights
    elif w is None:
        w = np.ones(src.shape[0], np.float32)
    if symmetric:
        src, dst = np.concatenate([src, dst]), np.concatenate([dst, src])
        if w is not None:
            w = np.concatenate([w, w])
    V = int(max(src.max(), dst.max())) + 1
    return V, src, dst, w


def oracle_graph(fx, variant, symmetric, dedup):
    V, src, dst, w = _inputs(fx, variant, symmetric)
    g = po.build_csr(V, src, dst, w, sort_mode=1, dedup=dedup)
    pull = None
    if variant != "u":
        pull = po.build_csr(V, g.dest, g.src, g.weight, sort_mode=1)
    return g, pull


@pytest.mark.parametrize("name", GOLDEN_GRAPHS)
def test_reference_dump_matches_reference_build(name):
    fx = load_golden(name)
    if "dump_out_degree" not in fx:
        pytest.skip("no CSR text dump shipped for this graph")
    # the shipped dumps were made from the directed graph with -o 1 (plus -s/-k on some)
    for v in ("dw", "dwk", "u"):
        if np.array_equal(fx["dump_out_degree"], fx[f"{v}_out_degree"]) and np.array_equal(
                fx["dump_dest"], fx[f"{v}_dest"]):
            assert np.array_equal(fx["dump_edges_idx"], fx[f"{v}_edges_idx"])
            return
    pytest.fail("no reference build variant reproduces the shipped CSR dump")


@pytest.mark.parametrize("name", GOLDEN_GRAPHS)
@pytest.mark.parametrize("variant,symmetric,dedup", VARIANTS)
def test_oracle_csr(name, variant, symmetric, dedup):
    fx = load_golden(name)
    g, _ = oracle_graph(fx, variant, symmetric, dedup)
    assert g.num_vertices == int(fx[f"{variant}_num_vertices"])
    np.testing.assert_array_equal(g.out_degree, fx[f"{variant}_out_degree"])
    np.testing.assert_array_equal(g.edges_idx, fx[f"{variant}_edges_idx"])
    np.testing.assert_array_equal(g.dest, fx[f"{variant}_dest"])
    np.testing.assert_array_equal(g.src, fx[f"{variant}_src"])
    if f"{variant}_weight" in fx:
        np.testing.assert_array_equal(g.weight, fx[f"{variant}_weight"])


@pytest.mark.parametrize("name", GOLDEN_GRAPHS)
@pytest.mark.parametrize("variant,symmetric,dedup", VARIANTS)
def test_oracle_algorithms(name, variant, symmetric, dedup):
    fx = load_golden(name)
    g, pull = oracle_graph(fx, variant, symmetric, dedup)
    for dist, meta in zip(fx[f"{variant}_bfs_distances"], fx[f"{variant}_bfs_meta"]):
        d, _, proc, it = po.bfs(g, int(meta[1]), pull)
        np.testing.assert_array_equal(d, dist)
        assert proc == meta[2] and it == meta[3]
    r, _, _ = po.pagerank(g, 20, 0.0, pull)
    np.testing.assert_array_equal(r, fx[f"{variant}_pr20"])  # bit-exact FP32
    r, its, _ = po.pagerank(g, 100, 1e-4, pull)
    assert its == int(fx[f"{variant}_pr_eps_iterations"])
    np.testing.assert_array_equal(r, fx[f"{variant}_pr_eps"])
    dist = po.sssp(g, int(fx[f"{variant}_sssp_source"]), 1, use_weights=(variant != "u"))
    np.testing.assert_array_equal(dist, fx[f"{variant}_sssp"])
    np.testing.assert_array_equal(po.cc(g, 1, pull), fx[f"{variant}_cc"])
    np.testing.assert_array_equal(po.cc(g, 0, pull), fx[f"{variant}_cc"])
    np.testing.assert_array_equal(po.cc(g, 2, pull), fx[f"{variant}_cc"])
    vals = None if variant == "u" else pull.weight
    y = po.spmv(g, fx[f"{variant}_spmv_x"], vals, 0.0001, 2, pull=pull)
    np.testing.assert_array_equal(y, fx[f"{variant}_spmv_y"])
    if variant == "u":
        assert po.triangle_count(g) == int(fx["u_tc"])


@pytest.mark.parametrize("name", GOLDEN_GRAPHS)
@pytest.mark.parametrize("variant,symmetric,dedup", VARIANTS)
def test_oracle_degree_reorder(name, variant, symmetric, dedup):
    fx = load_golden(name)
    V, src, dst, w = _inputs(fx, variant, symmetric)
    g = po.build_csr(V, src, dst, w, sort_mode=1, dedup=dedup)
    s, d, lab, inv = po.degree_reorder(V, g.src, g.dest, lmode=1)
    np.testing.assert_array_equal(lab, fx[f"{variant}_reorder_label"])
    np.testing.assert_array_equal(inv[lab], np.arange(V, dtype=np.uint32))
    g2 = po.build_csr(V, s, d, sort_mode=1)
    np.testing.assert_array_equal(g2.dest, fx[f"{variant}_reorder_dest"])
    np.testing.assert_array_equal(g2.out_degree, fx[f"{variant}_reorder_out_degree"])


@pytest.mark.parametrize("name", GOLDEN_GRAPHS)
@pytest.mark.parametrize("variant", ["u", "dw"])
def test_oracle_reorder_modes(name, variant):
    """In/in+out degree, DBG, HUBSort, HUBCluster and Corder labels of the
    reference on the CSR it reorders (the reference's own build output)."""
    fx = load_golden(name)
    rm = load_reorder_modes()
    V = int(fx[f"{variant}_num_vertices"])
    for lm in REORDER_MODES:
        s, d, lab, inv = po.degree_reorder(V, fx[f"{variant}_src"], fx[f"{variant}_dest"], lmode=lm)
        np.testing.assert_array_equal(lab, rm[f"{name}_{variant}_l{lm}"], err_msg=f"lmode {lm}")
        np.testing.assert_array_equal(inv[lab], np.arange(V, dtype=np.uint32))
        np.testing.assert_array_equal(s, lab[fx[f"{variant}_src"]])
        np.testing.assert_array_equal(d, lab[fx[f"{variant}_dest"]])


@pytest.mark.skipif(not po.ref_available("dw"), reason="reference build (oracle/_ref) not present")
def test_oracle_vs_reference_on_rmat(tmp_path):
    """Fresh inputs, not only the shipped ones: an RMAT graph written in the
    reference's .bin format and run through the reference host itself."""
    from graphblox_gb300.graph import generate_rmat, write_edge_list_bin

    src, dst = generate_rmat(11, 1 << 14, seed=3)
    f = tmp_path / "g.bin"
    write_edge_list_bin(str(f), src, dst)
    V = int(max(src.max(), dst.max())) + 1
    g = po.build_csr(V, src, dst, np.ones(src.shape[0], np.float32), sort_mode=1, dedup=True)
    pull = po.build_csr(V, g.dest, g.src, g.weight, sort_mode=1)
    for root in (0, 5):
        out = po.ref_run(f, "dw", 0, ["-o", "1", "-k", "-p", "2", "-r", str(root)])
        d, _, proc, it = po.bfs(g, out["source"], pull)
        np.testing.assert_array_equal(d, out["bfs_distances"])
        assert (proc, it) == (out["processed_nodes"], out["iteration"])
    out = po.ref_run(f, "dw", 1, ["-o", "1", "-k", "-i", "20", "-e", "0"])
    r, _, _ = po.pagerank(g, 20, 0.0, pull)
    np.testing.assert_array_equal(r, out["pr_ranks"])
