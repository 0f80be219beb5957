"""Mask mode (the reference's -M / -C, maskGraphProcess, reorder.c:1164-1475)
against the reference run with one thread (tests/golden/mask_modes.npz).

CPU: the oracle's hints on every test graph, build variant, mode and cache
size; the oracle's masked CSR (forward, and the inverse sorted on the
masked ids) written as a .csr file is byte-identical to the reference's.
GPU: gbx_mask_graph's hints; graph_csr_preprocessing(mmode=...) written
out byte-identical; BFS and PageRank on the masked graph, whose inverse
CSR has its runs out of vertex order (repacked by the upload).
"""
import re

import numpy as np
import pytest

import graphblox_gb300 as gbx
from conftest import load_golden, load_mask_modes
from oracle import pyoracle as po

MASK = load_mask_modes()
HINT_KEYS = sorted(k for k in MASK if re.search(r"_m\d_c\d+$", k))
CSR_KEYS = sorted(k for k in MASK if k.endswith("_csr"))
ALGO_GRAPHS = sorted({k[: -len("_dw_m1_bfs1")] for k in MASK if k.endswith("_dw_m1_bfs1")})
REL_L1_TOL = 1e-6


def _hint_case(key):
    name, variant, m, c = re.fullmatch(r"(.+)_(u|dw)_m(\d)_c(\d+)", key).groups()
    return name, variant, int(m), int(c)


def _csr_case(key):
    name, variant, m = re.fullmatch(r"(.+)_(u|dw)_m(\d)_csr", key).groups()
    return name, variant, int(m)


def _edges(fx, variant):
    return int(fx[f"{variant}_num_vertices"]), fx[f"{variant}_src"], fx[f"{variant}_dest"]


def _max_weight(fx):
    w = fx.get("weight")
    return float(max(0.0, float(w.max()))) if w is not None else 1.0


@pytest.mark.parametrize("key", HINT_KEYS)
def test_oracle_mask_hints(key):
    name, variant, m, cs = _hint_case(key)
    V, s, d = _edges(load_golden(name), variant)
    s2, d2, mask = po.mask_graph(V, s, d, m, cs)
    np.testing.assert_array_equal((mask >> 30).astype(np.uint8), MASK[key])
    if m in (1, 2):
        np.testing.assert_array_equal(s2, s | mask[s])
        np.testing.assert_array_equal(d2, d | mask[d])
    else:
        np.testing.assert_array_equal(d2, d)


def _oracle_masked_graph(fx, variant, m):
    V, s, d = _edges(fx, variant)
    s2, d2, mask = po.mask_graph(V, s, d, m)
    w = fx.get(f"{variant}_weight") if variant == "dw" else None
    g = gbx.GraphCSR(V, s2.shape[0], fx[f"{variant}_out_degree"], fx[f"{variant}_edges_idx"], d2, s2, w,
                     np.arange(V, dtype=np.uint32), np.arange(V, dtype=np.uint32), max_weight=_max_weight(fx))
    if variant == "dw":
        p = po.build_csr(V, d2, s2, w, sort_mode=1)
        g.inverse_out_degree, g.inverse_edges_idx = p.out_degree, p.edges_idx
        g.inverse_dest, g.inverse_src, g.inverse_weight = p.dest, p.src, p.weight
    return g


@pytest.mark.parametrize("key", CSR_KEYS)
def test_oracle_masked_csr_file(tmp_path, key):
    name, variant, m = _csr_case(key)
    g = _oracle_masked_graph(load_golden(name), variant, m)
    path = gbx.write_graph_csr_bin(str(tmp_path / "graph"), g, weighted=variant == "dw",
                                   directed=variant == "dw")
    np.testing.assert_array_equal(np.fromfile(path, np.uint8), MASK[key])


def test_masked_inverse_runs_out_of_vertex_order():
    """The reference's inverse CSR of a masked list is not in vertex order
    (the case the device upload repacks)."""
    g = _oracle_masked_graph(load_golden("v300_e2730"), "dw", 1)
    nz = g.inverse_out_degree > 0
    assert np.any(np.diff(g.inverse_edges_idx[nz].astype(np.int64)) < 0)


@pytest.mark.gpu
@pytest.mark.parametrize("key", HINT_KEYS)
def test_gpu_mask_hints(gbx, cuda_device, key):
    name, variant, m, cs = _hint_case(key)
    V, s, d = _edges(load_golden(name), variant)
    el = gbx.EdgeList(V, s.copy(), d.copy())
    gbx.mask_graph(el, m, cs)
    np.testing.assert_array_equal((el.mask_array >> 30).astype(np.uint8), MASK[key])
    if m in (1, 2):
        np.testing.assert_array_equal(el.src, s | el.mask_array[s])
        np.testing.assert_array_equal(el.dst, d | el.mask_array[d])
    else:
        np.testing.assert_array_equal(el.dst, d)


@pytest.mark.gpu
@pytest.mark.parametrize("key", CSR_KEYS)
def test_gpu_masked_preprocessing_writes_reference_file(gbx, cuda_device, tmp_path, key):
    name, variant, m = _csr_case(key)
    fx = load_golden(name)
    weighted_input = "weight" in fx
    inp = tmp_path / ("graph.wbin" if weighted_input else "graph.bin")
    gbx.write_edge_list_bin(str(inp), fx["src"], fx["dst"], fx.get("weight"))
    el = gbx.read_edge_list_bin(str(inp), symmetric=variant == "u", weighted=weighted_input)
    g = gbx.graph_csr_preprocessing(el, sort=1, dedup=variant == "u", directed=variant == "dw",
                                    keep_weights=variant == "dw", mmode=m)
    path = gbx.write_graph_csr_bin(str(tmp_path / "graph"), g, weighted=variant == "dw",
                                   directed=variant == "dw")
    np.testing.assert_array_equal(np.fromfile(path, np.uint8), MASK[key])


@pytest.mark.gpu
@pytest.mark.parametrize("name", ALGO_GRAPHS)
def test_gpu_algorithms_on_masked_graph(gbx, cuda_device, name):
    fx = load_golden(name)
    g = _oracle_masked_graph(fx, "dw", 1)
    with gbx.DeviceGraph.from_graph_csr(g) as dg:
        st = gbx.breadth_first_search(dg, 1, pushpull=2)
        np.testing.assert_array_equal(st.distances, MASK[f"{name}_dw_m1_bfs1"])
        pr = gbx.page_rank(dg, 20, 0.0)
    ref = MASK[f"{name}_dw_m1_pr20"].astype(np.float64)
    assert np.abs(np.asarray(pr.pageRanks, np.float64) - ref).sum() <= REL_L1_TOL * np.abs(ref).sum()
    # and against the FP64 restatement on the same graph with the hints cleared
    ID = np.uint32(0x3FFFFFFF)
    host = po.HostCSR(g.num_vertices, g.out_degree, g.edges_idx, g.dest & ID, g.weight, g.src & ID)
    pull = po.HostCSR(g.num_vertices, g.inverse_out_degree, g.inverse_edges_idx, g.inverse_dest & ID,
                      g.inverse_weight, g.inverse_src & ID)
    ref64, _, _ = po.pagerank(host, 20, 0.0, pull, fp64=True)
    assert po.fp32_close(np.asarray(pr.pageRanks), ref64, REL_L1_TOL)[0]
