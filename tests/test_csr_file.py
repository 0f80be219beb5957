"""The reference's binary CSR file (.csr, graphCSR.c:458-529 writer,
graphCSR.c:638-744 reader) against the files the reference itself wrote
(tests/golden/csr_files.npz).

CPU: the reader parses every reference file into the CSR arrays of the
reference build (<graph>.npz), the writer gives the same bytes back, and the
oracle's CSR build (forward and inverse) written out is byte-identical.
GPU: the library's CSR build (graph_csr_preprocessing) written out is
byte-identical to the reference's file.
"""
import numpy as np
import pytest

import graphblox_gb300 as gbx
from conftest import load_csr_files, load_golden
from oracle import pyoracle as po

CSR_FILES = load_csr_files()
KEYS = sorted(CSR_FILES)
# variant -> (symmetric read, dedup, WEIGHTED build, DIRECTED build)
BUILDS = {"u": (True, True, False, False), "dw": (False, False, True, True), "dwk": (False, True, True, True)}


def _split(key):
    name, variant = key.rsplit("_", 1)
    return name, variant


def _max_weight(fx):
    w = fx.get("weight")
    return float(max(0.0, float(w.max()))) if w is not None else 1.0


def _write_bytes(tmp_path, g, weighted, directed):
    path = gbx.write_graph_csr_bin(str(tmp_path / "graph"), g, weighted=weighted, directed=directed)
    assert path.endswith("graph.csr")
    return np.fromfile(path, dtype=np.uint8)


@pytest.mark.parametrize("key", KEYS)
def test_read_reference_csr_file(tmp_path, key):
    name, variant = _split(key)
    fx = load_golden(name)
    _, _, weighted, directed = BUILDS[variant]
    f = tmp_path / "ref.csr"
    CSR_FILES[key].tofile(f)
    g = gbx.read_graph_csr_bin(str(f))  # layout inferred from the size
    assert (g.weight is not None) == weighted and g.directed == directed
    assert g.num_vertices == int(fx[f"{variant}_num_vertices"])
    np.testing.assert_array_equal(g.out_degree, fx[f"{variant}_out_degree"])
    np.testing.assert_array_equal(g.edges_idx, fx[f"{variant}_edges_idx"])
    np.testing.assert_array_equal(g.dest, fx[f"{variant}_dest"])
    np.testing.assert_array_equal(g.src, fx[f"{variant}_src"])
    if weighted:
        np.testing.assert_array_equal(g.weight, fx[f"{variant}_weight"])
        assert g.max_weight == _max_weight(fx)
    if directed:
        # the inverse CSR is the transpose: same edge multiset, grouped by dest
        V = g.num_vertices
        np.testing.assert_array_equal(g.inverse_out_degree, np.bincount(g.dest, minlength=V))
        np.testing.assert_array_equal(g.inverse_src, np.repeat(np.arange(V), g.inverse_out_degree))
        fwd = np.sort(g.src.astype(np.uint64) << 32 | g.dest)
        inv = np.sort(g.inverse_dest.astype(np.uint64) << 32 | g.inverse_src)
        np.testing.assert_array_equal(fwd, inv)
    # reading with the build named explicitly gives the same graph; a wrong build is rejected
    g2 = gbx.read_graph_csr_bin(str(f), weighted=weighted, directed=directed)
    np.testing.assert_array_equal(g2.dest, g.dest)
    with pytest.raises(ValueError):
        gbx.read_graph_csr_bin(str(f), weighted=not weighted, directed=directed)


@pytest.mark.parametrize("key", KEYS)
def test_write_round_trip_is_byte_exact(tmp_path, key):
    _, variant = _split(key)
    _, _, weighted, directed = BUILDS[variant]
    f = tmp_path / "ref.csr"
    CSR_FILES[key].tofile(f)
    g = gbx.read_graph_csr_bin(str(f))
    np.testing.assert_array_equal(_write_bytes(tmp_path, g, weighted, directed), CSR_FILES[key])


@pytest.mark.parametrize("key", KEYS)
def test_oracle_csr_build_writes_reference_file(tmp_path, key):
    """Pins the oracle's forward AND inverse CSR build (the inverse is not in
    the text dumps) to the reference's file."""
    name, variant = _split(key)
    fx = load_golden(name)
    symmetric, dedup, weighted, directed = BUILDS[variant]
    src, dst = fx["src"], fx["dst"]
    w = fx.get("weight")
    w = np.ones(src.shape[0], np.float32) if w is None else w
    if symmetric:
        src, dst, w = np.concatenate([src, dst]), np.concatenate([dst, src]), np.concatenate([w, w])
    V = int(max(src.max(), dst.max())) + 1
    h = po.build_csr(V, src, dst, w if weighted else None, sort_mode=1, dedup=dedup)
    ident = np.arange(V, dtype=np.uint32)
    g = gbx.GraphCSR(V, h.num_edges, h.out_degree, h.edges_idx, h.dest, h.src, h.weight, ident, ident.copy(),
                     max_weight=_max_weight(fx))
    if directed:
        p = po.build_csr(V, h.dest, h.src, h.weight, sort_mode=1)
        g.inverse_out_degree, g.inverse_edges_idx = p.out_degree, p.edges_idx
        g.inverse_dest, g.inverse_src, g.inverse_weight = p.dest, p.src, p.weight
    np.testing.assert_array_equal(_write_bytes(tmp_path, g, weighted, directed), CSR_FILES[key])


def test_malformed_csr_files_rejected(tmp_path):
    f = tmp_path / "bad.csr"
    np.zeros(1, np.uint32).tofile(f)  # shorter than the header
    with pytest.raises(ValueError):
        gbx.read_graph_csr_bin(str(f))
    good = CSR_FILES["v51_e1021_dw"]
    good[:-4].tofile(f)  # truncated: no layout fits
    with pytest.raises(ValueError):
        gbx.read_graph_csr_bin(str(f))
    g = gbx.GraphCSR(2, 1, np.array([1, 0], np.uint32), np.zeros(2, np.uint32), np.array([1], np.uint32),
                     np.array([0], np.uint32), None, np.arange(2, dtype=np.uint32), np.arange(2, dtype=np.uint32))
    with pytest.raises(ValueError):
        gbx.write_graph_csr_bin(str(tmp_path / "x"), g, weighted=True)
    with pytest.raises(ValueError):
        gbx.write_graph_csr_bin(str(tmp_path / "x"), g, directed=True)


@pytest.mark.gpu
@pytest.mark.parametrize("key", KEYS)
def test_gpu_csr_build_writes_reference_file(tmp_path, key):
    """read_edge_list_bin -> graph_csr_preprocessing (the GPU CSR build,
    forward and inverse) -> write_graph_csr_bin gives the reference's bytes."""
    name, variant = _split(key)
    fx = load_golden(name)
    symmetric, dedup, weighted, directed = BUILDS[variant]
    inp = tmp_path / ("graph.wbin" if "weight" in fx else "graph.bin")
    gbx.write_edge_list_bin(str(inp), fx["src"], fx["dst"], fx.get("weight"))
    el = gbx.read_edge_list_bin(str(inp), symmetric=symmetric, weighted="weight" in fx)
    g = gbx.graph_csr_preprocessing(el, sort=1, dedup=dedup, directed=directed, keep_weights=weighted)
    np.testing.assert_array_equal(_write_bytes(tmp_path, g, weighted, directed), CSR_FILES[key])
