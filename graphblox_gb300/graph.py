"""Host-side mirror of the reference's graph-load and algorithm interfaces.

Names and argument meanings follow the GraphBlox host:
  EdgeList / read_edge_list_bin   -> struct EdgeList, readEdgeListsbin (edgeList.c:450-706)
  GraphCSR / graph_csr_preprocessing -> struct GraphCSR, graphCSRPreProcessingStep (graphCSR.c:243-327)
  DeviceGraph                     -> the device copy of a GraphCSR (gbx_graph_create_csr)
  breadth_first_search, page_rank, sssp, connected_components, triangle_count, spmv
                                  -> breadthFirstSearchGraphCSR, pageRankGraphCSR, SSSPGraphCSR,
                                     connectedComponentsGraphCSR, triangleCountGraphCSR, SPMVGraphCSR
Every compute step runs in libgbx.so on the GPU; this module only moves
arrays and keeps the reference's bookkeeping (label remapping of sources,
inverse CSR for directed graphs).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _lib
from ._lib import BcResult, BfsResult, PrResult, SsspResult, call

ID_MASK = np.uint32(0x3FFFFFFF)  # EXTRACT_VALUE, reorder.h:23


def _ptr(a) -> Optional[int]:
    """Address of a numpy array (host) or a torch tensor (host or device)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("arrays must be C-contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise ValueError("tensors must be contiguous")
        return a.data_ptr()
    raise TypeError(f"unsupported array type {type(a)!r}")


def _u32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32)


def _f32(a) -> Optional[np.ndarray]:
    return None if a is None else np.ascontiguousarray(a, dtype=np.float32)


# ---------------------------------------------------------------------------
# edge lists


@dataclass
class EdgeList:
    """struct EdgeList (edgeList.h:12-23), host arrays."""
    num_vertices: int
    src: np.ndarray
    dst: np.ndarray
    weight: Optional[np.ndarray] = None
    label_array: Optional[np.ndarray] = None
    inverse_label_array: Optional[np.ndarray] = None
    mask_array: Optional[np.ndarray] = None

    @property
    def num_edges(self) -> int:
        return int(self.src.shape[0])


def read_edge_list_bin(path: str, symmetric: bool = False, weighted: bool = False) -> EdgeList:
    """readEdgeListsbin: `.bin` is (uint32 src, uint32 dst) records, `.wbin`
    adds a float32 weight. symmetric appends every edge reversed; the vertex
    count is the largest id + 1; labels start as the identity."""
    raw = np.fromfile(path, dtype=np.uint32)
    width = 3 if weighted else 2
    n = raw.shape[0] // width
    rec = raw[: n * width].reshape(n, width)
    src = rec[:, 0].copy()
    dst = rec[:, 1].copy()
    w = rec[:, 2].copy().view(np.float32) if weighted else np.ones(n, dtype=np.float32)
    if symmetric:
        src, dst = np.concatenate([src, dst]), np.concatenate([dst, src])
        w = np.concatenate([w, w])
    nv = int(max(src.max(initial=0), dst.max(initial=0))) + 1 if n else 1
    ident = np.arange(nv, dtype=np.uint32)
    return EdgeList(nv, src, dst, w, ident.copy(), ident.copy())


def write_edge_list_bin(path: str, src, dst, weight=None) -> None:
    """Write the reference's binary edge-list format (.bin or .wbin with weights)."""
    src = _u32(src)
    dst = _u32(dst)
    if weight is None:
        rec = np.stack([src, dst], axis=1)
    else:
        rec = np.stack([src, dst, _f32(weight).view(np.uint32)], axis=1)
    np.ascontiguousarray(rec).tofile(path)


# ---------------------------------------------------------------------------
# CSR on the host (result of the GPU preprocessing step)


@dataclass
class GraphCSR:
    """struct GraphCSR (graphCSR.h:14-31) with host arrays. `inverse_*` hold
    the in-edge CSR (the reference's DIRECTED build) or None."""
    num_vertices: int
    num_edges: int
    out_degree: np.ndarray
    edges_idx: np.ndarray
    dest: np.ndarray
    src: np.ndarray
    weight: Optional[np.ndarray]
    label_array: np.ndarray
    inverse_label_array: np.ndarray
    inverse_out_degree: Optional[np.ndarray] = None
    inverse_edges_idx: Optional[np.ndarray] = None
    inverse_dest: Optional[np.ndarray] = None
    inverse_weight: Optional[np.ndarray] = None
    inverse_src: Optional[np.ndarray] = None
    max_weight: float = 0.0
    mask_array: Optional[np.ndarray] = None

    @property
    def avg_degree(self) -> int:
        return self.num_edges // self.num_vertices if self.num_vertices else 0

    @property
    def directed(self) -> bool:
        return self.inverse_dest is not None


def csr_build(src, dst, weight=None, *, num_vertices: int, symmetric: bool = False,
              dedup: bool = False, sort: int = 1, stream=None):
    """gbx_csr_build: stable sort (+ optional symmetrisation and dedup) and
    the per-vertex degree / first-edge arrays. Returns host arrays
    (out_degree, edges_idx, src, dst, weight)."""
    src = _u32(src)
    dst = _u32(dst)
    w = _f32(weight)
    e = src.shape[0]
    cap = 2 * e if symmetric else e
    V = int(num_vertices)
    out_degree = np.zeros(V, np.uint32)
    edges_idx = np.zeros(V, np.uint32)
    so = np.zeros(max(cap, 1), np.uint32)
    do = np.zeros(max(cap, 1), np.uint32)
    wo = np.zeros(max(cap, 1), np.float32) if w is not None else None
    n_out = _lib.u32(0)
    call("gbx_csr_build", e, _ptr(src), _ptr(dst), _ptr(w), int(symmetric), int(dedup), int(sort), V,
         _ptr(out_degree), _ptr(edges_idx), _ptr(so), _ptr(do), _ptr(wo), C.byref(n_out), stream)
    n = n_out.value
    return out_degree, edges_idx, so[:n].copy(), do[:n].copy(), (wo[:n].copy() if wo is not None else None)


def degree_reorder(el: EdgeList, lmode: int = 1, stream=None) -> EdgeList:
    """reorderGraphProcess on the GPU for lmode 1-9, 12, 13 (degree, DBG,
    HUBSort, HUBCluster, Corder): relabels el.src/el.dst in place and
    composes el.label_array / el.inverse_label_array. lmode 11 is
    relabel_from_file; lmode 10 (random) is not reproducible and rejected."""
    V = el.num_vertices
    if el.label_array is None:
        el.label_array = np.arange(V, dtype=np.uint32)
    if el.inverse_label_array is None:
        el.inverse_label_array = np.arange(V, dtype=np.uint32)
    el.src = _u32(el.src)
    el.dst = _u32(el.dst)
    call("gbx_degree_reorder", V, el.num_edges, _ptr(el.src), _ptr(el.dst), int(lmode),
         _ptr(el.label_array), _ptr(el.inverse_label_array), stream)
    return el


def relabel(el: EdgeList, new_labels, stream=None) -> EdgeList:
    """gbx_relabel: new_labels[v] is the new id of v (a permutation of
    [0, V)); relabels el.src/el.dst in place and composes the label arrays
    (relabelEdgeList + label composition, reorder.c:1618-1637,1703-1709)."""
    V = el.num_vertices
    if el.label_array is None:
        el.label_array = np.arange(V, dtype=np.uint32)
    if el.inverse_label_array is None:
        el.inverse_label_array = np.arange(V, dtype=np.uint32)
    el.src = _u32(el.src)
    el.dst = _u32(el.dst)
    nl = _u32(new_labels)
    if nl.shape[0] != V:
        raise ValueError(f"{nl.shape[0]} labels for {V} vertices")
    call("gbx_relabel", V, el.num_edges, _ptr(el.src), _ptr(el.dst), _ptr(nl), _ptr(el.label_array),
         _ptr(el.inverse_label_array), stream)
    return el


def mask_graph(el: EdgeList, mmode: int = 1, cache_size: int = 32768, stream=None) -> EdgeList:
    """maskGraphProcess (the reference's -M, -C): el.mask_array gets the
    hot/warm/lukewarm/cold hint of every vertex (top two id bits); mmode 1
    and 2 also OR the hints into el.src / el.dst. Run after the last sort;
    see gbx_mask_graph for the assignment."""
    el.src = _u32(el.src)
    el.dst = _u32(el.dst)
    mask = np.zeros(el.num_vertices, np.uint32)
    call("gbx_mask_graph", el.num_vertices, el.num_edges, _ptr(el.src), _ptr(el.dst), int(mmode),
         int(cache_size), _ptr(mask), stream)
    el.mask_array = mask
    return el


def read_label_file(path: str, num_vertices: int) -> np.ndarray:
    """The reference's label file (lmode 11, relabelEdgeListFromFile,
    reorder.c:1662-1700): one unsigned label per line, read up to
    num_vertices of them; fewer is an error here (the reference leaves the
    rest uninitialised)."""
    lab = np.loadtxt(path, dtype=np.int64, ndmin=1)[:num_vertices]
    if lab.shape[0] != num_vertices:
        raise ValueError(f"{path}: {lab.shape[0]} labels for {num_vertices} vertices")
    return lab.astype(np.uint32)


def relabel_from_file(el: EdgeList, path: str, stream=None) -> EdgeList:
    """lmode 11: relabel with the labels of the reference's label file."""
    return relabel(el, read_label_file(path, el.num_vertices), stream)


def graph_csr_preprocessing(el: EdgeList, *, sort: int = 0, dedup: bool = False, lmode: int = 0,
                            directed: bool = True, keep_weights: bool = True, mmode: int = 0,
                            cache_size: int = 32768, stream=None) -> GraphCSR:
    """graphCSRPreProcessingStep (graphCSR.c:243-327) on the GPU: sort, dedup
    (-k forces sort 1, GraphBlox.c:355-356), degree reorder + re-sort, mask
    mode (mmode, after the last sort, :285-286), CSR map, and for directed
    graphs the inverse CSR built from the swapped edges with the same sort
    (on the masked ids when mmode is 1 or 2)."""
    if dedup:
        sort = 1
    V = el.num_vertices
    w = el.weight if keep_weights else None
    deg, idx, s, d, ww = csr_build(el.src, el.dst, w, num_vertices=V, dedup=dedup, sort=sort, stream=stream)
    labels = el.label_array if el.label_array is not None else np.arange(V, dtype=np.uint32)
    inv_labels = el.inverse_label_array if el.inverse_label_array is not None else np.arange(V, dtype=np.uint32)
    if lmode:
        tmp = EdgeList(V, s, d, ww, labels.copy(), inv_labels.copy())
        degree_reorder(tmp, lmode, stream)
        labels, inv_labels = tmp.label_array, tmp.inverse_label_array
        deg, idx, s, d, ww = csr_build(tmp.src, tmp.dst, ww, num_vertices=V, sort=sort, stream=stream)
    mask = None
    if mmode:
        # the map strips the mask bits, so deg / idx of the sorted list stand
        m = mask_graph(EdgeList(V, s, d), mmode, cache_size, stream)
        s, d, mask = m.src, m.dst, m.mask_array
    g = GraphCSR(V, int(s.shape[0]), deg, idx, d, s, ww, labels, inv_labels, mask_array=mask)
    # max over the weights as read (edgeList.c:673-684), kept through dedup
    if el.weight is not None and el.num_edges:
        g.max_weight = float(max(0.0, float(np.max(el.weight))))
    if directed:
        ideg, iidx, isrc, idst, iw = csr_build(d, s, ww, num_vertices=V, sort=sort, stream=stream)
        g.inverse_out_degree, g.inverse_edges_idx, g.inverse_dest, g.inverse_weight = ideg, iidx, idst, iw
        g.inverse_src = isrc
    return g


# ---------------------------------------------------------------------------
# CSR segments (the reference's csrSegments / graphCSRSegments)


@dataclass
class Segment:
    """struct Segment (csrSegments.h:19-27): the segment's edges and the
    GraphCSR the reference builds from them. num_vertices is the reference's
    value, the largest id among the segment's edge ends; the segment's
    GraphCSR has one vertex more, so that this id has a row."""
    num_edges: int
    num_vertices: int
    edge_list: Optional[EdgeList]
    graph: Optional[GraphCSR] = None


@dataclass
class CSRSegments:
    """struct CSRSegments (csrSegments.h:30-43) with host arrays."""
    num_vertices: int
    num_edges: int
    num_segments: int
    out_degree: np.ndarray
    in_degree: np.ndarray
    vertex_segment_index: np.ndarray
    segments: list


def csr_segments(el: EdgeList, cache_size: int = 32768, num_segments: Optional[int] = None,
                 build_graphs: bool = True, directed: bool = True, keep_weights: bool = True,
                 stream=None) -> CSRSegments:
    """csrSegmentsNew (csrSegments.c:157-240) on the GPU: the partition by
    destination segment (gbx_csr_segments), then, per segment with edges,
    the preprocessing csrSegmentsCreationPreprocessing applies to it
    (:330-375: the argumentsNew defaults -- radix sort by source, no dedup --
    with degree reordering, lmode 1), on the segment's edges with
    largest id + 1 vertices."""
    V = int(el.num_vertices)
    S = int(num_segments) if num_segments else int(_lib.load().gbx_csr_segments_count(V, int(cache_size)))
    src, dst = _u32(el.src), _u32(el.dst)
    E = src.shape[0]
    w = _f32(el.weight) if keep_weights else None
    od, idg, vsi = (np.zeros(V, np.uint32) for _ in range(3))
    cnt, mx = np.zeros(S, np.uint32), np.zeros(S, np.uint32)
    ss, sd = np.zeros(max(E, 1), np.uint32), np.zeros(max(E, 1), np.uint32)
    sw = np.zeros(max(E, 1), np.float32) if w is not None else None
    call("gbx_csr_segments", E, _ptr(src), _ptr(dst), _ptr(w), V, S, _ptr(od), _ptr(idg), _ptr(vsi), _ptr(cnt),
         _ptr(mx), _ptr(ss), _ptr(sd), _ptr(sw), stream)
    segs = []
    pos = 0
    for j in range(S):
        n = int(cnt[j])
        if n == 0:
            segs.append(Segment(0, 0, None))
            continue
        es = EdgeList(int(mx[j]) + 1, ss[pos:pos + n].copy(), sd[pos:pos + n].copy(),
                      None if sw is None else sw[pos:pos + n].copy())
        seg = Segment(n, int(mx[j]), es)
        if build_graphs:
            seg.graph = graph_csr_preprocessing(EdgeList(es.num_vertices, es.src.copy(), es.dst.copy(),
                                                         None if es.weight is None else es.weight.copy()),
                                                sort=0, lmode=1, directed=directed,
                                                keep_weights=es.weight is not None, stream=stream)
        segs.append(seg)
        pos += n
    return CSRSegments(V, E, S, od, idg, vsi, segs)


# ---------------------------------------------------------------------------
# the reference's binary CSR file (.csr)


def _csr_record_types(weighted: bool, directed: bool):
    """Record layouts of the .csr file: one vertex record per vertex
    (graphCSR.c:486-500), then one edge record per edge (graphCSR.c:502-524);
    the inverse fields exist in DIRECTED builds, the weights in WEIGHTED
    builds. All fields are 4 bytes, native (little-endian) order, packed."""
    u4, f4 = np.dtype("<u4"), np.dtype("<f4")
    vf = [("out_degree", u4), ("in_degree", u4), ("edges_idx", u4)]
    ef = [("src", u4), ("dest", u4)] + ([("weight", f4)] if weighted else [])
    if directed:
        vf += [("inv_out_degree", u4), ("inv_in_degree", u4), ("inv_edges_idx", u4)]
        ef += [("inv_src", u4), ("inv_dest", u4)] + ([("inv_weight", f4)] if weighted else [])
    return np.dtype(vf), np.dtype(ef)


def _csr_file_size(V: int, E: int, weighted: bool, directed: bool) -> int:
    vt, et = _csr_record_types(weighted, directed)
    return 8 + (4 if weighted else 0) + V * vt.itemsize + E * et.itemsize


def write_graph_csr_bin(fname: str, g: GraphCSR, *, weighted: Optional[bool] = None,
                        directed: Optional[bool] = None) -> str:
    """writeToBinFileGraphCSR (graphCSR.c:458-529): writes `fname + ".csr"`
    and returns that path. Header: num_edges, num_vertices (uint32) and, in
    a WEIGHTED build, max_weight (float32); then the vertex and the edge
    records of _csr_record_types. in_degree is the other direction's
    out-degree in a DIRECTED build (vertex.c:291-310) and 0 otherwise.
    weighted / directed name the reference build whose file is written
    (default: what g holds)."""
    weighted = (g.weight is not None) if weighted is None else bool(weighted)
    directed = g.directed if directed is None else bool(directed)
    if weighted and g.weight is None:
        raise ValueError("a WEIGHTED .csr needs edge weights")
    if directed and (g.inverse_dest is None or g.inverse_out_degree is None or g.inverse_edges_idx is None):
        raise ValueError("a DIRECTED .csr needs the inverse CSR")
    V, E = int(g.num_vertices), int(g.num_edges)
    vt, et = _csr_record_types(weighted, directed)
    vrec = np.zeros(V, dtype=vt)
    vrec["out_degree"] = g.out_degree[:V]
    vrec["edges_idx"] = g.edges_idx[:V]
    erec = np.zeros(E, dtype=et)
    erec["src"] = g.src[:E]
    erec["dest"] = g.dest[:E]
    if weighted:
        erec["weight"] = g.weight[:E]
    if directed:
        ideg = _u32(g.inverse_out_degree[:V])
        vrec["in_degree"] = ideg
        vrec["inv_out_degree"] = ideg
        vrec["inv_in_degree"] = g.out_degree[:V]
        vrec["inv_edges_idx"] = g.inverse_edges_idx[:V]
        isrc = g.inverse_src if g.inverse_src is not None else np.repeat(np.arange(V, dtype=np.uint32), ideg)
        erec["inv_src"] = isrc[:E]
        erec["inv_dest"] = g.inverse_dest[:E]
        if weighted:
            iw = g.inverse_weight if g.inverse_weight is not None else np.ones(E, np.float32)
            erec["inv_weight"] = iw[:E]
    path = fname + ".csr"
    with open(path, "wb") as f:
        f.write(np.array([E, V], dtype="<u4").tobytes())
        if weighted:
            f.write(np.array([g.max_weight], dtype="<f4").tobytes())
        f.write(vrec.tobytes())
        f.write(erec.tobytes())
    return path


def read_graph_csr_bin(path: str, *, weighted: Optional[bool] = None,
                       directed: Optional[bool] = None) -> GraphCSR:
    """readFromBinFileGraphCSR (graphCSR.c:638-744). The file does not name
    its build; weighted / directed default to the one layout whose size
    matches the header's counts (the four sizes differ for any V >= 1). A
    size that matches no layout, or not the one asked for, is an error (the
    reference reads on past the end). Labels start as the identity."""
    raw = np.fromfile(path, dtype=np.uint8)
    if raw.shape[0] < 8:
        raise ValueError(f"{path}: {raw.shape[0]} bytes, no .csr header")
    E, V = (int(x) for x in raw[:8].view("<u4"))
    combos = [(w, d) for w in (False, True) for d in (False, True)
              if (weighted is None or w == weighted) and (directed is None or d == directed)]
    match = [(w, d) for w, d in combos if _csr_file_size(V, E, w, d) == raw.shape[0]]
    if len(match) != 1:
        raise ValueError(f"{path}: {raw.shape[0]} bytes fit no .csr layout for V={V} E={E}"
                         f" (weighted={weighted}, directed={directed})")
    weighted, directed = match[0]
    vt, et = _csr_record_types(weighted, directed)
    off = 8
    max_weight = 0.0
    if weighted:
        max_weight = float(raw[8:12].view("<f4")[0])
        off = 12
    vrec = raw[off:off + V * vt.itemsize].view(vt)
    off += V * vt.itemsize
    erec = raw[off:off + E * et.itemsize].view(et)
    ident = np.arange(V, dtype=np.uint32)
    g = GraphCSR(V, E, vrec["out_degree"].astype(np.uint32), vrec["edges_idx"].astype(np.uint32),
                 erec["dest"].astype(np.uint32), erec["src"].astype(np.uint32),
                 erec["weight"].astype(np.float32) if weighted else None, ident.copy(), ident.copy(),
                 max_weight=max_weight)
    if directed:
        g.inverse_out_degree = vrec["inv_out_degree"].astype(np.uint32)
        g.inverse_edges_idx = vrec["inv_edges_idx"].astype(np.uint32)
        g.inverse_dest = erec["inv_dest"].astype(np.uint32)
        g.inverse_src = erec["inv_src"].astype(np.uint32)
        g.inverse_weight = erec["inv_weight"].astype(np.float32) if weighted else None
    return g


# ---------------------------------------------------------------------------
# device graph


class DeviceGraph:
    """A GraphCSR resident on the GPU (gbx_graph)."""

    def __init__(self, handle: int, num_vertices: int, num_edges: int, label_array=None):
        self._h = C.c_void_p(handle)
        self.num_vertices = num_vertices
        self.num_edges = num_edges
        self.label_array = label_array

    @classmethod
    def from_graph_csr(cls, g: GraphCSR, stream=None, use_weights: bool = True) -> "DeviceGraph":
        h = C.c_void_p()
        w = g.weight if use_weights else None
        iw = g.inverse_weight if use_weights else None
        call("gbx_graph_create_csr", C.byref(h), g.num_vertices, g.num_edges,
             _ptr(_u32(g.edges_idx)), _ptr(_u32(g.out_degree)), _ptr(_u32(g.dest)), _ptr(_f32(w)),
             _ptr(None if g.inverse_edges_idx is None else _u32(g.inverse_edges_idx)),
             _ptr(None if g.inverse_out_degree is None else _u32(g.inverse_out_degree)),
             _ptr(None if g.inverse_dest is None else _u32(g.inverse_dest)), _ptr(_f32(iw)), stream)
        return cls(h.value, g.num_vertices, g.num_edges, g.label_array)

    @classmethod
    def from_offsets(cls, num_vertices, offsets, dest, weight=None, in_offsets=None, in_src=None,
                     in_weight=None, stream=None) -> "DeviceGraph":
        h = C.c_void_p()
        call("gbx_graph_create_offsets", C.byref(h), int(num_vertices), int(len(dest)), _ptr(offsets),
             _ptr(dest), _ptr(weight), _ptr(in_offsets), _ptr(in_src), _ptr(in_weight), stream)
        return cls(h.value, int(num_vertices), int(len(dest)))

    @property
    def handle(self):
        return self._h

    def set_tuning(self, key: str, value: float) -> None:
        call("gbx_graph_set_tuning", self._h, key.encode(), float(value))

    def get_tuning(self, key: str) -> float:
        v = C.c_double()
        call("gbx_graph_get_tuning", self._h, key.encode(), C.byref(v))
        return v.value

    def autotune(self, bfs: bool = True, sssp: bool = True, samples: int = 4, stream=None,
                 pull: bool = False) -> dict:
        """gbx_autotune: time candidate knob settings on this graph, keep the fastest."""
        call("gbx_autotune", self._h, (1 if bfs else 0) | (2 if sssp else 0) | (4 if pull else 0), int(samples),
             stream)
        return {k: self.get_tuning(k) for k in ("bfs_alpha", "bfs_beta", "sssp_delta", "pull_heavy_min")}

    def close(self) -> None:
        if self._h and self._h.value:
            _lib.load().gbx_graph_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def _map_source(dg: DeviceGraph, source: int) -> int:
    # BFS.c:153 / SSSP.c:493: the source is given in original ids
    if dg.label_array is not None:
        return int(dg.label_array[source])
    return int(source)


@dataclass
class BFSStats:
    distances: object
    parents: object
    processed_nodes: int
    iteration: int
    depth: int
    edges_traversed: int
    source: int


def breadth_first_search(dg: DeviceGraph, source: int, pushpull: int = 2, distances=None,
                         parents=None, stream=None, map_source: bool = True) -> BFSStats:
    """breadthFirstSearchGraphCSR: pushpull 0 pull, 1 push, 2 direction-optimising."""
    V = dg.num_vertices
    src = _map_source(dg, source) if map_source else int(source)
    if distances is None:
        distances = np.zeros(V, np.uint32)
    if parents is None:
        parents = np.zeros(V, np.int32)
    mode = {0: 0, 1: 1}.get(int(pushpull), 2)
    r = BfsResult()
    call("gbx_bfs", dg.handle, src, mode, _ptr(distances), _ptr(parents), C.byref(r), stream)
    return BFSStats(distances, parents, r.processed_nodes, r.iteration, r.depth, r.edges_traversed, src)


def breadth_first_search_trials(dg: DeviceGraph, sources, pushpull: int = 2, distances=None, parents=None,
                                out_stride: int = 0, stream=None, map_source: bool = True) -> list:
    """The reference's BFS trial loop (graphRun.c:463-595) through
    gbx_bfs_trials: one traversal per source, back to back on the stream,
    one host synchronisation. distances / parents are device tensors, host
    arrays (copied back while the next trial runs) or None; with out_stride
    0 the last trial's output remains in them, with out_stride >= V trial i
    writes [i*out_stride, i*out_stride + V).
    Returns one BFSStats per trial (its distances / parents fields hold the
    arrays passed in)."""
    srcs = np.asarray([_map_source(dg, s) if map_source else int(s) for s in sources], np.uint32)
    n = len(srcs)
    res = (BfsResult * max(n, 1))()
    mode = {0: 0, 1: 1}.get(int(pushpull), 2)
    call("gbx_bfs_trials", dg.handle, srcs.ctypes.data, n, mode, _ptr(distances), _ptr(parents), int(out_stride),
         res, stream)
    return [BFSStats(distances, parents, res[i].processed_nodes, res[i].iteration, res[i].depth,
                     res[i].edges_traversed, int(srcs[i])) for i in range(n)]


@dataclass
class PageRankStats:
    pageRanks: object
    iterations: int
    error_total: float
    active_last: int


def page_rank(dg: DeviceGraph, iterations: int = 20, epsilon: float = 1e-4, ranks=None,
              stream=None) -> PageRankStats:
    """pageRankPullGraphCSR (pushpull 0)."""
    if ranks is None:
        ranks = np.zeros(dg.num_vertices, np.float32)
    r = PrResult()
    call("gbx_pagerank_pull", dg.handle, int(iterations), float(epsilon), _ptr(ranks), C.byref(r), stream)
    return PageRankStats(ranks, r.iterations, r.error_total, r.active_last)


@dataclass
class PPRStats:
    ranks: object
    iterations: int
    residual: float


@dataclass
class PPRAdjointStats:
    grad_weights: object
    grad_teleport: object
    loss: float
    iterations: int
    residual: float


def _block_k(a, num_vertices: int) -> int:
    shape = tuple(a.shape)
    if len(shape) != 2 or shape[0] != num_vertices:
        raise ValueError(f"expected a [{num_vertices}, K] block, got shape {shape}")
    return int(shape[1])


def _like(a, shape):
    if isinstance(a, np.ndarray):
        return np.zeros(shape, np.float32)
    import torch

    return torch.zeros(shape, dtype=torch.float32, device=a.device)


def ppr_forward(dg: DeviceGraph, weights, teleport, damping: float = 0.85, tol: float = 1e-7,
                max_iterations: int = 1000, ranks=None, stream=None) -> PPRStats:
    """Personalised PageRank R = (1-d) T + d P R for the K columns of
    `teleport` ([V, K], K in 32/64/128/256); P from the forward-order edge
    `weights` normalised per source. No reference counterpart."""
    if isinstance(weights, np.ndarray):
        weights = _f32(weights)
    if isinstance(teleport, np.ndarray):
        teleport = _f32(teleport)
    K = _block_k(teleport, dg.num_vertices)
    if ranks is None:
        ranks = _like(teleport, (dg.num_vertices, K))
    r = _lib.PprResult()
    call("gbx_ppr_forward", dg.handle, K, _ptr(weights), _ptr(teleport), float(damping), float(tol),
         int(max_iterations), _ptr(ranks), C.byref(r), stream)
    return PPRStats(ranks, r.iterations, r.residual)


def ppr_adjoint(dg: DeviceGraph, weights, ranks, loss_weights, damping: float = 0.85, tol: float = 1e-7,
                max_iterations: int = 1000, grad_weights=None, grad_teleport=None, want_weights: bool = True,
                want_teleport: bool = True, stream=None) -> PPRAdjointStats:
    """Adjoint of ppr_forward for L = sum(loss_weights * ranks): solves
    Lam = W + d P^T Lam at the converged ranks and returns dL/dw (forward
    edge order) and dL/dT = (1-d) Lam."""
    if isinstance(weights, np.ndarray):
        weights = _f32(weights)
    if isinstance(ranks, np.ndarray):
        ranks = _f32(ranks)
    if isinstance(loss_weights, np.ndarray):
        loss_weights = _f32(loss_weights)
    K = _block_k(ranks, dg.num_vertices)
    if _block_k(loss_weights, dg.num_vertices) != K:
        raise ValueError("ranks and loss_weights differ in K")
    if grad_weights is None and want_weights:
        grad_weights = _like(ranks, (dg.num_edges,))
    if grad_teleport is None and want_teleport:
        grad_teleport = _like(ranks, (dg.num_vertices, K))
    r = _lib.PprResult()
    call("gbx_ppr_adjoint", dg.handle, K, _ptr(weights), _ptr(ranks), _ptr(loss_weights), float(damping),
         float(tol), int(max_iterations), _ptr(grad_weights), _ptr(grad_teleport), C.byref(r), stream)
    return PPRAdjointStats(grad_weights, grad_teleport, r.loss, r.adjoint_iterations, r.adjoint_residual)


@dataclass
class SSSPStats:
    distances: object
    reached: int
    rounds: int
    edges_relaxed: int
    edges_traversed: int
    source: int


def sssp(dg: DeviceGraph, source: int, delta: int = 0, distances=None, stream=None,
         map_source: bool = True) -> SSSPStats:
    """SSSPGraphCSR (delta-stepping). Unreached vertices report UINT32_MAX/2."""
    src = _map_source(dg, source) if map_source else int(source)
    if distances is None:
        distances = np.zeros(dg.num_vertices, np.uint32)
    r = SsspResult()
    call("gbx_sssp", dg.handle, src, int(delta), _ptr(distances), C.byref(r), stream)
    return SSSPStats(distances, r.reached, r.rounds, r.edges_relaxed, r.edges_traversed, src)


@dataclass
class BellmanFordStats:
    distances: object
    parents: object
    processed_nodes: int
    source: int


def bellman_ford(dg: DeviceGraph, source: int, distances=None, parents=None, stream=None,
                 map_source: bool = True) -> BellmanFordStats:
    """bellmanFordGraphCSR: the reference's distances (UINT32_MAX/2 when
    unreached) and a shortest-path parent per vertex (the smallest valid
    one; UINT32_MAX when unreached). processed_nodes = vertices reached."""
    src = _map_source(dg, source) if map_source else int(source)
    V = dg.num_vertices
    if distances is None:
        distances = np.zeros(V, np.uint32)
    if parents is None:
        parents = np.zeros(V, np.uint32)
    r = SsspResult()
    call("gbx_bellman_ford", dg.handle, src, _ptr(distances), _ptr(parents), C.byref(r), stream)
    return BellmanFordStats(distances, parents, r.reached, src)


@dataclass
class DFSStats:
    distances: object
    parents: object
    processed_nodes: int


def depth_first_search(dg: DeviceGraph, source: int, distances=None, parents=None,
                       stream=None) -> DFSStats:
    """depthFirstSearchGraphCSR: the reference's stack traversal (its source
    is used as given, without the label remapping of BFS/SSSP)."""
    V = dg.num_vertices
    if distances is None:
        distances = np.zeros(V, np.uint32)
    if parents is None:
        parents = np.zeros(V, np.int32)
    n = _lib.u32(0)
    call("gbx_dfs", dg.handle, int(source), _ptr(distances), _ptr(parents), C.byref(n), stream)
    return DFSStats(distances, parents, n.value)


BC_SEED = 27491095  # the reference's generator seed, graphConfig.c:84


@dataclass
class BetweennessCentralityStats:
    betweennessCentrality: object
    distances: object
    sigma: object
    dependency: object
    iteration: int
    processed_nodes: int
    roots: np.ndarray


def reference_roots(dg: DeviceGraph, n: int, seed: int = BC_SEED) -> np.ndarray:
    """The n roots the reference's Brandes draws from a freshly seeded
    generator (gbx_reference_roots)."""
    roots = np.zeros(max(int(n), 1), np.uint32)
    call("gbx_reference_roots", dg.handle, int(seed), int(n), _ptr(roots))
    return roots[:n]


def betweenness_centrality(dg: DeviceGraph, iterations: int = 20, roots=None, centrality=None,
                           seed: int = BC_SEED, distances=None, sigma=None, dependency=None,
                           stream=None) -> BetweennessCentralityStats:
    """betweennessCentralityBrandesGraphCSR: Brandes from `iterations` roots
    drawn like the reference's (or the given roots), centrality accumulated
    from zero (or into the given array). distances / sigma / dependency are
    the last root's (host arrays unless given)."""
    if roots is None:
        roots = reference_roots(dg, iterations, seed)
    roots = _u32(roots)
    V = dg.num_vertices
    if centrality is None:
        centrality = np.zeros(V, np.float32)
    dist = np.zeros(V, np.uint32) if distances is None else distances
    sig = np.zeros(V, np.int32) if sigma is None else sigma
    dep = np.zeros(V, np.float32) if dependency is None else dependency
    r = BcResult()
    call("gbx_betweenness", dg.handle, roots.shape[0], _ptr(roots), _ptr(centrality), _ptr(dist), _ptr(sig),
         _ptr(dep), C.byref(r), stream)
    return BetweennessCentralityStats(centrality, dist, sig, dep, r.iteration, r.processed_nodes, roots)


def connected_components(dg: DeviceGraph, variant: int = 1, components=None, stream=None):
    """connectedComponentsGraphCSR: 0 Shiloach-Vishkin, 1 Afforest, 2 label propagation."""
    if components is None:
        components = np.zeros(dg.num_vertices, np.uint32)
    it = _lib.u32(0)
    call("gbx_cc", dg.handle, int(variant), _ptr(components), C.byref(it), stream)
    return components, it.value


def triangle_count(dg: DeviceGraph, stream=None) -> int:
    """triangleCountGraphCSR (pull semantics)."""
    t = _lib.u64(0)
    call("gbx_tc", dg.handle, C.byref(t), stream)
    return int(t.value)


def spmv(dg: DeviceGraph, x, values=None, default_value: float = 0.0001, iterations: int = 1, y=None,
         stream=None):
    """SPMVGraphCSR pull: y += A x, `iterations` times (y defaults to zeros)."""
    if isinstance(x, np.ndarray):
        x = _f32(x)
    if isinstance(values, np.ndarray):
        values = _f32(values)
    if y is None:
        y = np.zeros(dg.num_vertices, np.float32)
    call("gbx_spmv", dg.handle, _ptr(values), float(default_value), _ptr(x), _ptr(y), int(iterations), stream)
    return y


# ---------------------------------------------------------------------------
# synthetic inputs


def generate_rmat(scale: int, num_edges: int, a: float = 0.57, b: float = 0.19, c: float = 0.19,
                  seed: int = 1):
    src = np.empty(num_edges, np.uint32)
    dst = np.empty(num_edges, np.uint32)
    call("gbx_generate_rmat", int(scale), int(num_edges), a, b, c, int(seed), _ptr(src), _ptr(dst))
    return src, dst


def generate_values(count: int, kind: int, lo: int = 0, hi: int = 0, seed: int = 1) -> np.ndarray:
    """kind 0 int U[lo,hi] as float, 1 U(0,1], 2 U[-1,1), 3 lognormal(0,1)."""
    out = np.empty(count, np.float32)
    call("gbx_generate_values", int(count), int(kind), int(lo), int(hi), int(seed), _ptr(out))
    return out


# ---------------------------------------------------------------------------
# batches of graphs (gbx_batch): one persistent launch per algorithm


def _results_dict(arr, fields):
    return {f: np.array([getattr(r, f) for r in arr]) for f in fields}


@dataclass
class PackedGraphs:
    """Back-to-back CSR of several graphs (the gbx_batch_create layout):
    graph g owns packed vertices vertex_base[g]..vertex_base[g+1]-1, offsets
    are global edge positions, dest / in_src hold graph-local ids."""
    vertex_base: np.ndarray
    offsets: np.ndarray
    dest: np.ndarray
    in_offsets: Optional[np.ndarray] = None
    in_src: Optional[np.ndarray] = None

    @property
    def num_graphs(self) -> int:
        return len(self.vertex_base) - 1

    def graph(self, g: int):
        """(V, offsets rebased to 0, dest, in_offsets, in_src) of graph g."""
        b, e = int(self.vertex_base[g]), int(self.vertex_base[g + 1])
        off = self.offsets[b:e + 1].astype(np.int64)
        out = [e - b, (off - off[0]).astype(np.uint32), self.dest[off[0]:off[-1]]]
        if self.in_offsets is not None:
            ioff = self.in_offsets[b:e + 1].astype(np.int64)
            out += [(ioff - ioff[0]).astype(np.uint32), self.in_src[ioff[0]:ioff[-1]]]
        else:
            out += [None, None]
        return tuple(out)


def pack_graphs(graphs, inverse: bool = True, stream=None) -> PackedGraphs:
    """Pack [(V, src, dst), ...] edge lists into one back-to-back CSR, rows
    grouped by source in input order (gbx_csr_build, sort by source, on the
    GPU), with the in-edge CSR when `inverse`."""
    nv = np.array([int(v) for v, _, _ in graphs], np.int64)
    vbase = np.zeros(len(graphs) + 1, np.int64)
    vbase[1:] = np.cumsum(nv)
    if vbase[-1] >= 1 << 30:
        raise ValueError("packed vertex count must stay below 2^30")
    counts = np.array([len(s) for _, s, _ in graphs], np.int64)
    shift = np.repeat(vbase[:-1], counts).astype(np.uint32)
    src = np.concatenate([np.asarray(s, np.uint32) for _, s, _ in graphs]) + shift
    dst = np.concatenate([np.asarray(d, np.uint32) for _, _, d in graphs]) + shift
    Vt = int(vbase[-1])

    def csr(a, b):
        deg, _, so, do, _ = csr_build(a, b, num_vertices=Vt, sort=0, stream=stream)
        off = np.zeros(Vt + 1, np.int64)
        off[1:] = np.cumsum(deg[:Vt], dtype=np.int64)
        base = np.repeat(vbase[:-1], np.diff(off[vbase])).astype(np.uint32)
        return off.astype(np.uint32), (do - base).astype(np.uint32)

    off, dest = csr(src, dst)
    ioff = isrc = None
    if inverse:
        ioff, isrc = csr(dst, src)
    return PackedGraphs(vbase.astype(np.uint32), off, dest, ioff, isrc)


class GraphBatch:
    """Many graphs resident on the GPU as one packed CSR (gbx_batch)."""

    def __init__(self, packed: PackedGraphs, stream=None):
        h = C.c_void_p()
        p = packed
        call("gbx_batch_create", C.byref(h), p.num_graphs, _ptr(_u32(p.vertex_base)), _ptr(_u32(p.offsets)),
             _ptr(_u32(p.dest)), _ptr(None if p.in_offsets is None else _u32(p.in_offsets)),
             _ptr(None if p.in_src is None else _u32(p.in_src)), stream)
        self._h = h
        self.num_graphs = p.num_graphs
        self.num_vertices = int(p.vertex_base[-1])
        self.num_edges = int(p.offsets[-1])

    @property
    def handle(self):
        return self._h

    def bfs(self, sources, distances=None, parents=None, stream=None):
        """gbx_bfs_batched: (distances, parents, per-graph results dict)."""
        if isinstance(sources, np.ndarray) or isinstance(sources, (list, tuple)):
            sources = _u32(sources)
        if distances is None:
            distances = np.zeros(self.num_vertices, np.uint32)
        res = (BfsResult * self.num_graphs)()
        call("gbx_bfs_batched", self._h, _ptr(sources), _ptr(distances), _ptr(parents), res, stream)
        return distances, parents, _results_dict(res, ("processed_nodes", "iteration", "depth", "top_down_steps",
                                                       "bottom_up_steps", "edges_traversed"))

    def page_rank(self, iterations: int = 20, epsilon: float = 1e-4, ranks=None, stream=None):
        """gbx_pr_batched: (ranks, per-graph results dict)."""
        if ranks is None:
            ranks = np.zeros(self.num_vertices, np.float32)
        res = (PrResult * self.num_graphs)()
        call("gbx_pr_batched", self._h, int(iterations), float(epsilon), _ptr(ranks), res, stream)
        return ranks, _results_dict(res, ("iterations", "active_last", "error_total"))

    def close(self) -> None:
        if self._h and self._h.value:
            _lib.load().gbx_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def generate_chung_lu(num_vertices: int, num_edges: int, exponent: float = 2.1, window: int = 4096,
                      local_fraction: float = 0.7, seed: int = 1, src=None, dst=None, stream=None):
    """gbx_generate_chung_lu (on the GPU): power-law out-degrees with the given
    exponent, local_fraction of the edges inside window-aligned id blocks.
    src/dst may be preallocated torch CUDA tensors (else host numpy arrays)."""
    if src is None:
        src = np.empty(num_edges, np.uint32)
    if dst is None:
        dst = np.empty(num_edges, np.uint32)
    call("gbx_generate_chung_lu", int(num_vertices), int(num_edges), float(exponent), int(window),
         float(local_fraction), int(seed), _ptr(src), _ptr(dst), stream)
    return src, dst


def bfs_multisource(dg: DeviceGraph, sources, distances=None, stream=None, map_source: bool = True):
    """gbx_bfs_multisource: up to 256 BFS runs in one bitmask sweep. Returns
    (distances [V, S] vertex-major, per-source results dict); sources are
    mapped through the graph's label array like breadth_first_search."""
    srcs = [(_map_source(dg, int(s)) if map_source else int(s)) for s in np.asarray(sources).ravel()]
    S = len(srcs)
    src = np.asarray(srcs, np.uint32)
    if distances is None:
        distances = np.zeros((dg.num_vertices, S), np.uint32)
    res = (BfsResult * S)()
    call("gbx_bfs_multisource", dg.handle, S, _ptr(src), _ptr(distances), res, stream)
    return distances, _results_dict(res, ("processed_nodes", "iteration", "depth", "top_down_steps",
                                          "bottom_up_steps", "edges_traversed"))


def generate_rmat_batch(num_graphs: int = 2048, seed: int = 1, scale_lo: float = 8.0, scale_hi: float = 15.0,
                        ef_lo: float = 4.0, ef_hi: float = 32.0):
    """Edge lists of `num_graphs` RMAT graphs (a/b/c = .57/.19/.19): scale
    s ~ U[scale_lo, scale_hi], V = floor(2^s), edge factor ~ U[ef_lo, ef_hi];
    each graph draws round(ef*V) edges at scale ceil(s) and keeps those with
    both ends below V. Returns [(V, src, dst), ...]."""
    rng = np.random.default_rng(seed)
    s = rng.uniform(scale_lo, scale_hi, num_graphs)
    ef = rng.uniform(ef_lo, ef_hi, num_graphs)
    out = []
    for g in range(num_graphs):
        V = int(np.floor(2.0 ** s[g]))
        sc = max(1, int(np.ceil(np.log2(V))))
        src, dst = generate_rmat(sc, int(round(ef[g] * V)), seed=seed * 1_000_003 + g)
        keep = (src < V) & (dst < V)
        out.append((V, src[keep], dst[keep]))
    return out
