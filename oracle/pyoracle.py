"""ctypes binding of liboracle.so -- the CPU restatement in gbx_oracle.c.

TEST INFRASTRUCTURE, NOT PRODUCT CODE. Imported only by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg, as the checker or
the timed CPU baseline. It also offers `ref_run`, which executes the
reference host built by build_ref.sh (present only where the reference
sources are, i.e. not on the GPU host).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile
from pathlib import Path
from typing import Optional

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"

u32 = C.c_uint32
u64 = C.c_uint64
vp = C.c_void_p
_lib = None


def load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
        lib = C.CDLL(str(LIB))
        sig = {
            "orc_sort_edges": (None, [u32, vp, vp, vp, C.c_int, C.c_int]),
            "orc_dedup_edges": (u32, [u32, vp, vp, vp]),
            "orc_map_vertices": (None, [u32, u32, vp, vp, vp]),
            "orc_degree_reorder": (None, [u32, u32, vp, vp, C.c_int, vp, vp, C.c_int]),
            "orc_mask_graph": (None, [u32, u32, vp, vp, C.c_int, u32, vp]),
            "orc_random_roots": (None, [u32, u32, u32, vp, u32, vp]),
            "orc_betweenness": (None, [u32, vp, vp, vp, u32, vp, vp, vp, vp, vp, vp]),
            "orc_dfs": (None, [u32, vp, vp, vp, u32, vp, vp, vp]),
            "orc_bfs": (None, [u32, u32, vp, vp, vp, vp, vp, vp, u32, vp, vp, vp, vp, C.c_int]),
            "orc_pagerank_pull": (None, [u32, vp, vp, vp, vp, u32, C.c_double, vp, vp, vp, C.c_int]),
            "orc_pagerank_pull_f64": (None, [u32, vp, vp, vp, vp, u32, C.c_double, vp, vp, C.c_int]),
            "orc_sssp": (None, [u32, vp, vp, vp, vp, u32, u32, vp, vp, C.c_int]),
            "orc_cc": (None, [u32, vp, vp, vp, vp, vp, vp, C.c_int, vp, vp, C.c_int]),
            "orc_triangle_count": (u64, [u32, vp, vp, vp, C.c_int]),
            "orc_triangle_count_range": (u64, [u32, vp, vp, vp, u32, u32, C.c_int]),
            "orc_generate_rmat": (C.c_int, [u32, u64, C.c_double, C.c_double, C.c_double, u64, vp, vp]),
            "orc_generate_values": (C.c_int, [u64, C.c_int, u32, u32, u64, vp]),
            "orc_csr_segments_count": (u32, [u32, u32]),
            "orc_csr_segments": (None, [u32, vp, vp, vp, u32, u32, vp, vp, vp, vp, vp, vp, vp, vp]),
            "orc_spmv_pull": (None, [u32, vp, vp, vp, vp, C.c_float, vp, vp, u32, C.c_int]),
            "orc_spmv_pull_f64": (None, [u32, vp, vp, vp, vp, C.c_float, vp, vp, u32, C.c_int]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


class HostCSR:
    """Reference-layout CSR in numpy (out_degree, edges_idx, dest[, weight])."""

    def __init__(self, num_vertices, out_degree, edges_idx, dest, weight=None, src=None):
        self.num_vertices = int(num_vertices)
        self.out_degree = _u32(out_degree)
        self.edges_idx = _u32(edges_idx)
        self.dest = _u32(dest)
        self.weight = None if weight is None else np.ascontiguousarray(weight, np.float32)
        self.src = None if src is None else _u32(src)

    @property
    def num_edges(self):
        return int(self.dest.shape[0])


def build_csr(num_vertices, src, dst, weight=None, sort_mode=1, dedup=False, threads=0):
    """Sort (+dedup) and map, like the reference's preprocessing. Returns
    (HostCSR, src_sorted)."""
    s = _u32(src).copy()
    d = _u32(dst).copy()
    w = None if weight is None else np.ascontiguousarray(weight, np.float32).copy()
    lib = load()
    lib.orc_sort_edges(s.shape[0], _p(s), _p(d), _p(w), sort_mode, threads)
    n = s.shape[0]
    if dedup:
        n = lib.orc_dedup_edges(n, _p(s), _p(d), _p(w))
        s, d = s[:n].copy(), d[:n].copy()
        if w is not None:
            w = w[:n].copy()
    deg = np.zeros(num_vertices, np.uint32)
    idx = np.zeros(num_vertices, np.uint32)
    lib.orc_map_vertices(num_vertices, n, _p(s), _p(deg), _p(idx))
    return HostCSR(num_vertices, deg, idx, d, w, s)


def degree_reorder(num_vertices, src, dst, lmode=1, labels=None, inverse_labels=None, threads=0):
    s = _u32(src).copy()
    d = _u32(dst).copy()
    lab = np.arange(num_vertices, dtype=np.uint32) if labels is None else _u32(labels).copy()
    inv = np.arange(num_vertices, dtype=np.uint32) if inverse_labels is None else _u32(inverse_labels).copy()
    load().orc_degree_reorder(num_vertices, s.shape[0], _p(s), _p(d), lmode, _p(lab), _p(inv), threads)
    return s, d, lab, inv


def mask_graph(num_vertices, src, dst, mmode=1, cache_size=32768):
    """Mask mode: returns (src, dst, mask); src/dst carry the hints for mmode 1, 2."""
    s = _u32(src).copy()
    d = _u32(dst).copy()
    m = np.zeros(num_vertices, np.uint32)
    load().orc_mask_graph(num_vertices, s.shape[0], _p(s), _p(d), int(mmode), int(cache_size), _p(m))
    return s, d, m


BC_SEED = 27491095  # graphConfig.c:84


def random_roots(g: HostCSR, n, seed=BC_SEED):
    """The roots the reference's Brandes draws (n of them, from a fresh generator)."""
    roots = np.zeros(max(int(n), 1), np.uint32)
    avg = g.num_edges // g.num_vertices if g.num_vertices else 0
    load().orc_random_roots(int(seed), int(n), g.num_vertices, _p(g.out_degree), avg, _p(roots))
    return roots[:n]


def betweenness(g: HostCSR, roots, pull: Optional[HostCSR] = None):
    """Returns (bc, distances, sigma, dependency, processed_nodes) -- the last
    four for the last root."""
    pull = pull or g
    V = g.num_vertices
    r = _u32(roots)
    bc = np.zeros(V, np.float32)
    dist = np.zeros(V, np.uint32)
    sig = np.zeros(V, np.int32)
    dep = np.zeros(V, np.float32)
    proc = u32(0)
    load().orc_betweenness(V, _p(pull.out_degree), _p(pull.edges_idx), _p(pull.dest), r.shape[0], _p(r),
                           _p(bc), _p(dist), _p(sig), _p(dep), C.byref(proc))
    return bc, dist, sig, dep, proc.value


def dfs(g: HostCSR, source):
    """Returns (distances, parents, processed_nodes)."""
    V = g.num_vertices
    dist = np.zeros(V, np.uint32)
    par = np.zeros(V, np.int32)
    proc = u32(0)
    load().orc_dfs(V, _p(g.out_degree), _p(g.edges_idx), _p(g.dest), int(source), _p(dist), _p(par),
                   C.byref(proc))
    return dist, par, proc.value


def bfs(g: HostCSR, source, pull: Optional[HostCSR] = None, threads=0):
    pull = pull or g
    V = g.num_vertices
    dist = np.zeros(V, np.uint32)
    par = np.zeros(V, np.int32)
    proc = u32(0)
    it = u32(0)
    load().orc_bfs(V, g.num_edges, _p(g.out_degree), _p(g.edges_idx), _p(g.dest), _p(pull.out_degree),
                   _p(pull.edges_idx), _p(pull.dest), int(source), _p(dist), _p(par), C.byref(proc),
                   C.byref(it), threads)
    return dist, par, proc.value, it.value


def pagerank(g: HostCSR, iterations=20, epsilon=0.0, pull: Optional[HostCSR] = None, threads=0, fp64=False):
    pull = pull or g
    V = g.num_vertices
    it = u32(0)
    if fp64:
        r = np.zeros(V, np.float64)
        load().orc_pagerank_pull_f64(V, _p(g.out_degree), _p(pull.out_degree), _p(pull.edges_idx),
                                     _p(pull.dest), int(iterations), float(epsilon), _p(r), C.byref(it), threads)
        return r, it.value, None
    r = np.zeros(V, np.float32)
    err = C.c_double(0)
    load().orc_pagerank_pull(V, _p(g.out_degree), _p(pull.out_degree), _p(pull.edges_idx), _p(pull.dest),
                             int(iterations), float(epsilon), _p(r), C.byref(it), C.byref(err), threads)
    return r, it.value, err.value


def sssp(g: HostCSR, source, delta=1, threads=0, use_weights=True):
    V = g.num_vertices
    dist = np.zeros(V, np.uint32)
    proc = u32(0)
    w = g.weight if use_weights else None
    load().orc_sssp(V, _p(g.out_degree), _p(g.edges_idx), _p(g.dest), _p(w), int(source), int(delta),
                    _p(dist), C.byref(proc), threads)
    return dist


def cc(g: HostCSR, variant=1, pull: Optional[HostCSR] = None, threads=0):
    V = g.num_vertices
    comp = np.zeros(V, np.uint32)
    it = u32(0)
    load().orc_cc(V, _p(g.out_degree), _p(g.edges_idx), _p(g.dest),
                  _p(pull.out_degree) if pull else None, _p(pull.edges_idx) if pull else None,
                  _p(pull.dest) if pull else None, variant, _p(comp), C.byref(it), threads)
    return comp


def triangle_count(g: HostCSR, threads=0, lo=0, hi=None):
    """Triangles whose largest vertex is in [lo, hi) (all of them by default)."""
    hi = g.num_vertices if hi is None else hi
    return int(load().orc_triangle_count_range(g.num_vertices, _p(g.out_degree), _p(g.edges_idx), _p(g.dest),
                                               int(lo), int(hi), threads))


def csr_segments(num_vertices, src, dst, weight=None, cache_size=32768, num_segments=None):
    """The partition of the reference's csrSegmentsNew: a dict with
    num_segments, out_degree, in_degree, vertex_segment_index,
    segment_num_edges, segment_max_id, seg_src, seg_dst[, seg_weight]."""
    lib = load()
    V = int(num_vertices)
    S = int(num_segments) if num_segments else int(lib.orc_csr_segments_count(V, int(cache_size)))
    s, d = _u32(src), _u32(dst)
    E = s.shape[0]
    w = None if weight is None else np.ascontiguousarray(weight, np.float32)
    out = {k: np.zeros(V, np.uint32) for k in ("out_degree", "in_degree", "vertex_segment_index")}
    out.update(segment_num_edges=np.zeros(S, np.uint32), segment_max_id=np.zeros(S, np.uint32),
               seg_src=np.zeros(E, np.uint32), seg_dst=np.zeros(E, np.uint32))
    sw = None if w is None else np.zeros(E, np.float32)
    lib.orc_csr_segments(E, _p(s), _p(d), _p(w), V, S, _p(out["out_degree"]), _p(out["in_degree"]),
                         _p(out["vertex_segment_index"]), _p(out["segment_num_edges"]), _p(out["segment_max_id"]),
                         _p(out["seg_src"]), _p(out["seg_dst"]), _p(sw))
    if sw is not None:
        out["seg_weight"] = sw
    out["num_segments"] = S
    return out


def generate_rmat(scale, num_edges, a=0.57, b=0.19, c=0.19, seed=1):
    """RMAT edges from the same stream as the library's generator."""
    src = np.zeros(int(num_edges), np.uint32)
    dst = np.zeros(int(num_edges), np.uint32)
    if load().orc_generate_rmat(int(scale), int(num_edges), a, b, c, int(seed), _p(src), _p(dst)) != 0:
        raise ValueError("bad RMAT parameters")
    return src, dst


def generate_values(count, kind, lo=0, hi=0, seed=1):
    """Values from the same stream as the library's generator."""
    out = np.zeros(int(count), np.float32)
    if load().orc_generate_values(int(count), int(kind), int(lo), int(hi), int(seed), _p(out)) != 0:
        raise ValueError("bad value-generator parameters")
    return out


def spmv(g: HostCSR, x, values=None, default_value=0.0001, iterations=1, y=None, pull: Optional[HostCSR] = None,
         threads=0, fp64=False):
    pull = pull or g
    V = g.num_vertices
    x = np.ascontiguousarray(x, np.float32)
    vals = None if values is None else np.ascontiguousarray(values, np.float32)
    if fp64:
        yy = np.zeros(V, np.float64) if y is None else np.ascontiguousarray(y, np.float64).copy()
        load().orc_spmv_pull_f64(V, _p(pull.out_degree), _p(pull.edges_idx), _p(pull.dest), _p(vals),
                                 float(default_value), _p(x), _p(yy), int(iterations), threads)
        return yy
    yy = np.zeros(V, np.float32) if y is None else np.ascontiguousarray(y, np.float32).copy()
    load().orc_spmv_pull(V, _p(pull.out_degree), _p(pull.edges_idx), _p(pull.dest), _p(vals),
                         float(default_value), _p(x), _p(yy), int(iterations), threads)
    return yy


def rel_l1(a, ref) -> float:
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    den = np.abs(ref).sum()
    return float(np.abs(a - ref).sum() / den) if den else float(np.abs(a - ref).sum())


FLT_MIN = float(np.finfo(np.float32).tiny)
FLT_SUBNORMAL_ULP = float(np.finfo(np.float32).smallest_subnormal)


def fp32_close(a, ref64, tol=1e-6, subnormal_ulps=64):
    """Relative-L1 check of an FP32 result against an FP64 reference.

    The relative bar applies to entries whose reference magnitude is in the
    normal FP32 range; subnormal entries carry only a few significant bits in
    FP32, so there each |a - ref| must stay within `subnormal_ulps` subnormal
    steps. Returns (ok, rel_l1_normal, worst_subnormal_ulps)."""
    a = np.asarray(a, np.float64)
    ref64 = np.asarray(ref64, np.float64)
    normal = np.abs(ref64) >= FLT_MIN
    err = rel_l1(a[normal], ref64[normal]) if normal.any() else 0.0
    sub = ~normal
    worst = float((np.abs(a[sub] - ref64[sub]) / FLT_SUBNORMAL_ULP).max()) if sub.any() else 0.0
    return (err <= tol and worst <= subnormal_ulps), err, worst


# ---- the reference host itself (only where its sources were compiled) -----

def ref_available(variant="dw") -> bool:
    return (REF_DIR / f"gbx_ref_{variant}").exists()


def ref_run(graph_file, variant="dw", algorithm=-1, flags=(), threads=4):
    """Run oracle/_ref/gbx_ref_<variant> and load its dumps as numpy arrays."""
    exe = REF_DIR / f"gbx_ref_{variant}"
    with tempfile.TemporaryDirectory() as td:
        cmd = [str(exe), str(graph_file), td, "-a", str(algorithm), "-n", str(threads), *map(str, flags)]
        res = subprocess.run(cmd, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True,
                             env={**os.environ, "OMP_NUM_THREADS": str(threads)})
        if res.returncode != 0:
            raise RuntimeError(f"reference run failed: {' '.join(cmd)}\n{res.stderr}")
        out = {}
        for f in Path(td).iterdir():
            if f.name == "scalars.txt":
                for line in f.read_text().splitlines():
                    k, v = line.split()
                    out[k] = float(v) if ("." in v or "e" in v) else int(v)
            else:
                stem, ext = f.name.rsplit(".", 1)
                dt = {"u32": np.uint32, "i32": np.int32, "f32": np.float32, "csr": np.uint8}[ext]
                out[stem] = np.fromfile(f, dtype=dt)
        return out
