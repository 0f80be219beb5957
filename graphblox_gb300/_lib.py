"""ctypes binding of libgbx.so (the C ABI declared in include/gbx.h).

The library is the only compute path: if it is missing or fails to load,
every call raises. There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libgbx.so"

u32 = C.c_uint32
u64 = C.c_uint64
i32 = C.c_int32
vp = C.c_void_p


class BfsResult(C.Structure):
    _fields_ = [("processed_nodes", u32), ("iteration", u32), ("depth", u32),
                ("top_down_steps", u32), ("bottom_up_steps", u32), ("reserved", u32),
                ("edges_traversed", u64)]


class PrResult(C.Structure):
    _fields_ = [("iterations", u32), ("active_last", u32), ("error_total", C.c_double)]


class PprResult(C.Structure):
    _fields_ = [("iterations", u32), ("adjoint_iterations", u32), ("residual", C.c_double),
                ("adjoint_residual", C.c_double), ("loss", C.c_double)]


class SsspResult(C.Structure):
    _fields_ = [("reached", u32), ("rounds", u32), ("edges_relaxed", u64), ("edges_traversed", u64)]


class BcResult(C.Structure):
    _fields_ = [("iteration", u32), ("processed_nodes", u32), ("levels", u32)]


# name -> (restype, argtypes)
SIGNATURES = {
    "gbx_status_string": (C.c_char_p, [C.c_int]),
    "gbx_last_error": (C.c_char_p, []),
    "gbx_version": (C.c_char_p, []),
    "gbx_set_device": (C.c_int, [C.c_int]),
    "gbx_kernel_launches": (u64, []),
    "gbx_graph_create_csr": (C.c_int, [C.POINTER(vp), u32, u32, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    "gbx_graph_create_offsets": (C.c_int, [C.POINTER(vp), u32, u32, vp, vp, vp, vp, vp, vp, vp]),
    "gbx_graph_destroy": (C.c_int, [vp]),
    "gbx_graph_info": (C.c_int, [vp, C.POINTER(u32), C.POINTER(u32), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "gbx_graph_device_arrays": (C.c_int, [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp),
                                          C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)]),
    "gbx_graph_set_tuning": (C.c_int, [vp, C.c_char_p, C.c_double]),
    "gbx_graph_get_tuning": (C.c_int, [vp, C.c_char_p, C.POINTER(C.c_double)]),
    "gbx_autotune": (C.c_int, [vp, u32, u32, vp]),
    "gbx_bfs": (C.c_int, [vp, u32, C.c_int, vp, vp, C.POINTER(BfsResult), vp]),
    "gbx_bfs_trials": (C.c_int, [vp, vp, u32, C.c_int, vp, vp, C.c_uint64, vp, vp]),
    "gbx_bfs_top_down_step": (C.c_int, [vp, vp, u32, vp, vp, vp, u32, C.POINTER(u32), C.POINTER(u32), vp]),
    "gbx_bfs_bottom_up_step": (C.c_int, [vp, vp, vp, vp, vp, C.POINTER(u32), vp]),
    "gbx_pagerank_pull": (C.c_int, [vp, u32, C.c_double, vp, C.POINTER(PrResult), vp]),
    "gbx_pagerank_pull_fp64": (C.c_int, [vp, u32, vp, vp]),
    "gbx_csr_segments_count": (u32, [u32, u32]),
    "gbx_csr_segments": (C.c_int, [u32, vp, vp, vp, u32, u32, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    "gbx_pagerank_pull_noalloc": (C.c_int, [u32, vp, vp, vp, u32, C.c_double, vp, C.POINTER(PrResult), vp]),
    "gbx_bfs_multisource": (C.c_int, [vp, u32, vp, vp, vp, vp]),
    "gbx_batch_create": (C.c_int, [C.POINTER(vp), u32, vp, vp, vp, vp, vp, vp]),
    "gbx_batch_destroy": (C.c_int, [vp]),
    "gbx_batch_info": (C.c_int, [vp, C.POINTER(u32), C.POINTER(u32), C.POINTER(u32)]),
    "gbx_bfs_batched": (C.c_int, [vp, vp, vp, vp, vp, vp]),
    "gbx_pr_batched": (C.c_int, [vp, u32, C.c_double, vp, vp, vp]),
    "gbx_ppr_forward": (C.c_int, [vp, u32, vp, vp, C.c_double, C.c_double, u32, vp, C.POINTER(PprResult), vp]),
    "gbx_ppr_adjoint": (C.c_int, [vp, u32, vp, vp, vp, C.c_double, C.c_double, u32, vp, vp,
                                  C.POINTER(PprResult), vp]),
    "gbx_sssp": (C.c_int, [vp, u32, u32, vp, C.POINTER(SsspResult), vp]),
    "gbx_bellman_ford": (C.c_int, [vp, u32, vp, vp, C.POINTER(SsspResult), vp]),
    "gbx_dfs": (C.c_int, [vp, u32, vp, vp, C.POINTER(u32), vp]),
    "gbx_betweenness": (C.c_int, [vp, u32, vp, vp, vp, vp, vp, C.POINTER(BcResult), vp]),
    "gbx_reference_roots": (C.c_int, [vp, u32, u32, vp]),
    "gbx_mt19937_next": (u32, [C.POINTER(C.c_ulong), C.POINTER(C.c_int)]),
    "gbx_cc": (C.c_int, [vp, C.c_int, vp, C.POINTER(u32), vp]),
    "gbx_tc": (C.c_int, [vp, C.POINTER(u64), vp]),
    "gbx_spmv": (C.c_int, [vp, vp, C.c_float, vp, vp, u32, vp]),
    "gbx_csr_build": (C.c_int, [u32, vp, vp, vp, C.c_int, C.c_int, C.c_int, u32, vp, vp, vp, vp, vp,
                                C.POINTER(u32), vp]),
    "gbx_degree_reorder": (C.c_int, [u32, u32, vp, vp, C.c_int, vp, vp, vp]),
    "gbx_relabel": (C.c_int, [u32, u32, vp, vp, vp, vp, vp, vp]),
    "gbx_mask_graph": (C.c_int, [u32, u32, vp, vp, C.c_int, u32, vp, vp]),
    "gbx_generate_rmat": (C.c_int, [u32, u64, C.c_double, C.c_double, C.c_double, u64, vp, vp]),
    "gbx_generate_values": (C.c_int, [u64, C.c_int, u32, u32, u64, vp]),
    "gbx_generate_chung_lu": (C.c_int, [u32, u64, C.c_double, u32, C.c_double, u64, vp, vp, vp]),
}

_lib = None
_lock = threading.Lock()


class GbxError(RuntimeError):
    def __init__(self, fn: str, status: int, msg: str):
        super().__init__(f"{fn} failed with status {status}: {msg}")
        self.status = status


def load() -> C.CDLL:
    """Load libgbx.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() "
                               "(the CUDA extension is required; there is no CPU fallback)")
        lib = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(fn_name: str, status: int) -> None:
    if status != 0:
        lib = load()
        msg = lib.gbx_last_error().decode(errors="replace")
        raise GbxError(fn_name, status, msg or lib.gbx_status_string(status).decode())


def call(fn_name: str, *args) -> None:
    lib = load()
    check(fn_name, getattr(lib, fn_name)(*args))
