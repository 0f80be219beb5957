"""The cuda integration's betweenness root draw on the CPU (no GPU call):
generateRandomRootBetweennessCentrality stepped on the reference's
mt19937state, seeded as the reference seeds it, gives the roots the
reference's own Brandes drew (tests/golden/bf_dfs_bc.npz), and leaves the
generator where the reference's would be (the next draws match too)."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_bf_dfs_bc, load_golden
from oracle import pyoracle as po
from test_gpu_integration import Arguments, Built, GraphCSRdw, _seed_mt


def _shim():
    import graphblox_gb300._build as b

    path = b.PKG / "libgbx_graphblox_dw.so"
    if not path.exists():
        pytest.skip("integration library not built")
    lib = C.CDLL(str(path))
    f = lib.generateRandomRootBetweennessCentrality
    f.restype = C.c_uint32
    f.argtypes = [C.c_void_p, C.POINTER(GraphCSRdw)]
    return f


@pytest.mark.parametrize("name", ["v300_e2730", "v1000_e10000", "v8192_e32768"])
def test_shim_root_draw_matches_reference(name):
    draw = _shim()
    more = load_bf_dfs_bc()
    fx = load_golden(name)
    b = Built(fx, "dw", directed=True)
    a = Arguments()
    _seed_mt(a)
    state = C.addressof(a) + Arguments.mt19937var.offset
    roots = [draw(state, C.byref(b.g)) for _ in range(len(more[f"{name}_dw_bc_roots"]))]
    np.testing.assert_array_equal(roots, more[f"{name}_dw_bc_roots"])
    # the stream continues: the next draws are the oracle's next draws
    host = po.HostCSR(b.V, fx["dw_out_degree"], fx["dw_edges_idx"], fx["dw_dest"], None, fx["dw_src"])
    nxt = [draw(state, C.byref(b.g)) for _ in range(3)]
    np.testing.assert_array_equal(nxt, po.random_roots(host, len(roots) + 3)[len(roots):])
