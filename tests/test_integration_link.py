"""The drop-in claim, checked at link level (no GPU): the reference host's own
sources -- graphRun.c's dispatcher, graph loading, preprocessing, utilities --
compiled against include/algorithms/cuda instead of the openmp headers, link
against libgbx_graphblox_dw.so + libgbx.so with every symbol resolved.
Needs the reference tree (present where the fixtures are generated)."""
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import pytest

from conftest import reference_root

ROOT = Path(__file__).resolve().parents[1]
_root = reference_root()
REF = (_root / "01_host") if _root else Path("reference-tree-not-present")
CFG = ROOT / "oracle" / "_ref" / "cfg_dw"

pytestmark = pytest.mark.skipif(not (REF / "src").exists() or not (CFG / "graphConfig.h").exists(),
                                reason="reference sources / oracle/_ref build not present")


def test_reference_host_links_against_cuda_integration(tmp_path, gbx):
    from graphblox_gb300 import _build

    _build.build_integration()
    inc = [f"-I{CFG}", f"-I{ROOT / 'include' / 'algorithms' / 'cuda'}", f"-I{REF / 'include' / 'structures'}",
           f"-I{REF / 'include' / 'preprocess'}", f"-I{REF / 'include' / 'utils_graph'}",
           f"-I{REF / 'include' / 'config'}", f"-I{ROOT / 'oracle' / 'judy_shim'}"]
    srcs = [p for d in ("structures", "preprocess", "utils_graph", "config") for p in sorted((REF / "src" / d).glob("*.c"))]

    def cc(src):
        obj = tmp_path / (src.stem + ".o")
        r = subprocess.run(["g++", "-x", "c++", "-w", "-fopenmp", "-O0", *inc, "-c", str(src), "-o", str(obj)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
        return obj

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(cc, srcs))
    main = tmp_path / "ref_driver.o"
    r = subprocess.run(["g++", "-w", "-fopenmp", "-O0", *inc, "-c", str(ROOT / "oracle" / "ref_driver.cpp"), "-o",
                        str(main)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    exe = tmp_path / "graphblox_cuda"
    r = subprocess.run(["g++", "-fopenmp", "-o", str(exe), *map(str, objs), str(main),
                        f"-L{ROOT / 'graphblox_gb300'}", "-lgbx_graphblox_dw", "-lgbx",
                        f"-Wl,-rpath,{ROOT / 'graphblox_gb300'}", "-Wl,--no-undefined"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    # the dispatcher's algorithm symbols come from the cuda integration library
    nm = subprocess.run(["nm", "-D", str(ROOT / "graphblox_gb300" / "libgbx_graphblox_dw.so")],
                        capture_output=True, text=True).stdout
    for sym in ("breadthFirstSearchGraphCSR", "pageRankGraphCSR", "SSSPGraphCSR", "connectedComponentsGraphCSR",
                "triangleCountGraphCSR", "SPMVGraphCSR", "freeBFSStats", "depthFirstSearchGraphCSR"):
        assert f" T {sym}" in nm, sym
