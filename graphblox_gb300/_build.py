"""In-tree build of libgbx.so (CUDA kernels + C ABI) for sm_103a.

Each translation unit under csrc/ is compiled separately and in parallel
(nvcc for .cu, g++ for .cpp), then linked into graphblox_gb300/libgbx.so.
Objects go to graphblox_gb300/_build/ and are rebuilt only when a source or
header is newer. The drop-in integration shims (integration/*.c) are built
into libgbx_graphblox_<variant>.so against libgbx.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INTEG = PKG / "integration"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"
LIB = PKG / "libgbx.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

# Drop-in integration variants: the reference's compile-time GraphCSR layout
# (01_host/include/config/graphConfig.h:13-14) selects which fields exist.
VARIANTS = {"u": (0, 0), "dw": (1, 1)}


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgbx.so")
    return cand


def _cuda_lib_dir() -> str:
    nvcc = Path(_nvcc()).resolve()
    for d in (nvcc.parent.parent / "lib64", nvcc.parent.parent / "lib"):
        if d.exists():
            return str(d)
    return "/usr/local/cuda/lib64"


def _newest_dep(headers: list[Path]) -> float:
    return max((h.stat().st_mtime for h in headers), default=0.0)


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def _compile_jobs() -> list[tuple[Path, Path, list[str]]]:
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    dep_time = _newest_dep(headers)
    jobs = []
    common_inc = [f"-I{INCLUDE}", f"-I{CSRC}"]
    for src in sorted(CSRC.glob("*.cu")):
        obj = BUILD / (src.stem + ".o")
        cmd = [_nvcc(), "-std=c++17", ARCH, "-O3", "-lineinfo", "--expt-relaxed-constexpr",
               "-Xcompiler", "-fPIC,-fopenmp", *common_inc, "-c", str(src), "-o", str(obj)]
        jobs.append((src, obj, cmd, dep_time))
    for src in sorted(CSRC.glob("*.cpp")):
        obj = BUILD / (src.stem + ".o")
        cmd = ["g++", "-std=c++17", "-O3", "-fPIC", "-fopenmp", "-Wall", *common_inc,
               "-c", str(src), "-o", str(obj)]
        jobs.append((src, obj, cmd, dep_time))
    return jobs


def build_lib(verbose: bool = False) -> Path:
    """Compile and link libgbx.so; returns its path."""
    BUILD.mkdir(exist_ok=True)
    jobs = _compile_jobs()
    todo = [(s, o, c) for s, o, c, dt in jobs
            if not o.exists() or o.stat().st_mtime < max(s.stat().st_mtime, dt)]
    workers = max(1, min(len(todo), os.cpu_count() or 4))
    if todo:
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            futs = [ex.submit(_run, c) for _, _, c in todo]
            for f in cf.as_completed(futs):
                f.result()
    objs = [str(o) for _, o, _, _ in jobs]
    if todo or not LIB.exists() or LIB.stat().st_mtime < max(Path(o).stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([_nvcc(), "-shared", ARCH, "-o", str(tmp), *objs, "-Xcompiler", "-fopenmp",
              f"-L{_cuda_lib_dir()}", "-lcudart", "-lgomp"])
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_integration(verbose: bool = False) -> list[Path]:
    """Build the drop-in openmp-symbol shims (one .so per GraphCSR layout)."""
    srcs = sorted(INTEG.glob("*.c"))
    if not srcs:
        return []
    out = []
    headers = list(INCLUDE.rglob("*.h"))
    dep_time = max(_newest_dep(headers), max(s.stat().st_mtime for s in srcs), LIB.stat().st_mtime)
    for name, (directed, weighted) in VARIANTS.items():
        target = PKG / f"libgbx_graphblox_{name}.so"
        if target.exists() and target.stat().st_mtime >= dep_time:
            out.append(target)
            continue
        cmd = ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-Wall", "-Wextra", "-Wno-unused-parameter",
               f"-DGBX_DIRECTED={directed}", f"-DGBX_WEIGHTED={weighted}",
               f"-I{INCLUDE}", f"-I{INCLUDE / 'graphblox'}", f"-I{INCLUDE / 'algorithms' / 'cuda'}",
               "-o", str(target), *map(str, srcs), f"-L{PKG}", "-lgbx", "-Wl,-rpath,$ORIGIN"]
        _run(cmd)
        out.append(target)
    if verbose:
        print("built", ", ".join(str(p) for p in out))
    return out


def build_oracle(verbose: bool = False) -> Path:
    """liboracle.so: the CPU restatement (test infrastructure only)."""
    _run(["make", "-s", "-C", str(ROOT / "oracle")])
    return ROOT / "oracle" / "liboracle.so"


def build_reference(verbose: bool = False, reference_root: str | None = None) -> bool:
    """Compile the reference host into oracle/_ref/ when its sources are present.

    The tree is `reference_root`, else $GBX_REFERENCE_ROOT, else the recipe's
    own default (oracle/build_ref.sh); the recipe exits 2 when no tree is there
    (the GPU host has none), which is not an error."""
    cmd = ["bash", str(ROOT / "oracle" / "build_ref.sh")]
    root = reference_root or os.environ.get("GBX_REFERENCE_ROOT")
    if root:
        cmd.append(root)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode == 2:
        return False
    if res.returncode != 0:
        raise RuntimeError(f"reference build failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return True


def build_all(verbose: bool = False) -> None:
    build_lib(verbose)
    build_integration(verbose)
    build_oracle(verbose)
    build_reference(verbose)


if __name__ == "__main__":
    build_all(verbose=True)
