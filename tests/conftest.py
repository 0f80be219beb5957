import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def reference_root():
    """The reference tree the tests may read (None where there is none): the
    GBX_REFERENCE_ROOT environment variable, else the tree oracle/build_ref.sh
    compiled oracle/_ref from."""
    import os

    env = os.environ.get("GBX_REFERENCE_ROOT")
    if env:
        return Path(env)
    rec = ROOT / "oracle" / "_ref" / "reference_root"
    return Path(rec.read_text().strip()) if rec.exists() else None

# one fixture per test graph; reorder_modes.npz holds the labels of the
# reorder modes for all of them, csr_files.npz the reference's .csr files,
# mask_modes.npz its mask mode, bf_dfs_bc.npz Bellman-Ford, DFS and
# betweenness centrality, csr_segments.npz the reference's CSR segments
GOLDEN_GRAPHS = sorted(p.stem for p in GOLDEN.glob("*.npz")
                       if p.stem not in ("reorder_modes", "csr_files", "mask_modes", "bf_dfs_bc", "csr_segments"))
REORDER_MODES = [2, 3, 4, 5, 6, 7, 8, 9, 12, 13]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 host)")


def load_reorder_modes() -> dict:
    with np.load(GOLDEN / "reorder_modes.npz") as z:
        return {k: z[k] for k in z.files}


def load_csr_files() -> dict:
    with np.load(GOLDEN / "csr_files.npz") as z:
        return {k: z[k] for k in z.files}


def load_bf_dfs_bc() -> dict:
    with np.load(GOLDEN / "bf_dfs_bc.npz") as z:
        return {k: z[k] for k in z.files}


def load_mask_modes() -> dict:
    with np.load(GOLDEN / "mask_modes.npz") as z:
        return {k: z[k] for k in z.files}


def load_golden(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def gbx():
    import graphblox_gb300

    graphblox_gb300.load()
    return graphblox_gb300


@pytest.fixture(scope="session")
def cuda_device():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    torch.cuda.set_device(0)
    return torch.device("cuda:0")
