"""Generate the golden fixtures in tests/golden/*.npz.

Run in a container that has the reference tree (the first argument, or
$GBX_REFERENCE_ROOT, or the tree oracle/_ref was built from) and
its build (oracle/build_ref.sh). For every test graph the reference ships in
03_data/TEST, the fixture stores:
  - the input edge list (graph.bin / graph.wbin records),
  - the reference's own CSR text dumps (03_data/TEST/<g>/graph.*bin.*),
  - outputs of the reference host (oracle/_ref) for each algorithm on that
    graph, per build variant ("u": as shipped, run on the symmetrised,
    deduplicated graph; "dw": DIRECTED 1 / WEIGHTED 1, run on the directed
    graph as is).
The GPU host has no reference tree, so the parity tests read only these
fixtures there.

Usage: python tests/golden/make_golden.py [REFERENCE_ROOT] [reorder|csr|mask|more]
("reorder" writes only reorder_modes.npz, the labels of the reorder modes;
"csr" writes only csr_files.npz, the reference's .csr files; "mask" writes
only mask_modes.npz, the reference's mask mode; "more" writes only
bf_dfs_bc.npz, Bellman-Ford, DFS and betweenness centrality.)
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import pyoracle as po  # noqa: E402

GRAPHS = ["v51_e1021", "v300_e2730", "v500_e500", "v529_e3500", "v1000_e10000", "v1024_e4096",
          "v8192_e32768", "graphbrew", "test"]
ROOTS = [0, 1, 7, 100]


def load_text(p: Path) -> np.ndarray:
    return np.loadtxt(p, dtype=np.int64, ndmin=1)


def main(ref_root: str) -> None:
    test_dir = Path(ref_root) / "03_data" / "TEST"
    out_dir = Path(__file__).resolve().parent
    for name in GRAPHS:
        gdir = test_dir / name
        weighted = (gdir / "graph.wbin").exists() and not (gdir / "graph.bin").exists()
        f = gdir / ("graph.wbin" if weighted else "graph.bin")
        raw = np.fromfile(f, dtype=np.uint32)
        width = 3 if weighted else 2
        rec = raw[: (raw.shape[0] // width) * width].reshape(-1, width)
        fx: dict[str, np.ndarray] = {
            "src": rec[:, 0].copy(),
            "dst": rec[:, 1].copy(),
            "weighted": np.array(int(weighted)),
        }
        if weighted:
            fx["weight"] = rec[:, 2].copy().view(np.float32)
        prefix = gdir / f.name
        if (gdir / (f.name + ".out_degree")).exists():
            od = load_text(Path(str(prefix) + ".out_degree"))
            fx["dump_num_vertices"] = np.array(od[0])
            fx["dump_out_degree"] = od[1:].astype(np.uint32)
            fx["dump_edges_idx"] = load_text(Path(str(prefix) + ".edges_idx")).astype(np.uint32)
            fx["dump_dest"] = load_text(Path(str(prefix) + ".edges_array_dest")).astype(np.uint32)
            fx["dump_src"] = load_text(Path(str(prefix) + ".edges_array_src"))[1:].astype(np.uint32)
        wflag = ["-w"] if weighted else []
        for variant, flags in (("u", ["-s", "-k"]), ("dw", []), ("dwk", ["-k"])):
            exe = "u" if variant == "u" else "dw"
            fl = ["-o", "1", *wflag, *flags]
            csr = po.ref_run(f, exe, -1, fl)
            for k in ("out_degree", "edges_idx", "dest", "src"):
                fx[f"{variant}_{k}"] = csr[k]
            if "weight" in csr:
                fx[f"{variant}_weight"] = csr["weight"]
            V = int(csr["num_vertices"])
            fx[f"{variant}_num_vertices"] = np.array(V)
            bfs_d, bfs_p, bfs_it = [], [], []
            for r in ROOTS:
                if r >= V:
                    continue
                out = po.ref_run(f, exe, 0, [*fl, "-p", "2", "-r", str(r)])
                bfs_d.append(out["bfs_distances"])
                bfs_p.append([r, out["source"], out["processed_nodes"], out["iteration"]])
            fx[f"{variant}_bfs_distances"] = np.stack(bfs_d)
            fx[f"{variant}_bfs_meta"] = np.array(bfs_p, dtype=np.int64)
            out = po.ref_run(f, exe, 1, [*fl, "-i", "20", "-e", "0"])
            fx[f"{variant}_pr20"] = out["pr_ranks"]
            out = po.ref_run(f, exe, 1, [*fl, "-i", "100", "-e", "1e-4"])
            fx[f"{variant}_pr_eps"] = out["pr_ranks"]
            fx[f"{variant}_pr_eps_iterations"] = np.array(out["iterations"])
            out = po.ref_run(f, exe, 2, [*fl, "-r", "1", "-b", "1"], threads=1)
            fx[f"{variant}_sssp"] = out["sssp_distances"]
            fx[f"{variant}_sssp_source"] = np.array(out["source"])
            out = po.ref_run(f, exe, 6, [*fl, "-p", "1"])
            fx[f"{variant}_cc"] = out["cc_components"]
            out = po.ref_run(f, exe, 5, [*fl, "-i", "2"])
            fx[f"{variant}_spmv_x"] = out["spmv_x"]
            fx[f"{variant}_spmv_y"] = out["spmv_y"]
            if variant == "u":
                out = po.ref_run(f, exe, 8, [*fl, "-p", "1"])
                fx["u_tc"] = np.array(out["total_counts"], dtype=np.uint64)
            # degree reordering (out-degree) of the same input
            out = po.ref_run(f, exe, -1, [*fl, "-l", "1"])
            fx[f"{variant}_reorder_label"] = out["label"]
            fx[f"{variant}_reorder_dest"] = out["dest"]
            fx[f"{variant}_reorder_out_degree"] = out["out_degree"]
        np.savez_compressed(out_dir / f"{name}.npz", **fx)
        print(f"wrote {name}.npz")


REORDER_MODES = [2, 3, 4, 5, 6, 7, 8, 9, 12, 13]


def reorder_modes(ref_root: str) -> None:
    """tests/golden/reorder_modes.npz: the reference's label_array after each
    deterministic reorder mode (in/in+out degree, DBG, HUBSort, HUBCluster,
    Corder) on every test graph and build variant (keys
    <graph>_<variant>_l<mode>); the CSR it reorders is <variant>_src /
    _dest / _num_vertices of <graph>.npz."""
    test_dir = Path(ref_root) / "03_data" / "TEST"
    fx: dict[str, np.ndarray] = {}
    for name in GRAPHS:
        gdir = test_dir / name
        weighted = (gdir / "graph.wbin").exists() and not (gdir / "graph.bin").exists()
        f = gdir / ("graph.wbin" if weighted else "graph.bin")
        wflag = ["-w"] if weighted else []
        for variant, flags in (("u", ["-s", "-k"]), ("dw", [])):
            exe = "u" if variant == "u" else "dw"
            fl = ["-o", "1", *wflag, *flags]
            key = f"{name}_{variant}"
            for lm in REORDER_MODES:
                fx[f"{key}_l{lm}"] = po.ref_run(f, exe, -1, [*fl, "-l", str(lm)])["label"]
    out = Path(__file__).resolve().parent / "reorder_modes.npz"
    np.savez_compressed(out, **fx)
    print(f"wrote {out.name}")


CSR_FILE_GRAPHS = ["v51_e1021", "v300_e2730", "v500_e500", "v1024_e4096", "test"]


def csr_files(ref_root: str) -> None:
    """tests/golden/csr_files.npz: the bytes of the .csr file the reference
    writes (writeToBinFileGraphCSR) for a few test graphs, in the shipped
    build (u: -s -k, no weights, no inverse), the DIRECTED 1 / WEIGHTED 1
    build on the graph as read (dw) and the same with dedup (dwk). Keys
    <graph>_<variant>."""
    test_dir = Path(ref_root) / "03_data" / "TEST"
    fx: dict[str, np.ndarray] = {}
    for name in CSR_FILE_GRAPHS:
        gdir = test_dir / name
        weighted = (gdir / "graph.wbin").exists() and not (gdir / "graph.bin").exists()
        f = gdir / ("graph.wbin" if weighted else "graph.bin")
        wflag = ["-w"] if weighted else []
        for variant, flags in (("u", ["-s", "-k"]), ("dw", []), ("dwk", ["-k"])):
            exe = "u" if variant == "u" else "dw"
            fx[f"{name}_{variant}"] = po.ref_run(f, exe, -1, ["-o", "1", *wflag, *flags, "-W"])["graph"]
    out = Path(__file__).resolve().parent / "csr_files.npz"
    np.savez_compressed(out, **fx)
    print(f"wrote {out.name}")


MASK_MODES = [1, 2, 3, 4, 5, 6]
MASK_CACHE_SIZES = [32768, 256]
MASK_CSR_GRAPHS = ["v51_e1021", "v300_e2730", "test"]


def mask_modes(ref_root: str) -> None:
    """tests/golden/mask_modes.npz: the reference's mask mode (-M, -C) run
    with one thread (its hint assignment is schedule-dependent with more).
    Keys: <graph>_<variant>_m<mode>_c<cache_size> = hint per vertex (id >>
    30, uint8) for every test graph, build variant (u, dw), mode 1-6 and two
    cache sizes (the default, whose regions are V/4 on these graphs, and 256,
    whose regions are cs*8, *4, *4 on the larger ones); <graph>_<variant>_m<mode>_csr
    = the .csr file the reference writes for modes 1, 2 (ids carry the hints;
    the DIRECTED build's inverse CSR is sorted on them) on three graphs; and
    <graph>_dw_m1_bfs1 / _pr20 = BFS levels from vertex 1 and 20 PageRank
    iterations on the masked dw graph."""
    test_dir = Path(ref_root) / "03_data" / "TEST"
    fx: dict[str, np.ndarray] = {}
    for name in GRAPHS:
        gdir = test_dir / name
        weighted = (gdir / "graph.wbin").exists() and not (gdir / "graph.bin").exists()
        f = gdir / ("graph.wbin" if weighted else "graph.bin")
        wflag = ["-w"] if weighted else []
        for variant, flags in (("u", ["-s", "-k"]), ("dw", [])):
            exe = "u" if variant == "u" else "dw"
            fl = ["-o", "1", *wflag, *flags]
            for m in MASK_MODES:
                for cs in MASK_CACHE_SIZES:
                    out = po.ref_run(f, exe, -1, [*fl, "-M", str(m), "-C", str(cs)], threads=1)
                    fx[f"{name}_{variant}_m{m}_c{cs}"] = (out["mask"] >> 30).astype(np.uint8)
                if m in (1, 2) and name in MASK_CSR_GRAPHS:
                    out = po.ref_run(f, exe, -1, [*fl, "-M", str(m), "-W"], threads=1)
                    fx[f"{name}_{variant}_m{m}_csr"] = out["graph"]
        if name in MASK_CSR_GRAPHS:
            fl = ["-o", "1", *wflag, "-M", "1"]
            out = po.ref_run(f, "dw", 0, [*fl, "-p", "2", "-r", "1"], threads=1)
            fx[f"{name}_dw_m1_bfs1"] = out["bfs_distances"]
            out = po.ref_run(f, "dw", 1, [*fl, "-i", "20", "-e", "0"], threads=1)
            fx[f"{name}_dw_m1_pr20"] = out["pr_ranks"]
    out = Path(__file__).resolve().parent / "mask_modes.npz"
    np.savez_compressed(out, **fx)
    print(f"wrote {out.name}")


BC_ROOTS = 4


def more_algorithms(ref_root: str) -> None:
    """tests/golden/bf_dfs_bc.npz: Bellman-Ford, DFS and betweenness
    centrality of the reference host on every test graph. Keys
    <graph>_<variant>_...: bf_r<root> (distances; the parents depend on the
    thread schedule), dfs_r<root> / dfs_parents_r<root> / dfs_processed_r<root>
    for roots 0 and 1, and for the DIRECTED 1 build (dw, dwk) bc_roots,
    bc (centrality after BC_ROOTS roots), bc_distances / bc_sigma /
    bc_dependency / bc_processed of the last root. The DIRECTED 0 build's
    Brandes writes past its predecessor lists (sized by in_degree, which
    that build leaves 0) and aborts, so it has no BC keys."""
    test_dir = Path(ref_root) / "03_data" / "TEST"
    fx: dict[str, np.ndarray] = {}
    for name in GRAPHS:
        gdir = test_dir / name
        weighted = (gdir / "graph.wbin").exists() and not (gdir / "graph.bin").exists()
        f = gdir / ("graph.wbin" if weighted else "graph.bin")
        wflag = ["-w"] if weighted else []
        for variant, flags in (("u", ["-s", "-k"]), ("dw", []), ("dwk", ["-k"])):
            exe = "u" if variant == "u" else "dw"
            fl = ["-o", "1", *wflag, *flags]
            key = f"{name}_{variant}"
            out = po.ref_run(f, exe, 3, [*fl, "-r", "1", "-p", "1"])
            fx[f"{key}_bf_r1"] = out["bf_distances"]
            for r in (0, 1):
                out = po.ref_run(f, exe, 4, [*fl, "-r", str(r)], threads=1)
                fx[f"{key}_dfs_r{r}"] = out["dfs_distances"]
                fx[f"{key}_dfs_parents_r{r}"] = out["dfs_parents"]
                fx[f"{key}_dfs_processed_r{r}"] = np.array(out["processed_nodes"])
            if exe == "dw":
                out = po.ref_run(f, exe, 7, [*fl, "-i", str(BC_ROOTS)])
                fx[f"{key}_bc_roots"] = out["bc_roots"]
                fx[f"{key}_bc"] = out["bc_centrality"]
                fx[f"{key}_bc_distances"] = out["bc_distances"]
                fx[f"{key}_bc_sigma"] = out["bc_sigma"]
                fx[f"{key}_bc_dependency"] = out["bc_dependency"]
                fx[f"{key}_bc_processed"] = np.array(out["processed_nodes"])
    out_path = Path(__file__).resolve().parent / "bf_dfs_bc.npz"
    np.savez_compressed(out_path, **fx)
    print(f"wrote {out_path.name}")


SMALL_FOR_SEGMENTS = ["v51_e1021", "v300_e2730", "v500_e500", "v529_e3500", "v1000_e10000", "v1024_e4096", "test"]


def csr_segments(ref_root: str) -> None:
    """csr_segments.npz: the reference's CSR segments (csrSegmentsNew's
    partition and the per-segment preprocessing, -a 100 of
    oracle/ref_driver.cpp, one thread) on every test graph: the directed
    weighted build on the graph as read (sorted by source and destination)
    with the fewest segments (4) and, on the graphs below 1,100 vertices, with
    many (cache size 512), and the undirected build on the symmetrised,
    deduplicated graph. The per-segment CSRs hold every vertex up to the
    segment's largest id, so many segments on a large graph would make the
    fixture large."""
    test_dir = Path(ref_root) / "03_data" / "TEST"
    fx: dict[str, np.ndarray] = {}
    for name in GRAPHS:
        gdir = test_dir / name
        weighted = (gdir / "graph.wbin").exists() and not (gdir / "graph.bin").exists()
        f = gdir / ("graph.wbin" if weighted else "graph.bin")
        wflag = ["-w"] if weighted else []
        runs = [(f"{name}_dw_c1048576", "dw", ["-o", "1", "-C", "1048576"]),
                (f"{name}_u_c1048576", "u", ["-o", "1", "-s", "-k", "-C", "1048576"])]
        if name in SMALL_FOR_SEGMENTS:
            runs.append((f"{name}_dw_c512", "dw", ["-o", "1", "-C", "512"]))
        for key, exe, flags in runs:
            out = po.ref_run(f, exe, 100, [*wflag, *flags], threads=1)
            for k, v in out.items():
                if k in ("num_vertices", "num_edges", "num_segments"):
                    fx[f"{key}_{k}"] = np.array(v)
                else:
                    fx[f"{key}_{k}"] = v
    out_path = Path(__file__).resolve().parent / "csr_segments.npz"
    np.savez_compressed(out_path, **fx)
    print(f"wrote {out_path.name}")


if __name__ == "__main__":
    # the reference tree: the first argument, else $GBX_REFERENCE_ROOT, else
    # the tree oracle/build_ref.sh compiled oracle/_ref from
    rec = Path(__file__).resolve().parents[2] / "oracle" / "_ref" / "reference_root"
    root = (sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GBX_REFERENCE_ROOT")
            or (rec.read_text().strip() if rec.exists() else ""))
    if not root:
        sys.exit("usage: make_golden.py REFERENCE_ROOT [reorder|csr|mask|more] (or set GBX_REFERENCE_ROOT)")
    if len(sys.argv) > 2 and sys.argv[2] == "reorder":
        reorder_modes(root)
    elif len(sys.argv) > 2 and sys.argv[2] == "csr":
        csr_files(root)
    elif len(sys.argv) > 2 and sys.argv[2] == "mask":
        mask_modes(root)
    elif len(sys.argv) > 2 and sys.argv[2] == "more":
        more_algorithms(root)
    elif len(sys.argv) > 2 and sys.argv[2] == "segments":
        csr_segments(root)
    else:
        main(root)
        reorder_modes(root)
