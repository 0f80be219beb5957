"""Benchmark: GraphBlox's CSR kernel set on one GB300, RMAT scale 22.

Workload (the full-kernel-set configuration): RMAT scale 22 (4,194,304
vertices, 2^26 generated edges, a/b/c/d = .57/.19/.19/.05, seed 1), self loops
and duplicates removed, uint32 CSR. One step runs, on the resident graph:
  bfs     direction-optimising BFS from 64 seeded non-isolated roots
  sssp    delta-stepping from 4 of those roots, uint32 weights U[1,255]
  cc      Afforest on the symmetrised graph
  tc      triangle count on the symmetrised, degree-ordered graph (DAG)
  spmv    y = A x, values U(0,1], x U[-1,1] (FP32)
  pr      pull PageRank, 20 iterations (FP32 ranks, FP64 residual)
  reorder count-sort degree reordering of the directed edge list
Metric: GTEPS per kernel and its fraction of the measured HBM roofline; the
headline `value` is the kernel set's aggregate GTEPS (sum of traversed edges
over sum of kernel times). Traversed edges follow the Graph500 convention
(BFS/SSSP: out-degree sum of reached vertices per source), E*iterations for
PR, E for SpMV/CC/reorder, |E+| (DAG edges) for TC.

`value` times kernels on device-resident inputs with CUDA events on the
launching stream, L2 flushed (256 MiB write) before every kernel. `e2e` is
the same metric through the C ABI with pinned host buffers: the CSR upload,
every kernel and the copy-back of every result inside the timed region.

--impl reference times the CPU oracle port (oracle/gbx_oracle.c, OpenMP on
all host cores) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import gc as pygc
import json
import os
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SCALE = 22
EDGE_FACTOR = 16
SEED = 1
N_ROOTS = 64
N_SSSP_ROOTS = 4
PR_ITERS = 20
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of each
# kernel, from ncu captures of this workload on a GB300 (profiles/): bfs and
# sssp one source (--set full), pr one iteration, spmv one launch.
NCU_TRAFFIC_PER_LAUNCH = {"pr": 0.4006e9, "bfs": 0.1688e9, "sssp": 1.946e9, "spmv": 0.6775e9}
W_LO, W_HI = 1, 255
# differentiable personalised PageRank: RMAT-20, 2^24 edges as generated,
# lognormal(0,1) weights, 64 teleport columns of 32 seeds, d 0.85 to 1e-7 L1
PPR_SCALE, PPR_EDGES, PPR_K, PPR_SEEDS, PPR_TOL, PPR_D = 20, 1 << 24, 64, 32, 1e-7, 0.85
# batched: 2,048 RMAT graphs, BFS from 0 plus 30 PageRank iterations each
BATCH_GRAPHS, BATCH_PR_ITERS = 2048, 30
MS_SOURCES = 256  # multi-source bitmask BFS on the RMAT-22 graph
C5_V, C5_MEAN = 40_000_000, 30  # scale-up: Chung-Lu 4e7 vertices, 1.2e9 edges (opt-in, --c5)


T0 = time.time()


def log(*a):
    print(f"[{time.time() - T0:6.1f}s]", *a, file=sys.stderr, flush=True)


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# workload construction (untimed)


def build_workload(gbx, scale=SCALE, ef=EDGE_FACTOR, seed=SEED):
    """The RMAT workload generated and built on the GPU (the library's own
    generator and gbx_csr_build / gbx_degree_reorder)."""
    V = 1 << scale
    t0 = time.time()
    src, dst = gbx.generate_rmat(scale, V * ef, seed=seed)
    w = gbx.generate_values(src.shape[0], 0, W_LO, W_HI, seed=seed + 11)
    el = gbx.EdgeList(V, src, dst, w)
    g = gbx.graph_csr_preprocessing(el, sort=1, dedup=True, directed=True, keep_weights=True)
    # symmetrised, deduplicated graph for CC/TC, and its degree-ordered form
    sym = gbx.EdgeList(V, np.concatenate([src, dst]), np.concatenate([dst, src]))
    gs = gbx.graph_csr_preprocessing(sym, sort=1, dedup=True, directed=False, keep_weights=False)
    elr = gbx.EdgeList(V, gs.src.copy(), gs.dest.copy())
    gbx.degree_reorder(elr, 1)
    gsr = gbx.graph_csr_preprocessing(elr, sort=1, directed=False, keep_weights=False)
    x = gbx.generate_values(V, 2, seed=seed + 21)
    vals = gbx.generate_values(g.num_edges, 1, seed=seed + 31)
    roots = pick_roots(g.out_degree, seed)
    log(f"workload built in {time.time() - t0:.1f}s: V={V} E={g.num_edges} Esym={gs.num_edges}")
    return dict(V=V, g=g, gs=gs, gsr=gsr, x=x, vals=vals, roots=roots, edges_src=g.src, edges_dst=g.dest,
                reorder_labels=(elr.label_array, elr.inverse_label_array))


def pick_roots(out_degree, seed=SEED):
    rng = np.random.default_rng(seed)
    nz = np.nonzero(out_degree)[0]
    return [int(r) for r in rng.choice(nz, N_ROOTS, replace=False)]


class HostGraph:
    """A CSR in the reference's layout, built on the CPU by the oracle."""

    def __init__(self, V, csr, inverse=None):
        self.num_vertices = V
        self.num_edges = int(csr.dest.shape[0])
        self.out_degree, self.edges_idx, self.dest, self.src, self.weight = (
            csr.out_degree, csr.edges_idx, csr.dest, csr.src, csr.weight)
        self.inverse_out_degree = self.inverse_edges_idx = self.inverse_dest = self.inverse_weight = None
        if inverse is not None:
            self.inverse_out_degree, self.inverse_edges_idx = inverse.out_degree, inverse.edges_idx
            self.inverse_dest, self.inverse_weight = inverse.dest, inverse.weight


def build_workload_oracle(scale=SCALE, ef=EDGE_FACTOR, seed=SEED):
    """The same workload generated and built on the host cores by the oracle
    (oracle/gbx_oracle.c: the same generator streams, the reference's sort /
    dedup / map and degree reordering), without the GPU library."""
    from oracle import pyoracle as po

    V = 1 << scale
    t0 = time.time()
    src, dst = po.generate_rmat(scale, V * ef, seed=seed)
    w = po.generate_values(src.shape[0], 0, W_LO, W_HI, seed=seed + 11)
    fwd = po.build_csr(V, src, dst, w, sort_mode=1, dedup=True)
    inv = po.build_csr(V, fwd.dest, fwd.src, fwd.weight, sort_mode=1)
    g = HostGraph(V, fwd, inv)
    sym = po.build_csr(V, np.concatenate([src, dst]), np.concatenate([dst, src]), None, sort_mode=1, dedup=True)
    gs = HostGraph(V, sym)
    rs, rd, lab, ilab = po.degree_reorder(V, sym.src, sym.dest, 1)
    gsr = HostGraph(V, po.build_csr(V, rs, rd, None, sort_mode=1))
    x = po.generate_values(V, 2, seed=seed + 21)
    vals = po.generate_values(g.num_edges, 1, seed=seed + 31)
    roots = pick_roots(g.out_degree, seed)
    log(f"oracle workload built on the host cores in {time.time() - t0:.1f}s")
    return dict(V=V, g=g, gs=gs, gsr=gsr, x=x, vals=vals, roots=roots, edges_src=g.src, edges_dst=g.dest,
                reorder_labels=(lab, ilab))


def tc_stats(gsr):
    """|E+| (DAG edges: neighbours with a smaller degree-order id) and the
    triangle count's byte figures: `compulsory` = the DAG read once,
    4(V+1) + 4|E+|, the roofline's bytes; `merge` = sum over DAG edges of
    4(d+u + d+v), what a merge-based intersection would stream (reported
    beside it, not used for the roofline)."""
    deg = gsr.out_degree.astype(np.int64)
    src = np.repeat(np.arange(gsr.num_vertices, dtype=np.int64), deg)
    dst = gsr.dest.astype(np.int64)
    lower = dst <= src
    dplus = np.bincount(src[lower], minlength=gsr.num_vertices).astype(np.int64)
    e_plus = int(lower.sum())
    compulsory = 4 * (gsr.num_vertices + 1) + 4 * e_plus
    merge = compulsory + int((4 * (dplus[src[lower]] + dplus[dst[lower]])).sum())
    return e_plus, compulsory, merge


# ---------------------------------------------------------------------------
# clocks


class collector_held:
    """Python's cyclic garbage collector is held off while steps are timed
    (it runs once just before): a collection inside a step stalls the host
    thread that issues the library calls, by tens of milliseconds with the
    workload's objects alive."""

    def __enter__(self):
        pygc.collect()
        self.was = pygc.isenabled()
        pygc.disable()

    def __exit__(self, *exc):
        if self.was:
            pygc.enable()
        return False


class ClockSampler:
    def __init__(self):
        self.proc = None
        # raw nvidia-smi samples; their summary goes into the JSON line
        self.path = Path(tempfile.gettempdir()) / f"gbx_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self, device_index=0):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9 or parts[0] != str(device_index):
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# replicas: one full workload per rank, no data-path collective


def reduce_over_ranks(dist, local_ms, local_edges, device=None):
    """(ms, GTEPS) of the whole job: the slowest rank's step time, and every
    rank's traversed edges over it. Every replica runs the same workload
    (weak scaling), so the job's edges are world * local_edges."""
    if not dist or not dist.is_initialized() or dist.get_world_size() == 1:
        return local_ms, (local_edges / (local_ms * 1e-3) / 1e9 if local_ms else 0.0)
    import torch

    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
    world = dist.get_world_size()
    return ms, (world * local_edges / (ms * 1e-3) / 1e9 if ms else 0.0)


def shard(n, rank, world):
    """The contiguous share [lo, hi) of n independent units (graphs of a
    batch, BFS sources) that rank `rank` of `world` runs."""
    return n * rank // world, n * (rank + 1) // world


def job_reduce(dist, ms, edges, device=None):
    """(slowest rank's ms, every rank's edges summed) for sharded work."""
    if not dist or not dist.is_initialized() or dist.get_world_size() == 1:
        return ms, edges
    import torch

    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    e = torch.tensor([float(edges)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(e, op=dist.ReduceOp.SUM)
    return float(t.item()), float(e.item())


# ---------------------------------------------------------------------------
# GPU arm


def run_gpu(args):
    import torch

    import graphblox_gb300 as gbx
    from graphblox_gb300 import _lib

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    _lib.call("gbx_set_device", local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    W = build_workload(gbx, scale=args.scale)
    g, gs, gsr = W["g"], W["gs"], W["gsr"]
    V, E = g.num_vertices, g.num_edges
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    dg = gbx.DeviceGraph.from_graph_csr(g, stream=sp)
    dgs = gbx.DeviceGraph.from_graph_csr(gs, use_weights=False, stream=sp)
    dgr = gbx.DeviceGraph.from_graph_csr(gsr, use_weights=False, stream=sp)
    for h in (dg, dgs, dgr):
        h.label_array = None  # roots are given in the graph's own ids
    # the in-house autotuner picks the BFS direction threshold and the SSSP
    # bucket width on this graph (untimed setup; results do not depend on them)
    if args.tuning:
        # fixed knob values (profiling runs that must not include autotuning launches)
        for kv in args.tuning.split(","):
            k, v = kv.split("=")
            dg.set_tuning(k, float(v))
        tuning = {k: dg.get_tuning(k) for k in ("bfs_alpha", "bfs_beta", "sssp_delta", "pull_heavy_min")}
    elif not args.no_autotune:
        tuning = dg.autotune(bfs=True, sssp=True, samples=4, stream=sp, pull=True)
    else:
        tuning = {}
    log(f"autotune: {tuning}")
    # device-resident buffers
    dist_d = torch.empty(V, dtype=torch.int32, device=dev)
    par_d = torch.empty(V, dtype=torch.int32, device=dev)
    sssp_d = torch.empty(V, dtype=torch.int32, device=dev)
    comp_d = torch.empty(V, dtype=torch.int32, device=dev)
    ranks_d = torch.empty(V, dtype=torch.float32, device=dev)
    x_d = torch.from_numpy(W["x"]).to(dev)
    vals_d = torch.from_numpy(W["vals"]).to(dev)
    y_d = torch.zeros(V, dtype=torch.float32, device=dev)
    es_d = torch.from_numpy(W["edges_src"].view(np.int32)).to(dev)
    ed_d = torch.from_numpy(W["edges_dst"].view(np.int32)).to(dev)
    es_w = torch.empty_like(es_d)
    ed_w = torch.empty_like(ed_d)
    lab_d = torch.empty(V, dtype=torch.int32, device=dev)
    inv_d = torch.empty(V, dtype=torch.int32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    e_plus, tc_bytes, tc_merge_bytes = tc_stats(gsr)
    roots = W["roots"]
    sssp_roots = roots[:N_SSSP_ROOTS]
    ident = torch.arange(V, dtype=torch.int32, device=dev)

    def kernels():
        """(name, fn) -> fn returns (traversed edges, algorithmic bytes)"""
        def bfs():
            # the reference's trial loop: one traversal per root, enqueued
            # back to back (gbx_bfs_trials), one host synchronisation
            te = tb = 0
            for st in gbx.breadth_first_search_trials(dg, roots, 2, distances=dist_d, parents=par_d, stream=sp):
                te += st.edges_traversed
                tb += 4 * (V + 1) + 4 * st.edges_traversed + 8 * V
            return te, tb

        def sssp():
            te = tb = 0
            for r in sssp_roots:
                st = gbx.sssp(dg, r, 0, distances=sssp_d, stream=sp)
                te += st.edges_traversed
                tb += 4 * (V + 1) + 8 * st.edges_traversed + 8 * V
            return te, tb

        def cc():
            gbx.connected_components(dgs, 1, components=comp_d, stream=sp)
            return gs.num_edges, 4 * (V + 1) + 8 * gs.num_edges + 8 * V

        def tc():
            gbx.triangle_count(dgr, stream=sp)
            return e_plus, tc_bytes

        def spmv():
            y_d.zero_()
            gbx.spmv(dg, x_d, values=vals_d, iterations=1, y=y_d, stream=sp)
            return E, 12 * E + 8 * V

        def pr():
            gbx.page_rank(dg, PR_ITERS, 0.0, ranks=ranks_d, stream=sp)
            return E * PR_ITERS, PR_ITERS * (8 * E + 20 * V)

        def reorder():
            es_w.copy_(es_d)
            ed_w.copy_(ed_d)
            lab_d.copy_(ident)
            _lib.call("gbx_degree_reorder", V, E, es_w.data_ptr(), ed_w.data_ptr(), 1, lab_d.data_ptr(),
                      inv_d.data_ptr(), sp)
            return E, 20 * E + 24 * V

        return [("bfs", bfs), ("sssp", sssp), ("cc", cc), ("tc", tc), ("spmv", spmv), ("pr", pr),
                ("reorder", reorder)]

    ks = [(n, f) for n, f in kernels() if not args.only or n in args.only.split(",")]
    ev = {n: [] for n, _ in ks}
    work = {}

    def one_step(record):
        for n, fn in ks:
            flush.fill_(1)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            te, tb = fn()
            b.record(stream)
            if record:
                ev[n].append((a, b))
                work[n] = (te, tb)

    for _ in range(args.warmup):
        one_step(False)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler()
    clocks.start()
    launches0 = _lib.load().gbx_kernel_launches()
    torch.cuda.synchronize()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    with collector_held():
        for _ in range(args.steps):
            one_step(True)
    t_end.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches = _lib.load().gbx_kernel_launches() - launches0
    clk = clocks.stop(local)
    wall_ms = t_start.elapsed_time(t_end)
    per = {}
    peak, peak_kind = peaks()
    tot_edges = tot_ms = 0.0
    for n, _ in ks:
        ms = float(np.mean([a.elapsed_time(b) for a, b in ev[n]]))
        te, tb = work[n]
        per[n] = {"ms": round(ms, 4), "gteps": round(te / (ms * 1e-3) / 1e9, 3),
                  "achieved_gbs": round(tb / (ms * 1e-3) / 1e9, 1),
                  "frac": round(tb / (ms * 1e-3) / 1e9 / peak, 3), "edges": int(te), "alg_bytes": int(tb)}
        if n in NCU_TRAFFIC_PER_LAUNCH:
            # DRAM bytes one launch moved under ncu, over this run's time per launch
            per_step = {"bfs": len(roots), "sssp": len(sssp_roots), "pr": PR_ITERS}.get(n, 1)
            per[n]["dram_frac"] = round(NCU_TRAFFIC_PER_LAUNCH[n] * per_step / (ms * 1e-3) / 1e9 / peak, 3)
        if n == "tc":
            per[n]["merge_bytes"] = int(tc_merge_bytes)
            per[n]["note"] = ("alg_bytes = the DAG read once, 4(V+1) + 4|E+|; merge_bytes = what a merge "
                              "intersection would stream; the kernel probes shared-memory tables instead")
        tot_edges += te
        tot_ms += ms
    ms_step, gteps = reduce_over_ranks(dist, tot_ms, tot_edges, torch.device("cuda", local) if dist else None)
    dom = max(per, key=lambda n: per[n]["ms"]) if per else None
    roof = None if dom is None else {"kernel": dom, "bound": "hbm", "achieved": per[dom]["achieved_gbs"], "peak": peak,
            "peak_kind": peak_kind, "unit": "GB/s", "frac": per[dom]["frac"],
            "traffic": args.traffic if args.traffic is not None else NCU_TRAFFIC_PER_LAUNCH.get(dom),
            "traffic_unit": "bytes per launch",
            "note": "achieved = algorithmic bytes / CUDA-event time; traffic = DRAM bytes of one launch from ncu"}

    ppr = None
    if not args.no_ppr and (not args.only or "ppr" in args.only.split(",")):
        ppr = run_ppr(args, torch, gbx, dev, stream, peak)
    batched = None
    if not args.no_batched and (not args.only or "batched" in args.only.split(",")):
        batched = run_batched(args, torch, gbx, _lib, dev, stream, peak, dist, rank, world)
        batched["multisource"] = run_multisource(args, torch, gbx, _lib, dg, W, dev, stream, peak, dist, rank,
                                                 world)
    more = None
    if not args.no_more and (not args.only or "more" in args.only.split(",")):
        more = run_more(args, torch, gbx, dg, g, stream, peak)
    c5 = None
    if not args.no_c5 and (not args.only or "c5" in args.only.split(",")):
        dg.close(), dgs.close(), dgr.close()
        torch.cuda.empty_cache()
        c5 = run_c5(args, torch, gbx, _lib, dev, stream, peak)
        dg = gbx.DeviceGraph.from_graph_csr(g, stream=sp)
        dgs = gbx.DeviceGraph.from_graph_csr(gs, use_weights=False, stream=sp)
        dgr = gbx.DeviceGraph.from_graph_csr(gsr, use_weights=False, stream=sp)
    e2e = None if args.no_e2e else run_e2e(gbx, _lib, W, args, roots, sssp_roots, e_plus, tuning)
    cpu = parity = None
    if rank == 0 and not (args.no_cpu_baseline and args.no_parity):
        Wc = build_workload_oracle(scale=args.scale)
        if args.no_cpu_baseline:
            from oracle import pyoracle as po

            tri_oracle = po.triangle_count(po.HostCSR(V, Wc["gsr"].out_degree, Wc["gsr"].edges_idx, Wc["gsr"].dest))
        else:
            cpu, tri_oracle = cpu_baseline(Wc)
        if not args.no_parity:
            t0 = time.time()
            parity = parity_kernel_set(torch, gbx, W, Wc, dg, dgs, dgr, tri_oracle, stream)
            log(f"parity checked in {time.time() - t0:.1f}s: all exact {parity['all_exact']}")
        del Wc
    dg.close(), dgs.close(), dgr.close()
    line = {
        "metric": "GTEPS per kernel (aggregate over the kernel set) & %HBM-peak per kernel",
        "value": round(gteps, 3), "unit": "GTEPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32 (ids, levels, distances) + f32 (ranks, SpMV)",
        "data": "synthetic",
        "config": workload_config(args, V, E, gs.num_edges, e_plus, world), "tuning": tuning,
        "kernels": per, "parity": parity, "batched": batched, "ppr_adjoint": ppr, "more": more, "c5": c5, "roofline": roof, "e2e": e2e, "cpu_baseline": cpu, "clocks": clk,
        "gpu_launches": int(launches), "wall_ms_timed_region": round(wall_ms, 3),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
        log("bench done")
    if dist:
        dist.destroy_process_group()


BC_ROOTS = 20  # the reference's default -i for Brandes (graphConfig.c:59)


def run_more(args, torch, gbx, dg, g, stream, peak):
    """Betweenness centrality, Bellman-Ford and DFS (outside the headline
    kernel set). Brandes runs the reference's default 20 roots on the RMAT-22
    graph in one gbx_betweenness call (each root's reached edges are counted
    in an untimed pass first); per root the algorithmic bytes are 16 E_r + 12 P + 44 V_r
    + 12 V (E_r: successor entries of reached vertices, read forward and
    backward with a level check each; P: DAG edges, which add sigma forward
    and read sigma and dependency backward; V_r: reached vertices; the three
    per-root arrays cleared). DFS walks one vertex at a time, so it runs on a
    small RMAT-16 graph."""
    from oracle import pyoracle as po

    sp = stream.cuda_stream
    V = g.num_vertices
    dev = stream.device
    deg = torch.from_numpy(g.out_degree.astype(np.int64)).to(dev)
    roots = gbx.reference_roots(dg, BC_ROOTS)
    bc = torch.zeros(V, dtype=torch.float32, device=dev)
    dist = torch.empty(V, dtype=torch.int32, device=dev)
    sig = torch.empty(V, dtype=torch.int32, device=dev)
    dep = torch.empty(V, dtype=torch.float32, device=dev)
    out = dict(centrality=bc, distances=dist, sigma=sig, dependency=dep, stream=sp)
    # untimed: each root's reached vertices and edges, one root per call
    e_r = p_tot = v_r = 0
    for r in roots:
        st = gbx.betweenness_centrality(dg, roots=[r], **out)
        torch.cuda.synchronize()
        reached = dist != -1
        e_r += int(deg[reached].sum().item())
        v_r += int(reached.sum().item())
        p_tot += st.processed_nodes
    # timed: the 20 roots in one call, as the reference's loop runs them
    bc.zero_()
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    gbx.betweenness_centrality(dg, roots=roots, **out)
    b.record(stream)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b)
    alg = 16 * e_r + 12 * p_tot + 44 * v_r + 12 * V * len(roots)
    bc_sec = {"roots": len(roots), "ms": round(ms, 3), "ms_per_root": round(ms / len(roots), 3),
              "gteps": round(2 * e_r / (ms * 1e-3) / 1e9, 3), "achieved_gbs": round(alg / (ms * 1e-3) / 1e9, 1),
              "frac": round(alg / (ms * 1e-3) / 1e9 / peak, 3), "alg_bytes": int(alg)}
    if not args.no_cpu_baseline:
        host = po.HostCSR(V, g.out_degree, g.edges_idx, g.dest, None, g.src)
        pull = po.HostCSR(V, g.inverse_out_degree, g.inverse_edges_idx, g.inverse_dest)
        t0 = time.time()
        po.betweenness(host, roots[:1], pull)
        bc_sec["cpu_ms_per_root"] = round((time.time() - t0) * 1e3, 1)
        bc_sec["cpu"] = "oracle/gbx_oracle.c Brandes, one root, one thread (the reference's Brandes loop is serial)"
    # Bellman-Ford: the SSSP engine plus the parent pass, 4 roots
    bf_roots = roots[:4]
    par = torch.empty(V, dtype=torch.int32, device=dev)
    a.record(stream)
    for r in bf_roots:
        gbx.bellman_ford(dg, int(r), distances=dist, parents=par, stream=sp, map_source=False)
    b.record(stream)
    torch.cuda.synchronize()
    bf_sec = {"roots": len(bf_roots), "ms_per_root": round(a.elapsed_time(b) / len(bf_roots), 3),
              "note": "SSSP engine (distances) + one parent pass over the forward CSR"}
    # DFS on RMAT-16
    Vs = 1 << 16
    src, dst = gbx.generate_rmat(16, Vs * 16, seed=5)
    gd = gbx.graph_csr_preprocessing(gbx.EdgeList(Vs, src, dst), sort=1, dedup=True, directed=False,
                                     keep_weights=False)
    dfs_sec = {}
    with gbx.DeviceGraph.from_graph_csr(gd, use_weights=False, stream=sp) as dd:
        nz = [int(v) for v in np.nonzero(gd.out_degree)[0][:4]]
        gbx.depth_first_search(dd, nz[0], stream=sp)
        torch.cuda.synchronize()
        a.record(stream)
        pops = 0
        for r in nz:
            pops += gbx.depth_first_search(dd, r, stream=sp).processed_nodes
        b.record(stream)
        torch.cuda.synchronize()
        dms = a.elapsed_time(b)
        dfs_sec = {"graph": "rmat16 directed", "roots": len(nz), "ms_per_root": round(dms / len(nz), 3),
                   "ns_per_pop": round(dms * 1e6 / max(pops, 1), 1)}
        if not args.no_cpu_baseline:
            hd = po.HostCSR(Vs, gd.out_degree, gd.edges_idx, gd.dest)
            t0 = time.time()
            for r in nz:
                po.dfs(hd, r)
            dfs_sec["cpu_ms_per_root"] = round((time.time() - t0) * 1e3 / len(nz), 3)
    return {"betweenness": bc_sec, "bellman_ford": bf_sec, "dfs": dfs_sec}


def run_ppr(args, torch, gbx, dev, stream, peak):
    """Personalised PageRank forward and adjoint (gbx_ppr_forward /
    gbx_ppr_adjoint) on device-resident inputs: mean CUDA-event time of each
    over `steps` calls after one untimed call of each, and (fwd+adj)/fwd.
    Algorithmic bytes per sweep, K columns: 4(V+1) offsets + 8E (index +
    weight) + 4K*E (neighbour-row gather) + 8K*V (row read + write)."""
    scale = args.ppr_scale
    V, E, K = 1 << scale, PPR_EDGES >> (PPR_SCALE - scale), PPR_K
    s, d = gbx.generate_rmat(scale, E, seed=SEED)
    order = np.argsort(s, kind="stable")
    dst = np.ascontiguousarray(d[order])
    off = np.zeros(V + 1, np.int64)
    off[1:] = np.cumsum(np.bincount(s, minlength=V))
    off = off.astype(np.uint32)
    w = gbx.generate_values(E, 3, seed=SEED + 1)
    rng = np.random.default_rng(SEED)
    T = np.zeros((V, K), np.float32)
    for k in range(K):
        T[rng.choice(V, PPR_SEEDS, replace=False), k] = 1.0 / PPR_SEEDS
    Wl = rng.standard_normal((V, K)).astype(np.float32)
    dg = gbx.DeviceGraph.from_offsets(V, off, dst)
    sp = stream.cuda_stream
    w_d, T_d, W_d = (torch.from_numpy(a).to(dev) for a in (w, T, Wl))
    R_d = torch.empty((V, K), dtype=torch.float32, device=dev)
    gw_d = torch.empty(E, dtype=torch.float32, device=dev)
    gt_d = torch.empty((V, K), dtype=torch.float32, device=dev)

    def fwd():
        return gbx.ppr_forward(dg, w_d, T_d, PPR_D, PPR_TOL, ranks=R_d, stream=sp)

    def adj():
        return gbx.ppr_adjoint(dg, w_d, R_d, W_d, PPR_D, PPR_TOL, grad_weights=gw_d, grad_teleport=gt_d, stream=sp)

    fwd(), adj()  # builds the graph's in-edge order and chunk tables (untimed)
    times = {"fwd": [], "adj": []}
    info = {}
    for _ in range(max(1, args.steps)):
        for name, fn in (("fwd", fwd), ("adj", adj)):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            st = fn()
            b.record(stream)
            torch.cuda.synchronize()
            times[name].append(a.elapsed_time(b))
            info[name] = st
    dg.close()
    f_ms, a_ms = float(np.mean(times["fwd"])), float(np.mean(times["adj"]))
    sweep_bytes = 4 * (V + 1) + 8 * E + 4 * K * E + 8 * K * V
    fi, ai = info["fwd"].iterations, info["adj"].iterations
    gbs_f = fi * sweep_bytes / (f_ms * 1e-3) / 1e9
    gbs_a = ai * sweep_bytes / (a_ms * 1e-3) / 1e9
    return {"workload": f"rmat{scale}_ppr_k{K}", "num_vertices": V, "num_edges": E, "K": K,
            "damping": PPR_D, "tol_l1": PPR_TOL, "forward_ms": round(f_ms, 3), "adjoint_ms": round(a_ms, 3),
            "fwd_plus_adjoint_over_fwd": round((f_ms + a_ms) / f_ms, 3),
            "forward_sweeps": fi, "adjoint_sweeps": ai, "loss": info["adj"].loss,
            "forward_gbs": round(gbs_f, 1), "adjoint_gbs": round(gbs_a, 1),
            "forward_frac": round(gbs_f / peak, 3), "adjoint_frac": round(gbs_a / peak, 3),
            "alg_bytes_per_sweep": int(sweep_bytes),
            "note": "adjoint_ms includes dL/dw (one more gather pass), dL/dT and the FP64 loss"}


def run_batched(args, torch, gbx, _lib, dev, stream, peak, dist=None, rank=0, world=1):
    """2,048 RMAT graphs (scale ~U[8,15], V = floor(2^s), edge factor
    ~U[4,32]) packed back to back: one step = BFS from vertex 0 plus 30
    PageRank iterations on every graph. Batched: gbx_bfs_batched +
    gbx_pr_batched (two persistent launches). Per instance: gbx_bfs +
    gbx_pagerank_pull called once per graph on resident single graphs, the
    same device output arrays. Both timed with CUDA events, mean of `steps`.
    With several ranks each takes a contiguous share of the graphs (the
    work queue's natural shard, no collective on the data path); the job's
    time is the slowest rank's and its edges are every rank's."""
    t0 = time.time()
    gl = gbx.generate_rmat_batch(args.batch_graphs, seed=SEED)
    lo, hi = shard(len(gl), rank, world)
    gl = gl[lo:hi]
    packed = gbx.pack_graphs(gl)
    del gl
    G = packed.num_graphs
    vb = packed.vertex_base.astype(np.int64)
    Vt, Et = int(vb[-1]), int(packed.offsets[-1])
    log(f"batch built in {time.time() - t0:.1f}s: {G} graphs, V={Vt} E={Et}")
    sp = stream.cuda_stream
    batch = gbx.GraphBatch(packed, stream=sp)
    singles = []
    for g in range(G):
        V, off, dest, ioff, isrc = packed.graph(g)
        singles.append(gbx.DeviceGraph.from_offsets(V, off, dest, in_offsets=ioff, in_src=isrc, stream=sp))
    src_d = torch.zeros(G, dtype=torch.int32, device=dev)
    dist_d = torch.empty(Vt, dtype=torch.int32, device=dev)
    par_d = torch.empty(Vt, dtype=torch.int32, device=dev)
    ranks_d = torch.empty(Vt, dtype=torch.float32, device=dev)
    bres = (_lib.BfsResult * G)()
    pres = (_lib.PrResult * G)()

    def batched():
        _lib.call("gbx_bfs_batched", batch.handle, src_d.data_ptr(), dist_d.data_ptr(), par_d.data_ptr(), bres, sp)
        _lib.call("gbx_pr_batched", batch.handle, BATCH_PR_ITERS, 0.0, ranks_d.data_ptr(), pres, sp)

    r1 = _lib.BfsResult()
    r2 = _lib.PrResult()

    def per_instance():
        for g, dg in enumerate(singles):
            o = int(vb[g]) * 4
            _lib.call("gbx_bfs", dg.handle, 0, 2, dist_d.data_ptr() + o, par_d.data_ptr() + o, _lib.C.byref(r1), sp)
            _lib.call("gbx_pagerank_pull", dg.handle, BATCH_PR_ITERS, 0.0, ranks_d.data_ptr() + o,
                      _lib.C.byref(r2), sp)

    def timed(fn, n):
        out = []
        for _ in range(n):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            out.append(a.elapsed_time(b))
        return float(np.mean(out))

    timed(batched, 2)
    l0 = _lib.load().gbx_kernel_launches()
    b_ms = timed(batched, max(1, args.steps))
    b_launches = (_lib.load().gbx_kernel_launches() - l0) // max(1, args.steps)
    timed(per_instance, 1)  # builds the single graphs' pull plans
    l0 = _lib.load().gbx_kernel_launches()
    p_ms = timed(per_instance, max(1, min(args.steps, 2)))
    p_launches = (_lib.load().gbx_kernel_launches() - l0) // max(1, min(args.steps, 2))
    parity = None
    if not args.no_parity:
        batched()
        torch.cuda.synchronize()
        parity = batched_parity(packed, dist_d.cpu().numpy().view(np.uint32), ranks_d.cpu().numpy(), bres, pres)
    m_reach = sum(int(r.edges_traversed) for r in bres)
    nv = np.diff(vb)
    edges = m_reach + BATCH_PR_ITERS * Et
    alg = (4 * (Vt + G) + 4 * m_reach + 8 * Vt) + BATCH_PR_ITERS * (8 * Et + 4 * (Vt + G) + 16 * Vt)
    for dg in singles:
        dg.close()
    batch.close()
    dev_r = dev if dist else None
    b_job, e_job = job_reduce(dist, b_ms, edges, dev_r)
    p_job, _ = job_reduce(dist, p_ms, 0, dev_r)
    return {"workload": f"rmat_batch_{args.batch_graphs}_graphs", "num_graphs": G, "num_vertices": Vt,
            "num_edges": Et, "rank_graphs": [int(lo), int(hi)], "job_batched_ms": round(b_job, 3),
            "job_per_instance_ms": round(p_job, 3), "job_batched_gteps": round(e_job / (b_job * 1e-3) / 1e9, 3),
            "graph_vertices_min_max": [int(nv.min()), int(nv.max())], "pr_iterations": BATCH_PR_ITERS,
            "batched_ms": round(b_ms, 3), "per_instance_ms": round(p_ms, 3),
            "speedup_vs_per_instance": round(p_ms / b_ms, 2),
            "batched_gteps": round(edges / (b_ms * 1e-3) / 1e9, 3),
            "per_instance_gteps": round(edges / (p_ms * 1e-3) / 1e9, 3),
            "batched_achieved_gbs": round(alg / (b_ms * 1e-3) / 1e9, 1),
            "batched_frac": round(alg / (b_ms * 1e-3) / 1e9 / peak, 3),
            "launches_batched": int(b_launches), "launches_per_instance": int(p_launches),
            "edges_per_step": int(edges), "alg_bytes_per_step": int(alg), "parity": parity}


def batched_parity(packed, dist, ranks, bres, pres, n_check=64, n_largest=10):
    """Per-graph results of the batched launches against the oracle run on
    each graph alone, for the n_largest largest graphs and graphs spread
    evenly over the rest (n_check in all): BFS levels, processed_nodes and
    iteration bit-exact; PageRank (BATCH_PR_ITERS iterations) within 1e-6
    relative L1 of the FP64 restatement."""
    from oracle import pyoracle as po

    G = packed.num_graphs
    vb = packed.vertex_base.astype(np.int64)
    nv = np.diff(vb)
    largest = [int(x) for x in np.argsort(-nv, kind="stable")[:n_largest]]
    rest = [g for g in np.linspace(0, G - 1, n_check - n_largest).astype(int).tolist() if g not in largest]
    pick = sorted(set(largest + rest))
    bad_bfs, bad_pr, worst = [], [], 0.0
    for g in pick:
        V, off, dest, ioff, isrc = packed.graph(g)
        deg = np.diff(off.astype(np.int64)).astype(np.uint32)
        ideg = np.diff(ioff.astype(np.int64)).astype(np.uint32)
        host = po.HostCSR(V, deg, off[:-1], dest)
        pull = po.HostCSR(V, ideg, ioff[:-1], isrc)
        d, _, proc, it = po.bfs(host, 0, pull)
        b, e = int(vb[g]), int(vb[g + 1])
        if not (np.array_equal(dist[b:e], d) and bres[g].processed_nodes == proc and bres[g].iteration == it):
            bad_bfs.append(g)
        r64, _, _ = po.pagerank(host, BATCH_PR_ITERS, 0.0, pull, fp64=True)
        ok, err, _ = po.fp32_close(ranks[b:e], r64, 1e-6)
        worst = max(worst, err)
        if not ok:
            bad_pr.append(g)
    return {"graphs_checked": len(pick), "largest_checked": n_largest,
            "largest_vertices": int(nv[largest[0]]), "bfs_exact": not bad_bfs, "bfs_mismatched": bad_bfs,
            "pr_worst_rel_l1_vs_fp64": float(f"{worst:.3e}"), "pr_within_1e-6": not bad_pr,
            "pr_mismatched": bad_pr}


def run_multisource(args, torch, gbx, _lib, dg, W, dev, stream, peak, dist=None, rank=0, world=1):
    """256-source BFS on the RMAT-22 graph: one gbx_bfs_multisource call
    (bitmask sweep) against 256 gbx_bfs calls, same sources (seeded,
    non-isolated), device outputs. Mean CUDA-event time of `steps` calls.
    With several ranks each takes a contiguous share of the sources."""
    V = W["V"]
    g = W["g"]
    rng = np.random.default_rng(SEED + 5)
    nz = np.nonzero(g.out_degree)[0]
    src = rng.choice(nz, MS_SOURCES, replace=False).astype(np.uint32)
    lo, hi = shard(MS_SOURCES, rank, world)
    src = src[lo:hi]
    n_src = int(src.shape[0])
    sp = stream.cuda_stream
    src_d = torch.from_numpy(src.view(np.int32)).to(dev)
    dist_d = torch.empty((V, n_src), dtype=torch.int32, device=dev)
    d1 = torch.empty(V, dtype=torch.int32, device=dev)
    res = (_lib.BfsResult * n_src)()
    r1 = _lib.BfsResult()

    def multi():
        _lib.call("gbx_bfs_multisource", dg.handle, n_src, src_d.data_ptr(), dist_d.data_ptr(), res, sp)

    def singles():
        for s in src:
            _lib.call("gbx_bfs", dg.handle, int(s), 2, d1.data_ptr(), None, _lib.C.byref(r1), sp)

    def timed(fn, n):
        out = []
        for _ in range(n):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            out.append(a.elapsed_time(b))
        return float(np.mean(out))

    timed(multi, 1)
    m_ms = timed(multi, max(1, args.steps))
    timed(singles, 1)
    s_ms = timed(singles, max(1, min(args.steps, 2)))
    edges = sum(int(r.edges_traversed) for r in res)
    levels = int(res[0].top_down_steps + res[0].bottom_up_steps)
    parity = None
    if not args.no_parity:
        from oracle import pyoracle as po

        multi()
        torch.cuda.synchronize()
        host = po.HostCSR(V, g.out_degree, g.edges_idx, g.dest)
        pull = po.HostCSR(V, g.inverse_out_degree, g.inverse_edges_idx, g.inverse_dest)
        bad = []
        cols = list(range(0, n_src, max(1, n_src // 8)))
        for k in cols:
            d, _, proc, it = po.bfs(host, int(src[k]), pull)
            col = dist_d[:, k].cpu().numpy().view(np.uint32)
            if not (np.array_equal(col, d) and res[k].processed_nodes == proc and res[k].iteration == it):
                bad.append(k)
        parity = {"sources_checked": len(cols), "exact": not bad, "mismatched": bad}
    del dist_d
    dev_r = dev if dist else None
    m_job, e_job = job_reduce(dist, m_ms, edges, dev_r)
    return {"workload": f"rmat{args.scale}_bfs_{MS_SOURCES}_sources", "sources": n_src,
            "rank_sources": [int(lo), int(hi)], "job_multisource_ms": round(m_job, 3),
            "job_multisource_gteps": round(e_job / (m_job * 1e-3) / 1e9, 3),
            "multisource_ms": round(m_ms, 3), "per_source_ms": round(s_ms, 3),
            "speedup_vs_per_source": round(s_ms / m_ms, 2),
            "multisource_gteps": round(edges / (m_ms * 1e-3) / 1e9, 3),
            "per_source_gteps": round(edges / (s_ms * 1e-3) / 1e9, 3),
            "levels": levels, "push_levels": int(res[0].top_down_steps), "pull_levels": int(res[0].bottom_up_steps),
            "edges_traversed": edges, "parity": parity}


def run_c5(args, torch, gbx, _lib, dev, stream, peak):
    """The scale-up configuration (opt-in, --c5): a Chung-Lu graph of 4e7
    vertices, mean out-degree 30 (1.2e9 edges, kept as generated), out-degree
    power-law exponent 2.1, 70% of edges inside 4,096-id windows, generated
    and built on the GPU. Timed with CUDA events: BFS from 4 seeded roots,
    pull PageRank to epsilon 1e-6, Afforest CC on the symmetrised graph
    (2.4e9 edges), one degree reordering of the edge list."""
    import ctypes as C

    sp = stream.cuda_stream
    V, E = C5_V, C5_V * C5_MEAN
    i32 = dict(dtype=torch.int32, device=dev)
    t0 = time.time()
    src = torch.empty(E, **i32)
    dst = torch.empty(E, **i32)
    gbx.generate_chung_lu(V, E, 2.1, 4096, 0.7, SEED, src=src, dst=dst, stream=sp)

    def build(a, b, symmetric=False):
        n = E * (2 if symmetric else 1)
        deg, idx = torch.empty(V, **i32), torch.empty(V, **i32)
        so, do = torch.empty(n, **i32), torch.empty(n, **i32)
        got = _lib.u32(0)
        _lib.call("gbx_csr_build", E, a.data_ptr(), b.data_ptr(), None, int(symmetric), 0, 0, V, deg.data_ptr(),
                  idx.data_ptr(), so.data_ptr(), do.data_ptr(), None, C.byref(got), sp)
        return deg, idx, so, do

    def create(deg, idx, dest, ideg=None, iidx=None, isrc=None, n=E):
        h = C.c_void_p()
        p = lambda t: None if t is None else t.data_ptr()  # noqa: E731
        _lib.call("gbx_graph_create_csr", C.byref(h), V, n, p(idx), p(deg), p(dest), None, p(iidx), p(ideg),
                  p(isrc), None, sp)
        return gbx.DeviceGraph(h.value, V, n)

    deg, idx, so, do = build(src, dst)
    ideg, iidx, _, ido = build(do, so)  # in-edges: sorted by destination, sources in the "dst" slot
    del so
    dg = create(deg, idx, do, ideg, iidx, ido)
    del do, ido, ideg, iidx
    torch.cuda.empty_cache()
    degs = deg.cpu().numpy()
    rng = np.random.default_rng(SEED)
    roots = [int(r) for r in rng.choice(np.nonzero(degs)[0], 4, replace=False)]
    log(f"c5 built in {time.time() - t0:.1f}s: V={V} E={E}")

    def ev(fn):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        out = fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b), out

    res = {}
    dist_d = torch.empty(V, **i32)
    par_d = torch.empty(V, **i32)
    gbx.breadth_first_search(dg, roots[0], 2, distances=dist_d, parents=par_d, stream=sp, map_source=False)
    ms, te = 0.0, 0
    for r in roots:
        t, st = ev(lambda: gbx.breadth_first_search(dg, r, 2, distances=dist_d, parents=par_d, stream=sp,
                                                    map_source=False))
        ms += t
        te += st.edges_traversed
    res["bfs"] = {"ms_per_root": round(ms / len(roots), 3), "gteps": round(te / (ms * 1e-3) / 1e9, 3),
                  "frac": round((len(roots) * (4 * (V + 1) + 8 * V) + 4 * te) / (ms * 1e-3) / 1e9 / peak, 3)}
    res["bfs"]["certificate"] = bfs_certificate(torch, src, dst, dist_d, par_d, roots[-1])
    ranks = torch.empty(V, dtype=torch.float32, device=dev)
    t, pr = ev(lambda: gbx.page_rank(dg, 1000, 1e-6, ranks=ranks, stream=sp))
    it = pr.iterations + 1 if pr.iterations < 1000 else 1000
    res["pr"] = {"ms": round(t, 3), "iterations": pr.iterations, "gteps": round(E * it / (t * 1e-3) / 1e9, 3),
                 "frac": round(it * (8 * E + 20 * V) / (t * 1e-3) / 1e9 / peak, 3), "epsilon": 1e-6}
    # the error against the same recurrence in FP64 on the GPU, run for the
    # iterations the FP32 solve executed (untimed)
    r64 = torch.empty(V, dtype=torch.float64, device=dev)
    t0 = time.time()
    _lib.call("gbx_pagerank_pull_fp64", dg.handle, it, r64.data_ptr(), sp)
    torch.cuda.synchronize()
    err = float(((ranks.double() - r64).abs().sum() / r64.abs().sum()).item())
    res["pr"]["rel_l1_vs_fp64_gpu"] = float(f"{err:.3e}")
    res["pr"]["within_1e-6"] = bool(err <= 1e-6)
    log(f"c5 FP64 PageRank ({it} iterations) in {time.time() - t0:.1f}s: rel L1 {err:.3e}")
    del r64
    dg.close()
    del dist_d, par_d, ranks
    # symmetrised graph for CC
    sdeg, sidx, sso, sdo = build(src, dst, symmetric=True)
    del sso
    torch.cuda.empty_cache()
    dgs = create(sdeg, sidx, sdo, n=2 * E)
    del sdo
    comp = torch.empty(V, **i32)
    gbx.connected_components(dgs, 1, components=comp, stream=sp)
    t, (c_out, sweeps) = ev(lambda: gbx.connected_components(dgs, 1, components=comp, stream=sp))
    res["cc"] = {"ms": round(t, 3), "gteps": round(2 * E / (t * 1e-3) / 1e9, 3), "num_edges": 2 * E,
                 "components": int(torch.unique(comp).numel())}
    dgs.close()
    del comp
    torch.cuda.empty_cache()
    lab, inv = torch.arange(V, **i32), torch.arange(V, **i32)
    t, _ = ev(lambda: _lib.call("gbx_degree_reorder", V, E, src.data_ptr(), dst.data_ptr(), 1, lab.data_ptr(),
                                inv.data_ptr(), sp))
    res["reorder"] = {"ms": round(t, 3), "gteps": round(E / (t * 1e-3) / 1e9, 3),
                      "frac": round((20 * E + 24 * V) / (t * 1e-3) / 1e9 / peak, 3)}
    del src, dst, lab, inv
    torch.cuda.empty_cache()
    return {"workload": "chung_lu_40M_1.2B", "num_vertices": V, "num_edges": E, "exponent": 2.1, "window": 4096,
            "local_fraction": 0.7, "offsets": "uint32 inside the library (E and 2E below 2^32)", "kernels": res}


def bfs_certificate(torch, src, dst, level, parent, root, chunk=1 << 28):
    """Size-independent checks of one BFS result (levels 0 for the root and
    for unreached vertices, the reference's convention) on the edge list it
    ran on, Graph500-style: every out-edge of a reached vertex reaches a
    vertex at most one level deeper, and every reached vertex but the root
    has a reached parent exactly one level up."""
    V = level.shape[0]
    lv = level.long()
    reached = lv > 0
    reached[root] = True
    ok_edges = True
    for b in range(0, src.shape[0], chunk):
        a = src[b:b + chunk].long()
        d = dst[b:b + chunk].long()
        ra = reached[a]
        ok_edges &= bool((~ra | reached[d]).all().item())
        ok_edges &= bool((~ra | (lv[d] <= lv[a] + 1)).all().item())
    idx = torch.nonzero(reached).flatten()
    idx = idx[idx != root]
    p = parent[idx].long()
    ok_par = bool((p >= 0).all().item())
    if ok_par:
        ok_par = bool((reached[p] & (lv[p] + 1 == lv[idx])).all().item())
    return {"root": int(root), "reached": int(idx.numel()) + 1, "edges_consistent": ok_edges,
            "parents_one_level_up": ok_par, "valid": ok_edges and ok_par}


def run_e2e(gbx, _lib, W, args, roots, sssp_roots, e_plus, tuning=None):
    """Same kernel set through the C ABI with pinned host buffers: upload of
    the CSRs and copy-back of every result inside the timed region. Each step
    creates fresh device graphs (their plans are rebuilt inside the timed
    region) and gives the directed one the knobs the untimed autotuning chose."""
    tuning = tuning or {}
    import torch

    g, gs, gsr = W["g"], W["gs"], W["gsr"]
    V, E = g.num_vertices, g.num_edges

    def pinned(a):
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        return t.numpy()

    hg = gbx.GraphCSR(V, E, pinned(g.out_degree), pinned(g.edges_idx), pinned(g.dest), pinned(g.src),
                      pinned(g.weight), g.label_array, g.inverse_label_array, pinned(g.inverse_out_degree),
                      pinned(g.inverse_edges_idx), pinned(g.inverse_dest), pinned(g.inverse_weight))
    hgs = gbx.GraphCSR(V, gs.num_edges, pinned(gs.out_degree), pinned(gs.edges_idx), pinned(gs.dest),
                       pinned(gs.src), None, gs.label_array, gs.inverse_label_array)
    hgr = gbx.GraphCSR(V, gsr.num_edges, pinned(gsr.out_degree), pinned(gsr.edges_idx), pinned(gsr.dest),
                       pinned(gsr.src), None, gsr.label_array, gsr.inverse_label_array)
    dist_h = pinned(np.zeros(V, np.uint32))
    par_h = pinned(np.zeros(V, np.int32))
    comp_h = pinned(np.zeros(V, np.uint32))
    ranks_h = pinned(np.zeros(V, np.float32))
    y_h = pinned(np.zeros(V, np.float32))
    x_h = pinned(W["x"])
    vals_h = pinned(W["vals"])
    # the degree reordering relabels its pinned edge list in place every step;
    # relabelling keeps the degree sequence, so every step does the same work
    el_h = gbx.EdgeList(V, pinned(g.src), pinned(g.dest), None, pinned(np.arange(V, dtype=np.uint32)),
                        pinned(np.arange(V, dtype=np.uint32)))
    h2d = d2h = 0

    # Every stream of the step is a non-blocking one: on the legacy default
    # stream the directed graph's copies would wait for the triangle count
    # running on another stream (measured: 5.7 ms per step).
    main = torch.cuda.Stream()  # the directed graph, its kernels, then CC
    sp = main.cuda_stream
    side = torch.cuda.Stream()  # the DAG's upload and its triangle count
    side2 = torch.cuda.Stream()  # the degree reordering
    side3 = torch.cuda.Stream()  # the symmetric graph's upload (CC)
    side4 = torch.cuda.Stream()  # the SpMV values' upload
    vals_t = torch.from_numpy(vals_h)
    vals_d = torch.empty(vals_h.shape[0], dtype=torch.float32, device=f"cuda:{torch.cuda.current_device()}")
    seen = {}  # the last step's triangle count

    def step():
        nonlocal h2d, d2h
        edges = 0
        h2d = d2h = 0
        # The SMs have nothing to do while the directed graph goes up, so a
        # second host thread uploads the degree-ordered DAG first and counts
        # its triangles (plan included) on a second stream during the other
        # uploads; a third uploads the symmetric graph (CC) once the DAG is
        # up; a fourth runs the degree reordering of the host edge list
        # during SSSP, SpMV and PageRank, when the host link is otherwise
        # idle. The C ABI releases the GIL. A persistent kernel queued behind
        # a running count only starts later: the count waits on nothing.
        later = {}
        dag_up = threading.Event()

        def side_tc():
            try:
                later["gsr"] = gbx.DeviceGraph.from_graph_csr(hgr, use_weights=False, stream=side.cuda_stream)
                dag_up.set()
                later["tc"] = gbx.triangle_count(later["gsr"], stream=side.cuda_stream)
            except Exception as e:  # re-raised by the step below
                later["error"] = e
            finally:
                dag_up.set()

        def side_cc_upload():
            try:
                later["gs"] = gbx.DeviceGraph.from_graph_csr(hgs, use_weights=False, stream=side3.cuda_stream)
            except Exception as e:
                later["error"] = e

        def side_reorder():
            try:
                gbx.degree_reorder(el_h, 1, stream=side2.cuda_stream)
            except Exception as e:
                later["error"] = e

        ta = threading.Thread(target=side_tc)
        ta.start()
        dag_up.wait()
        tb = threading.Thread(target=side_cc_upload)
        tb.start()
        dg = gbx.DeviceGraph.from_graph_csr(hg, stream=sp)
        dg.label_array = None
        for k, v in tuning.items():  # knobs the autotuner chose for this graph
            dg.set_tuning(k, v)
        # the SpMV values go up while BFS results come down (the link's
        # host-to-device direction is idle from here on)
        with torch.cuda.stream(side4):
            vals_d.copy_(vals_t, non_blocking=True)
            vals_up = torch.cuda.Event()
            vals_up.record(side4)
        h2d += sum(a.nbytes for a in (hg.out_degree, hg.edges_idx, hg.dest, hg.weight, hg.inverse_out_degree,
                                      hg.inverse_edges_idx, hg.inverse_dest, hg.inverse_weight))
        # the trial loop with host outputs: each root's levels and parents
        # come back to pinned host memory while the next root traverses
        for st in gbx.breadth_first_search_trials(dg, roots, 2, distances=dist_h, parents=par_h, stream=sp):
            edges += st.edges_traversed
            d2h += 8 * V
        tr = threading.Thread(target=side_reorder)
        tr.start()
        for r in sssp_roots:
            st = gbx.sssp(dg, r, 0, distances=dist_h, stream=sp)
            edges += st.edges_traversed
            d2h += 4 * V
        y_h[:] = 0
        main.wait_event(vals_up)
        gbx.spmv(dg, x_h, values=vals_d, iterations=1, y=y_h, stream=sp)
        h2d += x_h.nbytes + vals_h.nbytes + y_h.nbytes
        d2h += y_h.nbytes
        edges += E
        gbx.page_rank(dg, PR_ITERS, 0.0, ranks=ranks_h, stream=sp)
        d2h += 4 * V
        edges += E * PR_ITERS
        tb.join()
        if "error" in later:
            raise later["error"]
        dgs = later["gs"]
        h2d += hgs.out_degree.nbytes + hgs.edges_idx.nbytes + hgs.dest.nbytes
        gbx.connected_components(dgs, 1, components=comp_h, stream=sp)
        d2h += 4 * V
        edges += gs.num_edges
        ta.join()
        tr.join()
        # graph destruction synchronises the device: after every call is enqueued
        for h in (dg, dgs, later.get("gsr")):
            if h is not None:
                h.close()
        if "error" in later:
            raise later["error"]
        h2d += hgr.out_degree.nbytes + hgr.edges_idx.nbytes + hgr.dest.nbytes
        d2h += 8
        edges += e_plus
        seen["tc"] = later["tc"]
        h2d += 8 * E + 8 * V  # the degree reordering's edge list, up and back
        d2h += 8 * E + 8 * V
        edges += E
        return edges

    for _ in range(max(3, args.warmup)):  # at least 3 untimed steps, as for the kernel set
        step()
    torch.cuda.synchronize()
    times = []
    edges = 0
    with collector_held():
        for _ in range(max(1, min(args.steps, 5))):
            t0 = time.perf_counter()
            edges = step()
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
    t = float(np.mean(times))
    return {"value": round(edges / t / 1e9, 3), "unit": "GTEPS", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "ms_per_step": round(t * 1e3, 2),
            "step_ms": [round(x * 1e3, 2) for x in times], "tc_count": int(seen["tc"]),
            "path": "C ABI (gbx_graph_create_csr + per-kernel entry points, BFS through gbx_bfs_trials), pinned "
                    "host buffers, non-blocking streams; the TC graph goes up first and is counted on a second "
                    "stream while the directed and CC graphs go up, the SpMV values go up during BFS, the degree "
                    "reordering runs on a third stream during SSSP, SpMV and PageRank"}


# ---------------------------------------------------------------------------
# CPU oracle port (baseline and reference arm)

# The reference arm runs the kernel set in a cycle of CPU_CYCLE steps; one
# cycle holds exactly one full kernel-set step: step i runs BFS from roots
# [16 i, 16 i + 16), SSSP from root i, the triangles of the i-th quarter of
# the pivots (by work), 5 PageRank iterations, and CC (i = 0), SpMV (i = 1)
# or the degree reordering (i = 2).
CPU_CYCLE = 4


def cpu_info():
    model = ""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        model = next((ln.split(":", 1)[1].strip() for ln in out.splitlines() if ln.startswith("Model name")), "")
    except Exception:
        pass
    if not model:
        try:
            txt = Path("/proc/cpuinfo").read_text()
            model = next((ln.split(":", 1)[1].strip() for ln in txt.splitlines()
                          if ln.lower().startswith(("model name", "cpu part"))), "")
        except Exception:
            pass
    return {"cpu_model": model or "unknown", "nproc": os.cpu_count(),
            "omp_proc_bind": os.environ.get("OMP_PROC_BIND", "unset"),
            "omp_places": os.environ.get("OMP_PLACES", "unset")}


def cpu_plan(Wc):
    """Host views of the oracle-built graphs and the cycle's TC pivot slices
    (equal shares of sum over DAG edges (u,v) of d+(v), the pull count's work)."""
    from oracle import pyoracle as po

    g, gs, gsr = Wc["g"], Wc["gs"], Wc["gsr"]
    V = g.num_vertices
    host = po.HostCSR(V, g.out_degree, g.edges_idx, g.dest, g.weight, g.src)
    pull = po.HostCSR(V, g.inverse_out_degree, g.inverse_edges_idx, g.inverse_dest, g.inverse_weight)
    hs = po.HostCSR(V, gs.out_degree, gs.edges_idx, gs.dest)
    hr = po.HostCSR(V, gsr.out_degree, gsr.edges_idx, gsr.dest)
    src = np.repeat(np.arange(V, dtype=np.int64), gsr.out_degree.astype(np.int64))
    dst = gsr.dest.astype(np.int64)
    lower = dst <= src
    dplus = np.bincount(src[lower], minlength=V)
    cost = np.cumsum(np.bincount(src[lower], weights=dplus[dst[lower]], minlength=V))
    cuts = [0] + [int(np.searchsorted(cost, cost[-1] * k / CPU_CYCLE)) for k in range(1, CPU_CYCLE)] + [V]
    dag_per_pivot = np.cumsum(np.bincount(src[lower], minlength=V))
    dag_edges = [int((dag_per_pivot[hi - 1] if hi else 0) - (dag_per_pivot[lo - 1] if lo else 0))
                 for lo, hi in zip(cuts[:-1], cuts[1:])]
    return dict(host=host, pull=pull, hs=hs, hr=hr, tc_cuts=cuts, tc_dag_edges=dag_edges)


def cpu_step(Wc, plan, i, threads=0):
    """Step i of the cycle on the host cores (oracle/gbx_oracle.c, OpenMP).
    Returns ({kernel: (traversed edges, seconds)}, tc count of the slice);
    only the oracle calls are timed."""
    from oracle import pyoracle as po

    g = Wc["g"]
    V, E = g.num_vertices, g.num_edges
    host, pull, hs, hr = plan["host"], plan["pull"], plan["hs"], plan["hr"]
    i %= CPU_CYCLE
    per = N_ROOTS // CPU_CYCLE
    deg = g.out_degree.astype(np.int64)
    res = {}
    t = e = 0.0
    for r in Wc["roots"][per * i:per * (i + 1)]:
        t0 = time.perf_counter()
        d, _, _, _ = po.bfs(host, r, pull, threads)
        t += time.perf_counter() - t0
        reached = d > 0
        reached[r] = True
        e += int(deg[reached].sum())
    res["bfs"] = (e, t)
    r = Wc["roots"][i % N_SSSP_ROOTS]
    t0 = time.perf_counter()
    d = po.sssp(host, r, 64, threads)
    res["sssp"] = (int(deg[d != 0x7FFFFFFF].sum()), time.perf_counter() - t0)
    lo, hi = plan["tc_cuts"][i], plan["tc_cuts"][i + 1]
    t0 = time.perf_counter()
    tri = po.triangle_count(hr, threads, lo, hi)
    res["tc"] = (plan["tc_dag_edges"][i], time.perf_counter() - t0)
    t0 = time.perf_counter()
    po.pagerank(host, PR_ITERS // CPU_CYCLE, 0.0, pull, threads)
    res["pr"] = (E * (PR_ITERS // CPU_CYCLE), time.perf_counter() - t0)
    if i == 0:
        t0 = time.perf_counter()
        po.cc(hs, 1, None, threads)
        res["cc"] = (Wc["gs"].num_edges, time.perf_counter() - t0)
    elif i == 1:
        t0 = time.perf_counter()
        po.spmv(host, Wc["x"], Wc["vals"], pull=pull, threads=threads)
        res["spmv"] = (E, time.perf_counter() - t0)
    elif i == 2:
        t0 = time.perf_counter()
        po.degree_reorder(V, g.src, g.dest, 1, threads=threads)
        res["reorder"] = (E, time.perf_counter() - t0)
    return res, tri


def cpu_baseline(Wc):
    """One full cycle (one kernel-set step) on the host cores, all threads."""
    plan = cpu_plan(Wc)
    per = {}
    tri = 0
    for i in range(CPU_CYCLE):
        res, t = cpu_step(Wc, plan, i)
        tri += t
        for k, (e, s) in res.items():
            pe, ps = per.get(k, (0, 0.0))
            per[k] = (pe + e, ps + s)
    edges = sum(e for e, _ in per.values())
    secs = sum(s for _, s in per.values())
    out = {"value": round(edges / secs / 1e9, 4), "unit": "GTEPS", "cores": os.cpu_count(), "kind": "port",
           "sample": "one full kernel-set step on the RMAT-22 graph built on the host cores by the oracle, "
                     "run as four quarter steps (oracle/gbx_oracle.c, OpenMP, all host threads): BFS from the "
                     "64 roots, SSSP from 4 (delta 64), TC, 20 PR iterations, CC, SpMV, degree reorder",
           "seconds": round(secs, 2), "per_kernel_gteps": {k: round(e / s / 1e9, 4) for k, (e, s) in per.items()},
           **cpu_info()}
    return out, tri


def parity_kernel_set(torch, gbx, W, Wc, dg, dgs, dgr, tri_oracle, stream):
    """The GPU results of the kernel set on the RMAT-22 graph against the
    oracle on the same inputs (outside every timed region): the CSR builds
    and the degree reordering array for array; BFS levels, processed_nodes
    and iteration for all 64 roots; SSSP distances for the 4 roots; CC
    labels; the triangle count -- all bit-exact; PageRank (20 iterations)
    and SpMV as relative L1 against the FP64 restatement (tolerance 1e-6)."""
    from oracle import pyoracle as po

    sp = stream.cuda_stream
    g, gc = W["g"], Wc["g"]
    V = g.num_vertices
    out = {}
    fields = {"g": ("out_degree", "edges_idx", "dest", "weight", "inverse_out_degree", "inverse_edges_idx",
                    "inverse_dest", "inverse_weight"),
              "gs": ("out_degree", "edges_idx", "dest"), "gsr": ("out_degree", "edges_idx", "dest")}

    def same(a, b):
        if a is None or b is None:
            return a is None and b is None
        return a.shape == b.shape and np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))

    out["csr_build"] = all(same(getattr(W[k], f), getattr(Wc[k], f)) for k, fs in fields.items() for f in fs)
    out["degree_reorder_build"] = (same(W["reorder_labels"][0], Wc["reorder_labels"][0])
                                   and same(W["reorder_labels"][1], Wc["reorder_labels"][1]))
    host = po.HostCSR(V, gc.out_degree, gc.edges_idx, gc.dest, gc.weight, gc.src)
    pull = po.HostCSR(V, gc.inverse_out_degree, gc.inverse_edges_idx, gc.inverse_dest, gc.inverse_weight)
    dh = np.zeros(V, np.uint32)
    ph = np.zeros(V, np.int32)
    bad = []
    for r in W["roots"]:
        st = gbx.breadth_first_search(dg, r, 2, distances=dh, parents=ph, stream=sp)
        d, _, proc, it = po.bfs(host, r, pull)
        if not (np.array_equal(dh, d) and st.processed_nodes == proc and st.iteration == it):
            bad.append(int(r))
    out["bfs"] = {"roots": len(W["roots"]), "exact": not bad, "mismatched_roots": bad}
    bad = []
    for r in W["roots"][:N_SSSP_ROOTS]:
        gbx.sssp(dg, r, 0, distances=dh, stream=sp)
        if not np.array_equal(dh, po.sssp(host, r, 64)):
            bad.append(int(r))
    out["sssp"] = {"roots": N_SSSP_ROOTS, "exact": not bad, "mismatched_roots": bad}
    comp, _ = gbx.connected_components(dgs, 1, components=np.zeros(V, np.uint32), stream=sp)
    out["cc"] = bool(np.array_equal(np.asarray(comp), po.cc(po.HostCSR(V, Wc["gs"].out_degree, Wc["gs"].edges_idx,
                                                                         Wc["gs"].dest), 1)))
    # twice: a graph's first count searches the rows for the prefix lengths,
    # later counts read them from its plan (the timed steps used those)
    tri = gbx.triangle_count(dgr, stream=sp)
    tri2 = gbx.triangle_count(dgr, stream=sp)
    out["tc"] = {"count": int(tri), "oracle": int(tri_oracle),
                 "exact": int(tri) == int(tri_oracle) and int(tri2) == int(tri_oracle)}
    lab = np.arange(V, dtype=np.uint32)
    inv = np.arange(V, dtype=np.uint32)
    el = gbx.EdgeList(V, g.src.copy(), g.dest.copy(), None, lab, inv)
    gbx.degree_reorder(el, 1, stream=sp)
    rs, rd, olab, oinv = po.degree_reorder(V, gc.src, gc.dest, 1)
    out["reorder"] = bool(same(el.label_array, olab) and same(el.inverse_label_array, oinv)
                          and same(el.src, rs) and same(el.dst, rd))
    pr = np.asarray(gbx.page_rank(dg, PR_ITERS, 0.0, ranks=np.zeros(V, np.float32), stream=sp).pageRanks)
    r64, _, _ = po.pagerank(host, PR_ITERS, 0.0, pull, fp64=True)
    ok, err, sub = po.fp32_close(pr, r64, 1e-6)
    out["pr"] = {"iterations": PR_ITERS, "rel_l1_vs_fp64": float(f"{err:.3e}"), "within_1e-6": bool(ok)}
    y = np.zeros(V, np.float32)
    gbx.spmv(dg, Wc["x"], values=Wc["vals"], iterations=1, y=y, stream=sp)
    y64 = po.spmv(host, Wc["x"], Wc["vals"], pull=pull, fp64=True)
    ok, err, sub = po.fp32_close(y, y64, 1e-6)
    out["spmv"] = {"rel_l1_vs_fp64": float(f"{err:.3e}"), "within_1e-6": bool(ok)}
    out["all_exact"] = bool(out["csr_build"] and out["degree_reorder_build"] and out["bfs"]["exact"]
                            and out["sssp"]["exact"] and out["cc"] and out["tc"]["exact"] and out["reorder"]
                            and out["pr"]["within_1e-6"] and out["spmv"]["within_1e-6"])
    return out


def workload_config(args, V, E, Esym, e_plus, world):
    """The `config` both arms print (identical keys and values)."""
    return {"workload": f"rmat{args.scale}_full_kernel_set", "scale": args.scale, "num_vertices": V,
            "edges_generated": V * EDGE_FACTOR, "num_edges": E, "num_edges_symmetric": Esym,
            "dag_edges": e_plus, "bfs_roots": N_ROOTS, "sssp_roots": N_SSSP_ROOTS, "pr_iterations": PR_ITERS,
            "l2": "inputs larger than L2 (0.5 GB CSR); the GPU arm also writes 256 MiB before every kernel",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def run_reference(args):
    """The reference arm: the oracle port of the reference's OpenMP kernels on
    the host cores (all threads) on the same RMAT-22 workload, built on the
    host by the oracle (nothing from the GPU library). Each step is one
    quarter of the kernel set (CPU_CYCLE); value = traversed edges / seconds
    over the timed steps, ms_per_step = their mean wall time."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    Wc = build_workload_oracle(scale=args.scale)
    plan = cpu_plan(Wc)
    for i in range(args.warmup):
        cpu_step(Wc, plan, i)
    edges = secs = 0.0
    walls = []
    for i in range(args.steps):
        t0 = time.perf_counter()
        res, _ = cpu_step(Wc, plan, i)
        walls.append(time.perf_counter() - t0)
        edges += sum(e for e, _ in res.values())
        secs += sum(s for _, s in res.values())
    value = edges / secs / 1e9
    g, gs, gsr = Wc["g"], Wc["gs"], Wc["gsr"]
    e_plus = int(sum(plan["tc_dag_edges"]))
    line = {
        "metric": "GTEPS per kernel (aggregate over the kernel set) & %HBM-peak per kernel",
        "value": round(value, 4), "unit": "GTEPS", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(float(np.mean(walls)) * 1e3, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32 (ids, levels, distances) + f32 (ranks, SpMV)", "data": "synthetic",
        "config": workload_config(args, g.num_vertices, g.num_edges, gs.num_edges, e_plus,
                                  int(os.environ.get("WORLD_SIZE", "1"))),
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 4), "unit": "GTEPS", "cores": os.cpu_count(), "kind": "port",
                         "sample": f"each step a quarter of the kernel set ({CPU_CYCLE} steps = one full step: "
                                   "16 BFS roots, 1 SSSP root (delta 64), a quarter of the TC pivots by work, "
                                   "5 PR iterations, and CC, SpMV or the degree reordering) on the RMAT-22 "
                                   "graph the oracle built on the host cores (oracle/gbx_oracle.c, OpenMP, "
                                   "all threads; the reference tree is not on the GPU host, so its compiled "
                                   "form cannot run there)",
                         "seconds_timed": round(secs, 2), **cpu_info()},
        "e2e": {"value": round(value, 4), "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbx", choices=["gbx", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--scale", type=int, default=SCALE, help="RMAT scale (22 is the benchmark workload)")
    ap.add_argument("--only", default="", help="comma-separated kernel subset (profiling runs)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the full-size checks of the GPU results against the oracle")
    ap.add_argument("--no-ppr", action="store_true", help="skip the personalised PageRank forward/adjoint section")
    ap.add_argument("--no-more", action="store_true",
                    help="skip the betweenness / Bellman-Ford / DFS section")
    ap.add_argument("--no-batched", action="store_true", help="skip the 2,048-graph batched section")
    ap.add_argument("--ppr-scale", type=int, default=PPR_SCALE, help="RMAT scale of the PPR section (20 is the workload)")
    ap.add_argument("--batch-graphs", type=int, default=BATCH_GRAPHS, help="graphs in the batched section (2048)")
    ap.add_argument("--no-c5", action="store_true",
                    help="skip the Chung-Lu 4e7-vertex / 1.2e9-edge scale-up (BFS, PR to 1e-6 with its FP64 error, "
                         "CC, reorder)")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--tuning", default="", help="fixed knobs instead of autotuning, e.g. bfs_alpha=15,sssp_delta=4096")
    ap.add_argument("--traffic", type=float, default=None,
                    help="DRAM bytes per launch of the dominant kernel from an ncu capture")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one process per GPU: re-launch this command under torchrun
        import socket

        with socket.socket() as so:
            so.bind(("127.0.0.1", 0))
            port = so.getsockname()[1]
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
               "--master-addr=127.0.0.1", f"--master-port={port}", str(Path(__file__).resolve()), *sys.argv[1:]]
        sys.exit(subprocess.call(cmd))
    if args.warmup < 3 and args.impl == "gbx":
        log("note: fewer than 3 warm-up steps requested")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
