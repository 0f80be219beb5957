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
import json
import os
import subprocess
import sys
import tempfile
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
# kernel, from one `ncu --set full` capture of this workload on a GB300
# (tc, spmv: one launch; pr: one iteration; bfs, sssp: one source).
NCU_TRAFFIC_PER_LAUNCH = {"tc": 14.773e9, "pr": 0.4006e9, "bfs": 0.1761e9, "sssp": 1.427e9, "spmv": 0.6775e9}
W_LO, W_HI = 1, 255
# differentiable personalised PageRank: RMAT-20, 2^24 edges as generated,
# lognormal(0,1) weights, 64 teleport columns of 32 seeds, d 0.85 to 1e-7 L1
PPR_SCALE, PPR_EDGES, PPR_K, PPR_SEEDS, PPR_TOL, PPR_D = 20, 1 << 24, 64, 32, 1e-7, 0.85
# batched: 2,048 RMAT graphs, BFS from 0 plus 30 PageRank iterations each
BATCH_GRAPHS, BATCH_PR_ITERS = 2048, 30
MS_SOURCES = 256  # multi-source bitmask BFS on the RMAT-22 graph
C5_V, C5_MEAN = 40_000_000, 30  # scale-up: Chung-Lu 4e7 vertices, 1.2e9 edges (opt-in, --c5)


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# workload construction (untimed)


def build_workload(gbx, scale=SCALE, ef=EDGE_FACTOR, seed=SEED):
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
    rng = np.random.default_rng(seed)
    nz = np.nonzero(g.out_degree)[0]
    roots = [int(r) for r in rng.choice(nz, N_ROOTS, replace=False)]
    log(f"workload built in {time.time() - t0:.1f}s: V={V} E={g.num_edges} Esym={gs.num_edges}")
    return dict(V=V, g=g, gs=gs, gsr=gsr, x=x, vals=vals, roots=roots, edges_src=g.src, edges_dst=g.dest)


def dag_stats(gsr):
    """|E+| and the TC algorithmic bytes sum over DAG edges of 4(d+u + d+v),
    with d+(u) = number of neighbours with id <= u (ids are degree order)."""
    deg = gsr.out_degree.astype(np.int64)
    src = gsr.src.astype(np.int64)
    dst = gsr.dest.astype(np.int64)
    lower = dst <= src
    dplus = np.bincount(src[lower], minlength=gsr.num_vertices).astype(np.int64)
    e_plus = int(lower.sum())
    tc_bytes = 4 * (gsr.num_vertices + 1) + 4 * e_plus + int((4 * (dplus[src[lower]] + dplus[dst[lower]])).sum())
    return e_plus, tc_bytes


# ---------------------------------------------------------------------------
# clocks


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
    e_plus, tc_bytes = dag_stats(gsr)
    roots = W["roots"]
    sssp_roots = roots[:N_SSSP_ROOTS]
    ident = torch.arange(V, dtype=torch.int32, device=dev)

    def kernels():
        """(name, fn) -> fn returns (traversed edges, algorithmic bytes)"""
        def bfs():
            te = tb = 0
            for r in roots:
                st = gbx.breadth_first_search(dg, r, 2, distances=dist_d, parents=par_d, stream=sp)
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
        batched = run_batched(args, torch, gbx, _lib, dev, stream, peak)
        batched["multisource"] = run_multisource(args, torch, gbx, _lib, dg, W, dev, stream, peak)
    more = None
    if not args.no_more and (not args.only or "more" in args.only.split(",")):
        more = run_more(args, torch, gbx, dg, g, stream, peak)
    c5 = None
    if args.c5:
        dg.close(), dgs.close(), dgr.close()
        torch.cuda.empty_cache()
        c5 = run_c5(args, torch, gbx, _lib, dev, stream, peak)
        dg = gbx.DeviceGraph.from_graph_csr(g, stream=sp)
        dgs = gbx.DeviceGraph.from_graph_csr(gs, use_weights=False, stream=sp)
        dgr = gbx.DeviceGraph.from_graph_csr(gsr, use_weights=False, stream=sp)
    e2e = None if args.no_e2e else run_e2e(gbx, _lib, W, args, roots, sssp_roots, e_plus, stream, sp, tuning)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(W, args, roots)
    dg.close(), dgs.close(), dgr.close()
    line = {
        "metric": "GTEPS per kernel (aggregate over the kernel set) & %HBM-peak per kernel",
        "value": round(gteps, 3), "unit": "GTEPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32 (ids, levels, distances) + f32 (ranks, SpMV)",
        "data": "synthetic",
        "config": {"workload": f"rmat{args.scale}_full_kernel_set", "scale": args.scale, "num_vertices": V,
                   "edges_generated": V * EDGE_FACTOR, "num_edges": E, "num_edges_symmetric": gs.num_edges,
                   "dag_edges": e_plus, "bfs_roots": N_ROOTS, "sssp_roots": N_SSSP_ROOTS,
                   "pr_iterations": PR_ITERS, "l2": "flushed (256 MiB write) before every kernel",
                   "parallelism": "replicas" if world > 1 else "single GPU", "tuning": tuning},
        "kernels": per, "batched": batched, "ppr_adjoint": ppr, "more": more, "c5": c5, "roofline": roof, "e2e": e2e, "cpu_baseline": cpu, "clocks": clk,
        "gpu_launches": int(launches), "wall_ms_timed_region": round(wall_ms, 3),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
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


def run_batched(args, torch, gbx, _lib, dev, stream, peak):
    """2,048 RMAT graphs (scale ~U[8,15], V = floor(2^s), edge factor
    ~U[4,32]) packed back to back: one step = BFS from vertex 0 plus 30
    PageRank iterations on every graph. Batched: gbx_bfs_batched +
    gbx_pr_batched (two persistent launches). Per instance: gbx_bfs +
    gbx_pagerank_pull called once per graph on resident single graphs, the
    same device output arrays. Both timed with CUDA events, mean of `steps`."""
    t0 = time.time()
    gl = gbx.generate_rmat_batch(args.batch_graphs, seed=SEED)
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
    m_reach = sum(int(r.edges_traversed) for r in bres)
    nv = np.diff(vb)
    edges = m_reach + BATCH_PR_ITERS * Et
    alg = (4 * (Vt + G) + 4 * m_reach + 8 * Vt) + BATCH_PR_ITERS * (8 * Et + 4 * (Vt + G) + 16 * Vt)
    for dg in singles:
        dg.close()
    batch.close()
    return {"workload": f"rmat_batch_{G}_graphs", "num_graphs": G, "num_vertices": Vt, "num_edges": Et,
            "graph_vertices_min_max": [int(nv.min()), int(nv.max())], "pr_iterations": BATCH_PR_ITERS,
            "batched_ms": round(b_ms, 3), "per_instance_ms": round(p_ms, 3),
            "speedup_vs_per_instance": round(p_ms / b_ms, 2),
            "batched_gteps": round(edges / (b_ms * 1e-3) / 1e9, 3),
            "per_instance_gteps": round(edges / (p_ms * 1e-3) / 1e9, 3),
            "batched_achieved_gbs": round(alg / (b_ms * 1e-3) / 1e9, 1),
            "batched_frac": round(alg / (b_ms * 1e-3) / 1e9 / peak, 3),
            "launches_batched": int(b_launches), "launches_per_instance": int(p_launches),
            "edges_per_step": int(edges), "alg_bytes_per_step": int(alg)}


def run_multisource(args, torch, gbx, _lib, dg, W, dev, stream, peak):
    """256-source BFS on the RMAT-22 graph: one gbx_bfs_multisource call
    (bitmask sweep) against 256 gbx_bfs calls, same sources (seeded,
    non-isolated), device outputs. Mean CUDA-event time of `steps` calls."""
    V = W["V"]
    g = W["g"]
    rng = np.random.default_rng(SEED + 5)
    nz = np.nonzero(g.out_degree)[0]
    src = rng.choice(nz, MS_SOURCES, replace=False).astype(np.uint32)
    sp = stream.cuda_stream
    src_d = torch.from_numpy(src.view(np.int32)).to(dev)
    dist_d = torch.empty((V, MS_SOURCES), dtype=torch.int32, device=dev)
    d1 = torch.empty(V, dtype=torch.int32, device=dev)
    res = (_lib.BfsResult * MS_SOURCES)()
    r1 = _lib.BfsResult()

    def multi():
        _lib.call("gbx_bfs_multisource", dg.handle, MS_SOURCES, src_d.data_ptr(), dist_d.data_ptr(), res, sp)

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
    del dist_d
    return {"workload": f"rmat{args.scale}_bfs_{MS_SOURCES}_sources", "sources": MS_SOURCES,
            "multisource_ms": round(m_ms, 3), "per_source_ms": round(s_ms, 3),
            "speedup_vs_per_source": round(s_ms / m_ms, 2),
            "multisource_gteps": round(edges / (m_ms * 1e-3) / 1e9, 3),
            "per_source_gteps": round(edges / (s_ms * 1e-3) / 1e9, 3),
            "levels": levels, "push_levels": int(res[0].top_down_steps), "pull_levels": int(res[0].bottom_up_steps),
            "edges_traversed": edges}


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
    ranks = torch.empty(V, dtype=torch.float32, device=dev)
    t, pr = ev(lambda: gbx.page_rank(dg, 1000, 1e-6, ranks=ranks, stream=sp))
    it = pr.iterations + 1
    res["pr"] = {"ms": round(t, 3), "iterations": pr.iterations, "gteps": round(E * it / (t * 1e-3) / 1e9, 3),
                 "frac": round(it * (8 * E + 20 * V) / (t * 1e-3) / 1e9 / peak, 3), "epsilon": 1e-6}
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
            "local_fraction": 0.7, "offsets": "uint32 (E < 2^32)", "kernels": res}


def run_e2e(gbx, _lib, W, args, roots, sssp_roots, e_plus, stream, sp, tuning=None):
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

    def step():
        nonlocal h2d, d2h
        edges = 0
        h2d = d2h = 0
        dg = gbx.DeviceGraph.from_graph_csr(hg, stream=sp)
        dg.label_array = None
        for k, v in tuning.items():  # knobs the autotuner chose for this graph
            dg.set_tuning(k, v)
        h2d += sum(a.nbytes for a in (hg.out_degree, hg.edges_idx, hg.dest, hg.weight, hg.inverse_out_degree,
                                      hg.inverse_edges_idx, hg.inverse_dest, hg.inverse_weight))
        for r in roots:
            st = gbx.breadth_first_search(dg, r, 2, distances=dist_h, parents=par_h, stream=sp)
            edges += st.edges_traversed
            d2h += 8 * V
        for r in sssp_roots:
            st = gbx.sssp(dg, r, 0, distances=dist_h, stream=sp)
            edges += st.edges_traversed
            d2h += 4 * V
        y_h[:] = 0
        gbx.spmv(dg, x_h, values=vals_h, iterations=1, y=y_h, stream=sp)
        h2d += x_h.nbytes + vals_h.nbytes + y_h.nbytes
        d2h += y_h.nbytes
        edges += E
        gbx.page_rank(dg, PR_ITERS, 0.0, ranks=ranks_h, stream=sp)
        d2h += 4 * V
        edges += E * PR_ITERS
        dg.close()
        dgs = gbx.DeviceGraph.from_graph_csr(hgs, use_weights=False, stream=sp)
        h2d += hgs.out_degree.nbytes + hgs.edges_idx.nbytes + hgs.dest.nbytes
        gbx.connected_components(dgs, 1, components=comp_h, stream=sp)
        d2h += 4 * V
        edges += gs.num_edges
        dgs.close()
        dgr = gbx.DeviceGraph.from_graph_csr(hgr, use_weights=False, stream=sp)
        h2d += hgr.out_degree.nbytes + hgr.edges_idx.nbytes + hgr.dest.nbytes
        gbx.triangle_count(dgr, stream=sp)
        d2h += 8
        edges += e_plus
        dgr.close()
        gbx.degree_reorder(el_h, 1, stream=sp)
        h2d += 8 * E + 8 * V
        d2h += 8 * E + 8 * V
        edges += E
        return edges

    for _ in range(max(1, min(args.warmup, 2))):
        step()
    torch.cuda.synchronize()
    times = []
    edges = 0
    for _ in range(max(1, min(args.steps, 3))):
        t0 = time.perf_counter()
        edges = step()
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    t = float(np.mean(times))
    return {"value": round(edges / t / 1e9, 3), "unit": "GTEPS", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "ms_per_step": round(t * 1e3, 2),
            "path": "C ABI (gbx_graph_create_csr + per-kernel entry points), pinned host buffers"}


# ---------------------------------------------------------------------------
# CPU oracle port (baseline and reference arm)


def cpu_sample(W, roots, n_bfs=4, pr_iters=PR_ITERS, n_sssp=1, with_tc=True, threads=0):
    from oracle import pyoracle as po

    g, gs, gsr = W["g"], W["gs"], W["gsr"]
    V = g.num_vertices
    host = po.HostCSR(V, g.out_degree, g.edges_idx, g.dest, g.weight, g.src)
    pull = po.HostCSR(V, g.inverse_out_degree, g.inverse_edges_idx, g.inverse_dest, g.inverse_weight)
    hs = po.HostCSR(V, gs.out_degree, gs.edges_idx, gs.dest)
    hr = po.HostCSR(V, gsr.out_degree, gsr.edges_idx, gsr.dest)
    res = {}

    def timed(name, fn, edges):
        t0 = time.perf_counter()
        fn()
        dt = time.perf_counter() - t0
        res[name] = (edges() if callable(edges) else edges, dt)

    bfs_edges = []

    def bfs():
        for r in roots[:n_bfs]:
            d, _, _, _ = po.bfs(host, r, pull, threads)
            reached = (d > 0)
            reached[r] = True
            bfs_edges.append(int(g.out_degree[reached].astype(np.int64).sum()))

    timed("bfs", bfs, lambda: sum(bfs_edges))
    sssp_edges = []

    def sssp():
        for r in roots[:n_sssp]:
            d = po.sssp(host, r, 64, threads)
            sssp_edges.append(int(g.out_degree[d != 0x7FFFFFFF].astype(np.int64).sum()))

    timed("sssp", sssp, lambda: sum(sssp_edges))
    timed("cc", lambda: po.cc(hs, 1, None, threads), gs.num_edges)
    if with_tc:
        e_plus = int((gsr.dest <= gsr.src).sum())
        timed("tc", lambda: po.triangle_count(hr, threads), e_plus)
    timed("spmv", lambda: po.spmv(host, W["x"], W["vals"], pull=pull, threads=threads), g.num_edges)
    timed("pr", lambda: po.pagerank(host, pr_iters, 0.0, pull, threads), g.num_edges * pr_iters)
    timed("reorder", lambda: po.degree_reorder(V, g.src, g.dest, 1, threads=threads), g.num_edges)
    return res


def step_mix(W, res, n_bfs, n_sssp):
    """Traversed edges of one full kernel-set step (64 BFS roots, 4 SSSP roots,
    CC, TC, SpMV, 20 PR iterations, reorder), BFS/SSSP from the sampled roots'
    mean reach."""
    g, gs, gsr = W["g"], W["gs"], W["gsr"]
    E = g.num_edges
    return {"bfs": res["bfs"][0] / n_bfs * N_ROOTS, "sssp": res["sssp"][0] / n_sssp * N_SSSP_ROOTS,
            "cc": gs.num_edges, "tc": int((gsr.dest <= gsr.src).sum()), "spmv": E, "pr": E * PR_ITERS,
            "reorder": E}


def mix_gteps(res, mix):
    """Aggregate GTEPS of the full step at the sampled per-kernel rates: the
    same kernel mix as the GPU `value`."""
    secs = sum(mix[k] / (e / t) for k, (e, t) in res.items())
    return sum(mix[k] for k in res) / secs / 1e9, secs


def cpu_baseline(W, args, roots):
    res = cpu_sample(W, roots)
    value, secs = mix_gteps(res, step_mix(W, res, 4, 1))
    return {"value": round(value, 4), "unit": "GTEPS", "cores": os.cpu_count(), "kind": "port",
            "sample": "RMAT-22 kernel set on the host cores: BFS 4 roots, SSSP 1 root (delta 64), CC Afforest, "
                      "TC, SpMV, PR 20 iterations, degree reorder (oracle/gbx_oracle.c, OpenMP); value = the "
                      "full step's edges (64 BFS roots, 4 SSSP roots, ...) at the sampled per-kernel rates",
            "seconds_sampled": round(sum(t for _, t in res.values()), 2), "seconds_full_step": round(secs, 2),
            "per_kernel_gteps": {n: round(e / t / 1e9, 4) for n, (e, t) in res.items()}}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import graphblox_gb300 as gbx

    W = build_workload(gbx, scale=args.scale)
    roots = W["roots"]
    values, secs = [], []
    tc_res = None
    for i in range(args.warmup + args.steps):
        # the oracle's triangle count is most of a sample's CPU time (~15 s at
        # RMAT-22): it is timed once, in the first measured step, and its rate
        # is reused for the others, so the run stays within a few minutes for
        # any --steps / --warmup
        timed_tc = i >= args.warmup and tc_res is None
        res = cpu_sample(W, roots[i % len(roots):] + roots, n_bfs=2, pr_iters=5, n_sssp=1, with_tc=timed_tc)
        if timed_tc:
            tc_res = res["tc"]
        if i >= args.warmup:
            res["tc"] = tc_res
            v, s = mix_gteps(res, step_mix(W, res, 2, 1))
            values.append(v)
            secs.append(s)
    value = float(np.mean(values))
    line = {
        "metric": "GTEPS per kernel (aggregate over the kernel set) & %HBM-peak per kernel",
        "value": round(value, 4), "unit": "GTEPS", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(float(np.mean(secs)) * 1e3, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32 (ids, levels, distances) + f32 (ranks, SpMV)", "data": "synthetic",
        "config": {"workload": f"rmat{args.scale}_full_kernel_set", "scale": args.scale, "num_vertices": W["V"],
                   "num_edges": W["g"].num_edges},
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 4), "unit": "GTEPS", "cores": os.cpu_count(), "kind": "port",
                         "sample": "per step: BFS 2 roots, SSSP 1 root (delta 64), CC, SpMV, PR 5 "
                                   "iterations, degree reorder on the RMAT-22 graph, TC timed once in the first "
                                   "measured step (oracle/gbx_oracle.c, OpenMP; "
                                   "the reference tree is not on the GPU host, so its compiled form cannot run); "
                                   "value and ms_per_step = the full step's edges (64 BFS roots, 4 SSSP roots, "
                                   "20 PR iterations, ...) at the sampled per-kernel rates, the GPU value's mix"},
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
    ap.add_argument("--no-ppr", action="store_true", help="skip the personalised PageRank forward/adjoint section")
    ap.add_argument("--no-more", action="store_true",
                    help="skip the betweenness / Bellman-Ford / DFS section")
    ap.add_argument("--no-batched", action="store_true", help="skip the 2,048-graph batched section")
    ap.add_argument("--ppr-scale", type=int, default=PPR_SCALE, help="RMAT scale of the PPR section (20 is the workload)")
    ap.add_argument("--batch-graphs", type=int, default=BATCH_GRAPHS, help="graphs in the batched section (2048)")
    ap.add_argument("--c5", action="store_true",
                    help="also run the Chung-Lu 4e7-vertex / 1.2e9-edge scale-up (BFS, PR to 1e-6, CC, reorder)")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--tuning", default="", help="fixed knobs instead of autotuning, e.g. bfs_alpha=15,sssp_delta=4096")
    ap.add_argument("--traffic", type=float, default=None,
                    help="DRAM bytes per launch of the dominant kernel from an ncu capture")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gbx":
        log("note: fewer than 3 warm-up steps requested")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
