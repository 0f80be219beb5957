"""Parity at the benchmarked sizes (the size-dependent kernel paths switch on
only there: TC's wide and hybrid tables, BFS/SSSP hub chunks, the pull
engine's heavy-row combines, the batched global slots).

RMAT scale 22 (4,194,304 vertices, 2^26 generated edges, seed 1), built once
on the GPU and once on the host cores by the oracle from the same generator
streams: the CSR builds and the degree reordering array for array; BFS
levels, processed_nodes and iteration from the benchmark's 64 roots; SSSP
distances from 4 of them; CC labels; the triangle count; all bit-exact;
PageRank (20 iterations) and SpMV within 1e-6 relative L1 of the FP64
restatement. The 2,048-graph batch (scale ~U[8,15], edge factor ~U[4,32]):
per-graph BFS and 30-iteration PageRank for the 10 largest graphs and 54
spread over the rest, against the oracle run on each graph alone.
"""
import numpy as np
import pytest

import bench

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rmat22(gbx, cuda_device):
    W = bench.build_workload(gbx)
    Wc = bench.build_workload_oracle()
    return W, Wc


def test_rmat22_kernel_set_matches_oracle(gbx, cuda_device, rmat22):
    import torch

    from oracle import pyoracle as po

    W, Wc = rmat22
    gsr = Wc["gsr"]
    tri = po.triangle_count(po.HostCSR(gsr.num_vertices, gsr.out_degree, gsr.edges_idx, gsr.dest))
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    with gbx.DeviceGraph.from_graph_csr(W["g"], stream=sp) as dg, \
            gbx.DeviceGraph.from_graph_csr(W["gs"], use_weights=False, stream=sp) as dgs, \
            gbx.DeviceGraph.from_graph_csr(W["gsr"], use_weights=False, stream=sp) as dgr:
        for h in (dg, dgs, dgr):
            h.label_array = None  # roots are given in the graph's own ids
        par = bench.parity_kernel_set(torch, gbx, W, Wc, dg, dgs, dgr, tri, stream)
    assert par["csr_build"] and par["degree_reorder_build"], par
    assert par["bfs"]["exact"], par["bfs"]
    assert par["sssp"]["exact"], par["sssp"]
    assert par["cc"] and par["reorder"], par
    assert par["tc"]["exact"], par["tc"]
    assert par["pr"]["within_1e-6"], par["pr"]
    assert par["spmv"]["within_1e-6"], par["spmv"]


def test_batch_of_2048_graphs_matches_oracle(gbx, cuda_device):
    import torch

    gl = gbx.generate_rmat_batch(bench.BATCH_GRAPHS, seed=bench.SEED)
    packed = gbx.pack_graphs(gl)
    del gl
    G = packed.num_graphs
    Vt = int(packed.vertex_base[-1])
    dev = cuda_device
    with gbx.GraphBatch(packed) as batch:
        dist = torch.empty(Vt, dtype=torch.int32, device=dev)
        par_d = torch.empty(Vt, dtype=torch.int32, device=dev)
        ranks = torch.empty(Vt, dtype=torch.float32, device=dev)
        src = torch.zeros(G, dtype=torch.int32, device=dev)
        bres = (gbx._lib.BfsResult * G)()
        pres = (gbx._lib.PrResult * G)()
        sp = torch.cuda.current_stream().cuda_stream
        gbx._lib.call("gbx_bfs_batched", batch.handle, src.data_ptr(), dist.data_ptr(), par_d.data_ptr(), bres, sp)
        gbx._lib.call("gbx_pr_batched", batch.handle, bench.BATCH_PR_ITERS, 0.0, ranks.data_ptr(), pres, sp)
        torch.cuda.synchronize()
        par = bench.batched_parity(packed, dist.cpu().numpy().view(np.uint32), ranks.cpu().numpy(), bres, pres)
    assert par["graphs_checked"] >= 64 and par["largest_vertices"] > 30000, par
    assert par["bfs_exact"], par
    assert par["pr_within_1e-6"], par
