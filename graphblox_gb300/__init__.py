"""graphblox_gb300 -- GB300 (sm_103a) backend for GraphBlox's CSR graph kernels.

The compute path is libgbx.so (hand-written CUDA kernels behind the C ABI in
include/gbx.h). This package is the host-side mirror of the reference's
graph-load and algorithm interfaces; see graph.py.
"""
from ._lib import GbxError, load  # noqa: F401
from .graph import (  # noqa: F401
    BellmanFordStats,
    BetweennessCentralityStats,
    BFSStats,
    CSRSegments,
    DFSStats,
    DeviceGraph,
    EdgeList,
    GraphBatch,
    GraphCSR,
    PackedGraphs,
    PageRankStats,
    PPRAdjointStats,
    PPRStats,
    Segment,
    SSSPStats,
    bellman_ford,
    betweenness_centrality,
    bfs_multisource,
    breadth_first_search,
    breadth_first_search_trials,
    connected_components,
    csr_build,
    csr_segments,
    degree_reorder,
    depth_first_search,
    read_label_file,
    reference_roots,
    relabel,
    relabel_from_file,
    generate_chung_lu,
    generate_rmat,
    generate_rmat_batch,
    generate_values,
    mask_graph,
    graph_csr_preprocessing,
    pack_graphs,
    page_rank,
    ppr_adjoint,
    ppr_forward,
    read_edge_list_bin,
    read_graph_csr_bin,
    spmv,
    sssp,
    triangle_count,
    write_edge_list_bin,
    write_graph_csr_bin,
)

__version__ = "0.1.0"
