"""CSR segments (the reference's csrSegmentsNew, csrSegments.c:157-578).

tests/golden/csr_segments.npz holds the reference's own output (-a 100 of
oracle/ref_driver.cpp, one thread) on the test graphs: the partition --
segment count, degrees, the segment of every destination, per-segment edge
counts and largest ids, the edges grouped by segment -- and the GraphCSR it
builds per segment (radix sort by source, degree reordering), with one vertex
more than the segment's largest id. The CPU tests pin the oracle's
restatement to it; the GPU tests check the library (gbx_csr_segments and the
per-segment preprocessing of graph.csr_segments) against both."""
import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from oracle import pyoracle as po


def _fixture():
    with np.load(GOLDEN / "csr_segments.npz") as z:
        return {k: z[k] for k in z.files}


SEG = _fixture()
CASES = sorted({k.rsplit("_num_segments", 1)[0] for k in SEG if k.endswith("_num_segments")})


def _input(case):
    """(V, src, dst, weight, cache_size) of the edge list the reference
    segmented: the test graph sorted by (source, destination) for the
    directed build, symmetrised and deduplicated for the undirected one."""
    name, variant, cache = case.rsplit("_", 2)
    fx = load_golden(name)
    v = "dw" if variant == "dw" else "u"
    w = fx.get(f"{v}_weight") if v == "dw" else None
    return int(fx[f"{v}_num_vertices"]), fx[f"{v}_src"], fx[f"{v}_dest"], w, int(cache[1:])


def _segment_csrs(case):
    """The per-segment arrays of the fixture, split by segment."""
    nv = SEG[f"{case}_segcsr_num_vertices"]
    ne = SEG[f"{case}_seg_num_edges"]
    ne = ne[ne > 0]
    vo = np.concatenate([[0], np.cumsum(nv, dtype=np.int64)])
    eo = np.concatenate([[0], np.cumsum(ne, dtype=np.int64)])
    out = []
    for i in range(len(nv)):
        out.append({k: SEG[f"{case}_segcsr_{k}"][int(vo[i]):int(vo[i + 1])] for k in ("out_degree", "edges_idx", "label",
                                                                               "inverse_label")})
        out[-1]["dest"] = SEG[f"{case}_segcsr_dest"][int(eo[i]):int(eo[i + 1])]
        out[-1]["num_vertices"] = int(nv[i])
    return out


@pytest.mark.parametrize("case", CASES)
def test_oracle_partition_matches_reference(case):
    V, src, dst, w, cache = _input(case)
    assert po.load().orc_csr_segments_count(V, cache) == int(SEG[f"{case}_num_segments"])
    got = po.csr_segments(V, src, dst, w, cache_size=cache)
    for k, g in (("out_degree", "seg_out_degree"), ("in_degree", "seg_in_degree"),
                 ("vertex_segment_index", "seg_vertex_index"), ("segment_num_edges", "seg_num_edges"),
                 ("segment_max_id", "seg_num_vertices"), ("seg_src", "seg_src"), ("seg_dst", "seg_dst")):
        np.testing.assert_array_equal(got[k], SEG[f"{case}_{g}"], err_msg=k)
    if w is not None and f"{case}_seg_weight" in SEG:
        np.testing.assert_array_equal(got["seg_weight"].view(np.uint32), SEG[f"{case}_seg_weight"].view(np.uint32))


@pytest.mark.parametrize("case", CASES)
def test_oracle_segment_csrs_match_reference(case):
    want = _segment_csrs(case)
    src, dst = SEG[f"{case}_seg_src"], SEG[f"{case}_seg_dst"]
    ne = SEG[f"{case}_seg_num_edges"]
    mx = SEG[f"{case}_seg_num_vertices"]
    pos, i = 0, 0
    for j in range(len(ne)):
        n = int(ne[j])
        if n == 0:
            continue
        Vs = int(mx[j]) + 1
        s1 = po.build_csr(Vs, src[pos:pos + n], dst[pos:pos + n], sort_mode=0)
        rs, rd, lab, inv = po.degree_reorder(Vs, s1.src, s1.dest, 1)
        g = po.build_csr(Vs, rs, rd, sort_mode=0)
        assert want[i]["num_vertices"] == Vs
        np.testing.assert_array_equal(g.out_degree, want[i]["out_degree"])
        np.testing.assert_array_equal(g.edges_idx, want[i]["edges_idx"])
        np.testing.assert_array_equal(g.dest, want[i]["dest"])
        np.testing.assert_array_equal(lab, want[i]["label"])
        np.testing.assert_array_equal(inv, want[i]["inverse_label"])
        pos += n
        i += 1
    assert i == len(want)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_gpu_segments_match_reference(gbx, cuda_device, case):
    V, src, dst, w, cache = _input(case)
    el = gbx.EdgeList(V, src, dst, w)
    cs = gbx.csr_segments(el, cache_size=cache, directed=True, keep_weights=w is not None)
    assert cs.num_segments == int(SEG[f"{case}_num_segments"])
    np.testing.assert_array_equal(cs.out_degree, SEG[f"{case}_seg_out_degree"])
    np.testing.assert_array_equal(cs.in_degree, SEG[f"{case}_seg_in_degree"])
    np.testing.assert_array_equal(cs.vertex_segment_index, SEG[f"{case}_seg_vertex_index"])
    np.testing.assert_array_equal([s.num_edges for s in cs.segments], SEG[f"{case}_seg_num_edges"])
    np.testing.assert_array_equal([s.num_vertices for s in cs.segments], SEG[f"{case}_seg_num_vertices"])
    with_edges = [s for s in cs.segments if s.num_edges]
    np.testing.assert_array_equal(np.concatenate([s.edge_list.src for s in with_edges]), SEG[f"{case}_seg_src"])
    np.testing.assert_array_equal(np.concatenate([s.edge_list.dst for s in with_edges]), SEG[f"{case}_seg_dst"])
    for s, want in zip(with_edges, _segment_csrs(case)):
        g = s.graph
        assert g.num_vertices == want["num_vertices"]
        np.testing.assert_array_equal(g.out_degree, want["out_degree"])
        np.testing.assert_array_equal(g.edges_idx, want["edges_idx"])
        np.testing.assert_array_equal(g.dest, want["dest"])
        np.testing.assert_array_equal(g.label_array, want["label"])
        np.testing.assert_array_equal(g.inverse_label_array, want["inverse_label"])


@pytest.mark.gpu
@pytest.mark.parametrize("cache", [1 << 20, 4096, 512])
def test_gpu_partition_matches_oracle_on_rmat(gbx, cuda_device, cache):
    V = 1 << 16
    s, d = gbx.generate_rmat(16, V * 8, seed=3)
    w = gbx.generate_values(s.shape[0], 1, seed=4)
    cs = gbx.csr_segments(gbx.EdgeList(V, s, d, w), cache_size=cache, build_graphs=False)
    want = po.csr_segments(V, s, d, w, cache_size=cache)
    assert cs.num_segments == want["num_segments"]
    np.testing.assert_array_equal(cs.out_degree, want["out_degree"])
    np.testing.assert_array_equal(cs.in_degree, want["in_degree"])
    np.testing.assert_array_equal(cs.vertex_segment_index, want["vertex_segment_index"])
    np.testing.assert_array_equal([x.num_edges for x in cs.segments], want["segment_num_edges"])
    np.testing.assert_array_equal([x.num_vertices for x in cs.segments], want["segment_max_id"])
    segs = [x for x in cs.segments if x.num_edges]
    np.testing.assert_array_equal(np.concatenate([x.edge_list.src for x in segs]), want["seg_src"])
    np.testing.assert_array_equal(np.concatenate([x.edge_list.dst for x in segs]), want["seg_dst"])
    np.testing.assert_array_equal(np.concatenate([x.edge_list.weight for x in segs]).view(np.uint32),
                                  want["seg_weight"].view(np.uint32))


@pytest.mark.gpu
def test_gpu_segments_reject_bad_ids(gbx, cuda_device):
    with pytest.raises(gbx.GbxError):
        gbx.csr_segments(gbx.EdgeList(4, np.array([0, 1, 9], np.uint32), np.array([1, 2, 3], np.uint32)),
                         build_graphs=False)
