"""The benchmark's inputs built on the host cores without the GPU library
(the reference arm and the full-size parity checks use them): the oracle's
generators reproduce the library's RMAT and value streams bit for bit, and
the oracle-built workload has the shape the GPU build has. No GPU call: the
library's generators are host code."""
import numpy as np
import pytest

import bench
from oracle import pyoracle as po


@pytest.mark.parametrize("scale,edges,seed", [(4, 100, 1), (10, 20000, 3), (16, 1 << 20, 7)])
def test_rmat_streams_match(gbx, scale, edges, seed):
    a = gbx.generate_rmat(scale, edges, seed=seed)
    b = po.generate_rmat(scale, edges, seed=seed)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.parametrize("kind,lo,hi", [(0, 1, 255), (1, 0, 0), (2, 0, 0), (3, 0, 0)])
def test_value_streams_match(gbx, kind, lo, hi):
    a = gbx.generate_values(100_000, kind, lo, hi, seed=5)
    b = po.generate_values(100_000, kind, lo, hi, seed=5)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_oracle_workload_small():
    W = bench.build_workload_oracle(scale=12)
    g, gs, gsr = W["g"], W["gs"], W["gsr"]
    V = 1 << 12
    assert g.num_vertices == V and g.inverse_dest.shape[0] == g.num_edges
    assert gs.num_edges == gsr.num_edges and len(W["roots"]) == bench.N_ROOTS
    assert np.all(g.out_degree[W["roots"]] > 0)
    # the triangle count of the cycle's pivot slices adds up to the whole count
    plan = bench.cpu_plan(W)
    hr = plan["hr"]
    total = po.triangle_count(hr)
    cuts = plan["tc_cuts"]
    assert sum(po.triangle_count(hr, 0, lo, hi) for lo, hi in zip(cuts[:-1], cuts[1:])) == total
    assert sum(plan["tc_dag_edges"]) == bench.tc_stats(gsr)[0]
