"""CPU tests of what bench.py computes besides the GPU timings: the
committed ncu summaries it quotes beside its roofline, the HBM peak and the
algorithmic byte counts of its rooflines, and the seeded workload it times
(shape, jitter, reproducibility)."""
import numpy as np

import bench


def test_committed_profiles_parse():
    t = bench.traffic_table()
    assert t[("stage_sweep", "gauss1m")] > 0
    l1 = bench.profile_metric("k_sweep", "L1/TEX Cache Throughput")
    dram = bench.profile_metric("k_sweep", "DRAM Throughput")
    assert l1 is not None and 0.0 < l1 <= 1.0
    assert dram is not None and 0.0 < dram <= 1.0
    assert bench.profile_metric("k_sweep", "no such row") is None
    assert bench.profile_metric("no_such_kernel", "DRAM Throughput") is None


def test_peak_and_algorithmic_bytes():
    peak, kind = bench.peaks()
    assert peak > 0 and kind in ("measured", "fallback")
    b = bench.algorithmic_bytes(1 << 20, 5_700_000)
    assert b["total"] == 156 * (1 << 20) + 8 * 5_700_000
    assert b["total"] == sum(v for k, v in b.items() if k != "total")
    assert bench.rb_algorithmic_bytes(10, 80, 5, 3) == 276 * 10 + 96 * 80 + 8 * 5 + 156 * 10 + 8 * 3


def test_workload_inputs():
    n = 1 << 14
    sets, R = bench.make_inputs(0, n, 3)
    assert len(sets) == 3 and np.allclose(R @ R.T, np.eye(3), atol=1e-6)
    mn0, mx0 = sets[0]
    assert mn0.shape == (n, 4) and mn0.dtype == np.float32
    assert np.all(mx0[:, :3] >= mn0[:, :3]) and np.all(mn0[:, 3] == 0) and np.all(mx0[:, 3] == 0)
    # jittered copies move the centres, not the extents
    mn1, mx1 = sets[1]
    assert np.allclose(mx1 - mn1, mx0 - mn0, atol=1e-4)
    assert 0.01 < np.abs((mn1 - mn0)[:, :3]).mean() < 0.1
    # same seed, same scene
    again, _ = bench.make_inputs(0, n, 1)
    assert np.array_equal(again[0][0], mn0)
