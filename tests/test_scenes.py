"""CPU tests: the seeded synthetic workloads have the shapes, sizes and
value distributions of the benchmark configurations they stand in for
(no dataset is involved), and the same seed gives the same scene."""
import numpy as np

from gsap_gb300 import scenes


def test_uniform_16k_case():
    mn, mx = scenes.aabb_uniform(16384, 3)
    assert mn.shape == (16384, 4) and mn.dtype == np.float32
    c, h = 0.5 * (mn[:, :3] + mx[:, :3]), 0.5 * (mx[:, :3] - mn[:, :3])
    assert c.min() >= 0.0 and c.max() <= 100.0
    assert h.min() >= 0.1 - 1e-6 and h.max() <= 0.5 + 1e-6
    assert abs(c.mean() - 50.0) < 1.0 and abs(h.mean() - 0.3) < 0.01
    assert np.array_equal(scenes.aabb_uniform(16384, 3)[0], mn)


def test_gauss_1m_case_statistics():
    n = 1 << 18  # the 1M case's distribution, at a quarter of its size
    c, h, R = scenes.aabb_gauss_parts(n, seed=4)
    assert np.allclose(R @ R.T, np.eye(3), atol=1e-12) and np.linalg.det(R) > 0
    g = c.astype(np.float64) @ R  # back in the generating frame
    assert np.allclose(g.std(0), [100.0, 20.0, 5.0], rtol=0.01)
    assert np.allclose(g.mean(0), 0.0, atol=0.5)
    assert h.min() >= 0.05 and h.max() <= 2.0
    assert abs(np.log(h).mean() - (-1.0)) < 0.01  # exp(N(-1, 0.5^2)), clipped only far out
    j = scenes.jitter(c, seed=9)
    assert abs((j - c).std() - 0.05) < 0.001


def test_batched_case_sizes_and_offsets():
    sizes = scenes.batched_sizes(4096, seed=7)
    assert sizes.min() >= 64 and sizes.max() <= 65536
    # log-uniform: the log sizes spread evenly over [ln 64, ln 65536]
    ls = np.log(sizes)
    assert abs(ls.mean() - 0.5 * (np.log(64) + np.log(65536))) < 0.1
    mn, mx, off = scenes.batched_aabb(S=16, seed=7, lo=64, hi=2000)
    assert off[0] == 0 and off[-1] == len(mn) and np.all(np.diff(off) > 0)
    assert np.array_equal(np.diff(off), scenes.batched_sizes(16, 7, 64, 2000))
    h = 0.5 * (mx[:, :3] - mn[:, :3])
    assert h.min() >= 0.1 - 1e-5 and h.max() <= 0.5 + 1e-5
    assert np.all(mn[:, 3] == 0) and np.all(mx[:, 3] == 0)


def test_body_aabbs_bound_every_particle(oracle_lib):
    """scenes.body_aabbs (the tuning input of a body broadphase) equals the
    union of the particle spheres that the FP64 oracle places at the same
    pose (after one of its steps), to FP32 rounding."""
    sc = scenes.mixed_scenes(S=3, seed=2, lo=64, hi=256)
    st = scenes.to_f64(sc)
    oracle_lib.rb_step_cfg_f64(st, dict(dt=1.0 / 600.0, k=2e4, eta=50.0, kt=0.1, gravity_y=-9.81,
                                        box_lo=(0.0, 0.0, 0.0), box_hi=(100.0, 100.0, 100.0)))
    moved = dict(sc, pos=st["pos"], quat=st["quat"])
    mn, mx = scenes.body_aabbs(moved)
    p = st["p_pos"]  # particle centres and radii at the stepped pose
    owner = np.repeat(np.arange(len(sc["pos"])), sc["n_part"])
    lo = np.full((len(sc["pos"]), 3), np.inf)
    hi = np.full((len(sc["pos"]), 3), -np.inf)
    np.minimum.at(lo, owner, p[:, :3] - p[:, 3:4])
    np.maximum.at(hi, owner, p[:, :3] + p[:, 3:4])
    assert np.allclose(mn[:, :3], lo, rtol=0, atol=1e-4) and np.allclose(mx[:, :3], hi, rtol=0, atol=1e-4)
