"""GPU parity of the broadphase: the pair set, as a sorted (i < j) uint32
list, must equal the oracle's bit for bit (the reference's own
Aabb::overlaps golden lists, the O(n^2) brute force, and the CPU
restatement of the reference SaP at full size)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def to_dev(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(cuda)


def run_bp(sap, mn, mx, cuda, sorted=True, graph=False):
    out = sap.broadphase(to_dev(mn, cuda), to_dev(mx, cuda) if mx is not None else None, sorted=sorted,
                         graph=graph)
    p = out.cpu().numpy().astype(np.uint32)
    if not sorted:
        p = p[np.lexsort((p[:, 1], p[:, 0]))]
    return p


@pytest.fixture(scope="module")
def sap(cuda):
    from gsap_gb300 import Sap
    return Sap(1 << 16)


def test_golden_reference_lists(sap, cuda):
    g = np.load(os.path.join(GOLDEN, "aabb_bf_golden.npz"))
    for name in g["names"]:
        mn, mx, want = g[f"{name}__min"], g[f"{name}__max"], g[f"{name}__pairs"]
        got = run_bp(sap, mn, mx, cuda)
        assert np.array_equal(got, want), name
        got = run_bp(sap, mn, mx, cuda, sorted=False)
        assert np.array_equal(got, want), name


@pytest.mark.parametrize("axis_mode", [0, 1])
def test_uniform_16384_twenty_seeds(cuda, oracle_lib, axis_mode):
    from gsap_gb300 import Sap, scenes
    sap = Sap(16384, axis_mode=axis_mode)
    for seed in range(20):
        mn, mx = scenes.aabb_uniform(16384, seed)
        want = oracle_lib.bf_aabb(mn, mx)
        assert np.array_equal(run_bp(sap, mn, mx, cuda), want), seed


@pytest.mark.parametrize("n", [2, 3, 31, 513, 4095, 4097, 9000])
def test_odd_sizes_gauss(sap, cuda, oracle_lib, n):
    from gsap_gb300 import scenes
    c, h, _ = scenes.aabb_gauss_parts(n, seed=n, std=(10.0, 3.0, 1.0))
    mn = np.concatenate([c - h, np.zeros((n, 1), np.float32)], 1)
    mx = np.concatenate([c + h, np.zeros((n, 1), np.float32)], 1)
    assert np.array_equal(run_bp(sap, mn, mx, cuda), oracle_lib.bf_aabb(mn, mx))


def test_sphere_predicate(cuda, oracle_lib):
    from gsap_gb300 import MODE_SPHERE, Sap
    sap = Sap(20000, mode=MODE_SPHERE)
    rng = np.random.default_rng(7)
    for n, box in ((20000, 40.0), (3000, 8.0)):
        s = np.concatenate([rng.uniform(0, box, (n, 3)), rng.uniform(0.1, 0.4, (n, 1))], 1).astype(np.float32)
        # exactly touching and coincident spheres
        s[1] = s[0]
        s[3, :3] = s[2, :3] + np.float32([0.5, 0, 0]); s[2, 3] = 0.25; s[3, 3] = 0.25
        got = run_bp(sap, s, None, cuda)
        assert np.array_equal(got, oracle_lib.bf_sphere(s))


def test_empty_and_single(sap, cuda):
    for n in (0, 1):
        mn = np.zeros((n, 4), np.float32)
        assert len(run_bp(sap, mn, mn + 1, cuda)) == 0


def test_graph_mode_and_repeat_calls(sap, cuda, oracle_lib):
    from gsap_gb300 import scenes
    mn, mx = scenes.aabb_uniform(16384, 5)
    want = oracle_lib.bf_aabb(mn, mx)
    for _ in range(3):
        assert np.array_equal(run_bp(sap, mn, mx, cuda, graph=True), want)
    assert np.array_equal(run_bp(sap, mn, mx, cuda), want)


def test_capacity_error_reports_required_size(sap, cuda):
    import torch
    from gsap_gb300 import GsapError, _lib
    g = np.load(os.path.join(GOLDEN, "aabb_bf_golden.npz"))
    mn, mx = to_dev(g["identical_40__min"], cuda), to_dev(g["identical_40__max"], cuda)
    pairs = torch.empty((100, 2), dtype=torch.int32, device=cuda)
    import ctypes as C
    cnt = C.c_uint64(0)
    st = _lib.load().gsap_broadphase_aabb(sap.handle, mn.data_ptr(), mx.data_ptr(), 40, pairs.data_ptr(), 100,
                                          None, C.byref(cnt), 0, None)
    assert st == 2 and cnt.value == 780
    # the handle still works afterwards
    out = sap.broadphase(mn, mx)
    assert len(out) == 780


def test_allocation_failure_is_reported(cuda, oracle_lib):
    """A handle whose scratch cannot exist (34 TB of pair capacity) is refused
    at create with a CUDA status and a message, and the device stays usable."""
    from gsap_gb300 import GsapError, Sap, scenes
    with pytest.raises(GsapError) as ei:
        Sap(1000, pair_factor=(1 << 32) - 1)
    assert "allocation failed" in str(ei.value)
    mn, mx = scenes.aabb_uniform(4096, 5)
    assert np.array_equal(run_bp(Sap(4096), mn, mx, cuda), oracle_lib.bf_aabb(mn, mx))


def test_nonfinite_input_is_reported(sap, cuda):
    from gsap_gb300 import GsapError
    mn = np.zeros((100, 4), np.float32)
    mx = np.ones((100, 4), np.float32)
    mn[17, 1] = np.nan
    with pytest.raises(GsapError) as e:
        run_bp(sap, mn, mx, cuda)
    assert e.value.status == 5
    mn[17, 1] = 0.0
    assert len(run_bp(sap, mn, mx, cuda)) == 100 * 99 // 2


@pytest.mark.parametrize("sort_bits", [16, 32])
def test_batched_matches_per_scene(cuda, oracle_lib, sort_bits):
    """64 scenes in one batched call equal the per-scene brute force; with
    16-bit keys the scenes share at most 1024 cells (one each here), so every
    scene is swept along u1 alone."""
    import torch
    from gsap_gb300 import Sap, scenes
    mn, mx, off = scenes.batched_aabb(S=64, seed=3, lo=16, hi=3000)
    n = len(mn)
    bsap = Sap(n, max_scenes=64, sort_bits=sort_bits, pair_factor=64)
    got = bsap.broadphase_batched(to_dev(mn, cuda), to_dev(mx, cuda),
                                  torch.from_numpy(off.astype(np.int32)).to(cuda)).cpu().numpy().astype(np.uint32)
    want = []
    for s in range(64):
        a, b = off[s], off[s + 1]
        p = oracle_lib.bf_aabb(mn[a:b], mx[a:b]).astype(np.int64) + a
        want.append(p)
    want = np.concatenate(want).astype(np.uint32)
    assert np.array_equal(got, want)


def test_graph_mode_with_new_buffers_every_call(cuda, oracle_lib):
    """Graph mode where every call brings new input and output buffers:
    once the handle keeps its quota of graphs for the shape (set to 2 here),
    new buffers update a cached graph in place instead of adding one; every
    call's pair list is exact."""
    import ctypes as C

    import torch
    from gsap_gb300 import Sap, _lib, scenes
    L = _lib.load()
    sap = Sap(16384)
    assert L.gsap_debug_graph_cache(sap.handle, 2, None) == 0
    n = 16384
    big_mn = torch.empty((n + 64, 4), dtype=torch.float32, device=cuda)
    big_mx = torch.empty_like(big_mn)
    out = torch.empty((16 * n + 64, 2), dtype=torch.int32, device=cuda)
    for k in range(7):
        mn, mx = scenes.aabb_uniform(n, k)
        a = 3 * k  # a new window of the buffers every call: new pointers, same shape
        big_mn[a:a + n] = to_dev(mn, cuda)
        big_mx[a:a + n] = to_dev(mx, cuda)
        got = sap.broadphase(big_mn[a:a + n], big_mx[a:a + n], pairs=out[5 * k:5 * k + 16 * n], sorted=True,
                            graph=True)
        assert np.array_equal(got.cpu().numpy().astype(np.uint32), oracle_lib.bf_aabb(mn, mx)), k
        cnt = C.c_uint32(0)
        L.gsap_debug_graph_cache(sap.handle, 0, C.byref(cnt))
        assert cnt.value == min(k + 1, 2)


def test_batched_4096_scenes_full_size(cuda, oracle_lib):
    """The batched workload at its own size: 4096 scenes of 64 to 65,536
    AABBs (38.6M objects) in one batched call.  The sorted (i<j) list equals
    the oracle scene by scene (the O(n^2) test for every scene of at most
    8,192 objects, the same predicate on the pairs whose x intervals meet
    for larger ones), and sampled scenes run alone through the plain
    pipeline give the batch's rows for them."""
    import torch
    from gsap_gb300 import Sap, scenes
    mn, mx, off = scenes.batched_aabb(S=4096, seed=7)
    n = len(mn)
    dmn, dmx = to_dev(mn, cuda), to_dev(mx, cuda)
    doff = torch.from_numpy(off.astype(np.int32)).to(cuda)
    bsap = Sap(n, max_scenes=4096, pair_factor=2)
    got = bsap.broadphase_batched(dmn, dmx, doff).cpu().numpy().astype(np.uint32)
    bsap.close()
    want = oracle_lib.pairs_batched(mn, mx, off, bf_max=8192)
    assert len(got) == len(want) and np.array_equal(got, want)
    sizes = off[1:] - off[:-1]
    sample = [int(np.argmax(sizes)), int(np.argmin(sizes))] + list(range(0, 4096, 512))
    psap = Sap(int(sizes.max()))
    lo = np.searchsorted(got[:, 0], off[:-1])
    hi = np.searchsorted(got[:, 0], off[1:])
    for s in sample:
        a, b = int(off[s]), int(off[s + 1])
        alone = run_bp(psap, mn[a:b], mx[a:b], cuda).astype(np.int64) + a
        assert np.array_equal(alone.astype(np.uint32), got[lo[s]:hi[s]]), s


@pytest.mark.parametrize("axis_mode", [0, 1])
def test_gauss_1m_against_cpu_sap(cuda, oracle_lib, axis_mode):
    """Full-size 1,048,576-AABB case: equal to the CPU restatement of the
    reference SaP, plus size-independent properties."""
    from gsap_gb300 import Sap, scenes
    c, h, R = scenes.aabb_gauss_parts(1 << 20, seed=0)
    mn = np.concatenate([c - h, np.zeros((len(c), 1), np.float32)], 1)
    mx = np.concatenate([c + h, np.zeros((len(c), 1), np.float32)], 1)
    sap = Sap(1 << 20, axis_mode=axis_mode)
    got = run_bp(sap, mn, mx, cuda)
    # sorted, unique, i < j
    assert np.all(got[:, 0] < got[:, 1])
    key = got[:, 0].astype(np.uint64) << np.uint64(32) | got[:, 1].astype(np.uint64)
    assert np.all(np.diff(key.astype(np.int64)) > 0)
    # every pair overlaps
    a, b = got[:, 0], got[:, 1]
    assert np.all((mn[a, :3] <= mx[b, :3]) & (mn[b, :3] <= mx[a, :3]))
    want = oracle_lib.sap_ref(0, mn, mx)
    assert np.array_equal(got, want)
    if axis_mode == 0:
        ax = np.array(sap.scene_axes()["axes"][0])
        assert abs(abs(ax @ R[:, 0]) - 1.0) < 1e-3


@pytest.mark.parametrize("seed", range(3))
def test_device_scene_solve_matches_numpy(cuda, seed):
    """The scene solve as the GPU runs it (float-float sums of the box
    centres, FP64 covariance, FP32 Jacobi) against numpy's FP64 eigh of the
    same centres: eigenvalues within 2e-6 of the largest, axes orthonormal
    to 1e-5 and aligned to ~2e-4 rad."""
    from gsap_gb300 import Sap
    rng = np.random.default_rng(seed)
    R = np.linalg.qr(rng.normal(size=(3, 3)))[0]
    n = 20000
    pts = ((rng.normal(size=(n, 3)) * [40.0, 9.0, 2.0]) @ R.T + rng.normal(size=3) * 100).astype(np.float32)
    h = np.float32(0.05)
    mn = np.concatenate([pts - h, np.zeros((n, 1), np.float32)], 1)
    mx = np.concatenate([pts + h, np.zeros((n, 1), np.float32)], 1)
    sap = Sap(n)
    run_bp(sap, mn, mx, cuda)
    sc = sap.scene_axes()
    U, eig = np.array(sc["axes"]), np.array(sc["eig"])
    w, V = np.linalg.eigh(np.cov(pts.astype(np.float64).T, bias=True))
    assert np.allclose(eig, w[::-1], rtol=0, atol=2e-6 * w.max())
    assert np.allclose(U @ U.T, np.eye(3), atol=1e-5)
    for k in range(3):
        assert 1.0 - abs(U[k] @ V[:, 2 - k]) / np.linalg.norm(U[k]) < 2e-8
    assert np.linalg.det(U) > 0


def test_large_scene_sampled_rows_against_brute_force(cuda):
    """16,777,216 boxes (the 1M workload's object density at 16 times the
    objects; about 95M pairs): every reported pair overlaps, the list is
    sorted and unique, and for 512 sampled objects the partners in the list
    are exactly those a brute-force test against all boxes finds (run on the
    GPU with torch as the checker; the CPU oracle is too slow at this size)."""
    import torch
    from gsap_gb300 import Sap, scenes
    n = 1 << 24
    f = 16.0 ** (1.0 / 3.0)
    c, h, _ = scenes.aabb_gauss_parts(n, seed=77, std=(100.0 * f, 20.0 * f, 5.0 * f))
    mn = torch.from_numpy(np.concatenate([c - h, np.zeros((n, 1), np.float32)], 1)).to(cuda)
    mx = torch.from_numpy(np.concatenate([c + h, np.zeros((n, 1), np.float32)], 1)).to(cuda)
    del c, h
    sap = Sap(n)
    p = sap.broadphase(mn, mx, sorted=True).long()
    sap.close()
    P = p.shape[0]
    assert P > 2 * n
    a, b = p[:, 0], p[:, 1]
    assert bool((a < b).all())
    key = a * n + b
    assert bool((key[1:] > key[:-1]).all())
    del key
    step = 1 << 24
    for s in range(0, P, step):
        i, j = a[s:s + step], b[s:s + step]
        assert bool(((mn[i, :3] <= mx[j, :3]) & (mn[j, :3] <= mx[i, :3])).all())
    g = torch.Generator().manual_seed(3)
    for s in torch.randint(0, n, (512,), generator=g).tolist():
        hit = ((mn[s, :3] <= mx[:, :3]) & (mn[:, :3] <= mx[s, :3])).all(1)
        hit[s] = False
        want = torch.nonzero(hit).flatten()
        got = torch.cat([b[a == s], a[b == s]]).sort().values
        assert torch.equal(got, want), s


def test_autotune_keeps_the_pair_set(cuda, oracle_lib):
    """Every setting of the tuning grid gives the same pair set; the tuner's
    choice lies in the grid and the handle keeps using it."""
    import torch
    from gsap_gb300 import Sap, scenes
    n = 60_000
    c, h, _ = scenes.aabb_gauss_parts(n, seed=11, std=(30.0, 8.0, 2.0))
    mn = np.concatenate([c - h, np.zeros((n, 1), np.float32)], 1)
    mx = np.concatenate([c + h, np.zeros((n, 1), np.float32)], 1)
    want = oracle_lib.bf_aabb(mn, mx)
    sap = Sap(n)
    dmn, dmx = to_dev(mn, cuda), to_dev(mx, cuda)
    cfg = sap.autotune(dmn, dmx, reps=2)
    assert cfg["sort_bits"] in (16, 24, 32) and cfg["cell_factor"] in (1.0, 1.5, 2.0, 2.5, 3.0)
    for graph in (False, True):
        got = sap.broadphase(dmn, dmx, sorted=True, graph=graph).cpu().numpy().astype(np.uint32)
        assert np.array_equal(got, want)
    # batched form of the tuner
    mnb, mxb, off = scenes.batched_aabb(S=24, seed=5, lo=16, hi=3000)
    bsap = Sap(len(mnb), max_scenes=24)
    doff = torch.from_numpy(off.astype(np.int32)).to(cuda)
    bm, bx = to_dev(mnb, cuda), to_dev(mxb, cuda)
    bsap.autotune(bm, bx, offsets=doff, reps=1)
    got = bsap.broadphase_batched(bm, bx, doff).cpu().numpy().astype(np.uint32)
    for s in range(24):
        a, b = int(off[s]), int(off[s + 1])
        sub = got[(got[:, 0] >= a) & (got[:, 0] < b)] - a
        assert np.array_equal(sub, oracle_lib.bf_aabb(mnb[a:b], mxb[a:b])), s


@pytest.mark.parametrize("sort_mode,sort_tile", [(0, 4096), (0, 2048), (1, 4096)])
@pytest.mark.parametrize("sort_bits", [16, 24, 32])
@pytest.mark.parametrize("cell_factor", [0.5, 1.0, 2.0, 4.0])
def test_every_setting_gives_the_same_pairs(cuda, oracle_lib, sort_bits, cell_factor, sort_mode, sort_tile):
    """Sort (bucket, or radix with 4096- or 2048-key tiles), key width and
    cell size only move work between stages: the pair set is the brute
    force's for every setting the autotuner may pick."""
    from gsap_gb300 import Sap, scenes
    n = 30_000
    c, h, _ = scenes.aabb_gauss_parts(n, seed=21, std=(25.0, 6.0, 2.0))
    mn = np.concatenate([c - h, np.zeros((n, 1), np.float32)], 1)
    mx = np.concatenate([c + h, np.zeros((n, 1), np.float32)], 1)
    sap = Sap(n, sort_bits=sort_bits, cell_factor=cell_factor, sort_mode=sort_mode, sort_tile=sort_tile)
    assert np.array_equal(run_bp(sap, mn, mx, cuda), oracle_lib.bf_aabb(mn, mx))
    assert np.array_equal(run_bp(sap, mn, mx, cuda, sorted=False), oracle_lib.bf_aabb(mn, mx))


@pytest.mark.parametrize("sort_bits", [24, 32])
def test_bucket_sort_sub_bucket_larger_than_shared_memory(cuda, oracle_lib, sort_bits):
    """A dense line of 20,000 thin boxes inside one cell, stretched out by a
    few far outliers so that one sub-bucket holds far more entries than a
    CTA sorts in shared memory: the bucket sort takes its global-memory path
    and the pair set is still the brute force's (the radix path agrees)."""
    from gsap_gb300 import Sap
    rng = np.random.default_rng(31)
    m = 20_000
    c = np.stack([rng.uniform(0, 10, m), rng.uniform(0, 1, m), rng.uniform(0, 1, m)], 1)
    h = np.stack([np.full(m, 0.001), np.full(m, 0.5), np.full(m, 0.5)], 1)
    far = np.array([[1000.0, 0.5, 0.5], [-1000.0, 0.5, 0.5], [900.0, 0.4, 0.6], [-900.0, 0.6, 0.4]])
    c = np.concatenate([c, far]).astype(np.float32)
    h = np.concatenate([h, np.full((4, 3), 0.5)]).astype(np.float32)
    n = len(c)
    mn = np.concatenate([c - h, np.zeros((n, 1), np.float32)], 1)
    mx = np.concatenate([c + h, np.zeros((n, 1), np.float32)], 1)
    want = oracle_lib.bf_aabb(mn, mx)
    for sort_mode in (0, 1):
        sap = Sap(n, sort_bits=sort_bits, sort_mode=sort_mode)
        assert np.array_equal(run_bp(sap, mn, mx, cuda), want), sort_mode


def test_batched_with_empty_and_tiny_scenes(cuda, oracle_lib):
    """Scenes of 0, 1 and 2 objects between ordinary ones: no pair crosses a
    scene edge and the small scenes produce what brute force says."""
    import torch
    from gsap_gb300 import Sap, scenes
    sizes = [0, 1, 500, 0, 2, 1, 3000, 0, 64, 1, 2, 700]
    rng = np.random.default_rng(9)
    mns, mxs = [], []
    for m in sizes:
        cc = rng.uniform(0, 20, (m, 3)).astype(np.float32)
        hh = rng.uniform(0.1, 1.5, (m, 3)).astype(np.float32)
        mns.append(np.concatenate([cc - hh, np.zeros((m, 1), np.float32)], 1))
        mxs.append(np.concatenate([cc + hh, np.zeros((m, 1), np.float32)], 1))
    mn, mx = np.concatenate(mns), np.concatenate(mxs)
    off = np.zeros(len(sizes) + 1, np.int64)
    off[1:] = np.cumsum(sizes)
    bsap = Sap(len(mn), max_scenes=len(sizes))
    got = bsap.broadphase_batched(to_dev(mn, cuda), to_dev(mx, cuda),
                                  torch.from_numpy(off.astype(np.int32)).to(cuda)).cpu().numpy().astype(np.uint32)
    want = [oracle_lib.bf_aabb(mn[a:b], mx[a:b]).astype(np.int64) + a
            for a, b in zip(off[:-1], off[1:]) if b - a >= 2]
    want = np.concatenate(want).astype(np.uint32)
    assert np.array_equal(got, want)


def test_bounded_wait_reports_timeout_and_recovers(cuda, oracle_lib):
    """A device wait on a predecessor that never publishes gives up after its
    poll limit and reports GSAP_ERR_DEVICE_TIMEOUT; nothing hangs, and the
    same handle then produces the exact pair set."""
    import torch
    from gsap_gb300 import Sap, _lib, scenes
    sap = Sap(4096)
    L = _lib.load()
    st = L.gsap_debug_lookback_timeout(sap.handle, 1000, None)
    assert st == 4  # GSAP_ERR_DEVICE_TIMEOUT
    assert b"iteration cap" in L.gsap_last_error()
    torch.cuda.synchronize()
    mn, mx = scenes.aabb_uniform(4096, 3)
    assert np.array_equal(run_bp(sap, mn, mx, cuda), oracle_lib.bf_aabb(mn, mx))


@pytest.mark.parametrize("graph", [False, True])
def test_temporal_mode_is_exact_frame_to_frame(cuda, oracle_lib, graph):
    """GSAP_FLAG_TEMPORAL: every call sweeps with the previous call's grid
    while its own PCA runs beside it.  Jittered frames, a frame moved far
    away, a frame of another size: the pair set is the brute force's each
    time."""
    from gsap_gb300 import Sap, scenes
    n = 30_000
    c, h, _ = scenes.aabb_gauss_parts(n, seed=31, std=(25.0, 6.0, 2.0))
    sap = Sap(n + 1000)

    def frame(cc, hh):
        mn = np.concatenate([cc - hh, np.zeros((len(cc), 1), np.float32)], 1)
        mx = np.concatenate([cc + hh, np.zeros((len(cc), 1), np.float32)], 1)
        got = sap.broadphase(to_dev(mn, cuda), to_dev(mx, cuda), sorted=True, graph=graph, temporal=True)
        assert np.array_equal(got.cpu().numpy().astype(np.uint32), oracle_lib.bf_aabb(mn, mx))

    for k in range(4):
        frame(scenes.jitter(c, seed=100 + k), h)
    frame(c + np.float32([60.0, -20.0, 5.0]), h)    # far from the grid of the previous frame
    frame(c[::-1].copy() * np.float32(1.5), h[::-1].copy())  # rescaled and renumbered
    c2, h2, _ = scenes.aabb_gauss_parts(n + 1000, seed=32, std=(25.0, 6.0, 2.0))
    frame(c2, h2)                                   # another size: plain pipeline first
    frame(scenes.jitter(c2, seed=7), h2)


@pytest.mark.parametrize("batched", [False, True])
def test_temporal_next_grid_is_the_inputs_pca(cuda, batched):
    """In temporal mode the projection takes the call's PCA sums (one
    partial per projection CTA) and the scene solve prepares the next call's
    grid from them: after a temporal call on frame B the handle's axes,
    eigenvalues and mean are those a plain call computes on B (the two sum
    the same terms in a different order)."""
    import torch
    from gsap_gb300 import Sap, scenes
    n = 50_000
    c, h, _ = scenes.aabb_gauss_parts(n, seed=41, std=(30.0, 9.0, 3.0))
    mn = np.concatenate([c - h, np.zeros((n, 1), np.float32)], 1)
    mx = np.concatenate([c + h, np.zeros((n, 1), np.float32)], 1)
    b = scenes.jitter(c, seed=5) + np.float32([4.0, -2.0, 1.0])
    mnb = np.concatenate([b - h, np.zeros((n, 1), np.float32)], 1)
    mxb = np.concatenate([b + h, np.zeros((n, 1), np.float32)], 1)
    off = torch.tensor([0, n // 3, n], dtype=torch.int32, device=cuda)
    S = 2 if batched else 1

    def call(sap, a, z, temporal):
        if batched:
            sap.broadphase_batched(to_dev(a, cuda), to_dev(z, cuda), off, temporal=temporal)
        else:
            sap.broadphase(to_dev(a, cuda), to_dev(z, cuda), sorted=True, temporal=temporal)

    tsap, psap = Sap(n, max_scenes=S), Sap(n, max_scenes=S)
    call(tsap, mn, mx, True)    # no previous grid: plain pipeline
    call(tsap, mnb, mxb, True)  # temporal: sweeps with A's grid, prepares B's
    call(psap, mnb, mxb, False)
    for s in range(S):
        t, p = tsap.scene_axes(s), psap.scene_axes(s)
        assert np.allclose(t["axes"], p["axes"], rtol=0, atol=1e-9)
        assert np.allclose(t["eig"], p["eig"], rtol=1e-9, atol=0)
        assert np.allclose(t["mean"], p["mean"], rtol=1e-12, atol=1e-9)


def test_batched_temporal_frames_are_exact(cuda, oracle_lib):
    """GSAP_FLAG_TEMPORAL on batched calls: each scene's pairs stay the brute
    force's from frame to frame, including a frame where scene sizes change
    (same total and count) and a frame where one scene moves far away."""
    import torch
    from gsap_gb300 import Sap, scenes
    mn, mx, off = scenes.batched_aabb(S=16, seed=12, lo=16, hi=2500)
    n = len(mn)
    bsap = Sap(n, max_scenes=16)

    def frame(a, b, o):
        got = bsap.broadphase_batched(to_dev(a, cuda), to_dev(b, cuda), torch.from_numpy(o.astype(np.int32)).to(cuda),
                                      temporal=True).cpu().numpy().astype(np.uint32)
        want = [oracle_lib.bf_aabb(a[s:e], b[s:e]).astype(np.int64) + s for s, e in zip(o[:-1], o[1:]) if e - s >= 2]
        assert np.array_equal(got, np.concatenate(want).astype(np.uint32))

    rng = np.random.default_rng(1)
    for k in range(3):
        d = rng.normal(0, 0.05, (n, 3)).astype(np.float32)
        a, b = mn.copy(), mx.copy()
        a[:, :3] += d
        b[:, :3] += d
        frame(a, b, off)
    off2 = off.copy()
    off2[5] = (off[4] + off[6]) // 2  # scene edges move, same count and total
    frame(mn, mx, off2)
    a, b = mn.copy(), mx.copy()
    s, e = int(off2[7]), int(off2[8])
    a[s:e, :3] += 500.0
    b[s:e, :3] += 500.0
    frame(a, b, off2)


def test_bad_scene_offsets_are_reported(cuda, oracle_lib):
    """Offsets that decrease, or do not run from 0 to n, are clamped on the
    device (no access outside the input) and reported as GSAP_ERR_INVALID;
    the handle then serves a valid call."""
    import torch
    from gsap_gb300 import GsapError, Sap, scenes
    mn, mx, off = scenes.batched_aabb(S=4, seed=2, lo=100, hi=400)
    n = len(mn)
    bsap = Sap(n, max_scenes=4)
    dmn, dmx = to_dev(mn, cuda), to_dev(mx, cuda)
    for bad in ([0, 300, 200, 350, n], [0, 100, 200, 300, n + 50], [5, 100, 200, 300, n]):
        with pytest.raises(GsapError) as ei:
            bsap.broadphase_batched(dmn, dmx, torch.tensor(bad, dtype=torch.int32, device=cuda))
        assert ei.value.status == 1  # GSAP_ERR_INVALID
    got = bsap.broadphase_batched(dmn, dmx, torch.from_numpy(off.astype(np.int32)).to(cuda))
    want = [oracle_lib.bf_aabb(mn[a:b], mx[a:b]).astype(np.int64) + a for a, b in zip(off[:-1], off[1:])]
    assert np.array_equal(got.cpu().numpy().astype(np.uint32), np.concatenate(want).astype(np.uint32))


def test_degenerate_and_far_from_origin_scenes(cuda, oracle_lib):
    """All boxes identical (zero spread: the eigensolve's degenerate path, one
    cell, every pair overlapping), a flat scene (zero spread on one axis) and
    a cloud a million units from the origin (FP32 spacing ~0.06 there)."""
    from gsap_gb300 import Sap
    rng = np.random.default_rng(17)
    n = 300
    same = np.tile(np.float32([[1.0, 2.0, 3.0, 0.0]]), (n, 1))
    sap = Sap(4000, pair_factor=200)
    got = run_bp(sap, same - np.float32([0.5, 0.5, 0.5, 0]), same + np.float32([0.5, 0.5, 0.5, 0]), cuda)
    assert len(got) == n * (n - 1) // 2
    c = rng.uniform(0, 30, (4000, 3)).astype(np.float32)
    c[:, 2] = 7.0  # flat
    h = rng.uniform(0.1, 0.6, (4000, 3)).astype(np.float32)
    mn = np.concatenate([c - h, np.zeros((4000, 1), np.float32)], 1)
    mx = np.concatenate([c + h, np.zeros((4000, 1), np.float32)], 1)
    assert np.array_equal(run_bp(sap, mn, mx, cuda), oracle_lib.bf_aabb(mn, mx))
    # a box overlapping 3000 others: its row is longer than a warp sorts in
    # shared memory (rank placement path)
    big = np.concatenate([np.float32([[15.0, 15.0, 7.0]]), c[:2999]], 0)
    hb = np.concatenate([np.float32([[40.0, 40.0, 40.0]]), h[:2999]], 0)
    mn = np.concatenate([big - hb, np.zeros((3000, 1), np.float32)], 1)
    mx = np.concatenate([big + hb, np.zeros((3000, 1), np.float32)], 1)
    got = run_bp(sap, mn, mx, cuda)
    assert np.count_nonzero(got[:, 0] == 0) == 2999
    assert np.array_equal(got, oracle_lib.bf_aabb(mn, mx))
    far = (rng.uniform(0, 40, (4000, 3)) + 1.0e6).astype(np.float32)
    mn = np.concatenate([far - h, np.zeros((4000, 1), np.float32)], 1)
    mx = np.concatenate([far + h, np.zeros((4000, 1), np.float32)], 1)
    assert np.array_equal(run_bp(sap, mn, mx, cuda), oracle_lib.bf_aabb(mn, mx))


def test_rows_longer_than_the_shared_memory_sort(cuda, oracle_lib):
    """Rows past the rank kernel's shared-memory sort (4096 pairs): two large
    boxes (and spheres) each overlapping all 5,998 small ones, in the sorted
    (i<j) form and the both-direction collision form."""
    import torch
    from gsap_gb300 import MODE_SPHERE, Sap
    rng = np.random.default_rng(29)
    n = 6000
    c = rng.uniform(0, 30, (n, 3)).astype(np.float32)
    h = rng.uniform(0.1, 0.4, (n, 3)).astype(np.float32)
    c[:2] = 15.0
    h[:2] = 20.0
    mn = np.concatenate([c - h, np.zeros((n, 1), np.float32)], 1)
    mx = np.concatenate([c + h, np.zeros((n, 1), np.float32)], 1)
    got = run_bp(Sap(n), mn, mx, cuda)
    assert np.count_nonzero(got[:, 0] == 0) == n - 1
    assert np.array_equal(got, oracle_lib.bf_aabb(mn, mx))
    r = np.full((n, 1), 0.3, np.float32)
    r[:2] = 30.0
    sp = np.concatenate([c, r], 1)
    ssap = Sap(n, mode=MODE_SPHERE)
    pairs = torch.empty((16 * n, 2), dtype=torch.int32, device=cuda)
    ent = torch.empty(n + 1, dtype=torch.int32, device=cuda)
    n_pairs, n_ent = ssap.collision(0.0, torch.from_numpy(sp).to(cuda), pairs, ent)
    want_pairs, want_ent = oracle_lib.both_directions(oracle_lib.bf_sphere(sp))
    assert n_pairs == len(want_pairs) and n_ent == len(want_ent)
    assert np.array_equal(pairs[:n_pairs].cpu().numpy(), want_pairs)
    assert np.array_equal(ent[:n_ent].cpu().numpy(), want_ent)


def test_chains_alternating_with_a_dense_scene(cuda, oracle_lib):
    """Chains of boxes that each overlap only the next one (2047, 2048 and
    2049 pairs, rows of one pair, shuffled ids, a rank-1 spread) alternating
    on one handle with a dense scene: every call equals the brute force (a
    row counter left behind by one call would shift the next call's rows)."""
    from gsap_gb300 import Sap
    rng = np.random.default_rng(37)
    sap = Sap(8192)
    dense_c = rng.uniform(0, 12, (6000, 3)).astype(np.float32)
    dense_h = rng.uniform(0.2, 0.5, (6000, 3)).astype(np.float32)
    dense = (np.concatenate([dense_c - dense_h, np.zeros((6000, 1), np.float32)], 1),
             np.concatenate([dense_c + dense_h, np.zeros((6000, 1), np.float32)], 1))
    for m in (2048, 2049, 2050, 2049):
        x = np.arange(m, dtype=np.float32)
        c = np.stack([x, np.zeros(m, np.float32), np.zeros(m, np.float32)], 1)[rng.permutation(m)]
        h = np.float32([0.6, 0.5, 0.5])  # neighbours 1.0 apart overlap, next-but-one do not
        mn = np.concatenate([c - h, np.zeros((m, 1), np.float32)], 1)
        mx = np.concatenate([c + h, np.zeros((m, 1), np.float32)], 1)
        want = oracle_lib.bf_aabb(mn, mx)
        assert len(want) == m - 1
        assert np.array_equal(run_bp(sap, mn, mx, cuda), want)
        assert np.array_equal(run_bp(sap, *dense, cuda), oracle_lib.bf_aabb(*dense))


@pytest.mark.parametrize("both", [False, True])
def test_sparse_pairs_reset_row_counters_between_calls(cuda, oracle_lib, both):
    """Few pairs against many objects (fewer than n / 4): the scatter, not
    the row scan, puts the touched rows' counters back to zero.  Calls on
    one handle with different inputs, dense and sparse in turn, each equal
    the brute force (a stale counter would shift the next call's rows)."""
    from gsap_gb300 import MODE_SPHERE, Sap, scenes
    n = 60_000
    sap = Sap(n, mode=MODE_SPHERE if both else 0)
    rng = np.random.default_rng(11)
    for k, spread in enumerate((400.0, 40.0, 400.0, 900.0)):
        c = rng.uniform(-spread, spread, (n, 3)).astype(np.float32)
        if both:
            import torch
            sph = np.concatenate([c, np.full((n, 1), 0.5, np.float32)], 1)
            pairs = torch.empty((16 * n, 2), dtype=torch.int32, device=cuda)
            ent = torch.empty(n + 1, dtype=torch.int32, device=cuda)
            n_pairs, n_ent = sap.collision(0.0, to_dev(sph, cuda), pairs, ent)
            want_pairs, want_ent = oracle_lib.both_directions(oracle_lib.bf_sphere(sph))
            assert np.array_equal(pairs[:n_pairs].cpu().numpy(), want_pairs), k
            assert np.array_equal(ent[:n_ent].cpu().numpy(), want_ent), k
        else:
            h = np.full((n, 3), 0.5, np.float32)
            mn = np.concatenate([c - h, np.zeros((n, 1), np.float32)], 1)
            mx = np.concatenate([c + h, np.zeros((n, 1), np.float32)], 1)
            want = oracle_lib.bf_aabb(mn, mx)
            if spread > 100:
                assert 4 * len(want) < n  # the sparse case
            assert np.array_equal(run_bp(sap, mn, mx, cuda), want), k


def test_objects_spanning_many_cells(cuda, oracle_lib):
    """A few boxes hundreds of cells wide among small ones: the projection
    writes such objects' entries lane by lane (more entries per warp item
    than its shared-memory stage holds) and the rest through the stage; the
    pair set is the brute force's."""
    from gsap_gb300 import Sap
    rng = np.random.default_rng(17)
    n = 20_000
    c = rng.normal(0.0, [60.0, 12.0, 4.0], (n, 3)).astype(np.float32)
    h = rng.uniform(0.1, 0.6, (n, 3)).astype(np.float32)
    big = rng.choice(n, 40, replace=False)
    h[big] = rng.uniform(5.0, 15.0, (40, 3))  # each spans tens to hundreds of cells
    mn = np.concatenate([c - h, np.zeros((n, 1), np.float32)], 1)
    mx = np.concatenate([c + h, np.zeros((n, 1), np.float32)], 1)
    want = oracle_lib.bf_aabb(mn, mx)
    for cf in (0.5, 2.0):
        sap = Sap(n, cell_factor=cf, entry_factor=64, pair_factor=64)
        assert np.array_equal(run_bp(sap, mn, mx, cuda), want), cf
        assert sap.stats()["entries"] > n + 1000  # the big boxes really replicate
