"""CPU tests: the oracle against the golden vectors made by the reference's
own code (tests/golden/make_golden.py), and its internal consistency."""
import os

import numpy as np
import pytest

from conftest import GOLDEN


def load(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def test_bf_aabb_matches_reference_overlaps(oracle_lib):
    g = load("aabb_bf_golden.npz")
    for name in g["names"]:
        mn, mx, want = g[f"{name}__min"], g[f"{name}__max"], g[f"{name}__pairs"]
        got = oracle_lib.bf_aabb(mn, mx) if len(mn) else np.zeros((0, 2), np.uint32)
        assert np.array_equal(got, want), name


def test_sap_restatement_matches_reference_overlaps(oracle_lib):
    g = load("aabb_bf_golden.npz")
    for name in g["names"]:
        mn, mx, want = g[f"{name}__min"], g[f"{name}__max"], g[f"{name}__pairs"]
        if len(mn) == 0:
            continue
        got = oracle_lib.sap_ref(0, mn, mx)
        assert np.array_equal(got, want), name


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_sap_restatement_equals_brute_force(oracle_lib, seed):
    rng = np.random.default_rng(seed)
    n = 4000
    R, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    c = (rng.normal(size=(n, 3)) * np.array([30.0, 8.0, 3.0])) @ R.T
    h = np.exp(rng.normal(-1.0, 0.5, (n, 3))).clip(0.05, 2.0)
    mn, mx = (c - h).astype(np.float32), (c + h).astype(np.float32)
    assert np.array_equal(oracle_lib.sap_ref(0, mn, mx), oracle_lib.bf_aabb(mn, mx))
    sp = np.concatenate([c, h[:, :1]], 1).astype(np.float32)
    assert np.array_equal(oracle_lib.sap_ref(1, sp), oracle_lib.bf_sphere(sp))


def test_sap_slices_cover_the_full_sweep(oracle_lib):
    """The timing sample of the CPU baseline: the sweeps started from slice
    k of `parts` contiguous slices, over every k, find exactly the full
    call's pairs, and each call reports non-negative stage times."""
    import ctypes as C
    rng = np.random.default_rng(5)
    n = 6000
    c = rng.normal(size=(n, 3)) * np.array([40.0, 9.0, 3.0])
    h = np.exp(rng.normal(-1.0, 0.5, (n, 3))).clip(0.05, 2.0)
    mn = np.concatenate([c - h, np.zeros((n, 1))], 1).astype(np.float32)
    mx = np.concatenate([c + h, np.zeros((n, 1))], 1).astype(np.float32)
    full = oracle_lib.sap_ref(0, mn, mx)
    L = oracle_lib.lib()
    got = set()
    for k in range(8):
        out = np.empty((len(full), 2), np.uint32)
        secs = np.full(2, -1.0)
        m = L.orc_sap_ref_sampled(0, mn.ctypes.data, mx.ctypes.data, C.c_uint32(n), C.c_uint32(8), C.c_uint32(k),
                                  out.ctypes.data, C.c_int64(len(full)), 0, secs.ctypes.data)
        assert 0 < m <= len(full) and (secs >= 0).all()
        got |= {tuple(p) for p in out[:m]}
        assert oracle_lib.sap_ref_sampled(0, mn, mx, 8, k)[0] == m
    assert got == {tuple(p) for p in full}


@pytest.mark.parametrize("fixture", ["rb_ref_step_golden.npz", "rb_demo_steps_golden.npz"])
def test_rb_reference_step_matches_reference_kernels(oracle_lib, fixture):
    """The FP32 restatement reproduces the reference kernels bit for bit:
    a 64-body ring scene for 3 steps, and the headless demo's scene (two
    hexagon sizes, 256 bodies in contact) for 4 steps."""
    g = load(fixture)
    dt, spM, dpM, vmax, gy = (float(x) for x in g["params"])
    s = {k[len("init__"):]: g[k].copy() for k in g.files if k.startswith("init__")}
    oracle_lib.normalize_quats(s["quat"])  # setRbData's upload normalisation
    for step in range(int(g["steps"]) if "steps" in g.files else 3):
        npairs = oracle_lib.rb_step_ref(s, dt, spM, dpM, max_lin_vel=vmax, gravity_y=gy, floor_clamp=True,
                                        torque_quirk=True, pair_loop_quirk=True)
        assert npairs == int(g[f"step{step}__npairs"])
        for k in ("pos", "quat", "lin_vel", "ang_vel", "p_pos", "p_vel", "p_force"):
            assert np.array_equal(s[k], g[f"step{step}__{k}"]), (step, k)


def test_both_direction_format_matches_demo_dump(oracle_lib):
    """cudaPhysics/2_1024.txt: the reference's CPU broadphase dumps per frame
    (pairs in both directions, pairEntries).  The oracle's both-direction
    format reproduces each frame's pair set and entry offsets."""
    g = load("demo_2_1024.npz")
    for f in range(int(g["frames"])):
        ij = g[f"f{f}__ij"]
        n_pairs, n_ent = (int(x) for x in g[f"f{f}__counts"])
        assert len(ij) == n_pairs
        uniq = np.unique(np.sort(ij, axis=1), axis=0).astype(np.uint32)
        both, ent = oracle_lib.both_directions(uniq)
        assert len(both) == n_pairs
        assert len(ent) == n_ent
        assert set(map(tuple, both.tolist())) == set(map(tuple, ij.tolist()))
        # entries are offsets of the first pair of every distinct first id
        assert np.array_equal(ent, g[f"f{f}__entries"][:n_ent])


def test_sphere_predicate_on_demo_dump(oracle_lib):
    """Every pair of the dump overlaps under the squared strict test (the
    dump prints 6 significant digits, so near-touching pairs are skipped)."""
    g = load("demo_2_1024.npz")
    checked = 0
    for f in range(int(g["frames"])):
        pi, pj = g[f"f{f}__pi"].astype(np.float64), g[f"f{f}__pj"].astype(np.float64)
        d = np.linalg.norm(pi[:, :3] - pj[:, :3], axis=1)
        r = pi[:, 3] + pj[:, 3]
        clear = np.abs(d - r) > 1e-4 * r
        assert np.all(d[clear] < r[clear])
        pair = np.concatenate([pi, pj], 1).astype(np.float32).reshape(-1, 2, 4)
        for a, b in pair[clear]:
            got = oracle_lib.bf_sphere(np.stack([a, b]))
            assert len(got) == 1
            checked += 1
    assert checked > 100


def test_radix_sort_oracle_is_stable(oracle_lib):
    rng = np.random.default_rng(3)
    for bits in (8, 23, 24, 32):
        k = rng.integers(0, 1 << min(bits, 31), 5000, dtype=np.uint64).astype(np.uint32)
        k[::7] = k[0]
        v = np.arange(len(k), dtype=np.uint32)
        ks, vs = oracle_lib.radix_sort_u32(k, v, bits)
        order = np.argsort(k & np.uint32((1 << bits) - 1 if bits < 32 else 0xFFFFFFFF), kind="stable")
        assert np.array_equal(vs, order)


def test_float_flip_orders_floats(oracle_lib):
    x = np.array([-np.inf, -3.5, -1e-30, -0.0, 0.0, 1e-45, 2.0, np.inf], np.float32)
    u = oracle_lib.float_flip(x)
    assert np.all(np.diff(u.astype(np.int64)) >= 0)
    assert oracle_lib.lib().orc_float_flip(2.0) == int(oracle_lib.float_flip(np.float32(2.0)).reshape(-1)[0])


def test_cfg_f64_step_conserves_momentum_without_walls(oracle_lib):
    """Two overlapping cubes, no gravity, walls far away: internal contact
    forces cancel, so total linear momentum is unchanged."""
    from gsap_gb300 import scenes
    sc = scenes.cubes_in_box(2, box=1000.0, seed=0)
    sc["pos"][0, :3] = [500.0, 500.0, 500.0]
    sc["pos"][1, :3] = [501.2, 500.3, 500.1]
    st = scenes.to_f64(sc)
    p = dict(dt=1 / 600, k=2e4, eta=50.0, kt=0.1, gravity_y=0.0, box_lo=(0, 0, 0), box_hi=(1000, 1000, 1000))
    m = 1.0 / st["inv_mass"]
    p0 = (st["lin_vel"][:, :3] * m[:, None]).sum(0)
    for _ in range(5):
        oracle_lib.rb_step_cfg_f64(st, p)
    p1 = (st["lin_vel"][:, :3] * m[:, None]).sum(0)
    assert np.allclose(p0, p1, atol=1e-9)
    assert np.abs(st["lin_vel"][:, :3]).max() > 0  # they did collide


def test_fp64_body_pair_search_equals_brute_force(oracle_lib):
    """The sort-and-sweep body pair search of the FP64 rigid-body oracle
    finds the brute force's rows exactly, scenes respected, touching boxes
    included."""
    rng = np.random.default_rng(3)
    nb = 3000
    c = rng.uniform(0, 30, (nb, 3))
    h = rng.uniform(0.2, 1.2, (nb, 3))
    bmin, bmax = c - h, c + h
    bmin[10] = bmax[11] - np.array([2.0, 2.0, 2.0])  # 10 and 11 touch at a corner
    bmax[10] = bmax[11]
    bmin[12, 0] = bmax[13, 0]  # touching faces on x
    scene = np.repeat(np.arange(5), nb // 5).astype(np.int32)
    for sc in (None, scene):
        a = oracle_lib.body_neighbours(bmin, bmax, sc, brute=True)
        b = oracle_lib.body_neighbours(bmin, bmax, sc, brute=False)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        assert a[1].size > nb // 4


def test_batched_pairs_oracle(oracle_lib):
    """The batched pair oracle: per-scene brute force and the x-sorted form
    for large scenes give the same sorted list, equal to brute force of each
    scene with global ids; no pair crosses scenes."""
    from gsap_gb300 import scenes
    mn, mx, off = scenes.batched_aabb(S=12, seed=4, lo=16, hi=3000)
    mn[:, :3] *= 0.2  # crowd the scenes so they have pairs
    mx[:, :3] = mn[:, :3] + (mx[:, :3] - mn[:, :3]) * 5.0
    a = oracle_lib.pairs_batched(mn, mx, off, bf_max=1 << 30)
    b = oracle_lib.pairs_batched(mn, mx, off, bf_max=0)
    assert np.array_equal(a, b) and len(a) > 100
    want = [oracle_lib.bf_aabb(mn[off[s]:off[s + 1]], mx[off[s]:off[s + 1]]) + off[s] for s in range(12)]
    assert np.array_equal(a, np.concatenate(want).astype(np.uint32))
