"""CPU tests of the C ABI: libgsap.so loads without a GPU, exports every
function include/*.h declares, and its host-side pieces (the FP64 scene
solver the PCA kernel runs in its last CTA) behave."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT


def declared_functions():
    names = set()
    for h in ("gsap.h", "gsap_debug.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(gsap_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(gsap_lib):
    from gsap_gb300 import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True, check=True)
    exported = {l.split()[-1] for l in out.stdout.splitlines() if " T " in l}
    decl = declared_functions()
    assert len(decl) >= 40
    missing = decl - exported
    assert not missing, missing
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert decl == bound, (decl - bound, bound - decl)


def test_config_defaults(gsap_lib):
    from gsap_gb300._lib import Config
    c = Config()
    gsap_lib.gsap_config_default(C.byref(c))
    assert (c.mode, c.axis_mode, c.max_scenes, c.entry_factor, c.sort_bits) == (0, 0, 1, 8, 32)
    assert abs(c.cell_factor - 2.0) < 1e-7


def test_struct_sizes(gsap_lib):
    out = (C.c_uint32 * 4)()
    assert gsap_lib.gsap_debug_sizes(out) == 0
    ctrl, scene, partial, tile = list(out)
    assert ctrl % 8 == 0 and scene % 8 == 0
    assert partial == 4 * (18 * 2 + 4)
    assert tile == 4096


def solve(gsap_lib, pts, h, axis_mode=0, cell_factor=1.5, key_bits=32, entry_factor=8):
    pts = np.asarray(pts, np.float64)
    h = np.abs(np.asarray(h, np.float64))
    pilot = pts[0]
    d = pts - pilot
    sums = np.concatenate([d.sum(0), [(d[:, 0] * d[:, 0]).sum(), (d[:, 0] * d[:, 1]).sum(), (d[:, 0] * d[:, 2]).sum(),
                                      (d[:, 1] * d[:, 1]).sum(), (d[:, 1] * d[:, 2]).sum(), (d[:, 2] * d[:, 2]).sum()],
                           h.sum(0), [(h[:, 0] * h[:, 0]).sum(), (h[:, 0] * h[:, 1]).sum(), (h[:, 0] * h[:, 2]).sum(),
                                      (h[:, 1] * h[:, 1]).sum(), (h[:, 1] * h[:, 2]).sum(), (h[:, 2] * h[:, 2]).sum()]])
    out = (C.c_double * 17)()
    arr = lambda a: (C.c_double * len(a))(*a)
    n = len(pts)
    r = gsap_lib.gsap_debug_scene_solve(arr(sums), arr(h.max(0)), arr(pilot), float(n), n, axis_mode,
                                        C.c_float(cell_factor), key_bits, entry_factor * n + 4096, out)
    assert r == 0
    v = np.array(list(out))
    return v[:9].reshape(3, 3), v[9:12], v[12:15], int(v[15]), int(v[16])


@pytest.mark.parametrize("seed", range(5))
def test_eigensolve_matches_numpy(gsap_lib, seed):
    """The scene solve (covariance in FP64, FP32 Jacobi) against numpy's
    FP64 eigh: eigenvalues within a few FP32 ulps of the largest, axes
    orthonormal and aligned to ~1e-7."""
    rng = np.random.default_rng(seed)
    R = np.linalg.qr(rng.normal(size=(3, 3)))[0]
    pts = (rng.normal(size=(5000, 3)) * [40.0, 9.0, 2.0]) @ R.T + rng.normal(size=3) * 100
    U, eig, mean, G2, G3 = solve(gsap_lib, pts, np.full((5000, 3), 0.3))
    C_ = np.cov(pts.T, bias=True)
    w, V = np.linalg.eigh(C_)
    assert np.allclose(eig, w[::-1], rtol=0, atol=4e-7 * w.max())
    for k in range(3):  # angle to numpy's axis below ~1.4e-5
        assert 1.0 - abs(U[k] @ V[:, 2 - k]) / np.linalg.norm(U[k]) < 1e-10
    assert np.allclose(U @ U.T, np.eye(3), atol=1e-6)
    assert np.linalg.det(U) > 0
    assert np.allclose(mean, pts.mean(0), rtol=1e-12, atol=1e-9)
    assert G2 >= 1 and G3 >= 1


def test_degenerate_spreads_are_deterministic(gsap_lib):
    rng = np.random.default_rng(0)
    pts = rng.normal(size=(2000, 3))
    pts[:, 2] = 0.0  # rank 2
    a = solve(gsap_lib, pts, np.zeros((2000, 3)))
    b = solve(gsap_lib, pts, np.zeros((2000, 3)))
    assert np.array_equal(a[0], b[0])
    iso = np.tile([[1.0, 2.0, 3.0]], (100, 1))  # all centres equal
    U, eig, *_ = solve(gsap_lib, iso, np.full((100, 3), 0.5))
    assert np.allclose(U @ U.T, np.eye(3))
    assert np.allclose(eig, 0.0, atol=1e-12)


def test_reference_axis_rule(gsap_lib):
    """axisVecMultiple (SapKernel.cu:63-97): argmax of the diagonal with its
    tie order and fixed secondary axes."""
    rng = np.random.default_rng(1)
    for std, want in (([5, 1, 1], [0, 1, 2]), ([1, 5, 1], [1, 0, 2]), ([1, 1, 5], [2, 0, 1])):
        pts = rng.normal(size=(3000, 3)) * std
        U, *_ = solve(gsap_lib, pts, np.zeros((3000, 3)), axis_mode=1)
        assert np.array_equal(np.argmax(np.abs(U), axis=1), want)


def test_grid_respects_entry_bound(gsap_lib):
    """The chosen cell size keeps the worst-case replica count within the
    entry capacity, even for wide boxes."""
    rng = np.random.default_rng(2)
    for hw in (0.05, 0.5, 5.0, 50.0):
        pts = rng.normal(size=(20000, 3)) * [100, 20, 5]
        h = np.full((20000, 3), hw)
        U, eig, mean, G2, G3 = solve(gsap_lib, pts, h)
        s2 = (8 * np.sqrt(eig[1]) + 2 * (np.abs(U[1]) @ h[0])) / G2
        s3 = (8 * np.sqrt(eig[2]) + 2 * (np.abs(U[2]) @ h[0])) / G3
        w2, w3 = 2 * np.abs(U[1]) @ h[0], 2 * np.abs(U[2]) @ h[0]
        worst = min(G2, w2 / s2 + 2) * min(G3, w3 / s3 + 2) * len(pts)
        assert worst <= 8 * len(pts) + 4096


@pytest.mark.parametrize("key_bits,qmin", [(16, 6), (24, 8), (32, 12)])
def test_grid_leaves_the_key_its_q_bits(gsap_lib, key_bits, qmin):
    """Whatever the object count, the cells of a one-scene grid take at most
    key_bits - qmin bits of the sweep key (16-bit keys: at most 1024 cells),
    so the quantised lower bound keeps at least qmin bits."""
    rng = np.random.default_rng(3)
    for n in (500, 16384, 200000):
        pts = rng.uniform(0, 100, (n, 3))
        U, eig, mean, G2, G3 = solve(gsap_lib, pts, np.full((n, 3), 0.05), key_bits=key_bits)
        assert 1 <= G2 * G3 <= 2 ** (key_bits - qmin)


def test_demo_scene_and_snapshot_round_trip(tmp_path):
    """The headless demo's scene (DemoParticles::init layout) and its binary
    snapshots; no GPU needed."""
    from gsap_gb300 import demo
    sc = demo.demo_scene(512, n_row=8, seed=3)
    assert sc["pos"].shape == (512, 4) and sc["n_particles"] == 6 * 512
    assert np.array_equal(sc["shape_idx"][:4], [0, 1, 0, 1])
    # hexagon offsets: six particles at one radius from the body centre
    r0 = np.linalg.norm(sc["ref_pos"][0:6, :3], axis=1)
    r1 = np.linalg.norm(sc["ref_pos"][10:16, :3], axis=1)
    assert np.allclose(r0, 0.5005) and np.allclose(r1, 0.5005 * 1.2)
    assert sc["pos"][:, 1].min() == np.float32(3.6) and sc["pos"][:, 1].max() == np.float32(3.6 * 8)
    state = {k: sc[k] + 1.0 for k in ("pos", "quat", "lin_vel", "ang_vel")}
    path = tmp_path / "snap.npz"
    demo.save_snapshot(path, sc, state, step=7)
    back, step = demo.load_snapshot(path)
    assert step == 7 and back["n_particles"] == sc["n_particles"]
    for k in ("pos", "quat", "lin_vel", "ang_vel"):
        assert np.array_equal(back[k], state[k])
    for k in ("shape_idx", "p_start", "ref_pos", "shape_inv_inertia"):
        assert np.array_equal(back[k], sc[k])
