"""Generate the golden fixtures of tests/golden from the reference's own code.

Run where the reference tree is mounted (it is not needed afterwards):

    python tests/golden/make_golden.py [--ref /path/to/physicboxSap2.16_Fermi]

It builds oracle/_ref/libgsapref.so (``make -C oracle ref``), which compiles
the reference's Aabb::overlaps (include/aabb.h:47-57) and its particle
rigid-body kernels (ParticleRigidBody/ParticleRigidBodyKernel.h) for the host,
and writes:

  aabb_bf_golden.npz     inputs and the reference brute-force pair lists of
                         adversarial AABB cases (touching faces, identical and
                         zero-extent boxes, inverted boxes, n not a multiple
                         of 512, n = 0, 1)
  rb_ref_step_golden.npz a 64-body scene of six-particle ring bodies (the
                         demo's body layout, cudaPhysics/demoParticles.h:184-288)
                         and its state after each of 3 reference steps
  demo_2_1024.npz        the per-frame pair dumps of cudaPhysics/2_1024.txt
                         (CPU brute-force pairs of the demo with both spheres)
  rb_demo_steps_golden.npz
                         the headless demo's scene (hexagon bodies of two
                         sizes, 256 bodies packed into contact) and its state
                         after each of 4 reference steps
"""
from __future__ import annotations

import argparse
import ctypes as C
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402

DEFAULT_REF = "/root/reference/physicboxSap2.16_Fermi"


def f4(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def aabb_cases(rng):
    cases = {}
    # random boxes, cfg-1 statistics, n not a multiple of 512
    n = 1500
    c = rng.uniform(0, 25, (n, 3)).astype(np.float32)
    h = rng.uniform(0.1, 0.5, (n, 3)).astype(np.float32)
    cases["random_1500"] = (c - h, c + h)
    # unit cubes on a lattice touching face to face (closed test => pairs)
    g = np.stack(np.meshgrid(np.arange(6), np.arange(5), np.arange(4), indexing="ij"), -1).reshape(-1, 3)
    g = g.astype(np.float32)
    cases["touching_lattice"] = (g, g + 1.0)
    # identical boxes: every pair overlaps
    mn = np.tile(np.array([[1.0, 2.0, 3.0]], np.float32), (40, 1))
    cases["identical_40"] = (mn, mn + 0.5)
    # zero extents: points, some coincident
    p = rng.integers(0, 4, (300, 3)).astype(np.float32) * 0.5
    cases["points_300"] = (p, p.copy())
    # rotated anisotropic Gaussian, n = 517
    n = 517
    R, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    c = (rng.normal(size=(n, 3)) * np.array([20, 5, 1])) @ R.T
    h = np.exp(rng.normal(-1.0, 0.5, (n, 3))).clip(0.05, 2.0)
    cases["gauss_517"] = ((c - h).astype(np.float32), (c + h).astype(np.float32))
    # boxes whose min exceeds max on one axis (the reference predicate still applies)
    n = 200
    c = rng.uniform(0, 6, (n, 3)).astype(np.float32)
    h = rng.uniform(0.1, 0.6, (n, 3)).astype(np.float32)
    mn, mx = c - h, c + h
    flip = rng.random(n) < 0.2
    mn[flip, 1], mx[flip, 1] = mx[flip, 1].copy(), mn[flip, 1].copy()
    cases["inverted_200"] = (mn, mx)
    # large magnitudes with tiny boxes (ulp-level touching)
    n = 400
    c = (rng.uniform(-1, 1, (n, 3)) * 1e4).astype(np.float32)
    c[1::2] = c[0::2]
    h = np.full((n, 3), 1e-3, np.float32)
    mn, mx = c - h, c + h
    mx[1::2, 0] = mn[0::2, 0]  # exactly touching on x
    cases["ulp_touch_400"] = (mn, mx)
    cases["single"] = (np.zeros((1, 3), np.float32), np.ones((1, 3), np.float32))
    cases["empty"] = (np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32))
    return cases


def pad4(a):
    a = f4(a)
    return np.ascontiguousarray(np.concatenate([a, np.zeros((len(a), 1), np.float32)], 1))


def make_aabb(rng, out):
    data = {}
    names = []
    for name, (mn, mx) in aabb_cases(rng).items():
        mn4, mx4 = pad4(mn), pad4(mx)
        pairs = oracle.ref_bf_aabb(mn4, mx4) if len(mn4) else np.zeros((0, 2), np.uint32)
        data[f"{name}__min"] = mn4
        data[f"{name}__max"] = mx4
        data[f"{name}__pairs"] = pairs.astype(np.uint32)
        names.append(name)
        print(f"  aabb {name}: n={len(mn4)} pairs={len(pairs)}")
    data["names"] = np.array(names)
    np.savez_compressed(out, **data)


# ------------------------------------------------------------- rigid body

def ring_shape(radius_ring, r, k=6):
    """Six particles on a ring (the demo's hexagon bodies); w = radius."""
    ang = np.arange(k) * (2 * np.pi / k)
    pos = np.zeros((10, 4), np.float32)
    pos[:k, 0] = radius_ring * np.cos(ang)
    pos[:k, 2] = radius_ring * np.sin(ang)
    pos[:k, 3] = r
    return pos


def rb_scene(rng):
    nb, per = 64, 6
    r = 0.25
    shapes = [ring_shape(0.5005, r), ring_shape(0.62, r)]
    ref_pos = np.concatenate(shapes).astype(np.float32)            # (20, 4)
    ref_mass = np.zeros(20, np.float32)
    ref_mass[:6] = 10.0 / per
    ref_mass[10:16] = 10.0 / per
    shape_inv = np.zeros((2, 12), np.float32)
    for s in range(2):
        shape_inv[s, 0] = shape_inv[s, 5] = shape_inv[s, 10] = 1.0
    nrow, spacing = 4, 1.3
    i = np.arange(nb)
    pos = np.zeros((nb, 4), np.float32)
    pos[:, 0] = ((i % nrow) - nrow / 2) * spacing
    pos[:, 2] = (((i // nrow) % nrow) - nrow / 2) * spacing
    pos[:, 1] = (i // (nrow * nrow) + 1) * spacing * 0.5
    quat = rng.uniform(-1, 1, (nb, 4)).astype(np.float32)  # raw: normalised at upload
    ang = rng.uniform(-5, 5, (nb, 4)).astype(np.float32)
    lin = np.zeros((nb, 4), np.float32)
    lin[:, :3] = rng.uniform(-1, 1, (nb, 3))
    state = {
        "pos": pos, "quat": f4(quat), "lin_vel": lin, "ang_vel": ang,
        "shape_idx": (i % 2).astype(np.int32), "p_start": (per * i).astype(np.int32),
        "n_part": np.full(nb, per, np.int32), "inv_mass": np.full(nb, 0.1, np.float32),
        "inv_inertia": np.tile(np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], np.float32), (nb, 1)),
        "ref_pos": ref_pos, "ref_mass": ref_mass, "shape_inv_inertia": shape_inv,
        "p_pos": np.zeros((nb * per, 4), np.float32), "p_vel": np.zeros((nb * per, 4), np.float32),
        "p_force": np.zeros((nb * per, 4), np.float32), "p_mass": np.zeros(nb * per, np.float32),
    }
    return state


def ref_step(R, s, dt, spM, dpM, max_vel):
    """One step in the demo's order (demoParticles.h:875-912) with the
    reference kernels; the particle pair list is the CPU sphere broadphase."""
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    nb, np_ = len(s["pos"]), len(s["p_pos"])
    R.ref_integrate(P(s["pos"]), P(s["quat"]), P(s["lin_vel"]), P(s["ang_vel"]), C.c_float(dt), nb)
    R.ref_update_particle_data(P(s["pos"]), P(s["quat"]), P(s["lin_vel"]), P(s["ang_vel"]), P(s["shape_idx"]),
                               P(s["p_start"]), P(s["n_part"]), P(s["ref_pos"]), P(s["ref_mass"]), P(s["p_pos"]),
                               P(s["p_vel"]), P(s["p_mass"]), nb)
    pairs = oracle.bf_sphere(s["p_pos"])
    both, ent = oracle.both_directions(pairs)
    both = np.ascontiguousarray(both, np.int32)
    ent = np.ascontiguousarray(ent, np.int32)
    R.ref_prepare(P(s["quat"]), P(s["shape_idx"]), P(s["shape_inv_inertia"]), P(s["inv_inertia"]), nb)
    R.ref_clear_force(P(s["p_pos"]), P(s["p_vel"]), P(s["p_mass"]), P(s["p_force"]), C.c_float(spM),
                      C.c_float(dpM), np_, C.c_float(dt))
    # the reference kernel reads pairs[pairIdx] one past a row's end; pad
    # the list so that read stays inside the buffer and never matches a row
    padded = np.concatenate([both, np.full((1, 2), -1, np.int32)])
    R.ref_pair_force(P(s["p_pos"]), P(s["p_vel"]), P(padded), P(ent), len(ent), P(s["p_mass"]), C.c_float(spM),
                     C.c_float(dpM), P(s["p_force"]), C.c_float(dt))
    R.ref_update_velocity(P(s["lin_vel"]), P(s["ang_vel"]), P(s["quat"]), P(s["inv_mass"]), P(s["inv_inertia"]),
                          P(s["shape_idx"]), P(s["p_start"]), P(s["n_part"]), P(s["ref_pos"]), P(s["p_force"]), nb,
                          C.c_float(dt), C.c_float(max_vel), 1 if max_vel > 0 else 0)
    return len(both), len(ent)


def run_rb(s, dt, spM, dpM, max_vel, steps, out):
    """The scene's initial state and its state after each reference step."""
    R = oracle.ref_lib()
    for name in ("ref_normalize_quats", "ref_integrate", "ref_update_particle_data", "ref_prepare", "ref_clear_force", "ref_pair_force",
                 "ref_update_velocity"):
        getattr(R, name).restype = None
    data = {f"init__{k}": v.copy() for k, v in s.items()}  # quaternions as uploaded (raw)
    R.ref_normalize_quats(s["quat"].ctypes.data_as(C.c_void_p), len(s["quat"]))  # setRbData
    for step in range(steps):
        npairs, nent = ref_step(R, s, dt, spM, dpM, max_vel)
        for k in ("pos", "quat", "lin_vel", "ang_vel", "p_pos", "p_vel", "p_force", "inv_inertia"):
            data[f"step{step}__{k}"] = s[k].copy()
        data[f"step{step}__npairs"] = np.int64(npairs)
        print(f"  rb step {step}: both-direction pairs={npairs} entries={nent}")
    data["params"] = np.array([dt, spM, dpM, max_vel, -5.0], np.float32)
    data["steps"] = np.int64(steps)
    np.savez_compressed(out, **data)


def make_rb(rng, out):
    run_rb(rb_scene(rng), 0.025, 2.1, 0.8, 0.25 / 0.01, 3, out)


def make_rb_demo(out):
    """The headless demo's scene (DemoParticles::init layout: hexagon bodies
    of two sizes, random orientations and spins, gsap_gb300/demo.py) with
    256 bodies packed to 0.3 of the demo's spacing so they touch from the
    first step, under the demo's step parameters, for 4 reference steps."""
    from gsap_gb300 import demo
    sc = demo.demo_scene(256, n_row=8, seed=7)
    keys = ("pos", "quat", "lin_vel", "ang_vel", "shape_idx", "p_start", "n_part", "inv_mass", "inv_inertia",
            "ref_pos", "ref_mass", "shape_inv_inertia")
    s = {k: np.ascontiguousarray(sc[k]).copy() for k in keys}
    s["pos"][:, :3] *= np.float32(0.3)
    npart = int(sc["n_particles"])
    for k in ("p_pos", "p_vel", "p_force"):
        s[k] = np.zeros((npart, 4), np.float32)
    s["p_mass"] = np.zeros(npart, np.float32)
    run_rb(s, demo.DT, demo.SP_MULTIP, demo.DP_MULTIP, demo.SMALL_RADIUS / demo.VCAP_DT, 4, out)


# ---------------------------------------------------------- 2_1024.txt dump

def make_demo_dump(ref, out):
    path = os.path.join(ref, "cudaPhysics", "2_1024.txt")
    text = open(path).read()
    frames = text.split("-------------------------------------------------------------")
    pair_re = re.compile(r"\((\d+)\t(\d+)\)\n([^\n]+)\n([^\n]+)\n([^\n]+)")
    data = {}
    nf = 0
    # a frame: pair records, "overlap pairs N", separator, entries, "pairsEntries M"
    chunks = re.split(r"overlap pairs (\d+)", text)
    # chunks: [pairs0, N0, rest0(entries0 + pairs1), N1, ...]
    prev_tail = chunks[0]
    for k in range(1, len(chunks), 2):
        n_pairs = int(chunks[k])
        recs = pair_re.findall(prev_tail)
        ij = np.array([[int(a), int(b)] for a, b, *_ in recs], np.int32).reshape(-1, 2)
        pi = np.array([[float(x) for x in r[2].split()] for r in recs], np.float32).reshape(-1, 4)
        pj = np.array([[float(x) for x in r[3].split()] for r in recs], np.float32).reshape(-1, 4)
        tail = chunks[k + 1]
        m = re.search(r"pairsEntries (\d+)", tail)
        ent_txt = tail[: m.start()] if m else ""
        ents = np.array([int(x) for x in ent_txt.replace("-", " ").split()], np.int32)
        n_ent = int(m.group(1)) if m else -1
        data[f"f{nf}__ij"] = ij
        data[f"f{nf}__pi"] = pi
        data[f"f{nf}__pj"] = pj
        data[f"f{nf}__entries"] = ents
        data[f"f{nf}__counts"] = np.array([n_pairs, n_ent], np.int32)
        prev_tail = tail[m.end():] if m else ""
        nf += 1
    data["frames"] = np.int64(nf)
    np.savez_compressed(out, **data)
    print(f"  2_1024.txt: {nf} frames")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=DEFAULT_REF)
    ap.add_argument("--only", default=None, choices=["aabb", "rb", "dump", "rb_demo"],
                    help="write one fixture (default: all)")
    a = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "liboracle.so", "ref", f"REF={a.ref}"],
                   check=True)
    rng = np.random.default_rng(20240917)
    aabb_out = os.path.join(HERE, "aabb_bf_golden.npz")
    if a.only in (None, "aabb"):
        make_aabb(rng, aabb_out)
    else:
        aabb_cases(rng)  # advances the generator as make_aabb does, for the fixtures after it
    if a.only in (None, "rb"):
        make_rb(rng, os.path.join(HERE, "rb_ref_step_golden.npz"))
    if a.only in (None, "dump"):
        make_demo_dump(a.ref, os.path.join(HERE, "demo_2_1024.npz"))
    if a.only in (None, "rb_demo"):
        make_rb_demo(os.path.join(HERE, "rb_demo_steps_golden.npz"))


if __name__ == "__main__":
    main()
