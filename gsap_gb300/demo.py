"""Headless demo driver: the particle rigid-body scene of the reference's
DemoParticles::init (cudaPhysics/demoParticles.h:175-414) stepped in the
order of DemoParticles::step (:856-928), without the GLUT window and the GL
buffer export, plus binary snapshots of the state.

Scene: num_bodies bodies on an n_row x n_row grid, stacked in layers, 3.6
apart; random orientations and angular velocities; two six-particle hexagon
shapes in the body's xy plane alternating by index (particle radius 0.25 at
spacing 2r*1.001, and the same shape scaled by 1.2); body mass 10; diagonal
inertia from the reference's 1/12 (2r)^2 2m 0.2 rule.  Reference contact
model, dt = 0.025, spring/damping multipliers 2.1 / 0.8, velocity cap
0.25 / 0.01.  The reference draws its random numbers with rand(); here they
come from a seeded numpy generator.

    python -m gsap_gb300.demo --steps 200 --snapshot-out state.npz
"""
from __future__ import annotations

import argparse
import time

import numpy as np

from .scenes import MAXP

DT = 0.025
SP_MULTIP, DP_MULTIP = 2.1, 0.8
SMALL_RADIUS, VCAP_DT = 0.25, 0.01
RB_MASS = 10.0
SPACING = 3.6
PARTICLES = 6

_STATE = ("pos", "quat", "lin_vel", "ang_vel")
_STATIC = ("shape_idx", "p_start", "n_part", "inv_mass", "inv_inertia", "ref_pos", "ref_mass",
           "shape_inv_inertia")


def _hexagon(spacing: float) -> np.ndarray:
    s3 = np.sqrt(3.0) / 2.0
    return np.array([[-1, 0], [-0.5, s3], [0.5, s3], [1, 0], [0.5, -s3], [-0.5, -s3]]) * spacing


def demo_scene(num_bodies: int = 4096, n_row: int = 16, seed: int = 0) -> dict:
    """Scene dict in the layout ParticleRigidBody.load_scene takes."""
    rng = np.random.default_rng(seed)
    r = 0.25
    ps = r * 2 * 1.001
    ref_pos = np.zeros((2 * MAXP, 4), np.float32)
    ref_mass = np.zeros(2 * MAXP, np.float32)
    for s, scale in enumerate((1.0, 1.2)):
        ref_pos[s * MAXP:s * MAXP + PARTICLES, :2] = _hexagon(ps * scale)
        ref_pos[s * MAXP:s * MAXP + PARTICLES, 3] = r * scale
        ref_mass[s * MAXP:s * MAXP + PARTICLES] = RB_MASS / PARTICLES
    inertia = 1.0 / 12.0 * (2 * r) ** 2 * 2 * RB_MASS * 0.2
    shape_inv = np.zeros((2, 12), np.float32)
    for s, k in enumerate((1.0, 2.0)):
        for row in range(3):
            shape_inv[s, 4 * row + row] = 1.0 / (k * inertia)
    i = np.arange(num_bodies)
    pos = np.zeros((num_bodies, 4), np.float32)
    pos[:, 0] = ((i % n_row) - n_row // 2) * SPACING
    pos[:, 2] = (((i // n_row) % n_row) - n_row // 2) * SPACING
    pos[:, 1] = (i // (n_row * n_row) + 1) * SPACING
    inv_i = np.zeros((num_bodies, 12), np.float32)
    for row in range(3):
        inv_i[:, 4 * row + row] = 1.0
    return {
        "pos": pos,
        "quat": rng.uniform(-1.0, 1.0, (num_bodies, 4)).astype(np.float32),  # normalised on upload
        "lin_vel": np.zeros((num_bodies, 4), np.float32),
        "ang_vel": rng.uniform(-5.0, 5.0, (num_bodies, 4)).astype(np.float32),
        "shape_idx": (i % 2).astype(np.int32),
        "p_start": (PARTICLES * i).astype(np.int32),
        "n_part": np.full(num_bodies, PARTICLES, np.int32),
        "inv_mass": np.full(num_bodies, 1.0 / RB_MASS, np.float32),
        "inv_inertia": inv_i,
        "ref_pos": ref_pos,
        "ref_mass": ref_mass,
        "shape_inv_inertia": shape_inv,
        "n_particles": PARTICLES * num_bodies,
    }


def save_snapshot(path, scene: dict, state: dict | None = None, step: int = 0) -> None:
    """Binary snapshot: the static scene arrays, the body state (the scene's
    own unless `state` -- e.g. ParticleRigidBody.get_state() -- is given) and
    the step count."""
    arrs = {k: np.asarray(scene[k]) for k in _STATIC}
    src = state if state is not None else scene
    arrs.update({k: np.asarray(src[k], np.float32) for k in _STATE})
    np.savez(path, step=np.int64(step), n_particles=np.int64(scene["n_particles"]), **arrs)


def load_snapshot(path) -> tuple[dict, int]:
    """Scene dict (static data + saved body state) and the step count."""
    z = np.load(path)
    scene = {k: z[k] for k in _STATIC + _STATE}
    scene["n_particles"] = int(z["n_particles"])
    return scene, int(z["step"])


class Demo:
    """The demo's rigid-body system and sphere broadphase on the GPU."""

    def __init__(self, scene: dict, max_pairs_per_particle: int = 32):
        from . import MODE_SPHERE
        from .rigid import ParticleRigidBody
        from .sap import Sap
        nb, npart = len(scene["pos"]), int(scene["n_particles"])
        self.system = ParticleRigidBody(nb, npart, max_pairs_per_particle * npart)
        self.system.load_scene(scene)
        self.system.set_params(SP_MULTIP, DP_MULTIP)
        self.system.set_max_velocity(SMALL_RADIUS, VCAP_DT)
        self.sap = Sap(npart, mode=MODE_SPHERE)
        self.scene = scene
        self.steps = 0

    def run(self, steps: int, stream=None) -> None:
        for _ in range(steps):
            self.system.step(self.sap, DT, stream=stream)
        self.steps += steps

    def state(self) -> dict:
        return self.system.get_state()


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--bodies", type=int, default=4096)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--snapshot-in", default=None, help="start from a saved snapshot")
    ap.add_argument("--snapshot-out", default=None, help="save the final state here")
    args = ap.parse_args(argv)
    import torch
    if args.snapshot_in:
        scene, step0 = load_snapshot(args.snapshot_in)
    else:
        scene, step0 = demo_scene(args.bodies, seed=args.seed), 0
    demo = Demo(scene)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    demo.run(args.steps)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / max(args.steps, 1)
    demo.sap.check()
    st = demo.state()
    print(f"{len(scene['pos'])} bodies, {scene['n_particles']} particles: {args.steps} steps, "
          f"{dt * 1e3:.3f} ms/step, mean height {st['pos'][:, 1].mean():.3f}")
    if args.snapshot_out:
        save_snapshot(args.snapshot_out, scene, st, step0 + args.steps)


if __name__ == "__main__":
    main()
