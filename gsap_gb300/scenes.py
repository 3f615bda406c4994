"""Seeded synthetic scenes with the statistics of the benchmark workloads.

No public dataset is involved: every input is generated here from a seed.

* ``aabb_uniform``  16,384-AABB case: centres U[0,100]^3, half-extents
  U[0.1,0.5] per axis.
* ``aabb_gauss``    1,048,576-AABB case: centres R (g * (100, 20, 5)), g ~
  N(0, I), R a seeded Haar rotation; half-extents exp(N(-1, 0.5^2)) clipped
  to [0.05, 2]; ``jitter`` moves centres by N(0, 0.05^2) between calls.
* ``batched_aabb``  4096 scenes, sizes log-uniform in [64, 65536], per-scene
  std U[5,100]^3 and rotation, half-extents as the uniform case.
* ``cubes_in_box``  rigid cubes of 2x2x2 particles (r = 0.5, offsets
  +-0.5) at uniform random poses inside a walled box.
* ``mixed_scenes``  batched dynamics: scenes of 2x2x2 cubes, 4x1x1 rods and
  3-particle L shapes, body counts log-uniform in [256, 8192].

Rigid-body state uses the reference's layout (ParticleRigidBody.h:52-78):
float4 pos / quat (x, y, z, w) / velocities, per-body shape index, particle
start offset and count, inverse mass, 12-float inverse inertia; per shape up
to 10 reference particles (w = radius) and a 12-float inverse inertia.
"""
from __future__ import annotations

import numpy as np

MAXP = 10  # MAX_NUM_PARTICLES


def haar_rotation(rng) -> np.ndarray:
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def _pad4(a):
    a = np.asarray(a, np.float32)
    return np.ascontiguousarray(np.concatenate([a, np.zeros((len(a), 1), np.float32)], 1))


def aabb_uniform(n: int = 16384, seed: int = 0):
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.0, 100.0, (n, 3)).astype(np.float32)
    h = rng.uniform(0.1, 0.5, (n, 3)).astype(np.float32)
    return _pad4(c - h), _pad4(c + h)


def aabb_gauss_parts(n: int = 1 << 20, seed: int = 0, std=(100.0, 20.0, 5.0)):
    rng = np.random.default_rng(seed)
    R = haar_rotation(rng)
    c = (rng.standard_normal((n, 3)) * np.asarray(std)) @ R.T
    h = np.exp(rng.normal(-1.0, 0.5, (n, 3))).clip(0.05, 2.0)
    return c.astype(np.float32), h.astype(np.float32), R


def aabb_gauss(n: int = 1 << 20, seed: int = 0):
    c, h, _ = aabb_gauss_parts(n, seed)
    return _pad4(c - h), _pad4(c + h)


def jitter(c: np.ndarray, seed: int, sigma: float = 0.05) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return (c + rng.normal(0.0, sigma, c.shape)).astype(np.float32)


def batched_sizes(S: int = 4096, seed: int = 0, lo: int = 64, hi: int = 65536) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.round(np.exp(rng.uniform(np.log(lo), np.log(hi), S))).astype(np.int64)


def batched_aabb(S: int = 4096, seed: int = 0, lo: int = 64, hi: int = 65536):
    """Returns (mn, mx, offsets) with offsets of length S+1 (int64)."""
    rng = np.random.default_rng(seed)
    sizes = batched_sizes(S, seed, lo, hi)
    off = np.zeros(S + 1, np.int64)
    off[1:] = np.cumsum(sizes)
    n = int(off[-1])
    mn = np.empty((n, 4), np.float32)
    mx = np.empty((n, 4), np.float32)
    for s in range(S):
        m = int(sizes[s])
        std = rng.uniform(5.0, 100.0, 3)
        R = haar_rotation(rng)
        c = (rng.standard_normal((m, 3)) * std) @ R.T
        h = rng.uniform(0.1, 0.5, (m, 3))
        a, b = off[s], off[s + 1]
        mn[a:b, :3] = c - h
        mx[a:b, :3] = c + h
    mn[:, 3] = 0.0
    mx[:, 3] = 0.0
    return mn, mx, off


# ------------------------------------------------------------------ bodies

def _shape_cube(r=0.5):
    o = np.array([[x, y, z] for x in (-0.5, 0.5) for y in (-0.5, 0.5) for z in (-0.5, 0.5)])
    return o, r


def _shape_rod(r=0.5):
    return np.array([[x, 0.0, 0.0] for x in (-1.5, -0.5, 0.5, 1.5)]), r


def _shape_l(r=0.5):
    o = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])
    return o - o.mean(0), r


def _shape_tables(shapes, pmass=1.0):
    ns = len(shapes)
    ref_pos = np.zeros((MAXP * ns, 4), np.float32)
    ref_mass = np.zeros(MAXP * ns, np.float32)
    inv_i = np.zeros((ns, 12), np.float32)
    inv_i64 = np.zeros((ns, 9), np.float64)
    counts, masses = [], []
    for s, (off, r) in enumerate(shapes):
        k = len(off)
        ref_pos[MAXP * s:MAXP * s + k, :3] = off
        ref_pos[MAXP * s:MAXP * s + k, 3] = r
        ref_mass[MAXP * s:MAXP * s + k] = pmass
        I = np.zeros((3, 3))
        for p in off:
            I += pmass * (np.dot(p, p) * np.eye(3) - np.outer(p, p)) + 0.4 * pmass * r * r * np.eye(3)
        Ii = np.linalg.inv(I)
        inv_i64[s] = Ii.reshape(-1)
        for row in range(3):
            inv_i[s, 4 * row:4 * row + 3] = Ii[row]
        counts.append(k)
        masses.append(pmass * k)
    return ref_pos, ref_mass, inv_i, inv_i64, np.array(counts), np.array(masses)


def _random_quats(rng, n):
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return q.astype(np.float32)


def _bodies(shape_idx, counts, masses, pos, quat, inv_i, tables, scene=None):
    nb = len(shape_idx)
    npart = counts[shape_idx].astype(np.int32)
    pstart = np.zeros(nb, np.int32)
    pstart[1:] = np.cumsum(npart)[:-1]
    ref_pos, ref_mass, shape_inv, shape_inv64 = tables
    out = {
        "pos": _pad4(pos), "quat": np.ascontiguousarray(quat, np.float32),
        "lin_vel": np.zeros((nb, 4), np.float32), "ang_vel": np.zeros((nb, 4), np.float32),
        "shape_idx": shape_idx.astype(np.int32), "p_start": pstart, "n_part": npart,
        "inv_mass": (1.0 / masses[shape_idx]).astype(np.float32),
        "inv_inertia": np.ascontiguousarray(shape_inv[shape_idx]),
        "ref_pos": ref_pos, "ref_mass": ref_mass, "shape_inv_inertia": shape_inv,
        "shape_inv_inertia64": shape_inv64, "n_particles": int(npart.sum()),
    }
    if scene is not None:
        out["scene"] = scene.astype(np.int32)
    return out


def cubes_in_box(nb: int = 65536, box: float = 200.0, seed: int = 0):
    """2x2x2-particle cubes at uniform random poses inside [0, box]^3."""
    rng = np.random.default_rng(seed)
    ref_pos, ref_mass, inv_i, inv_i64, counts, masses = _shape_tables([_shape_cube()])
    margin = 1.5
    pos = rng.uniform(margin, box - margin, (nb, 3))
    return _bodies(np.zeros(nb, np.int64), counts, masses, pos, _random_quats(rng, nb), inv_i,
                   (ref_pos, ref_mass, inv_i, inv_i64))


def mixed_scenes(S: int = 1024, seed: int = 0, lo: int = 256, hi: int = 8192, box: float = 100.0):
    """Batched dynamics: per scene, bodies of three shapes mixed uniformly."""
    rng = np.random.default_rng(seed)
    sizes = np.round(np.exp(rng.uniform(np.log(lo), np.log(hi), S))).astype(np.int64)
    ref_pos, ref_mass, inv_i, inv_i64, counts, masses = _shape_tables([_shape_cube(), _shape_rod(), _shape_l()])
    nb = int(sizes.sum())
    shape_idx = rng.integers(0, 3, nb)
    margin = 2.5
    pos = rng.uniform(margin, box - margin, (nb, 3))
    scene = np.repeat(np.arange(S), sizes)
    out = _bodies(shape_idx, counts, masses, pos, _random_quats(rng, nb), inv_i,
                  (ref_pos, ref_mass, inv_i, inv_i64), scene)
    off = np.zeros(S + 1, np.int64)
    off[1:] = np.cumsum(sizes)
    out["body_offsets"] = off
    return out


def body_aabbs(sc: dict):
    """Body AABBs of a rigid-body scene dict at its current pose (particle
    centres x + R(q) ref, +/- radius), as (n, 4) float32 min / max arrays:
    the broadphase input of the config-model step, for tuning a body
    broadphase handle (Sap.autotune) before stepping."""
    q = np.asarray(sc["quat"], np.float64)
    q = q / np.linalg.norm(q, axis=1, keepdims=True)
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    R = np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], 1),
                  np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], 1),
                  np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], 1)], 1)
    pos = np.asarray(sc["pos"], np.float64)[:, :3]
    ref = np.asarray(sc["ref_pos"], np.float64)
    shape = np.asarray(sc["shape_idx"], np.int64)
    npart = np.asarray(sc["n_part"], np.int64)
    n = len(pos)
    lo = np.full((n, 3), np.inf)
    hi = np.full((n, 3), -np.inf)
    for k in range(int(npart.max()) if n else 0):
        m = npart > k
        rk = ref[shape[m] * MAXP + k]
        c = pos[m] + np.einsum("bij,bj->bi", R[m], rk[:, :3])
        lo[m] = np.minimum(lo[m], c - rk[:, 3:4])
        hi[m] = np.maximum(hi[m], c + rk[:, 3:4])
    mn = np.zeros((n, 4), np.float32)
    mx = np.zeros((n, 4), np.float32)
    mn[:, :3] = lo
    mx[:, :3] = hi
    return mn, mx


def subset_bodies(sc: dict, a: int, z: int) -> dict:
    """Bodies [a, z) of a scene dict as a scene of their own (particle
    starts re-based; shape tables shared)."""
    out = {k: np.ascontiguousarray(sc[k][a:z]) for k in ("pos", "quat", "lin_vel", "ang_vel", "shape_idx",
                                                          "n_part", "inv_mass", "inv_inertia")}
    ps = np.zeros(z - a, np.int32)
    ps[1:] = np.cumsum(out["n_part"])[:-1]
    out["p_start"] = ps
    for k in ("ref_pos", "ref_mass", "shape_inv_inertia", "shape_inv_inertia64"):
        out[k] = sc[k]
    out["n_particles"] = int(out["n_part"].sum())
    return out


def to_f64(sc: dict) -> dict:
    """State dict for the FP64 oracle (oracle.rb_step_cfg_f64)."""
    nb, np_ = len(sc["pos"]), sc["n_particles"]
    d = {k: np.ascontiguousarray(sc[k], np.float64) for k in ("pos", "quat", "lin_vel", "ang_vel", "inv_mass")}
    d.update({k: np.ascontiguousarray(sc[k], np.int32) for k in ("shape_idx", "p_start", "n_part")})
    d["ref_pos"] = np.ascontiguousarray(sc["ref_pos"], np.float64)
    d["shape_inv_inertia"] = np.ascontiguousarray(sc["shape_inv_inertia64"], np.float64)
    d["scene"] = np.ascontiguousarray(sc["scene"], np.int32) if "scene" in sc else None
    for k in ("p_pos", "p_vel", "p_force"):
        d[k] = np.zeros((np_, 4), np.float64)
    assert len(d["pos"]) == nb
    return d
