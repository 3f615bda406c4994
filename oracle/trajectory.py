"""FP64 trajectory checks of the GPU rigid-body step (test infrastructure:
used by tests/ and by bench.py as the checker, never on the measured path).

``fp64_errors`` runs the config-model step of a ``ParticleRigidBody`` handle
on the GPU against ``rb_step_cfg_f64`` (oracle/rb.c) from the same initial
state in two ways:

* re-synced: before every GPU step the body state is set to the FP64
  oracle's state rounded to FP32 (``gsap_rb_set_state``) and the oracle
  takes its step from that same rounded state, so each step is compared
  from identical input -- the per-step error of the FP32 step;
* free-running: the GPU steps on its own FP32 state for all the steps and
  its final state is compared with the oracle's -- the trajectory error.

Errors are max |gpu - fp64| / max |fp64| over the xyz components of the
checked bodies.  For batched scenes the oracle can run on the first
``check_scenes`` scenes only: scenes never interact, so the oracle's result
for them equals the one it would give on the whole batch.

Contact onset is discontinuous in this model: the damping term eta (v.n) n
switches on with the contact, so a particle pair whose penetration depth is
within the FP32 rounding of the contact geometry can be in contact on one
side and not on the other, and the velocity of its two bodies then differs
by eta |v.n| dt / m in that step -- a model property, not an arithmetic
error.
The per-step error is therefore taken over the bodies with no contact
within +-band of zero penetration (band = 8 FP32 ulps of the box extent),
and the number of bodies left out is reported with it; the error over all
bodies is reported as well.
"""
from __future__ import annotations

import numpy as np

from . import rb_step_cfg_f64

KEYS = ("pos", "quat", "lin_vel", "ang_vel")


def _rel(a, b, mask=None):
    a = np.asarray(a, np.float64)[:, :3]
    b = np.asarray(b, np.float64)[:, :3]
    d = np.abs(a - b)
    if mask is not None:
        d = d[mask]
    if d.size == 0:
        return 0.0
    return float(d.max() / max(np.abs(b).max(), 1e-30))


def onset_band(params: dict) -> float:
    """8 FP32 ulps of the largest box coordinate."""
    ext = max(max(abs(x) for x in params["box_lo"]), max(abs(x) for x in params["box_hi"]), 1.0)
    return 8.0 * ext * 2.0 ** -23


def checked_subset(sc: dict, check_scenes: int | None):
    """(oracle state dict in FP64, number of checked bodies): all bodies, or
    the bodies of the first check_scenes scenes of a batched scene dict."""
    from gsap_gb300 import scenes
    if check_scenes is None or "body_offsets" not in sc:
        return scenes.to_f64(sc), len(sc["pos"])
    nb = int(sc["body_offsets"][check_scenes])
    sub = scenes.subset_bodies(sc, 0, nb)
    sub["scene"] = np.ascontiguousarray(sc["scene"][:nb])
    return scenes.to_f64(sub), nb


def fp64_errors(prb, sap, sc: dict, params: dict, steps: int = 100, check_scenes: int | None = None,
                stream=None) -> dict:
    """Per-step (re-synced) and free-running errors of `steps` GPU steps
    against the FP64 oracle; prb must hold the scene `sc` (loaded, contact
    model and scenes set).  Leaves prb at the end of the re-synced run."""
    import torch
    dt = params["dt"]
    band = onset_band(params)
    init = {k: np.ascontiguousarray(sc[k], np.float32).copy() for k in KEYS}
    # free-running GPU trajectory
    prb.set_state(init)
    for _ in range(steps):
        prb.step(sap, dt, stream=stream)
    torch.cuda.synchronize()
    sap.check()
    free = prb.get_state()
    # Re-synced run: before every step the GPU state is set to the oracle's
    # state rounded to FP32, and the oracle steps from that same rounded
    # state, so the two compute one step from identical input; a separate
    # oracle trajectory, never rounded, is the reference of the free run.
    st_sync, nb = checked_subset(sc, check_scenes)
    st_true, _ = checked_subset(sc, check_scenes)
    prb.set_state(init)
    per = {"pos": [], "lin_vel": [], "ang_vel": []}
    per_all = {"pos": [], "lin_vel": [], "ang_vel": []}
    left_out = []
    worst = {}
    for step in range(steps):
        cur = prb.get_state()
        for k in KEYS:
            r = st_sync[k].astype(np.float32)
            cur[k][:nb] = r
            st_sync[k][...] = r.astype(np.float64)
        prb.set_state(cur)
        prb.step(sap, dt, stream=stream)
        amb = rb_step_cfg_f64(st_sync, params, band=band)
        rb_step_cfg_f64(st_true, params)
        got = prb.get_state()
        keep = amb == 0
        left_out.append(int(nb - keep.sum()))
        for k in per:
            e = _rel(got[k][:nb], st_sync[k], keep)
            per[k].append(e)
            per_all[k].append(_rel(got[k][:nb], st_sync[k]))
            if e >= max(per[k]):
                d = np.abs(np.asarray(got[k][:nb], np.float64)[:, :3] - st_sync[k][:, :3]).max(1)
                d[~keep] = 0.0
                b = int(np.argmax(d))
                worst[k] = {"step": step, "body": b, "abs_err": float(d[b]),
                            "max_abs_ref": float(np.abs(st_sync[k][:, :3]).max()),
                            "body_abs_ref": float(np.abs(st_sync[k][b, :3]).max())}
    st64 = st_true
    sap.check()
    return {"steps": steps, "checked_bodies": nb, "onset_band": band,
            "per_step_max": {k: max(v) for k, v in per.items()},
            "per_step_max_all_bodies": {k: max(v) for k, v in per_all.items()},
            "bodies_left_out_max": max(left_out), "bodies_left_out_mean": float(np.mean(left_out)),
            "per_step": per, "worst": worst,
            "free_running": {k: _rel(free[k][:nb], st64[k]) for k in ("pos", "lin_vel", "ang_vel")}}
