"""Host-side mirror of the reference's ``ParticleRigidBody`` class
(ParticleRigidBody/ParticleRigidBody.h:46-164).

Method names follow the reference (setRbData -> set_rb_data,
comupteFoceOnParticles -> compute_forces, ...); every call goes through the
C ABI of libgsap.so.  ``step`` is the whole reference-order step
(cudaPhysics/demoParticles.h:875-912) with the broadphase of a ``Sap``
handle, without host synchronisation.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from ._lib import CONTACT_CONFIG, CONTACT_REF, BodyData, ContactParams, GsapError, check, last_error, load
from .sap import _stream_ptr


def _host(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


class ParticleRigidBody:
    def __init__(self, max_bodies: int, max_particles: int, max_pairs: int):
        self._h = load().gsap_rb_create(max_bodies, max_particles, max_pairs)
        if not self._h:
            raise GsapError(3, last_error())
        self.max_bodies, self.max_particles, self.max_pairs = max_bodies, max_particles, max_pairs
        self.cp = ContactParams()
        self.cp.model = CONTACT_REF
        self.cp.sp_multip, self.cp.dp_multip = 0.5, 0.25
        self.cp.gravity_y = -5.0
        self.cp.floor_clamp = 1
        self.cp.torque_quirk = 1
        self.n_bodies = 0
        self.n_particles = 0

    def close(self):
        if getattr(self, "_h", None):
            load().gsap_rb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # ------------------------------------------------------------ uploads
    def set_rb_data(self, d: dict):
        """setRbData: dict of host arrays (pos, quat, lin_vel, ang_vel float4;
        shape_idx, p_start, n_part int; inv_mass; inv_inertia 12 floats)."""
        keep = {k: _host(d[k], np.float32) for k in ("pos", "quat", "lin_vel", "ang_vel", "inv_mass", "inv_inertia")}
        keep.update({k: _host(d[k], np.int32) for k in ("shape_idx", "p_start", "n_part")})
        bd = BodyData()
        bd.n_bodies = len(keep["pos"])
        bd.n_total_particles = int(keep["n_part"].sum()) if "n_particles" not in d else int(d["n_particles"])
        for k, v in keep.items():
            setattr(bd, k, v.ctypes.data)
        check(load().gsap_rb_set_body_data(self._h, C.byref(bd)))
        self.n_bodies, self.n_particles = bd.n_bodies, bd.n_total_particles

    def set_particle_data(self, ref_pos, mass):
        rp, m = _host(ref_pos, np.float32), _host(mass, np.float32)
        check(load().gsap_rb_set_particle_data(self._h, rp.ctypes.data, m.ctypes.data, len(rp)))

    def set_particle_shape_inv_inertia(self, inv, n_shapes=None):
        a = _host(inv, np.float32).reshape(-1, 12)
        check(load().gsap_rb_set_shape_inv_inertia(self._h, a.ctypes.data, n_shapes or len(a)))

    def set_params(self, sp_multip: float, dp_multip: float):
        self.cp.sp_multip, self.cp.dp_multip = sp_multip, dp_multip
        check(load().gsap_rb_set_contact(self._h, C.byref(self.cp)))

    def set_max_velocity(self, min_radius: float, dt: float):
        self.cp.max_lin_vel = min_radius / dt
        check(load().gsap_rb_set_contact(self._h, C.byref(self.cp)))

    def set_contact(self, **kw):
        for k, v in kw.items():
            if k in ("box_lo", "box_hi"):
                arr = getattr(self.cp, k)
                for i in range(3):
                    arr[i] = float(v[i])
            else:
                setattr(self.cp, k, v)
        check(load().gsap_rb_set_contact(self._h, C.byref(self.cp)))

    def set_scenes(self, body_offsets):
        off = _host(body_offsets, np.uint32)
        check(load().gsap_rb_set_scenes(self._h, off.ctypes.data, len(off) - 1))

    def load_scene(self, sc: dict):
        self.set_particle_data(sc["ref_pos"], sc["ref_mass"])
        self.set_particle_shape_inv_inertia(sc["shape_inv_inertia"])
        self.set_rb_data(sc)

    # --------------------------------------------------------- the steps
    def update_particle_data(self, stream=None):
        check(load().gsap_rb_update_particle_data(self._h, C.c_void_p(_stream_ptr(stream))))

    def prepare(self, stream=None):
        check(load().gsap_rb_prepare(self._h, C.c_void_p(_stream_ptr(stream))))

    def compute_forces(self, dt: float, stream=None):
        check(load().gsap_rb_compute_forces(self._h, C.c_float(dt), C.c_void_p(_stream_ptr(stream))))

    def update_velocity(self, dt: float, stream=None):
        check(load().gsap_rb_update_velocity(self._h, C.c_float(dt), C.c_void_p(_stream_ptr(stream))))

    def integrate(self, dt: float, stream=None):
        check(load().gsap_rb_integrate(self._h, C.c_float(dt), C.c_void_p(_stream_ptr(stream))))

    def step(self, sap, dt: float, stream=None):
        check(load().gsap_rb_step(self._h, sap.handle, C.c_float(dt), C.c_void_p(_stream_ptr(stream))))

    # ---------------------------------------------------------- pair list
    def set_num_pairs(self, num_pairs: int, num_entries: int):
        check(load().gsap_rb_set_num_pairs(self._h, num_pairs, num_entries))

    def copy_out(self, which: int, shape, dtype=np.float32) -> np.ndarray:
        """Host copy of a handle-owned array (GSAP_RB_* index)."""
        out = np.empty(shape, dtype)
        check(load().gsap_rb_copy_out(self._h, which, out.ctypes.data, out.nbytes, None))
        return out

    def copy_in(self, which: int, arr):
        a = np.ascontiguousarray(arr)
        check(load().gsap_rb_copy_in(self._h, which, a.ctypes.data, a.nbytes, None))

    def get_state(self, stream=None) -> dict:
        nb = self.n_bodies
        arrs = {k: np.empty((nb, 4), np.float32) for k in ("pos", "quat", "lin_vel", "ang_vel")}
        check(load().gsap_rb_get_state(self._h, arrs["pos"].ctypes.data, arrs["quat"].ctypes.data,
                                       arrs["lin_vel"].ctypes.data, arrs["ang_vel"].ctypes.data,
                                       C.c_void_p(_stream_ptr(stream))))
        return arrs

    def set_state(self, st: dict, stream=None):
        """gsap_rb_set_state: body pos / quat / lin_vel / ang_vel (n_bodies x 4
        float32, any key may be absent) written bit for bit, no
        normalisation."""
        arrs = {k: (_host(st[k], np.float32) if st.get(k) is not None else None)
                for k in ("pos", "quat", "lin_vel", "ang_vel")}
        for k, a in arrs.items():
            if a is not None and a.shape != (self.n_bodies, 4):
                raise ValueError(f"{k} must have shape ({self.n_bodies}, 4)")
        check(load().gsap_rb_set_state(self._h, *[a.ctypes.data if a is not None else None for a in arrs.values()],
                                       C.c_void_p(_stream_ptr(stream))))

    def contacts(self, reset: bool = False, stream=None) -> int:
        """Particle-particle contacts counted by the config-model force
        kernel since creation or the last reset (both sides counted)."""
        out = C.c_uint64(0)
        if load().gsap_debug_rb_contacts(self._h, C.byref(out), int(reset), C.c_void_p(_stream_ptr(stream))) != 0:
            raise GsapError(3, "contact counter read failed")
        return int(out.value)

    def get_particles(self) -> dict:
        np_ = self.n_particles
        return {"p_pos": self.copy_out(0, (np_, 4)), "p_vel": self.copy_out(1, (np_, 4)),
                "p_force": self.copy_out(2, (np_, 4))}
