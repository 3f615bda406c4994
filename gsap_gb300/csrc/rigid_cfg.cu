// Particle rigid-body step, config model (FP32 state).
//
// The contact model of the 65,536-cube and batched scenes: linear spring k
// on the penetration, normal damping eta, tangential damping kt * eta, six
// walls of an axis-aligned box, gravity along y.  For a particle i and a
// contact partner j (a particle, or a wall seen as a fixed particle):
//   n = (p_j - p_i) / |p_j - p_i|,  pen = r_i + r_j - |p_j - p_i|,
//   v = v_j - v_i,  f_i += -k pen n + eta (v.n) n + kt eta (v - (v.n) n).
// The step order is the reference's (cudaPhysics/demoParticles.h:875-912):
// integrate, place particles, broadphase, forces, velocity update; the
// velocity update uses I_w^-1 = R I_shape^-1 R^T (prepareK,
// ParticleRigidBodyKernel.h:30-45) rather than the reference's
// angVel += tau dt (:260-261).
//
// Kernels: one thread per particle for placement and forces (each particle
// gathers from the particles of the bodies that overlap its own body, in
// neighbour-id order, and writes its force once, no read-modify-write); one
// thread per body for the body AABB and for the compensated (two-sum)
// per-body force / torque reduction fused with the velocity update.
//
// Precision: a body position is a float-float pair x = hi + lo (hi is the
// FP32 position the caller sees, lo the rounding error that the FP32 update
// x += v dt leaves, carried from step to step; lo = 0 after the caller sets
// a position), and particles are kept as body-relative offsets r = R ref
// (|r| <= a few units).  A particle-particle vector is formed as
// (hi_b - hi_a) + (lo_b - lo_a) + (r_j - r_i): the difference of the high
// parts is exact for touching bodies (Sterbenz), so the penetration depth
// keeps ~1e-7 absolute accuracy.  With plain FP32 positions near 100 the
// rounding of every position update alone moves a contact by up to half an
// ulp (~4e-6), which the stiff spring turns into a force error of k * 4e-6
// -- several times the 1e-5 relative velocity error allowed per step.
// Absolute particle positions are produced only when the caller reads them.
#include "internal.cuh"
#include "rigid.cuh"

namespace gsap {

__device__ __forceinline__ void qrows(float4 q, float3 r[3]) {
    float x = q.x, y = q.y, z = q.z, w = q.w;
    r[0] = make_float3(1.f - 2.f * (y * y + z * z), 2.f * (x * y - w * z), 2.f * (x * z + w * y));
    r[1] = make_float3(2.f * (x * y + w * z), 1.f - 2.f * (x * x + z * z), 2.f * (y * z - w * x));
    r[2] = make_float3(2.f * (x * z - w * y), 2.f * (y * z + w * x), 1.f - 2.f * (x * x + y * y));
}
__device__ __forceinline__ float3 mv(const float3 r[3], float3 v) {
    return make_float3(r[0].x * v.x + r[0].y * v.y + r[0].z * v.z, r[1].x * v.x + r[1].y * v.y + r[1].z * v.z,
                       r[2].x * v.x + r[2].y * v.y + r[2].z * v.z);
}
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// (hi, lo) += d, renormalised so that hi = fl(hi + lo): two-sum of hi and d,
// the error joined to lo, then a fast two-sum (|s| >= |l| up to rounding
// for any |lo| < ulp(hi)).
__device__ __forceinline__ void ff_add(float& hi, float& lo, float d) {
    const float s = __fadd_rn(hi, d);
    const float bb = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(d, bb));
    const float l = __fadd_rn(lo, e);
    hi = __fadd_rn(s, l);
    lo = __fsub_rn(l, __fsub_rn(hi, s));
}

__global__ void k_integrate_cfg(float4* pos, float4* pos_lo, float4* quat, float4* lin, const float4* ang,
                                CfgParams p, int n) {
    pdl_wait();
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    float4 v = lin[b];
    v.y += p.gy * p.dt;
    lin[b] = v;
    float4 q = quat[b], w = ang[b];
    // (w, 0) (x) q = (q.w w + w x q_v, -w . q_v)
    float dx = q.w * w.x + (w.y * q.z - w.z * q.y);
    float dy = q.w * w.y + (w.z * q.x - w.x * q.z);
    float dz = q.w * w.z + (w.x * q.y - w.y * q.x);
    float dw = -(w.x * q.x + w.y * q.y + w.z * q.z);
    float h = 0.5f * p.dt;
    q.x += h * dx; q.y += h * dy; q.z += h * dz; q.w += h * dw;
    float il = rsqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    q.x *= il; q.y *= il; q.z *= il; q.w *= il;
    quat[b] = q;
    float4 x = pos[b];
    if (pos_lo) {
        float4 l = pos_lo[b];
        ff_add(x.x, l.x, v.x * p.dt);
        ff_add(x.y, l.y, v.y * p.dt);
        ff_add(x.z, l.z, v.z * p.dt);
        pos_lo[b] = l;
    } else {
        x.x += v.x * p.dt; x.y += v.y * p.dt; x.z += v.z * p.dt;
    }
    pos[b] = x;
}

__global__ void k_place_cfg(const float4* quat, const float4* lin, const float4* ang, const int* shape,
                            const int* pstart, const int* p_body, const float4* ref_pos, float4* p_rel,
                            float4* p_vel, int np) {
    pdl_wait();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    int b = p_body[i];
    float4 ref = ref_pos[kMaxParticlesPerBody * shape[b] + (i - pstart[b])];
    float3 R[3];
    qrows(quat[b], R);
    float3 r = mv(R, make_float3(ref.x, ref.y, ref.z));
    float4 v = lin[b], w = ang[b];
    float3 wr = cross3(make_float3(w.x, w.y, w.z), r);
    p_rel[i] = make_float4(r.x, r.y, r.z, ref.w);
    p_vel[i] = make_float4(v.x + wr.x, v.y + wr.y, v.z + wr.z, 0.f);
}

// absolute particle positions (readback only): hi + (lo + r)
__global__ void k_abs_pos(const float4* pos, const float4* pos_lo, const int* p_body, const float4* p_rel,
                          float4* p_pos, int np) {
    pdl_wait();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const int b = p_body[i];
    float4 x = pos[b], l = pos_lo[b], r = p_rel[i];
    p_pos[i] = make_float4(x.x + (l.x + r.x), x.y + (l.y + r.y), x.z + (l.z + r.z), r.w);
}

__global__ void k_body_aabb(const float4* pos, const float4* pos_lo, const float4* p_rel, const int* pstart,
                            const int* npart, float4* bmin, float4* bmax, int n) {
    pdl_wait();
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    int s = pstart[b], m = npart[b];
    const float4 x = pos[b], xl = pos_lo[b];
    float3 lo = make_float3(INFINITY, INFINITY, INFINITY), hi = make_float3(-INFINITY, -INFINITY, -INFINITY);
    for (int k = 0; k < m; ++k) {
        float4 r = p_rel[s + k];
        float rad = fabsf(r.w);
        // hi + (lo + r) -/+ rad, rounded outward at every step
        lo.x = fminf(lo.x, __fsub_rd(__fadd_rd(x.x, __fadd_rd(xl.x, r.x)), rad));
        lo.y = fminf(lo.y, __fsub_rd(__fadd_rd(x.y, __fadd_rd(xl.y, r.y)), rad));
        lo.z = fminf(lo.z, __fsub_rd(__fadd_rd(x.z, __fadd_rd(xl.z, r.z)), rad));
        hi.x = fmaxf(hi.x, __fadd_ru(__fadd_ru(x.x, __fadd_ru(xl.x, r.x)), rad));
        hi.y = fmaxf(hi.y, __fadd_ru(__fadd_ru(x.y, __fadd_ru(xl.y, r.y)), rad));
        hi.z = fmaxf(hi.z, __fadd_ru(__fadd_ru(x.z, __fadd_ru(xl.z, r.z)), rad));
    }
    if (m == 0) { lo = make_float3(0.f, 0.f, 0.f); hi = make_float3(-1.f, -1.f, -1.f); }
    bmin[b] = make_float4(lo.x, lo.y, lo.z, 0.f);
    bmax[b] = make_float4(hi.x, hi.y, hi.z, 0.f);
}

__device__ __forceinline__ void contact(const CfgParams& p, float3 n, float pen, float3 v, float3& f) {
    float vn = v.x * n.x + v.y * n.y + v.z * n.z;
    float ks = -p.k * pen + p.eta * vn;
    float kt = p.kt * p.eta;
    f.x += ks * n.x + kt * (v.x - vn * n.x);
    f.y += ks * n.y + kt * (v.y - vn * n.y);
    f.z += ks * n.z + kt * (v.z - vn * n.z);
}

__global__ void __launch_bounds__(256) k_forces_cfg(const float4* __restrict__ pos, const float4* __restrict__ pos_lo,
                                                    const float4* __restrict__ p_rel,
                                                    const float4* __restrict__ p_vel, const int* p_body,
                                                    const int* pstart, const int* npart, const uint2* body_pairs,
                                                    const uint32_t* rowoff, uint64_t pair_cap, CfgParams p,
                                                    float4* p_force, int np) {
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t ncontact = 0;  // particle-particle contacts of particle i (walls not counted)
    if (i < np) {
        const int a = p_body[i];
        const float4 xa = pos[a], la = pos_lo[a], ri = p_rel[i], iv = p_vel[i];
        float3 f = make_float3(0.f, 0.f, 0.f);
        float3 vw = make_float3(-iv.x, -iv.y, -iv.z);
        const float xs[3] = {xa.x, xa.y, xa.z}, rs[3] = {la.x + ri.x, la.y + ri.y, la.z + ri.z};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            // distance to the walls: (hi - wall_lo) + (lo + r) and (wall_hi - hi) - (lo + r)
            float pen_lo = ri.w - ((xs[k] - p.lo[k]) + rs[k]);
            float pen_hi = ri.w - ((p.hi[k] - xs[k]) - rs[k]);
            if (pen_lo > 0.f) {
                float3 n = make_float3(k == 0 ? -1.f : 0.f, k == 1 ? -1.f : 0.f, k == 2 ? -1.f : 0.f);
                contact(p, n, pen_lo, vw, f);
            }
            if (pen_hi > 0.f) {
                float3 n = make_float3(k == 0 ? 1.f : 0.f, k == 1 ? 1.f : 0.f, k == 2 ? 1.f : 0.f);
                contact(p, n, pen_hi, vw, f);
            }
        }
        uint32_t e0 = rowoff[a], e1 = rowoff[a + 1];
        if (e1 > pair_cap) e1 = (uint32_t)pair_cap;  // after an overflow (reported) rows stay in storage
        for (uint32_t e = e0; e < e1; ++e) {
            int b = (int)__ldg(&body_pairs[e].y);
            const float4 xb = __ldg(pos + b), lb = __ldg(pos_lo + b);
            const float bx = (xb.x - xa.x) + (lb.x - la.x), by = (xb.y - xa.y) + (lb.y - la.y),
                        bz = (xb.z - xa.z) + (lb.z - la.z);
            int s = __ldg(pstart + b), m = __ldg(npart + b);
            for (int l = 0; l < m; ++l) {
                float4 rj = __ldg(p_rel + s + l);
                float dx = bx + (rj.x - ri.x), dy = by + (rj.y - ri.y), dz = bz + (rj.z - ri.z);
                float d2 = dx * dx + dy * dy + dz * dz;
                float rr = ri.w + rj.w;
                if (d2 < rr * rr && d2 > 0.f) {
                    float dist = sqrtf(d2);
                    float inv = 1.f / dist;
                    float4 jv = __ldg(p_vel + s + l);
                    float3 n = make_float3(dx * inv, dy * inv, dz * inv);
                    contact(p, n, rr - dist, make_float3(jv.x - iv.x, jv.y - iv.y, jv.z - iv.z), f);
                    ++ncontact;
                }
            }
        }
        p_force[i] = make_float4(f.x, f.y, f.z, 0.f);
    }
    if (p.contacts) {  // one atomic per warp (blocks are whole warps)
        const uint32_t w = __reduce_add_sync(0xffffffffu, ncontact);
        if ((threadIdx.x & 31) == 0 && w) atomicAdd(p.contacts, (unsigned long long)w);
    }
}

__device__ __forceinline__ void ts_add(float& s, float& c, float x) {
    float t = s + x;
    float bp = t - s;
    c += (s - (t - bp)) + (x - bp);
    s = t;
}

__global__ void k_update_cfg(float4* lin, float4* ang, const float4* quat, const float* inv_mass, const int* shape,
                             const int* pstart, const int* npart, const float4* ref_pos, const float4* shape_inv,
                             const float4* p_force, CfgParams p, int n) {
    pdl_wait();
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    float3 R[3];
    qrows(quat[b], R);
    int s = pstart[b], m = npart[b], sh = shape[b];
    float F[3] = {0, 0, 0}, Fc[3] = {0, 0, 0}, T[3] = {0, 0, 0}, Tc[3] = {0, 0, 0};
    for (int k = 0; k < m; ++k) {
        float4 ref = ref_pos[kMaxParticlesPerBody * sh + k];
        float3 r = mv(R, make_float3(ref.x, ref.y, ref.z));
        float4 f4 = p_force[s + k];
        float3 f = make_float3(f4.x, f4.y, f4.z);
        float3 t = cross3(r, f);
        ts_add(F[0], Fc[0], f.x); ts_add(F[1], Fc[1], f.y); ts_add(F[2], Fc[2], f.z);
        ts_add(T[0], Tc[0], t.x); ts_add(T[1], Tc[1], t.y); ts_add(T[2], Tc[2], t.z);
    }
    float3 Fs = make_float3(F[0] + Fc[0], F[1] + Fc[1], F[2] + Fc[2]);
    float3 Ts = make_float3(T[0] + Tc[0], T[1] + Tc[1], T[2] + Tc[2]);
    float im = inv_mass[b];
    float4 v = lin[b];
    v.x += Fs.x * im * p.dt; v.y += Fs.y * im * p.dt; v.z += Fs.z * im * p.dt;
    lin[b] = v;
    // I_w^-1 tau = R (I_s^-1 (R^T tau))
    float3 t1 = make_float3(R[0].x * Ts.x + R[1].x * Ts.y + R[2].x * Ts.z,
                            R[0].y * Ts.x + R[1].y * Ts.y + R[2].y * Ts.z,
                            R[0].z * Ts.x + R[1].z * Ts.y + R[2].z * Ts.z);
    float4 i0 = shape_inv[3 * sh], i1 = shape_inv[3 * sh + 1], i2 = shape_inv[3 * sh + 2];
    float3 t2 = make_float3(i0.x * t1.x + i0.y * t1.y + i0.z * t1.z, i1.x * t1.x + i1.y * t1.y + i1.z * t1.z,
                            i2.x * t1.x + i2.y * t1.y + i2.z * t1.z);
    float3 dw = mv(R, t2);
    float4 w = ang[b];
    w.x += dw.x * p.dt; w.y += dw.y * p.dt; w.z += dw.z * p.dt;
    ang[b] = w;
}

static inline int gr(int n) { return n <= 0 ? 1 : (n + 255) / 256; }

cudaError_t rb_integrate_cfg(float4* pos, float4* pos_lo, float4* quat, float4* lin, const float4* ang,
                             const CfgParams& p, int n, cudaStream_t st) {
    if (n > 0) launch_pdl(k_integrate_cfg, gr(n), 256, 0, st, pos, pos_lo, quat, lin, ang, p, n);
    return cudaGetLastError();
}
cudaError_t rb_place_cfg(const float4* quat, const float4* lin, const float4* ang, const int* shape,
                         const int* pstart, const int* p_body, const float4* ref_pos, float4* p_rel, float4* p_vel,
                         int np, cudaStream_t st) {
    if (np > 0) launch_pdl(k_place_cfg, gr(np), 256, 0, st, quat, lin, ang, shape, pstart, p_body, ref_pos, p_rel,
            p_vel, np);
    return cudaGetLastError();
}
cudaError_t rb_abs_pos(const float4* pos, const float4* pos_lo, const int* p_body, const float4* p_rel, float4* p_pos,
                       int np, cudaStream_t st) {
    if (np > 0) launch_pdl(k_abs_pos, gr(np), 256, 0, st, pos, pos_lo, p_body, p_rel, p_pos, np);
    return cudaGetLastError();
}
cudaError_t rb_body_aabb(const float4* pos, const float4* pos_lo, const float4* p_rel, const int* pstart,
                         const int* npart, float4* bmin, float4* bmax, int n, cudaStream_t st) {
    if (n > 0) launch_pdl(k_body_aabb, gr(n), 256, 0, st, pos, pos_lo, p_rel, pstart, npart, bmin, bmax, n);
    return cudaGetLastError();
}
cudaError_t rb_forces_cfg(const float4* pos, const float4* pos_lo, const float4* p_rel, const float4* p_vel,
                          const int* p_body, const int* pstart, const int* npart, const uint2* body_pairs,
                          const uint32_t* rowoff, uint64_t pair_cap, const CfgParams& p, float4* p_force, int np,
                          cudaStream_t st) {
    if (np > 0)
        launch_pdl(k_forces_cfg, gr(np), 256, 0, st, pos, pos_lo, p_rel, p_vel, p_body, pstart, npart, body_pairs,
                rowoff, pair_cap, p, p_force, np);
    return cudaGetLastError();
}
cudaError_t rb_update_cfg(float4* lin, float4* ang, const float4* quat, const float* inv_mass, const int* shape,
                          const int* pstart, const int* npart, const float4* ref_pos, const float4* shape_inv,
                          const float4* p_force, const CfgParams& p, int n, cudaStream_t st) {
    if (n > 0)
        launch_pdl(k_update_cfg, gr(n), 256, 0, st, lin, ang, quat, inv_mass, shape, pstart, npart, ref_pos,
                shape_inv, p_force, p, n);
    return cudaGetLastError();
}

}  // namespace gsap
