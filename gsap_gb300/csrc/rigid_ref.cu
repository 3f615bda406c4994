// Particle rigid-body step, reference model (FP32).
//
// Same formulas and operation order as the reference kernels of
// ParticleRigidBody/ParticleRigidBodyKernel.h (integrateK :47-69,
// updateParticleDataK :71-104, prepareK :30-45,
// clearForceAndBoundaryConditionK :106-140, comupteFoceOnParticlesK
// :142-208, updateVelocityK :213-262) with the SDK float4 semantics they
// use: componentwise ops on all four lanes, a / s evaluated as a * (1/s),
// length = sqrtf(dot4), normalize = v * (1/sqrtf(dot4)).  This translation
// unit is compiled with -fmad=false so every product and sum is rounded
// separately, as in the reference's source order.
//
// Launch shapes differ from the reference where it helps the GPU: particle
// placement runs one thread per particle (coalesced float4 stores) instead
// of one thread per body looping over its particles; the arithmetic per
// particle is unchanged.
#include "internal.cuh"
#include "rigid.cuh"

namespace gsap {
namespace rbref {

struct f4 {
    float x, y, z, w;
};
__device__ __forceinline__ f4 mk(float x, float y, float z, float w) { return {x, y, z, w}; }
__device__ __forceinline__ f4 ld(const float4* p) { float4 v = *p; return {v.x, v.y, v.z, v.w}; }
__device__ __forceinline__ void st(float4* p, f4 a) { *p = make_float4(a.x, a.y, a.z, a.w); }
__device__ __forceinline__ f4 add(f4 a, f4 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ f4 sub(f4 a, f4 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
__device__ __forceinline__ f4 mul(f4 a, float s) { return mk(a.x * s, a.y * s, a.z * s, a.w * s); }
__device__ __forceinline__ f4 divs(f4 a, float s) { float inv = 1.0f / s; return mul(a, inv); }
__device__ __forceinline__ float dot4(f4 a, f4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
__device__ __forceinline__ float dot3(f4 a, f4 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float len4(f4 a) { return sqrtf(dot4(a, a)); }
__device__ __forceinline__ f4 cross(f4 a, f4 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x, 0.f);
}
// quaternion product: cross + a.w b + b.w a, w = a.w b.w - dot3
__device__ __forceinline__ f4 qmul(f4 a, f4 b) {
    f4 r = cross(a, b);
    r = add(r, add(mul(b, a.w), mul(a, b.w)));
    r.w = a.w * b.w - dot3(a, b);
    return r;
}
// q v q^-1 on the full float4 v (its w takes part, as in the reference)
__device__ __forceinline__ f4 qrot(f4 q, f4 v) {
    f4 qi = mk(-q.x, -q.y, -q.z, q.w);
    return qmul(qmul(q, v), qi);
}
__device__ __forceinline__ void qmat(f4 q, f4 m[3]) {
    float x2 = q.x * q.x, y2 = q.y * q.y, z2 = q.z * q.z;
    m[0] = mk(1 - 2 * y2 - 2 * z2, 2 * q.x * q.y - 2 * q.w * q.z, 2 * q.x * q.z + 2 * q.w * q.y, 0);
    m[1] = mk(2 * q.x * q.y + 2 * q.w * q.z, 1 - 2 * x2 - 2 * z2, 2 * q.y * q.z - 2 * q.w * q.x, 0);
    m[2] = mk(2 * q.x * q.z - 2 * q.w * q.y, 2 * q.y * q.z + 2 * q.w * q.x, 1 - 2 * x2 - 2 * y2, 0);
}
__device__ __forceinline__ void mmul(const f4 a[3], const f4 b[3], f4 o[3]) {
    f4 bt[3] = {mk(b[0].x, b[1].x, b[2].x, 0), mk(b[0].y, b[1].y, b[2].y, 0), mk(b[0].z, b[1].z, b[2].z, 0)};
    for (int i = 0; i < 3; ++i) o[i] = mk(dot3(a[i], bt[0]), dot3(a[i], bt[1]), dot3(a[i], bt[2]), 0);
}
__device__ __forceinline__ void spring(float imi, float jmi, float dt2i, float dti, float sp, float dp, float& s,
                                       float& d) {
    float m = imi + jmi;
    m = 1 / m;
    s = m * dt2i * sp;
    d = m * dti * (1.f - dp);
}

}  // namespace rbref

using namespace rbref;

__global__ void k_integrate_ref(float4* pos, float4* quat, float4* lin, float4* ang, float dt, int n, float gy,
                                int floor_clamp) {
    pdl_wait();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    f4 lv = add(ld(lin + i), mul(mk(0.0f, gy, 0.0f, 0.0f), dt));
    st(lin + i, lv);
    f4 q = ld(quat + i);
    f4 w = ld(ang + i);
    w.w = 0.f;
    q = add(q, mul(qmul(w, q), dt * 0.5f));
    q = divs(q, len4(q));
    st(quat + i, q);
    float4 x = pos[i];
    x.x += lv.x * dt;
    x.y += lv.y * dt;
    x.z += lv.z * dt;
    if (floor_clamp) {
        if ((i / 6) % 2 == 0 && x.y <= 0.25f) x.y = 0.25f;
        else if ((i / 6) % 2 == 1 && x.y <= 0.3f) x.y = 0.3f;
    }
    pos[i] = x;
}

// one thread per particle; p_body[p] = owning body
__global__ void k_place_ref(const float4* pos, const float4* quat, const float4* lin, const float4* ang,
                            const int* shape, const int* pstart, const int* p_body, const float4* ref_pos,
                            const float* ref_mass, float4* p_pos, float4* p_vel, float* p_mass, int np) {
    pdl_wait();
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    int b = p_body[p];
    int k = p - pstart[b];
    int ri = kMaxParticlesPerBody * shape[b] + k;
    f4 ref = ld(ref_pos + ri);
    f4 cp = qrot(ld(quat + b), ref);
    st(p_vel + p, add(ld(lin + b), cross(ld(ang + b), cp)));
    cp = add(cp, ld(pos + b));
    p_pos[p] = make_float4(cp.x, cp.y, cp.z, ref.w);
    p_mass[p] = ref_mass[ri];
}

__global__ void k_place_ref_body(const float4* pos, const float4* quat, const float4* lin, const float4* ang,
                                 const int* shape, const int* pstart, const int* npart, const float4* ref_pos,
                                 const float* ref_mass, float4* p_pos, float4* p_vel, float* p_mass, int n) {
    pdl_wait();
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    int s = pstart[b];
    f4 x = ld(pos + b), v = ld(lin + b), q = ld(quat + b), w = ld(ang + b);
    for (int k = 0; k < npart[b]; ++k) {
        int ri = kMaxParticlesPerBody * shape[b] + k;
        f4 ref = ld(ref_pos + ri);
        f4 cp = qrot(q, ref);
        st(p_vel + s + k, add(v, cross(w, cp)));
        cp = add(cp, x);
        p_pos[s + k] = make_float4(cp.x, cp.y, cp.z, ref.w);
        p_mass[s + k] = ref_mass[ri];
    }
}

__global__ void k_prepare_ref(const float4* quat, const int* shape, const float4* shape_inv, float4* inv_out, int n) {
    pdl_wait();
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    f4 r[3], rt[3], is[3], t[3], o[3];
    qmat(ld(quat + b), r);
    rt[0] = mk(r[0].x, r[1].x, r[2].x, 0);
    rt[1] = mk(r[0].y, r[1].y, r[2].y, 0);
    rt[2] = mk(r[0].z, r[1].z, r[2].z, 0);
    const float4* si = shape_inv + 3 * shape[b];
    for (int k = 0; k < 3; ++k) is[k] = ld(si + k);
    mmul(r, is, t);
    mmul(t, rt, o);
    for (int k = 0; k < 3; ++k) st(inv_out + 3 * b + k, o[k]);
}

__global__ void k_clear_force_ref(const float4* p_pos, const float4* p_vel, const float* p_mass, float4* p_force,
                                  float sp, float dp, int np, float dt) {
    pdl_wait();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    float dt2i = 1.f / (dt * dt), dti = 1.f / dt;
    f4 ip = ld(p_pos + i), iv = ld(p_vel + i);
    float im = p_mass[i];
    f4 force = mk(0, 0, 0, 0);
    float dist = ip.y;
    f4 rij = mk(0, 1, 0, 0);
    f4 vij = mk(-iv.x, -iv.y, -iv.z, -iv.w);
    if (dist < ip.w) {
        float sc, dc;
        spring(1.f / im, 0.5f / im, dt2i, dti, sp, dp, sc, dc);
        f4 sf = mul(mul(rij, -sc * (dist - ip.w)), 0.1f);
        f4 df = mul(vij, dc);
        force = add(sf, df);
    }
    st(p_force + i, force);
}

// One thread per pairEntry.  The row of entry e ends at the next entry (or
// at num_pairs for the last), so nothing is read past the list.  The
// reference loop also stops after the pair whose index equals
// numPairEntries (`if( pairIdx++ == numPairEntries ) break;`, :201);
// `quirk` reproduces that truncation for bit-level parity.
// Counts may live on the device (graph-capturable step): d_num_pairs2 is the
// number of i<j pairs (the list holds twice as many).
__global__ void k_pair_force_ref(const float4* p_pos, const float4* p_vel, const int2* pairs, const int* entries,
                                 int num_pairs, int num_entries, const unsigned long long* d_num_pairs2,
                                 const uint32_t* d_num_entries, const float* p_mass, float sp, float dp,
                                 float4* p_force, float dt, int quirk, int pair_cap, int entry_cap) {
    pdl_wait();
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (d_num_entries) num_entries = (int)min(*d_num_entries, (uint32_t)entry_cap);
    if (d_num_pairs2) num_pairs = (int)min(2ull * *d_num_pairs2, (unsigned long long)pair_cap);
    if (num_pairs > pair_cap) num_pairs = pair_cap;  // rows never leave the list's storage
    if (e >= num_entries) return;
    int b0 = entries[e], b1 = (e + 1 < num_entries) ? entries[e + 1] : num_pairs;
    if (b1 > num_pairs) b1 = num_pairs;
    if (b0 < 0 || b0 >= b1) return;
    int i = pairs[b0].x;
    float dt2i = 1.f / (dt * dt), dti = 1.f / dt;
    f4 ip = ld(p_pos + i), iv = ld(p_vel + i);
    float im = p_mass[i];
    f4 sf = mk(0, 0, 0, 0), df = mk(0, 0, 0, 0);
    for (int k = b0; k < b1; ++k) {
        int j = pairs[k].y;
        f4 jp = ld(p_pos + j), jv = ld(p_vel + j);
        float jm = p_mass[j];
        f4 rij = sub(jp, ip);
        rij.w = 0.f;
        f4 vij = sub(jv, iv);
        float dist = len4(rij);
        float od = ip.w + jp.w;
        float sc, dc;
        spring(1.f / im, 1.f / jm, dt2i, dti, sp, dp, sc, dc);
        float pen = od - dist;
        if (pen > 0.f) {
            sf = sub(sf, divs(mul(rij, sc * pen), dist));
            df = add(df, mul(vij, dc));
        }
        if (quirk && k == num_entries) break;
    }
    st(p_force + i, add(ld(p_force + i), add(sf, df)));
}

__global__ void k_update_velocity_ref(float4* lin, float4* ang, const float4* quat, const float* inv_mass,
                                      const float4* inv_inertia, const int* shape, const int* pstart,
                                      const int* npart, const float4* ref_pos, const float4* p_force, int n,
                                      float dt, float max_lin_vel, int cap, int torque_quirk) {
    pdl_wait();
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    f4 q = ld(quat + b);
    int s = pstart[b];
    f4 lf = mk(0, 0, 0, 0), af = mk(0, 0, 0, 0);
    for (int k = 0; k < npart[b]; ++k) {
        f4 cp = qrot(q, ld(ref_pos + kMaxParticlesPerBody * shape[b] + k));
        f4 f = ld(p_force + s + k);
        lf = add(lf, f);
        af = add(af, cross(cp, f));
    }
    f4 lv = add(ld(lin + b), mul(mul(lf, inv_mass[b]), dt));
    if (cap) {
        f4 l = lv;
        l.w = 0;
        float ll = len4(l);
        if (ll > max_lin_vel) {
            float inv = 1.0f / sqrtf(dot4(l, l));
            lv = mul(mul(l, inv), max_lin_vel);
        }
    }
    st(lin + b, lv);
    f4 w = ld(ang + b);
    if (torque_quirk) {
        w = add(w, mul(af, dt));
    } else {
        const float4* m = inv_inertia + 3 * b;
        f4 dw = mk(dot3(ld(m), af), dot3(ld(m + 1), af), dot3(ld(m + 2), af), 0);
        w = add(w, mul(dw, dt));
    }
    st(ang + b, w);
}

// --------------------------------------------------------------- launches

static inline int grid_for(int n) { return n <= 0 ? 1 : (n + 255) / 256; }

cudaError_t rb_integrate_ref(float4* pos, float4* quat, float4* lin, float4* ang, float dt, int n, float gy,
                             int floor_clamp, cudaStream_t st) {
    if (n > 0) launch_pdl(k_integrate_ref, grid_for(n), 256, 0, st, pos, quat, lin, ang, dt, n, gy, floor_clamp);
    return cudaGetLastError();
}
cudaError_t rb_place_ref(const float4* pos, const float4* quat, const float4* lin, const float4* ang,
                         const int* shape, const int* pstart, const int* npart, const int* p_body,
                         const float4* ref_pos, const float* ref_mass, float4* p_pos, float4* p_vel, float* p_mass,
                         int n, int np, cudaStream_t st) {
    if (p_body) {
        if (np > 0)
            launch_pdl(k_place_ref, grid_for(np), 256, 0, st, pos, quat, lin, ang, shape, pstart, p_body, ref_pos,
                    ref_mass, p_pos, p_vel, p_mass, np);
    } else if (n > 0) {
        launch_pdl(k_place_ref_body, grid_for(n), 256, 0, st, pos, quat, lin, ang, shape, pstart, npart, ref_pos,
                ref_mass, p_pos, p_vel, p_mass, n);
    }
    return cudaGetLastError();
}
cudaError_t rb_prepare_ref(const float4* quat, const int* shape, const float4* shape_inv, float4* inv_out, int n,
                           cudaStream_t st) {
    if (n > 0) launch_pdl(k_prepare_ref, grid_for(n), 256, 0, st, quat, shape, shape_inv, inv_out, n);
    return cudaGetLastError();
}
cudaError_t rb_clear_force_ref(const float4* p_pos, const float4* p_vel, const float* p_mass, float4* p_force,
                               float sp, float dp, int np, float dt, cudaStream_t st) {
    if (np > 0) launch_pdl(k_clear_force_ref, grid_for(np), 256, 0, st, p_pos, p_vel, p_mass, p_force, sp, dp, np,
            dt);
    return cudaGetLastError();
}
cudaError_t rb_pair_force_ref(const float4* p_pos, const float4* p_vel, const int2* pairs, const int* entries,
                              int num_pairs, int num_entries, int max_entries, const unsigned long long* d_np2,
                              const uint32_t* d_ne, const float* p_mass, float sp, float dp, float4* p_force,
                              float dt, int quirk, int pair_cap, cudaStream_t st) {
    int g = d_ne ? max_entries : num_entries;
    if (g > 0)
        launch_pdl(k_pair_force_ref, grid_for(g), 256, 0, st, p_pos, p_vel, pairs, entries, num_pairs, num_entries,
                d_np2, d_ne, p_mass, sp, dp, p_force, dt, quirk, pair_cap, g);
    return cudaGetLastError();
}
cudaError_t rb_update_velocity_ref(float4* lin, float4* ang, const float4* quat, const float* inv_mass,
                                   const float4* inv_inertia, const int* shape, const int* pstart, const int* npart,
                                   const float4* ref_pos, const float4* p_force, int n, float dt, float max_lin_vel,
                                   int cap, int torque_quirk, cudaStream_t st) {
    if (n > 0)
        launch_pdl(k_update_velocity_ref, grid_for(n), 256, 0, st, lin, ang, quat, inv_mass, inv_inertia, shape,
                pstart, npart, ref_pos, p_force, n, dt, max_lin_vel, cap, torque_quirk);
    return cudaGetLastError();
}

}  // namespace gsap
