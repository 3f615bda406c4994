// C ABI of the particle rigid-body step (include/gsap.h).
//
// Replaces the ParticleRigidBody DLL (ParticleRigidBody/ParticleRigidBody.cpp:
// 15-191) and its PRBWrap launchers (ParticleRigidBodyWrapper.h:11-54).  The
// handle owns the SoA state in device memory; uploads are plain host->device
// copies (the reference's GL pixel-buffer set-up, :88-98, is dropped: poses
// are read back with gsap_rb_get_state instead).  gsap_rb_step runs a whole
// step, broadphase included, without host synchronisation; its broadphase
// runs in temporal mode (GSAP_FLAG_TEMPORAL): the cell grid of the previous
// step while this step's PCA runs beside the sweep.  The pair list is exact
// either way.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/gsap.h"
#include "api_internal.h"
#include "internal.cuh"
#include "rigid.cuh"

using namespace gsap;

#define RCK(call)                                                                 \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess) return set_error(GSAP_ERR_CUDA, cudaGetErrorString(e_)); \
    } while (0)

struct gsap_rb {
    int max_bodies, max_particles, max_pairs;
    int n_bodies, n_particles, n_shapes;
    float4 *pos, *quat, *lin, *ang;
    float4* pos_lo;       // config model: low parts of the float-float body positions (zero after a set)
    int *shape, *pstart, *npart, *p_body;
    float* inv_mass;
    float4* inv_inertia;  // 3 rows per body
    float4 *p_pos, *p_vel, *p_force;
    float4* p_rel;        // config model: body-relative particle offsets (w = radius)
    bool abs_stale;       // config model: p_pos must be rebuilt from p_rel before a read
    float* p_mass;
    float4* ref_pos;      // kMaxParticlesPerBody * kMaxShapes
    float* ref_mass;
    float4* shape_inv;    // 3 rows per shape
    int2* pairs;          // reference-model particle pairs (both directions)
    int* entries;
    int num_pairs, num_entries;
    float4 *bmin, *bmax;  // config model: body AABBs
    uint2* body_pairs;    // config model: both-direction body pairs
    uint64_t body_pair_cap;
    uint32_t* scene_off;  // device scene offsets of the bodies
    uint32_t num_scenes;
    gsap_contact_params cp;
    unsigned long long* contacts;  // config model: particle-particle contacts counted by the force kernel
};

static void rb_free(gsap_rb* h) {
    void* p[] = {h->pos, h->pos_lo, h->quat, h->lin, h->ang, h->shape, h->pstart, h->npart, h->p_body, h->inv_mass,
                 h->inv_inertia, h->p_pos, h->p_vel, h->p_force, h->p_rel, h->p_mass, h->ref_pos, h->ref_mass, h->shape_inv,
                 h->pairs, h->entries, h->bmin, h->bmax, h->body_pairs, h->scene_off, h->contacts};
    for (void* q : p)
        if (q) cudaFree(q);
}

extern "C" gsap_rb* gsap_rb_create(int32_t max_bodies, int32_t max_particles, int32_t max_pairs) {
    if (max_bodies <= 0 || max_particles <= 0 || max_pairs < 0) {
        set_error(GSAP_ERR_INVALID, "gsap_rb_create: sizes must be positive");
        return nullptr;
    }
    gsap_rb* h = new gsap_rb();
    memset(h, 0, sizeof(*h));
    h->max_bodies = max_bodies;
    h->max_particles = max_particles;
    h->max_pairs = max_pairs > 0 ? max_pairs : 1;
    h->body_pair_cap = 32ull * max_bodies + 1024;
    bool ok = true;
    auto A = [&](void** q, size_t bytes) {
        if (!ok) return;
        if (cudaMalloc(q, bytes) != cudaSuccess || cudaMemset(*q, 0, bytes) != cudaSuccess) ok = false;
    };
    size_t B = (size_t)max_bodies, Pn = (size_t)max_particles;
    A((void**)&h->pos, 16 * B); A((void**)&h->pos_lo, 16 * B); A((void**)&h->quat, 16 * B); A((void**)&h->lin, 16 * B); A((void**)&h->ang, 16 * B);
    A((void**)&h->shape, 4 * B); A((void**)&h->pstart, 4 * B); A((void**)&h->npart, 4 * B);
    A((void**)&h->p_body, 4 * Pn);
    A((void**)&h->inv_mass, 4 * B); A((void**)&h->inv_inertia, 48 * B);
    A((void**)&h->p_pos, 16 * Pn); A((void**)&h->p_vel, 16 * Pn); A((void**)&h->p_force, 16 * Pn);
    A((void**)&h->p_rel, 16 * Pn);
    A((void**)&h->p_mass, 4 * Pn);
    A((void**)&h->ref_pos, 16ull * kMaxParticlesPerBody * kMaxShapes);
    A((void**)&h->ref_mass, 4ull * kMaxParticlesPerBody * kMaxShapes);
    A((void**)&h->shape_inv, 48ull * kMaxShapes);
    A((void**)&h->pairs, 8ull * h->max_pairs);
    A((void**)&h->entries, 4 * Pn + 4);
    A((void**)&h->bmin, 16 * B); A((void**)&h->bmax, 16 * B);
    A((void**)&h->body_pairs, 8ull * h->body_pair_cap);
    A((void**)&h->contacts, 8);
    if (!ok) {
        set_error(GSAP_ERR_CUDA, "gsap_rb_create: device allocation failed");
        rb_free(h);
        delete h;
        return nullptr;
    }
    // defaults of the reference (ParticleRigidBody.cpp:45-46, kernel gravity -5)
    h->cp.model = GSAP_CONTACT_REF;
    h->cp.sp_multip = 0.5f;
    h->cp.dp_multip = 0.25f;
    h->cp.max_lin_vel = 0.f;
    h->cp.gravity_y = -5.f;
    h->cp.floor_clamp = 1;
    h->cp.torque_quirk = 1;
    return h;
}

extern "C" void gsap_rb_destroy(gsap_rb* h) {
    if (!h) return;
    rb_free(h);
    delete h;
}

extern "C" gsap_status gsap_rb_set_body_data(gsap_rb* h, const gsap_body_data* d) {
    if (!h || !d) return set_error(GSAP_ERR_INVALID, "null argument");
    const int nb = d->n_bodies, np = d->n_total_particles;
    if (nb < 0 || nb > h->max_bodies) return set_error(GSAP_ERR_CAPACITY, "n_bodies exceeds max_bodies");
    if (np < 0 || np > h->max_particles) return set_error(GSAP_ERR_CAPACITY, "particles exceed max_particles");
    if (nb > 0 && (!d->pos || !d->quat || !d->lin_vel || !d->ang_vel || !d->shape_idx || !d->p_start ||
                   !d->n_part || !d->inv_mass || !d->inv_inertia))
        return set_error(GSAP_ERR_INVALID, "null body array");
    // quaternions are normalised on upload (setRbData, ParticleRigidBody.cpp:82-86):
    // q *= 1 / sqrtf(dot4(q, q)), sums left to right, one rounding per operation
    std::vector<float> q(d->quat, d->quat + 4 * (size_t)nb);
    for (int b = 0; b < nb; ++b) {
        float* v = &q[4 * b];
        float l = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2] + v[3] * v[3]);
        if (!(l > 0.f)) return set_error(GSAP_ERR_INVALID, "zero quaternion");
        float inv = 1.0f / l;
        for (int k = 0; k < 4; ++k) v[k] *= inv;
        if (d->n_part[b] < 0 || d->n_part[b] > kMaxParticlesPerBody)
            return set_error(GSAP_ERR_INVALID, "a body has more than 10 particles (MAX_NUM_PARTICLES)");
        if (d->shape_idx[b] < 0 || d->shape_idx[b] >= kMaxShapes) return set_error(GSAP_ERR_INVALID, "shape index out of range");
        if (d->p_start[b] < 0 || d->p_start[b] + d->n_part[b] > np)
            return set_error(GSAP_ERR_INVALID, "particle range of a body out of bounds");
    }
    std::vector<int> pb(np > 0 ? np : 1, -1);
    for (int b = 0; b < nb; ++b)
        for (int k = 0; k < d->n_part[b]; ++k) pb[d->p_start[b] + k] = b;
    for (int p = 0; p < np; ++p)
        if (pb[p] < 0) return set_error(GSAP_ERR_INVALID, "a particle belongs to no body");
    size_t B = (size_t)nb;
    RCK(cudaMemcpy(h->pos, d->pos, 16 * B, cudaMemcpyHostToDevice));
    RCK(cudaMemset(h->pos_lo, 0, 16 * B));
    RCK(cudaMemcpy(h->quat, q.data(), 16 * B, cudaMemcpyHostToDevice));
    RCK(cudaMemcpy(h->lin, d->lin_vel, 16 * B, cudaMemcpyHostToDevice));
    RCK(cudaMemcpy(h->ang, d->ang_vel, 16 * B, cudaMemcpyHostToDevice));
    RCK(cudaMemcpy(h->shape, d->shape_idx, 4 * B, cudaMemcpyHostToDevice));
    RCK(cudaMemcpy(h->pstart, d->p_start, 4 * B, cudaMemcpyHostToDevice));
    RCK(cudaMemcpy(h->npart, d->n_part, 4 * B, cudaMemcpyHostToDevice));
    RCK(cudaMemcpy(h->inv_mass, d->inv_mass, 4 * B, cudaMemcpyHostToDevice));
    RCK(cudaMemcpy(h->inv_inertia, d->inv_inertia, 48 * B, cudaMemcpyHostToDevice));
    RCK(cudaMemcpy(h->p_body, pb.data(), 4ull * np, cudaMemcpyHostToDevice));
    h->n_bodies = nb;
    h->n_particles = np;
    return GSAP_OK;
}

extern "C" gsap_status gsap_rb_set_particle_data(gsap_rb* h, const float* ref_pos, const float* mass, int32_t n) {
    if (!h || (n > 0 && (!ref_pos || !mass))) return set_error(GSAP_ERR_INVALID, "null argument");
    if (n < 0 || n > kMaxParticlesPerBody * kMaxShapes) return set_error(GSAP_ERR_CAPACITY, "too many reference particles");
    RCK(cudaMemcpy(h->ref_pos, ref_pos, 16ull * n, cudaMemcpyHostToDevice));
    RCK(cudaMemcpy(h->ref_mass, mass, 4ull * n, cudaMemcpyHostToDevice));
    return GSAP_OK;
}

extern "C" gsap_status gsap_rb_set_shape_inv_inertia(gsap_rb* h, const float* inv, int32_t n_shapes) {
    if (!h || (n_shapes > 0 && !inv)) return set_error(GSAP_ERR_INVALID, "null argument");
    if (n_shapes < 0 || n_shapes > kMaxShapes) return set_error(GSAP_ERR_CAPACITY, "too many shapes");
    RCK(cudaMemcpy(h->shape_inv, inv, 48ull * n_shapes, cudaMemcpyHostToDevice));
    h->n_shapes = n_shapes;
    return GSAP_OK;
}

extern "C" gsap_status gsap_rb_set_contact(gsap_rb* h, const gsap_contact_params* p) {
    if (!h || !p) return set_error(GSAP_ERR_INVALID, "null argument");
    if (p->model != GSAP_CONTACT_REF && p->model != GSAP_CONTACT_CONFIG)
        return set_error(GSAP_ERR_INVALID, "unknown contact model");
    // the reference model steps plain FP32 positions: low parts start at zero
    if (p->model != h->cp.model && h->max_bodies > 0) RCK(cudaMemset(h->pos_lo, 0, 16ull * h->max_bodies));
    h->cp = *p;
    return GSAP_OK;
}

extern "C" gsap_status gsap_rb_set_scenes(gsap_rb* h, const uint32_t* off, uint32_t S) {
    if (!h) return set_error(GSAP_ERR_INVALID, "null handle");
    if (S == 0 || !off) {
        if (h->scene_off) cudaFree(h->scene_off);
        h->scene_off = nullptr;
        h->num_scenes = 0;
        return GSAP_OK;
    }
    if (off[0] != 0 || off[S] != (uint32_t)h->n_bodies) return set_error(GSAP_ERR_INVALID, "scene offsets must run from 0 to n_bodies");
    for (uint32_t s = 0; s < S; ++s)
        if (off[s + 1] < off[s]) return set_error(GSAP_ERR_INVALID, "scene offsets must be non-decreasing");
    if (h->scene_off) cudaFree(h->scene_off);
    h->scene_off = nullptr;
    RCK(cudaMalloc(&h->scene_off, 4ull * (S + 1)));
    RCK(cudaMemcpy(h->scene_off, off, 4ull * (S + 1), cudaMemcpyHostToDevice));
    h->num_scenes = S;
    return GSAP_OK;
}

static CfgParams cfg_of(const gsap_rb* h, float dt) {
    CfgParams p;
    p.dt = dt;
    p.k = h->cp.k;
    p.eta = h->cp.eta;
    p.kt = h->cp.kt;
    p.gy = h->cp.gravity_y;
    for (int a = 0; a < 3; ++a) { p.lo[a] = h->cp.box_lo[a]; p.hi[a] = h->cp.box_hi[a]; }
    p.contacts = h->contacts;
    return p;
}

extern "C" gsap_status gsap_rb_integrate(gsap_rb* h, float dt, void* stream) {
    if (!h) return set_error(GSAP_ERR_INVALID, "null handle");
    cudaStream_t st = (cudaStream_t)stream;
    if (h->cp.model == GSAP_CONTACT_CONFIG)
        RCK(rb_integrate_cfg(h->pos, h->pos_lo, h->quat, h->lin, h->ang, cfg_of(h, dt), h->n_bodies, st));
    else RCK(rb_integrate_ref(h->pos, h->quat, h->lin, h->ang, dt, h->n_bodies, h->cp.gravity_y, (int)h->cp.floor_clamp, st));
    return GSAP_OK;
}

extern "C" gsap_status gsap_rb_update_particle_data(gsap_rb* h, void* stream) {
    if (!h) return set_error(GSAP_ERR_INVALID, "null handle");
    cudaStream_t st = (cudaStream_t)stream;
    if (h->cp.model == GSAP_CONTACT_CONFIG) {
        RCK(rb_place_cfg(h->quat, h->lin, h->ang, h->shape, h->pstart, h->p_body, h->ref_pos, h->p_rel, h->p_vel,
                         h->n_particles, st));
        h->abs_stale = true;
        return GSAP_OK;
    }
    RCK(rb_place_ref(h->pos, h->quat, h->lin, h->ang, h->shape, h->pstart, h->npart, h->p_body, h->ref_pos,
                     h->ref_mass, h->p_pos, h->p_vel, h->p_mass, h->n_bodies, h->n_particles, st));
    return GSAP_OK;
}

extern "C" gsap_status gsap_rb_prepare(gsap_rb* h, void* stream) {
    if (!h) return set_error(GSAP_ERR_INVALID, "null handle");
    RCK(rb_prepare_ref(h->quat, h->shape, h->shape_inv, h->inv_inertia, h->n_bodies, (cudaStream_t)stream));
    return GSAP_OK;
}

extern "C" gsap_status gsap_rb_compute_forces(gsap_rb* h, float dt, void* stream) {
    if (!h) return set_error(GSAP_ERR_INVALID, "null handle");
    if (h->cp.model != GSAP_CONTACT_REF)
        return set_error(GSAP_ERR_INVALID, "gsap_rb_compute_forces uses the reference pair list; the config model runs in gsap_rb_step");
    cudaStream_t st = (cudaStream_t)stream;
    RCK(rb_clear_force_ref(h->p_pos, h->p_vel, h->p_mass, h->p_force, h->cp.sp_multip, h->cp.dp_multip,
                           h->n_particles, dt, st));
    RCK(rb_pair_force_ref(h->p_pos, h->p_vel, h->pairs, h->entries, h->num_pairs, h->num_entries, h->num_entries,
                          nullptr, nullptr, h->p_mass, h->cp.sp_multip, h->cp.dp_multip, h->p_force, dt,
                          (int)h->cp.pair_loop_quirk, h->max_pairs, st));
    return GSAP_OK;
}

extern "C" gsap_status gsap_rb_update_velocity(gsap_rb* h, float dt, void* stream) {
    if (!h) return set_error(GSAP_ERR_INVALID, "null handle");
    cudaStream_t st = (cudaStream_t)stream;
    if (h->cp.model == GSAP_CONTACT_CONFIG) {
        RCK(rb_update_cfg(h->lin, h->ang, h->quat, h->inv_mass, h->shape, h->pstart, h->npart, h->ref_pos,
                          h->shape_inv, h->p_force, cfg_of(h, dt), h->n_bodies, st));
        return GSAP_OK;
    }
    const int cap = h->cp.max_lin_vel > 0.f ? 1 : 0;
    RCK(rb_update_velocity_ref(h->lin, h->ang, h->quat, h->inv_mass, h->inv_inertia, h->shape, h->pstart, h->npart,
                               h->ref_pos, h->p_force, h->n_bodies, dt, h->cp.max_lin_vel, cap,
                               (int)h->cp.torque_quirk, st));
    return GSAP_OK;
}

extern "C" int32_t* gsap_rb_pairs(gsap_rb* h) { return h ? (int32_t*)h->pairs : nullptr; }
extern "C" int32_t* gsap_rb_pair_entries(gsap_rb* h) { return h ? h->entries : nullptr; }
// Config model: absolute particle positions are rebuilt from the body poses
// and body-relative offsets before they are handed out.
static void refresh_abs(gsap_rb* h, cudaStream_t st) {
    if (h->cp.model == GSAP_CONTACT_CONFIG && h->abs_stale) {
        rb_abs_pos(h->pos, h->pos_lo, h->p_body, h->p_rel, h->p_pos, h->n_particles, st);
        cudaStreamSynchronize(st);
        h->abs_stale = false;
    }
}

extern "C" float* gsap_rb_particle_pos(gsap_rb* h) {
    if (!h) return nullptr;
    refresh_abs(h, nullptr);
    return (float*)h->p_pos;
}
extern "C" float* gsap_rb_particle_vel(gsap_rb* h) { return h ? (float*)h->p_vel : nullptr; }
extern "C" float* gsap_rb_particle_force(gsap_rb* h) { return h ? (float*)h->p_force : nullptr; }

extern "C" gsap_status gsap_rb_set_num_pairs(gsap_rb* h, int32_t num_pairs, int32_t num_entries) {
    if (!h) return set_error(GSAP_ERR_INVALID, "null handle");
    // setNumPairs asserts numPairs < maxPairs (ParticleRigidBody.h:100)
    if (num_pairs < 0 || num_pairs > h->max_pairs) return set_error(GSAP_ERR_CAPACITY, "num_pairs exceeds max_pairs");
    if (num_entries < 0 || num_entries > h->max_particles) return set_error(GSAP_ERR_CAPACITY, "num_entries exceeds max_particles");
    h->num_pairs = num_pairs;
    h->num_entries = num_entries;
    return GSAP_OK;
}

extern "C" gsap_status gsap_rb_step(gsap_rb* h, gsap_sap* bp, float dt, void* stream) {
    if (!h || !bp) return set_error(GSAP_ERR_INVALID, "null handle");
    NvtxRange range("gsap:rb_step");
    cudaStream_t st = (cudaStream_t)stream;
    gsap_status r;
    if (h->cp.model == GSAP_CONTACT_REF) {
        if ((r = gsap_rb_integrate(h, dt, stream)) != GSAP_OK) return r;
        if ((r = gsap_rb_update_particle_data(h, stream)) != GSAP_OK) return r;
        BpDeviceCounts dc;
        r = bp_both_async(bp, GSAP_MODE_SPHERE, h->p_pos, nullptr, nullptr, 1, (uint32_t)h->n_particles,
                          (uint2*)h->pairs, (uint64_t)h->max_pairs, h->entries, (uint64_t)h->max_particles, st, &dc,
                          GSAP_FLAG_TEMPORAL);
        if (r != GSAP_OK) return r;
        if ((r = gsap_rb_prepare(h, stream)) != GSAP_OK) return r;
        RCK(rb_clear_force_ref(h->p_pos, h->p_vel, h->p_mass, h->p_force, h->cp.sp_multip, h->cp.dp_multip,
                               h->n_particles, dt, st));
        RCK(rb_pair_force_ref(h->p_pos, h->p_vel, h->pairs, h->entries, 0, 0, h->n_particles, dc.num_pairs,
                              dc.num_entries, h->p_mass, h->cp.sp_multip, h->cp.dp_multip, h->p_force, dt,
                              (int)h->cp.pair_loop_quirk, h->max_pairs, st));
        return gsap_rb_update_velocity(h, dt, stream);
    }
    // config model
    CfgParams p = cfg_of(h, dt);
    RCK(rb_integrate_cfg(h->pos, h->pos_lo, h->quat, h->lin, h->ang, p, h->n_bodies, st));
    RCK(rb_place_cfg(h->quat, h->lin, h->ang, h->shape, h->pstart, h->p_body, h->ref_pos, h->p_rel, h->p_vel,
                     h->n_particles, st));
    h->abs_stale = true;
    RCK(rb_body_aabb(h->pos, h->pos_lo, h->p_rel, h->pstart, h->npart, h->bmin, h->bmax, h->n_bodies, st));
    BpDeviceCounts dc;
    r = bp_both_async(bp, GSAP_MODE_AABB, h->bmin, h->bmax, h->scene_off, h->num_scenes ? h->num_scenes : 1,
                      (uint32_t)h->n_bodies, h->body_pairs, h->body_pair_cap, nullptr, 0, st, &dc, GSAP_FLAG_TEMPORAL);
    if (r != GSAP_OK) return r;
    RCK(rb_forces_cfg(h->pos, h->pos_lo, h->p_rel, h->p_vel, h->p_body, h->pstart, h->npart, h->body_pairs, dc.rowoff,
                      h->body_pair_cap, p, h->p_force, h->n_particles, st));
    RCK(rb_update_cfg(h->lin, h->ang, h->quat, h->inv_mass, h->shape, h->pstart, h->npart, h->ref_pos, h->shape_inv,
                      h->p_force, p, h->n_bodies, st));
    return GSAP_OK;
}

extern "C" gsap_status gsap_rb_get_state(gsap_rb* h, float* pos, float* quat, float* lin, float* ang, void* stream) {
    if (!h) return set_error(GSAP_ERR_INVALID, "null handle");
    cudaStream_t st = (cudaStream_t)stream;
    size_t B = 16ull * h->n_bodies;
    if (pos) RCK(cudaMemcpyAsync(pos, h->pos, B, cudaMemcpyDeviceToHost, st));
    if (quat) RCK(cudaMemcpyAsync(quat, h->quat, B, cudaMemcpyDeviceToHost, st));
    if (lin) RCK(cudaMemcpyAsync(lin, h->lin, B, cudaMemcpyDeviceToHost, st));
    if (ang) RCK(cudaMemcpyAsync(ang, h->ang, B, cudaMemcpyDeviceToHost, st));
    RCK(cudaStreamSynchronize(st));
    return GSAP_OK;
}

extern "C" gsap_status gsap_rb_set_state(gsap_rb* h, const float* pos, const float* quat, const float* lin,
                                         const float* ang, void* stream) {
    if (!h) return set_error(GSAP_ERR_INVALID, "null handle");
    cudaStream_t st = (cudaStream_t)stream;
    size_t B = 16ull * h->n_bodies;
    if (pos) {
        RCK(cudaMemcpyAsync(h->pos, pos, B, cudaMemcpyHostToDevice, st));
        RCK(cudaMemsetAsync(h->pos_lo, 0, B, st));
    }
    if (quat) RCK(cudaMemcpyAsync(h->quat, quat, B, cudaMemcpyHostToDevice, st));
    if (lin) RCK(cudaMemcpyAsync(h->lin, lin, B, cudaMemcpyHostToDevice, st));
    if (ang) RCK(cudaMemcpyAsync(h->ang, ang, B, cudaMemcpyHostToDevice, st));
    RCK(cudaStreamSynchronize(st));
    h->abs_stale = h->cp.model == GSAP_CONTACT_CONFIG;
    return GSAP_OK;
}

static void* rb_array(gsap_rb* h, int which, uint64_t* cap) {
    switch (which) {
        case GSAP_RB_PARTICLE_POS: *cap = 16ull * h->max_particles; return h->p_pos;
        case GSAP_RB_PARTICLE_VEL: *cap = 16ull * h->max_particles; return h->p_vel;
        case GSAP_RB_PARTICLE_FORCE: *cap = 16ull * h->max_particles; return h->p_force;
        case GSAP_RB_PAIRS: *cap = 8ull * h->max_pairs; return h->pairs;
        case GSAP_RB_PAIR_ENTRIES: *cap = 4ull * h->max_particles + 4; return h->entries;
        case GSAP_RB_INV_INERTIA: *cap = 48ull * h->max_bodies; return h->inv_inertia;
        default: *cap = 0; return nullptr;
    }
}

extern "C" gsap_status gsap_rb_copy_out(gsap_rb* h, int32_t which, void* dst, uint64_t bytes, void* stream) {
    if (!h || (bytes && !dst)) return set_error(GSAP_ERR_INVALID, "null argument");
    uint64_t cap = 0;
    void* src = rb_array(h, which, &cap);
    if (!src) return set_error(GSAP_ERR_INVALID, "unknown array");
    if (bytes > cap) return set_error(GSAP_ERR_CAPACITY, "copy larger than the array");
    cudaStream_t st = (cudaStream_t)stream;
    if (which == GSAP_RB_PARTICLE_POS) refresh_abs(h, st);
    RCK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
    RCK(cudaStreamSynchronize(st));
    return GSAP_OK;
}

extern "C" gsap_status gsap_rb_copy_in(gsap_rb* h, int32_t which, const void* src, uint64_t bytes, void* stream) {
    if (!h || (bytes && !src)) return set_error(GSAP_ERR_INVALID, "null argument");
    uint64_t cap = 0;
    void* dst = rb_array(h, which, &cap);
    if (!dst) return set_error(GSAP_ERR_INVALID, "unknown array");
    if (bytes > cap) return set_error(GSAP_ERR_CAPACITY, "copy larger than the array");
    cudaStream_t st = (cudaStream_t)stream;
    RCK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
    RCK(cudaStreamSynchronize(st));
    if (which == GSAP_RB_PARTICLE_POS) h->abs_stale = false;
    return GSAP_OK;
}

extern "C" int gsap_debug_rb_contacts(gsap_rb* h, uint64_t* out, int reset, void* stream) {
    if (!h || !out) return -1;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned long long v = 0;
    if (cudaMemcpyAsync(&v, h->contacts, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess) return -1;
    if (reset && cudaMemsetAsync(h->contacts, 0, 8, st) != cudaSuccess) return -1;
    if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
    *out = v;
    return 0;
}

// ---------------------------------------------------- PRBWrap replacements

extern "C" gsap_status gsap_k_integrate(float* pos, float* quat, float* lin, float* ang, float dt, int32_t n,
                                        const gsap_contact_params* p, void* stream) {
    gsap_contact_params d;
    memset(&d, 0, sizeof(d));
    d.gravity_y = -5.f;
    d.floor_clamp = 1;
    if (!p) p = &d;
    cudaStream_t st = (cudaStream_t)stream;
    if (p->model == GSAP_CONTACT_CONFIG) {
        CfgParams c;
        memset(&c, 0, sizeof(c));
        c.dt = dt;
        c.gy = p->gravity_y;
        RCK(rb_integrate_cfg((float4*)pos, nullptr, (float4*)quat, (float4*)lin, (const float4*)ang, c, n, st));
    } else {
        RCK(rb_integrate_ref((float4*)pos, (float4*)quat, (float4*)lin, (float4*)ang, dt, n, p->gravity_y,
                             (int)p->floor_clamp, st));
    }
    return GSAP_OK;
}

extern "C" gsap_status gsap_k_update_particle_data(const float* pos, const float* quat, const float* lin,
                                                   const float* ang, const int32_t* shape, const int32_t* pstart,
                                                   const int32_t* npart, const float* ref_pos, const float* ref_mass,
                                                   float* p_pos, float* p_vel, float* p_mass, int32_t n, void* stream) {
    RCK(rb_place_ref((const float4*)pos, (const float4*)quat, (const float4*)lin, (const float4*)ang, shape, pstart,
                     npart, nullptr, (const float4*)ref_pos, ref_mass, (float4*)p_pos, (float4*)p_vel, p_mass, n, 0,
                     (cudaStream_t)stream));
    return GSAP_OK;
}

extern "C" gsap_status gsap_k_prepare(const float* quat, const int32_t* shape, const float* shape_inv, float* inv,
                                      int32_t n, void* stream) {
    RCK(rb_prepare_ref((const float4*)quat, shape, (const float4*)shape_inv, (float4*)inv, n, (cudaStream_t)stream));
    return GSAP_OK;
}

extern "C" gsap_status gsap_k_clear_force_and_boundary(const float* p_pos, const float* p_vel, const float* p_mass,
                                                       float* p_force, float sp, float dp, int32_t np, float dt,
                                                       void* stream) {
    RCK(rb_clear_force_ref((const float4*)p_pos, (const float4*)p_vel, p_mass, (float4*)p_force, sp, dp, np, dt,
                           (cudaStream_t)stream));
    return GSAP_OK;
}

extern "C" gsap_status gsap_k_compute_force_on_particles(const float* p_pos, const float* p_vel, const int32_t* pairs,
                                                         const int32_t* entries, int32_t num_pairs,
                                                         int32_t num_entries, const float* p_mass, float sp, float dp,
                                                         float* p_force, float dt, int32_t quirk, void* stream) {
    RCK(rb_pair_force_ref((const float4*)p_pos, (const float4*)p_vel, (const int2*)pairs, entries, num_pairs,
                          num_entries, num_entries, nullptr, nullptr, p_mass, sp, dp, (float4*)p_force, dt, quirk,
                          num_pairs, (cudaStream_t)stream));
    return GSAP_OK;
}

extern "C" gsap_status gsap_k_update_velocity(float* lin, float* ang, const float* quat, const float* inv_mass,
                                              const float* inv_inertia, const int32_t* shape, const int32_t* pstart,
                                              const int32_t* npart, const float* ref_pos, const float* p_force,
                                              int32_t n, float dt, float max_lin_vel, int32_t cap_vel,
                                              int32_t torque_quirk, void* stream) {
    RCK(rb_update_velocity_ref((float4*)lin, (float4*)ang, (const float4*)quat, inv_mass, (const float4*)inv_inertia,
                               shape, pstart, npart, (const float4*)ref_pos, (const float4*)p_force, n, dt,
                               max_lin_vel, cap_vel, torque_quirk, (cudaStream_t)stream));
    return GSAP_OK;
}
