/*
 * CPU oracle for the gSap broadphase and particle rigid-body step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: it is loaded by
 * tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline and
 * reference legs, and by nothing else.  The product (gsap_gb300 and
 * libgsap.so) never links, imports or calls it, and has no CPU fallback.
 *
 * Every routine restates the reference's algorithm in plain C; the reference
 * file:line each one follows is given beside it (paths relative to
 * physicboxSap2.16_Fermi/ of liufububai/gSap).  The file is compiled with
 * -ffp-contract=off so that every float expression is evaluated in the
 * written order with one rounding per operation.
 */
#ifndef GSAP_ORACLE_H
#define GSAP_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- broadphase */

/* O(n^2) AABB brute force with Aabb::overlaps semantics (include/aabb.h:47-57,
 * closed intervals on all three axes), pair order as Demo::cpuBroadphase
 * (cudaPhysics/demo.h:404-417): i<j, row-major, which is the sorted (i<j)
 * list.  mn/mx are n float4 (xyz used).  Writes min(count, cap) pairs as
 * interleaved uint32 (i, j); returns the full count. */
int64_t orc_bf_aabb(const float* mn, const float* mx, uint32_t n,
                    uint32_t* pairs, int64_t cap, int threads);

/* O(n^2) sphere brute force (cudaPhysics/demoParticles.h:1506-1537) with the
 * squared strict test of the GPU sweep (sapDetection/SapKernel.cu:1897-1903):
 * d2 = (dx*dx + dy*dy) + dz*dz, overlap iff d2 < (ri+rj)^2.  spheres are n
 * float4 (x, y, z, r).  Same output convention as orc_bf_aabb. */
int64_t orc_bf_sphere(const float* spheres, uint32_t n,
                      uint32_t* pairs, int64_t cap, int threads);

/* The reference's broadphase algorithm restated on the CPU (Sap::collision,
 * sapDetection/Sap.cpp:211-335): max-variance coordinate axis
 * (SapKernel.cu:63-97), four quadrant sweeps about the origin with the
 * quadrant offset in the key (SapKernel.cu:151-213), the cross pass over
 * objects within maxR of the quadrant planes (SapKernel.cu:557-635,
 * :968-1059, Sap.cpp:246-254), exact test, then sort + unique
 * (Sap.cpp:269-295).  mode 0 = AABB (mn, mx), mode 1 = sphere (mn holds the
 * float4 spheres, mx ignored).  Output: the sorted unique (i<j) list. */
int64_t orc_sap_ref(int mode, const float* mn, const float* mx, uint32_t n,
                    uint32_t* pairs, int64_t cap, int threads);

/* Same, with the sweeps started only from slice `part` of `parts` equal,
 * contiguous slices of each group's sorted order (axis choice, partition
 * and the group sorts stay full-size): a bounded sample of the reference
 * algorithm's work at the full scene's density, for timing; the slices
 * part = 0 .. parts-1 together do one full call's sweep work.  parts = 1
 * is orc_sap_ref.  When secs is not NULL the call splits its wall time:
 * secs[1] = the stages that scale with the number of sweep starts (the
 * sweep loops and the sort + unique of the pairs they find), secs[0] =
 * everything else (centres, axis choice, partition, group sorts).  Averaged
 * over the parts, secs[0] + parts * secs[1] is one full call's time. */
int64_t orc_sap_ref_sampled(int mode, const float* mn, const float* mx, uint32_t n, uint32_t parts,
                            uint32_t part, uint32_t* pairs, int64_t cap, int threads, double* secs);

/* The reference's output format (SapKernel.cu:2249-2360, Sap.cpp:326-329)
 * from a sorted unique (i<j) list: both directions (i,j) and (j,i) sorted by
 * (first, second), zero-based int2, plus pairEntries[k] = index of the first
 * pair of the k-th distinct first id.  Returns the number of entries; the
 * number of both-direction pairs is 2*np. */
int64_t orc_both_directions(const uint32_t* pairs, int64_t np,
                            int32_t* out_pairs, int32_t* out_entries);

/* Stable LSD radix sort of (key, value) u32 pairs on the low `bits` bits,
 * the semantic of RadixSort::sort (sapDetection/radixsort.cu:1384-1480). */
void orc_radix_sort_u32(uint32_t* keys, uint32_t* vals, uint32_t n, int bits);

/* Order-preserving float -> u32 key (sapDetection/radixsort.cu:110-121):
 * flips the sign bit of non-negative floats and all bits of negative ones. */
uint32_t orc_float_flip(float f);

/* ----------------------------------------------------------- rigid bodies */

/* One particle-rigid-body step in the reference's own order and formulas
 * (cudaPhysics/demoParticles.h:875-912; kernels in
 * ParticleRigidBody/ParticleRigidBodyKernel.h:30-262), FP32.  State arrays
 * are float4 per body; inv_inertia_shape / inv_inertia_body are 12 floats
 * (3 rows of float4) per shape / body as Matrix3x3 stores them.  The pair
 * list (both directions + pairEntries) for the step is produced by
 * orc_bf_sphere + orc_both_directions on the placed particles, which is the
 * CPU broadphase of DemoParticles::cpuBroadphase. */
typedef struct orc_rb_state {
    int n_bodies;
    int n_particles;
    float* pos;        /* [n_bodies*4] */
    float* quat;       /* [n_bodies*4] (x, y, z, w) */
    float* lin_vel;    /* [n_bodies*4] */
    float* ang_vel;    /* [n_bodies*4] */
    int* shape_idx;    /* [n_bodies] */
    int* p_start;      /* [n_bodies] */
    int* n_part;       /* [n_bodies] */
    float* inv_mass;   /* [n_bodies] */
    float* inv_inertia;/* [n_bodies*12] written by prepare */
    /* per-particle (outputs of the step) */
    float* p_pos;      /* [n_particles*4] w = radius */
    float* p_vel;      /* [n_particles*4] */
    float* p_force;    /* [n_particles*4] */
    float* p_mass;     /* [n_particles] */
    /* shapes */
    const float* ref_pos;          /* [10*n_shapes*4] (MAX_NUM_PARTICLES = 10) */
    const float* ref_mass;         /* [10*n_shapes] */
    const float* shape_inv_inertia;/* [n_shapes*12] */
} orc_rb_state;

typedef struct orc_ref_params {
    float dt;
    float sp_multip;   /* setParams(spM, dpM): ParticleRigidBody.h:87 */
    float dp_multip;
    float max_lin_vel; /* setMaxVelocity: minRadius/dt; <=0 disables the cap */
    float gravity_y;   /* -5 in ParticleRigidBodyKernel.h:55 */
    int floor_clamp;   /* 1 = the (idx/6)%2 clamp of integrateK :65-68 */
    int torque_quirk;  /* 1 = angVel += tau*dt (reference, :260-261); 0 = I^-1 tau dt */
    int pair_loop_quirk; /* 1 = stop a row after pair index numPairEntries (:201) */
} orc_ref_params;

/* Upload normalisation of setRbData (ParticleRigidBody.cpp:82-86):
 * q *= 1 / sqrtf(dot4(q, q)) for n float4 quaternions (quaternion.h:116-128). */
void orc_normalize_quats(float* quat, int n);

/* Reference-order FP32 step.  Uses a brute-force sphere pair list built
 * internally (pair capacity max_pairs).  Returns the number of
 * both-direction pairs used, or -1 on capacity overflow. */
int64_t orc_rb_step_ref(orc_rb_state* s, const orc_ref_params* p,
                        int64_t max_pairs, int threads);

/* Config-mode contact model (spring k, normal damping eta, tangential
 * damping ratio kt, gravity, six walls of an axis-aligned box) in float or
 * double.  Body-AABB broadphase (brute force over bodies, AABB of the
 * particles' spheres) then particle pairs between overlapping bodies. */
typedef struct orc_cfg_params {
    double dt, k, eta, kt, gravity_y;
    double box_lo[3], box_hi[3];
} orc_cfg_params;

typedef struct orc_rb_state_d {
    int n_bodies, n_particles;
    double *pos, *quat, *lin_vel, *ang_vel; /* [n_bodies*4] */
    int *shape_idx, *p_start, *n_part, *scene; /* scene: body -> scene id (may be NULL) */
    double *inv_mass;                       /* [n_bodies] */
    const double *ref_pos;                  /* [10*n_shapes*4] */
    const double *shape_inv_inertia;        /* [n_shapes*9] row-major */
    double *p_pos, *p_vel, *p_force;        /* [n_particles*4] */
} orc_rb_state_d;

/* One config-mode step in double precision.  Returns the number of
 * particle contact pairs (i<j, penetrating or not) examined. */
/* Batched scenes (object ids [off[s], off[s+1]) per scene): the sorted
 * (i<j) pairs of Aabb::overlaps within each scene, scenes in order.
 * Scenes of at most bf_max objects run the O(n^2) loop; larger ones test
 * the pairs whose x intervals meet (found by a sort on min x). */
int64_t orc_pairs_batched(const float* mn, const float* mx, const int64_t* off, int num_scenes, uint32_t bf_max,
                          uint32_t* pairs, int64_t cap, int threads);

int64_t orc_rb_step_cfg_f64(orc_rb_state_d* s, const orc_cfg_params* p, int threads);
/* The same step, flagging in amb[n_bodies] the bodies with a contact whose
 * penetration depth is within +-band of zero (see rb.c). */
int64_t orc_rb_step_cfg_f64_amb(orc_rb_state_d* s, const orc_cfg_params* p, int threads, double band, int* amb);

/* The body pair search of that step: rows of the bodies of the same scene
 * whose closed AABBs (bmin/bmax: 3 doubles per body) meet, ascending ids;
 * brute != 0 tests all pairs, else a sort-and-sweep on min x (same set).
 * cnt: nb + 1 row offsets.  Returns the total, or -1 when cap is short
 * (cnt[nb] then holds the total). */
int64_t orc_body_neighbours(int nb, const double* bmin, const double* bmax, const int* scene, int brute,
                            int threads, int* cnt, int* nbr, int64_t cap);

#ifdef __cplusplus
}
#endif
#endif
