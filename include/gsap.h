/*
 * gsap.h -- C ABI of the GB300 (sm_103a) sweep-and-prune broadphase and
 * particle rigid-body step.
 *
 * Drop-in boundary for the hot path of liufububai/gSap
 * (physicboxSap2.16_Fermi/): the Sap class (sapDetection/Sap.h:12-24) and the
 * ParticleRigidBody class and its PRBWrap launchers
 * (ParticleRigidBody/ParticleRigidBody.h:46-164,
 * ParticleRigidBody/ParticleRigidBodyWrapper.h:11-54).  Every entry point
 * below names the reference interface it replaces.
 *
 * Conventions
 *  - Plain C types only.  "d_" pointers are device pointers owned by the
 *    caller; "h_" pointers are host pointers.  A float4 array is 4 floats per
 *    element, 16-byte aligned.  `stream` is a cudaStream_t passed as void*
 *    (NULL = the legacy default stream).
 *  - Handles own all scratch; nothing is allocated inside a step after the
 *    handle is created (so a step can be captured in a CUDA graph).
 *  - Every call returns a gsap_status.  On GSAP_ERR_CAPACITY the count
 *    outputs hold the required size.  gsap_last_error() gives a message for
 *    the last failing call on the calling thread.
 *  - Handles are independent: calls on different handles may run
 *    concurrently from different threads; one handle is not reentrant.
 */
#ifndef GSAP_H
#define GSAP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GSAP_VERSION_MAJOR 1
#define GSAP_VERSION_MINOR 1

/* Error handling replaces cutilSafeCall aborts (Sap.cpp:65-86) and the
 * printf-and-return-0 overflow path (SapKernel.cu:2417, :2496). */
typedef enum gsap_status {
    GSAP_OK = 0,
    GSAP_ERR_INVALID = 1,        /* bad argument (null pointer, size, alignment) */
    GSAP_ERR_CAPACITY = 2,       /* an output or scratch capacity is too small */
    GSAP_ERR_CUDA = 3,           /* a CUDA runtime call failed */
    GSAP_ERR_DEVICE_TIMEOUT = 4, /* a bounded device-side wait gave up */
    GSAP_ERR_NONFINITE = 5       /* NaN or Inf in the input bounds */
} gsap_status;

/* Overlap predicate. */
enum {
    GSAP_MODE_AABB = 0,   /* closed 3-D AABB test, Aabb::overlaps (include/aabb.h:47-57) */
    GSAP_MODE_SPHERE = 1  /* strict |ci-cj|^2 < (ri+rj)^2 (SapKernel.cu:1897-1903) */
};

/* Sweep-axis choice. */
enum {
    GSAP_AXIS_PCA = 0, /* eigenvector of the largest eigenvalue of the centre covariance (FP64 solve) */
    GSAP_AXIS_REF = 1  /* coordinate axis of largest variance, as axisVecMultiple (SapKernel.cu:63-97) */
};

/* Flags of the broadphase calls. */
#define GSAP_FLAG_SORTED 0x1u /* output sorted by (i, j); otherwise any order */
#define GSAP_FLAG_GRAPH 0x2u  /* run the pipeline as a cached CUDA graph */
/* Temporal coherence for frame-to-frame calls: the call sweeps with the axes
 * and cell grid computed from the previous call's input (a call of the same
 * n, scene count, mode and settings on this handle) while its own PCA runs
 * beside the sweep and prepares the next call's.  The reference likewise
 * carries its sweep interval from one frame to the next (Sap.cpp:226-243).
 * The pair set is exact either way (any grid gives the same pairs); what
 * changes is the work: if the scene moved far since the previous call the
 * stale grid costs time, and objects that grew a lot can exceed the entry
 * capacity (GSAP_ERR_CAPACITY, after which the next call recomputes first).
 * The first call, or one of a different shape, runs the plain pipeline. */
#define GSAP_FLAG_TEMPORAL 0x4u

typedef struct gsap_config {
    uint32_t mode;          /* GSAP_MODE_* used by gsap_broadphase_* (gsap_sap_collision is always sphere) */
    uint32_t axis_mode;     /* GSAP_AXIS_* */
    uint32_t max_scenes;    /* scenes per batched call (>= 1) */
    uint32_t entry_factor;  /* sweep-entry capacity = entry_factor * max_n (0 -> 8) */
    uint32_t pair_factor;   /* internal pair capacity = pair_factor * max_n (0 -> 16) */
    uint32_t sort_bits;     /* radix key width, 16, 24 or 32 (0 -> 32) */
    float cell_factor;      /* cell size / mean projected width on the secondary axes (0 -> 2.0) */
    uint32_t spin_limit;    /* iteration cap of every device-side wait (0 -> default) */
    uint32_t sort_mode;     /* GSAP_SORT_* : how the sweep entries are sorted (0 -> radix) */
    uint32_t sort_tile;     /* keys per radix tile of the broadphase sort: 2048 or 4096 (0 -> 4096) */
} gsap_config;

/* Sort of the sweep entries (the pair set is the same either way). */
enum {
    GSAP_SORT_RADIX = 0,  /* LSD onesweep radix passes over all entries */
    GSAP_SORT_BUCKET = 1  /* counting scatter into sub-buckets, then a shared-memory sort of each */
};

/* Fills *cfg with the defaults. */
void gsap_config_default(gsap_config* cfg);

/* Message of the last failing call on this thread ("" if none). */
const char* gsap_last_error(void);

/* ------------------------------------------------------------ broadphase */

typedef struct gsap_sap gsap_sap;

/* Replaces Sap::Sap(uint mNbSpheres) (sapDetection/Sap.cpp:12-87): allocates
 * the scratch for up to max_n objects (summed over scenes for batched
 * calls) on the current device.  Returns NULL on failure. */
gsap_sap* gsap_sap_create(uint32_t max_n, const gsap_config* cfg);

/* Replaces Sap::~Sap() (Sap.cpp:89-114). */
void gsap_sap_destroy(gsap_sap* h);

/* Replaces Sap::collision(float spacing, float4* d_particleData, int2* pairs,
 * int* pairsEntries, int* NPairs, int* NPEntries) (Sap.cpp:211-335).
 * d_spheres: n float4 (x, y, z, r).  Output in the reference's format: every
 * overlapping pair in both directions, zero-based int2, sorted by (first,
 * second), unique; d_pair_entries[k] = index of the first pair of the k-th
 * distinct first id (SapKernel.cu:2338-2360).  `spacing` is accepted for
 * signature compatibility (the reference uses it only as the quadrant key
 * offset of its first call, Sap.cpp:226-232) and does not change the result.
 * pair_cap / entry_cap are the capacities of d_pairs (in int2) and
 * d_pair_entries; the reference leaves them unchecked (Sap.cpp:326-329).
 * Blocks until the counts are on the host, as the reference does. */
gsap_status gsap_sap_collision(gsap_sap* h, float spacing, const float* d_spheres, uint32_t n,
                               int32_t* d_pairs, int32_t* d_pair_entries,
                               int32_t* h_num_pairs, int32_t* h_num_entries,
                               uint64_t pair_cap, uint64_t entry_cap, void* stream);

/* AABB-list form of the per-step broadphase (same pipeline as
 * Sap::collision, AABB or sphere predicate from cfg.mode).
 * d_min / d_max: n float4 each (xyz used; for GSAP_MODE_SPHERE d_min holds
 * the spheres and d_max may be NULL).  Writes up to pair_cap pairs (i, j),
 * i < j, as interleaved uint32 to d_pairs.  The count goes to *d_count
 * (device, may be NULL; written asynchronously) and to *h_count (host, may
 * be NULL; if given the call synchronizes the stream).  With
 * GSAP_FLAG_SORTED the list is sorted by (i, j). */
gsap_status gsap_broadphase_aabb(gsap_sap* h, const float* d_min, const float* d_max, uint32_t n,
                                 uint32_t* d_pairs, uint64_t pair_cap,
                                 uint64_t* d_count, uint64_t* h_count,
                                 uint32_t flags, void* stream);

/* Batched broadphase: S independent scenes, scene s holding objects
 * [d_scene_offsets[s], d_scene_offsets[s+1]) of d_min / d_max (device array
 * of S+1 uint32, d_scene_offsets[0] = 0, d_scene_offsets[S] = n).  Pairs
 * (i, j), i < j, use global object ids and never cross a scene.  One launch
 * per pipeline stage for all scenes.  Offsets that decrease or do not run
 * from 0 to n are clamped on the device (nothing outside the input is read)
 * and reported as GSAP_ERR_INVALID when the call's status is read.  No
 * reference counterpart (the reference handles one scene per Sap object). */
gsap_status gsap_broadphase_batched(gsap_sap* h, const float* d_min, const float* d_max,
                                    const uint32_t* d_scene_offsets, uint32_t num_scenes, uint32_t n,
                                    uint32_t* d_pairs, uint64_t pair_cap,
                                    uint64_t* d_count, uint64_t* h_count,
                                    uint32_t flags, void* stream);

/* Reads and clears the device error word of the handle after an
 * asynchronous call (synchronizes the stream). */
gsap_status gsap_sap_check(gsap_sap* h, void* stream);

/* Axes and statistics of scene `scene` from the last call (synchronizes):
 * out[0..8] = u1, u2, u3 (rows), out[9..11] = eigenvalues (descending),
 * out[12..14] = centre mean.  For tests and diagnostics. */
gsap_status gsap_sap_scene_axes(gsap_sap* h, uint32_t scene, double* out, void* stream);

/* Per-stage timings (ms) of the last call made with timing enabled
 * (stage order: pca, project, sort, sweep, canonical).  Returns the number
 * of stages written. */
int gsap_sap_stage_times(gsap_sap* h, float* out_ms, int max_stages);
void gsap_sap_enable_timing(gsap_sap* h, int enable);

/* Autotuner: runs the broadphase on the given input (single scene when
 * d_scene_offsets is NULL, else batched) for every setting of a small grid
 * -- key width 24/32 bits (three or four radix passes) x cell factor
 * 1.0/1.5/2.0/2.5/3.0 (the u2/u3 cell edge, which trades sort volume
 * against sweep run length) -- times `reps` calls of each with CUDA events
 * on `stream`, and keeps the fastest setting in the handle (written to *out
 * if non-NULL).  d_pairs/pair_cap are used as output scratch.  Settings
 * that overflow the handle's capacities are skipped.  Any setting yields
 * the same pair set.  Synchronises `stream`.  No reference counterpart
 * (the reference reuses a fixed interval between frames, Sap.cpp:226-243). */
gsap_status gsap_sap_autotune(gsap_sap* h, const float* d_min, const float* d_max,
                              const uint32_t* d_scene_offsets, uint32_t num_scenes, uint32_t n,
                              uint32_t* d_pairs, uint64_t pair_cap, uint32_t flags, int reps,
                              gsap_config* out, void* stream);

/* Stable LSD radix sort of n (key, value) uint32 pairs on the low `bits`
 * bits with the onesweep kernels of the broadphase (decoupled look-back,
 * 8-bit digits).  Sorts in place; uses the handle's scratch (n must not
 * exceed its entry capacity); d_vals may be NULL (keys only).  Replaces
 * RadixSort::sort(uint* keys, uint* values, uint numElements, uint keyBits)
 * (sapDetection/radixsort.h:151-168).  For keys below 2^bits the order is
 * the reference's at every n (its paths for n <= 1024 sort on all 32 bits,
 * radixsort.cu:1396-1412). */
gsap_status gsap_radix_sort_u32(gsap_sap* h, uint32_t* d_keys, uint32_t* d_vals, uint32_t n,
                                uint32_t bits, void* stream);

/* Stable LSD radix sort of n float keys and uint32 values (d_vals may be
 * NULL), in place, on the handle's scratch.  Replaces RadixSort::sort(float*
 * keys, uint* values, uint numElements, uint keyBits, bool negativeKeys)
 * (sapDetection/radixsort.h:180-198), the overload of the reference's hot
 * path (sapDetection/Sap.cpp:235, keyBits 32 and negativeKeys true).
 *  - negative_keys != 0: ascending float order, -inf < ... < -0.0 < +0.0 <
 *    ... < +inf (NaNs with the sign bit set come first, the others last),
 *    through the order-preserving bit map of radixsort.cu:110-137, applied
 *    as the first pass loads the keys and undone as the last pass stores
 *    them.  key_bits must be 32: with fewer bits the reference sorts the
 *    mapped keys on their low bits and, for n > 1024, leaves them mapped
 *    (radixsort.cu:1414-1478), which this entry point does not reproduce.
 *  - negative_keys == 0: the keys' bit patterns are sorted as unsigned
 *    integers on their low key_bits bits (ascending for non-negative
 *    floats), as the reference does without the map. */
gsap_status gsap_radix_sort_f32(gsap_sap* h, float* d_keys, uint32_t* d_vals, uint32_t n,
                                uint32_t key_bits, int negative_keys, void* stream);

/* The same sort for callers that may not allocate device memory when they
 * sort (a pool allocator that owns the device, an allocation-free section
 * of a stream, a plugin handed only its buffers).  No counterpart in the
 * reference.  Needs no handle: its scratch is a fixed static device array,
 * so it makes no cudaMalloc/cudaFree call and calls no allocating library.
 *   - n is at most GSAP_NOALLOC_SORT_MAX_N; larger n returns
 *     GSAP_ERR_CAPACITY before any work is queued.
 *   - The first call on each device does the set-up (looks up the array,
 *     zeroes its control block and look-back words, synchronises the
 *     device).  A set-up that failed is retried by the next call.
 *   - d_keys / d_vals must be device memory of the current device; other
 *     pointers return GSAP_ERR_INVALID before any work is queued.
 *   - One scratch per device: calls that overlap in time (other streams,
 *     other host threads) race.  Serialise them.
 *   - d_vals may be NULL (keys only).  Synchronises `stream` to read the
 *     device error word. */
#define GSAP_NOALLOC_SORT_MAX_N (1u << 20)
gsap_status gsap_radix_sort_u32_noalloc(uint32_t* d_keys, uint32_t* d_vals, uint32_t n, uint32_t bits,
                                        void* stream);

/* ----------------------------------------------------------- rigid bodies */

typedef struct gsap_rb gsap_rb;

/* Host-side body data, mirror of ParticleRigidBody::RigidBodyData
 * (ParticleRigidBody.h:52-67).  inv_inertia: 12 floats per body (three
 * float4 rows, the Matrix3x3 layout). */
typedef struct gsap_body_data {
    int32_t n_bodies;
    int32_t n_total_particles;
    const float* pos;       /* float4 */
    const float* quat;      /* float4 (x, y, z, w), normalised by the call */
    const float* lin_vel;   /* float4 */
    const float* ang_vel;   /* float4 */
    const int32_t* shape_idx;
    const int32_t* p_start; /* m_pBufferStartOffset */
    const int32_t* n_part;  /* m_numParticles */
    const float* inv_mass;
    const float* inv_inertia;
} gsap_body_data;

/* Contact model. */
enum {
    GSAP_CONTACT_REF = 0,   /* reference formulas (ParticleRigidBodyKernel.h:13-22, :106-208) */
    GSAP_CONTACT_CONFIG = 1 /* spring k, damping eta, tangential ratio kt, six walls */
};

typedef struct gsap_contact_params {
    uint32_t model;        /* GSAP_CONTACT_* */
    /* reference model */
    float sp_multip, dp_multip; /* setParams (ParticleRigidBody.h:87) */
    float max_lin_vel;          /* setMaxVelocity result; <= 0 disables the cap */
    float gravity_y;            /* reference: -5 (ParticleRigidBodyKernel.h:55) */
    uint32_t floor_clamp;       /* reference's (idx/6)%2 floor clamp (:65-68) */
    uint32_t torque_quirk;      /* reference's angVel += tau*dt (:260-261) */
    uint32_t pair_loop_quirk;   /* reference's pair loop stops after pair index numPairEntries (:201) */
    /* config model */
    float k, eta, kt;
    float box_lo[3], box_hi[3];
} gsap_contact_params;

/* Replaces ParticleRigidBody(int maxNumBodies, int maxNumParticles, int
 * maxPairs) (ParticleRigidBody.cpp:15-50). */
gsap_rb* gsap_rb_create(int32_t max_bodies, int32_t max_particles, int32_t max_pairs);
/* Replaces ~ParticleRigidBody() (ParticleRigidBody.cpp:52-76). */
void gsap_rb_destroy(gsap_rb* h);
/* Replaces setRbData (ParticleRigidBody.cpp:78-110; GL buffer set-up dropped). */
gsap_status gsap_rb_set_body_data(gsap_rb* h, const gsap_body_data* host);
/* Replaces setParticleData(float4* pos, float* mass, int n) (:112-116):
 * reference particle positions (w = radius) and masses, indexed
 * 10*shape + k (MAX_NUM_PARTICLES = 10). */
gsap_status gsap_rb_set_particle_data(gsap_rb* h, const float* h_ref_pos, const float* h_mass, int32_t n);
/* Replaces setParticleShapeInvInertia(Matrix3x3*, int) (:118-121); 12 floats per shape. */
gsap_status gsap_rb_set_shape_inv_inertia(gsap_rb* h, const float* h_inv_inertia, int32_t n_shapes);
/* Replaces setParams / setMaxVelocity (ParticleRigidBody.h:87-88) and adds
 * the config-mode parameters. */
gsap_status gsap_rb_set_contact(gsap_rb* h, const gsap_contact_params* p);
/* Scene partition of the bodies for batched dynamics: scene s owns bodies
 * [h_body_offsets[s], h_body_offsets[s+1]).  Each scene has its own walls
 * (the same box) and its bodies meet only bodies of the same scene. */
gsap_status gsap_rb_set_scenes(gsap_rb* h, const uint32_t* h_body_offsets, uint32_t num_scenes);

/* The five device steps of the reference, on the handle's state. */
gsap_status gsap_rb_update_particle_data(gsap_rb* h, void* stream);         /* updateParticleData (:123-136) */
gsap_status gsap_rb_prepare(gsap_rb* h, void* stream);                      /* prepare (:138-146) */
gsap_status gsap_rb_compute_forces(gsap_rb* h, float dt, void* stream);     /* comupteFoceOnParticles (:148-167) */
gsap_status gsap_rb_update_velocity(gsap_rb* h, float dt, void* stream);    /* updateVelocity (:169-180) */
gsap_status gsap_rb_integrate(gsap_rb* h, float dt, void* stream);          /* integrate (:182-191) */

/* Pair list used by gsap_rb_compute_forces in the reference model
 * (getPairs/getPairEntries/setNumPairs/setNumPairEntries,
 * ParticleRigidBody.h:99-104). */
int32_t* gsap_rb_pairs(gsap_rb* h);          /* device int2[max_pairs] */
int32_t* gsap_rb_pair_entries(gsap_rb* h);   /* device int[max_particles] */
gsap_status gsap_rb_set_num_pairs(gsap_rb* h, int32_t num_pairs, int32_t num_entries);
float* gsap_rb_particle_pos(gsap_rb* h);     /* getParticlePos: device float4 (w = radius) */
float* gsap_rb_particle_vel(gsap_rb* h);     /* getParticleVel */
float* gsap_rb_particle_force(gsap_rb* h);   /* getParticleForce */

/* One whole step in the reference order (demoParticles.h:875-912):
 * integrate, particle placement, broadphase, prepare, forces, velocity.
 * Reference model: particle-sphere broadphase through `bp` in the
 * Sap::collision format.  Config model: body-AABB broadphase through `bp`
 * then particle contact between overlapping bodies (per scene when scenes
 * are set).  No host synchronisation inside the step.  The broadphase runs
 * with GSAP_FLAG_TEMPORAL (the previous step's cell grid; exact pairs either
 * way), as the reference's step carries its sweep interval over. */
gsap_status gsap_rb_step(gsap_rb* h, gsap_sap* bp, float dt, void* stream);

/* Handle-owned arrays for gsap_rb_copy_out / gsap_rb_copy_in. */
enum {
    GSAP_RB_PARTICLE_POS = 0,   /* float4 per particle (w = radius) */
    GSAP_RB_PARTICLE_VEL = 1,   /* float4 per particle */
    GSAP_RB_PARTICLE_FORCE = 2, /* float4 per particle */
    GSAP_RB_PAIRS = 3,          /* int2 per pair (reference model list) */
    GSAP_RB_PAIR_ENTRIES = 4,   /* int per entry */
    GSAP_RB_INV_INERTIA = 5     /* 12 floats per body (written by prepare) */
};
/* Host copies of handle-owned device arrays (headless readback of the
 * reference's getters, ParticleRigidBody.h:99-116); `bytes` must fit the
 * array's capacity.  Synchronous. */
gsap_status gsap_rb_copy_out(gsap_rb* h, int32_t which, void* h_dst, uint64_t bytes, void* stream);
gsap_status gsap_rb_copy_in(gsap_rb* h, int32_t which, const void* h_src, uint64_t bytes, void* stream);

/* Copies the body state to host arrays (float4 each; any may be NULL).
 * Headless replacement of the GL pose export (ParticleRigidBody.cpp:88-98). */
gsap_status gsap_rb_get_state(gsap_rb* h, float* h_pos, float* h_quat, float* h_lin_vel,
                              float* h_ang_vel, void* stream);

/* The inverse of gsap_rb_get_state: overwrites the body state of the
 * n_bodies bodies from host float4 arrays (any may be NULL), bit for bit --
 * the state half of setRbData (ParticleRigidBody.cpp:78-110) without its
 * quaternion normalisation, for restarting from a snapshot or re-syncing
 * to an external trajectory.  Synchronous. */
gsap_status gsap_rb_set_state(gsap_rb* h, const float* h_pos, const float* h_quat, const float* h_lin_vel,
                              const float* h_ang_vel, void* stream);

/* Low-level launchers on caller-owned device arrays, replacing the PRBWrap
 * functions (ParticleRigidBodyWrapper.h:15-50) without dim3 arguments
 * (launch shapes are internal). */
gsap_status gsap_k_integrate(float* d_pos, float* d_quat, float* d_lin_vel, float* d_ang_vel,
                             float dt, int32_t n, const gsap_contact_params* p, void* stream);
gsap_status gsap_k_update_particle_data(const float* d_pos, const float* d_quat, const float* d_lin_vel,
                                        const float* d_ang_vel, const int32_t* d_shape_idx,
                                        const int32_t* d_p_start, const int32_t* d_n_part,
                                        const float* d_ref_pos, const float* d_ref_mass,
                                        float* d_p_pos, float* d_p_vel, float* d_p_mass,
                                        int32_t n, void* stream);
gsap_status gsap_k_prepare(const float* d_quat, const int32_t* d_shape_idx, const float* d_shape_inv_inertia,
                           float* d_inv_inertia, int32_t n, void* stream);
gsap_status gsap_k_clear_force_and_boundary(const float* d_p_pos, const float* d_p_vel, const float* d_p_mass,
                                            float* d_p_force, float sp_multip, float dp_multip,
                                            int32_t n_particles, float dt, void* stream);
gsap_status gsap_k_compute_force_on_particles(const float* d_p_pos, const float* d_p_vel,
                                              const int32_t* d_pairs, const int32_t* d_pair_entries,
                                              int32_t num_pairs, int32_t num_entries,
                                              const float* d_p_mass, float sp_multip, float dp_multip,
                                              float* d_p_force, float dt, int32_t pair_loop_quirk,
                                              void* stream);
gsap_status gsap_k_update_velocity(float* d_lin_vel, float* d_ang_vel, const float* d_quat,
                                   const float* d_inv_mass, const float* d_inv_inertia,
                                   const int32_t* d_shape_idx, const int32_t* d_p_start,
                                   const int32_t* d_n_part, const float* d_ref_pos,
                                   const float* d_p_force, int32_t n, float dt,
                                   float max_lin_vel, int32_t cap_vel, int32_t torque_quirk,
                                   void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GSAP_H */
