// Internal declarations of the particle rigid-body kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gsap {

constexpr int kMaxParticlesPerBody = 10;  // MAX_NUM_PARTICLES (ParticleRigidBody.h:39)
constexpr int kMaxShapes = 64;

// reference model (rigid_ref.cu, compiled with -fmad=false)
cudaError_t rb_integrate_ref(float4* pos, float4* quat, float4* lin, float4* ang, float dt, int n, float gy,
                             int floor_clamp, cudaStream_t st);
cudaError_t rb_place_ref(const float4* pos, const float4* quat, const float4* lin, const float4* ang,
                         const int* shape, const int* pstart, const int* npart, const int* p_body,
                         const float4* ref_pos, const float* ref_mass, float4* p_pos, float4* p_vel, float* p_mass,
                         int n, int np, cudaStream_t st);
cudaError_t rb_prepare_ref(const float4* quat, const int* shape, const float4* shape_inv, float4* inv_out, int n,
                           cudaStream_t st);
cudaError_t rb_clear_force_ref(const float4* p_pos, const float4* p_vel, const float* p_mass, float4* p_force,
                               float sp, float dp, int np, float dt, cudaStream_t st);
cudaError_t rb_pair_force_ref(const float4* p_pos, const float4* p_vel, const int2* pairs, const int* entries,
                              int num_pairs, int num_entries, int max_entries, const unsigned long long* d_np2,
                              const uint32_t* d_ne, const float* p_mass, float sp, float dp, float4* p_force,
                              float dt, int quirk, int pair_cap, cudaStream_t st);
cudaError_t rb_update_velocity_ref(float4* lin, float4* ang, const float4* quat, const float* inv_mass,
                                   const float4* inv_inertia, const int* shape, const int* pstart, const int* npart,
                                   const float4* ref_pos, const float4* p_force, int n, float dt, float max_lin_vel,
                                   int cap, int torque_quirk, cudaStream_t st);

// config model (rigid_cfg.cu)
struct CfgParams {
    float dt, k, eta, kt, gy;
    float lo[3], hi[3];
    unsigned long long* contacts;  // if set: += particle-particle contacts, counted from both sides
};
// pos_lo: the low parts of the float-float body positions (nullptr: plain
// FP32 positions)
cudaError_t rb_integrate_cfg(float4* pos, float4* pos_lo, float4* quat, float4* lin, const float4* ang,
                             const CfgParams& p, int n, cudaStream_t st);
cudaError_t rb_place_cfg(const float4* quat, const float4* lin, const float4* ang, const int* shape,
                         const int* pstart, const int* p_body, const float4* ref_pos, float4* p_rel, float4* p_vel,
                         int np, cudaStream_t st);
cudaError_t rb_abs_pos(const float4* pos, const float4* pos_lo, const int* p_body, const float4* p_rel, float4* p_pos,
                       int np, cudaStream_t st);
cudaError_t rb_body_aabb(const float4* pos, const float4* pos_lo, const float4* p_rel, const int* pstart,
                         const int* npart, float4* bmin, float4* bmax, int n, cudaStream_t st);
cudaError_t rb_forces_cfg(const float4* pos, const float4* pos_lo, const float4* p_rel, const float4* p_vel,
                          const int* p_body, const int* pstart, const int* npart, const uint2* body_pairs,
                          const uint32_t* rowoff, uint64_t pair_cap, const CfgParams& p, float4* p_force, int np,
                          cudaStream_t st);
cudaError_t rb_update_cfg(float4* lin, float4* ang, const float4* quat, const float* inv_mass, const int* shape,
                          const int* pstart, const int* npart, const float4* ref_pos, const float4* shape_inv,
                          const float4* p_force, const CfgParams& p, int n, cudaStream_t st);

}  // namespace gsap
