/*
 * Host harness around the reference's OWN source, used only to pin the CPU
 * oracle (test infrastructure; built by `make ref` into oracle/_ref/ from the
 * reference tree in place -- no reference source is copied into this repo).
 *
 *  - Aabb::overlaps from include/aabb.h:47-57 drives an O(n^2) brute force
 *    in the pair order of Demo::cpuBroadphase (cudaPhysics/demo.h:404-417).
 *  - The particle rigid-body kernels of
 *    ParticleRigidBody/ParticleRigidBodyKernel.h:30-262 are compiled for the
 *    host (with a host compiler the CUDA headers expand __device__ and
 *    __global__ to nothing) and run as loops over the launch grid that
 *    ParticleRigidBody.cpp:123-191 uses, one emulated thread at a time.
 *    The class header ParticleRigidBody.h needs GL, so it is bypassed: the
 *    only member the kernels use, getParticleRefIdx (ParticleRigidBody.h:137-138),
 *    is declared here with the same body.
 */
#include <cuda_runtime.h>
#include <stdint.h>

static uint3 threadIdx;
static dim3 blockDim;
static uint3 blockIdx;

#define PARTICLE_RIGID_BODY
#define MAX_NUM_PARTICLES 10
#define MAX_PARTICLE_SHAPE_TYPE 4
struct ParticleRigidBody {
    static int getParticleRefIdx(int shapeIdx, int idx) { return MAX_NUM_PARTICLES * shapeIdx + idx; }
};
#include "ParticleRigidBodyKernel.h"
#include "aabb.h"

/* Emulated launch: 64-thread blocks as setGridBlockSize (ParticleRigidBody.h:122-134). */
template <class F>
static void launch(int n, F&& body) {
    const int bs = 64;
    int grid = n / bs + ((n % bs) ? 1 : 0);
    if (grid == 0) grid = 1;
    blockDim = dim3(bs, 1, 1);
    for (int b = 0; b < grid; ++b)
        for (int t = 0; t < bs; ++t) {
            blockIdx = make_uint3(b, 0, 0);
            threadIdx = make_uint3(t, 0, 0);
            body();
        }
}

extern "C" {

int64_t ref_bf_aabb(const float* mn, const float* mx, uint32_t n, uint32_t* pairs, int64_t cap) {
    int64_t np = 0;
    for (uint32_t i = 0; i < n; ++i) {
        Aabb a;
        a.m_min = make_float4(mn[4 * i], mn[4 * i + 1], mn[4 * i + 2], mn[4 * i + 3]);
        a.m_max = make_float4(mx[4 * i], mx[4 * i + 1], mx[4 * i + 2], mx[4 * i + 3]);
        for (uint32_t j = i + 1; j < n; ++j) {
            Aabb b;
            b.m_min = make_float4(mn[4 * j], mn[4 * j + 1], mn[4 * j + 2], mn[4 * j + 3]);
            b.m_max = make_float4(mx[4 * j], mx[4 * j + 1], mx[4 * j + 2], mx[4 * j + 3]);
            if (a.overlaps(b)) {
                if (np < cap) { pairs[2 * np] = i; pairs[2 * np + 1] = j; }
                ++np;
            }
        }
    }
    return np;
}

/* The upload normalisation of setRbData (ParticleRigidBody.cpp:82-86):
 * Quaternion::normalizeQ on every body quaternion. */
void ref_normalize_quats(float4* quat, int n) {
    for (int i = 0; i < n; ++i) ((Quaternion*)quat)[i].normalizeQ();
}

void ref_integrate(float4* pos, float4* quat, float4* linVel, float4* angVel, float dt, int n) {
    launch(n, [&] { integrateK(pos, (Quaternion*)quat, linVel, angVel, dt, n); });
}

void ref_update_particle_data(float4* pos, float4* quat, float4* linVel, float4* angVel,
                              int* shapeIdx, int* pStart, int* numParticles,
                              float4* refPos, float* refMass,
                              float4* pPos, float4* pVel, float* pMass, int n) {
    launch(n, [&] {
        updateParticleDataK(pos, (Quaternion*)quat, linVel, angVel, shapeIdx, pStart, numParticles,
                            refPos, refMass, pPos, pVel, pMass, n);
    });
}

void ref_prepare(float4* quat, int* shapeIdx, float* shapeInvInertia, float* rbInvInertia, int n) {
    launch(n, [&] {
        prepareK((Quaternion*)quat, shapeIdx, (Matrix3x3*)shapeInvInertia, (Matrix3x3*)rbInvInertia, n);
    });
}

void ref_clear_force(float4* pPos, float4* pVel, float* pMass, float4* pForce,
                     float spM, float dpM, int np, float dt) {
    launch(np, [&] { clearForceAndBoundaryConditionK(pPos, pVel, pMass, pForce, spM, dpM, np, dt); });
}

void ref_pair_force(float4* pPos, float4* pVel, int2* pairs, int* pairEntries, int numPairEntries,
                    float* pMass, float spM, float dpM, float4* pForce, float dt) {
    launch(numPairEntries, [&] {
        comupteFoceOnParticlesK(pPos, pVel, pairs, pairEntries, numPairEntries, pMass, spM, dpM, pForce, dt);
    });
}

void ref_update_velocity(float4* linVel, float4* angVel, float4* quat, float* invMass, float* invInertia,
                         int* shapeIdx, int* pStart, int* numParticles, float4* refPos, float4* pForce,
                         int n, float dt, float maxLinVel, int capVel) {
    launch(n, [&] {
        if (capVel)
            updateVelocityK<true>(linVel, angVel, (Quaternion*)quat, invMass, (Matrix3x3*)invInertia,
                                  shapeIdx, pStart, numParticles, refPos, pForce, n, dt, maxLinVel);
        else
            updateVelocityK<false>(linVel, angVel, (Quaternion*)quat, invMass, (Matrix3x3*)invInertia,
                                   shapeIdx, pStart, numParticles, refPos, pForce, n, dt, maxLinVel);
    });
}

} /* extern "C" */
