// K4: the sweep.
//
// Replaces the reference's sweep set-up and candidate kernels
// (sapDetection/SapKernel.cu:2448-2517: reorderSphere, calBoxHashSub32,
// CounterThreadSphPCATexSub + CUDPP scan + a blocking read of the thread
// total, assignThreadIDSphere, ZeroSetSphere, kernel_SphereTexCullPCAElong
// :1810-1921 writing a column-major candidate matrix, a second CUDPP scan, a
// second blocking read and the compaction assemPairsSphereSub :1649-1695),
// and the cross pass of SapKernel.cu:2364-2446.
//
// Persistent warps take 32 consecutive sorted entries at a time from an
// atomic counter (work stealing).  Each lane scans forward from its entry,
// kUnroll candidates per iteration with their loads issued together,
// while the candidate key is <= (bucket | q(hi1)): the q map is monotone, so
// every later entry of the same cell whose interval on u1 can meet this one
// is visited, and the scan stops at the cell (and scene) boundary by
// construction.  The last sort pass wrote every entry's bounds and
// lower-corner cell in sorted order, so lane L at step k reads entry
// e + L + k: the 32 lanes read one contiguous run and the next step re-reads
// it shifted by one (L1 hits) -- no random gathers in the hot loop.
// Candidates pass the exact test on the original FP32 bounds (closed AABB
// test of Aabb::overlaps, include/aabb.h:47-57, or the strict squared
// sphere test of SapKernel.cu:1897-1903 with one rounding per operation)
// and the owner-cell rule: a pair is reported only in the cell holding
// (max(lo2_i, lo2_j), max(lo3_i, lo3_j)), which both objects touch, so each
// overlapping pair comes out exactly once and no sort + unique pass is
// needed.  Hits are compacted through a per-warp shared-memory buffer that
// reserves global space with one atomic per up to 128 pairs.
#include "internal.cuh"

namespace gsap {

__device__ __forceinline__ float proj_hi(const float* u, float3 a, float3 b) {
    float h0 = fmaxf(__fmul_ru(u[0], a.x), __fmul_ru(u[0], b.x));
    float h1 = fmaxf(__fmul_ru(u[1], a.y), __fmul_ru(u[1], b.y));
    float h2 = fmaxf(__fmul_ru(u[2], a.z), __fmul_ru(u[2], b.z));
    return __fadd_ru(__fadd_ru(h0, h1), h2);
}

constexpr int kBuf = 128;  // pairs buffered per warp before a global reservation
constexpr int kUnroll = 4; // candidates per lane per iteration (loads issued together)

template <int MODE>
__global__ void __launch_bounds__(kThreads) k_sweep(BpScratch S, BpArgs A, const uint32_t* __restrict__ keys,
                                                    const uint32_t* __restrict__ vals, uint2* __restrict__ pairs,
                                                    uint64_t pair_cap, int count_rows) {
    __shared__ uint2 s_buf[kThreads / 32][kBuf];
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t lt = lanemask_lt();
    Ctrl* C = S.ctrl;
    const float4* __restrict__ smin = S.smin;
    const float4* __restrict__ smax = S.smax;
    const uint32_t* __restrict__ scell = S.scell;
    const uint32_t E = (uint32_t)min((uint64_t)C->entry_count, S.entry_cap);
    const uint32_t Q = C->qbits;
    const uint32_t qmask = (1u << Q) - 1u;
    const float qmax = (float)qmask;
    uint32_t nbuf = 0;
    uint32_t my_tests = 0, iters = 0;

    auto flush = [&]() {
        __syncwarp();
        unsigned long long base = 0;
        if (lane == 0 && nbuf) base = atomicAdd(&C->pair_count, (unsigned long long)nbuf);
        base = __shfl_sync(0xffffffffu, base, 0);
        for (uint32_t k = lane; k < nbuf; k += 32) {
            uint2 p = s_buf[wid][k];
            if (base + k < pair_cap) {  // rows count stored pairs only: the scatter undoes exactly these
                pairs[base + k] = p;
                if (count_rows) {
                    atomicAdd(&S.rowcnt[p.x], 1u);
                    if (count_rows == 2) atomicAdd(&S.rowcnt[p.y], 1u);
                }
            }
        }
        __syncwarp();
        nbuf = 0;
    };

    while (true) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&C->sweep_ctr, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= E) break;
        const uint32_t e = base + lane;
        bool live = e < E;
        uint32_t i = 0, kb = 0, bucket = 0, ci = 0, bbase = 0, g3 = 1;
        float4 pa = make_float4(0.f, 0.f, 0.f, 0.f), pb = pa;
        if (live) {
            const uint32_t key = keys[e];
            i = vals[e];
            const Scene* sc = &S.scenes[S.objscene ? S.objscene[i] : 0u];
            pa = smin[e];
            float3 a, b;
            if (MODE == 0) {
                pb = smax[e];
                a = make_float3(pa.x, pa.y, pa.z);
                b = make_float3(pb.x, pb.y, pb.z);
            } else {
                float r = fabsf(pa.w);
                a = make_float3(__fsub_rd(pa.x, r), __fsub_rd(pa.y, r), __fsub_rd(pa.z, r));
                b = make_float3(__fadd_ru(pa.x, r), __fadd_ru(pa.y, r), __fadd_ru(pa.z, r));
            }
            float u[3] = {sc->u[0], sc->u[1], sc->u[2]};
            float h1 = proj_hi(u, a, b);
            float t = __fmul_rn(__fsub_rn(h1, sc->q_org), sc->q_scale);
            uint32_t qh = (uint32_t)fminf(fmaxf(t, 0.f), qmax);
            kb = (key & ~qmask) | qh;
            bucket = key >> Q;
            bbase = sc->bucket_base;
            g3 = sc->G3;
            ci = scell[e];
        }
        uint32_t j = e + 1;
        while (true) {
            // the next kUnroll candidates: keys are sorted, so the active ones form a prefix
            bool act[kUnroll];
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) {
                const uint32_t jj = j + u;
                act[u] = live && jj < E && __ldg(keys + jj) <= kb;
            }
#pragma unroll
            for (int u = 1; u < kUnroll; ++u) act[u] = act[u] && act[u - 1];
            if (!__any_sync(0xffffffffu, act[0])) break;
            ++iters;
            float4 qa[kUnroll], qb[kUnroll];
#pragma unroll
            for (int u = 0; u < kUnroll; ++u)
                if (act[u]) {
                    qa[u] = __ldg(smin + j + u);
                    if (MODE == 0) qb[u] = __ldg(smax + j + u);
                }
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) {
                bool hit = false;
                uint32_t o = 0;
                if (act[u]) {
                    ++my_tests;
                    bool ov;
                    if (MODE == 0) {
                        ov = (pa.x <= qb[u].x) & (qa[u].x <= pb.x) & (pa.y <= qb[u].y) & (qa[u].y <= pb.y) &
                             (pa.z <= qb[u].z) & (qa[u].z <= pb.z);
                    } else {
                        float dx = __fsub_rn(pa.x, qa[u].x), dy = __fsub_rn(pa.y, qa[u].y),
                              dz = __fsub_rn(pa.z, qa[u].z);
                        float t1 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                        float r = __fadd_rn(pa.w, qa[u].w);
                        ov = t1 < __fmul_rn(r, r);
                    }
                    if (ov) {
                        // owner-cell rule: the pair belongs to the cell of (max lo2, max lo3)
                        const uint32_t co = __ldg(scell + j + u);
                        const uint32_t own = bbase + max(ci >> 16, co >> 16) * g3 + max(ci & 0xFFFFu, co & 0xFFFFu);
                        if (own == bucket) {
                            hit = true;
                            o = __ldg(vals + j + u);
                        }
                    }
                }
                const uint32_t hm = __ballot_sync(0xffffffffu, hit);
                if (hm) {
                    const uint32_t cnt = __popc(hm);
                    if (nbuf + cnt > kBuf) flush();
                    if (hit) s_buf[wid][nbuf + __popc(hm & lt)] = make_uint2(min(i, o), max(i, o));
                    nbuf += cnt;
                }
            }
            live = act[kUnroll - 1];
            j += kUnroll;
        }
    }
    flush();
    // diagnostics: candidate tests and warp iterations of this warp
    uint32_t t = my_tests;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
    if (lane == 0 && t) {
        atomicAdd(&C->tests, (unsigned long long)t);
        atomicAdd(&C->iters, (unsigned long long)iters);
    }
}

cudaError_t launch_sweep(const BpScratch& s, const BpArgs& a, const uint32_t* keys, const uint32_t* vals,
                         uint2* pairs, uint64_t pair_cap, int count_rows, cudaStream_t st) {
    static int grid[2] = {0, 0};
    int m = a.mode == 1 ? 1 : 0;
    if (grid[m] == 0) {
        int per_sm = 0;
        if (m == 0) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sweep<0>, kThreads, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sweep<1>, kThreads, 0);
        grid[m] = sm_count() * (per_sm > 0 ? per_sm : 1);
    }
    if (m == 0) k_sweep<0><<<grid[m], kThreads, 0, st>>>(s, a, keys, vals, pairs, pair_cap, count_rows);
    else k_sweep<1><<<grid[m], kThreads, 0, st>>>(s, a, keys, vals, pairs, pair_cap, count_rows);
    return cudaGetLastError();
}

}  // namespace gsap
