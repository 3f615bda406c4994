// K1: segmented PCA of the object centres.
//
// Replaces the reference's Sap::Deviation / reduceExt / calDev / reduce6 /
// axisVecMultiple chain (sapDetection/Sap.cpp:148-209,
// sapDetection/SapKernel.cu:1342-1403, :63-97): there, three separate
// tree reductions over float4 arrays (the covariance rows pre-divided by n
// and written to two 16n-byte temporaries) feed a <<<1,1>>> kernel that picks
// the coordinate axis of largest variance.  Here one pass over the input
// (k_pca) accumulates per 4096-object work item FP32 sums of d = c - pilot
// and d d^T (per thread plain, merged as compensated two-sum pairs), and of
// the half extents h and h h^T (they only size the grid); then one CTA per
// scene (k_pca_finish; k_pca_finish_batch for batches) combines its partials
// in float-float arithmetic in a fixed order (deterministic), forms the
// covariance in FP64, solves the 3x3 eigenproblem (FP32 Jacobi,
// scene_math.cuh) and chooses the sweep grid; the last scene lays out the
// keys and resets the counters of the later stages.
#include "internal.cuh"
#include "scene_math.cuh"
#include <math.h>

namespace gsap {

// Batched plan: first work item of every scene (one CTA, sequential scan in
// 1024-scene blocks).
__global__ void __launch_bounds__(1024) k_plan(BpScratch S, BpArgs A) {
    pdl_wait();
    __shared__ uint32_t s_tot[32];
    __shared__ uint32_t s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (uint32_t base = 0; base < A.num_scenes; base += 1024) {
        uint32_t s = base + threadIdx.x;
        uint32_t v = 0;
        if (s < A.num_scenes) {
            v = work_items(scene_end(A, s) - scene_begin(A, s));
            const bool bad = A.scene_off[s + 1] < A.scene_off[s] || (s == 0 && A.scene_off[0] != 0u) ||
                             (s + 1 == A.num_scenes && A.scene_off[s + 1] != A.n);
            if (bad) atomicOr(&S.ctrl->error, kErrOffsets);
        }
        uint32_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31) s_tot[wid] = x;
        __syncthreads();
        if (wid == 0) {
            uint32_t t = s_tot[lane];
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= (uint32_t)o) t += y;
            }
            s_tot[lane] = t;
        }
        __syncthreads();
        uint32_t excl = s_carry + (wid ? s_tot[wid - 1] : 0u) + x - v;
        if (s < A.num_scenes) {
            S.work_start[s] = excl;
            for (uint32_t k = 0; k < v; ++k) S.work_scene[excl + k] = s;  // the scene of each of its items
        }
        __syncthreads();
        if (threadIdx.x == 1023) s_carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) S.work_start[A.num_scenes] = s_carry;
}

// Centre of the scene's first object: every work item of a scene shifts its
// sums by it, which keeps the FP32 covariance sums free of cancellation.
__device__ __forceinline__ void pilot_of(const BpArgs& A, uint32_t sb, uint32_t se, float& px, float& py, float& pz) {
    px = py = pz = 0.f;
    if (se > sb) {
        float4 a = A.mn[sb];
        if (A.mode == 0) {
            float4 c = A.mx[sb];
            px = 0.5f * (a.x + c.x); py = 0.5f * (a.y + c.y); pz = 0.5f * (a.z + c.z);
        } else {
            px = a.x; py = a.y; pz = a.z;
        }
        if (!isfinite(px) || !isfinite(py) || !isfinite(pz)) px = py = pz = 0.f;
    }
}

// ---------------------------------------------------------------- K1

// split CTAs per work item, each over kChunk / split of its objects, each
// writing its own partial (partial index = CTA index): calls of a few work
// items spread over more SMs (kPcaSplitSmall), large calls take one CTA per
// item.
__global__ void __launch_bounds__(kThreads) k_pca(BpScratch S, BpArgs A, uint32_t split) {
    pdl_wait();
    const uint32_t tid = threadIdx.x;
    uint32_t scene, b, e, wfirst, nw;
    if (!map_work(blockIdx.x / split, S, A, scene, b, e, wfirst, nw)) return;
    const uint32_t sb = scene_begin(A, scene), se = scene_end(A, scene);
    {
        const uint32_t part = kChunk / split, sub = blockIdx.x % split;
        b = min(e, b + sub * part);
        e = min(e, b + part);
    }

    // pilot = centre of the scene's first object (shift against cancellation)
    float px = 0.f, py = 0.f, pz = 0.f;
    pilot_of(A, sb, se, px, py, pz);
    // Each thread sums its (at most kChunk / kThreads = 16) objects in plain
    // FP32: d is taken about the pilot, so its terms are of the scene's
    // spread and 16 of them lose at most ~16 ulps.  From there on the sums
    // are compensated: the CTA and cross-CTA merges carry (hi, lo) pairs.
    // (Compensating every object's terms cost ~120 FP32 operations per
    // object and made the kernel issue-bound on large batches.)
    float hi[kPcaQ], hm[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int q = 0; q < kPcaQ; ++q) hi[q] = 0.f;
    bool bad = false;
    constexpr int U = 4;  // objects in flight per thread
    for (uint32_t i0 = b + tid; i0 < e; i0 += U * kThreads) {
        float4 A4[U], B4[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            uint32_t i = i0 + u * kThreads;
            if (i < e) {
                A4[u] = A.mn[i];
                B4[u] = A.mode == 0 ? A.mx[i] : A4[u];
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (i0 + u * kThreads >= e) break;
            float4 a = A4[u], c = B4[u];
            float cx, cy, cz, hx, hy, hz;
            if (A.mode == 0) {
                cx = 0.5f * (a.x + c.x); cy = 0.5f * (a.y + c.y); cz = 0.5f * (a.z + c.z);
                hx = 0.5f * fabsf(c.x - a.x); hy = 0.5f * fabsf(c.y - a.y); hz = 0.5f * fabsf(c.z - a.z);
            } else {
                cx = a.x; cy = a.y; cz = a.z;
                hx = hy = hz = fabsf(a.w);
            }
            if (!(isfinite(cx) && isfinite(cy) && isfinite(cz) && isfinite(hx) && isfinite(hy) && isfinite(hz))) {
                bad = true;
                continue;
            }
            float dx = cx - px, dy = cy - py, dz = cz - pz;
            const float v[9] = {dx, dy, dz, dx * dx, dx * dy, dx * dz, dy * dy, dy * dz, dz * dz};
#pragma unroll
            for (int q = 0; q < 9; ++q) hi[q] += v[q];
            const float w[9] = {hx, hy, hz, hx * hx, hx * hy, hx * hz, hy * hy, hy * hz, hz * hz};
#pragma unroll
            for (int q = 0; q < 9; ++q) hi[9 + q] += w[q];
            hm[0] = fmaxf(hm[0], hx); hm[1] = fmaxf(hm[1], hy); hm[2] = fmaxf(hm[2], hz);
        }
    }
    if (bad) atomicOr(&S.ctrl->error, kErrNonFinite);
    // CTA reduction, one quantity per thread: every thread's sums go to
    // shared memory (rows of kQn words: an odd stride, no bank conflicts),
    // thread (q = t % kQn, g = t / kQn) merges rows g, g + kG, ... of
    // column q as compensated pairs, and kQn threads merge the kG group
    // results in order (deterministic).  Every chain is at most
    // kThreads / kG + kG merges long, against five shuffle levels of all 21
    // quantities in every warp.
    constexpr uint32_t kQn = kPcaQ + 3;
    constexpr uint32_t kG = kThreads / kQn;
    __shared__ float s_v[kThreads][kQn];
    __shared__ float s_gh[kG][kQn], s_gl[kG][kQn];
#pragma unroll
    for (int q = 0; q < kPcaQ; ++q) s_v[tid][q] = hi[q];
#pragma unroll
    for (int k = 0; k < 3; ++k) s_v[tid][kPcaQ + k] = hm[k];
    __syncthreads();
    {
        const uint32_t q = tid % kQn, g = tid / kQn;
        if (g < kG) {
            float h = 0.f, l = 0.f;
            for (uint32_t r = g; r < (uint32_t)kThreads; r += kG) {
                if (q < (uint32_t)kPcaQ) kahan_merge(h, l, s_v[r][q], 0.f);
                else h = fmaxf(h, s_v[r][q]);
            }
            s_gh[g][q] = h;
            s_gl[g][q] = l;
        }
    }
    __syncthreads();
    if (tid < kQn) {
        float h = s_gh[0][tid], l = s_gl[0][tid];
        for (uint32_t g = 1; g < kG; ++g) {
            if (tid < (uint32_t)kPcaQ) kahan_merge(h, l, s_gh[g][tid], s_gl[g][tid]);
            else h = fmaxf(h, s_gh[g][tid]);
        }
        if (tid < (uint32_t)kPcaQ) {
            S.partials[blockIdx.x].hi[tid] = h;
            S.partials[blockIdx.x].lo[tid] = l;
        } else {
            S.partials[blockIdx.x].hmax[tid - kPcaQ] = h;
        }
    }
}

// K1b: one CTA per scene combines the scene's partials (float-float, fixed
// order: deterministic), solves the 3x3 eigenproblem and picks the grid; the
// last scene to finish computes the global bucket bases and the key layout
// and resets the counters of the later stages.  In temporal mode it writes
// the next call's parameters instead and leaves the counters to the main
// branch.  A separate launch keeps the FP64 tail's registers out of the
// streaming kernel.
// Quantisation bits of the key's low field when `total` buckets take the
// high bits of a key_bits-bit key (0: the grid does not fit).
__device__ __forceinline__ uint32_t key_q_bits(uint32_t key_bits, uint32_t total) {
    uint32_t bbits = 0;
    while (bbits < 32 && (1ull << bbits) < (uint64_t)total) ++bbits;
    uint32_t q = key_bits > bbits ? key_bits - bbits : 0u;
    return q > 24 ? 24u : q;
}

// The per-call pipeline counters back to zero (the epoch is advanced by the
// caller).
__device__ __forceinline__ void reset_counters(Ctrl* C) {
    C->entry_count = 0;
    C->pair_count = 0ull;
    for (int p = 0; p < kMaxPasses + 4; ++p) C->tile_ctr[p] = 0;
    C->sweep_ctr = 0;
    C->scan_ctr = 0;
    C->scan_total = 0;
    C->long_rows = 0;
    C->tests = 0ull;
    C->iters = 0ull;
}

__global__ void __launch_bounds__(kThreads) k_pca_finish(BpScratch S, BpArgs A, uint64_t entry_cap, int temporal,
                                                         uint32_t split) {
    pdl_wait();
    Scene* const out = temporal ? S.scenes_next : S.scenes;
    __shared__ uint32_t s_flag;
    const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint32_t scene = blockIdx.x;
    if (scene >= A.num_scenes) return;
    const uint32_t sb = scene_begin(A, scene), se = scene_end(A, scene);
    const uint32_t wfirst = A.scene_off ? S.work_start[scene] : 0u;
    // (bad offsets can plan more work items than were launched: only
    // partials that k_pca wrote are read)
    const uint32_t nw0 = A.scene_off ? S.work_start[scene + 1] - wfirst : work_items(A.n);
    const uint32_t nw = (wfirst < A.num_work ? min(nw0, A.num_work - wfirst) : 0u) * split;
    // Thread 0's loads for later (the pilot object, and the epoch that the
    // one-scene reset below advances) are in flight during the merge.
    const bool one = A.num_scenes == 1;
    float px = 0.f, py = 0.f, pz = 0.f;
    uint32_t epoch0 = 0;
    if (tid == 0) {
        pilot_of(A, sb, se, px, py, pz);
        if (one && !temporal) epoch0 = S.ctrl->epoch;
    }
    // Combine the scene's partials in float-float (two-sum) arithmetic on the
    // FP32 pipes, one quantity per thread: thread t (quantity q = t % kQn,
    // group g = t / kQn) merges partials g, g + kG, ... of its quantity, then
    // kQn threads merge the kG group results in order (deterministic); only
    // the final hi + lo pairs go to FP64 (GB300's FP64 lane rate makes an FP64
    // reduction slow).  Every chain is at most nw / kG + kG merges long.
    constexpr uint32_t kQn = kPcaQ + 3;  // the sums, then the three maxima
    constexpr uint32_t kG = kThreads / kQn;
    __shared__ float s_gh[kG][kQn], s_gl[kG][kQn];
    __shared__ double s_tot[kQn];
    {
        const uint32_t q = tid % kQn, g = tid / kQn;
        if (g < kG) {
            const PcaPartial* P = S.partials + wfirst * split;
            const float* ph = q < (uint32_t)kPcaQ ? &P->hi[q] : &P->hmax[q - kPcaQ];
            const float* pl = q < (uint32_t)kPcaQ ? &P->lo[q] : &P->hmax[q - kPcaQ];
            constexpr uint32_t kStride = sizeof(PcaPartial) / sizeof(float);
            float h = 0.f, l = 0.f;
            // kU partials' loads in flight at once, then their merges in order
            constexpr int kU = 8;
            for (uint32_t k0 = g; k0 < nw; k0 += kU * kG) {
                float vh[kU], vl[kU];
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const uint32_t k = k0 + u * kG;
                    vh[u] = k < nw ? ph[(size_t)k * kStride] : 0.f;
                    vl[u] = k < nw ? pl[(size_t)k * kStride] : 0.f;
                }
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    if (q < (uint32_t)kPcaQ) kahan_merge(h, l, vh[u], vl[u]);
                    else h = fmaxf(h, vh[u]);
                }
            }
            s_gh[g][q] = h;
            s_gl[g][q] = l;
        }
    }
    __syncthreads();
    if (tid < kQn) {
        float h = s_gh[0][tid], l = s_gl[0][tid];
        for (uint32_t g = 1; g < kG; ++g) {
            if (tid < (uint32_t)kPcaQ) kahan_merge(h, l, s_gh[g][tid], s_gl[g][tid]);
            else h = fmaxf(h, s_gh[g][tid]);
        }
        s_tot[tid] = tid < (uint32_t)kPcaQ ? (double)h + (double)l : (double)h;
    }
    __syncthreads();
    Ctrl* C = S.ctrl;
    if (tid == 0) {
        SceneSums z;
        const double* t = s_tot;
        for (int k = 0; k < 3; ++k) { z.sd[k] = t[k]; z.sh[k] = t[9 + k]; z.hmax[k] = t[kPcaQ + k]; }
        for (int k = 0; k < 6; ++k) { z.sdd[k] = t[3 + k]; z.shh[k] = t[12 + k]; }
        z.pilot[0] = px; z.pilot[1] = py; z.pilot[2] = pz;
        z.n = (double)(se - sb);
        Scene sc;
        choose_scene(z, A, entry_cap, A.n, sc);
        if (one) {
            // The only scene: its bucket base is 0, the key layout follows
            // from its own grid, and the record is stored once, complete
            // (the general tail below reads the records back from memory).
            const uint32_t total = sc.G2 * sc.G3;
            const uint32_t q = key_q_bits(A.key_bits, total);
            if (q == 0) atomicOr(&C->error, kErrCellRange);
            sc.bucket_base = 0;
            sc.q_scale = __fdiv_rn((float)(1u << q), sc.q_range);
            out[0] = sc;
            C->scenes_done = 0;
            if (temporal) {
                C->qbits_next = q;
                C->key_bits_next = A.key_bits;
                C->total_buckets_next = total;
            } else {
                C->qbits = q;
                C->key_bits = A.key_bits;
                C->total_buckets = total;
                reset_counters(C);
                C->epoch = epoch0 + 1u;
            }
        } else {
            out[scene] = sc;
            __threadfence();
            uint32_t old = atomicAdd(&C->scenes_done, 1u);
            s_flag = (old == A.num_scenes - 1) ? 1u : 0u;
        }
    }
    if (one) {
        if (!temporal)
            for (uint32_t k = tid; k < kHistWords; k += 256u) (&C->hist[0][0])[k] = 0u;
        return;
    }
    __syncthreads();
    if (!s_flag) return;
    if (A.num_scenes > 1) __threadfence();  // the other scenes' records are read below
    // Last scene: global bucket bases, key layout, and counter reset.
    __shared__ uint32_t s_wsum[kThreads / 32];
    __shared__ uint32_t s_carry;
    if (tid == 0) s_carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < A.num_scenes; base += kThreads) {
        uint32_t s = base + tid;
        uint32_t v = 0;
        if (s < A.num_scenes) v = __ldcg(&out[s].G2) * __ldcg(&out[s].G3);
        uint32_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31) s_wsum[wid] = x;
        __syncthreads();
        uint32_t pre = 0;
        for (uint32_t w = 0; w < wid; ++w) pre += s_wsum[w];
        uint32_t excl = s_carry + pre + x - v;
        if (s < A.num_scenes) out[s].bucket_base = excl;
        __syncthreads();
        if (tid == kThreads - 1) s_carry = excl + v;
        __syncthreads();
    }
    __shared__ uint32_t s_q;
    if (tid == 0) {
        uint32_t total = s_carry;
        const uint32_t q = key_q_bits(A.key_bits, total);
        if (q == 0) atomicOr(&C->error, kErrCellRange);
        s_q = q;
        C->scenes_done = 0;
        if (temporal) {
            C->qbits_next = q;
            C->key_bits_next = A.key_bits;
            C->total_buckets_next = total;
        }
    }
    if (temporal) {  // the main branch owns the pipeline counters
        __syncthreads();
        const float qf = (float)(1u << s_q);
        for (uint32_t s = tid; s < A.num_scenes; s += kThreads) out[s].q_scale = __fdiv_rn(qf, __ldcg(&out[s].q_range));
        return;
    }
    if (tid == 0) {
        C->qbits = s_q;
        C->key_bits = A.key_bits;
        C->total_buckets = s_carry;
        reset_counters(C);
        C->epoch = C->epoch + 1u;
    }
    for (uint32_t k = tid; k < kHistWords; k += 256u) (&C->hist[0][0])[k] = 0u;
    __syncthreads();
    // quantisation scale of every scene, computed once for all kernels
    const float qf = (float)(1u << s_q);
    for (uint32_t s = tid; s < A.num_scenes; s += kThreads) out[s].q_scale = __fdiv_rn(qf, __ldcg(&out[s].q_range));
}

// Batched form of the finish (more than one scene).  A CTA takes
// kFinishScenes consecutive scenes: each of its warps merges the partials of
// some of them (lane l merges items l, l+32, ... in float-float, then a fixed
// shuffle tree, so the result does not depend on timing), and warp 0 then
// solves all of them side by side, one scene per lane, instead of one lane
// of a warp (or one thread of a CTA) per scene: a batch's serial solves then
// share warp instructions.  The last CTA to finish lays out the keys and
// resets the counters, as k_pca_finish does.
constexpr int kFinishWarps = 16;
constexpr int kFinishScenes = 32;
__global__ void __launch_bounds__(32 * kFinishWarps) k_pca_finish_batch(BpScratch S, BpArgs A, uint64_t entry_cap,
                                                                       int temporal, uint32_t split) {
    pdl_wait();
    __shared__ SceneSums s_z[kFinishScenes];
    Scene* const out = temporal ? S.scenes_next : S.scenes;
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t s0 = blockIdx.x * kFinishScenes;
    Ctrl* C = S.ctrl;
    for (uint32_t k = wid; k < (uint32_t)kFinishScenes; k += kFinishWarps) {
        const uint32_t scene = s0 + k;
        if (scene >= A.num_scenes) break;
        const uint32_t sb = scene_begin(A, scene), se = scene_end(A, scene);
        const uint32_t wfirst = S.work_start[scene];
        const uint32_t nw0 = S.work_start[scene + 1] - wfirst;
        const uint32_t nw = (wfirst < A.num_work ? min(nw0, A.num_work - wfirst) : 0u) * split;
        float px = 0.f, py = 0.f, pz = 0.f;
        if (lane == 0) pilot_of(A, sb, se, px, py, pz);
        float ah[kPcaQ], al[kPcaQ], am[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int q = 0; q < kPcaQ; ++q) { ah[q] = 0.f; al[q] = 0.f; }
        for (uint32_t j = lane; j < nw; j += 32) {
            const PcaPartial* P = &S.partials[wfirst * split + j];
#pragma unroll
            for (int q = 0; q < kPcaQ; ++q) kahan_merge(ah[q], al[q], P->hi[q], P->lo[q]);
#pragma unroll
            for (int q = 0; q < 3; ++q) am[q] = fmaxf(am[q], P->hmax[q]);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int q = 0; q < kPcaQ; ++q) {
                float h2 = __shfl_down_sync(0xffffffffu, ah[q], o);
                float l2 = __shfl_down_sync(0xffffffffu, al[q], o);
                kahan_merge(ah[q], al[q], h2, l2);
            }
#pragma unroll
            for (int q = 0; q < 3; ++q) am[q] = fmaxf(am[q], __shfl_down_sync(0xffffffffu, am[q], o));
        }
        if (lane == 0) {
            SceneSums& z = s_z[k];
            for (int q = 0; q < 3; ++q) {
                z.sd[q] = (double)ah[q] + (double)al[q];
                z.sh[q] = (double)ah[9 + q] + (double)al[9 + q];
                z.hmax[q] = (double)am[q];
            }
            for (int q = 0; q < 6; ++q) {
                z.sdd[q] = (double)ah[3 + q] + (double)al[3 + q];
                z.shh[q] = (double)ah[12 + q] + (double)al[12 + q];
            }
            z.pilot[0] = px; z.pilot[1] = py; z.pilot[2] = pz;
            z.n = (double)(se - sb);
        }
    }
    __syncthreads();
    __shared__ uint32_t s_last;
    if (wid == 0) {
        const uint32_t cnt = min((uint32_t)kFinishScenes, A.num_scenes - s0);
        if (lane < cnt) {
            Scene sc;
            choose_scene(s_z[lane], A, entry_cap, A.n, sc);
            out[s0 + lane] = sc;
        }
        __threadfence();
        __syncwarp();
        if (lane == 0) s_last = atomicAdd(&C->scenes_done, cnt) + cnt == A.num_scenes ? 1u : 0u;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();  // the other scenes' records are read below
    // Last CTA: global bucket bases (an exclusive scan of G2 * G3 over the
    // scenes, each thread a contiguous chunk whose loads are issued
    // together), key layout, counter reset, quantisation scales.
    constexpr uint32_t kT = 32 * kFinishWarps;
    const uint32_t tid = threadIdx.x;
    const uint32_t per = (A.num_scenes + kT - 1) / kT;
    const uint32_t c0 = min(tid * per, A.num_scenes), c1 = min(c0 + per, A.num_scenes);
    uint32_t mine = 0;
#pragma unroll 8
    for (uint32_t sc = c0; sc < c1; ++sc) mine += __ldcg(&out[sc].G2) * __ldcg(&out[sc].G3);
    __shared__ uint32_t s_wsum[kFinishWarps];
    uint32_t x = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_wsum[wid] = x;
    __syncthreads();
    uint32_t pre = 0, total = 0;
#pragma unroll
    for (int w = 0; w < kFinishWarps; ++w) {
        const uint32_t v = s_wsum[w];
        if ((uint32_t)w < wid) pre += v;
        total += v;
    }
    uint32_t run = pre + x - mine;
    for (uint32_t sc = c0; sc < c1; ++sc) {
        out[sc].bucket_base = run;
        run += __ldcg(&out[sc].G2) * __ldcg(&out[sc].G3);
    }
    const uint32_t q = key_q_bits(A.key_bits, total);
    if (tid == 0) {
        if (q == 0) atomicOr(&C->error, kErrCellRange);
        C->scenes_done = 0;
        if (temporal) {
            C->qbits_next = q;
            C->key_bits_next = A.key_bits;
            C->total_buckets_next = total;
        } else {
            C->qbits = q;
            C->key_bits = A.key_bits;
            C->total_buckets = total;
            reset_counters(C);
            C->epoch = C->epoch + 1u;
        }
    }
    if (!temporal)
        for (uint32_t k = tid; k < kHistWords; k += kT) (&C->hist[0][0])[k] = 0u;
    const float qf = (float)(1u << q);
    for (uint32_t sc = tid; sc < A.num_scenes; sc += kT) out[sc].q_scale = __fdiv_rn(qf, __ldcg(&out[sc].q_range));
}

cudaError_t launch_plan(const BpScratch& s, const BpArgs& a, cudaStream_t st) {
    launch_pdl(k_plan, 1, 1024, 0, st, s, a);
    return cudaGetLastError();
}

cudaError_t launch_pca(const BpScratch& s, const BpArgs& a, cudaStream_t st, int temporal) {
    const uint32_t split = a.num_work <= kPcaSmallWork ? kPcaSplitSmall : 1u;
    launch_pdl(k_pca, a.num_work * split, kThreads, 0, st, s, a, split);
    if (a.num_scenes > 1)
        launch_pdl(k_pca_finish_batch, (a.num_scenes + kFinishScenes - 1) / kFinishScenes, 32 * kFinishWarps, 0, st,
                s, a, s.entry_cap, temporal, split);
    else
        launch_pdl(k_pca_finish, 1, kThreads, 0, st, s, a, s.entry_cap, temporal, split);
    return cudaGetLastError();
}

// Temporal mode, main branch: the counter resets that the finish does in the
// plain pipeline.
__global__ void k_reset(BpScratch S) {
    pdl_wait();
    Ctrl* C = S.ctrl;
    const uint32_t tid = threadIdx.x;
    if (tid == 0) {
        reset_counters(C);
        C->epoch = C->epoch + 1u;
    }
    for (uint32_t k = tid; k < kHistWords; k += 256u) (&C->hist[0][0])[k] = 0u;
}

// Temporal mode, after both branches: the parameters computed from this
// call's input become the ones the next call uses.
__global__ void k_commit(BpScratch S, uint32_t num_scenes) {
    pdl_wait();
    // the records as 8-byte words, one per thread (coalesced)
    static_assert(sizeof(Scene) % 8 == 0, "Scene is copied in 8-byte words");
    const uint64_t words = (uint64_t)num_scenes * (sizeof(Scene) / 8);
    const uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w < words) reinterpret_cast<uint64_t*>(S.scenes)[w] = reinterpret_cast<const uint64_t*>(S.scenes_next)[w];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        Ctrl* C = S.ctrl;
        C->qbits = C->qbits_next;
        C->key_bits = C->key_bits_next;
        C->total_buckets = C->total_buckets_next;
    }
}

cudaError_t launch_reset(const BpScratch& s, cudaStream_t st) {
    launch_pdl(k_reset, 1, 256, 0, st, s);
    return cudaGetLastError();
}

cudaError_t launch_commit(const BpScratch& s, uint32_t num_scenes, cudaStream_t st) {
    const uint64_t words = (uint64_t)num_scenes * (sizeof(Scene) / 8);
    launch_pdl(k_commit, (unsigned)((words + 255) / 256), 256, 0, st, s, num_scenes);
    return cudaGetLastError();
}

}  // namespace gsap
