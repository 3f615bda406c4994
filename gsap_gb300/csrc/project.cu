// K2: projection of every object onto the scene's axes, cell replication
// and the histogram of the first radix digit (each sort pass counts the next
// digit while it has its tile staged in shared memory).
//
// Replaces projectSubMultiple (sapDetection/SapKernel.cu:151-213, key =
// u.c - r + quadrant * interval, id = i) and the 8x4 cell mask of
// calBoxHashSub32 (SapKernel.cu:1506-1633) together with the four-quadrant
// split about the origin and its cross pass (SapKernel.cu:557-635, :968-1059):
// the generalisation is a 2-D grid of cells on the two secondary axes, each
// cell a separate sweep segment.  An object gets one sweep entry per cell its
// projected (u2, u3) box touches; the entry key is
//   ((bucket_base(scene) + c2 * G3 + c3) << Q) | q(lo1)
// with q the clamped quantisation of the lower bound on u1.  All projections
// use directed rounding (the interval always contains the exact projection
// of the box), and the cell and q maps are monotone, so no overlapping pair
// can be lost: the exact 3-D test later decides.
#include "internal.cuh"

namespace gsap {

// Clamped monotone cell index.
__device__ __forceinline__ uint32_t cell_of(float x, float org, float inv, uint32_t G) {
    float t = __fmul_rn(__fsub_rn(x, org), inv);
    t = fminf(fmaxf(t, 0.f), (float)(G - 1u));
    return (uint32_t)t;
}

// Box corners of object i (sphere: centre -/+ |r|, rounded outward).
__device__ __forceinline__ bool load_box(const BpArgs& A, uint32_t i, float3& a, float3& b) {
    float4 p = A.mn[i];
    if (A.mode == 0) {
        float4 q = A.mx[i];
        a = make_float3(p.x, p.y, p.z);
        b = make_float3(q.x, q.y, q.z);
    } else {
        sphere_box(p, a, b);
    }
    return isfinite(a.x) && isfinite(a.y) && isfinite(a.z) && isfinite(b.x) && isfinite(b.y) && isfinite(b.z);
}

// ITEMS objects per thread, kThreads * ITEMS per CTA, kChunk / that CTAs
// per work item.  Large calls take 8 per thread (fewer CTAs, so fewer
// histogram atomics on the 256 shared counters); small calls (a few work
// items) take 1, so that the objects spread over 16 CTAs per work item
// instead of 2 and no thread walks 8 objects in turn.
constexpr int kProjItemsLarge = 8;
constexpr int kProjItemsSmall = 1;
constexpr uint32_t kProjSmallWork = 64;  // work items (64 x 4096 objects) up to which calls count as small
constexpr int kProjStage = 128;          // entries of one item staged per warp

// PASSES > 0: counts the first radix digit for the onesweep passes;
// PASSES == 0 (bucket sort): counts the entries of every sub-bucket instead
// (global atomics; sub_layout in internal.cuh).
template <int PASSES, int ITEMS>
__global__ void __launch_bounds__(kThreads, 4) k_project(BpScratch S, BpArgs A) {
    pdl_wait();
    constexpr int kProjItems = ITEMS;
    constexpr int kProjHalf = kThreads * kProjItems;  // objects per CTA
    constexpr int kProjSplit = kChunk / kProjHalf;    // CTAs per work item
    __shared__ uint32_t s_hist[PASSES > 0 ? PASSES : 1][256];
    __shared__ float s_f[16];
    __shared__ uint32_t s_i[4];
    __shared__ uint32_t s_wtot[kThreads / 32];
    __shared__ uint32_t s_base;
    // per warp: the entries of one item, staged for coalesced stores
    __shared__ uint32_t s_sk[kThreads / 32][kProjStage], s_sv[kThreads / 32][kProjStage];
    const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    uint32_t scene, b, e, wfirst, nw;
    if (!map_work(blockIdx.x / kProjSplit, S, A, scene, b, e, wfirst, nw)) return;
    for (uint32_t k = tid; k < 256u * (PASSES > 0 ? PASSES : 1); k += kThreads) (&s_hist[0][0])[k] = 0u;
    if (tid == 0) {
        const Scene& sc = S.scenes[scene];
        for (int k = 0; k < 9; ++k) s_f[k] = sc.u[k];
        uint32_t Q = S.ctrl->qbits;
        s_f[9] = sc.q_org;
        s_f[10] = sc.q_scale;
        s_f[11] = sc.c2_org;
        s_f[12] = sc.c2_inv;
        s_f[13] = sc.c3_org;
        s_f[14] = sc.c3_inv;
        s_i[0] = sc.G2;
        s_i[1] = sc.G3;
        s_i[2] = sc.bucket_base;
        s_i[3] = Q;
    }
    __syncthreads();
    const uint32_t G2 = s_i[0], G3 = s_i[1], bb = s_i[2], Q = s_i[3];
    const uint32_t sub_shift = PASSES == 0 ? sub_layout(S.ctrl).shift : 0u;
    const float qmax = (float)((1u << Q) - 1u);

    bool bad = false;
    {
    const uint32_t half = blockIdx.x % kProjSplit;
    uint32_t qlo[kProjItems], clo[kProjItems], ncl[kProjItems], pre[kProjItems];
    uint32_t running = 0;
    const uint32_t wb = b + half * kProjHalf + wid * (32 * kProjItems);
#pragma unroll
    for (int k = 0; k < kProjItems; ++k) {
        uint32_t i = wb + k * 32 + lane;
        uint32_t r = 0;
        qlo[k] = 0; clo[k] = 0; ncl[k] = 0;
        if (i < e) {
            float3 a, c;
            if (load_box(A, i, a, c)) {
                float l1, h1, l2, h2, l3, h3;
                project_box(&s_f[0], a, c, l1, h1);
                project_box(&s_f[3], a, c, l2, h2);
                project_box(&s_f[6], a, c, l3, h3);
                float t = __fmul_rn(__fsub_rn(l1, s_f[9]), s_f[10]);
                qlo[k] = (uint32_t)fminf(fmaxf(t, 0.f), qmax);
                uint32_t c2a = cell_of(l2, s_f[11], s_f[12], G2), c2b = cell_of(h2, s_f[11], s_f[12], G2);
                uint32_t c3a = cell_of(l3, s_f[13], s_f[14], G3), c3b = cell_of(h3, s_f[13], s_f[14], G3);
                uint32_t n2 = c2b >= c2a ? c2b - c2a + 1 : 0, n3 = c3b >= c3a ? c3b - c3a + 1 : 0;
                clo[k] = (c2a << 16) | c3a;
                ncl[k] = (n2 << 16) | n3;
                r = n2 * n3;
                if (S.objscene) S.objscene[i] = scene;
            } else {
                bad = true;
            }
        }
        uint32_t x = r;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        pre[k] = running + x - r;
        running += __shfl_sync(0xffffffffu, x, 31);
    }
    if (lane == 0) s_wtot[wid] = running;
    __syncthreads();
    if (tid == 0) {
        uint32_t t = 0;
        for (int w = 0; w < kThreads / 32; ++w) { uint32_t v = s_wtot[w]; s_wtot[w] = t; t += v; }
        uint32_t base = atomicAdd(&S.ctrl->entry_count, t);
        if ((uint64_t)base + t > S.entry_cap) atomicOr(&S.ctrl->error, kErrEntryCap);
        s_base = base;
    }
    __syncthreads();
    const uint64_t wpos = (uint64_t)s_base + s_wtot[wid];
    // Entries of item k of this warp occupy [wpos + base_k, wpos + base_k +
    // tot_k) (item-major, lanes in order).  When they fit the warp's stage
    // they are written there first and then stored by all 32 lanes in
    // order (coalesced, and the histogram counts run on full warps); an item
    // with more entries (objects spanning many cells) is stored lane by lane.
#pragma unroll
    for (int k = 0; k < kProjItems; ++k) {
        const uint32_t n2 = ncl[k] >> 16, n3 = ncl[k] & 0xFFFFu;
        const uint32_t i = wb + k * 32 + lane;
        const uint32_t c2a = clo[k] >> 16, c3a = clo[k] & 0xFFFFu;
        const uint32_t base_k = __shfl_sync(0xffffffffu, pre[k], 0);
        const uint32_t end_k = (k + 1 < kProjItems) ? __shfl_sync(0xffffffffu, pre[k + 1 < kProjItems ? k + 1 : k], 0)
                                                    : running;
        const uint32_t tot_k = end_k - base_k;
        if (tot_k <= (uint32_t)kProjStage) {
            uint32_t o = pre[k] - base_k;
            for (uint32_t x2 = 0; x2 < n2; ++x2)
                for (uint32_t x3 = 0; x3 < n3; ++x3, ++o) {
                    // owner flags: is this the object's lowest cell on u2 / u3?
                    const uint32_t fl = (x2 == 0 ? 1u : 0u) | (x3 == 0 ? 2u : 0u);
                    s_sk[wid][o] = ((bb + (c2a + x2) * G3 + (c3a + x3)) << Q) | qlo[k];
                    s_sv[wid][o] = i | (fl << kFlagShift);
                }
            __syncwarp();
            for (uint32_t j = lane; j < tot_k; j += 32) {
                const uint64_t pos = wpos + base_k + j;
                if (pos < S.entry_cap) {  // entries past the capacity are counted, never stored
                    const uint32_t key = s_sk[wid][j];
                    S.keys[0][pos] = key;
                    S.vals[0][pos] = s_sv[wid][j];
                    if (PASSES > 0) atomicAdd(&s_hist[0][key & 255u], 1u);  // later digits: counted by the sort passes
                    else atomicAdd(&S.subcnt[min(key >> sub_shift, kMaxSub - 1u)], 1u);
                }
            }
            __syncwarp();  // the stage is refilled by the next item
        } else {
            uint64_t pos = wpos + pre[k];
            for (uint32_t x2 = 0; x2 < n2; ++x2)
                for (uint32_t x3 = 0; x3 < n3; ++x3, ++pos) {
                    const uint32_t key = ((bb + (c2a + x2) * G3 + (c3a + x3)) << Q) | qlo[k];
                    if (pos < S.entry_cap) {
                        const uint32_t fl = (x2 == 0 ? 1u : 0u) | (x3 == 0 ? 2u : 0u);
                        S.keys[0][pos] = key;
                        S.vals[0][pos] = i | (fl << kFlagShift);
                        if (PASSES > 0) atomicAdd(&s_hist[0][key & 255u], 1u);
                        else atomicAdd(&S.subcnt[min(key >> sub_shift, kMaxSub - 1u)], 1u);
                    }
                }
        }
    }
    }
    if (bad) atomicOr(&S.ctrl->error, kErrNonFinite);
    __syncthreads();
    if (PASSES > 0)
        for (uint32_t k = tid; k < 256; k += kThreads) {
            uint32_t v = s_hist[0][k];
            if (v) atomicAdd(&S.ctrl->hist[0][k], v);
        }
}

cudaError_t launch_project(const BpScratch& s, const BpArgs& a, int passes, cudaStream_t st) {
    if (a.num_work <= kProjSmallWork) {
        constexpr int kSplit = kChunk / (kThreads * kProjItemsSmall);
        if (passes == 0) launch_pdl(k_project<0, kProjItemsSmall>, a.num_work * kSplit, kThreads, 0, st, s, a);
        else if (passes <= 3) launch_pdl(k_project<3, kProjItemsSmall>, a.num_work * kSplit, kThreads, 0, st, s, a);
        else launch_pdl(k_project<4, kProjItemsSmall>, a.num_work * kSplit, kThreads, 0, st, s, a);
    } else {
        constexpr int kSplit = kChunk / (kThreads * kProjItemsLarge);
        if (passes == 0) launch_pdl(k_project<0, kProjItemsLarge>, a.num_work * kSplit, kThreads, 0, st, s, a);
        else if (passes <= 3) launch_pdl(k_project<3, kProjItemsLarge>, a.num_work * kSplit, kThreads, 0, st, s, a);
        else launch_pdl(k_project<4, kProjItemsLarge>, a.num_work * kSplit, kThreads, 0, st, s, a);
    }
    return cudaGetLastError();
}

}  // namespace gsap
