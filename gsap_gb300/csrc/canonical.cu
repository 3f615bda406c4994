// K5: canonical pair output.
//
// Replaces the reference's pair canonicalisation (sapDetection/Sap.cpp:269-295:
// copyPairs, setSortIndex, two 23-bit radix sorts of the both-direction list,
// orderPairs, then cullRepetitivePairs = cullIndex, a CUDPP scan, a blocking
// read, setCullPairs, setPairsEntriesFlag, a second scan and setPairsEntries,
// SapKernel.cu:2122-2360, :2802-2855).  The sweep emits every pair exactly
// once and already counts pairs per row (first id, or both ids for the
// both-direction format), so canonicalisation is a counting sort:
//   1. exclusive look-back scan of the row counts -> row offsets;
//   2. scatter each pair into its row(s), slots taken by atomic decrement of
//      the row count (which leaves the counts at zero for the next call);
//   3. sort each row by its second id;
//   4. (both-direction format) compact the offsets of the non-empty rows
//      into pairEntries with a second scan.
#include "internal.cuh"

namespace gsap {

constexpr int kScanItems = 8;
constexpr int kScanTile = kThreads * kScanItems;

// mode 0: out[i] = exclusive prefix of in[i] (i < n), out[n] = total.
// mode 1: flag_i = rowoff[i+1] > rowoff[i]; entries[rank_i] = rowoff[i] for
//         flagged rows; total -> ctrl->scan_total.
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_scan(BpScratch S, const uint32_t* __restrict__ in, uint32_t* out,
                                                   int32_t* entries, uint64_t entry_cap, uint32_t n, int slot,
                                                   uint32_t spin) {
    __shared__ uint32_t s_w[8];
    __shared__ uint32_t s_tile, s_excl;
    const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    Ctrl* C = S.ctrl;
    const uint32_t ntiles = (n + kScanTile - 1) / kScanTile;
    const uint32_t tag = (C->epoch << 3) | (uint32_t)slot;
    while (true) {
        if (tid == 0) s_tile = atomicAdd(&C->tile_ctr[slot], 1u);
        __syncthreads();
        const uint32_t t = s_tile;
        if (t >= ntiles) break;
        const uint32_t b = t * kScanTile + tid * kScanItems;
        uint32_t v[kScanItems];
        uint32_t sum = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            uint32_t i = b + k;
            uint32_t x = 0;
            if (i < n) x = MODE == 0 ? in[i] : (in[i + 1] > in[i] ? 1u : 0u);
            v[k] = x;
            sum += x;
        }
        // CTA exclusive scan of the thread sums
        uint32_t x = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31) s_w[wid] = x;
        __syncthreads();
        uint32_t pre = 0, tot = 0;
#pragma unroll
        for (int w = 0; w < 8; ++w) {
            if ((uint32_t)w < wid) pre += s_w[w];
            tot += s_w[w];
        }
        if (tid == 0) {
            uint64_t* st = S.status + t;
            st_lb_u64(st, lb_word(tag, t == 0 ? kFlagPrefix : kFlagAgg, tot));
            uint32_t ex = 0;
            if (t > 0) {
                ex = lookback(S.status, t, 0, 1, tag, spin, &C->error);
                st_lb_u64(st, lb_word(tag, kFlagPrefix, ex + tot));
            }
            s_excl = ex;
            if (t == ntiles - 1) {
                if (MODE == 0) out[n] = ex + tot;
                else C->scan_total = ex + tot;
            }
        }
        __syncthreads();
        uint32_t run = s_excl + pre + x - sum;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            uint32_t i = b + k;
            if (i < n) {
                if (MODE == 0) out[i] = run;
                else if (v[k] && run < entry_cap) entries[run] = (int32_t)in[i];
            }
            run += v[k];
        }
        __syncthreads();
    }
}

// Scatter pairs into their rows.  both: row i gets (i, j) and row j (j, i).
// Each thread takes 4 pairs and issues their returning atomics back to back,
// so the grid keeps many of them in flight instead of chaining one per
// thread.
constexpr int kScatterPer = 4;
__global__ void __launch_bounds__(kThreads) k_scatter(BpScratch S, const uint2* __restrict__ in, uint64_t in_cap,
                                                      uint2* out, uint64_t out_cap, int both) {
    const uint64_t P = min((uint64_t)S.ctrl->pair_count, in_cap);
    const uint32_t* off = S.rowoff;
    const uint64_t stride = (uint64_t)gridDim.x * kThreads;
    for (uint64_t k0 = (uint64_t)blockIdx.x * kThreads + threadIdx.x; k0 < P; k0 += stride * kScatterPer) {
        uint2 p[kScatterPer];
        uint32_t a[kScatterPer], b[kScatterPer];
#pragma unroll
        for (int u = 0; u < kScatterPer; ++u) {
            uint64_t k = k0 + u * stride;
            p[u] = k < P ? in[k] : make_uint2(0xFFFFFFFFu, 0xFFFFFFFFu);
        }
#pragma unroll
        for (int u = 0; u < kScatterPer; ++u)
            if (p[u].x != 0xFFFFFFFFu) a[u] = atomicSub(&S.rowcnt[p[u].x], 1u);
        if (both) {
#pragma unroll
            for (int u = 0; u < kScatterPer; ++u)
                if (p[u].x != 0xFFFFFFFFu) b[u] = atomicSub(&S.rowcnt[p[u].y], 1u);
        }
#pragma unroll
        for (int u = 0; u < kScatterPer; ++u) {
            if (p[u].x == 0xFFFFFFFFu) continue;
            uint64_t s = (uint64_t)off[p[u].x] + a[u] - 1u;
            if (s < out_cap) out[s] = p[u];
            else atomicOr(&S.ctrl->error, kErrPairCap);
            if (both) {
                uint64_t s2 = (uint64_t)off[p[u].y] + b[u] - 1u;
                if (s2 < out_cap) out[s2] = make_uint2(p[u].y, p[u].x);
                else atomicOr(&S.ctrl->error, kErrPairCap);
            }
        }
    }
}

// Bitonic sorting network over N registers (every index is a compile-time
// constant after unrolling, so v[] stays in registers).
template <int N>
__device__ __forceinline__ void bitonic_regs(uint32_t (&v)[N]) {
#pragma unroll
    for (int k = 2; k <= N; k <<= 1)
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1)
#pragma unroll
            for (int i = 0; i < N; ++i) {
                const int l = i ^ j;
                if (l > i) {
                    const bool up = (i & k) == 0;
                    uint32_t a = v[i], b = v[l];
                    bool sw = up ? (a > b) : (a < b);
                    v[i] = sw ? b : a;
                    v[l] = sw ? a : b;
                }
            }
}

template <int N>
__device__ __forceinline__ void sort_row(uint2* out, uint64_t b, uint32_t len) {
    uint32_t v[N];
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] = ((uint32_t)k < len) ? out[b + k].y : 0xFFFFFFFFu;
    bitonic_regs<N>(v);
#pragma unroll
    for (int k = 0; k < N; ++k)
        if ((uint32_t)k < len) out[b + k].y = v[k];
}

// Sort every row by its second id: one thread per row with a register
// network for rows of up to 32 pairs (rows average ~5-11 pairs); longer
// rows are queued for k_rowsort_long.
__global__ void __launch_bounds__(kThreads) k_rowsort(BpScratch S, uint2* out, uint64_t out_cap, uint32_t n) {
    for (uint32_t r = blockIdx.x * kThreads + threadIdx.x; r < n; r += gridDim.x * kThreads) {
        uint64_t b = S.rowoff[r], e = S.rowoff[r + 1];
        if (e > out_cap) e = out_cap;
        if (e <= b + 1) continue;
        uint32_t len = (uint32_t)(e - b);
        if (len <= 8) sort_row<8>(out, b, len);
        else if (len <= 16) sort_row<16>(out, b, len);
        else if (len <= 32) sort_row<32>(out, b, len);
        else S.longrows[atomicAdd(&S.ctrl->long_rows, 1u)] = r;
    }
}

constexpr int kLongRow = 1024;  // per-warp shared-memory sort limit

// One warp per long row (rows of 33..1024 pairs; ~1% of rows at the 1M
// workload): bitonic sort in the warp's slice of shared memory.  Longer rows
// (pathological overlap) use an in-place odd-even transposition by the warp.
__global__ void __launch_bounds__(kThreads) k_rowsort_long(BpScratch S, uint2* out, uint64_t out_cap) {
    __shared__ uint32_t s_all[kThreads / 32][kLongRow];
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t* s = s_all[wid];
    const uint32_t nlong = S.ctrl->long_rows;
    const uint32_t warps = gridDim.x * (kThreads / 32);
    for (uint32_t q = blockIdx.x * (kThreads / 32) + wid; q < nlong; q += warps) {
        const uint32_t r = S.longrows[q];
        uint64_t b = S.rowoff[r], e = S.rowoff[r + 1];
        if (e > out_cap) e = out_cap;
        if (e <= b + 1) continue;
        const uint32_t len = (uint32_t)(e - b);
        if (len <= (uint32_t)kLongRow) {
            uint32_t P = 32;
            while (P < len) P <<= 1;
            for (uint32_t k = lane; k < P; k += 32) s[k] = k < len ? out[b + k].y : 0xFFFFFFFFu;
            __syncwarp();
            for (uint32_t k = 2; k <= P; k <<= 1)
                for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                    for (uint32_t i = lane; i < P; i += 32) {
                        const uint32_t l = i ^ j;
                        if (l > i) {
                            const bool up = (i & k) == 0;
                            const uint32_t a = s[i], c = s[l];
                            if (up ? (a > c) : (a < c)) { s[i] = c; s[l] = a; }
                        }
                    }
                    __syncwarp();
                }
            for (uint32_t k = lane; k < len; k += 32) out[b + k].y = s[k];
            __syncwarp();
        } else {
            for (uint32_t phase = 0; phase < len; ++phase) {
                for (uint32_t i = 2 * lane + (phase & 1); i + 1 < len; i += 64) {
                    const uint32_t a = out[b + i].y, c = out[b + i + 1].y;
                    if (a > c) { out[b + i].y = c; out[b + i + 1].y = a; }
                }
                __syncwarp();
            }
        }
    }
}

cudaError_t launch_canonical(const BpScratch& s, uint32_t n, const uint2* in_pairs, uint64_t in_cap,
                             uint2* out_pairs, uint64_t out_cap, int both, int32_t* entries, uint64_t entry_cap,
                             uint32_t spin, cudaStream_t st) {
    const int grid = sm_count() * 4;
    k_scan<0><<<grid, kThreads, 0, st>>>(s, s.rowcnt, s.rowoff, nullptr, 0, n, 5, spin);
    k_scatter<<<sm_count() * 32, kThreads, 0, st>>>(s, in_pairs, in_cap, out_pairs, out_cap, both);
    k_rowsort<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(s, out_pairs, out_cap, n);
    k_rowsort_long<<<sm_count() * 2, kThreads, 0, st>>>(s, out_pairs, out_cap);
    if (both && entries) k_scan<1><<<grid, kThreads, 0, st>>>(s, s.rowoff, nullptr, entries, entry_cap, n, 6, spin);
    return cudaGetLastError();
}

}  // namespace gsap
