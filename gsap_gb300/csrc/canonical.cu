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
            st_release_u64(st, lb_word(tag, t == 0 ? kFlagPrefix : kFlagAgg, tot));
            uint32_t ex = 0;
            if (t > 0) {
                ex = lookback(S.status, t, 0, 1, tag, spin, &C->error);
                st_release_u64(st, lb_word(tag, kFlagPrefix, ex + tot));
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
__global__ void __launch_bounds__(kThreads) k_scatter(BpScratch S, const uint2* __restrict__ in, uint64_t in_cap,
                                                      uint2* out, uint64_t out_cap, int both) {
    const uint64_t P = min((uint64_t)S.ctrl->pair_count, in_cap);
    const uint32_t* off = S.rowoff;
    for (uint64_t k = (uint64_t)blockIdx.x * kThreads + threadIdx.x; k < P; k += (uint64_t)gridDim.x * kThreads) {
        uint2 p = in[k];
        uint64_t s = (uint64_t)off[p.x] + atomicSub(&S.rowcnt[p.x], 1u) - 1u;
        if (s < out_cap) out[s] = p;
        else atomicOr(&S.ctrl->error, kErrPairCap);
        if (both) {
            uint64_t s2 = (uint64_t)off[p.y] + atomicSub(&S.rowcnt[p.y], 1u) - 1u;
            if (s2 < out_cap) out[s2] = make_uint2(p.y, p.x);
            else atomicOr(&S.ctrl->error, kErrPairCap);
        }
    }
}

// Sort every row by its second id (rows are short: insertion sort in
// registers up to 32, in place beyond).
__global__ void __launch_bounds__(kThreads) k_rowsort(BpScratch S, uint2* out, uint64_t out_cap, uint32_t n) {
    for (uint32_t r = blockIdx.x * kThreads + threadIdx.x; r < n; r += gridDim.x * kThreads) {
        uint64_t b = S.rowoff[r], e = S.rowoff[r + 1];
        if (e > out_cap) e = out_cap;
        if (e <= b + 1) continue;
        uint32_t len = (uint32_t)(e - b);
        if (len <= 32) {
            uint32_t y[32];
            for (uint32_t k = 0; k < len; ++k) y[k] = out[b + k].y;
            for (uint32_t k = 1; k < len; ++k) {
                uint32_t v = y[k];
                int m = (int)k - 1;
                while (m >= 0 && y[m] > v) { y[m + 1] = y[m]; --m; }
                y[m + 1] = v;
            }
            for (uint32_t k = 0; k < len; ++k) out[b + k].y = y[k];
        } else {
            for (uint64_t k = b + 1; k < e; ++k) {
                uint32_t v = out[k].y;
                uint64_t m = k;
                while (m > b && out[m - 1].y > v) { out[m].y = out[m - 1].y; --m; }
                out[m].y = v;
            }
        }
    }
}

cudaError_t launch_canonical(const BpScratch& s, uint32_t n, const uint2* in_pairs, uint64_t in_cap,
                             uint2* out_pairs, uint64_t out_cap, int both, int32_t* entries, uint64_t entry_cap,
                             uint32_t spin, cudaStream_t st) {
    const int grid = sm_count() * 4;
    k_scan<0><<<grid, kThreads, 0, st>>>(s, s.rowcnt, s.rowoff, nullptr, 0, n, 5, spin);
    k_scatter<<<grid * 2, kThreads, 0, st>>>(s, in_pairs, in_cap, out_pairs, out_cap, both);
    k_rowsort<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(s, out_pairs, out_cap, n);
    if (both && entries) k_scan<1><<<grid, kThreads, 0, st>>>(s, s.rowoff, nullptr, entries, entry_cap, n, 6, spin);
    return cudaGetLastError();
}

}  // namespace gsap
