// K5: canonical pair output.
//
// Replaces the reference's pair canonicalisation (sapDetection/Sap.cpp:269-295:
// copyPairs, setSortIndex, two 23-bit radix sorts of the both-direction list,
// orderPairs, then cullRepetitivePairs = cullIndex, a CUDPP scan, a blocking
// read, setCullPairs, setPairsEntriesFlag, a second scan and setPairsEntries,
// SapKernel.cu:2122-2360, :2802-2855).  The sweep emits every pair exactly
// once and already counts pairs per row (first id, or both ids for the
// both-direction format), so canonicalisation is a counting sort:
//   1. exclusive scan of the row counts -> row offsets (reduce, then scan);
//   2. scatter each pair into its row(s) of an internal buffer at the slot
//      the sweep drew from the row counter when it stored the pair (the
//      scan has read the counters and put them back to zero for the next
//      call);
//   3. place every pair at its final index: row offset + its rank by second
//      id within the row (one thread per pair counting the row's smaller
//      ids; rows are ~5-11 pairs long, so this costs sum(len^2) compares
//      and needs no per-row sort network); rows longer than kRankRow are
//      sorted by one warp each;
//   4. (both-direction format) compact the offsets of the non-empty rows
//      into pairEntries with a second scan.
#include "internal.cuh"

namespace gsap {

constexpr int kScanItems = 16;
constexpr int kScanTile = kThreads * kScanItems;

// Warp-wide look-back over single-word tile states: lane k reads the word of
// tile t-1-k, so a round trip covers 32 predecessors; aggregates are summed
// up to the nearest inclusive prefix.  Returns the exclusive prefix of tile
// t in every lane.  Bounded: on timeout sets kErrTimeout and returns what it
// has (positions then stay in range, only too small).
__device__ __forceinline__ uint32_t warp_lookback1(uint64_t* status, uint32_t t, uint32_t tag, uint32_t spin_limit,
                                                   uint32_t* err) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t excl = 0, spins = 0;
    int64_t top = (int64_t)t - 1;  // newest tile of the window
    while (top >= 0) {
        const int64_t j = top - (int64_t)lane;
        uint64_t w = 0;
        bool ready = true, pre = true;  // tiles before 0 act as a zero prefix
        if (j >= 0) {
            w = ld_lb_u64(status + j);
            ready = (uint32_t)(w >> 32) == tag && (w & (kFlagAgg | kFlagPrefix));
            pre = ready && (w & kFlagPrefix);
        }
        const uint32_t pm = __ballot_sync(0xffffffffu, pre);
        const uint32_t nr = __ballot_sync(0xffffffffu, !ready);
        const uint32_t p = pm ? (uint32_t)(__ffs(pm) - 1) : 32u;
        const uint32_t need = p >= 31 ? 0xffffffffu : ((2u << p) - 1u);
        if (nr & need) {
            if (++spins > spin_limit) {
                if (lane == 0) atomicOr(err, kErrTimeout);
                return __shfl_sync(0xffffffffu, excl, 0);
            }
            if (spins > 16) __nanosleep(32);
            continue;
        }
        uint32_t v = (j >= 0 && lane <= p) ? (uint32_t)(w & kValMask) : 0u;
        excl += __reduce_add_sync(0xffffffffu, v);
        if (p < 32) break;
        top -= 32;
    }
    return excl;
}

// mode 0: out[i] = exclusive prefix of in[i] (i < n), out[n] = total.
// mode 1: flag_i = rowoff[i+1] > rowoff[i]; entries[rank_i] = rowoff[i] for
//         flagged rows; total -> ctrl->scan_total.
// mode 0 also zeroes in[0..n) once read (the row counters of the next call).
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_scan(BpScratch S, uint32_t* in, uint32_t* out, int32_t* entries,
                                                   uint64_t entry_cap, uint32_t n, int slot, uint32_t spin) {
    pdl_wait();
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
        if (MODE == 0 && b + kScanItems <= n) {  // 64-byte aligned run: vector loads
            uint4* src = reinterpret_cast<uint4*>(in + b);
#pragma unroll
            for (int q = 0; q < kScanItems / 4; ++q) {
                const uint4 x4 = src[q];
                v[4 * q] = x4.x; v[4 * q + 1] = x4.y; v[4 * q + 2] = x4.z; v[4 * q + 3] = x4.w;
                src[q] = make_uint4(0u, 0u, 0u, 0u);
            }
        } else {
#pragma unroll
            for (int k = 0; k < kScanItems; ++k) {
                const uint32_t i = b + k;
                v[k] = i < n ? (MODE == 0 ? in[i] : (in[i + 1] > in[i] ? 1u : 0u)) : 0u;
                if (MODE == 0 && i < n) in[i] = 0u;
            }
        }
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) sum += v[k];
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
        if (wid == 0) {
            uint64_t* st = S.status + t;
            if (lane == 0) st_lb_u64(st, lb_word(tag, t == 0 ? kFlagPrefix : kFlagAgg, tot));
            uint32_t ex = 0;
            if (t > 0) {
                ex = warp_lookback1(S.status, t, tag, spin, &C->error);
                if (lane == 0) st_lb_u64(st, lb_word(tag, kFlagPrefix, ex + tot));
            }
            if (lane == 0) {
                s_excl = ex;
                if (t == ntiles - 1) {
                    if (MODE == 0) out[n] = ex + tot;
                    else C->scan_total = ex + tot;
                }
            }
        }
        __syncthreads();
        uint32_t run = s_excl + pre + x - sum;
        if (MODE == 0 && b + kScanItems <= n) {
            uint4* dst = reinterpret_cast<uint4*>(out + b);
#pragma unroll
            for (int q = 0; q < kScanItems / 4; ++q) {
                uint4 o4;
                o4.x = run; run += v[4 * q];
                o4.y = run; run += v[4 * q + 1];
                o4.z = run; run += v[4 * q + 2];
                o4.w = run; run += v[4 * q + 3];
                dst[q] = o4;
            }
        } else {
#pragma unroll
            for (int k = 0; k < kScanItems; ++k) {
                const uint32_t i = b + k;
                if (i < n) {
                    if (MODE == 0) out[i] = run;
                    else if (v[k] && run < entry_cap) entries[run] = (int32_t)in[i];
                }
                run += v[k];
            }
        }
        __syncthreads();
    }
}

// Row offsets in two launches with no look-back chain (mode 0 of k_scan as
// a reduce-then-scan): k_rowsum sums every 4096-count tile; k_rowscan adds
// up the sums of the tiles before its own, scans its counts into the
// offsets and puts the counters back to zero for the next call.
__device__ __forceinline__ uint32_t cta_sum256(uint32_t v, uint32_t* s_w) {
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = __reduce_add_sync(0xffffffffu, v);
    if (lane == 0) s_w[wid] = v;
    __syncthreads();
    uint32_t t = 0;
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) t += s_w[w];
    __syncthreads();
    return t;
}

__global__ void __launch_bounds__(kThreads) k_rowsum(const uint32_t* __restrict__ in, uint32_t* tsum, uint32_t n) {
    pdl_wait();
    __shared__ uint32_t s_w[kThreads / 32];
    const uint32_t b = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t sum = 0;
    if (b + kScanItems <= n) {
        const uint4* src = reinterpret_cast<const uint4*>(in + b);
#pragma unroll
        for (int q = 0; q < kScanItems / 4; ++q) {
            const uint4 x4 = src[q];
            sum += x4.x + x4.y + x4.z + x4.w;
        }
    } else {
        for (uint32_t i = b; i < n && i < b + kScanItems; ++i) sum += in[i];
    }
    const uint32_t t = cta_sum256(sum, s_w);
    if (threadIdx.x == 0) tsum[blockIdx.x] = t;
}

// Many tiles (n above kDirectTiles * 4096 rows): the tile sums are scanned
// once, in place, by one CTA (k_tilescan) instead of every tile summing all
// the sums before its own, which grows with the square of the tile count.
constexpr uint32_t kDirectTiles = 512;

__global__ void __launch_bounds__(1024) k_tilescan(uint32_t* tsum, uint32_t ntiles) {
    pdl_wait();
    __shared__ uint32_t s_w[32];
    __shared__ uint32_t s_carry;
    const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) s_carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < ntiles; base += 1024) {
        const uint32_t i = base + tid;
        const uint32_t v = i < ntiles ? tsum[i] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31) s_w[wid] = x;
        __syncthreads();
        uint32_t pre = 0;
        for (uint32_t w = 0; w < wid; ++w) pre += s_w[w];
        const uint32_t excl = s_carry + pre + x - v;
        if (i < ntiles) tsum[i] = excl;
        __syncthreads();
        if (tid == 1023) s_carry = excl + v;
        __syncthreads();
    }
}

// Who puts the row counters back to zero for the next call: the row scan
// (a sequential write of all n counters) when pairs are many, k_scatter
// (one write per stored pair, to rows it touches anyway) when they are few
// against the rows -- e.g. 0.8M pairs over 38.6M objects in a batch of
// scenes, where zeroing every counter would be a third of the scan's bytes.
// Both kernels decide from the same stored pair count.
__device__ __forceinline__ bool scatter_zeroes(uint64_t pairs, uint32_t n) { return pairs * 4ull < n; }

// scanned != 0: tsum holds every tile's exclusive offset (k_tilescan ran).
__global__ void __launch_bounds__(kThreads) k_rowscan(uint32_t* in, uint32_t* out, const uint32_t* __restrict__ tsum,
                                                      uint32_t n, int scanned, const Ctrl* __restrict__ C,
                                                      uint64_t pair_cap) {
    pdl_wait();
    const bool zero = !scatter_zeroes(min((uint64_t)C->pair_count, pair_cap), n);
    __shared__ uint32_t s_w[kThreads / 32];
    const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint32_t t = blockIdx.x;
    // offset of this tile: the sums of all tiles before it
    uint32_t tile_off;
    if (scanned) {
        tile_off = tsum[t];
    } else {
        uint32_t ps = 0;
        for (uint32_t k = tid; k < t; k += kThreads) ps += tsum[k];
        tile_off = cta_sum256(ps, s_w);
    }
    const uint32_t b = t * kScanTile + tid * kScanItems;
    uint32_t v[kScanItems];
    const bool full = b + kScanItems <= n;
    if (full) {
        uint4* src = reinterpret_cast<uint4*>(in + b);
#pragma unroll
        for (int q = 0; q < kScanItems / 4; ++q) {
            const uint4 x4 = src[q];
            v[4 * q] = x4.x; v[4 * q + 1] = x4.y; v[4 * q + 2] = x4.z; v[4 * q + 3] = x4.w;
            if (zero) src[q] = make_uint4(0u, 0u, 0u, 0u);
        }
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            const uint32_t i = b + k;
            v[k] = i < n ? in[i] : 0u;
            if (i < n && zero) in[i] = 0u;
        }
    }
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) sum += v[k];
    uint32_t x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_w[wid] = x;
    __syncthreads();
    uint32_t pre = 0, tot = 0;
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) {
        if ((uint32_t)w < wid) pre += s_w[w];
        tot += s_w[w];
    }
    uint32_t run = tile_off + pre + x - sum;
    if (t == gridDim.x - 1 && tid == 0) out[n] = tile_off + tot;
    if (full) {
        uint4* dst = reinterpret_cast<uint4*>(out + b);
#pragma unroll
        for (int q = 0; q < kScanItems / 4; ++q) {
            uint4 o4;
            o4.x = run; run += v[4 * q];
            o4.y = run; run += v[4 * q + 1];
            o4.z = run; run += v[4 * q + 2];
            o4.w = run; run += v[4 * q + 3];
            dst[q] = o4;
        }
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            if (b + k < n) out[b + k] = run;
            run += v[k];
        }
    }
}

// Scatter pairs into their rows at the slots the sweep drew.  both: row i
// gets (i, j) and row j (j, i).  No atomics.  With few pairs against the
// rows (scatter_zeroes) it also puts the counters of the rows it touches
// back to zero; the other rows' counters are zero already.
__global__ void __launch_bounds__(kThreads) k_scatter(BpScratch S, const uint2* __restrict__ in, uint64_t in_cap,
                                                      uint2* out, uint64_t out_cap, int both, uint32_t n) {
    pdl_wait();
    const uint64_t P = min((uint64_t)S.ctrl->pair_count, in_cap);
    const bool zero = scatter_zeroes(P, n);
    const uint32_t* off = S.rowoff;
    const uint32_t* __restrict__ rank1 = S.tmp_rank;
    const uint2* __restrict__ rank2 = reinterpret_cast<const uint2*>(S.tmp_rank);
    const uint64_t stride = (uint64_t)gridDim.x * kThreads;
    constexpr int kPer = 4;  // pairs per thread with their row-offset loads in flight together
    for (uint64_t k0 = (uint64_t)blockIdx.x * kThreads + threadIdx.x; k0 < P; k0 += stride * kPer) {
        uint2 p[kPer], r[kPer];
        uint32_t o1[kPer], o2[kPer];
#pragma unroll
        for (int u = 0; u < kPer; ++u) {
            const uint64_t k = k0 + u * stride;
            if (k < P) {
                p[u] = in[k];
                r[u] = both ? rank2[k] : make_uint2(rank1[k], 0u);
            }
        }
        if (zero) {
#pragma unroll
            for (int u = 0; u < kPer; ++u) {
                if (k0 + u * stride >= P) continue;
                S.rowcnt[p[u].x] = 0u;
                if (both) S.rowcnt[p[u].y] = 0u;
            }
        }
#pragma unroll
        for (int u = 0; u < kPer; ++u) {
            if (k0 + u * stride >= P) continue;
            o1[u] = __ldg(off + p[u].x);
            if (both) o2[u] = __ldg(off + p[u].y);
        }
#pragma unroll
        for (int u = 0; u < kPer; ++u) {
            if (k0 + u * stride >= P) continue;
            const uint64_t s = (uint64_t)o1[u] + r[u].x;
            if (s < out_cap) out[s] = p[u];
            else atomicOr(&S.ctrl->error, kErrPairCap);
            if (both) {
                const uint64_t s2 = (uint64_t)o2[u] + r[u].y;
                if (s2 < out_cap) out[s2] = make_uint2(p[u].y, p[u].x);
                else atomicOr(&S.ctrl->error, kErrPairCap);
            }
        }
    }
}

constexpr uint32_t kRankRow = 256;  // longer rows go to k_rowsort_long
constexpr int kLongRow = 1024;       // per-warp shared-memory sort limit

// Final placement: the pair at grouped index s (row x = its first id) goes
// to rowoff[x] + (number of pairs of row x with a smaller second id).
// Second ids are unique within a row, so the ranks are a permutation.
// A CTA owns the rows that start in its tile [lo, hi) of the grouped list;
// a row of at most kRankRow pairs then lies inside [lo, hi + kRankRow), which
// the CTA stages in shared memory with coalesced loads, so the rank loops
// run on shared memory instead of chaining L2 round trips.
constexpr uint32_t kRankTile = 2048;
__global__ void __launch_bounds__(kThreads) k_rank(BpScratch S, const uint2* __restrict__ grp, uint64_t grp_cap,
                                                   uint32_t n, uint2* out, uint64_t out_cap) {
    pdl_wait();
    __shared__ uint2 s_p[kRankTile + kRankRow];
    const uint32_t P = (uint32_t)min((uint64_t)S.rowoff[n], grp_cap);  // grouped entries
    const uint32_t ntiles = (P + kRankTile - 1) / kRankTile;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint32_t lo = tile * kRankTile;
        const uint32_t hi = min(lo + kRankTile, P);
        const uint32_t wend = min(hi + kRankRow, P);
        for (uint32_t s = lo + threadIdx.x; s < wend; s += kThreads) s_p[s - lo] = grp[s];
        __syncthreads();
        for (uint32_t s = lo + threadIdx.x; s < wend; s += kThreads) {
            const uint2 p = s_p[s - lo];
            const uint32_t b = __ldg(S.rowoff + p.x);
            if (b < lo || b >= hi) continue;  // row owned by another tile
            const uint32_t e = __ldg(S.rowoff + p.x + 1), len = e - b;
            if (len > kRankRow) {
                if (s == b) S.longrows[atomicAdd(&S.ctrl->long_rows, 1u)] = p.x;  // queued once per row
                continue;
            }
            uint32_t r = 0;
            for (uint32_t k = b - lo; k < e - lo; ++k) r += s_p[k].y < p.y;
            if ((uint64_t)b + r < out_cap) out[b + r] = p;
        }
        __syncthreads();
    }
}

// One warp per long row (more than kRankRow pairs; rare): bitonic sort of
// the second ids in the warp's slice of shared memory for rows up to
// kLongRow, rank placement by the warp beyond (pathological overlap).
__global__ void __launch_bounds__(kThreads) k_rowsort_long(BpScratch S, const uint2* __restrict__ grp, uint2* out,
                                                           uint64_t out_cap) {
    pdl_wait();
    __shared__ uint32_t s_all[kThreads / 32][kLongRow];
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t* s = s_all[wid];
    const uint32_t nlong = S.ctrl->long_rows;
    const uint32_t warps = gridDim.x * (kThreads / 32);
    for (uint32_t q = blockIdx.x * (kThreads / 32) + wid; q < nlong; q += warps) {
        const uint32_t r = S.longrows[q];
        const uint32_t b = S.rowoff[r], e = S.rowoff[r + 1];
        const uint32_t len = e - b;
        if (len <= (uint32_t)kLongRow) {
            uint32_t P = 32;
            while (P < len) P <<= 1;
            for (uint32_t k = lane; k < P; k += 32) s[k] = k < len ? grp[b + k].y : 0xFFFFFFFFu;
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
            for (uint32_t k = lane; k < len; k += 32)
                if ((uint64_t)b + k < out_cap) out[b + k] = make_uint2(r, s[k]);
            __syncwarp();
        } else {
            for (uint32_t k = lane; k < len; k += 32) {
                const uint32_t y = grp[b + k].y;
                uint32_t rk = 0;
                for (uint32_t m = b; m < e; ++m) rk += grp[m].y < y;
                if ((uint64_t)b + rk < out_cap) out[b + rk] = make_uint2(r, y);
            }
        }
    }
}

cudaError_t launch_canonical(const BpScratch& s, uint32_t n, const uint2* in_pairs, uint64_t in_cap,
                             uint2* out_pairs, uint64_t out_cap, int both, int32_t* entries, uint64_t entry_cap,
                             uint32_t spin, cudaStream_t st) {
    const int grid = sm_count() * 4;
    const uint32_t ntiles = (n + kScanTile - 1) / kScanTile;
    launch_pdl(k_rowsum, ntiles, kThreads, 0, st, s.rowcnt, s.tile_sums, n);
    const int scanned = ntiles > kDirectTiles ? 1 : 0;
    if (scanned) launch_pdl(k_tilescan, 1, 1024, 0, st, s.tile_sums, ntiles);
    launch_pdl(k_rowscan, ntiles, kThreads, 0, st, s.rowcnt, s.rowoff, s.tile_sums, n, scanned, s.ctrl, in_cap);
    const uint64_t grp_cap = 2 * s.pair_cap_internal;
    const uint64_t est_pairs = (uint64_t)n * kEstPairsPerObject * (both ? 2u : 1u);
    launch_pdl(k_scatter, call_grid(sm_count() * 16, est_pairs, kThreads * 4u), kThreads, 0, st, s, in_pairs, in_cap,
            s.grp_pairs, grp_cap, both, n);
    launch_pdl(k_rank, call_grid(sm_count() * 8, est_pairs, kRankTile), kThreads, 0, st, s, s.grp_pairs, grp_cap, n,
            out_pairs, out_cap);
    launch_pdl(k_rowsort_long, call_grid(sm_count() * 2, n, 4096u), kThreads, 0, st, s, s.grp_pairs, out_pairs,
            out_cap);
    if (both && entries)
        launch_pdl(k_scan<1>, call_grid(grid, ntiles, 1u), kThreads, 0, st, s, s.rowoff, nullptr, entries, entry_cap,
                n, 6, spin);
    return cudaGetLastError();
}

}  // namespace gsap
