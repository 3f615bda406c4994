// K3, alternative to the radix sort (GSAP_SORT_BUCKET): bucket sort of the
// sweep entries.
//
// The radix sort (sort.cu, three or four onesweep passes over all entries)
// is latency bound at these sizes: every pass is a chain of ranking,
// look-back and scatter per 4096-key tile.  This path trades the passes for
// one counting scatter and one shared-memory sort per sub-bucket.  The entry key
// is (cell << Q) | q(lo1), and its top bits -- the cell and the top T bits
// of q, a "sub-bucket" -- are known when the projection writes the entry.
// So the projection counts the entries of every sub-bucket, and
//   1. k_subsum + k_subscan turn the counts into sub-bucket offsets (and put
//      the counts back to zero for use as cursors);
//   2. k_subscatter moves every entry into its sub-bucket (one atomic per
//      entry on the sub-bucket's cursor; order inside a sub-bucket arbitrary);
//   3. k_subsort sorts every sub-bucket by the whole key in shared memory:
//      a CTA owns the sub-buckets that start in its 4096-entry tile, loads
//      them (kRegion = 8192 entries at most at once) and runs LSD passes of 8-bit
//      digits over only the key bits that differ within them; a sub-bucket
//      too large for shared memory is sorted by the same CTA in global
//      memory chunk by chunk.  The last step writes the sorted keys and
//      gathers each entry's bounds into the 32-byte sweep record, as the last
//      onesweep pass does.
// Entries with equal keys may come out in any order; the sweep's pair set
// does not depend on it (a pair of equal-key entries is tested once either
// way).  At the 1M workload the largest sub-bucket holds about 3.6k entries
// (T = 4), so every tile takes the shared-memory path.
#include "internal.cuh"

namespace gsap {

constexpr uint32_t kSubScanTile = 4096;           // counts per scan tile (256 threads x 16)
constexpr uint32_t kSubScanTiles = kMaxSub / kSubScanTile;
constexpr int kBsThreads = 1024;                  // k_subsort CTA (one per SM)
constexpr int kBsWarps = kBsThreads / 32;
constexpr int kBsItems = 8;
constexpr uint32_t kRegion = kBsThreads * kBsItems;  // entries sorted in shared memory at once
constexpr uint32_t kBsTile = 4096;                // entries whose sub-buckets one tile owns

// ------------------------------------------------------------ offsets

__device__ __forceinline__ uint32_t block_sum256(uint32_t v, uint32_t* s_w) {
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = __reduce_add_sync(0xffffffffu, v);
    if (lane == 0) s_w[wid] = v;
    __syncthreads();
    uint32_t t = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) t += s_w[w];
    __syncthreads();
    return t;
}

__global__ void __launch_bounds__(256) k_subsum(BpScratch S) {
    pdl_wait();
    __shared__ uint32_t s_w[8];
    const SubLayout L = sub_layout(S.ctrl);
    const uint32_t t = blockIdx.x;
    if (t * kSubScanTile >= L.count) {
        if (threadIdx.x == 0) S.subsum[t] = 0u;
        return;
    }
    // counts past L.count are never incremented, so whole vectors can be read
    const uint4* src = reinterpret_cast<const uint4*>(S.subcnt + t * kSubScanTile + threadIdx.x * 16u);
    uint32_t sum = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const uint4 x = src[q];
        sum += x.x + x.y + x.z + x.w;
    }
    sum = block_sum256(sum, s_w);
    if (threadIdx.x == 0) S.subsum[t] = sum;
}

// Exclusive offsets of the sub-buckets (substart[0..count]) and the counts
// back to zero.
__global__ void __launch_bounds__(256) k_subscan(BpScratch S) {
    pdl_wait();
    __shared__ uint32_t s_w[8];
    const SubLayout L = sub_layout(S.ctrl);
    const uint32_t t = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (L.count == 0) {
        if (t == 0 && tid == 0) S.substart[0] = 0u;
        return;
    }
    if (t * kSubScanTile >= L.count) return;
    uint32_t ps = 0;
    for (uint32_t k = tid; k < t; k += 256) ps += S.subsum[k];
    const uint32_t tile_off = block_sum256(ps, s_w);
    const uint32_t b = t * kSubScanTile + tid * 16u;
    uint32_t v[16];
    uint4* src = reinterpret_cast<uint4*>(S.subcnt + b);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const uint4 x = src[q];
        v[4 * q] = x.x; v[4 * q + 1] = x.y; v[4 * q + 2] = x.z; v[4 * q + 3] = x.w;
        src[q] = make_uint4(0u, 0u, 0u, 0u);
    }
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < 16; ++k) sum += v[k];
    uint32_t x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_w[wid] = x;
    __syncthreads();
    uint32_t pre = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w)
        if ((uint32_t)w < wid) pre += s_w[w];
    uint32_t run = tile_off + pre + x - sum;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const uint32_t i = b + k;
        if (i < L.count) S.substart[i] = run;
        run += v[k];
        if (i + 1 == L.count) S.substart[L.count] = run;
    }
}

// Every entry into its sub-bucket (cursor = the count, from zero).
__global__ void __launch_bounds__(256) k_subscatter(BpScratch S) {
    pdl_wait();
    const Ctrl* C = S.ctrl;
    const uint32_t E = (uint32_t)min((uint64_t)C->entry_count, S.entry_cap);
    const SubLayout L = sub_layout(C);
    const uint32_t* __restrict__ k0 = S.keys[0];
    const uint32_t* __restrict__ v0 = S.vals[0];
    const uint32_t stride = gridDim.x * blockDim.x;
    constexpr int U = 4;
    for (uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < E; i0 += U * stride) {
        uint32_t key[U], val[U], pos[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t i = i0 + u * stride;
            if (i < E) {
                key[u] = __ldcs(k0 + i);
                val[u] = __ldcs(v0 + i);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (i0 + u * stride >= E) continue;
            const uint32_t s = min(key[u] >> L.shift, kMaxSub - 1u);
            pos[u] = __ldg(S.substart + s) + atomicAdd(&S.subcnt[s], 1u);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (i0 + u * stride >= E) continue;
            if (pos[u] < E) {
                S.keys[1][pos[u]] = key[u];
                S.vals[1][pos[u]] = val[u];
            } else {
                atomicOr(&S.ctrl->error, kErrInternal);
            }
        }
    }
}

// ------------------------------------------------------------ local sort

struct BsShared {
    uint32_t k[kRegion];
    uint32_t v[kRegion];
    uint32_t wh[kBsWarps][256];  // per-warp digit counts, then per-warp digit offsets
    uint32_t dstart[256];        // start of every digit in the sorted chunk
    uint32_t red[2][kBsWarps];
    uint32_t info[4];
};

// Ranks the (up to kRegion) keys of a chunk by the digit at `shift`:
// key[k] of lane l of warp w is chunk item w * 32 kBsItems + 32 k + l.  On return
// pos[k] is the item's place in the digit-stable order of the chunk and
// B.dstart[d] the start of digit d; B.wh is used as scratch.
__device__ __forceinline__ void rank_chunk(BsShared& B, const uint32_t (&key)[kBsItems], uint32_t m, int shift,
                                           uint32_t (&pos)[kBsItems]) {
    const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint32_t lt = lanemask_lt();
    for (uint32_t k = tid; k < (uint32_t)kBsWarps * 256u; k += kBsThreads) (&B.wh[0][0])[k] = 0u;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kBsItems; ++k) {
        const uint32_t idx = wid * 32u * kBsItems + 32u * k + lane;
        const bool valid = idx < m;
        const uint32_t d = (key[k] >> shift) & 255u;
        uint32_t mk = __ballot_sync(0xffffffffu, valid);
#pragma unroll
        for (int bit = 0; bit < 8; ++bit) {
            const uint32_t bal = __ballot_sync(0xffffffffu, (d >> bit) & 1u);
            mk &= ((d >> bit) & 1u) ? bal : ~bal;
        }
        const uint32_t before = valid ? B.wh[wid][d] : 0u;
        const uint32_t r = __popc(mk & lt);
        __syncwarp();
        if (valid && r == 0) B.wh[wid][d] = before + __popc(mk);
        __syncwarp();
        pos[k] = before + r;
    }
    __syncthreads();
    // per digit: offsets of the warps, and the digit's total
    uint32_t tot = 0;
    if (tid < 256) {
#pragma unroll
        for (int w = 0; w < kBsWarps; ++w) {
            const uint32_t c = B.wh[w][tid];
            B.wh[w][tid] = tot;
            tot += c;
        }
    }
    // exclusive scan of the 256 totals (threads 0..255)
    uint32_t x = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31 && wid < 8) B.red[0][wid] = x;
    __syncthreads();
    if (tid < 256) {
        uint32_t pre = 0;
#pragma unroll
        for (int w = 0; w < 8; ++w)
            if ((uint32_t)w < wid) pre += B.red[0][w];
        B.dstart[tid] = pre + x - tot;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kBsItems; ++k) {
        const uint32_t d = (key[k] >> shift) & 255u;
        pos[k] += B.dstart[d] + B.wh[wid][d];
    }
}

// min and max of the keys in B.k[0..m) (block-wide).
__device__ __forceinline__ void key_range(BsShared& B, uint32_t m, uint32_t& kmin, uint32_t& kmax) {
    const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    uint32_t lo = 0xFFFFFFFFu, hi = 0u;
    for (uint32_t i = tid; i < m; i += kBsThreads) {
        lo = min(lo, B.k[i]);
        hi = max(hi, B.k[i]);
    }
    lo = __reduce_min_sync(0xffffffffu, lo);
    hi = __reduce_max_sync(0xffffffffu, hi);
    if (lane == 0) {
        B.red[0][wid] = lo;
        B.red[1][wid] = hi;
    }
    __syncthreads();
    kmin = 0xFFFFFFFFu;
    kmax = 0u;
#pragma unroll
    for (int w = 0; w < kBsWarps; ++w) {
        kmin = min(kmin, B.red[0][w]);
        kmax = max(kmax, B.red[1][w]);
    }
    __syncthreads();
}

__device__ __forceinline__ int varying_bits(uint32_t kmin, uint32_t kmax) {
    return kmin == kmax ? 0 : 32 - __clz(kmin ^ kmax);
}

// Output of one sorted entry: its key, and its sweep records (put_record).
__device__ __forceinline__ void put_entry(const BpScratch& S, const SortGather& G, uint32_t g, uint32_t key,
                                          uint32_t val) {
    S.keys[0][g] = key;
    put_record(S, G, g, key, val);
}

// Sorts entries [r0, r1) (at most kRegion) of keys[1] / vals[1] in shared
// memory and writes them out at [r0, r1).
__device__ void sort_region(BsShared& B, const BpScratch& S, const SortGather& G, uint32_t r0, uint32_t r1) {
    const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint32_t m = r1 - r0;
    for (uint32_t i = tid; i < m; i += kBsThreads) {
        B.k[i] = __ldcs(S.keys[1] + r0 + i);
        B.v[i] = __ldcs(S.vals[1] + r0 + i);
    }
    __syncthreads();
    uint32_t kmin, kmax;
    key_range(B, m, kmin, kmax);
    const int nbits = varying_bits(kmin, kmax);
    for (int shift = 0; shift < nbits; shift += 8) {
        uint32_t key[kBsItems], val[kBsItems], pos[kBsItems];
#pragma unroll
        for (int k = 0; k < kBsItems; ++k) {
            const uint32_t idx = wid * 32u * kBsItems + 32u * k + lane;
            key[k] = idx < m ? B.k[idx] : 0u;
            val[k] = idx < m ? B.v[idx] : 0u;
        }
        rank_chunk(B, key, m, shift, pos);  // (its first barrier orders the loads above before the writes below)
#pragma unroll
        for (int k = 0; k < kBsItems; ++k) {
            const uint32_t idx = wid * 32u * kBsItems + 32u * k + lane;
            if (idx < m) {
                B.k[pos[k]] = key[k];
                B.v[pos[k]] = val[k];
            }
        }
        __syncthreads();
    }
    for (uint32_t i = tid; i < m; i += kBsThreads) put_entry(S, G, r0 + i, B.k[i], B.v[i]);
    __syncthreads();
}

// Sorts a sub-bucket [b, e) larger than shared memory: LSD passes over its
// varying bits, each pass reading the segment in kRegion chunks in order
// and scattering every chunk's entries after those of the earlier chunks
// with the same digit (stable), between keys[1]/vals[1] and keys[0]/vals[0].
__device__ void sort_segment_global(BsShared& B, const BpScratch& S, const SortGather& G, uint32_t b, uint32_t e) {
    const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    __shared__ uint32_t s_gofs[256];
    // key range of the segment
    uint32_t lo = 0xFFFFFFFFu, hi = 0u;
    for (uint32_t i = b + tid; i < e; i += kBsThreads) {
        const uint32_t k = S.keys[1][i];
        lo = min(lo, k);
        hi = max(hi, k);
    }
    lo = __reduce_min_sync(0xffffffffu, lo);
    hi = __reduce_max_sync(0xffffffffu, hi);
    if (lane == 0) {
        B.red[0][wid] = lo;
        B.red[1][wid] = hi;
    }
    __syncthreads();
    uint32_t kmin = 0xFFFFFFFFu, kmax = 0u;
#pragma unroll
    for (int w = 0; w < kBsWarps; ++w) {
        kmin = min(kmin, B.red[0][w]);
        kmax = max(kmax, B.red[1][w]);
    }
    __syncthreads();
    const int nbits = varying_bits(kmin, kmax);
    uint32_t *ks = S.keys[1], *vs = S.vals[1], *kd = S.keys[0], *vd = S.vals[0];
    for (int shift = 0; shift < nbits; shift += 8) {
        // digit histogram of the segment -> start of every digit
        if (tid < 256) s_gofs[tid] = 0u;
        __syncthreads();
        for (uint32_t i = b + tid; i < e; i += kBsThreads) atomicAdd(&s_gofs[(ks[i] >> shift) & 255u], 1u);
        __syncthreads();
        uint32_t c = tid < 256 ? s_gofs[tid] : 0u;
        uint32_t x = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31 && wid < 8) B.red[0][wid] = x;
        __syncthreads();
        if (tid < 256) {
            uint32_t pre = 0;
#pragma unroll
            for (int w = 0; w < 8; ++w)
                if ((uint32_t)w < wid) pre += B.red[0][w];
            s_gofs[tid] = b + pre + x - c;
        }
        __syncthreads();
        for (uint32_t c0 = b; c0 < e; c0 += kRegion) {
            const uint32_t m = min(kRegion, e - c0);
            uint32_t key[kBsItems], val[kBsItems], pos[kBsItems];
#pragma unroll
            for (int k = 0; k < kBsItems; ++k) {
                const uint32_t idx = wid * 32u * kBsItems + 32u * k + lane;
                key[k] = idx < m ? ks[c0 + idx] : 0u;
                val[k] = idx < m ? vs[c0 + idx] : 0u;
            }
            rank_chunk(B, key, m, shift, pos);
            // pos - dstart[d] is the item's rank among the chunk's digit d
#pragma unroll
            for (int k = 0; k < kBsItems; ++k) {
                const uint32_t idx = wid * 32u * kBsItems + 32u * k + lane;
                if (idx < m) {
                    const uint32_t d = (key[k] >> shift) & 255u;
                    const uint32_t g = s_gofs[d] + pos[k] - B.dstart[d];
                    kd[g] = key[k];
                    vd[g] = val[k];
                }
            }
            __syncthreads();
            // the chunk's digit totals move every digit's start on
            if (tid < 256) {
                const uint32_t end = tid == 255 ? m : B.dstart[tid + 1];
                s_gofs[tid] += end - B.dstart[tid];
            }
            __syncthreads();
        }
        uint32_t* t = ks; ks = kd; kd = t;
        t = vs; vs = vd; vd = t;
    }
    // sorted entries are in ks / vs: write the keys and gather the records
    for (uint32_t i = b + tid; i < e; i += kBsThreads) put_entry(S, G, i, ks[i], vs[i]);
    __syncthreads();
}

__global__ void __launch_bounds__(kBsThreads, 1) k_subsort(BpScratch S, SortGather G) {
    pdl_wait();
    extern __shared__ __align__(16) unsigned char bs_smem[];
    BsShared& B = *reinterpret_cast<BsShared*>(bs_smem);
    const Ctrl* C = S.ctrl;
    const uint32_t E = (uint32_t)min((uint64_t)C->entry_count, S.entry_cap);
    const SubLayout L = sub_layout(C);
    const uint32_t ntiles = (E + kBsTile - 1) / kBsTile;
    const uint32_t* sst = S.substart;
    for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const uint32_t p0 = t * kBsTile, p1 = min(p0 + kBsTile, E);
        if (threadIdx.x == 0) {
            // owned sub-buckets: those starting in [p0, p1), i.e. [sa, sb) with
            // sa / sb the first with start >= p0 / >= p1 (lower bounds over
            // substart[0..count])
            uint32_t lo = 0, hi = L.count + 1;
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                if (sst[mid] < p0) lo = mid + 1; else hi = mid;
            }
            const uint32_t sa = lo;
            hi = L.count + 1;
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                if (sst[mid] < p1) lo = mid + 1; else hi = mid;
            }
            B.info[0] = sa;
            B.info[1] = lo;
        }
        __syncthreads();
        const uint32_t sa = B.info[0], sb = min(B.info[1], L.count);
        __syncthreads();
        if (sa >= sb) continue;
        // the cursors of the owned sub-buckets back to zero for the next call
        for (uint32_t s = sa + threadIdx.x; s < sb; s += kBsThreads) S.subcnt[s] = 0u;
        const uint32_t r0 = sst[sa], r1 = sst[sb];
        if (r1 - r0 <= kRegion) {
            sort_region(B, S, G, r0, r1);
        } else {
            for (uint32_t s = sa; s < sb; ++s) {
                const uint32_t b = sst[s], e = sst[s + 1];
                if (e - b <= kRegion) sort_region(B, S, G, b, e);
                else sort_segment_global(B, S, G, b, e);
            }
        }
    }
}

// Grid of k_subsort on the current device (one CTA per SM; the shared
// memory attribute is set once per device).
static int subsort_grid() {
    static std::once_flag once[kMaxDevices];
    static int val[kMaxDevices];
    return per_device(once, val, [] {
        const int smem = (int)sizeof(BsShared);
        cudaFuncSetAttribute(k_subsort, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_subsort, kBsThreads, smem);
        return sm_count() * (per_sm > 0 ? per_sm : 1);
    });
}

cudaError_t bucket_sort_setup() {
    (void)subsort_grid();
    return cudaGetLastError();
}

cudaError_t launch_bucket_sort(const BpScratch& s, const SortGather& G, uint32_t spin, cudaStream_t st) {
    (void)spin;
    launch_pdl(k_subsum, kSubScanTiles, 256, 0, st, s);
    launch_pdl(k_subscan, kSubScanTiles, 256, 0, st, s);
    launch_pdl(k_subscatter, sm_count() * 8, 256, 0, st, s);
    launch_pdl(k_subsort, subsort_grid(), kBsThreads, sizeof(BsShared), st, s, G);
    return cudaGetLastError();
}

}  // namespace gsap
