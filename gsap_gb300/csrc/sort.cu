// K3: onesweep LSD radix sort of (u32 key, u32 value) with 8-bit digits.
//
// Replaces the NVIDIA SDK radix sort of the reference
// (sapDetection/radixsort.cu:1116-1348 radixSortStep: per pass a 1024-key
// CTA-local split sort, findRadixOffsets, a CUDPP scan of the counters and
// reorderData, i.e. four launches and a library scan per 4-bit digit).
// Here every pass is one launch: the first digit's histogram is counted by
// the projection kernel and each pass counts the next digit's while its tile
// sits in shared memory; each CTA ranks a 4096-key tile with warp ballots
// (eight ballots give every lane the mask of lanes holding the same digit),
// publishes its per-digit counts, and finds its global offsets by a
// decoupled look-back over earlier tiles (one thread per digit, eight
// predecessor words per round trip) while the keys of its next tile load.
// Tiles are handed out in order by an atomic counter, so a tile only ever
// waits on tiles that running CTAs own; every wait is bounded and reports
// GSAP_ERR_DEVICE_TIMEOUT instead of hanging.  Stable: equal digits keep
// their input order, so the passes give the order of a stable sort.
#include "internal.cuh"

namespace gsap {

// Order-preserving map of IEEE-754 floats to uint32 (negative values: all
// bits inverted; non-negative: sign bit set), so that unsigned order of the
// images is the float order, -0.0 before +0.0 (the floatFlip /
// floatUnflip pair of sapDetection/radixsort.cu:110-137).
__device__ __forceinline__ uint32_t flip_f32(uint32_t f) { return f ^ ((f >> 31) ? 0xFFFFFFFFu : 0x80000000u); }
__device__ __forceinline__ uint32_t unflip_f32(uint32_t f) { return f ^ ((f >> 31) ? 0x80000000u : 0xFFFFFFFFu); }

// Exclusive scan over the 256 threads of a CTA; returns the exclusive value.
__device__ __forceinline__ uint32_t cta_excl_scan256(uint32_t v, uint32_t* s_w) {
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_w[wid] = x;
    __syncthreads();
    uint32_t pre = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w)
        if ((uint32_t)w < wid) pre += s_w[w];
    __syncthreads();
    return pre + x - v;
}

// 4096-key tiles run two CTAs per SM (128 registers), 2048-key tiles four
// (64 registers, no spills): the same keys in flight per SM either way.
template <int ITEMS>
__global__ void __launch_bounds__(kThreads, ITEMS <= 8 ? 4 : 2) k_onesweep(BpScratch S, const uint32_t* __restrict__ kin,
                                                       const uint32_t* __restrict__ vin,
                                                       uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                       const uint32_t* count_ptr, uint32_t cap, int pass,
                                                       uint32_t spin, SortGather G, int count_next, int fmode) {
    pdl_wait();
    constexpr int TILE = kThreads * ITEMS;
    __shared__ uint32_t s_k[TILE];
    __shared__ uint32_t s_next[256];  // histogram of the next pass's digit over this CTA's tiles
    __shared__ uint32_t s_v[TILE];
    __shared__ uint32_t s_wh[kThreads / 32][256];
    __shared__ uint32_t s_gdig[256];
    __shared__ uint32_t s_start[256];
    __shared__ uint32_t s_gb[256];
    __shared__ uint32_t s_scan[8];
    __shared__ uint32_t s_tile, s_tile_next;
    const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint32_t n = min(*count_ptr, cap);
    const uint32_t ntiles = (n + TILE - 1) / TILE;
    const int shift = 8 * pass;
    const uint32_t tag = (S.ctrl->epoch << 3) | (uint32_t)pass;
    const uint32_t lt = lanemask_lt();

    s_gdig[tid] = cta_excl_scan256(S.ctrl->hist[pass][tid], s_scan);
    if (tid == 0) s_tile = atomicAdd(&S.ctrl->tile_ctr[pass], 1u);
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) s_wh[w][tid] = 0u;
    s_next[tid] = 0u;
    __syncthreads();
    uint32_t t = s_tile;
    // The keys and values of the CTA's next tile are loaded while it waits in
    // the look-back of the current one (tickets are taken in order, so every
    // tile a CTA waits on belongs to a running CTA).
    uint32_t key[ITEMS], val[ITEMS];
    auto load_tile = [&](uint32_t tt) {
        const uint32_t wb0 = tt * TILE + wid * 32 * ITEMS;
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            const uint32_t idx = wb0 + k * 32 + lane;
            const bool in = tt < ntiles && idx < n;
            key[k] = in ? __ldcs(kin + idx) : 0u;
            if (fmode & kSortFlipIn) key[k] = flip_f32(key[k]);
            val[k] = in ? __ldcs(vin + idx) : 0u;
        }
    };
    load_tile(t);
    while (t < ntiles) {
        const uint32_t tbase = t * TILE;
        const uint32_t wb = tbase + wid * 32 * ITEMS;
        uint32_t tot = 0;
        {
            uint32_t rk[ITEMS];
            // warp-level multi-split ranking, items in index order
#pragma unroll
            for (int k = 0; k < ITEMS; ++k) {
                const bool valid = wb + k * 32 + lane < n;
                const uint32_t d = (key[k] >> shift) & 255u;
                uint32_t m = __ballot_sync(0xffffffffu, valid);
#pragma unroll
                for (int bit = 0; bit < 8; ++bit) {
                    uint32_t bal = __ballot_sync(0xffffffffu, (d >> bit) & 1u);
                    m &= ((d >> bit) & 1u) ? bal : ~bal;
                }
                uint32_t before = valid ? s_wh[wid][d] : 0u;
                uint32_t r = __popc(m & lt);
                __syncwarp();
                if (valid && r == 0) s_wh[wid][d] = before + __popc(m);
                __syncwarp();
                rk[k] = before + r;
            }
            __syncthreads();
            // per digit: exclusive warp offsets and the tile count
#pragma unroll
            for (int w = 0; w < kThreads / 32; ++w) {
                uint32_t c = s_wh[w][tid];
                s_wh[w][tid] = tot;
                tot += c;
            }
            // publish the aggregates before anything else
            st_lb_u64(S.status + (uint64_t)t * 256u + tid, lb_word(tag, t == 0 ? kFlagPrefix : kFlagAgg, tot));
            if (tid == 0) s_tile_next = atomicAdd(&S.ctrl->tile_ctr[pass], 1u);
            s_start[tid] = cta_excl_scan256(tot, s_scan);
            __syncthreads();  // every digit's tile start (and the next ticket) is read below
            // stage the tile in digit order (frees the registers for the next tile)
#pragma unroll
            for (int k = 0; k < ITEMS; ++k) {
                if (wb + k * 32 + lane < n) {
                    uint32_t d = (key[k] >> shift) & 255u;
                    uint32_t lp = s_start[d] + s_wh[wid][d] + rk[k];
                    if (lp < (uint32_t)TILE) {
                        s_k[lp] = key[k];
                        s_v[lp] = val[k];
                    } else {
                        atomicOr(&S.ctrl->error, kErrInternal);
                    }
                }
            }
        }
        const uint32_t t_next = s_tile_next;
        load_tile(t_next);  // in flight during the look-back and the write-out
        uint32_t excl = 0;
        if (t > 0) {
            excl = lookback(S.status, t, tid, 256u, tag, spin, &S.ctrl->error);
            st_lb_u64(S.status + (uint64_t)t * 256u + tid, lb_word(tag, kFlagPrefix, excl + tot));
        }
        s_gb[tid] = s_gdig[tid] + excl - s_start[tid];
        __syncthreads();
        const uint32_t tn = min((uint32_t)TILE, n - tbase);
        if (count_next)  // the next pass's digit histogram, counted here instead of up front
            for (uint32_t i = tid; i < tn; i += kThreads) atomicAdd(&s_next[(s_k[i] >> (shift + 8)) & 255u], 1u);
        for (uint32_t i = tid; i < tn; i += kThreads) {
            uint32_t kk = s_k[i];
            uint32_t g = s_gb[(kk >> shift) & 255u] + i;
            uint32_t vv = s_v[i];
            if (g >= n) {  // cannot happen with consistent counts; never write out of range
                atomicOr(&S.ctrl->error, kErrInternal);
                continue;
            }
            kout[g] = (fmode & kSortUnflipOut) ? unflip_f32(kk) : kk;
            if (vout) vout[g] = vv;
            if (G.smin) {  // last pass of the broadphase: entries in sorted order
                // The value holds the object index and the entry's owner
                // flags (set by the projection): a pair is owned by the cell
                // of (max lo2, max lo3), which both objects touch, so the
                // cell owns it iff each coordinate is some member's lowest.
                put_record(S, G, g, kk, vv);
            }
        }
        __syncthreads();  // s_k / s_v / s_wh are reused by the next tile
#pragma unroll
        for (int w = 0; w < kThreads / 32; ++w) s_wh[w][tid] = 0u;
        __syncthreads();
        t = t_next;
    }
    // One flush of the next digit's counts per CTA (not per tile): the 256
    // global counters take one atomic per CTA each instead of one per tile
    // (3.6M per pass for the 58M entries of a 4096-scene batch otherwise).
    if (count_next) {
        __syncthreads();
        const uint32_t c = s_next[tid];
        if (c) atomicAdd(&S.ctrl->hist[pass + 1][tid], c);
    }
}

// First pass of the broadphase sort (digit 0, the low bits of the quantised
// lower bound).  The first pass of an LSD sort need not keep the input order
// within a digit -- nothing earlier ordered the entries, and the later
// passes are stable -- so a tile needs neither the onesweep's ballot ranking
// nor its look-back chain: it counts its digits in shared memory, gives
// every entry a slot in its digit's run of the tile with a shared-memory
// atomic, stages the tile in digit order, reserves each digit's global range
// with one atomic on that digit's cursor (ranges start at the digit bases
// from the projection's histogram; tiles take them in any order) and writes
// the runs out coalesced.  Entries with equal keys may end in any order; the
// sweep's pair set does not depend on it.
template <int ITEMS>
__global__ void __launch_bounds__(kThreads, ITEMS <= 8 ? 4 : 2) k_pass0(BpScratch S, const uint32_t* __restrict__ kin,
                                                      const uint32_t* __restrict__ vin, uint32_t* __restrict__ kout,
                                                      uint32_t* __restrict__ vout, const uint32_t* count_ptr,
                                                      uint32_t cap) {
    pdl_wait();
    constexpr int TILE = kThreads * ITEMS;
    __shared__ uint32_t s_k[TILE];
    __shared__ uint32_t s_v[TILE];
    __shared__ uint32_t s_cnt[256];   // the tile's digit counts, then its slot cursors
    __shared__ uint32_t s_start[256]; // exclusive start of each digit's run in the tile
    __shared__ uint32_t s_gb[256];    // global position of each digit's run, minus its tile start
    __shared__ uint32_t s_base[256];  // digit bases of the pass
    __shared__ uint32_t s_next[256];  // counts of the next digit over this CTA's tiles
    __shared__ uint32_t s_scan[8];
    const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    Ctrl* C = S.ctrl;
    const uint32_t n = min(*count_ptr, cap);
    const uint32_t ntiles = (n + TILE - 1) / TILE;
    s_base[tid] = cta_excl_scan256(C->hist[0][tid], s_scan);
    s_next[tid] = 0u;
    for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const uint32_t tbase = t * TILE;
        const uint32_t wb = tbase + wid * 32 * ITEMS;
        uint32_t key[ITEMS], val[ITEMS];
        s_cnt[tid] = 0u;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            const uint32_t idx = wb + k * 32 + lane;
            key[k] = idx < n ? __ldcs(kin + idx) : 0u;
            val[k] = idx < n ? __ldcs(vin + idx) : 0u;
        }
#pragma unroll
        for (int k = 0; k < ITEMS; ++k)
            if (wb + k * 32 + lane < n) atomicAdd(&s_cnt[key[k] & 255u], 1u);
        __syncthreads();
        const uint32_t cnt = s_cnt[tid];
        const uint32_t st = cta_excl_scan256(cnt, s_scan);  // (has its own barriers)
        s_start[tid] = st;
        // this tile's range of the digit (any order among tiles)
        const uint32_t g = cnt ? atomicAdd(&C->cursor0[tid], cnt) : 0u;
        s_gb[tid] = s_base[tid] + g - st;
        s_cnt[tid] = st;  // slot cursors
        __syncthreads();
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            if (wb + k * 32 + lane < n) {
                const uint32_t lp = atomicAdd(&s_cnt[key[k] & 255u], 1u);
                s_k[lp] = key[k];
                s_v[lp] = val[k];
                atomicAdd(&s_next[(key[k] >> 8) & 255u], 1u);
            }
        }
        __syncthreads();
        const uint32_t tn = min((uint32_t)TILE, n - tbase);
        for (uint32_t i = tid; i < tn; i += kThreads) {
            const uint32_t kk = s_k[i];
            const uint32_t gp = s_gb[kk & 255u] + i;
            if (gp >= n) {  // cannot happen with consistent counts; never write out of range
                atomicOr(&C->error, kErrInternal);
                continue;
            }
            kout[gp] = kk;
            vout[gp] = s_v[i];
        }
        __syncthreads();  // s_k / s_v / s_cnt are reused by the next tile
    }
    __syncthreads();
    const uint32_t c = s_next[tid];
    if (c) atomicAdd(&C->hist[1][tid], c);
}

// Tile size: 4096 keys (three CTAs per SM) when the keys fill more than one
// round of such tiles, 2048 (five CTAs per SM) when they do not: a small
// call then spreads over twice the CTAs, each with half the serial work
// (16,384 boxes: 0.0431 against 0.0451 ms), while a large one keeps the
// fewer digit-cursor atomics of the larger tiles (1M: 0.4585 against 0.4639
// ms with 2048-key tiles).
cudaError_t launch_pass0(const BpScratch& s, const uint32_t* kin, const uint32_t* vin, uint32_t* kout,
                         uint32_t* vout, const uint32_t* count_ptr, uint64_t cap, cudaStream_t st,
                         uint64_t keys_hint) {
    static std::once_flag once[2][kMaxDevices];
    static int val[2][kMaxDevices];
    const int full_l = per_device(once[0], val[0], [] {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pass0<kSortItems>, kThreads, 0);
        return sm_count() * (per_sm > 0 ? per_sm : 1);
    });
    const uint32_t c = cap > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)cap;
    if (keys_hint && keys_hint <= (uint64_t)full_l * kSortTile) {
        const int full_s = per_device(once[1], val[1], [] {
            int per_sm = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pass0<kSortItemsSmall>, kThreads, 0);
            return sm_count() * (per_sm > 0 ? per_sm : 1);
        });
        launch_pdl(k_pass0<kSortItemsSmall>, call_grid(full_s, keys_hint, kSortTileMin), kThreads, 0, st, s, kin, vin,
                kout, vout, count_ptr, c);
    } else {
        const int grid = keys_hint ? call_grid(full_l, keys_hint, kSortTile) : full_l;
        launch_pdl(k_pass0<kSortItems>, grid, kThreads, 0, st, s, kin, vin, kout, vout, count_ptr, c);
    }
    return cudaGetLastError();
}

// Sweep records of the sorted entries.  The last radix pass used to write
// them from its scatter loop (two CTAs per SM, one entry per thread at a
// time): the two random 16-byte bound loads per entry then had few peers in
// flight, and with inputs larger than L2 (the 617 MB of a 4096-scene batch)
// the pass took three times as long as the others.  Here every thread of a
// full-occupancy grid issues the loads of kGatherU entries before it stores
// any record.
constexpr int kGatherU = 4;
__global__ void __launch_bounds__(kThreads) k_gather(BpScratch S, SortGather G, const uint32_t* __restrict__ vals,
                                                    const uint32_t* count_ptr, uint32_t cap) {
    pdl_wait();
    const uint32_t n = min(*count_ptr, cap);
    const uint32_t stride = gridDim.x * kThreads;
    for (uint32_t g0 = blockIdx.x * kThreads + threadIdx.x; g0 < n; g0 += stride * kGatherU) {
        uint32_t v[kGatherU];
        float4 lo[kGatherU], hi[kGatherU];
#pragma unroll
        for (int u = 0; u < kGatherU; ++u) {
            const uint32_t g = g0 + u * stride;
            v[u] = g < n ? __ldcs(vals + g) : 0u;
        }
#pragma unroll
        for (int u = 0; u < kGatherU; ++u) {
            if (g0 + u * stride >= n) continue;
            const uint32_t obj = v[u] & kObjMask;
            lo[u] = __ldg(G.mn + obj);
            if (G.mx) hi[u] = __ldg(G.mx + obj);
        }
#pragma unroll
        for (int u = 0; u < kGatherU; ++u) {
            const uint32_t g = g0 + u * stride;
            if (g >= n) continue;
            const uint32_t obj = v[u] & kObjMask, fl = v[u] >> kFlagShift;
            if (G.mx) {  // boxes: index and flags ride in the unused w lanes
                G.smin[g] = make_float4(lo[u].x, lo[u].y, lo[u].z, __uint_as_float(obj));
                G.smax[g] = make_float4(hi[u].x, hi[u].y, hi[u].z, __uint_as_float(fl));
            } else {     // spheres: radius in w, index and flags in the second record
                G.smin[g] = lo[u];
                G.smax[g] = make_float4(__uint_as_float(obj), __uint_as_float(fl), 0.f, 0.f);
            }
        }
    }
}

cudaError_t launch_gather(const BpScratch& s, const SortGather& G, const uint32_t* vals, const uint32_t* count_ptr,
                          uint64_t cap, cudaStream_t st) {
    static std::once_flag once[kMaxDevices];
    static int val[kMaxDevices];
    const int grid = per_device(once, val, [] {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gather, kThreads, 0);
        return sm_count() * (per_sm > 0 ? per_sm : 1);
    });
    const uint32_t c = cap > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)cap;
    launch_pdl(k_gather, grid, kThreads, 0, st, s, G, vals, count_ptr, c);
    return cudaGetLastError();
}

// Histograms of all passes for a standalone sort.
template <int PASSES>
__global__ void __launch_bounds__(kThreads) k_hist(Ctrl* C, const uint32_t* __restrict__ keys, uint32_t n,
                                                   int flip) {
    pdl_wait();
    __shared__ uint32_t s_hist[PASSES][256];
    for (uint32_t k = threadIdx.x; k < PASSES * 256; k += kThreads) (&s_hist[0][0])[k] = 0u;
    __syncthreads();
    for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
        uint32_t key = flip ? flip_f32(keys[i]) : keys[i];
#pragma unroll
        for (int p = 0; p < PASSES; ++p) atomicAdd(&s_hist[p][(key >> (8 * p)) & 255u], 1u);
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < PASSES * 256; k += kThreads) {
        uint32_t v = (&s_hist[0][0])[k];
        if (v) atomicAdd(&C->hist[0][0] + k, v);
    }
}

// Counter reset + new epoch for a standalone sort.
__global__ void k_sort_reset(Ctrl* C, uint32_t n, uint32_t* count_slot) {
    pdl_wait();
    uint32_t t = threadIdx.x;
    for (uint32_t k = t; k < kHistWords; k += 256u) (&C->hist[0][0])[k] = 0u;
    if (t == 0) {
        for (int p = 0; p < kMaxPasses + 4; ++p) C->tile_ctr[p] = 0;
        C->epoch = C->epoch + 1u;
        *count_slot = n;
    }
}

cudaError_t launch_sort_prep(const BpScratch& s, const uint32_t* keys, const uint32_t* count_ptr, uint32_t n,
                             int passes, cudaStream_t st, int flip) {
    launch_pdl(k_sort_reset, 1, 256, 0, st, s.ctrl, n, const_cast<uint32_t*>(count_ptr));
    int grid = sm_count() * 4;
    switch (passes) {
        case 1: launch_pdl(k_hist<1>, grid, kThreads, 0, st, s.ctrl, keys, n, flip); break;
        case 2: launch_pdl(k_hist<2>, grid, kThreads, 0, st, s.ctrl, keys, n, flip); break;
        case 3: launch_pdl(k_hist<3>, grid, kThreads, 0, st, s.ctrl, keys, n, flip); break;
        default: launch_pdl(k_hist<4>, grid, kThreads, 0, st, s.ctrl, keys, n, flip); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_sort_pass(const BpScratch& s, int pass, int passes, const uint32_t* kin, const uint32_t* vin,
                             uint32_t* kout, uint32_t* vout, const uint32_t* count_ptr, uint64_t cap,
                             uint32_t spin, cudaStream_t st, const SortGather* gather, bool count_next, int fmode,
                             int tile, uint64_t keys_hint) {
    SortGather G;
    if (gather) G = *gather;
    else G = SortGather{nullptr, nullptr, nullptr, nullptr};
    static std::once_flag once[2][kMaxDevices];
    static int val[2][kMaxDevices];
    const int small = tile == kSortTileMin ? 1 : 0;
    const int full = per_device(once[small], val[small], [small] {
        int per_sm = 0;
        if (small) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_onesweep<kSortItemsSmall>, kThreads, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_onesweep<kSortItems>, kThreads, 0);
        return sm_count() * (per_sm > 0 ? per_sm : 1);
    });
    const int grid = keys_hint ? call_grid(full, keys_hint, small ? kSortTileMin : kSortTile) : full;
    uint32_t c = cap > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)cap;
    const int next = (count_next && pass + 1 < passes) ? 1 : 0;
    if (small)
        launch_pdl(k_onesweep<kSortItemsSmall>, grid, kThreads, 0, st, s, kin, vin, kout, vout, count_ptr, c, pass,
                spin, G, next, fmode);
    else
        launch_pdl(k_onesweep<kSortItems>, grid, kThreads, 0, st, s, kin, vin, kout, vout, count_ptr, c, pass, spin,
                G, next, fmode);
    return cudaGetLastError();
}

}  // namespace gsap
