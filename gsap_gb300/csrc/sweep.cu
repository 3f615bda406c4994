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
// Persistent warps take 128 consecutive sorted entries at a time from an
// atomic counter (work stealing) and handle them in chunks of 32.  For its
// entry e a lane first finds, by a galloping then binary search over the
// sorted keys, the end of the run of
// entries with key <= (bucket | q(hi1)): the q map is monotone, so these are
// exactly the later entries of the same cell whose interval on u1 can meet
// e's, and the run stops at the cell (and scene) boundary by construction.
// The warp then flattens the 32 runs into one list of candidate tests (a
// warp scan of the run lengths) and works through it 32 tests per step, test
// t on lane t mod 32: every lane does useful work however uneven the runs
// are, and the lanes of a step read consecutive candidates (coalesced; the
// last sort pass wrote every entry's bounds in sorted order).  A lane finds
// the entry of its test from the run starts that fall into the step's
// window (one warp OR-reduction and a popcount) and reads that entry's
// bounds from shared memory.
// Candidates pass the exact test on the original FP32 bounds (closed AABB
// test of Aabb::overlaps, include/aabb.h:47-57, or the strict squared
// sphere test of SapKernel.cu:1897-1903 with one rounding per operation)
// and the owner-cell rule: a pair is reported only in the cell holding
// (max(lo2_i, lo2_j), max(lo3_i, lo3_j)), which both objects touch, so each
// overlapping pair comes out exactly once and no sort + unique pass is
// needed.  With the per-entry owner flags of the gather (is this cell the
// object's lowest on u2 / on u3) the rule is (f_i | f_j) == 3.  Object index
// and flags travel inside the two 16-byte bound records, so a test makes
// no load that depends on another.  Hits are compacted through a per-warp
// shared-memory buffer that reserves global space with one atomic per up to
// 128 pairs; for the canonical output every stored pair also draws its slot
// in its row from the row counters.
#include "internal.cuh"

namespace gsap {

__device__ __forceinline__ float proj_hi(const float* u, float3 a, float3 b) {
    float h0 = fmaxf(__fmul_ru(u[0], a.x), __fmul_ru(u[0], b.x));
    float h1 = fmaxf(__fmul_ru(u[1], a.y), __fmul_ru(u[1], b.y));
    float h2 = fmaxf(__fmul_ru(u[2], a.z), __fmul_ru(u[2], b.z));
    return __fadd_ru(__fadd_ru(h0, h1), h2);
}

constexpr int kBuf = 128;  // pairs buffered per warp before a global reservation
constexpr uint32_t kGrab = 4;  // 32-entry chunks taken per work-counter atomic
constexpr int kWarps = kThreads / 32;

template <int MODE>
__global__ void __launch_bounds__(kThreads) k_sweep(BpScratch S, BpArgs A, const uint32_t* __restrict__ keys,
                                                    uint2* __restrict__ pairs,
                                                    uint64_t pair_cap, int count_rows) {
    pdl_wait();
    __shared__ uint2 s_buf[kWarps][kBuf];
    // entries of the warp's chunk that have candidates, in run order
    // (boxes: (lo.xyz, jb), (hi.xyz, flags); spheres: (centre, radius),
    // (jb, flags, -, -)); the candidate of test t is jb + t
    __shared__ float4 s_t0[kWarps][32];
    __shared__ float4 s_t1[kWarps][32];
    __shared__ uint32_t s_id[kWarps][32];  // object index
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t lt = lanemask_lt();
    const uint32_t le = lt | (1u << lane);
    Ctrl* C = S.ctrl;
    const float4* __restrict__ smin = S.smin;
    const float4* __restrict__ smax = S.smax;
    const uint32_t E = (uint32_t)min((uint64_t)C->entry_count, S.entry_cap);
    const uint32_t Q = C->qbits;
    const uint32_t qmask = (1u << Q) - 1u;
    const float qmax = (float)qmask;
    uint32_t nbuf = 0;
    uint64_t tests = 0;
    uint32_t steps = 0;

    // Reserves global space for the warp's buffered pairs and stores them.
    // For the canonical output each stored pair also takes its slot in its
    // row (and, both-direction form, in its second id's row) from the row
    // counters; the returning atomics of a lane's pairs are issued together.
    auto flush = [&]() {
        __syncwarp();
        unsigned long long base = 0;
        if (lane == 0 && nbuf) base = atomicAdd(&C->pair_count, (unsigned long long)nbuf);
        base = __shfl_sync(0xffffffffu, base, 0);
        constexpr int kPer = kBuf / 32;
        uint2 p[kPer], rk[kPer];
        bool st[kPer];
#pragma unroll
        for (int u = 0; u < kPer; ++u) {
            const uint32_t k = lane + 32u * u;
            st[u] = k < nbuf && base + k < pair_cap;  // rows count stored pairs only
            rk[u] = make_uint2(0u, 0u);
            if (st[u]) {
                p[u] = s_buf[wid][k];
                if (count_rows) {
                    rk[u].x = atomicAdd(&S.rowcnt[p[u].x], 1u);
                    if (count_rows == 2) rk[u].y = atomicAdd(&S.rowcnt[p[u].y], 1u);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < kPer; ++u) {
            if (!st[u]) continue;
            const uint64_t k = base + lane + 32u * u;
            pairs[k] = p[u];
            if (count_rows == 2) reinterpret_cast<uint2*>(S.tmp_rank)[k] = rk[u];
            else if (count_rows) S.tmp_rank[k] = rk[u].x;
        }
        __syncwarp();
        nbuf = 0;
    };

    // Work is taken kGrab chunks of 32 entries at a time: every atomic on the
    // one shared counter serialises at its L2 slice, so fewer, larger grabs.
    // With fewer entries than kGrab chunks for every warp of the grid (small
    // calls), one chunk at a time, so that the work spreads over all warps.
    const uint32_t grab = (uint64_t)E >= (uint64_t)gridDim.x * kWarps * 32u * kGrab ? 32u * kGrab : 32u;
    // Entries for at most one chunk per warp (small calls): the warp's chunk
    // is its own index, with no round trip to the counter before or after.
    const bool one_chunk = (uint64_t)E <= (uint64_t)gridDim.x * kWarps * 32u;
    // first gallop step: runs are tens of entries in large calls, a few in
    // the sparse small ones
    const uint32_t step0 = one_chunk ? 2u : 16u;
    uint32_t base = 0, grab_end = 0;
    while (true) {
        if (base >= grab_end) {
            uint32_t g = 0;
            if (lane == 0)
                g = !one_chunk ? atomicAdd(&C->sweep_ctr, grab)
                               : (grab_end == 0 ? (blockIdx.x * kWarps + wid) * 32u : 0xFFFFFFFFu);
            base = __shfl_sync(0xffffffffu, g, 0);
            grab_end = base + grab;
        }
        if (base >= E) break;
        const uint32_t e = base + lane;
        base += 32u;
        uint32_t run = 0;  // candidates of entry e: e+1 .. e+run
        float4 pa = make_float4(0.f, 0.f, 0.f, 0.f), pb = pa;
        uint32_t i = 0;
        uint32_t fl = 0;
        if (e < E) {
            const uint32_t key = keys[e];
            pa = smin[e];
            pb = smax[e];
            i = __float_as_uint(MODE == 0 ? pa.w : pb.x);
            fl = __float_as_uint(MODE == 0 ? pb.w : pb.y);
            const Scene* sc = &S.scenes[S.objscene ? S.objscene[i] : 0u];
            float3 a, b;
            if (MODE == 0) {
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
            const uint32_t kb = (key & ~qmask) | qh;  // >= key: q(hi1) >= q(lo1)
            // last index with key <= kb: gallop from e with a first step near
            // the typical run length (step0), then bisect
            // (lo: key <= kb, hi: key > kb or E)
            uint32_t lo = e, hi = E, step = step0;
            while (true) {
                if (step >= E - lo) break;
                const uint32_t p = lo + step;
                if (__ldg(keys + p) > kb) { hi = p; break; }
                lo = p;
                step <<= 1;
            }
            while (hi - lo > 1) {
                const uint32_t mid = lo + ((hi - lo) >> 1);
                if (__ldg(keys + mid) <= kb) lo = mid;
                else hi = mid;
            }
            run = lo - e;
        }
        // flatten the runs: exclusive start of each run in the warp's test list
        uint32_t x = run;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, x, 31);
        const uint32_t start = x - run;
        const uint32_t nz = __ballot_sync(0xffffffffu, run > 0);
        if (run > 0) {
            const uint32_t r = __popc(nz & lt);
            const uint32_t jb = e + 1u - start;
            if (MODE == 0) {
                s_t0[wid][r] = make_float4(pa.x, pa.y, pa.z, __uint_as_float(jb));
                s_t1[wid][r] = make_float4(pb.x, pb.y, pb.z, __uint_as_float(fl));
            } else {
                s_t0[wid][r] = pa;
                s_t1[wid][r] = make_float4(__uint_as_float(jb), __uint_as_float(fl), 0.f, 0.f);
            }
            s_id[wid][r] = i;
        }
        __syncwarp();
        tests += total;
        uint32_t before = 0;  // runs that start before the current window
        // whole steps need no bound check; the last, partial step does
        auto step = [&](const uint32_t t0, const bool full) {
            ++steps;
            const uint32_t d = start - t0;
            const uint32_t starts = __reduce_or_sync(0xffffffffu, (run > 0 && d < 32u) ? (1u << d) : 0u);
            const uint32_t t = t0 + lane;
            bool hit = false;
            uint32_t o = 0, oi = 0;
            if (full || t < total) {
                const uint32_t m = before + __popc(starts & le) - 1u;  // run of test t
                const float4 ea = s_t0[wid][m], eb = s_t1[wid][m];
                const uint32_t j = __float_as_uint(MODE == 0 ? ea.w : eb.x) + t;
                const uint32_t efl = __float_as_uint(MODE == 0 ? eb.w : eb.y);
                const float4 qa = __ldg(smin + j);
                bool ov;
                uint32_t jid, jfl;
                if (MODE == 0) {
                    const float4 qb = __ldg(smax + j);
                    jid = __float_as_uint(qa.w);
                    jfl = __float_as_uint(qb.w);
                    ov = (ea.x <= qb.x) & (qa.x <= eb.x) & (ea.y <= qb.y) & (qa.y <= eb.y) & (ea.z <= qb.z) &
                         (qa.z <= eb.z);
                } else {
                    const uint2 w = __ldg(reinterpret_cast<const uint2*>(smax + j));
                    jid = w.x;
                    jfl = w.y;
                    float dx = __fsub_rn(ea.x, qa.x), dy = __fsub_rn(ea.y, qa.y), dz = __fsub_rn(ea.z, qa.z);
                    float t1 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                    float rr = __fadd_rn(ea.w, qa.w);
                    ov = t1 < __fmul_rn(rr, rr);
                }
                if (ov && (efl | jfl) == 3u) {
                    hit = true;
                    o = jid;
                    oi = s_id[wid][m];
                }
            }
            before += __popc(starts);
            const uint32_t hm = __ballot_sync(0xffffffffu, hit);
            if (hm) {
                const uint32_t cnt = __popc(hm);
                if (nbuf + cnt > kBuf) flush();
                if (hit) s_buf[wid][nbuf + __popc(hm & lt)] = make_uint2(min(oi, o), max(oi, o));
                nbuf += cnt;
            }
        };
        uint32_t t0 = 0;
        for (; t0 + 32u <= total; t0 += 32u) step(t0, true);
        if (t0 < total) step(t0, false);
        __syncwarp();  // the next chunk overwrites the run table
    }
    flush();
    // diagnostics: candidate tests and warp steps
    if (lane == 0 && tests) {
        atomicAdd(&C->tests, (unsigned long long)tests);
        atomicAdd(&C->iters, (unsigned long long)steps);
    }
}

cudaError_t launch_sweep(const BpScratch& s, const BpArgs& a, const uint32_t* keys,
                         uint2* pairs, uint64_t pair_cap, int count_rows, cudaStream_t st) {
    static std::once_flag once[2][kMaxDevices];
    static int val[2][kMaxDevices];
    const int m = a.mode == 1 ? 1 : 0;
    const int full = per_device(once[m], val[m], [m] {
        int per_sm = 0;
        if (m == 0) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sweep<0>, kThreads, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sweep<1>, kThreads, 0);
        return sm_count() * (per_sm > 0 ? per_sm : 1);
    });
    // one CTA per 512 estimated entries (two 32-entry chunks per warp)
    const int grid = call_grid(full, (uint64_t)a.n * kEstEntriesPerObject, 2u * kWarps * 32u);
    if (m == 0) launch_pdl(k_sweep<0>, grid, kThreads, 0, st, s, a, keys, pairs, pair_cap, count_rows);
    else launch_pdl(k_sweep<1>, grid, kThreads, 0, st, s, a, keys, pairs, pair_cap, count_rows);
    return cudaGetLastError();
}

}  // namespace gsap
