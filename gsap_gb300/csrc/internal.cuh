// Internal declarations shared by the sm_103a kernels and the C-ABI layer.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

namespace gsap {

// Launch constants (SM count, occupancy-derived grids) are cached per device
// ordinal: computed once per device under std::call_once, so concurrent
// first calls from several host threads are safe and a second device gets
// its own values.  Ordinals beyond the table are recomputed on every call.
constexpr int kMaxDevices = 64;
template <class F>
int per_device(std::once_flag (&once)[kMaxDevices], int (&val)[kMaxDevices], F compute) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return compute();
    std::call_once(once[dev], [&] { val[dev] = compute(); });
    return val[dev];
}

// Pipeline kernels are launched with programmatic stream serialisation: a
// kernel's CTAs may be scheduled as soon as every CTA of the kernel before it
// in the stream has exited, without waiting for that grid's completion to be
// processed, so the launch latency of each link of the chain overlaps the
// end of the previous one.  Every kernel launched this way begins with
// pdl_wait(), which waits (in hardware) until the previous kernel has
// completed and its writes are visible, before any other statement.  So a
// kernel still starts its work only after all earlier ones have finished,
// as under plain stream order.
template <typename... P, typename... A>
inline cudaError_t launch_pdl(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                              A&&... args) {
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<A&&>(args)...);
}

constexpr int kChunk = 4096;          // objects per PCA / projection work item
// Calls of at most kPcaSmallWork work items run kPcaSplitSmall PCA CTAs per
// item (one object per thread), each with its own partial.
constexpr uint32_t kPcaSmallWork = 64;
constexpr uint32_t kPcaSplitSmall = 16;
constexpr int kThreads = 256;         // threads per CTA of the streaming kernels
constexpr int kMaxPasses = 4;         // radix passes (8-bit digits, <= 32-bit keys)
constexpr int kSortItems = 16;        // keys per thread in a onesweep tile (default)
constexpr int kSortTile = kThreads * kSortItems;
constexpr int kSortItemsSmall = 8;    // the smaller tile the autotuner may choose
constexpr int kSortTileMin = kThreads * kSortItemsSmall;
constexpr uint32_t kDefaultSpin = 1u << 24;
// Bucket sort: a sub-bucket is a cell together with the top T bits of the
// quantised lower bound, i.e. the top bits of the key above `shift`; at most
// kMaxSub of them (the key layout keeps the cells at or below 2^20).
constexpr uint32_t kMaxSubBits = 20;
constexpr uint32_t kMaxSub = 1u << kMaxSubBits;
constexpr uint32_t kSubTopBits = 4;

// Sticky device error bits (ctrl->error).
enum : uint32_t {
    kErrEntryCap = 1u,     // sweep entries exceeded their capacity
    kErrPairCap = 2u,      // pairs exceeded the output capacity
    kErrTimeout = 4u,      // a bounded wait gave up
    kErrNonFinite = 8u,    // NaN / Inf in the input bounds
    kErrCellRange = 16u,   // internal: grid wider than 65535 cells per axis
    kErrInternal = 32u,    // an internal consistency check failed (index out of range)
    kErrOffsets = 64u,     // batched scene offsets not 0 .. n non-decreasing
};

// Look-back status word: [63:32] tag, [31:30] flag, [29:0] value.
constexpr uint64_t kFlagAgg = 1ull << 30;
constexpr uint64_t kFlagPrefix = 2ull << 30;
constexpr uint32_t kValMask = (1u << 30) - 1u;

// Control block: counters shared by the stages of one call.  Counters that a
// stage consumes are reset by the stage that runs before it (the PCA
// finish's last CTA resets the projection/sort/sweep counters; in temporal
// mode k_reset does), or by their own last user (per-scene PCA counters, the
// row counters zeroed by the row scan), so that no memset runs per call.
struct Ctrl {
    uint32_t error;
    uint32_t epoch;           // ++ once per pipeline run; tags look-back words
    uint32_t scenes_done;     // PCA: completed scenes (self-resetting)
    uint32_t entry_count;     // projection output count
    unsigned long long pair_count;
    uint32_t tile_ctr[kMaxPasses + 4];
    uint32_t sweep_ctr;
    uint32_t key_bits;        // total radix key width of this run
    uint32_t qbits;           // low bits of the key holding the quantised lower bound
    uint32_t total_buckets;
    uint32_t scan_total;      // total of the last look-back scan
    uint32_t scan_ctr;        // tile counter of the look-back scan
    uint32_t sort_n;          // key count of a standalone sort
    uint32_t long_rows;       // canonical output: rows queued for k_rowsort_long
    unsigned long long tests; // sweep: candidate pairs tested (diagnostics)
    unsigned long long iters; // sweep: warp iterations of the candidate loop (diagnostics)
    uint32_t hist[kMaxPasses][256];
    // first broadphase pass (k_pass0): entries placed so far per digit;
    // contiguous with hist and zeroed with it (kHistWords words)
    uint32_t cursor0[256];
    // temporal mode: the key layout computed from this call's input for the
    // next call (committed at the end of the call)
    uint32_t qbits_next, key_bits_next, total_buckets_next, pad_next;
};

constexpr uint32_t kHistWords = (kMaxPasses + 1) * 256u;

// Per-scene parameters written by the PCA kernel.
struct Scene {
    float u[9];          // sweep axis u1 then secondary axes u2, u3 (rows)
    float q_org, q_range; // lower-bound quantisation: q = (x - q_org) * (2^Q / q_range)
    float c2_org, c2_inv; // cell index on u2: floor((x - c2_org) * c2_inv), clamped
    float c3_org, c3_inv;
    uint32_t G2, G3;      // cells per secondary axis
    uint32_t bucket_base; // first global bucket id of this scene
    uint32_t n;           // objects in the scene
    float q_scale;        // 2^Q / q_range, set once Q is known (same value in every kernel)
    uint32_t pad;
    double eig[3];        // eigenvalues, descending
    double mean[3];       // centre mean
    double axes[9];       // FP64 axes (rows)
};

// PCA partial sums of one work item: 18 (hi, lo) compensated FP32 pairs
// (sum d, sum d d^T, sum h, sum h h^T with d = centre - pilot, h =
// |half extent|), then max |h| per axis.
constexpr int kPcaQ = 18;
struct PcaPartial {
    float hi[kPcaQ];
    float lo[kPcaQ];
    float hmax[3];
    float pad;
};

// Device scratch of a broadphase handle.
// A sweep entry's value: its object index in the low bits and its owner
// flags on top (bit 30: the entry's cell is the object's lowest on u2, bit
// 31: on u3).  The entry capacity is below 2^30, so object indices fit.
constexpr uint32_t kFlagShift = 30;
constexpr uint32_t kObjMask = (1u << kFlagShift) - 1u;

struct BpScratch {
    Ctrl* ctrl;
    Scene* scenes;
    PcaPartial* partials;
    uint32_t* scene_done;      // per-scene PCA completion counters
    Scene* scenes_next;        // temporal mode: per-scene parameters for the next call
    uint32_t* work_start;      // per-scene first work item (S+1), batched plan
    uint32_t* work_scene;      // scene of every work item, batched plan
    uint32_t* objscene;        // per object scene id (batched only)
    uint32_t* keys[2];
    uint32_t* vals[2];         // object index | owner flags << kFlagShift
    uint64_t* status;          // look-back words (per tile and digit)
    // Sweep entries in sorted order, one 32-byte record each.  Boxes:
    // smin = (lo.xyz, object index bits), smax = (hi.xyz, owner flag bits).
    // Spheres: smin = (centre.xyz, radius), smax = (object index bits, owner
    // flag bits, 0, 0).  Owner flags: bit 0 when the entry's cell column is
    // the object's lowest on u2, bit 1 when its row is the lowest on u3.
    float4* smin;
    float4* smax;
    uint32_t* longrows;        // canonical output: ids of rows placed by k_rowsort_long
    uint32_t* rowcnt;          // per object pair counts (canonical output)
    uint32_t* rowoff;          // exclusive offsets, n+1
    uint32_t* tile_sums;       // row-count sums per 4096-row tile (canonical output)
    uint32_t* tmp_pairs;       // unsorted pairs before canonicalisation
    uint2* grp_pairs;          // pairs grouped by row, before the in-row order (canonical output)
    uint32_t* tmp_rank;        // per unsorted pair k: its slot in row first (rank[k]); both-direction
                               // form: slots in row first and row second (rank[2k], rank[2k + 1])
    // bucket sort: entries per sub-bucket (zero between calls), their
    // exclusive offsets (M + 1), per-4096 sums of the offset scan
    uint32_t* subcnt;
    uint32_t* substart;
    uint32_t* subsum;
    uint64_t entry_cap;
    uint64_t pair_cap_internal;
    uint64_t status_words;
    uint32_t max_n;
    uint32_t max_scenes;
    uint32_t max_work;
};

struct BpArgs {
    const float4* mn;          // AABB min (or spheres)
    const float4* mx;          // AABB max (nullptr in sphere mode)
    const uint32_t* scene_off; // device S+1 offsets (nullptr: one scene)
    uint32_t n;
    uint32_t num_scenes;
    uint32_t num_work;         // upper bound of work items launched
    int mode;                  // 0 AABB, 1 sphere
    int axis_mode;             // 0 PCA, 1 reference axis
    uint32_t key_bits;         // 16, 24 or 32
    float cell_factor;
    uint32_t spin_limit;
};

// ---------------------------------------------------------------- launches
// Each returns cudaGetLastError() of its launch.
cudaError_t launch_plan(const BpScratch& s, const BpArgs& a, cudaStream_t st);
// temporal != 0: the finish writes the parameters into scenes_next and the
// *_next layout fields and leaves the pipeline counters alone (the main
// branch resets them with launch_reset and adopts the new parameters with
// launch_commit once both branches have finished).
cudaError_t launch_pca(const BpScratch& s, const BpArgs& a, cudaStream_t st, int temporal = 0);
cudaError_t launch_reset(const BpScratch& s, cudaStream_t st);
cudaError_t launch_commit(const BpScratch& s, uint32_t num_scenes, cudaStream_t st);
cudaError_t launch_project(const BpScratch& s, const BpArgs& a, int passes, cudaStream_t st);
// Gather epilogue of the last sort pass: entry g also gets the bounds of its
// object and its owner flags, so the sweep reads candidates in order.
struct SortGather {
    const float4* mn;
    const float4* mx;          // nullptr in sphere mode
    float4* smin;
    float4* smax;
};
// fmode of a sort pass: kSortFlipIn maps float keys to their ordered uint32
// image as they are loaded (first pass of a float sort), kSortUnflipOut maps
// them back as they are stored (last pass).
enum : int { kSortFlipIn = 1, kSortUnflipOut = 2 };
// tile: keys per tile, kSortTile or kSortTileMin (the status table must
// hold 256 words per tile of that size).  keys_hint: an estimate of the key
// count that sizes the grid (call_grid); 0 for the full-occupancy grid.
cudaError_t launch_sort_pass(const BpScratch& s, int pass, int passes, const uint32_t* kin,
                             const uint32_t* vin, uint32_t* kout, uint32_t* vout,
                             const uint32_t* count_ptr, uint64_t cap, uint32_t spin, cudaStream_t st,
                             const SortGather* gather = nullptr, bool count_next = false, int fmode = 0,
                             int tile = kSortTile, uint64_t keys_hint = 0);
// Counter reset and the digit histograms of a standalone sort (flip != 0:
// of the float images of the keys).
cudaError_t launch_sort_prep(const BpScratch& s, const uint32_t* keys, const uint32_t* count_ptr,
                             uint32_t n, int passes, cudaStream_t st, int flip = 0);
// Bucket sort of the projection's entries (keys[0] / vals[0], counted per
// sub-bucket by the projection): scan of the sub-bucket counts, scatter into
// sub-buckets (keys[1] / vals[1]), local sort of every sub-bucket; the
// sorted keys end in keys[0] and the entry records in G.smin / G.smax.
cudaError_t launch_bucket_sort(const BpScratch& s, const SortGather& G, uint32_t spin, cudaStream_t st);
// First radix pass of the broadphase (digit 0 of the projection's entries),
// not order-preserving: entries of one digit may land in any order, which
// the first pass of an LSD sort may do (the later passes are stable).
cudaError_t launch_pass0(const BpScratch& s, const uint32_t* kin, const uint32_t* vin, uint32_t* kout,
                         uint32_t* vout, const uint32_t* count_ptr, uint64_t cap, cudaStream_t st,
                         uint64_t keys_hint = 0);
// Sweep records of the sorted entries (put_record) from their sorted values
// (object index | owner flags), after the last radix pass: a kernel of its
// own at full occupancy, several entries' random bound loads in flight per
// thread.
cudaError_t launch_gather(const BpScratch& s, const SortGather& G, const uint32_t* vals, const uint32_t* count_ptr,
                          uint64_t cap, cudaStream_t st);
// Box bytes (32 per object) above which the broadphase gathers the sweep
// records in launch_gather instead of in its last radix pass.
constexpr uint64_t kGatherInPassBytes = 96ull << 20;
// Per-device set-up of the bucket sort's launch (kernel attributes); called
// when a handle is created, outside any stream capture.
cudaError_t bucket_sort_setup();

// Sub-bucket layout of a key layout: sub-bucket id = key >> shift, `count`
// sub-buckets (a cell and the top T <= kSubTopBits bits of its quantised
// lower bound, T chosen so that count <= kMaxSub).
struct SubLayout {
    uint32_t shift, count;
};
__host__ __device__ inline SubLayout sub_layout_of(uint32_t Q, uint32_t total_buckets) {
    uint32_t bb = 0;
    while (bb < 32 && (1ull << bb) < (uint64_t)total_buckets) ++bb;
    int T = (int)kSubTopBits;
    if (T > (int)Q) T = (int)Q;
    if (T > (int)kMaxSubBits - (int)bb) T = (int)kMaxSubBits - (int)bb;
    if (T < 0) T = 0;
    SubLayout L;
    L.shift = Q - (uint32_t)T;
    L.count = total_buckets << T;
    return L;
}
#ifdef __CUDACC__
__device__ inline SubLayout sub_layout(const Ctrl* C) { return sub_layout_of(C->qbits, C->total_buckets); }
#endif
cudaError_t launch_sweep(const BpScratch& s, const BpArgs& a, const uint32_t* keys,
                         uint2* pairs, uint64_t pair_cap, int count_rows, cudaStream_t st);
cudaError_t launch_canonical(const BpScratch& s, uint32_t n, const uint2* in_pairs, uint64_t in_cap,
                             uint2* out_pairs, uint64_t out_cap, int both, int32_t* entries,
                             uint64_t entry_cap, uint32_t spin, cudaStream_t st);
int sm_count();

// Grids of the persistent and grid-stride kernels (radix passes, sweep,
// scatter, rank) are sized for the call: at most one CTA per `per` units of
// an estimate of its work from the object count, and never more than the
// full-occupancy grid.  Any grid covers all the work (tickets, work stealing
// or grid-stride loops); the clamp spares a small call the hundreds of CTAs
// that would find nothing to do, each of which still has to be scheduled
// and run its prologue on the call's latency chain.
inline int call_grid(int full, uint64_t work, uint64_t per) {
    const uint64_t g = (work + per - 1) / per;
    return (int)(g < 1 ? 1 : (g < (uint64_t)full ? g : (uint64_t)full));
}
// Estimates of a call's work from its object count n: sweep entries (cell
// replication; about 2.3 per object at the 1M workload) and stored pairs.
constexpr uint64_t kEstEntriesPerObject = 4;
constexpr uint64_t kEstPairsPerObject = 8;

// ------------------------------------------------------------ device helpers
#ifdef __CUDACC__
// Look-back words hold flag and value in one 64-bit word, so a relaxed
// (single-copy atomic) load/store at gpu scope is enough: a reader sees the
// old word or the whole new one, and nothing else is published through it.
__device__ __forceinline__ uint64_t ld_lb_u64(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_lb_u64(uint64_t* p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}
// First statement of every kernel launched by launch_pdl: wait until the
// previous kernel of the stream has completed and its writes are visible.
// (No kernel signals its dependents early: a dependent scheduled while the
// current kernel still runs lands its CTAs unevenly on the SMs, which cost
// the grid-stride kernels more than the earlier start gained.)
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ uint64_t lb_word(uint32_t tag, uint64_t flag, uint32_t val) {
    return ((uint64_t)tag << 32) | flag | (uint64_t)(val & kValMask);
}

// Bounded decoupled look-back over the tiles before `tile` for column `col`
// of a status table with `cols` columns.  Returns the exclusive prefix; on
// timeout sets kErrTimeout and returns what it has (the caller still
// publishes, so no later tile can wait forever).
// The words of up to kLbWindow predecessors are loaded at once (independent
// loads), then consumed in order: aggregates are summed until a prefix is
// met; a word not yet published stops the window and is re-read.
constexpr int kLbWindow = 8;
__device__ __forceinline__ uint32_t lookback(uint64_t* status, uint32_t tile, uint32_t col, uint32_t cols,
                                             uint32_t tag, uint32_t spin_limit, uint32_t* err) {
    uint32_t excl = 0;
    int64_t j = (int64_t)tile - 1;
    uint32_t spins = 0;
    while (j >= 0) {
        uint64_t w[kLbWindow];
#pragma unroll
        for (int k = 0; k < kLbWindow; ++k)
            w[k] = (j - k >= 0) ? ld_lb_u64(status + (uint64_t)(j - k) * cols + col) : 0ull;
        int consumed = 0;
        bool done = false;
#pragma unroll
        for (int k = 0; k < kLbWindow; ++k) {
            if (j - k < 0) { done = true; break; }
            const uint64_t v = w[k];
            if (!((uint32_t)(v >> 32) == tag && (v & (kFlagAgg | kFlagPrefix)))) break;
            excl += (uint32_t)(v & kValMask);
            ++consumed;
            if (v & kFlagPrefix) { done = true; break; }
        }
        if (done) break;
        j -= consumed;
        if (consumed == 0) {
            if (++spins > spin_limit) {
                atomicOr(err, kErrTimeout);
                return excl;
            }
            if (spins > 64) __nanosleep(64);
        }
    }
    return excl;
}

// u . x over the box spanned by corners a, b (any order), rounded outward:
// [lo, hi] contains the exact projection of the box.
__device__ __forceinline__ void project_box(const float* u, float3 a, float3 b, float& lo, float& hi) {
    float l0 = fminf(__fmul_rd(u[0], a.x), __fmul_rd(u[0], b.x));
    float l1 = fminf(__fmul_rd(u[1], a.y), __fmul_rd(u[1], b.y));
    float l2 = fminf(__fmul_rd(u[2], a.z), __fmul_rd(u[2], b.z));
    float h0 = fmaxf(__fmul_ru(u[0], a.x), __fmul_ru(u[0], b.x));
    float h1 = fmaxf(__fmul_ru(u[1], a.y), __fmul_ru(u[1], b.y));
    float h2 = fmaxf(__fmul_ru(u[2], a.z), __fmul_ru(u[2], b.z));
    lo = __fadd_rd(__fadd_rd(l0, l1), l2);
    hi = __fadd_ru(__fadd_ru(h0, h1), h2);
}

// Box of a sphere (centre, radius in w): centre -/+ |r|, rounded outward.
__device__ __forceinline__ void sphere_box(float4 p, float3& a, float3& b) {
    const float r = fabsf(p.w);
    a = make_float3(__fsub_rd(p.x, r), __fsub_rd(p.y, r), __fsub_rd(p.z, r));
    b = make_float3(__fadd_ru(p.x, r), __fadd_ru(p.y, r), __fadd_ru(p.z, r));
}

// Sweep records of sorted entry g (value = object index | owner flags <<
// kFlagShift), written by the last step of either sort: the bounds of its
// object (boxes: (lo.xyz, object index), (hi.xyz, owner flags); spheres:
// (centre, radius), (object index, owner flags, 0, 0)).
__device__ __forceinline__ void put_record(const BpScratch& S, const SortGather& G, uint32_t g, uint32_t key,
                                           uint32_t val) {
    (void)S;
    (void)key;
    const uint32_t obj = val & kObjMask, fl = val >> kFlagShift;
    const float4 lo = __ldg(G.mn + obj);
    if (G.mx) {  // boxes: index and flags ride in the unused w lanes
        const float4 hi = __ldg(G.mx + obj);
        G.smin[g] = make_float4(lo.x, lo.y, lo.z, __uint_as_float(obj));
        G.smax[g] = make_float4(hi.x, hi.y, hi.z, __uint_as_float(fl));
    } else {     // spheres: radius in w, index and flags in the second record
        G.smin[g] = lo;
        G.smax[g] = make_float4(__uint_as_float(obj), __uint_as_float(fl), 0.f, 0.f);
    }
}

// Error-free transformation a + b = s + e (Knuth two-sum).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// Compensated accumulation (hi, lo) += x.
__device__ __forceinline__ void kahan_add(float& hi, float& lo, float x) {
    float s, e;
    two_sum(hi, x, s, e);
    hi = s;
    lo = __fadd_rn(lo, e);
}
// Merge two compensated sums.
__device__ __forceinline__ void kahan_merge(float& hi, float& lo, float hi2, float lo2) {
    float s, e;
    two_sum(hi, hi2, s, e);
    hi = s;
    lo = __fadd_rn(__fadd_rn(lo, lo2), e);
}
#endif

// ------------------------------------------------------------- work plan
#ifdef __CUDACC__

// Scene s covers objects [scene_begin, scene_end).  The caller's offsets are
// clamped into [0, n] and made non-decreasing here, so no kernel can index
// outside the input whatever the offsets hold; k_plan reports offsets that
// needed clamping (GSAP_ERR_INVALID).
__device__ __forceinline__ uint32_t scene_begin(const BpArgs& A, uint32_t s) {
    return A.scene_off ? min(A.scene_off[s], A.n) : 0u;
}
__device__ __forceinline__ uint32_t scene_end(const BpArgs& A, uint32_t s) {
    return A.scene_off ? min(max(A.scene_off[s + 1], scene_begin(A, s)), A.n) : A.n;
}
__device__ __forceinline__ uint32_t work_items(uint32_t n_s) {
    return n_s == 0 ? 1u : (n_s + kChunk - 1) / kChunk;
}

// Work item -> (scene, object range, first work item of the scene, count).
__device__ __forceinline__ bool map_work(uint32_t w, const BpScratch& S, const BpArgs& A, uint32_t& scene,
                                         uint32_t& b, uint32_t& e, uint32_t& wfirst, uint32_t& nw) {
    if (!A.scene_off) {
        nw = work_items(A.n);
        if (w >= nw) return false;
        scene = 0;
        wfirst = 0;
        b = w * kChunk;
        e = min(A.n, b + kChunk);
        return true;
    }
    if (w >= S.work_start[A.num_scenes]) return false;
    // the plan's table (a search over work_start here was a chain of ~12
    // dependent loads at the start of every CTA of a 4096-scene batch)
    const uint32_t lo = S.work_scene[w];
    scene = lo;
    wfirst = S.work_start[lo];
    nw = S.work_start[lo + 1] - wfirst;
    uint32_t sb = scene_begin(A, lo), se = scene_end(A, lo);
    b = sb + (w - wfirst) * kChunk;
    e = min(se, b + kChunk);
    return true;
}
#endif

}  // namespace gsap
