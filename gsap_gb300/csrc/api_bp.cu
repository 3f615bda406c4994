// C ABI of the broadphase (include/gsap.h): handle, scratch ownership and the
// launch sequence of one call.
//
// Replaces the host side of the reference's Sap class
// (sapDetection/Sap.cpp:12-335).  The reference sizes every launch on the
// host and reads counts back in between (>= 8 blocking device-to-host
// copies per Sap::collision, CUDPP plans created per call); here all counts
// stay on the device, each stage sizes itself from them, and a call is a
// fixed sequence of launches on the caller's stream (optionally a cached
// CUDA graph) followed, only when the caller asks for host counts, by one
// small read of the control block.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gsap.h"
#include "../../include/gsap_debug.h"
#include "api_internal.h"
#include "internal.cuh"
#include "scene_math.cuh"

using namespace gsap;

// ------------------------------------------------------------------ errors

static thread_local std::string g_err;

static gsap_status fail(gsap_status st, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return st;
}

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(GSAP_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                        __FILE__, __LINE__);                                                  \
    } while (0)

extern "C" const char* gsap_last_error(void) { return g_err.c_str(); }

gsap_status gsap::set_error(gsap_status st, const char* msg) { return fail(st, "%s", msg); }

namespace gsap {
int sm_count() {
    static std::once_flag once[kMaxDevices];
    static int val[kMaxDevices];
    return per_device(once, val, [] {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        return n > 0 ? n : 1;
    });
}
}  // namespace gsap

extern "C" void gsap_config_default(gsap_config* c) {
    if (!c) return;
    memset(c, 0, sizeof(*c));
    c->mode = GSAP_MODE_AABB;
    c->axis_mode = GSAP_AXIS_PCA;
    c->max_scenes = 1;
    c->entry_factor = 8;
    c->pair_factor = 16;
    c->sort_bits = 32;
    c->cell_factor = 2.0f;
    c->spin_limit = kDefaultSpin;
    c->sort_tile = kSortTile;
}

// ------------------------------------------------------------------ handle

// A cached pipeline graph is keyed by its shape (sizes, flags, settings) and
// by the caller's buffers.  A call whose buffers are new but whose shape is
// cached captures the launch sequence again and updates an instantiated
// graph of that shape in place (cudaGraphExecUpdate) once kPerShape graphs
// of the shape exist, instead of instantiating yet another one.
struct GraphShape {
    uint32_t n, S, flags, mode, both;
    uint32_t key_bits;
    float cell_factor;
    uint32_t sort_mode, sort_tile;
    uint64_t cap, ecap;
    bool operator==(const GraphShape& o) const { return memcmp(this, &o, sizeof(*this)) == 0; }
};
struct GraphKey {
    GraphShape shape;
    const void *mn, *mx, *off, *pairs, *dcount, *entries;
    bool operator==(const GraphKey& o) const { return memcmp(this, &o, sizeof(*this)) == 0; }
};

struct GraphEntry {
    GraphKey key;
    cudaGraphExec_t exec;
    uint64_t last_use;
};
constexpr size_t kMaxGraphs = 128;  // cached pipeline graphs per handle (LRU)
constexpr size_t kPerShape = 64;    // graphs of one shape before new buffers update one in place

struct gsap_sap {
    gsap_config cfg;
    BpScratch s;
    int device;
    uint32_t* h_ctrl;   // pinned copy of the head of the control block
    cudaStream_t cap_stream;
    std::vector<GraphEntry>* graphs;
    uint64_t use_clock;
    size_t per_shape;   // graphs of one shape kept before new buffers update one (default kPerShape)
    bool timing;
    cudaEvent_t ev[8];
    int nstages;
    // temporal mode: a side stream for the PCA branch, and what the
    // parameters in the scratch were last computed for
    cudaStream_t side;
    cudaEvent_t ev_fork, ev_join;
    bool tp_valid;
    uint32_t tp_n, tp_S, tp_mode, tp_bits, tp_axis;
    float tp_cf;
};

static void free_scratch(gsap_sap* h) {
    BpScratch& s = h->s;
    void* ptrs[] = {s.ctrl, s.scenes, s.scenes_next, s.partials, s.scene_done, s.work_start, s.work_scene, s.objscene,
                    s.keys[0], s.keys[1], s.vals[0], s.vals[1], s.status, s.rowcnt, s.rowoff, s.tmp_pairs,
                    s.grp_pairs, s.tmp_rank, s.smin, s.smax, s.longrows, s.tile_sums, s.subcnt, s.substart,
                    s.subsum};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (h->h_ctrl) cudaFreeHost(h->h_ctrl);
    if (h->graphs) {
        for (auto& g : *h->graphs) cudaGraphExecDestroy(g.exec);
        delete h->graphs;
        h->graphs = nullptr;
    }
    if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
    if (h->side) cudaStreamDestroy(h->side);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    for (auto& e : h->ev)
        if (e) cudaEventDestroy(e);
}

extern "C" gsap_sap* gsap_sap_create(uint32_t max_n, const gsap_config* cfg) {
    gsap_config c;
    gsap_config_default(&c);
    if (cfg) c = *cfg;
    if (c.max_scenes == 0) c.max_scenes = 1;
    if (c.entry_factor == 0) c.entry_factor = 8;
    if (c.pair_factor == 0) c.pair_factor = 16;
    if (c.sort_bits == 0) c.sort_bits = 32;
    if (c.sort_bits != 16 && c.sort_bits != 24 && c.sort_bits != 32) {
        fail(GSAP_ERR_INVALID, "sort_bits must be 16, 24 or 32");
        return nullptr;
    }
    if (c.cell_factor <= 0.f) c.cell_factor = 2.0f;
    if (c.spin_limit == 0) c.spin_limit = kDefaultSpin;
    if (c.sort_mode != GSAP_SORT_BUCKET && c.sort_mode != GSAP_SORT_RADIX) {
        fail(GSAP_ERR_INVALID, "unknown sort_mode %u", c.sort_mode);
        return nullptr;
    }
    if (c.sort_tile == 0) c.sort_tile = kSortTile;
    if (c.sort_tile != (uint32_t)kSortTile && c.sort_tile != (uint32_t)kSortTileMin) {
        fail(GSAP_ERR_INVALID, "sort_tile must be %d or %d", kSortTileMin, kSortTile);
        return nullptr;
    }
    if (max_n == 0) max_n = 1;
    uint64_t ecap = (uint64_t)c.entry_factor * max_n + 4096;
    if (ecap >= (1ull << 30)) { fail(GSAP_ERR_INVALID, "entry capacity %llu exceeds 2^30", (unsigned long long)ecap); return nullptr; }
    gsap_sap* h = new gsap_sap();
    memset(h, 0, sizeof(*h));
    h->cfg = c;
    h->graphs = new std::vector<GraphEntry>();
    h->per_shape = kPerShape;
    cudaGetDevice(&h->device);
    BpScratch& s = h->s;
    s.max_n = max_n;
    s.max_scenes = c.max_scenes;
    s.max_work = (max_n + kChunk - 1) / kChunk + c.max_scenes + 1;
    s.entry_cap = ecap;
    s.pair_cap_internal = (uint64_t)c.pair_factor * max_n + 4096;
    uint64_t tiles = (ecap + kSortTileMin - 1) / kSortTileMin + 1;  // status words for the smaller tile
    s.status_words = tiles * 256 + (max_n / 2048 + 2);  // digit words, scan words
    bool ok = true;
    auto A = [&](void** p, size_t bytes) {
        if (!ok) return;
        if (cudaMalloc(p, bytes) != cudaSuccess) { ok = false; return; }
        if (cudaMemset(*p, 0, bytes) != cudaSuccess) ok = false;
    };
    A((void**)&s.ctrl, sizeof(Ctrl));
    A((void**)&s.scenes, sizeof(Scene) * c.max_scenes);
    A((void**)&s.scenes_next, sizeof(Scene) * c.max_scenes);
    // one partial per PCA CTA: per work item, or kPcaSplitSmall per item for small calls
    A((void**)&s.partials, sizeof(PcaPartial) * std::max<uint64_t>(s.max_work, (uint64_t)kPcaSmallWork * kPcaSplitSmall));
    A((void**)&s.scene_done, 4ull * c.max_scenes);
    A((void**)&s.work_start, 4ull * (c.max_scenes + 1));
    A((void**)&s.work_scene, 4ull * s.max_work);
    if (c.max_scenes > 1) A((void**)&s.objscene, 4ull * max_n);
    for (int k = 0; k < 2; ++k) {
        A((void**)&s.keys[k], 4ull * ecap);
        A((void**)&s.vals[k], 4ull * ecap);
    }
    A((void**)&s.status, 8ull * s.status_words);
    A((void**)&s.smin, 16ull * ecap);
    A((void**)&s.smax, 16ull * ecap);
    A((void**)&s.longrows, 4ull * (max_n + 1));
    A((void**)&s.rowcnt, 4ull * (max_n + 1));
    A((void**)&s.rowoff, 4ull * (max_n + 1));
    A((void**)&s.tile_sums, 4ull * (max_n / 4096 + 2));
    A((void**)&s.tmp_pairs, 8ull * s.pair_cap_internal);
    A((void**)&s.grp_pairs, 16ull * s.pair_cap_internal);  // both-direction form: two entries per pair
    A((void**)&s.tmp_rank, 8ull * s.pair_cap_internal);
    A((void**)&s.subcnt, 4ull * kMaxSub);
    A((void**)&s.substart, 4ull * (kMaxSub + 1));
    A((void**)&s.subsum, 4ull * (kMaxSub / 4096));
    if (ok && bucket_sort_setup() != cudaSuccess) ok = false;
    if (ok && cudaMallocHost((void**)&h->h_ctrl, 64) != cudaSuccess) ok = false;
    if (ok && cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking) != cudaSuccess) ok = false;
    for (auto& e : h->ev)
        if (ok && cudaEventCreate(&e) != cudaSuccess) ok = false;
    if (ok && cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking) != cudaSuccess) ok = false;
    if (ok && cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) != cudaSuccess) ok = false;
    if (ok && cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess) ok = false;
    if (!ok) {
        cudaError_t e = cudaGetLastError();
        fail(GSAP_ERR_CUDA, "gsap_sap_create: allocation failed (%s)", cudaGetErrorString(e));
        free_scratch(h);
        delete h;
        return nullptr;
    }
    return h;
}

extern "C" void gsap_sap_destroy(gsap_sap* h) {
    if (!h) return;
    free_scratch(h);
    delete h;
}

extern "C" void gsap_sap_enable_timing(gsap_sap* h, int enable) {
    if (h) h->timing = enable != 0;
}

extern "C" int gsap_sap_stage_times(gsap_sap* h, float* out, int max_stages) {
    if (!h || !out) return 0;
    if (h->nstages > 0 && cudaEventSynchronize(h->ev[h->nstages]) != cudaSuccess) return 0;
    int k = 0;
    for (; k < h->nstages && k < max_stages; ++k)
        if (cudaEventElapsedTime(&out[k], h->ev[k], h->ev[k + 1]) != cudaSuccess) return k;
    return k;
}

// ---------------------------------------------------------------- pipeline

struct Call {
    const float4 *mn, *mx;
    const uint32_t* off;
    uint32_t n, S;
    int mode;
    uint2* pairs;
    uint64_t cap;
    uint64_t* d_count;
    int32_t* entries;   // both-direction format: pairEntries output
    uint64_t ecap;
    uint32_t flags;
    int both;           // 1: Sap::collision format
};

// Temporal mode is used when asked for and the scratch holds parameters
// computed for a call of the same shape; otherwise the call runs the plain
// pipeline (its TEMPORAL bit cleared, so it also has its own cached graph).
static void temporal_resolve(gsap_sap* h, Call& c) {
    if (!(c.flags & GSAP_FLAG_TEMPORAL)) return;
    const bool ok = h->tp_valid && !h->timing && h->tp_n == c.n && h->tp_S == c.S && h->tp_mode == (uint32_t)c.mode &&
                    h->tp_bits == h->cfg.sort_bits && h->tp_axis == h->cfg.axis_mode && h->tp_cf == h->cfg.cell_factor;
    if (!ok) c.flags &= ~GSAP_FLAG_TEMPORAL;
}

static void temporal_note(gsap_sap* h, const Call& c) {
    h->tp_valid = true;
    h->tp_n = c.n;
    h->tp_S = c.S;
    h->tp_mode = (uint32_t)c.mode;
    h->tp_bits = h->cfg.sort_bits;
    h->tp_axis = h->cfg.axis_mode;
    h->tp_cf = h->cfg.cell_factor;
}

static gsap_status record(gsap_sap* h, const Call& c, cudaStream_t st, bool timed) {
    BpScratch& s = h->s;
    BpArgs a;
    a.mn = c.mn;
    a.mx = c.mx;
    a.scene_off = c.off;
    a.n = c.n;
    a.num_scenes = c.S;
    a.num_work = (c.n + kChunk - 1) / kChunk + (c.off ? c.S : 1);
    a.mode = c.mode;
    a.axis_mode = (int)h->cfg.axis_mode;
    a.key_bits = h->cfg.sort_bits;
    a.cell_factor = h->cfg.cell_factor;
    a.spin_limit = h->cfg.spin_limit;
    const int passes = (int)(a.key_bits / 8);
    int ev = 0;
    static const char* const kStage[] = {"gsap:pca", "gsap:project", "gsap:sort", "gsap:sweep", "gsap:output"};
    NvtxRange nv;
    int stage = 0;
    auto mark = [&]() {
        if (timed) cudaEventRecord(h->ev[ev++], st);
        if (stage < 5) nv.next(kStage[stage]);
        ++stage;
    };
    mark();
    const bool temporal = (c.flags & GSAP_FLAG_TEMPORAL) != 0;
    if (c.off) CK(launch_plan(s, a, st));
    if (temporal) {
        // The projection, sort and sweep of this call use the parameters of
        // the previous call (already in the scratch); this call's PCA runs
        // beside them and prepares the next call's.  Any grid gives the same
        // pair set, so the result is exact either way.
        CK(cudaEventRecord(h->ev_fork, st));
        CK(cudaStreamWaitEvent(h->side, h->ev_fork, 0));
        CK(launch_pca(s, a, h->side, 1));
        CK(cudaEventRecord(h->ev_join, h->side));
        CK(launch_reset(s, st));
    } else {
        CK(launch_pca(s, a, st));
    }
    mark();
    const bool bucket = h->cfg.sort_mode == GSAP_SORT_BUCKET;
    CK(launch_project(s, a, bucket ? 0 : passes, st));
    mark();
    const uint32_t* count = &s.ctrl->entry_count;
    int src = 0;
    SortGather gather{c.mn, c.mode == GSAP_MODE_AABB ? c.mx : nullptr, s.smin, s.smax};
    if (bucket) {
        CK(launch_bucket_sort(s, gather, a.spin_limit, st));  // sorted keys in keys[0]
    } else {
        // The entries' bounds go into the sweep records in sorted order: from
        // the last pass's scatter loop, or, for a batch of scenes whose
        // boxes do not fit in L2, from a full-occupancy gather kernel.  A
        // batch's sorted entries touch one scene's boxes at a time, so the
        // gather kernel's many loads in flight find them in L2: 4.38 -> 4.09
        // ms for 4096 scenes (38.6M boxes).  One large scene's entries touch
        // its boxes at random, and there the pass's own loop, overlapped
        // with its scatter, is faster (16.8M boxes: 9.47 against 9.64 ms).
        const bool separate = c.S > 1 && (uint64_t)c.n * 32ull > kGatherInPassBytes;
        for (int p = 0; p < passes; ++p) {
            const bool last = p == passes - 1 && !separate;
            const uint64_t est = (uint64_t)c.n * kEstEntriesPerObject;
            if (p == 0)
                CK(launch_pass0(s, s.keys[src], s.vals[src], s.keys[src ^ 1], s.vals[src ^ 1], count, s.entry_cap,
                                st, est));
            else
                CK(launch_sort_pass(s, p, passes, s.keys[src], s.vals[src], s.keys[src ^ 1],
                                    last ? nullptr : s.vals[src ^ 1], count, s.entry_cap, a.spin_limit, st,
                                    last ? &gather : nullptr, true, 0, (int)h->cfg.sort_tile, est));
            src ^= 1;
        }
        if (separate) CK(launch_gather(s, gather, s.vals[src], count, s.entry_cap, st));
    }
    mark();
    const bool canon = (c.flags & GSAP_FLAG_SORTED) || c.both;
    uint2* sweep_out = canon ? (uint2*)s.tmp_pairs : c.pairs;
    uint64_t sweep_cap = canon ? s.pair_cap_internal : c.cap;
    CK(launch_sweep(s, a, s.keys[src], sweep_out, sweep_cap, canon ? (c.both ? 2 : 1) : 0, st));
    mark();
    if (canon) {
        CK(launch_canonical(s, c.n, (const uint2*)s.tmp_pairs, s.pair_cap_internal, c.pairs, c.cap, c.both,
                            c.entries, c.ecap, a.spin_limit, st));
        mark();
    }
    if (temporal) {
        CK(cudaStreamWaitEvent(st, h->ev_join, 0));
        CK(launch_commit(s, c.S, st));
    }
    if (c.d_count) CK(cudaMemcpyAsync(c.d_count, &s.ctrl->pair_count, 8, cudaMemcpyDeviceToDevice, st));
    if (timed) h->nstages = ev - 1;
    return GSAP_OK;
}

static gsap_status run(gsap_sap* h, const Call& c, cudaStream_t st) {
    int dev = -1;
    cudaGetDevice(&dev);
    if (dev != h->device) return fail(GSAP_ERR_INVALID, "handle was created on device %d, current is %d", h->device, dev);
    const bool use_graph = (c.flags & GSAP_FLAG_GRAPH) && !h->timing;
    if (!use_graph) return record(h, c, st, h->timing);
    GraphKey k;
    memset(&k, 0, sizeof(k));
    k.mn = c.mn; k.mx = c.mx; k.off = c.off; k.pairs = c.pairs; k.dcount = c.d_count; k.entries = c.entries;
    GraphShape& sh = k.shape;
    sh.n = c.n; sh.S = c.S; sh.flags = c.flags; sh.mode = (uint32_t)c.mode; sh.both = (uint32_t)c.both;
    sh.cap = c.cap; sh.ecap = c.ecap;
    sh.key_bits = h->cfg.sort_bits; sh.cell_factor = h->cfg.cell_factor;  // tuned settings are baked into a graph
    sh.sort_mode = h->cfg.sort_mode;
    sh.sort_tile = h->cfg.sort_tile;
    // LRU cache of captured pipelines, one per (inputs, outputs, sizes, flags)
    GraphEntry* hit = nullptr;
    size_t same = 0;
    GraphEntry* lru_same = nullptr;  // least recently used graph of this shape
    for (auto& g : *h->graphs) {
        if (g.key == k) { hit = &g; break; }
        if (g.key.shape == sh) {
            ++same;
            if (!lru_same || g.last_use < lru_same->last_use) lru_same = &g;
        }
    }
    if (!hit) {
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal));
        gsap_status r = record(h, c, h->cap_stream, false);
        cudaError_t e = cudaStreamEndCapture(h->cap_stream, &g);
        if (r != GSAP_OK) return r;
        if (e != cudaSuccess) return fail(GSAP_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
        if (same >= h->per_shape) {
            // new buffers, known shape: the same launches with other pointers
            cudaGraphExecUpdateResultInfo info;
            e = cudaGraphExecUpdate(lru_same->exec, g, &info);
            if (e == cudaSuccess) {
                lru_same->key = k;
                hit = lru_same;
            } else {  // topology differs after all: replace that graph
                cudaGetLastError();
                cudaGraphExecDestroy(lru_same->exec);
                h->graphs->erase(h->graphs->begin() + (lru_same - h->graphs->data()));
            }
        }
        if (!hit) {
            if (h->graphs->size() >= kMaxGraphs) {
                size_t old = 0;
                for (size_t i = 1; i < h->graphs->size(); ++i)
                    if ((*h->graphs)[i].last_use < (*h->graphs)[old].last_use) old = i;
                cudaGraphExecDestroy((*h->graphs)[old].exec);
                h->graphs->erase(h->graphs->begin() + old);
            }
            GraphEntry ent;
            ent.key = k;
            e = cudaGraphInstantiate(&ent.exec, g, 0);
            if (e != cudaSuccess) {
                cudaGraphDestroy(g);
                return fail(GSAP_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
            }
            h->graphs->push_back(ent);
            hit = &h->graphs->back();
        }
        cudaGraphDestroy(g);
    }
    hit->last_use = ++h->use_clock;
    CK(cudaGraphLaunch(hit->exec, st));
    return GSAP_OK;
}

// Reads error word and pair count (synchronizes), clears the error word.
static gsap_status finish(gsap_sap* h, cudaStream_t st, uint64_t* count_out, uint64_t cap) {
    CK(cudaMemcpyAsync(h->h_ctrl, h->s.ctrl, 24, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    uint32_t err = h->h_ctrl[0];
    uint64_t cnt;
    memcpy(&cnt, (char*)h->h_ctrl + 16, 8);
    if (count_out) *count_out = cnt;
    if (err) {
        h->tp_valid = false;  // the next call recomputes its parameters first
        CK(cudaMemsetAsync(&h->s.ctrl->error, 0, 4, st));
        CK(cudaStreamSynchronize(st));
        if (err & kErrTimeout) return fail(GSAP_ERR_DEVICE_TIMEOUT, "a device-side wait exceeded its iteration cap");
        if (err & kErrNonFinite) return fail(GSAP_ERR_NONFINITE, "NaN or Inf in the input bounds");
        if (err & kErrEntryCap) return fail(GSAP_ERR_CAPACITY, "sweep entries exceeded the handle's capacity (raise entry_factor)");
        if (err & kErrCellRange) return fail(GSAP_ERR_CAPACITY, "too many sweep cells for the key width");
        if (err & kErrPairCap) return fail(GSAP_ERR_CAPACITY, "pairs exceeded an output capacity");
        if (err & kErrOffsets) return fail(GSAP_ERR_INVALID, "scene offsets must run from 0 to n and never decrease");
        if (err & kErrInternal) return fail(GSAP_ERR_CUDA, "internal consistency check failed (device error word 0x%x)", err);
        return fail(GSAP_ERR_CUDA, "device error word 0x%x", err);
    }
    if (cnt > cap) return fail(GSAP_ERR_CAPACITY, "%llu pairs exceed the capacity %llu", (unsigned long long)cnt, (unsigned long long)cap);
    return GSAP_OK;
}

static bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

static gsap_status validate(gsap_sap* h, const float* mn, const float* mx, uint32_t n, int mode, const void* pairs,
                            uint32_t S) {
    if (!h) return fail(GSAP_ERR_INVALID, "null handle");
    if (n > h->s.max_n) return fail(GSAP_ERR_CAPACITY, "n = %u exceeds the handle's max_n = %u", n, h->s.max_n);
    if (S > h->s.max_scenes) return fail(GSAP_ERR_CAPACITY, "%u scenes exceed max_scenes = %u", S, h->s.max_scenes);
    if (n > 0 && (!mn || !aligned16(mn))) return fail(GSAP_ERR_INVALID, "bounds pointer null or not 16-byte aligned");
    if (n > 0 && mode == GSAP_MODE_AABB && (!mx || !aligned16(mx)))
        return fail(GSAP_ERR_INVALID, "max-bounds pointer null or not 16-byte aligned");
    if (n > 1 && !pairs) return fail(GSAP_ERR_INVALID, "null pair output");
    if (pairs && ((uintptr_t)pairs & 7u)) return fail(GSAP_ERR_INVALID, "pair output not 8-byte aligned");
    return GSAP_OK;
}

static gsap_status broadphase(gsap_sap* h, const float* d_min, const float* d_max, const uint32_t* off,
                              uint32_t S, uint32_t n, uint32_t* d_pairs, uint64_t cap, uint64_t* d_count,
                              uint64_t* h_count, uint32_t flags, void* stream) {
    if (!h) return fail(GSAP_ERR_INVALID, "null handle");
    NvtxRange range("gsap:broadphase");
    int mode = (int)h->cfg.mode;
    gsap_status v = validate(h, d_min, d_max, n, mode, d_pairs, S);
    if (v != GSAP_OK) return v;
    cudaStream_t st = (cudaStream_t)stream;
    if (n < 2 && !off) {
        if (d_count) CK(cudaMemsetAsync(d_count, 0, 8, st));
        if (h_count) *h_count = 0;
        return GSAP_OK;
    }
    Call c;
    memset(&c, 0, sizeof(c));
    c.mn = (const float4*)d_min;
    c.mx = mode == GSAP_MODE_AABB ? (const float4*)d_max : nullptr;
    c.off = off;
    c.n = n;
    c.S = off ? S : 1;
    c.mode = mode;
    c.pairs = (uint2*)d_pairs;
    c.cap = cap;
    c.d_count = d_count;
    c.flags = flags;
    temporal_resolve(h, c);
    gsap_status r = run(h, c, st);
    if (r != GSAP_OK) return r;
    temporal_note(h, c);
    // sorted output goes through the internal pair buffer first
    uint64_t eff = (flags & GSAP_FLAG_SORTED) ? (cap < h->s.pair_cap_internal ? cap : h->s.pair_cap_internal) : cap;
    if (h_count) return finish(h, st, h_count, eff);
    return GSAP_OK;
}

extern "C" gsap_status gsap_broadphase_aabb(gsap_sap* h, const float* d_min, const float* d_max, uint32_t n,
                                            uint32_t* d_pairs, uint64_t pair_cap, uint64_t* d_count,
                                            uint64_t* h_count, uint32_t flags, void* stream) {
    return broadphase(h, d_min, d_max, nullptr, 1, n, d_pairs, pair_cap, d_count, h_count, flags, stream);
}

// Times every (sort, key width, cell factor) setting of a small grid on the
// caller's input and keeps the fastest in the handle.  The sort is the
// bucket sort or the onesweep radix passes with 4096- or 2048-key tiles
// (more, shorter tiles: a longer look-back chain but more CTAs per SM); the
// digit width stays 8 bits (11-bit digits would multiply the look-back
// words and the per-tile digit counters by 8).  The key width sets the radix
// passes (16 bits: two 8-bit digits, 24 bits: three, 32 bits: four), and
// with the cells it shares the key with, the q resolution of the sweep and
// the most cells the grid may have; the cell factor sets the cell edge on u2/u3 and with it the
// replication (entries to sort) against the candidate run length (tests).
// Any setting gives the same pair set; only the time differs.
extern "C" gsap_status gsap_sap_autotune(gsap_sap* h, const float* d_min, const float* d_max,
                                         const uint32_t* d_scene_offsets, uint32_t num_scenes, uint32_t n,
                                         uint32_t* d_pairs, uint64_t pair_cap, uint32_t flags, int reps,
                                         gsap_config* out, void* stream) {
    if (!h) return fail(GSAP_ERR_INVALID, "null handle");
    if (reps < 1) reps = 1;
    if (d_scene_offsets && num_scenes == 0) return fail(GSAP_ERR_INVALID, "batched call needs scene offsets");
    const uint32_t S = d_scene_offsets ? num_scenes : 1;
    // (sort, radix tile): the bucket sort has no tile setting
    const uint32_t sort_grid[3][2] = {{GSAP_SORT_RADIX, (uint32_t)kSortTile},
                                      {GSAP_SORT_RADIX, (uint32_t)kSortTileMin},
                                      {GSAP_SORT_BUCKET, (uint32_t)kSortTile}};
    const uint32_t bits_grid[3] = {16, 24, 32};
    const float cf_grid[5] = {1.0f, 1.5f, 2.0f, 2.5f, 3.0f};
    const gsap_config saved = h->cfg;
    cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float best_ms = -1.f;
    gsap_config best = saved;
    for (const auto& sm : sort_grid)
        for (uint32_t bits : bits_grid)
            for (float cf : cf_grid) {
                // 16-bit keys leave room for at most 1024 cells: tried on
                // single scenes of up to 2^18 objects only (beyond, or shared
                // by a batch's scenes, the cells are too few to be worth it)
                if (bits == 16 && (S > 1 || n > (1u << 18))) continue;
                h->cfg.sort_mode = sm[0];
                h->cfg.sort_tile = sm[1];
                h->cfg.sort_bits = bits;
                h->cfg.cell_factor = cf;
                uint64_t cnt = 0;
                // untimed first call: builds the graph and checks capacities
                gsap_status r = broadphase(h, d_min, d_max, d_scene_offsets, S, n, d_pairs, pair_cap, nullptr, &cnt,
                                           flags, stream);
                if (r != GSAP_OK) continue;  // this setting does not fit the handle; try the next
                cudaEventRecord(e0, st);
                for (int k = 0; k < reps && r == GSAP_OK; ++k)
                    r = broadphase(h, d_min, d_max, d_scene_offsets, S, n, d_pairs, pair_cap, nullptr, nullptr,
                                   flags, stream);
                cudaEventRecord(e1, st);
                if (r == GSAP_OK) r = finish(h, st, &cnt, ~0ull);
                float ms = 0.f;
                if (r != GSAP_OK || cudaEventSynchronize(e1) != cudaSuccess ||
                    cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
                    continue;
                if (best_ms < 0.f || ms < best_ms) {
                    best_ms = ms;
                    best = h->cfg;
                }
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    h->cfg = best;
    if (best_ms < 0.f) return fail(GSAP_ERR_CAPACITY, "no setting of the tuning grid fits this input");
    if (out) *out = best;
    return GSAP_OK;
}

extern "C" gsap_status gsap_broadphase_batched(gsap_sap* h, const float* d_min, const float* d_max,
                                               const uint32_t* d_scene_offsets, uint32_t num_scenes, uint32_t n,
                                               uint32_t* d_pairs, uint64_t pair_cap, uint64_t* d_count,
                                               uint64_t* h_count, uint32_t flags, void* stream) {
    if (!d_scene_offsets || num_scenes == 0) return fail(GSAP_ERR_INVALID, "batched call needs scene offsets");
    if (!h) return fail(GSAP_ERR_INVALID, "null handle");
    if (h->s.max_scenes < 2 && num_scenes > 1)
        return fail(GSAP_ERR_INVALID, "handle created with max_scenes = %u", h->s.max_scenes);
    if (n == 0) {
        if (d_count) CK(cudaMemsetAsync(d_count, 0, 8, (cudaStream_t)stream));
        if (h_count) *h_count = 0;
        return GSAP_OK;
    }
    return broadphase(h, d_min, d_max, d_scene_offsets, num_scenes, n, d_pairs, pair_cap, d_count, h_count, flags,
                      stream);
}

extern "C" gsap_status gsap_sap_collision(gsap_sap* h, float spacing, const float* d_spheres, uint32_t n,
                                          int32_t* d_pairs, int32_t* d_pair_entries, int32_t* h_num_pairs,
                                          int32_t* h_num_entries, uint64_t pair_cap, uint64_t entry_cap,
                                          void* stream) {
    (void)spacing;
    gsap_status v = validate(h, d_spheres, nullptr, n, GSAP_MODE_SPHERE, d_pairs, 1);
    if (v != GSAP_OK) return v;
    if (!d_pair_entries && n > 1) return fail(GSAP_ERR_INVALID, "null pairEntries output");
    cudaStream_t st = (cudaStream_t)stream;
    if (n < 2) {
        if (h_num_pairs) *h_num_pairs = 0;
        if (h_num_entries) *h_num_entries = 0;
        return GSAP_OK;
    }
    Call c;
    memset(&c, 0, sizeof(c));
    c.mn = (const float4*)d_spheres;
    c.n = n;
    c.S = 1;
    c.mode = GSAP_MODE_SPHERE;
    c.pairs = (uint2*)d_pairs;
    c.cap = pair_cap;
    c.entries = d_pair_entries;
    c.ecap = entry_cap;
    c.both = 1;
    gsap_status r = run(h, c, st);
    if (r != GSAP_OK) return r;
    temporal_note(h, c);
    uint64_t np = 0;
    uint64_t half = pair_cap / 2;
    r = finish(h, st, &np, half < h->s.pair_cap_internal ? half : h->s.pair_cap_internal);
    uint32_t ne = 0;
    CK(cudaMemcpyAsync(&ne, &h->s.ctrl->scan_total, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (h_num_pairs) *h_num_pairs = (int32_t)(2 * np);
    if (h_num_entries) *h_num_entries = (int32_t)ne;
    if (r != GSAP_OK) return r;
    if (2 * np > pair_cap) return fail(GSAP_ERR_CAPACITY, "%llu pairs exceed the capacity %llu", (unsigned long long)(2 * np), (unsigned long long)pair_cap);
    if (ne > entry_cap) return fail(GSAP_ERR_CAPACITY, "%u pair entries exceed the capacity %llu", ne, (unsigned long long)entry_cap);
    return GSAP_OK;
}

extern "C" gsap_status gsap_sap_check(gsap_sap* h, void* stream) {
    if (!h) return fail(GSAP_ERR_INVALID, "null handle");
    return finish(h, (cudaStream_t)stream, nullptr, ~0ull);
}

extern "C" gsap_status gsap_sap_scene_axes(gsap_sap* h, uint32_t scene, double* out, void* stream) {
    if (!h || !out) return fail(GSAP_ERR_INVALID, "null argument");
    if (scene >= h->s.max_scenes) return fail(GSAP_ERR_INVALID, "scene index out of range");
    Scene sc;
    CK(cudaMemcpyAsync(&sc, &h->s.scenes[scene], sizeof(Scene), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    CK(cudaStreamSynchronize((cudaStream_t)stream));
    for (int k = 0; k < 9; ++k) out[k] = sc.axes[k];
    for (int k = 0; k < 3; ++k) { out[9 + k] = sc.eig[k]; out[12 + k] = sc.mean[k]; }
    out[15] = sc.G2;
    out[16] = sc.G3;
    return GSAP_OK;
}

// The standalone onesweep sort on a handle's scratch.  flip: the keys are
// floats, sorted through their order-preserving uint32 images (mapped as
// the first pass loads them, mapped back as the last pass stores them).
static gsap_status handle_sort(gsap_sap* h, uint32_t* d_keys, uint32_t* d_vals, uint32_t n, uint32_t bits, int flip,
                               void* stream) {
    if (n > h->s.entry_cap) return fail(GSAP_ERR_CAPACITY, "n = %u exceeds the sort capacity %llu", n, (unsigned long long)h->s.entry_cap);
    if (n < 2) return GSAP_OK;
    cudaStream_t st = (cudaStream_t)stream;
    BpScratch& s = h->s;
    const int passes = (int)((bits + 7) / 8);
    uint32_t* count = &s.ctrl->sort_n;
    CK(launch_sort_prep(s, d_keys, count, n, passes, st, flip));
    uint32_t* vals = d_vals ? d_vals : s.vals[0];
    if (!d_vals) CK(cudaMemsetAsync(vals, 0, 4ull * n, st));
    uint32_t* kb[2] = {d_keys, s.keys[1]};
    uint32_t* vb[2] = {vals, s.vals[1]};
    int src = 0;
    for (int p = 0; p < passes; ++p) {
        const int fmode = flip ? ((p == 0 ? kSortFlipIn : 0) | (p == passes - 1 ? kSortUnflipOut : 0)) : 0;
        CK(launch_sort_pass(s, p, passes, kb[src], vb[src], kb[src ^ 1], vb[src ^ 1], count, n, h->cfg.spin_limit, st,
                            nullptr, false, fmode));
        src ^= 1;
    }
    if (src) {
        CK(cudaMemcpyAsync(d_keys, kb[1], 4ull * n, cudaMemcpyDeviceToDevice, st));
        if (d_vals) CK(cudaMemcpyAsync(d_vals, vb[1], 4ull * n, cudaMemcpyDeviceToDevice, st));
    }
    return finish(h, st, nullptr, ~0ull);
}

extern "C" gsap_status gsap_radix_sort_u32(gsap_sap* h, uint32_t* d_keys, uint32_t* d_vals, uint32_t n,
                                           uint32_t bits, void* stream) {
    if (!h || (!d_keys && n)) return fail(GSAP_ERR_INVALID, "null argument");
    if (bits == 0 || bits > 32) return fail(GSAP_ERR_INVALID, "bits must be in 1..32");
    return handle_sort(h, d_keys, d_vals, n, bits, 0, stream);
}

extern "C" gsap_status gsap_radix_sort_f32(gsap_sap* h, float* d_keys, uint32_t* d_vals, uint32_t n,
                                           uint32_t key_bits, int negative_keys, void* stream) {
    if (!h || (!d_keys && n)) return fail(GSAP_ERR_INVALID, "null argument");
    if (key_bits == 0 || key_bits > 32) return fail(GSAP_ERR_INVALID, "key_bits must be in 1..32");
    if (negative_keys && key_bits != 32)
        return fail(GSAP_ERR_INVALID, "signed float keys are sorted on all 32 bits (key_bits must be 32)");
    return handle_sort(h, reinterpret_cast<uint32_t*>(d_keys), d_vals, n, key_bits, negative_keys ? 1 : 0, stream);
}

// ------------------------------------------------------------ debug hooks

extern "C" int gsap_debug_scene_solve(const double* sums18, const double* hmax3, const double* pilot3, double n,
                                      uint32_t n_total, uint32_t axis_mode, float cell_factor, uint32_t key_bits,
                                      uint64_t entry_cap, double* out17) {
    if (!sums18 || !hmax3 || !pilot3 || !out17) return -1;
    SceneSums z;
    for (int k = 0; k < 3; ++k) {
        z.sd[k] = sums18[k];
        z.sh[k] = sums18[9 + k];
        z.hmax[k] = hmax3[k];
        z.pilot[k] = pilot3[k];
    }
    for (int k = 0; k < 6; ++k) {
        z.sdd[k] = sums18[3 + k];
        z.shh[k] = sums18[12 + k];
    }
    z.n = n;
    BpArgs a;
    memset(&a, 0, sizeof(a));
    a.axis_mode = (int)axis_mode;
    a.cell_factor = cell_factor;
    a.key_bits = key_bits;
    Scene sc;
    memset(&sc, 0, sizeof(sc));
    choose_scene(z, a, entry_cap, n_total, sc);
    for (int k = 0; k < 9; ++k) out17[k] = sc.axes[k];
    for (int k = 0; k < 3; ++k) { out17[9 + k] = sc.eig[k]; out17[12 + k] = sc.mean[k]; }
    out17[15] = sc.G2;
    out17[16] = sc.G3;
    return 0;
}

extern "C" int gsap_debug_stats(gsap_sap* h, uint64_t* out8, void* stream) {
    if (!h || !out8) return -1;
    Ctrl c;
    if (cudaMemcpyAsync(&c, h->s.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, (cudaStream_t)stream) != cudaSuccess) return -1;
    if (cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) return -1;
    out8[0] = c.entry_count;
    out8[1] = c.tests;
    out8[2] = c.pair_count;
    out8[3] = c.total_buckets;
    out8[4] = c.qbits;
    out8[5] = c.long_rows;
    out8[6] = c.iters;
    out8[7] = c.error;
    return 0;
}

// One thread waits on look-back words that nothing publishes (slot 7 is
// used by no pass), with the pipeline's bounded wait.
__global__ void k_debug_lookback(BpScratch S, uint32_t spin_limit) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const uint32_t tag = (S.ctrl->epoch << 3) | 7u;
    (void)lookback(S.status, 1, 0, 1, tag, spin_limit, &S.ctrl->error);
}

extern "C" int gsap_debug_lookback_timeout(gsap_sap* h, uint32_t spin_limit, void* stream) {
    if (!h) return fail(GSAP_ERR_INVALID, "null handle");
    cudaStream_t st = (cudaStream_t)stream;
    k_debug_lookback<<<1, 32, 0, st>>>(h->s, spin_limit);
    CK(cudaGetLastError());
    return finish(h, st, nullptr, ~0ull);
}

extern "C" int gsap_debug_graph_cache(gsap_sap* h, uint32_t per_shape, uint32_t* out_count) {
    if (!h) return -1;
    if (per_shape) h->per_shape = per_shape;
    if (out_count) *out_count = (uint32_t)h->graphs->size();
    return 0;
}

extern "C" int gsap_debug_sizes(uint32_t* out) {
    if (!out) return -1;
    out[0] = sizeof(Ctrl);
    out[1] = sizeof(Scene);
    out[2] = sizeof(PcaPartial);
    out[3] = kSortTile;
    return 0;
}

gsap_status gsap::bp_both_async(gsap_sap* h, int mode, const float4* mn, const float4* mx, const uint32_t* off,
                                uint32_t S, uint32_t n, uint2* pairs, uint64_t cap, int32_t* entries,
                                uint64_t entry_cap, cudaStream_t st, BpDeviceCounts* out, uint32_t flags) {
    gsap_status v = validate(h, (const float*)mn, (const float*)mx, n, mode, pairs, off ? S : 1);
    if (v != GSAP_OK) return v;
    if (out) {
        out->num_pairs = &h->s.ctrl->pair_count;
        out->num_entries = &h->s.ctrl->scan_total;
        out->rowoff = h->s.rowoff;
    }
    Call c;
    memset(&c, 0, sizeof(c));
    c.mn = mn;
    c.mx = mode == GSAP_MODE_AABB ? mx : nullptr;
    c.off = off;
    c.n = n;
    c.S = off ? S : 1;
    c.mode = mode;
    c.pairs = pairs;
    c.cap = cap;
    c.entries = entries;
    c.ecap = entry_cap;
    c.both = 1;
    c.flags = flags & GSAP_FLAG_TEMPORAL;
    temporal_resolve(h, c);
    if (n < 2 && !off) {
        // empty list: zero the counts and row offsets the consumers read
        CK(cudaMemsetAsync(&h->s.ctrl->pair_count, 0, 8, st));
        CK(cudaMemsetAsync(&h->s.ctrl->scan_total, 0, 4, st));
        CK(cudaMemsetAsync(h->s.rowoff, 0, 4ull * (n + 1), st));
        return GSAP_OK;
    }
    // with timing enabled the stages of this call are timed too (a step
    // that is not graph-captured; gsap_sap_stage_times reads them)
    gsap_status r = record(h, c, st, h->timing);
    if (r == GSAP_OK) temporal_note(h, c);
    return r;
}
