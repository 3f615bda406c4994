// C++-only entry points shared between the broadphase and rigid-body C-ABI
// layers.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include "../../include/gsap.h"

namespace gsap {

// NVTX ranges for profilers (host-side enqueue of each stage; header-only,
// no cost without an attached tool).  A range opened here is closed by the
// next stage or when the object goes out of scope (error returns included).
struct NvtxRange {
    int open = 0;
    NvtxRange() = default;
    explicit NvtxRange(const char* name) { next(name); }
    void next(const char* name) {
        if (open) nvtxRangePop();
        nvtxRangePushA(name);
        open = 1;
    }
    ~NvtxRange() {
        if (open) nvtxRangePop();
    }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

struct BpDeviceCounts {
    const unsigned long long* num_pairs;  // i<j pairs of the last call (device)
    const uint32_t* num_entries;          // pairEntries count (device, both-direction format)
    const uint32_t* rowoff;               // per-object row offsets of the both-direction list (n+1)
};

// Both-direction canonical pair list (Sap::collision format, any predicate)
// without any host synchronisation: the counts stay on the device.  flags
// may hold GSAP_FLAG_TEMPORAL (the step-to-step callers of the rigid body).
gsap_status bp_both_async(gsap_sap* h, int mode, const float4* mn, const float4* mx, const uint32_t* scene_off,
                          uint32_t num_scenes, uint32_t n, uint2* pairs, uint64_t cap, int32_t* entries,
                          uint64_t entry_cap, cudaStream_t st, BpDeviceCounts* out, uint32_t flags = 0);

gsap_status set_error(gsap_status st, const char* msg);

}  // namespace gsap
