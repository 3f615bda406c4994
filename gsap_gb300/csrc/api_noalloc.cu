// gsap_radix_sort_u32_noalloc: the onesweep radix sort on scratch that lives
// in a file-scope device array instead of a handle's allocations.
//
// Who needs it: callers that may not allocate device memory at the point
// where they sort -- a custom allocator or memory pool that owns every byte
// of the device (cudaMalloc would bypass it or fail), a stream-ordered
// section where an allocation would synchronise the device, or a plugin that
// is handed only its input buffers and a stream.  gsap_radix_sort_u32 needs
// a gsap_sap handle, whose creation allocates; this entry point needs none.
//
// What it does not do: it makes no cudaMalloc/cudaFree call and calls no
// library that allocates (no torch, no CUB).  Its scratch is one
// `static __device__` array of fixed size, so n is capped at
// GSAP_NOALLOC_SORT_MAX_N; larger n is rejected before anything runs.  The
// array is shared by every caller on a device, so two calls that overlap in
// time (two streams, two host threads) race and corrupt each other's output.
//
// Set-up: the first call on each device looks the array up with
// cudaGetSymbolAddress and zeroes its control block and look-back words
// (synchronously).  Later calls look the address up again (this allocates nothing); a failed
// set-up is not remembered, so the next call retries it, and an address
// that changed (the module was loaded again after cudaDeviceReset) gets a
// fresh set-up.
//
// Pointers: the keys and values must be device memory of the current
// device; memory of another device, or host memory CUDA does not know,
// is rejected with GSAP_ERR_INVALID before anything runs.
//
// What must start at zero: the control block (error word, tile counters,
// digit histograms, epoch) and the look-back words.  Set-up zeroes them;
// afterwards each call resets the counters and histograms itself
// (k_sort_reset) and starts a new epoch, so look-back words left by earlier
// calls never match the current tag.  The key/value halves of the scratch
// need no initial value.
#include <cstdio>
#include <mutex>

#include "../../include/gsap.h"
#include "api_internal.h"
#include "internal.cuh"

using namespace gsap;

namespace {

constexpr uint64_t kAlign = 256;
constexpr uint64_t up(uint64_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

constexpr uint32_t kMaxN = GSAP_NOALLOC_SORT_MAX_N;
constexpr uint64_t kTiles = (kMaxN + kSortTile - 1) / kSortTile + 1;
// byte offsets of the regions inside the array
constexpr uint64_t kOffCtrl = 0;
constexpr uint64_t kOffStatus = up(sizeof(Ctrl));
constexpr uint64_t kZeroBytes = kOffStatus + up(8ull * kTiles * 256ull);  // what must start at zero
constexpr uint64_t kOffKeys = kZeroBytes;                                  // ping-pong key buffer
constexpr uint64_t kOffVals = kOffKeys + up(4ull * kMaxN);                 // ping-pong value buffer
constexpr uint64_t kOffVals0 = kOffVals + up(4ull * kMaxN);                // values when the caller has none
constexpr uint64_t kBytes = kOffVals0 + up(4ull * kMaxN);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kBytes];

struct Slot {
    std::mutex mu;
    unsigned char* base = nullptr;  // set only once a set-up succeeded for this address
};
Slot g_slots[kMaxDevices];

// The array's device address on device `dev` (current), set up on first use.
cudaError_t scratch_base(int dev, unsigned char** out) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    Slot& slot = g_slots[dev];
    std::lock_guard<std::mutex> lock(slot.mu);
    if (slot.base != (unsigned char*)p) {
        slot.base = nullptr;
        e = cudaMemset(p, 0, kZeroBytes);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return e;
        slot.base = (unsigned char*)p;
    }
    *out = slot.base;
    return cudaSuccess;
}

// GSAP_OK when p is device (or managed) memory usable on device `dev`.
gsap_status check_ptr(const void* p, int dev, const char* what) {
    if (!p) return GSAP_OK;
    cudaPointerAttributes a;
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    char buf[192];
    if (e != cudaSuccess) {
        cudaGetLastError();
        snprintf(buf, sizeof(buf), "gsap_radix_sort_u32_noalloc: %s is not a CUDA pointer (%s)", what,
                 cudaGetErrorString(e));
        return set_error(GSAP_ERR_INVALID, buf);
    }
    if (a.type == cudaMemoryTypeUnregistered) {
        snprintf(buf, sizeof(buf), "gsap_radix_sort_u32_noalloc: %s is host memory unknown to CUDA", what);
        return set_error(GSAP_ERR_INVALID, buf);
    }
    if (a.type == cudaMemoryTypeDevice && a.device != dev) {
        snprintf(buf, sizeof(buf), "gsap_radix_sort_u32_noalloc: %s is on device %d, the current device is %d", what,
                 a.device, dev);
        return set_error(GSAP_ERR_INVALID, buf);
    }
    return GSAP_OK;
}

gsap_status cuda_fail(cudaError_t e, const char* what) {
    char buf[256];
    snprintf(buf, sizeof(buf), "gsap_radix_sort_u32_noalloc: %s: %s", what, cudaGetErrorString(e));
    return set_error(GSAP_ERR_CUDA, buf);
}

}  // namespace

extern "C" gsap_status gsap_radix_sort_u32_noalloc(uint32_t* d_keys, uint32_t* d_vals, uint32_t n, uint32_t bits,
                                                   void* stream) {
    if (n > kMaxN) {
        char buf[160];
        snprintf(buf, sizeof(buf), "gsap_radix_sort_u32_noalloc: n = %u exceeds its fixed scratch (at most %u keys)", n,
                 kMaxN);
        return set_error(GSAP_ERR_CAPACITY, buf);
    }
    if (!d_keys && n) return set_error(GSAP_ERR_INVALID, "gsap_radix_sort_u32_noalloc: null keys");
    if (bits == 0 || bits > 32) return set_error(GSAP_ERR_INVALID, "gsap_radix_sort_u32_noalloc: bits must be in 1..32");
    if (n < 2) return GSAP_OK;

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return set_error(GSAP_ERR_INVALID, "gsap_radix_sort_u32_noalloc: device ordinal out of range");
    gsap_status pc = check_ptr(d_keys, dev, "keys");
    if (pc == GSAP_OK) pc = check_ptr(d_vals, dev, "values");
    if (pc != GSAP_OK) return pc;
    unsigned char* base = nullptr;
    e = scratch_base(dev, &base);
    if (e != cudaSuccess) return cuda_fail(e, "set-up of the static scratch");

    BpScratch s{};
    s.ctrl = (Ctrl*)(base + kOffCtrl);
    s.status = (uint64_t*)(base + kOffStatus);
    s.status_words = kTiles * 256ull;
    s.entry_cap = kMaxN;
    s.max_n = kMaxN;
    uint32_t* keys_alt = (uint32_t*)(base + kOffKeys);
    uint32_t* vals_alt = (uint32_t*)(base + kOffVals);
    uint32_t* vals0 = (uint32_t*)(base + kOffVals0);

    cudaStream_t st = (cudaStream_t)stream;
    const int passes = (int)((bits + 7) / 8);
    uint32_t* count = &s.ctrl->sort_n;
#define NA_CK(x)                                   \
    do {                                           \
        cudaError_t e_ = (x);                      \
        if (e_ != cudaSuccess) return cuda_fail(e_, #x); \
    } while (0)
    NA_CK(launch_sort_prep(s, d_keys, count, n, passes, st));
    uint32_t* vals = d_vals ? d_vals : vals0;
    if (!d_vals) NA_CK(cudaMemsetAsync(vals0, 0, 4ull * n, st));
    uint32_t* kb[2] = {d_keys, keys_alt};
    uint32_t* vb[2] = {vals, vals_alt};
    int src = 0;
    for (int p = 0; p < passes; ++p) {
        NA_CK(launch_sort_pass(s, p, passes, kb[src], vb[src], kb[src ^ 1], vb[src ^ 1], count, n, kDefaultSpin, st));
        src ^= 1;
    }
    if (src) {
        NA_CK(cudaMemcpyAsync(d_keys, keys_alt, 4ull * n, cudaMemcpyDeviceToDevice, st));
        if (d_vals) NA_CK(cudaMemcpyAsync(d_vals, vals_alt, 4ull * n, cudaMemcpyDeviceToDevice, st));
    }
    // the device error word (pageable host target: no host allocation either)
    uint32_t err = 0;
    NA_CK(cudaMemcpyAsync(&err, &s.ctrl->error, 4, cudaMemcpyDeviceToHost, st));
    NA_CK(cudaStreamSynchronize(st));
    if (err) {
        NA_CK(cudaMemsetAsync(&s.ctrl->error, 0, 4, st));
        NA_CK(cudaStreamSynchronize(st));
        if (err & kErrTimeout)
            return set_error(GSAP_ERR_DEVICE_TIMEOUT, "gsap_radix_sort_u32_noalloc: a device-side wait exceeded its iteration cap");
        char buf[128];
        snprintf(buf, sizeof(buf), "gsap_radix_sort_u32_noalloc: device error word 0x%x", err);
        return set_error(GSAP_ERR_CUDA, buf);
    }
#undef NA_CK
    return GSAP_OK;
}
