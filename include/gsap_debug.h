/*
 * gsap_debug.h -- test hooks of libgsap.so that run on the host (no GPU).
 * No counterpart in the reference: they expose internals of this
 * implementation so that the CPU test suite can check them.
 */
#ifndef GSAP_DEBUG_H
#define GSAP_DEBUG_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Host build of the FP64 per-scene solver that the PCA kernel runs in its
 * last CTA: sums18 = (sum d[3], sum d d^T[6: xx xy xz yy yz zz], sum h[3],
 * sum h h^T[6]) with d = centre - pilot, hmax3, pilot3, n objects of a scene
 * in a call of n_total objects.  out17 = axes u1,u2,u3 (rows), eigenvalues,
 * mean, G2, G3.  Returns 0 on success. */
int gsap_debug_scene_solve(const double* sums18, const double* hmax3, const double* pilot3, double n,
                           uint32_t n_total, uint32_t axis_mode, float cell_factor, uint32_t key_bits,
                           uint64_t entry_cap, double* out17);

/* Counters of the last broadphase call of a handle (synchronizes):
 * out8 = sweep entries, candidate tests, pairs, buckets, q bits, long rows
 * of the canonical sort, warp iterations of the sweep loop, device error
 * word.  Returns 0. */
struct gsap_sap;
int gsap_debug_stats(struct gsap_sap* h, uint64_t* out8, void* stream);

/* Failure-path check of the bounded device waits (needs a GPU): one thread
 * runs the radix look-back on a tile whose predecessor never publishes (a
 * tag no pass uses), so the wait gives up after spin_limit polls, sets the
 * timeout bit of the handle's error word and returns.  The call then reads
 * and clears the error word like any broadphase call: it returns
 * GSAP_ERR_DEVICE_TIMEOUT and leaves the handle and the context usable. */
int gsap_debug_lookback_timeout(struct gsap_sap* h, uint32_t spin_limit, void* stream);

/* Particle-particle contacts found by the config-model force kernel since
 * the handle was created or last reset (each contact counted from both
 * particles, so the contact pairs are *out / 2; walls not counted).  The
 * kernel adds one warp-aggregated count per warp of every step.  Reads the
 * counter (synchronizes) and zeroes it when reset != 0.  Returns 0. */
struct gsap_rb;
int gsap_debug_rb_contacts(struct gsap_rb* h, uint64_t* out, int reset, void* stream);

/* Graph cache of a broadphase handle: per_shape != 0 sets how many cached
 * graphs of one shape (sizes, flags, settings) the handle keeps before a
 * call with new buffers updates one of them in place (default 64);
 * *out_count (may be NULL) receives the number of cached graphs.
 * Returns 0. */
int gsap_debug_graph_cache(struct gsap_sap* h, uint32_t per_shape, uint32_t* out_count);

/* Sizes of internal device structures (control block, scene record, PCA
 * partial, sort tile) for layout checks.  Returns 0. */
int gsap_debug_sizes(uint32_t* out4);

#ifdef __cplusplus
}
#endif
#endif
