/*
 * CPU oracle, broadphase half.  TEST INFRASTRUCTURE ONLY (see oracle.h): the
 * checker for libgsap.so, never part of the product path.
 *
 * Compiled with -O2 -ffp-contract=off (and OpenMP when available): every
 * float expression is evaluated in source order with one rounding per
 * operation, which is how the GPU kernels evaluate the same predicates.
 */
#include "oracle.h"
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int nthreads(int t) {
#ifdef _OPENMP
    return t > 0 ? t : omp_get_max_threads();
#else
    (void)t;
    return 1;
#endif
}

/* Wall-clock seconds (process CPU time in a build without OpenMP, where
 * it is the same thing). */
static double wall(void) {
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return (double)clock() / CLOCKS_PER_SEC;
#endif
}

/* Aabb::overlaps (include/aabb.h:47-57): closed on all six faces. */
static inline int aabb_overlap(const float* ai, const float* xi,
                               const float* aj, const float* xj) {
    return ai[0] <= xj[0] && aj[0] <= xi[0] &&
           ai[1] <= xj[1] && aj[1] <= xi[1] &&
           ai[2] <= xj[2] && aj[2] <= xi[2];
}

/* Squared strict sphere test of kernel_SphereTexCullPCAElong
 * (sapDetection/SapKernel.cu:1897-1903): x0 = ci - cj per axis,
 * t1 = x0*x0 + y0*y0 + z0*z0 (left to right), e1 = (ri + rj)^2, t1 < e1. */
static inline int sphere_overlap(const float* a, const float* b) {
    float dx = a[0] - b[0];
    float dy = a[1] - b[1];
    float dz = a[2] - b[2];
    float r = a[3] + b[3];
    float t1 = dx * dx + dy * dy + dz * dz;
    float e1 = r * r;
    return t1 < e1;
}

typedef int (*pair_pred)(const float*, const float*, uint32_t, uint32_t);

static int pred_aabb_ix(const float* mn, const float* mx, uint32_t i, uint32_t j) {
    return aabb_overlap(mn + 4 * (size_t)i, mx + 4 * (size_t)i, mn + 4 * (size_t)j, mx + 4 * (size_t)j);
}
static int pred_sphere_ix(const float* s, const float* unused, uint32_t i, uint32_t j) {
    (void)unused;
    return sphere_overlap(s + 4 * (size_t)i, s + 4 * (size_t)j);
}

/* Row-major brute force: count per row, prefix, fill.  Two passes keep the
 * output in (i, j) order without per-thread buffers. */
static int64_t brute_force(const float* a, const float* b, uint32_t n,
                           uint32_t* pairs, int64_t cap, int threads,
                           int (*pred)(const float*, const float*, uint32_t, uint32_t)) {
    if (n < 2) return 0;
    int64_t* rowc = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
    int nt = nthreads(threads);
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        int64_t c = 0;
        for (uint32_t j = (uint32_t)i + 1; j < n; ++j) c += pred(a, b, (uint32_t)i, j);
        rowc[i + 1] = c;
    }
    for (uint32_t i = 0; i < n; ++i) rowc[i + 1] += rowc[i];
    int64_t total = rowc[n];
    if (pairs) {
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
        for (int64_t i = 0; i < (int64_t)n; ++i) {
            int64_t o = rowc[i];
            if (o >= cap) continue;
            for (uint32_t j = (uint32_t)i + 1; j < n && o < cap; ++j) {
                if (pred(a, b, (uint32_t)i, j)) {
                    pairs[2 * o] = (uint32_t)i;
                    pairs[2 * o + 1] = j;
                    ++o;
                }
            }
        }
    }
    free(rowc);
    return total;
}

int64_t orc_bf_aabb(const float* mn, const float* mx, uint32_t n,
                    uint32_t* pairs, int64_t cap, int threads) {
    return brute_force(mn, mx, n, pairs, cap, threads, pred_aabb_ix);
}

int64_t orc_bf_sphere(const float* spheres, uint32_t n,
                      uint32_t* pairs, int64_t cap, int threads) {
    return brute_force(spheres, NULL, n, pairs, cap, threads, pred_sphere_ix);
}

/* ------------------------------------------------------------ radix sort */

uint32_t orc_float_flip(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    uint32_t mask = (u & 0x80000000u) ? 0xFFFFFFFFu : 0x80000000u;
    return u ^ mask;
}

void orc_radix_sort_u32(uint32_t* keys, uint32_t* vals, uint32_t n, int bits) {
    if (n < 2 || bits <= 0) return;
    uint32_t* k2 = (uint32_t*)malloc((size_t)n * 4);
    uint32_t* v2 = (uint32_t*)malloc((size_t)n * 4);
    uint32_t *ks = keys, *vs = vals, *kd = k2, *vd = v2;
    for (int shift = 0; shift < bits; shift += 8) {
        size_t cnt[257];
        memset(cnt, 0, sizeof(cnt));
        uint32_t mask = (bits - shift >= 8) ? 0xFFu : ((1u << (bits - shift)) - 1u);
        for (uint32_t i = 0; i < n; ++i) cnt[((ks[i] >> shift) & mask) + 1]++;
        for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
        for (uint32_t i = 0; i < n; ++i) {
            size_t p = cnt[(ks[i] >> shift) & mask]++;
            kd[p] = ks[i];
            if (vals) vd[p] = vs[i];
        }
        uint32_t* t = ks; ks = kd; kd = t;
        t = vs; vs = vd; vd = t;
    }
    if (ks != keys) {
        memcpy(keys, ks, (size_t)n * 4);
        if (vals) memcpy(vals, vs, (size_t)n * 4);
    }
    free(k2);
    free(v2);
}

/* Parallel stable LSD radix sort (8-bit digits) of u32 keys with u32
 * values or of u64 keys, for the CPU baseline: per pass every thread counts
 * the digits of its contiguous chunk, an exclusive scan in (digit, thread)
 * order gives each thread its output offsets, and the threads scatter their
 * chunks in input order, so equal digits keep their order (stable). */
#define PR_MAXT 256
static void par_radix_u32(uint32_t* keys, uint32_t* vals, size_t n, int bits, int nt) {
    if (n < 2 || bits <= 0) return;
    if (nt > PR_MAXT) nt = PR_MAXT;
    if (n < 65536) nt = 1;
    uint32_t* k2 = (uint32_t*)malloc(n * 4);
    uint32_t* v2 = vals ? (uint32_t*)malloc(n * 4) : NULL;
    size_t(*cnt)[256] = (size_t(*)[256])malloc((size_t)nt * sizeof(*cnt));
    uint32_t *ks = keys, *vs = vals, *kd = k2, *vd = v2;
    for (int shift = 0; shift < bits; shift += 8) {
#pragma omp parallel num_threads(nt)
        {
#ifdef _OPENMP
            const int t = omp_get_thread_num();
#else
            const int t = 0;
#endif
            const size_t a = n * (size_t)t / (size_t)nt, b = n * (size_t)(t + 1) / (size_t)nt;
            size_t* c = cnt[t];
            memset(c, 0, sizeof(*cnt));
            for (size_t i = a; i < b; ++i) c[(ks[i] >> shift) & 0xFFu]++;
#pragma omp barrier
#pragma omp single
            {
                size_t run = 0;
                for (int d = 0; d < 256; ++d)
                    for (int u = 0; u < nt; ++u) {
                        size_t x = cnt[u][d];
                        cnt[u][d] = run;
                        run += x;
                    }
            }
            for (size_t i = a; i < b; ++i) {
                size_t p = c[(ks[i] >> shift) & 0xFFu]++;
                kd[p] = ks[i];
                if (vs) vd[p] = vs[i];
            }
        }
        uint32_t* x = ks; ks = kd; kd = x;
        x = vs; vs = vd; vd = x;
    }
    if (ks != keys) {
        memcpy(keys, ks, n * 4);
        if (vals) memcpy(vals, vs, n * 4);
    }
    free(cnt);
    free(k2);
    free(v2);
}

static void par_radix_u64(uint64_t* keys, size_t n, int bits, int nt) {
    if (n < 2) return;
    if (nt > PR_MAXT) nt = PR_MAXT;
    if (n < 65536) nt = 1;
    uint64_t* tmp = (uint64_t*)malloc(n * 8);
    size_t(*cnt)[256] = (size_t(*)[256])malloc((size_t)nt * sizeof(*cnt));
    uint64_t *s = keys, *d = tmp;
    for (int shift = 0; shift < bits; shift += 8) {
#pragma omp parallel num_threads(nt)
        {
#ifdef _OPENMP
            const int t = omp_get_thread_num();
#else
            const int t = 0;
#endif
            const size_t a = n * (size_t)t / (size_t)nt, b = n * (size_t)(t + 1) / (size_t)nt;
            size_t* c = cnt[t];
            memset(c, 0, sizeof(*cnt));
            for (size_t i = a; i < b; ++i) c[(s[i] >> shift) & 0xFF]++;
#pragma omp barrier
#pragma omp single
            {
                size_t run = 0;
                for (int q = 0; q < 256; ++q)
                    for (int u = 0; u < nt; ++u) {
                        size_t x = cnt[u][q];
                        cnt[u][q] = run;
                        run += x;
                    }
            }
            for (size_t i = a; i < b; ++i) d[c[(s[i] >> shift) & 0xFF]++] = s[i];
        }
        uint64_t* x = s; s = d; d = x;
    }
    if (s != keys) memcpy(keys, s, n * 8);
    free(cnt);
    free(tmp);
}

/* ------------------------------------------------------ reference SaP (CPU) */

typedef struct pvec { uint64_t* p; size_t n, cap; } pvec;
static void pv_push(pvec* v, uint64_t x) {
    if (v->n == v->cap) {
        v->cap = v->cap ? v->cap * 2 : 1024;
        v->p = (uint64_t*)realloc(v->p, v->cap * 8);
    }
    v->p[v->n++] = x;
}

/* Sweep one group of objects (ids[0..m)) along axis `ax`: sort by the lower
 * end of the projected interval (the flipped-float radix sort of
 * radixsort.cu), then scan forward while lo_j <= hi_i
 * (SapKernel.cu:1880-1913: break once d_pos[cur] > d_pos[i] + 2r). */
static void sweep_group(int mode, const float* mn, const float* mx, int ax,
                        uint32_t* ids, uint32_t m, pvec* out, int nt, uint32_t parts,
                        uint32_t part, double* t_sweep) {
    if (m < 2) return;
    uint32_t* keys = (uint32_t*)malloc((size_t)m * 4);
    float* lo = (float*)malloc((size_t)m * 4);
    float* hi = (float*)malloc((size_t)m * 4);
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t k = 0; k < (int64_t)m; ++k) {
        uint32_t i = ids[k];
        float l;
        if (mode == 0) {
            l = mn[4 * (size_t)i + ax];
        } else {
            float c = mn[4 * (size_t)i + ax], r = mn[4 * (size_t)i + 3];
            l = c - r;
        }
        keys[k] = orc_float_flip(l);
    }
    par_radix_u32(keys, ids, m, 32, nt);
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t k = 0; k < (int64_t)m; ++k) {
        uint32_t i = ids[k];
        if (mode == 0) {
            lo[k] = mn[4 * (size_t)i + ax];
            hi[k] = mx[4 * (size_t)i + ax];
        } else {
            float c = mn[4 * (size_t)i + ax], r = mn[4 * (size_t)i + 3];
            lo[k] = c - r;
            hi[k] = c + r;
        }
    }
    /* sweep starts: slice `part` of `parts` equal slices of the sorted
     * order (the whole order when parts == 1) */
    const int64_t a0 = (int64_t)((uint64_t)m * part / parts);
    const int64_t a1 = (int64_t)((uint64_t)m * (part + 1) / parts);
    double t0 = wall();
#pragma omp parallel num_threads(nt)
    {
        pvec local = {0, 0, 0};
#pragma omp for schedule(dynamic, 64)
        for (int64_t a = a0; a < a1; ++a) {
            uint32_t i = ids[a];
            float h = hi[a];
            for (uint32_t b = (uint32_t)a + 1; b < m && lo[b] <= h; ++b) {
                uint32_t j = ids[b];
                int hit = mode == 0 ? pred_aabb_ix(mn, mx, i, j) : pred_sphere_ix(mn, NULL, i, j);
                if (hit) {
                    uint32_t x = i < j ? i : j, y = i < j ? j : i;
                    pv_push(&local, ((uint64_t)x << 32) | y);
                }
            }
        }
#pragma omp critical
        {
            for (size_t q = 0; q < local.n; ++q) pv_push(out, local.p[q]);
        }
        free(local.p);
    }
    *t_sweep += wall() - t0;
    free(keys);
    free(lo);
    free(hi);
}

int64_t orc_sap_ref(int mode, const float* mn, const float* mx, uint32_t n,
                    uint32_t* pairs, int64_t cap, int threads) {
    return orc_sap_ref_sampled(mode, mn, mx, n, 1, 0, pairs, cap, threads, NULL);
}

int64_t orc_sap_ref_sampled(int mode, const float* mn, const float* mx, uint32_t n, uint32_t parts,
                            uint32_t part, uint32_t* pairs, int64_t cap, int threads, double* secs) {
    double t_start = wall(), t_var = 0.0;
    if (secs) secs[0] = secs[1] = 0.0;
    if (n < 2) return 0;
    if (parts == 0) parts = 1;
    part %= parts;
    int nt = nthreads(threads);
    /* centres: sphere xyz, or AABB midpoints */
    double mean[3] = {0, 0, 0}, var[3] = {0, 0, 0};
    float* cen = (float*)malloc((size_t)n * 12);
#pragma omp parallel for schedule(static) num_threads(nt) reduction(+ : mean[:3])
    for (int64_t i = 0; i < (int64_t)n; ++i)
        for (int k = 0; k < 3; ++k) {
            float c = mode == 0 ? 0.5f * (mn[4 * (size_t)i + k] + mx[4 * (size_t)i + k])
                                : mn[4 * (size_t)i + k];
            cen[3 * (size_t)i + k] = c;
            mean[k] += c;
        }
    for (int k = 0; k < 3; ++k) mean[k] /= n;
#pragma omp parallel for schedule(static) num_threads(nt) reduction(+ : var[:3])
    for (int64_t i = 0; i < (int64_t)n; ++i)
        for (int k = 0; k < 3; ++k) {
            double d = cen[3 * (size_t)i + k] - mean[k];
            var[k] += d * d;
        }
    /* axisVecMultiple (SapKernel.cu:63-97): argmax of the covariance
     * diagonal with the reference's tie order, secondary axes fixed. */
    int axis = var[0] >= var[1] ? 0 : 1;
    if (axis) axis = var[1] >= var[2] ? 1 : 2;
    else axis = var[0] >= var[2] ? 0 : 2;
    int a1 = axis == 0 ? 1 : 0;
    int a2 = 3 - axis - a1;

    /* projectSubMultiple (SapKernel.cu:151-213): quadrant of the centre on
     * the two secondary axes about the origin (mPoint1 = mPoint2 = 0). */
    uint32_t* grp[4];
    uint32_t gn[4] = {0, 0, 0, 0};
    for (int q = 0; q < 4; ++q) grp[q] = (uint32_t*)malloc((size_t)n * 4);
    for (uint32_t i = 0; i < n; ++i) {
        float y = cen[3 * (size_t)i + a1], z = cen[3 * (size_t)i + a2];
        int q = (y >= 0.f && z >= 0.f) ? 1 : (y < 0.f && z >= 0.f) ? 2 : (y >= 0.f && z < 0.f) ? 3 : 0;
        grp[q][gn[q]++] = i;
    }
    pvec all = {0, 0, 0};
    for (int q = 0; q < 4; ++q) sweep_group(mode, mn, mx, axis, grp[q], gn[q], &all, nt, parts, part, &t_var);

    /* Cross pass (cullCrossSphereMultiple :557-635, cullRelevantSphereMultiple
     * :968-1059): maxR over objects straddling a plane, then every object
     * within maxR of either plane is swept again without the quadrant key.
     * For AABBs maxR is the largest secondary-axis width of a straddler. */
    float maxR = 0.f;
    for (uint32_t i = 0; i < n; ++i) {
        float r, l1, h1, l2, h2;
        if (mode == 0) {
            l1 = mn[4 * (size_t)i + a1]; h1 = mx[4 * (size_t)i + a1];
            l2 = mn[4 * (size_t)i + a2]; h2 = mx[4 * (size_t)i + a2];
            float w1 = h1 - l1, w2 = h2 - l2;
            r = w1 > w2 ? w1 : w2;
        } else {
            r = mn[4 * (size_t)i + 3];
            float y = mn[4 * (size_t)i + a1], z = mn[4 * (size_t)i + a2];
            l1 = y - r; h1 = y + r; l2 = z - r; h2 = z + r;
        }
        if ((h1 >= 0.f && l1 <= 0.f) || (h2 >= 0.f && l2 <= 0.f))
            if (r > maxR) maxR = r;
    }
    uint32_t rn = 0;
    for (uint32_t i = 0; i < n; ++i) {
        float l1, h1, l2, h2;
        if (mode == 0) {
            l1 = mn[4 * (size_t)i + a1]; h1 = mx[4 * (size_t)i + a1];
            l2 = mn[4 * (size_t)i + a2]; h2 = mx[4 * (size_t)i + a2];
        } else {
            float r = mn[4 * (size_t)i + 3];
            float y = mn[4 * (size_t)i + a1], z = mn[4 * (size_t)i + a2];
            l1 = y - r; h1 = y + r; l2 = z - r; h2 = z + r;
        }
        if ((h1 >= -maxR && l1 <= maxR) || (h2 >= -maxR && l2 <= maxR)) grp[0][rn++] = i;
    }
    if (rn > 0 && rn < n) sweep_group(mode, mn, mx, axis, grp[0], rn, &all, nt, parts, part, &t_var);
    else if (rn == n) { /* every object is relevant: the quadrant sweeps are
                           not enough, sweep them all together */
        for (uint32_t i = 0; i < n; ++i) grp[0][i] = i;
        sweep_group(mode, mn, mx, axis, grp[0], n, &all, nt, parts, part, &t_var);
    }

    /* Canonicalise: sort + unique (Sap.cpp:269-291, cullIndex :2249-2265). */
    double t_canon = wall();
    int idbits = 1;
    while (idbits < 32 && ((uint64_t)1 << idbits) < n) ++idbits;
    par_radix_u64(all.p, all.n, 32 + ((idbits + 7) / 8) * 8, nt);
    /* unique: per-chunk counts of first occurrences, prefix, then write */
    int64_t u = 0;
    {
        int ct = nt > PR_MAXT ? PR_MAXT : nt;
        if (all.n < 65536) ct = 1;
        int64_t cu[PR_MAXT + 1];
        memset(cu, 0, sizeof(cu));
#pragma omp parallel num_threads(ct)
        {
#ifdef _OPENMP
            const int t = omp_get_thread_num();
#else
            const int t = 0;
#endif
            const size_t a = all.n * (size_t)t / (size_t)ct, b = all.n * (size_t)(t + 1) / (size_t)ct;
            int64_t c = 0;
            for (size_t k = a; k < b; ++k) c += (k == 0 || all.p[k] != all.p[k - 1]);
            cu[t + 1] = c;
#pragma omp barrier
#pragma omp single
            for (int q = 0; q < ct; ++q) cu[q + 1] += cu[q];
            int64_t o = cu[t];
            for (size_t k = a; k < b; ++k) {
                if (k > 0 && all.p[k] == all.p[k - 1]) continue;
                if (pairs && o < cap) {
                    pairs[2 * o] = (uint32_t)(all.p[k] >> 32);
                    pairs[2 * o + 1] = (uint32_t)all.p[k];
                }
                ++o;
            }
        }
        u = cu[ct];
    }
    t_var += wall() - t_canon;
    for (int q = 0; q < 4; ++q) free(grp[q]);
    free(cen);
    free(all.p);
    if (secs) {
        secs[1] = t_var;
        secs[0] = wall() - t_start - t_var;
    }
    return u;
}

int64_t orc_both_directions(const uint32_t* pairs, int64_t np,
                            int32_t* out_pairs, int32_t* out_entries) {
    if (np <= 0) return 0;
    uint32_t maxid = 0;
    for (int64_t k = 0; k < 2 * np; ++k) if (pairs[k] > maxid) maxid = pairs[k];
    size_t m = (size_t)maxid + 1;
    int64_t* off = (int64_t*)calloc(m + 1, sizeof(int64_t));
    for (int64_t k = 0; k < np; ++k) {
        off[pairs[2 * k] + 1]++;
        off[pairs[2 * k + 1] + 1]++;
    }
    int64_t ne = 0;
    for (size_t a = 0; a < m; ++a) {
        if (off[a + 1] > 0 && out_entries) out_entries[ne] = (int32_t)off[a];
        if (off[a + 1] > 0) ++ne;
        off[a + 1] += off[a];
    }
    /* stable fill in list order: rows come out sorted by second id */
    int64_t* cur = (int64_t*)malloc(m * sizeof(int64_t));
    memcpy(cur, off, m * sizeof(int64_t));
    if (out_pairs) {
        for (int64_t k = 0; k < np; ++k) {
            uint32_t i = pairs[2 * k], j = pairs[2 * k + 1];
            int64_t p = cur[i]++;
            out_pairs[2 * p] = (int32_t)i;
            out_pairs[2 * p + 1] = (int32_t)j;
            p = cur[j]++;
            out_pairs[2 * p] = (int32_t)j;
            out_pairs[2 * p + 1] = (int32_t)i;
        }
    }
    free(cur);
    free(off);
    return ne;
}

/* ------------------------------------------------------- batched scenes */

static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return (x > y) - (x < y);
}

/* Pairs of one scene [b, e) of a batch: every i < j of the scene with
 * Aabb::overlaps (include/aabb.h:47-57), as keys (i << 32) | j in ascending
 * order.  Scenes of at most bf_max objects test all pairs (the reference's
 * Demo::cpuBroadphase loop, cudaPhysics/demo.h:404-417); larger ones test
 * the same predicate on every pair whose x intervals meet, found by a sort
 * on min x (a pair whose x intervals are disjoint fails the predicate, so
 * the set is the brute force's). */
static pvec scene_pairs(const float* mn, const float* mx, uint32_t b, uint32_t e, uint32_t bf_max) {
    pvec out = {0, 0, 0};
    const uint32_t m = e - b;
    if (m < 2) return out;
    if (m <= bf_max) {
        for (uint32_t i = b; i < e; ++i)
            for (uint32_t j = i + 1; j < e; ++j)
                if (pred_aabb_ix(mn, mx, i, j)) pv_push(&out, ((uint64_t)i << 32) | j);
        return out;
    }
    uint64_t* ord = (uint64_t*)malloc((size_t)m * 8);  /* (flip(min x) << 32) | local index */
    for (uint32_t k = 0; k < m; ++k) ord[k] = ((uint64_t)orc_float_flip(mn[4 * (size_t)(b + k)]) << 32) | k;
    qsort(ord, m, 8, cmp_u64);
    for (uint32_t p = 0; p < m; ++p) {
        const uint32_t i = b + (uint32_t)ord[p];
        const float hx = mx[4 * (size_t)i];
        for (uint32_t q = p + 1; q < m; ++q) {
            const uint32_t j = b + (uint32_t)ord[q];
            if (!(mn[4 * (size_t)j] <= hx)) break;
            if (pred_aabb_ix(mn, mx, i, j)) pv_push(&out, i < j ? ((uint64_t)i << 32) | j : ((uint64_t)j << 32) | i);
        }
    }
    free(ord);
    qsort(out.p, out.n, 8, cmp_u64);
    return out;
}

int64_t orc_pairs_batched(const float* mn, const float* mx, const int64_t* off, int num_scenes, uint32_t bf_max,
                          uint32_t* pairs, int64_t cap, int threads) {
    const int nt = nthreads(threads);
    pvec* per = (pvec*)calloc((size_t)(num_scenes > 0 ? num_scenes : 1), sizeof(pvec));
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int s = 0; s < num_scenes; ++s) per[s] = scene_pairs(mn, mx, (uint32_t)off[s], (uint32_t)off[s + 1], bf_max);
    int64_t total = 0;
    for (int s = 0; s < num_scenes; ++s) {
        for (size_t k = 0; k < per[s].n; ++k, ++total) {
            if (pairs && total < cap) {
                pairs[2 * total] = (uint32_t)(per[s].p[k] >> 32);
                pairs[2 * total + 1] = (uint32_t)per[s].p[k];
            }
        }
        free(per[s].p);
    }
    free(per);
    return total;
}
