/*
 * CPU oracle, rigid-body half.  TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * orc_rb_step_ref restates the reference kernels of
 * ParticleRigidBody/ParticleRigidBodyKernel.h in FP32 with their exact
 * operation order (compiled with -ffp-contract=off; float4 helpers follow the
 * SDK float4 semantics used there: componentwise ops on all four lanes,
 * x / s evaluated as x * (1/s), length = sqrtf(dot4)).
 *
 * orc_rb_step_cfg_f64 is the FP64 trajectory oracle of the config-mode
 * contact model (spring k, normal damping eta, tangential damping ratio kt,
 * gravity, six box walls) that the GPU computes in FP32.
 */
#include "oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXP 10 /* MAX_NUM_PARTICLES, ParticleRigidBody.h:39 */

typedef struct f4 { float x, y, z, w; } f4;
static inline f4 mk(float x, float y, float z, float w) { f4 r = {x, y, z, w}; return r; }
static inline f4 ld4(const float* p) { return mk(p[0], p[1], p[2], p[3]); }
static inline void st4(float* p, f4 a) { p[0] = a.x; p[1] = a.y; p[2] = a.z; p[3] = a.w; }
static inline f4 add(f4 a, f4 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
static inline f4 sub(f4 a, f4 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
static inline f4 mul(f4 a, float s) { return mk(a.x * s, a.y * s, a.z * s, a.w * s); }
static inline f4 divs(f4 a, float s) { float inv = 1.0f / s; return mul(a, inv); }
static inline float dot4(f4 a, f4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
static inline float dot3(f4 a, f4 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float len4(f4 a) { return sqrtf(dot4(a, a)); }
/* cross of the xyz parts, w = 0 (quaternion.h:16-22) */
static inline f4 cross4(f4 a, f4 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x, 0.f);
}
/* Quaternion product (quaternion.h:130-139) */
static inline f4 qmul(f4 a, f4 b) {
    f4 ans = cross4(a, b);
    ans = add(ans, add(mul(b, a.w), mul(a, b.w)));
    ans.w = a.w * b.w - dot3(a, b);
    return ans;
}
/* q * v * q^-1 with the full float4 v, w included (quaternion.h:141-148) */
static inline f4 qrot(f4 q, f4 v) {
    f4 qi = mk(-q.x, -q.y, -q.z, q.w);
    return qmul(qmul(q, v), qi);
}
/* getRotationMatrix (quaternion.h:90-106), rows as float4 with w = 0 */
static void qmat(f4 q, f4 m[3]) {
    float x2 = q.x * q.x, y2 = q.y * q.y, z2 = q.z * q.z;
    m[0] = mk(1 - 2 * y2 - 2 * z2, 2 * q.x * q.y - 2 * q.w * q.z, 2 * q.x * q.z + 2 * q.w * q.y, 0);
    m[1] = mk(2 * q.x * q.y + 2 * q.w * q.z, 1 - 2 * x2 - 2 * z2, 2 * q.y * q.z - 2 * q.w * q.x, 0);
    m[2] = mk(2 * q.x * q.z - 2 * q.w * q.y, 2 * q.y * q.z + 2 * q.w * q.x, 1 - 2 * x2 - 2 * y2, 0);
}
/* Matrix3x3 product via rows of a and rows of transpose(b) (matrix3x3.h) */
static void mmul(const f4 a[3], const f4 b[3], f4 out[3]) {
    f4 bt[3] = {mk(b[0].x, b[1].x, b[2].x, 0), mk(b[0].y, b[1].y, b[2].y, 0), mk(b[0].z, b[1].z, b[2].z, 0)};
    for (int i = 0; i < 3; ++i) out[i] = mk(dot3(a[i], bt[0]), dot3(a[i], bt[1]), dot3(a[i], bt[2]), 0);
}

/* calcSpringCoeff (ParticleRigidBodyKernel.h:13-22) */
static inline void spring_coeff(float imi, float jmi, float dt2i, float dti, float sp, float dp,
                                float* s, float* d) {
    float m = imi + jmi;
    m = 1 / m;
    *s = m * dt2i * sp;
    *d = m * dti * (1.f - dp);
}

void orc_normalize_quats(float* quat, int n) {
    for (int i = 0; i < n; ++i) st4(quat + 4 * i, divs(ld4(quat + 4 * i), len4(ld4(quat + 4 * i))));
}

int64_t orc_rb_step_ref(orc_rb_state* s, const orc_ref_params* p, int64_t max_pairs, int threads) {
    const float dt = p->dt;
    const int nb = s->n_bodies;
    (void)threads;
    /* integrateK (:47-69) */
    for (int i = 0; i < nb; ++i) {
        f4 lv = add(ld4(s->lin_vel + 4 * i), mul(mk(0.0f, p->gravity_y, 0.0f, 0.0f), dt));
        st4(s->lin_vel + 4 * i, lv);
        f4 q = ld4(s->quat + 4 * i);
        f4 w = ld4(s->ang_vel + 4 * i);
        w.w = 0.f;
        q = add(q, mul(qmul(w, q), dt * 0.5f));
        q = divs(q, len4(q));
        st4(s->quat + 4 * i, q);
        float* x = s->pos + 4 * i;
        x[0] += lv.x * dt;
        x[1] += lv.y * dt;
        x[2] += lv.z * dt;
        if (p->floor_clamp) {
            if ((i / 6) % 2 == 0 && x[1] <= 0.25f) x[1] = 0.25f;
            else if ((i / 6) % 2 == 1 && x[1] <= 0.3f) x[1] = 0.3f;
        }
    }
    /* updateParticleDataK (:71-104) */
    for (int b = 0; b < nb; ++b) {
        int st = s->p_start[b];
        f4 x = ld4(s->pos + 4 * b), v = ld4(s->lin_vel + 4 * b), q = ld4(s->quat + 4 * b);
        f4 w = ld4(s->ang_vel + 4 * b);
        for (int k = 0; k < s->n_part[b]; ++k) {
            int ri = MAXP * s->shape_idx[b] + k;
            f4 ref = ld4(s->ref_pos + 4 * ri);
            f4 cp = qrot(q, ref);
            st4(s->p_vel + 4 * (st + k), add(v, cross4(w, cp)));
            cp = add(cp, x);
            st4(s->p_pos + 4 * (st + k), mk(cp.x, cp.y, cp.z, ref.w));
            s->p_mass[st + k] = s->ref_mass[ri];
        }
    }
    /* broadphase on the particles (DemoParticles::cpuBroadphase form) */
    const int np = s->n_particles;
    int64_t cap = max_pairs / 2;
    uint32_t* pr = (uint32_t*)malloc((size_t)(cap > 0 ? cap : 1) * 8);
    int64_t nu = orc_bf_sphere(s->p_pos, (uint32_t)np, pr, cap, threads);
    if (nu > cap) { free(pr); return -1; }
    int32_t* both = (int32_t*)malloc((size_t)(2 * nu > 0 ? 2 * nu : 1) * 8);
    int32_t* ent = (int32_t*)malloc((size_t)(np > 0 ? np : 1) * 4);
    int64_t ne = orc_both_directions(pr, nu, both, ent);
    free(pr);
    /* prepareK (:30-45) */
    for (int b = 0; b < nb; ++b) {
        f4 r[3], rt[3], is[3], t[3], o[3];
        qmat(ld4(s->quat + 4 * b), r);
        rt[0] = mk(r[0].x, r[1].x, r[2].x, 0);
        rt[1] = mk(r[0].y, r[1].y, r[2].y, 0);
        rt[2] = mk(r[0].z, r[1].z, r[2].z, 0);
        const float* si = s->shape_inv_inertia + 12 * s->shape_idx[b];
        for (int k = 0; k < 3; ++k) is[k] = ld4(si + 4 * k);
        mmul(r, is, t);
        mmul(t, rt, o);
        for (int k = 0; k < 3; ++k) st4(s->inv_inertia + 12 * b + 4 * k, o[k]);
    }
    /* clearForceAndBoundaryConditionK (:106-140) */
    const float dt2i = 1.f / (dt * dt), dti = 1.f / dt;
    for (int i = 0; i < np; ++i) {
        f4 ip = ld4(s->p_pos + 4 * i), iv = ld4(s->p_vel + 4 * i);
        float im = s->p_mass[i];
        f4 force = mk(0, 0, 0, 0);
        float dist = ip.y;
        f4 rij = mk(0, 1, 0, 0);
        f4 vij = mk(-iv.x, -iv.y, -iv.z, -iv.w);
        if (dist < ip.w) {
            float sc, dc;
            spring_coeff(1.f / im, 0.5f / im, dt2i, dti, p->sp_multip, p->dp_multip, &sc, &dc);
            f4 sf = mul(mul(rij, -sc * (dist - ip.w)), 0.1f);
            f4 df = mul(vij, dc);
            force = add(sf, df);
        }
        st4(s->p_force + 4 * i, force);
    }
    /* comupteFoceOnParticlesK (:142-208): one row of the CSR per entry; the
     * row ends at the next entry.  The reference's loop also stops after the
     * pair whose index equals numPairEntries (`if (pairIdx++ ==
     * numPairEntries) break;`, :201); pair_loop_quirk reproduces that. */
    for (int64_t e = 0; e < ne; ++e) {
        int64_t b0 = ent[e], b1 = (e + 1 < ne) ? ent[e + 1] : 2 * nu;
        int i = both[2 * b0];
        f4 ip = ld4(s->p_pos + 4 * i), iv = ld4(s->p_vel + 4 * i);
        float im = s->p_mass[i];
        f4 sf = mk(0, 0, 0, 0), df = mk(0, 0, 0, 0);
        for (int64_t k = b0; k < b1; ++k) {
            int j = both[2 * k + 1];
            f4 jp = ld4(s->p_pos + 4 * j), jv = ld4(s->p_vel + 4 * j);
            float jm = s->p_mass[j];
            f4 rij = sub(jp, ip);
            rij.w = 0.f;
            f4 vij = sub(jv, iv);
            float dist = len4(rij);
            float od = ip.w + jp.w;
            float sc, dc;
            spring_coeff(1.f / im, 1.f / jm, dt2i, dti, p->sp_multip, p->dp_multip, &sc, &dc);
            float pen = od - dist;
            if (pen > 0.f) {
                sf = sub(sf, divs(mul(rij, sc * pen), dist));
                df = add(df, mul(vij, dc));
            }
            if (p->pair_loop_quirk && k == ne) break;
        }
        f4 f = add(ld4(s->p_force + 4 * i), add(sf, df));
        st4(s->p_force + 4 * i, f);
    }
    /* updateVelocityK<CAP_VEL> (:213-262) */
    for (int b = 0; b < nb; ++b) {
        f4 q = ld4(s->quat + 4 * b);
        int st = s->p_start[b];
        f4 lf = mk(0, 0, 0, 0), af = mk(0, 0, 0, 0);
        for (int k = 0; k < s->n_part[b]; ++k) {
            int ri = MAXP * s->shape_idx[b] + k;
            f4 cp = qrot(q, ld4(s->ref_pos + 4 * ri));
            f4 f = ld4(s->p_force + 4 * (st + k));
            lf = add(lf, f);
            af = add(af, cross4(cp, f));
        }
        f4 lv = add(ld4(s->lin_vel + 4 * b), mul(mul(lf, s->inv_mass[b]), dt));
        if (p->max_lin_vel > 0.f) {
            f4 l = lv;
            l.w = 0;
            float ll = len4(l);
            if (ll > p->max_lin_vel) {
                float inv = 1.0f / sqrtf(dot4(l, l));
                lv = mul(mul(l, inv), p->max_lin_vel);
            }
        }
        st4(s->lin_vel + 4 * b, lv);
        f4 w = ld4(s->ang_vel + 4 * b);
        if (p->torque_quirk) {
            w = add(w, mul(af, dt));
        } else {
            const float* m = s->inv_inertia + 12 * b;
            f4 dw = mk(dot3(ld4(m), af), dot3(ld4(m + 4), af), dot3(ld4(m + 8), af), 0);
            w = add(w, mul(dw, dt));
        }
        st4(s->ang_vel + 4 * b, w);
    }
    free(both);
    free(ent);
    return 2 * nu;
}

/* ------------------------------------------------------------ FP64 config */

static inline void d_qmul(const double* a, const double* b, double* o) {
    double x = a[1] * b[2] - a[2] * b[1] + a[3] * b[0] + b[3] * a[0];
    double y = a[2] * b[0] - a[0] * b[2] + a[3] * b[1] + b[3] * a[1];
    double z = a[0] * b[1] - a[1] * b[0] + a[3] * b[2] + b[3] * a[2];
    double w = a[3] * b[3] - (a[0] * b[0] + a[1] * b[1] + a[2] * b[2]);
    o[0] = x; o[1] = y; o[2] = z; o[3] = w;
}
static inline void d_qmat(const double* q, double m[9]) {
    double x = q[0], y = q[1], z = q[2], w = q[3];
    m[0] = 1 - 2 * (y * y + z * z); m[1] = 2 * (x * y - w * z); m[2] = 2 * (x * z + w * y);
    m[3] = 2 * (x * y + w * z); m[4] = 1 - 2 * (x * x + z * z); m[5] = 2 * (y * z - w * x);
    m[6] = 2 * (x * z - w * y); m[7] = 2 * (y * z + w * x); m[8] = 1 - 2 * (x * x + y * y);
}
static inline void d_mv(const double m[9], const double* v, double* o) {
    double a = m[0] * v[0] + m[1] * v[1] + m[2] * v[2];
    double b = m[3] * v[0] + m[4] * v[1] + m[5] * v[2];
    double c = m[6] * v[0] + m[7] * v[1] + m[8] * v[2];
    o[0] = a; o[1] = b; o[2] = c;
}
static inline void d_cross(const double* a, const double* b, double* o) {
    double x = a[1] * b[2] - a[2] * b[1], y = a[2] * b[0] - a[0] * b[2], z = a[0] * b[1] - a[1] * b[0];
    o[0] = x; o[1] = y; o[2] = z;
}

/* Contact force on particle i from particle j (or a wall, jv = 0):
 * n = unit vector from i to j, pen = penetration depth, vrel = v_j - v_i,
 * f_i = -k pen n + eta (vrel.n) n + kt eta (vrel - (vrel.n) n). */
static inline void d_contact(const orc_cfg_params* p, const double* n, double pen,
                             const double* vrel, double* f) {
    double vn = vrel[0] * n[0] + vrel[1] * n[1] + vrel[2] * n[2];
    for (int a = 0; a < 3; ++a) {
        double vt = vrel[a] - vn * n[a];
        f[a] += -p->k * pen * n[a] + p->eta * vn * n[a] + p->kt * p->eta * vt;
    }
}

/* Body pair search of the FP64 oracle: per body the ids of every other body
 * of its scene whose closed AABB meets its own (the body broadphase the
 * GPU step runs), rows in ascending id order.  brute != 0 tests all pairs;
 * otherwise the bodies of each scene are sorted by min x and each sweeps
 * forward while the next min x is <= its max x (the same set, O(n log n)).
 * cnt[nb + 1] receives the row offsets; nbr (capacity cap) the ids.
 * Returns the total row length, or -1 if cap is too small. */
typedef struct { double key; int id; } key_id;
static int cmp_key_id(const void* a, const void* b) {
    const key_id* x = (const key_id*)a;
    const key_id* y = (const key_id*)b;
    if (x->key < y->key) return -1;
    if (x->key > y->key) return 1;
    return (x->id > y->id) - (x->id < y->id);
}
static int cmp_int(const void* a, const void* b) {
    int x = *(const int*)a, y = *(const int*)b;
    return (x > y) - (x < y);
}
static inline int box_meets(const double* bmin, const double* bmax, int a, int b) {
    int ov = 1;
    for (int k = 0; k < 3; ++k) ov &= bmin[3 * a + k] <= bmax[3 * b + k] && bmin[3 * b + k] <= bmax[3 * a + k];
    return ov;
}

int64_t orc_body_neighbours(int nb, const double* bmin, const double* bmax, const int* scene, int brute,
                            int threads, int* cnt, int* nbr, int64_t cap) {
    int nt = 1;
#ifdef _OPENMP
    nt = threads > 0 ? threads : omp_get_max_threads();
#else
    (void)threads;
#endif
    for (int a = 0; a <= nb; ++a) cnt[a] = 0;
    if (brute) {
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
        for (int a = 0; a < nb; ++a) {
            int c = 0;
            for (int b = 0; b < nb; ++b)
                if (b != a && !(scene && scene[a] != scene[b])) c += box_meets(bmin, bmax, a, b);
            cnt[a + 1] = c;
        }
        for (int a = 0; a < nb; ++a) cnt[a + 1] += cnt[a];
        if (cnt[nb] > cap) return -1;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
        for (int a = 0; a < nb; ++a) {
            int o = cnt[a];
            for (int b = 0; b < nb; ++b)
                if (b != a && !(scene && scene[a] != scene[b]) && box_meets(bmin, bmax, a, b)) nbr[o++] = b;
        }
        return cnt[nb];
    }
    /* group the bodies by scene (stable counting sort), then sort each group by min x */
    int ns = 1;
    if (scene)
        for (int a = 0; a < nb; ++a) if (scene[a] + 1 > ns) ns = scene[a] + 1;
    int* soff = (int*)calloc((size_t)ns + 1, sizeof(int));
    for (int a = 0; a < nb; ++a) soff[(scene ? scene[a] : 0) + 1]++;
    for (int k = 0; k < ns; ++k) soff[k + 1] += soff[k];
    int* fill = (int*)malloc((size_t)ns * sizeof(int));
    for (int k = 0; k < ns; ++k) fill[k] = soff[k];
    key_id* ord = (key_id*)malloc((size_t)(nb > 0 ? nb : 1) * sizeof(key_id));
    for (int a = 0; a < nb; ++a) {
        const int g = scene ? scene[a] : 0;
        ord[fill[g]].key = bmin[3 * a];
        ord[fill[g]].id = a;
        fill[g]++;
    }
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int k = 0; k < ns; ++k) qsort(ord + soff[k], (size_t)(soff[k + 1] - soff[k]), sizeof(key_id), cmp_key_id);
    /* forward sweep: count per body, then fill */
    int* grp_end = (int*)malloc((size_t)(nb > 0 ? nb : 1) * sizeof(int));
    for (int k = 0; k < ns; ++k)
        for (int q = soff[k]; q < soff[k + 1]; ++q) grp_end[q] = soff[k + 1];
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
    for (int q = 0; q < nb; ++q) {
        const int a = ord[q].id;
        const double hx = bmax[3 * a];
        int c = 0;
        for (int r = q + 1; r < grp_end[q] && ord[r].key <= hx; ++r) {
            const int b = ord[r].id;
            if (box_meets(bmin, bmax, a, b)) {
#pragma omp atomic
                cnt[b + 1]++;
                ++c;
            }
        }
#pragma omp atomic
        cnt[a + 1] += c;
    }
    for (int a = 0; a < nb; ++a) cnt[a + 1] += cnt[a];
    int64_t total = cnt[nb];
    if (total <= cap) {
        int* cur = (int*)malloc((size_t)(nb > 0 ? nb : 1) * sizeof(int));
        for (int a = 0; a < nb; ++a) cur[a] = cnt[a];
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
        for (int q = 0; q < nb; ++q) {
            const int a = ord[q].id;
            const double hx = bmax[3 * a];
            for (int r = q + 1; r < grp_end[q] && ord[r].key <= hx; ++r) {
                const int b = ord[r].id;
                if (box_meets(bmin, bmax, a, b)) {
                    int sa, sb;
#pragma omp atomic capture
                    sa = cur[a]++;
#pragma omp atomic capture
                    sb = cur[b]++;
                    nbr[sa] = b;
                    nbr[sb] = a;
                }
            }
        }
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
        for (int a = 0; a < nb; ++a) qsort(nbr + cnt[a], (size_t)(cnt[a + 1] - cnt[a]), sizeof(int), cmp_int);
        free(cur);
    }
    free(grp_end);
    free(ord);
    free(fill);
    free(soff);
    return total <= cap ? total : -1;
}

int64_t orc_rb_step_cfg_f64(orc_rb_state_d* s, const orc_cfg_params* p, int threads) {
    return orc_rb_step_cfg_f64_amb(s, p, threads, 0.0, NULL);
}

/* The same step; with amb != NULL also flags (amb[b] = 1, else 0) every body
 * with a contact whose penetration depth lies within +-band of zero: a
 * particle pair or a wall where a rounding of the state by about band can
 * switch the contact, and with it the damping force, on or off.  Body boxes
 * are widened by band for the pair search so that no such pair is missed. */
int64_t orc_rb_step_cfg_f64_amb(orc_rb_state_d* s, const orc_cfg_params* p, int threads, double band, int* amb) {
    const int nb = s->n_bodies;
    const double dt = p->dt;
    int nt = 1;
#ifdef _OPENMP
    nt = threads > 0 ? threads : omp_get_max_threads();
#else
    (void)threads;
#endif
    /* integrate: v += g dt; q += 0.5 dt (w,0) q, normalised; x += v dt */
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int b = 0; b < nb; ++b) {
        double* v = s->lin_vel + 4 * b;
        v[1] += p->gravity_y * dt;
        double* q = s->quat + 4 * b;
        double w[4] = {s->ang_vel[4 * b], s->ang_vel[4 * b + 1], s->ang_vel[4 * b + 2], 0.0};
        double dq[4];
        d_qmul(w, q, dq);
        for (int a = 0; a < 4; ++a) q[a] += 0.5 * dt * dq[a];
        double l = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
        for (int a = 0; a < 4; ++a) q[a] /= l;
        for (int a = 0; a < 3; ++a) s->pos[4 * b + a] += v[a] * dt;
    }
    /* place particles */
    double* bmin = (double*)malloc((size_t)(nb > 0 ? nb : 1) * 3 * sizeof(double));
    double* bmax = (double*)malloc((size_t)(nb > 0 ? nb : 1) * 3 * sizeof(double));
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int b = 0; b < nb; ++b) {
        double R[9];
        d_qmat(s->quat + 4 * b, R);
        for (int a = 0; a < 3; ++a) { bmin[3 * b + a] = 1e300; bmax[3 * b + a] = -1e300; }
        for (int k = 0; k < s->n_part[b]; ++k) {
            const double* ref = s->ref_pos + 4 * (MAXP * s->shape_idx[b] + k);
            double rp[3], wr[3];
            d_mv(R, ref, rp);
            d_cross(s->ang_vel + 4 * b, rp, wr);
            double* pp = s->p_pos + 4 * (s->p_start[b] + k);
            double* pv = s->p_vel + 4 * (s->p_start[b] + k);
            for (int a = 0; a < 3; ++a) {
                pp[a] = s->pos[4 * b + a] + rp[a];
                pv[a] = s->lin_vel[4 * b + a] + wr[a];
                if (pp[a] - ref[3] < bmin[3 * b + a]) bmin[3 * b + a] = pp[a] - ref[3];
                if (pp[a] + ref[3] > bmax[3 * b + a]) bmax[3 * b + a] = pp[a] + ref[3];
            }
            pp[3] = ref[3];
            pv[3] = 0;
        }
    }
    if (amb) {
        for (int b = 0; b < nb; ++b) {
            amb[b] = 0;
            for (int a = 0; a < 3; ++a) { bmin[3 * b + a] -= band; bmax[3 * b + a] += band; }
        }
    }
    /* body-AABB pairs (closed test) -> per-body neighbour rows in id order */
    int* cnt = (int*)malloc(((size_t)nb + 1) * sizeof(int));
    int64_t cap = 64 * (int64_t)nb + 1024;
    int* nbr = (int*)malloc((size_t)cap * sizeof(int));
    if (orc_body_neighbours(nb, bmin, bmax, s->scene, 0, threads, cnt, nbr, cap) < 0) {
        cap = cnt[nb];
        free(nbr);
        nbr = (int*)malloc((size_t)(cap > 0 ? cap : 1) * sizeof(int));
        orc_body_neighbours(nb, bmin, bmax, s->scene, 0, threads, cnt, nbr, cap);
    }
    int64_t examined = 0;
    /* particle forces: walls, then neighbour bodies in id order */
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt) reduction(+ : examined)
    for (int a = 0; a < nb; ++a) {
        for (int k = 0; k < s->n_part[a]; ++k) {
            int i = s->p_start[a] + k;
            const double* ip = s->p_pos + 4 * i;
            const double* iv = s->p_vel + 4 * i;
            double f[3] = {0, 0, 0};
            for (int ax = 0; ax < 3; ++ax) {
                double pen_lo = ip[3] - (ip[ax] - p->box_lo[ax]);
                double pen_hi = ip[3] - (p->box_hi[ax] - ip[ax]);
                if (amb && (fabs(pen_lo) < band || fabs(pen_hi) < band)) amb[a] = 1;
                double vrel[3] = {-iv[0], -iv[1], -iv[2]};
                if (pen_lo > 0) {
                    double n[3] = {0, 0, 0};
                    n[ax] = -1.0; /* from particle towards the wall */
                    d_contact(p, n, pen_lo, vrel, f);
                }
                if (pen_hi > 0) {
                    double n[3] = {0, 0, 0};
                    n[ax] = 1.0;
                    d_contact(p, n, pen_hi, vrel, f);
                }
            }
            for (int e = cnt[a]; e < cnt[a + 1]; ++e) {
                int b = nbr[e];
                for (int l = 0; l < s->n_part[b]; ++l) {
                    int j = s->p_start[b] + l;
                    const double* jp = s->p_pos + 4 * j;
                    const double* jv = s->p_vel + 4 * j;
                    double d[3] = {jp[0] - ip[0], jp[1] - ip[1], jp[2] - ip[2]};
                    double dist = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                    double pen = ip[3] + jp[3] - dist;
                    if (amb && fabs(pen) < band) amb[a] = 1;
                    ++examined;
                    if (pen > 0 && dist > 0) {
                        double n[3] = {d[0] / dist, d[1] / dist, d[2] / dist};
                        double vrel[3] = {jv[0] - iv[0], jv[1] - iv[1], jv[2] - iv[2]};
                        d_contact(p, n, pen, vrel, f);
                    }
                }
            }
            double* pf = s->p_force + 4 * i;
            pf[0] = f[0]; pf[1] = f[1]; pf[2] = f[2]; pf[3] = 0;
        }
    }
    /* per-body reduction and velocity update: omega += I_w^-1 tau dt */
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int b = 0; b < nb; ++b) {
        double R[9];
        d_qmat(s->quat + 4 * b, R);
        double F[3] = {0, 0, 0}, T[3] = {0, 0, 0};
        for (int k = 0; k < s->n_part[b]; ++k) {
            const double* ref = s->ref_pos + 4 * (MAXP * s->shape_idx[b] + k);
            double rp[3], c[3];
            d_mv(R, ref, rp);
            const double* f = s->p_force + 4 * (s->p_start[b] + k);
            d_cross(rp, f, c);
            for (int a = 0; a < 3; ++a) { F[a] += f[a]; T[a] += c[a]; }
        }
        const double* Is = s->shape_inv_inertia + 9 * s->shape_idx[b];
        /* I_w^-1 tau = R Is R^T tau */
        double t1[3], t2[3], t3[3];
        t1[0] = R[0] * T[0] + R[3] * T[1] + R[6] * T[2];
        t1[1] = R[1] * T[0] + R[4] * T[1] + R[7] * T[2];
        t1[2] = R[2] * T[0] + R[5] * T[1] + R[8] * T[2];
        d_mv(Is, t1, t2);
        d_mv(R, t2, t3);
        for (int a = 0; a < 3; ++a) {
            s->lin_vel[4 * b + a] += F[a] * s->inv_mass[b] * dt;
            s->ang_vel[4 * b + a] += t3[a] * dt;
        }
    }
    free(cnt);
    free(nbr);
    free(bmin);
    free(bmax);
    return examined;
}
