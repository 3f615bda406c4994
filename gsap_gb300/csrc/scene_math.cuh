// Scene statistics -> sweep axes and grid.  Host and device: the PCA kernel
// runs it in its last CTA per scene, and the library exports a host copy
// (gsap_debug_scene_solve) so the solver can be checked without a GPU.
//
// FP64 where the result needs it: the covariance combine (sums about a
// pilot point, so that the mean's square does not cancel the variance).  The
// 3x3 symmetric eigensolve runs in FP32 (eig3 below), and so does the grid
// choice that follows, a heuristic: any axes and any grid give the same pair
// set.
#pragma once
#include "internal.cuh"
#include <math.h>

namespace gsap {

// One cyclic Jacobi sweep step on (p, q) of a symmetric 3x3 matrix; T is
// float or double.  Rotation by (c, s) with t = tan of the angle that zeroes
// a[p][q]; accumulates the rotation into the columns of v.
template <class T>
__host__ __device__ inline void jacobi_rotate(T a[3][3], T v[3][3], int p, int q) {
    T apq = a[p][q];
    if (apq == T(0)) return;
    T diff = a[q][q] - a[p][p];
    T t;
    if (fabs(apq) < T(1e-6) * fabs(diff)) {
        t = apq / diff;  // small angle: tan(phi) = apq / diff to O(phi^3)
    } else {
        T theta = diff / (T(2) * apq);
        t = (theta >= T(0) ? T(1) : T(-1)) / (fabs(theta) + sqrt(theta * theta + T(1)));
    }
    T c = T(1) / sqrt(t * t + T(1)), s = t * c;
    for (int k = 0; k < 3; ++k) {  // A <- A J
        T akp = a[k][p], akq = a[k][q];
        a[k][p] = c * akp - s * akq;
        a[k][q] = s * akp + c * akq;
    }
    for (int k = 0; k < 3; ++k) {  // A <- J^T A
        T apk = a[p][k], aqk = a[q][k];
        a[p][k] = c * apk - s * aqk;
        a[q][k] = s * apk + c * aqk;
    }
    for (int k = 0; k < 3; ++k) {
        T vkp = v[k][p], vkq = v[k][q];
        v[k][p] = c * vkp - s * vkq;
        v[k][q] = s * vkp + c * vkq;
    }
}

// Sweeps until the off-diagonal part is below tol * |diag| or stops
// shrinking (it cannot go below a few ulps of the diagonal, so a tolerance
// under the type's epsilon would otherwise run every sweep).
template <class T>
__host__ __device__ inline void jacobi_sweeps(T a[3][3], T v[3][3], T tol, int max_sweeps) {
    const T scale = fabs(a[0][0]) + fabs(a[1][1]) + fabs(a[2][2]) + T(1e-30);
    T prev = T(-1);
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        T off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
        if (off <= tol * scale) break;
        if (prev >= T(0) && off >= T(0.5) * prev) break;  // converged to rounding level
        prev = off;
        jacobi_rotate(a, v, 0, 1);
        jacobi_rotate(a, v, 0, 2);
        jacobi_rotate(a, v, 1, 2);
    }
}

// Symmetric 3x3 eigensolve: cyclic Jacobi in FP32 on the covariance rounded
// to FP32, to rounding level (a is overwritten with the diagonalised matrix,
// v receives the eigenvectors as columns).  Eigenvalues come out within a few
// FP32 ulps of the largest one and the axes orthonormal to ~1e-7, far more
// than the sweep needs: any axes give the same pair set (the reference
// itself sweeps along the largest-variance coordinate axis,
// SapKernel.cu:63-97).  An FP64 refinement of these axes (Newton-Schulz
// orthonormalisation and a first-order eigenvector correction) was measured
// at 12 us more per 1M call for the one-scene finish: dependent FP64
// operations take hundreds of cycles on this GPU.
__host__ __device__ inline void eig3(float a[3][3], float v[3][3]) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) v[i][j] = (i == j) ? 1.f : 0.f;
    jacobi_sweeps<float>(a, v, 2.4e-7f, 12);
}

// Sums (FP64) of one scene -> axes, statistics and sweep grid.
struct SceneSums {
    double sd[3], sdd[6], sh[3], shh[6], hmax[3];
    double pilot[3];
    double n;
};

__host__ __device__ inline void choose_scene(const SceneSums& z, const BpArgs& A, uint64_t entry_cap, uint32_t n_total,
                                             Scene& out) {
    const double n = z.n > 0 ? z.n : 1.0;
    const double inv_n = 1.0 / n;
    double md[3] = {z.sd[0] * inv_n, z.sd[1] * inv_n, z.sd[2] * inv_n};
    // covariance about the mean, from sums about the pilot (FP64)
    double C[3][3];
    const int idx[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    for (int i = 0; i < 3; ++i)
        for (int j = i; j < 3; ++j) C[i][j] = C[j][i] = z.sdd[idx[i][j]] * inv_n - md[i] * md[j];
    double mean[3] = {z.pilot[0] + md[0], z.pilot[1] + md[1], z.pilot[2] + md[2]};

    // From here on FP32 (the FP64 fields of the record are written from it):
    // serial FP64 operations are slow on this GPU, and the axes need no more.
    float U[3][3], lam[3];
    if (A.axis_mode == 1) {
        // axisVecMultiple (SapKernel.cu:63-97): largest diagonal entry, the
        // reference's tie order, fixed secondary axes.
        int ax = C[0][0] >= C[1][1] ? 0 : 1;
        if (ax) ax = C[1][1] >= C[2][2] ? 1 : 2;
        else ax = C[0][0] >= C[2][2] ? 0 : 2;
        int a1 = ax == 0 ? 1 : 0, a2 = 3 - ax - a1;
        int order[3] = {ax, a1, a2};
        const double dg[3] = {C[0][0], C[1][1], C[2][2]};  // (no data-dependent index into C)
        for (int r = 0; r < 3; ++r) {
            for (int c = 0; c < 3; ++c) U[r][c] = (c == order[r]) ? 1.f : 0.f;
            lam[r] = (float)(order[r] == 0 ? dg[0] : order[r] == 1 ? dg[1] : dg[2]);
        }
    } else {
        float a[3][3], v[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) a[i][j] = (float)C[i][j];  // C is symmetric as built
        eig3(a, v);
        // Descending eigenvalues, stable on ties (the compare-exchanges of a
        // three-element bubble sort).  Columns are swapped with constant
        // indices only, so that a, v and U stay in registers on the GPU (an
        // index that depends on the data would put them in local memory,
        // under every Jacobi update).
        float ev[3] = {a[0][0], a[1][1], a[2][2]};
        auto order = [&](int i, int j) {
            if (ev[i] < ev[j]) {
                const float t = ev[i]; ev[i] = ev[j]; ev[j] = t;
                for (int c = 0; c < 3; ++c) { const float w = v[c][i]; v[c][i] = v[c][j]; v[c][j] = w; }
            }
        };
        order(0, 1);
        order(1, 2);
        order(0, 1);
        for (int r = 0; r < 3; ++r) {
            lam[r] = ev[r];
            for (int c = 0; c < 3; ++c) U[r][c] = v[c][r];
            // sign: largest-magnitude component positive (lowest index on ties)
            float big = U[r][0], abig = fabsf(U[r][0]);
            if (fabsf(U[r][1]) > abig) { big = U[r][1]; abig = fabsf(U[r][1]); }
            if (fabsf(U[r][2]) > abig) big = U[r][2];
            if (big < 0.f) for (int c = 0; c < 3; ++c) U[r][c] = -U[r][c];
        }
        // right-handed frame
        U[2][0] = U[0][1] * U[1][2] - U[0][2] * U[1][1];
        U[2][1] = U[0][2] * U[1][0] - U[0][0] * U[1][2];
        U[2][2] = U[0][0] * U[1][1] - U[0][1] * U[1][0];
    }
    for (int r = 0; r < 3; ++r) {
        out.eig[r] = lam[r];
        out.mean[r] = mean[r];
        for (int c = 0; c < 3; ++c) {
            out.axes[3 * r + c] = U[r][c];
            out.u[3 * r + c] = U[r][c];
        }
    }
    // ---- grid choice: a heuristic, FP32 from here on
    float Cf[3][3], meanf[3], shf[3], shhf[6];
    for (int i = 0; i < 3; ++i) {
        meanf[i] = (float)mean[i];
        shf[i] = (float)z.sh[i];
        for (int j = 0; j < 3; ++j) Cf[i][j] = (float)C[i][j];
    }
    for (int k = 0; k < 6; ++k) shhf[k] = (float)z.shh[k];
    const float nf = (float)n, invf = 1.f / nf;
    float mc[3], sig[3], hw[3], sw[3];
    for (int r = 0; r < 3; ++r) {
        const float* u = &out.u[3 * r];
        mc[r] = u[0] * meanf[0] + u[1] * meanf[1] + u[2] * meanf[2];
        float var = 0.f;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) var += u[i] * Cf[i][j] * u[j];
        sig[r] = sqrtf(var > 0.f ? var : 0.f);
        sw[r] = 2.f * (fabsf(u[0]) * shf[0] + fabsf(u[1]) * shf[1] + fabsf(u[2]) * shf[2]);  // sum of widths
        hw[r] = 0.5f * sw[r] * invf;                                                           // mean half width
    }
    // lower-bound quantisation range along u1
    float qr = 8.f * sig[0] + 4.f * hw[0];
    if (!(qr > 1e-30f) || !isfinite(qr)) qr = 1.f;
    out.q_org = mc[0] - 4.f * sig[0] - 2.f * hw[0];
    out.q_range = qr;
    // secondary-axis grid
    float r2 = 8.f * sig[1] + 2.f * hw[1], r3 = 8.f * sig[2] + 2.f * hw[2];
    if (!(r2 > 1e-30f) || !isfinite(r2)) r2 = 1.f;
    if (!(r3 > 1e-30f) || !isfinite(r3)) r3 = 1.f;
    const float width = hw[1] + hw[2];  // mean full width averaged over the two axes
    const float cf = A.cell_factor > 0 ? A.cell_factor : 2.0f;
    const float target = 16.f;           // aim for at least this many objects per cell
    float s = cf * width;
    float sd = sqrtf(r2 * r3 * target / (nf > 1.f ? nf : 1.f));
    if (s < sd) s = sd;
    if (!(s > 0.f) || !isfinite(s)) s = r2 > r3 ? r2 : r3;
    const int qmin = A.key_bits >= 32 ? 12 : (A.key_bits >= 24 ? 8 : 6);  // q bits kept for u1
    const float bmax = ldexpf(1.f, (int)A.key_bits - qmin);
    const float share = nf / (float)(n_total > 0 ? n_total : 1u);
    float bcap = floorf(bmax * share);
    if (bcap < 1.f) bcap = 1.f;
    const float ecap = floorf((float)entry_cap * share);
    // sum over objects of w2*w3: 4 sum_{m,l} |u2m| |u3l| sum h_m h_l
    const int hidx[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    float sww = 0.f;
    for (int m = 0; m < 3; ++m)
        for (int l = 0; l < 3; ++l) sww += 4.f * fabsf(out.u[3 + m]) * fabsf(out.u[6 + l]) * shhf[hidx[m][l]];
    float G2 = 1.f, G3 = 1.f;
    for (int it = 0; it < 400; ++it) {
        G2 = fminf(ceilf(r2 / s), 65535.f);
        G3 = fminf(ceilf(r3 / s), 65535.f);
        if (G2 < 1.f) G2 = 1.f;
        if (G3 < 1.f) G3 = 1.f;
        bool ok = G2 * G3 <= bcap;
        if (ok) {
            // worst-case entries: per axis min(G, w*inv + 2) cells
            float i2 = G2 / r2 * (1.f + 1e-4f), i3 = G3 / r3 * (1.f + 1e-4f);
            float e;
            if (G2 == 1.f && G3 == 1.f) e = nf;
            else if (G2 == 1.f) e = sw[2] * i3 + 2.f * nf;
            else if (G3 == 1.f) e = sw[1] * i2 + 2.f * nf;
            else e = 4.f * nf + 2.f * (sw[1] * i2 + sw[2] * i3) + sww * i2 * i3;
            ok = e * 1.01f + 64.f <= ecap;
        }
        if (ok) break;
        s *= 1.1f;
        if (it == 399) { G2 = 1.f; G3 = 1.f; }
    }
    out.G2 = (uint32_t)G2;
    out.G3 = (uint32_t)G3;
    out.c2_org = mc[1] - 4.f * sig[1] - hw[1];
    out.c3_org = mc[2] - 4.f * sig[2] - hw[2];
    out.c2_inv = G2 / r2;
    out.c3_inv = G3 / r3;
    out.n = (uint32_t)z.n;
}

}  // namespace gsap
