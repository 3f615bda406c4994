// FP64 scene statistics -> sweep axes and grid.  Host and device: the PCA
// kernel runs it in its last CTA per scene, and the library exports a host
// copy (gsap_debug_choose_scene) so the solver can be checked without a GPU.
#pragma once
#include "internal.cuh"
#include <math.h>

namespace gsap {


// Cyclic Jacobi for a symmetric 3x3 matrix (FP64).  On return a holds the
// diagonalised matrix and v the eigenvectors as columns.
__host__ __device__ inline void jacobi3(double a[3][3], double v[3][3]) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) v[i][j] = (i == j) ? 1.0 : 0.0;
    const double scale = fabs(a[0][0]) + fabs(a[1][1]) + fabs(a[2][2]) + 1e-300;
    for (int sweep = 0; sweep < 32; ++sweep) {
        double off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
        if (off <= 1e-17 * scale) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                double apq = a[p][q];
                if (fabs(apq) <= 1e-300) continue;
                double theta = (a[q][q] - a[p][p]) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; ++k) {  // A <- A J
                    double akp = a[k][p], akq = a[k][q];
                    a[k][p] = c * akp - s * akq;
                    a[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; ++k) {  // A <- J^T A
                    double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = c * apk - s * aqk;
                    a[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; ++k) {
                    double vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = c * vkp - s * vkq;
                    v[k][q] = s * vkp + c * vkq;
                }
            }
    }
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
    double md[3] = {z.sd[0] / n, z.sd[1] / n, z.sd[2] / n};
    // covariance about the mean, from sums about the pilot
    double C[3][3];
    const int idx[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) C[i][j] = z.sdd[idx[i][j]] / n - md[i] * md[j];
    double mean[3] = {z.pilot[0] + md[0], z.pilot[1] + md[1], z.pilot[2] + md[2]};

    double U[3][3], lam[3];
    if (A.axis_mode == 1) {
        // axisVecMultiple (SapKernel.cu:63-97): largest diagonal entry, the
        // reference's tie order, fixed secondary axes.
        int ax = C[0][0] >= C[1][1] ? 0 : 1;
        if (ax) ax = C[1][1] >= C[2][2] ? 1 : 2;
        else ax = C[0][0] >= C[2][2] ? 0 : 2;
        int a1 = ax == 0 ? 1 : 0, a2 = 3 - ax - a1;
        int order[3] = {ax, a1, a2};
        for (int r = 0; r < 3; ++r) {
            for (int c = 0; c < 3; ++c) U[r][c] = (c == order[r]) ? 1.0 : 0.0;
            lam[r] = C[order[r]][order[r]];
        }
    } else {
        double a[3][3], v[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) a[i][j] = 0.5 * (C[i][j] + C[j][i]);
        jacobi3(a, v);
        int o[3] = {0, 1, 2};
        double ev[3] = {a[0][0], a[1][1], a[2][2]};
        // descending eigenvalues, stable on ties
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 2 - i; ++j)
                if (ev[o[j]] < ev[o[j + 1]]) { int t = o[j]; o[j] = o[j + 1]; o[j + 1] = t; }
        for (int r = 0; r < 3; ++r) {
            lam[r] = ev[o[r]];
            for (int c = 0; c < 3; ++c) U[r][c] = v[c][o[r]];
            // sign: largest-magnitude component positive (lowest index on ties)
            int m = 0;
            for (int c = 1; c < 3; ++c) if (fabs(U[r][c]) > fabs(U[r][m])) m = c;
            if (U[r][m] < 0) for (int c = 0; c < 3; ++c) U[r][c] = -U[r][c];
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
            out.u[3 * r + c] = (float)U[r][c];
        }
    }
    // projected statistics on each axis (using the FP32 axes actually applied)
    double mc[3], sig[3], hw[3], sw[3];
    double mh[3] = {z.sh[0] / n, z.sh[1] / n, z.sh[2] / n};
    for (int r = 0; r < 3; ++r) {
        double u0 = out.u[3 * r], u1 = out.u[3 * r + 1], u2 = out.u[3 * r + 2];
        mc[r] = u0 * mean[0] + u1 * mean[1] + u2 * mean[2];
        double var = 0;
        double uu[3] = {u0, u1, u2};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) var += uu[i] * C[i][j] * uu[j];
        sig[r] = sqrt(var > 0 ? var : 0);
        hw[r] = fabs(u0) * mh[0] + fabs(u1) * mh[1] + fabs(u2) * mh[2];            // mean half width
        sw[r] = 2.0 * (fabs(u0) * z.sh[0] + fabs(u1) * z.sh[1] + fabs(u2) * z.sh[2]);  // sum of widths
    }
    // lower-bound quantisation range along u1
    double qr = 8.0 * sig[0] + 4.0 * hw[0];
    if (!(qr > 1e-30)) qr = 1.0;
    out.q_org = (float)(mc[0] - 4.0 * sig[0] - 2.0 * hw[0]);
    out.q_range = (float)qr;
    // secondary-axis grid
    double r2 = 8.0 * sig[1] + 2.0 * hw[1], r3 = 8.0 * sig[2] + 2.0 * hw[2];
    if (!(r2 > 1e-30)) r2 = 1.0;
    if (!(r3 > 1e-30)) r3 = 1.0;
    double width = hw[1] + hw[2];  // mean full width averaged over the two axes
    double cf = A.cell_factor > 0 ? A.cell_factor : 1.5;
    double target = 16.0;          // aim for at least this many objects per cell
    double s = cf * width;
    double sd = sqrt(r2 * r3 * target / (z.n > 1 ? z.n : 1.0));
    if (s < sd) s = sd;
    if (!(s > 0)) s = 1.0;
    const int qmin = A.key_bits >= 32 ? 12 : 8;
    double bmax = ldexp(1.0, (int)A.key_bits - qmin);
    double bcap = floor(bmax * (z.n > 0 ? z.n : 1.0) / (n_total > 0 ? n_total : 1u));
    if (bcap < 1) bcap = 1;
    double ecap = floor((double)entry_cap * (z.n > 0 ? z.n : 1.0) / (n_total > 0 ? n_total : 1u));
    // sum over objects of w2*w3: 4 sum_{m,l} |u2m| |u3l| sum h_m h_l
    const int hidx[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    double sww = 0;
    for (int m = 0; m < 3; ++m)
        for (int l = 0; l < 3; ++l)
            sww += 4.0 * fabs((double)out.u[3 + m]) * fabs((double)out.u[6 + l]) * z.shh[hidx[m][l]];
    double G2 = 1, G3 = 1;
    for (int it = 0; it < 400; ++it) {
        G2 = fmin(ceil(r2 / s), 65535.0);
        G3 = fmin(ceil(r3 / s), 65535.0);
        if (G2 < 1) G2 = 1;
        if (G3 < 1) G3 = 1;
        bool ok = G2 * G3 <= bcap;
        if (ok) {
            // worst-case entries: per axis min(G, w*inv + 2) cells
            double i2 = G2 / r2 * (1.0 + 1e-5), i3 = G3 / r3 * (1.0 + 1e-5);
            double e;
            if (G2 == 1 && G3 == 1) e = z.n;
            else if (G2 == 1) e = sw[2] * i3 + 2.0 * z.n;
            else if (G3 == 1) e = sw[1] * i2 + 2.0 * z.n;
            else e = 4.0 * z.n + 2.0 * (sw[1] * i2 + sw[2] * i3) + sww * i2 * i3;
            ok = e * 1.001 + 64.0 <= ecap;
        }
        if (ok) break;
        s *= 1.1;
        if (it == 399) { G2 = 1; G3 = 1; }
    }
    out.G2 = (uint32_t)G2;
    out.G3 = (uint32_t)G3;
    out.c2_org = (float)(mc[1] - 4.0 * sig[1] - hw[1]);
    out.c3_org = (float)(mc[2] - 4.0 * sig[2] - hw[2]);
    out.c2_inv = (float)(G2 / r2);
    out.c3_inv = (float)(G3 / r3);
    out.n = (uint32_t)z.n;
}

}  // namespace gsap
