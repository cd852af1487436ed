// The small DIIS solve on the device, one warp: shared by the batched 1-D
// solver (batch1d.cu) and the device-resident solve loop of the contexts
// (ctxloop.cu).
#pragma once
#include <cuda_runtime.h>

namespace nm {

// Solve A c = 1 (A: kd×kd in shared memory, row-major with stride kd+1 and
// the right-hand side in column kd) by Gaussian elimination with partial
// pivoting, FP64, one warp.  Same system as SFNewton::Ax (sfnewton.cpp:793).
__device__ inline void warp_solve(double* A, double* c, int kd) {
    const int lane = threadIdx.x & 31;
    const int ld = kd + 1;
    // pivots that rounding made (almost) zero are floored at 1e-30·max|A|
    // (near convergence A ≈ 1e-9·(all ones) is numerically singular; the
    // reference's SVD pseudo-inverse still returns finite coefficients)
    double amax = 0;
    for (int e = lane; e < kd * ld; e += 32)
        if (e % ld < kd) amax = fmax(amax, fabs(A[e]));
    for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    const double tiny = 1e-30 * amax;
    for (int k = 0; k < kd; k++) {
        // pivot: max |A[i][k]| for i >= k
        double best = -1;
        int bi = k;
        for (int i = k + lane; i < kd; i += 32) {
            double v = fabs(A[i * ld + k]);
            if (v > best) { best = v; bi = i; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            double ob = __shfl_down_sync(0xffffffffu, best, o);
            int oi = __shfl_down_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        bi = __shfl_sync(0xffffffffu, bi, 0);
        if (bi != k)
            for (int j = k + lane; j <= kd; j += 32) {
                double t = A[k * ld + j]; A[k * ld + j] = A[bi * ld + j]; A[bi * ld + j] = t;
            }
        __syncwarp();
        double piv = A[k * ld + k];
        if (!(fabs(piv) > tiny)) piv = piv < 0 ? -tiny : tiny;
        __syncwarp();
        if (lane == 0) A[k * ld + k] = piv;
        __syncwarp();
        int rows = kd - k - 1, cols = kd - k;  // columns k+1..kd
        for (int e = lane; e < rows * cols; e += 32) {
            int i = k + 1 + e / cols, j = k + 1 + e % cols;
            A[i * ld + j] -= (A[i * ld + k] / piv) * A[k * ld + j];
        }
        __syncwarp();
    }
    if (lane == 0)
        for (int i = kd - 1; i >= 0; i--) {
            double v = A[i * ld + kd];
            for (int j = i + 1; j < kd; j++) v -= A[i * ld + j] * c[j];
            c[i] = v / A[i * ld + i];
        }
    __syncwarp();
}

}  // namespace nm

namespace nm {

// Solve A c = 1 (A symmetric n×n, row-major in Ain, n ≤ 32) by the
// pseudo-inverse of a cyclic Jacobi eigen-decomposition, c = Q·diag(1/λ)·Qᵀ·1,
// one warp: the host's nm_pinv_solve with the same sweep and rotation order,
// lane k carrying index k of every row, column and eigenvector update, so
// each element sees the same operations in the same order.  a and q are n×n
// shared-memory scratch.  Near convergence, where A ≈ 1e-9·(all ones) is
// numerically singular, the rounding-noise eigenvectors are nearly
// orthogonal to the ones vector and c stays finite (an elimination there can
// divide by a noise pivot).
__device__ inline void warp_pinv_solve(const double* Ain, double* c, int n, double* a, double* q) {
    const int lane = threadIdx.x & 31;
    if (n == 1) {
        if (lane == 0) c[0] = 1.0;
        __syncwarp();
        return;
    }
    for (int e = lane; e < n * n; e += 32) {
        a[e] = Ain[e];
        q[e] = (e / n == e % n) ? 1.0 : 0.0;
    }
    __syncwarp();
    for (int sweep = 0; sweep < 60; sweep++) {
        int stop = 0;
        if (lane == 0) {
            double off = 0, dg = 0;
            for (int i = 0; i < n; i++)
                for (int j = 0; j < n; j++) {
                    const double v = a[i * n + j] * a[i * n + j];
                    if (i == j) dg += v; else off += v;
                }
            stop = (off == 0 || off <= 1e-30 * dg);
        }
        if (__shfl_sync(0xffffffffu, stop, 0)) break;
        for (int p = 0; p < n - 1; p++)
            for (int r = p + 1; r < n; r++) {
                const double apr = a[p * n + r];
                if (apr == 0) continue;  // the same value in every lane
                const double th = (a[r * n + r] - a[p * n + p]) / (2 * apr);
                const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1));
                const double cs = 1 / sqrt(t * t + 1), sn = t * cs;
                __syncwarp();
                if (lane < n) {  // columns p, r
                    const double u = a[lane * n + p], v = a[lane * n + r];
                    a[lane * n + p] = cs * u - sn * v;
                    a[lane * n + r] = sn * u + cs * v;
                }
                __syncwarp();
                if (lane < n) {  // rows p, r
                    const double u = a[p * n + lane], v = a[r * n + lane];
                    a[p * n + lane] = cs * u - sn * v;
                    a[r * n + lane] = sn * u + cs * v;
                }
                if (lane < n) {  // eigenvectors
                    const double u = q[lane * n + p], v = q[lane * n + r];
                    q[lane * n + p] = cs * u - sn * v;
                    q[lane * n + r] = sn * u + cs * v;
                }
                __syncwarp();
            }
    }
    if (lane < n) {
        double ci = 0;
        for (int j = 0; j < n; j++) {
            double proj = 0;  // (Qᵀ·1)_j, in the host's order
            for (int k = 0; k < n; k++) proj += q[k * n + j];
            const double w = proj / a[j * n + j];
            ci += q[lane * n + j] * w;
        }
        c[lane] = ci;
    }
    __syncwarp();
}

}  // namespace nm
