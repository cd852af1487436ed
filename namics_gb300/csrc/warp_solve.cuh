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
