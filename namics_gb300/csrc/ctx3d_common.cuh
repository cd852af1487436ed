// Device helpers shared by the 3-D step kernels (ctx3d.cu) and the
// cluster-resident 3-D sweeps (ctx3dc.cu).  Both paths compute a step and a
// composition update through these same functions, so their FP32 results
// are bit-identical.
#pragma once
#include <cuda_runtime.h>

namespace nm {

// exact 2^e for e <= 127 (0 below 2^-149), selects only
__device__ __forceinline__ float c3_p2f(int e) {
    const int bits = e >= -126 ? (e + 127) << 23 : (e >= -149 ? 1 << max(e + 149, 0) : 0);
    return __int_as_float(bits);
}
__device__ __forceinline__ int c3_expo(float v) {  // frexp exponent of v > 0, 0 for v <= 0
    const int e = ((__float_as_int(v) >> 23) & 0xff) - 126;
    return v > 0.f ? e : 0;
}

// halo coordinate -> the layer set_bounds copies into it (lattice.cpp:94-196)
__device__ __forceinline__ int c3_map(int c, int n, int b1, int bm) {
    return c == 0 ? b1 : (c == n + 1 ? bm : c);
}

// Scale factor of an FP32 step whose input vector has maximum `mx`:
// f = 2^-expo(mx)·(1/6), and the exponent e that the output adds.
__device__ __forceinline__ float c3_scale(float mx, int& e) {
    e = c3_expo(mx);
    return c3_p2f(-e) * (float)(1.0 / 6.0);
}

// One composition update of the FP32 path: ρ += Gf·Gb·d relative to
// 2^E(root), Es = E(Gf) + E(Gb) - E(root), the scale applied half to each
// factor, Kahan-compensated in (rh, rl).
__device__ __forceinline__ void c3_comp(float gf, float v, int Es, float d, float* rh, float* rl) {
    const int h = Es >> 1;
    const float sa = c3_p2f(min(h, 127)), sb = c3_p2f(min(Es - h, 127));
    const float yv = (gf * sa) * (v * sb * d) - *rl;
    const float t2 = *rh + yv;
    *rl = (t2 - *rh) - yv;
    *rh = t2;
}

}  // namespace nm
