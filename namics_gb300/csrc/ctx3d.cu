// 3-D simple-cubic propagator steps for the generic context (melts and other
// 3-gradient planar lattices with linear chains), FP64 or FP32.
//
// One step is G_out(x,y,z) = G1·(Σ of the six neighbours)/6
// (LGrad3::propagate, LGrad3.cpp:673-744, simple-cubic stencil), with the
// halo coordinates mapped to the layers set_bounds copies (mirror, periodic)
// or to the wall slot that holds 0 ('surface').  The grid is (z-chunk,
// y-chunk, x): a block runs 128 consecutive z of RY consecutive y rows,
// so no site index is ever divided, every warp load is 32 consecutive z,
// and the y±1 rows of a block's later rows come from L1.
//
// FP32 (block floating point per vector): every stored vector carries one
// power-of-two exponent E, G_true = G·2^E.  Each step kernel publishes the
// maximum of its output with atomicMax into 32 slots (block id mod 32, so
// same-address atomics do not serialise); the next step reduces the 32
// slots with one warp read, rescales by 2^-expo(max) and records
// E_out = E_in + e.  Nothing returns to the host between steps, so the whole
// residual is captured in a CUDA graph.  A melt's propagators span a few
// binary orders across the box, well inside FP32; the stretched 1-D brushes
// that need per-thread exponents go to the batched solver instead.
//
// Backward steps fuse the composition, ρ += d·Gf·Gb, accumulated in FP32
// with Kahan compensation (rho_hi, rho_lo) relative to 2^E(root) and
// converted once per residual to the FP64 ρ the normalisation reads.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "ctx3d_common.cuh"
#include "ctx_internal.h"

namespace nm {

#define C3_SLOTS 32  // maximum slots per stored vector
// rows along y per block: 2, 4 or 8, the context's c3_rows (4 unless the
// autotuner picks another; measured 4 > 8 > 16 on a 128³ melt)

// Step modes: 0 forward step, 1 forward start (copy G1), 2 backward start
// (copy G1 + composition), 3 backward step (+ composition).
template <typename T, int MODE, int RY>
__global__ void __launch_bounds__(128) k3_prop(L3 L, const T* __restrict__ in, const T* __restrict__ G1,
                                               T* __restrict__ out, unsigned* __restrict__ maxbits,
                                               int* __restrict__ E, int sin, int sout,
                                               const T* __restrict__ Gf, int sgf, int sroot,
                                               T* __restrict__ rhi, T* __restrict__ rlo, T d) {
    nmdev::pdl_begin();
    constexpr bool FP32 = sizeof(T) == 4;
    const int z = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int x = blockIdx.z + 1;
    int e = 0;
    T f = (T)(1.0 / 6.0);
    if (FP32 && (MODE == 0 || MODE == 3)) {
        unsigned mb = maxbits[sin * C3_SLOTS + (threadIdx.x & 31)];
        for (int o = 16; o > 0; o >>= 1) mb = max(mb, __shfl_xor_sync(0xffffffffu, mb, o));
        f = (T)c3_scale(__uint_as_float(mb), e);
    }
    const int Eout = FP32 ? ((MODE == 1 || MODE == 2) ? 0 : E[sin] + e) : 0;
    float vmax = 0.f;
#pragma unroll
    for (int yy = 0; yy < RY; yy++) {
        const int y = blockIdx.y * RY + yy + 1;
        T v = 0;
        if (z <= L.MZ && y <= L.MY) {
            const int s = x * L.JX + y * L.JY + z;
            if (MODE == 1 || MODE == 2) {
                v = G1[s];
            } else {
                const int xm = c3_map(x - 1, L.MX, L.b1x, L.bmx), xp = c3_map(x + 1, L.MX, L.b1x, L.bmx);
                const int ym = c3_map(y - 1, L.MY, L.b1y, L.bmy), yp = c3_map(y + 1, L.MY, L.b1y, L.bmy);
                const int zm = c3_map(z - 1, L.MZ, L.b1z, L.bmz), zp = c3_map(z + 1, L.MZ, L.b1z, L.bmz);
                const int yz = y * L.JY + z, xz = x * L.JX + z, xy = x * L.JX + y * L.JY;
                // summation order of LGrad3::propagate's simple-cubic branch: x pair, y pair, z pair
                T s6 = ((in[xm * L.JX + yz] + in[xp * L.JX + yz]) + (in[xz + ym * L.JY] + in[xz + yp * L.JY])) +
                       (in[xy + zm] + in[xy + zp]);
                v = FP32 ? s6 * f * G1[s] : s6 * (T)(1.0 / 6.0) * G1[s];
            }
            out[s] = v;
            if (MODE >= 2) {
                if constexpr (FP32) {
                    // ρ relative to 2^E(root): Gf·Gb·d·2^(Ef + Eout - Eroot)
                    c3_comp(Gf[s], v, E[sgf] + Eout - E[sroot], d, rhi + s, rlo + s);
                } else {
                    rhi[s] += d == (T)1 ? Gf[s] * v : d * Gf[s] * v;
                }
            }
        }
        vmax = fmaxf(vmax, (float)v);
    }
    if (FP32) {
        // block maximum of the output -> one of its 32 slots
        float m = vmax;
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        __shared__ float wm[4];
        if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int i = 1; i < (int)(blockDim.x >> 5); i++) m = fmaxf(m, wm[i]);
            const int b = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
            if (m > 0.f) atomicMax(&maxbits[sout * C3_SLOTS + (b & (C3_SLOTS - 1))], __float_as_uint(m));
            if (b == 0) E[sout] = Eout;
        }
    }
    nmdev::pdl_end();
}

// The same steps (modes 0 and 3) as a 2.5-D tile: a block owns 128
// consecutive z (plus the two z halo slots) of RY consecutive rows (plus the
// y halo rows) over XC consecutive planes (plus the x halo planes).  It first
// copies that whole slab of `in` into shared memory with asynchronous copies
// (cp.async, every load of the slab in flight at once), then computes its
// RY × XC rows from shared memory.  Each element of `in` is loaded once per
// block instead of up to seven times by the gather kernel, and the six
// neighbours are summed in the same order, so every output is bit-identical
// to k3_prop's.  Halo rows, slots and planes are staged from the layers
// set_bounds copies (c3_map).  Dynamic shared memory: (XC+2)(RY+2)·130
// elements.
__device__ __forceinline__ void c3_cp_async(void* dst, const void* src, int bytes) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if (bytes == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
    else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}

template <typename T, int MODE, int RY, int XC>
__global__ void __launch_bounds__(128) k3_tile(L3 L, const T* __restrict__ in, const T* __restrict__ G1,
                                               T* __restrict__ out, unsigned* __restrict__ maxbits,
                                               int* __restrict__ E, int sin, int sout,
                                               const T* __restrict__ Gf, int sgf, int sroot,
                                               T* __restrict__ rhi, T* __restrict__ rlo, T d) {
    static_assert(MODE == 0 || MODE == 3, "tile steps: forward and backward steps");
    constexpr bool FP32 = sizeof(T) == 4;
    constexpr int W = 130;                 // z slots of a staged row: 128 sites and 2 halo slots
    constexpr int PL = (RY + 2) * W;       // elements of one staged plane
    extern __shared__ __align__(16) unsigned char c3_smem[];
    T* tile = reinterpret_cast<T*>(c3_smem);  // [XC+2][RY+2][W]
    nmdev::pdl_begin();
    const int zc = blockIdx.x * 128;       // z of slot 0 (site z = zc + 1 + threadIdx.x)
    const int y0 = blockIdx.y * RY + 1;
    const int x0 = blockIdx.z * XC + 1;
    const int x1 = min(x0 + XC - 1, L.MX);
    const int np = x1 - x0 + 3;            // planes x0-1 .. x1+1
    for (int i = threadIdx.x; i < np * PL; i += blockDim.x) {
        const int pl = i / PL, rem = i - pl * PL, r = rem / W, zz = rem - r * W;
        const int x = x0 - 1 + pl, y = y0 - 1 + r, z = zc + zz;
        if (y <= L.MY + 1 && z <= L.MZ + 1) {
            const int g = c3_map(x, L.MX, L.b1x, L.bmx) * L.JX + c3_map(y, L.MY, L.b1y, L.bmy) * L.JY +
                          c3_map(z, L.MZ, L.b1z, L.bmz);
            c3_cp_async(tile + i, in + g, (int)sizeof(T));
        } else {
            tile[i] = (T)0;
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    int e = 0;
    T f = (T)(1.0 / 6.0);
    if (FP32) {
        unsigned mb = maxbits[sin * C3_SLOTS + (threadIdx.x & 31)];
        for (int o = 16; o > 0; o >>= 1) mb = max(mb, __shfl_xor_sync(0xffffffffu, mb, o));
        f = (T)c3_scale(__uint_as_float(mb), e);
    }
    const int Eout = FP32 ? E[sin] + e : 0;
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    const int c = threadIdx.x + 1;         // this thread's slot
    const int z = zc + c;
    float vmax = 0.f;
    if (z <= L.MZ) {
        for (int x = x0; x <= x1; x++) {
            const T* pm = tile + (x - x0) * PL;  // plane x-1
            const T* pc = pm + PL;               // plane x
            const T* pp = pc + PL;               // plane x+1
#pragma unroll
            for (int r = 1; r <= RY; r++) {
                const int y = y0 + r - 1;
                if (y > L.MY) break;
                const int s = x * L.JX + y * L.JY + z;
                const T s6 = ((pm[r * W + c] + pp[r * W + c]) + (pc[(r - 1) * W + c] + pc[(r + 1) * W + c])) +
                             (pc[r * W + c - 1] + pc[r * W + c + 1]);
                const T v = FP32 ? s6 * f * G1[s] : s6 * (T)(1.0 / 6.0) * G1[s];
                out[s] = v;
                if (MODE == 3) {
                    if constexpr (FP32) {
                        c3_comp(Gf[s], v, E[sgf] + Eout - E[sroot], d, rhi + s, rlo + s);
                    } else {
                        rhi[s] += d == (T)1 ? Gf[s] * v : d * Gf[s] * v;
                    }
                }
                vmax = fmaxf(vmax, (float)v);
            }
        }
    }
    if (FP32) {
        float m = vmax;
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        __shared__ float wm[4];
        if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int i = 1; i < (int)(blockDim.x >> 5); i++) m = fmaxf(m, wm[i]);
            const int b = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
            if (m > 0.f) atomicMax(&maxbits[sout * C3_SLOTS + (b & (C3_SLOTS - 1))], __float_as_uint(m));
            if (b == 0) E[sout] = Eout;
        }
    }
    nmdev::pdl_end();
}

// Σ_interior of an FP32 vector (FP64 partial sums), G(N) = Σ·2^E(root), and
// the true-scale FP64 ρ
__global__ void k3_wsum32(L3 L, const float* __restrict__ X, double* __restrict__ partial) {
    __shared__ double sh[8];
    double acc = 0;
    const int n = L.MX * L.MY * L.MZ;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int z = i % L.MZ + 1, r = i / L.MZ, y = r % L.MY + 1, x = r / L.MY + 1;
        acc += (double)X[x * L.JX + y * L.JY + z];
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) r += sh[i];
        partial[blockIdx.x] = r;
    }
}
__global__ void k3_gn32(const double* __restrict__ partial, int nb, const int* __restrict__ E, int sroot,
                        double* __restrict__ out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double r = 0;
        for (int i = 0; i < nb; i++) r += partial[i];  // fixed order
        *out = ldexp(r, E[sroot]);
    }
}
__global__ void k3_rho64(L3 L, const float* __restrict__ rhi, const float* __restrict__ rlo, const int* __restrict__ E,
                         int sroot, double* __restrict__ rho) {
    const double f = ldexp(1.0, E[sroot]);
    const int n = L.MX * L.MY * L.MZ;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int z = i % L.MZ + 1, r = i / L.MZ, y = r % L.MY + 1, x = r / L.MY + 1;
        const int s = x * L.JX + y * L.JY + z;
        rho[s] += ((double)rhi[s] + (double)rlo[s]) * f;
    }
}

// ------------------------------------------------------------------ host

L3 make_l3(const nm_plan* p) {
    auto src = [](int bc, int lo, int n) {  // lattice.cpp:94-196 halo source per axis side
        if (bc == NM_BC_MIRROR) return lo ? 1 : n;
        if (bc == NM_BC_PERIODIC) return lo ? n : 1;
        return lo ? 0 : n + 1;
    };
    L3 L;
    L.MX = p->MX; L.MY = p->MY; L.MZ = p->MZ; L.JX = p->JX; L.JY = p->JY;
    L.b1x = src(p->bc[0], 1, p->MX); L.bmx = src(p->bc[3], 0, p->MX);
    L.b1y = src(p->bc[1], 1, p->MY); L.bmy = src(p->bc[4], 0, p->MY);
    L.b1z = src(p->bc[2], 1, p->MZ); L.bmz = src(p->bc[5], 0, p->MZ);
    return L;
}

bool ctx3d_eligible(const nm_plan* p, std::string* why) {
    auto no = [&](const char* w) { if (why) *why = w; return false; };
    if (p->gradients != 3) return no("3-gradient lattices only");
    if (p->charged) return no("charged systems take the generic kernels (their halo composition)");
    if (p->lattice_type != NM_SIMPLE_CUBIC) return no("simple-cubic lattices only");
    if (p->geometry != NM_PLANAR) return no("planar geometry only");
    for (int m = 0; m < p->n_mol; m++) {
        const nm_molecule& mol = p->mols[m];
        for (int b = 0; b < mol.n_blocks; b++) {
            const nm_block& B = mol.blocks[b];
            if (B.n_child > 1 || (B.n_child == 1 && mol.blocks[mol.child_index[B.child0]].mult != 1))
                return no("linear chains only");
        }
    }
    return true;
}

template <typename T, int MODE, int RY, int XC>
static void k3t(Ctx& C, const T* in, const T* G1, T* out, int sin, int sout, const T* Gf, int sgf, int sroot, T* rhi,
                T* rlo, double d) {
    const nm_plan* p = C.plan;
    const size_t smem = sizeof(T) * (size_t)(XC + 2) * (RY + 2) * 130;
    dim3 grid((p->MZ + 127) / 128, (p->MY + RY - 1) / RY, (p->MX + XC - 1) / XC);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(128);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = C.stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = g_plain_launch ? 0 : 1;
    cudaLaunchKernelEx(&cfg, k3_tile<T, MODE, RY, XC>, C.l3, in, G1, out, C.d_maxbits, C.d_E, sin, sout, Gf, sgf,
                       sroot, rhi, rlo, (T)d);
    C.launches++;
}

template <typename T, int MODE>
static void k3(Ctx& C, const T* in, const T* G1, T* out, int sin, int sout, const T* Gf, int sgf, int sroot, T* rhi,
               T* rlo, double d) {
    const nm_plan* p = C.plan;
    if constexpr (MODE == 0 || MODE == 3) {
        // the 2.5-D tile kernel: c3_tile = rows per block × 100 + planes per block
        switch (C.c3_tile) {
            case 204: k3t<T, MODE, 2, 4>(C, in, G1, out, sin, sout, Gf, sgf, sroot, rhi, rlo, d); return;
            case 208: k3t<T, MODE, 2, 8>(C, in, G1, out, sin, sout, Gf, sgf, sroot, rhi, rlo, d); return;
            case 404: k3t<T, MODE, 4, 4>(C, in, G1, out, sin, sout, Gf, sgf, sroot, rhi, rlo, d); return;
            case 408: k3t<T, MODE, 4, 8>(C, in, G1, out, sin, sout, Gf, sgf, sroot, rhi, rlo, d); return;
            default: break;  // 0: the gather kernel
        }
    }
    const int ry = C.c3_rows;
    dim3 grid((p->MZ + 127) / 128, (p->MY + ry - 1) / ry, p->MX);
    if (ry == 2)
        launch_pdl(k3_prop<T, MODE, 2>, grid, 128, C.stream, C.l3, in, G1, out, C.d_maxbits, C.d_E, sin, sout, Gf, sgf,
                   sroot, rhi, rlo, (T)d);
    else if (ry == 8)
        launch_pdl(k3_prop<T, MODE, 8>, grid, 128, C.stream, C.l3, in, G1, out, C.d_maxbits, C.d_E, sin, sout, Gf, sgf,
                   sroot, rhi, rlo, (T)d);
    else
        launch_pdl(k3_prop<T, MODE, 4>, grid, 128, C.stream, C.l3, in, G1, out, C.d_maxbits, C.d_E, sin, sout, Gf, sgf,
                   sroot, rhi, rlo, (T)d);
    C.launches++;
}

// One molecule: forward sweep, G(N), backward sweep fused with the
// composition.  Exponent slots (FP32): forward s -> s, backward s ->
// n_store + s.  Storage: every Gf(s) (ck_stride 0), or with stride k > 1
// (the reference's save_memory, molecule.cpp:2300-2446, as a fixed stride)
// only Gf(s0 + j·k) and each block's last segment; the backward sweep then
// recomputes each group of k segments from the checkpoint that starts it
// into a buffer of k-1 vectors (small enough to stay in L2 on a 128³ box
// at k ≈ 10) with the same step kernel and inputs as the forward sweep, so
// every recomputed vector is bit-identical to the one a full store keeps.
template <typename T>
static int pass3d(Ctx& C, int m) {
    const nm_plan* p = C.plan;
    const nm_molecule& mol = p->mols[m];
    MolDev& D = C.mols[m];
    const size_t M = p->M;
    const int ns = mol.n_store;
    const bool f32 = sizeof(T) == 4;
    T* Gf = f32 ? (T*)D.Gf32 : (T*)D.Gf;
    const int k = C.ck_stride;
    auto vec = [&](size_t j) { return Gf + j * M; };
    // where the forward sweep leaves Gf(s)
    auto fwd = [&](int s) -> T* {
        if (k < 2) return vec(s);
        const int sl = D.slot[s];
        return sl >= 0 ? vec(sl) : vec((size_t)D.n_slots + (k - 1) + (s & 1));
    };
    auto kbuf = [&](int i) { return vec((size_t)D.n_slots + i - 1); };  // i = 1 .. k-1
    const T* G1 = f32 ? (const T*)C.d_G1f : (const T*)C.d_G1;
    T* gb = f32 ? (T*)C.d_gb32 : (T*)C.d_gb;
    T* rhi = f32 ? (T*)D.rho32 : (T*)D.rho;
    T* rlo = f32 ? (T*)D.rho32 + (size_t)mol.n_molmon * M : nullptr;
    if (f32) {
        cudaMemsetAsync(C.d_maxbits, 0, sizeof(unsigned) * 2 * ns * C3_SLOTS, C.stream);
        cudaMemsetAsync(D.rho32, 0, sizeof(float) * 2 * M * mol.n_molmon, C.stream);
    } else {
        cudaMemsetAsync(D.rho, 0, sizeof(double) * M * mol.n_molmon, C.stream);
    }
    const nm_block& R = mol.blocks[mol.n_blocks - 1];
    const int sroot = R.s0 + R.length - 1;
    if constexpr (sizeof(T) == 4) {
        if (C.c3c_on && k < 2) {  // both sweeps in one thread-block cluster each (ctx3dc.cu)
            if (int rc = ctx3dc_sweep(C, m, false, sroot)) return rc;
            const int nb = C.red_blocks;
            k3_wsum32<<<nb, 256, 0, C.stream>>>(C.l3, (const float*)fwd(sroot), C.d_partial);
            k3_gn32<<<1, 32, 0, C.stream>>>(C.d_partial, nb, C.d_E, sroot, C.d_sc + 5 * m);
            C.launches += 2;
            if (int rc = ctx3dc_sweep(C, m, true, sroot)) return rc;
            cudaMemsetAsync(D.rho, 0, sizeof(double) * M * mol.n_molmon, C.stream);
            for (int j = 0; j < mol.n_molmon; j++) {
                k3_rho64<<<4 * 152, 256, 0, C.stream>>>(C.l3, (const float*)rhi + (size_t)j * M,
                                                        (const float*)rlo + (size_t)j * M, C.d_E, sroot,
                                                        D.rho + (size_t)j * M);
                C.launches++;
            }
            return NM_OK;
        }
    }
    for (int b = 0; b < mol.n_blocks; b++) {
        const nm_block& B = mol.blocks[b];
        const T* g1 = G1 + (size_t)B.seg * M;
        if (B.n_child == 0) {
            k3<T, 1>(C, nullptr, g1, fwd(B.s0), 0, B.s0, nullptr, 0, 0, nullptr, nullptr, 1.0);
        } else {
            const nm_block& C0 = mol.blocks[mol.child_index[B.child0]];
            const int sl = C0.s0 + C0.length - 1;
            k3<T, 0>(C, fwd(sl), g1, fwd(B.s0), sl, B.s0, nullptr, 0, 0, nullptr, nullptr, 1.0);
        }
        for (int j = 1; j < B.length; j++) {
            const int s = B.s0 + j;
            k3<T, 0>(C, fwd(s - 1), g1, fwd(s), s - 1, s, nullptr, 0, 0, nullptr, nullptr, 1.0);
        }
    }
    if (f32) {
        int nb = C.red_blocks;
        k3_wsum32<<<nb, 256, 0, C.stream>>>(C.l3, (const float*)fwd(sroot), C.d_partial);
        k3_gn32<<<1, 32, 0, C.stream>>>(C.d_partial, nb, C.d_E, sroot, C.d_sc + 5 * m);
        C.launches += 2;
    } else {
        C.wsum((const double*)fwd(sroot), C.d_sc + 5 * m);
    }
    // backward: a linear chain walks its blocks from the root down, the
    // first segment of each block continuing the previous block's sweep
    int sprev = -1;
    for (int b = mol.n_blocks - 1; b >= 0; b--) {
        const nm_block& B = mol.blocks[b];
        const T* g1 = G1 + (size_t)B.seg * M;
        T* rh = rhi + (size_t)B.molmon * M;
        T* rl = rlo ? rlo + (size_t)B.molmon * M : nullptr;
        const int top = B.s0 + B.length - 1;
        const int kk = k < 2 ? B.length : k;  // group length: the whole block without checkpoints
        for (int c = B.s0 + ((B.length - 1) / kk) * kk; c >= B.s0; c -= kk) {
            const int e = std::min(c + kk - 1, top);
            // the group's forward propagators: stored (k < 2) or recomputed
            // from the checkpoint Gf(c)
            auto gf = [&](int s) -> const T* { return k < 2 || s == c ? fwd(s) : kbuf(s - c); };
            if (k >= 2)
                for (int s = c + 1; s <= e; s++)
                    k3<T, 0>(C, gf(s - 1), g1, kbuf(s - c), s - 1, s, nullptr, 0, 0, nullptr, nullptr, 1.0);
            for (int s = e; s >= c; s--) {
                T* o = gb + (size_t)(s & 1) * M;
                const int so = ns + s;
                if (sprev < 0)
                    k3<T, 2>(C, nullptr, g1, o, 0, so, gf(s), s, sroot, rh, rl, B.degeneracy);
                else
                    k3<T, 3>(C, gb + (size_t)(sprev & 1) * M, g1, o, ns + sprev, so, gf(s), s, sroot, rh, rl,
                             B.degeneracy);
                sprev = s;
            }
        }
    }
    if (f32) {
        cudaMemsetAsync(D.rho, 0, sizeof(double) * M * mol.n_molmon, C.stream);
        for (int k = 0; k < mol.n_molmon; k++) {
            k3_rho64<<<4 * 152, 256, 0, C.stream>>>(C.l3, (const float*)rhi + (size_t)k * M,
                                                    (const float*)rlo + (size_t)k * M, C.d_E, sroot,
                                                    D.rho + (size_t)k * M);
            C.launches++;
        }
    }
    return NM_OK;
}

// The tile kernels' dynamic shared-memory limit (above 48 KB it needs the
// opt-in), on the current device, before any launch or stream capture uses
// the tile.
template <int RY, int XC>
static cudaError_t tile_limits() {
    cudaError_t e = cudaSuccess;
    auto one = [&](auto k, size_t bytes) {
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    };
    one(k3_tile<float, 0, RY, XC>, 4 * (size_t)(XC + 2) * (RY + 2) * 130);
    one(k3_tile<float, 3, RY, XC>, 4 * (size_t)(XC + 2) * (RY + 2) * 130);
    one(k3_tile<double, 0, RY, XC>, 8 * (size_t)(XC + 2) * (RY + 2) * 130);
    one(k3_tile<double, 3, RY, XC>, 8 * (size_t)(XC + 2) * (RY + 2) * 130);
    return e;
}

int ctx3d_set_tile(Ctx& C, int tile) {
    cudaError_t e = cudaSuccess;
    switch (tile) {
        case 0: break;
        case 204: e = tile_limits<2, 4>(); break;
        case 208: e = tile_limits<2, 8>(); break;
        case 404: e = tile_limits<4, 4>(); break;
        case 408: e = tile_limits<4, 8>(); break;
        default: set_error("3-D tile 0, 204, 208, 404 or 408"); return NM_ERR_ARG;
    }
    if (e != cudaSuccess) { set_error(std::string("3-D tile: ") + cudaGetErrorString(e)); return NM_ERR_CUDA; }
    C.c3_tile = tile;
    return NM_OK;
}

int ctx3d_molecule_pass(Ctx& C, int m, bool fp32) {
    return fp32 ? pass3d<float>(C, m) : pass3d<double>(C, m);
}

}  // namespace nm
