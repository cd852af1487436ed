// FP32 propagators for 2-gradient contexts (cylindrical and planar lattices,
// linear chains, neutral or charged), FP64 everything else.
//
// Block floating point with one power-of-two exponent per lattice row x:
// G(x, y) = v(x, y)·2^E[x].  A grafted brush's propagators span hundreds of
// binary orders along x (the chain ends cannot reach far rows), which one
// exponent per vector cannot hold, while along y a row stays within a few
// orders.  A step reads rows x-1, x, x+1 with their exponents, takes the
// largest as its base (the neighbour rows enter scaled by 2^(E_k - base) <= 1,
// so nothing overflows and what underflows is negligible against the larger
// row), multiplies by G1 held in FP32, and renormalises its output row from
// the row maximum: one block per row, the maximum by a block reduction.  A row
// of zeros carries the exponent EMPTY and contributes nothing.
//
// The composition ρ += d·Gf·Gb and G(N) are accumulated in FP64 at true scale
// (2^(Ef + Eb) per row), so normalisation, φ, the residual and the
// electrostatics are the FP64 kernels unchanged.  For charged systems the
// halo part of ρ (the reference's flat-array sums at halo sites, see
// device_common.cuh) is evaluated in FP64 from the scaled FP32 rows.
//
// Steps are graph-captured per-step launches, like the FP64 path: one block
// per row plus, for the halo part, the two x-halo rows.
#include <cuda_runtime.h>

#include <climits>
#include <string>
#include <vector>

#include "ctx_internal.h"

using nmdev::Lat;

namespace nm {

namespace {

constexpr int E2_EMPTY = INT_MIN / 4;

__device__ __forceinline__ float p2f(int e) {  // 2^e for e <= 127, 0 below 2^-149
    const int bits = e >= -126 ? (e + 127) << 23 : (e >= -149 ? 1 << max(e + 149, 0) : 0);
    return __int_as_float(bits);
}
__device__ __forceinline__ int expo_f(float v) {  // frexp exponent of v > 0
    return ((__float_as_int(v) >> 23) & 0xff) - 126;
}
__device__ __forceinline__ double p2d(int e) {  // 2^e in FP64, 0 below 2^-1022
    e = e > 1023 ? 1023 : e;
    return e < -1022 ? 0.0 : __longlong_as_double((long long)(1023 + e) << 52);
}

// block maximum of non-negative floats (bit order = value order)
__device__ __forceinline__ float block_max(float v, unsigned* sh) {
    unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(v));
    const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if ((threadIdx.x & 31) == 0) sh[w] = m;
    __syncthreads();
    unsigned r = sh[0];
    for (int i = 1; i < nw; i++) r = max(r, sh[i]);
    __syncthreads();
    return __uint_as_float(r);
}

// FP32 neighbour sum at (x, y) with the three source rows scaled by fl, fc, fr
// (the same stencils as stencil_at, grouped by row)
__device__ __forceinline__ float sten_rows(const Lat& L, const float* __restrict__ in, int x, int y, float fl,
                                           float fc, float fr) {
    const int JX = L.JX;
    const int xm = nmdev::bmap(x - 1, L.MX, L.b1[0], L.bm[0]), xp = nmdev::bmap(x + 1, L.MX, L.b1[0], L.bm[0]);
    const int ym = nmdev::bmap(y - 1, L.MY, L.b1[1], L.bm[1]), yp = nmdev::bmap(y + 1, L.MY, L.b1[1], L.bm[1]);
    const float c = in[x * JX + y], yl = in[x * JX + ym], yh = in[x * JX + yp];
    const float xl = in[xm * JX + y], dll = in[xm * JX + ym], dlh = in[xm * JX + yp];
    const float xh = in[xp * JX + y], dhl = in[xp * JX + ym], dhh = in[xp * JX + yp];
    if (L.geom == 0) {
        if (L.lat == 0)
            return fc * ((16.f / 36.f) * c + (4.f / 36.f) * (yl + yh)) +
                   fl * ((4.f / 36.f) * xl + (1.f / 36.f) * (dll + dlh)) +
                   fr * ((4.f / 36.f) * xh + (1.f / 36.f) * (dhl + dhh));
        return (fc * (4.f * c + 2.f * (yl + yh)) + fl * (2.f * xl + dll + dlh) + fr * (2.f * xh + dhl + dhh)) *
               (1.f / 16.f);
    }
    float C1, C2, C3;
    if (L.lat == 0) { C1 = 4.f / 6.f; C2 = 1.f / 6.f; C3 = 4.f; }
    else { C1 = 0.5f; C2 = 0.25f; C3 = 2.f; }
    const int s = x * JX + y;
    const float lm = (float)L.lm1[s], lp = (float)L.l1[s];
    return (fc * (C3 * (C1 * c + C2 * (yl + yh))) + fl * (lm * (C3 * xl + dll + dlh)) +
            fr * (lp * (C3 * xh + dhl + dhh))) *
           C2;
}

struct Step32 {
    Lat L;
    const float* in;   // [M] (modes 0, 3)
    const int* Ein;    // [MX+2]
    const float* G1;   // [M] FP32 G1 of the step's segment
    float* out;        // [M]
    int* Eout;         // [MX+2]
    // backward composition (modes 2, 3)
    const float* gf;   // stored forward propagator of this s
    const int* Ef;
    double* rho;       // FP64, true scale
    double d;
    // charged halo part (mode 3)
    int nh;
    const double* G1d; // FP64 G1 (halo sites)
};

// modes: 0 forward step, 1 forward start (G1), 2 backward start (G1 +
// composition), 3 backward step (+ composition).  Block b handles row
// x = b (1..MX); with nh, blocks 0 and MX+1 handle the x-halo rows' ρ.
template <int MODE>
__global__ void __launch_bounds__(1024) k2f_step(Step32 a) {
    __shared__ unsigned sh[32];
    const Lat& L = a.L;
    const int x = blockIdx.x + (a.nh ? 0 : 1);
    const int MY = L.MY, JX = L.JX;
    const int y = threadIdx.x + 1;
    const bool haloRow = x == 0 || x == L.MX + 1;
    int Eb = 0;
    float fl = 0.f, fc = 1.f, fr = 0.f;
    if (MODE == 0 || MODE == 3) {
        const int xm = nmdev::bmap(x - 1 < 0 ? 0 : x - 1, L.MX, L.b1[0], L.bm[0]);
        const int xp = nmdev::bmap(x + 1 > L.MX + 1 ? L.MX + 1 : x + 1, L.MX, L.b1[0], L.bm[0]);
        const int el = a.Ein[xm], ec = a.Ein[x], er = a.Ein[xp];
        Eb = max(el, max(ec, er));
        fl = el == E2_EMPTY ? 0.f : p2f(el - Eb);
        fc = ec == E2_EMPTY ? 0.f : p2f(ec - Eb);
        fr = er == E2_EMPTY ? 0.f : p2f(er - Eb);
    }
    // ---- the row (interior rows only) ----
    float v = 0.f;
    const bool site = !haloRow && y <= MY;
    const int s = x * JX + y;
    if (site) {
        if (MODE == 1 || MODE == 2) v = a.G1[s];
        else if (Eb != E2_EMPTY) v = sten_rows(L, a.in, x, y, fl, fc, fr) * a.G1[s];
    }
    if (!haloRow) {
        const float m = block_max(v, sh);
        const int e = m > 0.f ? expo_f(m) : 0;
        // row maximum to [0.5, 1): e >= -126 (a subnormal maximum reads -126)
        const float w = m > 0.f ? v * p2f(-e) : 0.f;
        const int base = (MODE == 1 || MODE == 2) ? 0 : Eb;
        const int Eo = m > 0.f ? base + e : E2_EMPTY;
        if (site) a.out[s] = w;
        if (threadIdx.x == 0) a.Eout[x] = Eo;
        if (MODE >= 2 && site && Eo != E2_EMPTY) {
            const int ef = a.Ef[x];
            if (ef != E2_EMPTY) {
                const double t = (double)a.gf[s] * (double)w * p2d(ef + Eo);
                if (a.d == 1.0) a.rho[s] += t;
                else a.rho[s] += a.d * t;
            }
        }
    }
    // ---- halo part of ρ (charged systems, backward steps) ----
    if (MODE == 3 && a.nh) {
        int h = -1;
        if (haloRow) { if (threadIdx.x < JX) h = x * JX + threadIdx.x; }
        else if (threadIdx.x == 0) h = x * JX;
        else if (threadIdx.x == 1) h = x * JX + MY + 1;
        // the bounded input in FP64: element i after set_bounds, times its row's scale
        struct Ld {
            const float* p; const int* E; Lat L;
            __device__ double operator()(int i) const {
                const int src = nmdev::bc_source(L, i), e = E[src / L.JX];
                return e == E2_EMPTY ? 0.0 : (double)p[src] * p2d(e);
            }
        };
        if (h >= 0) {
            const Ld bl{a.in, a.Ein, L};
            const double vv = nmdev::flat_prop_at(L, bl, h) * a.G1d[h];
            const int src = nmdev::bc_source(L, h), ef = a.Ef[src / JX];
            const double gfv = ef == E2_EMPTY ? 0.0 : (double)a.gf[src] * p2d(ef);
            if (a.d == 1.0) a.rho[h] += gfv * vv;
            else a.rho[h] += a.d * gfv * vv;
        }
    }
}

// G(N) = Σ_rows 2^E[x]·Σ_y L·v: one block per row, then a fixed-order sum
__global__ void k2f_gn_rows(Lat L, const float* __restrict__ v, const int* __restrict__ E, const double* __restrict__ Lv,
                            double* __restrict__ part) {
    __shared__ double sh[32];
    const int x = blockIdx.x + 1, y = threadIdx.x + 1;
    double acc = 0;
    if (y <= L.MY) {
        const int s = x * L.JX + y;
        acc = Lv ? (double)v[s] * Lv[s] : (double)v[s];
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0;
        for (int i = 0; i < (int)((blockDim.x + 31) >> 5); i++) r += sh[i];
        const int e = E[x];
        part[x - 1] = e == E2_EMPTY ? 0.0 : r * p2d(e);
    }
}
__global__ void k2f_gn_sum(const double* __restrict__ part, int n, double* __restrict__ out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double r = 0;
        for (int i = 0; i < n; i++) r += part[i];
        *out = r;
    }
}

__global__ void k2f_fill(int* p, int n, int v) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = v;
}

}  // namespace

bool ctx2d32_eligible(const nm_plan* p, std::string* why) {
    auto no = [&](const char* w) { if (why) *why = w; return false; };
    if (p->gradients != 2) return no("2-gradient lattices only");
    if (p->MY > 1000) return no("at most 1000 layers along y (one block per row)");
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

int ctx2d32_init(Ctx& C) {
    const nm_plan* p = C.plan;
    const size_t M = p->M, R = (size_t)p->MX + 2;
    auto al = [&](void** q, size_t bytes) {
        if (cudaMallocAsync(q, bytes, C.stream) != cudaSuccess) return false;
        return cudaMemsetAsync(*q, 0, bytes, C.stream) == cudaSuccess;
    };
    if (!al((void**)&C.d_G1f, sizeof(float) * p->n_seg * M) || !al((void**)&C.d_gb32, sizeof(float) * 2 * M) ||
        !al((void**)&C.d_E2b, sizeof(int) * 2 * R) || !al((void**)&C.d_rowpart, sizeof(double) * R)) {
        set_error("cudaMallocAsync (2-D FP32 state)");
        return NM_ERR_NOMEM;
    }
    C.E2f.resize(p->n_mol, nullptr);
    for (int m = 0; m < p->n_mol; m++) {
        const nm_molecule& mol = p->mols[m];
        if (!al((void**)&C.mols[m].Gf32, sizeof(float) * mol.n_store * M) ||
            !al((void**)&C.E2f[m], sizeof(int) * mol.n_store * R)) {
            set_error("cudaMallocAsync (2-D FP32 propagators)");
            return NM_ERR_NOMEM;
        }
    }
    C.use2d32 = true;
    return NM_OK;
}

template <int MODE>
static void step(Ctx& C, Step32& a) {
    const nm_plan* p = C.plan;
    const int blocks = p->MX + (a.nh ? 2 : 0);
    int th = (p->MY + 31) / 32 * 32;
    if (a.nh && th < p->JX) th = (p->JX + 31) / 32 * 32;  // the x-halo rows' JX sites
    k2f_step<MODE><<<blocks, th, 0, C.stream>>>(a);
    C.launches++;
}

int ctx2d32_molecule_pass(Ctx& C, int m) {
    const nm_plan* p = C.plan;
    const nm_molecule& mol = p->mols[m];
    MolDev& D = C.mols[m];
    const size_t M = p->M, R = (size_t)p->MX + 2;
    const int ns = mol.n_store;
    int* Ef = C.E2f[m];
    if (cudaMemsetAsync(D.rho, 0, sizeof(double) * M * mol.n_molmon, C.stream) != cudaSuccess) {
        set_error("cudaMemsetAsync (2-D FP32 composition)");
        return NM_ERR_CUDA;
    }
    // halo rows of every exponent vector are EMPTY unless a step writes them
    k2f_fill<<<(int)((ns * R + 255) / 256), 256, 0, C.stream>>>(Ef, (int)(ns * R), E2_EMPTY);
    k2f_fill<<<1, 256, 0, C.stream>>>(C.d_E2b, (int)(2 * R), E2_EMPTY);
    C.launches += 2;
    std::vector<int> seg(ns), mm(ns);
    std::vector<double> deg(ns);
    for (int b = 0; b < mol.n_blocks; b++) {
        const nm_block& B = mol.blocks[b];
        for (int k = 0; k < B.length; k++) { seg[B.s0 + k] = B.seg; mm[B.s0 + k] = B.molmon; deg[B.s0 + k] = B.degeneracy; }
    }
    Step32 a{};
    a.L = C.lat;
    // forward
    a.nh = 0;
    a.G1 = C.d_G1f + (size_t)seg[0] * M;
    a.out = D.Gf32;
    a.Eout = Ef;
    step<1>(C, a);
    for (int s = 1; s < ns; s++) {
        a.in = D.Gf32 + (size_t)(s - 1) * M;
        a.Ein = Ef + (size_t)(s - 1) * R;
        a.G1 = C.d_G1f + (size_t)seg[s] * M;
        a.out = D.Gf32 + (size_t)s * M;
        a.Eout = Ef + (size_t)s * R;
        step<0>(C, a);
    }
    // G(N)
    const double* Lv = (p->geometry != NM_PLANAR) ? C.d_L : nullptr;
    int th = (p->MY + 31) / 32 * 32;
    k2f_gn_rows<<<p->MX, th, 0, C.stream>>>(C.lat, D.Gf32 + (size_t)(ns - 1) * M, Ef + (size_t)(ns - 1) * R, Lv,
                                           C.d_rowpart);
    k2f_gn_sum<<<1, 32, 0, C.stream>>>(C.d_rowpart, p->MX, C.d_sc + 5 * m);
    C.launches += 2;
    // backward with the composition
    const int top = ns - 1;
    a.G1 = C.d_G1f + (size_t)seg[top] * M;
    a.out = C.d_gb32 + (size_t)(top & 1) * M;
    a.Eout = C.d_E2b + (size_t)(top & 1) * R;
    a.gf = D.Gf32 + (size_t)top * M;
    a.Ef = Ef + (size_t)top * R;
    a.rho = D.rho + (size_t)mm[top] * M;
    a.d = deg[top];
    step<2>(C, a);
    for (int s = top - 1; s >= 0; s--) {
        a.in = C.d_gb32 + (size_t)((s + 1) & 1) * M;
        a.Ein = C.d_E2b + (size_t)((s + 1) & 1) * R;
        a.G1 = C.d_G1f + (size_t)seg[s] * M;
        a.out = C.d_gb32 + (size_t)(s & 1) * M;
        a.Eout = C.d_E2b + (size_t)(s & 1) * R;
        a.gf = D.Gf32 + (size_t)s * M;
        a.Ef = Ef + (size_t)s * R;
        a.rho = D.rho + (size_t)mm[s] * M;
        a.d = deg[s];
        a.nh = C.nh ? 1 : 0;
        a.G1d = C.d_G1 + (size_t)seg[s] * M;
        step<3>(C, a);
        a.nh = 0;
    }
    return NM_OK;
}

}  // namespace nm
