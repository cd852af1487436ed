// Batched 1-gradient SCF solver: one CTA per problem, the whole DIIS solve on
// the device (no host round trip per iteration).
//
// Inside one CTA, per DIIS iteration:
//   G1 = exp(-u)·mask                                 (segment.cpp:855-879)
//   per molecule: forward sweep, G(N), backward sweep fused with the
//   composition rho += d·Gf·Gb; joins for branched / dendrimer blocks
//                                                     (molecule.cpp:2300-2446,
//                                                      mol_branched.cpp:170-299,
//                                                      mol_dendrimer.cpp:113-184)
//   normalisation, φ, φ_side, residual                (system.cpp:2087-2560)
//   x -= δ·g, Gram row, small solve, x = Σ c_i xR_i   (sfnewton.cpp:837-1130)
// The running propagator lives in shared memory; forward propagators are
// stored in global memory (read back in the backward sweep).  Each step is one
// __syncthreads.  Propagators are FP64 (same arithmetic as the reference) or
// FP32 with a per-step power-of-two scale carried as an integer exponent, so
// chains of any length neither underflow nor overflow; composition,
// normalisation, residual and DIIS stay FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "ctx_internal.h"
#include "warp_solve.cuh"

namespace nm {

#define B1_THREADS 128
#define B1_KS 4         // sites per thread in the register path: MX <= 512
#define B1_MAXB 64      // blocks per molecule
#define B1_MAXM 12      // DIIS history in the batched path
// DIIS history of the FP32 phase (the FP64 phase keeps the input's m).  The
// FP32 residuals carry noise near the FP32 floor, and a short history both
// follows it better and makes each iteration's Gram row and small solve
// cheaper: on the 512-instance stream (m = 10) depths 3, 4, 5, 6, 8 and 10 gave
// 10 735, 12 447, 13 291, 12 979–13 107, 12 021 and 10 952 solves/s.
#define B1_M32 5

struct B1Mol {
    int freedom, pinned, n_blocks, n_store, n_molmon, mm0;  // mm0: first (mol, molmon) pair index
    double n_in, theta_in, phibulk_in, N;
    const nm_block* blocks;
    const int* child_index;
    // stored vectors: FP64 [M] (FP64 phase) or FP32 mantissas [128·SP]
    // with one exponent per thread (FP32 phase); same buffers for both
    void* Gf;            // [n_store] vectors
    int* ef;             // [n_store][128] exponents of Gf (FP32 phase)
    void* Pc;            // [n_blocks] vectors: P(Gf of the block's end)·KSAM
    int* epc;            // [n_blocks][128]
    void* Q;             // [n_blocks] vectors: backward start of each block
    int* eq;             // [n_blocks][128]
};

struct B1Prob {
    int MX, M, geom, b1, bm, ns, nit, nmol, solvent, n_mm, m, itlim, max_norm, iv;
    double lam, tol, dmax;
    const double *lm1, *l0, *l1, *L, *ksam, *gmask, *phi_frozen;
    int seg_it[NM_MAX_SEG], seg_frozen[NM_MAX_SEG], seg_inmol[NM_MAX_SEG], it_seg[NM_MAX_SEG];
    double chi[NM_MAX_SEG * NM_MAX_SEG];
    int mm_mol[NM_MAX_MM], mm_seg[NM_MAX_MM];
    double mm_frac[NM_MAX_MM];
    B1Mol mol[NM_MAX_MOL];
    double* x;           // [iv] in/out
    double* g;           // [iv] residual scratch
    double* xR;          // [m*iv]
    double* xx0;         // [m*iv]
    // results
    int iterations, fp32_iterations, status, eval_only;
    double residual, F, Omega, sw_tol, sw_floor;
    unsigned long long t_begin, t_end;  // %globaltimer (ns) at the CTA's start and end
    double sc[5 * NM_MAX_MOL];  // GN, norm, n, theta, phibulk per molecule
    double seg_phibulk[NM_MAX_SEG];
    // byte offsets of the stored propagators and the DIIS history inside a
    // slot of the work loop's scratch (k_batch1d_queue), per molecule
    struct { unsigned long long gf, pc, q, ef, epc, eq; } so[NM_MAX_MOL];
    unsigned long long so_xR, so_xx0;
};

// ---------------------------------------------------------------- helpers
// Hot lattice constants, kept in registers (the descriptor itself lives in
// global memory and would be re-read after every global store otherwise).
struct Lat1 { int MX, M, b1, bm, geom; };
template <typename T> struct Coef { T lam, lmid; const T* lm1; const T* l0; const T* l1; };

// 1-gradient neighbour sum at interior site x (LG1Planar.cpp:138-159,
// LGrad1.cpp:432-454).  WALL: a 'surface' halo is a frozen wall where every
// propagator is 0, so it is not read; otherwise the stored halo value is used
// (φ of a frozen wall segment, for Side()).
template <typename T, bool WALL>
__device__ __forceinline__ T sten1(const Lat1& L, const Coef<T>& C, const T* __restrict__ g, int x) {
    int xm = x - 1 == 0 ? L.b1 : x - 1;
    int xp = x + 1 == L.MX + 1 ? L.bm : x + 1;
    T gm = (WALL && xm == 0) ? (T)0 : g[xm];
    T gp = (WALL && xp == L.MX + 1) ? (T)0 : g[xp];
    if (L.geom == 0) return C.lam * gm + C.lmid * g[x] + C.lam * gp;
    return g[x] * C.l0[x] + gm * C.lm1[x] + gp * C.l1[x];
}

// Branch-free step stencil on a shared-memory propagator whose halo slots hold
// the values set_bounds would copy there (0 at a frozen 'surface' wall).
template <typename T, bool CURV>
__device__ __forceinline__ T stb(const T* __restrict__ g, int x, T lam, T lmid, T cm, T c0, T cp) {
    if (CURV) return g[x] * c0 + g[x - 1] * cm + g[x + 1] * cp;
    return lam * g[x - 1] + lmid * g[x] + lam * g[x + 1];
}

// One FP64 step at x with the site's weights already multiplied by G1
// (aL = λ_-1·G1, aC = λ_0·G1, aR = λ_1·G1): one multiply and two FMAs where
// the neighbour sum followed by the G1 product takes four operations, and
// GB300 issues ~2 FP64 operations per clock per SM.
__device__ __forceinline__ double st3(const double* __restrict__ g, int x, double aL, double aC, double aR) {
    return fma(aR, g[x + 1], fma(aC, g[x], aL * g[x - 1]));
}

__device__ __forceinline__ double b1_block_sum(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double r = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) r += red[i];  // fixed order, every thread
    __syncthreads();
    return r;
}

// exact 2^e without FP64 or library calls, subnormal powers included; 0
// below 2^-149, +inf above 2^127
__device__ __forceinline__ float pow2f(int e) {
    if (e < -149) return 0.f;
    if (e > 127) return __int_as_float(0x7f800000);
    if (e < -126) return __int_as_float(1 << (e + 149));
    return __int_as_float((e + 127) << 23);
}
__device__ __forceinline__ int expo(float v) {  // frexp exponent of v > 0
    int e = ((__float_as_int(v) >> 23) & 0xff) - 126;
    return v > 0.f ? e : 0;
}

}  // namespace nm
namespace nm {
// ---------------------------------------------------------------- kernel
struct B1S {
    double* G1;       // [ns*M] FP64 phase
    double* phi;      // [ns*M]
    double* rho;      // [n_mm*M]
    double* phitot;   // [M]
    double *cur, *nxt;  // [M] FP64 phase
    void* uni;        // start of the region G1/cur/nxt share with the FP32 phase's arrays
    double *red, *Aij, *Ci, *As, *sc, *spb, *gram;
    double* phif;
    int* phie;
    int* eg;
    int* status;
};

// One residual evaluation g(x) (System::Classical_residual) in FP64, the
// reference's arithmetic: G1, forward sweep, backward sweep fused with the
// composition into rho, then b1_finish.
template <bool CURV>
__device__ void b1_residual(B1Prob& P, const Lat1 L, const Coef<double> C, B1S& S, const double* __restrict__ x,
                            double* __restrict__ g) {
    typedef double T;
    const int M = L.M, MX = L.MX, ns = P.ns, n_mm = P.n_mm;
    const int tid = threadIdx.x, nth = blockDim.x;
    T* G1 = S.G1;
    T* rho = S.rho;
    T* cur = S.cur;
    T* nxt = S.nxt;
    double *red = S.red, *sc = S.sc;
    int nk = 0;
    for (int k = 0; k < B1_KS; k++) if (tid + 1 + k * nth <= MX) nk = k + 1;
    // per owned site: curved-lattice weights and the halo slots it feeds
    T cmr[B1_KS], c0r[B1_KS], cpr[B1_KS];
    bool lor[B1_KS], hir[B1_KS];
#pragma unroll
    for (int q = 0; q < B1_KS; q++) {
        int xk = tid + 1 + q * nth;
        bool ok = q < nk;
        cmr[q] = (CURV && ok) ? C.lm1[xk] : (T)0;
        c0r[q] = (CURV && ok) ? C.l0[xk] : (T)0;
        cpr[q] = (CURV && ok) ? C.l1[xk] : (T)0;
        lor[q] = ok && xk == L.b1;          // b1 in 1..MX unless 'surface'
        hir[q] = ok && xk == L.bm;          // bm in 1..MX unless 'surface'
    }
    const T lam = C.lam, lmid = C.lmid;
    if (tid == 0) { cur[0] = cur[MX + 1] = nxt[0] = nxt[MX + 1] = (T)0; }
    // G1 = exp(-u)·mask (PutU + Segment::PrepareForCalculations)
    for (int i = 0; i < ns; i++) {
        int itx = P.seg_it[i];
        const double* gm = P.gmask + i * M;
        for (int s = tid; s < M; s += nth) {
            int src = s == 0 ? L.b1 : (s == MX + 1 ? L.bm : s);
            double u = itx >= 0 ? x[itx * M + src] : 0.0;
            G1[i * M + s] = exp(-u) * gm[s];
        }
    }
    for (int i = tid; i < n_mm * M; i += nth) rho[i] = (T)0;
    __syncthreads();
    for (int m = 0; m < P.nmol; m++) {
        const B1Mol& D = P.mol[m];
        T* __restrict__ Gf = (T*)D.Gf;
        T* __restrict__ Pc = (T*)D.Pc;
        T* __restrict__ Qb = (T*)D.Q;
        // ---- forward sweep (post-order blocks) ----
        for (int b = 0; b < D.n_blocks; b++) {
            const nm_block B = D.blocks[b];
            const T* w = G1 + B.seg * M;
            T wr[B1_KS], aL[B1_KS], aC[B1_KS], aR[B1_KS];
#pragma unroll
            for (int q = 0; q < B1_KS; q++) {
                wr[q] = q < nk ? w[tid + 1 + q * nth] : (T)0;
                aL[q] = (CURV ? cmr[q] : lam) * wr[q];
                aC[q] = (CURV ? c0r[q] : lmid) * wr[q];
                aR[q] = (CURV ? cpr[q] : lam) * wr[q];
            }
            int s = B.s0;
            if (B.n_child == 0) {
#pragma unroll
                for (int q = 0; q < B1_KS; q++)
                    if (q < nk) {
                        int xk = tid + 1 + q * nth;
                        cur[xk] = wr[q];
                        if (lor[q]) cur[0] = wr[q];
                        if (hir[q]) cur[MX + 1] = wr[q];
                        Gf[(size_t)s * M + xk] = wr[q];
                    }
            } else {
                // join: Gf = P(Gf[c0])·G1 · Π_c [P(Gf[c])·KSAM]^mult
                int nc = B.n_child;
                int c0 = D.child_index[B.child0];
                const nm_block C0 = D.blocks[c0];
                bool simple = (nc == 1 && C0.mult == 1);
                if (!simple) {
                    for (int c = 0; c < nc; c++) {
                        int cb = D.child_index[B.child0 + c];
                        const nm_block Cb = D.blocks[cb];
                        int sl = Cb.s0 + Cb.length - 1;
                        for (int xx = tid + 1; xx <= MX; xx += nth)
                            Pc[(size_t)cb * M + xx] = sten1<T, true>(L, C, Gf + (size_t)sl * M, xx) * (T)P.ksam[xx];
                    }
                    __syncthreads();
                }
                int sl0 = C0.s0 + C0.length - 1;
                for (int xx = tid + 1; xx <= MX; xx += nth) {
                    T v = sten1<T, true>(L, C, Gf + (size_t)sl0 * M, xx) * w[xx];
                    if (!simple) {
                        for (int k = 1; k < C0.mult; k++) v = v * Pc[(size_t)c0 * M + xx];
                        for (int c = 1; c < nc; c++) {
                            int cb = D.child_index[B.child0 + c];
                            for (int k = 0; k < D.blocks[cb].mult; k++) v = v * Pc[(size_t)cb * M + xx];
                        }
                    }
                    cur[xx] = v;
                }
                __syncthreads();
                for (int xx = tid + 1; xx <= MX; xx += nth) {
                    Gf[(size_t)s * M + xx] = cur[xx];
                    if (xx == L.b1) cur[0] = cur[xx];
                    if (xx == L.bm) cur[MX + 1] = cur[xx];
                }
            }
            __syncthreads();
            // steps: Gf[s] = P(Gf[s-1])·G1
            for (int k = 1; k < B.length; k++) {
                s++;
                T* __restrict__ gs = Gf + (size_t)s * M;
#pragma unroll
                for (int q = 0; q < B1_KS; q++)
                    if (q < nk) {
                        int xk = tid + 1 + q * nth;
                        T v = st3(cur, xk, aL[q], aC[q], aR[q]);
                        nxt[xk] = v;
                        if (lor[q]) nxt[0] = v;
                        if (hir[q]) nxt[MX + 1] = v;
                        gs[xk] = v;
                    }
                __syncthreads();
                T* t = cur; cur = nxt; nxt = t;
            }
            __syncthreads();
        }
        // ---- G(N) = Σ Gf[root]·L (ComputeGN) ----
        const nm_block Rb = D.blocks[D.n_blocks - 1];
        int sroot = Rb.s0 + Rb.length - 1;
        {
            double acc = 0;
            for (int xx = tid + 1; xx <= MX; xx += nth) {
                double v = Gf[(size_t)sroot * M + xx];
                acc += P.L ? v * P.L[xx] : v;
            }
            double GN = b1_block_sum(acc, red);
            if (tid == 0) { sc[5 * m + 0] = GN; sc[5 * m + 3] = 0.0; }
        }
        // ---- backward sweep fused with composition (pre-order) ----
        int stack[B1_MAXB];
        int sp = 0;
        stack[sp++] = D.n_blocks - 1;
        while (sp > 0) {
            int b = stack[--sp];
            const nm_block B = D.blocks[b];
            const T* w = G1 + B.seg * M;
            T* rr = rho + (D.mm0 + B.molmon) * M;
            const T d = (T)B.degeneracy;
            const bool d1 = B.degeneracy == 1.0;
            T wr[B1_KS], acc[B1_KS], gfn[B1_KS], aL[B1_KS], aC[B1_KS], aR[B1_KS];
#pragma unroll
            for (int q = 0; q < B1_KS; q++) {
                wr[q] = q < nk ? w[tid + 1 + q * nth] : (T)0;
                aL[q] = (CURV ? cmr[q] : lam) * wr[q];
                aC[q] = (CURV ? c0r[q] : lmid) * wr[q];
                aR[q] = (CURV ? cpr[q] : lam) * wr[q];
                acc[q] = (T)0;
            }
            int s = B.s0 + B.length - 1;
            if (B.parent < 0) {
#pragma unroll
                for (int q = 0; q < B1_KS; q++)
                    if (q < nk) {
                        cur[tid + 1 + q * nth] = wr[q];
                        if (lor[q]) cur[0] = wr[q];
                        if (hir[q]) cur[MX + 1] = wr[q];
                    }
            } else {
                const T* q0 = Qb + (size_t)b * M;
#pragma unroll
                for (int q = 0; q < B1_KS; q++)
                    if (q < nk) {
                        int xk = tid + 1 + q * nth;
                        T v = sten1<T, true>(L, C, q0, xk) * wr[q];
                        cur[xk] = v;
                        if (lor[q]) cur[0] = v;
                        if (hir[q]) cur[MX + 1] = v;
                    }
            }
            __syncthreads();
            {   // top segment of the block
                const T* gsrc = Gf + (size_t)s * M;
#pragma unroll
                for (int q = 0; q < B1_KS; q++)
                    if (q < nk) acc[q] = gsrc[tid + 1 + q * nth] * cur[tid + 1 + q * nth] * d;
            }
            // prefetch the stored forward propagator of the next segment
            if (s - 1 >= B.s0) {
                const T* gsrc = Gf + (size_t)(s - 1) * M;
#pragma unroll
                for (int q = 0; q < B1_KS; q++) gfn[q] = q < nk ? gsrc[tid + 1 + q * nth] : (T)0;
            }
            for (s = s - 1; s >= B.s0; s--) {
                T gf[B1_KS];
#pragma unroll
                for (int q = 0; q < B1_KS; q++) gf[q] = gfn[q];
                if (s - 1 >= B.s0) {
                    const T* gsrc = Gf + (size_t)(s - 1) * M;
#pragma unroll
                    for (int q = 0; q < B1_KS; q++) if (q < nk) gfn[q] = gsrc[tid + 1 + q * nth];
                }
#pragma unroll
                for (int q = 0; q < B1_KS; q++)
                    if (q < nk) {
                        int xk = tid + 1 + q * nth;
                        T v = st3(cur, xk, aL[q], aC[q], aR[q]);
                        nxt[xk] = v;
                        if (lor[q]) nxt[0] = v;
                        if (hir[q]) nxt[MX + 1] = v;
                        // ρ += d·Gf·Gb in plain FP64, the reference's sum
                        // (GB300 issues ~2 FP64 operations per clock per SM:
                        // this loop is bound by them)
                        if (d1) acc[q] = fma(gf[q], v, acc[q]);
                        else acc[q] = fma(gf[q] * v, d, acc[q]);
                    }
                __syncthreads();
                T* t = cur; cur = nxt; nxt = t;
            }
#pragma unroll
            for (int q = 0; q < B1_KS; q++)
                if (q < nk) rr[tid + 1 + q * nth] += acc[q];
            __syncthreads();
            if (B.n_child == 0) continue;
            // backward starts of the children: Q = Gb(join)·Π other P(Gf)
            for (int c = 0; c < B.n_child; c++) {
                int cb = D.child_index[B.child0 + c];
                bool simple = (B.n_child == 1 && D.blocks[cb].mult == 1);
                T* q = Qb + (size_t)cb * M;
                for (int xx = tid + 1; xx <= MX; xx += nth) {
                    T v = cur[xx];
                    if (!simple) {
                        for (int k = 1; k < D.blocks[cb].mult; k++) v = v * Pc[(size_t)cb * M + xx];
                        for (int o = 0; o < B.n_child; o++) {
                            if (o == c) continue;
                            int ob = D.child_index[B.child0 + o];
                            for (int k = 0; k < D.blocks[ob].mult; k++) v = v * Pc[(size_t)ob * M + xx];
                        }
                    }
                    q[xx] = v;
                }
            }
            __syncthreads();
            for (int c = B.n_child - 1; c >= 0; c--) stack[sp++] = D.child_index[B.child0 + c];
        }
        __syncthreads();
    }
}

// Normalisation, φ, φ_tot and the residual (system.cpp:2324-2560 and
// System::Classical_residual, system.cpp:2087-2189), FP64, from rho in the
// natural site layout [n_mm][M] and G(N) in sc[5m].
//  SCALED = false: rho = Σ Gf·Gb (divided by G1 here), sc[5m] = G(N).
//  SCALED = true (FP32 phase): rho already divided by G1 and, like G(N),
//  stored relative to 2^e with e = sc[5m+3]: rho_true = rho·2^e,
//  G(N)_true = sc[5m]·2^e.  Restricted chains use n/GNm (the 2^e cancel);
//  free chains and the solvent carry φb/N·2^e.
template <bool SCALED>
__device__ __noinline__ void b1_finish(B1Prob& P, const Lat1 L, const Coef<double> C, B1S& S, const double* __restrict__ x,
                          double* __restrict__ g) {
    typedef double R;
    const int M = L.M, MX = L.MX, ns = P.ns, nit = P.nit, n_mm = P.n_mm;
    const int tid = threadIdx.x, nth = blockDim.x;
    const double* G1 = S.G1;
    R* phi = S.phi;
    R* rho = S.rho;
    R* phitot = S.phitot;
    double *sc = S.sc, *spb = S.spb;
    // ---- normalisation (system.cpp:2368-2560), one thread ----
    if (tid == 0) {
        double Bsum = 0;
        for (int m = 0; m < P.nmol; m++) {
            const B1Mol& D = P.mol[m];
            double* s5 = sc + 5 * m;
            double GNm = s5[0];
            int e = SCALED ? (int)s5[3] : 0;
            double GN = SCALED ? ldexp(GNm, e) : GNm;
            double norm = 0, fac = 0;
            int pe = 0;
            s5[0] = GN;
            s5[2] = D.n_in; s5[3] = D.theta_in;
            if (D.freedom == NM_MOL_FREE) {
                s5[4] = D.phibulk_in;
                norm = D.phibulk_in / D.N;
                s5[2] = norm * GN;
                Bsum += D.phibulk_in;
                fac = norm; pe = e;
            } else if (D.freedom == NM_MOL_RESTRICTED) {
                if (GNm > 0) {
                    norm = D.n_in / GN;
                    fac = SCALED ? D.n_in / GNm : norm;
                    if (D.pinned) s5[4] = 0;
                    else { s5[4] = D.N * norm; Bsum += s5[4]; }
                } else if (*S.status == 0) *S.status = NM_ERR_GN;
            } else { s5[4] = 0; pe = e; }
            s5[1] = norm;
            S.phif[m] = fac > 0 ? fac : 1.0;
            S.phie[m] = pe;
        }
        if (P.solvent >= 0) {
            int sv = P.solvent;
            double* s5 = sc + 5 * sv;
            s5[4] = 1.0 - Bsum;
            if (s5[4] < 0 && *S.status == 0) *S.status = NM_ERR_NEG_SOLVENT;
            double norm = s5[4] / P.mol[sv].N;
            s5[2] = norm * s5[0];
            s5[3] = s5[2] * P.mol[sv].N;
            s5[1] = norm;
            S.phif[sv] = norm > 0 ? norm : 1.0;
        }
        for (int i = 0; i < ns; i++) spb[i] = 0;
        for (int k = 0; k < n_mm; k++) spb[P.mm_seg[k]] += P.mm_frac[k] * sc[5 * P.mm_mol[k] + 4];
    }
    __syncthreads();
    // ---- φ = rho/G1·norm, φ_tot ----
    R mmf[NM_MAX_MM];
    for (int k = 0; k < n_mm; k++) {
        int m = P.mm_mol[k];
        mmf[k] = SCALED ? ldexp(S.phif[m], S.phie[m]) : S.phif[m];
    }
    for (int s = tid; s < M; s += nth) {
        bool in = s >= 1 && s <= MX;
        R pt = 0;
        for (int i = 0; i < ns; i++) {
            R v = (R)P.phi_frozen[i * M + s];
            phi[i * M + s] = v;
            if (P.seg_frozen[i]) pt += v;
        }
        if (in)
            for (int k = 0; k < n_mm; k++) {
                int sg = P.mm_seg[k];
                R v;
                if (SCALED) v = rho[k * M + s];
                else {
                    R g1 = G1[sg * M + s];
                    v = g1 != (R)0 ? rho[k * M + s] / g1 : (R)0;
                }
                v *= mmf[k];
                phi[sg * M + s] += v;
                pt += v;
            }
        phitot[s] = pt;
    }
    __syncthreads();
    // ---- residual (Classical_residual) ----
    R chir[NM_MAX_SEG * NM_MAX_SEG];
    for (int i = 0; i < nit; i++)
        for (int k = 0; k < ns; k++) chir[i * ns + k] = (R)P.chi[P.it_seg[i] * ns + k];
    R spbr[NM_MAX_SEG];
    for (int k = 0; k < ns; k++) spbr[k] = (R)spb[k];
    R rinv = (R)(1.0 / nit);
    for (int s = tid; s < M; s += nth) {
        if (s < 1 || s > MX) {
            for (int i = 0; i < nit; i++) g[i * M + s] = 0;
            continue;
        }
        R ps[NM_MAX_SEG];
        for (int k = 0; k < ns; k++) ps[k] = sten1<R, false>(L, C, phi + k * M, s);
        R pt = phitot[s];
        R gi[NM_MAX_SEG];
        R al = 0;
        for (int i = 0; i < nit; i++) {
            R v = (R)x[i * M + s];
            for (int k = 0; k < ns; k++) {
                R chi = chir[i * ns + k];
                if (chi != (R)0 && pt > (R)0) v = v - chi * (ps[k] / pt - spbr[k]);
            }
            gi[i] = v;
            al += v;
        }
        al = al * rinv;
        R km = (R)P.ksam[s];
        for (int i = 0; i < nit; i++) {
            R v = pt > (R)0 ? gi[i] - al + (R)1 / pt - (R)1 : (R)0;
            g[i * M + s] = (double)(v * km);
        }
    }
    __syncthreads();
}

}  // namespace nm
#include "batch1d_bfp.cuh"
namespace nm {

// Shared memory of k_batch1d, in doubles (host and device agree on it):
// tail arrays phi [ns·M], rho [n_mm·M], phitot [M]; then one region shared by
// the FP64 phase (G1 [ns·M], cur [M], nxt [M]) and the FP32 phase (G1s, rhos
// [ns+n_mm][Wl] and three weight rows of Wl floats, Wl = 128·SP); then
// reduction and DIIS scratch.
__host__ __device__ inline int b1_sp(int MX) {  // sites per thread: 1 to 4 (MX <= 512)
    return (MX + BC_NT - 1) / BC_NT;
}
__host__ __device__ inline size_t b1_uni_doubles(int ns, int n_mm, int M, int MX) {
    size_t f64 = (size_t)(ns + 2) * M;
    size_t f32 = ((size_t)(ns + n_mm + 3) * BC_NT * b1_sp(MX) + 1) / 2;
    return f64 > f32 ? f64 : f32;
}
__host__ __device__ inline size_t b1_smem_doubles(int ns, int n_mm, int M, int MX) {
    return (size_t)(ns + n_mm + 1) * M + b1_uni_doubles(ns, n_mm, M, MX) + 64 +
           B1_MAXM * B1_MAXM + B1_MAXM + B1_MAXM * (B1_MAXM + 1) + 5 * NM_MAX_MOL + NM_MAX_SEG + B1_MAXM;
}

// FP32 residual: sites per thread, curved lattice, periodic bounds
__device__ __noinline__ void bc_dispatch(B1Prob& P, const Lat1 L, const Coef<double> C64, B1S& S, BcX& X,
                                         const double* __restrict__ x, double* __restrict__ g, int sp) {
    const bool cv = L.geom != 0, per = (L.b1 == L.MX && L.bm == 1 && L.MX > 1);
#define BC_CALL(SPV)                                                             \
    if (cv) {                                                                    \
        if (per) bc_residual<SPV, true, true>(P, L, C64, S, X, x, g);            \
        else bc_residual<SPV, true, false>(P, L, C64, S, X, x, g);               \
    } else {                                                                     \
        if (per) bc_residual<SPV, false, true>(P, L, C64, S, X, x, g);           \
        else bc_residual<SPV, false, false>(P, L, C64, S, X, x, g);              \
    }
    switch (sp) {
        case 1: BC_CALL(1) break;
        case 2: BC_CALL(2) break;
        case 3: BC_CALL(3) break;
        default: BC_CALL(4) break;
    }
#undef BC_CALL
}

// One CTA per problem: residual + DIIS until ‖g‖ < tol or the iteration limit
// (Solve_scf / SFNewton::iterate_DIIS, sfnewton.cpp:1037-1130).
// mode 0: FP64 throughout, the reference's arithmetic.
// mode 1: FP32 block-floating-point propagators (batch1d_bfp.cuh) until
//   ‖g‖ < P.sw_tol, or a stall close to convergence, then FP64 in the same
//   CTA with the DIIS history restarted, so the stopping test ‖g‖ < tol is
//   always made on an FP64 residual.  A failure of the FP32 evaluation
//   (G(N) <= 0, a non-finite residual) is a failure of the reduced precision,
//   says nothing about the problem itself: the FP64 phase takes over at the same x.
__device__ __forceinline__ unsigned long long b1_clock() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The whole solve of one problem by one CTA (the body of both kernels below).
__device__ __forceinline__ void b1_solve(B1Prob& P, const int mode) {
    if (threadIdx.x == 0) P.t_begin = b1_clock();
    extern __shared__ double sm[];
    const int M = P.M, ns = P.ns, iv = P.iv, n_mm = P.n_mm, m = P.m;
    int mm = m;  // the DIIS depth of the current phase (B1_M32 in the FP32 phase)
    const int tid = threadIdx.x, nth = blockDim.x;
    const Lat1 L{P.MX, P.M, P.b1, P.bm, P.geom};
    B1S S;
    double* q = sm;
    S.phi = q; q += ns * M;
    S.rho = q; q += n_mm * M;
    S.phitot = q; q += M;
    S.uni = q;
    S.G1 = q;
    S.cur = q + ns * M;
    S.nxt = q + (ns + 1) * M;
    q += b1_uni_doubles(ns, n_mm, M, P.MX);
    S.red = q; q += 64;
    S.Aij = q; q += B1_MAXM * B1_MAXM;
    S.Ci = q; q += B1_MAXM;
    S.As = q; q += B1_MAXM * (B1_MAXM + 1);
    S.sc = q; q += 5 * NM_MAX_MOL;
    S.spb = q; q += NM_MAX_SEG;
    S.gram = q; q += B1_MAXM;
    __shared__ int sh_status;
    __shared__ double phif[NM_MAX_MOL];
    __shared__ int phie[NM_MAX_MOL];
    __shared__ int egs[NM_MAX_SEG];
    __shared__ BcX bcx;
    S.phif = phif; S.phie = phie; S.status = &sh_status; S.eg = egs;
    double* __restrict__ x = P.x;
    double* __restrict__ g = P.g;
    double *red = S.red, *Aij = S.Aij, *Ci = S.Ci;
    const Coef<double> C64{P.lam, 1.0 - 2.0 * P.lam, P.lm1, P.l0, P.l1};
    for (int i = tid; i < B1_MAXM * B1_MAXM; i += nth) Aij[i] = 0;
    if (tid == 0) sh_status = 0;
    __syncthreads();

    bool use32 = mode == 1;
    if (use32 && B1_M32 < m) mm = B1_M32;
    const int sp32 = b1_sp(P.MX);
    int it = 0, k_diis = 0, fp32_its = 0;
    double resid = 0, best = 1e300;
    int since_best = 0;
    for (;;) {
        if (use32) {
            bc_dispatch(P, L, C64, S, bcx, x, g, sp32);
            fp32_its++;
            if (sh_status && !P.eval_only) {  // reduced precision failed: FP64 from here
                __syncthreads();
                if (tid == 0) sh_status = 0;
                use32 = false;
                mm = m;
                k_diis = 0;
                __syncthreads();
                continue;
            }
        } else {
            if (L.geom == 0) b1_residual<false>(P, L, C64, S, x, g);
            else b1_residual<true>(P, L, C64, S, x, g);
            b1_finish<false>(P, L, C64, S, x, g);
        }
        if (sh_status || P.eval_only) break;
        // ---------------- DIIS (iterate_DIIS / DIIS / Ax), FP64 ----------------
        int k = it % mm;
        double* __restrict__ xRk = P.xR + (size_t)k * iv;
        double* __restrict__ xxk = P.xx0 + (size_t)k * iv;
        // ‖g‖ first: a non-finite FP32 residual must leave x as it was
        double gsq = 0;
        for (int i = tid; i < iv; i += nth) {
            double gv = g[i];
            gsq = P.max_norm ? fmax(gsq, fabs(gv)) : gsq + gv * gv;
        }
        if (P.max_norm) {
            for (int o = 16; o > 0; o >>= 1) gsq = fmax(gsq, __shfl_down_sync(0xffffffffu, gsq, o));
            __syncthreads();
            if ((tid & 31) == 0) red[tid >> 5] = gsq;
            __syncthreads();
            resid = 0;
            for (int i = 0; i < nth / 32; i++) resid = fmax(resid, red[i]);
            __syncthreads();
        } else resid = sqrt(b1_block_sum(gsq, red));
        if (use32 && !isfinite(resid)) {
            use32 = false;
            mm = m;
            k_diis = 0;
            continue;
        }
        for (int i = tid; i < iv; i += nth) {
            double xo = x[i];
            double xn = xo + (-P.dmax) * g[i];
            x[i] = xn;
            xRk[i] = xn;
            xxk[i] = xn - xo;
        }
        __syncthreads();
        if (it > 0) k_diis++;  // iteration 0 is the plain mixing step
        if (k_diis > 0) {
            int kd = k_diis > mm ? mm : k_diis;
            // Gram row: warp w takes histories i = w, w+4, ...
            int w = tid >> 5, l = tid & 31;
            for (int i = w; i < kd; i += nth / 32) {
                int posi = k - kd + 1 + i;
                if (posi < 0) posi += mm;
                const double* a = P.xx0 + (size_t)posi * iv;
                double acc = 0;
                for (int j = l; j < iv; j += 32) acc += a[j] * xxk[j];
                for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
                if (l == 0) S.gram[i] = acc;
            }
            __syncthreads();
            if (w == 0) {
                if (l == 0) {
                    if (k_diis > mm)
                        for (int i = 1; i < mm; i++)
                            for (int j = 1; j < mm; j++) Aij[mm * (i - 1) + j - 1] = Aij[mm * i + j];
                    for (int i = 0; i < kd; i++) Aij[i + mm * (kd - 1)] = Aij[kd - 1 + mm * i] = S.gram[i] + 1e-9;
                }
                __syncwarp();
                bool nan = false;
                for (int e = l; e < kd * kd; e += 32) {
                    int i = e / kd, j = e % kd;
                    double v = Aij[j + mm * i];
                    if (v != v) nan = true;
                    S.As[i * (kd + 1) + j] = v;
                }
                for (int i = l; i < kd; i += 32) S.As[i * (kd + 1) + kd] = 1.0;
                nan = __any_sync(0xffffffffu, nan);
                __syncwarp();
                if (nan) { if (l == 0) sh_status = NM_ERR_NAN_DIIS; }
                else {
                    if (kd == 1) { if (l == 0) Ci[0] = 1.0; }
                    else warp_solve(S.As, Ci, kd);
                    if (l == 0) {
                        double nC = 0;
                        for (int i = 0; i < kd; i++) nC += Ci[i];
                        for (int i = 0; i < kd; i++) {
                            Ci[i] = Ci[i] / nC;
                            if (Ci[i] != Ci[i]) sh_status = NM_ERR_NAN_SVD;
                        }
                    }
                }
            }
            __syncthreads();
            if (sh_status) break;
            for (int j = tid; j < iv; j += nth) {
                double v = 0;
                for (int i = 0; i < kd; i++) {
                    int posi = k - kd + 1 + i;
                    if (posi < 0) posi += mm;
                    v += Ci[i] * P.xR[(size_t)posi * iv + j];
                }
                x[j] = v;
            }
            __syncthreads();
        }
        if (use32) {
            // Leave the FP32 phase at the switch tolerance; at the FP32
            // accuracy floor sw_floor (~1e-7 per chain segment: below it a
            // residual is noise, so FP32 steps gain nothing more); on a stall
            // near the floor (DIIS stops making progress); or on a long stall
            // close to convergence.  Instances far from convergence stay in
            // FP32.
            if (resid < 0.9 * best) { best = resid; since_best = 0; } else since_best++;
            if (!(resid > P.sw_tol) || !(resid > P.sw_floor) || (since_best > 10 && resid < 10.0 * P.sw_floor) ||
                (since_best > 25 && resid < 1e-2)) {
                use32 = false;
                mm = m;
                k_diis = 0;  // restart the DIIS history on the FP64 residual
                if (it >= P.itlim) break;
                it++;
                continue;
            }
        } else if (!(resid > P.tol)) {
            break;
        }
        if (it >= P.itlim) break;
        it++;
    }
    if (tid == 0) {
        P.t_end = b1_clock();
        P.iterations = it;
        P.fp32_iterations = fp32_its;
        P.residual = resid;
        P.status = sh_status ? sh_status : (resid > P.tol || use32 ? NM_ERR_NOT_CONVERGED : NM_OK);
        for (int i = 0; i < 5 * P.nmol; i++) P.sc[i] = S.sc[i];
        for (int i = 0; i < ns; i++) P.seg_phibulk[i] = S.spb[i];
    }
}

// One CTA per problem: CTA b solves problem order[b] (order may be null).
// Three CTAs per SM (168 registers a thread): at four (128 registers) the
// FP32 residual spilled inside its step loops and a batch took 8% longer;
// at two the batch time is the same and the median solve waits longer.
__global__ void __launch_bounds__(B1_THREADS, 3) k_batch1d(B1Prob* __restrict__ probs, int mode,
                                                          const int* __restrict__ order) {
    b1_solve(probs[order ? order[blockIdx.x] : blockIdx.x], mode);
}

// The device-resident work loop: a persistent grid of resident CTAs, one per
// slot.  Each CTA takes the next problem from the queue (atomic head over
// order[0..n)), points the problem's stored propagators and DIIS history at
// its slot's scratch, solves it to convergence and takes the next one at
// once, so a long or non-converging problem holds one slot, not the batch.
// The batch lists its problems by descending steps per residual, so the
// longest solves start first.
__device__ __forceinline__ void b1_rebase(B1Prob& P, unsigned char* base) {
    for (int m = 0; m < P.nmol; m++) {
        B1Mol& D = P.mol[m];
        D.Gf = base + P.so[m].gf;
        D.Pc = base + P.so[m].pc;
        D.Q = base + P.so[m].q;
        D.ef = (int*)(base + P.so[m].ef);
        D.epc = (int*)(base + P.so[m].epc);
        D.eq = (int*)(base + P.so[m].eq);
    }
    P.xR = (double*)(base + P.so_xR);
    P.xx0 = (double*)(base + P.so_xx0);
}

// MINB resident CTAs per SM: 3 (168 registers a thread) or 4 (128); the
// autotuner picks the slot count, and with it the variant.
template <int MINB>
__global__ void __launch_bounds__(B1_THREADS, MINB) k_batch1d_queue(B1Prob* __restrict__ probs, int n, int mode,
                                                                   const int* __restrict__ order,
                                                                   unsigned char* __restrict__ slots,
                                                                   unsigned long long slot_bytes,
                                                                   unsigned int* __restrict__ head) {
    __shared__ unsigned int s_idx;
    unsigned char* base = slots + (size_t)blockIdx.x * slot_bytes;
    for (;;) {
        if (threadIdx.x == 0) s_idx = atomicAdd(head, 1u);
        __syncthreads();
        const unsigned int idx = s_idx;
        if (idx >= (unsigned int)n) break;  // the same idx in every thread
        B1Prob& P = probs[order ? order[idx] : (int)idx];
        if (threadIdx.x == 0) b1_rebase(P, base);
        __syncthreads();
        b1_solve(P, mode);
        __syncthreads();  // every thread is done with s_idx and the slot
    }
}

// ------------------------------------------------------------------ host
// Accuracy floor of an FP32-propagator residual: G1 held in FP32 is the exact
// G1 of a field perturbed by ~6e-8 per site, which a chain of N segments
// answers with a change of φ (and of the residual) up to ~N·6e-8.
static double b1_fp32_floor(const nm_plan* P) {
    double n = 1;
    for (int m = 0; m < P->n_mol; m++) n = std::max(n, P->mols[m].chainlength);
    return 1e-7 * n + 1e-6;
}

struct Batch {
    std::vector<const nm_plan*> plans;
    std::vector<B1Prob> hp;
    B1Prob* d_probs = nullptr;
    int* d_order = nullptr;  // queue order: longest solves first
    unsigned char* d_slots = nullptr;  // work-loop scratch, slots × slot_bytes
    unsigned int* d_head = nullptr;    // work-loop queue head
    size_t slot_bytes = 0;
    int slots = 0;                     // resident CTAs of the work loop
    std::vector<void*> allocs;
    double* d_x = nullptr;
    double* d_g = nullptr;
    std::vector<long long> offsets;
    int precision = NM_FP64;
    int slots_cap = 0;  // slots the scratch holds: as many CTAs as fit, at most one per problem
    int per_sm3 = 0;    // CTAs per SM of the 168-register variant
    size_t smem = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    long long launches = 0;

    // stream-ordered device memory (see nm_pool_setup): no device-wide
    // synchronisation when a batch is created or destroyed
    template <typename X>
    int alloc(X** p, size_t n) {
        if (n == 0) n = 1;
        cudaError_t e = cudaMallocAsync((void**)p, sizeof(X) * n, stream);
        if (e != cudaSuccess) { set_error(std::string("cudaMallocAsync: ") + cudaGetErrorString(e)); return NM_ERR_NOMEM; }
        allocs.push_back((void*)*p);
        cudaMemsetAsync(*p, 0, sizeof(X) * n, stream);
        return NM_OK;
    }
    template <typename X>
    int upload(X** p, const X* h, size_t n) {
        int rc = alloc(p, n);
        if (rc) return rc;
        // pageable source: staged before the call returns, so h may go away
        cudaError_t e = cudaMemcpyAsync(*p, h, sizeof(X) * n, cudaMemcpyHostToDevice, stream);
        if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
        return NM_OK;
    }
    ~Batch() {
        for (void* p : allocs) cudaFreeAsync(p, stream);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
};

#define TRYB(x) do { int r_ = (x); if (r_) return r_; } while (0)

struct StreamEntry;
struct StreamCtl;
__global__ void k_stream1d(StreamEntry* ring, double* xring, int cap, int iv_max, StreamCtl* ctl,
                           unsigned long long* head, unsigned char* slots, unsigned long long slot_bytes,
                           B1Prob* priv, double* xpriv, double* gpriv, unsigned long long idle_ns,
                           const unsigned char* blobs, unsigned char* cpriv, unsigned long long blob_max);

// Raise the dynamic shared-memory limit of k_batch1d, k_batch1d_queue and
// k_stream1d on device `dev` (current) to at least `bytes`.  The limit only ever rises, and every path that launches
// k_batch1d (batches, the server's workers, the allocation-free solve) goes
// through this one lock, so no caller can lower it under another's launch.
static cudaError_t b1_raise_smem(int dev, size_t bytes) {
    static std::mutex mu;
    static size_t set[64] = {};
    std::lock_guard<std::mutex> lk(mu);
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (bytes <= set[dev]) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(k_batch1d, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_batch1d_queue<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_batch1d_queue<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_stream1d, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) set[dev] = bytes;
    return e;
}

// what the batched solver takes (host checks, before the device is touched)
static int batch_check(const nm_plan* P) {
    if (P->gradients != 1) { set_error("batched solver takes 1-gradient problems only"); return NM_ERR_INPUT; }
    if (P->search_mol >= 0 || P->scan_mol >= 0) {
        set_error("a search or scan runs on a device context (nm_ctx_search, nm_plan_scan_value), not in a batch");
        return NM_ERR_INPUT;
    }
    if (P->MX > B1_KS * B1_THREADS) { set_error("batched solver takes at most 512 layers"); return NM_ERR_INPUT; }
    if (P->charged) { set_error("charged systems are not supported by the batched solver"); return NM_ERR_INPUT; }
    for (int m = 0; m < P->n_mol; m++)
        if (P->mols[m].markov == 2) {
            set_error("Markov 2 chains run on a device context, not in a batch");
            return NM_ERR_INPUT;
        }
    if (P->n_state > 0) { set_error("internal states run on a device context, not in a batch"); return NM_ERR_INPUT; }
    if (P->n_seg > NM_MAX_SEG || P->n_mol > NM_MAX_MOL || P->diis_m > B1_MAXM) {
        set_error("problem exceeds the batched solver's limits (segments, molecules, DIIS m <= 12)");
        return NM_ERR_INPUT;
    }
    return NM_OK;
}

// Device copies of one plan's constant arrays (curved-lattice weights, KSAM,
// G1 masks, frozen profiles, block trees), shared by every problem that
// uses the plan.
struct B1PlanDev {
    const double *lm1 = nullptr, *l0 = nullptr, *l1 = nullptr, *L = nullptr, *ksam = nullptr, *gmask = nullptr,
                 *phi_frozen = nullptr;
    const nm_block* blocks[NM_MAX_MOL] = {};
    const int* child_index[NM_MAX_MOL] = {};
};

// upload(dst, src, bytes): device copy of a host array (an allocation the
// caller owns)
template <typename Up>
static int b1_plan_upload(const nm_plan* P, B1PlanDev& D, Up&& upload) {
    const int M = P->M;
    auto up = [&](const void** dst, const void* src, size_t bytes) {
        void* d = nullptr;
        int rc = upload(&d, src, bytes);
        *dst = d;
        return rc;
    };
    if (P->geometry != NM_PLANAR) {
        TRYB(up((const void**)&D.lm1, P->lambda_1, sizeof(double) * M));
        TRYB(up((const void**)&D.l0, P->lambda0, sizeof(double) * M));
        TRYB(up((const void**)&D.l1, P->lambda1, sizeof(double) * M));
        TRYB(up((const void**)&D.L, P->L, sizeof(double) * M));
    }
    std::vector<double> ks(M);
    for (int s = 0; s < M; s++) ks[s] = P->ksam[s];
    TRYB(up((const void**)&D.ksam, ks.data(), sizeof(double) * M));
    TRYB(up((const void**)&D.gmask, P->seg_gmask, sizeof(double) * P->n_seg * M));
    TRYB(up((const void**)&D.phi_frozen, P->seg_phi_frozen, sizeof(double) * P->n_seg * M));
    for (int m = 0; m < P->n_mol; m++) {
        const nm_molecule& mol = P->mols[m];
        if (mol.n_blocks > B1_MAXB) { set_error("molecule has too many blocks for the batched solver"); return NM_ERR_INPUT; }
        std::vector<int> ci(mol.child_index, mol.child_index + (mol.n_blocks > 1 ? mol.n_blocks - 1 : 0));
        if (ci.empty()) ci.push_back(0);
        TRYB(up((const void**)&D.blocks[m], mol.blocks, sizeof(nm_block) * mol.n_blocks));
        TRYB(up((const void**)&D.child_index[m], ci.data(), sizeof(int) * ci.size()));
    }
    return NM_OK;
}

// The descriptor of one problem of plan P over its plan's device constants.
// Its stored propagators and DIIS history get byte offsets inside a slot of
// the work loop's scratch (256-byte aligned pieces): `scratch` returns the
// bytes one slot needs for it, `smem` the kernel's dynamic shared memory.
static int b1_describe(const nm_plan* P, const B1PlanDev& PD, B1Prob& H, size_t& scratch, size_t& smem) {
    std::memset(&H, 0, sizeof(H));
    const int M = P->M;
    // one stored vector: M doubles (FP64 phase) or 128·SP floats (FP32 phase)
    const size_t tsz = std::max((size_t)8 * M, (size_t)4 * BC_NT * b1_sp(P->MX));
    H.MX = P->MX; H.M = M; H.geom = P->geometry; H.ns = P->n_seg; H.nit = P->n_it;
    H.nmol = P->n_mol; H.solvent = P->solvent; H.m = P->diis_m; H.itlim = P->iterationlimit;
    H.max_norm = P->max_norm; H.iv = P->iv; H.lam = P->lambda; H.tol = P->tolerance; H.dmax = P->deltamax;
    H.b1 = P->bc[0] == NM_BC_MIRROR ? 1 : P->bc[0] == NM_BC_PERIODIC ? P->MX : 0;
    H.bm = P->bc[3] == NM_BC_MIRROR ? P->MX : P->bc[3] == NM_BC_PERIODIC ? 1 : P->MX + 1;
    H.lm1 = PD.lm1; H.l0 = PD.l0; H.l1 = PD.l1; H.L = PD.L;
    H.ksam = PD.ksam; H.gmask = PD.gmask; H.phi_frozen = PD.phi_frozen;
    size_t used = 0;
    auto take = [&used](size_t bytes) {
        size_t o = (used + 255) & ~(size_t)255;
        used = o + std::max<size_t>(bytes, 1);
        return (unsigned long long)o;
    };
    for (int i = 0; i < P->n_seg; i++) {
        H.seg_it[i] = P->seg_it[i];
        H.seg_frozen[i] = P->seg_freedom[i] == NM_SEG_FROZEN;
        H.seg_inmol[i] = P->seg_it[i] >= 0;
    }
    for (int i = 0; i < P->n_it; i++) H.it_seg[i] = P->it_seg[i];
    for (int i = 0; i < P->n_seg * P->n_seg; i++) H.chi[i] = P->chi[i];
    int kk = 0;
    for (int m = 0; m < P->n_mol; m++) {
        const nm_molecule& mol = P->mols[m];
        B1Mol& D = H.mol[m];
        D.freedom = mol.freedom; D.pinned = mol.pinned; D.n_blocks = mol.n_blocks; D.n_store = mol.n_store;
        D.n_molmon = mol.n_molmon; D.mm0 = kk;
        D.n_in = mol.n; D.theta_in = mol.theta; D.phibulk_in = mol.phibulk; D.N = mol.chainlength;
        D.blocks = PD.blocks[m]; D.child_index = PD.child_index[m];
        H.so[m].gf = take(tsz * (size_t)mol.n_store);
        H.so[m].pc = take(tsz * (size_t)mol.n_blocks);
        H.so[m].q = take(tsz * (size_t)mol.n_blocks);
        // power-of-two exponents: one per thread (128) per stored vector
        H.so[m].ef = take(sizeof(int) * BC_NT * (size_t)mol.n_store);
        H.so[m].epc = take(sizeof(int) * BC_NT * (size_t)mol.n_blocks);
        H.so[m].eq = take(sizeof(int) * BC_NT * (size_t)mol.n_blocks);
        for (int j = 0; j < mol.n_molmon; j++) {
            if (kk >= NM_MAX_MM) { set_error("too many (molecule, segment) pairs"); return NM_ERR_INPUT; }
            H.mm_mol[kk] = m; H.mm_seg[kk] = mol.molmon_seg[j]; H.mm_frac[kk] = mol.molmon_fraction[j];
            kk++;
        }
    }
    H.n_mm = kk;
    H.so_xR = take(sizeof(double) * (size_t)P->diis_m * P->iv);
    H.so_xx0 = take(sizeof(double) * (size_t)P->diis_m * P->iv);
    scratch = (used + 255) & ~(size_t)255;
    H.sw_tol = 2e-6;
    H.sw_floor = b1_fp32_floor(P);
    smem = sizeof(double) * b1_smem_doubles(P->n_seg, kk, M, P->MX);
    return NM_OK;
}

static int batch_init(Batch& B, const nm_plan* const* plans, int n, const nm_ctx_options* opt) {
    for (int p = 0; p < n; p++) {
        if (!plans[p]) { set_error("nm_batch_create: null plan"); return NM_ERR_ARG; }
        if (int rc = batch_check(plans[p])) return rc;
    }
    B.precision = opt ? opt->precision : NM_FP64;
    int dev = opt ? opt->device : 0;
    cudaError_t e = cudaSetDevice(dev);
    if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    nm_pool_setup(dev);
    if (opt && opt->stream) B.stream = (cudaStream_t)opt->stream;
    else { cudaStreamCreateWithFlags(&B.stream, cudaStreamNonBlocking); B.own_stream = true; }
    long long off = 0;
    size_t maxsmem = 0;
    B.hp.resize(n);
    B.offsets.resize(n + 1);
    std::map<const nm_plan*, B1PlanDev> pdev;
    auto upload = [&B](void** dst, const void* src, size_t bytes) -> int {
        char* d = nullptr;
        int rc = B.upload(&d, (const char*)src, bytes);
        *dst = d;
        return rc;
    };
    for (int p = 0; p < n; p++) {
        const nm_plan* P = plans[p];
        B.plans.push_back(P);
        auto found = pdev.find(P);
        if (found == pdev.end()) {
            B1PlanDev D;
            TRYB(b1_plan_upload(P, D, upload));
            found = pdev.emplace(P, D).first;
        }
        size_t scratch = 0, smem = 0;
        TRYB(b1_describe(P, found->second, B.hp[p], scratch, smem));
        B.slot_bytes = std::max(B.slot_bytes, scratch);
        maxsmem = std::max(maxsmem, smem);
        B.offsets[p] = off;
        off += P->iv;
    }
    B.offsets[n] = off;
    TRYB(B.alloc(&B.d_x, (size_t)off));
    TRYB(B.alloc(&B.d_g, (size_t)off));
    for (int p = 0; p < n; p++) { B.hp[p].x = B.d_x + B.offsets[p]; B.hp[p].g = B.d_g + B.offsets[p]; }
    TRYB(B.alloc(&B.d_probs, (size_t)n));
    {
        // a step's latency hardly depends on the lattice size (each thread
        // owns at most 4 sites), so a solve's length follows its steps per
        // residual, Σ n_store; larger lattices first among equals
        std::vector<long long> steps(n, 0);
        for (int p = 0; p < n; p++)
            for (int m = 0; m < plans[p]->n_mol; m++) steps[p] += plans[p]->mols[m].n_store;
        std::vector<int> ord(n);
        for (int p = 0; p < n; p++) ord[p] = p;
        std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
            return steps[a] != steps[b] ? steps[a] > steps[b] : plans[a]->MX > plans[b]->MX;
        });
        TRYB(B.upload(&B.d_order, ord.data(), (size_t)n));
    }
    B.smem = maxsmem;
    if (maxsmem > 220 * 1024) { set_error("problem too large for the batched solver's shared memory"); return NM_ERR_INPUT; }
    if (cudaError_t e1 = b1_raise_smem(dev, maxsmem)) {
        set_error(std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e1));
        return NM_ERR_CUDA;
    }
    // the work loop: as many slots as CTAs of k_batch1d_queue fit on the
    // device at once with this shared memory, at most one per problem
    int per_sm = 0, per_sm4 = 0, sms = 0;
    cudaError_t e2 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch1d_queue<3>, B1_THREADS, maxsmem);
    if (e2 == cudaSuccess)
        e2 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm4, k_batch1d_queue<4>, B1_THREADS, maxsmem);
    if (e2 == cudaSuccess) e2 = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e2 != cudaSuccess || per_sm < 1) {
        set_error(std::string("batched solver occupancy: ") + cudaGetErrorString(e2));
        return NM_ERR_CUDA;
    }
    // the default: the 168-register variant, as many CTAs as fit; the
    // scratch also holds the 128-register variant's larger count, for the tuner
    B.per_sm3 = per_sm;
    B.slots = std::min(n, per_sm * sms);
    B.slots_cap = std::min(n, std::max(per_sm, per_sm4) * sms);
    TRYB(B.alloc(&B.d_slots, B.slot_bytes * (size_t)B.slots_cap));
    TRYB(B.alloc(&B.d_head, 1));
    return NM_OK;
}

// the work loop over every problem of the batch; FP32 problems switch to FP64
// inside their CTA
static cudaError_t b1_launch(Batch& B, int mode) {
    int n = (int)B.hp.size();
    cudaError_t e = cudaMemsetAsync(B.d_head, 0, sizeof(unsigned int), B.stream);
    if (e != cudaSuccess) return e;
    int sms = 1, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (B.slots > B.per_sm3 * sms)  // more slots than the 168-register variant keeps resident
        k_batch1d_queue<4><<<B.slots, B1_THREADS, B.smem, B.stream>>>(B.d_probs, n, mode, B.d_order, B.d_slots,
                                                                      (unsigned long long)B.slot_bytes, B.d_head);
    else
        k_batch1d_queue<3><<<B.slots, B1_THREADS, B.smem, B.stream>>>(B.d_probs, n, mode, B.d_order, B.d_slots,
                                                                      (unsigned long long)B.slot_bytes, B.d_head);
    B.launches++;
    return cudaGetLastError();
}

static int batch_run(Batch& B) {
    int n = (int)B.hp.size();
    cudaError_t e = cudaMemcpyAsync(B.d_probs, B.hp.data(), sizeof(B1Prob) * n, cudaMemcpyHostToDevice, B.stream);
    if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    e = b1_launch(B, B.precision == NM_FP32 ? 1 : 0);
    if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    e = cudaMemcpyAsync(B.hp.data(), B.d_probs, sizeof(B1Prob) * n, cudaMemcpyDeviceToHost, B.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(B.stream);
    if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    return NM_OK;
}

}  // namespace nm

using nm::Batch;

extern "C" {

int nm_batch_create(const nm_plan* const* plans, int n_plans, const nm_ctx_options* opt, nm_batch** out) {
    if (!plans || n_plans < 1 || !out) { nm::set_error("nm_batch_create: bad argument"); return NM_ERR_ARG; }
    *out = nullptr;
    Batch* b = new Batch();
    int rc = nm::batch_init(*b, plans, n_plans, opt);
    if (rc) { delete b; return rc; }
    *out = reinterpret_cast<nm_batch*>(b);
    return NM_OK;
}

int nm_batch_destroy(nm_batch* b) {
    delete reinterpret_cast<Batch*>(b);
    return NM_OK;
}

static int fill_results(Batch* B, int* iterations, double* residual, int* status) {
    int n = (int)B->hp.size();
    for (int p = 0; p < n; p++) {
        if (iterations) iterations[p] = B->hp[p].iterations;
        if (residual) residual[p] = B->hp[p].residual;
        if (status) status[p] = B->hp[p].status;
    }
    return NM_OK;
}

int nm_batch_solve_dev(nm_batch* b, double* x_dev, int* iterations, double* residual, int* status) {
    Batch* B = reinterpret_cast<Batch*>(b);
    if (!B || !x_dev) { nm::set_error("nm_batch_solve_dev: bad argument"); return NM_ERR_ARG; }
    cudaError_t e = cudaMemcpyAsync(B->d_x, x_dev, sizeof(double) * B->offsets.back(), cudaMemcpyDeviceToDevice, B->stream);
    if (e != cudaSuccess) { nm::set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    int rc = nm::batch_run(*B);
    if (rc) return rc;
    e = cudaMemcpyAsync(x_dev, B->d_x, sizeof(double) * B->offsets.back(), cudaMemcpyDeviceToDevice, B->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(B->stream);
    if (e != cudaSuccess) { nm::set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    return fill_results(B, iterations, residual, status);
}

int nm_batch_solve_host(nm_batch* b, double* x_host, int* iterations, double* residual, int* status) {
    Batch* B = reinterpret_cast<Batch*>(b);
    if (!B || !x_host) { nm::set_error("nm_batch_solve_host: bad argument"); return NM_ERR_ARG; }
    cudaError_t e = cudaMemcpyAsync(B->d_x, x_host, sizeof(double) * B->offsets.back(), cudaMemcpyHostToDevice, B->stream);
    if (e != cudaSuccess) { nm::set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    int rc = nm::batch_run(*B);
    if (rc) return rc;
    e = cudaMemcpyAsync(x_host, B->d_x, sizeof(double) * B->offsets.back(), cudaMemcpyDeviceToHost, B->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(B->stream);
    if (e != cudaSuccess) { nm::set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    return fill_results(B, iterations, residual, status);
}

int nm_batch_offsets(nm_batch* b, long long* offsets) {
    Batch* B = reinterpret_cast<Batch*>(b);
    if (!B || !offsets) { nm::set_error("nm_batch_offsets: bad argument"); return NM_ERR_ARG; }
    for (size_t i = 0; i < B->offsets.size(); i++) offsets[i] = B->offsets[i];
    return NM_OK;
}

int nm_batch_residual_dev(nm_batch* b, const double* x_dev, double* g_dev, int precision) {
    Batch* B = reinterpret_cast<Batch*>(b);
    if (!B || !x_dev || !g_dev) { nm::set_error("nm_batch_residual_dev: bad argument"); return NM_ERR_ARG; }
    size_t n = (size_t)B->offsets.back();
    cudaError_t e = cudaMemcpyAsync(B->d_x, x_dev, sizeof(double) * n, cudaMemcpyDeviceToDevice, B->stream);
    if (e != cudaSuccess) { nm::set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    int np = (int)B->hp.size();
    for (int p = 0; p < np; p++) B->hp[p].eval_only = 1;
    e = cudaMemcpyAsync(B->d_probs, B->hp.data(), sizeof(nm::B1Prob) * np, cudaMemcpyHostToDevice, B->stream);
    if (e != cudaSuccess) { nm::set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    e = nm::b1_launch(*B, precision == NM_FP32 ? 1 : 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(g_dev, B->d_g, sizeof(double) * n, cudaMemcpyDeviceToDevice, B->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(B->stream);
    for (int p = 0; p < np; p++) B->hp[p].eval_only = 0;
    if (e != cudaSuccess) { nm::set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    return NM_OK;
}

int nm_batch_stats(nm_batch* b, int* fp32_iterations) {
    Batch* B = reinterpret_cast<Batch*>(b);
    if (!B || !fp32_iterations) { nm::set_error("nm_batch_stats: bad argument"); return NM_ERR_ARG; }
    for (size_t p = 0; p < B->hp.size(); p++) fp32_iterations[p] = B->hp[p].fp32_iterations;
    return NM_OK;
}

int nm_batch_times(nm_batch* b, double* seconds) {
    Batch* B = reinterpret_cast<Batch*>(b);
    if (!B || !seconds) { nm::set_error("nm_batch_times: bad argument"); return NM_ERR_ARG; }
    unsigned long long t0 = ~0ull;
    for (auto& h : B->hp) t0 = std::min(t0, h.t_begin);
    for (size_t p = 0; p < B->hp.size(); p++) seconds[p] = (double)(B->hp[p].t_end - t0) * 1e-9;
    return NM_OK;
}

int nm_batch_timings(nm_batch* b, double* queued, double* solving) {
    Batch* B = reinterpret_cast<Batch*>(b);
    if (!B || (!queued && !solving)) { nm::set_error("nm_batch_timings: bad argument"); return NM_ERR_ARG; }
    unsigned long long t0 = ~0ull;
    for (auto& h : B->hp) t0 = std::min(t0, h.t_begin);
    for (size_t p = 0; p < B->hp.size(); p++) {
        if (queued) queued[p] = (double)(B->hp[p].t_begin - t0) * 1e-9;
        if (solving) solving[p] = (double)(B->hp[p].t_end - B->hp[p].t_begin) * 1e-9;
    }
    return NM_OK;
}

int nm_batch_slots(nm_batch* b) {
    Batch* B = reinterpret_cast<Batch*>(b);
    return B ? B->slots : 0;
}

int nm_batch_set_slots(nm_batch* b, int slots) {
    Batch* B = reinterpret_cast<Batch*>(b);
    if (!B || slots < 1) { nm::set_error("nm_batch_set_slots: bad argument"); return NM_ERR_ARG; }
    if (slots > B->slots_cap) {
        nm::set_error("nm_batch_set_slots: more slots than resident CTAs fit (" + std::to_string(B->slots_cap) + ")");
        return NM_ERR_ARG;
    }
    B->slots = slots;  // the scratch was sized for slots_cap
    return NM_OK;
}

// The work loop's autotuner: one solve of the batch (from x_dev, which is not
// changed) per candidate number of resident CTAs per SM, 1 up to what fits.
// The objective is the loop's steady throughput, slots × problems / Σ of
// the problems' solve times (device timer): a batch's wall time is set by its
// longest solves, which fewer CTAs per SM speed up, while a long stream is
// served at the rate all slots together finish problems.  The best is kept
// and remembered for batches of the same shape.
int nm_batch_autotune(nm_batch* b, const double* x_dev, nm_batch_tuning* out) {
    using namespace nm;
    Batch* B = reinterpret_cast<Batch*>(b);
    if (!B || !x_dev || !out) { set_error("nm_batch_autotune: bad argument"); return NM_ERR_ARG; }
    static std::mutex mu;
    static std::map<std::string, int> tuned;  // shape -> CTAs per SM
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int n = (int)B->hp.size();
    int mx = 0;
    long long steps = 0;
    for (const nm_plan* P : B->plans) {
        mx = std::max(mx, P->MX);
        for (int m = 0; m < P->n_mol; m++) steps += P->mols[m].n_store;
    }
    const std::string key = std::to_string(n) + ":" + std::to_string(mx) + ":" + std::to_string(steps) + ":" +
                            std::to_string(B->precision) + ":" + std::to_string(B->slots_cap);
    out->candidates = 0;
    out->ms_per_solve = 0;
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = tuned.find(key);
        if (it != tuned.end()) {
            B->slots = std::min(B->slots_cap, it->second * sms);
            out->slots = B->slots;
            out->ctas_per_sm = it->second;
            return NM_OK;
        }
    }
    const int per_sm_max = std::max(1, (B->slots_cap + sms - 1) / sms);
    double best = 1e300;
    int pick = 1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = NM_OK;
    for (int k = 1; k <= per_sm_max && !rc; k++) {
        B->slots = std::min(B->slots_cap, k * sms);
        cudaError_t e = cudaMemcpyAsync(B->d_x, x_dev, sizeof(double) * B->offsets.back(), cudaMemcpyDeviceToDevice,
                                        B->stream);
        if (e == cudaSuccess) e = cudaEventRecord(e0, B->stream);
        if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); rc = NM_ERR_CUDA; break; }
        rc = batch_run(*B);
        if (rc) break;
        cudaEventRecord(e1, B->stream);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        double busy = 0;  // slot-seconds spent solving
        for (const B1Prob& h : B->hp) busy += (double)(h.t_end - h.t_begin) * 1e-9;
        const double cost = busy > 0 ? busy / B->slots : 1e300;  // seconds per batch at full occupancy
        out->candidates++;
        if (cost < best) { best = cost; pick = k; out->ms_per_solve = ms; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    B->slots = std::min(B->slots_cap, pick * sms);
    {
        std::lock_guard<std::mutex> lk(mu);
        tuned[key] = pick;
    }
    out->slots = B->slots;
    out->ctas_per_sm = pick;
    return NM_OK;
}

int nm_batch_free_energy(nm_batch* b, double* F, double* Omega) {
    Batch* B = reinterpret_cast<Batch*>(b);
    if (!B) { nm::set_error("nm_batch_free_energy: bad argument"); return NM_ERR_ARG; }
    // Evaluated by a device context per problem on the final field.
    for (size_t p = 0; p < B->hp.size(); p++) {
        nm_ctx* c = nullptr;
        nm_ctx_options o{NM_FP64, 0, 0, B->stream};
        int rc = nm_ctx_create(B->plans[p], &o, &c);
        if (rc) return rc;
        rc = nm_residual_dev(c, B->d_x + B->offsets[p], reinterpret_cast<nm::Ctx*>(c)->d_g);
        if (!rc) rc = nm_free_energy(c, F ? F + p : nullptr, Omega ? Omega + p : nullptr, nullptr);
        nm_ctx_destroy(c);
        if (rc) return rc;
    }
    return NM_OK;
}

long long nm_batch_launch_count(nm_batch* b) {
    Batch* B = reinterpret_cast<Batch*>(b);
    return B ? B->launches : 0;
}

}  // extern "C"

// ======================================================================
// Allocation-free single-problem solve.
//
// Some callers cannot allocate device memory at the point where they solve:
// a host that owns a fixed device memory budget sliced before work begins,
// or a re-solve on a latency-critical path that must not touch the
// allocator.  nm_solve1d_noalloc runs the
// same kernel as nm_batch_solve_dev on one 1-gradient problem, with every piece of device scratch
// carved from one file-scope array compiled into the library.  The array's
// address is looked up once per device (cudaGetSymbolAddress, with that
// device current) on the first call for that device; make that first call
// before any stream capture.  The scratch is shared, so calls that overlap
// in time (two host threads, or two streams in flight) race on it.  Each
// call synchronises its stream and returns its result on the host.
// ======================================================================
namespace nm {

static __device__ __align__(256) unsigned char g_noalloc_scratch[NM_NOALLOC_SCRATCH_BYTES];

#define NM_NOALLOC_MAX_DEVICES 64
static unsigned char* g_noalloc_base[NM_NOALLOC_MAX_DEVICES];

// bump allocator over the static scratch (256-byte aligned pieces)
struct StaticArena {
    unsigned char* base;
    size_t used = 0;
    bool overflow = false;
    template <typename X>
    X* take(size_t n) {
        if (n == 0) n = 1;
        size_t off = (used + 255) & ~(size_t)255;
        size_t bytes = sizeof(X) * n;
        if (off + bytes > (size_t)NM_NOALLOC_SCRATCH_BYTES) { overflow = true; return nullptr; }
        used = off + bytes;
        return reinterpret_cast<X*>(base + off);
    }
};

struct NoallocCopy { void* dst; const void* src; size_t bytes; };

// One problem's descriptor laid out in the arena, with the contents
// batch_init gives it.  Host sources of the copies to make are listed in
// `copies`; `ks` stages KSAM as doubles and must outlive those copies.
static int noalloc_layout(const nm_plan* P, StaticArena& A, double* x_dev, B1Prob& H, size_t& smem,
                          std::vector<double>& ks, std::vector<NoallocCopy>& copies) {
    if (P->gradients != 1) { set_error("nm_solve1d_noalloc: 1-gradient problems only"); return NM_ERR_INPUT; }
    if (P->search_mol >= 0 || P->scan_mol >= 0) {
        set_error("nm_solve1d_noalloc: a search or scan runs on a device context");
        return NM_ERR_INPUT;
    }
    if (P->MX > B1_KS * B1_THREADS) { set_error("nm_solve1d_noalloc: at most 512 layers"); return NM_ERR_INPUT; }
    if (P->charged) { set_error("nm_solve1d_noalloc: charged systems are not supported"); return NM_ERR_INPUT; }
    for (int m = 0; m < P->n_mol; m++)
        if (P->mols[m].markov == 2) { set_error("nm_solve1d_noalloc: Markov 2 chains are not supported"); return NM_ERR_INPUT; }
    if (P->n_state > 0) { set_error("nm_solve1d_noalloc: internal states are not supported"); return NM_ERR_INPUT; }
    if (P->n_seg > NM_MAX_SEG || P->n_mol > NM_MAX_MOL || P->diis_m > B1_MAXM) {
        set_error("nm_solve1d_noalloc: problem exceeds the limits (segments, molecules, DIIS m <= 12)");
        return NM_ERR_INPUT;
    }
    std::memset(&H, 0, sizeof(H));
    const int M = P->M;
    const size_t tsz = std::max((size_t)8 * M, (size_t)4 * BC_NT * b1_sp(P->MX));
    H.MX = P->MX; H.M = M; H.geom = P->geometry; H.ns = P->n_seg; H.nit = P->n_it;
    H.nmol = P->n_mol; H.solvent = P->solvent; H.m = P->diis_m; H.itlim = P->iterationlimit;
    H.max_norm = P->max_norm; H.iv = P->iv; H.lam = P->lambda; H.tol = P->tolerance; H.dmax = P->deltamax;
    H.b1 = P->bc[0] == NM_BC_MIRROR ? 1 : P->bc[0] == NM_BC_PERIODIC ? P->MX : 0;
    H.bm = P->bc[3] == NM_BC_MIRROR ? P->MX : P->bc[3] == NM_BC_PERIODIC ? 1 : P->MX + 1;
    auto put = [&](void* dst, const void* src, size_t bytes) { copies.push_back({dst, src, bytes}); };
    if (P->geometry != NM_PLANAR) {
        double* a = A.take<double>(M);
        double* b = A.take<double>(M);
        double* c = A.take<double>(M);
        double* dL = A.take<double>(M);
        if (A.overflow) goto full;
        put(a, P->lambda_1, sizeof(double) * M);
        put(b, P->lambda0, sizeof(double) * M);
        put(c, P->lambda1, sizeof(double) * M);
        put(dL, P->L, sizeof(double) * M);
        H.lm1 = a; H.l0 = b; H.l1 = c; H.L = dL;
    }
    {
        ks.assign(M, 0.0);
        for (int s = 0; s < M; s++) ks[s] = P->ksam[s];
        double* dk = A.take<double>(M);
        double* dg = A.take<double>((size_t)P->n_seg * M);
        double* dpf = A.take<double>((size_t)P->n_seg * M);
        if (A.overflow) goto full;
        put(dk, ks.data(), sizeof(double) * M);
        put(dg, P->seg_gmask, sizeof(double) * P->n_seg * M);
        put(dpf, P->seg_phi_frozen, sizeof(double) * P->n_seg * M);
        H.ksam = dk; H.gmask = dg; H.phi_frozen = dpf;
    }
    for (int i = 0; i < P->n_seg; i++) {
        H.seg_it[i] = P->seg_it[i];
        H.seg_frozen[i] = P->seg_freedom[i] == NM_SEG_FROZEN;
        H.seg_inmol[i] = P->seg_it[i] >= 0;
    }
    for (int i = 0; i < P->n_it; i++) H.it_seg[i] = P->it_seg[i];
    for (int i = 0; i < P->n_seg * P->n_seg; i++) H.chi[i] = P->chi[i];
    {
        int kk = 0;
        for (int m = 0; m < P->n_mol; m++) {
            const nm_molecule& mol = P->mols[m];
            if (mol.n_blocks > B1_MAXB) { set_error("nm_solve1d_noalloc: molecule has too many blocks"); return NM_ERR_INPUT; }
            B1Mol& D = H.mol[m];
            D.freedom = mol.freedom; D.pinned = mol.pinned; D.n_blocks = mol.n_blocks; D.n_store = mol.n_store;
            D.n_molmon = mol.n_molmon; D.mm0 = kk;
            D.n_in = mol.n; D.theta_in = mol.theta; D.phibulk_in = mol.phibulk; D.N = mol.chainlength;
            const int nci = mol.n_blocks > 1 ? mol.n_blocks - 1 : 1;
            nm_block* db = A.take<nm_block>(mol.n_blocks);
            int* dci = A.take<int>(nci);
            D.Gf = A.take<char>(tsz * (size_t)mol.n_store);
            D.Pc = A.take<char>(tsz * (size_t)mol.n_blocks);
            D.Q = A.take<char>(tsz * (size_t)mol.n_blocks);
            D.ef = A.take<int>(BC_NT * (size_t)mol.n_store);
            D.epc = A.take<int>(BC_NT * (size_t)mol.n_blocks);
            D.eq = A.take<int>(BC_NT * (size_t)mol.n_blocks);
            if (A.overflow) goto full;
            put(db, mol.blocks, sizeof(nm_block) * mol.n_blocks);
            if (mol.n_blocks > 1) put(dci, mol.child_index, sizeof(int) * nci);
            D.blocks = db; D.child_index = dci;
            for (int j = 0; j < mol.n_molmon; j++) {
                if (kk >= NM_MAX_MM) { set_error("nm_solve1d_noalloc: too many (molecule, segment) pairs"); return NM_ERR_INPUT; }
                H.mm_mol[kk] = m; H.mm_seg[kk] = mol.molmon_seg[j]; H.mm_frac[kk] = mol.molmon_fraction[j];
                kk++;
            }
        }
        H.n_mm = kk;
        H.xR = A.take<double>((size_t)P->diis_m * P->iv);
        H.xx0 = A.take<double>((size_t)P->diis_m * P->iv);
        H.g = A.take<double>((size_t)P->iv);
        if (A.overflow) goto full;
        H.x = x_dev;
        H.sw_tol = 2e-6;
        H.sw_floor = b1_fp32_floor(P);
        smem = sizeof(double) * b1_smem_doubles(P->n_seg, kk, M, P->MX);
        if (smem > 220 * 1024) { set_error("nm_solve1d_noalloc: problem too large for shared memory"); return NM_ERR_INPUT; }
    }
    return NM_OK;
full:
    set_error("nm_solve1d_noalloc: problem needs more than the " + std::to_string((size_t)NM_NOALLOC_SCRATCH_BYTES) +
              " bytes of static device scratch");
    return NM_ERR_INPUT;
}

}  // namespace nm

extern "C" int nm_solve1d_noalloc(const nm_plan* plan, double* x_dev, int precision, void* stream,
                                  nm_solve_result* res) {
    using namespace nm;
    if (!plan || !x_dev || !res) { set_error("nm_solve1d_noalloc: bad argument"); return NM_ERR_ARG; }
    if (precision != NM_FP32 && precision != NM_FP64) { set_error("nm_solve1d_noalloc: bad precision"); return NM_ERR_ARG; }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    if (dev < 0 || dev >= NM_NOALLOC_MAX_DEVICES) { set_error("nm_solve1d_noalloc: device ordinal out of range"); return NM_ERR_ARG; }
    if (!g_noalloc_base[dev]) {  // set-up, once per device, with that device current
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) { set_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)); return NM_ERR_CUDA; }
        g_noalloc_base[dev] = (unsigned char*)p;
    }
    cudaStream_t st = (cudaStream_t)stream;
    StaticArena A{g_noalloc_base[dev]};
    B1Prob* d_prob = A.take<B1Prob>(1);
    B1Prob H;
    size_t smem = 0;
    std::vector<double> ks;
    std::vector<NoallocCopy> copies;
    int rc = noalloc_layout(plan, A, x_dev, H, smem, ks, copies);
    if (rc) return rc;
    e = b1_raise_smem(dev, smem);
    if (e != cudaSuccess) { set_error(std::string("nm_solve1d_noalloc: ") + cudaGetErrorString(e)); return NM_ERR_CUDA; }
    // what the batch path's zero-filled allocations start from
    e = cudaMemsetAsync(A.base, 0, A.used, st);
    for (size_t i = 0; e == cudaSuccess && i < copies.size(); i++)
        e = cudaMemcpyAsync(copies[i].dst, copies[i].src, copies[i].bytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_prob, &H, sizeof(B1Prob), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    k_batch1d<<<1, B1_THREADS, smem, st>>>(d_prob, precision == NM_FP32 ? 1 : 0, nullptr);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&H, d_prob, sizeof(B1Prob), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    res->iterations = H.iterations;
    res->residual = H.residual;
    res->status = H.status;
    return H.status == NM_OK ? NM_OK : H.status;
}

// ======================================================================
// Streaming work loop (continuous batching of 1-gradient solves).
//
// The host appends requests to a ring while the loop runs; each resident
// CTA (slot) claims the next published request as soon as its last one has
// converged.  Ring entries, their fields x and their results live in pinned
// host memory mapped into the device's address space: the host publishes an
// entry with a release store of `tail` (system scope), a CTA claims it by a
// compare-and-swap on `head` in device memory, copies descriptor and field
// into its slot-private device memory with uncached loads, solves there
// (b1_solve, the batch kernel's body), writes the field and results back and
// marks the entry done with a release store (system scope).  A CTA that
// finds no work for `idle_ns` leaves the loop; the host relaunches the loop
// when a request arrives, or is waited for, and the loop is gone.  Every
// device-side wait is bounded by that idle limit.
// ======================================================================
namespace nm {

struct StreamEntry {
    B1Prob desc;                   // host-written; its constant-array pointers are rebased on the device
    // the problem's constant arrays, packed by the host into the entry's blob
    // (byte offsets; ~0 = absent): L, λ-1, λ0, λ+1, KSAM, G1 masks, frozen φ,
    // and per molecule the blocks and the children lists
    unsigned long long co_L, co_lm1, co_l0, co_l1, co_ksam, co_gmask, co_pf;
    unsigned long long co_blocks[NM_MAX_MOL], co_ci[NM_MAX_MOL];
    unsigned long long blob_bytes;
    int mode;                      // 0: FP64 propagators, 1: FP32 first
    int iv;
    // device-written results
    int iterations, fp32_iterations, status, pad;
    double residual;
    unsigned long long t_begin, t_end;  // device global timer, ns
    unsigned long long done;       // ticket + 1 once solved (release, system scope)
};

struct StreamCtl {
    unsigned long long tail;       // requests published (host, release)
    unsigned int stop;             // host: 1 ends the loop
    unsigned int pad;
};

__device__ __forceinline__ unsigned long long ld_acquire_sys(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.sys.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_sys(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.sys.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__global__ void __launch_bounds__(B1_THREADS, 3) k_stream1d(StreamEntry* ring, double* xring, int cap, int iv_max,
                                                           StreamCtl* ctl, unsigned long long* head,
                                                           unsigned char* slots, unsigned long long slot_bytes,
                                                           B1Prob* priv, double* xpriv, double* gpriv,
                                                           unsigned long long idle_ns, const unsigned char* blobs,
                                                           unsigned char* cpriv, unsigned long long blob_max) {
    __shared__ unsigned long long s_tk, s_blob;
    __shared__ int s_go, s_mode, s_iv;
    B1Prob& P = priv[blockIdx.x];
    unsigned char* base = slots + (size_t)blockIdx.x * slot_bytes;
    unsigned char* cbase = cpriv + (size_t)blockIdx.x * blob_max;
    double* xs = xpriv + (size_t)blockIdx.x * iv_max;
    double* gs = gpriv + (size_t)blockIdx.x * iv_max;
    for (;;) {
        if (threadIdx.x == 0) {
            s_go = 0;
            const unsigned long long t0 = b1_clock();
            for (;;) {  // ends on a claim, on stop, or after idle_ns without work
                const unsigned long long tail = ld_acquire_sys(&ctl->tail);
                if (*(volatile unsigned int*)&ctl->stop) break;
                const unsigned long long h = *(volatile unsigned long long*)head;
                if (h < tail) {
                    if (atomicCAS(head, h, h + 1) == h) { s_tk = h; s_go = 1; break; }
                    continue;
                }
                if (b1_clock() - t0 > idle_ns) break;
                __nanosleep(2000);
            }
            if (s_go) {
                const StreamEntry* E = ring + (s_tk % (unsigned long long)cap);
                s_mode = *(const volatile int*)&E->mode;
                s_iv = *(const volatile int*)&E->iv;
                s_blob = *(const volatile unsigned long long*)&E->blob_bytes;
            }
        }
        __syncthreads();
        if (!s_go) break;
        const unsigned long long tk = s_tk;
        const int slot = (int)(tk % (unsigned long long)cap);
        StreamEntry* E = ring + slot;
        {   // private copies: uncached loads of the host-written entry
            const unsigned long long* src = reinterpret_cast<const unsigned long long*>(&E->desc);
            unsigned long long* dst = reinterpret_cast<unsigned long long*>(&P);
            for (int i = threadIdx.x; i < (int)(sizeof(B1Prob) / 8); i += blockDim.x) dst[i] = __ldcv(src + i);
            const double* xsrc = xring + (size_t)slot * iv_max;
            for (int i = threadIdx.x; i < s_iv; i += blockDim.x) xs[i] = __ldcv(xsrc + i);
            const unsigned int* bsrc = reinterpret_cast<const unsigned int*>(blobs + (size_t)slot * blob_max);
            unsigned int* bdst = reinterpret_cast<unsigned int*>(cbase);
            for (int i = threadIdx.x; i < (int)(s_blob / 4); i += blockDim.x) bdst[i] = __ldcv(bsrc + i);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const volatile StreamEntry* V = E;
            auto at = [&](unsigned long long o) -> const double* {
                return o == ~0ull ? nullptr : reinterpret_cast<const double*>(cbase + o);
            };
            P.L = at(V->co_L); P.lm1 = at(V->co_lm1); P.l0 = at(V->co_l0); P.l1 = at(V->co_l1);
            P.ksam = at(V->co_ksam); P.gmask = at(V->co_gmask); P.phi_frozen = at(V->co_pf);
            for (int m = 0; m < P.nmol; m++) {
                P.mol[m].blocks = reinterpret_cast<const nm_block*>(cbase + V->co_blocks[m]);
                P.mol[m].child_index = reinterpret_cast<const int*>(cbase + V->co_ci[m]);
            }
            P.x = xs;
            P.g = gs;
            P.eval_only = 0;
            b1_rebase(P, base);
        }
        __syncthreads();
        b1_solve(P, s_mode);
        __syncthreads();
        {
            double* xdst = xring + (size_t)slot * iv_max;
            for (int i = threadIdx.x; i < s_iv; i += blockDim.x) ((volatile double*)xdst)[i] = xs[i];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            volatile StreamEntry* V = E;
            V->iterations = P.iterations;
            V->fp32_iterations = P.fp32_iterations;
            V->status = P.status;
            V->residual = P.residual;
            V->t_begin = P.t_begin;
            V->t_end = P.t_end;
            __threadfence_system();
            st_release_sys(&E->done, tk + 1);
        }
        __syncthreads();
    }
}

}  // namespace nm

#include <atomic>
#include <chrono>
#include <cstdlib>
#include <thread>

namespace nm {

// A persistent work loop occupies its stream's hardware work queue while it
// runs, so any stream mapped to the same queue waits behind it.  CUDA maps
// streams onto CUDA_DEVICE_MAX_CONNECTIONS queues (8 unless set) when the
// context is created; the library asks for 32 at load time, without
// overriding a value the process set, for contexts created after it loads.
__attribute__((constructor)) static void stream_connections_default() {
    setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0);
}

static double stream_now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Stream1D {
    int dev = 0, cap = 0, iv_max = 0, slots = 0;
    nm_stream_options env{};
    size_t slot_bytes = 0, smem = 0, blob_max = 0;
    unsigned long long idle_ns = 0;
    // pinned host memory mapped into the device's address space
    StreamEntry* ring = nullptr;  StreamEntry* ring_d = nullptr;
    double* xring = nullptr;      double* xring_d = nullptr;
    unsigned char* blobs = nullptr; unsigned char* blobs_d = nullptr;
    StreamCtl* ctl = nullptr;     StreamCtl* ctl_d = nullptr;
    // device memory
    unsigned long long* head = nullptr;
    unsigned char* d_slots = nullptr;
    unsigned char* d_cpriv = nullptr;
    B1Prob* d_priv = nullptr;
    double *d_xpriv = nullptr, *d_gpriv = nullptr;
    cudaStream_t loop_stream = nullptr;
    cudaEvent_t loop_done = nullptr;
    bool launched = false;
    long long launches = 0;
    std::mutex mu;
    unsigned long long tail = 0;      // next ticket
    unsigned long long reaped = 0;    // tickets below this are done (times recorded)
    std::vector<char> busy;           // per ring entry: submitted and not yet waited for
    std::vector<unsigned long long> owner;
    std::vector<double> t_submit, t_done;
    std::thread reaper;
    std::atomic<bool> quit{false};

    int broken = 0;                   // a CUDA error seen by the loop: every wait fails with it
    bool loop_alive() {
        if (!launched) return false;
        const cudaError_t e = cudaEventQuery(loop_done);
        if (e != cudaSuccess && e != cudaErrorNotReady && !broken) {
            broken = NM_ERR_CUDA;
            set_error(std::string("stream loop: ") + cudaGetErrorString(e));
        }
        return e == cudaErrorNotReady;
    }
    int launch_locked() {
        cudaSetDevice(dev);
        k_stream1d<<<slots, B1_THREADS, smem, loop_stream>>>(ring_d, xring_d, cap, iv_max, ctl_d, head, d_slots,
                                                            (unsigned long long)slot_bytes, d_priv, d_xpriv, d_gpriv,
                                                            idle_ns, blobs_d, d_cpriv,
                                                            (unsigned long long)blob_max);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventRecord(loop_done, loop_stream);
        if (e != cudaSuccess) { set_error(std::string("stream loop launch: ") + cudaGetErrorString(e)); return NM_ERR_CUDA; }
        launched = true;
        launches++;
        return NM_OK;
    }
    // completion times of finished requests, and a new loop if requests wait
    // while the loop is gone (its CTAs leave after idle_ns without work)
    void reap() {
        while (!quit.load()) {
            {
                std::lock_guard<std::mutex> lk(mu);
                while (reaped < tail) {
                    const int s = (int)(reaped % (unsigned long long)cap);
                    if (__atomic_load_n(&ring[s].done, __ATOMIC_ACQUIRE) != reaped + 1) break;
                    t_done[s] = stream_now();
                    reaped++;
                }
                if (reaped < tail && !loop_alive() && !broken && launch_locked()) broken = NM_ERR_CUDA;
            }
            std::this_thread::sleep_for(std::chrono::microseconds(20));
        }
    }
    ~Stream1D() {
        if (ctl) __atomic_store_n(&ctl->stop, 1u, __ATOMIC_RELEASE);
        quit.store(true);
        if (reaper.joinable()) reaper.join();
        if (launched) cudaEventSynchronize(loop_done);
        if (loop_done) cudaEventDestroy(loop_done);
        void* dev_ptrs[] = {head, d_slots, d_cpriv, d_priv, d_xpriv, d_gpriv};
        for (void* q : dev_ptrs) if (q) cudaFree(q);
        void* host_ptrs[] = {ring, xring, blobs, ctl};
        for (void* q : host_ptrs) if (q) cudaFreeHost(q);
        if (loop_stream) cudaStreamDestroy(loop_stream);
    }
};

// The problem's constant arrays into its entry's blob (16-byte aligned pieces)
static int stream_pack(const nm_plan* P, StreamEntry& E, unsigned char* blob, size_t blob_max) {
    const int M = P->M;
    size_t used = 0;
    bool ok = true;
    auto put = [&](const void* src, size_t bytes) -> unsigned long long {
        const size_t o = (used + 15) & ~(size_t)15;
        if (o + bytes > blob_max) { ok = false; return ~0ull; }
        std::memcpy(blob + o, src, bytes);
        used = o + bytes;
        return o;
    };
    const bool curved = P->geometry != NM_PLANAR;
    E.co_L = curved ? put(P->L, sizeof(double) * M) : ~0ull;
    E.co_lm1 = curved ? put(P->lambda_1, sizeof(double) * M) : ~0ull;
    E.co_l0 = curved ? put(P->lambda0, sizeof(double) * M) : ~0ull;
    E.co_l1 = curved ? put(P->lambda1, sizeof(double) * M) : ~0ull;
    std::vector<double> ks(M);
    for (int s = 0; s < M; s++) ks[s] = P->ksam[s];
    E.co_ksam = put(ks.data(), sizeof(double) * M);
    E.co_gmask = put(P->seg_gmask, sizeof(double) * P->n_seg * M);
    E.co_pf = put(P->seg_phi_frozen, sizeof(double) * P->n_seg * M);
    for (int m = 0; m < P->n_mol; m++) {
        const nm_molecule& mol = P->mols[m];
        E.co_blocks[m] = put(mol.blocks, sizeof(nm_block) * mol.n_blocks);
        const int nci = mol.n_blocks > 1 ? mol.n_blocks - 1 : 0;
        const int zero = 0;
        E.co_ci[m] = nci ? put(mol.child_index, sizeof(int) * nci) : put(&zero, sizeof(int));
    }
    E.blob_bytes = (used + 15) & ~(size_t)15;
    if (!ok) { set_error("request exceeds the stream's constant-array space"); return NM_ERR_INPUT; }
    return NM_OK;
}

}  // namespace nm

using nm::Stream1D;

extern "C" {

int nm_stream_create(const nm_stream_options* opt, nm_stream** out) {
    using namespace nm;
    if (!opt || !out) { set_error("nm_stream_create: bad argument"); return NM_ERR_ARG; }
    *out = nullptr;
    const nm_stream_options& o = *opt;
    if (o.capacity < 1 || o.max_layers < 1 || o.max_layers > B1_KS * B1_THREADS || o.max_segments < 1 ||
        o.max_segments > NM_MAX_SEG || o.max_pairs < 1 || o.max_pairs > NM_MAX_MM || o.max_molecules < 1 ||
        o.max_molecules > NM_MAX_MOL || o.max_store < 1 || o.max_blocks < 1 || o.max_diis < 1 || o.max_diis > B1_MAXM) {
        set_error("nm_stream_create: envelope out of range (layers <= 512, segments <= 16, pairs <= 32, "
                  "molecules <= 16, DIIS m <= 12)");
        return NM_ERR_ARG;
    }
    Stream1D* S = new Stream1D();
    S->env = o;
    S->dev = o.device;
    S->cap = o.capacity;
    cudaError_t e = cudaSetDevice(S->dev);
    if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); delete S; return NM_ERR_CUDA; }
    const int Mmax = o.max_layers + 2;
    S->iv_max = o.max_segments * Mmax;
    const size_t tsz = std::max((size_t)8 * Mmax, (size_t)4 * BC_NT * b1_sp(o.max_layers));
    const size_t nvec = (size_t)o.max_store + 2 * (size_t)o.max_blocks;
    S->slot_bytes = tsz * nvec + sizeof(int) * BC_NT * nvec + 2 * sizeof(double) * o.max_diis * (size_t)S->iv_max +
                    256 * (6 * (size_t)o.max_molecules + 4);
    S->slot_bytes = (S->slot_bytes + 255) & ~(size_t)255;
    S->blob_max = sizeof(double) * Mmax * (5 + 2 * (size_t)o.max_segments) +
                  (size_t)o.max_molecules * (sizeof(nm_block) + sizeof(int)) * o.max_blocks + 16 * (8 + 2 * o.max_molecules);
    S->blob_max = (S->blob_max + 255) & ~(size_t)255;
    S->smem = sizeof(double) * b1_smem_doubles(o.max_segments, o.max_pairs, Mmax, o.max_layers);
    S->idle_ns = (unsigned long long)((o.idle_seconds > 0 ? o.idle_seconds : 0.2) * 1e9);
    if (S->smem > 220 * 1024) { set_error("nm_stream_create: envelope too large for shared memory"); delete S; return NM_ERR_ARG; }
    auto fail = [&](cudaError_t err) {
        set_error(std::string("nm_stream_create: ") + cudaGetErrorString(err));
        delete S;
        return NM_ERR_CUDA;
    };
    if ((e = b1_raise_smem(S->dev, S->smem))) return fail(e);
    int per_sm = 0, sms = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_stream1d, B1_THREADS, S->smem))) return fail(e);
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, S->dev))) return fail(e);
    S->slots = std::max(1, per_sm * sms);
    if (o.slots > 0) S->slots = std::min(S->slots, o.slots);
    const unsigned fl = cudaHostAllocMapped | cudaHostAllocPortable;
    if ((e = cudaHostAlloc((void**)&S->ring, sizeof(StreamEntry) * S->cap, fl))) return fail(e);
    if ((e = cudaHostAlloc((void**)&S->xring, sizeof(double) * S->cap * (size_t)S->iv_max, fl))) return fail(e);
    if ((e = cudaHostAlloc((void**)&S->blobs, S->blob_max * S->cap, fl))) return fail(e);
    if ((e = cudaHostAlloc((void**)&S->ctl, sizeof(StreamCtl), fl))) return fail(e);
    std::memset((void*)S->ring, 0, sizeof(StreamEntry) * S->cap);
    std::memset(S->ctl, 0, sizeof(StreamCtl));
    if ((e = cudaHostGetDevicePointer((void**)&S->ring_d, S->ring, 0))) return fail(e);
    if ((e = cudaHostGetDevicePointer((void**)&S->xring_d, S->xring, 0))) return fail(e);
    if ((e = cudaHostGetDevicePointer((void**)&S->blobs_d, S->blobs, 0))) return fail(e);
    if ((e = cudaHostGetDevicePointer((void**)&S->ctl_d, S->ctl, 0))) return fail(e);
    if ((e = cudaMalloc((void**)&S->head, sizeof(unsigned long long)))) return fail(e);
    if ((e = cudaMemset(S->head, 0, sizeof(unsigned long long)))) return fail(e);
    if ((e = cudaMalloc((void**)&S->d_slots, S->slot_bytes * S->slots))) return fail(e);
    if ((e = cudaMemset(S->d_slots, 0, S->slot_bytes * S->slots))) return fail(e);
    if ((e = cudaMalloc((void**)&S->d_cpriv, S->blob_max * S->slots))) return fail(e);
    if ((e = cudaMalloc((void**)&S->d_priv, sizeof(B1Prob) * S->slots))) return fail(e);
    if ((e = cudaMalloc((void**)&S->d_xpriv, sizeof(double) * S->iv_max * (size_t)S->slots))) return fail(e);
    if ((e = cudaMalloc((void**)&S->d_gpriv, sizeof(double) * S->iv_max * (size_t)S->slots))) return fail(e);
    // the loop's CTAs are placed before pending blocks of other streams as
    // SMs free up (a relaunch while context kernels fill the device)
    int prio_low = 0, prio_high = 0;
    cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    if ((e = cudaStreamCreateWithPriority(&S->loop_stream, cudaStreamNonBlocking, prio_high))) return fail(e);
    if ((e = cudaEventCreateWithFlags(&S->loop_done, cudaEventDisableTiming))) return fail(e);
    if ((e = cudaDeviceSynchronize())) return fail(e);
    S->busy.assign(S->cap, 0);
    S->owner.assign(S->cap, 0);
    S->t_submit.assign(S->cap, 0.0);
    S->t_done.assign(S->cap, 0.0);
    S->reaper = std::thread([S] { S->reap(); });
    *out = reinterpret_cast<nm_stream*>(S);
    return NM_OK;
}

int nm_stream_submit(nm_stream* st, const nm_plan* P, const double* x_host, int precision, long long* ticket) {
    using namespace nm;
    Stream1D* S = reinterpret_cast<Stream1D*>(st);
    if (!S || !P || !x_host || !ticket) { set_error("nm_stream_submit: bad argument"); return NM_ERR_ARG; }
    if (precision != NM_FP32 && precision != NM_FP64) { set_error("nm_stream_submit: bad precision"); return NM_ERR_ARG; }
    if (int rc = batch_check(P)) return rc;
    const nm_stream_options& o = S->env;
    int store = 0, blocks = 0, pairs = 0;
    for (int m = 0; m < P->n_mol; m++) {
        store += P->mols[m].n_store; blocks += P->mols[m].n_blocks; pairs += P->mols[m].n_molmon;
    }
    if (P->MX > o.max_layers || P->n_seg > o.max_segments || pairs > o.max_pairs || P->n_mol > o.max_molecules ||
        store > o.max_store || blocks > o.max_blocks || P->diis_m > o.max_diis) {
        set_error("nm_stream_submit: the problem exceeds the stream's envelope");
        return NM_ERR_INPUT;
    }
    B1PlanDev none;
    size_t scratch = 0, smem = 0;
    B1Prob H;
    if (int rc = b1_describe(P, none, H, scratch, smem)) return rc;
    if (scratch > S->slot_bytes || smem > S->smem || P->iv > S->iv_max) {
        set_error("nm_stream_submit: the problem exceeds the stream's slot");
        return NM_ERR_INPUT;
    }
    std::lock_guard<std::mutex> lk(S->mu);
    const unsigned long long t = S->tail;
    const int s = (int)(t % (unsigned long long)S->cap);
    if (S->busy[s]) { set_error("nm_stream_submit: ring full (wait for earlier requests first)"); return NM_ERR_NOMEM; }
    StreamEntry& E = S->ring[s];
    E.desc = H;
    if (int rc = stream_pack(P, E, S->blobs + (size_t)s * S->blob_max, S->blob_max)) return rc;
    E.mode = precision == NM_FP32 ? 1 : 0;
    E.iv = P->iv;
    __atomic_store_n(&E.done, 0ull, __ATOMIC_RELAXED);
    std::memcpy(S->xring + (size_t)s * S->iv_max, x_host, sizeof(double) * P->iv);
    S->busy[s] = 1;
    S->owner[s] = t;
    S->t_submit[s] = stream_now();
    __atomic_store_n(&S->ctl->tail, t + 1, __ATOMIC_RELEASE);
    S->tail = t + 1;
    *ticket = (long long)t;
    if (S->broken) { set_error("nm_stream_submit: the loop failed with a CUDA error"); return S->broken; }
    if (!S->loop_alive()) return S->launch_locked();
    return NM_OK;
}

int nm_stream_wait(nm_stream* st, long long ticket, double* x_host, nm_solve_result* res, double* seconds) {
    using namespace nm;
    Stream1D* S = reinterpret_cast<Stream1D*>(st);
    if (!S || ticket < 0) { set_error("nm_stream_wait: bad argument"); return NM_ERR_ARG; }
    const int s = (int)((unsigned long long)ticket % (unsigned long long)S->cap);
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (!S->busy[s] || S->owner[s] != (unsigned long long)ticket) {
            set_error("nm_stream_wait: unknown or already collected ticket");
            return NM_ERR_ARG;
        }
    }
    const double t0 = stream_now();
    for (;;) {
        {
            std::lock_guard<std::mutex> lk(S->mu);
            if ((unsigned long long)ticket < S->reaped) break;  // done, time recorded
            if (S->broken) { set_error("nm_stream_wait: the loop failed with a CUDA error"); return S->broken; }
        }
        if (stream_now() - t0 > 3600.0) { set_error("nm_stream_wait: no result within an hour"); return NM_ERR_TIMEOUT; }
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    std::lock_guard<std::mutex> lk(S->mu);
    const StreamEntry& E = S->ring[s];
    if (x_host) std::memcpy(x_host, S->xring + (size_t)s * S->iv_max, sizeof(double) * E.iv);
    if (res) { res->iterations = E.iterations; res->residual = E.residual; res->status = E.status; }
    if (seconds) *seconds = S->t_done[s] - S->t_submit[s];
    S->busy[s] = 0;
    return E.status == NM_OK || E.status == NM_ERR_NOT_CONVERGED ? NM_OK : E.status;
}

int nm_stream_slots(nm_stream* st) {
    Stream1D* S = reinterpret_cast<Stream1D*>(st);
    return S ? S->slots : 0;
}

long long nm_stream_launch_count(nm_stream* st) {
    Stream1D* S = reinterpret_cast<Stream1D*>(st);
    if (!S) return 0;
    std::lock_guard<std::mutex> lk(S->mu);
    return S->launches;
}

int nm_stream_destroy(nm_stream* st) {
    delete reinterpret_cast<Stream1D*>(st);
    return NM_OK;
}

}  // extern "C"
