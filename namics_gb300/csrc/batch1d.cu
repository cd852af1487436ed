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

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "ctx_internal.h"

namespace nm {

#define B1_THREADS 256
#define B1_MAXB 64      // blocks per molecule
#define B1_MAXM 16      // DIIS history in the batched path

struct B1Mol {
    int freedom, pinned, n_blocks, n_store, n_molmon, mm0;  // mm0: first (mol, molmon) pair index
    double n_in, theta_in, phibulk_in, N;
    const nm_block* blocks;
    const int* child_index;
    void* Gf;            // T[n_store*M]
    int* ef;             // exponent of each stored forward propagator (scaled mode)
    void* Pc;            // T[n_blocks*M]
    int* epc;            // exponents of Pc
    void* Q;             // T[n_blocks*M]
    int* eq;
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
    double* xR;          // [m*iv]
    double* xx0;         // [m*iv]
    // results
    int iterations, fp32_iterations, status;
    double residual, F, Omega, sw_tol;
    double sc[5 * NM_MAX_MOL];  // GN, norm, n, theta, phibulk per molecule
    double seg_phibulk[NM_MAX_SEG];
};

// ---------------------------------------------------------------- helpers
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

__device__ __forceinline__ double b1_block_max(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double r = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) r = fmax(r, red[i]);
    __syncthreads();
    return r;
}

// one 1-gradient stencil value at interior site x of array g (halo mapped)
template <typename T>
__device__ __forceinline__ T b1_stencil(const B1Prob& P, const T* g, int x) {
    int xm = x - 1 == 0 ? P.b1 : x - 1;
    int xp = x + 1 == P.MX + 1 ? P.bm : x + 1;
    if (P.geom == 0) {
        T lam = (T)P.lam;
        return lam * g[xm] + ((T)1.0 - (T)2.0 * lam) * g[x] + lam * g[xp];
    }
    return g[x] * (T)P.l0[x] + g[xm] * (T)P.lm1[x] + g[xp] * (T)P.l1[x];
}

__device__ __forceinline__ double b1_stencil_d(const B1Prob& P, const double* g, int x) {
    return b1_stencil<double>(P, g, x);
}

// Scale bookkeeping for FP32 propagators: after a step, every thread knows
// the block-wide max of the new vector (double-buffered warp slots) and the
// next step multiplies by 2^-e.
struct Scaler {
    float* slots;  // [2][32]
    int par;
};

template <typename T, bool SCALED>
struct Prop {
    // out(x) = stencil(in)(x)·w(x)·2^-e_in for interior x; returns block max
    // exponent of out when SCALED (0 otherwise).  Ends with __syncthreads.
    __device__ static int step(const B1Prob& P, const T* in, const T* w, T* out, int e_in,
                               T* gstore, Scaler& sc) {
        float lmax = 0.f;
        T f = (T)1.0;
        if (SCALED) f = (T)ldexpf(1.0f, -e_in);
        for (int x = threadIdx.x + 1; x <= P.MX; x += blockDim.x) {
            T v = b1_stencil<T>(P, in, x) * w[x];
            if (SCALED) { v = v * f; lmax = fmaxf(lmax, fabsf((float)v)); }
            out[x] = v;
            if (gstore) gstore[x] = v;
        }
        int e = 0;
        if (SCALED) {
            for (int o = 16; o > 0; o >>= 1) lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
            if ((threadIdx.x & 31) == 0) sc.slots[sc.par * 32 + (threadIdx.x >> 5)] = lmax;
        }
        __syncthreads();
        if (SCALED) {
            float gm = 0.f;
            for (int i = 0; i < (int)(blockDim.x >> 5); i++) gm = fmaxf(gm, sc.slots[sc.par * 32 + i]);
            sc.par ^= 1;
            if (gm > 0.f) frexpf(gm, &e);
        }
        return e;
    }
};

// ---------------------------------------------------------------- kernel
// Shared-memory working set of one problem.
struct B1S {
    double *G1, *phi, *phitot, *alpha, *x, *g, *rho, *red, *Aij, *Ci, *sc, *spb, *gram;
    void *cur, *nxt, *G1t;
    double *phif;
    int *phie;
    int* status;
};

// One residual evaluation g(x) (System::Classical_residual) with propagators
// of type T.  Ends with __syncthreads; S.g holds the residual.
template <typename T, bool SCALED>
__device__ void b1_residual(B1Prob& P, B1S& S, Scaler& scl) {
    const int M = P.M, MX = P.MX, ns = P.ns, nit = P.nit;
    const int tid = threadIdx.x, nth = blockDim.x;
    double *G1 = S.G1, *phi = S.phi, *phitot = S.phitot, *alpha = S.alpha, *x = S.x, *g = S.g,
           *rho = S.rho, *red = S.red, *sc = S.sc, *spb = S.spb;
    T* cur = (T*)S.cur;
    T* nxt = (T*)S.nxt;
    T* G1t = (T*)S.G1t;
    // G1 (PutU + PrepareForCalculations)
    for (int s = tid; s < M; s += nth) {
        int src = s == 0 ? P.b1 : (s == MX + 1 ? P.bm : s);
        for (int i = 0; i < ns; i++) {
            int itx = P.seg_it[i];
            double u = itx >= 0 ? x[itx * M + src] : 0.0;
            double v = exp(-u) * P.gmask[i * M + s];
            G1[i * M + s] = v;
            G1t[i * M + s] = (T)v;
        }
    }
    for (int i = tid; i < P.n_mm * M; i += nth) rho[i] = 0;
    for (int i = tid; i < 2 * M; i += nth) cur[i] = (T)0;  // halos of cur/nxt are 0
    __syncthreads();
    for (int m = 0; m < P.nmol; m++) {
        const B1Mol& D = P.mol[m];
        T* Gf = (T*)D.Gf;
        T* Pc = (T*)D.Pc;
        T* Qb = (T*)D.Q;
        // forward sweep (post-order blocks)
        for (int b = 0; b < D.n_blocks; b++) {
            const nm_block B = D.blocks[b];
            const T* w = G1t + B.seg * M;
            int s = B.s0;
            int ecur = 0;
            if (B.n_child == 0) {
                for (int xx = tid + 1; xx <= MX; xx += nth) {
                    T v = w[xx];
                    cur[xx] = v;
                    Gf[(size_t)s * M + xx] = v;
                }
                if (SCALED && tid == 0) D.ef[s] = 0;
            } else {
                // join: Gf = P(Gf[c0])·G1 · Π_c [P(Gf[c])·KSAM]^mult
                int nc = B.n_child;
                int c0 = D.child_index[B.child0];
                const nm_block C0 = D.blocks[c0];
                bool simple = (nc == 1 && C0.mult == 1);
                if (!simple) {
                    for (int c = 0; c < nc; c++) {
                        int cb = D.child_index[B.child0 + c];
                        const nm_block C = D.blocks[cb];
                        int sl = C.s0 + C.length - 1;
                        const T* src = Gf + (size_t)sl * M;
                        T* dst = Pc + (size_t)cb * M;
                        for (int xx = tid + 1; xx <= MX; xx += nth)
                            dst[xx] = b1_stencil<T>(P, src, xx) * (T)P.ksam[xx];
                        if (SCALED && tid == 0) D.epc[cb] = D.ef[sl];
                    }
                    __syncthreads();
                }
                int sl0 = C0.s0 + C0.length - 1;
                const T* src = Gf + (size_t)sl0 * M;
                int ejoin = SCALED ? D.ef[sl0] : 0;
                for (int xx = tid + 1; xx <= MX; xx += nth) {
                    T v = b1_stencil<T>(P, src, xx) * w[xx];
                    if (!simple) {
                        for (int k = 1; k < C0.mult; k++) v = v * Pc[(size_t)c0 * M + xx];
                        for (int c = 1; c < nc; c++) {
                            int cb = D.child_index[B.child0 + c];
                            int mu = D.blocks[cb].mult;
                            for (int k = 0; k < mu; k++) v = v * Pc[(size_t)cb * M + xx];
                        }
                    }
                    cur[xx] = v;
                }
                if (SCALED && !simple) {
                    ejoin += (C0.mult - 1) * D.epc[c0];
                    for (int c = 1; c < nc; c++) {
                        int cb = D.child_index[B.child0 + c];
                        ejoin += D.blocks[cb].mult * D.epc[cb];
                    }
                }
                if (SCALED) {
                    float lmax = 0.f;
                    for (int xx = tid + 1; xx <= MX; xx += nth) lmax = fmaxf(lmax, fabsf((float)cur[xx]));
                    double gm = b1_block_max((double)lmax, red);  // syncs
                    int e = 0;
                    if (gm > 0) frexp(gm, &e);
                    T f = (T)ldexp(1.0, -e);
                    for (int xx = tid + 1; xx <= MX; xx += nth) cur[xx] = cur[xx] * f;
                    ejoin += e;
                }
                for (int xx = tid + 1; xx <= MX; xx += nth) Gf[(size_t)s * M + xx] = cur[xx];
                if (SCALED && tid == 0) D.ef[s] = ejoin;
                ecur = ejoin;
            }
            // exponent of cur's max, for the first step's scale
            int enext = 0;
            if (SCALED) {
                float lmax = 0.f;
                for (int xx = tid + 1; xx <= MX; xx += nth) lmax = fmaxf(lmax, fabsf((float)cur[xx]));
                double gm = b1_block_max((double)lmax, red);
                if (gm > 0) frexp(gm, &enext);
            } else {
                __syncthreads();
            }
            for (int k = 1; k < B.length; k++) {
                s++;
                int e2 = Prop<T, SCALED>::step(P, cur, w, nxt, enext, Gf + (size_t)s * M, scl);
                if (SCALED) { ecur += enext; if (tid == 0) D.ef[s] = ecur; }
                T* t = cur; cur = nxt; nxt = t;
                enext = e2;
            }
            __syncthreads();
        }
        // G(N) = Σ Gf[root]·L (ComputeGN; planar: plain sum)
        const nm_block R = D.blocks[D.n_blocks - 1];
        int sroot = R.s0 + R.length - 1;
        int eroot = SCALED ? D.ef[sroot] : 0;
        {
            double acc = 0;
            for (int xx = tid + 1; xx <= MX; xx += nth) {
                double v = (double)Gf[(size_t)sroot * M + xx];
                acc += P.L ? v * P.L[xx] : v;
            }
            double GN = b1_block_sum(acc, red);
            if (tid == 0) { sc[5 * m + 0] = GN; sc[5 * m + 3] = (double)eroot; }
        }
        // backward sweep (pre-order, explicit stack)
        int stack[B1_MAXB];
        int sp = 0;
        stack[sp++] = D.n_blocks - 1;
        while (sp > 0) {
            int b = stack[--sp];
            const nm_block B = D.blocks[b];
            const T* w = G1t + B.seg * M;
            double* rr = rho + (D.mm0 + B.molmon) * M;
            double d = B.degeneracy;
            int s = B.s0 + B.length - 1;
            int eb = 0, enext = 0;
            if (B.parent < 0) {
                for (int xx = tid + 1; xx <= MX; xx += nth) cur[xx] = w[xx];
                if (SCALED) {
                    float lmax = 0.f;
                    for (int xx = tid + 1; xx <= MX; xx += nth) lmax = fmaxf(lmax, fabsf((float)cur[xx]));
                    double gm = b1_block_max((double)lmax, red);
                    if (gm > 0) frexp(gm, &enext);
                } else __syncthreads();
            } else {
                const T* q = Qb + (size_t)b * M;
                eb = SCALED ? D.eq[b] : 0;
                enext = Prop<T, SCALED>::step(P, q, w, cur, 0, nullptr, scl);
            }
            for (int xx = tid + 1; xx <= MX; xx += nth) {
                double f = (double)Gf[(size_t)s * M + xx] * (double)cur[xx];
                if (SCALED) f = ldexp(f, D.ef[s] + eb - eroot);
                rr[xx] += d == 1.0 ? f : d * f;
            }
            for (s = s - 1; s >= B.s0; s--) {
                int e2 = Prop<T, SCALED>::step(P, cur, w, nxt, enext, nullptr, scl);
                if (SCALED) eb += enext;
                T* t = cur; cur = nxt; nxt = t;
                enext = e2;
                for (int xx = tid + 1; xx <= MX; xx += nth) {
                    double f = (double)Gf[(size_t)s * M + xx] * (double)cur[xx];
                    if (SCALED) f = ldexp(f, D.ef[s] + eb - eroot);
                    rr[xx] += d == 1.0 ? f : d * f;
                }
            }
            __syncthreads();
            if (B.n_child == 0) continue;
            // backward starts of the children: Q = Gb(join)·Π other P(Gf)
            for (int c = 0; c < B.n_child; c++) {
                int cb = D.child_index[B.child0 + c];
                bool simple = (B.n_child == 1 && D.blocks[cb].mult == 1);
                T* q = Qb + (size_t)cb * M;
                int eq = eb;
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
                if (SCALED && !simple) {
                    eq += (D.blocks[cb].mult - 1) * D.epc[cb];
                    for (int o = 0; o < B.n_child; o++) {
                        if (o == c) continue;
                        int ob = D.child_index[B.child0 + o];
                        eq += D.blocks[ob].mult * D.epc[ob];
                    }
                }
                if (SCALED && tid == 0) D.eq[cb] = eq;
            }
            __syncthreads();
            for (int c = B.n_child - 1; c >= 0; c--) stack[sp++] = D.child_index[B.child0 + c];
        }
        __syncthreads();
    }
    // normalisation (system.cpp:2368-2560), one thread.  In scaled mode rho
    // and G(N) carry the root exponent e: rho_true = rho·2^e and
    // GN_true = GNm·2^e.  Restricted chains use n/GNm (the exponents cancel);
    // free chains and the solvent apply φb/N and 2^e.
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
        for (int k = 0; k < P.n_mm; k++) spb[P.mm_seg[k]] += P.mm_frac[k] * sc[5 * P.mm_mol[k] + 4];
    }
    __syncthreads();
    // φ, φ_tot
    for (int s = tid; s < M; s += nth) {
        bool in = s >= 1 && s <= MX;
        double pt = 0;
        for (int i = 0; i < ns; i++) {
            double v = P.phi_frozen[i * M + s];
            phi[i * M + s] = v;
            if (P.seg_frozen[i]) pt += v;
        }
        if (in) {
            for (int k = 0; k < P.n_mm; k++) {
                int sg = P.mm_seg[k], m = P.mm_mol[k];
                double g1 = G1[sg * M + s];
                double v = g1 != 0 ? rho[k * M + s] / g1 : 0.0;
                v *= S.phif[m];
                if (SCALED && S.phie[m]) v = ldexp(v, S.phie[m]);
                phi[sg * M + s] += v;
                pt += v;
            }
        }
        phitot[s] = pt;
    }
    __syncthreads();
    // residual (Classical_residual)
    for (int s = tid; s < M; s += nth) {
        if (s < 1 || s > MX) {
            for (int i = 0; i < nit; i++) g[i * M + s] = 0;
            alpha[s] = 0;
            continue;
        }
        double ps[NM_MAX_SEG];
        for (int k = 0; k < ns; k++) ps[k] = b1_stencil_d(P, phi + k * M, s);
        double pt = phitot[s];
        double gi[NM_MAX_SEG];
        double al = 0;
        for (int i = 0; i < nit; i++) {
            double v = x[i * M + s];
            int r = P.it_seg[i];
            for (int k = 0; k < ns; k++) {
                double chi = P.chi[r * ns + k];
                if (chi != 0 && pt > 0) v = v - chi * (ps[k] / pt - spb[k]);
            }
            gi[i] = v;
            al += v;
        }
        al = al * (1.0 / nit);
        alpha[s] = al;
        double km = P.ksam[s];
        for (int i = 0; i < nit; i++) {
            double v = pt > 0 ? gi[i] - al + 1 / pt - 1.0 : 0.0;
            g[i * M + s] = v * km;
        }
    }
    __syncthreads();
}

// fp32_first: FP32 propagators until ‖g‖ < P.sw_tol or a stall, then FP64
// propagators (DIIS history restarted) for the final iterations, so the
// stopping test ‖g‖ < tol is always made on an FP64 residual.
__global__ void __launch_bounds__(B1_THREADS) k_batch1d(B1Prob* __restrict__ probs, int fp32_first) {
    B1Prob& P = probs[blockIdx.x];
    extern __shared__ double sm[];
    const int M = P.M, ns = P.ns, iv = P.iv;
    const int tid = threadIdx.x, nth = blockDim.x;
    B1S S;
    S.G1 = sm;
    S.phi = S.G1 + ns * M;
    S.phitot = S.phi + ns * M;
    S.alpha = S.phitot + M;
    S.x = S.alpha + M;
    S.g = S.x + iv;
    S.rho = S.g + iv;
    S.red = S.rho + P.n_mm * M;
    S.Aij = S.red + 64;
    S.Ci = S.Aij + B1_MAXM * B1_MAXM;
    S.sc = S.Ci + B1_MAXM;
    S.spb = S.sc + 5 * NM_MAX_MOL;
    S.gram = S.spb + NM_MAX_SEG;
    double* tail = S.gram + 8 * B1_MAXM;
    S.cur = tail;                 // sized for double
    S.nxt = tail + M;
    S.G1t = tail + 2 * M;
    __shared__ float slots[64];
    __shared__ int sh_status;
    __shared__ double phif[NM_MAX_MOL];
    __shared__ int phie[NM_MAX_MOL];
    S.phif = phif; S.phie = phie; S.status = &sh_status;
    Scaler scl{slots, 0};
    double *x = S.x, *g = S.g, *red = S.red, *Aij = S.Aij, *Ci = S.Ci, *gram = S.gram;

    for (int i = tid; i < iv; i += nth) x[i] = P.x[i];
    for (int i = tid; i < B1_MAXM * B1_MAXM; i += nth) Aij[i] = 0;
    if (tid == 0) sh_status = 0;
    __syncthreads();

    bool use32 = fp32_first != 0;
    int it = 0, k_diis = 0, fp32_its = 0;
    double resid = 0, best = 1e300;
    int since_best = 0;
    for (;;) {
        if (use32) { b1_residual<float, true>(P, S, scl); fp32_its++; }
        else b1_residual<double, false>(P, S, scl);
        if (sh_status) break;
        // ---------------- DIIS (iterate_DIIS / DIIS / Ax) ----------------
        int k = it % P.m;
        double* xRk = P.xR + (size_t)k * iv;
        double* xxk = P.xx0 + (size_t)k * iv;
        double gsq = 0;
        for (int i = tid; i < iv; i += nth) {
            double xo = x[i], gv = g[i];
            double xn = xo + (-P.dmax) * gv;
            x[i] = xn;
            xRk[i] = xn;
            xxk[i] = xn - xo;
            gsq = P.max_norm ? fmax(gsq, fabs(gv)) : gsq + gv * gv;
        }
        resid = P.max_norm ? b1_block_max(gsq, red) : sqrt(b1_block_sum(gsq, red));
        if (it > 0) k_diis++;  // iteration 0 is the plain mixing step
        if (k_diis > 0) {
            int kd = k_diis > P.m ? P.m : k_diis;
            double acc[B1_MAXM];
            for (int i = 0; i < kd; i++) acc[i] = 0;
            for (int j = tid; j < iv; j += nth) {
                double bk = xxk[j];
                for (int i = 0; i < kd; i++) {
                    int posi = k - kd + 1 + i;
                    if (posi < 0) posi += P.m;
                    acc[i] += P.xx0[(size_t)posi * iv + j] * bk;
                }
            }
            int w = tid >> 5, l = tid & 31;
            for (int i = 0; i < kd; i++) {
                double v = acc[i];
                for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
                if (l == 0) gram[w * B1_MAXM + i] = v;
            }
            __syncthreads();
            if (tid == 0) {
                int m = P.m;
                if (k_diis > m)
                    for (int i = 1; i < m; i++)
                        for (int j = 1; j < m; j++) Aij[m * (i - 1) + j - 1] = Aij[m * i + j];
                for (int i = 0; i < kd; i++) {
                    double D = 0;
                    for (int ww = 0; ww < nth / 32; ww++) D += gram[ww * B1_MAXM + i];
                    Aij[i + m * (kd - 1)] = Aij[kd - 1 + m * i] = D + 1e-9;
                }
                double A[B1_MAXM * B1_MAXM], c[B1_MAXM];
                bool nan = false;
                for (int i = 0; i < kd; i++)
                    for (int j = 0; j < kd; j++) {
                        double v = Aij[j + m * i];
                        if (v != v) nan = true;
                        A[i * kd + j] = v;
                    }
                if (nan) sh_status = NM_ERR_NAN_DIIS;
                else {
                    nm_small_solve(A, c, kd);
                    double nC = 0;
                    for (int i = 0; i < kd; i++) nC += c[i];
                    for (int i = 0; i < kd; i++) {
                        Ci[i] = c[i] / nC;
                        if (Ci[i] != Ci[i]) sh_status = NM_ERR_NAN_SVD;
                    }
                }
            }
            __syncthreads();
            if (sh_status) break;
            for (int j = tid; j < iv; j += nth) {
                double v = 0;
                for (int i = 0; i < kd; i++) {
                    int posi = k - kd + 1 + i;
                    if (posi < 0) posi += P.m;
                    v += Ci[i] * P.xR[(size_t)posi * iv + j];
                }
                x[j] = v;
            }
            __syncthreads();
        }
        if (use32) {
            // leave the FP32 phase on reaching the switch tolerance or stalling
            if (resid < 0.9 * best) { best = resid; since_best = 0; } else since_best++;
            if (!(resid > P.sw_tol) || since_best > 25) {
                use32 = false;
                k_diis = 0;  // restart the DIIS history on the FP64 residual
                best = 1e300;
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
    for (int i = tid; i < iv; i += nth) P.x[i] = x[i];
    if (tid == 0) {
        P.iterations = it;
        P.fp32_iterations = fp32_its;
        P.residual = resid;
        P.status = sh_status ? sh_status : (resid > P.tol || use32 ? NM_ERR_NOT_CONVERGED : NM_OK);
        for (int i = 0; i < 5 * P.nmol; i++) P.sc[i] = S.sc[i];
        for (int i = 0; i < ns; i++) P.seg_phibulk[i] = S.spb[i];
    }
}

// ------------------------------------------------------------------ host
struct Batch {
    std::vector<const nm_plan*> plans;
    std::vector<B1Prob> hp;
    B1Prob* d_probs = nullptr;
    std::vector<void*> allocs;
    double* d_x = nullptr;
    std::vector<long long> offsets;
    int precision = NM_FP64;
    size_t smem = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    long long launches = 0;

    template <typename X>
    int alloc(X** p, size_t n) {
        if (n == 0) n = 1;
        cudaError_t e = cudaMalloc((void**)p, sizeof(X) * n);
        if (e != cudaSuccess) { set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e)); return NM_ERR_NOMEM; }
        allocs.push_back((void*)*p);
        cudaMemset(*p, 0, sizeof(X) * n);
        return NM_OK;
    }
    template <typename X>
    int upload(X** p, const X* h, size_t n) {
        int rc = alloc(p, n);
        if (rc) return rc;
        cudaError_t e = cudaMemcpy(*p, h, sizeof(X) * n, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
        return NM_OK;
    }
    ~Batch() {
        for (void* p : allocs) cudaFree(p);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
};

#define TRYB(x) do { int r_ = (x); if (r_) return r_; } while (0)

static int batch_init(Batch& B, const nm_plan* const* plans, int n, const nm_ctx_options* opt) {
    B.precision = opt ? opt->precision : NM_FP64;
    int dev = opt ? opt->device : 0;
    cudaError_t e = cudaSetDevice(dev);
    if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    if (opt && opt->stream) B.stream = (cudaStream_t)opt->stream;
    else { cudaStreamCreateWithFlags(&B.stream, cudaStreamNonBlocking); B.own_stream = true; }
    size_t tsz = sizeof(double);  // storage sized for the FP64 phase
    long long off = 0;
    size_t maxsmem = 0;
    B.hp.resize(n);
    B.offsets.resize(n + 1);
    for (int p = 0; p < n; p++) {
        const nm_plan* P = plans[p];
        B.plans.push_back(P);
        if (P->gradients != 1) { set_error("batched solver takes 1-gradient problems only"); return NM_ERR_INPUT; }
        if (P->charged) { set_error("charged systems are not supported by the batched solver"); return NM_ERR_INPUT; }
        if (P->n_seg > NM_MAX_SEG || P->n_mol > NM_MAX_MOL || P->diis_m > B1_MAXM) {
            set_error("problem exceeds the batched solver's limits (segments, molecules, DIIS m <= 16)");
            return NM_ERR_INPUT;
        }
        B1Prob& H = B.hp[p];
        std::memset(&H, 0, sizeof(H));
        int M = P->M;
        H.MX = P->MX; H.M = M; H.geom = P->geometry; H.ns = P->n_seg; H.nit = P->n_it;
        H.nmol = P->n_mol; H.solvent = P->solvent; H.m = P->diis_m; H.itlim = P->iterationlimit;
        H.max_norm = P->max_norm; H.iv = P->iv; H.lam = P->lambda; H.tol = P->tolerance; H.dmax = P->deltamax;
        H.b1 = P->bc[0] == NM_BC_MIRROR ? 1 : P->bc[0] == NM_BC_PERIODIC ? P->MX : 0;
        H.bm = P->bc[3] == NM_BC_MIRROR ? P->MX : P->bc[3] == NM_BC_PERIODIC ? 1 : P->MX + 1;
        double *dL, *dk, *dg, *dpf;
        if (P->geometry != NM_PLANAR) {
            double *a, *b, *c;
            TRYB(B.upload(&a, P->lambda_1, M)); TRYB(B.upload(&b, P->lambda0, M)); TRYB(B.upload(&c, P->lambda1, M));
            H.lm1 = a; H.l0 = b; H.l1 = c;
            TRYB(B.upload(&dL, P->L, M));
            H.L = dL;
        } else H.L = nullptr;
        std::vector<double> ks(M);
        for (int s = 0; s < M; s++) ks[s] = P->ksam[s];
        TRYB(B.upload(&dk, ks.data(), M)); H.ksam = dk;
        TRYB(B.upload(&dg, P->seg_gmask, (size_t)P->n_seg * M)); H.gmask = dg;
        TRYB(B.upload(&dpf, P->seg_phi_frozen, (size_t)P->n_seg * M)); H.phi_frozen = dpf;
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
            if (mol.n_blocks > B1_MAXB) { set_error("molecule has too many blocks for the batched solver"); return NM_ERR_INPUT; }
            B1Mol& D = H.mol[m];
            D.freedom = mol.freedom; D.pinned = mol.pinned; D.n_blocks = mol.n_blocks; D.n_store = mol.n_store;
            D.n_molmon = mol.n_molmon; D.mm0 = kk;
            D.n_in = mol.n; D.theta_in = mol.theta; D.phibulk_in = mol.phibulk; D.N = mol.chainlength;
            nm_block* db; int* dci;
            TRYB(B.upload(&db, mol.blocks, mol.n_blocks));
            std::vector<int> ci(mol.child_index, mol.child_index + (mol.n_blocks > 1 ? mol.n_blocks - 1 : 0));
            if (ci.empty()) ci.push_back(0);
            TRYB(B.upload(&dci, ci.data(), ci.size()));
            D.blocks = db; D.child_index = dci;
            char *gf, *pc, *q;
            TRYB(B.alloc(&gf, tsz * (size_t)mol.n_store * M)); D.Gf = gf;
            TRYB(B.alloc(&pc, tsz * (size_t)mol.n_blocks * M)); D.Pc = pc;
            TRYB(B.alloc(&q, tsz * (size_t)mol.n_blocks * M)); D.Q = q;
            int *ef, *epc, *eq;
            TRYB(B.alloc(&ef, mol.n_store)); TRYB(B.alloc(&epc, mol.n_blocks)); TRYB(B.alloc(&eq, mol.n_blocks));
            D.ef = ef; D.epc = epc; D.eq = eq;
            for (int j = 0; j < mol.n_molmon; j++) {
                if (kk >= NM_MAX_MM) { set_error("too many (molecule, segment) pairs"); return NM_ERR_INPUT; }
                H.mm_mol[kk] = m; H.mm_seg[kk] = mol.molmon_seg[j]; H.mm_frac[kk] = mol.molmon_fraction[j];
                kk++;
            }
        }
        H.n_mm = kk;
        double *xR, *xx0;
        TRYB(B.alloc(&xR, (size_t)P->diis_m * P->iv)); TRYB(B.alloc(&xx0, (size_t)P->diis_m * P->iv));
        H.xR = xR; H.xx0 = xx0;
        B.offsets[p] = off;
        off += P->iv;
        H.sw_tol = 2e-6;
        size_t smem = sizeof(double) * ((size_t)(2 * P->n_seg + 2) * M + 2 * (size_t)P->iv + (size_t)kk * M + 64 +
                                        B1_MAXM * B1_MAXM + B1_MAXM + 5 * NM_MAX_MOL + NM_MAX_SEG + 8 * B1_MAXM +
                                        (size_t)2 * M + (size_t)P->n_seg * M) + 64;
        maxsmem = std::max(maxsmem, smem);
    }
    B.offsets[n] = off;
    TRYB(B.alloc(&B.d_x, (size_t)off));
    for (int p = 0; p < n; p++) B.hp[p].x = B.d_x + B.offsets[p];
    TRYB(B.alloc(&B.d_probs, (size_t)n));
    B.smem = maxsmem;
    if (maxsmem > 220 * 1024) { set_error("problem too large for the batched solver's shared memory"); return NM_ERR_INPUT; }
    cudaError_t e1 = cudaFuncSetAttribute(k_batch1d, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)maxsmem);
    if (e1 != cudaSuccess) { set_error("cudaFuncSetAttribute failed"); return NM_ERR_CUDA; }
    return NM_OK;
}

static int batch_run(Batch& B) {
    int n = (int)B.hp.size();
    cudaError_t e = cudaMemcpyAsync(B.d_probs, B.hp.data(), sizeof(B1Prob) * n, cudaMemcpyHostToDevice, B.stream);
    if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    k_batch1d<<<n, B1_THREADS, B.smem, B.stream>>>(B.d_probs, B.precision == NM_FP32 ? 1 : 0);
    B.launches++;
    e = cudaGetLastError();
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
