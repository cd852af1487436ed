// Device context: the SCF hot path for one problem of any gradient count.
//
// Per residual evaluation (System::Classical_residual, system.cpp:2087-2189):
//   k_g1          G1 = exp(-u)·mask·KSAM        (segment.cpp:855-879)
//   per molecule  forward sweep  k_prop         (molecule.cpp:2300-2362)
//                 G(N)           k_wsum_*       (LGrad*::ComputeGN)
//                 backward sweep k_prop_back    (molecule.cpp:2364-2446)
//                 fused with composition rho += d·Gf·Gb (LGrad1.cpp:876-922)
//   k_norms       normalisation of every molecule (system.cpp:2368-2560)
//   k_phi         φ = rho/G1·norm, φ_tot       (system.cpp:2438-2610)
//   k_residual    φ_side stencil + χ terms + α + incompressibility + KSAM
// and, for a charged system (elec.cu), k_field (ψ bounds, EE) before k_g1
// and k_charge + the Poisson update (ψ block of g) after k_residual.
// and per DIIS iteration (sfnewton.cpp:1078-1095, 837-880):
//   k_diis_step   x -= δ·g, history slot, ‖g‖² partials
//   k_gram        Gram row of the history (deterministic two-pass sums)
//   host          small solve A c = 1 by pseudo-inverse, c /= Σc (FP64)
//   k_diis_mix    x = Σ c_i xR_i
// All arithmetic is FP64; all reductions are two-pass with a fixed grid, so
// repeated runs are bit-identical.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ctx_internal.h"

using nmdev::Lat;

namespace nm {

#define CK(call)                                                                   \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) {                                                   \
            set_error(std::string("CUDA: ") + cudaGetErrorString(e_) + " at " +    \
                      __FILE__ + ":" + std::to_string(__LINE__));                  \
            return NM_ERR_CUDA;                                                    \
        }                                                                          \
    } while (0)

static const int RED_THREADS = 256;
thread_local bool g_plain_launch = false;

// ---------------------------------------------------------------- kernels --

// u = x (+ the charged terms −ε·EE + v·ψ, system.cpp:2001-2030) at the
// set_bounds source of each site; G1 = exp(−u)·mask·KSAM
// A segment with internal states: G1 = Σ_j α_bulk,j·exp(-u_j) over its
// states, each u_j from the state's block with the state's valence, and
// α_j = α_bulk,j·exp(-u_j)/G1 (segment.cpp:861-873); u_j and α_j are kept
// for the free energy and the states' volume fractions.
__global__ void k_g1(Lat L, int ns, const double* __restrict__ x, const int* __restrict__ seg_it,
                     const double* __restrict__ gmask, double* __restrict__ G1, float* __restrict__ G1f,
                     ChgArgs chg, const double* __restrict__ EE, const double* __restrict__ psi,
                     StArgs st, double* __restrict__ ust, double* __restrict__ ast) {
    int M = L.M;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < M; s += gridDim.x * blockDim.x) {
        int src = nmdev::bc_source(L, s);
        for (int i = 0; i < ns; i++) {
            int it = seg_it[i];
            if (it < 0 && st.n > 0) {
                bool with_states = false;
                for (int j = 0; j < st.n; j++) with_states = with_states || st.seg[j] == i;
                if (with_states) {
                    double g1 = 0;
                    for (int j = 0; j < st.n; j++) {
                        if (st.seg[j] != i) continue;
                        double u = x[(size_t)st.it[j] * M + src];
                        if (chg.on) {
                            u += -1.0 * chg.eps[i] * EE[src];
                            if (chg.val[ns + j] != 0) u += chg.val[ns + j] * psi[src];
                        }
                        const double a = exp(-u) * st.ab[j];
                        ust[(size_t)j * M + s] = u;
                        ast[(size_t)j * M + s] = a;
                        g1 += a;
                    }
                    for (int j = 0; j < st.n; j++)
                        if (st.seg[j] == i) {
                            double& a = ast[(size_t)j * M + s];
                            a = g1 != 0 ? a / g1 : 0.0;
                        }
                    const double v = g1 * gmask[(size_t)i * M + s];
                    if (G1f) {
                        const float f = (float)v;
                        G1f[(size_t)i * M + s] = f;
                        G1[(size_t)i * M + s] = (double)f;
                    } else {
                        G1[(size_t)i * M + s] = v;
                    }
                    continue;
                }
            }
            double u = it >= 0 ? x[(size_t)it * M + src] : 0.0;
            if (chg.on && it >= 0) {
                u += -1.0 * chg.eps[i] * EE[src];
                if (chg.val[i] != 0) u += chg.val[i] * psi[src];
            }
            if (G1f) {
                // FP32 phase: one FP32 exp serves both copies (the FP64 copy,
                // used by φ = ρ/G1, then matches the propagators' G1 exactly)
                float v = expf(-(float)u) * (float)gmask[(size_t)i * M + s];
                G1f[(size_t)i * M + s] = v;
                G1[(size_t)i * M + s] = (double)v;
            } else {
                G1[(size_t)i * M + s] = exp(-u) * gmask[(size_t)i * M + s];
            }
        }
    }
}

// out = stencil(in)·G1 at interior sites (G1 may be null: ≡ 1)
__global__ void k_prop(Lat L, const double* __restrict__ in, const double* __restrict__ G1,
                       double* __restrict__ out) {
    nmdev::pdl_begin();
    int n = nmdev::interior_count(L);
    nmdev::GLoad<double> ld{in};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int x, y, z;
        nmdev::site_coords(L, i, x, y, z);
        int s = x * L.JX + y * L.JY + z;
        double v = nmdev::stencil_at(L, ld, x, y, z);
        out[s] = G1 ? v * G1[s] : v;
    }
    nmdev::pdl_end();
}

// backward step fused with composition: out = stencil(in)·G1; rho += d·Gf·out.
// nh > 0 (charged systems): also the halo part of rho, the flat-array step
// at each halo site times the bounded Gf there (out's halo is not stored:
// the next step reads it through set_bounds).
__global__ void k_prop_back(Lat L, const double* __restrict__ in, const double* __restrict__ G1,
                            double* __restrict__ out, const double* __restrict__ Gf,
                            double* __restrict__ rho, double d, int nh) {
    nmdev::pdl_begin();
    int n = nmdev::interior_count(L);
    nmdev::GLoad<double> ld{in};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n + nh; i += gridDim.x * blockDim.x) {
        if (i >= n) {
            const int h = L.g == 3 ? i - n : nmdev::halo_site(L, i - n);
            if (L.g == 3 && nmdev::is_interior(L, h)) continue;
            nmdev::BLoad bl{in, L};
            const double v = nmdev::flat_prop_at(L, bl, h) * G1[h];
            const double gf = Gf[nmdev::bc_source(L, h)];
            if (d == 1.0) rho[h] += gf * v;
            else rho[h] += d * gf * v;
            continue;
        }
        int x, y, z;
        nmdev::site_coords(L, i, x, y, z);
        int s = x * L.JX + y * L.JY + z;
        double v = nmdev::stencil_at(L, ld, x, y, z) * G1[s];
        out[s] = v;
        if (d == 1.0) rho[s] += Gf[s] * v;
        else rho[s] += d * Gf[s] * v;
    }
    nmdev::pdl_end();
}

// root of the backward sweep: out = G1; rho += d·Gf·G1
__global__ void k_back_init(Lat L, const double* __restrict__ G1, double* __restrict__ out,
                            const double* __restrict__ Gf, double* __restrict__ rho, double d) {
    nmdev::pdl_begin();
    int n = nmdev::interior_count(L);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int x, y, z;
        nmdev::site_coords(L, i, x, y, z);
        int s = x * L.JX + y * L.JY + z;
        double v = G1[s];
        out[s] = v;
        if (d == 1.0) rho[s] += Gf[s] * v;
        else rho[s] += d * Gf[s] * v;
    }
    nmdev::pdl_end();
}

__global__ void k_copy_interior(Lat L, const double* __restrict__ in, double* __restrict__ out) {
    nmdev::pdl_begin();
    int n = nmdev::interior_count(L);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int x, y, z;
        nmdev::site_coords(L, i, x, y, z);
        int s = x * L.JX + y * L.JY + z;
        out[s] = in[s];
    }
    nmdev::pdl_end();
}

// out *= a^pow (interior)
__global__ void k_mul_pow(Lat L, double* __restrict__ out, const double* __restrict__ a, int pw) {
    nmdev::pdl_begin();
    int n = nmdev::interior_count(L);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int x, y, z;
        nmdev::site_coords(L, i, x, y, z);
        int s = x * L.JX + y * L.JY + z;
        double v = out[s];
        for (int k = 0; k < pw; k++) v *= a[s];
        out[s] = v;
    }
    nmdev::pdl_end();
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
    // fixed-order block reduction (deterministic)
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    double r = 0;
    if (threadIdx.x == 0) {
        int nw = (blockDim.x + 31) >> 5;
        for (int i = 0; i < nw; i++) r += sh[i];
    }
    __syncthreads();
    return r;
}

// partial sums of X (times L when given) over interior sites
__global__ void k_wsum_partial(Lat L, const double* __restrict__ X, const double* __restrict__ W,
                               double* __restrict__ partial) {
    __shared__ double sh[32];
    int n = nmdev::interior_count(L);
    double acc = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int x, y, z;
        nmdev::site_coords(L, i, x, y, z);
        int s = x * L.JX + y * L.JY + z;
        acc += W ? X[s] * W[s] : X[s];
    }
    double r = block_sum(acc, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = r;
}

__global__ void k_final_sum(const double* __restrict__ partial, int nb, double* __restrict__ out) {
    __shared__ double sh[32];
    double acc = 0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) acc += partial[i];
    double r = block_sum(acc, sh);
    if (threadIdx.x == 0) *out = r;
}

// molecule scalars: [GN, norm, n, theta, phibulk] per molecule
__global__ void k_norms(NormArgs a, double* __restrict__ sc, double* __restrict__ seg_phibulk,
                        int* __restrict__ status) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double A = 0, B = 0;
    int st = 0;
    for (int m = 0; m < a.n_mol; m++) {
        const MolScal& M = a.mol[m];
        double* s = sc + 5 * m;
        double GN = s[0], norm = 0;
        s[2] = M.n_in; s[3] = M.theta_in;
        if (M.freedom == NM_MOL_FREE) {
            s[4] = M.phibulk_in;
            norm = M.phibulk_in / M.N;
            s[2] = norm * GN;
            s[3] = s[2] * M.N;  // θ = n·N, as for the solvent below
            A += M.phibulk_in * M.charge; B += M.phibulk_in;
        } else if (M.freedom == NM_MOL_RESTRICTED) {
            if (GN > 0) {
                norm = M.n_in / GN;
                if (M.pinned) s[4] = 0;
                else { s[4] = M.N * norm; A += s[4] * M.charge; B += s[4]; }
            } else { st = NM_ERR_GN; norm = 0; }
        } else s[4] = 0;
        s[1] = norm;
    }
    if (a.neutralizer >= 0) {
        // the neutraliser's bulk fraction makes the bulk neutral
        // (system.cpp:2487-2515, 2560-2570)
        const MolScal& Nt = a.mol[a.neutralizer];
        double* s = sc + 5 * a.neutralizer;
        const double qs = a.solvent >= 0 ? a.mol[a.solvent].charge : 0.0;
        if (Nt.charge != qs) s[4] = ((B - 1.0) * qs - A) / (Nt.charge - qs);
        B += s[4];
        double norm = s[4] / Nt.N;
        s[2] = norm * s[0];
        s[3] = s[2] * Nt.N;
        s[1] = norm;
    }
    if (a.solvent >= 0) {
        double* s = sc + 5 * a.solvent;
        s[4] = 1.0 - B;
        if (s[4] < 0 && st == 0) st = NM_ERR_NEG_SOLVENT;
        double norm = s[4] / a.mol[a.solvent].N;
        s[2] = norm * s[0];
        s[3] = s[2] * a.mol[a.solvent].N;
        s[1] = norm;
    }
    for (int i = 0; i < a.ns; i++) seg_phibulk[i] = 0;
    for (int k = 0; k < a.n_mm; k++) seg_phibulk[a.mm_seg[k]] += a.mm_frac[k] * sc[5 * a.mm_mol[k] + 4];
    // states: φ_bulk,j = φ_bulk·α_bulk,j (Segment::SetPhiSide, segment.cpp:1339-1343)
    for (int j = 0; j < a.st.n; j++) seg_phibulk[a.ns + j] = seg_phibulk[a.st.seg[j]] * a.st.ab[j];
    if (st) *status = st;
}

// φ = frozen + rho/G1·norm and φ_tot.  halo != 0 (charged systems): φ_tot
// at halo sites also takes the halo part of rho, as the reference's flat
// arrays do (φ itself is read through set_bounds there).
__global__ void k_phi(Lat L, PhiArgs a, const double* __restrict__ sc, const double* __restrict__ G1,
                      const double* __restrict__ phi_frozen, const int* __restrict__ seg_frozen,
                      double* __restrict__ phi, double* __restrict__ phitot,
                      double* __restrict__ mol_phitot, int halo) {
    int M = L.M;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < M; s += gridDim.x * blockDim.x) {
        bool in = nmdev::is_interior(L, s);
        double pt = 0;
        for (int i = 0; i < a.ns; i++) {
            double v = phi_frozen[(size_t)i * M + s];
            phi[(size_t)i * M + s] = v;
            if (seg_frozen[i]) pt += v;
        }
        for (int m = 0; m < a.n_mol; m++) mol_phitot[(size_t)m * M + s] = 0;
        if (in) {
            for (int k = 0; k < a.n_mm; k++) {
                int sg = a.mm_seg[k], m = a.mm_mol[k];
                double g1 = G1[(size_t)sg * M + s];
                double v = g1 != 0 ? a.mm_rho[k][s] / g1 : 0.0;
                double norm = sc[5 * m + 1];
                if (norm > 0) v *= norm;
                phi[(size_t)sg * M + s] += v;
                pt += v;
                mol_phitot[(size_t)m * M + s] += v;
            }
        } else if (halo) {
            for (int k = 0; k < a.n_mm; k++) {
                int sg = a.mm_seg[k], m = a.mm_mol[k];
                double g1 = G1[(size_t)sg * M + s];
                double v = g1 != 0 ? a.mm_rho[k][s] / g1 : 0.0;
                double norm = sc[5 * m + 1];
                if (norm > 0) v *= norm;
                pt += v;
            }
        }
        phitot[s] = pt;
        // the states' volume fractions φ_j = α_j·φ(seg), rows after the
        // segments' (Segment::SetPhiSide, segment.cpp:1337-1343)
        for (int j = 0; j < a.st.n; j++)
            phi[(size_t)(a.ns + j) * M + s] = a.ast[(size_t)j * M + s] * phi[(size_t)a.st.seg[j] * M + s];
    }
}

__global__ void k_residual(Lat L, ResArgs a, const double* __restrict__ x, const double* __restrict__ phi,
                           const double* __restrict__ phitot, const double* __restrict__ seg_phibulk,
                           const double* __restrict__ ksam, double* __restrict__ g,
                           double* __restrict__ alpha, double* __restrict__ phi_side) {
    int M = L.M;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < M; s += gridDim.x * blockDim.x) {
        if (!nmdev::is_interior(L, s)) {
            for (int i = 0; i < a.nit; i++) g[(size_t)i * M + s] = 0;
            alpha[s] = 0;
            for (int k = 0; k < a.ns; k++) phi_side[(size_t)k * M + s] = 0;
            continue;
        }
        int cx, cy, cz;
        if (L.g == 1) { cx = s; cy = 0; cz = 0; }
        else if (L.g == 2) { cx = s / L.JX; cy = s % L.JX; cz = 0; }
        else { cx = s / L.JX; int r = s % L.JX; cy = r / L.JY; cz = r % L.JY; }
        double ps[NM_MAX_SEG];
        for (int k = 0; k < a.ns; k++) {
            if (!a.sp_on[k]) { ps[k] = 0; phi_side[(size_t)k * M + s] = 0; continue; }
            nmdev::GLoad<double> ld{phi + (size_t)k * M};
            ps[k] = nmdev::stencil_at(L, ld, cx, cy, cz);
            phi_side[(size_t)k * M + s] = ps[k];
        }
        double pt = phitot[s];
        double gi[NM_MAX_SEG];
        double al = 0;
        for (int i = 0; i < a.nit; i++) {
            double v = x[(size_t)i * M + s];
            int r = a.it_seg[i];
            for (int k = 0; k < a.ns; k++) {
                double chi = a.sp_on[k] ? a.chi[r * a.ns + k] : 0.0;
                if (chi != 0 && pt > 0) v = v - chi * (ps[k] / pt - seg_phibulk[k]);
            }
            gi[i] = v;
            al += v;
        }
        al = al * (1.0 / a.nit);
        alpha[s] = al;
        double km = ksam[s];
        for (int i = 0; i < a.nit; i++) {
            double v = pt > 0 ? gi[i] - al + 1 / pt - 1.0 : 0.0;
            g[(size_t)i * M + s] = v * km;
        }
    }
}

// x_new = x - δ·g ; xR[k] = x_new ; x_x0[k] = x_new - x ; partial Σ g² (or max|g|)
// x ← x − δ·g into history slot k, and the partial norms of g.  update = 0:
// the norms only, x untouched (checks an FP32 residual before x moves).
__global__ void k_diis_step(int n, double dmax, double* __restrict__ x, const double* __restrict__ g,
                            double* __restrict__ xR, double* __restrict__ xx0,
                            double* __restrict__ partial, int max_norm, int update = 1) {
    __shared__ double sh[32];
    double acc = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double gv = g[i];
        if (update) {
            double xo = x[i];
            double xn = xo + (-dmax) * gv;
            x[i] = xn;
            if (xR) xR[i] = xn;
            if (xx0) xx0[i] = xn - xo;
        }
        if (max_norm) acc = fmax(acc, fabs(gv));
        else acc += gv * gv;
    }
    if (max_norm) {
        for (int o = 16; o > 0; o >>= 1) acc = fmax(acc, __shfl_down_sync(0xffffffffu, acc, o));
        int w = threadIdx.x >> 5, l = threadIdx.x & 31;
        if (l == 0) sh[w] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double r = 0;
            for (int i = 0; i < (int)(blockDim.x >> 5); i++) r = fmax(r, sh[i]);
            partial[blockIdx.x] = r;
        }
    } else {
        double r = block_sum(acc, sh);
        if (threadIdx.x == 0) partial[blockIdx.x] = r;
    }
}

__global__ void k_final_norm(const double* __restrict__ partial, int nb, double* __restrict__ out, int max_norm) {
    __shared__ double sh[32];
    if (max_norm) {
        if (threadIdx.x == 0) {
            double r = 0;
            for (int i = 0; i < nb; i++) r = fmax(r, partial[i]);
            *out = r;
        }
        return;
    }
    double acc = 0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) acc += partial[i];
    double r = block_sum(acc, sh);
    if (threadIdx.x == 0) *out = sqrt(r);
}

// Gram row: partial[i*nb + b] = Σ_b x_x0[posi_i]·x_x0[k]
__global__ void k_gram(int n, const double* __restrict__ xx0, int k, int kd, int m,
                       double* __restrict__ partial) {
    __shared__ double sh[32];
    int i = blockIdx.y;
    int posi = k - kd + 1 + i;
    if (posi < 0) posi += m;
    const double* a = xx0 + (size_t)posi * n;
    const double* b = xx0 + (size_t)k * n;
    double acc = 0;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) acc += a[j] * b[j];
    double r = block_sum(acc, sh);
    if (threadIdx.x == 0) partial[(size_t)i * gridDim.x + blockIdx.x] = r;
}

// Finish the Gram row from its per-block partial sums (fixed order), slide
// the m×m window, set row/column kd-1 to ⟨Δx_i, Δx_k⟩ + 1e-9, solve A c = 1
// by the pseudo-inverse and normalise c /= Σc (SFNewton::DIIS and Ax,
// sfnewton.cpp:837-880, 793-835).  Host side; Aij is the m×m window.
static int diis_coefficients(const double* partial, int nb, int kd_in, int m, double* Aij, double* Ci) {
    int kd = kd_in;
    if (kd > m) {
        kd = m;
        for (int i = 1; i < m; i++)
            for (int j = 1; j < m; j++) Aij[m * (i - 1) + j - 1] = Aij[m * i + j];
    }
    for (int i = 0; i < kd; i++) {
        double D = 0;
        for (int b = 0; b < nb; b++) D += partial[(size_t)i * nb + b];
        Aij[i + m * (kd - 1)] = Aij[kd - 1 + m * i] = D + 1e-9;
    }
    double A[NM_MAX_DIIS * NM_MAX_DIIS], c[NM_MAX_DIIS];
    for (int i = 0; i < kd; i++)
        for (int j = 0; j < kd; j++) {
            double v = Aij[j + m * i];
            if (v != v) { set_error("NaN in the DIIS matrix"); return NM_ERR_NAN_DIIS; }
            A[i * kd + j] = v;
        }
    nm_pinv_solve(A, c, kd);
    double normC = 0;
    for (int i = 0; i < kd; i++) normC += c[i];
    for (int i = 0; i < kd; i++) {
        Ci[i] = c[i] / normC;
        if (Ci[i] != Ci[i]) { set_error("NaN in the DIIS coefficients"); return NM_ERR_NAN_SVD; }
    }
    return NM_OK;
}

__global__ void k_diis_mix(int n, double* __restrict__ x, const double* __restrict__ xR,
                           const double* __restrict__ Ci, int k, int kd_in, int m) {
    int kd = kd_in > m ? m : kd_in;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        double v = 0;
        for (int i = 0; i < kd; i++) {
            int posi = k - kd + 1 + i;
            if (posi < 0) posi += m;
            v += Ci[i] * xR[(size_t)posi * n + j];
        }
        x[j] = v;
    }
}

// free-energy and grand-potential densities (system.cpp:2809-3244)
// Species (segments, then states; a segment with states takes part through
// them): sp_on[k] = 0 for a segment with states, frozen[k] for frozen
// segments (never a state).  ns = segments, nsp = species.
struct FeArgs {
    int ns, nsp, n_mol, charged;
    const double *q, *psi, *EE, *eps;  // charged systems
    const double* ust;                 // u of each state (internal states)
    int seg_frozen[NM_MAX_SEG], seg_in_mol[NM_MAX_SEG], sp_on[NM_MAX_SEG];
    int st_seg[NM_MAX_SEG];
    double chi[NM_MAX_SEG * NM_MAX_SEG];
    double cF[NM_MAX_MOL], cF2[NM_MAX_MOL], invN[NM_MAX_MOL];
};

__global__ void k_fe_density(Lat L, FeArgs a, const double* __restrict__ sc, const double* __restrict__ phi,
                             const double* __restrict__ phi_side, const double* __restrict__ G1,
                             const double* __restrict__ mol_phitot, const double* __restrict__ alpha,
                             const double* __restrict__ seg_phibulk, const double* __restrict__ ksam,
                             double* __restrict__ F, double* __restrict__ GP) {
    int M = L.M;
    const int ns = a.ns, nsp = a.nsp;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < M; s += gridDim.x * blockDim.x) {
        if (!nmdev::is_interior(L, s)) { F[s] = 0; GP[s] = 0; continue; }
        double f = 0, gp = 0;
        for (int m = 0; m < a.n_mol; m++) f += a.cF[m] * mol_phitot[(size_t)m * M + s];
        for (int i = 0; i < ns; i++) {
            if (!a.seg_in_mol[i]) continue;
            if (!a.sp_on[i]) {  // a segment with states: -φ_j·u_j per state (system.cpp:2866-2888)
                for (int j = 0; j < nsp - ns; j++)
                    if (a.st_seg[j] == i)
                        f += -1.0 * (phi[(size_t)(ns + j) * M + s] * a.ust[(size_t)j * M + s]);
                continue;
            }
            double g1 = G1[(size_t)i * M + s];
            double ml = g1 > 0 ? -log(g1) : 0.0;
            f += -1.0 * (phi[(size_t)i * M + s] * ml);
        }
        // χ pairs (system.cpp:2890-2979): segment rows, then state rows; a
        // state-state pair reads the row state's own side fraction
        for (int j = 0; j < nsp; j++) {
            if (!a.sp_on[j] || a.seg_frozen[j]) continue;
            double pj = phi[(size_t)j * M + s];
            for (int k = 0; k < nsp; k++) {
                if (!a.sp_on[k]) continue;
                double chi = a.chi[j * nsp + k];
                if (!(a.seg_frozen[k] && j < ns)) chi = chi / 2;
                if (j >= ns && a.seg_frozen[k]) chi = a.chi[j * nsp + k];
                if (chi == 0) continue;
                const int ks = (j >= ns && k >= ns) ? j : k;
                f += chi * (pj * phi_side[(size_t)ks * M + s]);
            }
        }
        for (int m = 0; m < a.n_mol; m++) f += a.cF2[m] * mol_phitot[(size_t)m * M + s];
        double km = ksam[s];
        F[s] = f * km;
        if (a.charged) F[s] += a.q[s] * a.psi[s] * 0.5;  // system.cpp:3020-3028
        for (int m = 0; m < a.n_mol; m++) gp += (mol_phitot[(size_t)m * M + s] + (-sc[5 * m + 4])) * a.invN[m];
        gp += alpha[s];
        for (int j = 0; j < nsp; j++) {
            if (!a.sp_on[j] || a.seg_frozen[j]) continue;
            double pj = phi[(size_t)j * M + s], pbA = seg_phibulk[j];
            for (int k = 0; k < nsp; k++) {
                if (!a.sp_on[k] || a.seg_frozen[k]) continue;
                double chi = a.chi[j * nsp + k] / 2;
                if (chi == 0) continue;
                gp += chi * (pj * phi_side[(size_t)k * M + s] + (-pbA * seg_phibulk[k]));
            }
        }
        if (a.charged) {  // system.cpp:3225-3238
            double t = a.EE[s] * a.eps[s] * -2.0;
            t = (t + a.q[s] * a.psi[s]) * (-1.0 / 2.0);
            double qs = a.q[s];
            GP[s] = ((-gp) + t) * km + (qs - qs * km) * a.psi[s] * 0.5;
        } else {
            GP[s] = (-gp) * km;
        }
    }
}

// ------------------------------------------------------------- host side --

static int grid_for(int n, int threads = 256) {
    int b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > 4 * 152 * 8) b = 4 * 152 * 8;
    return b;
}

int Ctx::launch_prop(const double* in, const double* G1, double* out) {
    int n = interior;
    launch_pdl(k_prop, grid_for(n), 256, stream, lat, in, G1, out);
    launches++;
    return NM_OK;
}

int Ctx::wsum(const double* X, double* out_dev) {
    const double* W = (plan->gradients < 3 && plan->geometry != NM_PLANAR) ? d_L : nullptr;
    k_wsum_partial<<<red_blocks, RED_THREADS, 0, stream>>>(lat, X, W, d_partial);
    k_final_sum<<<1, RED_THREADS, 0, stream>>>(d_partial, red_blocks, out_dev);
    launches += 2;
    return NM_OK;
}

int Ctx::molecule_pass(int m) {
    if (plan->mols[m].markov == 2) return ctx_m2_molecule_pass(*this, m);
    const nm_molecule& mol = plan->mols[m];
    MolDev& D = mols[m];
    size_t M = plan->M;
    int n = interior;
    int gb = grid_for(n), gbh = grid_for(n + nh);
    CK(cudaMemsetAsync(D.rho, 0, sizeof(double) * M * mol.n_molmon, stream));
    // forward
    for (int b = 0; b < mol.n_blocks; b++) {
        const nm_block& B = mol.blocks[b];
        const double* G1 = d_G1 + (size_t)B.seg * M;
        double* out = D.Gf + (size_t)B.s0 * M;
        if (B.n_child == 0) {
            launch_pdl(k_copy_interior, gb, 256, stream, lat, G1, out);
            launches++;
        } else {
            bool simple = (B.n_child == 1 && mol.blocks[mol.child_index[B.child0]].mult == 1);
            if (!simple) {
                for (int c = 0; c < B.n_child; c++) {
                    int cb = mol.child_index[B.child0 + c];
                    const nm_block& C = mol.blocks[cb];
                    launch_prop(D.Gf + (size_t)(C.s0 + C.length - 1) * M, d_ksam, D.Pc + (size_t)cb * M);
                }
            }
            int c0 = mol.child_index[B.child0];
            const nm_block& C0 = mol.blocks[c0];
            launch_prop(D.Gf + (size_t)(C0.s0 + C0.length - 1) * M, G1, out);
            if (!simple) {
                if (C0.mult > 1) { launch_pdl(k_mul_pow, gb, 256, stream, lat, out, D.Pc + (size_t)c0 * M, C0.mult - 1); launches++; }
                for (int c = 1; c < B.n_child; c++) {
                    int cb = mol.child_index[B.child0 + c];
                    launch_pdl(k_mul_pow, gb, 256, stream, lat, out, D.Pc + (size_t)cb * M, mol.blocks[cb].mult);
                    launches++;
                }
            }
        }
        for (int k = 1; k < B.length; k++)
            launch_prop(D.Gf + (size_t)(B.s0 + k - 1) * M, G1, D.Gf + (size_t)(B.s0 + k) * M);
    }
    const nm_block& R = mol.blocks[mol.n_blocks - 1];
    wsum(D.Gf + (size_t)(R.s0 + R.length - 1) * M, d_sc + 5 * m);
    // backward (pre-order, explicit stack)
    std::vector<int> stack;
    stack.push_back(mol.n_blocks - 1);
    while (!stack.empty()) {
        int b = stack.back();
        stack.pop_back();
        const nm_block& B = mol.blocks[b];
        const double* G1 = d_G1 + (size_t)B.seg * M;
        double* rho = D.rho + (size_t)B.molmon * M;
        double* cur = d_gb;
        double* nxt = d_gb + M;
        int s = B.s0 + B.length - 1;
        if (B.parent < 0) {
            launch_pdl(k_back_init, gb, 256, stream, lat, G1, cur, D.Gf + (size_t)s * M, rho, B.degeneracy);
        } else {
            launch_pdl(k_prop_back, gbh, 256, stream, lat, D.Q + (size_t)b * M, G1, cur, D.Gf + (size_t)s * M, rho, B.degeneracy, nh);
        }
        launches++;
        for (s = s - 1; s >= B.s0; s--) {
            launch_pdl(k_prop_back, gbh, 256, stream, lat, cur, G1, nxt, D.Gf + (size_t)s * M, rho, B.degeneracy, nh);
            launches++;
            double* t = cur; cur = nxt; nxt = t;
        }
        if (B.n_child == 0) continue;
        for (int c = 0; c < B.n_child; c++) {
            int cb = mol.child_index[B.child0 + c];
            double* q = D.Q + (size_t)cb * M;
            launch_pdl(k_copy_interior, gb, 256, stream, lat, cur, q);
            launches++;
            bool simple = (B.n_child == 1 && mol.blocks[cb].mult == 1);
            if (!simple) {
                if (mol.blocks[cb].mult > 1) { launch_pdl(k_mul_pow, gb, 256, stream, lat, q, D.Pc + (size_t)cb * M, mol.blocks[cb].mult - 1); launches++; }
                for (int o = 0; o < B.n_child; o++) {
                    if (o == c) continue;
                    int ob = mol.child_index[B.child0 + o];
                    launch_pdl(k_mul_pow, gb, 256, stream, lat, q, D.Pc + (size_t)ob * M, mol.blocks[ob].mult);
                    launches++;
                }
            }
        }
        for (int c = B.n_child - 1; c >= 0; c--) stack.push_back(mol.child_index[B.child0 + c]);
    }
    return NM_OK;
}

// All launches of one residual evaluation, on `stream` (captured into a graph
// by residual() on the 3-D path).
int Ctx::launch_g1(const double* x, bool with32) {
    k_g1<<<grid_for(plan->M), 256, 0, stream>>>(lat, plan->n_seg, x, d_seg_it, d_gmask, d_G1,
                                                with32 ? d_G1f : nullptr, chg, d_EE, d_psi, st, d_ust, d_ast);
    launches++;
    return NM_OK;
}

int Ctx::residual_launches(const double* x, double* g) {
    int M = plan->M;
    if (charged) elec_field(x);
    launch_g1(x, phase32);
    for (int m = 0; m < plan->n_mol; m++) {
        int rc;
        if (use3d) rc = ctx3d_molecule_pass(*this, m, phase32);
        else if (phase32 && use2d32) rc = ctx2d32_molecule_pass(*this, m);
        else if (use2d && sweep2d && plan->mols[m].n_store > 1) rc = ctx2d_molecule_pass(*this, m);
        else rc = molecule_pass(m);
        if (rc) return rc;
    }
    k_norms<<<1, 32, 0, stream>>>(norm_args, d_sc, d_seg_phibulk, d_status);
    k_phi<<<grid_for(M), 256, 0, stream>>>(lat, phi_args, d_sc, d_G1, d_phi_frozen, d_seg_frozen, d_phi, d_phitot,
                                           d_mol_phitot, charged ? 1 : 0);
    k_residual<<<grid_for(M), 256, 0, stream>>>(lat, res_args, x, d_phi, d_phitot, d_seg_phibulk, d_ksam, g, d_alpha, d_phi_side);
    launches += 3;
    if (charged) elec_residual(x, g);
    return NM_OK;
}

// One residual evaluation.  It issues about two launches per chain segment
// with nothing returning to the host, so its launches are captured into a
// CUDA graph once per (x, g, precision) and replayed after that.
int Ctx::residual(const double* x, double* g) {
    if (!graph || graph_x != x || graph_g != g || graph_32 != phase32) {
        if (graph) { cudaGraphExecDestroy(graph); graph = nullptr; }
        long long l0 = launches;
        CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        int rc = residual_launches(x, g);
        cudaGraph_t gr = nullptr;
        cudaError_t e = cudaStreamEndCapture(stream, &gr);
        if (rc) { if (gr) cudaGraphDestroy(gr); return rc; }
        CK(e);
        e = cudaGraphInstantiate(&graph, gr, 0);
        cudaGraphDestroy(gr);
        CK(e);
        graph_x = x; graph_g = g; graph_32 = phase32;
        graph_launches = launches - l0;
        launches = l0;
    }
    CK(cudaGraphLaunch(graph, stream));
    launches += graph_launches;
    have_state = true;
    return NM_OK;
}

// Storage of every k-th forward propagator (k >= 2; 0: every one) on the 3-D
// path: the slot table of each molecule (block starts, every k-th segment
// and each block's last) within the vectors allocated for it.
int Ctx::set_ck_stride(int k) {
    if (k != 0 && (k < 2 || !use3d)) { set_error("checkpoint stride: 0, or >= 2 on the 3-D path"); return NM_ERR_ARG; }
    std::vector<std::vector<int>> slots(plan->n_mol);
    std::vector<int> n_slots(plan->n_mol, 0);
    for (int m = 0; m < plan->n_mol && !k; m++)
        if (gf_vectors.size() == (size_t)plan->n_mol && gf_vectors[m] < (size_t)plan->mols[m].n_store) {
            set_error("every propagator stored needs the storage the context was not created with");
            return NM_ERR_ARG;
        }
    for (int m = 0; m < plan->n_mol && k; m++) {
        const nm_molecule& mol = plan->mols[m];
        slots[m].assign(mol.n_store, -1);
        for (int b = 0; b < mol.n_blocks; b++) {
            const nm_block& B = mol.blocks[b];
            for (int j = 0; j < B.length; j++)
                if (j % k == 0 || j == B.length - 1) slots[m][B.s0 + j] = n_slots[m]++;
        }
        if ((size_t)n_slots[m] + (k - 1) + 2 > gf_vectors[m]) {
            set_error("checkpoint stride does not fit the propagator storage of this context");
            return NM_ERR_ARG;
        }
    }
    for (int m = 0; m < plan->n_mol; m++) {
        mols[m].slot = slots[m];
        mols[m].n_slots = n_slots[m];
    }
    ck_stride = k;
    return NM_OK;
}

int Ctx::check_status() {
    int st = 0;
    CK(cudaMemcpyAsync(&st, d_status, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    if (st) {
        CK(cudaMemsetAsync(d_status, 0, sizeof(int), stream));
        set_error("device status " + std::to_string(st));
    }
    return st;
}

int Ctx::solve(double* x, nm_solve_result* res, int max_iter) {
    if (device_loop) return ctx_loop_solve(*this, x, res, max_iter);
    int nvar = plan->iv, m = plan->diis_m;
    double dmax = plan->deltamax, tol = tol_override > 0 ? tol_override : plan->tolerance;
    int nb = red_blocks;
    int it = 0, k_diis = 0;
    double resid = 0;
    phase32 = fp32;
    double best = 1e300;
    int since_best = 0;
    std::vector<double> Ah((size_t)m * m, 0.0), ci(m), gpart((size_t)m * nb);
    // One residual evaluation.  In the FP32 phase its norm and status are
    // checked before x moves: a failure of the reduced precision (G(N) <= 0,
    // a non-finite residual) hands over to FP64 at the same x.
    auto eval = [&]() -> int {
        int r = residual(x, d_g);
        if (r || !phase32) return r;
        k_diis_step<<<nb, RED_THREADS, 0, stream>>>(nvar, 0.0, x, d_g, nullptr, nullptr, d_partial, plan->max_norm, 0);
        k_final_norm<<<1, RED_THREADS, 0, stream>>>(d_partial, nb, d_resid, plan->max_norm);
        launches += 2;
        double r32 = 0;
        CK(cudaMemcpyAsync(&r32, d_resid, sizeof(double), cudaMemcpyDeviceToHost, stream));
        int st = check_status();
        if (st || !std::isfinite(r32)) {
            phase32 = false;
            k_diis = 0;
            r = residual(x, d_g);
        }
        return r;
    };
    // initial residual and simple mixing step into slot 0
    int rc = eval();
    if (rc) return rc;
    k_diis_step<<<nb, RED_THREADS, 0, stream>>>(nvar, dmax, x, d_g, d_xR, d_xx0, d_partial, plan->max_norm);
    k_final_norm<<<1, RED_THREADS, 0, stream>>>(d_partial, nb, d_resid, plan->max_norm);
    launches += 2;
    CK(cudaMemcpyAsync(&resid, d_resid, sizeof(double), cudaMemcpyDeviceToHost, stream));
    rc = check_status();
    if (rc) { res->iterations = 0; res->residual = resid; res->status = rc; return rc; }
    while (!(resid <= tol) && it < max_iter) {  // a NaN residual never counts as converged
        it++;
        rc = eval();
        if (rc) return rc;
        int k = it % m;
        k_diis++;
        k_diis_step<<<nb, RED_THREADS, 0, stream>>>(nvar, dmax, x, d_g, d_xR + (size_t)k * nvar,
                                                    d_xx0 + (size_t)k * nvar, d_partial, plan->max_norm);
        k_final_norm<<<1, RED_THREADS, 0, stream>>>(d_partial, nb, d_resid, plan->max_norm);
        int kd = k_diis > m ? m : k_diis;
        dim3 gg(nb, kd);
        k_gram<<<gg, RED_THREADS, 0, stream>>>(nvar, d_xx0, k, kd, m, d_gram_partial);
        launches += 3;
        // one synchronisation per iteration: ‖g‖, the status and the Gram row
        // partials come back; the m×m solve runs on the host (SFNewton::DIIS,
        // sfnewton.cpp:837-880) and the coefficients go back for the mix
        CK(cudaMemcpyAsync(&resid, d_resid, sizeof(double), cudaMemcpyDeviceToHost, stream));
        CK(cudaMemcpyAsync(gpart.data(), d_gram_partial, sizeof(double) * kd * nb, cudaMemcpyDeviceToHost, stream));
        rc = check_status();
        if (!rc) rc = diis_coefficients(gpart.data(), nb, k_diis, m, Ah.data(), ci.data());
        if (!rc) {
            CK(cudaMemcpyAsync(d_Ci, ci.data(), sizeof(double) * kd, cudaMemcpyHostToDevice, stream));
            k_diis_mix<<<grid_for(nvar), 256, 0, stream>>>(nvar, x, d_xR, d_Ci, k, k_diis, m);
            launches++;
        }
        if (phase32) {
            // FP32 propagators until a stall near their accuracy floor (or an
            // FP32 failure); then FP64 residuals, DIIS history restarted, so
            // the stopping test is made on an FP64 residual
            if (resid < 0.9 * best) { best = resid; since_best = 0; } else since_best++;
            bool fail = rc != 0 || !std::isfinite(resid);
            if (fail || resid <= tol || resid < sw_floor || (since_best > 10 && resid < 10.0 * sw_floor) ||
                (since_best > 25 && resid < 1e-2 * std::sqrt((double)nvar))) {
                phase32 = false;
                rc = 0;
                k_diis = 0;
                resid = 1e300;  // re-evaluated in FP64 by the next iteration
                continue;
            }
        }
        if (!rc && !std::isfinite(resid)) { set_error("non-finite residual"); rc = NM_ERR_NAN_DIIS; }
        if (rc) break;
    }
    phase32 = fp32;
    res->iterations = it;
    res->residual = resid;
    res->status = rc ? rc : (resid > tol ? NM_ERR_NOT_CONVERGED : NM_OK);
    return rc;
}

int Ctx::free_energy(double* F, double* Omega, double* mu) {
    if (!have_state) { set_error("no residual evaluated yet"); return NM_ERR_ARG; }
    int M = plan->M, ns = plan->n_seg;
    std::vector<double> sc(5 * plan->n_mol), spb(nsp);
    CK(cudaMemcpyAsync(sc.data(), d_sc, sizeof(double) * sc.size(), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(spb.data(), d_seg_phibulk, sizeof(double) * nsp, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    FeArgs a;
    std::memset(&a, 0, sizeof(a));
    a.ns = ns; a.nsp = nsp; a.n_mol = plan->n_mol;
    a.charged = charged;
    a.q = d_q; a.psi = d_psi; a.EE = d_EE; a.eps = d_eps;
    a.ust = d_ust;
    for (int k = 0; k < nsp; k++) a.sp_on[k] = res_args.sp_on[k];
    for (int i = 0; i < ns; i++) a.seg_frozen[i] = plan->seg_freedom[i] == NM_SEG_FROZEN;
    for (int m = 0; m < plan->n_mol; m++)
        for (int q = 0; q < plan->mols[m].n_molmon; q++) a.seg_in_mol[plan->mols[m].molmon_seg[q]] = 1;
    for (int j = 0; j < nst; j++) a.st_seg[j] = st.seg[j];
    const std::vector<double>& chs = nst ? chi_sp : chi;  // χ between species
    for (int i = 0; i < nsp * nsp; i++) a.chi[i] = chs[i];
    for (int m = 0; m < plan->n_mol; m++) {
        const nm_molecule& mol = plan->mols[m];
        double N = mol.chainlength;
        a.cF[m] = std::log(N * sc[5 * m + 2] / sc[5 * m + 0]) / N;
        double constant = 0;
        for (int j = 0; j < mol.n_molmon; j++)
            for (int k = 0; k < mol.n_molmon; k++)
                constant -= mol.molmon_fraction[j] * mol.molmon_fraction[k] *
                            (chi[mol.molmon_seg[j] * ns + mol.molmon_seg[k]] / 2);
        a.cF2[m] = constant;
        a.invN[m] = 1.0 / N;
    }
    k_fe_density<<<grid_for(M), 256, 0, stream>>>(lat, a, d_sc, d_phi, d_phi_side, d_G1, d_mol_phitot,
                                                  d_alpha, d_seg_phibulk, d_ksam, d_tmpF, d_tmpGP);
    launches++;
    wsum(d_tmpF, d_resid + 1);
    wsum(d_tmpGP, d_resid + 2);
    double out[2];
    CK(cudaMemcpyAsync(out, d_resid + 1, 2 * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    if (F) *F = out[0];
    if (Omega) *Omega = out[1];
    if (mu) {
        for (int i = 0; i < plan->n_mol; i++) {
            const nm_molecule& mol = plan->mols[i];
            double NA = mol.chainlength;
            double Mu = std::log(NA * sc[5 * i + 2] / sc[5 * i + 0]) + 1;
            double constant = 0;
            for (int k = 0; k < plan->n_mol; k++) constant += sc[5 * k + 4] / plan->mols[k].chainlength;
            Mu = Mu - NA * constant;
            // pairs of species (system.cpp:3319-3400); a state's bulk share
            // of the molecule is fraction(seg)·α_bulk, and the state-state
            // term takes the row state's for both factors
            auto frac = [&](int seg) {
                double f = 0;
                for (int q = 0; q < mol.n_molmon; q++) if (mol.molmon_seg[q] == seg) f = mol.molmon_fraction[q];
                return f;
            };
            auto share = [&](int k) { return k < ns ? frac(k) : frac(st.seg[k - ns]) * st.ab[k - ns]; };
            for (int j = 0; j < nsp; j++) {
                if (!res_args.sp_on[j]) continue;
                const double FA = share(j);
                for (int k = 0; k < nsp; k++) {
                    if (!res_args.sp_on[k]) continue;
                    const double FB = (j >= ns && k >= ns) ? FA : share(k);
                    Mu = Mu - NA * (chs[j * nsp + k] / 2) * (spb[j] - FA) * (spb[k] - FB);
                }
            }
            mu[i] = Mu;
        }
    }
    return NM_OK;
}

// Device memory of contexts and batches is stream-ordered (cudaMallocAsync /
// cudaFreeAsync on the object's own stream): creating and destroying them
// never synchronises the device, so solves on other streams keep running
// (the request server overlaps many).  Freed memory stays in the device's
// default pool for the next object instead of going back to the driver.
void nm_pool_setup(int dev) {
    static bool done[64] = {};
    if (dev < 0 || dev >= 64 || done[dev]) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        unsigned long long keep = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    done[dev] = true;
}

template <typename T>
static int dalloc(T** p, size_t n, cudaStream_t st) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMallocAsync((void**)p, sizeof(T) * n, st);
    if (e != cudaSuccess) { set_error(std::string("cudaMallocAsync: ") + cudaGetErrorString(e)); return NM_ERR_NOMEM; }
    e = cudaMemsetAsync(*p, 0, sizeof(T) * n, st);
    if (e != cudaSuccess) { set_error(std::string("cudaMemsetAsync: ") + cudaGetErrorString(e)); return NM_ERR_CUDA; }
    return NM_OK;
}

#define TRY(x) do { int r_ = (x); if (r_) return r_; } while (0)

int Ctx::init(const nm_plan* p, const nm_ctx_options* opt) {
    plan = p;
    if (p->n_seg > NM_MAX_SEG || p->n_mol > NM_MAX_MOL || p->diis_m > NM_MAX_DIIS) {
        set_error("problem exceeds the device path's compiled limits (segments, molecules, DIIS m)");
        return NM_ERR_INPUT;
    }
    int dev = opt ? opt->device : 0;
    CK(cudaSetDevice(dev));
    nm_pool_setup(dev);
    if (opt && opt->stream) { stream = (cudaStream_t)opt->stream; own_stream = false; }
    else { CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking)); own_stream = true; }
    int M = p->M, ns = p->n_seg;
    lat = make_lat(p);
    bool want2d32 = false;
    {
        std::string why;
        use3d = ctx3d_eligible(p, &why);
        fp32 = opt && opt->precision == NM_FP32;
        if (fp32 && !use3d) {
            std::string why2;
            if (p->gradients == 3 || !ctx2d32_eligible(p, &why2)) {
                set_error("FP32 propagators in a device context: " + (p->gradients == 2 ? why2 : why) +
                          " (1-gradient problems take the batched solver, nm_batch_*)");
                return NM_ERR_INPUT;
            }
            want2d32 = true;
        }
        if (use3d) l3 = make_l3(p);
        phase32 = fp32;  // residual calls outside a solve use the context's precision
        // FP32 accuracy floor of ‖g‖₂: ~1e-7 per chain segment per entry
        double n = 1;
        for (int m = 0; m < p->n_mol; m++) n = std::max(n, p->mols[m].chainlength);
        sw_floor = (1e-7 * n + 1e-6) * std::sqrt((double)p->iv);
    }
    interior = p->gradients == 1 ? p->MX : (p->gradients == 2 ? p->MX * p->MY : p->MX * p->MY * p->MZ);
    red_blocks = 2 * 152;
    // constants
    TRY(dalloc(&d_L, M, stream));
    CK(cudaMemcpyAsync(d_L, p->L, sizeof(double) * M, cudaMemcpyHostToDevice, stream));
    if (p->lambda_1) {
        TRY(dalloc(&d_lm1, M, stream)); TRY(dalloc(&d_l0, M, stream)); TRY(dalloc(&d_l1, M, stream));
        CK(cudaMemcpyAsync(d_lm1, p->lambda_1, sizeof(double) * M, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(d_l0, p->lambda0, sizeof(double) * M, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(d_l1, p->lambda1, sizeof(double) * M, cudaMemcpyHostToDevice, stream));
        lat.lm1 = d_lm1; lat.l0 = d_l0; lat.l1 = d_l1;
    }
    std::vector<double> ks(M);
    for (int s = 0; s < M; s++) ks[s] = p->ksam[s];
    TRY(dalloc(&d_ksam, M, stream));
    CK(cudaMemcpyAsync(d_ksam, ks.data(), sizeof(double) * M, cudaMemcpyHostToDevice, stream));
    TRY(dalloc(&d_gmask, (size_t)ns * M, stream));
    CK(cudaMemcpyAsync(d_gmask, p->seg_gmask, sizeof(double) * ns * M, cudaMemcpyHostToDevice, stream));
    TRY(dalloc(&d_phi_frozen, (size_t)ns * M, stream));
    CK(cudaMemcpyAsync(d_phi_frozen, p->seg_phi_frozen, sizeof(double) * ns * M, cudaMemcpyHostToDevice, stream));
    TRY(dalloc(&d_seg_it, ns, stream));
    CK(cudaMemcpyAsync(d_seg_it, p->seg_it, sizeof(int) * ns, cudaMemcpyHostToDevice, stream));
    std::vector<int> sf(ns);
    for (int i = 0; i < ns; i++) sf[i] = p->seg_freedom[i] == NM_SEG_FROZEN;
    TRY(dalloc(&d_seg_frozen, ns, stream));
    CK(cudaMemcpyAsync(d_seg_frozen, sf.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, stream));
    // internal states: species rows after the segments'
    nst = p->n_state;
    nsp = ns + nst;
    if (nst > 0) {
        if (nsp > NM_MAX_SEG) { set_error("more than 16 interaction species"); return NM_ERR_INPUT; }
        st.n = nst;
        for (int j = 0; j < nst; j++) { st.seg[j] = p->state_seg[j]; st.it[j] = p->state_it[j]; st.ab[j] = p->state_alphabulk[j]; }
        TRY(dalloc(&d_ust, (size_t)nst * M, stream));
        TRY(dalloc(&d_ast, (size_t)nst * M, stream));
        chi_sp.assign(p->chi_sp, p->chi_sp + (size_t)nsp * nsp);
        st_fixed = reinterpret_cast<const PlanHolder*>(p)->state_ab_in;
        st_pK = plan_reaction_pK(p);
    }
    // state
    TRY(dalloc(&d_G1, (size_t)ns * M, stream));
    TRY(dalloc(&d_phi, (size_t)nsp * M, stream));
    TRY(dalloc(&d_phi_side, (size_t)nsp * M, stream));
    TRY(dalloc(&d_phitot, M, stream));
    TRY(dalloc(&d_alpha, M, stream));
    TRY(dalloc(&d_mol_phitot, (size_t)p->n_mol * M, stream));
    TRY(dalloc(&d_gb, 2 * (size_t)M, stream));
    TRY(dalloc(&d_tmpF, M, stream));
    TRY(dalloc(&d_tmpGP, M, stream));
    TRY(dalloc(&d_sc, 5 * (size_t)p->n_mol, stream));
    TRY(dalloc(&d_seg_phibulk, nsp, stream));
    TRY(dalloc(&d_status, 1, stream));
    TRY(dalloc(&d_partial, (size_t)red_blocks, stream));
    TRY(dalloc(&d_resid, 4, stream));
    if (p->charged) TRY(elec_init());
    if (ctx2d_eligible(p)) TRY(ctx2d_init(*this));
    mols.resize(p->n_mol);
    int max_store = 1;
    for (int m = 0; m < p->n_mol; m++) max_store = std::max(max_store, p->mols[m].n_store);
    if (use3d) {
        TRY(dalloc(&d_maxbits, 2 * 32 * (size_t)max_store, stream));  // 32 slots per stored vector
        TRY(dalloc(&d_E, 2 * (size_t)max_store, stream));
    }
    // checkpointed propagator storage (3-D path): the caller's stride, else
    // for save_memory inputs the reference's slot count per block,
    // n = round(√(2·N_block)) (molecule.cpp:174-186), as a stride
    std::vector<size_t> n_vec(p->n_mol);
    if (use3d) {
        ck_stride = opt && opt->checkpoint_stride > 1 ? opt->checkpoint_stride : 0;
        if (!ck_stride && p->save_memory)
            for (int m = 0; m < p->n_mol; m++)
                for (int b = 0; b < p->mols[m].n_blocks; b++) {
                    const int L = p->mols[m].blocks[b].length;
                    int n = std::min(L, (int)(std::sqrt(2.0 * L) + 0.5));
                    if (n > 0) ck_stride = std::max(ck_stride, (L + n - 1) / n);
                }
        if (ck_stride < 2) ck_stride = 0;
    }
    if (ck_stride) {
        gf_vectors.assign(p->n_mol, ~(size_t)0);
        int k = ck_stride;
        ck_stride = 0;
        TRY(set_ck_stride(k));  // the slot tables of the stride
    }
    for (int m = 0; m < p->n_mol; m++)
        n_vec[m] = ck_stride ? (size_t)mols[m].n_slots + (ck_stride - 1) + 2 : (size_t)p->mols[m].n_store;
    gf_vectors = n_vec;
    if (fp32 && use3d) {
        TRY(dalloc(&d_G1f, (size_t)ns * M, stream));
        TRY(dalloc(&d_gb32, 2 * (size_t)M, stream));
        for (int m = 0; m < p->n_mol; m++) {
            const nm_molecule& mol = p->mols[m];
            TRY(dalloc(&mols[m].Gf32, n_vec[m] * M, stream));
            TRY(dalloc(&mols[m].rho32, 2 * (size_t)mol.n_molmon * M, stream));
        }
        TRY(ctx3dc_init(*this));  // small boxes: sweeps in one thread-block cluster
    }
    for (int m = 0; m < p->n_mol; m++) {
        const nm_molecule& mol = p->mols[m];
        TRY(dalloc(&mols[m].Gf, n_vec[m] * M * (mol.markov == 2 ? 3 : 1), stream));  // Markov 2: 3 directions
        TRY(dalloc(&mols[m].rho, (size_t)mol.n_molmon * M, stream));
        TRY(dalloc(&mols[m].Pc, (size_t)mol.n_blocks * M, stream));
        TRY(dalloc(&mols[m].Q, (size_t)mol.n_blocks * M, stream));
    }
    // DIIS
    int mm = p->diis_m;
    TRY(dalloc(&d_xR, (size_t)mm * p->iv, stream));
    TRY(dalloc(&d_xx0, (size_t)mm * p->iv, stream));
    TRY(dalloc(&d_g, (size_t)p->iv, stream));
    TRY(dalloc(&d_x, (size_t)p->iv, stream));
    TRY(dalloc(&d_Ci, (size_t)mm, stream));
    TRY(dalloc(&d_gram_partial, (size_t)mm * red_blocks, stream));
    if (want2d32) TRY(ctx2d32_init(*this));  // after the molecules' state exists
    TRY(ctx_m2_init(*this));
    // kernel argument blocks
    std::memset(&norm_args, 0, sizeof(norm_args));
    std::memset(&phi_args, 0, sizeof(phi_args));
    std::memset(&res_args, 0, sizeof(res_args));
    norm_args.n_mol = p->n_mol; norm_args.solvent = p->solvent; norm_args.ns = ns;
    norm_args.neutralizer = p->charged ? p->neutralizer : -1;
    phi_args.ns = ns; phi_args.n_mol = p->n_mol;
    int k = 0;
    for (int m = 0; m < p->n_mol; m++) {
        const nm_molecule& mol = p->mols[m];
        MolScal& S = norm_args.mol[m];
        S.freedom = mol.freedom; S.pinned = mol.pinned; S.n_in = mol.n; S.theta_in = mol.theta;
        S.phibulk_in = mol.phibulk; S.N = mol.chainlength; S.charge = mol.charge;
        for (int j = 0; j < mol.n_molmon; j++) {
            if (k >= NM_MAX_MM) { set_error("too many (molecule, segment) pairs"); return NM_ERR_INPUT; }
            norm_args.mm_mol[k] = m; norm_args.mm_seg[k] = mol.molmon_seg[j]; norm_args.mm_frac[k] = mol.molmon_fraction[j];
            phi_args.mm_mol[k] = m; phi_args.mm_seg[k] = mol.molmon_seg[j];
            phi_args.mm_rho[k] = mols[m].rho + (size_t)j * M;
            k++;
        }
    }
    norm_args.n_mm = k; phi_args.n_mm = k;
    norm_args.st = st; phi_args.st = st; phi_args.ast = d_ast;
    res_args.ns = nsp; res_args.nit = p->n_it;
    for (int i = 0; i < p->n_it; i++) res_args.it_seg[i] = nst ? p->it_sp[i] : p->it_seg[i];
    for (int k2 = 0; k2 < nsp; k2++) res_args.sp_on[k2] = k2 >= ns || !nst || p->seg_nstate[k2] == 0;
    chi.assign(p->chi, p->chi + (size_t)ns * ns);
    const std::vector<double>& chs = nst ? chi_sp : chi;
    for (int i = 0; i < nsp * nsp; i++) res_args.chi[i] = chs[i];
    CK(cudaStreamSynchronize(stream));
    return NM_OK;
}

Ctx::~Ctx() {
    double* ptrs[] = {d_ust, d_ast, d_L, d_lm1, d_l0, d_l1, d_ksam, d_gmask, d_phi_frozen, d_G1, d_phi, d_phi_side,
                      d_phitot, d_alpha, d_mol_phitot, d_gb, d_tmpF, d_tmpGP, d_sc, d_seg_phibulk,
                      d_partial, d_resid, d_xR, d_xx0, d_g, d_x, d_Ci, d_gram_partial,
                      d_EE, d_psi, d_q, d_eps, d_X};
    for (double* q : ptrs) if (q) cudaFreeAsync(q, stream);
    if (d_seg_it) cudaFreeAsync(d_seg_it, stream);
    if (d_seg_frozen) cudaFreeAsync(d_seg_frozen, stream);
    if (d_status) cudaFreeAsync(d_status, stream);
    for (auto& D : mols) {
        cudaFreeAsync(D.Gf, stream); cudaFreeAsync(D.rho, stream); cudaFreeAsync(D.Pc, stream); cudaFreeAsync(D.Q, stream);
        if (D.Gf32) cudaFreeAsync(D.Gf32, stream);
        if (D.rho32) cudaFreeAsync(D.rho32, stream);
    }
    if (d_G1f) cudaFreeAsync(d_G1f, stream);
    if (d_gb32) cudaFreeAsync(d_gb32, stream);
    if (d_maxbits) cudaFreeAsync(d_maxbits, stream);
    if (d_E) cudaFreeAsync(d_E, stream);
    ctx3dc_free(*this);
    ctx_m2_free(*this);
    for (auto& T : sw_tabs) {
        if (T.seg) cudaFreeAsync(T.seg, stream);
        if (T.mm) cudaFreeAsync(T.mm, stream);
        if (T.deg) cudaFreeAsync(T.deg, stream);
    }
    if (d_flags) cudaFreeAsync(d_flags, stream);
    for (int* q : E2f) if (q) cudaFreeAsync(q, stream);
    if (d_E2b) cudaFreeAsync(d_E2b, stream);
    if (d_rowpart) cudaFreeAsync(d_rowpart, stream);
    if (graph) cudaGraphExecDestroy(graph);
    ctx_loop_drop(*this);
    if (d_loop) cudaFreeAsync(d_loop, stream);
    if (own_stream && stream) cudaStreamDestroy(stream);
}

Lat make_lat(const nm_plan* p) {
    Lat L;
    std::memset(&L, 0, sizeof(L));
    L.g = p->gradients; L.MX = p->MX; L.MY = p->MY; L.MZ = p->MZ;
    L.JX = p->JX; L.JY = p->JY; L.M = p->M;
    L.geom = p->geometry; L.lat = p->lattice_type; L.lam = p->lambda;
    int n[3] = {p->MX, p->MY, p->MZ};
    for (int d = 0; d < 3; d++) {
        int bl = p->bc[d], bh = p->bc[d + 3];
        L.b1[d] = bl == NM_BC_MIRROR ? 1 : bl == NM_BC_PERIODIC ? n[d] : 0;
        L.bm[d] = bh == NM_BC_MIRROR ? n[d] : bh == NM_BC_PERIODIC ? 1 : n[d] + 1;
    }
    return L;
}

}  // namespace nm

// ---------------------------------------------------------------- C ABI ---
using nm::Ctx;

extern "C" {

int nm_ctx_create(const nm_plan* plan, const nm_ctx_options* opt, nm_ctx** out) {
    if (!plan || !out) { nm::set_error("nm_ctx_create: null argument"); return NM_ERR_ARG; }
    *out = nullptr;
    Ctx* c = new Ctx();
    int rc = c->init(plan, opt);
    if (rc) { delete c; return rc; }
    *out = reinterpret_cast<nm_ctx*>(c);
    return NM_OK;
}

int nm_ctx_destroy(nm_ctx* ctx) {
    delete reinterpret_cast<Ctx*>(ctx);
    return NM_OK;
}

// Values of a live context for scans (the reference's Variate, variate.cpp,
// solve_scf.cpp:717-868): χ between two segment types ("mon : A : chi_W",
// set both ways) and a molecule's amount ("mol : pol : n | theta" for
// restricted, "mol : pol : phibulk" for free molecules).  All items are
// applied, then checked: χ must keep the iteration species (segments with
// equal χ rows, System::IsUnique) as they were, because x's layout follows
// them.  On any error nothing changes.  The captured residual is dropped;
// the next solve starts from the context's current field.
int nm_ctx_set_values(nm_ctx* ctx, const char* const* items, const double* values, int n) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c || (n > 0 && (!items || !values))) { nm::set_error("nm_ctx_set_values: bad argument"); return NM_ERR_ARG; }
    const nm_plan* p = c->plan;
    const int ns = p->n_seg;
    std::vector<double> chi = c->chi;
    nm::NormArgs na = c->norm_args;
    std::vector<double> st_fixed = c->st_fixed, st_pK = c->st_pK;
    bool states_changed = false;
    auto trim = [](std::string s) {
        size_t a = s.find_first_not_of(" \t"), b = s.find_last_not_of(" \t");
        return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
    };
    for (int i = 0; i < n; i++) {
        std::string it = items[i] ? items[i] : "";
        size_t p1 = it.find(':'), p2 = p1 == std::string::npos ? p1 : it.find(':', p1 + 1);
        if (p2 == std::string::npos) { nm::set_error("nm_ctx_set_values: not a 'key : name : property' item: " + it); return NM_ERR_ARG; }
        const std::string key = trim(it.substr(0, p1)), name = trim(it.substr(p1 + 1, p2 - p1 - 1)),
                          prop = trim(it.substr(p2 + 1));
        const double v = values[i];
        bool ok = false;
        if (key == "mon" && prop.rfind("chi_", 0) == 0 && c->nst > 0) {
            nm::set_error("nm_ctx_set_values: χ of a system with internal states is fixed at creation");
            return NM_ERR_ARG;
        }
        if (key == "mon" && prop.rfind("chi_", 0) == 0) {
            int a = -1, b = -1;
            for (int k = 0; k < ns; k++) {
                if (name == p->seg_name[k]) a = k;
                if (prop.substr(4) == p->seg_name[k]) b = k;
            }
            if (a >= 0 && b >= 0 && a != b) { chi[a * ns + b] = chi[b * ns + a] = v; ok = true; }
        } else if (key == "state" && prop == "alphabulk" && c->nst > 0) {
            // a fixed state's bulk fraction (State::PutValue, state.cpp:350-357)
            const nm::PlanHolder& H = *reinterpret_cast<const nm::PlanHolder*>(p);
            for (int j = 0; j < c->nst; j++)
                if (name == p->state_name[j] && H.state_fixed[j]) { st_fixed[j] = v; states_changed = ok = true; }
        } else if (key == "reaction" && prop == "pK" && c->nst > 0) {
            // a reaction's pK (Reaction::PutValue, reaction.cpp:443-452)
            const int r = nm::plan_reaction_index(p, name);
            if (r >= 0) { st_pK[r] = v; states_changed = ok = true; }
        } else if (key == "mol") {
            for (int m = 0; m < p->n_mol; m++) {
                if (!p->mol_name || name != p->mol_name[m]) continue;
                nm::MolScal& S = na.mol[m];
                if (S.freedom == NM_MOL_RESTRICTED && prop == "n") { S.n_in = v; S.theta_in = v * S.N; ok = true; }
                else if (S.freedom == NM_MOL_RESTRICTED && prop == "theta") { S.theta_in = v; S.n_in = v / S.N; ok = true; }
                else if (S.freedom == NM_MOL_FREE && prop == "phibulk") { S.phibulk_in = v; ok = true; }
            }
        }
        if (!ok) { nm::set_error("nm_ctx_set_values: not a value this context can change: " + it); return NM_ERR_ARG; }
    }
    // the iteration species must stay: rows of χ equal within a species, different across
    for (int a = 0; a < ns; a++)
        for (int b = a + 1; b < ns; b++) {
            if (p->seg_it[a] < 0 || p->seg_it[b] < 0) continue;
            bool same = true;
            for (int k = 0; k < ns; k++) same = same && chi[a * ns + k] == chi[b * ns + k];
            if (same != (p->seg_it[a] == p->seg_it[b])) {
                nm::set_error(std::string("nm_ctx_set_values: the new χ changes the iteration species (") +
                              p->seg_name[a] + ", " + p->seg_name[b] + ")");
                return NM_ERR_INPUT;
            }
        }
    nm::StArgs stn = c->st;
    if (states_changed) {
        // the bulk equilibrium again, its pK_eff from the bulk fractions of
        // the last residual as the reference's next solve reads them
        std::vector<double> spb((size_t)c->nsp), ab, charge;
        if (c->have_state) {
            cudaError_t e = cudaMemcpyAsync(spb.data(), c->d_seg_phibulk, sizeof(double) * spb.size(),
                                            cudaMemcpyDeviceToHost, c->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
            if (e != cudaSuccess) { nm::set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
        }
        std::string err;
        if (int rc = nm::plan_state_bulk(p, st_fixed, st_pK, c->have_state ? spb.data() : nullptr, ab, charge, err)) {
            nm::set_error("nm_ctx_set_values: " + err);
            return rc;
        }
        for (int j = 0; j < c->nst; j++) stn.ab[j] = ab[j];
        for (int m = 0; m < p->n_mol; m++) na.mol[m].charge = charge[m];
        na.st = stn;
    }
    c->chi = chi;
    if (!c->nst)  // with states the residual's χ is the species matrix, which no item changes
        for (int k = 0; k < ns * ns; k++) c->res_args.chi[k] = chi[k];
    c->norm_args = na;
    if (states_changed) {
        c->st = stn;
        c->phi_args.st = stn;
        c->st_fixed = st_fixed;
        c->st_pK = st_pK;
    }
    if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
    nm::ctx_loop_drop(*c);
    return NM_OK;
}

int nm_ctx_set_option(nm_ctx* ctx, int option, int value) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c) { nm::set_error("nm_ctx_set_option: null context"); return NM_ERR_ARG; }
    if (option == NM_OPT_SWEEP2D) {
        c->sweep2d = value != 0;
    } else if (option == NM_OPT_ROWS3D) {
        if (value != 2 && value != 4 && value != 8) { nm::set_error("nm_ctx_set_option: rows per block 2, 4 or 8"); return NM_ERR_ARG; }
        c->c3_rows = value;
    } else if (option == NM_OPT_CHECKPOINT) {
        if (int rc = c->set_ck_stride(value)) return rc;
    } else if (option == NM_OPT_TILE3D) {
        if (int rc = nm::ctx3d_set_tile(*c, value)) return rc;
    } else if (option == NM_OPT_CLUSTER3D) {
        if (value && !c->c3c_ctas) {
            nm::set_error("nm_ctx_set_option: no cluster sweep for this context (FP32 3-D linear chains on a box "
                          "whose two propagator buffers fit a cluster's shared memory)");
            return NM_ERR_ARG;
        }
        c->c3c_on = value != 0;
    } else if (option == NM_OPT_DEVICE_LOOP) {
        c->device_loop = value != 0;
    } else {
        nm::set_error("nm_ctx_set_option: unknown option");
        return NM_ERR_ARG;
    }
    if (c->graph) {  // the captured residual used the other kernels
        cudaGraphExecDestroy(c->graph);
        c->graph = nullptr;
    }
    nm::ctx_loop_drop(*c);
    return NM_OK;
}

int nm_residual_dev(nm_ctx* ctx, const double* x_dev, double* g_dev) {
    if (!ctx || !x_dev || !g_dev) { nm::set_error("nm_residual_dev: null argument"); return NM_ERR_ARG; }
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    int rc = c->residual(x_dev, g_dev);
    if (rc) return rc;
    return c->check_status();
}

int nm_solve_dev(nm_ctx* ctx, double* x_dev, nm_solve_result* res) {
    if (!ctx || !x_dev || !res) { nm::set_error("nm_solve_dev: null argument"); return NM_ERR_ARG; }
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    return c->solve(x_dev, res, c->plan->iterationlimit);
}

int nm_ctx_search(nm_ctx* ctx, double* x_dev, nm_search_result* out) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c || !x_dev || !out) { nm::set_error("nm_ctx_search: null argument"); return NM_ERR_ARG; }
    const nm_plan* p = c->plan;
    if (p->search_mol < 0) { nm::set_error("nm_ctx_search: the plan defines no search ('var' keys)"); return NM_ERR_ARG; }
    static const char* const what[] = {"theta", "n", "phibulk", "mu"};
    const std::string item = std::string("mol : ") + p->mol_name[p->search_mol] + " : " + what[p->search_what];
    const char* items[1] = {item.c_str()};
    const double tol = p->super_tolerance, dmax = p->super_deltamax;
    const int itlim = p->super_iterationlimit;
    nm_search_result r{};
    // inner solves to the search tolerance (solve_scf.cpp:839-846)
    struct TolGuard {
        Ctx* c; double old;
        ~TolGuard() { c->tol_override = old; }
    } guard{c, c->tol_override};
    c->tol_override = tol;
    nm_solve_result sr{};
    // the target's error (System::GetError, system.cpp:1405-1425;
    // Molecule::GetError, molecule.cpp:942-968)
    auto error_now = [&](double& g) -> int {
        const double t = p->target_value;
        std::vector<double> mu(p->n_mol);
        double F = 0, O = 0;
        if (p->target_kind <= 1 || p->target_what == 3) {
            int rc = c->free_energy(&F, &O, mu.data());
            if (rc) return rc;
        }
        if (p->target_kind == 0) { g = F - t; return NM_OK; }
        if (p->target_kind == 1) { g = -(O - t); return NM_OK; }
        double n = 0, th = 0, pb = 0;
        int rc = nm_get_molecule(ctx, p->target_mol, nullptr, &n, &th, &pb);
        if (rc) return rc;
        const double v = p->target_what == 0 ? th : p->target_what == 1 ? n : p->target_what == 2 ? pb : mu[p->target_mol];
        g = t != 0 ? v / t - 1.0 : v;
        if (p->target_what == 2) g = -g;
        return NM_OK;
    };
    // one evaluation: set the variable, solve from the current field, error
    auto R = [&](double v, double& g) -> int {
        int rc = nm_ctx_set_values(ctx, items, &v, 1);
        if (rc) return rc;
        rc = c->solve(x_dev, &sr, p->iterationlimit);
        r.solves++;
        if (rc && rc != NM_ERR_NOT_CONVERGED) return rc;
        return error_now(g);
    };
#define NM_TRY(e) do { int rc_ = (e); if (rc_) { r.status = rc_; *out = r; return rc_; } } while (0)
    // the variable's current value (the input's, or the last set_values);
    // the first evaluation solves there (namics.cpp:571-574 goes straight
    // to SuperIterate)
    const nm::MolScal& S0 = c->norm_args.mol[p->search_mol];
    double x = p->search_what == 0 ? S0.theta_in : p->search_what == 1 ? S0.n_in : S0.phibulk_in;
    // damped regula falsi on the scale of the variable relative to its value
    // at each (re)start (SFNewton::iterate_RF, sfnewton.cpp:1132-1185),
    // including its iteration count, which adds the inner steps of the
    // previous pass again at every restart
    double a = 0, b = 0, cc = 0, fa = 0, fb = 0, fc = 0, res = 100.0;
    int k = 0, it = 0;
    while (it < itlim && std::fabs(res) > tol) {
        const double xs = x;
        NM_TRY(R(x, fa));
        a = 1;
        x = (a + dmax) * xs;
        NM_TRY(R(x, fb));
        b = x / xs;
        cc = a - 0.5 * ((fa * (a - b)) / (fa - fb));
        x = cc * xs;
        NM_TRY(R(x, fc));
        res = fc;
        it += k;
        k = 0;
        while (k < itlim / 10 && std::fabs(res) > tol) {
            cc = a - 0.5 * ((fa * (a - b)) / (fa - fb));
            x = cc * xs;
            NM_TRY(R(x, fc));
            if (fc * fb < 0) {
                b = cc; x = b * xs; NM_TRY(R(x, fb)); res = fb;
            } else {
                a = cc; x = a * xs; NM_TRY(R(x, fa)); res = fa;
            }
            k++;
            it++;
        }
        if (!std::isfinite(res)) break;
    }
#undef NM_TRY
    r.value = x;
    r.error = res;
    r.iterations = it;
    r.status = std::fabs(res) <= tol ? NM_OK : NM_ERR_NOT_CONVERGED;
    *out = r;
    if (r.status) nm::set_error("nm_ctx_search: the target was not reached within super_iterationlimit");
    return r.status;
}

int nm_solve_host(nm_ctx* ctx, double* x_host, double* phi_host, nm_solve_result* res) {
    if (!ctx || !x_host || !res) { nm::set_error("nm_solve_host: null argument"); return NM_ERR_ARG; }
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    size_t iv = c->plan->iv;
    cudaError_t e = cudaMemcpyAsync(c->d_x, x_host, sizeof(double) * iv, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) { nm::set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    int rc = c->solve(c->d_x, res, c->plan->iterationlimit);
    e = cudaMemcpyAsync(x_host, c->d_x, sizeof(double) * iv, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && phi_host)
        e = cudaMemcpyAsync(phi_host, c->d_phi, sizeof(double) * c->plan->n_seg * c->plan->M,
                            cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) { nm::set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    return rc;
}

int nm_get_field(nm_ctx* ctx, int which, double* out_host) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c || !out_host || !c->have_state) { nm::set_error("nm_get_field: no state"); return NM_ERR_ARG; }
    if (which >= 6 && which <= 8 && !c->charged) { nm::set_error("nm_get_field: ψ, q and ε exist only for charged systems"); return NM_ERR_ARG; }
    size_t M = c->plan->M, ns = c->plan->n_seg;
    const double* src = nullptr;
    size_t n = 0;
    switch (which) {
        case 0: src = c->d_phi; n = ns * M; break;
        case 1: src = c->d_G1; n = ns * M; break;
        case 2: src = c->d_alpha; n = M; break;
        case 3: src = c->d_phitot; n = M; break;
        case 4: src = c->d_mol_phitot; n = c->plan->n_mol * M; break;
        case 5: src = c->d_phi_side; n = ns * M; break;
        case 6: src = c->d_psi; n = M; break;
        case 7: src = c->d_q; n = M; break;
        case 8: src = c->d_eps; n = M; break;
        case 9: case 10: case 11:
            if (!c->nst) { nm::set_error("nm_get_field: the plan has no internal states"); return NM_ERR_ARG; }
            src = which == 9 ? c->d_phi + ns * M : (which == 10 ? c->d_ast : c->d_ust);
            n = (size_t)c->nst * M;
            break;
        default: nm::set_error("nm_get_field: unknown field"); return NM_ERR_ARG;
    }
    cudaError_t e = cudaMemcpyAsync(out_host, src, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) { nm::set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    return NM_OK;
}

int nm_get_molecule(nm_ctx* ctx, int mol, double* GN, double* n, double* theta, double* phibulk) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c || !c->have_state || mol < 0 || mol >= c->plan->n_mol) { nm::set_error("nm_get_molecule: bad argument"); return NM_ERR_ARG; }
    double s[5];
    cudaError_t e = cudaMemcpyAsync(s, c->d_sc + 5 * mol, sizeof(s), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) { nm::set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    if (GN) *GN = s[0];
    if (n) *n = s[2];
    if (theta) *theta = s[3];
    if (phibulk) *phibulk = s[4];
    return NM_OK;
}

int nm_free_energy(nm_ctx* ctx, double* F, double* Omega, double* mu) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c) { nm::set_error("nm_free_energy: null context"); return NM_ERR_ARG; }
    return c->free_energy(F, Omega, mu);
}

int nm_propagate_dev(nm_ctx* ctx, double* G_in_dev, const double* G1_dev, double* G_out_dev) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c || !G_in_dev || !G_out_dev) { nm::set_error("nm_propagate_dev: null argument"); return NM_ERR_ARG; }
    c->launch_prop(G_in_dev, G1_dev, G_out_dev);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) { nm::set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    return NM_OK;
}

int nm_side_dev(nm_ctx* ctx, const double* X_dev, double* X_side_dev) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!c || !X_dev || !X_side_dev) { nm::set_error("nm_side_dev: null argument"); return NM_ERR_ARG; }
    c->launch_prop(X_dev, nullptr, X_side_dev);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) { nm::set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    return NM_OK;
}

long long nm_ctx_launch_count(nm_ctx* ctx) {
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    return c ? c->launches : 0;
}

}  // extern "C"
