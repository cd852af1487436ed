// Device context internals shared by ctx.cu and the C-ABI entry points.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "../../include/namics_gb300.h"
#include "device_common.cuh"
#include "plan_internal.h"

#define NM_MAX_SEG 16
#define NM_MAX_MOL 16
#define NM_MAX_MM 32
#define NM_MAX_DIIS 32

namespace nm {

// Solve A c = 1 (A: n×n row-major, n ≤ NM_MAX_DIIS) by Gaussian elimination
// with partial pivoting in FP64.  The reference solves the same system with an
// unregularised SVD pseudo-inverse (SFNewton::Ax, sfnewton.cpp:793-835); for a
// non-singular A both give the exact solution up to rounding.
__host__ __device__ inline void nm_small_solve(const double* Ain, double* c, int n) {
    double A[NM_MAX_DIIS * NM_MAX_DIIS];
    double b[NM_MAX_DIIS];
    for (int i = 0; i < n * n; i++) A[i] = Ain[i];
    for (int i = 0; i < n; i++) b[i] = 1.0;
    if (n == 1) { c[0] = 1.0; return; }  // Ax: N == 1 -> X[0] = 1
    for (int k = 0; k < n; k++) {
        int p = k;
        double best = A[k * n + k] < 0 ? -A[k * n + k] : A[k * n + k];
        for (int i = k + 1; i < n; i++) {
            double v = A[i * n + k] < 0 ? -A[i * n + k] : A[i * n + k];
            if (v > best) { best = v; p = i; }
        }
        if (p != k) {
            for (int j = 0; j < n; j++) { double t = A[k * n + j]; A[k * n + j] = A[p * n + j]; A[p * n + j] = t; }
            double t = b[k]; b[k] = b[p]; b[p] = t;
        }
        double piv = A[k * n + k];
        for (int i = k + 1; i < n; i++) {
            double f = A[i * n + k] / piv;
            for (int j = k; j < n; j++) A[i * n + j] -= f * A[k * n + j];
            b[i] -= f * b[k];
        }
    }
    for (int i = n - 1; i >= 0; i--) {
        double v = b[i];
        for (int j = i + 1; j < n; j++) v -= A[i * n + j] * c[j];
        c[i] = v / A[i * n + i];
    }
}

struct MolScal { int freedom, pinned; double n_in, theta_in, phibulk_in, N, charge; };
struct NormArgs {
    int n_mol, solvent, ns;
    MolScal mol[NM_MAX_MOL];
    int n_mm;
    int mm_mol[NM_MAX_MM], mm_seg[NM_MAX_MM];
    double mm_frac[NM_MAX_MM];
};
struct PhiArgs {
    int ns, n_mm, n_mol;
    int mm_mol[NM_MAX_MM], mm_seg[NM_MAX_MM];
    const double* mm_rho[NM_MAX_MM];
};
struct ResArgs {
    int ns, nit;
    int it_seg[NM_MAX_SEG];
    double chi[NM_MAX_SEG * NM_MAX_SEG];
};

struct MolDev {
    double* Gf = nullptr;   // forward propagators [n_store*M]
    double* rho = nullptr;  // Σ d·Gf·Gb per molecule segment type [n_molmon*M]
    double* Pc = nullptr;   // P(G_end)·KSAM of each child block [n_blocks*M]
    double* Q = nullptr;    // backward start of each child block [n_blocks*M]
};

nmdev::Lat make_lat(const nm_plan* p);

struct Ctx {
    const nm_plan* plan = nullptr;
    nmdev::Lat lat{};
    int interior = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int red_blocks = 0;
    bool have_state = false;
    long long launches = 0;
    double *d_L = nullptr, *d_lm1 = nullptr, *d_l0 = nullptr, *d_l1 = nullptr, *d_ksam = nullptr;
    double *d_gmask = nullptr, *d_phi_frozen = nullptr;
    int *d_seg_it = nullptr, *d_seg_frozen = nullptr, *d_status = nullptr;
    double *d_G1 = nullptr, *d_phi = nullptr, *d_phi_side = nullptr, *d_phitot = nullptr,
           *d_alpha = nullptr, *d_mol_phitot = nullptr, *d_gb = nullptr, *d_tmpF = nullptr,
           *d_tmpGP = nullptr, *d_sc = nullptr, *d_seg_phibulk = nullptr, *d_partial = nullptr,
           *d_resid = nullptr;
    double *d_xR = nullptr, *d_xx0 = nullptr, *d_g = nullptr, *d_x = nullptr, *d_Aij = nullptr,
           *d_Ci = nullptr, *d_gram_partial = nullptr;
    std::vector<MolDev> mols;
    NormArgs norm_args;
    PhiArgs phi_args;
    ResArgs res_args;

    int init(const nm_plan* p, const nm_ctx_options* opt);
    ~Ctx();
    int launch_prop(const double* in, const double* G1, double* out);
    int wsum(const double* X, double* out_dev);
    int molecule_pass(int m);
    int residual(const double* x, double* g);
    int check_status();
    int solve(double* x, nm_solve_result* res, int max_iter);
    int free_energy(double* F, double* Omega, double* mu);
};

}  // namespace nm
