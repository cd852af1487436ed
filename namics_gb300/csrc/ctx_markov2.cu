// Markov 2 (semiflexible) chains on 1-gradient simple-cubic lattices, FP64,
// in the generic device context.
//
// Every propagator of such a molecule holds FJC = 3 components, one per
// direction of the bond that arrives at a site: d = 0 down, 1 lateral (4 of
// the 6 simple-cubic directions), 2 up.  A step mixes the components with
// the bond-angle weights P[k] of the plan (angles k·π/2; P[2] = 0):
//   planar   LG1Planar::propagateF/B (LG1Planar.cpp:57-135),
//   curved   LGrad1::propagateF/B (LGrad1.cpp:285-429), the neighbour
//            weights l1 = λ1/λ, l_1 = λ_1/λ and their complements
//            (LGrad1.cpp:63-68), 0 on the halo layers.
// The reference calls set_bounds on the input of every step, in place: the
// halo of direction 0 takes direction 2's boundary value and the reverse (a
// reflected bond changes direction), the lateral direction its own
// (LGrad1.cpp:787-818).  Here the stored propagators keep the values a step
// wrote, and a step reads its input's halo layers through that same map,
// which gives every interior value the reference computes; the halo values a
// step writes are the reference's formula, so a 'surface' halo (which
// set_bounds leaves alone) carries what it carries there.
// The sweeps of a linear chain follow mol_linear.cpp:115-129 and
// molecule.cpp:2448-2615 (every propagator stored): Initiate copies G1 into
// every direction; G(N) = (Σ_0 + 4·Σ_1 + Σ_2)/6 of the last propagator's
// weighted sums (LGrad1.cpp:863-874); the composition adds
// Gf_0·Gb_0/6 + 4·Gf_1·Gb_1/6 + Gf_2·Gb_2/6 at every segment
// (LGrad1.cpp:876-905), here on the interior sites (a neutral system's
// residual reads no halo of φ).
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "ctx_internal.h"

namespace nm {

namespace {

constexpr int M2_FJC = 3;

struct M2Args {
    int M, MX, bx1, bxm;  // halo source layers (0 and MX+1: 'surface')
    double P0, P1;
    const double *l1, *l11, *l_1, *l_11;  // curved lattices only
};

// component values of the stored vector `in` at x, halos as set_bounds
// would leave them
__device__ __forceinline__ void m2_read(const M2Args& A, const double* __restrict__ in, int x, double& a0, double& a1,
                                        double& a2) {
    const double *i0 = in, *i1 = in + A.M, *i2 = in + 2 * A.M;
    if (x == 0) {
        a0 = i2[A.bx1];
        a2 = A.bx1 == 0 ? i2[0] : i0[A.bx1];
        a1 = i1[A.bx1];
    } else if (x == A.MX + 1) {
        a0 = i2[A.bxm];
        a2 = A.bxm == A.MX + 1 ? i2[A.MX + 1] : i0[A.bxm];
        a1 = i1[A.bxm];
    } else {
        a0 = i0[x];
        a1 = i1[x];
        a2 = i2[x];
    }
}

// One step over every site x of the padded array (halos included).  BWD:
// the backward step, fused with the composition ρ += Σ_d C_d·Gf_d·Gb_d on
// the interior sites.
template <bool BWD, bool CURV>
__global__ void k_m2_step(M2Args A, const double* __restrict__ in, const double* __restrict__ G1,
                          double* __restrict__ out, const double* __restrict__ gf, double* __restrict__ rho) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int M = A.M;
    if (x >= M) return;
    const double P0 = A.P0, P1 = A.P1;
    double c0, c1, c2, m0 = 0, m1 = 0, m2 = 0, p0 = 0, p1 = 0, p2 = 0;
    m2_read(A, in, x, c0, c1, c2);
    const bool lft = x >= 1, rgt = x <= M - 2;
    if (lft) m2_read(A, in, x - 1, m0, m1, m2);
    if (rgt) m2_read(A, in, x + 1, p0, p1, p2);
    double o0 = 0, o1 = 0, o2 = 0;
    if (!CURV) {
        if (!BWD) {  // LG1Planar::propagateF
            if (lft) { o0 += P0 * m0; o0 += 4 * P1 * m1; }
            o1 += P1 * c0; o1 += (2 * P1 + P0) * c1; o1 += P1 * c2;
            if (rgt) { o2 += 4 * P1 * p1; o2 += P0 * p2; }
        } else {     // LG1Planar::propagateB
            if (rgt) o0 += P0 * p0;
            o0 += 4 * P1 * c1;
            if (rgt) o1 += P1 * p0;
            o1 += (2 * P1 + P0) * c1;
            if (lft) o1 += P1 * m2;
            o2 += 4 * P1 * c1;
            if (lft) o2 += P0 * m2;
        }
    } else {
        if (!BWD) {  // LGrad1::propagateF
            if (lft) {
                double h = A.l_1[x] * m0;
                h += A.l_11[x] * c2;
                o0 += P0 * h;
                h = A.l_1[x] * m1;
                h += A.l_11[x] * c1;
                o0 += 4 * P1 * h;
            }
            o1 += P1 * c0; o1 += (2 * P1 + P0) * c1; o1 += P1 * c2;
            if (rgt) {
                double h = A.l1[x] * p1;
                h += A.l11[x] * c1;
                o2 += 4 * P1 * h;
                h = A.l1[x] * p2;
                h += A.l11[x] * c0;
                o2 += P0 * h;
            }
        } else {     // LGrad1::propagateB
            if (lft) {
                double h = A.l_1[x] * m2;
                h += A.l_11[x] * c0;
                o1 += P1 * h;
                o2 += P0 * h;
            }
            o0 += 4 * P1 * c1; o1 += (2 * P1 + P0) * c1; o2 += 4 * P1 * c1;
            if (rgt) {
                double h = A.l1[x] * p0;
                h += A.l11[x] * c2;
                o0 += P0 * h;
                o1 += P1 * h;
            }
        }
    }
    const double g = G1[x];
    o0 *= g; o1 *= g; o2 *= g;
    out[x] = o0;
    out[M + x] = o1;
    out[2 * M + x] = o2;
    if (BWD && x >= 1 && x <= A.MX) {
        double r = rho[x];
        r += (1.0 / 6.0) * gf[x] * o0;
        r += (4.0 / 6.0) * gf[M + x] * o1;
        r += (1.0 / 6.0) * gf[2 * M + x] * o2;
        rho[x] = r;
    }
}

// Initiate: every direction = G1 (all sites); with gf, also the composition
// of the backward sweep's first segment
__global__ void k_m2_init(int M, int MX, const double* __restrict__ G1, double* __restrict__ out,
                          const double* __restrict__ gf, double* __restrict__ rho) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= M) return;
    const double g = G1[x];
    out[x] = g;
    out[M + x] = g;
    out[2 * M + x] = g;
    if (gf && x >= 1 && x <= MX) {
        double r = rho[x];
        r += (1.0 / 6.0) * gf[x] * g;
        r += (4.0 / 6.0) * gf[M + x] * g;
        r += (1.0 / 6.0) * gf[2 * M + x] * g;
        rho[x] = r;
    }
}

// G(N) = (Σ_0 + 4·Σ_1 + Σ_2)/6 in the reference's order
__global__ void k_m2_gn(const double* __restrict__ w, double* __restrict__ out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double GN = w[0];
        GN += 4.0 * w[1];
        GN += w[2];
        *out = GN / 6.0;
    }
}

}  // namespace

// Device state of the context's Markov 2 molecules: the curvature weights
// and the backward pair (3 directions each), and three partial sums.
int ctx_m2_init(Ctx& C) {
    const nm_plan* p = C.plan;
    bool any = false;
    for (int m = 0; m < p->n_mol; m++) any = any || p->mols[m].markov == 2;
    if (!any) return NM_OK;
    if (p->gradients != 1 || p->lattice_type != NM_SIMPLE_CUBIC || C.fp32) {
        set_error("Markov 2 chains: FP64 contexts on 1-gradient simple-cubic lattices");
        return NM_ERR_INPUT;
    }
    const int M = p->M;
    auto grab = [&](double** q, size_t n) {
        return cudaMallocAsync((void**)q, sizeof(double) * n, C.stream) == cudaSuccess;
    };
    if (!grab(&C.d_m2gb, (size_t)2 * M2_FJC * M) || !grab(&C.d_m2w, 4)) {
        set_error("cudaMallocAsync (Markov 2)");
        return NM_ERR_NOMEM;
    }
    if (p->geometry != NM_PLANAR) {
        std::vector<double> l(4 * (size_t)M, 0.0);  // l1, l11, l_1, l_11; halos 0 (lattice.cpp:216-219)
        for (int i = 1; i < p->MX + 1; i++) {
            l[i] = p->lambda1[i] / p->lambda;
            l[M + i] = 1.0 - l[i];
            l[2 * M + i] = p->lambda_1[i] / p->lambda;
            l[3 * M + i] = 1.0 - l[2 * M + i];
        }
        if (!grab(&C.d_m2l, 4 * (size_t)M)) {
            set_error("cudaMallocAsync (Markov 2)");
            return NM_ERR_NOMEM;
        }
        if (cudaMemcpyAsync(C.d_m2l, l.data(), sizeof(double) * l.size(), cudaMemcpyHostToDevice, C.stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(C.stream) != cudaSuccess) {
            set_error("cudaMemcpyAsync (Markov 2)");
            return NM_ERR_CUDA;
        }
    }
    return NM_OK;
}

void ctx_m2_free(Ctx& C) {
    if (C.d_m2gb) cudaFreeAsync(C.d_m2gb, C.stream);
    if (C.d_m2w) cudaFreeAsync(C.d_m2w, C.stream);
    if (C.d_m2l) cudaFreeAsync(C.d_m2l, C.stream);
    C.d_m2gb = C.d_m2w = C.d_m2l = nullptr;
}

// Forward sweep (every Gf stored, 3·M each), G(N), backward sweep fused with
// the composition, of Markov 2 molecule m.
int ctx_m2_molecule_pass(Ctx& C, int m) {
    const nm_plan* p = C.plan;
    const nm_molecule& mol = p->mols[m];
    MolDev& D = C.mols[m];
    const int M = p->M, N = mol.n_store;
    const size_t V = (size_t)M2_FJC * M;
    M2Args A;
    A.M = M;
    A.MX = p->MX;
    A.bx1 = p->bc[0] == NM_BC_MIRROR ? 1 : (p->bc[0] == NM_BC_PERIODIC ? p->MX : 0);
    A.bxm = p->bc[3] == NM_BC_MIRROR ? p->MX : (p->bc[3] == NM_BC_PERIODIC ? 1 : p->MX + 1);
    A.P0 = mol.bend[0];
    A.P1 = mol.bend[1];
    const bool curv = p->geometry != NM_PLANAR;
    A.l1 = curv ? C.d_m2l : nullptr;
    A.l11 = curv ? C.d_m2l + M : nullptr;
    A.l_1 = curv ? C.d_m2l + 2 * M : nullptr;
    A.l_11 = curv ? C.d_m2l + 3 * M : nullptr;
    const int grid = (M + 127) / 128;
    if (cudaMemsetAsync(D.rho, 0, sizeof(double) * M * mol.n_molmon, C.stream) != cudaSuccess) {
        set_error("cudaMemsetAsync (Markov 2)");
        return NM_ERR_CUDA;
    }
    // forward
    int s = 0;
    for (int b = 0; b < mol.n_blocks; b++) {
        const nm_block& B = mol.blocks[b];
        const double* G1 = C.d_G1 + (size_t)B.seg * M;
        for (int k = 0; k < B.length; k++, s++) {
            double* out = D.Gf + (size_t)s * V;
            if (s == 0) k_m2_init<<<grid, 128, 0, C.stream>>>(M, p->MX, G1, out, nullptr, nullptr);
            else if (curv) k_m2_step<false, true><<<grid, 128, 0, C.stream>>>(A, out - V, G1, out, nullptr, nullptr);
            else k_m2_step<false, false><<<grid, 128, 0, C.stream>>>(A, out - V, G1, out, nullptr, nullptr);
            C.launches++;
        }
    }
    // G(N): the three directions' weighted sums of the last propagator
    const double* last = D.Gf + (size_t)(N - 1) * V;
    for (int d = 0; d < M2_FJC; d++) C.wsum(last + (size_t)d * M, C.d_m2w + d);
    k_m2_gn<<<1, 32, 0, C.stream>>>(C.d_m2w, C.d_sc + 5 * m);
    C.launches++;
    // backward, fused with the composition
    s = N - 1;
    for (int b = mol.n_blocks - 1; b >= 0; b--) {
        const nm_block& B = mol.blocks[b];
        const double* G1 = C.d_G1 + (size_t)B.seg * M;
        double* rho = D.rho + (size_t)B.molmon * M;
        for (int k = 0; k < B.length; k++, s--) {
            double* cur = C.d_m2gb + (size_t)(s % 2) * V;
            const double* gf = D.Gf + (size_t)s * V;
            if (s == N - 1) k_m2_init<<<grid, 128, 0, C.stream>>>(M, p->MX, G1, cur, gf, rho);
            else if (curv)
                k_m2_step<true, true><<<grid, 128, 0, C.stream>>>(A, C.d_m2gb + (size_t)((s + 1) % 2) * V, G1, cur, gf, rho);
            else
                k_m2_step<true, false><<<grid, 128, 0, C.stream>>>(A, C.d_m2gb + (size_t)((s + 1) % 2) * V, G1, cur, gf, rho);
            C.launches++;
        }
    }
    return NM_OK;
}

}  // namespace nm
