// Lattice- and molecule-level pieces of the hot path behind the C ABI, for a
// caller that keeps the reference's own Molecule::ComputePhi loop and moves
// only its arithmetic onto the device.  Each entry point works on device
// arrays of the context's lattice (length M, the reference's padded layout)
// on the context's stream, and returns after the stream has finished.
//
// Markov-1 chains (the kind these entry points take); the arithmetic over all M
// entries, halo layers included, as the reference's flat-array loops do:
//   AddPhiS(phi, Gf, Gb)              phi += Gf·Gb          (AddTimes)
//   AddPhiS(phi, Gf, Gb, d)           phi += d·Gf·Gb        (YplusisCtimesAtimesB)
//   AddPhiS(phi, Gf, Gb, G1, norm)    phi += norm·Gf·Gb/G1 where G1 > 0
//                                     (Composition; 1 gradient only, as in the
//                                     reference)
//   Initiate(G, Gz)                   G = Gz
//   Terminate(Gz, G)                  Gz = G
//   WeightedSum(X), ComputeGN(G)      halos zeroed in place (remove_bounds), then
//                                     Σ X (planar, 3-D) or Σ X·L (curved)
// LGrad1.cpp:213-220, 863-969; LGrad2.cpp:147-157, 1814-1960;
// LGrad3.cpp:40-46, 1883-1945; tools_host.h:349-356, 400-402.
#include <cuda_runtime.h>

#include <string>

#include "ctx_internal.h"

namespace nm {

// op 0: phi += a·b; op 1: phi += c·a·b; op 2: phi += c·a·b/g1 where g1 > 0
__global__ void k_addphi(int M, int op, double* __restrict__ phi, const double* __restrict__ a,
                         const double* __restrict__ b, const double* __restrict__ g1, double c) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
        if (op == 0) phi[i] = __dadd_rn(phi[i], __dmul_rn(a[i], b[i]));
        else if (op == 1) phi[i] = __dadd_rn(phi[i], __dmul_rn(__dmul_rn(c, a[i]), b[i]));
        else if (g1[i] > 0) phi[i] = __dadd_rn(phi[i], __ddiv_rn(__dmul_rn(__dmul_rn(c, a[i]), b[i]), g1[i]));
    }
}

__global__ void k_copy_all(int M, double* __restrict__ dst, const double* __restrict__ src) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) dst[i] = src[i];
}

// remove_bounds: every halo site of the padded array to 0
__global__ void k_remove_bounds(nmdev::Lat L, double* __restrict__ X) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L.M; i += gridDim.x * blockDim.x)
        if (!nmdev::is_interior(L, i)) X[i] = 0.0;
}

static int sync_ctx(Ctx* c, const char* who) {
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) { set_error(std::string(who) + ": " + cudaGetErrorString(e)); return NM_ERR_CUDA; }
    return NM_OK;
}

static int grid_m(int M) { return (M + 255) / 256 < 4096 ? (M + 255) / 256 : 4096; }

static int add_phi(nm_ctx* ctx, int op, double* phi, const double* Gf, const double* Gb, const double* G1, double c,
                   const char* who) {
    Ctx* C = reinterpret_cast<Ctx*>(ctx);
    if (!C || !phi || !Gf || !Gb || (op == 2 && !G1)) { set_error(std::string(who) + ": null argument"); return NM_ERR_ARG; }
    if (op == 2 && C->plan->gradients != 1) {
        // LGrad2/LGrad3::AddPhiS with G1 and norm print "not implemented" and
        // leave phi unchanged; here phi is left unchanged and the call fails
        set_error(std::string(who) + ": the G1/norm composition exists for 1-gradient lattices only");
        return NM_ERR_INPUT;
    }
    int M = C->plan->M;
    k_addphi<<<grid_m(M), 256, 0, C->stream>>>(M, op, phi, Gf, Gb, G1, c);
    C->launches++;
    return sync_ctx(C, who);
}

static int weighted_sum(nm_ctx* ctx, double* X, double* out, const char* who) {
    Ctx* C = reinterpret_cast<Ctx*>(ctx);
    if (!C || !X || !out) { set_error(std::string(who) + ": null argument"); return NM_ERR_ARG; }
    k_remove_bounds<<<grid_m(C->plan->M), 256, 0, C->stream>>>(C->lat, X);
    C->launches++;
    // Ctx::wsum sums the interior (the halo is 0 now), weighted by L on curved
    // 1- and 2-gradient lattices
    C->wsum(X, C->d_resid);
    cudaError_t e = cudaMemcpyAsync(out, C->d_resid, sizeof(double), cudaMemcpyDeviceToHost, C->stream);
    if (e != cudaSuccess) { set_error(std::string(who) + ": " + cudaGetErrorString(e)); return NM_ERR_CUDA; }
    return sync_ctx(C, who);
}

}  // namespace nm

using nm::Ctx;

extern "C" {

int nm_add_phi_dev(nm_ctx* ctx, double* phi_dev, const double* Gf_dev, const double* Gb_dev) {
    return nm::add_phi(ctx, 0, phi_dev, Gf_dev, Gb_dev, nullptr, 0.0, "nm_add_phi_dev");
}

int nm_add_phi_deg_dev(nm_ctx* ctx, double* phi_dev, const double* Gf_dev, const double* Gb_dev, double degeneracy) {
    return nm::add_phi(ctx, 1, phi_dev, Gf_dev, Gb_dev, nullptr, degeneracy, "nm_add_phi_deg_dev");
}

int nm_add_phi_norm_dev(nm_ctx* ctx, double* phi_dev, const double* Gf_dev, const double* Gb_dev,
                        const double* G1_dev, double norm) {
    return nm::add_phi(ctx, 2, phi_dev, Gf_dev, Gb_dev, G1_dev, norm, "nm_add_phi_norm_dev");
}

int nm_initiate_dev(nm_ctx* ctx, double* G_dev, const double* Gz_dev) {
    Ctx* C = reinterpret_cast<Ctx*>(ctx);
    if (!C || !G_dev || !Gz_dev) { nm::set_error("nm_initiate_dev: null argument"); return NM_ERR_ARG; }
    nm::k_copy_all<<<nm::grid_m(C->plan->M), 256, 0, C->stream>>>(C->plan->M, G_dev, Gz_dev);
    C->launches++;
    return nm::sync_ctx(C, "nm_initiate_dev");
}

int nm_terminate_dev(nm_ctx* ctx, double* Gz_dev, const double* G_dev) {
    Ctx* C = reinterpret_cast<Ctx*>(ctx);
    if (!C || !Gz_dev || !G_dev) { nm::set_error("nm_terminate_dev: null argument"); return NM_ERR_ARG; }
    nm::k_copy_all<<<nm::grid_m(C->plan->M), 256, 0, C->stream>>>(C->plan->M, Gz_dev, G_dev);
    C->launches++;
    return nm::sync_ctx(C, "nm_terminate_dev");
}

int nm_weighted_sum_dev(nm_ctx* ctx, double* X_dev, double* sum) {
    return nm::weighted_sum(ctx, X_dev, sum, "nm_weighted_sum_dev");
}

int nm_compute_gn_dev(nm_ctx* ctx, double* G_dev, double* GN) {
    return nm::weighted_sum(ctx, G_dev, GN, "nm_compute_gn_dev");
}

int nm_compose_dev(nm_ctx* ctx, int mol, const double* x_dev, double* rho_dev, double* GN) {
    Ctx* C = reinterpret_cast<Ctx*>(ctx);
    if (!C || !x_dev || !rho_dev) { nm::set_error("nm_compose_dev: null argument"); return NM_ERR_ARG; }
    const nm_plan* P = C->plan;
    if (mol < 0 || mol >= P->n_mol) { nm::set_error("nm_compose_dev: molecule index out of range"); return NM_ERR_ARG; }
    int M = P->M;
    if (C->charged) C->elec_field(x_dev);
    C->launch_g1(x_dev, false);
    int rc = C->use3d ? nm::ctx3d_molecule_pass(*C, mol, false) : C->molecule_pass(mol);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(rho_dev, C->mols[mol].rho, sizeof(double) * (size_t)M * P->mols[mol].n_molmon,
                                    cudaMemcpyDeviceToDevice, C->stream);
    if (e == cudaSuccess && GN)
        e = cudaMemcpyAsync(GN, C->d_sc + 5 * mol, sizeof(double), cudaMemcpyDeviceToHost, C->stream);
    if (e != cudaSuccess) { nm::set_error(std::string("nm_compose_dev: ") + cudaGetErrorString(e)); return NM_ERR_CUDA; }
    C->have_state = false;  // G1 and the propagators no longer belong to a residual
    return nm::sync_ctx(C, "nm_compose_dev");
}

}  // extern "C"
