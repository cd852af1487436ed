// The device-resident solve loop of a context (NM_OPT_DEVICE_LOOP): the
// whole DIIS iteration of Ctx::solve (Solve_scf / SFNewton::iterate_DIIS,
// sfnewton.cpp:1037-1130) as ONE CUDA graph with a conditional WHILE node,
// so a solve returns to the host once, at its end, instead of once per
// iteration.
//
// Graph:  WHILE (continue) {
//           pre        : IF handles ← the state's precision phase
//           IF (FP32)  { residual with FP32 propagators; its norm and status:
//                        a failure of the reduced precision switches to FP64
//                        at the same x (sets the FP64 handle) }
//           IF (FP64)  { residual with FP64 propagators }
//           step       : x ← x − δ·g into history slot k = it mod m, ‖g‖ partials
//           norm       : ‖g‖ (2-norm or max-norm, fixed-order sums)
//           gram       : ⟨Δx_i, Δx_k⟩ partials of the history window
//           control    : the Gram row (+1e-9), the small solve, the phase
//                        switch, the stopping test, it++ and the WHILE handle
//           mix        : x ← Σ c_i·xR_i }
// The control logic is the host loop's, statement for statement (the first
// pass is the initial residual and plain mixing step into slot 0), and so is
// the small solve: the pseudo-inverse of a cyclic Jacobi eigen-decomposition
// with the host's rotation order, one warp (warp_pinv_solve), so the two
// loops take the same DIIS path up to rounding.  (Gaussian elimination, the
// batched 1-D solver's warp_solve, was tried here first: on a 3-D melt whose
// early Gram matrices are ill-conditioned its coefficients ran the fields away
// within five iterations where the pseudo-inverse's stay finite.)  The WHILE
// loop ends: every pass increments `it` and stops at the iteration limit.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>

#include "ctx_internal.h"
#include "warp_solve.cuh"

namespace nm {

struct LoopState {
    int it, k_diis, phase32, rc, first, since_best, mix, mix_k, mix_kd, max_iter, n32, n64;
    double resid, resid_new, best, tol;
    double Aij[NM_MAX_DIIS * NM_MAX_DIIS];  // the Gram window, m×m
    double Ci[NM_MAX_DIIS];                 // the mixing coefficients
};

namespace {

constexpr int KL_THREADS = 256;

__device__ __forceinline__ double kl_block_sum(double v, double* sh) {  // fixed order
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    double r = 0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) r += sh[i];
    __syncthreads();
    return r;
}

// ‖g‖ from per-block partials: the max (max-norm) or √Σ, thread 0's value
__device__ double kl_final(const double* __restrict__ partial, int nb, int max_norm, double* sh) {
    if (max_norm) {
        double r = 0;
        if (threadIdx.x == 0)
            for (int i = 0; i < nb; i++) r = fmax(r, partial[i]);
        return r;
    }
    double acc = 0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) acc += partial[i];
    return sqrt(kl_block_sum(acc, sh));
}

__global__ void kl_pre(LoopState* S, cudaGraphConditionalHandle h32, cudaGraphConditionalHandle h64, int has32) {
    if (threadIdx.x == 0) {
        const int p = S->phase32;
        if (p) S->n32++;
        else S->n64++;
        if (has32) cudaGraphSetConditional(h32, p ? 1u : 0u);
        cudaGraphSetConditional(h64, p ? 0u : 1u);
    }
}

// Σ g² (or max |g|) partials; update = 1 also moves x and fills history slot k
__global__ void kl_step(LoopState* S, int n, int m, double dmax, double* __restrict__ x, const double* __restrict__ g,
                        double* __restrict__ xR, double* __restrict__ xx0, double* __restrict__ partial, int max_norm,
                        int update) {
    __shared__ double sh[32];
    const int k = S->first ? 0 : S->it % m;
    double* xr = xR + (size_t)k * n;
    double* xd = xx0 + (size_t)k * n;
    double acc = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double gv = g[i];
        if (update) {
            const double xo = x[i];
            const double xn = xo + (-dmax) * gv;
            x[i] = xn;
            xr[i] = xn;
            xd[i] = xn - xo;
        }
        if (max_norm) acc = fmax(acc, fabs(gv));
        else acc += gv * gv;
    }
    if (max_norm) {
        for (int o = 16; o > 0; o >>= 1) acc = fmax(acc, __shfl_down_sync(0xffffffffu, acc, o));
        const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
        if (l == 0) sh[w] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double r = 0;
            for (int i = 0; i < (int)(blockDim.x >> 5); i++) r = fmax(r, sh[i]);
            partial[blockIdx.x] = r;
        }
    } else {
        const double r = kl_block_sum(acc, sh);
        if (threadIdx.x == 0) partial[blockIdx.x] = r;
    }
}

// the FP32 residual's norm and the device status: a failure of the reduced
// precision (G(N) <= 0, a non-finite residual) hands over to FP64 at the same x
__global__ void kl_check32(LoopState* S, const double* __restrict__ partial, int nb, int max_norm, int* status,
                           cudaGraphConditionalHandle h64) {
    __shared__ double sh[32];
    const double r = kl_final(partial, nb, max_norm, sh);
    if (threadIdx.x == 0) {
        const int st = *status;
        if (st || !isfinite(r)) {
            *status = 0;
            S->phase32 = 0;
            S->k_diis = 0;
            S->n64++;
            cudaGraphSetConditional(h64, 1u);
        }
    }
}

__global__ void kl_norm(LoopState* S, const double* __restrict__ partial, int nb, int max_norm) {
    __shared__ double sh[32];
    const double r = kl_final(partial, nb, max_norm, sh);
    if (threadIdx.x == 0) S->resid_new = r;
}

// Gram row partials: partial[i·nb + b] = Σ_b Δx[posi_i]·Δx[k], i < kd
__global__ void kl_gram(LoopState* S, int n, int m, const double* __restrict__ xx0, double* __restrict__ partial) {
    __shared__ double sh[32];
    if (S->first) return;
    const int k = S->it % m;
    const int kd = min(S->k_diis + 1, m);
    const int i = blockIdx.y;
    if (i >= kd) return;
    int posi = k - kd + 1 + i;
    if (posi < 0) posi += m;
    const double* a = xx0 + (size_t)posi * n;
    const double* b = xx0 + (size_t)k * n;
    double acc = 0;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) acc += a[j] * b[j];
    const double r = kl_block_sum(acc, sh);
    if (threadIdx.x == 0) partial[(size_t)i * gridDim.x + blockIdx.x] = r;
}

// The host loop's control statements (Ctx::solve), one warp.
__global__ void kl_control(LoopState* S, const double* __restrict__ gpart, int nb, int m, int nvar, double sw_floor,
                           int* status, cudaGraphConditionalHandle hl) {
    __shared__ double As[NM_MAX_DIIS * NM_MAX_DIIS], Ci[NM_MAX_DIIS];
    __shared__ double Ja[NM_MAX_DIIS * NM_MAX_DIIS], Jq[NM_MAX_DIIS * NM_MAX_DIIS];
    const int lane = threadIdx.x & 31;
    // the state as the pass left it, in every lane before lane 0 changes it
    double resid = S->resid_new;
    const int first = S->first, it = S->it, k_diis0 = S->k_diis, max_iter = S->max_iter;
    const double tol = S->tol;
    __syncwarp();
    int cont;
    if (first) {  // the initial residual and plain mixing step
        int rc = 0;
        if (lane == 0) {
            S->first = 0;
            S->mix = 0;
            const int st = *status;
            if (st) { *status = 0; rc = st; }
            S->rc = rc;
            S->resid = resid;
        }
        rc = __shfl_sync(0xffffffffu, rc, 0);
        cont = !rc && !(resid <= tol) && it < max_iter;
    } else {
        int rc = 0;
        const int k = it % m;
        const int k_diis = k_diis0 + 1;
        const int kd = k_diis > m ? m : k_diis;
        if (lane == 0) {
            const int st = *status;
            if (st) { *status = 0; rc = st; }
            S->k_diis = k_diis;
        }
        rc = __shfl_sync(0xffffffffu, rc, 0);
        if (!rc) {
            // Gram row (fixed-order sums of the block partials), the m×m
            // window slid once it is full, +1e-9 (sfnewton.cpp:837-880)
            if (lane == 0) {
                if (k_diis > m)
                    for (int i = 1; i < m; i++)
                        for (int j = 1; j < m; j++) S->Aij[m * (i - 1) + j - 1] = S->Aij[m * i + j];
                for (int i = 0; i < kd; i++) {
                    double D = 0;
                    for (int b = 0; b < nb; b++) D += gpart[(size_t)i * nb + b];
                    S->Aij[i + m * (kd - 1)] = S->Aij[kd - 1 + m * i] = D + 1e-9;
                }
            }
            __syncwarp();
            bool nan = false;
            for (int e = lane; e < kd * kd; e += 32) {
                const int i = e / kd, j = e % kd;
                const double v = S->Aij[j + m * i];
                if (v != v) nan = true;
                As[i * kd + j] = v;
            }
            nan = __any_sync(0xffffffffu, nan);
            __syncwarp();
            if (nan) {
                rc = NM_ERR_NAN_DIIS;
            } else {
                warp_pinv_solve(As, Ci, kd, Ja, Jq);
                if (lane == 0) {
                    double nC = 0;
                    for (int i = 0; i < kd; i++) nC += Ci[i];
                    for (int i = 0; i < kd; i++) {
                        S->Ci[i] = Ci[i] / nC;
                        if (S->Ci[i] != S->Ci[i]) rc = NM_ERR_NAN_SVD;
                    }
                }
                rc = __shfl_sync(0xffffffffu, rc, 0);
            }
        }
        if (lane == 0) {
            S->mix = rc == 0;
            S->mix_k = k;
            S->mix_kd = kd;
            cont = -1;
            if (S->phase32) {
                // FP32 propagators until a stall near their accuracy floor (or
                // an FP32 failure), then FP64 residuals with the history restarted
                if (resid < 0.9 * S->best) { S->best = resid; S->since_best = 0; }
                else S->since_best++;
                const bool fail = rc != 0 || !isfinite(resid);
                if (fail || resid <= tol || resid < sw_floor || (S->since_best > 10 && resid < 10.0 * sw_floor) ||
                    (S->since_best > 25 && resid < 1e-2 * sqrt((double)nvar))) {
                    S->phase32 = 0;
                    rc = 0;
                    S->k_diis = 0;
                    resid = 1e300;  // re-evaluated in FP64 by the next pass
                    cont = it < max_iter;
                }
            }
            if (cont < 0) {
                if (!rc && !isfinite(resid)) rc = NM_ERR_NAN_DIIS;
                cont = !rc && !(resid <= tol) && it < max_iter;
            }
            S->rc = rc;
            S->resid = resid;
        }
        cont = __shfl_sync(0xffffffffu, cont, 0);
    }
    if (lane == 0) {
        if (cont) S->it = it + 1;
        cudaGraphSetConditional(hl, cont ? 1u : 0u);
    }
}

__global__ void kl_mix(const LoopState* S, int n, int m, double* __restrict__ x, const double* __restrict__ xR) {
    if (!S->mix) return;
    const int k = S->mix_k, kd = S->mix_kd;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        double v = 0;
        for (int i = 0; i < kd; i++) {
            int posi = k - kd + 1 + i;
            if (posi < 0) posi += m;
            v += S->Ci[i] * xR[(size_t)posi * n + j];
        }
        x[j] = v;
    }
}

}  // namespace

#define LK(call)                                                                           \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            set_error(std::string("device solve loop: ") + cudaGetErrorString(e_) + " (" + \
                      #call + ")");                                                        \
            return NM_ERR_CUDA;                                                            \
        }                                                                                  \
    } while (0)

static int add_if(Ctx& C, cudaGraphConditionalHandle h, cudaGraph_t* body_out) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    LK(cudaStreamGetCaptureInfo(C.stream, &cs, nullptr, &g, &deps, nullptr, &nd));
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeIf;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    LK(cudaGraphAddNode(&node, g, deps, nullptr, nd, &p));
    *body_out = p.conditional.phGraph_out[0];
    LK(cudaStreamUpdateCaptureDependencies(C.stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    return NM_OK;
}

// Build and instantiate the solve graph for the field x (device, in place).
static int build_loop(Ctx& C, double* x, bool plain_launches) {
    const nm_plan* p = C.plan;
    const int n = p->iv, m = p->diis_m, nb = C.red_blocks;
    LoopState* S = (LoopState*)C.d_loop;
    cudaGraph_t g = nullptr, body = nullptr, b32 = nullptr, b64 = nullptr;
    LK(cudaGraphCreate(&g, 0));
    struct Guard { cudaGraph_t& g; ~Guard() { if (g) cudaGraphDestroy(g); } } guard{g};
    cudaGraphConditionalHandle hl, h32, h64;
    LK(cudaGraphConditionalHandleCreate(&hl, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams wp = {};
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = hl;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wn;
    LK(cudaGraphAddNode(&wn, g, nullptr, nullptr, 0, &wp));
    body = wp.conditional.phGraph_out[0];
    // a handle must belong to a conditional node: an FP64 context has no FP32 branch
    h32 = 0;
    if (C.fp32) LK(cudaGraphConditionalHandleCreate(&h32, body, 0, 0));
    LK(cudaGraphConditionalHandleCreate(&h64, body, 0, 0));
    const bool saved = C.phase32;
    long long l0 = C.launches;
    struct Plain {
        explicit Plain(bool on) { g_plain_launch = on; }
        ~Plain() { g_plain_launch = false; }
    } plain(plain_launches);
    // the pass
    LK(cudaStreamBeginCaptureToGraph(C.stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    int rc = NM_OK;
    {
        kl_pre<<<1, 32, 0, C.stream>>>(S, h32, h64, C.fp32 ? 1 : 0);
        if (C.fp32) rc = add_if(C, h32, &b32);  // an FP64 context never takes the FP32 branch
        if (!rc) rc = add_if(C, h64, &b64);
        if (!rc) {
            kl_step<<<nb, KL_THREADS, 0, C.stream>>>(S, n, m, p->deltamax, x, C.d_g, C.d_xR, C.d_xx0, C.d_partial,
                                                    p->max_norm, 1);
            kl_norm<<<1, KL_THREADS, 0, C.stream>>>(S, C.d_partial, nb, p->max_norm);
            kl_gram<<<dim3(nb, m), KL_THREADS, 0, C.stream>>>(S, n, m, C.d_xx0, C.d_gram_partial);
            kl_control<<<1, 32, 0, C.stream>>>(S, C.d_gram_partial, nb, m, n, C.sw_floor, C.d_status, hl);
            kl_mix<<<(n + 255) / 256 < 4 * 152 ? (n + 255) / 256 : 4 * 152, 256, 0, C.stream>>>(S, n, m, x, C.d_xR);
        }
    }
    cudaGraph_t got = nullptr;
    cudaError_t e = cudaStreamEndCapture(C.stream, &got);
    if (rc) return rc;
    LK(e);
    C.loop_lrest = 6;
    // FP32 branch: the residual, then its norm and status
    if (C.fp32) {
        LK(cudaStreamBeginCaptureToGraph(C.stream, b32, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        C.phase32 = true;
        const long long a = C.launches;
        rc = C.residual_launches(x, C.d_g);
        if (!rc) {
            kl_step<<<nb, KL_THREADS, 0, C.stream>>>(S, n, m, 0.0, x, C.d_g, C.d_xR, C.d_xx0, C.d_partial,
                                                    p->max_norm, 0);
            kl_check32<<<1, KL_THREADS, 0, C.stream>>>(S, C.d_partial, nb, p->max_norm, C.d_status, h64);
        }
        C.loop_l32 = C.launches - a + 2;
        e = cudaStreamEndCapture(C.stream, &got);
        C.phase32 = saved;
        if (rc) return rc;
        LK(e);
    }
    LK(cudaStreamBeginCaptureToGraph(C.stream, b64, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    C.phase32 = false;
    const long long a = C.launches;
    rc = C.residual_launches(x, C.d_g);
    C.loop_l64 = C.launches - a;
    e = cudaStreamEndCapture(C.stream, &got);
    C.phase32 = saved;
    C.launches = l0;
    if (rc) return rc;
    LK(e);
    if (C.loop_graph) { cudaGraphExecDestroy(C.loop_graph); C.loop_graph = nullptr; }
    cudaGraphInstantiateParams ip = {};
    e = cudaGraphInstantiateWithParams(&C.loop_graph, g, &ip);
    if (e != cudaSuccess) {
        cudaGraphNodeType t = cudaGraphNodeTypeEmpty;
        if (ip.errNode_out) cudaGraphNodeGetType(ip.errNode_out, &t);
        set_error(std::string("device solve loop: instantiation: ") + cudaGetErrorString(e) + ", result " +
                  std::to_string((int)ip.result_out) + ", node type " + std::to_string((int)t));
        C.loop_graph = nullptr;
        return NM_ERR_CUDA;
    }
    C.loop_x = x;
    return NM_OK;
}

int ctx_loop_solve(Ctx& C, double* x, nm_solve_result* res, int max_iter) {
    const nm_plan* p = C.plan;
    if (!C.d_loop) LK(cudaMallocAsync(&C.d_loop, sizeof(LoopState), C.stream));
    if (!C.loop_graph || C.loop_x != x) {
        // plain stream-order edges inside the conditional bodies
        if (int rc = build_loop(C, x, true)) return rc;
    }
    LoopState h;
    std::memset(&h, 0, sizeof(h));
    h.phase32 = C.fp32 ? 1 : 0;
    h.first = 1;
    h.max_iter = max_iter;
    h.best = 1e300;
    h.tol = C.tol_override > 0 ? C.tol_override : p->tolerance;
    LK(cudaMemcpyAsync(C.d_loop, &h, sizeof(h), cudaMemcpyHostToDevice, C.stream));
    LK(cudaGraphLaunch(C.loop_graph, C.stream));
    LK(cudaMemcpyAsync(&h, C.d_loop, sizeof(h), cudaMemcpyDeviceToHost, C.stream));
    LK(cudaStreamSynchronize(C.stream));
    C.launches += (long long)h.n32 * C.loop_l32 + (long long)h.n64 * C.loop_l64 +
                  (long long)(h.n32 + h.n64) * C.loop_lrest;
    C.have_state = true;
    res->iterations = h.it;
    res->residual = h.resid;
    res->status = h.rc ? h.rc : (h.resid > h.tol ? NM_ERR_NOT_CONVERGED : NM_OK);
    if (h.rc) set_error("device status " + std::to_string(h.rc));
    return h.rc;
}

void ctx_loop_drop(Ctx& C) {
    if (C.loop_graph) { cudaGraphExecDestroy(C.loop_graph); C.loop_graph = nullptr; }
    C.loop_x = nullptr;
}

}  // namespace nm
