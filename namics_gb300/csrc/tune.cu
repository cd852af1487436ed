// The autotuner of the device contexts: for the problem at hand it times one
// residual evaluation per candidate of the kernel choices that leave the
// arithmetic unchanged, keeps the fastest and remembers it per shape.
//   3-D path: the step kernel (the gather kernel with 2, 4 or 8 rows along
//     y per block, or a 2.5-D shared-memory tile of 2 or 4 rows marching 4
//     or 8 planes) × the checkpoint stride of the stored propagators (0, 5,
//     10; recomputing a group of segments from L2 against reading every
//     forward propagator back from HBM);
//     On small FP32 boxes, also the cluster-resident sweeps (one
//     thread-block cluster per sweep, every propagator stored);
//   2-D linear chains: one launch per segment step or one persistent
//     cooperative launch per sweep.
// Every candidate gives bit-identical residuals, so the choice is speed only.
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "ctx_internal.h"

namespace nm {

namespace {

struct Choice { int rows, ck, sweep, tile, cluster; };

std::mutex g_tune_mu;
std::map<std::string, Choice> g_tuned;  // shape -> choice

std::string shape_key(const Ctx& C) {
    const nm_plan* p = C.plan;
    std::string k = std::to_string(p->gradients) + ":" + std::to_string(p->MX) + "x" + std::to_string(p->MY) + "x" +
                    std::to_string(p->MZ) + ":" + (C.fp32 ? "f32" : "f64");
    for (int m = 0; m < p->n_mol; m++) k += ":" + std::to_string(p->mols[m].n_store);
    return k;
}

void drop_graph(Ctx& C) {
    if (C.graph) {
        cudaGraphExecDestroy(C.graph);
        C.graph = nullptr;
    }
    ctx_loop_drop(C);
}

int apply(Ctx& C, const Choice& c) {
    if (c.rows > 0) C.c3_rows = c.rows;
    if (c.tile >= 0) {
        if (int rc = ctx3d_set_tile(C, c.tile)) return rc;
    }
    if (c.ck >= 0) {
        if (int rc = C.set_ck_stride(c.ck)) return rc;
    }
    if (c.sweep >= 0) C.sweep2d = c.sweep != 0;
    if (c.cluster >= 0) C.c3c_on = c.cluster != 0 && C.c3c_ctas > 0;
    drop_graph(C);
    return NM_OK;
}

// mean time of `reps` residual evaluations after one untimed one
int time_residual(Ctx& C, const double* x, int reps, double& ms) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = C.residual(x, C.d_g);
    if (!rc) {
        cudaEventRecord(e0, C.stream);
        for (int i = 0; i < reps && !rc; i++) rc = C.residual(x, C.d_g);
        cudaEventRecord(e1, C.stream);
    }
    cudaError_t e = cudaEventSynchronize(e1);
    float t = 0;
    if (!rc && e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!rc && e != cudaSuccess) { set_error(std::string("autotune: ") + cudaGetErrorString(e)); rc = NM_ERR_CUDA; }
    if (!rc) rc = C.check_status();
    ms = t / reps;
    return rc;
}

}  // namespace

}  // namespace nm

extern "C" int nm_ctx_autotune(nm_ctx* ctx, const double* x_dev, nm_ctx_tuning* out) {
    using namespace nm;
    Ctx* C = reinterpret_cast<Ctx*>(ctx);
    if (!C || !x_dev || !out) { set_error("nm_ctx_autotune: null argument"); return NM_ERR_ARG; }
    std::vector<Choice> cands;
    const int cl = C->c3c_ctas > 0 ? 0 : -1;  // per-step candidates leave the cluster sweeps off
    if (C->use3d) {
        for (int ck : {0, 5, 10}) {
            for (int rows : {2, 4, 8}) cands.push_back({rows, ck, -1, 0, cl});
            for (int tile : {204, 208, 404, 408}) cands.push_back({-1, ck, -1, tile, cl});
        }
        if (C->c3c_ctas > 0) cands.push_back({-1, 0, -1, 0, 1});
    } else if (C->use2d) {
        cands.push_back({-1, -1, 0, -1, -1});
        cands.push_back({-1, -1, 1, -1, -1});
    }
    out->rows = C->use3d ? C->c3_rows : -1;
    out->tile = C->use3d ? C->c3_tile : -1;
    out->checkpoint_stride = C->use3d ? C->ck_stride : -1;
    out->sweep2d = C->use2d ? (C->sweep2d ? 1 : 0) : -1;
    out->cluster3d = C->c3c_ctas > 0 ? (C->c3c_on ? 1 : 0) : -1;
    out->candidates = 0;
    out->ms_per_residual = 0;
    if (cands.empty()) return time_residual(*C, x_dev, 3, out->ms_per_residual);  // nothing to choose
    const std::string key = shape_key(*C);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end() && apply(*C, it->second) == NM_OK) {
            out->rows = C->use3d ? C->c3_rows : -1;
            out->tile = C->use3d ? C->c3_tile : -1;
            out->checkpoint_stride = C->use3d ? C->ck_stride : -1;
            out->sweep2d = C->use2d ? (C->sweep2d ? 1 : 0) : -1;
            out->cluster3d = C->c3c_ctas > 0 ? (C->c3c_on ? 1 : 0) : -1;
            return NM_OK;
        }
    }
    const Choice before{C->use3d ? C->c3_rows : -1, C->use3d ? C->ck_stride : -1,
                        C->use2d ? (C->sweep2d ? 1 : 0) : -1, C->use3d ? C->c3_tile : -1,
                        C->c3c_ctas > 0 ? (C->c3c_on ? 1 : 0) : -1};
    double best = 1e300;
    Choice pick = before;
    for (const Choice& c : cands) {
        if (apply(*C, c) != NM_OK) continue;  // a stride that does not fit the storage
        double ms = 0;
        if (int rc = time_residual(*C, x_dev, 3, ms)) { apply(*C, before); return rc; }
        out->candidates++;
        if (ms < best) { best = ms; pick = c; }
    }
    if (int rc = apply(*C, pick)) return rc;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tuned[key] = pick;
    }
    out->rows = C->use3d ? C->c3_rows : -1;
    out->tile = C->use3d ? C->c3_tile : -1;
    out->checkpoint_stride = C->use3d ? C->ck_stride : -1;
    out->sweep2d = C->use2d ? (C->sweep2d ? 1 : 0) : -1;
    out->cluster3d = C->c3c_ctas > 0 ? (C->c3c_on ? 1 : 0) : -1;
    out->ms_per_residual = best;
    return NM_OK;
}
