// Request server: continuous batching of SCF solves on one GPU.
//
// Requests of any gradient count arrive one at a time (nm_server_submit) and
// are solved on the device while others are running.
//   - 1-gradient requests go straight into the streaming work loop
//     (nm_stream_*): a persistent launch whose resident CTAs take each
//     request the moment one of them is free, with the field, stored
//     propagators and DIIS history in that slot's device memory until it
//     converged.  A request outside the loop's envelope, or one that finds
//     the ring full, takes the path below as a batched problem.
//   - W worker threads each own a CUDA stream.  A free worker takes work
//     from the queue: a waiting 1-gradient request together with every
//     other waiting one, up to max_batch, in one batched launch; any other
//     request alone in a device context (2-D, 3-D; FP32 propagators for 3-D
//     simple-cubic linear chains).
// Work is admitted by device footprint: a request (or group) starts only when
// its estimated memory fits beside what is already running, so memory never
// oversubscribes; a request larger than the whole budget is rejected at
// submit.  All state a solve needs is created on the worker's stream with
// stream-ordered allocation, so admitting a request never synchronises the
// device and solves on the other streams keep running.  Each request records
// the time from submit to completion.
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "ctx_internal.h"

namespace nm {

namespace {

using clk = std::chrono::steady_clock;

struct Request {
    long long id = 0;
    const nm_plan* plan = nullptr;
    std::vector<double> x;
    size_t bytes = 0;
    bool batched = false;
    long long ticket = -1;  // >= 0: solved by the streaming work loop
    clk::time_point t_submit, t_done;
    nm_solve_result res{};
    int rc = 0;
    bool done = false;
};

// Estimated device footprint of one request: stored propagators and block
// vectors, per-site arrays, DIIS history (both precisions' buffers counted
// where the FP32 path keeps both).
size_t footprint(const nm_plan* p, bool batched, int precision) {
    const size_t M = (size_t)p->M;
    size_t vec = 0;
    for (int m = 0; m < p->n_mol; m++) {
        const nm_molecule& mol = p->mols[m];
        vec += (size_t)mol.n_store + 3 * (size_t)mol.n_blocks + 2 * (size_t)mol.n_molmon;
    }
    size_t words = vec * M + (size_t)(12 + 4 * p->n_seg) * M + 2 * (size_t)p->diis_m * p->iv + 4 * (size_t)p->iv;
    size_t bytes = 8 * words;
    if (!batched && precision == NM_FP32) bytes += bytes / 2;  // FP32 copies beside the FP64 ones
    return bytes + (1 << 16);
}

}  // namespace

struct Server {
    nm_server_options opt{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request*> queue;
    std::map<long long, Request*> all;
    long long next_id = 1;
    size_t in_use = 0;
    bool stop = false;
    std::vector<std::thread> workers;
    std::atomic<long long> launches{0};
    nm_stream* loop = nullptr;  // the 1-gradient streaming work loop (may be null)

    void worker(int wi);
    void run_batch(std::vector<Request*>& group, cudaStream_t st);
    void run_single(Request* r, cudaStream_t st);
};

void Server::run_batch(std::vector<Request*>& group, cudaStream_t st) {
    const int n = (int)group.size();
    std::vector<const nm_plan*> plans(n);
    for (int i = 0; i < n; i++) plans[i] = group[i]->plan;
    nm_ctx_options o{opt.precision, 0, opt.device, st};
    nm_batch* b = nullptr;
    int rc = nm_batch_create(plans.data(), n, &o, &b);
    if (rc) {
        for (auto* r : group) r->rc = rc;
        return;
    }
    std::vector<long long> off(n + 1);
    nm_batch_offsets(b, off.data());
    std::vector<double> x((size_t)off[n]);
    for (int i = 0; i < n; i++) std::memcpy(x.data() + off[i], group[i]->x.data(), sizeof(double) * group[i]->x.size());
    std::vector<int> its(n), status(n);
    std::vector<double> res(n);
    rc = nm_batch_solve_host(b, x.data(), its.data(), res.data(), status.data());
    for (int i = 0; i < n; i++) {
        Request* r = group[i];
        r->rc = rc;
        if (!rc) {
            std::memcpy(r->x.data(), x.data() + off[i], sizeof(double) * r->x.size());
            r->res.iterations = its[i];
            r->res.residual = res[i];
            r->res.status = status[i];
        }
    }
    launches += nm_batch_launch_count(b);
    nm_batch_destroy(b);
}

void Server::run_single(Request* r, cudaStream_t st) {
    // FP32 propagators where they are the faster path (3-D simple-cubic
    // linear chains); FP64 otherwise.  2-D contexts have FP32 propagators
    // too, but their per-step kernels are latency-bound and measured slower
    // in FP32 (row maxima per step, a DIIS restart at the handover).
    int prec = opt.precision;
    if (prec == NM_FP32 && !ctx3d_eligible(r->plan, nullptr)) prec = NM_FP64;
    nm_ctx_options o{prec, 0, opt.device, st};
    nm_ctx* c = nullptr;
    int rc = nm_ctx_create(r->plan, &o, &c);
    if (!rc) {
        // fewer launches per iteration where the caller asked for them; an
        // option that does not apply to this context leaves it as it was
        if (opt.context_sweeps & 1) nm_ctx_set_option(c, NM_OPT_SWEEP2D, 1);
        if (opt.context_sweeps & 2) nm_ctx_set_option(c, NM_OPT_CLUSTER3D, 1);
        if (opt.context_sweeps & 4) nm_ctx_set_option(c, NM_OPT_DEVICE_LOOP, 1);
        rc = nm_solve_host(c, r->x.data(), nullptr, &r->res);
        if (rc == NM_ERR_NOT_CONVERGED) rc = NM_OK;  // reported in res.status
        launches += nm_ctx_launch_count(c);
        nm_ctx_destroy(c);
    }
    r->rc = rc;
}

void Server::worker(int wi) {
    (void)wi;
    cudaSetDevice(opt.device);
    cudaStream_t st;
    cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    for (;;) {
        std::vector<Request*> group;
        size_t bytes = 0;
        {
            std::unique_lock<std::mutex> lk(mu);
            for (;;) {
                if (stop && queue.empty()) { cudaStreamDestroy(st); return; }
                if (!queue.empty()) {
                    Request* head = queue.front();
                    if (in_use + head->bytes <= opt.memory_budget) {
                        if (head->batched) {
                            // the head and the other waiting 1-gradient requests that fit
                            for (auto it = queue.begin(); it != queue.end() && (int)group.size() < opt.max_batch;) {
                                Request* r = *it;
                                if (r->batched && in_use + bytes + r->bytes <= opt.memory_budget) {
                                    group.push_back(r);
                                    bytes += r->bytes;
                                    it = queue.erase(it);
                                } else {
                                    ++it;
                                }
                            }
                        } else {
                            group.push_back(head);
                            bytes = head->bytes;
                            queue.pop_front();
                        }
                        in_use += bytes;
                        break;
                    }
                }
                cv_work.wait(lk);
            }
        }
        if (group.size() == 1 && !group[0]->batched) run_single(group[0], st);
        else run_batch(group, st);
        {
            std::lock_guard<std::mutex> lk(mu);
            auto now = clk::now();
            for (auto* r : group) { r->t_done = now; r->done = true; }
            in_use -= bytes;
        }
        cv_done.notify_all();
        cv_work.notify_all();
    }
}

}  // namespace nm

using nm::Server;

extern "C" {

int nm_server_create(const nm_server_options* opt, nm_server** out) {
    if (!opt || !out || opt->workers < 1 || opt->memory_budget == 0) {
        nm::set_error("nm_server_create: bad options");
        return NM_ERR_ARG;
    }
    cudaError_t e = cudaSetDevice(opt->device);
    if (e != cudaSuccess) { nm::set_error(cudaGetErrorString(e)); return NM_ERR_CUDA; }
    nm::nm_pool_setup(opt->device);
    Server* s = new Server();
    s->opt = *opt;
    if (s->opt.max_batch < 1) s->opt.max_batch = 1;
    if (opt->stream_slots >= 0) {
        // envelope of the loop: brushes, stars and other 1-gradient problems
        // of up to 512 layers, six segment types and 1024 stored propagators;
        // two CTAs per SM by default leave room for the context kernels of
        // 2-D and 3-D requests beside it
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, opt->device);
        nm_stream_options so{opt->device, 1024, 512, 6, 6, 4, 1024, 32, 12,
                             opt->stream_slots > 0 ? opt->stream_slots : 2 * sms, 0.2};
        if (int rc = nm_stream_create(&so, &s->loop)) { delete s; return rc; }
    }
    for (int i = 0; i < opt->workers; i++) s->workers.emplace_back(&Server::worker, s, i);
    *out = reinterpret_cast<nm_server*>(s);
    return NM_OK;
}

int nm_server_submit(nm_server* srv, const nm_plan* plan, const double* x_host, long long* request_id) {
    Server* s = reinterpret_cast<Server*>(srv);
    if (!s || !plan || !x_host || !request_id) { nm::set_error("nm_server_submit: bad argument"); return NM_ERR_ARG; }
    if (plan->search_mol >= 0 || plan->scan_mol >= 0) {
        nm::set_error("nm_server_submit: a search or scan runs on a device context (nm_ctx_search, nm_plan_scan_value)");
        return NM_ERR_INPUT;
    }
    auto* r = new nm::Request();
    r->plan = plan;
    r->x.assign(x_host, x_host + plan->iv);
    r->batched = plan->gradients == 1 && !plan->charged && plan->MX <= 512;
    for (int m = 0; m < plan->n_mol; m++)
        if (plan->mols[m].markov == 2) r->batched = false;  // Markov 2 chains take a device context
    if (plan->n_state > 0) r->batched = false;              // so do internal states
    r->bytes = nm::footprint(plan, r->batched, s->opt.precision);
    if (r->bytes > s->opt.memory_budget) {
        delete r;
        nm::set_error("nm_server_submit: request needs more device memory than the server's budget");
        return NM_ERR_NOMEM;
    }
    r->t_submit = nm::clk::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) { delete r; nm::set_error("nm_server_submit: server is shutting down"); return NM_ERR_ARG; }
        if (r->batched && s->loop) {
            long long t = -1;
            const int rc = nm_stream_submit(s->loop, plan, x_host, s->opt.precision, &t);
            if (rc == NM_OK) r->ticket = t;
            else if (rc != NM_ERR_INPUT && rc != NM_ERR_NOMEM) { delete r; return rc; }
        }
        r->id = s->next_id++;
        s->all[r->id] = r;
        if (r->ticket < 0) s->queue.push_back(r);
        *request_id = r->id;
    }
    if (r->ticket < 0) s->cv_work.notify_one();
    return NM_OK;
}

int nm_server_wait(nm_server* srv, long long request_id, double* x_host, nm_solve_result* res, double* seconds) {
    Server* s = reinterpret_cast<Server*>(srv);
    if (!s) { nm::set_error("nm_server_wait: bad argument"); return NM_ERR_ARG; }
    nm::Request* r = nullptr;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->all.find(request_id);
        if (it == s->all.end()) { nm::set_error("nm_server_wait: unknown request"); return NM_ERR_ARG; }
        r = it->second;
        s->all.erase(it);
        if (r->ticket < 0) s->cv_done.wait(lk, [&] { return r->done; });
    }
    if (r->ticket >= 0) {  // the streaming loop: its own wait and clock
        const int rc = nm_stream_wait(s->loop, r->ticket, x_host, res, seconds);
        delete r;
        return rc;
    }
    if (x_host) std::memcpy(x_host, r->x.data(), sizeof(double) * r->x.size());
    if (res) *res = r->res;
    if (seconds) *seconds = std::chrono::duration<double>(r->t_done - r->t_submit).count();
    int rc = r->rc;
    if (rc) nm::set_error("request failed with status " + std::to_string(rc));
    delete r;
    return rc;
}

long long nm_server_launch_count(nm_server* srv) {
    Server* s = reinterpret_cast<Server*>(srv);
    if (!s) return 0;
    return s->launches.load() + (s->loop ? nm_stream_launch_count(s->loop) : 0);
}

int nm_server_destroy(nm_server* srv) {
    Server* s = reinterpret_cast<Server*>(srv);
    if (!s) return NM_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto& t : s->workers) t.join();
    for (auto& kv : s->all) delete kv.second;
    if (s->loop) nm_stream_destroy(s->loop);
    delete s;
    return NM_OK;
}

}  // extern "C"
