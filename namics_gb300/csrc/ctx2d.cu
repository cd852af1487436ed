// Persistent 2-D sweeps for the generic context (FP64, linear chains), an
// option (NM_OPT_SWEEP2D, off by default).
//
// A 2-D step touches MX·MY sites (40 804 for a 200×200 lattice), about 8
// warps per SM, so a step launched on its own costs a launch plus a memory
// round trip, ~4.4 µs.  Measured on GB300 the sweep below is slower still
// (7.2 µs per step on that lattice): a release/acquire hand-off between
// neighbouring CTAs costs more than a kernel boundary, and the FP64 work of a
// step concentrates on fewer SMs.  Here one
// cooperative launch runs a whole sweep: CTA c owns rows x ∈ [x0, x1] and,
// per step, waits only for the CTAs that own the rows its stencil reads
// (x0-R .. x1+R; R = 1, or 2 when the halo composition of a charged system
// reads the flat arrays' wrap-around), computes its rows, and publishes the
// step in its progress flag.  The arithmetic is the per-step kernels'
// (`stencil_at`, `flat_prop_at`, the same fused composition), so results
// are bit-identical to the per-step path.
//
// Ordering: a CTA stores its rows, bar.sync, then one thread stores the
// step number with release semantics (cumulative over the writes the
// barrier ordered before it); in a waiting CTA one thread per neighbour
// loads that neighbour's flag with acquire semantics, bar.sync, and every
// thread reads the neighbours' rows with ld.global.cg (L2; L1 is not
// coherent across SMs).  The backward sweep ping-pongs two buffers: writing step j into a
// buffer that neighbours read at step j-1 is safe because step j begins by
// waiting for their step j-1.
//
// Every wait is bounded (2 s of %globaltimer, and a poll count): a CTA that
// gives up sets the context's status to NM_ERR_TIMEOUT and returns, and so
// do the others when they see it, so a solve fails loudly instead of
// hanging.  All CTAs are co-resident by the cooperative launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "ctx_internal.h"

using nmdev::Lat;

namespace nm {

namespace {

struct CgLoad {  // an array another CTA writes during the launch
    const double* p;
    __device__ __forceinline__ double operator()(int i) const { return __ldcg(p + i); }
};
struct CgBLoad {  // the same through set_bounds
    const double* p;
    Lat L;
    __device__ __forceinline__ double operator()(int i) const { return __ldcg(p + nmdev::bc_source(L, i)); }
};

__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

struct Sw2 {
    Lat L;
    int rows;          // rows per CTA
    int R;             // rows of neighbours a step reads beyond its own
    int n_store;
    const int* seg;    // [n_store] segment of stored index s
    const int* mm;     // [n_store] molecule-segment (rho slot) of s
    const double* deg; // [n_store] degeneracy of s's block
    const double* G1;  // [ns][M]
    double* Gf;        // [n_store][M]
    double* gb;        // [2][M]
    double* rho;       // [n_molmon][M]
    int* flags;        // [gridDim.x], -1 before the launch
    int* status;       // the context's device status
    int nh;            // halo composition on (charged systems)
};

__device__ __forceinline__ void publish(const Sw2& a, int step) {
    __syncthreads();
    if (threadIdx.x == 0) st_release(a.flags + blockIdx.x, step);
}

// wait until every CTA owning rows x0-R .. x1+R has published `step`; thread
// t polls the t-th of those CTAs, so the waits overlap
__device__ bool wait_for(const Sw2& a, int x0, int x1, int step) {
    const int lo = max(x0 - a.R, 1), hi = min(x1 + a.R, a.L.MX);
    const int c0 = (lo - 1) / a.rows, c1 = (hi - 1) / a.rows;
    const int c = c0 + (int)threadIdx.x;
    int good = 1;
    if (c <= c1 && c != (int)blockIdx.x) {
        const unsigned long long t0 = gtimer();
        long long polls = 0;
        while (ld_acquire(a.flags + c) < step) {
            if ((++polls & 63) == 0) {
                if (*(volatile int*)a.status == NM_ERR_TIMEOUT) { good = 0; break; }
                if (polls > (1LL << 26) || gtimer() - t0 > 2000000000ull) {
                    atomicCAS(a.status, 0, NM_ERR_TIMEOUT);
                    good = 0;
                    break;
                }
            }
        }
    }
    return __syncthreads_and(good) != 0;
}

__global__ void __launch_bounds__(256) k2_fwd(Sw2 a) {
    const Lat& L = a.L;
    const int M = L.M, MY = L.MY, JX = L.JX;
    const int x0 = 1 + (int)blockIdx.x * a.rows, x1 = min(L.MX, x0 + a.rows - 1);
    const int n = (x1 - x0 + 1) * MY;
    {
        const double* g1 = a.G1 + (size_t)a.seg[0] * M;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int s = (x0 + i / MY) * JX + i % MY + 1;
            a.Gf[s] = g1[s];
        }
    }
    publish(a, 0);
    for (int k = 1; k < a.n_store; k++) {
        if (!wait_for(a, x0, x1, k - 1)) return;
        const CgLoad in{a.Gf + (size_t)(k - 1) * M};
        double* out = a.Gf + (size_t)k * M;
        const double* g1 = a.G1 + (size_t)a.seg[k] * M;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int x = x0 + i / MY, y = i % MY + 1, s = x * JX + y;
            out[s] = nmdev::stencil_at(L, in, x, y, 0) * g1[s];
        }
        publish(a, k);
    }
}

__global__ void __launch_bounds__(256) k2_bwd(Sw2 a) {
    const Lat& L = a.L;
    const int M = L.M, MY = L.MY, JX = L.JX;
    const int x0 = 1 + (int)blockIdx.x * a.rows, x1 = min(L.MX, x0 + a.rows - 1);
    const int n = (x1 - x0 + 1) * MY;
    // halo sites of this CTA: the y-halos of its rows, and the x-halo rows
    // below the first and above the last CTA
    const bool lo_row = blockIdx.x == 0, hi_row = blockIdx.x == gridDim.x - 1;
    const int nhalo = a.nh ? 2 * (x1 - x0 + 1) + (lo_row ? JX : 0) + (hi_row ? JX : 0) : 0;
    const int top = a.n_store - 1;
    {
        // root of the sweep: Gb = G1, rho += d·Gf·G1 (the stored root end is
        // cleared in the reference, so the halo part is zero)
        const double* g1 = a.G1 + (size_t)a.seg[top] * M;
        const double* gf = a.Gf + (size_t)top * M;
        double* cur = a.gb + (size_t)(top & 1) * M;
        double* rho = a.rho + (size_t)a.mm[top] * M;
        const double d = a.deg[top];
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int s = (x0 + i / MY) * JX + i % MY + 1;
            const double v = g1[s];
            cur[s] = v;
            if (d == 1.0) rho[s] += gf[s] * v;
            else rho[s] += d * gf[s] * v;
        }
    }
    publish(a, 0);
    for (int j = 1; j <= top; j++) {
        const int sidx = top - j;
        if (!wait_for(a, x0, x1, j - 1)) return;
        const double* inp = a.gb + (size_t)((sidx + 1) & 1) * M;
        const CgLoad in{inp};
        double* out = a.gb + (size_t)(sidx & 1) * M;
        const double* g1 = a.G1 + (size_t)a.seg[sidx] * M;
        const double* gf = a.Gf + (size_t)sidx * M;
        double* rho = a.rho + (size_t)a.mm[sidx] * M;
        const double d = a.deg[sidx];
        for (int i = threadIdx.x; i < n + nhalo; i += blockDim.x) {
            if (i >= n) {
                int h, k = i - n;
                if (k < 2 * (x1 - x0 + 1)) h = (x0 + k / 2) * JX + ((k & 1) ? MY + 1 : 0);
                else {
                    k -= 2 * (x1 - x0 + 1);
                    if (lo_row && k < JX) h = k;
                    else h = (L.MX + 1) * JX + (lo_row ? k - JX : k);
                }
                const CgBLoad bl{inp, L};
                const double v = nmdev::flat_prop_at(L, bl, h) * g1[h];
                const double f = gf[nmdev::bc_source(L, h)];
                if (d == 1.0) rho[h] += f * v;
                else rho[h] += d * f * v;
                continue;
            }
            const int x = x0 + i / MY, y = i % MY + 1, s = x * JX + y;
            const double v = nmdev::stencil_at(L, in, x, y, 0) * g1[s];
            out[s] = v;
            if (d == 1.0) rho[s] += gf[s] * v;
            else rho[s] += d * gf[s] * v;
        }
        publish(a, j);
    }
}

}  // namespace

bool ctx2d_eligible(const nm_plan* p) {
    if (p->gradients != 2) return false;
    // the x halo rows must take their values from rows next to them
    if (p->bc[0] == NM_BC_PERIODIC || p->bc[3] == NM_BC_PERIODIC) return false;
    for (int m = 0; m < p->n_mol; m++) {
        const nm_molecule& mol = p->mols[m];
        for (int b = 0; b < mol.n_blocks; b++) {
            const nm_block& B = mol.blocks[b];
            if (B.n_child > 1 || (B.n_child == 1 && mol.blocks[mol.child_index[B.child0]].mult != 1)) return false;
        }
    }
    return true;
}

int ctx2d_init(Ctx& C) {
    const nm_plan* p = C.plan;
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return NM_ERR_CUDA;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop || sms <= 0) return NM_OK;  // stays on the per-step kernels
    int a1 = 0, a2 = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a1, k2_fwd, 256, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a2, k2_bwd, 256, 0);
    per_sm = std::min(std::min(a1, a2), 2);
    if (per_sm < 1) return NM_OK;
    const int MX = p->MX;
    C.sw_rows = (MX + sms * per_sm - 1) / (sms * per_sm);
    // a charged system's halo composition reads two rows out: with two rows
    // per CTA those still belong to the adjacent CTAs only
    if (C.nh && C.sw_rows < 2) C.sw_rows = 2;
    C.sw_ctas = (MX + C.sw_rows - 1) / C.sw_rows;
    // per molecule: segment, rho slot and degeneracy of every stored s
    C.sw_tabs.resize(p->n_mol);
    for (int m = 0; m < p->n_mol; m++) {
        const nm_molecule& mol = p->mols[m];
        std::vector<int> seg(mol.n_store), mm(mol.n_store);
        std::vector<double> deg(mol.n_store);
        for (int b = 0; b < mol.n_blocks; b++) {
            const nm_block& B = mol.blocks[b];
            for (int k = 0; k < B.length; k++) {
                seg[B.s0 + k] = B.seg; mm[B.s0 + k] = B.molmon; deg[B.s0 + k] = B.degeneracy;
            }
        }
        auto& T = C.sw_tabs[m];
        if (cudaMallocAsync((void**)&T.seg, sizeof(int) * mol.n_store, C.stream) != cudaSuccess ||
            cudaMallocAsync((void**)&T.mm, sizeof(int) * mol.n_store, C.stream) != cudaSuccess ||
            cudaMallocAsync((void**)&T.deg, sizeof(double) * mol.n_store, C.stream) != cudaSuccess) {
            set_error("cudaMallocAsync (2-D sweep tables)");
            return NM_ERR_NOMEM;
        }
        cudaMemcpyAsync(T.seg, seg.data(), sizeof(int) * mol.n_store, cudaMemcpyHostToDevice, C.stream);
        cudaMemcpyAsync(T.mm, mm.data(), sizeof(int) * mol.n_store, cudaMemcpyHostToDevice, C.stream);
        cudaMemcpyAsync(T.deg, deg.data(), sizeof(double) * mol.n_store, cudaMemcpyHostToDevice, C.stream);
        // pageable sources: staged before the calls return
    }
    if (cudaMallocAsync((void**)&C.d_flags, sizeof(int) * C.sw_ctas, C.stream) != cudaSuccess) {
        set_error("cudaMallocAsync (2-D sweep flags)");
        return NM_ERR_NOMEM;
    }
    C.use2d = true;
    return NM_OK;
}

static int coop_launch(Ctx& C, void (*kern)(Sw2), Sw2& a) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(C.sw_ctas);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = C.stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, kern, a);
    if (e != cudaSuccess) { set_error(std::string("2-D sweep launch: ") + cudaGetErrorString(e)); return NM_ERR_CUDA; }
    C.launches++;
    return NM_OK;
}

// One molecule through the persistent sweeps: forward (every Gf stored),
// G(N), backward fused with the composition.
int ctx2d_molecule_pass(Ctx& C, int m) {
    const nm_plan* p = C.plan;
    const nm_molecule& mol = p->mols[m];
    MolDev& D = C.mols[m];
    const size_t M = p->M;
    Sw2 a;
    a.L = C.lat;
    a.rows = C.sw_rows;
    a.R = C.nh ? 2 : 1;
    a.n_store = mol.n_store;
    a.seg = C.sw_tabs[m].seg; a.mm = C.sw_tabs[m].mm; a.deg = C.sw_tabs[m].deg;
    a.G1 = C.d_G1; a.Gf = D.Gf; a.gb = C.d_gb; a.rho = D.rho;
    a.flags = C.d_flags; a.status = C.d_status; a.nh = C.nh;
    if (cudaMemsetAsync(D.rho, 0, sizeof(double) * M * mol.n_molmon, C.stream) != cudaSuccess ||
        cudaMemsetAsync(C.d_flags, 0xff, sizeof(int) * C.sw_ctas, C.stream) != cudaSuccess) {
        set_error("cudaMemsetAsync (2-D sweep)");
        return NM_ERR_CUDA;
    }
    int rc = coop_launch(C, k2_fwd, a);
    if (rc) return rc;
    C.wsum(D.Gf + (size_t)(mol.n_store - 1) * M, C.d_sc + 5 * m);
    if (cudaMemsetAsync(C.d_flags, 0xff, sizeof(int) * C.sw_ctas, C.stream) != cudaSuccess) {
        set_error("cudaMemsetAsync (2-D sweep)");
        return NM_ERR_CUDA;
    }
    return coop_launch(C, k2_bwd, a);
}

}  // namespace nm
