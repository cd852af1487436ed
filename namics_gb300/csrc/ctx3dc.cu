// Cluster-resident 3-D sweeps for small FP32 boxes (a 64³ melt): one
// thread-block cluster runs a whole forward sweep, or a whole backward sweep
// fused with the composition, in one launch.
//
// On a 64³ box one propagator is 1 MB of FP32, and a step launched on its own
// covers the whole GPU for ~5 µs, almost all of it launch and ramp-up: a
// solve's ~80 step launches per residual then occupy every SM, and several
// such solves running side by side (a served request stream) queue behind
// one another.  Here a cluster of n CTAs (one per SM, n ≤ 16) owns the box:
// CTA r holds the x-planes x0..x1 of the current and the next propagator
// in its shared memory, plus one halo plane on each side, in the global
// layout of a plane ((MY+2)·(MZ+2), y and z halo slots left zero and read
// through the set_bounds map).  A step reads the current buffer, writes the
// next one and the stored Gf(s) (global, for the backward sweep), and pushes
// each plane that another CTA's halo needs into that CTA's buffer through
// distributed shared memory (st.shared::cluster).  One cluster barrier per
// step (arrive.release / wait.acquire) orders those writes before the next
// step's reads; the two buffers alternate, so a step never writes what a
// slower CTA may still be reading.
//
// FP32 block floating point as in the per-step kernels: every vector has one
// power-of-two exponent.  Each CTA publishes the maximum of its part of a
// vector in its shared memory; after the barrier every warp reads the n
// maxima of the cluster and takes their maximum (exact), so the scale of a
// step is the per-step kernels' (k3_prop) scale.  A step computes
// ((x pair) + (y pair)) + (z pair) of the input, times f, times G1, and the
// composition update is the same function (c3_comp): the results are
// bit-identical to the per-step path, whatever the cluster size.
//
// There are no spin-waits: the cluster barrier is a hardware barrier that
// every thread of every CTA reaches the same number of times (the step loop
// has the same trip count in all of them, and no thread leaves early).
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "ctx3d_common.cuh"
#include "ctx_internal.h"

namespace nm {

namespace {

constexpr int C3C_THREADS = 1024;
constexpr int C3C_MAXCL = 16;      // CTAs per cluster at most (16 needs the non-portable opt-in)
constexpr int C3C_MAXPUSH = 4;     // halo planes a CTA feeds per step
constexpr int C3C_PMAX = 4;        // x-planes per CTA at most
constexpr int C3C_CMAX = 4;        // (y, z) columns per thread at most: MY·MZ <= 4096

struct C3C {
    L3 L;
    const float* G1;   // [ns][M] FP32 G1
    float* Gf;         // [n_store][M] stored forward propagators
    int* E;            // [2·n_store] exponents: forward s at s, backward s at n_store + s
    const int* seg;    // [n_store] segment type of stored index s
    const int* mm;     // [n_store] composition slot (molecule segment) of s
    const float* deg;  // [n_store] degeneracy of s's block
    float* rhi;        // [n_molmon][M] composition, Kahan sum
    float* rlo;        // [n_molmon][M] its compensation
    int n_store, sroot, P;  // P: planes per CTA
};

__device__ __forceinline__ unsigned cl_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cl_size() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
// every thread of the cluster; shared-memory writes before it (this CTA's and
// remote ones) are visible to every thread after it
__device__ __forceinline__ void cl_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// the address of this CTA's shared variable p in CTA `rank` of the cluster
__device__ __forceinline__ unsigned cl_addr(const void* p, unsigned rank) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
__device__ __forceinline__ void cl_st(unsigned addr, float v) {
    asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}
__device__ __forceinline__ float cl_ld(unsigned addr) {
    float v;
    asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(addr) : "memory");
    return v;
}

// Per-CTA setup shared by both sweeps: the planes it owns and the halo
// planes it feeds.  push[k] = {target CTA, target local plane, own local
// plane}; local plane 0 is the lower halo, 1..nown the owned planes,
// nown+1 the upper halo.
struct C3Own { int x0, nown, npush; int push[C3C_MAXPUSH][3]; };

__device__ void c3c_owner(const C3C& a, C3Own& o) {
    const L3& L = a.L;
    const int r = (int)cl_rank(), n = (int)cl_size();
    o.x0 = r * a.P + 1;
    o.nown = max(0, min(o.x0 + a.P - 1, L.MX) - o.x0 + 1);
    o.npush = 0;
    for (int q = 0; q < n; q++) {
        const int qx0 = q * a.P + 1, qx1 = min(qx0 + a.P - 1, L.MX), qn = qx1 - qx0 + 1;
        if (qn <= 0) continue;
        const int lo = c3_map(qx0 - 1, L.MX, L.b1x, L.bmx), hi = c3_map(qx1 + 1, L.MX, L.b1x, L.bmx);
        if (lo >= o.x0 && lo < o.x0 + o.nown && o.npush < C3C_MAXPUSH) {
            o.push[o.npush][0] = q; o.push[o.npush][1] = 0; o.push[o.npush][2] = lo - o.x0 + 1; o.npush++;
        }
        if (hi >= o.x0 && hi < o.x0 + o.nown && o.npush < C3C_MAXPUSH) {
            o.push[o.npush][0] = q; o.push[o.npush][1] = qn + 1; o.push[o.npush][2] = hi - o.x0 + 1; o.npush++;
        }
    }
}

// One sweep.  BWD = false: forward, Gf(s) for s = 0 .. n_store-1 (s = 0
// starts the chain from G1).  BWD = true: backward from the root end, the
// composition ρ += d·Gf(s)·Gb(s) at every s.
template <bool BWD>
__global__ void __launch_bounds__(C3C_THREADS, 1) k3c_sweep(C3C a) {
    extern __shared__ __align__(16) float c3c_buf[];  // [2][P+2][PS]
    __shared__ float s_mx[2];                         // this CTA's maximum of the vector in buffer 0 / 1
    __shared__ float s_wm[C3C_THREADS / 32];
    const L3 L = a.L;
    const int PS = L.JX, JY = L.JY;
    const size_t M = (size_t)(L.MX + 2) * PS;
    const int BUF = (a.P + 2) * PS;
    __shared__ C3Own s_own;
    const int tid = threadIdx.x, ncl = (int)cl_size();
    if (tid == 0) c3c_owner(a, s_own);
    for (int i = tid; i < 2 * BUF; i += C3C_THREADS) c3c_buf[i] = 0.f;  // y/z halo slots and 'surface' planes stay 0
    __syncthreads();
    const int x0 = s_own.x0, nown = s_own.nown, npush = s_own.npush;
    // remote base address of each push's target plane, per buffer
    __shared__ unsigned s_rbase[C3C_MAXPUSH][2];
    if (tid < 2 * npush) {
        const int k = tid >> 1, b = tid & 1;
        s_rbase[k][b] = cl_addr(c3c_buf + b * BUF + s_own.push[k][1] * PS, s_own.push[k][0]);
    }
    __syncthreads();
    const int cols = L.MY * L.MZ;
    // this thread's (y, z) columns c = tid + k·1024, packed y << 16 | z (0: none)
    int cyz[C3C_CMAX];
#pragma unroll
    for (int k = 0; k < C3C_CMAX; k++) {
        const int c = tid + k * C3C_THREADS;
        cyz[k] = c < cols ? ((c / L.MZ + 1) << 16) | (c % L.MZ + 1) : 0;
    }
    const int Eroot = BWD ? a.E[a.sroot] : 0;
    int Ecur = 0;
    cl_sync();  // every buffer of the cluster is zero before the first push
    for (int j = 0; j < a.n_store; j++) {
        const int s = BWD ? a.n_store - 1 - j : j;
        const int par = j & 1;  // this step's output buffer
        float* out = c3c_buf + par * BUF;
        const float* in = c3c_buf + (par ^ 1) * BUF;
        const bool start = j == 0;
        int e = 0;
        float f = 0.f;
        if (!start) {  // the cluster's maximum of the input vector
            const int lane = tid & 31;
            float mx = 0.f;
            if (lane < ncl) mx = cl_ld(cl_addr(&s_mx[par ^ 1], lane));
            for (int sh = 16; sh > 0; sh >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, sh));
            f = c3_scale(mx, e);
        }
        const int Eout = start ? 0 : Ecur + e;
        const float* __restrict__ g1 = a.G1 + (size_t)a.seg[s] * M;
        float* __restrict__ gf = a.Gf + (size_t)s * M;
        const int Es = BWD ? a.E[s] + Eout - Eroot : 0;
        const float d = BWD ? a.deg[s] : 0.f;
        float* __restrict__ rh = BWD ? a.rhi + (size_t)a.mm[s] * M : nullptr;
        float* __restrict__ rl = BWD ? a.rlo + (size_t)a.mm[s] * M : nullptr;
        float vmax = 0.f;
        // columns in batches: every global load of a batch is issued before
        // its first use, so a step waits for one L2 round trip per batch
        constexpr int HB = BWD ? 2 : C3C_CMAX;
#pragma unroll
        for (int h = 0; h < C3C_CMAX; h += HB) {
            float g1v[HB][C3C_PMAX], gfv[HB][C3C_PMAX], rhv[HB][C3C_PMAX], rlv[HB][C3C_PMAX];
#pragma unroll
            for (int kk = 0; kk < HB; kk++) {
                const int y = cyz[h + kk] >> 16, yz = y * JY + (cyz[h + kk] & 0xffff);
#pragma unroll
                for (int i = 0; i < C3C_PMAX; i++) {
                    const bool ok = y > 0 && i < nown;
                    const size_t gs = (size_t)(x0 + i) * PS + yz;
                    g1v[kk][i] = ok ? g1[gs] : 0.f;
                    if (BWD) {
                        gfv[kk][i] = ok ? gf[gs] : 0.f;
                        rhv[kk][i] = ok ? rh[gs] : 0.f;
                        rlv[kk][i] = ok ? rl[gs] : 0.f;
                    }
                }
            }
#pragma unroll
            for (int kk = 0; kk < HB; kk++) {
                const int y = cyz[h + kk] >> 16, z = cyz[h + kk] & 0xffff;
                if (y == 0) continue;
                const int yz = y * JY + z;
                const int ym = c3_map(y - 1, L.MY, L.b1y, L.bmy) * JY + z, yp = c3_map(y + 1, L.MY, L.b1y, L.bmy) * JY + z;
                const int zm = y * JY + c3_map(z - 1, L.MZ, L.b1z, L.bmz), zp = y * JY + c3_map(z + 1, L.MZ, L.b1z, L.bmz);
#pragma unroll
                for (int i = 0; i < C3C_PMAX; i++) {
                    if (i >= nown) break;
                    const int lo = (i + 1) * PS;
                    const size_t gs = (size_t)(x0 + i) * PS + yz;
                    float v;
                    if (start) {
                        v = g1v[kk][i];
                    } else {
                        // summation order of LGrad3::propagate's simple-cubic branch: x pair, y pair, z pair
                        const float s6 = ((in[lo - PS + yz] + in[lo + PS + yz]) + (in[lo + ym] + in[lo + yp])) +
                                         (in[lo + zm] + in[lo + zp]);
                        v = s6 * f * g1v[kk][i];
                    }
                    out[lo + yz] = v;
                    if (i == 0 || i == nown - 1)  // a boundary plane: into the halos that read it
                        for (int k = 0; k < npush; k++)
                            if (s_own.push[k][2] == i + 1) cl_st(s_rbase[k][par] + 4u * (unsigned)yz, v);
                    if (BWD) {
                        c3_comp(gfv[kk][i], v, Es, d, &rhv[kk][i], &rlv[kk][i]);
                        rh[gs] = rhv[kk][i];
                        rl[gs] = rlv[kk][i];
                    } else {
                        gf[gs] = v;
                    }
                    vmax = fmaxf(vmax, v);
                }
            }
        }
        for (int sh = 16; sh > 0; sh >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, sh));
        if ((tid & 31) == 0) s_wm[tid >> 5] = vmax;
        __syncthreads();
        if (tid == 0) {
            float m = 0.f;
            for (int w = 0; w < C3C_THREADS / 32; w++) m = fmaxf(m, s_wm[w]);
            s_mx[par] = m;
            if (cl_rank() == 0) a.E[BWD ? a.n_store + s : s] = Eout;
        }
        Ecur = Eout;
        cl_sync();
    }
}

// The sweeps' shared-memory limit (the device's opt-in maximum less room for
// the static variables) and the non-portable cluster sizes, set once per
// device under a lock: contexts of different shapes only differ in the
// dynamic size they launch with.
bool c3c_attrs(int dev, int smem_max) {
    static std::mutex mu;
    static int done[64] = {};
    std::lock_guard<std::mutex> lk(mu);
    if (dev < 0 || dev >= 64) return false;
    if (done[dev]) return done[dev] > 0;
    bool ok = true;
    for (auto k : {k3c_sweep<false>, k3c_sweep<true>})
        ok = ok && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max - 1024) == cudaSuccess &&
             cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
    cudaGetLastError();
    done[dev] = ok ? 1 : -1;
    return ok;
}

}  // namespace

// Pick the cluster for a context on the 3-D FP32 path, or leave it off
// (C.c3c_ctas = 0): linear chains whose blocks follow one another in the
// stored order, every propagator stored, and two buffers of a CTA's planes
// plus halos within a CTA's shared memory for some co-resident cluster size.
int ctx3dc_init(Ctx& C) {
    C.c3c_ctas = 0;
    const nm_plan* p = C.plan;
    if (!C.use3d || !C.fp32) return NM_OK;
    for (int m = 0; m < p->n_mol; m++) {
        const nm_molecule& mol = p->mols[m];
        for (int b = 0; b < mol.n_blocks; b++) {
            const nm_block& B = mol.blocks[b];
            if (b == 0 ? (B.n_child != 0 || B.s0 != 0)
                       : (B.n_child != 1 || mol.child_index[B.child0] != b - 1 ||
                          B.s0 != mol.blocks[b - 1].s0 + mol.blocks[b - 1].length))
                return NM_OK;
        }
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return NM_OK;
    int cl = 0, smem_max = 0;
    cudaDeviceGetAttribute(&cl, cudaDevAttrClusterLaunch, dev);
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (!cl) return NM_OK;
    if (p->MY * p->MZ > C3C_CMAX * C3C_THREADS || p->MZ >= (1 << 16)) return NM_OK;
    if (!c3c_attrs(dev, smem_max)) return NM_OK;
    const size_t PS = (size_t)(p->MY + 2) * (p->MZ + 2);
    for (int want : {C3C_MAXCL, 8, 4, 2, 1}) {
        const int P = (p->MX + want - 1) / want, n = (p->MX + P - 1) / P;
        const size_t smem = sizeof(float) * 2 * (P + 2) * PS;
        if (smem + 1024 > (size_t)smem_max || P > C3C_PMAX) break;  // fewer CTAs only need more
        bool ok = true;
        for (auto k : {k3c_sweep<false>, k3c_sweep<true>}) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(n);
            cfg.blockDim = dim3(C3C_THREADS);
            cfg.dynamicSmemBytes = smem;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = n;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int clusters = 0;
            if (cudaOccupancyMaxActiveClusters(&clusters, k, &cfg) != cudaSuccess || clusters < 1) ok = false;
        }
        cudaGetLastError();  // a refused size is not an error of the context
        if (!ok) continue;
        C.c3c_ctas = n;
        C.c3c_planes = P;
        C.c3c_smem = smem;
        break;
    }
    if (!C.c3c_ctas) return NM_OK;
    // per molecule: segment type, composition slot and degeneracy of every stored s
    C.c3c_tabs.resize(p->n_mol);
    for (int m = 0; m < p->n_mol; m++) {
        const nm_molecule& mol = p->mols[m];
        std::vector<int> seg(mol.n_store), mm(mol.n_store);
        std::vector<float> deg(mol.n_store);
        for (int b = 0; b < mol.n_blocks; b++) {
            const nm_block& B = mol.blocks[b];
            for (int k = 0; k < B.length; k++) {
                seg[B.s0 + k] = B.seg;
                mm[B.s0 + k] = B.molmon;
                deg[B.s0 + k] = (float)B.degeneracy;
            }
        }
        auto& T = C.c3c_tabs[m];
        if (cudaMallocAsync((void**)&T.seg, sizeof(int) * mol.n_store, C.stream) != cudaSuccess ||
            cudaMallocAsync((void**)&T.mm, sizeof(int) * mol.n_store, C.stream) != cudaSuccess ||
            cudaMallocAsync((void**)&T.deg, sizeof(float) * mol.n_store, C.stream) != cudaSuccess) {
            set_error("cudaMallocAsync (3-D cluster sweep tables)");
            return NM_ERR_NOMEM;
        }
        cudaMemcpyAsync(T.seg, seg.data(), sizeof(int) * mol.n_store, cudaMemcpyHostToDevice, C.stream);
        cudaMemcpyAsync(T.mm, mm.data(), sizeof(int) * mol.n_store, cudaMemcpyHostToDevice, C.stream);
        cudaMemcpyAsync(T.deg, deg.data(), sizeof(float) * mol.n_store, cudaMemcpyHostToDevice, C.stream);
        // pageable sources: staged before the calls return
    }
    C.c3c_on = false;  // selected by NM_OPT_CLUSTER3D or the autotuner
    return NM_OK;
}

void ctx3dc_free(Ctx& C) {
    for (auto& T : C.c3c_tabs) {
        if (T.seg) cudaFreeAsync(T.seg, C.stream);
        if (T.mm) cudaFreeAsync(T.mm, C.stream);
        if (T.deg) cudaFreeAsync(T.deg, C.stream);
    }
    C.c3c_tabs.clear();
}

// The forward (bwd = false) or backward sweep of molecule m through the
// cluster kernel, into the molecule's FP32 buffers.
int ctx3dc_sweep(Ctx& C, int m, bool bwd, int sroot) {
    const nm_plan* p = C.plan;
    const nm_molecule& mol = p->mols[m];
    MolDev& D = C.mols[m];
    const size_t M = p->M;
    C3C a;
    a.L = C.l3;
    a.G1 = C.d_G1f;
    a.Gf = D.Gf32;
    a.E = C.d_E;
    a.seg = C.c3c_tabs[m].seg;
    a.mm = C.c3c_tabs[m].mm;
    a.deg = C.c3c_tabs[m].deg;
    a.rhi = D.rho32;
    a.rlo = D.rho32 + (size_t)mol.n_molmon * M;
    a.n_store = mol.n_store;
    a.sroot = sroot;
    a.P = C.c3c_planes;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(C.c3c_ctas);
    cfg.blockDim = dim3(C3C_THREADS);
    cfg.dynamicSmemBytes = C.c3c_smem;
    cfg.stream = C.stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C.c3c_ctas;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaError_t e = bwd ? cudaLaunchKernelEx(&cfg, k3c_sweep<true>, a) : cudaLaunchKernelEx(&cfg, k3c_sweep<false>, a);
    if (e != cudaSuccess) {
        set_error(std::string("3-D cluster sweep launch: ") + cudaGetErrorString(e));
        return NM_ERR_CUDA;
    }
    C.launches++;
    return NM_OK;
}

}  // namespace nm
