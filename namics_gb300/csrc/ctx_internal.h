// Device context internals shared by ctx.cu and the C-ABI entry points.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/namics_gb300.h"
#include "device_common.cuh"
#include "plan_internal.h"

#define NM_MAX_SEG 16
#define NM_MAX_MOL 16
#define NM_MAX_MM 32
#define NM_MAX_DIIS 32

namespace nm {

// Solve A c = 1 for symmetric A (n×n row-major, n ≤ NM_MAX_DIIS) by the
// pseudo-inverse c = Q·diag(1/λ)·Qᵀ·1 from a cyclic Jacobi eigenvalue
// decomposition, FP64.  This is the solve the reference makes with its SVD
// (SFNewton::Ax, sfnewton.cpp:793-835): near convergence A ≈ 1e-9·(all
// ones) is numerically singular, and the pseudo-inverse stays finite there
// because the eigenvectors of the rounding-noise eigenvalues are nearly
// orthogonal to the ones vector, where an elimination can divide by a zero
// pivot.
__host__ __device__ inline void nm_pinv_solve(const double* Ain, double* c, int n) {
    if (n == 1) { c[0] = 1.0; return; }
    double a[NM_MAX_DIIS * NM_MAX_DIIS], q[NM_MAX_DIIS * NM_MAX_DIIS];
    for (int i = 0; i < n * n; i++) a[i] = Ain[i];
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) q[i * n + j] = i == j ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 60; sweep++) {
        double off = 0, dg = 0;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                const double v = a[i * n + j] * a[i * n + j];
                if (i == j) dg += v; else off += v;
            }
        if (off == 0 || off <= 1e-30 * dg) break;
        for (int p = 0; p < n - 1; p++)
            for (int r = p + 1; r < n; r++) {
                const double apr = a[p * n + r];
                if (apr == 0) continue;
                // rotation that zeroes a[p][r]: tan of the angle, smaller root
                const double th = (a[r * n + r] - a[p * n + p]) / (2 * apr);
                const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1));
                const double cs = 1 / sqrt(t * t + 1), sn = t * cs;
                for (int k = 0; k < n; k++) {  // columns p, r
                    const double u = a[k * n + p], v = a[k * n + r];
                    a[k * n + p] = cs * u - sn * v;
                    a[k * n + r] = sn * u + cs * v;
                }
                for (int k = 0; k < n; k++) {  // rows p, r
                    const double u = a[p * n + k], v = a[r * n + k];
                    a[p * n + k] = cs * u - sn * v;
                    a[r * n + k] = sn * u + cs * v;
                }
                for (int k = 0; k < n; k++) {  // eigenvectors
                    const double u = q[k * n + p], v = q[k * n + r];
                    q[k * n + p] = cs * u - sn * v;
                    q[k * n + r] = sn * u + cs * v;
                }
            }
    }
    for (int i = 0; i < n; i++) c[i] = 0;
    for (int j = 0; j < n; j++) {
        double proj = 0;  // (Qᵀ·1)_j
        for (int k = 0; k < n; k++) proj += q[k * n + j];
        const double w = proj / a[j * n + j];
        for (int i = 0; i < n; i++) c[i] += q[i * n + j] * w;
    }
}

struct MolScal { int freedom, pinned; double n_in, theta_in, phibulk_in, N, charge; };
// Internal states (plans with n_state > 0): state j belongs to segment
// seg[j], takes iteration block it[j] and has bulk fraction ab[j].  The
// interaction species are the segments (those without states take part)
// followed by the states: species n_seg + j is state j.
struct StArgs {
    int n;
    int seg[NM_MAX_SEG], it[NM_MAX_SEG];
    double ab[NM_MAX_SEG];
};
struct NormArgs {
    int n_mol, solvent, ns;
    int neutralizer;  // molecule index (charged systems) or -1
    MolScal mol[NM_MAX_MOL];
    int n_mm;
    int mm_mol[NM_MAX_MM], mm_seg[NM_MAX_MM];
    double mm_frac[NM_MAX_MM];
    StArgs st;        // states: φ_bulk,j = φ_bulk(seg)·α_bulk,j after the segments'
};
struct PhiArgs {
    int ns, n_mm, n_mol;
    int mm_mol[NM_MAX_MM], mm_seg[NM_MAX_MM];
    const double* mm_rho[NM_MAX_MM];
    StArgs st;                 // states: φ_j = α_j·φ(seg) into species rows
    const double* ast;         // α of each state [n*M]
};
// the residual over interaction species: ns = species count, sp_on[k] = 0
// for a segment with states (its states stand in for it), it_seg[i] = the
// species of block i's representative, chi between species
struct ResArgs {
    int ns, nit;
    int it_seg[NM_MAX_SEG];
    int sp_on[NM_MAX_SEG];
    double chi[NM_MAX_SEG * NM_MAX_SEG];
};

// Charged systems: per-segment relative permittivity and per-species
// valence (segments, then states; 0 for a segment with states), for the
// u += -ε·EE + v·ψ terms of PutU (system.cpp:2001-2030) and the charge
// density.
struct ChgArgs {
    int on, nsp;
    double eps[NM_MAX_SEG], val[NM_MAX_SEG];
};

// Constants of the electrostatics (namics.cpp:44-49 and the lattice's
// UpdateEE / UpdatePsi prefactors), evaluated on the host in the reference's
// operation order.
struct ElecConst {
    double pf;      // UpdateEE prefactor, geometry factors included
    double C;       // UpdatePsi prefactor, geometry factors included
    double offset;  // offset_first_layer
    const double* Lv;  // site volume L (device)
};

struct MolDev {
    double* Gf = nullptr;   // forward propagators [n_store*M]
    float* Gf32 = nullptr;  // FP32 forward propagators [n_store*M] (3-D FP32 path)
    float* rho32 = nullptr; // FP32 composition, Kahan sum and compensation [2*n_molmon*M]
    double* rho = nullptr;  // Σ d·Gf·Gb per molecule segment type [n_molmon*M]
    double* Pc = nullptr;   // P(G_end)·KSAM of each child block [n_blocks*M]
    double* Q = nullptr;    // backward start of each child block [n_blocks*M]
    // checkpointed storage (3-D path, Ctx::ck_stride > 1): slot[s] = the
    // stored vector of segment s or -1; n_slots stored vectors, then k-1
    // vectors of the backward sweep's recompute buffer, then 2 vectors of
    // the forward sweep's running propagator
    std::vector<int> slot;
    int n_slots = 0;
};

nmdev::Lat make_lat(const nm_plan* p);

// Set while the bodies of the device-resident solve loop are captured: the
// kernel edges inside a conditional node's body are plain stream-order
// edges, so launches there drop the programmatic-serialisation attribute
// (pdl_begin is then a no-op).
extern thread_local bool g_plain_launch;

// launch with programmatic stream serialisation (the kernel calls pdl_begin
// before it touches memory); also recorded that way in a captured graph
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = g_plain_launch ? 0 : 1;
    return cudaLaunchKernelEx(&cfg, k, args...);
}

// 3-D lattice for the dedicated simple-cubic kernels (ctx3d.cu)
struct L3 {
    int MX, MY, MZ, JX, JY;
    int b1x, bmx, b1y, bmy, b1z, bmz;  // halo source layer per axis side
};
struct Ctx;
void nm_pool_setup(int dev);  // keep freed stream-ordered memory in the device's pool
L3 make_l3(const nm_plan* p);
bool ctx3d_eligible(const nm_plan* p, std::string* why);
int ctx3d_molecule_pass(Ctx& C, int m, bool fp32);
int ctx3d_set_tile(Ctx& C, int tile);  // choose the 3-D step kernel (0: gather; R·100+P: a tile)
// cluster-resident FP32 sweeps for small 3-D boxes (ctx3dc.cu)
struct C3cTab { int* seg = nullptr; int* mm = nullptr; float* deg = nullptr; };
int ctx3dc_init(Ctx& C);                            // pick a cluster size, or none
void ctx3dc_free(Ctx& C);
int ctx3dc_sweep(Ctx& C, int m, bool bwd, int sroot);  // one sweep of molecule m
// Markov 2 chains, 1-gradient simple cubic (ctx_markov2.cu)
int ctx_m2_init(Ctx& C);
void ctx_m2_free(Ctx& C);
int ctx_m2_molecule_pass(Ctx& C, int m);
// the device-resident solve loop (ctxloop.cu)
int ctx_loop_solve(Ctx& C, double* x, nm_solve_result* res, int max_iter);
void ctx_loop_drop(Ctx& C);  // the captured loop used kernels or values that changed
// persistent 2-D sweeps (ctx2d.cu)
bool ctx2d_eligible(const nm_plan* p);
int ctx2d_init(Ctx& C);
int ctx2d_molecule_pass(Ctx& C, int m);
struct SweepTab { int* seg = nullptr; int* mm = nullptr; double* deg = nullptr; };
// FP32 propagators on 2-gradient lattices, one exponent per row (ctx2d32.cu)
bool ctx2d32_eligible(const nm_plan* p, std::string* why);
int ctx2d32_init(Ctx& C);
int ctx2d32_molecule_pass(Ctx& C, int m);

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
    double *d_xR = nullptr, *d_xx0 = nullptr, *d_g = nullptr, *d_x = nullptr,
           *d_Ci = nullptr, *d_gram_partial = nullptr;
    std::vector<MolDev> mols;
    // 3-D simple-cubic path (ctx3d.cu) and its FP32 propagators
    bool use3d = false;       // dedicated 3-D kernels for every molecule
    int ck_stride = 0;        // > 1: every k-th forward propagator stored (3-D path)
    int c3_rows = 4;          // rows along y per block of the 3-D gather step kernels (2, 4, 8)
    int c3_tile = 0;          // 3-D 2.5-D tile steps: rows × 100 + planes (204, 208, 404, 408); 0: gather
    std::vector<size_t> gf_vectors;  // per molecule: propagator vectors allocated (3-D path)
    // FP32 sweeps of small boxes in one thread-block cluster (ctx3dc.cu):
    // c3c_ctas CTAs of c3c_planes x-planes each, when eligible; c3c_on
    // selects them (NM_OPT_CLUSTER3D) while every propagator is stored
    int c3c_ctas = 0, c3c_planes = 0;
    size_t c3c_smem = 0;
    bool c3c_on = false;
    std::vector<C3cTab> c3c_tabs;
    int set_ck_stride(int k); // a stride that fits the allocation (NM_ERR_ARG otherwise)
    bool fp32 = false;        // context created with NM_FP32 propagators
    bool phase32 = false;     // the current residual uses FP32 propagators
    double sw_floor = 0;      // FP32 accuracy floor of ‖g‖ (switch to FP64 near it)
    L3 l3{};
    float *d_G1f = nullptr, *d_gb32 = nullptr;
    unsigned* d_maxbits = nullptr;  // per stored vector: 32 slots with bits of its maximum
    int* d_E = nullptr;             // per stored vector: power-of-two exponent
    // the residual's launches captured once per (x, g, precision) and replayed
    cudaGraphExec_t graph = nullptr;
    const double* graph_x = nullptr;
    double* graph_g = nullptr;
    bool graph_32 = false;
    long long graph_launches = 0;
    // Markov 2 chains (ctx_markov2.cu): the backward pair (3 directions
    // each), three partial sums for G(N), curved-lattice weights l1, l11,
    // l_1, l_11
    double *d_m2gb = nullptr, *d_m2w = nullptr, *d_m2l = nullptr;
    // the device-resident solve loop (NM_OPT_DEVICE_LOOP): one graph per
    // field pointer, its state in d_loop, launches per pass of each branch
    bool device_loop = false;
    void* d_loop = nullptr;
    cudaGraphExec_t loop_graph = nullptr;
    const double* loop_x = nullptr;
    long long loop_l32 = 0, loop_l64 = 0, loop_lrest = 0;
    NormArgs norm_args;
    PhiArgs phi_args;
    ResArgs res_args;
    std::vector<double> chi;  // the context's χ (nm_ctx_set_values may change it)
    // internal states: n_state, species count, u and α of each state
    // [n_state*M]; d_phi, d_phi_side and d_seg_phibulk hold one row per
    // species (the states' after the segments')
    int nst = 0, nsp = 0;
    StArgs st{};
    double *d_ust = nullptr, *d_ast = nullptr;
    std::vector<double> chi_sp;  // χ between species (plans with states)
    std::vector<double> st_fixed;  // the fixed states' alphabulk in force (nm_ctx_set_values)
    std::vector<double> st_pK;     // the reactions' pK in force (nm_ctx_set_values)
    // electrostatics (charged systems, 1 and 2 gradients): ψ is the last
    // block of x; halo sites of the composition are evaluated (nh of them)
    bool charged = false;
    int nh = 0;
    ChgArgs chg{};
    ElecConst ec{};
    double *d_EE = nullptr, *d_psi = nullptr, *d_q = nullptr, *d_eps = nullptr, *d_X = nullptr;
    // persistent 2-D sweeps: one cooperative launch per sweep (ctx2d.cu)
    bool use2d = false;      // eligible and set up
    bool sweep2d = false;    // nm_ctx_set_option(NM_OPT_SWEEP2D)
    int sw_rows = 0, sw_ctas = 0;
    int* d_flags = nullptr;  // per-CTA step published
    std::vector<SweepTab> sw_tabs;
    // FP32 propagators on 2-gradient lattices (ctx2d32.cu): per-row exponents
    bool use2d32 = false;
    int* d_E2b = nullptr;           // [2][MX+2] exponents of the backward pair
    double* d_rowpart = nullptr;    // [MX+2] per-row partial sums of G(N)
    std::vector<int*> E2f;          // per molecule [n_store][MX+2]

    int init(const nm_plan* p, const nm_ctx_options* opt);
    ~Ctx();
    int launch_prop(const double* in, const double* G1, double* out);
    int launch_g1(const double* x, bool with32);  // G1 (and its FP32 copy) from the field x
    int wsum(const double* X, double* out_dev);
    int molecule_pass(int m);
    int residual(const double* x, double* g);
    int residual_launches(const double* x, double* g);
    int check_status();
    int solve(double* x, nm_solve_result* res, int max_iter);
    double tol_override = 0;        // > 0: the solve's tolerance (a search's inner solves)
    int free_energy(double* F, double* Omega, double* mu);
    int elec_init();                                // constants and buffers
    int elec_field(const double* x);                // ψ with mirror bounds, EE
    int elec_residual(const double* x, double* g);  // q, ε, ψ block of g
};

}  // namespace nm
