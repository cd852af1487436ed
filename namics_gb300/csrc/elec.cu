// Electrostatics of a charged system in a device context (1, 2 and 3 gradients).
//
// ψ is the last block of the iteration vector x.  Per residual evaluation:
//   before G1   k_field        ψ with mirror bounds on every side and the
//                              field-energy weight EE (Lattice::UpdateEE,
//                              LG1Planar.cpp:162-200, LGrad1.cpp:593-640,
//                              LG2Planar.cpp:1130-1175, LGrad2.cpp:1392-1420)
//   after φ     k_charge       q = Σ vφ/φ_tot, ε = Σ εφ/φ_tot at every site
//                              (System::DoElectrostatics, system.cpp:1920-1953)
//               k_psi_*        g_ψ = ψ − X(ψ), X the Poisson update of ψ
//                              (Lattice::UpdatePsi, LGrad1.cpp:641-680,
//                              LGrad2.cpp:1420-1444, system.cpp:2161-2170)
// The Poisson update is an upwind (Gauss–Seidel-ordered) sweep on the planar
// and 1-D cylindrical lattices: each site takes the already updated value of
// its lower neighbours.  It runs as one thread along x in 1-D and as one
// block over anti-diagonals in 2-D; the spherical and 2-D cylindrical updates
// read only old values and run over all sites in parallel.  In 3-D it is a
// forward then a backward Gauss–Seidel sweep in place on ψ (LGrad3.cpp:
// 1155-1215): one block walks the planes x + y + z = d up, then down, which
// gives each site exactly the inputs of the reference's sequential sweeps.
#include <cuda_runtime.h>

#include <string>

#include "ctx_internal.h"

using nmdev::Lat;

namespace nm {

namespace {

constexpr double E_CHARGE = 1.60217e-19;
constexpr double K_BT = 1.38065e-23 * 298.15;
constexpr double EPS0 = 8.85418e-12;
constexpr double PIE = 3.14159265;

// site of the mirror bounds (set_M_bounds) that halo site s takes; in 3-D
// only the faces are set (LGrad3.cpp:1679-1702), edges and corners keep
// their own value
__device__ __forceinline__ int mirror_src(const Lat& L, int s) {
    if (L.g == 1) return s == 0 ? 1 : (s == L.MX + 1 ? L.MX : s);
    if (L.g == 3) {
        int x = s / L.JX, r = s % L.JX, y = r / L.JY, z = r % L.JY;
        const int ox = x == 0 || x == L.MX + 1, oy = y == 0 || y == L.MY + 1, oz = z == 0 || z == L.MZ + 1;
        if (ox + oy + oz != 1) return s;
        if (ox) x = x == 0 ? 1 : L.MX;
        if (oy) y = y == 0 ? 1 : L.MY;
        if (oz) z = z == 0 ? 1 : L.MZ;
        return x * L.JX + y * L.JY + z;
    }
    int x = s / L.JX, y = s % L.JX;
    x = x == 0 ? 1 : (x == L.MX + 1 ? L.MX : x);
    y = y == 0 ? 1 : (y == L.MY + 1 ? L.MY : y);
    return x * L.JX + y;
}

__global__ void k_field(Lat L, ElecConst c, const double* __restrict__ xpsi, double* __restrict__ psi,
                        double* __restrict__ EE) {
    const int M = L.M;
    auto P = [&](int i) { return xpsi[mirror_src(L, i)]; };
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < M; s += gridDim.x * blockDim.x) {
        psi[s] = P(s);
        double e = 0;
        if (L.g == 3) {
            // squared differences along z, x and y over the flat array
            // (AddGradSquare, tools_host.h:444), at every site that has both
            // neighbours in the array, then the prefactor
            const int dd[3] = {1, L.JX, L.JY};
            for (int k = 0; k < 3; k++) {
                const int d = dd[k];
                if (s >= d && s < M - d) {
                    const double u = P(s - d) - P(s), w = P(s) - P(s + d);
                    e += u * u + w * w;
                }
            }
            EE[s] = e * c.pf;
            continue;
        }
        if (nmdev::is_interior(L, s)) {
            const double pf = c.pf;
            if (L.g == 1) {
                const int x = s;
                if (L.geom == 0) {
                    double a = P(x - 1) - P(x), b = P(x) - P(x + 1);
                    e = pf * (a * a + b * b);
                } else if (L.geom == 1) {
                    const int r = (int)c.offset + x;
                    double a = P(x) - P(x - 1);
                    a *= (r - 1) * a;
                    double b = P(x) - P(x + 1);
                    b *= r * b;
                    e = pf * (a + b) / c.Lv[x];
                } else {
                    const int r0 = (int)(c.offset + 1.0);
                    double b = (r0 + x - 1) * (P(x) - P(x + 1));
                    b *= b;
                    if (x == 1) {
                        e = pf * b / c.Lv[x];
                    } else {
                        double a = (r0 + x - 2) * (P(x - 1) - P(x));
                        a *= a;
                        e = pf * (a + b) / c.Lv[x];
                    }
                }
            } else {
                const int JX = L.JX;
                const double p0 = P(s);
                double xm = p0 - P(s - JX), xp = p0 - P(s + JX);
                double ym = p0 - P(s - 1), yp = p0 - P(s + 1);
                ym *= ym;
                yp *= yp;
                if (L.geom == 0) {
                    xm *= xm;
                    xp *= xp;
                    e = pf * (xm + xp + ym + yp);
                } else {
                    const int r = (int)c.offset + s / JX;
                    xm *= (r - 0.5) * xm * 2 * PIE;
                    xp *= (r + 0.5) * xp * 2 * PIE;
                    e = pf * ((xm + xp) / c.Lv[s] + ym + yp);
                }
            }
        }
        EE[s] = e;
    }
}

// q and ε at every site from the bounded φ of each segment (halo sites take
// their set_bounds source); the division by φ_tot gives 0 where φ_tot = 0
__global__ void k_charge(Lat L, int ns, ChgArgs a, const double* __restrict__ phi,
                         const double* __restrict__ phitot, double* __restrict__ q, double* __restrict__ eps) {
    const int M = L.M;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < M; s += gridDim.x * blockDim.x) {
        const int src = nmdev::bc_source(L, s);
        double qv = 0, ev = 0;
        for (int i = 0; i < ns; i++) {
            const double p = phi[(size_t)i * M + src];
            qv += a.val[i] * p;
            ev += a.eps[i] * p;
        }
        // internal states: their volume fractions are the species rows
        // after the segments' (System::DoElectrostatics, system.cpp:1936-1941)
        for (int i = ns; i < a.nsp; i++) qv += a.val[i] * phi[(size_t)i * M + src];
        const double pt = phitot[s];
        q[s] = pt != 0 ? qv / pt : 0.0;
        eps[s] = pt != 0 ? ev / pt : 0.0;
    }
}

// 2-D planar with MX ≤ 1024: the same wavefront with one thread per row x.
// Site (x, y) of anti-diagonal d = x + y needs X(x, y-1), which the same
// thread made on diagonal d-1 (kept in a register), and X(x-1, y), which
// its neighbour thread made (read from shared memory, double-buffered by
// diagonal parity, one block barrier per diagonal).  The global loads of the
// next diagonal's site do not depend on the wavefront and are issued before
// the barrier.  Same expression as k_psi_sweep2, so the same values.
__global__ void __launch_bounds__(1024) k_psi_wave2(Lat L, ElecConst c, const double* __restrict__ xpsi,
                                                     const double* __restrict__ psi, const double* __restrict__ q,
                                                     const double* __restrict__ eps, double* __restrict__ X,
                                                     double* __restrict__ g) {
    __shared__ double wave[2][1026];
    const int MX = L.MX, MY = L.MY, JX = L.JX, M = L.M;
    const int x = 1 + (int)threadIdx.x;
    const bool row = x <= MX;
    double mine = 0;  // X(x, y-1)
    // the operands of site (x, d - x), loaded ahead of the wavefront
    double e0 = 0, exm = 0, exp_ = 0, eym = 0, eyp = 0, cq = 0, pxp = 0, pyp = 0, pxm = 0, pym = 0, xp = 0;
    auto load = [&](int d) {
        const int y = d - x;
        if (!row || y < 1 || y > MY) return;
        const int i = x * JX + y;
        e0 = eps[i];
        exm = e0 + eps[i - JX]; exp_ = e0 + eps[i + JX];
        eym = e0 + eps[i - 1]; eyp = e0 + eps[i + 1];
        cq = c.C * q[i];
        pxp = psi[i + JX]; pyp = psi[i + 1];
        pxm = psi[i - JX]; pym = psi[i - 1];
        xp = xpsi[i];
    };
    load(2);
    for (int d = 2; d <= MX + MY; d++) {
        const int y = d - x;
        const bool on = row && y >= 1 && y <= MY;
        double v = 0;
        if (on) {
            const int i = x * JX + y;
            const double ax = x == 1 ? pxm : wave[(d - 1) & 1][x - 1];
            const double ay = y == 1 ? pym : mine;
            v = (cq + exm * ax + exp_ * pxp + eym * ay + eyp * pyp) / (exm + exp_ + eym + eyp);
            X[i] = v;
            g[i] = xp - v;
            mine = v;
            wave[d & 1][x] = v;
        }
        load(d + 1);
        __syncthreads();
    }
    // halo sites of the ψ block of g
    for (int s = threadIdx.x; s < M; s += blockDim.x)
        if (!nmdev::is_interior(L, s)) g[s] = 0.0;
}

// 1-D planar and cylindrical: upwind sweep along x in one thread
__global__ void k_psi_sweep1(Lat L, ElecConst c, const double* __restrict__ xpsi, const double* __restrict__ psi,
                             const double* __restrict__ q, const double* __restrict__ eps, double* __restrict__ g) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int MX = L.MX;
    const bool cyl = L.geom == 1;
    double r = c.offset;
    double eplus = cyl ? r * (eps[0] + eps[1]) : eps[0] + eps[1];
    double a = psi[0];
    for (int x = 1; x <= MX; x++) {
        const double emin = eplus;
        if (cyl) {
            r += 1;
            eplus = r * (eps[x] + eps[x + 1]);
        } else {
            eplus = eps[x] + eps[x + 1];
        }
        const double X = (emin * a + c.C * q[x] + eplus * psi[x + 1]) / (emin + eplus);
        g[x] = xpsi[x] - X;
        a = X;
    }
    g[0] = 0;
    g[MX + 1] = 0;
}

// 2-D planar: upwind in x and y.  Site (x, y) needs the updated (x-1, y) and
// (x, y-1), so the block walks the anti-diagonals x + y = d in order.
__global__ void k_psi_sweep2(Lat L, ElecConst c, const double* __restrict__ xpsi, const double* __restrict__ psi,
                             const double* __restrict__ q, const double* __restrict__ eps, double* __restrict__ X,
                             double* __restrict__ g) {
    const int MX = L.MX, MY = L.MY, JX = L.JX, M = L.M;
    for (int d = 2; d <= MX + MY; d++) {
        const int x0 = d - MY > 1 ? d - MY : 1;
        const int x1 = d - 1 < MX ? d - 1 : MX;
        for (int x = x0 + (int)threadIdx.x; x <= x1; x += blockDim.x) {
            const int y = d - x;
            const int i = x * JX + y;
            const double exm = eps[i] + eps[i - JX], exp_ = eps[i] + eps[i + JX];
            const double eym = eps[i] + eps[i - 1], eyp = eps[i] + eps[i + 1];
            const double ax = x == 1 ? psi[i - JX] : X[i - JX];
            const double ay = y == 1 ? psi[i - 1] : X[i - 1];
            X[i] = (c.C * q[i] + exm * ax + exp_ * psi[i + JX] + eym * ay + eyp * psi[i + 1]) /
                   (exm + exp_ + eym + eyp);
        }
        __syncthreads();
    }
    for (int s = threadIdx.x; s < M; s += blockDim.x)
        g[s] = nmdev::is_interior(L, s) ? xpsi[s] - X[s] : 0.0;
}

// 3-D: forward and backward Gauss–Seidel sweeps in place on psi (mirror
// bounded), one block, plane x + y + z = d at a time; the backward sweep
// leaves g = x_ψ − ψ_new at interior sites
__global__ void k_psi_gs3(Lat L, ElecConst c, const double* __restrict__ xpsi, double* __restrict__ psi,
                          const double* __restrict__ q, const double* __restrict__ eps, double* __restrict__ g) {
    const int MX = L.MX, MY = L.MY, MZ = L.MZ, JX = L.JX, JY = L.JY, M = L.M;
    const int D = MX + MY + MZ;
    for (int pass = 0; pass < 2; pass++) {
        for (int k = 0; k <= D - 3; k++) {
            const int d = pass ? D - k : 3 + k;
            for (int idx = threadIdx.x; idx < MX * MY; idx += blockDim.x) {
                const int x = idx / MY + 1, y = idx % MY + 1, z = d - x - y;
                if (z < 1 || z > MZ) continue;
                const int i = x * JX + y * JY + z;
                const double ezm = eps[i - 1] + eps[i], ezp = eps[i] + eps[i + 1];
                const double eym = eps[i] + eps[i - JY], eyp = eps[i] + eps[i + JY];
                const double exm = eps[i] + eps[i - JX], exp_ = eps[i] + eps[i + JX];
                const double v = (exm * psi[i - JX] + exp_ * psi[i + JX] + eym * psi[i - JY] + eyp * psi[i + JY] +
                                  ezm * psi[i - 1] + ezp * psi[i + 1] + c.C * q[i]) /
                                 (exm + exp_ + eym + eyp + ezm + ezp);
                psi[i] = v;
                if (pass) g[i] = xpsi[i] - v;
            }
            __syncthreads();
        }
    }
    for (int s = threadIdx.x; s < M; s += blockDim.x)
        if (!nmdev::is_interior(L, s)) g[s] = 0.0;
}

// 1-D spherical and 2-D cylindrical: every site from old values
__global__ void k_psi_jacobi(Lat L, ElecConst c, const double* __restrict__ xpsi, const double* __restrict__ psi,
                             const double* __restrict__ q, const double* __restrict__ eps, double* __restrict__ g) {
    const int M = L.M;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < M; s += gridDim.x * blockDim.x) {
        if (!nmdev::is_interior(L, s)) { g[s] = 0; continue; }
        double X;
        if (L.g == 1) {
            const int x = s;
            const double rm = c.offset + (x - 1), r = c.offset + x;
            const double emin = rm * rm * (eps[x - 1] + eps[x]);
            const double eplus = r * r * (eps[x] + eps[x + 1]);
            X = (emin * psi[x - 1] + c.C * q[x] * c.Lv[x] + eplus * psi[x + 1]) / (emin + eplus);
        } else {
            const int JX = L.JX;
            const double r = c.offset + s / JX;
            const double exm = 2 * PIE * (r - 1) * (eps[s] + eps[s - JX]) / c.Lv[s];
            const double exp_ = 2 * PIE * r * (eps[s] + eps[s + JX]) / c.Lv[s];
            const double eym = eps[s] + eps[s - 1], eyp = eps[s] + eps[s + 1];
            X = (c.C * q[s] + exm * psi[s - JX] + exp_ * psi[s + JX] + eym * psi[s - 1] + eyp * psi[s + 1]) /
                (exm + exp_ + eym + eyp);
        }
        g[s] = xpsi[s] - X;
    }
}

int grid_of(int n) {
    int b = (n + 255) / 256;
    return b < 1 ? 1 : (b > 4 * 152 * 8 ? 4 * 152 * 8 : b);
}

}  // namespace

int Ctx::elec_init() {
    const nm_plan* p = plan;
    if (!(p->bond_length > 0)) {
        set_error("charged system needs a positive lattice bondlength");
        return NM_ERR_INPUT;
    }
    charged = true;
    chg.on = 1;
    for (int i = 0; i < p->n_seg; i++) { chg.eps[i] = p->seg_epsilon[i]; chg.val[i] = p->seg_valence[i]; }
    // the states' valences follow the segments' (species order); a segment
    // with states carries valence 0 in the plan
    chg.nsp = p->n_seg + p->n_state;
    for (int j = 0; j < p->n_state; j++) chg.val[p->n_seg + j] = p->state_valence[j];
    // UpdateEE prefactor and UpdatePsi constant, in the reference's order
    double pf = 0.5 * EPS0 * p->bond_length / K_BT * (K_BT / E_CHARGE) * (K_BT / E_CHARGE);
    double C = E_CHARGE * E_CHARGE / (EPS0 * K_BT * p->bond_length);
    if (p->gradients == 1) {
        if (p->geometry == NM_PLANAR) { pf = pf / 2.0; C = C * 2.0; }
        else if (p->geometry == NM_CYLINDRICAL) { pf = pf * PIE; C = C / PIE; }
        else { pf = pf * PIE * 2; C = C / (2.0 * PIE); }
    } else if (p->gradients == 3) {
        // planar only, no geometry factors (LGrad3.cpp:1132, 1170)
    } else {
        pf = pf / 2;
        C = p->geometry == NM_PLANAR ? C * 2.0 : C / 2;
    }
    ec.pf = pf;
    ec.C = C;
    ec.offset = p->offset_first_layer;
    ec.Lv = d_L;
    size_t M = p->M;
    for (double** b : {&d_EE, &d_psi, &d_q, &d_eps, &d_X}) {
        cudaError_t e = cudaMallocAsync((void**)b, sizeof(double) * M, stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(*b, 0, sizeof(double) * M, stream);
        if (e != cudaSuccess) { set_error(std::string("electrostatics buffers: ") + cudaGetErrorString(e)); return NM_ERR_NOMEM; }
    }
    // halo sites of the composition; in 3-D the halo part runs over all M
    // sites and skips the interior
    nh = p->gradients == 1 ? 2 : (p->gradients == 2 ? 2 * p->JX + 2 * p->MX : p->M);
    return NM_OK;
}

int Ctx::elec_field(const double* x) {
    const double* xpsi = x + (size_t)plan->n_it * plan->M;
    k_field<<<grid_of(plan->M), 256, 0, stream>>>(lat, ec, xpsi, d_psi, d_EE);
    launches++;
    return NM_OK;
}

int Ctx::elec_residual(const double* x, double* g) {
    const size_t off = (size_t)plan->n_it * plan->M;
    const double* xpsi = x + off;
    double* gp = g + off;
    const int M = plan->M;
    k_charge<<<grid_of(M), 256, 0, stream>>>(lat, plan->n_seg, chg, d_phi, d_phitot, d_q, d_eps);
    if (plan->gradients == 1 && plan->geometry != NM_SPHERICAL)
        k_psi_sweep1<<<1, 32, 0, stream>>>(lat, ec, xpsi, d_psi, d_q, d_eps, gp);
    else if (plan->gradients == 2 && plan->geometry == NM_PLANAR)
        if (plan->MX <= 1024)
            k_psi_wave2<<<1, (plan->MX + 31) / 32 * 32, 0, stream>>>(lat, ec, xpsi, d_psi, d_q, d_eps, d_X, gp);
        else
            k_psi_sweep2<<<1, 512, 0, stream>>>(lat, ec, xpsi, d_psi, d_q, d_eps, d_X, gp);
    else if (plan->gradients == 3)
        k_psi_gs3<<<1, 1024, 0, stream>>>(lat, ec, xpsi, d_psi, d_q, d_eps, gp);
    else
        k_psi_jacobi<<<grid_of(M), 256, 0, stream>>>(lat, ec, xpsi, d_psi, d_q, d_eps, gp);
    launches += 2;
    return NM_OK;
}

}  // namespace nm
