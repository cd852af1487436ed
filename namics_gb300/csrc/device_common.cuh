// Lattice description and the per-site stencils shared by all kernels.
//
// A propagation step computes, at every interior site, the weighted
// neighbour sum of Lattice::propagate / Lattice::Side (LG1Planar.cpp:28-55,
// 138-159; LGrad1.cpp:251-281, 432-454; LG2Planar.cpp:27-135, 1039-1127;
// LGrad2.cpp:207-278, 1053-1090; LGrad3.cpp:103-243, 673-782).  Halo values
// are never materialised: a neighbour coordinate in the halo layer is mapped
// to the site the reference's set_bounds copies into it (lattice.cpp:94-196:
// mirror -> first/last layer, periodic -> opposite layer, surface -> the halo
// slot itself, which holds a frozen wall).  Composing the per-axis maps
// reproduces the edge and corner order of LGrad2/LGrad3::set_bounds.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace nmdev {

struct Lat {
    int g, MX, MY, MZ, JX, JY, M;
    int geom, lat;                 // nm_geometry, nm_lattype
    int b1[3], bm[3];              // halo source layer per axis (lo, hi)
    double lam;
    const double* lm1;             // curved-lattice weights (device) or null
    const double* l1;
    const double* l0;
};

__device__ __forceinline__ int bmap(int c, int n, int b1, int bm) {
    return c == 0 ? b1 : (c == n + 1 ? bm : c);
}

// Load functor over a device array with halo mapping.
template <typename T>
struct GLoad {
    const T* __restrict__ p;
    __device__ __forceinline__ double operator()(int i) const { return (double)p[i]; }
};

// Neighbour sum at interior site (x,y,z) of array `ld` (site index via JX/JY).
template <typename LD>
__device__ __forceinline__ double stencil_at(const Lat& L, const LD& ld, int x, int y, int z) {
    if (L.g == 1) {
        int xm = bmap(x - 1, L.MX, L.b1[0], L.bm[0]);
        int xp = bmap(x + 1, L.MX, L.b1[0], L.bm[0]);
        double gm = ld(xm), g0 = ld(x), gp = ld(xp);
        if (L.geom == 0) return L.lam * gm + (1.0 - 2.0 * L.lam) * g0 + L.lam * gp;
        return g0 * L.l0[x] + gm * L.lm1[x] + gp * L.l1[x];
    }
    if (L.g == 2) {
        int JX = L.JX;
        int xm = bmap(x - 1, L.MX, L.b1[0], L.bm[0]);
        int xp = bmap(x + 1, L.MX, L.b1[0], L.bm[0]);
        int ym = bmap(y - 1, L.MY, L.b1[1], L.bm[1]);
        int yp = bmap(y + 1, L.MY, L.b1[1], L.bm[1]);
        double c = ld(x * JX + y);
        double xl = ld(xm * JX + y), xh = ld(xp * JX + y);
        double yl = ld(x * JX + ym), yh = ld(x * JX + yp);
        double dll = ld(xm * JX + ym), dlh = ld(xm * JX + yp);
        double dhl = ld(xp * JX + ym), dhh = ld(xp * JX + yp);
        if (L.geom == 0) {
            if (L.lat == 0)
                return (16.0 / 36.0) * c + (4.0 / 36.0) * ((xl + xh) + (yl + yh)) +
                       (1.0 / 36.0) * ((dll + dhh) + (dlh + dhl));
            return ((2.0 * c + (xl + xh) + (yl + yh)) * 2.0 + (dll + dhh) + (dlh + dhl)) * (1.0 / 16.0);
        }
        double C1, C2, C3;
        if (L.lat == 0) { C1 = 4.0 / 6.0; C2 = 1.0 / 6.0; C3 = 4.0; }
        else { C1 = 0.5; C2 = 0.25; C3 = 2.0; }
        int s = x * JX + y;
        double lm = L.lm1[s], lp = L.l1[s];
        double a = C1 * c + lm * xl + lp * xh + C2 * yl + C2 * yh;
        return (a * C3 + lm * (dll + dlh) + lp * (dhl + dhh)) * C2;
    }
    int JX = L.JX, JY = L.JY;
    int xm = bmap(x - 1, L.MX, L.b1[0], L.bm[0]);
    int xp = bmap(x + 1, L.MX, L.b1[0], L.bm[0]);
    int ym = bmap(y - 1, L.MY, L.b1[1], L.bm[1]);
    int yp = bmap(y + 1, L.MY, L.b1[1], L.bm[1]);
    int zm = bmap(z - 1, L.MZ, L.b1[2], L.bm[2]);
    int zp = bmap(z + 1, L.MZ, L.b1[2], L.bm[2]);
    if (L.lat == 0) {
        double s6 = ((ld(xm * JX + y * JY + z) + ld(xp * JX + y * JY + z)) +
                     (ld(x * JX + ym * JY + z) + ld(x * JX + yp * JY + z))) +
                    (ld(x * JX + y * JY + zm) + ld(x * JX + y * JY + zp));
        return s6 * (1.0 / 6.0);
    }
    int X[3] = {xm, x, xp}, Y[3] = {ym, y, yp}, Z[3] = {zm, z, zp};
    double acc[4] = {0, 0, 0, 0};  // by number of displaced axes
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++)
            for (int c = 0; c < 3; c++) {
                int nd = (a != 1) + (b != 1) + (c != 1);
                acc[nd] += ld(X[a] * JX + Y[b] * JY + Z[c]);
            }
    return (((2.0 * acc[0] + acc[1]) * 2.0 + acc[2]) * 2.0 + acc[3]) * (1.0 / 40.0);
}

__device__ __forceinline__ void site_coords(const Lat& L, int idx, int& x, int& y, int& z) {
    // idx enumerates interior sites in layout order
    if (L.g == 1) { x = idx + 1; y = 0; z = 0; return; }
    if (L.g == 2) { x = idx / L.MY + 1; y = idx % L.MY + 1; z = 0; return; }
    int yz = L.MY * L.MZ;
    x = idx / yz + 1;
    int r = idx - (x - 1) * yz;
    y = r / L.MZ + 1;
    z = r % L.MZ + 1;
}

__device__ __forceinline__ int interior_count(const Lat& L) {
    return L.g == 1 ? L.MX : (L.g == 2 ? L.MX * L.MY : L.MX * L.MY * L.MZ);
}

__device__ __forceinline__ bool is_interior(const Lat& L, int s) {
    if (L.g == 1) return s >= 1 && s <= L.MX;
    if (L.g == 2) { int x = s / L.JX, y = s % L.JX; return x >= 1 && x <= L.MX && y >= 1 && y <= L.MY; }
    int x = s / L.JX, r = s % L.JX, y = r / L.JY, z = r % L.JY;
    return x >= 1 && x <= L.MX && y >= 1 && y <= L.MY && z >= 1 && z <= L.MZ;
}

// ---- halo sites (1 and 2 gradients) --------------------------------------
// The reference keeps its propagators as flat padded arrays and applies the
// neighbour sum to every element, halo layers included.  The values it leaves
// in the halo are overwritten by set_bounds before any propagator is read
// again, with one exception that reaches the result: the halo part of the
// composition rho, which flows into φ_tot at halo sites and from there into
// the relative permittivity ε = Σ ε_i φ_i / φ_tot that the Poisson update
// reads at its boundary neighbours.  Charged systems therefore evaluate the
// flat-array neighbour sum at the halo sites as well.

__device__ __forceinline__ int halo_count(const Lat& L) {
    return L.g == 1 ? 2 : 2 * L.JX + 2 * L.MX;
}
// (3 gradients: the halo part runs over all M sites and skips the interior)

// j-th halo site: 1-D {0, MX+1}; 2-D the rows x = 0 and x = MX+1, then the
// columns y = 0 and y = MY+1 of x = 1..MX.
__device__ __forceinline__ int halo_site(const Lat& L, int j) {
    if (L.g == 1) return j == 0 ? 0 : L.MX + 1;
    const int JX = L.JX;
    if (j < JX) return j;
    j -= JX;
    if (j < JX) return (L.MX + 1) * JX + j;
    j -= JX;
    return (j / 2 + 1) * JX + ((j & 1) ? L.MY + 1 : 0);
}

// Lattice::propagate's neighbour sum at site s of the flat array (every
// term whose write and read positions lie inside the array, in the order
// the reference accumulates them): LG1Planar.cpp:138-159, LGrad1.cpp:
// 432-454, LG2Planar.cpp:1039-1127, LGrad2.cpp:1053-1090.  `g` loads an
// element of the already bounded input.
// one flat-array term: gs[w + i] += g[r + i] for i in [0, n)
template <typename LD>
__device__ __forceinline__ void flat_add(double& v, const LD& g, int s, int w, int r, int n) {
    if (s >= w && s < w + n) v += g(s - w + r);
}

template <typename LD>
__device__ __forceinline__ double flat_prop_at(const Lat& L, const LD& g, int s) {
    const int M = L.M, JX = L.JX;
    if (L.g == 3) {  // LGrad3.cpp:673-782, stencil_full
        const int JY = L.JY;
        double v = 0;
        if (L.lat != 0) v = 2.0 * g(s);
        flat_add(v, g, s, JX, 0, M - JX); flat_add(v, g, s, 0, JX, M - JX);
        flat_add(v, g, s, JY, 0, M - JY); flat_add(v, g, s, 0, JY, M - JY);
        flat_add(v, g, s, 1, 0, M - 1); flat_add(v, g, s, 0, 1, M - 1);
        if (L.lat == 0) return v * (1.0 / 6.0);
        v *= 2.0;
        flat_add(v, g, s, JX + JY, 0, M - JX - JY); flat_add(v, g, s, 0, JX + JY, M - JX - JY);
        flat_add(v, g, s, JX, JY, M - JX - JY); flat_add(v, g, s, JY, JX, M - JX - JY);
        flat_add(v, g, s, JX + 1, 0, M - JX - 1); flat_add(v, g, s, 1, JX, M - JX - 1);
        flat_add(v, g, s, JY + 1, 0, M - JY - 1); flat_add(v, g, s, 1, JY, M - JY - 1);
        flat_add(v, g, s, JX, 1, M - JX - 1); flat_add(v, g, s, 0, JX + 1, M - JX - 1);
        flat_add(v, g, s, JY, 1, M - JY - 1); flat_add(v, g, s, 0, JY + 1, M - JY - 1);
        v *= 2.0;
        const int n3 = M - JX - JY - 1;
        flat_add(v, g, s, JX + JY + 1, 0, n3); flat_add(v, g, s, 0, JX + JY + 1, n3);
        flat_add(v, g, s, JX + JY, 1, n3); flat_add(v, g, s, 1, JX + JY, n3);
        flat_add(v, g, s, JX + 1, JY, n3); flat_add(v, g, s, JY, JX + 1, n3);
        flat_add(v, g, s, JY + 1, JX, n3); flat_add(v, g, s, JX, JY + 1, n3);
        return v * (1.0 / 40.0);
    }
    if (L.g == 1) {
        if (L.geom == 0) {
            double v = 0;
            if (s >= 1) v += L.lam * g(s - 1);
            v += (1.0 - 2.0 * L.lam) * g(s);
            if (s < M - 1) v += L.lam * g(s + 1);
            return v;
        }
        double v = g(s) * L.l0[s];
        if (s >= 1) v += g(s - 1) * L.lm1[s];
        if (s < M - 1) v += g(s + 1) * L.l1[s];
        return v;
    }
    if (L.geom == 0) {
        if (L.lat == 0) {
            const double C1 = 16.0 / 36.0, C2 = 4.0 / 36.0, C3 = 1.0 / 36.0;
            double v = C1 * g(s);
            if (s >= 1) v += C2 * g(s - 1);
            if (s < M - 1) v += C2 * g(s + 1);
            if (s >= JX) v += C2 * g(s - JX);
            if (s < M - JX) v += C2 * g(s + JX);
            if (s >= JX + 1) v += C3 * g(s - JX - 1);
            if (s >= JX) v += C3 * g(s - JX + 1);
            if (s >= 1 && s < M - JX + 1) v += C3 * g(s + JX - 1);
            if (s < M - JX - 1) v += C3 * g(s + JX + 1);
            return v;
        }
        double v = 2.0 * g(s);
        if (s >= JX) v += g(s - JX);
        if (s < M - JX) v += g(s + JX);
        if (s >= 1) v += g(s - 1);
        if (s < M - 1) v += g(s + 1);
        v *= 2.0;
        if (s >= JX + 1) v += g(s - JX - 1);
        if (s < M - JX - 1) v += g(s + JX + 1);
        if (s >= JX && s < M - 1) v += g(s - JX + 1);
        if (s >= 1 && s < M - JX) v += g(s + JX - 1);
        return v * (1.0 / 16.0);
    }
    double C1, C2, C3;
    if (L.lat == 0) { C1 = 4.0 / 6.0; C2 = 1.0 / 6.0; C3 = 4.0; }
    else { C1 = 0.5; C2 = 0.25; C3 = 2.0; }
    double v = C1 * g(s);
    if (s >= JX) v += g(s - JX) * L.lm1[s];
    if (s < M - JX) v += g(s + JX) * L.l1[s];
    if (s >= 1) v += C2 * g(s - 1);
    if (s < M - 1) v += C2 * g(s + 1);
    v *= C3;
    if (s >= JX + 1) v += g(s - JX - 1) * L.lm1[s];
    if (s >= JX && s < M - 1) v += g(s - JX + 1) * L.lm1[s];
    if (s >= 1 && s < M - JX) v += g(s + JX - 1) * L.l1[s];
    if (s < M - JX - 1) v += g(s + JX + 1) * L.l1[s];
    return v * C2;
}

// Source site that set_bounds copies into site s (s itself when interior).
__device__ __forceinline__ int bc_source(const Lat& L, int s) {
    if (L.g == 1) return bmap(s, L.MX, L.b1[0], L.bm[0]);
    if (L.g == 2) {
        int x = s / L.JX, y = s % L.JX;
        return bmap(x, L.MX, L.b1[0], L.bm[0]) * L.JX + bmap(y, L.MY, L.b1[1], L.bm[1]);
    }
    int x = s / L.JX, r = s % L.JX, y = r / L.JY, z = r % L.JY;
    return bmap(x, L.MX, L.b1[0], L.bm[0]) * L.JX + bmap(y, L.MY, L.b1[1], L.bm[1]) * L.JY +
           bmap(z, L.MZ, L.b1[2], L.bm[2]);
}

// Programmatic dependent launch: a step kernel launched with the
// programmatic-serialisation attribute may be scheduled while its
// predecessor drains.  It waits for the predecessor's completion (all writes
// visible) before touching memory, and releases its own successor only after
// its stores; released at the start instead, chains of waiting grids filled
// the SMs and 2-D residuals ran twice as long.
__device__ __forceinline__ void pdl_begin() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_end() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Element i of an array after set_bounds: the halo takes its source site's
// value (a surface halo keeps its own, zero in every stored propagator).
struct BLoad {
    const double* __restrict__ p;
    Lat L;
    __device__ __forceinline__ double operator()(int i) const { return p[bc_source(L, i)]; }
};

}  // namespace nmdev
