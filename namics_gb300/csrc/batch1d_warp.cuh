// FP32 phase of the batched 1-gradient solver, one warp per problem.
//
// Lane l owns the contiguous sites x = l·S+1 .. l·S+S (S = 4, 8, 12 or 16, a
// compile-time chunk that covers MX <= 32·S), so a propagation step is
// register arithmetic plus two shuffles for the chunk-edge neighbours (two
// more for periodic bounds, which set_bounds fills from the opposite end,
// lattice.cpp:94-196).  There is no block barrier and no shared-memory round
// trip per step.  Propagators are block floating point: FP32 mantissas and a
// power-of-two exponent per lane, renormalised every BW_RS steps from the
// lane's own maximum (see bw_lnorm).  Stored forward propagators use a lane-major
// layout (element (l, j) at j·32 + l) so every warp store and load is
// coalesced.  φ, φ_side and the residual are evaluated in FP32 in this phase;
// G(N), the normalisation and the DIIS algebra are FP64.  The phase ends at
// ‖g‖ < sw_tol (or on a stall close to convergence) and hands the field and
// the iteration count to the FP64 kernel, which finishes the solve.
#pragma once

#define BW_FULL 0xffffffffu
#define BW_RS 4

namespace nm {

template <int S, typename T>
__device__ __forceinline__ T bw_pick(const T* v, int j) {
    T t = 0;
#pragma unroll
    for (int q = 0; q < S; q++)
        if (q == j) t = v[q];
    return t;
}

// Values a halo layer holds for register vector v: surface -> wall value,
// mirror -> first/last interior site, periodic -> opposite site.
template <int S, typename T>
__device__ __forceinline__ void bw_halos(const T* v, int b1, int bm, int MX, int lMX, int jMX, T wlo, T whi, T& lo,
                                         T& hi) {
    T v1 = __shfl_sync(BW_FULL, v[0], 0);
    T vmx = __shfl_sync(BW_FULL, bw_pick<S>(v, jMX), lMX);
    lo = (b1 == 0) ? wlo : (b1 == 1 ? v1 : vmx);
    hi = (bm == MX + 1) ? whi : (bm == MX ? vmx : v1);
}

// out = neighbour sum of v at the lane's sites (0 on padding sites)
template <int S, bool CURV, typename T>
__device__ __forceinline__ void bw_sten(const T* v, T lo, T hi, int lane, int MX, T lam, T lmid, const float* cm,
                                        const float* c0, const float* cp, T* out) {
    T lft = __shfl_up_sync(BW_FULL, v[S - 1], 1);
    T rgt = __shfl_down_sync(BW_FULL, v[0], 1);
    if (lane == 0) lft = lo;
    const int x0 = lane * S + 1;
#pragma unroll
    for (int j = 0; j < S; j++) {
        T l = j == 0 ? lft : v[j - 1];
        T r = j == S - 1 ? rgt : v[j + 1];
        if (x0 + j == MX) r = hi;
        T o = CURV ? (v[j] * (T)c0[j] + l * (T)cm[j] + r * (T)cp[j]) : (lam * l + lmid * v[j] + lam * r);
        out[j] = (x0 + j <= MX) ? o : (T)0;
    }
}

// ---------------------------------------------------------------------------
// Per-lane block floating point.  A propagator vector is held as FP32
// mantissas plus one power-of-two exponent per lane (per S contiguous
// sites): G(x) = v(x)·2^E(lane).  A warp-wide exponent is not enough for
// stretched chains: at a grafted brush's converged field the backward
// propagator near the wall is ~2^-240 of its own maximum, far below FP32's
// range, while its product with the forward propagator there is what the
// composition needs.  Across S sites the range is a few tens of binary
// orders at most, so each lane's mantissas stay well inside FP32.
// A propagation step reads one value from each neighbouring lane; it is
// brought to this lane's scale by fl = 2^(E_left - E), fr = 2^(E_right - E),
// which change only when the exponents do (every BW_RS steps).
// ---------------------------------------------------------------------------
#define BW_EMPTY (-0x7fffffff - 1)

// 2^e in FP64 for e <= 0 (0 below the subnormal range)
__device__ __forceinline__ double bw_p2d(int e) {
    return e < -1022 ? 0.0 : __longlong_as_double((long long)(1023 + e) << 52);
}

// neighbour scale factors of a lane with exponent E
__device__ __forceinline__ void bw_nbr(int E, int lane, int lMX, bool per, float& fl, float& fr) {
    int El = __shfl_up_sync(BW_FULL, E, 1);
    int Er = __shfl_down_sync(BW_FULL, E, 1);
    int E0 = __shfl_sync(BW_FULL, E, 0);
    int Em = __shfl_sync(BW_FULL, E, lMX);
    if (lane == 0) El = per ? Em : E;
    if (per && lane == lMX) Er = E0;
    fl = pow2f(min(El - E, 127));
    fr = pow2f(min(Er - E, 127));
}

// Scale the lane's values to a maximum in [0.5, 1) and add the power of two
// to its exponent.  A lane holding only zeros takes the largest exponent of
// the lanes that hold values, so that what flows in from a neighbour lands in
// range.
template <int S>
__device__ __forceinline__ void bw_lnorm(float* v, int& E) {
    float lm = 0.f;
#pragma unroll
    for (int j = 0; j < S; j++) lm = fmaxf(lm, v[j]);
    const int e = expo(lm);
    const float f = pow2f(-e);
#pragma unroll
    for (int j = 0; j < S; j++) v[j] *= f;
    E += e;
    const int Em = __reduce_max_sync(BW_FULL, lm > 0.f ? E : BW_EMPTY);
    if (!(lm > 0.f) && Em != BW_EMPTY) E = Em;
}

// The same from an FP64 vector with per-lane exponent Ein (joins: products of
// several propagators are formed in FP64, a few operations per join).
template <int S>
__device__ __forceinline__ int bw_lnorm_d(const double* v, int Ein, float* out) {
    double lm = 0.0;
#pragma unroll
    for (int j = 0; j < S; j++) lm = fmax(lm, v[j]);
    const int e = lm > 0.0 ? (int)((__double_as_longlong(lm) >> 52) & 0x7ff) - 1022 : 0;
    const double f = __longlong_as_double((long long)(1023 - e) << 52);  // 2^-e
#pragma unroll
    for (int j = 0; j < S; j++) out[j] = (float)(v[j] * f);
    int E = Ein + e;
    const int Em = __reduce_max_sync(BW_FULL, lm > 0.0 ? E : BW_EMPTY);
    if (!(lm > 0.0) && Em != BW_EMPTY) E = Em;
    return E;
}

// Stencil of a stored block-floating-point vector, in FP64 on the warp's
// common scale: out·2^(return value) = neighbour sum of the vector.
template <int S, bool CURV>
__device__ __forceinline__ int bw_sten_lanes(const float* __restrict__ p, const int* __restrict__ pe, int lane, int b1,
                                             int bm, int MX, int lMX, int jMX, double lam, double lmid,
                                             const float* cm, const float* c0, const float* cp, double* out) {
    const int El = pe[lane];
    const int Er = __reduce_max_sync(BW_FULL, El);
    const double f = bw_p2d(El - Er);
    double v[S], lo, hi;
#pragma unroll
    for (int j = 0; j < S; j++) v[j] = (double)p[j * 32 + lane] * f;
    bw_halos<S, double>(v, b1, bm, MX, lMX, jMX, 0.0, 0.0, lo, hi);
    bw_sten<S, CURV, double>(v, lo, hi, lane, MX, lam, lmid, cm, c0, cp, out);
    return Er;
}

// Propagation step with the boundary folded into per-site coefficients
// (aL, aC, aR already include G1): out = aL·v(x-1) + aC·v(x) + aR·v(x+1),
// the neighbouring lanes' edge values scaled by fl, fr.  PER: periodic
// bounds, whose wrap-around neighbours come from the opposite end of the
// chain (v(MX) left of site 1, v(1) right of site MX).
template <int S, bool PER>
__device__ __forceinline__ void bw_step(const float* v, const float* aL, const float* aC, const float* aR, float fl,
                                        float fr, int lane, int MX, int lMX, int jMX, float* out) {
    float lft = __shfl_up_sync(BW_FULL, v[S - 1], 1) * fl;
    float rgt = __shfl_down_sync(BW_FULL, v[0], 1) * fr;
    float hi = 0.f;
    if (PER) {
        float v1 = __shfl_sync(BW_FULL, v[0], 0);
        float vmx = __shfl_sync(BW_FULL, bw_pick<S>(v, jMX), lMX);
        if (lane == 0) lft = vmx * fl;
        hi = v1 * fr;
    } else if (lane == 0) lft = 0.f;
    const int x0 = lane * S + 1;
#pragma unroll
    for (int j = 0; j < S; j++) {
        float l = j == 0 ? lft : v[j - 1];
        float r = j == S - 1 ? rgt : v[j + 1];
        if (PER && x0 + j == MX) r = hi;
        out[j] = aL[j] * l + aC[j] * v[j] + aR[j] * r;
    }
}

__device__ __forceinline__ double bw_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(BW_FULL, v, o);
    return v;
}

template <int S>
__device__ __forceinline__ void bw_load(const float* __restrict__ p, int lane, float* v) {
#pragma unroll
    for (int j = 0; j < S; j++) v[j] = p[j * 32 + lane];
}
template <int S>
__device__ __forceinline__ void bw_store(float* __restrict__ p, int lane, const float* v) {
#pragma unroll
    for (int j = 0; j < S; j++) p[j * 32 + lane] = v[j];
}

template <int S, bool CURV>
__device__ void bw_phase(B1Prob& P, double* smd, float* smf) {
    const int lane = threadIdx.x & 31;
    const int MX = P.MX, M = P.M, ns = P.ns, nit = P.nit, n_mm = P.n_mm, iv = P.iv, m = P.m;
    const int b1 = P.b1, bm = P.bm;
    const int Wl = 32 * S;
    const int x0 = lane * S + 1;
    const int lMX = (MX - 1) / S, jMX = (MX - 1) % S;
    // shared: doubles then floats
    double* Aij = smd;                       // B1_MAXM^2
    double* Ci = Aij + B1_MAXM * B1_MAXM;    // B1_MAXM
    double* As = Ci + B1_MAXM;               // B1_MAXM*(B1_MAXM+1)
    double* sc = As + B1_MAXM * (B1_MAXM + 1);  // 5*NM_MAX_MOL
    double* spb = sc + 5 * NM_MAX_MOL;       // NM_MAX_SEG
    double* phif = spb + NM_MAX_SEG;         // NM_MAX_MOL
    double* gram = phif + NM_MAX_MOL;        // B1_MAXM
    int* phie = (int*)(gram + B1_MAXM);      // NM_MAX_MOL
    int* egs = phie + NM_MAX_MOL;            // NM_MAX_SEG
    float* G1s = smf;                        // ns*Wl (G1·2^-eg, lane layout)
    float* phis = G1s + ns * Wl;             // ns*Wl
    float* rhos = phis + ns * Wl;            // n_mm*Wl
    float* cLs = rhos + n_mm * Wl;           // Wl: stencil weights with the
    float* cCs = cLs + Wl;                   //     boundary folded in
    float* cRs = cCs + Wl;

    const float lam = (float)P.lam, lmid = 1.0f - 2.0f * (float)P.lam;
    float cm[S], c0[S], cp[S], ks[S];
#pragma unroll
    for (int j = 0; j < S; j++) {
        int xs = x0 + j;
        bool ok = xs <= MX;
        cm[j] = (CURV && ok) ? (float)P.lm1[xs] : 0.f;
        c0[j] = (CURV && ok) ? (float)P.l0[xs] : 0.f;
        cp[j] = (CURV && ok) ? (float)P.l1[xs] : 0.f;
        ks[j] = ok ? (float)P.ksam[xs] : 0.f;
    }
    // Boundary folded into the step weights: a 'surface' halo is a wall of
    // zero propagator (its weight drops); a mirror halo repeats the boundary
    // site (its weight joins the centre).  Periodic bounds keep both weights
    // and read the opposite end (bw_step<PER=true>).
    const bool per = (b1 == MX && bm == 1 && MX > 1);
#pragma unroll
    for (int j = 0; j < S; j++) {
        int xs = x0 + j;
        float wl, wc, wrr;
        if (CURV) { wl = cm[j]; wc = c0[j]; wrr = cp[j]; }
        else { wl = lam; wc = lmid; wrr = lam; }
        if (xs > MX) { wl = wc = wrr = 0.f; }
        if (xs == 1 && !per) { if (b1 == 1) wc += wl; wl = 0.f; }
        if (xs == MX && !per) { if (bm == MX) wc += wrr; wrr = 0.f; }
        cLs[j * 32 + lane] = wl; cCs[j * 32 + lane] = wc; cRs[j * 32 + lane] = wrr;
    }
    for (int i = lane; i < B1_MAXM * B1_MAXM; i += 32) Aij[i] = 0;
    double* __restrict__ x = P.x;
    double* __restrict__ g = P.g;
    int status = 0;
    int it = 0, k_diis = 0, fp32_its = 0, since_best = 0;
    double resid = 0, best = 1e300;
    bool handoff = false;
    __syncwarp();

    for (;;) {
        // ---------------- residual in FP32 ----------------
        // G1·2^-eg = 2^(-u·log2e - eg), eg = ceil(max(-u·log2e)) per segment
        for (int i = 0; i < ns; i++) {
            int itx = P.seg_it[i];
            float v[S];
            float vmax = -3.0e38f;
#pragma unroll
            for (int j = 0; j < S; j++) {
                int xs = x0 + j;
                bool ok = xs <= MX && P.gmask[i * M + (xs <= MX ? xs : 1)] != 0.0;
                v[j] = (itx >= 0 && xs <= MX) ? -(float)x[itx * M + xs] * 1.4426950408889634f : 0.f;
                if (ok) vmax = fmaxf(vmax, v[j]);
            }
            int key = __float_as_int(vmax);
            key = key >= 0 ? key : (key ^ 0x7fffffff);
            key = __reduce_max_sync(BW_FULL, key);
            key = key >= 0 ? key : (key ^ 0x7fffffff);
            float vm = __int_as_float(key);
            int e = vm > -1.0e30f ? (int)ceilf(vm) : 0;
            if (lane == 0) egs[i] = e;
#pragma unroll
            for (int j = 0; j < S; j++) {
                int xs = x0 + j;
                float gm = xs <= MX ? (float)P.gmask[i * M + xs] : 0.f;
                G1s[i * Wl + j * 32 + lane] = exp2f(v[j] - (float)e) * gm;
            }
        }
        for (int i = lane; i < n_mm * Wl; i += 32) rhos[i] = 0.f;
        __syncwarp();
        for (int mo = 0; mo < P.nmol; mo++) {
            const B1Mol& D = P.mol[mo];
            float* __restrict__ Gf = (float*)D.Gf;
            float* __restrict__ Pc = (float*)D.Pc;
            float* __restrict__ Qb = (float*)D.Q;
            int* __restrict__ ef = D.ef;    // [n_store][32] lane exponents of Gf
            int* __restrict__ epc = D.epc;  // [n_blocks][32] of Pc
            int* __restrict__ eqb = D.eq;   // [n_blocks][32] of Q
            // ---- forward sweep (post-order: children before parents) ----
            for (int b = 0; b < D.n_blocks; b++) {
                const nm_block B = D.blocks[b];
                const int eg = egs[B.seg];
                float wr[S], cur[S], nxt[S], t[S];
                bw_load<S>(G1s + B.seg * Wl, lane, wr);
                int s = B.s0, E;
                if (B.n_child == 0) {
#pragma unroll
                    for (int j = 0; j < S; j++) cur[j] = wr[j];
                    E = eg;
                    bw_lnorm<S>(cur, E);
                } else {
                    // join: G1 · P(Gf of the first child's end) · Π over the
                    // other children (and repeats) of P(Gf)·KSAM, in FP64
                    const int nc = B.n_child;
                    const int c0i = D.child_index[B.child0];
                    const nm_block C0 = D.blocks[c0i];
                    const bool simple = (nc == 1 && C0.mult == 1);
                    if (!simple) {
                        for (int c = 0; c < nc; c++) {
                            const int cb = D.child_index[B.child0 + c];
                            const nm_block Cb = D.blocks[cb];
                            const int sl = Cb.s0 + Cb.length - 1;
                            double td[S];
                            const int Er = bw_sten_lanes<S, CURV>(Gf + (size_t)sl * Wl, ef + sl * 32, lane, b1, bm, MX,
                                                                  lMX, jMX, lam, lmid, cm, c0, cp, td);
#pragma unroll
                            for (int j = 0; j < S; j++) td[j] *= (double)ks[j];
                            const int Eo = bw_lnorm_d<S>(td, Er, t);
                            bw_store<S>(Pc + (size_t)cb * Wl, lane, t);
                            epc[cb * 32 + lane] = Eo;
                        }
                        __syncwarp();
                    }
                    const int sl0 = C0.s0 + C0.length - 1;
                    double cd[S];
                    int Ed = bw_sten_lanes<S, CURV>(Gf + (size_t)sl0 * Wl, ef + sl0 * 32, lane, b1, bm, MX, lMX, jMX,
                                                    lam, lmid, cm, c0, cp, cd) + eg;
#pragma unroll
                    for (int j = 0; j < S; j++) cd[j] *= (double)wr[j];
                    if (!simple) {
                        for (int k = 1; k < C0.mult; k++) {
                            bw_load<S>(Pc + (size_t)c0i * Wl, lane, t);
#pragma unroll
                            for (int j = 0; j < S; j++) cd[j] *= (double)t[j];
                            Ed += epc[c0i * 32 + lane];
                        }
                        for (int c = 1; c < nc; c++) {
                            const int cb = D.child_index[B.child0 + c];
                            bw_load<S>(Pc + (size_t)cb * Wl, lane, t);
                            const int ec = epc[cb * 32 + lane];
                            for (int k = 0; k < D.blocks[cb].mult; k++) {
#pragma unroll
                                for (int j = 0; j < S; j++) cd[j] *= (double)t[j];
                                Ed += ec;
                            }
                        }
                    }
                    E = bw_lnorm_d<S>(cd, Ed, cur);
                }
                bw_store<S>(Gf + (size_t)s * Wl, lane, cur);
                ef[s * 32 + lane] = E;
                float fl, fr;
                bw_nbr(E, lane, lMX, per, fl, fr);
                float aL[S], aC[S], aR[S];
#pragma unroll
                for (int j = 0; j < S; j++) {
                    aL[j] = cLs[j * 32 + lane] * wr[j];
                    aC[j] = cCs[j * 32 + lane] * wr[j];
                    aR[j] = cRs[j * 32 + lane] * wr[j];
                }
                for (int k = 1; k < B.length; k++) {
                    s++;
                    if (per) bw_step<S, true>(cur, aL, aC, aR, fl, fr, lane, MX, lMX, jMX, nxt);
                    else bw_step<S, false>(cur, aL, aC, aR, fl, fr, lane, MX, lMX, jMX, nxt);
#pragma unroll
                    for (int j = 0; j < S; j++) cur[j] = nxt[j];
                    E += eg;
                    if ((k % BW_RS) == 0) {
                        bw_lnorm<S>(cur, E);
                        bw_nbr(E, lane, lMX, per, fl, fr);
                    }
                    bw_store<S>(Gf + (size_t)s * Wl, lane, cur);
                    ef[s * 32 + lane] = E;
                }
                __syncwarp();
            }
            // ---- G(N) = Σ_x L·Gf(root end), FP64 on the warp's common scale ----
            const nm_block Rb = D.blocks[D.n_blocks - 1];
            const int sroot = Rb.s0 + Rb.length - 1;
            int eroot;
            {
                const int El = ef[sroot * 32 + lane];
                eroot = __reduce_max_sync(BW_FULL, El);
                const double f = bw_p2d(El - eroot);
                double acc = 0;
#pragma unroll
                for (int j = 0; j < S; j++) {
                    int xs = x0 + j;
                    if (xs <= MX) {
                        double v = (double)Gf[(size_t)sroot * Wl + j * 32 + lane] * f;
                        acc += P.L ? v * P.L[xs] : v;
                    }
                }
                double GN = bw_sum(acc);
                if (lane == 0) { sc[5 * mo + 0] = GN; sc[5 * mo + 3] = (double)eroot; }
            }
            // ---- backward sweep (pre-order) fused with the composition ----
            int stack[B1_MAXB];
            int sp = 0;
            stack[sp++] = D.n_blocks - 1;
            while (sp > 0) {
                const int b = stack[--sp];
                const nm_block B = D.blocks[b];
                const int eg = egs[B.seg];
                float* rr = rhos + (D.mm0 + B.molmon) * Wl;
                const float d = (float)B.degeneracy;
                float wr[S], cur[S], nxt[S], acc[S], cmp[S], gfn[S];
                bw_load<S>(G1s + B.seg * Wl, lane, wr);
                int s = B.s0 + B.length - 1;
                int eb;
                if (B.parent < 0) {
#pragma unroll
                    for (int j = 0; j < S; j++) cur[j] = wr[j];
                    eb = eg;
                    bw_lnorm<S>(cur, eb);
                } else {
                    double td[S];
                    const int Er = bw_sten_lanes<S, CURV>(Qb + (size_t)b * Wl, eqb + b * 32, lane, b1, bm, MX, lMX,
                                                          jMX, lam, lmid, cm, c0, cp, td) + eg;
#pragma unroll
                    for (int j = 0; j < S; j++) td[j] *= (double)wr[j];
                    eb = bw_lnorm_d<S>(td, Er, cur);
                }
                float fl, fr;
                bw_nbr(eb, lane, lMX, per, fl, fr);
                // composition in the bounded form Gf·Gb/G1 (the reference divides
                // by G1 afterwards, system.cpp:2438); winv = d/(G1·2^-eg).  The
                // lane's scale 2^E, E = ef+eb-eroot-eg, is applied half to Gf
                // and half to Gb·winv so that no partial product leaves FP32.
                float winv[S];
#pragma unroll
                for (int j = 0; j < S; j++) winv[j] = wr[j] != 0.f ? d / wr[j] : 0.f;
                {
                    float gf0[S];
                    bw_load<S>(Gf + (size_t)s * Wl, lane, gf0);
                    const int E = ef[s * 32 + lane] + eb - eroot - eg, h = E >> 1;
                    const float sa = pow2f(h), sb = pow2f(E - h);
#pragma unroll
                    for (int j = 0; j < S; j++) { acc[j] = (gf0[j] * sa) * (cur[j] * winv[j] * sb); cmp[j] = 0.f; }
                }
                int efn = 0;
                if (s - 1 >= B.s0) { bw_load<S>(Gf + (size_t)(s - 1) * Wl, lane, gfn); efn = ef[(s - 1) * 32 + lane]; }
                float aL[S], aC[S], aR[S];
#pragma unroll
                for (int j = 0; j < S; j++) {
                    aL[j] = cLs[j * 32 + lane] * wr[j];
                    aC[j] = cCs[j * 32 + lane] * wr[j];
                    aR[j] = cRs[j * 32 + lane] * wr[j];
                }
                int kstep = 0;
                for (s = s - 1; s >= B.s0; s--) {
                    float gf[S];
#pragma unroll
                    for (int j = 0; j < S; j++) gf[j] = gfn[j];
                    const int efs = efn;
                    if (s - 1 >= B.s0) { bw_load<S>(Gf + (size_t)(s - 1) * Wl, lane, gfn); efn = ef[(s - 1) * 32 + lane]; }
                    if (per) bw_step<S, true>(cur, aL, aC, aR, fl, fr, lane, MX, lMX, jMX, nxt);
                    else bw_step<S, false>(cur, aL, aC, aR, fl, fr, lane, MX, lMX, jMX, nxt);
#pragma unroll
                    for (int j = 0; j < S; j++) cur[j] = nxt[j];
                    eb += eg;
                    if ((++kstep % BW_RS) == 0) {
                        bw_lnorm<S>(cur, eb);
                        bw_nbr(eb, lane, lMX, per, fl, fr);
                    }
                    const int E = efs + eb - eroot - eg, h = E >> 1;
                    const float sa = pow2f(h), sb = pow2f(E - h);
#pragma unroll
                    for (int j = 0; j < S; j++) {  // compensated sum
                        float y = (gf[j] * sa) * (cur[j] * winv[j] * sb) - cmp[j];
                        float t2 = acc[j] + y;
                        cmp[j] = (t2 - acc[j]) - y;
                        acc[j] = t2;
                    }
                }
#pragma unroll
                for (int j = 0; j < S; j++) rr[j * 32 + lane] += acc[j] - cmp[j];
                __syncwarp();
                if (B.n_child == 0) continue;
                // Q of each child: this block's first propagator times the other
                // children's P(Gf)·KSAM (and the repeats of its own), in FP64
                for (int c = 0; c < B.n_child; c++) {
                    const int cb = D.child_index[B.child0 + c];
                    const bool simple = (B.n_child == 1 && D.blocks[cb].mult == 1);
                    float q[S], t[S];
                    int eq = eb;
                    if (simple) {
#pragma unroll
                        for (int j = 0; j < S; j++) q[j] = cur[j];
                    } else {
                        double qd[S];
#pragma unroll
                        for (int j = 0; j < S; j++) qd[j] = (double)cur[j];
                        for (int k = 1; k < D.blocks[cb].mult; k++) {
                            bw_load<S>(Pc + (size_t)cb * Wl, lane, t);
#pragma unroll
                            for (int j = 0; j < S; j++) qd[j] *= (double)t[j];
                            eq += epc[cb * 32 + lane];
                        }
                        for (int o = 0; o < B.n_child; o++) {
                            if (o == c) continue;
                            const int ob = D.child_index[B.child0 + o];
                            bw_load<S>(Pc + (size_t)ob * Wl, lane, t);
                            const int eo = epc[ob * 32 + lane];
                            for (int k = 0; k < D.blocks[ob].mult; k++) {
#pragma unroll
                                for (int j = 0; j < S; j++) qd[j] *= (double)t[j];
                                eq += eo;
                            }
                        }
                        eq = bw_lnorm_d<S>(qd, eq, q);
                    }
                    bw_store<S>(Qb + (size_t)cb * Wl, lane, q);
                    eqb[cb * 32 + lane] = eq;
                }
                __syncwarp();
                for (int c = B.n_child - 1; c >= 0; c--) stack[sp++] = D.child_index[B.child0 + c];
            }
            __syncwarp();
        }
        // ---- normalisation (system.cpp:2368-2560), lane 0, FP64 ----
        if (lane == 0) {
            double Bsum = 0;
            for (int mo = 0; mo < P.nmol; mo++) {
                const B1Mol& D = P.mol[mo];
                double* s5 = sc + 5 * mo;
                double GNm = s5[0];
                int e = (int)s5[3];
                double GN = ldexp(GNm, e);
                double norm = 0, fac = 0;
                int pe = 0;
                s5[0] = GN;
                s5[2] = D.n_in; s5[3] = D.theta_in;
                if (D.freedom == NM_MOL_FREE) {
                    s5[4] = D.phibulk_in;
                    norm = D.phibulk_in / D.N;
                    s5[2] = norm * GN;
                    Bsum += D.phibulk_in;
                    fac = norm; pe = e;
                } else if (D.freedom == NM_MOL_RESTRICTED) {
                    if (GNm > 0) {
                        norm = D.n_in / GN;
                        fac = D.n_in / GNm;
                        if (D.pinned) s5[4] = 0;
                        else { s5[4] = D.N * norm; Bsum += s5[4]; }
                    } else if (status == 0) status = NM_ERR_GN;
                } else { s5[4] = 0; pe = e; }
                s5[1] = norm;
                phif[mo] = fac > 0 ? fac : 1.0;
                phie[mo] = pe;
            }
            if (P.solvent >= 0) {
                int sv = P.solvent;
                double* s5 = sc + 5 * sv;
                s5[4] = 1.0 - Bsum;
                if (s5[4] < 0 && status == 0) status = NM_ERR_NEG_SOLVENT;
                double norm = s5[4] / P.mol[sv].N;
                s5[2] = norm * s5[0];
                s5[3] = s5[2] * P.mol[sv].N;
                s5[1] = norm;
                phif[sv] = norm > 0 ? norm : 1.0;
            }
            for (int i = 0; i < ns; i++) spb[i] = 0;
            for (int k = 0; k < n_mm; k++) spb[P.mm_seg[k]] += P.mm_frac[k] * sc[5 * P.mm_mol[k] + 4];
        }
        status = __shfl_sync(BW_FULL, status, 0);
        __syncwarp();
        if (status) break;  // x untouched: the FP64 kernel re-evaluates it
        // ---- φ = rho/G1·norm (FP32), φ_tot ----
        float pt[S];
#pragma unroll
        for (int j = 0; j < S; j++) pt[j] = 0.f;
        for (int i = 0; i < ns; i++) {
            float ph[S];
#pragma unroll
            for (int j = 0; j < S; j++) {
                int xs = x0 + j;
                ph[j] = xs <= MX ? (float)P.phi_frozen[i * M + xs] : 0.f;
            }
            if (P.seg_frozen[i]) {
#pragma unroll
                for (int j = 0; j < S; j++) pt[j] += ph[j];
            }
            for (int k = 0; k < n_mm; k++) {
                if (P.mm_seg[k] != i) continue;
                int mo = P.mm_mol[k];
                float f = (float)ldexp(phif[mo], phie[mo]);
#pragma unroll
                for (int j = 0; j < S; j++) {
                    float v = rhos[k * Wl + j * 32 + lane] * f;
                    ph[j] += v;
                    pt[j] += v;
                }
            }
            bw_store<S>(phis + i * Wl, lane, ph);
        }
        __syncwarp();
        // ---- residual (Classical_residual), FP32 ----
        float al[S];
#pragma unroll
        for (int j = 0; j < S; j++) al[j] = 0.f;
        for (int i = 0; i < nit; i++) {
            float gi[S];
#pragma unroll
            for (int j = 0; j < S; j++) {
                int xs = x0 + j;
                gi[j] = xs <= MX ? (float)x[i * M + xs] : 0.f;
            }
            int r = P.it_seg[i];
            for (int k = 0; k < ns; k++) {
                float chi = (float)P.chi[r * ns + k];
                if (chi == 0.f) continue;
                float ph[S], ps[S], lo, hi;
                bw_load<S>(phis + k * Wl, lane, ph);
                bw_halos<S>(ph, b1, bm, MX, lMX, jMX, (float)P.phi_frozen[k * M], (float)P.phi_frozen[k * M + MX + 1],
                            lo, hi);
                bw_sten<S, CURV>(ph, lo, hi, lane, MX, lam, lmid, cm, c0, cp, ps);
                float pb = (float)spb[k];
#pragma unroll
                for (int j = 0; j < S; j++)
                    if (pt[j] > 0.f) gi[j] = gi[j] - chi * (ps[j] / pt[j] - pb);
            }
#pragma unroll
            for (int j = 0; j < S; j++) {
                al[j] += gi[j];
                int xs = x0 + j;
                if (xs <= MX) g[i * M + xs] = (double)gi[j];
            }
        }
        const float rinv = 1.0f / (float)nit;
        for (int i = 0; i < nit; i++) {
#pragma unroll
            for (int j = 0; j < S; j++) {
                int xs = x0 + j;
                if (xs <= MX) {
                    float a = al[j] * rinv;
                    float v = pt[j] > 0.f ? (float)g[i * M + xs] - a + 1.0f / pt[j] - 1.0f : 0.f;
                    g[i * M + xs] = (double)(v * ks[j]);
                }
            }
            if (lane == 0) { g[i * M] = 0; g[i * M + MX + 1] = 0; }
        }
        __syncwarp();
        fp32_its++;
        if (P.eval_only) break;
        // ---------------- DIIS (FP64, one warp) ----------------
        int k = it % m;
        double* __restrict__ xRk = P.xR + (size_t)k * iv;
        double* __restrict__ xxk = P.xx0 + (size_t)k * iv;
        // ‖g‖ first, so that a non-finite FP32 residual leaves x as it was
        double gsq = 0;
        for (int i = lane; i < iv; i += 32) {
            double gv = g[i];
            gsq = P.max_norm ? fmax(gsq, fabs(gv)) : gsq + gv * gv;
        }
        if (P.max_norm) {
            for (int o = 16; o > 0; o >>= 1) gsq = fmax(gsq, __shfl_xor_sync(BW_FULL, gsq, o));
            resid = gsq;
        } else resid = sqrt(bw_sum(gsq));
        if (!isfinite(resid)) { status = NM_ERR_NAN_DIIS; break; }
        for (int i = lane; i < iv; i += 32) {
            double xo = x[i];
            double xn = xo + (-P.dmax) * g[i];
            x[i] = xn;
            xRk[i] = xn;
            xxk[i] = xn - xo;
        }
        __syncwarp();
        if (it > 0) k_diis++;
        if (k_diis > 0) {
            int kd = k_diis > m ? m : k_diis;
            for (int i = 0; i < kd; i++) {
                int posi = k - kd + 1 + i;
                if (posi < 0) posi += m;
                const double* a = P.xx0 + (size_t)posi * iv;
                double acc = 0;
                for (int j = lane; j < iv; j += 32) acc += a[j] * xxk[j];
                acc = bw_sum(acc);
                if (lane == 0) gram[i] = acc;
            }
            __syncwarp();
            if (lane == 0) {
                if (k_diis > m)
                    for (int i = 1; i < m; i++)
                        for (int j = 1; j < m; j++) Aij[m * (i - 1) + j - 1] = Aij[m * i + j];
                for (int i = 0; i < kd; i++) Aij[i + m * (kd - 1)] = Aij[kd - 1 + m * i] = gram[i] + 1e-9;
            }
            __syncwarp();
            bool nan = false;
            for (int e = lane; e < kd * kd; e += 32) {
                int i = e / kd, j = e % kd;
                double v = Aij[j + m * i];
                if (v != v) nan = true;
                As[i * (kd + 1) + j] = v;
            }
            for (int i = lane; i < kd; i += 32) As[i * (kd + 1) + kd] = 1.0;
            nan = __any_sync(BW_FULL, nan);
            __syncwarp();
            if (nan) { status = NM_ERR_NAN_DIIS; break; }
            if (kd == 1) { if (lane == 0) Ci[0] = 1.0; }
            else warp_solve(As, Ci, kd);
            if (lane == 0) {
                double nC = 0;
                for (int i = 0; i < kd; i++) nC += Ci[i];
                for (int i = 0; i < kd; i++) {
                    Ci[i] = Ci[i] / nC;
                    if (Ci[i] != Ci[i]) status = NM_ERR_NAN_SVD;
                }
            }
            status = __shfl_sync(BW_FULL, status, 0);
            __syncwarp();
            if (status) break;
            for (int j = lane; j < iv; j += 32) {
                double v = 0;
                for (int i = 0; i < kd; i++) {
                    int posi = k - kd + 1 + i;
                    if (posi < 0) posi += m;
                    v += Ci[i] * P.xR[(size_t)posi * iv + j];
                }
                x[j] = v;
            }
            __syncwarp();
        }
        if (resid < 0.9 * best) { best = resid; since_best = 0; } else since_best++;
        if (resid <= P.sw_tol || (since_best > 25 && resid < 1e-2)) { handoff = true; break; }
        if (it >= P.itlim) break;
        it++;
    }
    if (lane == 0) {
        P.iterations = it;
        P.fp32_iterations = fp32_its;
        P.residual = resid;
        // An FP32 failure (G(N) <= 0, a non-finite residual or DIIS
        // matrix) is a failure of the reduced precision, not a verdict on
        // the problem: the FP64 kernel takes over from the current field
        // and reports its own status.
        P.handoff = ((handoff || status != 0) && !P.eval_only && it < P.itlim) ? 1 : 0;
        P.status = status ? status : NM_ERR_NOT_CONVERGED;
        for (int i = 0; i < 5 * P.nmol; i++) P.sc[i] = sc[i];
        for (int i = 0; i < ns; i++) P.seg_phibulk[i] = spb[i];
    }
}

}  // namespace nm
