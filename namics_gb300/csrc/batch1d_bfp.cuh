// FP32 phase of the batched 1-gradient solver: one residual evaluation
// g(x) with FP32 block-floating-point propagators, 128 threads per problem.
//
// Thread t owns the contiguous sites x = t·SP+1 .. t·SP+SP (SP = 1 to 4,
// so MX <= 512), kept in registers across the whole chain.  A propagation step
// is register arithmetic plus the two neighbour values of the thread's
// chunk: shuffles inside a warp, one shared-memory slot per warp edge across
// warps, with one block barrier per step (slots double-buffered by step
// parity, so a barrier per step is enough).
//
// Block floating point: each thread's SP values are FP32 mantissas with one
// power-of-two exponent E per thread, G(x) = v(x)·2^E.  A warp-wide or
// block-wide exponent is not enough for stretched chains: at a grafted
// brush's converged field the backward propagator near the wall is ~2^-240
// of its own maximum, far below FP32's range, while its product with the
// forward propagator there is exactly what the composition needs.  Over SP
// sites the range is a few binary orders, so mantissas stay well inside
// FP32.  Every BC_RS steps each thread rescales its chunk from its own
// maximum; a thread that holds only zeros then takes the largest exponent
// in the block, so that what flows in from a neighbour lands in range.  The
// neighbours' values enter scaled by fl = 2^(E_left-E), fr = 2^(E_right-E),
// refreshed after each rescale.
//
// Joins of branched chains multiply several propagators; they are formed in
// FP64 (a few operations per join, none per step).  G(N) is an FP64 sum on
// the block's common scale.  The composition accumulates Gf·Gb/G1 per site
// (Kahan-compensated FP32) with the scale applied in two halves so no
// partial product leaves FP32.  φ, the side stencil and the residual are
// then evaluated in FP64 from the FP32 ρ (b1_finish), which removes FP32
// rounding from the residual algebra; what remains is the propagators'
// rounding, ~1e-7 relative per step.
#pragma once

#define BC_NT 128
#define BC_NW 4
#define BC_RS 4
#define BC_EMPTY (-0x7fffffff - 1)
#define BC_FULL 0xffffffffu

namespace nm {

// shared exchange slots, double-buffered by step parity
struct BcX {
    float vL[2][BC_NW], vR[2][BC_NW], vP[2][2];  // warp edge values; site 1 and site MX
    int eM[2][BC_NW];                            // warp max exponent of non-empty threads
    int eL[2][BC_NW], eR[2][BC_NW], eP[2][2];    // edge threads' exponents (before adoption)
    int fL[2][BC_NW], fR[2][BC_NW], fP[2][2];    // edge threads empty?
    double dL[BC_NW], dR[BC_NW], dP[2];          // FP64 edge values (join stencils)
    int iw[BC_NW];
    double dw[BC_NW];
};

// per-thread scale state of the vector being propagated
struct BcV {
    int E;        // exponent of the thread's chunk
    bool emp;     // chunk all zero at the last rescale
    bool resc;    // rescaled since the last exchange: neighbours' factors stale
    float fl, fr;
};

template <int S, typename T>
__device__ __forceinline__ T bc_pick(const T* v, int j) {
    T t = 0;
#pragma unroll
    for (int q = 0; q < S; q++)
        if (q == j) t = v[q];
    return t;
}

// 2^e in FP64 for |e| <= 1022 (0 below)
__device__ __forceinline__ double bc_p2d(int e) {
    e = e > 1023 ? 1023 : e;
    return e < -1022 ? 0.0 : __longlong_as_double((long long)(1023 + e) << 52);
}

__device__ __forceinline__ int bc_max_i(int v, BcX& X) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int m = __reduce_max_sync(BC_FULL, v);
    __syncthreads();
    if (lane == 0) X.iw[w] = m;
    __syncthreads();
    int r = X.iw[0];
#pragma unroll
    for (int i = 1; i < BC_NW; i++) r = max(r, X.iw[i]);
    return r;
}

__device__ __forceinline__ double bc_max_d(double v, BcX& X) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(BC_FULL, v, o));
    __syncthreads();
    if (lane == 0) X.dw[w] = v;
    __syncthreads();
    double r = X.dw[0];
#pragma unroll
    for (int i = 1; i < BC_NW; i++) r = fmax(r, X.dw[i]);
    return r;
}

// fixed-order block sum (deterministic)
__device__ __forceinline__ double bc_sum_d(double v, BcX& X) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(BC_FULL, v, o);
    __syncthreads();
    if (lane == 0) X.dw[w] = v;
    __syncthreads();
    double r = 0;
#pragma unroll
    for (int i = 0; i < BC_NW; i++) r += X.dw[i];
    return r;
}

// 2^e for e <= 127, subnormal powers included, 0 below 2^-149; selects
// only (no branches in the step loops)
__device__ __forceinline__ float bc_p2f(int e) {
    const int bits = e >= -126 ? (e + 127) << 23 : (e >= -149 ? 1 << max(e + 149, 0) : 0);
    return __int_as_float(bits);
}

// Scale the chunk to a maximum in [0.5, 1); its empty flag and the
// neighbour factors are settled at the next exchange.
template <int SP>
__device__ __forceinline__ void bc_lnorm(float* v, BcV& st) {
    float lm = 0.f;
#pragma unroll
    for (int j = 0; j < SP; j++) lm = fmaxf(lm, v[j]);
    const int e = expo(lm);
    const float f = bc_p2f(-e);
#pragma unroll
    for (int j = 0; j < SP; j++) v[j] *= f;
    st.E += e;
    st.emp = !(lm > 0.f);
    st.resc = true;
}

// The same from an FP64 chunk with exponent Ein.
template <int SP>
__device__ __forceinline__ void bc_lnorm_d(const double* v, int Ein, float* out, BcV& st) {
    double lm = 0.0;
#pragma unroll
    for (int j = 0; j < SP; j++) lm = fmax(lm, v[j]);
    const int e = lm > 0.0 ? (int)((__double_as_longlong(lm) >> 52) & 0x7ff) - 1022 : 0;
    const double f = __longlong_as_double((long long)(1023 - e) << 52);  // 2^-e
#pragma unroll
    for (int j = 0; j < SP; j++) out[j] = (float)(v[j] * f);
    st.E = Ein + e;
    st.emp = !(lm > 0.0);
    st.resc = true;
}

// thread geometry
struct BcG {
    int t, lane, w, wl, wr, x0, MX, tMX, jMX, b1, bm;  // wl, wr: neighbouring warps (clamped)
    bool per;
};

// One propagation step with its neighbour exchange.  Publish the chunk's
// edge values (and, after a rescale, the edge threads' exponents) into the
// slots of parity `par`, one block barrier, then settle a pending rescale
// (RESC: empty threads adopt the block's largest exponent, neighbour factors
// recomputed) and step: cur ← aL·v(x-1) + aC·v(x) + aR·v(x+1), the boundary
// folded into the per-site weights (which include G1).
template <int SP, bool PER, bool RESC>
__device__ __forceinline__ void bc_xs(float* cur, const float* aL, const float* aC, const float* aR, const BcG& G,
                                      BcV& st, int& par, BcX& X) {
    if (G.lane == 0) X.vL[par][G.w] = cur[0];
    if (G.lane == 31) X.vR[par][G.w] = cur[SP - 1];
    if (PER) {
        if (G.t == 0) X.vP[par][0] = cur[0];
        if (G.t == G.tMX) X.vP[par][1] = bc_pick<SP>(cur, G.jMX);
    }
    if (RESC) {
        const int em = __reduce_max_sync(BC_FULL, st.emp ? BC_EMPTY : st.E);
        if (G.lane == 0) { X.eM[par][G.w] = em; X.eL[par][G.w] = st.E; X.fL[par][G.w] = st.emp; }
        if (G.lane == 31) { X.eR[par][G.w] = st.E; X.fR[par][G.w] = st.emp; }
        if (PER) {
            if (G.t == 0) { X.eP[par][0] = st.E; X.fP[par][0] = st.emp; }
            if (G.t == G.tMX) { X.eP[par][1] = st.E; X.fP[par][1] = st.emp; }
        }
    }
    __syncthreads();
    if (RESC) {
        int Em = X.eM[par][0];
#pragma unroll
        for (int i = 1; i < BC_NW; i++) Em = max(Em, X.eM[par][i]);
        const bool any = Em != BC_EMPTY;
        if (st.emp && any) st.E = Em;
        int El = __shfl_up_sync(BC_FULL, st.E, 1);
        int Er = __shfl_down_sync(BC_FULL, st.E, 1);
        const int eR = (X.fR[par][G.wl] && any) ? Em : X.eR[par][G.wl];
        const int eL = (X.fL[par][G.wr] && any) ? Em : X.eL[par][G.wr];
        if (G.lane == 0) El = G.w > 0 ? eR : (PER ? ((X.fP[par][1] && any) ? Em : X.eP[par][1]) : st.E);
        if (G.lane == 31) Er = G.w < BC_NW - 1 ? eL : st.E;
        if (PER && G.t == G.tMX) Er = (X.fP[par][0] && any) ? Em : X.eP[par][0];
        st.fl = bc_p2f(min(El - st.E, 127));
        st.fr = bc_p2f(min(Er - st.E, 127));
        st.resc = false;
    }
    float lft = __shfl_up_sync(BC_FULL, cur[SP - 1], 1);
    float rgt = __shfl_down_sync(BC_FULL, cur[0], 1);
    const float a = X.vR[par][G.wl], b = X.vL[par][G.wr];
    if (G.lane == 0) lft = G.w > 0 ? a : (PER ? X.vP[par][1] : 0.f);
    if (G.lane == 31) rgt = G.w < BC_NW - 1 ? b : 0.f;
    lft *= st.fl;
    rgt *= st.fr;
    float nx[SP];
#pragma unroll
    for (int j = 0; j < SP; j++) {
        const float l = j == 0 ? lft : cur[j - 1];
        const float r = j == SP - 1 ? rgt : cur[j + 1];
        nx[j] = aL[j] * l + aC[j] * cur[j] + aR[j] * r;
    }
    if (PER && G.t == G.tMX) {  // right of site MX is site 1
        const float hi = X.vP[par][0] * st.fr;
#pragma unroll
        for (int j = 0; j < SP; j++)
            if (j == G.jMX) nx[j] = aL[j] * (j == 0 ? lft : cur[j - 1]) + aC[j] * cur[j] + aR[j] * hi;
    }
#pragma unroll
    for (int j = 0; j < SP; j++) cur[j] = nx[j];
    par ^= 1;
}

// Neighbour sum of a stored block-floating-point vector (p: mantissas in the
// thread layout, pe: exponents), in FP64 on the block's common scale:
// out·2^(return value) = Σ_k λ_k v(x+k), halos as set_bounds fills them
// (lattice.cpp:94-196) with a 'surface' halo holding 0.
template <int SP, bool CURV>
__device__ int bc_sten_lanes(const float* __restrict__ p, const int* __restrict__ pe, const BcG& G, double lam,
                             double lmid, const B1Prob& P, BcX& X, double* out) {
    float v[SP];
    float lm = 0.f;
#pragma unroll
    for (int j = 0; j < SP; j++) { v[j] = p[j * BC_NT + G.t]; lm = fmaxf(lm, v[j]); }
    const int El = pe[G.t];
    int Eref = bc_max_i(lm > 0.f ? El : BC_EMPTY, X);
    if (Eref == BC_EMPTY) Eref = 0;
    const double f = lm > 0.f ? bc_p2d(El - Eref) : 0.0;
    double d[SP];
#pragma unroll
    for (int j = 0; j < SP; j++) d[j] = (double)v[j] * f;
    if (G.lane == 0) X.dL[G.w] = d[0];
    if (G.lane == 31) X.dR[G.w] = d[SP - 1];
    if (G.t == 0) X.dP[0] = d[0];
    if (G.t == G.tMX) X.dP[1] = bc_pick<SP>(d, G.jMX);
    __syncthreads();
    double lft = __shfl_up_sync(BC_FULL, d[SP - 1], 1);
    double rgt = __shfl_down_sync(BC_FULL, d[0], 1);
    const double v1 = X.dP[0], vmx = X.dP[1];
    const double lo = G.b1 == 0 ? 0.0 : (G.b1 == 1 ? v1 : vmx);
    const double hi = G.bm == G.MX + 1 ? 0.0 : (G.bm == G.MX ? vmx : v1);
    if (G.lane == 0) lft = G.w > 0 ? X.dR[G.w - 1] : lo;
    if (G.lane == 31) rgt = G.w < BC_NW - 1 ? X.dL[G.w + 1] : 0.0;
#pragma unroll
    for (int j = 0; j < SP; j++) {
        const int xs = G.x0 + j;
        double l = j == 0 ? lft : d[j - 1];
        double r = j == SP - 1 ? rgt : d[j + 1];
        if (xs == G.MX) r = hi;
        double o;
        if (CURV) o = xs <= G.MX ? d[j] * P.l0[xs] + l * P.lm1[xs] + r * P.l1[xs] : 0.0;
        else o = lam * l + lmid * d[j] + lam * r;
        out[j] = xs <= G.MX ? o : 0.0;
    }
    __syncthreads();  // slots free for the next user
    return Eref;
}

// Rows of a stored vector for the next BC_RS backward steps (segments
// s, s-1, ..., s-BC_RS+1; those below s_lo are left as zero), loaded a whole
// group ahead so the loads overlap a group of steps.
template <int SP>
__device__ __forceinline__ void bc_rows(const float* __restrict__ Gf, const int* __restrict__ ef, int s, int s_lo,
                                        int Wl, int t, float (&r)[BC_RS][SP], int (&e)[BC_RS]) {
#pragma unroll
    for (int i = 0; i < BC_RS; i++) {
        const int si = s - i;
        const bool ok = si >= s_lo;
#pragma unroll
        for (int j = 0; j < SP; j++) r[i][j] = ok ? Gf[(size_t)si * Wl + j * BC_NT + t] : 0.f;
        e[i] = ok ? ef[si * BC_NT + t] : 0;
    }
}

// composition of one segment: acc += Gf·Gb/G1·d on the thread's scale
// 2^E, E = ef + eb - (eroot + eg), applied half to each factor
template <int SP>
__device__ __forceinline__ void bc_comp(const float* gf, int efs, const float* cur, const float* winv, int eb,
                                        int ebase, float* acc, float* cmp) {
    const int E = efs + eb - ebase, h = E >> 1;
    const float sa = bc_p2f(min(h, 127)), sb = bc_p2f(min(E - h, 127));
#pragma unroll
    for (int j = 0; j < SP; j++) {  // compensated sum
        const float y = (gf[j] * sa) * (cur[j] * winv[j] * sb) - cmp[j];
        const float t2 = acc[j] + y;
        cmp[j] = (t2 - acc[j]) - y;
        acc[j] = t2;
    }
}

// One residual evaluation with FP32 block-floating-point propagators.
// Shared memory (from S.uni, thread layout j·128 + t, each element touched
// by its own thread only): G1s [ns][Wl] = G1·2^-eg, rhos [n_mm][Wl], and the
// per-site step weights cLs/cCs/cRs [Wl] with the boundary folded in.
template <int SP, bool CURV, bool PER>
__device__ void bc_residual(B1Prob& P, const Lat1 L, const Coef<double> C64, B1S& S, BcX& X,
                            const double* __restrict__ x, double* __restrict__ g) {
    const int MX = L.MX, M = L.M, ns = P.ns, n_mm = P.n_mm;
    const int Wl = BC_NT * SP;
    BcG G;
    G.t = threadIdx.x; G.lane = G.t & 31; G.w = G.t >> 5; G.x0 = G.t * SP + 1; G.MX = MX;
    G.wl = G.w > 0 ? G.w - 1 : 0; G.wr = G.w < BC_NW - 1 ? G.w + 1 : BC_NW - 1;
    G.tMX = (MX - 1) / SP; G.jMX = (MX - 1) % SP; G.b1 = L.b1; G.bm = L.bm;
    G.per = PER;
    const int t = G.t;
    float* G1s = (float*)S.uni;
    float* rhos = G1s + ns * Wl;
    float* cLs = rhos + n_mm * Wl;
    float* cCs = cLs + Wl;
    float* cRs = cCs + Wl;
    const float lam = (float)P.lam, lmid = 1.0f - 2.0f * (float)P.lam;
    const double lamd = P.lam, lmidd = 1.0 - 2.0 * P.lam;
#pragma unroll
    for (int j = 0; j < SP; j++) {
        const int xs = G.x0 + j;
        const bool ok = xs <= MX;
        // boundary folded into the step weights: a 'surface' halo is a wall
        // of zero propagator (its weight drops), a mirror halo repeats the
        // boundary site (its weight joins the centre); periodic bounds keep
        // both and read the opposite end
        float wl = lam, wc = lmid, wrr = lam;
        if (CURV && ok) { wl = (float)P.lm1[xs]; wc = (float)P.l0[xs]; wrr = (float)P.l1[xs]; }
        if (!ok) wl = wc = wrr = 0.f;
        if (xs == 1 && !PER) { if (G.b1 == 1) wc += wl; wl = 0.f; }
        if (xs == MX && !PER) { if (G.bm == MX) wc += wrr; wrr = 0.f; }
        cLs[j * BC_NT + t] = wl; cCs[j * BC_NT + t] = wc; cRs[j * BC_NT + t] = wrr;
    }
    // G1·2^-eg = 2^(-u·log2e - eg), eg = ceil(max over the segment's sites);
    // the exponent is split into integer and fraction in FP64 so the FP32
    // value carries a relative error of one exp2f rounding only
    for (int i = 0; i < ns; i++) {
        const int itx = P.seg_it[i];
        double dv[SP];
        double vmax = -1.0e300;
#pragma unroll
        for (int j = 0; j < SP; j++) {
            const int xs = G.x0 + j;
            const bool in = xs <= MX;
            dv[j] = (itx >= 0 && in) ? -x[itx * M + xs] * 1.4426950408889634 : 0.0;
            if (in && P.gmask[i * M + xs] != 0.0) vmax = fmax(vmax, dv[j]);
        }
        const double vm = bc_max_d(vmax, X);
        const int eg = vm > -1.0e299 ? (int)ceil(vm) : 0;
        if (t == 0) S.eg[i] = eg;
#pragma unroll
        for (int j = 0; j < SP; j++) {
            const int xs = G.x0 + j;
            const double gm = xs <= MX ? P.gmask[i * M + xs] : 0.0;
            float v = 0.f;
            if (gm != 0.0) {
                const double y = dv[j] - (double)eg;
                const double ip = floor(y);
                v = exp2f((float)(y - ip)) * bc_p2f((int)ip) * (float)gm;
            }
            G1s[i * Wl + j * BC_NT + t] = v;
        }
    }
    for (int k = 0; k < n_mm; k++)
#pragma unroll
        for (int j = 0; j < SP; j++) rhos[k * Wl + j * BC_NT + t] = 0.f;
    __syncthreads();  // S.eg
    int par = 0;
    for (int mo = 0; mo < P.nmol; mo++) {
        const B1Mol& D = P.mol[mo];
        float* __restrict__ Gf = (float*)D.Gf;
        float* __restrict__ Pc = (float*)D.Pc;
        float* __restrict__ Qb = (float*)D.Q;
        int* __restrict__ ef = D.ef;    // [n_store][128] thread exponents of Gf
        int* __restrict__ epc = D.epc;  // [n_blocks][128]
        int* __restrict__ eqb = D.eq;   // [n_blocks][128]
        // ---- forward sweep (post-order: children before parents) ----
        for (int b = 0; b < D.n_blocks; b++) {
            const nm_block B = D.blocks[b];
            const int eg = S.eg[B.seg];
            float wr[SP], cur[SP], tv[SP];
#pragma unroll
            for (int j = 0; j < SP; j++) wr[j] = G1s[B.seg * Wl + j * BC_NT + t];
            BcV st;
            st.fl = st.fr = 1.f;
            if (B.n_child == 0) {
#pragma unroll
                for (int j = 0; j < SP; j++) cur[j] = wr[j];
                st.E = eg;
                bc_lnorm<SP>(cur, st);
            } else {
                // join (mol_branched.cpp:170-230): G1 · P(Gf of the first
                // child's end) · Π over the other children (and repeats) of
                // P(Gf)·KSAM, in FP64
                const int nc = B.n_child;
                const int c0i = D.child_index[B.child0];
                const nm_block C0 = D.blocks[c0i];
                const bool simple = (nc == 1 && C0.mult == 1);
                if (!simple) {
                    for (int c = 0; c < nc; c++) {
                        const int cb = D.child_index[B.child0 + c];
                        const nm_block Cb = D.blocks[cb];
                        const int sl = Cb.s0 + Cb.length - 1;
                        double td[SP];
                        const int Er = bc_sten_lanes<SP, CURV>(Gf + (size_t)sl * Wl, ef + sl * BC_NT, G, lamd, lmidd,
                                                               P, X, td);
#pragma unroll
                        for (int j = 0; j < SP; j++) td[j] *= G.x0 + j <= MX ? P.ksam[G.x0 + j] : 0.0;
                        BcV so;
                        bc_lnorm_d<SP>(td, Er, tv, so);
#pragma unroll
                        for (int j = 0; j < SP; j++) Pc[(size_t)cb * Wl + j * BC_NT + t] = tv[j];
                        epc[cb * BC_NT + t] = so.E;
                    }
                }
                const int sl0 = C0.s0 + C0.length - 1;
                double cd[SP];
                int Ed = bc_sten_lanes<SP, CURV>(Gf + (size_t)sl0 * Wl, ef + sl0 * BC_NT, G, lamd, lmidd, P, X, cd) + eg;
#pragma unroll
                for (int j = 0; j < SP; j++) cd[j] *= (double)wr[j];
                if (!simple) {
                    for (int k = 1; k < C0.mult; k++) {
#pragma unroll
                        for (int j = 0; j < SP; j++) cd[j] *= (double)Pc[(size_t)c0i * Wl + j * BC_NT + t];
                        Ed += epc[c0i * BC_NT + t];
                    }
                    for (int c = 1; c < nc; c++) {
                        const int cb = D.child_index[B.child0 + c];
#pragma unroll
                        for (int j = 0; j < SP; j++) tv[j] = Pc[(size_t)cb * Wl + j * BC_NT + t];
                        const int ec = epc[cb * BC_NT + t];
                        for (int k = 0; k < D.blocks[cb].mult; k++) {
#pragma unroll
                            for (int j = 0; j < SP; j++) cd[j] *= (double)tv[j];
                            Ed += ec;
                        }
                    }
                }
                bc_lnorm_d<SP>(cd, Ed, cur, st);
            }
            float* __restrict__ gp = Gf + (size_t)B.s0 * Wl + t;
            int* __restrict__ ep = ef + B.s0 * BC_NT + t;
#pragma unroll
            for (int j = 0; j < SP; j++) gp[j * BC_NT] = cur[j];
            *ep = st.E;
            float aL[SP], aC[SP], aR[SP];
#pragma unroll
            for (int j = 0; j < SP; j++) {
                aL[j] = cLs[j * BC_NT + t] * wr[j];
                aC[j] = cCs[j * BC_NT + t] * wr[j];
                aR[j] = cRs[j * BC_NT + t] * wr[j];
            }
            // steps k = 1 .. length-1 in groups of BC_RS: the group's first
            // step settles the rescale that ended the previous group
            int k = 1;
            for (; k + BC_RS <= B.length; k += BC_RS) {
#pragma unroll
                for (int i = 0; i < BC_RS; i++) {
                    if (i == 0) bc_xs<SP, PER, true>(cur, aL, aC, aR, G, st, par, X);
                    else bc_xs<SP, PER, false>(cur, aL, aC, aR, G, st, par, X);
                    st.E += eg;
                    if (i == BC_RS - 1) bc_lnorm<SP>(cur, st);
                    gp += Wl;
                    ep += BC_NT;
#pragma unroll
                    for (int j = 0; j < SP; j++) gp[j * BC_NT] = cur[j];
                    *ep = st.E;
                }
            }
            for (; k < B.length; k++) {
                if (st.resc) bc_xs<SP, PER, true>(cur, aL, aC, aR, G, st, par, X);
                else bc_xs<SP, PER, false>(cur, aL, aC, aR, G, st, par, X);
                st.E += eg;
                gp += Wl;
                ep += BC_NT;
#pragma unroll
                for (int j = 0; j < SP; j++) gp[j * BC_NT] = cur[j];
                *ep = st.E;
            }
        }
        // ---- G(N) = Σ_x L·Gf(root end), FP64 on the block's common scale ----
        const nm_block Rb = D.blocks[D.n_blocks - 1];
        const int sroot = Rb.s0 + Rb.length - 1;
        int eroot;
        {
            float v[SP];
            float lm = 0.f;
#pragma unroll
            for (int j = 0; j < SP; j++) { v[j] = Gf[(size_t)sroot * Wl + j * BC_NT + t]; lm = fmaxf(lm, v[j]); }
            const int El = ef[sroot * BC_NT + t];
            eroot = bc_max_i(lm > 0.f ? El : BC_EMPTY, X);
            if (eroot == BC_EMPTY) eroot = 0;
            const double f = lm > 0.f ? bc_p2d(El - eroot) : 0.0;
            double acc = 0;
#pragma unroll
            for (int j = 0; j < SP; j++) {
                const int xs = G.x0 + j;
                if (xs <= MX) {
                    const double vv = (double)v[j] * f;
                    acc += P.L ? vv * P.L[xs] : vv;
                }
            }
            const double GN = bc_sum_d(acc, X);
            if (t == 0) { S.sc[5 * mo + 0] = GN; S.sc[5 * mo + 3] = (double)eroot; }
        }
        // ---- backward sweep (pre-order) fused with the composition ----
        const int ebase0 = eroot;
        int stack[B1_MAXB];
        int sp = 0;
        stack[sp++] = D.n_blocks - 1;
        while (sp > 0) {
            const int b = stack[--sp];
            const nm_block B = D.blocks[b];
            const int eg = S.eg[B.seg];
            const int ebase = ebase0 + eg;
            float* rr = rhos + (D.mm0 + B.molmon) * Wl;
            const float d = (float)B.degeneracy;
            float wr[SP], cur[SP], acc[SP], cmp[SP];
#pragma unroll
            for (int j = 0; j < SP; j++) wr[j] = G1s[B.seg * Wl + j * BC_NT + t];
            const int top = B.s0 + B.length - 1;
            BcV st;
            st.fl = st.fr = 1.f;
            if (B.parent < 0) {
#pragma unroll
                for (int j = 0; j < SP; j++) cur[j] = wr[j];
                st.E = eg;
                bc_lnorm<SP>(cur, st);
            } else {
                double td[SP];
                const int Er = bc_sten_lanes<SP, CURV>(Qb + (size_t)b * Wl, eqb + b * BC_NT, G, lamd, lmidd, P, X, td) + eg;
#pragma unroll
                for (int j = 0; j < SP; j++) td[j] *= (double)wr[j];
                bc_lnorm_d<SP>(td, Er, cur, st);
            }
            // composition in the bounded form Gf·Gb/G1 (the reference divides
            // by G1 afterwards, system.cpp:2438); winv = d/(G1·2^-eg)
            float winv[SP];
#pragma unroll
            for (int j = 0; j < SP; j++) {
                winv[j] = wr[j] != 0.f ? d / wr[j] : 0.f;
                acc[j] = 0.f;
                cmp[j] = 0.f;
            }
            {
                float gf0[SP];
#pragma unroll
                for (int j = 0; j < SP; j++) gf0[j] = Gf[(size_t)top * Wl + j * BC_NT + t];
                bc_comp<SP>(gf0, ef[top * BC_NT + t], cur, winv, st.E, ebase, acc, cmp);
            }
            float aL[SP], aC[SP], aR[SP];
#pragma unroll
            for (int j = 0; j < SP; j++) {
                aL[j] = cLs[j * BC_NT + t] * wr[j];
                aC[j] = cCs[j * BC_NT + t] * wr[j];
                aR[j] = cRs[j * BC_NT + t] * wr[j];
            }
            // steps k = 1 .. length-1 (segments top-1 down to s0) in groups of
            // BC_RS; each group's stored Gf rows were loaded a group earlier
            const int nsteps = B.length - 1;
            float rows[BC_RS][SP];
            int erows[BC_RS];
            bc_rows<SP>(Gf, ef, top - 1, B.s0, Wl, t, rows, erows);
            int k = 0, s = top - 1;
            for (; k + BC_RS <= nsteps; k += BC_RS, s -= BC_RS) {
                float nrows[BC_RS][SP];
                int nerows[BC_RS];
                bc_rows<SP>(Gf, ef, s - BC_RS, B.s0, Wl, t, nrows, nerows);
#pragma unroll
                for (int i = 0; i < BC_RS; i++) {
                    if (i == 0) bc_xs<SP, PER, true>(cur, aL, aC, aR, G, st, par, X);
                    else bc_xs<SP, PER, false>(cur, aL, aC, aR, G, st, par, X);
                    st.E += eg;
                    if (i == BC_RS - 1) bc_lnorm<SP>(cur, st);
                    bc_comp<SP>(rows[i], erows[i], cur, winv, st.E, ebase, acc, cmp);
                }
#pragma unroll
                for (int i = 0; i < BC_RS; i++) {
                    erows[i] = nerows[i];
#pragma unroll
                    for (int j = 0; j < SP; j++) rows[i][j] = nrows[i][j];
                }
            }
#pragma unroll
            for (int i = 0; i < BC_RS; i++) {  // remainder: fewer than BC_RS steps, no rescale
                if (k + i < nsteps) {
                    if (st.resc) bc_xs<SP, PER, true>(cur, aL, aC, aR, G, st, par, X);
                    else bc_xs<SP, PER, false>(cur, aL, aC, aR, G, st, par, X);
                    st.E += eg;
                    bc_comp<SP>(rows[i], erows[i], cur, winv, st.E, ebase, acc, cmp);
                }
            }
#pragma unroll
            for (int j = 0; j < SP; j++) rr[j * BC_NT + t] += acc[j] - cmp[j];
            if (B.n_child == 0) continue;
            // Q of each child: this block's first propagator times the other
            // children's P(Gf)·KSAM (and the repeats of its own), in FP64
            for (int c = 0; c < B.n_child; c++) {
                const int cb = D.child_index[B.child0 + c];
                const bool simple = (B.n_child == 1 && D.blocks[cb].mult == 1);
                float q[SP], tv[SP];
                int eq = st.E;
                if (simple) {
#pragma unroll
                    for (int j = 0; j < SP; j++) q[j] = cur[j];
                } else {
                    double qd[SP];
#pragma unroll
                    for (int j = 0; j < SP; j++) qd[j] = (double)cur[j];
                    for (int kk = 1; kk < D.blocks[cb].mult; kk++) {
#pragma unroll
                        for (int j = 0; j < SP; j++) qd[j] *= (double)Pc[(size_t)cb * Wl + j * BC_NT + t];
                        eq += epc[cb * BC_NT + t];
                    }
                    for (int o = 0; o < B.n_child; o++) {
                        if (o == c) continue;
                        const int ob = D.child_index[B.child0 + o];
#pragma unroll
                        for (int j = 0; j < SP; j++) tv[j] = Pc[(size_t)ob * Wl + j * BC_NT + t];
                        const int eo = epc[ob * BC_NT + t];
                        for (int kk = 0; kk < D.blocks[ob].mult; kk++) {
#pragma unroll
                            for (int j = 0; j < SP; j++) qd[j] *= (double)tv[j];
                            eq += eo;
                        }
                    }
                    BcV so;
                    bc_lnorm_d<SP>(qd, eq, q, so);
                    eq = so.E;
                }
#pragma unroll
                for (int j = 0; j < SP; j++) Qb[(size_t)cb * Wl + j * BC_NT + t] = q[j];
                eqb[cb * BC_NT + t] = eq;
            }
            for (int c = B.n_child - 1; c >= 0; c--) stack[sp++] = D.child_index[B.child0 + c];
        }
    }
    // ρ to the natural layout in FP64, then the shared FP64 tail
    double* rho = S.rho;
    for (int k = 0; k < n_mm; k++) {
#pragma unroll
        for (int j = 0; j < SP; j++) {
            const int xs = G.x0 + j;
            if (xs <= MX) rho[k * M + xs] = (double)rhos[k * Wl + j * BC_NT + t];
        }
        if (t == 0) { rho[k * M] = 0.0; rho[k * M + MX + 1] = 0.0; }
    }
    __syncthreads();
    b1_finish<true>(P, L, C64, S, x, g);
}

}  // namespace nm
