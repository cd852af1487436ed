/*
 * CPU oracle for the Namics SCF hot path — TEST INFRASTRUCTURE ONLY
 * (see scf_oracle.h).  A restatement of the reference algorithm in plain C.
 * Each function names the reference code it follows (file:line into
 * leermakers/Namics src/).  Arrays use the reference's padded flat layout
 * and its flat-array stencil semantics (neighbour sums taken over the whole
 * array, halo layers refreshed by set_bounds before each use), so halo
 * contents evolve exactly as in the reference.
 */
#include "scf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

struct orc_state {
    const nm_plan* P;
    int M;
    int BX1, BXM, BY1, BYM, BZ1, BZM;
    double *u, *G1, *phi, *phi_side, *phitot, *alpha, *tmp, *unity;
    double *mol_phitot;
    double **Gf, **rho, **jGb, **Pc, **Qb;
    double *gb;
    double *gb3;                        /* Markov 2: the backward pair, 3 directions each */
    double *m2l1, *m2l11, *m2l_1, *m2l_11; /* Markov 2, curved lattices: LGrad1.cpp:63-68 */
    double *GN, *norm, *mol_n, *mol_theta, *mol_phibulk, *seg_phibulk;
    double *psi, *EE, *q, *eps, *X;  /* electrostatics (charged systems) */
    /* internal states: u and α of each state [n_state*M]; the species'
     * bulk fractions [n_sp]; phi and phi_side hold n_sp rows, the states'
     * volume fractions after the segments'; in_mol: the segment occurs in
     * a molecule (SysMonList) */
    double *ust, *ast, *sp_phibulk;
    int *in_mol;
    /* the states' bulk fractions and the molecules' bulk charges in force
     * (the plan's, until orc_set_states changes them) */
    double *st_ab, *mol_charge;
    int have_state;
    /* molecule amounts in force (the plan's, until orc_set_amount changes
     * them, as a Variate scan or search step does) and a search's inner
     * tolerance (> 0 overrides the plan's) */
    double *amt_n, *amt_theta, *amt_phibulk;
    double tol_override;
};

/* ---- L0 primitives (tools_host.h:185-470) ------------------------------ */
static void Zero(double* P, int M) { memset(P, 0, sizeof(double) * (size_t)M); }
static void Cp(double* P, const double* A, int M) { memcpy(P, A, sizeof(double) * (size_t)M); }
static void Times(double* P, const double* A, const double* B, int M) { for (int i = 0; i < M; i++) P[i] = A[i] * B[i]; }
static void AddTimes(double* P, const double* A, const double* B, int M) { for (int i = 0; i < M; i++) P[i] += A[i] * B[i]; }
static void YplusisCtimesX(double* Y, const double* X, double C, int M) { for (int i = 0; i < M; i++) Y[i] += C * X[i]; }
static void Add(double* P, const double* A, int M) { for (int i = 0; i < M; i++) P[i] += A[i]; }
static void Norm(double* P, double C, int M) { for (int i = 0; i < M; i++) P[i] *= C; }
static double Sum(const double* X, int M) { double s = 0; for (int i = 0; i < M; i++) s += X[i]; return s; }
static double Dot(const double* X, const double* Y, int M) { double s = 0; for (int i = 0; i < M; i++) s += X[i] * Y[i]; return s; }
static void Div(double* P, const double* A, int M) { for (int i = 0; i < M; i++) { if (A[i] != 0) P[i] /= A[i]; else P[i] = 0; } }

/* internal states: a segment with states (Segment::ns > 1) and χ between
 * interaction species (segments, then states) */
static int has_states(const nm_plan* P, int i) { return P->n_state > 0 && P->seg_nstate[i] > 0; }
static double chi_of(const nm_plan* P, int a, int b) {
    return P->n_state > 0 ? P->chi_sp[(size_t)a * P->n_sp + b] : P->chi[(size_t)a * P->n_seg + b];
}

/* ---- boundaries -------------------------------------------------------- */
/* Halo source layers per boundary type (lattice.cpp:94-196, fjc = 1). */
static void bc_sources(orc_state* st) {
    const nm_plan* P = st->P;
    int n[3] = {P->MX, P->MY, P->MZ};
    int lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
        int bl = P->bc[d], bh = P->bc[d + 3];
        lo[d] = bl == NM_BC_MIRROR ? 1 : bl == NM_BC_PERIODIC ? n[d] : 0;
        hi[d] = bh == NM_BC_MIRROR ? n[d] : bh == NM_BC_PERIODIC ? 1 : n[d] + 1;
    }
    st->BX1 = lo[0]; st->BXM = hi[0];
    st->BY1 = lo[1]; st->BYM = hi[1];
    st->BZ1 = lo[2]; st->BZM = hi[2];
}

/* LGrad1.cpp:806-818, LGrad2.cpp:1652-1680, LGrad3.cpp:1549-1616 */
static void set_bounds(orc_state* st, double* X) {
    const nm_plan* P = st->P;
    int MX = P->MX, MY = P->MY, MZ = P->MZ, JX = P->JX, JY = P->JY;
    int BX1 = st->BX1, BXM = st->BXM, BY1 = st->BY1, BYM = st->BYM, BZ1 = st->BZ1, BZM = st->BZM;
    if (P->gradients == 1) {
        X[0] = X[BX1];
        X[MX + 1] = X[BXM];
    } else if (P->gradients == 2) {
        for (int x = 1; x < MX + 1; x++) { X[x * JX + 0] = X[x * JX + BY1]; X[x * JX + MY + 1] = X[x * JX + BYM]; }
        for (int y = 1; y < MY + 1; y++) { X[0 + y] = X[BX1 * JX + y]; X[(MX + 1) * JX + y] = X[BXM * JX + y]; }
        X[0] = X[BY1];
        X[MY + 1] = X[BYM];
        X[(MX + 1) * JX + 0] = X[(MX + 1) * JX + BY1];
        X[(MX + 1) * JX + MY + 1] = X[(MX + 1) * JX + BYM];
    } else {
        int x, y, z;
        for (x = 1; x < MX + 1; x++) for (y = 1; y < MY + 1; y++) {
            X[x * JX + y * JY + 0] = X[x * JX + y * JY + BZ1];
            X[x * JX + y * JY + MZ + 1] = X[x * JX + y * JY + BZM];
        }
        for (y = 1; y < MY + 1; y++) for (z = 1; z < MZ + 1; z++) {
            X[0 + y * JY + z] = X[BX1 * JX + y * JY + z];
            X[(MX + 1) * JX + y * JY + z] = X[BXM * JX + y * JY + z];
        }
        for (z = 1; z < MZ + 1; z++) for (x = 1; x < MX + 1; x++) {
            X[x * JX + 0 + z] = X[x * JX + BY1 * JY + z];
            X[x * JX + (MY + 1) * JY + z] = X[x * JX + BYM * JY + z];
        }
        x = 0;
        for (y = 1; y < MY + 1; y++) { X[y * JY + 0] = X[y * JY + BZ1]; X[y * JY + MZ + 1] = X[y * JY + BZM]; }
        for (z = 1; z < MZ + 1; z++) { X[0 + z] = X[BY1 * JY + z]; X[(MY + 1) * JY + z] = X[BYM * JY + z]; }
        x = MX + 1;
        for (y = 1; y < MY + 1; y++) { X[x * JX + y * JY + 0] = X[x * JX + y * JY + BZ1]; X[x * JX + y * JY + MZ + 1] = X[x * JX + y * JY + BZM]; }
        for (z = 1; z < MZ + 1; z++) { X[x * JX + 0 + z] = X[x * JX + BY1 * JY + z]; X[x * JX + (MY + 1) * JY + z] = X[x * JX + BYM * JY + z]; }
        y = 0;
        for (x = 1; x < MX + 1; x++) { X[x * JX + 0] = X[x * JX + BZ1]; X[x * JX + MZ + 1] = X[x * JX + BZM]; }
        y = MY + 1;
        for (x = 1; x < MX + 1; x++) { X[x * JX + y * JY + 0] = X[x * JX + y * JY + BZ1]; X[x * JX + y * JY + MZ + 1] = X[x * JX + y * JY + BZM]; }
        X[0] = X[BX1 * JX + BY1 * JY + BZ1];
        X[(MX + 1) * JX] = X[BXM * JX + BY1 * JY + BZ1];
        X[(MY + 1) * JY] = X[BX1 * JX + BYM * JY + BZ1];
        X[MZ + 1] = X[BX1 * JX + BY1 * JY + BZM];
        X[(MX + 1) * JX + (MY + 1) * JY] = X[BXM * JX + BYM * JY + BZ1];
        X[(MX + 1) * JX + MZ + 1] = X[BXM * JX + BY1 * JY + BZM];
        X[(MY + 1) * JY + MZ + 1] = X[BX1 * JX + BYM * JY + BZM];
        X[(MX + 1) * JX + (MY + 1) * JY + MZ + 1] = X[BXM * JX + BYM * JY + BZM];
    }
}

/* LGrad1.cpp:787-798, LGrad2.cpp remove_bounds, LGrad3.cpp:1521-1545 */
static void remove_bounds(orc_state* st, double* X) {
    const nm_plan* P = st->P;
    int MX = P->MX, MY = P->MY, MZ = P->MZ, JX = P->JX, JY = P->JY;
    if (P->gradients == 1) { X[0] = 0; X[MX + 1] = 0; return; }
    if (P->gradients == 2) {
        for (int x = 0; x < MX + 2; x++) { X[x * JX] = 0; X[x * JX + MY + 1] = 0; }
        for (int y = 0; y < MY + 2; y++) { X[y] = 0; X[(MX + 1) * JX + y] = 0; }
        return;
    }
    for (int y = 0; y < MY + 2; y++) for (int z = 0; z < MZ + 2; z++) { X[y * JY + z] = 0; X[(MX + 1) * JX + y * JY + z] = 0; }
    for (int x = 0; x < MX + 2; x++) for (int z = 0; z < MZ + 2; z++) { X[x * JX + z] = 0; X[x * JX + (MY + 1) * JY + z] = 0; }
    for (int x = 0; x < MX + 2; x++) for (int y = 0; y < MY + 2; y++) { X[x * JX + y * JY] = 0; X[x * JX + y * JY + MZ + 1] = 0; }
}

/* WeightedSum: LGrad1.cpp:213-221, LGrad2.cpp:147-157, LGrad3.cpp:40-46 */
static double weighted_sum(orc_state* st, double* X) {
    const nm_plan* P = st->P;
    remove_bounds(st, X);
    if (P->gradients == 3 || P->geometry == NM_PLANAR) return Sum(X, st->M);
    return Dot(X, P->L, st->M);
}

/* ---- stencils ------------------------------------------------------------
 * stencil(): the neighbour sum of Lattice::Side / Lattice::propagate, added
 * into a zeroed gs (LG1Planar.cpp:28-55,138-159; LGrad1.cpp:251-281,432-454;
 * LG2Planar.cpp:27-135,1039-1127; LGrad2.cpp:207-278,1053-1090;
 * LGrad3.cpp:103-243,673-782).  side != 0 picks the Side() operation order. */
static void stencil(orc_state* st, double* gs, const double* g, int side) {
    const nm_plan* P = st->P;
    int M = st->M, JX = P->JX, JY = P->JY;
    double lam = P->lambda;
    Zero(gs, M);
    if (P->gradients == 1) {
        if (P->geometry == NM_PLANAR) {
            if (side) {
                YplusisCtimesX(gs + 1, g, lam, M - 1);
                YplusisCtimesX(gs, g + 1, lam, M - 1);
                YplusisCtimesX(gs, g, 1.0 - 2.0 * lam, M);
            } else {
                YplusisCtimesX(gs + 1, g, lam, M - 1);
                YplusisCtimesX(gs, g, 1.0 - 2.0 * lam, M);
                YplusisCtimesX(gs, g + 1, lam, M - 1);
            }
        } else {
            AddTimes(gs, g, P->lambda0, M);
            AddTimes(gs + 1, g, P->lambda_1 + 1, M - 1);
            AddTimes(gs, g + 1, P->lambda1, M - 1);
        }
        return;
    }
    if (P->gradients == 2) {
        if (P->geometry == NM_PLANAR) {
            if (P->lattice_type == NM_SIMPLE_CUBIC) {
                double C1 = 16.0 / 36.0, C2 = 4.0 / 36.0, C3 = 1.0 / 36.0;
                YplusisCtimesX(gs, g, C1, M);
                YplusisCtimesX(gs + 1, g, C2, M - 1);
                YplusisCtimesX(gs, g + 1, C2, M - 1);
                YplusisCtimesX(gs + JX, g, C2, M - JX);
                YplusisCtimesX(gs, g + JX, C2, M - JX);
                YplusisCtimesX(gs + JX + 1, g, C3, M - JX - 1);
                YplusisCtimesX(gs + JX, g + 1, C3, M - JX);
                YplusisCtimesX(gs + 1, g + JX, C3, M - JX);
                YplusisCtimesX(gs, g + JX + 1, C3, M - JX - 1);
            } else {
                double Two = 2.0, C = 1.0 / 16.0;
                YplusisCtimesX(gs, g, Two, M);
                Add(gs + JX, g, M - JX);
                Add(gs, g + JX, M - JX);
                Add(gs + JY, g, M - JY);
                Add(gs, g + JY, M - JY);
                Norm(gs, Two, M);
                Add(gs + JX + JY, g, M - JX - JY);
                Add(gs, g + JX + JY, M - JX - JY);
                Add(gs + JX, g + JY, M - JX - JY);
                Add(gs + JY, g + JX, M - JX - JY);
                Norm(gs, C, M);
            }
        } else {
            double C1, C2, C3;
            if (P->lattice_type == NM_SIMPLE_CUBIC) { C1 = 4.0 / 6.0; C2 = 1.0 / 6.0; C3 = 4.0; }
            else { C1 = 0.5; C2 = 0.25; C3 = 2.0; }
            const double *l_1 = P->lambda_1, *l1 = P->lambda1;
            YplusisCtimesX(gs, g, C1, M);
            AddTimes(gs + JX, g, l_1 + JX, M - JX);
            AddTimes(gs, g + JX, l1, M - JX);
            YplusisCtimesX(gs + 1, g, C2, M - 1);
            YplusisCtimesX(gs, g + 1, C2, M - 1);
            Norm(gs, C3, M);
            AddTimes(gs + JX + 1, g, l_1 + JX + 1, M - JX - 1);
            AddTimes(gs + JX, g + 1, l_1 + JX, M - JX - 1);
            AddTimes(gs + 1, g + JX, l1 + 1, M - JX - 1);
            AddTimes(gs, g + JX + 1, l1, M - JX - 1);
            Norm(gs, C2, M);
        }
        return;
    }
    /* 3 gradients, stencil_full */
    if (P->lattice_type == NM_SIMPLE_CUBIC) {
        Add(gs + JX, g, M - JX);
        Add(gs, g + JX, M - JX);
        Add(gs + JY, g, M - JY);
        Add(gs, g + JY, M - JY);
        Add(gs + 1, g, M - 1);
        Add(gs, g + 1, M - 1);
        Norm(gs, 1.0 / 6.0, M);
    } else {
        double Two = 2.0, C = 1.0 / 40.0;
        YplusisCtimesX(gs, g, Two, M);
        Add(gs + JX, g, M - JX);
        Add(gs, g + JX, M - JX);
        Add(gs + JY, g, M - JY);
        Add(gs, g + JY, M - JY);
        Add(gs + 1, g, M - 1);
        Add(gs, g + 1, M - 1);
        Norm(gs, Two, M);
        Add(gs + JX + JY, g, M - JX - JY);
        Add(gs, g + JX + JY, M - JX - JY);
        Add(gs + JX, g + JY, M - JX - JY);
        Add(gs + JY, g + JX, M - JX - JY);
        Add(gs + JX + 1, g, M - JX - 1);
        Add(gs + 1, g + JX, M - JX - 1);
        Add(gs + JY + 1, g, M - JY - 1);
        Add(gs + 1, g + JY, M - JY - 1);
        Add(gs + JX, g + 1, M - JX - 1);
        Add(gs, g + JX + 1, M - JX - 1);
        Add(gs + JY, g + 1, M - JY - 1);
        Add(gs, g + JY + 1, M - JY - 1);
        Norm(gs, Two, M);
        Add(gs + JX + JY + 1, g, M - JX - JY - 1);
        Add(gs, g + JX + JY + 1, M - JX - JY - 1);
        Add(gs + JX + JY, g + 1, M - JX - JY - 1);
        Add(gs + 1, g + JX + JY, M - JX - JY - 1);
        Add(gs + JX + 1, g + JY, M - JX - JY - 1);
        Add(gs + JY, g + JX + 1, M - JX - JY - 1);
        Add(gs + JY + 1, g + JX, M - JX - JY - 1);
        Add(gs + JX, g + JY + 1, M - JX - JY - 1);
        Norm(gs, C, M);
    }
}

/* Lattice::propagate: Zero(gs); set_bounds(gs_1); stencil; Times(gs,G1). */
static void propagate(orc_state* st, double* gs, double* gs_1, const double* G1) {
    set_bounds(st, gs_1);
    stencil(st, gs, gs_1, 0);
    Times(gs, gs, G1, st->M);
}

void orc_propagate(orc_state* st, double* G_in, const double* G1, double* G_out) {
    propagate(st, G_out, G_in, G1 ? G1 : st->unity);
}

void orc_side(orc_state* st, double* X, double* X_side) { stencil(st, X_side, X, 1); }

/* ---- molecules ----------------------------------------------------------- */
static int blk_last(const nm_block* B) { return B->s0 + B->length - 1; }

/* Forward propagators of one molecule (Molecule::propagate_forward,
 * molecule.cpp:2300-2362; joins as mol_branched.cpp:250-299 and
 * mol_dendrimer.cpp:113-146).  A block's first segment joins its children:
 * Gf = P(Gf[child_0])*G1 * prod_c [P(Gf[c])*UNITY]^(mult-...) . */
static void mol_forward(orc_state* st, int m) {
    const nm_plan* P = st->P;
    const nm_molecule* mol = &P->mols[m];
    int M = st->M;
    double* Gf = st->Gf[m];
    for (int b = 0; b < mol->n_blocks; b++) {
        const nm_block* B = &mol->blocks[b];
        const double* G1 = st->G1 + (size_t)B->seg * M;
        int s = B->s0;
        if (B->n_child == 0) {
            Cp(Gf + (size_t)s * M, G1, M);  /* Initiate (LGrad1.cpp:943-949) */
        } else {
            /* every child's end propagator, once with UNITY, cached for the
             * backward pass */
            for (int c = 0; c < B->n_child; c++) {
                int cb = mol->child_index[B->child0 + c];
                propagate(st, st->Pc[m] + (size_t)cb * M, Gf + (size_t)blk_last(&mol->blocks[cb]) * M, st->unity);
            }
            int c0 = mol->child_index[B->child0];
            const nm_block* C0 = &mol->blocks[c0];
            double* out = Gf + (size_t)s * M;
            propagate(st, out, Gf + (size_t)blk_last(C0) * M, G1);
            for (int k = 1; k < C0->mult; k++) Times(out, out, st->Pc[m] + (size_t)c0 * M, M);
            for (int c = 1; c < B->n_child; c++) {
                int cb = mol->child_index[B->child0 + c];
                for (int k = 0; k < mol->blocks[cb].mult; k++) Times(out, out, st->Pc[m] + (size_t)cb * M, M);
            }
        }
        for (int k = 1; k < B->length; k++) {
            s++;
            propagate(st, Gf + (size_t)s * M, Gf + (size_t)(s - 1) * M, G1);
        }
    }
    /* GN = ComputeGN(G_root) (LGrad1.cpp:863-874): WeightedSum, which clears
     * the halo of the stored end propagator as a side effect. */
    const nm_block* R = &mol->blocks[mol->n_blocks - 1];
    st->GN[m] = weighted_sum(st, Gf + (size_t)blk_last(R) * M);
}

/* AddPhiS (LGrad1.cpp:876-922): rho += d*Gf*Gb */
static void add_phi(double* rho, const double* Gf, const double* Gb, double d, int M) {
    if (d == 1.0) AddTimes(rho, Gf, Gb, M);
    else for (int i = 0; i < M; i++) rho[i] += d * Gf[i] * Gb[i];
}

/* Backward sweep of block b starting from Q (NULL for the root block):
 * Molecule::propagate_backward (molecule.cpp:2364-2446), with the branch
 * logic of mol_branched.cpp:170-248 and mol_dendrimer.cpp:148-184. */
static void mol_backward_block(orc_state* st, int m, int b, double* Q) {
    const nm_plan* P = st->P;
    const nm_molecule* mol = &P->mols[m];
    const nm_block* B = &mol->blocks[b];
    int M = st->M;
    const double* G1 = st->G1 + (size_t)B->seg * M;
    double* rho = st->rho[m] + (size_t)B->molmon * M;
    double* Gf = st->Gf[m];
    double *cur = st->gb, *nxt = st->gb + M;
    int s = blk_last(B);
    if (!Q) Cp(cur, G1, M);
    else propagate(st, cur, Q, G1);
    add_phi(rho, Gf + (size_t)s * M, cur, B->degeneracy, M);
    for (s = s - 1; s >= B->s0; s--) {
        propagate(st, nxt, cur, G1);
        double* t = cur; cur = nxt; nxt = t;
        add_phi(rho, Gf + (size_t)s * M, cur, B->degeneracy, M);
    }
    if (B->n_child == 0) return;
    double* jg = st->jGb[m] + (size_t)b * M;
    Cp(jg, cur, M);
    for (int c = 0; c < B->n_child; c++) {
        int cb = mol->child_index[B->child0 + c];
        double* q = st->Qb[m] + (size_t)cb * M;
        Cp(q, jg, M);
        for (int k = 1; k < mol->blocks[cb].mult; k++) Times(q, q, st->Pc[m] + (size_t)cb * M, M);
        for (int o = 0; o < B->n_child; o++) {
            if (o == c) continue;
            int ob = mol->child_index[B->child0 + o];
            for (int k = 0; k < mol->blocks[ob].mult; k++) Times(q, q, st->Pc[m] + (size_t)ob * M, M);
        }
        mol_backward_block(st, m, cb, q);
    }
}

/* ---- Markov 2 (semiflexible) chains, 1-gradient simple-cubic lattices ----
 * Every propagator of such a molecule holds FJC = 3 direction components
 * d = 0, 1, 2 of the bond that arrives at a site (down, lateral, up; the
 * lateral one stands for 4 of the 6 simple-cubic directions).  The bond-angle
 * weights P[k] (angles k·π/2) are the plan's `bend`.  LG1Planar.cpp:57-135
 * (planar) and LGrad1.cpp:285-429 (curved) for the steps; LGrad1.cpp:863-960
 * for G(N), AddPhiS and Initiate; molecule.cpp:2448-2615 and
 * mol_linear.cpp:115-129 for the sweeps of a linear chain (every propagator
 * stored, no ring). */
#define M2_FJC 3

/* set_bounds of a direction pair (LGrad1.cpp:787-804, fjc = 1): the halo of
 * one direction takes the other's boundary value, a reflected bond */
static void m2_bounds_pair(orc_state* st, double* X, double* Y) {
    int MX = st->P->MX;
    X[0] = Y[st->BX1];
    X[MX + 1] = Y[st->BXM];
    Y[0] = X[st->BX1];
    Y[MX + 1] = X[st->BXM];
}

/* One step gs <- gs_1: forward (LG1Planar::propagateF, LGrad1::propagateF)
 * or backward (propagateB), simple cubic, fjc = 1. */
static void m2_propagate(orc_state* st, double* gs, double* gs_1, const double* G1, const double* P, int fwd) {
    int M = st->M;
    Zero(gs, M2_FJC * M);
    m2_bounds_pair(st, gs_1, gs_1 + 2 * M);
    set_bounds(st, gs_1 + M);
    double *gz0 = gs_1, *gz1 = gs_1 + M, *gz2 = gs_1 + 2 * M;
    double *gx0 = gs, *gx1 = gs + M, *gx2 = gs + 2 * M;
    if (st->P->geometry == NM_PLANAR) {
        if (fwd) {
            YplusisCtimesX(gx0 + 1, gz0, P[0], M - 1);
            YplusisCtimesX(gx0 + 1, gz1, 4 * P[1], M - 1);
            YplusisCtimesX(gx1, gz0, P[1], M);
            YplusisCtimesX(gx1, gz1, 2 * P[1] + P[0], M);
            YplusisCtimesX(gx1, gz2, P[1], M);
            YplusisCtimesX(gx2, gz1 + 1, 4 * P[1], M - 1);
            YplusisCtimesX(gx2, gz2 + 1, P[0], M - 1);
        } else {
            YplusisCtimesX(gx0, gz0 + 1, P[0], M - 1);
            YplusisCtimesX(gx0, gz1, 4 * P[1], M);
            YplusisCtimesX(gx1, gz0 + 1, P[1], M - 1);
            YplusisCtimesX(gx1, gz1, 2 * P[1] + P[0], M);
            YplusisCtimesX(gx1 + 1, gz2, P[1], M - 1);
            YplusisCtimesX(gx2, gz1, 4 * P[1], M);
            YplusisCtimesX(gx2 + 1, gz2, P[0], M - 1);
        }
    } else {
        const double *l1 = st->m2l1, *l11 = st->m2l11, *l_1 = st->m2l_1, *l_11 = st->m2l_11;
        double* H = st->tmp;
        if (fwd) {
            Times(H, l_1 + 1, gz0, M - 1);
            AddTimes(H, l_11 + 1, gz2 + 1, M - 1);
            YplusisCtimesX(gx0 + 1, H, P[0], M - 1);
            Times(H, l_1 + 1, gz1, M - 1);
            AddTimes(H, l_11 + 1, gz1 + 1, M - 1);
            YplusisCtimesX(gx0 + 1, H, 4 * P[1], M - 1);
            YplusisCtimesX(gx1, gz0, P[1], M);
            YplusisCtimesX(gx1, gz1, 2 * P[1] + P[0], M);
            YplusisCtimesX(gx1, gz2, P[1], M);
            Times(H + 1, l1, gz1 + 1, M - 1);
            AddTimes(H + 1, l11, gz1, M - 1);
            YplusisCtimesX(gx2, H + 1, 4 * P[1], M - 1);
            Times(H + 1, l1, gz2 + 1, M - 1);
            AddTimes(H + 1, l11, gz0, M - 1);
            YplusisCtimesX(gx2, H + 1, P[0], M - 1);
        } else {
            Times(H, l_1 + 1, gz2, M - 1);
            AddTimes(H, l_11 + 1, gz0 + 1, M - 1);
            YplusisCtimesX(gx1 + 1, H, P[1], M - 1);
            YplusisCtimesX(gx2 + 1, H, P[0], M - 1);
            YplusisCtimesX(gx0, gz1, 4 * P[1], M);
            YplusisCtimesX(gx1, gz1, 2 * P[1] + P[0], M);
            YplusisCtimesX(gx2, gz1, 4 * P[1], M);
            Times(H + 1, l1, gz0 + 1, M - 1);
            AddTimes(H + 1, l11, gz2, M - 1);
            YplusisCtimesX(gx0, H + 1, P[0], M - 1);
            YplusisCtimesX(gx1, H + 1, P[1], M - 1);
        }
    }
    for (int k = 0; k < M2_FJC; k++) Times(gs + k * M, gs + k * M, G1, M);
}

/* Initiate (LGrad1.cpp:943-949): every direction starts from Gz */
static void m2_initiate(double* G, const double* Gz, int M) {
    for (int k = 0; k < M2_FJC; k++) Cp(G + k * M, Gz, M);
}

/* AddPhiS (LGrad1.cpp:876-905, simple cubic): rho += Σ_d C_d·Gf_d·Gb_d */
static void m2_add_phi(double* rho, const double* Gf, const double* Gb, int M) {
    const double C1 = 1.0 / 6.0, C2 = 4.0 / 6.0;
    for (int i = 0; i < M; i++) rho[i] += C1 * Gf[i] * Gb[i];
    for (int i = 0; i < M; i++) rho[i] += C2 * Gf[M + i] * Gb[M + i];
    for (int i = 0; i < M; i++) rho[i] += C1 * Gf[2 * M + i] * Gb[2 * M + i];
}

/* Both sweeps of a Markov 2 linear chain (mol_linear.cpp:115-129 without a
 * ring, molecule.cpp:2448-2615 without save_memory): the forward sweep
 * stores every Gf(s); G(N) = Σ_d w_d·WeightedSum(Gf(N-1)_d)/6 with w = 1, 4,
 * 1 (LGrad1.cpp:863-874); the backward sweep from Initiate(G1) at the last
 * segment, AddPhiS at every s. */
static void m2_compose(orc_state* st, int m) {
    const nm_molecule* mol = &st->P->mols[m];
    int M = st->M, N = mol->n_store;
    double* Gf = st->Gf[m];
    const double* P = mol->bend;
    int s = 0;
    for (int b = 0; b < mol->n_blocks; b++) {
        const nm_block* B = &mol->blocks[b];
        const double* G1 = st->G1 + (size_t)B->seg * M;
        for (int k = 0; k < B->length; k++, s++) {
            if (s > 0) m2_propagate(st, Gf + (size_t)s * M2_FJC * M, Gf + (size_t)(s - 1) * M2_FJC * M, G1, P, 1);
            else m2_initiate(Gf, G1, M);
        }
    }
    double* last = Gf + (size_t)(N - 1) * M2_FJC * M;
    double GN = weighted_sum(st, last);
    GN += 4.0 * weighted_sum(st, last + M);
    GN += weighted_sum(st, last + 2 * M);
    st->GN[m] = GN / 6.0;
    s = N - 1;
    double* gb = st->gb3;
    for (int b = mol->n_blocks - 1; b >= 0; b--) {
        const nm_block* B = &mol->blocks[b];
        const double* G1 = st->G1 + (size_t)B->seg * M;
        double* rho = st->rho[m] + (size_t)B->molmon * M;
        for (int k = 0; k < B->length; k++, s--) {
            double* cur = gb + (size_t)(s % 2) * M2_FJC * M;
            if (s < N - 1) m2_propagate(st, cur, gb + (size_t)((s + 1) % 2) * M2_FJC * M, G1, P, 0);
            else m2_initiate(cur, G1, M);
            m2_add_phi(rho, Gf + (size_t)s * M2_FJC * M, cur, M);
        }
    }
}

/* ---- electrostatics (charged systems) ------------------------------------
 * Constants of namics.cpp:44-49; the lattice routines of LG1Planar.cpp:162-200,
 * LGrad1.cpp:593-680 and 820-833, LG2Planar.cpp:1130-1175, LGrad2.cpp:
 * 1392-1440 and 1702-1740 (fjc = 1; the fixed-ψ0 branches are not covered). */
#define ORC_E 1.60217e-19
#define ORC_KBT (1.38065e-23 * 298.15)
#define ORC_EPS0 8.85418e-12
#define ORC_PIE 3.14159265

/* mirror bounds on every side */
static void set_M_bounds(orc_state* st, double* X) {
    const nm_plan* P = st->P;
    int MX = P->MX;
    if (P->gradients == 1) { X[0] = X[1]; X[MX + 1] = X[MX]; return; }
    if (P->gradients == 3) {  /* LGrad3.cpp:1679-1702: the faces only */
        int MY = P->MY, MZ = P->MZ, JX = P->JX, JY = P->JY;
        for (int x = 1; x < MX + 1; x++) for (int y = 1; y < MY + 1; y++) {
            X[x * JX + y * JY + 0] = X[x * JX + y * JY + 1];
            X[x * JX + y * JY + MZ + 1] = X[x * JX + y * JY + MZ];
        }
        for (int y = 1; y < MY + 1; y++) for (int z = 1; z < MZ + 1; z++) {
            X[0 + y * JY + z] = X[1 * JX + y * JY + z];
            X[(MX + 1) * JX + y * JY + z] = X[MX * JX + y * JY + z];
        }
        for (int z = 1; z < MZ + 1; z++) for (int x = 1; x < MX + 1; x++) {
            X[x * JX + 0 + z] = X[x * JX + 1 * JY + z];
            X[x * JX + (MY + 1) * JY + z] = X[x * JX + MY * JY + z];
        }
        return;
    }
    int MY = P->MY, JX = P->JX;
    for (int x = 1; x < MX + 1; x++) { X[x * JX + 0] = X[x * JX + 1]; X[x * JX + MY + 1] = X[x * JX + MY]; }
    for (int y = 1; y < MY + 1; y++) { X[0 + y] = X[1 * JX + y]; X[(MX + 1) * JX + y] = X[MX * JX + y]; }
    X[0] = X[1]; X[MY + 1] = X[MY];
    X[(MX + 1) * JX + 0] = X[(MX + 1) * JX + 1]; X[(MX + 1) * JX + MY + 1] = X[(MX + 1) * JX + MY];
}

/* EE: the field-energy density weight of each site (Lattice::UpdateEE) */
static void update_EE(orc_state* st, double* EE, double* psi) {
    const nm_plan* P = st->P;
    int M = st->M, MX = P->MX;
    double pf = 0.5 * ORC_EPS0 * P->bond_length / ORC_KBT * (ORC_KBT / ORC_E) * (ORC_KBT / ORC_E);
    const double* L = P->L;
    set_M_bounds(st, psi);
    Zero(EE, M);
    if (P->gradients == 1) {
        if (P->geometry == NM_PLANAR) {
            pf = pf / 2.0 * 1 * 1;
            double Exmin, Explus = psi[0] - psi[1];
            Explus *= Explus;
            for (int x = 1; x < MX + 1; x++) {
                Exmin = Explus;
                Explus = psi[x] - psi[x + 1];
                Explus *= Explus;
                EE[x] = pf * (Exmin + Explus);
            }
        } else if (P->geometry == NM_CYLINDRICAL) {
            int r = (int)(P->offset_first_layer * 1);
            pf = pf * ORC_PIE;
            for (int x = 1; x < MX + 1; x++) {
                r++;
                double Exmin = psi[x] - psi[x - 1];
                Exmin *= (r - 1) * Exmin;
                double Explus = psi[x] - psi[x + 1];
                Explus *= (r) * Explus;
                EE[x] = pf * (Exmin + Explus) / L[x];
            }
        } else {
            pf = pf * ORC_PIE * 2 / 1;
            int r = (int)(P->offset_first_layer * 1 + 1.0);
            double Exmin, Explus = r * (psi[1] - psi[2]);
            Explus *= Explus;
            EE[1] = pf * Explus / (L[1]);
            for (int x = 2; x < MX + 1; x++) {
                r += 1.0;
                Exmin = Explus;
                Explus = r * (psi[x] - psi[x + 1]);
                Explus *= Explus;
                EE[x] = pf * (Exmin + Explus) / L[x];
            }
        }
        return;
    }
    if (P->gradients == 3) {
        /* LGrad3::UpdateEE (LGrad3.cpp:1131-1139): squared differences along
         * z, x and y over the flat array (AddGradSquare, tools_host.h:444),
         * then the prefactor */
        int JX = P->JX, JY = P->JY;
        int d3[3] = {1, JX, JY};
        for (int a = 0; a < 3; a++) {
            int d = d3[a];
            for (int i = 0; i < M - 2 * d; i++) {
                double u = psi[i] - psi[i + d], w = psi[i + d] - psi[i + 2 * d];
                EE[i + d] += u * u + w * w;
            }
        }
        Norm(EE, pf, M);
        return;
    }
    int MY = P->MY, JX = P->JX;
    pf = pf / 2;  /* both 2-D lattices halve pf once */
    if (P->geometry == NM_PLANAR) {
        for (int x = 1; x < MX + 1; x++)
            for (int y = 1; y < MY + 1; y++) {
                int z = x * JX + y;
                double Exmin = psi[z] - psi[z - JX]; Exmin *= Exmin;
                double Explus = psi[z] - psi[z + JX]; Explus *= Explus;
                double Eymin = psi[z] - psi[z - 1]; Eymin *= Eymin;
                double Eyplus = psi[z] - psi[z + 1]; Eyplus *= Eyplus;
                EE[x * JX + y] = pf * (Exmin + Explus + Eymin + Eyplus);
            }
        return;
    }
    int r = (int)(P->offset_first_layer * 1);
    for (int x = 1; x < MX + 1; x++) {
        r++;
        for (int y = 1; y < MY + 1; y++) {
            int z = x * JX + y;
            double Exmin = psi[z] - psi[z - JX];
            Exmin *= (r - 0.5) * Exmin * 2 * ORC_PIE;
            double Explus = psi[z] - psi[z + JX];
            Explus *= (r + 0.5) * Explus * 2 * ORC_PIE;
            double Eymin = (psi[z] - psi[z - 1]) * 1;
            Eymin *= Eymin;
            double Eyplus = (psi[z] - psi[z + 1]) * 1;
            Eyplus *= Eyplus;
            EE[z] = pf * ((Exmin + Explus) / L[z] + Eymin + Eyplus);
        }
    }
}

/* g -= X(ψ), X the Poisson update of ψ from the charge density q and the
 * relative permittivity eps (Lattice::UpdatePsi, not-fixed-ψ0 branch) */
static void update_psi(orc_state* st, double* g, const double* psi, const double* q, const double* eps) {
    const nm_plan* P = st->P;
    int M = st->M, MX = P->MX;
    const double* L = P->L;
    double* X = st->X;
    double C = ORC_E * ORC_E / (ORC_EPS0 * ORC_KBT * P->bond_length);
    if (P->gradients == 1) {
        if (P->geometry == NM_PLANAR) {
            C = C * 2.0 / 1 / 1;
            double epsXmin, epsXplus = eps[0] + eps[1];
            for (int x = 1; x < MX + 1; x++) {
                epsXmin = epsXplus;
                epsXplus = eps[x] + eps[x + 1];
                double a = x == 1 ? psi[0] : X[x - 1];  /* upwind */
                X[x] = (epsXmin * a + C * q[x] + epsXplus * psi[x + 1]) / (epsXmin + epsXplus);
            }
        } else if (P->geometry == NM_CYLINDRICAL) {
            C = C / ORC_PIE;
            double r = P->offset_first_layer * 1;
            double epsXmin, epsXplus = r * (eps[0] + eps[1]);
            for (int x = 1; x < MX + 1; x++) {
                r++;
                epsXmin = epsXplus;
                epsXplus = r * (eps[x] + eps[x + 1]);
                double a = x == 1 ? psi[0] : X[x - 1];  /* upwind */
                X[x] = (epsXmin * a + C * q[x] + epsXplus * psi[x + 1]) / (epsXmin + epsXplus);
            }
        } else {
            C = C / (2.0 * ORC_PIE) * 1;
            double r = P->offset_first_layer * 1;
            double epsXmin, epsXplus = r * r * (eps[0] + eps[1]);
            double a = 0, b = psi[0], c = psi[1];
            for (int x = 1; x < MX + 1; x++) {
                epsXmin = epsXplus;
                r++;
                epsXplus = r * r * (eps[x] + eps[x + 1]);
                a = b; b = c; c = psi[x + 1];
                X[x] = (epsXmin * a + C * q[x] * L[x] + epsXplus * c) / (epsXmin + epsXplus);
            }
        }
    } else if (P->gradients == 3) {
        /* LGrad3::UpdatePsi (LGrad3.cpp:1155-1215), not-fixed-ψ0 branch with
         * an empty mask: a forward and a backward Gauss-Seidel sweep in place
         * on psi; the backward sweep subtracts the new psi from g */
        int MY = P->MY, MZ = P->MZ, JX = P->JX, JY = P->JY;
        double* ps = (double*)psi;
        for (int pass = 0; pass < 2; pass++) {
            for (int xi = 1; xi < MX + 1; xi++)
                for (int yi = 1; yi < MY + 1; yi++)
                    for (int zi = 1; zi < MZ + 1; zi++) {
                        int x = pass ? MX + 1 - xi : xi, y = pass ? MY + 1 - yi : yi, z = pass ? MZ + 1 - zi : zi;
                        int i = x * JX + y * JY + z;
                        double ezm = eps[i - 1] + eps[i], ezp = eps[i] + eps[i + 1];
                        double eym = eps[i] + eps[i - JY], eyp = eps[i] + eps[i + JY];
                        double exm = eps[i] + eps[i - JX], exp_ = eps[i] + eps[i + JX];
                        ps[i] = (exm * ps[i - JX] + exp_ * ps[i + JX] + eym * ps[i - JY] + eyp * ps[i + JY] +
                                 ezm * ps[i - 1] + ezp * ps[i + 1] + C * q[i]) /
                                (exm + exp_ + eym + eyp + ezm + ezp);
                        if (pass) g[i] -= ps[i];
                    }
        }
        return;
    } else if (P->geometry == NM_PLANAR) {
        int MY = P->MY, JX = P->JX;
        C = C * 2.0 / 1 / 1;
        for (int x = 1; x < MX + 1; x++)
            for (int y = 1; y < MY + 1; y++) {
                int i = x * JX + y;
                double epsXmin = eps[i] + eps[i - JX], epsXplus = eps[i] + eps[i + JX];
                double epsYmin = eps[i] + eps[i - 1], epsYplus = eps[i] + eps[i + 1];
                double ax = x == 1 ? psi[i - JX] : X[i - JX];  /* upwind */
                double ay = y == 1 ? psi[i - 1] : X[i - 1];
                X[i] = (C * q[i] + epsXmin * ax + epsXplus * psi[i + JX] + epsYmin * ay + epsYplus * psi[i + 1]) /
                       (epsXmin + epsXplus + epsYmin + epsYplus);
            }
    } else {
        int MY = P->MY, JX = P->JX;
        C = C / 2 / 1 / 1;
        double r = P->offset_first_layer * 1;
        for (int x = 1; x < MX + 1; x++) {
            r++;
            for (int y = 1; y < MY + 1; y++) {
                int i = x * JX + y;
                double epsXmin = 2 * ORC_PIE * (r - 1) * (eps[i] + eps[i - JX]) / L[i] * 1 * 1;
                double epsXplus = 2 * ORC_PIE * r * (eps[i] + eps[i + JX]) / L[i] * 1 * 1;
                double epsYmin = eps[i] + eps[i - 1], epsYplus = eps[i] + eps[i + 1];
                X[i] = (C * q[i] + epsXmin * psi[i - JX] + epsXplus * psi[i + JX] + epsYmin * psi[i - 1] +
                        epsYplus * psi[i + 1]) /
                       (epsXmin + epsXplus + epsYmin + epsYplus);
            }
        }
    }
    for (int i = 0; i < M; i++) g[i] = g[i] - X[i];  /* YisAminB */
}

/* ---- residual ------------------------------------------------------------ */
static void prepare_G1(orc_state* st, const double* x) {
    const nm_plan* P = st->P;
    int M = st->M, ns = P->n_seg;
    /* PutU (system.cpp:1987-2085) + Segment::PrepareForCalculations
     * (segment.cpp:835-879): u = x[it(seg)], set_bounds(u), G1 = exp(-u),
     * times MASK (pinned) and KSAM.  Charged: ψ is the last block of x and
     * u += -ε·EE + v·ψ (system.cpp:2001-2030). */
    if (P->charged) {
        Cp(st->psi, x + (size_t)P->n_it * M, M);
        update_EE(st, st->EE, st->psi);
    }
    for (int i = 0; i < ns; i++) {
        double* u = st->u + (size_t)i * M;
        double* G1 = st->G1 + (size_t)i * M;
        if (has_states(P, i)) {
            /* G1 = Σ_j α_bulk,j·exp(-u_j) over the segment's states, α_j =
             * α_bulk,j·exp(-u_j)/G1 (segment.cpp:861-873), u_j from the
             * state's block with the state's valence (PutU) */
            Zero(G1, M);
            for (int j = 0; j < P->n_state; j++) {
                if (P->state_seg[j] != i) continue;
                double* uj = st->ust + (size_t)j * M;
                double* aj = st->ast + (size_t)j * M;
                Cp(uj, x + (size_t)P->state_it[j] * M, M);
                if (P->charged) {
                    YplusisCtimesX(uj, st->EE, -1.0 * P->seg_epsilon[i], M);
                    if (P->state_valence[j] != 0) YplusisCtimesX(uj, st->psi, P->state_valence[j], M);
                }
                set_bounds(st, uj);
                for (int s = 0; s < M; s++) aj[s] = exp(-uj[s]);
                Norm(aj, st->st_ab[j], M);
                Add(G1, aj, M);
            }
            for (int j = 0; j < P->n_state; j++)
                if (P->state_seg[j] == i) Div(st->ast + (size_t)j * M, G1, M);
            Zero(u, M);
            Times(G1, G1, P->seg_gmask + (size_t)i * M, M);
            Cp(st->phi + (size_t)i * M, P->seg_phi_frozen + (size_t)i * M, M);
            st->seg_phibulk[i] = 0;
            continue;
        }
        if (P->seg_it[i] >= 0) {
            Cp(u, x + (size_t)P->seg_it[i] * M, M);
            if (P->charged) {
                YplusisCtimesX(u, st->EE, -1.0 * P->seg_epsilon[i], M);
                if (P->seg_valence[i] != 0) YplusisCtimesX(u, st->psi, P->seg_valence[i], M);
            }
        } else Zero(u, M);
        set_bounds(st, u);
        for (int s = 0; s < M; s++) G1[s] = exp(-u[s]);
        Times(G1, G1, P->seg_gmask + (size_t)i * M, M);
        /* Segment phi: frozen -> MASK, else 0 */
        Cp(st->phi + (size_t)i * M, P->seg_phi_frozen + (size_t)i * M, M);
        st->seg_phibulk[i] = 0;
    }
}

/* Molecule::ComputePhi of molecule m: rho[m] = Σ d·Gf·Gb per segment type of
 * the molecule, GN[m] = G(N) (mol_linear.cpp:12-135, mol_branched.cpp,
 * mol_dendrimer.cpp; a monomer as molecule.cpp:2669-2683). */
static void compose_mol(orc_state* st, int m) {
    const nm_plan* P = st->P;
    int M = st->M;
    const nm_molecule* mol = &P->mols[m];
    Zero(st->rho[m], mol->n_molmon * M);
    Zero(st->mol_phitot + (size_t)m * M, M);
    if (mol->n_store == 1 && mol->n_blocks == 1) {
        const double* G1 = st->G1 + (size_t)mol->blocks[0].seg * M;
        double* phi = st->rho[m];
        Cp(phi, G1, M);
        st->GN[m] = weighted_sum(st, phi);
        Times(phi, phi, G1, M);
    } else if (mol->markov == 2) {
        m2_compose(st, m);
    } else {
        mol_forward(st, m);
        mol_backward_block(st, m, mol->n_blocks - 1, NULL);
    }
}

int orc_compose(orc_state* st, const double* x, int m, double* rho, double* GN) {
    if (m < 0 || m >= st->P->n_mol) return NM_ERR_ARG;
    prepare_G1(st, x);
    compose_mol(st, m);
    Cp(rho, st->rho[m], st->P->mols[m].n_molmon * st->M);
    if (GN) *GN = st->GN[m];
    st->have_state = 0;
    return NM_OK;
}

static int compute_phis(orc_state* st, const double* x) {
    const nm_plan* P = st->P;
    int M = st->M, ns = P->n_seg;
    prepare_G1(st, x);
    /* System::ComputePhis (system.cpp:2324-2640) */
    Zero(st->phitot, M);
    for (int i = 0; i < ns; i++)
        if (P->seg_freedom[i] == NM_SEG_FROZEN) Add(st->phitot, st->phi + (size_t)i * M, M);
    for (int m = 0; m < P->n_mol; m++) compose_mol(st, m);
    double A = 0, B = 0;
    for (int m = 0; m < P->n_mol; m++) {
        const nm_molecule* mol = &P->mols[m];
        double N = mol->chainlength;
        double norm = 0;
        const double a_n = st->amt_n[m], a_theta = st->amt_theta[m], a_phibulk = st->amt_phibulk[m];
        st->mol_n[m] = a_n; st->mol_theta[m] = a_theta;
        if (mol->freedom == NM_MOL_FREE) {
            st->mol_phibulk[m] = a_phibulk;
            norm = a_phibulk / N;
            st->mol_n[m] = norm * st->GN[m];
            st->mol_theta[m] = st->mol_n[m] * N;  /* θ = n·N (Molecule::theta of a free molecule) */
            A += a_phibulk * st->mol_charge[m]; B += a_phibulk;
        } else if (mol->freedom == NM_MOL_RESTRICTED) {
            if (st->GN[m] > 0) {
                norm = a_n / st->GN[m];
                if (mol->pinned) st->mol_phibulk[m] = 0;
                else {
                    st->mol_phibulk[m] = N * norm;
                    A += st->mol_phibulk[m] * st->mol_charge[m]; B += st->mol_phibulk[m];
                }
            } else return NM_ERR_GN;
        } else st->mol_phibulk[m] = 0;
        st->norm[m] = norm;
        for (int k = 0; k < mol->n_molmon; k++) {
            double* phi = st->rho[m] + (size_t)k * M;
            Div(phi, st->G1 + (size_t)mol->molmon_seg[k] * M, M);
            if (norm > 0) Norm(phi, norm, M);
        }
    }
    if (P->charged && P->neutralizer >= 0) {
        /* the neutraliser takes the bulk volume fraction that makes the bulk
         * neutral (system.cpp:2487-2515, 2560-2570) */
        int nt = P->neutralizer;
        const nm_molecule* mol = &P->mols[nt];
        double qs = P->solvent >= 0 ? st->mol_charge[P->solvent] : 0;
        if (st->mol_charge[nt] != qs) st->mol_phibulk[nt] = ((B - 1.0) * qs - A) / (st->mol_charge[nt] - qs);
        B += st->mol_phibulk[nt];
        double norm = st->mol_phibulk[nt] / mol->chainlength;
        st->mol_n[nt] = norm * st->GN[nt];
        st->mol_theta[nt] = st->mol_n[nt] * mol->chainlength;
        st->norm[nt] = norm;
        for (int k = 0; k < mol->n_molmon; k++)
            if (norm > 0) Norm(st->rho[nt] + (size_t)k * M, norm, M);
    }
    if (P->solvent >= 0) {
        int sv = P->solvent;
        const nm_molecule* mol = &P->mols[sv];
        st->mol_phibulk[sv] = 1.0 - B;
        if (st->mol_phibulk[sv] < 0) return NM_ERR_NEG_SOLVENT;
        double norm = st->mol_phibulk[sv] / mol->chainlength;
        st->mol_n[sv] = norm * st->GN[sv];
        st->mol_theta[sv] = st->mol_n[sv] * mol->chainlength;
        st->norm[sv] = norm;
        for (int k = 0; k < mol->n_molmon; k++)
            if (norm > 0) Norm(st->rho[sv] + (size_t)k * M, norm, M);
    }
    for (int m = 0; m < P->n_mol; m++) {
        const nm_molecule* mol = &P->mols[m];
        for (int k = 0; k < mol->n_molmon; k++) {
            int sg = mol->molmon_seg[k];
            double* pm = st->rho[m] + (size_t)k * M;
            Add(st->phi + (size_t)sg * M, pm, M);
            Add(st->phitot, pm, M);
            Add(st->mol_phitot + (size_t)m * M, pm, M);
            st->seg_phibulk[sg] += mol->molmon_fraction[k] * st->mol_phibulk[m];
        }
    }
    for (int i = 0; i < ns; i++) set_bounds(st, st->phi + (size_t)i * M);
    /* Segment::SetPhiSide (segment.cpp:1331-1353); a segment with states:
     * φ_j = α_j·φ per state, its side, and φ_bulk,j = φ_bulk·α_bulk,j */
    for (int i = 0; i < ns; i++) {
        st->sp_phibulk[i] = st->seg_phibulk[i];
        if (!has_states(P, i)) stencil(st, st->phi_side + (size_t)i * M, st->phi + (size_t)i * M, 1);
        else Zero(st->phi_side + (size_t)i * M, M);
    }
    for (int j = 0; j < P->n_state; j++) {
        const int sg = P->state_seg[j];
        double* pj = st->phi + (size_t)(ns + j) * M;
        Times(pj, st->ast + (size_t)j * M, st->phi + (size_t)sg * M, M);
        stencil(st, st->phi_side + (size_t)(ns + j) * M, pj, 1);
        st->sp_phibulk[ns + j] = st->seg_phibulk[sg] * st->st_ab[j];
    }
    return NM_OK;
}

int orc_residual(orc_state* st, const double* x, double* g) {
    const nm_plan* P = st->P;
    int M = st->M, ns = P->n_seg, nit = P->n_it;
    /* System::Classical_residual (system.cpp:2087-2189) */
    Cp(g, x, P->iv);
    int rc = compute_phis(st, x);
    st->have_state = (rc == NM_OK);
    if (rc) return rc;
    Zero(st->alpha, M);
    /* the species: segments without states, then the states (the
     * reference's loops over `ns < 2` mons and over StateList) */
    const int nsp = P->n_state > 0 ? P->n_sp : ns;
    for (int i = 0; i < nit; i++) {
        double* gi = g + (size_t)i * M;
        int r = P->n_state > 0 ? P->it_sp[i] : P->it_seg[i];
        for (int k = 0; k < nsp; k++) {
            if (k < ns && has_states(P, k)) continue;
            double chi = chi_of(P, r, k);
            if (chi == 0) continue;
            const double* ps = st->phi_side + (size_t)k * M;
            double pb = st->sp_phibulk[k];
            for (int s = 0; s < M; s++)  /* PutAlpha, tools_host.h:428-431 */
                if (st->phitot[s] > 0) gi[s] = gi[s] - chi * (ps[s] / st->phitot[s] - pb);
        }
    }
    for (int i = 0; i < nit; i++) Add(st->alpha, g + (size_t)i * M, M);
    Norm(st->alpha, 1.0 / nit, M);
    for (int i = 0; i < nit; i++) {
        double* gi = g + (size_t)i * M;
        for (int s = 0; s < M; s++) {  /* AddG, tools_host.h:446-451 */
            if (st->phitot[s] > 0) gi[s] = gi[s] - st->alpha[s] + 1 / st->phitot[s] - 1.0;
            else gi[s] = 0;
        }
        remove_bounds(st, gi);
        for (int s = 0; s < M; s++) gi[s] *= P->ksam[s];
    }
    if (P->charged) {
        /* the ψ block: DoElectrostatics (system.cpp:1920-1953), then
         * g = ψ - UpdatePsi(ψ) (system.cpp:2161-2170) */
        double* gp = g + (size_t)nit * M;
        Zero(st->q, M);
        Zero(st->eps, M);
        for (int i = 0; i < ns; i++) {
            double* phi = st->phi + (size_t)i * M;
            if (!has_states(P, i)) YplusisCtimesX(st->q, phi, P->seg_valence[i], M);
            set_bounds(st, phi);
            YplusisCtimesX(st->eps, phi, P->seg_epsilon[i], M);
        }
        for (int j = 0; j < P->n_state; j++)
            YplusisCtimesX(st->q, st->phi + (size_t)(ns + j) * M, P->state_valence[j], M);
        Div(st->q, st->phitot, M);
        Div(st->eps, st->phitot, M);
        Cp(st->psi, x + (size_t)nit * M, M);
        Cp(gp, st->psi, M);
        set_M_bounds(st, st->psi);
        set_M_bounds(st, st->psi);
        st->psi[0] = st->psi[1];
        update_psi(st, gp, st->psi, st->q, st->eps);
        remove_bounds(st, gp);
    }
    return NM_OK;
}

/* ---- DIIS (sfnewton.cpp:793-926, 1037-1130) ------------------------------ */
/* Solve A c = 1 for symmetric A by a cyclic Jacobi eigen-decomposition,
 * c = Q diag(1/λ) Qᵀ 1 — the unregularised pseudo-inverse that the
 * reference's SVD solve (Ax, sfnewton.cpp:793-835) evaluates. */
static int small_solve(const double* A, double* c, int n) {
    double a[100 * 100], q[100 * 100];
    for (int i = 0; i < n * n; i++) { if (A[i] != A[i]) return NM_ERR_NAN_DIIS; a[i] = A[i]; }
    if (n == 1) { c[0] = 1; return NM_OK; }
    for (int i = 0; i < n; i++) for (int j = 0; j < n; j++) q[i * n + j] = (i == j);
    for (int sweep = 0; sweep < 60; sweep++) {
        double off = 0, diag = 0;
        for (int i = 0; i < n; i++) for (int j = 0; j < n; j++) {
            if (i != j) off += a[i * n + j] * a[i * n + j]; else diag += a[i * n + j] * a[i * n + j];
        }
        if (off <= 1e-30 * diag || off == 0) break;
        for (int p = 0; p < n - 1; p++)
            for (int r = p + 1; r < n; r++) {
                double apr = a[p * n + r];
                if (apr == 0) continue;
                double app = a[p * n + p], arr = a[r * n + r];
                double theta = (arr - app) / (2 * apr);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1));
                double cs = 1 / sqrt(t * t + 1), sn = t * cs;
                for (int k = 0; k < n; k++) {
                    double akp = a[k * n + p], akr = a[k * n + r];
                    a[k * n + p] = cs * akp - sn * akr;
                    a[k * n + r] = sn * akp + cs * akr;
                }
                for (int k = 0; k < n; k++) {
                    double apk = a[p * n + k], ark = a[r * n + k];
                    a[p * n + k] = cs * apk - sn * ark;
                    a[r * n + k] = sn * apk + cs * ark;
                }
                for (int k = 0; k < n; k++) {
                    double qkp = q[k * n + p], qkr = q[k * n + r];
                    q[k * n + p] = cs * qkp - sn * qkr;
                    q[k * n + r] = sn * qkp + cs * qkr;
                }
            }
    }
    for (int i = 0; i < n; i++) c[i] = 0;
    for (int j = 0; j < n; j++) {
        double proj = 0;
        for (int k = 0; k < n; k++) proj += q[k * n + j];
        double w = proj / a[j * n + j];
        for (int i = 0; i < n; i++) c[i] += q[i * n + j] * w;
    }
    for (int i = 0; i < n; i++) if (c[i] != c[i]) return NM_ERR_NAN_SVD;
    return NM_OK;
}

static double resid_norm(const double* g, int n, int max_norm) {
    if (max_norm) {
        double mx = 0;
        for (int i = 0; i < n; i++) if (fabs(g[i]) > mx) mx = fabs(g[i]);
        return mx;
    }
    return sqrt(Dot(g, g, n));
}

int orc_solve_n(orc_state* st, double* x, int max_iter, int* iterations, double* residual) {
    const nm_plan* P = st->P;
    int nvar = P->iv, m = P->diis_m;
    double dmax = P->deltamax, tol = st->tol_override > 0 ? st->tol_override : P->tolerance;
    double* xR = calloc((size_t)m * nvar, sizeof(double));
    double* x_x0 = calloc((size_t)m * nvar, sizeof(double));
    double* x0 = calloc((size_t)nvar, sizeof(double));
    double* g = calloc((size_t)nvar, sizeof(double));
    double* Aij = calloc((size_t)m * m, sizeof(double));
    double* Apij = calloc((size_t)m * m, sizeof(double));
    double* Ci = calloc((size_t)m, sizeof(double));
    int it = 0, k_diis = 0, rc = NM_OK;
    double res = 0;
    Cp(x0, x, nvar);
    rc = orc_residual(st, x, g);
    if (rc) goto done;
    YplusisCtimesX(x, g, -dmax, nvar);
    for (int i = 0; i < nvar; i++) x_x0[i] = x[i] - x0[i];
    Cp(xR, x, nvar);
    res = resid_norm(g, nvar, P->max_norm);
    while (res > tol && it < max_iter) {
        it++;
        Cp(x0, x, nvar);
        rc = orc_residual(st, x, g);
        if (rc) goto done;
        int k = it % m;
        k_diis++;
        YplusisCtimesX(x, g, -dmax, nvar);
        Cp(xR + (size_t)k * nvar, x, nvar);
        for (int i = 0; i < nvar; i++) x_x0[(size_t)k * nvar + i] = x[i] - x0[i];
        /* SFNewton::DIIS (sfnewton.cpp:837-880) */
        int kd = k_diis;
        if (kd > m) {
            kd = m;
            for (int i = 1; i < m; i++) for (int j = 1; j < m; j++) Aij[m * (i - 1) + j - 1] = Aij[m * i + j];
        }
        for (int i = 0; i < kd; i++) {
            int posi = k - kd + 1 + i;
            if (posi < 0) posi += m;
            double D = Dot(x_x0 + (size_t)posi * nvar, x_x0 + (size_t)k * nvar, nvar);
            Aij[i + m * (kd - 1)] = Aij[kd - 1 + m * i] = D + 1e-9;
            for (int j = 0; j < kd; j++) Apij[j + kd * i] = Aij[j + m * i];
        }
        rc = small_solve(Apij, Ci, kd);
        if (rc) goto done;
        double normC = 0;
        for (int i = 0; i < kd; i++) normC += Ci[i];
        for (int i = 0; i < kd; i++) Ci[i] = Ci[i] / normC;
        Zero(x, nvar);
        int posi = k - kd + 1;
        if (posi < 0) posi += m;
        YplusisCtimesX(x, xR + (size_t)posi * nvar, Ci[0], nvar);  /* Xr_times_ci */
        for (int i = 1; i < kd; i++) {
            posi = k - kd + 1 + i;
            if (posi < 0) posi += m;
            YplusisCtimesX(x, xR + (size_t)posi * nvar, Ci[i], nvar);
        }
        res = resid_norm(g, nvar, P->max_norm);
    }
done:
    if (iterations) *iterations = it;
    if (residual) *residual = res;
    free(xR); free(x_x0); free(x0); free(g); free(Aij); free(Apij); free(Ci);
    return rc;
}

int orc_solve(orc_state* st, double* x, int* iterations, double* residual) {
    return orc_solve_n(st, x, st->P->iterationlimit, iterations, residual);
}

/* ---- outputs -------------------------------------------------------------- */
int orc_get_field(orc_state* st, int which, double* out) {
    const nm_plan* P = st->P;
    int M = st->M;
    if (!st->have_state) return NM_ERR_ARG;
    switch (which) {
        case 0: Cp(out, st->phi, P->n_seg * M); return NM_OK;
        case 1: Cp(out, st->G1, P->n_seg * M); return NM_OK;
        case 2: Cp(out, st->alpha, M); return NM_OK;
        case 3: Cp(out, st->phitot, M); return NM_OK;
        case 4: Cp(out, st->mol_phitot, P->n_mol * M); return NM_OK;
        case 5: Cp(out, st->phi_side, P->n_seg * M); return NM_OK;
        case 6: if (!P->charged) return NM_ERR_ARG; Cp(out, st->psi, M); return NM_OK;
        case 7: if (!P->charged) return NM_ERR_ARG; Cp(out, st->q, M); return NM_OK;
        case 8: if (!P->charged) return NM_ERR_ARG; Cp(out, st->eps, M); return NM_OK;
        case 9: if (!P->n_state) return NM_ERR_ARG; Cp(out, st->phi + (size_t)P->n_seg * M, P->n_state * M); return NM_OK;
        case 10: if (!P->n_state) return NM_ERR_ARG; Cp(out, st->ast, P->n_state * M); return NM_OK;
        case 11: if (!P->n_state) return NM_ERR_ARG; Cp(out, st->ust, P->n_state * M); return NM_OK;
    }
    return NM_ERR_ARG;
}

/* the bulk volume fractions of the interaction species of the last
 * residual (segments, then states) [n_sp] */
int orc_get_species_phibulk(orc_state* st, double* out) {
    const nm_plan* P = st->P;
    if (!st->have_state) return NM_ERR_ARG;
    const int nsp = P->n_seg + P->n_state;
    for (int k = 0; k < nsp; k++) out[k] = st->sp_phibulk[k];
    return NM_OK;
}

int orc_get_molecule(orc_state* st, int m, double* GN, double* n, double* theta, double* phibulk) {
    if (!st->have_state || m < 0 || m >= st->P->n_mol) return NM_ERR_ARG;
    if (GN) *GN = st->GN[m];
    if (n) *n = st->mol_n[m];
    if (theta) *theta = st->mol_theta[m];
    if (phibulk) *phibulk = st->mol_phibulk[m];
    return NM_OK;
}

/* GetFreeEnergy (system.cpp:2809-3029), GetGrandPotential (:3038-3244),
 * CreateMu (:3246-3400) for state-free systems, with the electrostatic
 * terms where the system is charged. */
/* Molecule::fraction of a segment (0 when the molecule has none) */
static double mol_fraction(const nm_molecule* mol, int seg) {
    double f = 0;
    for (int q = 0; q < mol->n_molmon; q++) if (mol->molmon_seg[q] == seg) f = mol->molmon_fraction[q];
    return f;
}

int orc_free_energy(orc_state* st, double* Fout, double* Omega, double* mu) {
    const nm_plan* P = st->P;
    int M = st->M, ns = P->n_seg;
    if (!st->have_state) return NM_ERR_ARG;
    double* F = calloc((size_t)M, sizeof(double));
    double* T = st->tmp;
    const int nst = P->n_state;
    for (int m = 0; m < P->n_mol; m++) remove_bounds(st, st->mol_phitot + (size_t)m * M);
    for (int i = 0; i < ns + nst; i++) remove_bounds(st, st->phi_side + (size_t)i * M);
    for (int m = 0; m < P->n_mol; m++) {
        const nm_molecule* mol = &P->mols[m];
        double N = mol->chainlength;
        double constant = log(N * st->mol_n[m] / st->GN[m]) / N;
        Cp(T, st->mol_phitot + (size_t)m * M, M);
        Norm(T, constant, M);
        Add(F, T, M);
    }
    /* SysMonList: segments that occur in molecules; a segment with states
     * counts -φ_j·u_j per state (system.cpp:2866-2888) */
    for (int i = 0; i < ns; i++) {
        if (!st->in_mol[i]) continue;
        if (has_states(P, i)) {
            for (int j = 0; j < nst; j++) {
                if (P->state_seg[j] != i) continue;
                const double* pj = st->phi + (size_t)(ns + j) * M;
                const double* uj = st->ust + (size_t)j * M;
                for (int s = 0; s < M; s++) F[s] += -1.0 * (pj[s] * uj[s]);
            }
            continue;
        }
        const double* G1 = st->G1 + (size_t)i * M;
        const double* phi = st->phi + (size_t)i * M;
        for (int s = 0; s < M; s++) {
            double ml = G1[s] > 0 ? -log(G1[s]) : 0;
            F[s] += -1.0 * (phi[s] * ml);
        }
    }
    for (int j = 0; j < ns; j++) {
        if (has_states(P, j)) continue;
        const double* phi = st->phi + (size_t)j * M;
        for (int k = 0; k < ns; k++) {
            if (has_states(P, k)) continue;
            double chi = (P->seg_freedom[k] == NM_SEG_FROZEN) ? chi_of(P, j, k) : chi_of(P, j, k) / 2;
            if (P->seg_freedom[j] == NM_SEG_FROZEN || chi == 0) continue;
            const double* ps = st->phi_side + (size_t)k * M;
            for (int s = 0; s < M; s++) F[s] += chi * (phi[s] * ps[s]);
        }
        for (int i = 0; i < nst; i++) {  /* system.cpp:2916-2929 */
            double chi = chi_of(P, j, ns + i) / 2;
            if (P->seg_freedom[j] == NM_SEG_FROZEN || chi == 0) continue;
            const double* ps = st->phi_side + (size_t)(ns + i) * M;
            for (int s = 0; s < M; s++) F[s] += chi * (phi[s] * ps[s]);
        }
    }
    for (int j = 0; j < nst; j++) {  /* system.cpp:2933-2979 */
        const double* phi = st->phi + (size_t)(ns + j) * M;
        for (int k = 0; k < ns; k++) {
            if (has_states(P, k)) continue;
            double chi = chi_of(P, ns + j, k);
            if (P->seg_freedom[k] != NM_SEG_FROZEN) chi = chi / 2;
            if (chi == 0) continue;
            const double* ps = st->phi_side + (size_t)k * M;
            for (int s = 0; s < M; s++) F[s] += chi * (phi[s] * ps[s]);
        }
        /* the state–state term reads the state's own side fraction
         * (system.cpp:2971-2977: phi_side of Sta[j], not of Sta[l]) */
        for (int l = 0; l < nst; l++) {
            double chi = chi_of(P, ns + j, ns + l) / 2;
            if (chi == 0) continue;
            const double* ps = st->phi_side + (size_t)(ns + j) * M;
            for (int s = 0; s < M; s++) F[s] += chi * (phi[s] * ps[s]);
        }
    }
    for (int m = 0; m < P->n_mol; m++) {
        const nm_molecule* mol = &P->mols[m];
        double constant = 0;
        for (int j = 0; j < mol->n_molmon; j++)
            for (int k = 0; k < mol->n_molmon; k++) {
                double fA = mol->molmon_fraction[j], fB = mol->molmon_fraction[k];
                double chi = P->chi[mol->molmon_seg[j] * ns + mol->molmon_seg[k]] / 2;
                constant -= fA * fB * chi;
            }
        Cp(T, st->mol_phitot + (size_t)m * M, M);
        Norm(T, constant, M);
        Add(F, T, M);
    }
    for (int s = 0; s < M; s++) F[s] *= P->ksam[s];
    if (P->charged) {  /* system.cpp:3020-3028 */
        Zero(T, M);
        AddTimes(T, st->q, st->psi, M);
        Norm(T, 0.5, M);
        Add(F, T, M);
    }
    double Fv = weighted_sum(st, F);
    /* grand potential */
    double* GP = F;
    Zero(GP, M);
    for (int m = 0; m < P->n_mol; m++) {
        double N = P->mols[m].chainlength;
        const double* pt = st->mol_phitot + (size_t)m * M;
        for (int s = 0; s < M; s++) T[s] = (pt[s] + (-st->mol_phibulk[m])) * (1.0 / N);
        Add(GP, T, M);
    }
    Add(GP, st->alpha, M);
    /* species pairs (system.cpp:3104-3206): segments without states and
     * states, frozen segments left out */
    for (int j = 0; j < ns + nst; j++) {
        if (j < ns && (P->seg_freedom[j] == NM_SEG_FROZEN || has_states(P, j))) continue;
        const double* phi = st->phi + (size_t)j * M;
        double pbA = st->sp_phibulk[j];
        for (int k = 0; k < ns + nst; k++) {
            if (k < ns && (P->seg_freedom[k] == NM_SEG_FROZEN || has_states(P, k))) continue;
            double chi = chi_of(P, j, k) / 2;
            if (chi == 0) continue;
            const double* ps = st->phi_side + (size_t)k * M;
            double pbB = st->sp_phibulk[k];
            for (int s = 0; s < M; s++) GP[s] += chi * (phi[s] * ps[s] + (-pbA * pbB));
        }
    }
    Norm(GP, -1.0, M);
    if (P->charged) {  /* system.cpp:3225-3238 */
        Zero(T, M);
        Times(T, st->EE, st->eps, M);
        Norm(T, -2.0, M);
        AddTimes(T, st->q, st->psi, M);
        Norm(T, -1.0 / 2.0, M);
        Add(GP, T, M);
        for (int s = 0; s < M; s++) GP[s] *= P->ksam[s];
        for (int s = 0; s < M; s++) T[s] = st->q[s] * P->ksam[s];
        for (int s = 0; s < M; s++) T[s] = st->q[s] - T[s];
        Times(T, T, st->psi, M);
        Norm(T, 0.5, M);
        Add(GP, T, M);
    } else {
        for (int s = 0; s < M; s++) GP[s] *= P->ksam[s];
    }
    double Ov = weighted_sum(st, GP);
    free(F);
    if (Fout) *Fout = Fv;
    if (Omega) *Omega = Ov;
    if (mu) {
        for (int i = 0; i < P->n_mol; i++) {
            const nm_molecule* mol = &P->mols[i];
            double NA = mol->chainlength;
            double Mu = log(NA * st->mol_n[i] / st->GN[i]) + 1;
            double constant = 0;
            for (int k = 0; k < P->n_mol; k++) constant += st->mol_phibulk[k] / P->mols[k].chainlength;
            Mu = Mu - NA * constant;
            for (int j = 0; j < ns; j++) {
                if (has_states(P, j)) continue;
                double pbA = st->seg_phibulk[j], FA = mol_fraction(mol, j);
                for (int k = 0; k < ns; k++) {
                    if (has_states(P, k)) continue;
                    double pbB = st->seg_phibulk[k], FB = mol_fraction(mol, k);
                    double chi = chi_of(P, j, k) / 2;
                    Mu = Mu - NA * chi * (pbA - FA) * (pbB - FB);
                }
                for (int l = 0; l < P->n_state; l++) {  /* system.cpp:3345-3358 */
                    double pbB = st->sp_phibulk[ns + l];
                    double FB = mol_fraction(mol, P->state_seg[l]) * st->st_ab[l];
                    double chi = chi_of(P, j, ns + l) / 2;
                    Mu = Mu - NA * chi * (pbA - FA) * (pbB - FB);
                }
            }
            for (int j = 0; j < P->n_state; j++) {  /* system.cpp:3361-3400 */
                double pbA = st->sp_phibulk[ns + j];
                double FA = mol_fraction(mol, P->state_seg[j]) * st->st_ab[j];
                for (int k = 0; k < ns; k++) {
                    if (has_states(P, k)) continue;
                    double pbB = st->seg_phibulk[k], FB = mol_fraction(mol, k);
                    double chi = chi_of(P, ns + j, k) / 2;
                    Mu = Mu - NA * chi * (pbA - FA) * (pbB - FB);
                }
                /* the state–state term takes FB of state j as well
                 * (system.cpp:3388-3391) */
                for (int k = 0; k < P->n_state; k++) {
                    double pbB = st->sp_phibulk[ns + k];
                    double FB = mol_fraction(mol, P->state_seg[j]) * st->st_ab[j];
                    double chi = chi_of(P, ns + j, ns + k) / 2;
                    Mu = Mu - NA * chi * (pbA - FA) * (pbB - FB);
                }
            }
            mu[i] = Mu;
        }
    }
    return NM_OK;
}

/* ---- lifetime --------------------------------------------------------------- */
orc_state* orc_create(const nm_plan* P) {
    orc_state* st = calloc(1, sizeof(orc_state));
    int M = P->M, ns = P->n_seg, nm = P->n_mol;
    st->P = P; st->M = M;
    bc_sources(st);
    st->amt_n = calloc((size_t)nm, sizeof(double));
    st->amt_theta = calloc((size_t)nm, sizeof(double));
    st->amt_phibulk = calloc((size_t)nm, sizeof(double));
    for (int m = 0; m < nm; m++) {
        st->amt_n[m] = P->mols[m].n; st->amt_theta[m] = P->mols[m].theta; st->amt_phibulk[m] = P->mols[m].phibulk;
    }
    const int nsp = ns + P->n_state;
    st->u = calloc((size_t)ns * M, sizeof(double));
    st->G1 = calloc((size_t)ns * M, sizeof(double));
    st->phi = calloc((size_t)nsp * M, sizeof(double));
    st->phi_side = calloc((size_t)nsp * M, sizeof(double));
    st->ust = calloc((size_t)(P->n_state + 1) * M, sizeof(double));
    st->ast = calloc((size_t)(P->n_state + 1) * M, sizeof(double));
    st->sp_phibulk = calloc((size_t)nsp, sizeof(double));
    st->in_mol = calloc((size_t)ns, sizeof(int));
    st->st_ab = calloc((size_t)(P->n_state + 1), sizeof(double));
    for (int j = 0; j < P->n_state; j++) st->st_ab[j] = P->state_alphabulk[j];
    st->mol_charge = calloc((size_t)nm, sizeof(double));
    for (int m = 0; m < nm; m++) st->mol_charge[m] = P->mols[m].charge;
    for (int m = 0; m < nm; m++)
        for (int k = 0; k < P->mols[m].n_molmon; k++) st->in_mol[P->mols[m].molmon_seg[k]] = 1;
    st->phitot = calloc((size_t)M, sizeof(double));
    st->alpha = calloc((size_t)M, sizeof(double));
    st->tmp = calloc((size_t)M, sizeof(double));
    st->unity = calloc((size_t)M, sizeof(double));
    for (int s = 0; s < M; s++) st->unity[s] = P->ksam[s];  /* UNITY = KSAM, molecule.cpp:304 */
    st->gb = calloc((size_t)2 * M, sizeof(double));
    st->mol_phitot = calloc((size_t)nm * M, sizeof(double));
    st->Gf = calloc((size_t)nm, sizeof(double*));
    st->rho = calloc((size_t)nm, sizeof(double*));
    st->jGb = calloc((size_t)nm, sizeof(double*));
    st->Pc = calloc((size_t)nm, sizeof(double*));
    st->Qb = calloc((size_t)nm, sizeof(double*));
    for (int m = 0; m < nm; m++) {
        const nm_molecule* mol = &P->mols[m];
        st->Gf[m] = calloc((size_t)mol->n_store * M * (mol->markov == 2 ? M2_FJC : 1), sizeof(double));
        st->rho[m] = calloc((size_t)mol->n_molmon * M, sizeof(double));
        st->jGb[m] = calloc((size_t)mol->n_blocks * M, sizeof(double));
        st->Pc[m] = calloc((size_t)mol->n_blocks * M, sizeof(double));
        st->Qb[m] = calloc((size_t)mol->n_blocks * M, sizeof(double));
    }
    for (int m = 0; m < nm; m++)
        if (P->mols[m].markov == 2 && !st->gb3) {
            st->gb3 = calloc((size_t)2 * M2_FJC * M, sizeof(double));
            st->m2l1 = calloc((size_t)M, sizeof(double));
            st->m2l11 = calloc((size_t)M, sizeof(double));
            st->m2l_1 = calloc((size_t)M, sizeof(double));
            st->m2l_11 = calloc((size_t)M, sizeof(double));
            if (P->geometry != NM_PLANAR)  /* interior only; the halo weights stay 0 */
                for (int i = 1; i < P->MX + 1; i++) {
                    st->m2l1[i] = P->lambda1[i] / P->lambda;
                    st->m2l11[i] = 1.0 - st->m2l1[i];
                    st->m2l_1[i] = P->lambda_1[i] / P->lambda;
                    st->m2l_11[i] = 1.0 - st->m2l_1[i];
                }
        }
    st->GN = calloc((size_t)nm, sizeof(double));
    st->norm = calloc((size_t)nm, sizeof(double));
    st->mol_n = calloc((size_t)nm, sizeof(double));
    st->mol_theta = calloc((size_t)nm, sizeof(double));
    st->mol_phibulk = calloc((size_t)nm, sizeof(double));
    st->seg_phibulk = calloc((size_t)ns, sizeof(double));
    st->psi = calloc((size_t)M, sizeof(double));
    st->EE = calloc((size_t)M, sizeof(double));
    st->q = calloc((size_t)M, sizeof(double));
    st->eps = calloc((size_t)M, sizeof(double));
    st->X = calloc((size_t)M, sizeof(double));
    return st;
}

/* New bulk fractions of the states (a scan step of a fixed state's
 * alphabulk, with the bulk equilibrium solved by the caller): the molecules'
 * bulk charges follow as Molecule::Charge (molecule.cpp:1866-1879) counts
 * them, Σ α_bulk·valence over each state segment's states. */
int orc_set_states(orc_state* st, const double* alphabulk) {
    const nm_plan* P = st->P;
    if (!P->n_state) return NM_ERR_ARG;
    for (int j = 0; j < P->n_state; j++) st->st_ab[j] = alphabulk[j];
    for (int m = 0; m < P->n_mol; m++) {
        const nm_molecule* mol = &P->mols[m];
        int with_states = 0;
        for (int k = 0; k < mol->n_molmon; k++) with_states |= has_states(P, mol->molmon_seg[k]);
        if (!with_states) continue;
        double q = 0;
        for (int k = 0; k < mol->n_molmon; k++) {
            const int sg = mol->molmon_seg[k];
            const double nmon = mol->molmon_fraction[k] * mol->chainlength;
            if (has_states(P, sg)) {
                for (int j = 0; j < P->n_state; j++)
                    if (P->state_seg[j] == sg) q += st->st_ab[j] * P->state_valence[j] * nmon;
            } else q += P->seg_valence[sg] * nmon;
        }
        st->mol_charge[m] = q / mol->chainlength;
    }
    return NM_OK;
}

/* A scan or search step's value change (Molecule::PutValue,
 * molecule.cpp:995-1010): what 0 θ (n = θ/N), 1 n (θ = n·N), 2 φ_bulk. */
int orc_set_amount(orc_state* st, int m, int what, double v) {
    const nm_plan* P = st->P;
    if (m < 0 || m >= P->n_mol) return NM_ERR_ARG;
    const double N = P->mols[m].chainlength;
    if (what == 0) { st->amt_theta[m] = v; st->amt_n[m] = v / N; }
    else if (what == 1) { st->amt_n[m] = v; st->amt_theta[m] = v * N; }
    else if (what == 2) st->amt_phibulk[m] = v;
    else return NM_ERR_ARG;
    return NM_OK;
}

/* The plan's search (Solve_scf::SuperIterate, solve_scf.cpp:717-750): the
 * damped regula falsi of SFNewton::iterate_RF (sfnewton.cpp:1132-1185) on
 * the variable's scale relative to its value at each (re)start, every
 * evaluation a DIIS solve from the current x to super_tolerance; the error
 * of System::GetError (system.cpp:1405-1425) or Molecule::GetError
 * (molecule.cpp:942-968). */
static int search_error(orc_state* st, double* g) {
    const nm_plan* P = st->P;
    const double t = P->target_value;
    double F = 0, O = 0;
    double* mu = calloc((size_t)P->n_mol, sizeof(double));
    int rc = orc_free_energy(st, &F, &O, mu);
    if (rc == NM_OK) {
        if (P->target_kind == 0) *g = F - t;
        else if (P->target_kind == 1) *g = -(O - t);
        else {
            const int m = P->target_mol;
            const double v = P->target_what == 0 ? st->mol_theta[m] : P->target_what == 1 ? st->mol_n[m]
                           : P->target_what == 2 ? st->mol_phibulk[m] : mu[m];
            *g = t != 0 ? v / t - 1.0 : v;
            if (P->target_what == 2) *g = -*g;
        }
    }
    free(mu);
    return rc;
}

static int search_eval(orc_state* st, double* x, double v, double* g, int* solves) {
    const nm_plan* P = st->P;
    int its; double res;
    orc_set_amount(st, P->search_mol, P->search_what, v);
    int rc = orc_solve(st, x, &its, &res);
    (*solves)++;
    if (rc) return rc;
    return search_error(st, g);
}

int orc_search(orc_state* st, double* x, double* value, double* error, int* iterations, int* solves) {
    const nm_plan* P = st->P;
    if (P->search_mol < 0) return NM_ERR_ARG;
    const double tol = P->super_tolerance, dmax = P->super_deltamax;
    const int itlim = P->super_iterationlimit;
    const int m = P->search_mol;
    double xv = P->search_what == 0 ? st->amt_theta[m] : P->search_what == 1 ? st->amt_n[m] : st->amt_phibulk[m];
    double a = 0, b = 0, c = 0, fa = 0, fb = 0, fc = 0, res = 100.0;
    int k = 0, it = 0, rc = NM_OK;
    *solves = 0;
    st->tol_override = tol;
    while (it < itlim && fabs(res) > tol) {
        const double xs = xv;
        if ((rc = search_eval(st, x, xv, &fa, solves))) goto done;
        a = 1;
        xv = (a + dmax) * xs;
        if ((rc = search_eval(st, x, xv, &fb, solves))) goto done;
        b = xv / xs;
        c = a - 0.5 * ((fa * (a - b)) / (fa - fb));
        xv = c * xs;
        if ((rc = search_eval(st, x, xv, &fc, solves))) goto done;
        res = fc;
        it += k;  /* the reference counts the previous pass's steps again */
        k = 0;
        while (k < itlim / 10 && fabs(res) > tol) {
            c = a - 0.5 * ((fa * (a - b)) / (fa - fb));
            xv = c * xs;
            if ((rc = search_eval(st, x, xv, &fc, solves))) goto done;
            if (fc * fb < 0) {
                b = c; xv = b * xs;
                if ((rc = search_eval(st, x, xv, &fb, solves))) goto done;
                res = fb;
            } else {
                a = c; xv = a * xs;
                if ((rc = search_eval(st, x, xv, &fa, solves))) goto done;
                res = fa;
            }
            k++;
            it++;
        }
        if (!(res == res)) break;
    }
done:
    st->tol_override = 0;
    *value = xv;
    *error = res;
    *iterations = it;
    if (rc) return rc;
    return fabs(res) <= tol ? NM_OK : NM_ERR_NOT_CONVERGED;
}

void orc_destroy(orc_state* st) {
    if (st) { free(st->amt_n); free(st->amt_theta); free(st->amt_phibulk); }
    if (!st) return;
    for (int m = 0; m < st->P->n_mol; m++) {
        free(st->Gf[m]); free(st->rho[m]); free(st->jGb[m]); free(st->Pc[m]); free(st->Qb[m]);
    }
    free(st->Gf); free(st->rho); free(st->jGb); free(st->Pc); free(st->Qb);
    free(st->u); free(st->G1); free(st->phi); free(st->phi_side); free(st->phitot);
    free(st->alpha); free(st->tmp); free(st->unity); free(st->gb); free(st->mol_phitot);
    free(st->GN); free(st->norm); free(st->mol_n); free(st->mol_theta); free(st->mol_phibulk);
    free(st->seg_phibulk);
    free(st->psi); free(st->EE); free(st->q); free(st->eps); free(st->X);
    free(st->gb3); free(st->m2l1); free(st->m2l11); free(st->m2l_1); free(st->m2l_11);
    free(st->ust); free(st->ast); free(st->sp_phibulk); free(st->in_mol); free(st->st_ab); free(st->mol_charge);
    free(st);
}
