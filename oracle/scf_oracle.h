/*
 * CPU oracle for the Namics SCF hot path — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference algorithm (leermakers/Namics,
 * file:line citations into its src/ directory at each function in
 * scf_oracle.c), used by tests/ as the parity checker and by bench.py as the
 * timed CPU baseline.  The product (namics_gb300/) never links or calls it.
 * The oracle is pinned against outputs of the reference program itself
 * (tests/golden/, produced by tests/golden/make_golden.py from the unmodified
 * reference built by oracle/Makefile.ref).
 */
#ifndef SCF_ORACLE_H
#define SCF_ORACLE_H
#include "../include/namics_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_state orc_state;

orc_state* orc_create(const nm_plan* plan);
void orc_destroy(orc_state* st);
/* g(x); both length plan->iv.  Returns NM_OK or a reference error code. */
int orc_residual(orc_state* st, const double* x, double* g);
/* DIIS solve (iterate_DIIS) from x (updated in place). */
int orc_solve(orc_state* st, double* x, int* iterations, double* residual);
/* same, but stops after `max_iter` iterations regardless of the plan */
int orc_solve_n(orc_state* st, double* x, int max_iter, int* iterations, double* residual);
/* fields of the last residual: same `which` codes as nm_get_field */
int orc_get_field(orc_state* st, int which, double* out);
int orc_get_molecule(orc_state* st, int mol, double* GN, double* n, double* theta,
                     double* phibulk);
/* bulk volume fractions of the interaction species [n_seg + n_state] */
int orc_get_species_phibulk(orc_state* st, double* out);
int orc_free_energy(orc_state* st, double* F, double* Omega, double* mu);
/* a molecule amount in force for the next solves (what: 0 θ, 1 n, 2 φ_bulk),
 * and the plan's search from x (updated in place) */
int orc_set_amount(orc_state* st, int mol, int what, double value);
/* the states' bulk fractions in force for the next solves [n_state] (a scan
 * of a fixed state's alphabulk; the bulk equilibrium is the caller's) */
int orc_set_states(orc_state* st, const double* alphabulk);
int orc_search(orc_state* st, double* x, double* value, double* error, int* iterations, int* solves);
/* Molecule::ComputePhi of molecule m at the field x: rho [n_molmon*M] =
 * Σ d·Gf·Gb per segment type (before System::ComputePhis divides by G1 and
 * normalises), GN = G(N) */
int orc_compose(orc_state* st, const double* x, int m, double* rho, double* GN);
/* Lattice::propagate and Lattice::Side on one array of length M */
void orc_propagate(orc_state* st, double* G_in, const double* G1, double* G_out);
void orc_side(orc_state* st, double* X, double* X_side);

#ifdef __cplusplus
}
#endif
#endif
