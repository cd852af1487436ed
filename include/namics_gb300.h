/*
 * namics_gb300 — GB300-native Scheutjens–Fleer SCF hot path behind a C ABI.
 *
 * The entry points below replace, one for one, the reference's hot path for
 * an SCF solve (leermakers/Namics; all citations are file:line into its
 * src/ directory):
 *
 *   Lattice  (lattice.h:123-155)  propagate / Side / set_bounds /
 *                                 ComputeGN / AddPhiS / WeightedSum
 *   Molecule (molecule.h:185-197) ComputePhi, propagate_forward/backward
 *   System   (system.cpp:2087)    Classical_residual (+ ComputePhis,
 *                                 PutU, PrepareForCalculations)
 *   SFNewton (sfnewton.h:102)     iterate_DIIS, DIIS, Ax, computeresidual
 *   System   (system.cpp:2809,3038,3246) GetFreeEnergy,
 *                                 GetGrandPotential, CreateMu
 *
 * Plain C types only.  Arrays named *_dev are device pointers (cudaMalloc'd
 * or any CUDA-visible allocation); all other arrays are host pointers.
 * Every entry point returns NM_OK (0) or a negative status; the reference's
 * integer exceptions map onto NM_ERR_GN (-1, system.cpp:2402),
 * NM_ERR_NAN_DIIS (-2, sfnewton.cpp:808), NM_ERR_NAN_SVD (-3,
 * tools.cpp:1225) and NM_ERR_NEG_SOLVENT (-4, system.cpp:2524).
 * nm_last_error() returns a thread-local message for the last failure.
 *
 * Layout: identical to the reference (lattice.cpp:245-254).  Sites are
 * padded by one halo layer per side; index = x*JX + y*JY + z with
 * 1-D: M=MX+2, JX=1; 2-D: M=(MX+2)(MY+2), JX=MY+2, JY=1;
 * 3-D: M=(MX+2)(MY+2)(MZ+2), JX=(MY+2)(MZ+2), JY=MZ+2.
 * The iteration vector x (and the residual g) is [n_it blocks of M]
 * (solve_scf.cpp:79-85), the same as the reference's `xx`.
 */
#ifndef NAMICS_GB300_H
#define NAMICS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define NM_OK               0
#define NM_ERR_GN          -1   /* G(N) <= 0 for a restricted molecule      */
#define NM_ERR_NAN_DIIS    -2   /* NaN in the DIIS matrix                   */
#define NM_ERR_NAN_SVD     -3   /* NaN in the small DIIS solve              */
#define NM_ERR_NEG_SOLVENT -4   /* solvent bulk volume fraction < 0         */
#define NM_ERR_INPUT      -10   /* input text not understood / unsupported  */
#define NM_ERR_CUDA       -11   /* CUDA runtime error                       */
#define NM_ERR_ARG        -12   /* bad argument                             */
#define NM_ERR_NOMEM      -13   /* device allocation failed                 */
#define NM_ERR_NOT_CONVERGED -14 /* iteration limit reached (solve only)   */
#define NM_ERR_TIMEOUT    -15   /* a bounded device wait gave up            */

/* ---- enumerations (values are part of the ABI) -------------------------- */
enum nm_geometry  { NM_PLANAR = 0, NM_CYLINDRICAL = 1, NM_SPHERICAL = 2 };
enum nm_lattype   { NM_SIMPLE_CUBIC = 0, NM_HEXAGONAL = 1 };
enum nm_bc        { NM_BC_MIRROR = 0, NM_BC_PERIODIC = 1, NM_BC_SURFACE = 2 };
enum nm_segfree   { NM_SEG_FREE = 0, NM_SEG_PINNED = 1, NM_SEG_FROZEN = 2 };
enum nm_molfree   { NM_MOL_FREE = 0, NM_MOL_RESTRICTED = 1, NM_MOL_SOLVENT = 2,
                    NM_MOL_NEUTRALIZER = 3 };
enum nm_precision { NM_FP64 = 0, NM_FP32 = 1 };

/* ---- compiled problem ("plan") -------------------------------------------
 * Produced on the host from Namics input text by nm_plan_create().  It holds
 * every per-site constant the hot path needs (masks, curvature weights) and
 * each molecule as a tree of blocks.  Read-only for callers.               */

/* One block: a run of `length` bonded segments of one segment type.  Blocks
 * form a tree rooted at the molecule's last segment (linear chains), at the
 * first-written segment of a branched composition (mol_branched, reversed
 * numbering, molecule.cpp:1740-1766) or at the dendrimer core
 * (mol_dendrimer.cpp:113-184).  Children attach to the block's first
 * segment.  `mult` identical copies of the child subtree attach there
 * (dendrimer arms; 1 otherwise); `degeneracy` is the number of equivalent
 * copies of each segment of the block in one molecule (d_mon). */
typedef struct nm_block {
    int    seg;          /* segment type                                   */
    int    molmon;       /* index into the molecule's monomer list          */
    int    length;       /* segments in the run                             */
    int    s0;           /* storage index of the run's first segment        */
    int    parent;       /* parent block (-1 for the root block)            */
    int    mult;         /* copies of this subtree at the parent's join      */
    double degeneracy;   /* d_mon                                           */
    int    n_child;      /* child blocks (each a distinct group)             */
    int    child0;       /* offset of this block's children in child_index  */
} nm_block;

typedef struct nm_molecule {
    int    freedom;          /* enum nm_molfree                              */
    int    pinned;           /* contains a pinned segment (IsPinned)         */
    double n, theta, phibulk;/* input values (restricted: n/theta; free: φb) */
    double chainlength;      /* N (with degeneracies)                        */
    int    n_molmon;         /* distinct segment types in the molecule       */
    const int*    molmon_seg;      /* [n_molmon] segment type              */
    const double* molmon_fraction; /* [n_molmon] fraction(seg)             */
    int    n_blocks;
    const nm_block* blocks;  /* [n_blocks], forward (post-)order: children
                                come before their parent; root is last      */
    const int* child_index;  /* children lists                               */
    int    n_store;          /* forward propagators stored per site          */
    double charge;           /* Σ valence·fraction (Mol::Charge)             */
    int    markov;           /* 1; or 2: semiflexible chain, every propagator
                                resolved into FJC = 3 bond directions
                                (molecule.cpp:627-674, 1-gradient simple-cubic
                                lattices)                                    */
    double bend[3];          /* Markov 2: bond-angle weights P[k] of angles
                                k·π/2 (molecule.cpp:135-152); P[2] = 0       */
} nm_molecule;

typedef struct nm_plan {
    /* lattice (fjc = 1) */
    int    gradients, MX, MY, MZ;
    int    geometry, lattice_type, stencil_full;
    int    bc[6];            /* x-low, y-low, z-low, x-high, y-high, z-high  */
    int    JX, JY, M;
    double lambda;           /* 1/6 simple cubic, 1/4 hexagonal             */
    double offset_first_layer, bond_length, volume;
    const double* L;         /* [M] site volume (1 for planar)               */
    const double* lambda_1;  /* [M] curved-lattice weights, NULL if planar  */
    const double* lambda0;
    const double* lambda1;
    const int*    ksam;      /* [M] 0 on frozen sites, 1 elsewhere          */
    /* segments */
    int    n_seg;
    const char* const* seg_name;
    const int*    seg_freedom;   /* enum nm_segfree                         */
    const int*    seg_it;        /* iteration block of each segment, -1 frozen
                                    or with internal states (their states
                                    carry the blocks: state_it)          */
    const double* seg_gmask;     /* [n_seg*M] G1 = exp(-u)·gmask           */
    const double* seg_phi_frozen;/* [n_seg*M] frozen volume fraction       */
    const double* chi;           /* [n_seg*n_seg]                           */
    const double* seg_valence;   /* [n_seg]; 0 for a segment with internal
                                    states (its states carry the charge) */
    const double* seg_epsilon;   /* [n_seg]                                 */
    int    n_it;                 /* iteration species (ItMonList, then
                                    ItStateList)                          */
    const int*    it_seg;        /* [n_it] representative segment (a state
                                    block: the state's segment)           */
    int    iv;                   /* length of x: n_it*M (+M if charged)    */
    int    charged;
    /* molecules */
    int    n_mol;
    const nm_molecule* mols;
    int    solvent, neutralizer; /* molecule index or -1                   */
    /* solver (newton : ... keys) */
    int    diis_m, iterationlimit, max_norm;
    double tolerance, deltamax;
    /* molecule names, in the order of `mols` (the `mol : <name>` keys) */
    const char* const* mol_name;
    /* a search (`var` keys; Solve_scf::SuperIterate, solve_scf.cpp:717-750):
     * search_mol < 0 when the input defines none.  search_what: 0 θ, 1 n,
     * 2 φ_bulk of molecule search_mol.  target_kind: 0 the free energy, 1
     * the grand potential, 2 a molecule's quantity (target_mol,
     * target_what: 0 θ, 1 n, 2 φ_bulk, 3 μ); target_value its value.
     * super_* are the `newton : … : super_*` keys with the reference's
     * defaults (tolerance·10, iterationlimit/10, 0.5; solve_scf.cpp:153-177). */
    int    search_mol, search_what, target_kind, target_mol, target_what;
    double target_value;
    double super_tolerance, super_deltamax;
    int    super_iterationlimit;
    /* a scan (`var : mol-<name> : scan : theta|n|phibulk` with step,
     * end_value, scale, steps; Molecule::PutVarScan, molecule.cpp:785-815):
     * scan_mol < 0 when the input defines none; steps k = 0 .. scan_n, the
     * values from nm_plan_scan_value */
    int    scan_mol, scan_what, scan_n, scan_exponential;
    double scan_start, scan_end, scan_step;
    /* `mol : <name> : save_memory : true` on any molecule (the reference's
     * checkpointed propagator storage, molecule.cpp:174-186): a context
     * created with checkpoint_stride 0 then stores every k-th forward
     * propagator with the reference's slot count, round(√(2·N_block)) per
     * block.  Results are the same either way. */
    int    save_memory;
    /* internal states (`state : <name> : mon | valence | alphabulk |
     * chi_<X>`, State::CheckInput state.cpp:37-106, Segment::AddState
     * segment.cpp:1981-2016) and the reactions that fix their bulk
     * fractions (`reaction : <name> : equation | pK | K`, reaction.cpp:
     * 37-145).  n_state = 0 when the input defines none; the arrays below
     * are then NULL and n_sp = n_seg.  A segment with states interacts
     * through its states only: the interaction species are the segments
     * (those without states count) followed by the states, species
     * n_seg + j being state j. */
    int    n_state;
    const char* const* state_name;  /* [n_state] in the input's order      */
    const int*    state_seg;        /* [n_state] the state's segment       */
    const double* state_valence;    /* [n_state]                           */
    const double* state_alphabulk;  /* [n_state] fraction of the segment in
                                       this state in the bulk, solved from
                                       the reactions (Solve_scf::Solve's
                                       WEAK pre-iteration, solve_scf.cpp:
                                       562-603)                           */
    const int*    state_it;         /* [n_state] iteration block           */
    const int*    seg_nstate;       /* [n_seg] states of each segment       */
    int    n_sp;                    /* interaction species: n_seg + n_state */
    const double* chi_sp;           /* [n_sp*n_sp] χ between species (the
                                       reference's Seg::chi / State::chi
                                       rows, system.cpp:1775-1915)        */
    const int*    it_sp;            /* [n_it] species of each iteration
                                       block's representative (ItMonList,
                                       then ItStateList)                  */
    /* a scan of a fixed state's bulk fraction (`var : state-<name> : scan :
     * alphabulk`, State::PutVarScan / UpdateVarInfo, state.cpp:262-318):
     * the state's index, or -1.  Its steps use scan_n, scan_exponential,
     * scan_start (the input's alphabulk), scan_end and scan_step, and
     * nm_plan_scan_value gives their values; nm_ctx_set_values takes each as
     * `state : <name> : alphabulk`. */
    int    scan_state;
    /* a scan of a reaction's pK (`var : reaction-<name> : scan : pK`,
     * linear steps, Reaction::PutVarScan, reaction.cpp:390-408): the
     * reaction's index in input order, or -1; nm_ctx_set_values takes each
     * step as `reaction : <name> : pK` */
    int    scan_reaction;
} nm_plan;

/* Parse Namics input text (the `lat/mon/mol/sys/newton` key subset of the
 * first `start` block; input.cpp:3-78) into a plan.  Replaces the object
 * construction of namics.cpp:165-417 and the Check/Prepare steps of
 * Lattice, Segment, Molecule and System.  On error returns NM_ERR_INPUT. */
int  nm_plan_create(const char* input_text, nm_plan** out);
void nm_plan_destroy(nm_plan* plan);
const char* nm_last_error(void);
const char* nm_version(void);

/* ---- device context --------------------------------------------------- */
typedef struct nm_ctx nm_ctx;

typedef struct nm_ctx_options {
    int precision;           /* enum nm_precision for propagators           */
    int checkpoint_stride;   /* k > 1: store every k-th forward propagator of
                                each block (and its last), recompute the rest
                                in the backward sweep from the checkpoint
                                before them; 0: every propagator, unless the
                                plan asks for save_memory; 3-gradient
                                simple-cubic linear chains (other problems
                                store every propagator); same results     */
    int device;              /* CUDA device ordinal                          */
    void* stream;            /* cudaStream_t, NULL = a private stream       */
} nm_ctx_options;

/* Allocates all device state for one problem (fields, G1, propagators,
 * volume fractions, DIIS history).  Replaces the AllocateMemory chain
 * (solve_scf.cpp:67-106, system.cpp:100-190, molecule.cpp:130-270). */
int nm_ctx_create(const nm_plan* plan, const nm_ctx_options* opt, nm_ctx** out);
int nm_ctx_destroy(nm_ctx* ctx);

/* Context options.  NM_OPT_SWEEP2D (default 0): 1 runs each propagator
 * sweep of a 2-gradient linear-chain problem as one persistent cooperative
 * launch (CTAs synchronised per step through neighbour progress flags)
 * instead of one launch per segment step.  Same arithmetic, same results;
 * on GB300 the per-step launches are the faster of the two. */
#define NM_OPT_SWEEP2D 1
/* NM_OPT_ROWS3D (default 4): rows along y per block of the 3-D step kernels,
 * 2, 4 or 8.  NM_OPT_CHECKPOINT: the checkpoint stride of the 3-D path, 0
 * (every propagator) or k >= 2, within the propagator storage the context
 * was created with (NM_ERR_ARG when it does not fit).  Same results. */
#define NM_OPT_ROWS3D 2
#define NM_OPT_CHECKPOINT 3
/* NM_OPT_TILE3D (default 0): the 3-D steps as 2.5-D shared-memory tiles, a
 * block of R rows × 128 z marching along P planes, value R·100 + P (204,
 * 208, 404, 408); 0 keeps the gather kernel.  Same results. */
#define NM_OPT_TILE3D 4
/* NM_OPT_CLUSTER3D (default 0; the autotuner may pick it): the FP32 sweeps of a small
 * 3-D box (linear chains, every propagator stored, two propagator buffers
 * within the shared memory of a thread-block cluster of up to 16 CTAs) run
 * as one cluster launch per sweep, the propagators held in distributed
 * shared memory; 0 keeps one launch per step.  Same results, bit for bit;
 * NM_ERR_ARG asks for it where it does not apply. */
#define NM_OPT_CLUSTER3D 5
/* NM_OPT_DEVICE_LOOP (default 0): 1 runs nm_solve_dev (and the solves of a
 * search) as one CUDA graph with a conditional WHILE node: residual, field
 * update, DIIS and the stopping test all on the device, one host
 * synchronisation per solve instead of one per iteration.  The small DIIS
 * solve is the same pseudo-inverse, run by one warp: the same path up to
 * rounding.  Measured slower than the host-driven loop on GB300. */
#define NM_OPT_DEVICE_LOOP 6
int nm_ctx_set_option(nm_ctx* ctx, int option, int value);

/* The autotuner: times one residual evaluation of this context at the field
 * x_dev (device, length iv) for each candidate of its tunable kernel
 * choices, keeps the fastest and caches it for contexts of the same shape
 * (a later call with the same shape applies the cached choice untimed).
 * 3-D path: the step kernel (the gather kernel with 2, 4 or 8 rows per
 * block, or a 2.5-D tile 204, 208, 404, 408) × checkpoint stride {0, 5, 10}
 * (the strides that fit the storage), and on small FP32 boxes the cluster
 * sweeps (NM_OPT_CLUSTER3D); 2-D linear chains: one launch per step or
 * one persistent launch per sweep (NM_OPT_SWEEP2D); other contexts have no
 * choice to make.  Results are the same for every candidate. */
typedef struct nm_ctx_tuning {
    int    rows;               /* rows per block of the gather kernel (3-D), -1 where it does not apply */
    int    tile;               /* 3-D tile (R·100 + P), 0 for the gather kernel, -1 where it does not apply */
    int    checkpoint_stride;  /* 3-D checkpoint stride, -1 where it does not apply */
    int    sweep2d;            /* 2-D persistent sweeps, -1 where it does not apply */
    int    cluster3d;          /* 3-D FP32 cluster sweeps (NM_OPT_CLUSTER3D), -1 where they do not apply */
    int    candidates;         /* configurations timed (0: taken from the cache) */
    double ms_per_residual;    /* the chosen configuration's time (0 if cached) */
} nm_ctx_tuning;
int nm_ctx_autotune(nm_ctx* ctx, const double* x_dev, nm_ctx_tuning* out);

/* The value of step k (0 .. plan->scan_n) of the plan's scan
 * (Molecule::UpdateVarInfo, molecule.cpp:884-930): start + k·step, or on the
 * exponential scale 10^((1 - k/n)·log10(start) + (k/n)·log10(end)).  The
 * caller sets it with nm_ctx_set_values and solves, one step at a time.
 * NM_ERR_ARG without a scan or with k out of range. */
int nm_plan_scan_value(const nm_plan* plan, int k, double* value);

/* The bulk equilibrium of a plan with internal states, as Solve_scf::Solve
 * runs it before each solve (solve_scf.cpp:562-603): the fixed states'
 * alphabulk from fixed_ab [n_state] (entries of states the reactions set
 * are ignored; NULL: the input's), the reactions' pK from pK [reactions, in
 * input order] (NULL: the input's), and pK_eff from the species' bulk
 * volume fractions sp_phibulk [n_sp] of the previous solve (NULL before
 * any: pK_eff = pK).  Writes the states' bulk fractions [n_state] and the
 * molecules' bulk charges [n_mol] (either may be NULL).  NM_ERR_ARG without
 * states, NM_ERR_INPUT where the equilibrium cannot be solved. */
int nm_plan_state_bulk(const nm_plan* plan, const double* fixed_ab, const double* pK,
                       const double* sp_phibulk, double* alphabulk, double* mol_charge);

/* Scans (the reference's Variate: variate.cpp, solve_scf.cpp:717-868): change
 * values of a live context and solve again from its current field (a warm
 * start).  items: "mon : <seg> : chi_<seg>" (set both ways; not on a plan
 * with internal states), "mol : <mol> : n | theta" (restricted), "mol :
 * <mol> : phibulk" (free), "state : <state> : alphabulk" (a state whose
 * alphabulk the input fixes), "reaction : <reaction> : pK".  All are
 * applied, then checked: χ must keep
 * the iteration species (segments with equal χ rows) unchanged.  A state's
 * or a reaction's new value solves the bulk equilibrium again, its pK_eff from the bulk
 * volume fractions of the context's last residual, as the reference's next
 * solve does (Reaction::pKeff, reaction.cpp:253-266); the molecules' bulk
 * charges follow.  On error nothing changes (NM_ERR_ARG, NM_ERR_INPUT). */
int nm_ctx_set_values(nm_ctx* ctx, const char* const* items, const double* values, int n);

/* One residual evaluation g(x) on device buffers of length plan->iv.
 * Replaces Solve_scf::residuals -> System::Classical_residual
 * (solve_scf.cpp:752-908, system.cpp:2087-2189). */
int nm_residual_dev(nm_ctx* ctx, const double* x_dev, double* g_dev);

typedef struct nm_solve_result {
    int    iterations;
    double residual;         /* ‖g‖₂ (or max|g|) at exit                     */
    int    status;           /* NM_OK, NM_ERR_NOT_CONVERGED or an error     */
} nm_solve_result;

/* DIIS solve from the field x (device, length iv; updated in place).
 * Replaces SFNewton::iterate_DIIS (sfnewton.cpp:1037-1130). */
int nm_solve_dev(nm_ctx* ctx, double* x_dev, nm_solve_result* res);

typedef struct nm_search_result {
    double value;            /* the search variable at exit                 */
    double error;            /* the target's error there (Var->GetError)    */
    int    iterations;       /* the reference's search iteration count      */
    int    solves;           /* SCF solves run (evaluations of the error)   */
    int    status;           /* NM_OK, NM_ERR_NOT_CONVERGED or an error     */
} nm_search_result;

/* The plan's search: one molecule quantity varied until the target's error
 * is below super_tolerance.  Replaces Solve_scf::SuperIterate with
 * SFNewton::iterate_RF (sfnewton.cpp:1132-1185): the damped regula falsi on
 * the variable's scale relative to its value at each (re)start, every
 * evaluation a solve from the current field x (device, updated in place) to
 * super_tolerance.  The molecule's value is left at the search's result,
 * as nm_ctx_set_values would leave it.  NM_ERR_ARG when the plan has no
 * search. */
int nm_ctx_search(nm_ctx* ctx, double* x_dev, nm_search_result* res);

/* Same solve with host buffers: copies x in, solves, copies x back and the
 * per-segment volume fractions out (phi_host: [n_seg*M], may be NULL). */
int nm_solve_host(nm_ctx* ctx, double* x_host, double* phi_host,
                  nm_solve_result* res);

/* Results of the last residual evaluation (device -> host copies).
 * which: 0 segment φ [n_seg*M], 1 G1 [n_seg*M], 2 α [M], 3 φ_tot [M],
 * 4 molecule φ_tot [n_mol*M], 5 φ_side [n_seg*M]; charged systems also
 * 6 ψ with mirror bounds [M], 7 charge density q [M], 8 relative
 * permittivity ε [M] (every site, halo layers included); plans with
 * internal states also 9 the states' φ, 10 their fractions α of the
 * segment's sites and 11 their potentials u, each [n_state*M]
 * (Segment::phi_state, alpha, u; segment.cpp:861-873, 1337-1343). */
int nm_get_field(nm_ctx* ctx, int which, double* out_host);

/* Per-molecule scalars of the last residual: GN, n, θ, φ_bulk.  Restricted
 * molecules report their input n and θ; free ones, the solvent and the
 * neutraliser n = norm·GN and θ = n·N (the reference's Molecule::n, theta). */
int nm_get_molecule(nm_ctx* ctx, int mol, double* GN, double* n,
                    double* theta, double* phibulk);

/* Free energy, grand potential and chemical potentials (mu: [n_mol]) of
 * the state of the last residual evaluation (system.cpp:2809-3244). */
int nm_free_energy(nm_ctx* ctx, double* F, double* Omega, double* mu);

/* Outputs of the last residual evaluation in the reference's file layouts
 * (Output::WriteOutput, output.cpp:385-564; LGrad*::PutProfiles).  items:
 * the `key : name : property` triples of an input's output block.
 * nm_write_pro: profiles, interior sites, one row per site ("mon : <seg> :
 * phi|G1", "mol : <mol> : phi", "sys : <any> : alpha|phitot", charged also
 * "sys : <any> : psi|q|eps").  nm_write_kal: one header line (unless
 * append) and one line of scalars ("sys : <any> : free_energy|
 * grand_potential", "newton : <any> : residual|iterations" from res,
 * "mol : <mol> : GN|n|theta|phibulk|Mu").  An unknown item is NM_ERR_ARG. */
int nm_write_pro(nm_ctx* ctx, const char* path, const char* const* items, int n_items);
int nm_write_kal(nm_ctx* ctx, const char* path, const char* const* items, int n_items,
                 const nm_solve_result* res, int append);

/* Unit-testable pieces on device arrays of length M.
 * nm_propagate: G_out = Side(set_bounds(G_in))·G1 (Lattice::propagate,
 * LG1Planar.cpp:138-159, LGrad1.cpp:432-454, LG2Planar.cpp:1039-1127,
 * LGrad2.cpp:1053-1090, LGrad3.cpp:673-744).  G_in's halo is updated in
 * place by set_bounds, as in the reference.  G1 may be NULL (≡1).
 * nm_side: X_side = Side(X) (Lattice::Side) without set_bounds. */
int nm_propagate_dev(nm_ctx* ctx, double* G_in_dev, const double* G1_dev,
                     double* G_out_dev);
int nm_side_dev(nm_ctx* ctx, const double* X_dev, double* X_side_dev);

/* Lattice and molecule pieces for a caller that keeps the reference's own
 * Molecule::ComputePhi loop (molecule.h:185-197) and moves its arithmetic
 * to the device.  Device arrays of length M (n_molmon·M for rho), the
 * reference's padded layout; all M entries, halo layers included, as the
 * reference's flat-array loops.  Markov-1 chains.
 * nm_add_phi_dev:      phi += Gf·Gb           Lattice::AddPhiS(phi,Gf,Gb,Markov,M)
 * nm_add_phi_deg_dev:  phi += d·Gf·Gb         AddPhiS(phi,Gf,Gb,degeneracy,Markov,M)
 * nm_add_phi_norm_dev: phi += norm·Gf·Gb/G1 where G1 > 0
 *                      AddPhiS(phi,Gf,Gb,G1,norm,Markov,M) (LGrad1.cpp:924-941);
 *                      2 and 3 gradients: NM_ERR_INPUT, phi unchanged (the
 *                      reference prints "not implemented" there)
 * nm_initiate_dev:     G = Gz                 Lattice::Initiate (LGrad1.cpp:943-949)
 * nm_terminate_dev:    Gz = G                 Lattice::Terminate (LGrad1.cpp:951-969,
 *                      LGrad2.cpp:1934-1960, LGrad3.cpp:1937-1950)
 * nm_weighted_sum_dev, nm_compute_gn_dev: zero X's halo in place
 *                      (remove_bounds), then Σ X (planar, 3-D) or Σ X·L
 *                      (curved): Lattice::WeightedSum, ComputeGN
 *                      (LGrad1.cpp:213-220, 863-874; LGrad2.cpp:147-157;
 *                      LGrad3.cpp:40-46)
 * nm_compose_dev:      Molecule::ComputePhi of molecule `mol` at the field
 *                      x (mol_linear.cpp:12-135, mol_branched.cpp:170-418,
 *                      mol_dendrimer.cpp:113-184): G1 from x, forward
 *                      sweep, G(N), backward sweep with the composition;
 *                      rho_dev [n_molmon·M] = Σ d·Gf·Gb per segment type of
 *                      the molecule (before the division by G1 and the
 *                      normalisation of System::ComputePhis), GN = G(N). */
int nm_add_phi_dev(nm_ctx* ctx, double* phi_dev, const double* Gf_dev, const double* Gb_dev);
int nm_add_phi_deg_dev(nm_ctx* ctx, double* phi_dev, const double* Gf_dev, const double* Gb_dev,
                       double degeneracy);
int nm_add_phi_norm_dev(nm_ctx* ctx, double* phi_dev, const double* Gf_dev, const double* Gb_dev,
                        const double* G1_dev, double norm);
int nm_initiate_dev(nm_ctx* ctx, double* G_dev, const double* Gz_dev);
int nm_terminate_dev(nm_ctx* ctx, double* Gz_dev, const double* G_dev);
int nm_weighted_sum_dev(nm_ctx* ctx, double* X_dev, double* sum);
int nm_compute_gn_dev(nm_ctx* ctx, double* G_dev, double* GN);
int nm_compose_dev(nm_ctx* ctx, int mol, const double* x_dev, double* rho_dev, double* GN);

/* Device launches issued by this context since creation (diagnostics). */
long long nm_ctx_launch_count(nm_ctx* ctx);

/* ---- batched 1-gradient solver ------------------------------------------
 * Many independent 1-gradient problems solved to convergence in one
 * persistent launch: a device-resident work loop of resident CTAs ("slots",
 * as many as fit on the device, at most one per problem), each taking the
 * next problem from a queue in device memory (longest first) as soon as its
 * previous one converged, with DIIS on the device.  Stored propagators and
 * DIIS histories live in the slot's scratch; fields x and residuals g are
 * per problem.  With NM_FP32 a problem starts with FP32 propagators and a
 * 5-deep DIIS history (at most the input's m) and switches to FP64 residuals
 * with the input's m, history restarted, at the FP32 accuracy floor
 * (1e-7·N + 1e-6), on a stall near it, or on any FP32 failure; its stopping
 * test is always made on an FP64 residual.  NM_FP64 runs the reference's
 * DIIS throughout. */
typedef struct nm_batch nm_batch;

int nm_batch_create(const nm_plan* const* plans, int n_plans,
                    const nm_ctx_options* opt, nm_batch** out);
int nm_batch_destroy(nm_batch* b);
/* x_dev: concatenated iteration vectors (offsets from nm_batch_offsets);
 * updated in place.  iterations/residual/status: [n_plans] host arrays. */
int nm_batch_solve_dev(nm_batch* b, double* x_dev, int* iterations,
                       double* residual, int* status);
int nm_batch_solve_host(nm_batch* b, double* x_host, int* iterations,
                        double* residual, int* status);
/* element offset of problem i's x in the concatenated vector; total in
 * offsets[n_plans] */
int nm_batch_offsets(nm_batch* b, long long* offsets);
/* One residual evaluation g(x) per problem (no DIIS), FP64 or FP32
 * propagators; x_dev and g_dev are concatenated like nm_batch_solve_dev. */
int nm_batch_residual_dev(nm_batch* b, const double* x_dev, double* g_dev, int precision);
/* per-problem iteration counts of the FP32-propagator phase of the last
 * solve (0 for FP64 batches) */
int nm_batch_stats(nm_batch* b, int* fp32_iterations);
/* per-problem time to convergence in the last solve: seconds from the
 * start of the batch's first CTA to the end of the problem's CTA (device
 * global timer), [n_plans] host array */
int nm_batch_times(nm_batch* b, double* seconds);
/* per-problem seconds of the last solve (device global timer): from the
 * start of the work loop to the problem's start in a slot (queued), and
 * from its start to its convergence (solving); either may be NULL */
int nm_batch_timings(nm_batch* b, double* queued, double* solving);
/* resident CTAs (slots) of the batch's work loop; nm_batch_set_slots runs
 * later solves on fewer of them (1 .. the number fixed at creation: as many
 * as fit on the device, at most one per problem) with identical results */
int nm_batch_slots(nm_batch* b);
int nm_batch_set_slots(nm_batch* b, int slots);
/* The work loop's autotuner: solves the batch from x_dev (not changed) once
 * per candidate number of resident CTAs per SM (1 up to what fits), keeps
 * the one with the highest steady throughput (slots × problems / the sum of
 * the problems' solve times: the rate of a long stream, not one batch's
 * wall time, which its longest solves set) for later solves and remembers
 * it for batches of the same shape (a later call applies it untimed).
 * Results are the same for every candidate. */
typedef struct nm_batch_tuning {
    int    ctas_per_sm;        /* the choice                                   */
    int    slots;              /* resident CTAs it gives                        */
    int    candidates;         /* solves timed (0: taken from the cache)        */
    double ms_per_solve;       /* the chosen configuration's batch time (0 if cached) */
} nm_batch_tuning;
int nm_batch_autotune(nm_batch* b, const double* x_dev, nm_batch_tuning* out);
/* per-problem free energy / grand potential of the final state */
int nm_batch_free_energy(nm_batch* b, double* F, double* Omega);
long long nm_batch_launch_count(nm_batch* b);

/* ---- streaming work loop (continuous batching of 1-gradient solves) -------
 * No single counterpart in the reference (it runs one Solve at a time): a
 * persistent launch whose resident CTAs ("slots") take 1-gradient solves
 * from a ring the host appends to while the loop runs.  A request is
 * admitted the moment a slot is free, its field, stored propagators and
 * DIIS history stay in the slot's device memory until it has converged, and
 * its result is handed back through pinned host memory; nothing waits for
 * other requests.  The ring, the fields and the results live in pinned host
 * memory mapped into the device.  A CTA without work for idle_seconds
 * leaves the loop; the next request (or a waiter) launches it again.
 * Requests must fit the envelope given at creation (it sizes the slots and
 * the ring's per-request space); a request outside it is NM_ERR_INPUT. */
typedef struct nm_stream nm_stream;
typedef struct nm_stream_options {
    int    device;
    int    capacity;       /* ring entries: requests submitted and not yet waited for */
    int    max_layers;     /* largest MX admitted (<= 512)                      */
    int    max_segments;   /* segment types (<= 16)                             */
    int    max_pairs;      /* (molecule, segment type) pairs (<= 32)            */
    int    max_molecules;  /* molecules (<= 16)                                 */
    int    max_store;      /* stored propagators, summed over the molecules     */
    int    max_blocks;     /* blocks, summed over the molecules                 */
    int    max_diis;       /* DIIS history m (<= 12)                            */
    int    slots;          /* resident CTAs; 0: as many as fit on the device    */
    double idle_seconds;   /* a CTA without work this long leaves; 0: 0.2 s     */
} nm_stream_options;
int nm_stream_create(const nm_stream_options* opt, nm_stream** out);
/* Queue one solve of `plan` (a 1-gradient, uncharged problem; the plan may
 * be destroyed after the call) from the field x_host (plan->iv values,
 * copied), with FP32-first (NM_FP32) or FP64 (NM_FP64) propagators.
 * NM_ERR_NOMEM when the ring is full of requests not yet waited for. */
int nm_stream_submit(nm_stream* s, const nm_plan* plan, const double* x_host, int precision,
                     long long* ticket);
/* Block until the request is solved: the field (may be NULL), the result,
 * and the seconds from submit to the solve's end (host clock).  Returns
 * NM_OK for a converged or iteration-limited solve (see res->status). */
int nm_stream_wait(nm_stream* s, long long ticket, double* x_host, nm_solve_result* res,
                   double* seconds);
int nm_stream_slots(nm_stream* s);
long long nm_stream_launch_count(nm_stream* s);
/* Stops the loop (requests not yet claimed are dropped) and frees it. */
int nm_stream_destroy(nm_stream* s);

/* ---- request server (continuous batching on one GPU) ----------------------
 * No single counterpart in the reference (it runs one Solve at a time): a
 * stream of independent solves of any gradient count, served while others
 * run.  1-gradient requests go to a streaming work loop (below) unless
 * stream_slots is -1 or the request falls outside its envelope.  `workers`
 * threads, one CUDA stream each, take the other requests from one FIFO
 * queue; 1-gradient requests waiting there together are solved in one
 * batched launch (up to max_batch), others one per device context.  Work of
 * the workers is admitted by estimated device footprint against
 * memory_budget bytes.
 * precision: NM_FP32 or NM_FP64 propagators (FP32 where the solver for the
 * request supports it, FP64 otherwise). */
typedef struct nm_server nm_server;
typedef struct nm_server_options {
    int    precision;        /* enum nm_precision                            */
    int    device;           /* CUDA device ordinal                          */
    int    workers;          /* concurrent solves (streams)                  */
    int    max_batch;        /* most 1-gradient requests per batched launch  */
    size_t memory_budget;    /* device bytes admitted requests may hold      */
    int    stream_slots;     /* 1-gradient requests go to a streaming work
                                loop (nm_stream_*) with this many resident
                                CTAs; 0: two per SM; -1: no loop, batched
                                launches only.  The loop's memory is fixed
                                at creation and outside memory_budget. */
    int    context_sweeps;   /* options of the 2-D and 3-D request contexts,
                                a bit mask: 1 persistent 2-D sweeps
                                (NM_OPT_SWEEP2D), 2 cluster sweeps of small
                                FP32 3-D boxes (NM_OPT_CLUSTER3D), 4 the
                                device-resident solve loop
                                (NM_OPT_DEVICE_LOOP); 0: one launch per
                                step and a host-driven loop.  Each applies
                                where the context supports it. */
} nm_server_options;
int nm_server_create(const nm_server_options* opt, nm_server** out);
/* Queue one solve from the field x_host (plan->iv values, copied).  The plan
 * must stay alive until the request has been waited for.  NM_ERR_NOMEM if
 * the request alone exceeds the memory budget. */
int nm_server_submit(nm_server* srv, const nm_plan* plan, const double* x_host,
                     long long* request_id);
/* Block until the request is done: the solved field (may be NULL), the solve
 * result and the seconds from submit to completion.  Returns the request's
 * status (a solve that hit its iteration limit returns NM_OK with
 * res->status = NM_ERR_NOT_CONVERGED). */
int nm_server_wait(nm_server* srv, long long request_id, double* x_host,
                   nm_solve_result* res, double* seconds);
long long nm_server_launch_count(nm_server* srv);
/* Finishes every queued request, then stops the workers. */
int nm_server_destroy(nm_server* srv);

/* ---- allocation-free single-problem solve --------------------------------
 * No counterpart in the reference.  For callers that cannot call the
 * device allocator when they solve: a host that hands out a fixed device
 * memory budget before work starts and owns every byte of it, or a
 * re-solve on a latency-critical path where an allocation could stall or
 * fail.  It
 * solves one 1-gradient problem with the batched solver's kernels, its
 * whole device scratch (descriptor, lattice arrays, stored propagators,
 * DIIS history, residual) carved from one static device array of
 * NM_NOALLOC_SCRATCH_BYTES compiled into the library.  A problem that needs
 * more is rejected with NM_ERR_INPUT and a message naming the limit.
 * The array's address is looked up on the first call for each device, with
 * that device current; make that first call before any stream capture.
 * All calls share the array: calls that overlap in time race on it.
 * x_dev: the plan's iteration vector (length iv), updated in place.
 * stream: cudaStream_t or NULL for the default stream; the call
 * synchronises that stream and returns the result on the host, after the
 * stream has finished the solve.  Returns res->status (NM_OK,
 * NM_ERR_NOT_CONVERGED or an error). */
#define NM_NOALLOC_SCRATCH_BYTES (8u << 20)
int nm_solve1d_noalloc(const nm_plan* plan, double* x_dev, int precision,
                       void* stream, nm_solve_result* res);

#ifdef __cplusplus
}
#endif
#endif /* NAMICS_GB300_H */
