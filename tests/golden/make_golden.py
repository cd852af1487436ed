"""Generate the golden fixtures in tests/golden/*.json from the reference.

Each case is a Namics input file plus a seeded initial field.  The field is
written as a reference guess file (the format Lattice::ReadGuess reads,
lattice.cpp:926-968, at %.17e) and the unmodified reference program
(oracle/_ref/namics, built by oracle/Makefile.ref from the reference sources)
is run on it.  Its .pro profiles (%.20g) and .kal scalars (%.16e) are parsed
and stored, together with the input text and the field, so the tests can
replay the same problem through the oracle and the GPU path without the
reference present.

Run from the repository root:  python tests/golden/make_golden.py
(--raw: the verbatim output files; --keys: which input keys the reference
accepts; --search, --scan: the reference's `var` searches and scans)
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
GOLDEN = Path(__file__).resolve().parent
REF_BIN = ROOT / "oracle" / "_ref" / "namics"

from namics_gb300 import Plan  # noqa: E402  (plan compiler only: no GPU needed)


def lat1d(n, lower="surface", upper="mirror", geom="planar", lattype="simple_cubic", offset=None):
    s = [f"lat : flat : n_layers : {n}", f"lat : flat : lattice_type : {lattype}",
         f"lat : flat : geometry : {geom}", "lat : flat : gradients : 1",
         f"lat : flat : lowerbound : {lower}", f"lat : flat : upperbound : {upper}"]
    if offset is not None:
        s.append(f"lat : flat : offset_first_layer : {offset}")
    return s


def lat2d(nx, ny, bcs, geom="planar", lattype="simple_cubic", offset=None):
    s = ["lat : flat : gradients : 2", f"lat : flat : n_layers_x : {nx}", f"lat : flat : n_layers_y : {ny}",
         f"lat : flat : geometry : {geom}", f"lat : flat : lattice_type : {lattype}"]
    for k, v in zip(["lowerbound_x", "upperbound_x", "lowerbound_y", "upperbound_y"], bcs):
        s.append(f"lat : flat : {k} : {v}")
    if offset is not None:
        s.append(f"lat : flat : offset_first_layer : {offset}")
    return s


def lat3d(n, bc="periodic", lattype="simple_cubic"):
    s = ["lat : flat : gradients : 3", f"lat : flat : n_layers_x : {n[0]}", f"lat : flat : n_layers_y : {n[1]}",
         f"lat : flat : n_layers_z : {n[2]}", "lat : flat : geometry : planar", f"lat : flat : lattice_type : {lattype}"]
    for ax in "xyz":
        s += [f"lat : flat : lowerbound_{ax} : {bc}", f"lat : flat : upperbound_{ax} : {bc}"]
    return s


def brush_lines(comp, n=None, theta=None, chi=0.5, chi_s=None, wall=True, pinned_range="firstlayer"):
    s = []
    if wall:
        s += ["mon : S : freedom : frozen", "mon : S : frozen_range : lowerbound"]
    s += ["mon : X : freedom : pinned", f"mon : X : pinned_range : {pinned_range}",
          "mon : A : freedom : free", "mon : W : freedom : free",
          f"mon : A : chi_W : {chi}", f"mon : X : chi_W : {chi}"]
    if chi_s is not None and wall:
        s += [f"mon : A : chi_S : {chi_s}", f"mon : X : chi_S : {chi_s}"]
    s += [f"mol : pol : composition : {comp}", "mol : pol : freedom : restricted"]
    s += [f"mol : pol : n : {n}"] if n is not None else [f"mol : pol : theta : {theta}"]
    s += ["mol : water : composition : (W)1", "mol : water : freedom : solvent"]
    return s


def newton(tol=1e-7, dmax=0.1, itlim=1000, m=10):
    return ["newton : isaac : method : DIIS", f"newton : isaac : tolerance : {tol}",
            f"newton : isaac : deltamax : {dmax}", f"newton : isaac : iterationlimit : {itlim}",
            f"newton : isaac : m : {m}", "newton : isaac : e_info : false"]


def cases() -> list[dict]:
    C = []
    # 1-gradient planar simple-cubic brush, 100 layers, A_100 (X1A99) at σ=0.05
    base = lat1d(100) + brush_lines("(X)1(A)99", n=0.05, chi=0.5)
    C.append(dict(name="brush1d_x100", lines=base, field=(-0.01, 0.01), seed=1, modes=["it0", "conv"]))
    # 3-arm star brush (the star variant of the batched workload)
    C.append(dict(name="star1d", lines=lat1d(80) + brush_lines("(X)1(A)19[(A)20](A)20", n=0.04, chi=0.4),
                  field=(-0.01, 0.01), seed=2, modes=["it0", "conv"]))
    # hexagonal planar brush with an adsorbing wall
    C.append(dict(name="brush1d_hex", lines=lat1d(60, lattype="hexagonal") +
                  brush_lines("(X)1(A)39", n=0.03, chi=0.8, chi_s=-0.5),
                  field=(-0.05, 0.05), seed=3, modes=["it0", "conv"]))
    # spherical brush
    C.append(dict(name="brush1d_sph", lines=lat1d(50, geom="spherical", offset=5) +
                  brush_lines("(X)1(A)29", theta=600, chi=0.3),
                  field=(-0.02, 0.02), seed=4, modes=["it0", "conv"]))
    # cylindrical homopolymer adsorption, hexagonal, free chains
    lines = lat1d(40, geom="cylindrical", lattype="hexagonal", offset=3) + [
        "mon : S : freedom : frozen", "mon : S : frozen_range : lowerbound",
        "mon : A : freedom : free", "mon : W : freedom : free", "mon : A : chi_S : -1.2",
        "mon : A : chi_W : 0.2",
        "mol : pol : composition : (A)30", "mol : pol : freedom : free", "mol : pol : phibulk : 0.01",
        "mol : water : composition : (W)1", "mol : water : freedom : solvent"]
    C.append(dict(name="ads1d_cyl_hex", lines=lines, field=(-0.05, 0.05), seed=5, modes=["it0", "conv"]))
    # symmetric dendrimer near an adsorbing wall
    lines = lat1d(40) + ["mon : S : freedom : frozen", "mon : S : frozen_range : lowerbound",
                         "mon : A : freedom : free", "mon : B : freedom : free", "mon : W : freedom : free",
                         "mon : A : chi_S : -0.8", "mon : B : chi_W : 0.6",
                         "mol : pol : composition : @dend(A,(B)3,3; A,(A)2(B)2,2)",
                         "mol : pol : freedom : restricted", "mol : pol : theta : 4",
                         "mol : water : composition : (W)1", "mol : water : freedom : solvent"]
    C.append(dict(name="dend1d", lines=lines, field=(-0.05, 0.05), seed=6, modes=["it0", "conv"]))
    # asymmetric dendrimers (several arm types per generation): near the wall,
    # in a 2-gradient box, and a 5-arm star grafted through its one odd arm
    asym = [ln.replace("@dend(A,(B)3,3; A,(A)2(B)2,2)", "@dend(A,(B)3,2,(A)2(B)4,1; A,(A)2(B)2,2,(B)3,1)")
            for ln in lines]
    C.append(dict(name="asym_dend1d", lines=asym, field=(-0.05, 0.05), seed=12, modes=["it0", "conv"]))
    lines2 = lat2d(20, 14, ["surface", "mirror", "mirror", "mirror"]) + [
        "mon : S : freedom : frozen", "mon : S : frozen_range : lowerbound",
        "mon : A : freedom : free", "mon : B : freedom : free", "mon : W : freedom : free",
        "mon : A : chi_S : -1", "mon : B : chi_W : 0.4",
        "mol : pol : composition : @dend(A,(B)4,2,(A)1(B)2,1; A,(B)3,2)",
        "mol : pol : freedom : free", "mol : pol : phibulk : 0.002",
        "mol : water : composition : (W)1", "mol : water : freedom : solvent"]
    C.append(dict(name="asym_dend2d", lines=lines2, field=(-0.05, 0.05), seed=13, modes=["it0", "conv"]))
    C.append(dict(name="asym_star1d", lines=lat1d(60) + brush_lines("@dend(A,(A)15,4,(A)14(X)1,1)", n=0.02, chi=0.4),
                  field=(-0.01, 0.01), seed=14, modes=["it0", "conv"]))
    # 2-gradient planar adsorption (the 2-D requests of the request stream, reduced size)
    lines = lat2d(24, 16, ["surface", "mirror", "mirror", "mirror"]) + [
        "mon : S : freedom : frozen", "mon : S : frozen_range : lowerbound",
        "mon : A : freedom : free", "mon : W : freedom : free", "mon : A : chi_S : -1",
        "mol : pol : composition : (A)40", "mol : pol : freedom : free", "mol : pol : phibulk : 1e-3",
        "mol : water : composition : (W)1", "mol : water : freedom : solvent"]
    C.append(dict(name="ads2d", lines=lines, field=(-0.05, 0.05), seed=7, modes=["it0", "conv"]))
    # 2-gradient hexagonal planar, periodic y
    lines = lat2d(16, 12, ["surface", "mirror", "periodic", "periodic"], lattype="hexagonal") + [
        "mon : S : freedom : frozen", "mon : S : frozen_range : lowerbound",
        "mon : A : freedom : free", "mon : W : freedom : free", "mon : A : chi_S : -1.5",
        "mon : A : chi_W : 0.4",
        "mol : pol : composition : (A)20", "mol : pol : freedom : free", "mol : pol : phibulk : 0.01",
        "mol : water : composition : (W)1", "mol : water : freedom : solvent"]
    C.append(dict(name="ads2d_hex", lines=lines, field=(-0.05, 0.05), seed=8, modes=["it0", "conv"]))
    # 2-gradient cylindrical brush (the charged cylindrical brush's geometry, uncharged, reduced)
    lines = lat2d(20, 10, ["surface", "mirror", "mirror", "mirror"], geom="cylindrical", offset=10) + \
        brush_lines("(X)1(A)39", n=12.0, chi=0.5, pinned_range="firstlayer")
    C.append(dict(name="brush2d_cyl", lines=lines, field=(-0.02, 0.02), seed=9, modes=["it0", "conv"]))
    # 3-gradient periodic diblock melt (the 128³ melt, reduced size)
    lines = lat3d((10, 10, 10)) + ["mon : A : freedom : free", "mon : B : freedom : free", "mon : A : chi_B : 0.3",
                                   "mol : AB : composition : (A)10(B)10", "mol : AB : freedom : solvent"]
    C.append(dict(name="melt3d", lines=lines, field=(-0.1, 0.1), seed=10, antisym=True,
                  modes=["it0", "it5"], newton=dict(dmax=0.01)))
    # 3-gradient hexagonal, mirror bounds, homopolymer in solvent
    lines = lat3d((8, 7, 6), bc="mirror", lattype="hexagonal") + [
        "mon : A : freedom : free", "mon : W : freedom : free", "mon : A : chi_W : 0.8",
        "mol : pol : composition : (A)12", "mol : pol : freedom : free", "mol : pol : phibulk : 0.1",
        "mol : water : composition : (W)1", "mol : water : freedom : solvent"]
    C.append(dict(name="sol3d_hex", lines=lines, field=(-0.1, 0.1), seed=11, modes=["it0", "it5"]))
    # charged grafted polyelectrolyte brushes (valence -0.1 on A) with a
    # neutralising counter-ion (Na) and added salt (Cl at phi_b 0.01), on the
    # four lattices the electrostatics covers (the charged cylindrical brush class, reduced)
    def charged_lines(comp, n):
        return ["lat : flat : bondlength : 5e-10",
                "mon : S : freedom : frozen", "mon : S : frozen_range : lowerbound",
                "mon : X : freedom : pinned", "mon : X : pinned_range : firstlayer",
                "mon : A : freedom : free", "mon : A : valence : -0.1",
                "mon : W : freedom : free",
                "mon : Na : freedom : free", "mon : Na : valence : 1",
                "mon : Cl : freedom : free", "mon : Cl : valence : -1",
                "mon : A : chi_W : 0.5", "mon : X : chi_W : 0.5",
                f"mol : pol : composition : {comp}", "mol : pol : freedom : restricted", f"mol : pol : n : {n}",
                "mol : water : composition : (W)1", "mol : water : freedom : solvent",
                "mol : Na : composition : (Na)1", "mol : Na : freedom : neutralizer",
                "mol : Cl : composition : (Cl)1", "mol : Cl : freedom : free", "mol : Cl : phibulk : 0.01"]
    C.append(dict(name="charged1d", lines=lat1d(40) + charged_lines("(X)1(A)39", 0.05),
                  field=(-0.01, 0.01), seed=20, modes=["it0", "conv"], conv_itlim=5000))
    C.append(dict(name="charged1d_cyl", lines=lat1d(30, geom="cylindrical", offset=10) +
                  charged_lines("(X)1(A)29", 3.0), field=(-0.01, 0.01), seed=21, modes=["it0", "conv"],
                  conv_itlim=5000, split_tol=1e-4))
    C.append(dict(name="charged2d", lines=lat2d(16, 10, ["surface", "mirror", "mirror", "mirror"]) +
                  charged_lines("(X)1(A)29", 0.5), field=(-0.01, 0.01), seed=22, modes=["it0", "it5", "conv"],
                  newton=dict(tol=1e-6), conv_itlim=5000, path_tol=3e-6))
    C.append(dict(name="charged2d_cyl", lines=lat2d(16, 10, ["surface", "mirror", "mirror", "mirror"],
                  geom="cylindrical", offset=10) + charged_lines("(X)1(A)29", 10.0),
                  field=(-0.01, 0.01), seed=23, modes=["it0", "it5", "conv"], newton=dict(tol=1e-6),
                  conv_itlim=5000, split_tol=1e-2))
    # the other Poisson updates and halo stencils: 1-D spherical (Jacobi
    # update), 2-D hexagonal planar (hexagonal flat halo sums), and a charged
    # 3-arm star (the halo composition through a branch join)
    C.append(dict(name="charged1d_sph", lines=lat1d(30, geom="spherical", offset=10) +
                  charged_lines("(X)1(A)29", 20.0), field=(-0.01, 0.01), seed=24, modes=["it0", "it5", "conv"],
                  conv_itlim=5000))
    C.append(dict(name="charged2d_hex", lines=lat2d(16, 10, ["surface", "mirror", "mirror", "mirror"],
                                                      lattype="hexagonal") + charged_lines("(X)1(A)29", 0.5),
                  field=(-0.01, 0.01), seed=25, modes=["it0", "it5", "conv"], newton=dict(tol=1e-6),
                  conv_itlim=5000, path_tol=2e-5))
    C.append(dict(name="charged_star1d", lines=lat1d(40) + charged_lines("(X)1(A)9[(A)10](A)10", 0.04),
                  field=(-0.01, 0.01), seed=26, modes=["it0", "it5", "conv"], conv_itlim=5000))
    # 3-gradient charged brush: the 3-D Poisson update (a forward and a
    # backward Gauss-Seidel sweep) and the 3-D halo sums
    # (a 3-D wall is a frozen layer inside the box: the reference refuses
    # 'surface' bounds in 3-D)
    lat = lat3d((9, 6, 6), bc="mirror")
    wall = [ln.replace("frozen_range : lowerbound", "frozen_range : 1,1,1;1,6,6")
            .replace("pinned_range : firstlayer", "pinned_range : 2,1,1;2,6,6") for ln in charged_lines("(X)1(A)15", 1.8)]
    C.append(dict(name="charged3d", lines=lat + wall, field=(-0.01, 0.01), seed=27,
                  modes=["it0", "it5", "conv"], conv_itlim=5000, split_tol=2e-4))
    # Markov 2 (semiflexible) chains, 1-gradient simple cubic: a planar brush
    # (LG1Planar's steps), a spherical brush (LGrad1's curved steps) and a
    # free two-block chain adsorbing from solution (a segment-type change
    # inside the chain)
    m2 = lambda mol, k: [f"mol : {mol} : Markov : 2", f"mol : {mol} : k_stiff : {k}"]
    C.append(dict(name="markov2_brush1d", lines=lat1d(60) + brush_lines("(X)1(A)39", n=0.05, chi=0.5) +
                  m2("pol", 1), field=(-0.01, 0.01), seed=31, modes=["it0", "conv"]))
    C.append(dict(name="markov2_sph", lines=lat1d(40, geom="spherical", offset=5) +
                  brush_lines("(X)1(A)29", theta=400, chi=0.3) + m2("pol", 2),
                  field=(-0.02, 0.02), seed=32, modes=["it0", "conv"]))
    lines = lat1d(50) + [
        "mon : S : freedom : frozen", "mon : S : frozen_range : lowerbound",
        "mon : A : freedom : free", "mon : B : freedom : free", "mon : W : freedom : free",
        "mon : A : chi_S : -1.2", "mon : B : chi_W : 0.6",
        "mol : pol : composition : (A)10(B)20", "mol : pol : freedom : free", "mol : pol : phibulk : 0.005",
        "mol : water : composition : (W)1", "mol : water : freedom : solvent"] + m2("pol", 0.5)
    C.append(dict(name="markov2_ads1d", lines=lines, field=(-0.01, 0.01), seed=33, modes=["it0", "conv"]))
    # internal states and reactions: a weak polyacid brush (AH + H2O = AM +
    # H3O) in water with its autoprotolysis (2 H2O = OH + H3O) and a 1:1
    # salt; the neutral acid state and H2O get their own χ, so the states
    # split into several iteration blocks.  pH 7: the reactions' analytic
    # guesses are the bulk fractions (the reference's Newton takes no step);
    # pH 5: its Newton iterates.  A 2-D planar and a 1-D spherical variant.
    def weak_lines(comp, n, h3o, chi_ah=0.8):
        return ["lat : flat : bondlength : 3e-10",
                "mon : S : freedom : frozen", "mon : S : frozen_range : lowerbound",
                "mon : X : freedom : pinned", "mon : X : pinned_range : firstlayer",
                "mon : A : freedom : free", "mon : W : freedom : free",
                "mon : Na : freedom : free", "mon : Na : valence : 1",
                "mon : Cl : freedom : free", "mon : Cl : valence : -1",
                "mon : A : chi_S : -1", "mon : X : chi_W : 0.5",
                "state : AH : mon : A", "state : AH : valence : 0",
                "state : AM : mon : A", "state : AM : valence : -1",
                "state : H3O : mon : W", "state : H3O : valence : 1",
                "state : H2O : mon : W", "state : H2O : valence : 0",
                "state : OH : mon : W", "state : OH : valence : -1",
                f"state : H3O : alphabulk : {h3o}",
                f"state : AH : chi_H2O : {chi_ah}",
                "reaction : weak : equation : 1(AH) + 1(H2O) = 1(AM) + 1(H3O)", "reaction : weak : pK : 6",
                "reaction : auto : equation : 2(H2O) = 1(OH) + 1(H3O)", "reaction : auto : pK : 14",
                f"mol : pol : composition : {comp}", "mol : pol : freedom : restricted", f"mol : pol : n : {n}",
                "mol : water : composition : (W)1", "mol : water : freedom : solvent",
                "mol : Na : composition : (Na)1", "mol : Na : freedom : neutralizer",
                "mol : Cl : composition : (Cl)1", "mol : Cl : freedom : free", "mol : Cl : phibulk : 0.01"]
    C.append(dict(name="states_weak1d", lines=lat1d(40) + weak_lines("(X)1(A)29", 0.05, "1e-7"),
                  field=(-0.01, 0.01), seed=41, modes=["it0", "it5", "conv"], conv_itlim=5000))
    C.append(dict(name="states_weak1d_ph5", lines=lat1d(40) + weak_lines("(X)1(A)29", 0.05, "1e-5", chi_ah=0.3),
                  field=(-0.01, 0.01), seed=42, modes=["it0", "it5", "conv"], conv_itlim=5000))
    C.append(dict(name="states_weak2d", lines=lat2d(14, 8, ["surface", "mirror", "mirror", "mirror"]) +
                  weak_lines("(X)1(A)19", 0.4, "1e-7"), field=(-0.01, 0.01), seed=43,
                  modes=["it0", "it5", "conv"], conv_itlim=5000, split_tol=1e-4))
    wall3 = [ln.replace("frozen_range : lowerbound", "frozen_range : 1,1,1;1,6,6")
             .replace("pinned_range : firstlayer", "pinned_range : 2,1,1;2,6,6")
             for ln in weak_lines("(X)1(A)15", 1.5, "1e-7")]
    C.append(dict(name="states_weak3d", lines=lat3d((9, 6, 6), bc="mirror") + wall3, field=(-0.01, 0.01),
                  seed=45, modes=["it0", "it5", "conv"], conv_itlim=5000, split_tol=1e-4))
    C.append(dict(name="states_weak1d_sph", lines=lat1d(30, geom="spherical", offset=8) +
                  weak_lines("(X)1(A)19", 10.0, "1e-6"), field=(-0.01, 0.01), seed=44,
                  modes=["it0", "it5", "conv"], conv_itlim=5000))
    # a sample of the batched workload: random 1-gradient brushes (seeded), 10% stars
    rng = np.random.default_rng(2024)
    for i in range(6):
        nl = int(rng.integers(50, 401))
        N = int(rng.integers(20, 501))
        sig = float(rng.uniform(0.01, 0.1))
        chi = float(rng.uniform(0, 1))
        star = (i == 5)
        if star:
            a = max(N // 3, 2)
            comp = f"(X)1(A){a - 1}[(A){a}](A){a}"
        else:
            comp = f"(X)1(A){N - 1}"
        nl = min(nl, 200)  # keep the reference run short
        C.append(dict(name=f"brushmix_{i}", lines=lat1d(nl) + brush_lines(comp, n=round(sig, 6), chi=round(chi, 6)),
                      field=(-0.01, 0.01), seed=100 + i, modes=["conv"]))
    return C


def outputs_block(plan: Plan) -> list[str]:
    s = ["output : pro : append : false"]
    for name in plan.seg_names:
        s.append(f"pro : mon : {name} : phi")
    for name in plan.seg_names:
        s.append(f"pro : mon : {name} : G1")
    # the states' profiles (Segment::GetPointer's phi-, alpha- and u-<state>,
    # segment.cpp:1896-1910).  phi- of a mon's first state is left out: the
    # reference writes zeros there (its profile index 2 is the 3-D phi[z]
    # average, reached for 1 and 2 gradients too).
    first = {}
    for j, st in enumerate(plan.state_names):
        seg = plan.seg_names[plan.c.state_seg[j]]
        if seg in first:
            s.append(f"pro : mon : {seg} : phi-{st}")
        first.setdefault(seg, st)
    for j, st in enumerate(plan.state_names):
        seg = plan.seg_names[plan.c.state_seg[j]]
        s += [f"pro : mon : {seg} : alpha-{st}", f"pro : mon : {seg} : u-{st}"]
    s.append("pro : sys : noname : alpha")
    if plan.c.charged:
        s += ["pro : sys : noname : psi", "pro : sys : noname : q", "pro : sys : noname : eps"]
    s.append("output : kal : append : false")
    s += ["kal : sys : noname : free_energy", "kal : sys : noname : grand_potential",
          "kal : newton : isaac : residual", "kal : newton : isaac : iterations"]
    for j, st in enumerate(plan.state_names):
        seg = plan.seg_names[plan.c.state_seg[j]]
        s += [f"kal : mon : {seg} : {q}_{st}" for q in ("alphabulk", "valence", "phibulk", "theta", "theta_exc")]
    for m in range(plan.n_mol):
        mn = MOLNAMES[m]
        s += [f"kal : mol : {mn} : GN", f"kal : mol : {mn} : n", f"kal : mol : {mn} : theta",
              f"kal : mol : {mn} : phibulk", f"kal : mol : {mn} : Mu"]
    return s


MOLNAMES: list[str] = []


def make_field(plan: Plan, lo: float, hi: float, seed: int, antisym: bool) -> np.ndarray:
    rng = np.random.default_rng(seed)
    x = rng.uniform(lo, hi, size=plan.iv)
    if antisym and plan.c.n_it == 2:
        M = plan.M
        x[M:2 * M] = -x[:M]
    return x


def write_guess(path: Path, plan: Plan, x: np.ndarray) -> None:
    c = plan.c
    names = plan.it_names
    n_mon = sum(1 for i in range(c.n_it) if c.n_state == 0 or c.it_sp[i] < c.n_seg)
    my = c.MY if c.gradients > 1 else 0
    mz = c.MZ if c.gradients > 2 else 0
    with open(path, "w") as f:
        f.write("DIIS\n")
        f.write(f" {c.MX}\t{my}\t{mz}\t1\n")
        f.write("true\n" if c.charged else "false\n")
        # ItMonList names, then ItStateList names (Solve_scf::Guess,
        # solve_scf.cpp:500-517)
        f.write(f"{n_mon}\n")
        for n in names[:n_mon]:
            f.write(n + "\n")
        f.write(f"{len(names) - n_mon}\n")
        for n in names[n_mon:]:
            f.write(n + "\n")
        for v in x:
            f.write(f"{v:.17e}\n")


def parse_pro(path: Path, ndim: int) -> dict:
    lines = path.read_text().strip().splitlines()
    head = [t for t in lines[0].split("\t") if t.strip()]
    data = np.array([[float(t) for t in ln.split("\t") if t.strip()] for ln in lines[1:]])
    return {"header": head, "data": data}


def parse_kal(path: Path) -> dict:
    lines = path.read_text().strip().splitlines()
    head = lines[0].split("\t")
    vals = [float(t) for t in lines[-1].split("\t")]
    return dict(zip(head, vals))


def run_case(case: dict, mode: str, workdir: Path) -> dict:
    global MOLNAMES
    body = list(case["lines"])
    nw = dict(case.get("newton", {}))
    base_text = "\n".join(body + newton(**nw)) + "\n"
    plan = Plan(base_text)
    MOLNAMES = [ln.split(":")[1].strip() for ln in body if ln.startswith("mol")]
    MOLNAMES = list(dict.fromkeys(MOLNAMES))
    x = make_field(plan, *case["field"], case["seed"], case.get("antisym", False))
    itlim = {"it0": 0, "it5": 5, "conv": case.get("conv_itlim", 1000)}[mode]
    nw["itlim"] = itlim
    text = "\n".join(body + newton(**nw)) + "\n"
    tag = f"{case['name']}_{mode}"
    guess = workdir / f"{tag}.guess"
    write_guess(guess, plan, x)
    full = text + "sys : noname : initial_guess : file\n" + f"sys : noname : guess_inputfile : {guess.name}\n"
    full += "\n".join(outputs_block(plan)) + "\nstart\n"
    (workdir / f"{tag}.in").write_text(full)
    r = subprocess.run([str(REF_BIN), f"{tag}.in"], cwd=workdir, capture_output=True, text=True, timeout=600)
    out = {"returncode": r.returncode, "stdout_tail": r.stdout[-2000:]}
    pro = workdir / "output" / f"{tag}.pro"
    kal = workdir / "output" / f"{tag}.kal"
    if r.returncode != 0 or not kal.exists():
        raise RuntimeError(f"reference failed on {tag}: {r.stdout[-1500:]} {r.stderr[-500:]}")
    prod = parse_pro(pro, plan.c.gradients)
    kald = parse_kal(kal)
    out = dict(input=text, x=x.tolist(), mode=mode, iterationlimit=itlim,
               pro_header=prod["header"], pro=prod["data"].tolist(), kal=kald,
               molnames=MOLNAMES)
    if case.get("raw"):
        # the reference's files verbatim, and the output items that made them
        out["pro_text"] = pro.read_text()
        out["kal_text"] = kal.read_text()
        ob = outputs_block(plan)
        out["pro_items"] = [ln for ln in ob if ln.startswith("pro :")]
        out["kal_items"] = [ln for ln in ob if ln.startswith("kal :")]
    return out


RAW_CASES = ["brush1d_x100", "brush2d_cyl", "melt3d", "charged1d", "states_weak1d", "states_weak2d"]


def main_raw():
    """tests/golden/raw_outputs.json: the reference's .pro and .kal files,
    verbatim, for the single-residual run of a 1-D, a 2-D cylindrical, a 3-D
    and a charged case (the file-format pin of nm_write_pro/nm_write_kal)."""
    out = {}
    with tempfile.TemporaryDirectory() as td:
        wd = Path(td)
        (wd / "output").mkdir()
        for case in cases():
            if case["name"] in RAW_CASES:
                case = dict(case, raw=True)
                out[case["name"]] = run_case(case, "it0", wd)
                print(case["name"], len(out[case["name"]]["pro_text"]), flush=True)
    (GOLDEN / "raw_outputs.json").write_text(json.dumps(out))


KEY_BASE = """lat : flat : n_layers : 20
lat : flat : lattice_type : simple_cubic
lat : flat : lowerbound : surface
mon : S : freedom : frozen
mon : S : frozen_range : lowerbound
mon : X : freedom : pinned
mon : X : pinned_range : firstlayer
mon : A : freedom : free
mon : W : freedom : free
mon : A : chi_W : 0.5
mon : X : chi_W : 0.5
mol : pol : composition : (X)1(A)19
mol : pol : freedom : restricted
mol : pol : n : 0.05
mol : water : composition : (W)1
mol : water : freedom : solvent
newton : isaac : method : DIIS
newton : isaac : iterationlimit : 0
"""

# one extra input line per case: keys the reference does not know, keys it
# knows that cannot change a DIIS solve, and keys it knows that do
KEY_LINES = [
    "mon : A : chi_Y : 1", "mon : A : bogus : 1", "lat : flat : bogus : 1", "mol : pol : bogus : 1",
    "newton : isaac : bogus : 1", "mol : pol : save_memory : true", "newton : isaac : s_info : true",
    "newton : isaac : e_info : false", "newton : isaac : deltamin : 0.01", "sys : noname : GPU : false",
    "sys : noname : calculation_type : equilibrium", "lat : flat : lambda : 0.2",
    "mol : pol : restricted_range : 1;3", "sys : noname : overflow_protection : true",
]


def main_keys():
    """tests/golden/key_checks.json: whether the reference accepts the base
    brush input with each line of KEY_LINES added (Input::CheckParameters
    refuses a key outside the class's list and the run stops)."""
    out = {"base": KEY_BASE, "cases": []}
    with tempfile.TemporaryDirectory() as td:
        wd = Path(td)
        (wd / "output").mkdir()
        for i, line in enumerate(KEY_LINES):
            text = KEY_BASE + line + "\noutput : kal : append : false\nkal : mol : pol : theta\nstart\n"
            (wd / f"k{i}.in").write_text(text)
            r = subprocess.run([str(REF_BIN), f"k{i}.in"], cwd=wd, capture_output=True, text=True, timeout=120)
            refused = "is unknown" in r.stdout or not (wd / "output" / f"k{i}.kal").exists()
            out["cases"].append({"line": line, "reference": "refused" if refused else "accepted"})
            print(f"{line:50s} {out['cases'][-1]['reference']}", flush=True)
    (GOLDEN / "key_checks.json").write_text(json.dumps(out, indent=1))


# searches: (fixture name, base fixture whose lines and seeded field are
# used, extra input lines)
SEARCHES = [
    ("search_theta_omega", "brush1d_x100",
     ["var : mol-pol : search : theta", "var : sys-noname : grand_potential : -0.4"]),
    ("search_theta_F", "brush1d_x100", ["var : mol-pol : search : theta", "var : sys-noname : free_energy : -2.4"]),
]


def main_search():
    """tests/golden/search_*.json: the reference's `var` searches (θ of the
    brush for a target grand potential or free energy), run from the base
    fixture's seeded field, with the .kal values at the search's end."""
    with tempfile.TemporaryDirectory() as td:
        wd = Path(td)
        (wd / "output").mkdir()
        for name, base_name, extra in SEARCHES:
            case = next(c for c in cases() if c["name"] == base_name)
            body = list(case["lines"]) + extra
            text = "\n".join(body + newton()) + "\n"
            plan = Plan(text)
            x = make_field(plan, *case["field"], case["seed"], False)
            write_guess(wd / f"{name}.guess", plan, x)
            full = text + "sys : noname : initial_guess : file\n" + f"sys : noname : guess_inputfile : {name}.guess\n"
            full += "output : kal : append : false\n" + "\n".join(
                f"kal : {k}" for k in ("mol : pol : theta", "mol : pol : n", "mol : pol : phibulk",
                                       "sys : noname : grand_potential", "sys : noname : free_energy")) + "\nstart\n"
            (wd / f"{name}.in").write_text(full)
            r = subprocess.run([str(REF_BIN), f"{name}.in"], cwd=wd, capture_output=True, text=True, timeout=600)
            kal = wd / "output" / f"{name}.kal"
            if r.returncode != 0 or not kal.exists():
                raise RuntimeError(f"reference failed on {name}: {r.stdout[-1500:]}")
            out = dict(input=text, x=x.tolist(), kal=parse_kal(kal),
                       super_iterations=[ln for ln in r.stdout.splitlines() if ln.startswith("s_it")])
            (GOLDEN / f"{name}.json").write_text(json.dumps(out))
            print(name, out["kal"], flush=True)


# scans: (fixture name, extra input lines) on the same brush
SCANS = [
    ("scan_theta_linear", ["var : mol-pol : scan : theta", "var : mol-pol : step : 0.5", "var : mol-pol : end_value : 7"]),
    ("scan_theta_truncated", ["var : mol-pol : scan : theta", "var : mol-pol : step : 0.1",
                              "var : mol-pol : end_value : 5.3"]),
    ("scan_theta_exponential", ["var : mol-pol : scan : theta", "var : mol-pol : scale : exponential",
                                "var : mol-pol : steps : 2", "var : mol-pol : end_value : 50"]),
]


def main_scan():
    """tests/golden/scan_*.json: the reference's `var` scans of θ of the
    brush (linear, linear with a step count the division truncates, and
    exponential), run from the brush fixture's seeded field, with one .kal
    row per step."""
    case = next(c for c in cases() if c["name"] == "brush1d_x100")
    with tempfile.TemporaryDirectory() as td:
        wd = Path(td)
        (wd / "output").mkdir()
        for name, extra in SCANS:
            body = list(case["lines"]) + extra
            text = "\n".join(body + newton()) + "\n"
            plan = Plan(text)
            x = make_field(plan, *case["field"], case["seed"], False)
            write_guess(wd / f"{name}.guess", plan, x)
            full = text + "sys : noname : initial_guess : file\n" + f"sys : noname : guess_inputfile : {name}.guess\n"
            full += "output : kal : append : true\n" + "\n".join(
                f"kal : {k}" for k in ("mol : pol : theta", "sys : noname : grand_potential",
                                       "sys : noname : free_energy")) + "\nstart\n"
            (wd / f"{name}.in").write_text(full)
            r = subprocess.run([str(REF_BIN), f"{name}.in"], cwd=wd, capture_output=True, text=True, timeout=600)
            kal = wd / "output" / f"{name}.kal"
            if r.returncode != 0 or not kal.exists():
                raise RuntimeError(f"reference failed on {name}: {r.stdout[-1500:]}")
            lines = kal.read_text().strip().splitlines()
            head = lines[0].split("\t")
            rows = [dict(zip(head, (float(t) for t in ln.split("\t")))) for ln in lines[1:]]
            (GOLDEN / f"{name}.json").write_text(json.dumps(dict(input=text, x=x.tolist(), rows=rows)))
            print(name, [round(rw["mol_pol_theta"], 6) for rw in rows], flush=True)
        # a pH scan of the weak-polyacid brush: the fixed H3O+ fraction from
        # 1e-7 to 1e-5, one step per decade; each step's bulk equilibrium
        # reads the previous solve's bulk fractions (Reaction::pKeff)
        # and a scan of the acid's pK from 6 to 8
        case = next(c for c in cases() if c["name"] == "states_weak1d")
        for name, extra in (("scan_states_h3o", ["var : state-H3O : scan : alphabulk",
                                                 "var : state-H3O : scale : exponential",
                                                 "var : state-H3O : end_value : 1e-5", "var : state-H3O : steps : 1"]),
                            ("scan_states_pk", ["var : reaction-weak : scan : pK", "var : reaction-weak : step : 1",
                                                "var : reaction-weak : end_value : 8"])):
            state_scan(wd, case, name, extra)


def state_scan(wd: Path, case: dict, name: str, extra: list[str]) -> None:
    """A scan of the weak-polyacid brush (states_weak1d) by the reference,
    one .kal row per step: the states' bulk fractions, θ, F, Ω (the
    reference's output has no reaction items)."""
    text = "\n".join(list(case["lines"]) + extra + newton()) + "\n"
    plan = Plan(text)
    x = make_field(plan, *case["field"], case["seed"], False)
    write_guess(wd / f"{name}.guess", plan, x)
    full = text + "sys : noname : initial_guess : file\n" + f"sys : noname : guess_inputfile : {name}.guess\n"
    items = [f"mon : {plan.seg_names[plan.c.state_seg[j]]} : alphabulk_{st}" for j, st in enumerate(plan.state_names)]
    items += ["mol : pol : theta", "sys : noname : free_energy", "sys : noname : grand_potential",
              "newton : isaac : iterations"]
    full += "output : kal : append : true\n" + "\n".join(f"kal : {k}" for k in items) + "\nstart\n"
    (wd / f"{name}.in").write_text(full)
    r = subprocess.run([str(REF_BIN), f"{name}.in"], cwd=wd, capture_output=True, text=True, timeout=600)
    kal = wd / "output" / f"{name}.kal"
    if r.returncode != 0 or not kal.exists():
        raise RuntimeError(f"reference failed on {name}: {r.stdout[-1500:]}")
    lines = kal.read_text().strip().splitlines()
    head = lines[0].split("\t")
    rows = [dict(zip(head, (float(t) for t in ln.split("\t")))) for ln in lines[1:]]
    (GOLDEN / f"{name}.json").write_text(json.dumps(dict(input=text, x=x.tolist(), items=items, rows=rows)))
    print(name, [round(rw["mon_A_alphabulk_AM"], 6) for rw in rows], flush=True)


def main():
    if not REF_BIN.exists():
        sys.exit(f"{REF_BIN} missing: build it with  make -f oracle/Makefile.ref")
    if sys.argv[1:2] == ["--raw"]:
        main_raw()
        return
    if sys.argv[1:2] == ["--keys"]:
        main_keys()
        return
    if sys.argv[1:2] == ["--search"]:
        main_search()
        return
    if sys.argv[1:2] == ["--scan"]:
        main_scan()
        return
    only = set(sys.argv[1:])
    with tempfile.TemporaryDirectory() as td:
        wd = Path(td)
        (wd / "output").mkdir()
        for case in cases():
            if only and case["name"] not in only:
                continue
            res = {"name": case["name"], "runs": {}, "split_tol": case.get("split_tol", 1e-5),
                   "path_tol": case.get("path_tol", 1e-8)}
            for mode in case["modes"]:
                res["runs"][mode] = run_case(case, mode, wd)
                k = res["runs"][mode]["kal"]
                print(f"{case['name']:>16s} {mode:5s} F={k.get('sys_noname_free_energy')!r:<24} "
                      f"res={k.get('newton_isaac_residual')!r:<12} it={k.get('newton_isaac_iterations')}", flush=True)
            (GOLDEN / f"{case['name']}.json").write_text(json.dumps(res))


if __name__ == "__main__":
    main()
