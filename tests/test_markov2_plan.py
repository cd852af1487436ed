"""Markov 2 (semiflexible) chains in the plan compiler (CPU).

`mol : … : Markov : 2` with `k_stiff` gives the molecule the bond-angle
weights of Molecule::AllocateMemory (molecule.cpp:135-152): on a simple-cubic
lattice P[k] ∝ exp(-k_stiff/2·(k·π/2)²) for k = 0, 1, normalised by
P[0] + 4·P[1], and P[2] = 0.  The reference prints them when it allocates a
Markov 2 molecule; for k_stiff = 1 it printed P[0] = 0.461925 and
P[1] = 0.134519 (six significant digits, its default cout precision).  What
the compiler does not cover is refused by name: other gradient counts, the
hexagonal lattice, branched or dendrimer chains, charged systems, a missing
k_stiff (the reference's default is the lattice's k_stiff, which it never
sets) and a k_stiff outside the reference's [0, 10].  The golden fixtures
markov2_* pin the oracle's sweeps to the reference's own runs
(test_oracle_golden) and the GPU tests the device path to the oracle."""
import math

import pytest

from namics_gb300 import NamicsError, Plan

BASE = """lat : flat : n_layers : 30
lat : flat : lattice_type : simple_cubic
lat : flat : geometry : planar
lat : flat : gradients : 1
lat : flat : lowerbound : surface
lat : flat : upperbound : mirror
mon : S : freedom : frozen
mon : S : frozen_range : lowerbound
mon : A : freedom : free
mon : W : freedom : free
mol : pol : composition : (A)20
mol : pol : freedom : free
mol : pol : phibulk : 0.01
mol : water : composition : (W)1
mol : water : freedom : solvent
"""


def test_bend_weights_are_the_references():
    p = Plan(BASE + "mol : pol : Markov : 2\nmol : pol : k_stiff : 1\n")
    mol = p.c.mols[0]
    assert mol.markov == 2 and p.c.mols[1].markov == 1
    assert abs(mol.bend[0] - 0.461925) < 5e-7 and abs(mol.bend[1] - 0.134519) < 5e-7 and mol.bend[2] == 0.0
    for ks in (0.0, 2.5, 10.0):
        m = Plan(BASE + f"mol : pol : Markov : 2\nmol : pol : k_stiff : {ks}\n").c.mols[0]
        p1 = math.exp(-0.5 * ks * (3.14159265 / 2) ** 2)
        assert m.bend[0] == pytest.approx(1 / (1 + 4 * p1), rel=1e-15)
        assert m.bend[1] == pytest.approx(p1 / (1 + 4 * p1), rel=1e-15)
        assert m.bend[0] + 4 * m.bend[1] == pytest.approx(1.0, rel=1e-15)


def test_markov1_default_and_k_stiff_alone():
    assert Plan(BASE).c.mols[0].markov == 1
    assert Plan(BASE + "mol : pol : Markov : 1\n").c.mols[0].markov == 1
    assert Plan(BASE + "mol : pol : k_stiff : 3\n").c.mols[0].markov == 1  # read, range-checked, unused


@pytest.mark.parametrize("text", [
    BASE + "mol : pol : Markov : 2\n",                                            # no k_stiff
    BASE + "mol : pol : Markov : 2\nmol : pol : k_stiff : 11\n",                  # out of range
    BASE + "mol : pol : k_stiff : -1\n",
    BASE + "mol : pol : Markov : 3\nmol : pol : k_stiff : 1\n",
    BASE.replace("simple_cubic", "hexagonal") + "mol : pol : Markov : 2\nmol : pol : k_stiff : 1\n",
    BASE.replace("(A)20", "(A)10[(A)5](A)5") + "mol : pol : Markov : 2\nmol : pol : k_stiff : 1\n",
    BASE.replace("(A)20", "@dend(A,(A)3,2)") + "mol : pol : Markov : 2\nmol : pol : k_stiff : 1\n",
    BASE + "mon : A : valence : -0.1\nmon : W : valence : 0.1\nmol : pol : Markov : 2\nmol : pol : k_stiff : 1\n",
    BASE.replace("lat : flat : n_layers : 30\n", "lat : flat : n_layers_x : 10\nlat : flat : n_layers_y : 10\n")
        .replace("gradients : 1", "gradients : 2").replace("lowerbound : surface", "lowerbound_x : surface")
        .replace("upperbound : mirror", "upperbound_x : mirror\nlat : flat : lowerbound_y : mirror\nlat : flat : upperbound_y : mirror")
    + "mol : pol : Markov : 2\nmol : pol : k_stiff : 1\n",
], ids=["no_k_stiff", "k_stiff_11", "k_stiff_negative", "markov3", "hexagonal", "branched", "dendrimer",
        "charged", "two_gradients"])
def test_refused(text):
    with pytest.raises(NamicsError):
        Plan(text)
