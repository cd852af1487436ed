"""CPU-side checks of the C ABI and the host plan compiler (no GPU needed)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from namics_gb300 import NamicsError, Plan, _abi

ROOT = Path(__file__).resolve().parents[1]

BRUSH = """lat : flat : n_layers : 20
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
mol : pol : composition : {comp}
mol : pol : freedom : restricted
mol : pol : n : 0.05
mol : water : composition : (W)1
mol : water : freedom : solvent
"""


def test_library_exports_every_declared_symbol():
    header = (ROOT / "include" / "namics_gb300.h").read_text()
    declared = set(re.findall(r"^\s*(?:int|void|const char\*|long long)\s+\*?(nm_\w+)\s*\(", header, re.M))
    assert declared, "no entry points parsed from the header"
    assert declared == set(_abi.declared_symbols())
    lib = _abi.load()
    missing = [n for n in declared if getattr(lib, n, None) is None]
    assert not missing, missing


def test_version_string():
    assert b"namics_gb300" in _abi.load().nm_version()


def test_linear_chain_blocks():
    p = Plan(BRUSH.format(comp="(X)1(A)19"))
    mol = p.c.mols[0]
    assert mol.chainlength == 20 and mol.n_store == 20 and mol.n_blocks == 2
    b0, b1 = mol.blocks[0], mol.blocks[1]
    assert (b0.length, b1.length, b0.parent, b1.parent) == (1, 19, 1, -1)
    assert p.c.M == 22 and p.c.iv == 2 * 22  # X is a copy of A; W
    assert [p.seg_names[i] for i in p.it_seg] == ["X", "W"]


def test_branched_chain_blocks_and_iteration_order():
    p = Plan(BRUSH.format(comp="(X)1(A)9[(A)10](A)10"))
    mol = p.c.mols[0]
    assert mol.chainlength == 30 and mol.n_store == 30
    root = mol.blocks[mol.n_blocks - 1]
    assert root.parent == -1
    # the branch point block has two children
    assert max(mol.blocks[i].n_child for i in range(mol.n_blocks)) == 2
    # branched compositions are numbered back to front: A is the representative
    assert [p.seg_names[i] for i in p.it_seg] == ["A", "W"]


def test_dendrimer_degeneracy():
    text = BRUSH.format(comp="@dend(A,(A)3,3; A,(A)2,2)").replace("mol : pol : freedom : restricted\nmol : pol : n : 0.05",
                                                                    "mol : pol : freedom : restricted\nmol : pol : theta : 2")
    p = Plan(text)
    mol = p.c.mols[0]
    # core 1 + 3 arms*3 + 3 branch points + 6 arms * 2
    assert mol.chainlength == 1 + 9 + 3 + 12
    ds = sorted(mol.blocks[i].degeneracy for i in range(mol.n_blocks))
    assert ds == [1.0, 3.0, 3.0, 6.0]


@pytest.mark.parametrize("bad", [
    "lat : flat : FJC_choices : 5",
    "mol : pol : composition : (X)1(Q)19",
    "mon : A : chi_Y : 1",
])
def test_unsupported_input_fails_loudly(bad):
    text = BRUSH.format(comp="(X)1(A)19") + bad + "\n"
    if "composition" in bad:
        text = BRUSH.format(comp="(X)1(Q)19")
    with pytest.raises(NamicsError) as ei:
        Plan(text)
    assert ei.value.code == _abi.NM_ERR_INPUT


def test_surface_without_frozen_wall_is_rejected():
    text = BRUSH.format(comp="(X)1(A)19").replace("mon : S : frozen_range : lowerbound", "mon : S : frozen_range : 3;3")
    with pytest.raises(NamicsError) as ei:
        Plan(text)
    assert ei.value.code == _abi.NM_ERR_INPUT


def test_compute_entry_points_refuse_without_gpu_context():
    lib = _abi.load()
    r = _abi.nm_solve_result()
    assert lib.nm_solve_dev(None, None, C.byref(r)) == _abi.NM_ERR_ARG
    assert lib.nm_residual_dev(None, None, None) == _abi.NM_ERR_ARG
