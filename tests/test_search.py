"""Searches and scans (`var` keys) of a molecule quantity.

tests/golden/search_*.json (make_golden.py --search) hold the reference's
searches of θ of the 1-D (X)1(A)99 brush for a target grand potential and a
target free energy, run from the brush fixture's seeded field, with the .kal
values at the end (Solve_scf::SuperIterate, SFNewton::iterate_RF).

- CPU: the plan compiler reads the `var` keys and the `super_*` controls
  with the reference's defaults, and refuses searches it cannot run.  The
  oracle's restatement of the search (orc_search) takes the reference's path
  (θ, F and Ω to 1e-9), and stepping the oracle through the plan's scan
  values gives the reference's rows.
- GPU: nm_ctx_search ends with the target's error below super_tolerance,
  at the reference's θ (both searches stop inside the same tolerance, so the
  θ agree to the tolerance over the slope of the target, about 1e-5
  relative here), and with the grand potential and free energy of the
  reference's end point.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from namics_gb300 import NM_FP64, NamicsError, Plan, _abi

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem for p in GOLDEN.glob("search_*.json"))


def _load(name):
    return json.loads((GOLDEN / f"{name}.json").read_text())


def test_search_keys_are_read():
    g = _load("search_theta_omega")
    plan = Plan(g["input"])  # keep alive while reading it
    p = plan.c
    mols = [p.mol_name[m].decode() for m in range(p.n_mol)]
    assert (p.search_mol, p.search_what) == (mols.index("pol"), 0)
    assert (p.target_kind, p.target_value) == (1, -0.4)
    assert p.super_tolerance == pytest.approx(10 * p.tolerance)
    assert p.super_iterationlimit == p.iterationlimit // 10
    assert p.super_deltamax == 0.5
    qplan = Plan(g["input"] + "newton : isaac : super_tolerance : 1e-5\nnewton : isaac : super_deltamax : 0.2\n")
    assert (qplan.c.super_tolerance, qplan.c.super_deltamax) == (1e-5, 0.2)
    fplan = Plan(_load("search_theta_F")["input"])
    assert fplan.c.target_kind == 0
    base = g["input"].replace("var : mol-pol : search : theta\n", "").replace(
        "var : sys-noname : grand_potential : -0.4\n", "")
    bplan = Plan(base)
    assert bplan.c.search_mol == -1


@pytest.mark.parametrize("extra", [
    "var : mol-pol : search : theta\n",                                    # no target
    "var : sys-noname : grand_potential : -0.4\n",                         # no search
    "var : mol-pol : search : theta\nvar : sys-noname : free_energy : -2\nvar : sys-noname : grand_potential : 0\n",
    "var : mol-water : search : theta\nvar : sys-noname : free_energy : -2\n",   # the solvent
    "var : mol-pol : search : phibulk\nvar : sys-noname : free_energy : -2\n",   # restricted: theta or n
    "var : mol-pol : scan : theta\n",                                      # scans are nm_ctx_set_values
    "var : pol : search : theta\nvar : sys-noname : free_energy : -2\n",   # not item-name
])
def test_unrunnable_searches_are_refused(extra):
    g = _load("search_theta_omega")
    base = g["input"].replace("var : mol-pol : search : theta\n", "").replace(
        "var : sys-noname : grand_potential : -0.4\n", "")
    with pytest.raises(NamicsError) as ei:
        Plan(base + extra)
    assert ei.value.code == _abi.NM_ERR_INPUT


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_search_matches_reference(name):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from namics_gb300 import Context
    g = _load(name)
    plan = Plan(g["input"])
    ctx = Context(plan, NM_FP64)
    x = torch.from_numpy(np.array(g["x"])).cuda()
    r = ctx.search(x.data_ptr())
    tol = plan.c.super_tolerance
    assert r.status == 0 and abs(r.error) <= tol, r
    k = g["kal"]
    assert abs(r.value - k["mol_pol_theta"]) <= 1e-4 * k["mol_pol_theta"], (r.value, k["mol_pol_theta"])
    F, O, _ = ctx.free_energy()
    if plan.c.target_kind == 1:
        assert abs(O - plan.c.target_value) <= tol
    else:
        assert abs(F - plan.c.target_value) <= tol
    assert abs(O - k["sys_noname_grand_potential"]) <= 1e-5 and abs(F - k["sys_noname_free_energy"]) <= 1e-5
    assert ctx.molecule(plan.c.search_mol)["theta"] == pytest.approx(r.value, rel=1e-12)


SCANS = sorted(p.stem for p in GOLDEN.glob("scan_*.json"))


@pytest.mark.parametrize("name", SCANS)
def test_scan_values_are_the_reference_steps(name):
    """tests/golden/scan_*.json (make_golden.py --scan): the reference's scans
    of θ and of a fixed state's alphabulk, one .kal row per step.  The plan's
    step values are the reference's (the step count truncated like its
    integer division)."""
    g = _load(name)
    plan = Plan(g["input"])
    vals = plan.scan_values()
    c = plan.c
    if c.scan_reaction >= 0:
        # the reference writes no reaction items: its pK steps start + k·step
        assert len(vals) == len(g["rows"]) and vals[0] == c.scan_start
        ref = [c.scan_start + k * c.scan_step for k in range(len(vals))]
    elif c.scan_state >= 0:
        col = f"mon_{plan.seg_names[c.state_seg[c.scan_state]]}_alphabulk_{plan.state_names[c.scan_state]}"
        ref = [r[col] for r in g["rows"]]
    else:
        ref = [r["mol_pol_theta"] for r in g["rows"]]
    assert len(vals) == len(ref)
    assert np.allclose(vals, ref, rtol=1e-12, atol=0)


@pytest.mark.parametrize("extra", [
    "var : mol-pol : scan : theta\nvar : mol-pol : step : 0.5\n",                               # no end_value
    "var : mol-pol : scan : theta\nvar : mol-pol : end_value : 7\n",                            # no step
    "var : mol-pol : scan : theta\nvar : mol-pol : step : -0.5\nvar : mol-pol : end_value : 7\n",  # wrong way
    "var : mol-pol : scan : phibulk\nvar : mol-pol : step : 0.5\nvar : mol-pol : end_value : 7\n",
    "var : mol-pol : scan : theta\nvar : mol-pol : scale : log\nvar : mol-pol : end_value : 7\n",
    "var : mol-pol : scan : theta\nvar : mol-pol : scale : exponential\nvar : mol-pol : end_value : 0\n",
    "var : mol-pol : scan : theta\nvar : mol-pol : step : 1e-9\nvar : mol-pol : end_value : 7\n",  # 2e9 steps
])
def test_unrunnable_scans_are_refused(extra):
    g = _load("scan_theta_linear")
    base = "\n".join(ln for ln in g["input"].splitlines() if not ln.startswith("var")) + "\n"
    with pytest.raises(NamicsError) as ei:
        Plan(base + extra)
    assert ei.value.code == _abi.NM_ERR_INPUT


def test_scan_ratio_truncating_to_zero_steps_is_accepted():
    """(end - start)/step = (4.8 - 5)/0.5 = -0.4: the reference assigns the
    ratio to an int first (molecule.cpp:807-812), so the scan has zero steps
    and runs once at the start value (the reference's own run of this input
    writes one .kal row at θ = 5)."""
    g = _load("scan_theta_linear")
    plan = Plan(g["input"].replace("end_value : 7", "end_value : 4.8"))
    assert plan.scan_values() == pytest.approx([5.0], rel=1e-12)


def _scan_item(plan, text):
    """The nm_ctx_set_values item a scan step sets."""
    c = plan.c
    if c.scan_state >= 0:
        return f"state : {plan.state_names[c.scan_state]} : alphabulk"
    if c.scan_reaction >= 0:
        vn = next(ln.split(":")[1].strip() for ln in text.splitlines() if ln.startswith("var : reaction-"))
        return f"reaction : {vn.split('-', 1)[1]} : pK"
    return "mol : pol : theta"


@pytest.mark.gpu
@pytest.mark.parametrize("name", SCANS)
def test_scan_matches_reference(name):
    """Each step: the step's value set on the live context, a solve warm-started
    from the previous step's field; F and Ω of every step match the
    reference's rows (both solved to ‖g‖ < 1e-7)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from namics_gb300 import Context
    g = _load(name)
    plan = Plan(g["input"])
    ctx = Context(plan, NM_FP64)
    x = torch.from_numpy(np.array(g["x"])).cuda()
    item = _scan_item(plan, g["input"])
    for v, row in zip(plan.scan_values(), g["rows"]):
        ctx.set_values({item: v})
        r = ctx.solve_dev(x.data_ptr())
        assert r.status == 0, (v, r)
        F, O, _ = ctx.free_energy()
        for got, want in ((F, row["sys_noname_free_energy"]), (O, row["sys_noname_grand_potential"])):
            assert abs(got - want) <= 1e-6 * max(1.0, abs(want)), (v, got, want)


def test_batch_refuses_searches_and_scans_before_the_device():
    """A plan with a search or a scan needs several solves on one context;
    the batched solver refuses it (and any plan it cannot take) with
    NM_ERR_INPUT before it touches the device, so this holds on a CPU host."""
    from namics_gb300 import Batch
    for name in ("search_theta_omega", "scan_theta_linear"):
        plan = Plan(_load(name)["input"])
        with pytest.raises(NamicsError) as ei:
            Batch([plan])
        assert ei.value.code == _abi.NM_ERR_INPUT
        assert "search or scan" in str(ei.value)
    text2d = (GOLDEN / "ads2d.json").read_text()
    plan2d = Plan(json.loads(text2d)["runs"]["conv"]["input"])
    with pytest.raises(NamicsError) as ei:
        Batch([plan2d])
    assert ei.value.code == _abi.NM_ERR_INPUT


def _oracle(plan):
    import sys
    sys.path.insert(0, str(GOLDEN.parents[1] / "oracle"))
    from orc import Oracle
    return Oracle(plan)


@pytest.mark.parametrize("name", CASES)
def test_oracle_search_follows_the_reference(name):
    """The oracle's restatement of the search (orc_search) takes the
    reference's path: the same θ, F and Ω at its end to 1e-9."""
    g = _load(name)
    plan = Plan(g["input"])
    orc = _oracle(plan)
    rc, _, value, error, _, _ = orc.search(np.array(g["x"]))
    assert rc == 0 and abs(error) <= plan.c.super_tolerance
    k = g["kal"]
    assert abs(value - k["mol_pol_theta"]) <= 1e-9 * k["mol_pol_theta"]
    F, O, _ = orc.free_energy()
    assert abs(F - k["sys_noname_free_energy"]) <= 1e-9 * abs(k["sys_noname_free_energy"])
    assert abs(O - k["sys_noname_grand_potential"]) <= 1e-9 * abs(k["sys_noname_grand_potential"])


@pytest.mark.parametrize("name", SCANS)
def test_oracle_scan_follows_the_reference(name):
    """The oracle stepping through the plan's scan values, each solve warm
    from the last, gives the reference's F and Ω at every step to 1e-7
    (a long step, as 15.8 -> 50 on the exponential scale, can end at another
    point of the ‖g‖ < 1e-7 ball: 7e-9 relative in F there)."""
    g = _load(name)
    plan = Plan(g["input"])
    orc = _oracle(plan)
    x = np.array(g["x"])
    c = plan.c
    for v, row in zip(plan.scan_values(), g["rows"]):
        if c.scan_state >= 0 or c.scan_reaction >= 0:
            # a pH or pK scan: the states' bulk fractions of each step are the
            # reference's own (its bulk equilibrium reads the previous solve;
            # the device context's restatement of that is tested on the GPU)
            orc.set_states([row[f"mon_{plan.seg_names[c.state_seg[j]]}_alphabulk_{st}"]
                            for j, st in enumerate(plan.state_names)])
        else:
            orc.set_amount(c.scan_mol, c.scan_what, v)
        rc, x, _, res = orc.solve(x)
        assert rc == 0 and res < plan.c.tolerance
        F, O, _ = orc.free_energy()
        assert abs(F - row["sys_noname_free_energy"]) <= 1e-7 * max(1.0, abs(row["sys_noname_free_energy"])), v
        assert abs(O - row["sys_noname_grand_potential"]) <= 1e-7 * max(1.0, abs(row["sys_noname_grand_potential"])), v


def test_free_molecule_theta_target_is_refused():
    """φ_bulk of a free polymer searched for a target θ: the reference's run
    of this search ends in NaN for every value tried, so the plan refuses it."""
    g = json.loads((GOLDEN / "ads1d_cyl_hex.json").read_text())["runs"]["conv"]
    text = g["input"] + "var : mol-pol : search : phibulk\nvar : mol-pol : theta : 56\n"
    with pytest.raises(NamicsError) as ei:
        Plan(text)
    assert ei.value.code == _abi.NM_ERR_INPUT
