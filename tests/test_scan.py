"""Scans on a live context (nm_ctx_set_values, the reference's Variate).

A scan step changes χ or a molecule's amount and solves again from the
context's current field.  It must give exactly what a fresh context built
from the edited input text gives from the same start field (bit-identical
field, same iterations, same free energy), on a 1-D and a 2-D brush; a χ
change that would split an iteration species is refused and changes nothing.
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from namics_gb300 import NM_FP64, Context, NamicsError, Plan  # noqa: E402
from namics_gb300._abi import NM_ERR_INPUT  # noqa: E402


def _solve(ctx, x):
    x = x.copy()
    r, _ = ctx.solve_host(x, want_phi=False)
    F, O, _ = ctx.free_energy()
    return r, x, F


@pytest.mark.parametrize("name", ["brush1d_x100", "brush2d_cyl"])
def test_scan_step_equals_fresh_context(name):
    run = load_golden(name)["runs"]["conv"]
    text = run["input"]
    plan = Plan(text)
    ctx = Context(plan, NM_FP64)
    r0, x1, _ = _solve(ctx, np.array(run["x"]))
    assert r0.status == 0
    steps = [({"mon : A : chi_W": 0.6, "mon : X : chi_W": 0.6},
              lambda t: t.replace("mon : A : chi_W : 0.5", "mon : A : chi_W : 0.6")
                         .replace("mon : X : chi_W : 0.5", "mon : X : chi_W : 0.6"))]
    n_line = next(ln for ln in text.splitlines() if ln.startswith("mol : pol : n :"))
    n_new = 1.1 * float(n_line.split(":")[-1])
    steps.append(({"mol : pol : n": n_new}, lambda t: t.replace(n_line, f"mol : pol : n : {n_new!r}")))
    x_prev = x1
    edited = text
    for values, edit in steps:
        ctx.set_values(values)
        r_scan, x_scan, F_scan = _solve(ctx, x_prev)
        edited = edit(edited)
        assert edited != text
        fresh_plan = Plan(edited)
        fresh = Context(fresh_plan, NM_FP64)
        r_new, x_new, F_new = _solve(fresh, x_prev)
        assert r_scan.status == 0 and r_new.status == 0
        assert r_scan.iterations == r_new.iterations and r_scan.residual == r_new.residual
        assert np.array_equal(x_scan, x_new)
        assert F_scan == F_new
        x_prev = x_scan


def test_scan_refuses_splitting_an_iteration_species():
    run = load_golden("brush1d_x100")["runs"]["conv"]
    plan = Plan(run["input"])
    ctx = Context(plan, NM_FP64)
    r0, xa, Fa = _solve(ctx, np.array(run["x"]))
    with pytest.raises(NamicsError) as e:
        ctx.set_values({"mon : A : chi_W": 0.7})  # A and X share a species
    assert e.value.code == NM_ERR_INPUT
    r1, xb, Fb = _solve(ctx, np.array(run["x"]))
    assert r1.iterations == r0.iterations and np.array_equal(xa, xb) and Fa == Fb


@pytest.mark.parametrize("name,item", [("scan_states_h3o", "state : H3O : alphabulk"),
                                       ("scan_states_pk", "reaction : weak : pK")])
def test_state_scan_matches_reference(name, item, tmp_path):
    """A pH scan of the weak-polyacid brush (`var : state-H3O : scan :
    alphabulk`, 1e-7 to 1e-5, one step per decade) and a scan of the acid's
    pK (`var : reaction-weak : scan : pK`, 6 to 8), each step set with
    nm_ctx_set_values and solved from the previous step's field, against the
    reference's own rows.  Each step's bulk equilibrium reads the previous
    solve's bulk volume fractions (Reaction::pKeff), which moves pK_eff by
    about 0.3 here: the bulk fractions must follow that, not the input pK."""
    g = load_golden(name)
    plan = Plan(g["input"])
    assert plan.c.scan_state >= 0 or plan.c.scan_reaction >= 0
    values = plan.scan_values()
    assert len(values) == len(g["rows"]) == 3
    ctx = Context(plan, NM_FP64)
    x = np.array(g["x"])
    items = [it for it in g["items"] if not it.startswith("newton")]
    for k, (v, row) in enumerate(zip(values, g["rows"])):
        if k > 0:
            ctx.set_values({item: v})
        r, x, F = _solve(ctx, x)
        assert r.status == 0
        path = tmp_path / f"s{k}.kal"
        ctx.write_kal(path, items)
        head, vals = path.read_text().strip().splitlines()
        got = dict(zip(head.split("\t"), (float(t) for t in vals.split("\t"))))
        for h, want in row.items():
            if h.startswith("newton"):
                continue
            # the two solves' bulk volume fractions agree to their
            # convergence (‖g‖ < 1e-7), and pK_eff and the bulk fractions
            # (relative: the OH- fraction is ~5e-9) with them
            tol = 1e-6 * (abs(want) if "alphabulk" in h else max(1.0, abs(want)))
            assert abs(got[h] - want) <= tol, (k, h, got[h], want)
        assert abs(r.iterations - int(row["newton_isaac_iterations"])) <= 3, (k, r.iterations)
