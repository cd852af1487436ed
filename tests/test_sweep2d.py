"""Persistent 2-D sweeps (csrc/ctx2d.cu) against the per-step kernels.

Both run the same arithmetic in the same order, so on every 2-gradient
golden case (neutral and charged, planar and cylindrical) the residual, the
fields and a whole solve must be bit-identical with the sweep on and off
(nm_ctx_set_option NM_OPT_SWEEP2D), and the sweep must use fewer launches.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from namics_gb300 import NM_FP64, Context, Plan  # noqa: E402
from namics_gb300._abi import NM_OPT_SWEEP2D  # noqa: E402


def _linear_chains(plan) -> bool:
    """The persistent sweep takes linear chains (no joins)."""
    for m in range(plan.n_mol):
        mol = plan.c.mols[m]
        for b in range(mol.n_blocks):
            B = mol.blocks[b]
            if B.n_child > 1 or B.mult != 1:
                return False
    return True


def _two_d():
    out = []
    for n in golden_names():
        run = next(iter(load_golden(n)["runs"].values()))
        plan = Plan(run["input"])  # keep alive while reading it
        if plan.c.gradients == 2 and _linear_chains(plan):
            out.append(n)
    return out


CASES = _two_d()


def _residual(plan, x, sweep):
    ctx = Context(plan, NM_FP64)
    ctx.set_option(NM_OPT_SWEEP2D, sweep)
    xd = torch.from_numpy(x).cuda()
    gd = torch.zeros_like(xd)
    ctx.residual_dev(xd.data_ptr(), gd.data_ptr())
    torch.cuda.synchronize()
    fields = [ctx.field(w) for w in (0, 1, 2, 3)]
    if plan.c.charged:
        fields += [ctx.field(w) for w in (6, 7, 8)]
    return gd.cpu().numpy(), fields, ctx.free_energy()[:2], ctx.launch_count()


def test_two_d_cases_present():
    assert len(CASES) >= 4, CASES


@pytest.mark.parametrize("name", CASES)
def test_sweep_residual_bit_identical(name):
    run = next(iter(load_golden(name)["runs"].values()))
    plan = Plan(run["input"])
    x = np.array(run["x"])
    g0, f0, fe0, l0 = _residual(plan, x, 0)
    g1, f1, fe1, l1 = _residual(plan, x, 1)
    assert np.array_equal(g0, g1)
    for a, b in zip(f0, f1):
        assert np.array_equal(a, b)
    assert fe0 == fe1
    assert l1 < l0


@pytest.mark.parametrize("name", CASES)
def test_sweep_solve_bit_identical(name):
    runs = load_golden(name)["runs"]
    run = runs.get("it5") or runs.get("conv")
    plan = Plan(run["input"])
    res = []
    for sweep in (0, 1):
        ctx = Context(plan, NM_FP64)
        ctx.set_option(NM_OPT_SWEEP2D, sweep)
        x = np.array(run["x"])
        r, phi = ctx.solve_host(x)
        res.append((r, x, phi))
    (r0, x0, p0), (r1, x1, p1) = res
    assert r0.iterations == r1.iterations and r0.status == r1.status and r0.residual == r1.residual
    assert np.array_equal(x0, x1) and np.array_equal(p0, p1)
