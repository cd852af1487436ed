"""FP32 propagators on 2-gradient lattices (csrc/ctx2d32.cu), neutral and
charged, against the FP64 oracle.

- One FP32 residual at each fixture's seeded start field sits within the FP32
  floor (1e-7·N + 1e-6 per entry, so times √iv in the 2-norm); a second call
  replays the captured graph and gives the same g.
- A solve with FP32 propagators (FP64 finish) ends at a field whose FP64
  residual, evaluated by the oracle, is below the fixture's tolerance: the
  FP32 phase only shortens the way there.
- On the well-conditioned neutral fixtures, FP32 and the oracle both solved
  to 1e-9 agree to 1e-6 on φ and 1e-7 on F (the FP32 tolerances of the
  hot-path contract).
"""
import re

import numpy as np
import pytest

from conftest import golden_names, load_golden
from helpers import interior, newton_tolerance, rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from namics_gb300 import NM_FP32, Context, Plan  # noqa: E402
from orc import Oracle  # noqa: E402


def _linear_chains(plan) -> bool:
    """The FP32 2-D path takes linear chains (no joins)."""
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


def _floor(plan) -> float:
    n = max(plan.chainlength(m) for m in range(plan.n_mol))
    return (1e-7 * n + 1e-6) * np.sqrt(plan.iv)


@pytest.mark.parametrize("name", CASES)
def test_fp32_2d_residual_close_to_oracle(name):
    run = next(iter(load_golden(name)["runs"].values()))
    plan = Plan(run["input"])
    x = np.array(run["x"])
    rc, go = Oracle(plan).residual(x)
    assert rc == 0
    ctx = Context(plan, NM_FP32)
    xd = torch.from_numpy(x).cuda()
    gd = torch.zeros_like(xd)
    ctx.residual_dev(xd.data_ptr(), gd.data_ptr())
    torch.cuda.synchronize()
    g1 = gd.cpu().numpy().copy()
    ctx.residual_dev(xd.data_ptr(), gd.data_ptr())
    torch.cuda.synchronize()
    g = gd.cpu().numpy()
    assert np.array_equal(g, g1)
    assert np.linalg.norm(g - go) < _floor(plan), (np.linalg.norm(g - go), _floor(plan))


@pytest.mark.parametrize("name", CASES)
def test_fp32_2d_solve_ends_at_an_fp64_solution(name):
    runs = load_golden(name)["runs"]
    run = runs.get("conv") or runs.get("it5")
    plan = Plan(run["input"])
    tol = newton_tolerance(run)
    ctx = Context(plan, NM_FP32)
    x = np.array(run["x"])
    res, _ = ctx.solve_host(x)
    assert res.status == 0 and res.residual < tol, res
    rc, g = Oracle(plan).residual(x)
    assert rc == 0
    assert np.linalg.norm(g) < 1.01 * tol, np.linalg.norm(g)


def _tight(text: str) -> str:
    text = re.sub(r"newton : isaac : tolerance : \S+", "newton : isaac : tolerance : 1e-9", text)
    return re.sub(r"newton : isaac : iterationlimit : \S+", "newton : isaac : iterationlimit : 5000", text)


@pytest.mark.parametrize("name", [n for n in CASES if not n.startswith("charged")])
def test_fp32_2d_matches_oracle_tight(name):
    runs = load_golden(name)["runs"]
    run = runs.get("conv") or runs.get("it5")
    plan = Plan(_tight(run["input"]))
    x0 = np.array(run["x"])
    orc = Oracle(plan)
    rc, _, _, ro = orc.solve(x0.copy())
    assert rc == 0 and ro < 1e-9
    Fo, _, _ = orc.free_energy()
    phio = orc.field(0).reshape(plan.n_seg, -1)
    ctx = Context(plan, NM_FP32)
    res, phi = ctx.solve_host(x0.copy())
    assert res.status == 0 and res.residual < 1e-9, res
    F, _, _ = ctx.free_energy()
    assert abs(F - Fo) <= 1e-7 * max(1, abs(Fo)), (F, Fo)
    phi = phi.reshape(plan.n_seg, -1)
    for i in range(plan.n_seg):
        assert rel_err(interior(plan, phi[i]), interior(plan, phio[i])) < 1e-6, i
