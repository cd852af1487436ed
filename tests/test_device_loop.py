"""The device-resident solve loop (NM_OPT_DEVICE_LOOP): the whole DIIS
iteration as one CUDA graph with a conditional WHILE node.

It takes the host loop's control path statement for statement, and its
small DIIS solve is the same Jacobi pseudo-inverse run by one warp, so the
two loops take the same path up to rounding.  Held here: every converging reference fixture
converges to the input's tolerance and lands on the reference's profiles
and free energy within the fixture's convergence ball (the reference's
split-path tolerance), in at most twice the host loop's iterations; an FP32-propagator 3-D context converges to the FP64
fixed point (φ); the iteration limit ends the loop with the host loop's
status; a search runs its inner solves on the device loop."""
import json
from pathlib import Path

import numpy as np
import pytest

from conftest import golden_names, load_golden
from helpers import interior, newton_tolerance, pro_column, rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from namics_gb300 import NM_FP32, NM_FP64, Context, Plan, _abi  # noqa: E402

CONV = [n for n in golden_names() if "conv" in load_golden(n)["runs"]]


def _ctx(plan, prec=NM_FP64, device=True):
    c = Context(plan, prec)
    if device:
        c.set_option(_abi.NM_OPT_DEVICE_LOOP, 1)
    return c


@pytest.mark.parametrize("name", CONV)
def test_device_loop_converges_to_reference(name):
    g = load_golden(name)
    run = g["runs"]["conv"]
    plan = Plan(run["input"])
    c = _ctx(plan)
    res, phi = c.solve_host(np.array(run["x"]))
    assert res.status == 0 and res.residual < newton_tolerance(run), res
    host, _ = _ctx(plan, device=False).solve_host(np.array(run["x"]))
    # slowly converging fixtures (the charged cylinder takes ~3000 iterations)
    # wander further apart near convergence
    assert res.iterations <= 2 * host.iterations + 10, (res.iterations, host.iterations)
    # the device loop's rounding (FMA contraction in the pseudo-inverse) splits
    # its path from the reference's: held to the fixture's convergence ball
    tol = g.get("split_tol", 1e-5)
    phi = phi.reshape(plan.n_seg, plan.M)
    for i, seg in enumerate(plan.seg_names):
        assert rel_err(interior(plan, phi[i]), pro_column(run, f"mon_{seg}_phi")) < tol, seg
    k = run["kal"]
    F, _, _ = c.free_energy()
    assert abs(F - k["sys_noname_free_energy"]) <= tol * max(1, abs(k["sys_noname_free_energy"]))


def test_device_loop_fp32_3d_and_iteration_limit():
    import bench
    # a 12³ melt at χ 0.05: the oracle's DIIS converges in 549 iterations (at
    # χ 0.3 a small box runs away to fields where G1 underflows)
    plan = Plan(bench.melt3d_text(12, 3000).replace("chi_B : 0.3", "chi_B : 0.05"))
    u = np.random.default_rng(4).uniform(-0.05, 0.05, plan.M)
    x0 = np.concatenate([u, -u])
    c64 = _ctx(plan, NM_FP64, device=False)
    x64 = x0.copy()
    r64, _ = c64.solve_host(x64)
    assert r64.status == 0 and r64.residual > 0 and np.abs(x64).max() < 1, (r64, np.abs(x64).max())
    rh, _ = _ctx(plan, NM_FP32, device=False).solve_host(x0.copy())
    c = _ctx(plan, NM_FP32)
    x = x0.copy()
    r, _ = c.solve_host(x)
    assert r.status == 0 and r.residual < plan.c.tolerance, (r, rh, r64)
    assert r.iterations <= 2 * rh.iterations + 10, (r, rh)
    # the same fixed point: φ of both segment types from one FP64 residual at
    # each solution (a melt's F is not defined: every molecule is the solvent)
    ref = _ctx(plan, NM_FP64, device=False)
    phis = []
    for xs in (x, x64):
        xd = torch.from_numpy(xs).cuda()
        gd = torch.zeros_like(xd)
        ref.residual_dev(xd.data_ptr(), gd.data_ptr())
        torch.cuda.synchronize()
        phis.append(ref.field(0).reshape(plan.n_seg, -1))
    for which in range(plan.n_seg):
        a, b = interior(plan, phis[0][which]), interior(plan, phis[1][which])
        assert np.isfinite(a).all() and np.isfinite(b).all(), (which, np.isnan(a).sum(), np.isnan(b).sum())
        assert rel_err(a, b) < 1e-5, (which, rel_err(a, b))
    # the iteration limit: the same status and count as the host loop
    lim = Plan(bench.melt3d_text(12, 7).replace("chi_B : 0.3", "chi_B : 0.05"))
    for prec in (NM_FP32, NM_FP64):
        rd, _ = _ctx(lim, prec).solve_host(x0.copy())
        rh, _ = _ctx(lim, prec, device=False).solve_host(x0.copy())
        assert (rd.iterations, rd.status) == (rh.iterations, rh.status) == (7, _abi.NM_ERR_NOT_CONVERGED)


def test_device_loop_search():
    gold = Path(__file__).resolve().parent / "golden" / "search_theta_omega.json"
    g = json.loads(gold.read_text())
    plan = Plan(g["input"])
    c = _ctx(plan)
    x = torch.from_numpy(np.array(g["x"])).cuda()
    r = c.search(x.data_ptr())
    tol = plan.c.super_tolerance
    assert r.status == 0 and abs(r.error) <= tol, r
    k = g["kal"]
    assert abs(r.value - k["mol_pol_theta"]) <= 1e-4 * k["mol_pol_theta"]
    _, O, _ = c.free_energy()
    assert abs(O - plan.c.target_value) <= tol
