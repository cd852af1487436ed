"""Parity at the workloads' own sizes (not only the small golden fixtures).

For each workload shape the bench measures, one residual evaluation at its
seeded start field on the device against the oracle:
  * the 1-D brush (100 layers, (X)1(A)99, σ 0.05) is the golden fixture
    brush1d_x100 and is covered by test_parity_tight.py at 1e-10 converged;
  * the 128³ periodic (A)50(B)50 melt, χ_AB 0.3, u_A = -u_B ~ U(-0.1, 0.1);
  * the 200×200 cylindrical charged brush (X)1(A)499, σ 0.02, χ_AS 0 and 0.5;
  * all 512 batched 1-D brushes/stars of the batch workload;
  * the request stream's 2-D 100×100 (A)200 adsorption and 3-D 64³ (A)20(B)20
    melt at χ_AB 0.4.
FP64: g, φ (every segment type, interior), GN and F within 1e-10 relative of
the oracle (ψ, q and ε too where charged).  FP32 propagators: max |Δφ| of the
same residual against the oracle, within the FP32 floor of a chain of N
segments, (1e-7·N + 1e-6); the measured value is printed and, when the
environment variable NM_PARITY_REPORT names a file, appended to it as JSON.
The 100×100 adsorption is also solved to its fixed point on both sides
(DIIS, then tests/helpers.anderson_polish below ‖g‖ = 1e-12) and compared
at 1e-10.
"""
import json
import os

import numpy as np
import pytest

import bench
from helpers import anderson_polish, interior, rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from namics_gb300 import NM_FP32, NM_FP64, Batch, Context, Plan  # noqa: E402
from orc import Oracle  # noqa: E402


def _report(**kv):
    print(json.dumps(kv))
    path = os.environ.get("NM_PARITY_REPORT")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps(kv) + "\n")


def _fp32_floor(plan) -> float:
    n = max(plan.chainlength(m) for m in range(plan.n_mol))
    return 1e-7 * n + 1e-6


def _residual(ctx, plan, x):
    xd = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    gd = torch.zeros_like(xd)
    ctx.residual_dev(xd.data_ptr(), gd.data_ptr())
    torch.cuda.synchronize()
    return gd.cpu().numpy()


def _check_single_residual(label, plan, x, fp32=True):
    orc = Oracle(plan)
    rc, go = orc.residual(x)
    assert rc == 0
    phio = orc.field(0).reshape(plan.n_seg, -1)
    Fo, Oo, _ = orc.free_energy()
    ctx = Context(plan, NM_FP64)
    g = _residual(ctx, plan, x)
    assert rel_err(g, go) < 1e-10, rel_err(g, go)
    phi = ctx.field(0).reshape(plan.n_seg, -1)
    for i in range(plan.n_seg):
        b = interior(plan, phio[i])
        if np.max(np.abs(b)) > 0:
            assert rel_err(interior(plan, phi[i]), b) < 1e-10, (plan.seg_names[i],)
    for m in range(plan.n_mol):
        assert abs(ctx.molecule(m)["GN"] / orc.molecule(m)["GN"] - 1) < 1e-10
    F, O, _ = ctx.free_energy()
    assert abs(F - Fo) <= 1e-10 * max(1, abs(Fo)), (F, Fo)
    assert abs(O - Oo) <= 1e-10 * max(1, abs(Oo)), (O, Oo)
    if plan.c.charged:
        assert rel_err(interior(plan, ctx.field(6)), interior(plan, orc.field(6))) < 1e-10
        for which in (7, 8):
            a, b = ctx.field(which), orc.field(which)
            assert np.allclose(a, b, rtol=1e-9, atol=1e-10), (which, np.max(np.abs(a - b)))
    ctx.close()
    out = {"workload": label, "fp64_rel_err_g": rel_err(g, go)}
    if fp32:
        c32 = Context(plan, NM_FP32)
        _residual(c32, plan, x)
        phi32 = c32.field(0).reshape(plan.n_seg, -1)
        dphi = max(float(np.max(np.abs(interior(plan, phi32[i]) - interior(plan, phio[i]))))
                   for i in range(plan.n_seg))
        F32, _, _ = c32.free_energy()
        c32.close()
        out.update(fp32_max_abs_dphi=dphi, fp32_rel_dF=abs(F32 - Fo) / max(1, abs(Fo)))
        assert dphi < _fp32_floor(plan), out
    _report(**out)


def test_melt128_single_residual():
    plan = Plan(bench.melt3d_text(128, 20))
    u = np.random.default_rng(bench.SEED).uniform(-0.1, 0.1, size=plan.M)
    _check_single_residual("128^3 (A)50(B)50 melt, chi 0.3", plan, np.concatenate([u, -u]))


@pytest.mark.parametrize("chi", [0.0, 0.5])
def test_cylinder200_charged_single_residual(chi):
    plan = bench.cyl2d_plan(200, 200, 500, 0.02, chi, 20)
    x = np.random.default_rng(bench.SEED + int(chi > 0)).uniform(-0.01, 0.01, size=plan.iv)
    _check_single_residual(f"200x200 cylindrical charged brush A500, chi {chi}", plan, x)


def test_ads100_single_residual():
    plan = Plan(bench.ads2d_text())
    x = np.random.default_rng(bench.SEED + 3).uniform(-0.01, 0.01, size=plan.iv)
    _check_single_residual("100x100 (A)200 adsorption", plan, x)


def test_melt64_single_residual():
    plan = Plan(bench.melt3d_small_text())
    u = np.random.default_rng(bench.SEED + 4).uniform(-0.1, 0.1, size=plan.M)
    _check_single_residual("64^3 (A)20(B)20 melt, chi 0.4", plan, np.concatenate([u, -u]))


def test_batch512_single_residuals():
    """Every instance of the 512-problem batch workload: one FP64 residual per
    problem within 1e-10 (max |Δg|) of the oracle, one FP32 residual within
    the FP32 floor."""
    texts = bench.workload(512)
    plans = [Plan(t) for t in texts]
    xs = bench.fields(plans)
    x = np.concatenate(xs)
    worst = {"fp64_max_abs_dg": 0.0, "fp32_rel_dg_over_floor": 0.0}
    for prec in (NM_FP64, NM_FP32):
        b = Batch(plans, prec)
        xd = torch.from_numpy(x).cuda()
        gd = torch.zeros_like(xd)
        b.residual_dev(xd.data_ptr(), gd.data_ptr(), prec)
        torch.cuda.synchronize()
        ga = gd.cpu().numpy()
        for i, p in enumerate(plans):
            lo, hi = b.offsets[i], b.offsets[i + 1]
            rc, go = Oracle(p).residual(xs[i])
            assert rc == 0
            if prec == NM_FP64:
                d = float(np.max(np.abs(ga[lo:hi] - go)))
                assert d < 1e-10, (i, d)
                worst["fp64_max_abs_dg"] = max(worst["fp64_max_abs_dg"], d)
            else:
                r = float(np.linalg.norm(ga[lo:hi] - go)) / (_fp32_floor(p) * max(1.0, np.linalg.norm(go)))
                assert r < 1.0, (i, r)
                worst["fp32_rel_dg_over_floor"] = max(worst["fp32_rel_dg_over_floor"], r)
        b.close()
    _report(workload="512 batched 1-D brushes/stars", **worst)


def test_ads100_fixed_point_matches_oracle_1e10():
    """The request stream's 2-D adsorption problem solved to its fixed point:
    the device context's DIIS then Anderson mixing over its own residual,
    against the oracle's DIIS then the same mixing over the oracle's."""
    plan = Plan(bench.ads2d_text())
    x0 = np.random.default_rng(bench.SEED + 3).uniform(-0.01, 0.01, size=plan.iv)
    ctx = Context(plan, NM_FP64)
    xg = x0.copy()
    res, _ = ctx.solve_host(xg, want_phi=False)
    assert res.status == 0, res

    def gres(x):
        return _residual(ctx, plan, x)
    xg, rg, _ = anderson_polish(gres, xg, tol=1e-13)
    orc = Oracle(plan)
    rc, xo, _, _ = orc.solve(x0.copy())
    assert rc == 0

    def ores(x):
        rc, g = orc.residual(x)
        return g if rc == 0 else np.full_like(x, np.nan)
    xo, ro, _ = anderson_polish(ores, xo, tol=1e-13)
    assert rg <= 1e-12 and ro <= 1e-12, (rg, ro)
    gres(xg)
    ores(xo)
    phi = ctx.field(0).reshape(plan.n_seg, -1)
    phio = orc.field(0).reshape(plan.n_seg, -1)
    for i in range(plan.n_seg):
        b = interior(plan, phio[i])
        if np.max(np.abs(b)) > 0:
            assert rel_err(interior(plan, phi[i]), b) < 1e-10, plan.seg_names[i]
    F, O, _ = ctx.free_energy()
    Fo, Oo, _ = orc.free_energy()
    assert abs(F - Fo) <= 1e-10 * max(1, abs(Fo)), (F, Fo)
    _report(workload="100x100 (A)200 adsorption, fixed point", gpu_resid=rg, oracle_resid=ro,
            rel_dF=abs(F - Fo) / max(1, abs(Fo)))
