"""The Lattice / Molecule pieces of the C ABI (nm_add_phi*, nm_initiate_dev,
nm_terminate_dev, nm_weighted_sum_dev, nm_compute_gn_dev, nm_compose_dev)
on every golden fixture's lattice.

Element-wise pieces against the reference's loops written out in numpy in
the reference's operation order (AddTimes, YplusisCtimesAtimesB,
Composition: tools_host.h:349-356, 400-402), bit for bit; the sums against
numpy at 1e-13 relative (another summation order); the composition of each
molecule at the fixture's field against the oracle's Molecule::ComputePhi
(orc_compose) at 1e-12 on interior sites, and its G(N) at 1e-12.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from helpers import interior, rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from namics_gb300 import NM_FP64, Context, NamicsError, Plan  # noqa: E402
from orc import Oracle  # noqa: E402

CASES = golden_names()


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def _plan(name):
    run = next(iter(load_golden(name)["runs"].values()))
    return Plan(run["input"]), np.array(run["x"])


@pytest.mark.parametrize("name", CASES)
def test_add_phi_initiate_terminate(name):
    plan, _ = _plan(name)
    ctx = Context(plan, NM_FP64)
    M = plan.M
    rng = np.random.default_rng(11)
    phi0, gf, gb = rng.uniform(0, 1, M), rng.uniform(0, 1, M), rng.uniform(0, 1, M)
    g1 = rng.uniform(0.1, 1, M)
    g1[::7] = 0.0
    d, norm = 3.0, 0.37
    ph, Gf, Gb, G1 = dev(phi0), dev(gf), dev(gb), dev(g1)
    ctx.add_phi_dev(ph.data_ptr(), Gf.data_ptr(), Gb.data_ptr())
    assert np.array_equal(host(ph), phi0 + gf * gb)
    ph = dev(phi0)
    ctx.add_phi_dev(ph.data_ptr(), Gf.data_ptr(), Gb.data_ptr(), degeneracy=d)
    assert np.array_equal(host(ph), phi0 + (d * gf) * gb)
    ph = dev(phi0)
    if plan.c.gradients == 1:
        ctx.add_phi_dev(ph.data_ptr(), Gf.data_ptr(), Gb.data_ptr(), g1_ptr=G1.data_ptr(), norm=norm)
        ok = g1 > 0
        want = phi0.copy()
        want[ok] = phi0[ok] + (norm * gf[ok]) * gb[ok] / g1[ok]
        assert np.array_equal(host(ph), want)
    else:
        with pytest.raises(NamicsError):
            ctx.add_phi_dev(ph.data_ptr(), Gf.data_ptr(), Gb.data_ptr(), g1_ptr=G1.data_ptr(), norm=norm)
        assert np.array_equal(host(ph), phi0)
    G = torch.zeros(M, dtype=torch.float64, device="cuda")
    ctx.initiate_dev(G.data_ptr(), Gf.data_ptr())
    assert np.array_equal(host(G), gf)
    Gz = dev(phi0)
    ctx.terminate_dev(Gz.data_ptr(), Gb.data_ptr())
    assert np.array_equal(host(Gz), gb)


@pytest.mark.parametrize("name", CASES)
def test_weighted_sum_and_gn(name):
    plan, _ = _plan(name)
    ctx = Context(plan, NM_FP64)
    rng = np.random.default_rng(12)
    X = rng.uniform(0, 1, plan.M)
    inside = plan.interior_mask()
    Xz = np.where(inside, X, 0.0)
    c = plan.c
    curved = c.geometry != 0 and c.gradients < 3
    want = float(np.sum(Xz * np.ctypeslib.as_array(c.L, shape=(plan.M,)))) if curved else float(np.sum(Xz))
    for fn in (ctx.weighted_sum_dev, ctx.compute_gn_dev):
        Xd = dev(X)
        got = fn(Xd.data_ptr())
        assert abs(got - want) <= 1e-13 * abs(want), (got, want)
        assert np.array_equal(host(Xd), Xz)  # remove_bounds acts in place


@pytest.mark.parametrize("name", CASES)
def test_compose_matches_oracle(name):
    plan, x = _plan(name)
    ctx = Context(plan, NM_FP64)
    orc = Oracle(plan)
    xd = dev(x)
    for m in range(plan.n_mol):
        nmm = plan.c.mols[m].n_molmon
        rho = torch.zeros(nmm * plan.M, dtype=torch.float64, device="cuda")
        gn = ctx.compose_dev(m, xd.data_ptr(), rho.data_ptr())
        ro, gno = orc.compose(x, m, nmm)
        assert abs(gn - gno) <= 1e-12 * abs(gno), (m, gn, gno)
        a = host(rho).reshape(nmm, -1)
        b = ro.reshape(nmm, -1)
        for k in range(nmm):
            assert rel_err(interior(plan, a[k]), interior(plan, b[k])) < 1e-12, (m, k)
    # the context still solves from a fresh residual afterwards
    g = torch.zeros_like(xd)
    ctx.residual_dev(xd.data_ptr(), g.data_ptr())
    _, go = orc.residual(x)
    assert rel_err(host(g), go) < 1e-10
