"""CUDA path against the CPU oracle and the reference's golden outputs.

Every call goes through the C ABI (include/namics_gb300.h).  Tolerances:
FP64 single residual evaluations agree with the oracle to 1e-10 relative
(the GPU contracts multiply-adds, the reference does not); converged solves
agree to 1e-8 relative when the DIIS path is the same and to the convergence
ball (1e-6 on φ and F) otherwise; the FP32-propagator solver is held to
1e-6 on φ and 1e-7 relative on F against the FP64 oracle.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from helpers import interior, newton_tolerance, pro_column, rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from namics_gb300 import NM_FP32, NM_FP64, Batch, Context, Plan  # noqa: E402
from orc import Oracle  # noqa: E402

CASES = golden_names()


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


@pytest.mark.parametrize("name", CASES)
def test_residual_matches_oracle(name):
    g = load_golden(name)
    run = next(iter(g["runs"].values()))
    plan = Plan(run["input"])
    ctx = Context(plan, NM_FP64)
    orc = Oracle(plan)
    x = np.array(run["x"])
    rc, g_orc = orc.residual(x)
    assert rc == 0
    xd, gd = dev(x), torch.zeros(plan.iv, dtype=torch.float64, device="cuda")
    ctx.residual_dev(xd.data_ptr(), gd.data_ptr())
    g_gpu = host(gd)
    assert rel_err(g_gpu, g_orc) < 1e-10
    for which in (0, 1):
        a, b = ctx.field(which).reshape(plan.n_seg, -1), orc.field(which).reshape(plan.n_seg, -1)
        for i in range(plan.n_seg):
            assert rel_err(interior(plan, a[i]), interior(plan, b[i])) < 1e-10, (which, i)
    assert rel_err(interior(plan, ctx.field(2)), interior(plan, orc.field(2))) < 1e-10
    if plan.c.n_state:  # the internal states' volume fractions, fractions α and potentials u
        for which in (9, 10, 11):
            a, b = ctx.field(which).reshape(plan.c.n_state, -1), orc.field(which).reshape(plan.c.n_state, -1)
            for j in range(plan.c.n_state):
                assert rel_err(interior(plan, a[j]), interior(plan, b[j])) < 1e-10, ("state", which, j)
    for m in range(plan.n_mol):
        assert abs(ctx.molecule(m)["GN"] / orc.molecule(m)["GN"] - 1) < 1e-10
    F, O, mu = ctx.free_energy()
    Fo, Oo, muo = orc.free_energy()
    assert abs(F - Fo) <= 1e-10 * max(1, abs(Fo))
    assert abs(O - Oo) <= 1e-10 * max(1, abs(Oo))
    assert np.allclose(mu, muo, rtol=1e-10, atol=1e-10)
    assert ctx.launch_count() > 0
    if plan.c.charged:
        # ψ, and q and ε at every site: ε at the halo layers comes from the
        # reference's flat-array composition there and feeds the Poisson update
        # (element-wise: ε reaches ~1e8 at halo sites where φ_tot is tiny)
        assert rel_err(interior(plan, ctx.field(6)), interior(plan, orc.field(6))) < 1e-10
        for which in (7, 8):
            a, b = ctx.field(which), orc.field(which)
            assert np.allclose(a, b, rtol=1e-9, atol=1e-10), (which, np.max(np.abs(a - b)))


@pytest.mark.parametrize("name", CASES)
def test_solve_matches_reference(name):
    g = load_golden(name)
    for mode, run in g["runs"].items():
        if mode == "it0":
            continue
        plan = Plan(run["input"])
        ctx = Context(plan, NM_FP64)
        res, phi = ctx.solve_host(np.array(run["x"]))
        k = run["kal"]
        same = res.iterations == int(k["newton_isaac_iterations"])
        if mode == "conv":
            assert res.status == 0 and res.residual < newton_tolerance(run)
        # along the reference's DIIS path: 1e-8 (the fixture's path_tol where
        # rounding drifts further); on a split path the convergence ball, which
        # the weakly constrained charged cylindrical fixtures widen (split_tol)
        split = g.get("split_tol", 1e-5)
        tol = g.get("path_tol", 1e-8) if same else (split if split > 1e-5 else 1e-6)
        if mode != "conv":
            tol = 1e-6  # a few iterations from an unstable start
        phi = phi.reshape(plan.n_seg, plan.M)
        # nm_solve_host returns φ of the last residual evaluation, like the .pro
        for i, seg in enumerate(plan.seg_names):
            assert rel_err(interior(plan, phi[i]), pro_column(run, f"mon_{seg}_phi")) < tol, (mode, seg)
        F, O, _ = ctx.free_energy()
        assert abs(F - k["sys_noname_free_energy"]) <= tol * max(1, abs(k["sys_noname_free_energy"]))


def _batch_cases():
    out = []
    for n in CASES:
        g = load_golden(n)
        if "conv" in g["runs"]:
            p = Plan(g["runs"]["conv"]["input"])
            markov2 = any(p.c.mols[m].markov == 2 for m in range(p.c.n_mol))
            # the batched solver's scope
            if p.c.gradients == 1 and not p.c.charged and not markov2 and not p.c.n_state:
                out.append(n)
    return out


def test_batched_fp64_matches_reference():
    """FP64 batched solver: the reference's arithmetic and DIIS path."""
    names = _batch_cases()
    runs = [load_golden(n)["runs"]["conv"] for n in names]
    plans = [Plan(r["input"]) for r in runs]
    b = Batch(plans, NM_FP64)
    x = np.concatenate([np.array(r["x"]) for r in runs])
    its, res, st = b.solve_host(x)
    assert (st == 0).all(), (names, st, res)
    assert (res < 1e-7).all()
    F, O = b.free_energy()
    for i, (n, r) in enumerate(zip(names, runs)):
        k = r["kal"]
        Fr = k["sys_noname_free_energy"]
        # curved lattices weight F by the site volume L (~4πr²), which turns the
        # convergence ball ‖g‖ < 1e-7 into F differences of a few 1e-7
        same = its[i] == int(k["newton_isaac_iterations"])
        tol = 1e-6 if same else 1e-5
        assert abs(F[i] - Fr) <= tol * max(1, abs(Fr)), (n, F[i], Fr, its[i], k["newton_isaac_iterations"])
        ctx = Context(plans[i], NM_FP64)
        xd = dev(x[b.offsets[i]:b.offsets[i + 1]])
        gd = torch.zeros_like(xd)
        ctx.residual_dev(xd.data_ptr(), gd.data_ptr())
        phi = ctx.field(0).reshape(plans[i].n_seg, -1)
        for j, seg in enumerate(plans[i].seg_names):
            assert rel_err(interior(plans[i], phi[j]), pro_column(r, f"mon_{seg}_phi")) < (1e-6 if same else 1e-5), (n, seg)


def _tight(text: str) -> str:
    import re
    text = re.sub(r"newton : isaac : tolerance : \S+", "newton : isaac : tolerance : 1e-10", text)
    return re.sub(r"newton : isaac : iterationlimit : \S+", "newton : isaac : iterationlimit : 3000", text)


def test_batched_fp32_matches_oracle():
    """FP32-propagator solver (FP64 finish): against the reference's converged
    outputs (both at ‖g‖ < 1e-7), and against the FP64 oracle with both
    solved to ‖g‖ < 1e-10, where φ must agree to 1e-6 and F to 1e-7."""
    names = _batch_cases()
    runs = [load_golden(n)["runs"]["conv"] for n in names]
    plans = [Plan(r["input"]) for r in runs]
    b = Batch(plans, NM_FP32)
    x = np.concatenate([np.array(r["x"]) for r in runs])
    its, res, st = b.solve_host(x)
    assert (st == 0).all(), (names, st, res)
    assert (res < 1e-7).all()
    F, _ = b.free_energy()
    for i, (n, r) in enumerate(zip(names, runs)):
        Fr = r["kal"]["sys_noname_free_energy"]
        assert abs(F[i] - Fr) <= 1e-5 * max(1, abs(Fr)), (n, F[i], Fr)
    tplans = [Plan(_tight(r["input"])) for r in runs]
    tb = Batch(tplans, NM_FP32)
    xt = np.concatenate([np.array(r["x"]) for r in runs])
    its, res, st = tb.solve_host(xt)
    assert (st == 0).all() and (res < 1e-10).all(), (st, res)
    Ft, _ = tb.free_energy()
    for i, (n, r) in enumerate(zip(names, runs)):
        orc = Oracle(tplans[i])
        rc, xo, _, ro = orc.solve(np.array(r["x"]))
        assert rc == 0 and ro < 1e-10
        Fo, _, _ = orc.free_energy()
        assert abs(Ft[i] - Fo) <= 1e-7 * max(1, abs(Fo)), (n, Ft[i], Fo)
        ctx = Context(tplans[i], NM_FP64)
        xd = dev(xt[tb.offsets[i]:tb.offsets[i + 1]])
        gd = torch.zeros_like(xd)
        ctx.residual_dev(xd.data_ptr(), gd.data_ptr())
        phi = ctx.field(0).reshape(tplans[i].n_seg, -1)
        phio = orc.field(0).reshape(tplans[i].n_seg, -1)
        for j in range(tplans[i].n_seg):
            assert rel_err(interior(tplans[i], phi[j]), interior(tplans[i], phio[j])) < 1e-6, (n, j)


def test_batched_fp64_equals_single_problem_path():
    """Same problem alone and inside a batch: identical results (the CTA of
    one problem does not depend on its neighbours)."""
    names = _batch_cases()[:4]
    runs = [load_golden(n)["runs"]["conv"] for n in names]
    plans = [Plan(r["input"]) for r in runs]
    x = np.concatenate([np.array(r["x"]) for r in runs])
    b = Batch(plans, NM_FP64)
    xb = x.copy()
    its_b, _, _ = b.solve_host(xb)
    for i in range(len(plans)):
        bi = Batch([plans[i]], NM_FP64)
        xi = np.array(runs[i]["x"])
        its_i, _, _ = bi.solve_host(xi)
        assert its_i[0] == its_b[i]
        assert np.array_equal(xi, xb[b.offsets[i]:b.offsets[i + 1]])


@pytest.mark.parametrize("name", CASES)
def test_propagate_and_side_match_oracle(name):
    g = load_golden(name)
    run = next(iter(g["runs"].values()))
    plan = Plan(run["input"])
    ctx = Context(plan, NM_FP64)
    orc = Oracle(plan)
    rng = np.random.default_rng(7)
    G = rng.uniform(0.5, 1.5, plan.M)
    G1 = rng.uniform(0.5, 1.5, plan.M)
    X = rng.uniform(0, 1, plan.M)
    # a 'surface' halo layer is a frozen wall: set_bounds leaves it alone and
    # every propagator of a solve is 0 there (G1 = 0 on frozen sites), so the
    # inputs carry that 0; φ_side reads the wall's frozen volume fraction,
    # which any value stands for
    wall = _surface_halo(plan)
    G[wall] = 0.0
    mask = plan.interior_mask()
    ref = orc.propagate(G * 1.0, G1)
    Gd, G1d, out = dev(G), dev(G1), torch.zeros(plan.M, dtype=torch.float64, device="cuda")
    ctx.propagate_dev(Gd.data_ptr(), G1d.data_ptr(), out.data_ptr())
    assert rel_err(host(out)[mask], ref[mask]) < 1e-12
    side_ref = orc.side(orc_bounds(orc, X))
    out2 = torch.zeros_like(out)
    ctx.side_dev(dev(X).data_ptr(), out2.data_ptr())
    assert rel_err(host(out2)[mask], side_ref[mask]) < 1e-12


def _surface_halo(plan):
    """Boolean [M]: the halo sites of faces whose boundary is 'surface'
    (bc order x-low, y-low, z-low, x-high, y-high, z-high)."""
    c = plan.c
    shape = plan.shape
    m = np.zeros(shape, dtype=bool)
    for ax in range(len(shape)):
        for side, k in ((0, ax), (1, ax + 3)):
            if c.bc[k] == 2:
                sl = [slice(None)] * len(shape)
                sl[ax] = 0 if side == 0 else shape[ax] - 1
                m[tuple(sl)] = True
    return m.reshape(-1)


def orc_bounds(orc, X):
    # Side() reads halos as set_bounds leaves them: apply set_bounds through a
    # propagate with G1 = 1 of a copy (propagate refreshes the input's halo)
    Y = np.ascontiguousarray(X, dtype=np.float64).copy()
    import ctypes as C
    from orc import load, _p
    out = np.zeros_like(Y)
    load().orc_propagate(orc._h, _p(Y), None, _p(out))
    return Y


def test_solves_are_deterministic():
    run = load_golden("brush2d_cyl")["runs"]["conv"]
    plan = Plan(run["input"])
    ctx = Context(plan, NM_FP64)
    x1 = np.array(run["x"])
    x2 = x1.copy()
    r1, _ = ctx.solve_host(x1)
    r2, _ = ctx.solve_host(x2)
    assert r1.iterations == r2.iterations
    assert np.array_equal(x1, x2)


def test_batched_residual_fp32_close_to_oracle():
    """One FP32-propagator residual per problem against the FP64 oracle, at
    the seeded start field and at the converged field (the FP32 phase hands
    over at ‖g‖ < 2e-6, so its residual must be accurate well below that)."""
    names = _batch_cases()
    runs = [load_golden(n)["runs"]["conv"] for n in names]
    plans = [Plan(r["input"]) for r in runs]
    b = Batch(plans, NM_FP32)
    x0 = np.concatenate([np.array(r["x"]) for r in runs])
    xc = x0.copy()
    Batch(plans, NM_FP64).solve_host(xc)
    for x in (x0, xc):
        xd = dev(x)
        g32 = torch.zeros_like(xd)
        g64 = torch.zeros_like(xd)
        b.residual_dev(xd.data_ptr(), g32.data_ptr(), NM_FP32)
        b.residual_dev(xd.data_ptr(), g64.data_ptr(), NM_FP64)
        a32, a64 = host(g32), host(g64)
        for i, p in enumerate(plans):
            lo, hi = b.offsets[i], b.offsets[i + 1]
            _, go = Oracle(p).residual(x[lo:hi])
            assert np.max(np.abs(a64[lo:hi] - go)) < 1e-10, names[i]
            assert np.linalg.norm(a32[lo:hi] - go) < _fp32_floor(p) * max(1.0, np.linalg.norm(go)), \
                (names[i], np.linalg.norm(a32[lo:hi] - go), np.linalg.norm(go))


def _fp32_floor(plan) -> float:
    """Accuracy of an FP32-propagator residual.  G1 held in FP32 is the exact
    G1 of a field perturbed by ~6e-8 per site, and a chain of N segments
    answers such a perturbation with a change of φ up to ~N·6e-8."""
    n = max(plan.chainlength(m) for m in range(plan.n_mol))
    return 1e-7 * n + 1e-6


def test_batched_residual_fp32_stretched_stars():
    """Grafted stars of the 1-D batch workload at their converged fields: the
    arms meet at the branch point with barely overlapping profiles, so the
    join product and the composition must not underflow in FP32."""
    import bench
    texts = bench.workload(512)
    pick = [319, 469, 479]
    plans = [Plan(texts[i]) for i in pick]
    xs = bench.fields([Plan(t) for t in texts])
    x = np.concatenate([xs[i] for i in pick])
    its, res, st = Batch(plans, NM_FP64).solve_host(x)
    assert (st == 0).all(), st
    b = Batch(plans, NM_FP32)
    xd = dev(x)
    g32 = torch.zeros_like(xd)
    g64 = torch.zeros_like(xd)
    b.residual_dev(xd.data_ptr(), g32.data_ptr(), NM_FP32)
    b.residual_dev(xd.data_ptr(), g64.data_ptr(), NM_FP64)
    a32, a64 = host(g32), host(g64)
    for i, p in enumerate(plans):
        lo, hi = b.offsets[i], b.offsets[i + 1]
        _, go = Oracle(p).residual(x[lo:hi])
        assert np.max(np.abs(a64[lo:hi] - go)) < 1e-10, pick[i]
        assert np.linalg.norm(a32[lo:hi] - go) < _fp32_floor(p), (pick[i], np.linalg.norm(a32[lo:hi] - go))


def _solve_tight(text: str, tol: str = "1e-10", itlim: int = 3000) -> str:
    import re
    text = re.sub(r"newton : isaac : tolerance : \S+", f"newton : isaac : tolerance : {tol}", text)
    return re.sub(r"newton : isaac : iterationlimit : \S+", f"newton : isaac : iterationlimit : {itlim}", text)


def test_context_fp32_3d_matches_oracle():
    """3-D simple-cubic melt with FP32 propagators (one power-of-two exponent
    per stored vector, FP64 normalisation, residual and DIIS, FP64 finish)
    against the FP64 oracle, both solved to ‖g‖ < 1e-9: φ to 1e-6 and F to
    1e-7 relative (the FP32 tolerances of the hot-path contract).  The FP64
    context on the same dedicated 3-D kernels is held to 1e-8 / 1e-9.
    (‖g‖₂ < 1e-10 over these 3456 entries puts the DIIS history matrix at the
    1e-9 regularisation, where the small solve is numerically degenerate for
    the reference's algorithm too.)"""
    run = load_golden("melt3d")["runs"]["it0"]
    plan = Plan(_solve_tight(run["input"], tol="1e-9"))
    x0 = np.array(run["x"])
    orc = Oracle(plan)
    rc, xo, _, ro = orc.solve(x0.copy())
    assert rc == 0 and ro < 1e-9
    Fo, Oo, _ = orc.free_energy()
    phio = orc.field(0).reshape(plan.n_seg, -1)
    for prec in (NM_FP32, NM_FP64):
        ctx = Context(plan, prec)
        res, phi = ctx.solve_host(x0.copy())
        assert res.status == 0 and res.residual < 1e-9, (prec, res)
        F, O, _ = ctx.free_energy()
        tol_phi, tol_F = (1e-6, 1e-7) if prec == NM_FP32 else (1e-8, 1e-9)
        assert abs(F - Fo) <= tol_F * max(1, abs(Fo)), (prec, F, Fo)
        phi = phi.reshape(plan.n_seg, -1)
        for i in range(plan.n_seg):
            assert rel_err(interior(plan, phi[i]), interior(plan, phio[i])) < tol_phi, (prec, i)


def test_context_fp32_residual_3d_close_to_oracle():
    """One FP32-propagator residual of the 3-D melt at its seeded start field;
    the second call replays the captured graph and must give the same g."""
    run = load_golden("melt3d")["runs"]["it0"]
    plan = Plan(run["input"])
    x = np.array(run["x"])
    _, go = Oracle(plan).residual(x)
    ctx = Context(plan, NM_FP32)
    xd, gd = dev(x), torch.zeros(plan.iv, dtype=torch.float64, device="cuda")
    ctx.residual_dev(xd.data_ptr(), gd.data_ptr())
    g1 = host(gd).copy()
    ctx.residual_dev(xd.data_ptr(), gd.data_ptr())
    g = host(gd)
    assert np.array_equal(g, g1)
    assert np.linalg.norm(g - go) < 1e-5 * max(1.0, np.linalg.norm(go)), np.linalg.norm(g - go)


def test_context_fp32_rejects_unsupported_plan():
    from namics_gb300 import NamicsError
    run = load_golden("brush1d_x100")["runs"]["conv"]
    with pytest.raises(NamicsError):
        Context(Plan(run["input"]), NM_FP32)


@pytest.mark.parametrize("nl,N,star", [(300, 240, False), (450, 300, False), (300, 240, True)])
def test_batched_fp32_wide_lattices(nl, N, star):
    """Lattices of 256 < MX <= 512, where the FP32 residual keeps three and
    four sites per thread (the golden fixtures stop at MX 200): one residual
    at the seeded field within the FP32 floor of the oracle, and an
    FP32-first solve to ‖g‖ < 1e-10 against the FP64 oracle solved as far,
    φ to 1e-6 and F to 1e-7."""
    import bench
    plan = Plan(_tight(bench.instance_text(nl, N, 0.05, 0.5, star)))
    assert plan.c.MX == nl
    x0 = bench.fields([plan])[0]
    b = Batch([plan], NM_FP32)
    xd = dev(x0)
    g32 = torch.zeros_like(xd)
    b.residual_dev(xd.data_ptr(), g32.data_ptr(), NM_FP32)
    orc = Oracle(plan)
    _, go = orc.residual(x0)
    assert np.linalg.norm(host(g32) - go) < _fp32_floor(plan) * max(1.0, np.linalg.norm(go))
    x = x0.copy()
    its, res, st = b.solve_host(x)
    assert st[0] == 0 and res[0] < 1e-10, (its, res, st)
    F, _ = b.free_energy()
    rc, xo, _, ro = orc.solve(x0.copy())
    assert rc == 0 and ro < 1e-10
    Fo, _, _ = orc.free_energy()
    assert abs(F[0] - Fo) <= 1e-7 * max(1, abs(Fo)), (F[0], Fo)
    ctx = Context(plan, NM_FP64)
    xd = dev(x)
    gd = torch.zeros_like(xd)
    ctx.residual_dev(xd.data_ptr(), gd.data_ptr())
    phi = ctx.field(0).reshape(plan.n_seg, -1)
    phio = orc.field(0).reshape(plan.n_seg, -1)
    for j in range(plan.n_seg):
        assert rel_err(interior(plan, phi[j]), interior(plan, phio[j])) < 1e-6, j


def test_work_loop_results_independent_of_slots():
    """The batch's work loop with every problem in its own slot and with three
    slots taking turns (each slot's scratch reused by many problems, stale
    contents included): identical iterations and fields, bit for bit, in
    both precisions; and the same as each problem solved alone."""
    import bench
    texts = bench.workload(24)
    plans = [Plan(t) for t in texts]
    x = np.concatenate(bench.fields(plans))
    for prec in (NM_FP64, NM_FP32):
        b = Batch(plans, prec)
        assert b.slots == len(plans)
        x_all = x.copy()
        its_a, res_a, st_a = b.solve_host(x_all)
        b.slots = 3
        x_3 = x.copy()
        its_3, res_3, st_3 = b.solve_host(x_3)
        assert np.array_equal(its_a, its_3) and np.array_equal(st_a, st_3)
        assert np.array_equal(x_all, x_3)
        q, s = b.timings()
        assert (s > 0).all() and (q >= 0).all()
        for i in (0, 9, 17):
            xi = x[b.offsets[i]:b.offsets[i + 1]].copy()
            its_i, _, _ = Batch([plans[i]], prec).solve_host(xi)
            assert its_i[0] == its_a[i]
            assert np.array_equal(xi, x_all[b.offsets[i]:b.offsets[i + 1]])


@pytest.mark.parametrize("prec", [NM_FP64, NM_FP32])
def test_checkpointed_storage_is_bit_identical(prec):
    """3-D melt: every forward propagator stored, against every k-th stored
    and the rest recomputed in the backward sweep (k = 3, 7, 10, and the
    reference's own slot count for `save_memory : true`, round(√(2·50)) = 10
    slots, a stride of 5): the same residual bit for bit, and the same solve."""
    import bench
    run = load_golden("melt3d")["runs"]["it0"]
    plan = Plan(run["input"])
    x0 = np.array(run["x"])
    big = Plan(bench.melt3d_text(24, 30))
    u = np.random.default_rng(5).uniform(-0.1, 0.1, big.M)
    for p, x in ((plan, x0), (big, np.concatenate([u, -u]))):
        ref = Context(p, prec)
        xd = dev(x)
        g0 = torch.zeros_like(xd)
        ref.residual_dev(xd.data_ptr(), g0.data_ptr())
        g0 = host(g0)
        variants = [Context(p, prec, checkpoint_stride=k) for k in (3, 7, 10)]
        text = run["input"] if p is plan else bench.melt3d_text(24, 30)
        sm = Plan(text.replace("mol : AB : freedom : solvent", "mol : AB : freedom : solvent\nmol : AB : save_memory : true")
                  if "mol : AB" in text else text)
        assert sm.c.save_memory == ("mol : AB" in text)
        variants.append(Context(sm, prec))
        for c in variants:
            g = torch.zeros_like(xd)
            c.residual_dev(xd.data_ptr(), g.data_ptr())
            assert np.array_equal(host(g), g0)
        if p is big:  # 30 DIIS iterations
            x1 = x.copy()
            r0, _ = ref.solve_host(x1)
            for c in variants:
                xc = x.copy()
                r, _ = c.solve_host(xc)
                assert (r.iterations, r.residual) == (r0.iterations, r0.residual)
                assert np.array_equal(xc, x1)


def test_autotuners_keep_results_and_cache_their_choice():
    """nm_ctx_autotune on a 3-D melt and nm_batch_autotune on a batch of the
    1-D workload: a choice among the candidates, the same residual and solve
    as the untuned defaults bit for bit, and the cached choice on a second
    call of the same shape (no candidates timed)."""
    import bench
    plan = Plan(bench.melt3d_text(24, 10))
    u = np.random.default_rng(9).uniform(-0.1, 0.1, plan.M)
    x = np.concatenate([u, -u])
    for prec in (NM_FP64, NM_FP32):
        ref = Context(plan, prec)
        xd = dev(x)
        g0 = torch.zeros_like(xd)
        ref.residual_dev(xd.data_ptr(), g0.data_ptr())
        c = Context(plan, prec)
        t = c.autotune(xd.data_ptr())
        # FP32: the cluster sweeps are one more candidate on this machine
        assert t["checkpoint_stride"] in (0, 5, 10) and t["candidates"] == (22 if prec == NM_FP32 else 21), t
        assert t["tile"] in (204, 208, 404, 408) or (t["tile"] == 0 and t["rows"] in (2, 4, 8)), t
        assert t["cluster3d"] in ((0, 1) if prec == NM_FP32 else (-1,)), t
        g = torch.zeros_like(xd)
        c.residual_dev(xd.data_ptr(), g.data_ptr())
        assert np.array_equal(host(g), host(g0))
        t2 = Context(plan, prec).autotune(xd.data_ptr())
        assert t2["candidates"] == 0
        assert (t2["rows"], t2["tile"], t2["checkpoint_stride"], t2["cluster3d"]) == \
            (t["rows"], t["tile"], t["checkpoint_stride"], t["cluster3d"])
    texts = bench.workload(48)
    plans = [Plan(t) for t in texts]
    xb = np.concatenate(bench.fields(plans))
    b = Batch(plans, NM_FP32)
    x0 = xb.copy()
    its0, _, _ = b.solve_host(x0)
    xbd = dev(xb)
    t = b.autotune(xbd.data_ptr())
    assert 1 <= t["ctas_per_sm"] <= 3 and t["candidates"] >= 1, t
    assert np.array_equal(host(xbd), xb)  # the tuner leaves the fields alone
    x1 = xb.copy()
    its1, _, _ = b.solve_host(x1)
    assert np.array_equal(its0, its1) and np.array_equal(x0, x1)
    assert Batch(plans, NM_FP32).autotune(xbd.data_ptr())["candidates"] == 0


@pytest.mark.parametrize("prec", [NM_FP64, NM_FP32])
def test_tiled_3d_steps_are_bit_identical(prec):
    """The 2.5-D shared-memory tile steps (every rows × planes variant)
    against the gather steps: the same residual bit for bit, on a periodic
    melt, on a mirror-bounded box whose edges are not multiples of the tile
    (partial row and plane blocks), and on a box wider than one 128-slot z
    chunk; and the same 12-iteration solve."""
    import bench
    from namics_gb300 import _abi
    texts = [bench.melt3d_text(24, 12),
             bench.melt3d_text(21, 12).replace("periodic", "mirror"),
             bench.melt3d_text(9, 12).replace("n_layers_z : 9", "n_layers_z : 150")]
    for text in texts:
        plan = Plan(text)
        u = np.random.default_rng(3).uniform(-0.1, 0.1, plan.M)
        x = np.concatenate([u, -u])
        xd = dev(x)
        ref = Context(plan, prec)
        if prec == NM_FP32:  # the gather and tile steps, not the cluster sweeps
            ref.set_option(_abi.NM_OPT_CLUSTER3D, 0)
        g0 = torch.zeros_like(xd)
        ref.residual_dev(xd.data_ptr(), g0.data_ptr())
        g0 = host(g0)
        x1 = x.copy()
        r0, _ = ref.solve_host(x1)
        for tile in (204, 208, 404, 408):
            c = Context(plan, prec)
            if prec == NM_FP32:
                c.set_option(_abi.NM_OPT_CLUSTER3D, 0)
            c.set_option(_abi.NM_OPT_TILE3D, tile)
            g = torch.zeros_like(xd)
            c.residual_dev(xd.data_ptr(), g.data_ptr())
            assert np.array_equal(host(g), g0), (text.splitlines()[1], tile)
            xt = x.copy()
            r, _ = c.solve_host(xt)
            assert (r.iterations, r.residual) == (r0.iterations, r0.residual) and np.array_equal(xt, x1)


def test_batched_fp32_first_agrees_with_fp64_on_the_workload():
    """FP32-first (5-deep FP32 DIIS history, FP64 finish) against FP64
    throughout on 128 instances of the batched workload: no solve ends on a
    degenerate zero residual, every problem both converge agrees to 1e-5 in
    the field, and FP32-first converges about as many."""
    import bench
    texts = bench.workload(128)
    plans = [Plan(t) for t in texts]
    x0 = np.concatenate(bench.fields(plans))
    out = {}
    for prec in (NM_FP32, NM_FP64):
        b = Batch(plans, prec)
        x = x0.copy()
        it, res, st = b.solve_host(x)
        out[prec] = (x, np.array(res), np.array(st), b.offsets.copy())
        b.close()
    x32, r32, s32, off = out[NM_FP32]
    x64, r64, s64, _ = out[NM_FP64]
    assert not np.any((s32 == 0) & (r32 == 0.0))
    both = np.where((s32 == 0) & (s64 == 0))[0]
    assert len(both) >= 0.9 * len(plans)
    for i in both:
        assert np.max(np.abs(x32[off[i]:off[i + 1]] - x64[off[i]:off[i + 1]])) < 1e-5, i
    assert np.sum(s32 == 0) >= np.sum(s64 == 0) - 2
