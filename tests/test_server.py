"""Request server (nm_server_*): continuous batching of mixed solves.

Each request's result must be the same when it is solved in the mix
(1-gradient requests in the streaming work loop or batched with each other,
overlapping on other streams, admitted under a memory budget) as when it is
solved alone through the existing entry points: bit-identical here, because
every reduction on the device has a fixed order and a problem's CTA does not
depend on its neighbours.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from namics_gb300 import NM_FP32, NM_FP64, Batch, Context, Plan, Server  # noqa: E402


def _cases():
    out = []
    for n in golden_names():
        runs = load_golden(n)["runs"]
        run = runs.get("conv") or runs.get("it5")
        if run is None:
            continue
        plan = Plan(run["input"])
        if plan.c.gradients == 3 and plan.c.lattice_type != 0:
            continue  # 3-D hexagonal: FP64 generic path, slow to converge; not needed here
        out.append((n, plan, np.array(run["x"])))
    return out


def _alone(plan, x, precision):
    markov2 = any(plan.c.mols[m].markov == 2 for m in range(plan.c.n_mol))
    if plan.c.gradients == 1 and not plan.c.charged and not markov2:  # the server batches these
        xx = x.copy()
        its, res, st = Batch([plan], precision).solve_host(xx)
        return int(its[0]), float(res[0]), int(st[0]), xx
    # the server uses FP32 propagators in a context only for 3-D simple-cubic
    # linear chains (the 3-D hexagonal fixture is left out above)
    prec = precision if (precision == NM_FP64 or (plan.c.gradients == 3 and not plan.c.charged)) else NM_FP64
    ctx = Context(plan, prec)
    xx = x.copy()
    r, _ = ctx.solve_host(xx)
    return r.iterations, r.residual, r.status, xx


@pytest.mark.parametrize("stream_slots", [0, -1])
@pytest.mark.parametrize("precision", [NM_FP32, NM_FP64])
def test_server_results_equal_alone_and_in_the_mix(precision, stream_slots):
    """1-gradient requests through the streaming work loop (stream_slots 0)
    or in batched launches (-1), the others in device contexts."""
    cases = _cases()
    kinds = {c[1].c.gradients for c in cases}
    assert kinds == {1, 2, 3}, kinds
    # a budget that holds only part of the mix at once, so requests queue
    srv = Server(precision=precision, workers=4, max_batch=8, memory_budget=256 << 20, stream_slots=stream_slots)
    ids = [(n, plan, x, srv.submit(plan, x)) for n, plan, x in cases for _ in range(2)]
    results = [(n, plan, x) + srv.wait(rid) for n, plan, x, rid in ids]
    assert srv.launch_count() > 0
    srv.close()
    for n, plan, x, res, xs, sec in results:
        its, resid, st, xa = _alone(plan, x, precision)
        assert res.status == st and res.iterations == its, (n, res, its, st)
        assert res.residual == resid, n
        assert np.array_equal(xs, xa), n
        assert sec > 0


def test_server_rejects_request_beyond_budget():
    from namics_gb300 import NamicsError
    n, plan, x = _cases()[0]
    srv = Server(precision=NM_FP64, workers=1, memory_budget=1 << 10)
    with pytest.raises(NamicsError):
        srv.submit(plan, x)
    srv.close()


def test_server_context_sweep_options_keep_results():
    """nm_server_options.context_sweeps 1 and 2 (persistent 2-D sweeps,
    cluster sweeps of small FP32 3-D boxes) change how the request contexts
    launch their steps, not their arithmetic: the results are those of the
    requests solved alone with one launch per step."""
    cases = [c for c in _cases() if c[1].c.gradients > 1]
    assert {c[1].c.gradients for c in cases} == {2, 3}
    srv = Server(precision=NM_FP32, workers=2, max_batch=8, memory_budget=256 << 20, context_sweeps=3)
    ids = [(n, plan, x, srv.submit(plan, x)) for n, plan, x in cases]
    results = [(n, plan, x) + srv.wait(rid) for n, plan, x, rid in ids]
    srv.close()
    for n, plan, x, res, xs, sec in results:
        its, resid, st, xa = _alone(plan, x, NM_FP32)
        assert res.status == st and res.iterations == its, (n, res, its, st)
        assert np.array_equal(xs, xa), n
