"""The streaming work loop (nm_stream_*): 1-gradient solves submitted while
the loop runs, each admitted into a free slot, against the same problems
solved by the batched work loop (nm_batch_*, the same solve per CTA): the
same iterations and the same field, bit for bit, in both precisions; a
request submitted after the loop left for want of work (idle exit) is
solved by a new launch of it."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import bench  # noqa: E402
from namics_gb300 import NM_FP32, NM_FP64, Batch, NamicsError, Plan, Stream  # noqa: E402


def _workload(n):
    texts = bench.workload(n)
    plans = [Plan(t) for t in texts]
    return plans, bench.fields(plans)


@pytest.mark.parametrize("prec", [NM_FP32, NM_FP64])
def test_stream_equals_batch(prec):
    plans, xs = _workload(40 if prec == NM_FP32 else 12)
    b = Batch(plans, prec)
    xb = np.concatenate(xs)
    its_b, res_b, st_b = b.solve_host(xb)
    s = Stream(capacity=64, idle_seconds=0.2)
    tickets = []
    for i, (p, x) in enumerate(zip(plans, xs)):
        tickets.append(s.submit(p, x, prec))
        if i % 7 == 3:
            time.sleep(0.01)  # later requests arrive while earlier ones run
    for i, t in enumerate(tickets):
        r, x, sec = s.wait(t, plans[i].iv)
        assert (r.iterations, r.status) == (int(its_b[i]), int(st_b[i])), i
        assert r.residual == res_b[i]
        assert np.array_equal(x, xb[b.offsets[i]:b.offsets[i + 1]]), i
        assert sec > 0
    # the loop leaves after 0.2 s without work; the next request relaunches it
    n0 = s.launch_count()
    time.sleep(0.6)
    t = s.submit(plans[0], xs[0], prec)
    r, x, _ = s.wait(t, plans[0].iv)
    assert s.launch_count() > n0
    assert r.iterations == int(its_b[0]) and np.array_equal(x, xb[b.offsets[0]:b.offsets[1]])
    s.close()


def test_stream_refuses_outside_envelope_and_full_ring():
    plans, xs = _workload(4)
    s = Stream(capacity=2, max_layers=100, idle_seconds=0.2)
    big = [i for i, p in enumerate(plans) if p.c.MX > 100]
    if big:
        with pytest.raises(NamicsError):
            s.submit(plans[big[0]], xs[big[0]])
    small = Plan(bench.instance_text(60, 40, 0.05, 0.5, False))
    x = bench.fields([small])[0]
    t1 = s.submit(small, x)
    t2 = s.submit(small, x)
    with pytest.raises(NamicsError):
        s.submit(small, x)  # two requests in a ring of two, neither waited for
    for t in (t1, t2):
        r, _, _ = s.wait(t, small.iv)
        assert r.status == 0
    t3 = s.submit(small, x)
    assert s.wait(t3, small.iv)[0].status == 0
    s.close()
