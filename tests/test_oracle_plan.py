"""The oracle's own plan builder (oracle/orc_plan.py) against the product's
plan compiler: on every 1-gradient neutral golden fixture without a keyword
composition or a Markov 2 chain, and on instances of the batch workload (linear brushes and
3-arm stars), the oracle gives bit-identical residuals and solves from
either record.  The CPU legs of the bench build their problems with
orc_plan only, so this is what ties them to the inputs the device solves."""
import numpy as np
import pytest

import bench
from conftest import golden_names, load_golden
from namics_gb300 import Plan
from orc import Oracle
from orc_plan import OraclePlan


def _cases():
    out = []
    for n in golden_names():
        run = next(iter(load_golden(n)["runs"].values()))
        t = run["input"]
        if "gradients : 1" in t and "valence" not in t and "@" not in t and "Markov : 2" not in t:
            out.append((n, t, np.array(run["x"])))
    return out


CASES = _cases()


def _same(text, x):
    a, b = Oracle(Plan(text)), Oracle(OraclePlan(text))
    ra, ga = a.residual(x)
    rb, gb = b.residual(x)
    assert ra == rb == 0
    assert np.array_equal(ga, gb)
    for which in (0, 1, 2, 3):
        assert np.array_equal(a.field(which), b.field(which)), which
    rca, xa, ita, resa = a.solve(x)
    rcb, xb, itb, resb = b.solve(x)
    assert (rca, ita, resa) == (rcb, itb, resb)
    assert np.array_equal(xa, xb)


def test_fixture_coverage():
    assert len(CASES) >= 11, [c[0] for c in CASES]


@pytest.mark.parametrize("name,text,x", CASES, ids=[c[0] for c in CASES])
def test_oracle_plan_matches_product_plan_on_fixtures(name, text, x):
    _same(text, x)


def test_oracle_plan_matches_product_plan_on_batch_workload():
    texts = bench.workload(40)
    xs = bench.fields([Plan(t) for t in texts])
    for i in list(range(0, 40, 7)) + [9, 19, 29, 39]:   # every 10th instance is a star
        _same(texts[i], xs[i])


def test_oracle_plan_refuses_what_it_does_not_restate():
    base = bench.instance_text(60, 40, 0.05, 0.5, False)
    with pytest.raises(ValueError):
        OraclePlan(base.replace("gradients : 1", "gradients : 2"))
    with pytest.raises(ValueError):
        OraclePlan(base.replace("(X)1(A)39", "@dend(A,(A)3,2)"))
