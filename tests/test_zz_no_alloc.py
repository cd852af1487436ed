"""nm_solve1d_noalloc: the allocation-free single-problem solve.

Called through the C ABI and compared with the batched entry point
(nm_batch_solve_dev on a batch of one) on two consecutive calls with
different problems, so the second call runs over scratch the first one
left behind.  Kept in the last-collected file so it also runs after every
other GPU test has used the device.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from namics_gb300 import NM_FP32, NM_FP64, Batch, Plan, _abi  # noqa: E402


def _one_gradient_cases():
    """(M, run) of every golden 1-gradient case with a converged run."""
    out = []
    for n in golden_names():
        runs = load_golden(n)["runs"]
        if "conv" in runs:
            plan = Plan(runs["conv"]["input"])  # keep alive while reading it
            markov2 = any(plan.c.mols[m].markov == 2 for m in range(plan.c.n_mol))
            if plan.c.gradients == 1 and not plan.c.charged and not markov2:
                out.append((plan.M, runs["conv"]))
    return out


def _noalloc(plan, x, precision):
    xd = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).cuda()
    r = _abi.nm_solve_result()
    rc = _abi.load().nm_solve1d_noalloc(plan.ptr, C.c_void_p(xd.data_ptr()), precision, None, C.byref(r))
    torch.cuda.synchronize()
    return rc, r, xd.cpu().numpy()


def _batched(plan, x, precision):
    xd = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).cuda()
    its, res, st = Batch([plan], precision).solve_dev(xd.data_ptr())
    torch.cuda.synchronize()
    return int(its[0]), float(res[0]), int(st[0]), xd.cpu().numpy()


@pytest.mark.parametrize("precision", [NM_FP32, NM_FP64])
def test_noalloc_matches_batched_on_consecutive_calls(precision):
    cases = sorted(_one_gradient_cases(), key=lambda c: -c[0])
    # two different problems, largest lattice first, so the second call
    # starts from the first call's leftovers in the shared scratch
    for _, run in (cases[0], cases[-1]):
        plan = Plan(run["input"])
        x0 = np.array(run["x"])
        rc, r, x = _noalloc(plan, x0, precision)
        its, res, st, xb = _batched(plan, x0, precision)
        assert rc == st == r.status
        assert r.iterations == its and r.residual == res
        assert np.array_equal(x, xb)
        assert st == 0 and res < 1e-7


def test_noalloc_rejects_problem_beyond_scratch():
    text = "\n".join([
        "lat : flat : n_layers : 500", "lat : flat : lattice_type : simple_cubic",
        "lat : flat : geometry : planar", "lat : flat : gradients : 1",
        "lat : flat : lowerbound : surface", "lat : flat : upperbound : mirror",
        "mon : S : freedom : frozen", "mon : S : frozen_range : lowerbound",
        "mon : X : freedom : pinned", "mon : X : pinned_range : firstlayer",
        "mon : A : freedom : free", "mon : W : freedom : free",
        "mol : pol : composition : (X)1(A)3999", "mol : pol : freedom : restricted", "mol : pol : n : 0.01",
        "mol : water : composition : (W)1", "mol : water : freedom : solvent",
    ])
    plan = Plan(text)
    rc, r, _ = _noalloc(plan, np.zeros(plan.iv), NM_FP32)
    assert rc == _abi.NM_ERR_INPUT
    assert "static device scratch" in _abi.load().nm_last_error().decode()
