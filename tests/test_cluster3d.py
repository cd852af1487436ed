"""Cluster-resident FP32 sweeps of small 3-D boxes (NM_OPT_CLUSTER3D): one
thread-block cluster holds the box's propagators in distributed shared
memory and runs a whole sweep per launch.  Against one launch per step:
the same residual bit for bit (periodic and mirror bounds, boxes
whose x extent does not divide into the cluster, several blocks of a
linear chain, the melt fixture of the reference), and the same solve; and
far fewer launches per residual."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import bench  # noqa: E402
from namics_gb300 import NM_FP32, Context, NamicsError, Plan, _abi  # noqa: E402


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def _resid(ctx, x):
    xd = _dev(x)
    g = torch.zeros_like(xd)
    n0 = ctx.launch_count()
    ctx.residual_dev(xd.data_ptr(), g.data_ptr())
    torch.cuda.synchronize()
    return g.cpu().numpy(), ctx.launch_count() - n0


def _texts():
    melt = bench.melt3d_text(24, 12)
    return [
        ("periodic 24^3", melt),
        ("mirror 21^3", bench.melt3d_text(21, 12).replace("periodic", "mirror")),
        ("64^3 A20B20", bench.melt3d_small_text()),
        ("x 19 mirror, y z periodic", bench.melt3d_text(19, 12)
         .replace("lowerbound_x : periodic", "lowerbound_x : mirror")
         .replace("upperbound_x : periodic", "upperbound_x : mirror")),
        ("three blocks", melt.replace("(A)50(B)50", "(A)10(B)20(A)15")),
    ]


def _field(plan, seed):
    u = np.random.default_rng(seed).uniform(-0.1, 0.1, plan.M)
    return np.concatenate([u, -u]) if plan.iv == 2 * plan.M else np.resize(u, plan.iv)


@pytest.mark.parametrize("label,text", _texts(), ids=[t[0] for t in _texts()])
def test_cluster_sweeps_bit_identical(label, text):
    plan = Plan(text)
    x = _field(plan, 11)
    on = Context(plan, NM_FP32)
    on.set_option(_abi.NM_OPT_CLUSTER3D, 1)
    off = Context(plan, NM_FP32)
    g_on, n_on = _resid(on, x)
    g_off, n_off = _resid(off, x)
    assert np.all(np.isfinite(g_on))
    assert np.array_equal(g_on, g_off), (label, np.max(np.abs(g_on - g_off)))
    assert n_on * 4 < n_off, (n_on, n_off)  # one launch per sweep instead of one per step
    for which in (0, 1, 2):
        assert np.array_equal(on.field(which), off.field(which)), which
    F1, O1, _ = on.free_energy()
    F2, O2, _ = off.free_energy()
    assert (F1, O1) == (F2, O2)


def test_cluster_solve_and_reference_fixture():
    run = load_golden("melt3d")["runs"]["it0"]
    plan = Plan(run["input"])
    x0 = np.array(run["x"])
    on, off = Context(plan, NM_FP32), Context(plan, NM_FP32)
    on.set_option(_abi.NM_OPT_CLUSTER3D, 1)
    assert np.array_equal(_resid(on, x0)[0], _resid(off, x0)[0])
    big = Plan(bench.melt3d_text(24, 30))
    x = _field(big, 5)
    on, off = Context(big, NM_FP32), Context(big, NM_FP32)
    on.set_option(_abi.NM_OPT_CLUSTER3D, 1)
    x1, x2 = x.copy(), x.copy()
    r1, _ = on.solve_host(x1)
    r2, _ = off.solve_host(x2)
    assert (r1.iterations, r1.residual, r1.status) == (r2.iterations, r2.residual, r2.status)
    assert np.array_equal(x1, x2)


def test_cluster_option_refused_where_it_does_not_apply():
    # a checkpointed context keeps the per-step kernels; a box too large for
    # a cluster's shared memory has no cluster sweep to turn on
    plan = Plan(bench.melt3d_text(24, 12))
    c = Context(plan, NM_FP32, checkpoint_stride=5)
    c.set_option(_abi.NM_OPT_CLUSTER3D, 1)  # selected, but the stride keeps the per-step kernels
    g_ck, n_ck = _resid(c, _field(plan, 2))
    ref = Context(plan, NM_FP32)
    ref.set_option(_abi.NM_OPT_CLUSTER3D, 1)
    g_ref, n_ref = _resid(ref, _field(plan, 2))
    assert np.array_equal(g_ref, g_ck) and n_ref * 4 < n_ck
    big = Plan(bench.melt3d_text(128, 2))
    c = Context(big, NM_FP32)
    with pytest.raises(NamicsError):
        c.set_option(_abi.NM_OPT_CLUSTER3D, 1)
    c.set_option(_abi.NM_OPT_CLUSTER3D, 0)
