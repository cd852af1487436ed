"""nm_write_pro / nm_write_kal against the reference's own output files.

tests/golden/raw_outputs.json holds the reference's .pro and .kal files
verbatim for the single-residual run of a 1-D, a 2-D cylindrical, a 3-D and a
charged case (make_golden.py --raw).

- CPU: every token of those files is reproduced by the number format the
  writer uses for it (coordinates %e; profiles %.20g in 1-D, %.20e in 2-D and
  3-D; scalars %.16e; integers %i): the format is pinned to the reference.
- GPU: the files a context writes after the same residual have the same
  header, the same number of lines, byte-identical coordinate columns, and
  values within 1e-10 of the reference's.
"""
import json
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
RAW = json.loads((HERE / "golden" / "raw_outputs.json").read_text())


def _rows(text):
    lines = text.rstrip("\n").split("\n")
    return lines[0], [ln.rstrip("\t").split("\t") for ln in lines[1:]]


def _ncoord(header):
    return 3 if header.startswith("x\ty\tz\t") else (2 if header.startswith("x\ty\t") else 1)


@pytest.mark.parametrize("name", sorted(RAW))
def test_reference_number_formats_are_the_writers(name):
    run = RAW[name]
    head, rows = _rows(run["pro_text"])
    nc = _ncoord(head)
    vfmt = "%.20g" if nc == 1 else "%.20e"
    for r in rows:
        for t in r[:nc]:
            assert "%e" % float(t) == t, (name, t)
        for t in r[nc:]:
            assert vfmt % float(t) == t, (name, t)
    khead, (kvals,) = _rows(run["kal_text"])
    for h, t in zip(khead.split("\t"), kvals):
        fmt = "%i" if h.endswith("_iterations") else "%.16e"
        assert fmt % (int(t) if fmt == "%i" else float(t)) == t, (name, h, t)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(RAW))
def test_written_outputs_match_reference_files(name, tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from namics_gb300 import NM_FP64, Context, Plan
    from namics_gb300 import SolveResult
    run = RAW[name]
    plan = Plan(run["input"])
    ctx = Context(plan, NM_FP64)
    x = torch.from_numpy(np.array(run["x"])).cuda()
    g = torch.zeros_like(x)
    ctx.residual_dev(x.data_ptr(), g.data_ptr())
    torch.cuda.synchronize()
    gnorm = float(torch.linalg.norm(g).item())
    strip = lambda items, k: [it.split(":", 1)[1].strip() for it in items if it.startswith(k)]  # noqa: E731
    ctx.write_pro(tmp_path / "out.pro", strip(run["pro_items"], "pro"))
    ctx.write_kal(tmp_path / "out.kal", strip(run["kal_items"], "kal"), SolveResult(0, gnorm, 0))
    ours_h, ours = _rows((tmp_path / "out.pro").read_text())
    ref_h, ref = _rows(run["pro_text"])
    assert ours_h == ref_h
    assert len(ours) == len(ref)
    nc = _ncoord(ref_h)
    assert [r[:nc] for r in ours] == [r[:nc] for r in ref]
    a = np.array([[float(t) for t in r[nc:]] for r in ours])
    b = np.array([[float(t) for t in r[nc:]] for r in ref])
    scale = np.maximum(np.max(np.abs(b), axis=0), 1e-300)
    assert np.all(np.max(np.abs(a - b), axis=0) / scale < 1e-10)
    kh, (kv,) = _rows((tmp_path / "out.kal").read_text())
    rh, (rv,) = _rows(run["kal_text"])
    assert kh == rh
    for h, t, u in zip(kh.split("\t"), kv, rv):
        assert abs(float(t) - float(u)) <= 1e-10 * max(1.0, abs(float(u))), (h, t, u)
