"""Input keys the plan compiler does not read, against the reference.

tests/golden/key_checks.json (make_golden.py --keys) records whether the
reference runs a brush input with one extra line added; it refuses keys
outside each class's list (Input::CheckParameters, input.cpp:366-431).

- A line the reference refuses is refused here too (NM_ERR_INPUT).
- A line the reference accepts and that cannot change a DIIS solve of this
  path (verbosity, the storage schedule, the GPU switch, the parameters of
  other Newton methods) is accepted, and the plan is the one without it.
- A line the reference accepts for a feature outside this path
  (restricted ranges, overflow protection) is refused by name rather than
  dropped, so no input runs with part of it silently ignored.
"""
import json
from pathlib import Path

import pytest

from namics_gb300 import NamicsError, Plan, _abi

KEYS = json.loads((Path(__file__).resolve().parent / "golden" / "key_checks.json").read_text())
NO_EFFECT = {"save_memory", "s_info", "e_info", "deltamin", "GPU", "calculation_type"}


def _summary(p: Plan):
    c = p.c
    return (p.iv, p.n_seg, p.n_mol, c.MX, c.gradients, c.tolerance, c.iterationlimit, c.diis_m, c.deltamax)


@pytest.mark.parametrize("case", KEYS["cases"], ids=lambda c: c["line"])
def test_unread_keys_follow_the_reference(case):
    key = case["line"].split(":")[2].strip()
    text = KEYS["base"] + case["line"] + "\n"
    if case["reference"] == "accepted" and key in NO_EFFECT:
        assert _summary(Plan(text)) == _summary(Plan(KEYS["base"]))
        return
    with pytest.raises(NamicsError) as ei:
        Plan(text)
    assert ei.value.code == _abi.NM_ERR_INPUT
    if case["reference"] == "accepted":  # a feature outside this path: named in the message
        assert key in str(ei.value)
