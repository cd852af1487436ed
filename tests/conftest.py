import json
import os
import sys
from pathlib import Path

# more hardware work queues than streams, so no stream waits behind the
# persistent work loop's queue (read when the CUDA context is created)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def golden_names():
    """The per-case fixtures (raw_outputs.json, the reference's output files
    verbatim, is read by test_outputs.py only; key_checks.json, the input keys
    the reference accepts, by test_input_keys.py; search_*.json, the
    reference's searches, and scan_*.json, its scans, by test_search.py)."""
    return sorted(p.stem for p in GOLDEN.glob("*.json")
                  if p.stem not in ("raw_outputs", "key_checks") and not p.stem.startswith(("search_", "scan_")))


def load_golden(name):
    return json.loads((GOLDEN / f"{name}.json").read_text())


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    """Build the product library and the oracle once per session (both are
    needed on CPU too: the plan compiler and the oracle run without a GPU)."""
    from namics_gb300 import build
    build.build_product()
    build.build_oracle()
    return True
