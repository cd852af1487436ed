"""bench.py's reference arm on CPU: one JSON line with the contract's keys.

`bench.py --impl reference` times the reference path's CPU restatement on the
host's threads, on a bounded sample of the batched 1-D workload per step; its
line carries impl, cpu_baseline (kind, cores, sample) and an e2e object with
no host-device bytes.
"""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "solves/s" and d["value"] > 0
    assert d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 0
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"] and cb["value"] == d["value"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_loads_no_product_library():
    """The reference arm builds its problems with the oracle's own plan
    builder and loads only the oracle library: the product's shared library
    must not be mapped into its process."""
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0'];"
            "runpy.run_path('bench.py', run_name='__main__');"
            "maps = open('/proc/self/maps').read();"
            "print('MAPPED', 'libnamics_gb300' in maps, 'liborc' in maps)")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    flags = [ln for ln in r.stdout.splitlines() if ln.startswith("MAPPED")]
    assert flags == ["MAPPED False True"], r.stdout[-500:]
    d = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][0])
    assert d["config"]["instances_per_step"] == 512 and d["config"]["solves"] == 512
    assert 0 < d["config"]["converged"] <= 512
