"""bench.py's reference arm on the CPU: one JSON line with the contract's keys.

The reference arm times the oracle (the C restatement of the reference's
setup and integer solve) on the host cores, without loading this repository's
library; here on a 16^3 system so that it finishes in a second."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "16",
                          "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["steps"] == 2 and d["warmup"] == 1
    assert d["higher_is_better"] is False and d["value"] > 0
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["explicit_res"] <= 1e-10
    assert "16^3" in d["config"]["workload"]
    assert d["config"]["stop"] == "explicit relative residual"


def test_reference_arm_does_not_load_the_library():
    """The reference arm's process maps the oracle, never libsagb.so."""
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--n', '12', '--steps', '1', "
            "'--warmup', '0']; runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); "
            "print('MAPS', 'liboracle' in maps, 'libsagb' in maps)")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr
    assert "MAPS True False" in out.stdout, out.stdout[-500:]
