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


def test_headline_line_keeps_its_comparisons_last():
    """The headline line puts its bulky per-level diagnostics first and the
    comparisons (V-cycle, level-0 SpMV, siblings, learned gain, speed-ups,
    roofline, CPU baseline, e2e) last, in a fixed order, so a log that keeps
    only the end of a long line still shows them; every key survives."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    line = {"metric": "m", "value": 1.0, "roofline": {"frac": 0.4}, "ops": [[0, "A"]] * 200,
            "fp64_batched": {"value": 2.0, "colour_cap_tuning": [{"caps": [8, 1]}]}, "e2e": {"value": 1.1},
            "plain": {"sweep_levels": [[0, 1, 2, 3]] * 50}, "cpu_baseline": {"value": 9.0}, "vcycle_ms": 0.5}
    out = bench.tail_last(line)
    keys = list(out)
    tail = [k for k in bench.TAIL_KEYS if k in line]
    assert keys[-len(tail):] == tail
    assert set(keys) == set(line) | {"fp64_batched_colour_cap_tuning"}
    assert "colour_cap_tuning" not in out["fp64_batched"] and "colour_cap_tuning" in line["fp64_batched"]
    s = json.dumps(out)
    assert '"e2e"' in s[-200:] and '"cpu_baseline"' in s[-200:]
