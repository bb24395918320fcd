"""bench.py's JSON line: the reference arm (the oracle's OpenMP restatement on
the host cores, the one arm that runs without a GPU) prints every field of the
contract, with the reference arm's own e2e and cpu_baseline, and never maps
the CUDA library (its workload sample comes from the oracle's generator)."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_prints_the_contract_line():
    env = dict(os.environ, OMP_NUM_THREADS=os.environ.get("OMP_NUM_THREADS", "4"))
    prog = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3']; "
            "runpy.run_path(%r, run_name='__main__'); "
            "print('MAPS', [l.split()[-1] for l in open('/proc/self/maps') if l.rstrip().endswith('.so')])"
            % os.path.join(ROOT, "bench.py"))
    out = subprocess.run([sys.executable, "-c", prog], capture_output=True, text=True, env=env, timeout=600,
                         check=True, cwd=ROOT).stdout
    lines = out.strip().splitlines()
    maps = [l for l in lines if l.startswith("MAPS")][0]
    assert "librvh" not in maps and "liboracle" in maps, maps
    line = json.loads([l for l in lines if l.startswith("{")][-1])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["steps"] == 1 and line["warmup"] >= 3 and line["n_gpus"] == 1
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert "workload" in line["config"]
