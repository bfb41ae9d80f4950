"""The benchmark's reference arm on CPU: at a small scale it runs the oracle
port alone -- its graph comes from the oracle's generator, so the product
library is never loaded into that process -- and prints the GPU arm's
config, metric and unit."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DRIVER = r"""
import json, runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--scale", "10", "--steps", "1", "--warmup", "3"]
try:
    runpy.run_path("bench.py", run_name="__main__")
except SystemExit as e:
    assert not e.code, e.code
maps = open("/proc/self/maps").read()
print(json.dumps({"librg_loaded": "librg.so" in maps, "oracle_loaded": "liboracle.so" in maps}))
"""


def test_reference_arm_runs_without_the_product_library():
    env = dict(os.environ)
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        env.pop(k, None)
    r = subprocess.run([sys.executable, "-c", DRIVER], cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    line, maps = lines[0], lines[-1]
    assert maps == {"librg_loaded": False, "oracle_loaded": True}
    sys.path.insert(0, ROOT)
    import bench
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == "GTEPS"
    assert line["config"] == bench.bench_config(10, line["config"]["n"], line["config"]["m"])
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    assert "nproc" in line["cpu_baseline"]["host"]
