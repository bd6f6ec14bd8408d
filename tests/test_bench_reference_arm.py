"""The reference arm of bench.py on CPU: it builds the GPU arm's workload with the
oracle, reports the GPU arm's config object, and never loads the GPU library."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]

_PROBE = r"""
import json, sys
sys.argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3", "--workload", "batch4096"]
import bench
bench.main()
mapped = sorted({l.split()[-1] for l in open("/proc/self/maps") if "libopencloth" in l})
print(json.dumps({"product_imported": "opencloth_gb300" in sys.modules, "mapped": mapped}))
"""


def test_reference_arm_is_isolated_and_reports_the_same_config():
    r = subprocess.run([sys.executable, "-c", _PROBE], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(x) for x in r.stdout.strip().splitlines()]
    line, probe = lines[0], lines[-1]
    assert probe == {"product_imported": False, "mapped": []}
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["value"] == line["value"]

    import bench

    specs, _, _, _ = bench.batch4096(20261203)
    assert line["config"] == bench.workload_config("batch4096", specs, 1)


def test_reference_arm_refuses_the_coupled_mode(capsys):
    import bench

    bench.run_reference(type("A", (), {"workload": "coupled1025", "steps": 1, "warmup": 3, "gpus": 1})())
    out = json.loads(capsys.readouterr().out)
    assert out["impl"] == "reference" and "unavailable" in out
