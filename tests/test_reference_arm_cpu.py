"""bench.py's reference arm times the oracle only: run in a fresh process, it
must print the same config as the GPU arm's and never map the product's
native library (its clip comes from the content cache and the oracle's own
container parser)."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_loads_no_product_library():
    sys.path.insert(0, str(ROOT))
    from govid_gb300 import workloads

    if not workloads.single_1080().path().exists():
        pytest.skip("the 1080p clip is not in the content cache (encoding it takes minutes)")
    code = (
        "import sys, json; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3'];"
        "sys.path.insert(0, %r); import bench; bench.main();"
        "maps = open('/proc/self/maps').read();"
        "print(json.dumps({'maps_product': 'libebivgpu' in maps}))" % str(ROOT)
    )
    out = subprocess.run([sys.executable, "-c", code], cwd=str(ROOT), capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [json.loads(x) for x in out.stdout.strip().splitlines() if x.startswith("{")]
    line, probe = lines[0], lines[-1]
    assert line["impl"] == "reference" and line["cpu_baseline"]["kind"] == "port"
    assert line["config"]["frames_per_step"] == 300 and "1920x1080" in line["config"]["workload"]
    assert probe == {"maps_product": False}
