"""bench.py's accounting helpers and the reference arm's JSON line (CPU only)."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


@pytest.mark.parametrize("n,flops", [(8, 1288), (16, 10640), (24, 36248), (32, 86304),
                                     (48, 292528), (64, 694848)])
def test_algorithmic_flops_per_matrix(n, flops):
    assert bench.flops_per_matrix(n) == flops


def test_bytes_and_launch_accounting():
    assert bench.bytes_per_matrix(24) == 16 * 24 * 24 + 21
    # 32 MiB chunks of 24 x 24 complex128 matrices: 3640 per chunk
    assert bench.host_chunks(24, 24, 32768) == 10
    assert bench.host_chunks(8, 8, 1) == 1
    assert [bench.mixed_launches_per_call(n) for n in (8, 16, 24, 32, 48)] == [1, 1, 2, 2, 1]
    assert bench.host_launches_per_call(24, 24, 32768, 2, True) == 1
    assert bench.host_launches_per_call(24, 24, 32768, 2, False) == 20
    assert bench.host_launches_per_call(24, 24, 32768, 1, True) == 10
    # the FP32 lane operations of the mixed method grow like n^3 and are dominated by the residual
    ops24 = bench.mixed_fp32_ops_per_matrix(24)
    assert 38 * sum(min(i, k) + 1 for i in range(24) for k in range(24)) < ops24 < 2e6


def test_reference_arm_json_line():
    proc = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "2",
                           "--warmup", "3"], cwd=ROOT, capture_output=True, text=True,
                          timeout=600)
    assert proc.returncode == 0, proc.stderr[-2000:]
    line = json.loads(proc.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for k in ("metric", "value", "unit", "steps", "warmup", "ms_per_step", "higher_is_better",
              "cpu_baseline", "e2e", "config"):
        assert k in line, k
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["cores"] >= 1


def test_reference_arm_loads_no_product_code():
    """The reference arm builds its inputs with the oracle's generators: the
    product library must not be mapped into that process, and its config object
    is the GPU arm's (bench.workload_config)."""
    code = (
        "import sys, json, io, contextlib; sys.argv = ['bench.py', '--impl', 'reference', "
        "'--steps', '1', '--warmup', '3', '--ref-sample', '512']\n"
        "import bench\n"
        "buf = io.StringIO()\n"
        "with contextlib.redirect_stdout(buf):\n"
        "    bench.main()\n"
        "maps = open('/proc/self/maps').read()\n"
        "print(json.dumps({'line': json.loads(buf.getvalue().strip().splitlines()[-1]), "
        "'loaded': 'liblufqhe.so' in maps}))\n")
    proc = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True,
                          timeout=600)
    assert proc.returncode == 0, proc.stderr[-2000:]
    res = json.loads(proc.stdout.strip().splitlines()[-1])
    assert res["loaded"] is False
    assert res["line"]["config"] == bench.workload_config("lll24", 1)
