"""The C++ host driver builds against include/lufqhe.h and liblufqhe.so alone
(CPU), and runs a few Monte Carlo steps on the GPU."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "lion-codes_gb300" / "host" / "mc_driver.cpp"
LIB = ROOT / "lion-codes_gb300" / "lib"


def build_driver(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    cuda = Path("/usr/local/cuda")
    exe = tmp_path / "mc_driver"
    cmd = [cxx, "-O2", "-std=c++17", str(SRC), "-I", str(ROOT / "include"),
           "-I", str(cuda / "include"), "-L", str(LIB), "-llufqhe",
           f"-Wl,-rpath,{LIB}", "-L", str(cuda / "lib64"), "-lcudart", "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_driver_builds(tmp_path, lufqhe_mod):
    assert build_driver(tmp_path).exists()


@pytest.mark.gpu
def test_driver_runs(tmp_path, cuda, lufqhe_mod):
    exe = build_driver(tmp_path)
    out = subprocess.run([str(exe), "16", "4096", "3", "2"], check=True, capture_output=True,
                         text=True, timeout=120).stdout
    lines = [l for l in out.splitlines() if l.startswith("RESULT")]
    assert len(lines) == 3
    for l in lines:
        vals = l.split()
        assert float(vals[4]) == float(vals[4])  # finite log|psi|
