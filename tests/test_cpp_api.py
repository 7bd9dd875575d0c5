"""The header-only C++ host API compiles and runs as a reference caller uses it
(tests/cpp/api_drop_in.cpp: the example_igm.cpp sequence up to RosyParameterization::setup(),
and the element handles / iterators), with the same results as the C ABI."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import metriko_gb300 as M
from metriko_gb300 import meshgen
from oracle import metriko_oracle as O

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def drop_in(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not found")
    M.lib()                                   # builds / loads the library the program links
    lib = ROOT / "metriko_gb300" / "libmetriko_cuda.so"
    exe = tmp_path_factory.mktemp("cpp") / "api_drop_in"
    cuda_inc = Path(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc").resolve().parent.parent / "include"
    cmd = ["g++", "-O1", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-I", str(ROOT / "include"),
           "-I", str(cuda_inc), str(ROOT / "tests" / "cpp" / "api_drop_in.cpp"), "-o", str(exe), str(lib),
           "-Wl,-rpath," + str(lib.parent)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


@pytest.mark.parametrize("name", ["ico3_noise", "torus_32x16", "genus2_s3"])
def test_reference_style_caller(drop_in, tmp_path, name):
    V, F, ratio, rs = meshgen.workload(name)
    ref = O.pipeline(V, F, ratio=0.03, stop_after="field")
    comp = np.asarray(ref["compressed"], complex)
    blob = tmp_path / "in.bin"
    with open(blob, "wb") as fh:
        fh.write(np.array([len(V), len(F)], np.int32).tobytes())
        fh.write(np.ascontiguousarray(V, np.float64).tobytes())
        fh.write(np.ascontiguousarray(F, np.int32).tobytes())
        fh.write(np.stack([comp.real, comp.imag], 1).astype(np.float64).tobytes())
    r = subprocess.run([str(drop_in), str(blob)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    out = {k: float(v) for k, v in (line.split() for line in r.stdout.split("\n") if line)}
    res = M.topology_from_field(V, F, comp, 0.03, False)
    c = res["counts"]
    assert out["nV"] == c["nV"] and out["nE"] == c["nE"] and out["nCut"] == c["nCut"]
    assert out["nT"] == c["nT"] and out["nS"] == c["nS"]
    assert out["singular"] == float(np.sum(np.abs(res["singular"]) * (np.arange(len(V)) + 1)))
    assert out["seam"] == float(res["seam"].sum())
    assert out["matching"] == float(np.sum(res["matching"] * (np.arange(c["nE"]) % 97 + 1)))
    assert out["loops"] == 3 * len(F) and out["rings"] == 2 * c["nE"] and out["bad"] == 0
    assert abs(out["area_minus_bary"]) < 1e-9
