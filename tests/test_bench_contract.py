"""bench.py's JSON line on the CPU: the host logic of the default run (one rank) with the library
and CUDA replaced by fakes that return fixed stage times.  Checks the keys and units the line
must carry and how value, e2e, launches and bytes are formed; the numbers themselves come from
the GPU run."""
import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture
def fake_bench(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import torch

    import bench
    import metriko_gb300 as M
    from metriko_gb300 import meshgen

    empty = torch.empty
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **k: None)
    monkeypatch.setattr(torch.cuda, "current_device", lambda: 0)
    monkeypatch.setattr(torch, "empty", lambda *a, device=None, **k: empty(*a, **k))

    class Ctx:
        def __init__(self, dev):
            self.k = 0

        def kernel_count(self):
            self.k += 250
            return self.k

        def close(self):
            pass

    def pipeline(ctx, V, F, ratio=0.02, round_seams=False, opts=None, **kw):
        fp64 = opts is not None and opts.precision == M.PREC_FP64
        st = dict(ms_field=500.0 * (1 + fp64), ms_integrate=150.0 * (1 + fp64), ms_rounding=350.0 * (1 + fp64),
                  ms_host=400.0, pcg_iters=1000, solves=3, resolves=10, max_rel_residual=1e-9,
                  igm_pcg_ms=300.0, igm_pcg_bytes=6e11, igm_pcg_launches=20,
                  field_pcg_ms=200.0, field_pcg_bytes=1e11, field_pcg_launches=100)
        nF = len(F)
        return dict(status=0, stats=st, cfn=np.zeros((nF, 12)), fullx=np.zeros(2 * len(V)),
                    singular=np.zeros(len(V), np.int32), compressed=np.zeros(nF, complex))

    small = meshgen.workload("ico2_noise")
    monkeypatch.setattr(M, "Context", Ctx)
    monkeypatch.setattr(M, "pipeline", pipeline)
    monkeypatch.setattr(M, "spmv_bench", lambda ctx, nbr, theta, prec, reps=20: (0.02, 7.3e7, 0.017))
    monkeypatch.setattr(meshgen, "workload", lambda name, seed=0: small)
    monkeypatch.setattr(meshgen, "icosphere", lambda lvl: small[:2])
    monkeypatch.setattr(bench, "cpu_baseline", lambda args: {"value": 1.0, "unit": "ms", "cores": 1, "kind": "port",
                                                             "sample": "fake", "measured": {"ms": 5000.0}})
    monkeypatch.setenv("RANK", "0")
    monkeypatch.setenv("WORLD_SIZE", "1")
    return bench, small


def test_bench_line_carries_the_contract_keys(fake_bench, capsys):
    bench, (V, F, _, _) = fake_bench

    class A:
        gpus, steps, warmup, impl = 1, 3, 3, "ours"
        workload, tol = "ico8_sh8", 1e-8
        no_cpu = no_fp64 = no_spmv = False

    bench.run_ours(A())
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    for k in ["metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "e2e", "gpu_launches", "roofline", "cpu_baseline", "clocks"]:
        assert k in line, k
    assert line["value"] == 1000.0 and line["unit"] == "ms" and line["higher_is_better"] is False
    assert line["n_gpus"] == 1 and line["steps"] == 3 and line["warmup"] == 3
    assert line["fp64_gpu_ms"] == 2000.0 and line["mixed_vs_fp64_speedup"] == 2.0
    assert line["gpu_launches"] == 250                       # kernel counter across the timed steps
    e2e = line["e2e"]
    assert e2e["unit"] == "ms" and e2e["h2d_bytes_per_step"] == V.nbytes + F.nbytes
    assert e2e["d2h_bytes_per_step"] == len(F) * 12 * 8 + 2 * len(V) * 8 + len(V) * 4 + len(F) * 16
    r = line["roofline"]
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["kernel"] == "igm_pcg"
    assert r["achieved"] == pytest.approx(6e11 / 0.3 / 1e9, rel=1e-6)   # bytes / event time
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"], rel=1e-3)
    assert line["spmv"]["level9"]["kernel"] == "spmv_ell<float>"
    assert "l2" in line["config"] and line["config"]["workload"] == "ico8_sh8"
    same = line["same_config"]          # the GPU on the CPU baseline's sample mesh
    assert same["workload"] == bench.LADDER[-1] and same["value"] == 1000.0
    assert same["cpu_ms"] == 5000.0 and same["cpu_over_gpu_value"] == 5.0
    assert line["fp64_gpu_steps"] == 3


def test_growth_fit_and_extrapolation():
    sys.path.insert(0, str(ROOT))
    import bench
    pts = [(1280, 2.0 * 1280 ** 1.3), (5120, 2.0 * 5120 ** 1.3), (20480, 2.0 * 20480 ** 1.3)]
    b, rms = bench.fit_growth(pts)
    assert b == pytest.approx(1.3, abs=1e-9) and rms < 1e-9
    v, b2, _ = bench.extrapolation(pts, 1310720)
    assert v == pytest.approx(2.0 * 1310720 ** 1.3, rel=1e-9) and b2 == pytest.approx(1.3)
