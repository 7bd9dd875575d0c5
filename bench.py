"""Benchmark: ms per smoothest-field + seamless-integration + IGM-rounding solve.

Workload (default): icosphere level 8 (655,362 vertices / 1,310,720 faces), radius
1 + sum_{l=1..8} a_lm Y_lm with a_lm ~ N(0, 0.05/l) (seed 0), grid ratio 0.01, N = 4, Curl
matching, seamless, no local injectivity, roundSeams = false -- the "1.3M faces" size of the
metric.  Synthetic seeded input (no dataset exists for this path).

One step = one call of the C-ABI pipeline (mtk_pipeline_run) from host buffers: Hmesh, field,
matching, seams, cut, combing, setup and integ.  Reported:
  value  device milliseconds of the solver stages (field + naive/LM integration + rounding
         loop, CUDA events inside the library), mixed precision, median over the K steps
  e2e    wall milliseconds of the whole call with host buffers in and out (H2D/D2H inside)
  fp64   the same device stages with the plain FP64 GPU path (median over K steps after the
         timed region)
The L2 is flushed (256 MiB write) before every step.

--impl reference: the FP64 CPU oracle (the reference algorithm restated with direct sparse
solves: one factorisation of L + 50 inverse-iteration solves, LU of the naive KKT system, one
SPD factorisation per LM iteration), single-threaded on the host.  The full 1.3M-face path takes
a quarter of an hour there, so each step runs the whole path on a seeded sample of the same
family (the level-5 sphere, 20,480 faces) and the value is extrapolated to the workload's face
count by the growth exponent fitted in the same run over a ladder of sizes (levels 3, 4, 5); the
line says so (cpu_baseline.value_kind).  The GPU arm reports its own times on the sample mesh
too, so one ratio is measured on the same configuration.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "ms per field+seamless+IGM solve @1.3M faces, mixed vs FP64 GPU at 1e-8 residual"
WORKLOAD_DESC = ("icosphere level 8 (655362 V / 1310720 F), SH degree-8 radial displacement "
                 "a_lm~N(0,0.05/l) seed 0, ratio 0.01, N=4, Curl matching, seamless, roundSeams=false")


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def replica_job(dev_ms, walls, t_total, steps, world, device=None):
    """Whole-job times of N independent replicas (one process per GPU, no collective on the data
    path): every rank solves its own workload once per step and the job lasts as long as its
    slowest rank, so each figure is the maximum over ranks; `value` and `e2e` are that maximum
    divided by the solves all ranks made in one step (N), `ms_per_step` the slowest rank's step.
    Works with any torch.distributed backend (NCCL with a CUDA `device`, gloo on the CPU)."""
    import torch

    t = torch.tensor([statistics.median(dev_ms), statistics.median(walls), t_total / steps],
                     dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dev_max, wall_max, step_max = t.tolist()
    return {"value": dev_max / world, "e2e": wall_max / world, "ms_per_step": step_max,
            "slowest_rank_ms": dev_max, "slowest_rank_e2e_ms": wall_max}


def rank_sum(x, world, device=None):
    """Sum of an integer over ranks (kernel launches of the whole job)."""
    if world <= 1:
        return int(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([int(x)], dtype=torch.int64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return int(t.item())


def flush_l2(buf):
    buf.add_(1.0)


# ncu --set full captures at 1.3M faces (ico8_sh8): DRAM read + write per pass of the FP32 inner
# solve (iterations + 1 passes per launch)
NCU_DRAM_PER_PASS = {
    "igm_pcg": {"bytes": 35.91e9 / 79, "source": "igm_pcg<float>, one 78-iteration launch: 35.91 GB DRAM "
                                                 "in 14.87 ms (profiles/igm_pcg_f32_ico8_sh8.md)"},
    "field_pcg": {"bytes": 12.49e9 / 33, "source": "pcg_complex_mg<float>, one 32-iteration launch: 12.49 GB "
                                                   "DRAM in 6.12 ms (profiles/pcg_complex_mg_f32_ico8_sh8.md)"},
}


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def run_ours(args):
    import torch

    import metriko_gb300 as M
    from metriko_gb300 import meshgen

    rank, world = env_rank()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dev = torch.cuda.current_device()
    V, F, ratio, rs = meshgen.workload(args.workload, seed=rank)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    ctx = M.Context(dev)
    opts_mixed = M.solve_opts("mixed", tol=args.tol)
    opts_fp64 = M.solve_opts("fp64", tol=args.tol)

    def step(opts, mesh=None):
        Vs, Fs, rat, rsm = mesh or (V, F, ratio, rs)
        flush_l2(flush)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = M.pipeline(ctx, Vs, Fs, ratio=rat, round_seams=rsm, opts=opts)
        wall = (time.perf_counter() - t0) * 1e3
        if r["status"] != 0:
            raise RuntimeError(f"pipeline status {r['status']}")
        st = r["stats"]
        return r, st, wall

    for _ in range(args.warmup):
        step(opts_mixed)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    k0 = ctx.kernel_count()
    sampler = ClockSampler()
    sampler.start()
    dev_ms, walls, stats = [], [], []
    t_start = time.perf_counter()
    for _ in range(args.steps):
        r, st, wall = step(opts_mixed)
        dev_ms.append(st["ms_field"] + st["ms_integrate"] + st["ms_rounding"])
        walls.append(wall)
        stats.append(st)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t_total = (time.perf_counter() - t_start) * 1e3
    clocks = sampler.stop()
    launches = ctx.kernel_count() - k0
    rdev = torch.device("cuda", dev) if world > 1 else None
    job = replica_job(dev_ms, walls, t_total, args.steps, world, device=rdev)
    launches = rank_sum(launches, world, device=rdev)
    # plain FP64 GPU path, same workload and step count (after the timed region), median
    if args.no_fp64:
        st64, fp64_ms = {"pcg_iters": None}, None
    else:
        runs64 = [step(opts_fp64) for _ in range(args.steps)]
        ms64 = [x[1]["ms_field"] + x[1]["ms_integrate"] + x[1]["ms_rounding"] for x in runs64]
        fp64_ms = statistics.median(ms64)
        st64 = runs64[len(runs64) // 2][1]
    # the same pipeline on the CPU baseline's sample mesh (the top rung of its ladder), so that
    # one GPU/CPU ratio is measured on the same configuration
    same = None
    if not args.no_cpu:
        sm = meshgen.workload(LADDER[-1], seed=rank)
        step(opts_mixed, sm)
        runs_s = [step(opts_mixed, sm) for _ in range(max(3, min(args.steps, 5)))]
        same = {"workload": LADDER[-1], "faces": len(sm[1]),
                "value": round(statistics.median([x[1]["ms_field"] + x[1]["ms_integrate"] + x[1]["ms_rounding"]
                                                  for x in runs_s]), 3),
                "e2e": round(statistics.median([x[2] for x in runs_s]), 3), "unit": "ms", "steps": len(runs_s)}
    # stand-alone SpMV of the field operator (after the timed region): FP32 and FP64, each SpMV
    # after an L2 flush, CUDA events around the kernel alone
    spmv = None
    if not args.no_spmv:
        pk, pk_kind = load_peaks()

        def spmv_entry(Vs, Fs, kernel):
            nbr, theta, _ = M.field_inputs(Vs, Fs)
            ms32, by32, cp32 = M.spmv_bench(ctx, nbr, theta, "mixed", reps=20)
            ms64, by64, cp64 = M.spmv_bench(ctx, nbr, theta, "fp64", reps=20)
            gbs32, gbs64 = by32 / (ms32 * 1e-3) / 1e9, by64 / (ms64 * 1e-3) / 1e9
            return {"kernel": kernel, "faces": len(Fs), "bytes_per_spmv": int(by32), "ms": round(ms32, 4),
                    "achieved": round(gbs32, 1), "peak": pk, "unit": "GB/s", "frac": round(gbs32 / pk, 4),
                    "peak_kind": pk_kind,
                    "copy_same_bytes_gbs": round(by32 / (cp32 * 1e-3) / 1e9, 1),
                    "frac_of_same_size_copy": round(cp32 / ms32, 4),
                    "fp64": {"bytes_per_spmv": int(by64), "ms": round(ms64, 4), "achieved": round(gbs64, 1),
                             "frac": round(gbs64 / pk, 4), "frac_of_same_size_copy": round(cp64 / ms64, 4)}}

        spmv = spmv_entry(V, F, "spmv_ell<float>")
        # the same kernel on a level-9 icosphere (5,242,880 faces): large enough to amortise launch
        V9, F9 = meshgen.icosphere(9)
        spmv["level9"] = spmv_entry(V9, F9, "spmv_ell<float>")
        spmv["l2"] = "flushed (256 MiB write) before every SpMV and every copy"
        spmv["reps"] = 20
    value = job["value"]
    st = stats[len(stats) // 2]
    peak, peak_kind = load_peaks()
    dominant = "igm_pcg" if st.get("igm_pcg_ms", 0) >= st.get("field_pcg_ms", 0) else "field_pcg"
    d_ms = st.get(f"{dominant}_ms", 0.0)
    d_bytes = st.get(f"{dominant}_bytes", 0.0)
    d_launch = max(1, st.get(f"{dominant}_launches", 1))
    d_passes = st.get(f"{dominant}_passes", 0)
    achieved = (d_bytes / d_launch) / (d_ms / d_launch * 1e-3) / 1e9 if d_ms > 0 else None
    # DRAM bytes per pass (one PCG iteration or the start pass) of one ncu --set full capture of
    # the kernel at 1.3M faces (dram__bytes_read.sum + dram__bytes_write.sum over iterations + 1),
    # scaled to this run's average launch; measured on the FP32 inner solves
    ncu_pass = NCU_DRAM_PER_PASS.get(dominant) if args.workload == "ico8_sh8" else None
    traffic = ncu_pass["bytes"] * d_passes / d_launch if (ncu_pass and d_passes) else None
    nV, nF = len(V), len(F)
    h2d = world * (V.nbytes + F.nbytes)      # every rank copies a mesh of the same size
    d2h = world * (r["cfn"].nbytes + r["fullx"].nbytes + r["singular"].nbytes + r["compressed"].nbytes)
    cpu = cpu_baseline(args) if (rank == 0 and not args.no_cpu) else None
    if same is not None and cpu is not None:
        same["cpu_ms"] = cpu["measured"]["ms"]
        same["cpu_over_gpu_e2e"] = round(cpu["measured"]["ms"] / same["e2e"], 2)
        same["cpu_over_gpu_value"] = round(cpu["measured"]["ms"] / same["value"], 2)
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "ms", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(job["ms_per_step"], 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 (mixed: FP32 PCG, FP64 refinement)",
        "data": "synthetic (seeded mesh generator)",
        "config": {"workload": args.workload, "description": WORKLOAD_DESC if args.workload == "ico8_sh8" else args.workload,
                   "faces": nF, "vertices": nV, "tol": args.tol, "parallelism": "replicas" if world > 1 else "single",
                   "l2": "flushed (256 MiB write) before every step",
                   "aggregation": ("median over steps of each rank; slowest rank / N (one solve per rank "
                                   "per step, replicas on their own seeded meshes)") if world > 1 else
                                  "median over steps"},
        "e2e": {"value": round(job["e2e"], 3), "unit": "ms", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "fp64_gpu_ms": round(fp64_ms, 3) if fp64_ms else None,
        "fp64_gpu_steps": None if args.no_fp64 else args.steps,
        "mixed_vs_fp64_speedup": (round(fp64_ms / statistics.median(dev_ms), 3)     # this rank's own runs
                                  if (fp64_ms and statistics.median(dev_ms) > 0) else None),
        "stages_ms": {"field": round(st["ms_field"], 3), "integrate": round(st["ms_integrate"], 3),
                      "rounding": round(st["ms_rounding"], 3), "host": round(st["ms_host"], 3)},
        "solver": {"pcg_iters": st["pcg_iters"], "solves": st["solves"], "resolves": st["resolves"],
                   "max_rel_residual": st["max_rel_residual"], "fp64_pcg_iters": st64["pcg_iters"]},
        "rounding_order": {"min_order_margin": st.get("min_order_margin"),
                           "strict_order_differs": st.get("strict_order_differs"),
                           "strict_order_gap": st.get("strict_order_gap"),
                           "note": ("greedy picks tied within 1e-8 are taken by position; strict_order_differs "
                                    "counts the steps whose pick is not the strict '<' pick, strict_order_gap the "
                                    "largest distance gap between the two")},
        "same_config": same,
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": round(achieved, 1) if achieved else None,
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4) if achieved else None,
                     "peak_kind": peak_kind,
                     "bytes_per_launch": round(d_bytes / d_launch, 1),
                     "traffic": round(traffic, 1) if traffic else None,
                     "traffic_source": ncu_pass["source"] if ncu_pass else None},
        "spmv": spmv,
        "clocks": clocks,
        "cpu_baseline": cpu,
    }
    if world > 1:
        line["replicas"] = {"slowest_rank_ms": round(job["slowest_rank_ms"], 3),
                            "slowest_rank_e2e_ms": round(job["slowest_rank_e2e_ms"], 3)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


LADDER = ["ico3_sh8", "ico4_sh8", "ico5_sh8"]   # CPU sample sizes: 1,280 / 5,120 / 20,480 faces


def cpu_info():
    """Host CPU model and core count (lscpu, else /proc/cpuinfo)."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if model is None:
        try:
            for line in Path("/proc/cpuinfo").read_text().splitlines():
                if line.lower().startswith(("model name", "cpu model")):
                    model = line.split(":", 1)[1].strip()
                    break
        except Exception:
            pass
    return {"cpu_model": model, "host_cores": os.cpu_count()}


def time_oracle(name):
    """The whole oracle path on one seeded workload, single-threaded: (ms, faces, re-solves,
    factorisations)."""
    from metriko_gb300 import meshgen
    from oracle import metriko_oracle as O

    V, F, ratio, rs = meshgen.workload(name)
    t0 = time.perf_counter()
    out = O.pipeline(V, F, ratio=ratio, round_seams=rs)
    ms = (time.perf_counter() - t0) * 1e3
    return ms, len(F), out["info"].get("resolves"), out["stats"].get("factorizations")


def fit_growth(points):
    """Least-squares fit of log(ms) = a + b log(faces): (b, rms of the log residuals)."""
    x = np.log([p[0] for p in points])
    y = np.log([p[1] for p in points])
    b, a = np.polyfit(x, y, 1)
    rms = float(np.sqrt(np.mean((y - (a + b * x)) ** 2)))
    return float(b), rms


def extrapolation(points, faces_target):
    """(ms at faces_target, exponent, rms): the largest measured point scaled by the fitted
    growth exponent."""
    b, rms = fit_growth(points)
    f_top, t_top = max(points)
    return t_top * (faces_target / f_top) ** b, b, rms


def workload_faces(name):
    from metriko_gb300 import meshgen
    return len(meshgen.workload(name)[1])


def cpu_baseline(args):
    """FP64 CPU oracle (the reference algorithm with direct sparse solves) timed on a bounded
    sample: the whole path once on each rung of LADDER, single-threaded; the value is the top
    rung's time extrapolated to the workload's face count by the exponent fitted over the
    ladder (labelled value_kind "extrapolated"); the top rung's measured time is the
    same-configuration number (`measured`)."""
    ladder = []
    for name in LADDER:
        ms, nf, rsv, fac = time_oracle(name)
        ladder.append({"workload": name, "faces": nf, "ms": round(ms, 1), "resolves": rsv, "factorizations": fac})
    nFw = workload_faces(args.workload)
    v, b, rms = extrapolation([(r["faces"], r["ms"]) for r in ladder], nFw)
    top = ladder[-1]
    return {"value": round(v, 1), "unit": "ms", "cores": 1, "kind": "port", "value_kind": "extrapolated",
            "sample": (f"whole oracle path (field: one SPD factorisation + 50 solves; naive KKT LU; one SPD "
                       f"factorisation per LM iteration) single-threaded on {', '.join(LADDER)}; "
                       f"{top['workload']} ({top['faces']} faces) = {top['ms']:.0f} ms measured, extrapolated to "
                       f"{nFw} faces by the fitted exponent {b:.3f}"),
            "exponent": round(b, 4), "fit_rms_log": round(rms, 4), "ladder": ladder,
            "measured": {"workload": top["workload"], "faces": top["faces"], "ms": top["ms"]}, **cpu_info()}


def run_reference(args):
    """The reference arm: every step runs the whole oracle path on the sample mesh (the top rung
    of LADDER); the lower rungs run once before the timed steps (with the warm-up) to fit the
    growth exponent, which the steps' median also enters."""
    rank, world = env_rank()
    if rank != 0:
        return
    for _ in range(max(0, min(args.warmup, 2))):
        time_oracle(LADDER[0])
    low = [time_oracle(name) for name in LADDER[:-1]]
    steps = [time_oracle(LADDER[-1]) for _ in range(max(1, args.steps))]
    t_med = statistics.median([s[0] for s in steps])
    pts = [(f, ms) for ms, f, _, _ in low] + [(steps[0][1], t_med)]
    nFw = workload_faces(args.workload)
    v, b, rms = extrapolation(pts, nFw)
    v = round(v, 1)
    cpu = {"value": v, "unit": "ms", "cores": 1, "kind": "port", "value_kind": "extrapolated",
           "sample": (f"whole oracle path single-threaded on {LADDER[-1]} ({steps[0][1]} faces) every step, median "
                      f"{t_med:.0f} ms; extrapolated to {nFw} faces by the exponent {b:.3f} fitted over "
                      f"{', '.join(LADDER)} (rms of log residuals {rms:.3f})"),
           "exponent": round(b, 4), "fit_rms_log": round(rms, 4),
           "ladder": [{"faces": f, "ms": round(ms, 1)} for f, ms in pts],
           "measured": {"workload": LADDER[-1], "faces": steps[0][1], "ms": round(t_med, 1),
                        "resolves": steps[0][2], "factorizations": steps[0][3]}, **cpu_info()}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "ms", "n_gpus": world,
            "steps": len(steps), "warmup": args.warmup, "higher_is_better": False, "dtype": "f64",
            "data": "synthetic (seeded mesh generator)", "vs_baseline": None,
            "config": {"workload": args.workload, "sample_workload": LADDER[-1]},
            "cpu_baseline": cpu,
            "e2e": {"value": v, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ico8_sh8")
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 GPU comparison run (profiling runs)")
    ap.add_argument("--no-spmv", action="store_true", help="skip the stand-alone SpMV measurement (profiling runs)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
