"""Generates the golden fixtures of the oracle (tests/golden/*.npz).

The reference (komietty/metriko) cannot be built here and ships no tests or golden data, so
these fixtures pin the FP64 CPU oracle's outputs on seeded meshes; the GPU tests check the CUDA
path against them and the CPU tests check that the oracle still reproduces them.

Small fixtures (ico2_noise, ico3_noise, torus_32x16, genus2_s3, and the open meshes cap3_noise,
cap4_sh8 -- disks -- and cyl_32x12 -- an annulus, seams rounded) store the mesh and every output
in full.  `icosphere_obj` is the reference's own model, example/models/icosphere.obj (a Blender
level-4 icosphere, 2562 vertices / 5120 faces), with the level-4 workload's radial N(0, 0.01)
displacement (seed 0) and grid ratio 0.03; it stores the displaced mesh, so the GPU side needs
no copy of the reference.  The large fixtures (ico5_sh8, ico6_sh8, ico7_sh8: up to 327,680
faces; cap6_sh8: an open disk of 52,982 faces) store the integer outputs in full -- singular indices, seams (packed bits), the combed
matching, the fixing order and values, the counts -- and the floating-point outputs on a
seeded sample (the field angle per face and the map's values at every fixed variable and at a
sample of the others); their meshes are regenerated by metriko_gb300.meshgen, checked against
stored sample positions.  Each fixture also records the oracle's tie statistics (steps where
the greedy pick differs from the strict '<' pick among fractional and among already-integral
candidates, the smallest margin) and its run time.

Run:  python tests/golden/make_golden.py [name ...]   (all fixtures when no name is given)
"""
import hashlib
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from metriko_gb300 import meshgen  # noqa: E402
from oracle import metriko_oracle as O  # noqa: E402

SMALL = ["ico2_noise", "ico3_noise", "torus_32x16", "genus2_s3", "cap3_noise", "cap4_sh8", "cyl_32x12"]
LARGE = ["ico5_sh8", "ico6_sh8", "ico7_sh8", "cap6_sh8"]
REFERENCE_OBJ = Path("/root/reference/example/models/icosphere.obj")
SAMPLE = 32768


def _tie_stats(info):
    sd = info["strict_differs"]
    frac = [g for _, g, dp in sd if dp > 10e-7]
    return dict(strict_differs=np.int32(len(frac)), integral_differs=np.int32(len(sd) - len(frac)),
                strict_gap_max=np.float64(max(frac, default=0.0)),
                min_margin=np.float64(min(info["margins"]) if info["margins"] else np.inf),
                resolves=np.int32(info["resolves"]))


def _small(name, V, F, ratio, rs, out, seconds):
    info = out["info"]
    return dict(V=V, F=F, ratio=ratio, round_seams=rs,
                compressed=out["compressed"], singular=out["singular"], seam=np.packbits(out["seam"]),
                n_edges=len(out["seam"]), combed_matching=out["combed_matching"].astype(np.int8),
                fix_order=np.asarray(info["fix_order"], np.int32), fix_vals=np.asarray(info["fix_vals"], np.int32),
                fullx=out["fullx"], x_naive=info["x0"], cutF=out["cutF"].astype(np.int32),
                oracle_seconds=np.float64(seconds), **_tie_stats(info))


def _large(name, V, F, ratio, rs, out, seconds):
    info = out["info"]
    rng = np.random.default_rng(1234)
    nF, nV = len(F), len(V)
    fullx = out["fullx"]
    fix = np.asarray(info["fix_order"], np.int32)
    fsamp = np.sort(rng.choice(nF, size=min(SAMPLE, nF), replace=False)).astype(np.int32)
    xsamp = np.sort(rng.choice(len(fullx), size=min(SAMPLE, len(fullx)), replace=False)).astype(np.int32)
    vsamp = np.sort(rng.choice(nV, size=min(1024, nV), replace=False)).astype(np.int32)
    st = out["setup"]
    return dict(workload=name, nV=np.int32(nV), nF=np.int32(nF), ratio=ratio, round_seams=rs,
                mesh_sha256=hashlib.sha256(V.tobytes() + F.astype(np.int32).tobytes()).hexdigest(),
                v_sample_idx=vsamp, v_sample=V[vsamp],
                singular=out["singular"].astype(np.int8), seam=np.packbits(out["seam"]), n_edges=len(out["seam"]),
                combed_matching=out["combed_matching"].astype(np.int8),
                fix_order=fix, fix_vals=np.asarray(info["fix_vals"], np.int32),
                n_full=np.int32(len(fullx)), nT=np.int32(st["nT"]), nS=np.int32(st["nS"]),
                face_sample=fsamp, field_angle=np.angle(out["compressed"][fsamp]),
                fullx_fixed=fullx[fix], x_sample_idx=xsamp, fullx_sample=fullx[xsamp],
                x_naive_sample=info["x0"][xsamp], uv_ptp=np.float64(np.ptp(fullx)),
                oracle_seconds=np.float64(seconds), **_tie_stats(info))


def main(names):
    # bit-identical LM normal matrices reuse their factorisation (identical results, far less time
    # on the level-7 mesh, where round-off keeps the reference's LM iterating)
    O.REUSE_IDENTICAL_FACTORIZATION = True
    for name in names:
        if name == "icosphere_obj":
            V0, F = meshgen.read_obj(REFERENCE_OBJ)
            V, ratio, rs = meshgen.radial_noise(V0, 0.01, 0), 0.03, False
        else:
            V, F, ratio, rs = meshgen.workload(name)
        t0 = time.perf_counter()
        out = O.pipeline(V, F, ratio=ratio, round_seams=rs)
        seconds = time.perf_counter() - t0
        data = (_large if name in LARGE else _small)(name, V, F, ratio, rs, out, seconds)
        np.savez_compressed(Path(__file__).parent / f"{name}.npz", **data)
        info = out["info"]
        print(f"{name}: {len(F)} faces, {len(info['fix_order'])} fixings, {info['resolves']} re-solves, "
              f"{int(data['strict_differs'])} fractional / {int(data['integral_differs'])} integral steps differ "
              f"from strict '<', oracle {seconds:.1f} s", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:] or SMALL + ["icosphere_obj"] + LARGE)
