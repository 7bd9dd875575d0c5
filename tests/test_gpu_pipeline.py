"""Whole path on the GPU (mtk_pipeline_run through the C ABI) against the oracle and the golden
fixtures: singularities, seams, combed matching, the greedy fixing order and the rounded values
are integer outputs and must be identical; uv (fullx) within 1e-6 of the uv bounding-box
diagonal; FP64 and mixed precision both."""
from pathlib import Path

import numpy as np
import pytest

import metriko_gb300 as M
from metriko_gb300 import meshgen
from oracle import metriko_oracle as O

from conftest import oracle_run

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).parent / "golden"
TOL = 1e-10


def _uv_diag(x):
    return max(np.ptp(x), 1.0) * np.sqrt(2.0)


@pytest.mark.parametrize("name", ["ico2_noise", "ico3_noise", "torus_32x16", "genus2_s3", "icosphere_obj"])
@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_pipeline_matches_golden(gpu_ctx, name, prec):
    """icosphere_obj is the reference's own model (example/models/icosphere.obj, the level-4
    workload's mesh) with the workload's radial noise; the others are seeded meshes."""
    g = np.load(GOLDEN / f"{name}.npz")
    r = M.pipeline(gpu_ctx, g["V"], g["F"], ratio=float(g["ratio"]), round_seams=bool(g["round_seams"]),
                   opts=M.solve_opts(prec, tol=TOL))
    assert r["status"] == 0
    assert np.array_equal(r["singular"], g["singular"])
    assert np.array_equal(r["seam"], np.unpackbits(g["seam"])[: int(g["n_edges"])].astype(bool))
    assert np.array_equal(r["matching"], g["combed_matching"])
    assert list(r["fix_order"]) == list(g["fix_order"])
    assert list(r["fix_vals"]) == list(g["fix_vals"])
    assert np.abs(r["fullx"] - g["fullx"]).max() <= 1e-6 * _uv_diag(g["fullx"])
    assert np.abs(r["x_naive"] - g["x_naive"]).max() <= 1e-6 * _uv_diag(g["x_naive"])
    assert np.abs(np.angle(r["compressed"] / g["compressed"])).max() / 4 < 1e-5


@pytest.mark.parametrize("name", ["ico4_noise", "torus_64x32"])
def test_pipeline_matches_oracle(gpu_ctx, name):
    V, F, ratio, rs, ref = oracle_run(name)
    r = M.pipeline(gpu_ctx, V, F, ratio=ratio, round_seams=rs, opts=M.solve_opts("mixed", tol=TOL))
    assert r["status"] == 0
    assert np.array_equal(r["singular"], ref["singular"])
    assert np.array_equal(r["seam"], ref["seam"])
    assert list(r["fix_order"]) == list(ref["info"]["fix_order"])
    assert list(r["fix_vals"]) == list(ref["info"]["fix_vals"])
    assert np.abs(r["fullx"] - ref["fullx"]).max() <= 1e-6 * _uv_diag(ref["fullx"])
    cfn = r["cfn"]
    assert np.abs(cfn - ref["cfn"]).max() <= 1e-6 * _uv_diag(ref["fullx"])


def test_pipeline_deterministic(gpu_ctx):
    V, F, ratio, rs = meshgen.workload("ico4_noise")
    a = M.pipeline(gpu_ctx, V, F, ratio=ratio)
    b = M.pipeline(gpu_ctx, V, F, ratio=ratio)
    assert np.array_equal(a["fullx"], b["fullx"])
    assert list(a["fix_order"]) == list(b["fix_order"])


@pytest.mark.parametrize("case", ["ico4_noise", "torus_32x16"])
def test_igm_z_state_in_global_memory_matches_shared(gpu_ctx, monkeypatch, case):
    """The IGM kernel keeps the replicated z state (constraint-kernel coordinates) of each CTA in
    shared memory, or in a global slice per CTA when it does not fit (meshes with many
    singularities; MTK_Z_GLOBAL=1 forces it).  Both give the same arithmetic: bit-identical maps,
    fixing order and iteration counts."""
    V, F, ratio, rs = meshgen.workload(case)
    opts = M.solve_opts("mixed", tol=1e-8)
    a = M.pipeline(gpu_ctx, V, F, ratio=ratio, round_seams=rs, opts=opts)
    monkeypatch.setenv("MTK_Z_GLOBAL", "1")
    b = M.pipeline(gpu_ctx, V, F, ratio=ratio, round_seams=rs, opts=opts)
    assert a["status"] == 0 and b["status"] == 0
    assert np.array_equal(a["fullx"], b["fullx"])
    assert list(a["fix_order"]) == list(b["fix_order"]) and list(a["fix_vals"]) == list(b["fix_vals"])
    assert a["stats"]["pcg_iters"] == b["stats"]["pcg_iters"]


@pytest.mark.parametrize("name", ["ico4_noise", "ico6_sh8", "torus_64x32"])
def test_igm_multigrid_device_build_matches_host(gpu_ctx, monkeypatch, name):
    """The multigrid set-up on the device (the default: the IGM free block, both hierarchies'
    products) gives the same arrays as the host set-up, so the whole pipeline is bit-identical
    either way."""
    V, F, ratio, rs = meshgen.workload(name)
    opts = M.solve_opts("mixed", tol=1e-8)
    a = M.pipeline(gpu_ctx, V, F, ratio=ratio, round_seams=rs, opts=opts)
    monkeypatch.setenv("MTK_MG_HOST", "1")
    b = M.pipeline(gpu_ctx, V, F, ratio=ratio, round_seams=rs, opts=opts)
    assert np.array_equal(a["fullx"], b["fullx"])
    assert list(a["fix_order"]) == list(b["fix_order"])
    assert a["stats"]["pcg_iters"] == b["stats"]["pcg_iters"]


def _wrap(a):
    return np.abs((a + np.pi) % (2.0 * np.pi) - np.pi)


@pytest.mark.parametrize("name", ["ico5_sh8", "ico6_sh8", "ico7_sh8"])
@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_pipeline_matches_large_golden(gpu_ctx, name, prec):
    """The oracle's outputs on the level-5/6/7 spheres with the level-7 workload's displacement
    (20,480 / 81,920 / 327,680 faces; level 7 is the workload itself): singular indices, seams,
    combed matching, the fixing order and the rounded values identical; the field within 1e-5
    rad per face and the map within 1e-6 of its bounding-box diagonal on the stored samples."""
    g = np.load(GOLDEN / f"{name}.npz")
    V, F, ratio, rs = meshgen.workload(name)
    assert len(V) == int(g["nV"]) and len(F) == int(g["nF"])
    assert np.abs(V[g["v_sample_idx"]] - g["v_sample"]).max() <= 1e-12
    r = M.pipeline(gpu_ctx, V, F, ratio=ratio, round_seams=rs, opts=M.solve_opts(prec, tol=TOL))
    assert r["status"] == 0
    assert np.array_equal(r["singular"], g["singular"].astype(np.int32))
    assert np.array_equal(r["seam"], np.unpackbits(g["seam"])[: int(g["n_edges"])].astype(bool))
    assert np.array_equal(r["matching"], g["combed_matching"].astype(np.int32))
    assert r["counts"]["nT"] == int(g["nT"]) and r["counts"]["nS"] == int(g["nS"])
    assert list(r["fix_order"]) == list(g["fix_order"])
    assert list(r["fix_vals"]) == list(g["fix_vals"])
    diag = max(float(g["uv_ptp"]), 1.0) * np.sqrt(2.0)
    assert len(r["fullx"]) == int(g["n_full"])
    assert np.abs(r["fullx"][g["fix_order"]] - g["fullx_fixed"]).max() <= 1e-6 * diag
    assert np.abs(r["fullx"][g["x_sample_idx"]] - g["fullx_sample"]).max() <= 1e-6 * diag
    assert np.abs(r["x_naive"][g["x_sample_idx"]] - g["x_naive_sample"]).max() <= 1e-6 * diag
    assert _wrap(np.angle(r["compressed"][g["face_sample"]]) - g["field_angle"]).max() / 4 < 1e-5


# full-size workloads: level-7 sphere (327,680 faces), the level-8 benchmark sphere (1,310,720
# faces), the 1024 x 512 torus (1,048,576 faces, seams rounded), the level-9 sphere with
# degree-16 displacement (5,242,880 faces)
@pytest.mark.parametrize("name,prec,chi", [("ico6_sh8", "mixed", 2), ("ico7_sh8", "mixed", 2), ("ico7_sh8", "fp64", 2),
                                           ("ico8_sh8", "mixed", 2), ("ico8_sh8", "fp64", 2),
                                           ("torus_1024x512", "mixed", 0), ("ico9_sh16", "mixed", 2)])
def test_pipeline_size_independent_properties(gpu_ctx, name, prec, chi):
    """At sizes beyond the oracle: sum of indices = 4 chi (Poincare-Hopf), every rounded value
    within 1e-6 of an integer and equal to the reported value, all solves at the requested
    residual."""
    V, F, ratio, rs = meshgen.workload(name)
    r = M.pipeline(gpu_ctx, V, F, ratio=ratio, round_seams=rs, opts=M.solve_opts(prec, tol=1e-8))
    assert r["status"] == 0
    assert r["singular"].sum() == 4 * chi
    X = r["fullx"]
    fo = r["fix_order"]
    if chi != 0:
        assert len(fo) == 2 * (r["counts"]["nS"] + r["counts"]["nT"])
    else:   # torus with round_seams: the translations of every transition are rounded
        assert len(fo) == 2 * r["counts"]["nT"] and len(fo) > 0
    assert np.abs(X[fo] - np.round(X[fo])).max() <= 1e-6
    assert np.array_equal(np.round(X[fo]).astype(int), r["fix_vals"])
    assert r["stats"]["max_rel_residual"] <= 1e-8 * 1.0001
