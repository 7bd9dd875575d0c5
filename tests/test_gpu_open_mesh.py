"""Meshes with boundary on the GPU: the whole path (mtk_pipeline_run) against the oracle's golden
fixtures of open disks (cap3_noise, cap4_sh8, cap6_sh8) and an open cylinder (cyl_32x12, seams
rounded), the field solve against the oracle's direct solves, the device field inputs and the
device Curl matching against the host / oracle, and larger open disks through size-independent
properties.  Same bars as the closed meshes: integer outputs identical, the field within 1e-5
rad per face and 1e-6 relative energy, uv within 1e-6 of the uv bounding-box diagonal; FP64 and
mixed precision both."""
from pathlib import Path

import numpy as np
import pytest

import metriko_gb300 as M
from metriko_gb300 import meshgen
from oracle import metriko_oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).parent / "golden"
TOL = 1e-10


def _uv_diag(x):
    return max(np.ptp(x), 1.0) * np.sqrt(2.0)


def _wrap(a):
    return np.abs((a + np.pi) % (2.0 * np.pi) - np.pi)


@pytest.mark.parametrize("name", ["cap3_noise", "cap4_sh8", "cyl_32x12"])
@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_open_pipeline_matches_golden(gpu_ctx, name, prec):
    g = np.load(GOLDEN / f"{name}.npz")
    r = M.pipeline(gpu_ctx, g["V"], g["F"], ratio=float(g["ratio"]), round_seams=bool(g["round_seams"]),
                   opts=M.solve_opts(prec, tol=TOL))
    assert r["status"] == 0, M.lib().mtk_last_error().decode()
    assert np.array_equal(r["singular"], g["singular"])
    assert np.array_equal(r["seam"], np.unpackbits(g["seam"])[: int(g["n_edges"])].astype(bool))
    assert np.array_equal(r["matching"], g["combed_matching"])
    assert list(r["fix_order"]) == list(g["fix_order"])
    assert list(r["fix_vals"]) == list(g["fix_vals"])
    assert np.abs(r["fullx"] - g["fullx"]).max() <= 1e-6 * _uv_diag(g["fullx"])
    assert np.abs(r["x_naive"] - g["x_naive"]).max() <= 1e-6 * _uv_diag(g["x_naive"])
    assert _wrap(np.angle(r["compressed"] / g["compressed"])).max() / 4 < 1e-5


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_open_pipeline_matches_large_golden(gpu_ctx, prec):
    """An open disk of 52,982 faces (the level-6 sphere's cap above z = -0.3, the level-7
    workload's displacement)."""
    g = np.load(GOLDEN / "cap6_sh8.npz")
    V, F, ratio, rs = meshgen.workload("cap6_sh8")
    assert len(V) == int(g["nV"]) and len(F) == int(g["nF"])
    assert np.abs(V[g["v_sample_idx"]] - g["v_sample"]).max() <= 1e-12
    r = M.pipeline(gpu_ctx, V, F, ratio=ratio, round_seams=rs, opts=M.solve_opts(prec, tol=TOL))
    assert r["status"] == 0, M.lib().mtk_last_error().decode()
    assert np.array_equal(r["singular"], g["singular"].astype(np.int32))
    assert np.array_equal(r["seam"], np.unpackbits(g["seam"])[: int(g["n_edges"])].astype(bool))
    assert np.array_equal(r["matching"], g["combed_matching"].astype(np.int32))
    assert r["counts"]["nT"] == int(g["nT"]) and r["counts"]["nS"] == int(g["nS"])
    assert list(r["fix_order"]) == list(g["fix_order"])
    assert list(r["fix_vals"]) == list(g["fix_vals"])
    diag = max(float(g["uv_ptp"]), 1.0) * np.sqrt(2.0)
    assert np.abs(r["fullx"][g["fix_order"]] - g["fullx_fixed"]).max() <= 1e-6 * diag
    assert np.abs(r["fullx"][g["x_sample_idx"]] - g["fullx_sample"]).max() <= 1e-6 * diag
    assert _wrap(np.angle(r["compressed"][g["face_sample"]]) - g["field_angle"]).max() / 4 < 1e-5


@pytest.mark.parametrize("name", ["cap4_sh8", "cyl_64x24"])
@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_open_field_matches_oracle(gpu_ctx, name, prec):
    """The field solve with boundary sides (nbr -1: the row's diagonal is its count of neighbours
    + 1e-9) through the multigrid path, against the oracle's 50 inverse iterations with direct
    solves from the same start vector.  The cylinder is flat: a parallel field has zero Dirichlet
    energy, L's smallest eigenvalue is the 1e-9 shift (condition ~6e9), so its first solves end
    at a true relative residual near cond(L) * eps rather than the tolerance, and the mixed path
    falls back to FP64 PCG (FP32 refinement cannot converge there); the field still matches."""
    V, F, _, _ = meshgen.workload(name)
    m = O.Hmesh(V, F)
    nbr, theta, area = M.field_inputs(V, F)
    assert (nbr == -1).any()
    x0 = O.seeded_init(m.nF, 0)
    c, st = M.field_smoothest(gpu_ctx, nbr, theta, area, x0, opts=M.solve_opts(prec, tol=1e-10))
    L = O.connection_laplacian(m, 4)
    ref = O.smallest_eig(L, O.mass_matrix(m), x0, 50)
    assert _wrap(np.angle(c / ref)).max() / 4 < 1e-5
    e, e_ref = np.vdot(c, L @ c).real, np.vdot(ref, L @ ref).real
    assert abs(e - e_ref) / e_ref < 1e-6
    assert st["max_rel_residual"] <= (1e-10 if name.startswith("cap") else 1e-6)


def test_open_device_field_inputs_match_host(gpu_ctx):
    V, F, _, _ = meshgen.workload("cap4_sh8")
    nbr_d, theta_d, area_d = M.mesh_field_inputs(gpu_ctx, V, F)
    nbr, theta, area = M.field_inputs(V, F)
    assert np.array_equal(nbr_d, nbr) and (nbr == -1).any()
    assert np.abs(theta_d - theta).max() <= 1e-12
    assert (theta_d[nbr == -1] == 0).all()
    assert np.array_equal(area_d, area)


@pytest.mark.parametrize("name", ["cap3_noise", "cap4_sh8", "cyl_32x12"])
def test_open_curl_matching_matches_oracle(gpu_ctx, name):
    """mtk_curl_matching with the halfedge arrays of a mesh with boundary: matching -1 on
    boundary edges, singular index 1 on boundary vertices, the rest identical to the oracle."""
    g = np.load(GOLDEN / f"{name}.npz")
    m = O.Hmesh(g["V"], g["F"])
    c = g["compressed"]
    match, sing = M.curl_matching(gpu_ctx, m.pos, m.idx, m.edge2vert, m.edge2face, m.vert2half, m.prev,
                                  m.angleDefect, c, twin=m.twin, half_edge=m.edge, edge_half=m.edge2half)
    fld = O.rosy_from_compressed(c, 4)
    ref_match, effort = O.c_matching(m, fld, O.compute_connection(m), 4)
    assert np.array_equal(match, ref_match)
    assert np.array_equal(sing, O.compute_singular(m, effort, 4))
    assert np.array_equal(sing, g["singular"])
    assert (match[m.isBE] == -1).all() and (sing[m.isBV] == 1).all()


@pytest.mark.parametrize("name", ["cap7_sh8", "cap8_sh8"])
def test_open_pipeline_size_independent_properties(gpu_ctx, name):
    """Open disks of 212K and 850K faces, beyond the oracle: every rounded value within 1e-6 of
    an integer and equal to the reported value, boundary vertices with index 1 and boundary
    edges on the seam, all solves at the requested residual."""
    V, F, ratio, rs = meshgen.workload(name)
    r = M.pipeline(gpu_ctx, V, F, ratio=ratio, round_seams=rs, opts=M.solve_opts("mixed", tol=1e-8))
    assert r["status"] == 0, M.lib().mtk_last_error().decode()
    EV, _, EF = O.edge_topology(F)                      # the edge numbering of the outputs
    isBE = (EF < 0).any(axis=1)
    isBV = np.zeros(len(V), bool)
    isBV[EV[isBE].ravel()] = True
    assert isBE.any()
    assert (r["singular"][isBV] == 1).all()
    assert r["seam"][isBE].all()
    assert (r["matching"][isBE] == -1).all()
    X = r["fullx"]
    fo = r["fix_order"]
    assert len(fo) == 2 * (r["counts"]["nS"] + r["counts"]["nT"]) and len(fo) > 0
    assert np.abs(X[fo] - np.round(X[fo])).max() <= 1e-6
    assert np.array_equal(np.round(X[fo]).astype(int), r["fix_vals"])
    assert r["stats"]["max_rel_residual"] <= 1e-8 * 1.0001
