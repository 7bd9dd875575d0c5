"""Smoothest-field parity on the GPU: the device inverse power iteration against the oracle's
direct-solve iteration from the same seeded start vector.

Tolerances (from the reference path's spec): per-face field angle within 1e-5 rad and the
Dirichlet energy c^H L c within 1e-6 relative, for both the FP64 and the mixed path."""
import numpy as np
import pytest

import metriko_gb300 as M
from metriko_gb300 import meshgen
from oracle import metriko_oracle as O

pytestmark = pytest.mark.gpu


def _inputs(name):
    V, F, _, _ = meshgen.workload(name)
    m = O.Hmesh(V, F)
    nbr = m.face[m.twin[m.FH]]
    theta = m.farg[m.FH] - m.farg[m.twin[m.FH]]
    return m, nbr, theta


@pytest.mark.parametrize("name", ["ico3_noise", "ico4_noise", "torus_32x16"])
@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_field_matches_oracle(gpu_ctx, name, prec):
    m, nbr, theta = _inputs(name)
    x0 = O.seeded_init(m.nF, 0)
    L = O.connection_laplacian(m, 4)
    Mm = O.mass_matrix(m)
    ref = O.smallest_eig(L, Mm, x0, 50)
    c, st = M.field_smoothest(gpu_ctx, nbr, theta, m.faceArea, x0, opts=M.solve_opts(prec, tol=1e-10))
    ang = np.abs(np.angle(c / ref)).max() / 4
    assert ang < 1e-5, ang
    e_ref = np.vdot(ref, L @ ref).real
    e_gpu = np.vdot(c, L @ c).real
    assert abs(e_gpu - e_ref) / e_ref < 1e-6
    assert abs(np.vdot(c, Mm @ c).real - 1) < 1e-9
    assert st["max_rel_residual"] <= 1e-10
    assert st["pcg_iters"] > 0


def test_field_is_deterministic(gpu_ctx):
    m, nbr, theta = _inputs("ico4_noise")
    x0 = O.seeded_init(m.nF, 3)
    a, _ = M.field_smoothest(gpu_ctx, nbr, theta, m.faceArea, x0)
    b, _ = M.field_smoothest(gpu_ctx, nbr, theta, m.faceArea, x0)
    assert np.array_equal(a, b)


def test_field_iteration_cap_reports_not_converged(gpu_ctx):
    m, nbr, theta = _inputs("ico3_noise")
    x0 = O.seeded_init(m.nF, 0)
    with pytest.raises(M.MetrikoError) as e:
        M.field_smoothest(gpu_ctx, nbr, theta, m.faceArea, x0, opts=M.solve_opts("fp64", tol=1e-12, max_iter=1))
    assert e.value.status == M._lib.NOT_CONVERGED


@pytest.mark.parametrize("bad", ["past_end", "minus_two", "own_face"])
def test_field_rejects_bad_neighbour(gpu_ctx, bad):
    """-1 marks a boundary side; any other index outside [0, nF), or the face's own, is rejected."""
    m, nbr, theta = _inputs("ico3_noise")
    nbr = nbr.copy()
    nbr[5, 1] = {"past_end": m.nF + 7, "minus_two": -2, "own_face": 5}[bad]
    with pytest.raises(M.MetrikoError) as e:
        M.field_smoothest(gpu_ctx, nbr, theta, m.faceArea, O.seeded_init(m.nF, 0))
    assert e.value.status == M._lib.BAD_INPUT


@pytest.mark.parametrize("name", ["ico3_noise", "torus_32x16"])
@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_field_solve_matches_oracle(gpu_ctx, name, prec):
    """mtk_field_solve (L x = rhs, the CurvatureAligned solve) against a direct sparse LU."""
    m, nbr, theta = _inputs(name)
    c_ref, rhs = O.curvature_aligned(m)
    c, st = M.field_solve(gpu_ctx, nbr, theta, m.faceArea, rhs, opts=M.solve_opts(prec, tol=1e-10))
    assert np.abs(c - c_ref).max() <= 1e-8 * np.abs(c_ref).max()
    assert st["max_rel_residual"] <= 1e-10


@pytest.mark.parametrize("name", ["ico4_noise", "torus_32x16"])
def test_curvature_aligned_pipeline_field_matches_oracle(gpu_ctx, name):
    """FieldType::CurvatureAligned through the pipeline: the host principal-curvature right-hand
    side and the device solve against the oracle; then the whole path runs to integral values."""
    V, F, ratio, rs = meshgen.workload(name)
    m = O.Hmesh(V, F)
    c_ref, _ = O.curvature_aligned(m)
    r = M.pipeline(gpu_ctx, V, F, ratio=ratio, round_seams=rs, field_type="curvature_aligned",
                   opts=M.solve_opts("fp64", tol=1e-10), stop_after=1)
    assert np.abs(r["compressed"] - c_ref).max() <= 1e-8 * np.abs(c_ref).max()
    full = M.pipeline(gpu_ctx, V, F, ratio=ratio, round_seams=rs, field_type="curvature_aligned")
    assert full["status"] == 0
    chi = 2 if name.startswith("ico") else 0
    assert full["singular"].sum() == 4 * chi
    X, fo = full["fullx"], full["fix_order"]
    assert np.abs(X[fo] - np.round(X[fo])).max() <= 1e-6
