"""The general sparse seam on the GPU (mtk_csr_create / mtk_csr_pcg / mtk_csr_smallest_eig):
assembled matrices -- the field's connection Laplacian (complex Hermitian) and the naive
integration's normal matrix (real SPD) of the oracle -- solved on the device and checked against
scipy's direct solves, one and several right-hand sides, FP64 and mixed precision; the
reference's solveSmallestEig on the assembled (L, M) against the oracle's."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import metriko_gb300 as M
from metriko_gb300 import meshgen
from oracle import metriko_oracle as O

pytestmark = pytest.mark.gpu


def _laplacian(name):
    V, F, _, _ = meshgen.workload(name)
    m = O.Hmesh(V, F)
    return m, O.connection_laplacian(m, 4), O.mass_matrix(m)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("nrhs", [1, 3, 6])
def test_csr_pcg_complex_hermitian(gpu_ctx, prec, nrhs):
    m, L, _ = _laplacian("ico4_noise")
    rng = np.random.default_rng(7)
    B = rng.normal(size=(m.nF, nrhs)) + 1j * rng.normal(size=(m.nF, nrhs))
    ref = spla.splu(L.tocsc()).solve(B)
    A = M.CsrMatrix(gpu_ctx, L)
    X, st = A.solve(B, opts=M.solve_opts(prec, tol=1e-10))
    for k in range(nrhs):
        assert np.linalg.norm(L @ X[:, k] - B[:, k]) <= 1.0001e-10 * np.linalg.norm(B[:, k])
        assert np.linalg.norm(X[:, k] - ref[:, k]) <= 1e-6 * np.linalg.norm(ref[:, k])
    assert st["pcg_iters"] > 0 and st["max_rel_residual"] <= 1.0001e-10


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_csr_pcg_real_spd(gpu_ctx, prec):
    """The naive integration's normal matrix X2F^T X2F plus the anchor's penalty rows."""
    V, F, ratio, rs = meshgen.workload("ico3_noise")
    out = O.pipeline(V, F, ratio=ratio, seamless=False, round_seams=rs)
    UFull = O.build_ufull(out["Cfull"])[0]
    X2F = ((out["G2"] @ out["fullx2N"]) @ UFull).tocsr()
    fixed = np.asarray(out["setup"]["fixedIdcs"])
    P = sp.csr_matrix((np.full(len(fixed), 1.0), (np.arange(len(fixed)), fixed)), shape=(len(fixed), UFull.shape[0]))
    K = (X2F.T @ X2F + 1e2 * (P @ UFull).T @ (P @ UFull)).tocsr()
    rng = np.random.default_rng(8)
    B = rng.normal(size=(K.shape[0], 2))
    ref = spla.spsolve(K.tocsc(), B)
    A = M.CsrMatrix(gpu_ctx, K)
    X, _ = A.solve(B, opts=M.solve_opts(prec, tol=1e-10))
    for k in range(2):
        assert np.linalg.norm(K @ X[:, k] - B[:, k]) <= 1.0001e-10 * np.linalg.norm(B[:, k])
        assert np.linalg.norm(X[:, k] - ref[:, k]) <= 1e-5 * np.linalg.norm(ref[:, k])


def test_csr_smallest_eig_matches_oracle(gpu_ctx):
    m, L, Mm = _laplacian("ico3_noise")
    x0 = O.seeded_init(m.nF, 0)
    ref = O.smallest_eig(L, Mm, x0, 50)
    c, _ = M.csr_smallest_eig(gpu_ctx, M.CsrMatrix(gpu_ctx, L), M.CsrMatrix(gpu_ctx, Mm), x0, 50,
                              opts=M.solve_opts("fp64", tol=1e-12))
    assert np.abs(np.angle(c / ref)).max() / 4 < 1e-5
    assert abs(np.vdot(c, L @ c).real - np.vdot(ref, L @ ref).real) <= 1e-6 * np.vdot(ref, L @ ref).real


def test_csr_rejects_a_matrix_without_positive_diagonal(gpu_ctx):
    A = sp.csr_matrix(np.array([[1.0, 0.5], [0.5, -2.0]]))
    with pytest.raises(M.MetrikoError) as e:
        M.CsrMatrix(gpu_ctx, A)
    assert e.value.status == M._lib.BAD_INPUT
