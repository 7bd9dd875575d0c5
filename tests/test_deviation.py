"""The check at the end of the reference's integ() (parameterization_integ.ipp:100-117): how far
the normalized per-face gradients of the map are from the normalized extrinsic field.  Host C++
(mtk_map_deviation, the function RosyParameterization::integ() uses) against the oracle on the
oracle's maps, and known answers from linear maps."""
import numpy as np
import pytest

import metriko_gb300 as M
from metriko_gb300 import meshgen
from oracle import metriko_oracle as O


def _linear_map(V, F, A):
    """Corner values of the linear functions u_k(x) = A[k] . x and, per face, the gradient of
    each restricted to the face plane (A[k] minus its normal component)."""
    p = V[F]
    n = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    N = len(A)
    cfn = np.concatenate([p[:, j] @ A.T for j in range(3)], axis=1)           # nF x 3N
    grad = A[None, :, :] - (n @ A.T)[:, :, None] * n[:, None, :]              # nF x N x 3
    return cfn, grad.reshape(len(F), 3 * N)


@pytest.mark.parametrize("name", ["ico2_noise", "torus_32x16", "genus2_s3"])
def test_linear_map_has_zero_deviation(name):
    V, F, _, _ = meshgen.workload(name)
    A = np.random.default_rng(0).normal(size=(4, 3))
    cfn, ext = _linear_map(V, F, A)
    assert M.map_deviation(V, F, cfn, ext) < 1e-12
    assert O.map_deviation(V, F, cfn, ext) < 1e-12
    # the opposite field: every normalized difference has length 2
    assert M.map_deviation(V, F, cfn, -ext) == pytest.approx(2.0, abs=1e-12)


@pytest.mark.parametrize("name", ["ico2_noise", "ico3_noise", "torus_32x16", "genus2_s3"])
def test_deviation_matches_oracle(name):
    V, F, ratio, rs = meshgen.workload(name)
    ref = O.pipeline(V, F, ratio=ratio, round_seams=rs)
    a = O.map_deviation(ref["cutV"], ref["cutF"], ref["cfn"], ref["ext"])
    b = M.map_deviation(ref["cutV"], ref["cutF"], ref["cfn"], ref["ext"])
    assert abs(a - b) <= 1e-12 * a
    assert 0 < a < 0.2            # the rounded map follows the field closely


def test_deviation_rejects_bad_input():
    V, F, _, _ = meshgen.workload("ico2_noise")
    cfn = np.zeros((len(F), 12))
    F2 = F.copy()
    F2[0, 0] = len(V)
    with pytest.raises(M.MetrikoError):
        M.map_deviation(V, F2, cfn, cfn)
    with pytest.raises(ValueError):
        M.map_deviation(V, F, cfn[:, :6], cfn)
