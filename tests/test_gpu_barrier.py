"""Device barrier and orientation check (the local-injectivity pieces) against the oracle."""
import numpy as np
import pytest

import metriko_gb300 as M
from metriko_gb300 import meshgen
from oracle import metriko_oracle as O

pytestmark = pytest.mark.gpu


def _random_fields(nF, seed):
    rng = np.random.default_rng(seed)
    ang = rng.uniform(0, 2 * np.pi, nF)
    mag = rng.uniform(0.5, 2.0, nF)
    F2 = np.zeros((nF, 4, 2))
    for j in range(4):
        F2[:, j, 0] = mag * np.cos(ang + j * np.pi / 2)
        F2[:, j, 1] = mag * np.sin(ang + j * np.pi / 2)
    # the field: the intrinsic one sheared and flipped on some faces, so that the volume ratio
    # covers r <= 0, 0 < r < 1/2 and r >= 1/2
    field = F2 + rng.normal(0, 0.8, F2.shape) * mag[:, None, None]
    return F2.reshape(-1), field.reshape(-1)


@pytest.mark.parametrize("nF", [1000, 200000])
def test_injective_barrier_matches_oracle(gpu_ctx, nF):
    F2, field = _random_fields(nF, nF)
    fB, der, S = M.injective_barrier(gpu_ctx, F2, field)
    rB, rder, rS = O.injective_barrier_update(F2, field)
    assert np.array_equal(np.isinf(fB), np.isinf(rB)) and np.isinf(rB).any() and (rB == 0).any()
    # 1/bar - 1 and bar' cancel near saturation (r -> 1/2, bar -> 1): the device forms the cubes
    # as products where the reference calls pow, so compare with an absolute floor there
    fin = np.isfinite(rB)
    assert np.allclose(fB[fin], rB[fin], rtol=1e-10, atol=1e-12)
    assert np.array_equal(np.isinf(der), np.isinf(rder))
    fd = np.isfinite(rder)
    assert np.allclose(der[fd], rder[fd], rtol=1e-10, atol=1e-10)
    assert np.array_equal(S, rS)
    fB2, d2, S2 = M.injective_barrier(gpu_ctx, F2, field, update_j=False)
    assert d2 is None and S2 is None and np.array_equal(np.isinf(fB2), np.isinf(fB))


@pytest.mark.parametrize("name", ["ico4_noise", "torus_64x32"])
def test_local_injectivity_matches_oracle(gpu_ctx, name):
    V, F, ratio, rs = meshgen.workload(name)
    r = M.pipeline(gpu_ctx, V, F, ratio=ratio, round_seams=rs)
    cfn = np.ascontiguousarray(r["cfn"])
    assert M.local_injectivity(gpu_ctx, cfn) == O.locally_injective(cfn)
    planted = cfn.copy().reshape(len(F), 3, 4)
    for f in (5, len(F) // 2):   # swap two corners' (u, v): reverses the orientation
        planted[f, 1, :2], planted[f, 2, :2] = planted[f, 2, :2].copy(), planted[f, 1, :2].copy()
    got = M.local_injectivity(gpu_ctx, planted)
    assert got == O.locally_injective(planted)
