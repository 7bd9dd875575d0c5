"""The oracle's size-field gradient (adjoint of the naive integration) against central finite
differences, on the CPU."""
import numpy as np
import pytest

import oracle.metriko_oracle as O
from metriko_gb300 import meshgen


@pytest.mark.parametrize("target", ["integration", "perturbed"])
def test_oracle_size_field_gradient_matches_finite_differences(target):
    V, F, ratio, _ = meshgen.workload("ico2_noise")
    out = O.pipeline(V, F, ratio=ratio, seamless=False)
    rng = np.random.default_rng(1)
    s = rng.normal(0, 0.2, len(V))
    T = None if target == "integration" else out["F2"] * (1 + 0.3 * rng.normal(size=out["F2"].shape))
    loss, g, _ = O.size_field_gradient(out, F, s, T, mu=0.1)
    assert np.isfinite(loss) and np.all(np.isfinite(g))
    h = 1e-4
    for _ in range(8):
        d = rng.normal(size=len(V))
        fd = (O.size_field_gradient(out, F, s + h * d, T, 0.1)[0] - O.size_field_gradient(out, F, s - h * d, T, 0.1)[0]) / (2 * h)
        assert abs(fd - g @ d) <= 1e-5 * max(abs(fd), 1.0)


def test_oracle_size_field_zero_field_reproduces_naive_integration():
    """s = 0 and the integration target: x(s) is the naive Poisson solution ni.x0."""
    V, F, ratio, _ = meshgen.workload("ico2_noise")
    out = O.pipeline(V, F, ratio=ratio, seamless=False)
    _, _, x = O.size_field_gradient(out, F, np.zeros(len(V)))
    assert np.allclose(x, out["info"]["x0"], rtol=1e-9, atol=1e-9 * np.abs(x).max())


@pytest.mark.parametrize("name", ["ico2_noise", "torus_32x16", "cap2_noise"])
def test_oracle_position_gradient_matches_finite_differences(name):
    """The oracle's vertex-position gradient (envelope of the naive integration, reverse pass of
    the 50-step inverse power iteration, complex-step face geometry) against FP64 central
    differences of the whole oracle path, on random directions whose perturbation leaves every
    integer decision (singularities, seams, combed matching) unchanged."""
    V, F, ratio, rs = meshgen.workload(name)
    rng = np.random.default_rng(5)
    s = rng.normal(0, 0.2, len(V))
    loss, gs, gV, _, aux = O.position_gradient(V, F, s, mu=0.1, ratio=ratio, round_seams=rs)
    assert np.isfinite(loss) and np.all(np.isfinite(gV))
    h, checked = 3e-6, 0
    for _ in range(6):
        d = rng.normal(size=V.shape)
        d /= np.linalg.norm(d)
        lp = O.position_gradient(V + h * d, F, s, mu=0.1, ratio=ratio, round_seams=rs)
        lm = O.position_gradient(V - h * d, F, s, mu=0.1, ratio=ratio, round_seams=rs)
        if not all(np.array_equal(x[4][k], aux[k]) for x in (lp, lm) for k in ("singular", "seam", "combed_matching")):
            continue
        fd = (lp[0] - lm[0]) / (2 * h)
        assert abs(fd - np.sum(gV * d)) <= 1e-6 * max(abs(fd), 1e-3 * np.linalg.norm(gV))
        checked += 1
    assert checked >= 4
