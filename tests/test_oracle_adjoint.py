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
