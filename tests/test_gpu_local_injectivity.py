"""The localInjectivity path of the whole pipeline on the GPU (mtk_pipeline_run with
local_injectivity set: the naive integration by the device IGM solver, then the damped LM of
NaiveIntegration with the injective barrier and the greedy rounding, each linear solve by the
device FP64 PCG (mtk_csr_pcg) and each orientation check by mtk_local_injectivity) against the
oracle's restatement of the reference (pipeline(..., local_injectivity=True)).

Integer outputs identical: the status (MTK_ERR_ROUNDING exactly where the reference's rounding
fails its integrality check), the fixing order and the rounded values.  uv within 1e-6 of the uv
bounding-box diagonal where the rounding succeeds, 1e-3 where it fails (the failing rounding
returns the last iterate of a damped LM that did not reach the lattice, where the iterative and
the direct solves part by about 1e-4 of the diagonal)."""
import numpy as np
import pytest

import metriko_gb300 as M
from metriko_gb300 import meshgen
from oracle import metriko_oracle as O

from test_qex import load_workload

pytestmark = pytest.mark.gpu
ROUNDING = 7

# the workloads' own grid ratios (the barrier inactive), a coarser grid where the barrier is
# active and the rounding still succeeds, and grids where the reference's rounding fails (the
# level-4 sphere at its own ratio among them: 5,120 faces)
CASES = [("ico2_noise", None), ("ico3_noise", 0.15), ("cap3_noise", None), ("ico2_noise", 0.3),
         ("ico3_noise", 0.3), ("torus_32x16", 0.3), ("ico4_noise", None), ("icosphere_obj", None)]


@pytest.mark.parametrize("name,ratio", CASES)
def test_pipeline_local_injectivity_matches_oracle(gpu_ctx, name, ratio):
    V, F, r0, rs = load_workload(name)
    ratio = r0 if ratio is None else ratio
    ref = O.pipeline(V, F, ratio=ratio, round_seams=rs, local_injectivity=True)
    r = M.pipeline(gpu_ctx, V, F, ratio=ratio, round_seams=rs, opts=M.solve_opts("mixed", tol=1e-10),
                   local_injectivity=True)
    assert r["status"] == (0 if ref["success"] else ROUNDING)
    assert np.array_equal(r["singular"], ref["singular"])
    assert np.array_equal(r["seam"], ref["seam"])
    assert list(r["fix_order"]) == list(ref["info"]["fix_order"])
    assert list(r["fix_vals"]) == list(ref["info"]["fix_vals"])
    diag = max(np.ptp(ref["fullx"]), 1.0) * np.sqrt(2.0)
    tol = 1e-6 if ref["success"] else 1e-3
    assert np.abs(r["fullx"] - ref["fullx"]).max() <= tol * diag
    if ref["success"]:
        # the rounded map is locally injective: no face of the cut mesh flipped
        assert M.local_injectivity(gpu_ctx, r["cfn"])[0] == 0


def test_pipeline_local_injectivity_off_is_plain_path(gpu_ctx):
    """local_injectivity=False leaves the plain path untouched (bit-identical fullx)."""
    V, F, ratio, rs = meshgen.workload("ico3_noise")
    a = M.pipeline(gpu_ctx, V, F, ratio=ratio, round_seams=rs)
    b = M.pipeline(gpu_ctx, V, F, ratio=ratio, round_seams=rs, local_injectivity=False)
    assert np.array_equal(a["fullx"], b["fullx"])
    assert list(a["fix_order"]) == list(b["fix_order"])
