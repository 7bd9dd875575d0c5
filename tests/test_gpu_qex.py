"""The reference's example_qex.cpp chain on the GPU product: mtk_pipeline_run with seamless and
localInjectivity on and roundSeams off, then the header-only quad extraction on its corner
parameterisation.  The uv agree with the oracle's to solver tolerance, so the grid points,
ports, q-edges and quads are compared exactly as combinatorics and the positions to 1e-6."""
import numpy as np
import pytest

import metriko_gb300 as M
from oracle import metriko_oracle as O

from test_qex import corner_uv, load_workload, oracle_qex, qex_harness, run_qex_harness  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,ratio", [("ico2_noise", None), ("ico3_noise", 0.15), ("icosphere_obj", None)])
def test_pipeline_qex_matches_oracle(gpu_ctx, qex_harness, tmp_path, name, ratio):  # noqa: F811
    V, F, r0, rs = load_workload(name)
    ratio = r0 if ratio is None else ratio
    ref = O.pipeline(V, F, ratio=ratio, round_seams=False, seamless=True, local_injectivity=True)
    _, q = oracle_qex(ref, F)
    r = M.pipeline(gpu_ctx, V, F, ratio=ratio, round_seams=False, seamless=True, local_injectivity=True,
                   opts=M.solve_opts("mixed", tol=1e-10))
    assert r["status"] == 0
    assert list(r["fix_order"]) == list(ref["info"]["fix_order"])
    uv = corner_uv(r["cfn"], len(F))
    res = run_qex_harness(qex_harness, tmp_path, V, F, uv, r["matching"], r["singular"])
    assert "error" not in res, res.get("error")
    for key in ("vq", "eq", "fq"):
        assert [(g[0], g[2]) for g in res[key]] == [(g[0], g[2]) for g in q[key]]
        if res[key]:
            np.testing.assert_allclose([g[1] for g in res[key]], [g[1] for g in q[key]], atol=1e-6)
    assert [(p[0], p[1], p[2], p[3], p[5], p[7], p[8]) for p in res["ports"]] == \
        [(p["idx"], p["vid"], p["eid"], p["fid"], p["dir"], p["next"], p["prev"]) for p in q["ports"]]
    assert res["edges"] == q["edges"]
    assert len(res["faces"]) == len(q["faces"])
