"""The reference's example_qgp.cpp chain on the GPU product: mtk_pipeline_run with seamless off
and localInjectivity on (the naive integration with the injective barrier), then the header-only
motorcycle graph and T-mesh on its corner parameterisation.  The uv agree with the oracle's to
solver tolerance, so the comparison is combinatorial and exact (ports, the crash structure of
every trace, T-edges, T-quads with their sides, th2sing) with the T-edge lengths within 1e-6
relative."""
import numpy as np
import pytest

import metriko_gb300 as M
from oracle import metriko_oracle as O

from test_tmesh import _corner_uv, harness, load_workload, oracle_graph, run_harness  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["ico3_noise", "genus2_s3", "icosphere_obj"])
def test_pipeline_motorcycle_graph_matches_oracle(gpu_ctx, harness, tmp_path, name):  # noqa: F811
    V, F, ratio, rs = load_workload(name)
    ref = O.pipeline(V, F, ratio=ratio, round_seams=rs, seamless=False, local_injectivity=True)
    _, ports, curves, tm = oracle_graph(ref, F)
    r = M.pipeline(gpu_ctx, V, F, ratio=ratio, round_seams=rs, seamless=False, local_injectivity=True,
                   opts=M.solve_opts("mixed", tol=1e-10))
    assert r["status"] == 0
    assert np.array_equal(r["singular"], ref["singular"])
    assert np.array_equal(r["matching"], ref["combed_matching"])
    uv = _corner_uv(r["cfn"], len(F))
    res = run_harness(harness, tmp_path, V, F, uv, r["matching"], r["singular"])
    assert "error" not in res, res.get("error")
    assert [(p[0], p[1], p[2], p[4], p[5], p[6]) for p in res["ports"]] == \
        [(p["id"], p["vert"], p["face"], p["dir"], p["next"], p["prev"]) for p in ports]
    assert [[(s[0], s[2], s[3], s[5], s[6]) for s in c] for c in res["curves"]] == \
        [[(s.face, s.fr.crash, s.fr.type, s.to.crash, s.to.type) for s in c.sgmts] for c in curves]
    assert res["tedges"] == [(ci, sfr.id, sto.id) for ci, sfr, sto in tm["tedges"]]
    assert res["tquads"] == [(list(t), list(s)) for t, s in tm["tquads"]]
    assert res["th2sing"] == tm["th2sing"]
    from oracle import tmesh_oracle as T
    np.testing.assert_allclose(res["R"], T.tedge_lengths(curves, tm), rtol=1e-6)
