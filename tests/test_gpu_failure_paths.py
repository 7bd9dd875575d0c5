"""Failure statuses of the device solvers, made on the host (no GPU fault, trap or hang).

* MTK_ERR_TIMEOUT: the context's grid-barrier wait limit is set to 0 polls, so the first CTA
  that finds a barrier of the persistent PCG kernel still closed gives up at once; the kernel
  leaves its loops and the call returns TIMEOUT.  The same context then solves normally with
  the default limit (nothing is left stuck on the device).
* MTK_ERR_BREAKDOWN: a NaN in the right-hand side of the field solve (FP64 and mixed).
"""
import numpy as np
import pytest

import metriko_gb300 as M
from metriko_gb300 import meshgen
from oracle import metriko_oracle as O

pytestmark = pytest.mark.gpu


def _inputs(name):
    V, F, _, _ = meshgen.workload(name)
    m = O.Hmesh(V, F)
    nbr = m.face[m.twin[m.FH]].astype(np.int32)
    theta = m.farg[m.FH] - m.farg[m.twin[m.FH]]
    return m, nbr, theta


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_barrier_wait_limit_reports_timeout_and_context_recovers(prec):
    m, nbr, theta = _inputs("ico4_noise")
    x0 = O.seeded_init(m.nF, 0)
    with M.Context(0) as ctx:
        ref, _ = M.field_smoothest(ctx, nbr, theta, m.faceArea, x0, opts=M.solve_opts(prec, tol=1e-10))
        ctx.set_wait_limit(0)
        with pytest.raises(M.MetrikoError) as e:
            M.field_smoothest(ctx, nbr, theta, m.faceArea, x0, opts=M.solve_opts(prec, tol=1e-10))
        assert e.value.status == M._lib.TIMEOUT
        ctx.set_wait_limit(1 << 24)
        again, _ = M.field_smoothest(ctx, nbr, theta, m.faceArea, x0, opts=M.solve_opts(prec, tol=1e-10))
    assert np.array_equal(again, ref)


def test_pipeline_reports_timeout():
    V, F, ratio, rs = meshgen.workload("ico3_noise")
    with M.Context(0) as ctx:
        ctx.set_wait_limit(0)
        r = M.pipeline(ctx, V, F, ratio=ratio, round_seams=rs, check=False)
        assert r["status"] == M._lib.TIMEOUT
        ctx.set_wait_limit(1 << 24)
        r = M.pipeline(ctx, V, F, ratio=ratio, round_seams=rs)
        assert r["status"] == 0


def test_wait_limit_rejects_negative():
    with M.Context(0) as ctx:
        with pytest.raises(M.MetrikoError) as e:
            ctx.set_wait_limit(-1)
        assert e.value.status == M._lib.BAD_INPUT


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_nan_right_hand_side_reports_breakdown(gpu_ctx, prec):
    m, nbr, theta = _inputs("ico3_noise")
    rhs = O.seeded_init(m.nF, 2)
    rhs[17] = complex(np.nan, 0.0)
    with pytest.raises(M.MetrikoError) as e:
        M.field_solve(gpu_ctx, nbr, theta, m.faceArea, rhs, opts=M.solve_opts(prec, tol=1e-10))
    assert e.value.status == M._lib.BREAKDOWN
