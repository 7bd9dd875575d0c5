"""The allocation-free field entry point (mtk_field_smoothest_noalloc).

It serves callers that cannot call cudaMalloc -- code inside a framework that owns all device
memory, or code that must not allocate after start-up: they pass their own device buffers and
the library works in a static device array.  This test calls it through the C ABI on device
buffers (allocated here by torch, standing in for the caller's allocator) and checks it against
mtk_field_smoothest, the regular entry point, and against the oracle's direct-solve inverse
iteration, on two calls in a row: the second call reuses the scratch array left by the first.  Tolerance as for the field parity tests: per-face field angle
within 1e-5 rad and the Dirichlet energy within 1e-6 relative.  The file is named so pytest
collects it last.
"""
import ctypes as C

import numpy as np
import pytest

import metriko_gb300 as M
from metriko_gb300 import meshgen
from oracle import metriko_oracle as O

pytestmark = pytest.mark.gpu


def _inputs(name):
    V, F, _, _ = meshgen.workload(name)
    m = O.Hmesh(V, F)
    nbr = m.face[m.twin[m.FH]].astype(np.int32)        # -1 on a boundary side
    theta = np.where(nbr >= 0, m.farg[m.FH] - m.farg[m.twin[m.FH]], 0.0)
    return m, nbr, theta


def _noalloc(torch, nbr, theta, area, x0, n_iter, tol, max_iter):
    dev = torch.device("cuda", 0)
    d_nbr = torch.from_numpy(np.ascontiguousarray(nbr.reshape(-1))).to(dev)
    d_theta = torch.from_numpy(np.ascontiguousarray(theta.reshape(-1))).to(dev)
    d_area = torch.from_numpy(np.ascontiguousarray(area)).to(dev)
    x = np.empty(2 * len(area))
    x[0::2], x[1::2] = x0.real, x0.imag
    d_x0 = torch.from_numpy(x).to(dev)
    d_out = torch.zeros(2 * len(area), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    torch.cuda.synchronize(dev)
    iters = C.c_int32(0)
    status = M.lib().mtk_field_smoothest_noalloc(len(area), 4, d_nbr.data_ptr(), d_theta.data_ptr(), d_area.data_ptr(),
                                                 d_x0.data_ptr(), n_iter, tol, max_iter, d_out.data_ptr(),
                                                 C.c_void_p(stream.cuda_stream), C.byref(iters))
    out = d_out.cpu().numpy()
    return status, out[0::2] + 1j * out[1::2], iters.value


def test_noalloc_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    m, nbr, theta = _inputs("ico4_noise")
    x0 = O.seeded_init(m.nF, 0)
    L = O.connection_laplacian(m, 4)
    with M.Context(0) as ctx:
        ref, _ = M.field_smoothest(ctx, nbr, theta, m.faceArea, x0, opts=M.solve_opts("fp64", tol=1e-10))
    e_ref = np.vdot(ref, L @ ref).real
    # the oracle: 50 inverse power steps with direct solves from the same start vector
    orc = O.smallest_eig(L, O.mass_matrix(m), x0, 50)
    e_orc = np.vdot(orc, L @ orc).real
    for _ in range(2):
        status, c, iters = _noalloc(torch, nbr, theta, m.faceArea, x0, 50, 1e-10, 50000)
        assert status == 0, M.lib().mtk_last_error().decode()
        assert iters > 0
        assert np.abs(np.angle(c / ref)).max() / 4 < 1e-5
        assert abs(np.vdot(c, L @ c).real - e_ref) / e_ref < 1e-6
        assert np.abs(np.angle(c / orc)).max() / 4 < 1e-5
        assert abs(np.vdot(c, L @ c).real - e_orc) / e_orc < 1e-6


def test_noalloc_open_mesh_matches_regular_entry_point():
    """A disk-shaped mesh: boundary sides (nbr -1) give rows with fewer neighbours, the same
    operator as the regular entry point and the oracle."""
    torch = pytest.importorskip("torch")
    m, nbr, theta = _inputs("cap4_sh8")
    assert (nbr == -1).any()
    x0 = O.seeded_init(m.nF, 2)
    L = O.connection_laplacian(m, 4)
    with M.Context(0) as ctx:
        ref, _ = M.field_smoothest(ctx, nbr, theta, m.faceArea, x0, opts=M.solve_opts("fp64", tol=1e-10))
    orc = O.smallest_eig(L, O.mass_matrix(m), x0, 50)
    for _ in range(2):
        status, c, iters = _noalloc(torch, nbr, theta, m.faceArea, x0, 50, 1e-10, 50000)
        assert status == 0, M.lib().mtk_last_error().decode()
        assert np.abs(np.angle(c / ref)).max() / 4 < 1e-5
        assert np.abs(np.angle(c / orc)).max() / 4 < 1e-5
        e, e_orc = np.vdot(c, L @ c).real, np.vdot(orc, L @ orc).real
        assert abs(e - e_orc) / e_orc < 1e-6


def test_noalloc_failure_statuses():
    """An inner solve capped at one iteration reports NOT_CONVERGED; a neighbour index outside
    [0, nF) other than -1 (-1 marks a boundary side), or a face's own index, is rejected on the
    device with BAD_INPUT and no solve; n_iter = 0 returns the start vector.  A good call
    afterwards still succeeds, so no state from the failed calls is left in the shared scratch
    array."""
    torch = pytest.importorskip("torch")
    m, nbr, theta = _inputs("ico3_noise")
    x0 = O.seeded_init(m.nF, 1)
    status, _, iters = _noalloc(torch, nbr, theta, m.faceArea, x0, 50, 1e-12, 1)
    assert status == M._lib.NOT_CONVERGED
    assert iters == 1
    bad = nbr.copy()
    bad[7, 1] = -2
    status, _, iters = _noalloc(torch, bad, theta, m.faceArea, x0, 50, 1e-10, 50000)
    assert status == M._lib.BAD_INPUT
    assert iters == 0
    assert "neighbour" in M.lib().mtk_last_error().decode()
    for v in (m.nF, 7):
        bad[7, 1] = v
        status, _, _ = _noalloc(torch, bad, theta, m.faceArea, x0, 50, 1e-10, 50000)
        assert status == M._lib.BAD_INPUT
    status, c, iters = _noalloc(torch, nbr, theta, m.faceArea, x0, 0, 1e-10, 50000)
    assert status == 0 and iters == 0
    assert np.array_equal(c, x0)
    status, c, iters = _noalloc(torch, nbr, theta, m.faceArea, x0, 50, 1e-10, 50000)
    assert status == 0 and iters > 0
    orc = O.smallest_eig(O.connection_laplacian(m, 4), O.mass_matrix(m), x0, 50)
    assert np.abs(np.angle(c / orc)).max() / 4 < 1e-5


def test_noalloc_rejects_sizes_beyond_its_scratch():
    status = M.lib().mtk_field_smoothest_noalloc(409601, 4, C.c_void_p(8), C.c_void_p(8), C.c_void_p(8), C.c_void_p(8),
                                                 50, 1e-8, 100, C.c_void_p(8), None, None)
    assert status == M._lib.BAD_INPUT
    assert "409600" in M.lib().mtk_last_error().decode()
