"""Size-field and vertex-position gradients on the GPU (adjoint solves + assembly backward):
against the oracle's direct-solve gradients, and through torch.autograd.Functions against FP64
central finite differences on random directions."""
import numpy as np
import pytest

import metriko_gb300 as M
import oracle.metriko_oracle as O
from metriko_gb300 import meshgen

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

TIGHT = dict(prec="fp64", tol=1e-12)


def _opts():
    return M.solve_opts(TIGHT["prec"], tol=TIGHT["tol"])


@pytest.mark.parametrize("name", ["ico3_noise", "torus_32x16", "cap3_noise"])
@pytest.mark.parametrize("target", ["integration", "perturbed"])
def test_size_field_gradient_matches_oracle(gpu_ctx, name, target):
    V, F, ratio, rs = meshgen.workload(name)
    out = O.pipeline(V, F, ratio=ratio, seamless=False, round_seams=rs)
    rng = np.random.default_rng(3)
    s = rng.normal(0, 0.2, len(V))
    T = None if target == "integration" else out["F2"] * (1 + 0.3 * rng.normal(size=out["F2"].shape))
    l_ref, g_ref, x_ref = O.size_field_gradient(out, F, s, T, mu=0.1)
    r = M.size_field_gradient(gpu_ctx, V, F, s, T=T, mu=0.1, ratio=ratio, round_seams=rs, opts=_opts())
    assert abs(r["loss"] - l_ref) <= 1e-8 * abs(l_ref)
    assert np.linalg.norm(r["grad"] - g_ref) <= 1e-6 * np.linalg.norm(g_ref)
    assert np.abs(r["fullx"] - x_ref).max() <= 1e-8 * np.abs(x_ref).max()


class SizeFieldLoss(torch.autograd.Function):
    """l(s) through the library; the gradient comes from the same call (adjoint solve), so
    backward only scales it: nothing of the forward solve is stored."""

    @staticmethod
    def forward(ctx, s, mesh, T, mu):
        V, F, ratio, gctx = mesh
        r = M.size_field_gradient(gctx, V, F, s.detach().cpu().double().numpy(), T=T, mu=mu, ratio=ratio,
                                  opts=_opts())
        ctx.save_for_backward(torch.from_numpy(r["grad"]).to(s.dtype))
        return torch.tensor(r["loss"], dtype=torch.float64)

    @staticmethod
    def backward(ctx, gout):
        (g,) = ctx.saved_tensors
        return gout.to(g.dtype) * g, None, None, None


def _fd_check(gpu_ctx, name, sigma, ndir, seed):
    V, F, ratio, _ = meshgen.workload(name)
    rng = np.random.default_rng(seed)
    s = torch.tensor(rng.normal(0, sigma, len(V)), dtype=torch.float64, requires_grad=True)
    mesh = (V, F, ratio, gpu_ctx)
    loss = SizeFieldLoss.apply(s, mesh, None, 0.1)
    loss.backward()
    g = s.grad.numpy()
    assert np.all(np.isfinite(g)) and np.linalg.norm(g) > 0
    h = 1e-4
    s0 = s.detach().numpy()
    for _ in range(ndir):
        d = rng.normal(size=len(V))
        lp = M.size_field_gradient(gpu_ctx, V, F, s0 + h * d, mu=0.1, ratio=ratio, opts=_opts())["loss"]
        lm = M.size_field_gradient(gpu_ctx, V, F, s0 - h * d, mu=0.1, ratio=ratio, opts=_opts())["loss"]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g @ d) <= 1e-5 * max(abs(fd), abs(g @ d), 1.0), (fd, g @ d)


def test_size_field_autograd_finite_differences_small(gpu_ctx):
    """Level-4 sphere (5,120 faces), 16 random directions."""
    _fd_check(gpu_ctx, "ico4_noise", 0.2, 16, 11)


def test_size_field_autograd_finite_differences_level7(gpu_ctx):
    """Differentiation workload: level-7 displaced sphere (327,680 faces), s ~ N(0, 0.2), 16 random
    directions."""
    _fd_check(gpu_ctx, "ico7_sh8", 0.2, 16, 12)


def test_size_field_gradient_level9(gpu_ctx):
    """Large workload: level-9 sphere (5,242,880 faces), s ~ N(0, 0.1), forward + adjoint
    gradient, one finite-difference direction."""
    _fd_check(gpu_ctx, "ico9_sh16", 0.1, 1, 13)


# ------------------------------------------------------------------------- vertex positions
def test_face_geometry_backward_matches_complex_step(gpu_ctx):
    """The per-face dual-number backward against the oracle's complex-step Jacobian of the same
    per-face formulas (area, halfedge angles, G2 entries), gathered to the vertices."""
    V, F, _, _ = meshgen.workload("ico3_noise")
    rng = np.random.default_rng(21)
    nF = len(F)
    gA, g1, g2 = rng.normal(size=nF), rng.normal(size=nF), rng.normal(size=nF)
    gx, gy = rng.normal(size=(nF, 3)), rng.normal(size=(nF, 3))
    _, J = O._face_geom_jacobian(V, F)
    gface = (gA[:, None] * J["A"] + g1[:, None] * J["f1"] + g2[:, None] * J["f2"]
             + np.einsum("fa,fqa->fq", gx, J["gx"]) + np.einsum("fa,fqa->fq", gy, J["gy"]))
    ref = np.zeros((len(V), 3))
    for c in range(3):
        np.add.at(ref, F[:, c], gface[:, 3 * c:3 * c + 3])
    got = M.face_geometry_backward(gpu_ctx, V, F, gA, g1, g2, gx, gy)
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()


@pytest.mark.parametrize("name", ["ico3_noise", "torus_32x16", "cap3_noise"])
def test_position_gradient_matches_oracle(gpu_ctx, name):
    """dl/dV (integration target, integer decisions frozen): GPU reverse power iteration, face
    partials and geometry backward against the oracle (direct solves, complex-step geometry).
    cap3_noise is an open disk: a boundary side carries no transport angle."""
    V, F, ratio, rs = meshgen.workload(name)
    rng = np.random.default_rng(4)
    s = rng.normal(0, 0.2, len(V))
    l_ref, gs_ref, gV_ref, _, _ = O.position_gradient(V, F, s, mu=0.1, ratio=ratio, round_seams=rs)
    r = M.position_gradient(gpu_ctx, V, F, s, mu=0.1, ratio=ratio, round_seams=rs, opts=_opts())
    assert abs(r["loss"] - l_ref) <= 1e-8 * abs(l_ref)
    assert np.linalg.norm(r["grad_s"] - gs_ref) <= 1e-6 * np.linalg.norm(gs_ref)
    assert np.linalg.norm(r["grad_V"] - gV_ref) <= 1e-6 * np.linalg.norm(gV_ref)


class PositionLoss(torch.autograd.Function):
    """l(V) through the library; backward scales the gradient the same call returned."""

    @staticmethod
    def forward(ctx, Vt, F, s, ratio, gctx):
        r = M.position_gradient(gctx, Vt.detach().cpu().double().numpy(), F, s, mu=0.1, ratio=ratio, opts=_opts())
        ctx.save_for_backward(torch.from_numpy(r["grad_V"]).to(Vt.dtype))
        return torch.tensor(r["loss"], dtype=torch.float64)

    @staticmethod
    def backward(ctx, gout):
        (g,) = ctx.saved_tensors
        return gout.to(g.dtype) * g, None, None, None, None


def _topology(gpu_ctx, V, F, ratio):
    r = M.pipeline(gpu_ctx, V, F, ratio=ratio, stop_after=2, opts=_opts())
    return r["singular"].copy(), r["seam"].copy(), r["matching"].copy()


def _position_fd_check(gpu_ctx, name, ndir, h, rtol, seed):
    V, F, ratio, _ = meshgen.workload(name)
    rng = np.random.default_rng(seed)
    s = rng.normal(0, 0.2, len(V))
    Vt = torch.tensor(V, dtype=torch.float64, requires_grad=True)
    loss = PositionLoss.apply(Vt, F, s, ratio, gpu_ctx)
    loss.backward()
    g = Vt.grad.numpy()
    assert np.all(np.isfinite(g)) and np.linalg.norm(g) > 0
    base = _topology(gpu_ctx, V, F, ratio)
    checked = 0
    for _ in range(ndir):
        d = rng.normal(size=V.shape)
        d /= np.linalg.norm(d)
        Vp, Vm = V + h * d, V - h * d
        if not all(np.array_equal(a, b) for W in (Vp, Vm) for a, b in zip(_topology(gpu_ctx, W, F, ratio), base)):
            continue
        # central differences at h and h/2, Richardson-combined (the field's near-degenerate
        # eigenvalue cluster makes the loss strongly curved in V)
        def central(t):
            lp = M.size_field_gradient(gpu_ctx, V + t * d, F, s, mu=0.1, ratio=ratio, opts=_opts())["loss"]
            lm = M.size_field_gradient(gpu_ctx, V - t * d, F, s, mu=0.1, ratio=ratio, opts=_opts())["loss"]
            return (lp - lm) / (2 * t)
        f1, f2 = central(h), central(h / 2)
        fd = f2 + (f2 - f1) / 3.0
        an = float(np.sum(g * d))
        assert abs(fd - an) <= rtol * max(abs(fd), abs(an), 1e-3 * np.linalg.norm(g)), (fd, an)
        checked += 1
    assert checked >= (3 * ndir) // 4


def test_position_autograd_finite_differences_small(gpu_ctx):
    """Level-3 sphere (1,280 faces), 16 random directions that keep every integer decision."""
    _position_fd_check(gpu_ctx, "ico3_noise", 16, 3e-6, 1e-5, 31)


def test_position_autograd_finite_differences_level7(gpu_ctx):
    """Differentiation workload: level-7 displaced sphere (327,680 faces), s ~ N(0, 0.2), 16 random
    directions that keep every integer decision."""
    _position_fd_check(gpu_ctx, "ico7_sh8", 16, 4e-5, 1e-4, 32)
