"""The FP64 oracle: invariants the reference guarantees, known answers of its building blocks,
and the committed golden fixtures (tests/golden, made by make_golden.py)."""
from pathlib import Path

import numpy as np
import pytest
import scipy.linalg as sla
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from metriko_gb300 import meshgen
from oracle import metriko_oracle as O

from conftest import oracle_run

GOLDEN = Path(__file__).parent / "golden"


def test_edge_topology_conventions():
    V, F = meshgen.icosphere(2)
    EV, FE, EF = O.edge_topology(F)
    assert len(EV) == 30 * 4 ** 2
    # sorted by (min, max); EF[e,0] runs min -> max
    key = EV[:, 0] * len(V) + EV[:, 1]
    assert np.all(np.diff(key) > 0)
    for e in range(len(EV)):
        f0 = EF[e, 0]
        row = list(F[f0])
        assert any(row[j] == EV[e, 0] and row[(j + 1) % 3] == EV[e, 1] for j in range(3))
    for f in range(len(F)):
        for j in range(3):
            e = FE[f, j]
            assert set(EV[e]) == {F[f, j], F[f, (j + 1) % 3]}


def test_halfedge_invariants():
    V, F = meshgen.icosphere(3)
    m = O.Hmesh(V, F)
    h = np.arange(m.nH)
    assert np.array_equal(m.next[m.next[m.next[h]]], h)
    assert np.array_equal(m.twin[m.twin[h]], h)
    assert np.array_equal(m.face[m.next[h]], m.face[h])
    assert np.array_equal(m.tail[m.twin[h]], m.head[h])
    assert np.array_equal(m.tail[m.face2half], F[:, 0])
    assert np.array_equal(m.tail[m.vert2half], np.arange(m.nV))
    # Gauss-Bonnet on the sphere
    assert abs(m.angleDefect.sum() - 4 * np.pi) < 1e-9


@pytest.mark.parametrize("g,s", [(1, 2), (2, 3), (3, 2)])
def test_holed_slab_is_a_closed_oriented_genus_g_surface(g, s):
    V, F = meshgen.holed_slab(g, s)
    m = O.Hmesh(V, F)                        # raises on boundary or non-manifold edges
    assert m.nV - m.nE + m.nF == 2 - 2 * g
    assert abs(m.angleDefect.sum() - 2 * np.pi * (2 - 2 * g)) < 1e-9   # Gauss-Bonnet
    a, b, c = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    vol = np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6
    assert abs(vol - ((2 * g + 1) * 3 - g)) < 0.05 * ((2 * g + 1) * 3 - g)   # outward, voxel volume


@pytest.mark.parametrize("name,chi", [("ico2_noise", 2), ("ico3_noise", 2), ("ico4_noise", 2), ("torus_32x16", 0),
                                      ("genus2_s3", -2), ("genus3_s2", -4)])
def test_singularity_index_sum(name, chi):
    """sum_v singular[v] = N * chi (face_rosy_field.h:100-107)."""
    V, F, ratio, rs = meshgen.workload(name)
    out = O.pipeline(V, F, ratio=ratio, stop_after="field")
    assert out["singular"].sum() == 4 * chi


def test_connection_laplacian_hermitian_pd():
    V, F, _, _ = meshgen.workload("ico3_noise")
    m = O.Hmesh(V, F)
    L = O.connection_laplacian(m, 4)
    assert abs(L - L.conj().T).max() < 1e-14
    lam = spla.eigsh(L, k=1, sigma=0, which="LM", return_eigenvectors=False)
    assert lam.min() > 0
    assert np.allclose(L.diagonal().real, 3 + 1e-9)


def test_field_is_in_the_lowest_eigen_cluster():
    """50 inverse iterations (sparse_linear_solver.h:29-54) land in the lowest cluster of
    L c = lambda M c.  On a sphere that cluster is nearly degenerate (9 eigenvalues within a
    few percent), so the iterate is not the single smallest eigenvector: its direction inside
    the cluster is set by the start vector, which is why the start is seeded."""
    V, F, _, _ = meshgen.workload("ico3_noise")
    m, L, M, c, field = O.run_field(V, F)
    rq = (np.vdot(c, L @ c) / np.vdot(c, M @ c)).real
    lam = np.sort(spla.eigsh(L, k=10, M=M, sigma=0, which="LM", return_eigenvectors=False))
    assert lam[0] <= rq <= lam[8] * (1 + 1e-9)
    assert lam[8] / lam[0] < 1.2 and lam[9] / lam[0] > 1.5
    assert abs(np.vdot(c, M @ c).real - 1) < 1e-12
    assert np.allclose(np.abs(field), 1)


def test_fullpiv_kernel_known_answer():
    A = np.array([[1.0, 2, 0, -1], [0, 1, 1, 0]])
    K = O.fullpiv_kernel(A)
    assert K.shape == (4, 2)
    assert np.abs(A @ K).max() < 1e-14
    # pivots by complete pivoting: |2| at (0,1) first, then the trailing block
    free = [i for i in range(4) if np.count_nonzero(K[i]) == 1 and np.abs(K[i]).max() == 1]
    assert len(free) >= 2
    assert np.linalg.matrix_rank(K) == 2
    R = np.random.default_rng(0).integers(-2, 3, size=(5, 9)).astype(float)
    K = O.fullpiv_kernel(R)
    assert K.shape[1] == 9 - np.linalg.matrix_rank(R)
    assert np.abs(R @ K).max() < 1e-12
    assert K.shape[1] == sla.null_space(R).shape[1]


def test_independent_rows():
    C = np.array([[1.0, 0, 1], [2, 0, 2], [0, 1, 0], [1, 1, 1]])
    assert list(O.independent_rows(C)) == [0, 2]
    S = O.structural_product(sp.csr_matrix([[1.0, 1.0]]), sp.csr_matrix([[1.0], [-1.0]]))
    assert S.nnz == 1 and S.data[0] == 0.0   # cancelled entry kept as a structural zero


@pytest.mark.parametrize("name", ["ico2_noise", "ico3_noise", "torus_32x16", "genus2_s3"])
def test_rounding_integrality_and_success(name):
    V, F, ratio, rs, out = oracle_run(name)
    assert out["success"]
    info = out["info"]
    X = out["fullx"]
    fixed = np.asarray(info["fix_order"])
    assert len(fixed) > 0
    assert np.abs(X[fixed] - O.cround(X[fixed])).max() <= 1e-6
    assert np.array_equal(O.cround(X[fixed]).astype(int), np.asarray(info["fix_vals"]))


@pytest.mark.parametrize("name", ["ico2_noise", "ico3_noise", "torus_32x16", "genus2_s3", "cap3_noise", "cap4_sh8",
                                  "cyl_32x12"])
def test_oracle_reproduces_golden(name):
    g = np.load(GOLDEN / f"{name}.npz")
    V, F, ratio, rs, out = oracle_run(name)
    assert np.array_equal(V, g["V"]) and np.array_equal(F, g["F"])
    assert np.array_equal(out["singular"], g["singular"])
    assert np.array_equal(out["seam"], np.unpackbits(g["seam"])[: int(g["n_edges"])].astype(bool))
    assert np.array_equal(out["combed_matching"], g["combed_matching"])
    assert np.array_equal(out["cutF"], g["cutF"])
    assert list(out["info"]["fix_order"]) == list(g["fix_order"])
    assert list(out["info"]["fix_vals"]) == list(g["fix_vals"])
    assert np.abs(out["compressed"] - g["compressed"]).max() < 1e-9
    assert np.abs(out["fullx"] - g["fullx"]).max() < 1e-6


@pytest.mark.parametrize("name", ["ico2_noise", "ico3_noise", "torus_32x16", "genus2_s3"])
def test_tie_window_matches_strict_order_up_to_roundoff_ties(name):
    """The greedy rounding counts distances <= 1e-6 as 0 and takes the first position among
    candidates within TIE_WINDOW (1e-8) of the smallest distance; the reference keeps the first
    strict '<' minimum (iter_rounding_loop.h:34-38).  Run both ways, the two give the same fixed (index, value)
    pairs, the same number of re-solves and the same map; every step whose pick differs is a
    tie of a few 1e-9 at most (round-off between constraint-linked or already-integral values)."""
    V, F, ratio, rs, out = oracle_run(name)
    strict = O.pipeline(V, F, ratio=ratio, round_seams=rs, tie_window=0.0)
    a, b = out["info"], strict["info"]
    assert sorted(zip(a["fix_order"], a["fix_vals"])) == sorted(zip(b["fix_order"], b["fix_vals"]))
    assert a["resolves"] == b["resolves"]
    diag = np.ptp(out["fullx"]) * np.sqrt(2.0)
    assert np.abs(out["fullx"] - strict["fullx"]).max() <= 1e-9 * diag
    # fractional ties: round-off between constraint-linked values; already-integral picks
    # (distance <= 1e-6, no re-solve) differ by the O(1 / penalty) residuals
    assert all(gap <= 5e-9 for _, gap, dp in a["strict_differs"] if dp > 1e-6)
    assert all(dp <= 1e-6 + 5e-9 for _, gap, dp in a["strict_differs"] if gap > 5e-9)
    assert b["strict_differs"] == []
    # the margin to the best candidate outside a tie group is far above the window
    assert min(a["margins"]) > 1e-5


def test_oracle_reproduces_reference_model_golden():
    """The reference's own model (example/models/icosphere.obj, level-4 icosphere) with the
    level-4 workload's radial noise: the fixture stores the displaced mesh."""
    g = np.load(GOLDEN / "icosphere_obj.npz")
    V, F = g["V"], g["F"]
    assert V.shape == (2562, 3) and F.shape == (5120, 3)
    out = O.pipeline(V, F, ratio=float(g["ratio"]), round_seams=bool(g["round_seams"]))
    assert out["success"]
    assert out["singular"].sum() == 8
    assert np.array_equal(out["singular"], g["singular"])
    assert np.array_equal(out["seam"], np.unpackbits(g["seam"])[: int(g["n_edges"])].astype(bool))
    assert np.array_equal(out["combed_matching"], g["combed_matching"])
    assert list(out["info"]["fix_order"]) == list(g["fix_order"])
    assert list(out["info"]["fix_vals"]) == list(g["fix_vals"])
    assert np.abs(out["fullx"] - g["fullx"]).max() < 1e-6


@pytest.mark.parametrize("name", ["ico5_sh8", "ico6_sh8", "ico7_sh8"])
def test_large_golden_meshes_regenerate(name):
    """The large fixtures keep no mesh: the seeded generator must still produce it."""
    g = np.load(GOLDEN / f"{name}.npz")
    V, F, ratio, rs = meshgen.workload(name)
    assert len(V) == int(g["nV"]) and len(F) == int(g["nF"])
    assert np.abs(V[g["v_sample_idx"]] - g["v_sample"]).max() <= 1e-12
    assert float(g["ratio"]) == ratio and bool(g["round_seams"]) == rs
    assert int(g["singular"].astype(int).sum()) == 8
    X = g["fullx_fixed"]
    assert np.abs(X - np.round(X)).max() <= 1e-6
    assert np.array_equal(np.round(X).astype(int), g["fix_vals"])


def test_oracle_reproduces_large_golden():
    """The level-5 fixture (20,480 faces, about 20 s of oracle time) is re-derived on the CPU;
    the level-6 and level-7 ones take minutes and are regenerated by make_golden.py only."""
    g = np.load(GOLDEN / "ico5_sh8.npz")
    V, F, ratio, rs = meshgen.workload("ico5_sh8")
    out = O.pipeline(V, F, ratio=ratio, round_seams=rs)
    assert np.array_equal(out["singular"], g["singular"].astype(int))
    assert np.array_equal(out["seam"], np.unpackbits(g["seam"])[: int(g["n_edges"])].astype(bool))
    assert np.array_equal(out["combed_matching"], g["combed_matching"].astype(int))
    assert list(out["info"]["fix_order"]) == list(g["fix_order"])
    assert list(out["info"]["fix_vals"]) == list(g["fix_vals"])
    assert np.abs(out["fullx"][g["x_sample_idx"]] - g["fullx_sample"]).max() < 1e-6
