"""Oracle restatement of the local-injectivity pieces (InjectiveBarrier, the orientation check)
against hand-computed values; no GPU."""
import numpy as np

from metriko_gb300 import meshgen
from oracle import metriko_oracle as O


def _face(v):   # one face, N = 4 vectors
    return np.asarray(v, float).reshape(-1)


def test_barrier_known_values():
    F2 = _face([[1, 0], [0, 1], [-1, 0], [0, -1]])          # orthonormal: V = 1 for every pair
    # pair (0,1): r = 0.3 -> q = 0.6, bar = 0.936, 1/bar - 1, d = 0.96, -d / bar^2
    # pair (1,2): r = cross((0, .3), (-1, 0)) = 0.3 as well; pair (2,3): cross((-1,0),(0,-2)) = 2
    # (>= s: 0); pair (3,0): cross((0,-2),(1,0)) = 2
    field = _face([[1, 0], [0, 0.3], [-1, 0], [0, -2]])
    fB, der, S = O.injective_barrier_update(F2, field)
    bar = 0.6 ** 3 - 3 * 0.6 ** 2 + 3 * 0.6
    assert np.isclose(fB[0], 1 / bar - 1, rtol=1e-14) and np.isclose(fB[1], 1 / bar - 1, rtol=1e-14)
    assert fB[2] == 0 and fB[3] == 0
    d = 3 * 0.09 / 0.125 - 6 * 0.3 / 0.25 + 6
    assert np.isclose(der[0], -d / bar ** 2, rtol=1e-13) and der[2] == 0
    assert np.allclose(S[0], [0.3, 0, 0, 1])                 # (v1.y, -v1.x, -v0.y, v0.x) / V


def test_barrier_flipped_and_saturated():
    F2 = _face([[2, 0], [0, 2], [-2, 0], [0, -2]])          # V = 4
    field = _face([[1, 0], [0, -1], [1, 0], [0, 1]])        # r: -0.25, 0.25, 0.25, -0.25
    fB, der, _ = O.injective_barrier_update(F2, field)
    assert np.isinf(fB[0]) and np.isinf(fB[3]) and np.isinf(der[0])
    assert np.isfinite(fB[1]) and fB[1] > 0 and der[1] < 0
    fB2, der2, S2 = O.injective_barrier_update(F2, field, update_j=False)
    assert der2 is None and S2 is None and np.array_equal(np.isinf(fB2), np.isinf(fB))


def test_orientation_check_and_corner_order():
    V, F, _, _ = meshgen.workload("ico2_noise")
    m = O.Hmesh(V, F)
    # the corners of locally_injectivity_check (tails of f.half(), next, prev) are F[f, 0..2]
    h = m.face2half
    assert np.array_equal(m.tail[h], F[:, 0]) and np.array_equal(m.tail[m.next[h]], F[:, 1])
    assert np.array_equal(m.tail[m.prev[h]], F[:, 2])
    # a planar map of the sphere's faces by their own face frames is orientation preserving
    P = np.asarray(V, float)
    cfn = np.zeros((len(F), 3, 4))
    for j in range(3):
        e = P[F[:, j]] - P[F[:, 0]]
        cfn[:, j, 0] = np.einsum("ij,ij->i", e, m.faceBasisX)
        cfn[:, j, 1] = np.einsum("ij,ij->i", e, m.faceBasisY)
    assert O.locally_injective(cfn) == (0, len(F))
    cfn[7, 1, :2], cfn[7, 2, :2] = cfn[7, 2, :2].copy(), cfn[7, 1, :2].copy()   # plant one flip
    cfn[11, 1, :2], cfn[11, 2, :2] = cfn[11, 2, :2].copy(), cfn[11, 1, :2].copy()
    assert O.locally_injective(cfn) == (2, 7)


def _si_barrier(out):
    si = out["info"]["si"]
    fB, _, _ = O.injective_barrier_update(out["F2"], si.X2F @ si.xCurr)
    return fB


def test_local_injectivity_path_matches_plain_when_inactive():
    """localInjectivity = true with the barrier inactive everywhere: the damped LMs converge to the
    undamped solutions (same fixes, the same map to round-off) and the map is locally injective."""
    V, F, ratio, rs = meshgen.workload("ico2_noise")
    a = O.pipeline(V, F, ratio=ratio, round_seams=rs)
    b = O.pipeline(V, F, ratio=ratio, round_seams=rs, local_injectivity=True)
    assert a["success"] and b["success"]
    assert b["info"]["fix_order"] == a["info"]["fix_order"]
    span = a["fullx"].max() - a["fullx"].min()
    assert np.abs(b["fullx"] - a["fullx"]).max() <= 1e-6 * span
    assert O.locally_injective(b["cfn"])[0] == 0
    assert (_si_barrier(a) == 0).all()


def test_local_injectivity_path_with_active_barrier():
    """A coarse grid (ratio 0.15) compresses the map next to the singularities: barrier rows are
    active (0 < r < 1/2) in the plain result; the local-injectivity path rounds successfully to a
    locally injective map with a finite barrier."""
    V, F, _, rs = meshgen.workload("ico3_noise")
    a = O.pipeline(V, F, ratio=0.15, round_seams=rs)
    fa = _si_barrier(a)
    assert ((fa > 0) & np.isfinite(fa)).any()
    b = O.pipeline(V, F, ratio=0.15, round_seams=rs, local_injectivity=True)
    assert b["success"]
    assert O.locally_injective(b["cfn"])[0] == 0
    assert np.isfinite(_si_barrier(b)).all()
