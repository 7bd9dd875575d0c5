"""Curl matching and singular indices on the device (mtk_curl_matching) against the oracle's
computeConnection / cMatching / computeSingular (face_rosy_field.h:100-202): integer outputs,
identical.  On the golden fixtures (their stored field), on seeded fields, and at the 1.3M-face
benchmark size on the field the GPU solves, where the host C++ path of mtk_topology_from_field
gives the singular indices to compare."""
from pathlib import Path

import numpy as np
import pytest

import metriko_gb300 as M
from metriko_gb300 import meshgen
from oracle import metriko_oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).parent / "golden"


def _oracle(m, c, N=4):
    fld = O.rosy_from_compressed(c, N)
    conn = O.compute_connection(m)
    iM, effort = O.c_matching(m, fld, conn, N)
    return iM, O.compute_singular(m, effort, N)


def _device(ctx, m, c, N=4):
    return M.curl_matching(ctx, m.pos, m.idx, m.edge2vert, m.edge2face, m.vert2half, m.prev, m.angleDefect, c, N=N)


@pytest.mark.parametrize("name", ["ico2_noise", "ico3_noise", "torus_32x16", "genus2_s3", "icosphere_obj"])
def test_curl_matching_golden_field(gpu_ctx, name):
    g = np.load(GOLDEN / f"{name}.npz")
    m = O.Hmesh(g["V"], g["F"])
    c = g["compressed"]
    match, sing = _device(gpu_ctx, m, c)
    ref_match, ref_sing = _oracle(m, c)
    assert np.array_equal(match, ref_match)
    assert np.array_equal(sing, ref_sing)
    assert np.array_equal(sing, g["singular"])


@pytest.mark.parametrize("N", [1, 2, 3, 4, 6])
@pytest.mark.parametrize("seed", [0, 1])
def test_curl_matching_seeded_field(gpu_ctx, N, seed):
    """A rough field (seeded, not smooth): many edges with large efforts and every matching
    value; N other than 4 goes through the generic kernel."""
    V, F, _, _ = meshgen.workload("ico3_noise")
    m = O.Hmesh(V, F)
    c = O.seeded_init(m.nF, seed)
    match, sing = _device(gpu_ctx, m, c, N)
    ref_match, ref_sing = _oracle(m, c, N)
    assert np.array_equal(match, ref_match)
    assert np.array_equal(sing, ref_sing)


def test_curl_matching_sums_to_euler_characteristic(gpu_ctx):
    """Sum of singular indices = N * chi on a smooth field: 8 on the sphere, 0 on the torus."""
    for name, want in [("ico4_noise", 8), ("torus_64x32", 0)]:
        V, F, _, _ = meshgen.workload(name)
        m = O.Hmesh(V, F)
        nbr = m.face[m.twin[m.FH]].astype(np.int32)
        theta = m.farg[m.FH] - m.farg[m.twin[m.FH]]
        c, _ = M.field_smoothest(gpu_ctx, nbr, theta, m.faceArea, O.seeded_init(m.nF, 0))
        _, sing = _device(gpu_ctx, m, c)
        assert int(sing.sum()) == want


def test_curl_matching_benchmark_size(gpu_ctx):
    """1,310,720 faces / 1,966,080 edges: the device matching equals the oracle's on every edge
    and the device singular indices equal the host C++ loops' (mtk_topology_from_field)."""
    V, F, ratio, rs = meshgen.workload("ico8_sh8")
    m = O.Hmesh(V, F)
    nbr = m.face[m.twin[m.FH]].astype(np.int32)
    theta = m.farg[m.FH] - m.farg[m.twin[m.FH]]
    c, _ = M.field_smoothest(gpu_ctx, nbr, theta, m.faceArea, O.seeded_init(m.nF, 0))
    match, sing = _device(gpu_ctx, m, c)
    fld = O.rosy_from_compressed(c, 4)
    ref_match, _ = O.c_matching(m, fld, O.compute_connection(m), 4)
    assert np.array_equal(match, ref_match)
    host = M.topology_from_field(V, F, c, ratio=ratio, round_seams=rs)
    assert np.array_equal(sing, host["singular"])
    assert int(sing.sum()) == 8


def test_curl_matching_rejects_open_mesh(gpu_ctx):
    V, F, _, _ = meshgen.workload("ico2_noise")
    m = O.Hmesh(V, F)
    ef = m.edge2face.copy()
    ef[5, 1] = -1
    with pytest.raises(M.MetrikoError) as e:
        M.curl_matching(gpu_ctx, m.pos, m.idx, m.edge2vert, ef, m.vert2half, m.prev, m.angleDefect,
                        O.seeded_init(m.nF, 0))
    assert e.value.status == M._lib.BAD_INPUT


@pytest.mark.parametrize("name", ["ico3_noise", "torus_64x32", "ico6_sh8"])
def test_mesh_field_inputs_match_host(gpu_ctx, name):
    """Face pairing, halfedge-angle differences and areas from the raw mesh on the device equal
    the halfedge mesh's on the host: pairing and areas bit for bit, theta to the rounding of acos."""
    V, F, _, _ = meshgen.workload(name)
    nbr_h, theta_h, area_h = M.field_inputs(V, F)
    nbr_d, theta_d, area_d = M.mesh_field_inputs(gpu_ctx, V, F)
    assert np.array_equal(nbr_d.reshape(-1), np.asarray(nbr_h).reshape(-1))
    assert np.array_equal(area_d, np.asarray(area_h))
    assert np.abs(theta_d.reshape(-1) - np.asarray(theta_h).reshape(-1)).max() <= 1e-13


def test_field_smoothest_mesh_matches_face_graph_entry(gpu_ctx):
    V, F, _, _ = meshgen.workload("ico4_noise")
    nbr, theta, area = M.field_inputs(V, F)
    x0 = O.seeded_init(len(F), 0)
    opts = M.solve_opts("mixed", tol=1e-10)
    a, _ = M.field_smoothest(gpu_ctx, nbr, theta, area, x0, opts=opts)
    b, _ = M.field_smoothest_mesh(gpu_ctx, V, F, x0, opts=opts)
    assert np.abs(np.angle(a / b)).max() / 4 < 1e-7


@pytest.mark.parametrize("case", ["flipped", "duplicate", "degenerate"])
def test_mesh_field_inputs_rejects(gpu_ctx, case):
    """Faces of opposite orientation, an edge with a third face and a side with equal end points
    are rejected (an edge with one face is a boundary side: tests/test_gpu_open_mesh.py)."""
    V, F, _, _ = meshgen.workload("ico2_noise")
    F = np.array(F, np.int32)
    if case == "flipped":
        F[3] = F[3, ::-1]
    elif case == "duplicate":
        F = np.vstack([F, F[:1]])
    else:
        F[5, 1] = F[5, 0]
    with pytest.raises(M.MetrikoError) as e:
        M.mesh_field_inputs(gpu_ctx, V, F)
    assert e.value.status == M._lib.BAD_INPUT


def _seam_inputs(m):
    """The spanning cut (libigl's cut with an all-zero matching) and the vertex rings of the
    oracle's mesh: what mtk_seam_paths starts from."""
    TT, TTi = O.triangle_triangle_adjacency(m)
    cuts = O.cut_mesh_from_singularities_zero(m, TT, TTi)
    in_cut = np.zeros(m.nV, np.uint8)
    in_cut[m.idx[cuts]] = 1
    seam0 = np.zeros(m.nE, np.uint8)
    seam0[m.face2edge[cuts]] = 1
    vptr, vv, ve = [0], [], []
    for v in range(m.nV):
        ring = m.ccw(m.vert2half[v])
        vv += [int(m.head[h]) for h in ring]
        ve += [int(m.edge[h]) for h in ring]
        vptr.append(len(vv))
    return in_cut, seam0, np.array(vptr), np.array(vv), np.array(ve)


@pytest.mark.parametrize("name", ["ico3_noise", "torus_32x16", "genus2_s3", "cap4_sh8", "cyl_32x12", "ico5_sh8"])
def test_seam_paths_match_oracle(gpu_ctx, name):
    """The singularity-path searches on the device (one cooperative launch, one grid barrier per
    level) give the oracle's seam bit for bit: spheres, a torus, a genus-2 surface, an open disk
    and an open cylinder (whose boundary vertices, index 1, are sources already on the cut)."""
    V, F, ratio, rs = meshgen.workload(name)
    ref = O.pipeline(V, F, ratio=ratio, round_seams=rs, stop_after="field")
    m = ref["mesh"]
    in_cut, seam0, vptr, vv, ve = _seam_inputs(m)
    src = np.flatnonzero(ref["singular"] != 0)
    cut, seam = M.seam_paths(gpu_ctx, m.nV, m.nE, vptr, vv, ve, src, in_cut, seam0)
    want = O.compute_seam(m, ref["singular"])
    assert np.array_equal(seam, want)
    assert cut[src].all() and set(np.flatnonzero(cut)) >= set(np.unique(m.edge2vert[want]).tolist())


@pytest.mark.parametrize("seed", [0, 1])
def test_seam_paths_many_sources(gpu_ctx, seed):
    """60 seeded random sources on a level-4 sphere: many searches, most ending on earlier paths."""
    V, F, _, _ = meshgen.workload("ico4_noise")
    m = O.Hmesh(V, F)
    sing = np.zeros(m.nV, np.int64)
    sing[np.random.default_rng(seed).choice(m.nV, 60, replace=False)] = 1
    in_cut, seam0, vptr, vv, ve = _seam_inputs(m)
    _, seam = M.seam_paths(gpu_ctx, m.nV, m.nE, vptr, vv, ve, np.flatnonzero(sing), in_cut, seam0)
    assert np.array_equal(seam, O.compute_seam(m, sing))


def _queue_turns(m, matching, seam, N=4):
    """compute_combbed_field's queue search (face_rosy_field.h:217-242): the turn of each face when
    it is first popped, -1 for faces never reached."""
    from collections import deque
    turns = np.full(m.nF, -1, np.int64)
    q = deque([(0, 0)])
    while q:
        i, mm = q.popleft()
        if turns[i] >= 0:
            continue
        turns[i] = mm
        for j in range(3):
            e = m.edge[m.FH[i, j]]
            if m.isBE[e] or seam[e]:
                continue
            b = m.edge2face[e, 0] == i
            fn = m.edge2face[e, 1] if b else m.edge2face[e, 0]
            if turns[fn] < 0:
                q.append((fn, ((1 if b else -1) * matching[e] + mm) % N))
    return turns


@pytest.mark.parametrize("name", ["ico3_noise", "torus_32x16", "genus2_s3", "cap4_sh8", "cyl_32x12", "ico5_sh8"])
def test_comb_turns_match_queue_search(gpu_ctx, name):
    """The combing turns from the device's level-by-level search equal the reference's queue
    order on every face (the turns do not depend on the path inside the cut disk)."""
    V, F, ratio, rs = meshgen.workload(name)
    ref = O.pipeline(V, F, ratio=ratio, round_seams=rs, stop_after="setup")
    m, seam, matching = ref["mesh"], ref["seam"], ref["matching"]
    nb = np.full((m.nF, 3), -1, np.int64)
    nm = np.zeros((m.nF, 3), np.int64)
    for j in range(3):
        e = m.edge[m.FH[:, j]]
        b = m.edge2face[e, 0] == np.arange(m.nF)
        other = np.where(b, m.edge2face[e, 1], m.edge2face[e, 0])
        nb[:, j] = np.where(seam[e] | m.isBE[e], -1, other)
        nm[:, j] = np.where(b, 1, -1) * matching[e]
    got = M.comb_turns(gpu_ctx, nb, nm)
    want = _queue_turns(m, matching, seam)
    assert np.array_equal(got, want)
    # and the combed field built from them is the oracle's
    _, cm = O.combed_field(m, ref["field"], matching, seam, 4)
    f0, f1 = O._interior_faces(m)
    t = np.maximum(got, 0)
    assert np.array_equal(np.where(m.isBE, -1, (t[f0] - t[f1] + matching + 4000) % 4), cm)
