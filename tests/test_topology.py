"""Host C++ topology stages (through the C ABI, no GPU) against the oracle: matching,
singularities, seams, combing and the cut mesh are integer outputs and must be bit-exact."""
import numpy as np
import pytest

import metriko_gb300 as M
from metriko_gb300 import meshgen
from oracle import metriko_oracle as O


@pytest.mark.parametrize("name", ["ico2_noise", "ico3_noise", "ico4_noise", "torus_32x16", "torus_64x32",
                                  "genus2_s3", "genus3_s2", "genus2_s4"])
def test_topology_matches_oracle(name):
    V, F, ratio, rs = meshgen.workload(name)
    ref = O.pipeline(V, F, ratio=ratio, round_seams=rs, stop_after="setup")
    res = M.topology_from_field(V, F, ref["compressed"], ratio, rs)
    assert np.array_equal(res["singular"], ref["singular"])
    assert np.array_equal(res["seam"], ref["seam"])
    assert np.array_equal(res["matching"], ref["combed_matching"])
    assert np.array_equal(res["cutF"], ref["cutF"])
    c = res["counts"]
    st = ref["setup"]
    assert c["nCut"] == len(ref["cutV"]) and c["nT"] == st["nT"] and c["nS"] == st["nS"]
    assert c["nFull"] == st["n"] * st["nR"]


def test_topology_length_and_ufull_sizes():
    name = "ico3_noise"
    V, F, ratio, rs = meshgen.workload(name)
    ref = O.pipeline(V, F, ratio=ratio, round_seams=rs)
    res = M.topology_from_field(V, F, ref["compressed"], ratio, rs)
    assert abs(res["length"] - ref["length"]) <= 1e-12 * ref["length"]
    ni = ref["info"]["ni"]
    assert res["counts"]["nJ"] == len(ni.uniqueJ)
    assert res["counts"]["nZ"] == ni.USmall.shape[1]


def test_seam_is_tree_through_singularities():
    """On a sphere the seam is a tree touching every singular vertex."""
    V, F, ratio, rs = meshgen.workload("ico3_noise")
    ref = O.pipeline(V, F, ratio=ratio, stop_after="field")
    res = M.topology_from_field(V, F, ref["compressed"], ratio, rs)
    m = O.Hmesh(V, F)
    E = m.edge2vert[res["seam"]]
    verts = np.unique(E)
    assert len(E) == len(verts) - 1          # a tree
    assert set(np.flatnonzero(res["singular"])) <= set(verts.tolist())


@pytest.mark.parametrize("name,genus", [("ico3_noise", 0), ("torus_32x16", 1), ("genus2_s3", 2), ("genus3_s2", 3)])
def test_cut_mesh_is_a_disk(name, genus):
    """The seam cuts every handle: the cut mesh is a topological disk (V - E + F = 1) and the seam
    graph has first Betti number 2g (E_seam - V_seam + 1 independent cycles)."""
    V, F, ratio, rs = meshgen.workload(name)
    ref = O.pipeline(V, F, ratio=ratio, stop_after="field")
    res = M.topology_from_field(V, F, ref["compressed"], ratio, rs)
    cutF = res["cutF"]
    e = np.unique(np.sort(np.concatenate([cutF[:, [0, 1]], cutF[:, [1, 2]], cutF[:, [2, 0]]]), axis=1), axis=0)
    assert res["counts"]["nCut"] - len(e) + len(cutF) == 1
    m = O.Hmesh(V, F)
    E = m.edge2vert[res["seam"]]
    assert len(E) - len(np.unique(E)) + 1 == 2 * genus


def test_field_inputs_match_oracle():
    """mtk_field_inputs (host): the neighbour and transport-angle inputs of the field solve."""
    V, F, _, _ = meshgen.workload("ico3_noise")
    nbr, theta, area = M.field_inputs(V, F)
    m = O.Hmesh(V, F)
    assert np.array_equal(nbr, m.face[m.twin[m.FH]])
    assert np.abs(theta - (m.farg[m.FH] - m.farg[m.twin[m.FH]])).max() < 1e-12
    assert np.array_equal(area, m.faceArea)


@pytest.mark.parametrize("name", ["ico3_noise", "torus_32x16", "genus2_s3"])
def test_mesh_vertex_and_edge_geometry_matches_oracle(name):
    """Hmesh's vertex frames, dual areas, cotangents, dihedral angles and vertex halfedge angles
    (mtk_mesh_geometry) against the oracle: the algebraic ones bit for bit, the ones through
    acos / atan2 to a few ulp (numpy's and the C library's functions may round differently)."""
    V, F, _, _ = meshgen.workload(name)
    g = M.mesh_geometry(V, F)
    m = O.Hmesh(V, F)
    o = m.vertex_geometry()
    for k in ["vertNormal", "vertBasisX", "vertBasisY", "baryDualArea", "circDualArea", "halfCotan", "edgeCotan"]:
        assert np.array_equal(g[k], o[k]), k
    for k in ["dihedralArg", "heArgOnVert", "angleDefect"]:
        assert np.abs(g[k] - o[k]).max() <= 1e-14, k
    area = m.faceArea.sum()
    assert abs(g["baryDualArea"].sum() - area) <= 1e-12 * area
    assert abs(g["circDualArea"].sum() - area) <= 1e-12 * area      # cotangent identity, closed mesh
    assert abs(g["angleDefect"].sum() - 2 * np.pi * (m.nV - m.nE + m.nF)) < 1e-9
    X, Y, Nn = g["vertBasisX"], g["vertBasisY"], g["vertNormal"]
    assert np.abs(np.einsum("ij,ij->i", X, Nn)).max() < 1e-12 and np.abs(np.einsum("ij,ij->i", X, Y)).max() < 1e-12
    assert np.abs(np.linalg.norm(Y, axis=1) - 1).max() < 1e-12


def test_constraint_reduction_with_many_singularities():
    """A noisy level-5 sphere (338 singularities, 1,652 constraint rows): the host's sparse
    Gram-Schmidt row selection and parallel full-pivot kernel give the oracle's dense results
    (constrained variables nJ and kernel dimension nZ)."""
    V, F, ratio, rs = meshgen.workload("ico5_noise")
    ref = O.pipeline(V, F, ratio=ratio, round_seams=rs, stop_after="setup")
    st = ref["setup"]
    Cfull = O.structural_product(st["constraint"], st["uncompress"])
    Cr = Cfull[O.independent_rows(Cfull)].tocsr()
    uj = np.unique(Cr.indices)
    K = O.fullpiv_kernel(Cr[:, uj].toarray())
    res = M.topology_from_field(V, F, ref["compressed"], ratio, rs)
    assert res["counts"]["nS"] > 300
    assert res["counts"]["nJ"] == len(uj) and res["counts"]["nZ"] == K.shape[1]


def _projected_field(V, F, a=(0.3, -0.2, 1.0)):
    """Compressed 4-RoSy field (unit, 4th power) of the tangential projection of the direction a,
    in each face's frame (x along F[f,1] - F[f,0])."""
    p0, p1, p2 = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    bx = p1 - p0
    bx /= np.linalg.norm(bx, axis=1, keepdims=True)
    n = np.cross(p1 - p0, p2 - p0)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    by = np.cross(n, bx)
    a = np.asarray(a, float) / np.linalg.norm(a)
    d = a - (n @ a)[:, None] * n
    z = np.einsum("ij,ij->i", d, bx) + 1j * np.einsum("ij,ij->i", d, by)
    return (z / np.abs(z)) ** 4


def test_host_topology_at_the_benchmark_size():
    """The host stages on the 1.3M-face benchmark mesh (two host threads, parallel edge topology)
    through size-independent properties: the singular indices sum to 4 chi, the seam is a tree
    that reaches every singular vertex, the cut mesh is a disk and the counts are consistent."""
    V, F, ratio, rs = meshgen.workload("ico8_sh8")
    res = M.topology_from_field(V, F, _projected_field(V, F), ratio, rs)
    c = res["counts"]
    assert c["nV"] == 655362 and c["nE"] == 1966080
    assert res["singular"].sum() == 8
    m_edges = np.sort(np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), axis=1)
    ev = np.unique(m_edges, axis=0)                     # edge_topology numbering: sorted (lo, hi)
    E = ev[res["seam"]]
    verts = np.unique(E)
    assert len(E) == len(verts) - 1                     # a tree
    assert set(np.flatnonzero(res["singular"])) <= set(verts.tolist())
    assert c["nCut"] == c["nV"] + len(E) - 1            # each tree edge opens into two boundary edges
    cutF = res["cutF"]
    ce = np.unique(np.sort(np.concatenate([cutF[:, [0, 1]], cutF[:, [1, 2]], cutF[:, [2, 0]]]), axis=1), axis=0)
    assert c["nCut"] - len(ce) + len(cutF) == 1         # a disk
    assert c["nS"] == int((res["singular"] != 0).sum()) and c["nFull"] == 2 * (c["nV"] + c["nT"])
