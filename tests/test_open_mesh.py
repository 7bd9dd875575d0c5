"""Meshes with boundary on the host (no GPU): the oracle's halfedge mesh against the reference's
numbering rules, and the C++ host stages (through the C ABI) against the oracle.

Open surfaces: ``cap<k>_noise`` (the part of a level-k icosphere above z = -0.3: a disk, one
boundary loop) and ``cyl_<u>x<v>`` (an open cylinder: an annulus, two boundary loops).  The
reference treats them as follows (all restated by the oracle): boundary halfedges are numbered
after the 3 nF interior ones, loop by loop (hmesh.h:393-418); boundary edges get no Laplacian
entry (face_rosy_field.h:64), no matching (-1) and no effort; boundary vertices keep the
singular index 1 (:101-102), so they all enter the seam search, whose spanning cut keeps every
boundary edge as a seam; the cut mesh, the transition ids and setup() start a boundary vertex's
fan at its first boundary-edge halfedge and stop at its boundary halfedge
(parameterization.h:80-82,136-140, parameterization_setup.ipp:26-36,76-105).
"""
from pathlib import Path

import numpy as np
import pytest

import metriko_gb300 as M
from metriko_gb300 import meshgen
from oracle import metriko_oracle as O

OPEN = ["cap2_noise", "cap3_noise", "cap4_noise", "cyl_16x6", "cyl_32x12"]


@pytest.mark.parametrize("name", OPEN)
def test_oracle_halfedge_mesh_with_boundary(name):
    V, F, _, _ = meshgen.workload(name)
    m = O.Hmesh(V, F)
    nI = 3 * m.nF
    h = np.arange(m.nH)
    assert m.is_boundary and m.nL == (1 if name.startswith("cap") else 2)
    assert np.array_equal(m.twin[m.twin], h)                       # involution
    assert np.array_equal(m.next[m.prev], h) and np.array_equal(m.prev[m.next], h)
    assert np.array_equal(m.head, m.tail[m.next])
    assert np.array_equal(m.tail[m.twin], m.head)
    assert (m.face[:nI] >= 0).all() and (m.face[nI:] == -1).all()   # boundary halfedges last
    assert np.array_equal(m.edge[m.twin], m.edge)
    # interior halfedges in (edge, slot) order, boundary halfedges loop by loop
    assert (np.diff(m.edge[:nI]) >= 0).all()
    loops = []
    for l0 in m.loop2half:
        loop = [l0]
        while m.next[loop[-1]] != l0:
            loop.append(m.next[loop[-1]])
        loops.append(loop)
    assert sorted(x for lp in loops for x in lp) == list(range(nI, m.nH))
    for lp in loops:
        assert lp == list(range(lp[0], lp[0] + len(lp)))            # consecutive ids per loop
    # boundary vertices: exactly the tails of boundary halfedges
    assert np.array_equal(np.flatnonzero(m.isBV), np.unique(m.tail[nI:]))
    assert m.nV - m.nE + m.nF == (1 if name.startswith("cap") else 0)


@pytest.mark.parametrize("name", OPEN)
def test_topology_matches_oracle_on_open_meshes(name):
    V, F, ratio, rs = meshgen.workload(name)
    ref = O.pipeline(V, F, ratio=ratio, round_seams=rs, stop_after="setup")
    res = M.topology_from_field(V, F, ref["compressed"], ratio, rs)
    m = ref["mesh"]
    assert np.array_equal(res["singular"], ref["singular"])
    assert (res["singular"][m.isBV] == 1).all()
    assert np.array_equal(res["seam"], ref["seam"])
    assert res["seam"][m.isBE].all()                    # boundary edges stay on the seam
    assert np.array_equal(res["matching"], ref["combed_matching"])
    assert (res["matching"][m.isBE] == -1).all()
    assert np.array_equal(res["cutF"], ref["cutF"])
    c = res["counts"]
    st = ref["setup"]
    assert c["nE"] == m.nE
    assert c["nCut"] == len(ref["cutV"]) and c["nT"] == st["nT"] and c["nS"] == st["nS"]
    assert c["nFull"] == st["n"] * st["nR"]


@pytest.mark.parametrize("name", ["cap3_noise", "cyl_16x6"])
def test_open_cut_mesh_is_a_disk(name):
    V, F, ratio, rs = meshgen.workload(name)
    ref = O.pipeline(V, F, ratio=ratio, stop_after="field")
    res = M.topology_from_field(V, F, ref["compressed"], ratio, rs)
    cutF = res["cutF"]
    e = np.unique(np.sort(np.concatenate([cutF[:, [0, 1]], cutF[:, [1, 2]], cutF[:, [2, 0]]]), axis=1), axis=0)
    assert res["counts"]["nCut"] - len(e) + len(cutF) == 1


@pytest.mark.parametrize("name", ["cap3_noise", "cyl_32x12"])
def test_open_mesh_geometry_matches_oracle(name):
    """The vertex and edge geometry on a mesh with boundary: dihedral angle 0 on boundary edges,
    cotangent 0 on boundary halfedges, the dual areas over the faces present, and the angle
    defect pi - sum at boundary vertices, whose ring includes the angle between their two
    boundary edges (hmesh.h:508-568)."""
    V, F, _, _ = meshgen.workload(name)
    g = M.mesh_geometry(V, F)
    m = O.Hmesh(V, F)
    o = m.vertex_geometry()
    for k in ["vertNormal", "vertBasisX", "vertBasisY", "baryDualArea", "circDualArea", "halfCotan", "edgeCotan"]:
        assert np.array_equal(g[k], o[k]), k
    for k in ["dihedralArg", "heArgOnVert", "angleDefect"]:
        assert np.abs(g[k] - o[k]).max() <= 1e-14, k
    assert (g["dihedralArg"][m.isBE[m.edge]] == 0).all()
    assert (g["halfCotan"][3 * m.nF:] == 0).all()
    assert abs(g["baryDualArea"].sum() - m.faceArea.sum()) <= 1e-12 * m.faceArea.sum()


def test_open_field_inputs_match_oracle():
    V, F, _, _ = meshgen.workload("cap3_noise")
    nbr, theta, area = M.field_inputs(V, F)
    m = O.Hmesh(V, F)
    onbr = m.face[m.twin[m.FH]]
    assert np.array_equal(nbr, onbr) and (onbr == -1).any()
    inner = onbr >= 0
    assert np.abs(theta[inner] - (m.farg[m.FH] - m.farg[m.twin[m.FH]])[inner]).max() < 1e-12
    assert (theta[~inner] == 0).all()
    assert np.array_equal(area, m.faceArea)


@pytest.mark.parametrize("name", ["cap2_noise", "cyl_16x6"])
def test_oracle_rounds_open_meshes(name):
    """The oracle's whole path on an open mesh ends with integral values (post_checking), and its
    Laplacian has the reference's diagonal (#interior neighbours + 1e-9)."""
    V, F, ratio, rs = meshgen.workload(name)
    out = O.pipeline(V, F, ratio=ratio, round_seams=rs)
    assert out["success"]
    m = out["mesh"]
    cnt = (m.face[m.twin[m.FH]] >= 0).sum(axis=1)
    assert np.abs(out["L"].diagonal().real - (cnt + 1e-9)).max() < 1e-15
    assert (cnt < 3).any()


def test_open_large_golden_mesh_regenerates():
    """The open-disk fixture of 52,982 faces keeps no mesh: the seeded generator must still
    produce it, and its stored rounded values are integral."""
    g = np.load(Path(__file__).parent / "golden" / "cap6_sh8.npz")
    V, F, ratio, rs = meshgen.workload("cap6_sh8")
    assert len(V) == int(g["nV"]) and len(F) == int(g["nF"])
    assert np.abs(V[g["v_sample_idx"]] - g["v_sample"]).max() <= 1e-12
    X = g["fullx_fixed"]
    assert np.abs(X - np.round(X)).max() <= 1e-6
    assert np.array_equal(np.round(X).astype(int), g["fix_vals"])
