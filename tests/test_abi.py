"""C ABI: the library loads, exports every symbol include/*.h declares, and its host-only
entry points behave without a GPU."""
import re
from pathlib import Path

import numpy as np
import pytest

import metriko_gb300 as M
from metriko_gb300 import _lib
from oracle import metriko_oracle as O

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b(mtk_[a-z0-9_]+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol():
    L = M.lib()
    names = declared_functions()
    assert "mtk_field_smoothest" in names and "mtk_iterative_rounding" in names
    for n in names:
        assert hasattr(L, n), n
    assert set(_lib.EXPORTS) == names


def test_status_strings():
    L = M.lib()
    assert L.mtk_status_string(0).decode() == "ok"
    assert "converged" in L.mtk_status_string(3).decode()
    assert L.mtk_status_string(99).decode() == "unknown status"


def test_default_opts():
    o = M.solve_opts()
    assert o.precision == M.PREC_MIXED and o.tol == 1e-8 and o.max_iter > 0


@pytest.mark.parametrize("seed", [0, 1, 12345])
def test_seeded_init_matches_oracle(seed):
    a = M.seeded_init(1000, seed)
    b = O.seeded_init(1000, seed)
    assert np.array_equal(a, b)
    assert np.abs(a.real).max() <= 1 and np.abs(a.imag).max() <= 1


def test_topology_rejects_inconsistent_orientation():
    """Two faces that run along their shared edge the same way (one face flipped) cannot be given
    the reference's halfedge numbering: MTK_ERR_BAD_INPUT with a message.  A single triangle, all
    boundary, is a valid open mesh."""
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]], float)
    F = np.array([[0, 1, 2], [1, 2, 3]], np.int32)
    with pytest.raises(M.MetrikoError) as e:
        M.topology_from_field(V, F, np.ones(2, complex))
    assert e.value.status == _lib.BAD_INPUT
    assert "oriented" in str(e.value)
    res = M.topology_from_field(V[:3], F[:1], np.ones(1, complex))
    assert list(res["singular"]) == [1, 1, 1] and res["seam"].all() and res["counts"]["nCut"] == 3


def test_topology_rejects_bad_index():
    V, F = M.meshgen.icosphere(1)
    F = F.copy()
    F[3, 1] = 10_000
    with pytest.raises(M.MetrikoError):
        M.topology_from_field(V, F, np.ones(len(F), complex))


@pytest.mark.parametrize("case", ["non_manifold", "isolated_vertex", "repeated_vertex"])
def test_topology_rejects_invalid_meshes(case):
    """Closed, edge-manifold meshes only: a third face on an edge, a vertex in no face and a face
    with a repeated vertex are rejected with MTK_ERR_BAD_INPUT and a message."""
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1]], float)
    tet = [[0, 2, 1], [0, 3, 2], [0, 1, 3], [1, 2, 3]]
    F = {"non_manifold": tet + [[0, 1, 4]], "isolated_vertex": tet,
         "repeated_vertex": [[0, 2, 2], [0, 3, 2], [0, 1, 3], [1, 2, 3]]}[case]
    F = np.array(F, np.int32)
    with pytest.raises(M.MetrikoError) as e:
        M.topology_from_field(V, F, np.ones(len(F), complex))
    assert e.value.status == _lib.BAD_INPUT
    msg = str(e.value)      # carries mtk_last_error()
    assert {"non_manifold": "edge-manifold", "isolated_vertex": "isolated vertex",
            "repeated_vertex": "bad face index"}[case] in msg


def test_ctx_create_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(M.MetrikoError) as e:
        M.Context(0)
    assert e.value.status == _lib.NO_DEVICE
