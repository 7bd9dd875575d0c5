"""Motorcycle graph and T-mesh (include/metriko/core/tmesh/, the reference's core/tmesh) on the
CPU against the oracle's restatement (oracle/tmesh_oracle.py), on parameterisations from the
oracle pipeline: the naive integration with the local-injectivity barrier (the configuration of
the reference's example_qgp.cpp: seamless off, localInjectivity on) and rounded seamless maps,
whose axis-aligned edges take the ports' edge-direction branch.  Everything is compared exactly:
ports, every segment end point (bit for bit), crash records, T-edges, T-quads with their sides,
th2sing and the T-edge lengths; plus the reference's invariants."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import metriko_gb300 as M
from metriko_gb300 import meshgen
from oracle import metriko_oracle as O
from oracle import tmesh_oracle as T

ROOT = Path(__file__).resolve().parents[1]


def load_workload(name):
    """meshgen workloads, and icosphere_obj: the reference's own model (example/models/icosphere.obj)
    as its golden fixture holds it."""
    if name == "icosphere_obj":
        g = np.load(ROOT / "tests" / "golden" / "icosphere_obj.npz")
        return g["V"], g["F"], float(g["ratio"]), bool(g["round_seams"])
    return meshgen.workload(name)


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not found")
    M.lib()
    lib = ROOT / "metriko_gb300" / "libmetriko_cuda.so"
    exe = tmp_path_factory.mktemp("cpp") / "tmesh_harness"
    cuda_inc = Path(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc").resolve().parent.parent / "include"
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-I", str(ROOT / "include"),
           "-I", str(cuda_inc), str(ROOT / "tests" / "cpp" / "tmesh_harness.cpp"), "-o", str(exe), str(lib),
           "-Wl,-rpath," + str(lib.parent)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def _corner_uv(cfn, nF):
    c = np.asarray(cfn).reshape(nF, 3, -1)
    return (c[:, :, 0] + 1j * c[:, :, 1]).reshape(-1)


def run_harness(exe, tmp, V, F, uv, matching, singular):
    blob, outp = tmp / "in.bin", tmp / "out.txt"
    nE = len(matching)
    with open(blob, "wb") as fh:
        fh.write(np.array([len(V), len(F), nE], np.int32).tobytes())
        fh.write(np.ascontiguousarray(V, np.float64).tobytes())
        fh.write(np.ascontiguousarray(F, np.int32).tobytes())
        fh.write(np.stack([uv.real, uv.imag], 1).astype(np.float64).tobytes())
        fh.write(np.ascontiguousarray(matching, np.int32).tobytes())
        fh.write(np.ascontiguousarray(singular, np.int32).tobytes())
    r = subprocess.run([str(exe), str(blob), str(outp)], capture_output=True, text=True, timeout=600)
    if r.returncode == 5:
        return dict(error=r.stderr.strip())
    assert r.returncode == 0, (r.returncode, r.stderr[-2000:])
    lines = outp.read_text().split("\n")
    k = 0

    def nxt():
        nonlocal k
        k += 1
        return lines[k - 1].split()

    out = dict(ports=[], curves=[], tedges=[], tquads=[])
    n = int(nxt()[1])
    for _ in range(n):
        t = nxt()
        out["ports"].append((int(t[1]), int(t[2]), int(t[3]), complex(float(t[4]), float(t[5])),
                             complex(float(t[6]), float(t[7])), int(t[8]), int(t[9])))
    n = int(nxt()[1])
    for _ in range(n):
        ns = int(nxt()[1])
        segs = []
        for _ in range(ns):
            t = nxt()
            segs.append((int(t[1]), complex(float(t[2]), float(t[3])), int(t[4]), int(t[5]),
                         complex(float(t[6]), float(t[7])), int(t[8]), int(t[9]), int(t[10]), int(t[11]), int(t[12])))
        out["curves"].append(segs)
    n = int(nxt()[1])
    for _ in range(n):
        t = nxt()
        out["tedges"].append((int(t[1]), int(t[2]), int(t[3])))
    n = int(nxt()[1])
    for _ in range(n):
        t = nxt()
        cnt = int(t[1])
        vals = list(map(int, t[2:2 + 2 * cnt]))
        out["tquads"].append((vals[0::2], vals[1::2]))
    out["th2sing"] = list(map(int, nxt()[1:]))
    out["R"] = [float(x) for x in nxt()[1:]]
    return out


def oracle_graph(out, F):
    uv = _corner_uv(out["cfn"], len(F))
    ports, curves = T.motorcycle_graph(out["mesh"], uv, out["combed_matching"], out["singular"])
    tm = T.tmesh(ports, curves)
    return uv, ports, curves, tm


CASES = [("ico2_noise", False), ("ico3_noise", False), ("genus2_s3", False), ("ico2_noise", True),
         ("ico3_noise", True), ("icosphere_obj", False)]


@pytest.mark.parametrize("name,seamless", CASES)
def test_motorcycle_graph_and_tmesh_match_oracle(harness, tmp_path, name, seamless):
    V, F, ratio, rs = load_workload(name)
    out = O.pipeline(V, F, ratio=ratio, round_seams=rs, seamless=seamless, local_injectivity=not seamless)
    uv, ports, curves, tm = oracle_graph(out, F)
    res = run_harness(harness, tmp_path, V, F, uv, out["combed_matching"], out["singular"])
    assert "error" not in res, res.get("error")
    assert res["ports"] == [(p["id"], p["vert"], p["face"], p["uv"], p["dir"], p["next"], p["prev"]) for p in ports]
    ref_curves = [[(s.face, s.fr.uv, s.fr.crash, s.fr.type, s.to.uv, s.to.crash, s.to.type, s.id, s.prev_id, s.next_id)
                   for s in c.sgmts] for c in curves]
    assert res["curves"] == ref_curves
    assert res["tedges"] == [(ci, sfr.id, sto.id) for ci, sfr, sto in tm["tedges"]]
    assert res["tquads"] == [(list(t), list(s)) for t, s in tm["tquads"]]
    assert res["th2sing"] == tm["th2sing"]
    assert res["R"] == T.tedge_lengths(curves, tm)
    # the reference's invariants: every trace ends in a crash (HitB) and has one start; every
    # T-quad has four sides in cyclic order, not starting inside a side; every T-half-edge lies
    # on exactly one quad
    for c in res["curves"]:
        assert c[-1][6] == T.HIT_B and all(s[6] != T.HIT_B for s in c[:-1])
    for thids, sides in res["tquads"]:
        assert sorted(set(sides)) == [0, 1, 2, 3] and sides[0] != sides[-1]
        assert all((b - a) % 4 in (0, 1) for a, b in zip(sides, sides[1:]))
    seen = sorted(t for thids, _ in res["tquads"] for t in thids)
    assert seen == list(range(2 * len(res["tedges"])))
    # three or five traces per singular vertex of index +-1/4, one start per trace
    assert sum(1 for s in res["th2sing"] if s >= 0) == len(res["ports"])


def test_tmesh_failure_matches_oracle(harness, tmp_path):
    """The rounded map of the genus-2 mesh gives a T-quad walk that does not close: the oracle
    and the C++ port both stop with an error (the reference loops)."""
    V, F, ratio, rs = meshgen.workload("genus2_s3")
    out = O.pipeline(V, F, ratio=ratio, round_seams=rs, seamless=True)
    with pytest.raises(RuntimeError):
        oracle_graph(out, F)
    uv = _corner_uv(out["cfn"], len(F))
    res = run_harness(harness, tmp_path, V, F, uv, out["combed_matching"], out["singular"])
    assert "error" in res and "T-quad" in res["error"]


def test_motorcycle_graph_rejects_flipped_face(harness, tmp_path):
    """A face whose corner values run clockwise stops the port generation, as in the
    reference (gen_ports: "Orientation should be ccw order")."""
    V, F, ratio, rs = meshgen.workload("ico2_noise")
    out = O.pipeline(V, F, ratio=ratio, round_seams=rs, seamless=False, local_injectivity=True)
    uv = _corner_uv(out["cfn"], len(F)).copy()
    sing = np.flatnonzero(out["singular"])[0]
    f = int(np.flatnonzero((F == sing).any(1))[0])
    uv[3 * f + 1], uv[3 * f + 2] = uv[3 * f + 2], uv[3 * f + 1]
    with pytest.raises(ValueError):
        T.motorcycle_graph(out["mesh"], uv, out["combed_matching"], out["singular"])
    res = run_harness(harness, tmp_path, V, F, uv, out["combed_matching"], out["singular"])
    assert "error" in res and "ccw" in res["error"]
