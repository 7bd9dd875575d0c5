"""Quad extraction (include/metriko/core/qex/qex.h, the reference's core/qex in the order of its
example_qex.cpp) on the CPU against the oracle's restatement (oracle/qex_oracle.py), on seamless
integer-grid maps from the oracle pipeline with the local-injectivity barrier (the reference
example's configuration: seamless, localInjectivity, roundSeams off).  Compared exactly: the
sanitized corner values, the grid points at vertices, on edges and in faces, every port, the
q-edges and the quads; plus the reference's invariants and the topology of the result (a closed
quad mesh of the sphere's Euler characteristic when grid points are merged)."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import metriko_gb300 as M
from metriko_gb300 import meshgen
from oracle import metriko_oracle as O
from oracle import qex_oracle as Q

ROOT = Path(__file__).resolve().parents[1]


def load_workload(name):
    """meshgen workloads, and icosphere_obj: the reference's own model (example/models/icosphere.obj)
    as its golden fixture holds it."""
    if name == "icosphere_obj":
        g = np.load(ROOT / "tests" / "golden" / "icosphere_obj.npz")
        return g["V"], g["F"], float(g["ratio"]), bool(g["round_seams"])
    return meshgen.workload(name)


@pytest.fixture(scope="module")
def qex_harness(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not found")
    M.lib()
    lib = ROOT / "metriko_gb300" / "libmetriko_cuda.so"
    exe = tmp_path_factory.mktemp("cpp") / "qex_harness"
    cuda_inc = Path(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc").resolve().parent.parent / "include"
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-I", str(ROOT / "include"),
           "-I", str(cuda_inc), str(ROOT / "tests" / "cpp" / "qex_harness.cpp"), "-o", str(exe), str(lib),
           "-Wl,-rpath," + str(lib.parent)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def corner_uv(cfn, nF):
    c = np.asarray(cfn).reshape(nF, 3, -1)
    return (c[:, :, 0] + 1j * c[:, :, 1]).reshape(-1)


def run_qex_harness(exe, tmp, V, F, uv, matching, singular):
    blob, outp = tmp / "qin.bin", tmp / "qout.txt"
    with open(blob, "wb") as fh:
        fh.write(np.array([len(V), len(F), len(matching)], np.int32).tobytes())
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

    t = nxt()
    vals = [float(x) for x in t[1:]]
    out = dict(cfn=[complex(vals[i], vals[i + 1]) for i in range(0, len(vals), 2)])
    for key in ("vq", "eq", "fq"):
        n = int(nxt()[2])
        g = []
        for _ in range(n):
            t = nxt()
            g.append((complex(float(t[1]), float(t[2])), (float(t[3]), float(t[4]), float(t[5])), int(t[6])))
        out[key] = g
    n = int(nxt()[1])
    ports = []
    for _ in range(n):
        t = nxt()
        ports.append((int(t[1]), int(t[2]), int(t[3]), int(t[4]), complex(float(t[5]), float(t[6])),
                      complex(float(t[7]), float(t[8])), (float(t[9]), float(t[10]), float(t[11])), int(t[12]),
                      int(t[13]), bool(int(t[14]))))
    out["ports"] = ports
    n = int(nxt()[1])
    out["edges"] = [tuple(map(int, nxt()[1:3])) for _ in range(n)]
    n = int(nxt()[1])
    out["faces"] = [tuple(map(int, nxt()[1:5])) for _ in range(n)]
    return out


def oracle_qex(out, F):
    uv = corner_uv(out["cfn"], len(F))
    q = Q.Qex(out["mesh"], uv, out["combed_matching"], out["singular"]).run()
    return uv, q


CASES = [("ico2_noise", 0.3), ("ico2_noise", None), ("ico3_noise", 0.15), ("icosphere_obj", None)]


@pytest.mark.parametrize("name,ratio", CASES)
def test_qex_matches_oracle(qex_harness, tmp_path, name, ratio):
    V, F, r0, rs = load_workload(name)
    ratio = r0 if ratio is None else ratio
    out = O.pipeline(V, F, ratio=ratio, round_seams=False, seamless=True, local_injectivity=True)
    assert out["success"]
    uv, q = oracle_qex(out, F)
    res = run_qex_harness(qex_harness, tmp_path, V, F, uv, out["combed_matching"], out["singular"])
    assert "error" not in res, res.get("error")
    assert res["cfn"] == q["cfn"]
    assert res["vq"] == q["vq"] and res["eq"] == q["eq"] and res["fq"] == q["fq"]
    assert res["ports"] == [(p["idx"], p["vid"], p["eid"], p["fid"], p["uv"], p["dir"], p["pos"], p["next"], p["prev"],
                             p["conn"]) for p in q["ports"]]
    assert res["edges"] == q["edges"]
    qh = []
    for a, b in q["edges"]:
        qh += [a, b]
    assert res["faces"] == [tuple(qh[k] for k in f) for f in q["faces"]]
    # invariants: every port connected exactly once; every port starts exactly one quad side
    ports, edges, faces = res["ports"], res["edges"], res["faces"]
    assert all(p[9] for p in ports)
    ends = sorted(x for e in edges for x in e)
    assert ends == list(range(len(ports)))
    starts = sorted(x for f in faces for x in f)
    assert starts == list(range(len(ports)))
    # topology: grid points (vertex, edge, face) are the quad mesh's vertices; its Euler
    # characteristic is the sphere's
    nqv = len(res["vq"]) + len(res["eq"]) + len(res["fq"])
    assert nqv - len(edges) + len(faces) == 2


def regular_torus(nu=8, nv=4, R=1.0, r=0.4):
    """A regular torus grid (two triangles per cell) with the seamless map uv = 2 (i, k): every
    vertex, every edge midpoint and no face interior on the integer grid; zero matching (the
    wrap is a translation), no singular vertex."""
    ii, kk = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    a, b = 2 * np.pi * ii.ravel() / nu, 2 * np.pi * kk.ravel() / nv
    V = np.stack([(R + r * np.cos(b)) * np.cos(a), (R + r * np.cos(b)) * np.sin(a), r * np.sin(b)], 1)
    vid = lambda i, k: (i % nu) * nv + (k % nv)  # noqa: E731
    F, uv = [], []
    for i in range(nu):
        for k in range(nv):
            for tri in (((i, k), (i + 1, k), (i + 1, k + 1)), ((i, k), (i + 1, k + 1), (i, k + 1))):
                F.append([vid(*c) for c in tri])
                uv += [complex(2 * c[0], 2 * c[1]) for c in tri]
    return V, np.array(F, np.int32), np.array(uv)


def test_qex_dense_edge_points_fail_like_the_reference(qex_harness, tmp_path):
    """Edge grid points share the reference's list of visited port directions, so two edge points
    one grid step apart along a line claim the same neighbour and one of them is left with three
    ports (the reference asserts four).  The oracle and the C++ port stop at the same place."""
    V, F, uv = regular_torus()
    hm = O.Hmesh(V, F)
    matching = np.zeros(hm.nE, np.int32)
    singular = np.zeros(hm.nV, np.int32)
    qx = Q.Qex(hm, uv, matching, singular)
    vq, eq, fq = qx.q_verts()
    assert len(vq) == hm.nV and len(eq) == hm.nE and len(fq) == 0
    with pytest.raises(ValueError, match="four ports"):
        qx.q_ports(vq, eq, fq)
    res = run_qex_harness(qex_harness, tmp_path, V, F, uv, matching, singular)
    assert "error" in res and "four ports" in res["error"]
