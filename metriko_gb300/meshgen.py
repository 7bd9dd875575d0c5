"""Seeded synthetic surface meshes for the field + integration + IGM path.

The reference quotes its path on closed triangle meshes (a level-4 icosphere ships with its
examples, example/models/icosphere.obj: 2562 vertices / 5120 faces).  There is no public
dataset, so every workload here is generated from a seed:

* ``icosphere(level)``            -- subdivided icosahedron on the unit sphere,
                                     V = 10*4^k + 2, F = 20*4^k, E = 30*4^k.
* ``radial_noise(V, sigma, seed)``  -- each vertex displaced radially by N(0, sigma).
* ``sh_displace(V, lmax, scale, seed)`` -- radius 1 + sum_{l=1..lmax} sum_m a_lm Y_lm with
                                     a_lm ~ N(0, scale / l) over real spherical harmonics.
* ``torus(nu, nv, R, r, flip_p, jitter, seed)`` -- genus-1 parametric grid, each quad's
                                     diagonal flipped with probability ``flip_p`` and each vertex
                                     jittered tangentially by N(0, jitter * edge).
* ``holed_slab(g, s, jitter, flip_p, seed)`` -- genus-g surface: the boundary of a one-voxel-thick
                                     slab of (2g+1) x 3 voxels with g square holes, each voxel
                                     split into s^3 cells, each boundary square cut into two
                                     triangles (diagonal flipped with probability ``flip_p``),
                                     vertices jittered by N(0, jitter / s).
* ``cap(level, zcut, sigma, seed, sh)`` -- open disk: the faces of a level-k icosphere above
                                     z = zcut, radial noise N(0, sigma) or the degree-8
                                     spherical-harmonic radius (one boundary loop).
* ``cylinder(nu, nv, ...)``       -- open cylinder on a periodic-by-open grid (two boundary
                                     loops), diagonals flipped at random, jittered.
* ``workload(name)``               -- the named workloads (config sizes) used by tests/bench.

Faces are consistently oriented with outward normals; vertex arrays are float64 (n x 3),
face arrays int32 (n x 3).  Child faces of one subdivided triangle are stored next to each
other, which keeps neighbouring faces close in memory for the device kernels.
"""
from __future__ import annotations

import math

import numpy as np

_PHI = (1.0 + 5.0 ** 0.5) / 2.0


def icosahedron():
    v = np.array([
        [-1, _PHI, 0], [1, _PHI, 0], [-1, -_PHI, 0], [1, -_PHI, 0],
        [0, -1, _PHI], [0, 1, _PHI], [0, -1, -_PHI], [0, 1, -_PHI],
        [_PHI, 0, -1], [_PHI, 0, 1], [-_PHI, 0, -1], [-_PHI, 0, 1],
    ], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([
        [0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
        [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
        [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
        [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1],
    ], dtype=np.int64)
    return v, _orient_outward(v, f)


def _orient_outward(v, f):
    a, b, c = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    n = np.cross(b - a, c - a)
    flip = np.einsum("ij,ij->i", n, (a + b + c) / 3.0) < 0
    f = f.copy()
    f[flip] = f[flip][:, [0, 2, 1]]
    return f


def icosphere(level: int):
    """Unit icosphere after ``level`` 1->4 subdivisions (midpoints projected to the sphere)."""
    v, f = icosahedron()
    for _ in range(level):
        nv = len(v)
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
        e.sort(axis=1)
        key = e[:, 0] * nv + e[:, 1]
        uk, inv = np.unique(key, return_inverse=True)
        lo, hi = uk // nv, uk % nv
        mid = v[lo] + v[hi]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        nf = len(f)
        m01 = nv + inv[:nf]
        m12 = nv + inv[nf:2 * nf]
        m20 = nv + inv[2 * nf:]
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        child = np.stack([
            np.stack([a, m01, m20], 1),
            np.stack([b, m12, m01], 1),
            np.stack([c, m20, m12], 1),
            np.stack([m01, m12, m20], 1),
        ], axis=1).reshape(-1, 3)
        v = np.concatenate([v, mid], axis=0)
        f = child
    return v, f.astype(np.int32)


def radial_noise(v, sigma: float, seed: int):
    rng = np.random.default_rng(seed)
    r = 1.0 + rng.normal(0.0, sigma, size=len(v))
    u = v / np.linalg.norm(v, axis=1, keepdims=True)
    return u * r[:, None]


def real_sph_harm_table(lmax: int, theta, phi):
    """Real orthonormal spherical harmonics Y_lm(theta, phi), l = 0..lmax, m = -l..l.

    Returns a dict (l, m) -> array.  Uses the fully normalised associated Legendre recurrence.
    """
    ct, st = np.cos(theta), np.sin(theta)
    p = {}
    p[(0, 0)] = np.full_like(theta, math.sqrt(1.0 / (4.0 * math.pi)))
    for m in range(1, lmax + 1):
        p[(m, m)] = -math.sqrt((2 * m + 1) / (2.0 * m)) * st * p[(m - 1, m - 1)]
    for m in range(0, lmax):
        p[(m + 1, m)] = math.sqrt(2 * m + 3) * ct * p[(m, m)]
    for m in range(0, lmax + 1):
        for l in range(m + 2, lmax + 1):
            a = math.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
            b = math.sqrt(((l - 1) ** 2 - m * m) / (4.0 * (l - 1) ** 2 - 1.0))
            p[(l, m)] = a * (ct * p[(l - 1, m)] - b * p[(l - 2, m)])
    y = {}
    s2 = math.sqrt(2.0)
    for l in range(lmax + 1):
        y[(l, 0)] = p[(l, 0)]
        for m in range(1, l + 1):
            y[(l, m)] = s2 * p[(l, m)] * np.cos(m * phi)
            y[(l, -m)] = s2 * p[(l, m)] * np.sin(m * phi)
    return y


def sh_displace(v, lmax: int, scale: float, seed: int):
    """Radius 1 + sum_{l=1..lmax, m=-l..l} a_lm Y_lm, a_lm ~ N(0, scale / l), drawn l-major."""
    rng = np.random.default_rng(seed)
    u = v / np.linalg.norm(v, axis=1, keepdims=True)
    theta = np.arccos(np.clip(u[:, 2], -1.0, 1.0))
    phi = np.arctan2(u[:, 1], u[:, 0])
    y = real_sph_harm_table(lmax, theta, phi)
    r = np.ones(len(v))
    for l in range(1, lmax + 1):
        for m in range(-l, l + 1):
            r += rng.normal(0.0, scale / l) * y[(l, m)]
    return u * r[:, None]


def torus(nu: int, nv: int, R: float = 1.0, r: float = 0.35, flip_p: float = 0.5,
          jitter: float = 0.1, seed: int = 0):
    """Closed torus on an nu x nv parametric grid (u around the ring, v around the tube)."""
    rng = np.random.default_rng(seed)
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    ju = rng.normal(0.0, jitter, size=i.shape)
    jv = rng.normal(0.0, jitter, size=j.shape)
    u = 2.0 * np.pi * (i + ju) / nu
    w = 2.0 * np.pi * (j + jv) / nv
    ring = R + r * np.cos(w)
    V = np.stack([ring * np.cos(u), ring * np.sin(u), r * np.sin(w)], axis=-1).reshape(-1, 3)
    idx = lambda a, b: (a % nu) * nv + (b % nv)  # noqa: E731
    a = idx(i, j).ravel()
    b = idx(i + 1, j).ravel()
    c = idx(i + 1, j + 1).ravel()
    d = idx(i, j + 1).ravel()
    flip = rng.random(a.shape) < flip_p
    t0 = np.where(flip[:, None], np.stack([a, b, d], 1), np.stack([a, b, c], 1))
    t1 = np.where(flip[:, None], np.stack([b, c, d], 1), np.stack([a, c, d], 1))
    F = np.stack([t0, t1], axis=1).reshape(-1, 3)
    return V, F.astype(np.int32)


def holed_slab(g: int, s: int = 3, jitter: float = 0.05, flip_p: float = 0.5, seed: int = 0):
    """Closed genus-g surface, the boundary of a polycube: a slab (2g+1) x 3 x 1 voxels with the
    voxels (2k+1, 1), k < g, removed (g through-holes).  No two cells meet only along an edge or at
    a corner, so the boundary is a 2-manifold; V - E + F = 2 - 2g.  Coordinates in voxel units."""
    rng = np.random.default_rng(seed)
    n = ((2 * g + 1) * s, 3 * s, s)
    solid = np.ones(n, bool)
    for k in range(g):
        solid[(2 * k + 1) * s:(2 * k + 2) * s, s:2 * s, :] = False
    pad = np.pad(solid, 1)
    quads = []
    for axis in range(3):
        u, w = (axis + 1) % 3, (axis + 2) % 3
        for sign in (1, -1):
            cells = np.argwhere(pad & ~np.roll(pad, -sign, axis=axis)) - 1
            base = cells.copy()
            base[:, axis] += sign > 0
            du = np.zeros(3, np.int64)
            dw = np.zeros(3, np.int64)
            du[u] = 1
            dw[w] = 1
            q = np.stack([base, base + du, base + du + dw, base + dw], axis=1)   # CCW about +axis
            quads.append(q if sign > 0 else q[:, ::-1])
    q = np.concatenate(quads)                                            # (nq, 4, 3) lattice points
    key = (q[..., 0] * (n[1] + 1) + q[..., 1]) * (n[2] + 1) + q[..., 2]
    uniq, inv = np.unique(key.ravel(), return_inverse=True)
    inv = inv.reshape(-1, 4)
    lat = np.stack([uniq // ((n[1] + 1) * (n[2] + 1)), (uniq // (n[2] + 1)) % (n[1] + 1), uniq % (n[2] + 1)], 1)
    V = lat / s + rng.normal(0.0, jitter / s, size=lat.shape)
    a, b, c, d = inv.T
    flip = rng.random(len(a)) < flip_p
    t0 = np.where(flip[:, None], np.stack([a, b, d], 1), np.stack([a, b, c], 1))
    t1 = np.where(flip[:, None], np.stack([b, c, d], 1), np.stack([a, c, d], 1))
    F = np.stack([t0, t1], axis=1).reshape(-1, 3)
    return V.astype(np.float64), F.astype(np.int32)


def _compact(V, F):
    """Drops the vertices no face uses and renumbers the rest in their original order."""
    used = np.zeros(len(V), bool)
    used[F.ravel()] = True
    new = np.cumsum(used) - 1
    return V[used], new[F].astype(np.int32)


def _check_manifold_boundary(F):
    """Every boundary vertex must lie on exactly two boundary edges (no two boundary loops
    touching at a vertex), and every edge on at most two faces."""
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
    key = np.sort(e, axis=1)
    u, cnt = np.unique(key, axis=0, return_counts=True)
    if cnt.max() > 2:
        raise ValueError("edge on more than two faces")
    bv = u[cnt == 1].ravel()
    if len(bv):
        vc = np.bincount(bv)
        if vc[vc > 0].max() != 2 or vc[vc > 0].min() != 2:
            raise ValueError("boundary loops touch at a vertex")


def cap(level: int, zcut: float = -0.3, sigma: float = 0.01, seed: int = 0, sh: bool = False):
    """Open surface with one boundary loop (a disk): the faces of a level-``level`` icosphere
    whose three vertices lie above z = ``zcut``, each vertex displaced radially by N(0, sigma), or
    with ``sh`` by the degree-8 spherical-harmonic radius of ``sh_displace`` (scale 0.05)."""
    v, f = icosphere(level)
    keep = (v[f][:, :, 2] > zcut).all(axis=1)
    V, F = _compact(v, f[keep])
    _check_manifold_boundary(F)
    if sh:
        return sh_displace(V, 8, 0.05, seed), F
    return radial_noise(V, sigma, seed), F


def cylinder(nu: int, nv: int, r: float = 0.5, h: float = 1.0, flip_p: float = 0.5, jitter: float = 0.1,
             seed: int = 0):
    """Open cylinder (an annulus: two boundary loops) on an nu x nv grid, u around the axis
    (periodic), v along it (nv + 1 rows of vertices); each quad's diagonal flipped with probability
    ``flip_p``, interior vertices jittered by N(0, jitter * edge) in u and v."""
    rng = np.random.default_rng(seed)
    i, j = np.meshgrid(np.arange(nu), np.arange(nv + 1), indexing="ij")
    ju = rng.normal(0.0, jitter, size=i.shape)
    jv = rng.normal(0.0, jitter, size=j.shape)
    jv[:, 0] = 0.0
    jv[:, nv] = 0.0
    u = 2.0 * np.pi * (i + ju) / nu
    z = h * (j + jv) / nv
    V = np.stack([r * np.cos(u), r * np.sin(u), z], axis=-1).reshape(-1, 3)
    ii, jj = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    idx = lambda a, b: (a % nu) * (nv + 1) + b  # noqa: E731
    a = idx(ii, jj).ravel()
    b = idx(ii + 1, jj).ravel()
    c = idx(ii + 1, jj + 1).ravel()
    d = idx(ii, jj + 1).ravel()
    flip = rng.random(a.shape) < flip_p
    t0 = np.where(flip[:, None], np.stack([a, b, d], 1), np.stack([a, b, c], 1))
    t1 = np.where(flip[:, None], np.stack([b, c, d], 1), np.stack([a, c, d], 1))
    F = np.stack([t0, t1], axis=1).reshape(-1, 3)
    return V, F.astype(np.int32)


# Named workloads: (builder, grid ratio).  The ratio is RosyParameterization's `ratio`
# argument (grid edge length = bbox diagonal * ratio / mean field norm).
def workload(name: str, seed: int = 0):
    """Returns (V, F, ratio, round_seams) for a named workload."""
    if name == "ico4_noise":        # 2562 V / 5120 F, radial N(0, 0.01), edge 0.03
        v, f = icosphere(4)
        return radial_noise(v, 0.01, seed), f, 0.03, False
    if name.startswith("ico") and name.endswith("_sh8"):   # e.g. ico7_sh8, ico8_sh8
        lvl = int(name[3:-4])
        v, f = icosphere(lvl)
        return sh_displace(v, 8, 0.05, seed), f, 0.01, False
    if name.startswith("ico") and name.endswith("_sh16"):  # ico9_sh16
        lvl = int(name[3:-5])
        v, f = icosphere(lvl)
        return sh_displace(v, 16, 0.03, seed), f, 0.01, False
    if name.startswith("ico") and name.endswith("_noise"):
        lvl = int(name[3:-6])
        v, f = icosphere(lvl)
        return radial_noise(v, 0.01, seed), f, 0.03, False
    if name == "torus_1024x512":    # 524288 V / 1048576 F, edge 0.005, rounds seams
        v, f = torus(1024, 512, seed=seed)
        return v, f, 0.005, True
    if name.startswith("torus_"):
        nu, nv = (int(t) for t in name[6:].split("x"))
        v, f = torus(nu, nv, seed=seed)
        return v, f, 0.02, True
    if name.startswith("cap") and name.endswith("_noise"):   # e.g. cap4_noise: open disk
        v, f = cap(int(name[3:-6]), seed=seed)
        return v, f, 0.03, False
    if name.startswith("cap") and name.endswith("_sh8"):     # e.g. cap7_sh8: smooth open disk
        v, f = cap(int(name[3:-4]), seed=seed, sh=True)
        return v, f, 0.01, False
    if name.startswith("cyl_"):     # e.g. cyl_32x12: open cylinder (two boundary loops)
        nu, nv = (int(t) for t in name[4:].split("x"))
        v, f = cylinder(nu, nv, seed=seed)
        return v, f, 0.03, True
    if name.startswith("genus"):    # e.g. genus2_s3: holed_slab(2, 3)
        g, sub = name[5:].split("_s")
        v, f = holed_slab(int(g), int(sub), seed=seed)
        return v, f, 0.02, False
    raise KeyError(name)


def read_obj(path):
    vs, fs = [], []
    with open(path) as fh:
        for line in fh:
            if line.startswith("v "):
                vs.append([float(t) for t in line.split()[1:4]])
            elif line.startswith("f "):
                fs.append([int(t.split("/")[0]) - 1 for t in line.split()[1:4]])
    return np.asarray(vs, np.float64), np.asarray(fs, np.int32)
