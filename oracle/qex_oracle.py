"""Test infrastructure: CPU restatement of the reference's quad extraction (QEx,
include/metriko/core/qex/{common,sanitization,gen_q_vert,gen_q_port,gen_q_edge,gen_q_face}.h of
komietty/metriko, with conversion_2d_3d / calc_coefficient of core/hmesh/utilities.h and
core/common/utilities.h), in the order example/example_qex.cpp calls it.  Used only by tests/
as the checker of the header-only C++ port (include/metriko/core/qex/qex.h).  Parity unpinned:
the reference needs Eigen and libigl, absent here; the restatement is checked against the C++
port (bit for bit) and against the reference's own invariants (four ports per edge grid point,
every port connected once, quads of four half-edges).

Arithmetic follows the reference's expressions: std::round (halves away from zero), Eigen's 2x2
cofactor inverse, Eigen's norm() = sqrt(x^2 + y^2 + z^2) and normalized() = v / sqrt(|v|^2), 3D
points combined per component left to right."""
import math

from .tmesh_oracle import Mesh, cadd, cmul, csub, cross, dot, extended_intersection, quater_rot

EPS = 1e-9


def std_round(x):
    """std::round: the nearest integer, halves away from zero."""
    if x < 0:
        return -std_round(-x)
    r = math.floor(x)
    return float(r + 1 if x - r >= 0.5 else r)


def cscale(a, s):
    return complex(a.real * s, a.imag * s)


def lerp(a, b, t):
    s = 1.0 - t
    return complex(a.real * s + b.real * t, a.imag * s + b.imag * t)


def v_sub(a, b):
    return (a[0] - b[0], a[1] - b[1], a[2] - b[2])


def v_add(a, b):
    return (a[0] + b[0], a[1] + b[1], a[2] + b[2])


def v_scale(a, s):
    return (a[0] * s, a[1] * s, a[2] * s)


def v_dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def v_norm(a):
    return math.sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2])


def v_normalized(a):
    z = a[0] * a[0] + a[1] * a[1] + a[2] * a[2]
    if z > 0:
        n = math.sqrt(z)
        return (a[0] / n, a[1] / n, a[2] / n)
    return a


# ---------------------------------------------------------------- qex/common.h
def orientation(pa, pb, pc):
    """qex::orientation (common.h:91-100)."""
    acx, bcx = pa.real - pc.real, pb.real - pc.real
    acy, bcy = pa.imag - pc.imag, pb.imag - pc.imag
    return acx * bcy - acy * bcx


def is_collinear(pa, pb, pc):
    return abs(orientation(pa, pb, pc)) < EPS


def is_points_into(p1, p2, p3, uv):
    return orientation(p1, p2, uv) > EPS and orientation(p1, p3, uv) < EPS


def is_inside_triangle(pa, pb, pc, uv):
    return orientation(pa, pb, uv) > EPS and orientation(pb, pc, uv) > EPS and orientation(pc, pa, uv) > EPS


def nearby_grid1(x, d):
    """nearby_grid(double, double) (common.h:131-137)."""
    if d == 0:
        return x
    f = abs(math.fmod(x, 1.0))
    if f < EPS or 1 - f < EPS:
        x += d * EPS
    return float(math.ceil(x) if d > 0 else math.floor(x))


def nearby_grid(uv, d=None):
    if d is None:
        return complex(std_round(uv.real), std_round(uv.imag))
    return complex(nearby_grid1(uv.real, d.real), nearby_grid1(uv.imag, d.imag))


def calc_coefficient(o, p1, p2, t):
    """common/utilities.h:109-123 with Eigen's 2x2 inverse."""
    v1, v2, d = csub(p1, o), csub(p2, o), csub(t, o)
    m00, m01, m10, m11 = v1.real, v2.real, v1.imag, v2.imag
    det = m00 * m11 - m10 * m01
    inv = 1.0 / det
    i00, i10, i01, i11 = m11 * inv, -m10 * inv, -m01 * inv, m00 * inv
    return complex(i00 * d.real + i01 * d.imag, i10 * d.real + i11 * d.imag)


def conversion(o2, a2, b2, o3, a3, b3, uv):
    """conversion_2d_3d (hmesh/utilities.h:23-34)."""
    c = calc_coefficient(o2, a2, b2, uv)
    return v_add(v_add(o3, v_scale(v_sub(a3, o3), c.real)), v_scale(v_sub(b3, o3), c.imag))


class Qex:
    """example_qex.cpp:125-205 after the parameterisation: sanitization, q-vertices, q-ports,
    q-edges, q-faces."""

    def __init__(self, hm, cfn, matching, singular, N=4):
        self.m = m = Mesh(hm)
        self.F = [[int(v) for v in row] for row in hm.idx]
        self.P = [tuple(float(c) for c in row) for row in hm.pos]
        self.nV, self.nF, self.nE = hm.nV, hm.nF, hm.nE
        self.matching = [int(v) for v in matching]
        self.singular = [int(v) for v in singular]
        self.N = N
        cfn = [complex(c) for c in cfn]
        self.cfn = self.sanitization(cfn)

    # ---- helpers on the halfedge mesh
    def cvert(self, c):
        return self.F[c // 3][c % 3]

    def conv_face(self, f, uv):
        m = self.m
        h = m.f2h[f]
        c1, c2, c3 = m.crnr[h], m.crnr[m.next[h]], m.crnr[m.prev[h]]
        cf = self.cfn
        return conversion(cf[c1], cf[c2], cf[c3], self.P[self.cvert(c1)], self.P[self.cvert(c2)], self.P[self.cvert(c3)], uv)

    def trs(self, cfn):
        """compute_trs_matrix (common.h:72-89): per halfedge, the map r uv + t from its face to its
        twin's."""
        m, N = self.m, self.N
        R, T = [], []
        for h in range(len(m.next)):
            uv1 = cfn[m.crnr[m.next[h]]]
            uv2 = cfn[m.crnr[m.prev[m.twin[h]]]]
            mm = (1 if m.canonical(h) else -1) * self.matching[m.edge[h]]
            mm = (N + int(math.fmod(mm, N))) % N if mm < 0 else mm % N
            r = quater_rot(mm)
            t = csub(uv2, cmul(r, uv1))
            R.append(r)
            T.append(complex(std_round(t.real), std_round(t.imag)))
        return R, T

    def sanitization(self, cfn):
        """qex/sanitization.h:11-56: per vertex, the first corner of its ring is snapped (to the
        grid at a singular vertex, to the precision of the ring's largest coordinate elsewhere)
        and the others are its transports across the ring's edges."""
        m = self.m
        R, T = self.trs(cfn)
        cfn = list(cfn)
        for v in range(self.nV):
            mx = 0.0
            ring = list(m.vert_halfs(v))
            for h in ring:
                uv = cfn[m.crnr[m.next[h]]]
                mx = max(mx, abs(uv.real))
                mx = max(mx, abs(uv.imag))
            for k, h in enumerate(ring):
                cc = m.crnr[m.next[h]]
                if k == 0:
                    uv = cfn[cc]
                    if self.singular[v]:
                        cfn[cc] = complex(std_round(uv.real), std_round(uv.imag))
                    else:
                        delta = math.pow(2.0, math.log2(mx)) if mx > 0 else 0.0
                        sign = complex(float((0 < uv.real) - (uv.real < 0)), float((0 < uv.imag) - (uv.imag < 0)))
                        ds = cscale(sign, delta)
                        cfn[cc] = csub(cadd(cfn[cc], ds), ds)
                else:
                    cp = m.crnr[m.prev[m.twin[h]]]
                    tw = m.twin[h]
                    cfn[cc] = cadd(cmul(R[tw], cfn[cp]), T[tw])
        return cfn

    # ---- gen_q_vert.h:11-59
    def q_verts(self):
        m, cfn = self.m, self.cfn
        vq, eq, fq = [], [], []
        for v in range(self.nV):
            uv = cfn[m.crnr[m.next[m.v2h[v]]]]
            x = math.fmod(abs(uv.real), 1.0)
            y = math.fmod(abs(uv.imag), 1.0)
            if (x < EPS or 1 - x < EPS) and (y < EPS or 1 - y < EPS):
                vq.append((complex(x, y), self.P[v], v))
        for e in range(self.nE):
            h = m.e2h[e]
            p1, p2 = self.P[m.tail[h]], self.P[m.head[h]]
            uv1, uv2 = cfn[m.crnr[m.next[h]]], cfn[m.crnr[m.prev[h]]]
            x0, y0 = math.floor(min(uv1.real, uv2.real)), math.floor(min(uv1.imag, uv2.imag))
            x1, y1 = math.ceil(max(uv1.real, uv2.real)), math.ceil(max(uv1.imag, uv2.imag))
            for x in range(x0, x1 + 1):
                for y in range(y0, y1 + 1):
                    xy = complex(float(x), float(y))
                    a = abs(csub(xy, uv1)) / abs(csub(uv2, uv1))
                    if is_collinear(uv1, uv2, xy) and a > EPS and a < 1 - EPS:
                        eq.append((xy, v_add(p1, v_scale(v_sub(p2, p1), a)), e))
        for f in range(self.nF):
            p = [self.P[self.F[f][j]] for j in range(3)]
            uv = [cfn[3 * f + j] for j in range(3)]
            x0 = math.floor(min(u.real for u in uv))
            y0 = math.floor(min(u.imag for u in uv))
            x1 = math.ceil(max(u.real for u in uv))
            y1 = math.ceil(max(u.imag for u in uv))
            for x in range(x0, x1 + 1):
                for y in range(y0, y1 + 1):
                    xy = complex(float(x), float(y))
                    pos = conversion(uv[0], uv[1], uv[2], p[0], p[1], p[2], xy)
                    if is_inside_triangle(uv[0], uv[1], uv[2], xy):
                        fq.append((xy, pos, f))
        return vq, eq, fq

    # ---- gen_q_port.h (ports: dict idx, vid, eid, fid, uv, dir, pos, conn, next, prev)
    def q_ports(self, vq, eq, fq):
        m, cfn = self.m, self.cfn
        ports = []

        def ring(tmp):
            s = len(tmp)
            for i in range(s):
                tmp[i]["idx"] = len(ports) + i
            for i in range(s):
                tmp[i]["prev"] = tmp[(i - 1 + s) % s]["idx"]
                tmp[i]["next"] = tmp[(i + 1) % s]["idx"]
            ports.extend(tmp)

        for uvq, pos, v in vq:   # generate_vqvert_qport (gen_q_port.h:79-108)
            tmp = []
            for h in m.vert_halfs(v):
                uv1, uv2, uv3 = cfn[m.crnr[m.next[h]]], cfn[m.crnr[m.prev[h]]], cfn[m.crnr[h]]
                r = 0
                while r < 4 and not is_points_into(uv1, uv2, uv3, cadd(uv1, quater_rot(r))):
                    r += 1
                for i in range(4):
                    d = quater_rot((r + i + 3) % 4)
                    f1 = is_points_into(uv1, uv2, uv3, cadd(uv1, d))
                    f2 = is_collinear(uv1, uv2, cadd(uv1, d))
                    f3 = dot(csub(uv2, uv1), d) > 0
                    if f1 or (f2 and f3):
                        tmp.append(dict(vid=v, eid=-1, fid=m.face[h], uv=uv1, dir=d, pos=pos, conn=False))
            ring(tmp)
        visit = []   # shared by every edge q-vertex, as in the reference
        for uvq, pos, e in eq:   # generate_eqvert_qport (gen_q_port.h:11-56)
            tmp = []
            h0 = m.e2h[e]
            for h in (h0, m.twin[h0]):
                c1, c2 = m.crnr[m.next[h]], m.crnr[m.prev[h]]
                uv1, uv2, uv3 = cfn[c1], cfn[c2], cfn[m.crnr[h]]
                p1, p2 = self.P[self.cvert(c1)], self.P[self.cvert(c2)]
                uv = lerp(uv1, uv2, v_norm(v_sub(pos, p1)) / v_norm(v_sub(p2, p1)))
                r = 0
                while r < 4 and not is_points_into(uv1, uv2, uv3, cadd(uv1, quater_rot(r))):
                    r += 1
                for i in range(4):
                    d = quater_rot((r + i + 2) % 4)
                    f1 = orientation(uv1, uv2, cadd(uv, d)) >= 0
                    ev = v_normalized(self.conv_face(m.face[h], cadd(uv, d)))
                    seen = any(v_norm(v_sub(ev, w)) < EPS for w in visit)
                    if f1 and not seen:
                        tmp.append(dict(vid=-1, eid=e, fid=m.face[h], uv=nearby_grid(uv), dir=d, pos=pos, conn=False))
                        visit.append(ev)
            if len(tmp) != 4:
                raise ValueError("an edge q-vertex without four ports")
            ring(tmp)
        for uvq, pos, f in fq:   # generate_fqvert_qport (gen_q_port.h:58-77)
            ring([dict(vid=-1, eid=-1, fid=f, uv=uvq, dir=quater_rot(i), pos=pos, conn=False) for i in range(4)])
        return ports

    # ---- gen_q_edge.h
    def collinear_pair(self, ori, d, f, p):
        """predict_extrinsic_collinear (gen_q_edge.h:11-27)."""
        pb1 = self.conv_face(f, ori)
        pb2 = self.conv_face(f, cadd(ori, d))
        pa1 = self.conv_face(p["fid"], p["uv"])
        pa2 = self.conv_face(p["fid"], cadd(p["uv"], p["dir"]))
        da = v_normalized(v_sub(pa2, pa1))
        db = v_normalized(v_sub(pb2, pb1))
        dc = v_normalized(v_sub(pa1, pb1))
        return abs(1.0 - v_dot(db, dc)) < EPS and abs(1.0 + v_dot(da, db)) < EPS

    def next_half(self, ori, d, f):
        """pick_next_half (gen_q_edge.h:29-43)."""
        m, cfn = self.m, self.cfn
        for h in m.face_halfs(f):
            uv1, uv2 = cfn[m.crnr[m.next[h]]], cfn[m.crnr[m.prev[h]]]
            r = extended_intersection(ori, cadd(ori, cscale(d, 1e2)), uv1, uv2)
            if r is not None and 0 < r[0] < 1 and 0 < r[1] < 1 and r[0] > EPS:
                return h, lerp(uv1, uv2, r[1])
        raise ValueError("no next half found")

    def q_edges(self, ports, max_steps=None):
        """generate_q_edge (gen_q_edge.h:45-121): from every port not yet connected, walk the grid
        line across faces (mapping uv by the edge transitions) until a face, edge or vertex port
        facing it is found."""
        m, cfn = self.m, self.cfn
        R, T = self.trs(cfn)
        cap = max_steps if max_steps is not None else 4 * self.nF + 16
        # the reference's searches run over all ports in index order with a face, edge or
        # vertex condition; buckets in index order give the same first match
        by_face, by_edge, by_vert = {}, {}, {}
        for p in ports:
            by_face.setdefault(p["fid"], []).append(p)
            if p["eid"] >= 0:
                by_edge.setdefault(p["eid"], []).append(p)
            if p["vid"] >= 0:
                by_vert.setdefault(p["vid"], []).append(p)
        edges = []
        for pfr in ports:
            if pfr["conn"]:
                continue
            ori, d = pfr["uv"], pfr["dir"]
            gri = nearby_grid(ori, d)
            f = pfr["fid"]
            steps = 0
            while True:
                hit = None
                if is_inside_triangle(cfn[3 * f], cfn[3 * f + 1], cfn[3 * f + 2], gri):
                    nd = complex(-d.real, -d.imag)
                    for p in by_face.get(f, ()):
                        if p["idx"] == pfr["idx"]:
                            continue
                        if abs(csub(p["dir"], nd)) < 1e-10 and abs(csub(p["uv"], gri)) < EPS:
                            hit = p
                            break
                    if hit is None:
                        raise ValueError("face q-port not found")
                if hit is None:
                    for h in m.face_halfs(f):
                        for p in by_edge.get(m.edge[h], ()):
                            if p["conn"] or p["eid"] == pfr["eid"]:
                                continue
                            if self.collinear_pair(ori, d, f, p):
                                hit = p
                                break
                        if hit is not None:
                            break
                if hit is None:
                    for h in m.face_halfs(f):
                        for p in by_vert.get(m.tail[h], ()):
                            if p["conn"] or p["vid"] == pfr["vid"]:
                                continue
                            if self.collinear_pair(ori, d, f, p):
                                hit = p
                                break
                        if hit is not None:
                            break
                if hit is not None:
                    pfr["conn"] = hit["conn"] = True
                    edges.append((pfr["idx"], hit["idx"]))
                    break
                nh, pt = self.next_half(ori, d, f)
                f = m.face[m.twin[nh]]
                ori = cadd(cmul(R[nh], pt), T[nh])
                d = cmul(R[nh], d)
                gri = nearby_grid(ori, d)
                steps += 1
                if steps > cap:
                    raise RuntimeError("q-edge trace does not close")
        return edges

    @staticmethod
    def q_faces(ports, edges):
        """generate_q_faces (gen_q_face.h:8-40): half-edges 2i (port1 -> port2) and 2i + 1; from
        each unvisited one, three steps to the half-edge starting at the previous port of the
        one it arrives at; quads of four kept."""
        qh = []
        for i, (a, b) in enumerate(edges):
            qh.append((a, b))
            qh.append((b, a))
        by_start = {}
        for k, (a, b) in enumerate(qh):
            by_start.setdefault(a, k)
        visit = [False] * len(qh)
        faces = []
        for k0 in range(len(qh)):
            if visit[k0]:
                continue
            fh = [k0]
            visit[k0] = True
            q = qh[k0][1]
            for _ in range(3):
                k = by_start.get(ports[q]["prev"])
                if k is None:
                    break
                fh.append(k)
                visit[k] = True
                q = qh[k][1]
            if len(fh) == 4:
                faces.append(fh)
        return faces

    def run(self):
        vq, eq, fq = self.q_verts()
        ports = self.q_ports(vq, eq, fq)
        edges = self.q_edges(ports)
        faces = self.q_faces(ports, edges)
        return dict(vq=vq, eq=eq, fq=fq, ports=ports, edges=edges, faces=faces, cfn=self.cfn)
