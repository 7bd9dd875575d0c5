"""Test infrastructure: CPU restatement of the reference's motorcycle graph and T-mesh
(include/metriko/core/tmesh/motorcycle.h, tmesh.h of komietty/metriko) and of the geometric
helpers they call (core/common/utilities.h, core/hmesh/utilities.h).  Used only by tests/ as
the checker of the header-only C++ implementation (include/metriko/core/tmesh/); nothing in the
product imports it.  Parity unpinned: the reference needs Eigen and libigl, which this
environment does not have, so this restatement is checked against the C++ port and against the
reference's invariants (every curve ends in a crash, every T-quad has four sides, every T-edge
has two half-edges on two quads or twice on one).

Floating-point operations follow the reference's expressions in order (complex products as
(ac - bd, ad + bc), lerp as a (1 - t) + b t, the 2x2 inverse of find_extended_intersection as
Eigen's cofactor form), so the C++ port compiled without floating-point contraction gives the
same bits."""
import cmath
import math

NONE, HIT_L, HIT_R, HIT_B = 0, 1, 2, 3


# ---------------------------------------------------------------- utilities.h (common)
def quater_rot(i):
    """get_quater_rot (common/utilities.h:11-19)."""
    return (1 + 0j, 1j, -1 + 0j, -1j)[(i % 4 + 4) % 4]


def cross(a, b):
    return a.real * b.imag - a.imag * b.real


def dot(a, b):
    return a.real * b.real + a.imag * b.imag


def lerp(a, b, t):
    """common/utilities.h:29-35: a (1 - t) + b t, componentwise."""
    s = 1.0 - t
    return complex(a.real * s + b.real * t, a.imag * s + b.imag * t)


def cmul(a, b):
    """std::complex<double> product (ac - bd, ad + bc)."""
    return complex(a.real * b.real - a.imag * b.imag, a.real * b.imag + a.imag * b.real)


def csub(a, b):
    return complex(a.real - b.real, a.imag - b.imag)


def cadd(a, b):
    return complex(a.real + b.real, a.imag + b.imag)


def isccw(a, b, c):
    """common/utilities.h:60-70."""
    return cross(csub(b, a), csub(c, a)) > 0


def orientation(a, b, c):
    return cross(csub(b, a), csub(c, a))


def points_into(d, a, b, c):
    """common/utilities.h:82-89."""
    ad = cadd(a, d)
    return isccw(a, b, ad) and isccw(a, ad, c)


def extended_intersection(a, b, c, d):
    """find_extended_intersection (common/utilities.h:127-142): the lines a-b and c-d; returns
    (ratio along a->b, ratio along c->d) or None for parallel lines.  The 2x2 system and its
    inverse as Eigen evaluates them (determinant m00 m11 - m10 m01, inverse = cofactors times
    1/det, product rows as m_i0 r0 + m_i1 r1)."""
    ba = csub(b, a)
    m00, m01 = d.real - c.real, -ba.real
    m10, m11 = d.imag - c.imag, -ba.imag
    det = m00 * m11 - m10 * m01
    if det == 0:
        return None
    inv = 1.0 / det
    i00, i10, i01, i11 = m11 * inv, -m10 * inv, -m01 * inv, m00 * inv
    r0, r1 = -c.real + a.real, -c.imag + a.imag
    v0 = i00 * r0 + i01 * r1
    v1 = i10 * r0 + i11 * r1
    return v1, v0


def strict_intersection(a, b, c, d):
    """find_strict_intersection (common/utilities.h:144-157)."""
    r = extended_intersection(a, b, c, d)
    if r is None:
        return None
    ab, cd = r
    if ab > 0 and ab < 1 and cd > 0 and cd < 1:
        return ab, cd
    return None


def equal(a, b, tol=1e-10):
    return abs(csub(a, b)) < tol


# ---------------------------------------------------------------- halfedge helpers
class Mesh:
    """The halfedge arrays of oracle.metriko_oracle.Hmesh plus corners: crnr(h) = 3 f + it with
    F[f, it] the vertex opposite h (hmesh.h:429-441)."""

    def __init__(self, hm):
        self.hm = hm
        F = hm.idx
        nH = len(hm.next)
        self.crnr = [-1] * nH
        for h in range(3 * hm.nF):
            f = int(hm.face[h])
            opp = int(hm.tail[hm.prev[h]])
            for it in range(3):
                if int(F[f, it]) == opp:
                    self.crnr[h] = 3 * f + it
        self.next = [int(v) for v in hm.next]
        self.prev = [int(v) for v in hm.prev]
        self.twin = [int(v) for v in hm.twin]
        self.tail = [int(v) for v in hm.tail]
        self.head = [int(v) for v in hm.head]
        self.face = [int(v) for v in hm.face]
        self.edge = [int(v) for v in hm.edge]
        self.v2h = [int(v) for v in hm.vert2half]
        self.f2h = [int(v) for v in hm.face2half]
        self.e2h = [int(v) for v in hm.edge2half]

    def vert_halfs(self, v):
        """Vert::adjHalfs() (ccw): from vert2half, h <- twin(prev(h)) (hmesh.h:158-161)."""
        h0 = self.v2h[v]
        h = h0
        while True:
            yield h
            h = self.twin[self.prev[h]]
            if h == h0:
                return

    def face_halfs(self, f):
        """Face::adjHalfs() (ccw): from face2half, h <- next(h)."""
        h0 = self.f2h[f]
        return [h0, self.next[h0], self.next[self.next[h0]]]

    def canonical(self, h):
        return self.e2h[self.edge[h]] == h


def opposite_half(m, cfn, origin, d, fr):
    """get_oppsite_half (hmesh/utilities.h:54-73)."""
    for h in m.face_halfs(m.face[fr]):
        if h == fr:
            continue
        a = csub(cfn[m.crnr[m.prev[h]]], origin)
        b = csub(cfn[m.crnr[m.next[h]]], origin)
        if cross(a, d) * cross(b, d) < 0:
            return h
    raise ValueError("the trace leaves no edge of the face strictly")


# ---------------------------------------------------------------- motorcycle.h
class Vert:
    __slots__ = ("uv", "crash", "type")

    def __init__(self, uv, crash=-1, typ=NONE):
        self.uv, self.crash, self.type = uv, crash, typ


class Sgmt:
    __slots__ = ("curv", "face", "fr", "to", "id", "prev_id", "next_id")

    def __init__(self, curv, face, fr, to):
        self.curv, self.face, self.fr, self.to = curv, face, fr, to
        self.id = self.prev_id = self.next_id = -1

    def same(self, o):
        """Msgmt::operator== (motorcycle.h:75-80): face and both end uv's."""
        return self.face == o.face and self.fr.uv == o.fr.uv and self.to.uv == o.to.uv

    def diff(self):
        return csub(self.to.uv, self.fr.uv)


class Curve:
    def __init__(self, port):
        self.port = port
        self.sgmts = []
        self.half, self.ratio, self.dir, self.intersected = -1, 0.0, 0j, False


def gen_ports(m, cfn, singular):
    """MotorcycleGraph::gen_ports (motorcycle.h:166-212): per singular vertex (in id order), per
    halfedge of its ring, the axis directions that leave into the face (or run along one of its
    two edges at the vertex), ordered by their projection on the first edge; ports of a vertex
    are linked in a ring."""
    ports = []
    counter = 0
    for v in range(m.hm.nV):
        if singular[v] == 0:
            continue
        vp = []
        for h in m.vert_halfs(v):
            a = cfn[m.crnr[m.next[h]]]
            b = cfn[m.crnr[m.prev[h]]]
            c = cfn[m.crnr[h]]
            if orientation(a, b, c) < 0:
                raise ValueError("Orientation should be ccw order")
            r = 0
            while r < 4:
                if not points_into(quater_rot(r), a, b, c) and r > 0:
                    break
                r += 1
            temps = []
            ba, ca = csub(b, a), csub(c, a)
            for i in range(4):
                d = quater_rot(r - i)
                if points_into(d, a, b, c) or cmath.phase(d) == cmath.phase(ba) or cmath.phase(d) == cmath.phase(ca):
                    temps.append(dict(id=-1, vert=v, face=m.face[h], uv=a, dir=d))
            temps = sorted(temps, key=lambda p: -dot(p["dir"], ba))
            for p in temps:
                p["id"] = counter
                counter += 1
            vp.extend(temps)
        s = len(vp)
        for i in range(s):
            vp[i]["prev"] = vp[(i - 1 + s) % s]["id"]
            vp[i]["next"] = vp[(i + 1 + s) % s]["id"]
        ports.extend(vp)
    return ports


def split_segment(curves, ci, target, crash, ratio):
    """Mcurv::split_segment (motorcycle.h:108-124)."""
    sg = curves[ci].sgmts
    for k, s in enumerate(sg):
        if s.same(target):
            ccw = cross(crash.diff(), s.diff()) > 0
            uv = lerp(s.fr.uv, s.to.uv, ratio)
            fr = Vert(uv, crash.curv, HIT_L if ccw else HIT_R)
            to = Vert(s.to.uv, s.to.crash, s.to.type)
            s.to = Vert(uv, crash.curv, HIT_R if ccw else HIT_L)
            sg.insert(k + 1, Sgmt(ci, s.face, fr, to))
            return
    raise ValueError("split target not found")


def add_segment(m, cfn, curves, ci, d, uv0, h):
    """Mcurv::add_segment (motorcycle.h:250-291)."""
    uv1 = cfn[m.crnr[m.prev[h]]]
    uv2 = cfn[m.crnr[m.next[h]]]
    r = extended_intersection(uv0, cadd(uv0, d), uv1, uv2)
    if r is None:
        raise ValueError("trace parallel to the exit edge")
    r_cd = r[1]
    uv3 = lerp(uv1, uv2, r_cd)
    face = m.face[h]
    best = None
    for cj, cv in enumerate(curves):
        if cj == ci:
            continue
        for s in cv.sgmts:
            if s.face != face:
                continue
            it = strict_intersection(uv0, uv3, s.fr.uv, s.to.uv)
            if it is not None and (best is None or it[0] < best[0]):
                best = (it[0], it[1], s)
    cur = curves[ci]
    if best is None:
        cur.sgmts.append(Sgmt(ci, face, Vert(uv0), Vert(uv3)))
        cur.half, cur.ratio, cur.dir, cur.intersected = h, r_cd, d, False
    else:
        ab, cd, s = best
        seg = Sgmt(ci, face, Vert(uv0), Vert(lerp(uv0, uv3, ab), s.curv, HIT_B))
        cur.sgmts.append(seg)
        cur.half, cur.ratio, cur.dir, cur.intersected = h, r_cd, d, True
        split_segment(curves, s.curv, s, seg, cd)


def motorcycle_graph(hm, cfn, matching, singular, max_segments=None):
    """MotorcycleGraph(mesh, cfn, matching, singular) (motorcycle.h:136-156).  cfn: 3 nF complex
    corner values (corner j of face f at 3 f + j); matching: per edge; singular: per vertex."""
    m = Mesh(hm)
    cfn = [complex(c) for c in cfn]
    ports = gen_ports(m, cfn, singular)
    curves = [Curve(p) for p in ports]
    for ci, cv in enumerate(curves):   # add_segment_init (motorcycle.h:215-227)
        p = cv.port
        h = -1
        for h_ in m.face_halfs(p["face"]):
            if m.head[h_] != p["vert"] and m.tail[h_] != p["vert"]:
                h = h_
        add_segment(m, cfn, curves, ci, p["dir"], p["uv"], h)
    cap = max_segments if max_segments is not None else 64 * (len(m.face) + 16)
    while any(not c.intersected for c in curves):
        for ci, cv in enumerate(curves):   # add_segment_next (motorcycle.h:230-247)
            if cv.intersected:
                continue
            h = m.twin[cv.half]
            mt = (1 if m.canonical(h) else -1) * int(matching[m.edge[h]])
            uv0 = lerp(cfn[m.crnr[m.next[h]]], cfn[m.crnr[m.prev[h]]], cv.ratio)
            d = cmul(cmath.rect(1.0, math.pi / 2 * mt), cv.dir)
            oh = opposite_half(m, cfn, uv0, d, h)
            add_segment(m, cfn, curves, ci, d, uv0, oh)
        if sum(len(c.sgmts) for c in curves) > cap:
            raise RuntimeError("motorcycle graph: traces do not close")
    for cv in curves:   # Mcurv::post_process (motorcycle.h:126-133)
        for i, s in enumerate(cv.sgmts):
            s.id = i
        for i in range(len(cv.sgmts) - 1):
            cv.sgmts[i].next_id = i + 1
            cv.sgmts[i + 1].prev_id = i
    return ports, curves


# ---------------------------------------------------------------- tmesh.h
def tmesh(ports, curves):
    """Tmesh(mcurvs) (tmesh.h:161-205): T-edges between consecutive crash vertices of every
    curve (two T-half-edges each, canonical first), T-quads by walking choose_next_thalf, and
    the per-half-edge quad, side, position and singular-vertex tables."""
    tedges = []      # (curve, seg_fr, seg_to) as Sgmt copies
    for ci, cv in enumerate(curves):
        start = cv.sgmts[0]
        for s in cv.sgmts:
            if s.to.type != NONE:
                tedges.append((ci, start, s))
                if s.next_id != -1:
                    start = cv.sgmts[s.next_id]
    nTE = len(tedges)
    thalfs = [(k // 2, k % 2 == 0) for k in range(2 * nTE)]   # (tedge, canonical)

    def find_th(ms, canonical):
        for th, (te, can) in enumerate(thalfs):
            if can == canonical and (tedges[te][1].same(ms) or tedges[te][2].same(ms)):
                return th
        raise ValueError("thalf not found")

    def choose_next(cur):
        """Tquad::choose_next_thalf (tmesh.h:260-305)."""
        te_i, can = thalfs[cur]
        ci, sfr, sto = tedges[te_i]
        if can:
            if sto.to.type == HIT_B:
                for ms in curves[sto.to.crash].sgmts:
                    if ms.face == sto.face:
                        uv2 = sto.to.uv
                        dif = sto.diff()
                        if equal(ms.fr.uv, uv2) and cross(dif, ms.diff()) > 0:
                            return find_th(ms, True), True
                        if equal(ms.to.uv, uv2) and cross(dif, -ms.diff()) > 0:
                            return find_th(ms, False), True
                raise ValueError("thalf not found")
            if sto.to.type == HIT_R:
                return find_th(curves[sto.to.crash].sgmts[-1], False), True
            return cur + 2, False
        if sfr.same(curves[sfr.curv].sgmts[0]):
            return find_th(curves[curves[sfr.curv].port["prev"]].sgmts[0], True), True
        if sfr.fr.type == HIT_R:
            return find_th(curves[sfr.fr.crash].sgmts[-1], False), True
        return cur - 2, False

    tquads = []
    visit = [False] * len(thalfs)
    while not all(visit):
        bgn = visit.index(False)
        thids, sides = [], []
        side, cur = 0, bgn
        guard = 0
        while True:
            thids.append(cur)
            sides.append(side)
            nxt, turn = choose_next(cur)
            if turn:
                side = (side + 1) % 4
            cur = nxt
            guard += 1
            if cur == bgn:
                break
            if guard > len(thalfs) + 4:
                raise RuntimeError("T-quad walk does not close")
        if sides[0] == sides[-1]:
            n = 0
            while n < len(sides) and sides[n] == sides[0]:
                n += 1
            sides = sides[n:] + sides[:n]
            thids = thids[n:] + thids[:n]
        if sides[0] == sides[-1]:
            raise ValueError("T-quad with one side")
        tquads.append((thids, sides))
        for t in thids:
            visit[t] = True
    nTH = len(thalfs)
    th2quad, th2side, th2iter = [0] * nTH, [0] * nTH, [0] * nTH
    for q, (thids, sides) in enumerate(tquads):
        for j, t in enumerate(thids):
            th2quad[t], th2side[t], th2iter[t] = q, sides[j], j
    th2sing = [-1] * nTH
    for ci, cv in enumerate(curves):
        for th, (te, can) in enumerate(thalfs):
            if tedges[te][1].same(cv.sgmts[0]):
                th2sing[th] = cv.port["vert"]
                break
    return dict(tedges=tedges, thalfs=thalfs, tquads=tquads, th2quad=th2quad, th2side=th2side,
                th2iter=th2iter, th2sing=th2sing)


def tedge_lengths(curves, tm):
    """example_qgp.cpp:84-94: R[i] = sum of |segment| from seg_fr to seg_to of T-edge i."""
    R = []
    for ci, sfr, sto in tm["tedges"]:
        s = 0.0
        on = False
        for seg in curves[ci].sgmts:
            if seg.same(sfr):
                on = True
            if on:
                s += abs(seg.diff())
                if seg.same(sto):
                    break
        R.append(s)
    return R
