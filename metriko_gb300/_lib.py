"""ctypes binding of libmetriko_cuda.so (C ABI declared in include/metriko_cuda.h).

The library is the product: there is no CPU fallback.  Loading fails loudly when the shared
library is missing, and every call raises MetrikoError on a non-zero status.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libmetriko_cuda.so"

OK, BAD_INPUT, CUDA, NOT_CONVERGED, BREAKDOWN, TIMEOUT, NO_DEVICE, ROUNDING = range(8)
PREC_FP64, PREC_MIXED = 0, 1

# every symbol include/metriko_cuda.h declares
EXPORTS = [
    "mtk_status_string", "mtk_last_error", "mtk_default_opts", "mtk_ctx_create", "mtk_ctx_destroy",
    "mtk_ctx_kernel_count", "mtk_field_smoothest", "mtk_iterative_rounding", "mtk_pipeline_run",
    "mtk_seeded_init", "mtk_topology_from_field", "mtk_field_smoothest_noalloc", "mtk_size_field_gradient",
    "mtk_pipeline_size_field_gradient", "mtk_field_solve", "mtk_field_inputs", "mtk_field_spmv_bench",
    "mtk_injective_barrier", "mtk_local_injectivity", "mtk_map_deviation",
    "mtk_mesh_geometry", "mtk_ctx_set_wait_limit", "mtk_pipeline_position_gradient", "mtk_size_field_position_partials",
    "mtk_field_power_adjoint", "mtk_face_geometry_backward", "mtk_csr_create", "mtk_csr_destroy", "mtk_csr_pcg",
    "mtk_csr_smallest_eig", "mtk_curl_matching", "mtk_mesh_field_inputs", "mtk_field_smoothest_mesh",
    "mtk_seam_paths", "mtk_comb_turns",
]


class MetrikoError(RuntimeError):
    def __init__(self, status, what, detail=""):
        super().__init__(f"{what}: status {status} ({detail})")
        self.status = status


class SolveOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("tol", C.c_double), ("max_iter", C.c_int32),
                ("max_refine", C.c_int32), ("inner_tol", C.c_double)]


class Stats(C.Structure):
    _fields_ = [("pcg_iters", C.c_int64), ("solves", C.c_int64), ("refinements", C.c_int64),
                ("spmv_calls", C.c_int64), ("kernel_launches", C.c_int64),
                ("max_rel_residual", C.c_double), ("ms_field", C.c_double),
                ("ms_integrate", C.c_double), ("ms_rounding", C.c_double), ("ms_host", C.c_double),
                ("ms_total", C.c_double), ("resolves", C.c_int64), ("lm_iterations", C.c_int64),
                ("min_order_margin", C.c_double), ("field_pcg_launches", C.c_int64),
                ("field_pcg_ms", C.c_double), ("field_pcg_bytes", C.c_double), ("igm_pcg_launches", C.c_int64),
                ("igm_pcg_ms", C.c_double), ("igm_pcg_bytes", C.c_double),
                ("strict_order_differs", C.c_int64), ("strict_order_gap", C.c_double),
                ("integral_order_differs", C.c_int64), ("field_pcg_passes", C.c_int64),
                ("igm_pcg_passes", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class PipelineOpts(C.Structure):
    _fields_ = [("seed", C.c_int32), ("n_iter", C.c_int32), ("ratio", C.c_double),
                ("round_seams", C.c_int32), ("seamless", C.c_int32), ("stop_after", C.c_int32),
                ("field_type", C.c_int32), ("local_injectivity", C.c_int32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() (nvcc, sm_103a)")
        L = C.CDLL(str(LIB_PATH))
        L.mtk_status_string.restype = C.c_char_p
        L.mtk_status_string.argtypes = [C.c_int]
        L.mtk_last_error.restype = C.c_char_p
        L.mtk_default_opts.argtypes = [C.POINTER(SolveOpts)]
        L.mtk_ctx_create.argtypes = [C.c_int, C.POINTER(C.c_void_p)]
        L.mtk_ctx_destroy.argtypes = [C.c_void_p]
        L.mtk_ctx_kernel_count.argtypes = [C.c_void_p]
        L.mtk_ctx_kernel_count.restype = C.c_int64
        L.mtk_ctx_set_wait_limit.argtypes = [C.c_void_p, C.c_int64]
        L.mtk_seeded_init.argtypes = [C.c_int32, C.c_int32, C.c_void_p]
        L.mtk_field_smoothest.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_int32, C.POINTER(SolveOpts), C.c_void_p,
                                          C.POINTER(Stats)]
        L.mtk_pipeline_run.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                       C.POINTER(PipelineOpts), C.POINTER(SolveOpts)] + [C.c_void_p] * 7 + \
                                      [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p,
                                       C.c_void_p, C.POINTER(Stats)]
        L.mtk_topology_from_field.argtypes = [C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                              C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_void_p]
        L.mtk_field_smoothest_noalloc.argtypes = [C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                                  C.c_void_p, C.c_int32, C.c_double, C.c_int32, C.c_void_p,
                                                  C.c_void_p, C.POINTER(C.c_int32)]
        L.mtk_field_inputs.argtypes = [C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.mtk_field_spmv_bench.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32,
                                           C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                           C.POINTER(C.c_double)]
        L.mtk_injective_barrier.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32,
                                            C.c_void_p, C.c_void_p, C.c_void_p]
        L.mtk_local_injectivity.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.POINTER(C.c_int32),
                                            C.POINTER(C.c_int32)]
        L.mtk_mesh_geometry.argtypes = [C.c_int32, C.c_int32] + [C.c_void_p] * 12
        L.mtk_map_deviation.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.POINTER(C.c_double)]
        L.mtk_field_solve.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.POINTER(SolveOpts), C.c_void_p, C.POINTER(Stats)]
        L.mtk_pipeline_size_field_gradient.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                                       C.POINTER(PipelineOpts), C.POINTER(SolveOpts), C.c_void_p,
                                                       C.c_void_p, C.c_double, C.POINTER(C.c_double), C.c_void_p,
                                                       C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(Stats)]
        L.mtk_pipeline_position_gradient.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                                     C.POINTER(PipelineOpts), C.POINTER(SolveOpts), C.c_void_p,
                                                     C.c_double, C.POINTER(C.c_double), C.c_void_p, C.c_void_p,
                                                     C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(Stats)]
        L.mtk_field_power_adjoint.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_int32, C.POINTER(SolveOpts), C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_void_p, C.POINTER(Stats)]
        L.mtk_face_geometry_backward.argtypes = [C.c_void_p, C.c_int32, C.c_int32] + [C.c_void_p] * 8
        L.mtk_csr_create.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                     C.POINTER(C.c_void_p)]
        L.mtk_csr_destroy.argtypes = [C.c_void_p]
        L.mtk_csr_pcg.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.POINTER(SolveOpts),
                                  C.POINTER(Stats)]
        L.mtk_csr_smallest_eig.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                           C.POINTER(SolveOpts), C.c_void_p, C.POINTER(Stats)]
        L.mtk_curl_matching.argtypes = [C.c_void_p] + [C.c_int32] * 4 + [C.c_void_p] * 13
        L.mtk_mesh_field_inputs.argtypes = [C.c_void_p, C.c_int32, C.c_int32] + [C.c_void_p] * 5
        L.mtk_seam_paths.argtypes = [C.c_void_p, C.c_int32, C.c_int32] + [C.c_void_p] * 3 + [C.c_int32] + [C.c_void_p] * 3
        L.mtk_comb_turns.argtypes = [C.c_void_p, C.c_int32, C.c_int32] + [C.c_void_p] * 3
        L.mtk_field_smoothest_mesh.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32,
                                               C.c_void_p, C.c_int32, C.POINTER(SolveOpts), C.c_void_p,
                                               C.POINTER(Stats)]
        _lib = L
    return _lib


def _check(status, what):
    if status != OK:
        L = lib()
        raise MetrikoError(status, what, f"{L.mtk_status_string(status).decode()}: {L.mtk_last_error().decode()}")


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def num_edges(F):
    """Number of distinct undirected edges of a triangle mesh (3 nF / 2 when it is closed)."""
    F = np.asarray(F, np.int64)
    e = np.sort(np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), axis=1)
    return int(len(np.unique(e[:, 0] * (int(F.max()) + 1) + e[:, 1]))) if len(F) else 0


def solve_opts(precision="mixed", tol=1e-8, max_iter=50000, max_refine=12, inner_tol=3e-6):
    o = SolveOpts()
    lib().mtk_default_opts(C.byref(o))
    o.precision = PREC_MIXED if precision == "mixed" else PREC_FP64
    o.tol, o.max_iter, o.max_refine, o.inner_tol = tol, max_iter, max_refine, inner_tol
    return o


class Context:
    """One CUDA device + stream (mtk_ctx)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        _check(lib().mtk_ctx_create(device, C.byref(h)), "mtk_ctx_create")
        self.handle = h

    def close(self):
        if self.handle:
            lib().mtk_ctx_destroy(self.handle)
            self.handle = None

    def kernel_count(self):
        return int(lib().mtk_ctx_kernel_count(self.handle))

    def set_wait_limit(self, polls: int):
        """Polls of a grid-barrier wait before the call gives up with TIMEOUT (default 2**24)."""
        _check(lib().mtk_ctx_set_wait_limit(self.handle, int(polls)), "mtk_ctx_set_wait_limit")

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def seeded_init(n: int, seed: int = 0) -> np.ndarray:
    out = np.empty(2 * n, np.float64)
    lib().mtk_seeded_init(n, seed, _ptr(out))
    return out[0::2] + 1j * out[1::2]


def field_smoothest(ctx: Context, nbr, theta, area, x0, n_rosy=4, n_iter=50, opts=None):
    """mtk_field_smoothest on face-graph inputs; returns (compressed field, stats dict)."""
    nbr = np.ascontiguousarray(nbr, np.int32).reshape(-1)
    theta = np.ascontiguousarray(theta, np.float64).reshape(-1)
    area = np.ascontiguousarray(area, np.float64)
    nF = len(area)
    x = np.empty(2 * nF)
    x[0::2], x[1::2] = np.real(x0), np.imag(x0)
    out = np.empty(2 * nF)
    st = Stats()
    o = opts or solve_opts()
    _check(lib().mtk_field_smoothest(ctx.handle, nF, n_rosy, _ptr(nbr), _ptr(theta), _ptr(area), _ptr(x), n_iter,
                                     C.byref(o), _ptr(out), C.byref(st)), "mtk_field_smoothest")
    return out[0::2] + 1j * out[1::2], st.as_dict()


def pipeline(ctx: Context, V, F, ratio=0.02, seed=0, round_seams=False, seamless=True, n_iter=50,
             opts=None, stop_after=0, check=True, field_type="smoothest", local_injectivity=False):
    """mtk_pipeline_run: Hmesh -> smoothest field -> Curl matching -> seams -> cut mesh ->
    combing -> RosyParameterization setup()/integ() (example_igm.cpp:13-31)."""
    V = np.ascontiguousarray(V, np.float64)
    F = np.ascontiguousarray(F, np.int32)
    nV, nF = len(V), len(F)
    nE = 3 * nF          # bound on the edge count; the outputs are cut to counts["nE"]
    singular = np.zeros(nV, np.int32)
    matching = np.zeros(nE, np.int32)
    seam = np.zeros(nE, np.uint8)
    compressed = np.zeros(2 * nF)
    cfn = np.zeros(nF * 12)
    cap = 2 * (nV + nE) + 16                      # n (nV + nT) full variables, nT <= nE
    fullx = np.zeros(cap)
    xnaive = np.zeros(cap)
    fix_cap = 2 * (nV + nE) + 16
    fix_order = np.zeros(fix_cap, np.int32)
    fix_vals = np.zeros(fix_cap, np.int32)
    counts = np.zeros(8, np.int32)
    n_full = C.c_int32(0)
    n_fixed = C.c_int32(0)
    p = PipelineOpts(seed, n_iter, ratio, int(round_seams), int(seamless), stop_after,
                     {"smoothest": 0, "curvature_aligned": 1}[field_type], int(local_injectivity))
    o = opts or solve_opts()
    st = Stats()
    status = lib().mtk_pipeline_run(ctx.handle, nV, nF, _ptr(V), _ptr(F), C.byref(p), C.byref(o),
                                    _ptr(singular), _ptr(matching), _ptr(seam), _ptr(compressed), _ptr(cfn),
                                    _ptr(fullx), _ptr(xnaive), cap, C.byref(n_full), _ptr(fix_order),
                                    _ptr(fix_vals), fix_cap, C.byref(n_fixed), _ptr(counts), C.byref(st))
    if check and status not in (OK, ROUNDING):
        _check(status, "mtk_pipeline_run")
    nfull, nfix = n_full.value, n_fixed.value
    ne = int(counts[1])
    return dict(status=status, singular=singular, matching=matching[:ne].copy(), seam=seam[:ne].astype(bool),
                compressed=compressed[0::2] + 1j * compressed[1::2], cfn=cfn.reshape(nF, 12),
                fullx=fullx[:nfull].copy(), x_naive=xnaive[:nfull].copy(),
                fix_order=fix_order[:nfix].copy(), fix_vals=fix_vals[:nfix].copy(),
                counts=dict(zip(["nV", "nE", "nCut", "nT", "nS", "nJ", "nZ", "nFull"], counts.tolist())),
                stats=st.as_dict())


def field_inputs(V, F):
    """mtk_field_inputs: (nbr (nF x 3), theta (nF x 3), area (nF)) of the field operator."""
    V = np.ascontiguousarray(V, np.float64)
    F = np.ascontiguousarray(F, np.int32)
    nF = len(F)
    nbr = np.empty(3 * nF, np.int32)
    theta = np.empty(3 * nF)
    area = np.empty(nF)
    _check(lib().mtk_field_inputs(len(V), nF, _ptr(V), _ptr(F), _ptr(nbr), _ptr(theta), _ptr(area)), "mtk_field_inputs")
    return nbr.reshape(nF, 3), theta.reshape(nF, 3), area


def injective_barrier(ctx: Context, intrinsic_field, field, N=4, update_j=True):
    """mtk_injective_barrier: (f_barrier (nF*N), bar_der (nF*N), s_rows (nF*N x 4)) of
    InjectiveBarrier(N, nF, intrinsic_field).update(field, update_j, ...)."""
    F2 = np.ascontiguousarray(intrinsic_field, np.float64).reshape(-1)
    fd = np.ascontiguousarray(field, np.float64).reshape(-1)
    if F2.size != fd.size or F2.size % (2 * N):
        raise ValueError("fields must have 2*N values per face")
    nF = F2.size // (2 * N)
    fB = np.empty(nF * N)
    dB = np.empty(nF * N) if update_j else None
    S = np.empty(4 * nF * N) if update_j else None
    _check(lib().mtk_injective_barrier(ctx.handle, nF, N, _ptr(F2), _ptr(fd), int(bool(update_j)), _ptr(fB),
                                       _ptr(dB) if update_j else None, _ptr(S) if update_j else None),
           "mtk_injective_barrier")
    return fB, dB, (S.reshape(-1, 4) if update_j else None)


def mesh_geometry(V, F):
    """mtk_mesh_geometry (host only): the vertex and edge geometry of the C++ Hmesh as a dict
    (vertNormal, vertBasisX, vertBasisY, baryDualArea, circDualArea, halfCotan, edgeCotan,
    dihedralArg, heArgOnVert, angleDefect)."""
    V = np.ascontiguousarray(V, np.float64)
    F = np.ascontiguousarray(F, np.int32)
    nV, nF = len(V), len(F)
    nE = num_edges(F)
    out = dict(vertNormal=np.zeros((nV, 3)), vertBasisX=np.zeros((nV, 3)), vertBasisY=np.zeros((nV, 3)),
               baryDualArea=np.zeros(nV), circDualArea=np.zeros(nV), halfCotan=np.zeros(2 * nE),
               edgeCotan=np.zeros(nE), dihedralArg=np.zeros(2 * nE), heArgOnVert=np.zeros(2 * nE),
               angleDefect=np.zeros(nV))
    _check(lib().mtk_mesh_geometry(nV, nF, _ptr(V), _ptr(F), *[_ptr(out[k]) for k in out]), "mtk_mesh_geometry")
    return out


def map_deviation(cutV, cutF, cfn, ext, N=4):
    """mtk_map_deviation (host only): the check at the end of the reference's integ() -- mean over
    faces and functions of |normalized(ext_k) - normalized(3D gradient of function k)|."""
    V = np.ascontiguousarray(cutV, np.float64)
    F = np.ascontiguousarray(cutF, np.int32)
    c = np.ascontiguousarray(cfn, np.float64)
    e = np.ascontiguousarray(ext, np.float64)
    nF = len(F)
    if c.size != 3 * N * nF or e.size != 3 * N * nF:
        raise ValueError("cfn and ext need 3N values per face")
    out = C.c_double(0)
    _check(lib().mtk_map_deviation(nF, N, len(V), _ptr(F), _ptr(V), _ptr(c), _ptr(e), C.byref(out)),
           "mtk_map_deviation")
    return out.value


def local_injectivity(ctx: Context, cfn, N=4):
    """mtk_local_injectivity: (flipped faces, first flipped face (nF when none)) of the map
    given by cfn (nF x 3N: the N function values at each corner)."""
    c = np.ascontiguousarray(cfn, np.float64).reshape(-1)
    nF = c.size // (3 * N)
    nf, first = C.c_int32(0), C.c_int32(0)
    _check(lib().mtk_local_injectivity(ctx.handle, nF, N, _ptr(c), C.byref(nf), C.byref(first)),
           "mtk_local_injectivity")
    return nf.value, first.value


def spmv_bench(ctx: Context, nbr, theta, precision="mixed", reps=20):
    """mtk_field_spmv_bench: (ms per SpMV, algorithmic bytes per SpMV, ms of a device copy of the
    same bytes); "mixed" times FP32."""
    nbr = np.ascontiguousarray(nbr, np.int32).reshape(-1)
    theta = np.ascontiguousarray(theta, np.float64).reshape(-1)
    ms, by, cp = C.c_double(0), C.c_double(0), C.c_double(0)
    _check(lib().mtk_field_spmv_bench(ctx.handle, len(nbr) // 3, 4, _ptr(nbr), _ptr(theta),
                                      PREC_FP64 if precision == "fp64" else PREC_MIXED, reps, C.byref(ms), C.byref(by),
                                      C.byref(cp)),
           "mtk_field_spmv_bench")
    return ms.value, by.value, cp.value


def field_solve(ctx: Context, nbr, theta, area, rhs, n_rosy=4, opts=None):
    """mtk_field_solve: one solve L x = rhs with the field's connection Laplacian."""
    nbr = np.ascontiguousarray(nbr, np.int32).reshape(-1)
    theta = np.ascontiguousarray(theta, np.float64).reshape(-1)
    area = np.ascontiguousarray(area, np.float64)
    nF = len(area)
    r = np.empty(2 * nF)
    r[0::2], r[1::2] = np.real(rhs), np.imag(rhs)
    out = np.empty(2 * nF)
    st = Stats()
    o = opts or solve_opts()
    _check(lib().mtk_field_solve(ctx.handle, nF, n_rosy, _ptr(nbr), _ptr(theta), _ptr(area), _ptr(r), C.byref(o),
                                 _ptr(out), C.byref(st)), "mtk_field_solve")
    return out[0::2] + 1j * out[1::2], st.as_dict()


def size_field_gradient(ctx: Context, V, F, s, T=None, mu=0.0, ratio=0.02, seed=0, round_seams=False, n_iter=50,
                        opts=None):
    """mtk_pipeline_size_field_gradient: loss l(s) = sum_f |length X2F_f x(s) - exp(sbar_f) T_f|^2 +
    mu sum_edges (s_i - s_j)^2 of the naive integration x(s) with size-scaled targets, and dl/ds
    by the adjoint solve.  T (nF x 8) defaults to the integration target."""
    V = np.ascontiguousarray(V, np.float64)
    F = np.ascontiguousarray(F, np.int32)
    nV, nF = len(V), len(F)
    s = np.ascontiguousarray(s, np.float64)
    if s.shape != (nV,):
        raise ValueError("s must have one value per vertex")
    Tp = None
    if T is not None:
        T = np.ascontiguousarray(T, np.float64).reshape(-1)
        if T.size != 8 * nF:
            raise ValueError("T must have 8 values per face")
        Tp = _ptr(T)
    cap = 2 * (nV + 3 * nF) + 16                  # n (nV + nT) full variables, nT <= nE <= 3 nF
    fullx = np.zeros(cap)
    grad = np.zeros(nV)
    loss = C.c_double(0)
    n_full = C.c_int32(0)
    p = PipelineOpts(seed, n_iter, ratio, int(round_seams), 0, 0, 0, 0)
    o = opts or solve_opts()
    st = Stats()
    _check(lib().mtk_pipeline_size_field_gradient(ctx.handle, nV, nF, _ptr(V), _ptr(F), C.byref(p), C.byref(o), _ptr(s),
                                                  Tp, float(mu), C.byref(loss), _ptr(grad), _ptr(fullx), cap,
                                                  C.byref(n_full), C.byref(st)),
           "mtk_pipeline_size_field_gradient")
    return dict(loss=loss.value, grad=grad, fullx=fullx[:n_full.value].copy(), stats=st.as_dict())


def position_gradient(ctx: Context, V, F, s, mu=0.0, ratio=0.02, seed=0, round_seams=False, n_iter=50, opts=None):
    """mtk_pipeline_position_gradient: the size-field loss with the integration target, its
    gradient with respect to s and to the vertex positions (integer decisions held fixed)."""
    V = np.ascontiguousarray(V, np.float64)
    F = np.ascontiguousarray(F, np.int32)
    nV, nF = len(V), len(F)
    s = np.ascontiguousarray(s, np.float64)
    if s.shape != (nV,):
        raise ValueError("s must have one value per vertex")
    cap = 2 * (nV + 3 * nF) + 16                  # n (nV + nT) full variables, nT <= nE <= 3 nF
    fullx = np.zeros(cap)
    grad_s = np.zeros(nV)
    grad_V = np.zeros((nV, 3))
    loss = C.c_double(0)
    n_full = C.c_int32(0)
    p = PipelineOpts(seed, n_iter, ratio, int(round_seams), 0, 0, 0, 0)
    o = opts or solve_opts()
    st = Stats()
    _check(lib().mtk_pipeline_position_gradient(ctx.handle, nV, nF, _ptr(V), _ptr(F), C.byref(p), C.byref(o), _ptr(s),
                                                float(mu), C.byref(loss), _ptr(grad_s), _ptr(grad_V), _ptr(fullx), cap,
                                                C.byref(n_full), C.byref(st)),
           "mtk_pipeline_position_gradient")
    return dict(loss=loss.value, grad_s=grad_s, grad_V=grad_V, fullx=fullx[:n_full.value].copy(), stats=st.as_dict())


def face_geometry_backward(ctx: Context, V, F, g_area, g_farg1, g_farg2, g_gx, g_gy):
    """mtk_face_geometry_backward: vertex-position gradient from per-face derivatives."""
    V = np.ascontiguousarray(V, np.float64)
    F = np.ascontiguousarray(F, np.int32)
    arrs = [np.ascontiguousarray(a, np.float64).reshape(-1) for a in (g_area, g_farg1, g_farg2, g_gx, g_gy)]
    out = np.zeros((len(V), 3))
    _check(lib().mtk_face_geometry_backward(ctx.handle, len(V), len(F), _ptr(V), _ptr(F), *[_ptr(a) for a in arrs],
                                            _ptr(out)),
           "mtk_face_geometry_backward")
    return out


def mesh_field_inputs(ctx: Context, V, F):
    """mtk_mesh_field_inputs: (nbr[nF, 3], theta[nF, 3], area[nF]) computed on the device."""
    V = np.ascontiguousarray(V, np.float64)
    F = np.ascontiguousarray(F, np.int32)
    nF = len(F)
    nbr = np.zeros((nF, 3), np.int32)
    theta = np.zeros((nF, 3))
    area = np.zeros(nF)
    _check(lib().mtk_mesh_field_inputs(ctx.handle, len(V), nF, _ptr(V), _ptr(F), _ptr(nbr), _ptr(theta), _ptr(area)),
           "mtk_mesh_field_inputs")
    return nbr, theta, area


def field_smoothest_mesh(ctx: Context, V, F, x0, n_rosy=4, n_iter=50, opts=None):
    """mtk_field_smoothest_mesh: the smoothest field from the raw mesh (inputs on the device)."""
    V = np.ascontiguousarray(V, np.float64)
    F = np.ascontiguousarray(F, np.int32)
    nF = len(F)
    x = np.empty(2 * nF)
    x[0::2], x[1::2] = np.real(x0), np.imag(x0)
    out = np.empty(2 * nF)
    st = Stats()
    o = opts if opts is not None else solve_opts()
    _check(lib().mtk_field_smoothest_mesh(ctx.handle, len(V), nF, _ptr(V), _ptr(F), n_rosy, _ptr(x), n_iter, C.byref(o),
                                          _ptr(out), C.byref(st)), "mtk_field_smoothest_mesh")
    return out[0::2] + 1j * out[1::2], st.as_dict()


def curl_matching(ctx: Context, V, F, edge_vert, edge_face, vert_half, prev_half, angle_defect, compressed, N=4,
                  twin=None, half_edge=None, edge_half=None):
    """mtk_curl_matching: Curl matching[nE] and singular indices[nV] on the device, from the mesh
    arrays in the Hmesh numbering and the compressed field (complex[nF]).  twin / half_edge /
    edge_half: the halfedge arrays of a mesh with boundary (None for a closed mesh)."""
    V = np.ascontiguousarray(V, np.float64)
    F = np.ascontiguousarray(F, np.int32)
    ev = np.ascontiguousarray(edge_vert, np.int32)
    ef = np.ascontiguousarray(edge_face, np.int32)
    vh = np.ascontiguousarray(vert_half, np.int32)
    pv = np.ascontiguousarray(prev_half, np.int32)
    ad = np.ascontiguousarray(angle_defect, np.float64)
    c = np.ascontiguousarray(np.asarray(compressed, np.complex128).view(np.float64))
    nE = len(ev)
    matching = np.zeros(nE, np.int32)
    singular = np.zeros(len(V), np.int32)
    extra = [None, None, None]
    if twin is not None:
        extra = [np.ascontiguousarray(a, np.int32) for a in (twin, half_edge, edge_half)]
    _check(lib().mtk_curl_matching(ctx.handle, len(V), len(F), nE, N, _ptr(V), _ptr(F), _ptr(ev), _ptr(ef), _ptr(vh),
                                   _ptr(pv), *(_ptr(a) for a in extra), _ptr(ad), _ptr(c), _ptr(matching),
                                   _ptr(singular)),
           "mtk_curl_matching")
    return matching, singular


def seam_paths(ctx: Context, nV, nE, vptr, vv, ve, sources, in_cut, seam):
    """mtk_seam_paths: the singularity-path searches on the device.  Returns (in_cut, seam) after
    every path joined the cut (copies of the inputs updated)."""
    vptr = np.ascontiguousarray(vptr, np.int32)
    vv = np.ascontiguousarray(vv, np.int32)
    ve = np.ascontiguousarray(ve, np.int32)
    src = np.ascontiguousarray(sources, np.int32)
    cut = np.ascontiguousarray(in_cut, np.uint8).copy()
    sm = np.ascontiguousarray(seam, np.uint8).copy()
    _check(lib().mtk_seam_paths(ctx.handle, nV, nE, _ptr(vptr), _ptr(vv), _ptr(ve), len(src), _ptr(src), _ptr(cut),
                                _ptr(sm)), "mtk_seam_paths")
    return cut.astype(bool), sm.astype(bool)


def comb_turns(ctx: Context, nb, nm, N=4):
    """mtk_comb_turns: each face's combing turn (-1 where the search does not reach)."""
    nb = np.ascontiguousarray(nb, np.int32).reshape(-1)
    nm = np.ascontiguousarray(nm, np.int32).reshape(-1)
    nF = len(nb) // 3
    turns = np.zeros(nF, np.int32)
    _check(lib().mtk_comb_turns(ctx.handle, nF, N, _ptr(nb), _ptr(nm), _ptr(turns)), "mtk_comb_turns")
    return turns


class CsrMatrix:
    """A device-resident assembled sparse matrix (mtk_csr): symmetric / Hermitian positive
    definite, real or complex; built from a scipy.sparse matrix."""

    def __init__(self, ctx: Context, A):
        import scipy.sparse as sp
        A = sp.csr_matrix(A)
        A.sort_indices()
        self.n = A.shape[0]
        self.complex = np.iscomplexobj(A.data)
        ptr = np.ascontiguousarray(A.indptr, np.int32)
        col = np.ascontiguousarray(A.indices, np.int32)
        if self.complex:
            val = np.empty(2 * A.nnz)
            val[0::2], val[1::2] = A.data.real, A.data.imag
        else:
            val = np.ascontiguousarray(A.data, np.float64)
        h = C.c_void_p()
        _check(lib().mtk_csr_create(ctx.handle, self.n, _ptr(ptr), _ptr(col), _ptr(val), int(self.complex), C.byref(h)),
               "mtk_csr_create")
        self.handle, self.ctx = h, ctx

    def close(self):
        if getattr(self, "handle", None):
            lib().mtk_csr_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _pack(self, v):
        v = np.asarray(v)
        v2 = v.reshape(self.n, -1, order="F")
        if self.complex:
            out = np.empty((2 * self.n, v2.shape[1]), order="F")
            out[0::2], out[1::2] = v2.real, v2.imag
            return out, v2.shape[1]
        return np.asfortranarray(v2, np.float64), v2.shape[1]

    def _unpack(self, w, shape):
        if self.complex:
            w = w[0::2] + 1j * w[1::2]
        return w.reshape(shape, order="F")

    def solve(self, b, x0=None, opts=None):
        """mtk_csr_pcg: A X = B (b: n or n x k); returns (x, stats)."""
        B, k = self._pack(b)
        X, _ = self._pack(np.zeros_like(np.asarray(b)) if x0 is None else x0)
        st = Stats()
        o = opts or solve_opts()
        _check(lib().mtk_csr_pcg(self.ctx.handle, self.handle, k, _ptr(B), _ptr(X), C.byref(o), C.byref(st)),
               "mtk_csr_pcg")
        return self._unpack(X, np.asarray(b).shape), st.as_dict()


def csr_smallest_eig(ctx: Context, L: CsrMatrix, M: CsrMatrix, x0, n_iter=50, opts=None):
    """mtk_csr_smallest_eig: the reference's solveSmallestEig on assembled (L, M)."""
    x = np.empty(2 * L.n)
    x[0::2], x[1::2] = np.real(x0), np.imag(x0)
    out = np.empty(2 * L.n)
    st = Stats()
    o = opts or solve_opts()
    _check(lib().mtk_csr_smallest_eig(ctx.handle, L.handle, M.handle, _ptr(x), n_iter, C.byref(o), _ptr(out), C.byref(st)),
           "mtk_csr_smallest_eig")
    return out[0::2] + 1j * out[1::2], st.as_dict()


def topology_from_field(V, F, compressed, ratio=0.02, round_seams=False):
    """Host-only stages (no GPU): matching, singularities, seam, cut mesh, combing, setup and
    the host part of integ() for a given field eigenvector."""
    V = np.ascontiguousarray(V, np.float64)
    F = np.ascontiguousarray(F, np.int32)
    nV, nF = len(V), len(F)
    nE = 3 * nF          # bound on the edge count; the outputs are cut to counts["nE"]
    c = np.empty(2 * nF)
    c[0::2], c[1::2] = np.real(compressed), np.imag(compressed)
    singular = np.zeros(nV, np.int32)
    matching = np.zeros(nE, np.int32)
    seam = np.zeros(nE, np.uint8)
    cutF = np.zeros(3 * nF, np.int32)
    counts = np.zeros(8, np.int32)
    length = C.c_double(0)
    _check(lib().mtk_topology_from_field(nV, nF, _ptr(V), _ptr(F), _ptr(c), ratio, int(round_seams),
                                         _ptr(singular), _ptr(matching), _ptr(seam), _ptr(cutF), _ptr(counts),
                                         C.byref(length)), "mtk_topology_from_field")
    ne = int(counts[1])
    return dict(singular=singular, matching=matching[:ne].copy(), seam=seam[:ne].astype(bool), cutF=cutF.reshape(nF, 3),
                counts=dict(zip(["nV", "nE", "nCut", "nT", "nS", "nJ", "nZ", "nFull"], counts.tolist())),
                length=length.value)
