/*
 * metriko-gb300 C ABI: the drop-in boundary between the header-only C++ host code
 * (include/metriko/...) and the sm_103a CUDA kernels in libmetriko_cuda.so.
 *
 * Every function returns an int status (MTK_OK on success).  Pointers are plain host
 * pointers unless a parameter says otherwise; no C++ or torch types cross this boundary.
 * Each context owns one CUDA device and one stream; calls on one context are not re-entrant.
 *
 * Reference interfaces replaced (paths inside the metriko project):
 *   mtk_field_smoothest   <- FaceRosyField(const Hmesh&, int, FieldType::Smoothest)
 *                            (include/metriko/core/vectorfield/face_rosy_field.h:17-23) with
 *                            connectionLaplacian (:46-76), galerkinMassMatrix (:78-84) and
 *                            solveSmallestEig(SprsC&, SprsC&, int nIter = 50)
 *                            (include/metriko/core/solver/sparse_linear_solver.h:29-54)
 *   mtk_iterative_rounding <- iterative_rounding(fixedIdcs, fixedVals, singularIdcs,
 *                            integerIdcs, length, Cfull, G2, N, n, nF, seamless, roundSeams,
 *                            localInjectivity, verbose, intrinsicField, iter_cb, fullx)
 *                            (include/metriko/core/igm/iterative_rounding/iter_rounding.h:33-113)
 *                            including NaiveIntegration (iter_rounding_init.h:16-233),
 *                            SeamlessIntegration (iter_rounding_loop.h:10-125) and the
 *                            LMSolver/CholeskyWrapper linear-solver seam
 *                            (include/metriko/core/solver/levenberg_marquardt.h:140-231,
 *                            iter_rounding.h:14-31)
 *   mtk_topology_from_field <- the host stages of the same sequence for a given field
 *                            (face_rosy_field.h:100-360, parameterization.h:43-152,
 *                            parameterization_setup.ipp:3-170, parameterization_integ.ipp:3-70)
 *   mtk_pipeline_run      <- the example_igm.cpp:13-31 call sequence (Hmesh -> field ->
 *                            matching -> seam -> cut -> combing -> RosyParameterization
 *                            setup()/integ()) as one call with host buffers
 *   mtk_mesh_geometry     <- the vertex and edge geometry of the Hmesh constructor
 *                            (include/metriko/core/hmesh/hmesh.h:491-568), host only
 *   mtk_map_deviation     <- the closing check of RosyParameterization::integ()
 *                            (parameterization_integ.ipp:100-117), host only
 *   mtk_injective_barrier, mtk_local_injectivity <- InjectiveBarrier
 *                            (iterative_rounding/injective_barrier.h:10-110) and
 *                            locally_injectivity_check (parameterization_integ.ipp:46-63)
 * The direct caller of iterative_rounding passes the descriptor mtk_igm_desc that
 * RosyParameterization::build_system fills, not an assembled Cfull / G2.
 */
#ifndef METRIKO_CUDA_H
#define METRIKO_CUDA_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum mtk_status {
    MTK_OK = 0,
    MTK_ERR_BAD_INPUT = 1,      /* invalid sizes / indices / non-manifold mesh          */
    MTK_ERR_CUDA = 2,           /* a CUDA runtime call failed (see mtk_last_error)      */
    MTK_ERR_NOT_CONVERGED = 3,  /* an iterative solve hit its iteration cap             */
    MTK_ERR_BREAKDOWN = 4,      /* PCG breakdown: p^H A p <= 0 or a NaN                 */
    MTK_ERR_TIMEOUT = 5,        /* a bounded device-side wait gave up                   */
    MTK_ERR_NO_DEVICE = 6,      /* no CUDA device is visible                            */
    MTK_ERR_ROUNDING = 7        /* post-rounding integrality check failed               */
};

enum mtk_precision {
    MTK_PREC_FP64 = 0,          /* FP64 SpMV, dots and PCG throughout                   */
    MTK_PREC_MIXED = 1          /* FP32 PCG inside FP64 iterative refinement            */
};

typedef struct mtk_ctx mtk_ctx;

typedef struct {
    int32_t precision;          /* mtk_precision                                        */
    double tol;                 /* relative residual ||b - A x|| / ||b|| per solve       */
    int32_t max_iter;           /* PCG iteration cap per inner solve                     */
    int32_t max_refine;         /* outer FP64 refinement steps (MIXED)                   */
    double inner_tol;           /* relative tolerance of each inner FP32 solve (MIXED; default 3e-6) */
} mtk_solve_opts;

typedef struct {
    int64_t pcg_iters;          /* PCG iterations summed over all solves                 */
    int64_t solves;             /* linear solves                                         */
    int64_t refinements;        /* FP64 residual evaluations                             */
    int64_t spmv_calls;         /* operator applications                                 */
    int64_t kernel_launches;    /* kernels launched by the library                       */
    double max_rel_residual;    /* worst final relative residual of any solve            */
    double ms_field;            /* device time, field stage                              */
    double ms_integrate;        /* device time, naive + LM integration                   */
    double ms_rounding;         /* device time, greedy rounding loop                     */
    double ms_host;             /* host-side topology time (pipeline only)               */
    double ms_total;            /* wall time of the call                                 */
    int64_t resolves;           /* IGM re-solves (rounded variables that needed a solve) */
    int64_t lm_iterations;      /* LM iterations over all LM solves                      */
    double min_order_margin;    /* smallest gap between best and second-best rounding    */
    /* persistent PCG kernels: launches, device ms (CUDA events around each launch) and
       algorithmic bytes (per-iteration formula evaluated on the actual sizes / nnz)       */
    int64_t field_pcg_launches;
    double field_pcg_ms;
    double field_pcg_bytes;
    int64_t igm_pcg_launches;
    double igm_pcg_ms;
    double igm_pcg_bytes;
    /* greedy rounding: steps whose pick (distances <= 1e-6 count as 0; first position among
       the candidates within 1e-8 of the smallest distance) is not the strict '<' pick of the
       reference -- among fractional candidates (with the largest distance gap between the two
       picks), and among already-integral ones (no re-solve follows such a pick)              */
    int64_t strict_order_differs;
    double strict_order_gap;
    int64_t integral_order_differs;
    /* passes of the persistent PCG kernels: iterations + 1 per launch (the start pass)      */
    int64_t field_pcg_passes;
    int64_t igm_pcg_passes;
} mtk_stats;

const char* mtk_status_string(int status);
const char* mtk_last_error(void);
void mtk_default_opts(mtk_solve_opts* opts);

int mtk_ctx_create(int device, mtk_ctx** out);
int mtk_ctx_destroy(mtk_ctx* ctx);
/* Number of library kernels launched on this context so far (instrumentation). */
int64_t mtk_ctx_kernel_count(const mtk_ctx* ctx);
/*
 * Polls a waiting CTA makes at a grid barrier of the persistent solver kernels before it gives
 * up: the kernel then leaves its loops and the call returns MTK_ERR_TIMEOUT, with the context
 * still usable.  Default 2^24 (about a second).  No counterpart in the reference (which has no
 * device code); small values exist to exercise the timeout path (0 = give up at the first poll
 * that finds the barrier still closed).  polls < 0 -> MTK_ERR_BAD_INPUT.
 */
int mtk_ctx_set_wait_limit(mtk_ctx* ctx, int64_t polls);

/*
 * Smoothest N-RoSy field: assemble the connection Laplacian L (face graph, up to 3 neighbours
 * per face) and the lumped mass M = diag(area) on the device, then run n_iter steps of inverse
 * power iteration  x = L^-1 M u,  x /= sqrt|x^H M x|,  u = x.
 *   nbr[3*f+j]   face across the j-th halfedge of face f (halfedge F(f,j) -> F(f,j+1)), or -1
 *                when that halfedge lies on the boundary (no entry, face_rosy_field.h:64); any
 *                other value outside [0, nF), or f itself -> MTK_ERR_BAD_INPUT
 *   theta[3*f+j] heArgOnFace(h) - heArgOnFace(twin(h)) for that halfedge; the off-diagonal
 *                entry is  L(f, nbr) = -(-exp(i theta))^nRosy,  the diagonal #nbr + 1e-9
 *   area[f]      face area;  x0[2*f], x0[2*f+1]  start vector (re, im)
 *   out[2*f], out[2*f+1]  the compressed field (re, im), unit M-norm
 */
int mtk_field_smoothest(mtk_ctx* ctx, int32_t nF, int32_t nRosy, const int32_t* nbr,
                        const double* theta, const double* area, const double* x0,
                        int32_t n_iter, const mtk_solve_opts* opts, double* out,
                        mtk_stats* stats);

/*
 * Integer-grid-map rounding system, in the reference's reduced coordinates
 * xs = [y ; z]: y = free full variables (identity rows of UFull), z = kernel coordinates of
 * the constrained block (UFull rows = USmall).  Full variables are n per raw vertex followed
 * by n per seam transition (n = N/2 under sign symmetry).
 */
typedef struct {
    int32_t nF, nCut, N, n;
    const int32_t* cutF;        /* nF*3 cut-mesh vertex of each corner                     */
    const double* cutV;         /* nCut*3 cut-mesh vertex positions                        */
    /* W: cut vertex c, function k < n  ->  sum_e w_val[e] * X[w_idx[e]], rows r = n*c + k */
    const int32_t* w_ptr;       /* n*nCut + 1                                              */
    const int32_t* w_idx;       /* full-variable indices                                   */
    const double* w_val;
    int32_t nFull;              /* n * (nV + nT)                                           */
    const int32_t* full2y;      /* nFull: y index of a free variable, else -1              */
    int32_t nJ, nZ;             /* constrained variables / kernel dimension                */
    const int32_t* uniqueJ;     /* nJ full indices of the constrained block (ascending)   */
    const double* USmall;       /* nJ x nZ row-major kernel basis                          */
    const double* F2;           /* 2*N*nF target field, face frame (rawF2Vec)              */
    double length;              /* grid edge length (bbox diagonal * ratio / norm)         */
    int32_t nFixed;             /* anchor of the naive solve (fixedIdcs / fixedVals)      */
    const int32_t* fixedIdcs;
    const double* fixedVals;
    int32_t nSingular;          /* singularIdcs (rounded first unless roundSeams)          */
    const int32_t* singularIdcs;
    int32_t nInteger;           /* integerIdcs (transition variables)                      */
    const int32_t* integerIdcs;
    int32_t seamless;           /* RosyParameterization::seamless                          */
    int32_t roundSeams;         /* RosyParameterization::roundSeams                        */
} mtk_igm_desc;

/*
 * Naive (Poisson) integration, the seamless LM solve and the greedy rounding loop.
 *   fullx[nFull]      result (reference iter_rounding.h:111)
 *   fix_order/fix_vals (capacity nSingular + nInteger) the rounded full indices and their
 *                      integer values in fixing order; *n_fixed receives the count
 *   x_naive[nFull]    optional (may be NULL): the naive Poisson solution ni.x0
 * Returns MTK_ERR_ROUNDING when the post-rounding integrality check fails (fullx is still
 * written, as the reference does).
 */
int mtk_iterative_rounding(mtk_ctx* ctx, const mtk_igm_desc* desc, const mtk_solve_opts* opts,
                           double* fullx, int32_t* fix_order, int32_t* fix_vals,
                           int32_t* n_fixed, double* x_naive, mtk_stats* stats);

/*
 * Whole path of example_igm.cpp with host buffers: V (nV*3), F (nF*3), N = 4, Smoothest
 * field, Curl matching, seamless = 1, localInjectivity = 0 unless popts->local_injectivity
 * (then the reference's damped LM with the injective barrier on the host, each of its linear
 * solves by mtk_csr_pcg and each orientation check by mtk_local_injectivity; MTK_ERR_ROUNDING
 * where its rounding fails the integrality check).  Outputs (caller-allocated,
 * may be NULL unless noted):
 *   singular[nV], matching[nE] (combed), seam[nE] (0/1), compressed[2*nF]
 *   cfn[nF*3*N]       corner parameterisation (row f: corner j, function k at N*j + k)
 *   fullx / x_naive   capacity given by fullx_cap; *n_full receives the length
 *   fix_order / fix_vals capacity fix_cap; *n_fixed receives the count
 *   counts[8]         nV, nE, nCut, nT, nS, nJ, nZ, nFull
 */
typedef struct {
    int32_t seed;               /* start vector seed (splitmix64, see mtk_seeded_init)   */
    int32_t n_iter;             /* power iterations (reference: 50)                       */
    double ratio;               /* RosyParameterization ratio (grid scale)                */
    int32_t round_seams;        /* RosyParameterization::roundSeams                       */
    int32_t seamless;           /* RosyParameterization::seamless                         */
    int32_t stop_after;         /* 0 = full path, 1 = after field+matching, 2 = after setup */
    int32_t field_type;         /* 0 = FieldType::Smoothest, 1 = FieldType::CurvatureAligned */
    int32_t local_injectivity;  /* RosyParameterization::localInjectivity (damped LM with the
                                   injective barrier; its linear solves on the device)      */
} mtk_pipeline_opts;

int mtk_pipeline_run(mtk_ctx* ctx, int32_t nV, int32_t nF, const double* V, const int32_t* F,
                     const mtk_pipeline_opts* popts, const mtk_solve_opts* sopts,
                     int32_t* singular, int32_t* matching, uint8_t* seam, double* compressed,
                     double* cfn, double* fullx, double* x_naive, int32_t fullx_cap,
                     int32_t* n_full, int32_t* fix_order, int32_t* fix_vals, int32_t fix_cap,
                     int32_t* n_fixed, int32_t* counts, mtk_stats* stats);

/*
 * Host-only topology stages for a caller-supplied field (no device work): Hmesh, Curl
 * matching and singularities, seams, cut mesh, combing, RosyParameterization::setup() and the
 * host part of integ() (constraint reduction, UFull kernel block, target field, grid length).
 * Replaces the face_rosy_field.h:100-360 and parameterization*.{h,ipp} host code.
 *   compressed[2*nF]  field eigenvector (re, im) -- e.g. the output of mtk_field_smoothest
 *   singular[nV], matching[nE] (combed), seam[nE], cutF[nF*3]
 *   counts[8]         nV, nE, nCut, nT, nS, nJ, nZ, nFull;   *length: grid edge length
 */
int mtk_topology_from_field(int32_t nV, int32_t nF, const double* V, const int32_t* F,
                            const double* compressed, double ratio, int32_t round_seams,
                            int32_t* singular, int32_t* matching, uint8_t* seam, int32_t* cutF,
                            int32_t* counts, double* length);

/*
 * Allocation-free variant of mtk_field_smoothest (FP64 path) for callers that cannot call
 * cudaMalloc -- code inside a host framework that owns all device memory through its own
 * allocator, or code that must not allocate after start-up.  No counterpart in the reference
 * (which has no GPU code); it allocates nothing and needs no mtk_ctx.
 *   All pointers are DEVICE pointers owned by the caller: nbr[3*nF], theta[3*nF], area[nF],
 *   x0[2*nF] (re, im), out[2*nF].  stream: a cudaStream_t (NULL = default stream).
 *   nbr as for mtk_field_smoothest: -1 marks a boundary side (the row's diagonal is then its
 *   count of neighbours + 1e-9); any other entry outside [0, nF) -> MTK_ERR_BAD_INPUT, detected
 *   on the device, with no solve.  n_iter = 0 copies x0 to out.  max_iter caps every inner PCG solve
 *   (MTK_ERR_NOT_CONVERGED when reached).
 *   Working memory is a 64 MiB static device array inside the library (held by every GPU that
 *   loads the library until exit), which limits nF to 409600; larger nF -> MTK_ERR_BAD_INPUT.
 *   The first call on a device looks the array up (cudaGetSymbolAddress) and keeps its address
 *   for the life of the process; make no call on a device after cudaDeviceReset().  All calls
 *   share the array: calls that overlap on the GPU race.  *iterations (may be NULL) receives the
 *   total PCG iterations.  The call reads its status back and waits for `stream` before it
 *   returns, so no call can be captured into a CUDA graph (call it outside any capture).
 */
int mtk_field_smoothest_noalloc(int32_t nF, int32_t nRosy, const int32_t* nbr, const double* theta,
                                const double* area, const double* x0, int32_t n_iter, double tol,
                                int32_t max_iter, double* out, void* stream, int32_t* iterations);

/*
 * One solve L x = rhs with the connection Laplacian of mtk_field_smoothest (same inputs, same
 * assembly, preconditioner and precision options).  Replaces solveSquare(lhs, rhs) of
 * face_rosy_field.h:25-33 / sparse_linear_solver.h:16-27 for FieldType::CurvatureAligned
 * (lambda = 0, so lhs = L).  rhs[2*nF] and out[2*nF] are (re, im) per face.
 */
int mtk_field_solve(mtk_ctx* ctx, int32_t nF, int32_t nRosy, const int32_t* nbr, const double* theta,
                    const double* area, const double* rhs, const mtk_solve_opts* opts, double* out,
                    mtk_stats* stats);

/*
 * Gradient of a parameterization-quality loss with respect to a per-vertex log-size field
 * (adjoint of the naive integration).  No counterpart in the reference, which has no
 * differentiation; it serves size-field optimisation on top of the integration of
 * iter_rounding_init.h:171-212.  The naive integration is run with the target of face f scaled
 * by exp(sbar_f), sbar_f the mean of s over the face's corners:
 *   length X2F^T X2F x = X2F^T (exp(sbar) F2),  anchored as in mtk_iterative_rounding,
 * and the loss
 *   l(s) = sum_f |length X2F_f x(s) - exp(sbar_f) T_f|^2 + mu sum_edges (s_i - s_j)^2
 * is differentiated by one adjoint solve with the same (symmetric) operator, K lambda = dl/dx,
 * plus the assembly backward of the right-hand side; the solver iterates are not stored.
 *   F[3*nF]      raw mesh faces (corner vertex ids < nV; the rows of the cut faces)
 *   s[nV]        log-size per raw vertex
 *   T[8*nF]      loss target per face in the F2 layout, or NULL for the integration target F2
 *   mu >= 0      edge smoothness weight: the term sums (s_i - s_j)^2 / 2 over face sides, i.e.
 *                every interior edge once and a boundary edge at half weight
 *   loss, grad_s[nV], fullx[nFull] (the integration result x(s) in full variables)
 * desc->seamless and the rounding fields are not used.
 */
int mtk_size_field_gradient(mtk_ctx* ctx, const mtk_igm_desc* desc, const mtk_solve_opts* opts, int32_t nV,
                            const int32_t* F, const double* s, const double* T, double mu, double* loss,
                            double* grad_s, double* fullx, mtk_stats* stats);

/*
 * mtk_size_field_gradient on the whole example_igm.cpp path with host buffers: Hmesh ->
 * field -> topology -> RosyParameterization::setup() -> the size-field gradient (instead of
 * integ()).  No counterpart in the reference.  fullx capacity fullx_cap, *n_full its length.
 */
int mtk_pipeline_size_field_gradient(mtk_ctx* ctx, int32_t nV, int32_t nF, const double* V, const int32_t* F,
                                     const mtk_pipeline_opts* popts, const mtk_solve_opts* sopts,
                                     const double* s, const double* T, double mu, double* loss,
                                     double* grad_s, double* fullx, int32_t fullx_cap, int32_t* n_full,
                                     mtk_stats* stats);

/*
 * Gradient of the size-field loss of mtk_size_field_gradient with respect to the VERTEX
 * POSITIONS as well (differentiation; no counterpart in the reference).  The loss uses the
 * integration target (T = F2, the combed field in each face frame); every integer decision
 * (matching, seams, cut, combing, anchors) is held at its value for V.  Because x minimises the
 * loss's first term under the constraints, dl/dV is the partial derivative at fixed x; V enters
 * through the per-face gradient operator G2, the grid length (bounding-box diagonal), and the
 * field angle phi_f = arg(c_f) / 4 of the target, where c is the 50-step inverse power iteration
 * of (L(V), M(V)).  That dependence is carried by mtk_field_power_adjoint (one Hermitian solve
 * per power step, in reverse) and mtk_face_geometry_backward (per-face derivatives of the area,
 * the halfedge angles and G2).  Whole path with host buffers, as mtk_pipeline_size_field_gradient:
 *   s[nV], mu >= 0; loss, grad_s[nV], grad_V[3 nV]; fullx (capacity fullx_cap, *n_full).
 */
int mtk_pipeline_position_gradient(mtk_ctx* ctx, int32_t nV, int32_t nF, const double* V, const int32_t* F,
                                   const mtk_pipeline_opts* popts, const mtk_solve_opts* sopts, const double* s,
                                   double mu, double* loss, double* grad_s, double* grad_V, double* fullx,
                                   int32_t fullx_cap, int32_t* n_full, mtk_stats* stats);

/*
 * mtk_size_field_gradient with the integration target, also returning the loss's partial
 * derivatives at fixed x (no counterpart in the reference): per face the derivative with
 * respect to the G2 entries of its corners (dgx[3 nF], dgy[3 nF], corner a of face f at 3 f + a,
 * the entries (g . bX, g . bY) of the corner's gradient), to the field angle phi_f (dphi[nF]),
 * and to the grid length (*dlength).
 */
int mtk_size_field_position_partials(mtk_ctx* ctx, const mtk_igm_desc* desc, const mtk_solve_opts* opts, int32_t nV,
                                     const int32_t* F, const double* s, double mu, double* loss, double* grad_s,
                                     double* fullx, double* dgx, double* dgy, double* dphi, double* dlength,
                                     mtk_stats* stats);

/*
 * Reverse pass of the smoothest field's inverse power iteration (no counterpart in the
 * reference).  Runs mtk_field_smoothest (same inputs; out[2 nF] = the field c) keeping the n_iter
 * iterates, then, for the loss derivative dphi[nF] with respect to the field angle
 * phi_f = arg(c_f) / nRosy, one solve with L per step in reverse order, giving the derivatives
 * with respect to theta (g_theta[3 nF], the transport angle of halfedge j of face f) and to the
 * face areas (g_area[nF]).  The solves use the same multigrid, precision and tolerance.
 */
int mtk_field_power_adjoint(mtk_ctx* ctx, int32_t nF, int32_t nRosy, const int32_t* nbr, const double* theta,
                            const double* area, const double* x0, int32_t n_iter, const mtk_solve_opts* opts,
                            const double* dphi, double* out, double* g_theta, double* g_area, mtk_stats* stats);

/*
 * Assembly backward of the per-face geometry (no counterpart in the reference): from the loss's
 * derivatives with respect to each face's area (g_area[nF]), the halfedge angles heArgOnFace of
 * its second and third halfedges (g_farg1, g_farg2 [nF]; the first is 0 by construction) and its
 * G2 entries (g_gx, g_gy [3 nF]), the gradient with respect to the vertex positions
 * grad_V[3 nV] (hmesh.h:461-489, parameterization_integ.ipp:11-24; forward-mode dual numbers per
 * face on the device, vertices summing their faces in ascending order).
 */
int mtk_face_geometry_backward(mtk_ctx* ctx, int32_t nV, int32_t nF, const double* V, const int32_t* F,
                               const double* g_area, const double* g_farg1, const double* g_farg2, const double* g_gx,
                               const double* g_gy, double* grad_V);

/*
 * The inputs of mtk_field_smoothest computed on the device from the raw mesh (V[3 nV], F[3 nF])
 * without the halfedge mesh: nbr[3 nF] the face across side j of face f (the side from F(f, j)
 * to F(f, j+1); -1 on a boundary side, with theta 0), theta[3 nF] = heArgOnFace(h) -
 * heArgOnFace(twin h) and area[nF] (include/metriko/core/hmesh/hmesh.h:313-489 of the reference:
 * the constructor's pairing, face frames and halfedge angles).  The same values as
 * mtk_field_inputs (the halfedge mesh on the host), theta up to the last-bit rounding of acos.
 * A non-manifold edge, faces of opposite orientation or a side with equal end points ->
 * MTK_ERR_BAD_INPUT.
 */
int mtk_mesh_field_inputs(mtk_ctx* ctx, int32_t nV, int32_t nF, const double* V, const int32_t* F, int32_t* nbr,
                          double* theta, double* area);
/* mtk_mesh_field_inputs followed by mtk_field_smoothest (same remaining arguments and outputs). */
int mtk_field_smoothest_mesh(mtk_ctx* ctx, int32_t nV, int32_t nF, const double* V, const int32_t* F, int32_t nRosy,
                             const double* x0, int32_t n_iter, const mtk_solve_opts* opts, double* out,
                             mtk_stats* stats);

/*
 * Curl matching and singular indices on the device: computeConnection, cMatching and
 * computeSingular of FaceRosyField::computeMatching(MatchingType::Curl)
 * (include/metriko/core/vectorfield/face_rosy_field.h:100-135, :169-202), one thread per edge and
 * one per vertex.  Mesh arrays in the Hmesh numbering: V[3 nV], F[3 nF], edge_vert[2 nE] (edge e
 * runs from edge_vert[2e] to edge_vert[2e+1] inside face edge_face[2e]; edge_face[2e+1] is the
 * other face, -1 on a boundary edge's faceless side), vert_half[nV], prev_half[2 nE],
 * angle_defect[nV]; compressed[2 nF] the field (re, im); N <= 8.  twin_half[2 nE],
 * half_edge[2 nE], edge_half[nE] (Hmesh twin, edge, edge2half): required for a mesh with
 * boundary, NULL (all three) for a closed mesh, whose halfedges 2e / 2e+1 give them.
 * Out: matching[nE] (-1 on boundary edges), singular[nV] (1 on boundary vertices, as the
 * reference leaves them).  The integer outputs equal the host loops' (the arithmetic is the same,
 * up to the last bit of the device's cos / sin / atan2 / sqrt).
 */
int mtk_curl_matching(mtk_ctx* ctx, int32_t nV, int32_t nF, int32_t nE, int32_t N, const double* V, const int32_t* F,
                      const int32_t* edge_vert, const int32_t* edge_face, const int32_t* vert_half,
                      const int32_t* prev_half, const int32_t* twin_half, const int32_t* half_edge,
                      const int32_t* edge_half, const double* angle_defect, const double* compressed,
                      int32_t* matching, int32_t* singular);

/*
 * The singularity-path searches of cut_mesh_with_singularities on the device
 * (include/metriko/core/vectorfield/face_rosy_field.h:287-326 of the reference, libigl's
 * unit-weight dijkstra): for each source in order, a breadth-first search until a level holds a
 * vertex of the cut; the path from the smallest-id such vertex back along the predecessors (each
 * vertex's smallest-id neighbour in the previous level) joins the cut.  The same paths as the
 * host search (compute_seam), found in one cooperative launch with one grid barrier per level.
 *   vptr[nV+1], vv[vptr[nV]]   each vertex's neighbours, ve[vptr[nV]] the edge of each entry
 *   src[n_src]                 the sources (the singular vertices, in vertex order)
 *   in_cut[nV] (in/out)        1 for vertices of the cut (the spanning cut's, then the paths')
 *   seam[nE] (in/out)          edge flags: set for every edge of a path (entries already set stay)
 */
int mtk_seam_paths(mtk_ctx* ctx, int32_t nV, int32_t nE, const int32_t* vptr, const int32_t* vv, const int32_t* ve,
                   int32_t n_src, const int32_t* src, uint8_t* in_cut, uint8_t* seam);

/*
 * The combing search of compute_combbed_field on the device
 * (include/metriko/core/vectorfield/face_rosy_field.h:217-242 of the reference): from face 0
 * (turn 0), across every face side that is neither a seam nor a boundary, the neighbour's turn is
 * (the side's signed matching + the face's turn) mod N.  Level by level, one grid barrier per
 * level; the turns do not depend on the path inside the cut disk (every singular vertex lies on
 * the seam), so they equal the reference's queue order's.
 *   nb[3 nF]     the face across side j of face f, -1 across a seam or a boundary edge
 *   nm[3 nF]     the side's signed matching ((+1 or -1) * matching[e], face_rosy_field.h:237-238)
 *   turns[nF]    out: each face's turn, -1 for a face the search does not reach
 */
int mtk_comb_turns(mtk_ctx* ctx, int32_t nF, int32_t N, const int32_t* nb, const int32_t* nm, int32_t* turns);

/*
 * Assembled sparse systems (the general linear-solver seam).  Replaces, for symmetric / Hermitian
 * positive-definite matrices, the direct solvers behind solveSquare(SprsC&, VecXc&) and
 * solveSmallestEig(SprsC&, SprsC&, int) (include/metriko/core/solver/sparse_linear_solver.h:16-54)
 * and the LMSolver's linear-solver template parameter CholeskyWrapper::factorize / solve
 * (include/metriko/core/igm/iterative_rounding/iter_rounding.h:14-31).
 *   mtk_csr_create   n x n CSR (ptr[n+1] with ptr[0] = 0, col[nnz], val[nnz] or, when
 *                    complex_values, val[2 nnz] as (re, im)); copied to the device once (FP64 and
 *                    FP32) with its Jacobi inverse.  A diagonal entry <= 0 -> MTK_ERR_BAD_INPUT.
 *   mtk_csr_pcg      A X = B for nrhs columns (column-major: column c at c * n (real) or
 *                    c * 2 n (complex, (re, im) pairs)); x in: start, out: solution.  Jacobi PCG,
 *                    up to four columns per launch (the matrix read once per iteration for all),
 *                    FP64 or FP32 inside FP64 refinement (opts->precision), each column to the
 *                    relative residual opts->tol.
 *   mtk_csr_smallest_eig  n_iter steps of x = L^-1 M u, x /= sqrt|x^H M x|, u = x from x0 (complex
 *                    (re, im) vectors; L and M complex Hermitian, e.g. M diagonal), the reference's
 *                    solveSmallestEig with iterative solves; out[2 n].
 */
typedef struct mtk_csr mtk_csr;
int mtk_csr_create(mtk_ctx* ctx, int32_t n, const int32_t* ptr, const int32_t* col, const double* val,
                   int32_t complex_values, mtk_csr** out);
int mtk_csr_destroy(mtk_csr* A);
int mtk_csr_pcg(mtk_ctx* ctx, const mtk_csr* A, int32_t nrhs, const double* b, double* x, const mtk_solve_opts* opts,
                mtk_stats* stats);
int mtk_csr_smallest_eig(mtk_ctx* ctx, const mtk_csr* L, const mtk_csr* M, const double* x0, int32_t n_iter,
                         const mtk_solve_opts* opts, double* out, mtk_stats* stats);

/*
 * Barrier of the local-injectivity option: InjectiveBarrier(N, nF, intrinsic_field) followed by
 * update(field, update_j, fBarrier, gBarrier) of core/igm/iterative_rounding/injective_barrier.h:
 * 18-106.  Layout of intrinsic_field and field: 2*N values per face (vector j of face i at
 * 2*N*i + 2*j).  Per row k = N*i + j (vectors j and (j+1) mod N of face i):
 *   f_barrier[k]  1/bar(r) - 1 with r the volume ratio of the two vectors (infinite for r <= 0,
 *                 0 for r >= 1/2)
 *   bar_der[k]    the diagonal of gBarrier (d f_barrier / d r), when update_j
 *   s_rows[4*k]   the row of dr/d(v0.x, v0.y, v1.x, v1.y) (gen_image_filed), when update_j
 * bar_der and s_rows may be NULL when update_j == 0.
 */
int mtk_injective_barrier(mtk_ctx* ctx, int32_t nF, int32_t N, const double* intrinsic_field, const double* field,
                          int32_t update_j, double* f_barrier, double* bar_der, double* s_rows);

/*
 * locally_injectivity_check of core/igm/parameterization_integ.ipp:46-63: the orientation of
 * every cut face in the parameterization.  cfn[nF*3*N]: the N function values at the three
 * corners of each cut face (corner j of face f at 3*N*f + N*j; corners in the order of the
 * face's halfedge, its next and its prev); functions 0 and 1 are the (u, v) of the map.
 * *n_flipped = faces with cross(b - a, c - a) < 0 (the map is locally injective when 0),
 * *first_flipped (may be NULL) = the lowest such face, nF when none.
 */
int mtk_local_injectivity(mtk_ctx* ctx, int32_t nF, int32_t N, const double* cfn, int32_t* n_flipped,
                          int32_t* first_flipped);

/*
 * The inputs of mtk_field_smoothest (host only): nbr[3*nF] the face across each face halfedge
 * (-1 on the boundary, theta 0 there), theta[3*nF] = farg(h) - farg(twin h)
 * (face_rosy_field.h:46-76), and area[nF] (may be NULL).
 */
int mtk_field_inputs(int32_t nV, int32_t nF, const double* V, const int32_t* F, int32_t* nbr, double* theta,
                     double* area);

/*
 * Host only (no GPU): the vertex and edge geometry of Hmesh (hmesh.h:444-568 of the reference:
 * the members vertNormal, vertBasisX, vertBasisY, baryDualArea, circDualArea, halfCotan,
 * edgeCotan, dihedralArg, heArgOnVert, angleDefect), in the reference's halfedge / edge
 * numbering (interior halfedges first, then the boundary loops; nH = 2 nE, nE from
 * mtk_topology_from_field's counts or 3 nF / 2 for a closed mesh).  Every output may be NULL:
 * vert_normal, vert_basis_x, vert_basis_y [3 nV]; bary_area, circ_area, angle_defect [nV];
 * half_cotan, dihedral, he_arg_on_vert [nH]; edge_cotan [nE].
 */
int mtk_mesh_geometry(int32_t nV, int32_t nF, const double* V, const int32_t* F, double* vert_normal,
                      double* vert_basis_x, double* vert_basis_y, double* bary_area, double* circ_area,
                      double* half_cotan, double* edge_cotan, double* dihedral, double* he_arg_on_vert,
                      double* angle_defect);

/*
 * Host only (no GPU): the check at the end of RosyParameterization::integ()
 * (parameterization_integ.ipp:100-117, with G3 of :11-27) -- the mean over faces and functions
 * of |normalized(ext_k) - normalized(grad_k)|, grad_k the 3D gradient on the face of function k
 * of the map.  cutV[3*nCut], cutF[3*nF] (cut mesh), cfn[nF*3N] (function k at corner j in
 * column N*j + k, as mtk_pipeline_run returns it), ext[nF*3N] (the combed extrinsic field,
 * vector k in columns 3k..3k+2).  RosyParameterization::integ() stores the same value in its
 * member `deviation`.
 */
int mtk_map_deviation(int32_t nF, int32_t N, int32_t nCut, const int32_t* cutF, const double* cutV,
                      const double* cfn, const double* ext, double* deviation);

/*
 * SpMV roofline measurement (no counterpart in the reference): assembles the field operator
 * of mtk_field_smoothest and times `reps` stand-alone SpMVs y = L x (FP32 or FP64), each after
 * an L2 flush and with its own CUDA events.  *bytes_per_spmv: algorithmic bytes per SpMV
 * (per row 3 x (value + column) + diagonal + x_i + y_i).  *ms_copy_same_bytes (may be NULL): a
 * device-to-device copy moving the same bytes under the same flush and timing, the bandwidth a
 * kernel of that size can reach.
 */
int mtk_field_spmv_bench(mtk_ctx* ctx, int32_t nF, int32_t nRosy, const int32_t* nbr, const double* theta,
                         int32_t precision, int32_t reps, double* ms_per_spmv, double* bytes_per_spmv,
                         double* ms_copy_same_bytes);

/* The deterministic start vector used by the pipeline: re/im of face f from splitmix64. */
void mtk_seeded_init(int32_t n, int32_t seed, double* out);

#ifdef __cplusplus
}
#endif
#endif
