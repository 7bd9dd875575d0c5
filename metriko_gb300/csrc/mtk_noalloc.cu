// Allocation-free smoothest-field solve (mtk_field_smoothest_noalloc).
//
// Some callers cannot call cudaMalloc at all: code running inside a host framework that owns
// every device allocation through its own pool, or code that must not allocate once the
// process is set up (for example after a memory budget has been fixed).  They already hold
// device buffers for their inputs and outputs, so this entry point takes device pointers and
// keeps all of its working memory in one file-scope device array instead of allocating.
//
// The array (kScratchBytes = 64 MiB) is part of the library image: every GPU that loads the
// library holds it until the process exits.  It bounds the problem size to kMaxFaces faces.
// The first call on a device looks the array's device address up with cudaGetSymbolAddress
// (host code cannot use the symbol itself: in host code it names a host-side stand-in).  No
// call can be captured into a CUDA graph: each one synchronizes its stream.  The address is kept for the life of
// the process; a cudaDeviceReset() unloads the module, and the entry point must not be called
// on that device after one.  Every call shares the array, which keeps the last call's
// contents: the barrier words, the error flag and the status word are cleared at the start of
// each call, and calls that overlap on the GPU (two streams, two threads) race.  Each call
// reads its status back and waits for its stream before it returns.
//
// A neighbour of -1 marks a boundary side (no entry in L).  As in the regular entry point every
// row keeps the diagonal 3 + 1e-9 and a boundary side acts as the entry -1 on the row's own
// column, so a row applies its count of neighbours + 1e-9 to its own value (the reference's
// diagonal).  Any other neighbour index outside [0, nF), or a face's own index, is found during
// assembly, the solve is skipped and the call returns MTK_ERR_BAD_INPUT.
//
// Algorithm: the same inverse power iteration as mtk_field_smoothest with the FP64 path
// (assembly of the connection Laplacian, then n_iter steps of x = L^-1 M u solved by PCG to
// the relative residual tol from the Galerkin start u (u^H M u)/(u^H L u), x /= sqrt|x^H M x|),
// run as one persistent cooperative kernel so no host round trip is needed inside the loop.
#include <mutex>

#include "mtk_common.cuh"

namespace {

using namespace mtk;

constexpr size_t kScratchBytes = size_t(64) << 20;    // 64 MiB
constexpr size_t kHeaderBytes = size_t(64) << 10;     // barrier, status, scalars, partials
constexpr size_t kBytesPerFace = 160;                 // 3 double2 values + 7 double2 vectors
constexpr int kMaxFaces = 409600;
static_assert(kHeaderBytes + kBytesPerFace * (size_t)kMaxFaces <= kScratchBytes, "scratch too small");
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// header layout (bytes): [0,16) barrier count/gen, [16,20) error flag, [20,24) bad-neighbour
// flag, [32,48) status + iterations, [256, 512) scalars, [4096, 65536) reduction partials
// (<= 7 slots per CTA)
struct Layout {
    unsigned int* bar;
    int* err;
    int* bad_nbr;
    int* status;
    double* scal;
    double* partials;
    int* nbr;          // not stored: callers' array is used directly
    double2* val;      // 3 n
    double2 *b, *x, *u, *r, *z, *p, *q;
};

__host__ __device__ inline Layout layout_of(unsigned char* base, int n) {
    Layout L{};
    L.bar = reinterpret_cast<unsigned int*>(base);
    L.err = reinterpret_cast<int*>(base + 16);
    L.bad_nbr = reinterpret_cast<int*>(base + 20);
    L.status = reinterpret_cast<int*>(base + 32);
    L.scal = reinterpret_cast<double*>(base + 256);
    L.partials = reinterpret_cast<double*>(base + 4096);
    double2* v = reinterpret_cast<double2*>(base + kHeaderBytes);
    L.val = v;
    v += 3 * (size_t)n;
    L.b = v; v += n;
    L.x = v; v += n;
    L.u = v; v += n;
    L.r = v; v += n;
    L.z = v; v += n;
    L.p = v; v += n;
    L.q = v;
    return L;
}

// val and x are written earlier in the same kernel, so they are read through L2 (__ldcg), not
// the read-only path.  nbr has been range-checked by the assembly before any call; a boundary
// side (-1) reads the row's own value with the entry -1 stored for it.
__device__ __forceinline__ double2 row_apply(int i, int n, const int* __restrict__ nbr, const double2* val,
                                             double diag, const double2* x) {
    double2 xi = __ldcg(x + i);
    double re = diag * xi.x, im = diag * xi.y;
#pragma unroll
    for (int j = 0; j < 3; j++) {
        int c = nbr[3 * i + j];
        if (c < 0) c = i;
        double2 a = __ldcg(val + j * n + i);
        double2 xc = __ldcg(x + c);
        re += a.x * xc.x - a.y * xc.y;
        im += a.x * xc.y + a.y * xc.x;
    }
    return make_double2(re, im);
}

__global__ void __launch_bounds__(kBlock) noalloc_power(unsigned char* base, int n, int N, const int* __restrict__ nbr,
                                                       const double* __restrict__ theta, const double* __restrict__ area,
                                                       const double* __restrict__ x0, int n_iter, double tol, int maxit,
                                                       double* out) {
    Layout L = layout_of(base, n);
    GridBarrier bar{L.bar, L.bar + 1, L.err};
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    const double diag = 3.0 + 1e-9;   // three sides per face + the 1e-9 shift (boundary sides: entry -1)
    const int G = gridDim.x;
    int status = 0;
    long long total_it = 0;
    // assembly (face_rosy_field.h:52-75), the neighbour range check and the start vector
    for (int f = t0; f < n; f += stride) {
        for (int j = 0; j < 3; j++) {
            const int g = nbr[3 * f + j];
            if (g < -1 || g >= n || g == f) atomicExch(L.bad_nbr, 1);
            if (g < 0) {
                L.val[j * n + f] = make_double2(-1.0, 0.0);
                continue;
            }
            double s, c;
            sincos((double)N * (theta[3 * f + j] + 3.14159265358979323846), &s, &c);
            L.val[j * n + f] = make_double2(-c, -s);
        }
        L.u[f] = make_double2(x0[2 * f], x0[2 * f + 1]);
    }
    if (!grid_sync(bar)) { status = MTK_ERR_TIMEOUT; goto done; }
    if (ld_volatile(L.bad_nbr) != 0) { status = MTK_ERR_BAD_INPUT; goto done; }   // same value in every CTA
    for (int k = 0; k < n_iter; k++) {
        // b = M u; Galerkin factor g = (u^H M u) / (u^H L u); |b|^2
        double red3[3] = {0, 0, 0};
        for (int i = t0; i < n; i += stride) {
            double2 ui = L.u[i];
            double2 li = row_apply(i, n, nbr, L.val, diag, L.u);
            double a = area[i];
            double2 bi = make_double2(a * ui.x, a * ui.y);
            L.b[i] = bi;
            red3[0] += ui.x * li.x + ui.y * li.y;
            red3[1] += a * (ui.x * ui.x + ui.y * ui.y);
            red3[2] += bi.x * bi.x + bi.y * bi.y;
        }
        publish_partials<double, 3>(red3, L.partials);
        if (!grid_sync(bar)) { status = MTK_ERR_TIMEOUT; break; }
        gather_partials<double, 3>(L.partials, red3);
        const double g = red3[0] > 0 ? red3[1] / red3[0] : 0.0;
        const double tol2 = tol * tol * red3[2];
        for (int i = t0; i < n; i += stride) {
            double2 ui = L.u[i];
            L.x[i] = make_double2(g * ui.x, g * ui.y);
        }
        if (!grid_sync(bar)) { status = MTK_ERR_TIMEOUT; break; }
        // PCG (Jacobi) on L x = b
        double red2[2] = {0, 0};
        for (int i = t0; i < n; i += stride) {
            double2 ax = row_apply(i, n, nbr, L.val, diag, L.x);
            double2 bi = L.b[i];
            double2 ri = make_double2(bi.x - ax.x, bi.y - ax.y);
            double2 zi = make_double2(ri.x / diag, ri.y / diag);
            L.r[i] = ri;
            L.z[i] = zi;
            L.p[i] = zi;
            red2[0] += ri.x * zi.x + ri.y * zi.y;
            red2[1] += ri.x * ri.x + ri.y * ri.y;
        }
        publish_partials<double, 2>(red2, L.partials + 3 * G);
        if (!grid_sync(bar)) { status = MTK_ERR_TIMEOUT; break; }
        gather_partials<double, 2>(L.partials + 3 * G, red2);
        double rz = red2[0], rr = red2[1];
        int it = 0;
        bool failed = false;
        while (rr > tol2) {
            if (it >= maxit) { status = MTK_ERR_NOT_CONVERGED; break; }
            double red1[1] = {0};
            for (int i = t0; i < n; i += stride) {
                double2 qi = row_apply(i, n, nbr, L.val, diag, L.p);
                L.q[i] = qi;
                double2 pi = L.p[i];
                red1[0] += pi.x * qi.x + pi.y * qi.y;
            }
            publish_partials<double, 1>(red1, L.partials + 5 * G);
            if (!grid_sync(bar)) { status = MTK_ERR_TIMEOUT; failed = true; break; }
            gather_partials<double, 1>(L.partials + 5 * G, red1);
            if (!(red1[0] > 0)) { status = MTK_ERR_BREAKDOWN; failed = true; break; }
            const double alpha = rz / red1[0];
            red2[0] = red2[1] = 0;
            for (int i = t0; i < n; i += stride) {
                double2 pi = L.p[i], qi = L.q[i], xi = L.x[i], ri = L.r[i];
                xi.x += alpha * pi.x; xi.y += alpha * pi.y;
                ri.x -= alpha * qi.x; ri.y -= alpha * qi.y;
                double2 zi = make_double2(ri.x / diag, ri.y / diag);
                L.x[i] = xi; L.r[i] = ri; L.z[i] = zi;
                red2[0] += ri.x * zi.x + ri.y * zi.y;
                red2[1] += ri.x * ri.x + ri.y * ri.y;
            }
            publish_partials<double, 2>(red2, L.partials + 3 * G);
            if (!grid_sync(bar)) { status = MTK_ERR_TIMEOUT; failed = true; break; }
            gather_partials<double, 2>(L.partials + 3 * G, red2);
            const double beta = red2[0] / rz;
            rz = red2[0];
            rr = red2[1];
            for (int i = t0; i < n; i += stride) {
                double2 zi = L.z[i], pi = L.p[i];
                L.p[i] = make_double2(zi.x + beta * pi.x, zi.y + beta * pi.y);
            }
            it++;
            if (!grid_sync(bar)) { status = MTK_ERR_TIMEOUT; failed = true; break; }
        }
        total_it += it;
        if (failed || status == MTK_ERR_NOT_CONVERGED) break;
        // x /= sqrt|x^H M x|;  u = x
        double red1[1] = {0};
        for (int i = t0; i < n; i += stride) {
            double2 xi = L.x[i];
            red1[0] += area[i] * (xi.x * xi.x + xi.y * xi.y);
        }
        publish_partials<double, 1>(red1, L.partials + 6 * G);
        if (!grid_sync(bar)) { status = MTK_ERR_TIMEOUT; break; }
        gather_partials<double, 1>(L.partials + 6 * G, red1);
        const double s = sqrt(fabs(red1[0]));
        for (int i = t0; i < n; i += stride) {
            double2 xi = L.x[i];
            L.u[i] = make_double2(xi.x / s, xi.y / s);
        }
        if (!grid_sync(bar)) { status = MTK_ERR_TIMEOUT; break; }
    }
    if (status == 0)
        for (int i = t0; i < n; i += stride) {
            double2 ui = L.u[i];
            out[2 * i] = ui.x;
            out[2 * i + 1] = ui.y;
        }
done:
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        L.status[0] = status;
        L.status[1] = (int)(total_it > 0x7fffffff ? 0x7fffffff : total_it);
    }
}

std::mutex g_setup_mutex;
unsigned char* g_base[kMaxDevices] = {};

// Once per device, with that device current: the device address of the scratch array.
int scratch_base(int device, unsigned char** base) {
    if (device < 0 || device >= kMaxDevices) return MTK_ERR_BAD_INPUT;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_base[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || p == nullptr) {
            mtk_set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
            return MTK_ERR_CUDA;
        }
        g_base[device] = static_cast<unsigned char*>(p);
    }
    *base = g_base[device];
    return MTK_OK;
}

}  // namespace

extern "C" int mtk_field_smoothest_noalloc(int32_t nF, int32_t nRosy, const int32_t* nbr, const double* theta,
                                           const double* area, const double* x0, int32_t n_iter, double tol,
                                           int32_t max_iter, double* out, void* stream, int32_t* iterations) {
    if (nF <= 0 || nRosy <= 0 || n_iter < 0 || max_iter < 0 || !nbr || !theta || !area || !x0 || !out || !(tol >= 0))
        return MTK_ERR_BAD_INPUT;
    if (nF > kMaxFaces) {
        mtk_set_last_error("mtk_field_smoothest_noalloc: more than 409600 faces (64 MiB static scratch)", __FILE__,
                           __LINE__);
        return MTK_ERR_BAD_INPUT;
    }
    int device = 0;
    MTK_CUDA_TRY(cudaGetDevice(&device));
    unsigned char* base = nullptr;
    MTK_TRY(scratch_base(device, &base));
    int sms = 0, coop = 0, per_sm = 0;
    MTK_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    MTK_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device));
    if (!coop) {
        mtk_set_last_error("mtk_field_smoothest_noalloc: the device does not support cooperative launches", __FILE__,
                           __LINE__);
        return MTK_ERR_CUDA;
    }
    MTK_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, noalloc_power, kBlock, 0));
    if (per_sm < 1) {
        mtk_set_last_error("mtk_field_smoothest_noalloc: the solver kernel does not fit on an SM", __FILE__, __LINE__);
        return MTK_ERR_CUDA;
    }
    const int grid = sms < 512 ? sms : 512;   // one CTA per SM; partials hold 7 slots x 512 CTAs
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // what must start at zero: barrier words, error flag, bad-neighbour flag, status
    MTK_CUDA_TRY(cudaMemsetAsync(base, 0, 64, st));
    int n = nF, N = nRosy, it = n_iter, mi = max_iter;
    double t = tol;
    void* params[] = {&base, &n, &N, (void*)&nbr, (void*)&theta, (void*)&area, (void*)&x0, &it, &t, &mi, &out};
    MTK_CUDA_TRY(cudaLaunchCooperativeKernel(reinterpret_cast<void*>(noalloc_power), dim3(grid), dim3(kBlock), params, 0, st));
    int h_status[2] = {0, 0};
    MTK_CUDA_TRY(cudaMemcpyAsync(h_status, base + 32, sizeof(h_status), cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaStreamSynchronize(st));
    if (iterations) *iterations = h_status[1];
    if (h_status[0] == MTK_ERR_BAD_INPUT)
        mtk_set_last_error("mtk_field_smoothest_noalloc: a neighbour index is outside [0, nF) (other than -1) or a "
                           "face's own index", __FILE__, __LINE__);
    return h_status[0];
}
