// mg_noalloc.cu — a V-cycle entry point that allocates no memory.
//
// Some callers cannot call cudaMalloc when they need the preconditioner: a solver callback in
// another library (for example a shell preconditioner invoked inside a foreign Krylov loop)
// that must not allocate or free on every application (cudaMalloc and cudaFree can synchronise
// the device and so stall that library's pipeline), and programs that reserve their whole
// device-memory budget up front and must not grow it.  numa_gpu_mg_apply_noalloc serves them: it
// runs the same FP64 V-cycle as numa_gpu_mg_apply, with the same kernels in the same order (so
// the result is bit-identical), but every work array lives in one static device array of
// 4.8 MB (NUMA_GPU_NOALLOC_MAX_DOUBLES doubles), enough for grids up to 63^3.  Each GPU that
// loads this library holds that array until the process exits.
//
// Set-up: each call that is not being captured into a CUDA graph resolves the array's device
// address with cudaGetSymbolAddress (the first one on a device may load the module) and keeps
// it for that device; a call under stream capture launches with the kept address and makes no
// other runtime call that capture forbids.  So make one uncaptured call on the device, in the
// context the graph will run in, before capturing; after cudaDeviceReset or a change of
// context, the next uncaptured call finds the new address (graphs captured before keep the old
// one and must be captured again).
//
// Sharing: every call uses the same array and leaves its contents behind.  The V-cycle writes
// every value before it reads it, except the level iterates when pre = 0, which are cleared
// with cudaMemsetAsync.  Calls that can overlap on the GPU (unordered streams) race on the
// array: order them, or use numa_gpu_mg_apply with separate hierarchies.
//
// Errors: a CUDA error already pending when the call starts is returned as NUMA_GPU_ERR_CUDA
// and left pending (cudaPeekAtLastError), so the caller still sees its own earlier failure.
#include <cstring>
#include <mutex>

#include "mg_kernels.cuh"

namespace numa::gpu {
namespace {

static __device__ __align__(256) double g_mg_scratch[NUMA_GPU_NOALLOC_MAX_DOUBLES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch[kMaxDevices] = {};

struct NaLevel {
    int n;
    double h2inv, inv;
    size_t ox, ob, obs;  // offsets into the static array (level 0: only obs)
    double *x, *b, *bs;
};

// The reference hierarchy (poisson_mg.hpp:44-63) laid out in the static array: b*h^2 and the
// residual of the finest level first, then x, b, b*h^2 of each coarser level.  Returns the
// number of doubles used, or 0 if it exceeds the array.
size_t layout(size_t n, NaLevel* lv, int& nlev) {
    size_t m = n;
    double h2 = (static_cast<double>(n) + 1.0) * (static_cast<double>(n) + 1.0);
    const size_t N0 = n * n * n;
    size_t used = 2 * N0;
    nlev = 0;
    for (;;) {
        if (nlev >= 16) return 0;
        NaLevel& L = lv[nlev];
        L.n = static_cast<int>(m);
        L.h2inv = h2;
        L.inv = 1.0 / h2;
        const size_t Nl = m * m * m;
        if (nlev == 0) {
            L.ox = L.ob = 0;
            L.obs = 0;
        } else {
            L.ox = used;
            L.ob = used + Nl;
            L.obs = used + 2 * Nl;
            used += 3 * Nl;
        }
        ++nlev;
        if (m % 2 == 0 || m <= 1) break;
        m = (m - 1) / 2;
        h2 /= 4.0;
    }
    return used <= NUMA_GPU_NOALLOC_MAX_DOUBLES ? used : 0;
}

// The FP64 V-cycle of PoissonMG::cycle<double> on the static layout.  Returns the first
// failing enqueue's status (cudaSuccess when every launch and the memset were accepted).
cudaError_t na_cycle(NaLevel* lv, int nlev, int l, double* resid, int pre, int post, cudaStream_t s) {
    NaLevel& L = lv[l];
    const int n = L.n;
    const dim3 blk(BX, BY);
    const dim3 cgrid(((n + 1) / 2 + BX - 1) / BX, (n + BY - 1) / BY, n);
    auto pass = [&](int colour, bool first) {
        if (first) k_rbgs<double, true, false><<<cgrid, blk, 0, s>>>(L.x, L.bs, nullptr, n, colour);
        else k_rbgs<double, false, false><<<cgrid, blk, 0, s>>>(L.x, L.bs, nullptr, n, colour);
    };
    auto sweep = [&](int order, bool first) {
        const int c0 = order == 0 ? 0 : 1;
        pass(c0, first);
        pass(1 - c0, false);
    };
    if (l + 1 == nlev) {
        if (n == 1) k_single<double><<<1, 1, 0, s>>>(L.b, L.x, nullptr, 6.0 * L.h2inv);
        else
            for (int sw = 0; sw < 30; ++sw) sweep(sw % 2, sw == 0);
        return cudaPeekAtLastError();
    }
    for (int sw = 0; sw < pre; ++sw) sweep(0, sw == 0);
    if (pre == 0) {
        const cudaError_t e = cudaMemsetAsync(L.x, 0, (size_t)n * n * n * sizeof(double), s);
        if (e != cudaSuccess) return e;
    }
    {
        const int ichunk = n >= 64 ? 8 : 1;
        const dim3 g((n + BX - 1) / BX, (n + BY - 1) / BY, (n + ichunk - 1) / ichunk);
        k_residual<double><<<g, blk, 0, s>>>(L.x, L.b, resid, n, ichunk, L.h2inv);
    }
    NaLevel& C = lv[l + 1];
    const int nc = C.n;
    k_restrict<double><<<dim3((nc + BX - 1) / BX, (nc + BY - 1) / BY, nc), blk, 0, s>>>(resid, C.b, C.bs, n, nc, C.inv);
    const cudaError_t ec = na_cycle(lv, nlev, l + 1, resid, pre, post, s);
    if (ec != cudaSuccess) return ec;
    if (post > 0)
        k_prolong<double, true><<<dim3(((n + 1) / 2 + BX - 1) / BX, (n + BY - 1) / BY, n), blk, 0, s>>>(C.x, L.x, nc, n);
    else
        k_prolong<double, false><<<dim3((n + BX - 1) / BX, (n + BY - 1) / BY, n), blk, 0, s>>>(C.x, L.x, nc, n);
    for (int sw = 0; sw < post; ++sw) sweep(1, false);
    return cudaPeekAtLastError();
}

}  // namespace
}  // namespace numa::gpu

using namespace numa::gpu;

extern "C" int numa_gpu_mg_apply_noalloc(size_t n, int pre, int post, const double* r, double* z, void* stream) {
    if (n == 0 || pre < 0 || post < 0 || !r || !z || r == z) return NUMA_GPU_ERR_INVALID_ARGUMENT;
    if (n > 1024) return NUMA_GPU_ERR_TOO_LARGE;
    NaLevel lv[16];
    int nlev = 0;
    if (layout(n, lv, nlev) == 0) return NUMA_GPU_ERR_TOO_LARGE;
    // an error left by an earlier call of the caller's is reported, not consumed
    if (cudaPeekAtLastError() != cudaSuccess) return NUMA_GPU_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return NUMA_GPU_ERR_NO_DEVICE;
    }
    if (dev < 0 || dev >= kMaxDevices) return NUMA_GPU_ERR_NOT_SUPPORTED;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // Outside stream capture the array's address is looked up on every call, so a call after
    // cudaDeviceReset or under another context of the device finds the current one; a call
    // being captured uses the address its device's last uncaptured call found.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) {
        cudaGetLastError();
        return NUMA_GPU_ERR_CUDA;
    }
    double* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_scratch[dev] || cap == cudaStreamCaptureStatusNone) {
            void* p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_mg_scratch);
            if (e != cudaSuccess || p == nullptr) {
                cudaGetLastError();
                return NUMA_GPU_ERR_CUDA;
            }
            g_scratch[dev] = static_cast<double*>(p);
        }
        base = g_scratch[dev];
    }
    for (int l = 0; l < nlev; ++l) {
        lv[l].x = base + lv[l].ox;
        lv[l].b = base + lv[l].ob;
        lv[l].bs = base + lv[l].obs;
    }
    const size_t N0 = n * n * n;
    double* resid = base + N0;
    // finest level: smooth in z, read r in place, b*h^2 into the array (poisson_mg.hpp:76-79)
    lv[0].x = z;
    lv[0].b = const_cast<double*>(r);
    const unsigned g = static_cast<unsigned>((N0 + 255) / 256 < 4096 ? (N0 + 255) / 256 : 4096);
    k_scale_in64<<<g, 256, 0, s>>>(r, lv[0].bs, lv[0].inv, N0);
    const cudaError_t e0 = cudaPeekAtLastError();
    const cudaError_t e = e0 != cudaSuccess ? e0 : na_cycle(lv, nlev, 0, resid, pre, post, s);
    if (e != cudaSuccess) {
        cudaGetLastError();  // this call's own launch error: reported through the status
        return NUMA_GPU_ERR_CUDA;
    }
    return NUMA_GPU_OK;
}
