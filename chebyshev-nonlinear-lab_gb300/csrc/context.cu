// context.cu — context, device vectors and the BLAS-1 kernels of operators/operator.hpp:19-41.
#include <cstdio>
#include <string>

#include "numa_internal.hpp"

namespace numa::gpu {

void throw_cuda(cudaError_t e, const char* what, const char* file, int line) {
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s failed at %s:%d: %s", what, file, line, cudaGetErrorString(e));
    if (e == cudaErrorMemoryAllocation) throw Status(NUMA_GPU_ERR_OUT_OF_MEMORY, buf);
    if (e == cudaErrorNoDevice || e == cudaErrorInvalidDevice || e == cudaErrorInsufficientDriver)
        throw Status(NUMA_GPU_ERR_NO_DEVICE, buf);
    throw Status(NUMA_GPU_ERR_CUDA, buf);
}

int smem_optin_limit(Context& ctx) {
    int v = 0;
    NUMA_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx.device));
    return v;
}

std::recursive_mutex& alloc_capture_mutex() {
    static std::recursive_mutex m;
    return m;
}

Context::Context(int dev) : device(dev) {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        cudaGetLastError();
        throw Status(NUMA_GPU_ERR_NO_DEVICE, "no CUDA device is available");
    }
    if (dev < 0 || dev >= count) throw Status(NUMA_GPU_ERR_NO_DEVICE, "device index out of range");
    NUMA_CUDA(cudaSetDevice(dev));
    NUMA_CUDA(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev));
    NUMA_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    std::lock_guard<std::recursive_mutex> lk(alloc_capture_mutex());
    NUMA_CUDA(cudaMalloc(reinterpret_cast<void**>(&red.partials),
                         sizeof(double) * kMaxRedBlocks * kMaxRedResults));
    NUMA_CUDA(cudaMalloc(reinterpret_cast<void**>(&red.ticket), sizeof(unsigned)));
    NUMA_CUDA(cudaMemset(red.ticket, 0, sizeof(unsigned)));
    NUMA_CUDA(cudaMalloc(reinterpret_cast<void**>(&d_scalars), sizeof(double) * kNumScalars));
    NUMA_CUDA(cudaMemset(d_scalars, 0, sizeof(double) * kNumScalars));
    NUMA_CUDA(cudaMallocHost(reinterpret_cast<void**>(&h_scalars), sizeof(double) * kNumScalars));
    NUMA_CUDA(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
    NUMA_CUDA(cudaDeviceSynchronize());
}

Context::~Context() {
    if (stream) cudaStreamSynchronize(stream);
    std::lock_guard<std::recursive_mutex> lk(alloc_capture_mutex());
    if (red.partials) cudaFree(red.partials);
    if (red.ticket) cudaFree(red.ticket);
    if (d_scalars) cudaFree(d_scalars);
    if (h_scalars) cudaFreeHost(h_scalars);
    if (done) cudaEventDestroy(done);
    if (stream) cudaStreamDestroy(stream);
}

void Context::sync() { NUMA_CUDA(cudaStreamSynchronize(stream)); }

void Context::fetch(const double* dsrc, int count, double* host) {
    if (count <= 0) return;
    if (count > kNumScalars) throw Status(NUMA_GPU_ERR_INVALID_ARGUMENT, "fetch too large");
    NUMA_CUDA(cudaMemcpyAsync(h_scalars, dsrc, sizeof(double) * count, cudaMemcpyDeviceToHost, stream));
    NUMA_CUDA(cudaStreamSynchronize(stream));
    for (int i = 0; i < count; ++i) host[i] = h_scalars[i];
}

unsigned Context::red_grid(size_t N) const {
    size_t want = (N + kRedThreads * 4 - 1) / (kRedThreads * 4);
    size_t cap = static_cast<size_t>(sm_count) * 8;
    if (want > cap) want = cap;
    if (want < 1) want = 1;
    return static_cast<unsigned>(want);
}

void Context::check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw_cuda(e, what, __FILE__, __LINE__);
}

// ------------------------------------------------------------------------------ kernels
namespace {

struct StoreSum {
    double* out;
    __device__ void operator()(const double (&t)[1]) const { *out = t[0]; }
};
struct StoreSqrt {
    double* out;
    __device__ void operator()(const double (&t)[1]) const { *out = __dsqrt_rn(t[0]); }
};

template <class Fin>
__global__ void __launch_bounds__(kRedThreads) k_dot(const double* __restrict__ a, const double* __restrict__ b,
                                                     size_t N, RedArgs red, Fin fin) {
    pdl_wait();
    pdl_trigger();
    __shared__ double sm[1][32];
    double s[1] = {0.0};
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride)
        s[0] = __fma_rn(a[i], b[i], s[0]);
    block_sum<1>(s, sm);
    grid_reduce_finish<1>(s, red, fin);
}

__global__ void k_axpy(double a, const double* __restrict__ x, double* __restrict__ y, size_t N) {
    pdl_wait();
    pdl_trigger();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride)
        y[i] = y[i] + a * x[i];
}

__global__ void k_fill(double* __restrict__ y, double v, size_t N) {
    pdl_wait();
    pdl_trigger();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride) y[i] = v;
}

__global__ void k_newton_step(const double* __restrict__ x, const double* __restrict__ z, double lam,
                              double* __restrict__ xn, size_t N) {
    pdl_wait();
    pdl_trigger();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride)
        xn[i] = x[i] - lam * z[i];
}

// xn = x - z: the full step (lam = 1, where lam z = z exactly), one FP64 instruction a point
__global__ void k_newton_full_step(const double* __restrict__ x, const double* __restrict__ z, double* __restrict__ xn,
                                   size_t N) {
    pdl_wait();
    pdl_trigger();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride) xn[i] = x[i] - z[i];
}

__global__ void k_cheb_step(const double* __restrict__ x, const double* __restrict__ z,
                            const double* __restrict__ u, double* __restrict__ xn, size_t N) {
    pdl_wait();
    pdl_trigger();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride)
        xn[i] = x[i] - z[i] - 0.5 * u[i];
}

__global__ void k_scale(double* __restrict__ y, double a, size_t N) {
    pdl_wait();
    pdl_trigger();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += stride) y[i] = a * y[i];
}

}  // namespace

static unsigned elementwise_grid(const Context& ctx, size_t N) {
    size_t want = (N + 255) / 256;
    size_t cap = static_cast<size_t>(ctx.sm_count) * 16;
    if (want > cap) want = cap;
    return static_cast<unsigned>(want < 1 ? 1 : want);
}

void dev_dot(Context& ctx, const double* a, const double* b, size_t N, double* out) {
    launch_pdl(k_dot<StoreSum>, ctx.red_grid(N), kRedThreads, 0, ctx.stream, a, b, N, ctx.red, StoreSum{out});
    ctx.count_launch();
    ctx.check_launch("dot");
}

void dev_norm2(Context& ctx, const double* a, size_t N, double* out) {
    launch_pdl(k_dot<StoreSqrt>, ctx.red_grid(N), kRedThreads, 0, ctx.stream, a, a, N, ctx.red, StoreSqrt{out});
    ctx.count_launch();
    ctx.check_launch("norm2");
}

void dev_axpy(Context& ctx, double a, const double* x, double* y, size_t N) {
    if (N == 0) return;
    launch_pdl(k_axpy, elementwise_grid(ctx, N), 256, 0, ctx.stream, a, x, y, N);
    ctx.count_launch();
    ctx.check_launch("axpy");
}

void dev_fill(Context& ctx, double* y, double value, size_t N) {
    if (N == 0) return;
    if (value == 0.0) {
        NUMA_CUDA(cudaMemsetAsync(y, 0, N * sizeof(double), ctx.stream));
        return;
    }
    launch_pdl(k_fill, elementwise_grid(ctx, N), 256, 0, ctx.stream, y, value, N);
    ctx.count_launch();
    ctx.check_launch("fill");
}

void dev_copy(Context& ctx, const double* src, double* dst, size_t N) {
    if (N == 0 || src == dst) return;
    NUMA_CUDA(cudaMemcpyAsync(dst, src, N * sizeof(double), cudaMemcpyDeviceToDevice, ctx.stream));
}

void dev_newton_step(Context& ctx, const double* x, const double* z, double lam, double* xn, size_t N) {
    if (lam == 1.0) launch_pdl(k_newton_full_step, elementwise_grid(ctx, N), 256, 0, ctx.stream, x, z, xn, N);
    else launch_pdl(k_newton_step, elementwise_grid(ctx, N), 256, 0, ctx.stream, x, z, lam, xn, N);
    ctx.count_launch();
    ctx.check_launch("newton_step");
}

void dev_cheb_step(Context& ctx, const double* x, const double* z, const double* u, double* xn, size_t N) {
    launch_pdl(k_cheb_step, elementwise_grid(ctx, N), 256, 0, ctx.stream, x, z, u, xn, N);
    ctx.count_launch();
    ctx.check_launch("cheb_step");
}

void dev_scale_inplace(Context& ctx, double* y, double a, size_t N) {
    launch_pdl(k_scale, elementwise_grid(ctx, N), 256, 0, ctx.stream, y, a, N);
    ctx.count_launch();
    ctx.check_launch("scale");
}

}  // namespace numa::gpu
