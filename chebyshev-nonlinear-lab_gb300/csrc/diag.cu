// diag.cu — diagnostics for the roofline report: the measured FP64 FMA rate of this GPU and
// event-timed launches of the dominant kernels.  No counterpart in the reference.
#include <algorithm>
#include <cmath>

#include "numa_internal.hpp"

namespace numa::gpu {
namespace {

// Eight independent FMA chains per thread: issue-bound on the FP64 pipe.
__global__ void k_fma_chain(double* out, int iters, double a, double b) {
    double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = __fma_rn(x0, a, b);
        x1 = __fma_rn(x1, a, b);
        x2 = __fma_rn(x2, a, b);
        x3 = __fma_rn(x3, a, b);
        x4 = __fma_rn(x4, a, b);
        x5 = __fma_rn(x5, a, b);
        x6 = __fma_rn(x6, a, b);
        x7 = __fma_rn(x7, a, b);
    }
    const double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == -12345.678) out[0] = s;  // keeps the chains live; never true for these inputs
}

// out = exp_tang(x) and, in ref, CUDA's exp(x) (for accuracy tests of the table-driven e^x)
__global__ void k_exp_pair(const double* __restrict__ x, double* __restrict__ out, double* __restrict__ ref,
                           size_t N) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < N; p += stride) {
        out[p] = exp_tang(x[p]);
        if (ref) ref[p] = exp(x[p]);
    }
}

// out = a / b through the finite-difference quotients' reciprocal form
__global__ void k_div_recip(const double* __restrict__ a, double b, double* __restrict__ out, size_t N) {
    const double y = recip_for_div(b);
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < N; p += stride)
        out[p] = div_by_recip(a[p], b, y);
}

}  // namespace

void diag_div(Context& ctx, const double* a, double b, double* out, size_t N) {
    size_t g = (N + 255) / 256, cap = (size_t)ctx.sm_count * 16;
    k_div_recip<<<(unsigned)std::max<size_t>(1, std::min(g, cap)), 256, 0, ctx.stream>>>(a, b, out, N);
    ctx.count_launch();
    ctx.check_launch("diag div");
}

void diag_exp(Context& ctx, const double* x, double* out, double* ref, size_t N) {
    size_t g = (N + 255) / 256, cap = (size_t)ctx.sm_count * 16;
    k_exp_pair<<<(unsigned)std::max<size_t>(1, std::min(g, cap)), 256, 0, ctx.stream>>>(x, out, ref, N);
    ctx.count_launch();
    ctx.check_launch("diag exp");
}

double diag_fp64_peak_tflops(Context& ctx) {
    const int blocks = ctx.sm_count * 8, threads = 256, iters = 2000;
    DeviceArray<double> sink(1);
    cudaEvent_t a, b;
    NUMA_CUDA(cudaEventCreate(&a));
    NUMA_CUDA(cudaEventCreate(&b));
    k_fma_chain<<<blocks, threads, 0, ctx.stream>>>(sink.p, 10, 0.999, 1e-3);
    NUMA_CUDA(cudaEventRecord(a, ctx.stream));
    k_fma_chain<<<blocks, threads, 0, ctx.stream>>>(sink.p, iters, 0.999, 1e-3);
    NUMA_CUDA(cudaEventRecord(b, ctx.stream));
    ctx.count_launch(2);
    NUMA_CUDA(cudaEventSynchronize(b));
    float ms = 0.f;
    NUMA_CUDA(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
    return flops / (ms * 1e-3) / 1e12;
}

}  // namespace numa::gpu
