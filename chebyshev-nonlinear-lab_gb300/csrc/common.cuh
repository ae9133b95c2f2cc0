// common.cuh — shared device helpers and the host-side context of libnuma_gpu.
//
// Design notes for GB300 (sm_103a):
//  * FP64 arithmetic runs at ~1.2 TFLOP/s on this part (measured), 1/58 of FP32, so every FP64
//    kernel here is bound by its FP64 instruction count, not by HBM.  Kernels therefore avoid
//    redundant FP64 work (no halo recomputation, cached lambda*e^u, precomputed b*h^2, the
//    3-operation correctly-rounded division by 6 below) and trade memory traffic for FP64 ops.
//  * FP32 kernels (the mixed-precision V-cycle) are bound by HBM bandwidth.
//  * The library is built with -fmad=false: no multiply-add is contracted unless written as an
//    explicit fma, so element-wise results follow the reference's IEEE operation sequence.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <mutex>
#include <utility>
#include <stdexcept>
#include <string>

#include "../../include/numa_gpu.h"

namespace numa::gpu {

// ------------------------------------------------------------------------------------------
// Errors: internal code throws Status; the C ABI converts it to an int status code.
struct Status : std::runtime_error {
    int code;
    Status(int c, const std::string& msg) : std::runtime_error(msg), code(c) {}
};

[[noreturn]] void throw_cuda(cudaError_t e, const char* what, const char* file, int line);

#define NUMA_CUDA(expr)                                                              \
    do {                                                                             \
        cudaError_t numa_cuda_err_ = (expr);                                         \
        if (numa_cuda_err_ != cudaSuccess)                                           \
            ::numa::gpu::throw_cuda(numa_cuda_err_, #expr, __FILE__, __LINE__);      \
    } while (0)

// ------------------------------------------------------------------------------------------
// Reduction protocol.  A reducing kernel accumulates per-thread FP64 sums, reduces them within
// the block (warp shuffles, then shared memory), writes one partial per block and result, and
// takes a ticket; the last block to arrive sums the partials in block order and calls the
// kernel's finaliser.  The summation order depends only on the launch shape, so results are
// reproducible run to run.
constexpr int kMaxRedBlocks = 8192;   // partials per result
constexpr int kMaxRedResults = 64;    // results per reducing kernel (multi-dot width)
constexpr int kRedThreads = 256;

struct RedArgs {
    double* partials;   // kMaxRedBlocks * kMaxRedResults
    unsigned* ticket;   // one counter, reset to 0 by the last block
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of R values per thread; every thread of the block must call it.  Returns the
// block totals in warp 0 lane 0 (others hold unspecified values).
template <int R>
__device__ __forceinline__ void block_sum(double (&v)[R], double (*smem)[32]) {
    const int lane = threadIdx.x & 31;
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int warp = tid >> 5;
    const int nwarps = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        double s = warp_sum(v[r]);
        if ((tid & 31) == 0) smem[r][warp] = s;
    }
    (void)lane;
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            double s = (tid < nwarps) ? smem[r][tid] : 0.0;
            v[r] = warp_sum(s);
        }
    }
    __syncthreads();
}

// Publishes this block's totals and, in the last block to finish, reduces all partials and
// calls fin(totals) on thread 0.  `v` must hold the block totals in thread 0 (block_sum output).
template <int R, class Fin>
__device__ __forceinline__ void grid_reduce_finish(const double (&v)[R], RedArgs red, Fin fin) {
    __shared__ bool am_last;
    __shared__ double tot_smem[R][32];
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const unsigned nblocks = gridDim.x * gridDim.y * gridDim.z;
    const unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    if (tid == 0) {
#pragma unroll
        for (int r = 0; r < R; ++r) red.partials[(size_t)r * kMaxRedBlocks + bid] = v[r];
        __threadfence();
        const unsigned t = atomicAdd(red.ticket, 1u);
        am_last = (t == nblocks - 1);
    }
    __syncthreads();
    if (!am_last) return;
    __threadfence();
    const int nthreads = blockDim.x * blockDim.y * blockDim.z;
    double acc[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        double s = 0.0;
        for (unsigned b = tid; b < nblocks; b += nthreads) s += __ldcg(red.partials + (size_t)r * kMaxRedBlocks + b);
        acc[r] = s;
    }
    block_sum<R>(acc, tot_smem);
    if (tid == 0) {
        fin(acc);
        *red.ticket = 0u;
    }
}

// ------------------------------------------------------------------------------------------
// Correctly rounded s / 6 in three FP64 operations (Markstein's correction: q = s*RN(1/6),
// e = s - 6q exactly by FMA, q + e*RN(1/6)).  Equal to IEEE s / 6.0 for every finite s outside
// the subnormal range (checked against IEEE division on the GPU and on 2e8 random values on the
// CPU); the sign of a zero result may differ, which no later operation observes.
__device__ __forceinline__ double div6(double s) {
    const double r = 0.16666666666666666;  // RN(1/6)
    const double q = __dmul_rn(s, r);
    const double e = __fma_rn(-q, 6.0, s);
    return __fma_rn(e, r, q);
}
__device__ __forceinline__ float div6(float s) {
    const float r = 0.16666667f;
    const float q = __fmul_rn(s, r);
    const float e = __fmaf_rn(-q, 6.0f, s);
    return __fmaf_rn(e, r, q);
}

// a / d given rd = RN(1/d): the same correction for a runtime divisor.  Within one ulp of IEEE
// division and equal to it for all but rare (a, d) pairs.
__device__ __forceinline__ double div_by(double a, double d, double rd) {
    const double q = __dmul_rn(a, rd);
    const double e = __fma_rn(-q, d, a);
    return __fma_rn(e, rd, q);
}

// ------------------------------------------------------------------------------------------
// FP64 <-> FP32 conversions in integer arithmetic.  On this GPU the hardware conversion
// instructions issue on the (slow) FP64 pipe; these use only integer instructions and give the
// same results: round-to-nearest-even from the IEEE-754 bit fields, with the rare cases (float
// subnormals, NaN) handed to the hardware instruction.
__device__ __forceinline__ float f64_to_f32(double d) {
    const unsigned hi = (unsigned)__double2hiint(d);
    const unsigned lo = (unsigned)__double2loint(d);
    const unsigned sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7FFu);
    const int ef = e - 896;  // re-biased exponent (1023 -> 127)
    if (ef >= 1 && ef < 255) {
        unsigned m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);  // top 23 fraction bits
        const unsigned rem = lo & 0x1FFFFFFFu;             // the 29 bits dropped
        unsigned bits = ((unsigned)ef << 23) | m;
        bits += (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) ? 1u : 0u;  // carries into the exponent
        if (bits >= 0x7F800000u) bits = 0x7F800000u;                                // overflow to infinity
        return __uint_as_float(sign | bits);
    }
    if (e == 0 || ef <= -25) return __uint_as_float(sign);  // zero, or too small for a float subnormal
    if (ef >= 255 && e != 0x7FF) return __uint_as_float(sign | 0x7F800000u);
    return __double2float_rn(d);  // float subnormals, infinities and NaN: the hardware conversion
}

__device__ __forceinline__ double f32_to_f64(float f) {
    const unsigned b = __float_as_uint(f);
    const unsigned ef = (b >> 23) & 0xFFu;
    if (ef - 1u < 254u) {  // normal: exact re-bias and shift
        const unsigned hi = (b & 0x80000000u) | ((ef + 896u) << 20) | ((b & 0x7FFFFFu) >> 3);
        const unsigned lo = b << 29;
        return __hiloint2double((int)hi, (int)lo);
    }
    if ((b & 0x7FFFFFFFu) == 0u) return __hiloint2double((int)(b & 0x80000000u), 0);
    return (double)f;  // subnormal, infinity, NaN
}

// RN(a / b) from y = RN(1/b), for many a divided by one b (Markstein's correction): q = RN(a y) is
// within one ulp of a/b, r = a - b q is exact by FMA, and RN(q + r y) is the correctly rounded
// quotient.  That needs a, q and y well inside the normal range (r ~ 2^-52 a must not underflow):
// outside [2^-960, 2^1001) — zeros, subnormals, infinities, NaN — the IEEE division runs instead.
// Three FP64 instructions instead of a full division.
__device__ __forceinline__ unsigned fp64_biased_exp(double v) {
    return ((unsigned)__double2hiint(v) >> 20) & 0x7FFu;
}
// y for div_by_recip: RN(1/b), or 0 (every quotient then takes the IEEE division) when b is outside
// [2^-960, 2^960].
__device__ __forceinline__ double recip_for_div(double b) {
    return fp64_biased_exp(b) - 63u <= 1920u ? __ddiv_rn(1.0, b) : 0.0;
}
__device__ __forceinline__ double div_by_recip(double a, double b, double y) {
    const double q = __dmul_rn(a, y);
    const double r = __fma_rn(-q, b, a);
    const double q2 = __fma_rn(r, y, q);
    if (fp64_biased_exp(a) - 63u > 1960u || fp64_biased_exp(q2) - 63u > 1960u) return __ddiv_rn(a, b);
    return q2;
}

// ------------------------------------------------------------------------------------------
// e^x by Tang's table-driven method (P. T. P. Tang, "Table-driven implementation of the
// exponential function in IEEE floating-point arithmetic", ACM TOMS 15(2):144-157, 1989):
//   x = (32 M + j) ln2/32 + r, |r| <= ln2/64,   e^x = 2^M * 2^(j/32) * e^r,
// with 2^(j/32) from a 32-entry table held as hi + lo (hi = RN(2^(j/32)), lo = RN(2^(j/32) - hi))
// and e^r - 1 = r + r^2 (1/2! + r (1/3! + r (1/4! + r (1/5! + r / 6!)))) (Taylor; truncation below
// 2e-18).  ln2/32 is split as L1 + L2 and N = round(32 x / ln2) comes from the 1.5 * 2^52
// shifter, so the reduction is exact to ~1e-21; the result is within ~0.54 ulp of e^x (Tang's
// bound).  Twelve FP64 instructions, against the FP64 pipe that bounds the residual kernels;
// the table index, 2^M and the range test are integer work.  |x| >= 708 (overflow, results near
// or below the smallest normal, infinities, NaN) is left to exp().
// Table: 2^(j/32), j = 0..31, computed at 60 significant digits.
__device__ const double2 kExp2Frac[32] = {
    {0x1.0000000000000p+0, 0x0.0p+0},
    {0x1.059b0d3158574p+0, 0x1.d73e2a475b465p-55},
    {0x1.0b5586cf9890fp+0, 0x1.8a62e4adc610bp-54},
    {0x1.11301d0125b51p+0, -0x1.6c51039449b3ap-54},
    {0x1.172b83c7d517bp+0, -0x1.19041b9d78a76p-55},
    {0x1.1d4873168b9aap+0, 0x1.e016e00a2643cp-54},
    {0x1.2387a6e756238p+0, 0x1.9b07eb6c70573p-54},
    {0x1.29e9df51fdee1p+0, 0x1.612e8afad1255p-55},
    {0x1.306fe0a31b715p+0, 0x1.6f46ad23182e4p-55},
    {0x1.371a7373aa9cbp+0, -0x1.63aeabf42eae2p-54},
    {0x1.3dea64c123422p+0, 0x1.ada0911f09ebcp-55},
    {0x1.44e086061892dp+0, 0x1.89b7a04ef80d0p-59},
    {0x1.4bfdad5362a27p+0, 0x1.d4397afec42e2p-56},
    {0x1.5342b569d4f82p+0, -0x1.07abe1db13cadp-55},
    {0x1.5ab07dd485429p+0, 0x1.6324c054647adp-54},
    {0x1.6247eb03a5585p+0, -0x1.383c17e40b497p-54},
    {0x1.6a09e667f3bcdp+0, -0x1.bdd3413b26456p-54},
    {0x1.71f75e8ec5f74p+0, -0x1.16e4786887a99p-55},
    {0x1.7a11473eb0187p+0, -0x1.41577ee04992fp-55},
    {0x1.82589994cce13p+0, -0x1.d4c1dd41532d8p-54},
    {0x1.8ace5422aa0dbp+0, 0x1.6e9f156864b27p-54},
    {0x1.93737b0cdc5e5p+0, -0x1.75fc781b57ebcp-57},
    {0x1.9c49182a3f090p+0, 0x1.c7c46b071f2bep-56},
    {0x1.a5503b23e255dp+0, -0x1.d2f6edb8d41e1p-54},
    {0x1.ae89f995ad3adp+0, 0x1.7a1cd345dcc81p-54},
    {0x1.b7f76f2fb5e47p+0, -0x1.5584f7e54ac3bp-56},
    {0x1.c199bdd85529cp+0, 0x1.11065895048ddp-55},
    {0x1.cb720dcef9069p+0, 0x1.503cbd1e949dbp-56},
    {0x1.d5818dcfba487p+0, 0x1.2ed02d75b3707p-55},
    {0x1.dfc97337b9b5fp+0, -0x1.1a5cd4f184b5cp-54},
    {0x1.ea4afa2a490dap+0, -0x1.e9c23179c2893p-54},
    {0x1.f50765b6e4540p+0, 0x1.9d3e12dd8a18bp-54},
};

__device__ __forceinline__ double exp_tang(double x) {
    if ((__double2hiint(x) & 0x7FFFFFFF) >= 0x40862000) return exp(x);  // |x| >= 708, inf, NaN
    const double shift = 0x1.8p52;
    const double t = __fma_rn(x, 0x1.71547652b82fep+5, shift);  // 32/ln2
    const double nd = __dsub_rn(t, shift);                       // N = round(32 x / ln2), exact
    const int N = __double2loint(t);
    double r = __fma_rn(-nd, 0x1.62e42fefa39efp-6, x);  // L1 = RN(ln2/32)
    r = __fma_rn(-nd, 0x1.abc9e3b39803fp-61, r);         // L2 = RN(ln2/32 - L1)
    double q = __fma_rn(r, 0x1.6c16c16c16c17p-10, 0x1.1111111111111p-7);
    q = __fma_rn(r, q, 0x1.5555555555555p-5);
    q = __fma_rn(r, q, 0x1.5555555555555p-3);
    q = __fma_rn(r, q, 0.5);
    const double p = __fma_rn(__dmul_rn(r, r), q, r);  // e^r - 1
    const double2 T = __ldg(&kExp2Frac[N & 31]);
    const double y = __dadd_rn(T.x, __fma_rn(T.x, p, T.y));  // 2^(j/32) e^r, in [0.98, 2.03]
    // y * 2^M, M = floor(N / 32), by adding M to the exponent field: for |x| < 708 the result is
    // a normal number
    return __hiloint2double(__double2hiint(y) + (N >> 5) * (1 << 20), __double2loint(y));
}

// ------------------------------------------------------------------------------------------
// One process-wide lock held across every CUDA-graph capture and around every device or pinned
// allocation and free: cudaFree / cudaMallocHost may synchronise the whole device, which would
// break a capture another thread (another context) has in progress.  Recursive, so a capture
// that allocated would fail in CUDA rather than deadlock here.
std::recursive_mutex& alloc_capture_mutex();

// ------------------------------------------------------------------------------------------
// Host-side context: one device, one stream, reduction scratch and device scalars.
constexpr int kNumScalars = 2048;
constexpr size_t kMaxRestart = 250;  // GMRES(m) limit of the device scalar layout below

struct Context {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    RedArgs red{};
    double* d_scalars = nullptr;  // kNumScalars device scalars
    double* h_scalars = nullptr;  // pinned host mirror
    cudaEvent_t done = nullptr;
    uint64_t launches = 0;
    bool timing = false;
    std::string last_error;

    explicit Context(int dev);
    ~Context();
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;

    void sync();
    // Copies count device doubles to host memory and waits for them.
    void fetch(const double* dsrc, int count, double* host);
    double fetch1(const double* dsrc) {
        double v;
        fetch(dsrc, 1, &v);
        return v;
    }
    double* scalar(int slot) { return d_scalars + slot; }
    // Number of blocks of kRedThreads threads for a grid-stride reduction over N elements.
    unsigned red_grid(size_t N) const;
    void count_launch(unsigned n = 1) { launches += n; }
    void check_launch(const char* what);
};
// Programmatic dependent launch.  A kernel launched by launch_pdl may be scheduled while its
// predecessor on the stream is still running; it must call pdl_wait() before it touches memory
// (griddepcontrol.wait returns once every prerequisite grid has completed and its writes are
// visible).  pdl_trigger() lets this grid's own dependents be scheduled once all its CTAs have
// issued it; they still wait for its completion.  Both are no-ops in a kernel launched normally.
// In a chain of small kernels (the coarse levels of a V-cycle) this hides the launch latency
// between consecutive kernels, on a stream or inside a captured graph.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <class... KArgs, class... Args>
void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    NUMA_CUDA(cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...));
}

// Largest dynamic shared memory a block may opt in to on the context's device (bytes).
int smem_optin_limit(Context& ctx);

// Sets a kernel's dynamic shared-memory limit to the most the device allows beside the kernel's
// static shared memory, and returns it.  The attribute belongs to the kernel, not to one caller:
// a fixed value lets hierarchies and grids of any size share the kernel (a caller setting its own
// need would lower the limit under another's launch).
template <class K>
int set_dynamic_smem_limit(Context& ctx, K* kernel) {
    cudaFuncAttributes a;
    NUMA_CUDA(cudaFuncGetAttributes(&a, kernel));
    const int lim = smem_optin_limit(ctx) - (int)a.sharedSizeBytes;
    NUMA_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, lim));
    return lim;
}

// Device scalar slots with fixed roles.
enum ScalarSlot : int {
    kSlotTmp0 = 0,        // public-API reductions
    kSlotTmp1 = 1,
    kSlotNormF = 8,       // ||F|| of the last evaluation
    kSlotFdH = 16,        // finite-difference step h, 1/h, zero-direction flag
    kSlotFdRh = 17,
    kSlotFdZero = 18,
    kSlotFdXnorm = 19,
    kSlotFdInvH = 20,     // RN(1/h) and RN(1/h^2) for the quotients
    kSlotFdInvHH = 21,
    kSlotGmresH = 64,     // Hessenberg column, m + 2 entries
    kSlotGmresH2 = 320,   // CGS2 second-pass coefficients, up to 8
    kSlotGmresY = 400,    // least-squares solution y, m entries
    kSlotGmresCoef = 700, // recycled-solve coefficients, 2k + 1 entries
    kSlotGmresSig2 = 1250, // lazily normalised basis: 1 / norm^2 of each vector, m + 1 entries
};

// Pinned host staging for small vectors moving to the device.
struct PinnedBuf {
    double* p = nullptr;
    size_t cap = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf&) = delete;
    PinnedBuf& operator=(const PinnedBuf&) = delete;
    ~PinnedBuf() {
        if (p) {
            std::lock_guard<std::recursive_mutex> lk(alloc_capture_mutex());
            cudaFreeHost(p);
        }
    }
    double* get(size_t count) {
        if (count > cap) {
            std::lock_guard<std::recursive_mutex> lk(alloc_capture_mutex());
            if (p) cudaFreeHost(p);
            p = nullptr;
            cap = 0;
            NUMA_CUDA(cudaMallocHost(reinterpret_cast<void**>(&p), count * sizeof(double)));
            cap = count;
        }
        return p;
    }
};

// Owning device array with capacity reuse.
template <class T>
struct DeviceArray {
    T* p = nullptr;
    size_t n = 0;
    size_t cap = 0;
    DeviceArray() = default;
    explicit DeviceArray(size_t count) { resize(count); }
    ~DeviceArray() { release(); }
    DeviceArray(const DeviceArray&) = delete;
    DeviceArray& operator=(const DeviceArray&) = delete;
    DeviceArray(DeviceArray&& o) noexcept : p(o.p), n(o.n), cap(o.cap) { o.p = nullptr; o.n = o.cap = 0; }
    DeviceArray& operator=(DeviceArray&& o) noexcept {
        if (this != &o) {
            release();
            p = o.p; n = o.n; cap = o.cap;
            o.p = nullptr; o.n = o.cap = 0;
        }
        return *this;
    }
    void resize(size_t count) {
        if (count > cap) {
            std::lock_guard<std::recursive_mutex> lk(alloc_capture_mutex());
            release();
            if (count > 0) {
                cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(T));
                if (e == cudaErrorMemoryAllocation) {
                    cudaGetLastError();
                    p = nullptr;
                    throw Status(NUMA_GPU_ERR_OUT_OF_MEMORY, "cudaMalloc failed: out of device memory");
                }
                NUMA_CUDA(e);
            }
            cap = count;
        }
        n = count;
    }
    void release() {
        if (p) {
            std::lock_guard<std::recursive_mutex> lk(alloc_capture_mutex());
            cudaFree(p);
        }
        p = nullptr;
        n = cap = 0;
    }
    void swap(DeviceArray& o) noexcept {
        std::swap(p, o.p);
        std::swap(n, o.n);
        std::swap(cap, o.cap);
    }
};

}  // namespace numa::gpu

// Public opaque handle types (declared in numa_gpu.h).
struct numa_gpu_ctx {
    numa::gpu::Context* impl;
};

struct numa_gpu_vec {
    numa_gpu_ctx* ctx;
    double* d;
    size_t n;
    bool owns;
};
