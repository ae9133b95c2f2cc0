// learned_conv.cuh — 3x3x3 convolutions of the learned preconditioner on the 5th-generation
// tensor cores (tcgen05.mma, BF16 operands, FP32 accumulators in tensor memory).
//
// Activation layout ("8-channel planes"): a tensor of C channels on an n^3 grid is C/8 planes;
// plane p holds channels 8p..8p+7 of every voxel of the zero-padded grid (n+2)^3 as one 16-byte
// row per voxel, x fastest, with slack rows before and after (VoxGrid).  The halo is zero and
// never written, so a convolution reads zeros outside the grid without a test.
//
// Implicit GEMM: a tile is 128 consecutive rows of the padded grid (M = 128, some rows are halo
// and their outputs are dropped); the 27 taps are the same rows shifted by dz (n+2)^2 + dy (n+2)
// + dx.  Each CTA copies, per tile, three spans of rows (one per dz) into shared memory; the A
// operand of tap (dz, dy, dx) is then the span of dz started dy (n+2) + dx rows later, i.e. a
// shared-memory descriptor with a shifted start address.  With 16-byte rows the span is in the
// canonical no-swizzle K-major layout of the tensor cores: core matrices of 8 rows x 16 bytes
// (stride-dimension offset 128 B), the two 8-channel halves of a 16-channel K step one plane
// apart (leading-dimension offset = span bytes).  The weights of the layer stay in shared memory
// for the whole kernel in the same layout (B operand, N = C_out rows).  One thread issues the
// 27 * C_in/16 MMAs of a tile (K = 16 each) into a tensor-memory accumulator of 128 lanes x C_out
// FP32 columns; tcgen05.commit signals an mbarrier; the four warps read their 32 lanes back with
// tcgen05.ld and apply bias / ReLU / the BF16 conversion.
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace numa::gpu {

// Geometry of an n^3 grid in the 8-channel plane layout.
struct VoxGrid {
    int n;      // interior points per dimension
    int np;     // n + 2
    int pp;     // (n + 2)^2
    int front;  // slack rows before the padded grid in each plane
    int rows;   // rows per plane: front + (n+2)^3 + back
    int span;   // rows of one shared-memory span: 128 + 2 (n + 2) + 2, rounded up to 8
    int tiles;  // tiles of 128 rows covering the planes z = 1..n of the padded grid
};

inline VoxGrid make_voxgrid(int n) {
    VoxGrid g;
    g.n = n;
    g.np = n + 2;
    g.pp = g.np * g.np;
    g.front = ((g.np + 2 + 63) / 64) * 64;
    g.rows = g.front + g.np * g.pp + 256 + g.np + 64;
    g.span = ((128 + 2 * g.np + 2 + 7) / 8) * 8;
    g.tiles = (n * g.pp + 127) / 128;
    return g;
}

// ------------------------------------------------------------------------------ PTX wrappers
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor (tcgen05), no swizzle: start address, leading-dimension byte
// offset (between the core matrices along K), stride-dimension byte offset (between 8-row groups),
// descriptor version 1.
__device__ __forceinline__ uint64_t umma_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// The same with A and B both MN-major (the "transpose A / transpose B" bits 15 and 16): A is M x K
// stored with M contiguous, B is K x N stored with N contiguous.
__host__ __device__ constexpr uint32_t umma_idesc_bf16_mn(int M, int N) {
    return umma_idesc_bf16(M, N) | (1u << 15) | (1u << 16);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

// Waits for the phase of the given parity to complete; gives up after `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int limit) {
    for (int i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Bulk copy by the tensor memory accelerator (non-tensor form): `bytes` (a multiple of 16) from
// global src to shared dst (both 16-byte aligned), counted as transaction bytes on mbarrier bar.
__device__ __forceinline__ void tma_bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
// One arrival on bar that also expects `bytes` of transactions before the phase can complete.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Warp-wide: allocate / free `ncols` tensor-memory columns (power of two >= 32); the address goes
// to *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive FP32 columns of this thread's tensor-memory lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// Shared memory of k_conv3d_tc: resident weights, then two buffers of the three spans.
template <int CIN, int COUT>
__host__ __device__ constexpr size_t conv_weight_bytes() {
    return (size_t)27 * (CIN / 16) * 2 * COUT * 16;
}
// Weights plus `stages` span buffers (three at the largest supported shape: 207 KB): the TMA fills
// the buffers of the next tiles while the MMAs of this tile read one.
template <int CIN, int COUT>
inline size_t conv_smem_bytes(const VoxGrid& g, int stages) {
    return conv_weight_bytes<CIN, COUT>() + (size_t)stages * 3 * (CIN / 8) * g.span * 16;
}

constexpr int kConvWaitLimit = 1 << 22;

// 8 consecutive FP32 columns of this thread's tensor-memory lane.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// One arrival on bar.
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

constexpr int kConvEpiWarps = 8;                          // warps that drain the accumulators
constexpr int kConvThreads = 32 * (kConvEpiWarps + 1);    // and one that feeds the TMA and the tensor cores

// out = act(conv(in) + bias) on the 8-channel plane layout, or (OUT32) FP32 channel-last output of
// the interior voxels [((z-1) n + y-1) n + x-1][C_out] without activation.
//   wg: the layer's BF16 weights in the B-operand layout [tap][k16 chunk][half][C_out][8].
//   err: set to 1 when an mbarrier wait gives up (no tile after that is computed).
// A persistent CTA walks its tiles (128 padded rows each) with its warps specialised and coupled
// only through mbarriers:
//  * warp 8, one thread: the TMA copies of each tile's spans into one of NST buffers (lbar), issued
//    NST - 1 tiles ahead, and the
//    27 x C_in/16 MMAs of each tile into one of two accumulators in tensor memory, committed to
//    full[b]; an accumulator is reused once the epilogue warps released it (empty[b]), a span buffer
//    once the MMAs that read it completed (full[b]);
//  * warps 0-7: for each tile, wait for its accumulator, read their lanes (warp w: tensor-memory lanes
//    32 (w mod 4) .. + 31, the columns of half w / 4) into registers, release the accumulator, then
//    add the bias and store.
// So the copies of tile t + 1, the MMAs of tile t and the stores of tile t - 1 overlap.  Every wait is
// bounded; the thread that gives up sets err and waits (bounded) for its copies and MMAs in flight
// before the shared and tensor memory are freed.
template <int CIN, int COUT, bool OUT32, int NST>
__global__ void __launch_bounds__(kConvThreads, 1) k_conv3d_tc(const uint4* __restrict__ in, const uint4* __restrict__ wg,
                                                            const float* __restrict__ bias, uint4* __restrict__ out,
                                                            float* __restrict__ out32, VoxGrid g, int relu,
                                                            unsigned* __restrict__ err) {
    static_assert(CIN % 16 == 0 && COUT % 16 == 0 && COUT >= 16 && COUT <= 32, "channel counts");
    constexpr int KC = CIN / 16, PL = CIN / 8;
    constexpr int HALF = COUT / 2;                           // accumulator columns an epilogue warp takes
    constexpr int NACC = 2;                                  // accumulators of COUT columns in tensor memory
    constexpr uint32_t kCols = NACC * COUT <= 32 ? 32 : (NACC * COUT <= 64 ? 64 : 128);
    extern __shared__ __align__(128) unsigned char conv_smem[];
    __shared__ __align__(8) uint64_t lbar[NST];    // span copies into buffer 0 .. NST - 1 complete
    __shared__ __align__(8) uint64_t full[NACC];   // MMAs into accumulator a complete
    __shared__ __align__(8) uint64_t empty[NACC];  // accumulator a read out by the epilogue warps
    __shared__ uint32_t tmem_slot;
    uint4* w_s = reinterpret_cast<uint4*>(conv_smem);
    uint4* a_s = reinterpret_cast<uint4*>(conv_smem + conv_weight_bytes<CIN, COUT>());
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int bufsz = 3 * PL * g.span;  // uint4 per span buffer
    const int ntile = (int)blockIdx.x < g.tiles ? (g.tiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x : 0;

    for (int e = tid; e < (int)(conv_weight_bytes<CIN, COUT>() / 16); e += kConvThreads) w_s[e] = wg[e];
    if (warp == 0) tmem_alloc(&tmem_slot, kCols);
    if (tid == 0) {
        for (int q = 0; q < NST; ++q) mbar_init(smem_addr(&lbar[q]), 1);
        for (int q = 0; q < NACC; ++q) {
            mbar_init(smem_addr(&full[q]), 1);
            mbar_init(smem_addr(&empty[q]), kConvEpiWarps);
        }
    }
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    if (warp == kConvEpiWarps) {
        if (lane == 0) {
            constexpr uint32_t idesc = umma_idesc_bf16(128, COUT);
            // the 3 * PL spans of tile number k (of this CTA) into buffer k mod NST, one bulk copy each
            auto issue = [&](int k) {
                const int b = k % NST;
                const uint32_t lb = smem_addr(&lbar[b]);
                mbar_arrive_expect_tx(lb, (uint32_t)bufsz * 16u);
                const int start = g.pp + 128 * ((int)blockIdx.x + k * (int)gridDim.x);  // padded row of tile row 0
                for (int dz = 0; dz < 3; ++dz)
                    for (int p = 0; p < PL; ++p) {
                        const int q0 = start + (dz - 1) * g.pp - g.np - 1;
                        tma_bulk_g2s(smem_addr(a_s + (size_t)b * bufsz + (size_t)(dz * PL + p) * g.span),
                                     in + (size_t)p * g.rows + g.front + q0, (uint32_t)g.span * 16u, lb);
                    }
            };
            int issued = 0, landed = 0, mmas = 0;  // tiles copied, waited for, given to the tensor cores
            bool ok = true;
            while (issued < ntile && issued < NST) issue(issued++);
            for (int it = 0; it < ntile; ++it) {
                const int b = it % NACC, sb = it % NST;  // accumulator, span buffer
                if (!mbar_wait(smem_addr(&lbar[sb]), (uint32_t)((it / NST) & 1), kConvWaitLimit)) {
                    ok = false;
                    break;
                }
                ++landed;
                if (it >= NACC && !mbar_wait(smem_addr(&empty[b]), (uint32_t)(((it - NACC) / NACC) & 1), kConvWaitLimit)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                // the descriptors of tap (dz, dy, dx), chunk kc are the buffer's and the weights' plus
                // an offset in 16-byte units in the start-address field (shared addresses stay below
                // 2^18, so the field does not carry)
                const uint64_t ad0 = umma_sdesc(smem_addr(a_s + (size_t)sb * bufsz), (uint32_t)g.span * 16, 128);
                const uint64_t bd0 = umma_sdesc(smem_addr(w_s), COUT * 16, 128);
                const uint32_t td = tmem + (uint32_t)(b * COUT);
                uint32_t acc = 0;
#pragma unroll 1
                for (int dz = 0; dz < 3; ++dz) {
#pragma unroll
                    for (int dy = 0; dy < 3; ++dy)
#pragma unroll
                        for (int dx = 0; dx < 3; ++dx)
#pragma unroll
                            for (int kc = 0; kc < KC; ++kc) {
                                const uint32_t ao = (uint32_t)((dz * PL + 2 * kc) * g.span + dy * g.np + dx);
                                const uint32_t bo = (uint32_t)(((dz * 9 + dy * 3 + dx) * KC + kc) * 2 * COUT);
                                umma_bf16(td, ad0 + ao, bd0 + bo, idesc, acc);
                                acc = 1;
                            }
                }
                umma_commit(smem_addr(&full[b]));
                ++mmas;
                if (it >= 1 && issued < ntile) {
                    // the previous tile's span buffer is free once its MMAs are done; tile it + NST - 1
                    // goes there
                    if (!mbar_wait(smem_addr(&full[(it - 1) % NACC]), (uint32_t)(((it - 1) / NACC) & 1), kConvWaitLimit)) {
                        ok = false;
                        break;
                    }
                    issue(issued++);
                }
            }
            if (!ok) {
                atomicOr(err, 1u);
                // copies and MMAs in flight finish (bounded) before the shared and tensor memory go
                for (int k = landed; k < issued; ++k)
                    mbar_wait(smem_addr(&lbar[k % NST]), (uint32_t)((k / NST) & 1), kConvWaitLimit);
                if (mmas > 0)
                    mbar_wait(smem_addr(&full[(mmas - 1) % NACC]), (uint32_t)(((mmas - 1) / NACC) & 1), kConvWaitLimit);
            }
        }
        __syncwarp();
    } else {
        const int quarter = warp & 3, half = warp >> 2;
        float bv[HALF];
#pragma unroll
        for (int i = 0; i < HALF; ++i) bv[i] = bias ? bias[half * HALF + i] : 0.0f;
        for (int it = 0; it < ntile; ++it) {
            const int b = it % NACC;
            // every lane waits (bounded); the warp goes on or gives up as one, converged for the
            // warp-wide tensor-memory load
            const int seen = mbar_wait(smem_addr(&full[b]), (uint32_t)((it / NACC) & 1), kConvWaitLimit) ? 1 : 0;
            if (!__all_sync(0xffffffffu, seen)) {
                if (lane == 0) atomicOr(err, 1u);
                break;
            }
            tc_fence_after();
            float v[HALF];
            const uint32_t ta = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(b * COUT + half * HALF);
            if constexpr (HALF == 16) {
                tmem_ld16(ta, v);
            } else {
                tmem_ld8(ta, v);
            }
            tc_fence_before();
            if (lane == 0) mbar_arrive(smem_addr(&empty[b]));
            const int q = g.pp + 128 * ((int)blockIdx.x + it * (int)gridDim.x) + 32 * quarter + lane;
            const int x = q % g.np, y = (q / g.np) % g.np, z = q / g.pp;
            if (x < 1 || x > g.n || y < 1 || y > g.n || z < 1 || z > g.n) continue;
            if (OUT32) {
                float4* o = reinterpret_cast<float4*>(out32 + ((size_t)((z - 1) * g.n + (y - 1)) * g.n + (x - 1)) * COUT +
                                                      half * HALF);
#pragma unroll
                for (int c = 0; c < HALF; c += 4)
                    o[c / 4] = make_float4(v[c] + bv[c], v[c + 1] + bv[c + 1], v[c + 2] + bv[c + 2], v[c + 3] + bv[c + 3]);
            } else {
#pragma unroll
                for (int c8 = 0; c8 < HALF / 8; ++c8) {
                    float w8[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const float s = v[8 * c8 + i] + bv[8 * c8 + i];
                        w8[i] = (relu && s < 0.0f) ? 0.0f : s;
                    }
                    uint4 pk;
                    pk.x = pack_bf16x2(w8[0], w8[1]);
                    pk.y = pack_bf16x2(w8[2], w8[3]);
                    pk.z = pack_bf16x2(w8[4], w8[5]);
                    pk.w = pack_bf16x2(w8[6], w8[7]);
                    out[(size_t)(half * HALF / 8 + c8) * g.rows + g.front + q] = pk;
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_free(tmem, kCols);
}

// ------------------------------------------------------------------------------ weight gradient
// dW[tap][ci][co] = sum over the voxels v of x[v + tap][ci] dy[v][co] (the gradient of a layer's
// weights), as implicit GEMMs on the tensor cores: K runs over voxel rows, and each operand is taken
// MN-major straight from the plane layout, where a voxel row holds 8 channels in 16 bytes and 8
// consecutive rows of one plane form a 128-byte core matrix (8 K rows x 8 channels).
//  * A (M x K): the input's spans of a tile, as the forward kernel copies them (one span of
//    g.span rows per dz and 8-channel plane, spans back to back).  The span of (dz, plane p) is
//    8-channel group dz * PL + p, so the three dz taps of one (dy, dx) stack along M with a
//    uniform group stride (the span bytes, SBO); the (dy, dx) shift is the descriptor's start
//    address, dy (n+2) + dx rows into the spans.  M = 128 rows: 3 * C_in real ones (48 or 96),
//    the rest read the following spans and their sums are never read.
//  * B (K x N): the output gradient's tile of 128 rows, one 2 KB block per 8-channel plane (SBO).
//  * D: one block of C_out FP32 columns per (dy, dx), 9 blocks, accumulated over every tile the
//    CTA takes; the halo rows of dy are zero, so tile rows outside the grid add nothing.
// Double-buffered: the copies of the next tile go in while the MMAs of this tile run, and a
// buffer is refilled only after the MMAs that read it have completed (commit on an mbarrier).
// Each CTA writes its partial dW to part[blockIdx.x]; k_dw_reduce adds the partials in CTA order.
template <int CIN, int COUT>
struct DwShape {
    static constexpr int PL = CIN / 8, QL = COUT / 8;
    static constexpr int GROUPS = 16;                              // M = 128 rows
    static constexpr int EXTRA = GROUPS - 3 * PL;                  // spans past the second buffer
    static constexpr uint32_t COLS = 9 * COUT <= 256 ? 256 : 512;  // tensor-memory columns
};
template <int CIN, int COUT>
inline size_t dw_smem_bytes(const VoxGrid& g) {
    using S = DwShape<CIN, COUT>;
    return (size_t)(2 * 3 * S::PL + S::EXTRA) * g.span * 16 + (size_t)2 * S::QL * 128 * 16;
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(128) k_conv_dw_tc(const uint4* __restrict__ x, const uint4* __restrict__ dy,
                                                    VoxGrid g, float* __restrict__ part, unsigned* __restrict__ err) {
    using S = DwShape<CIN, COUT>;
    constexpr int PL = S::PL, QL = S::QL;
    extern __shared__ __align__(128) unsigned char dw_smem[];
    __shared__ __align__(8) uint64_t mbar[2];  // MMAs of the tile in buffer 0 / 1
    __shared__ __align__(8) uint64_t lbar[2];  // copies into buffer 0 / 1
    __shared__ uint32_t tmem_slot;
    uint4* a_s = reinterpret_cast<uint4*>(dw_smem);
    uint4* b_s = a_s + (size_t)(2 * 3 * PL + S::EXTRA) * g.span;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int abuf = 3 * PL * g.span;  // uint4 per A buffer
    const int bbuf = QL * 128;         // uint4 per B buffer

    // the spans past the second buffer are read by the unused rows of M: keep them finite
    for (int e = tid; e < S::EXTRA * g.span; e += 128) a_s[(size_t)2 * abuf + e] = make_uint4(0u, 0u, 0u, 0u);
    if (warp == 0) tmem_alloc(&tmem_slot, S::COLS);
    if (tid == 0) {
        mbar_init(smem_addr(&mbar[0]), 1);
        mbar_init(smem_addr(&mbar[1]), 1);
        mbar_init(smem_addr(&lbar[0]), 1);
        mbar_init(smem_addr(&lbar[1]), 1);
    }
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    constexpr uint32_t idesc = umma_idesc_bf16_mn(128, COUT);

    auto issue = [&](int t, int b) {
        const uint32_t lb = smem_addr(&lbar[b]);
        mbar_arrive_expect_tx(lb, (uint32_t)(abuf + bbuf) * 16u);
        const int start = g.pp + 128 * t;
        for (int dz = 0; dz < 3; ++dz)
            for (int p = 0; p < PL; ++p) {
                const int q0 = start + (dz - 1) * g.pp - g.np - 1;
                tma_bulk_g2s(smem_addr(a_s + (size_t)b * abuf + (size_t)(dz * PL + p) * g.span),
                             x + (size_t)p * g.rows + g.front + q0, (uint32_t)g.span * 16u, lb);
            }
        for (int p = 0; p < QL; ++p)
            tma_bulk_g2s(smem_addr(b_s + (size_t)b * bbuf + (size_t)p * 128), dy + (size_t)p * g.rows + g.front + start,
                         128u * 16u, lb);
    };
    bool ok = true;
    int it = 0;
    int pend[2] = {-1, -1};  // iteration whose MMAs last read buffer 0 / 1 (not yet waited for)
    if (tid == 0 && (int)blockIdx.x < g.tiles) issue(blockIdx.x, 0);
    for (int t = blockIdx.x; t < g.tiles; t += gridDim.x, ++it) {
        const int b = it & 1;
        const int tn = t + (int)gridDim.x;
        if (tn < g.tiles) {
            // the other buffer is refilled once the MMAs that read it (iteration it - 1) are done
            int free_ok = 1;
            if (pend[b ^ 1] >= 0) {
                free_ok = mbar_wait(smem_addr(&mbar[b ^ 1]), (uint32_t)((pend[b ^ 1] >> 1) & 1), kConvWaitLimit) ? 1 : 0;
                pend[b ^ 1] = -1;
            }
            if (!__syncthreads_and(free_ok)) {
                ok = false;
                break;
            }
            if (tid == 0) issue(tn, b ^ 1);
        }
        const int landed = mbar_wait(smem_addr(&lbar[b]), (uint32_t)((it >> 1) & 1), kConvWaitLimit) ? 1 : 0;
        if (!__syncthreads_and(landed)) {
            ok = false;
            break;
        }
        if (tid == 0) {
            tc_fence_after();
            const uint32_t a0 = smem_addr(a_s + (size_t)b * abuf), b0 = smem_addr(b_s + (size_t)b * bbuf);
#pragma unroll 1
            for (int pr = 0; pr < 9; ++pr) {
                const int ddy = pr / 3, ddx = pr % 3;
#pragma unroll
                for (int kk = 0; kk < 8; ++kk) {
                    const uint32_t aa = a0 + (uint32_t)((ddy * g.np + ddx + 16 * kk) * 16);
                    const uint32_t bb = b0 + (uint32_t)(16 * kk * 16);
                    umma_bf16(tmem + (uint32_t)(pr * COUT), umma_sdesc(aa, 128, (uint32_t)g.span * 16),
                              umma_sdesc(bb, 128, 128 * 16), idesc, (it > 0 || kk > 0) ? 1u : 0u);
                }
            }
            umma_commit(smem_addr(&mbar[b]));
        }
        pend[b] = it;
    }
    // the last MMAs (bounded waits; a block that gave up reports it and writes nothing)
    int done = ok ? 1 : 0;
    for (int q = 0; q < 2; ++q)
        if (pend[q] >= 0) {
            if (!mbar_wait(smem_addr(&mbar[q]), (uint32_t)((pend[q] >> 1) & 1), kConvWaitLimit)) done = 0;
            pend[q] = -1;
        }
    done = __syncthreads_and(done);
    if (!done) {
        if (tid == 0) {
            atomicOr(err, 1u);
            // copies still in flight into either buffer finish before the shared memory is released
            mbar_wait(smem_addr(&lbar[it & 1]), (uint32_t)((it >> 1) & 1), kConvWaitLimit);
            mbar_wait(smem_addr(&lbar[(it + 1) & 1]), (uint32_t)(((it + 1) >> 1) & 1), kConvWaitLimit);
        }
    } else if (it > 0) {
        tc_fence_after();
        const int m = 32 * warp + lane;  // row of D = this thread's tensor-memory lane
        const bool real = m < 3 * CIN;
        const int dz = m / CIN, ci = m % CIN;
        float* pb = part + (size_t)blockIdx.x * 27 * CIN * COUT;
#pragma unroll 1
        for (int pr = 0; pr < 9; ++pr) {
#pragma unroll
            for (int c = 0; c < COUT; c += 16) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(pr * COUT + c), v);
                if (real) {
                    float* o = pb + ((size_t)(dz * 9 + pr) * CIN + ci) * COUT + c;
#pragma unroll
                    for (int i = 0; i < 16; ++i) o[i] = v[i];
                }
            }
        }
    } else {
        // no tile: a zero partial
        float* pb = part + (size_t)blockIdx.x * 27 * CIN * COUT;
        for (int e = tid; e < 27 * CIN * COUT; e += 128) pb[e] = 0.0f;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_free(tmem, S::COLS);
}

}  // namespace numa::gpu
