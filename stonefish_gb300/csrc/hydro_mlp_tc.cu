// hydro_mlp_tc.cu -- fused inference of the wrench surrogate on the 5th-
// generation tensor cores: a CTA takes blocks of 128 states through all four
// layers (16 -> 256 -> 256 -> 256 -> 16) with the activations kept in shared
// memory and the accumulators in tensor memory.
//
//   * persistent: one CTA per SM loops over the blocks; the next block's
//     features are loaded into registers while the current block runs, and
//     its first-layer weights are copied while the last layer runs;
//   * operands are K-major BF16 in the 128-byte-swizzled canonical layout
//     (8-row x 128-byte atoms, 16-byte chunk c of row r stored at chunk
//     c ^ (r % 8)); each [rows x 64] K-block is contiguous, blocks follow
//     each other;
//   * the weights are packed once into that image in global memory
//     (pack_sw128_kernel), so each layer's weights arrive with one 1-D bulk
//     copy (cp.async.bulk, mbarrier complete_tx) while the previous layer's
//     epilogue runs;
//   * one lane of a dedicated warp issues tcgen05.mma (M = 128, N = 256 or
//     16, K = 16 per instruction, FP32 accumulate) and commits to an
//     mbarrier; the accumulators of consecutive layers alternate between
//     the two halves of 512 TMEM columns;
//   * sixteen epilogue warps read a layer's accumulator with tcgen05.ld
//     (warp w reads TMEM lanes 32 (w % 4) .. +31), one 64-column K-block
//     at a time, add the bias, apply SiLU, round to BF16 and write that
//     K-block of the next layer's A operand, then arrive on the K-block's
//     mbarrier: the next layer's MMAs on K-block g start while the
//     epilogue works on K-blocks g + 1 ..;
//   * the next layer's weights stream in as four K-block copies, each on
//     its own mbarrier, as soon as the current layer's MMAs have retired;
//   * the input features are normalised and rounded in the kernel, the
//     output (bias added) is written as FP32 rows of 16.
//
// Every mbarrier wait is bounded (%globaltimer); a timeout sets *err, the
// CTA stops issuing work, waits (bounded) for its tensor-core work to
// retire, frees its tensor memory and returns.
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "hydro_internal.h"

namespace sfh {

typedef __nv_bfloat16 bf16;

namespace tc {

constexpr int kRows = 128;      // states per CTA = UMMA M
constexpr int kHid = 256;
constexpr int kIn = 16;         // features = layer-0 K
constexpr int kOut = 16;        // output columns (6 used)
constexpr int kEpiWarps = 16;                   // epilogue warps
constexpr int kThreads = (kEpiWarps + 1) * 32;  // + one MMA warp
constexpr uint32_t kTmemCols = 512;             // two 256-column accumulators

// shared-memory image (offsets from a 1024-byte-aligned base)
constexpr uint32_t kOffA = 0;                        // 128 x 256 bf16, 4 K-blocks of 16 KB
constexpr uint32_t kOffW = kOffA + 4 * 16384;        // 256 x 256 bf16, 4 K-blocks of 32 KB
constexpr uint32_t kOffW3 = kOffW + 4 * 32768;       // 16 x 256 bf16, 4 K-blocks of 2 KB
constexpr uint32_t kOffBias = kOffW3 + 4 * 2048;     // 3 x 256 + 16 floats
constexpr uint32_t kOffBar = kOffBias + (3 * kHid + kOut) * 4;   // 11 mbarriers
constexpr uint32_t kOffTmem = kOffBar + 12 * 8;
constexpr uint32_t kSmemBytes = kOffTmem + 16 + 1024; // + alignment slack

// global weight image (bytes)
constexpr uint32_t kImgW0 = 0;                       // 256 x 64 (K 16 used) = 32 KB
constexpr uint32_t kImgW1 = kImgW0 + 32768;
constexpr uint32_t kImgW2 = kImgW1 + 131072;
constexpr uint32_t kImgW3 = kImgW2 + 131072;         // 16 x 256 = 8 KB
constexpr uint32_t kImgBytes = kImgW3 + 8192;

__device__ __forceinline__ uint32_t sw128_offset(uint32_t rows, uint32_t r, uint32_t k)
{
    // byte offset of element (r, k) of a [rows x K] bf16 operand
    const uint32_t blk = k >> 6, kk = k & 63;
    return blk * rows * 128u + r * 128u + ((((kk >> 3) ^ (r & 7u)) & 7u) << 4) + ((kk & 7u) << 1);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// tcgen05 shared-memory matrix descriptor: K-major, 128-byte swizzle,
// 8-row groups 1024 bytes apart (SBO), descriptor version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr)
{
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1u << 16;                 // leading byte offset (unused by swizzled K-major)
    d |= (uint64_t)(1024u >> 4) << 32;       // stride byte offset
    d |= (uint64_t)1u << 46;                 // version
    d |= (uint64_t)2u << 61;                 // SWIZZLE_128B
    return d;
}

// instruction descriptor, kind::f16: BF16 A and B, FP32 D, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t M, uint32_t N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ uint64_t globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
    return ok != 0;
}

// bounded wait: gives up after limit_ns
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint64_t limit_ns)
{
    if (mbar_try(bar, parity)) return true;
    const uint64_t t0 = globaltimer();
    while (!mbar_try(bar, parity)) {
        if (globaltimer() - t0 > limit_ns) return false;
        __nanosleep(64);
    }
    return true;
}

__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
}

__device__ __forceinline__ void expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                 :: "r"(tmem_d), "l"(a), "l"(b), "r"(idesc), "r"(acc) : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :: "r"(bar) : "memory");
}

__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                   "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                   "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
                   "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
                   "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Split form of tmem_ld16 for software pipelining: the load is issued
// without waiting, and the wait names the destination registers as in-out
// operands so that no use of them can be scheduled before it.
__device__ __forceinline__ void tmem_ld16_issue(uint32_t taddr, uint32_t (&r)[16])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                   "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld_wait(uint32_t (&r)[16])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]),
                   "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]),
                   "+r"(r[14]), "+r"(r[15])
                 :: "memory");
}

__device__ __forceinline__ uint32_t pack2(float a, float b)
{
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(bar) : "memory");
}

// A hidden layer's epilogue, one K-block (64 columns) at a time: D (TMEM)
// + bias -> SiLU -> BF16 -> columns 64 g .. of the A operand (row = TMEM
// lane), then an arrival on K-block g's mbarrier so that the next layer's
// MMAs on it can start.  Warp w: lanes 32 (w % 4).., columns
// 64 g + 16 (w / 4) ..; the tensor-memory load of K-block g + 1 is in
// flight while K-block g is converted.
__device__ __forceinline__ void hidden_epilogue(uint32_t acc, unsigned char* base, const float* bias, uint32_t abar)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t q = (uint32_t)(warp & 3), sub = (uint32_t)(warp >> 2);
    const uint32_t row = 32u * q + (uint32_t)lane;
    const uint32_t lanes = (32u * q) << 16;
    uint32_t cur[16], nxt[16];
    tmem_ld16_issue(acc + lanes + 16u * sub, cur);
    tmem_ld_wait(cur);
#pragma unroll
    for (uint32_t g = 0; g < 4; ++g) {
        const uint32_t col = 64u * g + 16u * sub;
        if (g < 3) tmem_ld16_issue(acc + lanes + col + 64u, nxt);
        uint32_t w[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            // bias, then SiLU(z) = z sigmoid(z) = h + h tanh(h) with h = z / 2,
            // on two columns at a time with the packed FP32 instructions (each
            // half rounds as the scalar operation would): one hardware tanh
            // (tanh.approx.f32, relative error about 2^-11) per value, so the
            // absolute error is at most |z| 2^-12, below the BF16 rounding of
            // the activation that follows
            const float2 b2 = *reinterpret_cast<const float2*>(bias + col + 2 * i);
            const float2 z2 = __fadd2_rn(make_float2(__uint_as_float(cur[2 * i]), __uint_as_float(cur[2 * i + 1])), b2);
            const float2 h2 = __fmul2_rn(z2, make_float2(0.5f, 0.5f));
            float t0, t1;
            asm("tanh.approx.f32 %0, %1;" : "=f"(t0) : "f"(h2.x));
            asm("tanh.approx.f32 %0, %1;" : "=f"(t1) : "f"(h2.y));
            const float2 s2 = __ffma2_rn(h2, make_float2(t0, t1), h2);
            w[i] = pack2(s2.x, s2.y);
        }
#pragma unroll
        for (int c = 0; c < 2; ++c)
            *reinterpret_cast<uint4*>(base + kOffA + sw128_offset(kRows, row, col + 8u * c)) =
                make_uint4(w[4 * c], w[4 * c + 1], w[4 * c + 2], w[4 * c + 3]);
        fence_async_smem();
        mbar_arrive(abar + 8u * g);
        if (g < 3) {
            tmem_ld_wait(nxt);
#pragma unroll
            for (int i = 0; i < 16; ++i) cur[i] = nxt[i];
        }
    }
    fence_before();
}

}  // namespace tc

// Normalised BF16 inputs of one 128-state block: thread t < 256 holds row
// t % 128, features 8 (t / 128) .. + 7.
__device__ __forceinline__ void load_features(const float* __restrict__ feats, uint32_t n, uint32_t row0,
                                              const float* __restrict__ fmean, const float* __restrict__ fistd,
                                              float (&x)[8])
{
    using namespace tc;
    const uint32_t r = threadIdx.x & (kRows - 1), h = threadIdx.x >> 7;
    const uint32_t gr = row0 + r;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int k = (int)h * 8 + j;
        x[j] = gr < n ? (feats[(size_t)gr * kIn + k] - fmean[k]) * fistd[k] : 0.f;
    }
}

__device__ __forceinline__ void store_features(unsigned char* base, const float (&x)[8])
{
    using namespace tc;
    const uint32_t r = threadIdx.x & (kRows - 1), h = threadIdx.x >> 7;
    *reinterpret_cast<uint4*>(base + kOffA + sw128_offset(kRows, r, h * 8)) =
        make_uint4(pack2(x[0], x[1]), pack2(x[2], x[3]), pack2(x[4], x[5]), pack2(x[6], x[7]));
}

// Persistent: CTA c takes the 128-state blocks c, c + gridDim.x, ...; the
// tensor memory, the mbarriers, the biases and the last layer's weights are
// set up once.  While a block runs, the epilogue threads hold the next
// block's features in registers and write them once the block's last MMAs
// have retired; the next block's first-layer weights are copied as soon as
// the weight buffer is free.
__global__ void __launch_bounds__(tc::kThreads, 1)
mlp_tc_kernel(const float* __restrict__ feats, uint32_t n, const float* __restrict__ fmean,
              const float* __restrict__ fistd, const unsigned char* __restrict__ wimg,
              const float* __restrict__ b0, const float* __restrict__ b1, const float* __restrict__ b2,
              const float* __restrict__ b3, float* __restrict__ out, unsigned* __restrict__ err)
{
    using namespace tc;
    extern __shared__ unsigned char smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    unsigned char* base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    const uint32_t sb = smem_u32(base);
    // mbarriers: first-layer weights; MMA commits; the four K-block copies of
    // a hidden layer's weights; the four K-blocks of A; a block's features
    const uint32_t barW0 = sb + kOffBar, barM = barW0 + 8, wbar = barW0 + 16, abar = barW0 + 48,
                   barF = barW0 + 80;
    float* bias = reinterpret_cast<float*>(base + kOffBias);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(base + kOffTmem);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t n_blocks = (n + kRows - 1) / kRows;
    const uint64_t kLimit = 1000000000ull;   // 1 s per wait

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(tmem_slot)), "r"(kTmemCols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(barW0) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(barM) : "memory");
        for (uint32_t g = 0; g < 4; ++g) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(wbar + 8u * g) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(abar + 8u * g), "r"(kEpiWarps * 32)
                         : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(barF), "r"(kEpiWarps * 32) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;

    // the first block's first-layer weights and the last layer's (which stay)
    if (tid == 0) {
        expect_tx(barW0, 32768u + 8192u);
        bulk_load(sb + kOffW, wimg + kImgW0, 32768u, barW0);
        bulk_load(sb + kOffW3, wimg + kImgW3, 8192u, barW0);
    }
    for (int i = tid; i < kHid; i += kThreads) {
        bias[i] = b0[i];
        bias[kHid + i] = b1[i];
        bias[2 * kHid + i] = b2[i];
    }
    if (tid < kOut) bias[3 * kHid + tid] = b3[tid];
    float x[8];
    if (tid < kRows * (kIn / 8)) {
        load_features(feats, n, blockIdx.x * (uint32_t)kRows, fmean, fistd, x);
        store_features(base, x);
    }
    fence_async_smem();
    __syncthreads();

    bool ok = true;
    if (warp == kEpiWarps) {
        // ---- MMA warp: one lane issues every layer's MMAs and the weight copies
        if (lane == 0) {
            const uint32_t id_hid = idesc_bf16(128, 256), id_out = idesc_bf16(128, kOut);
            uint32_t w_pending = 0, w_par = 0;    // K-block copies issued and not yet waited for; their parity
            uint32_t w0_pending = 1, w0_par = 0;  // first-layer copy issued and not yet waited for; its parity
            uint32_t commits = 0, seen = 0;   // barM phases committed / observed complete
            uint32_t a_done = 0;              // completions of the A K-block barriers waited for
            uint32_t k = 0;
#pragma unroll 1
            for (uint32_t blk = blockIdx.x; blk < n_blocks && ok; blk += gridDim.x, ++k) {
                ok = mbar_wait(barW0, k & 1u, kLimit);
                if (ok) w0_pending = 0;
                // this block's features: written once the epilogue has seen
                // the previous block's last commit
                if (ok && k > 0) {
                    ok = mbar_wait(barF, (k - 1u) & 1u, kLimit);
                    if (ok) ++seen;
                }
                if (!ok) break;
                fence_after();
                mma(tmem, sw128_desc(sb + kOffA), sw128_desc(sb + kOffW), id_hid, 0u);   // layer 0: K = 16
                mma_commit(barM);
                ++commits;
#pragma unroll 1
                for (uint32_t l = 1; l <= 3 && ok; ++l) {
                    // layer l - 1's MMAs have retired: the weight buffer takes
                    // layer l's weights (or, before the last layer, the next
                    // block's first-layer weights)
                    ok = mbar_wait(barM, (l - 1u) & 1u, kLimit);
                    if (!ok) break;
                    ++seen;
                    if (l < 3) {
                        for (uint32_t g = 0; g < 4; ++g) {
                            expect_tx(wbar + 8u * g, 32768u);
                            bulk_load(sb + kOffW + 32768u * g, wimg + (l == 1 ? kImgW1 : kImgW2) + 32768u * g,
                                      32768u, wbar + 8u * g);
                        }
                        w_pending = 0xFu;
                        w_par = (l - 1u) & 1u;
                    } else if (blk + gridDim.x < n_blocks) {
                        expect_tx(barW0, 32768u);
                        bulk_load(sb + kOffW, wimg + kImgW0, 32768u, barW0);
                        w0_pending = 1;
                        w0_par = (k + 1u) & 1u;
                    }
                    const uint32_t acc = tmem + 256u * (l & 1u);
#pragma unroll 1
                    for (uint32_t g = 0; g < 4 && ok; ++g) {
                        if (l < 3) {
                            ok = mbar_wait(wbar + 8u * g, (l - 1u) & 1u, kLimit);
                            if (!ok) break;
                            w_pending &= ~(1u << g);
                        }
                        ok = mbar_wait(abar + 8u * g, a_done & 1u, kLimit);   // K-block g of layer l's input
                        if (!ok) break;
                        fence_after();
#pragma unroll
                        for (uint32_t j = 0; j < 4; ++j) {
                            const uint32_t off_a = kOffA + g * (kRows * 128u) + j * 32u;
                            if (l < 3) {
                                const uint32_t off_b = kOffW + g * (kHid * 128u) + j * 32u;
                                mma(acc, sw128_desc(sb + off_a), sw128_desc(sb + off_b), id_hid, (g | j) ? 1u : 0u);
                            } else {
                                const uint32_t off_b = kOffW3 + g * (kOut * 128u) + j * 32u;
                                mma(acc, sw128_desc(sb + off_a), sw128_desc(sb + off_b), id_out, (g | j) ? 1u : 0u);
                            }
                        }
                    }
                    if (!ok) break;
                    ++a_done;
                    mma_commit(barM);
                    ++commits;
                }
                // the epilogue waits for the last layer's commit; this warp
                // counts it as seen once the next block's features arrive
            }
            if (!ok) {
                // let issued tensor-core work and copies retire before the
                // tensor memory is freed and the CTA exits (bounded): one more
                // commit, then the barrier's phases in order
                atomicOr(err, 1u);
                mma_commit(barM);
                ++commits;
                for (uint32_t c = seen; c < commits; ++c) mbar_wait(barM, c & 1u, kLimit);
                for (uint32_t g = 0; g < 4; ++g)
                    if ((w_pending >> g) & 1u) mbar_wait(wbar + 8u * g, w_par, kLimit);
                if (w0_pending) mbar_wait(barW0, w0_par, kLimit);
            }
        }
        __syncwarp();
        ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
    } else {
        // ---- epilogue warps
#pragma unroll 1
        for (uint32_t blk = blockIdx.x; blk < n_blocks && ok; blk += gridDim.x) {
            const uint32_t next = blk + gridDim.x;
            if (tid < kRows * (kIn / 8)) {
                if (next < n_blocks) load_features(feats, n, next * (uint32_t)kRows, fmean, fistd, x);
            }
            // layers 0..2 feed the next layer K-block by K-block
#pragma unroll 1
            for (uint32_t l = 0; l < 3 && ok; ++l) {
                ok = mbar_wait(barM, l & 1u, kLimit);
                if (!ok) break;
                fence_after();
                hidden_epilogue(tmem + 256u * (l & 1u), base, bias + l * kHid, abar);
            }
            // output layer: N = 16, bias, FP32 rows of 16
            if (ok) ok = mbar_wait(barM, 1u, kLimit);
            if (!ok) break;
            fence_after();
            if (warp < 4) {
                float v[16];
                tmem_ld16(tmem + 256u + ((32u * (uint32_t)warp) << 16), v);
                const uint32_t gr = blk * (uint32_t)kRows + 32u * (uint32_t)warp + (uint32_t)lane;
                if (gr < n) {
                    float4* o = reinterpret_cast<float4*>(out + (size_t)gr * kOut);
                    const float* bb = bias + 3 * kHid;
#pragma unroll
                    for (int i = 0; i < 4; ++i)
                        o[i] = make_float4(v[4 * i] + bb[4 * i], v[4 * i + 1] + bb[4 * i + 1],
                                           v[4 * i + 2] + bb[4 * i + 2], v[4 * i + 3] + bb[4 * i + 3]);
                }
            }
            // the next block's features into A (its last MMAs have retired)
            if (next < n_blocks) {
                if (tid < kRows * (kIn / 8)) store_features(base, x);
                fence_before();
                fence_async_smem();
                mbar_arrive(barF);
            }
        }
        if (!ok && lane == 0) atomicOr(err, 1u);
    }
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(kTmemCols) : "memory");
    }
}

// dst = 128-byte-swizzled K-major image of src[rows][K] (row stride ld),
// K padded with zeros to kpad (a multiple of 64); one thread per 16 bytes.
__global__ void pack_sw128_kernel(const bf16* __restrict__ src, int rows, int K, int ld, int kpad,
                                  unsigned char* __restrict__ dst)
{
    const uint32_t chunks = (uint32_t)rows * (uint32_t)(kpad / 8);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= chunks) return;
    const uint32_t r = i / (uint32_t)(kpad / 8), k0 = (i % (uint32_t)(kpad / 8)) * 8u;
    uint16_t v[8];
    const uint16_t* s = reinterpret_cast<const uint16_t*>(src);
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = (k0 + j < (uint32_t)K) ? s[(size_t)r * ld + k0 + j] : (uint16_t)0;
    uint4 w;
    w.x = v[0] | ((uint32_t)v[1] << 16);
    w.y = v[2] | ((uint32_t)v[3] << 16);
    w.z = v[4] | ((uint32_t)v[5] << 16);
    w.w = v[6] | ((uint32_t)v[7] << 16);
    *reinterpret_cast<uint4*>(dst + tc::sw128_offset((uint32_t)rows, r, k0)) = w;
}

cudaError_t launch_pack_sw128(const void* src, int rows, int K, int ld, int kpad, void* dst, cudaStream_t s)
{
    if (rows <= 0 || K <= 0 || kpad % 64 || K > kpad || ld < K) return cudaErrorInvalidValue;
    const uint32_t chunks = (uint32_t)rows * (uint32_t)(kpad / 8);
    pack_sw128_kernel<<<(chunks + 255) / 256, 256, 0, s>>>(static_cast<const bf16*>(src), rows, K, ld, kpad,
                                                           static_cast<unsigned char*>(dst));
    return cudaGetLastError();
}

size_t mlp_tc_image_bytes() { return tc::kImgBytes; }

cudaError_t launch_mlp_tc(const float* feats, uint32_t n, const float* fmean, const float* fistd,
                          const void* wimg, const float* b0, const float* b1, const float* b2, const float* b3,
                          float* out, unsigned* err, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(mlp_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tc::kSmemBytes);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 1;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    const uint32_t blocks = (n + tc::kRows - 1) / tc::kRows;
    const uint32_t grid = blocks < (uint32_t)sms ? blocks : (uint32_t)sms;   // one CTA per SM
    mlp_tc_kernel<<<grid, tc::kThreads, tc::kSmemBytes, s>>>(feats, n, fmean, fistd,
                                                            static_cast<const unsigned char*>(wimg), b0, b1, b2,
                                                            b3, out, err);
    return cudaGetLastError();
}

}  // namespace sfh
