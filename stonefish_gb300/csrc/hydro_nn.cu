// hydro_nn.cu -- kernels of the learned wrench surrogate (an MLP on BF16
// tensor cores with FP32 accumulation) and the feature/gate kernels around
// it.  The surrogate replaces the exact integrator for states inside its
// training domain; states outside (the out-of-distribution gate) go to the
// exact kernels.  Nothing here has a counterpart in the reference.
//
// GEMM: C[M,N] = A[M,K] * B[K,N], A and B row-major BF16, FP32 accumulators,
// mma.sync m16n8k16 tiles fed by ldmatrix from shared memory; 64x64 CTA
// tiles, four warps of 32x32.  M, N multiples of 64 and K a multiple of 32
// (the host pads), so no tile is partial.
#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/stonefish_hydro.h"
#include "hydro_device.cuh"

namespace sfh {

typedef __nv_bfloat16 bf16;

struct EpiArgs {
    float* z;            // FP32 output (pre-activation or plain product)
    bf16* y;             // BF16 output (activation or gradient)
    const float* bias;   // per column
    const float* zprev;  // pre-activations of the layer the gradient flows into
    int ldc;             // leading dimension of the outputs
    size_t split_stride; // split-K (EPI_F32): floats between the partial products of consecutive K slices
};

enum : int { EPI_F32 = 0, EPI_BIAS_SILU = 1, EPI_BIAS = 2, EPI_SILU_GRAD = 3 };

__device__ __forceinline__ float sigmoidf_(float z) { return 1.f / (1.f + expf(-z)); }

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void* p)
{
    const uint32_t a = static_cast<uint32_t>(__cvta_generic_to_shared(p));
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(a));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const void* p)
{
    const uint32_t a = static_cast<uint32_t>(__cvta_generic_to_shared(p));
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(a));
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
                 "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

constexpr int BM = 64, BN = 64, BK = 32;
constexpr int APAD = 8, BPAD = 8;

template <int EPI>
__global__ void __launch_bounds__(128) gemm_kernel(const bf16* __restrict__ A, int lda,
                                                   const bf16* __restrict__ B, int ldb, int K,
                                                   EpiArgs e)
{
    // two stages: the next K-step's tiles are loaded into registers while
    // the current one is multiplied, then stored into the other stage
    __shared__ __align__(16) bf16 As[2][BM][BK + APAD];
    __shared__ __align__(16) bf16 Bs[2][BK][BN + BPAD];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    if (EPI == EPI_F32 && blockIdx.z > 0) {
        // split-K: slice z covers K columns z K .. of A and rows of B and
        // writes its partial product to its own plane of the workspace
        A += (size_t)blockIdx.z * K;
        B += (size_t)blockIdx.z * K * ldb;
        e.z += blockIdx.z * e.split_stride;
    }
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;

    uint4 ra[2], rb[2];
    auto load = [&](int k0) {
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int c = tid + i * 128;
            ra[i] = *reinterpret_cast<const uint4*>(A + (size_t)(m0 + (c >> 2)) * lda + k0 + (c & 3) * 8);
            rb[i] = *reinterpret_cast<const uint4*>(B + (size_t)(k0 + (c >> 3)) * ldb + n0 + (c & 7) * 8);
        }
    };
    auto store = [&](int st) {
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int c = tid + i * 128;
            *reinterpret_cast<uint4*>(&As[st][c >> 2][(c & 3) * 8]) = ra[i];
            *reinterpret_cast<uint4*>(&Bs[st][c >> 3][(c & 7) * 8]) = rb[i];
        }
    };
    load(0);
    store(0);
    __syncthreads();
    int st = 0;
    for (int k0 = 0; k0 < K; k0 += BK) {
        const bool more = k0 + BK < K;
        if (more) load(k0 + BK);
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            uint32_t a[2][4];
#pragma unroll
            for (int mi = 0; mi < 2; ++mi)
                ldsm_x4(a[mi], &As[st][wm + mi * 16 + (lane & 15)][kk + (lane >> 4) * 8]);
            uint32_t b[4][2];
#pragma unroll
            for (int nj = 0; nj < 2; ++nj) {
                const int j = lane >> 3;
                uint32_t r[4];
                ldsm_x4_t(r, &Bs[st][kk + (lane & 7) + 8 * (j & 1)][wn + nj * 16 + 8 * (j >> 1)]);
                b[2 * nj][0] = r[0];
                b[2 * nj][1] = r[1];
                b[2 * nj + 1][0] = r[2];
                b[2 * nj + 1][1] = r[3];
            }
#pragma unroll
            for (int mi = 0; mi < 2; ++mi)
#pragma unroll
                for (int ni = 0; ni < 4; ++ni) mma_bf16(acc[mi][ni], a[mi], b[ni][0], b[ni][1]);
        }
        // the other stage was last read before the previous barrier
        if (more) store(st ^ 1);
        __syncthreads();
        st ^= 1;
    }

#pragma unroll
    for (int mi = 0; mi < 2; ++mi) {
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int r = m0 + wm + mi * 16 + (lane >> 2) + 8 * h;
                const int c = n0 + wn + ni * 8 + (lane & 3) * 2;
                float v0 = acc[mi][ni][2 * h], v1 = acc[mi][ni][2 * h + 1];
                const size_t o = (size_t)r * e.ldc + c;
                if (EPI == EPI_F32) {
                    e.z[o] = v0;
                    e.z[o + 1] = v1;
                } else if (EPI == EPI_BIAS || EPI == EPI_BIAS_SILU) {
                    v0 += e.bias[c];
                    v1 += e.bias[c + 1];
                    if (EPI == EPI_BIAS || e.z) {   // inference needs no pre-activations
                        e.z[o] = v0;
                        e.z[o + 1] = v1;
                    }
                    if (EPI == EPI_BIAS_SILU) {
                        e.y[o] = __float2bfloat16(v0 * sigmoidf_(v0));
                        e.y[o + 1] = __float2bfloat16(v1 * sigmoidf_(v1));
                    }
                } else {   // EPI_SILU_GRAD: dZ = dY * silu'(zprev)
                    const float z0 = e.zprev[o], z1 = e.zprev[o + 1];
                    const float s0 = sigmoidf_(z0), s1 = sigmoidf_(z1);
                    e.y[o] = __float2bfloat16(v0 * (s0 + z0 * s0 * (1.f - s0)));
                    e.y[o + 1] = __float2bfloat16(v1 * (s1 + z1 * s1 * (1.f - s1)));
                }
            }
        }
    }
}

// out[r][c] (row stride ldc) = sum over the `splits` partial products in
// split order (deterministic).
__global__ void splitk_reduce_kernel(const float* __restrict__ ws, int splits, int M, int N, float* out, int ldc)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t mn = (size_t)M * N;
    if (i >= mn) return;
    float v = ws[i];
    for (int z = 1; z < splits; ++z) v += ws[z * mn + i];
    out[(i / N) * ldc + i % N] = v;
}

int gemm_splits(int epi, int M, int N, int K)
{
    // An EPI_F32 product with few output tiles and a long K (the weight
    // gradients: K = batch) is split along K so that the GPU fills: slices of
    // at least 256 columns, up to about two CTAs per SM.
    if (epi != EPI_F32) return 1;
    const int tiles = (M / BM) * (N / BN);
    int s = 1;
    while (s < 32 && K % (2 * s * BK) == 0 && K / (2 * s) >= 256 && tiles * 2 * s <= 320) s *= 2;
    return s;
}

cudaError_t launch_gemm(int epi, const void* A, int lda, const void* B, int ldb, int M, int N, int K,
                        float* z, void* y, const float* bias, const float* zprev, int ldc,
                        cudaStream_t s, float* ws, size_t ws_floats)
{
    if (M % BM || N % BN || K % BK || M <= 0 || N <= 0 || K <= 0) return cudaErrorInvalidValue;
    dim3 grid(N / BN, M / BM), block(128);
    EpiArgs e{z, static_cast<bf16*>(y), bias, zprev, ldc, 0};
    const bf16* a = static_cast<const bf16*>(A);
    const bf16* b = static_cast<const bf16*>(B);
    const int splits = gemm_splits(epi, M, N, K);
    if (splits > 1 && ws && (size_t)splits * M * N <= ws_floats) {
        EpiArgs w{ws, nullptr, nullptr, nullptr, N, (size_t)M * N};
        gemm_kernel<EPI_F32><<<dim3(N / BN, M / BM, splits), block, 0, s>>>(a, lda, b, ldb, K / splits, w);
        cudaError_t err = cudaGetLastError();
        if (err != cudaSuccess) return err;
        const size_t mn = (size_t)M * N;
        splitk_reduce_kernel<<<(unsigned)((mn + 255) / 256), 256, 0, s>>>(ws, splits, M, N, z, ldc);
        return cudaGetLastError();
    }
    switch (epi) {
    case EPI_F32: gemm_kernel<EPI_F32><<<grid, block, 0, s>>>(a, lda, b, ldb, K, e); break;
    case EPI_BIAS_SILU: gemm_kernel<EPI_BIAS_SILU><<<grid, block, 0, s>>>(a, lda, b, ldb, K, e); break;
    case EPI_BIAS: gemm_kernel<EPI_BIAS><<<grid, block, 0, s>>>(a, lda, b, ldb, K, e); break;
    case EPI_SILU_GRAD: gemm_kernel<EPI_SILU_GRAD><<<grid, block, 0, s>>>(a, lda, b, ldb, K, e); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------- small kernels
// dst[c][r] = src[r][c] for a rows x cols BF16 matrix (32x32 tiles).
__global__ void transpose_kernel(const bf16* __restrict__ src, bf16* __restrict__ dst, int rows, int cols)
{
    __shared__ bf16 t[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int r = r0 + i, c = c0 + threadIdx.x;
        if (r < rows && c < cols) t[i][threadIdx.x] = src[(size_t)r * cols + c];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int c = c0 + i, r = r0 + threadIdx.x;
        if (r < rows && c < cols) dst[(size_t)c * rows + r] = t[threadIdx.x][i];
    }
}

cudaError_t launch_transpose(const void* src, void* dst, int rows, int cols, cudaStream_t s)
{
    dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
    transpose_kernel<<<grid, block, 0, s>>>(static_cast<const bf16*>(src), static_cast<bf16*>(dst), rows, cols);
    return cudaGetLastError();
}

// Masked mean-squared error on the first n_out of ld columns against the
// normalised target t' = (t - tmean) * tistd (identity when tmean is null):
// dZ (BF16, padded columns zero) = 2 (z - t') / (rows * n_out), and
// loss += sum (z - t')^2 / (rows * n_out), summed per block in FP32 and
// added in FP64.
__global__ void mse_grad_kernel(const float* __restrict__ z, const float* __restrict__ t, int rows, int ld,
                                int n_out, const float* __restrict__ tmean, const float* __restrict__ tistd,
                                bf16* __restrict__ dz, double* loss)
{
    __shared__ float red[256];
    const uint32_t n = (uint32_t)rows * (uint32_t)ld;   // < 2^32, checked by the host
    const float scale = 1.f / (float)((size_t)rows * n_out);
    float acc = 0.f;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t r = i / (uint32_t)ld, c = i - r * (uint32_t)ld;
        float g = 0.f;
        if (c < (uint32_t)n_out) {
            float tv = t[(size_t)r * n_out + c];
            if (tmean) tv = (tv - tmean[c]) * tistd[c];
            const float d = z[i] - tv;
            acc += d * d;
            g = 2.f * d * scale;
        }
        dz[i] = __float2bfloat16(g);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0 && loss) atomicAdd(loss, (double)red[0] * (double)scale);
}

cudaError_t launch_mse_grad(const float* z, const float* t, int rows, int ld, int n_out, const float* tmean,
                            const float* tistd, void* dz, double* loss, cudaStream_t s)
{
    mse_grad_kernel<<<256, 256, 0, s>>>(z, t, rows, ld, n_out, tmean, tistd, static_cast<bf16*>(dz), loss);
    return cudaGetLastError();
}

// out[c] = sum_r g[r][c] (BF16 in, FP32 out).  One CTA per 32 columns:
// 32 row groups of 32 lanes (coalesced 64-byte row segments), then a
// shared-memory sum over the row groups in a fixed order.
__global__ void __launch_bounds__(1024) colsum_kernel(const bf16* __restrict__ g, int rows, int cols,
                                                      float* __restrict__ out)
{
    __shared__ float part[32][33];
    const int c = blockIdx.x * 32 + threadIdx.x;
    float s = 0.f;
    if (c < cols)
        for (int r = threadIdx.y; r < rows; r += 32) s += __bfloat162float(g[(size_t)r * cols + c]);
    part[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.y == 0 && c < cols) {
        float t = 0.f;
        for (int k = 0; k < 32; ++k) t += part[k][threadIdx.x];
        out[c] = t;
    }
}

// The same sums over many rows in two stages, so that more than a handful
// of SMs read the matrix: CTA (x, y) sums 32 columns over row slab y (the
// single-stage order within the slab) into ws[y][c], then out[c] adds the
// slabs' partial sums in slab order.
__global__ void __launch_bounds__(1024) colsum_slab_kernel(const bf16* __restrict__ g, int rows, int cols,
                                                           int slab_rows, float* __restrict__ ws)
{
    __shared__ float part[32][33];
    const int c = blockIdx.x * 32 + threadIdx.x;
    const int r0 = blockIdx.y * slab_rows, r1 = min(rows, r0 + slab_rows);
    float s = 0.f;
    if (c < cols)
        for (int r = r0 + threadIdx.y; r < r1; r += 32) s += __bfloat162float(g[(size_t)r * cols + c]);
    part[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.y == 0 && c < cols) {
        float t = 0.f;
        for (int k = 0; k < 32; ++k) t += part[k][threadIdx.x];
        ws[(size_t)blockIdx.y * cols + c] = t;
    }
}

__global__ void colsum_slabs_kernel(const float* __restrict__ ws, int slabs, int cols, float* __restrict__ out)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float t = 0.f;
    for (int k = 0; k < slabs; ++k) t += ws[(size_t)k * cols + c];
    out[c] = t;
}

int colsum_slabs(int rows) { return rows >= 2048 ? std::min(32, rows / 256) : 1; }

cudaError_t launch_colsum(const void* g, int rows, int cols, float* out, cudaStream_t s, float* ws,
                          size_t ws_floats)
{
    const int slabs = colsum_slabs(rows);
    if (slabs > 1 && ws && (size_t)slabs * cols <= ws_floats) {
        const int slab_rows = (rows + slabs - 1) / slabs;
        colsum_slab_kernel<<<dim3((cols + 31) / 32, slabs), dim3(32, 32), 0, s>>>(static_cast<const bf16*>(g), rows,
                                                                                   cols, slab_rows, ws);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        colsum_slabs_kernel<<<(cols + 255) / 256, 256, 0, s>>>(ws, slabs, cols, out);
        return cudaGetLastError();
    }
    colsum_kernel<<<(cols + 31) / 32, dim3(32, 32), 0, s>>>(static_cast<const bf16*>(g), rows, cols, out);
    return cudaGetLastError();
}

// AdamW on FP32 master weights (Loshchilov & Hutter, decoupled weight decay),
// then refresh of the BF16 copies: w16 = [rows][cols] row-major, wt16 its
// transpose [cols][rows].  grad is [rows][cols] FP32 (a bias: rows = 1).
__global__ void adamw_kernel(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                             const float* __restrict__ grad, int rows, int cols, int ldg, float lr,
                             float b1, float b2, float eps, float wd, float bc1, float bc2,
                             bf16* __restrict__ w16, bf16* __restrict__ wt16)
{
    const size_t n = (size_t)rows * cols;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(i / cols), c = (int)(i % cols);
        const float g = grad[(size_t)r * ldg + c];
        const float mi = b1 * m[i] + (1.f - b1) * g;
        const float vi = b2 * v[i] + (1.f - b2) * g * g;
        m[i] = mi;
        v[i] = vi;
        const float mh = mi / bc1, vh = vi / bc2;
        const float wi = w[i] * (1.f - lr * wd) - lr * mh / (sqrtf(vh) + eps);
        w[i] = wi;
        if (w16) w16[i] = __float2bfloat16(wi);
        if (wt16) wt16[(size_t)c * rows + r] = __float2bfloat16(wi);
    }
}

cudaError_t launch_adamw(float* w, float* m, float* v, const float* grad, int rows, int cols, int ldg,
                         float lr, float b1, float b2, float eps, float wd, int step, void* w16,
                         void* wt16, cudaStream_t s)
{
    const float bc1 = 1.f - powf(b1, (float)step), bc2 = 1.f - powf(b2, (float)step);
    const size_t n = (size_t)rows * cols;
    const int blocks = (int)((n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024);
    adamw_kernel<<<blocks, 256, 0, s>>>(w, m, v, grad, rows, cols, ldg, lr, b1, b2, eps, wd, bc1, bc2,
                                        static_cast<bf16*>(w16), static_cast<bf16*>(wt16));
    return cudaGetLastError();
}

// y = bf16((x - mean) * istd) with zero padding of the columns [n_in, ld);
// mean/istd may be null (identity).
__global__ void to_bf16_kernel(const float* __restrict__ x, int rows, int n_in, int ld,
                               const float* __restrict__ mean, const float* __restrict__ istd,
                               bf16* __restrict__ y)
{
    // rows x ld < 2^32 (checked by the host), so 32-bit index arithmetic
    const uint32_t n = (uint32_t)rows * (uint32_t)ld;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t r = i / (uint32_t)ld, c = i - r * (uint32_t)ld;
        float v = 0.f;
        if (c < (uint32_t)n_in) {
            v = x[(size_t)r * n_in + c];
            if (mean) v = (v - mean[c]) * istd[c];
        }
        y[i] = __float2bfloat16(v);
    }
}

cudaError_t launch_to_bf16(const float* x, int rows, int n_in, int ld, const float* mean, const float* istd,
                           void* y, cudaStream_t s)
{
    to_bf16_kernel<<<512, 256, 0, s>>>(x, rows, n_in, ld, mean, istd, static_cast<bf16*>(y));
    return cudaGetLastError();
}

// ---------------------------------------------------------------- features
// The 16 surrogate features of a body state: depth of the CG below the
// local surface (NED), roll, pitch (Z-Y-X Euler angles of T_CG), body-frame
// linear velocity, body-frame angular velocity, body-frame current, and four
// numbers describing the wave surface around the hull: the elevation at the
// CG, the mean slope along and across the heading over +-kWaveReach, and the
// curvature along the heading over the same reach (second difference of the
// elevations ahead of and behind the CG).  The heading is the horizontal
// projection of the body x axis, so the wave features do not depend on yaw.
constexpr float kWaveReach = 1.0f;

// The fields a state's features read, as 8-byte words of its hydro_body:
// T_CG (words 0..11: basis, origin) and v, omega (words 33..38).
constexpr int kFeatWords = 18;
constexpr int kFeatStride = kFeatWords + 1;   // odd: 8-byte reads of a warp free of bank conflicts
constexpr int kFeatBlock = 128;
static_assert(offsetof(hydro_body, T_CG) == 0 && offsetof(hydro_body, v) == 33 * 8 &&
                  offsetof(hydro_body, omega) == 36 * 8 && sizeof(hydro_body) % 8 == 0,
              "feature words of hydro_body");

__global__ void __launch_bounds__(kFeatBlock) features_kernel(const hydro_body* __restrict__ bodies, uint32_t n,
                                                              OceanDev o, float* __restrict__ f)
{
    // Each warp first copies the feature words of its 32 records into shared
    // memory, consecutive lanes reading consecutive words, so that a load
    // instruction touches two records instead of 32 (the records may be
    // page-locked host memory read in place).
    __shared__ double stage[kFeatBlock / 32][32 * kFeatStride];
    const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
    const uint32_t first = blockIdx.x * kFeatBlock + 32u * wib;
    const double* words = reinterpret_cast<const double*>(bodies);
    constexpr uint32_t kRecWords = sizeof(hydro_body) / 8;
#pragma unroll
    for (uint32_t j = 0; j < (uint32_t)kFeatWords; ++j) {
        const uint32_t t = lane + 32u * j, r = t / kFeatWords, p = t % kFeatWords;
        const uint32_t w = p < 12u ? p : 33u + (p - 12u);
        if (first + r < n) stage[wib][r * kFeatStride + p] = words[(size_t)(first + r) * kRecWords + w];
    }
    __syncwarp();
    const uint32_t i = first + lane;
    if (i >= n) return;
    const double* sw = &stage[wib][lane * kFeatStride];
    double R[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) R[k] = sw[k];
    const double x = sw[9], y = sw[10], z = sw[11];
    const double bv[3] = {sw[12], sw[13], sw[14]}, bw[3] = {sw[15], sw[16], sw[17]};
    // heading (unit horizontal projection of the body x axis), FP32
    float ux = (float)R[0], uy = (float)R[3];   // (same values as Rf[0], Rf[3] below)
    const float hn = sqrtf(ux * ux + uy * uy);
    if (hn > 1e-6f) {
        ux /= hn;
        uy /= hn;
    } else {   // body x axis vertical: any heading
        ux = 1.f;
        uy = 0.f;
    }
    float h = 0.f, s_al = 0.f, s_ac = 0.f, k_al = 0.f;
    if (o.waves) {
        const float a = kWaveReach;
        const float fx = (float)x, fy = (float)y;
        h = -wave_height(o, fx, fy);
        const float ef = -wave_height(o, fx + a * ux, fy + a * uy);
        const float eb = -wave_height(o, fx - a * ux, fy - a * uy);
        const float el = -wave_height(o, fx - a * uy, fy + a * ux);
        const float er = -wave_height(o, fx + a * uy, fy - a * ux);
        s_al = (ef - eb) / (2.f * a);
        s_ac = (el - er) / (2.f * a);
        k_al = (ef + eb - 2.f * h) / (a * a);
    }
    // R^T u for the body-frame vectors, in FP32 (GB300's FP64 pipe would
    // set this kernel's pace; the features are rounded to BF16 downstream)
    float Rf[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) Rf[k] = (float)R[k];
    auto tb = [&](const double* u, float* out) {
        const float u0 = (float)u[0], u1 = (float)u[1], u2 = (float)u[2];
        out[0] = (Rf[0] * u0 + Rf[3] * u1) + Rf[6] * u2;
        out[1] = (Rf[1] * u0 + Rf[4] * u1) + Rf[7] * u2;
        out[2] = (Rf[2] * u0 + Rf[5] * u1) + Rf[8] * u2;
    };
    float* o16 = f + (size_t)i * 16;
    o16[0] = (float)z + h;                          // depth below the local surface (NED: surface at -h)
    o16[1] = atan2f(Rf[7], Rf[8]);                  // roll
    o16[2] = asinf(fmaxf(-1.f, fminf(1.f, -Rf[6])));  // pitch
    tb(bv, o16 + 3);
    tb(bw, o16 + 6);
    double u[3] = {o.U[0], o.U[1], o.U[2]};
    tb(u, o16 + 9);
    o16[12] = h;
    o16[13] = s_al;
    o16[14] = s_ac;
    o16[15] = k_al;
}

cudaError_t launch_features(const hydro_body* bodies, uint32_t n, OceanDev o, float* f, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    features_kernel<<<(n + kFeatBlock - 1) / kFeatBlock, kFeatBlock, 0, s>>>(bodies, n, o, f);
    return cudaGetLastError();
}

// Out-of-distribution gate: mask[i] = 1 when feature vector i lies inside
// the per-feature box [lo, hi] and its squared Mahalanobis distance
// (x - mean)^T P (x - mean), P the inverse training covariance (16x16), is
// at most thresh; 0 sends the state to the exact integrator.
__global__ void gate_kernel(const float* __restrict__ f, uint32_t n, const float* __restrict__ lo,
                            const float* __restrict__ hi, const float* __restrict__ mean,
                            const float* __restrict__ P, float thresh, uint8_t* __restrict__ mask)
{
    __shared__ float Ps[256], ls[16], hs[16], ms[16];
    for (int k = threadIdx.x; k < 256; k += blockDim.x) Ps[k] = P[k];
    if (threadIdx.x < 16) {
        ls[threadIdx.x] = lo[threadIdx.x];
        hs[threadIdx.x] = hi[threadIdx.x];
        ms[threadIdx.x] = mean[threadIdx.x];
    }
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float d[16];
    bool in = true;
    const float4* f4 = reinterpret_cast<const float4*>(f + (size_t)i * 16);
#pragma unroll
    for (int k4 = 0; k4 < 4; ++k4) {
        const float4 v = f4[k4];
        const float xs[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int k = 4 * k4 + j;
            in = in && (xs[j] >= ls[k]) && (xs[j] <= hs[k]);
            d[k] = xs[j] - ms[k];
        }
    }
    float q = 0.f;
#pragma unroll
    for (int r = 0; r < 16; ++r) {
        float s = 0.f;
#pragma unroll
        for (int c = 0; c < 16; ++c) s += Ps[r * 16 + c] * d[c];
        q += d[r] * s;
    }
    mask[i] = (in && q <= thresh) ? 1 : 0;
}

cudaError_t launch_gate(const float* f, uint32_t n, const float* lo, const float* hi, const float* mean,
                        const float* P, float thresh, uint8_t* mask, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    gate_kernel<<<(n + 127) / 128, 128, 0, s>>>(f, n, lo, hi, mean, P, thresh, mask);
    return cudaGetLastError();
}

// Total wrench in the body frame for the surrogate's targets:
// out[i] = (R^T (Fb + Fdq + Fdf), R^T (Tb + Tdq + Tdf)).
__global__ void wrench_body_kernel(const hydro_body* __restrict__ bodies, const hydro_wrench* __restrict__ w,
                                   uint32_t n, float* __restrict__ out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* R = bodies[i].T_CG.basis;
    const hydro_wrench& x = w[i];
    double F[3], T[3];
    for (int k = 0; k < 3; ++k) {
        F[k] = x.Fb[k] + x.Fdq[k] + x.Fdf[k];
        T[k] = x.Tb[k] + x.Tdq[k] + x.Tdf[k];
    }
    for (int k = 0; k < 3; ++k) {
        out[(size_t)i * 6 + k] = (float)(R[k] * F[0] + R[3 + k] * F[1] + R[6 + k] * F[2]);
        out[(size_t)i * 6 + 3 + k] = (float)(R[k] * T[0] + R[3 + k] * T[1] + R[6 + k] * T[2]);
    }
}

cudaError_t launch_wrench_body(const hydro_body* bodies, const hydro_wrench* w, uint32_t n, float* out,
                               cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    wrench_body_kernel<<<(n + 127) / 128, 128, 0, s>>>(bodies, w, n, out);
    return cudaGetLastError();
}

// ------------------------------------------------- gate routing (exact path)
// Bodies the gate rejects (mask 0) are packed, in index order, to the front
// of a second body array that the exact integrator runs on; the rest of that
// array is switched off (mode DISABLED), which the exact step skips at no
// cost.  pos[i] is the packed slot of body i, or -1.
constexpr int kRouteBlock = 256;

__global__ void route_count_kernel(const uint8_t* __restrict__ mask, uint32_t n, uint32_t* __restrict__ counts)
{
    const uint32_t i = blockIdx.x * kRouteBlock + threadIdx.x;
    const bool out = i < n && mask[i] == 0;
    const int c = __syncthreads_count(out);
    if (threadIdx.x == 0) counts[blockIdx.x] = (uint32_t)c;
}

__global__ void route_pack_kernel(const hydro_body* __restrict__ bodies, const uint8_t* __restrict__ mask,
                                  uint32_t n, const uint32_t* __restrict__ counts, uint32_t n_blocks,
                                  hydro_body* __restrict__ packed, int32_t* __restrict__ pos,
                                  uint32_t* __restrict__ n_packed, hydro_wrench* __restrict__ exact)
{
    __shared__ uint32_t warp_base[kRouteBlock / 32];
    __shared__ uint32_t sums[2];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x < 32) {
        // block offset and total from the per-block counts (fixed order)
        uint32_t before = 0, total = 0;
        for (uint32_t k = lane; k < n_blocks; k += 32) {
            const uint32_t c = counts[k];
            total += c;
            if (k < blockIdx.x) before += c;
        }
        for (int o = 16; o; o >>= 1) {
            before += __shfl_xor_sync(0xffffffffu, before, o);
            total += __shfl_xor_sync(0xffffffffu, total, o);
        }
        if (lane == 0) {
            sums[0] = before;
            sums[1] = total;
        }
    }
    const uint32_t i = blockIdx.x * kRouteBlock + threadIdx.x;
    const bool out = i < n && mask[i] == 0;
    const unsigned bal = __ballot_sync(0xffffffffu, out);
    if (lane == 0) warp_base[warp] = __popc(bal);
    __syncthreads();
    uint32_t base = sums[0];
    for (int w = 0; w < warp; ++w) base += warp_base[w];
    const uint32_t total = sums[1];
    if (i < n) {
        if (out) {
            const uint32_t j = base + __popc(bal & ((1u << lane) - 1u));
            packed[j] = bodies[i];
            pos[i] = (int32_t)j;
            if (exact) {   // fresh in-out record for the exact step
                static_assert(sizeof(hydro_wrench) % 8 == 0, "zeroed as 8-byte words");
                uint64_t* w = reinterpret_cast<uint64_t*>(exact + j);
#pragma unroll
                for (uint32_t k = 0; k < sizeof(hydro_wrench) / 8; ++k) w[k] = 0ull;
            }
        } else {
            pos[i] = -1;
        }
        if (i >= total) packed[i].mode = HYDRO_MODE_DISABLED;
    }
    if (i == 0) *n_packed = total;
}

cudaError_t launch_route(const hydro_body* bodies, const uint8_t* mask, uint32_t n, uint32_t* counts,
                         hydro_body* packed, int32_t* pos, uint32_t* n_packed, hydro_wrench* exact,
                         cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    const uint32_t nb = (n + kRouteBlock - 1) / kRouteBlock;
    route_count_kernel<<<nb, kRouteBlock, 0, s>>>(mask, n, counts);
    route_pack_kernel<<<nb, kRouteBlock, 0, s>>>(bodies, mask, n, counts, nb, packed, pos, n_packed, exact);
    return cudaGetLastError();
}

// out[i] (6 floats, body frame) = the surrogate's row of z (ld floats) for
// gated-in bodies, else the exact wrench of packed slot pos[i].
__global__ void merge_kernel(const hydro_body* __restrict__ bodies, const float* __restrict__ z, int ld,
                             const int32_t* __restrict__ pos, const hydro_wrench* __restrict__ exact,
                             uint32_t n, float* __restrict__ out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t j = pos[i];
    if (j < 0) {
        for (int k = 0; k < 6; ++k) out[(size_t)i * 6 + k] = z[(size_t)i * ld + k];
        return;
    }
    const double* R = bodies[i].T_CG.basis;
    const hydro_wrench& x = exact[j];
    double F[3], T[3];
    for (int k = 0; k < 3; ++k) {
        F[k] = x.Fb[k] + x.Fdq[k] + x.Fdf[k];
        T[k] = x.Tb[k] + x.Tdq[k] + x.Tdf[k];
    }
    for (int k = 0; k < 3; ++k) {
        out[(size_t)i * 6 + k] = (float)(R[k] * F[0] + R[3 + k] * F[1] + R[6 + k] * F[2]);
        out[(size_t)i * 6 + 3 + k] = (float)(R[k] * T[0] + R[3 + k] * T[1] + R[6 + k] * T[2]);
    }
}

cudaError_t launch_merge(const hydro_body* bodies, const float* z, int ld, const int32_t* pos,
                         const hydro_wrench* exact, uint32_t n, float* out, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    merge_kernel<<<(n + 127) / 128, 128, 0, s>>>(bodies, z, ld, pos, exact, n, out);
    return cudaGetLastError();
}

// ------------------------------------------------------ ensemble and audit
// Two networks' outputs: za (ld floats per row, columns 0..5 the wrench)
// becomes their mean, and the gate mask of a row is cleared when the two
// disagree by more than tau in the wrench metric (force difference over the
// force scale, torque difference over the torque scale, the larger of two).
__global__ void ensemble_kernel(float* __restrict__ za, const float* __restrict__ zb, int ld, uint32_t n,
                                float inv_fs, float inv_ts, float tau, uint8_t* __restrict__ mask)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float* a = za + (size_t)i * ld;
    const float* b = zb + (size_t)i * ld;
    float df = 0.f, dt = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float x = a[k] - b[k], y = a[3 + k] - b[3 + k];
        df += x * x;
        dt += y * y;
    }
    const float d = fmaxf(sqrtf(df) * inv_fs, sqrtf(dt) * inv_ts);
#pragma unroll
    for (int k = 0; k < 6; ++k) a[k] = 0.5f * (a[k] + b[k]);
    if (d > tau) mask[i] = 0;
}

cudaError_t launch_ensemble(float* za, const float* zb, int ld, uint32_t n, float inv_fs, float inv_ts, float tau,
                            uint8_t* mask, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    ensemble_kernel<<<(n + 127) / 128, 128, 0, s>>>(za, zb, ld, n, inv_fs, inv_ts, tau, mask);
    return cudaGetLastError();
}

// Audit sample: rows phase, phase + stride, ... that the gate admitted are
// sent to the exact step as well (mask cleared, so their output is the exact
// wrench) and recorded in idx; other sample slots get -1.
__global__ void audit_pick_kernel(uint8_t* __restrict__ mask, uint32_t n, uint32_t stride, uint32_t phase,
                                  uint32_t k, int32_t* __restrict__ idx)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= k) return;
    const uint32_t i = phase + j * stride;
    int32_t r = -1;
    if (i < n && mask[i] != 0) {
        mask[i] = 0;
        r = (int32_t)i;
    }
    idx[j] = r;
}

cudaError_t launch_audit_pick(uint8_t* mask, uint32_t n, uint32_t stride, uint32_t phase, uint32_t k, int32_t* idx,
                              cudaStream_t s)
{
    if (k == 0) return cudaSuccess;
    audit_pick_kernel<<<(k + 127) / 128, 128, 0, s>>>(mask, n, stride, phase, k, idx);
    return cudaGetLastError();
}

// Error of the surrogate's row z[i] against the exact body-frame wrench of
// each audited row i = idx[j] (exact[pos[i]]): err[j] = max(|dF| / fs,
// |dT| / ts), or -1 for an empty sample slot.
__global__ void audit_error_kernel(const hydro_body* __restrict__ bodies, const float* __restrict__ z, int ld,
                                   const int32_t* __restrict__ pos, const hydro_wrench* __restrict__ exact,
                                   const int32_t* __restrict__ idx, uint32_t k, float inv_fs, float inv_ts,
                                   float* __restrict__ err)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= k) return;
    const int32_t i = idx[j];
    if (i < 0 || pos[i] < 0) {
        err[j] = -1.f;
        return;
    }
    const double* R = bodies[i].T_CG.basis;
    const hydro_wrench& x = exact[pos[i]];
    double F[3], T[3];
    for (int c = 0; c < 3; ++c) {
        F[c] = x.Fb[c] + x.Fdq[c] + x.Fdf[c];
        T[c] = x.Tb[c] + x.Tdq[c] + x.Tdf[c];
    }
    double df = 0.0, dt = 0.0;
    for (int c = 0; c < 3; ++c) {
        const double fb = R[c] * F[0] + R[3 + c] * F[1] + R[6 + c] * F[2];
        const double tb = R[c] * T[0] + R[3 + c] * T[1] + R[6 + c] * T[2];
        const double a = (double)z[(size_t)i * ld + c] - fb, b = (double)z[(size_t)i * ld + 3 + c] - tb;
        df += a * a;
        dt += b * b;
    }
    err[j] = (float)fmax(sqrt(df) * (double)inv_fs, sqrt(dt) * (double)inv_ts);
}

cudaError_t launch_audit_error(const hydro_body* bodies, const float* z, int ld, const int32_t* pos,
                               const hydro_wrench* exact, const int32_t* idx, uint32_t k, float inv_fs,
                               float inv_ts, float* err, cudaStream_t s)
{
    if (k == 0) return cudaSuccess;
    audit_error_kernel<<<(k + 127) / 128, 128, 0, s>>>(bodies, z, ld, pos, exact, idx, k, inv_fs, inv_ts, err);
    return cudaGetLastError();
}

}  // namespace sfh
