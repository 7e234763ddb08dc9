// hydro_fft_ocean.cu -- the reference's FFT ocean as CUDA: the wave field
// Stonefish computes with OpenGL shaders (OpenGLOcean::Simulate,
// Library/src/graphics/OpenGLOcean.cpp:455-540) and reads back for the
// hydrodynamics (OpenGLRealOcean.cpp:333-357), written here as kernels that
// fill the context's wave grid directly.
//
//   * spectrum (host, once): OpenGLOcean::GenerateWavesSpectrum / spectrum /
//     GetSpectrumSample (OpenGLOcean.cpp:929-1048), the Elfouhaily spectrum
//     for four grid sizes with random phases from the reference's LCG
//     (SystemUtil.hpp:208-218, seed 1234), stored as the reference stores it:
//     RGBA16F textures, so every value is rounded to binary16;
//   * init (per time t): oceanInit.frag -- h(k,t) of the four grids packed as
//     two complex fields per texel, (h1 + i h2, h3 + i h4);
//   * FFT: oceanFFTX.frag then oceanFFTY.frag -- log2(N) radix-2 passes per
//     direction driven by the butterfly table of
//     OpenGLOcean::ComputeButterflyLookupTable (:874-926), itself an RGBA16F
//     texture (indices and weights rounded to binary16); one CTA per line,
//     the line held in shared memory across its passes.
// The result is the readback the hydrodynamics use: N x N texels of
// (grid 0, grid 1, grid 2, grid 3) heights; the depth lookup reads channels
// 0 and 1 at the first two grid sizes (OpenGLRealOcean.cpp:321-331).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <vector>

#include "hydro_internal.h"

namespace sfh {

namespace fft {

constexpr double kPi = 3.14159265358979323846;

float h16(float x) { return __half2float(__float2half_rn(x)); }

// lrandom / frandom (SystemUtil.hpp:208-218)
float frandom(int64_t* seed)
{
    *seed = (*seed * 1103515245 + 12345) & 0x7FFFFFFF;
    const int64_t r = *seed >> (31 - 24);
    return (float)r / (float)(1 << 24);
}

struct Spectrum {
    const hydro_fft_ocean_params& p;
    float sqr(float x) const { return x * x; }
    float omega(float k) const { return (float)std::sqrt(9.81 * k * (1.0 + sqr(k / p.km))); }   // Eq 24

    // OpenGLOcean::spectrum (:940-1001), directional form
    float operator()(float kx, float ky) const
    {
        const float U10 = p.wind, Omega = p.omega;
        const float k = std::sqrt(kx * kx + ky * ky);
        const float c = omega(k) / k;
        const float kp = (float)(9.81 * sqr(Omega / U10));
        const float cp = omega(kp) / kp;
        const float z0 = (float)(3.7e-5 * sqr(U10) / 9.81 * std::pow(U10 / cp, 0.9f));
        const float u_star = (float)(0.41 * U10 / std::log(10.0 / z0));
        const float Lpm = (float)std::exp(-5.0 / 4.0 * sqr(kp / k));
        const float gamma = Omega < 1.0f ? 1.7f : (float)(1.7 + 6.0 * std::log(Omega));
        const float sigma = (float)(0.08 * (1.0 + 4.0 / std::pow(Omega, 3.0f)));
        const float Gamma = (float)std::exp(-1.0 / (2.0 * sqr(sigma)) * sqr((float)(std::sqrt(k / kp) - 1.0)));
        const float Jp = std::pow(gamma, Gamma);
        const float Fp = (float)(Lpm * Jp * std::exp(-Omega / std::sqrt(10.0) * (std::sqrt(k / kp) - 1.0)));
        const float alphap = (float)(0.006 * std::sqrt(Omega));
        float Bl = (float)(0.5 * alphap * cp / c * Fp);
        const float alpham = (float)(0.01 * (u_star < p.cm ? 1.0 + std::log(u_star / p.cm)
                                                           : 1.0 + 3.0 * std::log(u_star / p.cm)));
        const float Fm = (float)std::exp(-0.25 * sqr(k / p.km - 1.0f));
        float Bh = (float)(0.5 * alpham * p.cm / c * Fm);
        Bh *= Lpm;
        const float a0 = (float)(std::log(2.0) / 4.0);
        const float ap = 4.0f;
        const float am = (float)(0.13 * u_star / p.cm);
        const float Delta = (float)std::tanh(a0 + ap * std::pow(c / cp, 2.5f) + am * std::pow(p.cm / c, 2.5f));
        const float phi = std::atan2(ky, kx);
        if (p.propagate) {
            if (kx < 0.0f) return 0.0f;
            Bl *= 2.0f;
            Bh *= 2.0f;
        }
        return (float)(p.amplitude * (Bl + Bh) * (1.0 + Delta * std::cos(2.0 * phi)) /
                       (2.0 * kPi * sqr(sqr(k))));   // Eq 67
    }
};

// OpenGLOcean::GetSpectrumSample (:1004-1023)
void sample(const Spectrum& S, int i, int j, float L, float kMin, int64_t* seed, float* out)
{
    const float dk = (float)(2.0 * kPi / L);
    const float kx = i * dk, ky = j * dk;
    if (std::fabs(kx) < kMin && std::fabs(ky) < kMin) {
        out[0] = 0.0f;
        out[1] = 0.0f;
        return;
    }
    const float s = S(kx, ky);
    const float h = std::sqrt((float)(s / 2.0)) * dk;
    const float phi = (float)(frandom(seed) * 2.0 * kPi);
    out[0] = (float)(h * std::cos(phi));
    out[1] = (float)(h * std::sin(phi));
}

int bit_reverse(int i, int N)
{
    int sum = 0, w = 1;
    for (int m = N / 2; m != 0; m /= 2) {
        sum += ((i & m) > m - 1) * w;
        w *= 2;
    }
    return sum;
}

}  // namespace fft

void fft_ocean_spectrum(const hydro_fft_ocean_params& p, std::vector<float4>& s12, std::vector<float4>& s34)
{
    const int N = 1 << p.passes;
    s12.assign((size_t)N * N, make_float4(0, 0, 0, 0));
    s34.assign((size_t)N * N, make_float4(0, 0, 0, 0));
    const fft::Spectrum S{p};
    int64_t seed = 1234;
    const float* g = p.grid_sizes;
    const float kmin[4] = {(float)(fft::kPi / g[0]), (float)(fft::kPi * N / g[0]), (float)(fft::kPi * N / g[1]),
                           (float)(fft::kPi * N / g[2])};
    for (int y = 0; y < N; ++y) {
        for (int x = 0; x < N; ++x) {
            const int i = x >= N / 2 ? x - N : x;
            const int j = y >= N / 2 ? y - N : y;
            float r[8];
            for (int q = 0; q < 4; ++q) fft::sample(S, i, j, g[q], kmin[q], &seed, r + 2 * q);
            // RGBA16F textures
            s12[(size_t)y * N + x] = make_float4(fft::h16(r[0]), fft::h16(r[1]), fft::h16(r[2]), fft::h16(r[3]));
            s34[(size_t)y * N + x] = make_float4(fft::h16(r[4]), fft::h16(r[5]), fft::h16(r[6]), fft::h16(r[7]));
        }
    }
}

// OpenGLOcean::ComputeButterflyLookupTable (:874-926), decoded: per (pass,
// output) the two input indices and the binary16-rounded weight.
void fft_ocean_butterfly(int passes, std::vector<int2>& idx, std::vector<float2>& w)
{
    const int N = 1 << passes;
    idx.assign((size_t)N * passes, make_int2(0, 0));
    w.assign((size_t)N * passes, make_float2(0, 0));
    for (int i = 0; i < passes; ++i) {
        const int nBlocks = 1 << (passes - 1 - i), nH = 1 << i;
        for (int j = 0; j < nBlocks; ++j) {
            for (int k = 0; k < nH; ++k) {
                const int i1 = j * nH * 2 + k, i2 = j * nH * 2 + nH + k;
                const int j1 = i == 0 ? fft::bit_reverse(i1, N) : i1;
                const int j2 = i == 0 ? fft::bit_reverse(i2, N) : i2;
                const long double a = 2.0L * (long double)fft::kPi * (long double)(k * nBlocks) / (long double)N;
                const float wr = (float)cosl(a), wi = (float)sinl(a);
                idx[(size_t)i * N + i1] = make_int2(j1, j2);
                w[(size_t)i * N + i1] = make_float2(fft::h16(wr), fft::h16(wi));
                idx[(size_t)i * N + i2] = make_int2(j1, j2);
                w[(size_t)i * N + i2] = make_float2(fft::h16(-wr), fft::h16(-wi));
            }
        }
    }
}

// oceanInit.frag: h(k,t) of the four grids, (h1 + i h2, h3 + i h4)
__global__ void fft_init_kernel(const float4* __restrict__ s12, const float4* __restrict__ s34, int N, float4 inv_grid,
                                float t, float4* __restrict__ out)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= N) return;
    const float Nf = (float)N;
    const float tx = (x + 0.5f) / Nf, ty = (y + 0.5f) / Nf;
    const float stx = floorf(tx * Nf) / Nf, sty = floorf(ty * Nf) / Nf;
    const float X = tx > 0.5f ? stx - 1.0f : stx, Y = ty > 0.5f ? sty - 1.0f : sty;
    const float r2 = 1.414213562f;
    const int xc = (N - x) & (N - 1), yc = (N - y) & (N - 1);   // the -k texel (repeat wrap)
    const float4 a = s12[(size_t)y * N + x], b = s34[(size_t)y * N + x];
    const float4 ac = s12[(size_t)yc * N + xc], bc = s34[(size_t)yc * N + xc];
    const float s0[4][2] = {{a.x * r2, a.y * r2}, {a.z * r2, a.w * r2}, {b.x * r2, b.y * r2}, {b.z * r2, b.w * r2}};
    const float sc[4][2] = {{ac.x * r2, ac.y * r2}, {ac.z * r2, ac.w * r2}, {bc.x * r2, bc.y * r2}, {bc.z * r2, bc.w * r2}};
    const float ig[4] = {inv_grid.x, inv_grid.y, inv_grid.z, inv_grid.w};
    float h[4][2];
    for (int g = 0; g < 4; ++g) {
        const float kx = X * ig[g], ky = Y * ig[g];
        const float K = sqrtf(kx * kx + ky * ky);
        const float w = sqrtf(9.81f * K * (1.0f + K * K / (370.0f * 370.0f)));
        const float c = cosf(w * t), s = sinf(w * t);
        h[g][0] = (s0[g][0] + sc[g][0]) * c - (s0[g][1] + sc[g][1]) * s;
        h[g][1] = (s0[g][0] - sc[g][0]) * s + (s0[g][1] - sc[g][1]) * c;
    }
    out[(size_t)y * N + x] = make_float4(h[0][0] + -h[1][1], h[0][1] + h[1][0], h[2][0] + -h[3][1], h[2][1] + h[3][0]);
}

// oceanFFTX.frag / oceanFFTY.frag: all passes of one line in shared memory
__global__ void fft_lines_kernel(float4* __restrict__ data, int N, int passes, const int2* __restrict__ idx,
                                 const float2* __restrict__ w, int vertical)
{
    extern __shared__ float4 line[];
    float4* a = line;
    float4* b = line + N;
    const int l = blockIdx.x;
    for (int p = threadIdx.x; p < N; p += blockDim.x)
        a[p] = data[vertical ? (size_t)p * N + l : (size_t)l * N + p];
    __syncthreads();
    for (int pass = 0; pass < passes; ++pass) {
        for (int p = threadIdx.x; p < N; p += blockDim.x) {
            const int2 j = idx[(size_t)pass * N + p];
            const float2 ww = w[(size_t)pass * N + p];
            const float4 i1 = a[j.x], i2 = a[j.y];
            const float r1x = ww.x * i2.x - ww.y * i2.y;
            const float r1y = ww.y * i2.x + ww.x * i2.y;
            const float r2x = ww.x * i2.z - ww.y * i2.w;
            const float r2y = ww.y * i2.z + ww.x * i2.w;
            b[p] = make_float4(i1.x + r1x, i1.y + r1y, i1.z + r2x, i1.w + r2y);
        }
        __syncthreads();
        float4* t = a;
        a = b;
        b = t;
    }
    for (int p = threadIdx.x; p < N; p += blockDim.x)
        data[vertical ? (size_t)p * N + l : (size_t)l * N + p] = a[p];
}

cudaError_t launch_fft_ocean(const float4* s12, const float4* s34, const int2* idx, const float2* w, int passes,
                             float4 inv_grid, float t, float4* out, cudaStream_t s)
{
    const int N = 1 << passes;
    const int tpb = N < 256 ? N : 256;
    fft_init_kernel<<<dim3((N + tpb - 1) / tpb, N), tpb, 0, s>>>(s12, s34, N, inv_grid, t, out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const size_t smem = 2 * (size_t)N * sizeof(float4);
    fft_lines_kernel<<<N, tpb, smem, s>>>(out, N, passes, idx, w, 0);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    fft_lines_kernel<<<N, tpb, smem, s>>>(out, N, passes, idx, w, 1);
    return cudaGetLastError();
}

}  // namespace sfh

extern "C" hydro_status hydro_debug_fft_ocean_tables(const hydro_fft_ocean_params* params, float* s12, float* s34,
                                                     int32_t* butterfly_index, float* butterfly_weight)
{
    if (params == nullptr || params->passes < 1 || params->passes > 12) return HYDRO_ERR_INVALID_ARG;
    const size_t N = (size_t)1 << params->passes;
    std::vector<float4> a, b;
    sfh::fft_ocean_spectrum(*params, a, b);
    if (s12 != nullptr) std::memcpy(s12, a.data(), N * N * sizeof(float4));
    if (s34 != nullptr) std::memcpy(s34, b.data(), N * N * sizeof(float4));
    std::vector<int2> idx;
    std::vector<float2> w;
    sfh::fft_ocean_butterfly((int)params->passes, idx, w);
    if (butterfly_index != nullptr) std::memcpy(butterfly_index, idx.data(), idx.size() * sizeof(int2));
    if (butterfly_weight != nullptr) std::memcpy(butterfly_weight, w.data(), w.size() * sizeof(float2));
    return HYDRO_OK;
}
