/*
 * fft_ocean.c -- CPU restatement of the reference's FFT ocean for checking
 * the library's kernels (TEST INFRASTRUCTURE ONLY).
 *
 * Restates OpenGLOcean::GenerateWavesSpectrum / spectrum / GetSpectrumSample
 * (Library/src/graphics/OpenGLOcean.cpp:929-1048) with the reference's LCG
 * (Library/include/utils/SystemUtil.hpp:208-218), the butterfly table of
 * ComputeButterflyLookupTable (:856-926), and the shader arithmetic of
 * oceanInit.frag and oceanFFTX/Y.frag (Library/shaders) in FP32 without
 * contraction.  The reference stores the spectrum and the butterfly table
 * in RGBA16F textures; both are rounded to binary16 here as there.
 *
 * Parity unpinned: the reference's GL pipeline cannot run on this machine or
 * on the GPU machine (no graphics stack), so this restatement is the only
 * oracle.  GLSL's cos/sin and the GL compiler's contraction are unknown;
 * cosf/sinf and separate multiply/add are used.
 */
#include "hydro_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static const double PI_D = 3.14159265358979323846;

/* round to the nearest binary16 value, ties to even (IEEE 754-2008) */
static float h16(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    const uint32_t sign = u & 0x80000000u;
    uint32_t a = u & 0x7fffffffu;
    float af;
    memcpy(&af, &a, 4);
    if (a >= 0x7f800000u) return f;
    float r;
    if (af >= 65520.0f) {
        r = INFINITY;
    } else if (af < 6.103515625e-05f) {                /* subnormal binary16: quantum 2^-24 */
        const float q = 5.9604644775390625e-08f;
        r = nearbyintf(af / q) * q;
    } else {
        int e;
        frexpf(af, &e);
        const float q = ldexpf(1.0f, e - 11);
        r = nearbyintf(af / q) * q;
    }
    uint32_t ru;
    memcpy(&ru, &r, 4);
    ru |= sign;
    memcpy(&r, &ru, 4);
    return r;
}

static float frandom_(int64_t* seed)
{
    *seed = (*seed * 1103515245 + 12345) & 0x7FFFFFFF;
    return (float)(*seed >> 7) / (float)(1 << 24);
}

static float sqr(float x) { return x * x; }

typedef struct { const hydro_fft_ocean_params* p; } spec_t;

static float omega_k(const spec_t* S, float k) { return (float)sqrt(9.81 * k * (1.0 + sqr(k / S->p->km))); }

static float spectrum(const spec_t* S, float kx, float ky)
{
    const hydro_fft_ocean_params* p = S->p;
    const float U10 = p->wind, Omega = p->omega;
    const float k = sqrtf(kx * kx + ky * ky);
    const float c = omega_k(S, k) / k;
    const float kp = (float)(9.81 * sqr(Omega / U10));
    const float cp = omega_k(S, kp) / kp;
    const float z0 = (float)(3.7e-5 * sqr(U10) / 9.81 * powf(U10 / cp, 0.9f));
    const float u_star = (float)(0.41 * U10 / log(10.0 / z0));
    const float Lpm = (float)exp(-5.0 / 4.0 * sqr(kp / k));
    const float gamma = Omega < 1.0f ? 1.7f : (float)(1.7 + 6.0 * logf(Omega));
    const float sigma = (float)(0.08 * (1.0 + 4.0 / powf(Omega, 3.0f)));
    const float Gamma = (float)exp(-1.0 / (2.0 * sqr(sigma)) * sqr((float)(sqrtf(k / kp) - 1.0)));
    const float Jp = powf(gamma, Gamma);
    const float Fp = (float)(Lpm * Jp * exp(-Omega / sqrt(10.0) * (sqrtf(k / kp) - 1.0)));
    const float alphap = (float)(0.006 * sqrtf(Omega));
    float Bl = (float)(0.5 * alphap * cp / c * Fp);
    const float alpham = (float)(0.01 * (u_star < p->cm ? 1.0 + logf(u_star / p->cm) : 1.0 + 3.0 * logf(u_star / p->cm)));
    const float Fm = (float)exp(-0.25 * sqr(k / p->km - 1.0f));
    float Bh = (float)(0.5 * alpham * p->cm / c * Fm);
    Bh *= Lpm;
    const float a0 = (float)(log(2.0) / 4.0);
    const float ap = 4.0f;
    const float am = (float)(0.13 * u_star / p->cm);
    const float Delta = tanhf(a0 + ap * powf(c / cp, 2.5f) + am * powf(p->cm / c, 2.5f));
    const float phi = atan2f(ky, kx);
    if (p->propagate) {
        if (kx < 0.0f) return 0.0f;
        Bl *= 2.0f;
        Bh *= 2.0f;
    }
    return (float)(p->amplitude * (Bl + Bh) * (1.0 + Delta * cos(2.0 * phi)) / (2.0 * PI_D * sqr(sqr(k))));
}

static void sample(const spec_t* S, int i, int j, float L, float kMin, int64_t* seed, float* out)
{
    const float dk = (float)(2.0 * PI_D / L);
    const float kx = i * dk, ky = j * dk;
    if (fabsf(kx) < kMin && fabsf(ky) < kMin) { out[0] = 0.0f; out[1] = 0.0f; return; }
    const float s = spectrum(S, kx, ky);
    const float h = sqrtf((float)(s / 2.0)) * dk;
    const float phi = (float)(frandom_(seed) * 2.0 * PI_D);
    out[0] = (float)(h * cosf(phi));
    out[1] = (float)(h * sinf(phi));
}

static int bit_reverse(int i, int N)
{
    int sum = 0, w = 1;
    for (int m = N / 2; m != 0; m /= 2) { sum += ((i & m) > m - 1) * w; w *= 2; }
    return sum;
}

static void fft_ocean_impl(const hydro_fft_ocean_params* p, float t, float* out, int do_fft)
{
    const int N = 1 << p->passes, P = (int)p->passes;
    const size_t nn = (size_t)N * N;
    float* s12 = malloc(nn * 4 * sizeof(float));
    float* s34 = malloc(nn * 4 * sizeof(float));
    float* buf = malloc(nn * 4 * sizeof(float));
    float* tmp = malloc((size_t)N * 4 * sizeof(float));
    float* tmp2 = malloc((size_t)N * 4 * sizeof(float));
    int* bj = malloc((size_t)N * P * 2 * sizeof(int));
    float* bw = malloc((size_t)N * P * 2 * sizeof(float));
    /* spectrum (seed 1234) */
    spec_t S = {p};
    int64_t seed = 1234;
    const float* g = p->grid_sizes;
    const float kmin[4] = {(float)(PI_D / g[0]), (float)(PI_D * N / g[0]), (float)(PI_D * N / g[1]),
                           (float)(PI_D * N / g[2])};
    for (int y = 0; y < N; ++y)
        for (int x = 0; x < N; ++x) {
            const int i = x >= N / 2 ? x - N : x, j = y >= N / 2 ? y - N : y;
            float r[8];
            for (int q = 0; q < 4; ++q) sample(&S, i, j, g[q], kmin[q], &seed, r + 2 * q);
            for (int q = 0; q < 4; ++q) {
                s12[((size_t)y * N + x) * 4 + q] = h16(r[q]);
                s34[((size_t)y * N + x) * 4 + q] = h16(r[4 + q]);
            }
        }
    /* butterfly table */
    for (int i = 0; i < P; ++i) {
        const int nBlocks = 1 << (P - 1 - i), nH = 1 << i;
        for (int j = 0; j < nBlocks; ++j)
            for (int k = 0; k < nH; ++k) {
                const int i1 = j * nH * 2 + k, i2 = j * nH * 2 + nH + k;
                const int j1 = i == 0 ? bit_reverse(i1, N) : i1, j2 = i == 0 ? bit_reverse(i2, N) : i2;
                const long double a = 2.0L * (long double)PI_D * (long double)(k * nBlocks) / (long double)N;
                const float wr = (float)cosl(a), wi = (float)sinl(a);
                const size_t o1 = (size_t)i * N + i1, o2 = (size_t)i * N + i2;
                bj[2 * o1] = j1; bj[2 * o1 + 1] = j2; bw[2 * o1] = h16(wr); bw[2 * o1 + 1] = h16(wi);
                bj[2 * o2] = j1; bj[2 * o2 + 1] = j2; bw[2 * o2] = h16(-wr); bw[2 * o2 + 1] = h16(-wi);
            }
    }
    /* oceanInit.frag */
    float ig[4];
    for (int q = 0; q < 4; ++q) ig[q] = (float)(2.0 * PI_D * (float)N / g[q]);
    const float Nf = (float)N, r2 = 1.414213562f;
    for (int y = 0; y < N; ++y)
        for (int x = 0; x < N; ++x) {
            const float tx = (x + 0.5f) / Nf, ty = (y + 0.5f) / Nf;
            const float stx = floorf(tx * Nf) / Nf, sty = floorf(ty * Nf) / Nf;
            const float X = tx > 0.5f ? stx - 1.0f : stx, Y = ty > 0.5f ? sty - 1.0f : sty;
            const int xc = (N - x) & (N - 1), yc = (N - y) & (N - 1);
            const float* a = s12 + ((size_t)y * N + x) * 4;
            const float* b = s34 + ((size_t)y * N + x) * 4;
            const float* ac = s12 + ((size_t)yc * N + xc) * 4;
            const float* bc = s34 + ((size_t)yc * N + xc) * 4;
            const float s0[4][2] = {{a[0] * r2, a[1] * r2}, {a[2] * r2, a[3] * r2}, {b[0] * r2, b[1] * r2}, {b[2] * r2, b[3] * r2}};
            const float sc[4][2] = {{ac[0] * r2, ac[1] * r2}, {ac[2] * r2, ac[3] * r2}, {bc[0] * r2, bc[1] * r2}, {bc[2] * r2, bc[3] * r2}};
            float h[4][2];
            for (int q = 0; q < 4; ++q) {
                const float kx = X * ig[q], ky = Y * ig[q];
                const float K = sqrtf(kx * kx + ky * ky);
                const float w = sqrtf(9.81f * K * (1.0f + K * K / (370.0f * 370.0f)));
                const float c = cosf(w * t), s = sinf(w * t);
                h[q][0] = (s0[q][0] + sc[q][0]) * c - (s0[q][1] + sc[q][1]) * s;
                h[q][1] = (s0[q][0] - sc[q][0]) * s + (s0[q][1] - sc[q][1]) * c;
            }
            float* o = buf + ((size_t)y * N + x) * 4;
            o[0] = h[0][0] + -h[1][1]; o[1] = h[0][1] + h[1][0];
            o[2] = h[2][0] + -h[3][1]; o[3] = h[2][1] + h[3][0];
        }
    /* oceanFFTX.frag then oceanFFTY.frag, all passes per line */
    for (int dir = 0; dir < 2 * do_fft; ++dir)
        for (int l = 0; l < N; ++l) {
            for (int e = 0; e < N; ++e) {
                const size_t at = dir ? ((size_t)e * N + l) : ((size_t)l * N + e);
                memcpy(tmp + 4 * e, buf + 4 * at, 4 * sizeof(float));
            }
            for (int pass = 0; pass < P; ++pass) {
                for (int e = 0; e < N; ++e) {
                    const size_t o = (size_t)pass * N + e;
                    const float* i1 = tmp + 4 * bj[2 * o];
                    const float* i2 = tmp + 4 * bj[2 * o + 1];
                    const float wx = bw[2 * o], wy = bw[2 * o + 1];
                    const float r1x = wx * i2[0] - wy * i2[1];
                    const float r1y = wy * i2[0] + wx * i2[1];
                    const float r2x = wx * i2[2] - wy * i2[3];
                    const float r2y = wy * i2[2] + wx * i2[3];
                    tmp2[4 * e + 0] = i1[0] + r1x; tmp2[4 * e + 1] = i1[1] + r1y;
                    tmp2[4 * e + 2] = i1[2] + r2x; tmp2[4 * e + 3] = i1[3] + r2y;
                }
                float* sw = tmp; tmp = tmp2; tmp2 = sw;
            }
            for (int e = 0; e < N; ++e) {
                const size_t at = dir ? ((size_t)e * N + l) : ((size_t)l * N + e);
                memcpy(buf + 4 * at, tmp + 4 * e, 4 * sizeof(float));
            }
        }
    memcpy(out, buf, nn * 4 * sizeof(float));
    free(s12); free(s34); free(buf); free(tmp); free(tmp2); free(bj); free(bw);
}

void oracle_fft_ocean(const hydro_fft_ocean_params* p, float t, float* out) { fft_ocean_impl(p, t, out, 1); }

/* The h(k,t) field of oceanInit.frag alone (before the FFTs), for a DFT check. */
void oracle_fft_ocean_init_only(const hydro_fft_ocean_params* p, float t, float* out) { fft_ocean_impl(p, t, out, 0); }
