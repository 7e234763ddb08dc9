// hydro_internal.h -- launch interface between the C ABI (hydro_api.cu) and
// the kernels (hydro_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "hydro_device.cuh"

namespace sfh {

struct KParams {
    const ChunkDesc* chunks;
    const BodyInfo* binfo;
    const TileDesc* tiles;
    const hydro_body* bodies;
    hydro_wrench* io;
    BodyParams* bparams;     // per body, written by the prep kernel
    double* partials;        // n_chunks * kPartialStride
    unsigned* err;           // per-launch error word (bit 0: a bounded wait timed out)
    unsigned* work;          // kClaimClasses claim counters of the persistent kernel (reset by prep)
    unsigned* n_listed;      // kClaimClasses counts of listed chunks (atomicAdd in prep, reset by finalize)
    const uint32_t* n_active;  // optional (device): only bodies [0, *n_active) are evaluated
    hydro_aero_wrench* aero_io;            // OP_AERO / OP_AERO_BODY outputs
    const hydro_aero_params* aero_params;  // OP_AERO_BODY correction inputs
    ActiveChunk* active;     // chunks with a face loop, n_chunks entries of room
    uint32_t n_bodies;
    uint32_t n_chunks;
    OceanDev ocean;
    SettingsDev st;
    int op;                  // OP_BODY / OP_SURFACE / OP_SUBMERGED
    int frame;               // HYDRO_FRAME_WORLD / HYDRO_FRAME_CENTRED (body ops)
    // The list of active chunks is kept in claim classes by tile count,
    // largest first: class c (chunks of kMaxTilesPerChunk - 2c or one tile
    // fewer) owns active[class_start[c], class_start[c + 1]).
    uint32_t class_start[kClaimClasses + 1];
};

// Claim class of a chunk of n_tiles tiles (largest chunks first), and the
// class regions of a work list (exclusive prefix sums of the class sizes).
__host__ __device__ inline uint32_t claim_class(uint32_t n_tiles)
{
    const uint32_t t = n_tiles < 1u ? 1u : (n_tiles > (uint32_t)kMaxTilesPerChunk ? (uint32_t)kMaxTilesPerChunk : n_tiles);
    return ((uint32_t)kMaxTilesPerChunk - t) / 2u;
}

inline void claim_class_starts(const ChunkDesc* chunks, size_t n, uint32_t* starts)
{
    uint32_t count[kClaimClasses] = {};
    for (size_t i = 0; i < n; ++i) ++count[claim_class(chunks[i].n_tiles)];
    starts[0] = 0;
    for (int c = 0; c < kClaimClasses; ++c) starts[c + 1] = starts[c] + count[c];
}

// Compounds: the KParams bodies are the parts; these describe the grouping.
struct CompoundInfo {
    uint32_t first_part;
    uint32_t n_parts;
};

struct CompoundParams {
    const hydro_body* compounds;         // n_compounds
    const hydro_compound_part* parts;    // one per KParams body
    const CompoundInfo* cinfo;           // n_compounds
    const uint32_t* part_compound;       // part -> compound
    hydro_wrench* io;                    // per compound, in-out
    uint32_t n_compounds;
};

// Launch shape of the persistent chunk kernel.
struct LaunchShape {
    int grid;                // CTAs (a multiple of the SM count when work allows)
    int ctas_per_sm;
};

// Shared-memory bytes of the chunk kernel.
size_t chunk_kernel_smem();

// Resident CTAs per SM that the chunk-kernel variant compiled for
// `ctas_per_sm` (1 or 2) reaches (0 on error); aero selects the variant of
// the aerodynamic launches, field the one with jet or pipe currents.
int chunk_kernel_occupancy(int cut64, int waves, int ctas_per_sm, int aero, int field);

// The batched wrench step: prep (per body), persistent chunk kernel with a
// TMA-fed tile pipeline, finalise (per body).  `cut64` selects FP64 cut
// points.  Returns the number of kernels launched in *launches.
// ev (optional): four events recorded before prep, after prep, after the
// chunk kernel and after finalize.
cudaError_t launch_step(const KParams& P, LaunchShape shape, int cut64, cudaStream_t s,
                        uint32_t* launches, cudaEvent_t* ev = nullptr);

// Per-face surface-loop terms of one body for the parity tests: out holds
// n_faces * kQ floats in uploaded face order.  packed = 1 sends pairs of
// fully submerged faces through the packed FP32 path, 0 uses the scalar
// path for every face.
cudaError_t launch_face_terms(const TileDesc* tiles, uint32_t first_tile, uint32_t n_tiles,
                             const hydro_body* body, OceanDev ocean, SettingsDev st, int frame,
                             int cut64, int packed, float* out, cudaStream_t s);

// Outlines of the submerged face parts of one body's surface loop (the
// reference's DEBUG_HYDRO points): out holds n_faces * 13 floats in uploaded
// face order (count 0, 3 or 4, then four corners x, y, z), world frame.
cudaError_t launch_outline(const TileDesc* tiles, uint32_t first_tile, uint32_t n_tiles, const hydro_body* body,
                           OceanDev ocean, SettingsDev st, int cut64, float* out, cudaStream_t s);

// CorrectHydrodynamicForces on 4 vectors (io: Fdq, Tdq, Fdf, Tdf), one thread.
cudaError_t launch_correct(double density, double* io12, const double* Cd, const double* Cf,
                           const double* R_O, cudaStream_t s);

cudaError_t launch_fluid_position(OceanDev ocean, const double* aabb6, int* out, cudaStream_t s);

// Counts mismatches of the FMA-corrected divisions against IEEE division:
// counts[0] a/3 over all floats, counts[1] and counts[2] random pairs.
cudaError_t launch_division_check(uint64_t n_pairs, uint64_t seed, unsigned long long* counts,
                                  cudaStream_t s);

// Counts mismatches of the packed f32x2 ops against scalar IEEE ops in
// counts[3..6] (mul, add, sub, fma); ex receives one failing case per op.
cudaError_t launch_packed_check(uint64_t n, uint64_t seed, unsigned long long* counts, float* ex,
                                cudaStream_t s);

// A 1-CTA wait on an mbarrier that is never completed, bounded by limit_ns:
// writes HYDRO_ERR_TIMEOUT (or 0) to *status.
cudaError_t launch_wait_timeout(uint64_t limit_ns, int* status, cudaStream_t s);

cudaError_t launch_depth(OceanDev ocean, const float* xyz, uint32_t n, float* out, cudaStream_t s);

// ----------------------------------------------------- surrogate kernels
// C[M,N] = A[M,K] * B[K,N] (BF16 row-major, FP32 accumulate) with epilogue
// epi: 0 z = C; 1 z = C + bias, y = bf16(silu(z)); 2 z = C + bias;
// 3 y = bf16(C * silu'(zprev)).  M, N multiples of 64, K of 32.
// An EPI_F32 product with few output tiles and a long K runs split along K
// when `ws` holds gemm_splits(...) * M * N floats: each slice writes a
// partial product there, and a second kernel sums them in slice order.
int gemm_splits(int epi, int M, int N, int K);
cudaError_t launch_gemm(int epi, const void* A, int lda, const void* B, int ldb, int M, int N, int K,
                        float* z, void* y, const float* bias, const float* zprev, int ldc,
                        cudaStream_t s, float* ws = nullptr, size_t ws_floats = 0);
cudaError_t launch_transpose(const void* src, void* dst, int rows, int cols, cudaStream_t s);
cudaError_t launch_mse_grad(const float* z, const float* t, int rows, int ld, int n_out, const float* tmean,
                            const float* tistd, void* dz, double* loss, cudaStream_t s);
// Column sums; with ws holding colsum_slabs(rows) * cols floats, in two
// stages (row slabs, then the slabs in order).
int colsum_slabs(int rows);
cudaError_t launch_colsum(const void* g, int rows, int cols, float* out, cudaStream_t s, float* ws = nullptr,
                          size_t ws_floats = 0);
cudaError_t launch_adamw(float* w, float* m, float* v, const float* grad, int rows, int cols, int ldg,
                         float lr, float b1, float b2, float eps, float wd, int step, void* w16,
                         void* wt16, cudaStream_t s);
cudaError_t launch_to_bf16(const float* x, int rows, int n_in, int ld, const float* mean, const float* istd,
                           void* y, cudaStream_t s);
cudaError_t launch_features(const hydro_body* bodies, uint32_t n, OceanDev o, float* f, cudaStream_t s);
cudaError_t launch_gate(const float* f, uint32_t n, const float* lo, const float* hi, const float* mean,
                        const float* P, float thresh, uint8_t* mask, cudaStream_t s);
cudaError_t launch_route(const hydro_body* bodies, const uint8_t* mask, uint32_t n, uint32_t* counts,
                         hydro_body* packed, int32_t* pos, uint32_t* n_packed, hydro_wrench* exact,
                         cudaStream_t s);
cudaError_t launch_merge(const hydro_body* bodies, const float* z, int ld, const int32_t* pos,
                         const hydro_wrench* exact, uint32_t n, float* out, cudaStream_t s);
cudaError_t launch_wrench_body(const hydro_body* bodies, const hydro_wrench* w, uint32_t n, float* out,
                               cudaStream_t s);
cudaError_t launch_gate_inside(const hydro_body* bodies, uint32_t n, OceanDev o, uint8_t* mask, cudaStream_t s);
cudaError_t launch_ensemble(float* za, const float* zb, int ld, uint32_t n, float inv_fs, float inv_ts, float tau,
                            uint8_t* mask, cudaStream_t s);
cudaError_t launch_audit_pick(uint8_t* mask, uint32_t n, uint32_t stride, uint32_t phase, uint32_t k, int32_t* idx,
                              cudaStream_t s);
cudaError_t launch_audit_error(const hydro_body* bodies, const float* z, int ld, const int32_t* pos,
                               const hydro_wrench* exact, const int32_t* idx, uint32_t k, float inv_fs,
                               float inv_ts, float* err, cudaStream_t s);

cudaError_t launch_rigid_step(hydro_rigid_state* states, hydro_body* bodies, const hydro_wrench* exact,
                              const float* body_wrench, uint32_t n, double dt, double gravity, cudaStream_t s);
cudaError_t launch_rigid_write_bodies(const hydro_rigid_state* states, hydro_body* bodies, uint32_t n,
                                      cudaStream_t s);

cudaError_t launch_pack_sw128(const void* src, int rows, int K, int ld, int kpad, void* dst, cudaStream_t s);
size_t mlp_tc_image_bytes();
cudaError_t launch_mlp_tc(const float* feats, uint32_t n, const float* fmean, const float* fistd,
                          const void* wimg, const float* b0, const float* b1, const float* b2, const float* b3,
                          float* out, unsigned* err, cudaStream_t s);

cudaError_t launch_compound_step(const KParams& P, const CompoundParams& C, LaunchShape shape, int cut64,
                                 cudaStream_t s, uint32_t* launches);
cudaError_t launch_cable(const hydro_cable* cables, uint32_t n_cables, uint32_t n_nodes_total, const double* x,
                         const double* v, OceanDev o, SettingsDev st, double* seg, hydro_cable_node_forces* out,
                         unsigned* bad, cudaStream_t s);
cudaError_t launch_fft_ocean(const float4* s12, const float4* s34, const int2* idx, const float2* w, int passes,
                             float4 inv_grid, float t, float4* out, cudaStream_t s);
cudaError_t launch_mesh_props(const TileDesc* tiles, uint32_t first_tile, uint32_t n_tiles, int pass, double thickness,
                              double3 cg, double* out, cudaStream_t s);
cudaError_t launch_aero_correct(const hydro_aero_params* p, double* io6, cudaStream_t s);

}  // namespace sfh
