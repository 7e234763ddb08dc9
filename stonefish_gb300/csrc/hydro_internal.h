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
    unsigned* work;          // chunk counter of the persistent kernel
    uint8_t* chunk_active;   // per chunk: 1 when its body runs a face loop
    uint32_t n_bodies;
    uint32_t n_chunks;
    OceanDev ocean;
    SettingsDev st;
    int op;                  // OP_BODY / OP_SURFACE / OP_SUBMERGED
};

// Launch shape of the persistent chunk kernel.
struct LaunchShape {
    int grid;                // CTAs (a multiple of the SM count when work allows)
    int ctas_per_sm;
};

// Shared-memory bytes of the chunk kernel.
size_t chunk_kernel_smem();

// Resident CTAs per SM that the chunk-kernel variant compiled for
// `ctas_per_sm` (1 or 2) reaches (0 on error).
int chunk_kernel_occupancy(int cut64, int waves, int ctas_per_sm);

// The batched wrench step: prep (per body), persistent chunk kernel with a
// TMA-fed tile pipeline, finalise (per body).  `cut64` selects FP64 cut
// points.  Returns the number of kernels launched in *launches.
cudaError_t launch_step(const KParams& P, LaunchShape shape, int cut64, cudaStream_t s,
                        uint32_t* launches);

// Per-face surface-loop terms of one body for the parity tests: out holds
// n_faces * kQ floats in uploaded face order.  packed = 1 sends pairs of
// fully submerged faces through the packed FP32 path, 0 uses the scalar
// path for every face.
cudaError_t launch_face_terms(const TileDesc* tiles, uint32_t first_tile, uint32_t n_tiles,
                             const hydro_body* body, OceanDev ocean, SettingsDev st,
                             int cut64, int packed, float* out, cudaStream_t s);

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

}  // namespace sfh
