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
    double* partials;        // n_chunks * kPartialStride
    unsigned* counters;      // per body, zero between launches
    OceanDev ocean;
    SettingsDev st;
    int op;                  // OP_BODY / OP_SURFACE / OP_SUBMERGED
};

// The batched wrench step: one CTA per chunk; the last chunk of each body
// finalises it.  `cut64` selects FP64 cut points.
cudaError_t launch_chunks(const KParams& P, uint32_t n_chunks, int cut64, cudaStream_t s);

// Per-face surface-loop terms of one body for the parity tests: out holds
// n_faces * kQ floats in uploaded face order.
cudaError_t launch_face_terms(const TileDesc* tiles, uint32_t first_tile, uint32_t n_tiles,
                             const hydro_body* body, OceanDev ocean, SettingsDev st,
                             int cut64, float* out, cudaStream_t s);

// CorrectHydrodynamicForces on 4 vectors (io: Fdq, Tdq, Fdf, Tdf), one thread.
cudaError_t launch_correct(double density, double* io12, const double* Cd, const double* Cf,
                           const double* R_O, cudaStream_t s);

cudaError_t launch_fluid_position(OceanDev ocean, const double* aabb6, int* out, cudaStream_t s);

cudaError_t launch_depth(OceanDev ocean, const float* xyz, uint32_t n, float* out, cudaStream_t s);

}  // namespace sfh
