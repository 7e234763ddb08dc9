/*
 * hydro_oracle.h -- CPU oracle for the hydrodynamic wrench path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a clean-room CPU restatement of
 * Stonefish's SolidEntity hydrodynamics (Library/src/entities/SolidEntity.cpp
 * :1239-1850), Ocean depth/current queries (Library/src/entities/forcefields/
 * Ocean.cpp:149-201, Uniform.cpp:56-59, Jet.cpp:59-80, Pipe.cpp:57-79) and the
 * wave lookup (Library/src/graphics/OpenGLRealOcean.cpp:282-331).  Only the
 * tests, the smoke check and the CPU-baseline leg of the benchmark use it;
 * the GPU library never links or calls it.
 *
 * Parity unpinned: the reference cannot be compiled here (glm, SDL2, GL are
 * absent) and its own tests hold no active golden vectors for this path
 * (Tests/FluidDynamicsTest/FluidDynamicsTestManager.cpp:168-249 is commented
 * out).  The oracle is pinned instead by analytic known-answer tests and by
 * agreement between its FP32 and FP64 variants.  The vector arithmetic
 * restates glm >= 0.9.9 (not vendored in the reference): dot = (xx'+yy')+zz',
 * cross = (y z'-y' z, z x'-z' x, x y'-x' y), mat4*vec4 =
 * (c0 x + c1 y) + (c2 z + c3 w), vec/scalar = per-component division.
 *
 * Variants (the `variant` argument):
 *   ORACLE_REF32      the reference's arithmetic: FP32 faces in glm order,
 *                     FP32 cut points, FP32 serial sums, FP64 boundary;
 *   ORACLE_REF64      the same algorithm entirely in FP64 (no FP32 casts of
 *                     transforms, velocities or depths);
 *   ORACLE_MIRROR64   FP32 faces as REF32 but cut points in FP64 and sums in
 *                     FP64: the arithmetic of the GPU kernel's HYDRO_CUT_FP64
 *                     mode;
 *   ORACLE_MIRROR32   FP32 faces and cut points as REF32, sums in FP64: the
 *                     arithmetic of the GPU kernel's default HYDRO_CUT_FP32
 *                     mode.
 */
#ifndef HYDRO_ORACLE_H
#define HYDRO_ORACLE_H

#include <stddef.h>
#include <stdint.h>
#include "../include/stonefish_hydro.h"

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_REF32 = 0, ORACLE_REF64 = 1, ORACLE_MIRROR64 = 2, ORACLE_MIRROR32 = 3 };

typedef struct oracle_mesh {
    const float* xyz;        /* vertex positions, stride `stride` floats */
    uint32_t stride;         /* floats per vertex (3 for packed xyz) */
    uint32_t n_vertices;
    const uint32_t* idx;     /* 3 per face */
    uint32_t n_faces;
} oracle_mesh;

typedef struct oracle_waves {
    const float* data;       /* N*N*channels, NULL = no grid */
    uint32_t size;
    uint32_t channels;
    uint32_t n_layers;
    uint32_t layer_channel[HYDRO_MAX_WAVE_LAYERS];
    float layer_grid_size[HYDRO_MAX_WAVE_LAYERS];
} oracle_waves;

/* Per-face contributions of one face, as the GPU debug entry point writes
 * them: the 23 quantities the face adds to the body sums, in FP32. */
enum {
    ORACLE_T_FB = 0, ORACLE_T_TB = 3, ORACLE_T_FDQ = 6, ORACLE_T_TDQ = 9,
    ORACLE_T_FDF = 12, ORACLE_T_TDF = 15, ORACLE_T_SWET = 18, ORACLE_T_V6 = 19,
    ORACLE_T_CB6 = 20, ORACLE_T_N = 23
};

float oracle_depth(int variant, const hydro_ocean* ocean, const oracle_waves* waves,
                   float x, float y, float z);
double oracle_depth64(const hydro_ocean* ocean, const oracle_waves* waves,
                      double x, double y, double z);

int oracle_fluid_position(const hydro_ocean* ocean, const oracle_waves* waves,
                          const double aabb_min[3], const double aabb_max[3]);

void oracle_surface_forces(int variant, const hydro_settings* settings,
                           const oracle_mesh* mesh, const hydro_ocean* ocean,
                           const oracle_waves* waves, const hydro_transform* T_CG,
                           const hydro_transform* T_C, const double v[3],
                           const double omega[3], double Fb[3], double Tb[3],
                           double Fdq[3], double Tdq[3], double Fdf[3], double Tdf[3],
                           double* Swet, double* Vsub);

void oracle_submerged_forces(int variant, const oracle_mesh* mesh,
                             const hydro_ocean* ocean, const hydro_transform* T_CG,
                             const hydro_transform* T_C, const double v[3],
                             const double omega[3], double Fdq[3], double Tdq[3],
                             double Fdf[3], double Tdf[3]);

void oracle_correct_forces(const hydro_ocean* ocean, double Fdq[3], double Tdq[3],
                           double Fdf[3], double Tdf[3], const double Cd[3],
                           const double Cf[3], const double R_O[9]);

void oracle_body_forces(int variant, const hydro_body* body, const oracle_mesh* mesh,
                        const hydro_ocean* ocean, const oracle_waves* waves,
                        const hydro_settings* settings, hydro_wrench* io);

/* Per-face terms of the surface (crossing) loop: out has n_faces*ORACLE_T_N
 * floats; faces that contribute nothing are all zero.  Variants REF32,
 * MIRROR64 and MIRROR32 only. */
void oracle_surface_face_terms(int variant, const hydro_settings* settings,
                               const oracle_mesh* mesh, const hydro_ocean* ocean,
                               const oracle_waves* waves, const hydro_transform* T_CG,
                               const hydro_transform* T_C, const double v[3],
                               const double omega[3], float* out);

/* All bodies, one task per body on `threads` worker threads (the reference's
 * ThreadPool fan-out, SimulationManager.cpp:1620-1655).  meshes[] is indexed
 * by hydro_body.mesh.  Returns the wall time of the batch in seconds. */
double oracle_batch(int variant, int threads, const hydro_body* bodies,
                    uint32_t n_bodies, const oracle_mesh* meshes, uint32_t n_meshes,
                    const hydro_ocean* ocean, const oracle_waves* waves,
                    const hydro_settings* settings, hydro_wrench* io);

int oracle_hardware_threads(void);

/* ComputePhysicalProperties (GeometryFileUtil.cpp:335-566): out = mass,
 * volume, surface, CG[3], trace of the inertia tensor about the CG. */
void oracle_mesh_properties(const oracle_mesh* mesh, double thickness, double density, double out[7]);

/* The reference's FFT ocean at time t (oracle/fft_ocean.c): N x N x 4 heights. */
void oracle_fft_ocean(const hydro_fft_ocean_params* params, float t, float* out);
void oracle_fft_ocean_init_only(const hydro_fft_ocean_params* params, float t, float* out);

/* CableEntity::ComputeHydrodynamicForces (Library/src/entities/CableEntity.cpp:240-376). */
void oracle_cable_forces(const hydro_cable* cables, uint32_t n_cables, const double* x, const double* v,
                         uint32_t n_nodes_total, const hydro_ocean* ocean, const oracle_waves* waves,
                         const hydro_settings* settings, hydro_cable_node_forces* out);

/* Compound::ComputeHydrodynamicForces (Library/src/entities/solids/Compound.cpp:291-436):
 * part_meshes[i] is part i's mesh (NULL = nullptr). */
void oracle_compound_forces(int variant, const hydro_body* compound, const hydro_compound_part* parts,
                            uint32_t n_parts, const oracle_mesh* const* part_meshes,
                            const hydro_ocean* ocean, const oracle_waves* waves,
                            const hydro_settings* settings, hydro_wrench* io);

/* SolidEntity::ComputeAerodynamicForces (static form, SolidEntity.cpp:1865-1923)
 * and CorrectAerodynamicForces (:1925-1956). */
void oracle_aero_forces(int variant, const oracle_mesh* mesh, const hydro_atmosphere* atm,
                        const hydro_transform* T_CG, const hydro_transform* T_C, const double v[3],
                        const double omega[3], double Fda[3], double Tda[3]);
void oracle_aero_correct(const hydro_aero_params* params, double Fda[3], double Tda[3]);

#ifdef __cplusplus
}
#endif

#endif
