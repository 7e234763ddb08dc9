/*
 * stonefish_hydro.h -- C ABI of the GB300 geometry-based hydrodynamics path.
 *
 * The path replaced here is Stonefish's per-triangle hydrodynamic force
 * integration (Library/src/entities/SolidEntity.cpp:1239-1850): every face of
 * a body's physics mesh is clipped against the ocean surface, buoyancy,
 * pressure (form) drag and skin friction are integrated over the submerged
 * part, and the result is reduced to force/torque pairs at the body's centre
 * of gravity.  All entry points compute on the GPU (sm_103a); none falls back
 * to the CPU.
 *
 * Conventions (same as the reference):
 *   - world frame is NED: z points down, the flat ocean surface is z = 0 and
 *     depth = z (Ocean.cpp:149-168);
 *   - transforms are rigid: basis is row-major R[r][c] (btMatrix3x3 rows),
 *     origin is the translation; a point p maps to R*p + origin
 *     (btTransform::operator*, 3rdparty/LinearMath/btTransform.h:91-100);
 *   - every double is a btScalar (BT_USE_DOUBLE_PRECISION, CMakeLists.txt:53);
 *     face arithmetic runs in FP32 like the reference's glm code.
 *
 * Outputs follow the reference's in-out rules exactly: an OUTSIDE body gets
 * zeros, a CROSSING body whose submerged volume is tiny keeps its previous
 * Fb/Tb/Vsub, an INSIDE body keeps its previous Vsub, and a body whose physics
 * mode is neither FLOATING nor SUBMERGED is left untouched.
 *
 * Thread safety: one hydro_ctx may be used from several host threads; calls
 * on the same context are serialised internally.  No call aborts the process
 * and no C++ exception crosses this boundary.
 */
#ifndef STONEFISH_HYDRO_H
#define STONEFISH_HYDRO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HYDRO_ABI_VERSION 1

/* ---------------------------------------------------------------- status */
typedef enum hydro_status {
    HYDRO_OK = 0,
    HYDRO_ERR_INVALID_ARG = 1,  /* null pointer, zero/oversized count, bad enum */
    HYDRO_ERR_OOM = 2,          /* device or host allocation failed */
    HYDRO_ERR_TIMEOUT = 3,      /* a bounded device-side wait ran out */
    HYDRO_ERR_DEVICE = 4,       /* CUDA runtime error (see hydro_last_error) */
    HYDRO_ERR_NOT_FOUND = 5,    /* unknown mesh / batch handle */
    HYDRO_ERR_INDEX_RANGE = 6,  /* a face index >= vertex count */
    HYDRO_ERR_UNSUPPORTED = 7,  /* feature not available in this build */
    HYDRO_ERR_MISMATCH = 8      /* body table does not match its batch */
} hydro_status;

/* ------------------------------------------------------------ enumerations */
/* PhysicsMode, Library/include/entities/Entity.h:57 */
enum {
    HYDRO_MODE_DISABLED = 0,
    HYDRO_MODE_SURFACE = 1,
    HYDRO_MODE_FLOATING = 2,
    HYDRO_MODE_SUBMERGED = 3,
    HYDRO_MODE_AERODYNAMIC = 4
};

/* BodyFluidPosition, Library/include/entities/SolidEntity.h:41 */
enum {
    HYDRO_INSIDE = 0,
    HYDRO_OUTSIDE = 1,
    HYDRO_CROSSING_SURFACE = 2,
    HYDRO_SKIPPED = -1          /* mode gate: outputs untouched */
};

/* VelocityFieldType (Uniform.cpp, Jet.cpp, Pipe.cpp) */
enum {
    HYDRO_CURRENT_UNIFORM = 0,
    HYDRO_CURRENT_JET = 1,
    HYDRO_CURRENT_PIPE = 2
};

/* Precision of the waterline cut points (faces that straddle the surface).
 * HYDRO_CUT_FP32 (default) is the reference's own arithmetic: every face's
 * contribution equals the FP32 glm evaluation bit for bit.  HYDRO_CUT_FP64
 * interpolates the cut points in FP64 and rounds them once; GB300's FP64
 * rate makes that path several times slower for no measurable gain in the
 * wrench error against an all-FP64 evaluation. */
enum {
    HYDRO_CUT_FP64 = 0,
    HYDRO_CUT_FP32 = 1
};

/* Frame of the FP32 face arithmetic (hydro_set_frame).
 * HYDRO_FRAME_WORLD (default) is the reference's: the body's transforms are
 * cast to FP32 as they are (glMatrixFromTransform, OpenGLDataStructs.cpp:
 * 148-165) and every face is evaluated in world coordinates, so each face's
 * terms are the reference's bits.  HYDRO_FRAME_CENTRED subtracts the body's
 * CG x and y (rounded to FP32) in FP64 before the cast and evaluates the
 * faces in that horizontally centred frame; wave lookups and
 * position-dependent currents add the offset back.  The physics is the same
 * (the ocean is level and uniform in x and y), but the FP32 rounding no
 * longer grows with the body's distance from the world origin: on the
 * 4096-body mixed batch, whose bodies lie up to 50 m from it, the pair-scaled
 * error against an all-FP64 evaluation drops from a median of 1.0e-6 and a
 * 99th percentile of 3.5e-5 to 6e-8 and 2.6e-6.  The fluid position, the
 * submerged loop's branches and the outputs' meaning are unchanged.  Applies
 * to the body entry points (batches, single bodies, the allocation-free
 * step, aerodynamics); compounds and cables keep the world frame. */
enum {
    HYDRO_FRAME_WORLD = 0,
    HYDRO_FRAME_CENTRED = 1
};

#define HYDRO_MAX_CURRENTS 8
#define HYDRO_MAX_WAVE_LAYERS 4
#define HYDRO_NO_MESH 0xFFFFFFFFu   /* stands for the reference's mesh == nullptr */
/* Faces per mesh tile: work chunks (hydro_config.tile_faces, the chunk_faces
 * of hydro_batch_create_ex and of the autotuner) are whole tiles. */
#define HYDRO_TILE_FACES 448

typedef uint32_t hydro_mesh_id;
typedef struct hydro_ctx hydro_ctx;
typedef struct hydro_batch hydro_batch;

/* ------------------------------------------------------------------ types */
/* btTransform: basis rows then origin. */
typedef struct hydro_transform {
    double basis[9];
    double origin[3];
} hydro_transform;

/* HydrodynamicsSettings, Library/include/entities/forcefields/Ocean.h:36-40 */
typedef struct hydro_settings {
    int32_t damping_forces;      /* dampingForces */
    int32_t realistic_buoyancy;  /* reallisticBuoyancy */
} hydro_settings;

/* One VelocityField.  Fields used per type:
 *   UNIFORM: vel                         (Uniform.cpp:56-59)
 *   JET:     point=c, dir=n, radius=r, speed=vout              (Jet.cpp:59-80)
 *   PIPE:    point=p1, dir=n, radius=r1, radius2=r2, length=l,
 *            speed=vin, gamma                                  (Pipe.cpp:57-79) */
typedef struct hydro_current {
    int32_t type;
    int32_t enabled;             /* VelocityField::isEnabled() */
    double vel[3];
    double point[3];
    double dir[3];
    double radius;
    double radius2;
    double length;
    double speed;
    double gamma;
} hydro_current;

/* The Ocean as seen by the hydrodynamics path. */
typedef struct hydro_ocean {
    double density;              /* Fluid::density (MaterialManager.h:44) */
    double gravity;              /* SimulationManager::getGravity().z, 9.81 */
    int32_t waves;               /* Ocean::hasWaves(): depth = z - wave height */
    int32_t currents_enabled;    /* Ocean::EnableCurrents() was called */
    uint32_t n_currents;
    uint32_t reserved;
    hydro_current currents[HYDRO_MAX_CURRENTS];
} hydro_ocean;

/* The Atmosphere as seen by the aerodynamic path (Atmosphere.cpp:146-157):
 * gas density and the wind fields, all of which are summed (the atmosphere
 * has no per-field or global enable switch). */
typedef struct hydro_atmosphere {
    double density;              /* Atmosphere::getGas().density */
    uint32_t n_winds;
    uint32_t reserved;
    hydro_current winds[HYDRO_MAX_CURRENTS];
} hydro_atmosphere;

/* GeometryApproxType, Library/include/entities/SolidEntity.h:39 */
enum {
    HYDRO_APPROX_AUTO = 0,
    HYDRO_APPROX_SPHERE = 1,
    HYDRO_APPROX_CYLINDER = 2,
    HYDRO_APPROX_ELLIPSOID = 3
};

/* Per-body inputs of CorrectAerodynamicForces (SolidEntity.cpp:1925-1956). */
typedef struct hydro_aero_params {
    int32_t approx_type;         /* fdApproxType */
    int32_t reserved;
    double R_CG2H[9];            /* T_CG2H.getBasis(), rows */
    double approx_params[3];     /* fdApproxParams[0..2] (ellipsoid semi-axes) */
} hydro_aero_params;

/* Results of the aerodynamic path: the SolidEntity members Fda, Tda. */
typedef struct hydro_aero_wrench {
    double Fda[3], Tda[3];
    int32_t status;              /* per-body error word, 0 = ok */
    int32_t reserved;
} hydro_aero_wrench;

/* Per-body state read by SolidEntity::ComputeHydrodynamicForces
 * (SolidEntity.cpp:1799-1850) and its accessors (:215-226, :410-459). */
typedef struct hydro_body {
    hydro_transform T_CG;        /* getCGTransform() */
    hydro_transform T_C;         /* getCTransform(): physics-mesh frame */
    double R_O[9];               /* getOTransform().getBasis(), for the drag correction */
    double v[3];                 /* getLinearVelocity() */
    double omega[3];             /* getAngularVelocity() */
    double Cd[3];                /* fdCd */
    double Cf[3];                /* fdCf */
    double P_CB[3];              /* centre of buoyancy in the CG frame */
    double volume;               /* analytic volume (INSIDE buoyancy) */
    double surface;              /* analytic surface (INSIDE wetted area) */
    double aabb_min[3];          /* getAABB(): collision-shape AABB, world frame */
    double aabb_max[3];
    hydro_mesh_id mesh;          /* getPhysicsMesh(); HYDRO_NO_MESH = nullptr */
    int32_t mode;                /* PhysicsMode */
    int32_t buoyancy;            /* PhysicsSettings::buoyancy */
    int32_t reserved;
} hydro_body;

/* In-out results: the SolidEntity members Fb..Vsub (SolidEntity.h:400-437). */
typedef struct hydro_wrench {
    double Fb[3], Tb[3];         /* buoyancy force / torque */
    double Fdq[3], Tdq[3];       /* form (quadratic) drag force / torque */
    double Fdf[3], Tdf[3];       /* skin friction force / torque */
    double Swet;                 /* wetted surface */
    double Vsub;                 /* submerged volume */
    int32_t position;            /* BodyFluidPosition of this evaluation */
    int32_t status;              /* per-body error word, 0 = ok */
} hydro_wrench;

typedef struct hydro_config {
    int32_t device;              /* CUDA device ordinal */
    int32_t cut_precision;       /* HYDRO_CUT_FP32 (default) or HYDRO_CUT_FP64 */
    uint32_t tile_faces;         /* faces per work chunk, rounded up to whole tiles;
                                    0 = 4096 (hydro_batch_autotune picks per batch) */
    uint32_t ctas_per_sm;        /* resident CTAs per SM; 0 = 2 (or the autotuner's) */
    const char* tune_cache_path; /* autotuner cache file (copied), NULL = none */
} hydro_config;

/* -------------------------------------------------------------- lifecycle */
/* Fills *cfg with defaults (device 0, FP32 cut points, 4096-face chunks,
 * 2 CTAs per SM, no tuning cache). */
void hydro_config_default(hydro_config* cfg);

hydro_status hydro_create(hydro_ctx** ctx, const hydro_config* cfg);
void hydro_destroy(hydro_ctx* ctx);

/* Selects the frame of the FP32 face arithmetic for later calls on this
 * context (HYDRO_FRAME_WORLD or HYDRO_FRAME_CENTRED, see above).  No
 * counterpart in the reference, whose arithmetic is HYDRO_FRAME_WORLD. */
hydro_status hydro_set_frame(hydro_ctx* ctx, int32_t frame);

/* Message of the last failing call on this context (never NULL). */
const char* hydro_last_error(const hydro_ctx* ctx);
const char* hydro_status_string(hydro_status s);
int hydro_abi_version(void);

/* ----------------------------------------------------------------- meshes */
/* Uploads one physics mesh.  vertex_data/vertex_stride accept the
 * reference's own interleaved vertex arrays directly: the position is the
 * first three floats of each vertex, as in Vertex (24 B) and
 * TexturableVertex (44 B) of OpenGLDataStructs.h:120-155, i.e. what
 * Mesh::getVertexDataPointer() / getVertexSize() return; face_indices is
 * Mesh::faces (3 uint32 per face, getFaceDataPointer()).  The device keeps
 * a tiled copy; every index is range-checked here (HYDRO_ERR_INDEX_RANGE). */
hydro_status hydro_mesh_upload(hydro_ctx* ctx, const void* vertex_data,
                               size_t vertex_stride, uint32_t n_vertices,
                               const uint32_t* face_indices, uint32_t n_faces,
                               hydro_mesh_id* out_id);
hydro_status hydro_mesh_info(hydro_ctx* ctx, hydro_mesh_id id,
                             uint32_t* n_vertices, uint32_t* n_faces,
                             uint32_t* n_tiles);

/* ------------------------------------------------------------------ waves */
/* Sets the wave height data read by Ocean::GetDepth when ocean.waves != 0
 * (OpenGLRealOcean::ComputeWaveHeight, OpenGLRealOcean.cpp:282-331):
 * data is an N x N grid of `channels` interleaved floats (row j, column i at
 * (j*N+i)*channels); each of the n_layers layers reads channel
 * layer_channel[l] over a square of layer_grid_size[l] metres, and
 * wave height = -sum_l bilinear(layer l) (periodic, texel-centred).
 * N * N * channels must be below 2^32 (HYDRO_ERR_INVALID_ARG otherwise). */
hydro_status hydro_wave_grid_set(hydro_ctx* ctx, const float* data,
                                 uint32_t size, uint32_t channels,
                                 uint32_t n_layers,
                                 const uint32_t* layer_channel,
                                 const float* layer_grid_size);

/* Ocean::GetDepth for n points (xyz interleaved, host memory). */
hydro_status hydro_depth(hydro_ctx* ctx, const hydro_ocean* ocean,
                         const float* xyz, uint32_t n, float* depth);

/* ---------------------------------------------------------- batched path */
/* A batch fixes which mesh each body uses (bodies[i].mesh must equal
 * mesh_of_body[i] at compute time) and owns the device work list and the
 * per-tile scratch.  It replaces the per-body loop of the hydrodynamics
 * block of SimulationManager::SimulationTickCallback
 * (SimulationManager.cpp:1620-1655) and Ocean::ApplyFluidForces
 * (Ocean.cpp:219-268). */
hydro_status hydro_batch_create(hydro_ctx* ctx, const hydro_mesh_id* mesh_of_body,
                                uint32_t n_bodies, hydro_batch** out);

/* As hydro_batch_create, with the work-chunk size of this batch in faces
 * (rounded up to whole tiles of HYDRO_TILE_FACES faces, at most 32 tiles;
 * 0 = the context's setting).  Small chunks suit batches of which only a few bodies are
 * active at a time (no counterpart in the reference). */
hydro_status hydro_batch_create_ex(hydro_ctx* ctx, const hydro_mesh_id* mesh_of_body,
                                   uint32_t n_bodies, uint32_t chunk_faces, hydro_batch** out);
void hydro_batch_destroy(hydro_batch* batch);

/* Device-resident step: d_bodies and d_inout are device pointers; the call
 * enqueues on `stream` (a cudaStream_t, NULL = legacy default) and returns
 * without synchronising.  Three kernel launches per step (per-body setup,
 * the persistent face kernel, per-body finalisation); the call allocates
 * nothing after the batch exists and may be captured into a CUDA graph. */
hydro_status hydro_batch_compute_device(hydro_batch* batch, const hydro_body* d_bodies,
                                        const hydro_ocean* ocean,
                                        const hydro_settings* settings,
                                        hydro_wrench* d_inout, void* stream);

/* The per-body hydrodynamics loop of a simulation tick in one call
 * (SimulationManager.cpp:1620-1655 -> Ocean::ApplyFluidForces, Ocean.cpp:
 * 219-268 -> SolidEntity::ComputeHydrodynamicForces for every body):
 * hydro_batch_compute_device on a batch that the context builds for this
 * list of meshes on the first call and keeps until the list changes.
 * d_bodies and d_inout are device pointers, enqueued on `stream`. */
hydro_status hydro_compute_wrenches(hydro_ctx* ctx, const hydro_mesh_id* mesh_of_body, uint32_t n_bodies,
                                    const hydro_body* d_bodies, const hydro_ocean* ocean,
                                    const hydro_settings* settings, hydro_wrench* d_inout, void* stream);

/* As hydro_batch_compute_device for the first *d_count bodies only, the
 * count read on the device when the step runs (e.g. written by an earlier
 * kernel on the same stream); the other bodies' results are left as they
 * are and cost nothing (no counterpart in the reference). */
hydro_status hydro_batch_compute_device_prefix(hydro_batch* batch, const hydro_body* d_bodies,
                                               const uint32_t* d_count, const hydro_ocean* ocean,
                                               const hydro_settings* settings,
                                               hydro_wrench* d_inout, void* stream);

/* Host-buffer step, synchronous.  Page-locked mapped buffers (cudaHostAlloc,
 * cudaHostRegister with mapping, or a pinned torch tensor) are read and
 * written in place by the step's per-body kernels over the host link; other
 * host memory is staged: bodies and in-out wrenches copied host->device on
 * the batch's own stream, the wrenches copied back. */
hydro_status hydro_batch_compute(hydro_batch* batch, const hydro_body* bodies,
                                 const hydro_ocean* ocean,
                                 const hydro_settings* settings,
                                 hydro_wrench* inout);

/* Device address under which kernels can read and write the page-locked
 * mapped host memory at `host` (cudaHostAlloc, cudaHostRegister with
 * mapping, a pinned torch tensor); HYDRO_ERR_INVALID_ARG for other memory.
 * Lets device entry points take host buffers without staging copies (no
 * counterpart in the reference). */
hydro_status hydro_mapped_host_ptr(const void* host, void** device);

/* Autotuner (no counterpart in the reference).  Times the step on this
 * batch's own bodies for every work-chunk size in {2, 4, 8, 11, 16, 24, 32}
 * tiles ({896, 1792, 3584, 4928, 7168, 10752, 14336} faces) and 1 or 2
 * resident CTAs per SM (reps timed steps each, after one warm-up step),
 * keeps the fastest, and appends it to the context's
 * tune_cache_path (if set) under a key made of the GPU name, SM count, cut
 * precision, surface kind and the batch's face-count histogram.  A later
 * call with a cached key applies the cached choice without timing
 * (from_cache = 1).  d_scratch receives the results of the timing steps
 * (n_bodies hydro_wrench of device scratch).  Synchronises the stream; not
 * for use inside a stream capture. */
typedef struct hydro_tune_result {
    uint32_t chunk_faces;
    uint32_t ctas_per_sm;
    float ms_per_step;
    int32_t from_cache;
    uint32_t n_candidates;
    float candidate_ms[16];   /* in the order chunk size (outer) x CTAs per SM */
} hydro_tune_result;

hydro_status hydro_batch_autotune(hydro_batch* batch, const hydro_body* d_bodies,
                                  const hydro_ocean* ocean, const hydro_settings* settings,
                                  hydro_wrench* d_scratch, void* stream, uint32_t reps,
                                  hydro_tune_result* result);

/* Number of kernel launches the last compute call enqueued. */
uint32_t hydro_batch_last_launches(const hydro_batch* batch);

/* Per-kernel device times of a batch's steps (the reference's hydrodynamics
 * timer, PerformanceMonitor.cpp:80-88, at kernel granularity).  With
 * profiling on, each hydro_batch_compute(_device) call outside stream
 * capture records CUDA events around its three kernels on the launch
 * stream; hydro_batch_kernel_ms waits for the last recorded step and
 * returns its prep, chunk (face loop) and finalize durations. */
hydro_status hydro_batch_profile(hydro_batch* batch, int enable);
hydro_status hydro_batch_kernel_ms(hydro_batch* batch, float* prep_ms, float* chunk_ms, float* finalize_ms);

/* Allocation-free step (no counterpart in the reference).  For callers that
 * cannot allocate device memory while they run: a simulator evaluating the
 * hydrodynamics inside its real-time tick, where cudaMalloc may synchronise
 * the device and stall the tick, or an application whose device memory is
 * reserved up front by another allocator.  Same result as
 * hydro_batch_compute_device for the bodies (mesh_of_body is a host array,
 * d_bodies and d_inout device arrays, enqueued on `stream`), but every byte
 * of scratch lives in one static device array of HYDRO_STATIC_SCRATCH_BYTES
 * that each GPU loading this library holds until the process exits; no
 * cudaMalloc, cudaFree or other allocating routine is called.  Limits: at
 * most HYDRO_STATIC_MAX_BODIES bodies and a work list that fits the array
 * (about 16000 chunks of up to 8 tiles); larger requests return
 * HYDRO_ERR_INVALID_ARG and launch nothing.  The first call on a device
 * looks up the array's device address; meshes uploaded afterwards are
 * accepted as long as the device tile table does not need to grow
 * (otherwise HYDRO_ERR_INVALID_ARG).  Each call builds its work list on the
 * host in static (pageable) arrays and uploads it with cudaMemcpyAsync,
 * which may make the host wait while the driver stages the copy; it clears
 * the array's control words on `stream` before its kernels.  The call is
 * therefore not graph-capturable: do not issue it inside a stream capture
 * (a captured graph would replay whatever work list a later call left in
 * the host arrays); for a captured step use hydro_batch_compute_device.
 * All calls share the array and it keeps the last call's contents: calls
 * whose work overlaps on the GPU race. */
#define HYDRO_STATIC_SCRATCH_BYTES (4u << 20)
#define HYDRO_STATIC_MAX_BODIES 4096u
hydro_status hydro_compute_wrenches_static(hydro_ctx* ctx, const hydro_mesh_id* mesh_of_body,
                                           uint32_t n_bodies, const hydro_body* d_bodies,
                                           const hydro_ocean* ocean,
                                           const hydro_settings* settings,
                                           hydro_wrench* d_inout, void* stream);

/* --------------------------------------------- reference call surface */
/* SolidEntity::ComputeHydrodynamicForces (SolidEntity.cpp:1799-1850) for
 * one body: mode gate, CheckBodyFluidPosition, INSIDE/CROSSING branch and
 * CorrectHydrodynamicForces.  io holds the previous values on entry. */
hydro_status hydro_body_forces(hydro_ctx* ctx, const hydro_body* body,
                               const hydro_ocean* ocean,
                               const hydro_settings* settings,
                               hydro_wrench* io);

/* SolidEntity::ComputeHydrodynamicForcesSurface (SolidEntity.cpp:1289-1721).
 * mesh == HYDRO_NO_MESH behaves like mesh == nullptr.  Outputs are in-out:
 * Fb/Tb/Vsub keep their values when buoyancy is off or the submerged volume
 * is tiny; Fdq..Tdf are written only with damping_forces. */
hydro_status hydro_surface_forces(hydro_ctx* ctx, const hydro_settings* settings,
                                  hydro_mesh_id mesh, const hydro_ocean* ocean,
                                  const hydro_transform* T_CG,
                                  const hydro_transform* T_C,
                                  const double v[3], const double omega[3],
                                  double Fb[3], double Tb[3],
                                  double Fdq[3], double Tdq[3],
                                  double Fdf[3], double Tdf[3],
                                  double* Swet, double* Vsub);

/* SolidEntity::ComputeHydrodynamicForcesSubmerged (SolidEntity.cpp:1723-1797). */
hydro_status hydro_submerged_forces(hydro_ctx* ctx, hydro_mesh_id mesh,
                                    const hydro_ocean* ocean,
                                    const hydro_transform* T_CG,
                                    const hydro_transform* T_C,
                                    const double v[3], const double omega[3],
                                    double Fdq[3], double Tdq[3],
                                    double Fdf[3], double Tdf[3]);

/* SolidEntity::CorrectHydrodynamicForces (SolidEntity.cpp:1263-1287);
 * R_O is the basis of T_O (the body-origin transform). */
hydro_status hydro_correct_forces(hydro_ctx* ctx, const hydro_ocean* ocean,
                                  double Fdq[3], double Tdq[3],
                                  double Fdf[3], double Tdf[3],
                                  const double Cd[3], const double Cf[3],
                                  const double R_O[9]);

/* SolidEntity::CheckBodyFluidPosition (SolidEntity.cpp:1239-1261) from the
 * world AABB; writes HYDRO_INSIDE / HYDRO_OUTSIDE / HYDRO_CROSSING_SURFACE. */
hydro_status hydro_fluid_position(hydro_ctx* ctx, const hydro_ocean* ocean,
                                  const double aabb_min[3],
                                  const double aabb_max[3], int32_t* position);

/* ------------------------------------------------------------- compounds */
/* One part of a Compound (Library/src/entities/solids/Compound.cpp:291-436).
 * The compound itself is described by a hydro_body (T_CG, v, omega, the
 * compound's AABB, volume, surface, P_CB, mode and buoyancy; its mesh, T_C,
 * R_O, Cd and Cf are not used). */
typedef struct hydro_compound_part {
    hydro_transform T_C;         /* getOTransform() * parts[i].origin * solid->getO2CTransform() */
    double R_O[9];               /* basis of getOTransform() * parts[i].origin (correction frame) */
    double Cd[3];                /* solid->getHydrodynamicCoefficients() */
    double Cf[3];
    hydro_mesh_id mesh;          /* solid->getPhysicsMesh(); HYDRO_NO_MESH = nullptr */
    int32_t mode;                /* solid->getPhysicsMode() */
    int32_t buoyant;             /* solid->isBuoyant() */
    int32_t external;            /* parts[i].isExternal */
} hydro_compound_part;

typedef struct hydro_compound_batch hydro_compound_batch;

/* A set of compounds with a fixed list of parts: compound c owns the
 * parts_per_compound[c] consecutive entries of part_mesh (and of the part
 * array given at compute time), in the reference's part order. */
hydro_status hydro_compound_batch_create(hydro_ctx* ctx, const hydro_mesh_id* part_mesh,
                                         const uint32_t* parts_per_compound, uint32_t n_compounds,
                                         hydro_compound_batch** out);
void hydro_compound_batch_destroy(hydro_compound_batch* batch);

/* Compound::ComputeHydrodynamicForces (Compound.cpp:291-436) for every
 * compound: classification by the compound's AABB; INSIDE: buoyancy from the
 * compound's volume and P_CB, damping summed over the external fluid parts
 * (each part's submerged loop about the compound's CG, corrected with the
 * part's Cd/Cf in the part frame); CROSSING: each fluid part's surface loop
 * (buoyancy only for internal parts), corrected and summed, the per-part
 * in-out values carried from part to part as the reference's loop does.
 * Device pointers (d_io: one hydro_wrench per compound, in-out). */
hydro_status hydro_compound_compute_device(hydro_compound_batch* batch, const hydro_body* d_compounds,
                                           const hydro_compound_part* d_parts, const hydro_ocean* ocean,
                                           const hydro_settings* settings, hydro_wrench* d_io, void* stream);

/* Host-buffer version (synchronises). */
hydro_status hydro_compound_compute(hydro_compound_batch* batch, const hydro_body* compounds,
                                    const hydro_compound_part* parts, const hydro_ocean* ocean,
                                    const hydro_settings* settings, hydro_wrench* io);

/* ----------------------------------------------------------- mesh ingest */
/* Mass properties of a physics mesh (ComputePhysicalProperties,
 * Library/src/utils/GeometryFileUtil.cpp:335-566): solid (thickness <= 0,
 * signed tetrahedra) or shell (thickness > 0); CG, volume, surface and mass;
 * Ipri the principal moments about the CG and Irot (rows) the rotation whose
 * columns are the principal axes (identity when the tensor is diagonal). */
typedef struct hydro_mesh_properties {
    double mass;
    double volume;
    double surface;
    double CG[3];
    double Ipri[3];
    double Irot[9];
} hydro_mesh_properties;

/* The face sums on the GPU over the uploaded mesh (one CTA per tile, FP64),
 * the rest on the host. */
hydro_status hydro_mesh_compute_properties(hydro_ctx* ctx, hydro_mesh_id mesh, double thickness, double density,
                                           hydro_mesh_properties* out);

/* --------------------------------------------------- coefficient setup */
/* Result of SolidEntity::ComputeFluidDynamicsApprox (SolidEntity.cpp:698-1040):
 * the proxy shape fitted to the physics mesh and what it gives the body. */
typedef struct hydro_fluid_approx_result {
    int32_t approx_type;         /* fdApproxType: SPHERE, CYLINDER or ELLIPSOID (AUTO fits an ellipsoid) */
    int32_t n_params;            /* fdApproxParams.size(): 1, 2 or 3 */
    double params[3];            /* sphere: radius; cylinder: radius, length; ellipsoid: semi-axes */
    hydro_transform T_CG2H;      /* proxy frame in the CG frame (hydro_aero_params.R_CG2H) */
    double added_mass[3];        /* aMass */
    double added_inertia[3];     /* aI */
    double Cd[3];                /* fdCd, origin frame (hydro_body.Cd) */
    double Cf[3];                /* fdCf = 0.1 Cd (hydro_body.Cf) */
} hydro_fluid_approx_result;

/* The coefficient setup the reference runs once per body when it is built
 * (ComputeSphericalApprox :720-758, ComputeCylindricalApprox :760-847,
 * ComputeEllipsoidalApprox :849-1025).  vertex_data / vertex_stride /
 * n_vertices are the physics mesh's vertex array as getMeshVertices reads it
 * (Mesh::getVertexDataPointer(), getVertexSize(), getNumOfVertices(); the
 * position is the first three floats of each vertex); T_CG2C and T_CG2O are
 * the body's CG-to-mesh and CG-to-origin transforms, P_CB its centre of
 * buoyancy in the CG frame, density the ocean's liquid density (the
 * reference takes 1000 when the simulation has no ocean).  Host only, FP64,
 * the reference's bits.  HYDRO_ERR_INVALID_ARG for fewer than two vertices
 * (where the reference leaves the body's coefficients unchanged). */
hydro_status hydro_fluid_approx(const void* vertex_data, size_t vertex_stride, uint32_t n_vertices,
                                int32_t approx_type, const hydro_transform* T_CG2C,
                                const hydro_transform* T_CG2O, const double P_CB[3], double density,
                                hydro_fluid_approx_result* out);

/* OBJ text to the physics mesh the reference builds from it: positions
 * times scale (LoadOBJ scales only files that have normals; a file without
 * "vn" lines keeps its size, GeometryFileUtil.cpp:253-254), every face of
 * every shape, polygons triangulated as
 * rapidobj::Triangulate does (quads along the shorter diagonal, larger
 * polygons by ear slicing; LoadOBJ, GeometryFileUtil.cpp:52-230, physics
 * part), then, when
 * refine_threshold > 0, OpenGLContent::Refine (OpenGLContent.cpp:2833-2895;
 * Polyhedron uses 3).  Host only.  Sets *n_vertices and *n_faces; copies
 * xyz (n_vertices x 3) and faces (n_faces x 3) when the arrays are given
 * with enough room (capacities in vertices and faces), so a first call
 * with NULL arrays sizes them. */
hydro_status hydro_obj_parse(const char* text, size_t len, float scale, float refine_threshold, float* xyz,
                             uint32_t xyz_capacity, uint32_t* faces, uint32_t faces_capacity, uint32_t* n_vertices,
                             uint32_t* n_faces);

/* hydro_obj_parse and hydro_mesh_upload in one call. */
hydro_status hydro_mesh_upload_obj(hydro_ctx* ctx, const char* text, size_t len, float scale, float refine_threshold,
                                   hydro_mesh_id* out_id);

/* ------------------------------------------------------------- FFT ocean */
/* The reference's GPU ocean (OpenGLOcean, Library/src/graphics/OpenGLOcean.cpp)
 * as CUDA kernels writing this context's wave grid: Elfouhaily spectrum for
 * four grid sizes with the reference's random phases (host, once), then per
 * update h(k,t) (oceanInit.frag) and the log2(N)-pass inverse FFTs along x
 * and y (oceanFFTX/Y.frag) with the reference's binary16 butterfly table.
 * After an update the wave grid holds N x N texels of four heights and the
 * depth queries read channels 0 and 1 at grid sizes 0 and 1, as
 * OpenGLRealOcean::ComputeWaveHeight does (OpenGLRealOcean.cpp:321-331). */
typedef struct hydro_fft_ocean_params {
    float wind;                  /* params.wind, U10 [m/s] */
    float omega;                 /* params.omega, inverse wave age */
    float amplitude;             /* params.A */
    float km;                    /* params.km (370) */
    float cm;                    /* params.cm (0.23) */
    float grid_sizes[4];         /* params.gridSizes (893, 101, 21, 11) [m] */
    uint32_t passes;             /* params.passes: N = 2^passes texels per side (8) */
    int32_t propagate;           /* params.propagate (1) */
} hydro_fft_ocean_params;

/* The parameters OpenGLRealOcean uses for a sea state (OpenGLRealOcean.cpp:40-45,
 * OpenGLOcean.cpp:63-70): wind = 5 state + 2, omega = 5 exp(-state) + 0.2. */
void hydro_fft_ocean_params_for_state(float state, hydro_fft_ocean_params* params);

typedef struct hydro_fft_ocean hydro_fft_ocean;

/* Builds the spectrum (seed 1234 of the reference's generator) and the
 * butterfly table and makes the context's wave grid N x N x 4. */
hydro_status hydro_fft_ocean_create(hydro_ctx* ctx, const hydro_fft_ocean_params* params, hydro_fft_ocean** out);
void hydro_fft_ocean_destroy(hydro_fft_ocean* ocean);

/* The wave field at time t [s] into the context's wave grid (three kernel
 * launches on `stream`; later hydrodynamics calls on the same stream see
 * it). */
hydro_status hydro_fft_ocean_update(hydro_fft_ocean* ocean, float t, void* stream);

/* Copies the current wave grid (N x N x 4 floats) to host memory (synchronises). */
hydro_status hydro_fft_ocean_read(hydro_fft_ocean* ocean, float* out);

/* ---------------------------------------------------------------- cables */
/* One CableEntity: nodes first_node .. first_node + n_nodes - 1 of the
 * node arrays (Bullet soft-body nodes m_x, m_v), cylinder radius, physics
 * mode and PhysicsSettings::buoyancy. */
typedef struct hydro_cable {
    uint32_t first_node;
    uint32_t n_nodes;
    double radius;
    int32_t mode;
    int32_t buoyancy;
} hydro_cable;

/* The nodal forces of CableEntity (CableEntity.h:42-54). */
typedef struct hydro_cable_node_forces {
    double Fb[3];
    double Fdq[3];
    double Fdf[3];
} hydro_cable_node_forces;

/* CableEntity::ComputeHydrodynamicForces (CableEntity.cpp:240-376) for
 * n_cables cables: per segment the submerged volume of its cylinder, the
 * buoyancy and the form and skin drag from the segment's mean velocity
 * relative to the current, split between its nodes; the end nodes' forces
 * doubled.  Cables whose mode is neither FLOATING nor SUBMERGED, and cables
 * whose node range does not lie within n_nodes_total, are left untouched.
 * x and v are [n_nodes_total][3] FP64.  Device pointers on `stream`; the
 * call keeps n_nodes_total x 72 bytes of scratch per context. */
hydro_status hydro_cable_forces_device(hydro_ctx* ctx, const hydro_cable* d_cables, uint32_t n_cables,
                                       const double* d_x, const double* d_v, uint32_t n_nodes_total,
                                       const hydro_ocean* ocean, const hydro_settings* settings,
                                       hydro_cable_node_forces* d_out, void* stream);

/* Host-buffer version (synchronises). */
hydro_status hydro_cable_forces(hydro_ctx* ctx, const hydro_cable* cables, uint32_t n_cables, const double* x,
                                const double* v, uint32_t n_nodes_total, const hydro_ocean* ocean,
                                const hydro_settings* settings, hydro_cable_node_forces* out);

/* ---------------------------------------------------------- aerodynamics */
/* SolidEntity::ComputeAerodynamicForces(mesh, atm, T_CG, T_C, v, omega,
 * Fda, Tda) (SolidEntity.cpp:1865-1923): quadratic-law drag of the faces
 * whose normal velocity points into them, about the CG, for one body.  As in
 * the reference, each face's term is vn * 3 * A (glm's vec3::length() is the
 * component count, not the norm).  mesh HYDRO_NO_MESH gives zeros. */
hydro_status hydro_aero_forces(hydro_ctx* ctx, hydro_mesh_id mesh, const hydro_atmosphere* atm,
                               const hydro_transform* T_CG, const hydro_transform* T_C,
                               const double v[3], const double omega[3], double Fda[3], double Tda[3]);

/* SolidEntity::CorrectAerodynamicForces (SolidEntity.cpp:1925-1956). */
hydro_status hydro_aero_correct(hydro_ctx* ctx, const hydro_aero_params* params, double Fda[3],
                                double Tda[3]);

/* SolidEntity::ComputeAerodynamicForces(Atmosphere*) (SolidEntity.cpp:1852-1863)
 * for every body of the batch: bodies whose mode is not
 * HYDRO_MODE_AERODYNAMIC are left untouched; the others get the face loop
 * and the correction.  Device pointers, enqueued on `stream`. */
hydro_status hydro_batch_compute_aero_device(hydro_batch* batch, const hydro_body* d_bodies,
                                             const hydro_aero_params* d_params,
                                             const hydro_atmosphere* atm, hydro_aero_wrench* d_out,
                                             void* stream);

/* Host-buffer version of hydro_batch_compute_aero_device (synchronises). */
hydro_status hydro_batch_compute_aero(hydro_batch* batch, const hydro_body* bodies,
                                      const hydro_aero_params* params, const hydro_atmosphere* atm,
                                      hydro_aero_wrench* out);

/* ------------------------------------------------------------ diagnostics */
/* The debug geometry of the reference's surface loop: with DEBUG_HYDRO,
 * ComputeHydrodynamicForcesSurface (SolidEntity.cpp:1390-1396 and the
 * matching blocks of the other clip cases) records the outline of every
 * submerged triangle or quad it evaluates, as line segments, in the
 * `Renderable& debug` argument.  For one body (hydro_surface_forces's
 * inputs as a body record), this writes the same points in the same order:
 * faces in mesh order, each outline as 2 points per edge (6 for a triangle,
 * 8 for a quad), world frame, x y z floats.  Up to `capacity` points are
 * written; *n_points receives the total (call with capacity 0 to size the
 * buffer). */
hydro_status hydro_debug_surface_outline(hydro_ctx* ctx, const hydro_body* body,
                                         const hydro_ocean* ocean, const hydro_settings* settings,
                                         float* points, uint32_t capacity, uint32_t* n_points);

/* Per-face contributions of the surface loop (ComputeHydrodynamicForcesSurface,
 * SolidEntity.cpp:1337-1687) for one body, computed by the same device code
 * as the batched kernel: out receives n_faces * 23 floats in uploaded face
 * order, laid out Fb[3] Tb[3] Fdq[3] Tdq[3] Fdf[3] Tdf[3] Swet V6 CB6[3]
 * (V6 = 6 x the face's fan-tetra volume, CB6 = V6-weighted centroid).  For
 * validating the face arithmetic against a CPU restatement bit for bit.
 * packed != 0 evaluates pairs of consecutive fully submerged faces on the
 * packed FP32 path that the batched kernel uses; packed == 0 evaluates every
 * face on the scalar path. */
hydro_status hydro_debug_face_terms(hydro_ctx* ctx, const hydro_body* body,
                                    const hydro_ocean* ocean,
                                    const hydro_settings* settings, int32_t packed,
                                    float* out);

/* The tiling hydro_mesh_upload applies to a mesh (no device work, no
 * context): the faces in tile order (order[n_faces]) and each tile's first
 * position in it, followed by n_faces (tile_starts[n_tiles + 1]).  Tiles are
 * compact patches of at most HYDRO_TILE_FACES faces and 448 distinct
 * vertices, grown over shared vertices whatever the mesh's face order.
 * With starts_capacity < n_tiles + 1 nothing is written but *n_tiles and
 * HYDRO_ERR_INVALID_ARG is returned.  For checking and inspecting the mesh
 * layout; it has no counterpart in the reference. */
hydro_status hydro_debug_tile_order(const uint32_t* face_indices, uint32_t n_vertices, uint32_t n_faces,
                                    uint32_t* order, uint32_t* tile_starts, uint32_t starts_capacity,
                                    uint32_t* n_tiles);

/* Checks on the GPU that the division the kernels use for x/|n| and x/3
 * (a correctly rounded reciprocal plus one FMA correction) returns the bits
 * of IEEE round-to-nearest division: x/3 over every float, x/b over n_pairs
 * seeded random pairs in the face-length range and over n_pairs pairs of
 * normal floats.  mismatches[0..2] receive the three mismatch counts. */
hydro_status hydro_debug_division_check(hydro_ctx* ctx, uint64_t n_pairs, uint64_t seed,
                                        uint64_t mismatches[3]);

/* Failure detection without a GPU fault: one CTA waits, with the bounded
 * wait of the tile pipeline, on an mbarrier that nothing completes, gives up
 * after limit_us microseconds (1..2000000) and writes HYDRO_ERR_TIMEOUT to
 * *status; the context stays usable.  The same bounded waits in the batched
 * step turn a stalled pipeline into status HYDRO_ERR_TIMEOUT per body. */
hydro_status hydro_debug_wait_timeout(hydro_ctx* ctx, uint32_t limit_us, int32_t* status);

/* The division check above plus a check that the packed FP32 pair
 * instructions the kernels use for two faces at a time (mul, add, sub, fma
 * .rn.f32x2) return, in each half, the bits of the scalar IEEE operation:
 * packed[0..3] receive the mismatch counts over n_pairs random operand sets,
 * examples[4k..4k+3] one failing set (a, b, c, result) of op k.  packed and
 * examples may be NULL. */
hydro_status hydro_debug_arith_check(hydro_ctx* ctx, uint64_t n_pairs, uint64_t seed,
                                     uint64_t division[3], uint64_t packed[4],
                                     float examples[16]);

/* The host tables of the FFT ocean (no device work, no context): the wave
 * spectrum as hydro_fft_ocean_create builds it (OpenGLOcean::
 * GenerateWavesSpectrum, OpenGLOcean.cpp:1025-1048, seed 1234 of the
 * reference's generator; each value rounded to binary16 as the reference's
 * RGBA16F textures hold it), N x N x 4 floats each for s12 and s34, and the
 * butterfly table (ComputeButterflyLookupTable, :878-926) decoded per pass p
 * and output i at [p * N + i]: the two input indices (butterfly_index, 2
 * int32 each) and the binary16 weight (butterfly_weight, re and im).  Any
 * output may be NULL.  For checking the tables against the reference. */
hydro_status hydro_debug_fft_ocean_tables(const hydro_fft_ocean_params* params, float* s12, float* s34,
                                          int32_t* butterfly_index, float* butterfly_weight);

/* ------------------------------------------------------------------------
 * Learned wrench surrogate (no counterpart in the reference).
 *
 * Kernels of a small MLP that predicts a hull's body-frame wrench
 * (F[3], T[3] about the CG) from 16 state features, trained on wrenches the
 * exact step computes, and of the out-of-distribution gate that sends
 * states outside the training domain to the exact step.  All pointers are
 * device pointers; every call is asynchronous on `stream` (a cudaStream_t,
 * NULL = the legacy default stream).  Matrices are row-major; "bf16" buffers
 * hold IEEE bfloat16 values (uint16 bit patterns).
 * ---------------------------------------------------------------------- */

#define HYDRO_NN_FEATURES 16
#define HYDRO_NN_EPI_F32 0        /* z = A B */
#define HYDRO_NN_EPI_BIAS_SILU 1  /* z = A B + bias, y = bf16(silu(z)); z may be NULL */
#define HYDRO_NN_EPI_BIAS 2       /* z = A B + bias */
#define HYDRO_NN_EPI_SILU_GRAD 3  /* y = bf16((A B) * silu'(zprev)) */

/* C[M,N] = A[M,K] (bf16, row stride lda) x B[K,N] (bf16, row stride ldb)
 * on the BF16 tensor cores with FP32 accumulation, followed by `epilogue`;
 * outputs z (FP32) and y (bf16) have row stride ldc.  M and N must be
 * multiples of 64, K a multiple of 32.  A plain product (HYDRO_NN_EPI_F32)
 * with few 64 x 64 output tiles and a long K (a weight gradient, K = the
 * batch) is split along K into partial products in the context's
 * workspace, which a second kernel sums in a fixed order (deterministic).
 * The workspace is one per context: calls that use it (this, large-row
 * hydro_nn_colsum, hydro_nn_train) must not run concurrently on different
 * streams. */
hydro_status hydro_nn_gemm(hydro_ctx* ctx, int32_t epilogue, const void* A, int32_t lda,
                           const void* B, int32_t ldb, int32_t M, int32_t N, int32_t K,
                           float* z, void* y, const float* bias, const float* zprev,
                           int32_t ldc, void* stream);

/* dst[cols][rows] = transpose of the bf16 matrix src[rows][cols]. */
hydro_status hydro_nn_transpose(hydro_ctx* ctx, const void* src, void* dst, int32_t rows,
                                int32_t cols, void* stream);

/* Mean-squared-error gradient over the first n_out of ld columns of z
 * against the normalised target t' = (target - tmean) * tistd (tmean and
 * tistd both NULL: t' = target), target[rows][n_out]: dz (bf16, rows x ld,
 * other columns zero) = 2 (z - t') / (rows n_out); *loss += the mean
 * squared error when loss is non-NULL. */
hydro_status hydro_nn_mse_grad(hydro_ctx* ctx, const float* z, const float* target, int32_t rows,
                               int32_t ld, int32_t n_out, const float* tmean, const float* tistd,
                               void* dz, double* loss, void* stream);

/* out[c] = sum over rows of the bf16 matrix g[rows][cols] (bias gradients),
 * in a fixed order; from 2048 rows on, in row slabs whose partial sums go
 * through the context's workspace (see hydro_nn_gemm). */
hydro_status hydro_nn_colsum(hydro_ctx* ctx, const void* g, int32_t rows, int32_t cols, float* out,
                             void* stream);

/* One AdamW step (decoupled weight decay, bias-corrected moments, `step`
 * counted from 1) on FP32 master weights w[rows][cols] with gradient
 * grad (row stride ldg); then w16 = bf16(w) and wt16 = bf16(w)^T when
 * non-NULL. */
hydro_status hydro_nn_adamw(hydro_ctx* ctx, float* w, float* m, float* v, const float* grad,
                            int32_t rows, int32_t cols, int32_t ldg, float lr, float beta1,
                            float beta2, float eps, float weight_decay, int32_t step, void* w16,
                            void* wt16, void* stream);

/* One layer of the MLP as the training loop sees it (device pointers):
 * FP32 master weights w[k][n] and bias b[n], their AdamW moments (mw, vw,
 * mb, vb) and gradients (gw, gb), and the bf16 copies the GEMMs read
 * (w16 [k][n], wt16 [n][k]). */
typedef struct hydro_nn_layer {
    float* w;
    float* b;
    float* mw;
    float* vw;
    float* mb;
    float* vb;
    float* gw;
    float* gb;
    void* w16;
    void* wt16;
    int32_t k;
    int32_t n;
} hydro_nn_layer;

/* The four-layer MLP (layers 0..2: bias + SiLU, layer 3: bias) with the work
 * buffers of one training batch (device pointers): z[l] FP32 pre-
 * activations [batch][n_l]; x[l] (l < 3) bf16 activations [batch][n_l];
 * dz[l] bf16 gradients [batch][n_l]; xt[l] bf16 transposed layer inputs
 * [k_l][batch]; targets normalised by (t - tmean) * tistd (both NULL: raw);
 * the batch losses are added to *loss. */
typedef struct hydro_nn_net {
    hydro_nn_layer layer[4];
    float* z[4];
    void* x[3];
    void* dz[4];
    void* xt[4];
    const float* tmean;
    const float* tistd;
    double* loss;
    int32_t batch;
    int32_t n_out;
} hydro_nn_net;

/* n_steps AdamW steps of the MLP, launched from native code.  Step s reads
 * rows [rows[s], rows[s] + batch) of the bf16 network inputs X [n_rows][k_0]
 * and of the FP32 targets T [n_rows][n_out], runs the forward and backward
 * passes and updates every layer with learning rate lr[s] and step count
 * step0 + s + 1 (rows and lr are host arrays of n_steps).  It launches the
 * kernels of hydro_nn_gemm, hydro_nn_mse_grad, hydro_nn_transpose,
 * hydro_nn_colsum and hydro_nn_adamw with the same arguments in the same
 * order as calling those one by one, so the trained weights are the same
 * bits; a step then costs no round trip through the caller. */
hydro_status hydro_nn_train(hydro_ctx* ctx, const hydro_nn_net* net, const void* X, const float* T,
                            int64_t n_rows, const int64_t* rows, const float* lr, int32_t n_steps,
                            int32_t step0, float beta1, float beta2, float eps, float weight_decay,
                            void* stream);

/* y[rows][ld] = bf16((x - mean) * istd) of x[rows][n_in], zero in columns
 * n_in..ld-1; mean and istd both NULL for a plain conversion. */
hydro_status hydro_nn_to_bf16(hydro_ctx* ctx, const float* x, int32_t rows, int32_t n_in, int32_t ld,
                              const float* mean, const float* istd, void* y, void* stream);

/* The 16 features of each body state, FP32 [n][16]: depth of the CG below
 * the local surface, roll, pitch, body-frame v[3], omega[3] and current[3],
 * wave elevation at the CG, mean wave slope along and across the heading
 * over +-1 m, and the surface curvature along the heading over +-1 m (the
 * wave terms are 0 on a flat surface). */
hydro_status hydro_nn_features(hydro_ctx* ctx, const hydro_body* d_bodies, uint32_t n,
                               const hydro_ocean* ocean, float* d_features, void* stream);

/* Out-of-distribution gate: d_mask[i] = 1 when features[i] lie in the box
 * [lo, hi] and (f - mean)^T precision (f - mean) <= threshold (precision is
 * the 16x16 inverse covariance of the training features), else 0.  lo, hi,
 * mean, precision are device pointers. */
hydro_status hydro_nn_gate(hydro_ctx* ctx, const float* d_features, uint32_t n, const float* lo,
                           const float* hi, const float* mean, const float* precision,
                           float threshold, uint8_t* d_mask, void* stream);

/* Fused inference of the whole network on the 5th-generation tensor cores
 * (tcgen05 MMAs, FP32 accumulators in tensor memory, activations kept in
 * shared memory): d_out[i][16] = layer-3 output (bias added; columns 0..5
 * are the wrench) of the 16 features d_features[i] normalised as
 * (f - fmean) * fistd.  d_image holds HYDRO_NN_TC_IMAGE_BYTES of weights in
 * the kernels' shared-memory layout, written by hydro_nn_pack_sw128 at the
 * offsets 0 (W0^T, 256 x 64, K 16 used), 32768 (W1^T, 256 x 256), 163840
 * (W2^T) and 294912 (W3^T, 16 x 256); b0..b2 have 256 entries, b3 16.
 * *d_err gets bit 0 if a bounded wait ran out. */
#define HYDRO_NN_TC_IMAGE_BYTES 303104u
hydro_status hydro_nn_mlp_tc(hydro_ctx* ctx, const float* d_features, uint32_t n, const float* fmean,
                             const float* fistd, const void* d_image, const float* b0, const float* b1,
                             const float* b2, const float* b3, float* d_out, uint32_t* d_err, void* stream);

/* Writes src[rows][K] (bf16, row stride ld) into dst as the tensor-core
 * operand image: K-major, K zero-padded to kpad (a multiple of 64), each
 * [rows x 64] block in 8-row x 128-byte atoms with 16-byte chunk c of row r
 * stored at chunk c ^ (r % 8) (128-byte swizzle). */
hydro_status hydro_nn_pack_sw128(hydro_ctx* ctx, const void* src, int32_t rows, int32_t K, int32_t ld,
                                 int32_t kpad, void* dst, void* stream);

/* Packs the bodies with d_mask[i] == 0, in index order, to the front of
 * d_packed (n entries) and switches the rest of d_packed off (mode
 * HYDRO_MODE_DISABLED), so an exact step over d_packed integrates only the
 * rejected states; d_pos[i] = packed slot or -1, *d_n_packed = count.
 * d_counts holds ceil(n / 256) words of scratch.  d_exact (n records, may
 * be null): slots 0 .. count - 1 are zeroed, the fresh in-out records of
 * the exact step over d_packed. */
hydro_status hydro_nn_route(hydro_ctx* ctx, const hydro_body* d_bodies, const uint8_t* d_mask,
                            uint32_t n, uint32_t* d_counts, hydro_body* d_packed, int32_t* d_pos,
                            uint32_t* d_n_packed, hydro_wrench* d_exact, void* stream);

/* Clears d_mask[i] for the bodies whose fluid position is INSIDE (the AABB
 * rule of CheckBodyFluidPosition, SolidEntity.cpp:1239-1261): there the
 * reference uses its analytic buoyancy instead of the face integral
 * (:1827-1843), a regime the surrogate sees rarely and fits worst, so those
 * states take the exact step. */
hydro_status hydro_nn_gate_inside(hydro_ctx* ctx, const hydro_body* d_bodies, uint32_t n,
                                  const hydro_ocean* ocean, uint8_t* d_mask, void* stream);

/* Two-network ensemble: row i of d_za (row stride ld, columns 0..5 the
 * body-frame wrench) becomes the mean of the rows of d_za and d_zb, and
 * d_mask[i] is cleared when the two rows differ by more than tau in the
 * wrench metric max(|dF| / force_scale, |dT| / torque_scale). */
hydro_status hydro_nn_ensemble(hydro_ctx* ctx, float* d_za, const float* d_zb, int32_t ld, uint32_t n,
                               double force_scale, double torque_scale, float tau, uint8_t* d_mask,
                               void* stream);

/* Audit sample of the gated predictor: for j < k, row i = phase + j * stride
 * (i < n) that the gate admitted (d_mask[i] != 0) is also sent to the exact
 * step (its mask cleared) and d_idx[j] = i; otherwise d_idx[j] = -1.  After
 * the exact step and merge, hydro_nn_audit_error gives each sampled row's
 * error: d_err[j] = max(|dF| / force_scale, |dT| / torque_scale) of d_z's
 * row (the network's output) against the exact body-frame wrench
 * d_exact[d_pos[i]], or -1 for an empty slot. */
hydro_status hydro_nn_audit_pick(hydro_ctx* ctx, uint8_t* d_mask, uint32_t n, uint32_t stride, uint32_t phase,
                                 uint32_t k, int32_t* d_idx, void* stream);
hydro_status hydro_nn_audit_error(hydro_ctx* ctx, const hydro_body* d_bodies, const float* d_z, int32_t ld,
                                  const int32_t* d_pos, const hydro_wrench* d_exact, const int32_t* d_idx,
                                  uint32_t k, double force_scale, double torque_scale, float* d_err,
                                  void* stream);

/* d_out[i][6] = body-frame wrench: columns 0..5 of d_z[i] (row stride ld)
 * when d_pos[i] < 0, else R^T (Fb+Fdq+Fdf, Tb+Tdq+Tdf) of d_exact[d_pos[i]]. */
hydro_status hydro_nn_merge(hydro_ctx* ctx, const hydro_body* d_bodies, const float* d_z, int32_t ld,
                            const int32_t* d_pos, const hydro_wrench* d_exact, uint32_t n,
                            float* d_out, void* stream);

/* d_out[i][6] = R^T (Fb+Fdq+Fdf, Tb+Tdq+Tdf) of d_wrenches[i]: the
 * surrogate's training target. */
hydro_status hydro_nn_wrench_body(hydro_ctx* ctx, const hydro_body* d_bodies,
                                  const hydro_wrench* d_wrenches, uint32_t n, float* d_out,
                                  void* stream);

/* ------------------------------------------------------------------------
 * Device-resident rigid-body rollout (no counterpart in the reference,
 * which integrates bodies with Bullet on the CPU).
 *
 * State of one free hull, integrated without contacts the way Bullet
 * integrates a Stonefish rigid body (btRigidBody with the implicit
 * gyroscopic term, which SolidEntity::BuildRigidBody enables,
 * SolidEntity.cpp:1076-1086): semi-implicit Euler for the velocities, one
 * Newton step of implicit Euler for the gyroscopic term, positions from the
 * new velocities and orientation by the exponential map.  q is the
 * body-to-world rotation as a unit quaternion (w, x, y, z); p, v, w are the
 * CG position, linear and angular velocity in the world frame (NED); the
 * thrust wrench is fixed in the body frame (about the CG).  mass weighs the
 * hull (gravity = mass g); inertial_mass divides the force and inertia is
 * the diagonal body-frame inertia about the CG -- for a SUBMERGED body the
 * reference uses mass + added mass and Ipri + added inertia there
 * (SolidEntity::getAugmentedMass/getAugmentedInertia, :657-670).
 * half_extents is the collision-shape AABB half size in the body frame (the
 * body record's AABB is its rotation).
 * ---------------------------------------------------------------------- */
typedef struct hydro_rigid_state {
    double p[3];
    double q[4];
    double v[3];
    double w[3];
    double thrust_force[3];
    double thrust_torque[3];
    double mass;
    double inertial_mass;
    double inertia[3];
    double half_extents[3];
} hydro_rigid_state;

/* One step of dt seconds for n hulls.  The hydrodynamic wrench comes from
 * d_exact (world-frame hydro_wrench results of a step on d_bodies) or, when
 * d_exact is NULL, from d_body_wrench (body-frame F[3], T[3] per hull, e.g.
 * the surrogate's output); both NULL integrates thrust and gravity only.
 * gravity is g along +z.  Updates d_states and rewrites the pose, velocity
 * and AABB fields of d_bodies (other fields are left as they are). */
hydro_status hydro_rigid_step(hydro_ctx* ctx, hydro_rigid_state* d_states, hydro_body* d_bodies,
                              const hydro_wrench* d_exact, const float* d_body_wrench, uint32_t n,
                              double dt, double gravity, void* stream);

/* Writes the pose, velocity and AABB fields of d_bodies from d_states. */
hydro_status hydro_rigid_write_bodies(hydro_ctx* ctx, const hydro_rigid_state* d_states,
                                      hydro_body* d_bodies, uint32_t n, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* STONEFISH_HYDRO_H */
