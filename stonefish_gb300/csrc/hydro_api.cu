// hydro_api.cu -- C ABI of the GB300 hydrodynamic wrench path
// (include/stonefish_hydro.h).  Host C++ only: contexts, the tiled device
// copy of each mesh, batches (work lists and scratch) and the launches.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/stonefish_hydro.h"
#include "hydro_internal.h"

using namespace sfh;

namespace {

struct MeshRec {
    uint32_t n_vertices;
    uint32_t n_faces;
    uint32_t first_tile;
    uint32_t n_tiles;
};

struct Slab {
    char* base;
    size_t size;
    size_t used;
};

}  // namespace

struct hydro_batch;

struct hydro_ctx {
    int device = 0;
    int sm_count = 1;
    hydro_config cfg{};
    cudaStream_t stream = nullptr;
    std::recursive_mutex mu;
    std::string err = "";
    std::vector<MeshRec> meshes;
    std::vector<Slab> slabs;
    std::vector<TileDesc> tiles_h;
    TileDesc* tiles_d = nullptr;
    size_t tiles_d_cap = 0;
    size_t tiles_d_count = 0;
    // wave grid
    float* wave_d = nullptr;
    uint32_t wave_n = 0, wave_channels = 0, wave_layers = 0;
    uint32_t wave_channel[HYDRO_MAX_WAVE_LAYERS] = {0, 0, 0, 0};
    float wave_grid[HYDRO_MAX_WAVE_LAYERS] = {1.f, 1.f, 1.f, 1.f};
    // single-body calls
    std::unordered_map<uint32_t, hydro_batch*> single;
    // hydro_compute_wrenches: the batch of the last list of meshes
    hydro_batch* oneshot = nullptr;
    std::vector<hydro_mesh_id> oneshot_meshes;
    void* small_d = nullptr;   // scratch for the small entry points
    float* nn_ws = nullptr;    // split-K partial products of the surrogate's weight-gradient GEMMs
    size_t nn_ws_floats = 0;
    size_t small_cap = 0;
    std::string tune_path;     // autotuner cache file ("" = none)
    int frame = HYDRO_FRAME_WORLD;   // body-op frame (hydro_set_frame)
    double* cable_seg = nullptr;   // cable segment scratch (9 doubles per node)
    size_t cable_cap = 0;
    void* cable_stage = nullptr;   // host-buffer cable call staging
    size_t cable_stage_cap = 0;
    char gpu_name[256] = {0};
};

struct hydro_batch {
    hydro_ctx* ctx = nullptr;
    uint32_t n_bodies = 0;
    uint32_t n_chunks = 0;
    std::vector<uint32_t> mesh_of_body;
    ChunkDesc* chunks_d = nullptr;
    BodyInfo* binfo_d = nullptr;
    double* partials_d = nullptr;
    BodyParams* bparams_d = nullptr;
    unsigned* err_d = nullptr;
    ActiveChunk* active_d = nullptr;     // the launch's list of chunks with a face loop
    hydro_body* bodies_d = nullptr;    // staging for the host-buffer entry point
    hydro_wrench* io_d = nullptr;
    cudaStream_t stream = nullptr;
    uint32_t last_launches = 0;
    uint32_t chunk_tiles = 0;    // tiles per work chunk of this batch
    uint32_t class_start[kClaimClasses + 1] = {};   // claim-class regions of the active list
    uint32_t ctas_per_sm = 0;    // 0 = the context's setting
    hydro_aero_params* aparams_d = nullptr;   // staging for the host-buffer aerodynamic call
    hydro_aero_wrench* aio_d = nullptr;
    cudaEvent_t prof_ev[4] = {nullptr, nullptr, nullptr, nullptr};   // per-kernel timing, when enabled
    bool prof_recorded = false;
};

struct hydro_compound_batch {
    hydro_ctx* ctx = nullptr;
    hydro_batch* parts = nullptr;          // work list over the parts' meshes
    uint32_t n_compounds = 0;
    uint32_t n_parts = 0;
    CompoundInfo* cinfo_d = nullptr;
    uint32_t* part_compound_d = nullptr;
    hydro_body* compounds_d = nullptr;     // staging for the host-buffer call
    hydro_compound_part* parts_d = nullptr;
    hydro_wrench* io_d = nullptr;
    uint32_t last_launches = 0;
};

struct hydro_fft_ocean {
    hydro_ctx* ctx = nullptr;
    hydro_fft_ocean_params p{};
    uint32_t N = 0;
    float4* s12_d = nullptr;
    float4* s34_d = nullptr;
    int2* idx_d = nullptr;
    float2* w_d = nullptr;
};

namespace sfh {
bool parse_obj(const char* text, size_t len, float scale, std::vector<float>& xyz, std::vector<uint32_t>& faces,
               std::string& err);
void refine_mesh(std::vector<float>& xyz, std::vector<uint32_t>& faces, float threshold);
void finish_properties(double thickness, double density, const double* s0, const double* s1,
                       hydro_mesh_properties* out);
void fft_ocean_spectrum(const hydro_fft_ocean_params& p, std::vector<float4>& s12, std::vector<float4>& s34);
void fft_ocean_butterfly(int passes, std::vector<int2>& idx, std::vector<float2>& w);
}

namespace {

hydro_status fail(hydro_ctx* ctx, hydro_status s, const char* fmt, ...)
{
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        ctx->err = buf;
    }
    return s;
}

hydro_status cuda_fail(hydro_ctx* ctx, cudaError_t e, const char* what)
{
    if (e == cudaErrorMemoryAllocation)
        return fail(ctx, HYDRO_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
    return fail(ctx, HYDRO_ERR_DEVICE, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(ctx, call)                                              \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return cuda_fail((ctx), e_, #call); \
    } while (0)

constexpr size_t kSlabBytes = size_t(256) << 20;

// Bump allocation of device memory for mesh tiles (256-byte aligned).
hydro_status slab_alloc(hydro_ctx* ctx, size_t bytes, char** out)
{
    bytes = (bytes + 255) & ~size_t(255);
    if (ctx->slabs.empty() || ctx->slabs.back().size - ctx->slabs.back().used < bytes) {
        Slab s{};
        s.size = std::max(kSlabBytes, bytes);
        cudaError_t e = cudaMalloc(&s.base, s.size);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(mesh slab)");
        s.used = 0;
        ctx->slabs.push_back(s);
    }
    Slab& s = ctx->slabs.back();
    *out = s.base + s.used;
    s.used += bytes;
    return HYDRO_OK;
}

// Device copy of the tile table, grown on demand.
hydro_status sync_tiles(hydro_ctx* ctx)
{
    if (ctx->tiles_d_count == ctx->tiles_h.size()) return HYDRO_OK;
    if (ctx->tiles_h.size() > ctx->tiles_d_cap) {
        size_t cap = std::max<size_t>(ctx->tiles_h.size() * 2, 1024);
        TileDesc* p = nullptr;
        CK(ctx, cudaMalloc(&p, cap * sizeof(TileDesc)));
        if (ctx->tiles_d) cudaFree(ctx->tiles_d);
        ctx->tiles_d = p;
        ctx->tiles_d_cap = cap;
        ctx->tiles_d_count = 0;
    }
    size_t n = ctx->tiles_h.size() - ctx->tiles_d_count;
    CK(ctx, cudaMemcpy(ctx->tiles_d + ctx->tiles_d_count, ctx->tiles_h.data() + ctx->tiles_d_count,
                       n * sizeof(TileDesc), cudaMemcpyHostToDevice));
    ctx->tiles_d_count = ctx->tiles_h.size();
    return HYDRO_OK;
}

hydro_status ensure_small(hydro_ctx* ctx, size_t bytes)
{
    if (ctx->small_cap >= bytes) return HYDRO_OK;
    if (ctx->small_d) cudaFree(ctx->small_d);
    ctx->small_d = nullptr;
    ctx->small_cap = 0;
    size_t cap = std::max<size_t>(bytes, 4096);
    CK(ctx, cudaMalloc(&ctx->small_d, cap));
    ctx->small_cap = cap;
    return HYDRO_OK;
}

bool valid_ocean(const hydro_ocean* o)
{
    return o && o->n_currents <= HYDRO_MAX_CURRENTS;
}

bool valid_atmosphere(const hydro_atmosphere* a)
{
    return a && a->n_winds <= HYDRO_MAX_CURRENTS;
}

// The atmosphere in the ocean descriptor the kernels read: gas density and
// every wind field as an enabled current (Atmosphere::GetFluidVelocity sums
// all fields, Atmosphere.cpp:146-152); no waves.
hydro_ocean atmosphere_ocean(const hydro_atmosphere* a)
{
    hydro_ocean o{};
    o.density = a->density;
    o.gravity = 0.0;
    o.waves = 0;
    o.currents_enabled = 1;
    o.n_currents = a->n_winds;
    for (uint32_t i = 0; i < a->n_winds && i < HYDRO_MAX_CURRENTS; ++i) {
        o.currents[i] = a->winds[i];
        o.currents[i].enabled = 1;
    }
    return o;
}

// The kernels' view of the ocean: the position-independent currents are
// summed in FP64 in the reference's order and cast once (Ocean.cpp:183-201).
OceanDev make_ocean(const hydro_ctx* ctx, const hydro_ocean* o)
{
    OceanDev d{};
    d.density = o->density;
    d.gravity = o->gravity;
    d.waves = o->waves ? 1 : 0;
    d.currents_enabled = o->currents_enabled ? 1 : 0;
    d.n_currents = (int)o->n_currents;
    double u[3] = {0.0, 0.0, 0.0};
    int field = 0;
    if (o->currents_enabled) {
        for (uint32_t i = 0; i < o->n_currents; ++i) {
            const hydro_current& c = o->currents[i];
            if (!c.enabled) continue;
            if (c.type == HYDRO_CURRENT_UNIFORM) {
                u[0] += c.vel[0]; u[1] += c.vel[1]; u[2] += c.vel[2];
            } else {
                field = 1;
            }
        }
    }
    d.field_currents = field;
    d.U[0] = (float)u[0]; d.U[1] = (float)u[1]; d.U[2] = (float)u[2];
    for (int i = 0; i < HYDRO_MAX_CURRENTS; ++i) d.currents[i] = o->currents[i];
    if (!o->currents_enabled) d.n_currents = 0;
    d.wave_data = ctx->wave_d;
    d.wave_n = ctx->wave_n;
    d.wave_channels = ctx->wave_channels;
    d.wave_layers = ctx->wave_layers;
    d.wave_half = ctx->wave_n ? 0.5f / (float)ctx->wave_n : 0.f;
    for (int l = 0; l < HYDRO_MAX_WAVE_LAYERS; ++l) {
        d.wave_channel[l] = ctx->wave_channel[l];
        d.wave_grid[l] = ctx->wave_grid[l];
        d.wave_inv_grid[l] = 1.0f / ctx->wave_grid[l];
    }
    return d;
}

uint32_t tiles_per_chunk(const hydro_ctx* ctx, uint32_t chunk_faces = 0)
{
    uint32_t faces = chunk_faces ? chunk_faces : ctx->cfg.tile_faces ? ctx->cfg.tile_faces : 4096u;
    return std::min<uint32_t>((uint32_t)kMaxTilesPerChunk,
                              std::max<uint32_t>(1u, (faces + kTileFaces - 1) / kTileFaces));
}

void batch_free(hydro_batch* b)
{
    if (!b) return;
    cudaFree(b->chunks_d);
    cudaFree(b->binfo_d);
    cudaFree(b->partials_d);
    cudaFree(b->bparams_d);
    cudaFree(b->err_d);
    cudaFree(b->active_d);
    cudaFree(b->bodies_d);
    cudaFree(b->io_d);
    cudaFree(b->aparams_d);
    cudaFree(b->aio_d);
    for (cudaEvent_t ev : b->prof_ev)
        if (ev) cudaEventDestroy(ev);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

// (Re)builds a batch's work list: chunks of at most tpc tiles, body by body,
// with their per-chunk scratch.
hydro_status build_work(hydro_ctx* ctx, hydro_batch* b, uint32_t tpc)
{
    const uint32_t n = b->n_bodies;
    std::vector<ChunkDesc> chunks;
    std::vector<BodyInfo> info(n);
    for (uint32_t i = 0; i < n; ++i) {
        BodyInfo& bi = info[i];
        bi.first_chunk = (uint32_t)chunks.size();
        bi.mesh = b->mesh_of_body[i];
        uint32_t first = 0, nt = 0;
        if (bi.mesh != HYDRO_NO_MESH) {
            const MeshRec& m = ctx->meshes[bi.mesh];
            first = m.first_tile;
            nt = m.n_tiles;
            bi.n_faces = m.n_faces;
        } else {
            bi.n_faces = 0;
        }
        uint32_t k = 0;
        for (uint32_t t = 0; t < nt; t += tpc, ++k)
            chunks.push_back(ChunkDesc{i, first + t, std::min(tpc, nt - t), k});
        if (k == 0) chunks.push_back(ChunkDesc{i, first, 0u, 0u});   // finaliser only
        bi.n_chunks = (uint32_t)chunks.size() - bi.first_chunk;
    }
    cudaFree(b->chunks_d);
    cudaFree(b->binfo_d);
    cudaFree(b->partials_d);
    cudaFree(b->active_d);
    b->chunks_d = nullptr;
    b->binfo_d = nullptr;
    b->partials_d = nullptr;
    b->active_d = nullptr;
    b->n_chunks = (uint32_t)chunks.size();
    b->chunk_tiles = tpc;
    claim_class_starts(chunks.data(), chunks.size(), b->class_start);
    CK(ctx, cudaMalloc(&b->chunks_d, chunks.size() * sizeof(ChunkDesc)));
    CK(ctx, cudaMalloc(&b->binfo_d, n * sizeof(BodyInfo)));
    CK(ctx, cudaMalloc(&b->partials_d, chunks.size() * kPartialStride * sizeof(double)));
    CK(ctx, cudaMalloc(&b->active_d, chunks.size() * sizeof(ActiveChunk)));
    CK(ctx, cudaMemcpy(b->chunks_d, chunks.data(), chunks.size() * sizeof(ChunkDesc), cudaMemcpyHostToDevice));
    CK(ctx, cudaMemcpy(b->binfo_d, info.data(), n * sizeof(BodyInfo), cudaMemcpyHostToDevice));
    CK(ctx, cudaMemset(b->partials_d, 0, chunks.size() * kPartialStride * sizeof(double)));
    return HYDRO_OK;
}

hydro_status batch_build(hydro_ctx* ctx, const hydro_mesh_id* mesh_of_body, uint32_t n,
                         hydro_batch** out, uint32_t chunk_faces = 0)
{
    for (uint32_t i = 0; i < n; ++i) {
        if (mesh_of_body[i] != HYDRO_NO_MESH && mesh_of_body[i] >= ctx->meshes.size())
            return fail(ctx, HYDRO_ERR_NOT_FOUND, "body %u: unknown mesh %u", i, mesh_of_body[i]);
    }
    hydro_status st = sync_tiles(ctx);
    if (st != HYDRO_OK) return st;
    hydro_batch* b = new (std::nothrow) hydro_batch();
    if (!b) return fail(ctx, HYDRO_ERR_OOM, "host allocation");
    b->ctx = ctx;
    b->n_bodies = n;
    b->mesh_of_body.assign(mesh_of_body, mesh_of_body + n);
    cudaError_t e;
#define BK(call)                                              \
    do {                                                      \
        e = (call);                                           \
        if (e != cudaSuccess) {                               \
            batch_free(b);                                    \
            return cuda_fail(ctx, e, #call);                  \
        }                                                     \
    } while (0)
    BK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    BK(cudaMalloc(&b->bparams_d, n * sizeof(BodyParams)));
    BK(cudaMalloc(&b->err_d, 256));
    BK(cudaMemset(b->err_d, 0, 256));
#undef BK
    st = build_work(ctx, b, tiles_per_chunk(ctx, chunk_faces));
    if (st != HYDRO_OK) {
        batch_free(b);
        return st;
    }
    *out = b;
    return HYDRO_OK;
}

hydro_status batch_launch(hydro_batch* b, const hydro_body* d_bodies, const hydro_ocean* ocean,
                          const hydro_settings* settings, hydro_wrench* d_io, cudaStream_t s,
                          int op, const uint32_t* d_count = nullptr, hydro_aero_wrench* d_aero = nullptr,
                          const hydro_aero_params* d_aero_params = nullptr)
{
    hydro_ctx* ctx = b->ctx;
    hydro_status st = sync_tiles(ctx);
    if (st != HYDRO_OK) return st;
    KParams P{};
    P.chunks = b->chunks_d;
    P.binfo = b->binfo_d;
    P.tiles = ctx->tiles_d;
    P.bodies = d_bodies;
    P.io = d_io;
    P.partials = b->partials_d;
    P.bparams = b->bparams_d;
    P.err = b->err_d;
    P.work = b->err_d + 32;
    P.n_listed = b->err_d + 48;
    P.n_active = d_count;
    P.aero_io = d_aero;
    P.aero_params = d_aero_params;
    P.active = b->active_d;
    P.n_bodies = b->n_bodies;
    P.n_chunks = b->n_chunks;
    P.ocean = make_ocean(ctx, ocean);
    P.st.damping = settings->damping_forces ? 1 : 0;
    P.st.buoyancy = settings->realistic_buoyancy ? 1 : 0;
    P.op = op;
    P.frame = ctx->frame;
    std::memcpy(P.class_start, b->class_start, sizeof(P.class_start));
    if (P.ocean.waves && ctx->wave_d == nullptr)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "ocean.waves set but no wave grid was given");
    const int cut64 = ctx->cfg.cut_precision == HYDRO_CUT_FP64;
    LaunchShape shape{};
    const int want = b->ctas_per_sm ? (int)b->ctas_per_sm : ctx->cfg.ctas_per_sm ? (int)ctx->cfg.ctas_per_sm : 2;
    shape.ctas_per_sm = std::max(1, std::min(want, chunk_kernel_occupancy(cut64, P.ocean.waves, want,
                                                                            op == OP_AERO || op == OP_AERO_BODY,
                                                                            P.ocean.field_currents)));
    shape.grid = ctx->sm_count * shape.ctas_per_sm;
    uint32_t launches = 0;
    // kernel timing events (hydro_batch_profile) outside stream capture only
    cudaEvent_t* ev = nullptr;
    if (b->prof_ev[0]) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone) ev = b->prof_ev;
    }
    cudaError_t e = launch_step(P, shape, cut64, s, &launches, ev);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "wrench step launch");
    b->last_launches = launches;
    if (ev) b->prof_recorded = true;
    return HYDRO_OK;
}

hydro_status single_batch(hydro_ctx* ctx, hydro_mesh_id mesh, hydro_batch** out)
{
    auto it = ctx->single.find(mesh);
    if (it != ctx->single.end()) {
        *out = it->second;
        return HYDRO_OK;
    }
    hydro_batch* b = nullptr;
    hydro_status st = batch_build(ctx, &mesh, 1, &b);
    if (st != HYDRO_OK) return st;
    cudaError_t e1 = cudaMalloc(&b->bodies_d, sizeof(hydro_body));
    cudaError_t e2 = cudaMalloc(&b->io_d, sizeof(hydro_wrench));
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
        batch_free(b);
        return cuda_fail(ctx, e1 != cudaSuccess ? e1 : e2, "cudaMalloc(single body)");
    }
    ctx->single[mesh] = b;
    *out = b;
    return HYDRO_OK;
}

// One body through the batched kernel with host in/out.
hydro_status run_single(hydro_ctx* ctx, const hydro_body& body, const hydro_ocean* ocean,
                        const hydro_settings* settings, hydro_wrench& io, int op)
{
    hydro_batch* b = nullptr;
    hydro_status st = single_batch(ctx, body.mesh, &b);
    if (st != HYDRO_OK) return st;
    CK(ctx, cudaMemcpyAsync(b->bodies_d, &body, sizeof(hydro_body), cudaMemcpyHostToDevice, ctx->stream));
    CK(ctx, cudaMemcpyAsync(b->io_d, &io, sizeof(hydro_wrench), cudaMemcpyHostToDevice, ctx->stream));
    st = batch_launch(b, b->bodies_d, ocean, settings, b->io_d, ctx->stream, op);
    if (st != HYDRO_OK) return st;
    CK(ctx, cudaMemcpyAsync(&io, b->io_d, sizeof(hydro_wrench), cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    return HYDRO_OK;
}

void copy3(double* d, const double* s) { d[0] = s[0]; d[1] = s[1]; d[2] = s[2]; }

}  // namespace

// =================================================================== C ABI
extern "C" {

void hydro_config_default(hydro_config* cfg)
{
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->device = 0;
    cfg->cut_precision = HYDRO_CUT_FP32;
    cfg->tile_faces = 0;
    cfg->ctas_per_sm = 0;
    cfg->tune_cache_path = nullptr;
}

int hydro_abi_version(void) { return HYDRO_ABI_VERSION; }

hydro_status hydro_set_frame(hydro_ctx* ctx, int32_t frame)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (frame != HYDRO_FRAME_WORLD && frame != HYDRO_FRAME_CENTRED)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "frame %d: not HYDRO_FRAME_WORLD or HYDRO_FRAME_CENTRED", frame);
    ctx->frame = frame;
    return HYDRO_OK;
}

const char* hydro_status_string(hydro_status s)
{
    switch (s) {
    case HYDRO_OK: return "ok";
    case HYDRO_ERR_INVALID_ARG: return "invalid argument";
    case HYDRO_ERR_OOM: return "out of memory";
    case HYDRO_ERR_TIMEOUT: return "device wait timed out";
    case HYDRO_ERR_DEVICE: return "CUDA error";
    case HYDRO_ERR_NOT_FOUND: return "not found";
    case HYDRO_ERR_INDEX_RANGE: return "face index out of range";
    case HYDRO_ERR_UNSUPPORTED: return "unsupported";
    case HYDRO_ERR_MISMATCH: return "body table does not match batch";
    }
    return "unknown status";
}

const char* hydro_last_error(const hydro_ctx* ctx)
{
    return ctx ? ctx->err.c_str() : "null context";
}

hydro_status hydro_create(hydro_ctx** out, const hydro_config* cfg)
{
    if (!out) return HYDRO_ERR_INVALID_ARG;
    *out = nullptr;
    hydro_config c;
    if (cfg) c = *cfg;
    else hydro_config_default(&c);
    if (c.cut_precision != HYDRO_CUT_FP64 && c.cut_precision != HYDRO_CUT_FP32)
        return HYDRO_ERR_INVALID_ARG;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return HYDRO_ERR_DEVICE;
    if (c.device < 0 || c.device >= n) return HYDRO_ERR_INVALID_ARG;
    if (cudaSetDevice(c.device) != cudaSuccess) return HYDRO_ERR_DEVICE;
    hydro_ctx* ctx = new (std::nothrow) hydro_ctx();
    if (!ctx) return HYDRO_ERR_OOM;
    ctx->device = c.device;
    ctx->cfg = c;
    if (cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, c.device) != cudaSuccess)
        ctx->sm_count = 1;
    if (c.tune_cache_path) ctx->tune_path = c.tune_cache_path;
    ctx->cfg.tune_cache_path = nullptr;
    {
        cudaDeviceProp prop;
        if (cudaGetDeviceProperties(&prop, c.device) == cudaSuccess)
            snprintf(ctx->gpu_name, sizeof(ctx->gpu_name), "%s", prop.name);
    }
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return HYDRO_ERR_DEVICE;
    }
    *out = ctx;
    return HYDRO_OK;
}

void hydro_destroy(hydro_ctx* ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    for (auto& kv : ctx->single) batch_free(kv.second);
    if (ctx->oneshot) batch_free(ctx->oneshot);
    for (auto& s : ctx->slabs) cudaFree(s.base);
    cudaFree(ctx->tiles_d);
    cudaFree(ctx->wave_d);
    cudaFree(ctx->small_d);
    cudaFree(ctx->nn_ws);
    cudaFree(ctx->cable_seg);
    cudaFree(ctx->cable_stage);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

// Tile membership: faces grouped into compact patches of the surface, so
// that a tile lies wholly above or wholly under the water more often and
// shares more vertices between its faces.  A tile grows from a seed face by
// repeatedly taking, among the unused faces that share a vertex with it,
// one that adds the fewest new vertices (ties: the one reached first, so
// that the tile grows ring by ring).  The next tile starts from the face on
// the closed tile's border that comes first in upload order, so tiles
// follow one another across the surface whatever the upload order.  When a
// tile has used up its connected part of the mesh (the separately indexed
// sides of a box are separate parts), it
// closes if at least half full and otherwise takes the next unused face in
// upload order as a further seed, so that small parts share tiles.  A tile
// closes at kTileFaces faces or when no reachable face fits under
// kTileVerts vertices.  `order` lists the faces tile by tile, `starts` the
// tiles' first positions in it (plus the end).
static void build_tiles(uint32_t n_vertices, const uint32_t* fi, uint32_t n_faces, std::vector<uint32_t>& order,
                        std::vector<uint32_t>& starts)
{
    std::vector<uint32_t> first(n_vertices + 1, 0);          // faces around each vertex (CSR)
    for (size_t i = 0; i < 3 * (size_t)n_faces; ++i) ++first[fi[i] + 1];
    for (uint32_t v = 0; v < n_vertices; ++v) first[v + 1] += first[v];
    std::vector<uint32_t> around(3 * (size_t)n_faces);
    {
        std::vector<uint32_t> fill(first.begin(), first.end() - 1);
        for (uint32_t f = 0; f < n_faces; ++f)
            for (int k = 0; k < 3; ++k) around[fill[fi[3 * (size_t)f + k]]++] = f;
    }
    std::vector<uint8_t> used(n_faces, 0), best(n_faces, 4);
    std::vector<uint8_t> in_tile(n_vertices, 0);
    std::vector<uint32_t> tverts, touched;
    std::vector<uint32_t> queue[4];        // candidates by count of new vertices, in the order reached
    size_t head[4];
    order.clear();
    order.reserve(n_faces);
    starts.assign(1, 0u);
    auto fresh = [&](uint32_t f) {
        const uint32_t* t = fi + 3 * (size_t)f;
        uint32_t n = 0;
        for (int k = 0; k < 3; ++k) {
            bool dup = false;
            for (int j = 0; j < k; ++j) dup |= (t[j] == t[k]);
            if (!dup && !in_tile[t[k]]) ++n;
        }
        return n;
    };
    uint32_t seed = 0;
    uint32_t border = UINT32_MAX;          // a face on the last tile's border, if any
    while (order.size() < n_faces) {
        uint32_t tf = 0;
        for (int b = 0; b < 4; ++b) {
            queue[b].clear();
            head[b] = 0;
        }
        touched.clear();
        auto push = [&](uint32_t g) {
            if (used[g]) return;
            const uint32_t nw = fresh(g);
            if (nw >= best[g]) return;
            if (best[g] == 4) touched.push_back(g);
            best[g] = (uint8_t)nw;
            queue[nw].push_back(g);
        };
        // only the faces around a vertex that joins the tile change their
        // count of new vertices, so only those are (re)considered
        auto take = [&](uint32_t f) {
            used[f] = 1;
            order.push_back(f);
            ++tf;
            uint32_t joined[3];
            int nj = 0;
            for (int k = 0; k < 3; ++k) {
                const uint32_t v = fi[3 * (size_t)f + k];
                if (!in_tile[v]) {
                    in_tile[v] = 1;
                    tverts.push_back(v);
                    joined[nj++] = v;
                }
            }
            for (int k = 0; k < nj; ++k)
                for (uint32_t i = first[joined[k]]; i < first[joined[k] + 1]; ++i) push(around[i]);
        };
        if (border != UINT32_MAX && !used[border]) take(border);
        border = UINT32_MAX;
        while (tf < (uint32_t)kTileFaces) {
            int b = 0;
            while (b < 4 && head[b] == queue[b].size()) ++b;
            if (b == 4) {
                if (2 * tf >= (uint32_t)kTileFaces) break;
                while (seed < n_faces && used[seed]) ++seed;
                if (seed >= n_faces || tverts.size() + fresh(seed) > (size_t)kTileVerts) break;
                take(seed);
                continue;
            }
            const uint32_t g = queue[b][head[b]++];
            if (used[g] || best[g] != (uint8_t)b) continue;       // taken, or queued again with fewer
            if (tverts.size() + (size_t)b > (size_t)kTileVerts) continue;
            take(g);
        }
        // the next tile's seed: of the unused faces this tile reached, the
        // first in upload order (meshes generated in a sweep keep sweeping)
        for (int b = 0; b < 4; ++b)
            for (size_t i = head[b]; i < queue[b].size(); ++i)
                if (!used[queue[b][i]] && (border == UINT32_MAX || queue[b][i] < border)) border = queue[b][i];
        starts.push_back((uint32_t)order.size());
        for (uint32_t v : tverts) in_tile[v] = 0;
        tverts.clear();
        for (uint32_t g : touched) best[g] = 4;
    }
}

hydro_status hydro_mesh_upload(hydro_ctx* ctx, const void* vertex_data, size_t vertex_stride,
                               uint32_t n_vertices, const uint32_t* face_indices,
                               uint32_t n_faces, hydro_mesh_id* out_id)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!vertex_data || !face_indices || !out_id || n_vertices == 0 || n_faces == 0)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "mesh upload: null pointer or empty mesh");
    if (vertex_stride < 3 * sizeof(float))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "mesh upload: vertex stride %zu < 12", vertex_stride);
    for (size_t i = 0; i < (size_t)n_faces * 3; ++i) {
        if (face_indices[i] >= n_vertices)
            return fail(ctx, HYDRO_ERR_INDEX_RANGE, "face %zu index %u >= %u vertices",
                        i / 3, face_indices[i], n_vertices);
    }
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    const char* vbytes = static_cast<const char*>(vertex_data);
    auto pos = [&](uint32_t v, float* p) { std::memcpy(p, vbytes + (size_t)v * vertex_stride, 12); };

    // Tiles are compact patches of the surface (build_tiles); within a tile
    // faces keep the order in which they joined it.
    std::vector<uint32_t> order, starts;
    build_tiles(n_vertices, face_indices, n_faces, order, starts);
    std::vector<int32_t> local(n_vertices, -1);
    std::vector<uint32_t> tv;              // global ids of the open tile's vertices
    std::vector<uint32_t> ti;              // packed local indices of the open tile's faces
    std::vector<uint32_t> tid;             // upload indices of the open tile's faces
    std::vector<char> host;                // all tile blocks of this mesh
    struct Pending { size_t offset; uint16_t nv, nf; uint32_t first_face; float4 sphere, half; };
    std::vector<Pending> pend;
    auto close_tile = [&](uint32_t tile_first) {
        if (ti.empty()) return;
        const uint32_t nv = (uint32_t)tv.size(), nf = (uint32_t)ti.size();
        const uint32_t nvp = (nv + 3) & ~3u;
        const size_t bytes = tile_block_bytes(nv, nf);
        size_t off = host.size();
        host.resize(off + bytes, 0);
        float* f = reinterpret_cast<float*>(host.data() + off);
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (uint32_t k = 0; k < nv; ++k) {
            float p[3];
            pos(tv[k], p);
            f[k] = p[0];
            f[nvp + k] = p[1];
            f[2 * nvp + k] = p[2];
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::min(lo[a], (double)p[a]);
                hi[a] = std::max(hi[a], (double)p[a]);
            }
        }
        std::memcpy(host.data() + off + (size_t)nvp * 12, ti.data(), ti.size() * 4);
        std::memcpy(host.data() + off + tile_bytes(nv, nf), tid.data(), tid.size() * 4);
        // bounds: centre of the box, radius to the farthest vertex from the
        // stored (float) centre and half extents about it, rounded up
        float c[3];
        for (int a = 0; a < 3; ++a) c[a] = (float)(0.5 * (lo[a] + hi[a]));
        double r2 = 0.0, hx = 0.0, hy = 0.0, hz = 0.0;
        for (uint32_t k = 0; k < nv; ++k) {
            float p[3];
            pos(tv[k], p);
            const double dx = (double)p[0] - c[0], dy = (double)p[1] - c[1], dz = (double)p[2] - c[2];
            r2 = std::max(r2, dx * dx + dy * dy + dz * dz);
            hx = std::max(hx, std::fabs(dx));
            hy = std::max(hy, std::fabs(dy));
            hz = std::max(hz, std::fabs(dz));
        }
        auto up = [](double x) { return std::nextafter((float)(x * (1.0 + 1e-6)), 1e30f); };
        const float4 sphere = make_float4(c[0], c[1], c[2], up(std::sqrt(r2)));
        const float4 half = make_float4(up(hx), up(hy), up(hz), 0.f);
        pend.push_back(Pending{off, (uint16_t)nv, (uint16_t)nf, tile_first, sphere, half});
        for (uint32_t g : tv) local[g] = -1;
        tv.clear();
        ti.clear();
        tid.clear();
    };
    for (size_t t = 0; t + 1 < starts.size(); ++t) {
        for (uint32_t k = starts[t]; k < starts[t + 1]; ++k) {
            const uint32_t f = order[k];
            const uint32_t* fv = face_indices + 3 * (size_t)f;
            uint32_t word = 0;
            for (int j = 0; j < 3; ++j) {
                if (local[fv[j]] < 0) {
                    local[fv[j]] = (int32_t)tv.size();
                    tv.push_back(fv[j]);
                }
                word |= (uint32_t)local[fv[j]] << (9 * j);
            }
            ti.push_back(word);
            tid.push_back(f);
        }
        close_tile(starts[t]);
    }

    char* dev = nullptr;
    hydro_status st = slab_alloc(ctx, host.size(), &dev);
    if (st != HYDRO_OK) return st;
    CK(ctx, cudaMemcpy(dev, host.data(), host.size(), cudaMemcpyHostToDevice));
    MeshRec m{};
    m.n_vertices = n_vertices;
    m.n_faces = n_faces;
    m.first_tile = (uint32_t)ctx->tiles_h.size();
    m.n_tiles = (uint32_t)pend.size();
    for (const Pending& p : pend)
        ctx->tiles_h.push_back(TileDesc{reinterpret_cast<const float*>(dev + p.offset), p.nv, p.nf, p.first_face, p.sphere,
                                        p.half});
    *out_id = (hydro_mesh_id)ctx->meshes.size();
    ctx->meshes.push_back(m);
    return HYDRO_OK;
}

hydro_status hydro_mesh_info(hydro_ctx* ctx, hydro_mesh_id id, uint32_t* nv, uint32_t* nf,
                             uint32_t* nt)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (id >= ctx->meshes.size()) return fail(ctx, HYDRO_ERR_NOT_FOUND, "unknown mesh %u", id);
    const MeshRec& m = ctx->meshes[id];
    if (nv) *nv = m.n_vertices;
    if (nf) *nf = m.n_faces;
    if (nt) *nt = m.n_tiles;
    return HYDRO_OK;
}

hydro_status hydro_wave_grid_set(hydro_ctx* ctx, const float* data, uint32_t size,
                                 uint32_t channels, uint32_t n_layers,
                                 const uint32_t* layer_channel, const float* layer_grid_size)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!data || size == 0 || channels == 0 || n_layers == 0 || n_layers > HYDRO_MAX_WAVE_LAYERS ||
        !layer_channel || !layer_grid_size || size > 65536)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "wave grid: bad arguments");
    if ((uint64_t)size * size * channels >= (uint64_t(1) << 32))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "wave grid: N * N * channels must be below 2^32");
    for (uint32_t l = 0; l < n_layers; ++l) {
        if (layer_channel[l] >= channels || !(layer_grid_size[l] > 0.f))
            return fail(ctx, HYDRO_ERR_INVALID_ARG, "wave grid: bad layer %u", l);
    }
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    CK(ctx, cudaDeviceSynchronize());
    if (ctx->wave_d) cudaFree(ctx->wave_d);
    ctx->wave_d = nullptr;
    const size_t bytes = (size_t)size * size * channels * sizeof(float);
    CK(ctx, cudaMalloc(&ctx->wave_d, bytes));
    CK(ctx, cudaMemcpy(ctx->wave_d, data, bytes, cudaMemcpyHostToDevice));
    ctx->wave_n = size;
    ctx->wave_channels = channels;
    ctx->wave_layers = n_layers;
    for (uint32_t l = 0; l < HYDRO_MAX_WAVE_LAYERS; ++l) {
        ctx->wave_channel[l] = l < n_layers ? layer_channel[l] : 0;
        ctx->wave_grid[l] = l < n_layers ? layer_grid_size[l] : 1.f;
    }
    return HYDRO_OK;
}

hydro_status hydro_depth(hydro_ctx* ctx, const hydro_ocean* ocean, const float* xyz, uint32_t n,
                         float* depth)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!valid_ocean(ocean) || (!xyz && n) || (!depth && n))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "depth: bad arguments");
    if (n == 0) return HYDRO_OK;
    if (ocean->waves && !ctx->wave_d) return fail(ctx, HYDRO_ERR_INVALID_ARG, "depth: no wave grid");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    hydro_status st = ensure_small(ctx, (size_t)n * 16);
    if (st != HYDRO_OK) return st;
    float* dx = static_cast<float*>(ctx->small_d);
    float* dd = dx + 3 * (size_t)n;
    CK(ctx, cudaMemcpyAsync(dx, xyz, (size_t)n * 12, cudaMemcpyHostToDevice, ctx->stream));
    cudaError_t e = launch_depth(make_ocean(ctx, ocean), dx, n, dd, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "depth kernel");
    CK(ctx, cudaMemcpyAsync(depth, dd, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    return HYDRO_OK;
}

hydro_status hydro_batch_create(hydro_ctx* ctx, const hydro_mesh_id* mesh_of_body,
                                uint32_t n_bodies, hydro_batch** out)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!out || !mesh_of_body || n_bodies == 0)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "batch: null pointer or no bodies");
    *out = nullptr;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    return batch_build(ctx, mesh_of_body, n_bodies, out);
}

hydro_status hydro_batch_create_ex(hydro_ctx* ctx, const hydro_mesh_id* mesh_of_body, uint32_t n_bodies,
                                   uint32_t chunk_faces, hydro_batch** out)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!out || !mesh_of_body || n_bodies == 0)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "batch: null pointer or no bodies");
    *out = nullptr;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    return batch_build(ctx, mesh_of_body, n_bodies, out, chunk_faces);
}

void hydro_batch_destroy(hydro_batch* b)
{
    if (!b) return;
    std::lock_guard<std::recursive_mutex> lk(b->ctx->mu);
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->stream);
    batch_free(b);
}

hydro_status hydro_batch_compute_device(hydro_batch* b, const hydro_body* d_bodies,
                                        const hydro_ocean* ocean, const hydro_settings* settings,
                                        hydro_wrench* d_inout, void* stream)
{
    if (!b) return HYDRO_ERR_INVALID_ARG;
    hydro_ctx* ctx = b->ctx;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!d_bodies || !d_inout || !settings || !valid_ocean(ocean))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "batch compute: bad arguments");
    return batch_launch(b, d_bodies, ocean, settings, d_inout, static_cast<cudaStream_t>(stream), OP_BODY);
}

hydro_status hydro_batch_compute_device_prefix(hydro_batch* b, const hydro_body* d_bodies,
                                               const uint32_t* d_count, const hydro_ocean* ocean,
                                               const hydro_settings* settings, hydro_wrench* d_inout,
                                               void* stream)
{
    if (!b) return HYDRO_ERR_INVALID_ARG;
    hydro_ctx* ctx = b->ctx;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!d_bodies || !d_inout || !d_count || !settings || !valid_ocean(ocean))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "batch compute prefix: bad arguments");
    return batch_launch(b, d_bodies, ocean, settings, d_inout, static_cast<cudaStream_t>(stream), OP_BODY,
                        d_count);
}

hydro_status hydro_compute_wrenches(hydro_ctx* ctx, const hydro_mesh_id* mesh_of_body, uint32_t n_bodies,
                                    const hydro_body* d_bodies, const hydro_ocean* ocean,
                                    const hydro_settings* settings, hydro_wrench* d_inout, void* stream)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!mesh_of_body || n_bodies == 0)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "compute wrenches: no bodies");
    const bool same = ctx->oneshot && ctx->oneshot_meshes.size() == n_bodies &&
                      std::equal(mesh_of_body, mesh_of_body + n_bodies, ctx->oneshot_meshes.begin());
    if (!same) {
        hydro_batch* nb = nullptr;
        const hydro_status st = hydro_batch_create(ctx, mesh_of_body, n_bodies, &nb);
        if (st != HYDRO_OK) return st;
        if (ctx->oneshot) hydro_batch_destroy(ctx->oneshot);
        ctx->oneshot = nb;
        ctx->oneshot_meshes.assign(mesh_of_body, mesh_of_body + n_bodies);
    }
    return hydro_batch_compute_device(ctx->oneshot, d_bodies, ocean, settings, d_inout, stream);
}

// Device address of host memory that kernels can read and write in place
// (page-locked and mapped, e.g. from cudaHostAlloc), or null for memory
// that has to be staged through copies.
static void* mapped_host_ptr(const void* p)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

hydro_status hydro_mapped_host_ptr(const void* host, void** device)
{
    if (!host || !device) return HYDRO_ERR_INVALID_ARG;
    void* d = mapped_host_ptr(host);
    if (!d) return HYDRO_ERR_INVALID_ARG;
    *device = d;
    return HYDRO_OK;
}

hydro_status hydro_batch_compute(hydro_batch* b, const hydro_body* bodies, const hydro_ocean* ocean,
                                 const hydro_settings* settings, hydro_wrench* inout)
{
    if (!b) return HYDRO_ERR_INVALID_ARG;
    hydro_ctx* ctx = b->ctx;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!bodies || !inout || !settings || !valid_ocean(ocean))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "batch compute: bad arguments");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    const size_t nb = (size_t)b->n_bodies;
    // page-locked mapped buffers are read and written in place by the step's
    // per-body kernels (the face kernel never touches them); others are staged
    const hydro_body* db = static_cast<const hydro_body*>(mapped_host_ptr(bodies));
    hydro_wrench* dio = static_cast<hydro_wrench*>(mapped_host_ptr(inout));
    if (!db) {
        if (!b->bodies_d) CK(ctx, cudaMalloc(&b->bodies_d, nb * sizeof(hydro_body)));
        CK(ctx, cudaMemcpyAsync(b->bodies_d, bodies, nb * sizeof(hydro_body), cudaMemcpyHostToDevice, b->stream));
        db = b->bodies_d;
    }
    const bool staged_io = (dio == nullptr);
    if (staged_io) {
        if (!b->io_d) CK(ctx, cudaMalloc(&b->io_d, nb * sizeof(hydro_wrench)));
        CK(ctx, cudaMemcpyAsync(b->io_d, inout, nb * sizeof(hydro_wrench), cudaMemcpyHostToDevice, b->stream));
        dio = b->io_d;
    }
    hydro_status st = batch_launch(b, db, ocean, settings, dio, b->stream, OP_BODY);
    if (st != HYDRO_OK) return st;
    if (staged_io)
        CK(ctx, cudaMemcpyAsync(inout, b->io_d, nb * sizeof(hydro_wrench), cudaMemcpyDeviceToHost, b->stream));
    CK(ctx, cudaStreamSynchronize(b->stream));
    return HYDRO_OK;
}

uint32_t hydro_batch_last_launches(const hydro_batch* b) { return b ? b->last_launches : 0u; }

hydro_status hydro_batch_profile(hydro_batch* b, int enable)
{
    if (!b) return HYDRO_ERR_INVALID_ARG;
    hydro_ctx* ctx = b->ctx;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    if (enable && !b->prof_ev[0]) {
        for (cudaEvent_t& ev : b->prof_ev) {
            cudaError_t e = cudaEventCreate(&ev);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaEventCreate");
        }
    } else if (!enable) {
        for (cudaEvent_t& ev : b->prof_ev) {
            if (ev) cudaEventDestroy(ev);
            ev = nullptr;
        }
    }
    b->prof_recorded = false;
    return HYDRO_OK;
}

hydro_status hydro_batch_kernel_ms(hydro_batch* b, float* prep_ms, float* chunk_ms, float* finalize_ms)
{
    if (!b || !prep_ms || !chunk_ms || !finalize_ms) return HYDRO_ERR_INVALID_ARG;
    hydro_ctx* ctx = b->ctx;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!b->prof_ev[0] || !b->prof_recorded)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "kernel times: profiling off or no step recorded");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    cudaError_t e = cudaEventSynchronize(b->prof_ev[3]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(prep_ms, b->prof_ev[0], b->prof_ev[1]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(chunk_ms, b->prof_ev[1], b->prof_ev[2]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(finalize_ms, b->prof_ev[2], b->prof_ev[3]);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "kernel times");
    return HYDRO_OK;
}

hydro_status hydro_body_forces(hydro_ctx* ctx, const hydro_body* body, const hydro_ocean* ocean,
                               const hydro_settings* settings, hydro_wrench* io)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!body || !settings || !io || !valid_ocean(ocean))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "body forces: bad arguments");
    if (body->mesh != HYDRO_NO_MESH && body->mesh >= ctx->meshes.size())
        return fail(ctx, HYDRO_ERR_NOT_FOUND, "unknown mesh %u", body->mesh);
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    return run_single(ctx, *body, ocean, settings, *io, OP_BODY);
}

hydro_status hydro_surface_forces(hydro_ctx* ctx, const hydro_settings* settings, hydro_mesh_id mesh,
                                  const hydro_ocean* ocean, const hydro_transform* T_CG,
                                  const hydro_transform* T_C, const double v[3],
                                  const double omega[3], double Fb[3], double Tb[3],
                                  double Fdq[3], double Tdq[3], double Fdf[3], double Tdf[3],
                                  double* Swet, double* Vsub)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!settings || !valid_ocean(ocean) || !T_CG || !T_C || !v || !omega || !Fb || !Tb || !Fdq ||
        !Tdq || !Fdf || !Tdf || !Swet || !Vsub)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "surface forces: null argument");
    if (mesh != HYDRO_NO_MESH && mesh >= ctx->meshes.size())
        return fail(ctx, HYDRO_ERR_NOT_FOUND, "unknown mesh %u", mesh);
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    hydro_body b{};
    b.T_CG = *T_CG;
    b.T_C = *T_C;
    copy3(b.v, v);
    copy3(b.omega, omega);
    b.mesh = mesh;
    b.mode = HYDRO_MODE_SUBMERGED;
    b.buoyancy = 1;
    hydro_wrench w{};
    copy3(w.Fb, Fb); copy3(w.Tb, Tb); copy3(w.Fdq, Fdq); copy3(w.Tdq, Tdq);
    copy3(w.Fdf, Fdf); copy3(w.Tdf, Tdf);
    w.Swet = *Swet;
    w.Vsub = *Vsub;
    hydro_status st = run_single(ctx, b, ocean, settings, w, OP_SURFACE);
    if (st != HYDRO_OK) return st;
    copy3(Fb, w.Fb); copy3(Tb, w.Tb); copy3(Fdq, w.Fdq); copy3(Tdq, w.Tdq);
    copy3(Fdf, w.Fdf); copy3(Tdf, w.Tdf);
    *Swet = w.Swet;
    *Vsub = w.Vsub;
    return HYDRO_OK;
}

hydro_status hydro_submerged_forces(hydro_ctx* ctx, hydro_mesh_id mesh, const hydro_ocean* ocean,
                                    const hydro_transform* T_CG, const hydro_transform* T_C,
                                    const double v[3], const double omega[3], double Fdq[3],
                                    double Tdq[3], double Fdf[3], double Tdf[3])
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!valid_ocean(ocean) || !T_CG || !T_C || !v || !omega || !Fdq || !Tdq || !Fdf || !Tdf)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "submerged forces: null argument");
    if (mesh != HYDRO_NO_MESH && mesh >= ctx->meshes.size())
        return fail(ctx, HYDRO_ERR_NOT_FOUND, "unknown mesh %u", mesh);
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    hydro_body b{};
    b.T_CG = *T_CG;
    b.T_C = *T_C;
    copy3(b.v, v);
    copy3(b.omega, omega);
    b.mesh = mesh;
    b.mode = HYDRO_MODE_SUBMERGED;
    hydro_wrench w{};
    copy3(w.Fdq, Fdq); copy3(w.Tdq, Tdq); copy3(w.Fdf, Fdf); copy3(w.Tdf, Tdf);
    hydro_settings s{1, 0};
    hydro_status st = run_single(ctx, b, ocean, &s, w, OP_SUBMERGED);
    if (st != HYDRO_OK) return st;
    copy3(Fdq, w.Fdq); copy3(Tdq, w.Tdq); copy3(Fdf, w.Fdf); copy3(Tdf, w.Tdf);
    return HYDRO_OK;
}

hydro_status hydro_correct_forces(hydro_ctx* ctx, const hydro_ocean* ocean, double Fdq[3],
                                  double Tdq[3], double Fdf[3], double Tdf[3], const double Cd[3],
                                  const double Cf[3], const double R_O[9])
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!valid_ocean(ocean) || !Fdq || !Tdq || !Fdf || !Tdf || !Cd || !Cf || !R_O)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "correct forces: null argument");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    hydro_status st = ensure_small(ctx, 64 * sizeof(double));
    if (st != HYDRO_OK) return st;
    double h[27];
    copy3(h, Fdq); copy3(h + 3, Tdq); copy3(h + 6, Fdf); copy3(h + 9, Tdf);
    copy3(h + 12, Cd); copy3(h + 15, Cf);
    for (int i = 0; i < 9; ++i) h[18 + i] = R_O[i];
    double* d = static_cast<double*>(ctx->small_d);
    CK(ctx, cudaMemcpyAsync(d, h, sizeof(h), cudaMemcpyHostToDevice, ctx->stream));
    cudaError_t e = launch_correct(ocean->density, d, d + 12, d + 15, d + 18, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "correct kernel");
    CK(ctx, cudaMemcpyAsync(h, d, 12 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    copy3(Fdq, h); copy3(Tdq, h + 3); copy3(Fdf, h + 6); copy3(Tdf, h + 9);
    return HYDRO_OK;
}

// -------------------------------------------------------------- compounds
void compound_free(hydro_compound_batch* cb)
{
    if (!cb) return;
    if (cb->parts) batch_free(cb->parts);
    cudaFree(cb->cinfo_d);
    cudaFree(cb->part_compound_d);
    cudaFree(cb->compounds_d);
    cudaFree(cb->parts_d);
    cudaFree(cb->io_d);
    delete cb;
}

hydro_status hydro_compound_batch_create(hydro_ctx* ctx, const hydro_mesh_id* part_mesh,
                                         const uint32_t* parts_per_compound, uint32_t n_compounds,
                                         hydro_compound_batch** out)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!out || !parts_per_compound || n_compounds == 0)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "compound batch: null pointer or no compounds");
    *out = nullptr;
    uint64_t total = 0;
    for (uint32_t c = 0; c < n_compounds; ++c) total += parts_per_compound[c];
    if (total > 0xFFFFFFFull || (total && !part_mesh))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "compound batch: bad part list");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    hydro_compound_batch* cb = new (std::nothrow) hydro_compound_batch();
    if (!cb) return fail(ctx, HYDRO_ERR_OOM, "host allocation");
    cb->ctx = ctx;
    cb->n_compounds = n_compounds;
    cb->n_parts = (uint32_t)total;
    std::vector<CompoundInfo> info(n_compounds);
    std::vector<uint32_t> owner((size_t)total);
    uint32_t first = 0;
    for (uint32_t c = 0; c < n_compounds; ++c) {
        info[c] = CompoundInfo{first, parts_per_compound[c]};
        for (uint32_t k = 0; k < parts_per_compound[c]; ++k) owner[first + k] = c;
        first += parts_per_compound[c];
    }
    hydro_status st = HYDRO_OK;
    if (total) st = batch_build(ctx, part_mesh, (uint32_t)total, &cb->parts);
    if (st != HYDRO_OK) {
        compound_free(cb);
        return st;
    }
    cudaError_t e = cudaMalloc(&cb->cinfo_d, n_compounds * sizeof(CompoundInfo));
    if (e == cudaSuccess) e = cudaMalloc(&cb->part_compound_d, std::max<size_t>(1, total) * sizeof(uint32_t));
    if (e == cudaSuccess)
        e = cudaMemcpy(cb->cinfo_d, info.data(), n_compounds * sizeof(CompoundInfo), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && total)
        e = cudaMemcpy(cb->part_compound_d, owner.data(), total * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        compound_free(cb);
        return cuda_fail(ctx, e, "compound batch allocation");
    }
    *out = cb;
    return HYDRO_OK;
}

void hydro_compound_batch_destroy(hydro_compound_batch* cb)
{
    if (!cb) return;
    hydro_ctx* ctx = cb->ctx;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    compound_free(cb);
}

hydro_status compound_launch(hydro_compound_batch* cb, const hydro_body* d_compounds,
                             const hydro_compound_part* d_parts, const hydro_ocean* ocean,
                             const hydro_settings* settings, hydro_wrench* d_io, cudaStream_t s)
{
    hydro_ctx* ctx = cb->ctx;
    hydro_status st = sync_tiles(ctx);
    if (st != HYDRO_OK) return st;
    if (ocean->waves && !ctx->wave_d)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "ocean.waves set but no wave grid was given");
    KParams P{};
    hydro_batch* b = cb->parts;
    unsigned* err = nullptr;
    if (b) {
        P.chunks = b->chunks_d;
        P.binfo = b->binfo_d;
        P.partials = b->partials_d;
        P.bparams = b->bparams_d;
        P.active = b->active_d;
        P.n_bodies = b->n_bodies;
        P.n_chunks = b->n_chunks;
        std::memcpy(P.class_start, b->class_start, sizeof(P.class_start));
        err = b->err_d;
    } else {
        // no parts at all: a scratch error word from the context
        if ((st = ensure_small(ctx, 256)) != HYDRO_OK) return st;
        err = static_cast<unsigned*>(ctx->small_d);
        CK(ctx, cudaMemsetAsync(err, 0, 256, s));
    }
    P.tiles = ctx->tiles_d;
    P.err = err;
    P.work = err + 32;
    P.n_listed = err + 48;
    P.ocean = make_ocean(ctx, ocean);
    P.st.damping = settings->damping_forces ? 1 : 0;
    P.st.buoyancy = settings->realistic_buoyancy ? 1 : 0;
    P.op = OP_SURFACE;
    CompoundParams C{};
    C.compounds = d_compounds;
    C.parts = d_parts;
    C.cinfo = cb->cinfo_d;
    C.part_compound = cb->part_compound_d;
    C.io = d_io;
    C.n_compounds = cb->n_compounds;
    const int cut64 = ctx->cfg.cut_precision == HYDRO_CUT_FP64;
    LaunchShape shape{};
    const int want = (b && b->ctas_per_sm) ? (int)b->ctas_per_sm : ctx->cfg.ctas_per_sm ? (int)ctx->cfg.ctas_per_sm : 2;
    shape.ctas_per_sm = std::max(
        1, std::min(want, chunk_kernel_occupancy(cut64, P.ocean.waves, want, 0, P.ocean.field_currents)));
    shape.grid = ctx->sm_count * shape.ctas_per_sm;
    uint32_t launches = 0;
    cudaError_t e = launch_compound_step(P, C, shape, cut64, s, &launches);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "compound step launch");
    cb->last_launches = launches;
    return HYDRO_OK;
}

hydro_status hydro_compound_compute_device(hydro_compound_batch* cb, const hydro_body* d_compounds,
                                           const hydro_compound_part* d_parts, const hydro_ocean* ocean,
                                           const hydro_settings* settings, hydro_wrench* d_io, void* stream)
{
    if (!cb) return HYDRO_ERR_INVALID_ARG;
    hydro_ctx* ctx = cb->ctx;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!d_compounds || (!d_parts && cb->n_parts) || !d_io || !settings || !valid_ocean(ocean))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "compound compute: bad arguments");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    return compound_launch(cb, d_compounds, d_parts, ocean, settings, d_io, static_cast<cudaStream_t>(stream));
}

hydro_status hydro_compound_compute(hydro_compound_batch* cb, const hydro_body* compounds,
                                    const hydro_compound_part* parts, const hydro_ocean* ocean,
                                    const hydro_settings* settings, hydro_wrench* io)
{
    if (!cb) return HYDRO_ERR_INVALID_ARG;
    hydro_ctx* ctx = cb->ctx;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!compounds || (!parts && cb->n_parts) || !io || !settings || !valid_ocean(ocean))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "compound compute: bad arguments");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    const size_t nc = cb->n_compounds, np = std::max<uint32_t>(cb->n_parts, 1u);
    if (!cb->compounds_d) CK(ctx, cudaMalloc(&cb->compounds_d, nc * sizeof(hydro_body)));
    if (!cb->parts_d) CK(ctx, cudaMalloc(&cb->parts_d, np * sizeof(hydro_compound_part)));
    if (!cb->io_d) CK(ctx, cudaMalloc(&cb->io_d, nc * sizeof(hydro_wrench)));
    cudaStream_t s = ctx->stream;
    CK(ctx, cudaMemcpyAsync(cb->compounds_d, compounds, nc * sizeof(hydro_body), cudaMemcpyHostToDevice, s));
    if (cb->n_parts)
        CK(ctx, cudaMemcpyAsync(cb->parts_d, parts, cb->n_parts * sizeof(hydro_compound_part),
                                cudaMemcpyHostToDevice, s));
    CK(ctx, cudaMemcpyAsync(cb->io_d, io, nc * sizeof(hydro_wrench), cudaMemcpyHostToDevice, s));
    hydro_status st = compound_launch(cb, cb->compounds_d, cb->parts_d, ocean, settings, cb->io_d, s);
    if (st != HYDRO_OK) return st;
    CK(ctx, cudaMemcpyAsync(io, cb->io_d, nc * sizeof(hydro_wrench), cudaMemcpyDeviceToHost, s));
    CK(ctx, cudaStreamSynchronize(s));
    return HYDRO_OK;
}

// ------------------------------------------------------------ mesh ingest
hydro_status hydro_obj_parse(const char* text, size_t len, float scale, float refine_threshold, float* xyz,
                             uint32_t xyz_capacity, uint32_t* faces, uint32_t faces_capacity, uint32_t* n_vertices,
                             uint32_t* n_faces)
{
    if (!text || !n_vertices || !n_faces) return HYDRO_ERR_INVALID_ARG;
    std::vector<float> v;
    std::vector<uint32_t> f;
    std::string err;
    try {
        if (!parse_obj(text, len, scale, v, f, err)) return HYDRO_ERR_INVALID_ARG;
        if (refine_threshold > 0.f) refine_mesh(v, f, refine_threshold);
    } catch (...) {
        return HYDRO_ERR_OOM;
    }
    if (v.size() / 3 > 0xFFFFFFFFull || f.size() / 3 > 0xFFFFFFFFull) return HYDRO_ERR_INVALID_ARG;
    *n_vertices = (uint32_t)(v.size() / 3);
    *n_faces = (uint32_t)(f.size() / 3);
    if (xyz) {
        if (xyz_capacity < *n_vertices) return HYDRO_ERR_INVALID_ARG;
        memcpy(xyz, v.data(), v.size() * sizeof(float));
    }
    if (faces) {
        if (faces_capacity < *n_faces) return HYDRO_ERR_INVALID_ARG;
        memcpy(faces, f.data(), f.size() * sizeof(uint32_t));
    }
    return HYDRO_OK;
}

hydro_status hydro_mesh_upload_obj(hydro_ctx* ctx, const char* text, size_t len, float scale, float refine_threshold,
                                   hydro_mesh_id* out_id)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!text || !out_id) return fail(ctx, HYDRO_ERR_INVALID_ARG, "obj upload: null argument");
    std::vector<float> v;
    std::vector<uint32_t> f;
    std::string err;
    try {
        if (!parse_obj(text, len, scale, v, f, err)) return fail(ctx, HYDRO_ERR_INVALID_ARG, "obj: %s", err.c_str());
        if (refine_threshold > 0.f) refine_mesh(v, f, refine_threshold);
    } catch (...) {
        return fail(ctx, HYDRO_ERR_OOM, "obj: host allocation");
    }
    return hydro_mesh_upload(ctx, v.data(), 3 * sizeof(float), (uint32_t)(v.size() / 3), f.data(),
                             (uint32_t)(f.size() / 3), out_id);
}

hydro_status hydro_mesh_compute_properties(hydro_ctx* ctx, hydro_mesh_id mesh, double thickness, double density,
                                           hydro_mesh_properties* out)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!out) return fail(ctx, HYDRO_ERR_INVALID_ARG, "mesh properties: null argument");
    if (mesh >= ctx->meshes.size()) return fail(ctx, HYDRO_ERR_NOT_FOUND, "unknown mesh %u", mesh);
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    hydro_status st = sync_tiles(ctx);
    if (st != HYDRO_OK) return st;
    const MeshRec& m = ctx->meshes[mesh];
    const size_t bytes = (size_t)std::max<uint32_t>(m.n_tiles, 1u) * 12 * sizeof(double);
    if ((st = ensure_small(ctx, bytes)) != HYDRO_OK) return st;
    double* d = static_cast<double*>(ctx->small_d);
    std::vector<double> part((size_t)m.n_tiles * 12);
    double s0[12] = {0}, s1[12] = {0};
    for (int pass = 0; pass < 2; ++pass) {
        double3 cg = make_double3(0.0, 0.0, 0.0);
        if (pass == 1) {
            hydro_mesh_properties tmp{};
            finish_properties(thickness, density, s0, s1, &tmp);
            cg = make_double3(tmp.CG[0], tmp.CG[1], tmp.CG[2]);
        }
        cudaError_t e = launch_mesh_props(ctx->tiles_d, m.first_tile, m.n_tiles, pass, thickness, cg, d, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "mesh properties kernel");
        CK(ctx, cudaMemcpyAsync(part.data(), d, part.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        CK(ctx, cudaStreamSynchronize(ctx->stream));
        double* acc = pass == 0 ? s0 : s1;
        for (uint32_t t = 0; t < m.n_tiles; ++t)
            for (int k = 0; k < 12; ++k) acc[k] += part[(size_t)t * 12 + k];
    }
    finish_properties(thickness, density, s0, s1, out);
    return HYDRO_OK;
}

// -------------------------------------------------------------- FFT ocean
void hydro_fft_ocean_params_for_state(float state, hydro_fft_ocean_params* p)
{
    if (!p) return;
    p->wind = state * 5.f + 2.f;
    p->omega = 5.f * expf(-state) + 0.2f;
    p->amplitude = 1.f;
    p->km = 370.f;
    p->cm = 0.23f;
    p->grid_sizes[0] = 893.f;
    p->grid_sizes[1] = 101.f;
    p->grid_sizes[2] = 21.f;
    p->grid_sizes[3] = 11.f;
    p->passes = 8;
    p->propagate = 1;
}

void fft_ocean_free(hydro_fft_ocean* o)
{
    if (!o) return;
    cudaFree(o->s12_d);
    cudaFree(o->s34_d);
    cudaFree(o->idx_d);
    cudaFree(o->w_d);
    delete o;
}

hydro_status hydro_fft_ocean_create(hydro_ctx* ctx, const hydro_fft_ocean_params* params, hydro_fft_ocean** out)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!params || !out || params->passes < 2 || params->passes > 10 || !(params->wind > 0.f) ||
        !(params->omega > 0.f))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "fft ocean: bad parameters");
    for (int g = 0; g < 4; ++g)
        if (!(params->grid_sizes[g] > 0.f)) return fail(ctx, HYDRO_ERR_INVALID_ARG, "fft ocean: bad grid size");
    *out = nullptr;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    hydro_fft_ocean* o = new (std::nothrow) hydro_fft_ocean();
    if (!o) return fail(ctx, HYDRO_ERR_OOM, "host allocation");
    o->ctx = ctx;
    o->p = *params;
    o->N = 1u << params->passes;
    std::vector<float4> s12, s34;
    std::vector<int2> idx;
    std::vector<float2> w;
    fft_ocean_spectrum(o->p, s12, s34);
    fft_ocean_butterfly((int)o->p.passes, idx, w);
    const size_t nn = (size_t)o->N * o->N;
    cudaError_t e = cudaMalloc(&o->s12_d, nn * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&o->s34_d, nn * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&o->idx_d, idx.size() * sizeof(int2));
    if (e == cudaSuccess) e = cudaMalloc(&o->w_d, w.size() * sizeof(float2));
    if (e == cudaSuccess) e = cudaMemcpy(o->s12_d, s12.data(), nn * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(o->s34_d, s34.data(), nn * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(o->idx_d, idx.data(), idx.size() * sizeof(int2), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(o->w_d, w.data(), w.size() * sizeof(float2), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        fft_ocean_free(o);
        return cuda_fail(ctx, e, "fft ocean allocation");
    }
    // the context's wave grid becomes the N x N x 4 readback, zero until the first update
    std::vector<float> zero(nn * 4, 0.f);
    const uint32_t ch[2] = {0, 1};
    const float gs[2] = {params->grid_sizes[0], params->grid_sizes[1]};
    hydro_status st = hydro_wave_grid_set(ctx, zero.data(), o->N, 4, 2, ch, gs);
    if (st != HYDRO_OK) {
        fft_ocean_free(o);
        return st;
    }
    *out = o;
    return HYDRO_OK;
}

void hydro_fft_ocean_destroy(hydro_fft_ocean* o)
{
    if (!o) return;
    std::lock_guard<std::recursive_mutex> lk(o->ctx->mu);
    cudaSetDevice(o->ctx->device);
    fft_ocean_free(o);
}

hydro_status hydro_fft_ocean_update(hydro_fft_ocean* o, float t, void* stream)
{
    if (!o) return HYDRO_ERR_INVALID_ARG;
    hydro_ctx* ctx = o->ctx;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!ctx->wave_d || ctx->wave_n != o->N || ctx->wave_channels != 4)
        return fail(ctx, HYDRO_ERR_MISMATCH, "fft ocean: the context's wave grid was replaced");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    // inverseGridSizes = 2 pi N / L, evaluated in double and stored as float (OpenGLOcean.cpp:469-472)
    const double two_pi = 2.0 * 3.14159265358979323846;
    const float4 ig = make_float4((float)(two_pi * (float)o->N / o->p.grid_sizes[0]),
                                  (float)(two_pi * (float)o->N / o->p.grid_sizes[1]),
                                  (float)(two_pi * (float)o->N / o->p.grid_sizes[2]),
                                  (float)(two_pi * (float)o->N / o->p.grid_sizes[3]));
    cudaError_t e = launch_fft_ocean(o->s12_d, o->s34_d, o->idx_d, o->w_d, (int)o->p.passes, ig, t,
                                     reinterpret_cast<float4*>(ctx->wave_d), static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? HYDRO_OK : cuda_fail(ctx, e, "fft ocean kernels");
}

hydro_status hydro_fft_ocean_read(hydro_fft_ocean* o, float* out)
{
    if (!o || !out) return HYDRO_ERR_INVALID_ARG;
    hydro_ctx* ctx = o->ctx;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    CK(ctx, cudaDeviceSynchronize());
    CK(ctx, cudaMemcpy(out, ctx->wave_d, (size_t)o->N * o->N * 4 * sizeof(float), cudaMemcpyDeviceToHost));
    return HYDRO_OK;
}

// ----------------------------------------------------------------- cables
// Segment scratch (9 doubles per node) followed by one error word.
hydro_status cable_scratch(hydro_ctx* ctx, uint32_t n_nodes)
{
    const size_t need = (size_t)std::max<uint32_t>(n_nodes, 1u) * 9 + 32;
    if (ctx->cable_cap >= need) return HYDRO_OK;
    cudaFree(ctx->cable_seg);
    ctx->cable_seg = nullptr;
    ctx->cable_cap = 0;
    CK(ctx, cudaMalloc(&ctx->cable_seg, need * sizeof(double)));
    ctx->cable_cap = need;
    return HYDRO_OK;
}

hydro_status hydro_cable_forces_device(hydro_ctx* ctx, const hydro_cable* d_cables, uint32_t n_cables,
                                       const double* d_x, const double* d_v, uint32_t n_nodes_total,
                                       const hydro_ocean* ocean, const hydro_settings* settings,
                                       hydro_cable_node_forces* d_out, void* stream)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if ((n_cables && (!d_cables || !d_x || !d_v || !d_out)) || !settings || !valid_ocean(ocean))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "cable forces: bad arguments");
    if (ocean->waves && !ctx->wave_d) return fail(ctx, HYDRO_ERR_INVALID_ARG, "no wave grid");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    hydro_status st = cable_scratch(ctx, n_nodes_total);
    if (st != HYDRO_OK) return st;
    SettingsDev sd;
    sd.damping = settings->damping_forces ? 1 : 0;
    sd.buoyancy = settings->realistic_buoyancy ? 1 : 0;
    unsigned* bad = reinterpret_cast<unsigned*>(ctx->cable_seg + ctx->cable_cap - 32);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    CK(ctx, cudaMemsetAsync(bad, 0, sizeof(unsigned), s));
    cudaError_t e = launch_cable(d_cables, n_cables, n_nodes_total, d_x, d_v, make_ocean(ctx, ocean), sd,
                                 ctx->cable_seg, d_out, bad, s);
    return e == cudaSuccess ? HYDRO_OK : cuda_fail(ctx, e, "cable kernel");
}

hydro_status hydro_cable_forces(hydro_ctx* ctx, const hydro_cable* cables, uint32_t n_cables, const double* x,
                                const double* v, uint32_t n_nodes_total, const hydro_ocean* ocean,
                                const hydro_settings* settings, hydro_cable_node_forces* out)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if ((n_cables && (!cables || !x || !v || !out)) || !settings || !valid_ocean(ocean))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "cable forces: bad arguments");
    for (uint32_t c = 0; c < n_cables; ++c)
        if ((uint64_t)cables[c].first_node + cables[c].n_nodes > n_nodes_total)
            return fail(ctx, HYDRO_ERR_INDEX_RANGE, "cable %u: nodes beyond n_nodes_total", c);
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    const size_t bc = (size_t)n_cables * sizeof(hydro_cable), bx = (size_t)n_nodes_total * 3 * sizeof(double);
    const size_t bo = (size_t)n_nodes_total * sizeof(hydro_cable_node_forces);
    const size_t o1 = (bc + 255) & ~size_t(255), o2 = o1 + ((bx + 255) & ~size_t(255));
    const size_t o3 = o2 + ((bx + 255) & ~size_t(255)), need = o3 + bo + 256;
    if (ctx->cable_stage_cap < need) {
        cudaFree(ctx->cable_stage);
        ctx->cable_stage = nullptr;
        ctx->cable_stage_cap = 0;
        CK(ctx, cudaMalloc(&ctx->cable_stage, need));
        ctx->cable_stage_cap = need;
    }
    char* base = static_cast<char*>(ctx->cable_stage);
    cudaStream_t s = ctx->stream;
    if (bc) CK(ctx, cudaMemcpyAsync(base, cables, bc, cudaMemcpyHostToDevice, s));
    if (bx) {
        CK(ctx, cudaMemcpyAsync(base + o1, x, bx, cudaMemcpyHostToDevice, s));
        CK(ctx, cudaMemcpyAsync(base + o2, v, bx, cudaMemcpyHostToDevice, s));
        CK(ctx, cudaMemcpyAsync(base + o3, out, bo, cudaMemcpyHostToDevice, s));
    }
    hydro_status st = hydro_cable_forces_device(ctx, reinterpret_cast<const hydro_cable*>(base), n_cables,
                                                reinterpret_cast<const double*>(base + o1),
                                                reinterpret_cast<const double*>(base + o2), n_nodes_total, ocean,
                                                settings, reinterpret_cast<hydro_cable_node_forces*>(base + o3), s);
    if (st != HYDRO_OK) return st;
    if (bo) CK(ctx, cudaMemcpyAsync(out, base + o3, bo, cudaMemcpyDeviceToHost, s));
    CK(ctx, cudaStreamSynchronize(s));
    return HYDRO_OK;
}

// ------------------------------------------------------------ aerodynamics
hydro_status hydro_aero_forces(hydro_ctx* ctx, hydro_mesh_id mesh, const hydro_atmosphere* atm,
                               const hydro_transform* T_CG, const hydro_transform* T_C, const double v[3],
                               const double omega[3], double Fda[3], double Tda[3])
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!valid_atmosphere(atm) || !T_CG || !T_C || !v || !omega || !Fda || !Tda)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "aero forces: null argument");
    if (mesh != HYDRO_NO_MESH && mesh >= ctx->meshes.size())
        return fail(ctx, HYDRO_ERR_NOT_FOUND, "unknown mesh %u", mesh);
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    hydro_batch* b = nullptr;
    hydro_status st = single_batch(ctx, mesh, &b);
    if (st != HYDRO_OK) return st;
    if ((st = ensure_small(ctx, sizeof(hydro_aero_wrench))) != HYDRO_OK) return st;
    hydro_body body{};
    body.T_CG = *T_CG;
    body.T_C = *T_C;
    copy3(body.v, v);
    copy3(body.omega, omega);
    body.mesh = mesh;
    body.mode = HYDRO_MODE_AERODYNAMIC;
    hydro_aero_wrench w{};
    hydro_aero_wrench* d = static_cast<hydro_aero_wrench*>(ctx->small_d);
    const hydro_ocean o = atmosphere_ocean(atm);
    const hydro_settings none{0, 0};
    CK(ctx, cudaMemcpyAsync(b->bodies_d, &body, sizeof(body), cudaMemcpyHostToDevice, ctx->stream));
    CK(ctx, cudaMemcpyAsync(d, &w, sizeof(w), cudaMemcpyHostToDevice, ctx->stream));
    st = batch_launch(b, b->bodies_d, &o, &none, nullptr, ctx->stream, OP_AERO, nullptr, d, nullptr);
    if (st != HYDRO_OK) return st;
    CK(ctx, cudaMemcpyAsync(&w, d, sizeof(w), cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    copy3(Fda, w.Fda);
    copy3(Tda, w.Tda);
    return HYDRO_OK;
}

hydro_status hydro_aero_correct(hydro_ctx* ctx, const hydro_aero_params* params, double Fda[3], double Tda[3])
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!params || !Fda || !Tda) return fail(ctx, HYDRO_ERR_INVALID_ARG, "aero correct: null argument");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    hydro_status st = ensure_small(ctx, 256 + sizeof(hydro_aero_params));
    if (st != HYDRO_OK) return st;
    double h[6];
    copy3(h, Fda);
    copy3(h + 3, Tda);
    unsigned char* base = static_cast<unsigned char*>(ctx->small_d);
    double* d = reinterpret_cast<double*>(base);
    hydro_aero_params* dp = reinterpret_cast<hydro_aero_params*>(base + 256);
    CK(ctx, cudaMemcpyAsync(d, h, sizeof(h), cudaMemcpyHostToDevice, ctx->stream));
    CK(ctx, cudaMemcpyAsync(dp, params, sizeof(*params), cudaMemcpyHostToDevice, ctx->stream));
    cudaError_t e = launch_aero_correct(dp, d, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "aero correct kernel");
    CK(ctx, cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    copy3(Fda, h);
    copy3(Tda, h + 3);
    return HYDRO_OK;
}

hydro_status hydro_batch_compute_aero_device(hydro_batch* b, const hydro_body* d_bodies,
                                             const hydro_aero_params* d_params, const hydro_atmosphere* atm,
                                             hydro_aero_wrench* d_out, void* stream)
{
    if (!b) return HYDRO_ERR_INVALID_ARG;
    hydro_ctx* ctx = b->ctx;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!d_bodies || !d_params || !d_out || !valid_atmosphere(atm))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "aero batch: bad arguments");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    const hydro_ocean o = atmosphere_ocean(atm);
    const hydro_settings none{0, 0};
    return batch_launch(b, d_bodies, &o, &none, nullptr, static_cast<cudaStream_t>(stream), OP_AERO_BODY, nullptr,
                        d_out, d_params);
}

hydro_status hydro_batch_compute_aero(hydro_batch* b, const hydro_body* bodies, const hydro_aero_params* params,
                                      const hydro_atmosphere* atm, hydro_aero_wrench* out)
{
    if (!b) return HYDRO_ERR_INVALID_ARG;
    hydro_ctx* ctx = b->ctx;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!bodies || !params || !out || !valid_atmosphere(atm))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "aero batch: bad arguments");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    const size_t nb = (size_t)b->n_bodies;
    if (!b->bodies_d) CK(ctx, cudaMalloc(&b->bodies_d, nb * sizeof(hydro_body)));
    if (!b->aparams_d) CK(ctx, cudaMalloc(&b->aparams_d, nb * sizeof(hydro_aero_params)));
    if (!b->aio_d) CK(ctx, cudaMalloc(&b->aio_d, nb * sizeof(hydro_aero_wrench)));
    CK(ctx, cudaMemcpyAsync(b->bodies_d, bodies, nb * sizeof(hydro_body), cudaMemcpyHostToDevice, b->stream));
    CK(ctx, cudaMemcpyAsync(b->aparams_d, params, nb * sizeof(hydro_aero_params), cudaMemcpyHostToDevice,
                            b->stream));
    CK(ctx, cudaMemcpyAsync(b->aio_d, out, nb * sizeof(hydro_aero_wrench), cudaMemcpyHostToDevice, b->stream));
    const hydro_ocean o = atmosphere_ocean(atm);
    const hydro_settings none{0, 0};
    hydro_status st = batch_launch(b, b->bodies_d, &o, &none, nullptr, b->stream, OP_AERO_BODY, nullptr, b->aio_d,
                                   b->aparams_d);
    if (st != HYDRO_OK) return st;
    CK(ctx, cudaMemcpyAsync(out, b->aio_d, nb * sizeof(hydro_aero_wrench), cudaMemcpyDeviceToHost, b->stream));
    CK(ctx, cudaStreamSynchronize(b->stream));
    return HYDRO_OK;
}

hydro_status hydro_fluid_position(hydro_ctx* ctx, const hydro_ocean* ocean, const double aabb_min[3],
                                  const double aabb_max[3], int32_t* position)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!valid_ocean(ocean) || !aabb_min || !aabb_max || !position)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "fluid position: null argument");
    if (ocean->waves && !ctx->wave_d) return fail(ctx, HYDRO_ERR_INVALID_ARG, "no wave grid");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    hydro_status st = ensure_small(ctx, 64);
    if (st != HYDRO_OK) return st;
    double h[6];
    copy3(h, aabb_min);
    copy3(h + 3, aabb_max);
    double* d = static_cast<double*>(ctx->small_d);
    int* r = reinterpret_cast<int*>(d + 6);
    CK(ctx, cudaMemcpyAsync(d, h, sizeof(h), cudaMemcpyHostToDevice, ctx->stream));
    cudaError_t e = launch_fluid_position(make_ocean(ctx, ocean), d, r, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "fluid position kernel");
    int32_t out = 0;
    CK(ctx, cudaMemcpyAsync(&out, r, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    *position = out;
    return HYDRO_OK;
}

// The DEBUG_HYDRO outline of one body: the kernel writes per face a record
// of 13 floats (corner count, up to four corners of the evaluated submerged
// part), expanded here into line segments on the host.
hydro_status hydro_debug_surface_outline(hydro_ctx* ctx, const hydro_body* body, const hydro_ocean* ocean,
                                         const hydro_settings* settings, float* points, uint32_t capacity,
                                         uint32_t* n_points)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!body || !valid_ocean(ocean) || !settings || !n_points || (capacity && !points) ||
        body->mesh >= ctx->meshes.size())
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "surface outline: bad arguments");
    if (ocean->waves && !ctx->wave_d) return fail(ctx, HYDRO_ERR_INVALID_ARG, "no wave grid");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    hydro_status st = sync_tiles(ctx);
    if (st != HYDRO_OK) return st;
    const MeshRec& m = ctx->meshes[body->mesh];
    const size_t bytes = (size_t)m.n_faces * 13 * sizeof(float);
    st = ensure_small(ctx, bytes + sizeof(hydro_body) + 256);
    if (st != HYDRO_OK) return st;
    char* base = static_cast<char*>(ctx->small_d);
    hydro_body* db = reinterpret_cast<hydro_body*>(base);
    float* dout = reinterpret_cast<float*>(base + 256 * ((sizeof(hydro_body) + 255) / 256));
    CK(ctx, cudaMemcpyAsync(db, body, sizeof(hydro_body), cudaMemcpyHostToDevice, ctx->stream));
    SettingsDev sd{settings->damping_forces ? 1 : 0, settings->realistic_buoyancy ? 1 : 0};
    cudaError_t e = launch_outline(ctx->tiles_d, m.first_tile, m.n_tiles, db, make_ocean(ctx, ocean), sd,
                                   ctx->cfg.cut_precision == HYDRO_CUT_FP64, dout, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "outline kernel");
    std::vector<float> rec((size_t)m.n_faces * 13);
    CK(ctx, cudaMemcpyAsync(rec.data(), dout, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    // segments in the reference's order: faces in mesh order, each outline
    // as (c0, c1), (c1, c2), ..., (c_last, c0)
    uint32_t n = 0;
    for (size_t f = 0; f < m.n_faces; ++f) {
        const float* r = &rec[f * 13];
        const int k = std::min(std::max((int)r[0], 0), 4);   // a record holds at most four corners
        for (int i = 0; i < k; ++i) {
            const float* c[2] = {r + 1 + 3 * i, r + 1 + 3 * ((i + 1) % k)};
            for (int j = 0; j < 2; ++j, ++n)
                if (n < capacity) std::memcpy(points + 3 * (size_t)n, c[j], 3 * sizeof(float));
        }
    }
    *n_points = n;
    return HYDRO_OK;
}

hydro_status hydro_debug_face_terms(hydro_ctx* ctx, const hydro_body* body, const hydro_ocean* ocean,
                                    const hydro_settings* settings, int32_t packed, float* out)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!body || !valid_ocean(ocean) || !settings || !out || body->mesh >= ctx->meshes.size())
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "face terms: bad arguments");
    if (ocean->waves && !ctx->wave_d) return fail(ctx, HYDRO_ERR_INVALID_ARG, "no wave grid");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    hydro_status st = sync_tiles(ctx);
    if (st != HYDRO_OK) return st;
    const MeshRec& m = ctx->meshes[body->mesh];
    const size_t terms = (size_t)m.n_faces * kQ * sizeof(float);
    st = ensure_small(ctx, terms + sizeof(hydro_body) + 256);
    if (st != HYDRO_OK) return st;
    char* base = static_cast<char*>(ctx->small_d);
    hydro_body* db = reinterpret_cast<hydro_body*>(base);
    float* dout = reinterpret_cast<float*>(base + 256 * ((sizeof(hydro_body) + 255) / 256));
    CK(ctx, cudaMemcpyAsync(db, body, sizeof(hydro_body), cudaMemcpyHostToDevice, ctx->stream));
    SettingsDev sd{settings->damping_forces ? 1 : 0, settings->realistic_buoyancy ? 1 : 0};
    cudaError_t e = launch_face_terms(ctx->tiles_d, m.first_tile, m.n_tiles, db, make_ocean(ctx, ocean), sd,
                                      ctx->frame, ctx->cfg.cut_precision == HYDRO_CUT_FP64, packed ? 1 : 0,
                                      dout, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "face terms kernel");
    CK(ctx, cudaMemcpyAsync(out, dout, terms, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    return HYDRO_OK;
}

hydro_status hydro_debug_tile_order(const uint32_t* face_indices, uint32_t n_vertices, uint32_t n_faces,
                                    uint32_t* order, uint32_t* tile_starts, uint32_t starts_capacity,
                                    uint32_t* n_tiles)
{
    if (!face_indices || !order || !tile_starts || !n_tiles || n_vertices == 0 || n_faces == 0)
        return HYDRO_ERR_INVALID_ARG;
    for (size_t i = 0; i < (size_t)n_faces * 3; ++i)
        if (face_indices[i] >= n_vertices) return HYDRO_ERR_INDEX_RANGE;
    std::vector<uint32_t> ord, starts;
    build_tiles(n_vertices, face_indices, n_faces, ord, starts);
    *n_tiles = (uint32_t)starts.size() - 1u;
    if (starts.size() > (size_t)starts_capacity) return HYDRO_ERR_INVALID_ARG;
    std::memcpy(order, ord.data(), ord.size() * sizeof(uint32_t));
    std::memcpy(tile_starts, starts.data(), starts.size() * sizeof(uint32_t));
    return HYDRO_OK;
}

hydro_status hydro_debug_division_check(hydro_ctx* ctx, uint64_t n_pairs, uint64_t seed,
                                       uint64_t mismatches[3])
{
    return hydro_debug_arith_check(ctx, n_pairs, seed, mismatches, nullptr, nullptr);
}

hydro_status hydro_debug_arith_check(hydro_ctx* ctx, uint64_t n_pairs, uint64_t seed,
                                     uint64_t division[3], uint64_t packed[4], float examples[16])
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!division) return fail(ctx, HYDRO_ERR_INVALID_ARG, "arithmetic check: null output");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    hydro_status st = ensure_small(ctx, 256);
    if (st != HYDRO_OK) return st;
    unsigned long long* d = static_cast<unsigned long long*>(ctx->small_d);
    float* dex = reinterpret_cast<float*>(d + 8);
    CK(ctx, cudaMemsetAsync(d, 0, 8 * sizeof(unsigned long long) + 16 * sizeof(float), ctx->stream));
    cudaError_t e = launch_division_check(n_pairs, seed, d, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "division check kernel");
    if (packed) {
        e = launch_packed_check(n_pairs, seed + 1, d, dex, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "packed check kernel");
    }
    unsigned long long h[8];
    float hex[16];
    CK(ctx, cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaMemcpyAsync(hex, dex, sizeof(hex), cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < 3; ++i) division[i] = h[i];
    if (packed)
        for (int i = 0; i < 4; ++i) packed[i] = h[3 + i];
    if (examples)
        for (int i = 0; i < 16; ++i) examples[i] = hex[i];
    return HYDRO_OK;
}

}  // extern "C"

extern "C" hydro_status hydro_debug_wait_timeout(hydro_ctx* ctx, uint32_t limit_us, int32_t* status)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!status || limit_us == 0 || limit_us > 2000000u)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "wait check: limit must be in 1..2000000 us");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    hydro_status st = ensure_small(ctx, 64);
    if (st != HYDRO_OK) return st;
    int* d = static_cast<int*>(ctx->small_d);
    CK(ctx, cudaMemsetAsync(d, 0xff, sizeof(int), ctx->stream));
    cudaError_t e = launch_wait_timeout((uint64_t)limit_us * 1000ull, d, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "wait check kernel");
    int h = -1;
    CK(ctx, cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    *status = h;
    return HYDRO_OK;
}

// ============================================================ autotuner
namespace {

// Cache key: the GPU, the arithmetic variant and the batch's shape (body
// count per power-of-two face-count bin, total faces).
std::string tune_key(const hydro_ctx* ctx, const hydro_batch* b, int waves)
{
    uint32_t bins[32] = {0};
    uint64_t total = 0;
    for (uint32_t i = 0; i < b->n_bodies; ++i) {
        const uint32_t m = b->mesh_of_body[i];
        const uint32_t f = m == HYDRO_NO_MESH ? 0u : ctx->meshes[m].n_faces;
        total += f;
        int k = 0;
        while (k < 31 && (1u << (k + 1)) <= f) ++k;
        ++bins[f ? k + 1 : 0];
    }
    std::string key = std::string(ctx->gpu_name) + "|sm" + std::to_string(ctx->sm_count) + "|cut" +
                      std::to_string(ctx->cfg.cut_precision) + "|waves" + std::to_string(waves) + "|n" +
                      std::to_string(b->n_bodies) + "|f" + std::to_string(total) + "|h";
    for (int k = 0; k < 32; ++k)
        if (bins[k]) key += std::to_string(k) + ":" + std::to_string(bins[k]) + ",";
    for (char& c : key)
        if (c == ' ' || c == '\n' || c == '\t') c = '_';
    return key;
}

bool tune_lookup(const std::string& path, const std::string& key, uint32_t* faces, uint32_t* ctas, float* ms)
{
    if (path.empty()) return false;
    FILE* f = fopen(path.c_str(), "r");
    if (!f) return false;
    char line[2048];
    bool found = false;
    while (fgets(line, sizeof(line), f)) {
        char k[1800];
        unsigned a = 0, c = 0;
        float t = 0.f;
        if (sscanf(line, "%1799s %u %u %f", k, &a, &c, &t) == 4 && key == k) {
            *faces = a;
            *ctas = c;
            *ms = t;
            found = true;   // the last entry for a key wins
        }
    }
    fclose(f);
    return found;
}

}  // namespace

extern "C" hydro_status hydro_batch_autotune(hydro_batch* b, const hydro_body* d_bodies,
                                             const hydro_ocean* ocean, const hydro_settings* settings,
                                             hydro_wrench* d_scratch, void* stream, uint32_t reps,
                                             hydro_tune_result* out)
{
    if (!b) return HYDRO_ERR_INVALID_ARG;
    hydro_ctx* ctx = b->ctx;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (!d_bodies || !d_scratch || !settings || !valid_ocean(ocean) || !out)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "autotune: bad arguments");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");
    if (reps == 0) reps = 5;
    memset(out, 0, sizeof(*out));
    const std::string key = tune_key(ctx, b, ocean->waves);
    uint32_t faces = 0, ctas = 0;
    float ms = 0.f;
    if (tune_lookup(ctx->tune_path, key, &faces, &ctas, &ms)) {
        hydro_status st = build_work(ctx, b, tiles_per_chunk(ctx, faces));
        if (st != HYDRO_OK) return st;
        b->ctas_per_sm = ctas;
        out->chunk_faces = b->chunk_tiles * kTileFaces;
        out->ctas_per_sm = ctas;
        out->ms_per_step = ms;
        out->from_cache = 1;
        return HYDRO_OK;
    }
    static const uint32_t kTiles[] = {2, 4, 8, 11, 16, 24, 32};
    static const uint32_t kCtas[] = {1, 2};
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(ctx, cudaEventCreate(&e0));
    CK(ctx, cudaEventCreate(&e1));
    float best = 1e30f;
    uint32_t best_t = kTiles[0], best_c = kCtas[0], n = 0;
    hydro_status st = HYDRO_OK;
    for (uint32_t t : kTiles) {
        if ((st = build_work(ctx, b, t)) != HYDRO_OK) break;
        for (uint32_t c : kCtas) {
            b->ctas_per_sm = c;
            if ((st = batch_launch(b, d_bodies, ocean, settings, d_scratch, s, OP_BODY)) != HYDRO_OK) break;
            cudaEventRecord(e0, s);
            for (uint32_t r = 0; r < reps && st == HYDRO_OK; ++r)
                st = batch_launch(b, d_bodies, ocean, settings, d_scratch, s, OP_BODY);
            cudaEventRecord(e1, s);
            cudaError_t e = cudaEventSynchronize(e1);
            if (st != HYDRO_OK) break;
            if (e != cudaSuccess) {
                st = cuda_fail(ctx, e, "autotune timing");
                break;
            }
            float t_ms = 0.f;
            cudaEventElapsedTime(&t_ms, e0, e1);
            t_ms /= (float)reps;
            if (n < 16) out->candidate_ms[n] = t_ms;
            ++n;
            if (t_ms < best) {
                best = t_ms;
                best_t = t;
                best_c = c;
            }
        }
        if (st != HYDRO_OK) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != HYDRO_OK) return st;
    if ((st = build_work(ctx, b, best_t)) != HYDRO_OK) return st;
    b->ctas_per_sm = best_c;
    out->chunk_faces = best_t * kTileFaces;
    out->ctas_per_sm = best_c;
    out->ms_per_step = best;
    out->from_cache = 0;
    out->n_candidates = n;
    if (!ctx->tune_path.empty()) {
        FILE* f = fopen(ctx->tune_path.c_str(), "a");
        if (f) {
            fprintf(f, "%s %u %u %.6f\n", key.c_str(), out->chunk_faces, best_c, best);
            fclose(f);
        }
    }
    return HYDRO_OK;
}

// ====================================================== surrogate kernels
#define NN_CTX_CHECK()                                                                        \
    if (!ctx) return HYDRO_ERR_INVALID_ARG;                                                   \
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);                                        \
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice")

#define NN_RET(e, what) return (e) == cudaSuccess ? HYDRO_OK : cuda_fail(ctx, (e), (what))

// Room for `floats` split-K partial products in the context's workspace,
// grown on demand; not grown while the stream captures a graph (the GEMM
// then runs unsplit).  Returns false only when an allocation failed.
static bool nn_workspace(hydro_ctx* ctx, size_t floats, cudaStream_t s)
{
    if (floats <= ctx->nn_ws_floats) return true;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return true;
    }
    float* p = nullptr;
    if (cudaMalloc(&p, floats * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (ctx->nn_ws) {
        cudaDeviceSynchronize();   // a product on any stream may still read the old workspace
        cudaFree(ctx->nn_ws);
    }
    ctx->nn_ws = p;
    ctx->nn_ws_floats = floats;
    return true;
}

extern "C" hydro_status hydro_nn_gemm(hydro_ctx* ctx, int32_t epilogue, const void* A, int32_t lda,
                                      const void* B, int32_t ldb, int32_t M, int32_t N, int32_t K,
                                      float* z, void* y, const float* bias, const float* zprev,
                                      int32_t ldc, void* stream)
{
    NN_CTX_CHECK();
    if (!A || !B || M <= 0 || N <= 0 || K <= 0 || M % 64 || N % 64 || K % 32 || lda < K || ldb < N ||
        ldc < N || epilogue < 0 || epilogue > 3)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn gemm: bad shape (M, N multiples of 64, K of 32)");
    if ((epilogue == 0 || epilogue == 2) && !z)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn gemm: missing z");
    if ((epilogue == 1 || epilogue == 3) && !y) return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn gemm: missing y");
    if ((epilogue == 1 || epilogue == 2) && !bias) return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn gemm: missing bias");
    if (epilogue == 3 && !zprev) return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn gemm: missing zprev");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t ws = (size_t)gemm_splits(epilogue, M, N, K) * (size_t)M * (size_t)N;
    if (ws > (size_t)M * (size_t)N && !nn_workspace(ctx, ws, st))
        return fail(ctx, HYDRO_ERR_OOM, "nn gemm: split-K workspace");
    cudaError_t e = launch_gemm(epilogue, A, lda, B, ldb, M, N, K, z, y, bias, zprev, ldc, st, ctx->nn_ws,
                                ctx->nn_ws_floats);
    NN_RET(e, "nn gemm");
}

extern "C" hydro_status hydro_nn_transpose(hydro_ctx* ctx, const void* src, void* dst, int32_t rows,
                                           int32_t cols, void* stream)
{
    NN_CTX_CHECK();
    if (!src || !dst || rows <= 0 || cols <= 0) return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn transpose");
    NN_RET(launch_transpose(src, dst, rows, cols, static_cast<cudaStream_t>(stream)), "nn transpose");
}

extern "C" hydro_status hydro_nn_mse_grad(hydro_ctx* ctx, const float* z, const float* target, int32_t rows,
                                          int32_t ld, int32_t n_out, const float* tmean, const float* tistd,
                                          void* dz, double* loss, void* stream)
{
    NN_CTX_CHECK();
    if (!z || !target || !dz || rows <= 0 || n_out <= 0 || ld < n_out || (!tmean) != (!tistd) ||
        (uint64_t)rows * (uint64_t)ld >= (1ull << 32))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn mse");
    NN_RET(launch_mse_grad(z, target, rows, ld, n_out, tmean, tistd, dz, loss, static_cast<cudaStream_t>(stream)),
           "nn mse");
}

extern "C" hydro_status hydro_nn_colsum(hydro_ctx* ctx, const void* g, int32_t rows, int32_t cols, float* out,
                                        void* stream)
{
    NN_CTX_CHECK();
    if (!g || !out || rows <= 0 || cols <= 0) return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn colsum");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t ws = (size_t)colsum_slabs(rows) * (size_t)cols;
    if (ws > (size_t)cols && !nn_workspace(ctx, ws, st)) return fail(ctx, HYDRO_ERR_OOM, "nn colsum: workspace");
    NN_RET(launch_colsum(g, rows, cols, out, st, ctx->nn_ws, ctx->nn_ws_floats), "nn colsum");
}

extern "C" hydro_status hydro_nn_adamw(hydro_ctx* ctx, float* w, float* m, float* v, const float* grad,
                                       int32_t rows, int32_t cols, int32_t ldg, float lr, float beta1,
                                       float beta2, float eps, float weight_decay, int32_t step, void* w16,
                                       void* wt16, void* stream)
{
    NN_CTX_CHECK();
    if (!w || !m || !v || !grad || rows <= 0 || cols <= 0 || ldg < cols || step < 1)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn adamw");
    NN_RET(launch_adamw(w, m, v, grad, rows, cols, ldg, lr, beta1, beta2, eps, weight_decay, step, w16, wt16,
                        static_cast<cudaStream_t>(stream)), "nn adamw");
}

// The training loop: per step the forward GEMMs (bias + SiLU epilogues,
// then bias), the MSE gradient, and per layer from the last the transposed
// input, the weight-gradient GEMM, the bias-gradient column sums and the
// gradient GEMM through the SiLU derivative; then AdamW on every layer's
// weights (decayed) and bias (not decayed).  The launch sequence is the one
// a caller makes with the single entry points, kernel for kernel.
extern "C" hydro_status hydro_nn_train(hydro_ctx* ctx, const hydro_nn_net* net, const void* X, const float* T,
                                       int64_t n_rows, const int64_t* rows, const float* lr, int32_t n_steps,
                                       int32_t step0, float beta1, float beta2, float eps, float weight_decay,
                                       void* stream)
{
    NN_CTX_CHECK();
    if (!net || !X || !T || !rows || !lr || n_steps < 0 || step0 < 0 || n_rows <= 0)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn train: missing argument");
    const int B = net->batch;
    if (B <= 0 || B % 64 || net->n_out <= 0 || net->n_out > net->layer[3].n || !net->loss)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn train: batch must be a positive multiple of 64");
    for (int l = 0; l < 4; ++l) {
        const hydro_nn_layer& L = net->layer[l];
        if (!L.w || !L.b || !L.mw || !L.vw || !L.mb || !L.vb || !L.gw || !L.gb || !L.w16 || !L.wt16 || !net->z[l] ||
            !net->dz[l] || !net->xt[l] || (l < 3 && !net->x[l]) || L.k <= 0 || L.n <= 0 || L.k % 64 || L.n % 64 ||
            (l > 0 && L.k != net->layer[l - 1].n))
            return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn train: bad layer (k, n multiples of 64, chained)");
    }
    if ((!net->tmean) != (!net->tistd) || (uint64_t)B * (uint64_t)net->layer[3].n >= (1ull << 32))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn train: bad target normalisation");
    for (int32_t s = 0; s < n_steps; ++s)
        if (rows[s] < 0 || rows[s] > n_rows - B || (int64_t)step0 + s + 1 > (int64_t)INT32_MAX)
            return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn train: batch rows out of range");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const hydro_nn_layer* Ls = net->layer;
    const int k0 = Ls[0].k, n_out = net->n_out;
    size_t ws = 0;
    for (int l = 0; l < 4; ++l) {
        ws = std::max(ws, (size_t)gemm_splits(0, Ls[l].k, Ls[l].n, B) * (size_t)Ls[l].k * (size_t)Ls[l].n);
        ws = std::max(ws, (size_t)colsum_slabs(B) * (size_t)Ls[l].n);
    }
    if (!nn_workspace(ctx, ws, st)) return fail(ctx, HYDRO_ERR_OOM, "nn train: split-K workspace");
    cudaError_t e = cudaSuccess;
#define NN_TRAIN(call)                                  \
    do {                                                \
        e = (call);                                     \
        if (e != cudaSuccess) return cuda_fail(ctx, e, "nn train: " #call); \
    } while (0)
    for (int32_t s = 0; s < n_steps; ++s) {
        const void* X0 = static_cast<const unsigned char*>(X) + (size_t)rows[s] * (size_t)k0 * 2u;
        const float* T0 = T + (size_t)rows[s] * (size_t)n_out;
        const void* ins[4] = {X0, net->x[0], net->x[1], net->x[2]};
        for (int l = 0; l < 3; ++l)
            NN_TRAIN(launch_gemm(1, ins[l], Ls[l].k, Ls[l].w16, Ls[l].n, B, Ls[l].n, Ls[l].k, net->z[l], net->x[l],
                                 Ls[l].b, nullptr, Ls[l].n, st));
        NN_TRAIN(launch_gemm(2, ins[3], Ls[3].k, Ls[3].w16, Ls[3].n, B, Ls[3].n, Ls[3].k, net->z[3], nullptr, Ls[3].b,
                             nullptr, Ls[3].n, st));
        NN_TRAIN(launch_mse_grad(net->z[3], T0, B, Ls[3].n, n_out, net->tmean, net->tistd, net->dz[3], net->loss, st));
        for (int l = 3; l >= 0; --l) {
            const hydro_nn_layer& L = Ls[l];
            NN_TRAIN(launch_transpose(ins[l], net->xt[l], B, L.k, st));
            NN_TRAIN(launch_gemm(0, net->xt[l], B, net->dz[l], L.n, L.k, L.n, B, L.gw, nullptr, nullptr, nullptr,
                                 L.n, st, ctx->nn_ws, ctx->nn_ws_floats));
            NN_TRAIN(launch_colsum(net->dz[l], B, L.n, L.gb, st, ctx->nn_ws, ctx->nn_ws_floats));
            if (l > 0)
                NN_TRAIN(launch_gemm(3, net->dz[l], L.n, L.wt16, L.k, B, L.k, L.n, nullptr, net->dz[l - 1], nullptr,
                                     net->z[l - 1], L.k, st));
        }
        const int step = step0 + s + 1;
        for (int l = 0; l < 4; ++l) {
            const hydro_nn_layer& L = Ls[l];
            NN_TRAIN(launch_adamw(L.w, L.mw, L.vw, L.gw, L.k, L.n, L.n, lr[s], beta1, beta2, eps, weight_decay, step,
                                  L.w16, L.wt16, st));
            NN_TRAIN(launch_adamw(L.b, L.mb, L.vb, L.gb, 1, L.n, L.n, lr[s], beta1, beta2, eps, 0.0f, step, nullptr,
                                  nullptr, st));
        }
    }
#undef NN_TRAIN
    return HYDRO_OK;
}

extern "C" hydro_status hydro_nn_to_bf16(hydro_ctx* ctx, const float* x, int32_t rows, int32_t n_in, int32_t ld,
                                         const float* mean, const float* istd, void* y, void* stream)
{
    NN_CTX_CHECK();
    if (!x || !y || rows <= 0 || n_in <= 0 || ld < n_in || (!mean) != (!istd) ||
        (uint64_t)rows * (uint64_t)ld >= (1ull << 32))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn to_bf16");
    NN_RET(launch_to_bf16(x, rows, n_in, ld, mean, istd, y, static_cast<cudaStream_t>(stream)), "nn to_bf16");
}

extern "C" hydro_status hydro_nn_features(hydro_ctx* ctx, const hydro_body* d_bodies, uint32_t n,
                                          const hydro_ocean* ocean, float* d_features, void* stream)
{
    NN_CTX_CHECK();
    if (!d_bodies || !d_features || !valid_ocean(ocean)) return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn features");
    if (ocean->waves && !ctx->wave_d) return fail(ctx, HYDRO_ERR_INVALID_ARG, "no wave grid");
    NN_RET(launch_features(d_bodies, n, make_ocean(ctx, ocean), d_features, static_cast<cudaStream_t>(stream)),
           "nn features");
}

extern "C" hydro_status hydro_nn_gate(hydro_ctx* ctx, const float* d_features, uint32_t n, const float* lo,
                                      const float* hi, const float* mean, const float* precision,
                                      float threshold, uint8_t* d_mask, void* stream)
{
    NN_CTX_CHECK();
    if (!d_features || !lo || !hi || !mean || !precision || !d_mask || (reinterpret_cast<uintptr_t>(d_features) & 15))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn gate (features must be 16-byte aligned)");
    NN_RET(launch_gate(d_features, n, lo, hi, mean, precision, threshold, d_mask,
                       static_cast<cudaStream_t>(stream)), "nn gate");
}

extern "C" hydro_status hydro_nn_wrench_body(hydro_ctx* ctx, const hydro_body* d_bodies,
                                             const hydro_wrench* d_wrenches, uint32_t n, float* d_out,
                                             void* stream)
{
    NN_CTX_CHECK();
    if (!d_bodies || !d_wrenches || !d_out) return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn wrench_body");
    NN_RET(launch_wrench_body(d_bodies, d_wrenches, n, d_out, static_cast<cudaStream_t>(stream)),
           "nn wrench_body");
}

extern "C" hydro_status hydro_nn_pack_sw128(hydro_ctx* ctx, const void* src, int32_t rows, int32_t K, int32_t ld,
                                            int32_t kpad, void* dst, void* stream)
{
    NN_CTX_CHECK();
    if (!src || !dst || rows <= 0 || K <= 0 || kpad % 64 || K > kpad || ld < K ||
        (reinterpret_cast<uintptr_t>(dst) & 15))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn pack_sw128");
    NN_RET(launch_pack_sw128(src, rows, K, ld, kpad, dst, static_cast<cudaStream_t>(stream)), "nn pack_sw128");
}

extern "C" hydro_status hydro_nn_mlp_tc(hydro_ctx* ctx, const float* d_features, uint32_t n, const float* fmean,
                                        const float* fistd, const void* d_image, const float* b0, const float* b1,
                                        const float* b2, const float* b3, float* d_out, uint32_t* d_err,
                                        void* stream)
{
    NN_CTX_CHECK();
    if (!d_features || !fmean || !fistd || !d_image || !b0 || !b1 || !b2 || !b3 || !d_out || !d_err ||
        (reinterpret_cast<uintptr_t>(d_image) & 15) || (reinterpret_cast<uintptr_t>(d_out) & 15))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn mlp_tc");
    NN_RET(launch_mlp_tc(d_features, n, fmean, fistd, d_image, b0, b1, b2, b3, d_out, d_err,
                         static_cast<cudaStream_t>(stream)), "nn mlp_tc");
}

extern "C" hydro_status hydro_nn_route(hydro_ctx* ctx, const hydro_body* d_bodies, const uint8_t* d_mask,
                                       uint32_t n, uint32_t* d_counts, hydro_body* d_packed, int32_t* d_pos,
                                       uint32_t* d_n_packed, hydro_wrench* d_exact, void* stream)
{
    NN_CTX_CHECK();
    if (!d_bodies || !d_mask || !d_counts || !d_packed || !d_pos || !d_n_packed)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn route");
    NN_RET(launch_route(d_bodies, d_mask, n, d_counts, d_packed, d_pos, d_n_packed, d_exact,
                        static_cast<cudaStream_t>(stream)), "nn route");
}

extern "C" hydro_status hydro_nn_merge(hydro_ctx* ctx, const hydro_body* d_bodies, const float* d_z, int32_t ld,
                                       const int32_t* d_pos, const hydro_wrench* d_exact, uint32_t n,
                                       float* d_out, void* stream)
{
    NN_CTX_CHECK();
    if (!d_bodies || !d_z || ld < 6 || !d_pos || !d_exact || !d_out)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn merge");
    NN_RET(launch_merge(d_bodies, d_z, ld, d_pos, d_exact, n, d_out, static_cast<cudaStream_t>(stream)),
           "nn merge");
}

extern "C" hydro_status hydro_nn_gate_inside(hydro_ctx* ctx, const hydro_body* d_bodies, uint32_t n,
                                             const hydro_ocean* ocean, uint8_t* d_mask, void* stream)
{
    NN_CTX_CHECK();
    if (!d_bodies || !d_mask || !valid_ocean(ocean)) return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn gate inside");
    if (ocean->waves && !ctx->wave_d) return fail(ctx, HYDRO_ERR_INVALID_ARG, "ocean.waves set but no wave grid");
    NN_RET(launch_gate_inside(d_bodies, n, make_ocean(ctx, ocean), d_mask, static_cast<cudaStream_t>(stream)),
           "nn gate inside");
}

extern "C" hydro_status hydro_nn_ensemble(hydro_ctx* ctx, float* d_za, const float* d_zb, int32_t ld, uint32_t n,
                                          double force_scale, double torque_scale, float tau, uint8_t* d_mask,
                                          void* stream)
{
    NN_CTX_CHECK();
    if (!d_za || !d_zb || ld < 6 || !d_mask || !(force_scale > 0.0) || !(torque_scale > 0.0))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn ensemble");
    NN_RET(launch_ensemble(d_za, d_zb, ld, n, (float)(1.0 / force_scale), (float)(1.0 / torque_scale), tau, d_mask,
                           static_cast<cudaStream_t>(stream)), "nn ensemble");
}

extern "C" hydro_status hydro_nn_audit_pick(hydro_ctx* ctx, uint8_t* d_mask, uint32_t n, uint32_t stride,
                                            uint32_t phase, uint32_t k, int32_t* d_idx, void* stream)
{
    NN_CTX_CHECK();
    if (!d_mask || !d_idx || stride == 0) return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn audit pick");
    NN_RET(launch_audit_pick(d_mask, n, stride, phase, k, d_idx, static_cast<cudaStream_t>(stream)), "nn audit pick");
}

extern "C" hydro_status hydro_nn_audit_error(hydro_ctx* ctx, const hydro_body* d_bodies, const float* d_z,
                                             int32_t ld, const int32_t* d_pos, const hydro_wrench* d_exact,
                                             const int32_t* d_idx, uint32_t k, double force_scale,
                                             double torque_scale, float* d_err, void* stream)
{
    NN_CTX_CHECK();
    if (!d_bodies || !d_z || ld < 6 || !d_pos || !d_exact || !d_idx || !d_err || !(force_scale > 0.0) ||
        !(torque_scale > 0.0))
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "nn audit error");
    NN_RET(launch_audit_error(d_bodies, d_z, ld, d_pos, d_exact, d_idx, k, (float)(1.0 / force_scale),
                              (float)(1.0 / torque_scale), d_err, static_cast<cudaStream_t>(stream)),
           "nn audit error");
}

// ====================================================== rigid-body rollout
extern "C" hydro_status hydro_rigid_step(hydro_ctx* ctx, hydro_rigid_state* d_states, hydro_body* d_bodies,
                                         const hydro_wrench* d_exact, const float* d_body_wrench, uint32_t n,
                                         double dt, double gravity, void* stream)
{
    NN_CTX_CHECK();
    if (!d_states || !d_bodies || !(dt > 0.0)) return fail(ctx, HYDRO_ERR_INVALID_ARG, "rigid step");
    NN_RET(launch_rigid_step(d_states, d_bodies, d_exact, d_body_wrench, n, dt, gravity,
                             static_cast<cudaStream_t>(stream)), "rigid step");
}

extern "C" hydro_status hydro_rigid_write_bodies(hydro_ctx* ctx, const hydro_rigid_state* d_states,
                                                 hydro_body* d_bodies, uint32_t n, void* stream)
{
    NN_CTX_CHECK();
    if (!d_states || !d_bodies) return fail(ctx, HYDRO_ERR_INVALID_ARG, "rigid write bodies");
    NN_RET(launch_rigid_write_bodies(d_states, d_bodies, n, static_cast<cudaStream_t>(stream)),
           "rigid write bodies");
}

// ====================================================== allocation-free step
// Some callers cannot allocate device memory while they run: a simulator
// that evaluates the hydrodynamics inside its real-time tick (cudaMalloc
// may synchronise the device and stall the tick for milliseconds), or an
// application whose device memory is reserved up front by another
// allocator.  hydro_compute_wrenches_static runs the batched step with all
// of its scratch (work list, per-body parameters, per-chunk partial sums,
// error word) in one static device array instead of memory it allocates.
// Every GPU that loads this library holds the array until the process
// exits.  Calls share it: the last call's contents stay in it, and calls
// whose work overlaps on the GPU race.
namespace {

constexpr size_t kStaticScratchBytes = HYDRO_STATIC_SCRATCH_BYTES;
constexpr uint32_t kStaticMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_static_mu;
void* g_static_ptr[kStaticMaxDevices] = {};
ChunkDesc g_static_chunks[kStaticScratchBytes / 224];
BodyInfo g_static_binfo[HYDRO_STATIC_MAX_BODIES];

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

extern "C" hydro_status hydro_compute_wrenches_static(hydro_ctx* ctx, const hydro_mesh_id* mesh_of_body,
                                                      uint32_t n_bodies, const hydro_body* d_bodies,
                                                      const hydro_ocean* ocean,
                                                      const hydro_settings* settings,
                                                      hydro_wrench* d_inout, void* stream)
{
    if (!ctx) return HYDRO_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    std::lock_guard<std::mutex> slk(g_static_mu);
    if (!mesh_of_body || !d_bodies || !d_inout || !settings || !valid_ocean(ocean) || n_bodies == 0)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "static step: bad arguments");
    if (n_bodies > HYDRO_STATIC_MAX_BODIES)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "static step: %u bodies exceed the maximum of %u",
                    n_bodies, (unsigned)HYDRO_STATIC_MAX_BODIES);
    if (ocean->waves && !ctx->wave_d)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "ocean.waves set but no wave grid was given");
    if ((uint32_t)ctx->device >= kStaticMaxDevices)
        return fail(ctx, HYDRO_ERR_UNSUPPORTED, "static step: device ordinal %d too large", ctx->device);
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HYDRO_ERR_DEVICE, "cudaSetDevice");

    // Set-up, once per device with that device current: the device address
    // of the static array (its name in host code is only a stand-in).
    void*& base_ptr = g_static_ptr[ctx->device];
    if (!base_ptr) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGetSymbolAddress(static scratch)");
        base_ptr = p;
    }

    // The device tile table must already hold every uploaded mesh; copying
    // missing entries is allowed, growing it (an allocation) is not.
    if (ctx->tiles_h.size() > ctx->tiles_d_cap)
        return fail(ctx, HYDRO_ERR_INVALID_ARG,
                    "static step: the device tile table must grow; create a batch (or call any "
                    "other compute entry point) once after uploading meshes");
    if (ctx->tiles_d_count < ctx->tiles_h.size()) {
        CK(ctx, cudaMemcpy(ctx->tiles_d + ctx->tiles_d_count, ctx->tiles_h.data() + ctx->tiles_d_count,
                           (ctx->tiles_h.size() - ctx->tiles_d_count) * sizeof(TileDesc),
                           cudaMemcpyHostToDevice));
        ctx->tiles_d_count = ctx->tiles_h.size();
    }

    // Work list into static host arrays (no heap allocation).
    const uint32_t tpc = tiles_per_chunk(ctx);
    const size_t max_chunks = sizeof(g_static_chunks) / sizeof(g_static_chunks[0]);
    size_t nc = 0;
    for (uint32_t i = 0; i < n_bodies; ++i) {
        const uint32_t mesh = mesh_of_body[i];
        if (mesh != HYDRO_NO_MESH && mesh >= ctx->meshes.size())
            return fail(ctx, HYDRO_ERR_NOT_FOUND, "body %u: unknown mesh %u", i, mesh);
        BodyInfo& bi = g_static_binfo[i];
        bi.first_chunk = (uint32_t)nc;
        bi.mesh = mesh;
        uint32_t first = 0, nt = 0;
        if (mesh != HYDRO_NO_MESH) {
            first = ctx->meshes[mesh].first_tile;
            nt = ctx->meshes[mesh].n_tiles;
            bi.n_faces = ctx->meshes[mesh].n_faces;
        } else {
            bi.n_faces = 0;
        }
        uint32_t k = 0;
        for (uint32_t t = 0; t < nt || k == 0; t += tpc, ++k) {
            if (nc >= max_chunks)
                return fail(ctx, HYDRO_ERR_INVALID_ARG, "static step: more than %zu chunks", max_chunks);
            g_static_chunks[nc++] = ChunkDesc{i, first + t, nt > t ? std::min(tpc, nt - t) : 0u, k};
            if (nt == 0) { ++k; break; }
        }
        bi.n_chunks = (uint32_t)nc - bi.first_chunk;
    }

    // Layout of the static array.
    const size_t off_err = 0;
    const size_t off_binfo = align256(off_err + 256);
    const size_t off_bparams = align256(off_binfo + (size_t)n_bodies * sizeof(BodyInfo));
    const size_t off_chunks = align256(off_bparams + (size_t)n_bodies * sizeof(BodyParams));
    const size_t off_active = align256(off_chunks + nc * sizeof(ChunkDesc));
    const size_t off_partials = align256(off_active + nc * sizeof(ActiveChunk));
    const size_t total = off_partials + nc * kPartialStride * sizeof(double);
    if (total > kStaticScratchBytes)
        return fail(ctx, HYDRO_ERR_INVALID_ARG, "static step: needs %zu scratch bytes, the maximum is %zu",
                    total, kStaticScratchBytes);

    char* base = static_cast<char*>(base_ptr);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // The control block (error word, claim counters, the count of listed
    // chunks) must start at zero.  A previous call that failed between its
    // launches can leave a count behind in the shared array, so every call
    // clears the block on its own stream first (a memset allocates nothing).
    CK(ctx, cudaMemsetAsync(base + off_err, 0, 256, s));
    // The work list goes up from pageable host arrays: cudaMemcpyAsync stages
    // pageable memory and may make the host wait for that.
    CK(ctx, cudaMemcpyAsync(base + off_binfo, g_static_binfo, (size_t)n_bodies * sizeof(BodyInfo),
                            cudaMemcpyHostToDevice, s));
    CK(ctx, cudaMemcpyAsync(base + off_chunks, g_static_chunks, nc * sizeof(ChunkDesc),
                            cudaMemcpyHostToDevice, s));

    KParams P{};
    P.chunks = reinterpret_cast<const ChunkDesc*>(base + off_chunks);
    P.binfo = reinterpret_cast<const BodyInfo*>(base + off_binfo);
    P.tiles = ctx->tiles_d;
    P.bodies = d_bodies;
    P.io = d_inout;
    P.bparams = reinterpret_cast<BodyParams*>(base + off_bparams);
    P.partials = reinterpret_cast<double*>(base + off_partials);
    P.err = reinterpret_cast<unsigned*>(base + off_err);
    P.work = reinterpret_cast<unsigned*>(base + off_err) + 32;
    P.n_listed = reinterpret_cast<unsigned*>(base + off_err) + 48;
    P.active = reinterpret_cast<ActiveChunk*>(base + off_active);
    P.n_bodies = n_bodies;
    P.n_chunks = (uint32_t)nc;
    P.ocean = make_ocean(ctx, ocean);
    P.st.damping = settings->damping_forces ? 1 : 0;
    P.st.buoyancy = settings->realistic_buoyancy ? 1 : 0;
    P.op = OP_BODY;
    P.frame = ctx->frame;
    claim_class_starts(g_static_chunks, nc, P.class_start);
    const int cut64 = ctx->cfg.cut_precision == HYDRO_CUT_FP64;
    LaunchShape shape{};
    const int want = ctx->cfg.ctas_per_sm ? (int)ctx->cfg.ctas_per_sm : 2;
    shape.ctas_per_sm = std::max(
        1, std::min(want, chunk_kernel_occupancy(cut64, P.ocean.waves, want, 0, P.ocean.field_currents)));
    shape.grid = ctx->sm_count * shape.ctas_per_sm;
    uint32_t launches = 0;
    cudaError_t e = launch_step(P, shape, cut64, s, &launches);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "static wrench step launch");
    return HYDRO_OK;
}
