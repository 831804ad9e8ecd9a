// api.cu -- the C ABI (include/hrt.h): contexts, BLAS/TLAS objects, frames, batches.
// Host code only; kernels live in build.cu and trace.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "hrt_internal.h"

using namespace hrt;

struct hrt_context {
    int device = 0;
    int sm_count = 0;
    std::string last_error;
};

struct hrt_blas {
    hrt_context* ctx = nullptr;
    int type = 0, precision = 0;
    float transform[16];
    uint64_t nprims = 0;
    float build_ms = 0.0f;
    bool keep = false;
    float voxel_grid[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // voxels: origin xyz, size, res xyz
    BuildOutput out;
    // the topology, kept on the host for hrt_blas_refit
    uint32_t max_leaf = 1;
    uint64_t nvertices = 0, nstrands = 0;
    float const_radius = 0.0f;
    bool has_radius = false, has_normals = false;
    std::vector<uint32_t> line_off, vert_off, line_idx, tri_idx;
    // mesh material (device copies owned by the BLAS)
    float albedo[4] = {1.0f, 1.0f, 1.0f, 1.0f};
    float* uv = nullptr;  // float[ntris][6]
    float4* albedo_map = nullptr;
    uint32_t map_w = 0, map_h = 0;
};

namespace {
// Host copy of n uint32 values from host or device memory.
bool copy_u32(const uint32_t* src, uint64_t n, int32_t memory, std::vector<uint32_t>& dst) {
    dst.resize(n);
    if (!n) return true;
    if (memory == HRT_MEMORY_HOST) {
        memcpy(dst.data(), src, n * 4);
        return true;
    }
    return cudaMemcpy(dst.data(), src, n * 4, cudaMemcpyDeviceToHost) == cudaSuccess;
}
}  // namespace

struct hrt_tlas {
    hrt_context* ctx = nullptr;
    DevInstance* dev = nullptr;
    TlasNode* nodes = nullptr;  // instance BVH (null with fewer than two non-empty instances)
    uint32_t n = 0, nnodes = 0;
    uint32_t precision_mask = 0;  // bit per hrt_precision present
    uint32_t type_mask = 0;       // bit per hrt_geometry_type present
    uint64_t nprims = 0;          // primitives of all instances (a batch's cost estimate)
};

namespace {
// The frame-kernel build a launch uses: one node format when all its BLASes share it and every
// scene has one instance; otherwise the build that walks TLASes and takes each instance's format.
int node_mode(uint32_t precision_mask, bool any_tlas) {
    if (any_tlas || precision_mask == 3u) return kNodesPerInstance;
    if (precision_mask == (1u << HRT_PRECISION_QUANTISED)) return kNodesQ;
    return kNodesF;
}
}  // namespace

struct hrt_frame {
    hrt_context* ctx = nullptr;
    uint32_t w = 0, h = 0, spp = 0;
    float4* fb = nullptr;
    hrt_hit* hits = nullptr;
    SceneLaunch* dscene = nullptr;
    TraceCounters* counters = nullptr;
    uint32_t* resolve_list = nullptr;  // one entry per pixel (FP64 pass)
    float4* resolve_scratch = nullptr; // per-sample colours of the FP64 pass
    uint64_t scratch_cap = 0;
    hrt_frame_stats stats{};
    bool stats_pending = false;
    uint64_t pending_primary = 0;
};

// Scenes of one launch sequence, ordered by group (one group per primitive type when split),
// with the device resources the launches share: the scene table, one counter block per
// group, and the FP64 pass's pixel list and sample scratch (reused group after group, since
// the groups run in stream order).
struct ScenePlan {
    struct Group {
        uint32_t first = 0, count = 0, type_mask = 0, precision_mask = 0;
        bool any_tlas = false;
        uint64_t work = 0;
    };
    std::vector<SceneLaunch> table;
    std::vector<uint32_t> pos;  // table position of input scene i
    std::vector<Group> groups;
    uint64_t primary = 0, npix = 0, nsamp = 0, scap = 0;
    uint32_t max_spp = 1;
    SceneLaunch* dtable = nullptr;
    TraceCounters* counters = nullptr;
    uint32_t* list = nullptr;
    float4* scratch = nullptr;
    void release() {
        if (dtable) cudaFree(dtable);
        if (counters) cudaFree(counters);
        if (list) cudaFree(list);
        if (scratch) cudaFree(scratch);
        dtable = nullptr;
        counters = nullptr;
        list = nullptr;
        scratch = nullptr;
    }
};

struct hrt_batch {
    hrt_context* ctx = nullptr;
    ScenePlan plan;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<hrt_frame*> frames;
    bool async = false;
    // the groups' counters as the last replay left them (page-locked; the graph ends with their
    // copy), and an event recorded after each replay: async replays report a device error at
    // the next synchronising download, or at the next launch once the replay has finished
    TraceCounters* host_ctr = nullptr;
    cudaEvent_t done = nullptr;
    bool launched = false;
};

namespace {

// Log level from the environment variable HRT_LOG: 0 (default) silent, 1 failures, 2 also each
// build's summary; lines go to stderr with the prefix "[hrt]".
int log_level() {
    static const int level = [] {
        const char* v = getenv("HRT_LOG");
        return v ? int(strtol(v, nullptr, 10)) : 0;
    }();
    return level;
}

hrt_status fail(hrt_context* ctx, hrt_status s, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (ctx) ctx->last_error = buf;
    if (log_level() >= 1) fprintf(stderr, "[hrt] error %d (%s): %s\n", int(s), hrt_status_string(s), buf);
    return s;
}

// An NVTX range over a public entry point, so that profilers show the library's calls on their
// timelines (a no-op unless a profiler is attached).
struct Range {
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
};

hrt_status cuda_fail(hrt_context* ctx, cudaError_t e, const char* what) {
    if (e == cudaErrorMemoryAllocation)
        return fail(ctx, HRT_ERR_OOM, "%s: out of device memory", what);
    return fail(ctx, HRT_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(ctx, call, what)                                         \
    do {                                                            \
        cudaError_t e_ = (call);                                    \
        if (e_ != cudaSuccess) return cuda_fail((ctx), e_, (what)); \
    } while (0)

struct DeviceSet {  // makes ctx->device current for the scope of a call
    int prev = -1;
    explicit DeviceSet(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceSet() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

bool is_identity(const float* m) {
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r)
            if (m[4 * c + r] != (c == r ? 1.0f : 0.0f)) return false;
    return true;
}

// The status a launch's device error word stands for.
hrt_status error_status(hrt_context* ctx, uint32_t error) {
    if (error & kErrBounds)
        return fail(ctx, HRT_ERR_BOUNDS, "a device index check failed (a node, leaf slot or stream entry outside its array)");
    if (error & kErrStackOverflow)
        return fail(ctx, HRT_ERR_STACK_OVERFLOW, "a traversal overflowed its stack (max_depth entries, at most %d)",
                    kStackSize);
    if (error & kErrTimeout) return fail(ctx, HRT_ERR_TIMEOUT, "a traversal exceeded its step bound (max_steps)");
    return HRT_OK;
}

hrt_status read_counters(hrt_context* ctx, TraceCounters* dev, TraceCounters* host, cudaStream_t s) {
    CK(ctx, cudaMemcpyAsync(host, dev, sizeof(TraceCounters), cudaMemcpyDeviceToHost, s), "read counters");
    CK(ctx, cudaStreamSynchronize(s), "synchronise trace");
    return error_status(ctx, host->error);
}

// Traversal bounds of a launch from the caller's parameters (0 = the defaults).
RayBounds bounds_of(const hrt_trace_params* p) {
    return RayBounds{p->max_steps ? p->max_steps : kMaxTraversalSteps,
                     p->max_depth ? int32_t(p->max_depth) : int32_t(kStackSize)};
}

// Checks of the parameters every trace entry point shares.
hrt_status check_params(hrt_context* ctx, const hrt_trace_params* p, const char* who) {
    if (!(p->tmax > p->tmin)) return fail(ctx, HRT_ERR_INVALID_ARG, "%s: tmax must exceed tmin", who);
    if (p->shading > HRT_SHADE_LAMBERT_SHADOW) return fail(ctx, HRT_ERR_INVALID_ARG, "%s: unknown shading %u", who, p->shading);
    if (p->max_depth > uint32_t(kStackSize))
        return fail(ctx, HRT_ERR_INVALID_ARG, "%s: max_depth %u exceeds the %d-entry traversal stack", who, p->max_depth,
                    kStackSize);
    return HRT_OK;
}

void counters_to_stats(const TraceCounters& c, uint64_t primary, hrt_frame_stats* st) {
    st->primary_rays = primary;
    st->shadow_rays = c.shadow;
    st->nodes_visited = c.nodes;
    st->prims_tested = c.prims;
    st->fp64_resolves = c.fp64_resolves;
    st->fp64_hits = c.fp64_hits;
    st->warp_cycles_node = c.cycles_node;
    st->warp_cycles_leaf = c.cycles_leaf;
    st->warp_cycles_other = c.cycles_other;
}

void fill_scene(SceneLaunch& sl, const hrt_tlas* t, const hrt_camera* cam, hrt_frame* f, uint64_t work_begin) {
    sl.inst = t->dev;
    sl.tlas = t->nodes;
    sl.ninst = t->n;
    sl.width = f->w;
    sl.height = f->h;
    sl.spp = f->spp;
    sl.tiles_x = (f->w + 7) / 8;
    uint64_t tiles_y = (f->h + 3) / 4;
    sl.work_begin = work_begin;
    sl.work_count = uint64_t(sl.tiles_x) * tiles_y * 32;
    memcpy(sl.view_inv, cam->view_inverse, sizeof(sl.view_inv));
    memcpy(sl.proj_inv, cam->proj_inverse, sizeof(sl.proj_inv));
    sl.fb = f->fb;
    sl.hits = f->hits;
}

// The primitive type shared by every instance (selects a specialised kernel), or 3.
uint32_t prim_kind(uint32_t type_mask) {
    for (uint32_t k = 0; k < 3; ++k)
        if (type_mask == (1u << k)) return k;
    return 3;
}

// Samples the FP64 pass can run one per lane (beyond that it runs one pixel per lane).
constexpr uint64_t kScratchSamples = 1ull << 18;

TraceLaunch make_launch(const hrt_trace_params* p, const SceneLaunch* ds, uint32_t n, uint64_t total, TraceCounters* c,
                        uint32_t type_mask, uint32_t* resolve_list, uint64_t resolve_cap, float4* scratch,
                        uint64_t scratch_cap, uint32_t max_spp) {
    TraceLaunch L;
    L.prim_kind = prim_kind(type_mask);
    L.scenes = ds;
    L.nscenes = n;
    L.total_work = total;
    L.tmin = p->tmin;
    L.tmax = p->tmax;
    L.shadow_tmin = p->shadow_tmin;
    L.jitter = p->jitter;
    L.seed = p->seed;
    L.shading = p->shading;
    L.fp64_resolve = p->fp64_resolve;
    L.record_hits = p->record_hits;
    L.count_stats = p->count_stats;
    L.variant = p->kernel_variant;
    const uint32_t kind = prim_kind(type_mask);
    if (kind < 3 && ((p->variant_by_type >> (4 * kind)) & 15u)) L.variant = (p->variant_by_type >> (4 * kind)) & 15u;
    L.refill = p->refill > 32 ? 32 : p->refill;
    L.speculative = p->speculative;
    L.leaf_again = p->leaf_again > 32 ? 32 : p->leaf_again;
    const RayBounds rb = bounds_of(p);
    L.max_steps = rb.max_steps;
    L.max_depth = rb.max_depth;
    L.counters = c;
    L.resolve_list = resolve_list;
    L.resolve_cap = resolve_cap;
    L.resolve_scratch = scratch;
    L.scratch_cap = scratch ? scratch_cap : 0;
    L.max_spp = max_spp ? max_spp : 1;
    const bool env = p->env_map && p->env_width && p->env_height;
    L.env_map = env ? reinterpret_cast<const float4*>(p->env_map) : nullptr;
    L.env_w = env ? p->env_width : 0;
    L.env_h = env ? p->env_height : 0;
    return L;
}

// Validates the scenes and builds the plan (host table and device resources). split: one
// group (one persistent launch) per primitive type, scenes whose TLAS mixes types in a group
// of their own; otherwise one group.
hrt_status make_plan(hrt_context* ctx, const char* who, const hrt_scene_desc* scenes, uint32_t n, bool split,
                     bool need_hits, cudaStream_t s, ScenePlan& P) {
    for (uint32_t i = 0; i < n; ++i) {
        if (!scenes[i].tlas || !scenes[i].frame) return fail(ctx, HRT_ERR_INVALID_ARG, "%s: scene %u incomplete", who, i);
        if (need_hits && !scenes[i].frame->hits)
            return fail(ctx, HRT_ERR_INVALID_ARG, "%s: record_hits on a frame without hit records", who);
    }
    P.pos.assign(n, 0);
    auto key = [&](uint32_t i) -> uint32_t { return split ? prim_kind(scenes[i].tlas->type_mask) : 0u; };
    // Within a group the persistent warps take work items in table order, so the scenes whose
    // pixels cost most go first (samples per pixel, then primitives), as in longest-job-first
    // scheduling: the cheap pixels at the end fill the warps that would otherwise idle in the
    // launch's tail (C5: 4 % shorter steps than creation order). Results do not depend on it.
    std::vector<uint32_t> order(n);
    for (uint32_t i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        const uint32_t sa = scenes[a].frame->spp, sb = scenes[b].frame->spp;
        if (sa != sb) return sa > sb;
        return scenes[a].tlas->nprims > scenes[b].tlas->nprims;
    });
    for (uint32_t k = 0; k < 4; ++k) {
        ScenePlan::Group G;
        G.first = uint32_t(P.table.size());
        for (uint32_t i : order) {
            if (key(i) != k) continue;
            SceneLaunch sl;
            fill_scene(sl, scenes[i].tlas, &scenes[i].camera, scenes[i].frame, G.work);
            G.work += sl.work_count;
            G.type_mask |= scenes[i].tlas->type_mask;
            G.precision_mask |= scenes[i].tlas->precision_mask;
            G.any_tlas |= scenes[i].tlas->nodes != nullptr;
            P.pos[i] = uint32_t(P.table.size());
            P.table.push_back(sl);
            const hrt_frame* f = scenes[i].frame;
            P.primary += uint64_t(f->w) * f->h * f->spp;
            P.npix += uint64_t(f->w) * f->h;
            P.nsamp += uint64_t(f->w) * f->h * f->spp;
            P.max_spp = std::max(P.max_spp, f->spp);
        }
        G.count = uint32_t(P.table.size()) - G.first;
        if (G.count == 0) continue;
        if (G.work >= (1ull << 32)) return fail(ctx, HRT_ERR_UNSUPPORTED, "%s: more than 2^32 pixel work items", who);
        P.groups.push_back(G);
    }
    P.scap = std::min<uint64_t>(P.nsamp, kScratchSamples);
    cudaError_t e = cudaMalloc(&P.dtable, P.table.size() * sizeof(SceneLaunch));
    if (e == cudaSuccess) e = cudaMalloc(&P.counters, P.groups.size() * sizeof(TraceCounters));
    if (e == cudaSuccess) e = cudaMalloc(&P.list, P.npix * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&P.scratch, P.scap * sizeof(float4));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(P.dtable, P.table.data(), P.table.size() * sizeof(SceneLaunch), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        P.release();
        return cuda_fail(ctx, e, who);
    }
    return HRT_OK;
}

// Side streams for a plan's groups: groups that cannot run the FP64 pass go on their own
// branch (fork from and join back to the caller's stream), so the launches' tails overlap.
struct Branches {
    cudaStream_t aux[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t fork = nullptr, join[3] = {nullptr, nullptr, nullptr};
    cudaError_t create() {
        cudaError_t e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
        for (int k = 0; k < 3 && e == cudaSuccess; ++k) {
            e = cudaStreamCreateWithFlags(&aux[k], cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join[k], cudaEventDisableTiming);
        }
        return e;
    }
    void destroy() {
        for (int k = 0; k < 3; ++k) {
            if (aux[k]) cudaStreamDestroy(aux[k]);
            if (join[k]) cudaEventDestroy(join[k]);
            aux[k] = nullptr;
            join[k] = nullptr;
        }
        if (fork) cudaEventDestroy(fork);
        fork = nullptr;
    }
};

// Enqueues the plan's launches: per group, counter reset, frame pass, FP64 pass. With br, the
// groups without Phantom BLASes (no FP64 pass, so no use of the shared resolve list) run on
// side branches.
cudaError_t enqueue_plan(const ScenePlan& P, const hrt_trace_params* p, cudaStream_t s, int sm_count,
                         const Branches* br = nullptr) {
    const size_t ng = P.groups.size();
    std::vector<cudaStream_t> gs(ng, s);
    int naux = 0;
    if (br && ng > 1) {
        bool main_taken = false;
        for (size_t g = 0; g < ng; ++g)
            if (P.groups[g].type_mask & (1u << HRT_BLAS_PHANTOM)) main_taken = true;
        for (size_t g = 0; g < ng; ++g) {
            if (P.groups[g].type_mask & (1u << HRT_BLAS_PHANTOM)) continue;
            if (!main_taken) { main_taken = true; continue; }
            if (naux < 3) gs[g] = br->aux[naux++];
        }
    }
    cudaError_t e = cudaSuccess;
    if (naux) {
        e = cudaEventRecord(br->fork, s);
        for (int k = 0; k < naux && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(br->aux[k], br->fork, 0);
        if (e != cudaSuccess) return e;
    }
    for (size_t g = 0; g < ng; ++g) {
        const ScenePlan::Group& G = P.groups[g];
        e = cudaMemsetAsync(P.counters + g, 0, sizeof(TraceCounters), gs[g]);
        if (e != cudaSuccess) return e;
        TraceLaunch L = make_launch(p, P.dtable + G.first, G.count, G.work, P.counters + g, G.type_mask, P.list,
                                    P.npix, P.scratch, P.scap, P.max_spp);
        e = launch_trace(L, node_mode(G.precision_mask, G.any_tlas), gs[g], sm_count);
        if (e != cudaSuccess) return e;
    }
    for (int k = 0; k < naux && e == cudaSuccess; ++k) {
        e = cudaEventRecord(br->join[k], br->aux[k]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, br->join[k], 0);
    }
    return e;
}

// Sum of the groups' counters (error bits or-ed), with the device error checks.
hrt_status read_plan_counters(hrt_context* ctx, const ScenePlan& P, TraceCounters* sum, cudaStream_t s) {
    std::vector<TraceCounters> c(P.groups.size());
    CK(ctx, cudaMemcpyAsync(c.data(), P.counters, c.size() * sizeof(TraceCounters), cudaMemcpyDeviceToHost, s),
       "read counters");
    CK(ctx, cudaStreamSynchronize(s), "synchronise trace");
    memset(sum, 0, sizeof(*sum));
    for (const TraceCounters& x : c) {
        sum->shadow += x.shadow;
        sum->nodes += x.nodes;
        sum->prims += x.prims;
        sum->fp64_resolves += x.fp64_resolves;
        sum->fp64_hits += x.fp64_hits;
        sum->cycles_node += x.cycles_node;
        sum->cycles_leaf += x.cycles_leaf;
        sum->cycles_other += x.cycles_other;
        sum->error |= x.error;
    }
    return error_status(ctx, sum->error);
}

}  // namespace

extern "C" {

int hrt_abi_version(void) { return HRT_ABI_VERSION; }

const char* hrt_status_string(hrt_status s) {
    switch (s) {
        case HRT_OK: return "ok";
        case HRT_ERR_INVALID_ARG: return "invalid argument";
        case HRT_ERR_OOM: return "out of device memory";
        case HRT_ERR_CUDA: return "CUDA error";
        case HRT_ERR_STACK_OVERFLOW: return "traversal stack overflow";
        case HRT_ERR_TIMEOUT: return "device loop iteration cap reached";
        case HRT_ERR_UNSUPPORTED: return "unsupported";
        case HRT_ERR_BOUNDS: return "device index check failed";
    }
    return "unknown status";
}

hrt_status hrt_context_create(int device, hrt_context** out) {
    if (!out) return HRT_ERR_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return HRT_ERR_CUDA;
    if (device < 0 || device >= count) return HRT_ERR_INVALID_ARG;
    hrt_context* c = new (std::nothrow) hrt_context();
    if (!c) return HRT_ERR_OOM;
    c->device = device;
    DeviceSet ds(device);
    if (cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        prepare_frames() != cudaSuccess) {
        delete c;
        return HRT_ERR_CUDA;
    }
    *out = c;
    return HRT_OK;
}

hrt_status hrt_context_destroy(hrt_context* ctx) {
    delete ctx;
    return HRT_OK;
}

const char* hrt_last_error(const hrt_context* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

void hrt_blas_input_default(hrt_blas_input* in) {
    memset(in, 0, sizeof(*in));
    in->type = HRT_BLAS_PHANTOM;
    in->precision = HRT_PRECISION_FP32;
    in->memory = HRT_MEMORY_HOST;
    in->max_leaf = 1;
    in->const_radius = 0.02f;
    for (int k = 0; k < 4; ++k) in->transform[5 * k] = 1.0f;
}

// HRT_LOG >= 2: one line per built BLAS.
static void log_build(const hrt_blas* b) {
    if (log_level() < 2) return;
    fprintf(stderr, "[hrt] BLAS type %d precision %d: %llu primitives, %llu nodes, %llu device bytes, %.3f ms\n",
            b->type, b->precision, (unsigned long long)b->nprims, (unsigned long long)b->out.nnodes,
            (unsigned long long)b->out.device_bytes, double(b->build_ms));
}

// A mesh's material on the device: the albedo factor, and with a map and texture coordinates the
// per-triangle coordinates (gathered on the host through the kept triangle indices) and the map.
static hrt_status upload_material(hrt_context* ctx, const hrt_blas_input* in, hrt_blas* b) {
    for (int k = 0; k < 4; ++k) b->albedo[k] = in->albedo_factor[k];
    if (!in->albedo_map || !in->texcoords || b->nprims == 0) return HRT_OK;
    const uint32_t w = in->albedo_map_width, h = in->albedo_map_height;
    if (w < 1 || w > 16384 || h < 1 || h > 16384)
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_build: albedo map of %ux%u texels; each side must be 1..16384",
                    w, h);
    const bool host = in->memory == HRT_MEMORY_HOST;
    std::vector<float> tc;
    const float* t = in->texcoords;
    if (!host) {
        tc.resize(2 * b->nvertices);
        cudaError_t e = cudaMemcpy(tc.data(), in->texcoords, tc.size() * 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "hrt_blas_build: read texcoords");
        t = tc.data();
    }
    std::vector<float> uv(6 * b->nprims);
    for (uint64_t i = 0; i < b->nprims; ++i)
        for (int k = 0; k < 3; ++k) {
            const uint64_t v = b->tri_idx[3 * i + k];
            uv[6 * i + 2 * k] = t[2 * v];
            uv[6 * i + 2 * k + 1] = t[2 * v + 1];
        }
    const uint64_t map_bytes = uint64_t(w) * h * 16;
    cudaError_t e = cudaMalloc(&b->uv, uv.size() * 4);
    if (e == cudaSuccess) e = cudaMemcpy(b->uv, uv.data(), uv.size() * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&b->albedo_map, map_bytes);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->albedo_map, in->albedo_map, map_bytes, host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "hrt_blas_build: upload the material");
    b->map_w = w;
    b->map_h = h;
    return HRT_OK;
}

// Builds a triangle-mesh BLAS: gathers the indexed triangles (and vertex normals) on the device
// and runs the common BVH build over them.
static hrt_status build_mesh(hrt_context* ctx, const hrt_blas_input* in, cudaStream_t s, hrt_blas** out) {
    if (in->strand_offsets || in->line_indices)
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_build: a mesh takes tri_indices, not strands or lines");
    if (in->ntris && !in->tri_indices) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_build: null tri_indices");
    if (in->nvertices > 0 && !in->vertices) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_build: null vertices");
    if (in->nvertices >= (1ull << 32))
        return fail(ctx, HRT_ERR_UNSUPPORTED, "hrt_blas_build: more than 2^32 - 1 vertices");
    if (in->ntris >= (1ull << 29))
        return fail(ctx, HRT_ERR_UNSUPPORTED, "hrt_blas_build: %llu triangles; the limit is 2^29",
                    (unsigned long long)in->ntris);
    const uint32_t max_leaf = in->max_leaf ? in->max_leaf : 1;
    if (max_leaf > 3) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_build: max_leaf must be 1..3");
    const uint32_t width = in->width ? in->width : 8;
    if (width < 2 || width > 8) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_build: width must be 2..8");
    if (in->memory == HRT_MEMORY_HOST)
        for (uint64_t i = 0; i < 3 * in->ntris; ++i)
            if (in->tri_indices[i] >= in->nvertices)
                return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_build: triangle index %llu out of range",
                            (unsigned long long)i);
    const uint64_t n = in->ntris;
    hrt_blas* b = new (std::nothrow) hrt_blas();
    if (!b) return fail(ctx, HRT_ERR_OOM, "hrt_blas_build: host allocation");
    b->ctx = ctx;
    b->type = in->type;
    b->precision = in->precision;
    b->nprims = n;
    b->keep = (in->flags & HRT_BUILD_KEEP_INTERMEDIATE) != 0;
    memcpy(b->transform, in->transform, sizeof(b->transform));
    b->max_leaf = max_leaf;
    b->nvertices = in->nvertices;
    b->has_normals = in->normals != nullptr;
    if (!copy_u32(in->tri_indices, 3 * n, in->memory, b->tri_idx)) {
        delete b;
        return fail(ctx, HRT_ERR_CUDA, "hrt_blas_build: read triangle indices");
    }
    float *dv = nullptr, *dn = nullptr, *tris = nullptr, *tnrm = nullptr;
    uint32_t* didx = nullptr;
    const bool host = in->memory == HRT_MEMORY_HOST;
    auto cleanup = [&]() {
        if (host) {
            if (dv) cudaFree(dv);
            if (dn) cudaFree(dn);
            if (didx) cudaFree(didx);
        }
        if (tris) cudaFree(tris);
        if (tnrm) cudaFree(tnrm);
    };
    auto bail = [&](cudaError_t e, const char* what) {
        cleanup();
        free_build_output(b->out);
        delete b;
        return cuda_fail(ctx, e, what);
    };
    cudaError_t e = cudaSuccess;
    if (host && n) {
        if ((e = cudaMalloc(&dv, in->nvertices * 12)) != cudaSuccess) return bail(e, "allocate vertices");
        if ((e = cudaMemcpyAsync(dv, in->vertices, in->nvertices * 12, cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return bail(e, "copy vertices");
        if (in->normals) {
            if ((e = cudaMalloc(&dn, in->nvertices * 12)) != cudaSuccess) return bail(e, "allocate normals");
            if ((e = cudaMemcpyAsync(dn, in->normals, in->nvertices * 12, cudaMemcpyHostToDevice, s)) != cudaSuccess)
                return bail(e, "copy normals");
        }
        if ((e = cudaMalloc(&didx, n * 12)) != cudaSuccess) return bail(e, "allocate indices");
        if ((e = cudaMemcpyAsync(didx, in->tri_indices, n * 12, cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return bail(e, "copy indices");
    } else if (!host) {
        dv = const_cast<float*>(in->vertices);
        dn = const_cast<float*>(in->normals);
        didx = const_cast<uint32_t*>(in->tri_indices);
    }
    if (n) {
        if ((e = cudaMalloc(&tris, n * 36)) != cudaSuccess) return bail(e, "allocate triangles");
        if (in->normals && (e = cudaMalloc(&tnrm, n * 36)) != cudaSuccess) return bail(e, "allocate normals");
        if ((e = make_tris(dv, dn, didx, n, tris, tnrm, s)) != cudaSuccess) return bail(e, "gather triangles");
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    BuildInput bi{in->type, in->precision, int(max_leaf), int(width), nullptr, nullptr, n, b->keep, tris, tnrm};
    char msg[256] = {0};
    e = build_blas_device(bi, b->out, s, msg, sizeof(msg));
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&b->build_ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) {
        std::string m = msg;
        cleanup();
        free_build_output(b->out);
        delete b;
        if (e == cudaErrorMemoryAllocation) return fail(ctx, HRT_ERR_OOM, "BVH build: %s", m.c_str());
        return fail(ctx, HRT_ERR_CUDA, "BVH build: %s", m.empty() ? cudaGetErrorString(e) : m.c_str());
    }
    cleanup();
    const hrt_status st = upload_material(ctx, in, b);
    if (st != HRT_OK) {
        hrt_blas_destroy(b);
        return st;
    }
    log_build(b);
    *out = b;
    return HRT_OK;
}

hrt_status hrt_blas_build(hrt_context* ctx, const hrt_blas_input* in, void* stream, hrt_blas** out) {
    Range range("hrt_blas_build");
    if (!ctx) return HRT_ERR_INVALID_ARG;
    if (!in || !out) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_build: null input or output");
    *out = nullptr;
    if (in->type < HRT_BLAS_PHANTOM || in->type > HRT_BLAS_VOXELS)
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_build: unknown geometry type %d", in->type);
    const float voxel_size = in->voxel_size == 0.0f ? 0.1f : in->voxel_size;
    if (in->type == HRT_BLAS_VOXELS && !(voxel_size > 0.0f && voxel_size < 1e30f))
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_build: voxel_size must be > 0");
    if (in->precision != HRT_PRECISION_FP32 && in->precision != HRT_PRECISION_QUANTISED)
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_build: unknown precision %d", in->precision);
    if (in->memory != HRT_MEMORY_HOST && in->memory != HRT_MEMORY_DEVICE)
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_build: unknown memory kind %d", in->memory);
    if (in->type == HRT_BLAS_MESH) {
        DeviceSet dset(ctx->device);
        return build_mesh(ctx, in, static_cast<cudaStream_t>(stream), out);
    }
    if (!!in->strand_offsets == !!in->line_indices)
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_build: give exactly one of strand_offsets and line_indices");
    if (in->nvertices > 0 && !in->vertices)
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_build: null vertices");
    if (in->nvertices >= (1ull << 32))
        return fail(ctx, HRT_ERR_UNSUPPORTED, "hrt_blas_build: more than 2^32 - 1 vertices");
    uint32_t max_leaf = in->max_leaf ? in->max_leaf : 1;
    if (max_leaf > 3) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_build: max_leaf must be 1..3");
    const uint32_t width = in->width ? in->width : 8;
    if (width < 2 || width > 8) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_build: width must be 2..8");
    if (!in->radius && !(in->const_radius >= 0.0f))
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_build: const_radius must be >= 0");
    DeviceSet dset(ctx->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    // ---- lines: count and per-strand offsets (host) ------------------------------------------
    uint64_t nlines = 0;
    std::vector<uint32_t> line_off, vert_off;
    if (in->strand_offsets) {
        std::vector<uint32_t> so(in->nstrands + 1);
        if (in->memory == HRT_MEMORY_HOST) memcpy(so.data(), in->strand_offsets, so.size() * 4);
        else CK(ctx, cudaMemcpy(so.data(), in->strand_offsets, so.size() * 4, cudaMemcpyDeviceToHost), "read strand offsets");
        line_off.resize(in->nstrands + 1);
        vert_off.resize(in->nstrands + 1);
        for (uint64_t st = 0; st < in->nstrands; ++st) {
            if (so[st + 1] < so[st] || so[st + 1] > in->nvertices)
                return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_build: strand_offsets[%llu..] not increasing or past nvertices",
                            (unsigned long long)st);
            line_off[st] = uint32_t(nlines);
            vert_off[st] = so[st];
            uint32_t len = so[st + 1] - so[st];
            nlines += len >= 2 ? len - 1 : 0;
        }
        line_off[in->nstrands] = uint32_t(nlines);
        vert_off[in->nstrands] = so[in->nstrands];
    } else {
        nlines = in->nlines;
        if (in->memory == HRT_MEMORY_HOST)
            for (uint64_t i = 0; i < 2 * nlines; ++i)
                if (in->line_indices[i] >= in->nvertices)
                    return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_build: line index %llu out of range",
                                (unsigned long long)i);
    }
    if ((nlines << ref_shift(in->type)) >= (1ull << 29))
        return fail(ctx, HRT_ERR_UNSUPPORTED, "hrt_blas_build: %llu segments; the limit is 2^29 BVH references",
                    (unsigned long long)nlines);

    hrt_blas* b = new (std::nothrow) hrt_blas();
    if (!b) return fail(ctx, HRT_ERR_OOM, "hrt_blas_build: host allocation");
    b->ctx = ctx;
    b->type = in->type;
    b->precision = in->precision;
    b->nprims = nlines;
    b->keep = (in->flags & HRT_BUILD_KEEP_INTERMEDIATE) != 0;
    memcpy(b->transform, in->transform, sizeof(b->transform));
    b->max_leaf = max_leaf;
    b->nvertices = in->nvertices;
    b->nstrands = in->nstrands;
    b->const_radius = in->const_radius;
    b->has_radius = in->radius != nullptr;
    b->line_off = line_off;
    b->vert_off = vert_off;
    if (in->line_indices && !copy_u32(in->line_indices, 2 * nlines, in->memory, b->line_idx)) {
        delete b;
        return fail(ctx, HRT_ERR_CUDA, "hrt_blas_build: read line indices");
    }

    // ---- device copies of the inputs ------------------------------------------------------------
    float *dv = nullptr, *dr = nullptr, *lines = nullptr, *lrad = nullptr;
    uint32_t *dlo = nullptr, *dvo = nullptr, *didx = nullptr;
    auto cleanup = [&]() {
        if (in->memory == HRT_MEMORY_HOST) {
            if (dv) cudaFree(dv);
            if (dr) cudaFree(dr);
            if (didx) cudaFree(didx);
        }
        if (dlo) cudaFree(dlo);
        if (dvo) cudaFree(dvo);
        if (lines) cudaFree(lines);
        if (lrad) cudaFree(lrad);
    };
    auto bail = [&](cudaError_t e, const char* what) {
        cleanup();
        free_build_output(b->out);
        delete b;
        return cuda_fail(ctx, e, what);
    };
    cudaError_t e = cudaSuccess;
    if (in->memory == HRT_MEMORY_HOST) {
        if (in->nvertices) {
            if ((e = cudaMalloc(&dv, in->nvertices * 12)) != cudaSuccess) return bail(e, "allocate vertices");
            if ((e = cudaMemcpyAsync(dv, in->vertices, in->nvertices * 12, cudaMemcpyHostToDevice, s)) != cudaSuccess)
                return bail(e, "copy vertices");
            if (in->radius) {
                if ((e = cudaMalloc(&dr, in->nvertices * 4)) != cudaSuccess) return bail(e, "allocate radii");
                if ((e = cudaMemcpyAsync(dr, in->radius, in->nvertices * 4, cudaMemcpyHostToDevice, s)) != cudaSuccess)
                    return bail(e, "copy radii");
            }
        }
        if (in->line_indices && nlines) {
            if ((e = cudaMalloc(&didx, nlines * 8)) != cudaSuccess) return bail(e, "allocate line indices");
            if ((e = cudaMemcpyAsync(didx, in->line_indices, nlines * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess)
                return bail(e, "copy line indices");
        }
    } else {
        dv = const_cast<float*>(in->vertices);
        dr = const_cast<float*>(in->radius);
        didx = const_cast<uint32_t*>(in->line_indices);
    }
    if (in->strand_offsets) {
        if ((e = cudaMalloc(&dlo, line_off.size() * 4)) != cudaSuccess) return bail(e, "allocate strand tables");
        if ((e = cudaMalloc(&dvo, vert_off.size() * 4)) != cudaSuccess) return bail(e, "allocate strand tables");
        if ((e = cudaMemcpyAsync(dlo, line_off.data(), line_off.size() * 4, cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return bail(e, "copy strand tables");
        if ((e = cudaMemcpyAsync(dvo, vert_off.data(), vert_off.size() * 4, cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return bail(e, "copy strand tables");
    }
    if (nlines) {
        if ((e = cudaMalloc(&lines, nlines * 24)) != cudaSuccess) return bail(e, "allocate lines");
        if ((e = cudaMalloc(&lrad, nlines * 8)) != cudaSuccess) return bail(e, "allocate line radii");
        if ((e = make_lines(dv, dr, in->const_radius, dlo, dvo, in->nstrands, didx, nlines, lines, lrad, s)) != cudaSuccess)
            return bail(e, "generate lines");
    }

    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    BuildInput bi{in->type, in->precision, int(max_leaf), int(width), lines, lrad, nlines, b->keep};
    char msg[256] = {0};
    float* vox = nullptr;
    if (in->type == HRT_BLAS_VOXELS) {  // the lines become voxel boxes, the BVH primitives
        uint64_t nvox = 0;
        e = voxelize_device(lines, nlines, in->const_radius, voxel_size, &vox, &nvox, b->voxel_grid, s, msg,
                            sizeof(msg));
        bi.n = nvox;
        bi.voxels = vox;
        b->nprims = nvox;
    }
    if (e == cudaSuccess) e = build_blas_device(bi, b->out, s, msg, sizeof(msg));
    cudaEventRecord(e1, s);
    if (e != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        std::string m = msg;
        cudaStreamSynchronize(s);
        if (vox) cudaFree(vox);
        cleanup();
        free_build_output(b->out);
        delete b;
        if (e == cudaErrorInvalidValue && !m.empty()) return fail(ctx, HRT_ERR_UNSUPPORTED, "%s", m.c_str());
        if (e == cudaErrorMemoryAllocation) return fail(ctx, HRT_ERR_OOM, "BVH build: %s", m.c_str());
        return fail(ctx, HRT_ERR_CUDA, "BVH build: %s", m.empty() ? cudaGetErrorString(e) : m.c_str());
    }
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&b->build_ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (vox) cudaFree(vox);
    cleanup();
    log_build(b);
    *out = b;
    return HRT_OK;
}

hrt_status hrt_blas_refit(hrt_blas* b, const float* vertices, const float* per_vertex, int32_t memory, void* stream) {
    Range range("hrt_blas_refit");
    if (!b) return HRT_ERR_INVALID_ARG;
    hrt_context* ctx = b->ctx;
    if (b->type == HRT_BLAS_VOXELS)
        return fail(ctx, HRT_ERR_UNSUPPORTED, "hrt_blas_refit: moved strands fill other voxels (rebuild the voxel BLAS)");
    const bool mesh = b->type == HRT_BLAS_MESH;
    const bool want = mesh ? b->has_normals : b->has_radius;
    if (b->nvertices && !vertices) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_refit: null vertices");
    if (want != (per_vertex != nullptr))
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_refit: %s %s as at the build", mesh ? "normals" : "radii",
                    want ? "are required" : "must be null");
    if (memory != HRT_MEMORY_HOST && memory != HRT_MEMORY_DEVICE)
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_refit: unknown memory kind %d", memory);
    if (b->nprims == 0) return HRT_OK;
    DeviceSet ds(ctx->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint64_t n = b->nprims, nv = b->nvertices;
    const int per = mesh ? 3 : 1;  // floats per vertex of per_vertex
    float *dv = nullptr, *dp = nullptr, *g0 = nullptr, *g1 = nullptr;
    uint32_t *d0 = nullptr, *d1 = nullptr;
    const bool host = memory == HRT_MEMORY_HOST;
    auto cleanup = [&]() {
        if (host) {
            if (dv) cudaFree(dv);
            if (dp) cudaFree(dp);
        }
        void* p[] = {g0, g1, d0, d1};
        for (void* q : p)
            if (q) cudaFree(q);
    };
    cudaError_t e = cudaSuccess;
    if (host) {
        e = cudaMalloc(&dv, nv * 12);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dv, vertices, nv * 12, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && per_vertex) e = cudaMalloc(&dp, nv * 4 * per);
        if (e == cudaSuccess && per_vertex) e = cudaMemcpyAsync(dp, per_vertex, nv * 4 * per, cudaMemcpyHostToDevice, s);
    } else {
        dv = const_cast<float*>(vertices);
        dp = const_cast<float*>(per_vertex);
    }
    BuildInput bi{b->type, b->precision, int(b->max_leaf), 8, nullptr, nullptr, n, b->keep};
    if (mesh) {
        if (e == cudaSuccess) e = cudaMalloc(&d0, n * 12);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d0, b->tri_idx.data(), n * 12, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaMalloc(&g0, n * 36);
        if (e == cudaSuccess && dp) e = cudaMalloc(&g1, n * 36);
        if (e == cudaSuccess) e = make_tris(dv, dp, d0, n, g0, g1, s);
        bi.tris = g0;
        bi.tri_normals = g1;
    } else {
        if (b->line_idx.empty()) {
            if (e == cudaSuccess) e = cudaMalloc(&d0, b->line_off.size() * 4);
            if (e == cudaSuccess) e = cudaMalloc(&d1, b->vert_off.size() * 4);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(d0, b->line_off.data(), b->line_off.size() * 4, cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(d1, b->vert_off.data(), b->vert_off.size() * 4, cudaMemcpyHostToDevice, s);
        } else {
            if (e == cudaSuccess) e = cudaMalloc(&d0, n * 8);
            if (e == cudaSuccess) e = cudaMemcpyAsync(d0, b->line_idx.data(), n * 8, cudaMemcpyHostToDevice, s);
        }
        if (e == cudaSuccess) e = cudaMalloc(&g0, n * 24);
        if (e == cudaSuccess) e = cudaMalloc(&g1, n * 8);
        if (e == cudaSuccess)
            e = b->line_idx.empty() ? make_lines(dv, dp, b->const_radius, d0, d1, b->nstrands, nullptr, n, g0, g1, s)
                                    : make_lines(dv, dp, b->const_radius, nullptr, nullptr, 0, d0, n, g0, g1, s);
        bi.lines = g0;
        bi.lrad = g1;
    }
    if (e != cudaSuccess) {
        cleanup();
        return cuda_fail(ctx, e, "hrt_blas_refit");
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    char msg[256] = {0};
    e = refit_blas_device(bi, b->out, s, msg, sizeof(msg));
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&b->build_ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cleanup();
    if (e == cudaErrorInvalidValue) return fail(ctx, HRT_ERR_UNSUPPORTED, "%s", msg);
    if (e != cudaSuccess) return fail(ctx, HRT_ERR_CUDA, "%s", msg[0] ? msg : cudaGetErrorString(e));
    return HRT_OK;
}

hrt_status hrt_blas_destroy(hrt_blas* b) {
    if (!b) return HRT_OK;
    DeviceSet ds(b->ctx->device);
    free_build_output(b->out);
    if (b->uv) cudaFree(b->uv);
    if (b->albedo_map) cudaFree(b->albedo_map);
    delete b;
    return HRT_OK;
}

int32_t hrt_blas_type(const hrt_blas* b) { return b ? b->type : -1; }

hrt_status hrt_blas_transform(const hrt_blas* b, float out[16]) {
    if (!b || !out) return HRT_ERR_INVALID_ARG;
    memcpy(out, b->transform, sizeof(b->transform));
    return HRT_OK;
}

// ---- serialisation --------------------------------------------------------------------------
// Layout (little-endian): the header below, then level starts (u32), the refit topology
// (line offsets, vertex offsets, line indices, triangle indices: u32 each, lengths in the
// header), then the device arrays: nodes, records, the strand vertex stream (float4, quantised
// Phantom), slot map (u32). Records and
// the slot map have one entry per BVH reference (two per LSS or DOTS segment); the partner map
// of those two-reference types is rebuilt from the slot map when an image is read.
namespace {
struct SerialHeader {
    char magic[4];  // "HRTB"
    uint32_t version;
    int32_t type, precision;
    uint64_t nprims, nnodes, nverts, node_bytes, prim_bytes;
    float bounds[6];
    float transform[16];
    uint32_t max_leaf, reserved;
    uint64_t nvertices, nstrands;
    float const_radius;
    uint32_t has_radius, has_normals;
    uint64_t nlevels, n_line_off, n_vert_off, n_line_idx, n_tri_idx;
    float albedo[4];          // mesh material: factor, then n_uv texture-coordinate floats and
    uint32_t map_w, map_h;    // map_w x map_h RGBA texels after the arrays (none without a map)
    uint64_t n_uv;
};
constexpr uint32_t kSerialVersion = 4;

uint64_t material_bytes(const hrt_blas* b) {
    return b->albedo_map ? b->nprims * 24 + uint64_t(b->map_w) * b->map_h * 16 : 0;
}

uint64_t serial_size(const hrt_blas* b) {
    const BuildOutput& o = b->out;
    return sizeof(SerialHeader) +
           4 * (o.level_start.size() + b->line_off.size() + b->vert_off.size() + b->line_idx.size() + b->tri_idx.size()) +
           o.nnodes * o.node_bytes + o.nslots * o.prim_bytes + o.nverts * 16 + o.nslots * 4 + material_bytes(b);
}

// Reads a u32 array of n entries at *p, advancing it; false past the end.
bool take_u32(const uint8_t*& p, const uint8_t* end, uint64_t n, std::vector<uint32_t>& v) {
    if (n > uint64_t(end - p) / 4) return false;
    v.resize(n);
    if (n) memcpy(v.data(), p, n * 4);
    p += n * 4;
    return true;
}

// Host-side check of a deserialised tree, so that tracing it never reads outside its arrays:
// internal children below nnodes, leaf runs inside the records, quantised Phantom records' four
// stream entries inside the strand vertex stream.
const char* check_tree(int type, int precision, uint64_t nprims, uint64_t nnodes, uint64_t nverts, const uint8_t* nodes,
                       const uint8_t* prims, const std::vector<uint32_t>& levels) {
    const bool quant = precision == HRT_PRECISION_QUANTISED;
    for (uint64_t i = 0; i < nnodes; ++i) {
        uint32_t cb, pb;
        const uint8_t* meta;
        uint32_t imask;
        if (quant) {
            const NodeQ* q = reinterpret_cast<const NodeQ*>(nodes) + i;
            cb = q->child_base; pb = q->prim_base; meta = q->meta; imask = q->imask;
        } else {
            const NodeF* f = reinterpret_cast<const NodeF*>(nodes) + i;
            cb = f->child_base; pb = f->prim_base; meta = f->meta; imask = f->imask;
        }
        uint32_t rank = 0;
        for (int k = 0; k < 8; ++k) {
            const uint32_t m = meta[k];
            if (((imask >> k) & 1u) != ((m & 0x80u) ? 1u : 0u)) return "internal-child mask disagrees with meta";
            if (m & 0x80u) {
                if ((m & 0x78u) || (m & 7u) != rank) return "internal children are not ranked in slot order";
                if (uint64_t(cb) + rank >= nnodes || uint64_t(cb) + rank <= i) return "child index out of range";
                ++rank;
            } else if (m) {
                const uint32_t cnt = m >> 5, off = m & 31u;
                if (cnt == 0 || cnt > 3 || uint64_t(pb) + off + cnt > nprims) return "leaf run out of range";
            }
        }
    }
    for (size_t k = 0; k + 1 < levels.size(); ++k)
        if (levels[k] > levels[k + 1] || levels[k + 1] > nnodes) return "level starts out of order";
    if (!levels.empty() && levels.back() != nnodes) return "level starts do not end at the node count";
    if (type == HRT_BLAS_PHANTOM && quant)
        for (uint64_t i = 0; i < nprims; ++i) {
            uint32_t e;
            memcpy(&e, prims + 4 * i, 4);
            if (uint64_t(e) + 4 > nverts) return "record outside the strand vertex stream";
        }
    return nullptr;
}
}  // namespace

uint64_t hrt_blas_serialized_size(const hrt_blas* b) { return b ? serial_size(b) : 0; }

hrt_status hrt_blas_serialize(const hrt_blas* b, void* dst, uint64_t bytes) {
    if (!b || !dst) return HRT_ERR_INVALID_ARG;
    hrt_context* ctx = b->ctx;
    const uint64_t need = serial_size(b);
    if (bytes < need)
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_serialize: needs %llu bytes, got %llu", (unsigned long long)need,
                    (unsigned long long)bytes);
    DeviceSet ds(ctx->device);
    const BuildOutput& o = b->out;
    SerialHeader h{};
    memcpy(h.magic, "HRTB", 4);
    h.version = kSerialVersion;
    h.type = b->type;
    h.precision = b->precision;
    h.nprims = b->nprims;
    h.nnodes = o.nnodes;
    h.nverts = o.nverts;
    h.node_bytes = o.node_bytes;
    h.prim_bytes = o.prim_bytes;
    memcpy(h.bounds, o.bounds, sizeof(h.bounds));
    memcpy(h.transform, b->transform, sizeof(h.transform));
    h.max_leaf = b->max_leaf;
    h.nvertices = b->nvertices;
    h.nstrands = b->nstrands;
    h.const_radius = b->const_radius;
    h.has_radius = b->has_radius;
    h.has_normals = b->has_normals;
    h.nlevels = o.level_start.size();
    h.n_line_off = b->line_off.size();
    h.n_vert_off = b->vert_off.size();
    h.n_line_idx = b->line_idx.size();
    h.n_tri_idx = b->tri_idx.size();
    memcpy(h.albedo, b->albedo, sizeof(h.albedo));
    h.map_w = b->albedo_map ? b->map_w : 0;
    h.map_h = b->albedo_map ? b->map_h : 0;
    h.n_uv = b->albedo_map ? 6 * b->nprims : 0;
    uint8_t* p = static_cast<uint8_t*>(dst);
    memcpy(p, &h, sizeof(h));
    p += sizeof(h);
    for (const std::vector<uint32_t>* v : {&o.level_start, &b->line_off, &b->vert_off, &b->line_idx, &b->tri_idx}) {
        if (!v->empty()) memcpy(p, v->data(), v->size() * 4);
        p += v->size() * 4;
    }
    struct { const void* src; uint64_t n; } parts[] = {{o.nodes, o.nnodes * o.node_bytes},
                                                      {o.prims, o.nslots * o.prim_bytes},
                                                      {o.verts, o.nverts * 16},
                                                      {o.prim_ids, o.nslots * 4},
                                                      {b->uv, h.n_uv * 4},
                                                      {b->albedo_map, uint64_t(h.map_w) * h.map_h * 16}};
    for (auto& q : parts) {
        if (q.n) CK(ctx, cudaMemcpy(p, q.src, q.n, cudaMemcpyDeviceToHost), "hrt_blas_serialize");
        p += q.n;
    }
    return HRT_OK;
}

hrt_status hrt_blas_deserialize(hrt_context* ctx, const void* src, uint64_t bytes, void* stream, hrt_blas** out) {
    if (!ctx) return HRT_ERR_INVALID_ARG;
    if (!src || !out) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_deserialize: null argument");
    *out = nullptr;
    const uint8_t* p = static_cast<const uint8_t*>(src);
    const uint8_t* end = p + bytes;
    SerialHeader h;
    if (bytes < sizeof(h)) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_deserialize: truncated header");
    memcpy(&h, p, sizeof(h));
    p += sizeof(h);
    if (memcmp(h.magic, "HRTB", 4) != 0 || h.version != kSerialVersion)
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_deserialize: not a version-%u BLAS image", kSerialVersion);
    const bool quant = h.precision == HRT_PRECISION_QUANTISED;
    const uint64_t want_node = quant ? sizeof(NodeQ) : sizeof(NodeF);
    const uint64_t want_prim = h.type == HRT_BLAS_PHANTOM ? (quant ? 4 : 64)
                               : ((h.type == HRT_BLAS_LSS || h.type == HRT_BLAS_VOXELS) ? 32 : 80);
    if (h.type < HRT_BLAS_PHANTOM || h.type > HRT_BLAS_VOXELS || (h.precision != HRT_PRECISION_FP32 && !quant) ||
        h.node_bytes != want_node || h.prim_bytes != want_prim || h.nprims >= (1ull << 29) || (h.nprims << ref_shift(h.type)) >= (1ull << 29) ||
        h.nnodes > (h.nprims << ref_shift(h.type)) + 1 ||
        h.nverts > 4 * h.nprims || (h.type == HRT_BLAS_PHANTOM && quant ? (h.nprims && h.nverts < h.nprims + 3) : h.nverts != 0) ||
        (h.nprims && !h.nnodes) || h.max_leaf < 1 || h.max_leaf > 3 ||
        (h.n_uv ? (h.type != HRT_BLAS_MESH || h.n_uv != 6 * h.nprims || h.map_w < 1 || h.map_w > 16384 || h.map_h < 1 ||
                   h.map_h > 16384)
                : (h.map_w || h.map_h)))
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_deserialize: inconsistent header");
    hrt_blas* b = new (std::nothrow) hrt_blas();
    if (!b) return fail(ctx, HRT_ERR_OOM, "hrt_blas_deserialize: host allocation");
    auto reject = [&](const char* why) {
        free_build_output(b->out);
        delete b;
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_deserialize: %s", why);
    };
    b->ctx = ctx;
    b->type = h.type;
    b->precision = h.precision;
    b->nprims = h.nprims;
    memcpy(b->transform, h.transform, sizeof(h.transform));
    b->max_leaf = h.max_leaf;
    b->nvertices = h.nvertices;
    b->nstrands = h.nstrands;
    b->const_radius = h.const_radius;
    b->has_radius = h.has_radius != 0;
    b->has_normals = h.has_normals != 0;
    memcpy(b->albedo, h.albedo, sizeof(b->albedo));
    BuildOutput& o = b->out;
    if (!take_u32(p, end, h.nlevels, o.level_start) || !take_u32(p, end, h.n_line_off, b->line_off) ||
        !take_u32(p, end, h.n_vert_off, b->vert_off) || !take_u32(p, end, h.n_line_idx, b->line_idx) ||
        !take_u32(p, end, h.n_tri_idx, b->tri_idx))
        return reject("truncated tables");
    const uint32_t shift = ref_shift(h.type);
    const uint64_t nslots = h.nprims << shift;
    const uint64_t nb = h.nnodes * h.node_bytes, pbytes = nslots * h.prim_bytes, rb = h.nverts * 16, ib = nslots * 4;
    const uint64_t ub = h.n_uv * 4, mb = uint64_t(h.map_w) * h.map_h * 16;
    if (nb + pbytes + rb + ib + ub + mb > uint64_t(end - p)) return reject("truncated arrays");
    const uint8_t* nodes = p;
    const uint8_t* prims = p + nb;
    if (const char* why = check_tree(h.type, h.precision, nslots, h.nnodes, h.nverts, nodes, prims, o.level_start))
        return reject(why);
    // two references per segment: the slot map must be a permutation of the reference ids, and
    // the partner map follows from it
    std::vector<uint32_t> partner;
    if (shift) {
        std::vector<uint32_t> ids(nslots), slot_of(nslots, 0xffffffffu);
        if (nslots) memcpy(ids.data(), prims + pbytes + rb, ib);
        for (uint64_t i = 0; i < nslots; ++i) {
            if (ids[i] >= nslots || slot_of[ids[i]] != 0xffffffffu) return reject("slot map is not a permutation");
            slot_of[ids[i]] = uint32_t(i);
        }
        partner.resize(nslots);
        for (uint64_t i = 0; i < nslots; ++i) partner[i] = slot_of[ids[i] ^ 1u];
    }
    o.nnodes = h.nnodes;
    o.nverts = h.nverts;
    o.node_bytes = h.node_bytes;
    o.prim_bytes = h.prim_bytes;
    memcpy(o.bounds, h.bounds, sizeof(o.bounds));
    DeviceSet ds(ctx->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaSuccess;
    struct { void** dst; const uint8_t* src; uint64_t n; } parts[] = {{&o.nodes, nodes, nb},
                                                                     {&o.prims, prims, pbytes},
                                                                     {reinterpret_cast<void**>(&o.verts), prims + pbytes, rb},
                                                                     {reinterpret_cast<void**>(&o.prim_ids), prims + pbytes + rb, ib},
                                                                     {reinterpret_cast<void**>(&o.partner),
                                                                      reinterpret_cast<const uint8_t*>(partner.data()),
                                                                      partner.size() * 4},
                                                                     {reinterpret_cast<void**>(&b->uv), prims + pbytes + rb + ib, ub},
                                                                     {reinterpret_cast<void**>(&b->albedo_map),
                                                                      prims + pbytes + rb + ib + ub, mb}};
    for (auto& q : parts) {
        if (!q.n || e != cudaSuccess) continue;
        e = cudaMalloc(q.dst, q.n);
        if (e == cudaSuccess) e = cudaMemcpyAsync(*q.dst, q.src, q.n, cudaMemcpyHostToDevice, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        hrt_blas_destroy(b);
        return cuda_fail(ctx, e, "hrt_blas_deserialize");
    }
    b->map_w = h.map_w;
    b->map_h = h.map_h;
    o.nslots = nslots;
    o.device_bytes = nb + pbytes + rb + ib + partner.size() * 4;
    *out = b;
    return HRT_OK;
}

hrt_status hrt_blas_get_info(const hrt_blas* b, hrt_blas_info* o) {
    if (!b || !o) return HRT_ERR_INVALID_ARG;
    o->nprims = b->nprims;
    o->nnodes = b->out.nnodes;
    o->node_bytes = b->out.node_bytes;
    o->prim_bytes = b->out.prim_bytes;
    o->device_bytes = b->out.device_bytes + material_bytes(b);
    memcpy(o->bounds, b->out.bounds, sizeof(o->bounds));
    o->build_ms = b->build_ms;
    return HRT_OK;
}

hrt_status hrt_blas_get(const hrt_blas* b, int32_t part, void* dst, uint64_t bytes) {
    if (!b || !dst) return HRT_ERR_INVALID_ARG;
    hrt_context* ctx = b->ctx;
    DeviceSet ds(ctx->device);
    const uint64_t n = b->nprims;  // segments (triangles, voxels)
    const BuildOutput& o = b->out;
    const uint64_t ns = o.nslots;   // BVH references: the parts of the tree and its leaves
    const void* src = nullptr;
    uint64_t need = 0;
    switch (part) {
        case HRT_PART_PRIM_BOXES: src = o.prim_boxes; need = ns * 24; break;
        case HRT_PART_MORTON_SORTED: src = o.morton_sorted; need = ns * 8; break;
        case HRT_PART_SORTED_INDEX: src = o.sorted_index; need = ns * 4; break;
        case HRT_PART_BIN_LEFT: src = o.bin_left; need = ns ? (ns - 1) * 4 : 0; break;
        case HRT_PART_BIN_RIGHT: src = o.bin_right; need = ns ? (ns - 1) * 4 : 0; break;
        case HRT_PART_BIN_BOXES: src = o.bin_boxes; need = ns ? (ns - 1) * 24 : 0; break;
        case HRT_PART_NODES: src = o.nodes; need = o.nnodes * o.node_bytes; break;
        case HRT_PART_QNODES:
            src = b->precision == HRT_PRECISION_QUANTISED ? o.nodes : o.qnodes_aux;
            need = o.nnodes * sizeof(NodeQ);
            break;
        case HRT_PART_PRIM_ORDER: src = o.prim_ids; need = ns * 4; break;
        case HRT_PART_PRIMS: src = o.prims; need = ns * o.prim_bytes; break;
        case HRT_PART_CURVES: src = o.curves; need = n * 48; break;
        case HRT_PART_LSS: src = b->type == HRT_BLAS_LSS ? o.geom : nullptr; need = n * 32; break;
        case HRT_PART_STRAND_VERTICES: src = o.verts; need = o.nverts * 16; break;
        case HRT_PART_TRI_TEXCOORDS: src = b->uv; need = b->nprims * 24; break;
        case HRT_PART_DOTS_VERTICES: {
            if (b->type != HRT_BLAS_DOTS) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_get: not a DOTS BLAS");
            need = n * 144;
            if (bytes != need) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_get: part needs %llu bytes", (unsigned long long)need);
            if (!n) return HRT_OK;
            if (!o.geom) return fail(ctx, HRT_ERR_UNSUPPORTED, "hrt_blas_get: part %d was not kept when the BLAS was built", part);
            float* tmp = nullptr;
            CK(ctx, cudaMalloc(&tmp, need), "allocate DOTS vertices");
            cudaError_t e = expand_dots(o.geom, n, tmp, nullptr);
            if (e == cudaSuccess) e = cudaMemcpy(dst, tmp, need, cudaMemcpyDeviceToHost);
            cudaFree(tmp);
            CK(ctx, e, "expand DOTS vertices");
            return HRT_OK;
        }
        default: return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_get: unknown part %d", part);
    }
    if (bytes != need)
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_blas_get: part %d needs %llu bytes, got %llu", part,
                    (unsigned long long)need, (unsigned long long)bytes);
    if (need == 0) return HRT_OK;
    if (!src) return fail(ctx, HRT_ERR_UNSUPPORTED, "hrt_blas_get: part %d was not kept when the BLAS was built", part);
    CK(ctx, cudaMemcpy(dst, src, need, cudaMemcpyDeviceToHost), "hrt_blas_get");
    return HRT_OK;
}

namespace {
// A float at most x (lo = true) or at least x (lo = false): the outward rounding of a box corner.
float round_out(double x, bool lo) {
    float f = float(x);
    if (lo && double(f) > x) f = std::nextafter(f, -INFINITY);
    if (!lo && double(f) < x) f = std::nextafter(f, INFINITY);
    return f;
}
struct TlasItem {
    float lo[3], hi[3];
    double c[3];
    uint32_t inst;
};
// Median-split binary BVH over items[l, r): the longest axis of the centroids' box, split at the
// median centroid (ties by instance index, so the tree is deterministic). Returns the node index.
uint32_t build_tlas_node(std::vector<TlasItem>& items, size_t l, size_t r, std::vector<TlasNode>& nodes) {
    const uint32_t me = uint32_t(nodes.size());
    nodes.emplace_back();
    if (r - l == 1) {
        TlasNode& n = nodes[me];
        for (int k = 0; k < 3; ++k) { n.lo[k] = items[l].lo[k]; n.hi[k] = items[l].hi[k]; }
        n.a = kLeafFlag | items[l].inst;
        n.b = 0;
        return me;
    }
    double clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t i = l; i < r; ++i)
        for (int k = 0; k < 3; ++k) { clo[k] = std::min(clo[k], items[i].c[k]); chi[k] = std::max(chi[k], items[i].c[k]); }
    int ax = 0;
    for (int k = 1; k < 3; ++k)
        if (chi[k] - clo[k] > chi[ax] - clo[ax]) ax = k;
    const size_t mid = l + (r - l) / 2;
    std::nth_element(items.begin() + l, items.begin() + mid, items.begin() + r, [ax](const TlasItem& x, const TlasItem& y) {
        return x.c[ax] < y.c[ax] || (x.c[ax] == y.c[ax] && x.inst < y.inst);
    });
    const uint32_t left = build_tlas_node(items, l, mid, nodes);
    const uint32_t right = build_tlas_node(items, mid, r, nodes);
    TlasNode& n = nodes[me];
    for (int k = 0; k < 3; ++k) {
        n.lo[k] = std::min(nodes[left].lo[k], nodes[right].lo[k]);
        n.hi[k] = std::max(nodes[left].hi[k], nodes[right].hi[k]);
    }
    n.a = left;
    n.b = right;
    return me;
}
}  // namespace

hrt_status hrt_tlas_build(hrt_context* ctx, const hrt_blas* const* blases, uint32_t n, void* stream, hrt_tlas** out) {
    Range range("hrt_tlas_build");
    if (!ctx) return HRT_ERR_INVALID_ARG;
    if (!out || (n && !blases)) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_tlas_build: null argument");
    *out = nullptr;
    if (n > kMaxInstances) return fail(ctx, HRT_ERR_UNSUPPORTED, "hrt_tlas_build: %u instances; the limit is 2^24", n);
    DeviceSet ds(ctx->device);
    std::vector<DevInstance> inst(n);
    std::vector<TlasItem> items;
    uint32_t precision_mask = 0, type_mask = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const hrt_blas* b = blases[i];
        if (!b) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_tlas_build: null BLAS %u", i);
        precision_mask |= 1u << b->precision;
        type_mask |= 1u << b->type;
        DevInstance& d = inst[i];
        memset(&d, 0, sizeof(d));
        d.b.nodes = b->out.nodes;
        d.b.prims = b->out.prims;
        d.b.verts = b->out.verts;
        d.b.prim_ids = b->out.prim_ids;
        d.b.partner = b->out.partner;
        d.b.ref_shift = ref_shift(b->type);
        d.b.type = uint32_t(b->type);
        d.b.precision = uint32_t(b->precision);
        d.b.nprims = uint32_t(b->nprims);
        d.b.nnodes = uint32_t(b->out.nnodes);
        d.b.nverts = uint32_t(b->out.nverts);
#ifdef HRT_CHECKED
        // test hook of the checked build: report fewer nodes than the BLAS holds, so traversal
        // meets indices past the reported count (the loads there would still be inside the array)
        if (const char* lim = getenv("HRT_CHECKED_NODE_LIMIT"))
            d.b.nnodes = std::min<uint32_t>(d.b.nnodes, uint32_t(std::max(1L, strtol(lim, nullptr, 10))));
#endif
        for (int k = 0; k < 3; ++k) { d.b.lo[k] = b->out.bounds[k]; d.b.hi[k] = b->out.bounds[3 + k]; }
        for (int k = 0; k < 4; ++k) d.b.albedo[k] = b->albedo[k];
        d.b.uv = b->uv;
        d.b.albedo_map = b->albedo_map;
        d.b.map_w = b->map_w;
        d.b.map_h = b->map_h;
        d.identity = is_identity(b->transform) ? 1u : 0u;
        double m[16], iv[16];
        for (int k = 0; k < 16; ++k) m[k] = b->transform[k];
        if (!invert4(m, iv)) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_tlas_build: BLAS %u transform is singular", i);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 4; ++c) d.w2o[4 * r + c] = float(iv[4 * c + r]);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) d.nrm[3 * r + c] = float(iv[4 * r + c]);  // (M^-1)^T
        if (b->out.nnodes == 0) continue;  // nothing to hit: no TLAS leaf
        // world box: the 8 corners of the object-space bounds through the transform (double),
        // rounded outward
        TlasItem it;
        it.inst = i;
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int c = 0; c < 8; ++c) {
            const double p[3] = {b->out.bounds[(c & 1) ? 3 : 0], b->out.bounds[(c & 2) ? 4 : 1], b->out.bounds[(c & 4) ? 5 : 2]};
            for (int r = 0; r < 3; ++r) {
                const double w = m[r] * p[0] + m[4 + r] * p[1] + m[8 + r] * p[2] + m[12 + r];
                lo[r] = std::min(lo[r], w);
                hi[r] = std::max(hi[r], w);
            }
        }
        for (int k = 0; k < 3; ++k) {
            // a relative margin covers the double rounding of the transform
            const double pad = 1e-12 * (std::fabs(lo[k]) + std::fabs(hi[k]));
            it.lo[k] = round_out(lo[k] - pad, true);
            it.hi[k] = round_out(hi[k] + pad, false);
            it.c[k] = 0.5 * (lo[k] + hi[k]);
        }
        items.push_back(it);
    }
    std::vector<TlasNode> nodes;
    if (items.size() >= 2) {
        nodes.reserve(2 * items.size());
        build_tlas_node(items, 0, items.size(), nodes);
    }
    hrt_tlas* t = new (std::nothrow) hrt_tlas();
    if (!t) return fail(ctx, HRT_ERR_OOM, "hrt_tlas_build: host allocation");
    t->ctx = ctx;
    t->n = n;
    t->nnodes = uint32_t(nodes.size());
    t->precision_mask = precision_mask;
    t->type_mask = type_mask;
    for (uint32_t i = 0; i < n; ++i) t->nprims += blases[i]->nprims;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaSuccess;
    if (n) {
        e = cudaMalloc(&t->dev, n * sizeof(DevInstance));
        if (e == cudaSuccess) e = cudaMemcpyAsync(t->dev, inst.data(), n * sizeof(DevInstance), cudaMemcpyHostToDevice, s);
    }
    if (e == cudaSuccess && !nodes.empty()) {
        e = cudaMalloc(&t->nodes, nodes.size() * sizeof(TlasNode));
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(t->nodes, nodes.data(), nodes.size() * sizeof(TlasNode), cudaMemcpyHostToDevice, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        if (t->dev) cudaFree(t->dev);
        if (t->nodes) cudaFree(t->nodes);
        delete t;
        return cuda_fail(ctx, e, "hrt_tlas_build");
    }
    *out = t;
    return HRT_OK;
}

hrt_status hrt_tlas_destroy(hrt_tlas* t) {
    if (!t) return HRT_OK;
    DeviceSet ds(t->ctx->device);
    if (t->dev) cudaFree(t->dev);
    if (t->nodes) cudaFree(t->nodes);
    delete t;
    return HRT_OK;
}

void hrt_trace_params_default(hrt_trace_params* p) {
    memset(p, 0, sizeof(*p));
    p->tmin = 0.001f;
    p->tmax = 10000.0f;
    p->spp = 1;
    p->shading = HRT_SHADE_DEBUG;
    p->shadow_tmin = 1e-4f;
    p->fp64_resolve = 1;
    p->refill = 8;
    p->speculative = 1;
    p->leaf_again = 4;
}

hrt_status hrt_frame_create(hrt_context* ctx, uint32_t w, uint32_t h, uint32_t spp, int32_t with_hits, hrt_frame** out) {
    if (!ctx) return HRT_ERR_INVALID_ARG;
    if (!out || w == 0 || h == 0 || spp == 0 || spp > 1024)
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_frame_create: bad size %ux%u x %u spp", w, h, spp);
    if (uint64_t(w) * h * spp >= (1ull << 32))
        return fail(ctx, HRT_ERR_UNSUPPORTED, "hrt_frame_create: more than 2^32 samples");
    DeviceSet ds(ctx->device);
    hrt_frame* f = new (std::nothrow) hrt_frame();
    if (!f) return fail(ctx, HRT_ERR_OOM, "hrt_frame_create: host allocation");
    f->ctx = ctx;
    f->w = w;
    f->h = h;
    f->spp = spp;
    cudaError_t e = cudaMalloc(&f->fb, uint64_t(w) * h * sizeof(float4));
    if (e == cudaSuccess && with_hits) e = cudaMalloc(&f->hits, uint64_t(w) * h * spp * sizeof(hrt_hit));
    if (e == cudaSuccess) e = cudaMalloc(&f->dscene, sizeof(SceneLaunch));
    if (e == cudaSuccess) e = cudaMalloc(&f->counters, sizeof(TraceCounters));
    if (e == cudaSuccess) e = cudaMalloc(&f->resolve_list, uint64_t(w) * h * sizeof(uint32_t));
    f->scratch_cap = std::min<uint64_t>(uint64_t(w) * h * spp, kScratchSamples);
    if (e == cudaSuccess) e = cudaMalloc(&f->resolve_scratch, f->scratch_cap * sizeof(float4));
    if (e != cudaSuccess) {
        hrt_frame_destroy(f);
        return cuda_fail(ctx, e, "hrt_frame_create");
    }
    *out = f;
    return HRT_OK;
}

hrt_status hrt_frame_destroy(hrt_frame* f) {
    if (!f) return HRT_OK;
    DeviceSet ds(f->ctx->device);
    if (f->fb) cudaFree(f->fb);
    if (f->hits) cudaFree(f->hits);
    if (f->dscene) cudaFree(f->dscene);
    if (f->counters) cudaFree(f->counters);
    if (f->resolve_list) cudaFree(f->resolve_list);
    if (f->resolve_scratch) cudaFree(f->resolve_scratch);
    delete f;
    return HRT_OK;
}

hrt_status hrt_frame_device_ptrs(const hrt_frame* f, float** rgba, hrt_hit** hits) {
    if (!f) return HRT_ERR_INVALID_ARG;
    if (rgba) *rgba = reinterpret_cast<float*>(f->fb);
    if (hits) *hits = f->hits;
    return HRT_OK;
}

hrt_status hrt_frame_download(hrt_frame* f, float* rgba, hrt_hit* hits, void* stream) {
    if (!f) return HRT_ERR_INVALID_ARG;
    hrt_context* ctx = f->ctx;
    DeviceSet ds(ctx->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (rgba) CK(ctx, cudaMemcpyAsync(rgba, f->fb, uint64_t(f->w) * f->h * 16, cudaMemcpyDeviceToHost, s), "download frame");
    if (hits) {
        if (!f->hits) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_frame_download: frame has no hit records");
        CK(ctx, cudaMemcpyAsync(hits, f->hits, uint64_t(f->w) * f->h * f->spp * sizeof(hrt_hit), cudaMemcpyDeviceToHost, s),
           "download hits");
    }
    if (f->stats_pending) {  // an asynchronous trace: its status (and statistics) come with the download
        TraceCounters c;
        hrt_status st = read_counters(ctx, f->counters, &c, s);
        f->stats_pending = false;
        counters_to_stats(c, f->pending_primary, &f->stats);
        return st;
    }
    CK(ctx, cudaStreamSynchronize(s), "download frame");
    return HRT_OK;
}

hrt_status hrt_frame_get_stats(const hrt_frame* cf, hrt_frame_stats* out) {
    if (!cf || !out) return HRT_ERR_INVALID_ARG;
    hrt_frame* f = const_cast<hrt_frame*>(cf);
    if (f->stats_pending) {
        DeviceSet ds(f->ctx->device);
        TraceCounters c;
        hrt_status st = read_counters(f->ctx, f->counters, &c, nullptr);
        if (st != HRT_OK) return st;
        counters_to_stats(c, f->pending_primary, &f->stats);
        f->stats_pending = false;
    }
    *out = f->stats;
    return HRT_OK;
}

hrt_status hrt_trace(hrt_context* ctx, const hrt_tlas* tlas, const hrt_camera* cam, const hrt_trace_params* p,
                     hrt_frame* f, void* stream) {
    Range range("hrt_trace");
    if (!ctx) return HRT_ERR_INVALID_ARG;
    if (!tlas || !cam || !p || !f) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_trace: null argument");
    if (hrt_status ps = check_params(ctx, p, "hrt_trace")) return ps;
    if (p->record_hits && !f->hits) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_trace: record_hits on a frame without hit records");
    DeviceSet ds(ctx->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    SceneLaunch sl;
    fill_scene(sl, tlas, cam, f, 0);
    CK(ctx, cudaMemcpyAsync(f->dscene, &sl, sizeof(sl), cudaMemcpyHostToDevice, s), "upload scene");
    CK(ctx, cudaMemsetAsync(f->counters, 0, sizeof(TraceCounters), s), "reset counters");
    TraceLaunch L = make_launch(p, f->dscene, 1, sl.work_count, f->counters, tlas->type_mask, f->resolve_list,
                                uint64_t(f->w) * f->h, f->resolve_scratch, f->scratch_cap, f->spp);
    CK(ctx, launch_trace(L, node_mode(tlas->precision_mask, tlas->nodes != nullptr), s, ctx->sm_count), "launch trace");
    f->pending_primary = uint64_t(f->w) * f->h * f->spp;
    f->stats_pending = true;
    if (p->async) return HRT_OK;
    TraceCounters c;
    hrt_status st = read_counters(ctx, f->counters, &c, s);
    if (st != HRT_OK) return st;
    counters_to_stats(c, f->pending_primary, &f->stats);
    f->stats_pending = false;
    return HRT_OK;
}

hrt_status hrt_trace_rays(hrt_context* ctx, const hrt_tlas* tlas, const float* rays, uint64_t n, const hrt_trace_params* p,
                          hrt_hit* hits, int32_t memory, void* stream) {
    Range range("hrt_trace_rays");
    if (!ctx) return HRT_ERR_INVALID_ARG;
    if (!tlas || !p || (n && (!rays || !hits))) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_trace_rays: null argument");
    if (memory != HRT_MEMORY_HOST && memory != HRT_MEMORY_DEVICE)
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_trace_rays: unknown memory kind");
    if (hrt_status ps = check_params(ctx, p, "hrt_trace_rays")) return ps;
    if (n == 0) return HRT_OK;
    DeviceSet ds(ctx->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const float* dr = rays;
    hrt_hit* dh = hits;
    float* tr = nullptr;
    hrt_hit* th = nullptr;
    TraceCounters* ctr = nullptr;
    auto done = [&]() {
        if (tr) cudaFree(tr);
        if (th) cudaFree(th);
        if (ctr) cudaFree(ctr);
    };
    cudaError_t e = cudaMalloc(&ctr, sizeof(TraceCounters));
    if (e == cudaSuccess) e = cudaMemsetAsync(ctr, 0, sizeof(TraceCounters), s);
    if (e == cudaSuccess && memory == HRT_MEMORY_HOST) {
        e = cudaMalloc(&tr, n * 24);
        if (e == cudaSuccess) e = cudaMalloc(&th, n * sizeof(hrt_hit));
        if (e == cudaSuccess) e = cudaMemcpyAsync(tr, rays, n * 24, cudaMemcpyHostToDevice, s);
        dr = tr;
        dh = th;
    }
    if (e == cudaSuccess)
        e = launch_trace_rays(tlas->dev, tlas->nodes, tlas->n, dr, n, p->tmin, p->tmax, p->fp64_resolve, bounds_of(p),
                              dh, ctr, s, ctx->sm_count);
    if (e == cudaSuccess && memory == HRT_MEMORY_HOST) e = cudaMemcpyAsync(hits, th, n * sizeof(hrt_hit), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) {
        done();
        return cuda_fail(ctx, e, "hrt_trace_rays");
    }
    TraceCounters c;
    hrt_status st = read_counters(ctx, ctr, &c, s);
    done();
    return st;
}

hrt_status hrt_trace_rays_noalloc(hrt_context* ctx, const hrt_tlas* tlas, const float* rays, uint64_t n,
                                  const hrt_trace_params* p, hrt_hit* hits, void* stream) {
    if (!ctx) return HRT_ERR_INVALID_ARG;
    if (!tlas || !p || (n && (!rays || !hits))) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_trace_rays_noalloc: null argument");
    if (n > HRT_NOALLOC_MAX_RAYS)
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_trace_rays_noalloc: %llu rays; at most %u per call",
                    (unsigned long long)n, HRT_NOALLOC_MAX_RAYS);
    if (hrt_status ps = check_params(ctx, p, "hrt_trace_rays_noalloc")) return ps;
    DeviceSet ds(ctx->device);
    // the call copies through pageable host memory and synchronises the stream, neither of which
    // a stream capture allows: refuse a capturing stream before enqueueing anything
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    CK(ctx, cudaStreamIsCapturing(static_cast<cudaStream_t>(stream), &cap), "hrt_trace_rays_noalloc");
    if (cap != cudaStreamCaptureStatusNone)
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_trace_rays_noalloc: the stream is being captured");
    uint32_t err = 0;
    cudaError_t e = trace_rays_noalloc(ctx->device, tlas->dev, tlas->nodes, tlas->n, rays, n, p->tmin, p->tmax,
                                       p->fp64_resolve, bounds_of(p), hits, static_cast<cudaStream_t>(stream),
                                       ctx->sm_count, &err);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "hrt_trace_rays_noalloc");
    return error_status(ctx, err);
}

hrt_status hrt_batch_create(hrt_context* ctx, const hrt_scene_desc* scenes, uint32_t n, const hrt_trace_params* p,
                            void* stream, hrt_batch** out) {
    Range range("hrt_batch_create");
    if (!ctx) return HRT_ERR_INVALID_ARG;
    if (!scenes || !n || !p || !out) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_batch_create: null or empty argument");
    *out = nullptr;
    if (hrt_status ps = check_params(ctx, p, "hrt_batch_create")) return ps;
    DeviceSet ds(ctx->device);
    hrt_batch* b = new (std::nothrow) hrt_batch();
    if (!b) return fail(ctx, HRT_ERR_OOM, "hrt_batch_create: host allocation");
    b->ctx = ctx;
    b->async = p->async != 0;
    for (uint32_t i = 0; i < n; ++i) b->frames.push_back(scenes[i].frame);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    hrt_status st = make_plan(ctx, "hrt_batch_create", scenes, n, p->split_types != 0, p->record_hits != 0, s, b->plan);
    if (st != HRT_OK) {
        hrt_batch_destroy(b);
        return st;
    }
    // capture: per group, counter reset + the persistent trace launch (+ the FP64 pass); then the
    // counters to page-locked host memory
    cudaStream_t cap = nullptr;
    cudaError_t e = cudaMallocHost(&b->host_ctr, b->plan.groups.size() * sizeof(TraceCounters));
    if (e == cudaSuccess) memset(b->host_ctr, 0, b->plan.groups.size() * sizeof(TraceCounters));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
    Branches br;
    if (e == cudaSuccess) e = br.create();
    if (e == cudaSuccess) e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t e2 = enqueue_plan(b->plan, p, cap, ctx->sm_count, &br);
        if (e2 == cudaSuccess)
            e2 = cudaMemcpyAsync(b->host_ctr, b->plan.counters, b->plan.groups.size() * sizeof(TraceCounters),
                                 cudaMemcpyDeviceToHost, cap);
        cudaError_t e3 = cudaStreamEndCapture(cap, &b->graph);
        e = e2 != cudaSuccess ? e2 : e3;
    }
    br.destroy();
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (cap) cudaStreamDestroy(cap);
    if (e != cudaSuccess) {
        hrt_batch_destroy(b);
        return cuda_fail(ctx, e, "hrt_batch_create");
    }
    *out = b;
    return HRT_OK;
}

hrt_status hrt_batch_launch(hrt_batch* b, void* stream) {
    Range range("hrt_batch_launch");
    if (!b) return HRT_ERR_INVALID_ARG;
    hrt_context* ctx = b->ctx;
    DeviceSet ds(ctx->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (b->async && b->launched && cudaEventQuery(b->done) == cudaSuccess) {
        // the previous replay has finished: report its device error before replaying again
        uint32_t err = 0;
        for (size_t g = 0; g < b->plan.groups.size(); ++g) err |= b->host_ctr[g].error;
        if (hrt_status st = error_status(ctx, err)) return st;
    }
    CK(ctx, cudaGraphLaunch(b->exec, s), "hrt_batch_launch");
    CK(ctx, cudaEventRecord(b->done, s), "hrt_batch_launch");
    b->launched = true;
    if (b->async) return HRT_OK;
    TraceCounters c;
    hrt_status st = read_plan_counters(ctx, b->plan, &c, s);
    if (st != HRT_OK) return st;
    // the batch's counters are shared; report them on the first frame
    if (!b->frames.empty()) {
        counters_to_stats(c, b->plan.primary, &b->frames[0]->stats);
        b->frames[0]->stats_pending = false;
    }
    return HRT_OK;
}

hrt_status hrt_batch_set_cameras(hrt_batch* b, const hrt_camera* cams, uint32_t n, void* stream) {
    if (!b) return HRT_ERR_INVALID_ARG;
    hrt_context* ctx = b->ctx;
    if (!cams || n != b->plan.pos.size())
        return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_batch_set_cameras: need one camera per scene (%zu)", b->plan.pos.size());
    DeviceSet ds(ctx->device);
    for (uint32_t i = 0; i < n; ++i) {
        SceneLaunch& sl = b->plan.table[b->plan.pos[i]];
        memcpy(sl.view_inv, cams[i].view_inverse, sizeof(sl.view_inv));
        memcpy(sl.proj_inv, cams[i].proj_inverse, sizeof(sl.proj_inv));
    }
    // from pageable memory: the copy is staged before the call returns, so the table may change again
    CK(ctx, cudaMemcpyAsync(b->plan.dtable, b->plan.table.data(), b->plan.table.size() * sizeof(SceneLaunch),
                            cudaMemcpyHostToDevice, static_cast<cudaStream_t>(stream)),
       "hrt_batch_set_cameras");
    return HRT_OK;
}

uint64_t hrt_batch_table_bytes(const hrt_batch* b) { return b ? b->plan.table.size() * sizeof(SceneLaunch) : 0; }

hrt_status hrt_batch_download(hrt_batch* b, float* const* rgba, void* stream, int32_t synchronise) {
    if (!b) return HRT_ERR_INVALID_ARG;
    hrt_context* ctx = b->ctx;
    if (!rgba) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_batch_download: null destination array");
    DeviceSet ds(ctx->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    for (size_t i = 0; i < b->frames.size(); ++i) {
        if (!rgba[i]) continue;
        const hrt_frame* f = b->frames[i];
        CK(ctx, cudaMemcpyAsync(rgba[i], f->fb, uint64_t(f->w) * f->h * 16, cudaMemcpyDeviceToHost, s),
           "hrt_batch_download");
    }
    if (!synchronise) return HRT_OK;
    CK(ctx, cudaStreamSynchronize(s), "hrt_batch_download");
    // the replay before these copies has finished (same stream): its device error, if any
    if (b->launched && cudaEventQuery(b->done) == cudaSuccess) {
        uint32_t err = 0;
        for (size_t g = 0; g < b->plan.groups.size(); ++g) err |= b->host_ctr[g].error;
        return error_status(ctx, err);
    }
    return HRT_OK;
}

hrt_status hrt_autotune(hrt_context* ctx, const hrt_scene_desc* scenes, uint32_t n, const hrt_trace_params* base,
                        uint32_t reps, void* stream, hrt_trace_params* best, float* best_ms) {
    Range range("hrt_autotune");
    if (!ctx) return HRT_ERR_INVALID_ARG;
    if (!scenes || !n || !base || !best) return fail(ctx, HRT_ERR_INVALID_ARG, "hrt_autotune: null or empty argument");
    if (hrt_status ps = check_params(ctx, base, "hrt_autotune")) return ps;
    if (reps == 0) reps = 3;
    DeviceSet ds(ctx->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // one plan per grouping (split by type only matters when the scenes mix types)
    ScenePlan plans[2];
    hrt_status st = make_plan(ctx, "hrt_autotune", scenes, n, false, false, s, plans[0]);
    uint32_t nplans = 1;
    uint32_t kinds = 0;  // primitive types present
    if (st == HRT_OK) {
        for (uint32_t i = 0; i < n; ++i) kinds |= scenes[i].tlas->type_mask;
        if (prim_kind(kinds) == 3) {
            st = make_plan(ctx, "hrt_autotune", scenes, n, true, false, s, plans[1]);
            nplans = 2;
        }
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    Branches br;
    auto cleanup = [&]() {
        plans[0].release();
        plans[1].release();
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        br.destroy();
    };
    if (st != HRT_OK) {
        cleanup();
        return st;
    }
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = br.create();
    const uint32_t variants[3] = {1, 2, 3}, refills[2] = {8, 16}, agains[3] = {2, 4, 8};
    float best_t = -1.0f;
    hrt_trace_params bp = *base;
    for (uint32_t split = 0; split < nplans && e == cudaSuccess; ++split)
        for (uint32_t v : variants)
            for (uint32_t r : refills)
                for (uint32_t la : agains) {
                    hrt_trace_params p = *base;
                    p.kernel_variant = v;
                    p.refill = r;
                    p.speculative = 1;
                    p.leaf_again = la;
                    p.split_types = split;
                    p.record_hits = 0;
                    p.count_stats = 0;
                    float tot = 0.0f;
                    for (uint32_t k = 0; k <= reps && e == cudaSuccess; ++k) {
                        e = cudaEventRecord(e0, s);
                        if (e == cudaSuccess) e = enqueue_plan(plans[split], &p, s, ctx->sm_count, &br);
                        if (e == cudaSuccess) e = cudaEventRecord(e1, s);
                        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                        float ms = 0.0f;
                        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
                        if (k > 0) tot += ms;  // the first run warms up
                    }
                    if (e != cudaSuccess) break;
                    TraceCounters c;
                    st = read_plan_counters(ctx, plans[split], &c, s);
                    if (st != HRT_OK) {
                        cleanup();
                        return st;
                    }
                    float mean = tot / float(reps);
                    if (best_t < 0.0f || mean < best_t) {
                        best_t = mean;
                        bp = p;
                        bp.record_hits = base->record_hits;
                        bp.count_stats = base->count_stats;
                    }
                }
    // per-type variants: with one launch per primitive type, each type's group may prefer
    // another occupancy than the others (Phantom's long solve against LSS and DOTS)
    if (e == cudaSuccess && bp.split_types && nplans == 2) {
        for (uint32_t t = 0; t < 3 && e == cudaSuccess; ++t) {
            if (!((kinds >> t) & 1u)) continue;
            for (uint32_t v : variants) {
                if (v == bp.kernel_variant) continue;
                hrt_trace_params p = bp;
                p.record_hits = 0;
                p.count_stats = 0;
                p.variant_by_type = (bp.variant_by_type & ~(15u << (4 * t))) | (v << (4 * t));
                float tot = 0.0f;
                for (uint32_t k = 0; k <= reps && e == cudaSuccess; ++k) {
                    e = cudaEventRecord(e0, s);
                    if (e == cudaSuccess) e = enqueue_plan(plans[1], &p, s, ctx->sm_count, &br);
                    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
                    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                    float ms = 0.0f;
                    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
                    if (k > 0) tot += ms;
                }
                if (e != cudaSuccess) break;
                TraceCounters c;
                st = read_plan_counters(ctx, plans[1], &c, s);
                if (st != HRT_OK) {
                    cleanup();
                    return st;
                }
                const float mean = tot / float(reps);
                if (mean < best_t) {
                    best_t = mean;
                    bp.variant_by_type = p.variant_by_type;
                }
            }
        }
    }
    cleanup();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "hrt_autotune");
    *best = bp;
    if (best_ms) *best_ms = best_t;
    return HRT_OK;
}

hrt_status hrt_batch_destroy(hrt_batch* b) {
    if (!b) return HRT_OK;
    DeviceSet ds(b->ctx->device);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->done) cudaEventDestroy(b->done);
    if (b->host_ctr) cudaFreeHost(b->host_ctr);
    b->plan.release();
    delete b;
    return HRT_OK;
}

}  // extern "C"
