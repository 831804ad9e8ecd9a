// hrt_internal.h -- layouts shared by the BVH build (build.cu), the trace kernels (trace.cu)
// and the C ABI (api.cu). Device memory only; nothing here is part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "hrt.h"

namespace hrt {

constexpr uint32_t kLeafFlag = 0x80000000u;
constexpr int kStackSize = 64;          // traversal stack entries per ray (the most a launch may use)
constexpr uint32_t kMaxTraversalSteps = 1u << 16;  // per ray by default; exceeding it sets kErrTimeout

// Device error word bits (read back by the host after a launch).
constexpr uint32_t kErrStackOverflow = 1u;
constexpr uint32_t kErrTimeout = 2u;
constexpr uint32_t kErrBounds = 4u;  // HRT_CHECKED builds: an index outside its array (the load skipped)

// ---- BVH8 nodes -----------------------------------------------------------------------------
// Both node formats describe the same tree (same children, same order):
//   meta[k] == 0            empty slot
//   meta[k] & 0x80          internal child, node index child_base + (meta & 7)
//   otherwise               leaf: (meta >> 5) primitives from slot prim_base + (meta & 31)
// Child slots: a node's children sit in the 8 slots by direction (slot s holds the child whose
// centre lies furthest along (s&1 ? +x : -x, s&2 ? +y : -y, s&4 ? +z : -z) from the node's
// centre), so a ray visits slots in the order i ^ octant(ray) roughly front to back. Internal
// children are numbered from child_base in slot order, leaf primitives from prim_base in slot
// order. Empty slots hold an empty box (FP32: lo = +inf, hi = -inf; 8-bit: qlo = 255, qhi = 0).
struct alignas(16) NodeF {  // 224 bytes, FP32 child boxes (structure of arrays)
    float lo_x[8], hi_x[8], lo_y[8], hi_y[8], lo_z[8], hi_z[8];
    uint32_t child_base, prim_base;
    uint32_t imask;  // bit s set when slot s holds an internal child
    uint32_t pad0;
    uint8_t meta[8];
    uint32_t pad[2];
};
static_assert(sizeof(NodeF) == 224, "NodeF layout");

struct alignas(16) NodeQ {  // 80 bytes, child boxes as 8-bit offsets on a per-axis 2^e grid
    float px, py, pz;       // grid origin (min of the child boxes)
    uint8_t ex, ey, ez;     // e + 127
    uint8_t imask;          // bit s set when slot s holds an internal child
    uint32_t child_base, prim_base;
    uint8_t meta[8];
    uint8_t qlo_x[8], qhi_x[8], qlo_y[8], qhi_y[8], qlo_z[8], qhi_z[8];
};
static_assert(sizeof(NodeQ) == 80, "NodeQ layout");

// ---- primitive records (leaf slot order) ----------------------------------------------------
// Phantom FP32 (64 B): {start, r0} {cp1, r1} {cp2, id} {end, 0}
// Phantom quantised (4 B): the segment's first entry e in the strand vertex stream (float4
//                      {x, y, z, radius} per entry): entries e .. e + 3 are the GenerateCurves
//                      neighbours p0, p1, p2, p3, from which the leaf rebuilds the control points
//                      exactly; the id comes from the slot map
// LSS (32 B): {p0, r0} {p1, r1}; id from prim_ids
// DOTS (80 B): start, end, s*r0, t*r0, s*r1, t*r1 (18 floats), id, pad
struct alignas(16) PrimPhantomF { float4 a, b, c, d; };
struct alignas(16) PrimLss { float4 a, b; };
struct alignas(16) PrimDots { float4 a, b, c, d, e; };
// Mesh triangle (80 B): {v0, id} {v1, n0.x} {v2, n0.y} {n0.z, n1} {n2, has normals (0/1 bits)}
struct alignas(16) PrimTri { float4 a, b, c, d, e; };

// LSS and DOTS segments enter the BVH as two references, the boxes of the segment's halves (a
// long, thin segment's box holds far more empty space than its two halves' boxes); each
// reference's leaf slot holds a copy of the segment's record, and the slot map gives reference
// ids 2 s + h. Phantom segments stay single: their leaf test is long however tight the box,
// so halving buys fewer tests only of the kind that ends early.
inline constexpr uint32_t ref_shift(int type) { return (type == HRT_BLAS_LSS || type == HRT_BLAS_DOTS) ? 1u : 0u; }

struct DevBlas {
    const void* nodes;        // NodeF or NodeQ
    const void* prims;        // records in slot order
    const float4* verts;      // quantised Phantom: the strand vertex stream
    const uint32_t* prim_ids; // slot -> reference id (segment index << ref_shift | half)
    const uint32_t* partner;  // slot -> the slot of the same segment's other reference (LSS, DOTS)
    uint32_t type, precision, nprims, nnodes, ref_shift;
    float lo[3], hi[3];
    // mesh material: albedo factor, and with both set the map sampled at the per-triangle
    // texture coordinates
    float albedo[4];
    const float* uv;          // float[ntris][6], triangle order, or null
    const float4* albedo_map; // map_w x map_h RGBA texels, row 0 at v = 0, or null
    uint32_t map_w, map_h;
    uint32_t nverts;          // strand vertex stream entries (quantised Phantom)
};

struct DevInstance {
    DevBlas b;
    float w2o[12];   // world -> object, rows of a 3x4 affine matrix
    float nrm[9];    // object -> world normal matrix (inverse transpose, rows)
    uint32_t identity;
};

// TLAS: a binary BVH over the instances' world-space boxes (the reference's driver-built
// instance BVH, top_level_acceleration_structure.cpp:19-113), built on the host by median splits.
// Node 0 is the root. Internal node: a = left child, b = right child; leaf: a = kLeafFlag |
// instance index. A ray walks it with a stack of kTlasStack entries (the tree's depth is at most
// ceil(log2(instances)) + 1, and instances are limited to 2^24).
struct alignas(16) TlasNode {
    float lo[3];
    uint32_t a;
    float hi[3];
    uint32_t b;
};
static_assert(sizeof(TlasNode) == 32, "TlasNode layout");
constexpr int kTlasStack = 32;
constexpr uint32_t kMaxInstances = 1u << 24;

// Node format of a launch's BLASes: every instance FP32, every instance 8-bit, or per instance
// (a TLAS or a batch that mixes the two; the kernel branches on each instance's precision).
enum NodeMode : int { kNodesF = 0, kNodesQ = 1, kNodesPerInstance = 2 };

// One scene of a launch (a frame, or one scene of a batch).
struct SceneLaunch {
    const DevInstance* inst;
    const TlasNode* tlas;      // instance BVH (null for a scene of one instance)
    uint32_t ninst;
    uint32_t width, height, spp;
    uint32_t tiles_x;          // 8x4 pixel tiles per row
    uint64_t work_begin;       // first global work item (a tile-ordered pixel) of the scene
    uint64_t work_count;       // tiles * 32
    float view_inv[16], proj_inv[16];
    float4* fb;
    hrt_hit* hits;
};

struct TraceCounters {
    unsigned long long work;     // next work item
    unsigned long long primary, shadow, nodes, prims, fp64_resolves, fp64_hits;
    unsigned long long cycles_node, cycles_leaf, cycles_other;  // per-warp clock, with count_stats
    uint32_t error;
    uint32_t pad;
    unsigned long long resolve_n;  // pixels listed by the first pass for the FP64 pass
    unsigned long long work2;      // next list entry of the FP64 pass
};

struct TraceLaunch {
    const SceneLaunch* scenes;
    uint32_t nscenes;
    uint64_t total_work;
    float tmin, tmax, shadow_tmin;
    uint32_t jitter, seed, shading, fp64_resolve, record_hits, count_stats;
    uint32_t prim_kind;  // the primitive type of every instance, or 3 when they differ
    uint32_t variant;    // kernel variant (occupancy / register split), 0 = default
    uint32_t refill;     // idle lanes of a warp that trigger a work fetch (0 = 16)
    uint32_t speculative;  // lanes holding a leaf keep traversing while others search
    uint32_t leaf_again;   // repeat the leaf phase while this many lanes hold leaves (0 = once)
    uint32_t max_steps;    // traversal steps per ray (exceeding them sets kErrTimeout)
    int32_t max_depth;     // stack entries per ray, <= kStackSize (exceeding them sets kErrStackOverflow)
    TraceCounters* counters;
    // Two-pass FP64 re-solve: the first pass lists the work items (pixels) that met a Phantom
    // candidate whose FP32 solve did not converge; the second re-renders just those with the
    // FP64 re-solve inline. resolve_cap >= the number of pixels, so the list cannot overflow.
    uint32_t* resolve_list;
    uint64_t resolve_cap;
    // The FP64 pass takes one sample per lane when the listed pixels' samples fit the scratch
    // (per-sample colours, averaged per pixel in sample order by a third launch); otherwise one
    // pixel per lane.
    float4* resolve_scratch;
    uint64_t scratch_cap;  // samples
    uint32_t max_spp;      // over the scenes of the launch
    const float4* env_map; // miss shading (or null)
    uint32_t env_w, env_h;
};

// ---- host helpers (workload.cpp) ------------------------------------------------------------
// Inverse of a column-major 4x4 matrix in double (false when singular).
bool invert4(const double* m, double* out);

// ---- launch wrappers (trace.cu) --------------------------------------------------------------
cudaError_t launch_trace(const TraceLaunch& L, int node_mode, cudaStream_t s, int sm_count);
cudaError_t prepare_frames();  // frame kernels' attributes (shared memory / L1 split), once per context
// Per-ray traversal bounds of an explicit-ray launch.
struct RayBounds {
    uint32_t max_steps;
    int32_t max_depth;
};
cudaError_t launch_trace_rays(const DevInstance* inst, const TlasNode* tlas, uint32_t ninst, const float* rays,
                              uint64_t n, float tmin, float tmax, uint32_t fp64_resolve, RayBounds bounds,
                              hrt_hit* hits, TraceCounters* counters, cudaStream_t s, int sm_count);

// Closest hit for host rays through the static scratch array of trace.cu (no allocation);
// error_word receives the device error bits.
cudaError_t trace_rays_noalloc(int device, const DevInstance* inst, const TlasNode* tlas, uint32_t ninst,
                               const float* host_rays, uint64_t n, float tmin, float tmax, uint32_t fp64_resolve,
                               RayBounds bounds, hrt_hit* host_hits, cudaStream_t s, int sm_count,
                               uint32_t* error_word);

// ---- BVH build (build.cu) ----------------------------------------------------------------------
// Voxel primitive record (HRT_BLAS_VOXELS): box lo + grid index (bits), box hi.
struct PrimVoxel {
    float4 lo_id, hi;
};
struct BuildInput {
    int type, precision, max_leaf;
    int width;            // BVH node fan-out, 2..8
    const float* lines;   // device, n x 6
    const float* lrad;    // device, n x 2 (per line end)
    uint64_t n;
    bool keep_intermediate;
    const float* tris = nullptr;         // mesh: device, n x 9 (triangle vertices)
    const float* tri_normals = nullptr;  // mesh: device, n x 9 (vertex normals), or null
    const float* voxels = nullptr;       // voxels: device, n x 7 (box lo xyz, hi xyz, grid index bits)
};
// Voxelises nlines device lines (6 floats each) as capsules of radius r on cubes of `size`:
// allocates *vox (7 floats per filled voxel, ascending grid index), sets *nvox and grid
// (origin xyz, size, res xyz as floats).
cudaError_t voxelize_device(const float* lines, uint64_t nlines, float r, float size, float** vox, uint64_t* nvox,
                            float grid[8], cudaStream_t s, char* msg, size_t msglen);
struct BuildOutput {
    // owned device allocations (freed by the BLAS)
    void* nodes = nullptr;        // NodeF or NodeQ (per precision)
    void* qnodes_aux = nullptr;   // NodeQ copy when nodes are NodeF (inspection) or vice versa
    void* prims = nullptr;
    float4* verts = nullptr;      // quantised Phantom strand vertex stream
    uint32_t* prim_ids = nullptr;  // slot -> reference id
    uint32_t* partner = nullptr;   // slot -> partner slot (two references per segment only)
    float* prim_boxes = nullptr;  // nslots x 6, reference order
    float* curves = nullptr;      // Phantom n x 12 (FP32, segment order)
    float* geom = nullptr;        // DOTS n x 18 / LSS n x 8 (segment order)
    uint64_t* morton_sorted = nullptr;
    uint32_t* sorted_index = nullptr;
    uint32_t* bin_left = nullptr;
    uint32_t* bin_right = nullptr;
    float* bin_boxes = nullptr;
    uint32_t* prim_order = nullptr;
    uint64_t nnodes = 0, nverts = 0, node_bytes = 0, prim_bytes = 0, device_bytes = 0;
    uint64_t nslots = 0;  // BVH references = leaf slots = records
    float bounds[6] = {0, 0, 0, 0, 0, 0};
    std::vector<uint32_t> level_start;  // first node of each breadth-first level, then nnodes
};
// Runs the whole device build; returns a CUDA error or cudaSuccess; msg gets a reason.
cudaError_t build_blas_device(const BuildInput& in, BuildOutput& out, cudaStream_t s, char* msg, size_t msglen);
// Moves a built BLAS to new geometry of the same topology (in.n segments or triangles): boxes,
// records and the BVH8 node boxes (refitted bottom-up, level by level) are recomputed; the
// tree's topology and leaf order are kept.
cudaError_t refit_blas_device(const BuildInput& in, BuildOutput& out, cudaStream_t s, char* msg, size_t msglen);
void free_build_output(BuildOutput& out);
cudaError_t expand_dots(const float* geom, uint64_t n, float* out36, cudaStream_t s);
// Line generation from vertices (device pointers); see hrt_blas_input.
// Gathers mesh triangles (and their vertex normals when given) into n x 9 arrays.
cudaError_t make_tris(const float* verts, const float* vnrm, const uint32_t* idx, uint64_t ntris, float* tris,
                      float* tri_nrm, cudaStream_t s);
cudaError_t make_lines(const float* verts, const float* vrad, float const_radius, const uint32_t* strand_line_off,
                       const uint32_t* strand_vert_off, uint64_t nstrands, const uint32_t* line_idx, uint64_t nlines,
                       float* lines, float* lrad, cudaStream_t s);

}  // namespace hrt
