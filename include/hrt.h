/* include/hrt.h -- C ABI of the GB300 hair ray tracer (libhrt.so).
 *
 * The entry points replace the reference's (mmzala/vkhrt) hair path:
 *   hrt_blas_build   <- BottomLevelAccelerationStructure(const BLASInput&, ...)
 *                       include/bottom_level_acceleration_structure.hpp:34, together with the
 *                       geometry processing that produces its input
 *                       (ProcessHairCurves / ProcessHairLSS / ProcessHairDOTS,
 *                       source/resources/model/geometry_processor.cpp:604-779) and the
 *                       per-type BLASInput assembly (source/renderer.cpp:543-692)
 *   hrt_blas_type    <- BottomLevelAccelerationStructure::Type()       (hpp:41)
 *   hrt_blas_transform <- BottomLevelAccelerationStructure::Transform() (hpp:42)
 *   hrt_tlas_build   <- TopLevelAccelerationStructure(const std::vector<BLAS>&, ...)
 *                       include/top_level_acceleration_structure.hpp:12
 *   hrt_trace        <- Renderer::Render -> traceRaysKHR(W, H, 1)  (source/renderer.cpp:83-166)
 *                       running ray_gen.rgen / hair_intersection.rint / hair_closest_hit.rchit /
 *                       triangle_closest_hit.rchit / miss.rmiss
 *   hrt_camera_look_at <- FlyCamera::ViewMatrix/ProjectionMatrix (source/fly_camera.cpp:25-35)
 *                       and CameraResource::Update (source/resources/camera_resource.cpp:16-22)
 *
 * Conventions: opaque handles, the caller destroys them; host input arrays are copied (the
 * caller may free them on return, as after the staging copies of model.cpp:52-223); every
 * call returns an hrt_status instead of aborting (the reference's VkCheckResult logs and
 * aborts, vk_common.cpp:5-15); hrt_last_error() gives the message of the last failure on a
 * context. A context is used by one host thread at a time. Work is ordered on the CUDA stream
 * passed in (NULL = the legacy default stream).
 */
#ifndef HRT_H
#define HRT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HRT_ABI_VERSION 10

typedef enum hrt_status {
    HRT_OK = 0,
    HRT_ERR_INVALID_ARG = 1,
    HRT_ERR_OOM = 2,
    HRT_ERR_CUDA = 3,
    HRT_ERR_STACK_OVERFLOW = 4, /* traversal stack depth exceeded (device error word) */
    HRT_ERR_TIMEOUT = 5,        /* a bounded device loop hit its iteration cap */
    HRT_ERR_UNSUPPORTED = 6,
    HRT_ERR_BOUNDS = 7          /* a device index check failed (builds with HRT_CHECKED only) */
} hrt_status;

typedef struct hrt_context hrt_context;
typedef struct hrt_blas hrt_blas;
typedef struct hrt_tlas hrt_tlas;
typedef struct hrt_frame hrt_frame;
typedef struct hrt_batch hrt_batch;

/* Intersector of a BLAS; replaces BLASType {eMesh, eHair, eVoxels}
 * (include/bottom_level_acceleration_structure.hpp:12-17), where the reference tags LSS as
 * eMesh (renderer.cpp:656) and picks the hit group by that type (top_level...cpp:32). */
typedef enum hrt_geometry_type {
    HRT_BLAS_PHANTOM = 0, /* cubic Bezier segments, Phantom ray-hair intersector */
    HRT_BLAS_LSS = 1,     /* linear swept spheres (round cones, both end caps) */
    HRT_BLAS_DOTS = 2,    /* disjoint orthogonal triangle strips, 4 triangles per segment */
    HRT_BLAS_MESH = 3,    /* indexed triangle mesh (BLASType::eMesh), optional per-vertex normals */
    HRT_BLAS_VOXELS = 4   /* hair voxelised into boxes (BLASType::eVoxels), ray-box hits */
} hrt_geometry_type;

typedef enum hrt_precision {
    HRT_PRECISION_FP32 = 0,      /* FP32 BVH8 boxes, FP32 primitives */
    HRT_PRECISION_QUANTISED = 1  /* 8-bit BVH8 child boxes; Phantom segments as a 4-byte index
                                    into the BLAS's strand vertex stream (the strands' FP32
                                    vertices and radii, 16 B each, shared by the two segments
                                    that meet there), from which the leaf test rebuilds the
                                    Bezier control points bit for bit */
} hrt_precision;

typedef enum hrt_memory {
    HRT_MEMORY_HOST = 0,
    HRT_MEMORY_DEVICE = 1
} hrt_memory;

/* Hair geometry of one BLAS. Lines come either from strands (strand_offsets: the vertices of
 * strand s are vertices[strand_offsets[s] .. strand_offsets[s+1]-1], consecutive vertices form
 * lines) or from explicit index pairs (line_indices, as GenerateLines,
 * geometry_processor.cpp:45-67). Radii: per vertex when `radius` is non-NULL, otherwise
 * const_radius (the reference's literal 0.02, geometry_processor.cpp:635,681,765). */
typedef struct hrt_blas_input {
    int32_t type;                   /* hrt_geometry_type */
    int32_t precision;              /* hrt_precision */
    int32_t memory;                 /* hrt_memory of the pointers below */
    uint32_t max_leaf;              /* primitives per BVH8 leaf, 1..3 (0 = default 1) */
    const float* vertices;          /* 3 floats per vertex */
    const float* radius;            /* 1 float per vertex, or NULL */
    const uint32_t* strand_offsets; /* nstrands + 1 entries, or NULL */
    const uint32_t* line_indices;   /* 2 per line, or NULL */
    uint64_t nvertices;
    uint64_t nstrands;
    uint64_t nlines;                /* with line_indices */
    float const_radius;
    float transform[16];            /* object to world, column major (glm::mat4) */
    uint32_t width;                 /* BVH node fan-out, 2..8 (0 = 8): children per node of the
                                       8-slot node formats (narrower trees are for measurement) */
    uint32_t flags;                 /* HRT_BUILD_* */
    /* HRT_BLAS_MESH (renderer.cpp:543-582): 3 vertex indices per triangle; triangle i reports
     * primitive id i. strand_offsets and line_indices must be NULL. */
    const uint32_t* tri_indices;
    uint64_t ntris;
    const float* normals;           /* 3 floats per vertex (interpolated at the hit), or NULL (face normal) */
    /* HRT_BLAS_VOXELS (GenerateVoxelMesh, geometry_processor.cpp:515-602): the strands' lines are
     * voxelised as capsules of radius const_radius on a grid of voxel_size cubes (0 = 0.1, the
     * reference's); every filled voxel is a box primitive reporting its grid index
     * x + y res_x + z res_x res_y as primitive id. Per-vertex radii are not used. */
    float voxel_size;
    /* Material of a HRT_BLAS_MESH (other types ignore it, as the reference's hair output does):
     * the reference's Material albedo (include/resources/gpu_resources.hpp:160-180) as
     * triangle_closest_hit.rchit:71-81 fetches it. albedo = albedo_factor x the albedo map sampled
     * at the hit's texture coordinate, which interpolates texcoords with the hit's barycentrics
     * (1 - u - v, u, v) like the normal (rchit:39); bilinear, repeat addressing, texel centres at
     * ((i + 0.5) / width, (j + 0.5) / height), full resolution (the reference's default sampler,
     * gpu_resources.hpp:44-62; a closest-hit shader has no derivatives, so mip level 0). The
     * Lambert shading modes multiply their colour by albedo.rgb; HRT_SHADE_DEBUG, the reference's
     * output (rchit:84), does not use it. `memory` applies to texcoords and albedo_map. */
    const float* texcoords;         /* 2 floats per vertex, or NULL (no map lookup) */
    float albedo_factor[4];         /* RGBA, default 1, 1, 1, 1 */
    const float* albedo_map;        /* width x height RGBA floats, row-major, row 0 at v = 0, or NULL */
    uint32_t albedo_map_width, albedo_map_height; /* each 1..16384 with a map */
} hrt_blas_input;

#define HRT_BUILD_KEEP_INTERMEDIATE 1u /* keep Morton codes, binary tree, boxes (hrt_blas_get) */

typedef struct hrt_blas_info {
    uint64_t nprims;        /* primitives: line segments (LSS, DOTS: two BVH references each), triangles, voxels */
    uint64_t nnodes;        /* BVH8 nodes */
    uint64_t node_bytes;    /* bytes per node (224 FP32, 80 quantised) */
    uint64_t prim_bytes;    /* bytes per primitive record */
    uint64_t device_bytes;  /* total device memory held */
    float bounds[6];        /* object-space lo xyz, hi xyz */
    float build_ms;         /* device time of the last build or refit */
} hrt_blas_info;

/* Parts of a built BLAS copied to the host for inspection (bit-exact tests). A BLAS keeps only
 * what tracing reads (NODES, PRIMS, PRIM_ORDER, STRAND_VERTICES); the other parts need
 * HRT_BUILD_KEEP_INTERMEDIATE (otherwise hrt_blas_get returns HRT_ERR_UNSUPPORTED).
 * n below is the number of BVH references: nprims, or 2 nprims for LSS and DOTS BLASes, whose
 * segments enter the BVH as the boxes of their two halves (reference id 2 segment + half).
 * CURVES, DOTS_VERTICES and LSS have one row per segment. */
typedef enum hrt_blas_part {
    HRT_PART_PRIM_BOXES = 0,    /* float[n][6], reference order */
    HRT_PART_MORTON_SORTED = 1, /* uint64[n] (needs HRT_BUILD_KEEP_INTERMEDIATE) */
    HRT_PART_SORTED_INDEX = 2,  /* uint32[n] (needs KEEP_INTERMEDIATE) */
    HRT_PART_BIN_LEFT = 3,      /* uint32[n-1] (needs KEEP_INTERMEDIATE) */
    HRT_PART_BIN_RIGHT = 4,
    HRT_PART_BIN_BOXES = 5,     /* float[n-1][6] */
    HRT_PART_NODES = 6,         /* raw BVH8 nodes, nnodes * node_bytes */
    HRT_PART_PRIM_ORDER = 7,    /* uint32[n]: leaf slot -> reference id */
    HRT_PART_PRIMS = 8,         /* raw primitive records in slot order, n * prim_bytes */
    HRT_PART_CURVES = 9,        /* float[nprims][12] Bezier control points (Phantom, FP32) */
    HRT_PART_DOTS_VERTICES = 10,/* float[nprims][36] (DOTS), the reference's 12 vertices/segment */
    HRT_PART_LSS = 11,          /* float[nprims][8]: p0 xyz, p1 xyz, r0, r1 */
    HRT_PART_QNODES = 12,       /* raw quantised nodes (80 B each); of an FP32 BLAS only when kept */
    HRT_PART_STRAND_VERTICES = 13,/* float[nentries][4] quantised Phantom strand vertex stream:
                                     per run of joined lines (each starting where the previous ends,
                                     with the same radius there) the point before it, its start,
                                     each line's end, the point after it; {x, y, z, radius} */
    HRT_PART_TRI_TEXCOORDS = 14   /* float[ntris][6]: a textured mesh's texture coordinates per
                                     triangle, in triangle order (u0 v0 u1 v1 u2 v2) */
} hrt_blas_part;

typedef struct hrt_camera {
    float view_inverse[16]; /* column major, CameraUniformData::viewInverse */
    float proj_inverse[16]; /* column major, CameraUniformData::projInverse */
} hrt_camera;

typedef enum hrt_shading {
    HRT_SHADE_DEBUG = 0,        /* GetDebugColor(primitive id): the reference's closest-hit output */
    HRT_SHADE_LAMBERT = 1,      /* shading.glsl Shade(normal) */
    HRT_SHADE_LAMBERT_SHADOW = 2/* Shade(normal) with one shadow ray toward the light */
} hrt_shading;

typedef struct hrt_trace_params {
    float tmin;         /* 0.001 (ray_gen.rgen:27) */
    float tmax;         /* 10000 (ray_gen.rgen:28) */
    uint32_t spp;       /* samples per pixel */
    uint32_t jitter;    /* 0: pixel centre when spp == 1; jittered otherwise */
    uint32_t seed;
    uint32_t shading;   /* hrt_shading */
    float shadow_tmin;  /* 1e-4 */
    uint32_t fp64_resolve; /* re-solve non-converged Phantom candidates in FP64 (default 1) */
    uint32_t record_hits;  /* write per-sample hit records into the frame */
    uint32_t async;        /* 0: synchronise and check the device error word before returning */
    uint32_t count_stats;  /* accumulate traversal counters into the frame stats */
    uint32_t kernel_variant; /* resident blocks per SM (the register split): 0, 1: 4; 2: 3 (more registers
                                per thread); 3: 5 (fewer) */
    uint32_t refill;         /* idle lanes of a warp that trigger a work fetch, 1..32 (0 = 16; default 8) */
    uint32_t speculative;    /* lanes that hold a leaf keep traversing while others search (0/1; default 1) */
    uint32_t split_types;    /* batches: one persistent launch per primitive type instead of one for all (0/1) */
    /* Environment map for primary rays that miss (miss.rmiss:17-37), or NULL for the constant black
     * background: device float4 RGBA texels, env_height rows of env_width, equirectangular, row 0 at
     * v = 0; sampled bilinearly (u repeats, v clamps to the edge rows), then 1 - exp(-c) and gamma
     * 1/2.2 as the reference's miss shader. */
    const float* env_map;
    uint32_t env_width, env_height;
    uint32_t leaf_again;     /* repeat the leaf phase while at least this many lanes of a warp hold untested
                                leaf children (0 = one leaf per lane per phase; default 4) */
    /* Bounds of every ray's traversal (0 = the defaults, 65536 steps and 64 stack entries; a
     * depth above 64 is refused). A ray that exceeds one stops, the launch stops taking work, and
     * the call (or the next call that reads the launch's status: hrt_frame_get_stats,
     * hrt_frame_download, hrt_batch_download with synchronise, hrt_batch_launch without async)
     * returns HRT_ERR_TIMEOUT or HRT_ERR_STACK_OVERFLOW; the context stays usable. */
    uint32_t max_steps;
    uint32_t max_depth;
    /* kernel_variant per primitive type, for a launch (or a batch group) whose BLASes all have one
     * hair type: 4 bits per hrt_geometry_type t (Phantom, LSS, DOTS) at bits 4t..4t+3, 0 =
     * kernel_variant; launches of meshes, voxels or mixed types use kernel_variant. hrt_autotune
     * fills it when per-type variants beat one variant for all groups. */
    uint32_t variant_by_type;
} hrt_trace_params;

typedef struct hrt_hit {
    float t;         /* closest hit distance, or -1 on a miss */
    uint32_t prim;   /* reported primitive id (gl_PrimitiveID), 0xffffffff on a miss */
    uint32_t inst;   /* instance (gl_InstanceCustomIndexEXT), 0xffffffff on a miss */
    uint32_t flags;  /* HRT_HIT_* */
} hrt_hit;

#define HRT_HIT_SHADOWED 1u    /* the shadow ray was blocked */
#define HRT_HIT_FP64 2u        /* the closest hit came from the FP64 re-solve */

typedef struct hrt_frame_stats {
    uint64_t primary_rays;
    uint64_t shadow_rays;
    uint64_t nodes_visited;   /* with count_stats */
    uint64_t prims_tested;    /* with count_stats */
    uint64_t fp64_resolves;   /* FP64 re-solves run */
    uint64_t fp64_hits;       /* re-solves that produced a hit */
    uint64_t warp_cycles_node;  /* with count_stats: summed per-warp SM clocks in the node phase, */
    uint64_t warp_cycles_leaf;  /* the intersector (leaf) phase */
    uint64_t warp_cycles_other; /* and ray setup, shading and work fetch */
} hrt_frame_stats;

/* ---- context ------------------------------------------------------------------------- */
hrt_status hrt_context_create(int device, hrt_context** out);
hrt_status hrt_context_destroy(hrt_context* ctx);
const char* hrt_last_error(const hrt_context* ctx);
const char* hrt_status_string(hrt_status s);
int hrt_abi_version(void);

/* ---- BLAS (BottomLevelAccelerationStructure) ------------------------------------------ */
void hrt_blas_input_default(hrt_blas_input* in);
hrt_status hrt_blas_build(hrt_context* ctx, const hrt_blas_input* in, void* stream, hrt_blas** out);
hrt_status hrt_blas_destroy(hrt_blas* blas);
/* Moves the primitives of a built BLAS (animated strands): new vertex positions, and per-vertex
 * radii (hair) or normals (mesh) exactly when the build had them, for the same vertex count and
 * topology. Geometry, primitive boxes and records are recomputed and the BVH8 boxes refitted
 * bottom-up; the tree's topology and leaf order are kept, so its quality falls with large
 * motions (build anew then). TLASes that hold the BLAS must be built again afterwards (they
 * copy its bounds). No counterpart in the reference (it builds once). */
hrt_status hrt_blas_refit(hrt_blas* blas, const float* vertices, const float* per_vertex, int32_t memory, void* stream);
/* A built BLAS as bytes (host memory): tree, records, strand vertex stream, slot map, mesh
 * material and the refit topology (image version 4; LSS and DOTS records and slot-map entries
 * are per BVH reference, two per segment). hrt_blas_deserialize checks the image (header, sizes,
 * every node's child and leaf ranges, quantised Phantom records inside the strand vertex stream,
 * the slot map of two-reference BLASes, the material's sizes) before anything reaches the device
 * and rejects a corrupt one, or one of another version, with HRT_ERR_INVALID_ARG. No counterpart
 * in the reference (it rebuilds at every start). */
uint64_t hrt_blas_serialized_size(const hrt_blas* blas);
hrt_status hrt_blas_serialize(const hrt_blas* blas, void* dst, uint64_t bytes);
hrt_status hrt_blas_deserialize(hrt_context* ctx, const void* src, uint64_t bytes, void* stream, hrt_blas** out);
int32_t hrt_blas_type(const hrt_blas* blas);
hrt_status hrt_blas_transform(const hrt_blas* blas, float out[16]);
hrt_status hrt_blas_get_info(const hrt_blas* blas, hrt_blas_info* out);
/* Copies part `part` into host memory `dst` of `bytes` bytes (the exact size is required). */
hrt_status hrt_blas_get(const hrt_blas* blas, int32_t part, void* dst, uint64_t bytes);

/* ---- TLAS (TopLevelAccelerationStructure) ------------------------------------------------
 * Instance i = blases[i] with its transform, custom index i and the intersector of its type. */
hrt_status hrt_tlas_build(hrt_context* ctx, const hrt_blas* const* blases, uint32_t n, void* stream,
                          hrt_tlas** out);
hrt_status hrt_tlas_destroy(hrt_tlas* tlas);

/* ---- camera -------------------------------------------------------------------------------
 * lookAt (right handed) and perspectiveRH_ZO with the Y axis flipped (fly_camera.cpp:25-35),
 * inverted; computed in double and rounded to float. */
hrt_status hrt_camera_look_at(const float eye[3], const float center[3], const float up[3], float fovy_deg,
                              float aspect, float znear, float zfar, hrt_camera* out);

/* ---- frames and tracing ------------------------------------------------------------------ */
void hrt_trace_params_default(hrt_trace_params* p);
/* A device framebuffer (RGBA32F, width*height*4 floats) and, with record_hits, per-sample hit
 * records (width*height*spp hrt_hit). */
hrt_status hrt_frame_create(hrt_context* ctx, uint32_t width, uint32_t height, uint32_t spp, int32_t with_hits,
                            hrt_frame** out);
hrt_status hrt_frame_destroy(hrt_frame* f);
hrt_status hrt_frame_device_ptrs(const hrt_frame* f, float** rgba, hrt_hit** hits);
/* Copies the framebuffer (and hits, if non-NULL) to host memory; synchronises `stream`. */
hrt_status hrt_frame_download(hrt_frame* f, float* rgba, hrt_hit* hits, void* stream);
hrt_status hrt_frame_get_stats(const hrt_frame* f, hrt_frame_stats* out);

/* One frame: W*H*spp primary rays from `cam`, closest hit, shading, optional shadow rays. */
hrt_status hrt_trace(hrt_context* ctx, const hrt_tlas* tlas, const hrt_camera* cam, const hrt_trace_params* p,
                     hrt_frame* frame, void* stream);

/* Closest hit for explicit rays: rays = n x {ox, oy, oz, dx, dy, dz} floats, hits = n records;
 * both in `memory` (host or device). Uses p->tmin, p->tmax, p->fp64_resolve. */
hrt_status hrt_trace_rays(hrt_context* ctx, const hrt_tlas* tlas, const float* rays, uint64_t n,
                          const hrt_trace_params* p, hrt_hit* hits, int32_t memory, void* stream);

/* ---- closest hit without any device allocation -----------------------------------------------
 * No counterpart in the reference. For callers that cannot allocate device memory: a picking or
 * probing query issued from an interactive loop, where cudaFree's implicit device-wide
 * synchronisation would stall frames in flight, or an integration that runs under a fixed
 * device-memory budget. Same closest-hit kernel and results as hrt_trace_rays, with rays and
 * hits in HOST memory (n x {ox, oy, oz, dx, dy, dz} floats in, n hrt_hit out); the device
 * staging for both and the kernel's counters live in one static device array of
 * HRT_NOALLOC_SCRATCH_BYTES that every GPU loading the library keeps until the process exits.
 * n above HRT_NOALLOC_MAX_RAYS is rejected with HRT_ERR_INVALID_ARG. The first call on a device
 * looks up the array's device address; make that first call before any stream capture begins.
 * Each call copies the rays and hits through pageable host memory and synchronises `stream`
 * before it returns, so a call on a stream that is being captured is refused with
 * HRT_ERR_INVALID_ARG. Every call shares the array: calls that overlap on the GPU (other
 * streams, other host threads) race, so serialise them. */
#define HRT_NOALLOC_MAX_RAYS 65536u
#define HRT_NOALLOC_SCRATCH_BYTES (256u + HRT_NOALLOC_MAX_RAYS * 40u)
hrt_status hrt_trace_rays_noalloc(hrt_context* ctx, const hrt_tlas* tlas, const float* rays, uint64_t n,
                                  const hrt_trace_params* p, hrt_hit* hits, void* stream);

/* ---- batched multi-scene rendering ---------------------------------------------------------
 * All scenes are traced by one persistent launch (or, with split_types, one per primitive
 * type), captured once in a CUDA graph by hrt_batch_create and replayed by hrt_batch_launch. The
 * launch takes the scenes' pixels longest job first (most samples per pixel, then most
 * primitives), whatever their order in `scenes`; results do not depend on it. */
typedef struct hrt_scene_desc {
    const hrt_tlas* tlas;
    hrt_camera camera;
    hrt_frame* frame;   /* its width/height/spp give the scene's resolution */
} hrt_scene_desc;
hrt_status hrt_batch_create(hrt_context* ctx, const hrt_scene_desc* scenes, uint32_t n, const hrt_trace_params* p,
                            void* stream, hrt_batch** out);
hrt_status hrt_batch_launch(hrt_batch* b, void* stream);
hrt_status hrt_batch_destroy(hrt_batch* b);
/* New cameras for the batch's scenes (one per scene, in creation order), uploaded with the scene
 * table on `stream` ahead of the next hrt_batch_launch; the captured graph is reused. */
hrt_status hrt_batch_set_cameras(hrt_batch* b, const hrt_camera* cams, uint32_t n, void* stream);
/* Bytes one hrt_batch_set_cameras uploads. */
uint64_t hrt_batch_table_bytes(const hrt_batch* b);
/* Copies every scene's framebuffer to host memory: rgba[i] receives scene i's width*height
 * RGBA floats (scenes in creation order; NULL entries are skipped). The copies are enqueued on
 * `stream` (after an hrt_batch_launch on the same stream); with synchronise != 0 the call waits
 * for them, otherwise the caller synchronises the stream. Page-locked destinations make the
 * copies asynchronous. One call per batch in place of one hrt_frame_download (and one
 * synchronisation) per scene: the per-frame readback of the reference's present step. */
hrt_status hrt_batch_download(hrt_batch* b, float* const* rgba, void* stream, int32_t synchronise);

/* ---- autotuner ------------------------------------------------------------------------------
 * Times every candidate kernel configuration on the given scenes (occupancy variant 3/4/5 blocks
 * per SM x refill threshold 8/16 x leaf repetition 2/4/8, speculative traversal on, and for
 * scenes of mixed primitive types x one launch or one per type: HRT_AUTOTUNE_CANDIDATES or twice
 * that), each `reps` times with plain launches after one warm-up, and writes the fastest into
 * `best` (a copy of `base` with kernel_variant, refill, speculative, leaf_again and split_types
 * replaced) and its mean frame time into `best_ms`. */
#define HRT_AUTOTUNE_CANDIDATES 18u  /* 3 x 2 x 3, then up to 3 per primitive type (variant_by_type) */
hrt_status hrt_autotune(hrt_context* ctx, const hrt_scene_desc* scenes, uint32_t n, const hrt_trace_params* base,
                        uint32_t reps, void* stream, hrt_trace_params* best, float* best_ms);

/* ---- synthetic strands (stand-in for the reference's glTF hair assets) --------------------
 * Roots uniform on the unit-sphere cap of polar angle < cap_deg about +y; each strand grows
 * along the root normal in `step` increments, the direction of step k being
 * normalize(n - (0, droop * k, 0)); vertex k > 0 is displaced by
 * curl * (sin(curl_freq k + phase) b1 + cos(curl_freq k + phase) b2) in the plane normal to n;
 * radius tapers linearly from r_root to r_tip. Deterministic on every host (no libm calls). */
typedef struct hrt_strand_params {
    uint64_t seed;
    uint32_t nstrands;
    uint32_t nverts;    /* vertices per strand (>= 2) */
    float step, droop, curl, curl_freq, r_root, r_tip, cap_deg;
} hrt_strand_params;
void hrt_strand_params_default(hrt_strand_params* p);
/* vertices: nstrands*nverts*3 floats; radius: nstrands*nverts; offsets: nstrands+1 (host). */
hrt_status hrt_generate_strands(const hrt_strand_params* p, float* vertices, float* radius, uint32_t* offsets);
/* FNV-1a 64 over the bytes of the vertex and radius arrays. */
uint64_t hrt_checksum(const void* a, uint64_t abytes, const void* b, uint64_t bbytes);

#ifdef __cplusplus
}
#endif
#endif /* HRT_H */
