/* include/hrt.hpp -- C++ host interface of the hair ray tracer over the C ABI of hrt.h, with the
 * reference's class names and call shapes, so that C++ code written against mmzala/vkhrt's hair
 * path keeps its structure:
 *   BLASType, BLASInput, BottomLevelAccelerationStructure (Structure(), Type(), Transform(); move
 *     only)                 <- include/bottom_level_acceleration_structure.hpp:12-52
 *   TopLevelAccelerationStructure (neither copyable nor movable)
 *                           <- include/top_level_acceleration_structure.hpp:9-24
 *   Render(context, tlas, camera, params, frame)  <- Renderer::Render -> traceRaysKHR
 *                              (source/renderer.cpp:83-166)
 *   Batch (many scenes, one CUDA-graph replay per step; no counterpart in the reference, whose
 *     renderer traces one scene per frame)
 *   LookAt(...)             <- FlyCamera::ViewMatrix/ProjectionMatrix (source/fly_camera.cpp:25-35)
 *   TraceRays(...)          <- traceRayEXT for caller-supplied rays (shaders/ray_gen.rgen:34-45)
 *   BLAS Serialize/Load/Refit (no counterpart: the reference rebuilds at every start)
 * Header only; links against libhrt.so. Where the reference logs and aborts on a failed call
 * (VkCheckResult, source/vk_common.cpp:5-15) these classes throw hrt::Error, which carries the
 * status and hrt_last_error's message; a caller that wants the reference's behaviour catches it,
 * logs and aborts. Host arrays are copied by the calls that take them. */
#ifndef HRT_HPP
#define HRT_HPP

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "hrt.h"

namespace hrt {

class Error : public std::runtime_error {
public:
    Error(hrt_status s, const std::string& what) : std::runtime_error(what), status(s) {}
    hrt_status status;
};

// The error carries the context's message (or the status's name), prefixed with the call unless
// the message already starts with it.
inline void Check(const hrt_context* ctx, hrt_status s, const char* call) {
    if (s == HRT_OK) return;
    const char* m = ctx ? hrt_last_error(ctx) : nullptr;
    std::string msg = m && *m ? m : hrt_status_string(s);
    if (msg.rfind(call, 0) != 0) msg = std::string(call) + ": " + msg;
    throw Error(s, msg);
}

// One device (the compute part of the reference's VulkanContext).
class Context {
public:
    explicit Context(int device = 0) { Check(nullptr, hrt_context_create(device, &_ctx), "hrt_context_create"); }
    ~Context() { hrt_context_destroy(_ctx); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    hrt_context* Get() const { return _ctx; }

private:
    hrt_context* _ctx = nullptr;
};

// The reference's BLAS kinds (bottom_level_acceleration_structure.hpp:12-17): LSS and DOTS hair
// are eMesh BLASes there (renderer.cpp:656), Phantom hair is eHair.
enum class BLASType : uint8_t { eMesh, eHair, eVoxels };

inline BLASType TypeOf(hrt_geometry_type g) {
    return g == HRT_BLAS_PHANTOM ? BLASType::eHair : (g == HRT_BLAS_VOXELS ? BLASType::eVoxels : BLASType::eMesh);
}

inline std::array<float, 16> Identity() {
    return {1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f};
}

// Geometry of one BLAS in host memory (the reference passes device buffer addresses and build
// ranges, renderer.cpp:543-692; here the positions, radii and topology themselves).
struct BLASInput {
    hrt_geometry_type geometry = HRT_BLAS_PHANTOM;  // the intersector (the reference's hit group)
    hrt_precision precision = HRT_PRECISION_FP32;
    std::array<float, 16> transform = Identity();    // object to world, column major (glm::mat4)
    std::vector<float> positions;                     // 3 floats per vertex
    std::vector<float> radius;                        // per vertex, or empty: constRadius
    std::vector<uint32_t> strandOffsets;              // strands (nstrands + 1), or empty
    std::vector<uint32_t> lineIndices;                // or index pairs (GenerateLines)
    std::vector<uint32_t> triIndices;                 // HRT_BLAS_MESH
    std::vector<float> normals;                       // HRT_BLAS_MESH, per vertex, or empty
    float constRadius = 0.02f;                        // geometry_processor.cpp:635
    float voxelSize = 0.0f;                           // HRT_BLAS_VOXELS (0 = 0.1)
    uint32_t width = 0;                               // BVH node fan-out 2..8 (0 = 8)
    // HRT_BLAS_MESH material (triangle_closest_hit.rchit:71-81): albedo factor, and a map
    // (albedoMapWidth x albedoMapHeight RGBA floats, row 0 at v = 0) sampled at texCoords
    std::vector<float> texCoords;                     // 2 floats per vertex, or empty
    std::array<float, 4> albedoFactor = {1.0f, 1.0f, 1.0f, 1.0f};
    std::vector<float> albedoMap;
    uint32_t albedoMapWidth = 0, albedoMapHeight = 0;
};

class BottomLevelAccelerationStructure {
public:
    BottomLevelAccelerationStructure(const BLASInput& in, Context& ctx, void* stream = nullptr)
        : _ctx(ctx.Get()), _type(TypeOf(in.geometry)) {
        hrt_blas_input b;
        hrt_blas_input_default(&b);
        b.type = in.geometry;
        b.precision = in.precision;
        b.memory = HRT_MEMORY_HOST;
        b.vertices = in.positions.data();
        b.nvertices = in.positions.size() / 3;
        b.radius = in.radius.empty() ? nullptr : in.radius.data();
        b.const_radius = in.constRadius;
        if (!in.strandOffsets.empty()) {
            b.strand_offsets = in.strandOffsets.data();
            b.nstrands = in.strandOffsets.size() - 1;
        }
        if (!in.lineIndices.empty()) {
            b.line_indices = in.lineIndices.data();
            b.nlines = in.lineIndices.size() / 2;
        }
        if (!in.triIndices.empty()) {
            b.tri_indices = in.triIndices.data();
            b.ntris = in.triIndices.size() / 3;
        }
        b.normals = in.normals.empty() ? nullptr : in.normals.data();
        b.voxel_size = in.voxelSize;
        b.width = in.width;
        b.texcoords = in.texCoords.empty() ? nullptr : in.texCoords.data();
        for (int k = 0; k < 4; ++k) b.albedo_factor[k] = in.albedoFactor[k];
        b.albedo_map = in.albedoMap.empty() ? nullptr : in.albedoMap.data();
        b.albedo_map_width = in.albedoMapWidth;
        b.albedo_map_height = in.albedoMapHeight;
        for (int k = 0; k < 16; ++k) b.transform[k] = in.transform[k];
        _transform = in.transform;
        Check(ctx.Get(), hrt_blas_build(ctx.Get(), &b, stream, &_blas), "hrt_blas_build");
    }
    ~BottomLevelAccelerationStructure() { hrt_blas_destroy(_blas); }
    BottomLevelAccelerationStructure(BottomLevelAccelerationStructure&& o) noexcept
        : _ctx(o._ctx), _blas(std::exchange(o._blas, nullptr)), _type(o._type), _transform(o._transform) {}

    // A BLAS from the bytes of Serialize() (hrt_blas_deserialize checks them first).
    static BottomLevelAccelerationStructure Load(Context& ctx, const std::vector<uint8_t>& image,
                                                 void* stream = nullptr) {
        hrt_blas* b = nullptr;
        Check(ctx.Get(), hrt_blas_deserialize(ctx.Get(), image.data(), image.size(), stream, &b),
              "hrt_blas_deserialize");
        return BottomLevelAccelerationStructure(ctx.Get(), b);
    }
    // The BLAS as bytes (host memory), for Load in this or another process.
    std::vector<uint8_t> Serialize() const {
        std::vector<uint8_t> out(hrt_blas_serialized_size(_blas));
        Check(_ctx, hrt_blas_serialize(_blas, out.data(), out.size()), "hrt_blas_serialize");
        return out;
    }
    // New vertex positions (3 floats each) and radii (hair) or normals (mesh) exactly when the
    // build had them; TLASes holding the BLAS must be built again afterwards.
    void Refit(const std::vector<float>& positions, const std::vector<float>& perVertex, void* stream = nullptr) {
        Check(_ctx, hrt_blas_refit(_blas, positions.data(), perVertex.empty() ? nullptr : perVertex.data(),
                                   HRT_MEMORY_HOST, stream), "hrt_blas_refit");
    }
    BottomLevelAccelerationStructure& operator=(BottomLevelAccelerationStructure&&) = delete;
    BottomLevelAccelerationStructure(const BottomLevelAccelerationStructure&) = delete;
    BottomLevelAccelerationStructure& operator=(const BottomLevelAccelerationStructure&) = delete;

    hrt_blas* Structure() const { return _blas; }
    BLASType Type() const { return _type; }
    const std::array<float, 16>& Transform() const { return _transform; }
    hrt_blas_info Info() const {
        hrt_blas_info i;
        hrt_blas_get_info(_blas, &i);
        return i;
    }

private:
    BottomLevelAccelerationStructure(hrt_context* ctx, hrt_blas* b)
        : _ctx(ctx), _blas(b), _type(TypeOf(hrt_geometry_type(hrt_blas_type(b)))) {
        hrt_blas_transform(b, _transform.data());
    }
    hrt_context* _ctx = nullptr;
    hrt_blas* _blas = nullptr;
    BLASType _type;
    std::array<float, 16> _transform;
};

// Instance i of the TLAS is blases[i] with its transform and custom index i
// (top_level_acceleration_structure.cpp:19-113).
class TopLevelAccelerationStructure {
public:
    TopLevelAccelerationStructure(const std::vector<BottomLevelAccelerationStructure>& blases, Context& ctx,
                                  void* stream = nullptr) {
        std::vector<const hrt_blas*> h;
        for (const auto& b : blases) h.push_back(b.Structure());
        Check(ctx.Get(), hrt_tlas_build(ctx.Get(), h.data(), uint32_t(h.size()), stream, &_tlas), "hrt_tlas_build");
    }
    ~TopLevelAccelerationStructure() { hrt_tlas_destroy(_tlas); }
    TopLevelAccelerationStructure(const TopLevelAccelerationStructure&) = delete;
    TopLevelAccelerationStructure& operator=(const TopLevelAccelerationStructure&) = delete;
    TopLevelAccelerationStructure(TopLevelAccelerationStructure&&) = delete;
    TopLevelAccelerationStructure& operator=(TopLevelAccelerationStructure&&) = delete;

    hrt_tlas* Structure() const { return _tlas; }

private:
    hrt_tlas* _tlas = nullptr;
};

// A device framebuffer (RGBA32F) with optional per-sample hit records.
class Frame {
public:
    Frame(Context& ctx, uint32_t width, uint32_t height, uint32_t spp = 1, bool withHits = false)
        : _ctx(ctx.Get()), _w(width), _h(height), _spp(spp) {
        Check(_ctx, hrt_frame_create(_ctx, width, height, spp, withHits ? 1 : 0, &_f), "hrt_frame_create");
    }
    ~Frame() { hrt_frame_destroy(_f); }
    Frame(const Frame&) = delete;
    Frame& operator=(const Frame&) = delete;

    hrt_frame* Get() const { return _f; }
    uint32_t Width() const { return _w; }
    uint32_t Height() const { return _h; }
    // The framebuffer (width * height * 4 floats) and, when given, the hit records.
    std::vector<float> Download(std::vector<hrt_hit>* hits = nullptr, void* stream = nullptr) const {
        std::vector<float> rgba(size_t(_w) * _h * 4);
        if (hits) hits->resize(size_t(_w) * _h * _spp);
        Check(_ctx, hrt_frame_download(_f, rgba.data(), hits ? hits->data() : nullptr, stream), "hrt_frame_download");
        return rgba;
    }
    hrt_frame_stats Stats() const {
        hrt_frame_stats s;
        Check(_ctx, hrt_frame_get_stats(_f, &s), "hrt_frame_get_stats");
        return s;
    }

private:
    hrt_context* _ctx;
    uint32_t _w, _h, _spp;
    hrt_frame* _f = nullptr;
};

inline hrt_trace_params DefaultParams() {
    hrt_trace_params p;
    hrt_trace_params_default(&p);
    return p;
}

inline hrt_camera LookAt(const std::array<float, 3>& eye, const std::array<float, 3>& center,
                         const std::array<float, 3>& up, float fovyDeg, float aspect, float znear = 0.1f,
                         float zfar = 1000.0f) {
    hrt_camera c;
    Check(nullptr, hrt_camera_look_at(eye.data(), center.data(), up.data(), fovyDeg, aspect, znear, zfar, &c),
          "hrt_camera_look_at");
    return c;
}

// Closest hits of explicit rays (6 floats each: origin, direction), the reference's traceRayEXT
// for caller-supplied rays (ray_gen.rgen:34-45).
inline std::vector<hrt_hit> TraceRays(Context& ctx, const TopLevelAccelerationStructure& tlas,
                                      const std::vector<float>& rays, const hrt_trace_params& params,
                                      void* stream = nullptr) {
    std::vector<hrt_hit> hits(rays.size() / 6);
    Check(ctx.Get(), hrt_trace_rays(ctx.Get(), tlas.Structure(), rays.data(), hits.size(), &params, hits.data(),
                                    HRT_MEMORY_HOST, stream), "hrt_trace_rays");
    return hits;
}

// One frame: the reference's Renderer::Render for the hair path.
inline void Render(Context& ctx, const TopLevelAccelerationStructure& tlas, const hrt_camera& cam,
                   const hrt_trace_params& params, Frame& frame, void* stream = nullptr) {
    Check(ctx.Get(), hrt_trace(ctx.Get(), tlas.Structure(), &cam, &params, frame.Get(), stream), "hrt_trace");
}

// Many scenes rendered by one replay of a captured CUDA graph: each scene is a TLAS, a camera
// and the frame it renders into (its size and samples). The TLASes and frames must outlive the
// batch. SetCameras moves the cameras without recapturing; Download reads every framebuffer.
class Batch {
public:
    struct Scene {
        const TopLevelAccelerationStructure* tlas;
        hrt_camera camera;
        Frame* frame;
    };
    Batch(Context& ctx, const std::vector<Scene>& scenes, const hrt_trace_params& params, void* stream = nullptr)
        : _ctx(ctx.Get()) {
        std::vector<hrt_scene_desc> d;
        for (const Scene& s : scenes) {
            d.push_back(hrt_scene_desc{s.tlas->Structure(), s.camera, s.frame->Get()});
            _frames.push_back(s.frame);
        }
        Check(_ctx, hrt_batch_create(_ctx, d.data(), uint32_t(d.size()), &params, stream, &_b), "hrt_batch_create");
    }
    ~Batch() { hrt_batch_destroy(_b); }
    Batch(const Batch&) = delete;
    Batch& operator=(const Batch&) = delete;

    void Launch(void* stream = nullptr) { Check(_ctx, hrt_batch_launch(_b, stream), "hrt_batch_launch"); }
    void SetCameras(const std::vector<hrt_camera>& cams, void* stream = nullptr) {
        Check(_ctx, hrt_batch_set_cameras(_b, cams.data(), uint32_t(cams.size()), stream), "hrt_batch_set_cameras");
    }
    // Every scene's framebuffer (width * height * 4 floats each), in creation order; waits for
    // the copies.
    std::vector<std::vector<float>> Download(void* stream = nullptr) {
        std::vector<std::vector<float>> out(_frames.size());
        std::vector<float*> dst(_frames.size());
        for (size_t i = 0; i < _frames.size(); ++i) {
            out[i].resize(size_t(_frames[i]->Width()) * _frames[i]->Height() * 4);
            dst[i] = out[i].data();
        }
        Check(_ctx, hrt_batch_download(_b, dst.data(), stream, 1), "hrt_batch_download");
        return out;
    }

private:
    hrt_context* _ctx;
    hrt_batch* _b = nullptr;
    std::vector<Frame*> _frames;
};

}  // namespace hrt

#endif  // HRT_HPP
