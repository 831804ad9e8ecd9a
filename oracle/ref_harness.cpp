// oracle/ref_harness.cpp -- TEST INFRASTRUCTURE: the reference's own code, compiled as host
// C++ by oracle/build_ref.sh into oracle/_ref/libhrtref.so. Only the tests and the golden
// fixture generator load it; it pins the oracle restatement (oracle/hrt_oracle.cpp).
//
// Everything included below comes from the reference checkout (via oracle/_ref/, produced by
// build_ref.sh); this file only provides the GLSL/glm vocabulary and C entry points.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "glsl_shim.hpp"

// GLSL `out` parameters become C++ references.
#define out outref::

namespace ref32 {
SHIM_GLSL_VOCABULARY(float)
namespace outref { using vec3 = ::shim::tvec3<float>&; }
static thread_local vec3 attribNormal;  // hitAttributeEXT written by Prhi
#include "glsl32/ray.glsl"
#include "glsl32/curve.glsl"
#include "glsl32/cone.glsl"
#include "glsl32/cylinder.glsl"
#include "glsl32/shading.glsl"
#include "glsl32/prhi.inc"
struct CameraProperties { mat4 viewInverse; mat4 projInverse; };
static void RayGen(uvec3 gl_LaunchIDEXT, uvec3 gl_LaunchSizeEXT, const CameraProperties& cam,
                   vec3& o, vec3& dir) {
#include "glsl32/raygen_body.inc"
    o = origin.xyz;
    dir = direction.xyz;
}
}  // namespace ref32

namespace ref64 {
SHIM_GLSL_VOCABULARY(double)
namespace outref { using vec3 = ::shim::tvec3<double>&; }
#define float double
static thread_local vec3 attribNormal;
#include "glsl64/ray.glsl"
#include "glsl64/curve.glsl"
#include "glsl64/cone.glsl"
#include "glsl64/cylinder.glsl"
#include "glsl64/shading.glsl"
#include "glsl64/prhi.inc"
#undef float
}  // namespace ref64

#undef out

// ---- host geometry processing, glm stand-in ---------------------------------------------
namespace refgeo {
namespace glm {
using vec3 = ::shim::tvec3<float>;
using vec2 = ::shim::tvec2<float>;
inline vec3 normalize(vec3 v) { return ::shim::normalize(v); }
inline vec3 cross(vec3 a, vec3 b) { return ::shim::cross(a, b); }
inline vec3 min(vec3 a, vec3 b) { return ::shim::vmin(a, b); }
inline vec3 max(vec3 a, vec3 b) { return ::shim::vmax(a, b); }
inline float max(float a, float b) { return ::shim::gmax(a, b); }
inline vec3 abs(vec3 a) { return ::shim::vabs(a); }
}  // namespace glm
using glm::abs;
using glm::cross;
struct Line { glm::vec3 start{}; glm::vec3 end{}; };
struct alignas(16) Curve { glm::vec3 start{}; glm::vec3 controlPoint1{}; glm::vec3 controlPoint2{}; glm::vec3 end{}; };
struct alignas(16) AABB { glm::vec3 min{}; glm::vec3 max{}; };
struct Mesh {
    struct Vertex { glm::vec3 position{}; glm::vec3 normal{}; glm::vec2 texCoord{}; };
    uint32_t indexCount{};
    uint32_t firstIndex{};
    uint32_t firstVertex{};
};
struct LSSMesh { uint32_t vertexCount{}; uint32_t firstVertex{}; };
#include "geometry_fns.inc"
}  // namespace refgeo

namespace {
template <class V> V v3(const float* p) { return V(p[0], p[1], p[2]); }
template <class V> void put3(float* p, const V& v) { p[0] = float(v.x); p[1] = float(v.y); p[2] = float(v.z); }
}  // namespace

extern "C" {

// Prhi on one (ray, curve) pair. ray = origin[3], direction[3]; curve = 4 x xyz.
// Returns the reported distance (0 = no report) and writes attribNormal.
float ref_prhi_f32(const float* ray, const float* curve, float* normal_out) {
    ref32::Ray r;
    r.origin = v3<ref32::vec3>(ray);
    r.direction = v3<ref32::vec3>(ray + 3);
    ref32::Curve c;
    c.start = v3<ref32::vec3>(curve);
    c.controlPoint1 = v3<ref32::vec3>(curve + 3);
    c.controlPoint2 = v3<ref32::vec3>(curve + 6);
    c.end = v3<ref32::vec3>(curve + 9);
    ref32::attribNormal = ref32::vec3(0.f, 0.f, 0.f);
    float t = ref32::Prhi(r, c);
    put3(normal_out, ref32::attribNormal);
    return t;
}

double ref_prhi_f64(const double* ray, const double* curve, double* normal_out) {
    ref64::Ray r;
    r.origin = ref64::vec3(ray[0], ray[1], ray[2]);
    r.direction = ref64::vec3(ray[3], ray[4], ray[5]);
    ref64::Curve c;
    c.start = ref64::vec3(curve[0], curve[1], curve[2]);
    c.controlPoint1 = ref64::vec3(curve[3], curve[4], curve[5]);
    c.controlPoint2 = ref64::vec3(curve[6], curve[7], curve[8]);
    c.end = ref64::vec3(curve[9], curve[10], curve[11]);
    ref64::attribNormal = ref64::vec3(0.0, 0.0, 0.0);
    double t = ref64::Prhi(r, c);
    normal_out[0] = ref64::attribNormal.x;
    normal_out[1] = ref64::attribNormal.y;
    normal_out[2] = ref64::attribNormal.z;
    return t;
}

// cone.glsl RayConeIntersectRCC; cone = center[3], radius, axis[3], slant.
// out = {isIntersection, s, dt, dp, dc, sp}
void ref_cone_f32(const float* cone, float* out6) {
    ref32::Cone c;
    c.center = v3<ref32::vec3>(cone);
    c.radius = cone[3];
    c.axis = v3<ref32::vec3>(cone + 4);
    c.slant = cone[7];
    ref32::RayConeIntersection r = ref32::RayConeIntersectRCC(c);
    out6[0] = r.isIntersection ? 1.f : 0.f;
    out6[1] = r.s; out6[2] = r.dt; out6[3] = r.dp; out6[4] = r.dc; out6[5] = r.sp;
}

// cylinder.glsl RayCylinderIntersect; ray[6], cyl = p0[3], p1[3], radius.
int ref_cylinder_f32(const float* ray, const float* cyl) {
    ref32::Ray r;
    r.origin = v3<ref32::vec3>(ray);
    r.direction = v3<ref32::vec3>(ray + 3);
    ref32::Cylinder c;
    c.p0 = v3<ref32::vec3>(cyl);
    c.p1 = v3<ref32::vec3>(cyl + 3);
    c.radius = cyl[6];
    return ref32::RayCylinderIntersect(r, c) ? 1 : 0;
}

// curve.glsl SampleCurvePoint / SampleCurveAxis; out = point[3], axis[3]
void ref_curve_sample_f32(const float* curve, float t, float* out6) {
    ref32::Curve c;
    c.start = v3<ref32::vec3>(curve);
    c.controlPoint1 = v3<ref32::vec3>(curve + 3);
    c.controlPoint2 = v3<ref32::vec3>(curve + 6);
    c.end = v3<ref32::vec3>(curve + 9);
    put3(out6, ref32::SampleCurvePoint(c, t));
    put3(out6 + 3, ref32::SampleCurveAxis(c, t));
}

// ray.glsl CreateRCCMatrix (column major 16 floats)
void ref_rcc_matrix_f32(const float* ray, float* m16) {
    ref32::Ray r;
    r.origin = v3<ref32::vec3>(ray);
    r.direction = v3<ref32::vec3>(ray + 3);
    ref32::mat4 m = ref32::CreateRCCMatrix(r);
    for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) m16[c * 4 + k] = m[c][k];
}

// shading.glsl Shade
void ref_shade_f32(const float* n, float* rgb) { put3(rgb, ref32::Shade(v3<ref32::vec3>(n))); }

// ray_gen.rgen:18-24 for one launch id; view_inv/proj_inv column major.
void ref_raygen_f32(const float* view_inv, const float* proj_inv, uint32_t px, uint32_t py,
                    uint32_t w, uint32_t h, float* o3, float* d3) {
    ref32::CameraProperties cam;
    for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) {
            cam.viewInverse[c][k] = view_inv[c * 4 + k];
            cam.projInverse[c][k] = proj_inv[c * 4 + k];
        }
    shim::uvec3 id;
    id.x = px; id.y = py; id.z = 0;
    shim::uvec3 size;
    size.x = w; size.y = h; size.z = 1;
    ref32::vec3 o, d;
    ref32::RayGen(id, size, cam, o, d);
    put3(o3, o);
    put3(d3, d);
}

// GenerateCurves over n lines (each start[3], end[3]) -> n curves (4 x xyz).
void ref_generate_curves(const float* lines, int64_t n, float* curves_out) {
    std::vector<refgeo::Line> ls(n);
    for (int64_t i = 0; i < n; ++i) {
        ls[i].start = v3<refgeo::glm::vec3>(lines + 6 * i);
        ls[i].end = v3<refgeo::glm::vec3>(lines + 6 * i + 3);
    }
    std::vector<refgeo::Curve> cs = refgeo::GenerateCurves(ls);
    for (int64_t i = 0; i < n; ++i) {
        put3(curves_out + 12 * i, cs[i].start);
        put3(curves_out + 12 * i + 3, cs[i].controlPoint1);
        put3(curves_out + 12 * i + 6, cs[i].controlPoint2);
        put3(curves_out + 12 * i + 9, cs[i].end);
    }
}

// GenerateAABBs(curves, r) -> n x (min[3], max[3])
void ref_generate_aabbs(const float* curves, int64_t n, float radius, float* aabbs_out) {
    std::vector<refgeo::Curve> cs(n);
    for (int64_t i = 0; i < n; ++i) {
        cs[i].start = v3<refgeo::glm::vec3>(curves + 12 * i);
        cs[i].controlPoint1 = v3<refgeo::glm::vec3>(curves + 12 * i + 3);
        cs[i].controlPoint2 = v3<refgeo::glm::vec3>(curves + 12 * i + 6);
        cs[i].end = v3<refgeo::glm::vec3>(curves + 12 * i + 9);
    }
    std::vector<refgeo::AABB> bs = refgeo::GenerateAABBs(cs, radius);
    for (int64_t i = 0; i < n; ++i) {
        put3(aabbs_out + 6 * i, bs[i].min);
        put3(aabbs_out + 6 * i + 3, bs[i].max);
    }
}

// GenerateDisjointOrthogonalTriangleStrips -> 12 n vertex positions and 12 n indices
void ref_generate_dots(const float* lines, int64_t n, float radius, float* pos_out, uint32_t* idx_out) {
    std::vector<refgeo::Line> ls(n);
    for (int64_t i = 0; i < n; ++i) {
        ls[i].start = v3<refgeo::glm::vec3>(lines + 6 * i);
        ls[i].end = v3<refgeo::glm::vec3>(lines + 6 * i + 3);
    }
    std::vector<refgeo::Mesh::Vertex> vb;
    std::vector<uint32_t> ib;
    refgeo::GenerateDisjointOrthogonalTriangleStrips(ls, vb, ib, radius);
    for (size_t i = 0; i < vb.size(); ++i) put3(pos_out + 3 * i, vb[i].position);
    std::memcpy(idx_out, ib.data(), ib.size() * sizeof(uint32_t));
}

// GenerateLinearSweptSpheres -> 2n positions and 2n radii
void ref_generate_lss(const float* lines, int64_t n, float radius, float* pos_out, float* rad_out) {
    std::vector<refgeo::Line> ls(n);
    for (int64_t i = 0; i < n; ++i) {
        ls[i].start = v3<refgeo::glm::vec3>(lines + 6 * i);
        ls[i].end = v3<refgeo::glm::vec3>(lines + 6 * i + 3);
    }
    std::vector<refgeo::glm::vec3> pb;
    std::vector<float> rb;
    refgeo::GenerateLinearSweptSpheres(ls, pb, rb, radius);
    for (size_t i = 0; i < pb.size(); ++i) put3(pos_out + 3 * i, pb[i]);
    std::memcpy(rad_out, rb.data(), rb.size() * sizeof(float));
}

}  // extern "C"
