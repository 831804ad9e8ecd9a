// oracle/hrt_oracle.cpp -- TEST INFRASTRUCTURE: the CPU oracle for the hair ray-tracing path.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this library
// (oracle/_build/libhrtoracle.so); the product never links it.
//
// It restates, in FP32 and FP64 (templated on the scalar), every stage of the reference's
// hair path plus the stages the reference delegates to the Vulkan driver:
//   * shader math: curve.glsl:9-47, cone.glsl:21-62, cylinder.glsl:8-46, ray.glsl:13-33,
//     shading.glsl:1-10, debug.glsl:1-7, Prhi hair_intersection.rint:15-130,
//     ray generation ray_gen.rgen:18-32;
//   * host geometry processing: GenerateCurves geometry_processor.cpp:123-156,
//     GenerateAABBs :422-436, PerpStark/BuildFrame :201-219, DOTS :221-271, LSS :273-298;
//   * what the driver and RT cores do (no reference source; defined by this project):
//     the LBVH build (63-bit Morton codes, stable sort, Karras hierarchy, refit), the
//     collapse to an 8-wide BVH and its 8-bit quantisation, linear-swept-sphere and
//     watertight triangle intersection, closest-hit traversal, and the shadow ray.
// The FP32 instantiation of the shader math is checked bit for bit against the reference's
// own code compiled through the same shim (oracle/_ref, built by oracle/build_ref.sh).
// Compile with -ffp-contract=off: no multiply-add may be fused.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "glsl_shim.hpp"

namespace orc {
using shim::tvec3;
using shim::tvec4;
using shim::tmat4;
using shim::gmin;
using shim::gmax;
using shim::gabs;

template <class T> struct Ray { tvec3<T> origin, direction; };
template <class T> struct Curve { tvec3<T> start, cp1, cp2, end; };
template <class T> struct Cylinder { tvec3<T> p0, p1; T radius; };
template <class T> struct Cone { tvec3<T> center; T radius; tvec3<T> axis; T slant; };
template <class T> struct ConeHit { bool isIntersection; T s, dt, dp, dc, sp; };

// ---- curve.glsl ---------------------------------------------------------------------------
// SampleCurvePoint curve.glsl:9-21
template <class T> tvec3<T> sample_point(const Curve<T>& c, T t) {
    T u = T(1) - t;
    T tt = t * t;
    T uu = u * u;
    T uuu = uu * u;
    T ttt = tt * t;
    return uuu * c.start + T(3) * uu * t * c.cp1 + T(3) * u * tt * c.cp2 + ttt * c.end;
}
// SampleCurveAxis curve.glsl:23-31
template <class T> tvec3<T> sample_axis(const Curve<T>& c, T t) {
    T u = T(1) - t;
    return T(-3) * u * u * c.start + T(3) * (T(3) * t * t - T(4) * t + T(1)) * c.cp1 +
           T(3) * (T(2) - T(3) * t) * t * c.cp2 + T(3) * t * t * c.end;
}
// TransformCurve curve.glsl:33-42
template <class T> Curve<T> transform_curve(const Curve<T>& c, const tmat4<T>& m) {
    Curve<T> r;
    r.start = (m * tvec4<T>(c.start, T(1))).xyz;
    r.cp1 = (m * tvec4<T>(c.cp1, T(1))).xyz;
    r.cp2 = (m * tvec4<T>(c.cp2, T(1))).xyz;
    r.end = (m * tvec4<T>(c.end, T(1))).xyz;
    return r;
}
// CurveDistanceToCylinder curve.glsl:44-47
template <class T> T curve_distance_to_cylinder(const Curve<T>& c, tvec3<T> p) {
    return shim::length(shim::cross(p - c.start, p - c.end)) / shim::length(c.end - c.start);
}

// ---- cylinder.glsl:8-46 -------------------------------------------------------------------
template <class T> bool ray_cylinder(const Ray<T>& ray, const Cylinder<T>& cyl) {
    tvec3<T> ba = cyl.p1 - cyl.p0;
    tvec3<T> oc = ray.origin - cyl.p0;
    T baba = shim::dot(ba, ba);
    T bard = shim::dot(ba, ray.direction);
    T baoc = shim::dot(ba, oc);
    T k2 = baba - bard * bard;
    T k1 = baba * shim::dot(oc, ray.direction) - baoc * bard;
    T k0 = baba * shim::dot(oc, oc) - baoc * baoc - cyl.radius * cyl.radius * baba;
    T h = k1 * k1 - k2 * k0;
    if (h < T(0)) return false;
    h = std::sqrt(h);
    T t = (-k1 - h) / k2;
    T y = baoc + t * bard;
    if (y > T(0) && y < baba) return true;
    t = ((y < T(0) ? T(0) : baba) - baoc) / bard;
    if (gabs(k1 + k2 * t) < h) return true;
    return false;
}

// ---- cone.glsl:21-62 (RayConeIntersectRCC, ray-centric coordinates) -----------------------
template <class T> ConeHit<T> ray_cone_rcc(const Cone<T>& cone) {
    T r2 = cone.radius * cone.radius;
    T drr = cone.radius * cone.slant;
    T ddd = cone.axis.x * cone.axis.x + cone.axis.y * cone.axis.y;
    T dp = cone.center.x * cone.center.x + cone.center.y * cone.center.y;
    T cdd = cone.center.x * cone.axis.x + cone.center.y * cone.axis.y;
    T cxd = cone.center.x * cone.axis.y - cone.center.y * cone.axis.x;
    T c = ddd;
    T b = cone.axis.z * (drr - cdd);
    T cdz2 = cone.axis.z * cone.axis.z;
    ddd += cdz2;
    T a = T(2) * drr * cdd + cxd * cxd - ddd * r2 + dp * cdz2;
    T det = b * b - a * c;
    ConeHit<T> r;
    r.isIntersection = det > T(0);
    r.s = (b - (r.isIntersection ? std::sqrt(det) : T(0))) / c;
    r.dt = (r.s * cone.axis.z - cdd) / ddd;
    r.dc = r.s * r.s + dp;
    r.sp = cdd / cone.axis.z;
    r.dp = dp + r.sp * r.sp;
    return r;
}

// ---- ray.glsl:13-33 -----------------------------------------------------------------------
template <class T> void orthonormal_basis(tvec3<T>& u, tvec3<T>& v, tvec3<T> w) {
    v = gabs(w.x) > gabs(w.y) ? shim::normalize(tvec3<T>(-w.z, T(0), w.x))
                              : shim::normalize(tvec3<T>(T(0), w.z, -w.y));
    u = shim::cross(v, w);
}
template <class T> tmat4<T> rcc_matrix(const Ray<T>& ray) {
    tvec3<T> e1, e2, e3 = shim::normalize(ray.direction);
    orthonormal_basis(e1, e2, e3);
    tmat4<T> m(tvec4<T>(e1, T(0)), tvec4<T>(e2, T(0)), tvec4<T>(e3, T(0)), tvec4<T>(ray.origin, T(1)));
    return shim::inverse(m);
}

// ---- shading.glsl:1-10, debug.glsl:1-7 ----------------------------------------------------
template <class T> tvec3<T> shade(tvec3<T> n) {
    tvec3<T> lightColor(T(0.4f), T(0.2f), T(0.1f));
    tvec3<T> lightDirection(T(0), T(-1), T(0));
    tvec3<T> ambient(T(0.3f), T(0.3f), T(0.3f));
    tvec3<T> color = gabs(shim::dot(n, lightDirection)) * lightColor;
    color += ambient;
    return color;
}
static const float kPalette[6][3] = {{1.0f, 0.0f, 0.3f}, {0.8f, 0.2f, 0.3f}, {0.6f, 0.4f, 0.3f},
                                     {0.4f, 0.6f, 0.3f}, {0.2f, 0.8f, 0.3f}, {0.0f, 1.0f, 0.3f}};

// ---- Prhi hair_intersection.rint:15-130 ---------------------------------------------------
// Radius: the reference hard-codes 0.02 (hair_intersection.rint:18). Here the cone radius is
// r0 + (r1 - r0) t along the segment (taper), which is exactly the constant when r0 == r1;
// the bounding-cylinder pad is max(r0, r1).
// status: 0 miss, 1 hit, 2 unresolved (a side used all 8 iterations inside [0,1]), 3 unresolved
// with a real cone intersection at the last step of such a side (the run had not converged).
// shift: evaluate from the ray point nearest the chord midpoint instead of the ray origin
// (the bounding-cylinder test is on the infinite line and the cone step is translation
// invariant along the ray, so the result is the same in exact arithmetic; in FP32 this removes
// the cancellation of the world-space test, hair_intersection.rint:29). The reference-literal
// form is shift = false.
enum { kMiss = 0, kHit = 1, kUnresolved = 2, kUnresolvedNear = 3 };
template <class T>
T prhi(const Ray<T>& ray_in, const Curve<T>& curve, T r0, T r1, tvec3<T>* normal, int* status, bool shift = false,
       bool polish = false) {
    T result = T(0);
    *status = kMiss;
    Ray<T> ray = ray_in;
    T tshift = T(0);
    Curve<T> local = curve;  // the curve in the coordinates the solve runs in
    if (shift) {
        // o' = o + tshift d is never rounded: each P - o' is P - o exactly (TwoSum) minus
        // tshift d in one fused operation, so the relative vectors keep full precision.
        tvec3<T> mid = (curve.start + curve.end) * T(0.5);
        tshift = shim::dot(mid - ray_in.origin, ray_in.direction) / shim::dot(ray_in.direction, ray_in.direction);
        auto rel = [&](const tvec3<T>& p) {
            tvec3<T> r;
            for (int k = 0; k < 3; ++k) {
                T a = p[k], c = -ray_in.origin[k];
                T sum = a + c, cc = sum - a, err = (a - (sum - cc)) + (c - cc);
                r[k] = std::fma(-tshift, ray_in.direction[k], sum) + err;
            }
            return r;
        };
        local = Curve<T>{rel(curve.start), rel(curve.cp1), rel(curve.cp2), rel(curve.end)};
        ray.origin = tvec3<T>(T(0), T(0), T(0));
    }
    T rmax = curve_distance_to_cylinder(curve, sample_point(curve, T(0.5)));
    rmax += gmax(r0, r1);
    Cylinder<T> cyl{local.start, local.end, rmax};
    if (!ray_cylinder(ray, cyl)) return result;
    tmat4<T> rcc = rcc_matrix(ray);
    Curve<T> rc = transform_curve(local, rcc);
    const tvec3<T> rayDirection(T(0), T(0), T(1));
    tvec3<T> curveDirection = shim::normalize(rc.end - rc.start);
    T tStart = shim::dot(curveDirection, rayDirection) > T(0) ? T(0) : T(1);
    bool exhausted_any = false, exhausted_isect = false;
    for (uint32_t side = 0; side < 2; ++side) {
        const uint32_t maxIterations = 8;
        T t = tStart;
        T told = T(0), dt1 = T(0), dt2 = T(0);
        bool exhausted = true, last_isect = false;
        for (uint32_t i = 0; i < maxIterations; ++i) {
            Cone<T> cone;
            cone.center = sample_point(rc, t);
            cone.radius = (r0 == r1) ? r0 : r0 + (r1 - r0) * t;
            cone.axis = sample_axis(rc, t);
            cone.slant = T(0);
            ConeHit<T> rci = ray_cone_rcc(cone);
            last_isect = rci.isIntersection;
            if (rci.isIntersection && gabs(rci.dt) < T(5e-5)) {
                if (polish) {  // one more cone step from the converged parameter
                    T tp = t + rci.dt;
                    if (tp >= T(0) && tp <= T(1)) {
                        Cone<T> c2;
                        c2.center = sample_point(rc, tp);
                        c2.radius = (r0 == r1) ? r0 : r0 + (r1 - r0) * tp;
                        c2.axis = sample_axis(rc, tp);
                        c2.slant = T(0);
                        ConeHit<T> r2 = ray_cone_rcc(c2);
                        if (r2.isIntersection) { t = tp; rci = r2; cone = c2; }
                    }
                }
                rci.s += cone.center.z;
                result = rci.s + tshift;
                tvec3<T> hitPosition = ray_in.origin + result * ray_in.direction;
                tvec3<T> curvePosition = sample_point(curve, t);
                if (normal) *normal = shim::normalize(hitPosition - curvePosition);
                exhausted = false;
                break;
            }
            rci.dt = gmin(rci.dt, T(0.5));
            rci.dt = gmax(rci.dt, T(-0.5));
            dt1 = dt2;
            dt2 = rci.dt;
            if (dt1 * dt2 < T(0)) {
                T tnext;
                if ((i & 3) == 0) tnext = T(0.5) * (told + t);
                else tnext = (dt2 * told - dt1 * t) / (dt2 - dt1);
                told = t;
                t = tnext;
            } else {
                told = t;
                t += rci.dt;
            }
            if (t < T(0) || t > T(1)) { exhausted = false; break; }
        }
        exhausted_any |= exhausted;
        exhausted_isect |= exhausted && last_isect;
        if (result > T(0)) break;
        tStart = T(1) - tStart;
    }
    *status = result > T(0) ? kHit : (exhausted_isect ? kUnresolvedNear : (exhausted_any ? kUnresolved : kMiss));
    return result;
}

// ---- linear swept sphere (round cone between spheres (a, ra) and (b, rb)) ----------------
// Not in the reference's source: VK_NV_ray_tracing_linear_swept_spheres intersects in
// hardware (renderer.cpp:664-678, eList indexing). The surface is the envelope of the spheres
// centred on a + u (b - a) with radius ra + u (rb - ra), u in [0,1], both end caps on.
// Points on the tangent cone satisfy m |P-a|^2 - (y + ra dr)^2 - m ra^2 = 0 with
// y = (b-a).(P-a), dr = rb - ra, m = |b-a|^2 - dr^2, and envelope parameter
// u = (y + ra dr) / m. The first crossing is the least t >= tmin over the cone roots with
// u in [0,1] and the two sphere roots. Returns t (or -1) and u.
template <class T> T sphere_roots(tvec3<T> o, tvec3<T> d, tvec3<T> c, T r, T tmin, T best) {
    tvec3<T> oc = o - c;
    T A = shim::dot(d, d);
    T B = shim::dot(oc, d);
    tvec3<T> cx = shim::cross(oc, d);
    T h = r * r * A - shim::dot(cx, cx);  // = B^2 - A (|oc|^2 - r^2) by Lagrange's identity
    if (h < T(0)) return best;
    T sh = std::sqrt(h);
    T t0 = (-B - sh) / A;
    T t1 = (-B + sh) / A;
    if (t0 >= tmin && t0 < best) return t0;
    if (t1 >= tmin && t1 < best) return t1;
    return best;
}
// Solved from the ray point nearest the segment midpoint (t = tshift + t'), so the quadratic's
// terms are of the segment's size rather than the camera distance.
template <class T>
T lss_intersect(tvec3<T> o_in, tvec3<T> d, tvec3<T> a, tvec3<T> b, T ra, T rb, T tmin_in, T* u_out) {
    const T kNone = T(INFINITY);
    T tshift = shim::dot((a + b) * T(0.5) - o_in, d) / shim::dot(d, d);
    tvec3<T> o = o_in + tshift * d;
    T tmin = tmin_in - tshift;
    T best = kNone, bu = T(0);
    tvec3<T> ba = b - a;
    tvec3<T> oa = o - a;
    T L2 = shim::dot(ba, ba);
    T dr = rb - ra;
    T m = L2 - dr * dr;
    if (m > T(0)) {
        // coefficients through c1 = ba x oa, c2 = ba x d (Lagrange's identity), free of the
        // cancellation of m |oa|^2 - yo^2
        tvec3<T> c1 = shim::cross(ba, oa), c2 = shim::cross(ba, d);
        T yd = shim::dot(ba, d);
        T ybo = shim::dot(ba, oa);
        T yo = ybo + ra * dr;
        T A = shim::dot(c2, c2) - dr * dr * shim::dot(d, d);
        T B = shim::dot(c1, c2) - dr * dr * shim::dot(oa, d) - ra * dr * yd;
        T C = shim::dot(c1, c1) - dr * dr * shim::dot(oa, oa) - T(2) * ra * dr * ybo - ra * ra * L2;
        T h = B * B - A * C;
        if (h >= T(0) && A != T(0)) {
            T sh = std::sqrt(h);
            T r0 = (-B - sh) / A, r1 = (-B + sh) / A;
            T lo = gmin(r0, r1), hi = gmax(r0, r1);
            for (T tc : {lo, hi}) {
                if (!(tc >= tmin) || !(tc < best)) continue;
                T u = (yo + tc * yd) / m;
                if (u >= T(0) && u <= T(1)) { best = tc; bu = u; break; }
            }
        }
    }
    T ta = sphere_roots(o, d, a, ra, tmin, best);
    if (ta < best) { best = ta; bu = T(0); }
    T tb = sphere_roots(o, d, b, rb, tmin, best);
    if (tb < best) { best = tb; bu = T(1); }
    if (best == kNone) return T(-1);
    *u_out = bu;
    return best + tshift;
}

// ---- watertight ray/triangle (Woop, Benthin and Wald, JCGT 2013) --------------------------
// Not in the reference's source: DOTS triangles are intersected by RT hardware with facing
// culling disabled (top_level_acceleration_structure.cpp:28). Returns t or -1.
template <class T>
T tri_intersect(tvec3<T> o, tvec3<T> d, tvec3<T> v0, tvec3<T> v1, tvec3<T> v2, T tmin, T tmax, T* b1 = nullptr,
                T* b2 = nullptr) {
    int kz = 0;
    T ax = gabs(d.x), ay = gabs(d.y), az = gabs(d.z);
    if (ay > ax && ay >= az) kz = 1;
    else if (az > ax && az > ay) kz = 2;
    int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
    if (d[kz] < T(0)) std::swap(kx, ky);
    T Sx = d[kx] / d[kz], Sy = d[ky] / d[kz], Sz = T(1) / d[kz];
    tvec3<T> A = v0 - o, B = v1 - o, C = v2 - o;
    T Ax = A[kx] - Sx * A[kz], Ay = A[ky] - Sy * A[kz];
    T Bx = B[kx] - Sx * B[kz], By = B[ky] - Sy * B[kz];
    T Cx = C[kx] - Sx * C[kz], Cy = C[ky] - Sy * C[kz];
    T U = Cx * By - Cy * Bx;
    T V = Ax * Cy - Ay * Cx;
    T W = Bx * Ay - By * Ax;
    if ((U < T(0) || V < T(0) || W < T(0)) && (U > T(0) || V > T(0) || W > T(0))) return T(-1);
    T det = U + V + W;
    if (det == T(0)) return T(-1);
    T Az = Sz * A[kz], Bz = Sz * B[kz], Cz = Sz * C[kz];
    T Tn = U * Az + V * Bz + W * Cz;
    T t = Tn / det;
    if (!(t >= tmin) || !(t <= tmax)) return T(-1);
    if (b1) { *b1 = V / det; *b2 = W / det; }  // barycentric weights of v1 and v2
    return t;
}

// ---- host geometry processing (FP32, reference op order) ----------------------------------
using v3f = tvec3<float>;
static v3f ld3(const float* p) { return v3f(p[0], p[1], p[2]); }
static void st3(float* p, v3f v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }

// GenerateCurves geometry_processor.cpp:123-156 (tension 1): neighbouring lines are detected
// by exact equality of end and start points; strand ends reuse the line itself.
static void generate_curves(const float* lines, int64_t n, float* out) {
    if (n <= 0) return;
    auto L = [&](int64_t k, int e) {  // k indexes the padded list [first, lines..., last]
        int64_t j = k == 0 ? 0 : (k == n + 1 ? n - 1 : k - 1);
        return ld3(lines + 6 * j + 3 * e);
    };
    const float tension = 1.0f;
    for (int64_t i = 1; i <= n; ++i) {
        int64_t prev = L(i - 1, 1) == L(i, 0) ? i - 1 : i;
        int64_t next = L(i, 1) == L(i + 1, 0) ? i + 1 : i;
        v3f p0 = L(prev, 0), p1 = L(i, 0), p2 = L(i, 1), p3 = L(next, 1);
        float* c = out + 12 * (i - 1);
        st3(c, p1);
        st3(c + 3, p1 + (p2 - p0) * (tension / 6.0f));
        st3(c + 6, p2 - (p3 - p1) * (tension / 6.0f));
        st3(c + 9, p2);
    }
}

// PerpStark / BuildFrame geometry_processor.cpp:201-219
static v3f perp_stark(v3f u) {
    v3f a = shim::vabs(u);
    uint32_t uyx = (a.x - a.y) < 0 ? 1 : 0;
    uint32_t uzx = (a.x - a.z) < 0 ? 1 : 0;
    uint32_t uzy = (a.y - a.z) < 0 ? 1 : 0;
    uint32_t xm = uyx & uzx;
    uint32_t ym = (1 ^ xm) & uzy;
    uint32_t zm = 1 ^ (xm | ym);
    return shim::normalize(shim::cross(u, v3f(float(xm), float(ym), float(zm))));
}

// DOTS geometry_processor.cpp:221-271 with per-end radii (the reference passes one radius,
// 0.02, :681; r0 == r1 reproduces it exactly). 12 vertices per line, triangle k of line i is
// vertices 12 i + 3 k .. + 2, i.e. primitive id 4 i + k.
static void generate_dots(const float* lines, const float* radii, float const_r, int64_t n, float* out) {
    for (int64_t i = 0; i < n; ++i) {
        v3f s0 = ld3(lines + 6 * i), e0 = ld3(lines + 6 * i + 3);
        float ra = radii ? radii[2 * i] : const_r, rb = radii ? radii[2 * i + 1] : const_r;
        v3f fwd = shim::normalize(e0 - s0);
        v3f s = perp_stark(fwd);
        v3f t = shim::cross(fwd, s);
        v3f v[2] = {s, t};
        for (int face = 0; face < 2; ++face) {
            float* o = out + 36 * i + 18 * face;
            st3(o + 0, s0 + v[face] * ra);
            st3(o + 3, e0 - v[face] * rb);
            st3(o + 6, e0 + v[face] * rb);
            st3(o + 9, s0 + v[face] * ra);
            st3(o + 12, s0 - v[face] * ra);
            st3(o + 15, e0 - v[face] * rb);
        }
    }
}

// ---- deterministic FP32 helpers shared by the BVH pipeline --------------------------------
struct Box { float lo[3], hi[3]; };
static inline float fmin_t(float a, float b) { return (b < a) ? b : a; }  // glm min order
static inline float fmax_t(float a, float b) { return (a < b) ? b : a; }

// BVH primitive boxes (one primitive = one strand segment).
//   Phantom: control hull +- max(r0, r1)  (GenerateAABBs geometry_processor.cpp:431-432)
//   LSS:     min/max of (p0 -+ r0, p1 -+ r1)
//   DOTS:    min/max over the segment's 12 vertices, in vertex order
//   mesh:    min/max over the triangle's 3 vertices, in vertex order
enum { kPhantom = 0, kLss = 1, kDots = 2, kMesh = 3, kVoxel = 4 };
static Box prim_box(int type, const float* data, const float* radius, int64_t i) {
    Box b;
    if (type == kPhantom) {
        const float* c = data + 12 * i;
        float r = fmax_t(radius[2 * i], radius[2 * i + 1]);
        for (int k = 0; k < 3; ++k) {
            b.lo[k] = fmin_t(fmin_t(c[k], c[9 + k]), fmin_t(c[3 + k], c[6 + k])) - r;
            b.hi[k] = fmax_t(fmax_t(c[k], c[9 + k]), fmax_t(c[3 + k], c[6 + k])) + r;
        }
    } else if (type == kLss) {
        const float* p = data + 6 * i;
        float ra = radius[2 * i], rb = radius[2 * i + 1];
        for (int k = 0; k < 3; ++k) {
            b.lo[k] = fmin_t(p[k] - ra, p[3 + k] - rb);
            b.hi[k] = fmax_t(p[k] + ra, p[3 + k] + rb);
        }
    } else if (type == kMesh) {
        const float* v = data + 9 * i;
        for (int k = 0; k < 3; ++k) {
            b.lo[k] = fmin_t(fmin_t(v[k], v[3 + k]), v[6 + k]);
            b.hi[k] = fmax_t(fmax_t(v[k], v[3 + k]), v[6 + k]);
        }
    } else if (type == kVoxel) {  // lo xyz, hi xyz, grid index (bits)
        const float* v = data + 7 * i;
        for (int k = 0; k < 3; ++k) { b.lo[k] = v[k]; b.hi[k] = v[3 + k]; }
    } else {
        const float* v = data + 36 * i;
        for (int k = 0; k < 3; ++k) {
            b.lo[k] = v[k];
            b.hi[k] = v[k];
            for (int j = 1; j < 12; ++j) {
                b.lo[k] = fmin_t(b.lo[k], v[3 * j + k]);
                b.hi[k] = fmax_t(b.hi[k], v[3 * j + k]);
            }
        }
    }
    return b;
}

// BVH references of a BLAS's primitives, the boxes its LBVH sorts: one per primitive, or for LSS
// and DOTS two per segment, the boxes of its halves (reference 2 i + h), as the device build forms
// them. LSS: the half u <= 1/2 of the round cone lies in the hull of the sphere at a and the
// sphere at the midpoint m with radius (ra + rb) / 2. DOTS: each quad is a trapezoid, s0 +- va
// at the start (vertices 0 and 4 of its six) and e0 +- vb at the end (vertices 2 and 1), so its
// first half is the hull of the start edge and the edge midpoints, its second half the hull of
// the midpoints and the end edge.
static int ref_shift_of(int type) { return (type == kLss || type == kDots) ? 1 : 0; }
static void ref_boxes(int type, const float* data, const float* radius, int64_t i, Box* out) {
    if (type == kLss) {
        const float* p = data + 6 * i;
        const float ra = radius[2 * i], rb = radius[2 * i + 1], rm = 0.5f * (ra + rb);
        for (int k = 0; k < 3; ++k) {
            const float m = 0.5f * (p[k] + p[3 + k]);
            out[0].lo[k] = fmin_t(p[k] - ra, m - rm);
            out[0].hi[k] = fmax_t(p[k] + ra, m + rm);
            out[1].lo[k] = fmin_t(m - rm, p[3 + k] - rb);
            out[1].hi[k] = fmax_t(m + rm, p[3 + k] + rb);
        }
    } else if (type == kDots) {
        const float* v = data + 36 * i;
        for (int k = 0; k < 3; ++k) {
            float lo0 = INFINITY, hi0 = -INFINITY, lo1 = INFINITY, hi1 = -INFINITY;
            for (int face = 0; face < 2; ++face) {
                const float* f = v + 18 * face;
                const float a = f[k], b = f[12 + k], c = f[6 + k], d = f[3 + k];
                const float mp = 0.5f * (a + c), mm = 0.5f * (b + d);
                lo0 = fmin_t(lo0, fmin_t(fmin_t(a, b), fmin_t(mp, mm)));
                hi0 = fmax_t(hi0, fmax_t(fmax_t(a, b), fmax_t(mp, mm)));
                lo1 = fmin_t(lo1, fmin_t(fmin_t(mp, mm), fmin_t(c, d)));
                hi1 = fmax_t(hi1, fmax_t(fmax_t(mp, mm), fmax_t(c, d)));
            }
            out[0].lo[k] = lo0;
            out[0].hi[k] = hi0;
            out[1].lo[k] = lo1;
            out[1].hi[k] = hi1;
        }
    } else {
        out[0] = prim_box(type, data, radius, i);
    }
}

// ---- LBVH: Morton codes, stable sort, Karras hierarchy, refit ----------------------------
// Centroid c = (lo + hi) * 0.5; per axis q = (c - cmin) * (2^21 / (cmax - cmin)) truncated
// to [0, 2^21 - 1] (0 when the extent is 0). Code = interleave with x in bit 3i+2, y in
// 3i+1, z in 3i (63 bits).
static inline uint64_t expand21(uint32_t v) {
    uint64_t x = v & 0x1fffff;
    x = (x | (x << 32)) & 0x1f00000000ffffULL;
    x = (x | (x << 16)) & 0x1f0000ff0000ffULL;
    x = (x | (x << 8)) & 0x100f00f00f00f00fULL;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ULL;
    x = (x | (x << 2)) & 0x1249249249249249ULL;
    return x;
}
static void morton_codes(const Box* boxes, int64_t n, uint64_t* codes) {
    float cmin[3] = {INFINITY, INFINITY, INFINITY}, cmax[3] = {-INFINITY, -INFINITY, -INFINITY};
    std::vector<float> cen(3 * n);
    for (int64_t i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            float c = (boxes[i].lo[k] + boxes[i].hi[k]) * 0.5f;
            cen[3 * i + k] = c;
            cmin[k] = fmin_t(cmin[k], c);
            cmax[k] = fmax_t(cmax[k], c);
        }
    float scale[3];
    for (int k = 0; k < 3; ++k) {
        float ext = cmax[k] - cmin[k];
        scale[k] = ext > 0.0f ? 2097152.0f / ext : 0.0f;
    }
    for (int64_t i = 0; i < n; ++i) {
        uint64_t code = 0;
        for (int k = 0; k < 3; ++k) {
            float q = (cen[3 * i + k] - cmin[k]) * scale[k];
            uint32_t qi = !(q > 0.0f) ? 0u : (q >= 2097151.0f ? 2097151u : uint32_t(q));  // NaN -> 0
            code |= expand21(qi) << (2 - k);
        }
        codes[i] = code;
    }
}

static inline int clz64(uint64_t x) { return x ? __builtin_clzll(x) : 64; }
static inline int clz32(uint32_t x) { return x ? __builtin_clz(x) : 32; }

// Karras 2012 hierarchy over sorted codes; duplicate codes are ordered by sorted position.
// Child encoding: bit 31 set = leaf (sorted primitive index), else internal node index.
// Internal node i covers sorted range [first[i], last[i]].
struct Binary {
    std::vector<uint32_t> left, right, first, last, parent_int, parent_leaf;
    std::vector<Box> box;  // internal node boxes
};
static void karras(const uint64_t* k, int64_t n, Binary& bt) {
    int64_t ni = n - 1;
    bt.left.assign(ni, 0); bt.right.assign(ni, 0); bt.first.assign(ni, 0); bt.last.assign(ni, 0);
    bt.parent_int.assign(ni, 0xffffffffu); bt.parent_leaf.assign(n, 0xffffffffu);
    auto delta = [&](int64_t i, int64_t j) -> int {
        if (j < 0 || j >= n) return -1;
        if (k[i] != k[j]) return clz64(k[i] ^ k[j]);
        return 64 + clz32(uint32_t(i) ^ uint32_t(j));
    };
    for (int64_t i = 0; i < ni; ++i) {
        int d = (delta(i, i + 1) - delta(i, i - 1)) > 0 ? 1 : -1;
        int dmin = delta(i, i - d);
        int64_t lmax = 2;
        while (delta(i, i + lmax * d) > dmin) lmax *= 2;
        int64_t l = 0;
        for (int64_t t = lmax / 2; t >= 1; t /= 2)
            if (delta(i, i + (l + t) * d) > dmin) l += t;
        int64_t j = i + l * d;
        int dnode = delta(i, j);
        int64_t s = 0;
        for (int64_t div = 2;; div *= 2) {
            int64_t t = (l + div - 1) / div;
            if (delta(i, i + (s + t) * d) > dnode) s += t;
            if (t == 1) break;
        }
        int64_t g = i + s * d + std::min(d, 0);
        int64_t lo = std::min(i, j), hi = std::max(i, j);
        bt.first[i] = uint32_t(lo);
        bt.last[i] = uint32_t(hi);
        if (lo == g) { bt.left[i] = 0x80000000u | uint32_t(g); bt.parent_leaf[g] = uint32_t(i); }
        else { bt.left[i] = uint32_t(g); bt.parent_int[g] = uint32_t(i); }
        if (hi == g + 1) { bt.right[i] = 0x80000000u | uint32_t(g + 1); bt.parent_leaf[g + 1] = uint32_t(i); }
        else { bt.right[i] = uint32_t(g + 1); bt.parent_int[g + 1] = uint32_t(i); }
    }
}
static Box box_union(const Box& a, const Box& b) {
    Box r;
    for (int k = 0; k < 3; ++k) { r.lo[k] = fmin_t(a.lo[k], b.lo[k]); r.hi[k] = fmax_t(a.hi[k], b.hi[k]); }
    return r;
}
// Refit: union of the children, left first (min/max order as the GPU's bottom-up pass).
static void refit(Binary& bt, const Box* sorted_boxes, int64_t n) {
    int64_t ni = n - 1;
    bt.box.assign(ni, Box{});
    std::vector<uint8_t> done(ni, 0);
    // post-order: process nodes whose children are complete, repeatedly (n is small here)
    std::vector<uint32_t> order;
    order.reserve(ni);
    std::vector<uint32_t> stack;
    if (ni > 0) stack.push_back(0);
    while (!stack.empty()) {  // reverse pre-order gives children before parents
        uint32_t i = stack.back();
        stack.pop_back();
        order.push_back(i);
        if (!(bt.left[i] & 0x80000000u)) stack.push_back(bt.left[i]);
        if (!(bt.right[i] & 0x80000000u)) stack.push_back(bt.right[i]);
    }
    for (auto it = order.rbegin(); it != order.rend(); ++it) {
        uint32_t i = *it;
        auto cb = [&](uint32_t c) -> const Box& {
            return (c & 0x80000000u) ? sorted_boxes[c & 0x7fffffffu] : bt.box[c];
        };
        bt.box[i] = box_union(cb(bt.left[i]), cb(bt.right[i]));
        done[i] = 1;
    }
}

// ---- collapse to an 8-wide BVH (breadth-first layout) ------------------------------------
// The binary tree's nodes are distributed over wide nodes by cost, a restatement of the
// dynamic program of Ylitalo, Immonen and Karras (HPG 2017, "Efficient incoherent ray
// traversal on GPUs through compressed wide BVHs", section 3): with A the surface-area measure
// (dx*dy + dy*dz) + dz*dx, cost(x, k) is the least cost of x's subtree when it fills k slots
// (k = 1..8) of its parent:
//   a primitive: A for every k;
//   dist(k) = min over j = 1..k-1 of cost(left, j) + cost(right, k - j)   (k >= 2);
//   cost(x, 1) = A c when x holds c <= max_leaf primitives (a leaf slot), else A + dist(W);
//   cost(x, k) = min(cost(x, k - 1), dist(k)).
// W is the node fan-out (8 by default; a narrower tree uses W of the 8 slots). Each wide node
// starts from a binary internal node b whose W slots go to its children as j and W - j, j the
// least minimiser of cost(left, j) + cost(right, W - j); a child given k slots takes
// the fewest k' <= k of the same cost and, with k' > 1, splits them again between its own
// children, left before right. A child holding at most max_leaf primitives becomes a leaf (a
// contiguous run of sorted primitives), a larger one a wide node of the next level. The
// children are then placed in the 8 slots by direction (octant_slots below).
// Nodes are numbered breadth first; a node's internal children take consecutive indices from
// child_base in slot order, and its leaf primitives are copied to consecutive slots from
// prim_base in slot order (the primitive order array).
// meta byte per slot: 0 empty, 0x80|rank internal, (count<<5)|offset leaf; an empty slot's box
// is lo = +inf, hi = -inf.
struct Wide {
    std::vector<uint32_t> child_base, prim_base;
    std::vector<uint8_t> meta;     // 8 per node
    std::vector<Box> cbox;         // 8 per node
    std::vector<uint32_t> prim_order;  // slot -> sorted primitive index
};
static float sa_measure(const Box& b) {
    float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return (dx * dy + dy * dz) + dz * dx;
}
// Slot of each child by direction: cost(c, s) = ((+-dx) + (+-dy)) + (+-dz) with
// d = (lo + hi of the child) - (lo + hi of the node), the sign on an axis + when bit
// (x 1, y 2, z 4) of s is set. The (child, slot) pair of largest cost is taken first,
// repeatedly; ties go to the lower child, then the lower slot, and a NaN cost never replaces a
// candidate already held. kid_in[s] = child index or -1. (A ray then visits slots in the order
// i ^ octant, octant bit k set when the ray's direction is negative on axis k: nearest first.)
static void octant_slots(const Box& parent, const Box* const* kid_box, int n, int* kid_in) {
    const float pc[3] = {parent.lo[0] + parent.hi[0], parent.lo[1] + parent.hi[1], parent.lo[2] + parent.hi[2]};
    int slot_of[8];
    for (int q = 0; q < 8; ++q) { kid_in[q] = -1; slot_of[q] = -1; }
    for (int r = 0; r < n; ++r) {
        int bq = -1, bs = -1;
        float bc = 0.0f;
        for (int q = 0; q < n; ++q) {
            if (slot_of[q] >= 0) continue;
            const Box& b = *kid_box[q];
            float d0 = (b.lo[0] + b.hi[0]) - pc[0], d1 = (b.lo[1] + b.hi[1]) - pc[1], d2 = (b.lo[2] + b.hi[2]) - pc[2];
            for (int s2 = 0; s2 < 8; ++s2) {
                if (kid_in[s2] >= 0) continue;
                float c = ((s2 & 1 ? d0 : -d0) + (s2 & 2 ? d1 : -d1)) + (s2 & 4 ? d2 : -d2);
                if (bq < 0 || c > bc) { bq = q; bs = s2; bc = c; }
            }
        }
        slot_of[bq] = bs;
        kid_in[bs] = bq;
    }
}

static void collapse(const Binary& bt, const Box* sorted_boxes, int64_t n, int max_leaf, int width, Wide& w) {
    w = Wide{};
    if (n <= 0) return;
    auto count = [&](uint32_t c) -> uint32_t {
        return (c & 0x80000000u) ? 1u : bt.last[c] - bt.first[c] + 1;
    };
    auto cbox = [&](uint32_t c) -> const Box& {
        return (c & 0x80000000u) ? sorted_boxes[c & 0x7fffffffu] : bt.box[c];
    };
    auto cfirst = [&](uint32_t c) -> uint32_t { return (c & 0x80000000u) ? (c & 0x7fffffffu) : bt.first[c]; };
    // collapse costs, children before parents (reverse pre-order)
    std::vector<float> dpc(n >= 2 ? 8 * size_t(n - 1) : 0);
    auto cost = [&](uint32_t c, int k) -> float {
        return (c & 0x80000000u) ? sa_measure(sorted_boxes[c & 0x7fffffffu]) : dpc[8 * size_t(c) + (k - 1)];
    };
    if (n >= 2) {
        std::vector<uint32_t> pre, stk{0u};
        while (!stk.empty()) {
            uint32_t x = stk.back();
            stk.pop_back();
            pre.push_back(x);
            if (!(bt.left[x] & 0x80000000u)) stk.push_back(bt.left[x]);
            if (!(bt.right[x] & 0x80000000u)) stk.push_back(bt.right[x]);
        }
        for (size_t o = pre.size(); o-- > 0;) {
            const uint32_t x = pre[o], l = bt.left[x], r = bt.right[x];
            float dist[9];
            for (int k = 2; k <= 8; ++k) {
                float best = INFINITY;
                for (int i = 1; i < k; ++i) {
                    const float v = cost(l, i) + cost(r, k - i);
                    if (v < best) best = v;
                }
                dist[k] = best;
            }
            const uint32_t cnt = count(x);
            const float a = sa_measure(bt.box[x]);
            float* c = &dpc[8 * size_t(x)];
            c[0] = cnt <= uint32_t(max_leaf) ? a * float(cnt) : a + dist[width];
            for (int k = 2; k <= 8; ++k) c[k - 1] = dist[k] < c[k - 2] ? dist[k] : c[k - 2];
        }
    }
    auto split = [&](uint32_t x, int k) -> int {
        int bj = 1;
        float bv = INFINITY;
        for (int j = 1; j < k; ++j) {
            const float v = cost(bt.left[x], j) + cost(bt.right[x], k - j);
            if (v < bv) { bv = v; bj = j; }
        }
        return bj;
    };
    std::vector<uint32_t> level;  // binary node per wide node (0x80000000|p for a 1-prim root)
    level.push_back(n == 1 ? 0x80000000u : 0u);
    uint32_t next_node = 1, next_prim = 0;
    while (!level.empty()) {
        std::vector<uint32_t> nxt;
        for (uint32_t b : level) {
            uint32_t kids[8];
            int nk = 0;
            if (b & 0x80000000u) kids[nk++] = b;
            else {
                std::vector<std::pair<uint32_t, int>> work;  // (binary node, slots), left on top
                const int j = split(b, width);
                work.push_back({bt.right[b], width - j});
                work.push_back({bt.left[b], j});
                while (!work.empty()) {
                    auto [x, k] = work.back();
                    work.pop_back();
                    if (x & 0x80000000u) { kids[nk++] = x; continue; }
                    while (k > 1 && cost(x, k) == cost(x, k - 1)) --k;
                    if (k == 1) { kids[nk++] = x; continue; }
                    const int jj = split(x, k);
                    work.push_back({bt.right[x], k - jj});
                    work.push_back({bt.left[x], jj});
                }
            }
            size_t base = w.meta.size();
            w.meta.resize(base + 8, 0);
            w.cbox.resize(base + 8, Box{{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}});
            w.child_base.push_back(next_node);
            w.prim_base.push_back(next_prim);
            const Box* kb[8];
            for (int q = 0; q < nk; ++q) kb[q] = &cbox(kids[q]);
            int kid_in[8];
            octant_slots(cbox(b), kb, nk, kid_in);
            uint32_t rank = 0, poff = 0;
            for (int q = 0; q < 8; ++q) {
                if (kid_in[q] < 0) continue;
                uint32_t c = kids[kid_in[q]];
                w.cbox[base + q] = cbox(c);
                uint32_t cnt = count(c);
                if (!(c & 0x80000000u) && cnt > uint32_t(max_leaf)) {
                    w.meta[base + q] = uint8_t(0x80u | rank++);
                    nxt.push_back(c);
                } else {
                    w.meta[base + q] = uint8_t((cnt << 5) | poff);
                    for (uint32_t j = 0; j < cnt; ++j) w.prim_order.push_back(cfirst(c) + j);
                    poff += cnt;
                }
            }
            next_node += rank;
            next_prim += poff;
        }
        level.swap(nxt);
    }
}

// ---- 8-bit quantisation of a wide node's child boxes --------------------------------------
// Origin p = min of the child boxes; per axis the smallest e with 255 * 2^e >= extent
// (extent in double, exactly); qlo = floor((lo - p) 2^-e), qhi = ceil((hi - p) 2^-e), in
// double, clamped to [0, 255]. Decoding p + q 2^e in one rounded operation never shrinks a box.
// Exponent byte = e + 127 (e clamped to [-126, 127]). Empty slots: qlo = 255, qhi = 0.
static void quantise_node(const Box* cb, const uint8_t* meta, float* p_out, uint8_t* e_out,
                          uint8_t* qlo, uint8_t* qhi) {
    float p[3] = {INFINITY, INFINITY, INFINITY}, P[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int q = 0; q < 8; ++q) {
        if (!meta[q]) continue;
        for (int k = 0; k < 3; ++k) { p[k] = fmin_t(p[k], cb[q].lo[k]); P[k] = fmax_t(P[k], cb[q].hi[k]); }
    }
    for (int k = 0; k < 3; ++k) {
        double ext = double(P[k]) - double(p[k]);
        int e;
        if (!(ext > 0.0)) e = -126;
        else {
            int ex;
            double m = std::frexp(ext / 255.0, &ex);
            e = (m == 0.5) ? ex - 1 : ex;
            while (std::ldexp(255.0, e) < ext) ++e;
            if (e < -126) e = -126;
            if (e > 127) e = 127;
        }
        p_out[k] = p[k];
        e_out[k] = uint8_t(e + 127);
        for (int q = 0; q < 8; ++q) {
            if (!meta[q]) { qlo[8 * k + q] = 255; qhi[8 * k + q] = 0; continue; }
            double lo = std::floor((double(cb[q].lo[k]) - double(p[k])) * std::ldexp(1.0, -e));
            double hi = std::ceil((double(cb[q].hi[k]) - double(p[k])) * std::ldexp(1.0, -e));
            qlo[8 * k + q] = uint8_t(std::min(255.0, std::max(0.0, lo)));
            qhi[8 * k + q] = uint8_t(std::min(255.0, std::max(0.0, hi)));
        }
    }
}

// ---- voxel hair ------------------------------------------------------------------------------
// Restated from GenerateVoxelMesh (geometry_processor.cpp:515-602), the capsule voxelisation of
// "Real-Time Rendering of Dynamic Line Sets using Voxel Ray Tracing" that it follows, with what
// the reference leaves unfinished defined here:
//   grid: origin = min over the line end points (coordinates + 0, so no -0) minus r; extent =
//     (max + r) - origin; res = max(1, ceil(extent / size)) per axis (the reference starts at the
//     mesh bounds and has no room for the capsules' radius);
//   per line, d = end - start; the axes sorted by |d| descending (ties: lower axis first) are
//     a0 (major), a1, a2; a line with |d[a0]| = 0 fills nothing. v0, v1 = the end points ordered
//     along +a0; s = d / d[a0]; vr0 = v0 - s r, vr1 = v1 + s r; dn = sqrt((dx dx + dy dy) + dz dz);
//     r1 = r / sqrt(1 - (d[a1]/dn)^2), r2 likewise with a2. From t0 = tmin = vr0[a0] while
//     t0 < tmax = vr1[a0]: t1 = min(tmax, t0 + size), p1 = vr0 + s (t1 - tmin), the box from
//     min(p0, p1) - (r1 on a1, r2 on a2) to max(p0, p1) + (r1, r2) fills every voxel of its index
//     range floor((corner - origin) / size), clamped to the grid (the reference fills only the
//     cells at the range's lowest x, geometry_processor.cpp:586-592); t0 = t1, p0 = p1;
//   the filled voxels in ascending grid index i = x + y res_x + z res_x res_y become boxes
//     lo = origin + float(x, y, z) size, hi = lo + size, reporting primitive id i (the reference
//     gives every grid cell an AABB, geometry_processor.cpp:452-471, and its intersection shader
//     reports t = 1 for all of them, voxel_intersection.rint:14: here a ray-box hit).
struct VoxelGrid {
    float origin[3], size;
    int32_t res[3];
};
static VoxelGrid voxel_grid(const float* lines, int64_t n, float r, float size) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = 0; i < n; ++i)
        for (int e = 0; e < 2; ++e)
            for (int k = 0; k < 3; ++k) {
                const float v = lines[6 * i + 3 * e + k] + 0.0f;
                lo[k] = fmin_t(lo[k], v);
                hi[k] = fmax_t(hi[k], v);
            }
    VoxelGrid g;
    g.size = size;
    for (int k = 0; k < 3; ++k) {
        g.origin[k] = lo[k] - r;
        const float ext = (hi[k] + r) - g.origin[k];
        const float c = std::ceil(ext / size);
        g.res[k] = c >= 1.0f ? int32_t(c) : 1;
    }
    return g;
}
static void voxel_axes(const float* d, int* a) {
    a[0] = 0; a[1] = 1; a[2] = 2;
    for (int i = 1; i < 3; ++i)  // insertion sort by |d| descending, ties keep the lower axis first
        for (int j = i; j > 0 && std::fabs(d[a[j]]) > std::fabs(d[a[j - 1]]); --j) std::swap(a[j], a[j - 1]);
}
// Fills the voxels of one line (grid indices into `filled`); returns false past 2^20 steps.
static bool voxel_line(const float* line, float r, const VoxelGrid& g, std::vector<uint8_t>& filled) {
    const float* p = line;
    const float* q = line + 3;
    float d[3] = {q[0] - p[0], q[1] - p[1], q[2] - p[2]};
    int a[3];
    voxel_axes(d, a);
    if (!(std::fabs(d[a[0]]) > 0.0f)) return true;
    const float* v0 = d[a[0]] < 0.0f ? q : p;
    const float* v1 = d[a[0]] < 0.0f ? p : q;
    float sv[3], vr0[3], vr1[3];
    for (int k = 0; k < 3; ++k) {
        sv[k] = d[k] / d[a[0]];
        const float sr = sv[k] * r;
        vr0[k] = v0[k] - sr;
        vr1[k] = v1[k] + sr;
    }
    const float dn = std::sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
    const float q1 = d[a[1]] / dn, q2 = d[a[2]] / dn;
    const float r1 = r / std::sqrt(1.0f - q1 * q1), r2 = r / std::sqrt(1.0f - q2 * q2);
    const float tmin = vr0[a[0]], tmax = vr1[a[0]];
    float t0 = tmin, p0[3] = {vr0[0], vr0[1], vr0[2]};
    const int64_t rx = g.res[0], rxy = int64_t(g.res[0]) * g.res[1];
    for (int step = 0; t0 < tmax; ++step) {
        if (step >= (1 << 20)) return false;
        const float tn = t0 + g.size;
        const float t1 = tn < tmax ? tn : tmax;
        float p1[3], wmin[3], wmax[3];
        for (int k = 0; k < 3; ++k) {
            p1[k] = vr0[k] + sv[k] * (t1 - tmin);
            wmin[k] = fmin_t(p0[k], p1[k]);
            wmax[k] = fmax_t(p0[k], p1[k]);
        }
        wmin[a[1]] -= r1;
        wmin[a[2]] -= r2;
        wmax[a[1]] += r1;
        wmax[a[2]] += r2;
        int32_t mi[3], ma[3];
        for (int k = 0; k < 3; ++k) {
            const float f0 = std::floor((wmin[k] - g.origin[k]) / g.size), f1 = std::floor((wmax[k] - g.origin[k]) / g.size);
            mi[k] = f0 < 0.0f ? 0 : (f0 > float(g.res[k] - 1) ? g.res[k] - 1 : int32_t(f0));
            ma[k] = f1 < 0.0f ? 0 : (f1 > float(g.res[k] - 1) ? g.res[k] - 1 : int32_t(f1));
        }
        for (int32_t z = mi[2]; z <= ma[2]; ++z)
            for (int32_t y = mi[1]; y <= ma[1]; ++y)
                for (int32_t x = mi[0]; x <= ma[0]; ++x) filled[size_t(x + y * rx + z * rxy)] = 1;
        t0 = t1;
        for (int k = 0; k < 3; ++k) p0[k] = p1[k];
    }
    return true;
}

// ---- tracer ---------------------------------------------------------------------------------
struct Blas {
    int type = kPhantom;
    int64_t nprim = 0;
    std::vector<float> data, radius;  // see prim_box for the layouts
    std::vector<Box> boxes;           // per primitive (original order)
    std::vector<uint32_t> sorted;     // sorted position -> primitive
    Binary bt;
    Box root;
    // mesh material: albedo factor; with a map, texture coordinates per triangle (6 floats)
    float albedo[4] = {1.0f, 1.0f, 1.0f, 1.0f};
    std::vector<float> uv, map;
    uint32_t map_w = 0, map_h = 0;
};
struct Instance {
    int blas;
    double xf[16];      // object to world, column major
    double inv[16];     // world to object
    bool identity;
};
struct Scene {
    std::vector<Blas> blas;
    std::vector<Instance> inst;
};

static void build_blas(Blas& b) {
    int64_t n = b.nprim;
    b.boxes.resize(n);
    for (int64_t i = 0; i < n; ++i) b.boxes[i] = prim_box(b.type, b.data.data(), b.radius.data(), i);
    std::vector<uint64_t> codes(n);
    morton_codes(b.boxes.data(), n, codes.data());
    b.sorted.resize(n);
    for (int64_t i = 0; i < n; ++i) b.sorted[i] = uint32_t(i);
    std::stable_sort(b.sorted.begin(), b.sorted.end(), [&](uint32_t x, uint32_t y) { return codes[x] < codes[y]; });
    std::vector<uint64_t> sk(n);
    std::vector<Box> sb(n);
    for (int64_t i = 0; i < n; ++i) { sk[i] = codes[b.sorted[i]]; sb[i] = b.boxes[b.sorted[i]]; }
    if (n >= 2) {
        karras(sk.data(), n, b.bt);
        refit(b.bt, sb.data(), n);
        b.root = b.bt.box[0];
    } else if (n == 1) b.root = sb[0];
}

template <class T> struct HitT {
    T t;
    uint32_t inst, prim, seg;  // prim = reported primitive id; seg = BVH primitive (segment)
    T u;                       // curve / segment parameter (mesh: barycentric weight of v1)
    T v;                       // mesh: barycentric weight of v2
    tvec3<T> n;                // world-space normal
    int resolved64;
};

template <class T> static inline bool slab(const Box& b, const tvec3<T>& o, const tvec3<T>& inv, T tmin, T tmax) {
    T t0 = tmin, t1 = tmax;
    for (int k = 0; k < 3; ++k) {
        T a = (T(b.lo[k]) - o[k]) * inv[k];
        T c = (T(b.hi[k]) - o[k]) * inv[k];
        if (a > c) std::swap(a, c);
        t0 = a > t0 ? a : t0;
        t1 = c < t1 ? c : t1;
    }
    return t0 <= t1 * T(1.0000004);  // conservative: rounding may only admit extra boxes
}

static inline double xf_point(const double* m, const double* p, int k) {
    return ((m[k] * p[0] + m[4 + k] * p[1]) + m[8 + k] * p[2]) + m[12 + k];
}
static inline double xf_dir(const double* m, const double* p, int k) {
    return (m[k] * p[0] + m[4 + k] * p[1]) + m[8 + k] * p[2];
}

// Intersect one BVH primitive; returns true and fills *h when it beats (t, prim) of *h.
// mode64: 0 = precision T only; 1 = T then FP64 re-solve of unresolved Phantom candidates.
// Diagnostics: FP32 unresolved candidates (far / near) and how many the FP64 re-solve turned
// into hits (far / near).
static std::atomic<int64_t> g_stat[4];
// Closest-hit order: smaller t, then smaller instance, then smaller primitive id.
template <class T>
static bool intersect_prim(const Blas& b, uint32_t inst, uint32_t s, const tvec3<T>& o, const tvec3<T>& d, T tmin,
                           HitT<T>* h, int resolve64, bool unit_dir) {
    bool better = false;
    auto take = [&](T t, uint32_t prim, T u, int r64) {
        if (!(t >= tmin) || !(t <= h->t)) return;
        if (t == h->t && (inst > h->inst || (inst == h->inst && prim >= h->prim))) return;
        h->t = t; h->inst = inst; h->prim = prim; h->seg = s; h->u = u; h->resolved64 = r64;
        better = true;
    };
    if (b.type == kPhantom) {
        const float* c = b.data.data() + 12 * s;
        Curve<T> cv{tvec3<T>(T(c[0]), T(c[1]), T(c[2])), tvec3<T>(T(c[3]), T(c[4]), T(c[5])),
                    tvec3<T>(T(c[6]), T(c[7]), T(c[8])), tvec3<T>(T(c[9]), T(c[10]), T(c[11]))};
        // Prhi measures the hit as a length along the ray's unit direction (the reference runs it
        // on the unit world ray, hair_intersection.rint:138-141). The object-space ray of a
        // transformed instance is o + t d with |d| != 1: Prhi runs on the unit direction and its
        // length becomes the parameter t = length / |d|, so hits compare across instances.
        const T dlen = unit_dir ? T(1) : shim::length(d);
        Ray<T> ray{o, unit_dir ? d : d * (T(1) / dlen)};
        int st;
        tvec3<T> nrm;
        bool shift = (resolve64 & 2) != 0, polish = (resolve64 & 4) != 0;
        T t = prhi(ray, cv, T(b.radius[2 * s]), T(b.radius[2 * s + 1]), &nrm, &st, shift, polish);
        if (!unit_dir) t = t / dlen;
        if (st == kUnresolved || st == kUnresolvedNear) g_stat[st == kUnresolved ? 0 : 1]++;
        if (st == kHit) { take(t, s, T(0), 0); if (better) h->n = nrm; }
        else if (st == kUnresolvedNear && (resolve64 & 1)) {  // failed convergence test only
            Curve<double> cd{tvec3<double>(c[0], c[1], c[2]), tvec3<double>(c[3], c[4], c[5]),
                             tvec3<double>(c[6], c[7], c[8]), tvec3<double>(c[9], c[10], c[11])};
            const double dl2 = unit_dir ? 1.0 : double(dlen);
            Ray<double> rd{tvec3<double>(o.x, o.y, o.z), tvec3<double>(double(ray.direction.x), double(ray.direction.y),
                                                                      double(ray.direction.z))};
            int st2;
            tvec3<double> n2;
            double t2 = prhi(rd, cd, double(b.radius[2 * s]), double(b.radius[2 * s + 1]), &n2, &st2, shift, polish);
            if (!unit_dir) t2 = t2 / dl2;
            if (st2 == kHit) {
                g_stat[st == kUnresolved ? 2 : 3]++;
                take(T(t2), s, T(0), 1);
                if (better) h->n = tvec3<T>(T(n2.x), T(n2.y), T(n2.z));
            }
        }
    } else if (b.type == kLss) {
        const float* p = b.data.data() + 6 * s;
        tvec3<T> a = tvec3<T>{T(p[0]), T(p[1]), T(p[2])}, e = tvec3<T>{T(p[3]), T(p[4]), T(p[5])};
        T u;
        T t = lss_intersect(o, d, a, e, T(b.radius[2 * s]), T(b.radius[2 * s + 1]), tmin, &u);
        if (t >= T(0)) {
            take(t, s, u, 0);
            if (better) {
                tvec3<T> hp = o + t * d;
                h->n = shim::normalize(hp - (a + u * (e - a)));
            }
        }
    } else if (b.type == kMesh) {
        // triangle i reports primitive id i; the normal interpolates the vertex normals with the
        // hit's barycentrics (triangle_closest_hit.rchit:19-41), else it is the face normal
        const float* q = b.data.data() + 9 * s;
        tvec3<T> v0 = tvec3<T>{T(q[0]), T(q[1]), T(q[2])}, v1 = tvec3<T>{T(q[3]), T(q[4]), T(q[5])},
                 v2 = tvec3<T>{T(q[6]), T(q[7]), T(q[8])};
        T b1, b2;
        T t = tri_intersect(o, d, v0, v1, v2, tmin, h->t, &b1, &b2);
        if (t >= T(0)) {
            take(t, s, b1, 0);
            if (better) {
                h->v = b2;
                if (!b.radius.empty()) {
                    const float* m = b.radius.data() + 9 * s;
                    T w = T(1) - b1 - b2;
                    tvec3<T> n0{T(m[0]), T(m[1]), T(m[2])}, n1{T(m[3]), T(m[4]), T(m[5])}, n2{T(m[6]), T(m[7]), T(m[8])};
                    h->n = shim::normalize(w * n0 + b1 * n1 + b2 * n2);
                } else {
                    h->n = shim::normalize(shim::cross(v1 - v0, v2 - v0));
                }
            }
        }
    } else if (b.type == kVoxel) {
        // ray-box: per axis the slab's entry and exit (an axis the ray runs parallel to only
        // rejects an origin outside the slab); hit at the entry distance, or at tmin when the
        // ray starts inside; the normal is the entry face's (the axis of the latest entry, the
        // lower axis on ties), facing the ray
        const float* v = b.data.data() + 7 * s;
        T tn = -T(INFINITY), tf = T(INFINITY);
        int ax = 0;
        bool miss = false;
        for (int k = 0; k < 3; ++k) {
            if (d[k] == T(0)) {
                if (o[k] < T(v[k]) || o[k] > T(v[3 + k])) miss = true;
                continue;
            }
            T a0 = (T(v[k]) - o[k]) / d[k], a1 = (T(v[3 + k]) - o[k]) / d[k];
            if (a0 > a1) std::swap(a0, a1);
            if (a0 > tn) { tn = a0; ax = k; }
            if (a1 < tf) tf = a1;
        }
        if (!miss && tn <= tf) {
            const T t = tn >= tmin ? tn : (tf >= tmin ? tmin : T(-1));
            uint32_t id;
            std::memcpy(&id, v + 6, 4);
            if (t >= tmin) {
                take(t, id, T(ax), 0);
                if (better) {
                    tvec3<T> nn(T(0), T(0), T(0));
                    nn[ax] = d[ax] > T(0) ? T(-1) : T(1);
                    h->n = nn;
                }
            }
        }
    } else {
        const float* v = b.data.data() + 36 * s;
        for (int k = 0; k < 4; ++k) {
            const float* q = v + 9 * k;
            tvec3<T> v0 = tvec3<T>{T(q[0]), T(q[1]), T(q[2])}, v1 = tvec3<T>{T(q[3]), T(q[4]), T(q[5])},
                     v2 = tvec3<T>{T(q[6]), T(q[7]), T(q[8])};
            T t = tri_intersect(o, d, v0, v1, v2, tmin, h->t);
            if (t >= T(0)) {
                bool was = better;
                better = false;
                take(t, 4 * s + k, T(0), 0);
                if (better) h->n = shim::normalize(shim::cross(v1 - v0, v2 - v0));
                better = better || was;
            }
        }
    }
    return better;
}

// Closest hit (any_hit = false) or any hit excluding (skip_inst, skip_seg).
template <class T>
static bool trace_one(const Scene& sc, const tvec3<T>& wo, const tvec3<T>& wd, T tmin, T tmax, bool any_hit,
                      uint32_t skip_inst, uint32_t skip_seg, int resolve64, HitT<T>* out) {
    HitT<T> h;
    h.t = tmax; h.inst = 0xffffffffu; h.prim = 0xffffffffu; h.seg = 0xffffffffu; h.u = T(0);
    h.n = tvec3<T>(T(0), T(0), T(0)); h.resolved64 = 0;
    bool found = false;
    for (uint32_t ii = 0; ii < sc.inst.size(); ++ii) {
        const Instance& in = sc.inst[ii];
        const Blas& b = sc.blas[in.blas];
        if (b.nprim == 0) continue;
        tvec3<T> o = wo, d = wd;
        if (!in.identity) {
            double po[3] = {double(wo.x), double(wo.y), double(wo.z)}, pd[3] = {double(wd.x), double(wd.y), double(wd.z)};
            o = tvec3<T>(T(xf_point(in.inv, po, 0)), T(xf_point(in.inv, po, 1)), T(xf_point(in.inv, po, 2)));
            d = tvec3<T>(T(xf_dir(in.inv, pd, 0)), T(xf_dir(in.inv, pd, 1)), T(xf_dir(in.inv, pd, 2)));
        }
        tvec3<T> inv(T(1) / d.x, T(1) / d.y, T(1) / d.z);
        if (!slab(b.root, o, inv, tmin, h.t)) continue;
        uint32_t stack[128];
        int sp = 0;
        uint32_t cur = b.nprim == 1 ? 0x80000000u : 0u;
        for (;;) {
            if (cur & 0x80000000u) {
                uint32_t s = b.sorted[cur & 0x7fffffffu];
                bool skip = any_hit && ii == skip_inst && s == skip_seg;
                if (!skip) {
                    if (intersect_prim(b, ii, s, o, d, tmin, &h, resolve64, in.identity)) {
                        found = true;
                        if (!in.identity) {
                            double pn[3] = {double(h.n.x), double(h.n.y), double(h.n.z)};
                            // normals transform by the inverse transpose
                            tvec3<T> n2;
                            for (int k = 0; k < 3; ++k)
                                n2[k] = T((in.inv[4 * k] * pn[0] + in.inv[4 * k + 1] * pn[1]) + in.inv[4 * k + 2] * pn[2]);
                            h.n = shim::normalize(n2);
                        }
                        if (any_hit) { *out = h; return true; }
                    }
                }
            } else {
                uint32_t l = b.bt.left[cur], r = b.bt.right[cur];
                const Box& bl = (l & 0x80000000u) ? b.boxes[b.sorted[l & 0x7fffffffu]] : b.bt.box[l];
                const Box& br = (r & 0x80000000u) ? b.boxes[b.sorted[r & 0x7fffffffu]] : b.bt.box[r];
                bool hl = slab(bl, o, inv, tmin, h.t), hr = slab(br, o, inv, tmin, h.t);
                if (hl && hr) { stack[sp++] = r; cur = l; continue; }
                if (hl) { cur = l; continue; }
                if (hr) { cur = r; continue; }
            }
            if (sp == 0) break;
            cur = stack[--sp];
        }
    }
    *out = h;
    return found;
}

}  // namespace orc

// =============================================================================================
// C entry points (ctypes)
// =============================================================================================
using namespace orc;

namespace {
// Precision codes of the tracing entry points.
//   64    FP64, Phantom evaluated from the shifted origin (the oracle of record)
//   6400  FP64, the reference-literal evaluation from the ray origin
//   32    FP32, reference-literal; 3264 the same with FP64 re-solve of unresolved candidates
//   33    FP32 from the shifted origin; 3364 the same with FP64 re-solve
// The literal world-space bounding-cylinder test (cylinder.glsl:8-46) assumes a unit direction;
// with a float-normalised direction its error grows with the squared distance of the ray
// origin from the segment, so from a camera a few units away it misjudges rays in roughly the
// outer tenth of the bounding radius even in exact arithmetic. The shifted evaluation is the
// same formula on the same line, with that term made negligible.
int fp32_mode(int precision) {
    int p = precision % 1000000;
    int m = (p == 3264 || p == 3364 ? 1 : 0) | (p == 33 || p == 3364 ? 2 : 0);
    return m | (precision >= 1000000 ? 4 : 0);
}
int fp64_mode(int precision) { return (precision % 1000000 == 6400 ? 0 : 2) | (precision >= 1000000 ? 4 : 0); }
template <class F> void parallel_for(int64_t n, int nthreads, F f) {
    if (nthreads <= 1 || n < 256) { for (int64_t i = 0; i < n; ++i) f(i); return; }
    std::atomic<int64_t> next{0};
    std::vector<std::thread> th;
    for (int k = 0; k < nthreads; ++k)
        th.emplace_back([&]() {
            for (;;) {
                int64_t s = next.fetch_add(64);
                if (s >= n) break;
                int64_t e = std::min(n, s + 64);
                for (int64_t i = s; i < e; ++i) f(i);
            }
        });
    for (auto& t : th) t.join();
}
uint32_t hash_u32(uint32_t x) {  // integer finaliser (splitmix-style), used for jitter
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}
}  // namespace

extern "C" {

// ---- shader math (bit-for-bit comparison with oracle/_ref) ---------------------------------
float orc_prhi_f32(const float* ray, const float* curve, float r0, float r1, float* normal, int* status) {
    Ray<float> r{v3f(ray[0], ray[1], ray[2]), v3f(ray[3], ray[4], ray[5])};
    Curve<float> c{ld3(curve), ld3(curve + 3), ld3(curve + 6), ld3(curve + 9)};
    v3f n(0.f, 0.f, 0.f);
    float t = prhi(r, c, r0, r1, &n, status);
    st3(normal, n);
    return t;
}
double orc_prhi_f64(const double* ray, const double* curve, double r0, double r1, double* normal, int* status) {
    using v3d = tvec3<double>;
    Ray<double> r{v3d(ray[0], ray[1], ray[2]), v3d(ray[3], ray[4], ray[5])};
    Curve<double> c{v3d(curve[0], curve[1], curve[2]), v3d(curve[3], curve[4], curve[5]),
                    v3d(curve[6], curve[7], curve[8]), v3d(curve[9], curve[10], curve[11])};
    v3d n(0.0, 0.0, 0.0);
    double t = prhi(r, c, r0, r1, &n, status);
    normal[0] = n.x; normal[1] = n.y; normal[2] = n.z;
    return t;
}
void orc_cone_f32(const float* cone, float* out6) {
    Cone<float> c{ld3(cone), cone[3], ld3(cone + 4), cone[7]};
    ConeHit<float> r = ray_cone_rcc(c);
    out6[0] = r.isIntersection ? 1.f : 0.f;
    out6[1] = r.s; out6[2] = r.dt; out6[3] = r.dp; out6[4] = r.dc; out6[5] = r.sp;
}
int orc_cylinder_f32(const float* ray, const float* cyl) {
    Ray<float> r{ld3(ray), ld3(ray + 3)};
    Cylinder<float> c{ld3(cyl), ld3(cyl + 3), cyl[6]};
    return ray_cylinder(r, c) ? 1 : 0;
}
void orc_curve_sample_f32(const float* curve, float t, float* out6) {
    Curve<float> c{ld3(curve), ld3(curve + 3), ld3(curve + 6), ld3(curve + 9)};
    st3(out6, sample_point(c, t));
    st3(out6 + 3, sample_axis(c, t));
}
void orc_rcc_matrix_f32(const float* ray, float* m16) {
    Ray<float> r{ld3(ray), ld3(ray + 3)};
    tmat4<float> m = rcc_matrix(r);
    for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) m16[c * 4 + k] = m[c][k];
}
void orc_shade_f32(const float* n, float* rgb) { st3(rgb, shade(ld3(n))); }

// ray_gen.rgen:18-24 with a sub-pixel offset (jx, jy) in place of the pixel centre 0.5.
void orc_raygen_f32(const float* vi, const float* pi, uint32_t px, uint32_t py, uint32_t w, uint32_t h,
                    float jx, float jy, float* o3, float* d3) {
    tmat4<float> V, P;
    for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) { V[c][k] = vi[c * 4 + k]; P[c][k] = pi[c * 4 + k]; }
    float cx = float(px) + jx, cy = float(py) + jy;
    float ux = cx / float(w), uy = cy / float(h);
    float dx = ux * 2.0f - 1.0f, dy = uy * 2.0f - 1.0f;
    tvec4<float> origin = V * tvec4<float>(0.f, 0.f, 0.f, 1.f);
    tvec4<float> target = P * tvec4<float>(dx, dy, 1.f, 1.f);
    tvec4<float> dir = V * tvec4<float>(shim::normalize(target.xyz), 0.f);
    st3(o3, origin.xyz);
    st3(d3, dir.xyz);
}

// ---- geometry processing ---------------------------------------------------------------
void orc_generate_curves(const float* lines, int64_t n, float* out) { generate_curves(lines, n, out); }
void orc_generate_aabbs(const float* curves, int64_t n, float r, float* out) {
    for (int64_t i = 0; i < n; ++i) {
        const float* c = curves + 12 * i;
        for (int k = 0; k < 3; ++k) {
            out[6 * i + k] = fmin_t(fmin_t(c[k], c[9 + k]), fmin_t(c[3 + k], c[6 + k])) - r;
            out[6 * i + 3 + k] = fmax_t(fmax_t(c[k], c[9 + k]), fmax_t(c[3 + k], c[6 + k])) + r;
        }
    }
}
void orc_generate_dots(const float* lines, const float* radii, float const_r, int64_t n, float* out) {
    generate_dots(lines, radii, const_r, n, out);
}
void orc_generate_lss(const float* lines, int64_t n, float r, float* pos, float* rad) {
    float lr = fmax_t(r, 0.001f);
    for (int64_t i = 0; i < n; ++i) {
        for (int k = 0; k < 6; ++k) pos[6 * i + k] = lines[6 * i + k];
        rad[2 * i] = lr;
        rad[2 * i + 1] = lr;
    }
}

// Quantised Phantom geometry: the strand vertex stream. A run is a maximal range of lines in
// which each line starts exactly where the previous one ends (the neighbour rule of
// GenerateCurves, geometry_processor.cpp:140-141) with the same radius at the joint. Run r of
// lines [a, b) fills the b - a + 3 entries from a + 3 r: the point before the run (the previous
// line's start when that line ends where the run starts, else the run's own start), the run's
// start, each line's end, and the point after the run (the next line's end when it starts where
// the run ends, else the run's own end); an entry is {x, y, z, radius at the point}, and the two
// outer entries carry the radius of the point beside them. Line i gets entry i + 3 r: entries
// e .. e + 3 are its curve's neighbours p0, p1, p2, p3. Returns the number of entries; `entries`
// holds 4 (n + 3 n) floats at most.
int64_t orc_strand_stream(const float* lines, const float* lrad, int64_t n, float* entries, uint32_t* line_entry) {
    int64_t run = -1;
    auto put = [&](int64_t e, const float* p, float r) {
        entries[4 * e] = p[0]; entries[4 * e + 1] = p[1]; entries[4 * e + 2] = p[2]; entries[4 * e + 3] = r;
    };
    auto joins = [&](int64_t i) {  // line i starts where line i - 1 ends
        return i > 0 && i < n && ld3(lines + 6 * (i - 1) + 3) == ld3(lines + 6 * i);
    };
    for (int64_t i = 0; i < n; ++i) {
        const bool start = !(joins(i) && lrad[2 * i - 1] == lrad[2 * i]);
        if (start) ++run;
        const int64_t e = i + 3 * run;
        line_entry[i] = uint32_t(e);
        const float* L = lines + 6 * i;
        if (start) {
            put(e, joins(i) ? lines + 6 * (i - 1) : L, lrad[2 * i]);
            put(e + 1, L, lrad[2 * i]);
        }
        put(e + 2, L + 3, lrad[2 * i + 1]);
        const bool last = i + 1 == n || !(joins(i + 1) && lrad[2 * i + 1] == lrad[2 * i + 2]);
        if (last) put(e + 3, joins(i + 1) ? lines + 6 * (i + 1) + 3 : L + 3, lrad[2 * i + 1]);
    }
    return n + 3 * (run + 1);
}

// ---- LBVH pipeline (for bit-exact comparison with the device build) -------------------------
void orc_prim_boxes(int type, const float* data, const float* radius, int64_t n, float* boxes_out) {
    for (int64_t i = 0; i < n; ++i) {
        Box b = prim_box(type, data, radius, i);
        std::memcpy(boxes_out + 6 * i, &b, sizeof(Box));
    }
}
// The BVH references' boxes (n << ref_shift_of(type) of them, see ref_boxes); returns their count.
int64_t orc_ref_boxes(int type, const float* data, const float* radius, int64_t n, float* boxes_out) {
    const int sh = ref_shift_of(type);
    for (int64_t i = 0; i < n; ++i) {
        Box b[2];
        ref_boxes(type, data, radius, i, b);
        std::memcpy(boxes_out + (6 << sh) * i, b, sizeof(Box) << sh);
    }
    return n << sh;
}
void orc_morton(const float* boxes, int64_t n, uint64_t* codes) {
    morton_codes(reinterpret_cast<const Box*>(boxes), n, codes);
}
// sorted (n), left/right/first/last/parent (n-1), node boxes (n-1)*6
void orc_lbvh(const float* boxes, int64_t n, uint64_t* codes_sorted, uint32_t* sorted, uint32_t* left,
              uint32_t* right, uint32_t* first, uint32_t* last, uint32_t* parent_int, uint32_t* parent_leaf,
              float* node_boxes) {
    const Box* bx = reinterpret_cast<const Box*>(boxes);
    std::vector<uint64_t> codes(n);
    morton_codes(bx, n, codes.data());
    std::vector<uint32_t> idx(n);
    for (int64_t i = 0; i < n; ++i) idx[i] = uint32_t(i);
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t x, uint32_t y) { return codes[x] < codes[y]; });
    std::vector<uint64_t> sk(n);
    std::vector<Box> sb(n);
    for (int64_t i = 0; i < n; ++i) { sk[i] = codes[idx[i]]; sb[i] = bx[idx[i]]; sorted[i] = idx[i]; codes_sorted[i] = sk[i]; }
    if (n < 2) return;
    Binary bt;
    karras(sk.data(), n, bt);
    refit(bt, sb.data(), n);
    for (int64_t i = 0; i < n - 1; ++i) {
        left[i] = bt.left[i]; right[i] = bt.right[i]; first[i] = bt.first[i]; last[i] = bt.last[i];
        parent_int[i] = bt.parent_int[i];
        std::memcpy(node_boxes + 6 * i, &bt.box[i], sizeof(Box));
    }
    for (int64_t i = 0; i < n; ++i) parent_leaf[i] = bt.parent_leaf[i];
}
// Voxelises n lines (6 floats each) as capsules of radius r on voxel_size cubes: grid_out gets
// origin xyz, size, res xyz (as floats); out receives 7 floats per filled voxel (lo xyz, hi xyz,
// grid index as bits) in ascending grid index, at most max_out. Returns the number of filled
// voxels, -1 when the grid exceeds 2^31 voxels or a line needs more than 2^20 steps.
int64_t orc_voxelize(const float* lines, int64_t n, float r, float voxel_size, float* grid_out, float* out,
                     int64_t max_out) {
    const VoxelGrid g = voxel_grid(lines, n, r, voxel_size);
    for (int k = 0; k < 3; ++k) { grid_out[k] = g.origin[k]; grid_out[4 + k] = float(g.res[k]); }
    grid_out[3] = g.size;
    const int64_t total = int64_t(g.res[0]) * g.res[1] * g.res[2];
    if (n == 0) return 0;
    if (total > (int64_t(1) << 31)) return -1;
    std::vector<uint8_t> filled(size_t(total), 0);
    for (int64_t i = 0; i < n; ++i)
        if (!voxel_line(lines + 6 * i, r, g, filled)) return -1;
    int64_t m = 0;
    const int64_t rx = g.res[0], rxy = int64_t(g.res[0]) * g.res[1];
    for (int64_t i = 0; i < total; ++i) {
        if (!filled[size_t(i)]) continue;
        if (m < max_out) {
            const int64_t xyz[3] = {i % rx, (i / rx) % g.res[1], i / rxy};
            float* o = out + 7 * m;
            for (int k = 0; k < 3; ++k) {
                o[k] = g.origin[k] + float(xyz[k]) * g.size;
                o[3 + k] = o[k] + g.size;
            }
            const uint32_t id = uint32_t(i);
            std::memcpy(o + 6, &id, 4);
        }
        ++m;
    }
    return m;
}
// Collapse; returns the number of wide nodes. Outputs must hold max_nodes entries
// (child_base, prim_base: max_nodes; meta: 8 max_nodes; cbox: 48 max_nodes floats;
// prim_order: n). Quantised fields: qp (3 per node), qe (3), qlo/qhi (24 each).
// max_leaf: primitives per leaf slot (1..3); bits 8-11 the node fan-out W (2..8; 0 = 8).
int64_t orc_bvh8(const float* boxes, int64_t n, int max_leaf, int64_t max_nodes, uint32_t* child_base,
                 uint32_t* prim_base, uint8_t* meta, float* cbox, uint32_t* prim_order, float* qp, uint8_t* qe,
                 uint8_t* qlo, uint8_t* qhi) {
    const int width = (max_leaf >> 8) & 15 ? (max_leaf >> 8) & 15 : 8;
    max_leaf &= 0xff;
    const Box* bx = reinterpret_cast<const Box*>(boxes);
    std::vector<uint64_t> codes(n);
    morton_codes(bx, n, codes.data());
    std::vector<uint32_t> idx(n);
    for (int64_t i = 0; i < n; ++i) idx[i] = uint32_t(i);
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t x, uint32_t y) { return codes[x] < codes[y]; });
    std::vector<uint64_t> sk(n);
    std::vector<Box> sb(n);
    for (int64_t i = 0; i < n; ++i) { sk[i] = codes[idx[i]]; sb[i] = bx[idx[i]]; }
    Binary bt;
    if (n >= 2) { karras(sk.data(), n, bt); refit(bt, sb.data(), n); }
    Wide w;
    collapse(bt, sb.data(), n, max_leaf, width, w);
    int64_t nn = int64_t(w.child_base.size());
    if (nn > max_nodes) return -nn;
    for (int64_t i = 0; i < nn; ++i) {
        child_base[i] = w.child_base[i];
        prim_base[i] = w.prim_base[i];
        for (int q = 0; q < 8; ++q) {
            meta[8 * i + q] = w.meta[8 * i + q];
            std::memcpy(cbox + 48 * i + 6 * q, &w.cbox[8 * i + q], sizeof(Box));
        }
        quantise_node(&w.cbox[8 * i], &w.meta[8 * i], qp + 3 * i, qe + 3 * i, qlo + 24 * i, qhi + 24 * i);
    }
    for (size_t i = 0; i < w.prim_order.size(); ++i) prim_order[i] = idx[w.prim_order[i]];
    return nn;
}

// ---- scenes and tracing -----------------------------------------------------------------
void* orc_scene_create() { return new Scene(); }
void orc_scene_destroy(void* s) { delete static_cast<Scene*>(s); }
// type: 0 Phantom (data 12 floats/prim, radius 2/prim), 1 LSS (6, 2), 2 DOTS (36, unused),
// 3 mesh (9 floats/triangle; "radius" = 9 vertex-normal floats per triangle, or null).
// Returns the BLAS index.
int orc_scene_add_blas(void* s, int type, int64_t nprim, const float* data, const float* radius) {
    Scene* sc = static_cast<Scene*>(s);
    Blas b;
    b.type = type;
    b.nprim = nprim;
    int per = type == kPhantom ? 12 : (type == kLss ? 6 : (type == kMesh ? 9 : (type == kVoxel ? 7 : 36)));
    b.data.assign(data, data + per * nprim);
    if (type == kMesh) {
        if (radius) b.radius.assign(radius, radius + 9 * nprim);  // vertex normals per triangle
    } else if (type != kDots && type != kVoxel) {
        b.radius.assign(radius, radius + 2 * nprim);
    }
    build_blas(b);
    sc->blas.push_back(std::move(b));
    return int(sc->blas.size() - 1);
}
// xf: object-to-world, column major, or null for identity.
int orc_scene_add_instance(void* s, int blas, const float* xf) {
    Scene* sc = static_cast<Scene*>(s);
    Instance in;
    in.blas = blas;
    in.identity = xf == nullptr;
    for (int k = 0; k < 16; ++k) in.xf[k] = xf ? double(xf[k]) : ((k % 5) == 0 ? 1.0 : 0.0);
    shim::tmat4<double> m;
    for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) m[c][k] = in.xf[c * 4 + k];
    shim::tmat4<double> iv = shim::inverse(m);
    for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) in.inv[c * 4 + k] = iv[c][k];
    sc->inst.push_back(in);
    return int(sc->inst.size() - 1);
}

// Material of a mesh BLAS: albedo factor (4 floats), and with a map (w x h RGBA floats, row 0 at
// v = 0) the texture coordinates of each triangle (6 floats: u0 v0 u1 v1 u2 v2). Returns 0, or -1
// when the BLAS is not a mesh.
int orc_scene_set_material(void* s, int blas, const float* albedo4, const float* uv, const float* map, uint32_t w,
                           uint32_t h) {
    Blas& b = static_cast<Scene*>(s)->blas[blas];
    if (b.type != kMesh) return -1;
    for (int k = 0; k < 4; ++k) b.albedo[k] = albedo4[k];
    b.uv.clear();
    b.map.clear();
    b.map_w = b.map_h = 0;
    if (uv && map && w && h) {
        b.uv.assign(uv, uv + 6 * b.nprim);
        b.map.assign(map, map + size_t(w) * h * 4);
        b.map_w = w;
        b.map_h = h;
    }
    return 0;
}

// Closest hit for explicit rays (o[3], d[3] per ray, FP32 inputs).
// precision: 32 = FP32, 64 = FP64, 3264 = FP32 with FP64 re-solve of unresolved candidates.
// Outputs per ray: t (double, -1 miss), prim, inst, normal (3 doubles).
void orc_trace_rays(void* s, const float* rays, int64_t n, float tmin, float tmax, int precision, int nthreads,
                    double* t_out, uint32_t* prim_out, uint32_t* inst_out, double* n_out) {
    const Scene& sc = *static_cast<Scene*>(s);
    parallel_for(n, nthreads, [&](int64_t i) {
        const float* r = rays + 6 * i;
        if (precision % 1000000 == 64 || precision % 1000000 == 6400) {
            HitT<double> h;
            bool f = trace_one<double>(sc, tvec3<double>(r[0], r[1], r[2]), tvec3<double>(r[3], r[4], r[5]), double(tmin),
                                       double(tmax), false, 0, 0, fp64_mode(precision), &h);
            t_out[i] = f ? h.t : -1.0;
            prim_out[i] = f ? h.prim : 0xffffffffu;
            inst_out[i] = f ? h.inst : 0xffffffffu;
            for (int k = 0; k < 3; ++k) n_out[3 * i + k] = f ? h.n[k] : 0.0;
        } else {
            HitT<float> h;
            bool f = trace_one<float>(sc, v3f(r[0], r[1], r[2]), v3f(r[3], r[4], r[5]), tmin, tmax, false, 0, 0,
                                      fp32_mode(precision), &h);
            t_out[i] = f ? double(h.t) : -1.0;
            prim_out[i] = f ? h.prim : 0xffffffffu;
            inst_out[i] = f ? h.inst : 0xffffffffu;
            for (int k = 0; k < 3; ++k) n_out[3 * i + k] = f ? double(h.n[k]) : 0.0;
        }
    });
}

// Render W x H x spp. Shading: 0 debug colour (the reference's closest-hit output), 1 Shade(n),
// 2 Shade(n) with one shadow ray toward +y (light direction (0,-1,0)), skipping the hit
// segment, from the hit point with tmin = shadow_tmin.
// Jitter: spp == 1 and jitter == 0 uses the pixel centre 0.5 (ray_gen.rgen:18); otherwise the
// offset of sample k of pixel p is (h1 >> 8) * 2^-24, (h2 >> 8) * 2^-24 with
// h1 = hash(seed ^ hash(p * spp + k)), h2 = hash(h1).
// Pixels: first_pixel .. first_pixel + npixels - 1, or pixel_list[0 .. npixels-1] when given.
// Per-sample outputs (npixels*spp): t (double, -1 miss), prim, inst, shadow flag;
// framebuffer npixels*4 floats (RGBA, A = 1), averaged over samples in sample order.
// miss.rmiss:17-37: the environment along -d (equirectangular DirectionToUV), bilinear with u
// repeating and v clamped to the edge rows (texel centres at (i + 0.5) / size), then
// 1 - exp(-c) and gamma 1/2.2. env: RGBA float texels, ew x eh, row 0 at v = 0.
extern "C++" template <class T>
void env_color(const float* env, uint32_t ew, uint32_t eh, const T d[3], T out[3]) {
    T n = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    T v[3] = {-d[0] / n, -d[1] / n, -d[2] / n};
    const T k1OverPi = T(0.3183098861837);
    T gamma = std::asin(std::min(std::max(v[1], T(-1)), T(1))), theta = std::atan2(v[0], -v[2]);
    T u = theta * k1OverPi * T(0.5) + T(0.5), vv = gamma * k1OverPi + T(0.5);
    T x = u * T(ew) - T(0.5), y = vv * T(eh) - T(0.5);
    T fx = std::floor(x), fy = std::floor(y), ax = x - fx, ay = y - fy;
    int64_t x0 = int64_t(fx) % int64_t(ew);
    if (x0 < 0) x0 += ew;
    int64_t x1 = (x0 + 1) % int64_t(ew);
    int64_t y0 = std::min<int64_t>(std::max<int64_t>(int64_t(fy), 0), eh - 1);
    int64_t y1 = std::min<int64_t>(std::max<int64_t>(int64_t(fy) + 1, 0), eh - 1);
    for (int k = 0; k < 3; ++k) {
        T c00 = env[4 * (y0 * ew + x0) + k], c10 = env[4 * (y0 * ew + x1) + k];
        T c01 = env[4 * (y1 * ew + x0) + k], c11 = env[4 * (y1 * ew + x1) + k];
        T a = c00 + ax * (c10 - c00), b = c01 + ax * (c11 - c01);
        T c = a + ay * (b - a);
        out[k] = std::pow(T(1) - std::exp(-c), T(1) / T(2.2));
    }
}

// triangle_closest_hit.rchit:71-81, restated: a mesh hit's albedo, the factor times the map at
// the texture coordinate interpolated with the hit's barycentrics (1 - u - v, u, v); bilinear,
// repeat addressing (the coordinate wrapped into [0, 1) first), texel centres at (i + 0.5) / size.
extern "C++" template <class T> tvec3<T> mesh_albedo(const Blas& b, const HitT<T>& hh) {
    tvec3<T> a(T(b.albedo[0]), T(b.albedo[1]), T(b.albedo[2]));
    if (b.map.empty() || b.uv.empty()) return a;
    const float* q = b.uv.data() + 6 * size_t(hh.prim);
    const T u = hh.u, v = hh.v, w = T(1) - u - v;
    T s = w * T(q[0]) + u * T(q[2]) + v * T(q[4]);
    T t = w * T(q[1]) + u * T(q[3]) + v * T(q[5]);
    s -= std::floor(s);
    t -= std::floor(t);
    const int64_t W = b.map_w, H = b.map_h;
    const T x = s * T(W) - T(0.5), y = t * T(H) - T(0.5);
    const T fx = std::floor(x), fy = std::floor(y), ax = x - fx, ay = y - fy;
    const int64_t x0 = fx >= T(0) ? std::min<int64_t>(int64_t(fx), W - 1) : W - 1;
    const int64_t y0 = fy >= T(0) ? std::min<int64_t>(int64_t(fy), H - 1) : H - 1;
    const int64_t x1 = x0 + 1 == W ? 0 : x0 + 1, y1 = y0 + 1 == H ? 0 : y0 + 1;
    T c[3];
    for (int k = 0; k < 3; ++k) {
        const T c00 = b.map[4 * (y0 * W + x0) + k], c10 = b.map[4 * (y0 * W + x1) + k];
        const T c01 = b.map[4 * (y1 * W + x0) + k], c11 = b.map[4 * (y1 * W + x1) + k];
        const T lo = c00 + ax * (c10 - c00), hi = c01 + ax * (c11 - c01);
        c[k] = lo + ay * (hi - lo);
    }
    return tvec3<T>(a.x * c[0], a.y * c[1], a.z * c[2]);
}

void orc_render(void* s, const float* view_inv, const float* proj_inv, uint32_t w, uint32_t h, uint32_t spp,
                int jitter, uint32_t seed, float tmin, float tmax, int shading, float shadow_tmin, int precision,
                int nthreads, int64_t first_pixel, int64_t npixels, const uint32_t* pixel_list, double* t_out,
                uint32_t* prim_out, uint32_t* inst_out, uint8_t* shadow_out, float* fb, const float* env,
                uint32_t env_w, uint32_t env_h) {
    const Scene& sc = *static_cast<Scene*>(s);
    parallel_for(npixels, nthreads, [&](int64_t pi) {
        int64_t p = pixel_list ? int64_t(pixel_list[pi]) : first_pixel + pi;
        uint32_t px = uint32_t(p % w), py = uint32_t(p / w);
        double acc[3] = {0, 0, 0};
        float accf[3] = {0, 0, 0};
        for (uint32_t k = 0; k < spp; ++k) {
            float jx = 0.5f, jy = 0.5f;
            if (jitter || spp > 1) {
                uint32_t h1 = hash_u32(seed ^ hash_u32(uint32_t(p) * spp + k));
                uint32_t h2 = hash_u32(h1);
                jx = float(h1 >> 8) * 5.9604644775390625e-08f;
                jy = float(h2 >> 8) * 5.9604644775390625e-08f;
            }
            float o[3], d[3];
            orc_raygen_f32(view_inv, proj_inv, px, py, w, h, jx, jy, o, d);
            int64_t si = pi * spp + k;
            double col[3] = {0, 0, 0};
            bool found;
            uint32_t sh = 0;
            if (precision % 1000000 == 64 || precision % 1000000 == 6400) {
                HitT<double> hh;
                tvec3<double> od(o[0], o[1], o[2]), dd(d[0], d[1], d[2]);
                found = trace_one<double>(sc, od, dd, tmin, tmax, false, 0, 0, fp64_mode(precision), &hh);
                t_out[si] = found ? hh.t : -1.0;
                prim_out[si] = found ? hh.prim : 0xffffffffu;
                inst_out[si] = found ? hh.inst : 0xffffffffu;
                if (found) {
                    if (shading == 0) for (int c = 0; c < 3; ++c) col[c] = kPalette[hh.prim % 6][c];
                    else {
                        bool lit = true;
                        if (shading == 2) {
                            tvec3<double> hp = od + hh.t * dd;
                            HitT<double> sh2;
                            lit = !trace_one<double>(sc, hp, tvec3<double>(0.0, 1.0, 0.0), double(shadow_tmin), double(tmax),
                                                     true, hh.inst, hh.seg, fp64_mode(precision), &sh2);
                        }
                        sh = lit ? 0 : 1;
                        tvec3<double> c3 = lit ? shade(hh.n) : tvec3<double>(0.3f, 0.3f, 0.3f);
                        const Blas& hb = sc.blas[sc.inst[hh.inst].blas];
                        if (hb.type == kMesh) {
                            const tvec3<double> a = mesh_albedo(hb, hh);
                            c3 = tvec3<double>(c3.x * a.x, c3.y * a.y, c3.z * a.z);
                        }
                        col[0] = c3.x; col[1] = c3.y; col[2] = c3.z;
                    }
                } else if (env) {
                    const double dv[3] = {double(d[0]), double(d[1]), double(d[2])};
                    env_color(env, env_w, env_h, dv, col);
                }
                for (int c = 0; c < 3; ++c) acc[c] += col[c];
            } else {
                HitT<float> hh;
                v3f od(o[0], o[1], o[2]), dd(d[0], d[1], d[2]);
                found = trace_one<float>(sc, od, dd, tmin, tmax, false, 0, 0, fp32_mode(precision), &hh);
                t_out[si] = found ? double(hh.t) : -1.0;
                prim_out[si] = found ? hh.prim : 0xffffffffu;
                inst_out[si] = found ? hh.inst : 0xffffffffu;
                float cf[3] = {0, 0, 0};
                if (found) {
                    if (shading == 0) for (int c = 0; c < 3; ++c) cf[c] = kPalette[hh.prim % 6][c];
                    else {
                        bool lit = true;
                        if (shading == 2) {
                            v3f hp = od + hh.t * dd;
                            HitT<float> sh2;
                            lit = !trace_one<float>(sc, hp, v3f(0.f, 1.f, 0.f), shadow_tmin, tmax, true, hh.inst, hh.seg,
                                                    fp32_mode(precision), &sh2);
                        }
                        sh = lit ? 0 : 1;
                        v3f c3 = lit ? shade(hh.n) : v3f(0.3f, 0.3f, 0.3f);
                        const Blas& hb = sc.blas[sc.inst[hh.inst].blas];
                        if (hb.type == kMesh) {
                            const v3f a = mesh_albedo(hb, hh);
                            c3 = v3f(c3.x * a.x, c3.y * a.y, c3.z * a.z);
                        }
                        cf[0] = c3.x; cf[1] = c3.y; cf[2] = c3.z;
                    }
                } else if (env) {
                    env_color(env, env_w, env_h, d, cf);
                }
                for (int c = 0; c < 3; ++c) accf[c] += cf[c];
            }
            shadow_out[si] = uint8_t(sh);
        }
        float* px4 = fb + 4 * pi;
        if (precision % 1000000 == 64 || precision % 1000000 == 6400) for (int c = 0; c < 3; ++c) px4[c] = float(acc[c] / double(spp));
        else for (int c = 0; c < 3; ++c) px4[c] = accf[c] * (1.0f / float(spp));
        px4[3] = 1.0f;
    });
}

int orc_hardware_threads() { return int(std::thread::hardware_concurrency()); }
void orc_resolve_stats(int64_t* out4, int reset) {
    for (int k = 0; k < 4; ++k) { out4[k] = g_stat[k].load(); if (reset) g_stat[k] = 0; }
}

}  // extern "C"
