// trace_device.cuh -- device code of the trace pass (included by trace.cu and by the two
// compilations of trace_frames.cu): ray generation, BVH8 traversal, the three hair
// intersectors, closest-hit shading and the shadow ray, the persistent frame kernel and its
// launch helpers. Everything is in an anonymous namespace, so each translation unit
// instantiates only the kernels it launches.
//
// Replaces ray_gen.rgen:16-48 -> traceRayEXT (RT-core traversal) -> hair_intersection.rint /
// hardware LSS and triangle tests -> hair_closest_hit.rchit / triangle_closest_hit.rchit ->
// miss.rmiss (constant black background, the payload's initial value ray_gen.rgen:30).
//
// Work: warps take 32 work items at a time from a global counter; 32 consecutive items are one
// 8x4 pixel tile of one scene, so a warp's rays are coherent. Each thread traces all samples
// of its pixel (primary ray, shading, shadow ray) and writes the averaged pixel.
// Traversal (frame kernel): children sit in slots by direction, so a ray visits the hit
// children of a node in the order i ^ octant(ray) without sorting; the stack holds node groups
// (child_base, hit bits, internal-child mask) and parked leaf groups, one entry per visited
// node at most. The explicit-ray kernel keeps a per-thread stack of (reference, entry
// distance) with the hits of a node sorted by a sorting network. All waits are bounded: a full
// stack (the launch's max_depth entries, at most kStackSize) or more than the launch's max_steps
// traversal steps ends the ray and sets a bit in the device error word.
#pragma once
#include <cuda_fp16.h>

#include <mutex>
#include <type_traits>

#include "hrt_internal.h"

namespace hrt {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kThreads = 128;

// ---------------------------------------------------------------- small vector helpers
template <class T> struct V3 { T x, y, z; };
template <class T> __device__ __forceinline__ V3<T> mk(T x, T y, T z) { return {x, y, z}; }
template <class T> __device__ __forceinline__ V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> __device__ __forceinline__ V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> __device__ __forceinline__ V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> __device__ __forceinline__ T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> __device__ __forceinline__ V3<T> cross(V3<T> x, V3<T> y) {
    return {x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y};
}
__device__ __forceinline__ float rsq(float x) { return 1.0f / sqrtf(x); }
__device__ __forceinline__ double rsq(double x) { return 1.0 / sqrt(x); }
template <class T> __device__ __forceinline__ V3<T> normalize(V3<T> v) { return rsq(dot(v, v)) * v; }
template <class T> __device__ __forceinline__ T length(V3<T> v) { return sqrt(dot(v, v)); }
template <class T> __device__ __forceinline__ T gmin(T x, T y) { return (y < x) ? y : x; }  // glm order
template <class T> __device__ __forceinline__ T gmax(T x, T y) { return (x < y) ? y : x; }
template <class T> __device__ __forceinline__ T gabs(T x) { return x >= T(0) ? x : -x; }

// Explicitly rounded forms (fixed fused multiply-adds, no contraction left to the compiler),
// for values that must not depend on how a kernel variant is compiled: instance transforms,
// normals, shading.
__device__ __forceinline__ float dot_rn(V3<float> a, V3<float> b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, __fmul_rn(a.x, b.x))); }
__device__ __forceinline__ V3<float> normalize_rn(V3<float> v) {
    const float k = __fdiv_rn(1.0f, __fsqrt_rn(dot_rn(v, v)));
    return mk(__fmul_rn(k, v.x), __fmul_rn(k, v.y), __fmul_rn(k, v.z));
}
__device__ __forceinline__ V3<float> cross_rn(V3<float> x, V3<float> y) {
    return mk(fmaf(x.y, y.z, -__fmul_rn(y.y, x.z)), fmaf(x.z, y.x, -__fmul_rn(y.z, x.x)), fmaf(x.x, y.y, -__fmul_rn(y.x, x.y)));
}
// rows of a 3x4 affine matrix applied to a point / a direction
__device__ __forceinline__ V3<float> xform_point(const float* m, V3<float> p) {
    return mk(fmaf(m[2], p.z, fmaf(m[1], p.y, fmaf(m[0], p.x, m[3]))), fmaf(m[6], p.z, fmaf(m[5], p.y, fmaf(m[4], p.x, m[7]))),
              fmaf(m[10], p.z, fmaf(m[9], p.y, fmaf(m[8], p.x, m[11]))));
}
__device__ __forceinline__ V3<float> xform_dir(const float* m, V3<float> v) {
    return mk(fmaf(m[2], v.z, fmaf(m[1], v.y, __fmul_rn(m[0], v.x))), fmaf(m[6], v.z, fmaf(m[5], v.y, __fmul_rn(m[4], v.x))),
              fmaf(m[10], v.z, fmaf(m[9], v.y, __fmul_rn(m[8], v.x))));
}

// ---------------------------------------------------------------- Phantom (Prhi)
// curve.glsl:9-31
template <class T> __device__ __forceinline__ V3<T> bez_point(const V3<T>* c, T t) {
    T u = T(1) - t, tt = t * t, uu = u * u;
    T uuu = uu * u, ttt = tt * t;
    return uuu * c[0] + (T(3) * uu * t) * c[1] + (T(3) * u * tt) * c[2] + ttt * c[3];
}
template <class T> __device__ __forceinline__ V3<T> bez_axis(const V3<T>* c, T t) {
    T u = T(1) - t;
    return (T(-3) * u * u) * c[0] + (T(3) * (T(3) * t * t - T(4) * t + T(1))) * c[1] +
           (T(3) * (T(2) - T(3) * t) * t) * c[2] + (T(3) * t * t) * c[3];
}
// The quotients of the FP32 Phantom solve use the fast division (__fdividef, within 2 ulp):
// the solve's results differ from the FP64 solve by far more than that, and the FP64 pass
// re-solves the candidates whose FP32 iteration does not converge. FP64 divides exactly.
template <class T> __device__ __forceinline__ T prhi_div(T a, T b) { return a / b; }
template <> __device__ __forceinline__ float prhi_div<float>(float a, float b) { return __fdividef(a, b); }
// Square roots of the FP32 intersectors: the approximate root of PTX (sqrt.approx.f32), which
// left the hit ids, distances and colours of the FP32 solves against the FP64 solve as they were
// with the IEEE root (0 mismatches on the sampled rays of a 3.15 M-segment LSS frame, a
// 19 M-segment Phantom frame and a 16-scene batch); FP64 takes the exact root.
template <class T> __device__ __forceinline__ T prhi_sqrt(T x) { return sqrt(x); }
template <> __device__ __forceinline__ float prhi_sqrt<float>(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
// cylinder.glsl:8-46 (capped cylinder, boolean; no range test on t)
template <class T> __device__ __forceinline__ bool ray_cylinder(V3<T> o, V3<T> d, V3<T> p0, V3<T> p1, T r) {
    V3<T> ba = p1 - p0, oc = o - p0;
    T baba = dot(ba, ba), bard = dot(ba, d), baoc = dot(ba, oc);
    T k2 = baba - bard * bard;
    T k1 = baba * dot(oc, d) - baoc * bard;
    T k0 = baba * dot(oc, oc) - baoc * baoc - r * r * baba;
    T h = k1 * k1 - k2 * k0;
    if (h < T(0)) return false;
    h = prhi_sqrt(h);
    T t = prhi_div(-k1 - h, k2);
    T y = baoc + t * bard;
    if (y > T(0) && y < baba) return true;
    t = prhi_div((y < T(0) ? T(0) : baba) - baoc, bard);
    return gabs(k1 + k2 * t) < h;
}

// ray_cylinder for a ray through the origin and the cylinder p0 .. p0 + ba, with baba = |ba|^2
// given (FP32 Phantom early-out, on coordinates relative to the ray's reference point)
__device__ __forceinline__ bool ray_cylinder0(V3<float> d, V3<float> p0, V3<float> ba, float baba, float r) {
    const float bard = dot(ba, d), baoc = -dot(ba, p0);
    const float k2 = baba - bard * bard;
    const float k1 = -baba * dot(p0, d) - baoc * bard;
    const float k0 = baba * dot(p0, p0) - baoc * baoc - r * r * baba;
    float h = k1 * k1 - k2 * k0;
    if (h < 0.0f) return false;
    h = prhi_sqrt(h);
    float t = prhi_div(-k1 - h, k2);
    const float y = baoc + t * bard;
    if (y > 0.0f && y < baba) return true;
    t = prhi_div((y < 0.0f ? 0.0f : baba) - baoc, bard);
    return fabsf(k1 + k2 * t) < h;
}

// The cubic in power form, C3 t^3 + C2 t^2 + C1 t + C0, and its derivative
// (3 C3 t + 2 C2) t + C1 = (C3 (1.5 t) + C2) (2 t) + C1, by Horner's rule.
template <class T> __device__ __forceinline__ void power_eval(const V3<T>* C, T t, V3<T>& c, V3<T>& ax) {
    const T t15 = T(1.5) * t, t2 = t + t;
    c = mk(fma(fma(fma(C[3].x, t, C[2].x), t, C[1].x), t, C[0].x), fma(fma(fma(C[3].y, t, C[2].y), t, C[1].y), t, C[0].y),
           fma(fma(fma(C[3].z, t, C[2].z), t, C[1].z), t, C[0].z));
    ax = mk(fma(fma(C[3].x, t15, C[2].x), t2, C[1].x), fma(fma(C[3].y, t15, C[2].y), t2, C[1].y),
            fma(fma(C[3].z, t15, C[2].z), t2, C[1].z));
}
// FP32: x and y in packed pairs (each half rounds exactly as fmaf, so the values are the same)
__device__ __forceinline__ void power_eval(const V3<float>* C, float t, V3<float>& c, V3<float>& ax) {
    const float t15 = 1.5f * t, t2 = t + t;
    const float2 tt = make_float2(t, t), tt15 = make_float2(t15, t15), tt2 = make_float2(t2, t2);
    const float2 c0 = make_float2(C[0].x, C[0].y), c1 = make_float2(C[1].x, C[1].y);
    const float2 c2 = make_float2(C[2].x, C[2].y), c3 = make_float2(C[3].x, C[3].y);
    const float2 pxy = __ffma2_rn(__ffma2_rn(__ffma2_rn(c3, tt, c2), tt, c1), tt, c0);
    const float2 axy = __ffma2_rn(__ffma2_rn(c3, tt15, c2), tt2, c1);
    c = mk(pxy.x, pxy.y, fmaf(fmaf(fmaf(C[3].z, t, C[2].z), t, C[1].z), t, C[0].z));
    ax = mk(axy.x, axy.y, fmaf(fmaf(C[3].z, t15, C[2].z), t2, C[1].z));
}

// kUnresolved: no hit, and a side used all 8 iterations inside [0, 1] with a real cone
// intersection at its last step (det > 0 but |dt| >= 5e-5): the FP32 run failed its
// convergence test. Runs that exhaust without an intersection are misses.
enum { kMiss = 0, kHit = 1, kUnresolved = 2 };
template <class T> struct PrhiOut {  // s = ts + sl
    T s; T sl; T ts; T tc; int status;
};

// ray.glsl:13-17 MakeOrthonormalBasis; the RCC transform (ray.glsl:19-33) is the inverse of
// [e1 e2 e3 | o], applied here as the transpose of the orthonormal frame after the translation.
// inv_len = 1 / |d|: distances along e3 are lengths, the ray's parameter is length / |d| (the
// object-space direction of a scaled instance is not a unit vector).
template <class T> struct Frame { V3<T> e1, e2, e3; T inv_len; };
template <class T> __device__ __forceinline__ Frame<T> make_frame(V3<T> d) {
    Frame<T> f;
    f.inv_len = rsq(dot(d, d));
    f.e3 = f.inv_len * d;
    V3<T> w = f.e3;
    f.e2 = gabs(w.x) > gabs(w.y) ? normalize(mk(-w.z, T(0), w.x)) : normalize(mk(T(0), w.z, -w.y));
    f.e1 = cross(f.e2, w);
    return f;
}

// a - b - ts * d to full precision: a - b exactly by TwoSum, then one fused multiply-add.
template <class T> __device__ __forceinline__ T rel_coord(T a, T b, T ts, T d) {
    T c = -b;
    T sum = a + c;
    T cc = sum - a;
    T err = (a - (sum - cc)) + (c - cc);
    return fma(-ts, d, sum) + err;
}

// hair_intersection.rint:15-130 with the cone radius r0 + (r1 - r0) t (constant when equal).
// The solve runs from o' = o + ts d, the ray point nearest the chord midpoint, on the vectors
// P - o' (o' itself is never rounded); ts is added back to the distance. The result is the
// same in exact arithmetic; in FP32 it removes the cancellation of the world-space
// bounding-cylinder test from a distant origin (hair_intersection.rint:29). The bounding radius
// is sqrt(|cross|^2 / |chord|^2) (one root instead of two), and the Newton iteration evaluates
// the Bezier point and tangent from the power form of the control points (Horner's rule,
// power_eval) instead of the Bernstein weights of curve.glsl: the same polynomials, in fewer
// operations. prhi_solve is the iteration on the control points relative to o' (W), with
// out.ts holding the distance of o' along the ray.
template <class T>
__device__ __forceinline__ PrhiOut<T> prhi_solve(const Frame<T>& F, const V3<T>* W, T r0, T r1, PrhiOut<T> out) {
    V3<T> Q[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) Q[k] = mk(dot(F.e1, W[k]), dot(F.e2, W[k]), dot(F.e3, W[k]));
    V3<T> PC[4] = {Q[0], T(3) * (Q[1] - Q[0]), T(3) * ((Q[0] - Q[1]) + (Q[2] - Q[1])), (Q[3] - Q[0]) + T(3) * (Q[1] - Q[2])};
    T tStart = (Q[3].z - Q[0].z) > T(0) ? T(0) : T(1);
    bool unresolved = false;
    for (int side = 0; side < 2; ++side) {
        T t = tStart, told = T(0), dt1 = T(0), dt2 = T(0);
        bool exhausted = true, last_isect = false;
        for (int i = 0; i < 8; ++i) {
            V3<T> c, ax;
            power_eval(PC, t, c, ax);
            T rad = (r0 == r1) ? r0 : r0 + (r1 - r0) * t;
            // cone.glsl:21-62 with slant 0
            T ddd = ax.x * ax.x + ax.y * ax.y;
            T dp = c.x * c.x + c.y * c.y;
            T cdd = c.x * ax.x + c.y * ax.y;
            T cxd = c.x * ax.y - c.y * ax.x;
            T cc = ddd;
            T b = ax.z * (-cdd);
            T cdz2 = ax.z * ax.z;
            ddd += cdz2;
            T a = cxd * cxd - ddd * (rad * rad) + dp * cdz2;
            T det = b * b - a * cc;
            bool isect = det > T(0);
            last_isect = isect;
            T s = prhi_div(b - (isect ? prhi_sqrt(det) : T(0)), cc);
            T dt = prhi_div(s * ax.z - cdd, ddd);
            if (isect && gabs(dt) < T(5e-5)) {
                out.sl = (s + c.z) * F.inv_len;  // length along e3 -> the ray's parameter
                out.s = out.sl + out.ts;
                out.tc = t;
                exhausted = false;
                break;
            }
            dt = gmin(dt, T(0.5));
            dt = gmax(dt, T(-0.5));
            dt1 = dt2;
            dt2 = dt;
            if (dt1 * dt2 < T(0)) {
                T tnext = ((i & 3) == 0) ? T(0.5) * (told + t) : prhi_div(dt2 * told - dt1 * t, dt2 - dt1);
                told = t;
                t = tnext;
            } else {
                told = t;
                t += dt;
            }
            if (t < T(0) || t > T(1)) { exhausted = false; break; }
        }
        unresolved |= exhausted && last_isect;
        if (out.s > T(0)) break;
        tStart = T(1) - tStart;
    }
    out.status = out.s > T(0) ? kHit : (unresolved ? kUnresolved : kMiss);
    return out;
}

// FP32 prhi from P0 and the control-point differences D1 = P1 - P0, D2 = P2 - P0, ch = P3 - P0:
// P0 - o' exactly, the other points as (P0 - o') + D (rounded at the scale of a segment, not of
// the camera distance: 3 exact relative coordinates instead of 12). With
// mid - P0 = (3 D1 + 3 D2 + ch) / 8 the bounding radius's |(mid - P0) x (mid - P3)| is
// (3/8) |ch x (D1 + D2)|.
__device__ __forceinline__ PrhiOut<float> prhi_diff(const Frame<float>& F, V3<float> o, V3<float> d, V3<float> P0,
                                                    V3<float> D1, V3<float> D2, V3<float> ch, float r0, float r1) {
    PrhiOut<float> out{0.0f, 0.0f, 0.0f, 0.0f, kMiss};
    const V3<float> cm = mk(fmaf(0.5f, ch.x, P0.x), fmaf(0.5f, ch.y, P0.y), fmaf(0.5f, ch.z, P0.z));
    const float ts = dot(cm - o, d) * (F.inv_len * F.inv_len);
    out.ts = ts;
    const V3<float> cr = cross(ch, D1 + D2);
    const float chch = dot(ch, ch);
    const float rmax = 0.375f * prhi_sqrt(prhi_div(dot(cr, cr), chch)) + gmax(r0, r1);
    V3<float> W[4];
    W[0] = mk(rel_coord(P0.x, o.x, ts, d.x), rel_coord(P0.y, o.y, ts, d.y), rel_coord(P0.z, o.z, ts, d.z));
    // the capped-cylinder test (cylinder.glsl) takes a unit direction: e3, the ray's own for a
    // unit d, the normalised object-space direction of a scaled instance
    if (!ray_cylinder0(F.e3, W[0], ch, chch, rmax)) return out;
    W[1] = W[0] + D1;
    W[2] = W[0] + D2;
    W[3] = W[0] + ch;
    return prhi_solve(F, W, r0, r1, out);
}

// hair_intersection.rint:15-130 on the four control points (FP64: every relative coordinate
// exact; FP32: prhi_diff)
template <class T>
__device__ __forceinline__ PrhiOut<T> prhi(const Frame<T>& F, V3<T> o, V3<T> d, const V3<T>* P, T r0, T r1) {
    if constexpr (std::is_same<T, float>::value) {
        return prhi_diff(F, o, d, P[0], P[1] - P[0], P[2] - P[0], P[3] - P[0], r0, r1);
    } else {
        PrhiOut<T> out{T(0), T(0), T(0), T(0), kMiss};
        V3<T> cm = T(0.5) * (P[0] + P[3]);
        T ts = dot(cm - o, d) * (F.inv_len * F.inv_len);
        out.ts = ts;
        // the end points first: the bounding-cylinder early-out needs only them
        V3<T> W[4];
        V3<T> mid = bez_point(P, T(0.5));
        const V3<T> cr = cross(mid - P[0], mid - P[3]), ch = P[3] - P[0];
        T rmax = prhi_sqrt(prhi_div(dot(cr, cr), dot(ch, ch))) + gmax(r0, r1);
#pragma unroll
        for (int k = 0; k < 4; k += 3)
            W[k] = mk(rel_coord(P[k].x, o.x, ts, d.x), rel_coord(P[k].y, o.y, ts, d.y), rel_coord(P[k].z, o.z, ts, d.z));
        if (!ray_cylinder(mk(T(0), T(0), T(0)), F.e3, W[0], W[3], rmax)) return out;
#pragma unroll
        for (int k = 1; k < 3; ++k)
            W[k] = mk(rel_coord(P[k].x, o.x, ts, d.x), rel_coord(P[k].y, o.y, ts, d.y), rel_coord(P[k].z, o.z, ts, d.z));
        return prhi_solve(F, W, r0, r1, out);
    }
}

// FP64 re-solve of one candidate, kept out of line so the FP32 path keeps its registers.
__device__ __noinline__ void prhi_fp64(float ox, float oy, float oz, float dx, float dy, float dz, const float* cp,
                                       float r0, float r1, double* s_out, double* sl_out, double* ts_out,
                                       double* tc_out) {
    V3<double> o = mk(double(ox), double(oy), double(oz)), d = mk(double(dx), double(dy), double(dz));
    Frame<double> F = make_frame(d);
    V3<double> P[4];
    for (int k = 0; k < 4; ++k) P[k] = mk(double(cp[3 * k]), double(cp[3 * k + 1]), double(cp[3 * k + 2]));
    PrhiOut<double> r = prhi(F, o, d, P, double(r0), double(r1));
    *s_out = r.status == kHit ? r.s : -1.0;
    *sl_out = r.sl;
    *ts_out = r.ts;
    *tc_out = r.tc;
}

// ---------------------------------------------------------------- LSS (round cone)
// Envelope of spheres a + u (b-a), radius ra + u (rb-ra): tangent-cone roots with u in [0,1]
// and both end spheres; the least t >= tmin wins. Solved from o' = o + ts d (the ray point
// nearest the segment midpoint) on a - o' at full precision and b - o' = (a - o') + (b - a);
// t = ts + t'.
// Quadratic coefficients are formed with cross products (Lagrange's identity) so that no term
// is the small difference of two large ones: for the sphere, h = r^2 |d|^2 - |oc x d|^2.
// Quotients by a reciprocal from the fast division (within 2 ulp); the hit distances stay
// within the FP32 tolerance of the FP64 round-cone solve.
__device__ __forceinline__ float lss_rcp(float x) { return __fdividef(1.0f, x); }
__device__ __forceinline__ float sphere_hit(V3<float> oc, V3<float> d, float r, float tmin, float best) {
    float A = dot(d, d), B = dot(oc, d);
    V3<float> c = cross(oc, d);
    float h = r * r * A - dot(c, c);
    if (h < 0.0f) return best;
    float sh = prhi_sqrt(h);
    const float iA = lss_rcp(A);
    float t0 = (-B - sh) * iA, t1 = (-B + sh) * iA;
    if (t0 >= tmin && t0 < best) return t0;
    if (t1 >= tmin && t1 < best) return t1;
    return best;
}
// Tangent cone: m |P-a|^2 - (y + ra dr)^2 - m ra^2 = 0 with y = (b-a).(P-a), m = L^2 - dr^2;
// with c1 = ba x oa and c2 = ba x d the quadratic A t^2 + 2 B t + C has
//   A = |c2|^2 - dr^2 |d|^2,  B = c1.c2 - dr^2 (oa.d) - ra dr (ba.d),
//   C = |c1|^2 - dr^2 |oa|^2 - 2 ra dr (ba.oa) - ra^2 L^2.
__device__ __forceinline__ float lss_hit(V3<float> o_in, V3<float> d, V3<float> a, V3<float> b, float ra, float rb,
                                         float tmin_in, float* u_out, float* tl_out, float* ts_out) {
    const float kNone = __int_as_float(0x7f800000);
    float ts = dot(0.5f * (a + b) - o_in, d) * lss_rcp(dot(d, d));
    V3<float> wa = mk(rel_coord(a.x, o_in.x, ts, d.x), rel_coord(a.y, o_in.y, ts, d.y), rel_coord(a.z, o_in.z, ts, d.z));
    V3<float> ba = b - a;
    V3<float> wb = wa + ba;  // b - o' through the segment vector (rounded at its own scale)
    V3<float> oa = mk(-wa.x, -wa.y, -wa.z);
    float tmin = tmin_in - ts;
    float best = kNone, bu = 0.0f;
    float dr = rb - ra;
    float L2 = dot(ba, ba);
    float m = L2 - dr * dr;
    if (m > 0.0f) {
        V3<float> c1 = cross(ba, oa), c2 = cross(ba, d);
        float yd = dot(ba, d), ybo = dot(ba, oa);
        float yo = ybo + ra * dr;
        float A = dot(c2, c2) - dr * dr * dot(d, d);
        float B = dot(c1, c2) - dr * dr * dot(oa, d) - ra * dr * yd;
        float C = dot(c1, c1) - dr * dr * dot(oa, oa) - 2.0f * ra * dr * ybo - ra * ra * L2;
        float h = B * B - A * C;
        if (h >= 0.0f && A != 0.0f) {
            float sh = prhi_sqrt(h);
            const float iA = lss_rcp(A), im = lss_rcp(m);
            float r0 = (-B - sh) * iA, r1 = (-B + sh) * iA;
            float lo = gmin(r0, r1), hi = gmax(r0, r1);
            float u = (yo + lo * yd) * im;
            if (lo >= tmin && lo < best && u >= 0.0f && u <= 1.0f) { best = lo; bu = u; }
            else {
                u = (yo + hi * yd) * im;
                if (hi >= tmin && hi < best && u >= 0.0f && u <= 1.0f) { best = hi; bu = u; }
            }
        }
    }
    float ta = sphere_hit(oa, d, ra, tmin, best);
    if (ta < best) { best = ta; bu = 0.0f; }
    float tb = sphere_hit(mk(-wb.x, -wb.y, -wb.z), d, rb, tmin, best);
    if (tb < best) { best = tb; bu = 1.0f; }
    if (best == kNone) return -1.0f;
    *u_out = bu;
    *tl_out = best;
    *ts_out = ts;
    return best + ts;
}

// ---------------------------------------------------------------- triangles (watertight)
struct TriRay { int kx, ky, kz; float Sx, Sy, Sz; };
__device__ __forceinline__ TriRay make_triray(V3<float> d) {
    TriRay r;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    r.kz = 0;
    if (ay > ax && ay >= az) r.kz = 1;
    else if (az > ax && az > ay) r.kz = 2;
    r.kx = r.kz == 2 ? 0 : r.kz + 1;
    r.ky = r.kx == 2 ? 0 : r.kx + 1;
    float dk[3] = {d.x, d.y, d.z};
    if (dk[r.kz] < 0.0f) { int t = r.kx; r.kx = r.ky; r.ky = t; }
    r.Sx = dk[r.kx] / dk[r.kz];
    r.Sy = dk[r.ky] / dk[r.kz];
    r.Sz = 1.0f / dk[r.kz];
    return r;
}
__device__ __forceinline__ float comp(V3<float> v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
// b1, b2 (when given): barycentric weights of v1 and v2 at the hit (v0's is 1 - b1 - b2).
__device__ __forceinline__ float tri_hit(const TriRay& R, V3<float> o, V3<float> v0, V3<float> v1, V3<float> v2,
                                         float tmin, float tmax, float* b1 = nullptr, float* b2 = nullptr) {
    V3<float> A = v0 - o, B = v1 - o, C = v2 - o;
    float Akz = comp(A, R.kz), Bkz = comp(B, R.kz), Ckz = comp(C, R.kz);
    float Ax = comp(A, R.kx) - R.Sx * Akz, Ay = comp(A, R.ky) - R.Sy * Akz;
    float Bx = comp(B, R.kx) - R.Sx * Bkz, By = comp(B, R.ky) - R.Sy * Bkz;
    float Cx = comp(C, R.kx) - R.Sx * Ckz, Cy = comp(C, R.ky) - R.Sy * Ckz;
    float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return -1.0f;
    float det = U + V + W;
    if (det == 0.0f) return -1.0f;
    float Tn = U * (R.Sz * Akz) + V * (R.Sz * Bkz) + W * (R.Sz * Ckz);
    float t = __fdividef(Tn, det);
    if (!(t >= tmin) || !(t <= tmax)) return -1.0f;
    if (b1) {
        const float inv = 1.0f / det;
        *b1 = V * inv;
        *b2 = W * inv;
    }
    return t;
}

// The two triangles (A0, A1, A2) and (A0, B1, A1) of a quad, sharing the edge A0-A1: the shared
// vertices are transformed once and the second triangle's edge function on A0-A1 is the exact
// negation of the first's, so no ray passes between them. t0 / t1 as tri_hit returns them.
__device__ __forceinline__ void quad_hit(const TriRay& R, V3<float> o, V3<float> A0, V3<float> A1, V3<float> A2,
                                         V3<float> B1, float tmin, float tmax, float* t0, float* t1) {
    auto xf = [&](V3<float> v, float* px, float* py, float* pz) {
        const V3<float> q = v - o;
        const float z = comp(q, R.kz);
        *px = comp(q, R.kx) - R.Sx * z;
        *py = comp(q, R.ky) - R.Sy * z;
        *pz = z;
    };
    float ax, ay, az, bx, by, bz, cx, cy, cz, dx, dy, dz;
    xf(A0, &ax, &ay, &az);
    xf(A1, &bx, &by, &bz);
    xf(A2, &cx, &cy, &cz);
    xf(B1, &dx, &dy, &dz);
    const float wab = bx * ay - by * ax;  // edge A0-A1 of the first triangle
    auto finish = [&](float U, float V, float W, float az0, float bz0, float cz0) -> float {
        if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return -1.0f;
        const float det = U + V + W;
        if (det == 0.0f) return -1.0f;
        const float Tn = U * (R.Sz * az0) + V * (R.Sz * bz0) + W * (R.Sz * cz0);
        const float t = __fdividef(Tn, det);
        if (!(t >= tmin) || !(t <= tmax)) return -1.0f;
        return t;
    };
    // (A0, A1, A2): U = E(A2, A1), V = E(A0, A2), W = E(A1, A0)
    *t0 = finish(cx * by - cy * bx, ax * cy - ay * cx, wab, az, bz, cz);
    // (A0, B1, A1): U = E(A1, B1), V = E(A0, A1) = -W of the first, W = E(B1, A0)
    *t1 = finish(bx * dy - by * dx, -wab, dx * ay - dy * ax, az, dz, bz);
}

// ---------------------------------------------------------------- hit state
struct Hit {
    float t;
    uint32_t id;    // reported primitive id
    uint32_t inst;
    uint32_t slot;  // leaf slot of the hit segment
    float u;        // curve / segment parameter
    float ts, sl;   // t = ts + sl: the primitive's reference point o + ts d and the distance from it
    uint32_t flags; // HRT_HIT_FP64
};
__device__ __forceinline__ bool beats(float t, uint32_t inst, uint32_t id, const Hit& h) {
    if (t < h.t) return true;
    if (t > h.t) return false;
    return inst < h.inst || (inst == h.inst && id < h.id);
}

struct RayState {
    V3<float> o, d, inv;
    float tmin;
    Frame<float> F;   // Phantom ray-centric frame
    TriRay tr;
};

struct Stats { uint32_t nodes, prims, r64, h64, need64; };

// ---------------------------------------------------------------- leaves
// The control points and radii of the Phantom segment in leaf slot `slot`. FP32 records hold
// them (and the id); the quantised format rebuilds them from the strand vertex stream with the
// operations of the curve kernel (GenerateCurves, tension 1: cp1 = p1 + (p2 - p0) / 6,
// cp2 = p2 - (p3 - p1) / 6, each operation rounded separately), so they equal the FP32 curves bit
// for bit, and its id is read from the slot map when a hit needs it (phantom_id).
// kPrec: the record format when the launch fixes it (0 FP32, 1 quantised), -1 to read it from B.
template <int kPrec = -1>
__device__ __forceinline__ void load_phantom(const DevBlas& B, uint32_t slot, V3<float>* P, float* r0, float* r1,
                                             uint32_t* id) {
    if (kPrec < 0 ? B.precision == HRT_PRECISION_QUANTISED : kPrec == 1) {
        const uint32_t e = __ldg(static_cast<const uint32_t*>(B.prims) + slot);
        const float4 v0 = __ldg(B.verts + e), v1 = __ldg(B.verts + e + 1), v2 = __ldg(B.verts + e + 2),
                     v3 = __ldg(B.verts + e + 3);
        const float k = 1.0f / 6.0f;
        P[0] = mk(v1.x, v1.y, v1.z);
        P[1] = mk(__fadd_rn(v1.x, __fmul_rn(__fsub_rn(v2.x, v0.x), k)), __fadd_rn(v1.y, __fmul_rn(__fsub_rn(v2.y, v0.y), k)),
                  __fadd_rn(v1.z, __fmul_rn(__fsub_rn(v2.z, v0.z), k)));
        P[2] = mk(__fsub_rn(v2.x, __fmul_rn(__fsub_rn(v3.x, v1.x), k)), __fsub_rn(v2.y, __fmul_rn(__fsub_rn(v3.y, v1.y), k)),
                  __fsub_rn(v2.z, __fmul_rn(__fsub_rn(v3.z, v1.z), k)));
        P[3] = mk(v2.x, v2.y, v2.z);
        *r0 = v1.w;
        *r1 = v2.w;
        *id = 0xffffffffu;
    } else {
        const PrimPhantomF* pr = static_cast<const PrimPhantomF*>(B.prims) + slot;
        float4 a = __ldg(&pr->a), b = __ldg(&pr->b), c = __ldg(&pr->c), d = __ldg(&pr->d);
        P[0] = mk(a.x, a.y, a.z);
        P[1] = mk(b.x, b.y, b.z);
        P[2] = mk(c.x, c.y, c.z);
        P[3] = mk(d.x, d.y, d.z);
        *r0 = a.w;
        *r1 = b.w;
        *id = __float_as_uint(c.w);
    }
}
// The reported id of the Phantom segment in `slot` (id_rec: what load_phantom returned).
template <int kPrec = -1>
__device__ __forceinline__ uint32_t phantom_id(const DevBlas& B, uint32_t slot, uint32_t id_rec) {
    return (kPrec < 0 ? B.precision == HRT_PRECISION_QUANTISED : kPrec == 1) ? __ldg(&B.prim_ids[slot]) : id_rec;
}

// Tests one leaf slot; returns true if it produced an accepted hit. kType is the primitive
// type when every instance of the launch has the same one, kMixed to branch on the BLAS.
// kFlag64: a non-converged Phantom candidate only sets st.need64 (the FP64 re-solve runs in a
// later pass); otherwise it is re-solved here. kPrec: the Phantom record format when the launch
// fixes it (0 FP32, 1 quantised), -1 to read it from the BLAS.
constexpr int kMixed = 3;
template <int kType = kMixed, bool kFlag64 = false, int kPrec = -1>
__device__ __forceinline__ bool leaf_test(const DevBlas& B, uint32_t slot, uint32_t inst, const RayState& R, Hit& h,
                                          bool fp64_resolve, Stats& st) {
    const uint32_t type = kType == kMixed ? B.type : uint32_t(kType);
    if (type == HRT_BLAS_PHANTOM) {
        V3<float> P[4];
        float r0, r1;
        uint32_t id;
        load_phantom<kPrec>(B, slot, P, &r0, &r1, &id);
        PrhiOut<float> r = prhi(R.F, R.o, R.d, P, r0, r1);
        if (r.status == kHit) {
            if (r.s >= R.tmin && r.s <= h.t && beats(r.s, inst, id = phantom_id<kPrec>(B, slot, id), h)) {
                h = Hit{r.s, id, inst, slot, r.tc, r.ts, r.sl, 0u};
                return true;
            }
        } else if (kFlag64 && r.status == kUnresolved && fp64_resolve) {
            st.need64 = 1u;
        } else if (!kFlag64 && r.status == kUnresolved && fp64_resolve) {
            float cp[12];
#pragma unroll
            for (int k = 0; k < 4; ++k) { cp[3 * k] = P[k].x; cp[3 * k + 1] = P[k].y; cp[3 * k + 2] = P[k].z; }
            double s64, sl64, tc64, ts64;
            prhi_fp64(R.o.x, R.o.y, R.o.z, R.d.x, R.d.y, R.d.z, cp, r0, r1, &s64, &sl64, &ts64, &tc64);
            ++st.r64;
            if (s64 > 0.0) {
                ++st.h64;
                float s = float(s64);
                if (s >= R.tmin && s <= h.t && beats(s, inst, id = phantom_id<kPrec>(B, slot, id), h)) {
                    h = Hit{s, id, inst, slot, float(tc64), float(ts64), float(s64 - double(float(ts64))), HRT_HIT_FP64};
                    return true;
                }
            }
        }
        return false;
    }
    if (type == HRT_BLAS_LSS) {
        const PrimLss* pr = static_cast<const PrimLss*>(B.prims) + slot;
        float4 a = __ldg(&pr->a), b = __ldg(&pr->b);
        float u, tl, ts;
        float t = lss_hit(R.o, R.d, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), a.w, b.w, R.tmin, &u, &tl, &ts);
        if (t >= 0.0f && t <= h.t) {
            uint32_t id = __ldg(&B.prim_ids[slot]) >> B.ref_shift;
            if (beats(t, inst, id, h)) { h = Hit{t, id, inst, slot, u, ts, tl, 0u}; return true; }
        }
        return false;
    }
    if (type == HRT_BLAS_VOXELS) {
        // a voxel box: per axis the slab's entry and exit (an axis the ray runs parallel to only
        // rejects an origin outside the slab); hit at the entry distance, or at tmin when the ray
        // starts inside; the entry face is the axis of the latest entry (the lower axis on ties)
        const PrimVoxel* pr = static_cast<const PrimVoxel*>(B.prims) + slot;
        const float4 lo = __ldg(&pr->lo_id), hi = __ldg(&pr->hi);
        const float L3[3] = {lo.x, lo.y, lo.z}, H3[3] = {hi.x, hi.y, hi.z};
        const float O3[3] = {R.o.x, R.o.y, R.o.z}, D3[3] = {R.d.x, R.d.y, R.d.z};
        float tn = -__int_as_float(0x7f800000), tf = __int_as_float(0x7f800000);
        int ax = 0;
        bool miss = false;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (D3[k] == 0.0f) {
                if (O3[k] < L3[k] || O3[k] > H3[k]) miss = true;
                continue;
            }
            float a0 = __fdiv_rn(L3[k] - O3[k], D3[k]), a1 = __fdiv_rn(H3[k] - O3[k], D3[k]);
            if (a0 > a1) { const float t = a0; a0 = a1; a1 = t; }
            if (a0 > tn) { tn = a0; ax = k; }
            if (a1 < tf) tf = a1;
        }
        if (miss || !(tn <= tf)) return false;
        const float t = tn >= R.tmin ? tn : (tf >= R.tmin ? R.tmin : -1.0f);
        if (!(t >= R.tmin) || !(t <= h.t)) return false;
        const uint32_t id = __float_as_uint(lo.w);
        if (!beats(t, inst, id, h)) return false;
        const float face = float(ax + 1) * (D3[ax] > 0.0f ? -1.0f : 1.0f);
        h = Hit{t, id, inst, slot, face, 0.0f, 0.0f, 0u};
        return true;
    }
    if (type == HRT_BLAS_MESH) {  // renderer.cpp:543-582: one triangle per slot, id = triangle index
        const PrimTri* pr = static_cast<const PrimTri*>(B.prims) + slot;
        const float4 a = __ldg(&pr->a), b = __ldg(&pr->b), c = __ldg(&pr->c);
        float b1, b2;
        const float t = tri_hit(R.tr, R.o, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), mk(c.x, c.y, c.z), R.tmin, h.t, &b1, &b2);
        if (t >= 0.0f) {
            const uint32_t id = __float_as_uint(a.w);
            if (beats(t, inst, id, h)) { h = Hit{t, id, inst, slot, b1, b2, 0.0f, 0u}; return true; }
        }
        return false;
    }
    // DOTS: two orthogonal quads of the segment; triangle k has id 4 * segment + k
    const PrimDots* pr = static_cast<const PrimDots*>(B.prims) + slot;
    float4 a = __ldg(&pr->a), b = __ldg(&pr->b), c = __ldg(&pr->c), d = __ldg(&pr->d), e = __ldg(&pr->e);
    V3<float> s0 = mk(a.x, a.y, a.z), e0 = mk(a.w, b.x, b.y);
    V3<float> va[2] = {mk(b.z, b.w, c.x), mk(c.y, c.z, c.w)};
    V3<float> vb[2] = {mk(d.x, d.y, d.z), mk(d.w, e.x, e.y)};
    uint32_t seg = __float_as_uint(e.z);
    bool any = false;
#pragma unroll
    for (int face = 0; face < 2; ++face) {
        V3<float> A0 = s0 + va[face], A1 = e0 - vb[face], A2 = e0 + vb[face];
        V3<float> B1 = s0 - va[face];
        // triangle 2 face: (start+v*ra, end-v*rb, end+v*rb); 2 face+1: (start+v*ra, start-v*ra, end-v*rb)
        float t0, t1;
        quad_hit(R.tr, R.o, A0, A1, A2, B1, R.tmin, h.t, &t0, &t1);
        if (t0 >= 0.0f) {
            uint32_t id = 4u * seg + 2u * face;
            if (beats(t0, inst, id, h)) { h = Hit{t0, id, inst, slot, 0.0f, 0.0f, 0.0f, 0u}; any = true; }
        }
        if (t1 >= 0.0f) {
            uint32_t id = 4u * seg + 2u * face + 1u;
            if (beats(t1, inst, id, h)) { h = Hit{t1, id, inst, slot, 0.0f, 0.0f, 0.0f, 0u}; any = true; }
        }
    }
    return any;
}

// ---------------------------------------------------------------- nodes

// Reciprocal direction with zero components replaced by +-1e20, so slab distances stay finite
// (a ray inside a slab gets -huge..+huge, one outside a pair of equal signs).
// Three-input minimum and maximum (sm_100 and later); like fminf/fmaxf, a NaN input is ignored
// unless all are NaN.
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

__device__ __forceinline__ V3<float> safe_inv(V3<float> d) {
    // the IEEE reciprocal (round to nearest): the same value as 1 / x, without a full division
    auto r = [](float x) { return __frcp_rn(fabsf(x) > 1e-20f ? x : copysignf(1e-20f, x)); };
    return mk(r(d.x), r(d.y), r(d.z));
}

// Child entry distances of one node; returns a bit mask of hit children and fills tn[8].
// Near and far planes are chosen per axis by the sign of the direction (octant), so a child
// needs three maxima and three minima. FP32 boxes: t = (plane - o) inv, accepted when
// tnear <= tfar (1 + 2^-20). 8-bit boxes: t = q (2^e inv) + (p - o) inv, one fused operation
// per plane; its rounding on an axis is below 2^-20 (|p - o| |inv| + 33023 2^e |inv|), and that
// bound is subtracted from the axis's near planes and added to its far planes, so a box is
// never lost to rounding (a near-parallel axis widens only its own planes). The planes of two
// children go through one packed fused multiply-add (__ffma2_rn, each half rounded as fmaf).
// Empty slots hold empty boxes and fail the test. tn (when given) receives the entry distances;
// kWithT: also prim_base and the meta words m0/m1 (sorted traversal).
template <bool kQuant, bool kWithT = true>
__device__ __forceinline__ uint32_t test_node(const void* nodes, uint32_t ni, const RayState& R, float tfar,
                                              float* tn, uint32_t* base, uint32_t* pbase, uint32_t* m0, uint32_t* m1,
                                              uint32_t* imask = nullptr) {
    uint32_t mask = 0;
    const bool nx = R.inv.x < 0.0f, ny = R.inv.y < 0.0f, nz = R.inv.z < 0.0f;
    if (!kQuant) {
        const float kEps = 1.0f + 9.5367431640625e-07f;  // 1 + 2^-20
        const float4* p = reinterpret_cast<const float4*>(static_cast<const NodeF*>(nodes) + ni);
        // float4 index of lo_x, hi_x, lo_y, hi_y, lo_z, hi_z: 0, 2, 4, 6, 8, 10
        const int ax = nx ? 2 : 0, ay = ny ? 6 : 4, az = nz ? 10 : 8;
        float4 n0 = __ldg(p + ax), n1 = __ldg(p + ax + 1), f0 = __ldg(p + (2 - ax)), f1 = __ldg(p + (3 - ax));
        float4 n2 = __ldg(p + ay), n3 = __ldg(p + ay + 1), f2 = __ldg(p + (10 - ay)), f3 = __ldg(p + (11 - ay));
        float4 n4 = __ldg(p + az), n5 = __ldg(p + az + 1), f4 = __ldg(p + (18 - az)), f5 = __ldg(p + (19 - az));
        const float4 tail = __ldg(p + 12);  // child_base, prim_base, imask, pad
        *base = __float_as_uint(tail.x);
        if (imask) *imask = __float_as_uint(tail.z);
        if (kWithT) {
            const float2 mw = __ldg(reinterpret_cast<const float2*>(p + 13));
            *pbase = __float_as_uint(tail.y);
            *m0 = __float_as_uint(mw.x);
            *m1 = __float_as_uint(mw.y);
        }
        const float NX[8] = {n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, n1.z, n1.w};
        const float FX[8] = {f0.x, f0.y, f0.z, f0.w, f1.x, f1.y, f1.z, f1.w};
        const float NY[8] = {n2.x, n2.y, n2.z, n2.w, n3.x, n3.y, n3.z, n3.w};
        const float FY[8] = {f2.x, f2.y, f2.z, f2.w, f3.x, f3.y, f3.z, f3.w};
        const float NZ[8] = {n4.x, n4.y, n4.z, n4.w, n5.x, n5.y, n5.z, n5.w};
        const float FZ[8] = {f4.x, f4.y, f4.z, f4.w, f5.x, f5.y, f5.z, f5.w};
        // t = plane inv + (-o inv) in one fused operation. -o inv is rounded once (error below
        // 2^-24 |o inv|), so each axis's near offsets take 2^-22 |o inv| off and its far offsets
        // add it; the product-sum's own rounding and that of inv are relative to t and covered
        // by the 2^-20 relative margin of the final test.
        const float ox = -R.o.x * R.inv.x, oy = -R.o.y * R.inv.y, oz = -R.o.z * R.inv.z;
        const float kO = 2.384185791015625e-07f;  // 2^-22
        const float ex = kO * fabsf(ox), ey = kO * fabsf(oy), ez = kO * fabsf(oz);
        const float oxn = ox - ex, oxf = ox + ex, oyn = oy - ey, oyf = oy + ey, ozn = oz - ez, ozf = oz + ez;
        // two children per packed fused multiply-add (each half rounds exactly as fmaf)
        const float2 ix = make_float2(R.inv.x, R.inv.x), iy = make_float2(R.inv.y, R.inv.y);
        const float2 iz = make_float2(R.inv.z, R.inv.z);
        const float2 oxn2 = make_float2(oxn, oxn), oxf2 = make_float2(oxf, oxf), oyn2 = make_float2(oyn, oyn);
        const float2 oyf2 = make_float2(oyf, oyf), ozn2 = make_float2(ozn, ozn), ozf2 = make_float2(ozf, ozf);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float2 tnx = __ffma2_rn(make_float2(NX[2 * j], NX[2 * j + 1]), ix, oxn2);
            const float2 tfx = __ffma2_rn(make_float2(FX[2 * j], FX[2 * j + 1]), ix, oxf2);
            const float2 tny = __ffma2_rn(make_float2(NY[2 * j], NY[2 * j + 1]), iy, oyn2);
            const float2 tfy = __ffma2_rn(make_float2(FY[2 * j], FY[2 * j + 1]), iy, oyf2);
            const float2 tnz = __ffma2_rn(make_float2(NZ[2 * j], NZ[2 * j + 1]), iz, ozn2);
            const float2 tfz = __ffma2_rn(make_float2(FZ[2 * j], FZ[2 * j + 1]), iz, ozf2);
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const int q = 2 * j + k;
                const float a = max3f(k ? tnx.y : tnx.x, k ? tny.y : tny.x, fmaxf(k ? tnz.y : tnz.x, R.tmin));
                const float b = min3f(k ? tfx.y : tfx.x, k ? tfy.y : tfy.x, fminf(k ? tfz.y : tfz.x, tfar));
                if (tn) tn[q] = a;
                if (a <= b * kEps) mask |= 1u << q;
            }
        }
        return mask;
    } else {
        const uint4* p = reinterpret_cast<const uint4*>(static_cast<const NodeQ*>(nodes) + ni);
        uint4 w0 = __ldg(p), w1 = __ldg(p + 1), w2 = __ldg(p + 2), w3 = __ldg(p + 3), w4 = __ldg(p + 4);
        // per node: s = 2^e inv (one grid step in t), b = (p - o) inv
        const float sx = __uint_as_float((w0.w & 0xffu) << 23) * R.inv.x;
        const float sy = __uint_as_float(((w0.w >> 8) & 0xffu) << 23) * R.inv.y;
        const float sz = __uint_as_float(((w0.w >> 16) & 0xffu) << 23) * R.inv.z;
        const float bx = (__uint_as_float(w0.x) - R.o.x) * R.inv.x;
        const float by = (__uint_as_float(w0.y) - R.o.y) * R.inv.y;
        const float bz = (__uint_as_float(w0.z) - R.o.z) * R.inv.z;
        // One byte permute per plane makes the float 0x3F80qq00 = 1 + q 2^-15 (q under the
        // exponent of 1), and t = (1 + q 2^-15) S + (b - S) with S = 2^15 s: one packed fused
        // multiply-add per plane pair of two children. The roundings (offset, slack, product-sum)
        // are each below 2^-24 (|b| + 33023 |s|), so E = 2^-20 (|b| + 33023 |s|) per axis, taken
        // from the near planes and given to the far planes, never loses a box to rounding (about
        // 1/128 of a grid step at the scale of the node).
        const float kS = 9.5367431640625e-07f;  // 2^-20
        const float ex = kS * fmaf(33023.0f, fabsf(sx), fabsf(bx)), ey = kS * fmaf(33023.0f, fabsf(sy), fabsf(by));
        const float ez = kS * fmaf(33023.0f, fabsf(sz), fabsf(bz));
        const float Sx = 32768.0f * sx, Sy = 32768.0f * sy, Sz = 32768.0f * sz;
        const float cx = bx - Sx, cy = by - Sy, cz = bz - Sz;
        const float cxn = cx - ex, cxf = cx + ex, cyn = cy - ey, cyf = cy + ey, czn = cz - ez, czf = cz + ez;
        if (imask) *imask = w0.w >> 24;
        *base = w1.x;
        if (kWithT) {
            *pbase = w1.y;
            *m0 = w1.z;
            *m1 = w1.w;
        }
        // near / far byte words per axis (qlo = .x .y, qhi = .z .w)
        const uint32_t nxw0 = nx ? w2.z : w2.x, nxw1 = nx ? w2.w : w2.y, fxw0 = nx ? w2.x : w2.z, fxw1 = nx ? w2.y : w2.w;
        const uint32_t nyw0 = ny ? w3.z : w3.x, nyw1 = ny ? w3.w : w3.y, fyw0 = ny ? w3.x : w3.z, fyw1 = ny ? w3.y : w3.w;
        const uint32_t nzw0 = nz ? w4.z : w4.x, nzw1 = nz ? w4.w : w4.y, fzw0 = nz ? w4.x : w4.z, fzw1 = nz ? w4.y : w4.w;
        auto q15 = [](uint32_t w, uint32_t sel) { return __uint_as_float(__byte_perm(w, 0x3F800000u, sel)); };
        const float2 sx2 = make_float2(Sx, Sx), sy2 = make_float2(Sy, Sy), sz2 = make_float2(Sz, Sz);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t s0 = (j & 1) ? 0x7624u : 0x7604u, s1 = (j & 1) ? 0x7634u : 0x7614u;
            const uint32_t a = j < 2 ? nxw0 : nxw1, b = j < 2 ? fxw0 : fxw1, c = j < 2 ? nyw0 : nyw1;
            const uint32_t d = j < 2 ? fyw0 : fyw1, e = j < 2 ? nzw0 : nzw1, f = j < 2 ? fzw0 : fzw1;
            const float2 tnx = __ffma2_rn(make_float2(q15(a, s0), q15(a, s1)), sx2, make_float2(cxn, cxn));
            const float2 tfx = __ffma2_rn(make_float2(q15(b, s0), q15(b, s1)), sx2, make_float2(cxf, cxf));
            const float2 tny = __ffma2_rn(make_float2(q15(c, s0), q15(c, s1)), sy2, make_float2(cyn, cyn));
            const float2 tfy = __ffma2_rn(make_float2(q15(d, s0), q15(d, s1)), sy2, make_float2(cyf, cyf));
            const float2 tnz = __ffma2_rn(make_float2(q15(e, s0), q15(e, s1)), sz2, make_float2(czn, czn));
            const float2 tfz = __ffma2_rn(make_float2(q15(f, s0), q15(f, s1)), sz2, make_float2(czf, czf));
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const int q = 2 * j + k;
                const float lo = max3f(k ? tnx.y : tnx.x, k ? tny.y : tny.x, fmaxf(k ? tnz.y : tnz.x, R.tmin));
                const float hi = min3f(k ? tfx.y : tfx.x, k ? tfy.y : tfy.x, fminf(k ? tfz.y : tfz.x, tfar));
                if (tn) tn[q] = lo;
                if (lo <= hi) mask |= 1u << q;
            }
        }
        return mask;
    }
}

// {child_base, prim_base, meta[0..3], meta[4..7]} of node ni.
template <bool kQuant>
__device__ __forceinline__ uint4 node_header(const void* nodes, uint32_t ni) {
    if (kQuant) return __ldg(reinterpret_cast<const uint4*>(static_cast<const NodeQ*>(nodes) + ni) + 1);
    const uint4* p = reinterpret_cast<const uint4*>(static_cast<const NodeF*>(nodes) + ni);
    const uint4 t = __ldg(p + 12);
    const uint2 m = __ldg(reinterpret_cast<const uint2*>(p + 13));
    return make_uint4(t.x, t.y, m.x, m.y);
}

// The node test and header of either format: kNodes fixes it for the launch (kNodesF, kNodesQ), or
// kNodesPerInstance picks it from the current instance (q).
template <int kNodes>
__device__ __forceinline__ uint32_t test_node_of(const void* nodes, bool q, uint32_t ni, const RayState& R, float tfar,
                                                 uint32_t* base, uint32_t* imask) {
    if (kNodes == kNodesPerInstance)
        return q ? test_node<true, false>(nodes, ni, R, tfar, nullptr, base, nullptr, nullptr, nullptr, imask)
                 : test_node<false, false>(nodes, ni, R, tfar, nullptr, base, nullptr, nullptr, nullptr, imask);
    return test_node<kNodes == kNodesQ, false>(nodes, ni, R, tfar, nullptr, base, nullptr, nullptr, nullptr, imask);
}
template <int kNodes>
__device__ __forceinline__ uint4 node_header_of(const void* nodes, bool q, uint32_t ni) {
    if (kNodes == kNodesPerInstance) return q ? node_header<true>(nodes, ni) : node_header<false>(nodes, ni);
    return node_header<kNodes == kNodesQ>(nodes, ni);
}

// A TLAS node's world box against the world ray (o, inv) within [tmin, tfar], with the relative
// slack of the FP32 node test (rounding only admits extra boxes).
__device__ __forceinline__ bool tlas_box_hit(const TlasNode* nodes, uint32_t ni, V3<float> o, V3<float> inv, float tmin,
                                             float tfar, uint32_t* a, uint32_t* b) {
    const float4 lo = __ldg(reinterpret_cast<const float4*>(nodes + ni));
    const float4 hi = __ldg(reinterpret_cast<const float4*>(nodes + ni) + 1);
    *a = __float_as_uint(lo.w);
    *b = __float_as_uint(hi.w);
    const float x0 = (lo.x - o.x) * inv.x, x1 = (hi.x - o.x) * inv.x;
    const float y0 = (lo.y - o.y) * inv.y, y1 = (hi.y - o.y) * inv.y;
    const float z0 = (lo.z - o.z) * inv.z, z1 = (hi.z - o.z) * inv.z;
    const float n = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), tmin));
    const float f = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fminf(fmaxf(z0, z1), tfar));
    return n <= f * (1.0f + 9.5367431640625e-07f);
}

// Slot-order mask -> traversal order for a ray of direction octant oct: bit i <- bit i ^ oct.
__device__ __forceinline__ uint32_t oct_permute(uint32_t m, uint32_t oct) {
    if (oct & 1u) m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
    if (oct & 2u) m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
    if (oct & 4u) m = ((m & 0x0fu) << 4) | ((m >> 4) & 0x0fu);
    return m;
}

__device__ __forceinline__ void cswap(uint32_t& a, uint32_t& b) {
    uint32_t lo = min(a, b), hi = max(a, b);
    a = lo;
    b = hi;
}

// HRT_CHECKED builds test each node index, leaf slot and strand-stream entry against its array
// before the loads that use it, and stop the ray with kErrBounds instead of loading; other builds
// compile the tests away.
#ifdef HRT_CHECKED
#define HRT_BAD_INDEX(cond) (cond)
#else
#define HRT_BAD_INDEX(cond) false
#endif
__device__ __forceinline__ bool bad_slot(const DevBlas& B, uint32_t slot) {
    if (slot >= (B.nprims << B.ref_shift)) return true;
    return B.type == HRT_BLAS_PHANTOM && B.precision == HRT_PRECISION_QUANTISED &&
           uint64_t(__ldg(static_cast<const uint32_t*>(B.prims) + slot)) + 4u > B.nverts;
}

// Traverses one BLAS for the closest hit (explicit rays; the frame kernel has its own traversal).
template <bool kQuant>
__device__ bool traverse(const DevBlas& B, uint32_t inst, const RayState& R, Hit& h, bool fp64_resolve,
                         RayBounds bounds, Stats& st, uint32_t& err) {
    if (B.nnodes == 0) return false;
    uint2 stack[kStackSize];
    int sp = 0;
    stack[sp++] = make_uint2(0u, __float_as_uint(R.tmin));
    bool found = false;
    uint32_t steps = 0;
    while (sp > 0) {
        if (++steps > bounds.max_steps) { err |= kErrTimeout; break; }
        uint2 e = stack[--sp];
        if (__uint_as_float(e.y) > h.t) continue;
        if (e.x & kLeafFlag) {
            uint32_t first = (e.x & ~kLeafFlag) >> 2, cnt = (e.x & 3u) + 1u;
            for (uint32_t j = 0; j < cnt; ++j) {
                if (HRT_BAD_INDEX(bad_slot(B, first + j))) {
                    err |= kErrBounds;
                    return found;
                }
                ++st.prims;
                if (leaf_test(B, first + j, inst, R, h, fp64_resolve, st)) found = true;
            }
            continue;
        }
        if (HRT_BAD_INDEX(e.x >= B.nnodes)) {
            err |= kErrBounds;
            break;
        }
        ++st.nodes;
        float tn[8];
        uint32_t base, pbase, m0, m1;
        uint32_t mask = test_node<kQuant>(B.nodes, e.x, R, h.t, tn, &base, &pbase, &m0, &m1);
        if (!mask) continue;
        uint32_t key[8];
#pragma unroll
        for (int q = 0; q < 8; ++q)
            key[q] = (mask >> q) & 1u ? ((__float_as_uint(fmaxf(tn[q], 0.0f)) & ~7u) | uint32_t(q)) : 0xffffffffu;
        // 19-comparator sorting network for 8 keys (ascending)
        cswap(key[0], key[2]); cswap(key[1], key[3]); cswap(key[4], key[6]); cswap(key[5], key[7]);
        cswap(key[0], key[4]); cswap(key[1], key[5]); cswap(key[2], key[6]); cswap(key[3], key[7]);
        cswap(key[0], key[1]); cswap(key[2], key[3]); cswap(key[4], key[5]); cswap(key[6], key[7]);
        cswap(key[2], key[4]); cswap(key[3], key[5]);
        cswap(key[1], key[4]); cswap(key[3], key[6]);
        cswap(key[1], key[2]); cswap(key[3], key[4]); cswap(key[5], key[6]);
        int npush = __popc(mask);
        if (sp + npush > bounds.max_depth) { err |= kErrStackOverflow; break; }
#pragma unroll
        for (int k = 7; k >= 0; --k) {
            if (k >= npush) continue;
            uint32_t q = key[k] & 7u;
            uint32_t m = ((q < 4 ? m0 : m1) >> (8 * (q & 3))) & 0xffu;
            if (m == 0) continue;  // an empty slot (only a degenerate ray can pass its empty box)
            uint32_t ref = (m & 0x80u) ? base + (m & 7u)
                                       : (kLeafFlag | ((pbase + (m & 31u)) << 2) | ((m >> 5) - 1u));
            stack[sp++] = make_uint2(ref, key[k] & ~7u);
        }
    }
    return found;
}

// World-space ray through the instances of a scene (the TLAS's, or the one instance): the closest
// hit. Each instance is traversed in its own node format.
__device__ bool trace_scene(const DevInstance* insts, const TlasNode* tlas, uint32_t ninst, V3<float> wo, V3<float> wd,
                            float tmin, float tmax, Hit& h, bool fp64_resolve, RayBounds bounds, Stats& st,
                            uint32_t& err) {
    h = Hit{tmax, 0xffffffffu, 0xffffffffu, 0xffffffffu, 0.0f, 0.0f, 0.0f, 0u};
    bool found = false;
    uint32_t tstack[kTlasStack];
    int tsp = 0;
    const V3<float> winv = safe_inv(wd);
    if (tlas) tstack[tsp++] = 0;
    for (uint32_t k = 0;; ++k) {
        uint32_t i;
        if (tlas) {  // the next instance whose world box the ray meets before the closest hit
            i = 0xffffffffu;
            while (tsp > 0) {
                uint32_t a, b;
                if (!tlas_box_hit(tlas, tstack[--tsp], wo, winv, tmin, h.t, &a, &b)) continue;
                if (a & kLeafFlag) {
                    i = a & ~kLeafFlag;
                    if (HRT_BAD_INDEX(i >= ninst)) { err |= kErrBounds; i = 0xffffffffu; tsp = 0; }
                    break;
                }
                if (tsp + 2 > kTlasStack) { err |= kErrStackOverflow; tsp = 0; break; }
                tstack[tsp++] = b;
                tstack[tsp++] = a;
            }
            if (i == 0xffffffffu) break;
        } else {
            if (k >= ninst) break;
            i = k;
        }
        const DevInstance& I = insts[i];
        RayState R;
        if (I.identity) { R.o = wo; R.d = wd; }
        else {
            const float* m = I.w2o;
            R.o = xform_point(m, wo);
            R.d = xform_dir(m, wd);
        }
        R.inv = safe_inv(R.d);
        R.tmin = tmin;
        // instance bounds (object space) against the current closest distance
        {
            const DevBlas& B = I.b;
            float x0 = (B.lo[0] - R.o.x) * R.inv.x, x1 = (B.hi[0] - R.o.x) * R.inv.x;
            float y0 = (B.lo[1] - R.o.y) * R.inv.y, y1 = (B.hi[1] - R.o.y) * R.inv.y;
            float z0 = (B.lo[2] - R.o.z) * R.inv.z, z1 = (B.hi[2] - R.o.z) * R.inv.z;
            float a = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), tmin));
            float b = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fminf(fmaxf(z0, z1), h.t));
            if (!(a <= b * (1.0f + 9.5367431640625e-07f))) continue;
        }
        if (I.b.type == HRT_BLAS_PHANTOM) R.F = make_frame(R.d);
        else if (I.b.type == HRT_BLAS_DOTS || I.b.type == HRT_BLAS_MESH) R.tr = make_triray(R.d);
        const bool f = I.b.precision == HRT_PRECISION_QUANTISED ? traverse<true>(I.b, i, R, h, fp64_resolve, bounds, st, err)
                                                               : traverse<false>(I.b, i, R, h, fp64_resolve, bounds, st, err);
        if (f) found = true;
    }
    return found;
}

// Barycentric weights (of v1 and v2) of the hit point o + t d on a triangle, for shading. The
// watertight test's weights come from coordinates relative to the ray origin, so for a small
// triangle far from the camera they carry errors of about 2^-24 (distance / size)^2 (4e-4 at a
// distance of 3 for a 0.05 triangle); here every vector is relative to v0, so the rounding is at
// the triangle's scale. Falls back to the given weights for a degenerate triangle.
__device__ __noinline__ void tri_weights(V3<float> v0, V3<float> v1, V3<float> v2, V3<float> o, V3<float> d, float t,
                                            float* u, float* v) {
    const V3<float> e1 = v1 - v0, e2 = v2 - v0;
    const V3<float> w = mk(fmaf(t, d.x, o.x - v0.x), fmaf(t, d.y, o.y - v0.y), fmaf(t, d.z, o.z - v0.z));
    const float d11 = dot_rn(e1, e1), d12 = dot_rn(e1, e2), d22 = dot_rn(e2, e2);
    const float d1 = dot_rn(w, e1), d2 = dot_rn(w, e2);
    const float den = fmaf(d11, d22, -__fmul_rn(d12, d12));
    if (!(den > 0.0f)) return;
    *u = __fdiv_rn(fmaf(d22, d1, -__fmul_rn(d12, d2)), den);
    *v = __fdiv_rn(fmaf(d11, d2, -__fmul_rn(d12, d1)), den);
}

// Object-space normal of the final hit (closest-hit stage). kType: the launch's primitive type
// (only that type's branch is compiled), or kMixed to branch on the BLAS; kPrec as for leaf_test.
template <int kType, int kPrec = -1>
__device__ V3<float> hit_normal(const DevInstance& I, const Hit& h, V3<float> wo, V3<float> wd) {
    const DevBlas& B = I.b;
    const uint32_t type = kType == kMixed ? B.type : uint32_t(kType);
    V3<float> o = wo, d = wd;
    if (!I.identity) {
        const float* m = I.w2o;
        o = xform_point(m, wo);
        d = xform_dir(m, wd);
    }
    // Normals are differences of points a hair radius apart; they are formed from the
    // full-precision vectors relative to the primitive's reference point o' = o + ts d.
    V3<float> n;
    if (type == HRT_BLAS_PHANTOM) {
        // hair_intersection.rint:74-76: normalize(hit - curve(t))
        V3<float> P[4];
        float r0, r1;
        uint32_t id;
        load_phantom<kPrec>(B, h.slot, P, &r0, &r1, &id);
        float ts = h.ts;
        V3<float> W[4];
        for (int k = 0; k < 4; ++k)
            W[k] = mk(rel_coord(P[k].x, o.x, ts, d.x), rel_coord(P[k].y, o.y, ts, d.y), rel_coord(P[k].z, o.z, ts, d.z));
        // the curve point in Bernstein form with fixed fused operations
        const float u = h.u, v = __fsub_rn(1.0f, u);
        const float b0 = __fmul_rn(__fmul_rn(v, v), v), b1 = __fmul_rn(__fmul_rn(3.0f, __fmul_rn(v, v)), u);
        const float b2 = __fmul_rn(__fmul_rn(3.0f, v), __fmul_rn(u, u)), b3 = __fmul_rn(__fmul_rn(u, u), u);
        V3<float> c;
        c.x = fmaf(b3, W[3].x, fmaf(b2, W[2].x, fmaf(b1, W[1].x, __fmul_rn(b0, W[0].x))));
        c.y = fmaf(b3, W[3].y, fmaf(b2, W[2].y, fmaf(b1, W[1].y, __fmul_rn(b0, W[0].y))));
        c.z = fmaf(b3, W[3].z, fmaf(b2, W[2].z, fmaf(b1, W[1].z, __fmul_rn(b0, W[0].z))));
        n = normalize_rn(mk(fmaf(h.sl, d.x, -c.x), fmaf(h.sl, d.y, -c.y), fmaf(h.sl, d.z, -c.z)));
    } else if (type == HRT_BLAS_LSS) {
        // triangle_closest_hit.rchit:43-58: hit - mix(p0, p1, u)
        const PrimLss* pr = static_cast<const PrimLss*>(B.prims) + h.slot;
        float4 a = __ldg(&pr->a), b = __ldg(&pr->b);
        V3<float> p0 = mk(a.x, a.y, a.z), p1 = mk(b.x, b.y, b.z);
        float ts = h.ts;
        V3<float> w0 = mk(rel_coord(p0.x, o.x, ts, d.x), rel_coord(p0.y, o.y, ts, d.y), rel_coord(p0.z, o.z, ts, d.z));
        const V3<float> ax = mk(__fsub_rn(p1.x, p0.x), __fsub_rn(p1.y, p0.y), __fsub_rn(p1.z, p0.z));
        n = normalize_rn(mk(fmaf(-h.u, ax.x, fmaf(h.sl, d.x, -w0.x)), fmaf(-h.u, ax.y, fmaf(h.sl, d.y, -w0.y)),
                            fmaf(-h.u, ax.z, fmaf(h.sl, d.z, -w0.z))));
    } else if (type == HRT_BLAS_VOXELS) {
        // the entry face's normal, facing the ray; h.u = +-(axis + 1), negative when the ray
        // runs along +axis
        const float u = h.u;
        const int ax = int(fabsf(u)) - 1;
        const float sg = u < 0.0f ? -1.0f : 1.0f;
        n = mk(ax == 0 ? sg : 0.0f, ax == 1 ? sg : 0.0f, ax == 2 ? sg : 0.0f);
    } else if (type == HRT_BLAS_MESH) {
        // triangle_closest_hit.rchit:19-41: vertex normals interpolated with the hit's
        // barycentrics (1 - u - v, u, v); without normals, the face normal
        const PrimTri* pr = static_cast<const PrimTri*>(B.prims) + h.slot;
        const float4 a = __ldg(&pr->a), b = __ldg(&pr->b), c = __ldg(&pr->c), d4 = __ldg(&pr->d), e4 = __ldg(&pr->e);
        if (__float_as_uint(e4.w)) {  // n0 = (b.w, c.w, d.x), n1 = d.yzw, n2 = e.xyz
            float u = h.u, v = h.ts;
            tri_weights(mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), mk(c.x, c.y, c.z), o, d, h.t, &u, &v);
            const float w = __fsub_rn(__fsub_rn(1.0f, u), v);
            n = normalize_rn(mk(fmaf(v, e4.x, fmaf(u, d4.y, __fmul_rn(w, b.w))),
                                fmaf(v, e4.y, fmaf(u, d4.z, __fmul_rn(w, c.w))),
                                fmaf(v, e4.z, fmaf(u, d4.w, __fmul_rn(w, d4.x)))));
        } else {
            const V3<float> v0 = mk(a.x, a.y, a.z), v1 = mk(b.x, b.y, b.z), v2 = mk(c.x, c.y, c.z);
            n = normalize_rn(cross_rn(v1 - v0, v2 - v0));
        }
    } else {
        // DOTS vertices carry no normals (geometry_processor.cpp:259-264): the face normal
        const PrimDots* pr = static_cast<const PrimDots*>(B.prims) + h.slot;
        float4 a = __ldg(&pr->a), b = __ldg(&pr->b), c = __ldg(&pr->c), dd = __ldg(&pr->d), e = __ldg(&pr->e);
        V3<float> s0 = mk(a.x, a.y, a.z), e0 = mk(a.w, b.x, b.y);
        uint32_t k = h.id & 3u, face = k >> 1;
        V3<float> va = face ? mk(c.y, c.z, c.w) : mk(b.z, b.w, c.x);
        V3<float> vb = face ? mk(dd.w, e.x, e.y) : mk(dd.x, dd.y, dd.z);
        V3<float> A0 = s0 + va, A1 = e0 - vb;
        V3<float> third = (k & 1u) ? (s0 - va) : (e0 + vb);
        V3<float> v1 = (k & 1u) ? third : A1, v2 = (k & 1u) ? A1 : third;
        n = normalize_rn(cross_rn(v1 - A0, v2 - A0));
    }
    if (!I.identity) {
        const float* q = I.nrm;
        n = normalize_rn(mk(fmaf(q[2], n.z, fmaf(q[1], n.y, __fmul_rn(q[0], n.x))),
                            fmaf(q[5], n.z, fmaf(q[4], n.y, __fmul_rn(q[3], n.x))),
                            fmaf(q[8], n.z, fmaf(q[7], n.y, __fmul_rn(q[6], n.x)))));
    }
    return n;
}

// miss.rmiss:17-37: the environment seen along -d (the map is inverted), equirectangular
// (DirectionToUV), bilinear with u repeating and v clamped, then 1 - exp(-c) and gamma 1/2.2.
__device__ V3<float> env_color(const float4* env, uint32_t w, uint32_t h, V3<float> d) {
    const V3<float> v = normalize_rn(mk(-d.x, -d.y, -d.z));
    const float k1OverPi = 0.3183098861837f;  // M_1_OVER_PI of the shader
    const float gamma = asinf(fminf(fmaxf(v.y, -1.0f), 1.0f)), theta = atan2f(v.x, -v.z);
    const float u = fmaf(theta * k1OverPi, 0.5f, 0.5f), vv = fmaf(gamma, k1OverPi, 0.5f);
    // texel centres at (i + 0.5) / w
    const float x = fmaf(u, float(w), -0.5f), y = fmaf(vv, float(h), -0.5f);
    const float fx = floorf(x), fy = floorf(y);
    const float ax = x - fx, ay = y - fy;
    int x0 = int(fx) % int(w);
    if (x0 < 0) x0 += int(w);
    const int x1 = (x0 + 1) % int(w);
    const int y0 = min(max(int(fy), 0), int(h) - 1), y1 = min(max(int(fy) + 1, 0), int(h) - 1);
    const float4 c00 = __ldg(env + size_t(y0) * w + x0), c10 = __ldg(env + size_t(y0) * w + x1);
    const float4 c01 = __ldg(env + size_t(y1) * w + x0), c11 = __ldg(env + size_t(y1) * w + x1);
    auto lerp = [](float a, float b, float t) { return fmaf(t, b - a, a); };
    float c[3] = {lerp(lerp(c00.x, c10.x, ax), lerp(c01.x, c11.x, ax), ay),
                  lerp(lerp(c00.y, c10.y, ax), lerp(c01.y, c11.y, ax), ay),
                  lerp(lerp(c00.z, c10.z, ax), lerp(c01.z, c11.z, ax), ay)};
    for (int k = 0; k < 3; ++k) c[k] = powf(1.0f - expf(-c[k]), 1.0f / 2.2f);
    return mk(c[0], c[1], c[2]);
}

// triangle_closest_hit.rchit:71-81: the mesh material's albedo at a hit, albedo_factor x the
// map at the interpolated texture coordinate (rchit:39, barycentrics (1 - u - v, u, v) of the hit
// point, as for the normal). Bilinear with repeat addressing, texel centres at (i + 0.5) / size,
// row 0 at v = 0; the coordinate is wrapped into [0, 1) first, and every texel index stays in the
// map. wo, wd: the world ray.
__device__ V3<float> mesh_albedo(const DevInstance& I, const Hit& h, V3<float> wo, V3<float> wd) {
    const DevBlas& B = I.b;
    V3<float> a = mk(B.albedo[0], B.albedo[1], B.albedo[2]);
    if (!B.albedo_map || !B.uv) return a;
    V3<float> o = wo, d = wd;
    if (!I.identity) {
        o = xform_point(I.w2o, wo);
        d = xform_dir(I.w2o, wd);
    }
    const PrimTri* pr = static_cast<const PrimTri*>(B.prims) + h.slot;
    const float4 p0 = __ldg(&pr->a), p1 = __ldg(&pr->b), p2 = __ldg(&pr->c);
    float u = h.u, v = h.ts;
    tri_weights(mk(p0.x, p0.y, p0.z), mk(p1.x, p1.y, p1.z), mk(p2.x, p2.y, p2.z), o, d, h.t, &u, &v);
    const float* q = B.uv + 6 * size_t(h.id);
    const float w = __fsub_rn(__fsub_rn(1.0f, u), v);
    float s = fmaf(v, __ldg(q + 4), fmaf(u, __ldg(q + 2), __fmul_rn(w, __ldg(q))));
    float t = fmaf(v, __ldg(q + 5), fmaf(u, __ldg(q + 3), __fmul_rn(w, __ldg(q + 1))));
    s = __fsub_rn(s, floorf(s));
    t = __fsub_rn(t, floorf(t));
    const int W = int(B.map_w), H = int(B.map_h);
    const float x = fmaf(s, float(W), -0.5f), y = fmaf(t, float(H), -0.5f);
    const float fx = floorf(x), fy = floorf(y);
    const float ax = __fsub_rn(x, fx), ay = __fsub_rn(y, fy);
    // fx, fy in [-1, size - 1]; anything else (a NaN coordinate) takes the last texel
    const int x0 = fx >= 0.0f ? min(int(fx), W - 1) : W - 1, y0 = fy >= 0.0f ? min(int(fy), H - 1) : H - 1;
    const int x1 = x0 + 1 == W ? 0 : x0 + 1, y1 = y0 + 1 == H ? 0 : y0 + 1;
    const float4* m = B.albedo_map;
    const float4 c00 = __ldg(m + size_t(y0) * W + x0), c10 = __ldg(m + size_t(y0) * W + x1);
    const float4 c01 = __ldg(m + size_t(y1) * W + x0), c11 = __ldg(m + size_t(y1) * W + x1);
    auto lerp = [](float p, float r, float f) { return fmaf(f, __fsub_rn(r, p), p); };
    a.x = __fmul_rn(a.x, lerp(lerp(c00.x, c10.x, ax), lerp(c01.x, c11.x, ax), ay));
    a.y = __fmul_rn(a.y, lerp(lerp(c00.y, c10.y, ax), lerp(c01.y, c11.y, ax), ay));
    a.z = __fmul_rn(a.z, lerp(lerp(c00.z, c10.z, ax), lerp(c01.z, c11.z, ax), ay));
    return a;
}

// ray_gen.rgen:18-24, every operation rounded separately (matches the CPU restatement).
__device__ void raygen(const float* V, const float* P, uint32_t px, uint32_t py, uint32_t w, uint32_t hgt, float jx,
                       float jy, V3<float>* o, V3<float>* d) {
    float cx = __fadd_rn(float(px), jx), cy = __fadd_rn(float(py), jy);
    float ux = __fdiv_rn(cx, float(w)), uy = __fdiv_rn(cy, float(hgt));
    float dx = __fsub_rn(__fmul_rn(ux, 2.0f), 1.0f), dy = __fsub_rn(__fmul_rn(uy, 2.0f), 1.0f);
    float org[3], tgt[3], dir[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        org[k] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(V[k], 0.0f), __fmul_rn(V[4 + k], 0.0f)), __fmul_rn(V[8 + k], 0.0f)),
                           __fmul_rn(V[12 + k], 1.0f));
        tgt[k] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(P[k], dx), __fmul_rn(P[4 + k], dy)), __fmul_rn(P[8 + k], 1.0f)),
                           __fmul_rn(P[12 + k], 1.0f));
    }
    float dd = __fadd_rn(__fadd_rn(__fmul_rn(tgt[0], tgt[0]), __fmul_rn(tgt[1], tgt[1])), __fmul_rn(tgt[2], tgt[2]));
    float inv = __fdiv_rn(1.0f, __fsqrt_rn(dd));
    float n[3] = {__fmul_rn(tgt[0], inv), __fmul_rn(tgt[1], inv), __fmul_rn(tgt[2], inv)};
#pragma unroll
    for (int k = 0; k < 3; ++k)
        dir[k] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(V[k], n[0]), __fmul_rn(V[4 + k], n[1])), __fmul_rn(V[8 + k], n[2])),
                           __fmul_rn(V[12 + k], 0.0f));
    *o = mk(org[0], org[1], org[2]);
    *d = mk(dir[0], dir[1], dir[2]);
}

__device__ __forceinline__ uint32_t hash_u32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}

__constant__ float kPalette[6][3] = {{1.0f, 0.0f, 0.3f}, {0.8f, 0.2f, 0.3f}, {0.6f, 0.4f, 0.3f},
                                     {0.4f, 0.6f, 0.3f}, {0.2f, 0.8f, 0.3f}, {0.0f, 1.0f, 0.3f}};

__device__ __forceinline__ void warp_add(unsigned long long* ctr, uint32_t v) {
    // one atomic per warp
    uint32_t s = v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(kFull, s, o);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(ctr, (unsigned long long)s);
}

// ---------------------------------------------------------------- the frame kernel
// Persistent while-while traversal (Aila and Laine, HPG 2009): every lane owns a ray task (a
// pixel: its samples, each a primary ray and, when shading with shadows, one shadow ray).
//   refill     lanes without a task take pixels with one warp-aggregated atomic once enough
//              lanes are idle (ballot + popc ranks), so finished rays do not idle the warp;
//   node phase lanes test the next child of their node group together until each holds
//              leaf children or runs dry;
//   leaf phase lanes with leaf children test one each (the Phantom solve is long, so keeping
//              it out of the node loop keeps the warp converged);
//   completion a finished ray moves to the next instance, spawns its shadow ray, shades, or
//              finishes the pixel.
// The stack's bottom kShort entries live in shared memory (one column per thread), deeper
// ones in local memory. Results do not depend on scheduling: one lane handles all samples of a
// pixel in order and each ray's closest hit is the least (t, instance, id).
constexpr int kShort = 16;
constexpr int kRefill = 16;

// kPass 1: the frame (non-converged Phantom candidates flag their pixel); kPass 2: the listed
// pixels again, with the FP64 re-solve inline (adds only the FP64 counts).
template <int kNodes, int kType, int kMinBlocks, int kPass>
__global__ void __launch_bounds__(kThreads, kMinBlocks) frame_kernel(TraceLaunch L) {
    __shared__ uint2 s_stack[kShort][kThreads];
    // the hit's albedo while its shadow ray runs (mixed-type kernel: mesh materials), kept out of
    // the registers the traversal needs
    __shared__ float s_alb[kType == kMixed ? 3 : 1][kType == kMixed ? kThreads : 1];
    uint2 l_stack[kStackSize - kShort];
    const int tid = threadIdx.x, lane = tid & 31;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const volatile uint32_t* errword = &L.counters->error;
    Stats st{0, 0, 0, 0, 0};
    uint32_t shadow_rays = 0, err = 0;

    bool has_ray = false, fetch_done = false, per_sample = false;
    // a task's bookkeeping, touched once per sample: in shared memory, out of the registers the
    // traversal needs
    __shared__ uint32_t s_task[6][kThreads];
    __shared__ uint64_t s_task64[2][kThreads];
    __shared__ float s_acc[4][kThreads];
    uint32_t& si = s_task[0][tid];
    uint32_t& px = s_task[1][tid];
    uint32_t& py = s_task[2][tid];
    uint32_t& sample = s_task[3][tid];
    uint32_t& g_cur = s_task[4][tid];
    uint32_t& prim_flags = s_task[5][tid];
    uint64_t& item = s_task64[0][tid];  // FP64 pass, one sample per lane: the scratch index of the sample
    uint64_t& pix = s_task64[1][tid];
    float& acc0 = s_acc[0][tid];
    float& acc1 = s_acc[1][tid];
    float& acc2 = s_acc[2][tid];
    float& ndl = s_acc[3][tid];
    si = px = py = sample = g_cur = prim_flags = 0;
    item = pix = 0;
    acc0 = acc1 = acc2 = ndl = 0.0f;
    bool shadow = false, shadow_hit = false;
    V3<float> wo = mk(0.0f, 0.0f, 0.0f), wd = mk(0.0f, 0.0f, 1.0f);
    float cur_tmin = 0.0f;
    RayState R;
    Hit h{0.0f, 0xffffffffu, 0xffffffffu, 0xffffffffu, 0.0f, 0.0f, 0.0f, 0u};
    uint32_t inst_cur = 0, skip_inst = 0xffffffffu, skip_slot = 0xffffffffu, skip_slot2 = 0xffffffffu;
    int sp = 0;
    uint32_t steps = 0;
    const void* nodes = nullptr;                 // node array of the current instance's BLAS
    // Multi-instance scenes (a TLAS) run in the kNodesPerInstance build only, so the builds for
    // one node format keep the lean single-instance loop.
    constexpr bool kTlas = kNodes == kNodesPerInstance;
    constexpr int kPrec = kNodes == kNodesF ? 0 : (kNodes == kNodesQ ? 1 : -1);  // Phantom record format
    bool qnodes = false;                         // the current instance's format (kNodesPerInstance)
    uint32_t tstack[kTlas ? kTlasStack : 1];     // TLAS walk (local memory)
    int tsp = 0;
    uint32_t oct = 0;                            // direction octant of the object-space ray
    uint32_t cur_base = 0, cur_bits = 0;         // node group: hits in visiting order (bits 0-7), imask (8-15)
    uint32_t leaf_node = 0, leaf_bits = 0;       // untested leaf children of node leaf_node, visiting order

    auto push = [&](uint2 e) {
        if (sp < kShort) s_stack[sp][tid] = e;
        else l_stack[sp - kShort] = e;
        ++sp;
    };
    auto pop = [&]() -> uint2 {
        --sp;
        return sp < kShort ? s_stack[sp][tid] : l_stack[sp - kShort];
    };
    // Object-space ray for instance i; pushes its root when the instance box is hit.
    auto setup_instance = [&](uint32_t i) -> bool {
        const DevInstance& I = L.scenes[si].inst[i];
        if (I.identity) { R.o = wo; R.d = wd; }
        else {
            const float* m = I.w2o;
            R.o = xform_point(m, wo);
            R.d = xform_dir(m, wd);
        }
        R.inv = safe_inv(R.d);
        R.tmin = cur_tmin;
        const DevBlas& B = I.b;
        if (B.nnodes == 0) return false;
        float x0 = (B.lo[0] - R.o.x) * R.inv.x, x1 = (B.hi[0] - R.o.x) * R.inv.x;
        float y0 = (B.lo[1] - R.o.y) * R.inv.y, y1 = (B.hi[1] - R.o.y) * R.inv.y;
        float z0 = (B.lo[2] - R.o.z) * R.inv.z, z1 = (B.hi[2] - R.o.z) * R.inv.z;
        float a = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), cur_tmin));
        float b = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fminf(fmaxf(z0, z1), h.t));
        if (!(a <= b * (1.0f + 9.5367431640625e-07f))) return false;
        const uint32_t type = kType == kMixed ? B.type : uint32_t(kType);
        if (type == HRT_BLAS_PHANTOM) R.F = make_frame(R.d);
        else if (type == HRT_BLAS_DOTS || type == HRT_BLAS_MESH) R.tr = make_triray(R.d);
        nodes = B.nodes;
        if (kNodes == kNodesPerInstance) qnodes = B.precision == HRT_PRECISION_QUANTISED;
        oct = (R.inv.x < 0.0f ? 1u : 0u) | (R.inv.y < 0.0f ? 2u : 0u) | (R.inv.z < 0.0f ? 4u : 0u);
        cur_base = 0;  // the root as a group of one internal child in slot 0
        cur_bits = (1u << oct) | (1u << 8);
        return true;
    };
    // The ray's next candidate instance: of a multi-instance scene, the next TLAS leaf whose world
    // box the ray meets before its closest hit; of a one-instance scene, the next index. ~0u when
    // there is none. (The completion step sets the candidate up; one call site keeps the kernel's
    // code as compact as it was without a TLAS.)
    auto advance = [&]() -> uint32_t {
        const SceneLaunch& S = L.scenes[si];
        if (!kTlas || !S.tlas) return inst_cur + 1 < S.ninst ? inst_cur + 1 : 0xffffffffu;
        const V3<float> winv = safe_inv(wd);
        while (tsp > 0) {
            uint32_t a, b;
            if (!tlas_box_hit(S.tlas, tstack[--tsp], wo, winv, cur_tmin, h.t, &a, &b)) continue;
            if (a & kLeafFlag) {
                if (HRT_BAD_INDEX((a & ~kLeafFlag) >= S.ninst)) {
                    err |= kErrBounds;
                    tsp = 0;
                    break;
                }
                return a & ~kLeafFlag;
            }
            if (tsp + 2 > kTlasStack) {  // deeper than a TLAS is built (bounded all the same)
                err |= kErrStackOverflow;
                tsp = 0;
                break;
            }
            tstack[tsp++] = b;
            tstack[tsp++] = a;
        }
        return 0xffffffffu;
    };
    auto start_ray = [&](V3<float> o, V3<float> d, float tmin, float tmax) {
        wo = o;
        wd = d;
        cur_tmin = tmin;
        h = Hit{tmax, 0xffffffffu, 0xffffffffu, 0xffffffffu, 0.0f, 0.0f, 0.0f, 0u};
        sp = 0;
        cur_bits = 0;
        leaf_bits = 0;
        steps = 0;
        const SceneLaunch& S = L.scenes[si];
        if (kTlas && S.tlas) {  // the completion step walks the TLAS from its root
            tsp = 0;
            tstack[tsp++] = 0;
            inst_cur = 0xffffffffu;
        } else {
            for (inst_cur = 0; inst_cur < S.ninst; ++inst_cur)
                if (setup_instance(inst_cur)) break;
        }
    };
    auto start_primary = [&]() {
        const SceneLaunch& S = L.scenes[si];
        float jx = 0.5f, jy = 0.5f;
        if (L.jitter || S.spp > 1) {
            uint32_t h1 = hash_u32(L.seed ^ hash_u32(uint32_t(pix) * S.spp + sample));
            uint32_t h2 = hash_u32(h1);
            jx = float(h1 >> 8) * 5.9604644775390625e-08f;
            jy = float(h2 >> 8) * 5.9604644775390625e-08f;
        }
        V3<float> o, d;
        raygen(S.view_inv, S.proj_inv, px, py, S.width, S.height, jx, jy, &o, &d);
        shadow = false;
        start_ray(o, d, L.tmin, L.tmax);
    };
    // shading.glsl Shade(): |n.l| light + ambient, times the albedo (1 except on meshes with a material)
    auto add_shade = [&](float l) {
        float c0 = fmaf(l, 0.4f, 0.3f), c1 = fmaf(l, 0.2f, 0.3f), c2 = fmaf(l, 0.1f, 0.3f);
        if (kType == kMixed) {
            c0 = __fmul_rn(c0, s_alb[0][tid]);
            c1 = __fmul_rn(c1, s_alb[1][tid]);
            c2 = __fmul_rn(c2, s_alb[2][tid]);
        }
        acc0 = __fadd_rn(acc0, c0);
        acc1 = __fadd_rn(acc1, c1);
        acc2 = __fadd_rn(acc2, c2);
    };
    auto next_sample = [&]() {
        const SceneLaunch& S = L.scenes[si];
        ++sample;
        if (kPass == 2 && per_sample) {  // this sample's colour; a later launch averages
            L.resolve_scratch[item] = make_float4(acc0, acc1, acc2, 0.0f);
            has_ray = false;
            return;
        }
        if (sample < S.spp) { start_primary(); return; }
        float inv = 1.0f / float(S.spp);
        S.fb[pix] = make_float4(__fmul_rn(acc0, inv), __fmul_rn(acc1, inv), __fmul_rn(acc2, inv), 1.0f);
        has_ray = false;
        if (kPass == 1 && st.need64) {  // list the pixel for the FP64 pass
            st.need64 = 0;
            unsigned long long k = atomicAdd(&L.counters->resolve_n, 1ull);
            if (k < L.resolve_cap) L.resolve_list[k] = g_cur;
        }
    };
    auto finish_phase = [&]() {
        const SceneLaunch& S = L.scenes[si];
        uint64_t rec = pix * S.spp + sample;
        if (!shadow) {
            bool found = h.id != 0xffffffffu;
            prim_flags = h.flags;
            if (L.record_hits && S.hits) {
                hrt_hit r;
                r.t = found ? h.t : -1.0f;
                r.prim = h.id;
                r.inst = h.inst;
                r.flags = found ? h.flags : 0u;
                S.hits[rec] = r;
            }
            if (!found) {
                if (L.env_map) {
                    const V3<float> c = env_color(L.env_map, L.env_w, L.env_h, wd);
                    acc0 = __fadd_rn(acc0, c.x);
                    acc1 = __fadd_rn(acc1, c.y);
                    acc2 = __fadd_rn(acc2, c.z);
                }
                next_sample();
                return;
            }
            if (L.shading == HRT_SHADE_DEBUG) {
                uint32_t c = h.id % 6u;
                acc0 = __fadd_rn(acc0, kPalette[c][0]);
                acc1 = __fadd_rn(acc1, kPalette[c][1]);
                acc2 = __fadd_rn(acc2, kPalette[c][2]);
                next_sample();
                return;
            }
            V3<float> n = hit_normal<kType, kPrec>(S.inst[h.inst], h, wo, wd);
            ndl = fabsf(n.y);  // shading.glsl: |dot(n, (0,-1,0))|
            if (kType == kMixed) {  // meshes run in the mixed-type kernel only
                const DevBlas& HB = S.inst[h.inst].b;
                const V3<float> a = HB.type == HRT_BLAS_MESH ? mesh_albedo(S.inst[h.inst], h, wo, wd) : mk(1.0f, 1.0f, 1.0f);
                s_alb[0][tid] = a.x;
                s_alb[1][tid] = a.y;
                s_alb[2][tid] = a.z;
            }
            if (L.shading == HRT_SHADE_LAMBERT_SHADOW) {
                skip_inst = h.inst;
                // the hit segment's slots: its own and, for two-reference BLASes, its partner's
                skip_slot = h.slot;
                skip_slot2 = S.inst[h.inst].b.partner ? __ldg(&S.inst[h.inst].b.partner[h.slot]) : h.slot;
                shadow_hit = false;
                shadow = true;
                ++shadow_rays;
                V3<float> hp = mk(fmaf(h.t, wd.x, wo.x), fmaf(h.t, wd.y, wo.y), fmaf(h.t, wd.z, wo.z));
                start_ray(hp, mk(0.0f, 1.0f, 0.0f), L.shadow_tmin, L.tmax);
                return;
            }
            add_shade(ndl);
            next_sample();
            return;
        }
        add_shade(shadow_hit ? 0.0f : ndl);
        if (shadow_hit && L.record_hits && S.hits) S.hits[rec].flags = prim_flags | HRT_HIT_SHADOWED;
        shadow = false;
        next_sample();
    };

    const int refill = L.refill ? int(L.refill) : kRefill;  // idle lanes that trigger a fetch
    const bool spec = L.speculative != 0;
    const int leaf_again = int(L.leaf_again);
    // work items: pass 1 every item; pass 2 the samples of the listed pixels, or the listed
    // pixels when their samples do not fit the scratch, or every item if the list overflowed
    unsigned long long* const work_ctr = kPass == 1 ? &L.counters->work : &L.counters->work2;
    uint64_t total = L.total_work;
    bool use_list = false;
    if (kPass == 2) {
        const unsigned long long nl = __ldcg(&L.counters->resolve_n);
        if (nl <= L.resolve_cap) { total = nl; use_list = true; }
        if (use_list && nl * L.max_spp <= L.scratch_cap) { total = nl * L.max_spp; per_sample = true; }
    }
    // FP64 pass: only the first lanes of a warp take work (at once, whenever one is idle), two
    // while the listed items fit two per warp of the grid, more when there are more: the few
    // listed samples then spread over many warps instead of packing 32 divergent FP64 solves into
    // one (the pass is as long as its slowest warp and sits on the batch's critical path; the
    // 16-scene batch ran 3.4 % faster than with 32 lanes)
    uint32_t take = kFull;
    if (kPass == 2) {
        const uint64_t warps = uint64_t(gridDim.x) * (blockDim.x / 32);
        const uint64_t per = (total + warps - 1) / warps;
        take = per <= 2 ? 0x3u : (per >= 32 ? kFull : ((1u << uint32_t(per)) - 1u));
    }
    unsigned long long cyc_node = 0, cyc_leaf = 0, cyc_other = 0;
    long long clk = clock64();
    for (;;) {
        // ---- refill idle lanes
        uint32_t idle = __ballot_sync(kFull, !has_ray) & take;
        if (idle && !fetch_done && (__popc(idle) >= refill || idle == take || (kPass == 2))) {
            int n = __popc(idle), leader = __ffs(idle) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = *errword ? total : atomicAdd(work_ctr, (unsigned long long)n);
            base = __shfl_sync(kFull, base, leader);
            if (base + uint64_t(n) >= total) fetch_done = true;
            if (!has_ray && ((take >> lane) & 1u)) {
                uint64_t g = base + __popc(idle & lt_mask);
                if (g < total) {
                    uint32_t s0 = 0;
                    if (per_sample) {
                        item = g;
                        s0 = uint32_t(g % L.max_spp);
                        g = g / L.max_spp;
                    }
                    if (use_list) g = __ldcg(&L.resolve_list[g]);
                    g_cur = uint32_t(g);
                    si = 0;
                    while (si + 1 < L.nscenes && L.scenes[si + 1].work_begin <= g) ++si;
                    const SceneLaunch& S = L.scenes[si];
                    uint64_t local = g - S.work_begin, tile = local >> 5;
                    uint32_t within = uint32_t(local & 31u);
                    px = uint32_t(tile % S.tiles_x) * 8u + (within & 7u);
                    py = uint32_t(tile / S.tiles_x) * 4u + (within >> 3);
                    if (px < S.width && py < S.height && s0 < S.spp) {
                        pix = uint64_t(py) * S.width + px;
                        has_ray = true;
                        sample = s0;
                        acc0 = acc1 = acc2 = 0.0f;
                        start_primary();
                    }
                }
            }
        }
        if (!__any_sync(kFull, has_ray)) {
            if (fetch_done) break;
            continue;
        }
        if (L.count_stats) { long long c = clock64(); cyc_other += c - clk; clk = c; }
        // ---- node phase: runs while some lane still searches for a leaf; with speculation,
        // lanes that already hold leaves keep walking nodes (further leaves go on the stack).
        // A lane visits the children of its current node group in the order i ^ oct (slots are
        // laid out by direction, so roughly near to far); a visited node's internal hits become
        // the new group (the rest of the old one goes on the stack) and its leaf hits become
        // the lane's pending leaves.
        bool stalled = false;
        for (;;) {
            const bool more = (cur_bits & 0xffu) != 0u || sp > 0;
            const bool searching = has_ray && !leaf_bits && more;
            if (!__any_sync(kFull, searching)) break;
            const bool want = searching || (spec && has_ray && leaf_bits && !stalled && more);
            if (!want) continue;
            if (++steps > L.max_steps) {
                err |= kErrTimeout;
                sp = 0;
                cur_bits = leaf_bits = 0;
                continue;
            }
            if (!(cur_bits & 0xffu)) {
                const uint2 e = pop();
                if (e.x & kLeafFlag) {  // leaves parked by a speculating lane (no distances kept)
                    if (leaf_bits) {
                        push(e);
                        stalled = true;
                    } else {
                        leaf_node = e.x & ~kLeafFlag;
                        leaf_bits = oct_permute(e.y, oct);
                    }
                    continue;
                }
                cur_base = e.x;
                cur_bits = e.y;
            }
            const uint32_t i = __ffs(cur_bits & 0xffu) - 1;
            cur_bits &= ~(1u << i);
            const uint32_t slot = i ^ oct;
            const uint32_t child = cur_base + __popc((cur_bits >> 8) & ((1u << slot) - 1u));
            if (HRT_BAD_INDEX(child >= L.scenes[si].inst[inst_cur].b.nnodes)) {
                err |= kErrBounds;
                sp = 0;
                cur_bits = leaf_bits = 0;
                continue;
            }
            ++st.nodes;
            uint32_t base, imask;
            const uint32_t mask = test_node_of<kNodes>(nodes, qnodes, child, R, h.t, &base, &imask);
            const uint32_t ih = mask & imask, lh = mask & ~imask;
            if (sp + 2 > L.max_depth) {
                err |= kErrStackOverflow;
                sp = 0;
                cur_bits = leaf_bits = 0;
                continue;
            }
            if (lh) {
                if (!leaf_bits) {
                    leaf_node = child;
                    leaf_bits = oct_permute(lh, oct);
                } else {
                    push(make_uint2(kLeafFlag | child, lh));
                    stalled = true;
                }
            }
            if (ih) {
                if (cur_bits & 0xffu) push(make_uint2(cur_base, cur_bits));
                cur_base = base;
                cur_bits = oct_permute(ih, oct) | (imask << 8);
            }
        }
        if (L.count_stats) { __syncwarp(); long long c = clock64(); cyc_node += c - clk; clk = c; }
        // ---- leaf phase: one leaf child per lane, in visiting order; repeated (at most 8 rounds)
        // while at least leaf_again lanes still hold leaf children, so lanes whose test ended
        // early take their next leaf instead of idling
        for (int round = 0; round < 8; ++round) {
            if (round > 0 && (!leaf_again || __popc(__ballot_sync(kFull, leaf_bits != 0u)) < leaf_again)) break;
        if (leaf_bits) {
            const DevBlas& B = L.scenes[si].inst[inst_cur].b;
            const uint32_t q = (__ffs(leaf_bits) - 1) ^ oct;
            leaf_bits &= leaf_bits - 1u;
            const uint4 hd = node_header_of<kNodes>(nodes, qnodes, leaf_node);
            const uint32_t m = ((q < 4 ? hd.z : hd.w) >> (8 * (q & 3))) & 0xffu;
            const uint32_t first = hd.y + (m & 31u), cnt = m >> 5;
            for (uint32_t j = 0; j < cnt; ++j) {
                uint32_t slot = first + j;
                if (shadow && inst_cur == skip_inst && (slot == skip_slot || slot == skip_slot2)) continue;
                if (HRT_BAD_INDEX(bad_slot(B, slot))) {
                    err |= kErrBounds;
                    sp = 0;
                    cur_bits = leaf_bits = 0;
                    break;
                }
                ++st.prims;
                if (leaf_test<kType, kPass == 1, kPrec>(B, slot, inst_cur, R, h, L.fp64_resolve != 0, st) && shadow) {
                    shadow_hit = true;
                    sp = 0;
                    cur_bits = leaf_bits = 0;
                    break;
                }
            }
        }
        }
        if (L.count_stats) { __syncwarp(); long long c = clock64(); cyc_leaf += c - clk; clk = c; }
        // ---- completion
        if (has_ray && !leaf_bits && sp == 0 && !(cur_bits & 0xffu)) {
            if (err) {
                // a bounded loop gave up: drop the task and raise the launch's error word; every
                // warp (this one too) stops taking work at its next fetch, which reads the word,
                // so fetch_done stays the same in all lanes of a warp (the warp-wide votes and
                // shuffles of the loop need all 32 lanes)
                atomicOr(&L.counters->error, err);
                has_ray = false;
            } else {
                bool more = false;
                if (!(shadow && shadow_hit))
                    for (uint32_t i; (i = advance()) != 0xffffffffu;) {
                        inst_cur = i;
                        if (setup_instance(i)) { more = true; break; }
                    }
                if (!more) finish_phase();
            }
        }
    }
    if (kPass == 1) warp_add(&L.counters->shadow, shadow_rays);
    if (kPass == 1 && L.count_stats) {
        warp_add(&L.counters->nodes, st.nodes);
        warp_add(&L.counters->prims, st.prims);
        cyc_other += clock64() - clk;
        if (lane == 0) {  // warp-level phase clocks
            atomicAdd(&L.counters->cycles_node, cyc_node);
            atomicAdd(&L.counters->cycles_leaf, cyc_leaf);
            atomicAdd(&L.counters->cycles_other, cyc_other);
        }
    }
    warp_add(&L.counters->fp64_resolves, st.r64);
    warp_add(&L.counters->fp64_hits, st.h64);
    if (err) atomicOr(&L.counters->error, err);
}

#ifdef HRT_RAY_KERNEL  // compiled by trace.cu only
__global__ void __launch_bounds__(kThreads) trace_rays_kernel(const DevInstance* inst, const TlasNode* tlas,
                                                              uint32_t ninst, const float* rays, uint64_t n, float tmin,
                                                              float tmax, uint32_t fp64_resolve, RayBounds bounds,
                                                              hrt_hit* hits, TraceCounters* ctr) {
    Stats st{0, 0, 0, 0, 0};
    uint32_t err = 0;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
        const float* r = rays + 6 * i;
        Hit h;
        bool f = trace_scene(inst, tlas, ninst, mk(r[0], r[1], r[2]), mk(r[3], r[4], r[5]), tmin, tmax, h,
                             fp64_resolve != 0, bounds, st, err);
        hrt_hit o;
        o.t = f ? h.t : -1.0f;
        o.prim = f ? h.id : 0xffffffffu;
        o.inst = f ? h.inst : 0xffffffffu;
        o.flags = f ? h.flags : 0u;
        hits[i] = o;
    }
    warp_add(&ctr->fp64_resolves, st.r64);
    warp_add(&ctr->fp64_hits, st.h64);
    if (err) atomicOr(&ctr->error, err);
}
#endif

// Shared memory / L1 split of the SM for a frame kernel: the smallest shared configuration that
// holds the variant's resident blocks, so the rest of the array serves as L1 for the node and
// record loads (0.2-0.8 % faster than the default split; the largest L1 split cuts the resident
// blocks, the largest shared split is 2-4 % slower). Set once per kernel when the context is
// created (not during a graph capture).
template <int kNodes, int kType, int kMinBlocks, int kPass>
cudaError_t set_carveout() {
    // A block holds its static shared memory (16 KB of short stacks, 7 KB of task state, 1.5 KB
    // more for the mixed-type kernel's albedo) plus 1 KB the hardware reserves. The smallest of
    // the SM's shared-memory configurations from 100 KB up that holds kMinBlocks of them is asked
    // for as a percentage of the 228 KB array, rounded up so that it maps to that configuration:
    // 100 KB for four blocks of the hair kernels, 132 KB for five, or for four mixed-type blocks.
    auto* k = frame_kernel<kNodes, kType, kMinBlocks, kPass>;
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, k);
    if (e != cudaSuccess) return e;
    const size_t need = size_t(kMinBlocks) * (fa.sharedSizeBytes + 1024);
    int kb = 228;
    for (int c : {100, 132, 164, 196, 228})
        if (size_t(c) * 1024 >= need) {
            kb = c;
            break;
        }
    return cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, (kb * 100 + 227) / 228);
}
template <int kNodes>
cudaError_t prepare_frame_kernels() {
    cudaError_t e = cudaSuccess;
    if constexpr (kNodes == kNodesPerInstance) {  // the mixed-type kernel only
        e = set_carveout<kNodes, kMixed, 4, 1>();
        if (e == cudaSuccess) e = set_carveout<kNodes, kMixed, 1, 2>();
        return e;
    } else {
        auto all = [&](auto minb) {
            constexpr int kB = decltype(minb)::value;
            if (e == cudaSuccess) e = set_carveout<kNodes, HRT_BLAS_PHANTOM, kB, 1>();
            if (e == cudaSuccess) e = set_carveout<kNodes, HRT_BLAS_LSS, kB, 1>();
            if (e == cudaSuccess) e = set_carveout<kNodes, HRT_BLAS_DOTS, kB, 1>();
            if (e == cudaSuccess) e = set_carveout<kNodes, kMixed, kB, 1>();
        };
        all(std::integral_constant<int, 3>{});
        all(std::integral_constant<int, 4>{});
        all(std::integral_constant<int, 5>{});
        if (e == cudaSuccess) e = set_carveout<kNodes, HRT_BLAS_PHANTOM, 1, 2>();
        if (e == cudaSuccess) e = set_carveout<kNodes, kMixed, 1, 2>();
        return e;
    }
}

template <int kNodes, int kType, int kMinBlocks, int kPass>
cudaError_t launch_frame(const TraceLaunch& L, cudaStream_t s, int sm_count) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, frame_kernel<kNodes, kType, kMinBlocks, kPass>, kThreads, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    unsigned grid = unsigned(sm_count * per_sm);
    uint64_t max_blocks = (L.total_work + kThreads - 1) / kThreads;
    if (grid > max_blocks) grid = unsigned(max_blocks ? max_blocks : 1);
    frame_kernel<kNodes, kType, kMinBlocks, kPass><<<grid, kThreads, 0, s>>>(L);
    return cudaGetLastError();
}

template <int kNodes, int kMinBlocks>
cudaError_t launch_kind(const TraceLaunch& L, cudaStream_t s, int sm_count) {
    switch (L.prim_kind) {  // one primitive type in every instance -> the specialised kernel
        case HRT_BLAS_PHANTOM: return launch_frame<kNodes, HRT_BLAS_PHANTOM, kMinBlocks, 1>(L, s, sm_count);
        case HRT_BLAS_LSS: return launch_frame<kNodes, HRT_BLAS_LSS, kMinBlocks, 1>(L, s, sm_count);
        case HRT_BLAS_DOTS: return launch_frame<kNodes, HRT_BLAS_DOTS, kMinBlocks, 1>(L, s, sm_count);
        default: return launch_frame<kNodes, kMixed, kMinBlocks, 1>(L, s, sm_count);
    }
}

// After a per-sample FP64 pass: each listed pixel's colour is the mean of its samples' colours,
// summed in sample order from zero (the frame pass's own accumulation, bit for bit).
__global__ void __launch_bounds__(kThreads) resolve_average_kernel(TraceLaunch L) {
    const unsigned long long nl = __ldcg(&L.counters->resolve_n);
    if (nl > L.resolve_cap || nl * L.max_spp > L.scratch_cap) return;  // the pass ran per pixel
    for (uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < nl; k += uint64_t(gridDim.x) * blockDim.x) {
        const uint32_t g = __ldcg(&L.resolve_list[k]);
        uint32_t si = 0;
        while (si + 1 < L.nscenes && L.scenes[si + 1].work_begin <= g) ++si;
        const SceneLaunch& S = L.scenes[si];
        const uint64_t local = g - S.work_begin, tile = local >> 5;
        const uint32_t within = uint32_t(local & 31u);
        const uint32_t px = uint32_t(tile % S.tiles_x) * 8u + (within & 7u);
        const uint32_t py = uint32_t(tile / S.tiles_x) * 4u + (within >> 3);
        float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
        for (uint32_t s2 = 0; s2 < S.spp; ++s2) {
            const float4 c = __ldcg(&L.resolve_scratch[k * L.max_spp + s2]);
            a0 = __fadd_rn(a0, c.x);
            a1 = __fadd_rn(a1, c.y);
            a2 = __fadd_rn(a2, c.z);
        }
        const float inv = 1.0f / float(S.spp);
        S.fb[uint64_t(py) * S.width + px] = make_float4(__fmul_rn(a0, inv), __fmul_rn(a1, inv), __fmul_rn(a2, inv), 1.0f);
    }
}

// The FP64 pass: only launches that hold Phantom BLASes can list pixels.
template <int kNodes>
cudaError_t launch_resolve(const TraceLaunch& L, cudaStream_t s, int sm_count) {
    if (!L.fp64_resolve || !L.resolve_list) return cudaSuccess;
    cudaError_t e = cudaSuccess;
    if (kNodes != kNodesPerInstance && L.prim_kind == HRT_BLAS_PHANTOM)
        e = launch_frame<kNodes, kNodes == kNodesPerInstance ? kMixed : HRT_BLAS_PHANTOM, 1, 2>(L, s, sm_count);
    else if (kNodes == kNodesPerInstance || L.prim_kind == kMixed) e = launch_frame<kNodes, kMixed, 1, 2>(L, s, sm_count);
    else return cudaSuccess;
    if (e != cudaSuccess || !L.resolve_scratch) return e;
    resolve_average_kernel<<<unsigned(sm_count), kThreads, 0, s>>>(L);
    return cudaGetLastError();
}

}  // namespace
}  // namespace hrt
