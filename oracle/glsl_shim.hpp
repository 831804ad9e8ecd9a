// oracle/glsl_shim.hpp -- TEST INFRASTRUCTURE (the oracle), never linked into the product.
//
// A small GLSL / glm stand-in, templated on the scalar type, so that
//   (1) the reference's own shader math (shaders/curve.glsl, cone.glsl, cylinder.glsl,
//       ray.glsl, shading.glsl and the Prhi function of hair_intersection.rint) can be
//       compiled unmodified as host C++ (oracle/ref_harness.cpp), and
//   (2) the oracle's restatement (oracle/hrt_oracle.cpp) runs on exactly the same vector
//       library, so the two can be compared bit for bit in FP32.
//
// Semantics follow glm 1.0.1 (the library the reference's host code uses, pinned by
// external/CMakeLists.txt:64-72 of the reference); glm is not available here, so its
// published definitions are restated:
//   dot(a,b)       = (a.x*b.x + a.y*b.y) + a.z*b.z         (tmp = a*b; tmp.x+tmp.y+tmp.z)
//   length(v)      = sqrt(dot(v,v))
//   normalize(v)   = v * (1 / sqrt(dot(v,v)))               (v * inversesqrt(dot(v,v)))
//   cross(x,y)     = (x.y*y.z - y.y*x.z, x.z*y.x - y.z*x.x, x.x*y.y - y.x*x.y)
//   min(x,y)       = (y < x) ? y : x ;  max(x,y) = (x < y) ? y : x
//   abs(x)         = x >= 0 ? x : -x
// Everything must be compiled with -ffp-contract=off so that no multiply-add is fused.
#pragma once
#include <cmath>
#include <cstdint>

namespace shim {

// GLSL uvec3 with the .xy swizzle used by ray_gen.rgen (gl_LaunchIDEXT.xy).
struct uvec2 { uint32_t x, y; };
struct uvec3 {
    union {
        struct { uint32_t x, y, z; };
        uvec2 xy;
    };
};

template <class T> struct tvec2 {
    T x, y;
    tvec2() = default;
    constexpr tvec2(T a, T b) : x(a), y(b) {}
    template <class U> explicit constexpr tvec2(U s) : x(T(s)), y(T(s)) {}
    explicit constexpr tvec2(uvec2 u) : x(T(u.x)), y(T(u.y)) {}
    template <class U> explicit constexpr tvec2(const tvec2<U>& o) : x(T(o.x)), y(T(o.y)) {}
};

template <class T> struct tvec3 {
    T x, y, z;
    tvec3() = default;
    constexpr tvec3(T a, T b, T c) : x(a), y(b), z(c) {}
    // glm::vec3(uint, uint, uint) and mixed-argument constructors.
    template <class A, class B, class C>
    constexpr tvec3(A a, B b, C c) : x(T(a)), y(T(b)), z(T(c)) {}
    template <class U> explicit constexpr tvec3(U s) : x(T(s)), y(T(s)), z(T(s)) {}
    template <class U> explicit constexpr tvec3(const tvec3<U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
    T& operator[](int i) { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
};

template <class T> struct tvec4 {
    union {
        struct { T x, y, z, w; };
        tvec3<T> xyz;
    };
    tvec4() = default;
    template <class A, class B, class C, class D>
    constexpr tvec4(A a, B b, C c, D d) : x(T(a)), y(T(b)), z(T(c)), w(T(d)) {}
    template <class D>
    constexpr tvec4(const tvec3<T>& v, D d) : x(v.x), y(v.y), z(v.z), w(T(d)) {}
    T& operator[](int i) { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
};

// ---- vec2 arithmetic -------------------------------------------------------------------
template <class T> inline tvec2<T> operator+(tvec2<T> a, tvec2<T> b) { return {a.x + b.x, a.y + b.y}; }
template <class T> inline tvec2<T> operator/(tvec2<T> a, tvec2<T> b) { return {a.x / b.x, a.y / b.y}; }
template <class T> inline tvec2<T> operator*(tvec2<T> a, double s) { return {a.x * T(s), a.y * T(s)}; }
template <class T> inline tvec2<T> operator-(tvec2<T> a, double s) { return {a.x - T(s), a.y - T(s)}; }

// ---- vec3 arithmetic (component-wise, left to right) -----------------------------------
template <class T> inline tvec3<T> operator+(tvec3<T> a, tvec3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline tvec3<T> operator-(tvec3<T> a, tvec3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline tvec3<T> operator*(tvec3<T> a, tvec3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> inline tvec3<T> operator/(tvec3<T> a, tvec3<T> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class T> inline tvec3<T> operator-(tvec3<T> a) { return {-a.x, -a.y, -a.z}; }
// vec3 (op) scalar and scalar (op) vec3: the scalar is converted to the vector's type first,
// as GLSL and glm do (a float literal times a dvec3 is computed in double).
template <class T, class S> inline tvec3<T> operator*(tvec3<T> a, S s) { T t = T(s); return {a.x * t, a.y * t, a.z * t}; }
template <class T, class S> inline tvec3<T> operator*(S s, tvec3<T> a) { T t = T(s); return {t * a.x, t * a.y, t * a.z}; }
template <class T, class S> inline tvec3<T> operator/(tvec3<T> a, S s) { T t = T(s); return {a.x / t, a.y / t, a.z / t}; }
template <class T, class S> inline tvec3<T> operator+(tvec3<T> a, S s) { T t = T(s); return {a.x + t, a.y + t, a.z + t}; }
template <class T, class S> inline tvec3<T> operator-(tvec3<T> a, S s) { T t = T(s); return {a.x - t, a.y - t, a.z - t}; }
template <class T> inline tvec3<T>& operator+=(tvec3<T>& a, tvec3<T> b) { a = a + b; return a; }
template <class T> inline bool operator==(tvec3<T> a, tvec3<T> b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
template <class T> inline bool operator!=(tvec3<T> a, tvec3<T> b) { return !(a == b); }

// ---- scalar functions (glm semantics) --------------------------------------------------
template <class T> inline T gmin(T x, T y) { return (y < x) ? y : x; }
template <class T> inline T gmax(T x, T y) { return (x < y) ? y : x; }
template <class T> inline T gabs(T x) { return x >= T(0) ? x : -x; }

// ---- geometric functions (glm semantics) -----------------------------------------------
template <class T> inline T dot(tvec3<T> a, tvec3<T> b) {
    tvec3<T> t = a * b;
    return t.x + t.y + t.z;
}
template <class T> inline T length(tvec3<T> v) { return std::sqrt(dot(v, v)); }
template <class T> inline tvec3<T> normalize(tvec3<T> v) { return v * (T(1) / std::sqrt(dot(v, v))); }
template <class T> inline tvec3<T> cross(tvec3<T> x, tvec3<T> y) {
    return tvec3<T>(x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y);
}
template <class T> inline tvec3<T> vmin(tvec3<T> a, tvec3<T> b) { return {gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)}; }
template <class T> inline tvec3<T> vmax(tvec3<T> a, tvec3<T> b) { return {gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)}; }
template <class T> inline tvec3<T> vabs(tvec3<T> a) { return {gabs(a.x), gabs(a.y), gabs(a.z)}; }

// ---- mat4, column major as in GLSL and glm ---------------------------------------------
template <class T> struct tmat4 {
    tvec4<T> c[4];
    tmat4() = default;
    tmat4(tvec4<T> c0, tvec4<T> c1, tvec4<T> c2, tvec4<T> c3) { c[0] = c0; c[1] = c1; c[2] = c2; c[3] = c3; }
    tvec4<T>& operator[](int i) { return c[i]; }
    const tvec4<T>& operator[](int i) const { return c[i]; }
};

// M * v = sum_i column_i * v_i, accumulated in column order (as glm's operator*).
template <class T> inline tvec4<T> operator*(const tmat4<T>& m, tvec4<T> v) {
    tvec4<T> r;
    for (int k = 0; k < 4; ++k)
        r[k] = ((m.c[0][k] * v.x + m.c[1][k] * v.y) + m.c[2][k] * v.z) + m.c[3][k] * v.w;
    return r;
}

// Inverse by the adjugate: 2x2 sub-determinants of the lower and upper column pairs, then
// cofactors, then division of each by the determinant (written from the Laplace expansion).
template <class T> inline tmat4<T> inverse(const tmat4<T>& m) {
    auto a = [&](int col, int row) { return m.c[col][row]; };
    // sub-determinants of rows (0,1) and rows (2,3) for each column pair
    T s0 = a(0, 0) * a(1, 1) - a(1, 0) * a(0, 1);
    T s1 = a(0, 0) * a(2, 1) - a(2, 0) * a(0, 1);
    T s2 = a(0, 0) * a(3, 1) - a(3, 0) * a(0, 1);
    T s3 = a(1, 0) * a(2, 1) - a(2, 0) * a(1, 1);
    T s4 = a(1, 0) * a(3, 1) - a(3, 0) * a(1, 1);
    T s5 = a(2, 0) * a(3, 1) - a(3, 0) * a(2, 1);
    T c5 = a(2, 2) * a(3, 3) - a(3, 2) * a(2, 3);
    T c4 = a(1, 2) * a(3, 3) - a(3, 2) * a(1, 3);
    T c3 = a(1, 2) * a(2, 3) - a(2, 2) * a(1, 3);
    T c2 = a(0, 2) * a(3, 3) - a(3, 2) * a(0, 3);
    T c1 = a(0, 2) * a(2, 3) - a(2, 2) * a(0, 3);
    T c0 = a(0, 2) * a(1, 3) - a(1, 2) * a(0, 3);
    T det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    T inv = T(1) / det;
    tmat4<T> r;
    // r[col][row]: entry (row, col) of the inverse = cofactor (col, row) / det
    r.c[0][0] = ( a(1, 1) * c5 - a(2, 1) * c4 + a(3, 1) * c3) * inv;
    r.c[1][0] = (-a(1, 0) * c5 + a(2, 0) * c4 - a(3, 0) * c3) * inv;
    r.c[2][0] = ( a(1, 3) * s5 - a(2, 3) * s4 + a(3, 3) * s3) * inv;
    r.c[3][0] = (-a(1, 2) * s5 + a(2, 2) * s4 - a(3, 2) * s3) * inv;
    r.c[0][1] = (-a(0, 1) * c5 + a(2, 1) * c2 - a(3, 1) * c1) * inv;
    r.c[1][1] = ( a(0, 0) * c5 - a(2, 0) * c2 + a(3, 0) * c1) * inv;
    r.c[2][1] = (-a(0, 3) * s5 + a(2, 3) * s2 - a(3, 3) * s1) * inv;
    r.c[3][1] = ( a(0, 2) * s5 - a(2, 2) * s2 + a(3, 2) * s1) * inv;
    r.c[0][2] = ( a(0, 1) * c4 - a(1, 1) * c2 + a(3, 1) * c0) * inv;
    r.c[1][2] = (-a(0, 0) * c4 + a(1, 0) * c2 - a(3, 0) * c0) * inv;
    r.c[2][2] = ( a(0, 3) * s4 - a(1, 3) * s2 + a(3, 3) * s0) * inv;
    r.c[3][2] = (-a(0, 2) * s4 + a(1, 2) * s2 - a(3, 2) * s0) * inv;
    r.c[0][3] = (-a(0, 1) * c3 + a(1, 1) * c1 - a(2, 1) * c0) * inv;
    r.c[1][3] = ( a(0, 0) * c3 - a(1, 0) * c1 + a(2, 0) * c0) * inv;
    r.c[2][3] = (-a(0, 3) * s3 + a(1, 3) * s1 - a(2, 3) * s0) * inv;
    r.c[3][3] = ( a(0, 2) * s3 - a(1, 2) * s1 + a(2, 2) * s0) * inv;
    return r;
}

}  // namespace shim

// Declares, inside the current namespace, the GLSL vocabulary for scalar type REAL. Used once
// per precision so that the same shader text compiles in FP32 and FP64.
#define SHIM_GLSL_VOCABULARY(REAL)                                                             \
    using vec2 = ::shim::tvec2<REAL>;                                                          \
    using vec3 = ::shim::tvec3<REAL>;                                                          \
    using vec4 = ::shim::tvec4<REAL>;                                                          \
    using mat4 = ::shim::tmat4<REAL>;                                                          \
    using uint = uint32_t;                                                                     \
    using ::shim::uvec2;                                                                       \
    using ::shim::uvec3;                                                                       \
    using ::shim::dot;                                                                         \
    using ::shim::cross;                                                                       \
    using ::shim::length;                                                                      \
    using ::shim::normalize;                                                                   \
    using ::shim::inverse;                                                                     \
    inline REAL sqrt(REAL x) { return std::sqrt(x); }                                          \
    inline REAL abs(REAL x) { return ::shim::gabs(x); }                                        \
    inline vec3 abs(vec3 x) { return ::shim::vabs(x); }                                        \
    inline REAL min(REAL x, REAL y) { return ::shim::gmin(x, y); }                             \
    inline REAL max(REAL x, REAL y) { return ::shim::gmax(x, y); }
