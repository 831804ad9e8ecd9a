// workload.cpp -- host code that defines a traced workload: seeded synthetic hair strands (the
// reference loads Claire's glTF hair through assimp, source/resources/model/model_loader.cpp:274-336;
// those assets are not available, so strands of the same kind are generated) and the camera
// matrices (FlyCamera, source/fly_camera.cpp:25-35). Compiled with -ffp-contract=off; the strand
// generator is free of libm transcendental calls, so its output is bit-identical on every host.
// The CPU oracle's library compiles this same file, so that a CPU-only run traces exactly the
// strands and cameras the GPU library would.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <utility>

#include "hrt.h"

namespace {

const double kPi = 3.14159265358979323846;

// sin on [-pi/2, pi/2] by its Taylor series to x^23 (truncation error < 1e-20 there).
double sin_core(double x) {
    double x2 = x * x;
    double term = x, sum = x;
    for (int k = 1; k <= 11; ++k) {
        term = -term * x2 / double((2 * k) * (2 * k + 1));
        sum = sum + term;
    }
    return sum;
}
double sin_det(double x) {
    double r = x - 2.0 * kPi * std::floor(x / (2.0 * kPi) + 0.5);  // [-pi, pi]
    if (r > 0.5 * kPi) r = kPi - r;
    else if (r < -0.5 * kPi) r = -kPi - r;
    return sin_core(r);
}
double cos_det(double x) { return sin_det(x + 0.5 * kPi); }

// splitmix64 (Vigna): a 64-bit state stepped by the golden-ratio increment, then mixed.
uint64_t splitmix(uint64_t& s) {
    s += 0x9E3779B97F4A7C15ULL;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
double unit(uint64_t& s) { return double(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

struct D3 { double x, y, z; };
D3 add(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
D3 scale(D3 a, double k) { return {a.x * k, a.y * k, a.z * k}; }
D3 crs(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
D3 nrm(D3 a) {
    double l = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return {a.x / l, a.y / l, a.z / l};
}

}  // namespace

namespace hrt {
// Inverse of a column-major 4x4 matrix in double: Gauss-Jordan elimination with partial
// pivoting on the row-major copy [A | I].
bool invert4(const double* m, double* out) {
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            a[r][c] = m[4 * c + r];
            a[r][4 + c] = r == c ? 1.0 : 0.0;
        }
    for (int col = 0; col < 4; ++col) {
        int piv = col;
        for (int r = col + 1; r < 4; ++r)
            if (std::fabs(a[r][col]) > std::fabs(a[piv][col])) piv = r;
        if (!(std::fabs(a[piv][col]) > 0.0) || !std::isfinite(a[piv][col])) return false;
        if (piv != col)
            for (int c = 0; c < 8; ++c) std::swap(a[piv][c], a[col][c]);
        double d = a[col][col];
        for (int c = 0; c < 8; ++c) a[col][c] /= d;
        for (int r = 0; r < 4; ++r) {
            if (r == col || a[r][col] == 0.0) continue;
            double f = a[r][col];
            for (int c = 0; c < 8; ++c) a[r][c] -= f * a[col][c];
        }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[4 * c + r] = a[r][4 + c];
    return true;
}
}  // namespace hrt

extern "C" {

hrt_status hrt_camera_look_at(const float eye[3], const float center[3], const float up[3], float fovy_deg,
                              float aspect, float znear, float zfar, hrt_camera* out) {
    if (!eye || !center || !up || !out || !(aspect > 0.0f) || !(zfar > znear) || !(fovy_deg > 0.0f) ||
        !(fovy_deg < 180.0f))
        return HRT_ERR_INVALID_ARG;
    // glm::lookAtRH: f = normalize(center - eye), s = normalize(cross(f, up)), u = cross(s, f)
    double e[3] = {eye[0], eye[1], eye[2]}, c[3] = {center[0], center[1], center[2]}, u0[3] = {up[0], up[1], up[2]};
    double f[3] = {c[0] - e[0], c[1] - e[1], c[2] - e[2]};
    double fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    if (!(fl > 0.0)) return HRT_ERR_INVALID_ARG;
    for (double& x : f) x /= fl;
    double s[3] = {f[1] * u0[2] - f[2] * u0[1], f[2] * u0[0] - f[0] * u0[2], f[0] * u0[1] - f[1] * u0[0]};
    double sl = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    if (!(sl > 0.0)) return HRT_ERR_INVALID_ARG;
    for (double& x : s) x /= sl;
    double u[3] = {s[1] * f[2] - s[2] * f[1], s[2] * f[0] - s[0] * f[2], s[0] * f[1] - s[1] * f[0]};
    double V[16] = {0};
    V[0] = s[0]; V[4] = s[1]; V[8] = s[2];
    V[1] = u[0]; V[5] = u[1]; V[9] = u[2];
    V[2] = -f[0]; V[6] = -f[1]; V[10] = -f[2];
    V[12] = -(s[0] * e[0] + s[1] * e[1] + s[2] * e[2]);
    V[13] = -(u[0] * e[0] + u[1] * e[1] + u[2] * e[2]);
    V[14] = f[0] * e[0] + f[1] * e[1] + f[2] * e[2];
    V[15] = 1.0;
    // glm::perspectiveRH_ZO, then [1][1] *= -1 (fly_camera.cpp:32-33)
    double th = std::tan(double(fovy_deg) * 3.14159265358979323846 / 360.0);
    double P[16] = {0};
    P[0] = 1.0 / (double(aspect) * th);
    P[5] = -(1.0 / th);
    P[10] = double(zfar) / (double(znear) - double(zfar));
    P[11] = -1.0;
    P[14] = -(double(zfar) * double(znear)) / (double(zfar) - double(znear));
    double Vi[16], Pi[16];
    if (!hrt::invert4(V, Vi) || !hrt::invert4(P, Pi)) return HRT_ERR_INVALID_ARG;
    for (int k = 0; k < 16; ++k) {
        out->view_inverse[k] = float(Vi[k]);
        out->proj_inverse[k] = float(Pi[k]);
    }
    return HRT_OK;
}

void hrt_strand_params_default(hrt_strand_params* p) {
    memset(p, 0, sizeof(*p));
    p->seed = 1001;
    p->nstrands = 2000;
    p->nverts = 32;
    p->step = 0.05f;
    p->droop = 0.02f;
    p->curl = 0.01f;
    p->curl_freq = 0.7f;
    p->r_root = 0.004f;
    p->r_tip = 0.001f;
    p->cap_deg = 60.0f;
}

hrt_status hrt_generate_strands(const hrt_strand_params* p, float* vertices, float* radius, uint32_t* offsets) {
    if (!p || !vertices || p->nverts < 2 || p->nstrands == 0) return HRT_ERR_INVALID_ARG;
    if (uint64_t(p->nstrands) * p->nverts >= (1ull << 32)) return HRT_ERR_UNSUPPORTED;
    const double cos_cap = cos_det(double(p->cap_deg) * kPi / 180.0);
    const uint32_t V = p->nverts;
    for (uint32_t s = 0; s < p->nstrands; ++s) {
        uint64_t st = p->seed ^ (0xD1B54A32D192ED03ULL * (uint64_t(s) + 1));
        double u1 = unit(st), u2 = unit(st), u3 = unit(st);
        double ct = 1.0 - u1 * (1.0 - cos_cap);  // uniform in area on the cap
        double sn = std::sqrt(ct * ct < 1.0 ? 1.0 - ct * ct : 0.0);
        double phi = 2.0 * kPi * u2, phase = 2.0 * kPi * u3;
        D3 n = {sn * cos_det(phi), ct, sn * sin_det(phi)};
        D3 a = std::fabs(n.z) < 0.9 ? D3{0.0, 0.0, 1.0} : D3{1.0, 0.0, 0.0};
        D3 b1 = nrm(crs(n, a));
        D3 b2 = crs(n, b1);
        D3 pos = n;
        uint64_t base = uint64_t(s) * V;
        for (uint32_t k = 0; k < V; ++k) {
            D3 v = pos;
            if (k > 0) {
                double ang = double(p->curl_freq) * double(k) + phase;
                v = add(v, scale(add(scale(b1, sin_det(ang)), scale(b2, cos_det(ang))), double(p->curl)));
            }
            vertices[3 * (base + k)] = float(v.x);
            vertices[3 * (base + k) + 1] = float(v.y);
            vertices[3 * (base + k) + 2] = float(v.z);
            if (radius)
                radius[base + k] =
                    float(double(p->r_root) + (double(p->r_tip) - double(p->r_root)) * double(k) / double(V - 1));
            D3 dir = nrm(D3{n.x, n.y - double(p->droop) * double(k), n.z});
            pos = add(pos, scale(dir, double(p->step)));
        }
        if (offsets) offsets[s] = uint32_t(base);
    }
    if (offsets) offsets[p->nstrands] = uint32_t(uint64_t(p->nstrands) * V);
    return HRT_OK;
}

uint64_t hrt_checksum(const void* a, uint64_t abytes, const void* b, uint64_t bbytes) {
    uint64_t h = 0xcbf29ce484222325ULL;  // FNV-1a 64
    const unsigned char* pa = static_cast<const unsigned char*>(a);
    for (uint64_t i = 0; pa && i < abytes; ++i) { h ^= pa[i]; h *= 0x100000001b3ULL; }
    const unsigned char* pb = static_cast<const unsigned char*>(b);
    for (uint64_t i = 0; pb && i < bbytes; ++i) { h ^= pb[i]; h *= 0x100000001b3ULL; }
    return h;
}

}  // extern "C"
