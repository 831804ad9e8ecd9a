// build.cu -- device BVH build for one BLAS: geometry processing, LBVH, BVH8 collapse, encoding.
//
// Compiled with --fmad=false: every float operation is a separately rounded IEEE operation and
// division / square root are correctly rounded, so each stage is bit-identical to the CPU
// restatement (compiled with -ffp-contract=off) on the same inputs.
//
// Pipeline (one stream, temporaries from the stream-ordered allocator):
//   lines -> per type: Bezier curves (GenerateCurves, geometry_processor.cpp:123-156) and, for
//   the quantised format, the strand vertex stream | LSS spheres (:273-298) | DOTS frames
//   (:201-271) -> primitive boxes -> centroid bounds -> 63-bit Morton codes -> stable LSD radix
//   sort (8 passes of 8 bits) -> Karras hierarchy -> bottom-up refit -> greedy surface-area
//   collapse to BVH8, breadth first -> FP32 and 8-bit quantised node encodings -> primitive
//   records in leaf-slot order.
#include <cuda_fp16.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "hrt_internal.h"

namespace hrt {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float fmin_t(float a, float b) { return (b < a) ? b : a; }  // glm::min
__device__ __forceinline__ float fmax_t(float a, float b) { return (a < b) ? b : a; }  // glm::max

struct f3 { float x, y, z; };
__device__ __forceinline__ f3 ld3(const float* p) { return {p[0], p[1], p[2]}; }
__device__ __forceinline__ void st3(float* p, f3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ bool operator==(f3 a, f3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
// glm: dot = (x*x' + y*y') + z*z'; normalize = v * (1 / sqrt(dot(v, v)))
__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 normalize3(f3 v) { return v * (1.0f / sqrtf(dot3(v, v))); }
__device__ __forceinline__ f3 cross3(f3 x, f3 y) {
    return {x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y};
}
__device__ __forceinline__ float gabs(float x) { return x >= 0.0f ? x : -x; }

inline unsigned grid_for(uint64_t n, unsigned threads) { return unsigned((n + threads - 1) / threads); }

// ================================ scans ===========================================================
constexpr int kScanThreads = 256, kScanItems = 4, kScanTile = kScanThreads * kScanItems;
struct SumOp {
    __device__ static uint32_t id() { return 0u; }
    __device__ uint32_t operator()(uint32_t a, uint32_t b) const { return a + b; }
};
struct MaxOp {
    __device__ static uint32_t id() { return 0u; }
    __device__ uint32_t operator()(uint32_t a, uint32_t b) const { return a > b ? a : b; }
};

template <class Op>
__device__ uint32_t block_inclusive(uint32_t v, uint32_t* sm, uint32_t* total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    Op op;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t n = __shfl_up_sync(kFull, v, o);
        if (lane >= o) v = op(n, v);
    }
    if (lane == 31) sm[w] = v;
    __syncthreads();
    if (w == 0) {
        uint32_t s = lane < nw ? sm[lane] : Op::id();
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t n = __shfl_up_sync(kFull, s, o);
            if (lane >= o) s = op(n, s);
        }
        sm[lane] = s;
    }
    __syncthreads();
    if (w > 0) v = op(sm[w - 1], v);
    *total = sm[nw - 1];
    __syncthreads();
    return v;
}

template <class Op>
__global__ void scan_reduce_kernel(const uint32_t* in, uint64_t n, uint32_t* sums) {
    __shared__ uint32_t sm[32];
    Op op;
    uint64_t base = uint64_t(blockIdx.x) * kScanTile + uint64_t(threadIdx.x) * kScanItems;
    uint32_t acc = Op::id();
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) acc = op(acc, in[base + k]);
    uint32_t total;
    block_inclusive<Op>(acc, sm, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

template <class Op>
__global__ void scan_apply_kernel(const uint32_t* in, uint32_t* out, uint64_t n, const uint32_t* prefix,
                                  bool inclusive, uint32_t* grand_total) {
    __shared__ uint32_t sm[32];
    Op op;
    uint64_t base = uint64_t(blockIdx.x) * kScanTile + uint64_t(threadIdx.x) * kScanItems;
    uint32_t v[kScanItems];
    uint32_t acc = Op::id();
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < n ? in[base + k] : Op::id();
        acc = op(acc, v[k]);
    }
    uint32_t total;
    uint32_t incl = block_inclusive<Op>(acc, sm, &total);
    uint32_t pre = prefix ? prefix[blockIdx.x] : Op::id();
    __shared__ uint32_t s_incl[kScanThreads];
    s_incl[threadIdx.x] = incl;
    __syncthreads();
    uint32_t excl_block = threadIdx.x > 0 ? s_incl[threadIdx.x - 1] : Op::id();
    uint32_t run;
    run = op(pre, excl_block);
    for (int k = 0; k < kScanItems; ++k) {
        uint32_t before = run;
        run = op(run, v[k]);
        if (base + k < n) out[base + k] = inclusive ? run : before;
    }
    if (grand_total && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *grand_total = op(pre, total);
}

// Scan of n uint32 values (exclusive or inclusive) with Op; optional device grand total.
template <class Op>
cudaError_t device_scan(const uint32_t* in, uint32_t* out, uint64_t n, bool inclusive, uint32_t* grand_total,
                        cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    uint64_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 1) {
        scan_apply_kernel<Op><<<1, kScanThreads, 0, s>>>(in, out, n, nullptr, inclusive, grand_total);
        return cudaGetLastError();
    }
    uint32_t* sums = nullptr;
    cudaError_t e = cudaMallocAsync(&sums, nb * sizeof(uint32_t) * 2, s);
    if (e != cudaSuccess) return e;
    uint32_t* pre = sums + nb;
    scan_reduce_kernel<Op><<<unsigned(nb), kScanThreads, 0, s>>>(in, n, sums);
    e = device_scan<Op>(sums, pre, nb, false, nullptr, s);
    if (e == cudaSuccess) {
        scan_apply_kernel<Op><<<unsigned(nb), kScanThreads, 0, s>>>(in, out, n, pre, inclusive, grand_total);
        e = cudaGetLastError();
    }
    cudaFreeAsync(sums, s);
    return e;
}

// ================================ lines ===========================================================
__global__ void lines_from_strands_kernel(const float* v, const float* vr, float cr, const uint32_t* line_off,
                                          const uint32_t* vert_off, uint64_t nstrands, uint64_t nlines,
                                          float* lines, float* lrad) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= nlines) return;
    uint64_t lo = 0, hi = nstrands;  // largest s with line_off[s] <= i
    while (hi - lo > 1) {
        uint64_t mid = (lo + hi) / 2;
        if (line_off[mid] <= i) lo = mid; else hi = mid;
    }
    uint64_t a = uint64_t(vert_off[lo]) + (i - line_off[lo]);
    uint64_t b = a + 1;
    for (int k = 0; k < 3; ++k) { lines[6 * i + k] = v[3 * a + k]; lines[6 * i + 3 + k] = v[3 * b + k]; }
    lrad[2 * i] = vr ? vr[a] : cr;
    lrad[2 * i + 1] = vr ? vr[b] : cr;
}

__global__ void lines_from_indices_kernel(const float* v, const float* vr, float cr, const uint32_t* idx,
                                          uint64_t nlines, float* lines, float* lrad) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= nlines) return;
    uint64_t a = idx[2 * i], b = idx[2 * i + 1];
    for (int k = 0; k < 3; ++k) { lines[6 * i + k] = v[3 * a + k]; lines[6 * i + 3 + k] = v[3 * b + k]; }
    lrad[2 * i] = vr ? vr[a] : cr;
    lrad[2 * i + 1] = vr ? vr[b] : cr;
}

// ============================ geometry processing =================================================
// GenerateCurves geometry_processor.cpp:123-156, tension 1: neighbours by exact point equality.
__global__ void curves_kernel(const float* lines, uint64_t n, float* curves) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* L = lines + 6 * i;
    f3 p1 = ld3(L), p2 = ld3(L + 3);
    uint64_t prev = (i > 0 && ld3(lines + 6 * (i - 1) + 3) == p1) ? i - 1 : i;
    uint64_t next = (i + 1 < n && p2 == ld3(lines + 6 * (i + 1))) ? i + 1 : i;
    f3 p0 = ld3(lines + 6 * prev), p3 = ld3(lines + 6 * next + 3);
    const float k = 1.0f / 6.0f;
    float* c = curves + 12 * i;
    st3(c, p1);
    st3(c + 3, p1 + (p2 - p0) * k);
    st3(c + 6, p2 - (p3 - p1) * k);
    st3(c + 9, p2);
}

// Quantised Phantom geometry: the strand vertex stream. A stream run is a maximal range of
// lines in which every line starts where the previous one ends (exact equality, the neighbour
// rule of GenerateCurves) with the same radius at the joint. Run r of lines [a, b) occupies the
// b - a + 3 entries from a + 3 r: the point before it (the previous line's start when that line
// joins it geometrically, otherwise its own start), its start, the end of each of its lines, and
// the point after it (the next line's end when that line joins it, otherwise its own end); each
// entry is {x, y, z, radius at the point}. Line i of run r has entry e = i + 3 r, and its
// GenerateCurves neighbours p0, p1, p2, p3 are entries e .. e + 3, so the leaf test rebuilds the
// line's Bezier control points from the FP32 vertices with the curve kernel's operations, bit for
// bit.
__global__ void stream_flags_kernel(const float* lines, const float* lrad, uint64_t n, uint32_t* flags) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool joined = i > 0 && ld3(lines + 6 * (i - 1) + 3) == ld3(lines + 6 * i) && lrad[2 * i - 1] == lrad[2 * i];
    flags[i] = joined ? 0u : 1u;
}
// run_incl: inclusive scan of the flags (run index + 1); writes the entries and line_entry[i].
__global__ void stream_kernel(const float* lines, const float* lrad, const uint32_t* flags, const uint32_t* run_incl,
                              uint64_t n, float4* verts, uint32_t* line_entry) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t e = i + 3ull * (run_incl[i] - 1u);
    line_entry[i] = uint32_t(e);
    const float* L = lines + 6 * i;
    if (flags[i]) {  // first line of its run: the point before it and its start
        const bool geo_prev = i > 0 && ld3(lines + 6 * (i - 1) + 3) == ld3(L);
        const float* q = geo_prev ? lines + 6 * (i - 1) : L;
        verts[e] = make_float4(q[0], q[1], q[2], lrad[2 * i]);
        verts[e + 1] = make_float4(L[0], L[1], L[2], lrad[2 * i]);
    }
    verts[e + 2] = make_float4(L[3], L[4], L[5], lrad[2 * i + 1]);
    if (i + 1 == n || flags[i + 1]) {  // last line of its run: the point after it
        const bool geo_next = i + 1 < n && ld3(L + 3) == ld3(lines + 6 * (i + 1));
        const float* q = geo_next ? lines + 6 * (i + 1) + 3 : L + 3;
        verts[e + 3] = make_float4(q[0], q[1], q[2], lrad[2 * i + 1]);
    }
}

// GenerateLinearSweptSpheres geometry_processor.cpp:273-298: radius glm::max(r, 0.001).
__global__ void lss_kernel(const float* lines, const float* lrad, uint64_t n, float* geom) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float* g = geom + 8 * i;
    for (int k = 0; k < 6; ++k) g[k] = lines[6 * i + k];
    g[6] = fmax_t(lrad[2 * i], 0.001f);
    g[7] = fmax_t(lrad[2 * i + 1], 0.001f);
}

// PerpStark geometry_processor.cpp:201-212
__device__ f3 perp_stark(f3 u) {
    f3 a = {gabs(u.x), gabs(u.y), gabs(u.z)};
    uint32_t uyx = (a.x - a.y) < 0 ? 1 : 0;
    uint32_t uzx = (a.x - a.z) < 0 ? 1 : 0;
    uint32_t uzy = (a.y - a.z) < 0 ? 1 : 0;
    uint32_t xm = uyx & uzx;
    uint32_t ym = (1 ^ xm) & uzy;
    uint32_t zm = 1 ^ (xm | ym);
    return normalize3(cross3(u, f3{float(xm), float(ym), float(zm)}));
}
// DOTS frame per segment (geometry_processor.cpp:237-265): geom = start, end, s*ra, t*ra,
// s*rb, t*rb; the reference's vertices are start +- v*ra and end +- v*rb.
__global__ void dots_kernel(const float* lines, const float* lrad, uint64_t n, float* geom) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    f3 s0 = ld3(lines + 6 * i), e0 = ld3(lines + 6 * i + 3);
    float ra = lrad[2 * i], rb = lrad[2 * i + 1];
    f3 fwd = normalize3(e0 - s0);
    f3 s = perp_stark(fwd);
    f3 t = cross3(fwd, s);
    float* g = geom + 18 * i;
    st3(g, s0);
    st3(g + 3, e0);
    st3(g + 6, s * ra);
    st3(g + 9, t * ra);
    st3(g + 12, s * rb);
    st3(g + 15, t * rb);
}

// ============================== primitive boxes ==================================================
// Phantom: hull +- max(r0, r1) (GenerateAABBs :431-432); LSS: spheres; DOTS: 12 vertices in
// the reference's order.
__global__ void boxes_phantom_kernel(const float* curves, const float* rad, uint64_t n, float* boxes) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* c = curves + 12 * i;
    float r = fmax_t(rad[2 * i], rad[2 * i + 1]);
    for (int k = 0; k < 3; ++k) {
        boxes[6 * i + k] = fmin_t(fmin_t(c[k], c[9 + k]), fmin_t(c[3 + k], c[6 + k])) - r;
        boxes[6 * i + 3 + k] = fmax_t(fmax_t(c[k], c[9 + k]), fmax_t(c[3 + k], c[6 + k])) + r;
    }
}
// LSS: two references per segment (see ref_shift). The round cone is the union of the spheres
// a + u (b - a) with radius ra + u (rb - ra), so its half u <= 1/2 lies in the hull of the end
// sphere at a and the sphere at the midpoint m, radius rm = (ra + rb) / 2; m and rm are computed
// once and bound both halves, so the two boxes meet without a gap.
__global__ void boxes_lss_kernel(const float* geom, uint64_t n, float* boxes) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* g = geom + 8 * i;
    const float ra = g[6], rb = g[7], rm = 0.5f * (ra + rb);
    for (int k = 0; k < 3; ++k) {
        const float m = 0.5f * (g[k] + g[3 + k]);
        boxes[12 * i + k] = fmin_t(g[k] - ra, m - rm);
        boxes[12 * i + 3 + k] = fmax_t(g[k] + ra, m + rm);
        boxes[12 * i + 6 + k] = fmin_t(m - rm, g[3 + k] - rb);
        boxes[12 * i + 9 + k] = fmax_t(m + rm, g[3 + k] + rb);
    }
}
__device__ void dots_vertices(const float* g, float* v36) {
    f3 s0 = ld3(g), e0 = ld3(g + 3);
    for (int face = 0; face < 2; ++face) {
        f3 va = ld3(g + 6 + 3 * face), vb = ld3(g + 12 + 3 * face);
        float* o = v36 + 18 * face;
        st3(o + 0, s0 + va);
        st3(o + 3, e0 - vb);
        st3(o + 6, e0 + vb);
        st3(o + 9, s0 + va);
        st3(o + 12, s0 - va);
        st3(o + 15, e0 - vb);
    }
}
// DOTS: two references per segment (see ref_shift). Each quad is a trapezoid, s0 +- va at the
// start and e0 +- vb at the end (vertices 0, 4 and 2, 1 of its six), whose width is linear
// along the segment, so its first half is the hull of the start edge and the edge midpoints
// (v0 + v2) / 2, (v4 + v1) / 2, and its second half the hull of those midpoints and the end
// edge; the midpoints are shared by both halves.
__global__ void boxes_dots_kernel(const float* geom, uint64_t n, float* boxes) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float v[36];
    dots_vertices(geom + 18 * i, v);
    for (int k = 0; k < 3; ++k) {
        float lo0 = __int_as_float(0x7f800000), hi0 = -lo0, lo1 = lo0, hi1 = hi0;
        for (int face = 0; face < 2; ++face) {
            const float* f = v + 18 * face;
            const float a = f[k], b = f[12 + k], c = f[6 + k], d = f[3 + k];  // v0, v4, v2, v1
            const float mp = 0.5f * (a + c), mm = 0.5f * (b + d);
            lo0 = fmin_t(lo0, fmin_t(fmin_t(a, b), fmin_t(mp, mm)));
            hi0 = fmax_t(hi0, fmax_t(fmax_t(a, b), fmax_t(mp, mm)));
            lo1 = fmin_t(lo1, fmin_t(fmin_t(mp, mm), fmin_t(c, d)));
            hi1 = fmax_t(hi1, fmax_t(fmax_t(mp, mm), fmax_t(c, d)));
        }
        boxes[12 * i + k] = lo0;
        boxes[12 * i + 3 + k] = hi0;
        boxes[12 * i + 6 + k] = lo1;
        boxes[12 * i + 9 + k] = hi1;
    }
}
// Mesh triangle box: min/max of the three vertices, in vertex order.
__global__ void boxes_tri_kernel(const float* tris, uint64_t n, float* boxes) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* v = tris + 9 * i;
    for (int k = 0; k < 3; ++k) {
        boxes[6 * i + k] = fmin_t(fmin_t(v[k], v[3 + k]), v[6 + k]);
        boxes[6 * i + 3 + k] = fmax_t(fmax_t(v[k], v[3 + k]), v[6 + k]);
    }
}
__global__ void tris_kernel(const float* verts, const float* vnrm, const uint32_t* idx, uint64_t n, float* tris,
                            float* tri_nrm) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int j = 0; j < 3; ++j) {
        const uint64_t v = idx[3 * i + j];
        for (int k = 0; k < 3; ++k) {
            tris[9 * i + 3 * j + k] = verts[3 * v + k];
            if (tri_nrm) tri_nrm[9 * i + 3 * j + k] = vnrm[3 * v + k];
        }
    }
}
__global__ void expand_dots_kernel(const float* geom, uint64_t n, float* out36) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dots_vertices(geom + 18 * i, out36 + 36 * i);
}

// ================================ Morton codes ===================================================
__device__ __forceinline__ uint32_t f2ord(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}
__global__ void centroid_bounds_kernel(const float* boxes, uint64_t n, uint32_t* ob /*6: min xyz, max xyz*/) {
    __shared__ uint32_t s[6];
    if (threadIdx.x < 3) s[threadIdx.x] = 0xffffffffu;
    else if (threadIdx.x < 6) s[threadIdx.x] = 0u;
    __syncthreads();
    uint32_t lmin[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, lmax[3] = {0, 0, 0};
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
        for (int k = 0; k < 3; ++k) {
            float cf = (boxes[6 * i + k] + boxes[6 * i + 3 + k]) * 0.5f;
            if (!(cf == cf)) continue;  // NaN centroids (degenerate input) do not widen the bounds
            uint32_t c = f2ord(cf);
            lmin[k] = min(lmin[k], c);
            lmax[k] = max(lmax[k], c);
        }
    for (int k = 0; k < 3; ++k) { atomicMin(&s[k], lmin[k]); atomicMax(&s[3 + k], lmax[k]); }
    __syncthreads();
    if (threadIdx.x < 3) atomicMin(&ob[threadIdx.x], s[threadIdx.x]);
    else if (threadIdx.x < 6) atomicMax(&ob[threadIdx.x], s[threadIdx.x]);
}
__device__ __forceinline__ uint64_t expand21(uint32_t v) {
    uint64_t x = v & 0x1fffff;
    x = (x | (x << 32)) & 0x1f00000000ffffULL;
    x = (x | (x << 16)) & 0x1f0000ff0000ffULL;
    x = (x | (x << 8)) & 0x100f00f00f00f00fULL;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ULL;
    x = (x | (x << 2)) & 0x1249249249249249ULL;
    return x;
}
__global__ void morton_kernel(const float* boxes, uint64_t n, const uint32_t* ob, uint64_t* codes, uint32_t* values) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t code = 0;
    for (int k = 0; k < 3; ++k) {
        float cmin = ord2f(ob[k]), cmax = ord2f(ob[3 + k]);
        float ext = cmax - cmin;
        float scale = ext > 0.0f ? 2097152.0f / ext : 0.0f;
        float c = (boxes[6 * i + k] + boxes[6 * i + 3 + k]) * 0.5f;
        float q = (c - cmin) * scale;
        uint32_t qi = !(q > 0.0f) ? 0u : (q >= 2097151.0f ? 2097151u : uint32_t(q));
        code |= expand21(qi) << (2 - k);
    }
    codes[i] = code;
    values[i] = uint32_t(i);
}

// ================================ radix sort =====================================================
// Stable LSD sort of 64-bit keys with 32-bit values, 8 bits per pass. Per pass: tile histograms
// (digit-major), one exclusive scan, then a stable scatter: each tile is walked in 256-key
// rounds; within a round keys are ranked per warp with __match_any_sync and across warps by a
// per-digit prefix, so equal digits keep their input order.
constexpr int kSortThreads = 256, kSortItems = 8, kSortTile = kSortThreads * kSortItems;

__global__ void __launch_bounds__(kSortThreads) radix_hist_kernel(const uint64_t* keys, uint64_t n, int shift,
                                                                  uint32_t* counts, uint32_t nblocks) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    uint64_t base = uint64_t(blockIdx.x) * kSortTile;
    for (int r = 0; r < kSortItems; ++r) {
        uint64_t i = base + uint64_t(r) * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    counts[uint64_t(threadIdx.x) * nblocks + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kSortThreads) radix_scatter_kernel(const uint64_t* kin, const uint32_t* vin,
                                                                     uint64_t* kout, uint32_t* vout, uint64_t n,
                                                                     int shift, const uint32_t* offsets,
                                                                     uint32_t nblocks) {
    __shared__ uint32_t s_base[256];
    __shared__ uint32_t s_w[8][256];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    s_base[t] = offsets[uint64_t(t) * nblocks + blockIdx.x];
    uint64_t base = uint64_t(blockIdx.x) * kSortTile;
    for (int r = 0; r < kSortItems; ++r) {
        for (int k = t; k < 8 * 256; k += kSortThreads) (&s_w[0][0])[k] = 0;
        __syncthreads();
        uint64_t i = base + uint64_t(r) * kSortThreads + t;
        bool valid = i < n;
        uint64_t key = valid ? kin[i] : 0;
        uint32_t val = valid ? vin[i] : 0;
        uint32_t digit = valid ? uint32_t((key >> shift) & 255u) : 256u;
        uint32_t peers = __match_any_sync(kFull, digit);
        uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && lane == __ffs(peers) - 1) s_w[w][digit] = __popc(peers);
        __syncthreads();
        uint32_t run = s_base[t];
        for (int ww = 0; ww < 8; ++ww) {
            uint32_t c = s_w[ww][t];
            s_w[ww][t] = run;
            run += c;
        }
        s_base[t] = run;
        __syncthreads();
        if (valid) {
            uint32_t pos = s_w[w][digit] + rank;
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
    }
}

cudaError_t radix_sort(uint64_t* keys, uint32_t* vals, uint64_t n, cudaStream_t s) {
    if (n <= 1) return cudaSuccess;
    uint32_t nb = uint32_t((n + kSortTile - 1) / kSortTile);
    uint64_t* k2 = nullptr;
    uint32_t* v2 = nullptr;
    uint32_t* counts = nullptr;
    cudaError_t e = cudaMallocAsync(&k2, n * 8, s);
    if (e == cudaSuccess) e = cudaMallocAsync(&v2, n * 4, s);
    if (e == cudaSuccess) e = cudaMallocAsync(&counts, uint64_t(nb) * 256 * 4 * 2, s);
    uint64_t* ka = keys;
    uint64_t* kb = k2;
    uint32_t* va = vals;
    uint32_t* vb = v2;
    for (int pass = 0; pass < 8 && e == cudaSuccess; ++pass) {
        int shift = 8 * pass;
        radix_hist_kernel<<<nb, kSortThreads, 0, s>>>(ka, n, shift, counts, nb);
        e = device_scan<SumOp>(counts, counts + uint64_t(nb) * 256, uint64_t(nb) * 256, false, nullptr, s);
        if (e != cudaSuccess) break;
        radix_scatter_kernel<<<nb, kSortThreads, 0, s>>>(ka, va, kb, vb, n, shift, counts + uint64_t(nb) * 256, nb);
        e = cudaGetLastError();
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    // 8 passes: the result is back in (keys, vals)
    cudaFreeAsync(k2, s);
    cudaFreeAsync(v2, s);
    cudaFreeAsync(counts, s);
    return e;
}

// ============================ Karras hierarchy + refit ==========================================
__device__ __forceinline__ int delta(const uint64_t* k, int64_t n, int64_t i, int64_t j) {
    if (j < 0 || j >= n) return -1;
    uint64_t a = k[i], b = k[j];
    if (a != b) return __clzll(a ^ b);
    return 64 + __clz(uint32_t(i) ^ uint32_t(j));
}
__global__ void karras_kernel(const uint64_t* k, int64_t n, uint32_t* left, uint32_t* right, uint32_t* first,
                              uint32_t* last, uint32_t* parent_int, uint32_t* parent_leaf) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = (delta(k, n, i, i + 1) - delta(k, n, i, i - 1)) > 0 ? 1 : -1;
    int dmin = delta(k, n, i, i - d);
    int64_t lmax = 2;
    while (delta(k, n, i, i + lmax * d) > dmin) lmax *= 2;
    int64_t l = 0;
    for (int64_t t = lmax / 2; t >= 1; t /= 2)
        if (delta(k, n, i, i + (l + t) * d) > dmin) l += t;
    int64_t j = i + l * d;
    int dnode = delta(k, n, i, j);
    int64_t s = 0;
    for (int64_t div = 2;; div *= 2) {
        int64_t t = (l + div - 1) / div;
        if (delta(k, n, i, i + (s + t) * d) > dnode) s += t;
        if (t == 1) break;
    }
    int64_t g = i + s * d + (d < 0 ? d : 0);
    int64_t lo = i < j ? i : j, hi = i < j ? j : i;
    first[i] = uint32_t(lo);
    last[i] = uint32_t(hi);
    if (lo == g) { left[i] = kLeafFlag | uint32_t(g); parent_leaf[g] = uint32_t(i); }
    else { left[i] = uint32_t(g); parent_int[g] = uint32_t(i); }
    if (hi == g + 1) { right[i] = kLeafFlag | uint32_t(g + 1); parent_leaf[g + 1] = uint32_t(i); }
    else { right[i] = uint32_t(g + 1); parent_int[g + 1] = uint32_t(i); }
}

__global__ void gather_boxes_kernel(const float* boxes, const uint32_t* order, uint64_t n, float* out) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t j = order[i];
    for (int k = 0; k < 6; ++k) out[6 * i + k] = boxes[6 * j + k];
}

// Bottom-up refit: the second thread to reach a node computes union(left, right).
__device__ __forceinline__ float sa_measure(const float* bx) {
    float dx = bx[3] - bx[0], dy = bx[4] - bx[1], dz = bx[5] - bx[2];
    return (dx * dy + dy * dz) + dz * dx;
}

// Bottom-up box refit; the second child to arrive computes its parent. With dpc, the node's
// collapse costs as well (dpc[8 node + k - 1], k = 1..8 slots; see collapse_expand_kernel):
//   dist(k) = min over j = 1..k-1 of cost(left, j) + cost(right, k - j)     (k >= 2)
//   cost(node, 1) = A c if it holds c <= max_leaf primitives (a leaf slot), else A + dist(W)
//   cost(node, k) = min(cost(node, k - 1), dist(k))
// with A the node's surface-area measure and W the node fan-out (width, 8 by default); a
// primitive costs its own measure for every k.
// Node visits and primitive tests are weighted alike.
__global__ void refit_kernel(const uint32_t* parent_leaf, const uint32_t* parent_int, const uint32_t* left,
                             const uint32_t* right, const uint32_t* first, const uint32_t* last, const float* sboxes,
                             float* nboxes, uint32_t* visits, uint64_t n, uint32_t* err, float* dpc, int max_leaf,
                             int width) {
    uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    uint32_t node = parent_leaf[j];
    for (int steps = 0; node != 0xffffffffu; ++steps) {
        if (steps > 200) { atomicOr(err, kErrTimeout); return; }
        __threadfence();
        if (atomicAdd(&visits[node], 1u) == 0u) return;
        __threadfence();
        float b[6], v[2][6];
        uint32_t c[2] = {left[node], right[node]};
        for (int q = 0; q < 2; ++q) {
            const float* src = (c[q] & kLeafFlag) ? sboxes + 6 * uint64_t(c[q] & ~kLeafFlag) : nboxes + 6 * uint64_t(c[q]);
            for (int k = 0; k < 6; ++k) v[q][k] = __ldcg(src + k);
        }
        for (int k = 0; k < 6; ++k) b[k] = v[0][k];
        for (int k = 0; k < 3; ++k) { b[k] = fmin_t(b[k], v[1][k]); b[3 + k] = fmax_t(b[3 + k], v[1][3 + k]); }
        for (int k = 0; k < 6; ++k) __stcg(nboxes + 6 * uint64_t(node) + k, b[k]);
        if (dpc) {
            float cc[2][8];
            for (int q = 0; q < 2; ++q) {
                if (c[q] & kLeafFlag) {
                    const float a = sa_measure(v[q]);
                    for (int k = 0; k < 8; ++k) cc[q][k] = a;
                } else {
                    for (int k = 0; k < 8; ++k) cc[q][k] = __ldcg(dpc + 8 * uint64_t(c[q]) + k);
                }
            }
            float dist[9];
            for (int k = 2; k <= 8; ++k) {
                float best = __int_as_float(0x7f800000);
                for (int i = 1; i < k; ++i) {
                    const float x = cc[0][i - 1] + cc[1][k - i - 1];
                    if (x < best) best = x;
                }
                dist[k] = best;
            }
            const uint32_t cnt = last[node] - first[node] + 1u;
            const float a = sa_measure(b);
            float cost[8];
            cost[0] = cnt <= uint32_t(max_leaf) ? a * float(cnt) : a + dist[width];
            for (int k = 2; k <= 8; ++k) cost[k - 1] = dist[k] < cost[k - 2] ? dist[k] : cost[k - 2];
            for (int k = 0; k < 8; ++k) __stcg(dpc + 8 * uint64_t(node) + k, cost[k]);
        }
        node = parent_int[node];
    }
}

// ============================ collapse to BVH8 ====================================================
struct BinView {
    const uint32_t *left, *right, *first, *last;
    const float* nboxes;  // internal node boxes
    const float* sboxes;  // sorted leaf boxes
    const float* dpc;     // collapse costs, 8 per internal node
};
__device__ __forceinline__ uint32_t bcount(const BinView& b, uint32_t c) {
    return (c & kLeafFlag) ? 1u : b.last[c] - b.first[c] + 1u;
}
__device__ __forceinline__ const float* bbox(const BinView& b, uint32_t c) {
    return (c & kLeafFlag) ? b.sboxes + 6 * uint64_t(c & ~kLeafFlag) : b.nboxes + 6 * uint64_t(c);
}
__device__ __forceinline__ uint32_t bfirst(const BinView& b, uint32_t c) {
    return (c & kLeafFlag) ? (c & ~kLeafFlag) : b.first[c];
}
// cost(c, k) of the collapse (refit_kernel): a primitive costs its measure for every k.
__device__ __forceinline__ float dp_cost(const BinView& b, uint32_t c, int k) {
    return (c & kLeafFlag) ? sa_measure(bbox(b, c)) : __ldg(b.dpc + 8 * uint64_t(c) + (k - 1));
}
// The k slots of internal node x go to its children as j and k - j slots, j the least of the
// minimisers of cost(left, j) + cost(right, k - j).
__device__ __forceinline__ int dp_split(const BinView& b, uint32_t x, int k) {
    const uint32_t l = b.left[x], r = b.right[x];
    int bj = 1;
    float bv = __int_as_float(0x7f800000);
    for (int j = 1; j < k; ++j) {
        const float v = dp_cost(b, l, j) + dp_cost(b, r, k - j);
        if (v < bv) { bv = v; bj = j; }
    }
    return bj;
}

// Children of the wide node made from binary node b, by the collapse costs: b's W slots are
// split between its children; a child given k slots takes the fewest k' <= k of the same
// cost, and with k' > 1 splits them again between its own children (left before right), so the
// children come out in the binary tree's left-to-right order. A child holding at most max_leaf
// primitives becomes a leaf slot; a larger one becomes a wide node of the next level.
__global__ void collapse_expand_kernel(BinView bv, const uint32_t* level, uint32_t count, int max_leaf, int width,
                                       uint32_t* kids, uint32_t* nk, uint32_t* nint, uint32_t* nprim) {
    uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= count) return;
    uint32_t b = level[w];
    uint32_t k[8];
    int n = 0;
    if (b & kLeafFlag) k[n++] = b;
    else {
        uint32_t sx[8];
        int sk[8], sp = 0;
        const int j = dp_split(bv, b, width);
        sx[sp] = bv.right[b]; sk[sp++] = width - j;
        sx[sp] = bv.left[b]; sk[sp++] = j;
        while (sp > 0) {
            const uint32_t x = sx[--sp];
            int kk = sk[sp];
            if (x & kLeafFlag) { k[n++] = x; continue; }
            while (kk > 1 && dp_cost(bv, x, kk) == dp_cost(bv, x, kk - 1)) --kk;
            if (kk == 1) { k[n++] = x; continue; }
            const int jj = dp_split(bv, x, kk);
            sx[sp] = bv.right[x]; sk[sp++] = kk - jj;
            sx[sp] = bv.left[x]; sk[sp++] = jj;
        }
    }
    uint32_t ni = 0, np = 0;
    for (int q = 0; q < n; ++q) {
        uint32_t c = k[q];
        kids[8 * uint64_t(w) + q] = c;
        uint32_t cnt = bcount(bv, c);
        if (!(c & kLeafFlag) && cnt > uint32_t(max_leaf)) ++ni;
        else np += cnt;
    }
    nk[w] = uint32_t(n);
    nint[w] = ni;
    nprim[w] = np;
}

// Slot of each child by direction: cost(c, s) = ((+-dx) + (+-dy)) + (+-dz), d = (lo + hi of
// the child) - (lo + hi of the node), the sign on an axis + when bit (x 1, y 2, z 4) of s is
// set; the (child, slot) pair of largest cost is taken first, repeatedly (ties: lower child,
// then lower slot; a NaN cost never wins over a taken candidate). kid_in[s] = child or -1.
__device__ void octant_slots(const BinView& bv, uint32_t b, const uint32_t* kids, int n, int* kid_in) {
    const float* pb = bbox(bv, b);
    const float pc[3] = {pb[0] + pb[3], pb[1] + pb[4], pb[2] + pb[5]};
    int slot_of[8];
    for (int q = 0; q < 8; ++q) { kid_in[q] = -1; slot_of[q] = -1; }
    for (int r = 0; r < n; ++r) {
        int bq = -1, bs = -1;
        float bc = 0.0f;
        for (int q = 0; q < n; ++q) {
            if (slot_of[q] >= 0) continue;
            const float* bx = bbox(bv, kids[q]);
            float d0 = (bx[0] + bx[3]) - pc[0], d1 = (bx[1] + bx[4]) - pc[1], d2 = (bx[2] + bx[5]) - pc[2];
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

__global__ void collapse_emit_kernel(BinView bv, const uint32_t* level, uint32_t count, int max_leaf,
                                     const uint32_t* kids, const uint32_t* nk, const uint32_t* int_off,
                                     const uint32_t* prim_off, uint32_t node_base, uint32_t next_node_base,
                                     uint32_t prim_base_g, NodeF* nodes, uint32_t* next_level, uint32_t* prim_order) {
    uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= count) return;
    const float kInf = __int_as_float(0x7f800000);
    NodeF nd;
    for (int q = 0; q < 8; ++q) {
        nd.lo_x[q] = nd.lo_y[q] = nd.lo_z[q] = kInf;
        nd.hi_x[q] = nd.hi_y[q] = nd.hi_z[q] = -kInf;
        nd.meta[q] = 0;
    }
    nd.imask = 0;
    nd.pad0 = 0;
    nd.pad[0] = nd.pad[1] = 0;
    nd.child_base = next_node_base + int_off[w];
    nd.prim_base = prim_base_g + prim_off[w];
    int n = int(nk[w]);
    int kid_in[8];
    octant_slots(bv, level[w], kids + 8 * uint64_t(w), n, kid_in);
    uint32_t rank = 0, poff = 0;
    for (int s2 = 0; s2 < 8; ++s2) {
        if (kid_in[s2] < 0) continue;
        uint32_t c = kids[8 * uint64_t(w) + kid_in[s2]];
        const float* bx = bbox(bv, c);
        nd.lo_x[s2] = bx[0]; nd.lo_y[s2] = bx[1]; nd.lo_z[s2] = bx[2];
        nd.hi_x[s2] = bx[3]; nd.hi_y[s2] = bx[4]; nd.hi_z[s2] = bx[5];
        uint32_t cnt = bcount(bv, c);
        if (!(c & kLeafFlag) && cnt > uint32_t(max_leaf)) {
            nd.meta[s2] = uint8_t(0x80u | rank);
            nd.imask |= 1u << s2;
            next_level[int_off[w] + rank] = c;
            ++rank;
        } else {
            nd.meta[s2] = uint8_t((cnt << 5) | poff);
            uint32_t f = bfirst(bv, c);
            for (uint32_t j = 0; j < cnt; ++j) prim_order[nd.prim_base + poff + j] = f + j;
            poff += cnt;
        }
    }
    nodes[node_base + w] = nd;
}

// ============================ encodings ===========================================================
// 8-bit child boxes: origin p = min of the child boxes; e = least exponent with 255*2^e >= extent
// (in double); qlo = floor((lo-p)*2^-e), qhi = ceil((hi-p)*2^-e), clamped to [0,255].
__global__ void quantise_kernel(const NodeF* in, uint64_t nn, NodeQ* out) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    const NodeF& a = in[i];
    NodeQ q;
    const float* LO[3] = {a.lo_x, a.lo_y, a.lo_z};
    const float* HI[3] = {a.hi_x, a.hi_y, a.hi_z};
    uint8_t* QL[3] = {q.qlo_x, q.qlo_y, q.qlo_z};
    uint8_t* QH[3] = {q.qhi_x, q.qhi_y, q.qhi_z};
    float pp[3];
    uint8_t ee[3];
    uint32_t im = 0;
    for (int c = 0; c < 8; ++c) im |= (a.meta[c] & 0x80u ? 1u : 0u) << c;
    for (int k = 0; k < 3; ++k) {
        float p = __int_as_float(0x7f800000), P = -__int_as_float(0x7f800000);
        for (int c = 0; c < 8; ++c) {
            if (!a.meta[c]) continue;
            p = fmin_t(p, LO[k][c]);
            P = fmax_t(P, HI[k][c]);
        }
        double ext = double(P) - double(p);
        int e;
        if (!(ext > 0.0)) e = -126;
        else {
            int ex;
            double m = frexp(ext / 255.0, &ex);
            e = (m == 0.5) ? ex - 1 : ex;
            while (ldexp(255.0, e) < ext) ++e;
            if (e < -126) e = -126;
            if (e > 127) e = 127;
        }
        pp[k] = p;
        ee[k] = uint8_t(e + 127);
        double inv = ldexp(1.0, -e);
        for (int c = 0; c < 8; ++c) {
            if (!a.meta[c]) { QL[k][c] = 255; QH[k][c] = 0; continue; }
            double lo = floor((double(LO[k][c]) - double(p)) * inv);
            double hi = ceil((double(HI[k][c]) - double(p)) * inv);
            QL[k][c] = uint8_t(lo < 0.0 ? 0.0 : (lo > 255.0 ? 255.0 : lo));
            QH[k][c] = uint8_t(hi < 0.0 ? 0.0 : (hi > 255.0 ? 255.0 : hi));
        }
    }
    q.px = pp[0]; q.py = pp[1]; q.pz = pp[2];
    q.ex = ee[0]; q.ey = ee[1]; q.ez = ee[2];
    q.imask = uint8_t(im);
    q.child_base = a.child_base;
    q.prim_base = a.prim_base;
    for (int c = 0; c < 8; ++c) q.meta[c] = a.meta[c];
    out[i] = q;
}

// Two references per segment: slot_of[reference] = slot, then partner[slot] = the slot of the
// same segment's other reference (reference id ^ 1).
__global__ void slot_of_kernel(const uint32_t* ids, uint64_t n, uint32_t* slot_of) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) slot_of[ids[i]] = uint32_t(i);
}
__global__ void partner_kernel(const uint32_t* ids, const uint32_t* slot_of, uint64_t n, uint32_t* partner) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) partner[i] = slot_of[ids[i] ^ 1u];
}
__global__ void map_order_kernel(const uint32_t* sorted_pos, const uint32_t* sorted_index, uint64_t n, uint32_t* out) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = sorted_index[sorted_pos[i]];
}

// Primitive records in slot order. Quantised Phantom: the segment's first strand-stream entry.
__global__ void records_kernel(int type, int precision, uint32_t shift, const uint32_t* ids, uint64_t n, const float* curves,
                               const float* lrad, const float* geom, const uint32_t* line_entry, const float* tri_nrm,
                               void* prims) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t s = ids[i] >> shift;  // the slot's segment
    if (type == HRT_BLAS_PHANTOM && precision == HRT_PRECISION_FP32) {
        const float* c = curves + 12 * uint64_t(s);
        PrimPhantomF r;
        r.a = make_float4(c[0], c[1], c[2], lrad[2 * uint64_t(s)]);
        r.b = make_float4(c[3], c[4], c[5], lrad[2 * uint64_t(s) + 1]);
        r.c = make_float4(c[6], c[7], c[8], __uint_as_float(s));
        r.d = make_float4(c[9], c[10], c[11], 0.0f);
        static_cast<PrimPhantomF*>(prims)[i] = r;
    } else if (type == HRT_BLAS_PHANTOM) {
        static_cast<uint32_t*>(prims)[i] = line_entry[s];
    } else if (type == HRT_BLAS_LSS) {
        const float* g = geom + 8 * uint64_t(s);
        PrimLss r;
        r.a = make_float4(g[0], g[1], g[2], g[6]);
        r.b = make_float4(g[3], g[4], g[5], g[7]);
        static_cast<PrimLss*>(prims)[i] = r;
    } else if (type == HRT_BLAS_VOXELS) {
        const float* v = geom + 7 * uint64_t(s);
        PrimVoxel r;
        r.lo_id = make_float4(v[0], v[1], v[2], v[6]);
        r.hi = make_float4(v[3], v[4], v[5], 0.0f);
        static_cast<PrimVoxel*>(prims)[i] = r;
    } else if (type == HRT_BLAS_MESH) {
        const float* v = geom + 9 * uint64_t(s);
        const float* m = tri_nrm ? tri_nrm + 9 * uint64_t(s) : nullptr;
        float nn[9];
        for (int k = 0; k < 9; ++k) nn[k] = m ? m[k] : 0.0f;
        PrimTri r;
        r.a = make_float4(v[0], v[1], v[2], __uint_as_float(s));
        r.b = make_float4(v[3], v[4], v[5], nn[0]);
        r.c = make_float4(v[6], v[7], v[8], nn[1]);
        r.d = make_float4(nn[2], nn[3], nn[4], nn[5]);
        r.e = make_float4(nn[6], nn[7], nn[8], __uint_as_float(m ? 1u : 0u));
        static_cast<PrimTri*>(prims)[i] = r;
    } else {
        const float* g = geom + 18 * uint64_t(s);
        PrimDots r;
        r.a = make_float4(g[0], g[1], g[2], g[3]);
        r.b = make_float4(g[4], g[5], g[6], g[7]);
        r.c = make_float4(g[8], g[9], g[10], g[11]);
        r.d = make_float4(g[12], g[13], g[14], g[15]);
        r.e = make_float4(g[16], g[17], __uint_as_float(s), 0.0f);
        static_cast<PrimDots*>(prims)[i] = r;
    }
}

// ============================ voxel hair ==========================================================
// The voxeliser of the oracle's voxel_line (capsule walk along the major axis, every voxel of
// each step's index range, clamped to the grid), one thread per line, filled voxels as bits.
struct VoxGrid {
    float origin[3], size;
    int32_t res[3];
};
__global__ void voxel_bounds_kernel(const float* lines, uint64_t n, uint32_t* ob /*6: min xyz, max xyz*/) {
    __shared__ uint32_t sm[6];
    if (threadIdx.x < 3) sm[threadIdx.x] = 0xffffffffu;
    else if (threadIdx.x < 6) sm[threadIdx.x] = 0u;
    __syncthreads();
    uint32_t lmin[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, lmax[3] = {0, 0, 0};
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
        for (int e = 0; e < 2; ++e)
            for (int k = 0; k < 3; ++k) {
                const float v = lines[6 * i + 3 * e + k] + 0.0f;
                if (!(v == v)) continue;
                const uint32_t c = f2ord(v);
                lmin[k] = min(lmin[k], c);
                lmax[k] = max(lmax[k], c);
            }
    for (int k = 0; k < 3; ++k) { atomicMin(&sm[k], lmin[k]); atomicMax(&sm[3 + k], lmax[k]); }
    __syncthreads();
    if (threadIdx.x < 3) atomicMin(&ob[threadIdx.x], sm[threadIdx.x]);
    else if (threadIdx.x < 6) atomicMax(&ob[threadIdx.x], sm[threadIdx.x]);
}
__global__ void voxel_fill_kernel(const float* lines, uint64_t n, float r, VoxGrid g, uint32_t* bits, uint32_t* err) {
    const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* p = lines + 6 * i;
    const float* q = p + 3;
    const float d[3] = {q[0] - p[0], q[1] - p[1], q[2] - p[2]};
    int a[3] = {0, 1, 2};
    for (int u = 1; u < 3; ++u)
        for (int j = u; j > 0 && fabsf(d[a[j]]) > fabsf(d[a[j - 1]]); --j) { const int t = a[j]; a[j] = a[j - 1]; a[j - 1] = t; }
    if (!(fabsf(d[a[0]]) > 0.0f)) return;
    const float* v0 = d[a[0]] < 0.0f ? q : p;
    const float* v1 = d[a[0]] < 0.0f ? p : q;
    float sv[3], vr0[3], vr1[3];
    for (int k = 0; k < 3; ++k) {
        sv[k] = __fdiv_rn(d[k], d[a[0]]);
        const float sr = sv[k] * r;
        vr0[k] = v0[k] - sr;
        vr1[k] = v1[k] + sr;
    }
    const float dn = __fsqrt_rn((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
    const float q1 = __fdiv_rn(d[a[1]], dn), q2 = __fdiv_rn(d[a[2]], dn);
    const float r1 = __fdiv_rn(r, __fsqrt_rn(1.0f - q1 * q1)), r2 = __fdiv_rn(r, __fsqrt_rn(1.0f - q2 * q2));
    const float tmin = vr0[a[0]], tmax = vr1[a[0]];
    float t0 = tmin, p0[3] = {vr0[0], vr0[1], vr0[2]};
    const int64_t rx = g.res[0], rxy = int64_t(g.res[0]) * g.res[1];
    for (int step = 0; t0 < tmax; ++step) {
        if (step >= (1 << 20)) { atomicOr(err, 1u); return; }
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
            const float f0 = floorf(__fdiv_rn(wmin[k] - g.origin[k], g.size));
            const float f1 = floorf(__fdiv_rn(wmax[k] - g.origin[k], g.size));
            mi[k] = f0 < 0.0f ? 0 : (f0 > float(g.res[k] - 1) ? g.res[k] - 1 : int32_t(f0));
            ma[k] = f1 < 0.0f ? 0 : (f1 > float(g.res[k] - 1) ? g.res[k] - 1 : int32_t(f1));
        }
        for (int32_t z = mi[2]; z <= ma[2]; ++z)
            for (int32_t y = mi[1]; y <= ma[1]; ++y)
                for (int32_t x = mi[0]; x <= ma[0]; ++x) {
                    const uint64_t v = uint64_t(x + y * rx + z * rxy);
                    atomicOr(&bits[v >> 5], 1u << (v & 31u));
                }
        t0 = t1;
        for (int k = 0; k < 3; ++k) p0[k] = p1[k];
    }
}
__global__ void popc_kernel(const uint32_t* bits, uint64_t nw, uint32_t* cnt) {
    const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < nw) cnt[i] = __popc(bits[i]);
}
__global__ void voxel_emit_kernel(const uint32_t* bits, const uint32_t* off, uint64_t nw, VoxGrid g, float* vox) {
    const uint64_t w = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (w >= nw) return;
    uint32_t b = bits[w], o = off[w];
    const int64_t rx = g.res[0], rxy = int64_t(g.res[0]) * g.res[1];
    while (b) {
        const uint32_t j = __ffs(b) - 1;
        b &= b - 1u;
        const int64_t idx = int64_t(w) * 32 + j;
        const int64_t xyz[3] = {idx % rx, (idx / rx) % g.res[1], idx / rxy};
        float* v = vox + 7 * uint64_t(o++);
        for (int k = 0; k < 3; ++k) {
            v[k] = g.origin[k] + float(xyz[k]) * g.size;
            v[3 + k] = v[k] + g.size;
        }
        v[6] = __uint_as_float(uint32_t(idx));
    }
}
__global__ void boxes_voxel_kernel(const float* vox, uint64_t n, float* boxes) {
    const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int k = 0; k < 6; ++k) boxes[6 * i + k] = vox[7 * i + k];
}

template <class T> cudaError_t dalloc(T** p, uint64_t count, cudaStream_t s) {
    return cudaMallocAsync(reinterpret_cast<void**>(p), count * sizeof(T) + 16, s);
}

}  // namespace

// =================================================================================================
cudaError_t make_tris(const float* verts, const float* vnrm, const uint32_t* idx, uint64_t ntris, float* tris,
                      float* tri_nrm, cudaStream_t s) {
    if (ntris == 0) return cudaSuccess;
    tris_kernel<<<grid_for(ntris, 256), 256, 0, s>>>(verts, vnrm, idx, ntris, tris, tri_nrm);
    return cudaGetLastError();
}

cudaError_t make_lines(const float* verts, const float* vrad, float const_radius, const uint32_t* strand_line_off,
                       const uint32_t* strand_vert_off, uint64_t nstrands, const uint32_t* line_idx, uint64_t nlines,
                       float* lines, float* lrad, cudaStream_t s) {
    if (nlines == 0) return cudaSuccess;
    if (line_idx)
        lines_from_indices_kernel<<<grid_for(nlines, 256), 256, 0, s>>>(verts, vrad, const_radius, line_idx, nlines, lines, lrad);
    else
        lines_from_strands_kernel<<<grid_for(nlines, 256), 256, 0, s>>>(verts, vrad, const_radius, strand_line_off,
                                                                         strand_vert_off, nstrands, nlines, lines, lrad);
    return cudaGetLastError();
}

void free_build_output(BuildOutput& o) {
    void* ptrs[] = {o.nodes, o.qnodes_aux, o.prims, o.verts, o.prim_ids, o.partner, o.prim_boxes, o.curves, o.geom,
                    o.morton_sorted, o.sorted_index, o.bin_left, o.bin_right, o.bin_boxes, o.prim_order};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    o = BuildOutput{};
}

#define HRT_CK(x)                                                                              \
    do {                                                                                       \
        cudaError_t e_ = (x);                                                                  \
        if (e_ != cudaSuccess) {                                                               \
            snprintf(msg, msglen, "%s failed: %s (build.cu:%d)", #x, cudaGetErrorString(e_), __LINE__); \
            return e_;                                                                         \
        }                                                                                      \
    } while (0)

static float ord2f_host(uint32_t u) {
    const uint32_t b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    float f;
    memcpy(&f, &b, 4);
    return f;
}
cudaError_t voxelize_device(const float* lines, uint64_t nlines, float r, float size, float** vox, uint64_t* nvox,
                            float grid[8], cudaStream_t s, char* msg, size_t msglen) {
    *vox = nullptr;
    *nvox = 0;
    const unsigned T = 256;
    uint32_t* ob = nullptr;
    HRT_CK(dalloc(&ob, 6, s));
    const uint32_t init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
    HRT_CK(cudaMemcpyAsync(ob, init, sizeof(init), cudaMemcpyHostToDevice, s));
    if (nlines)
        voxel_bounds_kernel<<<unsigned(grid_for(nlines, T) < 1024 ? grid_for(nlines, T) : 1024), T, 0, s>>>(lines, nlines, ob);
    uint32_t hob[6];
    HRT_CK(cudaMemcpyAsync(hob, ob, sizeof(hob), cudaMemcpyDeviceToHost, s));
    HRT_CK(cudaStreamSynchronize(s));
    cudaFreeAsync(ob, s);
    // grid (the oracle's voxel_grid: adds, one division and a ceiling per axis)
    VoxGrid g;
    g.size = size;
    uint64_t total = 1;
    for (int k = 0; k < 3; ++k) {
        const float lo = ord2f_host(hob[k]), hi = ord2f_host(hob[3 + k]);
        g.origin[k] = lo - r;
        const float ext = (hi + r) - g.origin[k];
        const float c = std::ceil(ext / size);
        g.res[k] = c >= 1.0f ? int32_t(c) : 1;
        if (!(c < 2147483648.0f)) g.res[k] = 0x7fffffff;
        total *= uint64_t(g.res[k]);
        grid[k] = g.origin[k];
        grid[4 + k] = float(g.res[k]);
    }
    grid[3] = size;
    if (nlines == 0) return cudaSuccess;
    if (total > (1ull << 31)) {
        snprintf(msg, msglen, "voxel grid of %llu cells; the limit is 2^31 (raise voxel_size)", (unsigned long long)total);
        return cudaErrorInvalidValue;
    }
    const uint64_t nw = (total + 31) / 32;
    uint32_t *bits = nullptr, *cnt = nullptr, *off = nullptr, *tot = nullptr, *err = nullptr;
    HRT_CK(dalloc(&bits, nw, s));
    HRT_CK(dalloc(&cnt, nw, s));
    HRT_CK(dalloc(&off, nw, s));
    HRT_CK(dalloc(&tot, 1, s));
    HRT_CK(dalloc(&err, 1, s));
    HRT_CK(cudaMemsetAsync(bits, 0, nw * 4, s));
    HRT_CK(cudaMemsetAsync(err, 0, 4, s));
    voxel_fill_kernel<<<grid_for(nlines, T), T, 0, s>>>(lines, nlines, r, g, bits, err);
    popc_kernel<<<grid_for(nw, T), T, 0, s>>>(bits, nw, cnt);
    HRT_CK(cudaGetLastError());
    HRT_CK(device_scan<SumOp>(cnt, off, nw, false, tot, s));
    uint32_t h[2];
    HRT_CK(cudaMemcpyAsync(&h[0], tot, 4, cudaMemcpyDeviceToHost, s));
    HRT_CK(cudaMemcpyAsync(&h[1], err, 4, cudaMemcpyDeviceToHost, s));
    HRT_CK(cudaStreamSynchronize(s));
    if (h[1]) {
        snprintf(msg, msglen, "a line needs more than 2^20 voxel steps (raise voxel_size)");
        cudaFreeAsync(bits, s); cudaFreeAsync(cnt, s); cudaFreeAsync(off, s); cudaFreeAsync(tot, s); cudaFreeAsync(err, s);
        return cudaErrorInvalidValue;
    }
    *nvox = h[0];
    if (h[0]) {
        HRT_CK(cudaMalloc(vox, uint64_t(h[0]) * 7 * sizeof(float)));
        voxel_emit_kernel<<<grid_for(nw, T), T, 0, s>>>(bits, off, nw, g, *vox);
        HRT_CK(cudaGetLastError());
    }
    cudaFreeAsync(bits, s);
    cudaFreeAsync(cnt, s);
    cudaFreeAsync(off, s);
    cudaFreeAsync(tot, s);
    cudaFreeAsync(err, s);
    return cudaSuccess;
}

// Geometry processing shared by build and refit: per-segment boxes into `boxes`, the
// intersected geometry into out.curves / out.geom and, for quantised Phantom, the strand vertex
// stream into out.verts (each allocated when null; a refit reuses them) with each line's first
// stream entry in g.line_entry.
struct GeomTmp {
    uint32_t* line_entry = nullptr;
    void release(cudaStream_t s) {
        if (line_entry) cudaFreeAsync(line_entry, s);
        *this = GeomTmp{};
    }
};
cudaError_t geometry_stage(const BuildInput& in, BuildOutput& out, float* boxes, GeomTmp& g, cudaStream_t s,
                           char* msg, size_t msglen) {
    const uint64_t n = in.n;
    const unsigned T = 256;
    if (in.type == HRT_BLAS_PHANTOM) {
        if (!out.curves) HRT_CK(cudaMalloc(&out.curves, n * 12 * sizeof(float)));
        curves_kernel<<<grid_for(n, T), T, 0, s>>>(in.lines, n, out.curves);
        HRT_CK(cudaGetLastError());
        // boxes of the FP32 curves: the quantised format rebuilds exactly these curves
        boxes_phantom_kernel<<<grid_for(n, T), T, 0, s>>>(out.curves, in.lrad, n, boxes);
        if (in.precision == HRT_PRECISION_QUANTISED) {
            uint32_t *flags, *run_incl, *total;
            HRT_CK(dalloc(&flags, n, s));
            HRT_CK(dalloc(&run_incl, n, s));
            HRT_CK(dalloc(&total, 1, s));
            HRT_CK(dalloc(&g.line_entry, n, s));
            stream_flags_kernel<<<grid_for(n, T), T, 0, s>>>(in.lines, in.lrad, n, flags);
            HRT_CK(device_scan<SumOp>(flags, run_incl, n, true, total, s));
            uint32_t nruns = 0;
            HRT_CK(cudaMemcpyAsync(&nruns, total, 4, cudaMemcpyDeviceToHost, s));
            HRT_CK(cudaStreamSynchronize(s));
            const uint64_t nverts = n + 3ull * nruns;
            if (out.verts && nverts != out.nverts) {
                snprintf(msg, msglen, "refit: the strands' runs changed (%llu stream entries, built with %llu)",
                         (unsigned long long)nverts, (unsigned long long)out.nverts);
                cudaFreeAsync(flags, s);
                cudaFreeAsync(run_incl, s);
                cudaFreeAsync(total, s);
                return cudaErrorInvalidValue;
            }
            if (!out.verts) HRT_CK(cudaMalloc(&out.verts, nverts * sizeof(float4)));
            out.nverts = nverts;
            stream_kernel<<<grid_for(n, T), T, 0, s>>>(in.lines, in.lrad, flags, run_incl, n, out.verts, g.line_entry);
            HRT_CK(cudaGetLastError());
            cudaFreeAsync(flags, s);
            cudaFreeAsync(run_incl, s);
            cudaFreeAsync(total, s);
        }
    } else if (in.type == HRT_BLAS_LSS) {
        if (!out.geom) HRT_CK(cudaMalloc(&out.geom, n * 8 * sizeof(float)));
        lss_kernel<<<grid_for(n, T), T, 0, s>>>(in.lines, in.lrad, n, out.geom);
        boxes_lss_kernel<<<grid_for(n, T), T, 0, s>>>(out.geom, n, boxes);
    } else if (in.type == HRT_BLAS_MESH) {
        boxes_tri_kernel<<<grid_for(n, T), T, 0, s>>>(in.tris, n, boxes);
    } else if (in.type == HRT_BLAS_VOXELS) {
        boxes_voxel_kernel<<<grid_for(n, T), T, 0, s>>>(in.voxels, n, boxes);
    } else {
        if (!out.geom) HRT_CK(cudaMalloc(&out.geom, n * 18 * sizeof(float)));
        dots_kernel<<<grid_for(n, T), T, 0, s>>>(in.lines, in.lrad, n, out.geom);
        boxes_dots_kernel<<<grid_for(n, T), T, 0, s>>>(out.geom, n, boxes);
    }
    HRT_CK(cudaGetLastError());
    return cudaSuccess;
}

cudaError_t build_blas_device(const BuildInput& in, BuildOutput& out, cudaStream_t s, char* msg, size_t msglen) {
    // n: BVH references (leaf slots, records); the geometry stage works on the in.n segments
    const uint32_t shift = ref_shift(in.type);
    const uint64_t n = in.n << shift;
    out.nslots = n;
    const unsigned T = 256;
    out.node_bytes = in.precision == HRT_PRECISION_QUANTISED ? sizeof(NodeQ) : sizeof(NodeF);
    if (in.type == HRT_BLAS_PHANTOM) out.prim_bytes = in.precision == HRT_PRECISION_QUANTISED ? 4 : 64;
    else out.prim_bytes = (in.type == HRT_BLAS_LSS || in.type == HRT_BLAS_VOXELS) ? 32 : 80;  // DOTS, mesh: 80
    if (n == 0) return cudaSuccess;

    // ---- geometry processing -> per-segment boxes (and the intersected geometry) ----------------
    HRT_CK(cudaMalloc(&out.prim_boxes, n * 6 * sizeof(float)));
    GeomTmp gt;
    {
        cudaError_t ge = geometry_stage(in, out, out.prim_boxes, gt, s, msg, msglen);
        if (ge != cudaSuccess) {
            gt.release(s);
            return ge;
        }
    }
    uint32_t* line_entry = gt.line_entry;

    // ---- Morton codes + sort ----------------------------------------------------------------
    uint32_t* ob;
    uint64_t* codes;
    uint32_t* order;
    float* sboxes;
    uint32_t* err;
    HRT_CK(dalloc(&ob, 6, s));
    HRT_CK(dalloc(&err, 1, s));
    HRT_CK(cudaMemsetAsync(err, 0, 4, s));
    uint32_t init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
    HRT_CK(cudaMemcpyAsync(ob, init, sizeof(init), cudaMemcpyHostToDevice, s));
    centroid_bounds_kernel<<<unsigned(grid_for(n, T) < 1024 ? grid_for(n, T) : 1024), T, 0, s>>>(out.prim_boxes, n, ob);
    HRT_CK(cudaMalloc(&codes, n * 8));
    HRT_CK(cudaMalloc(&order, n * 4));
    morton_kernel<<<grid_for(n, T), T, 0, s>>>(out.prim_boxes, n, ob, codes, order);
    HRT_CK(cudaGetLastError());
    HRT_CK(radix_sort(codes, order, n, s));
    HRT_CK(dalloc(&sboxes, n * 6, s));
    gather_boxes_kernel<<<grid_for(n, T), T, 0, s>>>(out.prim_boxes, order, n, sboxes);

    // ---- Karras + refit -------------------------------------------------------------------------
    uint64_t ni = n - 1;
    uint32_t *left = nullptr, *right = nullptr, *first = nullptr, *last = nullptr, *pint = nullptr, *pleaf = nullptr,
             *visits = nullptr;
    float* nboxes = nullptr;
    float* dpc = nullptr;
    if (n >= 2) {
        HRT_CK(cudaMalloc(&left, ni * 4));
        HRT_CK(cudaMalloc(&right, ni * 4));
        HRT_CK(dalloc(&first, ni, s));
        HRT_CK(dalloc(&last, ni, s));
        HRT_CK(dalloc(&pint, ni, s));
        HRT_CK(dalloc(&pleaf, n, s));
        HRT_CK(dalloc(&visits, ni, s));
        HRT_CK(cudaMalloc(&nboxes, ni * 6 * sizeof(float)));
        HRT_CK(dalloc(&dpc, ni * 8, s));
        HRT_CK(cudaMemsetAsync(pint, 0xff, ni * 4, s));
        HRT_CK(cudaMemsetAsync(visits, 0, ni * 4, s));
        karras_kernel<<<grid_for(ni, T), T, 0, s>>>(codes, int64_t(n), left, right, first, last, pint, pleaf);
        refit_kernel<<<grid_for(n, T), T, 0, s>>>(pleaf, pint, left, right, first, last, sboxes, nboxes, visits, n, err,
                                                  dpc, in.max_leaf, in.width);
        HRT_CK(cudaGetLastError());
    }

    // ---- collapse to BVH8, breadth first -----------------------------------------------------
    BinView bv{left, right, first, last, nboxes, sboxes, dpc};
    NodeF* nodes_tmp;
    HRT_CK(dalloc(&nodes_tmp, n, s));
    uint32_t *lvl_a, *lvl_b, *kids, *nk, *nint, *nprim, *int_off, *prim_off, *totals, *porder;
    HRT_CK(dalloc(&lvl_a, n, s));
    HRT_CK(dalloc(&lvl_b, n, s));
    HRT_CK(dalloc(&kids, 8 * n, s));
    HRT_CK(dalloc(&nk, n, s));
    HRT_CK(dalloc(&nint, n, s));
    HRT_CK(dalloc(&nprim, n, s));
    HRT_CK(dalloc(&int_off, n, s));
    HRT_CK(dalloc(&prim_off, n, s));
    HRT_CK(dalloc(&totals, 2, s));
    HRT_CK(dalloc(&porder, n, s));
    uint32_t root = n == 1 ? kLeafFlag : 0u;
    HRT_CK(cudaMemcpyAsync(lvl_a, &root, 4, cudaMemcpyHostToDevice, s));
    uint32_t count = 1, node_base = 0, next_node_base = 1, prim_base = 0;
    out.level_start.clear();
    for (int level = 0; count > 0; ++level) {
        if (level > 4096) { snprintf(msg, msglen, "BVH8 collapse did not terminate"); return cudaErrorUnknown; }
        out.level_start.push_back(node_base);
        collapse_expand_kernel<<<grid_for(count, T), T, 0, s>>>(bv, lvl_a, count, in.max_leaf, in.width, kids, nk, nint,
                                                                nprim);
        HRT_CK(cudaGetLastError());
        HRT_CK(device_scan<SumOp>(nint, int_off, count, false, totals, s));
        HRT_CK(device_scan<SumOp>(nprim, prim_off, count, false, totals + 1, s));
        collapse_emit_kernel<<<grid_for(count, T), T, 0, s>>>(bv, lvl_a, count, in.max_leaf, kids, nk, int_off, prim_off,
                                                              node_base, next_node_base, prim_base, nodes_tmp, lvl_b,
                                                              porder);
        HRT_CK(cudaGetLastError());
        uint32_t h_tot[2];
        HRT_CK(cudaMemcpyAsync(h_tot, totals, 8, cudaMemcpyDeviceToHost, s));
        HRT_CK(cudaStreamSynchronize(s));
        node_base = next_node_base;
        next_node_base += h_tot[0];
        prim_base += h_tot[1];
        count = h_tot[0];
        std::swap(lvl_a, lvl_b);
    }
    out.nnodes = node_base;
    out.level_start.push_back(node_base);
    if (prim_base != n) {
        snprintf(msg, msglen, "BVH8 collapse placed %u of %llu primitives", prim_base, (unsigned long long)n);
        return cudaErrorUnknown;
    }

    // ---- encodings and primitive records -----------------------------------------------------
    NodeQ* qn;
    HRT_CK(cudaMalloc(&qn, out.nnodes * sizeof(NodeQ)));
    quantise_kernel<<<grid_for(out.nnodes, T), T, 0, s>>>(nodes_tmp, out.nnodes, qn);
    NodeF* fnodes;
    HRT_CK(cudaMalloc(&fnodes, out.nnodes * sizeof(NodeF)));
    HRT_CK(cudaMemcpyAsync(fnodes, nodes_tmp, out.nnodes * sizeof(NodeF), cudaMemcpyDeviceToDevice, s));
    if (in.precision == HRT_PRECISION_QUANTISED) { out.nodes = qn; out.qnodes_aux = fnodes; }
    else { out.nodes = fnodes; out.qnodes_aux = qn; }
    HRT_CK(cudaMalloc(&out.prim_ids, n * 4));
    map_order_kernel<<<grid_for(n, T), T, 0, s>>>(porder, order, n, out.prim_ids);
    if (shift) {
        // the slot of each slot's partner reference: slot_of[reference] first, then a gather
        uint32_t* slot_of;
        HRT_CK(dalloc(&slot_of, n, s));
        HRT_CK(cudaMalloc(&out.partner, n * 4));
        slot_of_kernel<<<grid_for(n, T), T, 0, s>>>(out.prim_ids, n, slot_of);
        partner_kernel<<<grid_for(n, T), T, 0, s>>>(out.prim_ids, slot_of, n, out.partner);
        HRT_CK(cudaGetLastError());
        cudaFreeAsync(slot_of, s);
    }
    HRT_CK(cudaMalloc(&out.prims, n * out.prim_bytes));
    records_kernel<<<grid_for(n, T), T, 0, s>>>(in.type, in.precision, shift, out.prim_ids, n, out.curves, in.lrad,
                                                in.type == HRT_BLAS_MESH ? in.tris : (in.type == HRT_BLAS_VOXELS ? in.voxels : out.geom), line_entry,
                                                in.tri_normals, out.prims);
    HRT_CK(cudaGetLastError());

    // bounds: union of all primitive boxes = root of the binary tree
    float hb[6];
    HRT_CK(cudaMemcpyAsync(hb, n >= 2 ? nboxes : sboxes, 24, cudaMemcpyDeviceToHost, s));
    uint32_t h_err = 0;
    HRT_CK(cudaMemcpyAsync(&h_err, err, 4, cudaMemcpyDeviceToHost, s));
    HRT_CK(cudaStreamSynchronize(s));
    memcpy(out.bounds, hb, sizeof(hb));
    if (h_err) { snprintf(msg, msglen, "refit exceeded its depth bound"); return cudaErrorUnknown; }

    if (!in.keep_intermediate) {
        // tracing reads nodes, records, the strand vertex stream and the slot maps; the rest of the
        // build's outputs (the other node encoding, primitive boxes, FP32 curves, LSS/DOTS
        // geometry) are kept only for inspection
        void* extra[] = {out.qnodes_aux, out.prim_boxes, out.curves, out.geom};
        for (void* p : extra)
            if (p) cudaFreeAsync(p, s);
        out.qnodes_aux = nullptr;
        out.prim_boxes = nullptr;
        out.curves = nullptr;
        out.geom = nullptr;
    }
    if (in.keep_intermediate) {
        out.morton_sorted = codes;
        out.sorted_index = order;
        out.bin_left = left;
        out.bin_right = right;
        out.bin_boxes = nboxes;
        out.prim_order = nullptr;
    } else {
        cudaFree(codes);
        cudaFree(order);
        if (left) cudaFree(left);
        if (right) cudaFree(right);
        if (nboxes) cudaFree(nboxes);
    }
    void* tmps[] = {ob, err, sboxes, first, last, pint, pleaf, visits, dpc, nodes_tmp, lvl_a, lvl_b, kids, nk, nint,
                    nprim, int_off, prim_off, totals, porder, line_entry};
    for (void* p : tmps)
        if (p) cudaFreeAsync(p, s);
    HRT_CK(cudaStreamSynchronize(s));
    // n references: records, slot map, partner map; in.n segments: curves and LSS/DOTS geometry
    out.device_bytes = out.nnodes * out.node_bytes + n * out.prim_bytes + out.nverts * 16 + n * 4 + (shift ? n * 4 : 0);
    if (in.keep_intermediate)
        out.device_bytes += n * 24 + (out.curves ? in.n * 48 : 0) +
                            (out.geom ? in.n * (in.type == HRT_BLAS_LSS ? 32 : 72) : 0) +
                            out.nnodes * (in.precision == HRT_PRECISION_QUANTISED ? sizeof(NodeF) : sizeof(NodeQ)) +
                            n * 8 + n * 4 + (n ? (n - 1) * 32 : 0);
    return cudaSuccess;
}

// ============================ refit ===============================================================
// One breadth-first level of the BVH8, deepest first: each slot's box is the union of its leaf
// primitives' boxes or its child node's box (nbox, written by the level below); the node's own
// box is the union of its slots. The header (child_base, prim_base, imask, meta) is read from
// either encoding and copied into the FP32 node written to `outf`.
__global__ void refit_level_kernel(const void* nodes, int quant, uint32_t first, uint32_t count, const uint32_t* prim_ids,
                                   const float* boxes, float* nbox, NodeF* outf) {
    uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= count) return;
    const uint32_t i = first + w;
    uint32_t cb, pb, im;
    uint8_t meta[8];
    if (quant) {
        const NodeQ& q = static_cast<const NodeQ*>(nodes)[i];
        cb = q.child_base;
        pb = q.prim_base;
        im = q.imask;
        for (int k = 0; k < 8; ++k) meta[k] = q.meta[k];
    } else {
        const NodeF& f = static_cast<const NodeF*>(nodes)[i];
        cb = f.child_base;
        pb = f.prim_base;
        im = f.imask;
        for (int k = 0; k < 8; ++k) meta[k] = f.meta[k];
    }
    const float kInf = __int_as_float(0x7f800000);
    NodeF nd;
    float nb[6] = {kInf, kInf, kInf, -kInf, -kInf, -kInf};
    for (int q = 0; q < 8; ++q) {
        float b[6] = {kInf, kInf, kInf, -kInf, -kInf, -kInf};
        const uint32_t m = meta[q];
        if (m & 0x80u) {
            const float* c = nbox + 6 * uint64_t(cb + (m & 7u));
            for (int k = 0; k < 6; ++k) b[k] = c[k];
        } else if (m) {
            for (uint32_t j = 0; j < (m >> 5); ++j) {
                const float* c = boxes + 6 * uint64_t(prim_ids[pb + (m & 31u) + j]);
                for (int k = 0; k < 3; ++k) { b[k] = fmin_t(b[k], c[k]); b[3 + k] = fmax_t(b[3 + k], c[3 + k]); }
            }
        }
        nd.lo_x[q] = b[0]; nd.lo_y[q] = b[1]; nd.lo_z[q] = b[2];
        nd.hi_x[q] = b[3]; nd.hi_y[q] = b[4]; nd.hi_z[q] = b[5];
        nd.meta[q] = meta[q];
        if (m) for (int k = 0; k < 3; ++k) { nb[k] = fmin_t(nb[k], b[k]); nb[3 + k] = fmax_t(nb[3 + k], b[3 + k]); }
    }
    nd.child_base = cb;
    nd.prim_base = pb;
    nd.imask = im;
    nd.pad0 = 0;
    nd.pad[0] = nd.pad[1] = 0;
    outf[i] = nd;
    for (int k = 0; k < 6; ++k) nbox[6 * uint64_t(i) + k] = nb[k];
}

cudaError_t refit_blas_device(const BuildInput& in, BuildOutput& out, cudaStream_t s, char* msg, size_t msglen) {
    const uint64_t n = in.n;
    const unsigned T = 256;
    if (n == 0) return cudaSuccess;
    const uint32_t shift = ref_shift(in.type);
    const uint64_t nslots = n << shift;  // BVH references (two per LSS or DOTS segment)
    const bool quant = in.precision == HRT_PRECISION_QUANTISED;
    float* boxes = out.prim_boxes;  // kept for inspection, else a temporary
    bool own_boxes = false, own_curves = !out.curves, own_geom = !out.geom;
    if (!boxes) {
        HRT_CK(dalloc(&boxes, nslots * 6, s));
        own_boxes = true;
    }
    GeomTmp gt;
    cudaError_t e = geometry_stage(in, out, boxes, gt, s, msg, msglen);
    float* nbox = nullptr;
    NodeF* fn = nullptr;
    if (e == cudaSuccess) e = dalloc(&nbox, out.nnodes * 6, s);
    if (e == cudaSuccess) {
        // FP32 nodes are refitted in place; 8-bit nodes through an FP32 copy, then re-quantised
        if (quant) e = dalloc(&fn, out.nnodes, s);
        else fn = static_cast<NodeF*>(out.nodes);
    }
    for (size_t L = out.level_start.size() - 1; e == cudaSuccess && L-- > 0;) {
        const uint32_t first = out.level_start[L], count = out.level_start[L + 1] - first;
        refit_level_kernel<<<grid_for(count, T), T, 0, s>>>(out.nodes, quant ? 1 : 0, first, count, out.prim_ids, boxes,
                                                            nbox, fn);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && quant) {
        quantise_kernel<<<grid_for(out.nnodes, T), T, 0, s>>>(fn, out.nnodes, static_cast<NodeQ*>(out.nodes));
        if (out.qnodes_aux) e = cudaMemcpyAsync(out.qnodes_aux, fn, out.nnodes * sizeof(NodeF), cudaMemcpyDeviceToDevice, s);
    } else if (e == cudaSuccess && out.qnodes_aux) {
        quantise_kernel<<<grid_for(out.nnodes, T), T, 0, s>>>(fn, out.nnodes, static_cast<NodeQ*>(out.qnodes_aux));
    }
    if (e == cudaSuccess) {
        records_kernel<<<grid_for(nslots, T), T, 0, s>>>(in.type, in.precision, shift, out.prim_ids, nslots, out.curves, in.lrad,
                                                    in.type == HRT_BLAS_MESH ? in.tris : out.geom, gt.line_entry,
                                                    in.tri_normals, out.prims);
        e = cudaGetLastError();
    }
    float hb[6];
    if (e == cudaSuccess) e = cudaMemcpyAsync(hb, nbox, 24, cudaMemcpyDeviceToHost, s);  // the root's box
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) memcpy(out.bounds, hb, sizeof(hb));
    gt.release(s);
    if (nbox) cudaFreeAsync(nbox, s);
    if (quant && fn) cudaFreeAsync(fn, s);
    if (own_boxes) cudaFreeAsync(boxes, s);
    if (!in.keep_intermediate) {  // the geometry stage's outputs are kept only for inspection
        if (own_curves && out.curves) { cudaFreeAsync(out.curves, s); out.curves = nullptr; }
        if (own_geom && out.geom) { cudaFreeAsync(out.geom, s); out.geom = nullptr; }
    }
    cudaError_t e2 = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess && !msg[0]) snprintf(msg, msglen, "refit: %s", cudaGetErrorString(e));
    return e;
}

// Expands DOTS frames into the reference's 12 vertices per segment (inspection only).
cudaError_t expand_dots(const float* geom, uint64_t n, float* out36, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    expand_dots_kernel<<<grid_for(n, 256), 256, 0, s>>>(geom, n, out36);
    return cudaGetLastError();
}

}  // namespace hrt
