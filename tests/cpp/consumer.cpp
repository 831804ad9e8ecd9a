// tests/cpp/consumer.cpp -- a C++ program that drives the tracer through include/hrt.hpp, the
// reference-shaped classes over the C ABI, the way the reference's renderer builds its
// acceleration structures and renders (source/renderer.cpp:694-727, :83-166).
//   consumer host            host-only calls, no device needed: ABI version, defaults, camera,
//                            strands, argument errors; prints "host ok <checksum>"
//   consumer gpu <out.bin>   a Phantom BLAS and a translated LSS BLAS (both quantised) in one
//                            TLAS, one 128x96 frame with Shade(), shadow rays and hit records;
//                            writes width, height, the pixels and the hit records to out.bin;
//                            the same frame rendered through a two-scene Batch must match it
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "hrt.hpp"

namespace {

struct Strands {
    std::vector<float> v, r;
    std::vector<uint32_t> off;
};

Strands MakeStrands(uint64_t seed, uint32_t nstrands, uint32_t nverts) {
    hrt_strand_params p;
    hrt_strand_params_default(&p);
    p.seed = seed;
    p.nstrands = nstrands;
    p.nverts = nverts;
    Strands s;
    s.v.resize(size_t(nstrands) * nverts * 3);
    s.r.resize(size_t(nstrands) * nverts);
    s.off.resize(nstrands + 1);
    hrt::Check(nullptr, hrt_generate_strands(&p, s.v.data(), s.r.data(), s.off.data()), "hrt_generate_strands");
    return s;
}

int Host() {
    if (hrt_abi_version() != HRT_ABI_VERSION) return 1;
    hrt_trace_params p = hrt::DefaultParams();
    if (p.tmin != 0.001f || p.tmax != 10000.0f || p.spp != 1) return 2;  // ray_gen.rgen:27-28
    hrt_camera cam = hrt::LookAt({0.0f, 0.0f, 3.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, 40.0f, 4.0f / 3.0f);
    if (!(cam.view_inverse[14] == 3.0f)) return 3;  // the eye is the view inverse's translation
    try {
        hrt::LookAt({0.0f, 0.0f, 3.0f}, {0.0f, 0.0f, 3.0f}, {0.0f, 1.0f, 0.0f}, 40.0f, 1.0f);
        return 4;  // eye == center must be refused
    } catch (const hrt::Error& e) {
        if (e.status != HRT_ERR_INVALID_ARG) return 5;
    }
    Strands s = MakeStrands(1001, 2000, 32);
    uint64_t sum = hrt_checksum(s.v.data(), s.v.size() * 4, s.r.data(), s.r.size() * 4);
    hrt_blas_input in;
    hrt_blas_input_default(&in);
    hrt_blas* b = nullptr;
    if (hrt_blas_build(nullptr, &in, nullptr, &b) != HRT_ERR_INVALID_ARG || b) return 6;
    std::printf("host ok %016llx\n", static_cast<unsigned long long>(sum));
    return 0;
}

int Gpu(const char* path) {
    hrt::Context ctx(0);
    Strands a = MakeStrands(501, 300, 24), c = MakeStrands(502, 300, 24);
    std::vector<hrt::BottomLevelAccelerationStructure> blases;
    hrt::BLASInput hair;
    hair.geometry = HRT_BLAS_PHANTOM;
    hair.precision = HRT_PRECISION_QUANTISED;
    hair.positions = a.v;
    hair.radius = a.r;
    hair.strandOffsets = a.off;
    blases.emplace_back(hair, ctx);
    hrt::BLASInput lss = hair;
    lss.geometry = HRT_BLAS_LSS;
    lss.positions = c.v;
    lss.radius = c.r;
    lss.strandOffsets = c.off;
    lss.transform[12] = 0.35f;  // translated along x (column-major: the fourth column)
    blases.emplace_back(lss, ctx);
    if (blases[0].Type() != hrt::BLASType::eHair || blases[1].Type() != hrt::BLASType::eMesh) return 10;
    hrt::TopLevelAccelerationStructure tlas(blases, ctx);
    const uint32_t w = 128, h = 96;
    hrt::Frame frame(ctx, w, h, 1, true);
    hrt_trace_params p = hrt::DefaultParams();
    p.shading = HRT_SHADE_LAMBERT_SHADOW;
    p.record_hits = 1;
    hrt::Render(ctx, tlas, hrt::LookAt({0.0f, 0.0f, 3.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, 40.0f, float(w) / h),
                p, frame);
    std::vector<hrt_hit> hits;
    std::vector<float> rgba = frame.Download(&hits);
    FILE* f = std::fopen(path, "wb");
    if (!f) return 11;
    std::fwrite(&w, 4, 1, f);
    std::fwrite(&h, 4, 1, f);
    std::fwrite(rgba.data(), 4, rgba.size(), f);
    std::fwrite(hits.data(), sizeof(hrt_hit), hits.size(), f);
    std::fclose(f);
    // the same scene through a batch (beside a second, smaller view): same pixels within the
    // rounding of the separately compiled occupancy variants
    hrt::Frame f0(ctx, w, h, 1), f1(ctx, 64, 48, 1);
    hrt_trace_params pb = p;
    pb.record_hits = 0;  // the batch's frames keep no hit records
    hrt::Batch batch(ctx,
                     {{&tlas, hrt::LookAt({0.0f, 0.0f, 3.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, 40.0f, float(w) / h), &f0},
                      {&tlas, hrt::LookAt({1.0f, 0.5f, 2.5f}, {0.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, 40.0f, 4.0f / 3.0f), &f1}},
                     pb);
    batch.Launch();
    std::vector<std::vector<float>> got = batch.Download();
    if (got.size() != 2 || got[0].size() != rgba.size() || got[1].size() != size_t(64) * 48 * 4) return 12;
    for (size_t i = 0; i < rgba.size(); ++i)
        if (!(std::fabs(got[0][i] - rgba[i]) <= 1e-6f)) return 13;
    // the Phantom BLAS alone, and a copy of it through a serialised image: explicit rays give the
    // same hits bit for bit; a refit copy still traces
    std::vector<hrt::BottomLevelAccelerationStructure> one, loaded;
    one.emplace_back(hair, ctx);
    loaded.push_back(hrt::BottomLevelAccelerationStructure::Load(ctx, one[0].Serialize()));
    if (loaded[0].Type() != hrt::BLASType::eHair || loaded[0].Transform() != one[0].Transform()) return 14;
    hrt::TopLevelAccelerationStructure t_one(one, ctx), t_loaded(loaded, ctx);
    std::vector<float> rays;
    for (int i = 0; i < 64; ++i)
        for (int j = 0; j < 64; ++j) {
            const float x = -0.6f + 1.2f * float(i) / 63.0f, y = -0.2f + 1.2f * float(j) / 63.0f;
            rays.insert(rays.end(), {x, y, 3.0f, 0.0f, 0.0f, -1.0f});
        }
    const std::vector<hrt_hit> h1 = hrt::TraceRays(ctx, t_one, rays, p), h2 = hrt::TraceRays(ctx, t_loaded, rays, p);
    size_t rhit = 0;
    for (size_t i = 0; i < h1.size(); ++i) {
        if (std::memcmp(&h1[i], &h2[i], sizeof(hrt_hit)) != 0) return 15;
        rhit += h1[i].t >= 0.0f;
    }
    if (rhit < 20) return 16;
    std::vector<float> moved = a.v;
    for (size_t i = 1; i < moved.size(); i += 3) moved[i] += 0.01f;
    loaded[0].Refit(moved, a.r);
    hrt::TopLevelAccelerationStructure t_moved(loaded, ctx);
    const std::vector<hrt_hit> h3 = hrt::TraceRays(ctx, t_moved, rays, p);
    size_t mhit = 0;
    for (const hrt_hit& x : h3) mhit += x.t >= 0.0f;
    if (mhit < 20) return 17;
    size_t nhit = 0;
    for (const hrt_hit& x : hits) nhit += x.t >= 0.0f;
    std::printf("gpu ok %zu hits\n", nhit);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    try {
        if (argc >= 2 && std::strcmp(argv[1], "host") == 0) return Host();
        if (argc >= 3 && std::strcmp(argv[1], "gpu") == 0) return Gpu(argv[2]);
    } catch (const hrt::Error& e) {
        std::fprintf(stderr, "hrt error %d: %s\n", int(e.status), e.what());
        return 100 + int(e.status);
    }
    std::fprintf(stderr, "usage: consumer host | consumer gpu <out.bin>\n");
    return 64;
}
