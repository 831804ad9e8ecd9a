#!/usr/bin/env bash
# oracle/build_ref.sh -- TEST INFRASTRUCTURE: builds oracle/_ref/libhrtref.so, the reference's
# own shader and geometry code compiled as host C++ through oracle/glsl_shim.hpp.
#
# Reads the reference checkout (HRT_REFERENCE, else a `reference` directory beside the repository)
# where it lies; writes only into oracle/_ref/ (git-ignored). Nothing from the reference is committed.
#   * shaders/{ray,curve,cone,cylinder,shading}.glsl are included as they are. For the FP32
#     build every unsuffixed floating literal gets an `f` suffix, because in GLSL `0.5` is a
#     float while in C++ it is a double; the FP64 build includes them untouched with
#     `#define float double`.
#   * Prhi (shaders/hair_intersection.rint:15-130) and the body of ray_gen.rgen:18-24 are cut
#     out of the stage files, which carry #version/#extension/layout lines C++ cannot parse.
#   * GenerateCurves, PerpStark, BuildFrame, GenerateDisjointOrthogonalTriangleStrips,
#     GenerateLinearSweptSpheres and GenerateAABBs(curves) are cut out of
#     source/resources/model/geometry_processor.cpp (:123-156, :199-298, :422-436).
# If the checkout is absent the script prints a note and exits 0.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${HRT_REFERENCE:-$(cd "$HERE/../.." && pwd)/reference}"
OUT="$HERE/_ref"
if [ ! -d "$REF/shaders" ]; then
    echo "build_ref: reference checkout not found at $REF; oracle/_ref not built"
    exit 0
fi
mkdir -p "$OUT/glsl32" "$OUT/glsl64"
SUFFIX='s/(?<![\w.])(\d+\.\d*(?:[eE][-+]?\d+)?|\d+[eE][-+]?\d+)(?![\w.])/$1f/g'
for f in ray curve cone cylinder shading; do
    perl -pe "$SUFFIX" "$REF/shaders/$f.glsl" > "$OUT/glsl32/$f.glsl"
    cp "$REF/shaders/$f.glsl" "$OUT/glsl64/$f.glsl"
done
# Prhi: from its signature up to (not including) the stage entry point.
awk '/^float Prhi\(/{p=1} /^void main\(/{p=0} p' "$REF/shaders/hair_intersection.rint" > "$OUT/glsl64/prhi.inc"
perl -pe "$SUFFIX" "$OUT/glsl64/prhi.inc" > "$OUT/glsl32/prhi.inc"
# ray_gen body: pixel centre through the world-space direction.
awk '/pixelCenter =/{p=1} p{print} /vec4 direction =/{p=0}' "$REF/shaders/ray_gen.rgen" > "$OUT/glsl64/raygen_body.inc"
perl -pe "$SUFFIX" "$OUT/glsl64/raygen_body.inc" > "$OUT/glsl32/raygen_body.inc"
# Host geometry functions (FP32 C++ already; taken verbatim).
GP="$REF/source/resources/model/geometry_processor.cpp"
{
    awk '/^std::vector<Curve> GenerateCurves\(/{p=1} p{print} p&&/^}$/{p=0}' "$GP"
    awk '/^inline glm::vec3 PerpStark\(/{p=1} p{print} p&&/^}$/{p=0}' "$GP"
    awk '/^inline void BuildFrame\(/{p=1} p{print} p&&/^}$/{p=0}' "$GP"
    awk '/^Mesh GenerateDisjointOrthogonalTriangleStrips\(/{p=1} p{print} p&&/^}$/{p=0}' "$GP"
    awk '/^LSSMesh GenerateLinearSweptSpheres\(/{p=1} p{print} p&&/^}$/{p=0}' "$GP"
    awk '/^std::vector<AABB> GenerateAABBs\(const std::vector<Curve>/{p=1} p{print} p&&/^}$/{p=0}' "$GP"
} > "$OUT/geometry_fns.inc"
for f in "$OUT/glsl64/prhi.inc" "$OUT/glsl64/raygen_body.inc" "$OUT/geometry_fns.inc"; do
    [ -s "$f" ] || { echo "build_ref: extraction produced an empty $f" >&2; exit 1; }
done
g++ -std=c++17 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared \
    -I"$HERE" -I"$OUT" "$HERE/ref_harness.cpp" -o "$OUT/libhrtref.so"
echo "build_ref: built $OUT/libhrtref.so"
