#!/usr/bin/env bash
# build_ref.sh -- stage and compile Lantern's own integrator as a CPU library.
#
# TEST INFRASTRUCTURE ONLY: the result, oracle/_ref/liblantern_ref.so, is the
# reference CPU path used by tests/ (oracle pinning, golden vectors) and by
# bench.py --impl reference. It is never part of the shipped library.
#
# Stage (only where the reference tree exists: LANTERN_REFERENCE, else a
# checkout named "reference" next to this repository): copy the reference sources this build needs into
# oracle/_ref/src, unmodified except for integrator.cpp, where the two loop
# constants of RenderPixel (maxBounces = 1500 at :114, the roulette threshold
# "bounces > 3" at :235) become variables. oracle/_ref is git-ignored.
# Compile (wherever oracle/_ref/src exists, also on a machine without the
# reference tree): g++ with the project shims in oracle/ref_shim (scalar Embree
# math, parallel_for, rtc* over the oracle intersector, headless driver).
set -euo pipefail
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${LANTERN_REFERENCE:-$(cd "$HERE/../.." && pwd)/reference}
OUT=$HERE/_ref
SRC=$OUT/src
OBJ=$OUT/obj

if [ -d "$REF/source/core" ]; then
    rm -rf "$SRC"
    mkdir -p "$SRC/core" "$SRC/embree/include" "$SRC/json" "$SRC/jsv" "$SRC/stb"
    for d in camera integrator io materials math scene; do
        cp -r "$REF/source/core/$d" "$SRC/core/$d"
    done
    cp -r "$REF/third_party/embree/include/embree3" "$SRC/embree/include/"
    cp "$REF/third_party/json/json.hpp" "$SRC/json/"
    cp -r "$REF/third_party/json_schema_validator/include" "$REF/third_party/json_schema_validator/src" "$SRC/jsv/"
    cp -r "$REF/third_party/stb/include" "$SRC/stb/"
    cp "$REF/third_party/stb/stb.cpp" "$SRC/stb/"
    I="$SRC/core/integrator/integrator.cpp"
    chmod u+w "$I"
    [ "$(grep -c 'const uint maxBounces = 1500;' "$I")" = 1 ]
    [ "$(grep -c 'if (bounces > 3) {' "$I")" = 1 ]
    [ "$(grep -c '^#include <algorithm>' "$I")" = 1 ]
    sed -i -e 's/const uint maxBounces = 1500;/const uint maxBounces = lt_ref_max_bounces;/' \
           -e 's/if (bounces > 3) {/if (bounces > lt_ref_rr_depth) {/' \
           -e 's/^#include <algorithm>/#include <algorithm>\nextern "C" unsigned lt_ref_max_bounces, lt_ref_rr_depth;/' "$I"
fi

if [ ! -d "$SRC/core" ]; then
    echo "build_ref.sh: no staged reference sources in $SRC" >&2
    exit 2
fi

mkdir -p "$OBJ"
CXX=${CXX:-g++}
CC=${CC:-gcc}
FLAGS="-O2 -fPIC -ffp-contract=off -fno-strict-aliasing -w"
CXXFLAGS="$FLAGS -std=c++14 -include cstdint -include cstring -include cstdio -include fstream -include string -DEMBREE_STATIC_LIB -I$HERE/ref_shim -I$SRC/core -I$SRC/embree/include -I$SRC/json -I$SRC/jsv/include -I$SRC/stb/include"

units=(
  "$SRC/core/camera/pinhole_camera.cpp" "$SRC/core/camera/reconstruction_filter.cpp"
  "$SRC/core/camera/frame_buffer.cpp" "$SRC/core/integrator/integrator.cpp"
  "$SRC/core/math/vector_math.cpp" "$SRC/core/scene/area_light.cpp" "$SRC/core/scene/scene.cpp"
  "$SRC/core/scene/geometry_generator.cpp" "$SRC/core/scene/image_cache.cpp"
  "$SRC/core/io/lantern_model_file.cpp"
  "$SRC/jsv/src/json-schema-draft4.json.cpp" "$SRC/jsv/src/json-uri.cpp" "$SRC/jsv/src/json-validator.cpp"
  "$SRC/stb/stb.cpp" "$HERE/ref_shim/rtc_shim.cpp" "$HERE/ref_shim/ref_driver.cpp"
)
pids=()
objs=()
for u in "${units[@]}"; do
    o="$OBJ/$(echo "$u" | sed -e "s|$SRC/||" -e "s|$HERE/||" -e 's|/|_|g').o"
    objs+=("$o")
    $CXX $CXXFLAGS -c "$u" -o "$o" &
    pids+=($!)
done
$CC $FLAGS -std=c11 -c "$HERE/lt_oracle.c" -o "$OBJ/lt_oracle.o" &
pids+=($!)
objs+=("$OBJ/lt_oracle.o")
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
[ $rc = 0 ] || { echo "build_ref.sh: compile failed" >&2; exit 1; }
$CXX -shared -o "$OUT/liblantern_ref.so" "${objs[@]}" -lstdc++fs -lpthread
# permissive scene schema: the reference validates against scenes/scene.schema.json,
# which forbids the extension keys the project writes (render, henyey_greenstein)
printf '{"type": "object"}\n' > "$OUT/scene.schema.json"
echo "built $OUT/liblantern_ref.so"
