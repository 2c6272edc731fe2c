#!/usr/bin/env bash
# Test infrastructure: compiles the reference's own hot-path sources, where
# they lie, against the shim headers in oracle/shim into
# oracle/_ref/libturner_ref.so (the checker that pins oracle/oracle.cpp and
# generates tests/golden/). The reference's CMake build is not used: its
# third-party dependencies (assimp, cereal, docopt, ThreadPool) are absent.
#
# Flags follow the parity contract: -O2 -ffp-contract=off, no -march.
# Usage: oracle/build_ref.sh REFERENCE_ROOT
set -euo pipefail
if [ $# -lt 1 ]; then
    echo "usage: $0 REFERENCE_ROOT (the reference's source tree)" >&2
    exit 2
fi
REF="$1"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/lib/kdtree.cpp" ]; then
    echo "build_ref: reference sources not found at $REF; skipping" >&2
    exit 0
fi
mkdir -p "$OUT"
FLAGS=(-std=c++17 -O2 -ffp-contract=off -DNDEBUG -fPIC -w -include "$HERE/shim/geometry_prelude.h" -I "$HERE/shim" -I "$REF")
pids=()
g++ "${FLAGS[@]}" -c "$REF/lib/kdtree.cpp" -o "$OUT/kdtree.o" & pids+=($!)
g++ "${FLAGS[@]}" -c "$HERE/ref_driver.cpp" -o "$OUT/ref_driver.o" & pids+=($!)
g++ "${FLAGS[@]}" -c "$HERE/geometry_prelude.cpp" -o "$OUT/geometry_prelude.o" & pids+=($!)
g++ "${FLAGS[@]}" -c "$HERE/ref_fixtures.cpp" -o "$OUT/ref_fixtures.o" & pids+=($!)
# the raytracer and raycaster each define trace() and USAGE: one translation
# unit each, with those names (and the raytracer's copy of the header-defined
# lambertian()) renamed
g++ "${FLAGS[@]}" -Dtrace=ref_raytracer_trace -DUSAGE=ref_raytracer_USAGE -Dlambertian=ref_raytracer_lambertian -c "$REF/raytracer.cpp" \
    -o "$OUT/raytracer.o" & pids+=($!)
g++ "${FLAGS[@]}" -Dtrace=ref_raycaster_trace -DUSAGE=ref_raycaster_USAGE -c "$REF/raycaster.cpp" \
    -o "$OUT/raycaster.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -o "$OUT/libturner_ref.so" "$OUT/kdtree.o" "$OUT/ref_driver.o" "$OUT/geometry_prelude.o" \
    "$OUT/ref_fixtures.o" "$OUT/raytracer.o" "$OUT/raycaster.o" -lpthread
echo "build_ref: wrote $OUT/libturner_ref.so"
