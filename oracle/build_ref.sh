#!/usr/bin/env bash
# Test infrastructure (oracle only): compile the reference's own hot-path C++ sources, where
# they lie in the reference checkout, into oracle/_ref/libforte2_ref.so together with the
# nanobind/sparse shims (oracle/ref_shim), the BLAS bridge and the C-ABI wrapper ref_capi.cc.
# Usage: oracle/build_ref.sh REFERENCE_ROOT   (or set FORTE2_REFERENCE_ROOT)
# Nothing is copied out of the reference tree; outputs go only to oracle/_ref/.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${FORTE2_REFERENCE_ROOT:-}}"
if [ -z "$REF" ]; then
    echo "usage: $0 REFERENCE_ROOT (the forte2 checkout; or set FORTE2_REFERENCE_ROOT)" >&2
    exit 2
fi
SRC="$REF/forte2"
OUT="$HERE/_ref"
if [ ! -f "$SRC/ci/ci_sigma_builder.cc" ]; then
    echo "reference sources not found under $SRC" >&2
    exit 3
fi
mkdir -p "$OUT/obj"
CXX="${CXX:-g++}"
FLAGS="-std=c++20 -O2 -fPIC -DNDEBUG -w -include cassert -I$HERE/ref_shim -I$SRC"
SOURCES=(
    ci/ci_strings.cc
    ci/ci_strings_makers.cc
    ci/ci_occupation.cc
    ci/ci_string_class.cc
    ci/ci_string_address.cc
    ci/ci_sigma_builder.cc
    ci/ci_sigma_builder_harrison_zarrabian.cc
    ci/ci_sigma_builder_knowles_handy.cc
    ci/ci_sigma_builder_1rdm.cc
    ci/ci_sigma_builder_2rdm.cc
    ci/ci_sigma_builder_3rdm.cc
    determinant/slater_rules.cc
    determinant/ci_spin_adapter.cc
    ci/rel_ci_sigma_builder.cc
    ci/rel_ci_sigma_builder_harrison_zarrabian.cc
    ci/rel_ci_sigma_builder_rdm.cc
    determinant/rel_slater_rules.cc
)
OBJS=()
pids=()
for s in "${SOURCES[@]}"; do
    o="$OUT/obj/$(echo "$s" | tr '/' '_').o"
    OBJS+=("$o")
    $CXX $FLAGS -c "$SRC/$s" -o "$o" &
    pids+=($!)
done
$CXX $FLAGS -c "$HERE/ref_capi.cc" -o "$OUT/obj/ref_capi.o" &
pids+=($!)
$CXX -std=c++20 -O2 -fPIC -c "$HERE/blas_bridge.cc" -o "$OUT/obj/blas_bridge.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
$CXX -shared -o "$OUT/libforte2_ref.so" "${OBJS[@]}" "$OUT/obj/ref_capi.o" "$OUT/obj/blas_bridge.o" -ldl -lpthread
echo "built $OUT/libforte2_ref.so"
