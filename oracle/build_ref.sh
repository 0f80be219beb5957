#!/usr/bin/env bash
# Build the reference OpenMP host (GraphBlox 01_host) from its own sources,
# in place under the read-only reference tree, into oracle/_ref/.
#
# Test infrastructure only. Outputs (git-ignored):
#   oracle/_ref/gbx_ref_u    DIRECTED 0, WEIGHTED 0 (as shipped)
#   oracle/_ref/gbx_ref_dw   DIRECTED 1, WEIGHTED 1
# Each is the reference's algorithms/openmp, structures, preprocess,
# utils_graph and config sources plus oracle/ref_driver.cpp (a dump main) and
# oracle/judy_shim (libJudy is not installed here). The two variants differ
# only by a graphConfig.h whose three macros are rewritten with sed into
# oracle/_ref/cfg_<variant>/, which precedes the reference include dirs.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   REFERENCE_ROOT defaults to $GBX_REFERENCE_ROOT, else /root/reference.
#   Exits 2 (nothing built) when the reference sources are not there.
#   The tree it compiled from is recorded in oracle/_ref/reference_root, where
#   the tests that read the reference sources look it up.
set -euo pipefail
REF="${1:-${GBX_REFERENCE_ROOT:-/root/reference}}"
HOST="$REF/01_host"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$HOST/src" ]; then
    echo "reference host sources not found under $HOST" >&2
    exit 2
fi
mkdir -p "$OUT"
printf '%s\n' "$(cd "$REF" && pwd)" > "$OUT/reference_root"
CXX="${CXX:-g++}"
JOBS="$(nproc)"
SRCS=$(ls "$HOST"/src/algorithms/openmp/*.c "$HOST"/src/structures/*.c \
          "$HOST"/src/preprocess/*.c "$HOST"/src/utils_graph/*.c "$HOST"/src/config/*.c)
INC="-I$HOST/include/structures -I$HOST/include/algorithms/openmp -I$HOST/include/preprocess \
     -I$HOST/include/utils_graph -I$HOST/include/config -I$HERE/judy_shim"

build_variant() {
    local name="$1" directed="$2" weighted="$3"
    local cfg="$OUT/cfg_$name" obj="$OUT/obj_$name"
    mkdir -p "$cfg" "$obj"
    sed -e "s/^#define WEIGHTED .*/#define WEIGHTED $weighted/" \
        -e "s/^#define DIRECTED .*/#define DIRECTED $directed/" \
        "$HOST/include/config/graphConfig.h" > "$cfg/graphConfig.h.new"
    if ! cmp -s "$cfg/graphConfig.h.new" "$cfg/graphConfig.h" 2>/dev/null; then
        mv "$cfg/graphConfig.h.new" "$cfg/graphConfig.h"
        rm -f "$obj"/*.o
    else
        rm -f "$cfg/graphConfig.h.new"
    fi
    local flags="-x c++ -w -m64 -fopenmp -O3 -I$cfg $INC"
    # compile each reference source (object name = file stem)
    printf '%s\n' $SRCS | xargs -P "$JOBS" -I{} sh -c \
        'src="{}"; o="'"$obj"'/$(basename "$src" .c).o"; [ "$o" -nt "$src" ] || '"$CXX"' '"$flags"' -c "$src" -o "$o"'
    $CXX -w -O2 -fopenmp -I"$cfg" $INC -c "$HERE/ref_driver.cpp" -o "$obj/ref_driver.o"
    $CXX -w -O2 -I"$HERE/judy_shim" -c "$HERE/judy_shim/judy_shim.cpp" -o "$obj/judy_shim.o"
    $CXX -fopenmp -o "$OUT/gbx_ref_$name" "$obj"/*.o -lm
}

build_variant u 0 0
build_variant dw 1 1
echo "built $OUT/gbx_ref_u $OUT/gbx_ref_dw"
