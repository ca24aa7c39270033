#!/usr/bin/env bash
# ORACLE -- test infrastructure only. Builds the reference FMM library
# (dnparikh/fmm-blis: frame/, plugin/ and the vendored BLIS in blis/) from a
# scratch copy of its sources into oracle/_ref/, so that tests/golden/
# make_ref_fixtures.py can record the reference's own outputs of
# bli_strassen_ab_ex as golden fixtures. Nothing in the product, the GPU tests
# or the benchmark runs what this builds (the reference sources exist only in
# this container).
#
# The FMM path cannot compile from its own few files: it is written against
# BLIS's object API and plugin mechanism, whose headers BLIS's configure
# generates. So the recipe is BLIS's documented one (README of the reference:
# configure, make, configure-plugin --build fmm_blis), pinned to the haswell
# configuration (the plugin's operand swap assumes a row-preferring
# micro-kernel), run on a copy under oracle/_ref/src/; the reference tree is
# only read.
#
# Two builds of the FMM layer result:
#   _ref/asis/    the sources as shipped (correct for 222.txt only);
#   _ref/patched/ three one-line fixes applied to the scratch copy:
#     frame/base/bli_strassen_ab.c:248  loop r < fmm.R, not FMM_BLIS_MULTS (= 7)
#     frame/base/bli_read_fmm.c:7       line buffer 1024 (444.txt rows exceed 128)
#     frame/base/bli_read_fmm.c:33      header read as m~ k~ n~ R (the files' order)
#   and plugin/bli_plugin_fmm_blis.h:56 MAX_NUM_PARTS 256 (two-level
#   Kronecker algorithms have up to 256 sub-blocks per operand).
# Each holds libfmm_ref.a, libblis_fmm_blis.a (the plugin) and ref_fixture.x
# (oracle/ref_fixture.c linked with them and libblis.a).
#
# Usage: oracle/build_ref.sh [reference dir]   (default /root/reference)
set -euo pipefail

REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$HERE/_ref
SRC=$OUT/src
INST=$OUT/blis-inst
JOBS=$(nproc)

[ -f "$REF/frame/base/bli_strassen_ab.c" ] || { echo "reference sources not found at $REF" >&2; exit 2; }
mkdir -p "$OUT"

# 1. scratch copy of the sources
if [ ! -f "$SRC/.copied" ]; then
    rm -rf "$SRC"
    mkdir -p "$SRC"
    cp -r "$REF/blis" "$REF/frame" "$REF/plugin" "$REF/test" "$SRC/"
    touch "$SRC/.copied"
fi

# 2. BLIS, haswell configuration, OpenMP, static library
if [ ! -f "$INST/lib/libblis.a" ]; then
    (cd "$SRC/blis" && ./configure --prefix="$INST" --disable-shared -t openmp haswell > "$OUT/blis-configure.log" 2>&1 &&
        make -j"$JOBS" > "$OUT/blis-make.log" 2>&1 && make install > "$OUT/blis-install.log" 2>&1)
fi
# the installed library and headers are all that is used from here on
rm -rf "$SRC/blis"

CFLAGS="-O2 -g -w -fopenmp -m64 -mavx2 -mfma -fPIC"

# 3. the plugin and the FMM layer, as shipped and patched
build_variant() {
    local name=$1 patch=$2
    local V=$OUT/$name
    mkdir -p "$V"
    if [ ! -f "$V/plugin/.copied" ]; then
        rm -rf "$V/plugin" "$V/frame"
        cp -r "$SRC/plugin" "$SRC/frame" "$V/"
        if [ "$patch" = 1 ]; then
            sed -i 's/r < FMM_BLIS_MULTS;/r < fmm.R;/' "$V/frame/base/bli_strassen_ab.c"
            sed -i 's/^#define LINE_N .*/#define LINE_N 1024/' "$V/frame/base/bli_read_fmm.c"
            sed -i 's/&fmm.m_tilde, &fmm.n_tilde, &fmm.k_tilde, &fmm.R/\&fmm.m_tilde, \&fmm.k_tilde, \&fmm.n_tilde, \&fmm.R/' "$V/frame/base/bli_read_fmm.c"
            sed -i 's/^#define MAX_NUM_PARTS .*/#define MAX_NUM_PARTS 256/' "$V/plugin/bli_plugin_fmm_blis.h"
            grep -q 'r < fmm.R;' "$V/frame/base/bli_strassen_ab.c"
            grep -q '^#define LINE_N 1024' "$V/frame/base/bli_read_fmm.c"
            grep -q '&fmm.m_tilde, &fmm.k_tilde, &fmm.n_tilde, &fmm.R' "$V/frame/base/bli_read_fmm.c"
            grep -q '^#define MAX_NUM_PARTS 256' "$V/plugin/bli_plugin_fmm_blis.h"
        fi
        touch "$V/plugin/.copied"
    fi
    if [ ! -f "$V/plugin/lib/haswell/libblis_fmm_blis.a" ]; then
        (cd "$V/plugin" && "$INST/share/blis/configure-plugin" --build fmm_blis > "$V/plugin-configure.log" 2>&1 &&
            make -j"$JOBS" > "$V/plugin-make.log" 2>&1)
    fi
    if [ -x "$V/ref_fixture.x" ] && [ "$V/ref_fixture.x" -nt "$HERE/ref_fixture.c" ]; then
        return 0
    fi
    local objs=()
    for f in frame/util/bli_fmm_util.c frame/base/bli_strassen_ab.c frame/base/bli_read_fmm.c; do
        local o=$V/$(basename "$f" .c).o
        gcc $CFLAGS -I"$V/frame/include" -I"$V/plugin" -I"$INST/include/blis" -c "$V/$f" -o "$o"
        objs+=("$o")
    done
    rm -f "$V/libfmm_ref.a"
    ar cr "$V/libfmm_ref.a" "${objs[@]}"
    gcc $CFLAGS -I"$V/frame/include" -I"$V/plugin" -I"$INST/include/blis" "$HERE/ref_fixture.c" \
        "$V/libfmm_ref.a" "$V/plugin/lib/haswell/libblis_fmm_blis.a" "$INST/lib/libblis.a" \
        -o "$V/ref_fixture.x" -lpthread -lm
}

build_variant asis 0
build_variant patched 1
echo "reference built in $OUT"
