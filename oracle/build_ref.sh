#!/bin/sh
# Build recipe for the reference oracle -- TEST INFRASTRUCTURE ONLY.
#
# Compiles the reference Moldy sources where they lie (MOLDY_SRC, default
# /root/reference/src) -- nothing is copied into this repository -- into
# oracle/_ref/:
#   libmoldyref.so        strict IEEE FP64 (-O2, no -ffast-math, no FMA
#                         contraction): the parity oracle
#   libmoldyref_fast.so   the reference's own release flags for gcc,
#                         -O2 -ffast-math (src/configure.ac:140-148), with
#                         -funroll-loops on auxil.c (src/Makefile.am:75-88):
#                         the timed CPU baseline
#   moldy_ref_harness[_fast]  oracle/ref_harness.c linked against each
#   moldy_ref_examples        oracle/ref_examples.c (start-up of the examples)
#   moldy_ref_md[_fast]       oracle/ref_md.c (constant-energy do_step runs)
# main.c is left out of the libraries (the harness defines control/ithread/
# nthreads, src/main.c:83-84); it is compiled alone into obj_main/main.o for
# the test that links the reference's own program against libmoldy_gb300.so.
# The source directory used is recorded in oracle/_ref/SRC_DIR.  version.h
# (normally written by a git hook) is generated
# into oracle/_ref/.  Exits 0 without building when the sources are absent.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
SRC=${MOLDY_SRC:-/root/reference/src}
OUT="$HERE/_ref"
if [ ! -f "$SRC/force.c" ]; then
    echo "build_ref: reference sources not found at $SRC; skipping"
    exit 0
fi
mkdir -p "$OUT/obj" "$OUT/obj_fast"
cat > "$OUT/version.h" <<'EOF'
#define REVISION "oracle"
#define REVISION_DATE "oracle"
#define REVISION_STATE "oracle"
EOF
DEFS="-DSTDC_HEADERS -DHAVE_STDARG_H -DHAVE_VOID_PTRS -DHAVE_TIMES -DHAVE_SYS_TIMES_H -Dxdr_float=xdr_int"
FILES="accel algorith alloc ansi auxil convert dump ewald force input eigens kernel leapfrog matrix output quaterns rdf restart startup values xdr parallel"
CC=${CC:-gcc}
pids=""
for f in $FILES; do
    $CC -O2 -fPIC -std=gnu89 -w -ffp-contract=off -I"$OUT" -I"$SRC" $DEFS -c "$SRC/$f.c" -o "$OUT/obj/$f.o" &
    pids="$pids $!"
    extra=""
    [ "$f" = auxil ] && extra="-funroll-loops"
    $CC -O2 -ffast-math $extra -fPIC -std=gnu89 -w -I"$OUT" -I"$SRC" $DEFS -c "$SRC/$f.c" -o "$OUT/obj_fast/$f.o" &
    pids="$pids $!"
done
mkdir -p "$OUT/obj_main"
$CC -O2 -fPIC -std=gnu89 -w -I"$OUT" -I"$SRC" $DEFS -c "$SRC/main.c" -o "$OUT/obj_main/main.o" &
pids="$pids $!"
for p in $pids; do wait $p; done
(cd "$SRC" && pwd) > "$OUT/SRC_DIR"
$CC -shared -o "$OUT/libmoldyref.so" "$OUT"/obj/*.o -lm
$CC -shared -o "$OUT/libmoldyref_fast.so" "$OUT"/obj_fast/*.o -lm
$CC -O2 -std=gnu99 -w -I"$SRC" -I"$OUT" $DEFS "$HERE/ref_harness.c" -o "$OUT/moldy_ref_harness" \
    -L"$OUT" -lmoldyref -Wl,-rpath,"$OUT" -rdynamic -ldl -lm
$CC -O2 -std=gnu99 -w -I"$SRC" -I"$OUT" $DEFS "$HERE/ref_harness.c" -o "$OUT/moldy_ref_harness_fast" \
    -L"$OUT" -lmoldyref_fast -Wl,-rpath,"$OUT" -rdynamic -ldl -lm
echo "build_ref: built $OUT/moldy_ref_harness and $OUT/moldy_ref_harness_fast"
$CC -O2 -std=gnu99 -w -I"$SRC" -I"$OUT" $DEFS "$HERE/ref_examples.c" -o "$OUT/moldy_ref_examples" \
    -L"$OUT" -lmoldyref -Wl,-rpath,"$OUT" -ldl -lm
$CC -O2 -std=gnu99 -w -I"$SRC" -I"$OUT" $DEFS "$HERE/ref_md.c" -o "$OUT/moldy_ref_md" \
    -L"$OUT" -lmoldyref -Wl,-rpath,"$OUT" -ldl -lm
$CC -O2 -std=gnu99 -w -I"$SRC" -I"$OUT" $DEFS "$HERE/ref_md.c" -o "$OUT/moldy_ref_md_fast" \
    -L"$OUT" -lmoldyref_fast -Wl,-rpath,"$OUT" -ldl -lm
