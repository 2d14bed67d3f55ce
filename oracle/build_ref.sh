#!/usr/bin/env bash
# Builds the reference MMC CPU engine (SSE4 + OpenMP, xorshift128+) straight from
# its sources where they lie, into oracle/_ref/.  Test infrastructure only: the
# binary produces golden fixtures (tests/golden/make_golden.py) and is never part
# of the product.  Nothing is copied out of the reference tree.
#
#   MMC_REFERENCE=/path/to/mmc  oracle/build_ref.sh
#
# Without MMC_REFERENCE the recipe reads the sources at the development
# checkout's location below; where neither exists it exits with status 2 and
# nothing is built (the GPU machine has no reference tree and needs none).
#
# Needs: gcc/g++, zlib headers, an x86-64 host (the reference's branchless
# Badouel tracer is written with SSE4.1 intrinsics; without MMC_USE_SSE its
# tracer_build skips the plane offsets and only the Plucker tracer works).
set -euo pipefail
REF=${MMC_REFERENCE:-${REF:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
SRC="$REF/src"
if [ ! -d "$SRC" ]; then
    echo "reference sources not found at $SRC" >&2
    exit 2
fi
case "$(uname -m)" in
    x86_64) ;;
    *) echo "reference CPU engine needs SSE4.1 (x86-64); host is $(uname -m)" >&2; exit 3 ;;
esac
mkdir -p "$OUT/obj"
# The reference's own Makefile adds -ffast-math; it is left out here so the
# binary follows the IEEE semantics of the reference source, which the oracle
# pins bit for bit (volumes of jittered tets cancel badly and fast-math
# reassociation moves them by ~1e-3).
CFLAGS="-O3 -fopenmp -fno-strict-aliasing -w -DMMC_USE_SSE -DHAVE_SSE2 -msse -msse2 -msse3 -mssse3 -msse4.1 -DMMC_XORSHIFT -DUSE_OS_TIMER -I$SRC -I$SRC/zmat/easylzma -I$SRC/ubj -include $HERE/ref_shim.h"
ZFLAGS="-DNO_LZMA -DNO_LZ4 -DNO_BLOSC2 -DNO_ZSTD"
CSRCS="mmc mmc_host mmc_utils mmc_mesh mmc_raytrace mmc_rand_xorshift128p mmc_tictoc mmc_bench cjson/cJSON ubj/ubjw"
CXXSRCS="mmc_highorder mmc_neurojson"
pids=()
for f in $CSRCS; do
    o="$OUT/obj/$(echo "$f" | tr '/' '_').o"
    gcc $CFLAGS -c "$SRC/$f.c" -o "$o" &
    pids+=($!)
done
for f in $CXXSRCS; do
    g++ $CFLAGS -c "$SRC/$f.cpp" -o "$OUT/obj/$f.o" &
    pids+=($!)
done
gcc $CFLAGS $ZFLAGS -c "$SRC/zmat/zmatlib.c" -o "$OUT/obj/zmatlib.o" &
pids+=($!)
gcc -c "$HERE/ref_shim.c" -o "$OUT/obj/ref_shim.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
gcc $CFLAGS -c "$HERE/ref_driver.c" -o "$OUT/ref_driver.o"
g++ -fopenmp -o "$OUT/mmc" "$OUT"/obj/*.o -lz -lm
# same objects with the reference's main replaced by the table-dumping driver
g++ -fopenmp -o "$OUT/mmc_detp" $(ls "$OUT"/obj/*.o | grep -v '/mmc\.o$') "$OUT/ref_driver.o" -lz -lm
# where the sources were found: tests that compile against the reference's own
# headers (tests/test_integration_shim.py) read it
echo "$REF" > "$OUT/REF_PATH"
echo "built $OUT/mmc and $OUT/mmc_detp"
