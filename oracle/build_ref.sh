#!/usr/bin/env bash
# Builds the unmodified MetaPart reference C sources into oracle/_ref/ as the
# CPU checker (test infrastructure; never linked into the GPU product).
#
#   usage: oracle/build_ref.sh [REFERENCE_ROOT]      (default /root/reference)
#
# The reference needs MPI; oracle/mpi_shim/mpi.h stands in for it at one rank.
# Outputs (x86/Arm native, git-ignored):
#   oracle/_ref/genFastqIdx                  src/genFastqIdx.c
#   oracle/_ref/genHistograms_metapart       src/genHistograms.c + src/countMmers.c
#   oracle/_ref/genHistograms_metapartmin    src/genHistograms.c + src/countMmers_3minimizers.c -DMIN3
#   oracle/_ref/metapart                     src/metapart.c + src/enumerateKmers.c
#   oracle/_ref/metapartmin                  src/metapart.c + src/enumerateKmers_3minimizers.c -DMIN3
#   oracle/_ref/metapart_dump[min]           the same, through oracle/ref_hooks.c (stage dumps)
set -euo pipefail
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
SRC="$REF/src"
if [ ! -f "$SRC/metapart.c" ]; then
    echo "build_ref: reference sources not found under $SRC" >&2
    exit 2
fi
mkdir -p "$OUT"
CC="${CC:-gcc}"
CF="-O3 -fopenmp -w -I$HERE/mpi_shim"
$CC -O3 -w -o "$OUT/genFastqIdx" "$SRC/genFastqIdx.c" -lm &
$CC $CF -o "$OUT/genHistograms_metapart" "$SRC/genHistograms.c" "$SRC/countMmers.c" -lm &
$CC $CF -DMIN3 -o "$OUT/genHistograms_metapartmin" "$SRC/genHistograms.c" "$SRC/countMmers_3minimizers.c" -lm &
$CC $CF -o "$OUT/metapart" "$SRC/metapart.c" "$SRC/enumerateKmers.c" -lm &
$CC $CF -DMIN3 -o "$OUT/metapartmin" "$SRC/metapart.c" "$SRC/enumerateKmers_3minimizers.c" -lm &
$CC $CF -I"$SRC" -o "$OUT/metapart_dump" "$HERE/ref_hooks.c" "$SRC/enumerateKmers.c" -lm &
$CC $CF -DMIN3 -I"$SRC" -o "$OUT/metapart_dumpmin" "$HERE/ref_hooks.c" "$SRC/enumerateKmers_3minimizers.c" -lm &
wait
for b in genFastqIdx genHistograms_metapart genHistograms_metapartmin metapart metapartmin metapart_dump metapart_dumpmin; do
    test -x "$OUT/$b" || { echo "build_ref: $b missing" >&2; exit 1; }
done
(cd "$REF" && pwd) > "$OUT/REFERENCE_ROOT"
echo "build_ref: ok -> $OUT"
