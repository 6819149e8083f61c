#!/usr/bin/env bash
# Compile the reference's own CPU code (SRC/*.c minus the MPI main) and the bundled
# ZFP 0.5.5 sources, where they lie in the reference tree, into oracle/_ref/.
# Test infrastructure: the result pins the oracle (rtm_oracle.c) and makes golden
# fixtures.  The prebuilt ZFP objects/libraries shipped in the reference are not used.
#
# usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   default: $RTM_REFERENCE_ROOT, else a "reference" directory beside the repository
set -euo pipefail
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${RTM_REFERENCE_ROOT:-$HERE/../../reference}}
OUT="$HERE/_ref"
ZFP="$REF/ZFP_LIBRARY_0.5.5"
if [ ! -d "$REF/SRC" ] || [ ! -d "$ZFP/src" ]; then
  echo "build_ref: reference sources not found under $REF" >&2
  exit 2
fi
mkdir -p "$OUT/obj"
CC=${CC:-gcc}
# -ffp-contract=off: no FMA contraction, so the oracle (same flag) matches bit for bit.
FLAGS="-O2 -fPIC -fopenmp -ffp-contract=off"
pids=()
for f in "$ZFP"/src/*.c; do
  b=$(basename "$f" .c)
  $CC $FLAGS -std=gnu99 -w -I"$ZFP/include" -c "$f" -o "$OUT/obj/zfp_$b.o" & pids+=($!)
done
for f in "$REF"/SRC/*.c; do
  b=$(basename "$f" .c)
  [ "$b" = "mpi_rtm_iso2d" ] && continue
  $CC $FLAGS -std=gnu99 -w -include "$HERE/ref_runtime_params.h" -I"$ZFP/include" \
      -c "$f" -o "$OUT/obj/ref_$b.o" & pids+=($!)
done
$CC $FLAGS -std=gnu99 -c "$HERE/ref_runtime_params.c" -o "$OUT/obj/ref_params.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
$CC -shared -fopenmp -o "$OUT/libref_rtm.so" "$OUT"/obj/*.o -lm
echo "build_ref: $OUT/libref_rtm.so"
