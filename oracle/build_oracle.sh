#!/usr/bin/env bash
# Build the oracle (CPU restatement, test infrastructure) into oracle/_build/:
#   liboracle.so       -O2 -ffp-contract=off : the parity reference (matches the reference bit for bit)
#   liboracle_fast.so  -O3, FMA contraction on : the timed CPU baseline ("port")
# Plain gcc + OpenMP; builds the same on x86-64 and aarch64.
set -euo pipefail
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_build"
mkdir -p "$OUT"
CC=${CC:-gcc}
$CC -O2 -fPIC -fopenmp -ffp-contract=off -std=gnu99 -shared -o "$OUT/liboracle.so" \
    "$HERE/rtm_oracle.c" -lm &
p1=$!
$CC -O3 -fPIC -fopenmp -ffp-contract=fast -std=gnu99 -shared -o "$OUT/liboracle_fast.so" \
    "$HERE/rtm_oracle.c" -lm &
p2=$!
wait $p1; wait $p2
echo "build_oracle: $OUT/liboracle.so $OUT/liboracle_fast.so"
