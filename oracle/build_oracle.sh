#!/usr/bin/env bash
# Test infrastructure: builds the oracle restatement (oracle/emfa_oracle.c)
# as oracle/_build/libemfa_oracle.so with a float (or32_*) and a double
# (or64_*) instance.  Plain gcc, no fast-math, so float arithmetic follows
# IEEE single precision as the reference's does.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
B="$HERE/_build"
mkdir -p "$B"
CFLAGS="-O2 -fPIC -std=c11 -ffp-contract=off -fno-fast-math"
gcc $CFLAGS -DREAL=float '-DPFX(n)=or32_##n' -c "$HERE/emfa_oracle.c" -o "$B/or32.o" &
gcc $CFLAGS -DREAL=double '-DPFX(n)=or64_##n' -c "$HERE/emfa_oracle.c" -o "$B/or64.o" &
gcc $CFLAGS -c "$HERE/oracle_common.c" -o "$B/common.o" &
wait
gcc -shared -o "$B/libemfa_oracle.so" "$B/or32.o" "$B/or64.o" "$B/common.o" -lm
echo "build_oracle: $B/libemfa_oracle.so"
