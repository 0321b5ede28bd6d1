#!/usr/bin/env bash
# Builds the oracle's C restatement (test infrastructure only) into oracle/_build/.
# No reference sources are compiled: the reference is MATLAB.
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$here/_build"
gcc -O2 -fopenmp -fPIC -shared -o "$here/_build/liboracle_interp.so.tmp" "$here/interp_ref.c" -lm
mv "$here/_build/liboracle_interp.so.tmp" "$here/_build/liboracle_interp.so"
