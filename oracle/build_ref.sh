#!/usr/bin/env bash
# Build the reference cmtj extension (_cmtj) from its own sources, in place,
# into oracle/_ref/.  The product never loads this: it is the checker that
# pins the C++ restatement in oracle/ and generates tests/golden/ fixtures.
#
# Reads:   $CMTJ_REF (required: the reference checkout): python/cmtj.cpp + core/*.hpp
# Writes:  oracle/_ref/_cmtj<ext-suffix>, oracle/_ref/libalpha_ref.so,
#          oracle/_ref/cmtj/__init__.py (shim), and oracle/_ref/fma/ (the
#          same, compiled with FMA contraction)
#
# Flags follow setup.py:51-88 on Linux (C++17, -fvisibility=hidden,
# -Wno-unused-variable) at -O3, plus -ffp-contract=off so that no compiler
# fuses a*b+c into an FMA (x86-64 baseline has no FMA; aarch64 does, and GCC
# contracts by default there).  The kissfft submodule is not vendored, so the
# project-written stand-in header under oracle/stubs/ satisfies noise.hpp.
# oracle/_ref/fma/ holds a second build with -ffp-contract=fast (and -mfma on
# x86-64): the reference as GCC compiles it by default on an FMA machine such
# as aarch64, whose last bits differ from the build above.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${CMTJ_REF:-}"
OUT="$HERE/_ref"
if [ -z "$REF" ] || [ ! -f "$REF/python/cmtj.cpp" ]; then
  echo "reference sources not found (set CMTJ_REF to the reference checkout); skipping _cmtj build" >&2
  exit 0
fi
mkdir -p "$OUT"
EXT="$(python3 -c 'import sysconfig;print(sysconfig.get_config_var("EXT_SUFFIX"))')"
PYBIND_INC="$(python3 -m pybind11 --includes)"
TARGET="$OUT/_cmtj$EXT"
STUB="$HERE/stubs/third_party/kissfft/kissfft.hh"
if [ ! -f "$TARGET" ] || [ "$REF/core/junction.hpp" -nt "$TARGET" ] || [ "$STUB" -nt "$TARGET" ]; then
  g++ -O3 -shared -fPIC -std=c++17 -fvisibility=hidden -Wno-unused-variable \
      -ffp-contract=off -DVERSION_INFO='"ref-local"' \
      -I"$REF" -I"$REF/core" -I"$HERE/stubs/third_party" \
      $PYBIND_INC "$REF/python/cmtj.cpp" -o "$TARGET.tmp"
  mv "$TARGET.tmp" "$TARGET"
fi
FMA_OUT="$OUT/fma"
mkdir -p "$FMA_OUT"
FMA_TARGET="$FMA_OUT/_cmtj$EXT"
FMA_FLAGS="-ffp-contract=fast"
if [ "$(uname -m)" = "x86_64" ]; then FMA_FLAGS="$FMA_FLAGS -mfma"; fi
if [ ! -f "$FMA_TARGET" ] || [ "$REF/core/junction.hpp" -nt "$FMA_TARGET" ] || [ "$STUB" -nt "$FMA_TARGET" ]; then
  g++ -O3 -shared -fPIC -std=c++17 -fvisibility=hidden -Wno-unused-variable \
      $FMA_FLAGS -DVERSION_INFO='"ref-local-fma"' \
      -I"$REF" -I"$REF/core" -I"$HERE/stubs/third_party" \
      $PYBIND_INC "$REF/python/cmtj.cpp" -o "$FMA_TARGET.tmp"
  mv "$FMA_TARGET.tmp" "$FMA_TARGET"
fi
# The reference's BufferedAlphaNoise behind a C entry point (alpha_ref.cpp).
ALPHA="$OUT/libalpha_ref.so"
if [ ! -f "$ALPHA" ] || [ "$REF/core/noise.hpp" -nt "$ALPHA" ] || [ "$HERE/alpha_ref.cpp" -nt "$ALPHA" ] || \
   [ "$STUB" -nt "$ALPHA" ]; then
  g++ -O2 -shared -fPIC -std=c++17 -ffp-contract=off -I"$REF/core" -I"$HERE/stubs/third_party" \
      "$HERE/alpha_ref.cpp" -o "$ALPHA.tmp"
  mv "$ALPHA.tmp" "$ALPHA"
fi
# A shim package named `cmtj` whose submodules (cmtj.utils, cmtj.stack, ...)
# resolve from the reference tree, so no reference file is copied here.
for D in "$OUT" "$FMA_OUT"; do
  mkdir -p "$D/cmtj"
  cat > "$D/cmtj/__init__.py" <<EOF
import os as _os
__path__ = [_os.path.join("$REF", "cmtj")]
__version__ = "ref-local"
import _cmtj
from _cmtj import *
EOF
done
echo "built $TARGET"
