#!/usr/bin/env bash
# Builds the reference's own C++ FFT (kjear/fyFFT, header-only) into oracle/_ref/ for pinning the
# oracle and as the timed CPU baseline.  Test infrastructure only; nothing here is part of the
# product, and nothing here edits the reference.
#
# Usage: oracle/ref/build_ref.sh [--emulate] [REFERENCE_DIR]
#   REFERENCE_DIR: the reference checkout; default $FYFFT_REFERENCE_DIR, else /root/reference
#   (the container's read-only mount).  When no checkout is found, the sources staged by an
#   earlier run under oracle/_ref/src/ are compiled instead (a GPU host has no checkout).
#
# Two builds of the same unmodified sources:
#   native    (x86-64 with AVX2/FMA)  -> oracle/_ref/libfyref.so
#   emulated  (any host; default off x86-64, or --emulate) -> oracle/_ref/libfyref.so, or
#             oracle/_ref/libfyref_emu.so on x86-64: the reference's AVX2 code paths compiled
#             against oracle/ref/portable_intrin.h (every intrinsic it uses, exact lane
#             semantics) with FOYE_FFT_FORCE_ENABLE_AVX2, the reference's own switch.
# Both use -ffp-contract=off: each intrinsic stays one rounding, as in the reference's MSVC
# build, so the emulated build reproduces the native one bit for bit.
#
# Shims that let g++ accept the MSVC-only sources, applied to a staged copy:
#   * a stand-in <Windows.h> (oracle/ref/windows_stub.h);
#   * "src\foye_FFT_X.hpp" includes with a literal backslash: the staged file names carry it;
#   * g++ rejects `static alignas(32)` (src/foye_FFT_radix5.hpp:74, src/foye_FFT_radix7.hpp:79):
#     those two headers are staged with the specifiers reordered;
#   * native build only: aligned load/store intrinsics mapped to unaligned ones
#     (oracle/ref/gcc_shim.h; the reference issues them at unaligned addresses).
# Staging: oracle/_ref/ is git-ignored and never committed; the staged headers travel with the
# working tree to the aarch64 GPU host, which has no reference checkout, and are compiled there.
set -euo pipefail
EMULATE=0
if [ "${1:-}" = "--emulate" ]; then EMULATE=1; shift; fi
REF=${1:-${FYFFT_REFERENCE_DIR:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$(cd "$HERE/.." && pwd)/_ref
STAGE="$OUT/src"
ARCH=$(uname -m)
if [ "$ARCH" != "x86_64" ]; then EMULATE=1; fi

mkdir -p "$OUT"
if [ -f "$REF/foye_FFT.hpp" ]; then
  rm -rf "$STAGE"
  mkdir -p "$STAGE"
  cp "$HERE/windows_stub.h" "$STAGE/Windows.h"
  cp "$REF/foye_FFT.hpp" "$STAGE/foye_FFT.hpp"
  for f in "$REF"/src/foye_FFT_*.hpp; do
    b=$(basename "$f")
    case "$b" in
      foye_FFT_radix5.hpp|foye_FFT_radix7.hpp)
        sed 's/static alignas(32)/alignas(32) static/' "$f" > "$STAGE/src\\$b" ;;
      *) cp "$f" "$STAGE/src\\$b" ;;
    esac
  done
elif [ ! -f "$STAGE/foye_FFT.hpp" ]; then
  echo "build_ref: no reference checkout at $REF and no staged sources in $STAGE" >&2; exit 3
fi

TMP=$(mktemp -d)
trap 'rm -rf "$TMP"' EXIT
# with a checkout: compile the headers where they lie (links, plus the two reordered headers);
# without one: compile the staged copy
if [ -f "$REF/foye_FFT.hpp" ]; then
  INC="$TMP/inc"
  mkdir -p "$INC"
  cp "$HERE/windows_stub.h" "$INC/Windows.h"
  ln -s "$REF/foye_FFT.hpp" "$INC/foye_FFT.hpp"
  for f in "$REF"/src/foye_FFT_*.hpp; do
    b=$(basename "$f")
    case "$b" in
      foye_FFT_radix5.hpp|foye_FFT_radix7.hpp) cp "$STAGE/src\\$b" "$INC/src\\$b" ;;
      *) ln -s "$f" "$INC/src\\$b" ;;
    esac
  done
else
  INC="$STAGE"
fi
COMMON=(-std=c++20 -O2 -ffp-contract=off -fPIC -shared -w -Wno-psabi -pthread)
if [ "$EMULATE" = 1 ]; then
  mkdir -p "$TMP/emu"
  printf '#include "%s"\n' "$HERE/portable_intrin.h" > "$TMP/emu/immintrin.h"
  if [ "$ARCH" = "x86_64" ]; then LIBNAME=libfyref_emu.so; else LIBNAME=libfyref.so; fi
  g++ "${COMMON[@]}" -DFOYE_FFT_FORCE_ENABLE_AVX2 -DFYREF_EMULATED=1 -I "$TMP/emu" -I "$INC" \
      "$HERE/ref_capi.cpp" -o "$OUT/$LIBNAME.tmp"
else
  LIBNAME=libfyref.so
  g++ "${COMMON[@]}" -mavx2 -mfma -include "$HERE/gcc_shim.h" -I "$INC" \
      "$HERE/ref_capi.cpp" -o "$OUT/$LIBNAME.tmp"
fi
mv "$OUT/$LIBNAME.tmp" "$OUT/$LIBNAME"
echo "build_ref: wrote $OUT/$LIBNAME ($([ "$EMULATE" = 1 ] && echo emulated || echo native) AVX2, $ARCH)"
