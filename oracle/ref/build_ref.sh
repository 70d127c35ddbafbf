#!/usr/bin/env bash
# Builds the reference's own C++ FFT (unmodified headers read where they lie under the
# reference checkout) into oracle/_ref/libfyref.so, for pinning the oracle and as the timed
# CPU baseline. Test infrastructure only; nothing here is part of the product.
#
# Needs an x86-64 host with AVX2/FMA (the reference is AVX2-only). Usage:
#   oracle/ref/build_ref.sh [REFERENCE_DIR]        (default /root/reference)
# What it does to make g++ accept the MSVC-only sources, without editing them in place:
#   * a stand-in <Windows.h> (oracle/ref/windows_stub.h);
#   * the reference includes "src\foye_FFT_X.hpp" with a literal backslash: file names with that
#     backslash are created as symlinks in a temporary include directory;
#   * g++ rejects `static alignas(32)` (src/foye_FFT_radix5.hpp:74, src/foye_FFT_radix7.hpp:79):
#     those two headers are staged into that directory with the specifiers reordered;
#   * aligned load/store intrinsics are mapped to unaligned ones (oracle/ref/gcc_shim.h).
set -euo pipefail
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$(cd "$HERE/.." && pwd)/_ref
if [ "$(uname -m)" != "x86_64" ]; then
  echo "build_ref: reference is x86 AVX2-only; not building on $(uname -m)" >&2; exit 3
fi
if [ ! -f "$REF/foye_FFT.hpp" ]; then
  echo "build_ref: no reference at $REF" >&2; exit 3
fi
mkdir -p "$OUT"
INC=$(mktemp -d)            # staging include dir, removed on exit; only the .so lands in _ref
trap 'rm -rf "$INC"' EXIT
cp "$HERE/windows_stub.h" "$INC/Windows.h"
for f in "$REF"/src/foye_FFT_*.hpp; do
  b=$(basename "$f")
  case "$b" in
    foye_FFT_radix5.hpp|foye_FFT_radix7.hpp)
      sed 's/static alignas(32)/alignas(32) static/' "$f" > "$INC/src\\$b" ;;
    *) ln -s "$f" "$INC/src\\$b" ;;
  esac
done
ln -s "$REF/foye_FFT.hpp" "$INC/foye_FFT.hpp"
g++ -std=c++20 -O2 -mavx2 -mfma -fPIC -shared -w -pthread \
    -include "$HERE/gcc_shim.h" -I "$INC" \
    "$HERE/ref_capi.cpp" -o "$OUT/libfyref.so"
echo "build_ref: wrote $OUT/libfyref.so"
