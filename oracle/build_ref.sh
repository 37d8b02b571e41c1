#!/usr/bin/env bash
# Builds the reference project's own CPU code for the oracle's pins into oracle/_ref/:
#   libconncomp_ref.so   src/segment/ConnComponents.cpp, unmodified, + oracle/ref_shim.cpp
#   libmorph_ref.so      the reference's serial reconstruction functions (line ranges of
#                        MorphologicOperations.cpp and PixelOperations.cpp, copied verbatim
#                        as text by `sed -n`) + ConnComponents.cpp, over oracle/cv_shim.hpp
#                        with OpenCV's CV_32S wrap-around (oracle/ref_morph.cpp)
#   libmorph_ref_sat.so  the same with saturating CV_32S arithmetic
# TEST INFRASTRUCTURE ONLY.
#
# Usage: build_ref.sh [REFERENCE_ROOT]   (or NSGB_REFERENCE_DIR=REFERENCE_ROOT build_ref.sh)
# REFERENCE_ROOT is the reference project's root (the directory holding src/segment).  With
# it, the sources are first copied into oracle/_ref/src/ (each range checked against the
# line it must start and end with); without it, the copies made earlier are compiled (the
# reference tree is only readable where the fixtures are made).  With neither, nothing is
# built and the script exits 0.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
out="$here/_ref"
srcdir="$out/src"
ref="${1:-${NSGB_REFERENCE_DIR:-}}"

# range FILE FIRST LAST FIRST_LINE_REGEX LAST_LINE_REGEX
range() {
  local f="$1" a="$2" b="$3" ra="$4" rb="$5"
  local first last
  first="$(sed -n "${a}p" "$f")"
  last="$(sed -n "${b}p" "$f")"
  if ! [[ "$first" =~ $ra ]] || ! [[ "$last" =~ $rb ]]; then
    echo "build_ref.sh: $f lines $a-$b do not match the expected reference version" >&2
    exit 1
  fi
  echo "// ---- $(basename "$f"):$a-$b (verbatim)"
  sed -n "${a},${b}p" "$f"
}

if [ -n "$ref" ]; then
  seg="$ref/src/segment"
  common="$ref/src/common"
  if [ ! -f "$seg/MorphologicOperations.cpp" ] || [ ! -f "$seg/ConnComponents.cpp" ]; then
    echo "build_ref.sh: no reference sources under $ref" >&2
    exit 1
  fi
  mkdir -p "$srcdir"
  mo="$seg/MorphologicOperations.cpp"
  {
    range "$mo" 428 439 '^template <typename T>$' '^}$'
    range "$mo" 665 838 '^template <typename T>$' '^}$'
    range "$mo" 1665 1673 '^template <typename T>$' '^}$'
    range "$mo" 1688 1829 '^template <typename T>$' '^}$'
    range "$mo" 1859 1926 '^template <typename T>$' '^}$'
    range "$mo" 1929 1951 '^template <typename T>$' '^}$'
    range "$mo" 2012 2035 '^Mat_<int> bwlabel2\(' '^}$'
    range "$mo" 2199 2232 '^Mat bwareaopen2\(' '^}$'
    range "$mo" 2260 2282 '^template <typename T>$' '^}$'
  } > "$srcdir/morph_ref.inc"
  range "$seg/PixelOperations.cpp" 17 39 '^template <typename T>$' '^}$' > "$srcdir/pixel_invert.inc"
  install -m 644 "$seg/ConnComponents.cpp" "$seg/ConnComponents.h" "$common/TypeUtils.h" "$srcdir/"
fi

if [ ! -f "$srcdir/morph_ref.inc" ]; then
  echo "reference sources not present; skipping oracle/_ref" >&2
  exit 0
fi

CXX="${CXX:-g++}"
flags=(-O2 -fPIC -shared -w -std=c++17 -ffp-contract=off -I"$here" -I"$srcdir")
"$CXX" "${flags[@]}" "$srcdir/ConnComponents.cpp" "$here/ref_shim.cpp" -o "$out/libconncomp_ref.so"
"$CXX" "${flags[@]}" -pthread "$srcdir/ConnComponents.cpp" "$here/ref_morph.cpp" -o "$out/libmorph_ref.so" &
p1=$!
"$CXX" "${flags[@]}" -pthread -DNSGB_SHIM_SATURATE_32S "$srcdir/ConnComponents.cpp" "$here/ref_morph.cpp" \
  -o "$out/libmorph_ref_sat.so" &
p2=$!
wait "$p1"
wait "$p2"
echo "built $out/libconncomp_ref.so, libmorph_ref.so, libmorph_ref_sat.so"
