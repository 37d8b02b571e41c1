#!/usr/bin/env bash
# Builds oracle/_ref/libconncomp_ref.so from the reference project's own
# src/segment/ConnComponents.cpp (compiled unmodified, in place, from the read-only source
# tree) plus oracle/ref_shim.cpp.  Used only to pin the CPU oracle.  Needs the reference
# tree; exits 0 without building when it is absent.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${NSGB_REFERENCE_DIR:-/root/reference/fastIA-master}"
src="$ref/src/segment"
if [ ! -f "$src/ConnComponents.cpp" ]; then
  echo "reference sources not present; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$here/_ref"
g++ -O2 -fPIC -shared -w -I"$src" "$src/ConnComponents.cpp" "$here/ref_shim.cpp" \
    -o "$here/_ref/libconncomp_ref.so"
echo "built $here/_ref/libconncomp_ref.so"
