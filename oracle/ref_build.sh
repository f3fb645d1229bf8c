#!/bin/sh
# Builds the reference's own SolCx analytic solution (benchmarks/solcx/solcx.h,
# function _Velic_solCx) into oracle/_ref/libsolcx.so, compiled from the
# reference source where it lies. The function body is taken by line range at
# build time into oracle/_ref/ (git-ignored); nothing of it enters the repo.
# Used only to generate the golden fixtures under tests/golden/.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
# the reference tree: $ASPECT_REFERENCE, else a directory "reference" beside the repository
REF=${ASPECT_REFERENCE:-$(cd "$HERE/../.." && pwd)/reference}
OUT="$HERE/_ref"
SRC="$REF/benchmarks/solcx/solcx.h"
[ -f "$SRC" ] || { echo "reference not present: $SRC" >&2; exit 2; }
mkdir -p "$OUT"
start=$(grep -n "void _Velic_solCx(" "$SRC" | head -1 | cut -d: -f1)
# the function ends at the first line that is exactly six spaces and a brace after $start
end=$(awk -v s="$start" 'NR>s && /^      }$/ {print NR; exit}' "$SRC")
{
  echo '#include <cmath>'
  echo '#include <cassert>'
  echo 'namespace numbers { constexpr double PI = 3.14159265358979323846; }'
  echo 'extern "C" {'
  sed -n "${start},${end}p" "$SRC"
  echo '}'
} > "$OUT/solcx_extract.cc"
${CXX:-g++} -O2 -fPIC -shared -o "$OUT/libsolcx.so" "$OUT/solcx_extract.cc"
echo "$OUT/libsolcx.so"
