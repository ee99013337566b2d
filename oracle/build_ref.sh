#!/usr/bin/env bash
# Builds the unmodified reference (biointec/blamm) CPU binary from its own
# sources into oracle/_ref/, bypassing its CMake (which needs a Fortran
# compiler only to probe the BLAS name mangling).  Test infrastructure only:
# the binary is the checker that pins the oracle restatement and generates the
# golden fixtures; nothing in the product links or runs it.
#
#   usage: oracle/build_ref.sh [reference_root]
#   (default: $BLAMM_REFERENCE_DIR, else the DEFAULT_REF below)
#
# BLAS: scipy's bundled LP64 OpenBLAS (exports scipy_sgemm_).  numpy's
# scipy_openblas64_ is ILP64 and must not be used (wrong integer width).
set -euo pipefail
DEFAULT_REF=/root/reference
REF=${1:-${BLAMM_REFERENCE_DIR:-$DEFAULT_REF}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
[ -d "$REF/src" ] || { echo "reference sources not found at $REF" >&2; exit 2; }
mkdir -p "$OUT"

SCIPY_LIBS=$(python3 - <<'PY'
import os, scipy
print(os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs"))
PY
)
BLAS=$(ls "$SCIPY_LIBS"/libscipy_openblas-*.so 2>/dev/null | grep -v openblas64 | head -1 || true)
[ -n "$BLAS" ] || { echo "no LP64 scipy OpenBLAS found in $SCIPY_LIBS" >&2; exit 3; }

# hand-written config.h: the F77 mangling of scipy's OpenBLAS
cat > "$OUT/config.h" <<'EOF'
#ifndef CMAKE_CONFIG_H
#define CMAKE_CONFIG_H
#define F77_FUNC(name,NAME) scipy_ ## name ## _
#endif
EOF

SRCS="dict hist blstools bls phylotree matrix pwmscan motif sequence ortho species settings"
OBJS=""
pids=""
for s in $SRCS; do
  # -include: species.h uses std::array (and others) without including them under gcc 13
  g++ -O3 -std=c++11 -DNDEBUG -DHAVE_CONFIG_H -DBLAMM_MAJOR_VERSION=1 -DBLAMM_MINOR_VERSION=0 \
      -DBLAMM_PATCH_LEVEL=0 -I"$OUT" -I"$REF/src" \
      -include array -include mutex -include cassert -include limits -include stdexcept -include map \
      -w -c "$REF/src/$s.cpp" -o "$OUT/$s.o" &
  pids="$pids $!"
  OBJS="$OBJS $OUT/$s.o"
done
for p in $pids; do wait $p; done
g++ -o "$OUT/blamm" $OBJS -L"$(dirname "$BLAS")" -l:"$(basename "$BLAS")" \
    -Wl,-rpath,"$(dirname "$BLAS")" -lpthread
rm -f $OBJS
echo "built $OUT/blamm (BLAS: $BLAS)"
