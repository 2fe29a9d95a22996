#!/usr/bin/env bash
# Builds the reference's own C++ (exafac/cpp_ext, read where it lies under the
# reference checkout) into oracle/_ref/exafac_ref*.so, for golden-vector
# generation and oracle pinning.  Test infrastructure only.
#
#   oracle/build_ref.sh [REFERENCE_ROOT]     (default: /root/reference)
#
# Stand-ins: oracle/ref_shim/{mpi.h,cblas.h,lapacke.h} (single-rank MPI;
# CBLAS/LAPACKE names bound to scipy's bundled OpenBLAS).  The reference's
# cppimport build is replaced by one g++ call.  Flags: the reference uses
# -Ofast -march=native (config_template.json:2); golden vectors are built with
# IEEE semantics (-O2, no fast-math) so that the sequential sums in
# std::discrete_distribution and the tree descents keep their written order.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-/root/reference}"
SRC="$REF/exafac/cpp_ext"
if [ ! -d "$SRC" ]; then
    echo "reference sources not found at $SRC; skipping oracle/_ref" >&2
    exit 0
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
PY=${PYTHON:-python3}
PYINC=$($PY -c "import sysconfig; print(sysconfig.get_paths()['include'])")
PBINC=$($PY -c "import pybind11; print(pybind11.get_include())" 2>/dev/null || \
        $PY -c "import torch, os; print(os.path.join(os.path.dirname(torch.__file__), 'include'))")
SUFFIX=$($PY -c "import sysconfig; print(sysconfig.get_config_var('EXT_SUFFIX'))")
BLASDIR=$($PY -c "import scipy, os; print(os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), 'scipy.libs'))")
BLASLIB=$(ls "$BLASDIR" | grep -m1 '^libscipy_openblas.*\.so$')
g++ -std=c++2a -O2 -fopenmp -fPIC -shared -w \
    -I"$HERE/ref_shim" -I"$SRC" -I"$PBINC" -I"$PYINC" \
    "$HERE/ref_harness.cpp" -o "$OUT/exafac_ref$SUFFIX" \
    -L"$BLASDIR" -l:"$BLASLIB" -Wl,-rpath,"$BLASDIR"
echo "built $OUT/exafac_ref$SUFFIX"
