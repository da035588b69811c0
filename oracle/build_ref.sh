#!/usr/bin/env bash
# Compile the reference's own OpenMP extensions (perm_c_omp.c,
# perm_binary_omp.c, perm_polynomial_omp.c and perm_mod3_omp.c) and the
# device code of its CUDA tools (perm_modp_cuda.cu, perm_binary_cuda.cu,
# perm_parallel_cuda.cu) from the reference checkout into oracle/_ref/.
# The extension modules are the CPU checker, the golden-vector generator and
# the CPU baseline; the cubins are the reference's GPU kernels for the
# same-GPU comparison and parity checks.  No reference source is copied into
# this repository.
#
# usage: oracle/build_ref.sh REFERENCE_DIR   (the rivin-perm checkout)
set -euo pipefail
if [ $# -ne 1 ]; then
  echo "usage: $0 REFERENCE_DIR" >&2
  exit 2
fi
REF="$1"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/perm_c_omp.c" ]; then
  echo "reference sources not found under $REF; oracle/_ref not built" >&2
  exit 0
fi
mkdir -p "$OUT" "$HERE/.tmp"
export TMPDIR="$HERE/.tmp"      # the compiler's temporary files stay in the tree
PYINC="$(python3 -c 'import sysconfig; print(sysconfig.get_paths()["include"])')"
NPINC="$(python3 -c 'import numpy; print(numpy.get_include())')"
SUFFIX="$(python3 -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')"
# outputs newer than their source are kept
fresh() { [ -f "$2" ] && [ "$2" -nt "$1" ]; }
fresh "$REF/perm_c_omp.c" "$OUT/perm_c_ext$SUFFIX" ||
  gcc -O3 -fopenmp -fPIC -shared -I"$PYINC" "$REF/perm_c_omp.c" -o "$OUT/perm_c_ext$SUFFIX" &
fresh "$REF/perm_binary_omp.c" "$OUT/perm_binary_ext$SUFFIX" ||
  gcc -O3 -fopenmp -fPIC -shared -I"$PYINC" "$REF/perm_binary_omp.c" -o "$OUT/perm_binary_ext$SUFFIX" &
fresh "$REF/perm_polynomial_omp.c" "$OUT/perm_polynomial_ext$SUFFIX" ||
  gcc -O3 -std=c11 -fopenmp -fPIC -shared -I"$PYINC" "$REF/perm_polynomial_omp.c" \
      -o "$OUT/perm_polynomial_ext$SUFFIX" &
fresh "$REF/perm_mod3_omp.c" "$OUT/perm_mod3_omp$SUFFIX" ||
  gcc -O3 -fopenmp -fPIC -shared -I"$PYINC" -I"$NPINC" "$REF/perm_mod3_omp.c" \
      -o "$OUT/perm_mod3_omp$SUFFIX" &
# the reference's CUDA kernels, device code only (cubins for sm_103a, loaded
# through the CUDA driver API by oracle/ref_cuda.py; the host code around
# them is restated there)
if command -v nvcc > /dev/null; then
  for f in perm_modp_cuda perm_binary_cuda perm_parallel_cuda; do
    fresh "$REF/$f.cu" "$OUT/$f.cubin" ||
      nvcc -gencode arch=compute_103a,code=sm_103a -O3 -cubin "$REF/$f.cu" -o "$OUT/$f.cubin" &
  done
fi
wait
echo "built the reference extensions into $OUT"
