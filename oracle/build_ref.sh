#!/bin/sh
# Builds oracle/_ref/libcmsl_ref.so: the reference's own kernels and host set-up
# code (jhb6617-arch/cmsl, HZO_Code_github/) compiled for the host CPU through
# oracle/shim/cuda_shim.h, plus oracle/ref_harness.cpp.  Test infrastructure
# only; the output stays in oracle/_ref/ (git-ignored).
#
# The reference is compiled from the sources where they lie.  Three files are
# used whole (kernels_evol.cu, global.cu, get_InputParams.cu, grain_io.cu,
# generate.cu);
# the kernel section of depol_varEPS.cu (lines 5-329), the kernel and the
# non-dimensionalisation functions of main.cu (lines 13-42, 200-256) and the
# host part of Init_Conf (init_conf.cu:108-279) are cut out with sed into
# oracle/_ref/ because the rest of those files needs a GPU runtime (cuBLAS,
# cuRAND, kernel launches) or does not compile as shipped (main.cu:483).
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default $CMSL_REFERENCE_ROOT, else /root/reference)
set -eu
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${CMSL_REFERENCE_ROOT:-/root/reference}}
SRC="$REF/HZO_Code_github/src"
INC="$REF/HZO_Code_github/include"
OUT="$HERE/_ref"
if [ ! -f "$SRC/kernels_evol.cu" ]; then
    echo "reference sources not found under $REF" >&2
    exit 3
fi
mkdir -p "$OUT"

{
    echo '#include "header.h"'
    sed -n '5,329p' "$SRC/depol_varEPS.cu"
} > "$OUT/depol_kernels.cpp"
{
    echo '#include "header.h"'
    sed -n '13,42p' "$SRC/main.cu"
    sed -n '200,256p' "$SRC/main.cu"
} > "$OUT/main_parts.cpp"
{
    echo '#include "header.h"'
    echo '#include <stdlib.h>'
    sed -n '108,279p' "$SRC/init_conf.cu"
    echo '}'
} > "$OUT/init_conf_host.cpp"

CXX=${CXX:-g++}
FLAGS="-O2 -fPIC -std=c++17 -fopenmp -ffp-contract=off -w -include $HERE/shim/cuda_shim.h -I$INC"
$CXX $FLAGS -shared -o "$OUT/libcmsl_ref.so" \
    -x c++ "$SRC/kernels_evol.cu" \
    -x c++ "$SRC/global.cu" \
    -x c++ "$SRC/get_InputParams.cu" \
    -x c++ "$SRC/grain_io.cu" \
    -x c++ "$SRC/generate.cu" \
    "$OUT/depol_kernels.cpp" "$OUT/main_parts.cpp" "$OUT/init_conf_host.cpp" \
    "$HERE/ref_harness.cpp" -lm
echo "built $OUT/libcmsl_ref.so"
