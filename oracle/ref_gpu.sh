#!/bin/sh
# The reference program (HZO_Code_github: FP64 CUDA kernels, cuBLAS PCG) built
# for sm_103a, to time "the plain FP64 GPU path" beside this library.  Test
# and measurement infrastructure only; nothing of the library links it.
#
#   oracle/ref_gpu.sh stage [REFERENCE_ROOT]
#       (where the reference sources lie; default $CMSL_REFERENCE_ROOT, else
#       /root/reference) copies HZO_Code_github/src/*.cu and include/ into
#       baseline/_ref/hzo (git-ignored, so it is never committed; it travels
#       with the working tree to a GPU machine) and makes the three changes
#       the shipped sources need to compile with CUDA 13:
#         - -std=c++17 instead of the Makefile's -std=c++14 (CUB needs C++17);
#         - the stray closing brace at src/evolve.cu:442 removed;
#         - src/main.cu:483 calls ReadGrainCount with its one declared
#           argument (include/header.h:22, src/grain_io.cu:10).
#   oracle/ref_gpu.sh build
#       (on the GPU machine) compiles baseline/_ref/hzo/Pfmhzo.exe with the
#       Makefile's flags and libraries (Makefile:12-17) for sm_103a, and
#       Pfmhzo_gb: the same program linked with this library's compat layer
#       (Evolve / Depol_field on libcmsl_gb).
set -eu
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(dirname "$HERE")
OUT="$ROOT/baseline/_ref/hzo"
case "${1:-}" in
stage)
    REF=${2:-${CMSL_REFERENCE_ROOT:-/root/reference}}
    SRC="$REF/HZO_Code_github"
    [ -f "$SRC/src/evolve.cu" ] || { echo "reference sources not found under $REF" >&2; exit 3; }
    mkdir -p "$OUT/src" "$OUT/include"
    cp "$SRC"/src/*.cu "$OUT/src/"
    cp "$SRC"/include/*.h "$OUT/include/"
    # the stray brace: line 442 must be exactly "}"
    [ "$(sed -n 442p "$OUT/src/evolve.cu")" = "}" ] || { echo "evolve.cu:442 is not the stray brace" >&2; exit 4; }
    sed -i '442d' "$OUT/src/evolve.cu"
    grep -q 'ReadGrainCount(struct_dir, grain_tag);' "$OUT/src/main.cu" || { echo "main.cu:483 changed" >&2; exit 4; }
    sed -i 's/ReadGrainCount(struct_dir, grain_tag);/ReadGrainCount(grain_tag);/' "$OUT/src/main.cu"
    echo "staged $OUT"
    ;;
build)
    [ -f "$OUT/src/evolve.cu" ] || { echo "not staged: run oracle/ref_gpu.sh stage where the reference is" >&2; exit 3; }
    NVCC=${NVCC:-nvcc}
    mkdir -p "$OUT/build"
    pids=""
    for f in "$OUT"/src/*.cu; do
        b=$(basename "$f" .cu)
        $NVCC -gencode arch=compute_103a,code=sm_103a -O2 -std=c++17 -I"$OUT/include" -dc \
              -Xcompiler -Wno-deprecated-declarations "$f" -o "$OUT/build/$b.o" &
        pids="$pids $!"
    done
    for p in $pids; do wait "$p"; done
    $NVCC -gencode arch=compute_103a,code=sm_103a "$OUT"/build/*.o -o "$OUT/Pfmhzo.exe" \
          -lcurand -lcufft -lcublas -lcusparse -lm -lstdc++
    echo "built $OUT/Pfmhzo.exe"
    # the same program with this library's hot path: the set-up and driver
    # objects with cmsl_gb300/cmsl_refcompat.o in place of evolve.cu,
    # kernels_evol.cu and depol_varEPS.cu (build the library first)
    if [ -f "$ROOT/cmsl_gb300/cmsl_refcompat.o" ] && [ -f "$ROOT/cmsl_gb300/libcmsl_gb.so" ]; then
        B="$OUT/build"
        $NVCC -gencode arch=compute_103a,code=sm_103a -rdc=true "$B/main.o" "$B/init_conf.o" "$B/grain_io.o" \
              "$B/get_InputParams.o" "$B/allocateVars.o" "$B/cleanup.o" "$B/generate.o" "$B/global.o" \
              "$ROOT/cmsl_gb300/cmsl_refcompat.o" -L"$ROOT/cmsl_gb300" -lcmsl_gb -lcurand \
              -Xlinker -rpath,"$ROOT/cmsl_gb300" -o "$OUT/Pfmhzo_gb"
        echo "built $OUT/Pfmhzo_gb"
    fi
    ;;
*)
    echo "usage: $0 stage [REFERENCE_ROOT] | build" >&2
    exit 2
    ;;
esac
