#!/bin/sh
# Links the reference program against libcmsl_gb: the reference's main.cu,
# init_conf.cu, grain_io.cu, get_InputParams.cu, allocateVars.cu, cleanup.cu,
# generate.cu and global.cu, compiled where they lie, plus
# cmsl_gb300/cmsl_refcompat.o in place of evolve.cu, kernels_evol.cu and
# depol_varEPS.cu.  main.cu calls ReadGrainCount with two arguments where it is
# declared with one (main.cu:483 vs include/header.h:22); the call is
# corrected on a copy in the output directory.  Test infrastructure only.
# Usage: link_reference.sh REFERENCE_ROOT REPO_ROOT OUT_DIR
set -eu
R="$1/HZO_Code_github"
REPO="$2"
OUT="$3"
ARCH="-gencode arch=compute_103a,code=sm_103a"
mkdir -p "$OUT"
sed 's/ReadGrainCount(struct_dir, grain_tag);/ReadGrainCount(grain_tag);/' "$R/src/main.cu" > "$OUT/main_fixed.cu"
for f in init_conf grain_io get_InputParams allocateVars cleanup generate global; do
    nvcc $ARCH -std=c++17 -dc -I"$R/include" "$R/src/$f.cu" -o "$OUT/$f.o"
done
nvcc $ARCH -std=c++17 -dc -I"$R/include" "$OUT/main_fixed.cu" -o "$OUT/main.o"
nvcc $ARCH -rdc=true "$OUT"/main.o "$OUT"/init_conf.o "$OUT"/grain_io.o "$OUT"/get_InputParams.o \
    "$OUT"/allocateVars.o "$OUT"/cleanup.o "$OUT"/generate.o "$OUT"/global.o \
    "$REPO/cmsl_gb300/cmsl_refcompat.o" -L"$REPO/cmsl_gb300" -lcmsl_gb -lcurand \
    -Xlinker -rpath,"$REPO/cmsl_gb300" -o "$OUT/Pfmhzo_gb"
echo "linked $OUT/Pfmhzo_gb"
