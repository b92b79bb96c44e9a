#!/bin/sh
# Builds the reference's own RRSPH_OMP compute core from its sources, together
# with oracle/ref_driver.cpp, into oracle/_ref/rrsph_ref (TEST INFRASTRUCTURE:
# used to pin the C oracle and as the "reference" CPU baseline). Outputs go to
# oracle/_ref/ only, which is kept out of version control.
#
# Where the reference checkout is present ($RRSPH_REFERENCE, default
# /root/reference), the few files the core needs are first staged, unchanged,
# under oracle/_ref/src/sources/ (the include directories of RRSPH_PARAMS,
# RRSPH_COMMON, RRSPH_OMP and RR, the six compiled .cpp files and the version
# templates); the core is always compiled from that staged copy, so a machine
# that has the staged copy but not the checkout builds the same binary.
#
# Only the compute core builds here: the reference's executable needs fmt and
# googletest, which it does not vendor. Two things differ from the reference
# tree, which itself is never written:
#   - the version headers are generated into oracle/_ref/gen/ from the
#     reference's *.h.in templates (CMake configure_file values of
#     CMakeLists.txt: RRSPH 3.1.4, RRSPH_COMMON 1.3.4, RRSPH_OMP 1.4.1);
#   - in the staged copy of RRFloatnDArray.h the MSVC-only
#     `throw std::exception{"..."}` becomes `throw std::runtime_error{"..."}`
#     (with <stdexcept>) so that GCC accepts it.
set -eu
REF="${RRSPH_REFERENCE:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
STAGE="$OUT/src/sources"
if [ -d "$REF/sources/RRSPH_OMP/src" ]; then
    R="$REF/sources"
    rm -rf "$OUT/src"
    mkdir -p "$STAGE/RRSPH_OMP/src" "$STAGE/RRSPH_COMMON/src" "$STAGE/RRSPH_PARAMS" "$STAGE/RRSPH_COMMON" \
             "$STAGE/RRSPH_OMP" "$STAGE/RR"
    cp -R "$R/RRSPH_PARAMS/include" "$STAGE/RRSPH_PARAMS/"
    cp -R "$R/RRSPH_COMMON/include" "$STAGE/RRSPH_COMMON/"
    cp -R "$R/RRSPH_OMP/include" "$STAGE/RRSPH_OMP/"
    cp -R "$R/RR/include" "$STAGE/RR/"
    for f in GridFind UpdateAcceleration PredictHalfStep WholeStep WaveMaker; do
        cp "$R/RRSPH_OMP/src/$f.cpp" "$STAGE/RRSPH_OMP/src/"
    done
    cp "$R/RRSPH_COMMON/src/EOS.cpp" "$STAGE/RRSPH_COMMON/src/"
    # the reference's parameter loaders, for the binding check (ref_params)
    mkdir -p "$STAGE/RRSPH_PARAMS/src" "$STAGE/RR/src" "$OUT/src/3d_party/nlohmann"
    cp "$R/RRSPH_PARAMS/src/ParticleParams.cpp" "$R/RRSPH_PARAMS/src/ModelParams.cpp" \
       "$R/RRSPH_PARAMS/src/Version.h" "$STAGE/RRSPH_PARAMS/src/"
    cp "$R/RR/src/Logger.cpp" "$STAGE/RR/src/"
    cp -R "$R/../3d_party/nlohmann/nlohmann" "$OUT/src/3d_party/nlohmann/"
    cp "$R/RRSPH_PARAMS/ParamsVersion.h.in" "$STAGE/RRSPH_PARAMS/"
    cp "$R/RRSPHVersion.h.in" "$STAGE/"
    cp "$R/RRSPH_COMMON/RRSPHCOMMONVersion.h.in" "$STAGE/RRSPH_COMMON/"
    cp "$R/RRSPH_OMP/RRSPHOMPVersion.h.in" "$STAGE/RRSPH_OMP/"
    chmod -R u+w "$OUT/src"
elif [ ! -d "$STAGE/RRSPH_OMP/src" ]; then
    echo "build_ref: reference sources not found under $REF or $STAGE; nothing built"
    exit 0
fi
S="$STAGE"
mkdir -p "$OUT/gen"
ver() { sed "s/@PROJECT_VERSION_MAJOR@/$2/;s/@PROJECT_VERSION_MINOR@/$3/;s/@PROJECT_VERSION_PATCH@/$4/" "$1"; }
ver "$S/RRSPH_PARAMS/ParamsVersion.h.in" 3 1 4 > "$OUT/gen/ParamsVersion.h"
ver "$S/RRSPHVersion.h.in" 3 1 4 > "$OUT/gen/RRSPHVersion.h"
ver "$S/RRSPH_COMMON/RRSPHCOMMONVersion.h.in" 1 3 4 > "$OUT/gen/RRSPHCOMMONVersion.h"
ver "$S/RRSPH_OMP/RRSPHOMPVersion.h.in" 1 4 1 > "$OUT/gen/RRSPHOMPVersion.h"
# the one-token GCC fix, applied to the staged copy (once)
FA="$S/RRSPH_PARAMS/include/RRFloatnDArray.h"
if grep -q 'std::exception{' "$FA"; then
    sed -e 's/std::exception{/std::runtime_error{/' -e 's/#include <variant>/#include <variant>\n#include <stdexcept>/' \
        "$FA" > "$FA.tmp" && mv "$FA.tmp" "$FA"
fi
rm -f "$OUT/gen/Params.h" "$OUT/gen/Types.h" "$OUT/gen/RRFloatnDArray.h"
chmod u+w "$OUT/gen/"*

CXX="${CXX:-g++}"
"$CXX" -std=c++20 -O2 -fopenmp -ffp-contract=off -w \
    -DRRSPH_OMP -DDO_ON_CPU=1 -DDO_ON_GPU=0 -DLOGGING_LEVEL=0 \
    -I"$OUT/gen" -I"$S/RRSPH_PARAMS/include" -I"$S/RRSPH_COMMON/include" \
    -I"$S/RRSPH_OMP/include" -I"$S/RR/include" \
    "$S/RRSPH_OMP/src/GridFind.cpp" "$S/RRSPH_OMP/src/UpdateAcceleration.cpp" \
    "$S/RRSPH_OMP/src/PredictHalfStep.cpp" "$S/RRSPH_OMP/src/WholeStep.cpp" \
    "$S/RRSPH_OMP/src/WaveMaker.cpp" "$S/RRSPH_COMMON/src/EOS.cpp" \
    "$HERE/ref_driver.cpp" -o "$OUT/rrsph_ref.tmp"
mv "$OUT/rrsph_ref.tmp" "$OUT/rrsph_ref"
echo "build_ref: built $OUT/rrsph_ref"

# The RRSPH_CUDA binding (sph2d_gb300/integration/) against the reference's
# headers: its parameter mapping linked with the reference's own loaders into
# oracle/_ref/ref_params, and its time_integration compiled (syntax only: the
# reference's RRSPHOutput needs fmt, which the reference does not vendor).
ROOT="$(cd "$HERE/.." && pwd)"
INTEG="$ROOT/sph2d_gb300/integration"
if [ -f "$S/RRSPH_PARAMS/src/ModelParams.cpp" ]; then
    "$CXX" -std=c++20 -O1 -w -DLOGGING_LEVEL=0 \
        -I"$OUT/gen" -I"$S/RRSPH_PARAMS/include" -I"$S/RRSPH_PARAMS/src" -I"$S/RR/include" \
        -I"$OUT/src/3d_party/nlohmann" -I"$ROOT/include" -I"$INTEG" -I"$ROOT/sph2d_gb300/host" \
        "$S/RRSPH_PARAMS/src/ParticleParams.cpp" "$S/RRSPH_PARAMS/src/ModelParams.cpp" "$S/RR/src/Logger.cpp" \
        "$INTEG/rrsph_cuda_params.cpp" "$HERE/ref_params_driver.cpp" -o "$OUT/ref_params.tmp"
    mv "$OUT/ref_params.tmp" "$OUT/ref_params"
    "$CXX" -std=c++20 -fsyntax-only -w -DRRSPH_CUDA -DDO_ON_CPU=1 -DDO_ON_GPU=0 -DLOGGING_LEVEL=0 \
        -I"$OUT/gen" -I"$S/RRSPH_PARAMS/include" -I"$S/RRSPH_COMMON/include" -I"$S/RRSPH_OMP/include" \
        -I"$S/RR/include" -I"$ROOT/include" -I"$INTEG" "$INTEG/TimeIntegration.cpp"
    echo "build_ref: built $OUT/ref_params; the RRSPH_CUDA time_integration compiles"
fi
