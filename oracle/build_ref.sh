#!/bin/sh
# Compiles the reference's own host sources for the single histogram filter,
# the permutation generator and the demo's biome layer chain, where they lie in the read-only reference
# tree, against the builder-written shims in oracle/refshim, into
# oracle/_ref/libstpref.so; and the reference's device code for simplex noise,
# the droplet, the demo's multi-biome and splatmap generator scripts with the
# splat rule lookups, the erosion brush and the format kernel, compiled as
# host C++ against oracle/refshim/device, into
# oracle/_ref/libstpref_device.so.  Run in the development container only (the
# reference tree is not present on GPU machines).  The reference's CMake
# build is not used.
set -e
REF=${STP_REFERENCE_ROOT:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
[ -d "$REF/SuperTerrain+" ] || { echo "reference tree not found at $REF" >&2; exit 3; }
mkdir -p "$OUT/src"
CORE="$REF/SuperTerrain+/SuperTerrain+"
ALG="$REF/SuperTerrain+/SuperAlgorithm+"
CUDA_INC=${CUDA_HOME:-/usr/local/cuda}/include
# The filter source is written for MSVC, which accepts a dependent type name
# without `typename` (STPSingleHistogramFilter.cpp:766-767); GCC does not.  The
# recipe adds that keyword on the fly into the git-ignored build folder
# and compiles the result; nothing of the reference is committed.
sed -e 's/typedef decay_t<decltype(memory)>::element_type BufferMemory;/typedef typename decay_t<decltype(memory)>::element_type BufferMemory;/' \
	-e 's/^\(\s*\)BufferMemory::STPWorkplace\* workplace;/\1typename BufferMemory::STPWorkplace* workplace;/' \
	"$ALG/Host/Private/STPSingleHistogramFilter.cpp" > "$OUT/src/STPSingleHistogramFilter.cpp"
# -O3 -mavx2 -mfma mirror the reference's release flags on x86
# (CMake/SetupEnvironment.cmake:34); other hosts get plain -O3.
ARCHFLAGS=""
case "$(uname -m)" in x86_64) ARCHFLAGS="-mavx2 -mfma";; esac
g++ -std=c++20 -O3 $ARCHFLAGS -fPIC -shared -pthread \
	-DSUPERTERRAINPLUS_EXPORTS -DSUPERALGORITHMPLUS_HOST_EXPORTS \
	-I"$HERE/refshim" -I"$CORE/Public" -I"$ALG/Host/Public" -I"$REF/SuperDemo+" -I"$CUDA_INC" -I"$CUDA_INC/cccl" \
	"$OUT/src/STPSingleHistogramFilter.cpp" \
	"$ALG/Host/Private/STPPermutationGenerator.cpp" \
	"$ALG/Host/Private/STPAlgorithmEnvironment.cpp" \
	"$CORE/Private/Utility/STPThreadPool.cpp" \
	"$CORE/Private/STPException.cpp" \
	"$CORE/Private/World/Diversity/STPLayer.cpp" \
	"$CORE/Private/World/Diversity/STPBiomeFactory.cpp" \
	"$REF/SuperDemo+/World/Layers/STPAllLayers.cpp" \
	"$REF/SuperDemo+/World/Biomes/STPBiomeRegistry.cpp" \
	"$HERE/refshim/cudart_host_shim.cpp" \
	"$HERE/refshim/ref_api.cpp" \
	-o "$OUT/libstpref.so"
echo "built $OUT/libstpref.so"
# Device code as host C++: the CUDA language extensions come from
# refshim/device/device_prelude.hpp (forced include), CUDA and libcu++ headers
# from the stand-ins beside it; no contraction into fused multiply-adds, so
# that every float operation rounds as written.  Two pieces are not whole
# files: the erosion brush generator is a static template inside
# STPHeightfieldGenerator.cpp, and the erosion and format kernels sit in
# STPHeightfieldKernel.cu beside the curand set-up kernel.  Their text is
# copied into the git-ignored build folder and included by
# refshim/device/ref_brush.cpp, ref_erosion_kernel.cpp and ref_format.cpp.
sed -n '/^static T generateErosionBrush/,/Populate Device Memory/p' \
	"$CORE/Private/World/Chunk/STPHeightfieldGenerator.cpp" > "$OUT/src/brush_generator.inc"
sed -n '/^#include <cuda\/std\/limits>/,$p' "$CORE/Private/GPGPU/STPHeightfieldKernel.cu" > "$OUT/src/format_kernel.inc"
sed -n '/^__global__ void hydraulicErosionKERNEL/,/^}/p' "$CORE/Private/GPGPU/STPHeightfieldKernel.cu" > "$OUT/src/erosion_kernel.inc"
for f in brush_generator format_kernel erosion_kernel; do
	[ -s "$OUT/src/$f.inc" ] || { echo "$f source not found" >&2; exit 4; }
done
g++ -std=c++20 -O2 -ffp-contract=off -fPIC -shared -Wl,--no-undefined -Wno-unknown-pragmas \
	-include "$HERE/refshim/device/device_prelude.hpp" -D__CUDACC__ -D__CUDACC_RTC__ -DSTP_IMPLEMENTATION -DNDEBUG \
	-I"$HERE/refshim/device" -I"$HERE/refshim" -I"$CORE/Public" -I"$ALG/Device/Public" -I"$ALG/Host/Public" \
	-I"$REF/SuperDemo+" -I"$OUT/src" \
	-x c++ "$ALG/Device/Private/STPSimplexNoise.cu" \
	"$CORE/Private/GPGPU/STPRainDrop.cu" \
	"$REF/SuperDemo+/Script/STPCommonGenerator.cu" \
	"$REF/SuperDemo+/Script/STPMultiHeightGenerator.cu" \
	"$REF/SuperDemo+/Script/STPSplatmapGenerator.cu" \
	"$ALG/Device/Private/STPTextureSplatRuleWrapper.cu" \
	-x none "$HERE/refshim/device/ref_device_api.cpp" \
	"$HERE/refshim/device/ref_splat_api.cpp" \
	"$HERE/refshim/device/ref_brush.cpp" \
	"$HERE/refshim/device/ref_format.cpp" \
	"$HERE/refshim/device/ref_erosion_kernel.cpp" \
	-o "$OUT/libstpref_device.so"
echo "built $OUT/libstpref_device.so"
