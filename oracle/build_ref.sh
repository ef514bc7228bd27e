#!/bin/sh
# Compiles the reference's own code for the oracle's pins (test
# infrastructure only; the reference's CMake build is not used):
#   oracle/_ref/libstpref.so        host sources: the single histogram filter,
#                                   the permutation generator and the demo's
#                                   biome layer chain, against oracle/refshim;
#   oracle/_ref/libstpref_device.so device code compiled as host C++ against
#                                   oracle/refshim/device: simplex noise, the
#                                   droplet, the demo's multi-biome and
#                                   splatmap generator scripts with the splat
#                                   rule lookups, the erosion brush, the
#                                   erosion kernel and the format kernel;
#   oracle/_ref/libstpref_gpu.so    the erosion kernel and the droplet
#                                   compiled by nvcc for sm_103a (relocatable
#                                   device code, -DNDEBUG as the reference's
#                                   release build) with the harness in
#                                   oracle/refshim/gpu.
# Sources: with STP_REFERENCE_ROOT set to a reference checkout, the recipe
# first copies the subset of the tree these builds read into the git-ignored
# oracle/_ref/tree (so that machines without the checkout can rebuild from
# it); without it, it builds from that copy.  Nothing of the reference is
# committed.  The three libraries compile in parallel.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
TREE="$OUT/tree"
if [ -n "$STP_REFERENCE_ROOT" ]; then
	[ -d "$STP_REFERENCE_ROOT/SuperTerrain+" ] || { echo "no reference tree at STP_REFERENCE_ROOT=$STP_REFERENCE_ROOT" >&2; exit 3; }
	rm -rf "$TREE.tmp"
	mkdir -p "$TREE.tmp"
	for d in "SuperTerrain+/SuperTerrain+/Public" "SuperTerrain+/SuperTerrain+/Private" "SuperTerrain+/SuperAlgorithm+" \
		"SuperDemo+/World" "SuperDemo+/Script" "SuperTest+/SuperTerrain+/STPTest2DChunk.cpp"; do
		mkdir -p "$TREE.tmp/$(dirname "$d")"
		cp -R "$STP_REFERENCE_ROOT/$d" "$TREE.tmp/$d"
	done
	rm -rf "$TREE"
	mv "$TREE.tmp" "$TREE"
fi
[ -d "$TREE/SuperTerrain+" ] || { echo "no reference sources: set STP_REFERENCE_ROOT to a reference checkout" >&2; exit 3; }
REF="$TREE"
mkdir -p "$OUT/src"
CORE="$REF/SuperTerrain+/SuperTerrain+"
ALG="$REF/SuperTerrain+/SuperAlgorithm+"
CUDA_HOME=${CUDA_HOME:-/usr/local/cuda}
CUDA_INC=$CUDA_HOME/include
# The filter source is written for MSVC, which accepts a dependent type name
# without `typename` (STPSingleHistogramFilter.cpp:766-767); GCC does not.  The
# recipe adds that keyword on the fly into the git-ignored build folder
# and compiles the result.
sed -e 's/typedef decay_t<decltype(memory)>::element_type BufferMemory;/typedef typename decay_t<decltype(memory)>::element_type BufferMemory;/' \
	-e 's/^\(\s*\)BufferMemory::STPWorkplace\* workplace;/\1typename BufferMemory::STPWorkplace* workplace;/' \
	"$ALG/Host/Private/STPSingleHistogramFilter.cpp" > "$OUT/src/STPSingleHistogramFilter.cpp"
# Two pieces are not whole files: the erosion brush generator is a static
# template inside STPHeightfieldGenerator.cpp, and the erosion and format
# kernels sit in STPHeightfieldKernel.cu beside the curand set-up kernel.
# Their text is copied into the build folder and included by
# refshim/device/ref_brush.cpp, ref_erosion_kernel.cpp, ref_format.cpp and
# refshim/gpu/ref_erosion_gpu.cu.
sed -n '/^static T generateErosionBrush/,/Populate Device Memory/p' \
	"$CORE/Private/World/Chunk/STPHeightfieldGenerator.cpp" > "$OUT/src/brush_generator.inc"
sed -n '/^#include <cuda\/std\/limits>/,$p' "$CORE/Private/GPGPU/STPHeightfieldKernel.cu" > "$OUT/src/format_kernel.inc"
sed -n '/^__global__ void hydraulicErosionKERNEL/,/^}/p' "$CORE/Private/GPGPU/STPHeightfieldKernel.cu" > "$OUT/src/erosion_kernel.inc"
for f in brush_generator format_kernel erosion_kernel; do
	[ -s "$OUT/src/$f.inc" ] || { echo "$f source not found" >&2; exit 4; }
done

# -O3 -mavx2 -mfma mirror the reference's release flags on x86
# (CMake/SetupEnvironment.cmake:34); other hosts get plain -O3.
ARCHFLAGS=""
case "$(uname -m)" in x86_64) ARCHFLAGS="-mavx2 -mfma";; esac
# -Bsymbolic binds the library's calls of the CUDA runtime to the host
# stand-ins it carries (refshim/cudart_host_shim.cpp), also in a process
# that has loaded the real runtime globally first (as PyTorch does).
build_host() {
	g++ -std=c++20 -O3 $ARCHFLAGS -fPIC -shared -pthread -Wl,-Bsymbolic \
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
		-o "$OUT/libstpref.so.tmp" && mv "$OUT/libstpref.so.tmp" "$OUT/libstpref.so" && echo "built $OUT/libstpref.so"
}
# Device code as host C++: the CUDA language extensions come from
# refshim/device/device_prelude.hpp (forced include), CUDA and libcu++ headers
# from the stand-ins beside it; no contraction into fused multiply-adds, so
# that every float operation rounds as written.
build_device_host() {
	g++ -std=c++20 -O3 -ffp-contract=off -fPIC -shared -Wl,--no-undefined,-Bsymbolic -Wno-unknown-pragmas \
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
		-o "$OUT/libstpref_device.so.tmp" && mv "$OUT/libstpref_device.so.tmp" "$OUT/libstpref_device.so" \
		&& echo "built $OUT/libstpref_device.so"
}
# The reference's erosion for the GPU: its release flags (-O3, -DNDEBUG,
# separable compilation, --extended-lambda: CMake/SetupEnvironment.cmake:45-47)
# for sm_103a, against the vector subset in refshim/glm, whose functions are
# host and device functions under nvcc.
build_gpu() {
	NVCC="$CUDA_HOME/bin/nvcc"
	[ -x "$NVCC" ] || NVCC=nvcc
	"$NVCC" -gencode arch=compute_103a,code=sm_103a -O3 -rdc=true --extended-lambda -std=c++20 \
		-DSTP_IMPLEMENTATION -DNDEBUG -Xcompiler -fPIC -shared \
		-I"$HERE/refshim" -I"$CORE/Public" -I"$OUT/src" \
		"$CORE/Private/GPGPU/STPRainDrop.cu" "$HERE/refshim/gpu/ref_erosion_gpu.cu" \
		-o "$OUT/libstpref_gpu.so.tmp" && mv "$OUT/libstpref_gpu.so.tmp" "$OUT/libstpref_gpu.so" \
		&& echo "built $OUT/libstpref_gpu.so"
}
build_host & P1=$!
build_device_host & P2=$!
build_gpu & P3=$!
RC=0
wait $P1 || RC=1
wait $P2 || RC=1
wait $P3 || RC=1
exit $RC
