#!/bin/sh
# Compiles the reference's own host sources for the single histogram filter,
# the permutation generator and the demo's biome layer chain, where they lie in the read-only reference
# tree, against the builder-written shims in oracle/refshim, into
# oracle/_ref/libstpref.so.  Run in the development container only (the
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
