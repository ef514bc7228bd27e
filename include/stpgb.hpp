/*
 * stpgb.hpp — C++ façade over the C ABI (stpgb.h) with the reference's class
 * names, namespaces and exception types for the heightfield path, so that a
 * C++ caller of SuperTerrain+ switches by changing includes and linking
 * libstpgb.so.  Header-only; vector-like arguments accept any type with
 * .x / .y members (glm::vec2, glm::uvec2, ...).
 *
 *   SuperTerrainPlus::STPAlgorithm::STPPermutationGenerator::generate
 *       (SuperAlgorithm+Host/STPPermutationGenerator.h:23-50)
 *   SuperTerrainPlus::STPAlgorithm::STPSingleHistogramFilter + STPFilterBuffer
 *       (SuperAlgorithm+Host/STPSingleHistogramFilter.h:36-190)
 *   SuperTerrainPlus::STPHeightfieldGenerator(STPGeneratorSetup), generate / erode
 *       (SuperTerrain+/World/Chunk/STPHeightfieldGenerator.h:35-45,121,145,159)
 *   SuperTerrainPlus::STPDiversityGenerator, the nearest-neighbour texture buffers
 *       (SuperTerrain+/World/Chunk/STPDiversityGenerator.hpp:14-39,
 *        STPNearestNeighbourTextureBuffer.h), STPDemo::STPBiomefieldGenerator
 *       (SuperDemo+/World/Biomes/STPBiomefieldGenerator.h:26-98)
 *   SuperTerrainPlus::STPDiversity::STPBiomeFactory, STPDemo::STPLayerChainBuilder
 *       (SuperTerrain+/World/Diversity/STPBiomeFactory.h:19-63, SuperDemo+/World/Layers/STPAllLayers.h)
 *   SuperTerrainPlus::STPChunk coordinate functions
 *       (SuperTerrain+/World/Chunk/STPChunk.h:110-157)
 *   SuperTerrainPlus::STPException::{STPNumericDomainError, STPInvalidEnvironment, STPCUDAError}
 */
#ifndef STPGB_HPP_
#define STPGB_HPP_

#include "stpgb.h"

#include <cstdint>
#include <exception>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace SuperTerrainPlus {

typedef uint16_t STPSample_t;
typedef float STPHeightFloat_t;
typedef uint16_t STPHeightFixed_t;
typedef uint64_t STPSeed_t;

namespace STPException {

class STPFundamentalException : public std::runtime_error {
public:
	using std::runtime_error::runtime_error;
};
class STPNumericDomainError : public STPFundamentalException {
public:
	using STPFundamentalException::STPFundamentalException;
};
class STPInvalidEnvironment : public STPFundamentalException {
public:
	using STPFundamentalException::STPFundamentalException;
};
class STPCUDAError : public STPFundamentalException {
public:
	using STPFundamentalException::STPFundamentalException;
};
class STPInsufficientMemory : public STPFundamentalException {
public:
	using STPFundamentalException::STPFundamentalException;
};

} // namespace STPException

namespace detail {

// Throws the reference's exception type for a C ABI status; `environment`
// selects STPInvalidEnvironment for setting validation failures.
inline void check(int rc, bool environment = false) {
	if (rc == STPGB_OK) {
		return;
	}
	const std::string msg = stpgb_last_error();
	switch (rc) {
	case STPGB_EINVAL:
		if (environment) {
			throw STPException::STPInvalidEnvironment(msg);
		}
		throw STPException::STPNumericDomainError(msg);
	case STPGB_ECUDA:
		throw STPException::STPCUDAError(msg);
	case STPGB_ENOMEM:
		throw STPException::STPInsufficientMemory(msg);
	default:
		throw STPException::STPFundamentalException("status " + std::to_string(rc) + ": " + msg);
	}
}

template<class V>
stpgb_nn_info nn(const V& map, const V& neighbour) {
	stpgb_nn_info i {};
	i.MapSize[0] = static_cast<uint32_t>(map.x);
	i.MapSize[1] = static_cast<uint32_t>(map.y);
	i.ChunkNearestNeighbour[0] = static_cast<uint32_t>(neighbour.x);
	i.ChunkNearestNeighbour[1] = static_cast<uint32_t>(neighbour.y);
	i.TotalMapSize[0] = i.MapSize[0] * i.ChunkNearestNeighbour[0];
	i.TotalMapSize[1] = i.MapSize[1] * i.ChunkNearestNeighbour[1];
	return i;
}

} // namespace detail

namespace STPEnvironment {

struct STPSimplexNoiseSetting : stpgb_simplex_setting {
	void validate() const {
		detail::check(stpgb_simplex_setting_validate(this), true);
	}
};

struct STPRainDropSetting : stpgb_raindrop_setting {
	void validate() const {
		detail::check(stpgb_raindrop_setting_validate(this), true);
	}
};

} // namespace STPEnvironment

namespace STPAlgorithm {

/* STPSingleHistogram (SuperAlgorithm+Host/STPSingleHistogram.hpp:15-50) */
struct STPSingleHistogram {
	typedef stpgb_bin STPBin;
	const STPBin* Bin;
	const unsigned int* HistogramStartOffset;
};

class STPSingleHistogramFilter {
public:
	class STPFilterBuffer {
	public:
		enum class STPExecutionType : unsigned char { Serial = 0x00u, Parallel = 0x01u };
		typedef std::pair<size_t, size_t> STPHistogramSize;

		explicit STPFilterBuffer(STPExecutionType type) : Type(type) {}

		STPSingleHistogram readHistogram() const {
			return STPSingleHistogram { Bins.data(), Offsets.data() };
		}
		STPHistogramSize size() const {
			return { Bins.size(), Offsets.size() };
		}
		STPExecutionType type() const noexcept {
			return Type;
		}

	private:
		friend class STPSingleHistogramFilter;
		STPExecutionType Type;
		std::vector<stpgb_bin> Bins;
		std::vector<unsigned int> Offsets;
	};

	/* `nn_info` is any STPNearestNeighbourInformation-like value with
	 * MapSize / ChunkNearestNeighbour members (.x, .y).  Both execution
	 * types run the same GPU filter and give the reference's result. */
	template<class NN>
	STPSingleHistogram operator()(const STPSample_t* samplemap, const NN& nn_info, STPFilterBuffer& buffer,
		unsigned int radius) {
		const stpgb_nn_info info = detail::nn(nn_info.MapSize, nn_info.ChunkNearestNeighbour);
		const size_t npix = static_cast<size_t>(info.MapSize[0]) * info.MapSize[1];
		const uint64_t side = 2ull * radius + 1ull;
		const uint64_t cap = npix * (side * side < 256u ? side * side : 256u);
		buffer.Offsets.resize(npix + 1u);
		buffer.Bins.resize(static_cast<size_t>(cap > 0u ? cap : 1u));
		uint64_t n = 0u;
		detail::check(stpgb_shf_filter_host(samplemap, &info, radius, buffer.Offsets.data(), buffer.Bins.data(), cap, &n));
		buffer.Bins.resize(static_cast<size_t>(n));
		return buffer.readHistogram();
	}
};

/* STPPermutation (SuperAlgorithm+Host/STPPermutation.hpp:9-22), device pointers */
typedef stpgb_permutation STPPermutation;

namespace STPPermutationGenerator {

/* Host copies of the generated tables; Permutation points at device copies
 * made by upload() (the reference keeps only device memory). */
class STPPermutationTable {
public:
	std::vector<uint8_t> HostPermutation;
	std::vector<float> HostGradient2D;
	STPPermutation Permutation {};
};

inline STPPermutationTable generate(const STPEnvironment::STPSimplexNoiseSetting& setting) {
	setting.validate();
	STPPermutationTable t;
	t.HostPermutation.resize(512u);
	t.HostGradient2D.resize(2u * setting.Distribution);
	detail::check(stpgb_permutation_generate(&setting, t.HostPermutation.data(), t.HostGradient2D.data(),
		static_cast<uint32_t>(t.HostGradient2D.size())), true);
	t.Permutation.Gradient2DSize = setting.Distribution;
	return t;
}

} // namespace STPPermutationGenerator

} // namespace STPAlgorithm

namespace STPDiversity {

/* STPBiomeFactory (SuperTerrain+/World/Diversity/STPBiomeFactory.h:19-63)
 * over a linear chain of the demo's layer kinds, evaluated on the GPU:
 * factory(biomemap, offset) fills a host array of BiomeDimension.x *
 * BiomeDimension.y samples of world pixels offset + (x, z), row-major, as
 * STPBiomeFactory::operator() (STPBiomeFactory.cpp:24-41) does. */
class STPBiomeFactory {
public:
	template<class V>
	STPBiomeFactory(const V& dimension, STPSeed_t global_seed, std::vector<stpgb_layer> chain,
		const stpgb_layer_biomes& ids) :
		DimX(static_cast<uint32_t>(dimension.x)), DimY(static_cast<uint32_t>(dimension.y)), Seed(global_seed),
		Chain(std::move(chain)), Ids(ids) {
		if (dimension.x <= 0 || dimension.y <= 0) {
			throw STPException::STPNumericDomainError(
				"Biomemap should have strictly positive dimension in both vector components");
		}
	}

	template<class IV>
	void operator()(STPSample_t* biomemap, const IV& offset) const {
		detail::check(stpgb_layer_biomemap_host(Chain.data(), static_cast<uint32_t>(Chain.size()), Seed, &Ids,
			biomemap, DimX, DimY, static_cast<int32_t>(offset.x), static_cast<int32_t>(offset.y)));
	}

	uint32_t dimensionX() const noexcept {
		return DimX;
	}
	uint32_t dimensionY() const noexcept {
		return DimY;
	}

private:
	uint32_t DimX, DimY;
	STPSeed_t Seed;
	std::vector<stpgb_layer> Chain;
	stpgb_layer_biomes Ids;
};

/* The splatmap generator (STPTextureFactory::operator(),
 * SuperTerrain+/Private/World/Diversity/STPTextureFactory.cpp:211-232, with
 * the demo's STPSplatmapGenerator kernel): rules added per biome sample as
 * STPTextureSplatBuilder::addAltitude / addGradient add them, then one call
 * per rendering buffer on device pointers. */
class STPTextureSplatGenerator {
public:
	template<class V>
	STPTextureSplatGenerator(const std::vector<stpgb_altitude_rule>& altitude,
		const std::vector<stpgb_gradient_rule>& gradient, const STPEnvironment::STPSimplexNoiseSetting& simplex,
		const V& map_size) {
		simplex.validate();
		stpgb_splat_generator* g = nullptr;
		detail::check(stpgb_splat_generator_create(altitude.data(), static_cast<uint32_t>(altitude.size()),
			gradient.data(), static_cast<uint32_t>(gradient.size()), &simplex, static_cast<uint32_t>(map_size.x),
			static_cast<uint32_t>(map_size.y), &g));
		Handle.reset(g);
	}

	/* Regions (uint8, 255 = none) of the requested chunks of a width x height
	 * rendering buffer; the maps' pitches are in elements. */
	void operator()(const STPSample_t* biomemap, uint32_t biome_pitch, const STPHeightFixed_t* heightmap,
		uint32_t height_pitch, uint8_t* splatmap, uint32_t splat_pitch, uint32_t width, uint32_t height,
		const std::vector<stpgb_splat_chunk>& chunks, void* stream) {
		detail::check(stpgb_splatmap(Handle.get(), biomemap, biome_pitch, heightmap, height_pitch, splatmap, splat_pitch,
			width, height, chunks.data(), static_cast<uint32_t>(chunks.size()), nullptr, nullptr, stream));
	}

private:
	struct Deleter {
		void operator()(stpgb_splat_generator* g) const {
			stpgb_splat_generator_destroy(g);
		}
	};
	std::unique_ptr<stpgb_splat_generator, Deleter> Handle;
};

} // namespace STPDiversity

namespace detail {

inline std::vector<stpgb_layer> demo_chain() {
	std::vector<stpgb_layer> c(STPGB_MAX_LAYERS);
	uint32_t n = 0u;
	check(stpgb_layer_chain_demo(c.data(), static_cast<uint32_t>(c.size()), &n));
	c.resize(n);
	return c;
}

inline stpgb_layer_biomes demo_ids() {
	stpgb_layer_biomes ids {};
	stpgb_layer_biomes_demo(&ids);
	return ids;
}

} // namespace detail

namespace detail {

// Two-component results of STPChunk; they convert to any vector type built
// as V { x, y }, such as glm::ivec2 / glm::uvec2 / glm::dvec2.
template<class T>
struct vec2_of {
	T x, y;
	template<class V>
	operator V() const {
		return V { x, y };
	}
	bool operator==(const vec2_of& o) const {
		return x == o.x && y == o.y;
	}
	bool operator!=(const vec2_of& o) const {
		return !(*this == o);
	}
};

template<class T, class V>
void put2(T* out, const V& v) {
	out[0] = static_cast<T>(v.x);
	out[1] = static_cast<T>(v.y);
}

} // namespace detail

#ifdef GLM_VERSION
using STPVec2 = glm::vec2;
using STPUVec2 = glm::uvec2;
using STPDVec2 = glm::dvec2;
using STPDVec3 = glm::dvec3;
#else
using STPVec2 = detail::vec2_of<float>;
using STPUVec2 = detail::vec2_of<uint32_t>;
using STPDVec2 = detail::vec2_of<double>;
struct STPDVec3 {
	double x, y, z;
};
#endif

namespace STPEnvironment {

/* STPChunkSetting (SuperTerrain+/Environment/STPChunkSetting.h:15-45) with
 * validate() as STPEnvironment.cpp:17-41; the heightfield generator reads
 * MapSize and the two nearest-neighbour counts. */
struct STPChunkSetting {
	STPUVec2 ChunkSize {}, MapSize {};
	STPDVec3 ChunkOffset {};
	STPDVec2 ChunkScale {}, MapOffset {};
	STPUVec2 DiversityNearestNeighbour {}, ErosionNearestNeighbour {}, SplatNearestNeighbour {}, RenderDistance {};

	void validate() const {
		const auto positive = [](const STPUVec2& v) { return v.x > 0u && v.y > 0u; };
		const auto odd = [](const STPUVec2& v) { return (v.x & 1u) && (v.y & 1u); };
		const bool ok = positive(ChunkSize) && positive(MapSize) && ChunkScale.x > 0.0 && ChunkScale.y > 0.0
			&& positive(DiversityNearestNeighbour) && positive(ErosionNearestNeighbour) && positive(SplatNearestNeighbour)
			&& positive(RenderDistance) && odd(DiversityNearestNeighbour) && odd(ErosionNearestNeighbour)
			&& odd(SplatNearestNeighbour) && odd(RenderDistance);
		if (!ok) {
			throw STPException::STPInvalidEnvironment("STPChunkSetting validation failed");
		}
	}
};

} // namespace STPEnvironment

/* STPNearestNeighbourInformation (SuperTerrain+/World/Chunk/STPNearestNeighbourInformation.hpp:13-25) */
struct STPNearestNeighbourInformation {
	STPUVec2 MapSize, ChunkNearestNeighbour, TotalMapSize;
};

enum class STPNearestNeighbourTextureBufferMemoryMode : unsigned char {
	ReadOnly = 0x00u,
	WriteOnly = 0x01u,
	ReadWrite = 0x02u
};

/* STPNearestNeighbourTextureBuffer (SuperTerrain+/World/Chunk/STPNearestNeighbourTextureBuffer.h),
 * the buffers a diversity plugin receives.  The merged neighbourhood already
 * lives on the device: STPMergedBuffer(DeviceMemory) hands it out directly;
 * STPMergedBuffer(HostMemory) stages it in host memory (read from the
 * caller's chunk arrays or the device copy) and, for a writable buffer,
 * copies the host copy back to the device when it is destroyed, as the
 * reference's merged buffer unpacks on destruction.  DeviceMemInfo.second is
 * the call's stream (a cudaStream_t as void*); there is no memory pool. */
template<typename T, STPNearestNeighbourTextureBufferMemoryMode MM>
class STPNearestNeighbourTextureBuffer {
public:
	using TextureType = std::conditional_t<MM == STPNearestNeighbourTextureBufferMemoryMode::ReadOnly, const T, T>;
	typedef std::pair<void*, void*> STPDeviceMemoryOperator;

	enum class STPMemoryLocation : unsigned char {
		HostMemory = 0x00u,
		DeviceMemory = 0x01u
	};

	class STPMergedBuffer {
	public:
		using MutableT = std::remove_const_t<T>;

		const STPMemoryLocation Location;

		STPMergedBuffer(const STPNearestNeighbourTextureBuffer& main, const STPMemoryLocation location) :
			Location(location), Main(main) {
			if (location != STPMemoryLocation::HostMemory) {
				return;
			}
			const STPNearestNeighbourInformation& nn = Main.NeighbourInfo;
			Host.resize(static_cast<size_t>(nn.TotalMapSize.x) * nn.TotalMapSize.y);
			if constexpr (MM == STPNearestNeighbourTextureBufferMemoryMode::WriteOnly) {
				return;
			}
			if (Main.HostChunks) {
				stpgb_nn_info i = Main.info();
				detail::check(stpgb_nn_merge_host(reinterpret_cast<const void* const*>(Main.HostChunks), sizeof(T), &i,
					Host.data()));
			} else {
				detail::check(stpgb_copy(Host.data(), Main.Device, Host.size() * sizeof(T), Main.DeviceMemInfo.second, 1));
			}
		}
		STPMergedBuffer(const STPMergedBuffer&) = delete;
		STPMergedBuffer& operator=(const STPMergedBuffer&) = delete;
		~STPMergedBuffer() noexcept(false) {
			if constexpr (MM != STPNearestNeighbourTextureBufferMemoryMode::ReadOnly) {
				if (Location == STPMemoryLocation::HostMemory) {
					detail::check(stpgb_copy(const_cast<MutableT*>(Main.Device), Host.data(), Host.size() * sizeof(T),
						Main.DeviceMemInfo.second, 1));
				}
			}
		}

		MutableT* getHost() const noexcept {
			return Host.empty() ? nullptr : const_cast<MutableT*>(Host.data());
		}
		MutableT* getDevice() const noexcept {
			return const_cast<MutableT*>(Main.Device);
		}

	private:
		const STPNearestNeighbourTextureBuffer& Main;
		std::vector<MutableT> Host;
	};

	const STPNearestNeighbourInformation& NeighbourInfo;
	const STPDeviceMemoryOperator DeviceMemInfo;

	/* Made by the generator around its device buffers; `host_chunks` (may be
	 * null) are the caller's host arrays of the neighbourhood's chunks. */
	STPNearestNeighbourTextureBuffer(TextureType* device_merged, const T* const* host_chunks,
		const STPNearestNeighbourInformation& info, void* stream) :
		NeighbourInfo(info), DeviceMemInfo(nullptr, stream), Device(device_merged), HostChunks(host_chunks) {}
	STPNearestNeighbourTextureBuffer(const STPNearestNeighbourTextureBuffer&) = delete;
	STPNearestNeighbourTextureBuffer& operator=(const STPNearestNeighbourTextureBuffer&) = delete;

private:
	TextureType* const Device;
	const T* const* const HostChunks;

	stpgb_nn_info info() const {
		stpgb_nn_info i {};
		i.MapSize[0] = NeighbourInfo.MapSize.x;
		i.MapSize[1] = NeighbourInfo.MapSize.y;
		i.ChunkNearestNeighbour[0] = NeighbourInfo.ChunkNearestNeighbour.x;
		i.ChunkNearestNeighbour[1] = NeighbourInfo.ChunkNearestNeighbour.y;
		i.TotalMapSize[0] = NeighbourInfo.TotalMapSize.x;
		i.TotalMapSize[1] = NeighbourInfo.TotalMapSize.y;
		return i;
	}
};

typedef STPNearestNeighbourTextureBuffer<STPHeightFloat_t, STPNearestNeighbourTextureBufferMemoryMode::WriteOnly>
	STPNearestNeighbourHeightFloatWTextureBuffer;
typedef STPNearestNeighbourTextureBuffer<STPHeightFloat_t, STPNearestNeighbourTextureBufferMemoryMode::ReadWrite>
	STPNearestNeighbourHeightFloatRWTextureBuffer;
typedef STPNearestNeighbourTextureBuffer<STPSample_t, STPNearestNeighbourTextureBufferMemoryMode::ReadOnly>
	STPNearestNeighbourSampleRTextureBuffer;
typedef STPNearestNeighbourTextureBuffer<STPHeightFixed_t, STPNearestNeighbourTextureBufferMemoryMode::WriteOnly>
	STPNearestNeighbourHeightFixedWTextureBuffer;

namespace detail {

// The exception a diversity plugin threw, carried across the C boundary on
// the calling thread and rethrown by the generator's caller.
inline std::exception_ptr& plugin_exception() {
	thread_local std::exception_ptr e;
	return e;
}

inline STPNearestNeighbourInformation nn_of(const stpgb_nn_info& i) {
	STPNearestNeighbourInformation n;
	n.MapSize = STPUVec2 { i.MapSize[0], i.MapSize[1] };
	n.ChunkNearestNeighbour = STPUVec2 { i.ChunkNearestNeighbour[0], i.ChunkNearestNeighbour[1] };
	n.TotalMapSize = STPUVec2 { i.TotalMapSize[0], i.TotalMapSize[1] };
	return n;
}

inline void rethrow_plugin(int rc, bool environment = false) {
	if (rc != STPGB_OK && plugin_exception()) {
		std::exception_ptr e = plugin_exception();
		plugin_exception() = nullptr;
		std::rethrow_exception(e);
	}
	check(rc, environment);
}

} // namespace detail

/* STPDiversityGenerator (SuperTerrain+/World/Chunk/STPDiversityGenerator.hpp:14-39):
 * the multi-biome heightmap plugin of the heightfield generator.  operator()
 * writes one chunk's heightmap from its biome neighbourhood; an exception it
 * throws reaches the caller of STPHeightfieldGenerator::generate. */
class STPDiversityGenerator {
public:
	STPDiversityGenerator() = default;
	virtual ~STPDiversityGenerator() = default;

	virtual void operator()(const STPNearestNeighbourHeightFloatWTextureBuffer&,
		const STPNearestNeighbourSampleRTextureBuffer&, STPVec2) = 0;

	/* The plugin as an stpgb_diversity_generator for the C ABI. */
	stpgb_diversity_generator cPlugin() noexcept {
		return stpgb_diversity_generator { &STPDiversityGenerator::call, this };
	}

private:
	static int call(void* user, const stpgb_diversity_call* c) noexcept {
		try {
			const STPNearestNeighbourInformation hnn = detail::nn_of(c->heightmap_nn), bnn = detail::nn_of(c->biomemap_nn);
			const STPNearestNeighbourHeightFloatWTextureBuffer height(c->heightmap, nullptr, hnn, c->stream);
			const STPNearestNeighbourSampleRTextureBuffer biome(c->biomemap, c->biomemap_chunks_host, bnn, c->stream);
			(*static_cast<STPDiversityGenerator*>(user))(height, biome, STPVec2 { c->offset_x, c->offset_y });
			return STPGB_OK;
		} catch (...) {
			detail::plugin_exception() = std::current_exception();
			return STPGB_EINVAL;
		}
	}
};


/* STPHeightfieldGenerator (SuperTerrain+/World/Chunk/STPHeightfieldGenerator.h:35-45,121,145,159).
 * The reference's constructor takes an STPGeneratorSetup with a diversity
 * plugin; a second constructor folds the demo plugin in. */
class STPHeightfieldGenerator {
public:
	struct STPGeneratorSetup {
		const STPEnvironment::STPChunkSetting* ChunkSetting;
		const STPEnvironment::STPRainDropSetting* RainDropSetting;
		STPDiversityGenerator* DiversityGenerator;
	};

	/* STPHeightfieldGenerator(const STPGeneratorSetup&) (STPHeightfieldGenerator.cpp:115-150):
	 * validates both settings; the plugin must outlive the generator. */
	explicit STPHeightfieldGenerator(const STPGeneratorSetup& setup) {
		if (!setup.ChunkSetting || !setup.RainDropSetting || !setup.DiversityGenerator) {
			throw STPException::STPInvalidEnvironment("STPGeneratorSetup: null member");
		}
		setup.ChunkSetting->validate();
		setup.RainDropSetting->validate();
		stpgb_chunk_setting c {};
		detail::put2(c.MapSize, setup.ChunkSetting->MapSize);
		detail::put2(c.DiversityNearestNeighbour, setup.ChunkSetting->DiversityNearestNeighbour);
		detail::put2(c.ErosionNearestNeighbour, setup.ChunkSetting->ErosionNearestNeighbour);
		Plugin = setup.DiversityGenerator->cPlugin();
		const stpgb_generator_setup cs { &c, setup.RainDropSetting, &Plugin };
		stpgb_generator* g = nullptr;
		detail::check(stpgb_generator_create_setup(&cs, &g), true);
		Handle.reset(g);
	}

	/* The demo plugin folded in: its biome table and interpolation radius
	 * are constructor arguments. */
	template<class V>
	STPHeightfieldGenerator(const V& map_size, const V& diversity_nn, const V& erosion_nn,
		const STPEnvironment::STPRainDropSetting& raindrop, const STPEnvironment::STPSimplexNoiseSetting& simplex,
		const std::vector<stpgb_biome_property>& biome_table, unsigned int interpolation_radius) {
		stpgb_chunk_setting c {};
		c.MapSize[0] = static_cast<uint32_t>(map_size.x);
		c.MapSize[1] = static_cast<uint32_t>(map_size.y);
		c.DiversityNearestNeighbour[0] = static_cast<uint32_t>(diversity_nn.x);
		c.DiversityNearestNeighbour[1] = static_cast<uint32_t>(diversity_nn.y);
		c.ErosionNearestNeighbour[0] = static_cast<uint32_t>(erosion_nn.x);
		c.ErosionNearestNeighbour[1] = static_cast<uint32_t>(erosion_nn.y);
		stpgb_generator* g = nullptr;
		detail::check(stpgb_generator_create(&c, &raindrop, &simplex, biome_table.data(),
			static_cast<uint32_t>(biome_table.size()), interpolation_radius, &g), true);
		Handle.reset(g);
	}

	/* STPHeightfieldGenerator::generate (STPHeightfieldGenerator.cpp:158-169) */
	template<class V>
	void generate(STPHeightFloat_t* heightfield, const STPSample_t* const* biomemap, const V& offset) {
		detail::rethrow_plugin(stpgb_generator_generate(Handle.get(), heightfield, biomemap, static_cast<float>(offset.x),
			static_cast<float>(offset.y)));
	}

	/* STPHeightfieldGenerator::erode (STPHeightfieldGenerator.cpp:171-197) */
	void erode(STPHeightFloat_t* const* heightfield, STPHeightFixed_t* const* heightfield_fixed) {
		detail::check(stpgb_generator_erode(Handle.get(), heightfield, heightfield_fixed));
	}

private:
	struct Deleter {
		void operator()(stpgb_generator* g) const {
			stpgb_generator_destroy(g);
		}
	};
	stpgb_diversity_generator Plugin {};
	std::unique_ptr<stpgb_generator, Deleter> Handle;
};


/* The static coordinate functions of STPChunk
 * (SuperTerrain+/World/Chunk/STPChunk.h:110-157): chunk coordinates are in
 * world units.  Arguments the reference leaves undefined (zero sizes, int32
 * overflow, a non-finite position) throw STPNumericDomainError. */
struct STPChunk {
#ifdef GLM_VERSION
	// glm included before this header: the reference's own result types
	using ivec2 = glm::ivec2;
	using uvec2 = glm::uvec2;
	using dvec2 = glm::dvec2;
#else
	using ivec2 = detail::vec2_of<int32_t>;
	using uvec2 = detail::vec2_of<uint32_t>;
	using dvec2 = detail::vec2_of<double>;
#endif
	using STPChunkNeighbourOffset = std::vector<ivec2>;

	template<class P, class U, class D>
	static ivec2 calcWorldChunkCoordinate(const P& pointPos, const U& chunkSize, const D& scale) {
		uint32_t cs[2];
		double sc[2];
		detail::put2(cs, chunkSize);
		detail::put2(sc, scale);
		int32_t out[2];
		detail::check(stpgb_chunk_world_coordinate(static_cast<double>(pointPos.x), static_cast<double>(pointPos.z),
			cs, sc, out));
		return ivec2 { out[0], out[1] };
	}

	template<class U>
	static uvec2 calcLocalChunkCoordinate(unsigned int chunkID, const U& chunkRange) {
		uint32_t r[2], out[2];
		detail::put2(r, chunkRange);
		detail::check(stpgb_chunk_local_coordinate(chunkID, r, out));
		return uvec2 { out[0], out[1] };
	}

	template<class I, class U, class N>
	static ivec2 calcLocalChunkOrigin(const I& centreChunkCoord, const U& chunkSize, const N& neighbourSize) {
		int32_t c[2], out[2];
		uint32_t cs[2], ns[2];
		detail::put2(c, centreChunkCoord);
		detail::put2(cs, chunkSize);
		detail::put2(ns, neighbourSize);
		detail::check(stpgb_chunk_local_origin(c, cs, ns, out));
		return ivec2 { out[0], out[1] };
	}

	template<class I, class U, class M, class D>
	static dvec2 calcChunkMapOffset(const I& chunkCoord, const U& chunkSize, const M& mapSize, const D& mapOffset) {
		int32_t c[2];
		uint32_t cs[2], ms[2];
		double mo[2], out[2];
		detail::put2(c, chunkCoord);
		detail::put2(cs, chunkSize);
		detail::put2(ms, mapSize);
		detail::put2(mo, mapOffset);
		detail::check(stpgb_chunk_map_offset(c, cs, ms, mo, out));
		return dvec2 { out[0], out[1] };
	}

	template<class I, class U, class O>
	static ivec2 offsetChunk(const I& chunkCoord, const U& chunkSize, const O& offset) {
		int32_t c[2], o[2], out[2];
		uint32_t cs[2];
		detail::put2(c, chunkCoord);
		detail::put2(cs, chunkSize);
		detail::put2(o, offset);
		detail::check(stpgb_chunk_offset(c, cs, o, out));
		return ivec2 { out[0], out[1] };
	}

	template<class U, class R>
	static STPChunkNeighbourOffset calcChunkNeighbourOffset(const U& chunkSize, const R& regionSize) {
		uint32_t cs[2], rs[2], n = 0u;
		detail::put2(cs, chunkSize);
		detail::put2(rs, regionSize);
		std::vector<int32_t> xy(2u * static_cast<size_t>(rs[0]) * rs[1]);
		detail::check(stpgb_chunk_neighbour_offset(cs, rs, xy.data(), static_cast<uint32_t>(xy.size() / 2u), &n));
		STPChunkNeighbourOffset out(n);
		for (uint32_t i = 0u; i < n; i++) {
			out[i] = ivec2 { xy[2u * i], xy[2u * i + 1u] };
		}
		return out;
	}
};

} // namespace SuperTerrainPlus

namespace STPDemo {

/* STPLayerChainBuilder (SuperDemo+/World/Layers/STPAllLayers.h): the demo's
 * 14-layer production line (STPAllLayers.cpp:59-105) with the demo's biome
 * IDs, or other IDs for the same chain. */
class STPLayerChainBuilder : public SuperTerrainPlus::STPDiversity::STPBiomeFactory {
public:
	template<class V>
	STPLayerChainBuilder(const V& dimension, SuperTerrainPlus::STPSeed_t global_seed) :
		STPBiomeFactory(dimension, global_seed, SuperTerrainPlus::detail::demo_chain(),
			SuperTerrainPlus::detail::demo_ids()) {}
	template<class V>
	STPLayerChainBuilder(const V& dimension, SuperTerrainPlus::STPSeed_t global_seed, const stpgb_layer_biomes& ids) :
		STPBiomeFactory(dimension, global_seed, SuperTerrainPlus::detail::demo_chain(), ids) {}
};

/* The demo's multi-biome plugin STPBiomefieldGenerator
 * (SuperDemo+/World/Biomes/STPBiomefieldGenerator.h:26-98): the single
 * histogram filter and the multi-biome fractal simplex heightmap, on the
 * device.  The biome table and interpolation radius are constructor
 * arguments (the demo reads them from its ini files). */
class STPBiomefieldGenerator : public SuperTerrainPlus::STPDiversityGenerator {
public:
	STPBiomefieldGenerator(const SuperTerrainPlus::STPEnvironment::STPSimplexNoiseSetting& simplex,
		const std::vector<stpgb_biome_property>& biome_table, unsigned int interpolation_radius) {
		stpgb_biomefield* f = nullptr;
		SuperTerrainPlus::detail::check(stpgb_biomefield_create(&simplex, biome_table.data(), static_cast<uint32_t>(biome_table.size()),
			interpolation_radius, &f), true);
		Handle.reset(f);
	}

	void operator()(const SuperTerrainPlus::STPNearestNeighbourHeightFloatWTextureBuffer& heightmap_buffer,
		const SuperTerrainPlus::STPNearestNeighbourSampleRTextureBuffer& biomemap_buffer, const SuperTerrainPlus::STPVec2 offset) override {
		const SuperTerrainPlus::STPNearestNeighbourHeightFloatWTextureBuffer::STPMergedBuffer height(heightmap_buffer,
			SuperTerrainPlus::STPNearestNeighbourHeightFloatWTextureBuffer::STPMemoryLocation::DeviceMemory);
		const SuperTerrainPlus::STPNearestNeighbourSampleRTextureBuffer::STPMergedBuffer biome(biomemap_buffer,
			SuperTerrainPlus::STPNearestNeighbourSampleRTextureBuffer::STPMemoryLocation::DeviceMemory);
		stpgb_diversity_call c {};
		c.heightmap = height.getDevice();
		c.biomemap = biome.getDevice();
		c.heightmap_nn = SuperTerrainPlus::detail::nn(heightmap_buffer.NeighbourInfo.MapSize, heightmap_buffer.NeighbourInfo.ChunkNearestNeighbour);
		c.biomemap_nn = SuperTerrainPlus::detail::nn(biomemap_buffer.NeighbourInfo.MapSize, biomemap_buffer.NeighbourInfo.ChunkNearestNeighbour);
		c.offset_x = static_cast<float>(offset.x);
		c.offset_y = static_cast<float>(offset.y);
		c.stream = heightmap_buffer.DeviceMemInfo.second;
		SuperTerrainPlus::detail::check(stpgb_biomefield_generate(Handle.get(), &c));
	}

private:
	struct Deleter {
		void operator()(stpgb_biomefield* f) const {
			stpgb_biomefield_destroy(f);
		}
	};
	std::unique_ptr<stpgb_biomefield, Deleter> Handle;
};

} // namespace STPDemo

#endif /* STPGB_HPP_ */
