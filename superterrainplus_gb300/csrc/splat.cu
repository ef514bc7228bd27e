// Texture splatmap: the texture region of every rendered pixel from its
// biome, altitude and slope.
//
// Per pixel (SuperDemo+/Script/STPSplatmapGenerator.cu:56-128): four taps of
// the fixed-point heightmap 2.5 pixels above, left, right and below, scaled by
// HeightFactor, give a gradient (top - bottom, GradientBias, left - right) and
// the slope factor 1 - GradientBias / |gradient|; three octaves of simplex
// noise (persistence 0.7, lacunarity 1.88, scale 91.5, x 0.15) are added to
// the pixel's height; the biome's splat rules then pick a region: the first
// gradient rule whose slope and altitude ranges hold, else the first altitude
// rule whose upper bound reaches the altitude
// (SuperTerrain+/SuperAlgorithm+/Device/Private/STPTextureSplatRuleWrapper.cu:55-126).
//
// The reference reads the heightmap through a texture with linear filtering,
// normalised-float reads, clamped addressing and unnormalised coordinates,
// and the biomemap through a point-filtered one
// (SuperTerrain+/Private/World/STPWorldPipeline.cpp:682-696); here the same
// two samplers are bound to the caller's pitched device buffers, so the
// texture units do the same bilinear filtering.  One thread per pixel, 16 x 16
// blocks for texture-cache locality, one grid layer per requested chunk, the
// permutation and reduced gradient tables of the noise in shared memory.
#include "simplex.cuh"

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

namespace stpgb {

namespace {

constexpr uint32_t kSplatTile = 16u;
constexpr uint32_t kMaxSplatChunks = 64u;
constexpr uint32_t kNoRegion = 0xFFFFFFFFu; // STPTextureSplatRuleWrapper::NoRegion

// SuperDemo+/Script/STPSplatmapGenerator.cu:2-20
constexpr float kGradientBias = 5.5f;
constexpr float kKernelRadius = 2.5f;
constexpr float kNoiseScale = 91.5f;
constexpr float kNoiseContribution = 0.15f;
constexpr float kHeightFactor = 875.5f;
constexpr float kPersistence = 0.7f;
constexpr float kLacunarity = 1.88f;
constexpr uint32_t kNoiseOctaves = 3u;

struct SplatRegistry {
	uint32_t AltitudeEntry, AltitudeSize, GradientEntry, GradientSize;
};
struct AltitudeNode {
	uint32_t RegionIndex;
	float UpperBound;
};
struct GradientNode {
	uint32_t RegionIndex;
	float minGradient, maxGradient, LowerBound, UpperBound;
};

// STPSplatRuleDatabase: device arrays
struct SplatRules {
	const uint16_t* dict;
	uint32_t dict_count;
	const SplatRegistry* reg;
	const AltitudeNode* alt;
	const GradientNode* gra;
};

struct SplatLaunch {
	SplatRules rules;
	stpgb_permutation perm;
	uint8_t* out;
	float* slope;
	float* altitude;
	uint32_t out_pitch;
	uint32_t map_x, map_y;
	float half_x, half_y;
	stpgb_splat_chunk chunk[kMaxSplatChunks];
};

// STPTextureSplatRuleWrapper::findSplatRegistry: lower bound of the sample in
// the sorted dictionary.  Like the reference, a sample missing from the
// dictionary takes the registry of the next larger one, if any.
__device__ __forceinline__ const SplatRegistry* find_registry(const SplatRules& R, const uint16_t sample) {
	uint32_t first = 0u, count = R.dict_count;
	while (count > 0u) {
		const uint32_t step = count / 2u, it = first + step;
		if (R.dict[it] < sample) {
			first = it + 1u;
			count -= step + 1u;
		} else {
			count = step;
		}
	}
	return first == R.dict_count ? nullptr : R.reg + first;
}

// STPTextureSplatRuleWrapper::gradientRegion: first rule whose ranges hold
__device__ __forceinline__ uint32_t gradient_region(const SplatRules& R, const SplatRegistry* reg, const float gra,
	const float alt) {
	if (!reg) {
		return kNoRegion;
	}
	const uint32_t end = reg->GradientEntry + reg->GradientSize;
	for (uint32_t i = reg->GradientEntry; i < end; i++) {
		const GradientNode n = R.gra[i];
		if (gra >= n.minGradient && gra <= n.maxGradient && alt >= n.LowerBound && alt <= n.UpperBound) {
			return n.RegionIndex;
		}
	}
	return kNoRegion;
}

// STPTextureSplatRuleWrapper::altitudeRegion: lower bound on the upper bounds
__device__ __forceinline__ uint32_t altitude_region(const SplatRules& R, const SplatRegistry* reg, const float alt) {
	if (!reg) {
		return kNoRegion;
	}
	uint32_t first = reg->AltitudeEntry, count = reg->AltitudeSize;
	const uint32_t end = first + count;
	while (count > 0u) {
		const uint32_t step = count / 2u, it = first + step;
		if (R.alt[it].UpperBound < alt) {
			first = it + 1u;
			count -= step + 1u;
		} else {
			count = step;
		}
	}
	return first == end ? kNoRegion : R.alt[first].RegionIndex;
}

__global__ void __launch_bounds__(kSplatTile * kSplatTile) splat_kernel(const cudaTextureObject_t biome_tex,
	const cudaTextureObject_t height_tex, const SplatLaunch L) {
	__shared__ uint8_t sperm[512];
	__shared__ float2 gtab[512];
	simplex::load_tables(L.perm, sperm, gtab);
	__syncthreads();
	const uint32_t x = blockIdx.x * kSplatTile + threadIdx.x, y = blockIdx.y * kSplatTile + threadIdx.y;
	if (x >= L.map_x || y >= L.map_y) {
		return;
	}
	const stpgb_splat_chunk& C = L.chunk[blockIdx.z];
	const uint32_t sx = x + L.map_x * C.LocalChunkCoordinateX, sy = y + L.map_y * C.LocalChunkCoordinateY;
	const float fx = static_cast<float>(sx), fy = static_cast<float>(sy);
	// taps {0,-1} top, {-1,0} left, {1,0} right, {0,1} bottom, KernelRadius apart
	const float top = tex2D<float>(height_tex, fx, fy - kKernelRadius) * kHeightFactor;
	const float left = tex2D<float>(height_tex, fx - kKernelRadius, fy) * kHeightFactor;
	const float right = tex2D<float>(height_tex, fx + kKernelRadius, fy) * kHeightFactor;
	const float bottom = tex2D<float>(height_tex, fx, fy + kKernelRadius) * kHeightFactor;
	const float gradient[3] = { top - bottom, kGradientBias, left - right };
	const float slope = 1.0f - (gradient[1] * rnormf(3, gradient));
	const float noise = simplex::fractal(sperm, gtab, ((1.0f * x - L.half_x) + C.ChunkMapOffsetX) / kNoiseScale,
		((1.0f * y - L.half_y) + C.ChunkMapOffsetY) / kNoiseScale, kNoiseOctaves, kPersistence, kLacunarity)
		* kNoiseContribution;
	const uint16_t biome = tex2D<unsigned short>(biome_tex, fx, fy);
	const float alt = __saturatef(tex2D<float>(height_tex, fx, fy) + noise);
	const SplatRegistry* const reg = find_registry(L.rules, biome);
	uint32_t region = gradient_region(L.rules, reg, slope, alt);
	if (region == kNoRegion) {
		region = altitude_region(L.rules, reg, alt);
	}
	const size_t o = static_cast<size_t>(sy) * L.out_pitch + sx;
	L.out[o] = static_cast<uint8_t>(region);
	if (L.slope) {
		L.slope[o] = slope;
	}
	if (L.altitude) {
		L.altitude[o] = alt;
	}
}

} // namespace

} // namespace stpgb

using namespace stpgb;

struct stpgb_splat_generator {
	uint32_t map_x = 0u, map_y = 0u;
	unsigned char* mem = nullptr; // rules and permutation tables
	SplatRules rules {};
	stpgb_permutation perm {};
	std::mutex mu;
	// texture objects per bound buffer: (address, width, height, pitch, linear)
	std::map<std::tuple<const void*, uint32_t, uint32_t, uint32_t, bool>, cudaTextureObject_t> textures;

	int texture(const uint16_t* p, const uint32_t w, const uint32_t h, const uint32_t pitch, const bool linear,
		cudaTextureObject_t* out) {
		const auto key = std::make_tuple(static_cast<const void*>(p), w, h, pitch, linear);
		std::lock_guard<std::mutex> lock(mu);
		const auto it = textures.find(key);
		if (it != textures.end()) {
			*out = it->second;
			return STPGB_OK;
		}
		cudaResourceDesc rd {};
		rd.resType = cudaResourceTypePitch2D;
		rd.res.pitch2D.devPtr = const_cast<uint16_t*>(p);
		rd.res.pitch2D.desc = cudaCreateChannelDesc<unsigned short>();
		rd.res.pitch2D.width = w;
		rd.res.pitch2D.height = h;
		rd.res.pitch2D.pitchInBytes = static_cast<size_t>(pitch) * sizeof(uint16_t);
		cudaTextureDesc td {};
		td.addressMode[0] = cudaAddressModeClamp;
		td.addressMode[1] = cudaAddressModeClamp;
		td.addressMode[2] = cudaAddressModeClamp;
		td.normalizedCoords = 0;
		td.filterMode = linear ? cudaFilterModeLinear : cudaFilterModePoint;
		td.readMode = linear ? cudaReadModeNormalizedFloat : cudaReadModeElementType;
		cudaTextureObject_t t = 0;
		STPGB_CUDA_TRY(cudaCreateTextureObject(&t, &rd, &td, nullptr));
		textures.emplace(key, t);
		*out = t;
		return STPGB_OK;
	}

	~stpgb_splat_generator() {
		if (!textures.empty()) {
			cudaDeviceSynchronize();
			for (auto& kv : textures) {
				cudaDestroyTextureObject(kv.second);
			}
		}
		if (mem) {
			cudaFree(mem);
		}
	}
};

extern "C" {

int stpgb_splat_rules_demo(stpgb_altitude_rule* altitude, const uint32_t altitude_capacity, uint32_t* altitude_count,
	stpgb_gradient_rule* gradient, const uint32_t gradient_capacity, uint32_t* gradient_count) {
	// SuperDemo+/Script/STPBiomeSplatRule.tdl: textures [redrock, grass, mossrock, sand, soil, darkrock]
	enum : uint32_t { Redrock, Grass, Mossrock, Sand, Soil, Darkrock };
	static const stpgb_altitude_rule alt[] = {
		{ 0u, 1.0f, Soil },
		{ 1u, 0.5f, Sand },
		{ 1u, 0.72f, Mossrock },
		{ 1u, 1.0f, Grass },
	};
	static const stpgb_gradient_rule gra[] = {
		{ 0u, 0.0f, 0.2f, 0.0f, 0.27f, Sand },
		{ 1u, 0.4f, 0.65f, 0.58f, 0.8f, Darkrock },
		{ 1u, 0.625f, 1.0f, 0.65f, 1.0f, Redrock },
	};
	constexpr uint32_t na = sizeof(alt) / sizeof(alt[0]), ng = sizeof(gra) / sizeof(gra[0]);
	if (!altitude_count || !gradient_count) {
		return inval("stpgb_splat_rules_demo: null count");
	}
	*altitude_count = na;
	*gradient_count = ng;
	if (!altitude || !gradient || altitude_capacity < na || gradient_capacity < ng) {
		return inval("stpgb_splat_rules_demo: capacity below 4 altitude / 3 gradient rules");
	}
	std::copy(alt, alt + na, altitude);
	std::copy(gra, gra + ng, gradient);
	return STPGB_OK;
}

int stpgb_splat_generator_create(const stpgb_altitude_rule* altitude, const uint32_t altitude_count,
	const stpgb_gradient_rule* gradient, const uint32_t gradient_count, const stpgb_simplex_setting* simplex,
	const uint32_t map_x, const uint32_t map_y, stpgb_splat_generator** out) {
	if (!out || !simplex || (altitude_count && !altitude) || (gradient_count && !gradient)) {
		return inval("stpgb_splat_generator_create: null argument");
	}
	if (map_x == 0u || map_y == 0u) {
		return inval("stpgb_splat_generator_create: MapSize must be positive");
	}
	for (uint32_t i = 0u; i < gradient_count; i++) {
		if (!(gradient[i].minGradient <= gradient[i].maxGradient) || !(gradient[i].LowerBound <= gradient[i].UpperBound)) {
			return inval("stpgb_splat_generator_create: a gradient rule has an empty range");
		}
	}
	STPGB_TRY(stpgb_simplex_setting_validate(simplex));
	// the texture database's order (STPTextureDatabase.cpp:357-411): altitude
	// rules by sample then upper bound, gradient rules by sample, samples ascending
	std::vector<stpgb_altitude_rule> alt(altitude, altitude + altitude_count);
	std::vector<stpgb_gradient_rule> gra(gradient, gradient + gradient_count);
	std::stable_sort(alt.begin(), alt.end(), [](const stpgb_altitude_rule& a, const stpgb_altitude_rule& b) {
		return a.Sample != b.Sample ? a.Sample < b.Sample : a.UpperBound < b.UpperBound;
	});
	std::stable_sort(gra.begin(), gra.end(), [](const stpgb_gradient_rule& a, const stpgb_gradient_rule& b) {
		return a.Sample < b.Sample;
	});
	std::vector<uint16_t> dict;
	for (const auto& a : alt) {
		dict.push_back(a.Sample);
	}
	for (const auto& g : gra) {
		dict.push_back(g.Sample);
	}
	std::sort(dict.begin(), dict.end());
	dict.erase(std::unique(dict.begin(), dict.end()), dict.end());
	std::vector<SplatRegistry> reg(dict.size());
	std::vector<AltitudeNode> an;
	std::vector<GradientNode> gn;
	for (size_t d = 0u; d < dict.size(); d++) {
		reg[d].AltitudeEntry = static_cast<uint32_t>(an.size());
		for (const auto& a : alt) {
			if (a.Sample == dict[d]) {
				an.push_back(AltitudeNode { a.RegionIndex, a.UpperBound });
			}
		}
		reg[d].AltitudeSize = static_cast<uint32_t>(an.size()) - reg[d].AltitudeEntry;
		reg[d].GradientEntry = static_cast<uint32_t>(gn.size());
		for (const auto& g : gra) {
			if (g.Sample == dict[d]) {
				gn.push_back(GradientNode { g.RegionIndex, g.minGradient, g.maxGradient, g.LowerBound, g.UpperBound });
			}
		}
		reg[d].GradientSize = static_cast<uint32_t>(gn.size()) - reg[d].GradientEntry;
	}
	std::vector<uint8_t> perm(512u);
	std::vector<float> grad(2u * simplex->Distribution);
	STPGB_TRY(stpgb_permutation_generate(simplex, perm.data(), grad.data(), static_cast<uint32_t>(grad.size())));

	auto al = [](size_t v) { return (v + 255u) & ~size_t(255u); };
	const size_t o_dict = 0u, o_reg = al(o_dict + dict.size() * sizeof(uint16_t) + 1u),
		o_alt = al(o_reg + reg.size() * sizeof(SplatRegistry) + 1u), o_gra = al(o_alt + an.size() * sizeof(AltitudeNode) + 1u),
		o_perm = al(o_gra + gn.size() * sizeof(GradientNode) + 1u), o_grad = al(o_perm + 512u),
		total = o_grad + grad.size() * sizeof(float);
	std::vector<unsigned char> host(total, 0u);
	std::copy(reinterpret_cast<const unsigned char*>(dict.data()),
		reinterpret_cast<const unsigned char*>(dict.data() + dict.size()), host.begin() + o_dict);
	std::copy(reinterpret_cast<const unsigned char*>(reg.data()),
		reinterpret_cast<const unsigned char*>(reg.data() + reg.size()), host.begin() + o_reg);
	std::copy(reinterpret_cast<const unsigned char*>(an.data()),
		reinterpret_cast<const unsigned char*>(an.data() + an.size()), host.begin() + o_alt);
	std::copy(reinterpret_cast<const unsigned char*>(gn.data()),
		reinterpret_cast<const unsigned char*>(gn.data() + gn.size()), host.begin() + o_gra);
	std::copy(perm.begin(), perm.end(), host.begin() + o_perm);
	std::copy(reinterpret_cast<const unsigned char*>(grad.data()),
		reinterpret_cast<const unsigned char*>(grad.data() + grad.size()), host.begin() + o_grad);

	auto* g = new stpgb_splat_generator();
	g->map_x = map_x;
	g->map_y = map_y;
	cudaError_t e = cudaMalloc(&g->mem, total);
	if (e == cudaSuccess) {
		e = cudaMemcpy(g->mem, host.data(), total, cudaMemcpyHostToDevice);
	}
	if (e != cudaSuccess) {
		delete g;
		return cuda_fail(e, "stpgb_splat_generator_create");
	}
	g->rules.dict = reinterpret_cast<const uint16_t*>(g->mem + o_dict);
	g->rules.dict_count = static_cast<uint32_t>(dict.size());
	g->rules.reg = reinterpret_cast<const SplatRegistry*>(g->mem + o_reg);
	g->rules.alt = reinterpret_cast<const AltitudeNode*>(g->mem + o_alt);
	g->rules.gra = reinterpret_cast<const GradientNode*>(g->mem + o_gra);
	g->perm.Permutation = g->mem + o_perm;
	g->perm.Gradient2D = reinterpret_cast<const float*>(g->mem + o_grad);
	g->perm.Gradient2DSize = simplex->Distribution;
	*out = g;
	return STPGB_OK;
}

int stpgb_splat_generator_destroy(stpgb_splat_generator* generator) {
	delete generator;
	return STPGB_OK;
}

int stpgb_splatmap(stpgb_splat_generator* g, const uint16_t* biomemap, const uint32_t biome_pitch,
	const uint16_t* heightmap, const uint32_t height_pitch, uint8_t* splatmap, const uint32_t splat_pitch,
	const uint32_t width, const uint32_t height, const stpgb_splat_chunk* chunks, const uint32_t count, float* slope,
	float* altitude, void* stream) {
	if (!g || !biomemap || !heightmap || !splatmap || (count && !chunks)) {
		return inval("stpgb_splatmap: null argument");
	}
	if (width == 0u || height == 0u || biome_pitch < width || height_pitch < width || splat_pitch < width) {
		return inval("stpgb_splatmap: empty buffer or pitch below width");
	}
	int dev = 0, base_align = 0, pitch_align = 0;
	STPGB_CUDA_TRY(cudaGetDevice(&dev));
	STPGB_CUDA_TRY(cudaDeviceGetAttribute(&base_align, cudaDevAttrTextureAlignment, dev));
	STPGB_CUDA_TRY(cudaDeviceGetAttribute(&pitch_align, cudaDevAttrTexturePitchAlignment, dev));
	const size_t bp = static_cast<size_t>(biome_pitch) * sizeof(uint16_t),
		hp = static_cast<size_t>(height_pitch) * sizeof(uint16_t);
	if (reinterpret_cast<uintptr_t>(biomemap) % base_align != 0u || reinterpret_cast<uintptr_t>(heightmap) % base_align != 0u
		|| bp % pitch_align != 0u || hp % pitch_align != 0u) {
		return inval("stpgb_splatmap: biomemap and heightmap must start on a " + std::to_string(base_align)
			+ "-byte boundary with a row pitch that is a multiple of " + std::to_string(pitch_align) + " bytes");
	}
	for (uint32_t c = 0u; c < count; c++) {
		const uint64_t x1 = (static_cast<uint64_t>(chunks[c].LocalChunkCoordinateX) + 1u) * g->map_x;
		const uint64_t y1 = (static_cast<uint64_t>(chunks[c].LocalChunkCoordinateY) + 1u) * g->map_y;
		if (x1 > width || y1 > height) {
			return inval("stpgb_splatmap: chunk " + std::to_string(c) + " lies outside the rendering buffer");
		}
	}
	cudaTextureObject_t bt = 0, ht = 0;
	STPGB_TRY(g->texture(biomemap, width, height, biome_pitch, false, &bt));
	STPGB_TRY(g->texture(heightmap, width, height, height_pitch, true, &ht));
	SplatLaunch L {};
	L.rules = g->rules;
	L.perm = g->perm;
	L.out = splatmap;
	L.slope = slope;
	L.altitude = altitude;
	L.out_pitch = splat_pitch;
	L.map_x = g->map_x;
	L.map_y = g->map_y;
	// HalfDimension = MapSize / 2 (SuperDemo+/World/Biomes/STPCommonCompiler.cpp:236)
	L.half_x = static_cast<float>(g->map_x) / 2.0f;
	L.half_y = static_cast<float>(g->map_y) / 2.0f;
	const cudaStream_t s = as_stream(stream);
	for (uint32_t c0 = 0u; c0 < count; c0 += kMaxSplatChunks) {
		const uint32_t n = std::min(kMaxSplatChunks, count - c0);
		std::copy(chunks + c0, chunks + c0 + n, L.chunk);
		const dim3 grid((g->map_x + kSplatTile - 1u) / kSplatTile, (g->map_y + kSplatTile - 1u) / kSplatTile, n);
		splat_kernel<<<grid, dim3(kSplatTile, kSplatTile), 0, s>>>(bt, ht, L);
		STPGB_CUDA_TRY(cudaGetLastError());
	}
	return STPGB_OK;
}

} // extern "C"
