// The reference's own test scenarios for the heightfield path, written
// against the C++ façade (include/stpgb.hpp) the way a SuperTerrain+ caller
// would: SuperTest+/SuperAlgorithm+/STPTestHistogram.cpp (known-answer
// histograms and error cases), STPTestPermutation.cpp (gradients,
// repetition, seeds, invalid setting), STPTest2DChunk.cpp (chunk coordinate
// known answers), a generate/erode round trip, and the
// demo's biome layer chain against maps of the compiled reference.
// `--cpu` runs the parts that fail before any device work.
#include "stpgb.hpp"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <vector>

using namespace SuperTerrainPlus;
using STPAlgorithm::STPSingleHistogramFilter;
using FiltBuf = STPSingleHistogramFilter::STPFilterBuffer;

namespace {

int failures = 0;

#define CHECK(cond)                                                            \
	do {                                                                       \
		if (!(cond)) {                                                         \
			std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond);      \
			failures++;                                                        \
		}                                                                      \
	} while (0)

template<class E, class F>
bool throws(F f) {
	try {
		f();
	} catch (const E&) {
		return true;
	} catch (...) {
		return false;
	}
	return false;
}

struct uvec2 {
	unsigned int x, y;
};
struct vec2 {
	float x, y;
};
struct NNInfo {
	uvec2 MapSize, ChunkNearestNeighbour, TotalMapSize;
};

// STPTestHistogram.cpp:44-57
const STPSample_t Texture[] = {
	2, 0, 2, 0, 1, 1, 0, 3, 3, 2, 1, 2,
	0, 1, 2, 1, 1, 1, 3, 2, 2, 0, 0, 1,
	0, 1, 0, 2, 1, 3, 1, 1, 1, 2, 1, 0,
	3, 3, 0, 1, 1, 2, 2, 2, 2, 0, 0, 3,
	3, 2, 3, 3, 0, 3, 2, 2, 1, 0, 0, 3,
	2, 0, 0, 1, 2, 0, 2, 2, 0, 2, 0, 3,
	1, 2, 3, 0, 3, 2, 1, 2, 2, 3, 0, 2,
	1, 1, 0, 3, 0, 2, 1, 0, 3, 2, 2, 1,
	2, 2, 0, 1, 0, 2, 0, 0, 0, 0, 1, 1,
	0, 1, 3, 3, 0, 3, 3, 3, 1, 0, 1, 1,
	3, 1, 3, 0, 2, 1, 1, 0, 2, 2, 2, 0,
	2, 0, 1, 1, 2, 3, 1, 2, 3, 2, 0, 1
};
const NNInfo Data = { { 4u, 4u }, { 3u, 3u }, { 12u, 12u } };

void histogram_errors() {
	STPSingleHistogramFilter filter;
	FiltBuf serial(FiltBuf::STPExecutionType::Serial), parallel(FiltBuf::STPExecutionType::Parallel);
	CHECK(throws<STPException::STPNumericDomainError>([&] { filter(Texture, Data, serial, 0u); }));
	CHECK(throws<STPException::STPNumericDomainError>([&] { filter(Texture, Data, parallel, 128u); }));
	CHECK(throws<STPException::STPNumericDomainError>([&] { filter(Texture, Data, serial, 3u); }));
}

void histogram_known_answer() {
	STPSingleHistogramFilter filter;
	for (auto type : { FiltBuf::STPExecutionType::Serial, FiltBuf::STPExecutionType::Parallel }) {
		FiltBuf buf(type);
		for (int again = 0; again < 2; again++) {
			const STPAlgorithm::STPSingleHistogram h = filter(Texture, Data, buf, 2u);
			// STPTestHistogram.cpp:77-105
			const unsigned int trial[] = { 0u, 8u, 15u };
			const std::pair<STPSample_t, float> expected[] = { { 0, .24f }, { 3, .24f }, { 2, .28f }, { 1, .24f },
				{ 0, .36f }, { 3, .24f }, { 1, .16f }, { 2, .24f }, { 0, .32f }, { 3, .2f }, { 1, .12f }, { 2, .36f } };
			for (int t = 0; t < 3; t++) {
				const unsigned int o = trial[t];
				int counter = 0;
				for (unsigned int i = h.HistogramStartOffset[o]; i < h.HistogramStartOffset[o + 1u]; i++, counter++) {
					const auto [item, weight] = expected[counter + t * 4];
					CHECK(h.Bin[i].Item == item);
					CHECK(std::fabs(h.Bin[i].Weight - weight) <= std::numeric_limits<float>::epsilon() * 5.0f * weight);
				}
				CHECK(counter == 4);
			}
			CHECK(buf.type() == type);
			const auto [bins, offsets] = buf.size();
			CHECK(offsets == 17u);
			CHECK(bins == h.HistogramStartOffset[offsets - 1u]);
		}
	}
}

void permutation() {
	STPEnvironment::STPSimplexNoiseSetting invalid {};
	invalid.Distribution = 0u;
	CHECK(throws<STPException::STPInvalidEnvironment>([&] { STPAlgorithm::STPPermutationGenerator::generate(invalid); }));
	// STPTestPermutation.cpp:37-41
	STPEnvironment::STPSimplexNoiseSetting s {};
	s.Seed = 6666u;
	s.Distribution = 10u;
	s.Offset = 6.5 * 3.14159265358979323846 / 180.0;
	const auto t = STPAlgorithm::STPPermutationGenerator::generate(s);
	CHECK(t.Permutation.Gradient2DSize == 10u);
	const double degs[] = { 6.5, 114.5, 258.5 };
	const int idx[] = { 0, 6, 14 };
	for (int k = 0; k < 3; k++) {
		const double a = degs[k] * 3.14159265358979323846 / 180.0;
		CHECK(std::fabs(t.HostGradient2D[idx[k]] - std::cos(a)) <= 10.0 * std::numeric_limits<float>::epsilon() * std::fabs(std::cos(a)));
		CHECK(std::fabs(t.HostGradient2D[idx[k] + 1] - std::sin(a)) <= 10.0 * std::numeric_limits<float>::epsilon() * std::fabs(std::sin(a)));
	}
	for (int i = 0; i < 256; i++) {
		CHECK(t.HostPermutation[i] == t.HostPermutation[i + 256]);
	}
	const auto same = STPAlgorithm::STPPermutationGenerator::generate(s);
	CHECK(same.HostPermutation == t.HostPermutation);
	s.Seed = 183457092u;
	const auto other = STPAlgorithm::STPPermutationGenerator::generate(s);
	CHECK(other.HostPermutation != t.HostPermutation);
}

STPEnvironment::STPRainDropSetting raindrop(unsigned int count) {
	STPEnvironment::STPRainDropSetting r {};
	r.Seed = 42u;
	r.RainDropCount = count;
	r.Inertia = 0.05f;
	r.SedimentCapacityFactor = 4.0f;
	r.minSedimentCapacity = 0.01f;
	r.initWaterVolume = 1.0f;
	r.minWaterVolume = stpgb_lifetime_min_water_volume(1.0f, 0.01f, 30u);
	r.Friction = 0.1f;
	r.initSpeed = 1.0f;
	r.ErodeSpeed = 0.3f;
	r.DepositSpeed = 0.3f;
	r.EvaporateSpeed = 0.01f;
	r.Gravity = 4.0f;
	r.ErosionBrushRadius = 3u;
	return r;
}

void generator_errors() {
	STPEnvironment::STPSimplexNoiseSetting s {};
	s.Seed = 1u;
	s.Distribution = 8u;
	s.Offset = 0.2;
	std::vector<stpgb_biome_property> table(2, stpgb_biome_property { 128.0f, 4u, 0.5f, 2.0f, 0.0f, 1.0f });
	auto bad = raindrop(100u);
	bad.Inertia = 2.0f;
	CHECK(throws<STPException::STPInvalidEnvironment>([&] {
		STPHeightfieldGenerator g(uvec2 { 32u, 32u }, uvec2 { 3u, 3u }, uvec2 { 3u, 3u }, bad, s, table, 8u);
	}));
	CHECK(throws<STPException::STPInvalidEnvironment>([&] {
		STPHeightfieldGenerator g(uvec2 { 32u, 32u }, uvec2 { 2u, 3u }, uvec2 { 3u, 3u }, raindrop(100u), s, table, 8u);
	}));
}

void generator_round_trip() {
	const unsigned int S = 64u;
	STPEnvironment::STPSimplexNoiseSetting s {};
	s.Seed = 42u;
	s.Distribution = 8u;
	s.Offset = 0.2181661565;
	std::vector<stpgb_biome_property> table = { { 128.0f, 6u, 0.5f, 2.0f, 0.0f, 1.0f }, { 64.0f, 4u, 0.5f, 2.0f, 0.1f, 0.5f } };
	STPHeightfieldGenerator gen(uvec2 { S, S }, uvec2 { 3u, 3u }, uvec2 { 3u, 3u }, raindrop(20000u), s, table, 16u);
	std::vector<std::vector<STPSample_t>> biomes(9, std::vector<STPSample_t>(S * S));
	for (int c = 0; c < 9; c++) {
		for (unsigned int i = 0; i < S * S; i++) {
			biomes[c][i] = static_cast<STPSample_t>(((i % S) / 20u + (i / S) / 24u + c) % 2u);
		}
	}
	std::vector<const STPSample_t*> biome_ptr;
	for (auto& b : biomes) {
		biome_ptr.push_back(b.data());
	}
	std::vector<std::vector<float>> heights(9, std::vector<float>(S * S));
	std::vector<std::vector<STPHeightFixed_t>> fixed(9, std::vector<STPHeightFixed_t>(S * S));
	std::vector<float*> hp;
	std::vector<STPHeightFixed_t*> fp;
	for (int c = 0; c < 9; c++) {
		gen.generate(heights[c].data(), biome_ptr.data(), vec2 { float((c % 3) * S), float((c / 3) * S) });
		hp.push_back(heights[c].data());
		fp.push_back(fixed[c].data());
	}
	double before = 0.0;
	for (auto& h : heights) {
		for (float v : h) {
			CHECK(v >= 0.0f && v <= 1.1f);
			before += v;
		}
	}
	gen.erode(hp.data(), fp.data());
	double after = 0.0;
	bool changed = false;
	for (int c = 0; c < 9; c++) {
		for (unsigned int i = 0; i < S * S; i++) {
			after += heights[c][i];
			const float cl = heights[c][i] < 0.0f ? 0.0f : (heights[c][i] > 1.0f ? 1.0f : heights[c][i]);
			CHECK(fixed[c][i] == static_cast<STPHeightFixed_t>(std::rint(cl * 65535.0f)));
			changed = changed || fixed[c][i] != 0u;
		}
	}
	CHECK(changed);
	CHECK(after <= before + 1e-3 * before); // sediment only leaves the map
}

// A user-written diversity plugin, as a SuperTerrain+ caller writes one
// against STPDiversityGenerator.hpp: both maps staged in host memory through
// STPMergedBuffer; the height of a pixel is a function of its own biome
// sample, its four axis neighbours 7 pixels away in the merged neighbourhood
// (reaching into the neighbour chunks) and the chunk offset.
struct TerracePlugin : STPDiversityGenerator {
	unsigned int Calls = 0u;
	void operator()(const STPNearestNeighbourHeightFloatWTextureBuffer& heightmap_buffer,
		const STPNearestNeighbourSampleRTextureBuffer& biomemap_buffer, const STPVec2 offset) override {
		using HB = STPNearestNeighbourHeightFloatWTextureBuffer;
		using BB = STPNearestNeighbourSampleRTextureBuffer;
		const HB::STPMergedBuffer height(heightmap_buffer, HB::STPMemoryLocation::HostMemory);
		const BB::STPMergedBuffer biome(biomemap_buffer, BB::STPMemoryLocation::HostMemory);
		const auto& nn = biomemap_buffer.NeighbourInfo;
		const unsigned int W = nn.MapSize.x, H = nn.MapSize.y, TW = nn.TotalMapSize.x;
		const unsigned int ox = (nn.ChunkNearestNeighbour.x / 2u) * W, oy = (nn.ChunkNearestNeighbour.y / 2u) * H;
		const STPSample_t* const b = biome.getHost();
		float* const h = height.getHost();
		for (unsigned int y = 0u; y < H; y++) {
			for (unsigned int x = 0u; x < W; x++) {
				const size_t c = static_cast<size_t>(y + oy) * TW + (x + ox);
				const unsigned int around = b[c - 7u] + b[c + 7u] + b[c - 7u * TW] + b[c + 7u * TW];
				h[static_cast<size_t>(y) * W + x] = 0.1f * b[c] + 0.01f * around + 1e-4f * static_cast<float>(offset.x);
			}
		}
		Calls++;
	}
};

struct FailingPlugin : STPDiversityGenerator {
	struct Refused : std::runtime_error {
		using std::runtime_error::runtime_error;
	};
	void operator()(const STPNearestNeighbourHeightFloatWTextureBuffer&, const STPNearestNeighbourSampleRTextureBuffer&,
		STPVec2) override {
		throw Refused("this plugin refuses every chunk");
	}
};

STPEnvironment::STPChunkSetting chunk_setting(unsigned int S) {
	STPEnvironment::STPChunkSetting c;
	c.ChunkSize = STPUVec2 { S, S };
	c.MapSize = STPUVec2 { S, S };
	c.ChunkScale = STPDVec2 { 1.0, 1.0 };
	c.DiversityNearestNeighbour = STPUVec2 { 3u, 3u };
	c.ErosionNearestNeighbour = STPUVec2 { 3u, 3u };
	c.SplatNearestNeighbour = STPUVec2 { 3u, 3u };
	c.RenderDistance = STPUVec2 { 5u, 5u };
	return c;
}

void plugin_setup_errors() {
	TerracePlugin plugin;
	auto chunk = chunk_setting(32u);
	const auto rain = raindrop(100u);
	CHECK(throws<STPException::STPInvalidEnvironment>([&] {
		STPHeightfieldGenerator g(STPHeightfieldGenerator::STPGeneratorSetup { &chunk, &rain, nullptr });
	}));
	chunk.DiversityNearestNeighbour = STPUVec2 { 2u, 3u };
	CHECK(throws<STPException::STPInvalidEnvironment>([&] {
		STPHeightfieldGenerator g(STPHeightfieldGenerator::STPGeneratorSetup { &chunk, &rain, &plugin });
	}));
	CHECK(plugin.Calls == 0u);
}

void user_plugin_generates() {
	const unsigned int S = 48u;
	TerracePlugin plugin;
	const auto chunk = chunk_setting(S);
	const auto rain = raindrop(5000u);
	STPHeightfieldGenerator gen(STPHeightfieldGenerator::STPGeneratorSetup { &chunk, &rain, &plugin });
	std::vector<std::vector<STPSample_t>> biomes(9, std::vector<STPSample_t>(S * S));
	std::vector<const STPSample_t*> bp;
	for (int c = 0; c < 9; c++) {
		for (unsigned int i = 0; i < S * S; i++) {
			biomes[c][i] = static_cast<STPSample_t>((i * 7u + (i / S) * 3u + static_cast<unsigned int>(c) * 5u) % 11u);
		}
		bp.push_back(biomes[c].data());
	}
	std::vector<float> h(S * S, -1.0f);
	gen.generate(h.data(), bp.data(), vec2 { 96.0f, -48.0f });
	CHECK(plugin.Calls == 1u);
	// the same formula on the caller's own chunks
	auto at = [&](int x, int y) {
		const int cx = (x + static_cast<int>(S)) / static_cast<int>(S), cy = (y + static_cast<int>(S)) / static_cast<int>(S);
		const int lx = x + static_cast<int>(S) - cx * static_cast<int>(S), ly = y + static_cast<int>(S) - cy * static_cast<int>(S);
		return static_cast<unsigned int>(biomes[cy * 3 + cx][ly * S + lx]);
	};
	bool equal = true;
	for (int y = 0; y < static_cast<int>(S); y++) {
		for (int x = 0; x < static_cast<int>(S); x++) {
			const unsigned int around = at(x - 7, y) + at(x + 7, y) + at(x, y - 7) + at(x, y + 7);
			const float want = 0.1f * at(x, y) + 0.01f * around + 1e-4f * 96.0f;
			equal = equal && h[y * S + x] == want;
		}
	}
	CHECK(equal);
	// an exception thrown by the plugin reaches the caller of generate unchanged
	FailingPlugin bad;
	STPHeightfieldGenerator gen_bad(STPHeightfieldGenerator::STPGeneratorSetup { &chunk, &rain, &bad });
	CHECK(throws<FailingPlugin::Refused>([&] { gen_bad.generate(h.data(), bp.data(), vec2 { 0.0f, 0.0f }); }));
	// the demo plugin through the setup constructor gives the folded constructor's heightmap
	STPEnvironment::STPSimplexNoiseSetting s {};
	s.Seed = 42u;
	s.Distribution = 8u;
	s.Offset = 0.2181661565;
	std::vector<stpgb_biome_property> table(11, stpgb_biome_property { 96.0f, 5u, 0.5f, 2.0f, 0.0f, 0.7f });
	STPDemo::STPBiomefieldGenerator field(s, table, 8u);
	STPHeightfieldGenerator via_setup(STPHeightfieldGenerator::STPGeneratorSetup { &chunk, &rain, &field });
	STPHeightfieldGenerator folded(uvec2 { S, S }, uvec2 { 3u, 3u }, uvec2 { 3u, 3u }, rain, s, table, 8u);
	std::vector<float> a(S * S), b(S * S);
	via_setup.generate(a.data(), bp.data(), vec2 { 48.0f, 0.0f });
	folded.generate(b.data(), bp.data(), vec2 { 48.0f, 0.0f });
	CHECK(a == b);
}

struct ivec2 {
	int x, y;
	ivec2(int a, int b) : x(a), y(b) {}
	bool operator==(const ivec2& o) const {
		return x == o.x && y == o.y;
	}
};

uint64_t fnv1a(const std::vector<STPSample_t>& v) {
	uint64_t h = 0xcbf29ce484222325ull;
	for (const STPSample_t s : v) {
		for (int b = 0; b < 2; b++) {
			h ^= static_cast<uint8_t>(s >> (8 * b));
			h *= 0x100000001b3ull;
		}
	}
	return h;
}

void biome_factory_errors() {
	CHECK(throws<STPException::STPNumericDomainError>([] { STPDemo::STPLayerChainBuilder f(ivec2 { 0, 4 }, 1u); }));
}

// SuperTest+/SuperTerrain+/STPTest2DChunk.cpp:30-89, with the test's own vector types
struct dvec2 {
	double x, y;
	dvec2(double a, double b) : x(a), y(b) {}
	bool operator==(const dvec2& o) const {
		return x == o.x && y == o.y;
	}
};
struct dvec3 {
	double x, y, z;
};

void chunk_coordinates() {
	const dvec3 camera { -573.74, 679.5, 845.982 };
	const uvec2 chunk_size { 8u, 5u };
	const dvec2 scale(2.5, 4.0);
	const ivec2 position = STPChunk::calcWorldChunkCoordinate(camera, chunk_size, scale);
	CHECK(position == ivec2(-232, 210));
	const dvec2 map_offset = STPChunk::calcChunkMapOffset(position, chunk_size, uvec2 { 512u, 256u }, dvec2(25.5, -57.5));
	CHECK(map_offset == dvec2(-14822.5, 10694.5));
	CHECK(static_cast<ivec2>(STPChunk::offsetChunk(ivec2(30, -30), chunk_size, ivec2(3, -2))) == ivec2(54, -40));
	const uvec2 region { 5u, 7u };
	const uvec2 l7 = STPChunk::calcLocalChunkCoordinate(7u, region), l12 = STPChunk::calcLocalChunkCoordinate(12u, region),
		l20 = STPChunk::calcLocalChunkCoordinate(20u, region);
	CHECK(l7.x == 2u && l7.y == 1u);
	CHECK(l12.x == 2u && l12.y == 2u);
	CHECK(l20.x == 0u && l20.y == 4u);
	CHECK(static_cast<ivec2>(STPChunk::calcLocalChunkOrigin(ivec2(-24, 50), chunk_size, region)) == ivec2(-40, 35));
	const auto offsets = STPChunk::calcChunkNeighbourOffset(chunk_size, region);
	CHECK(offsets.size() == 35u);
	CHECK(static_cast<ivec2>(offsets[0]) == ivec2(-16, -15));
	CHECK(static_cast<ivec2>(offsets[9]) == ivec2(16, -10));
	CHECK(static_cast<ivec2>(offsets[17]) == ivec2(0, 0));
	CHECK(static_cast<ivec2>(offsets[23]) == ivec2(8, 5));
	CHECK(static_cast<ivec2>(offsets[34]) == ivec2(16, 15));
	CHECK(throws<STPException::STPNumericDomainError>([&] { STPChunk::calcLocalChunkCoordinate(1u, uvec2 { 0u, 3u }); }));
}

void splat_generator_errors() {
	STPEnvironment::STPSimplexNoiseSetting s {};
	s.Seed = 1u;
	s.Distribution = 8u;
	s.Offset = 0.1;
	// a gradient rule whose slope range is empty (min > max)
	CHECK(throws<STPException::STPNumericDomainError>([&] {
		STPDiversity::STPTextureSplatGenerator g({}, { { 0u, 0.5f, 0.2f, 0.0f, 1.0f, 1u } }, s, uvec2 { 64u, 64u });
	}));
	STPEnvironment::STPSimplexNoiseSetting bad = s;
	bad.Distribution = 0u;
	CHECK(throws<STPException::STPInvalidEnvironment>([&] {
		STPDiversity::STPTextureSplatGenerator g({ { 0u, 1.0f, 4u } }, {}, bad, uvec2 { 64u, 64u });
	}));
}

// tests/golden/layer_biomemap.npz cases 4 and 7: the reference's own layer
// chain (STPLayerChainBuilder, compiled from its sources), FNV-1a of the
// little-endian uint16 map.
void biome_factory_reference_maps() {
	STPDemo::STPLayerChainBuilder a(ivec2 { 1024, 1024 }, 11u);
	std::vector<STPSample_t> m(1024u * 1024u);
	a(m.data(), ivec2 { -512, -512 });
	CHECK(fnv1a(m) == 0x5a656f9c4454cb0cull);
	STPDemo::STPLayerChainBuilder b(ivec2 { 512, 512 }, 0u);
	std::vector<STPSample_t> n(512u * 512u);
	b(n.data(), ivec2 { 1000000, -2000000 });
	CHECK(fnv1a(n) == 0x9e90f7226ff73ea4ull);
}

} // namespace

int main(int argc, char** argv) {
	const bool cpu_only = argc > 1 && std::strcmp(argv[1], "--cpu") == 0;
	histogram_errors();
	permutation();
	generator_errors();
	biome_factory_errors();
	splat_generator_errors();
	chunk_coordinates();
	plugin_setup_errors();
	if (!cpu_only) {
		user_plugin_generates();
		histogram_known_answer();
		generator_round_trip();
		biome_factory_reference_maps();
	}
	std::printf("%s: %d failure(s)\n", cpu_only ? "cpu" : "all", failures);
	return failures == 0 ? 0 : 1;
}
