// Biome layer chain: STPBiomeFactory::operator() over the demo's STPLayer
// production line, one fused launch.
//
// The reference samples the last layer pixel by pixel on one CPU thread;
// every layer pulls the parent samples it needs through a small hash cache
// (SuperTerrain+/Private/World/Diversity/STPLayer.cpp:57-88,162-170,
// STPBiomeFactory.cpp:24-41).  Here one CTA owns a square tile of the output:
// it first walks the chain from the sampled layer up to the first ancestor
// to find the rectangle each layer must supply (a x2 zoom halves it, a
// cross layer widens it by one, a x4 Voronoi zoom quarters it), then
// evaluates the layers from the first ancestor down, each over its whole
// rectangle, reading the parent rectangle from shared memory and writing its
// own into the other half of a ping-pong pair.  Only the last layer touches
// global memory (2 bytes per output pixel, coalesced rows).  The ancestors'
// rectangles are a few hundred samples per tile, so the small redundant
// overlap between tiles costs little next to the last layer.
//
// Layer arithmetic is the reference's, in 64-bit integers:
//   mixSeed s*(s*6364136223846793005 + 1442695040888963407) + fac   (STPLayer.cpp:146-150)
//   seedLayer / seedLocal / STPLocalSampler                          (STPLayer.cpp:96-145)
//   continent, scale, land, island, voronoi                          (SuperDemo+/World/Layers/*.h)
// The Voronoi layer compares eight squared distances that the reference
// computes in double precision.  Each candidate cell's jitter (eight mixes)
// is computed once per tile into shared memory (in FP32 for the fast path,
// with the three 10-bit draws kept); the distances are then compared in
// FP32.  Error bound of one FP32 distance against the reference's double:
// jitter 2.7e-8 (0.9f and one rounding), offset t = f + jitter 8.7e-8
// (|t| < 1.45), square 2.5e-7 + half an ulp, and two fused adds of values
// below 6.4, in all under 1.4e-6; two distances compare correctly when
// their FP32 gap exceeds 2.8e-6.  When the smallest FP32 distance is not
// ahead of the runner-up by kVoronoiGap (2^-17 = 7.6e-6) the pixel redoes
// all eight distances in double precision with the reference's operation
// order, so the chosen cell, and the tie rule (first strict minimum), are
// the reference's exactly.  About 2.5e-5 of the pixels take that path; it
// is kept rare because FP64 issues slowly on this part.
#include "layers.cuh"

#include <algorithm>
#include <vector>

namespace stpgb {

namespace {

constexpr uint32_t kLayerThreads = 256u;
constexpr float kVoronoiGap = 1.0f / 131072.0f;
// blocks a layer launch aims for per SM of the device
constexpr uint32_t kTargetBlocksPerSM = 2u;
constexpr size_t kSmemLimit = 48u * 1024u;
constexpr int64_t kCoordLimit = int64_t(1) << 30;

enum : uint32_t {
	kContinent = STPGB_LAYER_CONTINENT,
	kScale = STPGB_LAYER_SCALE,
	kLand = STPGB_LAYER_LAND,
	kIsland = STPGB_LAYER_ISLAND,
	kVoronoi = STPGB_LAYER_VORONOI
};

constexpr uint64_t kMulA = 6364136223846793005ull;
constexpr uint64_t kAddB = 1442695040888963407ull;

__host__ __device__ __forceinline__ uint64_t lcg_mix(const uint64_t s, const uint64_t fac) {
	return s * (s * kMulA + kAddB) + fac;
}

__host__ __device__ __forceinline__ uint64_t sext(const int v) {
	return static_cast<uint64_t>(static_cast<int64_t>(v));
}

uint64_t layer_seed_of(const uint64_t global, const uint64_t salt) {
	uint64_t mid = lcg_mix(salt, salt);
	mid = lcg_mix(mid, mid);
	mid = lcg_mix(mid, mid);
	uint64_t s = lcg_mix(global, mid);
	s = lcg_mix(s, mid);
	return lcg_mix(s, mid);
}

__device__ __forceinline__ uint64_t local_seed(const uint64_t layer, const int x, const int z) {
	uint64_t s = lcg_mix(layer, sext(x));
	s = lcg_mix(s, sext(z));
	s = lcg_mix(s, sext(x));
	return lcg_mix(s, sext(z));
}

// STPLocalSampler::nextValue with a compile-time range.
template<uint32_t R>
__device__ __forceinline__ uint32_t draw(uint64_t& state, const uint64_t layer) {
	const uint32_t v = static_cast<uint32_t>((state >> 24) % R);
	state = lcg_mix(state, layer);
	return v;
}

// Ranges 1..4 of the land layer's growing counter.
__device__ __forceinline__ uint32_t draw_upto4(uint64_t& state, const uint64_t layer, const uint32_t range) {
	const uint64_t v = state >> 24;
	state = lcg_mix(state, layer);
	switch (range) {
	case 1u:
		return 0u;
	case 2u:
		return static_cast<uint32_t>(v & 1u);
	case 3u:
		return static_cast<uint32_t>(v % 3u);
	default:
		return static_cast<uint32_t>(v & 3u);
	}
}

struct Region {
	int x0, z0, x1, z1; // half-open
};

// The rectangle a layer of kind `kind` reads from its parent to cover `r`.
__device__ __forceinline__ Region parent_region(const uint32_t kind, const Region r) {
	switch (kind) {
	case kScale:
		return Region { r.x0 >> 1, r.z0 >> 1, (r.x1 >> 1) + 1, (r.z1 >> 1) + 1 };
	case kVoronoi:
		return Region { (r.x0 - 2) >> 2, (r.z0 - 2) >> 2, ((r.x1 - 3) >> 2) + 2, ((r.z1 - 3) >> 2) + 2 };
	default: // land, island
		return Region { r.x0 - 1, r.z0 - 1, r.x1 + 1, r.z1 + 1 };
	}
}

// Upper bound of the parent extent for an extent of w anywhere on the axis.
uint32_t parent_extent(const uint32_t kind, const uint32_t w) {
	switch (kind) {
	case kScale:
		return ((w + 1u) >> 1) + 1u;
	case kVoronoi:
		return ((w + 2u) >> 2) + 2u;
	default:
		return w + 2u;
	}
}

struct Ids {
	uint16_t ocean, plains, forest, shallow[5];
	__device__ __forceinline__ bool so(const uint16_t v) const {
		return v == shallow[0] || v == shallow[1] || v == shallow[2] || v == shallow[3] || v == shallow[4];
	}
};

// Parent rectangle in shared memory.
struct Parent {
	const uint16_t* v;
	Region r;
	int w;
	__device__ __forceinline__ uint16_t at(const int x, const int z) const {
		return v[(z - r.z0) * w + (x - r.x0)];
	}
};

__device__ __forceinline__ uint16_t scale_sample(const Parent& P, const uint64_t seed, const bool fuzzy, const int x,
	const int z) {
	const uint16_t c = P.at(x >> 1, z >> 1);
	const int odd_x = x & 1, odd_z = z & 1;
	if (!odd_x && !odd_z) {
		return c;
	}
	uint64_t st = local_seed(seed, x & -2, z & -2);
	const uint16_t s = P.at(x >> 1, (z + 1) >> 1);
	const uint16_t along_z = draw<2>(st, seed) == 0u ? c : s;
	if (!odd_x) {
		return along_z;
	}
	const uint16_t e = P.at((x + 1) >> 1, z >> 1);
	const uint16_t along_x = draw<2>(st, seed) == 0u ? c : e;
	if (!odd_z) {
		return along_x;
	}
	const uint16_t se = P.at((x + 1) >> 1, (z + 1) >> 1);
	const uint32_t k = draw<4>(st, seed);
	const uint16_t any = k == 0u ? c : k == 1u ? e : k == 2u ? s : se;
	if (fuzzy) {
		return any;
	}
	if (e == s && e == se) {
		return e;
	}
	if (c == e && (c == se || s != se)) {
		return c;
	}
	if (c == s && (c == se || e != se)) {
		return c;
	}
	if (c == se && e != s) {
		return c;
	}
	if (e == s && c != se) {
		return e;
	}
	if (e == se && c != s) {
		return e;
	}
	if (s == se && c != e) {
		return s;
	}
	return any;
}

__device__ __forceinline__ uint16_t land_sample(const Parent& P, const uint64_t seed, const Ids& id, const int x,
	const int z) {
	const uint16_t c = P.at(x, z), ne = P.at(x + 1, z - 1), se = P.at(x + 1, z + 1), sw = P.at(x - 1, z + 1),
		nw = P.at(x - 1, z - 1);
	const bool so_c = id.so(c), so_ne = id.so(ne), so_se = id.so(se), so_sw = id.so(sw), so_nw = id.so(nw);
	uint64_t st = local_seed(seed, x, z);
	if (!so_c || (so_sw && so_se && so_ne && so_nw)) {
		if (so_c || (!so_sw && !so_se && !so_ne && !so_nw) || draw<5>(st, seed) != 0u) {
			return c;
		}
		const uint16_t coast = so_nw ? nw : so_sw ? sw : so_ne ? ne : so_se ? se : c;
		if (!(so_nw || so_sw || so_ne || so_se)) {
			return c;
		}
		return c == id.forest ? id.forest : coast;
	}
	uint32_t range = 1u;
	uint16_t chosen = 1u;
	if (!so_nw && draw_upto4(st, seed, range++) == 0u) {
		chosen = nw;
	}
	if (!so_ne && draw_upto4(st, seed, range++) == 0u) {
		chosen = ne;
	}
	if (!so_sw && draw_upto4(st, seed, range++) == 0u) {
		chosen = sw;
	}
	if (!so_se && draw_upto4(st, seed, range) == 0u) {
		chosen = se;
	}
	if (draw<3>(st, seed) == 0u) {
		return chosen;
	}
	return chosen == id.forest ? id.forest : c;
}

__device__ __forceinline__ uint16_t island_sample(const Parent& P, const uint64_t seed, const Ids& id, const int x,
	const int z) {
	const uint16_t c = P.at(x, z);
	if (!(id.so(c) && id.so(P.at(x, z - 1)) && id.so(P.at(x + 1, z)) && id.so(P.at(x, z + 1))
			&& id.so(P.at(x - 1, z)))) {
		return c;
	}
	uint64_t st = local_seed(seed, x, z);
	return draw<2>(st, seed) == 0u ? id.plains : c;
}

// (k / 1024 - 0.5) * 0.9 in double, as STPVoronoiLayer.h's distribute().
__device__ __forceinline__ double jitter_d(const uint32_t k) {
	return __dmul_rn(__dadd_rn(static_cast<double>(k) * 0.0009765625, -0.5), 0.9);
}

// The same jitter in FP32 for the fast comparison (within 4e-8 of the double).
__device__ __forceinline__ float jitter_f(const uint32_t k) {
	return (static_cast<float>(k) * 0.0009765625f - 0.5f) * 0.9f;
}

// Jitter of the Voronoi cells (cx, cy, cz) over the parent rectangle, planes
// cy = -1 and cy = 0, for the FP32 comparison: x jitter, z jitter, and the
// squared y offset, which is the same for every pixel of a 2-D layer
// (y = 0 sits at fraction 0.5 of cell -1); .w keeps the three 10-bit draws.
__device__ __forceinline__ void voronoi_cells(float4* cells, const Region pr, const uint64_t vseed) {
	const int pw = pr.x1 - pr.x0, parea = pw * (pr.z1 - pr.z0);
	for (int idx = threadIdx.x; idx < 2 * parea; idx += blockDim.x) {
		const int plane = idx >= parea ? 1 : 0, rem = idx - plane * parea;
		const int cx = pr.x0 + rem % pw, cz = pr.z0 + rem / pw, cy = plane - 1;
		uint64_t h = lcg_mix(vseed, sext(cx));
		h = lcg_mix(h, sext(cy));
		h = lcg_mix(h, sext(cz));
		h = lcg_mix(h, sext(cx));
		h = lcg_mix(h, sext(cy));
		h = lcg_mix(h, sext(cz));
		const uint32_t kx = static_cast<uint32_t>(h >> 24) & 1023u;
		h = lcg_mix(h, vseed);
		const uint32_t ky = static_cast<uint32_t>(h >> 24) & 1023u;
		h = lcg_mix(h, vseed);
		const uint32_t kz = static_cast<uint32_t>(h >> 24) & 1023u;
		const float ty = (0.5f - static_cast<float>(plane)) + jitter_f(ky);
		cells[idx] = make_float4(jitter_f(kx), jitter_f(kz), ty * ty, __uint_as_float(kx | (ky << 10) | (kz << 20)));
	}
}

// The reference's eight double-precision distances (summed z, y, x) and its
// first-strict-minimum rule, for a pixel whose FP32 comparison was too close.
__device__ __noinline__ int voronoi_exact(const float4* cells, const int base, const int pw, const int parea,
	const int qx, const int qz) {
	const double fx = qx * 0.25, fy = 0.5, fz = qz * 0.25;
	int best = 0;
	double best_d = 0.0;
#pragma unroll 1
	for (int c = 0; c < 8; c++) {
		const int hx = (c >> 2) & 1, hy = (c >> 1) & 1, hz = c & 1;
		const uint32_t k = __float_as_uint(cells[base + hy * parea + hz * pw + hx].w);
		const double tz = __dadd_rn(fz - hz, jitter_d((k >> 20) & 1023u));
		const double ty = __dadd_rn(fy - hy, jitter_d((k >> 10) & 1023u));
		const double tx = __dadd_rn(fx - hx, jitter_d(k & 1023u));
		const double d = __dadd_rn(__dadd_rn(__dmul_rn(tz, tz), __dmul_rn(ty, ty)), __dmul_rn(tx, tx));
		if (c == 0 || d < best_d) {
			best = c;
			best_d = d;
		}
	}
	return best;
}

// A Voronoi layer over rectangle r.  The pixels of one 4 x 4 block (x - 2
// and z - 2 in the same multiple of four) share their eight candidate cells;
// a work item is one row of a block: it loads each candidate once and
// updates the four pixels' best and runner-up distances.
template<class Emit>
__device__ __forceinline__ void voronoi_region(const Parent& P, const float4* cells, const Region r, Emit emit) {
	const int parea = P.w * (P.r.z1 - P.r.z0);
	const int bx0 = (r.x0 - 2) >> 2;
	const int nbx = ((r.x1 - 3) >> 2) - bx0 + 1, rows = r.z1 - r.z0;
	for (int j = threadIdx.x; j < nbx * rows; j += blockDim.x) {
		const int z = r.z0 + j / nbx, cx = bx0 + j % nbx;
		const int cz = (z - 2) >> 2, qz = (z - 2) & 3;
		const int base = (cz - P.r.z0) * P.w + (cx - P.r.x0);
		const int px0 = 4 * cx + 2;
		const float fz = qz * 0.25f;
		float m1[4], m2[4];
		int best[4];
#pragma unroll
		for (int q = 0; q < 4; q++) {
			m1[q] = 3.0e38f;
			m2[q] = 3.0e38f;
			best[q] = 0;
		}
#pragma unroll
		for (int c = 0; c < 8; c++) {
			const int hx = (c >> 2) & 1, hy = (c >> 1) & 1, hz = c & 1;
			const float4 J = cells[base + hy * parea + hz * P.w + hx];
			const float tz = (fz - hz) + J.y;
			const float zy = fmaf(tz, tz, J.z);
#pragma unroll
			for (int q = 0; q < 4; q++) {
				const float tx = (q * 0.25f - hx) + J.x;
				const float d = fmaf(tx, tx, zy);
				if (d < m1[q]) {
					m2[q] = m1[q];
					m1[q] = d;
					best[q] = c;
				} else if (d < m2[q]) {
					m2[q] = d;
				}
			}
		}
#pragma unroll
		for (int q = 0; q < 4; q++) {
			const int x = px0 + q;
			if (x < r.x0 || x >= r.x1) {
				continue;
			}
			int b = best[q];
			if (m2[q] - m1[q] < kVoronoiGap) {
				b = voronoi_exact(cells, base, P.w, parea, q, qz);
			}
			emit(x, z, P.at(cx + ((b >> 2) & 1), cz + (b & 1)));
		}
	}
}

__global__ void __launch_bounds__(kLayerThreads) layer_kernel(const LayerChain chain,
	const BiomemapJob* __restrict__ jobs, const BiomemapJob single, const uint32_t tile, const uint32_t cap,
	const uint32_t cell_cap) {
	const BiomemapJob& J = jobs ? jobs[blockIdx.y] : single;
	if (blockIdx.x >= J.tiles) {
		return;
	}
	extern __shared__ float4 smem[];
	uint16_t* const buf0 = reinterpret_cast<uint16_t*>(smem);
	uint16_t* const buf1 = buf0 + cap;
	float4* const cells = reinterpret_cast<float4*>(buf0 + 2u * cap);
	__shared__ Region reg[kMaxLayers];

	const int n = static_cast<int>(chain.count);
	if (threadIdx.x == 0) {
		const uint32_t tx = blockIdx.x % J.tiles_x, tz = blockIdx.x / J.tiles_x;
		Region r;
		const int gx = J.gx0 + static_cast<int>(tx * tile), gz = J.gz0 + static_cast<int>(tz * tile);
		r.x0 = max(gx, J.x0);
		r.z0 = max(gz, J.z0);
		r.x1 = min(gx + static_cast<int>(tile), J.x0 + static_cast<int>(J.width));
		r.z1 = min(gz + static_cast<int>(tile), J.z0 + static_cast<int>(J.height));
		reg[n - 1] = r;
		for (int i = n - 1; i > 0; i--) {
			reg[i - 1] = parent_region(chain.kind[i], reg[i]);
		}
	}
	__syncthreads();
	const Ids id { chain.ocean, chain.plains, chain.forest,
		{ chain.shallow[0], chain.shallow[1], chain.shallow[2], chain.shallow[3], chain.shallow[4] } };

	for (int i = 0; i < n; i++) {
		const Region r = reg[i];
		const int w = r.x1 - r.x0, area = w * (r.z1 - r.z0);
		const bool last = i == n - 1;
		const uint32_t kind = chain.kind[i];
		const uint64_t seed = chain.seed[i];
		Parent P { (i & 1) ? buf0 : buf1, Region {}, 1 };
		if (i > 0) {
			P.r = reg[i - 1];
			P.w = P.r.x1 - P.r.x0;
		}
		// The host sizes cap / cell_cap from upper bounds of these areas;
		// the check keeps every shared-memory access in bounds regardless.
		const int parea = P.w * (P.r.z1 - P.r.z0);
		if ((!last && area > static_cast<int>(cap)) || (kind == kVoronoi && 2 * parea > static_cast<int>(cell_cap))) {
			return;
		}
		if (kind == kVoronoi) {
			voronoi_cells(cells, P.r, chain.voronoi_seed);
			__syncthreads();
		}
		uint16_t* const dst = (i & 1) ? buf1 : buf0;
		if (kind == kVoronoi) {
			if (last) {
				voronoi_region(P, cells, r, [&](const int x, const int z, const uint16_t v) {
					J.out[static_cast<size_t>(z - J.z0) * J.pitch + static_cast<uint32_t>(x - J.x0)] = v;
				});
			} else {
				voronoi_region(P, cells, r, [&](const int x, const int z, const uint16_t v) {
					dst[(z - r.z0) * w + (x - r.x0)] = v;
				});
			}
			__syncthreads();
			continue;
		}
		for (int s = threadIdx.x; s < area; s += blockDim.x) {
			const int x = r.x0 + s % w, z = r.z0 + s / w;
			uint16_t v;
			switch (kind) {
			case kContinent: {
				uint64_t st = local_seed(seed, x, z);
				v = draw<10>(st, seed) == 0u ? id.plains : id.ocean;
				break;
			}
			case kScale:
				v = scale_sample(P, seed, chain.param[i] != 0u, x, z);
				break;
			case kLand:
				v = land_sample(P, seed, id, x, z);
				break;
			default:
				v = island_sample(P, seed, id, x, z);
				break;
			}
			if (last) {
				J.out[static_cast<size_t>(z - J.z0) * J.pitch + static_cast<uint32_t>(x - J.x0)] = v;
			} else {
				dst[s] = v;
			}
		}
		__syncthreads();
	}
}

struct SmemPlan {
	uint32_t cap, cell_cap;
	size_t bytes;
};

SmemPlan plan_smem(const LayerChain& chain, const uint32_t tile) {
	uint32_t ext[kMaxLayers];
	const uint32_t n = chain.count;
	ext[n - 1] = tile;
	for (uint32_t i = n - 1; i > 0; i--) {
		ext[i - 1] = parent_extent(chain.kind[i], ext[i]);
	}
	SmemPlan p { 8u, 0u, 0u };
	for (uint32_t i = 0; i + 1 < n; i++) {
		p.cap = std::max(p.cap, ext[i] * ext[i]);
	}
	for (uint32_t i = 1; i < n; i++) {
		if (chain.kind[i] == kVoronoi) {
			p.cell_cap = std::max(p.cell_cap, 2u * ext[i - 1] * ext[i - 1]);
		}
	}
	p.cap = (p.cap + 7u) & ~7u;
	p.bytes = 2u * p.cap * sizeof(uint16_t) + p.cell_cap * sizeof(float4);
	return p;
}

} // namespace

int layer_chain_prepare(const stpgb_layer* chain, const uint32_t count, const uint64_t global_seed,
	const stpgb_layer_biomes* ids, LayerChain* out) {
	if (!chain || !ids || !out) {
		return inval("layer chain: null argument");
	}
	if (count == 0u || count > kMaxLayers) {
		return inval("layer chain: layer count must be in [1, " + std::to_string(kMaxLayers) + "]");
	}
	LayerChain c {};
	c.count = count;
	c.ocean = ids->Ocean;
	c.plains = ids->Plains;
	c.forest = ids->Forest;
	std::copy(ids->ShallowOcean, ids->ShallowOcean + 5, c.shallow);
	// STPVoronoiLayer seeds with std::hash<STPSeed_t>{}(global), the identity in libstdc++.
	c.voronoi_seed = global_seed;
	for (uint32_t i = 0; i < count; i++) {
		const stpgb_layer& L = chain[i];
		if ((i == 0u) != (L.Kind == kContinent)) {
			return inval("layer chain: the first layer, and only the first, must be a continent layer");
		}
		if (L.Kind < kContinent || L.Kind > kVoronoi) {
			return inval("layer chain: unknown layer kind " + std::to_string(L.Kind));
		}
		if (L.Kind == kScale && L.Param > STPGB_SCALE_FUZZY) {
			return inval("layer chain: scale type must be STPGB_SCALE_NORMAL or STPGB_SCALE_FUZZY");
		}
		if (L.Kind == kVoronoi && L.Param != 0u) {
			return inval("layer chain: only 2-D Voronoi layers are supported");
		}
		c.kind[i] = L.Kind;
		c.param[i] = L.Param;
		c.seed[i] = layer_seed_of(global_seed, L.Salt);
	}
	*out = c;
	return STPGB_OK;
}

uint32_t layer_tile_for(const uint64_t pixels) {
	const uint64_t target_blocks = uint64_t { kTargetBlocksPerSM } * current_sm_count();
	if (pixels >= target_blocks * 128u * 128u) {
		return 128u;
	}
	if (pixels >= target_blocks * 64u * 64u) {
		return 64u;
	}
	if (pixels >= target_blocks * 32u * 32u) {
		return 32u;
	}
	return 16u;
}

int layer_job_tiling(BiomemapJob& job, const uint32_t tile) {
	if (job.width == 0u || job.height == 0u) {
		return inval("layer biomemap: width and height must be positive");
	}
	const int64_t lo_x = job.x0, lo_z = job.z0, hi_x = lo_x + job.width, hi_z = lo_z + job.height;
	if (std::max(std::max(-lo_x, hi_x), std::max(-lo_z, hi_z)) >= kCoordLimit) {
		return inval("layer biomemap: the rectangle must stay within |coordinate| < 2^30");
	}
	if (job.pitch < job.width) {
		return inval("layer biomemap: pitch must be at least width");
	}
	// Tiles start on x, z = 2 (mod 4), the Voronoi block lattice, so that a
	// tile holds whole 4 x 4 blocks except at the rectangle's own edges.
	const uint32_t sx = static_cast<uint32_t>(job.x0 - 2) & 3u, sz = static_cast<uint32_t>(job.z0 - 2) & 3u;
	job.gx0 = job.x0 - static_cast<int32_t>(sx);
	job.gz0 = job.z0 - static_cast<int32_t>(sz);
	job.tiles_x = (job.width + sx + tile - 1u) / tile;
	job.tiles = job.tiles_x * ((job.height + sz + tile - 1u) / tile);
	return STPGB_OK;
}

int layer_biomemap_launch(const LayerChain& chain, const BiomemapJob* jobs, const BiomemapJob& single,
	const uint32_t njobs, const uint32_t max_tiles, uint32_t tile, cudaStream_t stream) {
	const SmemPlan plan = plan_smem(chain, tile);
	if (plan.bytes > kSmemLimit) {
		return inval("layer biomemap: the chain needs more shared memory than a tile of " + std::to_string(tile)
			+ " allows");
	}
	if (njobs == 0u || max_tiles == 0u) {
		return STPGB_OK;
	}
	const dim3 grid(max_tiles, njobs);
	layer_kernel<<<grid, kLayerThreads, plan.bytes, stream>>>(chain, jobs, single, tile, plan.cap, plan.cell_cap);
	STPGB_CUDA_TRY(cudaGetLastError());
	return STPGB_OK;
}

// Chooses the largest tile (<= `tile`) whose shared-memory plan fits.
static uint32_t fit_tile(const LayerChain& chain, uint32_t tile) {
	while (tile > 8u && plan_smem(chain, tile).bytes > kSmemLimit) {
		tile >>= 1;
	}
	return tile;
}

uint32_t layer_tile(const LayerChain& chain, const uint64_t pixels) {
	return fit_tile(chain, layer_tile_for(pixels));
}

int layer_chain_demo(const uint64_t global_seed, LayerChain* out) {
	stpgb_layer chain[kMaxLayers];
	uint32_t n = 0u;
	STPGB_TRY(stpgb_layer_chain_demo(chain, kMaxLayers, &n));
	stpgb_layer_biomes ids;
	stpgb_layer_biomes_demo(&ids);
	return layer_chain_prepare(chain, n, global_seed, &ids, out);
}

} // namespace stpgb

using namespace stpgb;

extern "C" {

int stpgb_layer_chain_demo(stpgb_layer* chain, const uint32_t capacity, uint32_t* count) {
	// STPAllLayers.cpp:59-105: A0 .. D5 with their salts.
	static const stpgb_layer demo[] = {
		{ STPGB_LAYER_CONTINENT, 0u, 23457829ull },
		{ STPGB_LAYER_SCALE, STPGB_SCALE_FUZZY, 875944ull },
		{ STPGB_LAYER_LAND, 0u, 5748329ull },
		{ STPGB_LAYER_SCALE, STPGB_SCALE_NORMAL, 8947358941ull },
		{ STPGB_LAYER_LAND, 0u, 361249673ull },
		{ STPGB_LAYER_LAND, 0u, 8769575ull },
		{ STPGB_LAYER_LAND, 0u, 43562783426564ull },
		{ STPGB_LAYER_ISLAND, 0u, 74368ull },
		{ STPGB_LAYER_SCALE, STPGB_SCALE_NORMAL, 1ull },
		{ STPGB_LAYER_SCALE, STPGB_SCALE_NORMAL, 2ull },
		{ STPGB_LAYER_SCALE, STPGB_SCALE_NORMAL, 3ull },
		{ STPGB_LAYER_VORONOI, 0u, 4ull },
		{ STPGB_LAYER_VORONOI, 0u, 5ull },
		{ STPGB_LAYER_VORONOI, 0u, 6ull },
	};
	constexpr uint32_t n = sizeof(demo) / sizeof(demo[0]);
	if (!count) {
		return inval("stpgb_layer_chain_demo: null count");
	}
	*count = n;
	if (!chain || capacity < n) {
		return inval("stpgb_layer_chain_demo: capacity below " + std::to_string(n));
	}
	std::copy(demo, demo + n, chain);
	return STPGB_OK;
}

void stpgb_layer_biomes_demo(stpgb_layer_biomes* ids) {
	if (ids) {
		*ids = stpgb_layer_biomes { 0u, 1u, 3u, { 0u, 0u, 0u, 0u, 0u } };
	}
}

int stpgb_layer_biomemap(const stpgb_layer* chain, const uint32_t count, const uint64_t global_seed,
	const stpgb_layer_biomes* ids, uint16_t* biomemap, const uint32_t pitch, const uint32_t width,
	const uint32_t height, const int32_t offset_x, const int32_t offset_z, void* stream) {
	LayerChain c;
	STPGB_TRY(layer_chain_prepare(chain, count, global_seed, ids, &c));
	if (!biomemap) {
		return inval("stpgb_layer_biomemap: null biomemap");
	}
	BiomemapJob job {};
	job.out = biomemap;
	job.x0 = offset_x;
	job.z0 = offset_z;
	job.pitch = pitch;
	job.width = width;
	job.height = height;
	const uint32_t tile = fit_tile(c, layer_tile_for(uint64_t(width) * height));
	STPGB_TRY(layer_job_tiling(job, tile));
	return layer_biomemap_launch(c, nullptr, job, 1u, job.tiles, tile, as_stream(stream));
}

int stpgb_layer_biomemap_host(const stpgb_layer* chain, const uint32_t count, const uint64_t global_seed,
	const stpgb_layer_biomes* ids, uint16_t* biomemap, const uint32_t width, const uint32_t height,
	const int32_t offset_x, const int32_t offset_z) {
	if (!biomemap) {
		return inval("stpgb_layer_biomemap_host: null biomemap");
	}
	LayerChain c;
	STPGB_TRY(layer_chain_prepare(chain, count, global_seed, ids, &c));
	const size_t bytes = size_t(width) * height * sizeof(uint16_t);
	if (bytes == 0u) {
		return inval("stpgb_layer_biomemap_host: width and height must be positive");
	}
	cudaStream_t s = nullptr;
	uint16_t* dev = nullptr;
	STPGB_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
	int rc = STPGB_OK;
	const cudaError_t ea = cudaMallocAsync(&dev, bytes, s);
	if (ea != cudaSuccess) {
		rc = cuda_fail(ea, "cudaMallocAsync");
	} else {
		rc = stpgb_layer_biomemap(chain, count, global_seed, ids, dev, width, width, height, offset_x, offset_z, s);
		if (rc == STPGB_OK) {
			const cudaError_t ec = cudaMemcpyAsync(biomemap, dev, bytes, cudaMemcpyDeviceToHost, s);
			if (ec != cudaSuccess) {
				rc = cuda_fail(ec, "cudaMemcpyAsync");
			}
		}
		cudaFreeAsync(dev, s);
	}
	const cudaError_t es = cudaStreamSynchronize(s);
	cudaStreamDestroy(s);
	if (rc == STPGB_OK && es != cudaSuccess) {
		rc = cuda_fail(es, "cudaStreamSynchronize");
	}
	return rc;
}

} // extern "C"
