/*
 * oracle/stp_oracle.cpp — CPU restatement of the SuperTerrain+ heightfield
 * path.  TEST INFRASTRUCTURE ONLY: it is what the parity tests, the
 * smoke test and the CPU-baseline leg of bench.py compare the CUDA path
 * against.  The product never links or calls it.
 *
 * Pinning: the permutation and single-histogram-filter restatements are
 * checked against the reference's own golden vectors
 * (SuperTest+/SuperAlgorithm+/STPTestHistogram.cpp:44-105,
 *  SuperTest+/SuperAlgorithm+/STPTestPermutation.cpp:37-41,108-115) and
 * against the reference's own host sources compiled in this container
 * (oracle/build_ref.sh -> oracle/_ref), through committed fixtures in
 * tests/golden/.  The biome layer chain is pinned the same way against the
 * reference's STPLayer / STPBiomeFactory / demo layer sources.  Noise, the
 * multi-biome blend, the erosion brush, the FP32 serial droplet loop and the
 * format are pinned bit for bit against the reference's own device code
 * compiled as host C++ (oracle/refshim/device, oracle/_ref/libstpref_device.so;
 * fixtures in tests/golden/device_reference.npz).  The splatmap's region
 * maps equal the demo's script and rule lookups compiled the same way; its
 * texture reads and rnormf restate the texture unit and the math function
 * (the same stand-ins serve the compiled script).
 *
 * Build: g++ -O2 -std=c++17 -ffp-contract=off -shared -fPIC (oracle/build.py).
 * -ffp-contract=off keeps every float operation separately rounded.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <thread>
#include <utility>
#include <vector>

extern "C" {

typedef struct orc_bin {
	uint16_t Item;
	float Weight;
} orc_bin;

typedef struct orc_raindrop {
	uint64_t Seed;
	uint32_t RainDropCount;
	float Inertia;
	float SedimentCapacityFactor;
	float minSedimentCapacity;
	float initWaterVolume;
	float minWaterVolume;
	float Friction;
	float initSpeed;
	float ErodeSpeed;
	float DepositSpeed;
	float EvaporateSpeed;
	float Gravity;
	uint32_t ErosionBrushRadius;
} orc_raindrop;

typedef struct orc_biome {
	float Scale;
	uint32_t Octave;
	float Persistence;
	float Lacunarity;
	float Depth;
	float Variation;
} orc_biome;

/* ------------------------------------------------------- permutation --
 * STPPermutationGenerator.cpp:40-73: mt19937_64(seed), std::shuffle of
 * 0..255, duplicated to 512 entries; gradient ring of `distribution` unit
 * vectors at angle += 2pi/N (double accumulation) + Offset.
 * Returns 0, 1 for an invalid setting (STPAlgorithmEnvironment.cpp:13-17),
 * or 2 when the reference's loop would have run one extra time (the extra
 * entry is not written). */
int orc_permutation(uint64_t seed, uint32_t distribution, double offset, uint8_t* perm, float* grad) {
	const double two_pi = 2.0 * 3.14159265358979323846264338327950288;
	if (distribution == 0u || !(offset >= 0.0) || !(offset < two_pi)) {
		return 1;
	}
	std::mt19937_64 rng(seed);
	for (int i = 0; i < 256; i++) {
		perm[i] = static_cast<uint8_t>(i);
	}
	std::shuffle(perm, perm + 256, rng);
	std::memcpy(perm + 256, perm, 256);

	const double step = two_pi / (distribution * 1.0);
	uint32_t counter = 0u;
	for (double angle = 0.0; angle < two_pi; angle += step, counter++) {
		if (counter < distribution) {
			grad[counter * 2u] = static_cast<float>(std::cos(angle + offset));
			grad[counter * 2u + 1u] = static_cast<float>(std::sin(angle + offset));
		}
	}
	return counter > distribution ? 2 : 0;
}

/* ------------------------------------------- single histogram filter --
 * STPSingleHistogramFilter.cpp:400-450 (accumulator), :483-506 (copy and
 * normalise), :522-563 (vertical pass), :608-679 (horizontal pass),
 * :870-902 (checks and ranges).  Restated with std containers; the order of
 * bins is the accumulator's insertion order with erase-compaction. */
namespace {

struct Acc {
	std::vector<uint32_t> slot; // item -> index in bins, or ~0u
	std::vector<std::pair<uint16_t, uint32_t>> bins;

	void clear() {
		for (const auto& b : bins) {
			slot[b.first] = ~0u;
		}
		bins.clear();
	}
	void add(uint16_t item, uint32_t count) {
		if (slot.size() <= item) {
			slot.resize(static_cast<size_t>(item) + 1u, ~0u);
		}
		uint32_t& s = slot[item];
		if (s == ~0u) {
			bins.emplace_back(item, count);
			s = static_cast<uint32_t>(bins.size() - 1u);
		} else {
			bins[s].second += count;
		}
	}
	void sub(uint16_t item, uint32_t count) {
		uint32_t& s = slot[item];
		uint32_t& q = bins[s].second;
		if (q <= count) {
			bins.erase(bins.begin() + s);
			for (size_t k = s; k < bins.size(); k++) {
				slot[bins[k].first]--;
			}
			s = ~0u;
		} else {
			q -= count;
		}
	}
};

} // namespace

/* Returns 0 ok, 1 domain error (radius), 5 capacity too small (nbins_out = needed). */
int orc_shf(const uint16_t* samplemap, uint32_t map_x, uint32_t map_y, uint32_t nn_x, uint32_t nn_y,
	uint32_t radius, uint32_t* offsets, orc_bin* bins, uint64_t bins_capacity, uint64_t* nbins_out) {
	const uint32_t sx = map_x * (nn_x / 2u), sy = map_y * (nn_y / 2u);
	if (!(radius > 0u && (radius & 1u) == 0u) || radius > sx || radius > sy) {
		return 1;
	}
	const uint32_t total_x = map_x * nn_x;
	const uint32_t ncols = map_x + 2u * radius;
	const int r = static_cast<int>(radius);

	// vertical pass, column-major output (column k, row y) -> k * map_y + y
	std::vector<std::vector<std::pair<uint16_t, uint32_t>>> vert(static_cast<size_t>(ncols) * map_y);
	Acc acc;
	for (uint32_t k = 0u; k < ncols; k++) {
		const uint32_t c = sx - radius + k;
		acc.clear();
		for (int j = -r; j <= r; j++) {
			acc.add(samplemap[static_cast<size_t>(sy + j) * total_x + c], 1u);
		}
		vert[static_cast<size_t>(k) * map_y] = acc.bins;
		for (uint32_t y = 1u; y < map_y; y++) {
			acc.add(samplemap[static_cast<size_t>(sy + y + radius) * total_x + c], 1u);
			acc.sub(samplemap[static_cast<size_t>(sy + y - 1u - radius) * total_x + c], 1u);
			vert[static_cast<size_t>(k) * map_y + y] = acc.bins;
		}
	}

	// horizontal pass, row-major output
	uint64_t n = 0u;
	bool fits = true;
	auto emit = [&](uint32_t pixel) {
		offsets[pixel] = static_cast<uint32_t>(n);
		uint32_t sum = 0u;
		for (const auto& b : acc.bins) {
			sum += b.second;
		}
		const float norm = 1.0f / static_cast<float>(sum);
		for (const auto& b : acc.bins) {
			if (n < bins_capacity) {
				bins[n].Item = b.first;
				bins[n].Weight = static_cast<float>(b.second) * norm;
			} else {
				fits = false;
			}
			n++;
		}
	};
	for (uint32_t y = 0u; y < map_y; y++) {
		acc.clear();
		for (uint32_t k = 0u; k <= 2u * radius; k++) {
			for (const auto& b : vert[static_cast<size_t>(k) * map_y + y]) {
				acc.add(b.first, b.second);
			}
		}
		emit(y * map_x);
		for (uint32_t x = 1u; x < map_x; x++) {
			for (const auto& b : vert[static_cast<size_t>(x + 2u * radius) * map_y + y]) {
				acc.add(b.first, b.second);
			}
			for (const auto& b : vert[static_cast<size_t>(x - 1u) * map_y + y]) {
				acc.sub(b.first, b.second);
			}
			emit(y * map_x + x);
		}
	}
	offsets[static_cast<size_t>(map_x) * map_y] = static_cast<uint32_t>(n);
	*nbins_out = n;
	return fits ? 0 : 5;
}

/* -------------------------------------------------------------- noise --
 * STPSimplexNoise.cu:5-16 (constants, floori), :18-82 (simplex2D),
 * :84-110 (simplex2DFractal); STPMultiHeightGenerator.cu:35-72 (per-pixel
 * blend over histogram bins). Float arithmetic, no contraction. */
static const float kF2 = 0.3660254038f;
static const float kG2 = 0.2113248654f;
static const float kH2 = -1.0f + 2.0f * kG2;

static inline int floori(const float x) {
	return x > 0.0f ? static_cast<int>(x) : static_cast<int>(x - 1.0f);
}

static float simplex2d(const uint8_t* perm, const float* grad, uint32_t grad_size, const float x, const float y) {
	float corner[3], dx[3], dy[3], w[3];
	const float s = (x + y) * kF2;
	const int i = floori(x + s), j = floori(y + s);
	const float t = (i + j) * kG2, X0 = i - t, Y0 = j - t;
	dx[0] = x - X0;
	dy[0] = y - Y0;
	const unsigned int i1 = (dx[0] > dy[0]) ? 1u : 0u, j1 = 1u - i1;
	dx[1] = dx[0] - i1 + kG2;
	dy[1] = dy[0] - j1 + kG2;
	dx[2] = dx[0] + kH2;
	dy[2] = dy[0] + kH2;
	const unsigned int ii = static_cast<unsigned int>(i) & 255u, jj = static_cast<unsigned int>(j) & 255u;
	unsigned int g[3];
	g[0] = perm[ii + perm[jj]] % grad_size;
	g[1] = perm[ii + i1 + perm[jj + j1]] % grad_size;
	g[2] = perm[ii + 1u + perm[jj + 1u]] % grad_size;
	for (int v = 0; v < 3; v++) {
		w[v] = 0.5f - dx[v] * dx[v] - dy[v] * dy[v];
		if (w[v] <= 0.0f) {
			corner[v] = 0.0f;
		} else {
			w[v] *= w[v];
			corner[v] = w[v] * w[v] * (grad[g[v] * 2u] * dx[v] + grad[g[v] * 2u + 1u] * dy[v]);
		}
	}
	return 70.0f * (corner[0] + corner[1] + corner[2]);
}

static inline float saturatef(const float v) {
	// __saturatef: clamp to [0,1], NaN -> 0
	if (!(v > 0.0f)) {
		return 0.0f;
	}
	return v > 1.0f ? 1.0f : v;
}

float orc_simplex2d(const uint8_t* perm, const float* grad, uint32_t grad_size, float x, float y) {
	return simplex2d(perm, grad, grad_size, x, y);
}

float orc_fractal(const uint8_t* perm, const float* grad, uint32_t grad_size, float x, float y,
	float pers, float lacu, uint32_t oct, float scale, float off_x, float off_y, float half_x, float half_y) {
	float fractal = 0.0f, amplitude = 1.0f, frequency = 1.0f, range = 0.0f;
	for (uint32_t i = 0u; i < oct; i++) {
		const float sx = ((x - half_x) + off_x) / scale * frequency, sy = ((y - half_y) + off_y) / scale * frequency;
		fractal += simplex2d(perm, grad, grad_size, sx, sy) * amplitude;
		range += amplitude;
		amplitude *= pers;
		frequency *= lacu;
	}
	return saturatef((fractal + range) / (2.0f * range));
}

/* Heightmap of one MapSize chunk from its histogram (offsets/bins), rows
 * [row_begin, row_end). */
static void multibiome_rows(float* out, const uint32_t* offsets, const orc_bin* bins, const orc_biome* table,
	const uint8_t* perm, const float* grad, uint32_t grad_size, uint32_t map_x, uint32_t map_y,
	float off_x, float off_y, uint32_t row_begin, uint32_t row_end) {
	const float half_x = static_cast<float>(map_x) / 2.0f, half_y = static_cast<float>(map_y) / 2.0f;
	for (uint32_t y = row_begin; y < row_end; y++) {
		for (uint32_t x = 0u; x < map_x; x++) {
			const uint32_t idx = x + y * map_x;
			float h = 0.0f;
			for (uint32_t b = offsets[idx]; b < offsets[idx + 1u]; b++) {
				const orc_biome& p = table[bins[b].Item];
				const float f = orc_fractal(perm, grad, grad_size, 1.0f * x, 1.0f * y, p.Persistence, p.Lacunarity,
					p.Octave, p.Scale, off_x, off_y, half_x, half_y);
				h += bins[b].Weight * (f * p.Variation + p.Depth);
			}
			out[idx] = h;
		}
	}
}

/* `threads` <= 1: serial; otherwise rows split over std::threads. */
void orc_multibiome(float* out, const uint32_t* offsets, const orc_bin* bins, const orc_biome* table,
	const uint8_t* perm, const float* grad, uint32_t grad_size, uint32_t map_x, uint32_t map_y,
	float off_x, float off_y, int threads) {
	if (threads <= 1) {
		multibiome_rows(out, offsets, bins, table, perm, grad, grad_size, map_x, map_y, off_x, off_y, 0u, map_y);
		return;
	}
	std::vector<std::thread> pool;
	for (int t = 0; t < threads; t++) {
		const uint32_t b = static_cast<uint32_t>(static_cast<uint64_t>(map_y) * t / threads),
			e = static_cast<uint32_t>(static_cast<uint64_t>(map_y) * (t + 1) / threads);
		pool.emplace_back(multibiome_rows, out, offsets, bins, table, perm, grad, grad_size, map_x, map_y,
			off_x, off_y, b, e);
	}
	for (auto& th : pool) {
		th.join();
	}
}

/* -------------------------------------------------------------- brush --
 * STPHeightfieldGenerator.cpp:44-77: every (dx,dy) with dx^2+dy^2 < r^2 in
 * y-major order, weight 1 - sqrt(d2)/r (double), normalised by 1/sum in
 * double and cast to float; index dy*dimX + dx. Returns the brush size. */
uint32_t orc_brush(uint32_t dim_x, uint32_t radius, int32_t* index, float* weight) {
	const int r = static_cast<int>(radius), r2 = r * r;
	double sum = 0.0;
	std::vector<float> w;
	uint32_t n = 0u;
	for (int by = -r; by <= r; by++) {
		for (int bx = -r; bx <= r; bx++) {
			const double d2 = static_cast<double>(bx * bx + by * by);
			if (d2 < r2) {
				const double cw = 1.0 - std::sqrt(d2) / r;
				sum += cw;
				index[n] = by * static_cast<int>(dim_x) + bx;
				w.push_back(static_cast<float>(cw));
				n++;
			}
		}
	}
	const double f = 1.0 / sum;
	for (uint32_t k = 0u; k < n; k++) {
		weight[k] = static_cast<float>(w[k] * f);
	}
	return n;
}

/* ------------------------------------------------------------ erosion --
 * STPRainDrop.cu:23-51 (bilinear height + gradient), :53-165 (droplet
 * loop), STPHeightfieldKernel.cu:93-107 (spawn in the central chunk, here
 * from an explicit start array). Serial droplets in index order. glm::mix
 * is taken as x*(1-a) + y*a and glm::length as sqrt(dot). T = double gives
 * the FP64 oracle, T = float the FP32 serial baseline. */
} // extern "C"

template<typename T>
static double erode_serial(T* map, uint32_t dim_x, uint32_t dim_y, const orc_raindrop& s, const float* starts,
	uint32_t count, const int32_t* bidx, const float* bw, uint32_t bsize, uint64_t* steps_out) {
	double residual = 0.0;
	uint64_t steps = 0u;
	const T one = static_cast<T>(1);
	const T zero = static_cast<T>(0);
	auto calc = [&](T px, T py, T& h, T& gx, T& gy) {
		const uint32_t rx = static_cast<uint32_t>(px), ry = static_cast<uint32_t>(py);
		const T cx = px - static_cast<T>(rx), cy = py - static_cast<T>(ry);
		const size_t base = static_cast<size_t>(ry) * dim_x + rx;
		const T h00 = map[base], h10 = map[base + 1u], h01 = map[base + dim_x], h11 = map[base + dim_x + 1u];
		h = h00 * (one - cx) * (one - cy) + h10 * cx * (one - cy) + h01 * (one - cx) * cy + h11 * cx * cy;
		gx = (h10 - h00) * (one - cy) + (h11 - h01) * cy;
		gy = (h01 - h00) * (one - cx) + (h11 - h10) * cx;
	};
	const T brush_r = static_cast<T>(s.ErosionBrushRadius);
	const T lim_x = static_cast<T>(1.0f * dim_x - s.ErosionBrushRadius);
	const T lim_y = static_cast<T>(1.0f * dim_y - s.ErosionBrushRadius);
	for (uint32_t d = 0u; d < count; d++) {
		T px = starts[2u * d], py = starts[2u * d + 1u];
		T dirx = zero, diry = zero;
		// the water volume drives the loop test, so it stays in float as on the
		// device (the lifetime set through minWaterVolume is a float sequence)
		float volf = s.initWaterVolume;
		T speed = s.initSpeed, sed = zero;
		// a start whose 2x2 bilinear footprint is outside the map dies at once
		if (!(starts[2u * d] >= 0.0f && starts[2u * d] < dim_x - 1.0f && starts[2u * d + 1u] >= 0.0f
				&& starts[2u * d + 1u] < dim_y - 1.0f)) {
			volf = 0.0f;
		}
		while (volf >= s.minWaterVolume) {
			const T vol = static_cast<T>(volf);
			steps++;
			const size_t mi = static_cast<size_t>(static_cast<uint32_t>(py)) * dim_x + static_cast<uint32_t>(px);
			const T ox = px - static_cast<T>(static_cast<int>(px)), oy = py - static_cast<T>(static_cast<int>(py));
			T h, gx, gy;
			calc(px, py, h, gx, gy);
			const T inertia = s.Inertia;
			dirx = (-gx) * (one - inertia) + dirx * inertia;
			diry = (-gy) * (one - inertia) + diry * inertia;
			const T len = std::sqrt(dirx * dirx + diry * diry);
			if (len != zero) {
				dirx /= len;
				diry /= len;
			}
			px += dirx;
			py += diry;
			if ((dirx == zero && diry == zero) || !(px >= brush_r && px < lim_x && py >= brush_r && py < lim_y)) {
				residual += static_cast<double>(sed);
				volf = 0.0f;
				sed = zero;
				break;
			}
			T h2, g2x, g2y;
			calc(px, py, h2, g2x, g2y);
			const T dh = h2 - h;
			const T cap = std::max(-dh * speed * vol * static_cast<T>(s.SedimentCapacityFactor),
				static_cast<T>(s.minSedimentCapacity));
			if (sed > cap || dh > zero) {
				const T dep = (dh > zero) ? std::min(dh, sed) : (sed - cap) * static_cast<T>(s.DepositSpeed);
				sed -= dep;
				map[mi] += dep * (one - ox) * (one - oy);
				map[mi + 1u] += dep * ox * (one - oy);
				map[mi + dim_x] += dep * (one - ox) * oy;
				map[mi + dim_x + 1u] += dep * ox * oy;
			} else {
				const T ero = std::min((cap - sed) * static_cast<T>(s.ErodeSpeed), -dh);
				for (uint32_t b = 0u; b < bsize; b++) {
					const size_t ei = static_cast<size_t>(static_cast<int64_t>(mi) + bidx[b]);
					const T we = ero * static_cast<T>(bw[b]);
					const T ds = (map[ei] < we) ? map[ei] : we;
					map[ei] -= ds;
					sed += ds;
				}
			}
			speed = std::sqrt(std::max(zero, speed * speed + dh * static_cast<T>(s.Gravity)));
			speed *= one - static_cast<T>(s.Friction);
			volf *= 1.0f - s.EvaporateSpeed;
		}
		// a droplet that evaporated takes its sediment with it (zero after a kill)
		residual += static_cast<double>(sed);
	}
	if (steps_out) {
		*steps_out = steps;
	}
	return residual;
}

extern "C" {

/* FP64 serial oracle: `map` is a double array (in/out). */
double orc_erode_f64(double* map, uint32_t dim_x, uint32_t dim_y, const orc_raindrop* s, const float* starts,
	uint32_t count, const int32_t* bidx, const float* bw, uint32_t bsize, uint64_t* steps) {
	return erode_serial<double>(map, dim_x, dim_y, *s, starts, count, bidx, bw, bsize, steps);
}

/* FP32 serial restatement (CPU baseline). */
double orc_erode_f32(float* map, uint32_t dim_x, uint32_t dim_y, const orc_raindrop* s, const float* starts,
	uint32_t count, const int32_t* bidx, const float* bw, uint32_t bsize, uint64_t* steps) {
	return erode_serial<float>(map, dim_x, dim_y, *s, starts, count, bidx, bw, bsize, steps);
}

/* STPHeightfieldKernel.cu:112-122. */
void orc_format(const float* in, uint16_t* out, uint64_t n) {
	for (uint64_t i = 0u; i < n; i++) {
		out[i] = static_cast<uint16_t>(std::rint(saturatef(in[i]) * 65535));
	}
}

/* ----------------------------------------------------- synthetic inputs --
 * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
 * easy as 1, 2, 3", SC'11): 10 rounds of the 4x32 S-box with multipliers
 * 0xD2511F53 / 0xCD9E8D57 and Weyl key increments 0x9E3779B9 / 0xBB67AE85. */
static void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
	for (int round = 0; round < 10; round++) {
		const uint64_t p0 = static_cast<uint64_t>(0xD2511F53u) * c[0];
		const uint64_t p1 = static_cast<uint64_t>(0xCD9E8D57u) * c[2];
		const uint32_t hi0 = static_cast<uint32_t>(p0 >> 32), lo0 = static_cast<uint32_t>(p0);
		const uint32_t hi1 = static_cast<uint32_t>(p1 >> 32), lo1 = static_cast<uint32_t>(p1);
		const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
		c[0] = n0;
		c[1] = lo1;
		c[2] = n2;
		c[3] = lo0;
		k0 += 0x9E3779B9u;
		k1 += 0xBB67AE85u;
	}
}

/* u32 -> float in (0, 1]: ((x >> 8) + 1) * 2^-24, exact. */
static inline float unit_open_closed(uint32_t x) {
	return static_cast<float>((x >> 8) + 1u) * (1.0f / 16777216.0f);
}

/* Droplet starts: u in (0,1]^2 * (MapSize-1) + (NN/2)*MapSize, as
 * STPHeightfieldKernel.cu:93-104 maps its two uniforms. */
void orc_droplet_starts(float* xy, uint32_t count, uint64_t seed, uint64_t counter_base, uint32_t map_x,
	uint32_t map_y, uint32_t nn_x, uint32_t nn_y) {
	const float base_x = static_cast<float>(map_x - 1u), base_y = static_cast<float>(map_y - 1u);
	const float range_x = static_cast<float>((nn_x / 2u) * map_x), range_y = static_cast<float>((nn_y / 2u) * map_y);
	for (uint32_t i = 0u; i < count; i++) {
		const uint64_t ctr = counter_base + i;
		uint32_t c[4] = { static_cast<uint32_t>(ctr), static_cast<uint32_t>(ctr >> 32), 0u, 0u };
		philox4x32_10(c, static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
		float x = unit_open_closed(c[0]), y = unit_open_closed(c[1]);
		x *= base_x;
		y *= base_y;
		x += range_x;
		y += range_y;
		xy[2u * i] = x;
		xy[2u * i + 1u] = y;
	}
}

static inline uint64_t splitmix64(uint64_t z) {
	z += 0x9E3779B97F4A7C15ull;
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

static inline int64_t floordiv(int64_t a, int64_t b) {
	const int64_t q = a / b;
	return (a % b != 0 && ((a < 0) != (b < 0))) ? q - 1 : q;
}

/* Seeded Voronoi biome map (see stpgb_voronoi_biomemap). */
void orc_voronoi(uint16_t* out, uint32_t pitch, uint32_t width, uint32_t height, int64_t origin_x, int64_t origin_y,
	uint32_t cell, uint32_t biome_count, uint64_t seed) {
	for (uint32_t y = 0u; y < height; y++) {
		for (uint32_t x = 0u; x < width; x++) {
			const int64_t gx = origin_x + x, gy = origin_y + y;
			const int64_t cx = floordiv(gx, cell), cy = floordiv(gy, cell);
			int64_t best = INT64_MAX;
			uint64_t best_h = 0u;
			for (int dy = -1; dy <= 1; dy++) {
				for (int dx = -1; dx <= 1; dx++) {
					const int64_t nx = cx + dx, ny = cy + dy;
					const uint64_t h = splitmix64(seed ^ splitmix64(static_cast<uint64_t>(nx) * 0x9E3779B97F4A7C15ull
						^ static_cast<uint64_t>(ny) * 0xC2B2AE3D27D4EB4Full));
					const int64_t px = nx * cell + static_cast<int64_t>(h % cell),
						py = ny * cell + static_cast<int64_t>((h >> 32) % cell);
					const int64_t d = (px - gx) * (px - gx) + (py - gy) * (py - gy);
					if (d < best) {
						best = d;
						best_h = h;
					}
				}
			}
			out[static_cast<size_t>(y) * pitch + x] = static_cast<uint16_t>(splitmix64(best_h) % biome_count);
		}
	}
}

} // extern "C"

/* ------------------------------------------------------------------------
 * Biome layer chain: STPBiomeFactory::operator() over a linear chain of the
 * demo's layers, evaluated per pixel by recursion with one exact memo table
 * per layer (the reference's per-layer hash cache is pure memoisation).
 *   local RNG and seeding:  SuperTerrain+/Private/World/Diversity/STPLayer.cpp:96-160
 *   factory loop:           SuperTerrain+/Private/World/Diversity/STPBiomeFactory.cpp:24-41
 *   layers:                 SuperDemo+/World/Layers/STP{Continent,Scale,Land,Island,Voronoi}Layer.h,
 *                           STP{Cross,XCross}Layer.h
 * Kinds: 1 continent, 2 scale (param 0 normal, 1 fuzzy), 3 land, 4 island,
 * 5 voronoi (2-D).  ids = {ocean, plains, forest, shallow ocean x5}.
 * ------------------------------------------------------------------------ */
#include <unordered_map>

namespace {

inline uint64_t lcg_mix(uint64_t s, uint64_t fac) {
	// STPLayer::mixSeed: s *= s * A + B; s += fac (64-bit wrap-around)
	return s * (s * 6364136223846793005ull + 1442695040888963407ull) + fac;
}

inline uint64_t sext(int v) {
	return static_cast<uint64_t>(static_cast<int64_t>(v));
}

uint64_t layer_seed_of(uint64_t global, uint64_t salt) {
	uint64_t mid = salt;
	for (int i = 0; i < 3; i++) {
		mid = lcg_mix(mid, mid);
	}
	uint64_t s = global;
	for (int i = 0; i < 3; i++) {
		s = lcg_mix(s, mid);
	}
	return s;
}

uint64_t local_seed_of(uint64_t layer_seed, int x, int z) {
	uint64_t s = lcg_mix(layer_seed, sext(x));
	s = lcg_mix(s, sext(z));
	s = lcg_mix(s, sext(x));
	return lcg_mix(s, sext(z));
}

struct LocalRng {
	uint64_t state, layer;
	uint16_t next(uint32_t range) {
		const uint16_t v = static_cast<uint16_t>((state >> 24) % range);
		state = lcg_mix(state, layer);
		return v;
	}
};

struct OrcLayerDesc {
	uint32_t kind, param;
	uint64_t salt;
};

class LayerChainOracle {
public:
	LayerChainOracle(const OrcLayerDesc* chain, uint32_t count, uint64_t global, const uint16_t* ids) :
		desc(chain, chain + count), seed(count), memo(count), voronoi_seed(global) {
		for (uint32_t i = 0; i < count; i++) {
			seed[i] = layer_seed_of(global, chain[i].salt);
		}
		ocean = ids[0];
		plains = ids[1];
		forest = ids[2];
		std::copy(ids + 3, ids + 8, shallow);
	}

	uint16_t get(int layer, int x, int z) {
		if (layer + 1 == static_cast<int>(desc.size())) {
			return eval(layer, x, z);
		}
		const uint64_t key = (static_cast<uint64_t>(static_cast<uint32_t>(x)) << 32) | static_cast<uint32_t>(z);
		auto& m = memo[layer];
		const auto it = m.find(key);
		if (it != m.end()) {
			return it->second;
		}
		const uint16_t v = eval(layer, x, z);
		m.emplace(key, v);
		return v;
	}

private:
	std::vector<OrcLayerDesc> desc;
	std::vector<uint64_t> seed;
	std::vector<std::unordered_map<uint64_t, uint16_t>> memo;
	uint64_t voronoi_seed;
	uint16_t ocean, plains, forest, shallow[5];

	bool so(uint16_t v) const {
		for (uint16_t s : shallow) {
			if (v == s) {
				return true;
			}
		}
		return false;
	}

	LocalRng rng(int layer, int x, int z) const {
		return LocalRng { local_seed_of(seed[layer], x, z), seed[layer] };
	}

	uint16_t eval(int layer, int x, int z) {
		const int up = layer - 1;
		switch (desc[layer].kind) {
		case 1: {
			LocalRng r = rng(layer, x, z);
			return r.next(10u) == 0u ? plains : ocean;
		}
		case 2: {
			const uint16_t c = get(up, x >> 1, z >> 1);
			LocalRng r = rng(layer, x & -2, z & -2);
			const int odd_x = x & 1, odd_z = z & 1;
			if (!odd_x && !odd_z) {
				return c;
			}
			const uint16_t below = get(up, x >> 1, (z + 1) >> 1);
			const uint16_t pick_z = r.next(2u) == 0u ? c : below;
			if (!odd_x) {
				return pick_z;
			}
			const uint16_t right = get(up, (x + 1) >> 1, z >> 1);
			const uint16_t pick_x = r.next(2u) == 0u ? c : right;
			if (!odd_z) {
				return pick_x;
			}
			const uint16_t diag = get(up, (x + 1) >> 1, (z + 1) >> 1);
			return scale_corner(c, right, below, diag, r, desc[layer].param != 0u);
		}
		case 3: {
			const uint16_t c = get(up, x, z), ne = get(up, x + 1, z - 1), se = get(up, x + 1, z + 1),
				sw = get(up, x - 1, z + 1), nw = get(up, x - 1, z - 1);
			LocalRng r = rng(layer, x, z);
			const bool all_so = so(sw) && so(se) && so(ne) && so(nw);
			const bool none_so = !so(sw) && !so(se) && !so(ne) && !so(nw);
			if (!so(c) || all_so) {
				if (so(c) || none_so || r.next(5u) != 0u) {
					return c;
				}
				const uint16_t order[4] = { nw, sw, ne, se };
				for (uint16_t n : order) {
					if (so(n)) {
						return c == forest ? forest : n;
					}
				}
				return c;
			}
			uint32_t tries = 1u;
			uint16_t chosen = 1u;
			const uint16_t order[4] = { nw, ne, sw, se };
			for (int k = 0; k < 4; k++) {
				if (!so(order[k])) {
					const uint32_t range = tries;
					if (k < 3) {
						tries++;
					}
					if (r.next(range) == 0u) {
						chosen = order[k];
					}
				}
			}
			if (r.next(3u) == 0u) {
				return chosen;
			}
			return chosen == forest ? forest : c;
		}
		case 4: {
			const uint16_t c = get(up, x, z), n = get(up, x, z - 1), e = get(up, x + 1, z), s = get(up, x, z + 1),
				w = get(up, x - 1, z);
			LocalRng r = rng(layer, x, z);
			return so(c) && so(n) && so(e) && so(s) && so(w) && r.next(2u) == 0u ? plains : c;
		}
		case 5:
			return voronoi(up, x, z);
		default:
			return 0u;
		}
	}

	static uint16_t scale_corner(uint16_t c, uint16_t e, uint16_t s, uint16_t se, LocalRng& r, bool fuzzy) {
		const uint32_t k = r.next(4u);
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

	static double jitter(uint64_t h) {
		const double u = static_cast<double>(static_cast<uint32_t>((h >> 24) % 1024u)) / 1024.0;
		return (u - 0.5) * 0.9;
	}

	// Squared distance from the pixel to the jittered point of cell (cx,cy,cz),
	// summed z, y, x as the reference does (STPVoronoiLayer.h sqrtDist).
	double cell_distance(int cx, int cy, int cz, double fx, double fy, double fz) const {
		uint64_t h = voronoi_seed;
		const int axis[6] = { cx, cy, cz, cx, cy, cz };
		for (int a : axis) {
			h = lcg_mix(h, sext(a));
		}
		const double jx = jitter(h);
		h = lcg_mix(h, voronoi_seed);
		const double jy = jitter(h);
		h = lcg_mix(h, voronoi_seed);
		const double jz = jitter(h);
		const double tz = fz + jz, ty = fy + jy, tx = fx + jx;
		return tz * tz + ty * ty + tx * tx;
	}

	uint16_t voronoi(int up, int x, int z) {
		const int bx = x - 2, by = -2, bz = z - 2;
		const int cx = bx >> 2, cy = by >> 2, cz = bz >> 2;
		const double fx = (bx & 3) / 4.0, fy = (by & 3) / 4.0, fz = (bz & 3) / 4.0;
		int best = 0;
		double best_d = 0.0;
		for (int c = 0; c < 8; c++) {
			const int hx = (c >> 2) & 1, hy = (c >> 1) & 1, hz = c & 1;
			const double d = cell_distance(cx + hx, cy + hy, cz + hz, fx - hx, fy - hy, fz - hz);
			if (c == 0 || d < best_d) {
				best = c;
				best_d = d;
			}
		}
		return get(up, cx + ((best >> 2) & 1), cz + (best & 1));
	}
};

} // namespace

extern "C" {

uint64_t orc_mix_seed(uint64_t s, int64_t fac) {
	return lcg_mix(s, static_cast<uint64_t>(fac));
}

uint64_t orc_layer_seed(uint64_t global, uint64_t salt) {
	return layer_seed_of(global, salt);
}

uint64_t orc_local_seed(uint64_t global, uint64_t salt, int32_t x, int32_t z) {
	return local_seed_of(layer_seed_of(global, salt), x, z);
}

/* chain: count x {uint32 kind, uint32 param, uint64 salt}, first ancestor
 * first; ids: ocean, plains, forest, shallow ocean x5.  Writes
 * out[z * width + x] for the world rectangle starting at (offset_x, offset_z). */
void orc_layer_biomemap(const void* chain, uint32_t count, uint64_t global_seed, const uint16_t* ids, uint16_t* out,
	uint32_t width, uint32_t height, int32_t offset_x, int32_t offset_z) {
	LayerChainOracle o(static_cast<const OrcLayerDesc*>(chain), count, global_seed, ids);
	for (uint32_t z = 0u; z < height; z++) {
		for (uint32_t x = 0u; x < width; x++) {
			out[static_cast<size_t>(z) * width + x] = o.get(static_cast<int>(count) - 1,
				static_cast<int>(x) + offset_x, static_cast<int>(z) + offset_z);
		}
	}
}

} // extern "C"

/* ------------------------------------------------------------------------
 * Texture splatmap (SuperDemo+/Script/STPSplatmapGenerator.cu:56-128, rule
 * lookups SuperTerrain+/SuperAlgorithm+/Device/Private/
 * STPTextureSplatRuleWrapper.cu:55-126).  The texture reads follow the
 * sampler the reference configures (STPWorldPipeline.cpp:682-696):
 * unnormalised coordinates, clamped addressing; linear filtering blends
 * texels floor(u - 0.5) and the next one with weight frac(u - 0.5) in
 * 1/256 steps; point filtering takes texel floor(u).  For a uint16 texture
 * read as normalised float, the GB300 texture unit forms the weighted sum of
 * the integer texels exactly, rounds it to the nearest integer q with halves
 * up, and returns float(q) / 65535 correctly rounded: measured bit for bit on
 * 26,880 samples at the positions this kernel uses (weights 0 and 1/2).
 * rnormf(3, g) is 1 / |g| rounded from double (CUDA's may differ by an ulp).
 * ------------------------------------------------------------------------ */
namespace {

struct OrcSplatRegistry {
	uint32_t AltitudeEntry, AltitudeSize, GradientEntry, GradientSize;
};
struct OrcAltitudeNode {
	uint32_t RegionIndex;
	float UpperBound;
};
struct OrcGradientNode {
	uint32_t RegionIndex;
	float minGradient, maxGradient, LowerBound, UpperBound;
};
struct OrcSplatChunk {
	uint32_t lx, ly;
	float off_x, off_y;
};

int64_t texel(const uint16_t* m, uint32_t pitch, uint32_t w, uint32_t h, int x, int y) {
	x = std::min(std::max(x, 0), static_cast<int>(w) - 1);
	y = std::min(std::max(y, 0), static_cast<int>(h) - 1);
	return m[static_cast<size_t>(y) * pitch + x];
}

float tex_linear(const uint16_t* m, uint32_t pitch, uint32_t w, uint32_t h, float u, float v) {
	const float xb = u - 0.5f, yb = v - 0.5f;
	const float x0 = std::floor(xb), y0 = std::floor(yb);
	const int64_t a = std::lround((xb - x0) * 256.0f), b = std::lround((yb - y0) * 256.0f);
	const int i = static_cast<int>(x0), j = static_cast<int>(y0);
	const int64_t sum = (256 - a) * (256 - b) * texel(m, pitch, w, h, i, j)
		+ a * (256 - b) * texel(m, pitch, w, h, i + 1, j) + (256 - a) * b * texel(m, pitch, w, h, i, j + 1)
		+ a * b * texel(m, pitch, w, h, i + 1, j + 1);
	const int64_t q = (sum + 32768) >> 16;
	return static_cast<float>(q) / 65535.0f;
}

} // namespace

extern "C" {

/* Region map of `count` chunks of a width x height rendering buffer; rules
 * as the generator lays them out (dictionary of `dict_count` sorted samples,
 * one registry per sample, altitude and gradient node arrays).  slope and
 * altitude (may be NULL) receive the tested values. */
void orc_splatmap(const uint16_t* biomemap, const uint16_t* heightmap, uint32_t map_pitch, uint32_t width,
	uint32_t height, const void* chunks_v, uint32_t count, uint32_t map_x, uint32_t map_y, const uint16_t* dict,
	uint32_t dict_count, const void* reg_v, const void* alt_v, const void* gra_v, const uint8_t* perm,
	const float* grad, uint32_t grad_size, uint8_t* out, uint32_t out_pitch, float* slope_out, float* alt_out) {
	const auto* chunks = static_cast<const OrcSplatChunk*>(chunks_v);
	const auto* reg = static_cast<const OrcSplatRegistry*>(reg_v);
	const auto* altn = static_cast<const OrcAltitudeNode*>(alt_v);
	const auto* gran = static_cast<const OrcGradientNode*>(gra_v);
	const float half_x = static_cast<float>(map_x) / 2.0f, half_y = static_cast<float>(map_y) / 2.0f;
	for (uint32_t c = 0u; c < count; c++) {
		for (uint32_t y = 0u; y < map_y; y++) {
			for (uint32_t x = 0u; x < map_x; x++) {
				const uint32_t sx = x + map_x * chunks[c].lx, sy = y + map_y * chunks[c].ly;
				const float fx = static_cast<float>(sx), fy = static_cast<float>(sy);
				const float top = tex_linear(heightmap, map_pitch, width, height, fx, fy - 2.5f) * 875.5f;
				const float left = tex_linear(heightmap, map_pitch, width, height, fx - 2.5f, fy) * 875.5f;
				const float right = tex_linear(heightmap, map_pitch, width, height, fx + 2.5f, fy) * 875.5f;
				const float bottom = tex_linear(heightmap, map_pitch, width, height, fx, fy + 2.5f) * 875.5f;
				const double g0 = top - bottom, g1 = 5.5, g2 = left - right;
				const float rn = static_cast<float>(1.0 / std::sqrt(g0 * g0 + g1 * g1 + g2 * g2));
				const float slope = 1.0f - 5.5f * rn;
				const float noise = orc_fractal(perm, grad, grad_size, 1.0f * x, 1.0f * y, 0.7f, 1.88f, 3u, 91.5f,
					chunks[c].off_x, chunks[c].off_y, half_x, half_y) * 0.15f;
				const int bx = std::min(static_cast<int>(sx), static_cast<int>(width) - 1),
					by = std::min(static_cast<int>(sy), static_cast<int>(height) - 1);
				const uint16_t biome = biomemap[static_cast<size_t>(by) * map_pitch + bx];
				const float alt = saturatef(tex_linear(heightmap, map_pitch, width, height, fx, fy) + noise);
				// findSplatRegistry: lower bound; a missing sample takes the next larger one's registry
				const uint32_t d = static_cast<uint32_t>(std::lower_bound(dict, dict + dict_count, biome) - dict);
				uint32_t region = 0xFFFFFFFFu;
				if (d < dict_count) {
					const OrcSplatRegistry& r = reg[d];
					for (uint32_t i = r.GradientEntry; i < r.GradientEntry + r.GradientSize; i++) {
						const OrcGradientNode& n = gran[i];
						if (slope >= n.minGradient && slope <= n.maxGradient && alt >= n.LowerBound && alt <= n.UpperBound) {
							region = n.RegionIndex;
							break;
						}
					}
					if (region == 0xFFFFFFFFu) {
						for (uint32_t i = r.AltitudeEntry; i < r.AltitudeEntry + r.AltitudeSize; i++) {
							if (!(altn[i].UpperBound < alt)) {
								region = altn[i].RegionIndex;
								break;
							}
						}
					}
				}
				const size_t o = static_cast<size_t>(sy) * out_pitch + sx;
				out[o] = static_cast<uint8_t>(region);
				if (slope_out) {
					slope_out[o] = slope;
				}
				if (alt_out) {
					alt_out[o] = alt;
				}
			}
		}
	}
}

} // extern "C"
