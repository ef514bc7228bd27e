// Serving engine: continuous batching of eroded-chunk requests.
//
// The reference's world pipeline (SuperTerrain+/SuperTerrain+/Private/World/
// STPWorldPipeline.cpp:411-662) generates and erodes chunks on demand from a
// pool of host threads, one synchronous call per chunk.  Here a single
// scheduler thread owns the GPU work:
//
//   * admission: a request is admitted while fewer than MaxInFlight are in
//     flight and its result buffers (merged map, fixed-point map, droplet
//     starts) fit in the device pool -- one allocation of HbmBudget bytes,
//     sub-allocated first-fit on the host;
//   * continuous batching: whenever a stream is free, every admitted request
//     not yet launched (up to MaxBatch) goes into one fixed sequence of
//     batched launches -- Voronoi biome regions and filter + noise for the
//     chunks not yet resident, gather of each request's 3x3 neighbourhood,
//     droplet starts, erosion, formatting -- while earlier sequences are
//     still running on the other streams;
//   * residency: a generated chunk heightfield (before erosion) stays in the
//     pool, keyed by (side, chunk, radius), and serves every later request
//     whose neighbourhood contains it; least recently used chunks that no
//     launched request still needs are evicted when the pool is full.  A
//     request that needs a chunk another sequence is still generating waits
//     for that sequence's event on the device, not on the host;
//   * erosion, private mode (default): each request erodes a private merged
//     copy of its neighbourhood, so its result is the same alone and in a
//     mix (up to the erosion's own run-to-run spread);
//   * erosion, in-place mode (the reference's semantics, STPWorldPipeline.cpp:
//     339-403,485-541,640-662): a request gathers its neighbourhood from the
//     resident chunks, erodes it and scatters it back, so chunks carry their
//     neighbours' erosion; a centre is eroded once; the requests of one
//     sequence run in the reference's priority levels (a centre takes the
//     lowest level none of its neighbourhood's chunks has, smallest level
//     first, one level after another on the stream) and a sequence that
//     touches chunks an earlier sequence still uses waits for it on the
//     device.
#include "erosion.cuh"
#include "noise.cuh"
#include "serve.cuh"
#include "layers.cuh"
#include "shf.cuh"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cmath>
#include <deque>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

using namespace stpgb;

namespace {

using Clock = std::chrono::steady_clock;

size_t al(size_t v) {
	return (v + 255u) & ~static_cast<size_t>(255u);
}

// First-fit sub-allocator over byte offsets [0, size), with coalescing.
class Pool {
public:
	void reset(size_t size) {
		free_.clear();
		free_[0] = size;
		size_ = size;
		used_ = 0u;
	}
	bool alloc(size_t bytes, size_t& off) {
		bytes = al(std::max<size_t>(bytes, 1u));
		for (auto it = free_.begin(); it != free_.end(); ++it) {
			if (it->second >= bytes) {
				off = it->first;
				const size_t rest = it->second - bytes;
				free_.erase(it);
				if (rest) {
					free_[off + bytes] = rest;
				}
				used_ += bytes;
				return true;
			}
		}
		return false;
	}
	void release(size_t off, size_t bytes) {
		bytes = al(std::max<size_t>(bytes, 1u));
		used_ -= bytes;
		auto it = free_.emplace(off, bytes).first;
		auto next = std::next(it);
		if (next != free_.end() && it->first + it->second == next->first) {
			it->second += next->second;
			free_.erase(next);
		}
		if (it != free_.begin()) {
			auto prev = std::prev(it);
			if (prev->first + prev->second == it->first) {
				prev->second += it->second;
				free_.erase(it);
			}
		}
	}
	size_t used() const {
		return used_;
	}

private:
	std::map<size_t, size_t> free_;
	size_t size_ = 0u, used_ = 0u;
};

struct ChunkKey {
	uint32_t S, r;
	int32_t x, y;
	bool operator==(const ChunkKey& o) const {
		return S == o.S && r == o.r && x == o.x && y == o.y;
	}
};

struct ChunkKeyHash {
	size_t operator()(const ChunkKey& k) const {
		uint64_t h = (static_cast<uint64_t>(static_cast<uint32_t>(k.x)) << 32) ^ static_cast<uint32_t>(k.y);
		h ^= (static_cast<uint64_t>(k.S) << 20) ^ (static_cast<uint64_t>(k.r) << 48);
		h *= 0x9E3779B97F4A7C15ull;
		return static_cast<size_t>(h ^ (h >> 29));
	}
};

struct Iteration;

struct Chunk {
	size_t off = 0u;
	bool resident = false;             // generated and complete
	std::shared_ptr<Iteration> maker;  // the sequence generating it, while not resident
	int refs = 0;                      // launched requests still to gather it
	uint64_t last_use = 0u;
	// in-place mode: eroded (or scheduled to be) as a centre, and the last
	// launched sequence that reads or writes the chunk
	bool centre_done = false;
	std::shared_ptr<Iteration> toucher;
};

struct Request {
	uint64_t ticket = 0u;
	stpgb_serve_request req {};
	Clock::time_point submitted;
	size_t off = 0u, bytes = 0u, merged = 0u, fixed = 0u, starts = 0u;
	uint32_t droplets = 0u;
	double latency_ms = 0.0, residual = 0.0;
	int status = STPGB_OK;
	bool complete = false;
	// in-place mode: whether the request erodes (its centre was not yet done),
	// its priority level in its sequence and its place in the erosion order
	bool erode = true;
	uint32_t level = 0u;
	uint64_t order = 0u;
};

struct StreamSlot {
	cudaStream_t stream = nullptr;
	cudaEvent_t done = nullptr;
	bool busy = false;
	// device job tables and their pinned host staging
	unsigned char* dev = nullptr;
	unsigned char* host = nullptr;
	size_t bytes = 0u;
};

struct Iteration {
	int slot = -1;
	std::vector<uint64_t> tickets;
	std::vector<ChunkKey> generated, used;
	size_t scratch_off = 0u, scratch_bytes = 0u;
	double* residual_host = nullptr; // pinned, in the slot's staging area
	uint32_t* status_host = nullptr;
};

constexpr size_t kStagingBytes = 4u << 20;

} // namespace

struct stpgb_server {
	stpgb_server_config cfg {};
	stpgb_raindrop_setting base {};
	uint32_t biome_count = 0u, max_items = 0u;
	// device tables (allocated once at creation)
	uint8_t* perm = nullptr;
	float* grad = nullptr;
	stpgb_permutation permutation {};
	stpgb_biome_property* table = nullptr;
	LayerChain chain {}; // the biome layer chain, when cfg.BiomeSource selects it
	unsigned char* pool_mem = nullptr;
	Pool pool;
	std::vector<StreamSlot> slots;
	// brush tables per (side, radius)
	std::map<std::pair<uint32_t, uint32_t>, std::pair<size_t, uint32_t>> brushes; // -> (pool offset, size)

	std::mutex mu;
	std::condition_variable cv_work, cv_done;
	std::thread worker;
	bool stop = false;
	int fatal = STPGB_OK;
	std::string fatal_msg;

	uint64_t next_ticket = 1u, clock = 0u, erosion_order = 0u;
	std::unordered_map<uint64_t, Request> requests;
	std::deque<uint64_t> pending, admitted;
	std::deque<uint64_t> done;
	std::list<std::shared_ptr<Iteration>> inflight;
	std::unordered_map<ChunkKey, Chunk, ChunkKeyHash> chunks;
	stpgb_server_stats stats {};

	~stpgb_server() {
		{
			std::lock_guard<std::mutex> lk(mu);
			stop = true;
		}
		cv_work.notify_all();
		if (worker.joinable()) {
			worker.join();
		}
		for (auto& s : slots) {
			if (s.stream) {
				cudaStreamSynchronize(s.stream);
				cudaStreamDestroy(s.stream);
			}
			if (s.done) {
				cudaEventDestroy(s.done);
			}
			if (s.dev) {
				cudaFree(s.dev);
			}
			if (s.host) {
				cudaFreeHost(s.host);
			}
		}
		for (void* p : { static_cast<void*>(perm), static_cast<void*>(grad), static_cast<void*>(table),
				 static_cast<void*>(pool_mem) }) {
			if (p) {
				cudaFree(p);
			}
		}
	}

	unsigned char* at(size_t off) const {
		return pool_mem + off;
	}

	uint32_t droplets_of(const stpgb_serve_request& r) const {
		return static_cast<uint32_t>(std::lround(static_cast<double>(r.DropletsPerPixel) * r.MapSize * r.MapSize));
	}

	static size_t request_bytes(uint32_t S, uint32_t droplets) {
		const size_t n = 9u * static_cast<size_t>(S) * S;
		return al(n * sizeof(float)) + al(n * sizeof(uint16_t)) + al(2u * sizeof(float) * droplets);
	}

	size_t generation_bytes(uint32_t S, uint32_t r) const {
		const size_t npix = static_cast<size_t>(S) * S;
		const ShfLayout l = shf_layout(S, S, r, shf_kcap_v(r, max_items));
		const uint64_t cap = npix * std::min<uint64_t>(shf_kcap_h(r, max_items), (2ull * r + 1u) * (2ull * r + 1u));
		return al(9u * npix * sizeof(uint16_t)) + al(l.total) + al((npix + 1u) * sizeof(uint32_t)) + al(cap * sizeof(stpgb_bin));
	}

	// pool allocation, evicting unused resident chunks (least recently used first) when full
	bool alloc_evict(size_t bytes, size_t& off) {
		while (!pool.alloc(bytes, off)) {
			auto victim = chunks.end();
			for (auto it = chunks.begin(); it != chunks.end(); ++it) {
				if (it->second.resident && it->second.refs == 0
					&& (victim == chunks.end() || it->second.last_use < victim->second.last_use)) {
					victim = it;
				}
			}
			if (victim == chunks.end()) {
				return false;
			}
			pool.release(victim->second.off, static_cast<size_t>(victim->first.S) * victim->first.S * sizeof(float));
			chunks.erase(victim);
			stats.ChunksEvicted++;
		}
		return true;
	}

	int brush_for(uint32_t S, uint32_t radius, size_t& off, uint32_t& size) {
		auto it = brushes.find({ S, radius });
		if (it != brushes.end()) {
			off = it->second.first;
			size = it->second.second;
			return STPGB_OK;
		}
		uint32_t bs = 0u;
		stpgb_erosion_brush_generate(3u * S, radius, nullptr, nullptr, 0u, &bs);
		std::vector<int32_t> idx(bs);
		std::vector<float> w(bs);
		STPGB_TRY(stpgb_erosion_brush_generate(3u * S, radius, idx.data(), w.data(), bs, &bs));
		if (!pool.alloc(bs * 8u, off)) {
			set_error("stpgb_server: no pool room for an erosion brush");
			return STPGB_ENOMEM;
		}
		STPGB_CUDA_TRY(cudaMemcpy(at(off), idx.data(), bs * sizeof(int32_t), cudaMemcpyHostToDevice));
		STPGB_CUDA_TRY(cudaMemcpy(at(off) + bs * sizeof(int32_t), w.data(), bs * sizeof(float), cudaMemcpyHostToDevice));
		brushes[{ S, radius }] = { off, bs };
		size = bs;
		return STPGB_OK;
	}

	bool in_place() const {
		return cfg.ErosionMode == STPGB_EROSION_IN_PLACE;
	}

	// checks a submitted request and fills its sizes (no lock needed)
	int prepare(const stpgb_serve_request& q, Request& r) const;

	// The reference's erosion schedule (STPWorldPipeline.cpp:339-403) over the
	// eroding requests of one sequence, in admission order: a centre whose
	// neighbourhood holds no scheduled chunk takes level 1; otherwise the
	// level below the smallest one present if that is above 1, else the first
	// free level above a run of consecutive ones; all nine chunks then carry
	// its level.  Levels run smallest first, one after another; requests that
	// do not erode come after every level.  Reorders `take` by level (stable)
	// and numbers the requests in that order.
	void schedule_levels(std::vector<uint64_t>& take) {
		std::unordered_multimap<ChunkKey, uint32_t, ChunkKeyHash> scheduled;
		for (const uint64_t t : take) {
			Request& r = requests[t];
			if (!r.erode) {
				r.level = 0xFFFFFFFFu;
				continue;
			}
			std::vector<uint32_t> present;
			for (int c = 0; c < 9; c++) {
				const ChunkKey k { r.req.MapSize, r.req.InterpolationRadius, r.req.ChunkX + (c % 3) - 1,
					r.req.ChunkY + (c / 3) - 1 };
				const auto range = scheduled.equal_range(k);
				for (auto e = range.first; e != range.second; ++e) {
					if (std::find(present.begin(), present.end(), e->second) == present.end()) {
						present.push_back(e->second);
					}
				}
			}
			std::sort(present.begin(), present.end());
			uint32_t level = 1u;
			if (!present.empty()) {
				if (present.front() > 1u) {
					level = present.front() - 1u;
				} else {
					level = present.back() + 1u;
					for (size_t i = 0; i + 1u < present.size(); i++) {
						if (present[i + 1u] - present[i] > 1u) {
							level = present[i] + 1u;
							break;
						}
					}
				}
			}
			r.level = level;
			for (int c = 0; c < 9; c++) {
				scheduled.emplace(ChunkKey { r.req.MapSize, r.req.InterpolationRadius, r.req.ChunkX + (c % 3) - 1,
					r.req.ChunkY + (c / 3) - 1 }, level);
			}
		}
		std::stable_sort(take.begin(), take.end(),
			[this](const uint64_t a, const uint64_t b) { return requests[a].level < requests[b].level; });
		for (const uint64_t t : take) {
			Request& r = requests[t];
			r.order = r.erode ? ++erosion_order : 0u;
		}
	}

	// ---------------------------------------------------------------- worker

	void complete(const std::shared_ptr<Iteration>& it) {
		const auto now = Clock::now();
		StreamSlot& sl = slots[static_cast<size_t>(it->slot)];
		const int st = (*it->status_host & STATUS_CAPACITY) ? STPGB_ECAPACITY
			: ((*it->status_host & STATUS_TIMEOUT) ? STPGB_ETIMEOUT : STPGB_OK);
		for (size_t i = 0; i < it->tickets.size(); i++) {
			Request& r = requests[it->tickets[i]];
			r.latency_ms = std::chrono::duration<double, std::milli>(now - r.submitted).count();
			r.residual = it->residual_host[i];
			r.status = st;
			r.complete = true;
			done.push_back(r.ticket);
			stats.Completed++;
		}
		for (const ChunkKey& k : it->generated) {
			Chunk& c = chunks[k];
			c.resident = true;
			c.maker.reset();
		}
		for (const ChunkKey& k : it->used) {
			Chunk& c = chunks[k];
			c.refs--;
			if (c.toucher == it) {
				c.toucher.reset();
			}
		}
		if (it->scratch_bytes) {
			pool.release(it->scratch_off, it->scratch_bytes);
		}
		sl.busy = false;
	}

	void admit() {
		while (!pending.empty() && admitted.size() + launched_requests() < cfg.MaxInFlight) {
			Request& r = requests[pending.front()];
			size_t off = 0u;
			if (!alloc_evict(r.bytes, off)) {
				break; // head of line waits for memory
			}
			r.off = off;
			r.merged = off;
			const size_t n = 9u * static_cast<size_t>(r.req.MapSize) * r.req.MapSize;
			r.fixed = off + al(n * sizeof(float));
			r.starts = r.fixed + al(n * sizeof(uint16_t));
			admitted.push_back(r.ticket);
			pending.pop_front();
			stats.Admitted++;
		}
	}

	size_t launched_requests() const {
		size_t n = 0u;
		for (const auto& it : inflight) {
			n += it->tickets.size();
		}
		return n;
	}

	// forms and launches one sequence on slot `si`; returns false if nothing could be launched
	bool launch(int si) {
		StreamSlot& sl = slots[static_cast<size_t>(si)];
		auto it = std::make_shared<Iteration>();
		it->slot = si;
		std::vector<ChunkKey> gen;
		std::vector<std::shared_ptr<Iteration>> waits;
		std::vector<uint64_t> take;
		size_t scratch = 0u;
		// the chunks of a request are pinned (refs) while it is being placed
		while (!admitted.empty() && take.size() < cfg.MaxBatch) {
			const Request& r = requests[admitted.front()];
			const uint32_t S = r.req.MapSize, rad = r.req.InterpolationRadius;
			std::vector<ChunkKey> keys;
			for (int c = 0; c < 9; c++) {
				keys.push_back(ChunkKey { S, rad, r.req.ChunkX + (c % 3) - 1, r.req.ChunkY + (c / 3) - 1 });
			}
			std::vector<ChunkKey> new_keys;
			size_t need = 0u;
			for (const ChunkKey& k : keys) {
				if (!chunks.count(k) && std::find(new_keys.begin(), new_keys.end(), k) == new_keys.end()
					&& std::find(gen.begin(), gen.end(), k) == gen.end()) {
					new_keys.push_back(k);
					need += generation_bytes(S, rad);
				}
			}
			// pin what is already there, then make room for the new chunks and their scratch
			for (const ChunkKey& k : keys) {
				auto f = chunks.find(k);
				if (f != chunks.end()) {
					f->second.refs++;
				}
			}
			bool ok = true;
			std::vector<ChunkKey> made;
			for (const ChunkKey& k : new_keys) {
				size_t off = 0u;
				if (!alloc_evict(static_cast<size_t>(S) * S * sizeof(float), off)) {
					ok = false;
					break;
				}
				Chunk c;
				c.off = off;
				c.maker = it;
				c.refs = 1; // this request
				chunks[k] = c;
				made.push_back(k);
			}
			if (!ok) {
				for (const ChunkKey& k : keys) {
					auto f = chunks.find(k);
					if (f != chunks.end() && std::find(made.begin(), made.end(), k) == made.end()) {
						f->second.refs--;
					}
				}
				for (const ChunkKey& k : made) {
					pool.release(chunks[k].off, static_cast<size_t>(S) * S * sizeof(float));
					chunks.erase(k);
				}
				break;
			}
			for (const ChunkKey& k : keys) {
				Chunk& c = chunks[k];
				c.last_use = ++clock;
				if (!c.resident && c.maker && c.maker != it
					&& std::find(waits.begin(), waits.end(), c.maker) == waits.end()) {
					waits.push_back(c.maker);
				}
				it->used.push_back(k);
			}
			for (const ChunkKey& k : made) {
				gen.push_back(k);
			}
			scratch += need;
			take.push_back(r.ticket);
			admitted.pop_front();
		}
		if (take.empty()) {
			return false;
		}
		if (scratch && !alloc_evict(scratch, it->scratch_off)) {
			// no room for the generation scratch now: undo and retry on a later pass
			for (const ChunkKey& k : it->used) {
				chunks[k].refs--;
			}
			for (const ChunkKey& k : gen) {
				pool.release(chunks[k].off, static_cast<size_t>(k.S) * k.S * sizeof(float));
				chunks.erase(k);
			}
			for (auto t = take.rbegin(); t != take.rend(); ++t) {
				admitted.push_front(*t);
			}
			return false;
		}
		it->scratch_bytes = scratch;
		if (in_place()) {
			// the sequence is placed: in admission order, a request erodes if its
			// centre has not been eroded (or scheduled) before; every chunk it
			// touches makes the sequence wait for the last earlier sequence that
			// touched it, and then belongs to this one
			for (const uint64_t t : take) {
				Request& rq = requests[t];
				for (int c = 0; c < 9; c++) {
					Chunk& ch = chunks[ChunkKey { rq.req.MapSize, rq.req.InterpolationRadius, rq.req.ChunkX + (c % 3) - 1,
						rq.req.ChunkY + (c / 3) - 1 }];
					if (ch.toucher && ch.toucher != it && std::find(waits.begin(), waits.end(), ch.toucher) == waits.end()) {
						waits.push_back(ch.toucher);
					}
					ch.toucher = it;
					if (c == 4) {
						rq.erode = !ch.centre_done;
						ch.centre_done = true;
					}
				}
			}
			schedule_levels(take);
		}
		it->tickets = take;
		it->generated = gen;
		const int rc = enqueue(*it, sl, waits);
		if (rc != STPGB_OK) {
			fatal = rc;
			fatal_msg = stpgb_last_error();
			return false;
		}
		sl.busy = true;
		inflight.push_back(it);
		stats.Launches++;
		stats.ChunksGenerated += gen.size();
		return true;
	}

	int enqueue(Iteration& it, StreamSlot& sl, const std::vector<std::shared_ptr<Iteration>>& waits) {
		const cudaStream_t s = sl.stream;
		// job tables, laid out in the slot's pinned staging area, copied in one transfer
		size_t o = 0u;
		auto carve = [&](size_t bytes) {
			const size_t at_ = o;
			o = al(o + bytes);
			return at_;
		};
		const size_t ng = it.generated.size(), nr = it.tickets.size();
		const size_t o_vor = carve(ng * sizeof(VoronoiJob)), o_lay = carve(ng * sizeof(BiomemapJob)),
			o_shf = carve(ng * sizeof(ShfJob)),
			o_noise = carve(ng * sizeof(NoiseJob)), o_gather = carve(nr * sizeof(GatherJob)),
			o_starts = carve(nr * sizeof(StartsJob)), o_ero = carve(nr * sizeof(ErosionJob)),
			o_fmt = carve(nr * sizeof(FormatJob)), o_res = carve(nr * sizeof(double)), o_status = carve(sizeof(uint32_t));
		if (o > sl.bytes) {
			return inval("stpgb_server: job tables exceed the staging area; lower MaxBatch");
		}
		VoronoiJob* vor = reinterpret_cast<VoronoiJob*>(sl.host + o_vor);
		BiomemapJob* lay = reinterpret_cast<BiomemapJob*>(sl.host + o_lay);
		const bool layers = cfg.BiomeSource == STPGB_BIOMES_LAYER_CHAIN;
		uint32_t tile = 0u, maxTiles = 0u;
		if (layers) {
			uint64_t px = 0u;
			for (const ChunkKey& k : it.generated) {
				px += 9ull * k.S * k.S;
			}
			tile = layer_tile(chain, px);
		}
		ShfJob* shf = reinterpret_cast<ShfJob*>(sl.host + o_shf);
		NoiseJob* noise = reinterpret_cast<NoiseJob*>(sl.host + o_noise);
		GatherJob* gat = reinterpret_cast<GatherJob*>(sl.host + o_gather);
		StartsJob* sts = reinterpret_cast<StartsJob*>(sl.host + o_starts);
		ErosionJob* ero = reinterpret_cast<ErosionJob*>(sl.host + o_ero);
		FormatJob* fmt = reinterpret_cast<FormatJob*>(sl.host + o_fmt);
		it.residual_host = reinterpret_cast<double*>(sl.host + o_res);
		it.status_host = reinterpret_cast<uint32_t*>(sl.host + o_status);
		double* res_dev = reinterpret_cast<double*>(sl.dev + o_res);
		uint32_t* status_dev = reinterpret_cast<uint32_t*>(sl.dev + o_status);

		uint32_t maxS = 0u, maxR = 0u, maxRS = 0u, maxCount = 0u;
		size_t so = it.scratch_off;
		for (size_t j = 0; j < ng; j++) {
			const ChunkKey& k = it.generated[j];
			const uint32_t S = k.S;
			const size_t npix = static_cast<size_t>(S) * S;
			const uint32_t kv = shf_kcap_v(k.r, max_items);
			const ShfLayout l = shf_layout(S, S, k.r, kv);
			const uint64_t cap = npix * std::min<uint64_t>(shf_kcap_h(k.r, max_items), (2ull * k.r + 1u) * (2ull * k.r + 1u));
			uint16_t* const region = reinterpret_cast<uint16_t*>(at(so));
			so += al(9u * npix * sizeof(uint16_t));
			unsigned char* const ws = at(so);
			so += al(l.total);
			uint32_t* const offsets = reinterpret_cast<uint32_t*>(at(so));
			so += al((npix + 1u) * sizeof(uint32_t));
			stpgb_bin* const bins = reinterpret_cast<stpgb_bin*>(at(so));
			so += al(cap * sizeof(stpgb_bin));
			// the biome map is a function of world pixels: cell scaled with the side
			const uint32_t cell = std::max<uint32_t>(1u, static_cast<uint32_t>(
				static_cast<uint64_t>(cfg.VoronoiCell) * S / 512u));
			vor[j] = VoronoiJob { region, (static_cast<int64_t>(k.x) - 1) * S, (static_cast<int64_t>(k.y) - 1) * S, 3u * S,
				3u * S, cell };
			if (layers) {
				// the 3x3 chunks around chunk k, world pixels ((k - 1) * S, ...)
				BiomemapJob& lj = lay[j];
				lj = BiomemapJob {};
				lj.out = region;
				lj.x0 = static_cast<int32_t>((static_cast<int64_t>(k.x) - 1) * S);
				lj.z0 = static_cast<int32_t>((static_cast<int64_t>(k.y) - 1) * S);
				lj.pitch = lj.width = lj.height = 3u * S;
				STPGB_TRY(layer_job_tiling(lj, tile));
				maxTiles = std::max(maxTiles, lj.tiles);
			}
			ShfJob& sj = shf[j];
			sj = ShfJob {};
			sj.samplemap = region;
			sj.pitch = 3u * S;
			sj.W = sj.H = S;
			sj.sx = sj.sy = S;
			sj.r = k.r;
			sj.kcap_v = kv;
			shf_bind_workspace(sj, ws, l);
			sj.offsets = offsets;
			sj.bins = bins;
			sj.bins_capacity = cap;
			sj.status = status_dev;
			noise[j] = NoiseJob { reinterpret_cast<float*>(at(chunks[k].off)), S, offsets, bins, S, S,
				static_cast<float>(static_cast<int64_t>(k.x) * S), static_cast<float>(static_cast<int64_t>(k.y) * S) };
			maxS = std::max(maxS, S);
			maxR = std::max(maxR, k.r);
		}
		for (size_t i = 0; i < nr; i++) {
			const Request& r = requests[it.tickets[i]];
			const uint32_t S = r.req.MapSize;
			GatherJob g {};
			for (int c = 0; c < 9; c++) {
				const ChunkKey k { S, r.req.InterpolationRadius, r.req.ChunkX + (c % 3) - 1, r.req.ChunkY + (c / 3) - 1 };
				g.chunk[c] = reinterpret_cast<const float*>(at(chunks[k].off));
			}
			g.merged = reinterpret_cast<float*>(at(r.merged));
			g.S = S;
			gat[i] = g;
			// droplet counter space keyed by the request's side and centre chunk
			const uint64_t ctr_base = (static_cast<uint64_t>(static_cast<uint32_t>(r.req.ChunkX)) << 40)
				^ (static_cast<uint64_t>(static_cast<uint32_t>(r.req.ChunkY)) << 16) ^ (static_cast<uint64_t>(S) << 60);
			sts[i] = StartsJob { reinterpret_cast<float*>(at(r.starts)), ctr_base, r.droplets, S };
			size_t boff = 0u;
			uint32_t bsize = 0u;
			STPGB_TRY(brush_for(S, r.req.BrushRadius, boff, bsize));
			stpgb_raindrop_setting rs = this->base;
			rs.RainDropCount = std::max(1u, r.droplets);
			rs.ErosionBrushRadius = r.req.BrushRadius;
			if (r.req.Lifetime) {
				rs.minWaterVolume = stpgb_lifetime_min_water_volume(rs.initWaterVolume, rs.EvaporateSpeed, r.req.Lifetime);
			}
			ErosionJob e {};
			e.map = reinterpret_cast<float*>(at(r.merged));
			e.dim_x = e.dim_y = 3u * S;
			e.pitch = 3u * S;
			e.starts = reinterpret_cast<const float*>(at(r.starts));
			e.count = r.droplets;
			e.brush_index = reinterpret_cast<const int32_t*>(at(boff));
			e.brush_weight = reinterpret_cast<const float*>(at(boff) + bsize * sizeof(int32_t));
			e.brush_size = bsize;
			e.p = rain_params(rs);
			e.residual = res_dev + i;
			e.status = status_dev;
			e.start_area = S * S;
			ero[i] = e;
			fmt[i] = FormatJob { e.map, 3ull * S, reinterpret_cast<uint16_t*>(at(r.fixed)), 3ull * S, 3u * S, 3u * S };
			maxRS = std::max(maxRS, S);
			maxCount = std::max(maxCount, r.droplets);
		}
		// Erosion variant groups: every request takes its own default kernel
		// (erosion_choice on its brush, its droplet density and its droplets in
		// flight per pixel), the jobs of one variant are made contiguous and
		// eroded by one launch.  One variant for the whole sequence would hold
		// every request to what its densest one allows.  In the in-place mode
		// each priority level is grouped on its own.
		struct ErosionGroup {
			ErosionChoice ec;
			uint32_t dpg, first, n, maxCount, maxBrush, minRadius;
		};
		auto group_range = [&](const size_t b, const size_t e, std::vector<ErosionGroup>& egroups) {
			std::vector<ErosionJob> by_request(ero + b, ero + e);
			std::vector<std::pair<uint32_t, uint32_t>> keyed(e - b); // (variant key, request)
			std::vector<ErosionChoice> choice(e - b);
			std::vector<uint32_t> dpgs(e - b);
			for (size_t q = 0; q < e - b; q++) {
				const Request& r = requests[it.tickets[b + q]];
				const double area = static_cast<double>(r.req.MapSize) * r.req.MapSize;
				const double density = r.droplets / area, in_flight = erosion_in_flight(r.droplets, area);
				choice[q] = erosion_choice(r.req.BrushRadius, by_request[q].brush_size, density, in_flight, true);
				// the stable point-wise variant with two droplets per group where rows are not allowed
				dpgs[q] = !choice[q].rows && choice[q].lanes >= 4u
						&& erosion_variant_stable(choice[q].lanes, 2u, false, density, in_flight)
					? 2u
					: 1u;
				keyed[q] = { choice[q].lanes * 8u + dpgs[q] * 2u + (choice[q].rows ? 1u : 0u), static_cast<uint32_t>(q) };
			}
			std::stable_sort(keyed.begin(), keyed.end(),
				[](const auto& x, const auto& y) { return x.first < y.first; });
			for (size_t pos = 0; pos < e - b; pos++) {
				const uint32_t q = keyed[pos].second;
				ero[b + pos] = by_request[q];
				if (pos == 0u || keyed[pos].first != keyed[pos - 1u].first) {
					egroups.push_back(ErosionGroup { choice[q], dpgs[q], static_cast<uint32_t>(b + pos), 0u, 0u, 0u,
						0xFFFFFFFFu });
				}
				ErosionGroup& g = egroups.back();
				g.n++;
				g.maxCount = std::max(g.maxCount, ero[b + pos].count);
				g.maxBrush = std::max(g.maxBrush, ero[b + pos].brush_size);
				g.minRadius = std::min(g.minRadius, requests[it.tickets[b + q]].req.BrushRadius);
			}
		};
		// request ranges eroded one after another: every request (private mode),
		// or one range per priority level of the eroding requests (in place)
		struct Level {
			size_t b, e;
			std::vector<ErosionGroup> groups;
		};
		std::vector<Level> levels;
		size_t n_erode = nr;
		if (in_place()) {
			n_erode = 0u;
			while (n_erode < nr && requests[it.tickets[n_erode]].erode) {
				n_erode++;
			}
			for (size_t i = 0; i < n_erode;) {
				size_t j = i + 1u;
				while (j < n_erode && requests[it.tickets[j]].level == requests[it.tickets[i]].level) {
					j++;
				}
				levels.push_back(Level { i, j, {} });
				i = j;
			}
		} else if (nr) {
			levels.push_back(Level { 0u, nr, {} });
		}
		for (Level& L : levels) {
			group_range(L.b, L.e, L.groups);
		}
		std::fill(it.residual_host, it.residual_host + nr, 0.0);
		*it.status_host = 0u;
		STPGB_CUDA_TRY(cudaMemcpyAsync(sl.dev, sl.host, o, cudaMemcpyHostToDevice, s));
		if (ng) {
			if (layers) {
				STPGB_TRY(layer_biomemap_launch(chain, reinterpret_cast<BiomemapJob*>(sl.dev + o_lay), lay[0],
					static_cast<uint32_t>(ng), maxTiles, tile, s));
			} else {
				STPGB_TRY(voronoi_jobs_launch(reinterpret_cast<VoronoiJob*>(sl.dev + o_vor), static_cast<uint32_t>(ng),
					3u * maxS, 3u * maxS, cfg.BiomeSeed, biome_count, s));
			}
			STPGB_TRY(shf_launch(reinterpret_cast<ShfJob*>(sl.dev + o_shf), shf[0], static_cast<uint32_t>(ng), maxS, maxS,
				maxR, shf_kcap_v(maxR, max_items), shf_kcap_h(maxR, max_items), s));
			STPGB_TRY(noise_launch(reinterpret_cast<NoiseJob*>(sl.dev + o_noise), noise[0], static_cast<uint32_t>(ng),
				static_cast<uint64_t>(maxS) * maxS, permutation, table, biome_count, s));
		}
		for (const auto& w : waits) {
			STPGB_CUDA_TRY(cudaStreamWaitEvent(s, slots[static_cast<size_t>(w->slot)].done, 0));
		}
		GatherJob* const gat_dev = reinterpret_cast<GatherJob*>(sl.dev + o_gather);
		StartsJob* const sts_dev = reinterpret_cast<StartsJob*>(sl.dev + o_starts);
		for (const Level& L : levels) {
			const uint32_t n = static_cast<uint32_t>(L.e - L.b);
			STPGB_TRY(gather_jobs_launch(gat_dev + L.b, n, maxRS, s));
			STPGB_TRY(starts_jobs_launch(sts_dev + L.b, n, maxCount, this->base.Seed, s));
			// brush rows in 16-byte blocks (pool blocks are 256-byte aligned,
			// pitches 3 * MapSize); each job reads several blocks per round trip
			// where few of its droplets are in flight per pixel; the
			// warp-cooperative kernel alternates the blocks of every job of its
			// group (the batch autotuner's choice for sixteen 512^2 jobs)
			for (const ErosionGroup& g : L.groups) {
				STPGB_TRY(erosion_launch(reinterpret_cast<ErosionJob*>(sl.dev + o_ero) + g.first, ero[g.first], g.n,
					g.maxCount, g.maxBrush, s, g.ec.lanes, false, g.dpg, g.ec.rows, erosion_rows_wide(g.minRadius),
					erosion_rows_atomic(g.minRadius, g.ec.lanes), g.n));
			}
			if (in_place()) {
				// the eroded neighbourhoods go back into the resident chunks
				STPGB_TRY(scatter_jobs_launch(gat_dev + L.b, n, maxRS, s));
			}
		}
		if (n_erode < nr) {
			// requests whose centre was eroded before: the current state, after every level
			STPGB_TRY(gather_jobs_launch(gat_dev + n_erode, static_cast<uint32_t>(nr - n_erode), maxRS, s));
		}
		STPGB_TRY(format_batch_launch(reinterpret_cast<FormatJob*>(sl.dev + o_fmt), static_cast<uint32_t>(nr), 3u * maxRS,
			3u * maxRS, s));
		STPGB_CUDA_TRY(cudaMemcpyAsync(it.residual_host, res_dev, nr * sizeof(double), cudaMemcpyDeviceToHost, s));
		STPGB_CUDA_TRY(cudaMemcpyAsync(it.status_host, status_dev, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
		STPGB_CUDA_TRY(cudaEventRecord(sl.done, s));
		return STPGB_OK;
	}

	void run() {
		cudaSetDevice(device);
		std::unique_lock<std::mutex> lk(mu);
		while (!stop) {
			bool progress = false;
			for (auto i = inflight.begin(); i != inflight.end();) {
				const cudaError_t q = cudaEventQuery(slots[static_cast<size_t>((*i)->slot)].done);
				if (q == cudaSuccess) {
					complete(*i);
					i = inflight.erase(i);
					progress = true;
				} else if (q != cudaErrorNotReady) {
					fatal = cuda_fail(q, "stpgb_server: device work failed");
					fatal_msg = stpgb_last_error();
					stop = true;
					break;
				} else {
					++i;
				}
			}
			if (progress) {
				cv_done.notify_all();
			}
			admit();
			for (size_t si = 0; si < slots.size() && !admitted.empty() && fatal == STPGB_OK; si++) {
				if (!slots[si].busy && launch(static_cast<int>(si))) {
					progress = true;
				}
			}
			if (fatal != STPGB_OK) {
				stop = true;
				cv_done.notify_all();
				break;
			}
			if (!progress) {
				cv_work.wait_for(lk, std::chrono::microseconds(inflight.empty() ? 2000 : 50));
			}
		}
		cv_done.notify_all();
	}

	int device = 0;
};

extern "C" {

int stpgb_server_create(const stpgb_server_config* cfg, const stpgb_raindrop_setting* base,
	const stpgb_simplex_setting* simplex, const stpgb_biome_property* biome_table, uint32_t biome_count,
	stpgb_server** out) {
	if (!cfg || !base || !simplex || !biome_table || biome_count == 0u || !out) {
		return inval("stpgb_server_create: null argument or empty biome table");
	}
	if (cfg->HbmBudget == 0u || cfg->MaxInFlight == 0u || cfg->MaxBatch == 0u || cfg->Streams == 0u
		|| cfg->VoronoiCell == 0u) {
		return inval("stpgb_server_create: budget, in-flight limit, batch, streams and cell must be positive");
	}
	STPGB_TRY(stpgb_simplex_setting_validate(simplex));
	STPGB_TRY(stpgb_raindrop_setting_validate(base));
	auto sv = std::make_unique<stpgb_server>();
	sv->cfg = *cfg;
	sv->base = *base;
	if (cfg->BiomeSource > STPGB_BIOMES_LAYER_CHAIN) {
		return inval("stpgb_server_create: BiomeSource must be STPGB_BIOMES_VORONOI or STPGB_BIOMES_LAYER_CHAIN");
	}
	if (cfg->ErosionMode > STPGB_EROSION_IN_PLACE) {
		return inval("stpgb_server_create: ErosionMode must be STPGB_EROSION_PRIVATE or STPGB_EROSION_IN_PLACE");
	}
	if (cfg->BiomeSource == STPGB_BIOMES_LAYER_CHAIN) {
		STPGB_TRY(layer_chain_demo(cfg->BiomeSeed, &sv->chain));
	}
	sv->biome_count = biome_count;
	sv->max_items = std::min<uint32_t>(biome_count, kShfMaxItems);
	STPGB_CUDA_TRY(cudaGetDevice(&sv->device));
	std::vector<uint8_t> perm(512);
	std::vector<float> grad(2u * simplex->Distribution);
	STPGB_TRY(stpgb_permutation_generate(simplex, perm.data(), grad.data(), static_cast<uint32_t>(grad.size())));
	STPGB_CUDA_TRY(cudaMalloc(&sv->perm, 512));
	STPGB_CUDA_TRY(cudaMalloc(&sv->grad, grad.size() * sizeof(float)));
	STPGB_CUDA_TRY(cudaMalloc(&sv->table, biome_count * sizeof(stpgb_biome_property)));
	STPGB_CUDA_TRY(cudaMemcpy(sv->perm, perm.data(), 512, cudaMemcpyHostToDevice));
	STPGB_CUDA_TRY(cudaMemcpy(sv->grad, grad.data(), grad.size() * sizeof(float), cudaMemcpyHostToDevice));
	STPGB_CUDA_TRY(cudaMemcpy(sv->table, biome_table, biome_count * sizeof(stpgb_biome_property), cudaMemcpyHostToDevice));
	sv->permutation = stpgb_permutation { sv->perm, sv->grad, simplex->Distribution };
	{
		const cudaError_t e = cudaMalloc(&sv->pool_mem, cfg->HbmBudget);
		if (e != cudaSuccess) {
			cudaGetLastError();
			set_error("stpgb_server_create: the HBM budget could not be allocated");
			return STPGB_ENOMEM;
		}
	}
	sv->pool.reset(cfg->HbmBudget);
	sv->slots.resize(cfg->Streams);
	for (auto& s : sv->slots) {
		STPGB_CUDA_TRY(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking));
		STPGB_CUDA_TRY(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming));
		STPGB_CUDA_TRY(cudaMalloc(&s.dev, kStagingBytes));
		STPGB_CUDA_TRY(cudaMallocHost(&s.host, kStagingBytes));
		s.bytes = kStagingBytes;
	}
	stpgb_server* raw = sv.get();
	sv->worker = std::thread([raw]() { raw->run(); });
	*out = sv.release();
	return STPGB_OK;
}

int stpgb_server_destroy(stpgb_server* sv) {
	delete sv;
	return STPGB_OK;
}

int stpgb_server_submit(stpgb_server* sv, const stpgb_serve_request* req, uint64_t* ticket) {
	return stpgb_server_submit_batch(sv, req, 1u, ticket);
}

int stpgb_server_submit_batch(stpgb_server* sv, const stpgb_serve_request* reqs, uint32_t count, uint64_t* tickets) {
	if (!sv || (!reqs && count)) {
		return inval("stpgb_server_submit: null argument");
	}
	std::vector<Request> batch(count);
	for (uint32_t i = 0u; i < count; i++) {
		STPGB_TRY(sv->prepare(reqs[i], batch[i]));
	}
	{
		std::lock_guard<std::mutex> lk(sv->mu);
		if (sv->fatal != STPGB_OK) {
			set_error(sv->fatal_msg);
			return sv->fatal;
		}
		for (uint32_t i = 0u; i < count; i++) {
			Request& r = batch[i];
			r.ticket = sv->next_ticket++;
			if (tickets) {
				tickets[i] = r.ticket;
			}
			sv->requests[r.ticket] = r;
			sv->pending.push_back(r.ticket);
			sv->stats.Submitted++;
		}
	}
	sv->cv_work.notify_one();
	return STPGB_OK;
}

} // extern "C"

int stpgb_server::prepare(const stpgb_serve_request& q, Request& r) const {
	const stpgb_serve_request* const req = &q;
	if (req->MapSize == 0u || (req->MapSize & 7u) || req->MapSize > 16384u || req->InterpolationRadius == 0u
		|| (req->InterpolationRadius & 1u) || req->InterpolationRadius > req->MapSize || req->BrushRadius == 0u
		|| !(req->DropletsPerPixel >= 0.0f)) {
		return inval("stpgb_server_submit: MapSize must be a multiple of 8 and at most 16384, radius positive, even "
					 "and <= MapSize, brush positive");
	}
	r.req = *req;
	r.submitted = Clock::now();
	r.droplets = droplets_of(*req);
	r.bytes = stpgb_server::request_bytes(req->MapSize, r.droplets);
	const size_t gen = 9u * (generation_bytes(req->MapSize, req->InterpolationRadius)
		+ static_cast<size_t>(req->MapSize) * req->MapSize * sizeof(float));
	if (r.bytes + gen > cfg.HbmBudget) {
		set_error("stpgb_server_submit: one request of this size does not fit the HBM budget");
		return STPGB_ENOMEM;
	}
	return STPGB_OK;
}

extern "C" {

int stpgb_server_poll(stpgb_server* sv, stpgb_serve_result* out, uint32_t capacity, uint32_t* count, int wait_ms) {
	if (!sv || (!out && capacity) || !count) {
		return inval("stpgb_server_poll: null argument");
	}
	std::unique_lock<std::mutex> lk(sv->mu);
	if (sv->done.empty() && wait_ms != 0 && sv->fatal == STPGB_OK) {
		auto pred = [sv]() { return !sv->done.empty() || sv->fatal != STPGB_OK; };
		if (wait_ms < 0) {
			sv->cv_done.wait(lk, pred);
		} else {
			sv->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), pred);
		}
	}
	uint32_t n = 0u;
	while (n < capacity && !sv->done.empty()) {
		const Request& r = sv->requests[sv->done.front()];
		sv->done.pop_front();
		stpgb_serve_result& o = out[n++];
		o.Ticket = r.ticket;
		o.UserTag = r.req.UserTag;
		o.Status = r.status;
		o.LatencyMs = r.latency_ms;
		o.Heightmap = reinterpret_cast<const float*>(sv->at(r.merged));
		o.HeightmapFixed = reinterpret_cast<const uint16_t*>(sv->at(r.fixed));
		o.ResidualSediment = r.residual;
		o.MapSize = r.req.MapSize;
		o.ErosionOrder = r.order;
	}
	*count = n;
	if (sv->fatal != STPGB_OK) {
		set_error(sv->fatal_msg);
		return sv->fatal;
	}
	return STPGB_OK;
}

int stpgb_server_release(stpgb_server* sv, uint64_t ticket) {
	if (!sv) {
		return inval("stpgb_server_release: null server");
	}
	{
		std::lock_guard<std::mutex> lk(sv->mu);
		auto it = sv->requests.find(ticket);
		if (it == sv->requests.end() || !it->second.complete) {
			return inval("stpgb_server_release: unknown or incomplete ticket");
		}
		sv->pool.release(it->second.off, it->second.bytes);
		sv->requests.erase(it);
	}
	sv->cv_work.notify_one();
	return STPGB_OK;
}

int stpgb_server_download(stpgb_server* sv, uint64_t ticket, float* heightmap, uint16_t* heightmap_fixed) {
	if (!sv) {
		return inval("stpgb_server_download: null server");
	}
	size_t merged = 0u, fixed = 0u, n = 0u;
	{
		std::lock_guard<std::mutex> lk(sv->mu);
		auto it = sv->requests.find(ticket);
		if (it == sv->requests.end() || !it->second.complete) {
			return inval("stpgb_server_download: unknown or incomplete ticket");
		}
		merged = it->second.merged;
		fixed = it->second.fixed;
		n = 9u * static_cast<size_t>(it->second.req.MapSize) * it->second.req.MapSize;
	}
	if (heightmap) {
		STPGB_CUDA_TRY(cudaMemcpy(heightmap, sv->at(merged), n * sizeof(float), cudaMemcpyDeviceToHost));
	}
	if (heightmap_fixed) {
		STPGB_CUDA_TRY(cudaMemcpy(heightmap_fixed, sv->at(fixed), n * sizeof(uint16_t), cudaMemcpyDeviceToHost));
	}
	return STPGB_OK;
}

int stpgb_server_stats_get(stpgb_server* sv, stpgb_server_stats* out) {
	if (!sv || !out) {
		return inval("stpgb_server_stats_get: null argument");
	}
	std::lock_guard<std::mutex> lk(sv->mu);
	*out = sv->stats;
	out->PoolBytesUsed = sv->pool.used();
	out->ResidentChunks = sv->chunks.size();
	return STPGB_OK;
}

int stpgb_server_replay(stpgb_server* sv, const stpgb_serve_request* reqs, const double* arrival_s, uint32_t n,
	double* latency_ms, double* wall_s) {
	if (!sv || (!reqs && n) || (!arrival_s && n)) {
		return inval("stpgb_server_replay: null argument");
	}
	std::vector<uint64_t> tickets(n);
	std::unordered_map<uint64_t, uint32_t> index;
	const auto t0 = Clock::now();
	uint32_t next = 0u, finished = 0u;
	std::vector<stpgb_serve_result> res(64);
	while (finished < n) {
		const double now = std::chrono::duration<double>(Clock::now() - t0).count();
		while (next < n && arrival_s[next] <= now) {
			STPGB_TRY(stpgb_server_submit(sv, &reqs[next], &tickets[next]));
			index[tickets[next]] = next;
			next++;
		}
		uint32_t got = 0u;
		double wait = next < n ? (arrival_s[next] - std::chrono::duration<double>(Clock::now() - t0).count()) : 0.01;
		const int wms = next < n ? std::max(0, static_cast<int>(wait * 1000.0)) : 5;
		STPGB_TRY(stpgb_server_poll(sv, res.data(), static_cast<uint32_t>(res.size()), &got, wms));
		for (uint32_t i = 0u; i < got; i++) {
			if (res[i].Status != STPGB_OK) {
				set_error("stpgb_server_replay: a request failed on the device");
				return res[i].Status;
			}
			if (latency_ms) {
				latency_ms[index[res[i].Ticket]] = res[i].LatencyMs;
			}
			STPGB_TRY(stpgb_server_release(sv, res[i].Ticket));
			finished++;
		}
		if (next < n && got == 0u) {
			const double rest = arrival_s[next] - std::chrono::duration<double>(Clock::now() - t0).count();
			if (rest > 0.0) {
				std::this_thread::sleep_for(std::chrono::duration<double>(std::min(rest, 0.0005)));
			}
		}
	}
	if (wall_s) {
		*wall_s = std::chrono::duration<double>(Clock::now() - t0).count();
	}
	return STPGB_OK;
}

} // extern "C"
