"""GB300-native SuperTerrain+ heightfield pipeline.

Host-side mirror of the reference interface for the heightfield path, over
the C ABI of libstpgb.so (include/stpgb.h):

* STPPermutationGenerator.generate        (SuperAlgorithm+Host/STPPermutationGenerator.h:50)
* STPSingleHistogramFilter / STPFilterBuffer (SuperAlgorithm+Host/STPSingleHistogramFilter.h:36-190)
* STPHeightfieldGenerator.generate / erode (SuperTerrain+/World/Chunk/STPHeightfieldGenerator.h:145,159)
* STPBiomeFactory over the demo's layer chain (STPLayerChainBuilder,
  SuperDemo+/World/Layers/STPAllLayers.h; SuperTerrain+/World/Diversity/STPBiomeFactory.h:19-63)
* kernel-level calls on device buffers (shf_filter, multibiome_heightmap,
  hydraulic_erosion, format_heightmap, droplet_starts, voronoi_biomemap,
  layer_biomemap)

Device buffers are torch CUDA tensors (PyTorch is only the allocator and the
stream provider here); the compute runs in the CUDA kernels of libstpgb.so.
"""
import ctypes as C

import numpy as np

from ._capi import (STPGB_EINVAL, STPGB_MAX_LAYERS, STPGB_OK, AltitudeRule, BiomeProperty, ChunkSetting, GradientRule, Layer, LayerBiomes,
                    NNInfo, Permutation, RaindropSetting, SimplexSetting, SplatChunk, STPCapacityError, STPCUDAError, STPException, STPInsufficientMemory, STPInvalidEnvironment,
                    STPNumericDomainError, STPTimeout, check, lib)

__all__ = [
    "BiomeProperty", "ChunkSetting", "NNInfo", "Permutation", "RaindropSetting", "SimplexSetting",
    "STPCapacityError", "STPCUDAError", "STPException", "STPInsufficientMemory", "STPInvalidEnvironment",
    "STPNumericDomainError", "STPTimeout", "STPDiversityGenerator", "STPBiomefieldGenerator", "BIN_DTYPE", "BIOME_DTYPE", "lib", "check",
    "permutation_generate", "erosion_brush", "lifetime_min_water_volume", "STPSingleHistogramFilter",
    "STPFilterBuffer", "STPHeightfieldGenerator", "DeviceOps", "Batch", "Layer", "LayerBiomes",
    "layer_chain_demo", "STPLayerChainBuilder", "AltitudeRule", "GradientRule", "SplatChunk", "splat_rules_demo",
    "STPSplatmapGenerator", "STPChunk", "nn_merge_host", "nn_unmerge_host",
]

BIN_DTYPE = np.dtype([("Item", "<u2"), ("_pad", "<u2"), ("Weight", "<f4")])
BIOME_DTYPE = np.dtype([("Scale", "<f4"), ("Octave", "<u4"), ("Persistence", "<f4"),
                        ("Lacunarity", "<f4"), ("Depth", "<f4"), ("Variation", "<f4")])


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _data(a):
    """Host address of a numpy array, or NULL for None (a request the call skips)."""
    return a.ctypes.data if a is not None else None


# ------------------------------------------------------------ host tables


def permutation_generate(seed, distribution, offset):
    """STPPermutationGenerator::generate, host half: (perm u8[512], grad f32[2N])."""
    s = SimplexSetting(seed, distribution, offset)
    perm = np.zeros(512, np.uint8)
    grad = np.zeros(2 * max(distribution, 1), np.float32)
    check(lib().stpgb_permutation_generate(C.byref(s), _p(perm), _p(grad), grad.size), env_error=True)
    return perm, grad


def erosion_brush(dimension_x, radius):
    """generateErosionBrush: (index i32[n], weight f32[n])."""
    n = C.c_uint32(0)
    rc = lib().stpgb_erosion_brush_generate(dimension_x, radius, None, None, 0, C.byref(n))
    if rc not in (0, 5):
        check(rc)
    idx = np.zeros(n.value, np.int32)
    w = np.zeros(n.value, np.float32)
    check(lib().stpgb_erosion_brush_generate(dimension_x, radius, _p(idx), _p(w), n.value, C.byref(n)))
    return idx, w


def lifetime_min_water_volume(init_water_volume, evaporate_speed, lifetime):
    return float(lib().stpgb_lifetime_min_water_volume(init_water_volume, evaporate_speed, lifetime))


# ------------------------------------------------------ chunk coordinates


def _vec(values, ctype):
    return (ctype * 2)(*values)


class STPChunk:
    """The static coordinate functions of STPChunk (SuperTerrain+/World/Chunk/STPChunk.h:110-157) over
    the C ABI.  Vectors are (x, y) pairs; a chunk coordinate is in world units (a multiple of the chunk
    size).  Arguments the reference leaves undefined (zero sizes, int32 overflow) raise
    STPNumericDomainError."""

    @staticmethod
    def calcWorldChunkCoordinate(point_pos, chunk_size, scale):
        """point_pos is (x, y, z); the chunk holding (x, z)."""
        out = (C.c_int32 * 2)()
        check(lib().stpgb_chunk_world_coordinate(float(point_pos[0]), float(point_pos[2]),
                                                 _vec(chunk_size, C.c_uint32), _vec(scale, C.c_double), out))
        return tuple(out)

    @staticmethod
    def calcLocalChunkCoordinate(chunk_id, chunk_range):
        out = (C.c_uint32 * 2)()
        check(lib().stpgb_chunk_local_coordinate(chunk_id, _vec(chunk_range, C.c_uint32), out))
        return tuple(out)

    @staticmethod
    def calcLocalChunkOrigin(centre, chunk_size, neighbour_size):
        out = (C.c_int32 * 2)()
        check(lib().stpgb_chunk_local_origin(_vec(centre, C.c_int32), _vec(chunk_size, C.c_uint32),
                                             _vec(neighbour_size, C.c_uint32), out))
        return tuple(out)

    @staticmethod
    def calcChunkMapOffset(chunk_coord, chunk_size, map_size, map_offset):
        out = (C.c_double * 2)()
        check(lib().stpgb_chunk_map_offset(_vec(chunk_coord, C.c_int32), _vec(chunk_size, C.c_uint32),
                                           _vec(map_size, C.c_uint32), _vec(map_offset, C.c_double), out))
        return tuple(out)

    @staticmethod
    def offsetChunk(chunk_coord, chunk_size, offset):
        out = (C.c_int32 * 2)()
        check(lib().stpgb_chunk_offset(_vec(chunk_coord, C.c_int32), _vec(chunk_size, C.c_uint32),
                                       _vec(offset, C.c_int32), out))
        return tuple(out)

    @staticmethod
    def calcChunkNeighbourOffset(chunk_size, region_size):
        """List of (x, y) offsets from the centre chunk, in chunk-index order."""
        n = C.c_uint32(0)
        cs, rs = _vec(chunk_size, C.c_uint32), _vec(region_size, C.c_uint32)
        count = int(region_size[0]) * int(region_size[1])
        out = (C.c_int32 * (2 * max(count, 1)))()
        check(lib().stpgb_chunk_neighbour_offset(cs, rs, out, count, C.byref(n)))
        return [(out[2 * i], out[2 * i + 1]) for i in range(n.value)]


def nn_merge_host(chunks, nn_info):
    """Pack the ChunkNearestNeighbour.x * .y chunk maps (numpy arrays of MapSize, one dtype, chunk
    index order) into one merged TotalMapSize map (STPNearestNeighbourTextureBuffer host mode)."""
    chunks = [np.ascontiguousarray(c) for c in chunks]
    merged = np.empty((nn_info.TotalMapSize[1], nn_info.TotalMapSize[0]), chunks[0].dtype)
    ptrs = (C.c_void_p * len(chunks))(*[c.ctypes.data for c in chunks])
    check(lib().stpgb_nn_merge_host(ptrs, chunks[0].dtype.itemsize, C.byref(nn_info), _p(merged)))
    return merged


def nn_unmerge_host(merged, nn_info, chunks):
    """Unpack a merged map back into the chunk maps `chunks` (contiguous numpy arrays, written in place)."""
    merged = np.ascontiguousarray(merged)
    ptrs = (C.c_void_p * len(chunks))(*[c.ctypes.data for c in chunks])
    check(lib().stpgb_nn_unmerge_host(_p(merged), merged.dtype.itemsize, C.byref(nn_info), ptrs))


# ------------------------------------------------- single histogram filter


# ------------------------------------------------------ biome layer chain


def layer_chain_demo():
    """The demo's production line (SuperDemo+/World/Layers/STPAllLayers.cpp:59-105), first
    ancestor first, and the demo's biome IDs: (ctypes Layer array, LayerBiomes)."""
    buf = (Layer * STPGB_MAX_LAYERS)()
    n = C.c_uint32(0)
    check(lib().stpgb_layer_chain_demo(buf, STPGB_MAX_LAYERS, C.byref(n)))
    chain = (Layer * n.value)(*buf[:n.value])
    ids = LayerBiomes()
    lib().stpgb_layer_biomes_demo(C.byref(ids))
    return chain, ids


def _layer_array(chain):
    if isinstance(chain, C.Array):
        return chain
    return (Layer * len(chain))(*[c if isinstance(c, Layer) else Layer(*c) for c in chain])


class STPLayerChainBuilder:
    """STPBiomeFactory with the demo's layer chain (STPDemo::STPLayerChainBuilder,
    SuperDemo+/World/Layers/STPAllLayers.h): `factory(biomemap, offset)` fills a
    uint16 host array of `dimension` (x, y) with the biomes of world pixels
    offset + (x, z), as STPBiomeFactory::operator() (STPBiomeFactory.cpp:24-41).
    The chain runs on the GPU; `chain` / `ids` replace the demo's layers and IDs."""

    def __init__(self, dimension, global_seed, chain=None, ids=None):
        if dimension[0] <= 0 or dimension[1] <= 0:
            raise STPNumericDomainError("Biomemap should have strictly positive dimension in both vector components")
        self.BiomeDimension = (int(dimension[0]), int(dimension[1]))
        self.GlobalSeed = int(global_seed)
        demo_chain, demo_ids = layer_chain_demo()
        self.chain = _layer_array(chain) if chain is not None else demo_chain
        self.ids = ids if ids is not None else demo_ids

    def __call__(self, biomemap, offset):
        w, h = self.BiomeDimension
        if biomemap.dtype != np.uint16 or biomemap.size != w * h or not biomemap.flags.c_contiguous:
            raise STPNumericDomainError("biomemap must be a contiguous uint16 array of the factory's dimension")
        check(lib().stpgb_layer_biomemap_host(self.chain, len(self.chain), self.GlobalSeed, C.byref(self.ids),
                                              _p(biomemap), w, h, int(offset[0]), int(offset[1])))


# ---------------------------------------------------------------- splatmap


def splat_rules_demo():
    """The demo's splat rules (SuperDemo+/Script/STPBiomeSplatRule.tdl): (altitude, gradient) ctypes arrays."""
    a, g = (AltitudeRule * 16)(), (GradientRule * 16)()
    na, ng = C.c_uint32(0), C.c_uint32(0)
    check(lib().stpgb_splat_rules_demo(a, 16, C.byref(na), g, 16, C.byref(ng)))
    return (AltitudeRule * na.value)(*a[:na.value]), (GradientRule * ng.value)(*g[:ng.value])


class STPSplatmapGenerator:
    """The splatmap generator (SuperDemo+/World/Biomes/STPSplatmapGenerator.h with the rule database
    of STPTextureFactory): `gen(biomemap, heightmap, map_pitch, splatmap, splat_pitch, width, height,
    chunks)` on torch CUDA tensors (or raw device addresses) fills the region of every pixel of the
    requested chunks (STPTextureFactory::operator(),
    SuperTerrain+/Private/World/Diversity/STPTextureFactory.cpp:211-232); `map_pitch` is one pitch for
    both maps or a (biome pitch, height pitch) pair."""

    def __init__(self, altitude_rules, gradient_rules, simplex_setting, map_size):
        h = C.c_void_p()
        alt = altitude_rules if isinstance(altitude_rules, C.Array) else \
            (AltitudeRule * len(altitude_rules))(*[AltitudeRule(*r) for r in altitude_rules])
        gra = gradient_rules if isinstance(gradient_rules, C.Array) else \
            (GradientRule * len(gradient_rules))(*[GradientRule(*r) for r in gradient_rules])
        check(lib().stpgb_splat_generator_create(alt, len(alt), gra, len(gra), C.byref(simplex_setting),
                                                 map_size[0], map_size[1], C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().stpgb_splat_generator_destroy(h)
            self._h = None

    def __call__(self, biomemap, heightmap, map_pitch, splatmap, splat_pitch, width, height, chunks, slope=None,
                 altitude=None, stream=None):
        import torch
        ch = (SplatChunk * max(len(chunks), 1))(*[c if isinstance(c, SplatChunk) else SplatChunk(*c)
                                                  for c in chunks])
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        bp, hp = map_pitch if isinstance(map_pitch, tuple) else (map_pitch, map_pitch)
        addr = lambda t: t if isinstance(t, int) else t.data_ptr()
        check(lib().stpgb_splatmap(self._h, C.c_void_p(addr(biomemap)), bp, C.c_void_p(addr(heightmap)), hp,
                                   C.c_void_p(addr(splatmap)), splat_pitch, width, height, ch, len(chunks),
                                   C.c_void_p(addr(slope) if slope is not None else 0),
                                   C.c_void_p(addr(altitude) if altitude is not None else 0), C.c_void_p(s)))


class STPFilterBuffer:
    """STPSingleHistogramFilter::STPFilterBuffer (STPSingleHistogramFilter.h:43-123).

    Holds the last filter output (host arrays).  The execution type is kept
    for API parity; both types run the same GPU filter and give identical
    results, as the reference's serial and parallel filters do."""

    Serial, Parallel = 0, 1

    def __init__(self, execution_type=Serial):
        if execution_type not in (self.Serial, self.Parallel):
            raise STPException(f"invalid STPExecutionType {execution_type}")
        self._type = execution_type
        self.offsets = np.zeros(0, np.uint32)
        self.bins = np.zeros(0, BIN_DTYPE)

    def type(self):
        return self._type

    def size(self):
        """(bin count, offset count), as STPFilterBuffer::size."""
        return len(self.bins), len(self.offsets)

    def readHistogram(self):
        return self.bins, self.offsets


class STPSingleHistogramFilter:
    """STPSingleHistogramFilter::operator() on the GPU (host arrays in and out)."""

    def __call__(self, samplemap, nn_info, filter_buffer, radius):
        sm = np.ascontiguousarray(samplemap, np.uint16)
        mx, my = nn_info.MapSize
        npix = mx * my
        offsets = np.zeros(npix + 1, np.uint32)
        cap = npix * min(256, (2 * radius + 1) ** 2) if radius else 0
        bins = np.zeros(max(cap, 1), BIN_DTYPE)
        n = C.c_uint64(0)
        rc = lib().stpgb_shf_filter_host(_p(sm), C.byref(nn_info), radius, _p(offsets), _p(bins), cap, C.byref(n))
        check(rc)
        filter_buffer.offsets = offsets
        filter_buffer.bins = bins[: n.value].copy()
        return filter_buffer.readHistogram()


# ------------------------------------------------------ plain generator


class STPDiversityGenerator:
    """STPDiversityGenerator (SuperTerrain+/World/Chunk/STPDiversityGenerator.hpp:14-39): subclass and
    implement __call__(heightmap, biomemap, offset, call), where `heightmap` (device address, MapSize
    float32, row-major) is the chunk to write, `biomemap` (device address) the merged biome
    neighbourhood, `offset` the chunk's map offset and `call` the full stpgb_diversity_call (nearest-
    neighbour information, stream).  Work goes on call.stream; an exception fails the generate call."""

    def __call__(self, heightmap, biomemap, offset, call):
        raise NotImplementedError

    def c_plugin(self):
        """The stpgb_diversity_generator that calls this object."""
        from ._capi import DIVERSITY_FN, DiversityGenerator

        def fn(user, call):
            c = call.contents
            try:
                self(c.heightmap, c.biomemap, (c.offset_x, c.offset_y), c)
                return STPGB_OK
            except Exception as e:  # the C boundary carries a status; the exception is kept for the caller
                self.error = e
                return STPGB_EINVAL

        self._fn = DIVERSITY_FN(fn)
        return DiversityGenerator(self._fn, None)


class STPBiomefieldGenerator:
    """The demo's multi-biome plugin STPBiomefieldGenerator (SuperDemo+/World/Biomes/
    STPBiomefieldGenerator.cpp:44-152): single histogram filter + multi-biome fractal simplex
    heightmap on the device (stpgb_biomefield_*)."""

    def __init__(self, simplex_setting, biome_table, interpolation_radius):
        table = np.ascontiguousarray(biome_table, BIOME_DTYPE)
        h = C.c_void_p()
        check(lib().stpgb_biomefield_create(C.byref(simplex_setting), _p(table), len(table), interpolation_radius,
                                            C.byref(h)), env_error=True)
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().stpgb_biomefield_destroy(h)
            self._h = None

    def c_plugin(self):
        from ._capi import DIVERSITY_FN, DiversityGenerator
        self._fn = DIVERSITY_FN(("stpgb_biomefield_generate", lib()))
        return DiversityGenerator(self._fn, self._h)


class STPHeightfieldGenerator:
    """STPHeightfieldGenerator over host arrays.  Either the reference's constructor,
    STPHeightfieldGenerator.setup(chunk_setting, raindrop_setting, diversity_generator)
    (STPHeightfieldGenerator.h:35-45,121), with any diversity plugin, or this constructor, which folds
    the demo's multi-biome plugin in."""

    def __init__(self, chunk_setting, raindrop_setting, simplex_setting, biome_table, interpolation_radius):
        table = np.ascontiguousarray(biome_table, BIOME_DTYPE)
        h = C.c_void_p()
        rc = lib().stpgb_generator_create(C.byref(chunk_setting), C.byref(raindrop_setting), C.byref(simplex_setting),
                                          _p(table), len(table), interpolation_radius, C.byref(h))
        check(rc, env_error=True)
        self._h = h
        self.chunk = chunk_setting
        self.raindrop = raindrop_setting
        self.plugin = None

    @classmethod
    def setup(cls, chunk_setting, raindrop_setting, diversity_generator):
        """STPHeightfieldGenerator(const STPGeneratorSetup&): `diversity_generator` is an
        STPDiversityGenerator subclass instance or an STPBiomefieldGenerator; it is kept alive by the
        generator."""
        from ._capi import GeneratorSetup
        self = cls.__new__(cls)
        self._h = None
        self.plugin = diversity_generator
        self._c_plugin = diversity_generator.c_plugin()
        st = GeneratorSetup(C.pointer(chunk_setting), C.pointer(raindrop_setting), C.pointer(self._c_plugin))
        h = C.c_void_p()
        check(lib().stpgb_generator_create_setup(C.byref(st), C.byref(h)), env_error=True)
        self._h = h
        self.chunk = chunk_setting
        self.raindrop = raindrop_setting
        return self

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().stpgb_generator_destroy(h)
            self._h = None

    def generate(self, heightfield, biomemap, offset):
        """heightfield: float32[MapSize] (written); biomemap: list of uint16 chunk arrays."""
        arrs = [np.ascontiguousarray(b, np.uint16) for b in biomemap]
        ptrs = (C.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
        assert heightfield.dtype == np.float32 and heightfield.flags.c_contiguous
        rc = lib().stpgb_generator_generate(self._h, _p(heightfield), ptrs, offset[0], offset[1])
        err = getattr(self.plugin, "error", None)
        if rc != STPGB_OK and err is not None:
            self.plugin.error = None
            raise err
        check(rc)

    def erode(self, heightfield, heightfield_fixed, starts=None):
        """heightfield: list of float32 chunks (in/out); heightfield_fixed: list of uint16 chunks (out).
        With `starts` (float32 xy pairs, merged coordinates) returns the residual sediment."""
        for a in heightfield:
            assert a.dtype == np.float32 and a.flags.c_contiguous
        for a in heightfield_fixed:
            assert a.dtype == np.uint16 and a.flags.c_contiguous
        hp = (C.c_void_p * len(heightfield))(*[a.ctypes.data for a in heightfield])
        fp = (C.c_void_p * len(heightfield_fixed))(*[a.ctypes.data for a in heightfield_fixed])
        if starts is None:
            check(lib().stpgb_generator_erode(self._h, hp, fp))
            return None
        st = np.ascontiguousarray(starts, np.float32)
        res = C.c_double(0.0)
        check(lib().stpgb_generator_erode_starts(self._h, hp, fp, _p(st), st.size // 2, C.byref(res)))
        return res.value


# ------------------------------------------------------- batched pipeline


class Batch:
    """Many eroded-chunk requests through one batched launch sequence (stpgb_batch_*).

    `requests`: iterable of dicts with MapSize, ChunkX, ChunkY, InterpolationRadius,
    DropletCount, BrushRadius, Lifetime.  `stream` arguments are raw
    cudaStream_t values (int) or None for the legacy default stream."""

    def __init__(self, requests, base_setting, simplex_setting, biome_table, hbm_budget=0, graph=True,
                 autotune=False):
        from ._capi import STPGB_BATCH_AUTOTUNE, STPGB_BATCH_GRAPH, BatchRequest
        reqs = list(requests)
        arr = (BatchRequest * len(reqs))(*[BatchRequest(**r) for r in reqs])
        table = np.ascontiguousarray(biome_table, BIOME_DTYPE)
        h = C.c_void_p()
        rc = lib().stpgb_batch_create(arr, len(reqs), C.byref(base_setting), C.byref(simplex_setting), _p(table),
                                      len(table), hbm_budget,
                                      (STPGB_BATCH_GRAPH if graph else 0) | (STPGB_BATCH_AUTOTUNE if autotune else 0),
                                      C.byref(h))
        check(rc)
        self._h = h
        self.requests = reqs

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().stpgb_batch_destroy(h)
            self._h = None

    @staticmethod
    def _s(stream):
        return C.c_void_p(stream or 0)

    @property
    def device_bytes(self):
        return int(lib().stpgb_batch_device_bytes(self._h))

    def buffers(self, i):
        b, hgt, fx, st = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
        check(lib().stpgb_batch_buffers(self._h, i, C.byref(b), C.byref(hgt), C.byref(fx), C.byref(st)))
        return b.value, hgt.value, fx.value, st.value

    def synthesize(self, voronoi_cell, seed, stream=None):
        check(lib().stpgb_batch_synthesize_inputs(self._h, voronoi_cell, seed, self._s(stream)))

    def synthesize_layer_biomes(self, seed, stream=None):
        """Biome regions from the demo's layer chain (after synthesize(), which makes the starts)."""
        check(lib().stpgb_batch_synthesize_layer_biomes(self._h, seed, self._s(stream)))

    def run(self, stream=None):
        check(lib().stpgb_batch_run(self._h, self._s(stream)))

    def run_plain(self, stream=None):
        check(lib().stpgb_batch_run_plain(self._h, self._s(stream)))

    def run_stage(self, stage, stream=None):
        check(lib().stpgb_batch_run_stage(self._h, stage, self._s(stream)))

    def upload(self, biome_regions, starts=None, stream=None):
        n = len(self.requests)
        bp = (C.c_void_p * n)(*[a.ctypes.data for a in biome_regions])
        sp = (C.c_void_p * n)(*[a.ctypes.data for a in starts]) if starts is not None else None
        check(lib().stpgb_batch_upload(self._h, bp, sp, self._s(stream)))

    def download(self, heights=None, fixed=None, residual=None, stream=None):
        n = len(self.requests)
        hp = (C.c_void_p * n)(*[_data(a) for a in heights]) if heights is not None else None
        fp = (C.c_void_p * n)(*[_data(a) for a in fixed]) if fixed is not None else None
        rp = residual.ctypes.data_as(C.c_void_p) if residual is not None else None
        check(lib().stpgb_batch_download(self._h, hp, fp, rp, self._s(stream)))

    def download_inputs(self, biome_regions=None, starts=None, stream=None):
        n = len(self.requests)
        bp = (C.c_void_p * n)(*[_data(a) for a in biome_regions]) if biome_regions is not None else None
        sp = (C.c_void_p * n)(*[_data(a) for a in starts]) if starts is not None else None
        check(lib().stpgb_batch_download_inputs(self._h, bp, sp, self._s(stream)))

    def status(self, stream=None):
        check(lib().stpgb_batch_status(self._h, self._s(stream)))

    def tune(self):
        """Autotune on the current inputs (synchronous) and re-capture the graph."""
        check(lib().stpgb_batch_tune(self._h))

    def tuning(self):
        """((lanes per droplet, droplets per group, brush rows) in use,
        {(lanes, droplets, rows): autotuner erosion ms}); rows is 1 for the
        brush updated in 16-byte row blocks, 0 for point by point."""
        lanes, dpg, rows = C.c_uint32(0), C.c_uint32(0), C.c_uint32(0)
        ms = (C.c_float * 36)()
        check(lib().stpgb_batch_tuning(self._h, C.byref(lanes), C.byref(dpg), C.byref(rows), ms))
        return ((lanes.value, dpg.value, rows.value),
                {(1 << ((i % 18) // 3), 1 << (i % 3), i // 18): ms[i] for i in range(36) if ms[i] > 0})

    def tuning_stages(self):
        """The autotuner's filter segment count (0 = from the launch size) and noise block size,
        with {candidate: ms} for each (candidates not tried are left out), and the jobs the
        warp-cooperative erosion kernel interleaves (0 where the dominant group runs another)."""
        seg, blk, q = C.c_uint32(0), C.c_uint32(0), C.c_uint32(0)
        sms, nms = (C.c_float * 6)(), (C.c_float * 3)()
        check(lib().stpgb_batch_tuning_stages(self._h, C.byref(seg), sms, C.byref(blk), nms, C.byref(q)))
        return (seg.value, {c: sms[i] for i, c in enumerate((0, 1, 2, 4, 8, 16)) if sms[i] > 0},
                blk.value, {c: nms[i] for i, c in enumerate((128, 256, 512)) if nms[i] > 0}, q.value)

    def tuning_filter_path(self):
        """The filter path the autotuner chose (0 by size, 1 few-values packed slides, 2 row bands,
        3 general slides) and {path: ms} for the ones it timed."""
        p = C.c_uint32(0)
        ms = (C.c_float * 4)()
        check(lib().stpgb_batch_tuning_filter_path(self._h, C.byref(p), ms))
        return p.value, {c: ms[c] for c in range(4) if ms[c] > 0}

    def kernels_per_run(self):
        """Kernels one run launches (the kernel nodes of the batch's graph)."""
        k = C.c_uint32(0)
        check(lib().stpgb_batch_kernels_per_run(self._h, C.byref(k)))
        return k.value

    def counters(self, reset=True):
        a, b = C.c_uint64(0), C.c_uint64(0)
        check(lib().stpgb_batch_counters(self._h, C.byref(a), C.byref(b), int(reset)))
        return a.value, b.value


# --------------------------------------------- kernel-level device calls


class DeviceOps:
    """Kernel-level calls on torch CUDA tensors (device pointers), enqueued on
    the current torch stream."""

    def __init__(self):
        import torch  # plumbing only: device memory and streams
        self.torch = torch

    def _stream(self):
        return C.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def empty(self, shape, dtype):
        return self.torch.empty(shape, dtype=dtype, device="cuda")

    def shf_filter(self, samplemap, map_size, nn, radius, max_items=0, bins_capacity=None, workspace=None):
        """samplemap: int16/uint16 tensor of TotalMapSize; returns (offsets i32, bins i64-view, status)."""
        t = self.torch
        info = NNInfo.make(map_size, nn)
        ws = C.c_size_t(0)
        check(lib().stpgb_shf_workspace_size(C.byref(info), radius, max_items, C.byref(ws)))
        if workspace is None or workspace.numel() < ws.value:
            workspace = self.empty(max(ws.value, 1), t.uint8)
        npix = map_size[0] * map_size[1]
        cap = bins_capacity if bins_capacity is not None else npix * min(max_items or 256, (2 * radius + 1) ** 2)
        offsets = self.empty(npix + 1, t.int32)
        bins = self.empty(max(cap, 1), t.int64)
        status = self.empty(1, t.int32)
        check(lib().stpgb_shf_filter(C.c_void_p(samplemap.data_ptr()), C.byref(info), radius, max_items,
                                     C.c_void_p(workspace.data_ptr()), ws.value, C.c_void_p(offsets.data_ptr()),
                                     C.c_void_p(bins.data_ptr()), cap, C.c_void_p(status.data_ptr()), self._stream()))
        return offsets, bins, status

    def shf_filter_path(self, workspace, map_size, nn, radius, max_items=0):
        """The path the last shf_filter call with `workspace` took: 0 the general slides, 1 the
        few-values packed slides, 2 the few-values row bands (at most 8 distinct values in the
        chunk's read region)."""
        info = NNInfo.make(map_size, nn)
        path = C.c_uint32(0)
        check(lib().stpgb_shf_filter_path(C.byref(info), radius, max_items, C.c_void_p(workspace.data_ptr()),
                                          C.byref(path), self._stream()))
        return path.value

    @staticmethod
    def shf_set_path(path):
        """Process-wide filter path for later launches: 0 by size, 1 packed slides, 2 row bands,
        3 general slides."""
        check(lib().stpgb_shf_set_path(path))

    def shf_workspace(self, map_size, nn, radius, max_items=0):
        """A device workspace of stpgb_shf_workspace_size bytes."""
        info = NNInfo.make(map_size, nn)
        ws = C.c_size_t(0)
        check(lib().stpgb_shf_workspace_size(C.byref(info), radius, max_items, C.byref(ws)))
        return self.empty(max(ws.value, 1), self.torch.uint8)

    def status_check(self, status):
        check(lib().stpgb_status_check(C.c_void_p(status.data_ptr()), self._stream()))

    def multibiome_heightmap(self, out, pitch, offsets, bins, map_size, offset, perm_dev, grad_dev, table_dev):
        p = Permutation(perm_dev.data_ptr(), grad_dev.data_ptr(), grad_dev.numel() // 2)
        check(lib().stpgb_multibiome_heightmap(C.c_void_p(out.data_ptr()), pitch, C.c_void_p(offsets.data_ptr()),
                                               C.c_void_p(bins.data_ptr()), map_size[0], map_size[1], offset[0],
                                               offset[1], C.byref(p), C.c_void_p(table_dev.data_ptr()),
                                               table_dev.numel() // 6, self._stream()))

    def droplet_starts(self, out, count, seed, counter_base, map_size, nn):
        info = NNInfo.make(map_size, nn)
        check(lib().stpgb_droplet_starts(C.c_void_p(out.data_ptr()), count, seed, counter_base, C.byref(info),
                                         self._stream()))

    def hydraulic_erosion(self, heightmap, map_size, nn, setting, starts, count, brush_index, brush_weight,
                          residual=None, status=None, lanes=0, exact_clamp=False, droplets_per_group=1,
                          pointwise=False):
        """stpgb_hydraulic_erosion_ex on a merged map tensor.  lanes=0 takes the default kernel for the
        brush and the droplet density; lanes=1 with row blocks allowed (pointwise=False, an aligned
        map) runs the warp-cooperative kernel, lanes=1 with pointwise=True the one-lane reference
        kernel, lanes=2/4 the lane-group kernels."""
        info = NNInfo.make(map_size, nn)
        check(lib().stpgb_hydraulic_erosion_ex(
            C.c_void_p(heightmap.data_ptr()), C.byref(info), C.byref(setting), C.c_void_p(starts.data_ptr()), count,
            C.c_void_p(brush_index.data_ptr()), C.c_void_p(brush_weight.data_ptr()), brush_index.numel(),
            C.c_void_p(residual.data_ptr() if residual is not None else 0),
            C.c_void_p(status.data_ptr() if status is not None else 0), lanes, droplets_per_group,
            int(exact_clamp) | (2 if pointwise else 0), self._stream()), env_error=True)

    def format_heightmap(self, src, dst, map_x, map_y):
        check(lib().stpgb_format_heightmap(C.c_void_p(src.data_ptr()), C.c_void_p(dst.data_ptr()), map_x, map_y,
                                           self._stream()))

    def layer_biomemap(self, chain, ids, global_seed, out, pitch, width, height, offset):
        chain = _layer_array(chain)
        check(lib().stpgb_layer_biomemap(chain, len(chain), global_seed, C.byref(ids), C.c_void_p(out.data_ptr()),
                                         pitch, width, height, int(offset[0]), int(offset[1]), self._stream()))

    def voronoi_biomemap(self, out, pitch, width, height, origin, cell, biome_count, seed):
        check(lib().stpgb_voronoi_biomemap(C.c_void_p(out.data_ptr()), pitch, width, height, origin[0], origin[1],
                                           cell, biome_count, seed, self._stream()))
