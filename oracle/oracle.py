"""ctypes front end of the oracle (test infrastructure only).

Only the tests, the smoke check and bench.py's CPU-baseline leg use this
module; it is what the product is compared with, never the product.  `Oracle` wraps the CPU
restatement (oracle/liboracle.so), `Reference` wraps the reference's own
compiled host sources (oracle/_ref/libstpref.so) and `DeviceReference` its
device code compiled as host C++ (oracle/_ref/libstpref_device.so), where
they could be built.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

BIN_DTYPE = np.dtype([("Item", "<u2"), ("_pad", "<u2"), ("Weight", "<f4")])
RAINDROP_FIELDS = [
    ("Seed", C.c_uint64), ("RainDropCount", C.c_uint32), ("Inertia", C.c_float),
    ("SedimentCapacityFactor", C.c_float), ("minSedimentCapacity", C.c_float),
    ("initWaterVolume", C.c_float), ("minWaterVolume", C.c_float), ("Friction", C.c_float),
    ("initSpeed", C.c_float), ("ErodeSpeed", C.c_float), ("DepositSpeed", C.c_float),
    ("EvaporateSpeed", C.c_float), ("Gravity", C.c_float), ("ErosionBrushRadius", C.c_uint32),
]
BIOME_DTYPE = np.dtype([("Scale", "<f4"), ("Octave", "<u4"), ("Persistence", "<f4"),
                        ("Lacunarity", "<f4"), ("Depth", "<f4"), ("Variation", "<f4")])


class OrcRaindrop(C.Structure):
    _fields_ = RAINDROP_FIELDS


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Oracle:
    def __init__(self):
        self.lib = C.CDLL(_build.build())
        L = self.lib
        vp, u32, u64, f32, f64, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float, C.c_double, C.c_int
        L.orc_permutation.argtypes = [u64, u32, f64, vp, vp]
        L.orc_permutation.restype = i32
        L.orc_shf.argtypes = [vp, u32, u32, u32, u32, u32, vp, vp, u64, C.POINTER(u64)]
        L.orc_shf.restype = i32
        L.orc_simplex2d.argtypes = [vp, vp, u32, f32, f32]
        L.orc_simplex2d.restype = f32
        L.orc_fractal.argtypes = [vp, vp, u32, f32, f32, f32, f32, u32, f32, f32, f32, f32, f32]
        L.orc_fractal.restype = f32
        L.orc_multibiome.argtypes = [vp, vp, vp, vp, vp, vp, u32, u32, u32, f32, f32, i32]
        L.orc_multibiome.restype = None
        L.orc_brush.argtypes = [u32, u32, vp, vp]
        L.orc_brush.restype = u32
        for name in ("orc_erode_f64", "orc_erode_f32"):
            fn = getattr(L, name)
            fn.argtypes = [vp, u32, u32, C.POINTER(OrcRaindrop), vp, u32, vp, vp, u32, C.POINTER(u64)]
            fn.restype = f64
        L.orc_format.argtypes = [vp, vp, u64]
        L.orc_format.restype = None
        L.orc_droplet_starts.argtypes = [vp, u32, u64, u64, u32, u32, u32, u32]
        L.orc_droplet_starts.restype = None
        L.orc_voronoi.argtypes = [vp, u32, u32, u32, C.c_int64, C.c_int64, u32, u32, u64]
        L.orc_voronoi.restype = None
        L.orc_layer_biomemap.argtypes = [vp, u32, u64, vp, vp, u32, u32, i32, i32]
        L.orc_layer_biomemap.restype = None
        L.orc_splatmap.argtypes = [vp, vp, u32, u32, u32, vp, u32, u32, u32, vp, u32, vp, vp, vp, vp, vp, u32, vp,
                                   u32, vp, vp]
        L.orc_splatmap.restype = None
        L.orc_mix_seed.argtypes = [u64, C.c_int64]
        L.orc_layer_seed.argtypes = [u64, u64]
        L.orc_local_seed.argtypes = [u64, u64, i32, i32]
        for name in ("orc_mix_seed", "orc_layer_seed", "orc_local_seed"):
            getattr(L, name).restype = u64

    # -- permutation
    def permutation(self, seed, distribution, offset):
        perm = np.zeros(512, np.uint8)
        grad = np.zeros(2 * max(distribution, 1), np.float32)
        rc = self.lib.orc_permutation(seed, distribution, offset, _p(perm), _p(grad))
        return rc, perm, grad

    # -- single histogram filter
    def shf(self, samplemap, map_size, nn, radius, capacity=None):
        mx, my = map_size
        samplemap = np.ascontiguousarray(samplemap, np.uint16)
        assert samplemap.size == mx * nn[0] * my * nn[1]
        offsets = np.zeros(mx * my + 1, np.uint32)
        cap = capacity if capacity is not None else mx * my * min(64, (2 * radius + 1) ** 2)
        bins = np.zeros(cap, BIN_DTYPE)
        n = C.c_uint64(0)
        rc = self.lib.orc_shf(_p(samplemap), mx, my, nn[0], nn[1], radius, _p(offsets), _p(bins), cap, C.byref(n))
        if rc == 5:
            return self.shf(samplemap, map_size, nn, radius, capacity=n.value)
        return rc, offsets, bins[: n.value]

    # -- noise
    def multibiome(self, offsets, bins, table, perm, grad, map_size, offset, threads=1):
        mx, my = map_size
        out = np.zeros(mx * my, np.float32)
        bins = np.ascontiguousarray(bins, BIN_DTYPE)
        table = np.ascontiguousarray(table, BIOME_DTYPE)
        self.lib.orc_multibiome(_p(out), _p(np.ascontiguousarray(offsets, np.uint32)), _p(bins), _p(table),
                                _p(perm), _p(grad), len(grad) // 2, mx, my, offset[0], offset[1], threads)
        return out.reshape(my, mx)

    # -- brush
    def brush(self, dim_x, radius):
        cap = (2 * radius + 1) ** 2
        idx = np.zeros(cap, np.int32)
        w = np.zeros(cap, np.float32)
        n = self.lib.orc_brush(dim_x, radius, _p(idx), _p(w))
        return idx[:n], w[:n]

    # -- erosion
    def erode(self, heightmap, setting, starts, brush_index, brush_weight, fp64=True):
        """Serial droplets; returns (map, residual sediment, realised steps)."""
        dim_y, dim_x = heightmap.shape
        s = OrcRaindrop(**setting)
        starts = np.ascontiguousarray(starts, np.float32)
        steps = C.c_uint64(0)
        if fp64:
            m = np.ascontiguousarray(heightmap, np.float64).copy()
            fn = self.lib.orc_erode_f64
        else:
            m = np.ascontiguousarray(heightmap, np.float32).copy()
            fn = self.lib.orc_erode_f32
        res = fn(_p(m), dim_x, dim_y, C.byref(s), _p(starts), len(starts) // 2,
                 _p(np.ascontiguousarray(brush_index, np.int32)), _p(np.ascontiguousarray(brush_weight, np.float32)),
                 len(brush_index), C.byref(steps))
        return m, res, steps.value

    def format(self, heightmap):
        h = np.ascontiguousarray(heightmap, np.float32)
        out = np.zeros(h.shape, np.uint16)
        self.lib.orc_format(_p(h), _p(out), h.size)
        return out

    def droplet_starts(self, count, seed, counter_base, map_size, nn):
        xy = np.zeros(2 * count, np.float32)
        self.lib.orc_droplet_starts(_p(xy), count, seed, counter_base, map_size[0], map_size[1], nn[0], nn[1])
        return xy

    def voronoi(self, width, height, origin, cell, biome_count, seed):
        out = np.zeros((height, width), np.uint16)
        self.lib.orc_voronoi(_p(out), width, width, height, origin[0], origin[1], cell, biome_count, seed)
        return out


    # -- biome layer chain
    def layer_biomemap(self, chain, ids, seed, width, height, offset):
        """chain: sequence of (kind, param, salt), first ancestor first; ids: (ocean, plains, forest, 5 x shallow)."""
        desc = np.array([tuple(c) for c in chain], LAYER_DTYPE)
        idv = np.ascontiguousarray(ids, np.uint16)
        assert idv.size == 8
        out = np.zeros((height, width), np.uint16)
        self.lib.orc_layer_biomemap(_p(desc), len(desc), seed, _p(idv), _p(out), width, height, offset[0], offset[1])
        return out

    def mix_seed(self, s, fac):
        return self.lib.orc_mix_seed(s, fac)

    def layer_seed(self, global_seed, salt):
        return self.lib.orc_layer_seed(global_seed, salt)

    def local_seed(self, global_seed, salt, x, z):
        return self.lib.orc_local_seed(global_seed, salt, x, z)


    # -- splatmap
    def splatmap(self, biomemap, heightmap, chunks, map_size, altitude_rules, gradient_rules, perm, grad):
        """Region map (uint8, 255 = none), slope factor and tested altitude of the requested chunks
        of a rendering buffer; chunks: (local x, local y, map offset x, map offset y);
        rules: (sample, upper bound, region) and (sample, min g, max g, lower, upper, region)."""
        h, w = heightmap.shape
        dict_, reg, alt, gra = splat_rule_tables(altitude_rules, gradient_rules)
        ch = np.array([tuple(c) for c in chunks], SPLAT_CHUNK_DTYPE)
        out = np.full((h, w), 0, np.uint8)
        slope = np.zeros((h, w), np.float32)
        altitude = np.zeros((h, w), np.float32)
        self.lib.orc_splatmap(_p(np.ascontiguousarray(biomemap, np.uint16)), _p(np.ascontiguousarray(heightmap,
                              np.uint16)), w, w, h, _p(ch), len(ch), map_size[0], map_size[1], _p(dict_), len(dict_),
                              _p(reg), _p(alt), _p(gra), _p(perm), _p(grad), len(grad) // 2, _p(out), w, _p(slope),
                              _p(altitude))
        return out, slope, altitude


SPLAT_CHUNK_DTYPE = np.dtype([("lx", "<u4"), ("ly", "<u4"), ("ox", "<f4"), ("oy", "<f4")])
SPLAT_REG_DTYPE = np.dtype([("AltitudeEntry", "<u4"), ("AltitudeSize", "<u4"), ("GradientEntry", "<u4"),
                            ("GradientSize", "<u4")])
ALT_NODE_DTYPE = np.dtype([("RegionIndex", "<u4"), ("UpperBound", "<f4")])
GRA_NODE_DTYPE = np.dtype([("RegionIndex", "<u4"), ("minGradient", "<f4"), ("maxGradient", "<f4"),
                           ("LowerBound", "<f4"), ("UpperBound", "<f4")])


def splat_rule_tables(altitude_rules, gradient_rules):
    """The rule database as the reference's texture database orders it
    (SuperTerrain+/Private/World/Diversity/STPTextureDatabase.cpp:357-411,
    STPTextureFactory.cpp:138-172): samples ascending; per sample its
    altitude rules by upper bound and its gradient rules in the order added."""
    alt = sorted(enumerate(altitude_rules), key=lambda t: (t[1][0], t[1][1], t[0]))
    gra = sorted(enumerate(gradient_rules), key=lambda t: (t[1][0], t[0]))
    samples = sorted({r[0] for _, r in alt} | {r[0] for _, r in gra})
    reg = np.zeros(max(len(samples), 1), SPLAT_REG_DTYPE)
    an, gn = [], []
    for d, smp in enumerate(samples):
        reg[d]["AltitudeEntry"] = len(an)
        an += [(r[2], r[1]) for _, r in alt if r[0] == smp]
        reg[d]["AltitudeSize"] = len(an) - reg[d]["AltitudeEntry"]
        reg[d]["GradientEntry"] = len(gn)
        gn += [(r[5], r[1], r[2], r[3], r[4]) for _, r in gra if r[0] == smp]
        reg[d]["GradientSize"] = len(gn) - reg[d]["GradientEntry"]
    # the node arrays keep one unused entry when empty so that they have an address
    return (np.array(samples, np.uint16), reg, np.array(an or [(0, 0.0)], ALT_NODE_DTYPE),
            np.array(gn or [(0, 0.0, 0.0, 0.0, 0.0)], GRA_NODE_DTYPE))


LAYER_DTYPE = np.dtype([("Kind", "<u4"), ("Param", "<u4"), ("Salt", "<u8")])


class Reference:
    """The reference's own STPSingleHistogramFilter / STPPermutationGenerator, compiled from its sources."""

    def __init__(self, path=None):
        path = path or _build.build_ref()
        if not path or not os.path.exists(path):
            raise FileNotFoundError("reference build unavailable")
        self.lib = C.CDLL(path)
        vp, u32, u64 = C.c_void_p, C.c_uint32, C.c_uint64
        self.lib.ref_shf.argtypes = [vp, u32, u32, u32, u32, u32, C.c_int, vp, vp, u64, C.POINTER(u64)]
        self.lib.ref_shf.restype = C.c_int
        self.lib.ref_permutation.argtypes = [u64, u32, C.c_double, vp, vp]
        self.lib.ref_permutation.restype = C.c_int
        u16, i32 = C.c_uint16, C.c_int32
        self.lib.ref_layer_biomemap.argtypes = [u64, u16, u16, u16, u16, u32, u32, i32, i32, vp]
        self.lib.ref_layer_biomemap.restype = C.c_int
        self.lib.ref_mix_seed.argtypes = [u64, C.c_int64]
        self.lib.ref_layer_seed.argtypes = [u64, u64]
        self.lib.ref_local_seed.argtypes = [u64, u64, i32, i32]
        for name in ("ref_mix_seed", "ref_layer_seed", "ref_local_seed"):
            getattr(self.lib, name).restype = u64

    def shf(self, samplemap, map_size, nn, radius, parallel=False, capacity=None):
        mx, my = map_size
        samplemap = np.ascontiguousarray(samplemap, np.uint16)
        offsets = np.zeros(mx * my + 1, np.uint32)
        cap = capacity if capacity is not None else mx * my * min(64, (2 * radius + 1) ** 2)
        bins = np.zeros(max(cap, 1), BIN_DTYPE)
        n = C.c_uint64(0)
        rc = self.lib.ref_shf(_p(samplemap), mx, my, nn[0], nn[1], radius, int(parallel), _p(offsets), _p(bins),
                              cap, C.byref(n))
        if rc == 5:
            return self.shf(samplemap, map_size, nn, radius, parallel, capacity=n.value)
        return rc, offsets, bins[: n.value]

    def permutation(self, seed, distribution, offset):
        perm = np.zeros(512, np.uint8)
        grad = np.zeros(2 * max(distribution, 1), np.float32)
        rc = self.lib.ref_permutation(seed, distribution, offset, _p(perm), _p(grad))
        return rc, perm, grad

    def layer_biomemap(self, seed, width, height, offset, ocean=0, plains=1, desert=2, forest=3):
        """The demo's STPLayerChainBuilder through STPBiomeFactory::operator()."""
        out = np.zeros((height, width), np.uint16)
        rc = self.lib.ref_layer_biomemap(seed, ocean, plains, desert, forest, width, height, offset[0], offset[1],
                                         _p(out))
        assert rc == 0
        return out

    def mix_seed(self, s, fac):
        return self.lib.ref_mix_seed(s, fac)

    def layer_seed(self, global_seed, salt):
        return self.lib.ref_layer_seed(global_seed, salt)

    def local_seed(self, global_seed, salt, x, z):
        return self.lib.ref_local_seed(global_seed, salt, x, z)


class DeviceReference:
    """The reference's own device code compiled as host C++ (oracle/_ref/libstpref_device.so):
    simplex2D / simplex2DFractal (STPSimplexNoise.cu), the droplet (STPRainDrop.cu), the demo's
    multi-biome generator script (STPMultiHeightGenerator.cu, two biomes), the demo's splatmap
    script with the rule lookups (STPSplatmapGenerator.cu, STPTextureSplatRuleWrapper.cu; texture
    fetches and rnormf are stand-ins), the erosion kernel with its droplet spawn
    (STPHeightfieldKernel.cu:80-108; curand draws supplied by the caller), the erosion brush generator
    (STPHeightfieldGenerator.cpp:44-77) and the format kernel (STPHeightfieldKernel.cu:110-121).
    Kernels run as serial host loops; every float operation rounds as written."""

    def __init__(self, path=None):
        path = path or _build.build_ref(device=True)
        if not path or not os.path.exists(path):
            raise FileNotFoundError("reference device build unavailable")
        self.lib = L = C.CDLL(path)
        vp, u32, f32 = C.c_void_p, C.c_uint32, C.c_float
        L.ref_simplex2d.argtypes = [vp, vp, u32, f32, f32]
        L.ref_simplex2d.restype = f32
        L.ref_fractal.argtypes = [vp, vp, u32, f32, f32, f32, f32, u32, f32, f32, f32, f32, f32]
        L.ref_fractal.restype = f32
        L.ref_multibiome.argtypes = [vp, vp, vp, vp, vp, vp, u32, u32, u32, f32, f32]
        L.ref_multibiome.restype = C.c_int
        L.ref_erode.argtypes = [vp, u32, u32, vp, vp, u32, vp, vp, u32]
        L.ref_erode.restype = C.c_int
        L.ref_brush.argtypes = [u32, u32, vp, vp]
        L.ref_brush.restype = u32
        L.ref_format.argtypes = [vp, vp, u32]
        L.ref_format.restype = None
        L.ref_splatmap.argtypes = [vp, vp, u32, u32, u32, vp, u32, u32, u32, vp, u32, vp, vp, vp, vp, vp, u32, vp, u32]
        L.ref_splatmap.restype = C.c_int
        L.ref_erosion_kernel.argtypes = [vp, vp, vp, vp, vp, u32, vp, vp, u32]
        L.ref_erosion_kernel.restype = C.c_int

    def simplex2d(self, perm, grad, x, y):
        return self.lib.ref_simplex2d(_p(perm), _p(grad), len(grad) // 2, x, y)

    def fractal(self, perm, grad, x, y, pers, lacu, oct, scale, off, half):
        return self.lib.ref_fractal(_p(perm), _p(grad), len(grad) // 2, x, y, pers, lacu, oct, scale, off[0], off[1],
                                    half[0], half[1])

    def multibiome(self, offsets, bins, table, perm, grad, map_size, offset):
        mx, my = map_size
        out = np.zeros(mx * my, np.float32)
        table = np.ascontiguousarray(table, BIOME_DTYPE)
        assert len(table) == 2
        rc = self.lib.ref_multibiome(_p(out), _p(np.ascontiguousarray(offsets, np.uint32)),
                                     _p(np.ascontiguousarray(bins, BIN_DTYPE)), _p(table), _p(perm), _p(grad),
                                     len(grad) // 2, mx, my, offset[0], offset[1])
        assert rc == 0, "the generator script's biome table holds biomes 0 and 1 only"
        return out.reshape(my, mx)

    def erode(self, heightmap, setting, starts, brush_index, brush_weight):
        """Droplets one after another in start order on a float32 copy of `heightmap`."""
        dim_y, dim_x = heightmap.shape
        m = np.ascontiguousarray(heightmap, np.float32).copy()
        s = OrcRaindrop(**setting)
        starts = np.ascontiguousarray(starts, np.float32)
        rc = self.lib.ref_erode(_p(m), dim_x, dim_y, C.byref(s), _p(starts), len(starts) // 2,
                                _p(np.ascontiguousarray(brush_index, np.int32)),
                                _p(np.ascontiguousarray(brush_weight, np.float32)), len(brush_index))
        assert rc == 0
        return m

    def brush(self, dim_x, radius):
        cap = (2 * radius + 1) ** 2
        idx = np.zeros(cap, np.int32)
        w = np.zeros(cap, np.float32)
        n = self.lib.ref_brush(dim_x, radius, _p(idx), _p(w))
        return idx[:n], w[:n]

    def format(self, heightmap):
        h = np.ascontiguousarray(heightmap, np.float32).ravel()
        out = np.zeros(h.shape, np.uint16)
        self.lib.ref_format(_p(h), _p(out), h.size)
        return out.reshape(np.shape(heightmap))

    def splatmap(self, biomemap, heightmap, chunks, map_size, altitude_rules, gradient_rules, perm, grad):
        """Region map (uint8, 255 = none) of the requested chunks, as Oracle.splatmap."""
        h, w = heightmap.shape
        dict_, reg, alt, gra = splat_rule_tables(altitude_rules, gradient_rules)
        ch = np.array([tuple(c) for c in chunks], SPLAT_CHUNK_DTYPE)
        out = np.zeros((h, w), np.uint8)
        rc = self.lib.ref_splatmap(_p(np.ascontiguousarray(biomemap, np.uint16)),
                                   _p(np.ascontiguousarray(heightmap, np.uint16)), w, w, h, _p(ch), len(ch),
                                   map_size[0], map_size[1], _p(dict_), len(dict_), _p(reg), _p(alt), _p(gra),
                                   _p(perm), _p(grad), len(grad) // 2, _p(out), w)
        assert rc == 0, "a write left the surface"
        return out

    def erosion_kernel(self, heightmap, map_size, nn, setting, uniforms, brush_index, brush_weight):
        """hydraulicErosionKERNEL over droplets 0..count-1 in index order on a float32 copy of the
        merged map; `uniforms` holds each droplet's two curand_uniform draws."""
        m = np.ascontiguousarray(heightmap, np.float32).copy()
        s = OrcRaindrop(**setting)
        u = np.ascontiguousarray(uniforms, np.float32)
        ms, n = np.array(map_size, np.uint32), np.array(nn, np.uint32)
        rc = self.lib.ref_erosion_kernel(_p(m), _p(ms), _p(n), C.byref(s), _p(u), len(u) // 2,
                                         _p(np.ascontiguousarray(brush_index, np.int32)),
                                         _p(np.ascontiguousarray(brush_weight, np.float32)), len(brush_index))
        assert rc == 0
        return m


def spawn_draws(starts, map_size, nn, guess=None):
    """Draws in (0, 1] for the reference kernel's own spawn (u * (MapSize - 1) + (NN / 2) * MapSize,
    STPHeightfieldKernel.cu:93-104) that give exactly `starts` (x, y interleaved) whether the
    compiler evaluates the multiply-add in two roundings or fuses it into one: per coordinate the
    float nearest to `guess` (default (start - offset) / (MapSize - 1)) for which both evaluations
    land on the start.  Returns (draws, the fraction of droplets whose two draws meet that)."""
    starts = np.ascontiguousarray(starts, np.float32)
    count = len(starts) // 2
    base = np.tile(np.array([map_size[0] - 1, map_size[1] - 1], np.float32), count)
    rng = np.tile(np.array([(nn[0] // 2) * map_size[0], (nn[1] // 2) * map_size[1]], np.float32), count)
    if guess is None:
        guess = ((starts.astype(np.float64) - rng) / base).astype(np.float32)
    u = np.clip(np.asarray(guess, np.float32), np.float32(2.0 ** -24), np.float32(1.0))
    # two roundings (float32 operations); one rounding (the product and sum are exact in float64)
    plain = lambda v: v * base + rng
    fused = lambda v: (v.astype(np.float64) * base.astype(np.float64) + rng.astype(np.float64)).astype(np.float32)
    both = lambda v: (plain(v) == starts) & (fused(v) == starts)
    out = u.copy()
    done = both(u)
    for k in (1, -1, 2, -2, 3, -3, 4, -4, 5, -5, 6, -6):
        cand = (u.view(np.int32) + np.int32(k)).view(np.float32)
        ok = ~done & (cand > 0.0) & (cand <= 1.0) & both(cand)
        out[ok] = cand[ok]
        done |= ok
    pair = done.reshape(-1, 2).all(axis=1)
    return out, float(pair.mean()) if count else 1.0


def droplet_draws(oracle, count, seed, counter_base, map_size, nn):
    """Draws for the reference kernel's spawn that place exactly the droplets
    oracle.droplet_starts(count, seed, counter_base, map_size, nn) places: each droplet's Philox
    draws (the starts of a 1x1 neighbourhood of 2^2 chunks, whose spawn maps u to u), or the nearest
    floats to them that spawn_draws accepts.  Returns (draws, fraction spawned exactly)."""
    u = oracle.droplet_starts(count, seed, counter_base, (2, 2), (1, 1))
    return spawn_draws(oracle.droplet_starts(count, seed, counter_base, map_size, nn), map_size, nn, guess=u)


class ReferenceGPU:
    """The reference's erosion kernel (hydraulicErosionKERNEL with STPRainDrop, STPHeightfieldKernel.cu:80-108,
    STPRainDrop.cu) compiled by nvcc for sm_103a with the reference's release flags
    (oracle/_ref/libstpref_gpu.so, oracle/build_ref.sh).  Test infrastructure only: its run-to-run
    spread is the erosion tolerance.  Arguments are device addresses (integers); each droplet's two
    curand draws come from `uniforms` (2 floats per droplet in (0, 1]), so it erodes the same droplets
    as a kernel fed the starts those draws map to."""

    def __init__(self, path=None):
        path = path or _build.build_ref(gpu=True)
        if not path or not os.path.exists(path):
            raise FileNotFoundError("reference GPU build unavailable")
        self.lib = L = C.CDLL(path)
        vp, u32 = C.c_void_p, C.c_uint32
        L.ref_gpu_erosion.argtypes = [vp, u32, u32, u32, u32, vp, vp, u32, vp, vp, u32, vp]
        L.ref_gpu_erosion.restype = C.c_int
        L.ref_gpu_erosion_block_size.argtypes = [u32]
        L.ref_gpu_erosion_block_size.restype = C.c_int

    def erode(self, map_ptr, map_size, nn, setting, uniforms_ptr, count, brush_index_ptr, brush_weight_ptr,
              brush_size, stream=0):
        """One launch on the device map at `map_ptr`; synchronises `stream`."""
        s = OrcRaindrop(**setting)
        rc = self.lib.ref_gpu_erosion(C.c_void_p(map_ptr), map_size[0], map_size[1], nn[0], nn[1], C.byref(s),
                                      C.c_void_p(uniforms_ptr), count, C.c_void_p(brush_index_ptr),
                                      C.c_void_p(brush_weight_ptr), brush_size, C.c_void_p(stream))
        if rc != 0:
            raise RuntimeError(f"reference erosion kernel: CUDA error {rc}")

    def block_size(self, brush_size):
        return self.lib.ref_gpu_erosion_block_size(brush_size)
