"""ctypes binding of libstpgb.so (the C ABI declared in include/stpgb.h).

The library must exist: importing this module without it raises, there is
no fallback path.  Status codes are turned into the exception types the
reference throws (STPNumericDomainError, STPInvalidEnvironment,
STPCUDAError) plus STPTimeout / STPInsufficientMemory / STPCapacityError.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libstpgb.so")

STPGB_OK, STPGB_EINVAL, STPGB_ECUDA, STPGB_ETIMEOUT, STPGB_ENOMEM, STPGB_ECAPACITY = range(6)


class STPException(RuntimeError):
    """Base of the error types (SuperTerrain+/SuperTerrain+/Public/SuperTerrain+/Exception)."""


class STPNumericDomainError(STPException):
    pass


class STPInvalidEnvironment(STPException):
    pass


class STPCUDAError(STPException):
    pass


class STPTimeout(STPException):
    pass


class STPInsufficientMemory(STPException):
    pass


class STPCapacityError(STPException):
    pass


class NNInfo(C.Structure):
    _fields_ = [("MapSize", C.c_uint32 * 2), ("ChunkNearestNeighbour", C.c_uint32 * 2),
                ("TotalMapSize", C.c_uint32 * 2)]

    @classmethod
    def make(cls, map_size, nn):
        i = cls()
        i.MapSize[:] = list(map_size)
        i.ChunkNearestNeighbour[:] = list(nn)
        i.TotalMapSize[:] = [map_size[0] * nn[0], map_size[1] * nn[1]]
        return i


class SimplexSetting(C.Structure):
    _fields_ = [("Seed", C.c_uint64), ("Distribution", C.c_uint32), ("Offset", C.c_double)]


class RaindropSetting(C.Structure):
    _fields_ = [
        ("Seed", C.c_uint64), ("RainDropCount", C.c_uint32), ("Inertia", C.c_float),
        ("SedimentCapacityFactor", C.c_float), ("minSedimentCapacity", C.c_float),
        ("initWaterVolume", C.c_float), ("minWaterVolume", C.c_float), ("Friction", C.c_float),
        ("initSpeed", C.c_float), ("ErodeSpeed", C.c_float), ("DepositSpeed", C.c_float),
        ("EvaporateSpeed", C.c_float), ("Gravity", C.c_float), ("ErosionBrushRadius", C.c_uint32),
    ]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class BiomeProperty(C.Structure):
    _fields_ = [("Scale", C.c_float), ("Octave", C.c_uint32), ("Persistence", C.c_float),
                ("Lacunarity", C.c_float), ("Depth", C.c_float), ("Variation", C.c_float)]


class Permutation(C.Structure):
    _fields_ = [("Permutation", C.c_void_p), ("Gradient2D", C.c_void_p), ("Gradient2DSize", C.c_uint32)]


class ChunkSetting(C.Structure):
    _fields_ = [("MapSize", C.c_uint32 * 2), ("DiversityNearestNeighbour", C.c_uint32 * 2),
                ("ErosionNearestNeighbour", C.c_uint32 * 2)]


vp, u16, u32, u64, i32, i64, f32, f64, sz = (C.c_void_p, C.c_uint16, C.c_uint32, C.c_uint64, C.c_int32,
                                             C.c_int64, C.c_float, C.c_double, C.c_size_t)

class BatchRequest(C.Structure):
    _fields_ = [("MapSize", C.c_uint32), ("ChunkX", C.c_int32), ("ChunkY", C.c_int32),
                ("InterpolationRadius", C.c_uint32), ("DropletCount", C.c_uint32), ("BrushRadius", C.c_uint32),
                ("Lifetime", C.c_uint32)]


class ServerConfig(C.Structure):
    _fields_ = [("HbmBudget", C.c_uint64), ("MaxInFlight", C.c_uint32), ("MaxBatch", C.c_uint32),
                ("Streams", C.c_uint32), ("VoronoiCell", C.c_uint32), ("BiomeSeed", C.c_uint64),
                ("BiomeSource", C.c_uint32), ("ErosionMode", C.c_uint32)]


STPGB_BIOMES_VORONOI, STPGB_BIOMES_LAYER_CHAIN = 0, 1
STPGB_EROSION_PRIVATE, STPGB_EROSION_IN_PLACE = 0, 1


class ServeRequest(C.Structure):
    _fields_ = [("ChunkX", C.c_int32), ("ChunkY", C.c_int32), ("MapSize", C.c_uint32),
                ("InterpolationRadius", C.c_uint32), ("DropletsPerPixel", C.c_float), ("BrushRadius", C.c_uint32),
                ("Lifetime", C.c_uint32), ("UserTag", C.c_uint64)]


class ServeResult(C.Structure):
    _fields_ = [("Ticket", C.c_uint64), ("UserTag", C.c_uint64), ("Status", C.c_int), ("MapSize", C.c_uint32),
                ("LatencyMs", C.c_double), ("Heightmap", C.c_void_p), ("HeightmapFixed", C.c_void_p),
                ("ResidualSediment", C.c_double), ("ErosionOrder", C.c_uint64)]


class ServerStats(C.Structure):
    _fields_ = [("Submitted", C.c_uint64), ("Admitted", C.c_uint64), ("Completed", C.c_uint64),
                ("Launches", C.c_uint64), ("ChunksGenerated", C.c_uint64), ("ChunksEvicted", C.c_uint64),
                ("PoolBytesUsed", C.c_uint64), ("ResidentChunks", C.c_uint64)]


class Layer(C.Structure):
    _fields_ = [("Kind", u32), ("Param", u32), ("Salt", u64)]


class LayerBiomes(C.Structure):
    _fields_ = [("Ocean", u16), ("Plains", u16), ("Forest", u16), ("ShallowOcean", u16 * 5)]


STPGB_LAYER_CONTINENT, STPGB_LAYER_SCALE, STPGB_LAYER_LAND, STPGB_LAYER_ISLAND, STPGB_LAYER_VORONOI = range(1, 6)
STPGB_SCALE_NORMAL, STPGB_SCALE_FUZZY = 0, 1
STPGB_MAX_LAYERS = 32

class AltitudeRule(C.Structure):
    _fields_ = [("Sample", u16), ("UpperBound", f32), ("RegionIndex", u32)]


class GradientRule(C.Structure):
    _fields_ = [("Sample", u16), ("minGradient", f32), ("maxGradient", f32), ("LowerBound", f32),
                ("UpperBound", f32), ("RegionIndex", u32)]


class SplatChunk(C.Structure):
    _fields_ = [("LocalChunkCoordinateX", u32), ("LocalChunkCoordinateY", u32), ("ChunkMapOffsetX", f32),
                ("ChunkMapOffsetY", f32)]


class DiversityCall(C.Structure):
    """stpgb_diversity_call: one call of a multi-biome heightmap plugin (STPDiversityGenerator::operator())."""
    _fields_ = [("heightmap", vp), ("biomemap", vp), ("biomemap_chunks_host", vp), ("heightmap_nn", NNInfo),
                ("biomemap_nn", NNInfo), ("offset_x", f32), ("offset_y", f32), ("stream", vp)]


DIVERSITY_FN = C.CFUNCTYPE(C.c_int, vp, C.POINTER(DiversityCall))


class DiversityGenerator(C.Structure):
    _fields_ = [("generate", DIVERSITY_FN), ("user", vp)]


class GeneratorSetup(C.Structure):
    _fields_ = [("ChunkSetting", C.POINTER(ChunkSetting)), ("RainDropSetting", C.POINTER(RaindropSetting)),
                ("DiversityGenerator", C.POINTER(DiversityGenerator))]


STPGB_BATCH_GRAPH = 1
STPGB_BATCH_AUTOTUNE = 2

# name -> (restype, argtypes); the single source of the binding
PROTOTYPES = {
    "stpgb_last_error": (C.c_char_p, []),
    "stpgb_version": (C.c_char_p, []),
    "stpgb_simplex_setting_validate": (C.c_int, [C.POINTER(SimplexSetting)]),
    "stpgb_raindrop_setting_validate": (C.c_int, [C.POINTER(RaindropSetting)]),
    "stpgb_permutation_generate": (C.c_int, [C.POINTER(SimplexSetting), vp, vp, u32]),
    "stpgb_erosion_brush_generate": (C.c_int, [u32, u32, vp, vp, u32, C.POINTER(u32)]),
    "stpgb_lifetime_min_water_volume": (f32, [f32, f32, u32]),
    "stpgb_chunk_world_coordinate": (C.c_int, [f64, f64, vp, vp, vp]),
    "stpgb_chunk_local_coordinate": (C.c_int, [u32, vp, vp]),
    "stpgb_chunk_local_origin": (C.c_int, [vp, vp, vp, vp]),
    "stpgb_chunk_map_offset": (C.c_int, [vp, vp, vp, vp, vp]),
    "stpgb_chunk_offset": (C.c_int, [vp, vp, vp, vp]),
    "stpgb_chunk_neighbour_offset": (C.c_int, [vp, vp, vp, u32, C.POINTER(u32)]),
    "stpgb_nn_merge_host": (C.c_int, [vp, u32, C.POINTER(NNInfo), vp]),
    "stpgb_nn_unmerge_host": (C.c_int, [vp, u32, C.POINTER(NNInfo), vp]),
    "stpgb_shf_workspace_size": (C.c_int, [C.POINTER(NNInfo), u32, u32, C.POINTER(sz)]),
    "stpgb_shf_filter": (C.c_int, [vp, C.POINTER(NNInfo), u32, u32, vp, sz, vp, vp, u64, vp, vp]),
    "stpgb_shf_filter_host": (C.c_int, [vp, C.POINTER(NNInfo), u32, vp, vp, u64, C.POINTER(u64)]),
    "stpgb_shf_filter_noalloc": (C.c_int, [vp, C.POINTER(NNInfo), u32, u32, vp, vp, u64, vp, vp]),
    "stpgb_shf_filter_path": (C.c_int, [C.POINTER(NNInfo), u32, u32, vp, C.POINTER(u32), vp]),
    "stpgb_shf_set_path": (C.c_int, [u32]),
    "stpgb_status_check": (C.c_int, [vp, vp]),
    "stpgb_multibiome_heightmap": (C.c_int, [vp, u32, vp, vp, u32, u32, f32, f32, C.POINTER(Permutation), vp,
                                             u32, vp]),
    "stpgb_droplet_starts": (C.c_int, [vp, u32, u64, u64, C.POINTER(NNInfo), vp]),
    "stpgb_hydraulic_erosion": (C.c_int, [vp, C.POINTER(NNInfo), C.POINTER(RaindropSetting), vp, u32, vp, vp, u32,
                                          vp, vp, vp]),
    "stpgb_hydraulic_erosion_ex": (C.c_int, [vp, C.POINTER(NNInfo), C.POINTER(RaindropSetting), vp, u32, vp, vp,
                                             u32, vp, vp, u32, u32, u32, vp]),
    "stpgb_format_heightmap": (C.c_int, [vp, vp, u32, u32, vp]),
    "stpgb_erosion_choice": (C.c_int, [u32, u32, u32, C.POINTER(u32), C.POINTER(u32)]),
    "stpgb_voronoi_biomemap": (C.c_int, [vp, u32, u32, u32, i64, i64, u32, u32, u64, vp]),
    "stpgb_layer_chain_demo": (C.c_int, [vp, u32, C.POINTER(u32)]),
    "stpgb_splat_rules_demo": (C.c_int, [vp, u32, C.POINTER(u32), vp, u32, C.POINTER(u32)]),
    "stpgb_splat_generator_create": (C.c_int, [vp, u32, vp, u32, C.POINTER(SimplexSetting), u32, u32,
                                               C.POINTER(vp)]),
    "stpgb_splat_generator_destroy": (C.c_int, [vp]),
    "stpgb_splatmap": (C.c_int, [vp, vp, u32, vp, u32, vp, u32, u32, u32, vp, u32, vp, vp, vp]),
    "stpgb_layer_biomes_demo": (None, [C.POINTER(LayerBiomes)]),
    "stpgb_layer_biomemap": (C.c_int, [vp, u32, u64, C.POINTER(LayerBiomes), vp, u32, u32, u32, i32, i32, vp]),
    "stpgb_layer_biomemap_host": (C.c_int, [vp, u32, u64, C.POINTER(LayerBiomes), vp, u32, u32, i32, i32]),
    "stpgb_generator_create": (C.c_int, [C.POINTER(ChunkSetting), C.POINTER(RaindropSetting),
                                         C.POINTER(SimplexSetting), vp, u32, u32, C.POINTER(vp)]),
    "stpgb_generator_destroy": (C.c_int, [vp]),
    "stpgb_generator_create_setup": (C.c_int, [C.POINTER(GeneratorSetup), C.POINTER(vp)]),
    "stpgb_biomefield_create": (C.c_int, [C.POINTER(SimplexSetting), vp, u32, u32, C.POINTER(vp)]),
    "stpgb_biomefield_destroy": (C.c_int, [vp]),
    "stpgb_biomefield_generate": (C.c_int, [vp, C.POINTER(DiversityCall)]),
    "stpgb_copy": (C.c_int, [vp, vp, sz, vp, C.c_int]),
    "stpgb_roofline_launch": (C.c_int, [u32, vp, u64, u32, u32, vp, vp]),
    "stpgb_generator_generate": (C.c_int, [vp, vp, vp, f32, f32]),
    "stpgb_generator_erode": (C.c_int, [vp, vp, vp]),
    "stpgb_generator_erode_starts": (C.c_int, [vp, vp, vp, vp, u32, C.POINTER(f64)]),
    "stpgb_batch_create": (C.c_int, [C.POINTER(BatchRequest), u32, C.POINTER(RaindropSetting),
                                     C.POINTER(SimplexSetting), vp, u32, u64, u32, C.POINTER(vp)]),
    "stpgb_batch_destroy": (C.c_int, [vp]),
    "stpgb_batch_device_bytes": (u64, [vp]),
    "stpgb_batch_buffers": (C.c_int, [vp, u32, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)]),
    "stpgb_batch_synthesize_inputs": (C.c_int, [vp, u32, u64, vp]),
    "stpgb_batch_synthesize_layer_biomes": (C.c_int, [vp, u64, vp]),
    "stpgb_batch_run": (C.c_int, [vp, vp]),
    "stpgb_batch_run_plain": (C.c_int, [vp, vp]),
    "stpgb_batch_upload": (C.c_int, [vp, vp, vp, vp]),
    "stpgb_batch_download": (C.c_int, [vp, vp, vp, vp, vp]),
    "stpgb_batch_status": (C.c_int, [vp, vp]),
    "stpgb_batch_run_stage": (C.c_int, [vp, u32, vp]),
    "stpgb_batch_tuning": (C.c_int, [vp, C.POINTER(u32), C.POINTER(u32), C.POINTER(u32), vp]),
    "stpgb_batch_tuning_stages": (C.c_int, [vp, C.POINTER(u32), vp, C.POINTER(u32), vp, C.POINTER(u32)]),
    "stpgb_batch_tuning_filter_path": (C.c_int, [vp, C.POINTER(u32), vp]),
    "stpgb_batch_kernels_per_run": (C.c_int, [vp, C.POINTER(u32)]),
    "stpgb_batch_tune": (C.c_int, [vp]),
    "stpgb_batch_download_inputs": (C.c_int, [vp, vp, vp, vp]),
    "stpgb_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(RaindropSetting), C.POINTER(SimplexSetting),
                                      vp, u32, C.POINTER(vp)]),
    "stpgb_server_destroy": (C.c_int, [vp]),
    "stpgb_server_submit": (C.c_int, [vp, C.POINTER(ServeRequest), C.POINTER(u64)]),
    "stpgb_server_submit_batch": (C.c_int, [vp, vp, u32, vp]),
    "stpgb_server_poll": (C.c_int, [vp, C.POINTER(ServeResult), u32, C.POINTER(u32), C.c_int]),
    "stpgb_server_release": (C.c_int, [vp, u64]),
    "stpgb_server_download": (C.c_int, [vp, u64, vp, vp]),
    "stpgb_server_stats_get": (C.c_int, [vp, C.POINTER(ServerStats)]),
    "stpgb_server_replay": (C.c_int, [vp, C.POINTER(ServeRequest), vp, u32, vp, C.POINTER(f64)]),
    "stpgb_batch_counters": (C.c_int, [vp, C.POINTER(u64), C.POINTER(u64), C.c_int]),
}

_lib = None


def lib():
    """The loaded library; raises if libstpgb.so has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'` "
                              "(the CUDA extension is required; there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


_ERRORS = {
    STPGB_EINVAL: STPNumericDomainError,
    STPGB_ECUDA: STPCUDAError,
    STPGB_ETIMEOUT: STPTimeout,
    STPGB_ENOMEM: STPInsufficientMemory,
    STPGB_ECAPACITY: STPCapacityError,
}


def check(rc, env_error=False):
    """Raise the reference-style exception for a non-zero status."""
    if rc == STPGB_OK:
        return
    msg = (lib().stpgb_last_error() or b"").decode(errors="replace")
    if rc == STPGB_EINVAL and (env_error or msg.startswith("STP") and "Setting" in msg):
        raise STPInvalidEnvironment(msg)
    raise _ERRORS.get(rc, STPException)(f"status {rc}: {msg}")
