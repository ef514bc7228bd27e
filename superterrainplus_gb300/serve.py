"""Serving: the continuous-batching chunk server (stpgb_server_*) and a
seeded camera-walk request stream.

A camera walks the world at `speed` chunks per second and turns to a random
heading every `turn_every` seconds; requests arrive as a Poisson process of
`rate` per second.  Each request asks for the not-yet-requested chunk nearest
the camera at a level of detail drawn from `lods` with `probs`, so its 3x3
neighbourhood overlaps those of earlier requests."""
import ctypes as C

import numpy as np

from . import BIOME_DTYPE
from ._capi import ServeRequest, ServeResult, ServerConfig, ServerStats, check, lib


def camera_walk(n, seed, rate=200.0, speed=1.0, turn_every=5.0, lods=(256, 512, 1024), probs=(0.5, 0.35, 0.15),
                radius=32, droplets_per_px=2.3, brush=4, lifetime=50):
    """(list of request dicts, arrival times in seconds)."""
    rng = np.random.default_rng(seed)
    times = np.cumsum(rng.exponential(1.0 / rate, n))
    # camera path: piecewise straight at `speed`, new heading every `turn_every` s
    legs = int(times[-1] // turn_every) + 2 if n else 1
    headings = rng.uniform(0.0, 2.0 * np.pi, legs)
    starts = np.zeros((legs, 2))
    for i in range(1, legs):
        starts[i] = starts[i - 1] + speed * turn_every * np.array([np.cos(headings[i - 1]), np.sin(headings[i - 1])])
    requested = set()
    reqs = []
    for k, t in enumerate(times):
        leg = int(t // turn_every)
        pos = starts[leg] + speed * (t - leg * turn_every) * np.array([np.cos(headings[leg]), np.sin(headings[leg])])
        lod = int(rng.choice(lods, p=probs))
        cx0, cy0 = int(np.floor(pos[0])), int(np.floor(pos[1]))
        pick = None
        for ring in range(0, 64):
            cand = [(cx0 + dx, cy0 + dy) for dy in range(-ring, ring + 1) for dx in range(-ring, ring + 1)
                    if max(abs(dx), abs(dy)) == ring and (lod, cx0 + dx, cy0 + dy) not in requested]
            if cand:
                pick = cand[int(rng.integers(len(cand)))]
                break
        requested.add((lod, pick[0], pick[1]))
        reqs.append(dict(ChunkX=pick[0], ChunkY=pick[1], MapSize=lod, InterpolationRadius=radius,
                         DropletsPerPixel=droplets_per_px, BrushRadius=brush, Lifetime=lifetime, UserTag=k))
    return reqs, times


class Server:
    def __init__(self, base_setting, simplex_setting, biome_table, hbm_budget=40 << 30, max_in_flight=64,
                 max_batch=16, streams=3, voronoi_cell=192, biome_seed=42, layer_chain_biomes=False,
                 in_place=False):
        """`layer_chain_biomes`: generate biomemaps with the demo's layer chain (the reference's
        STPLayerChainBuilder) instead of the synthetic Voronoi map.  `in_place`: erode the resident
        chunks in place in the reference's priority-batched order (STPGB_EROSION_IN_PLACE) instead
        of a private copy per request."""
        table = np.ascontiguousarray(biome_table, BIOME_DTYPE)
        cfg = ServerConfig(hbm_budget, max_in_flight, max_batch, streams, voronoi_cell, biome_seed,
                           int(bool(layer_chain_biomes)), int(bool(in_place)))
        h = C.c_void_p()
        check(lib().stpgb_server_create(C.byref(cfg), C.byref(base_setting), C.byref(simplex_setting),
                                        table.ctypes.data_as(C.c_void_p), len(table), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().stpgb_server_destroy(self._h)
            self._h = None

    __del__ = close

    def submit(self, **req):
        t = C.c_uint64(0)
        check(lib().stpgb_server_submit(self._h, C.byref(ServeRequest(**req)), C.byref(t)))
        return t.value

    def submit_many(self, requests):
        """All `requests` enter the queue together (stpgb_server_submit_batch); returns their tickets."""
        n = len(requests)
        arr = (ServeRequest * n)(*[ServeRequest(**r) for r in requests])
        t = (C.c_uint64 * n)()
        check(lib().stpgb_server_submit_batch(self._h, arr, n, t))
        return list(t)

    def poll(self, capacity=64, wait_ms=0):
        out = (ServeResult * capacity)()
        n = C.c_uint32(0)
        check(lib().stpgb_server_poll(self._h, out, capacity, C.byref(n), wait_ms))
        return [out[i] for i in range(n.value)]

    def download(self, result):
        """Host copies (merged eroded heightmap, uint16 format) of a completed result."""
        w = 3 * result.MapSize
        h = np.zeros((w, w), np.float32)
        f = np.zeros((w, w), np.uint16)
        check(lib().stpgb_server_download(self._h, result.Ticket, h.ctypes.data_as(C.c_void_p),
                                          f.ctypes.data_as(C.c_void_p)))
        return h, f

    def release(self, ticket):
        check(lib().stpgb_server_release(self._h, ticket))

    def stats(self):
        s = ServerStats()
        check(lib().stpgb_server_stats_get(self._h, C.byref(s)))
        return {n: getattr(s, n) for n, _ in s._fields_}

    def replay(self, requests, arrivals):
        """Submits on the arrival schedule; returns (latency ms per request, wall seconds)."""
        n = len(requests)
        arr = (ServeRequest * n)(*[ServeRequest(**r) for r in requests])
        t = np.ascontiguousarray(arrivals, np.float64)
        lat = np.zeros(n, np.float64)
        wall = C.c_double(0.0)
        check(lib().stpgb_server_replay(self._h, arr, t.ctypes.data_as(C.c_void_p), n,
                                        lat.ctypes.data_as(C.c_void_p), C.byref(wall)))
        return lat, wall.value
