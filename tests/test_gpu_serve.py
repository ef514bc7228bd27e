"""The continuous-batching server: generation of resident chunks against the
oracle (through the mass balance of every eroded result), results the same
alone and in a mix (within the erosion's run-to-run spread), admission under
a small HBM budget, refusal of a request larger than the budget, and a short
camera-walk replay."""
import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu

NB, SEED, CELL = 6, 11, 160
REQS = [dict(ChunkX=x, ChunkY=y, MapSize=S, InterpolationRadius=16, DropletsPerPixel=2.3, BrushRadius=3,
             Lifetime=30, UserTag=i)
        for i, (x, y, S) in enumerate([(0, 0, 64), (1, 0, 64), (0, 1, 64), (1, 1, 64), (-1, -1, 64), (3, 0, 64),
                                       (0, 0, 128), (1, 0, 128)])]


def make_server(stpgb, **kw):
    from superterrainplus_gb300.serve import Server
    base = stpgb.RaindropSetting(**helpers.raindrop_dict(1000, radius=3, lifetime=30, seed=SEED))
    simplex = stpgb.SimplexSetting(SEED, 8, 0.2181661565)
    args = dict(hbm_budget=1 << 30, max_in_flight=16, max_batch=8, streams=3, voronoi_cell=CELL, biome_seed=SEED)
    args.update(kw)
    return Server(base, simplex, helpers.biome_table(NB, SEED), **args)


def run_all(server, reqs):
    tickets = {server.submit(**r): r["UserTag"] for r in reqs}
    out = {}
    while len(out) < len(tickets):
        for res in server.poll(wait_ms=2000):
            assert res.Status == 0
            h, f = server.download(res)
            out[res.UserTag] = (h, f, res.ResidualSediment, res.LatencyMs)
            server.release(res.Ticket)
    return out


def expected_merged(oracle, stpgb, r, layer_chain=False):
    """Pre-erosion neighbourhood of a request from the oracle (Voronoi or the demo's biome layer
    chain, filter, noise)."""
    from test_layers import DEMO_CHAIN, demo_ids
    S, rad = r["MapSize"], r["InterpolationRadius"]
    table = helpers.biome_table(NB, SEED)
    perm, grad = stpgb.permutation_generate(SEED, 8, 0.2181661565)
    cell = max(1, CELL * S // 512)
    out = np.zeros((3 * S, 3 * S), np.float32)
    for c in range(9):
        kx, ky = r["ChunkX"] + c % 3 - 1, r["ChunkY"] + c // 3 - 1
        if layer_chain:
            region = oracle.layer_biomemap(DEMO_CHAIN, demo_ids(), SEED, 3 * S, 3 * S, ((kx - 1) * S, (ky - 1) * S))
        else:
            region = oracle.voronoi(3 * S, 3 * S, ((kx - 1) * S, (ky - 1) * S), cell, NB, SEED)
        rc, off, bins = oracle.shf(region, (S, S), (3, 3), rad)
        assert rc == 0
        h = oracle.multibiome(off, bins, table, perm, grad, (S, S), (float(kx * S), float(ky * S)))
        out[(c // 3) * S:(c // 3 + 1) * S, (c % 3) * S:(c % 3 + 1) * S] = h
    return out


def test_serve_generation_mass_balance_and_format(stpgb, dev, oracle):
    sv = make_server(stpgb)
    res = run_all(sv, REQS)
    st = sv.stats()
    # neighbourhoods overlap: far fewer chunks generated than 9 per request
    assert st["ChunksGenerated"] < 9 * len(REQS)
    for r in REQS:
        h, f, residual, lat = res[r["UserTag"]]
        pre = expected_merged(oracle, stpgb, r).astype(np.float64)
        total = pre.sum()
        assert abs((total - h.astype(np.float64).sum()) - residual) <= 1e-5 * total, r
        assert np.array_equal(f, oracle.format(h))
        assert lat > 0.0
    sv.close()


def test_serve_with_layer_chain_biomes(stpgb, dev, oracle):
    """BiomeSource = the demo's layer chain: every eroded result balances against the oracle's
    neighbourhood built from the oracle's layer chain (biome IDs 0 / 1 / 3 in a 6-biome table),
    and the chain's biomes differ from the Voronoi ones."""
    reqs = [dict(r, ChunkX=x, ChunkY=y) for r, (x, y) in zip(REQS[:4], [(0, 0), (10, -7), (-25, 30), (31, 31)])]
    sv = make_server(stpgb, layer_chain_biomes=True)
    res = run_all(sv, reqs)
    vor = run_all(make_server(stpgb), reqs[:1])
    for r in reqs:
        h, f, residual, _ = res[r["UserTag"]]
        pre = expected_merged(oracle, stpgb, r, layer_chain=True).astype(np.float64)
        total = pre.sum()
        assert abs((total - h.astype(np.float64).sum()) - residual) <= 1e-5 * total, r
        assert np.array_equal(f, oracle.format(h))
    assert not np.allclose(vor[0][0], res[0][0])
    sv.close()


def test_serve_same_alone_and_in_the_mix(stpgb, dev):
    mix = run_all(make_server(stpgb), REQS)
    alone1, alone2 = {}, {}
    for r in REQS:
        alone1.update(run_all(make_server(stpgb), [r]))
        alone2.update(run_all(make_server(stpgb), [r]))
    for res in (mix, alone1, alone2):
        for h, _, _, _ in res.values():
            assert np.isfinite(h).all() and h.min() >= 0.0 and h.max() <= 1.0  # heights stay physical
    spread = max(float(np.sqrt(np.mean((alone1[k][0] - alone2[k][0]).astype(np.float64) ** 2))) for k in alone1)
    for k in alone1:
        d = float(np.sqrt(np.mean((alone1[k][0] - mix[k][0]).astype(np.float64) ** 2)))
        print(f"request {k}: RMS alone vs mix {d:.3g}, run-to-run spread {spread:.3g}")
        assert d <= 2.0 * spread + 1e-6


def test_serve_admission_under_small_budget(stpgb, dev):
    # about two 64-side requests with their generation scratch fit at once
    budget = 24 << 20
    sv = make_server(stpgb, hbm_budget=budget, max_in_flight=64)
    reqs = [dict(r, UserTag=i) for i, r in enumerate(REQS[:6])]
    res = run_all(sv, reqs)
    assert len(res) == 6
    st = sv.stats()
    assert st["Completed"] == 6 and st["PoolBytesUsed"] <= budget
    sv.close()


def test_serve_refuses_request_above_budget(stpgb, dev):
    sv = make_server(stpgb, hbm_budget=8 << 20)
    with pytest.raises(stpgb.STPInsufficientMemory):
        sv.submit(**dict(REQS[-1], MapSize=512))
    sv.close()


def test_serve_camera_walk_replay(stpgb, dev):
    from superterrainplus_gb300.serve import camera_walk
    reqs, times = camera_walk(40, 3, rate=400.0, lods=(64, 128), probs=(0.6, 0.4), radius=16, brush=3, lifetime=30)
    keys = {(r["MapSize"], r["ChunkX"], r["ChunkY"]) for r in reqs}
    assert len(keys) == len(reqs)  # every request is a chunk not requested before
    sv = make_server(stpgb)
    lat, wall = sv.replay(reqs, times)
    assert np.all(lat > 0.0) and wall >= times[-1]
    assert sv.stats()["Completed"] == len(reqs)
    sv.close()


# ------------------------------------------------------------ in-place erosion (the reference's world pipeline)


def run_serial(server, reqs):
    """One request at a time: each is submitted after the previous one completed."""
    out = {}
    for r in reqs:
        server.submit(**r)
        got = []
        while not got:
            got = server.poll(wait_ms=5000)
        (res,) = got
        assert res.Status == 0
        h, _ = server.download(res)
        out[res.UserTag] = (h, res.ErosionOrder)
        server.release(res.Ticket)
    return out


def test_in_place_priority_levels_follow_the_reference_schedule(stpgb):
    """One sequence of [A (0,0), B (2,0), C (4,0)]: B's neighbourhood shares chunk column 1 with A's, C's
    shares column 3 with B's only.  The reference's schedule (STPWorldPipeline.cpp:339-403) gives A level
    1, B level 2 (a chunk of level 1 in its neighbourhood) and C level 1 (the only level present, 2, is
    above 1): C erodes together with A, before B, although it came after B."""
    sv = make_server(stpgb, in_place=True, max_batch=3, streams=1)
    reqs = [dict(REQS[0], ChunkX=x, ChunkY=0, UserTag=t) for t, x in enumerate([0, 2, 4])]
    sv.submit_many(reqs)
    order = {}
    while len(order) < 3:
        for res in sv.poll(wait_ms=5000):
            assert res.Status == 0
            order[res.UserTag] = res.ErosionOrder
            sv.release(res.Ticket)
    sv.close()
    assert sorted(order.values()) == [1, 2, 3]
    assert order[2] < order[1] and order[0] < order[1]


def test_in_place_results_carry_earlier_erosion(stpgb):
    """A (0,0) erodes its neighbourhood and writes it back; a second request for centre (0,0) returns that
    state without eroding again (ErosionOrder 0, the same heights bit for bit); B (1,0) then erodes a
    neighbourhood that shares two chunk columns with A's, and a third request for (0,0) sees column -1 as A
    left it and columns 0 and 1 as B left them."""
    S = REQS[0]["MapSize"]
    sv = make_server(stpgb, in_place=True, max_batch=1, streams=1)
    base = dict(REQS[0], ChunkY=0)
    out = run_serial(sv, [dict(base, ChunkX=0, UserTag=0), dict(base, ChunkX=0, UserTag=1),
                          dict(base, ChunkX=1, UserTag=2), dict(base, ChunkX=0, UserTag=3)])
    sv.close()
    (a, oa), (a2, oa2), (b, ob), (d, od) = out[0], out[1], out[2], out[3]
    assert oa == 1 and oa2 == 0 and ob == 2 and od == 0
    assert np.array_equal(a2, a)
    assert not np.array_equal(b[:, :2 * S], a[:, S:])  # B eroded the shared columns further
    assert np.array_equal(d[:, :S], a[:, :S])
    assert np.array_equal(d[:, S:], b[:, :2 * S])


def test_in_place_camera_walk_matches_a_serial_replay(stpgb):
    """A camera walk of 24 overlapping 64^2 requests, all submitted at once, through the in-place server
    (sequences of up to 6 requests in priority levels, three streams, sequences that share chunks ordered on
    the device) against a serial replay of the same requests one at a time in the server's erosion order.
    Each request's eroded neighbourhood agrees with the serial one within the erosion's run-to-run spread:
    three times the largest RMS between two serial replays."""
    from superterrainplus_gb300.serve import camera_walk
    reqs, _ = camera_walk(24, 5, rate=1e6, speed=3.0, turn_every=2.0, lods=(64,), probs=(1.0,), radius=16,
                          droplets_per_px=2.3, brush=3, lifetime=30)
    sv = make_server(stpgb, in_place=True, max_batch=6, streams=3)
    sv.submit_many(reqs)
    batched = {}
    while len(batched) < len(reqs):
        for res in sv.poll(wait_ms=5000):
            assert res.Status == 0
            h, _ = sv.download(res)
            batched[res.UserTag] = (h, res.ErosionOrder)
            sv.release(res.Ticket)
    sv.close()
    orders = sorted(o for _, o in batched.values())
    assert orders == list(range(1, len(reqs) + 1))  # distinct centres: every request erodes once
    in_order = sorted(reqs, key=lambda r: batched[r["UserTag"]][1])
    serial = []
    for _ in range(2):
        s = make_server(stpgb, in_place=True, max_batch=1, streams=1)
        serial.append(run_serial(s, in_order))
        s.close()
    rms = lambda a, b: float(np.sqrt(np.mean((a.astype(np.float64) - b) ** 2)))
    spread = max(rms(serial[0][t][0], serial[1][t][0]) for t in batched)
    worst = max(rms(batched[t][0], serial[0][t][0]) for t in batched)
    print(f"in-place camera walk: batched vs serial RMS {worst:.3g}, serial run-to-run spread {spread:.3g}")
    assert worst <= 3.0 * spread + 1e-6
    # the walk's neighbourhoods overlap: erosion carried between requests changes later results
    private = make_server(stpgb, max_batch=1, streams=1)
    alone = run_serial(private, in_order[-1:])
    private.close()
    t_last = in_order[-1]["UserTag"]
    assert rms(alone[t_last][0], serial[0][t_last][0]) > 3.0 * spread
