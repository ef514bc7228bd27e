"""The uneven batch at full size: 64 independent eroded chunks, sides drawn
log-uniform from 128 to 1024 (multiples of 32), 1-16 biomes and an even
filter radius of 8-48 per chunk, 2.3 droplets per pixel, brush radius 2-5,
all in one batched launch sequence captured in a CUDA graph and autotuned.

Checked at full size:
  * every request's mass balance within 1e-5 relative, every height finite
    and within 5 % of its start range of the start heights (no runaway), and
    its uint16 format bit for bit against the oracle, for the autotuned graph
    and for the plain per-chunk call sequence;
  * filter + noise heights within 2e-6 of the oracle, chunk by chunk, for
    eight of the requests (the four smallest, the two largest, two middle
    ones): the oracle's filter and noise for all 64 take minutes of CPU;
  * the biome regions of the two smallest requests bit for bit.
"""
import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu

COUNT = 64
TABLE_BIOMES = 16
CELL = 96
SEED = 31


class _Ptr:
    """A device address in the shape the kernel-level calls take (data_ptr())."""

    def __init__(self, p):
        self.p = p

    def data_ptr(self):
        return self.p


def uneven_requests():
    rng = np.random.default_rng(SEED)
    reqs, biomes = [], []
    for n in range(COUNT):
        side = int(np.exp(rng.uniform(np.log(128.0), np.log(1024.0))))
        side = min(1024, max(128, 32 * int(round(side / 32.0))))
        reqs.append(dict(MapSize=side, ChunkX=40 * n - 1000, ChunkY=7 * n - 200,
                         InterpolationRadius=2 * int(rng.integers(4, 25)),
                         DropletCount=int(round(2.3 * side * side)), BrushRadius=int(rng.integers(2, 6)),
                         Lifetime=30))
        biomes.append(int(rng.integers(1, TABLE_BIOMES + 1)))
    return reqs, biomes


def test_uneven_batch_full_size(stpgb, dev, oracle):
    import torch
    reqs, biomes = uneven_requests()
    base = stpgb.RaindropSetting(**helpers.raindrop_dict(1000, radius=3, lifetime=30, seed=SEED))
    simplex = stpgb.SimplexSetting(SEED, 8, 0.2181661565)
    table = helpers.biome_table(TABLE_BIOMES, SEED)
    b = stpgb.Batch(reqs, base, simplex, table, graph=True)
    b.synthesize(CELL, SEED)
    # each request's own biome count: its 5x5-chunk region uses IDs 0 .. biomes-1
    for n, r in enumerate(reqs):
        S = r["MapSize"]
        region = b.buffers(n)[0]
        dev.voronoi_biomemap(_Ptr(region), 5 * S, 5 * S, 5 * S, ((r["ChunkX"] - 2) * S, (r["ChunkY"] - 2) * S),
                             CELL, biomes[n], SEED)
    torch.cuda.synchronize()

    order = sorted(range(COUNT), key=lambda n: reqs[n]["MapSize"])
    checked = sorted(set(order[:4] + order[-2:] + order[COUNT // 2 - 1:COUNT // 2 + 1]))
    regions = [np.zeros((5 * r["MapSize"],) * 2, np.uint16) if n in checked else None for n, r in enumerate(reqs)]
    b.download_inputs(regions)
    b.status()
    for n in order[:2]:
        S = reqs[n]["MapSize"]
        want = oracle.voronoi(5 * S, 5 * S, ((reqs[n]["ChunkX"] - 2) * S, (reqs[n]["ChunkY"] - 2) * S), CELL,
                              biomes[n], SEED)
        assert np.array_equal(regions[n], want), n

    def heights():
        out = [np.zeros((3 * r["MapSize"],) * 2, np.float32) for r in reqs]
        fixed = [np.zeros((3 * r["MapSize"],) * 2, np.uint16) for r in reqs]
        res = np.zeros(COUNT, np.float64)
        b.download(out, fixed, res)
        b.status()
        return out, fixed, res

    b.run_stage(0)
    b.run_stage(1)
    before, _, _ = heights()
    perm, grad = stpgb.permutation_generate(SEED, 8, 0.2181661565)
    for n in checked:
        r = reqs[n]
        S = r["MapSize"]
        for c in range(9):
            cx, cy = c % 3, c // 3
            sub = np.ascontiguousarray(regions[n][cy * S:cy * S + 3 * S, cx * S:cx * S + 3 * S])
            rc, off, bins = oracle.shf(sub, (S, S), (3, 3), r["InterpolationRadius"])
            assert rc == 0
            off_xy = (float((r["ChunkX"] + cx - 1) * S), float((r["ChunkY"] + cy - 1) * S))
            ref = oracle.multibiome(off, bins, table, perm, grad, (S, S), off_xy, threads=16)
            got = before[n][cy * S:(cy + 1) * S, cx * S:(cx + 1) * S]
            assert np.abs(got - ref).max() <= 2e-6, (n, c)

    b.tune()
    choice, ms = b.tuning()
    assert choice in ms
    print(f"uneven batch: autotuner chose {choice} from {ms}")
    failures = []
    for run in (b.run, b.run_plain):
        run()
        after, fixed, res = heights()
        for n, r in enumerate(reqs):
            t0 = before[n].astype(np.float64).sum()
            bal = (t0 - after[n].astype(np.float64).sum()) - res[n]
            what = (run.__name__, n, r["MapSize"], r["BrushRadius"])
            if not abs(bal) <= 1e-5 * t0:
                failures.append(what + ("mass balance", bal))
            # no runaway: racing droplets can dig a little below the lowest start height or pile
            # deposits a little above the highest (the one-lane reference kernel did, by more than
            # 1e-3, on a 128^2 chunk with all 37,683 droplets in flight), never by 5 % of the range
            band = 0.05 * float(before[n].max() - before[n].min())
            if not np.isfinite(after[n]).all():
                failures.append(what + ("not finite",))
            elif not (after[n].min() >= before[n].min() - band and after[n].max() <= before[n].max() + band):
                failures.append(what + ("out of range", float(after[n].min() - before[n].min()),
                                        float(after[n].max() - before[n].max())))
            if np.array_equal(before[n], after[n]):
                failures.append(what + ("not eroded",))
            if not np.array_equal(fixed[n], oracle.format(after[n])):
                failures.append(what + ("format",))
    assert not failures, failures
