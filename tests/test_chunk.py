"""Chunk coordinate arithmetic (STPChunk's static functions) and the host
memory mode of the nearest-neighbour merge (STPNearestNeighbourTextureBuffer)
through the C ABI: the reference's own known answers
(SuperTest+/SuperTerrain+/STPTest2DChunk.cpp:30-89, STPTestNearestNeighbour.cpp:49-101)
and properties over many inputs.  Host-only: no GPU needed."""
import itertools
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def chunk(stpgb):
    return stpgb.STPChunk


def test_reference_known_answers(chunk):
    # STPTest2DChunk.cpp:33-41: camera at (-573.74, 679.5, 845.982), chunk size (8, 5), scale (2.5, 4)
    size = (8, 5)
    assert chunk.calcWorldChunkCoordinate((-573.74, 679.5, 845.982), size, (2.5, 4.0)) == (-232, 210)
    # :45-51
    assert chunk.calcChunkMapOffset((-232, 210), size, (512, 256), (25.5, -57.5)) == (-14822.5, 10694.5)
    # :56-62
    assert chunk.offsetChunk((30, -30), size, (3, -2)) == (54, -40)
    # :65-72, region (5, 7)
    region = (5, 7)
    assert chunk.calcLocalChunkCoordinate(7, region) == (2, 1)
    assert chunk.calcLocalChunkCoordinate(12, region) == (2, 2)
    assert chunk.calcLocalChunkCoordinate(20, region) == (0, 4)
    # :74-77
    assert chunk.calcLocalChunkOrigin((-24, 50), size, region) == (-40, 35)
    # :79-86
    offsets = chunk.calcChunkNeighbourOffset(size, region)
    assert len(offsets) == 35
    for i, want in ((0, (-16, -15)), (9, (16, -10)), (17, (0, 0)), (23, (8, 5)), (34, (16, 15))):
        assert offsets[i] == want


def test_local_coordinate_round_trip(chunk):
    for rx, ry in ((1, 1), (3, 3), (5, 7), (16, 2)):
        for i in range(rx * ry):
            x, y = chunk.calcLocalChunkCoordinate(i, (rx, ry))
            assert 0 <= x < rx and y * rx + x == i


def test_neighbour_offsets_cover_the_region(chunk):
    for size, region in (((8, 5), (3, 3)), ((512, 512), (5, 5)), ((7, 3), (4, 6)), ((1, 1), (1, 1))):
        offs = chunk.calcChunkNeighbourOffset(size, region)
        origin = chunk.calcLocalChunkOrigin((0, 0), size, region)
        assert offs[0] == origin
        for i, (ox, oy) in enumerate(offs):
            lx, ly = chunk.calcLocalChunkCoordinate(i, region)
            assert (ox, oy) == chunk.offsetChunk(origin, size, (lx, ly))
        if region[0] % 2 and region[1] % 2:
            assert offs[len(offs) // 2] == (0, 0)


def test_world_coordinate_is_floor_of_scaled_position(chunk):
    rng = np.random.default_rng(3)
    for _ in range(200):
        size = tuple(int(v) for v in rng.integers(1, 600, 2))
        scale = tuple(float(v) for v in rng.uniform(0.25, 8.0, 2))
        p = tuple(float(v) for v in rng.uniform(-1e6, 1e6, 3))
        got = chunk.calcWorldChunkCoordinate(p, size, scale)
        want = tuple(int(math.floor(q / (s * c))) * s for q, s, c in zip((p[0], p[2]), size, scale))
        assert got == want


def test_map_offset_is_linear_in_chunk_units(chunk):
    size, mapsize, off = (8, 5), (512, 256), (25.5, -57.5)
    for ux, uy in itertools.product(range(-3, 4), repeat=2):
        coord = chunk.offsetChunk((0, 0), size, (ux, uy))
        assert chunk.calcChunkMapOffset(coord, size, mapsize, off) == (ux * 512 + 25.5, uy * 256 - 57.5)


def test_undefined_arguments_are_refused(chunk, stpgb):
    with pytest.raises(stpgb.STPNumericDomainError):
        chunk.calcLocalChunkCoordinate(3, (0, 4))
    with pytest.raises(stpgb.STPNumericDomainError):
        chunk.calcWorldChunkCoordinate((1.0, 0.0, 1.0), (0, 5), (1.0, 1.0))
    with pytest.raises(stpgb.STPNumericDomainError):
        chunk.calcWorldChunkCoordinate((float("nan"), 0.0, 1.0), (8, 5), (1.0, 1.0))
    with pytest.raises(stpgb.STPNumericDomainError):
        chunk.offsetChunk((2**31 - 8, 0), (8, 5), (1, 0))
    with pytest.raises(stpgb.STPNumericDomainError):
        chunk.calcChunkMapOffset((8, 5), (0, 5), (512, 256), (0.0, 0.0))
    with pytest.raises(stpgb.STPNumericDomainError):
        chunk.calcChunkNeighbourOffset((8, 5), (0, 3))


@pytest.mark.parametrize("dtype", [np.uint16, np.float32])
def test_nearest_neighbour_merge_reference_scenario(stpgb, dtype):
    """STPTestNearestNeighbour.cpp:49-101: a 3x3 neighbourhood of 2x2 chunks, chunk i filled with i,
    merges into the map whose pixel (x, y) holds its chunk's index (x / 2) + (y / 2) * 3, and the
    merged map unmerges back into the chunks."""
    info = stpgb.NNInfo.make((2, 2), (3, 3))
    chunks = [np.full((2, 2), i, dtype) for i in range(9)]
    y, x = np.mgrid[0:6, 0:6]
    want = ((x // 2) + (y // 2) * 3).astype(dtype)
    assert np.array_equal(stpgb.nn_merge_host(chunks, info), want)
    back = [np.zeros((2, 2), dtype) for _ in range(9)]
    stpgb.nn_unmerge_host(want, info, back)
    assert all(np.array_equal(b, c) for b, c in zip(back, chunks))


def test_nearest_neighbour_merge_round_trip(stpgb):
    rng = np.random.default_rng(4)
    for ms, nn in (((7, 4), (5, 3)), ((16, 16), (1, 1)), ((3, 9), (1, 5))):
        info = stpgb.NNInfo.make(ms, nn)
        chunks = [rng.random((ms[1], ms[0])).astype(np.float32) for _ in range(nn[0] * nn[1])]
        merged = stpgb.nn_merge_host(chunks, info)
        assert merged.shape == (ms[1] * nn[1], ms[0] * nn[0])
        for i, c in enumerate(chunks):
            lx, ly = i % nn[0], i // nn[0]
            assert np.array_equal(merged[ly * ms[1]:(ly + 1) * ms[1], lx * ms[0]:(lx + 1) * ms[0]], c)
        back = [np.zeros_like(c) for c in chunks]
        stpgb.nn_unmerge_host(merged, info, back)
        assert all(np.array_equal(b, c) for b, c in zip(back, chunks))
    bad = stpgb.NNInfo.make((2, 2), (3, 3))
    bad.TotalMapSize[0] = 5
    with pytest.raises(stpgb.STPNumericDomainError):
        stpgb.nn_merge_host([np.zeros((2, 2), np.float32)] * 9, bad)
