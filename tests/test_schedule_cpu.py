"""The persistent pair kernel's work schedule, host arithmetic only (no device): every cell of every
scene belongs to exactly one work item, the items come in the order the kernel's tickets take them,
and the z chunk length follows the stated rule (at least four items per CTA where chunks of 16
planes allow it; among those, the fewest planes for the busiest CTA, one re-read plane per chunk
above a scene's first plane)."""
import numpy as np
import pytest

from em_lab_gb300 import grid

CTAS = [4 * 152, 2 * 152, 152, 7]
ITEMS_PER_CTA, MIN_PLANES = 4, 16


def stack(rng, n):
    nx = rng.integers(8, 300, n)
    ny = rng.integers(8, 300, n)
    nz = rng.integers(1, 200, n)
    z0 = np.concatenate([[0], np.cumsum(nz + 1)[:-1]])
    return z0, nx, ny, nz


def tiles_of(nx, ny, ty):
    return ((nx + 63) // 64) * ((ny + ty - 1) // ty)


def cost(items, zc, rereads, ctas):
    return -(-items // ctas) * (zc + (1 if rereads else 0))


def ragged_cost(nx, ny, nz, ty, ctas, zc):
    chunks = -(-nz // zc)
    items = int((tiles_of(nx, ny, ty) * chunks).sum())
    return items, cost(items, zc, (chunks > 1).any(), ctas)


@pytest.mark.parametrize("ty", [4, 8, 16])
@pytest.mark.parametrize("seed", range(6))
def test_ragged_items_cover_every_cell_once(ty, seed):
    rng = np.random.default_rng(seed)
    z0, nx, ny, nz = stack(rng, int(rng.integers(1, 40)))
    for ctas in CTAS:
        it = grid.ragged_items(z0, nx, ny, nz, ty, ctas)
        x0, y0, zs, ze, sc = it.T
        assert (np.diff(sc) >= 0).all(), "scene by scene"
        zc = int((ze - zs).max())
        for s in range(len(z0)):
            m = sc == s
            # every tile of the scene's own cross-section, nothing outside it
            want_tiles = {(tx * 64, t * ty) for tx in range(-(-nx[s] // 64)) for t in range(-(-ny[s] // ty))}
            got_tiles = set(zip(x0[m].tolist(), y0[m].tolist()))
            assert got_tiles == want_tiles
            # per tile: z chunks tiling the scene's planes exactly, all of one length but the last
            for tile in want_tiles:
                k = m & (x0 == tile[0]) & (y0 == tile[1])
                a, b = zs[k], ze[k]
                assert a[0] == z0[s] and b[-1] == z0[s] + nz[s]
                assert (a[1:] == b[:-1]).all() and (b > a).all()
                assert ((b - a)[:-1] == zc).all() and (b - a)[-1] <= zc
            # launch order within a scene: z chunk by z chunk, tile by tile (x fastest)
            order = np.lexsort((x0[m], y0[m], zs[m]))
            assert (order == np.arange(m.sum())).all()
        assert len(it) == int(ragged_cost(nx, ny, nz, ty, ctas, zc)[0])


@pytest.mark.parametrize("ty", [4, 8, 16])
@pytest.mark.parametrize("seed", range(6))
def test_ragged_chunk_length_follows_the_rule(ty, seed):
    rng = np.random.default_rng(100 + seed)
    z0, nx, ny, nz = stack(rng, int(rng.integers(1, 40)))
    deepest = int(nz.max())
    for ctas in CTAS:
        it = grid.ragged_items(z0, nx, ny, nz, ty, ctas)
        zc = int((it[:, 3] - it[:, 2]).max())
        want = min(ITEMS_PER_CTA * ctas, int((tiles_of(nx, ny, ty) * np.maximum(1, nz // MIN_PLANES)).sum()))
        cand = {z: ragged_cost(nx, ny, nz, ty, ctas, z) for z in range(min(deepest, 4), deepest + 1)}
        ok = {z: c for z, (items, c) in cand.items() if items >= want}
        if ok:
            assert zc in ok and ok[zc] == min(ok.values())
        else:  # no chunk length reaches `want`: the finest split
            assert zc == min(deepest, 4) or deepest < 4


def test_ragged_single_plane_and_large_cross_sections():
    it = grid.ragged_items([0, 2], [1, 65535], [1, 3], [1, 5], 16, 304)
    assert (it[it[:, 4] == 0] == [0, 0, 0, 1, 0]).all()
    big = it[it[:, 4] == 1]
    assert big[:, 0].max() == 65472 and set(big[:, 1].tolist()) == {0}
    assert big[:, 2].min() == 2 and big[:, 3].max() == 7


def test_ragged_items_reject_bad_arguments():
    with pytest.raises(grid.EmlabError):
        grid.ragged_items([0], [65536], [8], [8], 8, 304)
    with pytest.raises(grid.EmlabError):
        grid.ragged_items([0], [8], [8], [0], 8, 304)
    with pytest.raises(grid.EmlabError):
        grid.ragged_items([0], [8], [8], [8], 6, 304)
    with pytest.raises(grid.EmlabError):
        grid.pair_schedule(8, 8, 8, 8, 0)


@pytest.mark.parametrize("ty", [4, 8, 16])
@pytest.mark.parametrize("shape", [(512, 512, 512), (128, 128, 128), (384, 384, 256), (48, 40, 9), (70, 37, 3),
                                   (1000, 20, 1000), (64, 8, 1)])
def test_uniform_schedule(ty, shape):
    nx, ny, nz = shape
    tiles = -(-nx // 64) * -(-ny // ty)
    max_chunks = max(1, nz // 4)
    for ctas in CTAS:
        zc, items = grid.pair_schedule(nx, ny, nz, ty, ctas)
        chunks = -(-nz // zc)
        assert items == chunks * tiles and 1 <= zc <= nz and (chunks - 1) * zc < nz
        want = min(ITEMS_PER_CTA * ctas, max(1, nz // MIN_PLANES) * tiles)
        cand = {}
        for c in range(1, max_chunks + 1):
            z = -(-nz // c)
            n = -(-nz // z)
            cand.setdefault(z, (n * tiles, cost(n * tiles, z, n > 1, ctas)))
        ok = {z: c for z, (i, c) in cand.items() if i >= want}
        if ok:
            assert zc in ok and ok[zc] == min(ok.values())
        else:
            assert zc == -(-nz // max_chunks)
        # one scene as a stack never does worse than the uniform schedule under the same cost
        it = grid.ragged_items([0], [nx], [ny], [nz], ty, ctas)
        rz = int((it[:, 3] - it[:, 2]).max())
        if ok:
            assert ragged_cost(np.array([nx]), np.array([ny]), np.array([nz]), ty, ctas, rz)[1] <= ok[zc]
