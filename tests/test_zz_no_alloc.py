"""The allocation-free flux entry point (emlab_flux_planes_noalloc) against emlab_flux_planes.

It serves callers that must not allocate device memory while they measure: frame loops that cannot
afford the device-wide wait of cudaFree while the solver steps, and hosts that budget all device
memory themselves. Its scratch is a fixed device array shared
by every call, so two calls in a row must each give exactly what the allocating entry point gives
for the same fields, and requests beyond the fixed limits must be refused. This file is collected
last so a failure here cannot hide the other tests.
"""
import numpy as np
import pytest

import oracle
from em_lab_gb300 import EmlabError, SimulationGrid, abi, configs

pytestmark = pytest.mark.gpu


def box_planes(lo, hi):
    planes = []
    for ax in range(3):
        u, v = (1, 2) if ax == 0 else ((0, 2) if ax == 1 else (0, 1))
        for idx in (lo[ax], hi[ax]):
            planes.append(abi.FluxPlane(ax, idx, (lo[u], lo[v]), (hi[u] + 1, hi[v] + 1)))
    return planes


def test_flux_planes_noalloc_matches_allocating_entry_point():
    sc = configs.random_scene(size=(48, 40, 36), pml=5, seed=21)
    g = SimulationGrid(sc.grid)
    oracle.load_scene(g, sc)
    planes = box_planes((8, 7, 6), (38, 31, 28)) + [abi.FluxPlane(2, 18, (0, 0), (48, 40)),
                                                     abi.FluxPlane(0, 100, (0, 0), (4, 4))]  # out of the grid: 0
    g.step(60)
    first = (g.flux_planes(planes), g.flux_planes_noalloc(planes))
    g.step(25)
    second = (g.flux_planes(planes), g.flux_planes_noalloc(planes))
    for want, got in (first, second):
        assert np.array_equal(got, want)  # bit for bit, the tolerance of every flux test here
    assert not np.array_equal(first[0], second[0])  # the fields moved on between the two calls
    assert second[1][-1] == 0.0
    # the same result again from a call with fewer planes (scratch reused from offset 0)
    assert np.array_equal(g.flux_planes_noalloc(planes[:2]), second[0][:2])


def test_flux_planes_noalloc_rejects_requests_beyond_its_scratch():
    g = SimulationGrid(abi.GridConfig((16, 520, 520), pml_thickness=0))
    g.write_components([np.random.default_rng(2).standard_normal((520, 520, 16)).astype(np.float32)
                        for _ in range(6)])
    plane = abi.FluxPlane(0, 5, (0, 0), (520, 520))  # 33 x 33 = 1089 workgroup partials
    with pytest.raises(EmlabError) as e:
        g.flux_planes_noalloc([plane] * (abi.FLUX_NOALLOC_MAX_PLANES + 1))
    assert e.value.code == abi.EMLAB_ERR_INVALID
    with pytest.raises(EmlabError) as e:  # 61 x 1089 partials > 65536
        g.flux_planes_noalloc([plane] * 61)
    assert e.value.code == abi.EMLAB_ERR_INVALID
    ok = [plane] * 60  # 65340 partials: fits
    assert np.array_equal(g.flux_planes_noalloc(ok), g.flux_planes(ok))
