"""Stacks of independent scenes (emlab_stack_*): every scene of a stack evolves bit for bit as it
does alone, before and after compaction, with its sources, thin wires, lossy and metal cells, its own
absorber and its port; the batched sweep runner against one grid per scene."""
import numpy as np
import pytest

import oracle
from em_lab_gb300 import abi, batch, configs
from em_lab_gb300.grid import SceneStack, SimulationGrid

pytestmark = pytest.mark.gpu


def stack_of(scenes):
    st = SceneStack(scenes[0].grid, [sc.grid.size[2] for sc in scenes])
    for k, sc in enumerate(scenes):
        m = sc.materials
        st.upload_scene_materials(k, m.sigma, m.epsilon_r, sc.edges, sc.wires)
    st.set_scene_sources([sc.sources for sc in scenes])
    return st


def oracle_run(sc, steps):
    o = oracle.Oracle(sc.grid, "f32")
    oracle.load_scene(o, sc)
    o.step(steps)
    return o.read_components()


def scenes_xy(nx, ny, depths, seeds, **kw):
    return [configs.random_scene(size=(nx, ny, nz), seed=s, **kw) for nz, s in zip(depths, seeds)]


@pytest.mark.parametrize("kernel", [abi.KERNEL_FUSED, abi.KERNEL_SPLIT])
def test_stack_scenes_equal_scenes_alone(kernel):
    scenes = scenes_xy(24, 20, (18, 26, 21), (1, 2, 3), pml=4)
    st = stack_of(scenes)
    st.set_kernel(kernel)
    st.step(45)
    comps = st.read_components()
    z0, nz = st.layout()
    assert nz == [18, 26, 21] and z0 == [0, 19, 46]
    for k, sc in enumerate(scenes):
        ref = oracle_run(sc, 45)
        got = st.scene_components(k, comps)
        for c in range(6):
            np.testing.assert_array_equal(got[c], ref[c], err_msg=f"scene {k} component {c}")
    for c in range(6):  # the separator planes never leave zero
        assert not comps[c][18].any() and not comps[c][45].any()
    st.close()


@pytest.mark.parametrize("tiling", [32, 64, 128, 8])
def test_stack_tilings(tiling):
    scenes = scenes_xy(70, 37, (19, 40), (5, 6), pml=5)
    st = stack_of(scenes)
    st.set_tiling(tiling)
    st.step(30)
    comps = st.read_components()
    for k, sc in enumerate(scenes):
        ref = oracle_run(sc, 30)
        for c, (a, b) in enumerate(zip(st.scene_components(k, comps), ref)):
            np.testing.assert_array_equal(a, b, err_msg=f"tiling {tiling} scene {k} component {c}")
    st.close()


def test_sources_near_scene_faces_stay_in_their_scene():
    """A source whose footprint reaches the top face of its scene does not leak into the separator or
    the next scene (its cell list is clamped to the scene, as on a grid of its own)."""
    scenes = scenes_xy(24, 24, (20, 20), (7, 8), pml=3)
    top = scenes[0]
    s = top.sources[0]
    s.center = (12.3, 11.7, 19.6)
    s.softness = (1.5, 1.5, 1.5)
    bottom = scenes[1]
    bottom.sources[0].center = (10.2, 12.9, 0.4)
    st = stack_of(scenes)
    st.step(25)
    comps = st.read_components()
    for k, sc in enumerate(scenes):
        ref = oracle_run(sc, 25)
        for c, (a, b) in enumerate(zip(st.scene_components(k, comps), ref)):
            np.testing.assert_array_equal(a, b, err_msg=f"scene {k} component {c}")
    st.close()


def test_compaction_keeps_scenes_bit_exact():
    scenes = scenes_xy(24, 20, (18, 22, 19, 20), (11, 12, 13, 14), pml=4)
    st = stack_of(scenes)
    st.step(20)
    st.compact([True, False, True, False])
    assert st.layout() == ([0, 19], [18, 19])
    st.step(17)
    comps = st.read_components()
    for k, sc in zip(range(2), (scenes[0], scenes[2])):
        ref = oracle_run(sc, 37)
        for c, (a, b) in enumerate(zip(st.scene_components(k, comps), ref)):
            np.testing.assert_array_equal(a, b, err_msg=f"kept scene {k} component {c}")
    assert st.step_count() == 37
    st.close()


def test_stack_port_series_equal_single_grid():
    scs = [configs.batched_scene(3, i) for i in range(40)]
    small = [sc for sc in scs if sc.grid.size[0] == 48][:3]
    assert len(small) >= 2
    st = stack_of(small)
    z0, _ = st.layout()
    ports = []
    for k, sc in enumerate(small):
        p = sc.ports[0]
        ports.append(abi.Port(p.texel[0], p.texel[1], p.texel[2] + z0[k], p.axis, p.edges, 1 if p.sign >= 0 else -1))
    st.ports_configure(ports, small[0].wavelength, 4.0, False, 64)
    st.step(64)
    ser = st.ports_take_series(64)
    st.step(64)
    ser = np.concatenate([ser, st.ports_take_series(64)])
    assert ser.shape == (128, len(small), 2)
    for k, sc in enumerate(small):
        g = SimulationGrid(sc.grid)
        oracle.load_scene(g, sc)
        g.ports_configure([sc.ports[0].to_c()], sc.wavelength, 4.0, False, 128)
        g.step(128)
        np.testing.assert_array_equal(ser[:, k], g.ports_series()[:, 0], err_msg=f"scene {k}")
        g.close()
    st.close()


def test_batch_runner_equals_single_runs():
    scs = [configs.batched_scene(9, i) for i in range(60)]
    pick = [sc for sc in scs if sc.grid.size[0] in (48, 64)][:5]
    done = []
    run = batch.BatchRunner(pick, chunk=64, max_steps=20000)
    res = run.run(on_done=lambda i, r: done.append(i))
    assert sorted(done) == list(range(len(pick)))
    for i, sc in enumerate(pick):
        series, sweep = batch.run_single(sc, chunk=64, max_steps=20000)
        r = res[i]
        got = np.concatenate(r.series)
        assert got.shape == series.shape, f"scene {i}: {got.shape} vs {series.shape}"
        np.testing.assert_array_equal(got, series)
        np.testing.assert_array_equal(r.sweep["z"], sweep["z"])
        assert abs(r.sweep["s11"]).max() < 200.0


def test_batch_runner_decision_stops_or_continues():
    """decide_at / decide: the stack steps exactly to each decision step (a short chunk), scenes the
    callback accepts stop there; rejected scenes run on to ring-down with the same series (bit for
    bit) and Z(f) as a run without any decision."""
    scs = [configs.batched_scene(9, i) for i in range(60)]
    pick = [sc for sc in scs if sc.grid.size[0] in (48, 64)][:6]
    plain = batch.BatchRunner(pick, chunk=64, max_steps=20000)
    ref = plain.run()
    plain.close()
    at = [150 + 10 * i for i in range(len(pick))]
    seen = []

    def decide(idx, series):
        for i, ser in zip(idx, series):
            assert ser.shape[0] == at[i]
            seen.append(i)
        return [i % 2 == 0 for i in idx]  # accept the even scenes

    run = batch.BatchRunner(pick, chunk=64, max_steps=20000, decide_at=at, decide=decide)
    res = run.run()
    run.close()
    assert sorted(seen) == [i for i in range(len(pick)) if ref[i].steps > at[i]]
    for i, (r, q) in enumerate(zip(res, ref)):
        if i in seen and i % 2 == 0:
            assert r.accepted and r.sweep is None and r.steps == at[i]
            np.testing.assert_array_equal(np.concatenate(r.series), np.concatenate(q.series)[: r.steps])
        else:
            assert not r.accepted and r.steps == q.steps
            np.testing.assert_array_equal(np.concatenate(r.series), np.concatenate(q.series))
            np.testing.assert_array_equal(r.sweep["z"], q.sweep["z"])


@pytest.mark.parametrize("chunk", [16, 64])
def test_graph_chunks_equal_launch_by_launch(chunk):
    """Captured step graphs give the same fields, port series, port/far-field/line phasors."""
    sc = configs.random_scene(size=(40, 36, 30), pml=5, seed=21)
    out = []
    for graph in (False, True):
        g = SimulationGrid(sc.grid)
        oracle.load_scene(g, sc)
        if graph:
            g.set_graph(chunk)
        ports = [p.to_c() for p in sc.ports] or [abi.Port(20, 18, 15, 2, 1, 1)]
        g.ports_configure(ports, 12.0, 4.0, False, chunk)
        g.ntff_configure((9, 9, 9), (30, 26, 20), 12.0)
        g.lines_configure([[0, 2, 0, 0]], [[20, 18, 15, 2], [20, 18, 16, 2]], [1.0, 0.5], 12.0)
        series = []
        for _ in range(3):
            g.step(chunk)
            series.append(g.ports_take_series(chunk))
        g.step(5)  # a partial chunk: launch by launch
        g.step(chunk)
        series.append(g.ports_take_series(chunk + 5))
        out.append((g.read_components(), np.concatenate(series), g.ports_phasors(), g.ntff_phasors(),
                    g.lines_read()[0], g.step_count()))
        g.close()
    (c0, s0, p0, n0, l0, k0), (c1, s1, p1, n1, l1, k1) = out
    assert k0 == k1 == 4 * chunk + 5
    for a, b in zip(c0, c1):
        np.testing.assert_array_equal(a, b)
    for a, b in ((s0, s1), (p0, p1), (n0, n1), (l0, l1)):
        np.testing.assert_array_equal(a, b)


def test_graph_chunks_on_a_stack_after_compaction():
    scenes = scenes_xy(24, 20, (18, 22, 19), (31, 32, 33), pml=4)
    st = stack_of(scenes)
    st.set_graph(8)
    st.step(8)
    st.step(8)
    st.compact([True, False, True])
    st.step(8)
    st.step(8)
    comps = st.read_components()
    for k, sc in zip(range(2), (scenes[0], scenes[2])):
        ref = oracle_run(sc, 32)
        for c, (a, b) in enumerate(zip(st.scene_components(k, comps), ref)):
            np.testing.assert_array_equal(a, b, err_msg=f"scene {k} component {c}")
    st.close()


def test_asynchronous_series_takes_equal_the_synchronous_take():
    """emlab_ports_take_series_async / _collect_series: two takes may wait at once, each holds the
    rows recorded before it, and the series equals the synchronous take of the same steps; a third
    take while both slots wait, collecting a free slot, or configuring ports while a take waits, is
    refused."""
    sc = configs.batched_scene(3, 0)
    out = []
    for mode in ("sync", "async"):
        g = SimulationGrid(sc.grid)
        oracle.load_scene(g, sc)
        g.ports_configure([sc.ports[0].to_c()], sc.wavelength, 4.0, False, 64)
        g.set_graph(64)
        if mode == "sync":
            parts = []
            for _ in range(3):
                g.step(64)
                parts.append(g.ports_take_series(64))
        else:
            g.step(64)
            a = g.ports_take_series_async()
            g.step(64)
            b = g.ports_take_series_async()
            with pytest.raises(RuntimeError, match="both series slots"):
                g.ports_take_series_async()
            parts = [g.ports_collect_series(*a)]
            with pytest.raises(RuntimeError, match="no pending take"):
                g.ports_collect_series(a[0], a[1])
            g.step(64)
            c = g.ports_take_series_async()
            with pytest.raises(RuntimeError, match="pending series takes"):
                g.ports_configure([sc.ports[0].to_c()], sc.wavelength, 4.0, False, 64)
            parts += [g.ports_collect_series(*b), g.ports_collect_series(*c)]
            assert a[1] == b[1] == c[1] == 64
        out.append(np.concatenate(parts))
        g.close()
    np.testing.assert_array_equal(out[0], out[1])
