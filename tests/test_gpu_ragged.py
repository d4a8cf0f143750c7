"""Stacks of scenes with their own cross-sections (emlab_stack_configure_scenes): one launch of the
persistent pair kernel steps every scene, each of which evolves bit for bit as it does on a grid of
its own (its absorber on all six faces, its materials, thin wires and sources), before and after
compaction; the cells of a scene's planes outside its cross-section never leave zero; and the
batched sweep runner gives the same series and Z(f) in one stack as in one stack per cross-section."""
import numpy as np
import pytest

import oracle
from em_lab_gb300 import abi, batch, configs
from em_lab_gb300.grid import EmlabError, SceneStack

pytestmark = pytest.mark.gpu

DIMS = [(24, 20, 18), (40, 28, 26), (33, 45, 21), (70, 37, 19)]


def scenes_of(dims, seed0=10, **kw):
    return [configs.random_scene(size=d, seed=seed0 + k, **kw) for k, d in enumerate(dims)]


def ragged_stack(scenes):
    st = SceneStack(scenes[0].grid, scene_dims=[tuple(sc.grid.size) for sc in scenes])
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


def frozen_cells_are_zero(st, comps):
    z0, nz = st.layout()
    for (nx, ny, _), z, d in zip(st.scene_dims(), z0, nz):
        for c in comps:
            block = c[z: z + d]
            assert not block[:, ny:, :].any() and not block[:, :, nx:].any()


@pytest.mark.parametrize("tiling", [64, 32, 128])
def test_ragged_stack_scenes_equal_scenes_alone(tiling):
    scenes = scenes_of(DIMS, pml=4)
    st = ragged_stack(scenes)
    st.set_tiling(tiling)
    assert st.scene_dims() == [tuple(d) for d in DIMS]
    assert st.size()[:2] == (70, 45)
    st.step(45)
    comps = st.read_components()
    for k, sc in enumerate(scenes):
        ref = oracle_run(sc, 45)
        for c, (a, b) in enumerate(zip(st.scene_components(k, comps), ref)):
            np.testing.assert_array_equal(a, b, err_msg=f"tiling {tiling} scene {k} component {c}")
    frozen_cells_are_zero(st, comps)
    st.close()


def test_ragged_compaction_keeps_scenes_bit_exact():
    scenes = scenes_of(DIMS, seed0=30, pml=5)
    st = ragged_stack(scenes)
    st.step(20)
    st.compact([False, True, False, True])
    assert st.scene_dims() == [DIMS[1], DIMS[3]]
    st.step(17)
    comps = st.read_components()
    for k, sc in enumerate((scenes[1], scenes[3])):
        ref = oracle_run(sc, 37)
        for c, (a, b) in enumerate(zip(st.scene_components(k, comps), ref)):
            np.testing.assert_array_equal(a, b, err_msg=f"kept scene {k} component {c}")
    frozen_cells_are_zero(st, comps)
    st.close()


def test_ragged_stack_refuses_other_kernels():
    scenes = scenes_of(DIMS[:2], pml=4)
    st = ragged_stack(scenes)
    with pytest.raises(EmlabError, match="pair"):
        st.set_tiling(8)
    with pytest.raises(EmlabError, match="fused kernel only"):
        st.set_kernel(abi.KERNEL_SPLIT)
    st.step(2)
    st.close()


def test_ragged_batch_runner_equals_one_stack_per_cross_section():
    scs = [configs.batched_scene(9, i) for i in range(60)]
    pick = [sc for sc in scs if sc.grid.size[0] in (48, 64, 80)][:7]
    assert len({sc.grid.size[0] for sc in pick}) >= 2
    out = {}
    for layout in ("ragged", "cross_section"):
        run = batch.BatchRunner(pick, chunk=64, max_steps=20000, layout=layout)
        out[layout] = run.run()
        assert len(run.groups) == (1 if layout == "ragged" else len({sc.grid.size[0] for sc in pick}))
        run.close()
    for a, b in zip(out["ragged"], out["cross_section"]):
        assert a.done and a.rung_down and a.steps == b.steps
        np.testing.assert_array_equal(np.concatenate(a.series), np.concatenate(b.series))
        np.testing.assert_array_equal(a.sweep["z"], b.sweep["z"])
