"""The surface DFT of stacked scenes (emlab_ntff_dft_configure_boxes, emlab_ntff_dft_spectra): the
sums of every box equal those of its scene on a grid of its own, bit for bit, before and after a
stack compaction; the per-box spectra equal the single-box pattern evaluation; and the batched
runner's far-field spectra equal one grid per scene's."""
import numpy as np
import pytest

from em_lab_gb300 import abi, batch, configs
from em_lab_gb300.grid import SceneStack, SimulationGrid

pytestmark = pytest.mark.gpu

WL = [12.0, 14.5, 17.0, 23.0]


def scenes_xy(nx, ny, depths, seeds, **kw):
    return [configs.random_scene(size=(nx, ny, nz), seed=s, **kw) for nz, s in zip(depths, seeds)]


def stack_of(scenes):
    st = SceneStack(scenes[0].grid, [sc.grid.size[2] for sc in scenes])
    for k, sc in enumerate(scenes):
        m = sc.materials
        st.upload_scene_materials(k, m.sigma, m.epsilon_r, sc.edges, sc.wires)
    st.set_scene_sources([sc.sources for sc in scenes])
    return st


def alone(sc, parts, engine, block=64):
    """The scene on its own grid with its box, stepped in `parts` (the sums folded after each part)."""
    g = SimulationGrid(sc.grid)
    m = sc.materials
    g.upload_materials(m.sigma, m.epsilon_r, sc.edges, sc.wires)
    g.set_sources(sc.sources)
    g.ntff_dft_configure_boxes([batch.FarField.box(sc)], WL, block=block)
    g.ntff_dft_engine(engine)
    for n in parts:
        g.step(n)
        x = g.ntff_dft_read()
    g.close()
    return x


def box_slices(st, x):
    """Split the stack's sums (f, points, 6, 2) into its boxes, in order."""
    out, first = [], 0
    for sc, z in zip(*st._far_scenes):
        b = batch.FarField.box(sc, z)
        n = [b[3] - b[0] + 1, b[4] - b[1] + 1, b[5] - b[2] + 1]
        pts = 2 * (n[1] * n[2] + n[0] * n[2] + n[0] * n[1])
        out.append(x[:, first:first + pts])
        first += pts
    assert first == x.shape[1]
    return out


def attach(st, scenes, block=64):
    z0, _ = st.layout()
    st.ntff_dft_configure_boxes([batch.FarField.box(sc, z) for sc, z in zip(scenes, z0)], WL, block=block)
    st._far_scenes = (scenes, z0)


@pytest.mark.parametrize("engine", [abi.DFT_TENSOR, abi.DFT_CUDA_CORES])
def test_boxes_of_a_stack_equal_scenes_alone(engine):
    scenes = scenes_xy(24, 20, (18, 26, 21), (1, 2, 3), pml=4)
    st = stack_of(scenes)
    attach(st, scenes)
    st.ntff_dft_engine(engine)
    st.step(150)  # two whole 64-sample blocks and a partial one
    x = st.ntff_dft_read()
    assert st.ntff_dft_info()[1] == 150
    for k, (got, sc) in enumerate(zip(box_slices(st, x), scenes)):
        ref = alone(sc, [150], engine)
        assert got.shape == ref.shape
        np.testing.assert_array_equal(got, ref, err_msg=f"box {k}")
        assert np.abs(ref).max() > 0.0
    st.close()


def test_compaction_keeps_the_boxes_of_kept_scenes():
    scenes = scenes_xy(24, 20, (18, 26, 21), (4, 5, 6), pml=4)
    st = stack_of(scenes)
    attach(st, scenes)
    st.step(100)
    st.compact([True, False, True])
    kept = [scenes[0], scenes[2]]
    st._far_scenes = (kept, st.layout()[0])
    st.step(70)
    x = st.ntff_dft_read()
    assert st.ntff_dft_info()[1] == 170
    for got, sc in zip(box_slices(st, x), kept):
        # the compaction folds the partial block at step 100: the scene alone folds there too
        np.testing.assert_array_equal(got, alone(sc, [100, 70], abi.DFT_TENSOR))
    st.close()


def test_spectra_of_one_box_equal_the_pattern_evaluation():
    sc = scenes_xy(28, 28, (28,), (7,), pml=4)[0]
    g = SimulationGrid(sc.grid)
    m = sc.materials
    g.upload_materials(m.sigma, m.epsilon_r, sc.edges, sc.wires)
    g.set_sources(sc.sources)
    g.ntff_dft_configure_boxes([batch.FarField.box(sc)], WL, block=0)
    g.step(200)
    ff = batch.FarField(len(WL))
    spec = g.ntff_dft_spectra(0, ff.dirs)
    ref = g.ntff_dft_evaluate_all(ff.dirs)
    np.testing.assert_array_equal(spec, ref)
    assert spec[:, 0, 1].min() > 0.0 and np.isfinite(spec).all()
    g.close()


def test_spectra_need_a_valid_box_and_samples():
    sc = scenes_xy(24, 20, (18, 21), (8, 9), pml=4)
    st = stack_of(sc)
    attach(st, sc)
    ff = batch.FarField(len(WL))
    with pytest.raises(RuntimeError, match="no far-field DFT samples"):
        st.ntff_dft_spectra(0, ff.dirs)
    st.step(10)
    with pytest.raises(RuntimeError, match="no such far-field DFT box"):
        st.ntff_dft_spectra(2, ff.dirs)
    with pytest.raises(RuntimeError, match="several boxes"):
        st.ntff_dft_evaluate_all(ff.dirs)
    with pytest.raises(RuntimeError, match="leaves the grid"):
        st.ntff_dft_configure_boxes([[0, 1, 1, 10, 10, 10]], WL)
    st.close()


def test_batched_far_field_spectra_equal_one_grid_per_scene():
    """The batched runner (scene stacks, compaction) records each scene's spectra at ring-down and at
    its snapshot steps; they equal the scene run alone to the same step (the folds fall at other
    steps, so to FP32 rounding), and a dipole's directivity is a dipole's."""
    scenes = [configs.batched_scene(31, i, edges=(48,)) for i in range(4)]
    ff = batch.FarField(32)
    snap = [[100] for _ in scenes]  # these scenes ring down within 300 to 600 steps
    run = batch.BatchRunner(scenes, chunk=64, max_steps=20000, far_field=ff, snap_at=snap)
    res = run.run()
    run.close()
    for sc, r in zip(scenes, res):
        assert r.done and r.rung_down and 100 in r.far and r.steps in r.far
        _, sweep = batch.run_single(sc, chunk=64, far_field=ff)
        np.testing.assert_allclose(r.far[r.steps], sweep["far"], rtol=1e-4, atol=1e-3)
        dbi = r.far[r.steps][0]
        assert np.all(np.isfinite(dbi)) and 1.0 < np.median(dbi) < 6.0, dbi
        # the snapshot at step 100 is an early window: less energy radiated than at the end
        assert np.median(r.far[100][1]) < np.median(r.far[r.steps][1])


@pytest.mark.parametrize("dims", [(40, 36, 30), (36, 28, 44)])
def test_factorised_pattern_equals_the_direct_sums(dims):
    """emlab_ntff_dft_pattern_gemm (per-face complex GEMMs on the tensor cores with split BF16
    operands) against emlab_ntff_dft_evaluate_all (the direct sums): the pattern within 2e-4 of its
    maximum at every frequency, the radiated power within 1e-5, on boxes whose faces all differ."""
    sc = scenes_xy(dims[0], dims[1], (dims[2],), (11,), pml=4)[0]
    g = SimulationGrid(sc.grid)
    m = sc.materials
    g.upload_materials(m.sigma, m.epsilon_r, sc.edges, sc.wires)
    g.set_sources(sc.sources)
    g.ntff_dft_configure_boxes([batch.FarField.box(sc)], WL, block=0)
    g.step(300)
    rng = np.random.default_rng(5)
    extra = rng.standard_normal((37, 3))
    dirs = np.concatenate([batch.FarField(len(WL)).dirs, extra / np.linalg.norm(extra, axis=1, keepdims=True)])
    got = g.ntff_dft_pattern_gemm(0, dirs)
    ref = g.ntff_dft_evaluate_all(dirs)
    for f in range(len(WL)):
        peak = np.abs(ref[f, :, 0]).max()
        assert peak > 0.0
        assert np.abs(got[f, :, 0] - ref[f, :, 0]).max() <= 2e-4 * peak, f
        assert got[f, 0, 1] == pytest.approx(ref[f, 0, 1], rel=1e-5)
        assert not got[f, 1:, 1].any()
    g.close()
