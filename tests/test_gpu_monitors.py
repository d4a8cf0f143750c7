"""GPU parity of the per-step and on-demand monitors (ports, far-field accumulation and pattern,
coax lines, probes, flux, frequency sweep) and of the golden fixtures made from the reference's
own shader code. Every per-step FP32 output must equal the oracle bit for bit; the far-field
pattern (sin/cos of CUDA vs the host libm) and the FP64 sweep sums have stated tolerances."""
import os

import numpy as np
import pytest

import oracle
from em_lab_gb300 import SimulationGrid, abi, configs

import golden.make_golden as mg

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PATTERN_RTOL = 2e-5  # far-field intensity, relative to the pattern maximum (FP32 sin/cos differences)


def compare(got, want, pattern_rtol=PATTERN_RTOL):
    for k in want:
        if k == "pattern":
            scale = np.abs(want[k][:, 0]).max()
            assert np.max(np.abs(got[k][:, 0] - want[k][:, 0])) <= pattern_rtol * scale, k
            assert abs(got[k][0, 1] - want[k][0, 1]) <= pattern_rtol * abs(want[k][0, 1]) + 1e-30, "radiated power"
        else:
            assert np.array_equal(got[k], want[k]), k


@pytest.mark.parametrize("seed,size,pml", [(1, (24, 20, 18), 4), (2, (37, 29, 23), 5), (8, (48, 40, 36), 6)])
def test_monitors_equal_oracle(seed, size, pml):
    sc = configs.random_scene(size=size, pml=pml, seed=seed)
    g = SimulationGrid(sc.grid)
    got = mg.run(g, sc, 70)
    want = mg.run(oracle.Oracle(sc.grid, "f32"), sc, 70)
    compare(got, want)


@pytest.mark.parametrize("name", ["random_s1", "random_s2", "vacuum_pml0"])
def test_gpu_matches_golden_fixtures(name):
    case = {c[0]: c for c in mg.CASES}[name]
    gold = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    sc = configs.random_scene(**case[1])
    out = mg.run(SimulationGrid(sc.grid), sc, int(gold["steps"]))
    assert mg.field_hash([out[f"f{c}"] for c in range(6)]) == str(gold["sha256"])
    want = {k: gold[k] for k in gold.files if k not in ("steps", "sha256") and not k.startswith("mid")}
    compare({k: out[k] for k in want}, want)


def test_sweep_sums_fp64():
    sc = configs.random_scene(size=(30, 28, 26), pml=5, seed=12)
    sc.sources[-1].waveform = abi.WAVE_PULSE
    ports = [p.to_c() for p in sc.ports]
    res = []
    for t in (SimulationGrid(sc.grid), oracle.Oracle(sc.grid, "f32")):
        oracle.load_scene(t, sc)
        t.ports_configure(ports, 12.0, 4.0, sweep=True)
        t.step(300)
        res.append((t.ports_series(), *t.ports_sweep_sums(8.0, 30.0, 64)))
    (s_gpu, sums_gpu, r_gpu), (s_cpu, sums_cpu, r_cpu) = res
    assert np.array_equal(s_gpu, s_cpu)
    scale = np.abs(sums_cpu).max()
    assert np.max(np.abs(sums_gpu - sums_cpu)) <= 1e-12 * scale * 300
    assert r_gpu == r_cpu


def test_port_residuals_on_the_device():
    """emlab_ports_residuals (every port's ring-down residual of Ports.cpp:206-213, on the device)
    equals the host evaluation of the same recorded series, for several lengths."""
    from em_lab_gb300 import batch
    sc = configs.random_scene(size=(30, 28, 26), pml=5, seed=12)
    sc.sources[-1].waveform = abi.WAVE_PULSE
    g = SimulationGrid(sc.grid)
    oracle.load_scene(g, sc)
    g.ports_configure([p.to_c() for p in sc.ports], 12.0, 4.0, sweep=True)
    for steps in (1, 19, 40, 333):
        g.step(steps if steps == 1 else steps - g.step_count())
        ser = g.ports_series()
        got = g.ports_residuals()
        want = [batch.residual(ser[:, p, 0]) for p in range(ser.shape[1])]
        assert np.array_equal(got, np.asarray(want)), (steps, got, want)
    g.close()


def test_check_finite():
    grid = abi.GridConfig((96, 96, 96), pml_thickness=8)
    g = SimulationGrid(grid)
    assert g.check_finite()
    comps = [np.zeros((96, 96, 96), np.float32) for _ in range(6)]
    comps[4][50, 40, 30] = np.nan
    g.write_components(comps)
    g.step(2)
    assert not g.check_finite()


def test_bounded_host_wait_runs_out():
    """A bounded host wait on the grid's stream (emlab_grid_synchronize) that runs out returns
    EMLAB_ERR_TIMEOUT and leaves the grid usable. The stream is kept busy deterministically: a
    bounded device sleep of about 0.2 s queued on the grid's own stream after the steps."""
    import torch
    from em_lab_gb300 import EmlabError
    g = SimulationGrid(abi.GridConfig((64, 64, 64), pml_thickness=8))
    g.step(10)
    g.synchronize(60000)
    with torch.cuda.stream(torch.cuda.ExternalStream(g.stream_handle())):
        torch.cuda._sleep(int(4e8))  # ~0.2 s of cycles at 2 GHz: a bounded spin, not a hang
    with pytest.raises(EmlabError) as e:
        g.synchronize(1)
    assert e.value.code == abi.EMLAB_ERR_TIMEOUT
    g.synchronize(60000)  # the same wait with room to finish succeeds
    g.step(4)
    g.synchronize(60000)
    assert g.step_count() == 14
    g.close()


@pytest.mark.parametrize("rows", [64, 8])
def test_device_wait_that_runs_out_reports_timeout(rows):
    """The solver kernel's bounded barrier wait made to run out (the test hook sets its poll count
    to 0): the CTAs record the error, wait with the full bound for the copies they already issued
    and leave; the host reports EMLAB_ERR_TIMEOUT; with the normal bound restored the same grid then
    steps bit for bit like the oracle (persistent pair tiles, tiling 64, and single-cell tiles, 8)."""
    from em_lab_gb300 import EmlabError, grid as gridmod
    sc = configs.random_scene(size=(70, 40, 36), pml=5, seed=31)
    g = SimulationGrid(sc.grid)
    g.set_tiling(rows)
    oracle.load_scene(g, sc)
    g.step(3)
    g.synchronize(60000)
    try:
        gridmod.debug_set_wait_limit(0)
        g.step(1)
        with pytest.raises(EmlabError) as e:
            g.synchronize(60000)
        assert e.value.code == abi.EMLAB_ERR_TIMEOUT
    finally:
        gridmod.debug_set_wait_limit(gridmod.WAIT_POLLS_DEFAULT)
    g.synchronize(60000)  # the error word was cleared by the report
    o = oracle.Oracle(sc.grid, "f32")
    oracle.load_scene(o, sc)
    oracle.load_scene(g, sc)  # fresh state on the same grid (fields, time) after the failed step
    for t in (g, o):
        t.step(25)
    for c, (a, b) in enumerate(zip(g.read_components(), o.read_components())):
        assert np.array_equal(a, b), c
    g.close()
    o.close()


def test_fold_wait_that_runs_out_reports_timeout():
    """The tensor-core DFT fold's bounded MMA wait made to run out: the fold records the error,
    waits with the full bound for its MMAs, frees its tensor memory and leaves; the host reports
    EMLAB_ERR_TIMEOUT and later folds on the same device are correct again."""
    from em_lab_gb300 import EmlabError, grid as gridmod
    sc = configs.random_scene(size=(40, 36, 34), pml=5, seed=37)
    g = SimulationGrid(sc.grid)
    oracle.load_scene(g, sc)
    g.ntff_dft_configure((7, 7, 7), (32, 28, 26), [9.0, 15.0])
    g.step(70)
    try:
        gridmod.debug_set_wait_limit(0)
        with pytest.raises(EmlabError) as e:
            g.ntff_dft_read()  # folds the partial block
            g.synchronize(60000)
        assert e.value.code == abi.EMLAB_ERR_TIMEOUT
    finally:
        gridmod.debug_set_wait_limit(gridmod.WAIT_POLLS_DEFAULT)
    g.synchronize(60000)
    o = oracle.Oracle(sc.grid, "f32")
    res = []
    for t in (g, o):
        oracle.load_scene(t, sc)  # fresh fields and time on the same grid
        t.ntff_dft_configure((7, 7, 7), (32, 28, 26), [9.0, 15.0])
        t.step(300)
        res.append(t.ntff_dft_read())
    g.close()
    o.close()
    scale = np.abs(res[1]).max()
    assert scale > 0 and np.max(np.abs(res[0] - res[1])) <= DFT_RTOL * scale


def test_plain_small_2000_steps():
    """The 128^3 plain-method workload run to 2000 steps: fields, probe block, flux box and far-field
    phasors bit-identical to the oracle; the FP64 error floor is reported per component."""
    sc = configs.plain_small()
    steps = 2000
    L = sc.grid.pml_thickness
    ff = sc.far_field
    bmin, bmax = sc.fluxes[0].box_min, sc.fluxes[0].box_max
    planes = []
    for ax in range(3):
        u, v = (1, 2) if ax == 0 else ((0, 2) if ax == 1 else (0, 1))
        for idx in (bmin[ax], bmax[ax]):
            planes.append(abi.FluxPlane(ax, idx, (bmin[u], bmin[v]), (bmax[u] + 1, bmax[v] + 1)))
    origin = [(33, 63, 63)]
    out = {}
    for label, t in (("gpu", SimulationGrid(sc.grid)), ("f32", oracle.Oracle(sc.grid, "f32")),
                     ("f64", oracle.Oracle(sc.grid, "f64"))):
        oracle.load_scene(t, sc)
        t.ntff_configure(ff["box_min"], ff["box_max"], ff["wavelength"], ff["averaging"])
        t.step(steps)
        out[label] = dict(f=t.read_components(), probe=t.probe_gather(origin), flux=t.flux_planes(planes),
                          ntff=t.ntff_phasors())
    for c in range(6):
        assert np.array_equal(out["gpu"]["f"][c], out["f32"]["f"][c]), c
        b = out["f64"]["f"][c]
        rel = np.linalg.norm(out["gpu"]["f"][c].astype(np.float64) - b) / np.linalg.norm(b)
        print(f"component {c}: relative L2 vs FP64 oracle {rel:.3e}")
        assert rel < 1e-5  # measured on GB300: 6.2e-7 .. 6.2e-6 (Bz largest)
    for k in ("probe", "flux", "ntff"):
        assert np.array_equal(out["gpu"][k], out["f32"][k]), k


DFT_RTOL = 2e-6  # multi-frequency DFT sums, relative to the largest |sum| (FP32 in-block arithmetic)


@pytest.mark.parametrize("engine", [abi.DFT_TENSOR, abi.DFT_CUDA_CORES])
def test_multifrequency_dft_matches_fp64_oracle(engine):
    """The time-blocked multi-frequency far-field DFT (FP32 samples; in-block sums on the tensor
    cores with split TF32 operands, or FP32 FMA sums; block phase applied in FP32 from FP64 cos/sin;
    FP64 accumulation) against the oracle's FP64 DFT with exact phases on the same FP32 samples; a
    read in the middle folds a partial block and stepping continues."""
    sc = configs.random_scene(size=(36, 32, 30), pml=4, seed=13)
    wls = [9.0, 12.0, 16.0, 24.0, 40.0]
    res = []
    for t in (SimulationGrid(sc.grid), oracle.Oracle(sc.grid, "f32")):
        oracle.load_scene(t, sc)
        if isinstance(t, SimulationGrid):
            t.ntff_dft_engine(engine)
        box = t.ntff_dft_configure((6, 6, 6), (29, 25, 23), wls)
        t.step(100)
        mid = t.ntff_dft_read()
        t.step(90)
        res.append((box, mid, t.ntff_dft_read()))
    (bg, mg_, xg), (bc, mc, xc) = res
    assert bg == bc
    for got, want in ((mg_, mc), (xg, xc)):
        scale = np.abs(want).max()
        assert scale > 0
        err = np.max(np.abs(got - want)) / scale
        print(f"engine {engine}: max |DFT - FP64 oracle| / max |DFT| = {err:.3e}")
        assert err <= DFT_RTOL
    g = SimulationGrid(sc.grid)
    oracle.load_scene(g, sc)
    g.ntff_dft_configure((6, 6, 6), (29, 25, 23), wls)
    g.step(130)
    pat = g.ntff_dft_evaluate(2, configs.fibonacci_directions(200))
    assert np.all(np.isfinite(pat)) and pat[0, 1] != 0.0


PATTERN_FAST_RTOL = 1e-4  # |fast - parity| / max pattern: 2-pi reduced hardware sin/cos and FMA sums


def test_dft_pattern_all_frequencies_matches_parity_kernel():
    """emlab_ntff_dft_evaluate_all (two directions per thread, range-reduced hardware sin/cos, FMA
    sums) against emlab_ntff_dft_evaluate (the reference-parity pattern sums) at every frequency,
    over 1000 directions (more than one 256-direction block and a ragged last block), including
    the radiated power reported on the first direction only."""
    sc = configs.random_scene(size=(48, 44, 40), pml=5, seed=23)
    wls = [6.0, 9.0, 14.0, 30.0]
    g = SimulationGrid(sc.grid)
    oracle.load_scene(g, sc)
    g.ntff_dft_configure((7, 7, 7), (40, 36, 32), wls)
    g.step(150)
    dirs = configs.fibonacci_directions(1000)
    fast = g.ntff_dft_evaluate_all(dirs)
    assert fast.shape == (len(wls), len(dirs), 2)
    for f in range(len(wls)):
        ref = g.ntff_dft_evaluate(f, dirs)
        scale = ref[:, 0].max()
        assert scale > 0
        err = np.max(np.abs(fast[f, :, 0] - ref[:, 0])) / scale
        print(f"frequency {f}: max |fast - parity| / max pattern = {err:.2e}")
        assert err <= PATTERN_FAST_RTOL
        assert fast[f, 0, 1] == pytest.approx(ref[0, 1], rel=1e-5)
        assert np.all(fast[f, 1:, 1] == 0.0)
    g.close()


@pytest.mark.parametrize("nf", [1, 16, 48, 128])
def test_dft_tensor_engine_equals_cuda_cores(nf):
    """Tensor-core and CUDA-core folds of the same samples over several blocks and a partial one,
    for MMA widths N = 32, 96 and 256 (tensor-core blocks of 256, 256, 128 and 64 samples folded as
    64-sample chunks; CUDA-core blocks of 64): the two engines agree to the FP32 level of the
    in-block sums."""
    sc = configs.random_scene(size=(44, 40, 38), pml=5, seed=17)
    wls = list(np.linspace(6.0, 60.0, nf)) if nf > 1 else [16.0]
    out = []
    for engine in (abi.DFT_TENSOR, abi.DFT_CUDA_CORES):
        g = SimulationGrid(sc.grid)
        oracle.load_scene(g, sc)
        g.ntff_dft_engine(engine)
        g.ntff_dft_configure((7, 7, 7), (36, 32, 30), wls)
        g.step(256 * 2 + 81)
        out.append(g.ntff_dft_read())
    a, b = out
    scale = np.abs(b).max()
    assert scale > 0 and np.all(np.isfinite(a))
    assert np.max(np.abs(a - b)) <= DFT_RTOL * scale


def test_dft_engine_switch_inside_a_block():
    """Switching the fold engine in the middle of a block folds the partial block with the engine
    that gathered it; the sums match a run on one engine throughout."""
    sc = configs.random_scene(size=(40, 36, 34), pml=5, seed=19)
    wls = [8.0, 13.0, 21.0]
    out = []
    for switch in (True, False):
        g = SimulationGrid(sc.grid)
        oracle.load_scene(g, sc)
        g.ntff_dft_configure((7, 7, 7), (32, 28, 26), wls)
        g.step(150)  # inside the tensor engine's first 256-sample block
        if switch:
            g.ntff_dft_engine(abi.DFT_CUDA_CORES)
        g.step(200)
        out.append(g.ntff_dft_read())
        g.close()
    scale = np.abs(out[1]).max()
    assert scale > 0 and np.max(np.abs(out[0] - out[1])) <= DFT_RTOL * scale


def test_analyzer_submit_collect_matches_synchronous_reads():
    """FieldAnalyzer::submit / collect returns, one frame late, exactly what the synchronous probe
    gather and flux planes return at the step it was submitted."""
    import numpy as np
    from em_lab_gb300 import SimulationGrid, abi, configs
    import oracle
    sc = configs.random_scene(size=(40, 36, 30), pml=5, seed=3)
    g = SimulationGrid(sc.grid)
    oracle.load_scene(g, sc)
    origins = [(10, 12, 9), (0, 0, 0), (37, 33, 27)]
    planes = [abi.FluxPlane(0, 12, (3, 4), (30, 25)), abi.FluxPlane(2, 15, (0, 0), (40, 36))]
    assert g.analyzer_collect() is None
    expected = []
    for frame in range(4):
        g.step(3)
        expected.append((g.probe_gather(origins), g.flux_planes(planes)))
        got = g.analyzer_collect()
        if frame:
            np.testing.assert_array_equal(got[0], expected[frame - 1][0])
            np.testing.assert_array_equal(got[1], expected[frame - 1][1])
        g.analyzer_submit(origins, planes)
    got = g.analyzer_collect()
    np.testing.assert_array_equal(got[0], expected[3][0])
    np.testing.assert_array_equal(got[1], expected[3][1])
    g.close()
