"""The learned extrapolator's kernels on the GPU: the tcgen05 BF16 GEMM against FP64 products of the
same BF16 operands, the whole forward and backward pass against the CPU restatement
(oracle/extrap_ref.py), and training that reduces the loss.

Tolerances: GEMM results within 1e-5 of max |C| (the products of BF16 operands are exact in FP32;
only the accumulation order differs). Network outputs and gradients within 2e-2 in norm: both sides
round activations and backward operands to BF16 at the same points, and a last-bit difference of an
FP32 sum can move such a rounding by one BF16 step (2^-8)."""
import numpy as np
import pytest

from em_lab_gb300 import extrap
from oracle import extrap_ref as R

pytestmark = pytest.mark.gpu


def gemm_case(M, N, K, transA, transB, seed=0):
    import torch
    rng = np.random.default_rng(seed)
    a = R.bf16(rng.standard_normal((M, K)).astype(np.float32))
    b = R.bf16(rng.standard_normal((N, K)).astype(np.float32))
    ref = a.astype(np.float64) @ b.astype(np.float64).T
    # store A as (M, K) or (K, M), B as (N, K) or (K, N); pass the matching strides
    A = torch.from_numpy(np.ascontiguousarray(a.T if transA else a)).to("cuda").to(torch.bfloat16)
    Bm = torch.from_numpy(np.ascontiguousarray(b.T if transB else b)).to("cuda").to(torch.bfloat16)
    sam, sak = (1, M) if transA else (K, 1)
    sbn, sbk = (1, N) if transB else (K, 1)
    out = torch.zeros((M, N), dtype=torch.float32, device="cuda")
    net = extrap.Net.__new__(extrap.Net)  # only the launch helper is used
    net.torch = torch
    net.lib = extrap._nn_lib()
    net._gemm(M, N, K, A, sam, sak, Bm, sbn, sbk, out, N)
    net.status()
    return out.cpu().numpy().astype(np.float64), ref


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (300, 200, 100), (7, 129, 1), (256, 1280, 256), (64, 16, 4096)])
@pytest.mark.parametrize("transA,transB", [(False, False), (True, False), (False, True), (True, True)])
def test_gemm_bf16_tensor_cores(M, N, K, transA, transB):
    got, ref = gemm_case(M, N, K, transA, transB, seed=M + N + K)
    scale = max(np.abs(ref).max(), 1.0)
    assert np.abs(got - ref).max() <= 1e-5 * scale * max(1.0, K / 64)


def test_forward_and_gradients_match_the_cpu_restatement():
    rng = np.random.default_rng(3)
    params = extrap.init_params(5)
    params = {k: (w, (rng.standard_normal(b.shape) * 0.05).astype(np.float32)) for k, (w, b) in params.items()}
    n = 37  # fewer rows than the batch: padding rows must not contribute
    x = rng.standard_normal((n, extrap.T_IN, 2)).astype(np.float32)
    zt = (rng.standard_normal((n, extrap.AUX)) * 0.5).astype(np.float32)
    t = (rng.standard_normal((n, extrap.OUT)) * 0.5).astype(np.float32)
    net = extrap.Net(params, batch=64)
    net.load(x, zt, t)
    y = net.forward()[:n].cpu().numpy()
    net.backward()
    net.status()
    g = net.grads()
    yr, cache = R.forward(params, x, zt)
    gr = R.backward(params, cache, t, n)

    def rel(a, b):
        return np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30)

    assert rel(y, yr) < 2e-2
    for name in gr:
        assert rel(g[name][0], gr[name][0]) < 2e-2, name
        assert rel(g[name][1], gr[name][1]) < 2e-2, name
    loss = float(net.loss.item())
    assert loss == pytest.approx(float(np.mean((yr - t) ** 2)), rel=2e-2)


def test_training_reduces_the_loss():
    """A learnable mapping (targets a fixed smooth function of the truncated-DFT features and of
    the signal) is fitted: the loss falls at least fivefold."""
    rng = np.random.default_rng(0)
    n = 512
    x = rng.standard_normal((n, extrap.T_IN, 2)).astype(np.float32) * 0.3
    zt = rng.standard_normal((n, extrap.AUX)).astype(np.float32) * 0.5
    t = (0.8 * zt[:, :extrap.OUT] + 0.2 * np.tanh(zt[:, ::-1][:, :extrap.OUT]) + 0.1 * x[:, :1, 0]).astype(np.float32)
    net, losses = extrap.train(x, zt, t, epochs=200, batch=64, lr=2e-3, seed=1)
    assert losses[-1] < 0.2 * losses[0]
    assert all(np.isfinite(losses))


def test_trained_network_beats_the_truncated_dft_on_held_out_scenes():
    """Trained on runs of small seeded scenes (edges 48 and 64) generated by the batched solver, the
    network's Z(f) from the early window is closer to the plain ring-down result than the early window's
    own DFT (the method without the network) on scenes of another seed."""
    out, _ = extrap.experiment(101, 512, 202, 64, epochs=200, edges=(48, 64))
    net, trunc = out["eval"]["network"], out["eval"]["truncated_dft"]
    assert out["eval"]["compared"] >= 60
    assert net["dz_median"] < 0.7 * trunc["dz_median"]
    assert net["s11_db_median"] < trunc["s11_db_median"]
    assert out["speedup"] > 1.0


def test_ensemble_with_plain_fallback_on_two_windows():
    """The learned path with its fallback: ensembles of two networks per early window (2 and 4
    design periods), a spread threshold from a validation split, the rejected scenes re-run by the
    plain solver (their Z(f) is then the plain solver's own), and the single-grid plain arm."""
    out, _ = extrap.experiment(303, 384, 404, 32, epochs=60, edges=(48, 64), periods=(2, 4), members=2,
                               val_frac=0.25, single=True)
    assert set(out["windows"]) == {"2", "4"} and out["chosen_window"] in out["windows"]
    assert out["plain"]["single_sweeps_per_hour"] > 0
    for w in out["windows"].values():
        v = w["validation"]
        assert 0.0 <= v["accepted"] <= 1.0 and 0.0 < v["cell_steps_vs_plain"] <= 1.0 + 1e-9
        hyb, net = w["eval"]["with_fallback"], w["eval"]["network"]
        assert hyb["dz_median"] <= net["dz_median"] + 1e-12 or w["eval"]["fallback_scenes"] == 0
        assert w["sweeps_per_hour"] > 0 and w["speedup_vs_single_plain"] > 0
