"""Learned ring-down extrapolator: predicts a scene's converged port impedance Z(f) and far-field
spectra from the first few periods of its port V(t), I(t) and of its surface DFT, so an antenna
sweep can stop each scene early.

Network (every layer a GEMM on the tcgen05 tensor cores with BF16 operands and FP32 accumulation,
csrc/learn.cu; FP32 master weights and Adam):
  encoder  conv1d 2 -> 32 channels (kernel 8, stride 4, pad 2, ReLU): 256 samples -> 64 positions
           conv1d 32 -> 64 channels (kernel 8, stride 4, pad 2, ReLU): 64 -> 16 positions
  head     [1024 encoder features | 256 truncated-DFT Z features | 64 surface-DFT features]
           -> 256 -> 256 -> 256 -> 256 (ReLU)
           -> 320 outputs: Re, Im of Z(f) / 100 ohm at the 128 sweep frequencies, then the far-field
              spectra at the 32 surface-DFT frequencies: directivity (dBi / 10) and radiated energy
              (dB / 10, batch.FarField).
Inputs (host, from the early window of `PERIODS_IN` design periods): V and I resampled to 256
points in units of the period (I scaled by eta0 / 100, both by the window's peak); the "method
without the network": Z_trunc(f) = -V(f) / I(f) * eta0 from the DFT of the early window alone, and
the far-field spectra of the Huygens box's DFT over the early window alone (32 surface-DFT channels:
the directivity and the radiated energy at each frequency).
Targets: Z(f) and the far-field spectra of the whole run to -60 dB ring-down (the plain solver is
the reference result).
PyTorch only allocates the device buffers and moves the batches; every forward and backward
operation is a kernel of this library.
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np

from .batch import K_ETA0, FarField, sweep_sums
from .grid import _check, load_library

T_IN = 256             # resampled early-window samples per channel
PERIODS_IN = 4.0       # early window, design periods
NF = 128               # sweep frequencies
NFF = 32               # far-field (surface-DFT) frequencies
Z_SCALE = 100.0        # ohm per output unit
Z_CLIP = 10.0          # feature / target clip (units of Z_SCALE)
DB_SCALE = 10.0        # dB per far-field output unit
I_SCALE = K_ETA0 / 100.0
AUX = 2 * NF + 2 * NFF  # head inputs beside the encoder: truncated Z(f), truncated far-field spectra
OUT = 2 * NF + 2 * NFF  # outputs: Z(f), far-field spectra

CONV = [  # (name, c_in, c_out, kernel, stride, pad, L_in, L_out)
    ("conv1", 2, 32, 8, 4, 2, 256, 64),
    ("conv2", 32, 64, 8, 4, 2, 64, 16),
]
ENC = CONV[-1][2] * CONV[-1][7]  # 1024 encoder features
HEAD = [("fc1", ENC + AUX, 256, True), ("fc2", 256, 256, True), ("fc3", 256, 256, True),
        ("fc4", 256, 256, True), ("out", 256, OUT, False)]


def far_field() -> FarField:
    """The surface DFT the extrapolator reads and predicts: NFF frequencies over the sweep band."""
    return FarField(NFF)


def layer_shapes():
    """(name, fan_out, fan_in) of every weight matrix; conv weights are (c_out, kernel * c_in)."""
    s = [(n, co, k * ci) for n, ci, co, k, *_ in CONV]
    s += [(n, o, i) for n, i, o, _ in HEAD]
    return s


def init_params(seed: int = 0):
    """He-initialised FP32 weights and zero biases: {name: (W (out, in), b (out,))}."""
    rng = np.random.default_rng(seed)
    p = {}
    for name, o, i in layer_shapes():
        scale = math.sqrt(2.0 / i) if name != "out" else math.sqrt(1.0 / i)
        p[name] = (rng.standard_normal((o, i)).astype(np.float32) * np.float32(scale), np.zeros(o, np.float32))
    return p


# ---- features ------------------------------------------------------------------------------------
def early_steps(sc, periods: float | None = None) -> int:
    p = PERIODS_IN if periods is None else float(periods)
    return int(math.ceil(p * sc.wavelength / float(sc.grid.courant)))


def truncated_z(sc, series_early):
    """The method without the network: Z(f) from the DFT of the early window alone."""
    from .batch import impedance
    sw = sc.sweep
    sums = sweep_sums(series_early, sw["wavelength_min"], sw["wavelength_max"], NF, float(sc.grid.courant))
    return impedance(sums, sw["wavelength_min"], sw["wavelength_max"], float(sc.ports[0].impedance_ohm))["z"]


def far_units(spec):
    """Far-field spectra (2, NFF) (dBi, dB) -> 2 NFF network units (clipped)."""
    return np.clip(np.asarray(spec, np.float64).reshape(-1) / DB_SCALE, -Z_CLIP, Z_CLIP).astype(np.float32)


def features(sc, series, far_early):
    """(x (T_IN, 2) float32 position-major, aux (AUX,) float32, Z_trunc complex (NF,)) from the first
    early_steps(sc) rows of a scene's (V, I) series and the far-field spectra (2, NFF) of its
    surface DFT over the same steps."""
    n = early_steps(sc)
    ser = np.asarray(series[:n], np.float64)
    if ser.shape[0] < n:
        raise ValueError("series shorter than the early window")
    t = np.arange(T_IN) * (n / T_IN)
    k = np.arange(n)
    v = np.interp(t, k, ser[:, 0])
    i = np.interp(t, k, ser[:, 1]) * I_SCALE
    peak = max(np.abs(v).max(), np.abs(i).max(), 1e-30)
    x = np.stack([v / peak, i / peak], axis=1).astype(np.float32)
    zt = truncated_z(sc, ser.astype(np.float32))
    zf = np.concatenate([np.clip(zt.real / Z_SCALE, -Z_CLIP, Z_CLIP), np.clip(zt.imag / Z_SCALE, -Z_CLIP, Z_CLIP),
                         far_units(far_early)])
    return x, zf.astype(np.float32), zt


def target(z_conv, far_conv):
    return np.concatenate([np.clip(z_conv.real / Z_SCALE, -Z_CLIP, Z_CLIP),
                           np.clip(z_conv.imag / Z_SCALE, -Z_CLIP, Z_CLIP), far_units(far_conv)]).astype(np.float32)


def to_z(y):
    y = np.asarray(y, np.float64)
    return (y[..., :NF] + 1j * y[..., NF:2 * NF]) * Z_SCALE


def to_far(y):
    """Network outputs -> far-field spectra (..., 2, NFF): dBi, dB."""
    y = np.asarray(y, np.float64)[..., 2 * NF:2 * NF + 2 * NFF] * DB_SCALE
    return y.reshape(y.shape[:-1] + (2, NFF))


# ---- device network --------------------------------------------------------------------------------
class Net:
    """The extrapolator on the GPU: FP32 master weights, BF16 copies, Adam state, activations for a
    batch of up to `batch` rows. forward() / backward() / step() launch this library's kernels."""

    def __init__(self, params, batch: int = 256, device: str = "cuda"):
        import torch
        self.torch = torch
        self.lib = _nn_lib()
        self.B = int(batch)
        self.dev = device
        f32, bf16 = torch.float32, torch.bfloat16
        self.W, self.Wb, self.b, self.mW, self.vW, self.mb, self.vb, self.gW, self.gb = {}, {}, {}, {}, {}, {}, {}, {}, {}
        for name, o, i in layer_shapes():
            w, b = params[name]
            self.W[name] = torch.from_numpy(np.ascontiguousarray(w)).to(device)
            self.Wb[name] = torch.empty((o, i), dtype=bf16, device=device)
            self.b[name] = torch.from_numpy(np.ascontiguousarray(b)).to(device)
            for d, shape in ((self.mW, (o, i)), (self.vW, (o, i)), (self.gW, (o, i)), (self.mb, (o,)),
                             (self.vb, (o,)), (self.gb, (o,))):
                d[name] = torch.zeros(shape, dtype=f32, device=device)
            self._conv(self.W[name], self.Wb[name])
        B = self.B
        z = lambda *s, dt=f32: torch.zeros(s, dtype=dt, device=device)  # noqa: E731
        self.x0 = z(B, T_IN, 2, dt=bf16)
        self.cols1 = z(B * 64, 16, dt=bf16)
        self.z1 = z(B * 64, 32)
        self.a1 = z(B * 64, 32, dt=bf16)
        self.cols2 = z(B * 16, 256, dt=bf16)
        self.z2 = z(B * 16, 64)
        self.X0 = z(B, ENC + AUX, dt=bf16)
        self.zh = {n: z(B, o) for n, i, o, _ in HEAD}
        self.ah = {n: z(B, o, dt=bf16) for n, i, o, r in HEAD if r}
        self.y = self.zh["out"]
        self.t = z(B, OUT)
        self.dy = z(B, OUT)
        self.dz = {n: z(B, o) for n, i, o, _ in HEAD}
        self.dzb = {n: z(B, o, dt=bf16) for n, i, o, _ in HEAD}
        self.dx = {n: z(B, i) for n, i, o, _ in HEAD}
        self.dz2 = z(B * 16, 64)
        self.dz2b = z(B * 16, 64, dt=bf16)
        self.dcols2 = z(B * 16, 256)
        self.da1 = z(B * 64, 32)
        self.dz1 = z(B * 64, 32)
        self.dz1b = z(B * 64, 32, dt=bf16)
        self.loss = z(1)
        self.t_step = 0
        self.n = 0

    # -- helpers
    @property
    def stream(self):
        return C.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def _p(self, t):
        return C.c_void_p(t.data_ptr())

    def _fp(self, t):
        return C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_float))

    def _conv(self, src, dst_bf, ldo=None, cols=None, off=0):
        n = src.numel()
        cols = cols or (src.shape[-1] if src.dim() > 1 else n)
        _check(self.lib.emlab_nn_to_bf16(self._fp(src), n, self._p(dst_bf), ldo or cols, cols, off, self.stream))

    def _gemm(self, M, N, K, A, sam, sak, B, sbn, sbk, Cc, ldc):
        _check(self.lib.emlab_nn_gemm(M, N, K, self._p(A), sam, sak, self._p(B), sbn, sbk, self._fp(Cc), ldc,
                                      self.stream))

    def _bias_act(self, z, bias, M, N, relu, out, ldo, off, bias_n):
        _check(self.lib.emlab_nn_bias_act(self._fp(z), self._fp(bias), M, N, bias_n, 1 if relu else 0,
                                          self._p(out) if out is not None else None, ldo, off, self.stream))

    def load(self, x, zt, t=None):
        """A batch: x (n, T_IN, 2), head inputs zt (n, AUX), targets t (n, OUT) (float32 host arrays)."""
        torch = self.torch
        n = x.shape[0]
        assert n <= self.B
        self.n = n
        xs = torch.zeros((self.B, T_IN, 2), dtype=torch.float32, device=self.dev)
        xs[:n] = torch.from_numpy(np.ascontiguousarray(x, np.float32)).to(self.dev)
        zs = torch.zeros((self.B, AUX), dtype=torch.float32, device=self.dev)
        zs[:n] = torch.from_numpy(np.ascontiguousarray(zt, np.float32)).to(self.dev)
        self._conv(xs.view(self.B * T_IN, 2), self.x0.view(self.B * T_IN, 2))
        self._conv(zs, self.X0, ldo=ENC + AUX, cols=AUX, off=ENC)
        self.t.zero_()
        if t is not None:
            self.t[:n] = torch.from_numpy(np.ascontiguousarray(t, np.float32)).to(self.dev)

    # -- forward / backward
    def forward(self):
        B, lib, s = self.B, self.lib, self.stream
        c1, c2 = CONV
        _check(lib.emlab_nn_im2col(self._p(self.x0), B, c1[6], c1[1], c1[3], c1[4], c1[5], c1[7], self._p(self.cols1), s))
        self._gemm(B * 64, 32, 16, self.cols1, 16, 1, self.Wb["conv1"], 16, 1, self.z1, 32)
        self._bias_act(self.z1, self.b["conv1"], B * 64, 32, True, self.a1, 32, 0, 32)
        _check(lib.emlab_nn_im2col(self._p(self.a1), B, c2[6], c2[1], c2[3], c2[4], c2[5], c2[7], self._p(self.cols2), s))
        self._gemm(B * 16, 64, 256, self.cols2, 256, 1, self.Wb["conv2"], 256, 1, self.z2, 64)
        # rows (b, l) of z2 are the encoder features of sample b at columns l * 64 + c
        self._bias_act(self.z2, self.b["conv2"], B, ENC, True, self.X0, ENC + AUX, 0, 64)
        x = self.X0
        for name, i, o, relu in HEAD:
            self._gemm(B, o, i, x, i, 1, self.Wb[name], i, 1, self.zh[name], o)
            out = self.ah.get(name)
            self._bias_act(self.zh[name], self.b[name], B, o, relu, out, o, 0, o)
            x = out
        return self.y

    def backward(self):
        """MSE gradients of every weight and bias (loss over the loaded rows; padding rows carry zero
        targets and zero outputs' gradient is masked by the row count)."""
        B, lib, s = self.B, self.lib, self.stream
        n = self.n
        self.loss.zero_()
        # only the loaded rows contribute: gradient rows beyond n are zero
        self.dy.zero_()
        _check(lib.emlab_nn_mse(self._fp(self.y), self._fp(self.t), n * OUT, self._fp(self.dy),
                                self._fp(self.loss), s))
        up = self.dy
        ins = {"fc1": self.X0}
        for k in range(1, len(HEAD)):
            ins[HEAD[k][0]] = self.ah[HEAD[k - 1][0]]
        for name, i, o, relu in reversed(HEAD):
            dz, dzb = self.dz[name], self.dzb[name]
            _check(lib.emlab_nn_act_grad(self._fp(up), o, 0, self._fp(self.zh[name]), B, o, 1 if relu else 0,
                                         self._fp(dz), self._p(dzb), s))
            self._gemm(o, i, B, dzb, 1, o, ins[name], 1, i, self.gW[name], i)
            _check(lib.emlab_nn_col_sum(self._fp(dz), B, o, self._fp(self.gb[name]), s))
            self._gemm(B, i, o, dzb, o, 1, self.Wb[name], 1, i, self.dx[name], i)
            up = self.dx[name]
        c2 = CONV[1]
        # conv2: dz2 over rows (b, l) x 64 channels = the encoder part of d(X0)
        _check(lib.emlab_nn_act_grad(self._fp(up), ENC + AUX, 0, self._fp(self.z2), B, ENC, 1, self._fp(self.dz2),
                                     self._p(self.dz2b), s))
        self._gemm(64, 256, B * 16, self.dz2b, 1, 64, self.cols2, 1, 256, self.gW["conv2"], 256)
        _check(lib.emlab_nn_col_sum(self._fp(self.dz2), B * 16, 64, self._fp(self.gb["conv2"]), s))
        self._gemm(B * 16, 256, 64, self.dz2b, 64, 1, self.Wb["conv2"], 1, 256, self.dcols2, 256)
        _check(lib.emlab_nn_col2im(self._fp(self.dcols2), B, c2[6], c2[1], c2[3], c2[4], c2[5], c2[7],
                                   self._fp(self.da1), s))
        _check(lib.emlab_nn_act_grad(self._fp(self.da1), 32, 0, self._fp(self.z1), B * 64, 32, 1, self._fp(self.dz1),
                                     self._p(self.dz1b), s))
        self._gemm(32, 16, B * 64, self.dz1b, 1, 32, self.cols1, 1, 16, self.gW["conv1"], 16)
        _check(lib.emlab_nn_col_sum(self._fp(self.dz1), B * 64, 32, self._fp(self.gb["conv1"]), s))

    def step(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.t_step += 1
        for name, o, i in layer_shapes():
            _check(self.lib.emlab_nn_adam(self._fp(self.W[name]), self._fp(self.mW[name]), self._fp(self.vW[name]),
                                          self._fp(self.gW[name]), o * i, lr, b1, b2, eps, self.t_step,
                                          self._p(self.Wb[name]), self.stream))
            _check(self.lib.emlab_nn_adam(self._fp(self.b[name]), self._fp(self.mb[name]), self._fp(self.vb[name]),
                                          self._fp(self.gb[name]), o, lr, b1, b2, eps, self.t_step, None,
                                          self.stream))

    def status(self):
        _check(self.lib.emlab_nn_status(self.stream))

    def predict(self, x, zt):
        out = []
        for s in range(0, x.shape[0], self.B):
            self.load(x[s:s + self.B], zt[s:s + self.B])
            self.forward()
            out.append(self.y[: self.n].cpu().numpy())
        self.status()
        return np.concatenate(out) if out else np.zeros((0, OUT), np.float32)

    def params(self):
        return {n: (self.W[n].cpu().numpy(), self.b[n].cpu().numpy()) for n, _, _ in layer_shapes()}

    def grads(self):
        return {n: (self.gW[n].cpu().numpy(), self.gb[n].cpu().numpy()) for n, _, _ in layer_shapes()}


def _nn_lib():
    lib = load_library()
    if getattr(lib, "_nn_ready", False):
        return lib
    P, I, L, F = C.c_void_p, C.c_int, C.c_longlong, C.c_float
    fp = C.POINTER(C.c_float)
    sig = {
        "emlab_nn_gemm": [I, I, I, P, L, L, P, L, L, fp, L, P],
        "emlab_nn_status": [P],
        "emlab_nn_bias_act": [fp, fp, I, I, I, I, P, L, I, P],
        "emlab_nn_act_grad": [fp, L, I, fp, I, I, I, fp, P, P],
        "emlab_nn_col_sum": [fp, I, I, fp, P],
        "emlab_nn_im2col": [P, I, I, I, I, I, I, I, P, P],
        "emlab_nn_col2im": [fp, I, I, I, I, I, I, I, fp, P],
        "emlab_nn_mse": [fp, fp, L, fp, fp, P],
        "emlab_nn_adam": [fp, fp, fp, fp, L, F, F, F, F, I, P, P],
        "emlab_nn_to_bf16": [fp, L, P, L, I, I, P],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes, fn.restype = args, I
    lib._nn_ready = True
    return lib


# ---- data, training, evaluation --------------------------------------------------------------------
def train(x, zt, t, epochs=40, batch=256, lr=1e-3, seed=0, log=None):
    """Adam on the MSE of Z(f) / 100 ohm with a cosine learning-rate decay; returns (Net, per-epoch
    mean losses)."""
    net = Net(init_params(seed), batch=batch)
    rng = np.random.default_rng(seed)
    n = x.shape[0]
    losses = []
    for ep in range(epochs):
        order = rng.permutation(n)
        tot, cnt = 0.0, 0
        lr_ep = lr * 0.5 * (1.0 + math.cos(math.pi * ep / max(epochs, 1)))
        for s in range(0, n, batch):
            idx = order[s:s + batch]
            net.load(x[idx], zt[idx], t[idx])
            net.forward()
            net.backward()
            net.step(lr=lr_ep)
            tot += float(net.loss.item()) * len(idx)
            cnt += len(idx)
        net.status()
        losses.append(tot / max(cnt, 1))
        if log:
            log(f"epoch {ep}: loss {losses[-1]:.5f}")
    return net, losses


def rel_error(z_pred, z_ref):
    """|Z_pred - Z_ref| / |Z_ref| per frequency."""
    return np.abs(z_pred - z_ref) / np.maximum(np.abs(z_ref), 1e-9)


def s11_db(z, z0=50.0):
    g = np.abs((z - z0) / (z + z0))
    return 20.0 * np.log10(np.maximum(g, 1e-10))


def summary(z_pred, z_ref):
    """Per-scene median |dZ| / |Z| over the band, and |S11| dB error, summarised over scenes."""
    rel = np.median(rel_error(z_pred, z_ref), axis=1)
    ds11 = np.median(np.abs(s11_db(z_pred) - s11_db(z_ref)), axis=1)
    return {"dz_median": float(np.median(rel)), "dz_p90": float(np.percentile(rel, 90)),
            "within_2pct": float(np.mean(rel <= 0.02)), "s11_db_median": float(np.median(ds11)),
            "s11_db_p90": float(np.percentile(ds11, 90)), "scenes": int(rel.size)}


def far_errors(f_pred, f_ref):
    """Per-scene band medians of the far-field errors: |dD| (dB) and |d radiated energy| (dB)."""
    f_pred, f_ref = np.asarray(f_pred, np.float64), np.asarray(f_ref, np.float64)
    return np.median(np.abs(f_pred[:, 0] - f_ref[:, 0]), axis=1), np.median(np.abs(f_pred[:, 1] - f_ref[:, 1]), axis=1)


def far_summary(f_pred, f_ref):
    dd, dp = far_errors(f_pred, f_ref)
    return {"directivity_db_median": float(np.median(dd)), "directivity_db_p90": float(np.percentile(dd, 90)),
            "energy_db_median": float(np.median(dp)), "energy_db_p90": float(np.percentile(dp, 90)),
            "scenes": int(dd.size)}


def run_scenes(scenes, early: bool):
    """Steps scenes in stacks, each with its surface DFT: to ring-down (early False) or for their
    early window only; returns (results, wall seconds of the run, stack set-up excluded). The
    results hold the far-field spectra at the last step (result.far)."""
    from .batch import BatchRunner
    stop = [early_steps(sc) for sc in scenes] if early else None
    r = BatchRunner(scenes, chunk=64, stop_steps=stop, far_field=far_field())
    res = r.run()
    r.close()
    return res, r.wall_s


WAVE = 256  # scenes stepped together at most (device memory: stacks and their surface DFTs)


def record(sc, r):
    """What the extrapolator keeps of a run that rang down: the scene quantities features() reads,
    the whole (V, I) series with its converged Z(f), and the far-field spectra by step (the early
    windows and the last step); None for a run that did not ring down."""
    from types import SimpleNamespace as NS
    if not (r.done and r.rung_down and r.sweep is not None):
        return None
    series = np.ascontiguousarray(np.concatenate(r.series), np.float32)
    far = dict(getattr(r, "far", {}) or {})
    return NS(wavelength=sc.wavelength, grid=NS(courant=sc.grid.courant), sweep=dict(sc.sweep),
              cells=int(np.prod(sc.grid.size)),
              ports=[NS(impedance_ohm=sc.ports[0].impedance_ohm)],
              series=series, z=r.sweep["z"], far=far, far_final=far.get(series.shape[0]))


def generate(seed, n, edges, log=None, periods=None):
    """Runs scenes 0..n-1 of the generator's `seed` to ring-down with the batched solver, in waves,
    recording the far-field spectra at the end of each early window in `periods` (design periods)
    and at the last step; returns (records of the runs that rang down, wall seconds of stepping)."""
    from . import configs
    from .batch import BatchRunner
    periods = list(periods) if periods else [PERIODS_IN]
    recs, wall = [], 0.0
    for w0 in range(0, n, WAVE):
        scenes = [configs.batched_scene(seed, i, edges=edges) for i in range(w0, min(n, w0 + WAVE))]
        r = BatchRunner(scenes, chunk=64, far_field=far_field(),
                        snap_at=[[early_steps(sc, P) for P in periods] for sc in scenes])
        res = r.run()
        r.close()
        wall += r.wall_s
        recs += [q for q in (record(sc, x) for sc, x in zip(scenes, res)) if q is not None]
        if log:
            log(f"training runs {w0 + len(scenes)}/{n}: {r.wall_s:.1f} s")
    return recs, wall


def dataset_of(records):
    """(x, aux, t, z_trunc, z_conv, far_trunc, far_conv) of the records whose series and far-field
    snapshots cover the current early window."""
    rows = [[] for _ in range(7)]
    for q in records:
        n = early_steps(q)
        far_e = q.far.get(n)
        if q.series.shape[0] < n or far_e is None or q.far_final is None:
            continue
        x, zf, ztrunc = features(q, q.series, far_e)
        for k, v in enumerate((x, zf, target(q.z, q.far_final), ztrunc, q.z, far_e, q.far_final)):
            rows[k].append(v)
    if not rows[0]:
        return None
    return tuple(np.stack(r) for r in rows)


def ensemble_predict(nets, x, zt):
    """(mean Z(f) of the members, per-scene spread = band median of the largest member deviation
    |Z_m - Z_mean| / |Z_mean|, mean far-field spectra (n, 2, NFF)): the spread is the extrapolator's
    own estimate of its error."""
    ys = np.stack([n.predict(x, zt) for n in nets])
    zs = to_z(ys)
    zm = zs.mean(axis=0)
    dev = np.abs(zs - zm[None]).max(axis=0) / np.maximum(np.abs(zm), 1e-9)
    return zm, np.median(dev, axis=1), to_far(ys).mean(axis=0)


def per_scene_errors(z_pred, z_ref):
    """Per-scene band medians of |dZ| / |Z| and of the |S11| dB error."""
    return (np.median(rel_error(z_pred, z_ref), axis=1),
            np.median(np.abs(s11_db(z_pred) - s11_db(z_ref)), axis=1))


def select_threshold(spread, dz, ds11, dz_p90=0.02, s11_p90=0.5):
    """The largest spread threshold whose accepted scenes keep the p90 over ALL scenes of |dZ| at or
    below dz_p90 and of the S11 error at or below s11_p90, the rest falling back to the plain solver
    (error 0). Chosen on validation runs; -inf (every scene falls back) when no threshold qualifies."""
    best = -np.inf
    for tau in np.unique(spread):
        acc = spread <= tau
        if (np.percentile(np.where(acc, dz, 0.0), 90) <= dz_p90 and
                np.percentile(np.where(acc, ds11, 0.0), 90) <= s11_p90):
            best = float(tau)
    return best


def run_with_fallback(scenes, nets, tau):
    """The learned path with the plain solver as its fallback, in one batched run: at its early
    window each scene's ensemble prediction and spread are computed (one batched inference per stack
    and chunk); a spread within `tau` stops the scene there, otherwise it steps on from where it is
    to ring-down and its Z(f) and far-field spectra are the plain solver's. Returns ({scene: Z(f)},
    {scene: far-field spectra}, wall seconds including the inference, number of fallback scenes)."""
    from .batch import BatchRunner
    pred, pred_far = {}, {}

    def decide(idx, series, fars):
        xs, zts = [], []
        for i, ser, fe in zip(idx, series, fars):
            x, zf, _ = features(scenes[i], ser, fe)
            xs.append(x), zts.append(zf)
        zm, spread, fm = ensemble_predict(nets, np.stack(xs), np.stack(zts))
        for i, z, f in zip(idx, zm, fm):
            pred[i], pred_far[i] = z, f
        return [bool(v <= tau) for v in spread]

    r = BatchRunner(scenes, chunk=64, decide_at=[early_steps(sc) for sc in scenes], decide=decide,
                    far_field=far_field())
    res = r.run()
    r.close()
    z, far = {}, {}
    for i, q in enumerate(res):
        if q.accepted:
            z[i], far[i] = pred[i], pred_far[i]
        elif q.sweep is not None:
            z[i], far[i] = q.sweep["z"], q.far.get(q.steps)
    return z, far, r.wall_s, sum(1 for q in res if not q.accepted)


def experiment(train_seed, n_train, eval_seed, n_eval, epochs=60, batch=256, lr=1e-3, seed=0, edges=None, log=None,
               periods=None, members=1, val_frac=0.0, single=False):
    """Generates training runs with the batched solver (every scene to -60 dB ring-down, in waves of
    WAVE scenes, each with its surface DFT) and, for each early window in `periods` (design periods;
    default PERIODS_IN), trains `members` networks on them and evaluates on held-out scenes against
    the reference result, the plain solver run to ring-down:
      (a) the plain solver: batched stacks (and with `single`, one SimulationGrid per scene, the
          reference's way) — sweeps/hr, the converged Z(f) and far-field spectra;
      (b) the early window's truncated DFTs (the method without the network);
      (c) the network's prediction (the ensemble mean) from the same early window;
      (d) with members > 1 and val_frac > 0, the learned path with its fallback: scenes whose
          ensemble spread exceeds a threshold chosen on a validation split of the training runs
          (p90 |dZ| <= 2 % and p90 S11 error <= 0.5 dB over all validation scenes) continue with
          the plain solver, and their Z(f) and spectra are the plain solver's.
    Sweeps/hr are wall-clock figures of stepping, read-back, far-field evaluation, features and
    inference (stack set-up excluded). Returns (result dict, parameters of the first member of the
    last window)."""
    from . import batch as batch_solver, configs
    global PERIODS_IN
    edges = edges or configs.BATCH_EDGES
    periods = list(periods) if periods else [PERIODS_IN]
    out = {}
    t0 = time.perf_counter()
    recs, tr_wall = generate(train_seed, n_train, edges, log, periods)
    out["train_runs"] = {"scenes": n_train, "usable": len(recs), "wall_s": tr_wall}
    n_val = int(round(val_frac * len(recs))) if members > 1 else 0
    val_recs, fit_recs = recs[:n_val], recs[n_val:]

    eval_scenes = [configs.batched_scene(eval_seed, i, edges=edges) for i in range(n_eval)]
    ev_res, plain_wall = run_scenes(eval_scenes, early=False)
    out["plain"] = {"batched_s": plain_wall, "sweeps_per_hour": n_eval / plain_wall * 3600.0,
                    "steps_median": float(np.median([r.steps for r in ev_res]))}
    if single:
        run_s = 0.0
        ff = far_field()
        for sc in eval_scenes:
            tm = {}
            batch_solver.run_single(sc, chunk=64, timing=tm, far_field=ff)
            run_s += tm["run_s"]
        out["plain"].update(single_s=run_s, single_sweeps_per_hour=n_eval / run_s * 3600.0)

    windows, params = {}, None
    saved = PERIODS_IN
    try:
        for P in periods:
            PERIODS_IN = float(P)
            w = {"periods": float(P)}
            x, zt, t = dataset_of(fit_recs)[:3]
            t1 = time.perf_counter()
            nets, last = [], []
            for m in range(members):
                net, losses = train(x, zt, t, epochs=epochs, batch=batch, lr=lr, seed=seed + m, log=log)
                nets.append(net)
                last.append(losses[-1])
            w["training"] = {"epochs": epochs, "samples": int(x.shape[0]), "members": members,
                             "loss_last": last, "wall_s": time.perf_counter() - t1}
            params = nets[0].params()
            tau = None
            if n_val:
                vx, vzt, _, _, vz, _, vfar = dataset_of(val_recs)
                vzm, vspread, vfm = ensemble_predict(nets, vx, vzt)
                vdz, vds = per_scene_errors(vzm, vz)
                tau = select_threshold(vspread, vdz, vds)
                # cell-steps of the learned path with fallback relative to the plain runs (a rejected
                # scene runs on from its early window)
                usable = [q for q in val_recs if q.series.shape[0] >= early_steps(q) and early_steps(q) in q.far
                          and q.far_final is not None]
                full = np.array([q.cells * q.series.shape[0] for q in usable], np.float64)
                early = np.array([q.cells * early_steps(q) for q in usable], np.float64)
                cost = float(np.where(vspread > tau, full, early).sum() / full.sum())
                w["validation"] = {"scenes": int(vx.shape[0]), "threshold": tau,
                                   "accepted": float(np.mean(vspread <= tau)), "cell_steps_vs_plain": cost,
                                   "network_dz_median": float(np.median(vdz)),
                                   "network_s11_db_median": float(np.median(vds)),
                                   "network_far": far_summary(vfm, vfar)}
            # the learned path on the held-out scenes: early window (with its surface DFT), features,
            # inference
            early_res, early_wall = run_scenes(eval_scenes, early=True)
            t2 = time.perf_counter()
            xs, zts, ztr, ftr, keep = [], [], [], [], []
            for k, (sc, r) in enumerate(zip(eval_scenes, early_res)):
                ser = np.concatenate(r.series)
                fe = r.far.get(early_steps(sc))
                if ser.shape[0] < early_steps(sc) or fe is None:
                    continue
                xe, ze, zr = features(sc, ser, fe)
                xs.append(xe), zts.append(ze), ztr.append(zr), ftr.append(fe), keep.append(k)
            z_pred, _, f_pred = ensemble_predict(nets, np.stack(xs), np.stack(zts))
            infer_wall = time.perf_counter() - t2
            # the learned path with its fallback, in one run: every scene is stopped at its early
            # window if the ensemble's spread is within the threshold, else it runs on to ring-down
            fb_wall, n_fallback, z_hyb_of, f_hyb_of = 0.0, 0, {}, {}
            if tau is not None:
                z_hyb_of, f_hyb_of, fb_wall, n_fallback = run_with_fallback(eval_scenes, nets, tau)
            learned_wall = (early_wall + infer_wall) if tau is None else fb_wall
            z_trunc, f_trunc = np.stack(ztr), np.stack(ftr)
            ok = [j for j, k in enumerate(keep) if ev_res[k].rung_down]
            z_conv = np.stack([ev_res[keep[j]].sweep["z"] for j in ok])
            f_conv = np.stack([ev_res[keep[j]].far[ev_res[keep[j]].steps] for j in ok])
            w["eval"] = {"scenes": n_eval, "compared": len(ok), "network": summary(z_pred[ok], z_conv),
                         "truncated_dft": summary(z_trunc[ok], z_conv),
                         "network_far": far_summary(f_pred[ok], f_conv),
                         "truncated_dft_far": far_summary(f_trunc[ok], f_conv)}
            if tau is not None:
                z_hyb = np.stack([z_hyb_of[keep[j]] for j in ok])
                f_hyb = np.stack([f_hyb_of[keep[j]] for j in ok])
                w["eval"]["with_fallback"] = summary(z_hyb, z_conv)
                w["eval"]["with_fallback_far"] = far_summary(f_hyb, f_conv)
                w["eval"]["fallback_scenes"] = n_fallback
            w["wall"] = {"early_s": early_wall, "features_inference_s": infer_wall, "with_fallback_s": fb_wall}
            net_wall = early_wall + infer_wall  # every scene stops at the early window
            w["network_only"] = {"sweeps_per_hour": n_eval / net_wall * 3600.0,
                                 "speedup_vs_batched_plain": plain_wall / net_wall}
            if single:
                w["network_only"]["speedup_vs_single_plain"] = out["plain"]["single_s"] / net_wall
            w["sweeps_per_hour"] = n_eval / learned_wall * 3600.0
            w["speedup_vs_batched_plain"] = plain_wall / learned_wall
            if single:
                w["speedup_vs_single_plain"] = out["plain"]["single_s"] / learned_wall
            w["early_steps_median"] = float(np.median([early_steps(sc) for sc in eval_scenes]))
            windows[f"{P:g}"] = w
            if log:
                log(f"window {P:g} periods: {json_safe(w)}")
    finally:
        PERIODS_IN = saved
    out["windows"] = windows
    # the chosen window's figures at the top level: the lowest validation cost with a fallback,
    # otherwise the first window
    costs = {k: w["validation"]["cell_steps_vs_plain"] for k, w in windows.items() if "validation" in w}
    chosen = min(costs, key=costs.get) if costs else f"{periods[0]:g}"
    out["chosen_window"] = chosen
    # the network alone: the shortest window whose validation medians meet |dZ| <= 2 % and S11 <= 0.5 dB
    fit = [k for k, w in windows.items() if "validation" in w and w["validation"]["network_dz_median"] <= 0.02
           and w["validation"]["network_s11_db_median"] <= 0.5]
    out["chosen_window_network_only"] = min(fit, key=lambda k: windows[k]["periods"]) if fit else None
    w0 = windows[chosen]
    out["eval"] = w0["eval"]
    out["training"] = w0["training"]
    out["sweeps_per_hour"] = {"plain": out["plain"]["sweeps_per_hour"], "learned": w0["sweeps_per_hour"]}
    out["speedup"] = w0["speedup_vs_batched_plain"]
    out["wall"] = dict(w0["wall"], plain_s=plain_wall)
    out["steps"] = {"plain_median": out["plain"]["steps_median"], "early_median": w0["early_steps_median"]}
    out["wall_s"] = time.perf_counter() - t0
    return out, params


def json_safe(d):
    """A compact one-line rendering of a result dict for the log."""
    import json
    return json.dumps(d, default=float)[:600]
