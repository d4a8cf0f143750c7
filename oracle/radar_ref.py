"""CPU restatement of the radar back-projection (test infrastructure).

Follows src/Radar.cpp:606-646 (RadarMonitor::computeImage's imaging loop) and :87-103 (txDelay):
FP32 geometry, FP64 sums, in the reference's operation order. Only the tests import this module.
"""
from __future__ import annotations

import math

import numpy as np

f32 = np.float32


def _len(v):
    return f32(math.sqrt(float(f32(f32(v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]))))


def tx_delay(p, tx, ax2, tx_pos, tx_amp, w):
    ar = ad = 0j
    mag = 0.0
    for j in range(len(tx_amp)):
        v = (p - tx_pos[j]).astype(f32)
        d = max(float(_len(v)), 0.5)
        g = max(float(f32(f32(v[0] * ax2[0] + v[1] * ax2[1]) + v[2] * ax2[2])) / d, 0.0)
        term = (tx_amp[j] * g / d) * complex(math.cos(-w * d), math.sin(-w * d))
        ar += term
        ad += d * term
        mag += tx_amp[j] * g / d
    if abs(ar) < 1e-3 * mag:
        return float(_len((p - tx).astype(f32)))
    return (ad / ar).real


def backproject(geo, z, elem_pos, weights, tx_pos, tx_amp):
    """power (nr, nel, naz) for an abi.RadarGeometry and complex64 z (M, C)."""
    tx = np.asarray(geo.tx[:], f32)
    ax = np.asarray(geo.axes[:], f32).reshape(3, 3)
    lo, hi = np.asarray(geo.interior_min[:], f32), np.asarray(geo.interior_max[:], f32)
    M, C = z.shape
    out = np.zeros((geo.nr, geo.nel, geo.naz))
    w, dt, sdt = geo.omega, geo.dt, geo.sample_dt
    for ie in range(geo.nel):
        for ia in range(geo.naz):
            az = f32(geo.az0) + f32(ia) * f32(geo.daz)
            el = f32(geo.el0) + f32(ie) * f32(geo.del_)
            a, e = f32(az * f32(0.017453292519943295)), f32(el * f32(0.017453292519943295))
            sa, ca, se, ce = f32(math.sin(a)), f32(math.cos(a)), f32(math.sin(e)), f32(math.cos(e))
            d = ((ax[0] * f32(sa * ce) + ax[1] * se) + ax[2] * f32(ca * ce)).astype(f32)
            for ir in range(geo.nr):
                r = f32(geo.r0) + f32(ir) * f32(geo.dr)
                P = (tx + d * r).astype(f32)
                if np.any(P < lo) or np.any(P > hi):
                    out[ir, ie, ia] = -1.0
                    continue
                ob = tx_delay(P, tx, ax[2], tx_pos, tx_amp, w)
                s_ = 0j
                for i in range(C):
                    t = ob + float(_len((P - elem_pos[i]).astype(f32)))
                    s = (t + 0.5 * dt) / sdt
                    if s < 0.0 or s >= M - 1:
                        continue
                    m0 = int(s)
                    f = f32(s - m0)
                    v = z[m0, i] * (f32(1.0) - f) + z[m0 + 1, i] * f
                    s_ += weights[i] * complex(v) * complex(math.cos(w * t), math.sin(w * t))
                out[ir, ie, ia] = s_.real * s_.real + s_.imag * s_.imag
    return out


def random_case(seed, nr=40):
    """A seeded back-projection problem: (geometry, wavelength, z (M, C) complex64, element
    positions, weights, transmit positions, transmit amplitudes). Ranges reach 10 + 2 (nr - 1)
    cells from the transmit centre, so with the default nr the far bins leave the volume."""
    from em_lab_gb300 import abi
    rng = np.random.default_rng(seed)
    C, M = 9, 60
    g = abi.RadarGeometry()
    tx = np.array([20.3, 40.1, 39.7], f32)
    for k in range(3):
        g.tx[k] = float(tx[k])
        g.interior_min[k] = 5.0
        g.interior_max[k] = 90.0
    for k, v in enumerate([0, -1, 0, 0, 0, 1, 1, 0, 0]):  # right, up, boresight (+x)
        g.axes[k] = float(v)
    wl = 16.0
    g.omega, g.dt, g.sample_dt = 2 * math.pi / wl, 0.5, 2.0
    g.r0, g.dr, g.az0, g.daz, g.el0, g.del_ = 10.0, 2.0, -12.0, 3.0, -9.0, 3.0
    g.nr, g.naz, g.nel = nr, 9, 7
    z = (rng.standard_normal((M, C)) + 1j * rng.standard_normal((M, C))).astype(np.complex64)
    ep = (tx + rng.uniform(-6, 6, (C, 3))).astype(f32)
    w = rng.uniform(0.3, 1.0, C)
    tp = (tx + rng.uniform(-2, 2, (3, 3))).astype(f32)
    ta = rng.uniform(0.5, 1.5, 3)
    return g, wl, z, ep, w, tp, ta
