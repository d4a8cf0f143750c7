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
