// radar.cu - back-projection imaging of the pulsed phased-array radar (src/Radar.cpp:606-646).
//
// For every image point P = tx + r * direction(az, el) inside the simulated volume, the complex
// baseband echoes z_i of all receive elements are sampled at the point's round-trip delay
// (transmit group delay of the near-field array factor, Radar.cpp:87-103, plus the distance back to
// element i), interpolated linearly between decimated samples, weighted by the receive taper and
// re-phased to the carrier: power = |sum_i w_i z_i(t_i) e^{j w t_i}|^2. One thread per image point;
// geometry in FP32 and the sums in FP64 as the reference computes them (compiled without
// contraction). The reference spreads elevation rows over CPU threads; here the whole
// range x elevation x azimuth volume is one launch.
#include <cuda_runtime.h>

#include "../../include/emlab.h"
#include "emlab_internal.h"

namespace emlab {
namespace {

struct F3 {
    float x, y, z;
};
__device__ __forceinline__ F3 f3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ F3 sub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 add(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ F3 mul(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float len(F3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ F3 ld3(const float* p) { return {p[0], p[1], p[2]}; }

struct Geo {
    F3 tx, ax0, ax1, ax2, lo, hi;
};

// RadarMonitor::txDelay (Radar.cpp:87-103)
__device__ double tx_delay(const Geo& g, F3 p, const float* tx_pos, const double* tx_amp, int ntx, double w) {
    double ar = 0.0, ai = 0.0, adr = 0.0, adi = 0.0, mag = 0.0;
    for (int j = 0; j < ntx; ++j) {
        const F3 v = sub(p, ld3(tx_pos + 3 * j));
        const double d = fmax((double)len(v), 0.5);
        const double gj = fmax((double)dot(v, g.ax2) / d, 0.0);
        const double a = tx_amp[j] * gj / d;
        double s, c;
        sincos(-w * d, &s, &c);
        const double tr = a * c, ti = a * s;
        ar += tr, ai += ti;
        adr += d * tr, adi += d * ti;
        mag += tx_amp[j] * gj / d;
    }
    const double absa = sqrt(ar * ar + ai * ai);
    if (absa < 1e-3 * mag) return (double)len(sub(p, g.tx));
    // real(ad / a)
    return (adr * ar + adi * ai) / (ar * ar + ai * ai);
}

__global__ void backproject_kernel(emlab_radar_geometry geo, const float2* z, int M, int C, const float* elem_pos,
                                   const double* weights, const float* tx_pos, const double* tx_amp, int ntx,
                                   double* power) {
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = (long long)geo.nr * geo.nel * geo.naz;
    if (idx >= total) return;
    const int ia = (int)(idx % geo.naz);
    const int ie = (int)((idx / geo.naz) % geo.nel);
    const int ir = (int)(idx / ((long long)geo.naz * geo.nel));
    Geo g;
    g.tx = ld3(geo.tx), g.ax0 = ld3(geo.axes), g.ax1 = ld3(geo.axes + 3), g.ax2 = ld3(geo.axes + 6);
    g.lo = ld3(geo.interior_min), g.hi = ld3(geo.interior_max);
    // RadarMonitor::direction (Radar.cpp:69-72)
    const float az = geo.az0 + (float)ia * geo.daz, el = geo.el0 + (float)ie * geo.del;
    const float a = az * 0.01745329251994329577f, e = el * 0.01745329251994329577f;
    const float sa = sinf(a), ca = cosf(a), se = sinf(e), ce = cosf(e);
    const F3 dir = add(add(mul(g.ax0, sa * ce), mul(g.ax1, se)), mul(g.ax2, ca * ce));
    const float r = geo.r0 + (float)ir * geo.dr;
    const F3 P = add(g.tx, mul(dir, r));
    if (P.x < g.lo.x || P.y < g.lo.y || P.z < g.lo.z || P.x > g.hi.x || P.y > g.hi.y || P.z > g.hi.z) {
        power[idx] = -1.0;  // outside the simulated volume
        return;
    }
    const double w = geo.omega, dt = geo.dt, sdt = geo.sample_dt;
    const double outbound = tx_delay(g, P, tx_pos, tx_amp, ntx, w);
    double sr = 0.0, si = 0.0;
    for (int i = 0; i < C; ++i) {
        const double t = outbound + (double)len(sub(P, ld3(elem_pos + 3 * i)));  // path delay
        const double s = (t + 0.5 * dt) / sdt;                                       // decimated sample
        if (s < 0.0 || s >= (double)(M - 1)) continue;
        const int m0 = (int)s;
        const float f = (float)(s - (double)m0);
        const float2 z0 = z[(long long)m0 * C + i], z1 = z[(long long)(m0 + 1) * C + i];
        const float vr = z0.x * (1.0f - f) + z1.x * f, vi = z0.y * (1.0f - f) + z1.y * f;
        double sn, cs;
        sincos(w * t, &sn, &cs);
        const double wr = weights[i] * (double)vr, wi = weights[i] * (double)vi;
        sr += wr * cs - wi * sn;
        si += wr * sn + wi * cs;
    }
    power[idx] = sr * sr + si * si;
}

}  // namespace
}  // namespace emlab

using namespace emlab;

extern "C" int emlab_radar_backproject(const emlab_radar_geometry* geo, const float* z, int M, int C,
                                       const float* elem_pos, const double* weights, const float* tx_pos,
                                       const double* tx_amp, int ntx, double* power) {
    if (!geo || !z || !elem_pos || !weights || !tx_pos || !tx_amp || !power || M < 2 || C < 1 || ntx < 1 ||
        geo->nr < 1 || geo->naz < 1 || geo->nel < 1)
        return report_error(EMLAB_ERR_INVALID, "bad radar back-projection arguments");
    const long long total = (long long)geo->nr * geo->nel * geo->naz;
    if (total > (1ll << 31)) return report_error(EMLAB_ERR_INVALID, "radar image too large");
    float2* dz = nullptr;
    float *de = nullptr, *dt = nullptr;
    double *dw = nullptr, *da = nullptr, *dp = nullptr;
    auto release = [&]() {
        cudaFree(dz), cudaFree(de), cudaFree(dt), cudaFree(dw), cudaFree(da), cudaFree(dp);
    };
    const size_t zb = (size_t)M * C * 8;
    if (cudaMalloc(&dz, zb) != cudaSuccess || cudaMalloc(&de, (size_t)C * 12) != cudaSuccess ||
        cudaMalloc(&dt, (size_t)ntx * 12) != cudaSuccess || cudaMalloc(&dw, (size_t)C * 8) != cudaSuccess ||
        cudaMalloc(&da, (size_t)ntx * 8) != cudaSuccess || cudaMalloc(&dp, (size_t)total * 8) != cudaSuccess) {
        release();
        return report_error(EMLAB_ERR_OOM, "radar: device allocation failed");
    }
    cudaError_t e = cudaMemcpy(dz, z, zb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(de, elem_pos, (size_t)C * 12, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dt, tx_pos, (size_t)ntx * 12, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dw, weights, (size_t)C * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(da, tx_amp, (size_t)ntx * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        backproject_kernel<<<(unsigned)((total + 127) / 128), 128>>>(*geo, dz, M, C, de, dw, dt, da, ntx, dp);
        count_launches(1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(power, dp, (size_t)total * 8, cudaMemcpyDeviceToHost);
    release();
    if (e != cudaSuccess) return report_error(EMLAB_ERR_CUDA, cudaGetErrorString(e));
    return EMLAB_OK;
}
