// yee_common.cuh - the per-cell Yee arithmetic shared by every solver kernel.
//
// Follows shaders/update_B.comp:35-67 and shaders/update_E.comp:41-64 operation for operation
// (compile with -fmad=false). Inside the absorber the coefficient pair
// (e^{-x}, dt * phi(x)), x = sigma * dt, depends only on the three per-axis depth classes of the
// sample position; it is read from a host-built K^3 table whose entries are computed with the very
// same float operations (common.glsl:23-36, 50-54), so the values are bit-identical to evaluating
// exp() in the kernel. The table serves every B component and the E components of vacuum cells
// (class 0); E components of other materials inside the absorber evaluate exp() on the device.
#pragma once

#include "emlab_internal.h"

namespace emlab {

__device__ __forceinline__ bool in_pml(const YeeArgs& a, int x, int y, int z) {
    // common.glsl:40-43 (the z test is a per-plane table: a stack of scenes has one layer per scene face)
    return x < a.L || y < a.L || x >= a.nx - (a.L + 1) || y >= a.ny - (a.L + 1) || __ldg(a.pml_z + z) != 0;
}

template <typename Idx>
__device__ __forceinline__ unsigned load_class(const YeeArgs& a, long long i) {
    return (unsigned)__ldg(static_cast<const Idx*>(a.cls) + i);
}

// Depth classes of (x, y, z) on the integer (I) and half-integer (H) lattices, per axis.
struct PmlIdx {
    int ix, iy, iz, hx, hy, hz;
};

__device__ __forceinline__ PmlIdx pml_idx(const YeeArgs& a, int x, int y, int z) {
    const int S = a.pml_stride;
    const unsigned char* c = a.pml_cls;
    return {__ldg(c + x), __ldg(c + S + y), __ldg(c + 2 * S + z), __ldg(c + 3 * S + x), __ldg(c + 4 * S + y),
            __ldg(c + 5 * S + z)};
}

__device__ __forceinline__ float2 pml_coef(const YeeArgs& a, int i, int j, int k) {
    return __ldg(a.pml_coef + (i * a.pml_K + j) * a.pml_K + k);
}

// E update inside the absorber for a non-vacuum edge material (update_E.comp:51-64).
__device__ __forceinline__ float e_pml(float e, float curl, float sigma, float eps, float dt) {
    const float dtEps = dt / eps;
    const float x = sigma * dtEps;
    return emlab_expf(-x) * e + (dtEps * emlab_phi(x)) * curl;
}

// B^{n+1/2} at cell (x,y,z) from E^n at the cell and at +x, +y, +z (update_B.comp:35-67).
__device__ __forceinline__ void b_cell(const YeeArgs& a, float& bx, float& by, float& bz, float e0x, float e0y,
                                       float e0z, float exy, float exz, float eyx, float eyz, float ezx, float ezy,
                                       unsigned c, int x, int y, int z) {
    float t0x = eyz - e0z, t0y = ezx - e0x, t0z = exy - e0y;
    float t1x = ezy - e0y, t1y = exz - e0z, t1z = eyx - e0x;
    if (c >= a.wire_start) {
        const float4 w0 = __ldg(a.tabW + 2 * c), w1 = __ldg(a.tabW + 2 * c + 1);
        t0x = t0x * w0.x, t0y = t0y * w0.y, t0z = t0z * w0.z;
        t1x = t1x * w0.w, t1y = t1y * w1.x, t1z = t1z * w1.y;
    }
    const float cx = t0x - t1x, cy = t0y - t1y, cz = t0z - t1z;
    if (in_pml(a, x, y, z)) {
        // sigma_m at (x, y+1/2, z+1/2), (x+1/2, y, z+1/2), (x+1/2, y+1/2, z)
        const PmlIdx p = pml_idx(a, x, y, z);
        const float2 kx = pml_coef(a, p.ix, p.hy, p.hz), ky = pml_coef(a, p.hx, p.iy, p.hz),
                     kz = pml_coef(a, p.hx, p.hy, p.iz);
        bx = kx.x * bx - kx.y * cx;
        by = ky.x * by - ky.y * cy;
        bz = kz.x * bz - kz.y * cz;
    } else {
        const float dt = a.dt;
        bx = bx - dt * cx;
        by = by - dt * cy;
        bz = bz - dt * cz;
    }
}

// E^{n+1} at cell (x,y,z) from curl B^{n+1/2} (update_E.comp:41-64).
__device__ __forceinline__ void e_cell(const YeeArgs& a, float& ex, float& ey, float& ez, float cx, float cy, float cz,
                                       unsigned c, int x, int y, int z) {
    if (!in_pml(a, x, y, z)) {
        const float4 t0 = __ldg(a.tabE + 2 * c), t1 = __ldg(a.tabE + 2 * c + 1);
        ex = t0.x * ex + t0.w * cx;
        ey = t0.y * ey + t1.x * cy;
        ez = t0.z * ez + t1.y * cz;
    } else if (c == 0) {
        // sigma at (x+1/2, y, z), (x, y+1/2, z), (x, y, z+1/2) on vacuum edges
        const PmlIdx p = pml_idx(a, x, y, z);
        const float2 kx = pml_coef(a, p.hx, p.iy, p.iz), ky = pml_coef(a, p.ix, p.hy, p.iz),
                     kz = pml_coef(a, p.ix, p.iy, p.hz);
        ex = kx.x * ex + kx.y * cx;
        ey = ky.x * ey + ky.y * cy;
        ez = kz.x * ez + kz.y * cz;
    } else {
        const float4 m0 = __ldg(a.tabM + 2 * c), m1 = __ldg(a.tabM + 2 * c + 1);
        const int S = a.pml_stride;
        const float ix = __ldg(a.pml + x), iy = __ldg(a.pml + S + y), iz = __ldg(a.pml + 2 * S + z);
        const float hx = __ldg(a.pml + 3 * S + x), hy = __ldg(a.pml + 4 * S + y), hz = __ldg(a.pml + 5 * S + z);
        ex = e_pml(ex, cx, m0.x + ((hx + iy) + iz), m0.w, a.dt);
        ey = e_pml(ey, cy, m0.y + ((ix + hy) + iz), m1.x, a.dt);
        ez = e_pml(ez, cz, m0.z + ((ix + iy) + hz), m1.y, a.dt);
    }
}

}  // namespace emlab
