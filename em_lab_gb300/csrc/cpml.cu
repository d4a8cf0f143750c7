// cpml.cu - the opt-in convolutional PML (no counterpart in the reference).
//
// The reference absorbs outgoing waves with a graded conductivity and a matched magnetic loss
// (shaders/common.glsl:15-43, update_E.comp:51-61, update_B.comp:58-66); that stays the default and
// the parity path. emlab_grid_set_cpml replaces it with a convolutional PML with a
// complex-frequency-shifted stretch (Roden & Gedney 2000): inside the absorber slabs every spatial
// derivative dF of the curl along an axis a becomes dF / kappa_a + psi, with the auxiliary field
// psi <- b_a psi + c_a dF kept per cell and per (component, axis) pair. Coefficients b, c, 1/kappa
// depend on the position along one axis only (emlab_cpml_coef) and live in per-axis tables for
// the integer positions (the E update's backward differences) and the half-integer positions (the B
// update's forward differences). The reference absorber's conductivity is switched off (its tables
// are built with sigma_max 0, which leaves the plain update bit for bit), so the materials' own
// (ca, cb) and thin-wire factors apply everywhere.
//
// psi storage: only the slabs, L + 1 cells at each end of the axis the derivative runs along
// (S = 2 (L + 1) positions per axis), four FP32 arrays per axis: the two E components and the two
// B components whose curl differentiates along it. Array slot j of axis a: 0 = E component
// (a+2)%3 (its term0 = d_a F), 1 = E component (a+1)%3 (its term1 = d_a F), 2 and 3 the same for
// B. Layout per axis (s = slab position): x: ((z ny + y) S + s), y: ((z S + s) nx + x),
// z: ((s ny + y) nx + x), so consecutive threads (consecutive x) touch consecutive entries except
// along x.
//
// The step runs as two in-place passes over the current field generation, B then E (the
// reference's pass order, SimulationGrid.cpp:394-410), followed by the ordinary source pass.
// Bandwidth: E and B read and written, the class index, plus the psi of slab cells; this is a
// correctness path, not the tuned stencil.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "emlab_internal.h"
#include "emlab_math.h"
#include "grid_state.h"

namespace emlab {

namespace {

struct CpmlArgs {
    const float4* coef;  // [lattice: 0 integer, 1 half][axis][stride]: (b, c, 1/kappa, 0)
    int stride;
    int L1;              // slab positions per side: L + 1
    float* psi[3];       // per derivative axis: 4 arrays of slab[axis] entries
    long long slab[3];
};

__device__ __forceinline__ int slab_pos(int i, int n, int L1) {
    return i < L1 ? i : (i >= n - L1 ? i - n + 2 * L1 : -1);
}

// dF / kappa + psi at (x, y, z) for the derivative along `axis` of the component in psi slot
// `slot`, updating psi; the plain dF outside the slabs.
__device__ __forceinline__ float cpml_term(const CpmlArgs& p, const YeeArgs& a, int lattice, int axis, int slot, int x,
                                           int y, int z, float d) {
    const int i = axis == 0 ? x : (axis == 1 ? y : z);
    const int n = axis == 0 ? a.nx : (axis == 1 ? a.ny : a.nz);
    const int s = slab_pos(i, n, p.L1);
    if (s < 0) return d;
    const int S = 2 * p.L1;
    const long long at = axis == 0 ? ((long long)z * a.ny + y) * S + s
                                   : (axis == 1 ? ((long long)z * S + s) * a.nx + x : ((long long)s * a.ny + y) * a.nx + x);
    float* psi = p.psi[axis] + (long long)slot * p.slab[axis] + at;
    const float4 k = __ldg(p.coef + (lattice * 3 + axis) * p.stride + i);
    const float v = k.x * *psi + k.y * d;
    *psi = v;
    return d * k.z + v;
}

// B^{n+1/2} = B^{n-1/2} - dt curl E^n with the stretched derivatives (forward differences at the
// half-integer positions; E beyond the upper faces is 0 as in update_B.comp:27-29).
template <typename Idx>
__global__ void __launch_bounds__(128) cpml_b_kernel(YeeArgs a, CpmlArgs p) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= a.nx) return;
    const long long o = (long long)z * a.plane + (long long)y * a.pitch + x;
    const float e0x = a.wex[o], e0y = a.wey[o], e0z = a.wez[o];
    const bool xp = x + 1 < a.nx, yp = y + 1 < a.ny, zp = z + 1 < a.nz;
    const float ey_x = xp ? a.wey[o + 1] : 0.0f, ez_x = xp ? a.wez[o + 1] : 0.0f;
    const float ex_y = yp ? a.wex[o + a.pitch] : 0.0f, ez_y = yp ? a.wez[o + a.pitch] : 0.0f;
    const float ex_z = zp ? a.wex[o + a.plane] : 0.0f, ey_z = zp ? a.wey[o + a.plane] : 0.0f;
    // curl_c E = term0 - term1, term0 = d_{c+1} E_{c+2}, term1 = d_{c+2} E_{c+1}
    float t0[3] = {ez_y - e0z, ex_z - e0x, ey_x - e0y};
    float t1[3] = {ey_z - e0y, ez_x - e0z, ex_y - e0x};
    const unsigned c = (unsigned)__ldg(static_cast<const Idx*>(a.cls) + o);
    if (c >= a.wire_start) {
        const float4 w0 = __ldg(a.tabW + 2 * c), w1 = __ldg(a.tabW + 2 * c + 1);
        t0[0] = t0[0] * w0.x, t0[1] = t0[1] * w0.y, t0[2] = t0[2] * w0.z;
        t1[0] = t1[0] * w0.w, t1[1] = t1[1] * w1.x, t1[2] = t1[2] * w1.y;
    }
    float* const B[3] = {a.wbx, a.wby, a.wbz};
    const float dt = a.dt;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int a0 = (k + 1) % 3, a1 = (k + 2) % 3;
        const float u0 = cpml_term(p, a, 1, a0, 2, x, y, z, t0[k]);
        const float u1 = cpml_term(p, a, 1, a1, 3, x, y, z, t1[k]);
        const float curl = u0 - u1;
        B[k][o] = B[k][o] - dt * curl;
    }
}

// E^{n+1} = ca E^n + cb curl B^{n+1/2} with the stretched derivatives (backward differences at the
// integer positions; B below the lower faces is 0 as in update_E.comp:27-29); (ca, cb) of the edge
// material (no absorber conductivity).
template <typename Idx>
__global__ void __launch_bounds__(128) cpml_e_kernel(YeeArgs a, CpmlArgs p) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= a.nx) return;
    const long long o = (long long)z * a.plane + (long long)y * a.pitch + x;
    const float b0x = a.wbx[o], b0y = a.wby[o], b0z = a.wbz[o];
    const bool xm = x > 0, ym = y > 0, zm = z > 0;
    const float by_x = xm ? a.wby[o - 1] : 0.0f, bz_x = xm ? a.wbz[o - 1] : 0.0f;
    const float bx_y = ym ? a.wbx[o - a.pitch] : 0.0f, bz_y = ym ? a.wbz[o - a.pitch] : 0.0f;
    const float bx_z = zm ? a.wbx[o - a.plane] : 0.0f, by_z = zm ? a.wby[o - a.plane] : 0.0f;
    // curl_c B = term0 - term1, term0 = d_{c+1} B_{c+2}, term1 = d_{c+2} B_{c+1}
    const float t0[3] = {b0z - bz_y, b0x - bx_z, b0y - by_x};
    const float t1[3] = {b0y - by_z, b0z - bz_x, b0x - bx_y};
    const unsigned c = (unsigned)__ldg(static_cast<const Idx*>(a.cls) + o);
    const float4 m0 = __ldg(a.tabE + 2 * c), m1 = __ldg(a.tabE + 2 * c + 1);
    const float ca[3] = {m0.x, m0.y, m0.z}, cb[3] = {m0.w, m1.x, m1.y};
    float* const E[3] = {a.wex, a.wey, a.wez};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int a0 = (k + 1) % 3, a1 = (k + 2) % 3;
        const float u0 = cpml_term(p, a, 0, a0, 0, x, y, z, t0[k]);
        const float u1 = cpml_term(p, a, 0, a1, 1, x, y, z, t1[k]);
        const float curl = u0 - u1;
        E[k][o] = ca[k] * E[k][o] + cb[k] * curl;
    }
}

CpmlArgs cpml_args(emlab_grid* g) {
    CpmlArgs p{};
    p.coef = g->cpml_coef.p;
    p.stride = g->cpml_stride;
    p.L1 = g->cfg.pml_thickness + 1;
    for (int ax = 0; ax < 3; ++ax) {
        p.slab[ax] = g->cpml_slab[ax];
        p.psi[ax] = g->cpml_psi.p + g->cpml_psi_off[ax];
    }
    return p;
}

}  // namespace

int cpml_prepare(emlab_grid* g) {
    const emlab_grid_config& c = g->cfg;
    const int n[3] = {c.nx, c.ny, c.nz};
    const int L = c.pml_thickness, L1 = L + 1, S = 2 * L1;
    const int stride = std::max(c.nx, std::max(c.ny, c.nz));
    std::vector<float4> coef((size_t)2 * 3 * stride, make_float4(1.0f, 0.0f, 1.0f, 0.0f));
    for (int lat = 0; lat < 2; ++lat)
        for (int ax = 0; ax < 3; ++ax)
            for (int i = 0; i < n[ax]; ++i) {
                float k[3];
                emlab_cpml_coef((double)i + (lat ? 0.5 : 0.0), n[ax], L, g->cpml.sigma_max, g->cpml.kappa_max,
                                g->cpml.alpha_max, g->cpml.order, (double)c.courant, k);
                coef[((size_t)lat * 3 + ax) * stride + i] = make_float4(k[0], k[1], k[2], 0.0f);
            }
    g->cpml_stride = stride;
    const long long area[3] = {(long long)c.ny * c.nz, (long long)c.nx * c.nz, (long long)c.nx * c.ny};
    long long total = 0;
    for (int ax = 0; ax < 3; ++ax) {
        g->cpml_slab[ax] = area[ax] * S;
        g->cpml_psi_off[ax] = total;
        total += 4 * g->cpml_slab[ax];
    }
    EMLAB_CUDA(g->cpml_coef.alloc(coef.size()));
    EMLAB_CUDA(cudaMemcpyAsync(g->cpml_coef.p, coef.data(), coef.size() * sizeof(float4), cudaMemcpyHostToDevice, g->stream));
    EMLAB_CUDA(g->cpml_psi.alloc((size_t)total));
    EMLAB_CUDA(cudaMemsetAsync(g->cpml_psi.p, 0, (size_t)total * sizeof(float), g->stream));
    return EMLAB_OK;
}

int cpml_clear(emlab_grid* g) {
    if (g->cpml_on && g->cpml_psi.p)
        EMLAB_CUDA(cudaMemsetAsync(g->cpml_psi.p, 0, g->cpml_psi.n * sizeof(float), g->stream));
    return EMLAB_OK;
}

void launch_cpml(emlab_grid* g, const YeeArgs& a, bool wide, cudaStream_t s) {
    const CpmlArgs p = cpml_args(g);
    const dim3 grid((a.nx + 127) / 128, a.ny, a.nz);
    if (wide) {
        cpml_b_kernel<uint32_t><<<grid, 128, 0, s>>>(a, p);
        cpml_e_kernel<uint32_t><<<grid, 128, 0, s>>>(a, p);
    } else {
        cpml_b_kernel<uint16_t><<<grid, 128, 0, s>>>(a, p);
        cpml_e_kernel<uint16_t><<<grid, 128, 0, s>>>(a, p);
    }
}

}  // namespace emlab

using namespace emlab;

extern "C" int emlab_grid_set_cpml(emlab_grid* g, const emlab_cpml* params) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(g->stack.scenes() == 0, "the convolutional PML is not available for stacks of scenes");
    if (params) {
        EMLAB_REQUIRE(params->sigma_max >= 0.0f && params->kappa_max >= 1.0f && params->alpha_max >= 0.0f &&
                          params->order >= 1.0f && params->order <= 8.0f,
                      "CPML parameters out of range (sigma_max >= 0, kappa_max >= 1, alpha_max >= 0, 1 <= order <= 8)");
    }
    EMLAB_CUDA(cudaSetDevice(g->device));
    EMLAB_CUDA(cudaStreamSynchronize(g->stream));
    g->cpml_on = params != nullptr;
    if (params) g->cpml = *params;
    if (int rc = upload_pml(g)) return rc;  // the reference absorber's tables: off under the CPML
    if (g->cpml_on) {
        if (int rc = cpml_prepare(g)) return rc;
    } else {
        g->cpml_psi.release(), g->cpml_coef.release();
    }
    if (int rc = clear_fields(g)) return rc;
    g->step = 0;
    return EMLAB_OK;
}
