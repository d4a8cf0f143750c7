// pattern_tc.cu - the far-field pattern of a Huygens box as per-face GEMMs on the tensor cores.
//
// The pattern sums of ntff_pattern.comp:45-110 over the box surface,
//   N(r) = sum_p J_p e^{+jk r.(p - c)},   L(r) = sum_p M_p e^{+jk r.(p - c)},
// with J = n x H w and M = -n x E w (w: the trapezoid edge weights), are separable on a face: its
// nodes form an (nu + 1) x (nv + 1) lattice at fixed a (the face normal axis), so
//   N_q(r) = e^{jk r_a p_a} sum_iu e^{jk r_u p_u(iu)} [ sum_iv e^{jk r_v p_v(iv)} F_q(iv, iu) ]
// for the four tangential fields F_q = J_u, J_v, M_u, M_v. The bracket is a complex GEMM over iv
// for all directions at once (M = directions, N = 4 (nu + 1), K = nv + 1), run on the tcgen05
// tensor cores by nn_gemm (learn.cu) with BF16 operands split into high and low halves
// (A_hi B_hi + A_lo B_hi + A_hi B_lo, concatenated along K: about 16 significant bits per
// operand, FP32 accumulation); the sum over iu is a per-direction dot product with its own twiddles
// (one warp per direction). The sin/cos count falls from directions x points to directions x
// (nu + nv + 2) per face. |N_perp - r x L|^2 and the radiated power follow ntff_reduce.comp:19-39.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/emlab.h"
#include "../../include/emlab_nn.h"
#include "grid_state.h"
#include "sincos_reduced.cuh"

using namespace emlab;

namespace {

struct FaceGeo {
    int a, u, v, side;     // normal axis, tangential axes (u, v as ntff_common.glsl orders them), side
    int nu1, nv1;          // nodes along u (fastest) and v
    int first;             // the face's first point in the DFT's point list
    float pa, pu0, pv0;    // positions relative to the box centre: the plane, the first u and v nodes
    float sign;            // the outward normal's sign
};

FaceGeo face_geo(const int* b, int f) {
    FaceGeo g;
    g.a = f >> 1, g.side = f & 1;
    g.u = g.a == 0 ? 1 : 0, g.v = g.a == 2 ? 1 : 2;
    g.nu1 = b[3 + g.u] - b[g.u] + 1, g.nv1 = b[3 + g.v] - b[g.v] + 1;
    g.first = b[13] + b[6 + f];
    float c[3];
    for (int k = 0; k < 3; ++k) c[k] = 0.5f * (float)(b[k] + b[3 + k]);
    g.pa = (float)(g.side ? b[3 + g.a] : b[g.a]) - c[g.a];
    g.pu0 = (float)b[g.u] - c[g.u];
    g.pv0 = (float)b[g.v] - c[g.v];
    g.sign = g.side ? 1.0f : -1.0f;
    return g;
}

__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16& hi, __nv_bfloat16& lo) {
    hi = __float2bfloat16(x);
    lo = __float2bfloat16(x - __bfloat162float(hi));
}

// The face's tangential fields as the GEMM's B operand, B[q * nu1 + iu][k], k = s * 2 nv1 + h nv1 +
// iv (s: split part hi, hi, lo; h: re, im), rows ld elements apart, and the face's radiated power per
// block (FP32 partials).
__global__ void face_fields_kernel(FaceGeo g, const double2* X, long long total, int f, double scale,
                                   __nv_bfloat16* B, int ld, float* power_part) {
    __shared__ float sp[256];
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = g.nu1 * g.nv1;
    float P = 0.0f;
    if (id < n) {
        const int iu = id % g.nu1, iv = id / g.nu1;
        const double2* x = X + (size_t)f * 6 * total + g.first + id;
        float er[3], ei[3], hr[3], hi[3];
        for (int c = 0; c < 3; ++c) {
            const double2 e = x[(size_t)c * total], h = x[(size_t)(3 + c) * total];
            er[c] = (float)(e.x * scale), ei[c] = (float)(e.y * scale);
            hr[c] = (float)(h.x * scale), hi[c] = (float)(h.y * scale);
        }
        const float w = ((iu == 0 || iu == g.nu1 - 1) ? 0.5f : 1.0f) * ((iv == 0 || iv == g.nv1 - 1) ? 0.5f : 1.0f);
        // n x V for n = sign e_a: component u is sign * (e_a x V)_u, and e_a x e_v = e_u when (a, v, u)
        // is cyclic (a = 1: v = z, u = x), -e_u otherwise
        const float cyc = g.a == 1 ? 1.0f : -1.0f;
        auto cross_u = [&](const float* V) { return g.sign * cyc * V[g.v]; };
        auto cross_v = [&](const float* V) { return -g.sign * cyc * V[g.u]; };
        const float vals[4][2] = {{w * cross_u(hr), w * cross_u(hi)},
                                  {w * cross_v(hr), w * cross_v(hi)},
                                  {-w * cross_u(er), -w * cross_u(ei)},
                                  {-w * cross_v(er), -w * cross_v(ei)}};
        for (int q = 0; q < 4; ++q) {
            __nv_bfloat16* row = B + (size_t)(q * g.nu1 + iu) * ld;
            for (int h = 0; h < 2; ++h) {
                __nv_bfloat16 vh, vl;
                split_bf16(vals[q][h], vh, vl);
                row[0 * 2 * g.nv1 + h * g.nv1 + iv] = vh;
                row[1 * 2 * g.nv1 + h * g.nv1 + iv] = vh;
                row[2 * 2 * g.nv1 + h * g.nv1 + iv] = vl;
            }
        }
        // Re(E x H*) . n w (ntff_pattern.comp's power sum; halved in pattern_finish_kernel)
        float c1[3], c2[3];
        c1[0] = er[1] * hr[2] - hr[1] * er[2], c1[1] = er[2] * hr[0] - hr[2] * er[0], c1[2] = er[0] * hr[1] - hr[0] * er[1];
        c2[0] = ei[1] * hi[2] - hi[1] * ei[2], c2[1] = ei[2] * hi[0] - hi[2] * ei[0], c2[2] = ei[0] * hi[1] - hi[0] * ei[1];
        P = w * g.sign * (c1[g.a] + c2[g.a]);
    }
    sp[threadIdx.x] = P;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sp[threadIdx.x] = sp[threadIdx.x] + sp[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) power_part[blockIdx.x] = sp[0];
}

// The GEMM's A operand for D directions: rows d (real part) and D + d (imaginary part) of
// [Vr -Vi | Vi Vr] (V = e^{jk r_v p_v(iv)}), split as [hi, lo, hi] along K, rows ld elements apart.
__global__ void face_twiddles_kernel(FaceGeo g, const float4* dirs, int D, float kw, __nv_bfloat16* A, int ld) {
    const long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (id >= (long long)D * g.nv1) return;
    const int d = (int)(id / g.nv1), iv = (int)(id % g.nv1);
    const float4 r = dirs[d];
    const float rv = g.v == 0 ? r.x : (g.v == 1 ? r.y : r.z);
    float s, c;
    sincos_reduced(kw * rv * (g.pv0 + (float)iv), &s, &c);
    __nv_bfloat16 ch, cl, sh, sl, nsh, nsl;
    split_bf16(c, ch, cl);
    split_bf16(s, sh, sl);
    split_bf16(-s, nsh, nsl);
    __nv_bfloat16* re = A + (size_t)d * ld;        // Re(V F) = Vr Fr - Vi Fi
    __nv_bfloat16* im = A + (size_t)(D + d) * ld;  // Im(V F) = Vi Fr + Vr Fi
    const int n2 = 2 * g.nv1;
    re[iv] = ch, re[g.nv1 + iv] = nsh, re[n2 + iv] = cl, re[n2 + g.nv1 + iv] = nsl, re[2 * n2 + iv] = ch,
    re[2 * n2 + g.nv1 + iv] = nsh;
    im[iv] = sh, im[g.nv1 + iv] = ch, im[n2 + iv] = sl, im[n2 + g.nv1 + iv] = cl, im[2 * n2 + iv] = sh,
    im[2 * n2 + g.nv1 + iv] = ch;
}

// One warp per direction: sum over iu of e^{jk r_u p_u(iu)} G_q(r, iu) for the four fields, times the
// plane's phase e^{jk r_a p_a}, added to the direction's N and L (12 floats: N re, N im, L re, L im).
__global__ void face_contract_kernel(FaceGeo g, const float4* dirs, int D, float kw, const float* C, int ldc,
                                     float* NL) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= D) return;
    const int d = warp;
    const float4 r = dirs[d];
    const float rr[3] = {r.x, r.y, r.z};
    const float ru = rr[g.u];
    float acc[4][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
    const float* cre = C + (size_t)d * ldc;
    const float* cim = C + (size_t)(D + d) * ldc;
    for (int iu = lane; iu < g.nu1; iu += 32) {
        float s, c;
        sincos_reduced(kw * ru * (g.pu0 + (float)iu), &s, &c);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float gr = cre[q * g.nu1 + iu], gi = cim[q * g.nu1 + iu];
            acc[q][0] = fmaf(c, gr, fmaf(-s, gi, acc[q][0]));
            acc[q][1] = fmaf(s, gr, fmaf(c, gi, acc[q][1]));
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc[q][h] += __shfl_xor_sync(0xffffffffu, acc[q][h], o);
    if (lane) return;
    float s, c;
    sincos_reduced(kw * rr[g.a] * g.pa, &s, &c);
    float* o = NL + (size_t)d * 12;
    const int comp[4] = {g.u, g.v, g.u, g.v};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float re = c * acc[q][0] - s * acc[q][1], im = s * acc[q][0] + c * acc[q][1];
        const int base = q < 2 ? 0 : 6;
        o[base + comp[q]] += re;
        o[base + 3 + comp[q]] += im;
    }
}

// ntff_reduce.comp:19-39 from the accumulated N, L: out[2 d] = |N_perp - r x L|^2 (both parts),
// out[1] = P / 2 for the first direction.
__global__ void pattern_finish_kernel(const float4* dirs, int D, const float* NL, const float* power_part,
                                      int n_parts, float* out) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= D) return;
    const float4 r = dirs[d];
    const float rv[3] = {r.x, r.y, r.z};
    const float* o = NL + (size_t)d * 12;
    float F2 = 0.0f;
    for (int part = 0; part < 2; ++part) {
        const float* N = o + 3 * part;
        const float* L = o + 6 + 3 * part;
        const float dn = N[0] * rv[0] + N[1] * rv[1] + N[2] * rv[2];
        const float rl0 = rv[1] * L[2] - L[1] * rv[2];
        const float rl1 = rv[2] * L[0] - L[2] * rv[0];
        const float rl2 = rv[0] * L[1] - L[0] * rv[1];
        const float F0 = (N[0] - dn * rv[0]) - rl0, F1 = (N[1] - dn * rv[1]) - rl1, Fz = (N[2] - dn * rv[2]) - rl2;
        F2 = F2 + (F0 * F0 + F1 * F1 + Fz * Fz);
    }
    out[2 * (size_t)d] = F2;
    if (d == 0) {
        float P = 0.0f;
        for (int k = 0; k < n_parts; ++k) P += power_part[k];
        out[1] = 0.5f * P;
    } else {
        out[2 * (size_t)d + 1] = 0.0f;
    }
}

}  // namespace

extern "C" int emlab_ntff_dft_pattern_gemm(emlab_grid* g, int box, const float* directions, int n_dirs, float* out) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(g->dft_on, "no far-field DFT attached");
    EMLAB_REQUIRE(box >= 0 && box < g->dft_nbox, "no such far-field DFT box");
    EMLAB_REQUIRE(directions && out && n_dirs > 0 && n_dirs <= (1 << 20), "bad direction arguments");
    EMLAB_CUDA(cudaSetDevice(g->device));
    if (int rc = dft_fold_now(g)) return rc;
    const uint64_t samples = g->dft_samples;
    EMLAB_REQUIRE(samples > 0, "no far-field DFT samples yet");
    const int* b = g->dft_boxes.data() + (size_t)box * kDftBoxInts;
    const double scale = 2.0 / (double)samples;
    const int D = n_dirs;
    // the largest face sets the scratch sizes
    int max_k = 0, max_n = 0, max_pts = 0;
    for (int f = 0; f < 6; ++f) {
        const FaceGeo fg = face_geo(b, f);
        max_k = std::max(max_k, (6 * fg.nv1 + 7) / 8 * 8), max_n = std::max(max_n, 4 * fg.nu1);
        max_pts = std::max(max_pts, fg.nu1 * fg.nv1);
    }
    const int parts_per_face = (max_pts + 255) / 256;
    DevBuf<float4> d_dirs;
    DevBuf<__nv_bfloat16> d_a, d_b;
    DevBuf<float> d_c, d_nl, d_out, d_pow;
    EMLAB_CUDA(d_dirs.alloc((size_t)D));
    EMLAB_CUDA(d_a.alloc((size_t)2 * D * max_k));
    EMLAB_CUDA(d_b.alloc((size_t)max_n * max_k));
    EMLAB_CUDA(d_c.alloc((size_t)2 * D * max_n));
    EMLAB_CUDA(d_nl.alloc((size_t)D * 12));
    EMLAB_CUDA(d_out.alloc((size_t)g->dft_nf * D * 2));
    EMLAB_CUDA(d_pow.alloc((size_t)6 * parts_per_face));
    std::vector<float4> dirs((size_t)D);
    for (int d = 0; d < D; ++d)
        dirs[(size_t)d] = make_float4(directions[4 * d], directions[4 * d + 1], directions[4 * d + 2], 0.0f);
    EMLAB_CUDA(cudaMemcpyAsync(d_dirs.p, dirs.data(), (size_t)D * 16, cudaMemcpyHostToDevice, g->stream));
    const double2* X = reinterpret_cast<const double2*>(g->d_dft_x.p);
    for (int f = 0; f < g->dft_nf; ++f) {
        const float kw = (float)g->dft_omega[(size_t)f];
        EMLAB_CUDA(cudaMemsetAsync(d_nl.p, 0, (size_t)D * 12 * 4, g->stream));
        EMLAB_CUDA(cudaMemsetAsync(d_pow.p, 0, d_pow.n * 4, g->stream));
        for (int face = 0; face < 6; ++face) {
            const FaceGeo fg = face_geo(b, face);
            // K = 6 nv1 (two split parts of A against the high part of B, then the reverse; real and
            // imaginary halves); rows padded to 16 bytes so the GEMM stages them 16 bytes at a time
            const int K = 6 * fg.nv1, ld = (K + 7) / 8 * 8, N = 4 * fg.nu1, pts = fg.nu1 * fg.nv1;
            face_fields_kernel<<<(pts + 255) / 256, 256, 0, g->stream>>>(fg, X, g->dft_points, f, scale, d_b.p, ld,
                                                                         d_pow.p + (size_t)face * parts_per_face);
            const long long tw = (long long)D * fg.nv1;
            face_twiddles_kernel<<<(unsigned)((tw + 255) / 256), 256, 0, g->stream>>>(fg, d_dirs.p, D, kw, d_a.p, ld);
            if (int rc = emlab_nn_gemm(2 * D, N, K, d_a.p, ld, 1, d_b.p, ld, 1, d_c.p, N, g->stream)) return rc;
            face_contract_kernel<<<(D * 32 + 255) / 256, 256, 0, g->stream>>>(fg, d_dirs.p, D, kw, d_c.p, N, d_nl.p);
            count_launches(3);
        }
        pattern_finish_kernel<<<(D + 255) / 256, 256, 0, g->stream>>>(d_dirs.p, D, d_nl.p, d_pow.p,
                                                                      6 * parts_per_face,
                                                                      d_out.p + (size_t)f * D * 2);
        count_launches(1);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return fail(EMLAB_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    }
    if (int rc = emlab_nn_status(g->stream)) return rc;
    EMLAB_CUDA(cudaMemcpyAsync(out, d_out.p, (size_t)g->dft_nf * D * 8, cudaMemcpyDeviceToHost, g->stream));
    return emlab_grid_synchronize(g, 0);
}
