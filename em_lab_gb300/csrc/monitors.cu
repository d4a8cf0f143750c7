// monitors.cu - per-step and on-demand monitor kernels on sm_103a.
//
// Each kernel restates one reference shader (file:line on each) and, like the solver, is compiled
// with -fmad=false so its per-step FP32 arithmetic matches the CPU restatement bit for bit.
// Monitors read the field generation that the step just produced.
#include "emlab_internal.h"
#include "sincos_reduced.cuh"

namespace emlab {

namespace {

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__device__ __forceinline__ long long cidx(const MonitorArgs& m, int x, int y, int z) {
    x = clampi(x, 0, m.nx - 1), y = clampi(y, 0, m.ny - 1), z = clampi(z, 0, m.nz - 1);
    return (long long)z * m.plane + (long long)y * m.pitch + x;
}

__device__ __forceinline__ const float* ecomp(const MonitorArgs& m, int c) { return c == 0 ? m.ex : (c == 1 ? m.ey : m.ez); }
__device__ __forceinline__ const float* bcomp(const MonitorArgs& m, int c) { return c == 0 ? m.bx : (c == 1 ? m.by : m.bz); }

// field_sampling.glsl:17-23 (clamp-to-edge fetches)
__device__ __forceinline__ void e_at_node(const MonitorArgs& m, int x, int y, int z, float& ex, float& ey, float& ez) {
    ex = 0.5f * (m.ex[cidx(m, x, y, z)] + m.ex[cidx(m, x - 1, y, z)]);
    ey = 0.5f * (m.ey[cidx(m, x, y, z)] + m.ey[cidx(m, x, y - 1, z)]);
    ez = 0.5f * (m.ez[cidx(m, x, y, z)] + m.ez[cidx(m, x, y, z - 1)]);
}

// field_sampling.glsl:25-32
__device__ __forceinline__ void b_at_node(const MonitorArgs& m, int x, int y, int z, float& bx, float& by, float& bz) {
    const float sx = m.bx[cidx(m, x, y, z)] + m.bx[cidx(m, x, y - 1, z)] + m.bx[cidx(m, x, y, z - 1)] +
                     m.bx[cidx(m, x, y - 1, z - 1)];
    const float sy = m.by[cidx(m, x, y, z)] + m.by[cidx(m, x - 1, y, z)] + m.by[cidx(m, x, y, z - 1)] +
                     m.by[cidx(m, x - 1, y, z - 1)];
    const float sz = m.bz[cidx(m, x, y, z)] + m.bz[cidx(m, x - 1, y, z)] + m.bz[cidx(m, x, y - 1, z)] +
                     m.bz[cidx(m, x - 1, y - 1, z)];
    bx = 0.25f * sx, by = 0.25f * sy, bz = 0.25f * sz;
}

// port_accumulate.comp:46-50
__device__ __forceinline__ float edge_current(const MonitorArgs& m, int x, int y, int z, int a) {
    const int u = (a + 1) % 3, v = (a + 2) % 3;
    int pu[3] = {x, y, z}, pv[3] = {x, y, z};
    pu[u] -= 1, pv[v] -= 1;
    const float b0v = bcomp(m, v)[cidx(m, x, y, z)], b0u = bcomp(m, u)[cidx(m, x, y, z)];
    const float buv = bcomp(m, v)[cidx(m, pu[0], pu[1], pu[2])];
    const float bvu = bcomp(m, u)[cidx(m, pv[0], pv[1], pv[2])];
    return (b0v - buv) - (b0u - bvu);
}

// port_accumulate.comp:52-83
__global__ void ports_kernel(MonitorArgs m, const int4* ports, int n, float* ph, float* series, long long rec,
                             const float4* rot, const float* blend, int k) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int4 p = ports[2 * i], info = ports[2 * i + 1];
    const int a = p.w;
    const float s = (float)info.y;
    float V = 0.0f, I = 0.0f;
    if (info.x == 4) {
        int eu[3] = {0, 0, 0}, ev[3] = {0, 0, 0};
        eu[(a + 1) % 3] = 1, ev[(a + 2) % 3] = 1;
        for (int q = 0; q < 4; ++q) {
            const int ox = (q & 1 ? eu[0] : 0) + (q & 2 ? ev[0] : 0);
            const int oy = (q & 1 ? eu[1] : 0) + (q & 2 ? ev[1] : 0);
            const int oz = (q & 1 ? eu[2] : 0) + (q & 2 ? ev[2] : 0);
            V = V + 0.25f * ecomp(m, a)[cidx(m, p.x + ox, p.y + oy, p.z + oz)];
            I = I + edge_current(m, p.x + ox, p.y + oy, p.z + oz, a);
        }
    } else {
        V = ecomp(m, a)[cidx(m, p.x, p.y, p.z)];
        I = edge_current(m, p.x, p.y, p.z, a);
    }
    V = V * s;
    I = I * s;
    if (rec >= 0) {
        series[(rec * n + i) * 2 + 0] = V;
        series[(rec * n + i) * 2 + 1] = I;
    }
    const float4 r = rot[k];
    const float b = blend[k];
    const float o0 = (2.0f * r.x) * V, o1 = (-2.0f * r.y) * V, o2 = (2.0f * r.z) * I, o3 = (-2.0f * r.w) * I;
    float* q = ph + 8 * i;
    q[0] = q[0] + b * (o0 - q[0]);
    q[1] = q[1] + b * (o1 - q[1]);
    q[2] = q[2] + b * (o2 - q[2]);
    q[3] = q[3] + b * (o3 - q[3]);
    q[4] = q[4] + b * (q[0] - q[4]);
    q[5] = q[5] + b * (q[1] - q[5]);
    q[6] = q[6] + b * (q[2] - q[6]);
    q[7] = q[7] + b * (q[3] - q[7]);
}

// ntff_common.glsl:30-53; box = (min xyz, max xyz, face offsets[7])
__device__ __forceinline__ void ntff_point(const int* box, int index, int node[3], float n[3], float& w) {
    int f = 0;
    for (int i = 1; i < 6; ++i)
        if (index >= box[6 + i]) f = i;
    const int a = f >> 1, side = f & 1;
    const int u = a == 0 ? 1 : 0, v = a == 2 ? 1 : 2;
    const int nu = box[3 + u] - box[u], nv = box[3 + v] - box[v];
    const int local = index - box[6 + f];
    const int iu = local % (nu + 1), iv = local / (nu + 1);
    node[0] = box[0], node[1] = box[1], node[2] = box[2];
    node[a] = side == 1 ? box[3 + a] : box[a];
    node[u] = box[u] + iu;
    node[v] = box[v] + iv;
    w = ((iu == 0 || iu == nu) ? 0.5f : 1.0f) * ((iv == 0 || iv == nv) ? 0.5f : 1.0f);
    n[0] = n[1] = n[2] = 0.0f;
    n[a] = side == 1 ? 1.0f : -1.0f;
}

// ntff_accumulate.comp:30-52: 32 floats per point (stage1 eRe, eIm, hRe, hIm, stage2 ...). The
// block's 128 x 128 B of state move between HBM and shared memory as one contiguous chunk
// (consecutive threads, consecutive float4s), rows padded to 9 float4s against bank conflicts;
// each thread then updates its own point there. Every load a thread makes (its eight float4s of
// the block's state and the 18 field values of its node) is issued before the first is used, so
// the kernel waits one memory round trip instead of nine. Same arithmetic per point.
constexpr int kNtffThreads = 128;
__global__ void __launch_bounds__(kNtffThreads) ntff_kernel(MonitorArgs m, const int* box, int points, float4* ph,
                                                            const float4* rot, const float* blend, int k) {
    __shared__ int sbox[13];
    __shared__ float4 st[kNtffThreads * 9];
    if (threadIdx.x < 13) sbox[threadIdx.x] = box[threadIdx.x];
    const int first = blockIdx.x * kNtffThreads;
    const int count = min(kNtffThreads, points - first);
    float4* base = ph + 8 * (long long)first;
    float4 v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int j = threadIdx.x + q * kNtffThreads;
        if (j < 8 * count) v[q] = base[j];
    }
    __syncthreads();  // sbox
    const int i = first + threadIdx.x;
    const bool live = i < points;
    float E[3], Hh[3];
    if (live) {
        int node[3];
        float n[3], w;
        ntff_point(sbox, i, node, n, w);
        e_at_node(m, node[0], node[1], node[2], E[0], E[1], E[2]);
        b_at_node(m, node[0], node[1], node[2], Hh[0], Hh[1], Hh[2]);
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int j = threadIdx.x + q * kNtffThreads;
        if (j < 8 * count) st[9 * (j >> 3) + (j & 7)] = v[q];
    }
    __syncthreads();
    if (live) {
        const float4 r = rot[k];
        const float b = blend[k];
        float4* p = st + 9 * threadIdx.x;
        float4 s1[4] = {p[0], p[1], p[2], p[3]}, s2[4] = {p[4], p[5], p[6], p[7]};
        const float f[4] = {2.0f * r.x, -2.0f * r.y, 2.0f * r.z, -2.0f * r.w};
        for (int q = 0; q < 4; ++q) {
            const float* src = q < 2 ? E : Hh;
            s1[q].x = s1[q].x + b * (f[q] * src[0] - s1[q].x);
            s1[q].y = s1[q].y + b * (f[q] * src[1] - s1[q].y);
            s1[q].z = s1[q].z + b * (f[q] * src[2] - s1[q].z);
        }
        for (int q = 0; q < 4; ++q) {
            s2[q].x = s2[q].x + b * (s1[q].x - s2[q].x);
            s2[q].y = s2[q].y + b * (s1[q].y - s2[q].y);
            s2[q].z = s2[q].z + b * (s1[q].z - s2[q].z);
        }
        for (int q = 0; q < 4; ++q) p[q] = s1[q], p[4 + q] = s2[q];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int j = threadIdx.x + q * kNtffThreads;
        if (j < 8 * count) base[j] = st[9 * (j >> 3) + (j & 7)];
    }
}

// line_accumulate.comp:30-48
__global__ void lines_kernel(MonitorArgs m, const int4* qs, int nq, const int4* terms, const float* weights, float4* ph,
                             float* now, const float4* rot, const float* blend, int k) {
    const int qi = blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= nq) return;
    const int4 info = qs[qi];
    float sum = 0.0f;
    for (int t = info.x; t < info.x + info.y; ++t) {
        const int4 tt = terms[t];
        const long long j = cidx(m, tt.x, tt.y, tt.z);
        const float f = tt.w < 3 ? ecomp(m, tt.w % 3)[j] : bcomp(m, tt.w % 3)[j];
        sum = sum + weights[t] * f;
    }
    now[qi] = sum;
    const float4 r = rot[k];
    const float b = blend[k];
    const float r0 = info.z == 0 ? r.x : r.z, r1 = info.z == 0 ? r.y : r.w;
    const float o0 = (2.0f * sum) * r0, o1 = (2.0f * sum) * -r1;
    float4 p = ph[qi];
    p.x = p.x + b * (o0 - p.x);
    p.y = p.y + b * (o1 - p.y);
    p.z = p.z + b * (p.x - p.z);
    p.w = p.w + b * (p.y - p.w);
    ph[qi] = p;
}

// probe_gather.comp:20-26 (alpha channels are filled on the host)
__global__ void probe_kernel(MonitorArgs m, const int4* origins, int n, float4* out) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n * 54) return;
    const int probe = id / 54, k = id % 54, t = k % 27;
    const int4 o = origins[probe];
    const long long j = cidx(m, o.x + t % 3, o.y + (t / 3) % 3, o.z + t / 9);
    out[id] = k < 27 ? make_float4(m.ex[j], m.ey[j], m.ez[j], 0.0f) : make_float4(m.bx[j], m.by[j], m.bz[j], 0.0f);
}

// poynting_flux.comp:32-63: one partial per 16x16 workgroup, tree reduction in the shader's order
__global__ void __launch_bounds__(256) flux_kernel(MonitorArgs m, int axis, int index, int rmin0, int rmin1, int rs0,
                                                   int rs1, float* partials) {
    __shared__ float sp[256];
    const int lu = blockIdx.x * 16 + threadIdx.x, lv = blockIdx.y * 16 + threadIdx.y;
    const int lid = threadIdx.y * 16 + threadIdx.x;
    float flux = 0.0f;
    if (lu < rs0 && lv < rs1) {
        const int u = rmin0 + lu, v = rmin1 + lv;
        int p[3];
        if (axis == 0) p[0] = index, p[1] = u, p[2] = v;
        else if (axis == 1) p[0] = u, p[1] = index, p[2] = v;
        else p[0] = u, p[1] = v, p[2] = index;
        if (p[0] >= 0 && p[1] >= 0 && p[2] >= 0 && p[0] < m.nx && p[1] < m.ny && p[2] < m.nz) {
            float E[3], Bn[3];
            e_at_node(m, p[0], p[1], p[2], E[0], E[1], E[2]);
            b_at_node(m, p[0], p[1], p[2], Bn[0], Bn[1], Bn[2]);
            const float S0 = E[1] * Bn[2] - Bn[1] * E[2];
            const float S1 = E[2] * Bn[0] - Bn[2] * E[0];
            const float S2 = E[0] * Bn[1] - Bn[0] * E[1];
            flux = axis == 0 ? S0 : (axis == 1 ? S1 : S2);
        }
    }
    sp[lid] = flux;
    __syncthreads();
    for (int stride = 128; stride > 0; stride >>= 1) {
        if (lid < stride) sp[lid] = sp[lid] + sp[lid + stride];
        __syncthreads();
    }
    if (lid == 0) partials[blockIdx.y * gridDim.x + blockIdx.x] = sp[0];
}

// ntff_pattern.comp:45-110 (128 directions x one surface slice per block)
__global__ void __launch_bounds__(128) ntff_pattern_kernel(const int* box, int points, const float4* ph,
                                                           const float4* dirs, int first, int count, int slices,
                                                           float kw, float4* partials) {
    __shared__ float4 sPos[128], sJr[128], sJi[128], sMr[128], sMi[128];
    __shared__ float sP[128];
    __shared__ int sbox[13];
    const int lid = threadIdx.x;
    if (lid < 13) sbox[lid] = box[lid];
    __syncthreads();
    const int local = blockIdx.x * 128 + lid;
    const int d = first + local;
    const int slice = blockIdx.y;
    const bool inRange = d < first + count;
    const float4 rr = inRange ? dirs[d] : make_float4(0.0f, 0.0f, 1.0f, 0.0f);
    const bool power = blockIdx.x == 0 && first == 0;
    const float cx = 0.5f * (float)(sbox[0] + sbox[3]), cy = 0.5f * (float)(sbox[1] + sbox[4]),
                cz = 0.5f * (float)(sbox[2] + sbox[5]);
    const int per = (points + slices - 1) / slices;
    const int f0 = slice * per, last = min(f0 + per, points);
    float Nr[3] = {0, 0, 0}, Ni[3] = {0, 0, 0}, Lr[3] = {0, 0, 0}, Li[3] = {0, 0, 0};
    float P = 0.0f;
    for (int base = f0; base < last; base += 128) {
        const int i = base + lid;
        if (i < last) {
            int node[3];
            float n[3], w;
            ntff_point(sbox, i, node, n, w);
            const float4* s2 = ph + 8 * (long long)i + 4;
            const float4 eR = s2[0], eI = s2[1], hR = s2[2], hI = s2[3];
            sPos[lid] = make_float4((float)node[0] - cx, (float)node[1] - cy, (float)node[2] - cz, 0.0f);
            // cross(n, v) = (n1 v2 - v1 n2, n2 v0 - v2 n0, n0 v1 - v0 n1)
#define EMLAB_CROSS(A0, A1, A2, B0, B1, B2) \
    make_float4(A1 * B2 - B1 * A2, A2 * B0 - B2 * A0, A0 * B1 - B0 * A1, 0.0f)
            const float4 jr = EMLAB_CROSS(n[0], n[1], n[2], hR.x, hR.y, hR.z);
            const float4 ji = EMLAB_CROSS(n[0], n[1], n[2], hI.x, hI.y, hI.z);
            const float4 mr = EMLAB_CROSS(n[0], n[1], n[2], eR.x, eR.y, eR.z);
            const float4 mi = EMLAB_CROSS(n[0], n[1], n[2], eI.x, eI.y, eI.z);
            sJr[lid] = make_float4(w * jr.x, w * jr.y, w * jr.z, 0.0f);
            sJi[lid] = make_float4(w * ji.x, w * ji.y, w * ji.z, 0.0f);
            sMr[lid] = make_float4(-w * mr.x, -w * mr.y, -w * mr.z, 0.0f);
            sMi[lid] = make_float4(-w * mi.x, -w * mi.y, -w * mi.z, 0.0f);
            if (power) {
                const float4 c1 = EMLAB_CROSS(eR.x, eR.y, eR.z, hR.x, hR.y, hR.z);
                const float4 c2 = EMLAB_CROSS(eI.x, eI.y, eI.z, hI.x, hI.y, hI.z);
                const float s0 = c1.x + c2.x, s1 = c1.y + c2.y, s2v = c1.z + c2.z;
                P = P + w * (s0 * n[0] + s1 * n[1] + s2v * n[2]);
            }
#undef EMLAB_CROSS
        }
        __syncthreads();
        const int cnt = min(128, last - base);
        for (int q = 0; q < cnt; ++q) {
            const float4 pos = sPos[q];
            const float psi = kw * (rr.x * pos.x + rr.y * pos.y + rr.z * pos.z);
            float sn, cs;
            sincosf(psi, &sn, &cs);
            const float4 jr = sJr[q], ji = sJi[q], mr = sMr[q], mi = sMi[q];
            Nr[0] = Nr[0] + (jr.x * cs - ji.x * sn), Nr[1] = Nr[1] + (jr.y * cs - ji.y * sn), Nr[2] = Nr[2] + (jr.z * cs - ji.z * sn);
            Ni[0] = Ni[0] + (jr.x * sn + ji.x * cs), Ni[1] = Ni[1] + (jr.y * sn + ji.y * cs), Ni[2] = Ni[2] + (jr.z * sn + ji.z * cs);
            Lr[0] = Lr[0] + (mr.x * cs - mi.x * sn), Lr[1] = Lr[1] + (mr.y * cs - mi.y * sn), Lr[2] = Lr[2] + (mr.z * cs - mi.z * sn);
            Li[0] = Li[0] + (mr.x * sn + mi.x * cs), Li[1] = Li[1] + (mr.y * sn + mi.y * cs), Li[2] = Li[2] + (mr.z * sn + mi.z * cs);
        }
        __syncthreads();
    }
    sP[lid] = P;
    __syncthreads();
    for (int stride = 64; stride > 0; stride >>= 1) {
        if (lid < stride) sP[lid] = sP[lid] + sP[lid + stride];
        __syncthreads();
    }
    if (inRange) {
        const long long o = 4ll * ((long long)local * slices + slice);
        partials[o + 0] = make_float4(Nr[0], Nr[1], Nr[2], (power && lid == 0) ? sP[0] : 0.0f);
        partials[o + 1] = make_float4(Ni[0], Ni[1], Ni[2], 0.0f);
        partials[o + 2] = make_float4(Lr[0], Lr[1], Lr[2], 0.0f);
        partials[o + 3] = make_float4(Li[0], Li[1], Li[2], 0.0f);
    }
}


// Surface sources of the fast pattern sums. PhasorSource: the stage-2 phasors of ntff_pattern.comp's
// layout (8 float4 per point). DftSource: the far-field DFT sums of frequency f straight from X
// ([f][c][i] complex FP64), scaled and rounded to FP32 as dft_to_phasor_kernel stages them, for a
// box whose first point in X is `first`.
struct PhasorSource {
    const float4* ph;
    float k;
    __device__ float kw(int) const { return k; }
    __device__ void load(int, int i, float4& eR, float4& eI, float4& hR, float4& hI) const {
        const float4* s2 = ph + 8 * (long long)i + 4;
        eR = s2[0], eI = s2[1], hR = s2[2], hI = s2[3];
    }
};
struct DftSource {
    const double* X;
    long long total;
    int first;
    const double* omega;
    double scale;
    __device__ float kw(int f) const { return (float)omega[f]; }
    __device__ void load(int f, int i, float4& eR, float4& eI, float4& hR, float4& hI) const {
        const double2* x = reinterpret_cast<const double2*>(X) + (size_t)f * 6 * total + first + i;
        double2 v[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) v[c] = x[(size_t)c * total];
        eR = make_float4((float)(v[0].x * scale), (float)(v[1].x * scale), (float)(v[2].x * scale), 0.0f);
        eI = make_float4((float)(v[0].y * scale), (float)(v[1].y * scale), (float)(v[2].y * scale), 0.0f);
        hR = make_float4((float)(v[3].x * scale), (float)(v[4].x * scale), (float)(v[5].x * scale), 0.0f);
        hI = make_float4((float)(v[3].y * scale), (float)(v[4].y * scale), (float)(v[5].y * scale), 0.0f);
    }
};

// The same sums as ntff_pattern_kernel for 256 directions per block (two per thread, sharing every
// staged surface point), with sincos_reduced and explicit multiply-adds: the far-field DFT's
// pattern over large angle grids. blockIdx.z is the source's frequency; each frequency has its own
// block of partials (count * slices * 4 float4).
template <class Src>
__global__ void __launch_bounds__(128) ntff_pattern_fast_kernel(const int* box, int points, Src src,
                                                                const float4* dirs, int first, int count, int slices,
                                                                float4* partials) {
    __shared__ float4 sPos[128], sJr[128], sJi[128], sMr[128], sMi[128];
    __shared__ float sP[128];
    __shared__ int sbox[13];
    const int lid = threadIdx.x;
    const int fq = blockIdx.z;
    const float kw = src.kw(fq);
    partials += (size_t)fq * count * slices * 4;
    if (lid < 13) sbox[lid] = box[lid];
    __syncthreads();
    const int local0 = blockIdx.x * 256 + lid, local1 = local0 + 128;
    const int slice = blockIdx.y;
    const bool in0 = local0 < count, in1 = local1 < count;
    const float4 r0 = in0 ? dirs[first + local0] : make_float4(0.0f, 0.0f, 1.0f, 0.0f);
    const float4 r1 = in1 ? dirs[first + local1] : make_float4(0.0f, 0.0f, 1.0f, 0.0f);
    const bool power = blockIdx.x == 0 && first == 0;
    const float cx = 0.5f * (float)(sbox[0] + sbox[3]), cy = 0.5f * (float)(sbox[1] + sbox[4]),
                cz = 0.5f * (float)(sbox[2] + sbox[5]);
    const int per = (points + slices - 1) / slices;
    const int f0 = slice * per, last = min(f0 + per, points);
    float a[2][12];
#pragma unroll
    for (int t = 0; t < 2; ++t)
#pragma unroll
        for (int j = 0; j < 12; ++j) a[t][j] = 0.0f;
    float P = 0.0f;
    const float k0x = kw * r0.x, k0y = kw * r0.y, k0z = kw * r0.z, k1x = kw * r1.x, k1y = kw * r1.y, k1z = kw * r1.z;
    for (int base = f0; base < last; base += 128) {
        const int i = base + lid;
        if (i < last) {
            int node[3];
            float n[3], w;
            ntff_point(sbox, i, node, n, w);
            float4 eR, eI, hR, hI;
            src.load(fq, i, eR, eI, hR, hI);
            sPos[lid] = make_float4((float)node[0] - cx, (float)node[1] - cy, (float)node[2] - cz, 0.0f);
#define EMLAB_CROSS(A0, A1, A2, B0, B1, B2) \
    make_float4(A1 * B2 - B1 * A2, A2 * B0 - B2 * A0, A0 * B1 - B0 * A1, 0.0f)
            const float4 jr = EMLAB_CROSS(n[0], n[1], n[2], hR.x, hR.y, hR.z);
            const float4 ji = EMLAB_CROSS(n[0], n[1], n[2], hI.x, hI.y, hI.z);
            const float4 mr = EMLAB_CROSS(n[0], n[1], n[2], eR.x, eR.y, eR.z);
            const float4 mi = EMLAB_CROSS(n[0], n[1], n[2], eI.x, eI.y, eI.z);
            sJr[lid] = make_float4(w * jr.x, w * jr.y, w * jr.z, 0.0f);
            sJi[lid] = make_float4(w * ji.x, w * ji.y, w * ji.z, 0.0f);
            sMr[lid] = make_float4(-w * mr.x, -w * mr.y, -w * mr.z, 0.0f);
            sMi[lid] = make_float4(-w * mi.x, -w * mi.y, -w * mi.z, 0.0f);
            if (power) {
                const float4 c1 = EMLAB_CROSS(eR.x, eR.y, eR.z, hR.x, hR.y, hR.z);
                const float4 c2 = EMLAB_CROSS(eI.x, eI.y, eI.z, hI.x, hI.y, hI.z);
                P = P + w * ((c1.x + c2.x) * n[0] + (c1.y + c2.y) * n[1] + (c1.z + c2.z) * n[2]);
            }
#undef EMLAB_CROSS
        }
        __syncthreads();
        const int cnt = min(128, last - base);
        for (int q = 0; q < cnt; ++q) {
            const float4 pos = sPos[q];
            const float4 jr = sJr[q], ji = sJi[q], mr = sMr[q], mi = sMi[q];
            float sn[2], cs[2];
            sincos_reduced(fmaf(k0x, pos.x, fmaf(k0y, pos.y, k0z * pos.z)), &sn[0], &cs[0]);
            sincos_reduced(fmaf(k1x, pos.x, fmaf(k1y, pos.y, k1z * pos.z)), &sn[1], &cs[1]);
#pragma unroll
            for (int t = 0; t < 2; ++t) {
                const float c = cs[t], s = sn[t];
                a[t][0] = fmaf(jr.x, c, fmaf(-ji.x, s, a[t][0]));
                a[t][1] = fmaf(jr.y, c, fmaf(-ji.y, s, a[t][1]));
                a[t][2] = fmaf(jr.z, c, fmaf(-ji.z, s, a[t][2]));
                a[t][3] = fmaf(jr.x, s, fmaf(ji.x, c, a[t][3]));
                a[t][4] = fmaf(jr.y, s, fmaf(ji.y, c, a[t][4]));
                a[t][5] = fmaf(jr.z, s, fmaf(ji.z, c, a[t][5]));
                a[t][6] = fmaf(mr.x, c, fmaf(-mi.x, s, a[t][6]));
                a[t][7] = fmaf(mr.y, c, fmaf(-mi.y, s, a[t][7]));
                a[t][8] = fmaf(mr.z, c, fmaf(-mi.z, s, a[t][8]));
                a[t][9] = fmaf(mr.x, s, fmaf(mi.x, c, a[t][9]));
                a[t][10] = fmaf(mr.y, s, fmaf(mi.y, c, a[t][10]));
                a[t][11] = fmaf(mr.z, s, fmaf(mi.z, c, a[t][11]));
            }
        }
        __syncthreads();
    }
    sP[lid] = P;
    __syncthreads();
    for (int stride = 64; stride > 0; stride >>= 1) {
        if (lid < stride) sP[lid] = sP[lid] + sP[lid + stride];
        __syncthreads();
    }
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        const int local = t ? local1 : local0;
        if (!(t ? in1 : in0)) continue;
        const long long o = 4ll * ((long long)local * slices + slice);
        partials[o + 0] = make_float4(a[t][0], a[t][1], a[t][2], (power && lid == 0 && t == 0) ? sP[0] : 0.0f);
        partials[o + 1] = make_float4(a[t][3], a[t][4], a[t][5], 0.0f);
        partials[o + 2] = make_float4(a[t][6], a[t][7], a[t][8], 0.0f);
        partials[o + 3] = make_float4(a[t][9], a[t][10], a[t][11], 0.0f);
    }
}

// ntff_reduce.comp:19-39 (blockIdx.y: the frequency of a multi-frequency pattern, each with its own
// partials and outputs)
__global__ void ntff_reduce_kernel(const float4* dirs, const float4* partials, int first, int count, int slices,
                                   float* out) {
    partials += (size_t)blockIdx.y * count * slices * 4;
    out += (size_t)blockIdx.y * count * 2;
    const int local = blockIdx.x * blockDim.x + threadIdx.x;
    const int d = first + local;
    if (local >= count) return;
    const float4 r = dirs[d];
    float N[2][3] = {{0, 0, 0}, {0, 0, 0}}, L[2][3] = {{0, 0, 0}, {0, 0, 0}};
    float P = 0.0f;
    for (int s = 0; s < slices; ++s) {
        const long long o = 4ll * ((long long)local * slices + s);
        const float4 a = partials[o], b = partials[o + 1], c = partials[o + 2], e = partials[o + 3];
        N[0][0] = N[0][0] + a.x, N[0][1] = N[0][1] + a.y, N[0][2] = N[0][2] + a.z;
        P = P + a.w;
        N[1][0] = N[1][0] + b.x, N[1][1] = N[1][1] + b.y, N[1][2] = N[1][2] + b.z;
        L[0][0] = L[0][0] + c.x, L[0][1] = L[0][1] + c.y, L[0][2] = L[0][2] + c.z;
        L[1][0] = L[1][0] + e.x, L[1][1] = L[1][1] + e.y, L[1][2] = L[1][2] + e.z;
    }
    const float rv[3] = {r.x, r.y, r.z};
    float F2 = 0.0f;
    for (int part = 0; part < 2; ++part) {
        const float dn = N[part][0] * rv[0] + N[part][1] * rv[1] + N[part][2] * rv[2];
        const float rl0 = rv[1] * L[part][2] - L[part][1] * rv[2];
        const float rl1 = rv[2] * L[part][0] - L[part][2] * rv[0];
        const float rl2 = rv[0] * L[part][1] - L[part][0] * rv[1];
        const float F0 = (N[part][0] - dn * rv[0]) - rl0, F1 = (N[part][1] - dn * rv[1]) - rl1,
                    F2c = (N[part][2] - dn * rv[2]) - rl2;
        F2 = F2 + (F0 * F0 + F1 * F1 + F2c * F2c);
    }
    out[2 * d] = F2;
    out[2 * d + 1] = 0.5f * P;
}

// PortMonitor::evaluateSweep sums (Ports.cpp:215-242) in FP64: one block per (port, frequency)
__global__ void __launch_bounds__(256) sweep_kernel(const float* series, long long steps, int nports, double nu_lo,
                                                    double nu_hi, int points, double dt, double* out) {
    const int pf = blockIdx.x;
    const int p = pf / points, f = pf % points;
    const double nu = nu_lo + (nu_hi - nu_lo) * f / (points - 1);
    const double w = 6.283185307179586476925 * nu;
    double acc[4] = {0, 0, 0, 0};
    for (long long k = threadIdx.x; k < steps; k += blockDim.x) {
        double s, c;
        sincos(-w * dt * (double)k, &s, &c);
        const double V = (double)series[(k * nports + p) * 2], I = (double)series[(k * nports + p) * 2 + 1];
        acc[0] += V * c, acc[1] += V * s, acc[2] += I * c, acc[3] += I * s;
    }
    __shared__ double red[4][256];
    for (int q = 0; q < 4; ++q) red[q][threadIdx.x] = acc[q];
    __syncthreads();
    for (int stride = blockDim.x / 2; stride > 0; stride >>= 1) {
        if (threadIdx.x < stride)
            for (int q = 0; q < 4; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + stride];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double sh, ch;
        sincos(w * 0.5 * dt, &sh, &ch);
        double* o = out + (long long)pf * 4;
        o[0] = red[0][0], o[1] = red[1][0];
        o[2] = red[2][0] * ch - red[3][0] * sh, o[3] = red[2][0] * sh + red[3][0] * ch;
    }
}

__global__ void finite_kernel(MonitorArgs m, unsigned* flag) {
    const long long total = (long long)m.nz * m.plane;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % m.pitch);
        if (x >= m.nx) continue;
        if (!isfinite(m.ex[i]) || !isfinite(m.ey[i]) || !isfinite(m.ez[i]) || !isfinite(m.bx[i]) ||
            !isfinite(m.by[i]) || !isfinite(m.bz[i])) {
            atomicOr(flag, 1u);
            return;
        }
    }
}

// Multi-frequency far-field DFT, per step: the co-located E and H (field_sampling.glsl:17-32) of
// every Huygens-box node into slot t of the time block, component-major: blk[(t * 6 + c) * P + i],
// P the points of all boxes, i = the box's first point + the node's index in its box. blockIdx.y is
// the box.
__global__ void __launch_bounds__(256) dft_sample_kernel(MonitorArgs m, const int* boxes, int points, float* blk,
                                                         int t) {
    __shared__ int sbox[kDftBoxInts];
    if (threadIdx.x < kDftBoxInts) sbox[threadIdx.x] = boxes[(size_t)blockIdx.y * kDftBoxInts + threadIdx.x];
    __syncthreads();
    const int local = blockIdx.x * blockDim.x + threadIdx.x;
    if (local >= sbox[14]) return;
    const int i = sbox[13] + local;
    int node[3];
    float n[3], w;
    ntff_point(sbox, local, node, n, w);
    float E[3], Hh[3];
    e_at_node(m, node[0], node[1], node[2], E[0], E[1], E[2]);
    b_at_node(m, node[0], node[1], node[2], Hh[0], Hh[1], Hh[2]);
    float* o = blk + (size_t)t * 6 * points + i;
    o[0] = E[0], o[(size_t)points] = E[1], o[2 * (size_t)points] = E[2];
    o[3 * (size_t)points] = Hh[0], o[4 * (size_t)points] = Hh[1], o[5 * (size_t)points] = Hh[2];
}

// Folds T samples of every column (component c of node i) into the FP64 sums:
//   X_f += e^{-i w_f t0} sum_k F(t0 + k dt) e^{-i w_f k dt},
// t0 = n0 dt for E and (n0 - 1/2) dt for H (B lags half a step). The block-relative twiddles
// W[f][k] = (cos w_f k dt, -sin w_f k dt) are FP32 (from FP64 on the host); the in-block sums are
// FP32 (<= 64 terms); the block phase e^{-i w_f t0} is evaluated in FP64 once per CTA and applied in
// FP32; the accumulation is FP64. X layout: [f][c][i][re, im]. The CUDA-core twin of the
// tensor-core fold (dft_tc.cu), which differs only in how the in-block sums are formed.
constexpr int kDftMaxT = 64;
__global__ void __launch_bounds__(128) dft_fold_kernel(const float* blk, int T, int points, int nf, const float2* W,
                                                       const double* omega, long long n0, double dt, double* X) {
    extern __shared__ float2 sW[];  // [nf][kDftMaxT], then the block phases [nf][E, H]
    float2* rot = sW + nf * kDftMaxT;
    for (int j = threadIdx.x; j < nf * kDftMaxT; j += blockDim.x) sW[j] = W[j];
    for (int j = threadIdx.x; j < 2 * nf; j += blockDim.x) {
        const double t0 = ((double)n0 - ((j & 1) ? 0.5 : 0.0)) * dt;
        double sn, cs;
        sincos(omega[j >> 1] * t0, &sn, &cs);
        rot[j] = make_float2((float)cs, (float)sn);
    }
    __syncthreads();
    const long long col = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (col >= 6ll * points) return;
    const int c = (int)(col / points), i = (int)(col % points), h = c >= 3 ? 1 : 0;
    float v[kDftMaxT];
#pragma unroll
    for (int k = 0; k < kDftMaxT; ++k) v[k] = k < T ? blk[(size_t)k * 6 * points + col] : 0.0f;
    double2* xo = reinterpret_cast<double2*>(X) + (size_t)c * points + i;  // + f * 6 * points
    const size_t fstride = (size_t)6 * points;
    constexpr int G = 4;  // frequencies per group: their X loads are issued before any store
    for (int f0 = 0; f0 < nf; f0 += G) {
        double2 acc[G];
#pragma unroll
        for (int g = 0; g < G; ++g)
            if (f0 + g < nf) acc[g] = xo[(size_t)(f0 + g) * fstride];
#pragma unroll
        for (int g = 0; g < G; ++g) {
            const int f = f0 + g;
            if (f >= nf) break;
            float re = 0.0f, im = 0.0f;
#pragma unroll
            for (int k = 0; k < kDftMaxT; ++k) {
                const float2 w = sW[f * kDftMaxT + k];
                re = re + w.x * v[k];
                im = im + w.y * v[k];
            }
            const float2 r = rot[2 * f + h];
            const float xr = re * r.x + im * r.y, xi = im * r.x - re * r.y;  // (re + i im)(cos - i sin)
            acc[g].x += (double)xr, acc[g].y += (double)xi;
            xo[(size_t)f * fstride] = acc[g];
        }
    }
}

// The sums of the boxes a stack compaction keeps, moved to their places in the shorter point list.
__global__ void dft_gather_kernel(const double2* x_old, int old_points, const int* map, int new_points,
                                  double2* x_new) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= new_points) return;
    const size_t fc = blockIdx.y;
    x_new[fc * new_points + j] = x_old[fc * old_points + map[j]];
}

// Stage-2 phasor layout of ntff_pattern.comp (PhasorPair, 8 float4 per node) from the DFT sums of
// one frequency, scaled by `scale` (2 / samples turns a sum into the amplitude of a steady tone).
__global__ void dft_to_phasor_kernel(const double* X, int points, int f, double scale, float4* ph) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= points) return;
    const double2* x = reinterpret_cast<const double2*>(X) + (size_t)f * 6 * points + i;
    double2 v[6];
    for (int c = 0; c < 6; ++c) v[c] = x[(size_t)c * points];
    float4* p = ph + 8 * (size_t)i;
    p[4] = make_float4((float)(v[0].x * scale), (float)(v[1].x * scale), (float)(v[2].x * scale), 0.0f);  // E re
    p[5] = make_float4((float)(v[0].y * scale), (float)(v[1].y * scale), (float)(v[2].y * scale), 0.0f);  // E im
    p[6] = make_float4((float)(v[3].x * scale), (float)(v[4].x * scale), (float)(v[5].x * scale), 0.0f);  // H re
    p[7] = make_float4((float)(v[3].y * scale), (float)(v[4].y * scale), (float)(v[5].y * scale), 0.0f);  // H im
}

__global__ void expf_kernel(const float* in, float* out, size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = emlab_expf(in[i]);
}

}  // namespace

void launch_ports(const MonitorArgs& m, const int4* ports, int n, float* phasors, float* series, long long rec,
                  const float4* rot, const float* blend, int k, cudaStream_t s) {
    ports_kernel<<<(n + 63) / 64, 64, 0, s>>>(m, ports, n, phasors, series, rec, rot, blend, k);
}

void launch_ntff(const MonitorArgs& m, const int* box, int points, float* phasors, const float4* rot,
                 const float* blend, int k, cudaStream_t s) {
    ntff_kernel<<<(points + kNtffThreads - 1) / kNtffThreads, kNtffThreads, 0, s>>>(
        m, box, points, reinterpret_cast<float4*>(phasors), rot, blend, k);
}

void launch_lines(const MonitorArgs& m, const int4* q, int nq, const int4* terms, const float* weights,
                  float* phasors, float* now, const float4* rot, const float* blend, int k, cudaStream_t s) {
    lines_kernel<<<(nq + 63) / 64, 64, 0, s>>>(m, q, nq, terms, weights, reinterpret_cast<float4*>(phasors), now, rot,
                                                blend, k);
}

void launch_probe_gather(const MonitorArgs& m, const int4* origins, int n, float4* out, const float*, const float*,
                         cudaStream_t s) {
    probe_kernel<<<(n * 54 + 63) / 64, 64, 0, s>>>(m, origins, n, out);
}

void launch_flux_plane(const MonitorArgs& m, int axis, int index, int rmin0, int rmin1, int rs0, int rs1,
                       float* partials, cudaStream_t s) {
    const dim3 grid((rs0 + 15) / 16, (rs1 + 15) / 16);
    flux_kernel<<<grid, dim3(16, 16), 0, s>>>(m, axis, index, rmin0, rmin1, rs0, rs1, partials);
}

void launch_ntff_pattern(const int* box, int points, const float* phasors, const float4* dirs, int first, int count,
                         int slices, float k, float4* partials, cudaStream_t s) {
    const dim3 grid((count + 127) / 128, slices);
    ntff_pattern_kernel<<<grid, 128, 0, s>>>(box, points, reinterpret_cast<const float4*>(phasors), dirs, first, count,
                                             slices, k, partials);
}

void launch_ntff_pattern_fast(const int* box, int points, const float* phasors, const float4* dirs, int first,
                              int count, int slices, float k, float4* partials, cudaStream_t s) {
    const dim3 grid((count + 255) / 256, slices);
    ntff_pattern_fast_kernel<<<grid, 128, 0, s>>>(box, points, PhasorSource{reinterpret_cast<const float4*>(phasors), k},
                                                  dirs, first, count, slices, partials);
}

void launch_ntff_spectra(const int* box, int first, int points, int total_points, const double* X, int nf,
                         const double* omega, double scale, const float4* dirs, int count, int slices,
                         float4* partials, cudaStream_t s) {
    const dim3 grid((count + 255) / 256, slices, nf);
    ntff_pattern_fast_kernel<<<grid, 128, 0, s>>>(box, points, DftSource{X, total_points, first, omega, scale}, dirs,
                                                  0, count, slices, partials);
}

void launch_ntff_reduce_multi(const float4* dirs, const float4* partials, int count, int slices, int nf, float* out,
                              cudaStream_t s) {
    ntff_reduce_kernel<<<dim3((count + 63) / 64, nf), 64, 0, s>>>(dirs, partials, 0, count, slices, out);
}

void launch_ntff_reduce(const float4* dirs, const float4* partials, int first, int count, int slices, float* out,
                        cudaStream_t s) {
    ntff_reduce_kernel<<<(count + 63) / 64, 64, 0, s>>>(dirs, partials, first, count, slices, out);
}

void launch_sweep_sums(const float* series, long long steps, int nports, double nu_lo, double nu_hi, int points,
                       double dt, double* out, cudaStream_t s) {
    sweep_kernel<<<nports * points, 256, 0, s>>>(series, steps, nports, nu_lo, nu_hi, points, dt, out);
}

// Ring-down residual of every port (PortMonitor::evaluateSweep, Ports.cpp:206-213): the largest |V|
// of the last max(n / 20, 1) recorded steps over the largest |V| of all n (1 when there is no
// signal). One block per port; |V| maxima are exact in any order, so the result equals the host's.
__global__ void __launch_bounds__(256) residual_kernel(const float* series, long long steps, int nports, double* out) {
    __shared__ float s_peak[256], s_late[256];
    const int p = blockIdx.x;
    const long long tail = steps / 20 > 1 ? steps / 20 : 1, late_from = steps - tail;
    float peak = 0.0f, late = 0.0f;
    for (long long k = threadIdx.x; k < steps; k += blockDim.x) {
        const float v = fabsf(series[(k * nports + p) * 2]);
        peak = fmaxf(peak, v);
        if (k >= late_from) late = fmaxf(late, v);
    }
    s_peak[threadIdx.x] = peak, s_late[threadIdx.x] = late;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            s_peak[threadIdx.x] = fmaxf(s_peak[threadIdx.x], s_peak[threadIdx.x + w]);
            s_late[threadIdx.x] = fmaxf(s_late[threadIdx.x], s_late[threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) out[p] = s_peak[0] > 0.0f ? (double)s_late[0] / (double)s_peak[0] : 1.0;
}

void launch_port_residuals(const float* series, long long steps, int nports, double* out, cudaStream_t s) {
    residual_kernel<<<nports, 256, 0, s>>>(series, steps, nports, out);
}

void launch_check_finite(const MonitorArgs& m, unsigned* flag, cudaStream_t s) {
    finite_kernel<<<152 * 8, 256, 0, s>>>(m, flag);
}

void launch_dft_sample(const MonitorArgs& m, const int* boxes, int nbox, int box_max, int points, float* blk, int t,
                       cudaStream_t s) {
    dft_sample_kernel<<<dim3((box_max + 255) / 256, nbox), 256, 0, s>>>(m, boxes, points, blk, t);
}

void launch_dft_gather(const double* x_old, int old_points, const int* map, int new_points, int nf, double* x_new,
                       cudaStream_t s) {
    dft_gather_kernel<<<dim3((new_points + 255) / 256, nf * 6), 256, 0, s>>>(
        reinterpret_cast<const double2*>(x_old), old_points, map, new_points, reinterpret_cast<double2*>(x_new));
}

void launch_dft_fold(const float* blk, int T, int points, int nf, const float2* W, const double* omega, long long n0,
                     double dt, double* X, cudaStream_t s) {
    const long long cols = 6ll * points;
    const size_t smem = (size_t)(nf * kDftMaxT + 2 * nf) * sizeof(float2);
    static size_t smem_set = 48 * 1024;
    if (smem > smem_set &&
        cudaFuncSetAttribute(dft_fold_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess)
        smem_set = smem;
    dft_fold_kernel<<<(unsigned)((cols + 127) / 128), 128, smem, s>>>(blk, T, points, nf, W, omega, n0, dt, X);
}

void launch_dft_to_phasor(const double* X, int points, int f, double scale, float* ph, cudaStream_t s) {
    dft_to_phasor_kernel<<<(points + 255) / 256, 256, 0, s>>>(X, points, f, scale, reinterpret_cast<float4*>(ph));
}

void launch_debug_expf(const float* in, float* out, size_t n, cudaStream_t s) {
    expf_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, out, n);
}

}  // namespace emlab
