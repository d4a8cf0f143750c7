// render.cu - headless volume rendering of the fields (the reference's screenshot path).
//
// One thread per pixel evaluates the emission/absorption ray march of shaders/raymarch.frag:
// the primary ray through the inverse view-projection, the slab test against the cutaway box,
// a jittered start (interleaved gradient noise), and front-to-back compositing of |E| (cyan),
// |B| (magenta), |E x B| or a signed E component, with metals, dielectrics and lossy media drawn
// as shaded surfaces from the cell sigma / eps_r gradients; then the tone curve, gamma and
// dither. Field samples are trilinear with clamp-to-edge over texel centres, like a linear
// sampler3D on the reference's RGBA32F field textures (rgb = E or B at the texel, alpha = cell
// sigma or eps_r). Arithmetic is FP32 in the shader's order (compiled without contraction);
// exp() is emlab_expf as everywhere else, so only pow() and the hardware's texture-filter
// precision separate this from a GL driver's result.
#include "emlab_internal.h"

namespace emlab {
namespace {

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
__device__ __forceinline__ float dot3(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ float len3(V3 a) { return sqrtf(dot3(a, a)); }
__device__ __forceinline__ V3 norm3(V3 a) {
    const float l = len3(a);
    return {a.x / l, a.y / l, a.z / l};
}
__device__ __forceinline__ V3 cross3(V3 a, V3 b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
__device__ __forceinline__ V3 mix3(V3 a, V3 b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float smooth(float e0, float e1, float x) {
    const float t = clampf((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
__device__ __forceinline__ float fractf(float x) { return x - floorf(x); }
__device__ __forceinline__ float ign(float px, float py) {  // interleavedGradientNoise
    return fractf(52.9829189f * fractf(px * 0.06711056f + py * 0.00583715f));
}
__device__ __forceinline__ float response(float x) {
    const float x2 = x * x;
    return x2 / (1.0f + x2);
}

struct Volume {
    const float* f[6];  // Ex, Ey, Ez, Bx, By, Bz
    const float* sigma; // cell sigma (E texture alpha), may be null
    const float* eps;   // cell eps_r (B texture alpha), may be null
    int nx, ny, nz, pitch;
    long long plane;
};

// Trilinear over texel centres with clamp-to-edge: channels 0..2 of field (E or B), 3 = alpha.
__device__ void sample(const Volume& v, V3 uvw, bool bfield, float out[4]) {
    const float px = uvw.x * (float)v.nx - 0.5f, py = uvw.y * (float)v.ny - 0.5f, pz = uvw.z * (float)v.nz - 0.5f;
    const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
    const float ax = px - fx, ay = py - fy, az = pz - fz;
    const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    out[0] = out[1] = out[2] = out[3] = 0.0f;
    const float* alpha = bfield ? v.eps : v.sigma;
    const int c0 = bfield ? 3 : 0;
    for (int dz = 0; dz <= 1; ++dz)
        for (int dy = 0; dy <= 1; ++dy)
            for (int dx = 0; dx <= 1; ++dx) {
                const float w = (dx ? ax : 1.0f - ax) * (dy ? ay : 1.0f - ay) * (dz ? az : 1.0f - az);
                const int x = min(max(ix + dx, 0), v.nx - 1), y = min(max(iy + dy, 0), v.ny - 1),
                          z = min(max(iz + dz, 0), v.nz - 1);
                const long long i = (long long)z * v.plane + (long long)y * v.pitch + x;
                const long long ci = ((long long)z * v.ny + y) * v.nx + x;
                out[0] += w * __ldg(v.f[c0] + i);
                out[1] += w * __ldg(v.f[c0 + 1] + i);
                out[2] += w * __ldg(v.f[c0 + 2] + i);
                out[3] += w * (alpha ? __ldg(alpha + ci) : (bfield ? 1.0f : 0.0f));
            }
}

__device__ float alpha_at(const Volume& v, V3 uvw, bool bfield) {
    float s[4];
    sample(v, uvw, bfield, s);
    return s[3];
}

__device__ V3 material_normal(const Volume& v, V3 uvw, bool metal, V3 rd) {
    const V3 h = v3(1.0f / (float)v.nx, 1.0f / (float)v.ny, 1.0f / (float)v.nz);
    const bool b = !metal;
    const V3 g = v3(alpha_at(v, uvw + v3(h.x, 0, 0), b) - alpha_at(v, uvw - v3(h.x, 0, 0), b),
                    alpha_at(v, uvw + v3(0, h.y, 0), b) - alpha_at(v, uvw - v3(0, h.y, 0), b),
                    alpha_at(v, uvw + v3(0, 0, h.z), b) - alpha_at(v, uvw - v3(0, 0, h.z), b));
    const float l = len3(g);
    return l > 1e-5f ? v3(-g.x / l, -g.y / l, -g.z / l) : v3(-rd.x, -rd.y, -rd.z);
}

__device__ V3 shade(V3 n, V3 rd, V3 albedo, float specular) {
    const V3 key = norm3(v3(0.45f, -0.35f, 0.82f));
    const V3 vv = v3(-rd.x, -rd.y, -rd.z);
    const float ndl = fmaxf(dot3(n, key), 0.0f);
    const float head = fmaxf(dot3(n, vv), 0.0f);
    const V3 hv = norm3(key + vv);
    const float spec = powf(fmaxf(dot3(n, hv), 0.0f), 48.0f) * specular;
    const float rim = powf(1.0f - head, 3.0f);
    const float k = (0.18f + 0.55f * ndl) + 0.30f * head;
    return (albedo * k + v3(spec, spec, spec)) + v3(0.35f, 0.45f, 0.6f) * rim;
}

__device__ void finalize(V3 c, float exposure, float fx, float fy, unsigned char* out) {
    const float d = (ign(fx + 17.0f, fy + 17.0f) - 0.5f) / 255.0f;
    const float ch[3] = {c.x, c.y, c.z};
    for (int k = 0; k < 3; ++k) {
        float x = 1.0f - emlab_expf(-ch[k] * exposure);
        x = powf(x, 1.0f / 2.2f) + d;
        out[k] = (unsigned char)__float2int_rn(clampf(x, 0.0f, 1.0f) * 255.0f);
    }
    out[3] = 255;
}

__global__ void __launch_bounds__(128) raymarch_kernel(Volume v, emlab_render_params p, unsigned char* img) {
    const int px = blockIdx.x * 16 + (threadIdx.x & 15), py = blockIdx.y * 8 + (threadIdx.x >> 4);
    if (px >= p.width || py >= p.height) return;
    const float fx = (float)px + 0.5f, fy = (float)py + 0.5f;  // gl_FragCoord (origin bottom-left)
    const float nx = fx / (float)p.width * 2.0f - 1.0f, ny = fy / (float)p.height * 2.0f - 1.0f;
    const float* m = p.inv_view_proj;  // column-major
    const float hx = ((m[0] * nx + m[4] * ny) + m[8]) + m[12], hy = ((m[1] * nx + m[5] * ny) + m[9]) + m[13],
                hz = ((m[2] * nx + m[6] * ny) + m[10]) + m[14], hw = ((m[3] * nx + m[7] * ny) + m[11]) + m[15];
    const V3 ro = v3(p.cam_pos[0], p.cam_pos[1], p.cam_pos[2]);
    const V3 rd = norm3(v3(hx / hw, hy / hw, hz / hw) - ro);
    unsigned char* out = img + 4 * ((size_t)py * p.width + px);

    const float hgt = clampf(rd.z * 0.5f + 0.5f, 0.0f, 1.0f);
    const V3 bg = mix3(v3(0.004f, 0.006f, 0.014f), v3(0.018f, 0.028f, 0.060f), hgt);
    // slab test
    const V3 srd = v3(fabsf(rd.x) < 1e-8f ? 1e-8f : rd.x, fabsf(rd.y) < 1e-8f ? 1e-8f : rd.y,
                      fabsf(rd.z) < 1e-8f ? 1e-8f : rd.z);
    const V3 inv = v3(1.0f / srd.x, 1.0f / srd.y, 1.0f / srd.z);
    const V3 t0 = (v3(p.clip_min[0], p.clip_min[1], p.clip_min[2]) - ro) * inv;
    const V3 t1 = (v3(p.clip_max[0], p.clip_max[1], p.clip_max[2]) - ro) * inv;
    float tin = fmaxf(fmaxf(fminf(t0.x, t1.x), fminf(t0.y, t1.y)), fminf(t0.z, t1.z));
    const float tout = fminf(fminf(fmaxf(t0.x, t1.x), fmaxf(t0.y, t1.y)), fmaxf(t0.z, t1.z));
    tin = fmaxf(tin, 0.0f);
    if (tin >= tout) {
        finalize(bg, p.exposure, fx, fy, out);
        return;
    }
    const V3 vmin = v3(p.vol_min[0], p.vol_min[1], p.vol_min[2]);
    const V3 vsize = v3(p.vol_size[0], p.vol_size[1], p.vol_size[2]);
    const float voxel = vsize.x / (float)v.nx;
    const float ds = fmaxf(p.step_voxels, 0.05f) * voxel;
    const float step_vox = ds / voxel;
    float t = tin + ds * ign(fx, fy);
    const int steps = min((int)((tout - t) / ds) + 1, 4096);
    V3 accum = v3(0, 0, 0);
    float alpha = 0.0f;
    for (int i = 0; i < steps; ++i, t += ds) {
        const V3 uvw = ((ro + rd * t) - vmin) / vsize;
        float e[4], b[4];
        sample(v, uvw, false, e);
        sample(v, uvw, true, b);
        V3 emission = v3(0, 0, 0);
        float ext = 0.0f;
        if (p.mode == 0 || p.mode == 1) {
            const float iE = response(len3(v3(e[0], e[1], e[2])) * p.gain_e);
            V3 col = mix3(v3(0.02f, 0.22f, 1.0f), v3(0.05f, 0.95f, 1.0f), iE);
            col = mix3(col, v3(0.8f, 1.0f, 1.0f), smooth(0.8f, 1.0f, iE));
            emission = emission + col * (iE * iE * 2.0f);
            ext += iE;
        }
        if (p.mode == 0 || p.mode == 2) {
            const float iB = response(len3(v3(b[0], b[1], b[2])) * p.gain_b);
            V3 col = mix3(v3(1.0f, 0.03f, 0.10f), v3(1.0f, 0.10f, 0.62f), iB);
            col = mix3(col, v3(1.0f, 0.85f, 1.0f), smooth(0.8f, 1.0f, iB));
            emission = emission + col * (iB * iB * 2.0f);
            ext += iB;
        }
        if (p.mode == 3) {
            const float iS = response(len3(cross3(v3(e[0], e[1], e[2]), v3(b[0], b[1], b[2]))) * p.gain_e * p.gain_b);
            V3 col = mix3(v3(1.0f, 0.35f, 0.02f), v3(1.0f, 0.85f, 0.25f), iS);
            col = mix3(col, v3(1.0f, 1.0f, 0.85f), smooth(0.8f, 1.0f, iS));
            emission = emission + col * (iS * iS * 2.0f);
            ext += iS;
        }
        if (p.mode == 4) {
            const float val = e[min(max(p.signed_axis, 0), 2)] * p.gain_e;
            const float iV = response(val);
            const V3 col = val >= 0.0f ? mix3(v3(0.02f, 0.3f, 1.0f), v3(0.1f, 1.0f, 1.0f), iV)
                                       : mix3(v3(0.9f, 0.15f, 0.02f), v3(1.0f, 0.65f, 0.1f), iV);
            emission = emission + col * (iV * iV * 2.0f);
            ext += iV;
        }
        emission = emission * (0.045f * p.emission);
        ext *= 0.022f * p.density;
        const float metal = smooth(1.0f, 20.0f, e[3]);
        const float glass = clampf((b[3] - 1.0f) * 0.5f, 0.0f, 1.0f);
        const float absorber = smooth(0.02f, 1.0f, e[3]) * (1.0f - metal);
        V3 surface = v3(0, 0, 0);
        float mat_ext = 0.0f;
        if ((metal + glass) + absorber > 0.01f) {
            const V3 n = material_normal(v, uvw, metal >= glass, rd);
            const V3 mc = shade(n, rd, v3(0.50f, 0.53f, 0.58f), 0.9f);
            const V3 gc = shade(n, rd, v3(0.30f, 0.65f, 0.70f), 0.6f);
            const V3 lc = shade(n, rd, v3(0.35f, 0.22f, 0.12f), 0.1f);
            const float wM = metal * p.material_opacity;
            const float wG = glass * p.material_opacity * 0.02f;
            const float wA = absorber * p.material_opacity * 0.4f;
            mat_ext = (wM + wG) + wA;
            const float dn = fmaxf(mat_ext, 1e-6f);
            surface = ((mc * wM + gc * wG) + lc * wA) / v3(dn, dn, dn);
        }
        const float a_field = 1.0f - emlab_expf(-ext * step_vox);
        const float a_mat = 1.0f - emlab_expf(-mat_ext * step_vox);
        const float tr = 1.0f - alpha;
        accum = accum + ((emission * step_vox) * (1.0f - a_mat) + surface * a_mat) * tr;
        alpha += tr * (1.0f - (1.0f - a_field) * (1.0f - a_mat));
        if (alpha > 0.995f) break;
    }
    finalize(accum + bg * (1.0f - alpha), p.exposure, fx, fy, out);
}

}  // namespace

void launch_raymarch(const MonitorArgs& m, const float* sigma, const float* eps, const emlab_render_params& p,
                     unsigned char* img, cudaStream_t s) {
    Volume v;
    v.f[0] = m.ex, v.f[1] = m.ey, v.f[2] = m.ez, v.f[3] = m.bx, v.f[4] = m.by, v.f[5] = m.bz;
    v.sigma = sigma, v.eps = eps;
    v.nx = m.nx, v.ny = m.ny, v.nz = m.nz, v.pitch = m.pitch, v.plane = m.plane;
    const dim3 grid((p.width + 15) / 16, (p.height + 7) / 8);
    raymarch_kernel<<<grid, 128, 0, s>>>(v, p, img);
}

}  // namespace emlab
