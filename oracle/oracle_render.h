/* oracle_render.h - CPU restatement of the reference's volume pass (test infrastructure).
 *
 * Restates shaders/raymarch.frag (primary ray, slab test, jittered start, front-to-back
 * emission/absorption compositing, material shading, tone curve, gamma, dither) in the GLSL
 * evaluation order, over the reference's two RGBA32F field textures (rgb = E or B, alpha = cell
 * sigma or eps_r), with the sampler3D's linear filter and clamp-to-edge restated as trilinear
 * weights over texel centres, and vNdc / gl_FragCoord taken at pixel centres (origin bottom-left).
 * The uniforms are emlab_render_params, set as src/VolumeRenderer.cpp:89-112 sets them.
 * Included by emlab_oracle.c; compiled with -ffp-contract=off. exp() is emlab_expf; pow() is libm
 * powf (GLSL leaves its precision to the implementation).
 */
#ifndef ORACLE_RENDER_H
#define ORACLE_RENDER_H

typedef struct {
    float x, y, z;
} ov3;

static ov3 ov(float x, float y, float z) {
    ov3 r = {x, y, z};
    return r;
}
static ov3 ov_add(ov3 a, ov3 b) { return ov(a.x + b.x, a.y + b.y, a.z + b.z); }
static ov3 ov_sub(ov3 a, ov3 b) { return ov(a.x - b.x, a.y - b.y, a.z - b.z); }
static ov3 ov_mul(ov3 a, float s) { return ov(a.x * s, a.y * s, a.z * s); }
static float ov_dot(ov3 a, ov3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static float ov_len(ov3 a) { return sqrtf(ov_dot(a, a)); }
static ov3 ov_norm(ov3 a) {
    const float l = ov_len(a);
    return ov(a.x / l, a.y / l, a.z / l);
}
static ov3 ov_mix(ov3 a, ov3 b, float t) { return ov_add(ov_mul(a, 1.0f - t), ov_mul(b, t)); }
static float o_max(float a, float b) { return a < b ? b : a; } /* GLSL max(x, y): y if x < y */
static float o_min(float a, float b) { return b < a ? b : a; }
static float o_clamp(float x, float lo, float hi) { return o_min(o_max(x, lo), hi); }
static float o_smooth(float e0, float e1, float x) {
    const float t = o_clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
static float o_fract(float x) { return x - floorf(x); }
/* interleavedGradientNoise (raymarch.frag:53-55) */
static float o_ign(float px, float py) { return o_fract(52.9829189f * o_fract(px * 0.06711056f + py * 0.00583715f)); }
static float o_response(float x) {
    const float x2 = x * x;
    return x2 / (1.0f + x2);
}

typedef struct {
    const float* rgba;
    int nx, ny, nz;
} OTex;

/* texture(sampler3D, uvw) with GL_LINEAR and GL_CLAMP_TO_EDGE: the eight texels around
 * uvw * size - 0.5, weights (1 - a or a) per axis multiplied x, y, z, accumulated z-, y-, x-major. */
static void o_texture(const OTex* t, ov3 uvw, float out[4]) {
    const float px = uvw.x * (float)t->nx - 0.5f, py = uvw.y * (float)t->ny - 0.5f, pz = uvw.z * (float)t->nz - 0.5f;
    const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
    const float ax = px - fx, ay = py - fy, az = pz - fz;
    const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    out[0] = out[1] = out[2] = out[3] = 0.0f;
    for (int dz = 0; dz <= 1; ++dz)
        for (int dy = 0; dy <= 1; ++dy)
            for (int dx = 0; dx <= 1; ++dx) {
                const float w = (dx ? ax : 1.0f - ax) * (dy ? ay : 1.0f - ay) * (dz ? az : 1.0f - az);
                int x = ix + dx, y = iy + dy, z = iz + dz;
                x = x < 0 ? 0 : (x > t->nx - 1 ? t->nx - 1 : x);
                y = y < 0 ? 0 : (y > t->ny - 1 ? t->ny - 1 : y);
                z = z < 0 ? 0 : (z > t->nz - 1 ? t->nz - 1 : z);
                const float* q = t->rgba + 4 * (((long long)z * t->ny + y) * t->nx + x);
                for (int k = 0; k < 4; ++k) out[k] = out[k] + w * q[k];
            }
}

static float o_alpha(const OTex* t, ov3 uvw) {
    float s[4];
    o_texture(t, uvw, s);
    return s[3];
}

/* materialNormal (raymarch.frag:68-83) */
static ov3 o_material_normal(const OTex* et, const OTex* bt, ov3 uvw, int metal, ov3 rd) {
    const ov3 h = ov(1.0f / (float)et->nx, 1.0f / (float)et->ny, 1.0f / (float)et->nz);
    const OTex* t = metal ? et : bt;
    const ov3 g = ov(o_alpha(t, ov_add(uvw, ov(h.x, 0, 0))) - o_alpha(t, ov_sub(uvw, ov(h.x, 0, 0))),
                     o_alpha(t, ov_add(uvw, ov(0, h.y, 0))) - o_alpha(t, ov_sub(uvw, ov(0, h.y, 0))),
                     o_alpha(t, ov_add(uvw, ov(0, 0, h.z))) - o_alpha(t, ov_sub(uvw, ov(0, 0, h.z))));
    const float len = ov_len(g);
    return len > 1e-5f ? ov(-g.x / len, -g.y / len, -g.z / len) : ov(-rd.x, -rd.y, -rd.z);
}

/* shadeSurface (raymarch.frag:85-94) */
static ov3 o_shade(ov3 n, ov3 rd, ov3 albedo, float specular) {
    const ov3 key = ov_norm(ov(0.45f, -0.35f, 0.82f));
    const ov3 v = ov(-rd.x, -rd.y, -rd.z);
    const float ndl = o_max(ov_dot(n, key), 0.0f);
    const float head = o_max(ov_dot(n, v), 0.0f);
    const ov3 hv = ov_norm(ov_add(key, v));
    const float spec = powf(o_max(ov_dot(n, hv), 0.0f), 48.0f) * specular;
    const float rim = powf(1.0f - head, 3.0f);
    const ov3 base = ov_mul(albedo, 0.18f + 0.55f * ndl + 0.30f * head);
    return ov_add(ov(base.x + spec, base.y + spec, base.z + spec), ov_mul(ov(0.35f, 0.45f, 0.6f), rim));
}

/* finalize (raymarch.frag:96-101), then the RGBA8 framebuffer's unorm conversion (round to nearest). */
static void o_finalize(ov3 c, float exposure, float fx, float fy, unsigned char* out) {
    const float d = (o_ign(fx + 17.0f, fy + 17.0f) - 0.5f) / 255.0f;
    const float ch[3] = {c.x, c.y, c.z};
    for (int k = 0; k < 3; ++k) {
        float x = 1.0f - emlab_expf(-ch[k] * exposure);
        x = powf(x, 1.0f / 2.2f) + d;
        out[k] = (unsigned char)lrintf(o_clamp(x, 0.0f, 1.0f) * 255.0f);
    }
    out[3] = 255;
}

/* main (raymarch.frag:103-197) for the pixel whose centre is (fx, fy). */
static void o_raymarch_pixel(const OTex* et, const OTex* bt, const emlab_render_params* p, float fx, float fy,
                             unsigned char* out) {
    const float ndx = fx / (float)p->width * 2.0f - 1.0f, ndy = fy / (float)p->height * 2.0f - 1.0f;
    const float* m = p->inv_view_proj; /* column-major mat4 */
    const float hx = m[0] * ndx + m[4] * ndy + m[8] * 1.0f + m[12] * 1.0f;
    const float hy = m[1] * ndx + m[5] * ndy + m[9] * 1.0f + m[13] * 1.0f;
    const float hz = m[2] * ndx + m[6] * ndy + m[10] * 1.0f + m[14] * 1.0f;
    const float hw = m[3] * ndx + m[7] * ndy + m[11] * 1.0f + m[15] * 1.0f;
    const ov3 ro = ov(p->cam_pos[0], p->cam_pos[1], p->cam_pos[2]);
    const ov3 rd = ov_norm(ov_sub(ov(hx / hw, hy / hw, hz / hw), ro));

    const float hb = o_clamp(rd.z * 0.5f + 0.5f, 0.0f, 1.0f);
    const ov3 bg = ov_mix(ov(0.004f, 0.006f, 0.014f), ov(0.018f, 0.028f, 0.060f), hb);

    /* intersectBox */
    const ov3 srd = ov(fabsf(rd.x) < 1e-8f ? 1e-8f : rd.x, fabsf(rd.y) < 1e-8f ? 1e-8f : rd.y,
                       fabsf(rd.z) < 1e-8f ? 1e-8f : rd.z);
    const ov3 inv = ov(1.0f / srd.x, 1.0f / srd.y, 1.0f / srd.z);
    const ov3 c0 = ov(p->clip_min[0], p->clip_min[1], p->clip_min[2]);
    const ov3 c1 = ov(p->clip_max[0], p->clip_max[1], p->clip_max[2]);
    const ov3 t0 = ov((c0.x - ro.x) * inv.x, (c0.y - ro.y) * inv.y, (c0.z - ro.z) * inv.z);
    const ov3 t1 = ov((c1.x - ro.x) * inv.x, (c1.y - ro.y) * inv.y, (c1.z - ro.z) * inv.z);
    const ov3 tmin = ov(o_min(t0.x, t1.x), o_min(t0.y, t1.y), o_min(t0.z, t1.z));
    const ov3 tmax = ov(o_max(t0.x, t1.x), o_max(t0.y, t1.y), o_max(t0.z, t1.z));
    float hit_x = o_max(o_max(tmin.x, tmin.y), tmin.z);
    const float hit_y = o_min(o_min(tmax.x, tmax.y), tmax.z);
    hit_x = o_max(hit_x, 0.0f);
    if (hit_x >= hit_y) {
        o_finalize(bg, p->exposure, fx, fy, out);
        return;
    }

    const ov3 vmin = ov(p->vol_min[0], p->vol_min[1], p->vol_min[2]);
    const ov3 vsize = ov(p->vol_size[0], p->vol_size[1], p->vol_size[2]);
    const float voxel = vsize.x / (float)et->nx;
    const float ds = o_max(p->step_voxels, 0.05f) * voxel;
    const float step_vox = ds / voxel;
    float t = hit_x + ds * o_ign(fx, fy);
    int steps = (int)((hit_y - t) / ds) + 1;
    if (steps > 4096) steps = 4096;
    const int axis = p->signed_axis < 0 ? 0 : (p->signed_axis > 2 ? 2 : p->signed_axis);

    ov3 accum = ov(0, 0, 0);
    float alpha = 0.0f;
    for (int i = 0; i < steps; ++i, t += ds) {
        const ov3 pos = ov_add(ro, ov_mul(rd, t));
        const ov3 uvw = ov((pos.x - vmin.x) / vsize.x, (pos.y - vmin.y) / vsize.y, (pos.z - vmin.z) / vsize.z);
        float e[4], b[4];
        o_texture(et, uvw, e);
        o_texture(bt, uvw, b);
        ov3 emission = ov(0, 0, 0);
        float ext = 0.0f;
        if (p->mode == 0 || p->mode == 1) {
            const float iE = o_response(ov_len(ov(e[0], e[1], e[2])) * p->gain_e);
            ov3 col = ov_mix(ov(0.02f, 0.22f, 1.0f), ov(0.05f, 0.95f, 1.0f), iE);
            col = ov_mix(col, ov(0.8f, 1.0f, 1.0f), o_smooth(0.8f, 1.0f, iE));
            emission = ov_add(emission, ov_mul(col, iE * iE * 2.0f));
            ext += iE;
        }
        if (p->mode == 0 || p->mode == 2) {
            const float iB = o_response(ov_len(ov(b[0], b[1], b[2])) * p->gain_b);
            ov3 col = ov_mix(ov(1.0f, 0.03f, 0.10f), ov(1.0f, 0.10f, 0.62f), iB);
            col = ov_mix(col, ov(1.0f, 0.85f, 1.0f), o_smooth(0.8f, 1.0f, iB));
            emission = ov_add(emission, ov_mul(col, iB * iB * 2.0f));
            ext += iB;
        }
        if (p->mode == 3) {
            const ov3 s = ov(e[1] * b[2] - b[1] * e[2], e[2] * b[0] - b[2] * e[0], e[0] * b[1] - b[0] * e[1]);
            const float iS = o_response(ov_len(s) * p->gain_e * p->gain_b);
            ov3 col = ov_mix(ov(1.0f, 0.35f, 0.02f), ov(1.0f, 0.85f, 0.25f), iS);
            col = ov_mix(col, ov(1.0f, 1.0f, 0.85f), o_smooth(0.8f, 1.0f, iS));
            emission = ov_add(emission, ov_mul(col, iS * iS * 2.0f));
            ext += iS;
        }
        if (p->mode == 4) {
            const float v = e[axis] * p->gain_e;
            const float iV = o_response(v);
            const ov3 col = v >= 0.0f ? ov_mix(ov(0.02f, 0.3f, 1.0f), ov(0.1f, 1.0f, 1.0f), iV)
                                      : ov_mix(ov(0.9f, 0.15f, 0.02f), ov(1.0f, 0.65f, 0.1f), iV);
            emission = ov_add(emission, ov_mul(col, iV * iV * 2.0f));
            ext += iV;
        }
        emission = ov_mul(emission, 0.045f * p->emission);
        ext *= 0.022f * p->density;

        const float metal = o_smooth(1.0f, 20.0f, e[3]);
        const float glass = o_clamp((b[3] - 1.0f) * 0.5f, 0.0f, 1.0f);
        const float absorber = o_smooth(0.02f, 1.0f, e[3]) * (1.0f - metal);
        ov3 surface = ov(0, 0, 0);
        float mat_ext = 0.0f;
        if (metal + glass + absorber > 0.01f) {
            const ov3 n = o_material_normal(et, bt, uvw, metal >= glass, rd);
            const ov3 mc = o_shade(n, rd, ov(0.50f, 0.53f, 0.58f), 0.9f);
            const ov3 gc = o_shade(n, rd, ov(0.30f, 0.65f, 0.70f), 0.6f);
            const ov3 lc = o_shade(n, rd, ov(0.35f, 0.22f, 0.12f), 0.1f);
            const float wM = metal * p->material_opacity;
            const float wG = glass * p->material_opacity * 0.02f;
            const float wA = absorber * p->material_opacity * 0.4f;
            mat_ext = wM + wG + wA;
            const ov3 num = ov_add(ov_add(ov_mul(mc, wM), ov_mul(gc, wG)), ov_mul(lc, wA));
            const float dn = o_max(mat_ext, 1e-6f);
            surface = ov(num.x / dn, num.y / dn, num.z / dn);
        }
        const float a_field = 1.0f - emlab_expf(-ext * step_vox);
        const float a_mat = 1.0f - emlab_expf(-mat_ext * step_vox);
        const float tr = 1.0f - alpha;
        const ov3 inc = ov_add(ov_mul(ov_mul(emission, step_vox), 1.0f - a_mat), ov_mul(surface, a_mat));
        accum = ov_add(accum, ov(tr * inc.x, tr * inc.y, tr * inc.z));
        alpha += tr * (1.0f - (1.0f - a_field) * (1.0f - a_mat));
        if (alpha > 0.995f) break;
    }
    const float rest = 1.0f - alpha;
    o_finalize(ov_add(accum, ov(rest * bg.x, rest * bg.y, rest * bg.z)), p->exposure, fx, fy, out);
}

/* One frame: rgba (height rows of width RGBA8 pixels, bottom row first) from the two RGBA32F
 * textures of an nx x ny x nz grid (x fastest). */
int oracle_render(const float* e_rgba, const float* b_rgba, int nx, int ny, int nz, const emlab_render_params* p,
                  unsigned char* rgba) {
    if (!e_rgba || !b_rgba || !p || !rgba || nx <= 0 || ny <= 0 || nz <= 0 || p->width <= 0 || p->height <= 0 ||
        !isfinite(p->step_voxels))
        return -1;
    const OTex et = {e_rgba, nx, ny, nz}, bt = {b_rgba, nx, ny, nz};
    emlab_render_params q = *p; /* VolumeRenderer::render's clamps (src/VolumeRenderer.cpp:100, 111) */
    q.step_voxels = o_clamp(q.step_voxels, 0.1f, 4.0f);
    q.signed_axis = q.signed_axis < 0 ? 0 : (q.signed_axis > 2 ? 2 : q.signed_axis);
    p = &q;
    const int w = p->width, h = p->height;
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
            o_raymarch_pixel(&et, &bt, p, (float)x + 0.5f, (float)y + 0.5f, rgba + 4 * ((size_t)y * w + x));
    return 0;
}

#endif
