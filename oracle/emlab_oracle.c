/* emlab_oracle.c - CPU restatement of EM_Lab's FDTD time-stepping path (test infrastructure).
 *
 * This is the checker, never the product: only tests/, __graft_entry__.smoke() and the CPU-baseline
 * leg of bench.py load it. It restates, operation for operation in the GLSL evaluation order, the
 * reference's solver shaders (shaders/common.glsl, update_B.comp, update_E.comp, apply_sources.comp),
 * its monitors (port_accumulate.comp, ntff_accumulate.comp, ntff_pattern.comp, ntff_reduce.comp,
 * field_sampling.glsl, poynting_flux.comp, probe_gather.comp, line_accumulate.comp) and the host
 * set-up that feeds them (src/SimulationGrid.cpp: configure, uploadMaterials, setSources,
 * SourceDesc::signal, step; src/Ports.cpp; src/FarField.cpp; src/FieldAnalyzer.cpp).
 *
 * Two instantiations: *_f32 (FP32, the parity oracle; exp() is emlab_expf, or libm expf when
 * created with use_libm = 1) and *_f64 (FP64, the error floor; libm exp). Build with
 * -ffp-contract=off so that no multiply-add is fused; OpenMP parallelises the cell loops (each
 * cell's result does not depend on the thread count).
 *
 * oracle_render.h restates the volume pass of the screenshot path (shaders/raymarch.frag).
 *
 * Pinning: oracle/build_ref.py compiles the reference's own shader files (from the reference tree)
 * as C++ through a GLSL shim into oracle/_ref; tests/test_oracle_ref.py checks this restatement
 * against them bit for bit, and tests/golden/ holds fixtures produced by that build.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../em_lab_gb300/csrc/emlab_math.h"
#include "../include/emlab.h"

#ifdef _OPENMP
#include <omp.h>
#endif

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

float oracle_expf(float x) { return emlab_expf(x); }
uint16_t oracle_float_to_half(float x) { return emlab_float_to_half(x); }
float oracle_half_to_float(uint16_t h) { return emlab_half_to_float(h); }

/* SimulationGrid::configure clamps (SimulationGrid.cpp:149-156) */
void oracle_clamp_config(emlab_grid_config* c) {
    c->pml_thickness = c->pml_thickness < 0 ? 0 : (c->pml_thickness > 64 ? 64 : c->pml_thickness);
    const int min_size = 2 * c->pml_thickness + 8;
    if (c->nx < min_size) c->nx = min_size;
    if (c->ny < min_size) c->ny = min_size;
    if (c->nz < min_size) c->nz = min_size;
    const float max_courant = 0.99f / 1.7320508f;
    c->courant = c->courant < 0.05f ? 0.05f : (c->courant > max_courant ? max_courant : c->courant);
    c->pml_sigma_max = c->pml_sigma_max > 0.0f ? c->pml_sigma_max : 0.0f;
    c->pml_grading = c->pml_grading < 0.25f ? 0.25f : (c->pml_grading > 12.0f ? 12.0f : c->pml_grading);
}

/* uploadMaterials edge averaging, overrides and binary16 packing (SimulationGrid.cpp:224-262).
 * Outputs the unpacked halves (what unpackHalf2x16 returns in update_E.comp:46-49). */
void oracle_edge_average(const float* sig, const float* eps, int nx, int ny, int nz, const emlab_edge_override* edges,
                         size_t ne, float** out_sig, float** out_eps) {
    const int64_t n = (int64_t)nx * ny * nz;
    float* es = (float*)malloc((size_t)n * 3 * sizeof(float));
    float* ee = (float*)malloc((size_t)n * 3 * sizeof(float));
    if (!es || !ee) {
        free(es), free(ee);
        *out_sig = *out_eps = NULL;
        return;
    }
#define OR_IDX(x, y, z) \
    (((int64_t)((z) > 0 ? (z) : 0) * ny + ((y) > 0 ? (y) : 0)) * nx + ((x) > 0 ? (x) : 0))
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const int64_t c00 = OR_IDX(x, y, z);
                const int64_t ex[4] = {c00, OR_IDX(x, y - 1, z), OR_IDX(x, y, z - 1), OR_IDX(x, y - 1, z - 1)};
                const int64_t ey[4] = {c00, OR_IDX(x - 1, y, z), OR_IDX(x, y, z - 1), OR_IDX(x - 1, y, z - 1)};
                const int64_t ez[4] = {c00, OR_IDX(x - 1, y, z), OR_IDX(x, y - 1, z), OR_IDX(x - 1, y - 1, z)};
                const int64_t* sets[3] = {ex, ey, ez};
                for (int a = 0; a < 3; ++a) {
                    const int64_t* c = sets[a];
                    es[c00 * 3 + a] = 0.25f * (sig[c[0]] + sig[c[1]] + sig[c[2]] + sig[c[3]]);
                    ee[c00 * 3 + a] = 0.25f * (eps[c[0]] + eps[c[1]] + eps[c[2]] + eps[c[3]]);
                }
            }
#undef OR_IDX
    for (size_t k = 0; k < ne; ++k) {
        const emlab_edge_override* o = &edges[k];
        if (o->x < 0 || o->y < 0 || o->z < 0 || o->x >= nx || o->y >= ny || o->z >= nz || o->axis < 0 || o->axis > 2)
            continue;
        const int64_t i = ((int64_t)o->z * ny + o->y) * nx + o->x;
        es[i * 3 + o->axis] = o->sigma > 0.0f ? o->sigma : 0.0f;
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n * 3; ++i) {
        const float s = es[i] < 6.0e4f ? es[i] : 6.0e4f; /* glm::min(v, 6e4): kPerfectEdgeSigma */
        es[i] = emlab_half_round(s);
        ee[i] = emlab_half_round(ee[i]);
    }
    *out_sig = es;
    *out_eps = ee;
}

/* thin-wire factors (SimulationGrid.cpp:279-291), unpacked from binary16 */
void oracle_wire_factors(int nx, int ny, int nz, const emlab_wire_term* w, size_t nw, float** out0, float** out1) {
    const int64_t n = (int64_t)nx * ny * nz;
    float* f0 = (float*)malloc((size_t)n * 3 * sizeof(float));
    float* f1 = (float*)malloc((size_t)n * 3 * sizeof(float));
    if (!f0 || !f1) {
        free(f0), free(f1);
        *out0 = *out1 = NULL;
        return;
    }
    for (int64_t i = 0; i < n * 3; ++i) f0[i] = f1[i] = 1.0f;
    for (size_t k = 0; k < nw; ++k) {
        const emlab_wire_term* t = &w[k];
        if (t->x < 0 || t->y < 0 || t->z < 0 || t->x >= nx || t->y >= ny || t->z >= nz || t->component < 0 ||
            t->component > 2)
            continue;
        const int64_t i = (((int64_t)t->z * ny + t->y) * nx + t->x) * 3 + t->component;
        if (t->term == 0) f0[i] = t->factor;
        else f1[i] = t->factor;
    }
    for (int64_t i = 0; i < n * 3; ++i) f0[i] = emlab_half_round(f0[i]), f1[i] = emlab_half_round(f1[i]);
    *out0 = f0;
    *out1 = f1;
}

/* setSources packing (SimulationGrid.cpp:302-314): GPUSource = center, halfExtent, polAmp, softness */
int oracle_pack_sources(const emlab_source* s, size_t n, emlab_source* desc, float (*src)[16]) {
    int k = 0;
    for (size_t i = 0; i < n && k < 256; ++i) {
        const float* p = s[i].polarization;
        const float len = sqrtf(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]); /* glm::length */
        if (!s[i].enabled || !(len > 1e-6f) || !isfinite(len)) continue;
        float* g = src[k];
        for (int a = 0; a < 3; ++a) {
            const float h = s[i].half_extent[a];
            g[a] = s[i].center[a];
            g[4 + a] = h < 0.0f ? 0.0f : (h > 1.0e5f ? 1.0e5f : h);
            g[8 + a] = p[a] / len;
            g[12 + a] = s[i].softness[a] > 0.25f ? s[i].softness[a] : 0.25f;
        }
        g[3] = g[7] = g[15] = 0.0f;
        g[11] = s[i].amplitude;
        desc[k] = s[i];
        ++k;
    }
    return k;
}

typedef struct {
    uint32_t cell, src;
} oracle_pair;

static int oracle_pair_cmp(const void* a, const void* b) {
    const oracle_pair* p = (const oracle_pair*)a;
    const oracle_pair* q = (const oracle_pair*)b;
    if (p->cell != q->cell) return p->cell < q->cell ? -1 : 1;
    return p->src < q->src ? -1 : (p->src > q->src ? 1 : 0);
}

static int oracle_clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* per-cell source lists (SimulationGrid.cpp:320-350); returns the cell count (-1 on failure) */
int oracle_source_lists(float (*src)[16], int nsrc, const int n[3], int32_t** out_cells, int32_t** out_lists) {
    size_t cap = 1024, np = 0;
    oracle_pair* pairs = (oracle_pair*)malloc(cap * sizeof(oracle_pair));
    if (!pairs) return -1;
    for (int i = 0; i < nsrc; ++i) {
        int lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
            const float c = src[i][a], h = src[i][4 + a], w = src[i][12 + a];
            lo[a] = oracle_clampi((int)floorf(c - h - 3.5f * w) - 1, 0, n[a] - 1);
            hi[a] = oracle_clampi((int)ceilf(c + h + 3.5f * w), 0, n[a] - 1);
        }
        for (int z = lo[2]; z <= hi[2]; ++z)
            for (int y = lo[1]; y <= hi[1]; ++y)
                for (int x = lo[0]; x <= hi[0]; ++x) {
                    if (np == cap) {
                        cap *= 2;
                        oracle_pair* p2 = (oracle_pair*)realloc(pairs, cap * sizeof(oracle_pair));
                        if (!p2) {
                            free(pairs);
                            return -1;
                        }
                        pairs = p2;
                    }
                    pairs[np].cell = (uint32_t)((z * n[1] + y) * n[0] + x);
                    pairs[np].src = (uint32_t)i;
                    ++np;
                }
    }
    qsort(pairs, np, sizeof(oracle_pair), oracle_pair_cmp);
    int32_t* cells = (int32_t*)malloc((np + 1) * 4 * sizeof(int32_t));
    int32_t* lists = (int32_t*)malloc((np > 0 ? np : 1) * sizeof(int32_t));
    int nc = 0;
    for (size_t k = 0; k < np; ++k) {
        if (k == 0 || pairs[k].cell != pairs[k - 1].cell) {
            const uint32_t idx = pairs[k].cell;
            cells[nc * 4 + 0] = (int32_t)(idx % (uint32_t)n[0]);
            cells[nc * 4 + 1] = (int32_t)((idx / (uint32_t)n[0]) % (uint32_t)n[1]);
            cells[nc * 4 + 2] = (int32_t)(idx / (uint32_t)(n[0] * n[1]));
            cells[nc * 4 + 3] = (int32_t)k;
            ++nc;
        }
        lists[k] = (int32_t)pairs[k].src;
    }
    cells[nc * 4 + 0] = cells[nc * 4 + 1] = cells[nc * 4 + 2] = 0;
    cells[nc * 4 + 3] = (int32_t)np; /* sentinel: end of the last list */
    if (np == 0) lists[0] = 0;
    free(pairs);
    *out_cells = cells;
    *out_lists = lists;
    return nc;
}

/* SourceDesc::signal (SimulationGrid.cpp:103-130), FP64 */
double oracle_signal(const emlab_source* s, double tAbs) {
    const double wl = (double)s->wavelength > 1e-3 ? (double)s->wavelength : 1e-3;
    const double delay = (double)s->delay_periods > 0.0 ? (double)s->delay_periods : 0.0;
    const double t = tAbs - delay * wl;
    if (!s->enabled || t < 0.0) return 0.0;
    const double period = wl;
    const double w = 6.28318530717958647692 / wl;
    if (s->waveform == EMLAB_WAVE_CW) {
        const double rampT = ((double)s->ramp_periods > 0.0 ? (double)s->ramp_periods : 0.0) * period;
        double ramp = 1.0;
        if (rampT > 0.0 && t < rampT) {
            const double r = t / rampT;
            ramp = r * r * r * (10.0 + r * (-15.0 + 6.0 * r));
        }
        return ramp * sin(w * t + (double)s->phase);
    }
    const double tau = ((double)s->ramp_periods > 0.1 ? (double)s->ramp_periods : 0.1) * period;
    const double t0 = 3.0 * tau;
    double tl = t;
    if (s->repeat_periods > 0.0f) {
        const double rep0 = (double)s->repeat_periods * period;
        const double rep = rep0 > 2.0 * t0 ? rep0 : 2.0 * t0;
        tl = fmod(t, rep);
    }
    const double u = (tl - t0) / tau;
    if (fabs(u) > 6.0) return 0.0;
    return exp(-u * u) * sin(w * (tl - t0) + (double)s->phase);
}

/* ---- the two instantiations -------------------------------------------------------------- */
#define R float
#define OR_DOUBLE 0
#define NAME(x) x##_f32
#include "oracle_impl.h"
#undef R
#undef OR_DOUBLE
#undef NAME

#define R double
#define OR_DOUBLE 1
#define NAME(x) x##_f64
#include "oracle_impl.h"
#undef R
#undef OR_DOUBLE
#undef NAME

/* the volume pass of the screenshot path (shaders/raymarch.frag) */
#include "oracle_render.h"
