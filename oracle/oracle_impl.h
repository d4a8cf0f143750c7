/* oracle_impl.h - body of the CPU restatement, instantiated twice by emlab_oracle.c:
 * R = float (the parity oracle) and R = double (the error floor). NAME(x) mangles each exported
 * symbol with the precision suffix. TEST INFRASTRUCTURE: only tests, smoke() and the bench's CPU
 * baseline use this code; nothing in the product links it.
 *
 * Every routine follows one reference routine operation for operation, in the GLSL evaluation
 * order (left to right, no contraction); the file:line it follows is given on each.
 */

typedef struct {
    R c[3];
} NAME(vec3);

typedef struct {
    emlab_grid_config cfg;
    int64_t n;
    int use_libm;      /* R = float only: exp() from libm instead of emlab_expf */
    R* E;              /* 4 per texel: Ex, Ey, Ez, sigma_cell (E_Field_Tex) */
    R* B;              /* 4 per texel: Bx, By, Bz, eps_cell (B_Field_Tex) */
    float* esig;       /* 3 per texel: edge sigma after binary16 rounding (unpackHalf2x16) */
    float* eeps;       /* 3 per texel: edge eps_r after binary16 rounding */
    float* w0;         /* 3 per texel: thin-wire factor of term0 (binary16 rounded) */
    float* w1;         /* 3 per texel: thin-wire factor of term1 */
    int thin;
    /* sources (SimulationGrid.cpp:297-357) */
    int nsrc;
    emlab_source desc[256];
    float src[256][16];  /* GPUSource: center.xyzw, halfExtent, polAmp, softness */
    int ncells;
    int32_t* cells;      /* 4 per list cell + sentinel */
    int32_t* lists;
    uint64_t step;
    /* ports (Ports.cpp) */
    int nports;
    emlab_port ports[256];
    float port_wavelength, port_avg;
    R* port_phasor;      /* 8 per port */
    R* series;           /* 2 per port per recorded step */
    size_t series_cap, recorded;
    int recording;
    /* NTFF (FarField.cpp) */
    int ntff_on;
    int box_min[3], box_max[3];
    int face_offset[7];
    int points;
    float ntff_wavelength, ntff_avg;
    R* ntff;             /* 32 per point: stage1 eRe,eIm,hRe,hIm (xyzw), stage2 ... */
    /* coax lines (Coax.cpp, line_accumulate.comp) */
    int nq, nterms;
    int32_t* q;          /* 4 per quantity */
    int32_t* terms;      /* 4 per term */
    float* weights;
    float line_wavelength, line_avg;
    R* line_phasor;      /* 4 per quantity */
    R* line_now;
    /* multi-frequency DFT of the Huygens-box fields (ntffPoint sampling, FP64 sums) */
    int dft_on;
    int dft_min[3], dft_max[3], dft_face[7], dft_points, dft_nf;
    double* dft_w;       /* omega per frequency */
    double* dft;         /* [f][point][6][2] */
    /* opt-in convolutional PML (the library's cpml.cu): per-axis (b, c, 1/kappa) at integer and
       half-integer positions, and the slab auxiliary fields, four arrays per derivative axis */
    int cpml_on;
    float* cpml_coef[2][3]; /* [lattice][axis][i * 3 + {b, c, 1/kappa}] */
    R* cpml_psi[3];         /* [axis][slot * slab + compact index] */
    int64_t cpml_slab[3];
} NAME(grid);

static inline R NAME(exp)(const NAME(grid) * g, R x) {
#if OR_DOUBLE
    (void)g;
    return exp(x);
#else
    return g->use_libm ? expf(x) : emlab_expf(x);
#endif
}

static void NAME(cpml_free)(NAME(grid) * g);

static inline R NAME(rmax)(R a, R b) { return a > b ? a : b; } /* GLSL max(x, y): y if x < y */
static inline R NAME(rmin)(R a, R b) { return b < a ? b : a; }

/* common.glsl:23-27 (off under the convolutional PML, which replaces the graded conductivity) */
static R NAME(pml_profile)(const NAME(grid) * g, R depth) {
    if (depth <= (R)0 || g->cpml_on) return (R)0;
    R u = NAME(rmin)(depth / (R)g->cfg.pml_thickness, (R)1);
    return (R)g->cfg.pml_sigma_max * (NAME(exp)(g, (R)g->cfg.pml_grading * u) - (R)1) /
           (NAME(exp)(g, (R)g->cfg.pml_grading) - (R)1);
}

/* common.glsl:31-36 */
static R NAME(pml_sigma)(const NAME(grid) * g, R x, R y, R z) {
    const R L = (R)g->cfg.pml_thickness;
    const R hx = (R)(g->cfg.nx - 1) - L, hy = (R)(g->cfg.ny - 1) - L, hz = (R)(g->cfg.nz - 1) - L;
    const R dx = NAME(rmax)(L - x, x - hx), dy = NAME(rmax)(L - y, y - hy), dz = NAME(rmax)(L - z, z - hz);
    return NAME(pml_profile)(g, dx) + NAME(pml_profile)(g, dy) + NAME(pml_profile)(g, dz);
}

/* common.glsl:40-43 */
static int NAME(in_pml)(const NAME(grid) * g, int x, int y, int z) {
    const int L = g->cfg.pml_thickness;
    return x < L || y < L || z < L || x >= g->cfg.nx - (L + 1) || y >= g->cfg.ny - (L + 1) ||
           z >= g->cfg.nz - (L + 1);
}

/* common.glsl:50-54 (mix(series, exact, step(1e-2, x)) picks one branch) */
static R NAME(phi)(const NAME(grid) * g, R x) {
    const R series = (R)1 - x * ((R)0.5 - x * ((R)1 / (R)6 - x * ((R)1 / (R)24)));
    const R exact = ((R)1 - NAME(exp)(g, -x)) / NAME(rmax)(x, (R)1e-12);
    return x < (R)1e-2 ? series : exact;
}

static inline int64_t NAME(idx)(const NAME(grid) * g, int x, int y, int z) {
    return ((int64_t)z * g->cfg.ny + y) * g->cfg.nx + x;
}

/* texelFetch with the update_B.comp:27-29 rule: E beyond the upper faces is 0 */
static inline R NAME(fetchE0)(const NAME(grid) * g, int x, int y, int z, int c) {
    if (x >= g->cfg.nx || y >= g->cfg.ny || z >= g->cfg.nz) return (R)0;
    return g->E[NAME(idx)(g, x, y, z) * 4 + c];
}
/* update_E.comp:27-29: B below the lower faces is 0 */
static inline R NAME(fetchB0)(const NAME(grid) * g, int x, int y, int z, int c) {
    if (x < 0 || y < 0 || z < 0) return (R)0;
    return g->B[NAME(idx)(g, x, y, z) * 4 + c];
}
static inline int NAME(clampi)(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
/* clamp-to-edge fetch of the monitors (field_sampling.glsl:14-15, port_accumulate.comp:40-41) */
static inline R NAME(fetchEc)(const NAME(grid) * g, int x, int y, int z, int c) {
    x = NAME(clampi)(x, 0, g->cfg.nx - 1), y = NAME(clampi)(y, 0, g->cfg.ny - 1), z = NAME(clampi)(z, 0, g->cfg.nz - 1);
    return g->E[NAME(idx)(g, x, y, z) * 4 + c];
}
static inline R NAME(fetchBc)(const NAME(grid) * g, int x, int y, int z, int c) {
    x = NAME(clampi)(x, 0, g->cfg.nx - 1), y = NAME(clampi)(y, 0, g->cfg.ny - 1), z = NAME(clampi)(z, 0, g->cfg.nz - 1);
    return g->B[NAME(idx)(g, x, y, z) * 4 + c];
}

/* ---------------------------------------------------------------------------------------- */
/* SimulationGrid::configure (SimulationGrid.cpp:149-199) */
static void NAME(free_buffers)(NAME(grid) * g) {
    free(g->E), free(g->B), free(g->esig), free(g->eeps), free(g->w0), free(g->w1);
    g->E = g->B = NULL;
    g->esig = g->eeps = g->w0 = g->w1 = NULL;
}

void* NAME(oracle_create)(const emlab_grid_config* req, int use_libm) {
    NAME(grid)* g = (NAME(grid)*)calloc(1, sizeof(NAME(grid)));
    if (!g) return NULL;
    emlab_grid_config c = *req;
    oracle_clamp_config(&c);
    g->cfg = c;
    g->use_libm = use_libm;
    g->n = (int64_t)c.nx * c.ny * c.nz;
    g->E = (R*)calloc((size_t)g->n * 4, sizeof(R));
    g->B = (R*)calloc((size_t)g->n * 4, sizeof(R));
    g->esig = (float*)calloc((size_t)g->n * 3, sizeof(float));
    g->eeps = (float*)malloc((size_t)g->n * 3 * sizeof(float));
    if (!g->E || !g->B || !g->esig || !g->eeps) {
        NAME(free_buffers)(g);
        free(g);
        return NULL;
    }
    /* vacuum: E.a = 0, B.a = 1, edge eps 1 (SimulationGrid.cpp:185-192) */
    for (int64_t i = 0; i < g->n; ++i) {
        g->B[i * 4 + 3] = (R)1;
        g->eeps[i * 3 + 0] = g->eeps[i * 3 + 1] = g->eeps[i * 3 + 2] = 1.0f;
    }
    return g;
}

void NAME(oracle_destroy)(void* h) {
    NAME(grid)* g = (NAME(grid)*)h;
    if (!g) return;
    NAME(free_buffers)(g);
    free(g->cells), free(g->lists), free(g->port_phasor), free(g->series), free(g->ntff);
    free(g->q), free(g->terms), free(g->weights), free(g->line_phasor), free(g->line_now);
    free(g->dft_w), free(g->dft);
    NAME(cpml_free)(g);
    free(g);
}

void NAME(oracle_get_config)(void* h, emlab_grid_config* out) { *out = ((NAME(grid)*)h)->cfg; }
uint64_t NAME(oracle_step_count)(void* h) { return ((NAME(grid)*)h)->step; }
int NAME(oracle_source_cells)(void* h) { return ((NAME(grid)*)h)->ncells; }

/* SimulationGrid::uploadMaterials (SimulationGrid.cpp:209-295) */
int NAME(oracle_upload_materials)(void* h, const float* sig, const float* eps, int nx, int ny, int nz,
                                  const emlab_edge_override* edges, size_t ne, const emlab_wire_term* wires,
                                  size_t nw) {
    NAME(grid)* g = (NAME(grid)*)h;
    if (nx != g->cfg.nx || ny != g->cfg.ny || nz != g->cfg.nz) return EMLAB_ERR_INVALID;
    float *es = NULL, *ee = NULL;
    oracle_edge_average(sig, eps, nx, ny, nz, edges, ne, &es, &ee);
    if (!es) return EMLAB_ERR_OOM;
    for (int64_t i = 0; i < g->n; ++i) {
        g->E[i * 4 + 0] = g->E[i * 4 + 1] = g->E[i * 4 + 2] = (R)0;
        g->B[i * 4 + 0] = g->B[i * 4 + 1] = g->B[i * 4 + 2] = (R)0;
        g->E[i * 4 + 3] = (R)sig[i];
        g->B[i * 4 + 3] = (R)eps[i];
    }
    free(g->esig), free(g->eeps);
    g->esig = es, g->eeps = ee;
    free(g->w0), free(g->w1);
    g->w0 = g->w1 = NULL;
    g->thin = nw > 0;
    if (g->thin) {
        oracle_wire_factors(nx, ny, nz, wires, nw, &g->w0, &g->w1);
        if (!g->w0) return EMLAB_ERR_OOM;
    }
    g->step = 0;
    return EMLAB_OK;
}

/* read-back of the edge materials and wire factors as the shaders see them */
void NAME(oracle_edge_materials)(void* h, float* sig3, float* eps3, float* w0, float* w1) {
    NAME(grid)* g = (NAME(grid)*)h;
    memcpy(sig3, g->esig, (size_t)g->n * 3 * sizeof(float));
    memcpy(eps3, g->eeps, (size_t)g->n * 3 * sizeof(float));
    for (int64_t i = 0; i < g->n * 3; ++i) {
        if (w0) w0[i] = g->thin ? g->w0[i] : 1.0f;
        if (w1) w1[i] = g->thin ? g->w1[i] : 1.0f;
    }
}

/* SimulationGrid::setSources (SimulationGrid.cpp:297-357) */
int NAME(oracle_set_sources)(void* h, const emlab_source* s, size_t n) {
    NAME(grid)* g = (NAME(grid)*)h;
    free(g->cells), free(g->lists);
    g->cells = NULL, g->lists = NULL;
    g->nsrc = oracle_pack_sources(s, n, g->desc, g->src);
    int dims[3] = {g->cfg.nx, g->cfg.ny, g->cfg.nz};
    g->ncells = oracle_source_lists(g->src, g->nsrc, dims, &g->cells, &g->lists);
    return g->ncells < 0 ? EMLAB_ERR_OOM : EMLAB_OK;
}

/* SimulationGrid::resetFields (SimulationGrid.cpp:359-366) */
void NAME(oracle_reset_fields)(void* h) {
    NAME(grid)* g = (NAME(grid)*)h;
    for (int64_t i = 0; i < g->n; ++i)
        for (int c = 0; c < 3; ++c) g->E[i * 4 + c] = g->B[i * 4 + c] = (R)0;
    for (int a = 0; a < 3; ++a)
        if (g->cpml_psi[a]) memset(g->cpml_psi[a], 0, (size_t)g->cpml_slab[a] * 4 * sizeof(R));
    g->step = 0;
}

/* ---------------------------------------------------------------------------------------- */
/* The opt-in convolutional PML, restated from its definition (Roden & Gedney's recursive
   convolution: psi <- b psi + c dF, derivative -> dF / kappa + psi inside slabs of L + 1 cells at
   each face), in the operation order the library's cpml.cu uses; coefficients from the shared
   emlab_cpml_coef (FP64 -> FP32). */
static void NAME(cpml_free)(NAME(grid) * g) {
    for (int l = 0; l < 2; ++l)
        for (int a = 0; a < 3; ++a) free(g->cpml_coef[l][a]), g->cpml_coef[l][a] = NULL;
    for (int a = 0; a < 3; ++a) free(g->cpml_psi[a]), g->cpml_psi[a] = NULL;
    g->cpml_on = 0;
}

int NAME(oracle_set_cpml)(void* h, int on, float sigma_max, float kappa_max, float alpha_max, float order) {
    NAME(grid)* g = (NAME(grid)*)h;
    NAME(cpml_free)(g);
    if (on) {
        const int n[3] = {g->cfg.nx, g->cfg.ny, g->cfg.nz};
        const int L = g->cfg.pml_thickness, S = 2 * (L + 1);
        for (int l = 0; l < 2; ++l)
            for (int a = 0; a < 3; ++a) {
                g->cpml_coef[l][a] = (float*)malloc((size_t)n[a] * 3 * sizeof(float));
                if (!g->cpml_coef[l][a]) return EMLAB_ERR_OOM;
                for (int i = 0; i < n[a]; ++i)
                    emlab_cpml_coef((double)i + (l ? 0.5 : 0.0), n[a], L, sigma_max, kappa_max, alpha_max, order,
                                    (double)g->cfg.courant, g->cpml_coef[l][a] + (size_t)i * 3);
            }
        const int64_t area[3] = {(int64_t)n[1] * n[2], (int64_t)n[0] * n[2], (int64_t)n[0] * n[1]};
        for (int a = 0; a < 3; ++a) {
            g->cpml_slab[a] = area[a] * S;
            g->cpml_psi[a] = (R*)calloc((size_t)g->cpml_slab[a] * 4, sizeof(R));
            if (!g->cpml_psi[a]) return EMLAB_ERR_OOM;
        }
        g->cpml_on = 1;
    }
    NAME(oracle_reset_fields)(h);
    return EMLAB_OK;
}

/* dF / kappa + psi for the derivative along `axis` (lattice 0: integer positions, 1: half) of the
   component in psi slot `slot`, at (x, y, z); dF outside the slabs */
static inline R NAME(cpml_term)(NAME(grid) * g, int lattice, int axis, int slot, int x, int y, int z, R d) {
    const int n[3] = {g->cfg.nx, g->cfg.ny, g->cfg.nz};
    const int p[3] = {x, y, z};
    const int L1 = g->cfg.pml_thickness + 1, S = 2 * L1;
    const int i = p[axis];
    int s = -1;
    if (i < L1) s = i;
    else if (i >= n[axis] - L1) s = i - n[axis] + 2 * L1;
    if (s < 0) return d;
    int64_t at;
    if (axis == 0) at = ((int64_t)z * n[1] + y) * S + s;
    else if (axis == 1) at = ((int64_t)z * S + s) * n[0] + x;
    else at = ((int64_t)s * n[1] + y) * n[0] + x;
    R* psi = g->cpml_psi[axis] + (int64_t)slot * g->cpml_slab[axis] + at;
    const float* k = g->cpml_coef[lattice][axis] + (size_t)i * 3;
    const R v = (R)k[0] * *psi + (R)k[1] * d;
    *psi = v;
    return d * (R)k[2] + v;
}

static void NAME(cpml_update_B)(NAME(grid) * g) {
    const int nx = g->cfg.nx, ny = g->cfg.ny, nz = g->cfg.nz;
    const R dt = (R)g->cfg.courant;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const int64_t i = NAME(idx)(g, x, y, z);
                const R* e0 = g->E + i * 4;
                const R exy = NAME(fetchE0)(g, x + 1, y, z, 1), exz = NAME(fetchE0)(g, x + 1, y, z, 2);
                const R eyx = NAME(fetchE0)(g, x, y + 1, z, 0), eyz = NAME(fetchE0)(g, x, y + 1, z, 2);
                const R ezx = NAME(fetchE0)(g, x, y, z + 1, 0), ezy = NAME(fetchE0)(g, x, y, z + 1, 1);
                R t0[3] = {eyz - e0[2], ezx - e0[0], exy - e0[1]};
                R t1[3] = {ezy - e0[1], exz - e0[2], eyx - e0[0]};
                if (g->thin) {
                    for (int c = 0; c < 3; ++c) {
                        t0[c] = t0[c] * (R)g->w0[i * 3 + c];
                        t1[c] = t1[c] * (R)g->w1[i * 3 + c];
                    }
                }
                R* b = g->B + i * 4;
                for (int c = 0; c < 3; ++c) {
                    const R u0 = NAME(cpml_term)(g, 1, (c + 1) % 3, 2, x, y, z, t0[c]);
                    const R u1 = NAME(cpml_term)(g, 1, (c + 2) % 3, 3, x, y, z, t1[c]);
                    const R curl = u0 - u1;
                    b[c] = b[c] - dt * curl;
                }
            }
}

static void NAME(e_coeffs)(const NAME(grid) * g, int x, int y, int z, R ca[3], R cb[3]);

static void NAME(cpml_update_E)(NAME(grid) * g) {
    const int nx = g->cfg.nx, ny = g->cfg.ny, nz = g->cfg.nz;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const int64_t i = NAME(idx)(g, x, y, z);
                const R* b0 = g->B + i * 4;
                const R bxy = NAME(fetchB0)(g, x - 1, y, z, 1), bxz = NAME(fetchB0)(g, x - 1, y, z, 2);
                const R byx = NAME(fetchB0)(g, x, y - 1, z, 0), byz = NAME(fetchB0)(g, x, y - 1, z, 2);
                const R bzx = NAME(fetchB0)(g, x, y, z - 1, 0), bzy = NAME(fetchB0)(g, x, y, z - 1, 1);
                const R t0[3] = {b0[2] - byz, b0[0] - bzx, b0[1] - bxy};
                const R t1[3] = {b0[1] - bzy, b0[2] - bxz, b0[0] - byx};
                R ca[3], cb[3];
                NAME(e_coeffs)(g, x, y, z, ca, cb);
                R* e = g->E + i * 4;
                for (int c = 0; c < 3; ++c) {
                    const R u0 = NAME(cpml_term)(g, 0, (c + 1) % 3, 0, x, y, z, t0[c]);
                    const R u1 = NAME(cpml_term)(g, 0, (c + 2) % 3, 1, x, y, z, t1[c]);
                    const R curl = u0 - u1;
                    e[c] = ca[c] * e[c] + cb[c] * curl;
                }
            }
}

/* ---------------------------------------------------------------------------------------- */
/* update_B.comp:31-70 */
static void NAME(update_B)(NAME(grid) * g) {
    const int nx = g->cfg.nx, ny = g->cfg.ny, nz = g->cfg.nz;
    const R dt = (R)g->cfg.courant;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const int64_t i = NAME(idx)(g, x, y, z);
                const R* e0 = g->E + i * 4;
                const R exy = NAME(fetchE0)(g, x + 1, y, z, 1), exz = NAME(fetchE0)(g, x + 1, y, z, 2);
                const R eyx = NAME(fetchE0)(g, x, y + 1, z, 0), eyz = NAME(fetchE0)(g, x, y + 1, z, 2);
                const R ezx = NAME(fetchE0)(g, x, y, z + 1, 0), ezy = NAME(fetchE0)(g, x, y, z + 1, 1);
                R t0[3] = {eyz - e0[2], ezx - e0[0], exy - e0[1]};
                R t1[3] = {ezy - e0[1], exz - e0[2], eyx - e0[0]};
                if (g->thin) {
                    for (int c = 0; c < 3; ++c) {
                        t0[c] = t0[c] * (R)g->w0[i * 3 + c];
                        t1[c] = t1[c] * (R)g->w1[i * 3 + c];
                    }
                }
                R* b = g->B + i * 4;
                R curl[3];
                for (int c = 0; c < 3; ++c) curl[c] = t0[c] - t1[c];
                if (NAME(in_pml)(g, x, y, z)) {
                    const R px = (R)x, py = (R)y, pz = (R)z, h = (R)0.5;
                    R sm[3] = {NAME(pml_sigma)(g, px, py + h, pz + h), NAME(pml_sigma)(g, px + h, py, pz + h),
                               NAME(pml_sigma)(g, px + h, py + h, pz)};
                    for (int c = 0; c < 3; ++c) {
                        const R xx = sm[c] * dt;
                        b[c] = NAME(exp)(g, -xx) * b[c] - (dt * NAME(phi)(g, xx)) * curl[c];
                    }
                } else {
                    for (int c = 0; c < 3; ++c) b[c] = b[c] - dt * curl[c];
                }
            }
}

/* coefficient Cb of update_E.comp:46-61 (also apply_sources.comp:64-75) */
static void NAME(e_coeffs)(const NAME(grid) * g, int x, int y, int z, R ca[3], R cb[3]) {
    const int64_t i = NAME(idx)(g, x, y, z);
    const R dt = (R)g->cfg.courant;
    R sigma[3], eps[3];
    for (int c = 0; c < 3; ++c) {
        sigma[c] = NAME(rmax)((R)g->esig[i * 3 + c], (R)0);
        eps[c] = NAME(rmax)((R)g->eeps[i * 3 + c], (R)1);
    }
    if (NAME(in_pml)(g, x, y, z)) {
        const R px = (R)x, py = (R)y, pz = (R)z, h = (R)0.5;
        sigma[0] = sigma[0] + NAME(pml_sigma)(g, px + h, py, pz);
        sigma[1] = sigma[1] + NAME(pml_sigma)(g, px, py + h, pz);
        sigma[2] = sigma[2] + NAME(pml_sigma)(g, px, py, pz + h);
    }
    for (int c = 0; c < 3; ++c) {
        const R dtEps = dt / eps[c];
        const R xx = sigma[c] * dtEps;
        if (ca) ca[c] = NAME(exp)(g, -xx);
        cb[c] = dtEps * NAME(phi)(g, xx);
    }
}

/* update_E.comp:31-66 */
static void NAME(update_E)(NAME(grid) * g) {
    const int nx = g->cfg.nx, ny = g->cfg.ny, nz = g->cfg.nz;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const int64_t i = NAME(idx)(g, x, y, z);
                const R* b0 = g->B + i * 4;
                const R bxy = NAME(fetchB0)(g, x - 1, y, z, 1), bxz = NAME(fetchB0)(g, x - 1, y, z, 2);
                const R byx = NAME(fetchB0)(g, x, y - 1, z, 0), byz = NAME(fetchB0)(g, x, y - 1, z, 2);
                const R bzx = NAME(fetchB0)(g, x, y, z - 1, 0), bzy = NAME(fetchB0)(g, x, y, z - 1, 1);
                const R curl[3] = {(b0[2] - byz) - (b0[1] - bzy), (b0[0] - bzx) - (b0[2] - bxz),
                                   (b0[1] - bxy) - (b0[0] - byx)};
                R ca[3], cb[3];
                NAME(e_coeffs)(g, x, y, z, ca, cb);
                R* e = g->E + i * 4;
                for (int c = 0; c < 3; ++c) e[c] = ca[c] * e[c] + cb[c] * curl[c];
            }
}

/* apply_sources.comp:37-40 */
static R NAME(footprint)(const NAME(grid) * g, const float* s, R x, R y, R z) {
    const R p[3] = {x, y, z};
    R d[3];
    for (int c = 0; c < 3; ++c) {
        R a = p[c] - (R)s[c];
        a = a < (R)0 ? -a : a;
        d[c] = NAME(rmax)(a - (R)s[4 + c], (R)0) / (R)s[12 + c];
    }
    return NAME(exp)(g, -(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]));
}

/* apply_sources.comp:42-79 with the signals of one sub-step */
static void NAME(apply_sources)(NAME(grid) * g, const float* signals) {
#pragma omp parallel for schedule(static)
    for (int id = 0; id < g->ncells; ++id) {
        const int32_t* entry = g->cells + (size_t)id * 4;
        const int end = g->cells[(size_t)(id + 1) * 4 + 3];
        const int x = entry[0], y = entry[1], z = entry[2];
        const R cx = (R)x, cy = (R)y, cz = (R)z, h = (R)0.5;
        R J[3] = {0, 0, 0};
        for (int k = entry[3]; k < end; ++k) {
            const int si = g->lists[k];
            const float signal = signals[si];
            if (signal == 0.0f) continue;
            const float* s = g->src[si];
            const R w[3] = {NAME(footprint)(g, s, cx + h, cy, cz), NAME(footprint)(g, s, cx, cy + h, cz),
                            NAME(footprint)(g, s, cx, cy, cz + h)};
            const R as = (R)s[11] * (R)signal;
            for (int c = 0; c < 3; ++c) J[c] = J[c] + ((R)s[8 + c] * as) * w[c];
        }
        if (J[0] == (R)0 && J[1] == (R)0 && J[2] == (R)0) continue;
        R cb[3];
        NAME(e_coeffs)(g, x, y, z, NULL, cb);
        R* e = g->E + NAME(idx)(g, x, y, z) * 4;
        for (int c = 0; c < 3; ++c) e[c] = e[c] - cb[c] * J[c];
    }
}

/* field_sampling.glsl:17-32 */
static void NAME(e_at_node)(const NAME(grid) * g, int x, int y, int z, R out[3]) {
    out[0] = (R)0.5 * (NAME(fetchEc)(g, x, y, z, 0) + NAME(fetchEc)(g, x - 1, y, z, 0));
    out[1] = (R)0.5 * (NAME(fetchEc)(g, x, y, z, 1) + NAME(fetchEc)(g, x, y - 1, z, 1));
    out[2] = (R)0.5 * (NAME(fetchEc)(g, x, y, z, 2) + NAME(fetchEc)(g, x, y, z - 1, 2));
}
static void NAME(b_at_node)(const NAME(grid) * g, int x, int y, int z, R out[3]) {
    const R bx = NAME(fetchBc)(g, x, y, z, 0) + NAME(fetchBc)(g, x, y - 1, z, 0) + NAME(fetchBc)(g, x, y, z - 1, 0) +
                 NAME(fetchBc)(g, x, y - 1, z - 1, 0);
    const R by = NAME(fetchBc)(g, x, y, z, 1) + NAME(fetchBc)(g, x - 1, y, z, 1) + NAME(fetchBc)(g, x, y, z - 1, 1) +
                 NAME(fetchBc)(g, x - 1, y, z - 1, 1);
    const R bz = NAME(fetchBc)(g, x, y, z, 2) + NAME(fetchBc)(g, x - 1, y, z, 2) + NAME(fetchBc)(g, x, y - 1, z, 2) +
                 NAME(fetchBc)(g, x - 1, y - 1, z, 2);
    out[0] = (R)0.25 * bx, out[1] = (R)0.25 * by, out[2] = (R)0.25 * bz;
}

/* ntff_common.glsl:30-53 */
static void NAME(ntff_point)(const NAME(grid) * g, int index, int node[3], R normal[3], R* weight) {
    int f = 0;
    for (int i = 1; i < 6; ++i)
        if (index >= g->face_offset[i]) f = i;
    const int a = f >> 1, side = f & 1;
    const int u = a == 0 ? 1 : 0, v = a == 2 ? 1 : 2;
    const int nu = g->box_max[u] - g->box_min[u], nv = g->box_max[v] - g->box_min[v];
    const int local = index - g->face_offset[f];
    const int iu = local % (nu + 1), iv = local / (nu + 1);
    node[0] = g->box_min[0], node[1] = g->box_min[1], node[2] = g->box_min[2];
    node[a] = side == 1 ? g->box_max[a] : g->box_min[a];
    node[u] = g->box_min[u] + iu;
    node[v] = g->box_min[v] + iv;
    *weight = ((iu == 0 || iu == nu) ? (R)0.5 : (R)1) * ((iv == 0 || iv == nv) ? (R)0.5 : (R)1);
    normal[0] = normal[1] = normal[2] = (R)0;
    normal[a] = side == 1 ? (R)1 : (R)-1;
}

/* ntffPoint on an explicit box (same arithmetic as ntff_common.glsl:30-53) */
static void NAME(box_point)(const int* mn, const int* mx, const int* face, int index, int node[3]) {
    int f = 0;
    for (int i = 1; i < 6; ++i)
        if (index >= face[i]) f = i;
    const int a = f >> 1, side = f & 1;
    const int u = a == 0 ? 1 : 0, v = a == 2 ? 1 : 2;
    const int nu = mx[u] - mn[u];
    const int local = index - face[f];
    const int iu = local % (nu + 1), iv = local / (nu + 1);
    node[0] = mn[0], node[1] = mn[1], node[2] = mn[2];
    node[a] = side == 1 ? mx[a] : mn[a];
    node[u] = mn[u] + iu;
    node[v] = mn[v] + iv;
}

/* multi-frequency running DFT: X_f += F(t) e^{-i w_f t}, t = n dt for E and (n - 1/2) dt for H,
   with the fields co-located as field_sampling.glsl:17-32 does (FP32/FP64 samples, FP64 sums) */
static void NAME(dft_accumulate)(NAME(grid) * g) {
    const double dt = (double)g->cfg.courant;
    const double tE = (double)g->step * dt, tH = tE - 0.5 * dt;
    const int P = g->dft_points, nf = g->dft_nf;
    /* the phases depend on the frequency only: evaluated once per step (nf <= 128) */
    double rot[128][4];
    for (int f = 0; f < nf && f < 128; ++f) {
        const double w = g->dft_w[f];
        rot[f][0] = cos(w * tE), rot[f][1] = sin(w * tE), rot[f][2] = cos(w * tH), rot[f][3] = sin(w * tH);
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < P; ++i) {
        int node[3];
        NAME(box_point)(g->dft_min, g->dft_max, g->dft_face, i, node);
        R E[3], H[3];
        NAME(e_at_node)(g, node[0], node[1], node[2], E);
        NAME(b_at_node)(g, node[0], node[1], node[2], H);
        for (int f = 0; f < nf && f < 128; ++f) {
            const double ce = rot[f][0], se = rot[f][1], ch = rot[f][2], sh = rot[f][3];
            double* x = g->dft + ((size_t)f * P + (size_t)i) * 12;
            for (int c = 0; c < 3; ++c) {
                x[2 * c] += (double)E[c] * ce, x[2 * c + 1] -= (double)E[c] * se;
                x[6 + 2 * c] += (double)H[c] * ch, x[6 + 2 * c + 1] -= (double)H[c] * sh;
            }
        }
    }
}

/* FarFieldMonitor::accumulate (FarField.cpp:198-217) + ntff_accumulate.comp:30-52 */
static void NAME(ntff_accumulate)(NAME(grid) * g) {
    const double w = 6.28318530717958647692 / (double)g->ntff_wavelength;
    const double dt = (double)g->cfg.courant;
    const double tE = (double)g->step * dt, tH = tE - 0.5 * dt;
    const R rot[4] = {(R)(float)cos(w * tE), (R)(float)sin(w * tE), (R)(float)cos(w * tH), (R)(float)sin(w * tH)};
    const double tau = (double)g->ntff_avg * (double)g->ntff_wavelength;
    const R blend = (R)(float)(1.0 - exp(-dt / (0.5 * tau)));
#pragma omp parallel for schedule(static)
    for (int i = 0; i < g->points; ++i) {
        int node[3];
        R n[3], wgt;
        NAME(ntff_point)(g, i, node, n, &wgt);
        R E[3], H[3];
        NAME(e_at_node)(g, node[0], node[1], node[2], E);
        NAME(b_at_node)(g, node[0], node[1], node[2], H);
        R* p = g->ntff + (size_t)i * 32;
        for (int c = 0; c < 3; ++c) {
            p[0 + c] = p[0 + c] + blend * (((R)2 * rot[0]) * E[c] - p[0 + c]);
            p[4 + c] = p[4 + c] + blend * (((R)-2 * rot[1]) * E[c] - p[4 + c]);
            p[8 + c] = p[8 + c] + blend * (((R)2 * rot[2]) * H[c] - p[8 + c]);
            p[12 + c] = p[12 + c] + blend * (((R)-2 * rot[3]) * H[c] - p[12 + c]);
        }
        for (int c = 0; c < 3; ++c)
            for (int k = 0; k < 4; ++k) p[16 + 4 * k + c] = p[16 + 4 * k + c] + blend * (p[4 * k + c] - p[16 + 4 * k + c]);
    }
}

/* port_accumulate.comp:46-50 */
static R NAME(edge_current)(const NAME(grid) * g, int x, int y, int z, int a) {
    const int u = (a + 1) % 3, v = (a + 2) % 3;
    int pu[3] = {x, y, z}, pv[3] = {x, y, z};
    pu[u] -= 1, pv[v] -= 1;
    const R b0v = NAME(fetchBc)(g, x, y, z, v), b0u = NAME(fetchBc)(g, x, y, z, u);
    const R buv = NAME(fetchBc)(g, pu[0], pu[1], pu[2], v);
    const R bvu = NAME(fetchBc)(g, pv[0], pv[1], pv[2], u);
    return (b0v - buv) - (b0u - bvu);
}

/* PortMonitor::accumulate (Ports.cpp:113-136) + port_accumulate.comp:52-83 */
static void NAME(ports_accumulate)(NAME(grid) * g) {
    const double w = 6.28318530717958647692 / (double)g->port_wavelength;
    const double dt = (double)g->cfg.courant;
    const double tE = (double)g->step * dt, tH = tE - 0.5 * dt;
    const double tau = (double)g->port_avg * (double)g->port_wavelength;
    const R rot[4] = {(R)(float)cos(w * tE), (R)(float)sin(w * tE), (R)(float)cos(w * tH), (R)(float)sin(w * tH)};
    const R blend = (R)(float)(1.0 - exp(-dt / (0.5 * tau)));
    const int record = g->recording && g->recorded < g->series_cap;
    for (int i = 0; i < g->nports; ++i) {
        const emlab_port* pt = &g->ports[i];
        const int a = pt->axis;
        const R s = (R)pt->sign;
        R V = (R)0, I = (R)0;
        if (pt->edges == 4) {
            int eu[3] = {0, 0, 0}, ev[3] = {0, 0, 0};
            eu[(a + 1) % 3] = 1, ev[(a + 2) % 3] = 1;
            const int offs[4][3] = {{0, 0, 0}, {eu[0], eu[1], eu[2]}, {ev[0], ev[1], ev[2]},
                                    {eu[0] + ev[0], eu[1] + ev[1], eu[2] + ev[2]}};
            for (int k = 0; k < 4; ++k) {
                const int x = pt->x + offs[k][0], y = pt->y + offs[k][1], z = pt->z + offs[k][2];
                V = V + (R)0.25 * NAME(fetchEc)(g, x, y, z, a);
                I = I + NAME(edge_current)(g, x, y, z, a);
            }
        } else {
            V = NAME(fetchEc)(g, pt->x, pt->y, pt->z, a);
            I = NAME(edge_current)(g, pt->x, pt->y, pt->z, a);
        }
        V = V * s;
        I = I * s;
        if (record) {
            g->series[(g->recorded * (size_t)g->nports + (size_t)i) * 2 + 0] = V;
            g->series[(g->recorded * (size_t)g->nports + (size_t)i) * 2 + 1] = I;
        }
        const R obs[4] = {((R)2 * rot[0]) * V, ((R)-2 * rot[1]) * V, ((R)2 * rot[2]) * I, ((R)-2 * rot[3]) * I};
        R* ph = g->port_phasor + (size_t)i * 8;
        for (int c = 0; c < 4; ++c) ph[c] = ph[c] + blend * (obs[c] - ph[c]);
        for (int c = 0; c < 4; ++c) ph[4 + c] = ph[4 + c] + blend * (ph[c] - ph[4 + c]);
    }
    if (record) ++g->recorded;
}

/* CoaxMonitor::accumulate (Coax.cpp:179-197) + line_accumulate.comp:30-48 */
static void NAME(lines_accumulate)(NAME(grid) * g) {
    const double w = 6.28318530717958647692 / (double)g->line_wavelength;
    const double dt = (double)g->cfg.courant;
    const double tE = (double)g->step * dt, tH = tE - 0.5 * dt;
    const double tau = (double)g->line_avg * (double)g->line_wavelength;
    const R rot[4] = {(R)(float)cos(w * tE), (R)(float)sin(w * tE), (R)(float)cos(w * tH), (R)(float)sin(w * tH)};
    const R blend = (R)(float)(1.0 - exp(-dt / (0.5 * tau)));
    for (int qi = 0; qi < g->nq; ++qi) {
        const int32_t* info = g->q + (size_t)qi * 4;
        R sum = (R)0;
        for (int k = info[0]; k < info[0] + info[1]; ++k) {
            const int32_t* t = g->terms + (size_t)k * 4;
            const R f = t[3] < 3 ? NAME(fetchEc)(g, t[0], t[1], t[2], t[3] % 3) : NAME(fetchBc)(g, t[0], t[1], t[2], t[3] % 3);
            sum = sum + (R)g->weights[k] * f;
        }
        g->line_now[qi] = sum;
        const R r0 = info[2] == 0 ? rot[0] : rot[2], r1 = info[2] == 0 ? rot[1] : rot[3];
        const R obs[2] = {((R)2 * sum) * r0, ((R)2 * sum) * -r1};
        R* ph = g->line_phasor + (size_t)qi * 4;
        ph[0] = ph[0] + blend * (obs[0] - ph[0]);
        ph[1] = ph[1] + blend * (obs[1] - ph[1]);
        ph[2] = ph[2] + blend * (ph[0] - ph[2]);
        ph[3] = ph[3] + blend * (ph[1] - ph[3]);
    }
}

/* SimulationGrid::step (SimulationGrid.cpp:368-433) with Instruments::onStep's monitors
   (Instruments.cpp:189-195) as the per-step callback */
void NAME(oracle_step)(void* h, int count) {
    NAME(grid)* g = (NAME(grid)*)h;
    if (count <= 0) return;
    float signals[256];
    for (int k = 0; k < count; ++k) {
        const double t = ((double)(g->step) + 0.5) * (double)g->cfg.courant;
        for (int s = 0; s < g->nsrc; ++s) signals[s] = (float)oracle_signal(&g->desc[s], t);
        if (g->cpml_on) {
            NAME(cpml_update_B)(g);
            NAME(cpml_update_E)(g);
        } else {
            NAME(update_B)(g);
            NAME(update_E)(g);
        }
        if (g->ncells > 0) NAME(apply_sources)(g, signals);
        ++g->step;
        if (g->ntff_on) NAME(ntff_accumulate)(g);
        if (g->nports > 0) NAME(ports_accumulate)(g);
        if (g->nq > 0) NAME(lines_accumulate)(g);
        if (g->dft_on) NAME(dft_accumulate)(g);
    }
}

/* the multi-frequency DFT monitor: box clamped like FarFieldMonitor::configure; nf = 0 disables */
int NAME(oracle_ntff_dft_configure)(void* h, const int mn[3], const int mx[3], const float* wavelengths, int nf,
                                    int box_out[6]) {
    NAME(grid)* g = (NAME(grid)*)h;
    free(g->dft_w), free(g->dft);
    g->dft_w = NULL, g->dft = NULL, g->dft_on = 0;
    if (nf <= 0) return EMLAB_OK;
    if (nf > 128) return EMLAB_ERR_INVALID; /* as the device monitor: at most 128 frequencies */
    const int n[3] = {g->cfg.nx, g->cfg.ny, g->cfg.nz};
    const int L = g->cfg.pml_thickness;
    for (int a = 0; a < 3; ++a) {
        const int lo = L + 1, hi = n[a] - L - 2;
        int b0 = mn[a] < mx[a] ? mn[a] : mx[a], b1 = mn[a] < mx[a] ? mx[a] : mn[a];
        b0 = b0 < lo ? lo : (b0 > hi ? hi : b0);
        b1 = b1 < lo ? lo : (b1 > hi ? hi : b1);
        if (b1 - b0 < 4) return EMLAB_ERR_INVALID;
        g->dft_min[a] = b0, g->dft_max[a] = b1;
        if (box_out) box_out[a] = b0, box_out[3 + a] = b1;
    }
    g->dft_face[0] = 0;
    for (int f = 0; f < 6; ++f) {
        const int a = f >> 1, u = a == 0 ? 1 : 0, v = a == 2 ? 1 : 2;
        g->dft_face[f + 1] =
            g->dft_face[f] + (g->dft_max[u] - g->dft_min[u] + 1) * (g->dft_max[v] - g->dft_min[v] + 1);
    }
    g->dft_points = g->dft_face[6];
    g->dft_nf = nf;
    g->dft_w = (double*)malloc((size_t)nf * sizeof(double));
    for (int f = 0; f < nf; ++f) g->dft_w[f] = 6.28318530717958647692 / (double)(wavelengths[f] > 2.0f ? wavelengths[f] : 2.0f);
    g->dft = (double*)calloc((size_t)nf * g->dft_points * 12, sizeof(double));
    g->dft_on = 1;
    return EMLAB_OK;
}

int NAME(oracle_ntff_dft_points)(void* h) { return ((NAME(grid)*)h)->dft_points; }

void NAME(oracle_ntff_dft_read)(void* h, double* out) {
    NAME(grid)* g = (NAME(grid)*)h;
    memcpy(out, g->dft, (size_t)g->dft_nf * g->dft_points * 12 * sizeof(double));
}

/* ---------------------------------------------------------------------------------------- */
void NAME(oracle_read_components)(void* h, R* ex, R* ey, R* ez, R* bx, R* by, R* bz) {
    NAME(grid)* g = (NAME(grid)*)h;
    R* out[6] = {ex, ey, ez, bx, by, bz};
    for (int c = 0; c < 6; ++c) {
        if (!out[c]) continue;
        const R* src = c < 3 ? g->E : g->B;
        for (int64_t i = 0; i < g->n; ++i) out[c][i] = src[i * 4 + (c % 3)];
    }
}

void NAME(oracle_write_components)(void* h, const R* ex, const R* ey, const R* ez, const R* bx, const R* by,
                                   const R* bz) {
    NAME(grid)* g = (NAME(grid)*)h;
    const R* in[6] = {ex, ey, ez, bx, by, bz};
    for (int c = 0; c < 6; ++c) {
        if (!in[c]) continue;
        R* dst = c < 3 ? g->E : g->B;
        for (int64_t i = 0; i < g->n; ++i) dst[i * 4 + (c % 3)] = in[c][i];
    }
}

/* PortMonitor::configure (Ports.cpp:43-75) */
int NAME(oracle_ports_configure)(void* h, const emlab_port* ports, size_t n, float wavelength, float avg, int sweep,
                                 size_t record_steps) {
    NAME(grid)* g = (NAME(grid)*)h;
    if (n > 256) n = 256;
    g->nports = (int)n;
    if (n) memcpy(g->ports, ports, n * sizeof(emlab_port));
    g->port_avg = avg > 0.5f ? avg : 0.5f;
    g->port_wavelength = wavelength > 2.0f ? wavelength : 2.0f;
    free(g->port_phasor), free(g->series);
    g->port_phasor = NULL, g->series = NULL;
    g->recorded = 0, g->series_cap = 0, g->recording = 0;
    if (!n) return EMLAB_OK;
    g->port_phasor = (R*)calloc(n * 8, sizeof(R));
    if (sweep || record_steps > 0) {
        size_t cap = ((size_t)1 << 23) / (2 * n);
        if (!sweep && record_steps < cap) cap = record_steps;
        g->series_cap = cap;
        g->series = (R*)calloc(cap * n * 2, sizeof(R));
        g->recording = 1;
    }
    return EMLAB_OK;
}

void NAME(oracle_ports_read_phasors)(void* h, R* out) {
    NAME(grid)* g = (NAME(grid)*)h;
    memcpy(out, g->port_phasor, (size_t)g->nports * 8 * sizeof(R));
}

size_t NAME(oracle_ports_read_series)(void* h, R* out, size_t max_steps) {
    NAME(grid)* g = (NAME(grid)*)h;
    size_t s = g->recorded < max_steps ? g->recorded : max_steps;
    if (out && s) memcpy(out, g->series, s * (size_t)g->nports * 2 * sizeof(R));
    return g->recorded;
}

/* PortMonitor::evaluateSweep sums (Ports.cpp:215-242), exact phase per sample */
void NAME(oracle_ports_sweep_sums)(void* h, double lmin, double lmax, int points, double* out, double* residual) {
    NAME(grid)* g = (NAME(grid)*)h;
    const size_t n = g->recorded, np = (size_t)g->nports;
    const double dt = (double)g->cfg.courant;
    const double nuLo = 1.0 / (lmax > lmin ? lmax : lmin), nuHi = 1.0 / (lmax < lmin ? lmax : lmin);
    if (points < 2) points = 2;
    double peak = 0.0, late = 0.0;
    const size_t tail = n / 20 > 1 ? n / 20 : 1;
    for (size_t k = 0; k < n; ++k) {
        const double v = fabs((double)g->series[k * np * 2]);
        peak = v > peak ? v : peak;
        if (k >= n - tail && v > late) late = v;
    }
    if (residual) *residual = peak > 0.0 ? late / peak : 1.0;
    for (size_t p = 0; p < np; ++p)
        for (int f = 0; f < points; ++f) {
            const double nu = nuLo + (nuHi - nuLo) * f / (points - 1);
            const double w = 6.28318530717958647692 * nu;
            double vr = 0, vi = 0, ir = 0, ii = 0;
            for (size_t k = 0; k < n; ++k) {
                const double ph = -w * dt * (double)k;
                const double c = cos(ph), s = sin(ph);
                const double V = (double)g->series[(k * np + p) * 2], I = (double)g->series[(k * np + p) * 2 + 1];
                vr += V * c, vi += V * s, ir += I * c, ii += I * s;
            }
            const double cr = cos(w * 0.5 * dt), ci = sin(w * 0.5 * dt);
            double* o = out + ((size_t)p * points + f) * 4;
            o[0] = vr, o[1] = vi, o[2] = ir * cr - ii * ci, o[3] = ir * ci + ii * cr;
        }
}

/* FarFieldMonitor::configure (FarField.cpp:126-174) */
int NAME(oracle_ntff_configure)(void* h, const int mn[3], const int mx[3], float wavelength, float avg, int box_out[6]) {
    NAME(grid)* g = (NAME(grid)*)h;
    free(g->ntff);
    g->ntff = NULL;
    g->ntff_on = 0;
    if (!(wavelength > 0.0f)) return EMLAB_OK;
    const int n[3] = {g->cfg.nx, g->cfg.ny, g->cfg.nz};
    const int L = g->cfg.pml_thickness;
    for (int a = 0; a < 3; ++a) {
        const int lo = L + 1, hi = n[a] - L - 2;
        int b0 = mn[a] < mx[a] ? mn[a] : mx[a], b1 = mn[a] < mx[a] ? mx[a] : mn[a];
        b0 = b0 < lo ? lo : (b0 > hi ? hi : b0);
        b1 = b1 < lo ? lo : (b1 > hi ? hi : b1);
        g->box_min[a] = b0, g->box_max[a] = b1;
        if (b1 - b0 < 4) return EMLAB_ERR_INVALID;
    }
    if (box_out)
        for (int a = 0; a < 3; ++a) box_out[a] = g->box_min[a], box_out[3 + a] = g->box_max[a];
    g->ntff_wavelength = wavelength > 2.0f ? wavelength : 2.0f;
    g->ntff_avg = avg > 0.5f ? avg : 0.5f;
    g->face_offset[0] = 0;
    for (int f = 0; f < 6; ++f) {
        const int a = f >> 1, u = a == 0 ? 1 : 0, v = a == 2 ? 1 : 2;
        g->face_offset[f + 1] =
            g->face_offset[f] + (g->box_max[u] - g->box_min[u] + 1) * (g->box_max[v] - g->box_min[v] + 1);
    }
    g->points = g->face_offset[6];
    g->ntff = (R*)calloc((size_t)g->points * 32, sizeof(R));
    g->ntff_on = 1;
    return EMLAB_OK;
}

int NAME(oracle_ntff_point_count)(void* h) { return ((NAME(grid)*)h)->points; }
void NAME(oracle_ntff_read_phasors)(void* h, R* out) {
    NAME(grid)* g = (NAME(grid)*)h;
    memcpy(out, g->ntff, (size_t)g->points * 32 * sizeof(R));
}

/* ntff_pattern.comp:45-110 + ntff_reduce.comp:19-39 for directions [0, n_dirs) in one dispatch
   (slices of FarField.cpp:297), out[2d] = |F|^2, out[1] = P/2 */
void NAME(oracle_ntff_evaluate)(void* h, const float* dirs, int n_dirs, R* out) {
    NAME(grid)* g = (NAME(grid)*)h;
    const int P = g->points;
    int slices = (P + 4095) / 4096;
    slices = slices < 1 ? 1 : (slices > 64 ? 64 : slices);
    const R k = (R)(float)(6.28318530717958647692 / (double)g->ntff_wavelength);
    const R cen[3] = {(R)(0.5f * (float)(g->box_min[0] + g->box_max[0])), (R)(0.5f * (float)(g->box_min[1] + g->box_max[1])),
                      (R)(0.5f * (float)(g->box_min[2] + g->box_max[2]))};
    const int per = (P + slices - 1) / slices;
    /* per-point surface currents, as staged into shared memory */
    R* cur = (R*)malloc((size_t)P * 16 * sizeof(R));
    R* pw = (R*)malloc((size_t)P * sizeof(R));
    for (int i = 0; i < P; ++i) {
        int node[3];
        R n[3], w;
        NAME(ntff_point)(g, i, node, n, &w);
        const R* ph = g->ntff + (size_t)i * 32 + 16; /* stage2 */
        const R* eRe = ph, *eIm = ph + 4, *hRe = ph + 8, *hIm = ph + 12;
        R* c = cur + (size_t)i * 16;
        for (int a = 0; a < 3; ++a) c[a] = (R)node[a] - cen[a];
        /* GLSL cross(x, y) = (x1 y2 - y1 x2, x2 y0 - y2 x0, x0 y1 - y0 x1) */
#define OR_CROSS(o, X, Y)                  \
    o[0] = X[1] * Y[2] - Y[1] * X[2];      \
    o[1] = X[2] * Y[0] - Y[2] * X[0];      \
    o[2] = X[0] * Y[1] - Y[0] * X[1];
        R t[3];
        OR_CROSS(t, n, hRe);
        for (int a = 0; a < 3; ++a) c[4 + a] = w * t[a];
        OR_CROSS(t, n, hIm);
        for (int a = 0; a < 3; ++a) c[8 + a] = w * t[a];
        OR_CROSS(t, n, eRe);
        for (int a = 0; a < 3; ++a) c[12 + a] = -w * t[a];
        OR_CROSS(t, n, eIm);
        R mi[3];
        for (int a = 0; a < 3; ++a) mi[a] = -w * t[a];
        /* c[3], c[7], c[11], c[15] unused slots: M imaginary kept separately below */
        c[3] = mi[0], c[7] = mi[1], c[11] = mi[2];
        R x1[3], x2[3];
        OR_CROSS(x1, eRe, hRe);
        OR_CROSS(x2, eIm, hIm);
        const R s[3] = {x1[0] + x2[0], x1[1] + x2[1], x1[2] + x2[2]};
        pw[i] = w * (s[0] * n[0] + s[1] * n[1] + s[2] * n[2]);
    }
    /* power: direction 0's slice partials (tree reduction of 128 per-thread sums) */
    double Ptot = 0.0;
    R Pslices = (R)0;
    for (int sl = 0; sl < slices; ++sl) {
        const int first = sl * per, last = first + per < P ? first + per : P;
        R acc[128];
        for (int l = 0; l < 128; ++l) acc[l] = (R)0;
        for (int base = first; base < last; base += 128)
            for (int l = 0; l < 128; ++l) {
                const int i = base + l;
                if (i < last) acc[l] = acc[l] + pw[i];
            }
        for (int stride = 64; stride > 0; stride >>= 1)
            for (int l = 0; l < stride; ++l) acc[l] = acc[l] + acc[l + stride];
        Pslices = Pslices + acc[0];
    }
    (void)Ptot;
#pragma omp parallel for schedule(dynamic, 16)
    for (int d = 0; d < n_dirs; ++d) {
        const R r[3] = {(R)dirs[d * 4 + 0], (R)dirs[d * 4 + 1], (R)dirs[d * 4 + 2]};
        R N[2][3] = {{0, 0, 0}, {0, 0, 0}}, Lv[2][3] = {{0, 0, 0}, {0, 0, 0}};
        for (int sl = 0; sl < slices; ++sl) {
            const int first = sl * per, last = first + per < P ? first + per : P;
            R Nr[3] = {0, 0, 0}, Ni[3] = {0, 0, 0}, Lr[3] = {0, 0, 0}, Li[3] = {0, 0, 0};
            for (int i = first; i < last; ++i) {
                const R* c = cur + (size_t)i * 16;
                const R psi = k * (r[0] * c[0] + r[1] * c[1] + r[2] * c[2]);
#if OR_DOUBLE
                const R cs = cos(psi), sn = sin(psi);
#else
                const R cs = cosf(psi), sn = sinf(psi);
#endif
                const R jr[3] = {c[4], c[5], c[6]}, ji[3] = {c[8], c[9], c[10]};
                const R mr[3] = {c[12], c[13], c[14]}, mi[3] = {c[3], c[7], c[11]};
                for (int a = 0; a < 3; ++a) {
                    Nr[a] = Nr[a] + (jr[a] * cs - ji[a] * sn);
                    Ni[a] = Ni[a] + (jr[a] * sn + ji[a] * cs);
                    Lr[a] = Lr[a] + (mr[a] * cs - mi[a] * sn);
                    Li[a] = Li[a] + (mr[a] * sn + mi[a] * cs);
                }
            }
            for (int a = 0; a < 3; ++a) {
                N[0][a] = N[0][a] + Nr[a], N[1][a] = N[1][a] + Ni[a];
                Lv[0][a] = Lv[0][a] + Lr[a], Lv[1][a] = Lv[1][a] + Li[a];
            }
        }
        R F2 = (R)0;
        for (int part = 0; part < 2; ++part) {
            const R dn = N[part][0] * r[0] + N[part][1] * r[1] + N[part][2] * r[2];
            R rl[3];
            OR_CROSS(rl, r, Lv[part]);
            R F[3];
            for (int a = 0; a < 3; ++a) F[a] = (N[part][a] - dn * r[a]) - rl[a];
            F2 = F2 + (F[0] * F[0] + F[1] * F[1] + F[2] * F[2]);
        }
        out[2 * d] = F2;
        out[2 * d + 1] = (R)0;
    }
#undef OR_CROSS
    if (n_dirs > 0) out[1] = (R)0.5 * Pslices;
    free(cur), free(pw);
}

/* CoaxMonitor line quantities (line_accumulate.comp:17-23) */
int NAME(oracle_lines_configure)(void* h, const int* q, int nq, const int* terms, const float* weights, int nterms,
                                 float wavelength, float avg) {
    NAME(grid)* g = (NAME(grid)*)h;
    free(g->q), free(g->terms), free(g->weights), free(g->line_phasor), free(g->line_now);
    g->q = NULL, g->terms = NULL, g->weights = NULL, g->line_phasor = NULL, g->line_now = NULL;
    g->nq = nq > 0 ? nq : 0;
    g->nterms = nterms;
    if (!g->nq) return EMLAB_OK;
    g->q = (int32_t*)malloc((size_t)nq * 4 * sizeof(int32_t));
    g->terms = (int32_t*)malloc((size_t)(nterms > 0 ? nterms : 1) * 4 * sizeof(int32_t));
    g->weights = (float*)malloc((size_t)(nterms > 0 ? nterms : 1) * sizeof(float));
    memcpy(g->q, q, (size_t)nq * 4 * sizeof(int32_t));
    if (nterms > 0) {
        memcpy(g->terms, terms, (size_t)nterms * 4 * sizeof(int32_t));
        memcpy(g->weights, weights, (size_t)nterms * sizeof(float));
    }
    g->line_wavelength = wavelength > 2.0f ? wavelength : 2.0f;
    g->line_avg = avg;
    g->line_phasor = (R*)calloc((size_t)nq * 4, sizeof(R));
    g->line_now = (R*)calloc((size_t)nq, sizeof(R));
    return EMLAB_OK;
}

void NAME(oracle_lines_read)(void* h, R* ph, R* now) {
    NAME(grid)* g = (NAME(grid)*)h;
    if (ph) memcpy(ph, g->line_phasor, (size_t)g->nq * 4 * sizeof(R));
    if (now) memcpy(now, g->line_now, (size_t)g->nq * sizeof(R));
}

/* probe_gather.comp:20-26 */
void NAME(oracle_probe_gather)(void* h, const int* origins, int n, R* out) {
    NAME(grid)* g = (NAME(grid)*)h;
    for (int id = 0; id < n * 54; ++id) {
        const int probe = id / 54, k = id % 54, t = k % 27;
        const int* o = origins + probe * 4;
        const int x = NAME(clampi)(o[0] + t % 3, 0, g->cfg.nx - 1);
        const int y = NAME(clampi)(o[1] + (t / 3) % 3, 0, g->cfg.ny - 1);
        const int z = NAME(clampi)(o[2] + t / 9, 0, g->cfg.nz - 1);
        const R* src = (k < 27 ? g->E : g->B) + NAME(idx)(g, x, y, z) * 4;
        for (int c = 0; c < 4; ++c) out[(size_t)id * 4 + c] = src[c];
    }
}

/* poynting_flux.comp:32-63 per plane, partials added in FP64 (FieldAnalyzer.cpp:356-357) */
void NAME(oracle_flux_planes)(void* h, const emlab_flux_plane* planes, int n, double* out) {
    NAME(grid)* g = (NAME(grid)*)h;
    const int size[3] = {g->cfg.nx, g->cfg.ny, g->cfg.nz};
    for (int pi = 0; pi < n; ++pi) {
        const emlab_flux_plane* pl = &planes[pi];
        out[pi] = 0.0;
        const int axis = pl->axis;
        if (pl->index < 0 || pl->index >= size[axis]) continue;
        const int u = axis == 0 ? 1 : 0, v = axis == 2 ? 1 : 2;
        int mn[2] = {pl->rect_min[0] > 0 ? pl->rect_min[0] : 0, pl->rect_min[1] > 0 ? pl->rect_min[1] : 0};
        int mx[2] = {pl->rect_max[0] < size[u] ? pl->rect_max[0] : size[u],
                     pl->rect_max[1] < size[v] ? pl->rect_max[1] : size[v]};
        const int rs[2] = {mx[0] - mn[0], mx[1] - mn[1]};
        if (rs[0] <= 0 || rs[1] <= 0) continue;
        const int gx = (rs[0] + 15) / 16, gy = (rs[1] + 15) / 16;
        double sum = 0.0;
        for (int by = 0; by < gy; ++by)
            for (int bx = 0; bx < gx; ++bx) {
                R part[256];
                for (int ly = 0; ly < 16; ++ly)
                    for (int lx = 0; lx < 16; ++lx) {
                        const int lu = bx * 16 + lx, lv = by * 16 + ly;
                        R flux = (R)0;
                        if (lu < rs[0] && lv < rs[1]) {
                            int p[3];
                            p[axis] = pl->index, p[u] = mn[0] + lu, p[v] = mn[1] + lv;
                            if (p[0] >= 0 && p[1] >= 0 && p[2] >= 0 && p[0] < size[0] && p[1] < size[1] && p[2] < size[2]) {
                                R E[3], Bn[3];
                                NAME(e_at_node)(g, p[0], p[1], p[2], E);
                                NAME(b_at_node)(g, p[0], p[1], p[2], Bn);
                                const R S[3] = {E[1] * Bn[2] - Bn[1] * E[2], E[2] * Bn[0] - Bn[2] * E[0],
                                                E[0] * Bn[1] - Bn[0] * E[1]};
                                flux = S[axis];
                            }
                        }
                        part[ly * 16 + lx] = flux;
                    }
                for (int stride = 128; stride > 0; stride >>= 1)
                    for (int l = 0; l < stride; ++l) part[l] = part[l] + part[l + stride];
                sum += (double)part[0];
            }
        out[pi] = sum;
    }
}
