// ref_driver.cpp - runs the reference's own shader bodies (rewritten into oracle/_ref/*.hpp by
// oracle/build_ref.py) over the CPU, dispatch for dispatch, in the order of SimulationGrid::step
// (src/SimulationGrid.cpp:368-433) and Instruments::onStep (src/Instruments.cpp:189-195).
// TEST INFRASTRUCTURE: it pins the CPU restatement (oracle/emlab_oracle.c) to the reference.
//
// Host-side set-up (edge averaging, binary16 packing, source lists, signals) comes from the
// restatement's C functions, linked into the same library; only the shader arithmetic is the
// reference's. Workgroups with barrier() run their invocations as ucontext fibers.
#include <ucontext.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "glsl_shim.hpp"

extern "C" {
#include "../include/emlab.h"
void oracle_clamp_config(emlab_grid_config* c);
void oracle_edge_average(const float* sig, const float* eps, int nx, int ny, int nz, const emlab_edge_override* edges,
                         size_t ne, float** out_sig, float** out_eps);
void oracle_wire_factors(int nx, int ny, int nz, const emlab_wire_term* w, size_t nw, float** out0, float** out1);
int oracle_pack_sources(const emlab_source* s, size_t n, emlab_source* desc, float (*src)[16]);
int oracle_source_lists(float (*src)[16], int nsrc, const int n[3], int32_t** out_cells, int32_t** out_lists);
double oracle_signal(const emlab_source* s, double tAbs);
}

namespace glsl {
bool g_libm_exp = false;
thread_local uvec3 gl_GlobalInvocationID;
thread_local uvec3 gl_WorkGroupID;
thread_local uint gl_LocalInvocationIndex;
thread_local uvec3 gl_NumWorkGroups;
thread_local void (*g_barrier_hook)() = nullptr;

namespace sh_update_B {
#include "update_B.comp.hpp"
}
namespace sh_update_E {
#include "update_E.comp.hpp"
}
namespace sh_apply_sources {
#include "apply_sources.comp.hpp"
}
namespace sh_clear {
#include "clear_fields.comp.hpp"
}
namespace sh_port {
#include "port_accumulate.comp.hpp"
}
namespace sh_probe {
#include "probe_gather.comp.hpp"
}
namespace sh_flux {
#include "poynting_flux.comp.hpp"
}
namespace sh_ntff_acc {
#include "ntff_accumulate.comp.hpp"
}
namespace sh_ntff_pat {
#include "ntff_pattern.comp.hpp"
}
namespace sh_ntff_red {
#include "ntff_reduce.comp.hpp"
}
namespace sh_lines {
#include "line_accumulate.comp.hpp"
}
thread_local vec4 gl_FragCoord;
namespace sh_raymarch {
#include "raymarch.frag.hpp"
}
}  // namespace glsl

using namespace glsl;

namespace {

// ---- fibers for workgroups with barriers ------------------------------------------------------
struct FiberGroup {
    static constexpr size_t kStack = 64 * 1024;
    ucontext_t sched;
    std::vector<ucontext_t> ctx;
    std::vector<std::vector<char>> stacks;
    std::vector<int> state;  // 0 runnable, 1 at a barrier, 2 finished
    int cur = 0;
    void (*body)() = nullptr;
    uvec3 group_id, groups, local_size;
};
thread_local FiberGroup* tl_group = nullptr;

void fiber_barrier() {
    FiberGroup* g = tl_group;
    const int i = g->cur;
    g->state[i] = 1;
    swapcontext(&g->ctx[i], &g->sched);
}

void fiber_entry() {
    FiberGroup* g = tl_group;
    const int i = g->cur;
    g->body();
    g->state[i] = 2;
}

void set_ids(FiberGroup& g, int i) {
    const uint lx = (uint)i % g.local_size.x, ly = (uint)i / g.local_size.x;
    gl_LocalInvocationIndex = (uint)i;
    gl_WorkGroupID = g.group_id;
    gl_NumWorkGroups = g.groups;
    gl_GlobalInvocationID = uvec3{g.group_id.x * g.local_size.x + lx, g.group_id.y * g.local_size.y + ly, 0};
}

// One workgroup of local size lx * ly, every invocation as a fiber; barrier() suspends.
void run_group(void (*body)(), uvec3 group, uvec3 groups, uint lx, uint ly) {
    thread_local FiberGroup fg;
    const int n = (int)(lx * ly);
    if ((int)fg.ctx.size() < n) {
        fg.ctx.resize(n);
        fg.stacks.resize(n);
        for (auto& s : fg.stacks) s.resize(FiberGroup::kStack);
    }
    fg.state.assign(n, 0);
    fg.body = body;
    fg.group_id = group, fg.groups = groups, fg.local_size = uvec3{lx, ly, 1};
    tl_group = &fg;
    g_barrier_hook = fiber_barrier;
    for (int i = 0; i < n; ++i) {
        getcontext(&fg.ctx[i]);
        fg.ctx[i].uc_stack.ss_sp = fg.stacks[i].data();
        fg.ctx[i].uc_stack.ss_size = FiberGroup::kStack;
        fg.ctx[i].uc_link = &fg.sched;
        makecontext(&fg.ctx[i], fiber_entry, 0);
    }
    for (;;) {
        bool any = false;
        for (int i = 0; i < n; ++i) {
            if (fg.state[i] == 2) continue;
            any = true;
            fg.state[i] = 0;
            fg.cur = i;
            set_ids(fg, i);
            swapcontext(&fg.sched, &fg.ctx[i]);
        }
        if (!any) break;
    }
    g_barrier_hook = nullptr;
    tl_group = nullptr;
}

struct RefGrid {
    emlab_grid_config cfg{};
    ivec3 n;
    long long cells = 0;
    std::vector<float> E, B;           // RGBA textures
    std::vector<uint32_t> edge, wire;  // RGBA32UI textures
    ivec3 wire_size;
    bool thin = false;
    int nsrc = 0;
    emlab_source desc[256];
    float src[256][16];
    int ncells = 0;
    int32_t* cells_buf = nullptr;
    int32_t* lists = nullptr;
    std::vector<float> signals;
    uint64_t step = 0;
    // ports
    std::vector<sh_port::Port> ports;
    std::vector<sh_port::PortPhasor> port_ph;
    std::vector<vec2> series;
    size_t series_cap = 0, recorded = 0;
    bool recording = false;
    float port_wl = 16, port_avg = 4;
    // ntff
    bool ntff_on = false;
    ivec3 bmin, bmax;
    int face[7] = {};
    int points = 0;
    float ntff_wl = 16, ntff_avg = 4;
    std::vector<sh_ntff_acc::PhasorPair> ntff;
    // lines
    std::vector<ivec4> q, terms;
    std::vector<float> weights, now;
    std::vector<vec4> line_ph;
    float line_wl = 16, line_avg = 4;
};

uint32_t pack2(float a, float b) { return (uint32_t)emlab_float_to_half(a) | ((uint32_t)emlab_float_to_half(b) << 16); }

#define SOLVER_UNIFORMS(NS)                            \
    NS::uGridSize = g.n;                               \
    NS::uDt = g.cfg.courant;                           \
    NS::uPmlThickness = g.cfg.pml_thickness;           \
    NS::uPmlSigmaMax = g.cfg.pml_sigma_max;            \
    NS::uPmlGrading = g.cfg.pml_grading;

void for_cells(const RefGrid& g, void (*body)()) {
#pragma omp parallel for schedule(static)
    for (int z = 0; z < g.n.z; ++z)
        for (int y = 0; y < g.n.y; ++y)
            for (int x = 0; x < g.n.x; ++x) {
                gl_GlobalInvocationID = uvec3{(uint)x, (uint)y, (uint)z};
                body();
            }
}

void for_ids(int count, void (*body)()) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < count; ++i) {
        gl_GlobalInvocationID = uvec3{(uint)i, 0, 0};
        body();
    }
}

void rotation(double w, double tE, double dt, vec4& r, float& blend, float avg, float wl) {
    const double tH = tE - 0.5 * dt;
    r = vec4((float)std::cos(w * tE), (float)std::sin(w * tE), (float)std::cos(w * tH), (float)std::sin(w * tH));
    const double tau = (double)avg * (double)wl;
    blend = (float)(1.0 - std::exp(-dt / (0.5 * tau)));
}

void dispatch_step(RefGrid& g, int k) {
    (void)k;
    {  // update_B.comp (SimulationGrid.cpp:394-400)
        namespace S = sh_update_B;
        SOLVER_UNIFORMS(S)
        S::uBField = image3D{g.B.data(), g.n};
        S::uEField = sampler3D{g.E.data(), g.n};
        S::uWireCoef = usampler3D{g.wire.data(), g.wire_size};
        S::uThinWires = g.thin ? 1 : 0;
        for_cells(g, S::main);
    }
    {  // update_E.comp (:402-408)
        namespace S = sh_update_E;
        SOLVER_UNIFORMS(S)
        S::uEField = image3D{g.E.data(), g.n};
        S::uBField = sampler3D{g.B.data(), g.n};
        S::uEdgeMaterial = usampler3D{g.edge.data(), g.n};
        for_cells(g, S::main);
    }
    if (g.ncells > 0) {  // apply_sources.comp (:410-420)
        namespace S = sh_apply_sources;
        SOLVER_UNIFORMS(S)
        S::uEField = image3D{g.E.data(), g.n};
        S::uEdgeMaterial = usampler3D{g.edge.data(), g.n};
        S::uSources = reinterpret_cast<S::Source*>(g.src);
        S::uSignals = g.signals.data();
        S::uCells = reinterpret_cast<ivec4*>(g.cells_buf);
        S::uSourceList = g.lists;
        S::uCellCount = g.ncells;
        S::uSignalBase = 0;
        for_ids(g.ncells, S::main);
    }
    ++g.step;
    const double dt = (double)g.cfg.courant, tE = (double)g.step * dt;
    if (g.ntff_on) {  // FarFieldMonitor::accumulate (FarField.cpp:198-217)
        namespace S = sh_ntff_acc;
        S::uEField = sampler3D{g.E.data(), g.n};
        S::uBField = sampler3D{g.B.data(), g.n};
        S::uGridSize = g.n;
        S::uBoxMin = g.bmin, S::uBoxMax = g.bmax;
        for (int i = 0; i < 7; ++i) S::uFaceOffset[i] = g.face[i];
        S::uPhasors = g.ntff.data();
        S::uPointCount = g.points;
        rotation(6.28318530717958647692 / g.ntff_wl, tE, dt, S::uRotation, S::uBlend, g.ntff_avg, g.ntff_wl);
        for_ids(g.points, S::main);
    }
    if (!g.ports.empty()) {  // PortMonitor::accumulate (Ports.cpp:113-136)
        namespace S = sh_port;
        S::uEField = sampler3D{g.E.data(), g.n};
        S::uBField = sampler3D{g.B.data(), g.n};
        S::uGridSize = g.n;
        S::uPortCount = (int)g.ports.size();
        S::uPorts = g.ports.data();
        S::uPhasors = g.port_ph.data();
        S::uSeries = g.series.empty() ? nullptr : g.series.data();
        rotation(6.28318530717958647692 / g.port_wl, tE, dt, S::uRotation, S::uBlend, g.port_avg, g.port_wl);
        const bool record = g.recording && g.recorded < g.series_cap;
        S::uRecordIndex = record ? (int)g.recorded : -1;
        for_ids((int)g.ports.size(), S::main);
        if (record) ++g.recorded;
    }
    if (!g.q.empty()) {  // CoaxMonitor::accumulate (Coax.cpp:179-197)
        namespace S = sh_lines;
        S::uEField = sampler3D{g.E.data(), g.n};
        S::uBField = sampler3D{g.B.data(), g.n};
        S::uGridSize = g.n;
        S::uCount = (int)g.q.size();
        S::uQuantities = g.q.data();
        S::uTerms = g.terms.data();
        S::uWeights = g.weights.data();
        S::uPhasors = g.line_ph.data();
        S::uNow = g.now.data();
        rotation(6.28318530717958647692 / g.line_wl, tE, dt, S::uRotation, S::uBlend, g.line_avg, g.line_wl);
        for_ids((int)g.q.size(), S::main);
    }
}

}  // namespace

extern "C" {

void* oracle_create_ref(const emlab_grid_config* req, int use_libm) {
    RefGrid* g = new RefGrid();
    g->cfg = *req;
    oracle_clamp_config(&g->cfg);
    g->n = ivec3(g->cfg.nx, g->cfg.ny, g->cfg.nz);
    g->cells = (long long)g->cfg.nx * g->cfg.ny * g->cfg.nz;
    g->E.assign((size_t)g->cells * 4, 0.0f);
    g->B.assign((size_t)g->cells * 4, 0.0f);
    for (long long i = 0; i < g->cells; ++i) g->B[(size_t)i * 4 + 3] = 1.0f;
    g->edge.assign((size_t)g->cells * 4, 0u);
    for (long long i = 0; i < g->cells; ++i) {  // SimulationGrid.cpp:190-192
        g->edge[(size_t)i * 4 + 0] = pack2(0.0f, 0.0f);
        g->edge[(size_t)i * 4 + 1] = pack2(0.0f, 1.0f);
        g->edge[(size_t)i * 4 + 2] = pack2(1.0f, 1.0f);
    }
    g->wire.assign(4, pack2(1.0f, 1.0f));
    g->wire_size = ivec3(1);
    glsl::g_libm_exp = use_libm != 0;
    return g;
}

void oracle_destroy_ref(void* h) {
    RefGrid* g = (RefGrid*)h;
    if (!g) return;
    free(g->cells_buf);
    free(g->lists);
    delete g;
}

void oracle_get_config_ref(void* h, emlab_grid_config* out) { *out = ((RefGrid*)h)->cfg; }
uint64_t oracle_step_count_ref(void* h) { return ((RefGrid*)h)->step; }
int oracle_source_cells_ref(void* h) { return ((RefGrid*)h)->ncells; }

int oracle_upload_materials_ref(void* h, const float* sig, const float* eps, int nx, int ny, int nz,
                                const emlab_edge_override* edges, size_t ne, const emlab_wire_term* wires, size_t nw) {
    RefGrid* g = (RefGrid*)h;
    if (nx != g->cfg.nx || ny != g->cfg.ny || nz != g->cfg.nz) return EMLAB_ERR_INVALID;
    float *es = nullptr, *ee = nullptr;
    oracle_edge_average(sig, eps, nx, ny, nz, edges, ne, &es, &ee);
    for (long long i = 0; i < g->cells; ++i) {
        float* e = &g->E[(size_t)i * 4];
        float* b = &g->B[(size_t)i * 4];
        e[0] = e[1] = e[2] = 0.0f, e[3] = sig[i];
        b[0] = b[1] = b[2] = 0.0f, b[3] = eps[i];
        const float* s = es + i * 3;
        const float* p = ee + i * 3;
        g->edge[(size_t)i * 4 + 0] = pack2(s[0], s[1]);
        g->edge[(size_t)i * 4 + 1] = pack2(s[2], p[0]);
        g->edge[(size_t)i * 4 + 2] = pack2(p[1], p[2]);
        g->edge[(size_t)i * 4 + 3] = 0u;
    }
    free(es), free(ee);
    g->thin = nw > 0;
    if (g->thin) {
        float *w0 = nullptr, *w1 = nullptr;
        oracle_wire_factors(nx, ny, nz, wires, nw, &w0, &w1);
        g->wire.assign((size_t)g->cells * 4, 0u);
        for (long long i = 0; i < g->cells; ++i)
            for (int c = 0; c < 3; ++c) g->wire[(size_t)i * 4 + c] = pack2(w0[i * 3 + c], w1[i * 3 + c]);
        free(w0), free(w1);
        g->wire_size = g->n;
    } else {
        g->wire.assign(4, pack2(1.0f, 1.0f));
        g->wire_size = ivec3(1);
    }
    g->step = 0;
    return EMLAB_OK;
}

int oracle_set_sources_ref(void* h, const emlab_source* s, size_t n) {
    RefGrid* g = (RefGrid*)h;
    free(g->cells_buf), free(g->lists);
    g->cells_buf = nullptr, g->lists = nullptr;
    g->nsrc = oracle_pack_sources(s, n, g->desc, g->src);
    const int dims[3] = {g->cfg.nx, g->cfg.ny, g->cfg.nz};
    g->ncells = oracle_source_lists(g->src, g->nsrc, dims, &g->cells_buf, &g->lists);
    return g->ncells < 0 ? EMLAB_ERR_OOM : EMLAB_OK;
}

void oracle_reset_fields_ref(void* h) {
    RefGrid* g = (RefGrid*)h;
    namespace S = sh_clear;  // clear_fields.comp
    S::uEField = image3D{g->E.data(), g->n};
    S::uBField = image3D{g->B.data(), g->n};
    S::uGridSize = g->n;
    for_cells(*g, S::main);
    g->step = 0;
}

void oracle_step_ref(void* h, int count) {
    RefGrid* g = (RefGrid*)h;
    for (int k = 0; k < count; ++k) {
        g->signals.assign((size_t)std::max(g->nsrc, 1), 0.0f);
        const double t = ((double)g->step + 0.5) * (double)g->cfg.courant;
        for (int s = 0; s < g->nsrc; ++s) g->signals[(size_t)s] = (float)oracle_signal(&g->desc[s], t);
        dispatch_step(*g, k);
    }
}

void oracle_read_components_ref(void* h, float* ex, float* ey, float* ez, float* bx, float* by, float* bz) {
    RefGrid* g = (RefGrid*)h;
    float* out[6] = {ex, ey, ez, bx, by, bz};
    for (int c = 0; c < 6; ++c) {
        if (!out[c]) continue;
        const std::vector<float>& t = c < 3 ? g->E : g->B;
        for (long long i = 0; i < g->cells; ++i) out[c][i] = t[(size_t)i * 4 + c % 3];
    }
}

void oracle_write_components_ref(void* h, const float* ex, const float* ey, const float* ez, const float* bx,
                                 const float* by, const float* bz) {
    RefGrid* g = (RefGrid*)h;
    const float* in[6] = {ex, ey, ez, bx, by, bz};
    for (int c = 0; c < 6; ++c) {
        if (!in[c]) continue;
        std::vector<float>& t = c < 3 ? g->E : g->B;
        for (long long i = 0; i < g->cells; ++i) t[(size_t)i * 4 + c % 3] = in[c][i];
    }
}

void oracle_edge_materials_ref(void* h, float* sig3, float* eps3, float* w0, float* w1) {
    RefGrid* g = (RefGrid*)h;
    for (long long i = 0; i < g->cells; ++i) {
        const vec2 a = unpackHalf2x16(g->edge[(size_t)i * 4]), b = unpackHalf2x16(g->edge[(size_t)i * 4 + 1]),
                   c = unpackHalf2x16(g->edge[(size_t)i * 4 + 2]);
        sig3[i * 3 + 0] = a.x, sig3[i * 3 + 1] = a.y, sig3[i * 3 + 2] = b.x;
        eps3[i * 3 + 0] = b.y, eps3[i * 3 + 1] = c.x, eps3[i * 3 + 2] = c.y;
        for (int k = 0; k < 3; ++k) {
            const vec2 w = g->thin ? unpackHalf2x16(g->wire[(size_t)i * 4 + k]) : vec2(1.0f, 1.0f);
            if (w0) w0[i * 3 + k] = w.x;
            if (w1) w1[i * 3 + k] = w.y;
        }
    }
}

int oracle_ports_configure_ref(void* h, const emlab_port* ports, size_t n, float wavelength, float avg, int sweep,
                               size_t record_steps) {
    RefGrid* g = (RefGrid*)h;
    n = std::min<size_t>(n, 256);
    g->ports.clear();
    for (size_t i = 0; i < n; ++i) {
        sh_port::Port p;
        p.texelAxis = ivec4(ports[i].x, ports[i].y, ports[i].z, ports[i].axis);
        p.info = ivec4(ports[i].edges, ports[i].sign >= 0 ? 1 : -1, 0, 0);
        g->ports.push_back(p);
    }
    g->port_ph.assign(n, sh_port::PortPhasor{});
    g->port_avg = std::max(avg, 0.5f);
    g->port_wl = std::max(wavelength, 2.0f);
    g->recorded = 0, g->series_cap = 0, g->recording = false;
    g->series.clear();
    if (n && (sweep || record_steps > 0)) {
        size_t cap = ((size_t)1 << 23) / (2 * n);
        if (!sweep) cap = std::min(cap, record_steps);
        g->series_cap = cap;
        g->series.assign(cap * n, vec2());
        g->recording = true;
    }
    return EMLAB_OK;
}

void oracle_ports_read_phasors_ref(void* h, float* out) {
    RefGrid* g = (RefGrid*)h;
    for (size_t i = 0; i < g->port_ph.size(); ++i) {
        const sh_port::PortPhasor& p = g->port_ph[i];
        const float v[8] = {p.stage1.x, p.stage1.y, p.stage1.z, p.stage1.w, p.stage2.x, p.stage2.y, p.stage2.z,
                            p.stage2.w};
        std::memcpy(out + i * 8, v, sizeof v);
    }
}

size_t oracle_ports_read_series_ref(void* h, float* out, size_t max_steps) {
    RefGrid* g = (RefGrid*)h;
    const size_t s = std::min(max_steps, g->recorded);
    for (size_t k = 0; out && k < s * g->ports.size(); ++k) out[2 * k] = g->series[k].x, out[2 * k + 1] = g->series[k].y;
    return g->recorded;
}

int oracle_ntff_configure_ref(void* h, const int mn[3], const int mx[3], float wavelength, float avg, int box_out[6]) {
    RefGrid* g = (RefGrid*)h;
    g->ntff_on = false;
    if (!(wavelength > 0.0f)) return EMLAB_OK;
    const int n[3] = {g->cfg.nx, g->cfg.ny, g->cfg.nz};
    const int L = g->cfg.pml_thickness;
    for (int a = 0; a < 3; ++a) {
        const int lo = L + 1, hi = n[a] - L - 2;
        g->bmin[a] = std::clamp(std::min(mn[a], mx[a]), lo, hi);
        g->bmax[a] = std::clamp(std::max(mn[a], mx[a]), lo, hi);
        if (g->bmax[a] - g->bmin[a] < 4) return EMLAB_ERR_INVALID;
        if (box_out) box_out[a] = g->bmin[a], box_out[3 + a] = g->bmax[a];
    }
    g->ntff_wl = std::max(wavelength, 2.0f);
    g->ntff_avg = std::max(avg, 0.5f);
    g->face[0] = 0;
    for (int f = 0; f < 6; ++f) {
        const int a = f >> 1, u = a == 0 ? 1 : 0, v = a == 2 ? 1 : 2;
        g->face[f + 1] = g->face[f] + (g->bmax[u] - g->bmin[u] + 1) * (g->bmax[v] - g->bmin[v] + 1);
    }
    g->points = g->face[6];
    g->ntff.assign((size_t)g->points, sh_ntff_acc::PhasorPair{});
    g->ntff_on = true;
    return EMLAB_OK;
}

int oracle_ntff_point_count_ref(void* h) { return ((RefGrid*)h)->points; }

void oracle_ntff_read_phasors_ref(void* h, float* out) {
    RefGrid* g = (RefGrid*)h;
    std::memcpy(out, g->ntff.data(), (size_t)g->points * 32 * sizeof(float));
}

// FarFieldMonitor::evaluate (FarField.cpp:226-243, 278-335): chunked pattern + reduce dispatches
void oracle_ntff_evaluate_ref(void* h, const float* dirs, int n_dirs, float* out) {
    RefGrid* g = (RefGrid*)h;
    const int slices = std::clamp((g->points + 4095) / 4096, 1, 64);
    const int chunk = std::clamp((int)(1.5e8 / std::max(g->points, 1)) / 128 * 128, 128, 4096);
    std::vector<vec4> d((size_t)n_dirs);
    for (int i = 0; i < n_dirs; ++i) d[(size_t)i] = vec4(dirs[i * 4], dirs[i * 4 + 1], dirs[i * 4 + 2], dirs[i * 4 + 3]);
    std::vector<vec4> partials((size_t)chunk * slices * 4);
    std::vector<float> o((size_t)n_dirs * 2, 0.0f);
    namespace P = sh_ntff_pat;
    namespace R = sh_ntff_red;
    P::uBoxMin = g->bmin, P::uBoxMax = g->bmax;
    for (int i = 0; i < 7; ++i) P::uFaceOffset[i] = g->face[i];
    P::uPhasors = reinterpret_cast<P::PhasorPair*>(g->ntff.data());
    P::uDirections = d.data();
    P::uPartials = partials.data();
    P::uPointCount = g->points;
    P::uSlices = slices;
    P::uK = (float)(6.28318530717958647692 / (double)g->ntff_wl);
    P::uCenter = 0.5f * vec3(ivec3(g->bmin.x + g->bmax.x, g->bmin.y + g->bmax.y, g->bmin.z + g->bmax.z));
    R::uDirections = d.data();
    R::uPartials = partials.data();
    R::uOut = o.data();
    R::uSlices = slices;
    for (int first = 0; first < n_dirs; first += chunk) {
        const int count = std::min(chunk, n_dirs - first);
        P::uDirectionOffset = first;
        P::uDirectionCount = first + count;
        const uint gx = (uint)((count + 127) / 128);
        const uvec3 groups{gx, (uint)slices, 1};
#pragma omp parallel for schedule(dynamic, 1)
        for (int gi = 0; gi < (int)(gx * slices); ++gi)
            run_group(P::main, uvec3{(uint)(gi % gx), (uint)(gi / gx), 0}, groups, 128, 1);
        R::uDirectionOffset = first;
        R::uDirectionCount = first + count;
        for_ids(count, R::main);
    }
    std::memcpy(out, o.data(), o.size() * sizeof(float));
}

int oracle_lines_configure_ref(void* h, const int* q, int nq, const int* terms, const float* weights, int nterms,
                               float wavelength, float avg) {
    RefGrid* g = (RefGrid*)h;
    g->q.clear(), g->terms.clear(), g->weights.clear();
    for (int i = 0; i < nq; ++i) g->q.emplace_back(q[i * 4], q[i * 4 + 1], q[i * 4 + 2], q[i * 4 + 3]);
    for (int i = 0; i < nterms; ++i) {
        g->terms.emplace_back(terms[i * 4], terms[i * 4 + 1], terms[i * 4 + 2], terms[i * 4 + 3]);
        g->weights.push_back(weights[i]);
    }
    g->line_ph.assign((size_t)std::max(nq, 0), vec4());
    g->now.assign((size_t)std::max(nq, 0), 0.0f);
    g->line_wl = std::max(wavelength, 2.0f);
    g->line_avg = avg;
    return EMLAB_OK;
}

void oracle_lines_read_ref(void* h, float* ph, float* now) {
    RefGrid* g = (RefGrid*)h;
    for (size_t i = 0; i < g->line_ph.size(); ++i) {
        if (ph) ph[i * 4] = g->line_ph[i].x, ph[i * 4 + 1] = g->line_ph[i].y, ph[i * 4 + 2] = g->line_ph[i].z,
                ph[i * 4 + 3] = g->line_ph[i].w;
        if (now) now[i] = g->now[i];
    }
}

void oracle_probe_gather_ref(void* h, const int* origins, int n, float* out) {
    RefGrid* g = (RefGrid*)h;
    namespace S = sh_probe;
    std::vector<ivec4> o;
    for (int i = 0; i < n; ++i) o.emplace_back(origins[i * 4], origins[i * 4 + 1], origins[i * 4 + 2], 0);
    std::vector<vec4> blocks((size_t)n * 54);
    S::uEField = sampler3D{g->E.data(), g->n};
    S::uBField = sampler3D{g->B.data(), g->n};
    S::uOrigins = o.data();
    S::uBlocks = blocks.data();
    S::uProbeCount = n;
    S::uGridSize = g->n;
    for_ids(n * 54, S::main);
    for (size_t i = 0; i < blocks.size(); ++i)
        out[i * 4] = blocks[i].x, out[i * 4 + 1] = blocks[i].y, out[i * 4 + 2] = blocks[i].z, out[i * 4 + 3] = blocks[i].w;
}

// FieldAnalyzer::dispatchPlane + FP64 sum of the partials (FieldAnalyzer.cpp:100-124, 356-357)
void oracle_flux_planes_ref(void* h, const emlab_flux_plane* planes, int n, double* out) {
    RefGrid* g = (RefGrid*)h;
    namespace S = sh_flux;
    const int size[3] = {g->cfg.nx, g->cfg.ny, g->cfg.nz};
    for (int pi = 0; pi < n; ++pi) {
        const emlab_flux_plane& p = planes[pi];
        out[pi] = 0.0;
        const int axis = std::clamp(p.axis, 0, 2);
        if (p.index < 0 || p.index >= size[axis]) continue;
        const int u = axis == 0 ? 1 : 0, v = axis == 2 ? 1 : 2;
        const int m0 = std::max(p.rect_min[0], 0), m1 = std::max(p.rect_min[1], 0);
        const int r0 = std::min(p.rect_max[0], size[u]) - m0, r1 = std::min(p.rect_max[1], size[v]) - m1;
        if (r0 <= 0 || r1 <= 0) continue;
        const uint gx = (uint)((r0 + 15) / 16), gy = (uint)((r1 + 15) / 16);
        std::vector<float> partials((size_t)gx * gy);
        S::uEField = sampler3D{g->E.data(), g->n};
        S::uBField = sampler3D{g->B.data(), g->n};
        S::uPartials = partials.data();
        S::uGridSize = g->n;
        S::uAxis = axis;
        S::uPlaneIndex = p.index;
        S::uRectMin = ivec2(m0, m1);
        S::uRectSize = ivec2(r0, r1);
        S::uPartialOffset = 0;
#pragma omp parallel for schedule(dynamic, 1)
        for (int gi = 0; gi < (int)(gx * gy); ++gi)
            run_group(S::main, uvec3{(uint)(gi % gx), (uint)(gi / gx), 0}, uvec3{gx, gy, 1}, 16, 16);
        double sum = 0.0;
        for (float f : partials) sum += (double)f;
        out[pi] = sum;
    }
}

// The volume pass (raymarch.frag) over the reference's two RGBA32F textures, one fragment per pixel
// centre of a width x height target (bottom row first), uniforms as VolumeRenderer::render sets
// them (src/VolumeRenderer.cpp:96-112), the RGBA8 target's unorm conversion rounding to nearest.
int oracle_render_ref(const float* e_rgba, const float* b_rgba, int nx, int ny, int nz, const emlab_render_params* p,
                      unsigned char* rgba) {
    namespace S = sh_raymarch;
    if (!e_rgba || !b_rgba || !p || !rgba || nx <= 0 || ny <= 0 || nz <= 0 || p->width <= 0 || p->height <= 0 ||
        !std::isfinite(p->step_voxels))
        return -1;
    for (int c = 0; c < 4; ++c)
        S::uInvViewProj.c[c] = vec4(p->inv_view_proj[4 * c], p->inv_view_proj[4 * c + 1], p->inv_view_proj[4 * c + 2],
                                    p->inv_view_proj[4 * c + 3]);
    S::uEField = sampler3D{e_rgba, ivec3(nx, ny, nz)};
    S::uBField = sampler3D{b_rgba, ivec3(nx, ny, nz)};
    S::uCamPos = vec3(p->cam_pos[0], p->cam_pos[1], p->cam_pos[2]);
    S::uVolMin = vec3(p->vol_min[0], p->vol_min[1], p->vol_min[2]);
    S::uVolSize = vec3(p->vol_size[0], p->vol_size[1], p->vol_size[2]);
    S::uClipMin = vec3(p->clip_min[0], p->clip_min[1], p->clip_min[2]);
    S::uClipMax = vec3(p->clip_max[0], p->clip_max[1], p->clip_max[2]);
    S::uGridSize = vec3((float)nx, (float)ny, (float)nz);
    S::uStepVoxels = std::clamp(p->step_voxels, 0.1f, 4.0f);
    S::uGainE = p->gain_e;
    S::uGainB = p->gain_b;
    S::uDensity = p->density;
    S::uEmission = p->emission;
    S::uMaterialOpacity = p->material_opacity;
    S::uExposure = p->exposure;
    S::uMode = p->mode;
    S::uSignedAxis = std::clamp(p->signed_axis, 0, 2);
    const int w = p->width, h = p->height;
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const float fx = (float)x + 0.5f, fy = (float)y + 0.5f;
            gl_FragCoord = vec4(fx, fy, 0.5f, 1.0f);
            S::vNdc = vec2(fx / (float)w * 2.0f - 1.0f, fy / (float)h * 2.0f - 1.0f);
            S::main();
            unsigned char* o = rgba + 4 * ((size_t)y * w + x);
            for (int k = 0; k < 4; ++k) o[k] = (unsigned char)lrintf(std::clamp(S::oColor[k], 0.0f, 1.0f) * 255.0f);
        }
    return 0;
}

}  // extern "C"
