// capi.cu - the C ABI (include/emlab.h): device buffers, the step loop and the monitors.
//
// SimulationGrid (src/SimulationGrid.cpp) keeps its state in GL textures and dispatches one compute
// pass per kernel per sub-step from the host. Here the state lives in plain device arrays owned by
// the handle, every launch goes to the handle's own CUDA stream, and the host only precomputes the
// per-step scalars the reference also computes on the host (source signals and monitor rotations,
// in FP64), uploading them once per chunk of steps.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/emlab.h"
#include "grid_state.h"

using namespace emlab;

namespace {

thread_local std::string g_last_error;
std::atomic<uint64_t> g_launches{0};
std::atomic<int> g_wait_polls{kWaitPolls};

}  // namespace

int emlab::wait_limit() { return g_wait_polls.load(); }

int emlab::fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

namespace {

YeeArgs yee_args(emlab_grid* g) {
    YeeArgs a{};
    a.nx = g->cfg.nx, a.ny = g->cfg.ny, a.nz = g->cfg.nz;
    a.pitch = g->pitch;
    a.plane = g->plane;
    const int c = g->cur, n = g->cur ^ 1;
    a.ex = g->comp(c, 0), a.ey = g->comp(c, 1), a.ez = g->comp(c, 2);
    a.bx = g->comp(c, 3), a.by = g->comp(c, 4), a.bz = g->comp(c, 5);
    a.nex = g->comp(n, 0), a.ney = g->comp(n, 1), a.nez = g->comp(n, 2);
    a.nbx = g->comp(n, 3), a.nby = g->comp(n, 4), a.nbz = g->comp(n, 5);
    a.wex = g->comp(c, 0), a.wey = g->comp(c, 1), a.wez = g->comp(c, 2);
    a.wbx = g->comp(c, 3), a.wby = g->comp(c, 4), a.wbz = g->comp(c, 5);
    a.cls = g->cls.p;
    a.tabE = g->tabE.p, a.tabM = g->tabM.p, a.tabW = g->tabW.p;
    a.wire_start = g->wire_start;
    a.pml = g->pml.p;
    a.pml_stride = g->pml_stride;
    a.pml_cls = g->pml_cls.p;
    a.pml_coef = g->pml_coef.p;
    a.pml_z = g->pml_z.p;
    a.pml_K = g->pml_K;
    a.L = g->cfg.pml_thickness;
    a.dt = g->cfg.courant;
    // tile height and z chunks: enough CTAs for ~4 per SM, but at least 8 planes each (the first
    // plane of a chunk is recomputed)
    const int mode = g->tile_rows == 0 ? 64 : g->tile_rows;  // automatic: 64 x 8 pair tiles
    const int ty = mode == 16 || mode == 128 ? 16 : (mode == 32 ? 4 : 8);
    const int tx = (mode == 32 || mode == 64 || mode == 128) && g->kernel == EMLAB_KERNEL_FUSED ? 64 : 32;
    a.tile_rows = g->kernel == EMLAB_KERNEL_FUSED ? mode : ty;
    const long long xy = (long long)((a.nx + tx - 1) / tx) * ((a.ny + ty - 1) / ty);
    const long long want = 152 * 4;
    int chunks = (int)std::max<long long>(1, (want + xy - 1) / xy);
    int zc = (a.nz + chunks - 1) / chunks;
    zc = std::max(zc, std::min(8, a.nz));
    a.zchunk = zc;
    a.work = g->d_work.p;
    a.work_base = g->work_base;
    a.wait_polls = wait_limit();
    a.pml_cls_xy = g->pml_cls.p, a.pml_xy = g->pml.p, a.pml_xy_stride = g->pml_stride, a.pml_xy_scene = 0;
    a.items = nullptr, a.n_items = 0, a.scene_xy = nullptr;
    if (g->stack.ragged) {
        const int ti = ty == 4 ? 0 : (ty == 8 ? 1 : 2);
        a.pml_cls_xy = g->d_pml_cls_xy.p, a.pml_xy = g->d_pml_xy.p;
        a.pml_xy_stride = g->pml_xy_stride, a.pml_xy_scene = 6 * g->pml_xy_stride;
        a.items = g->d_items[ti].p, a.n_items = g->n_items[ti];
        a.scene_xy = g->d_scene_xy.p;
    }
    return a;
}

MonitorArgs monitor_args(emlab_grid* g) {
    MonitorArgs m{};
    m.nx = g->cfg.nx, m.ny = g->cfg.ny, m.nz = g->cfg.nz, m.pitch = g->pitch, m.plane = g->plane;
    const int c = g->cur;
    m.ex = g->comp(c, 0), m.ey = g->comp(c, 1), m.ez = g->comp(c, 2);
    m.bx = g->comp(c, 3), m.by = g->comp(c, 4), m.bz = g->comp(c, 5);
    return m;
}

int check_launch() {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(EMLAB_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return EMLAB_OK;
}

}  // namespace

void emlab::invalidate_graphs(emlab_grid* g) {
    for (auto& row : g->graph_exec)
        for (auto& e : row)
            if (e) cudaGraphExecDestroy(e), e = nullptr;
}

int emlab::upload_class_table(emlab_grid* g, const ClassTable& t) {
    invalidate_graphs(g);
    const long long ncls = (long long)t.cls.size();
    g->wide = t.classes > 65536u;
    EMLAB_CUDA(g->cls.alloc((size_t)ncls * (g->wide ? 4 : 2)));
    if (g->wide) {
        EMLAB_CUDA(cudaMemcpyAsync(g->cls.p, t.cls.data(), (size_t)ncls * 4, cudaMemcpyHostToDevice, g->stream));
        EMLAB_CUDA(cudaStreamSynchronize(g->stream));
    } else {
        std::vector<uint16_t> narrow((size_t)ncls);
        for (long long i = 0; i < ncls; ++i) narrow[(size_t)i] = (uint16_t)t.cls[(size_t)i];
        EMLAB_CUDA(cudaMemcpyAsync(g->cls.p, narrow.data(), (size_t)ncls * 2, cudaMemcpyHostToDevice, g->stream));
        EMLAB_CUDA(cudaStreamSynchronize(g->stream));
    }
    EMLAB_CUDA(g->tabE.alloc(t.classes * 2));
    EMLAB_CUDA(g->tabM.alloc(t.classes * 2));
    EMLAB_CUDA(g->tabW.alloc(t.classes * 2));
    EMLAB_CUDA(cudaMemcpyAsync(g->tabE.p, t.tabE.data(), t.tabE.size() * 4, cudaMemcpyHostToDevice, g->stream));
    EMLAB_CUDA(cudaMemcpyAsync(g->tabM.p, t.tabM.data(), t.tabM.size() * 4, cudaMemcpyHostToDevice, g->stream));
    EMLAB_CUDA(cudaMemcpyAsync(g->tabW.p, t.tabW.data(), t.tabW.size() * 4, cudaMemcpyHostToDevice, g->stream));
    g->classes = t.classes;
    g->wire_start = t.wire_start;
    return EMLAB_OK;
}

// Tensor maps of both field generations and the class index (the TMA kernel's inputs).
void emlab::refresh_tma(emlab_grid* g) {
    invalidate_graphs(g);
    if (!g->tma) g->tma = tma_maps_create();
    const int cur = g->cur;
    for (int gen = 0; gen < 2; ++gen) {
        g->cur = gen;
        tma_maps_encode(g->tma, gen, yee_args(g), g->wide);
    }
    g->cur = cur;
}

int emlab::clear_fields(emlab_grid* g) {
    EMLAB_CUDA(cudaMemsetAsync(g->fields.p, 0, g->fields.n * sizeof(float), g->stream));
    g->cur = 0;
    return cpml_clear(g);
}

// Absorber tables of the configured size (common.glsl:23-43). In a stack, the z entries are each
// scene's own tables at its planes; separator planes lie outside every layer.
int emlab::upload_pml(emlab_grid* g) {
    invalidate_graphs(g);
    emlab_grid_config c = g->cfg;
    if (g->cpml_on) c.pml_sigma_max = 0.0f;  // the convolutional PML replaces the graded conductivity
    const int S = std::max(c.nx, std::max(c.ny, c.nz));
    g->pml_stride = S;
    std::vector<float> pt = pml_tables(c, S);
    std::vector<uint8_t> pcls;
    std::vector<float> coef;
    pml_class_tables(c, S, pcls, coef, g->pml_K);
    std::vector<uint8_t> pz((size_t)c.nz, 0);
    const int L = c.pml_thickness;
    if (g->stack.scenes() == 0) {
        for (int z = 0; z < c.nz; ++z) pz[(size_t)z] = (z < L || z >= c.nz - (L + 1)) ? 1 : 0;
    } else {
        for (int z = 0; z < c.nz; ++z) {  // separators: no absorber
            pt[(size_t)2 * S + z] = 0.0f, pt[(size_t)5 * S + z] = 0.0f;
            pcls[(size_t)2 * S + z] = 0, pcls[(size_t)5 * S + z] = 0;
        }
        for (int i = 0; i < g->stack.scenes(); ++i) {
            emlab_grid_config ci = c;
            ci.nz = g->stack.nz[i];
            const int Si = std::max(ci.nx, std::max(ci.ny, ci.nz));
            const std::vector<float> ti = pml_tables(ci, Si);
            std::vector<uint8_t> ci_cls;
            std::vector<float> ci_coef;
            int Ki = 0;
            pml_class_tables(ci, Si, ci_cls, ci_coef, Ki);
            for (int z = 0; z < ci.nz; ++z) {
                const size_t zz = (size_t)g->stack.z0[i] + z;
                pt[2 * (size_t)S + zz] = ti[2 * (size_t)Si + z];
                pt[5 * (size_t)S + zz] = ti[5 * (size_t)Si + z];
                pcls[2 * (size_t)S + zz] = ci_cls[2 * (size_t)Si + z];
                pcls[5 * (size_t)S + zz] = ci_cls[5 * (size_t)Si + z];
                pz[zz] = (z < L || z >= ci.nz - (L + 1)) ? 1 : 0;
            }
        }
    }
    if (g->stack.ragged) {
        // every scene's own x / y profiles and depth classes ([6][SXY] per scene, rows 0, 1, 3, 4 used),
        // its nx, ny, and the pair kernel's work items for each tile height
        const StackLayout& st = g->stack;
        const int n = st.scenes(), SXY = std::max(c.nx, c.ny);
        std::vector<float> pxy((size_t)n * 6 * SXY, 0.0f);
        std::vector<uint8_t> cxy((size_t)n * 6 * SXY, 0);
        std::vector<int2> dims((size_t)n);
        for (int i = 0; i < n; ++i) {
            emlab_grid_config ci = c;
            ci.nx = st.nx[(size_t)i], ci.ny = st.ny[(size_t)i], ci.nz = st.nz[(size_t)i];
            const int Si = std::max(ci.nx, std::max(ci.ny, ci.nz));
            const std::vector<float> ti = pml_tables(ci, Si);
            std::vector<uint8_t> ci_cls;
            std::vector<float> ci_coef;
            int Ki = 0;
            pml_class_tables(ci, Si, ci_cls, ci_coef, Ki);
            if (Ki != g->pml_K || ci_coef != coef)
                return fail(EMLAB_ERR_INVALID, "stack: scenes' absorber coefficient tables differ");
            for (int r : {0, 1, 3, 4}) {
                const int len = (r == 0 || r == 3) ? ci.nx : ci.ny;
                for (int p = 0; p < len; ++p) {
                    pxy[((size_t)i * 6 + r) * SXY + p] = ti[(size_t)r * Si + p];
                    cxy[((size_t)i * 6 + r) * SXY + p] = ci_cls[(size_t)r * Si + p];
                }
            }
            dims[(size_t)i] = make_int2(ci.nx, ci.ny);
        }
        g->pml_xy_stride = SXY;
        EMLAB_CUDA(g->d_pml_xy.alloc(pxy.size()));
        EMLAB_CUDA(cudaMemcpyAsync(g->d_pml_xy.p, pxy.data(), pxy.size() * 4, cudaMemcpyHostToDevice, g->stream));
        EMLAB_CUDA(g->d_pml_cls_xy.alloc(cxy.size()));
        EMLAB_CUDA(cudaMemcpyAsync(g->d_pml_cls_xy.p, cxy.data(), cxy.size(), cudaMemcpyHostToDevice, g->stream));
        EMLAB_CUDA(g->d_scene_xy.alloc(dims.size()));
        EMLAB_CUDA(cudaMemcpyAsync(g->d_scene_xy.p, dims.data(), dims.size() * 8, cudaMemcpyHostToDevice, g->stream));
        int dev = 0, sms = 0;
        EMLAB_CUDA(cudaGetDevice(&dev));
        EMLAB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const int tys[3] = {4, 8, 16}, per_sm[3] = {4, 2, 1};
        for (int t = 0; t < 3; ++t) {
            const std::vector<int4> items = ragged_items(st.z0, st.nx, st.ny, st.nz, tys[t], per_sm[t] * sms);
            EMLAB_REQUIRE(!items.empty(), "stack: no work items");
            EMLAB_CUDA(g->d_items[t].alloc(items.size()));
            EMLAB_CUDA(cudaMemcpyAsync(g->d_items[t].p, items.data(), items.size() * 16, cudaMemcpyHostToDevice, g->stream));
            g->n_items[t] = (int)items.size();
        }
    } else {
        for (auto& d : g->d_items) d.release();
        g->n_items[0] = g->n_items[1] = g->n_items[2] = 0;
        g->d_scene_xy.release(), g->d_pml_cls_xy.release(), g->d_pml_xy.release();
    }
    EMLAB_CUDA(g->pml.alloc(pt.size()));
    EMLAB_CUDA(cudaMemcpyAsync(g->pml.p, pt.data(), pt.size() * 4, cudaMemcpyHostToDevice, g->stream));
    EMLAB_CUDA(g->pml_cls.alloc(pcls.size()));
    EMLAB_CUDA(cudaMemcpyAsync(g->pml_cls.p, pcls.data(), pcls.size(), cudaMemcpyHostToDevice, g->stream));
    EMLAB_CUDA(g->pml_coef.alloc(coef.size() / 2));
    EMLAB_CUDA(cudaMemcpyAsync(g->pml_coef.p, coef.data(), coef.size() * 4, cudaMemcpyHostToDevice, g->stream));
    EMLAB_CUDA(g->pml_z.alloc(pz.size()));
    EMLAB_CUDA(cudaMemcpyAsync(g->pml_z.p, pz.data(), pz.size(), cudaMemcpyHostToDevice, g->stream));
    return EMLAB_OK;
}

// Packed sources and their per-cell lists on the device (zoff: empty for a single scene).
int emlab::upload_sources(emlab_grid* g, const std::vector<float>& packed, const std::vector<int32_t>& cells,
                          const std::vector<int32_t>& lists, const std::vector<int32_t>& zoff,
                          const std::vector<int32_t>& scene) {
    invalidate_graphs(g);
    g->ncells = (int)(cells.size() / 4) - 1;
    EMLAB_CUDA(cudaStreamSynchronize(g->stream));  // buffers may be in use by queued steps
    EMLAB_CUDA(g->d_src.alloc(std::max<size_t>(1, packed.size() / 4)));
    if (!packed.empty())
        EMLAB_CUDA(cudaMemcpyAsync(g->d_src.p, packed.data(), packed.size() * 4, cudaMemcpyHostToDevice, g->stream));
    EMLAB_CUDA(g->d_cells.alloc(cells.size() / 4));
    EMLAB_CUDA(cudaMemcpyAsync(g->d_cells.p, cells.data(), cells.size() * 4, cudaMemcpyHostToDevice, g->stream));
    EMLAB_CUDA(g->d_lists.alloc(std::max<size_t>(1, lists.size())));
    if (!lists.empty())
        EMLAB_CUDA(cudaMemcpyAsync(g->d_lists.p, lists.data(), lists.size() * 4, cudaMemcpyHostToDevice, g->stream));
    g->d_zoff.release();
    if (!zoff.empty()) {
        EMLAB_CUDA(g->d_zoff.alloc(zoff.size()));
        EMLAB_CUDA(cudaMemcpyAsync(g->d_zoff.p, zoff.data(), zoff.size() * 4, cudaMemcpyHostToDevice, g->stream));
    }
    g->d_cell_scene.release();
    if (!scene.empty()) {
        EMLAB_CUDA(g->d_cell_scene.alloc(scene.size()));
        EMLAB_CUDA(cudaMemcpyAsync(g->d_cell_scene.p, scene.data(), scene.size() * 4, cudaMemcpyHostToDevice, g->stream));
    }
    return EMLAB_OK;
}

namespace {

void rotation(double w, double tE, double dt, float4& r) {
    const double tH = tE - 0.5 * dt;
    r = make_float4((float)std::cos(w * tE), (float)std::sin(w * tE), (float)std::cos(w * tH), (float)std::sin(w * tH));
}

float blend_of(float avg, float wl, double dt) {
    const double tau = (double)avg * (double)wl;
    return (float)(1.0 - std::exp(-dt / (0.5 * tau)));
}

int ensure_stage(emlab_grid* g, size_t bytes) {
    if (bytes <= g->stage_bytes) return EMLAB_OK;
    invalidate_graphs(g);
    for (int s = 0; s < 2; ++s) {
        if (g->stage_done[s]) cudaEventSynchronize(g->stage_done[s]);
        if (g->h_stage[s]) cudaFreeHost(g->h_stage[s]);
        g->h_stage[s] = nullptr;
        EMLAB_CUDA(cudaMallocHost(&g->h_stage[s], bytes));
    }
    EMLAB_CUDA(g->d_stage.alloc(bytes));
    g->stage_bytes = bytes;
    return EMLAB_OK;
}

// Folds the recorded event pairs into timed_ms (waits for the last one).
int drain_timing(emlab_grid* g) {
    if (!g->ev_used) return EMLAB_OK;
    EMLAB_CUDA(cudaEventSynchronize(g->ev_stop[g->ev_used - 1]));
    for (size_t i = 0; i < g->ev_used; ++i) {
        float ms = 0.0f;
        EMLAB_CUDA(cudaEventElapsedTime(&ms, g->ev_start[i], g->ev_stop[i]));
        g->timed_ms += ms;
    }
    g->timed_launches += g->ev_used;
    g->ev_used = 0;
    return EMLAB_OK;
}

int timing_pair(emlab_grid* g, cudaEvent_t* start, cudaEvent_t* stop) {
    if (g->ev_used == 4096)
        if (int rc = drain_timing(g)) return rc;
    while (g->ev_start.size() <= g->ev_used) {
        cudaEvent_t a, b;
        EMLAB_CUDA(cudaEventCreate(&a));
        EMLAB_CUDA(cudaEventCreate(&b));
        g->ev_start.push_back(a);
        g->ev_stop.push_back(b);
    }
    *start = g->ev_start[g->ev_used];
    *stop = g->ev_stop[g->ev_used];
    ++g->ev_used;
    return EMLAB_OK;
}

constexpr int kDftCoreBlock = 64;  // samples per CUDA-core fold (that kernel's register block)

// Samples per time block of the engine in use: the tensor-core fold takes up to four 64-sample
// chunks per launch (dft_tc_block), the CUDA-core fold 64.
int dft_block(const emlab_grid* g) {
    const int b = g->dft_engine == EMLAB_DFT_TENSOR ? dft_tc_block(g->dft_nf) : kDftCoreBlock;
    return g->dft_block_cap > 0 ? std::min(b, g->dft_block_cap) : b;
}

// Folds the samples gathered so far into the FP64 sums.
int dft_fold(emlab_grid* g) {
    if (!g->dft_on || g->dft_t == 0) return EMLAB_OK;
    const double dt = (double)g->cfg.courant;
    if (g->dft_engine == EMLAB_DFT_TENSOR &&
        launch_dft_fold_tc(g->d_dft_blk.p, g->dft_t, g->dft_points, g->dft_nf, g->d_dft_bhi.p, g->d_dft_blo.p,
                           g->d_dft_omega.p, g->dft_n0, dt, g->d_dft_x.p, g->d_err.p, g->stream)) {
        ++g_launches;
    } else {
        // CUDA-core folds of 64 samples each, every one with the phase of its own first sample
        const size_t rows = (size_t)6 * g->dft_points;
        for (int off = 0; off < g->dft_t; off += kDftCoreBlock) {
            launch_dft_fold(g->d_dft_blk.p + (size_t)off * rows, std::min(kDftCoreBlock, g->dft_t - off),
                            g->dft_points, g->dft_nf, g->d_dft_w.p, g->d_dft_omega.p, g->dft_n0 + off, dt,
                            g->d_dft_x.p, g->stream);
            ++g_launches;
        }
    }
    g->dft_samples += (uint64_t)g->dft_t;
    g->dft_t = 0;
    return EMLAB_OK;
}

}  // namespace

int emlab::reset_monitors(emlab_grid* g) {
    int rc = emlab_ports_configure(g, nullptr, 0, 16.0f, 4.0f, 0, 0);
    int zero[3] = {0, 0, 0};
    if (!rc) rc = emlab_ntff_configure(g, zero, zero, 0.0f, 4.0f, nullptr);
    if (!rc) rc = emlab_lines_configure(g, nullptr, 0, nullptr, nullptr, 0, 16.0f, 4.0f);
    if (!rc) rc = emlab_ntff_dft_configure(g, zero, zero, nullptr, 0, nullptr);
    return rc;
}

// The launches of one sub-step k of a staged chunk: the Yee pass (advancing the field generation),
// the sources on the new generation, then the per-step monitors. In a graph capture (graph = true)
// the persistent kernel's ticket counter is reset before the launch and its base is 0. Returns the
// number of kernel launches.
namespace {
uint64_t enqueue_step(emlab_grid* g, int k, bool graph, const float* d_sig, const float4* d_prot,
                      const float4* d_nrot, const float4* d_lrot, const float* d_bl, long long rec, cudaEvent_t ev0,
                      cudaEvent_t ev1) {
    uint64_t launched = 0;
    YeeArgs a = yee_args(g);
    if (ev0) cudaEventRecord(ev0, g->stream);
    if (g->cpml_on) {
        launch_cpml(g, a, g->wide, g->stream);  // in place on the current generation
        launched += 2;
    } else if (g->kernel == EMLAB_KERNEL_SPLIT) {
        launch_yee_split(a, g->wide, g->stream);
        launched += 2;
    } else {
        unsigned long long tickets = 0;
        bool tma = false;
        if (g->kernel == EMLAB_KERNEL_FUSED) {
            if (graph) {
                cudaMemsetAsync(g->d_work.p, 0, 8, g->stream);
                a.work_base = 0;
            }
            tma = launch_yee_tma(a, g->tma, g->cur, g->wide, g->d_err.p, g->stream, &tickets);
        }
        if (graph) g->graph_tickets = tickets;
        else g->work_base += tickets;
        if (!tma && g->stack.ragged) g->launch_failed = true;  // no kernel here knows the scenes' cross-sections
        else if (!tma) launch_yee_fused(a, g->wide, g->stream);
        launched += 1;
        g->cur ^= 1;
        a = yee_args(g);  // sources act on the new generation
    }
    if (ev1) cudaEventRecord(ev1, g->stream);
    if (g->ncells > 0) {
        SourceArgs sa{};
        sa.cells = g->d_cells.p, sa.zoff = g->d_zoff.p, sa.lists = g->d_lists.p, sa.src = g->d_src.p;
        sa.scene = g->stack.ragged ? g->d_cell_scene.p : nullptr;
        sa.signals = d_sig, sa.nsrc = g->nsrc, sa.ncells = g->ncells;
        launch_sources(a, sa, k, g->wide, g->stream);
        launched += 1;
    }
    if (!graph) ++g->step;
    const MonitorArgs mon = monitor_args(g);
    if (g->ntff_on) {
        launch_ntff(mon, g->d_box.p, g->points, g->d_ntff.p, d_nrot + k, d_bl + 1, 0, g->stream);
        launched += 1;
    }
    if (g->nports) {
        launch_ports(mon, g->d_ports.p, g->nports, g->d_port_ph.p, g->d_series.p, rec, d_prot + k, d_bl, 0, g->stream);
        launched += 1;
    }
    if (g->nq) {
        launch_lines(mon, g->d_q.p, g->nq, g->d_terms.p, g->d_weights.p, g->d_line_ph.p, g->d_line_now.p, d_lrot + k,
                     d_bl + 2, 0, g->stream);
        launched += 1;
    }
    return launched;
}
}  // namespace

int emlab::require_grid(const emlab_grid* g) {
    if (!g) return fail(EMLAB_ERR_INVALID, "null grid handle");
    if (!g->configured) return fail(EMLAB_ERR_INVALID, "grid is not configured");
    return EMLAB_OK;
}

namespace emlab {
int grid_view(emlab_grid* g, MonitorArgs* m, cudaStream_t* stream, int* device) {
    if (int rc = require_grid(g)) return rc;
    cudaError_t e = cudaSetDevice(g->device);
    if (e != cudaSuccess) return fail(EMLAB_ERR_CUDA, cudaGetErrorString(e));
    *m = monitor_args(g);
    *stream = g->stream;
    *device = g->device;
    return EMLAB_OK;
}
int report_error(int code, const char* msg) { return fail(code, msg); }
void count_launches(int n) { g_launches += (uint64_t)n; }
}  // namespace emlab

extern "C" {

const char* emlab_last_error(void) { return g_last_error.c_str(); }
int emlab_version(void) { return 1; }
uint64_t emlab_launch_count(void) { return g_launches.load(); }

int emlab_grid_create(emlab_grid** out) {
    if (!out) return fail(EMLAB_ERR_INVALID, "null output pointer");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return fail(EMLAB_ERR_NO_DEVICE, "no CUDA device is visible");
    emlab_grid* g = new (std::nothrow) emlab_grid();
    if (!g) return fail(EMLAB_ERR_OOM, "host allocation failed");
    cudaGetDevice(&g->device);
    if (cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&g->stage_done[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&g->stage_done[1], cudaEventDisableTiming) != cudaSuccess ||
        g->d_flag.alloc(1) != cudaSuccess || g->d_err.alloc(1) != cudaSuccess ||
        cudaMemsetAsync(g->d_err.p, 0, 4, g->stream) != cudaSuccess || g->d_work.alloc(1) != cudaSuccess ||
        cudaMemsetAsync(g->d_work.p, 0, 8, g->stream) != cudaSuccess) {
        delete g;
        return fail(EMLAB_ERR_CUDA, "stream or event creation failed");
    }
    *out = g;
    return EMLAB_OK;
}

int emlab_grid_destroy(emlab_grid* g) {
    if (!g) return EMLAB_OK;
    cudaSetDevice(g->device);
    if (g->stream) cudaStreamSynchronize(g->stream);
    for (int s = 0; s < 2; ++s) {
        if (g->h_stage[s]) cudaFreeHost(g->h_stage[s]);
        if (g->stage_done[s]) cudaEventDestroy(g->stage_done[s]);
        if (g->h_series[s]) cudaFreeHost(g->h_series[s]);
        if (g->series_done[s]) cudaEventDestroy(g->series_done[s]);
    }
    for (size_t i = 0; i < g->ev_start.size(); ++i) cudaEventDestroy(g->ev_start[i]), cudaEventDestroy(g->ev_stop[i]);
    if (g->tma) tma_maps_destroy(g->tma);
    invalidate_graphs(g);
    for (auto& a : g->analyzer) {
        if (a.h_probe) cudaFreeHost(a.h_probe);
        if (a.h_part) cudaFreeHost(a.h_part);
        if (a.done) cudaEventDestroy(a.done);
    }
    cudaStream_t s = g->stream;
    delete g;
    if (s) cudaStreamDestroy(s);
    return EMLAB_OK;
}

int emlab_grid_configure(emlab_grid* g, const emlab_grid_config* req) {
    if (!g || !req) return fail(EMLAB_ERR_INVALID, "null argument");
    EMLAB_CUDA(cudaSetDevice(g->device));
    emlab_grid_config c = *req;
    clamp_config(c);
    const int pitch = row_pitch(c.nx);
    const long long plane = (long long)pitch * c.ny;
    const long long padded = plane * c.nz;
    if (!g->configured || c.nx != g->cfg.nx || c.ny != g->cfg.ny || c.nz != g->cfg.nz || !g->fields.p) {
        g->fields.release();
        g->cls.release();
        cudaError_t e = g->fields.alloc((size_t)padded * 12);
        if (e != cudaSuccess) {
            g->configured = false;
            return fail(EMLAB_ERR_OOM, "SimulationGrid: field allocation failed (grid too large for device memory)");
        }
    }
    g->cfg = c;
    g->pitch = pitch, g->plane = plane, g->padded = padded;
    g->stack = StackLayout();  // a single scene
    if (int rc = upload_pml(g)) return rc;
    if (g->cpml_on) {  // the convolutional PML follows the new size and absorber thickness
        if (int rc = cpml_prepare(g)) return rc;
    }
    // vacuum materials: class 0 everywhere (SimulationGrid.cpp:185-192)
    const long long n = g->cells();
    try {
        g->cell_sigma.assign((size_t)n, 0.0f);
        g->cell_eps.assign((size_t)n, 1.0f);
    } catch (const std::bad_alloc&) {
        return fail(EMLAB_ERR_OOM, "host allocation failed");
    }
    ClassTable t;
    t.classes = 1, t.wire_start = 1;
    t.tabM = {0, 0, 0, 1, 1, 1, 0, 0};
    t.tabW = {1, 1, 1, 1, 1, 1, 0, 0};
    t.tabE.assign(8, 0.0f);
    class_coefficients(t, c.courant);
    g->wide = false;
    EMLAB_CUDA(g->cls.alloc((size_t)padded * 2));
    EMLAB_CUDA(cudaMemsetAsync(g->cls.p, 0, (size_t)padded * 2, g->stream));
    EMLAB_CUDA(g->tabE.alloc(2));
    EMLAB_CUDA(g->tabM.alloc(2));
    EMLAB_CUDA(g->tabW.alloc(2));
    EMLAB_CUDA(cudaMemcpyAsync(g->tabE.p, t.tabE.data(), 32, cudaMemcpyHostToDevice, g->stream));
    EMLAB_CUDA(cudaMemcpyAsync(g->tabM.p, t.tabM.data(), 32, cudaMemcpyHostToDevice, g->stream));
    EMLAB_CUDA(cudaMemcpyAsync(g->tabW.p, t.tabW.data(), 32, cudaMemcpyHostToDevice, g->stream));
    g->classes = 1, g->wire_start = 1;
    int rc = clear_fields(g);
    if (rc) return rc;
    refresh_tma(g);
    g->step = 0;
    g->configured = true;
    // the source lists index cells of the old size: rebuild them for the new one
    if (!g->desc.empty()) {
        std::vector<emlab_source> d = g->desc;
        rc = emlab_grid_set_sources(g, d.data(), d.size());
        if (rc) return rc;
    }
    if (int rc2 = reset_monitors(g)) return rc2;
    EMLAB_CUDA(cudaStreamSynchronize(g->stream));
    return EMLAB_OK;
}

int emlab_grid_get_config(const emlab_grid* g, emlab_grid_config* out) {
    if (int rc = require_grid(g)) return rc;
    if (!out) return fail(EMLAB_ERR_INVALID, "null output");
    *out = g->cfg;
    return EMLAB_OK;
}

int emlab_grid_upload_materials(emlab_grid* g, const float* sigma, const float* eps_r, int nx, int ny, int nz,
                                const emlab_edge_override* edges, size_t n_edges, const emlab_wire_term* wires,
                                size_t n_wires) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(g->stack.scenes() == 0, "a stack of scenes takes materials per scene (emlab_stack_upload_materials)");
    if (nx != g->cfg.nx || ny != g->cfg.ny || nz != g->cfg.nz)
        return fail(EMLAB_ERR_INVALID, "SimulationGrid: material volume size does not match the grid");
    EMLAB_REQUIRE(sigma && eps_r, "null material array");
    EMLAB_REQUIRE((edges || n_edges == 0) && (wires || n_wires == 0), "null override array");
    EMLAB_CUDA(cudaSetDevice(g->device));
    ClassTable t;
    std::string err;
    if (!build_classes(sigma, eps_r, nx, ny, nz, edges, n_edges, wires, n_wires, g->cfg.courant, t, err))
        return fail(EMLAB_ERR_OOM, err);
    if (int rc = upload_class_table(g, t)) return rc;
    refresh_tma(g);
    const long long n = g->cells();
    std::memcpy(g->cell_sigma.data(), sigma, (size_t)n * 4);
    std::memcpy(g->cell_eps.data(), eps_r, (size_t)n * 4);
    if (int rc = clear_fields(g)) return rc;
    g->step = 0;
    EMLAB_CUDA(cudaStreamSynchronize(g->stream));
    return EMLAB_OK;
}

int emlab_grid_set_sources(emlab_grid* g, const emlab_source* sources, size_t n) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(sources || n == 0, "null source array");
    EMLAB_REQUIRE(g->stack.scenes() == 0, "a stack of scenes takes sources per scene (emlab_stack_set_sources)");
    EMLAB_CUDA(cudaSetDevice(g->device));
    std::vector<emlab_source> desc;
    std::vector<float> packed;
    g->nsrc = pack_sources(sources, n, desc, packed);
    g->desc = desc;
    g->packed = packed;
    std::vector<int32_t> cells, lists;
    const int dims[3] = {g->cfg.nx, g->cfg.ny, g->cfg.nz};
    source_lists(packed, g->nsrc, dims, cells, lists);
    return upload_sources(g, packed, cells, lists, {});
}

int emlab_grid_reset_fields(emlab_grid* g) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_CUDA(cudaSetDevice(g->device));
    if (int rc = clear_fields(g)) return rc;
    g->step = 0;
    return EMLAB_OK;
}

int emlab_grid_step(emlab_grid* g, int count) {
    if (int rc = require_grid(g)) return rc;
    if (count <= 0) return EMLAB_OK;
    EMLAB_CUDA(cudaSetDevice(g->device));
    if (int rc = stack_commit(g)) return rc;
    if (g->stack.ragged && !(tma_maps_ready(g->tma, 0) && tma_maps_ready(g->tma, 1)))
        return fail(EMLAB_ERR_CUDA, "a stack of scenes with different cross-sections needs the TMA pair kernel, "
                                    "and its tensor maps could not be encoded");
    const double dt = (double)g->cfg.courant;
    const int nsrc = g->nsrc;
    for (int base = 0; base < count; base += kChunk) {
        const int m = std::min(kChunk, count - base);
        // stage layout: signals m*nsrc floats | port rot m float4 | ntff rot | line rot | 3 blends
        const size_t sig_bytes = ((size_t)m * nsrc * 4 + 15) / 16 * 16;
        const size_t rot_bytes = (size_t)m * 16;
        const size_t bytes = sig_bytes + 3 * rot_bytes + 16 * 3;
        if (int rc = ensure_stage(g, bytes)) return rc;
        const int slot = g->stage_slot;
        g->stage_slot ^= 1;
        EMLAB_CUDA(cudaEventSynchronize(g->stage_done[slot]));  // the slot's previous copy has finished
        uint8_t* h = g->h_stage[slot];
        float* sig = reinterpret_cast<float*>(h);
        float4* prot = reinterpret_cast<float4*>(h + sig_bytes);
        float4* nrot = prot + m;
        float4* lrot = nrot + m;
        float* blends = reinterpret_cast<float*>(lrot + m);
        for (int k = 0; k < m; ++k) {
            // E^{n+1} uses J at t = (n + 1/2) dt (SimulationGrid.cpp:371-387)
            const double t = ((double)(g->step + (uint64_t)k) + 0.5) * dt;
            for (int s = 0; s < nsrc; ++s) sig[(size_t)k * nsrc + s] = (float)source_signal(g->desc[s], t);
            // monitors see the time of the completed step: t_E = n dt, t_H = t_E - dt/2
            const double tE = (double)(g->step + (uint64_t)k + 1) * dt;
            if (g->nports) rotation(6.28318530717958647692 / g->port_wl, tE, dt, prot[k]);
            if (g->ntff_on) rotation(6.28318530717958647692 / g->ntff_wl, tE, dt, nrot[k]);
            if (g->nq) rotation(6.28318530717958647692 / g->line_wl, tE, dt, lrot[k]);
        }
        blends[0] = blend_of(g->port_avg, g->port_wl, dt);
        blends[1] = blend_of(g->ntff_avg, g->ntff_wl, dt);
        blends[2] = blend_of(g->line_avg, g->line_wl, dt);
        uint8_t* d = g->d_stage.p;
        const float* d_sig = reinterpret_cast<const float*>(d);
        const float4* d_prot = reinterpret_cast<const float4*>(d + sig_bytes);
        const float4* d_nrot = d_prot + m;
        const float4* d_lrot = d_nrot + m;
        const float* d_bl = reinterpret_cast<const float*>(d_lrot + m);
        // A chunk of exactly graph_chunk steps replays a captured graph of the same launches (the
        // staging copy included); the per-step host work is then one graph launch per chunk. Port
        // recording restarts at row 0 every chunk, so the caller takes the series after each chunk.
        const bool graph = g->graph_chunk > 0 && m == g->graph_chunk && (m % 2) == 0 && !g->timing && !g->dft_on &&
                           (!g->nports || !g->recording || (g->recorded == 0 && g->series_cap >= (size_t)m));
        if (graph && g->graph_warm) {
            cudaGraphExec_t& ex = g->graph_exec[slot][g->cur];
            if (!ex) {
                const int cur0 = g->cur;
                const unsigned long long base0 = g->work_base;
                uint64_t launched = 0;
                EMLAB_CUDA(cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal));
                cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, g->stream);
                for (int k = 0; k < m; ++k)
                    launched += enqueue_step(g, k, true, d_sig, d_prot, d_nrot, d_lrot, d_bl,
                                             g->nports && g->recording ? k : -1, nullptr, nullptr);
                cudaGraph_t graph_def = nullptr;
                const cudaError_t ce = cudaStreamEndCapture(g->stream, &graph_def);
                g->cur = cur0, g->work_base = base0;
                cudaError_t ie = ce;
                if (ce == cudaSuccess) ie = cudaGraphInstantiate(&ex, graph_def, 0);
                if (graph_def) cudaGraphDestroy(graph_def);
                cudaGetLastError();
                if (g->launch_failed) {  // the captured chunk lacks its solver launches: never replay it
                    g->launch_failed = false;
                    if (ex) cudaGraphExecDestroy(ex);
                    ex = nullptr;
                    return fail(EMLAB_ERR_CUDA, "the pair kernel could not be launched for a stack of scenes with "
                                                "different cross-sections");
                }
                if (ie != cudaSuccess) {
                    ex = nullptr;
                    return fail(EMLAB_ERR_CUDA, std::string("step graph capture: ") + cudaGetErrorString(ie));
                }
                g->graph_launches = launched;
            }
            EMLAB_CUDA(cudaGraphLaunch(ex, g->stream));
            EMLAB_CUDA(cudaEventRecord(g->stage_done[slot], g->stream));
            g->step += (uint64_t)m;
            if (g->nports && g->recording) g->recorded = (size_t)m;
            if (g->kernel != EMLAB_KERNEL_SPLIT && g->graph_tickets) g->work_base = g->graph_tickets;
            g_launches += g->graph_launches;
            if (int rc = check_launch()) return rc;
            continue;
        }
        if (graph) g->graph_warm = true;  // one ordinary chunk first: the launchers' one-time set-up
        EMLAB_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, g->stream));
        EMLAB_CUDA(cudaEventRecord(g->stage_done[slot], g->stream));
        // monitor kernels get this sub-step's rotation and their blend by pointer (index 0)
        for (int k = 0; k < m; ++k) {
            long long rec = -1;
            if (g->nports && g->recording && g->recorded < g->series_cap) rec = (long long)g->recorded++;
            cudaEvent_t ev0 = nullptr, ev1 = nullptr;
            if (g->timing)
                if (int rc = timing_pair(g, &ev0, &ev1)) return rc;
            g_launches += enqueue_step(g, k, false, d_sig, d_prot, d_nrot, d_lrot, d_bl, rec, ev0, ev1);
            if (g->launch_failed) {
                g->launch_failed = false;
                return fail(EMLAB_ERR_CUDA, "the pair kernel could not be launched for a stack of scenes with "
                                            "different cross-sections");
            }
            if (g->dft_on) {
                if (g->dft_t == 0) g->dft_n0 = (long long)g->step;  // time index of the block's first sample
                launch_dft_sample(monitor_args(g), g->d_dft_box.p, g->dft_nbox, g->dft_box_max, g->dft_points,
                                  g->d_dft_blk.p, g->dft_t, g->stream);
                g_launches += 1;
                if (++g->dft_t == dft_block(g)) dft_fold(g);
            }
            if (int rc = check_launch()) return rc;
        }
    }
    return EMLAB_OK;
}

int emlab_grid_set_graph(emlab_grid* g, int chunk) {
    if (!g) return fail(EMLAB_ERR_INVALID, "null grid handle");
    EMLAB_REQUIRE(chunk == 0 || (chunk >= 2 && chunk <= kChunk && chunk % 2 == 0),
                  "graph chunk must be 0 (off) or an even number of steps up to 1024");
    invalidate_graphs(g);
    g->graph_chunk = chunk;
    g->graph_warm = false;
    return EMLAB_OK;
}

int emlab_grid_synchronize(emlab_grid* g, int timeout_ms) {
    if (!g) return fail(EMLAB_ERR_INVALID, "null grid handle");
    const auto limit = std::chrono::milliseconds(timeout_ms > 0 ? timeout_ms : 60000);
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t e = cudaStreamQuery(g->stream);
        if (e == cudaSuccess) {
            unsigned err = 0;
            EMLAB_CUDA(cudaMemcpy(&err, g->d_err.p, 4, cudaMemcpyDeviceToHost));
            if (err) {
                EMLAB_CUDA(cudaMemsetAsync(g->d_err.p, 0, 4, g->stream));
                return fail(EMLAB_ERR_TIMEOUT, "a solver kernel gave up a bounded wait on the device");
            }
            return EMLAB_OK;
        }
        if (e != cudaErrorNotReady) return fail(EMLAB_ERR_CUDA, std::string("stream: ") + cudaGetErrorString(e));
        if (std::chrono::steady_clock::now() - t0 > limit) return fail(EMLAB_ERR_TIMEOUT, "grid stream wait timed out");
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

int emlab_grid_get_state(const emlab_grid* g, emlab_grid_state* out) {
    if (int rc = require_grid(g)) return rc;
    if (!out) return fail(EMLAB_ERR_INVALID, "null output");
    out->dt = g->cfg.courant;
    out->step_count = g->step;
    out->time = (double)g->step * (double)g->cfg.courant;
    out->nx = g->cfg.nx, out->ny = g->cfg.ny, out->nz = g->cfg.nz;
    out->device_bytes = g->fields.n * 4 + g->cls.n + (g->tabE.n + g->tabM.n + g->tabW.n) * 16 + g->pml.n * 4 +
                        g->d_ntff.n * 4 + g->d_series.n * 4;
    out->source_cells = g->ncells;
    out->kernel = g->kernel;
    return EMLAB_OK;
}

static int read_comp(emlab_grid* g, int c, float* host, int stride, int offset) {
    const int nx = g->cfg.nx, ny = g->cfg.ny, nz = g->cfg.nz;
    std::vector<float> tmp((size_t)g->padded);
    EMLAB_CUDA(cudaMemcpyAsync(tmp.data(), g->comp(g->cur, c), (size_t)g->padded * 4, cudaMemcpyDeviceToHost, g->stream));
    EMLAB_CUDA(cudaStreamSynchronize(g->stream));
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y) {
            const float* src = tmp.data() + (size_t)z * g->plane + (size_t)y * g->pitch;
            const size_t row = ((size_t)z * ny + y) * nx;
            for (int x = 0; x < nx; ++x) host[(row + x) * stride + offset] = src[x];
        }
    return EMLAB_OK;
}

int emlab_grid_read_fields(emlab_grid* g, float* e_rgba, float* b_rgba) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_CUDA(cudaSetDevice(g->device));
    const long long n = g->cells();
    if (int rc = ensure_cell_materials(g)) return rc;
    for (int c = 0; c < 6; ++c) {
        float* dst = c < 3 ? e_rgba : b_rgba;
        if (!dst) continue;
        if (int rc = read_comp(g, c, dst, 4, c % 3)) return rc;
    }
    for (long long i = 0; i < n; ++i) {
        if (e_rgba) e_rgba[i * 4 + 3] = g->cell_sigma[(size_t)i];
        if (b_rgba) b_rgba[i * 4 + 3] = g->cell_eps[(size_t)i];
    }
    return EMLAB_OK;
}

int emlab_grid_read_components(emlab_grid* g, float* ex, float* ey, float* ez, float* bx, float* by, float* bz) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_CUDA(cudaSetDevice(g->device));
    float* out[6] = {ex, ey, ez, bx, by, bz};
    for (int c = 0; c < 6; ++c)
        if (out[c])
            if (int rc = read_comp(g, c, out[c], 1, 0)) return rc;
    return EMLAB_OK;
}

int emlab_grid_write_components(emlab_grid* g, const float* ex, const float* ey, const float* ez, const float* bx,
                                const float* by, const float* bz) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_CUDA(cudaSetDevice(g->device));
    const float* in[6] = {ex, ey, ez, bx, by, bz};
    const int nx = g->cfg.nx, ny = g->cfg.ny, nz = g->cfg.nz;
    std::vector<float> tmp((size_t)g->padded, 0.0f);
    for (int c = 0; c < 6; ++c) {
        if (!in[c]) continue;
        for (int z = 0; z < nz; ++z)
            for (int y = 0; y < ny; ++y)
                std::memcpy(tmp.data() + (size_t)z * g->plane + (size_t)y * g->pitch, in[c] + ((size_t)z * ny + y) * nx,
                            (size_t)nx * 4);
        EMLAB_CUDA(cudaMemcpyAsync(g->comp(g->cur, c), tmp.data(), (size_t)g->padded * 4, cudaMemcpyHostToDevice,
                                   g->stream));
        EMLAB_CUDA(cudaStreamSynchronize(g->stream));
    }
    return EMLAB_OK;
}

int emlab_grid_set_kernel(emlab_grid* g, int kernel) {
    if (!g) return fail(EMLAB_ERR_INVALID, "null grid handle");
    EMLAB_REQUIRE(kernel == EMLAB_KERNEL_FUSED || kernel == EMLAB_KERNEL_SPLIT || kernel == EMLAB_KERNEL_FUSED_LDG,
                  "unknown kernel");
    EMLAB_REQUIRE(!g->stack.ragged || kernel == EMLAB_KERNEL_FUSED,
                  "a stack of scenes with different cross-sections steps with the fused kernel only");
    g->kernel = kernel;
    if (g->configured) refresh_tma(g);
    return EMLAB_OK;
}

int emlab_grid_set_tiling(emlab_grid* g, int tile_rows) {
    if (!g) return fail(EMLAB_ERR_INVALID, "null grid handle");
    EMLAB_REQUIRE(tile_rows == 0 || tile_rows == 8 || tile_rows == 16 || tile_rows == 32 || tile_rows == 64 ||
                      tile_rows == 128,
                  "tiling must be 0 (automatic), 8 or 16 (32-cell rows), 32, 64 or 128 (64 x 4, 64 x 8 or 64 x 16 "
                  "tiles of cell pairs)");
    EMLAB_REQUIRE(!g->stack.ragged || tile_rows == 0 || tile_rows == 32 || tile_rows == 64 || tile_rows == 128,
                  "a stack of scenes with different cross-sections steps with tiles of cell pairs only (0, 32, 64, 128)");
    g->tile_rows = tile_rows;
    if (g->configured) refresh_tma(g);  // the TMA boxes depend on the tile height
    return EMLAB_OK;
}

int emlab_grid_field_ptr(emlab_grid* g, float** ptrs, int* pitch, long long* plane) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(ptrs && pitch && plane, "null argument");
    for (int c = 0; c < 6; ++c) ptrs[c] = g->comp(g->cur, c);
    *pitch = g->pitch;
    *plane = g->plane;
    return EMLAB_OK;
}

int emlab_grid_stream(emlab_grid* g, void** stream) {
    if (!g || !stream) return fail(EMLAB_ERR_INVALID, "null argument");
    *stream = (void*)g->stream;
    return EMLAB_OK;
}

int emlab_grid_set_timing(emlab_grid* g, int enabled) {
    if (!g) return fail(EMLAB_ERR_INVALID, "null grid handle");
    if (!enabled)
        if (int rc = drain_timing(g)) return rc;
    g->timing = enabled != 0;
    return EMLAB_OK;
}

int emlab_grid_kernel_time(emlab_grid* g, double* ms, uint64_t* launches, int reset) {
    if (!g) return fail(EMLAB_ERR_INVALID, "null grid handle");
    if (int rc = drain_timing(g)) return rc;
    if (ms) *ms = g->timed_ms;
    if (launches) *launches = g->timed_launches;
    if (reset) g->timed_ms = 0.0, g->timed_launches = 0;
    return EMLAB_OK;
}

int emlab_grid_check_finite(emlab_grid* g) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_CUDA(cudaSetDevice(g->device));
    EMLAB_CUDA(cudaMemsetAsync(g->d_flag.p, 0, 4, g->stream));
    launch_check_finite(monitor_args(g), g->d_flag.p, g->stream);
    ++g_launches;
    if (int rc = check_launch()) return rc;
    unsigned flag = 0;
    EMLAB_CUDA(cudaMemcpyAsync(&flag, g->d_flag.p, 4, cudaMemcpyDeviceToHost, g->stream));
    if (int rc = emlab_grid_synchronize(g, 0)) return rc;
    if (flag) return fail(EMLAB_ERR_NONFINITE, "non-finite field values detected");
    return EMLAB_OK;
}

// ---- ports ---------------------------------------------------------------------------------
int emlab_ports_configure(emlab_grid* g, const emlab_port* ports, size_t n, float wavelength, float averaging_periods,
                          int sweep, size_t record_steps) {
    if (int rc = require_grid(g)) return rc;
    // a pending take's rows are laid out for the current ports
    EMLAB_REQUIRE(!g->series_busy[0] && !g->series_busy[1], "collect the pending series takes before configuring ports");
    invalidate_graphs(g);
    EMLAB_REQUIRE(ports || n == 0, "null port array");
    EMLAB_CUDA(cudaSetDevice(g->device));
    EMLAB_CUDA(cudaStreamSynchronize(g->stream));
    n = std::min<size_t>(n, 256);
    g->nports = (int)n;
    g->port_avg = std::max(averaging_periods, 0.5f);
    g->port_wl = std::max(wavelength, 2.0f);
    g->recorded = 0, g->series_cap = 0, g->recording = false;
    g->d_ports.release(), g->d_port_ph.release(), g->d_series.release();
    if (!n) return EMLAB_OK;
    std::vector<int4> pk;
    for (size_t i = 0; i < n; ++i) {
        pk.push_back(make_int4(ports[i].x, ports[i].y, ports[i].z, ports[i].axis));
        pk.push_back(make_int4(ports[i].edges, ports[i].sign >= 0 ? 1 : -1, 0, 0));
    }
    EMLAB_CUDA(g->d_ports.alloc(pk.size()));
    EMLAB_CUDA(cudaMemcpyAsync(g->d_ports.p, pk.data(), pk.size() * 16, cudaMemcpyHostToDevice, g->stream));
    EMLAB_CUDA(g->d_port_ph.alloc(n * 8));
    EMLAB_CUDA(cudaMemsetAsync(g->d_port_ph.p, 0, n * 32, g->stream));
    if (sweep || record_steps > 0) {
        size_t cap = ((size_t)1 << 23) / (2 * n);  // Ports.cpp:16, 209-210
        if (!sweep) cap = std::min(cap, record_steps);
        EMLAB_CUDA(g->d_series.alloc(cap * n * 2));
        g->series_cap = cap;
        g->recording = true;
    }
    return EMLAB_OK;
}

int emlab_ports_read_phasors(emlab_grid* g, float* out) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(out || g->nports == 0, "null output");
    if (!g->nports) return EMLAB_OK;
    EMLAB_CUDA(cudaMemcpyAsync(out, g->d_port_ph.p, (size_t)g->nports * 32, cudaMemcpyDeviceToHost, g->stream));
    return emlab_grid_synchronize(g, 0);
}

int emlab_ports_read_series(emlab_grid* g, float* out, size_t max_steps, size_t* steps) {
    if (int rc = require_grid(g)) return rc;
    if (steps) *steps = g->recorded;
    if (!out || !g->recorded) return EMLAB_OK;
    const size_t s = std::min(max_steps, g->recorded);
    EMLAB_CUDA(cudaMemcpyAsync(out, g->d_series.p, s * g->nports * 8, cudaMemcpyDeviceToHost, g->stream));
    return emlab_grid_synchronize(g, 0);
}

int emlab_ports_take_series(emlab_grid* g, float* out, size_t max_steps, size_t* steps) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(out || max_steps == 0, "null output");
    const size_t s = std::min(max_steps, g->recorded);
    if (steps) *steps = s;
    if (s) EMLAB_CUDA(cudaMemcpyAsync(out, g->d_series.p, s * g->nports * 8, cudaMemcpyDeviceToHost, g->stream));
    if (int rc = emlab_grid_synchronize(g, 0)) return rc;
    g->recorded = 0;  // the next step records from the start of the buffer again
    return EMLAB_OK;
}

int emlab_ports_take_series_async(emlab_grid* g, int* slot, size_t* steps) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(slot && steps, "null output");
    EMLAB_CUDA(cudaSetDevice(g->device));
    const int k = g->series_next;
    EMLAB_REQUIRE(!g->series_busy[k], "both series slots are waiting to be collected");
    const size_t s = g->recorded, bytes = s * (size_t)g->nports * 8;
    if (!g->series_done[k]) EMLAB_CUDA(cudaEventCreateWithFlags(&g->series_done[k], cudaEventDisableTiming));
    if (bytes > g->h_series_cap[k]) {
        if (g->h_series[k]) cudaFreeHost(g->h_series[k]);
        g->h_series[k] = nullptr, g->h_series_cap[k] = 0;
        EMLAB_CUDA(cudaMallocHost(&g->h_series[k], bytes));
        g->h_series_cap[k] = bytes;
    }
    if (bytes) EMLAB_CUDA(cudaMemcpyAsync(g->h_series[k], g->d_series.p, bytes, cudaMemcpyDeviceToHost, g->stream));
    EMLAB_CUDA(cudaEventRecord(g->series_done[k], g->stream));
    g->h_series_rows[k] = s;
    g->series_busy[k] = true;
    g->series_next ^= 1;
    g->recorded = 0;  // the next step records from the start of the buffer again (after this copy, in stream order)
    *slot = k, *steps = s;
    return EMLAB_OK;
}

int emlab_ports_collect_series(emlab_grid* g, int slot, float* out, size_t max_steps, int timeout_ms) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(slot == 0 || slot == 1, "no such series slot");
    EMLAB_REQUIRE(g->series_busy[slot], "the series slot holds no pending take");
    EMLAB_REQUIRE(out || max_steps == 0, "null output");
    EMLAB_CUDA(cudaSetDevice(g->device));
    const auto limit = std::chrono::milliseconds(timeout_ms > 0 ? timeout_ms : 60000);
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        const cudaError_t e = cudaEventQuery(g->series_done[slot]);
        if (e == cudaSuccess) break;
        if (e != cudaErrorNotReady) return fail(EMLAB_ERR_CUDA, std::string("series copy: ") + cudaGetErrorString(e));
        if (std::chrono::steady_clock::now() - t0 > limit)
            return fail(EMLAB_ERR_TIMEOUT, "series copy did not complete within the timeout");
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    unsigned err = 0;
    EMLAB_CUDA(cudaMemcpy(&err, g->d_err.p, 4, cudaMemcpyDeviceToHost));
    if (err) return fail(EMLAB_ERR_TIMEOUT, "a solver kernel's bounded wait ran out");
    const size_t s = std::min(max_steps, g->h_series_rows[slot]);
    if (s) std::memcpy(out, g->h_series[slot], s * (size_t)g->nports * 8);
    g->series_busy[slot] = false;
    return EMLAB_OK;
}

int emlab_ports_sweep_sums(emlab_grid* g, double lambda_min, double lambda_max, int points, double* out,
                           double* residual) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(g->nports > 0 && g->recorded > 0, "no recorded port series");
    EMLAB_REQUIRE(out, "null output");
    points = std::max(points, 2);
    const double nu_lo = 1.0 / std::max(lambda_max, lambda_min), nu_hi = 1.0 / std::min(lambda_max, lambda_min);
    DevBuf<double> d_out;
    EMLAB_CUDA(d_out.alloc((size_t)g->nports * points * 4));
    launch_sweep_sums(g->d_series.p, (long long)g->recorded, g->nports, nu_lo, nu_hi, points, (double)g->cfg.courant,
                      d_out.p, g->stream);
    ++g_launches;
    if (int rc = check_launch()) return rc;
    EMLAB_CUDA(cudaMemcpyAsync(out, d_out.p, d_out.n * 8, cudaMemcpyDeviceToHost, g->stream));
    if (int rc = emlab_grid_synchronize(g, 0)) return rc;
    if (residual) {
        // ring-down: late-time |V| of port 0 relative to its peak (Ports.cpp:206-213), on the device
        std::vector<double> r((size_t)g->nports);
        if (int rc = emlab_ports_residuals(g, r.data())) return rc;
        *residual = r[0];
    }
    return EMLAB_OK;
}

int emlab_ports_residuals(emlab_grid* g, double* out) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(out, "null output");
    EMLAB_REQUIRE(g->nports > 0, "no port monitor");
    if (g->recorded == 0) {
        for (int p = 0; p < g->nports; ++p) out[p] = 1.0;
        return EMLAB_OK;
    }
    DevBuf<double> d_out;
    EMLAB_CUDA(d_out.alloc((size_t)g->nports));
    launch_port_residuals(g->d_series.p, (long long)g->recorded, g->nports, d_out.p, g->stream);
    ++g_launches;
    if (int rc = check_launch()) return rc;
    EMLAB_CUDA(cudaMemcpyAsync(out, d_out.p, d_out.n * 8, cudaMemcpyDeviceToHost, g->stream));
    return emlab_grid_synchronize(g, 0);
}

// ---- far field -----------------------------------------------------------------------------
int emlab_ntff_configure(emlab_grid* g, const int box_min[3], const int box_max[3], float wavelength,
                         float averaging_periods, int box_out[6]) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_CUDA(cudaSetDevice(g->device));
    EMLAB_CUDA(cudaStreamSynchronize(g->stream));
    invalidate_graphs(g);
    g->ntff_on = false;
    g->d_ntff.release();
    if (!(wavelength > 0.0f)) return EMLAB_OK;
    EMLAB_REQUIRE(box_min && box_max, "null box");
    const int n[3] = {g->cfg.nx, g->cfg.ny, g->cfg.nz};
    const int L = g->cfg.pml_thickness;
    int bmin[3], bmax[3];
    for (int a = 0; a < 3; ++a) {
        // FarField.cpp:263-268: keep every node and its -1 neighbours out of the absorber
        const int lo = L + 1, hi = n[a] - L - 2;
        bmin[a] = std::clamp(std::min(box_min[a], box_max[a]), lo, hi);
        bmax[a] = std::clamp(std::max(box_min[a], box_max[a]), lo, hi);
        if (bmax[a] - bmin[a] < 4)
            return fail(EMLAB_ERR_INVALID,
                        "far_field box is degenerate after clamping to the region inside the absorbing layer");
    }
    for (int a = 0; a < 3; ++a) g->box[a] = bmin[a], g->box[3 + a] = bmax[a];
    if (box_out)
        for (int a = 0; a < 3; ++a) box_out[a] = bmin[a], box_out[3 + a] = bmax[a];
    g->box[6] = 0;
    for (int f = 0; f < 6; ++f) {
        const int a = f >> 1, u = a == 0 ? 1 : 0, v = a == 2 ? 1 : 2;
        g->box[7 + f] = g->box[6 + f] + (bmax[u] - bmin[u] + 1) * (bmax[v] - bmin[v] + 1);
    }
    g->points = g->box[12];
    g->ntff_wl = std::max(wavelength, 2.0f);
    g->ntff_avg = std::max(averaging_periods, 0.5f);
    EMLAB_CUDA(g->d_box.alloc(13));
    EMLAB_CUDA(cudaMemcpyAsync(g->d_box.p, g->box, 13 * 4, cudaMemcpyHostToDevice, g->stream));
    EMLAB_CUDA(g->d_ntff.alloc((size_t)g->points * 32));
    EMLAB_CUDA(cudaMemsetAsync(g->d_ntff.p, 0, (size_t)g->points * 128, g->stream));
    g->ntff_on = true;
    return EMLAB_OK;
}

int emlab_ntff_point_count(emlab_grid* g, int* points) {
    if (int rc = require_grid(g)) return rc;
    if (!points) return fail(EMLAB_ERR_INVALID, "null output");
    *points = g->ntff_on ? g->points : 0;
    return EMLAB_OK;
}

int emlab_ntff_read_phasors(emlab_grid* g, float* out) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(g->ntff_on, "far-field monitor is not configured");
    EMLAB_REQUIRE(out, "null output");
    EMLAB_CUDA(cudaMemcpyAsync(out, g->d_ntff.p, (size_t)g->points * 128, cudaMemcpyDeviceToHost, g->stream));
    return emlab_grid_synchronize(g, 0);
}

int emlab_ntff_evaluate(emlab_grid* g, const float* directions, int n_dirs, float* out) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(g->ntff_on, "far-field monitor is not configured");
    EMLAB_REQUIRE(directions && out && n_dirs > 0, "bad direction arguments");
    EMLAB_CUDA(cudaSetDevice(g->device));
    const int slices = std::clamp((g->points + 4095) / 4096, 1, 64);  // FarField.cpp:297
    const int chunk = 4096;
    DevBuf<float4> d_dirs, d_part;
    DevBuf<float> d_out;
    EMLAB_CUDA(d_dirs.alloc((size_t)n_dirs));
    EMLAB_CUDA(cudaMemcpyAsync(d_dirs.p, directions, (size_t)n_dirs * 16, cudaMemcpyHostToDevice, g->stream));
    EMLAB_CUDA(d_part.alloc((size_t)chunk * slices * 4));
    EMLAB_CUDA(d_out.alloc((size_t)n_dirs * 2));
    const float k = (float)(6.28318530717958647692 / (double)g->ntff_wl);
    for (int first = 0; first < n_dirs; first += chunk) {
        const int count = std::min(chunk, n_dirs - first);
        launch_ntff_pattern(g->d_box.p, g->points, g->d_ntff.p, d_dirs.p, first, count, slices, k, d_part.p, g->stream);
        launch_ntff_reduce(d_dirs.p, d_part.p, first, count, slices, d_out.p, g->stream);
        g_launches += 2;
        if (int rc = check_launch()) return rc;
    }
    std::vector<float> tmp((size_t)n_dirs * 2);
    EMLAB_CUDA(cudaMemcpyAsync(tmp.data(), d_out.p, tmp.size() * 4, cudaMemcpyDeviceToHost, g->stream));
    if (int rc = emlab_grid_synchronize(g, 0)) return rc;
    // only the dispatch starting at direction 0 carries the power (ntff_pattern.comp:52)
    for (int d = 0; d < n_dirs; ++d) out[2 * d] = tmp[2 * (size_t)d], out[2 * d + 1] = d == 0 ? tmp[1] : 0.0f;
    return EMLAB_OK;
}

// ---- multi-frequency far-field DFT ----------------------------------------------------------------
namespace {
// Attaches the far-field DFT to `nbox` boxes (6 ints each, min xyz and max xyz, already checked):
// box records with their face offsets and their places in the concatenated point list, twiddles,
// zeroed sums and the time block.
int dft_setup(emlab_grid* g, const int* boxes, int nbox, const float* wavelengths, int n_freq, int block_cap) {
    g->dft_boxes.assign((size_t)nbox * kDftBoxInts, 0);
    long long total = 0;
    int largest = 0;
    for (int k = 0; k < nbox; ++k) {
        int* b = g->dft_boxes.data() + (size_t)k * kDftBoxInts;
        for (int a = 0; a < 6; ++a) b[a] = boxes[6 * k + a];
        b[6] = 0;
        for (int f = 0; f < 6; ++f) {
            const int a = f >> 1, u = a == 0 ? 1 : 0, v = a == 2 ? 1 : 2;
            b[7 + f] = b[6 + f] + (b[3 + u] - b[u] + 1) * (b[3 + v] - b[v] + 1);
        }
        b[13] = (int)total;
        b[14] = b[12];
        total += b[12];
        largest = std::max(largest, b[12]);
    }
    EMLAB_REQUIRE(total < (1ll << 28), "far-field DFT boxes have too many points");
    g->dft_nbox = nbox;
    g->dft_box_max = largest;
    g->dft_points = (int)total;
    g->dft_nf = n_freq;
    g->dft_block_cap = block_cap;
    g->dft_wl.assign(wavelengths, wavelengths + n_freq);
    g->dft_omega.assign((size_t)n_freq, 0.0);
    std::vector<float2> w((size_t)n_freq * kDftCoreBlock);
    const double dt = (double)g->cfg.courant;
    for (int f = 0; f < n_freq; ++f) {
        g->dft_omega[(size_t)f] = 6.28318530717958647692 / (double)std::max(wavelengths[f], 2.0f);
        for (int k = 0; k < kDftCoreBlock; ++k) {
            const double ph = g->dft_omega[(size_t)f] * dt * k;
            w[(size_t)f * kDftCoreBlock + k] = make_float2((float)std::cos(ph), (float)-std::sin(ph));
        }
    }
    EMLAB_CUDA(g->d_dft_box.alloc(g->dft_boxes.size()));
    EMLAB_CUDA(cudaMemcpyAsync(g->d_dft_box.p, g->dft_boxes.data(), g->dft_boxes.size() * 4, cudaMemcpyHostToDevice, g->stream));
    EMLAB_CUDA(g->d_dft_w.alloc(w.size()));
    EMLAB_CUDA(cudaMemcpyAsync(g->d_dft_w.p, w.data(), w.size() * 8, cudaMemcpyHostToDevice, g->stream));
    EMLAB_CUDA(g->d_dft_omega.alloc((size_t)n_freq));
    EMLAB_CUDA(cudaMemcpyAsync(g->d_dft_omega.p, g->dft_omega.data(), (size_t)n_freq * 8, cudaMemcpyHostToDevice, g->stream));
    std::vector<float> bhi, blo;
    dft_tc_twiddles(n_freq, g->dft_omega.data(), dt, bhi, blo);
    EMLAB_CUDA(g->d_dft_bhi.alloc(bhi.size()));
    EMLAB_CUDA(g->d_dft_blo.alloc(blo.size()));
    EMLAB_CUDA(cudaMemcpyAsync(g->d_dft_bhi.p, bhi.data(), bhi.size() * 4, cudaMemcpyHostToDevice, g->stream));
    EMLAB_CUDA(cudaMemcpyAsync(g->d_dft_blo.p, blo.data(), blo.size() * 4, cudaMemcpyHostToDevice, g->stream));
    // room for the longer of the two engines' blocks (the engine may change between folds), or the cap
    const int block = block_cap > 0 ? block_cap : std::max(kDftCoreBlock, dft_tc_block(n_freq));
    EMLAB_CUDA(g->d_dft_blk.alloc((size_t)block * 6 * g->dft_points));
    EMLAB_CUDA(g->d_dft_x.alloc((size_t)n_freq * g->dft_points * 12));
    EMLAB_CUDA(cudaMemsetAsync(g->d_dft_x.p, 0, g->d_dft_x.n * 8, g->stream));
    g->dft_t = 0, g->dft_samples = 0;
    g->dft_on = true;
    return EMLAB_OK;
}

int dft_detach(emlab_grid* g) {
    EMLAB_CUDA(cudaSetDevice(g->device));
    EMLAB_CUDA(cudaStreamSynchronize(g->stream));
    invalidate_graphs(g);
    g->dft_on = false;
    g->dft_nbox = 0, g->dft_points = 0;
    g->d_dft_x.release(), g->d_dft_blk.release();
    return EMLAB_OK;
}
}  // namespace

int emlab_ntff_dft_configure(emlab_grid* g, const int box_min[3], const int box_max[3], const float* wavelengths,
                             int n_freq, int box_out[6]) {
    if (int rc = require_grid(g)) return rc;
    if (int rc = dft_detach(g)) return rc;
    if (n_freq <= 0) return EMLAB_OK;
    EMLAB_REQUIRE(box_min && box_max && wavelengths, "null DFT argument");
    EMLAB_REQUIRE(n_freq <= 128, "at most 128 DFT frequencies");
    const int n[3] = {g->cfg.nx, g->cfg.ny, g->cfg.nz};
    const int L = g->cfg.pml_thickness;
    int b[6];
    for (int a = 0; a < 3; ++a) {
        const int lo = L + 1, hi = n[a] - L - 2;
        b[a] = std::clamp(std::min(box_min[a], box_max[a]), lo, hi);
        b[3 + a] = std::clamp(std::max(box_min[a], box_max[a]), lo, hi);
        if (b[3 + a] - b[a] < 4)
            return fail(EMLAB_ERR_INVALID, "far-field DFT box is degenerate after clamping to the region inside the "
                                           "absorbing layer");
        if (box_out) box_out[a] = b[a], box_out[3 + a] = b[3 + a];
    }
    return dft_setup(g, b, 1, wavelengths, n_freq, 0);
}

int emlab_ntff_dft_configure_boxes(emlab_grid* g, const int* boxes, int n_boxes, const float* wavelengths,
                                   int n_freq, int block) {
    if (int rc = require_grid(g)) return rc;
    if (int rc = dft_detach(g)) return rc;
    if (n_freq <= 0 || n_boxes <= 0) return EMLAB_OK;
    EMLAB_REQUIRE(boxes && wavelengths, "null DFT argument");
    EMLAB_REQUIRE(n_freq <= 128, "at most 128 DFT frequencies");
    EMLAB_REQUIRE(n_boxes <= 65535, "too many far-field DFT boxes");
    EMLAB_REQUIRE(block == 0 || (block >= kDftCoreBlock && block <= dft_tc_block(n_freq) && block % kDftCoreBlock == 0),
                  "DFT block must be 0 or a multiple of 64 up to the tensor-core fold's block");
    const int n[3] = {g->cfg.nx, g->cfg.ny, g->cfg.nz};
    for (int k = 0; k < n_boxes; ++k)
        for (int a = 0; a < 3; ++a) {
            const int lo = boxes[6 * k + a], hi = boxes[6 * k + 3 + a];
            if (lo < 1 || hi > n[a] - 2 || hi - lo < 4)
                return fail(EMLAB_ERR_INVALID, "far-field DFT box " + std::to_string(k) +
                                                   " leaves the grid's interior or is degenerate (< 4 cells)");
        }
    return dft_setup(g, boxes, n_boxes, wavelengths, n_freq, block);
}

int emlab_ntff_dft_info(emlab_grid* g, int* points, uint64_t* samples) {
    if (int rc = require_grid(g)) return rc;
    if (points) *points = g->dft_on ? g->dft_points : 0;
    if (samples) *samples = g->dft_samples + (uint64_t)g->dft_t;
    return EMLAB_OK;
}

int emlab_ntff_dft_read(emlab_grid* g, double* out) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(g->dft_on, "far-field DFT monitor is not configured");
    EMLAB_REQUIRE(out, "null output");
    EMLAB_CUDA(cudaSetDevice(g->device));
    if (int rc = dft_fold(g)) return rc;
    if (int rc = check_launch()) return rc;
    std::vector<double> x(g->d_dft_x.n);  // device layout [f][c][i][2] -> [f][i][c][2]
    EMLAB_CUDA(cudaMemcpyAsync(x.data(), g->d_dft_x.p, x.size() * 8, cudaMemcpyDeviceToHost, g->stream));
    if (int rc = emlab_grid_synchronize(g, 0)) return rc;
    const size_t P = (size_t)g->dft_points;
    for (size_t f = 0; f < (size_t)g->dft_nf; ++f)
        for (size_t c = 0; c < 6; ++c)
            for (size_t i = 0; i < P; ++i) {
                const size_t src = ((f * 6 + c) * P + i) * 2, dst = ((f * P + i) * 6 + c) * 2;
                out[dst] = x[src], out[dst + 1] = x[src + 1];
            }
    return EMLAB_OK;
}

int emlab_ntff_dft_engine(emlab_grid* g, int engine) {
    if (!g) return fail(EMLAB_ERR_INVALID, "null grid handle");
    EMLAB_REQUIRE(engine == EMLAB_DFT_TENSOR || engine == EMLAB_DFT_CUDA_CORES, "unknown DFT engine");
    if (engine != g->dft_engine && g->dft_on) {
        if (int rc = require_grid(g)) return rc;
        if (int rc = dft_fold(g)) return rc;  // the partial block is folded with the engine that gathered it
    }
    g->dft_engine = engine;
    return EMLAB_OK;
}

int emlab_ntff_dft_evaluate(emlab_grid* g, int f, const float* directions, int n_dirs, float* out) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(g->dft_on && f >= 0 && f < g->dft_nf, "far-field DFT frequency out of range");
    EMLAB_REQUIRE(g->dft_nbox == 1, "the DFT has several boxes: evaluate them one by one with emlab_ntff_dft_spectra");
    EMLAB_REQUIRE(directions && out && n_dirs > 0, "bad direction arguments");
    EMLAB_CUDA(cudaSetDevice(g->device));
    if (int rc = dft_fold(g)) return rc;
    const uint64_t samples = g->dft_samples;
    EMLAB_REQUIRE(samples > 0, "no far-field DFT samples yet");
    DevBuf<float> ph;
    EMLAB_CUDA(ph.alloc((size_t)g->dft_points * 32));
    launch_dft_to_phasor(g->d_dft_x.p, g->dft_points, f, 2.0 / (double)samples, ph.p, g->stream);
    const int slices = std::clamp((g->dft_points + 4095) / 4096, 1, 64);
    const int chunk = 4096;
    DevBuf<float4> d_dirs, d_part;
    DevBuf<float> d_out;
    EMLAB_CUDA(d_dirs.alloc((size_t)n_dirs));
    EMLAB_CUDA(cudaMemcpyAsync(d_dirs.p, directions, (size_t)n_dirs * 16, cudaMemcpyHostToDevice, g->stream));
    EMLAB_CUDA(d_part.alloc((size_t)chunk * slices * 4));
    EMLAB_CUDA(d_out.alloc((size_t)n_dirs * 2));
    const float k = (float)g->dft_omega[(size_t)f];
    for (int first = 0; first < n_dirs; first += chunk) {
        const int count = std::min(chunk, n_dirs - first);
        launch_ntff_pattern(g->d_dft_box.p, g->dft_points, ph.p, d_dirs.p, first, count, slices, k, d_part.p,
                            g->stream);
        launch_ntff_reduce(d_dirs.p, d_part.p, first, count, slices, d_out.p, g->stream);
        g_launches += 2;
    }
    g_launches += 1;
    if (int rc = check_launch()) return rc;
    std::vector<float> tmp((size_t)n_dirs * 2);
    EMLAB_CUDA(cudaMemcpyAsync(tmp.data(), d_out.p, tmp.size() * 4, cudaMemcpyDeviceToHost, g->stream));
    if (int rc = emlab_grid_synchronize(g, 0)) return rc;
    for (int d = 0; d < n_dirs; ++d) out[2 * d] = tmp[2 * (size_t)d], out[2 * d + 1] = d == 0 ? tmp[1] : 0.0f;
    return EMLAB_OK;
}

int emlab_ntff_dft_evaluate_all(emlab_grid* g, const float* directions, int n_dirs, float* out) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(g->dft_on, "no far-field DFT attached");
    EMLAB_REQUIRE(g->dft_nbox == 1, "the DFT has several boxes: evaluate them one by one with emlab_ntff_dft_spectra");
    EMLAB_REQUIRE(directions && out && n_dirs > 0, "bad direction arguments");
    EMLAB_CUDA(cudaSetDevice(g->device));
    if (int rc = dft_fold(g)) return rc;
    const uint64_t samples = g->dft_samples;
    EMLAB_REQUIRE(samples > 0, "no far-field DFT samples yet");
    const int slices = std::clamp((g->dft_points + 4095) / 4096, 1, 64);
    const int chunk = 8192;
    DevBuf<float> ph, d_out;
    DevBuf<float4> d_dirs, d_part;
    EMLAB_CUDA(ph.alloc((size_t)g->dft_points * 32));
    EMLAB_CUDA(d_dirs.alloc((size_t)n_dirs));
    EMLAB_CUDA(cudaMemcpyAsync(d_dirs.p, directions, (size_t)n_dirs * 16, cudaMemcpyHostToDevice, g->stream));
    EMLAB_CUDA(d_part.alloc((size_t)chunk * slices * 4));
    EMLAB_CUDA(d_out.alloc((size_t)g->dft_nf * n_dirs * 2));
    for (int f = 0; f < g->dft_nf; ++f) {
        launch_dft_to_phasor(g->d_dft_x.p, g->dft_points, f, 2.0 / (double)samples, ph.p, g->stream);
        const float k = (float)g->dft_omega[(size_t)f];
        for (int first = 0; first < n_dirs; first += chunk) {
            const int count = std::min(chunk, n_dirs - first);
            launch_ntff_pattern_fast(g->d_dft_box.p, g->dft_points, ph.p, d_dirs.p, first, count, slices, k,
                                     d_part.p, g->stream);
            launch_ntff_reduce(d_dirs.p, d_part.p, first, count, slices, d_out.p + (size_t)f * n_dirs * 2, g->stream);
            g_launches += 2;
        }
        g_launches += 1;
    }
    if (int rc = check_launch()) return rc;
    EMLAB_CUDA(cudaMemcpyAsync(out, d_out.p, (size_t)g->dft_nf * n_dirs * 8, cudaMemcpyDeviceToHost, g->stream));
    if (int rc = emlab_grid_synchronize(g, 0)) return rc;
    for (int f = 0; f < g->dft_nf; ++f)  // the radiated power is reported once per frequency (first direction)
        for (int d = 1; d < n_dirs; ++d) out[((size_t)f * n_dirs + d) * 2 + 1] = 0.0f;
    return EMLAB_OK;
}

int emlab_ntff_dft_spectra(emlab_grid* g, int box, const float* directions, int n_dirs, float* out) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(g->dft_on, "no far-field DFT attached");
    EMLAB_REQUIRE(box >= 0 && box < g->dft_nbox, "no such far-field DFT box");
    EMLAB_REQUIRE(directions && out && n_dirs > 0 && n_dirs <= 8192, "bad direction arguments (1 to 8192 directions)");
    EMLAB_CUDA(cudaSetDevice(g->device));
    if (int rc = dft_fold(g)) return rc;
    const uint64_t samples = g->dft_samples;
    EMLAB_REQUIRE(samples > 0, "no far-field DFT samples yet");
    const int* rec = g->dft_boxes.data() + (size_t)box * kDftBoxInts;
    const int first = rec[13], points = rec[14];
    const int slices = std::clamp((points + 4095) / 4096, 1, 64);
    const size_t part = (size_t)g->dft_nf * n_dirs * slices * 4, outs = (size_t)g->dft_nf * n_dirs * 2;
    // the scratch grows to the largest request and stays (no allocation in a steady loop)
    if (g->d_spec_dirs.n < (size_t)n_dirs) EMLAB_CUDA(g->d_spec_dirs.alloc((size_t)n_dirs));
    if (g->d_spec_part.n < part) EMLAB_CUDA(g->d_spec_part.alloc(part));
    if (g->d_spec_out.n < outs) EMLAB_CUDA(g->d_spec_out.alloc(outs));
    EMLAB_CUDA(cudaMemcpyAsync(g->d_spec_dirs.p, directions, (size_t)n_dirs * 16, cudaMemcpyHostToDevice, g->stream));
    launch_ntff_spectra(g->d_dft_box.p + (size_t)box * kDftBoxInts, first, points, g->dft_points, g->d_dft_x.p,
                        g->dft_nf, g->d_dft_omega.p, 2.0 / (double)samples, g->d_spec_dirs.p, n_dirs, slices,
                        g->d_spec_part.p, g->stream);
    launch_ntff_reduce_multi(g->d_spec_dirs.p, g->d_spec_part.p, n_dirs, slices, g->dft_nf, g->d_spec_out.p, g->stream);
    g_launches += 2;
    if (int rc = check_launch()) return rc;
    EMLAB_CUDA(cudaMemcpyAsync(out, g->d_spec_out.p, outs * 4, cudaMemcpyDeviceToHost, g->stream));
    if (int rc = emlab_grid_synchronize(g, 0)) return rc;
    for (int f = 0; f < g->dft_nf; ++f)  // the radiated power is reported once per frequency (first direction)
        for (int d = 1; d < n_dirs; ++d) out[((size_t)f * n_dirs + d) * 2 + 1] = 0.0f;
    return EMLAB_OK;
}

}  // extern "C"

int emlab::dft_fold_now(emlab_grid* g) {
    if (int rc = dft_fold(g)) return rc;
    return check_launch();
}

int emlab::dft_carry_take(emlab_grid* g, const std::vector<int>& old_z0, const std::vector<int>& old_nz,
                          const std::vector<int>& idx, const std::vector<int>& new_z0, DftCarry& c) {
    c = DftCarry();
    if (!g->dft_on) return EMLAB_OK;
    if (int rc = dft_fold(g)) return rc;
    for (int k = 0; k < g->dft_nbox; ++k) {
        const int* b = g->dft_boxes.data() + (size_t)k * kDftBoxInts;
        for (size_t j = 0; j < idx.size(); ++j) {
            const int s = idx[j], z0 = old_z0[(size_t)s];
            if (b[2] < z0 || b[5] >= z0 + old_nz[(size_t)s]) continue;  // the box lies inside scene s
            const int shift = new_z0[j] - z0;
            c.boxes.insert(c.boxes.end(), {b[0], b[1], b[2] + shift, b[3], b[4], b[5] + shift});
            c.old_first.push_back(b[13]);
        }
    }
    c.on = !c.old_first.empty();
    c.wl = g->dft_wl;
    c.old_points = g->dft_points;
    c.block_cap = g->dft_block_cap;
    c.engine = g->dft_engine;
    c.samples = g->dft_samples;
    std::swap(c.x.p, g->d_dft_x.p), std::swap(c.x.n, g->d_dft_x.n);  // the old sums stay alive for the gather
    return EMLAB_OK;
}

int emlab::dft_carry_restore(emlab_grid* g, DftCarry& c) {
    if (!c.on) return EMLAB_OK;
    const int nbox = (int)c.old_first.size();
    if (int rc = dft_setup(g, c.boxes.data(), nbox, c.wl.data(), (int)c.wl.size(), c.block_cap)) return rc;
    g->dft_engine = c.engine;
    std::vector<int> map((size_t)g->dft_points);
    for (int k = 0; k < nbox; ++k) {
        const int* b = g->dft_boxes.data() + (size_t)k * kDftBoxInts;
        for (int i = 0; i < b[14]; ++i) map[(size_t)b[13] + i] = c.old_first[(size_t)k] + i;
    }
    DevBuf<int> d_map;
    EMLAB_CUDA(d_map.alloc(map.size()));
    EMLAB_CUDA(cudaMemcpyAsync(d_map.p, map.data(), map.size() * 4, cudaMemcpyHostToDevice, g->stream));
    launch_dft_gather(c.x.p, c.old_points, d_map.p, g->dft_points, g->dft_nf, g->d_dft_x.p, g->stream);
    ++g_launches;
    if (int rc = check_launch()) return rc;
    EMLAB_CUDA(cudaStreamSynchronize(g->stream));
    g->dft_samples = c.samples;
    g->dft_t = 0;
    return EMLAB_OK;
}

extern "C" {

// ---- probes and flux ----------------------------------------------------------------------
int emlab_probe_gather(emlab_grid* g, const int* origins, int n_probes, float* out) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(origins && out && n_probes > 0, "bad probe arguments");
    EMLAB_CUDA(cudaSetDevice(g->device));
    DevBuf<int4> d_o;
    DevBuf<float4> d_out;
    EMLAB_CUDA(d_o.alloc((size_t)n_probes));
    EMLAB_CUDA(d_out.alloc((size_t)n_probes * 54));
    EMLAB_CUDA(cudaMemcpyAsync(d_o.p, origins, (size_t)n_probes * 16, cudaMemcpyHostToDevice, g->stream));
    launch_probe_gather(monitor_args(g), d_o.p, n_probes, d_out.p, nullptr, nullptr, g->stream);
    ++g_launches;
    if (int rc = check_launch()) return rc;
    EMLAB_CUDA(cudaMemcpyAsync(out, d_out.p, (size_t)n_probes * 54 * 16, cudaMemcpyDeviceToHost, g->stream));
    if (int rc = emlab_grid_synchronize(g, 0)) return rc;
    if (int rc = ensure_cell_materials(g)) return rc;
    const int nx = g->cfg.nx, ny = g->cfg.ny, nz = g->cfg.nz;
    for (int id = 0; id < n_probes * 54; ++id) {
        const int probe = id / 54, k = id % 54, t = k % 27;
        const int* o = origins + probe * 4;
        const int x = std::clamp(o[0] + t % 3, 0, nx - 1), y = std::clamp(o[1] + (t / 3) % 3, 0, ny - 1),
                  z = std::clamp(o[2] + t / 9, 0, nz - 1);
        const size_t ci = ((size_t)z * ny + y) * nx + x;
        out[(size_t)id * 4 + 3] = k < 27 ? g->cell_sigma[ci] : g->cell_eps[ci];
    }
    return EMLAB_OK;
}

int emlab_render(emlab_grid* g, const emlab_render_params* params, unsigned char* rgba) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(params && rgba, "null render argument");
    EMLAB_REQUIRE(params->width > 0 && params->height > 0 && params->width <= 16384 && params->height <= 16384,
                  "render size must be 1..16384 pixels per side");
    EMLAB_REQUIRE(std::isfinite(params->step_voxels), "render step must be finite");
    // the host-side clamps of VolumeRenderer::render (src/VolumeRenderer.cpp:102, 110)
    emlab_render_params q = *params;
    q.step_voxels = std::clamp(q.step_voxels, 0.1f, 4.0f);
    q.signed_axis = std::clamp(q.signed_axis, 0, 2);
    EMLAB_CUDA(cudaSetDevice(g->device));
    const size_t cells = (size_t)g->cfg.nx * g->cfg.ny * g->cfg.nz;
    const size_t pixels = (size_t)q.width * q.height;
    DevBuf<float> d_sigma, d_eps;
    DevBuf<unsigned char> d_img;
    if (int rc = ensure_cell_materials(g)) return rc;
    const bool mats = g->cell_sigma.size() == cells && g->cell_eps.size() == cells;
    if (mats) {
        EMLAB_CUDA(d_sigma.alloc(cells));
        EMLAB_CUDA(d_eps.alloc(cells));
        EMLAB_CUDA(cudaMemcpyAsync(d_sigma.p, g->cell_sigma.data(), cells * 4, cudaMemcpyHostToDevice, g->stream));
        EMLAB_CUDA(cudaMemcpyAsync(d_eps.p, g->cell_eps.data(), cells * 4, cudaMemcpyHostToDevice, g->stream));
    }
    EMLAB_CUDA(d_img.alloc(pixels * 4));
    launch_raymarch(monitor_args(g), mats ? d_sigma.p : nullptr, mats ? d_eps.p : nullptr, q, d_img.p, g->stream);
    ++g_launches;
    if (int rc = check_launch()) return rc;
    EMLAB_CUDA(cudaMemcpyAsync(rgba, d_img.p, pixels * 4, cudaMemcpyDeviceToHost, g->stream));
    return emlab_grid_synchronize(g, 0);
}

int emlab_flux_planes(emlab_grid* g, const emlab_flux_plane* planes, int n_planes, double* out) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(planes && out && n_planes >= 0, "bad flux arguments");
    EMLAB_CUDA(cudaSetDevice(g->device));
    const int size[3] = {g->cfg.nx, g->cfg.ny, g->cfg.nz};
    struct Rect {
        int axis, index, m0, m1, r0, r1;
        size_t groups, offset;
    };
    std::vector<Rect> rects;
    size_t total = 0;
    for (int i = 0; i < n_planes; ++i) {
        const emlab_flux_plane& p = planes[i];
        Rect r{std::clamp(p.axis, 0, 2), p.index, 0, 0, 0, 0, 0, total};
        const int u = r.axis == 0 ? 1 : 0, v = r.axis == 2 ? 1 : 2;
        r.m0 = std::max(p.rect_min[0], 0), r.m1 = std::max(p.rect_min[1], 0);
        r.r0 = std::min(p.rect_max[0], size[u]) - r.m0, r.r1 = std::min(p.rect_max[1], size[v]) - r.m1;
        if (p.index < 0 || p.index >= size[r.axis] || r.r0 <= 0 || r.r1 <= 0) r.groups = 0;
        else r.groups = (size_t)((r.r0 + 15) / 16) * ((r.r1 + 15) / 16);
        total += r.groups;
        rects.push_back(r);
    }
    DevBuf<float> d_part;
    EMLAB_CUDA(d_part.alloc(std::max<size_t>(total, 1)));
    const MonitorArgs m = monitor_args(g);
    for (const Rect& r : rects) {
        if (!r.groups) continue;
        launch_flux_plane(m, r.axis, r.index, r.m0, r.m1, r.r0, r.r1, d_part.p + r.offset, g->stream);
        ++g_launches;
    }
    if (int rc = check_launch()) return rc;
    std::vector<float> part(std::max<size_t>(total, 1));
    EMLAB_CUDA(cudaMemcpyAsync(part.data(), d_part.p, part.size() * 4, cudaMemcpyDeviceToHost, g->stream));
    if (int rc = emlab_grid_synchronize(g, 0)) return rc;
    for (int i = 0; i < n_planes; ++i) {
        double s = 0.0;  // FP64 sum of the FP32 workgroup partials (FieldAnalyzer.cpp:356-357)
        for (size_t k = 0; k < rects[i].groups; ++k) s += (double)part[rects[i].offset + k];
        out[i] = s;
    }
    return EMLAB_OK;
}

// ---- FieldAnalyzer::submit / collect (src/FieldAnalyzer.cpp:126-272) ------------------------
int emlab_analyzer_submit(emlab_grid* g, const int* origins, int n_probes, const emlab_flux_plane* planes,
                          int n_planes) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(n_probes >= 0 && n_planes >= 0 && (origins || !n_probes) && (planes || !n_planes),
                  "bad analyzer arguments");
    AnalyzerSlot& a = g->analyzer[g->analyzer_next];
    EMLAB_REQUIRE(!a.pending, "two measurements are in flight: collect one first");
    EMLAB_CUDA(cudaSetDevice(g->device));
    if (!a.done) EMLAB_CUDA(cudaEventCreateWithFlags(&a.done, cudaEventDisableTiming));
    const int size[3] = {g->cfg.nx, g->cfg.ny, g->cfg.nz};
    a.planes.clear();
    size_t total = 0;
    std::vector<int> geo;  // axis, index, m0, m1, r0, r1 per plane with partials
    for (int i = 0; i < n_planes; ++i) {
        const emlab_flux_plane& p = planes[i];
        const int axis = std::clamp(p.axis, 0, 2);
        const int u = axis == 0 ? 1 : 0, v = axis == 2 ? 1 : 2;
        const int m0 = std::max(p.rect_min[0], 0), m1 = std::max(p.rect_min[1], 0);
        const int r0 = std::min(p.rect_max[0], size[u]) - m0, r1 = std::min(p.rect_max[1], size[v]) - m1;
        size_t groups = 0;
        if (p.index >= 0 && p.index < size[axis] && r0 > 0 && r1 > 0)
            groups = (size_t)((r0 + 15) / 16) * ((r1 + 15) / 16);
        a.planes.emplace_back(total, groups);
        geo.insert(geo.end(), {axis, p.index, m0, m1, r0, r1});
        total += groups;
    }
    if ((size_t)n_probes > a.probe_cap) {
        if (a.h_probe) cudaFreeHost(a.h_probe);
        a.h_probe = nullptr;
        a.probe_cap = 0;  // a failed allocation below leaves the slot empty, not a null buffer of old capacity
        EMLAB_CUDA(cudaMallocHost(&a.h_probe, (size_t)n_probes * 54 * 16));
        EMLAB_CUDA(a.d_origins.alloc((size_t)n_probes));
        EMLAB_CUDA(a.d_probe.alloc((size_t)n_probes * 54));
        a.probe_cap = (size_t)n_probes;
    }
    if (total > a.part_cap) {
        if (a.h_part) cudaFreeHost(a.h_part);
        a.h_part = nullptr;
        a.part_cap = 0;
        EMLAB_CUDA(cudaMallocHost(&a.h_part, total * 4));
        EMLAB_CUDA(a.d_part.alloc(total));
        a.part_cap = total;
    }
    a.origins.assign(origins, origins + (size_t)n_probes * 4);
    a.n_probes = n_probes;
    const MonitorArgs m = monitor_args(g);
    if (n_probes) {
        EMLAB_CUDA(cudaMemcpyAsync(a.d_origins.p, a.origins.data(), (size_t)n_probes * 16, cudaMemcpyHostToDevice,
                                   g->stream));
        launch_probe_gather(m, a.d_origins.p, n_probes, a.d_probe.p, nullptr, nullptr, g->stream);
        ++g_launches;
        EMLAB_CUDA(cudaMemcpyAsync(a.h_probe, a.d_probe.p, (size_t)n_probes * 54 * 16, cudaMemcpyDeviceToHost,
                                   g->stream));
    }
    for (int i = 0; i < n_planes; ++i) {
        if (!a.planes[(size_t)i].second) continue;
        const int* q = &geo[(size_t)i * 6];
        launch_flux_plane(m, q[0], q[1], q[2], q[3], q[4], q[5], a.d_part.p + a.planes[(size_t)i].first, g->stream);
        ++g_launches;
    }
    if (total) EMLAB_CUDA(cudaMemcpyAsync(a.h_part, a.d_part.p, total * 4, cudaMemcpyDeviceToHost, g->stream));
    if (int rc = check_launch()) return rc;
    EMLAB_CUDA(cudaEventRecord(a.done, g->stream));
    a.pending = true;
    g->analyzer_next ^= 1;
    return EMLAB_OK;
}

int emlab_analyzer_collect(emlab_grid* g, float* probe_out, double* flux_out, int* ready) {
    if (int rc = require_grid(g)) return rc;
    if (ready) *ready = 0;
    AnalyzerSlot& a = g->analyzer[g->analyzer_oldest];
    if (!a.pending) return EMLAB_OK;
    EMLAB_REQUIRE((probe_out || !a.n_probes) && (flux_out || a.planes.empty()), "null analyzer output");
    EMLAB_CUDA(cudaSetDevice(g->device));
    EMLAB_CUDA(cudaEventSynchronize(a.done));
    if (int rc = ensure_cell_materials(g)) return rc;
    const int nx = g->cfg.nx, ny = g->cfg.ny, nz = g->cfg.nz;
    for (int id = 0; id < a.n_probes * 54; ++id) {
        const int probe = id / 54, k = id % 54, t = k % 27;
        const int* o = a.origins.data() + probe * 4;
        const int x = std::clamp(o[0] + t % 3, 0, nx - 1), y = std::clamp(o[1] + (t / 3) % 3, 0, ny - 1),
                  z = std::clamp(o[2] + t / 9, 0, nz - 1);
        const size_t ci = ((size_t)z * ny + y) * nx + x;
        const float4 v = a.h_probe[id];
        float* out = probe_out + (size_t)id * 4;
        out[0] = v.x, out[1] = v.y, out[2] = v.z;
        out[3] = k < 27 ? g->cell_sigma[ci] : g->cell_eps[ci];
    }
    for (size_t i = 0; i < a.planes.size(); ++i) {
        double s = 0.0;  // FP64 sum of the FP32 workgroup partials (FieldAnalyzer::collect, FieldAnalyzer.cpp:264-269)
        for (size_t k = 0; k < a.planes[i].second; ++k) s += (double)a.h_part[a.planes[i].first + k];
        flux_out[i] = s;
    }
    a.pending = false;
    g->analyzer_oldest ^= 1;
    if (ready) *ready = 1;
    return EMLAB_OK;
}

// ---- coax lines ----------------------------------------------------------------------------
int emlab_lines_configure(emlab_grid* g, const int* quantities, int n_quantities, const int* terms,
                          const float* weights, int n_terms, float wavelength, float averaging_periods) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_CUDA(cudaSetDevice(g->device));
    EMLAB_CUDA(cudaStreamSynchronize(g->stream));
    invalidate_graphs(g);
    g->nq = 0;
    g->d_q.release(), g->d_terms.release(), g->d_weights.release(), g->d_line_ph.release(), g->d_line_now.release();
    if (n_quantities <= 0) return EMLAB_OK;
    EMLAB_REQUIRE(quantities && (n_terms == 0 || (terms && weights)), "null line arrays");
    for (int q = 0; q < n_quantities; ++q) {
        const int* info = quantities + 4 * q;
        EMLAB_REQUIRE(info[0] >= 0 && info[1] >= 0 && info[0] + info[1] <= n_terms, "line quantity term range");
    }
    for (int t = 0; t < n_terms; ++t) EMLAB_REQUIRE(terms[4 * t + 3] >= 0 && terms[4 * t + 3] < 6, "line term component");
    EMLAB_CUDA(g->d_q.alloc((size_t)n_quantities));
    EMLAB_CUDA(cudaMemcpyAsync(g->d_q.p, quantities, (size_t)n_quantities * 16, cudaMemcpyHostToDevice, g->stream));
    EMLAB_CUDA(g->d_terms.alloc((size_t)std::max(n_terms, 1)));
    EMLAB_CUDA(g->d_weights.alloc((size_t)std::max(n_terms, 1)));
    if (n_terms > 0) {
        EMLAB_CUDA(cudaMemcpyAsync(g->d_terms.p, terms, (size_t)n_terms * 16, cudaMemcpyHostToDevice, g->stream));
        EMLAB_CUDA(cudaMemcpyAsync(g->d_weights.p, weights, (size_t)n_terms * 4, cudaMemcpyHostToDevice, g->stream));
    }
    EMLAB_CUDA(g->d_line_ph.alloc((size_t)n_quantities * 4));
    EMLAB_CUDA(cudaMemsetAsync(g->d_line_ph.p, 0, (size_t)n_quantities * 16, g->stream));
    EMLAB_CUDA(g->d_line_now.alloc((size_t)n_quantities));
    EMLAB_CUDA(cudaMemsetAsync(g->d_line_now.p, 0, (size_t)n_quantities * 4, g->stream));
    g->nq = n_quantities;
    g->line_wl = std::max(wavelength, 2.0f);
    g->line_avg = averaging_periods;
    return EMLAB_OK;
}

int emlab_lines_read(emlab_grid* g, float* phasors, float* now) {
    if (int rc = require_grid(g)) return rc;
    if (!g->nq) return EMLAB_OK;
    if (phasors)
        EMLAB_CUDA(cudaMemcpyAsync(phasors, g->d_line_ph.p, (size_t)g->nq * 16, cudaMemcpyDeviceToHost, g->stream));
    if (now) EMLAB_CUDA(cudaMemcpyAsync(now, g->d_line_now.p, (size_t)g->nq * 4, cudaMemcpyDeviceToHost, g->stream));
    return emlab_grid_synchronize(g, 0);
}

// ---- host-side set-up ----------------------------------------------------------------------
int emlab_edge_materials(const float* sigma, const float* eps_r, int nx, int ny, int nz,
                         const emlab_edge_override* edges, size_t n_edges, const emlab_wire_term* wires,
                         size_t n_wires, float* edge_sigma, float* edge_eps, float* wire0, float* wire1,
                         uint32_t* classes) {
    EMLAB_REQUIRE(sigma && eps_r && nx > 0 && ny > 0 && nz > 0, "bad material arguments");
    EMLAB_REQUIRE((edges || n_edges == 0) && (wires || n_wires == 0), "null override array");
    ClassTable t;
    std::string err;
    if (!build_classes(sigma, eps_r, nx, ny, nz, edges, n_edges, wires, n_wires, 0.5f, t, err))
        return fail(EMLAB_ERR_OOM, err);
    const int pitch = row_pitch(nx);
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const size_t i = ((size_t)z * ny + y) * nx + x;
                const uint32_t c = t.cls[((size_t)z * ny + y) * pitch + x];
                const float* m = &t.tabM[(size_t)c * 8];
                const float* w = &t.tabW[(size_t)c * 8];
                for (int a = 0; a < 3; ++a) {
                    if (edge_sigma) edge_sigma[i * 3 + a] = m[a];
                    if (edge_eps) edge_eps[i * 3 + a] = m[3 + a];
                    if (wire0) wire0[i * 3 + a] = w[a];
                    if (wire1) wire1[i * 3 + a] = w[3 + a];
                }
            }
    if (classes) *classes = t.classes;
    return EMLAB_OK;
}

double emlab_source_signal(const emlab_source* source, double t) { return source ? source_signal(*source, t) : 0.0; }

int emlab_source_lists(const emlab_source* sources, size_t n, int nx, int ny, int nz, float* packed, int32_t* cells,
                       int32_t* lists, int* n_sources, int* n_cells, int* n_lists) {
    EMLAB_REQUIRE((sources || n == 0) && nx > 0 && ny > 0 && nz > 0 && n_sources && n_cells && n_lists,
                  "bad source-list arguments");
    std::vector<emlab_source> desc;
    std::vector<float> pk;
    const int nsrc = pack_sources(sources, n, desc, pk);
    std::vector<int32_t> c, l;
    const int size[3] = {nx, ny, nz};
    source_lists(pk, nsrc, size, c, l);
    *n_sources = nsrc;
    *n_cells = (int)(c.size() / 4) - 1;  // the sentinel is not a cell
    *n_lists = (int)l.size();
    if (packed) std::copy(pk.begin(), pk.end(), packed);
    if (cells) std::copy(c.begin(), c.end(), cells);
    if (lists) std::copy(l.begin(), l.end(), lists);
    return EMLAB_OK;
}

// ---- self-checks ---------------------------------------------------------------------------
int emlab_debug_set_wait_limit(int polls) {
    EMLAB_REQUIRE(polls >= 0, "negative poll count");
    g_wait_polls = polls > 0 ? std::min(polls, kWaitPolls) : 0;
    return EMLAB_OK;
}

int emlab_debug_pair_schedule(int nx, int ny, int nz, int tile_rows, int ctas, int* zc, int* items) {
    EMLAB_REQUIRE(zc && items, "null output");
    EMLAB_REQUIRE(nx > 0 && ny > 0 && nz > 0, "empty grid");
    EMLAB_REQUIRE(tile_rows == 4 || tile_rows == 8 || tile_rows == 16, "pair tiles have 4, 8 or 16 rows");
    EMLAB_REQUIRE(ctas > 0, "no CTAs");
    pair_schedule_shape(nx, ny, nz, tile_rows, ctas, zc, items);
    return EMLAB_OK;
}

int emlab_debug_ragged_items(const int* z0, const int* nx, const int* ny, const int* nz, int n_scenes, int tile_rows,
                             int ctas, int* out, size_t cap, size_t* n_items) {
    EMLAB_REQUIRE(z0 && nx && ny && nz && n_items && n_scenes > 0, "null argument or no scenes");
    EMLAB_REQUIRE(tile_rows == 4 || tile_rows == 8 || tile_rows == 16, "pair tiles have 4, 8 or 16 rows");
    EMLAB_REQUIRE(ctas > 0, "no CTAs");
    std::vector<int> vz0(z0, z0 + n_scenes), vnx(nx, nx + n_scenes), vny(ny, ny + n_scenes), vnz(nz, nz + n_scenes);
    for (int i = 0; i < n_scenes; ++i)
        EMLAB_REQUIRE(vnx[i] > 0 && vny[i] > 0 && vnz[i] > 0 && vnx[i] < 65536 && vny[i] < 65536 && vz0[i] >= 0,
                      "scene extents out of range");
    const std::vector<int4> items = ragged_items(vz0, vnx, vny, vnz, tile_rows, ctas);
    *n_items = items.size();
    if (!out) return EMLAB_OK;
    EMLAB_REQUIRE(cap >= items.size(), "output too small");
    for (size_t k = 0; k < items.size(); ++k) {
        const int4 t = items[k];
        int* o = out + 5 * k;
        o[0] = t.x & 0xffff, o[1] = (int)((unsigned)t.x >> 16), o[2] = t.y, o[3] = t.z, o[4] = t.w;
    }
    return EMLAB_OK;
}

int emlab_debug_expf(const float* in, float* out, size_t n) {
    if (!in || !out) return fail(EMLAB_ERR_INVALID, "null argument");
    if (!n) return EMLAB_OK;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return fail(EMLAB_ERR_NO_DEVICE, "no CUDA device");
    DevBuf<float> d_in, d_out;
    EMLAB_CUDA(d_in.alloc(n));
    EMLAB_CUDA(d_out.alloc(n));
    EMLAB_CUDA(cudaMemcpy(d_in.p, in, n * 4, cudaMemcpyHostToDevice));
    launch_debug_expf(d_in.p, d_out.p, n, 0);
    ++g_launches;
    if (int rc = check_launch()) return rc;
    EMLAB_CUDA(cudaMemcpy(out, d_out.p, n * 4, cudaMemcpyDeviceToHost));
    return EMLAB_OK;
}

}  // extern "C"
