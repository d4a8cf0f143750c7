// grid_state.h - the state behind an emlab_grid handle, shared by the C-ABI translation units
// (capi.cu: single grids and monitors; stack.cu: stacks of independent scenes).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "emlab_internal.h"
#include "setup.h"

namespace emlab {

// Records msg as the calling thread's last error and returns code.
int fail(int code, const std::string& msg);

#define EMLAB_CUDA(call)                                                                                      \
    do {                                                                                                      \
        cudaError_t e_ = (call);                                                                              \
        if (e_ != cudaSuccess)                                                                                \
            return fail(e_ == cudaErrorMemoryAllocation ? EMLAB_ERR_OOM : EMLAB_ERR_CUDA,                     \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                                  \
    } while (0)

#define EMLAB_REQUIRE(cond, msg) \
    do {                         \
        if (!(cond)) return fail(EMLAB_ERR_INVALID, msg); \
    } while (0)

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t alloc(size_t count) {
        release();
        if (count == 0) return cudaSuccess;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e == cudaSuccess) n = count;
        else p = nullptr;
        return e;
    }
};

constexpr int kChunk = 1024;  // sub-steps whose host-side scalars are uploaded together

// One queued FieldAnalyzer measurement: device outputs, pinned host copies, the event that ends it.
struct AnalyzerSlot {
    DevBuf<int4> d_origins;
    DevBuf<float4> d_probe;
    DevBuf<float> d_part;
    float4* h_probe = nullptr;
    float* h_part = nullptr;
    size_t probe_cap = 0, part_cap = 0;
    cudaEvent_t done = nullptr;
    std::vector<int> origins;                 // 4 ints per probe
    std::vector<std::pair<size_t, size_t>> planes;  // (first partial, count) per plane
    int n_probes = 0;
    bool pending = false;
};

// A stack of independent scenes of equal nx x ny along z: scene i occupies planes z0[i] ..
// z0[i] + nz[i] - 1, and one separator plane of a frozen class (never changes from zero) lies
// between consecutive scenes.
struct StackLayout {
    std::vector<int> z0, nz;
    std::vector<int> nx, ny;  // per scene; below the grid's own nx, ny only in a ragged stack
    bool ragged = false;      // scenes of different cross-sections (each at x = y = 0, the rest frozen)
    std::vector<ClassTable> tabs;                    // per-scene class tables until they are merged
    std::vector<bool> has_tab;
    std::vector<std::vector<emlab_source>> sources;  // per-scene sources (scene coordinates)
    // per-scene conductivity / permittivity as uploaded (empty: vacuum); the grid's host copies
    // (cell_sigma, cell_eps: read-back only) are assembled from them on demand
    std::vector<std::vector<float>> sig, eps;
    bool cells_stale = true;
    bool dirty = false;                              // per-scene tables not merged yet
    int scenes() const { return (int)z0.size(); }
};

}  // namespace emlab

struct emlab_grid {
    template <typename T>
    using DevBuf = emlab::DevBuf<T>;
    int device = 0;
    cudaStream_t stream = nullptr;
    emlab_grid_config cfg{};
    bool configured = false;
    int pitch = 0;
    long long plane = 0;
    long long padded = 0;  // floats per component array
    DevBuf<float> fields;  // 12 component arrays: generation 0 (Ex..Bz), generation 1
    int cur = 0;
    int kernel = EMLAB_KERNEL_FUSED;
    int tile_rows = 0;  // 0: automatic
    // materials
    DevBuf<uint8_t> cls;
    bool wide = false;
    DevBuf<float4> tabE, tabM, tabW;
    uint32_t classes = 0, wire_start = 0;
    DevBuf<float> pml;
    int pml_stride = 0;
    DevBuf<uint8_t> pml_cls;
    DevBuf<float2> pml_coef;
    DevBuf<uint8_t> pml_z;  // per plane: inside the absorber along z
    int pml_K = 0;
    emlab::TmaMaps* tma = nullptr;
    DevBuf<unsigned> d_err;  // set by a solver kernel whose bounded on-device wait ran out
    DevBuf<unsigned long long> d_work;  // ticket counter of the persistent Yee kernel (never reset)
    unsigned long long work_base = 0;   // tickets consumed by the launches issued so far
    std::vector<float> cell_sigma, cell_eps;  // alpha channels of the textures (read-back only)
    // sources
    std::vector<emlab_source> desc;
    std::vector<float> packed;
    DevBuf<float4> d_src;
    DevBuf<int4> d_cells;
    DevBuf<int> d_lists;
    DevBuf<int> d_zoff;  // stacks: per source cell, the first plane of its scene
    DevBuf<int> d_cell_scene;  // ragged stacks: per source cell, its scene
    int nsrc = 0, ncells = 0;
    // stack of scenes (empty: a single scene)
    emlab::StackLayout stack;
    uint32_t stack_sep = 0;  // class of the separator planes
    // ragged stack: pair-kernel work items per tile height (4, 8, 16 rows), every scene's nx, ny,
    // and per-scene x / y absorber tables
    DevBuf<int4> d_items[3];
    int n_items[3] = {0, 0, 0};
    DevBuf<int2> d_scene_xy;
    DevBuf<uint8_t> d_pml_cls_xy;
    DevBuf<float> d_pml_xy;
    int pml_xy_stride = 0;
    bool launch_failed = false;  // set by a step whose solver launch was impossible (ragged stack)
    // per-chunk scalars: signals[k][nsrc], port rot[k], ntff rot[k], line rot[k], blends
    DevBuf<uint8_t> d_stage;
    uint8_t* h_stage[2] = {nullptr, nullptr};
    cudaEvent_t stage_done[2] = {nullptr, nullptr};
    size_t stage_bytes = 0;
    int stage_slot = 0;
    uint64_t step = 0;
    // ports
    int nports = 0;
    DevBuf<int4> d_ports;
    DevBuf<float> d_port_ph, d_series;
    size_t series_cap = 0, recorded = 0;
    // asynchronous takes of the recorded series: two pinned slots, each with its copy's event
    float* h_series[2] = {nullptr, nullptr};
    size_t h_series_cap[2] = {0, 0}, h_series_rows[2] = {0, 0};
    cudaEvent_t series_done[2] = {nullptr, nullptr};
    bool series_busy[2] = {false, false};
    int series_next = 0;
    bool recording = false;
    float port_wl = 16.0f, port_avg = 4.0f;
    // ntff
    bool ntff_on = false;
    int box[13] = {};
    int points = 0;
    DevBuf<int> d_box;
    DevBuf<float> d_ntff;
    float ntff_wl = 16.0f, ntff_avg = 4.0f;
    // lines
    int nq = 0;
    DevBuf<int4> d_q, d_terms;
    DevBuf<float> d_weights, d_line_ph, d_line_now;
    float line_wl = 16.0f, line_avg = 4.0f;
    // multi-frequency far-field DFT
    bool dft_on = false;
    // one or more Huygens boxes; box b is dft_boxes[kDftBoxInts * b + ...]: min xyz, max xyz, the
    // seven face offsets (box-local point indices), its first point in the concatenated point list,
    // its point count
    std::vector<int> dft_boxes;
    int dft_nbox = 0, dft_box_max = 0;  // boxes, the largest box's points
    int dft_block_cap = 0;              // samples per fold at most (0: the engine's own block)
    std::vector<float> dft_wl;          // wavelengths as configured (kept across stack compaction)
    int dft_points = 0, dft_nf = 0, dft_t = 0;
    long long dft_n0 = 0;
    uint64_t dft_samples = 0;
    std::vector<double> dft_omega;
    DevBuf<int> d_dft_box;
    DevBuf<float2> d_dft_w;
    DevBuf<double> d_dft_omega, d_dft_x;
    DevBuf<float> d_dft_blk;
    DevBuf<float> d_dft_bhi, d_dft_blo;  // tensor-core twiddles (split hi/lo, MMA operand layout)
    int dft_engine = EMLAB_DFT_TENSOR;
    // far-field spectra scratch (emlab_ntff_dft_spectra), grown on demand and kept
    DevBuf<float4> d_spec_dirs, d_spec_part;
    DevBuf<float> d_spec_out;
    // opt-in convolutional PML (cpml.cu): parameters, per-axis coefficient tables, slab psi arrays
    bool cpml_on = false;
    emlab_cpml cpml{};
    DevBuf<float4> cpml_coef;
    DevBuf<float> cpml_psi;
    int cpml_stride = 0;
    long long cpml_slab[3] = {0, 0, 0}, cpml_psi_off[3] = {0, 0, 0};
    // scratch
    DevBuf<unsigned> d_flag;
    // asynchronous FieldAnalyzer read-back: two measurements in flight, collected in order
    emlab::AnalyzerSlot analyzer[2];
    int analyzer_next = 0, analyzer_oldest = 0;
    // CUDA graphs of `graph_chunk` steps, one per (staging slot, field generation at the chunk start)
    int graph_chunk = 0;  // 0: launches are issued one by one
    bool graph_warm = false;
    cudaGraphExec_t graph_exec[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    unsigned long long graph_tickets = 0;  // work tickets the last solver launch of a chunk consumes
    uint64_t graph_launches = 0;           // kernel launches in one chunk graph
    // solver-pass timing: event pairs recorded around each Yee launch, read back lazily
    bool timing = false;
    std::vector<cudaEvent_t> ev_start, ev_stop;
    size_t ev_used = 0;
    double timed_ms = 0.0;
    uint64_t timed_launches = 0;

    float* comp(int gen, int c) { return fields.p + (size_t)(gen * 6 + c) * padded; }
    long long cells() const { return (long long)cfg.nx * cfg.ny * cfg.nz; }
};

namespace emlab {
// helpers of capi.cu used by stack.cu
int require_grid(const emlab_grid* g);
int upload_class_table(emlab_grid* g, const ClassTable& t);
int upload_pml(emlab_grid* g);
void refresh_tma(emlab_grid* g);
int clear_fields(emlab_grid* g);
int reset_monitors(emlab_grid* g);
// drops the captured step graphs (any change of a buffer, a monitor or a launch setting)
void invalidate_graphs(emlab_grid* g);
int upload_sources(emlab_grid* g, const std::vector<float>& packed, const std::vector<int32_t>& cells,
                   const std::vector<int32_t>& lists, const std::vector<int32_t>& zoff,
                   const std::vector<int32_t>& scene = {});
// stack.cu: merges per-scene materials uploaded since the last step
int stack_commit(emlab_grid* g);
// the host copies of a stack's per-cell materials, assembled from the scenes' own (no-op for a grid)
int ensure_cell_materials(emlab_grid* g);
// cpml.cu: tables and psi arrays for the configured size, psi reset, and the two in-place passes
int cpml_prepare(emlab_grid* g);
int cpml_clear(emlab_grid* g);
void launch_cpml(emlab_grid* g, const YeeArgs& a, bool wide, cudaStream_t s);
// capi.cu: the far-field DFT across a stack compaction. dft_carry_take folds the partial block and
// keeps the sums of the boxes that lie inside kept scenes (old scene idx[k] becomes scene k at
// new_z0[k]); dft_carry_restore re-attaches those boxes at their new planes with their sums.
struct DftCarry {
    bool on = false;
    std::vector<int> boxes;      // kept boxes, 6 ints each, in the new layout
    std::vector<int> old_first;  // their first point in the old point list
    std::vector<float> wl;
    int old_points = 0, block_cap = 0, engine = 0;
    uint64_t samples = 0;
    DevBuf<double> x;
};
int dft_carry_take(emlab_grid* g, const std::vector<int>& old_z0, const std::vector<int>& old_nz,
                   const std::vector<int>& idx, const std::vector<int>& new_z0, DftCarry& c);
int dft_carry_restore(emlab_grid* g, DftCarry& c);
// folds the samples of the far-field DFT's partial block into its sums (capi.cu)
int dft_fold_now(emlab_grid* g);
}  // namespace emlab
