// stack.cu - stacks of independent scenes stepped as one grid (batched scene sweeps).
//
// Many small scenes (an antenna-length or material sweep) each fill only a few SMs and pay the
// launch overhead of every pass on their own. Here scenes of equal nx x ny are laid out one after
// another along z in a single grid, with one separator plane between consecutive scenes, and the
// ordinary solver passes (the persistent TMA Yee kernel, sources, ports) step all of them in one
// launch each. Nothing couples the scenes:
//  * every scene keeps its own absorber: the z entries of the absorber tables and the per-plane
//    absorber flag are the scene's own (capi.cu upload_pml);
//  * every scene keeps its own edge materials: the class table of each scene is built from that
//    scene alone (edge averaging clamps at its own faces, src/SimulationGrid.cpp:224-248) and the
//    tables are merged, identical classes shared;
//  * the separator plane holds a frozen class: its thin-wire factors are 0, so its B stays 0 (the
//    reference's "B below the lower face is 0"), and its permittivity is infinite, so its E stays 0
//    in and outside the absorber (dt / eps = 0: ca = 1, cb = 0; "E beyond the upper face is 0");
//  * source footprints are evaluated in scene coordinates (SourceArgs::zoff), so the float
//    arithmetic of apply_sources.comp:37-40 is that of the scene on its own grid.
// A scene of the stack therefore evolves bit for bit as it does alone. Scenes that have finished
// (e.g. rung down) are dropped by compaction, which copies the remaining scenes' fields and class
// indices into a shorter stack on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <vector>

#include "../../include/emlab.h"
#include "grid_state.h"

using namespace emlab;

namespace {

// The class every cell of a scene without uploaded materials has (SimulationGrid.cpp:185-192).
ClassTable vacuum_table(float dt) {
    ClassTable t;
    t.classes = 1, t.wire_start = 1;
    t.tabM = {0, 0, 0, 1, 1, 1, 0, 0};
    t.tabW = {1, 1, 1, 1, 1, 1, 0, 0};
    t.tabE.assign(8, 0.0f);
    class_coefficients(t, dt);
    return t;
}

using ClassKey = std::array<uint32_t, 24>;

ClassKey key_of(const ClassTable& t, uint32_t c) {
    ClassKey k;
    std::memcpy(k.data(), &t.tabE[(size_t)c * 8], 32);
    std::memcpy(k.data() + 8, &t.tabM[(size_t)c * 8], 32);
    std::memcpy(k.data() + 16, &t.tabW[(size_t)c * 8], 32);
    return k;
}

// c.nx, c.ny: the grid's cross-section (the largest scene's in a ragged stack); nx, ny: every
// scene's own (equal to c's in a uniform stack).
int configure_layout(emlab_grid* g, const emlab_grid_config& c, const std::vector<int>& nz, const std::vector<int>& nx,
                     const std::vector<int>& ny) {
    const int n = (int)nz.size();
    emlab_grid_config t = c;
    long long total = n - 1;
    for (int v : nz) total += v;
    if (total > (1 << 30)) return fail(EMLAB_ERR_INVALID, "stack too deep");
    t.nz = (int)total;
    const int pitch = row_pitch(t.nx);
    const long long plane = (long long)pitch * t.ny;
    const long long padded = plane * t.nz;
    g->cpml_on = false;  // a stack always uses the reference absorber
    g->cpml_psi.release(), g->cpml_coef.release();
    g->fields.release();
    g->cls.release();
    if (g->fields.alloc((size_t)padded * 12) != cudaSuccess) {
        g->configured = false;
        return fail(EMLAB_ERR_OOM, "stack: field allocation failed (too large for device memory)");
    }
    g->cfg = t;
    g->pitch = pitch, g->plane = plane, g->padded = padded;
    StackLayout s;
    s.nz = nz;
    s.nx = nx, s.ny = ny;
    for (int i = 0; i < n; ++i) s.ragged = s.ragged || nx[(size_t)i] != t.nx || ny[(size_t)i] != t.ny;
    if (s.ragged) {
        g->kernel = EMLAB_KERNEL_FUSED;  // the pair kernel reads each item's scene; the others do not
        if (g->tile_rows != 0 && g->tile_rows != 32 && g->tile_rows != 64 && g->tile_rows != 128) g->tile_rows = 0;
    }
    s.z0.resize((size_t)n);
    int z = 0;
    for (int i = 0; i < n; ++i) s.z0[(size_t)i] = z, z += nz[(size_t)i] + 1;
    s.tabs.resize((size_t)n);
    s.has_tab.assign((size_t)n, false);
    s.sources.resize((size_t)n);
    s.sig.resize((size_t)n), s.eps.resize((size_t)n);
    s.dirty = true;
    g->stack = std::move(s);
    return upload_pml(g);
}

// Merges the per-scene class tables into one (vacuum first, then every scene's ordinary classes,
// then the thin-wire classes, then the separator) and uploads the stack's class index.
int commit(emlab_grid* g) {
    StackLayout& s = g->stack;
    const float dt = g->cfg.courant;
    const ClassTable vac = vacuum_table(dt);
    std::map<ClassKey, uint32_t> plain, wired;
    std::vector<ClassKey> plain_keys, wired_keys;
    auto add = [](std::map<ClassKey, uint32_t>& m, std::vector<ClassKey>& keys, const ClassKey& k) {
        auto it = m.find(k);
        if (it != m.end()) return it->second;
        const uint32_t id = (uint32_t)keys.size();
        m.emplace(k, id);
        keys.push_back(k);
        return id;
    };
    add(plain, plain_keys, key_of(vac, 0));
    const int n = s.scenes();
    std::vector<std::vector<uint32_t>> remap((size_t)n);  // scene class -> provisional id (wire: | 1 << 31)
    for (int i = 0; i < n; ++i) {
        if (!s.has_tab[(size_t)i]) continue;
        const ClassTable& t = s.tabs[(size_t)i];
        remap[(size_t)i].resize(t.classes);
        for (uint32_t c = 0; c < t.classes; ++c)
            remap[(size_t)i][c] = c < t.wire_start ? add(plain, plain_keys, key_of(t, c))
                                                   : (add(wired, wired_keys, key_of(t, c)) | 0x80000000u);
    }
    const uint32_t wire_start = (uint32_t)plain_keys.size();
    const uint32_t sep = wire_start + (uint32_t)wired_keys.size();
    ClassTable m;
    m.classes = sep + 1;
    m.wire_start = wire_start;
    m.tabE.resize((size_t)m.classes * 8), m.tabM.resize((size_t)m.classes * 8), m.tabW.resize((size_t)m.classes * 8);
    auto put = [&](uint32_t id, const ClassKey& k) {
        std::memcpy(&m.tabE[(size_t)id * 8], k.data(), 32);
        std::memcpy(&m.tabM[(size_t)id * 8], k.data() + 8, 32);
        std::memcpy(&m.tabW[(size_t)id * 8], k.data() + 16, 32);
    };
    for (uint32_t i = 0; i < wire_start; ++i) put(i, plain_keys[i]);
    for (uint32_t i = 0; i < (uint32_t)wired_keys.size(); ++i) put(wire_start + i, wired_keys[i]);
    // separator: ca = 1, cb = 0; sigma 0, eps = +inf; thin-wire factors 0
    const float inf = std::numeric_limits<float>::infinity();
    const float e_sep[8] = {1, 1, 1, 0, 0, 0, 0, 0}, m_sep[8] = {0, 0, 0, inf, inf, inf, 0, 0};
    std::memcpy(&m.tabE[(size_t)sep * 8], e_sep, 32);
    std::memcpy(&m.tabM[(size_t)sep * 8], m_sep, 32);
    std::fill(m.tabW.begin() + (size_t)sep * 8, m.tabW.begin() + (size_t)sep * 8 + 8, 0.0f);
    try {
        m.cls.assign((size_t)g->padded, sep);
    } catch (const std::bad_alloc&) {
        return fail(EMLAB_ERR_OOM, "host allocation failed while merging the scene classes");
    }
    const size_t plane = (size_t)g->plane, pitch = (size_t)g->pitch;
    for (int i = 0; i < n; ++i) {
        // the scene's cells (x < its nx, y < its ny); the rest of its planes keeps the frozen class
        uint32_t* dst = m.cls.data() + (size_t)s.z0[(size_t)i] * plane;
        const int sx = s.nx[(size_t)i], sy = s.ny[(size_t)i], sz = s.nz[(size_t)i];
        const size_t spitch = (size_t)row_pitch(sx);
        const std::vector<uint32_t>* r = s.has_tab[(size_t)i] ? &remap[(size_t)i] : nullptr;
        const uint32_t* src = r ? s.tabs[(size_t)i].cls.data() : nullptr;
#pragma omp parallel for schedule(static)
        for (long long row = 0; row < (long long)sz * sy; ++row) {
            const size_t z = (size_t)row / sy, y = (size_t)row % sy;
            uint32_t* d = dst + z * plane + y * pitch;
            if (!r) {
                std::fill(d, d + sx, 0u);
                continue;
            }
            const uint32_t* q = src + (z * sy + y) * spitch;
            for (int x = 0; x < sx; ++x) {
                const uint32_t v = (*r)[q[x]];
                d[x] = v & 0x80000000u ? wire_start + (v & 0x7fffffffu) : v;
            }
        }
        if (r) {
            s.tabs[(size_t)i] = ClassTable();  // merged: the per-scene copy is no longer needed
            s.has_tab[(size_t)i] = false;
        }
    }
    if (int rc = upload_class_table(g, m)) return rc;
    g->stack_sep = sep;
    refresh_tma(g);
    s.dirty = false;
    return EMLAB_OK;
}

// Packs every scene's sources (setSources per scene) and merges the per-cell lists with the
// scenes' plane offsets.
int merge_sources(emlab_grid* g) {
    StackLayout& s = g->stack;
    std::vector<emlab_source> all_desc;
    std::vector<float> all_packed;
    std::vector<int32_t> cells, lists, zoff, scene;
    for (int i = 0; i < s.scenes(); ++i) {
        const std::vector<emlab_source>& in = s.sources[(size_t)i];
        if (in.empty()) continue;
        std::vector<emlab_source> desc;
        std::vector<float> packed;
        const int ns = pack_sources(in.data(), in.size(), desc, packed);
        std::vector<int32_t> c, l;
        const int dims[3] = {s.nx[(size_t)i], s.ny[(size_t)i], s.nz[(size_t)i]};
        source_lists(packed, ns, dims, c, l);
        const int32_t src0 = (int32_t)all_desc.size(), list0 = (int32_t)lists.size();
        const size_t nc = c.size() / 4 - 1;
        for (size_t k = 0; k < nc; ++k) {
            cells.insert(cells.end(), {c[4 * k], c[4 * k + 1], c[4 * k + 2], c[4 * k + 3] + list0});
            zoff.push_back(s.z0[(size_t)i]);
            scene.push_back(i);
        }
        const int32_t used = c[4 * nc + 3];  // the sentinel: list entries of this scene
        for (int32_t k = 0; k < used; ++k) lists.push_back(l[(size_t)k] + src0);
        all_desc.insert(all_desc.end(), desc.begin(), desc.begin() + ns);
        all_packed.insert(all_packed.end(), packed.begin(), packed.begin() + (size_t)ns * 16);
    }
    cells.insert(cells.end(), {0, 0, 0, (int32_t)lists.size()});
    if (lists.empty()) lists.push_back(0);
    if (zoff.empty()) zoff.push_back(0);
    if (scene.empty()) scene.push_back(0);
    g->nsrc = (int)all_desc.size();
    g->desc = all_desc;
    g->packed = all_packed;
    return upload_sources(g, all_packed, cells, lists, zoff, s.ragged ? scene : std::vector<int32_t>());
}

}  // namespace

int emlab::stack_commit(emlab_grid* g) { return g->stack.dirty ? commit(g) : EMLAB_OK; }

int emlab::ensure_cell_materials(emlab_grid* g) {
    StackLayout& s = g->stack;
    const size_t cells = (size_t)g->cells();
    if (s.scenes() == 0 || (!s.cells_stale && g->cell_sigma.size() == cells)) return EMLAB_OK;
    try {
        g->cell_sigma.assign(cells, 0.0f);
        g->cell_eps.assign(cells, 1.0f);
    } catch (const std::bad_alloc&) {
        return fail(EMLAB_ERR_OOM, "host allocation failed");
    }
    const size_t gx = (size_t)g->cfg.nx, gy = (size_t)g->cfg.ny;
    for (int i = 0; i < s.scenes(); ++i) {
        const std::vector<float>& sg = s.sig[(size_t)i];
        const std::vector<float>& ep = s.eps[(size_t)i];
        if (sg.empty()) continue;  // vacuum
        const size_t nx = (size_t)s.nx[(size_t)i], ny = (size_t)s.ny[(size_t)i], nz = (size_t)s.nz[(size_t)i];
        for (size_t z = 0; z < nz; ++z)
            for (size_t y = 0; y < ny; ++y) {
                const size_t d = (((size_t)s.z0[(size_t)i] + z) * gy + y) * gx, q = (z * ny + y) * nx;
                std::memcpy(g->cell_sigma.data() + d, sg.data() + q, nx * 4);
                std::memcpy(g->cell_eps.data() + d, ep.data() + q, nx * 4);
            }
    }
    s.cells_stale = false;
    return EMLAB_OK;
}

extern "C" {

namespace {
int configure_scenes(emlab_grid* g, const emlab_grid_config* req, const int* dims, int n_scenes) {
    EMLAB_REQUIRE(n_scenes >= 1, "a stack needs at least one scene");
    EMLAB_CUDA(cudaSetDevice(g->device));
    EMLAB_CUDA(cudaStreamSynchronize(g->stream));
    emlab_grid_config c = *req;
    std::vector<int> nx((size_t)n_scenes), ny((size_t)n_scenes), nz((size_t)n_scenes);
    int mx = 0, my = 0;
    for (int i = 0; i < n_scenes; ++i) {  // each scene is clamped as SimulationGrid::configure clamps it
        emlab_grid_config ci = *req;
        ci.nx = dims[3 * i], ci.ny = dims[3 * i + 1], ci.nz = dims[3 * i + 2];
        clamp_config(ci);
        nx[(size_t)i] = ci.nx, ny[(size_t)i] = ci.ny, nz[(size_t)i] = ci.nz;
        mx = std::max(mx, ci.nx), my = std::max(my, ci.ny);
        c = ci;
    }
    EMLAB_REQUIRE(mx < 65536 && my < 65536, "stack cross-section too large");
    c.nx = mx, c.ny = my;
    if (int rc = configure_layout(g, c, nz, nx, ny)) return rc;
    g->cell_sigma.clear(), g->cell_eps.clear();  // assembled from the scenes' materials when read back
    if (int rc = commit(g)) return rc;
    if (int rc = clear_fields(g)) return rc;
    g->step = 0;
    g->configured = true;
    if (int rc = merge_sources(g)) return rc;
    if (int rc = reset_monitors(g)) return rc;
    EMLAB_CUDA(cudaStreamSynchronize(g->stream));
    return EMLAB_OK;
}
}  // namespace

int emlab_stack_configure(emlab_grid* g, const emlab_grid_config* req, const int* scene_nz, int n_scenes) {
    if (!g || !req || !scene_nz) return fail(EMLAB_ERR_INVALID, "null argument");
    std::vector<int> dims;
    for (int i = 0; i < n_scenes; ++i) dims.insert(dims.end(), {req->nx, req->ny, scene_nz[i]});
    return configure_scenes(g, req, dims.data(), n_scenes);
}

int emlab_stack_configure_scenes(emlab_grid* g, const emlab_grid_config* req, const int* dims, int n_scenes) {
    if (!g || !req || !dims) return fail(EMLAB_ERR_INVALID, "null argument");
    return configure_scenes(g, req, dims, n_scenes);
}

int emlab_stack_scene_dims(const emlab_grid* g, int* dims) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(dims, "null argument");
    const StackLayout& s = g->stack;
    for (int i = 0; i < s.scenes(); ++i)
        dims[3 * i] = s.nx[(size_t)i], dims[3 * i + 1] = s.ny[(size_t)i], dims[3 * i + 2] = s.nz[(size_t)i];
    return EMLAB_OK;
}

int emlab_stack_info(const emlab_grid* g, int* n_scenes, int* z0, int* nz) {
    if (int rc = require_grid(g)) return rc;
    const int n = g->stack.scenes();
    if (n_scenes) *n_scenes = n;
    for (int i = 0; i < n; ++i) {
        if (z0) z0[i] = g->stack.z0[(size_t)i];
        if (nz) nz[i] = g->stack.nz[(size_t)i];
    }
    return EMLAB_OK;
}

int emlab_stack_upload_materials(emlab_grid* g, int scene, const float* sigma, const float* eps_r, int nx, int ny,
                                 int nz, const emlab_edge_override* edges, size_t n_edges,
                                 const emlab_wire_term* wires, size_t n_wires) {
    if (int rc = require_grid(g)) return rc;
    StackLayout& s = g->stack;
    EMLAB_REQUIRE(scene >= 0 && scene < s.scenes(), "no such scene in the stack");
    if (nx != s.nx[(size_t)scene] || ny != s.ny[(size_t)scene] || nz != s.nz[(size_t)scene])
        return fail(EMLAB_ERR_INVALID, "SimulationGrid: material volume size does not match the grid");
    EMLAB_REQUIRE(sigma && eps_r, "null material array");
    EMLAB_REQUIRE((edges || n_edges == 0) && (wires || n_wires == 0), "null override array");
    std::string err;
    ClassTable t;
    if (!build_classes(sigma, eps_r, nx, ny, nz, edges, n_edges, wires, n_wires, g->cfg.courant, t, err))
        return fail(EMLAB_ERR_OOM, err);
    s.tabs[(size_t)scene] = std::move(t);
    s.has_tab[(size_t)scene] = true;
    s.dirty = true;
    // the scene's own copies (read-back only)
    const size_t count = (size_t)nx * ny * nz;
    s.sig[(size_t)scene].assign(sigma, sigma + count);
    s.eps[(size_t)scene].assign(eps_r, eps_r + count);
    s.cells_stale = true;
    EMLAB_CUDA(cudaSetDevice(g->device));
    if (int rc = clear_fields(g)) return rc;  // uploadMaterials starts the scenes over
    g->step = 0;
    EMLAB_CUDA(cudaStreamSynchronize(g->stream));
    return EMLAB_OK;
}

int emlab_stack_commit(emlab_grid* g) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_CUDA(cudaSetDevice(g->device));
    EMLAB_CUDA(cudaStreamSynchronize(g->stream));
    return stack_commit(g);
}

int emlab_stack_set_sources(emlab_grid* g, const emlab_source* sources, const int* scene_of, size_t n) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE((sources && scene_of) || n == 0, "null source array");
    StackLayout& s = g->stack;
    EMLAB_REQUIRE(s.scenes() > 0, "not a stack of scenes");
    for (size_t k = 0; k < n; ++k) EMLAB_REQUIRE(scene_of[k] >= 0 && scene_of[k] < s.scenes(), "no such scene");
    for (auto& v : s.sources) v.clear();
    for (size_t k = 0; k < n; ++k) s.sources[(size_t)scene_of[k]].push_back(sources[k]);
    EMLAB_CUDA(cudaSetDevice(g->device));
    return merge_sources(g);
}

int emlab_stack_compact(emlab_grid* g, const unsigned char* keep) {
    if (int rc = require_grid(g)) return rc;
    EMLAB_REQUIRE(keep, "null keep array");
    StackLayout& s = g->stack;
    const int n = s.scenes();
    EMLAB_REQUIRE(n > 0, "not a stack of scenes");
    EMLAB_REQUIRE(!g->series_busy[0] && !g->series_busy[1], "collect the pending series takes before compacting");
    EMLAB_CUDA(cudaSetDevice(g->device));
    EMLAB_CUDA(cudaStreamSynchronize(g->stream));
    if (int rc = stack_commit(g)) return rc;
    std::vector<int> idx;
    for (int i = 0; i < n; ++i)
        if (keep[i]) idx.push_back(i);
    EMLAB_REQUIRE(!idx.empty(), "a stack keeps at least one scene");
    if ((int)idx.size() == n) return EMLAB_OK;
    // new layout; the old device arrays stay alive until the copies are done
    DevBuf<float> old_fields;
    DevBuf<uint8_t> old_cls;
    std::swap(old_fields.p, g->fields.p), std::swap(old_fields.n, g->fields.n);
    std::swap(old_cls.p, g->cls.p), std::swap(old_cls.n, g->cls.n);
    const std::vector<int> old_z0 = s.z0, old_nz = s.nz;
    const long long old_padded = g->padded;
    const int old_cur = g->cur;
    std::vector<int> nz, nxk, nyk;
    std::vector<std::vector<emlab_source>> src;
    std::vector<std::vector<float>> sigk, epsk;
    for (int i : idx) {
        nz.push_back(s.nz[(size_t)i]), nxk.push_back(s.nx[(size_t)i]), nyk.push_back(s.ny[(size_t)i]);
        src.push_back(s.sources[(size_t)i]);
        sigk.push_back(std::move(s.sig[(size_t)i])), epsk.push_back(std::move(s.eps[(size_t)i]));
    }
    const emlab_grid_config c = g->cfg;
    if (int rc = configure_layout(g, c, nz, nxk, nyk)) return rc;
    s.sources = src;
    s.sig = std::move(sigk), s.eps = std::move(epsk);
    g->cell_sigma.clear(), g->cell_eps.clear();
    s.dirty = false;
    const size_t plane = (size_t)g->plane, esize = g->wide ? 4 : 2;
    EMLAB_CUDA(cudaMemsetAsync(g->fields.p, 0, g->fields.n * 4, g->stream));
    EMLAB_CUDA(g->cls.alloc((size_t)g->padded * esize));
    {  // separator planes: the frozen class
        std::vector<uint8_t> sep_plane(plane * esize);
        for (size_t j = 0; j < plane; ++j) {
            if (esize == 4) std::memcpy(&sep_plane[j * 4], &g->stack_sep, 4);
            else {
                const uint16_t v = (uint16_t)g->stack_sep;
                std::memcpy(&sep_plane[j * 2], &v, 2);
            }
        }
        for (size_t k = 0; k + 1 < idx.size(); ++k) {
            const size_t z = (size_t)s.z0[k] + (size_t)s.nz[k];
            EMLAB_CUDA(cudaMemcpyAsync(g->cls.p + z * plane * esize, sep_plane.data(), plane * esize, cudaMemcpyHostToDevice, g->stream));
        }
    }
    for (size_t k = 0; k < idx.size(); ++k) {
        const size_t zo = (size_t)old_z0[(size_t)idx[k]], zn = (size_t)s.z0[k], depth = (size_t)s.nz[k];
        for (int comp = 0; comp < 6; ++comp) {
            const float* from = old_fields.p + (size_t)(old_cur * 6 + comp) * old_padded + zo * plane;
            EMLAB_CUDA(cudaMemcpyAsync(g->comp(0, comp) + zn * plane, from, depth * plane * 4,
                                       cudaMemcpyDeviceToDevice, g->stream));
        }
        EMLAB_CUDA(cudaMemcpyAsync(g->cls.p + zn * plane * esize, old_cls.p + zo * plane * esize,
                                   depth * plane * esize, cudaMemcpyDeviceToDevice, g->stream));
    }
    g->cur = 0;
    refresh_tma(g);
    EMLAB_CUDA(cudaStreamSynchronize(g->stream));
    if (int rc = merge_sources(g)) return rc;
    // far-field DFT boxes inside kept scenes carry their sums over; the other monitors are reset
    // and the caller re-attaches its ports at the new planes
    DftCarry carry;
    if (int rc = dft_carry_take(g, old_z0, old_nz, idx, s.z0, carry)) return rc;
    if (int rc = reset_monitors(g)) return rc;
    if (int rc = dft_carry_restore(g, carry)) return rc;
    EMLAB_CUDA(cudaStreamSynchronize(g->stream));
    return EMLAB_OK;
}

}  // extern "C"
