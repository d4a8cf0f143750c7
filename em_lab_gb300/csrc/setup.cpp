// setup.cpp - host-side set-up arithmetic (see setup.h). Compiled with -ffp-contract=off so that
// the float expressions round exactly as written, like the shaders' and the kernels'.
#include "setup.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <utility>

#include "emlab_math.h"

namespace emlab {

void clamp_config(emlab_grid_config& c) {
    c.pml_thickness = std::clamp(c.pml_thickness, 0, 64);
    const int min_size = 2 * c.pml_thickness + 8;
    c.nx = std::max(c.nx, min_size);
    c.ny = std::max(c.ny, min_size);
    c.nz = std::max(c.nz, min_size);
    const float max_courant = 0.99f / 1.7320508f;  // strictly below 1/sqrt(3)
    c.courant = std::clamp(c.courant, 0.05f, max_courant);
    c.pml_sigma_max = std::max(c.pml_sigma_max, 0.0f);
    c.pml_grading = std::clamp(c.pml_grading, 0.25f, 12.0f);
}

namespace {

struct Key {
    uint16_t h[12];  // sig xyz, eps xyz, w0 xyz, w1 xyz (binary16 bit patterns)
    bool operator==(const Key& o) const { return std::memcmp(h, o.h, sizeof h) == 0; }
};
struct KeyHash {
    size_t operator()(const Key& k) const {
        uint64_t a, b, c;
        std::memcpy(&a, k.h, 8), std::memcpy(&b, k.h + 4, 8), std::memcpy(&c, k.h + 8, 8);
        uint64_t x = a * 0x9E3779B97F4A7C15ull ^ (b + 0x632BE59BD9B4E019ull) * 0xC2B2AE3D27D4EB4Full ^ c;
        x ^= x >> 29;
        return (size_t)(x * 0xBF58476D1CE4E5B9ull);
    }
};

constexpr uint16_t kHalfOne = 0x3c00;

}  // namespace

void class_coefficients(ClassTable& t, float dt) {
    for (uint32_t c = 0; c < t.classes; ++c) {
        const float* m = &t.tabM[c * 8];
        const float sig[3] = {m[0], m[1], m[2]}, eps[3] = {m[3], m[4], m[5]};
        float ca[3], cb[3];
        for (int a = 0; a < 3; ++a) {
            // update_E.comp:58-61 outside the absorber
            const float dtEps = dt / eps[a];
            const float x = sig[a] * dtEps;
            ca[a] = emlab_expf(-x);
            cb[a] = dtEps * emlab_phi(x);
        }
        float* e = &t.tabE[c * 8];
        e[0] = ca[0], e[1] = ca[1], e[2] = ca[2], e[3] = cb[0], e[4] = cb[1], e[5] = cb[2], e[6] = e[7] = 0.0f;
    }
}

bool build_classes(const float* sig, const float* eps, int nx, int ny, int nz, const emlab_edge_override* edges,
                   size_t n_edges, const emlab_wire_term* wires, size_t n_wires, float dt, ClassTable& out,
                   std::string& err) {
    const int64_t n = (int64_t)nx * ny * nz;
    const int pitch = row_pitch(nx);
    std::vector<uint16_t> halves;
    try {
        halves.resize((size_t)n * 6);
        out.cls.assign((size_t)pitch * ny * nz, 0u);
    } catch (const std::bad_alloc&) {
        err = "host allocation failed while building the edge materials";
        return false;
    }
    // Edge averaging (SimulationGrid.cpp:224-248): the four cells sharing each edge, clamped to the
    // edge cell at the low boundary; binary16 rounding after the 6e4 clamp (:256-262).
    auto I = [&](int x, int y, int z) {
        x = std::max(x, 0), y = std::max(y, 0), z = std::max(z, 0);
        return ((int64_t)z * ny + y) * nx + x;
    };
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const int64_t c00 = I(x, y, z);
                const int64_t sets[3][4] = {{c00, I(x, y - 1, z), I(x, y, z - 1), I(x, y - 1, z - 1)},
                                            {c00, I(x - 1, y, z), I(x, y, z - 1), I(x - 1, y, z - 1)},
                                            {c00, I(x - 1, y, z), I(x, y - 1, z), I(x - 1, y - 1, z)}};
                uint16_t* h = &halves[(size_t)c00 * 6];
                for (int a = 0; a < 3; ++a) {
                    const int64_t* c = sets[a];
                    const float s = 0.25f * (sig[c[0]] + sig[c[1]] + sig[c[2]] + sig[c[3]]);
                    const float e = 0.25f * (eps[c[0]] + eps[c[1]] + eps[c[2]] + eps[c[3]]);
                    h[a] = emlab_float_to_half(std::min(s, 6.0e4f));
                    h[3 + a] = emlab_float_to_half(e);
                }
            }
    // Sub-cell overrides replace the averaged conductivity; invalid ones are skipped (:250-254).
    for (size_t k = 0; k < n_edges; ++k) {
        const emlab_edge_override& o = edges[k];
        if (o.x < 0 || o.y < 0 || o.z < 0 || o.x >= nx || o.y >= ny || o.z >= nz || o.axis < 0 || o.axis > 2) continue;
        const int64_t i = ((int64_t)o.z * ny + o.y) * nx + o.x;
        halves[(size_t)i * 6 + o.axis] = emlab_float_to_half(std::min(std::max(o.sigma, 0.0f), 6.0e4f));
    }
    // Thin-wire factors (:279-291): sparse, later entries win.
    std::unordered_map<int64_t, std::array<float, 6>> wire;
    for (size_t k = 0; k < n_wires; ++k) {
        const emlab_wire_term& w = wires[k];
        if (w.x < 0 || w.y < 0 || w.z < 0 || w.x >= nx || w.y >= ny || w.z >= nz || w.component < 0 || w.component > 2)
            continue;
        const int64_t i = ((int64_t)w.z * ny + w.y) * nx + w.x;
        auto it = wire.find(i);
        if (it == wire.end()) it = wire.emplace(i, std::array<float, 6>{1, 1, 1, 1, 1, 1}).first;
        it->second[(w.term == 0 ? 0 : 3) + w.component] = w.factor;
    }

    std::unordered_map<Key, uint32_t, KeyHash> map;
    std::vector<Key> keys;
    auto lookup = [&](const Key& k) -> uint32_t {
        auto it = map.find(k);
        if (it != map.end()) return it->second;
        const uint32_t id = (uint32_t)keys.size();
        map.emplace(k, id);
        keys.push_back(k);
        return id;
    };
    // class 0 is vacuum so a cleared index array means "vacuum everywhere"
    Key vac;
    for (int a = 0; a < 3; ++a) vac.h[a] = 0, vac.h[3 + a] = kHalfOne, vac.h[6 + a] = vac.h[9 + a] = kHalfOne;
    lookup(vac);
    Key last = vac;
    uint32_t last_id = 0;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const int64_t i = ((int64_t)z * ny + y) * nx + x;
                Key k;
                std::memcpy(k.h, &halves[(size_t)i * 6], 12);
                for (int a = 6; a < 12; ++a) k.h[a] = kHalfOne;
                if (!wire.empty() && wire.count(i)) continue;  // wire classes are numbered after the others
                uint32_t id;
                if (k == last) {
                    id = last_id;
                } else {
                    id = lookup(k);
                    last = k, last_id = id;
                }
                out.cls[((size_t)z * ny + y) * pitch + x] = id;
            }
    out.wire_start = (uint32_t)keys.size();
    if (!wire.empty()) {
        std::unordered_map<Key, uint32_t, KeyHash> wmap;
        std::vector<std::pair<int64_t, std::array<float, 6>>> sorted(wire.begin(), wire.end());
        std::sort(sorted.begin(), sorted.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
        for (const auto& [i, f] : sorted) {
            Key k;
            std::memcpy(k.h, &halves[(size_t)i * 6], 12);
            for (int a = 0; a < 6; ++a) k.h[6 + a] = emlab_float_to_half(f[a]);
            auto it = wmap.find(k);
            uint32_t id;
            if (it != wmap.end()) {
                id = it->second;
            } else {
                id = (uint32_t)keys.size();
                wmap.emplace(k, id);
                keys.push_back(k);
            }
            const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((int64_t)nx * ny));
            out.cls[((size_t)z * ny + y) * pitch + x] = id;
        }
    }
    out.classes = (uint32_t)keys.size();
    out.tabE.assign((size_t)out.classes * 8, 0.0f);
    out.tabM.assign((size_t)out.classes * 8, 0.0f);
    out.tabW.assign((size_t)out.classes * 8, 0.0f);
    for (uint32_t c = 0; c < out.classes; ++c) {
        const Key& k = keys[c];
        float* m = &out.tabM[c * 8];
        float* w = &out.tabW[c * 8];
        for (int a = 0; a < 3; ++a) {
            // update_E.comp:48-49: sigma >= 0, eps >= 1 after unpacking
            m[a] = std::max(emlab_half_to_float(k.h[a]), 0.0f);
            m[3 + a] = std::max(emlab_half_to_float(k.h[3 + a]), 1.0f);
            w[a] = emlab_half_to_float(k.h[6 + a]);
            w[3 + a] = emlab_half_to_float(k.h[9 + a]);
        }
    }
    class_coefficients(out, dt);
    return true;
}

std::vector<float> pml_tables(const emlab_grid_config& c, int stride) {
    std::vector<float> t((size_t)6 * stride, 0.0f);
    const int n[3] = {c.nx, c.ny, c.nz};
    for (int a = 0; a < 3; ++a)
        for (int i = 0; i < n[a]; ++i) {
            const float pi = (float)i, ph = (float)i + 0.5f;
            t[(size_t)a * stride + i] = emlab_pml_profile(emlab_pml_depth(pi, n[a], c.pml_thickness), c.pml_thickness,
                                                          c.pml_sigma_max, c.pml_grading);
            t[(size_t)(3 + a) * stride + i] = emlab_pml_profile(emlab_pml_depth(ph, n[a], c.pml_thickness),
                                                                c.pml_thickness, c.pml_sigma_max, c.pml_grading);
        }
    return t;
}

void pml_class_tables(const emlab_grid_config& c, int stride, std::vector<uint8_t>& cls, std::vector<float>& coef,
                      int& K) {
    const int L = c.pml_thickness;
    K = 2 * L + 2;
    std::vector<float> V((size_t)K, 0.0f);
    for (int k = 1; k <= L; ++k) V[(size_t)k] = emlab_pml_profile((float)k, L, c.pml_sigma_max, c.pml_grading);
    for (int m = 0; m <= L; ++m)
        V[(size_t)(L + 1 + m)] = emlab_pml_profile((float)m + 0.5f, L, c.pml_sigma_max, c.pml_grading);
    cls.assign((size_t)6 * stride, 0);
    const int n[3] = {c.nx, c.ny, c.nz};
    for (int a = 0; a < 3; ++a)
        for (int i = 0; i < n[a]; ++i) {
            const float di = emlab_pml_depth((float)i, n[a], L);
            const float dh = emlab_pml_depth((float)i + 0.5f, n[a], L);
            // integer depths are whole numbers, half-integer depths are m + 0.5 (both at most L + 0.5)
            cls[(size_t)a * stride + i] = (uint8_t)(di <= 0.0f ? 0 : (int)di);
            cls[(size_t)(3 + a) * stride + i] = (uint8_t)(dh <= 0.0f ? 0 : L + 1 + (int)(dh - 0.5f));
        }
    const float dt = c.courant;
    coef.assign((size_t)K * K * K * 2, 0.0f);
    for (int i = 0; i < K; ++i)
        for (int j = 0; j < K; ++j)
            for (int k = 0; k < K; ++k) {
                const float sigma = (V[(size_t)i] + V[(size_t)j]) + V[(size_t)k];
                const float x = sigma * dt;
                float* e = &coef[(((size_t)i * K + j) * K + k) * 2];
                e[0] = emlab_expf(-x);
                e[1] = dt * emlab_phi(x);
            }
}

int pack_sources(const emlab_source* s, size_t n, std::vector<emlab_source>& desc, std::vector<float>& packed) {
    desc.clear();
    packed.clear();
    for (size_t i = 0; i < n && desc.size() < 256; ++i) {
        const float* p = s[i].polarization;
        const float len = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);  // glm::length
        if (!s[i].enabled || !(len > 1e-6f) || !std::isfinite(len)) continue;
        float g[16];
        for (int a = 0; a < 3; ++a) {
            g[a] = s[i].center[a];
            g[4 + a] = std::clamp(s[i].half_extent[a], 0.0f, 1.0e5f);
            g[8 + a] = p[a] / len;
            g[12 + a] = std::max(s[i].softness[a], 0.25f);
        }
        g[3] = g[7] = g[15] = 0.0f;
        g[11] = s[i].amplitude;
        packed.insert(packed.end(), g, g + 16);
        desc.push_back(s[i]);
    }
    return (int)desc.size();
}

void source_lists(const std::vector<float>& packed, int nsrc, const int n[3], std::vector<int32_t>& cells,
                  std::vector<int32_t>& lists) {
    std::vector<std::pair<uint32_t, uint32_t>> pairs;
    for (int i = 0; i < nsrc; ++i) {
        const float* g = &packed[(size_t)i * 16];
        int lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
            const float c = g[a], h = g[4 + a], w = g[12 + a];
            lo[a] = std::clamp((int)std::floor(c - h - 3.5f * w) - 1, 0, n[a] - 1);
            hi[a] = std::clamp((int)std::ceil(c + h + 3.5f * w), 0, n[a] - 1);
        }
        for (int z = lo[2]; z <= hi[2]; ++z)
            for (int y = lo[1]; y <= hi[1]; ++y)
                for (int x = lo[0]; x <= hi[0]; ++x)
                    pairs.emplace_back((uint32_t)((z * n[1] + y) * n[0] + x), (uint32_t)i);
    }
    std::sort(pairs.begin(), pairs.end());
    cells.clear();
    lists.clear();
    for (size_t k = 0; k < pairs.size(); ++k) {
        if (k == 0 || pairs[k].first != pairs[k - 1].first) {
            const uint32_t idx = pairs[k].first;
            cells.push_back((int32_t)(idx % (uint32_t)n[0]));
            cells.push_back((int32_t)((idx / (uint32_t)n[0]) % (uint32_t)n[1]));
            cells.push_back((int32_t)(idx / (uint32_t)(n[0] * n[1])));
            cells.push_back((int32_t)lists.size());
        }
        lists.push_back((int32_t)pairs[k].second);
    }
    const int32_t end = (int32_t)lists.size();
    cells.insert(cells.end(), {0, 0, 0, end});  // sentinel: end of the last list
    if (lists.empty()) lists.push_back(0);
}

double source_signal(const emlab_source& s, double tAbs) {
    const double wl = std::max((double)s.wavelength, 1e-3);
    const double t = tAbs - std::max((double)s.delay_periods, 0.0) * wl;
    if (!s.enabled || t < 0.0) return 0.0;
    const double period = wl;
    const double w = 6.28318530717958647692 / wl;
    if (s.waveform == EMLAB_WAVE_CW) {
        const double rampT = std::max((double)s.ramp_periods, 0.0) * period;
        double ramp = 1.0;
        if (rampT > 0.0 && t < rampT) {
            const double r = t / rampT;
            ramp = r * r * r * (10.0 + r * (-15.0 + 6.0 * r));  // C2 smootherstep
        }
        return ramp * std::sin(w * t + (double)s.phase);
    }
    const double tau = std::max((double)s.ramp_periods, 0.1) * period;
    const double t0 = 3.0 * tau;
    double tl = t;
    if (s.repeat_periods > 0.0f) {
        const double rep = std::max((double)s.repeat_periods * period, 2.0 * t0);
        tl = std::fmod(t, rep);
    }
    const double u = (tl - t0) / tau;
    if (std::abs(u) > 6.0) return 0.0;
    return std::exp(-u * u) * std::sin(w * (tl - t0) + (double)s.phase);
}

}  // namespace emlab
