// emlab_simulation_grid.hpp - header-only C++ facade with the interface of the reference's
// SimulationGrid (src/SimulationGrid.hpp:155-216) over the C ABI of include/emlab.h.
//
// A maintainer swaps the GL solver for this class: the member names, argument meaning and error
// behaviour are the reference's (std::runtime_error where SimulationGrid throws, silent skipping
// of invalid sub-cell overrides, at most 256 sources). GL texture names are replaced by device
// component pointers that co-resident monitors read; the monitors themselves attach through the
// emlab_ports_*, emlab_ntff_*, emlab_lines_* entry points and run inside step() on the device.
#pragma once

#include <algorithm>
#include <array>
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "emlab.h"

namespace emlab_cpp {

struct ivec3 {
    int x = 0, y = 0, z = 0;
};
struct vec3 {
    float x = 0, y = 0, z = 0;
};

// GridConfig (src/SimulationGrid.hpp:25-31)
struct GridConfig {
    ivec3 size{128, 128, 128};
    float courant = 0.5f;
    int pmlThickness = 16;
    float pmlSigmaMax = 1.6f;
    float pmlGrading = 3.0f;
};

// MaterialVolume (src/SimulationGrid.hpp:46-69)
class MaterialVolume {
public:
    MaterialVolume() = default;
    explicit MaterialVolume(const ivec3& size) : m_size{std::max(size.x, 0), std::max(size.y, 0), std::max(size.z, 0)} {
        const size_t n = (size_t)m_size.x * m_size.y * m_size.z;
        m_sigma.assign(n, 0.0f);
        m_epsR.assign(n, 1.0f);
    }
    const ivec3& size() const noexcept { return m_size; }
    bool contains(const ivec3& p) const noexcept {
        return p.x >= 0 && p.y >= 0 && p.z >= 0 && p.x < m_size.x && p.y < m_size.y && p.z < m_size.z;
    }
    size_t index(const ivec3& p) const noexcept { return ((size_t)p.z * m_size.y + p.y) * m_size.x + p.x; }
    void set(const ivec3& p, float sigma, float epsR) {
        if (!contains(p)) return;
        m_sigma[index(p)] = std::max(sigma, 0.0f);
        m_epsR[index(p)] = std::max(epsR, 1.0f);
    }
    const std::vector<float>& sigma() const noexcept { return m_sigma; }
    const std::vector<float>& epsilonR() const noexcept { return m_epsR; }

private:
    ivec3 m_size{};
    std::vector<float> m_sigma, m_epsR;
};

// SubcellModel (src/SimulationGrid.hpp:96-101)
struct SubcellModel {
    std::vector<emlab_edge_override> edges;
    std::vector<emlab_wire_term> wireTerms;
};

class SimulationGrid {
public:
    static constexpr int kMaxSources = 256;

    SimulationGrid() { check(emlab_grid_create(&m_g)); }
    ~SimulationGrid() { emlab_grid_destroy(m_g); }
    SimulationGrid(const SimulationGrid&) = delete;
    SimulationGrid& operator=(const SimulationGrid&) = delete;

    void configure(const GridConfig& c) {
        emlab_grid_config cfg{c.size.x, c.size.y, c.size.z, c.courant, c.pmlThickness, c.pmlSigmaMax, c.pmlGrading};
        check(emlab_grid_configure(m_g, &cfg));
        emlab_grid_config out{};
        check(emlab_grid_get_config(m_g, &out));
        m_config = GridConfig{{out.nx, out.ny, out.nz}, out.courant, out.pml_thickness, out.pml_sigma_max, out.pml_grading};
    }
    void uploadMaterials(const MaterialVolume& m, const SubcellModel& subcell = {}) {
        if (m.size().x != m_config.size.x || m.size().y != m_config.size.y || m.size().z != m_config.size.z)
            throw std::runtime_error("SimulationGrid: material volume size does not match the grid");
        check(emlab_grid_upload_materials(m_g, m.sigma().data(), m.epsilonR().data(), m.size().x, m.size().y,
                                          m.size().z, subcell.edges.data(), subcell.edges.size(),
                                          subcell.wireTerms.data(), subcell.wireTerms.size()));
    }
    void setSources(const std::vector<emlab_source>& sources) {
        check(emlab_grid_set_sources(m_g, sources.data(), sources.size()));
        m_sources = sources;
    }
    const std::vector<emlab_source>& sources() const noexcept { return m_sources; }
    void resetFields() { check(emlab_grid_reset_fields(m_g)); }
    // afterEachStep runs on the host after every completed step (monitors attached through the
    // C ABI already run on the device inside the step, so the callback is usually empty).
    void step(int count, const std::function<void()>& afterEachStep = {}) {
        if (count <= 0) return;
        if (!afterEachStep) {
            check(emlab_grid_step(m_g, count));
            return;
        }
        for (int k = 0; k < count; ++k) {
            check(emlab_grid_step(m_g, 1));
            afterEachStep();
        }
    }
    void synchronize(int timeoutMs = 0) { check(emlab_grid_synchronize(m_g, timeoutMs)); }
    const GridConfig& config() const noexcept { return m_config; }
    const ivec3& size() const noexcept { return m_config.size; }
    float dt() const noexcept { return m_config.courant; }
    double time() const { return state().time; }
    std::uint64_t stepCount() const { return state().step_count; }
    size_t gpuMemoryBytes() const { return (size_t)state().device_bytes; }
    emlab_grid* handle() const noexcept { return m_g; }
    // In place of eFieldTexture() / bFieldTexture(): device arrays Ex, Ey, Ez, Bx, By, Bz of the
    // current generation, cell (x, y, z) at [z * plane + y * pitch + x]; valid until the next step.
    struct FieldView {
        float* component[6];
        int pitch;
        long long plane;
    };
    FieldView fieldView() const {
        FieldView v{};
        check(emlab_grid_field_ptr(m_g, v.component, &v.pitch, &v.plane));
        return v;
    }

private:
    static void check(int rc) {
        if (rc != EMLAB_OK) throw std::runtime_error(std::string("SimulationGrid: ") + emlab_last_error());
    }
    emlab_grid_state state() const {
        emlab_grid_state s{};
        check(emlab_grid_get_state(m_g, &s));
        return s;
    }
    emlab_grid* m_g = nullptr;
    GridConfig m_config{};
    std::vector<emlab_source> m_sources;
};

}  // namespace emlab_cpp
