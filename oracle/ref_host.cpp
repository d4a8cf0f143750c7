// ref_host.cpp - the reference's own host-side C++ for the solver set-up and the radar image,
// compiled here as written (TEST INFRASTRUCTURE: it pins the restatement's and the library's set-up
// code to the reference). oracle/build_ref.py copies the pure-CPU parts out of the reference tree
// into oracle/_ref/*.inc (never committed):
//   SimulationGrid.hpp  GridConfig, Material, MaterialVolume, EdgeOverride, WireCoefficient,
//                       SubcellModel, Waveform, SourceDesc (the types)
//   SimulationGrid.cpp  GPUSource; MaterialVolume and SourceDesc member definitions (signal,
//                       dipole, planeWave, ...); from uploadMaterials the edge averaging, the
//                       overrides and the binary16 packing of the edge and thin-wire textures
//                       (:224-264, :276-289); from setSources the source filtering and packing and
//                       the per-cell source lists (:297-349)
//   Radar.cpp           RadarMonitor::direction, RadarMonitor::txDelay and the back-projection loop
//                       of computeImage (:606-646)
// Nothing of the graphics API is compiled: the extracted spans stop before every GL call, and the
// wrappers below hand their results (the texel arrays the reference would upload) back to the caller.
// glm is replaced by oracle/glm_host.hpp.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <utility>
#include <vector>

#include "glm_host.hpp"

extern "C" {
#include "../include/emlab.h"
}

namespace refhost {

#include "ref_types.inc"

namespace {
#include "ref_gpusource.inc"
}  // namespace

#include "ref_defs.inc"

// The members of SimulationGrid that the extracted set-up spans read or write.
struct GridMembers {
    static constexpr int kMaxSources = 256;  // SimulationGrid::kMaxSources (SimulationGrid.hpp)
    GridConfig m_config;
    std::vector<SourceDesc> m_sources;
    int m_sourceCellCount = 0;
    std::vector<glm::uvec4> edge_texels;  // what uploadMaterials sends to the edge-material texture
    std::vector<glm::uvec4> wire_texels;  // ... and to the thin-wire texture (empty: no thin wires)
    std::vector<GPUSource> packed_sources;
    std::vector<glm::ivec4> source_cells;
    std::vector<std::int32_t> source_lists;

    void uploadMaterials(const MaterialVolume& materials, const SubcellModel& subcell) {
        const size_t n = materials.sigma().size();
#include "ref_upload_edges.inc"
        edge_texels = edge;
        wire_texels.clear();
        if (!subcell.wireTerms.empty()) {
#include "ref_upload_wires.inc"
            wire_texels = packed;
        }
    }

    void setSources(const std::vector<SourceDesc>& sources) {
#include "ref_sources_pack.inc"
#include "ref_sources_lists.inc"
        packed_sources = packed;
        source_cells = cells;
        source_lists = lists;
    }
};

// The members of RadarMonitor that direction(), txDelay() and the back-projection loop read.
struct RadarCore {
    glm::vec3 m_tx{0.0f};
    glm::vec3 m_axes[3]{{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    float m_wavelength = 16.0f;
    glm::vec3 m_interiorMin{0.0f}, m_interiorMax{0.0f};
    std::vector<glm::vec3> m_elementPos;
    std::vector<double> m_weights;
    std::vector<glm::vec3> m_txPos;
    std::vector<double> m_txAmp;

    glm::vec3 direction(float azDeg, float elDeg) const;
    double txDelay(const glm::vec3& p) const;

    struct Image {
        int nr = 0, naz = 0, nel = 0;
        float r0 = 0.0f, az0 = 0.0f, daz = 1.0f, el0 = 0.0f, del = 1.0f;
    };

    // computeImage's back-projection over every elevation row: power[(ir * nel + ie) * naz + ia]
    void backproject(const Image& img, float dr, const std::vector<std::complex<float>>& z, size_t M, size_t C,
                     double dt, double sampleDt, std::vector<double>& power) const {
        const double w = glm::two_pi<double>() / m_wavelength;
#include "ref_radar_rows.inc"
        rows(0, img.nel);
    }
};

#include "ref_radar_members.inc"

// The adaptive GPS array's weight computation (Crpa.cpp): the helpers of its anonymous namespace
// (toDb, meanPower, dotH, solve), the hybrid channels and computeWeights up to its SINR scores.
#include "ref_crpa_types.inc"
namespace crpa {
#include "ref_crpa_algebra.inc"
}
using crpa::cd;

struct CrpaCore {
    CrpaSetup m_setup;
    std::vector<EmitterSetup> m_emitters;
    std::vector<std::pair<int, int>> m_elementPorts;
    int m_satellite = 0;
    glm::vec3 m_center{0.0f};
    float m_wavelength = 16.0f, m_cellSize = 1e-3f;
    std::vector<std::vector<cd>> m_baseband;
    std::vector<std::vector<cd>> m_response;
    CrpaResult m_result;

    std::vector<cd> channels(const std::vector<cd>& ports, bool lhcp = false) const;

    void computeWeights() {
        using namespace crpa;
        CrpaResult r;
        const size_t N = m_elementPorts.size(), E = m_emitters.size();
        (void)E;
#include "ref_crpa_weights.inc"
        r.valid = true;
        m_result = std::move(r);
    }
};

#include "ref_crpa_channels.inc"

SourceDesc from_c(const emlab_source& c) {
    SourceDesc s;
    s.center = glm::vec3(c.center[0], c.center[1], c.center[2]);
    s.halfExtent = glm::vec3(c.half_extent[0], c.half_extent[1], c.half_extent[2]);
    s.softness = glm::vec3(c.softness[0], c.softness[1], c.softness[2]);
    s.polarization = glm::vec3(c.polarization[0], c.polarization[1], c.polarization[2]);
    s.amplitude = c.amplitude;
    s.wavelength = c.wavelength;
    s.phase = c.phase;
    s.waveform = c.waveform == EMLAB_WAVE_PULSE ? Waveform::GaussianPulse : Waveform::ContinuousWave;
    s.rampPeriods = c.ramp_periods;
    s.repeatPeriods = c.repeat_periods;
    s.delayPeriods = c.delay_periods;
    s.enabled = c.enabled != 0;
    return s;
}

void to_c(const SourceDesc& s, emlab_source* c) {
    for (int i = 0; i < 3; ++i) {
        c->center[i] = s.center[i], c->half_extent[i] = s.halfExtent[i];
        c->softness[i] = s.softness[i], c->polarization[i] = s.polarization[i];
    }
    c->amplitude = s.amplitude, c->wavelength = s.wavelength, c->phase = s.phase;
    c->waveform = s.waveform == Waveform::GaussianPulse ? EMLAB_WAVE_PULSE : EMLAB_WAVE_CW;
    c->ramp_periods = s.rampPeriods, c->repeat_periods = s.repeatPeriods, c->delay_periods = s.delayPeriods;
    c->enabled = s.enabled ? 1 : 0;
}

}  // namespace refhost

using namespace refhost;

extern "C" {

// SourceDesc::signal (SimulationGrid.cpp:103-130).
double ref_host_signal(const emlab_source* src, double t) { return from_c(*src).signal(t); }

// SourceDesc::dipole (SimulationGrid.cpp:70-82) and SourceDesc::planeWave (:84-97).
void ref_host_dipole(const float center[3], const float axis[3], float wavelength, float current, float length,
                     emlab_source* out) {
    to_c(SourceDesc::dipole(glm::vec3(center[0], center[1], center[2]), glm::vec3(axis[0], axis[1], axis[2]),
                            wavelength, current, length),
         out);
}
void ref_host_plane_wave(int normal_axis, float position, const float pol[3], float wavelength, float amplitude,
                         emlab_source* out) {
    to_c(SourceDesc::planeWave(normal_axis, position, glm::vec3(pol[0], pol[1], pol[2]), wavelength, amplitude), out);
}

// uploadMaterials' host arithmetic: the MaterialVolume is filled cell by cell through
// MaterialVolume::set (its clamps), then edge_out receives 4 uint32 per cell (the RGBA32UI edge
// texel: half2(sx, sy), half2(sz, ex), half2(ey, ez), 0) and, when wires are given, wire_out
// receives 4 uint32 per cell (half2 factors of Bx, By, Bz terms, 0). Returns 0, or 1 when
// wire_out is needed but NULL.
int ref_host_upload_materials(const float* sigma, const float* eps_r, int nx, int ny, int nz,
                              const emlab_edge_override* edges, size_t n_edges, const emlab_wire_term* wires,
                              size_t n_wires, uint32_t* edge_out, uint32_t* wire_out) {
    MaterialVolume materials(glm::ivec3(nx, ny, nz));
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const size_t i = ((size_t)z * ny + y) * nx + x;
                materials.set(glm::ivec3(x, y, z), Material{sigma[i], eps_r[i]});
            }
    SubcellModel subcell;
    for (size_t k = 0; k < n_edges; ++k) {
        EdgeOverride o;
        o.texel = glm::ivec3(edges[k].x, edges[k].y, edges[k].z);
        o.axis = edges[k].axis;
        o.sigma = edges[k].sigma;
        subcell.edges.push_back(o);
    }
    for (size_t k = 0; k < n_wires; ++k) {
        WireCoefficient w;
        w.texel = glm::ivec3(wires[k].x, wires[k].y, wires[k].z);
        w.component = wires[k].component;
        w.term = wires[k].term;
        w.factor = wires[k].factor;
        subcell.wireTerms.push_back(w);
    }
    GridMembers g;
    g.m_config.size = glm::ivec3(nx, ny, nz);
    g.uploadMaterials(materials, subcell);
    std::memcpy(edge_out, g.edge_texels.data(), g.edge_texels.size() * sizeof(glm::uvec4));
    if (!g.wire_texels.empty()) {
        if (!wire_out) return 1;
        std::memcpy(wire_out, g.wire_texels.data(), g.wire_texels.size() * sizeof(glm::uvec4));
    }
    return 0;
}

// setSources' host arithmetic: packed receives 16 floats per kept source (GPUSource: centre,
// half extent, polarisation | amplitude, softness as vec4s); cells 4 ints per listed cell plus the
// sentinel; lists the source indices. Returns the number of kept sources; *n_cells (without the
// sentinel) and *n_lists are the sizes. Output arrays must hold n sources, and the cells and lists
// the caller sizes with a first call whose cells / lists are NULL.
int ref_host_set_sources(const emlab_source* src, size_t n, int nx, int ny, int nz, float* packed, int32_t* cells,
                         int32_t* lists, int* n_cells, int* n_lists) {
    std::vector<SourceDesc> sources;
    for (size_t i = 0; i < n; ++i) sources.push_back(from_c(src[i]));
    GridMembers g;
    g.m_config.size = glm::ivec3(nx, ny, nz);
    g.setSources(sources);
    *n_cells = g.m_sourceCellCount;
    *n_lists = (int)g.source_lists.size();
    if (packed) std::memcpy(packed, g.packed_sources.data(), g.packed_sources.size() * sizeof(GPUSource));
    if (cells) std::memcpy(cells, g.source_cells.data(), g.source_cells.size() * sizeof(glm::ivec4));
    if (lists) std::memcpy(lists, g.source_lists.data(), g.source_lists.size() * sizeof(int32_t));
    return (int)g.packed_sources.size();
}

// RadarMonitor::computeImage's back-projection with the arguments of emlab_radar_backproject
// (z as [m][element] float pairs), the carrier given as the wavelength the monitor stores.
void ref_host_radar_backproject(const emlab_radar_geometry* geo, float wavelength, const float* z, int M, int C,
                                const float* elem_pos, const double* weights, const float* tx_pos,
                                const double* tx_amp, int ntx, double* power) {
    RadarCore r;
    r.m_tx = glm::vec3(geo->tx[0], geo->tx[1], geo->tx[2]);
    for (int a = 0; a < 3; ++a) r.m_axes[a] = glm::vec3(geo->axes[3 * a], geo->axes[3 * a + 1], geo->axes[3 * a + 2]);
    r.m_wavelength = wavelength;
    r.m_interiorMin = glm::vec3(geo->interior_min[0], geo->interior_min[1], geo->interior_min[2]);
    r.m_interiorMax = glm::vec3(geo->interior_max[0], geo->interior_max[1], geo->interior_max[2]);
    for (int i = 0; i < C; ++i) {
        r.m_elementPos.push_back(glm::vec3(elem_pos[3 * i], elem_pos[3 * i + 1], elem_pos[3 * i + 2]));
        r.m_weights.push_back(weights[i]);
    }
    for (int j = 0; j < ntx; ++j) {
        r.m_txPos.push_back(glm::vec3(tx_pos[3 * j], tx_pos[3 * j + 1], tx_pos[3 * j + 2]));
        r.m_txAmp.push_back(tx_amp[j]);
    }
    std::vector<std::complex<float>> zz((size_t)M * C);
    for (size_t k = 0; k < zz.size(); ++k) zz[k] = std::complex<float>(z[2 * k], z[2 * k + 1]);
    RadarCore::Image img;
    img.nr = geo->nr, img.naz = geo->naz, img.nel = geo->nel;
    img.r0 = geo->r0, img.az0 = geo->az0, img.daz = geo->daz, img.el0 = geo->el0, img.del = geo->del;
    std::vector<double> out((size_t)img.nr * img.nel * img.naz, 0.0);
    r.backproject(img, geo->dr, zz, (size_t)M, (size_t)C, geo->dt, geo->sample_dt, out);
    std::memcpy(power, out.data(), out.size() * sizeof(double));
}

// CrpaMonitor::computeWeights from the measured responses: elements (their X, Y port indices and
// phase centres), emitters (positions; `satellite` is the wanted one), response[e][p] as complex
// pairs, and in blind mode the noise-free snapshots baseband[k][i]. weights receives N complex
// pairs, scores (sinrSingleDb, sinrSteeringDb, sinrMvdrDb, satelliteGainDb).
void ref_host_crpa_weights(int n_elem, const int* element_ports, const float* element_centers, int n_emit,
                           const float* emitter_pos, int n_ports, const double* response, int satellite,
                           const float center[3], float wavelength, float cell_size, float jnr_db, float snr_db,
                           int measured_steering, int mvdr, int blind, unsigned noise_seed, float snapshot_periods,
                           int n_snap, const double* baseband, double* weights, double* scores) {
    CrpaCore c;
    for (int i = 0; i < n_elem; ++i) {
        c.m_elementPorts.emplace_back(element_ports[2 * i], element_ports[2 * i + 1]);
        CrpaElement el;
        el.center = glm::vec3(element_centers[3 * i], element_centers[3 * i + 1], element_centers[3 * i + 2]);
        c.m_setup.elements.push_back(el);
    }
    for (int e = 0; e < n_emit; ++e) {
        EmitterSetup em;
        em.position = glm::vec3(emitter_pos[3 * e], emitter_pos[3 * e + 1], emitter_pos[3 * e + 2]);
        c.m_emitters.push_back(em);
        std::vector<cd> r((size_t)n_ports);
        for (int p = 0; p < n_ports; ++p)
            r[(size_t)p] = cd(response[((size_t)e * n_ports + p) * 2], response[((size_t)e * n_ports + p) * 2 + 1]);
        c.m_response.push_back(r);
    }
    for (int k = 0; k < n_snap; ++k) {
        std::vector<cd> s((size_t)n_elem);
        for (int i = 0; i < n_elem; ++i)
            s[(size_t)i] = cd(baseband[((size_t)k * n_elem + i) * 2], baseband[((size_t)k * n_elem + i) * 2 + 1]);
        c.m_baseband.push_back(s);
    }
    c.m_satellite = satellite;
    c.m_center = glm::vec3(center[0], center[1], center[2]);
    c.m_wavelength = wavelength, c.m_cellSize = cell_size;
    c.m_setup.jnrDb = jnr_db, c.m_setup.snrDb = snr_db;
    c.m_setup.measuredSteering = measured_steering != 0, c.m_setup.mvdr = mvdr != 0, c.m_setup.blind = blind != 0;
    c.m_setup.noiseSeed = noise_seed, c.m_setup.snapshotPeriods = snapshot_periods;
    c.computeWeights();
    for (int i = 0; i < n_elem; ++i) {
        weights[2 * i] = c.m_result.weights[(size_t)i].real();
        weights[2 * i + 1] = c.m_result.weights[(size_t)i].imag();
    }
    scores[0] = c.m_result.sinrSingleDb, scores[1] = c.m_result.sinrSteeringDb;
    scores[2] = c.m_result.sinrMvdrDb, scores[3] = c.m_result.satelliteGainDb;
}

// Crpa.cpp's solve (Gaussian elimination with partial pivoting): A n x n, b n, x n, complex pairs.
void ref_host_crpa_solve(const double* A, const double* b, int n, double* x) {
    std::vector<cd> a((size_t)n * n), bb((size_t)n);
    for (size_t k = 0; k < a.size(); ++k) a[k] = cd(A[2 * k], A[2 * k + 1]);
    for (int k = 0; k < n; ++k) bb[(size_t)k] = cd(b[2 * k], b[2 * k + 1]);
    const std::vector<cd> r = crpa::solve(a, bb, (size_t)n);
    for (int k = 0; k < n; ++k) x[2 * k] = r[(size_t)k].real(), x[2 * k + 1] = r[(size_t)k].imag();
}

}  // extern "C"
