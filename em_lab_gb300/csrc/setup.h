// setup.h - host-side set-up arithmetic of the solver (no CUDA calls): configuration clamps,
// edge-averaged materials and their class table, PML profile tables, source packing and per-cell
// source lists, source signals. Each routine names the reference code it follows.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/emlab.h"

namespace emlab {

// SimulationGrid::configure clamps (src/SimulationGrid.cpp:149-156).
void clamp_config(emlab_grid_config& c);

// Rows padded to 32 floats.
inline int row_pitch(int nx) { return (nx + 31) / 32 * 32; }

struct ClassTable {
    std::vector<uint32_t> cls;   // per cell, pitched layout (z * ny + y) * pitch + x
    std::vector<float> tabE;     // 8 floats per class: ca.xyz, cb.x | cb.yz, 0, 0
    std::vector<float> tabM;     // 8 floats per class: sig.xyz, eps.x | eps.yz, 0, 0
    std::vector<float> tabW;     // 8 floats per class: w0.xyz, w1.x | w1.yz, 0, 0
    uint32_t classes = 0;
    uint32_t wire_start = 0;     // classes >= wire_start carry thin-wire factors
};

// uploadMaterials' edge averaging, overrides, binary16 packing and thin-wire factors
// (src/SimulationGrid.cpp:224-291) folded into a class table. The coefficients use dt.
// Returns false and sets err on allocation failure.
bool build_classes(const float* sigma, const float* eps, int nx, int ny, int nz, const emlab_edge_override* edges,
                   size_t n_edges, const emlab_wire_term* wires, size_t n_wires, float dt, ClassTable& out,
                   std::string& err);

// Recomputes tabE (ca, cb) for a new dt without rebuilding the classes.
void class_coefficients(ClassTable& t, float dt);

// Absorber conductivity at integer (I) and half-integer (H) positions per axis
// (common.glsl:23-36): 6 tables of `stride` floats: I_x, I_y, I_z, H_x, H_y, H_z.
std::vector<float> pml_tables(const emlab_grid_config& c, int stride);

// Absorber coefficients by depth class: each axis position (integer or half-integer) maps to a
// class k in [0, K), K = 2L + 2 (0: outside the layer, 1..L: integer depths, L+1..2L+1: depths
// 0.5..L+0.5), and coef[(i K + j) K + k] = (e^{-x}, dt phi(x)) with x = ((V_i + V_j) + V_k) dt,
// V the profile of common.glsl:23-27 at the class depth. cls: 6 tables of `stride` bytes in the
// order of pml_tables.
void pml_class_tables(const emlab_grid_config& c, int stride, std::vector<uint8_t>& cls, std::vector<float>& coef,
                      int& K);

// setSources (src/SimulationGrid.cpp:302-349): packed sources (16 floats: center, halfExtent,
// polAmp, softness) and the sorted per-cell lists (cells: 4 ints per cell + sentinel).
int pack_sources(const emlab_source* s, size_t n, std::vector<emlab_source>& desc, std::vector<float>& packed);
void source_lists(const std::vector<float>& packed, int nsrc, const int n[3], std::vector<int32_t>& cells,
                  std::vector<int32_t>& lists);

// SourceDesc::signal (src/SimulationGrid.cpp:103-130) in FP64.
double source_signal(const emlab_source& s, double t);

}  // namespace emlab
