// emlab_internal.h - device layout and kernel entry points shared by the library's translation units.
//
// Field layout in HBM: six FP32 component arrays (Ex, Ey, Ez, Bx, By, Bz), x fastest, rows padded
// to a multiple of 32 floats (128 bytes) so every warp-wide row access is one aligned line.
// Two copies of the six arrays: the fused kernel reads generation `cur` and writes `cur ^ 1`
// (in-place updates are impossible when one pass computes B and then E from it across tile halos).
// Materials: one class index per cell (uint16, or uint32 above 65535 classes) into a table holding,
// per class, the edge conductivity/permittivity (after binary16 rounding), the exponential
// integrator coefficients ca/cb for cells outside the absorber (computed on the host by the very
// formula the kernel would evaluate, so the values are bit-identical), and thin-wire factors.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "emlab.h"
#include "emlab_math.h"

namespace emlab {

// Per-class table entries (float4 pairs, see build_classes in setup.cpp):
//   tabE[2c]   = (ca.x, ca.y, ca.z, cb.x)     tabE[2c+1] = (cb.y, cb.z, 0, 0)
//   tabM[2c]   = (sig.x, sig.y, sig.z, eps.x) tabM[2c+1] = (eps.y, eps.z, 0, 0)
//   tabW[2c]   = (w0.x, w0.y, w0.z, w1.x)     tabW[2c+1] = (w1.y, w1.z, 0, 0)
// Classes >= wire_start carry thin-wire factors other than 1.
struct YeeArgs {
    int nx, ny, nz;
    int pitch;          // floats per row
    long long plane;    // floats per z plane (pitch * ny)
    const float* ex; const float* ey; const float* ez;
    const float* bx; const float* by; const float* bz;
    float* nex; float* ney; float* nez;   // fused kernel: next generation (split kernels: unused)
    float* nbx; float* nby; float* nbz;
    float* wex; float* wey; float* wez;   // split kernels: in-place targets
    float* wbx; float* wby; float* wbz;
    const void* cls;
    const float4* tabE;
    const float4* tabM;
    const float4* tabW;
    unsigned wire_start;
    const float* pml;   // [6][pml_stride]: I_x, I_y, I_z (integer positions), H_x, H_y, H_z (half)
    int pml_stride;
    const unsigned char* pml_cls;  // [6][pml_stride]: depth class of each position (same order)
    const float2* pml_coef;        // [K][K][K]: (e^{-x}, dt phi(x)), x = dt ((V_i + V_j) + V_k)
    const unsigned char* pml_z;    // [nz]: 1 where the plane lies in the absorber along z (common.glsl:40-43;
                                   // per scene in a stack of scenes)
    int pml_K;
    int L;
    float dt;
    int zchunk;
    int tile_rows;   // tiling mode of the fused kernels (8, 16: single-cell tiles; 64, 128: pair tiles)
    unsigned long long* work;      // work-item ticket counter of the persistent kernel (monotonic)
    unsigned long long work_base;  // tickets consumed by all earlier launches on this counter
    int wait_polls;                // polls of a plane's copy barrier before the CTA gives up (wait_limit())
    // x / y absorber lookups of the pair kernel: rows 0 (I_x), 1 (I_y), 3 (H_x), 4 (H_y) of a
    // [6][pml_xy_stride] table pair, one pair per scene of a stack whose scenes have their own
    // cross-sections (pml_xy_scene elements apart), else the grid's own tables (pml_xy_scene 0)
    const unsigned char* pml_cls_xy;
    const float* pml_xy;
    int pml_xy_stride;
    int pml_xy_scene;
    // such a stack's pair-kernel work items (x0 | y0 << 16, first plane, end plane, scene), each inside
    // one scene, and every scene's nx, ny; null for a grid whose items follow from its size
    const int4* items;
    int n_items;
    const int2* scene_xy;
};

// Polls of an on-device wait (mbarrier) before a kernel reports EMLAB_ERR_TIMEOUT: about a second by
// default. emlab_debug_set_wait_limit lowers it so a test can make the first wait of a launch run
// out; the waits that drain copies already in flight before a CTA leaves always keep the default.
constexpr int kWaitPolls = 1 << 20;
int wait_limit();

struct SourceArgs {
    const int4* cells;       // xyz = cell (scene coordinates), w = first list entry; entry n is the sentinel
    const int* zoff;         // per cell: first plane of its scene in a stack of scenes (null: 0)
    const int* scene;        // per cell: its scene in a stack of scenes with their own cross-sections (or null)
    const int* lists;
    const float4* src;       // 4 float4 per source: center, halfExtent, polAmp, softness
    const float* signals;    // [step][nsrc]
    int nsrc;
    int ncells;
};

struct MonitorArgs {
    int nx, ny, nz, pitch;
    long long plane;
    const float* ex; const float* ey; const float* ez;
    const float* bx; const float* by; const float* bz;
};

void launch_yee_fused(const YeeArgs& a, bool wide, cudaStream_t s);

// TMA-staged fused kernel: tensor maps of one field generation and the class index.
struct TmaMaps;
TmaMaps* tma_maps_create();
void tma_maps_destroy(TmaMaps* m);
// Encodes the maps for generation `gen` (0 or 1); returns false if TMA cannot be used.
bool tma_maps_encode(TmaMaps* m, int gen, const YeeArgs& a, bool wide);
bool tma_maps_ready(const TmaMaps* m, int gen);
// pair-kernel work items of a stack of scenes with their own cross-sections (scene by scene, z
// chunk by chunk, tile by tile): tiles of 64 x ty cells over each scene's nx x ny, z chunks of one
// length for all scenes, chosen for g CTAs as the uniform schedule chooses it
std::vector<int4> ragged_items(const std::vector<int>& z0, const std::vector<int>& nx, const std::vector<int>& ny,
                               const std::vector<int>& nz, int ty, int g);
// the uniform grid's pair-kernel schedule for g CTAs: planes per z chunk and work items
void pair_schedule_shape(int nx, int ny, int nz, int ty, int g, int* zc, int* items);
// Launches the TMA kernel reading generation `gen`; err receives a nonzero word if a wait timed out.
// *tickets receives the work-counter tickets the launch consumes (0 for the non-persistent kernels)
bool launch_yee_tma(const YeeArgs& a, const TmaMaps* m, int gen, bool wide, unsigned* err, cudaStream_t s,
                    unsigned long long* tickets);
void launch_yee_split(const YeeArgs& a, bool wide, cudaStream_t s);
void launch_sources(const YeeArgs& a, const SourceArgs& sa, int k, bool wide, cudaStream_t s);

// ports: ports[2i] = (x, y, z, axis), ports[2i+1] = (edges, sign, 0, 0); phasors 8 per port;
// params[k] = (cos wtE, sin wtE, cos wtH, sin wtH) and blend for sub-step k.
void launch_ports(const MonitorArgs& m, const int4* ports, int n, float* phasors, float* series, long long rec_index,
                  const float4* rot, const float* blend, int k, cudaStream_t s);
void launch_ntff(const MonitorArgs& m, const int* box, int points, float* phasors, const float4* rot,
                 const float* blend, int k, cudaStream_t s);
void launch_lines(const MonitorArgs& m, const int4* q, int nq, const int4* terms, const float* weights,
                  float* phasors, float* now, const float4* rot, const float* blend, int k, cudaStream_t s);
void launch_probe_gather(const MonitorArgs& m, const int4* origins, int n, float4* out, const float* cell_sig,
                         const float* cell_eps, cudaStream_t s);
void launch_flux_plane(const MonitorArgs& m, int axis, int index, int rmin0, int rmin1, int rs0, int rs1,
                       float* partials, cudaStream_t s);
void launch_ntff_pattern(const int* box, int points, const float* phasors, const float4* dirs, int first, int count,
                         int slices, float k, float4* partials, cudaStream_t s);
void launch_ntff_pattern_fast(const int* box, int points, const float* phasors, const float4* dirs, int first,
                              int count, int slices, float k, float4* partials, cudaStream_t s);
void launch_ntff_reduce(const float4* dirs, const float4* partials, int first, int count, int slices, float* out,
                        cudaStream_t s);
void launch_port_residuals(const float* series, long long steps, int nports, double* out, cudaStream_t s);
void launch_sweep_sums(const float* series, long long steps, int nports, double nu_lo, double nu_hi, int points,
                       double dt, double* out, cudaStream_t s);
void launch_check_finite(const MonitorArgs& m, unsigned* flag, cudaStream_t s);
// multi-frequency far-field DFT: per-step sampling into a time block, FP64 fold of a block. A box
// record is kDftBoxInts ints: min xyz, max xyz, seven face offsets (box-local point indices), the
// box's first point in the concatenated point list, its point count.
constexpr int kDftBoxInts = 16;
void launch_dft_sample(const MonitorArgs& m, const int* boxes, int nbox, int box_max, int points, float* blk, int t,
                       cudaStream_t s);
// far-field spectra of one box (`points` nodes from point `first` of X's `total_points`) straight
// from the DFT sums scaled by `scale`: per frequency the partial sums of the pattern over direction
// chunks and surface slices, then the per-direction reduction (|N_perp - r x L|^2 and the radiated
// power at direction 0), one launch each for all frequencies; out[(f * count + d) * 2 + {0, 1}]
void launch_ntff_spectra(const int* box, int first, int points, int total_points, const double* X, int nf,
                         const double* omega, double scale, const float4* dirs, int count, int slices,
                         float4* partials, cudaStream_t s);
void launch_ntff_reduce_multi(const float4* dirs, const float4* partials, int count, int slices, int nf, float* out,
                              cudaStream_t s);
// X_new[f][c][j] = X_old[f][c][map[j]] for the carried boxes of a stack compaction
void launch_dft_gather(const double* x_old, int old_points, const int* map, int new_points, int nf, double* x_new,
                       cudaStream_t s);
void launch_dft_fold(const float* blk, int T, int points, int nf, const float2* W, const double* omega, long long n0,
                     double dt, double* X, cudaStream_t s);
void launch_dft_to_phasor(const double* X, int points, int f, double scale, float* ph, cudaStream_t s);
void launch_raymarch(const MonitorArgs& m, const float* sigma, const float* eps, const emlab_render_params& p,
                     unsigned char* img, cudaStream_t s);
// tensor-core fold (dft_tc.cu): MMA N for nf frequencies, host twiddle tables (hi, lo) in the
// kernel's shared-memory layout, and the launcher (false if nf is too large or set-up failed)
int dft_tc_mma_n(int nf);
int dft_tc_block(int nf);  // samples per tensor-core fold: 64 x min(4, 256 / MMA N)
void dft_tc_twiddles(int nf, const double* omega, double dt, std::vector<float>& hi, std::vector<float>& lo);
bool launch_dft_fold_tc(const float* blk, int T, int points, int nf, const float* b_hi, const float* b_lo,
                        const double* omega, long long n0, double dt, double* X, unsigned* err, cudaStream_t s);
void launch_debug_expf(const float* in, float* out, size_t n, cudaStream_t s);

}  // namespace emlab

struct emlab_grid;

namespace emlab {
// The current field generation, stream and device of a configured grid (EMLAB_OK or an error code
// with the message set); records an error message for the calling thread; counts kernel launches.
int grid_view(emlab_grid* g, MonitorArgs* m, cudaStream_t* stream, int* device);
int report_error(int code, const char* msg);
void count_launches(int n);
}  // namespace emlab
