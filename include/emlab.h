/* emlab.h - C ABI of the GB300 FDTD solver (the drop-in boundary for EM_Lab's time-stepping path).
 *
 * Every entry point replaces one member of the reference's solver or monitor classes; the comment
 * on each names the reference function (src/ or shaders/ file:line) whose behaviour it keeps.
 * Conventions:
 *   - lattice layout and units follow shaders/common.glsl:4-12 (c = eps0 = mu0 = 1, dx = 1,
 *     dt = Courant number, B stored as c*B; texel (i,j,k) holds Ex at (i+1/2,j,k), Ey at (i,j+1/2,k),
 *     Ez at (i,j,k+1/2), Bx at (i,j+1/2,k+1/2), By at (i+1/2,j,k+1/2), Bz at (i+1/2,j+1/2,k));
 *   - host arrays are x-fastest: index = (z * ny + y) * nx + x (MaterialVolume::index,
 *     src/SimulationGrid.hpp:55-57);
 *   - every function returns EMLAB_OK (0) or an EMLAB_ERR_* code; emlab_last_error() gives the
 *     message of the calling thread's last failure (the reference throws std::runtime_error);
 *   - caller arrays are borrowed for the duration of the call only;
 *   - one handle is used by one thread at a time; distinct handles are independent.
 */
#ifndef EMLAB_H
#define EMLAB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EMLAB_OK 0
#define EMLAB_ERR_INVALID 1   /* bad argument: size mismatch, out-of-range value, null pointer */
#define EMLAB_ERR_OOM 2       /* device or host allocation failed (grid too large) */
#define EMLAB_ERR_CUDA 3      /* a CUDA call failed; the message names it */
#define EMLAB_ERR_TIMEOUT 4   /* a bounded host wait ran out */
#define EMLAB_ERR_NONFINITE 5 /* non-finite field values detected */
#define EMLAB_ERR_NO_DEVICE 6 /* no CUDA device is visible */

/* Solver kernels, all bit-identical: the fused single-pass Yee step with TMA-staged z planes
 * (default; falls back to the load-staged variant where tensor maps cannot be built), the
 * load-staged fused step, or the reference's two-pass layout. */
#define EMLAB_KERNEL_FUSED 0
#define EMLAB_KERNEL_SPLIT 1
#define EMLAB_KERNEL_FUSED_LDG 2

/* Waveforms of emlab_source (src/SimulationGrid.hpp:108-111). */
#define EMLAB_WAVE_CW 0
#define EMLAB_WAVE_PULSE 1

/* GridConfig (src/SimulationGrid.hpp:25-31). */
typedef struct emlab_grid_config {
    int nx, ny, nz;
    float courant;       /* c dt / dx, clamped to [0.05, 0.99/sqrt(3)] */
    int pml_thickness;   /* absorbing layer depth in cells, clamped to [0, 64] */
    float pml_sigma_max; /* conductivity at the outer edge of the layer */
    float pml_grading;   /* exponential grading g, clamped to [0.25, 12] */
} emlab_grid_config;

/* EdgeOverride (src/SimulationGrid.hpp:76-81): replaces the averaged conductivity of one E edge. */
typedef struct emlab_edge_override {
    int x, y, z; /* owning texel: the edge E_axis sits at texel + 0.5 e_axis */
    int axis;    /* 0, 1, 2 */
    float sigma; /* normalised conductivity */
} emlab_edge_override;

/* WireCoefficient (src/SimulationGrid.hpp:86-94): thin-wire factor on one curl term of one B
 * component; with c1 = c+1, c2 = c+2 (mod 3): curl_c E = term0 - term1, term0 = d_{c1} E_{c2}. */
typedef struct emlab_wire_term {
    int x, y, z;
    int component; /* 0, 1, 2 = Bx, By, Bz */
    int term;      /* 0 or 1 */
    float factor;  /* 2 / ln(cell / radius) */
} emlab_wire_term;

/* SourceDesc (src/SimulationGrid.hpp:113-150): J(x,t) = p A w(x) s(t). */
typedef struct emlab_source {
    float center[3];       /* cell coordinates */
    float half_extent[3];  /* flat-top half extents (0 = point) */
    float softness[3];     /* per-axis Gaussian edge width, clamped >= 0.25 */
    float polarization[3]; /* normalised on upload; zero-length sources are dropped */
    float amplitude;       /* J0 */
    float wavelength;      /* cells; omega = 2 pi / wavelength */
    float phase;           /* radians */
    int waveform;          /* EMLAB_WAVE_CW or EMLAB_WAVE_PULSE */
    float ramp_periods;    /* CW: smooth turn-on; pulse: 1/e half-width tau in periods */
    float repeat_periods;  /* pulse repetition interval (0 = single shot) */
    float delay_periods;   /* start delay */
    int enabled;
} emlab_source;

/* Port of port_accumulate.comp:20-23 / PortSetup (src/Ports.hpp:30-40), solver-facing part. */
typedef struct emlab_port {
    int x, y, z; /* owning texel of the (first) gap edge */
    int axis;
    int edges;   /* 1 = thin-wire gap edge, 4 = corner edges of a 1x1-cell rod gap */
    int sign;    /* +1 / -1 feed orientation */
} emlab_port;

/* One flux plane of poynting_flux.comp:21-26 (box faces are six of these). */
typedef struct emlab_flux_plane {
    int axis;        /* plane normal 0, 1, 2 */
    int index;       /* lattice index along the normal */
    int rect_min[2]; /* first cell along the tangential axes (u, v) = (x,y,z) order skipping axis */
    int rect_max[2]; /* one past the last cell */
} emlab_flux_plane;

/* Solver state read-back: time(), dt(), stepCount(), size(), gpuMemoryBytes()
 * (src/SimulationGrid.hpp:183-188). */
typedef struct emlab_grid_state {
    double time;
    float dt;
    uint64_t step_count;
    int nx, ny, nz;
    uint64_t device_bytes;
    int source_cells; /* cells in the source lists (SimulationGrid.cpp:348) */
    int kernel;       /* EMLAB_KERNEL_* in use */
} emlab_grid_state;

typedef struct emlab_grid emlab_grid;

/* ---- library ---------------------------------------------------------------------------- */
const char* emlab_last_error(void);
int emlab_version(void);
/* Kernels this library has launched since load (graph launches count their kernel nodes). */
uint64_t emlab_launch_count(void);


/* ---- solver: SimulationGrid (src/SimulationGrid.hpp:155-216) ------------------------------ */
/* SimulationGrid::SimulationGrid (src/SimulationGrid.cpp:135-147): binds the current CUDA device
 * and creates the handle's stream. */
int emlab_grid_create(emlab_grid** out);
int emlab_grid_destroy(emlab_grid* g);
/* SimulationGrid::configure (src/SimulationGrid.cpp:149-199): clamps the request, reallocates
 * when the size changed, clears fields and materials (vacuum), rewinds time. Monitors are reset. */
int emlab_grid_configure(emlab_grid* g, const emlab_grid_config* cfg);
/* config() (src/SimulationGrid.hpp:183): the clamped configuration in use. */
int emlab_grid_get_config(const emlab_grid* g, emlab_grid_config* out);
/* SimulationGrid::uploadMaterials (src/SimulationGrid.cpp:209-295): per-cell sigma and eps_r
 * (nx*ny*nz each), edge averaging, sub-cell overrides (invalid ones silently skipped), binary16
 * rounding, thin-wire factors; clears E and B and time. EMLAB_ERR_INVALID on a size mismatch. */
int emlab_grid_upload_materials(emlab_grid* g, const float* sigma, const float* eps_r, int nx, int ny, int nz,
                                const emlab_edge_override* edges, size_t n_edges, const emlab_wire_term* wires,
                                size_t n_wires);
/* SimulationGrid::setSources (src/SimulationGrid.cpp:297-357): drops disabled and zero-polarisation
 * sources, keeps at most 256, builds the per-cell source lists; fields are kept. */
int emlab_grid_set_sources(emlab_grid* g, const emlab_source* sources, size_t n);
/* SimulationGrid::resetFields (src/SimulationGrid.cpp:359-366). */
int emlab_grid_reset_fields(emlab_grid* g);
/* SimulationGrid::step (src/SimulationGrid.cpp:368-433): count leapfrog steps (B, E, sources),
 * then every monitor attached to the grid samples the step, on the device. Returns when the work
 * is queued on the grid's stream; emlab_grid_synchronize waits for it. */
int emlab_grid_step(emlab_grid* g, int count);
/* Bounded wait for the grid's stream (EMLAB_ERR_TIMEOUT after timeout_ms; <= 0 waits 60 s). Also
 * EMLAB_ERR_TIMEOUT if a solver kernel gave up a bounded on-device wait since the last call. */
int emlab_grid_synchronize(emlab_grid* g, int timeout_ms);
int emlab_grid_get_state(const emlab_grid* g, emlab_grid_state* out);
/* Read-back of the E and B textures in the reference's RGBA32F layout (E.a = cell sigma,
 * B.a = cell eps_r; src/SimulationGrid.hpp:4-6), 4 floats per cell. Either pointer may be NULL. */
int emlab_grid_read_fields(emlab_grid* g, float* e_rgba, float* b_rgba);
/* Read-back as six component arrays (nx*ny*nz floats each); NULL pointers are skipped. */
int emlab_grid_read_components(emlab_grid* g, float* ex, float* ey, float* ez, float* bx, float* by, float* bz);
/* Overwrites the field components (for checkpoints and tests); materials and time are kept. */
int emlab_grid_write_components(emlab_grid* g, const float* ex, const float* ey, const float* ez, const float* bx,
                                const float* by, const float* bz);
/* Selects the solver kernel (EMLAB_KERNEL_FUSED or EMLAB_KERNEL_SPLIT); results are identical. */
int emlab_grid_set_kernel(emlab_grid* g, int kernel);
/* Tile shape of the fused kernels: 8 or 16 (rows of 32 cells per CTA, one cell per thread), 32, 64
 * or 128 (64 x 4, 64 x 8 or 64 x 16 tiles, two cells per thread; TMA kernel only) or 0 for the
 * automatic choice. A tuning knob only: every choice gives bit-identical results. */
int emlab_grid_set_tiling(emlab_grid* g, int tile_rows);
/* The cudaStream_t the grid launches on (for events and for ordering caller work). */
int emlab_grid_stream(emlab_grid* g, void** stream);
/* Device view of the field state, in place of eFieldTexture() / bFieldTexture()
 * (src/SimulationGrid.hpp:181-182) for monitors that run on the same GPU: ptrs[0..5] receive the
 * device arrays of Ex, Ey, Ez, Bx, By, Bz of the generation that holds the state once the work
 * queued so far has run; the value of cell (x, y, z) is p[z * plane + y * pitch + x]. Valid until
 * the next emlab_grid_step, reset, configure or destroy (a step writes the other generation).
 * Order device reads after the grid's work through emlab_grid_stream. */
int emlab_grid_field_ptr(emlab_grid* g, float** ptrs, int* pitch, long long* plane);
/* Kernel timing of the solver pass: when enabled, CUDA events bracket every Yee launch (the fused
 * kernel, or the split pair) on the grid's stream; emlab_grid_kernel_time returns the accumulated
 * device time in ms and the number of timed launches since the last reset (reset = 1 clears). */
int emlab_grid_set_timing(emlab_grid* g, int enabled);
int emlab_grid_kernel_time(emlab_grid* g, double* ms, uint64_t* launches, int reset);
/* Chunks of exactly `chunk` steps (even, <= 1024; 0 = off) replay a captured CUDA graph of their
 * launches instead of issuing them one by one (no reference counterpart: the reference issues one
 * dispatch per pass per sub-step, src/SimulationGrid.cpp:368-433). Results are identical. Chunks
 * with the multi-frequency far-field DFT attached, or with solver timing on, run without a graph;
 * with port recording on, a chunk uses its graph when the caller has taken the series
 * (emlab_ports_take_series) since the last chunk. */
int emlab_grid_set_graph(emlab_grid* g, int chunk);
/* Opt-in convolutional PML (no counterpart in the reference, whose absorber is the graded
 * conductivity with matched magnetic loss of shaders/common.glsl:15-43; that absorber stays the
 * default and the parity path). With params, the absorber cells of the grid (pml_thickness of the
 * configuration, plus one, at every face) stretch each spatial derivative of the curl along an axis
 * as dF / kappa + psi, psi <- b psi + c dF (Roden & Gedney's recursive convolution with the complex
 * frequency shift), with sigma = sigma_max d^m, kappa = 1 + (kappa_max - 1) d^m,
 * alpha = alpha_max (1 - d) at normalised depth d; the graded conductivity is off. NULL restores the
 * reference absorber. Either way the fields, the auxiliary fields and time are cleared. Not
 * available for stacks of scenes. Stepping then uses two in-place passes (B, E) of its own kernels. */
typedef struct emlab_cpml {
    float sigma_max; /* conductivity at the outer edge (normalised); about 0.8 (m + 1) is the usual optimum */
    float kappa_max; /* coordinate stretch at the outer edge (>= 1) */
    float alpha_max; /* frequency shift at the inner edge (>= 0) */
    float order;     /* grading exponent m (1 .. 8) */
} emlab_cpml;
int emlab_grid_set_cpml(emlab_grid* g, const emlab_cpml* params);
/* Non-finite check over E and B on the device (Instruments::applyMeasurement's stability check,
 * src/Instruments.cpp:271-275): EMLAB_ERR_NONFINITE if any component is NaN or infinite. */
int emlab_grid_check_finite(emlab_grid* g);

/* ---- port monitor: PortMonitor (src/Ports.hpp:84-140) ------------------------------------- */
/* PortMonitor::configure (src/Ports.cpp:43-75): at most 256 ports; phasors cleared; the (V, I)
 * series is recorded every step when record_steps > 0 (capacity 2^23 floats, src/Ports.cpp:16)
 * or when sweep != 0 (whole capacity). n = 0 disables the monitor. */
int emlab_ports_configure(emlab_grid* g, const emlab_port* ports, size_t n, float wavelength, float averaging_periods,
                          int sweep, size_t record_steps);
/* Phasor state (port_accumulate.comp:24-27): 8 floats per port, stage1 (V re, V im, I re, I im)
 * then stage2. */
int emlab_ports_read_phasors(emlab_grid* g, float* out);
/* Recorded (V, I) pairs, [step][port], recordedSteps() x ports x 2 floats (PortMonitor::readSeries,
 * src/Ports.cpp:138-143). *steps receives recordedSteps(); out may be NULL to query it. */
int emlab_ports_read_series(emlab_grid* g, float* out, size_t max_steps, size_t* steps);
/* Copies the recorded steps (at most max_steps) like emlab_ports_read_series, then restarts the
 * recording at the start of the buffer: chunked read-back of long runs (a ring-down watch). */
int emlab_ports_take_series(emlab_grid* g, float* out, size_t max_steps, size_t* steps);
/* The same take without waiting: queues the copy of the series recorded since the last take into one
 * of two pinned host slots behind the work already queued on the grid's stream, and restarts the
 * recording (the steps queued next record from the start of the buffer). *slot names the slot,
 * *steps the rows it will hold. At most two takes may wait to be collected; while one waits,
 * emlab_ports_configure and emlab_stack_compact are refused (its rows are laid out for the current
 * ports). */
int emlab_ports_take_series_async(emlab_grid* g, int* slot, size_t* steps);
/* Waits (bounded: EMLAB_ERR_TIMEOUT after timeout_ms; <= 0 waits 60 s) for a slot's copy, copies at
 * most max_steps rows to out ((steps, ports, 2) floats) and frees the slot. Work queued after the
 * take keeps running. EMLAB_ERR_TIMEOUT also if a solver kernel gave up a bounded wait. */
int emlab_ports_collect_series(emlab_grid* g, int slot, float* out, size_t max_steps, int timeout_ms);
/* Running DFT of the recorded series at `points` frequencies evenly spaced in 1/lambda between
 * 1/lambda_max and 1/lambda_min, in FP64 on the device (the sums of PortMonitor::evaluateSweep,
 * src/Ports.cpp:215-242, I corrected by e^{i w dt/2}): out[(port * points + f) * 4 + {0..3}] =
 * (sumV re, sumV im, sumI re, sumI im). Also returns the ring-down residual of port 0. */
int emlab_ports_sweep_sums(emlab_grid* g, double lambda_min, double lambda_max, int points, double* out,
                           double* residual);
/* The ring-down residual of PortMonitor::evaluateSweep (src/Ports.cpp:206-213) for every port, on
 * the device over the series recorded since the last take: out[p] = largest |V| of the last
 * max(n / 20, 1) steps / largest |V| of all n steps (1 without signal). The reference reports a
 * sweep as settled once the residual of its first port is at most 1e-3 (-60 dB). */
int emlab_ports_residuals(emlab_grid* g, double* out);

/* ---- far-field monitor: FarFieldMonitor (src/FarField.hpp:75-133) ------------------------ */
/* FarFieldMonitor::configure (src/FarField.cpp:126-174): box clamped into [L+1, n-L-2];
 * EMLAB_ERR_INVALID if degenerate (< 4 cells on an axis). box_out receives the clamped box.
 * wavelength <= 0 disables the monitor. */
int emlab_ntff_configure(emlab_grid* g, const int box_min[3], const int box_max[3], float wavelength,
                         float averaging_periods, int box_out[6]);
/* Huygens-box point count (FarField.cpp:274-282). */
int emlab_ntff_point_count(emlab_grid* g, int* points);
/* PhasorPair per point (ntff_common.glsl:17-28): 32 floats each. */
int emlab_ntff_read_phasors(emlab_grid* g, float* out);
/* ntff_pattern.comp + ntff_reduce.comp (FarField.cpp:226-243, 294-335): for each direction
 * (4 floats, xyz used) out[2d] = |N_perp - r x L|^2 and out[1] = radiated power P. */
int emlab_ntff_evaluate(emlab_grid* g, const float* directions, int n_dirs, float* out);

/* Multi-frequency far-field DFT on a Huygens box (the reference's far-field monitor tracks one
 * frequency with a two-stage running average, ntff_accumulate.comp; this one keeps exact DFT sums at
 * up to 128 frequencies for pulsed runs). Every step samples the co-located E and H of each box node
 * (ntff_common.glsl / field_sampling.glsl) into a 64-step time block; each full block is folded into
 * FP64 sums X_f = sum_k F(t_k) e^{-i w_f t_k}, t_k = n_k dt for E and (n_k - 1/2) dt for H.
 * Box clamped as FarFieldMonitor::configure; n_freq = 0 disables. box_out may be NULL. */
int emlab_ntff_dft_configure(emlab_grid* g, const int box_min[3], const int box_max[3], const float* wavelengths,
                             int n_freq, int box_out[6]);
/* Engine of the block fold: EMLAB_DFT_TENSOR (default; tcgen05 TF32 MMAs with split hi/lo operands
 * and FP32 accumulation in tensor memory, up to 128 frequencies) or EMLAB_DFT_CUDA_CORES (FP32
 * FMA sums). Both apply the block phase in FP32 from FP64 cos/sin and accumulate in FP64. */
#define EMLAB_DFT_TENSOR 0
#define EMLAB_DFT_CUDA_CORES 1
int emlab_ntff_dft_engine(emlab_grid* g, int engine);
/* Box nodes and samples folded so far. */
int emlab_ntff_dft_info(emlab_grid* g, int* points, uint64_t* samples);
/* Folds any partial block and returns the sums: out[((f * points + i) * 6 + c) * 2 + {re, im}],
 * c = Ex, Ey, Ez, Hx, Hy, Hz. */
int emlab_ntff_dft_read(emlab_grid* g, double* out);
/* ntff_pattern.comp + ntff_reduce.comp at frequency index f from the DFT sums scaled by 2/samples
 * (the amplitude of a steady tone): out[2d] = |N_perp - r x L|^2, out[1] = radiated power. */
int emlab_ntff_dft_evaluate(emlab_grid* g, int f, const float* directions, int n_dirs, float* out);
/* The pattern at every configured frequency: out[(f * n_dirs + d) * 2] = |N_perp - r x L|^2,
 * out[f * n_dirs * 2 + 1] = radiated power at f. Same sums as emlab_ntff_dft_evaluate with the
 * surface phases from a 2-pi range reduction and hardware sin/cos (relative difference about 1e-5),
 * two directions per thread: for large angle grids. */
int emlab_ntff_dft_evaluate_all(emlab_grid* g, const float* directions, int n_dirs, float* out);
/* The far-field DFT on several Huygens boxes at once (the boxes of the scenes of a stack): boxes[6k ..
 * 6k + 5] = min xyz, max xyz of box k in grid coordinates, each inside [1, n - 2] on every axis with
 * at least 4 cells (no clamping: the caller keeps each box inside its scene's absorber);
 * EMLAB_ERR_INVALID otherwise. Their nodes are sampled and folded together, box after box in one
 * point list (emlab_ntff_dft_read returns them in that order). block: samples per fold at most, 0
 * for the engine's own block or a multiple of 64 (a shorter block holds fewer samples per node in
 * device memory). A stack compaction keeps the boxes of the kept scenes with their sums.
 * emlab_ntff_dft_evaluate and _evaluate_all need a single box; emlab_ntff_dft_spectra evaluates one
 * box of several. */
int emlab_ntff_dft_configure_boxes(emlab_grid* g, const int* boxes, int n_boxes, const float* wavelengths,
                                   int n_freq, int block);
/* The pattern of box `box` at every configured frequency (1 to 8192 directions, 4 floats each, xyz
 * used), in the layout of emlab_ntff_dft_evaluate_all: out[(f * n_dirs + d) * 2] = |N_perp - r x L|^2,
 * out[f * n_dirs * 2 + 1] = radiated power at f, from the sums scaled by 2 / samples. Two launches
 * for all frequencies; the device scratch grows to the largest request and is kept. */
int emlab_ntff_dft_spectra(emlab_grid* g, int box, const float* directions, int n_dirs, float* out);
/* The same pattern as emlab_ntff_dft_spectra (all frequencies, one box, out in its layout), the sums
 * factorised face by face: on each face the phase e^{jk r.p} splits into a u and a v factor, the sum
 * over v is one complex GEMM over all directions on the tcgen05 tensor cores (BF16 operands split
 * into high and low halves, FP32 accumulation) and the sum over u a per-direction dot product; the
 * sines and cosines drop from directions x points to directions x (nu + nv) per face. Within about
 * 1e-4 of the pattern maximum of the direct sums. 1 to 2^20 directions. */
int emlab_ntff_dft_pattern_gemm(emlab_grid* g, int box, const float* directions, int n_dirs, float* out);

/* ---- volume rendering: VolumeRenderer (src/VolumeRenderer.cpp:66-118, shaders/raymarch.frag) */
/* Camera and look of one rendered frame. inv_view_proj: inverse of projection * view, column-
 * major (glm layout); world space is the lattice mapped to [-1, 1] along the longest axis
 * (VolumeRenderer::latticeToWorld). mode: 0 E + B, 1 E, 2 B, 3 |E x B|, 4 signed E component. */
typedef struct emlab_render_params {
    int width, height;
    float inv_view_proj[16];
    float cam_pos[3];
    float vol_min[3], vol_size[3];     /* world box of the whole grid */
    float clip_min[3], clip_max[3];    /* world box actually marched (cutaway) */
    float step_voxels, gain_e, gain_b, density, emission, material_opacity, exposure;
    int mode, signed_axis;
} emlab_render_params;
/* Ray-marches the current fields into rgba (width * height * 4 bytes, rows bottom-up as
 * glReadPixels returns them); the cell sigma / eps_r of the uploaded MaterialVolume are drawn as
 * metal / dielectric surfaces. The headless replacement of the reference's on-screen renderer and
 * of --screenshot. */
int emlab_render(emlab_grid* g, const emlab_render_params* params, unsigned char* rgba);

/* ---- radar imaging: RadarMonitor::computeImage back-projection (src/Radar.cpp:606-646) ---- */
/* Image grid and array geometry: transmit phase centre, axes (azimuth, elevation, boresight as
 * three rows), the simulated volume inside the absorber, the carrier omega = 2 pi / lambda, the
 * solver dt and the decimated sample spacing, range bins r0 + i dr, azimuth and elevation bins in
 * degrees. */
typedef struct emlab_radar_geometry {
    float tx[3];
    float axes[9];
    float interior_min[3], interior_max[3];
    double omega, dt, sample_dt;
    float r0, dr, az0, daz, el0, del;
    int nr, naz, nel;
} emlab_radar_geometry;
/* power[(ir * nel + ie) * naz + ia] = |sum_i w_i z_i(t_i) e^{j omega t_i}|^2 (-1 outside the volume);
 * z: M decimated complex baseband samples of C elements ([m][i] as float pairs); elem_pos (C x 3),
 * weights (C); tx_pos (ntx x 3) and tx_amp (ntx): the transmitting elements. Host arrays. */
int emlab_radar_backproject(const emlab_radar_geometry* geo, const float* z, int M, int C, const float* elem_pos,
                            const double* weights, const float* tx_pos, const double* tx_amp, int ntx,
                            double* power);

/* ---- stacks of independent scenes (batched sweeps; no reference counterpart: the reference steps
 * one SimulationGrid per scene, src/SimulationGrid.cpp:149-199, 368-433) ----
 * Scenes of equal nx x ny and equal solver settings lie one after another along z in one grid,
 * scene i at planes z0[i] .. z0[i] + nz[i] - 1, one frozen separator plane between scenes; every
 * step launch covers all of them, and each scene evolves bit for bit as it would alone. */
/* Configures g as a stack: cfg gives nx, ny and the solver settings (cfg->nz is ignored), scene_nz
 * the depth of each scene (each clamped as SimulationGrid::configure clamps). Fields cleared, every
 * scene vacuum, no sources, monitors detached. */
int emlab_stack_configure(emlab_grid* g, const emlab_grid_config* cfg, const int* scene_nz, int n_scenes);
/* A stack of scenes of different cross-sections: dims[3i .. 3i + 2] = nx, ny, nz of scene i (each
 * clamped as SimulationGrid::configure clamps), the solver settings from cfg (its nx, ny, nz are
 * ignored). The grid's cross-section is the largest scene's; every scene lies at x = y = 0 of its
 * planes, and the cells of its planes outside its nx x ny hold the separator's frozen class (E and B
 * stay 0 there, as outside a grid of its own). Each scene keeps its own absorber on all six faces.
 * One launch of the persistent pair kernel steps every scene: its work items are the tiles of each
 * scene's own cross-section. Such a stack runs the fused kernel with tiles of cell pairs only
 * (emlab_grid_set_kernel / _set_tiling refuse the others). Otherwise as emlab_stack_configure. */
int emlab_stack_configure_scenes(emlab_grid* g, const emlab_grid_config* cfg, const int* dims, int n_scenes);
/* nx, ny, nz of every scene (3 ints per scene). */
int emlab_stack_scene_dims(const emlab_grid* g, int* dims);
/* Layout: number of scenes, first plane and depth of each (arrays of n_scenes entries, or NULL). */
int emlab_stack_info(const emlab_grid* g, int* n_scenes, int* z0, int* nz);
/* uploadMaterials for one scene, in the scene's own coordinates (nx, ny, nz = the scene's). Clears the
 * fields of the stack and its step count. The merged class table is built at the next step or
 * emlab_stack_commit. */
int emlab_stack_upload_materials(emlab_grid* g, int scene, const float* sigma, const float* eps_r, int nx, int ny,
                                 int nz, const emlab_edge_override* edges, size_t n_edges,
                                 const emlab_wire_term* wires, size_t n_wires);
int emlab_stack_commit(emlab_grid* g);
/* setSources per scene: sources[k] (scene coordinates) belongs to scene scene_of[k]; each scene's
 * sources are filtered and capped as setSources does for one grid. */
int emlab_stack_set_sources(emlab_grid* g, const emlab_source* sources, const int* scene_of, size_t n);
/* Drops the scenes whose keep[i] is 0: the others' fields, materials and sources move to a shorter
 * stack (device copies; step count kept). The far-field DFT boxes that lie inside kept scenes move
 * with them, sums included (emlab_ntff_dft_configure_boxes); the other monitors are detached: ports
 * are re-attached by the caller at the scenes' new planes (emlab_stack_info). Refused while an
 * asynchronous series take waits to be collected. */
int emlab_stack_compact(emlab_grid* g, const unsigned char* keep);

/* ---- probes and flux: FieldAnalyzer (src/FieldAnalyzer.hpp:73-130) ----------------------- */
/* probe_gather.comp (FieldAnalyzer.cpp:274-303): origins are 4 ints per probe (xyz used); out
 * receives 54 texels (27 E, then 27 B, 4 floats each) per probe. */
int emlab_probe_gather(emlab_grid* g, const int* origins, int n_probes, float* out);
/* poynting_flux.comp per plane (FieldAnalyzer.cpp:100-124, 317-358): out[i] = FP64 sum of the
 * FP32 16x16-workgroup partial sums of plane i (without the box orientation sign). */
int emlab_flux_planes(emlab_grid* g, const emlab_flux_plane* planes, int n_planes, double* out);

/* Flux through planes for callers that must not allocate device memory (no counterpart in the
 * reference). emlab_flux_planes allocates and frees its per-workgroup partial sums on every call.
 * Two kinds of caller cannot accept that: a frame loop that measures flux every other frame while
 * the solver runs (cudaFree waits for the whole device, so each measurement would stall the
 * stepping), and an application that budgets all device memory itself (a library allocation it
 * did not plan for can fail part-way through a run, or push its own allocations out). This entry
 * point allocates nothing: its scratch is a fixed file-scope device array of
 * EMLAB_FLUX_NOALLOC_MAX_PARTIALS FP32 workgroup partials (256 KB) plus
 * EMLAB_FLUX_NOALLOC_MAX_PLANES FP64 sums, held by every device that loads the library until the
 * process exits. Requests needing more planes or partials fail with EMLAB_ERR_INVALID. The first
 * call on a device looks the scratch up (cudaGetSymbolAddress, with the grid's device current);
 * make that first call before any stream capture. Every call shares the scratch and overwrites all
 * of it that it reads, so calls whose kernels overlap on the GPU (grids on different streams of one
 * device) race. The call waits for the grid's stream and copies the sums to `out` before it
 * returns. Results equal emlab_flux_planes bit for bit. */
#define EMLAB_FLUX_NOALLOC_MAX_PLANES 64
#define EMLAB_FLUX_NOALLOC_MAX_PARTIALS 65536
int emlab_flux_planes_noalloc(emlab_grid* g, const emlab_flux_plane* planes, int n_planes, double* out);
/* FieldAnalyzer::submit / collect (src/FieldAnalyzer.cpp:126-272): submit queues probe gathers
 * (as emlab_probe_gather) and flux planes (as emlab_flux_planes) on the grid's stream into buffers
 * the grid owns (pinned host staging) and returns at once; collect waits for the oldest submitted
 * measurement and returns it, so a frame loop reads the previous frame's values while the next
 * steps run. At most two measurements are in flight. *ready = 0 when nothing was pending. */
int emlab_analyzer_submit(emlab_grid* g, const int* probe_origins, int n_probes, const emlab_flux_plane* planes,
                          int n_planes);
int emlab_analyzer_collect(emlab_grid* g, float* probe_out, double* flux_out, int* ready);

/* ---- coax line monitor: line_accumulate.comp (src/Coax.cpp:179-197) ---------------------- */
/* quantities: 4 ints each (first term, term count, 0 = E integral / 1 = B integral, unused);
 * terms: 4 ints each (x, y, z, component 0-5 = Ex..Ez, Bx..Bz); weights: one per term.
 * n_quantities = 0 disables the monitor. */
int emlab_lines_configure(emlab_grid* g, const int* quantities, int n_quantities, const int* terms,
                          const float* weights, int n_terms, float wavelength, float averaging_periods);
/* Phasors (4 floats per quantity: stage1 re, im, stage2 re, im) and instantaneous values. */
int emlab_lines_read(emlab_grid* g, float* phasors, float* now);

/* ---- host-side set-up (no device needed) ------------------------------------------------- */
/* The edge materials uploadMaterials derives (src/SimulationGrid.cpp:224-291), as the shaders see
 * them after unpackHalf2x16: per cell 3 conductivities (x, y, z edges, >= 0), 3 permittivities
 * (>= 1) and the thin-wire factors of term0 and term1 (3 each); any output pointer may be NULL.
 * Also returns the number of distinct material classes the device table will hold. */
int emlab_edge_materials(const float* sigma, const float* eps_r, int nx, int ny, int nz,
                         const emlab_edge_override* edges, size_t n_edges, const emlab_wire_term* wires,
                         size_t n_wires, float* edge_sigma, float* edge_eps, float* wire0, float* wire1,
                         uint32_t* classes);
/* SourceDesc::signal (src/SimulationGrid.cpp:103-130): the FP64 source waveform at time t. */
double emlab_source_signal(const emlab_source* source, double t);
/* The source records and per-cell source lists setSources derives (src/SimulationGrid.cpp:297-349)
 * on a grid of nx x ny x nz cells: packed receives 16 floats per kept source (centre, half extent,
 * polarisation | amplitude, softness, as vec4s); cells 4 ints per listed cell (x, y, z, first list
 * entry) plus the sentinel (0, 0, 0, list length); lists the source index of every (cell, source)
 * pair. *n_sources, *n_cells (without the sentinel) and *n_lists receive the sizes; any of packed,
 * cells, lists may be NULL (a first call sizes the arrays). */
int emlab_source_lists(const emlab_source* sources, size_t n, int nx, int ny, int nz, float* packed, int32_t* cells,
                       int32_t* lists, int* n_sources, int* n_cells, int* n_lists);

/* ---- self-checks ------------------------------------------------------------------------- */
/* Test hook of the bounded on-device waits (no counterpart in the reference; its bounded waits are
 * host-side, src/FarField.cpp:287, src/Ports.cpp:152): the number of polls a solver or far-field-fold
 * kernel makes on a copy or MMA barrier before it records EMLAB_ERR_TIMEOUT and leaves, for launches
 * queued from now on in this process. 0 makes every such launch give up at its first wait (after
 * waiting, with the full bound, for the copies it already issued); values above the default (about a
 * second of polling) are clamped to it. Restore with emlab_debug_set_wait_limit(1 << 20). */
int emlab_debug_set_wait_limit(int polls);
/* Evaluates the device emlab_expf on n inputs (bit-exactness check against the host). */
int emlab_debug_expf(const float* in, float* out, size_t n);
/* Host-side schedule of the persistent pair kernel (no device needed), for `ctas` resident CTAs and
 * 64 x tile_rows tiles: on a single grid, the planes per z chunk and the number of work items;
 * on a stack of scenes with their own cross-sections (emlab_stack_configure_scenes), the work items
 * themselves, 5 ints each (x0, y0, first plane, end plane, scene) in launch order. *n_items receives
 * the count; out may be NULL to query it, else it holds cap items. */
int emlab_debug_pair_schedule(int nx, int ny, int nz, int tile_rows, int ctas, int* zc, int* items);
int emlab_debug_ragged_items(const int* z0, const int* nx, const int* ny, const int* nz, int n_scenes, int tile_rows,
                             int ctas, int* out, size_t cap, size_t* n_items);

#ifdef __cplusplus
}
#endif

#endif /* EMLAB_H */
