// yee_tma.cu - the fused Yee step with TMA-staged z planes (sm_103a).
//
// Same arithmetic and traversal as yee_fused (yee.cu): a CTA owns a 32 x TY column of cells and
// marches it along z, computing B^{n+1/2} for its cells plus the -x/-y halo cells, then E^{n+1}.
// Difference: the inputs of each z plane (E^n with a one-cell halo, B^n and the class index with
// the low halo) arrive by cp.async.bulk.tensor into a 4- or 6-deep shared-memory ring, issued by
// a control warp and completed on per-stage mbarriers, so several planes are in flight while the
// CTA computes; threads never form global addresses for loads. The control warp also computes the
// halo B components, so the cell warps run a branch-free update with hoisted invariants.
// B^{n+1/2} of the plane is kept in a double-buffered shared tile so one __syncthreads per plane
// suffices. Results go to the other field generation with coalesced 128-byte warp stores.
//
// TMA boxes start at x0-4 (x0-8 for a 16-bit class index) so the innermost coordinate stays
// 16-byte aligned; coordinates outside the grid read zeros, which is exactly the reference's
// rule that E beyond the upper faces is 0 (update_B.comp:27-29). Every mbarrier wait is bounded:
// on expiry the CTA records an error word and leaves (the host reports EMLAB_ERR_TIMEOUT).
#include <cuda.h>

#include <algorithm>
#include <mutex>

#include "yee_common.cuh"

namespace emlab {

struct TmaMaps {
    CUtensorMap e[2][3];
    CUtensorMap b[2][3];
    CUtensorMap cls;
    bool ok[2] = {false, false};
    bool cls_ok = false;
};

namespace {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: `polls` tries, about a second of polling at the default kWaitPolls (try_wait itself
// suspends for a while); 0 tries gives up at once (the test hook of emlab_debug_set_wait_limit).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int polls = kWaitPolls) {
    for (int i = 0; i < polls; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

template <int TY, typename Idx>
struct Layout {
    static constexpr int STAGES = TY <= 8 ? 6 : 4;           // planes in the shared-memory ring
    static constexpr int EW = 40;                         // E box: x0-4 .. x0+35, TY+2 rows
    static constexpr int BW = 36;                         // B box: x0-4 .. x0+31, TY+1 rows
    static constexpr int CW = sizeof(Idx) == 2 ? 40 : 36;  // class box width
    static constexpr int CX = sizeof(Idx) == 2 ? 8 : 4;    // class box starts at x0 - CX
    static constexpr int E_BYTES = EW * (TY + 2) * 4;
    static constexpr int B_BYTES = BW * (TY + 1) * 4;
    static constexpr int C_BYTES = CW * (TY + 1) * (int)sizeof(Idx);
    static constexpr int EP = (E_BYTES + 127) / 128 * 128;  // 128-byte aligned TMA destinations
    static constexpr int BP = (B_BYTES + 127) / 128 * 128;
    static constexpr int CP = (C_BYTES + 127) / 128 * 128;
    static constexpr int E_OFF = 0;
    static constexpr int B_OFF = 3 * EP;
    static constexpr int C_OFF = B_OFF + 3 * BP;
    static constexpr int STAGE = C_OFF + CP;
    static constexpr uint32_t TX_BYTES = 3 * E_BYTES + 3 * B_BYTES + C_BYTES;
    static constexpr int SB_OFF = STAGES * STAGE;                    // B^{n+1/2}: [2][3][TY+1][33]
    static constexpr int SB_BYTES = 2 * 3 * (TY + 1) * 33 * 4;
    static constexpr int BAR_OFF = (SB_OFF + SB_BYTES + 127) / 128 * 128;
    static constexpr int SMEM = BAR_OFF + 8 * STAGES;
};

// Warps 0..TY-1 own the tile's cells (warp w = row y0+w, lane = x0+lane). Warp TY is the halo and
// control warp: it issues the TMA copies, waits on the mbarriers (so no other warp ever polls), and
// computes the B^{n+1/2} components of the -y row and -x column that the E update of the tile
// needs (Bx, Bz at (x0+lane, y0-1); By, Bz at (x0-1, y0+lane)).
template <int TY, typename Idx>
__global__ void __launch_bounds__(32 * (TY + 1), TY <= 8 ? 3 : 1)
    yee_tma(const __grid_constant__ CUtensorMap tex, const __grid_constant__ CUtensorMap tey,
            const __grid_constant__ CUtensorMap tez, const __grid_constant__ CUtensorMap tbx,
            const __grid_constant__ CUtensorMap tby, const __grid_constant__ CUtensorMap tbz,
            const __grid_constant__ CUtensorMap tcls, YeeArgs a, unsigned* err) {
    using Lay = Layout<TY, Idx>;
    constexpr int S_ = Lay::STAGES;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + Lay::BAR_OFF);
    float* sB = reinterpret_cast<float*>(smem + Lay::SB_OFF);

    const int lane = threadIdx.x, warp = threadIdx.y;
    const bool ctl = warp == TY;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * TY;
    const int zs = blockIdx.z * a.zchunk;
    const int ze = min(a.nz, zs + a.zchunk);
    if (zs >= ze) return;
    const int zstart = zs > 0 ? zs - 1 : zs;  // a chunk above z = 0 first rebuilds B^{n+1/2}(zs-1)
    const int zlast = ze;                      // planes zstart .. ze are read (ze as the "z+1" plane)

    auto issue = [&](int p) {
        unsigned char* st = smem + ((p - zstart) % S_) * Lay::STAGE;
        uint64_t* bar = bars + (p - zstart) % S_;
        mbar_expect_tx(bar, Lay::TX_BYTES);
        tma_load_3d(st + Lay::E_OFF + 0 * Lay::EP, &tex, x0 - 4, y0 - 1, p, bar);
        tma_load_3d(st + Lay::E_OFF + 1 * Lay::EP, &tey, x0 - 4, y0 - 1, p, bar);
        tma_load_3d(st + Lay::E_OFF + 2 * Lay::EP, &tez, x0 - 4, y0 - 1, p, bar);
        tma_load_3d(st + Lay::B_OFF + 0 * Lay::BP, &tbx, x0 - 4, y0 - 1, p, bar);
        tma_load_3d(st + Lay::B_OFF + 1 * Lay::BP, &tby, x0 - 4, y0 - 1, p, bar);
        tma_load_3d(st + Lay::B_OFF + 2 * Lay::BP, &tbz, x0 - 4, y0 - 1, p, bar);
        tma_load_3d(st + Lay::C_OFF, &tcls, x0 - Lay::CX, y0 - 1, p, bar);
    };
    const bool leader = ctl && lane == 0;
    if (leader) {
        for (int s = 0; s < S_; ++s) mbar_init(bars + s, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    bool failed = false;
    int issued_hi = zstart - 1;  // leader: last plane whose loads were issued
    int waited_ok = zstart - 1;  // leader: last plane whose loads were seen complete
    // on an expired wait: record the error, then give every copy still in flight (the plane that
    // timed out included) a bounded time to land before the CTA leaves and its shared memory goes
    auto bail = [&]() {
        if (leader) {
            atomicOr(err, 1u);
            for (int p = waited_ok + 1; p <= issued_hi; ++p)
                mbar_wait(bars + (p - zstart) % S_, ((p - zstart) / S_) & 1);
        }
    };
    if (leader) {
        for (int p = zstart; p <= zlast && p < zstart + S_; ++p) issue(p), issued_hi = p;
        // planes zstart and zstart+1 before the first B phase; later planes one iteration ahead,
        // just before the per-plane barrier, which passes the TMA writes on to the other warps
        failed = !mbar_wait(bars + 0, 0, a.wait_polls);
        if (!failed) waited_ok = zstart, failed = !mbar_wait(bars + 1, 0, a.wait_polls);
        if (!failed) waited_ok = zstart + 1;
    }
    if (__syncthreads_or(failed)) {
        bail();
        return;
    }

    auto SB = [&](int buf, int c, int r, int col) -> float& { return sB[((buf * 3 + c) * (TY + 1) + r) * 33 + col]; };
    constexpr int EPF = Lay::EP / 4, BPF = Lay::BP / 4;
    const int L = a.L, K = a.pml_K, PS = a.pml_stride;
    const unsigned char* pcls = a.pml_cls;
    const float2* T = a.pml_coef;
    const float dt = a.dt;

    // ---- per-thread invariants of the z march ----
    // own warps: cell (x, y); halo warp: row cell (x0+lane, y0-1) and column cell (x0-1, y0+lane)
    const int x = ctl ? x0 + lane : x0 + lane;
    const int y = ctl ? y0 - 1 : y0 + warp;
    const bool own = !ctl && x < a.nx && y < a.ny;
    const bool row_live = ctl && y0 > 0 && x < a.nx;                        // (x0+lane, y0-1)
    const int cy = y0 + lane;                                               // column cell y
    const bool col_live = ctl && lane < TY && x0 > 0 && cy < a.ny;          // (x0-1, y0+lane)
    auto pml_rows = [&](int px, int py, int& R1, int& R2, int& R3, int& R4) {
        const int ix = __ldg(pcls + px), iy = __ldg(pcls + PS + py), hx = __ldg(pcls + 3 * PS + px),
                  hy = __ldg(pcls + 4 * PS + py);
        R1 = (ix * K + hy) * K, R2 = (hx * K + iy) * K, R3 = (hx * K + hy) * K, R4 = (ix * K + iy) * K;
    };
    auto pml_xy_of = [&](int px, int py) { return px < L || py < L || px >= a.nx - (L + 1) || py >= a.ny - (L + 1); };
    int R1 = 0, R2 = 0, R3 = 0, R4 = 0, C1 = 0, C2 = 0, C3 = 0, C4 = 0;
    if (own || row_live) pml_rows(x, y, R1, R2, R3, R4);
    if (col_live) pml_rows(x0 - 1, cy, C1, C2, C3, C4);
    const bool pml_xy = (own || row_live) && pml_xy_of(x, y);
    const bool pml_xy_c = col_live && pml_xy_of(x0 - 1, cy);
    // shared-memory offsets: own/row cell and column cell (E/B box column 3 = x0-1)
    const int me = (ctl ? 0 : warp + 1) * Lay::EW + lane + 4;
    const int mb = (ctl ? 0 : warp + 1) * Lay::BW + lane + 4;
    const int mc = (ctl ? 0 : warp + 1) * Lay::CW + lane + Lay::CX;
    const int ce = (lane + 1) * Lay::EW + 3, cb = (lane + 1) * Lay::BW + 3, cc = (lane + 1) * Lay::CW + Lay::CX - 1;
    const long long row_off = (long long)y * a.pitch + x;

    float bpx = 0.0f, bpy = 0.0f;  // B^{n+1/2}(x, y, z-1).xy (B below the lower face is 0)
    for (int z = zstart; z < ze; ++z) {
        const int rel = z - zstart;
        const unsigned char* st = smem + (rel % S_) * Lay::STAGE;
        const unsigned char* st1 = smem + ((rel + 1) % S_) * Lay::STAGE;
        const bool emit = z >= zs;
        const int buf = rel & 1;
        const bool pz = __ldg(a.pml_z + z) != 0;
        const int iz = __ldg(pcls + 2 * PS + z), hz = __ldg(pcls + 5 * PS + z);
        const float* Es = reinterpret_cast<const float*>(st + Lay::E_OFF);
        const float* E1 = reinterpret_cast<const float*>(st1 + Lay::E_OFF);
        const float* Bs = reinterpret_cast<const float*>(st + Lay::B_OFF);
        const Idx* Cs = reinterpret_cast<const Idx*>(st + Lay::C_OFF);
        const long long off = (long long)z * a.plane + row_off;
        float bx = 0.0f, by = 0.0f, bz = 0.0f, e0x = 0.0f, e0y = 0.0f, e0z = 0.0f;
        unsigned c = 0;
        if (own) {
            // update_B.comp:35-67 for the own cell
            e0x = Es[me], e0y = Es[EPF + me], e0z = Es[2 * EPF + me];
            bx = Bs[mb], by = Bs[BPF + mb], bz = Bs[2 * BPF + mb];
            c = (unsigned)Cs[mc];
            const float exy = Es[EPF + me + 1], exz = Es[2 * EPF + me + 1];
            const float eyx = Es[me + Lay::EW], eyz = Es[2 * EPF + me + Lay::EW];
            const float ezx = E1[me], ezy = E1[EPF + me];
            float t0x = eyz - e0z, t0y = ezx - e0x, t0z = exy - e0y;
            float t1x = ezy - e0y, t1y = exz - e0z, t1z = eyx - e0x;
            if (c >= a.wire_start) {
                const float4 w0 = __ldg(a.tabW + 2 * c), w1 = __ldg(a.tabW + 2 * c + 1);
                t0x = t0x * w0.x, t0y = t0y * w0.y, t0z = t0z * w0.z;
                t1x = t1x * w0.w, t1y = t1y * w1.x, t1z = t1z * w1.y;
            }
            const float cx = t0x - t1x, cy_ = t0y - t1y, cz = t0z - t1z;
            if (pml_xy || pz) {
                const float2 kx = __ldg(T + R1 + hz), ky = __ldg(T + R2 + hz), kz = __ldg(T + R3 + iz);
                bx = kx.x * bx - kx.y * cx;
                by = ky.x * by - ky.y * cy_;
                bz = kz.x * bz - kz.y * cz;
            } else {
                bx = bx - dt * cx;
                by = by - dt * cy_;
                bz = bz - dt * cz;
            }
            SB(buf, 0, warp + 1, lane + 1) = bx, SB(buf, 1, warp + 1, lane + 1) = by, SB(buf, 2, warp + 1, lane + 1) = bz;
            if (emit) a.nbx[off] = bx, a.nby[off] = by, a.nbz[off] = bz;
        } else if (ctl && emit) {
            // -y row: Bx, Bz at (x0+lane, y0-1) (update_B.comp:41-66, components x and z)
            float hbx = 0.0f, hbz = 0.0f;  // B below the lower faces is 0
            if (row_live) {
                const float f0x = Es[me], f0y = Es[EPF + me], f0z = Es[2 * EPF + me];
                const unsigned hc = (unsigned)Cs[mc];
                float t0x = Es[2 * EPF + me + Lay::EW] - f0z, t1x = E1[EPF + me] - f0y;  // d_y Ez, d_z Ey
                float t0z = Es[EPF + me + 1] - f0y, t1z = Es[me + Lay::EW] - f0x;      // d_x Ey, d_y Ex
                if (hc >= a.wire_start) {
                    const float4 w0 = __ldg(a.tabW + 2 * hc), w1 = __ldg(a.tabW + 2 * hc + 1);
                    t0x = t0x * w0.x, t0z = t0z * w0.z, t1x = t1x * w0.w, t1z = t1z * w1.y;
                }
                const float cx = t0x - t1x, cz = t0z - t1z;
                hbx = Bs[mb], hbz = Bs[2 * BPF + mb];
                if (pml_xy || pz) {
                    const float2 kx = __ldg(T + R1 + hz), kz = __ldg(T + R3 + iz);
                    hbx = kx.x * hbx - kx.y * cx;
                    hbz = kz.x * hbz - kz.y * cz;
                } else {
                    hbx = hbx - dt * cx;
                    hbz = hbz - dt * cz;
                }
            }
            SB(buf, 0, 0, lane + 1) = hbx, SB(buf, 2, 0, lane + 1) = hbz;
            // -x column: By, Bz at (x0-1, y0+lane)
            if (lane < TY) {
                float hby = 0.0f, hbz2 = 0.0f;
                if (col_live) {
                    const float f0x = Es[ce], f0y = Es[EPF + ce], f0z = Es[2 * EPF + ce];
                    const unsigned hc = (unsigned)Cs[cc];
                    float t0y = E1[ce] - f0x, t1y = Es[2 * EPF + ce + 1] - f0z;   // d_z Ex, d_x Ez
                    float t0z = Es[EPF + ce + 1] - f0y, t1z = Es[ce + Lay::EW] - f0x;  // d_x Ey, d_y Ex
                    if (hc >= a.wire_start) {
                        const float4 w0 = __ldg(a.tabW + 2 * hc), w1 = __ldg(a.tabW + 2 * hc + 1);
                        t0y = t0y * w0.y, t0z = t0z * w0.z, t1y = t1y * w1.x, t1z = t1z * w1.y;
                    }
                    const float cyy = t0y - t1y, cz = t0z - t1z;
                    hby = Bs[BPF + cb], hbz2 = Bs[2 * BPF + cb];
                    if (pml_xy_c || pz) {
                        const float2 ky = __ldg(T + C2 + hz), kz = __ldg(T + C3 + iz);
                        hby = ky.x * hby - ky.y * cyy;
                        hbz2 = kz.x * hbz2 - kz.y * cz;
                    } else {
                        hby = hby - dt * cyy;
                        hbz2 = hbz2 - dt * cz;
                    }
                }
                SB(buf, 1, lane + 1, 0) = hby, SB(buf, 2, lane + 1, 0) = hbz2;
            }
        }
        // the next iteration's B phase reads plane z+2: the leader waits for it before the barrier
        if (leader && z + 1 < ze) {
            failed = !mbar_wait(bars + (rel + 2) % S_, ((rel + 2) / S_) & 1, a.wait_polls);
            if (!failed) waited_ok = z + 2;
        }
        if (__syncthreads_or(failed)) {
            bail();
            return;
        }
        // every warp is past its reads of plane z-1's stage: refill it with plane z-1+STAGES
        if (leader && z > zstart && z - 1 + S_ <= zlast) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(z - 1 + S_);
            issued_hi = z - 1 + S_;
        }
        if (emit && own) {
            // update_E.comp:41-64 for the own cell
            const float bxm_y = SB(buf, 1, warp + 1, lane), bxm_z = SB(buf, 2, warp + 1, lane);  // B(x-1)
            const float bym_x = SB(buf, 0, warp, lane + 1), bym_z = SB(buf, 2, warp, lane + 1);  // B(y-1)
            const float cx = (bz - bym_z) - (by - bpy);
            const float cy_ = (bx - bpx) - (bz - bxm_z);
            const float cz = (by - bxm_y) - (bx - bym_x);
            float ex = e0x, ey = e0y, ez = e0z;
            if (!(pml_xy || pz)) {
                if (c == 0) {  // vacuum: ca = 1 and cb = dt exactly, so 1 * e + dt * curl == e + dt * curl
                    ex = ex + dt * cx;
                    ey = ey + dt * cy_;
                    ez = ez + dt * cz;
                } else {
                    const float4 t0 = __ldg(a.tabE + 2 * c), t1 = __ldg(a.tabE + 2 * c + 1);
                    ex = t0.x * ex + t0.w * cx;
                    ey = t0.y * ey + t1.x * cy_;
                    ez = t0.z * ez + t1.y * cz;
                }
            } else if (c == 0) {
                const float2 kx = __ldg(T + R2 + iz), ky = __ldg(T + R1 + iz), kz = __ldg(T + R4 + hz);
                ex = kx.x * ex + kx.y * cx;
                ey = ky.x * ey + ky.y * cy_;
                ez = kz.x * ez + kz.y * cz;
            } else {
                e_cell(a, ex, ey, ez, cx, cy_, cz, c, x, y, z);
            }
            a.nex[off] = ex, a.ney[off] = ey, a.nez[off] = ez;
        }
        bpx = bx, bpy = by;
    }
}

// ------------------------------------------------------------------------------------------------
// Two cells per thread along x: a CTA owns a 64 x TY tile (warp w = row y0+w, lane l = cells
// x0+2l and x0+2l+1) and moves pairs with 64-bit shared and global accesses, so the per-plane
// bookkeeping and most address arithmetic are paid once per two cells. Same arithmetic per cell.
template <int TY, typename Idx>
struct Layout2 {
    static constexpr int STAGES = TY == 8 ? 4 : 5;
    static constexpr int W = 72;                        // box row width of E, B and the class index
    static constexpr int CX = sizeof(Idx) == 2 ? 8 : 4;  // boxes start at x0 - 4 (16-bit class: x0 - 8)
    static constexpr int DC = CX - 4;                   // class element offset from the E/B element
    static constexpr int E_BYTES = W * (TY + 2) * 4;    // rows y0-1 .. y0+TY
    static constexpr int B_BYTES = W * (TY + 1) * 4;    // rows y0-1 .. y0+TY-1
    static constexpr int C_BYTES = W * (TY + 1) * (int)sizeof(Idx);
    static constexpr int EP = (E_BYTES + 127) / 128 * 128;
    static constexpr int BP = (B_BYTES + 127) / 128 * 128;
    static constexpr int CP = (C_BYTES + 127) / 128 * 128;
    static constexpr int E_OFF = 0;
    static constexpr int B_OFF = 3 * EP;
    static constexpr int C_OFF = B_OFF + 3 * BP;
    static constexpr int STAGE = C_OFF + CP;
    static constexpr uint32_t TX_BYTES = 3 * E_BYTES + 3 * B_BYTES + C_BYTES;
    // B tile row: element e of a box row maps to slot e - 2 (col 1 = x0-1, col 2+i = x0+i)
    static constexpr int SB_OFF = STAGES * STAGE;
    static constexpr int SB_BYTES = 2 * 3 * (TY + 1) * W * 4;
    static constexpr int BAR_OFF = (SB_OFF + SB_BYTES + 127) / 128 * 128;
    static constexpr int PROD_OFF = BAR_OFF + 8 * STAGES;           // producer cursor (leader only)
    static constexpr int QUEUE_OFF = PROD_OFF + 8 * 4;               // item numbers [8], -1 = done
    static constexpr int COL_OFF = (QUEUE_OFF + 8 * 4 + 15) / 16 * 16;  // column-halo rows, int4 [TY]
    static constexpr int SMEM = COL_OFF + TY * 16;
    static_assert(COL_OFF % 16 == 0 && BAR_OFF % 8 == 0 && SB_OFF % 16 == 0, "shared-memory alignment");
    static_assert(SMEM <= 227 * 1024, "shared memory per CTA");
};

// The next field generation is not read again in the launch: its stores leave L2 first, so the
// current generation's planes stay for the neighbouring tiles' halo reads. The policy is made at
// each use (one instruction) rather than held in a register across the z march.
__device__ __forceinline__ uint64_t evict_first_policy() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ void st_pair(float* p, float2 v, uint64_t policy) {
    asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(v.x), "f"(v.y), "l"(policy)
                 : "memory");
}
__device__ __forceinline__ void st_one(float* p, float v, uint64_t policy) {
    asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(p), "f"(v), "l"(policy) : "memory");
}

template <typename Idx>
__device__ __forceinline__ void load_class_pair(const Idx* p, unsigned& a, unsigned& b);
template <>
__device__ __forceinline__ void load_class_pair<uint16_t>(const uint16_t* p, unsigned& a, unsigned& b) {
    const unsigned v = *reinterpret_cast<const unsigned*>(p);
    a = v & 0xffffu, b = v >> 16;
}
template <>
__device__ __forceinline__ void load_class_pair<uint32_t>(const uint32_t* p, unsigned& a, unsigned& b) {
    const uint2 v = *reinterpret_cast<const uint2*>(p);
    a = v.x, b = v.y;
}

// B^{n+1/2} of one cell outside/inside the absorber from its curl terms (update_B.comp:47-67).
__device__ __forceinline__ void b_update(const YeeArgs& a, float& bx, float& by, float& bz, float t0x, float t0y,
                                         float t0z, float t1x, float t1y, float t1z, unsigned c, bool inp, int R1,
                                         int R2, int R3, int iz, int hz) {
    if (c >= a.wire_start) {
        const float4 w0 = __ldg(a.tabW + 2 * c), w1 = __ldg(a.tabW + 2 * c + 1);
        t0x = t0x * w0.x, t0y = t0y * w0.y, t0z = t0z * w0.z;
        t1x = t1x * w0.w, t1y = t1y * w1.x, t1z = t1z * w1.y;
    }
    const float cx = t0x - t1x, cy = t0y - t1y, cz = t0z - t1z;
    if (inp) {
        const float2 kx = __ldg(a.pml_coef + R1 + hz), ky = __ldg(a.pml_coef + R2 + hz),
                     kz = __ldg(a.pml_coef + R3 + iz);
        bx = kx.x * bx - kx.y * cx;
        by = ky.x * by - ky.y * cy;
        bz = kz.x * bz - kz.y * cz;
    } else {
        const float dt = a.dt;
        bx = bx - dt * cx;
        by = by - dt * cy;
        bz = bz - dt * cz;
    }
}

// E^{n+1} of one cell from its curl (update_E.comp:41-64).
__device__ __forceinline__ void e_update(const YeeArgs& a, float& ex, float& ey, float& ez, float cx, float cy,
                                         float cz, unsigned c, bool inp, int R1, int R2, int R4, int iz, int hz, int x,
                                         int y, int z, int scene) {
    if (!inp) {
        if (c == 0) {  // vacuum: ca = 1 and cb = dt exactly, so 1 * e + dt * curl == e + dt * curl
            const float dt = a.dt;
            ex = ex + dt * cx;
            ey = ey + dt * cy;
            ez = ez + dt * cz;
        } else {
            const float4 t0 = __ldg(a.tabE + 2 * c), t1 = __ldg(a.tabE + 2 * c + 1);
            ex = t0.x * ex + t0.w * cx;
            ey = t0.y * ey + t1.x * cy;
            ez = t0.z * ez + t1.y * cz;
        }
    } else if (c == 0) {
        const float2 kx = __ldg(a.pml_coef + R2 + iz), ky = __ldg(a.pml_coef + R1 + iz),
                     kz = __ldg(a.pml_coef + R4 + hz);
        ex = kx.x * ex + kx.y * cx;
        ey = ky.x * ey + ky.y * cy;
        ez = kz.x * ez + kz.y * cz;
    } else {
        // a non-vacuum edge material inside the absorber (update_E.comp:51-64), the x / y profiles
        // those of the cell's scene: e_cell's arithmetic
        const float4 m0 = __ldg(a.tabM + 2 * c), m1 = __ldg(a.tabM + 2 * c + 1);
        const float* pxy = a.pml_xy + (long long)scene * a.pml_xy_scene;
        const int SX = a.pml_xy_stride, S = a.pml_stride;
        const float ix = __ldg(pxy + x), iy = __ldg(pxy + SX + y), izv = __ldg(a.pml + 2 * S + z);
        const float hx = __ldg(pxy + 3 * SX + x), hy = __ldg(pxy + 4 * SX + y), hzv = __ldg(a.pml + 5 * S + z);
        ex = e_pml(ex, cx, m0.x + ((hx + iy) + izv), m0.w, a.dt);
        ey = e_pml(ey, cy, m0.y + ((ix + hy) + izv), m1.x, a.dt);
        ez = e_pml(ez, cz, m0.z + ((ix + iy) + hzv), m1.y, a.dt);
    }
}

// Dynamic schedule of the persistent pair kernel: work items are (z chunk, tile) pairs, chunk-major,
// handed out in order by a ticket counter. Items in progress at any moment are a window of
// consecutive tiles at nearly the same z, so the halos that neighbouring tiles share are L2 hits;
// a static assignment lets slow CTAs (absorber columns) drift planes apart from their neighbours.
// The counter is never reset: launch n consumes exactly items + G tickets (every CTA's last grab
// fails), and the host passes the sum over earlier launches as `base`. After a launch that stopped
// early the counter lags; tickets below the base are skipped.
struct PairSched {
    int tiles_x;  // 64-cell tiles along x
    int tiles;    // tiles per z chunk
    int items;    // tiles * z chunks
    int zc;       // planes per z chunk
    unsigned long long* work;
    unsigned long long base;
    const int4* tab;  // a stack of scenes with their own cross-sections: the items themselves
};

struct PairItem {
    int x0, y0, zs, ze, zstart, scene;
};

template <int TY>
__device__ __forceinline__ PairItem pair_item(const PairSched& ps, int nz, int item) {
    PairItem it;
    if (ps.tab) {
        const int4 t = __ldg(ps.tab + item);
        it.x0 = t.x & 0xffff, it.y0 = (int)((unsigned)t.x >> 16), it.zs = t.y, it.ze = t.z, it.scene = t.w;
    } else {
        const int c = item / ps.tiles, t = item - c * ps.tiles;
        it.x0 = (t % ps.tiles_x) * 64;
        it.y0 = (t / ps.tiles_x) * TY;
        it.zs = c * ps.zc;
        it.ze = min(nz, it.zs + ps.zc);
        it.scene = 0;
    }
    it.zstart = it.zs > 0 ? it.zs - 1 : 0;  // a chunk above z = 0 first rebuilds B^{n+1/2}(zs-1)
    return it;
}

// The CTA's loads form one sequence over its items: for each item, planes zstart .. ze (plane ze
// is read as the "z+1" neighbour of the last plane; ze = nz reads TMA zeros). Load j goes to ring
// stage j % STAGES and completes phase (j / STAGES) & 1 of that stage's mbarrier. The ring runs
// on across item boundaries, so the pipeline never drains inside a launch. The leader takes the
// next item when its loads reach it and posts the item number in a small shared ring that the
// other warps read at their item boundary (always at least one barrier later).
// 64 x 4 tiles: four 160-thread CTAs per SM; 64 x 8: two 288-thread CTAs; 64 x 16: one 544-thread
// CTA. Registers are allocated per SM quadrant and 17-20 warps put 5 warps on one quadrant: 96
// registers at most.
template <int TY, typename Idx>
__global__ void __launch_bounds__(32 * (TY + 1), TY == 4 ? 4 : (TY == 8 ? 2 : 1))
    yee_tma2(const __grid_constant__ CUtensorMap tex, const __grid_constant__ CUtensorMap tey,
             const __grid_constant__ CUtensorMap tez, const __grid_constant__ CUtensorMap tbx,
             const __grid_constant__ CUtensorMap tby, const __grid_constant__ CUtensorMap tbz,
             const __grid_constant__ CUtensorMap tcls, YeeArgs a, PairSched ps, unsigned* err) {
    static_assert(TY == 4 || TY == 8 || TY == 16, "register budget assumes 5, 9 or 17 warps per CTA");
    using Lay = Layout2<TY, Idx>;
    constexpr int S_ = Lay::STAGES;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + Lay::BAR_OFF);
    float* sB = reinterpret_cast<float*>(smem + Lay::SB_OFF);
    // producer cursor: item, x0, y0, z, zend, issued, waited, item ordinal
    int* prod = reinterpret_cast<int*>(smem + Lay::PROD_OFF);
    int* queue = reinterpret_cast<int*>(smem + Lay::QUEUE_OFF);  // item of ordinal n at [n & 7]
    int4* colrow = reinterpret_cast<int4*>(smem + Lay::COL_OFF);

    const int lane = threadIdx.x, warp = threadIdx.y;
    const bool ctl = warp == TY;
    const bool leader = ctl && lane == 0;

    // ---- producer (leader thread): cursor over the load sequence, kept in shared memory ----
    auto grab = [&]() -> int {  // next work item, or -1 when all are taken
        for (;;) {
            const unsigned long long t = atomicAdd(ps.work, 1ull);
            if (t < ps.base) continue;  // left over from a launch that stopped early
            return t - ps.base < (unsigned long long)ps.items ? (int)(t - ps.base) : -1;
        }
    };
    auto p_seek = [&]() {
        if (prod[0] >= 0) {
            const PairItem it = pair_item<TY>(ps, a.nz, prod[0]);
            prod[1] = it.x0, prod[2] = it.y0, prod[3] = it.zstart, prod[4] = it.ze;
        }
    };
    auto issue_upto = [&](int last) {  // issue loads up to index `last` while the sequence lasts
        int issued = prod[5];
        while (issued <= last && prod[0] >= 0) {
            unsigned char* st = smem + (issued % S_) * Lay::STAGE;
            uint64_t* bar = bars + issued % S_;
            const int px = prod[1] - 4, py = prod[2] - 1, pz = prod[3];
            mbar_expect_tx(bar, Lay::TX_BYTES);
            tma_load_3d(st + Lay::E_OFF + 0 * Lay::EP, &tex, px, py, pz, bar);
            tma_load_3d(st + Lay::E_OFF + 1 * Lay::EP, &tey, px, py, pz, bar);
            tma_load_3d(st + Lay::E_OFF + 2 * Lay::EP, &tez, px, py, pz, bar);
            tma_load_3d(st + Lay::B_OFF + 0 * Lay::BP, &tbx, px, py, pz, bar);
            tma_load_3d(st + Lay::B_OFF + 1 * Lay::BP, &tby, px, py, pz, bar);
            tma_load_3d(st + Lay::B_OFF + 2 * Lay::BP, &tbz, px, py, pz, bar);
            tma_load_3d(st + Lay::C_OFF, &tcls, px - Lay::DC, py, pz, bar);
            ++issued;
            if (++prod[3] > prod[4]) {  // item complete: take the next one and post it
                prod[0] = grab();
                queue[++prod[7] & 7] = prod[0];
                p_seek();
            }
        }
        prod[5] = issued;
    };
    auto wait_upto = [&](int last) {  // false if a load did not complete within the bound
        int waited = prod[6];
        bool ok = true;
        while (ok && waited < last) {
            ++waited;
            ok = mbar_wait(bars + waited % S_, (waited / S_) & 1, a.wait_polls);
        }
        prod[6] = waited;
        return ok;
    };
    // on an expired wait: record the error, then give every copy still in flight a bounded time to
    // land before the CTA leaves and its shared memory goes. prod[6] is the load whose wait ran out
    // (not complete), prod[5] - 1 the last load issued.
    auto bail = [&]() {
        if (leader) {
            atomicOr(err, 1u);
            for (int w = prod[6] < 0 ? 0 : prod[6]; w < prod[5]; ++w) mbar_wait(bars + w % S_, (w / S_) & 1);
        }
    };

    if (leader) {
        for (int s = 0; s < S_; ++s) mbar_init(bars + s, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        prod[0] = grab(), prod[5] = 0, prod[6] = -1, prod[7] = 0;
        queue[0] = prod[0];
    }
    __syncthreads();
    if (queue[0] < 0) return;  // uniform: no work for this CTA
    bool failed = false;
    if (leader) {
        p_seek();
        issue_upto(S_ - 1);
        failed = !wait_upto(1);  // the first iteration reads loads 0 and 1
    }
    if (__syncthreads_or(failed)) {
        bail();
        return;
    }

    constexpr int EPF = Lay::EP / 4, BPF = Lay::BP / 4, W = Lay::W, SBC = (TY + 1) * W;
    const int L = a.L, K = a.pml_K, PS = a.pml_stride;
    const unsigned char* pcls = a.pml_cls;
    // box element of the own / halo-row pair (E, B and 32-bit class boxes share it; the 16-bit class
    // box is DC elements further) and of the column cell (x0-1, y0+lane); B tile slot = element - 2
    const int me = (ctl ? 0 : warp + 1) * W + 2 * lane + 4;
    const int ce = (lane + 1) * W + 3;
    const int SX = a.pml_xy_stride;
    // x / y depth classes from the item's scene's table (pcx), z from the grid's
    auto pml_rows = [&](const unsigned char* pcx, int px, int py, int& R1, int& R2, int& R3, int& R4) {
        const int ix = __ldg(pcx + px), iy = __ldg(pcx + SX + py), hx = __ldg(pcx + 3 * SX + px),
                  hy = __ldg(pcx + 4 * SX + py);
        R1 = (ix * K + hy) * K, R2 = (hx * K + iy) * K, R3 = (hx * K + hy) * K, R4 = (ix * K + iy) * K;
    };

    int k = 0;     // load index of the current iteration's plane z
    int iter = 0;  // iteration counter: parity selects the B tile buffer
    for (int ord = 0, item = queue[0]; item >= 0; item = queue[++ord & 7]) {
        const PairItem itm = pair_item<TY>(ps, a.nz, item);
        const int x0 = itm.x0, y0 = itm.y0, zs = itm.zs, ze = itm.ze, scene = itm.scene;
        // the absorber of the item's scene (common.glsl:40-43 with the scene's own nx, ny)
        const unsigned char* pcx = a.pml_cls_xy + (long long)scene * a.pml_xy_scene;
        int snx = a.nx, sny = a.ny;
        if (a.scene_xy) {
            const int2 d = __ldg(a.scene_xy + scene);
            snx = d.x, sny = d.y;
        }
        auto pml_xy_of = [&](int px, int py) { return px < L || py < L || px >= snx - (L + 1) || py >= sny - (L + 1); };

        // per-item invariants: own warps hold cells (xa, y), (xa+1, y); the halo warp holds the row
        // cells (xa, y0-1), (xa+1, y0-1) and the column cell (x0-1, y0+lane)
        // cells outside the item's scene (a ragged stack's frozen cells) are neither updated nor
        // written: they keep their initial 0 in both field generations
        const int xa = x0 + 2 * lane;
        const int y = ctl ? y0 - 1 : y0 + warp;
        const bool rowok = ctl ? y0 > 0 : y < sny;
        const bool o0 = rowok && xa < snx, o1 = rowok && xa + 1 < snx;
        int A1 = 0, A2 = 0, A3 = 0, A4 = 0, B1 = 0, B2 = 0, B3 = 0, B4 = 0;
        if (o0) pml_rows(pcx, xa, y, A1, A2, A3, A4);
        if (o1) pml_rows(pcx, xa + 1, y, B1, B2, B3, B4);
        const bool pxy0 = o0 && pml_xy_of(xa, y), pxy1 = o1 && pml_xy_of(xa + 1, y);
        if (ctl && lane < TY) {  // column cell: live flag | absorber flag, then its table rows
            const int cy = y0 + lane;
            int4 cr = make_int4(0, 0, 0, 0);
            if (x0 > 0 && cy < sny) {
                int r4;
                pml_rows(pcx, x0 - 1, cy, cr.y, cr.z, cr.w, r4);
                cr.x = 1 | (pml_xy_of(x0 - 1, cy) ? 2 : 0);
            }
            colrow[lane] = cr;  // read by the same thread only
        }
        const long long row_off = (long long)y * a.pitch + xa;

        float2 bp_x = make_float2(0.0f, 0.0f), bp_y = bp_x;  // B^{n+1/2}(z-1).x, .y of the pair
        int iz = __ldg(pcls + 2 * PS + itm.zstart), hz = __ldg(pcls + 5 * PS + itm.zstart);
        for (int z = itm.zstart; z < ze; ++z, ++k, ++iter) {
            const unsigned char* st = smem + (k % S_) * Lay::STAGE;
            const unsigned char* st1 = smem + ((k + 1) % S_) * Lay::STAGE;
            const bool emit = z >= zs;
            float* sb = sB + (iter & 1) * 3 * SBC - 2;  // indexed by box element
            const bool pz = __ldg(a.pml_z + z) != 0;
            const int zn = min(z + 1, a.nz - 1);
            const int iz_n = __ldg(pcls + 2 * PS + zn), hz_n = __ldg(pcls + 5 * PS + zn);
            const float* Es = reinterpret_cast<const float*>(st + Lay::E_OFF);
            const float* E1 = reinterpret_cast<const float*>(st1 + Lay::E_OFF);
            const float* Bs = reinterpret_cast<const float*>(st + Lay::B_OFF);
            const Idx* Cs = reinterpret_cast<const Idx*>(st + Lay::C_OFF) + Lay::DC;
            const long long off = (long long)z * a.plane + row_off;
            float2 e0x = make_float2(0.0f, 0.0f), e0y = e0x, e0z = e0x, bx = e0x, by = e0x, bz = e0x;
            unsigned ca = 0, cb = 0;
            if (!ctl) {
                // update_B.comp:35-67 for both cells (halo values beyond the grid are TMA zeros)
                e0x = *reinterpret_cast<const float2*>(Es + me);
                e0y = *reinterpret_cast<const float2*>(Es + EPF + me);
                e0z = *reinterpret_cast<const float2*>(Es + 2 * EPF + me);
                bx = *reinterpret_cast<const float2*>(Bs + me);
                by = *reinterpret_cast<const float2*>(Bs + BPF + me);
                bz = *reinterpret_cast<const float2*>(Bs + 2 * BPF + me);
                load_class_pair<Idx>(Cs + me, ca, cb);
                const float e2y = Es[EPF + me + 2], e2z = Es[2 * EPF + me + 2];          // E(xa+2)
                const float2 eyx = *reinterpret_cast<const float2*>(Es + me + W);         // E(y+1)
                const float2 eyz = *reinterpret_cast<const float2*>(Es + 2 * EPF + me + W);
                const float2 ezx = *reinterpret_cast<const float2*>(E1 + me);            // E(z+1)
                const float2 ezy = *reinterpret_cast<const float2*>(E1 + EPF + me);
                b_update(a, bx.x, by.x, bz.x, eyz.x - e0z.x, ezx.x - e0x.x, e0y.y - e0y.x, ezy.x - e0y.x,
                         e0z.y - e0z.x, eyx.x - e0x.x, ca, pxy0 || pz, A1, A2, A3, iz, hz);
                b_update(a, bx.y, by.y, bz.y, eyz.y - e0z.y, ezx.y - e0x.y, e2y - e0y.y, ezy.y - e0y.y, e2z - e0z.y,
                         eyx.y - e0x.y, cb, pxy1 || pz, B1, B2, B3, iz, hz);
                *reinterpret_cast<float2*>(sb + me) = bx;
                *reinterpret_cast<float2*>(sb + SBC + me) = by;
                *reinterpret_cast<float2*>(sb + 2 * SBC + me) = bz;
                if (emit) {
                    const uint64_t evict_first = evict_first_policy();
                    if (o1) {
                        st_pair(a.nbx + off, bx, evict_first);
                        st_pair(a.nby + off, by, evict_first);
                        st_pair(a.nbz + off, bz, evict_first);
                    } else if (o0) {
                        st_one(a.nbx + off, bx.x, evict_first);
                        st_one(a.nby + off, by.x, evict_first);
                        st_one(a.nbz + off, bz.x, evict_first);
                    }
                }
            } else if (emit) {
                // -y row: Bx, Bz of (xa, y0-1) and (xa+1, y0-1); B below the lower faces is 0
                float2 hx2 = make_float2(0.0f, 0.0f), hz2 = hx2;
                if (o0) {
                    const float2 f0x = *reinterpret_cast<const float2*>(Es + me);
                    const float2 f0y = *reinterpret_cast<const float2*>(Es + EPF + me);
                    const float2 f0z = *reinterpret_cast<const float2*>(Es + 2 * EPF + me);
                    const float e2y = Es[EPF + me + 2];
                    const float2 eyx = *reinterpret_cast<const float2*>(Es + me + W);
                    const float2 eyz = *reinterpret_cast<const float2*>(Es + 2 * EPF + me + W);
                    const float2 ezy = *reinterpret_cast<const float2*>(E1 + EPF + me);
                    unsigned ha, hb;
                    load_class_pair<Idx>(Cs + me, ha, hb);
                    hx2 = *reinterpret_cast<const float2*>(Bs + me);
                    hz2 = *reinterpret_cast<const float2*>(Bs + 2 * BPF + me);
                    float unused0 = 0.0f, unused1 = 0.0f;
                    b_update(a, hx2.x, unused0, hz2.x, eyz.x - f0z.x, 0.0f, f0y.y - f0y.x, ezy.x - f0y.x, 0.0f,
                             eyx.x - f0x.x, ha, pxy0 || pz, A1, A2, A3, iz, hz);
                    if (o1)
                        b_update(a, hx2.y, unused1, hz2.y, eyz.y - f0z.y, 0.0f, e2y - f0y.y, ezy.y - f0y.y, 0.0f,
                                 eyx.y - f0x.y, hb, pxy1 || pz, B1, B2, B3, iz, hz);
                    else
                        hx2.y = 0.0f, hz2.y = 0.0f;
                }
                *reinterpret_cast<float2*>(sb + me) = hx2;
                *reinterpret_cast<float2*>(sb + 2 * SBC + me) = hz2;
                // -x column: By, Bz of (x0-1, y0+lane)
                if (lane < TY) {
                    float hby = 0.0f, hbz = 0.0f, hbx = 0.0f;
                    const int4 cr = colrow[lane];
                    if (cr.x & 1) {
                        const float f0x = Es[ce], f0y = Es[EPF + ce], f0z = Es[2 * EPF + ce];
                        hby = Bs[BPF + ce], hbz = Bs[2 * BPF + ce];
                        b_update(a, hbx, hby, hbz, 0.0f, E1[ce] - f0x, Es[EPF + ce + 1] - f0y, 0.0f,
                                 Es[2 * EPF + ce + 1] - f0z, Es[ce + W] - f0x, (unsigned)Cs[ce], (cr.x & 2) || pz,
                                 cr.y, cr.z, cr.w, iz, hz);
                    }
                    sb[SBC + ce] = hby;
                    sb[2 * SBC + ce] = hbz;
                }
            }
            // the next iteration reads loads k+1, k+2 (or k+2, k+3 at the start of the next item)
            if (leader) {  // at the last plane the next item was taken when its first load was issued
                const int need = z + 1 < ze ? k + 2 : (queue[(ord + 1) & 7] < 0 ? -1 : k + 3);
                if (need >= 0) failed = !wait_upto(need);
            }
            if (__syncthreads_or(failed)) {
                bail();
                return;
            }
            // every warp is past its reads of loads <= k: refill up to k + STAGES
            if (leader) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue_upto(k + S_);
            }
            if (emit && !ctl && o0) {
                // update_E.comp:41-64 for both cells
                const float bxm_y = sb[SBC + me - 1], bxm_z = sb[2 * SBC + me - 1];             // B(xa-1).y, .z
                const float2 bym_x = *reinterpret_cast<const float2*>(sb + me - W);            // B(y-1).x
                const float2 bym_z = *reinterpret_cast<const float2*>(sb + 2 * SBC + me - W);  // B(y-1).z
                float2 ex = e0x, ey = e0y, ez = e0z;
                e_update(a, ex.x, ey.x, ez.x, (bz.x - bym_z.x) - (by.x - bp_y.x), (bx.x - bp_x.x) - (bz.x - bxm_z),
                         (by.x - bxm_y) - (bx.x - bym_x.x), ca, pxy0 || pz, A1, A2, A4, iz, hz, xa, y, z, scene);
                e_update(a, ex.y, ey.y, ez.y, (bz.y - bym_z.y) - (by.y - bp_y.y), (bx.y - bp_x.y) - (bz.y - bz.x),
                         (by.y - by.x) - (bx.y - bym_x.y), cb, pxy1 || pz, B1, B2, B4, iz, hz, xa + 1, y, z, scene);
                const uint64_t evict_first = evict_first_policy();
                if (o1) {
                    st_pair(a.nex + off, ex, evict_first);
                    st_pair(a.ney + off, ey, evict_first);
                    st_pair(a.nez + off, ez, evict_first);
                } else {
                    st_one(a.nex + off, ex.x, evict_first);
                    st_one(a.ney + off, ey.x, evict_first);
                    st_one(a.nez + off, ez.x, evict_first);
                }
            }
            bp_x = bx, bp_y = by;
            iz = iz_n, hz = hz_n;
        }
        ++k;  // the item's last load (plane ze) was only read as the z+1 neighbour
    }
}

using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encode_fn() {
    static const EncodeFn fn = [] {  // initialised once, thread-safe
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<EncodeFn>(p);
        return (EncodeFn) nullptr;
    }();
    return fn;
}

std::mutex g_launch_setup;  // the launchers' one-time attribute set-up (grids may step from several threads)

bool encode(CUtensorMap* m, CUtensorMapDataType type, int elem, const void* base, const YeeArgs& a, int box_w,
            int box_h) {
    EncodeFn fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)a.nx, (cuuint64_t)a.ny, (cuuint64_t)a.nz};
    const cuuint64_t strides[2] = {(cuuint64_t)a.pitch * elem, (cuuint64_t)a.plane * elem};
    const cuuint32_t box[3] = {(cuuint32_t)box_w, (cuuint32_t)box_h, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return fn(m, type, 3, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// tiling modes: 8, 16 = 32 x TY tiles of single cells (yee_tma); 64, 128 = 64 x 8 and 64 x 16 tiles
// of cell pairs (yee_tma2)
int tile_rows(const YeeArgs& a) { return a.tile_rows == 16 || a.tile_rows == 128 ? 16 : (a.tile_rows == 32 ? 4 : 8); }
bool pair_tiles(const YeeArgs& a) { return a.tile_rows == 32 || a.tile_rows == 64 || a.tile_rows == 128; }

template <int TY, typename Idx>
bool launch_t(const YeeArgs& a, const TmaMaps* m, int gen, unsigned* err, cudaStream_t s) {
    using Lay = Layout<TY, Idx>;
    static bool configured = false;
    {
        std::lock_guard<std::mutex> lk(g_launch_setup);
        if (!configured) {
            if (cudaFuncSetAttribute(yee_tma<TY, Idx>, cudaFuncAttributeMaxDynamicSharedMemorySize, Lay::SMEM) !=
                cudaSuccess)
                return false;
            configured = true;
        }
    }
    const dim3 grid((a.nx + 31) / 32, (a.ny + TY - 1) / TY, (a.nz + a.zchunk - 1) / a.zchunk);
    yee_tma<TY, Idx><<<grid, dim3(32, TY + 1), Lay::SMEM, s>>>(m->e[gen][0], m->e[gen][1], m->e[gen][2], m->b[gen][0],
                                                           m->b[gen][1], m->b[gen][2], m->cls, a, err);
    return true;
}

// Chooses the z chunk length of the persistent schedule: the CTA with the most items bounds the
// launch, and every chunk above z = 0 re-reads one plane, so minimise ceil(items / G) * (zc + 1).
// Items differ in cost (a tile with absorber or material cells takes longer per plane), and the
// ticket schedule evens them out only when every CTA takes several: the chunk length is chosen among
// those giving at least kItemsPerCta items per CTA, as far as chunks of kMinBalancedPlanes planes
// allow (shorter chunks would re-read too many planes: every chunk above z = 0 re-reads one).
constexpr int kItemsPerCta = 4;
constexpr int kMinBalancedPlanes = 16;

PairSched pair_schedule(const YeeArgs& a, int TY, int G) {
    PairSched ps;
    ps.tiles_x = (a.nx + 63) / 64;
    ps.tiles = ps.tiles_x * ((a.ny + TY - 1) / TY);
    const int max_chunks = std::max(1, a.nz / 4);
    const long long want = std::min((long long)kItemsPerCta * G,
                                    (long long)std::max(1, a.nz / kMinBalancedPlanes) * ps.tiles);
    long long best = -1;
    for (int chunks = 1; chunks <= max_chunks; ++chunks) {
        const int zc = (a.nz + chunks - 1) / chunks;
        const int n = (a.nz + zc - 1) / zc;
        const long long items = (long long)n * ps.tiles;
        if (items < want) continue;
        const long long cost = (items + G - 1) / G * (zc + (n > 1 ? 1 : 0));
        if (best < 0 || cost < best) best = cost, ps.zc = zc, ps.items = (int)items;
    }
    if (best < 0) {  // no chunk count reaches `want` exactly (zc rounding): the finest split
        ps.zc = (a.nz + max_chunks - 1) / max_chunks;
        ps.items = (int)((long long)((a.nz + ps.zc - 1) / ps.zc) * ps.tiles);
    }
    return ps;
}

template <int TY, typename Idx>
bool launch_p(const YeeArgs& a, const TmaMaps* m, int gen, unsigned* err, cudaStream_t s,
              unsigned long long* tickets) {
    using Lay = Layout2<TY, Idx>;
    static int resident = 0, sms = 0;  // per process: one device model
    std::unique_lock<std::mutex> lk(g_launch_setup);
    if (!resident) {
        int dev = 0, smem_sm = 0;
        // shared-memory carveout for exactly the CTAs wanted per SM (two 64 x 8 or one 64 x 16): the
        // rest of the SM's 256 KB stays L1, which caches the per-class and absorber tables
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
            smem_sm <= 0 ||
            cudaFuncSetAttribute(yee_tma2<TY, Idx>, cudaFuncAttributeMaxDynamicSharedMemorySize, Lay::SMEM) !=
                cudaSuccess ||
            cudaFuncSetAttribute(yee_tma2<TY, Idx>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 std::min(100, (100 * (TY == 4 ? 4 : (TY == 8 ? 2 : 1)) * (Lay::SMEM + 1024) +
                                                smem_sm - 1) / smem_sm)) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, yee_tma2<TY, Idx>, 32 * (TY + 1), Lay::SMEM) !=
                cudaSuccess ||
            resident < 1) {
            resident = 0;
            return false;
        }
    }
    lk.unlock();
    PairSched ps{};
    if (a.items) {
        ps.items = a.n_items;
        ps.tab = a.items;
    } else {
        ps = pair_schedule(a, TY, resident * sms);
        ps.tab = nullptr;
    }
    if (ps.items <= 0) return false;
    const int grid = std::min(ps.items, resident * sms);
    ps.work = a.work, ps.base = a.work_base;
    yee_tma2<TY, Idx><<<grid, dim3(32, TY + 1), Lay::SMEM, s>>>(m->e[gen][0], m->e[gen][1], m->e[gen][2],
                                                               m->b[gen][0], m->b[gen][1], m->b[gen][2], m->cls, a,
                                                               ps, err);
    *tickets = (unsigned long long)ps.items + (unsigned long long)grid;
    return true;
}

}  // namespace

TmaMaps* tma_maps_create() { return new TmaMaps(); }
void tma_maps_destroy(TmaMaps* m) { delete m; }

bool tma_maps_encode(TmaMaps* m, int gen, const YeeArgs& a, bool wide) {
    const int ty = tile_rows(a);
    const bool pair = pair_tiles(a);
    const int ew = pair ? 72 : 40, bw = pair ? 72 : 36, cw16 = pair ? 72 : 40, cw32 = pair ? 72 : 36;
    bool ok = (a.pitch % 4) == 0;
    const float* e[3] = {a.ex, a.ey, a.ez};
    const float* b[3] = {a.bx, a.by, a.bz};
    for (int c = 0; c < 3 && ok; ++c) {
        ok = encode(&m->e[gen][c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, e[c], a, ew, ty + 2) &&
             encode(&m->b[gen][c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, b[c], a, bw, ty + 1);
    }
    if (ok)
        ok = wide ? encode(&m->cls, CU_TENSOR_MAP_DATA_TYPE_UINT32, 4, a.cls, a, cw32, ty + 1)
                  : encode(&m->cls, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, a.cls, a, cw16, ty + 1);
    m->ok[gen] = ok;
    m->cls_ok = ok;
    return ok;
}

bool tma_maps_ready(const TmaMaps* m, int gen) { return m && m->ok[gen] && m->cls_ok; }

void pair_schedule_shape(int nx, int ny, int nz, int ty, int g, int* zc, int* items) {
    YeeArgs a{};
    a.nx = nx, a.ny = ny, a.nz = nz;
    const PairSched ps = pair_schedule(a, ty, g);
    *zc = ps.zc, *items = ps.items;
}

std::vector<int4> ragged_items(const std::vector<int>& z0, const std::vector<int>& nx, const std::vector<int>& ny,
                               const std::vector<int>& nz, int ty, int g) {
    const size_t n = z0.size();
    std::vector<long long> tiles(n);
    int deepest = 1;
    for (size_t i = 0; i < n; ++i) {
        tiles[i] = (long long)((nx[i] + 63) / 64) * ((ny[i] + ty - 1) / ty);
        deepest = std::max(deepest, nz[i]);
    }
    // one chunk length for every scene: the CTA with the most items bounds the launch, and every
    // chunk above a scene's first plane re-reads one plane
    // as pair_schedule: at least kItemsPerCta items per CTA where the scenes allow it
    long long finest = 0;
    for (size_t i = 0; i < n; ++i) finest += tiles[i] * std::max(1, nz[i] / kMinBalancedPlanes);
    const long long want = std::min((long long)kItemsPerCta * g, finest);
    int zc_best = std::min(deepest, 4);
    long long best = -1;
    for (int zc = std::min(deepest, 4); zc <= deepest; ++zc) {
        long long items = 0, extra = 0;
        for (size_t i = 0; i < n; ++i) {
            const long long c = (nz[i] + zc - 1) / zc;
            items += tiles[i] * c;
            extra += c > 1 ? 1 : 0;
        }
        if (items < want) continue;
        const long long cost = (items + g - 1) / g * (zc + (extra ? 1 : 0));
        if (best < 0 || cost < best) best = cost, zc_best = zc;
    }
    std::vector<int4> out;
    for (size_t i = 0; i < n; ++i) {
        const int tx = (nx[i] + 63) / 64, tyn = (ny[i] + ty - 1) / ty;
        for (int zs = 0; zs < nz[i]; zs += zc_best)
            for (int t = 0; t < tx * tyn; ++t)
                out.push_back(make_int4((t % tx) * 64 | ((t / tx) * ty) << 16, z0[i] + zs,
                                        z0[i] + std::min(nz[i], zs + zc_best), (int)i));
    }
    return out;
}

bool launch_yee_tma(const YeeArgs& a, const TmaMaps* m, int gen, bool wide, unsigned* err, cudaStream_t s,
                    unsigned long long* tickets) {
    *tickets = 0;
    if (!m || !m->ok[gen] || !m->cls_ok) return false;
    if (pair_tiles(a) && tile_rows(a) == 16)
        return wide ? launch_p<16, uint32_t>(a, m, gen, err, s, tickets)
                    : launch_p<16, uint16_t>(a, m, gen, err, s, tickets);
    if (pair_tiles(a) && tile_rows(a) == 4)
        return wide ? launch_p<4, uint32_t>(a, m, gen, err, s, tickets)
                    : launch_p<4, uint16_t>(a, m, gen, err, s, tickets);
    if (pair_tiles(a))
        return wide ? launch_p<8, uint32_t>(a, m, gen, err, s, tickets)
                    : launch_p<8, uint16_t>(a, m, gen, err, s, tickets);
    if (tile_rows(a) == 16) return wide ? launch_t<16, uint32_t>(a, m, gen, err, s) : launch_t<16, uint16_t>(a, m, gen, err, s);
    return wide ? launch_t<8, uint32_t>(a, m, gen, err, s) : launch_t<8, uint16_t>(a, m, gen, err, s);
}

}  // namespace emlab
