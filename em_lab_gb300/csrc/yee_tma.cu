// yee_tma.cu - the fused Yee step with TMA-staged z planes (sm_103a).
//
// Same arithmetic and traversal as yee_fused (yee.cu): a CTA owns a 32 x TY column of cells and
// marches it along z, computing B^{n+1/2} for its cells plus the -x/-y halo cells, then E^{n+1}.
// Difference: the inputs of each z plane (E^n with a one-cell halo, B^n and the class index with
// the low halo) arrive by cp.async.bulk.tensor into a STAGES-deep shared-memory ring, issued by
// one thread and completed on per-stage mbarriers, so several planes are in flight while the CTA
// computes; threads never form global addresses for loads. B^{n+1/2} of the plane is kept in a
// double-buffered shared tile so one __syncthreads per plane suffices. Results go to the other
// field generation with coalesced 128-byte warp stores.
//
// TMA boxes start at x0-4 (x0-8 for a 16-bit class index) so the innermost coordinate stays
// 16-byte aligned; coordinates outside the grid read zeros, which is exactly the reference's
// rule that E beyond the upper faces is 0 (update_B.comp:27-29). Every mbarrier wait is bounded:
// on expiry the CTA records an error word and leaves (the host reports EMLAB_ERR_TIMEOUT).
#include <cuda.h>

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

constexpr int kStages = 4;

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

// Bounded wait: about a second of polling at most (try_wait itself suspends for a while).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (int i = 0; i < (1 << 20); ++i)
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
    static constexpr int SB_OFF = kStages * STAGE;                   // B^{n+1/2}: [2][3][TY+1][33]
    static constexpr int SB_BYTES = 2 * 3 * (TY + 1) * 33 * 4;
    static constexpr int BAR_OFF = (SB_OFF + SB_BYTES + 127) / 128 * 128;
    static constexpr int SMEM = BAR_OFF + 8 * kStages;
};

template <int TY, typename Idx>
__global__ void __launch_bounds__(32 * TY) yee_tma(const __grid_constant__ CUtensorMap tex,
                                                   const __grid_constant__ CUtensorMap tey,
                                                   const __grid_constant__ CUtensorMap tez,
                                                   const __grid_constant__ CUtensorMap tbx,
                                                   const __grid_constant__ CUtensorMap tby,
                                                   const __grid_constant__ CUtensorMap tbz,
                                                   const __grid_constant__ CUtensorMap tcls, YeeArgs a, unsigned* err) {
    using Lay = Layout<TY, Idx>;
    constexpr int TX = 32, NW = TY;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + Lay::BAR_OFF);
    float* sB = reinterpret_cast<float*>(smem + Lay::SB_OFF);

    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int zs = blockIdx.z * a.zchunk;
    const int ze = min(a.nz, zs + a.zchunk);
    if (zs >= ze) return;
    const int zstart = zs > 0 ? zs - 1 : zs;  // a chunk above z = 0 first rebuilds B^{n+1/2}(zs-1)
    const int zlast = ze;                      // planes zstart .. ze are read (ze as the "z+1" plane)
    const int x = x0 + tx, y = y0 + ty;
    const bool own = x < a.nx && y < a.ny;

    auto stage_ptr = [&](int p) { return smem + ((p - zstart) % kStages) * Lay::STAGE; };
    auto issue = [&](int p) {
        unsigned char* st = stage_ptr(p);
        uint64_t* bar = bars + (p - zstart) % kStages;
        mbar_expect_tx(bar, Lay::TX_BYTES);
        tma_load_3d(st + Lay::E_OFF + 0 * Lay::EP, &tex, x0 - 4, y0 - 1, p, bar);
        tma_load_3d(st + Lay::E_OFF + 1 * Lay::EP, &tey, x0 - 4, y0 - 1, p, bar);
        tma_load_3d(st + Lay::E_OFF + 2 * Lay::EP, &tez, x0 - 4, y0 - 1, p, bar);
        tma_load_3d(st + Lay::B_OFF + 0 * Lay::BP, &tbx, x0 - 4, y0 - 1, p, bar);
        tma_load_3d(st + Lay::B_OFF + 1 * Lay::BP, &tby, x0 - 4, y0 - 1, p, bar);
        tma_load_3d(st + Lay::B_OFF + 2 * Lay::BP, &tbz, x0 - 4, y0 - 1, p, bar);
        tma_load_3d(st + Lay::C_OFF, &tcls, x0 - Lay::CX, y0 - 1, p, bar);
    };

    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(bars + s, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0)
        for (int p = zstart; p <= zlast && p < zstart + kStages; ++p) issue(p);

    // typed views of a stage
    auto E = [&](unsigned char* st, int c, int r, int col) -> float {
        return reinterpret_cast<const float*>(st + Lay::E_OFF + c * Lay::EP)[r * Lay::EW + col];
    };
    auto Bo = [&](unsigned char* st, int c, int r, int col) -> float {
        return reinterpret_cast<const float*>(st + Lay::B_OFF + c * Lay::BP)[r * Lay::BW + col];
    };
    auto CL = [&](unsigned char* st, int r, int col) -> unsigned {
        return (unsigned)reinterpret_cast<const Idx*>(st + Lay::C_OFF)[r * Lay::CW + col];
    };
    auto SB = [&](int buf, int c, int r, int col) -> float& { return sB[((buf * 3 + c) * (TY + 1) + r) * 33 + col]; };

    // halo cells handled by this thread: item h = ty + NW * lane for lanes covering 32 + TY items
    // (items 0..31: (x0+h, y0-1); items 32..: (x0-1, y0+h-32)); spread so every warp does one share.
    const int nitems = 32 + TY;
    const int h = ty + NW * tx;
    const bool has_halo = h < nitems;

    float bpx = 0.0f, bpy = 0.0f;  // B^{n+1/2}(x, y, z-1).xy (B below the lower face is 0)
    bool failed = false;
    for (int z = zstart; z < ze; ++z) {
        const int use = (z - zstart) / kStages;
        unsigned char* st = stage_ptr(z);
        unsigned char* st1 = stage_ptr(z + 1);
        if (!mbar_wait(bars + (z - zstart) % kStages, use & 1)) failed = true;
        if (!mbar_wait(bars + (z + 1 - zstart) % kStages, ((z + 1 - zstart) / kStages) & 1)) failed = true;
        const bool emit = z >= zs;
        const int buf = (z - zstart) & 1;
        const int r = ty + 1, col = tx + 4;
        const float e0x = E(st, 0, r, col), e0y = E(st, 1, r, col), e0z = E(st, 2, r, col);
        float bx = 0.0f, by = 0.0f, bz = 0.0f;
        unsigned c = 0;
        if (own) {
            bx = Bo(st, 0, r, col), by = Bo(st, 1, r, col), bz = Bo(st, 2, r, col);
            c = CL(st, r, tx + Lay::CX);
            b_cell(a, bx, by, bz, e0x, e0y, e0z, E(st, 1, r, col + 1), E(st, 2, r, col + 1), E(st, 0, r + 1, col),
                   E(st, 2, r + 1, col), E(st1, 0, r, col), E(st1, 1, r, col), c, x, y, z);
            SB(buf, 0, r, tx + 1) = bx, SB(buf, 1, r, tx + 1) = by, SB(buf, 2, r, tx + 1) = bz;
            if (emit) {
                const long long i = (long long)z * a.plane + (long long)y * a.pitch + x;
                a.nbx[i] = bx, a.nby[i] = by, a.nbz[i] = bz;
            }
        }
        if (emit && has_halo) {
            int hr, hc, gx, gy;  // tile row/column (E/B box coordinates) and lattice cell
            if (h < 32) hr = 0, hc = h + 4, gx = x0 + h, gy = y0 - 1;
            else hr = h - 32 + 1, hc = 3, gx = x0 - 1, gy = y0 + h - 32;
            float hbx = 0.0f, hby = 0.0f, hbz = 0.0f;  // B below the lower faces is 0
            if (gx >= 0 && gy >= 0 && gx < a.nx && gy < a.ny) {
                hbx = Bo(st, 0, hr, hc), hby = Bo(st, 1, hr, hc), hbz = Bo(st, 2, hr, hc);
                b_cell(a, hbx, hby, hbz, E(st, 0, hr, hc), E(st, 1, hr, hc), E(st, 2, hr, hc), E(st, 1, hr, hc + 1),
                       E(st, 2, hr, hc + 1), E(st, 0, hr + 1, hc), E(st, 2, hr + 1, hc), E(st1, 0, hr, hc),
                       E(st1, 1, hr, hc), CL(st, hr, hc - 4 + Lay::CX), gx, gy, z);
            }
            const int sr = h < 32 ? 0 : h - 32 + 1, sc = h < 32 ? h + 1 : 0;
            SB(buf, 0, sr, sc) = hbx, SB(buf, 1, sr, sc) = hby, SB(buf, 2, sr, sc) = hbz;
        }
        if (__syncthreads_or(failed)) {
            if (tid == 0) atomicOr(err, 1u);
            return;
        }
        // every thread is past its reads of plane z-1's stage (E phase of the previous plane and
        // B phase of this one): refill it with plane z-1+kStages
        if (tid == 0 && z > zstart) {
            const int p = z - 1 + kStages;
            if (p <= zlast) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue(p);
            }
        }
        if (emit && own) {
            const float bxm_y = SB(buf, 1, r, tx), bxm_z = SB(buf, 2, r, tx);          // B(x-1)
            const float bym_x = SB(buf, 0, r - 1, tx + 1), bym_z = SB(buf, 2, r - 1, tx + 1);  // B(y-1)
            const float cx = (bz - bym_z) - (by - bpy);
            const float cy = (bx - bpx) - (bz - bxm_z);
            const float cz = (by - bxm_y) - (bx - bym_x);
            float ex = e0x, ey = e0y, ez = e0z;
            e_cell(a, ex, ey, ez, cx, cy, cz, c, x, y, z);
            const long long i = (long long)z * a.plane + (long long)y * a.pitch + x;
            a.nex[i] = ex, a.ney[i] = ey, a.nez[i] = ez;
        }
        bpx = bx, bpy = by;
    }
}

using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encode_fn() {
    static EncodeFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeFn>(p);
    }
    return fn;
}

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

int tile_rows(const YeeArgs& a) { return a.ny >= 256 ? 16 : 8; }

template <int TY, typename Idx>
bool launch_t(const YeeArgs& a, const TmaMaps* m, int gen, unsigned* err, cudaStream_t s) {
    using Lay = Layout<TY, Idx>;
    static bool configured = false;
    if (!configured) {
        if (cudaFuncSetAttribute(yee_tma<TY, Idx>, cudaFuncAttributeMaxDynamicSharedMemorySize, Lay::SMEM) !=
            cudaSuccess)
            return false;
        configured = true;
    }
    const dim3 grid((a.nx + 31) / 32, (a.ny + TY - 1) / TY, (a.nz + a.zchunk - 1) / a.zchunk);
    yee_tma<TY, Idx><<<grid, dim3(32, TY), Lay::SMEM, s>>>(m->e[gen][0], m->e[gen][1], m->e[gen][2], m->b[gen][0],
                                                           m->b[gen][1], m->b[gen][2], m->cls, a, err);
    return true;
}

}  // namespace

TmaMaps* tma_maps_create() { return new TmaMaps(); }
void tma_maps_destroy(TmaMaps* m) { delete m; }

bool tma_maps_encode(TmaMaps* m, int gen, const YeeArgs& a, bool wide) {
    const int ty = tile_rows(a);
    bool ok = (a.pitch % 4) == 0;
    const float* e[3] = {a.ex, a.ey, a.ez};
    const float* b[3] = {a.bx, a.by, a.bz};
    for (int c = 0; c < 3 && ok; ++c) {
        ok = encode(&m->e[gen][c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, e[c], a, 40, ty + 2) &&
             encode(&m->b[gen][c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, b[c], a, 36, ty + 1);
    }
    if (ok)
        ok = wide ? encode(&m->cls, CU_TENSOR_MAP_DATA_TYPE_UINT32, 4, a.cls, a, 36, ty + 1)
                  : encode(&m->cls, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, a.cls, a, 40, ty + 1);
    m->ok[gen] = ok;
    m->cls_ok = ok;
    return ok;
}

bool launch_yee_tma(const YeeArgs& a, const TmaMaps* m, int gen, bool wide, unsigned* err, cudaStream_t s) {
    if (!m || !m->ok[gen] || !m->cls_ok) return false;
    if (tile_rows(a) == 16) return wide ? launch_t<16, uint32_t>(a, m, gen, err, s) : launch_t<16, uint16_t>(a, m, gen, err, s);
    return wide ? launch_t<8, uint32_t>(a, m, gen, err, s) : launch_t<8, uint16_t>(a, m, gen, err, s);
}

}  // namespace emlab
