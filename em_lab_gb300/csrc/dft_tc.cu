// dft_tc.cu - the far-field DFT fold on the 5th-generation tensor cores (sm_103a tcgen05).
//
// One fold turns a block of T <= 64 C samples of every Huygens-box column (component c of node i,
// row r = c * P + i of the block) into sums over the block and adds them to the FP64 sums:
//   X_f += e^{-i w_f t0} sum_c e^{-i w_f 64 c dt} S_fc,   S_fc = sum_k F(t0 + (64 c + k) dt) e^{-i w_f k dt}.
// Each chunk's S_fc is one dense contraction
//   D_c[r][n] = sum_k A_c[r][k] B[n][k],   A_c = samples 64c .. 64c+63 (rows x 64), B = twiddles (N x 64),
// B rows 2f and 2f+1 holding cos(w_f k dt) and -sin(w_f k dt) (rows >= 2F are zero), the same B
// for every chunk. It runs as TF32 tcgen05.mma with split-precision operands: A = A_hi + A_lo and
// B = B_hi + B_lo, each part rounded to TF32 (cvt.rna), and D = A_hi B_hi + A_lo B_hi + A_hi B_lo
// accumulated in FP32 in tensor memory, one accumulator of N columns per chunk; the dropped
// A_lo B_lo term and the rounding of the low parts leave about 2^-21 of each product. The
// twiddles come from FP64 cos/sin on the host and are split there.
//
// Why chunks: the FP64 read-modify-write of 2F sums per row is the fold's cost (GB300's FP64 pipe
// is narrow and the sums are 2F x 16 B per row). C chunks per fold divide it by C per sample;
// C = min(4, 256 / N), so the C accumulators fit 256 tensor-memory columns (two CTAs per SM).
//
// A CTA of eight warps walks 128-row tiles. For each chunk, thread t loads half of row t % 128's 64
// samples (k in 32 (t / 128) .. +31; coalesced: the block is time-major, blk[k][r]) into registers,
// splits them and stores them K-major in the no-swizzle canonical layout of 8-row x 16-byte core
// matrices (LBO 128 B between the core matrices along K, SBO 2048 B between 8-row groups); one
// thread issues 8 K-steps x 3 MMAs (M 128, N <= 256, K 8) into the chunk's accumulator and commits
// them to an mbarrier, and the next chunk's loads are issued while they run. After the last chunk,
// warp w reads TMEM lanes 32 (w % 4) .. +31 (its 32 rows) and the column groups j with j % 2 = w / 4,
// combines the chunks with their FP32 phase factors (cos, sin of w_f 64 c dt from FP64), rotates by
// the block phase (w_f t0 in FP64 per CTA, applied in FP32) and accumulates in FP64. Every mbarrier
// wait is bounded; on expiry the CTA records an error, waits (bounded) for the MMAs it issued,
// releases its tensor memory and leaves.
#include <mutex>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "emlab_internal.h"

namespace emlab {
namespace {

constexpr int kRows = 128;  // MMA M: rows per tile = TMEM lanes
constexpr int kK = 64;      // samples per block = MMA K per tile (8 MMAs of K 8)
constexpr int kAbytes = kRows * kK * 4;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor (tcgen05): start address, leading- and stride-dimension byte
// offsets (all >> 4), the fixed descriptor version 1 at bit 46, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(const void* p, uint32_t lbo, uint32_t sbo) {
    const uint64_t a = smem_addr(p);
    return ((a & 0x3FFFFull) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::tf32: D FP32 (bits 4-5 = 1), A and B TF32 (bits 7-9, 10-12 = 2),
// both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t tf32_idesc(int m, int n) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ float to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ void mbar_init1(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int polls = kWaitPolls) {
    for (int i = 0; i < polls; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

constexpr int kThreads = 256;  // eight warps: two threads per row for the loads, two warps per lane quarter
constexpr int kMaxChunks = 4;

__host__ __device__ inline int tc_chunks(int n_mma) {
    const int c = 256 / n_mma;
    return c < 1 ? 1 : (c > kMaxChunks ? kMaxChunks : c);
}

struct TcLayout {
    int n;       // MMA N (multiple of 32, <= 256)
    int chunks;  // 64-sample chunks per fold, one TMEM accumulator each
    int ncols;   // TMEM columns allocated (power of two >= chunks * n)
    int b_off, rot_off, crot_off, bar_off, smem;
};

__host__ __device__ inline TcLayout tc_layout(int n_mma, int nf) {
    TcLayout l;
    l.n = n_mma;
    l.chunks = tc_chunks(n_mma);
    l.ncols = 32;
    while (l.ncols < l.chunks * n_mma) l.ncols *= 2;
    l.b_off = 2 * kAbytes;
    l.rot_off = l.b_off + 2 * n_mma * kK * 4;
    l.crot_off = l.rot_off + 2 * nf * 8;
    l.bar_off = (l.crot_off + kMaxChunks * nf * 8 + 15) / 16 * 16;
    l.smem = l.bar_off + 16;
    return l;
}

__global__ void __launch_bounds__(kThreads, 2)
    dft_fold_tc_kernel(const float* blk, int T, int points, int nf, int n_mma, const float4* b_hi, const float4* b_lo,
                       const double* omega, long long n0, double dt, double* X, unsigned* err, int polls) {
    extern __shared__ __align__(1024) unsigned char sm[];
    const TcLayout lay = tc_layout(n_mma, nf);
    float* a_hi = reinterpret_cast<float*>(sm);
    float* a_lo = reinterpret_cast<float*>(sm + kAbytes);
    float4* sb_hi = reinterpret_cast<float4*>(sm + lay.b_off);
    float4* sb_lo = sb_hi + n_mma * kK / 4;
    float2* rot = reinterpret_cast<float2*>(sm + lay.rot_off);    // [f][E, H]: (cos w t0, sin w t0)
    float2* crot = reinterpret_cast<float2*>(sm + lay.crot_off);  // [c][f]: (cos w 64 c dt, sin w 64 c dt)
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + lay.bar_off);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + lay.bar_off + 8);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int trow = tid & (kRows - 1), khalf = tid >> 7;  // loads: row trow, samples 32 khalf .. +31
    const long long rows = 6ll * points;
    const long long tiles = (rows + kRows - 1) / kRows;
    const int chunks = (T + kK - 1) / kK;  // <= lay.chunks (the host sizes blocks by tc_block)

    for (int j = tid; j < n_mma * kK / 4; j += blockDim.x) sb_hi[j] = b_hi[j], sb_lo[j] = b_lo[j];
    for (int j = tid; j < 2 * nf; j += blockDim.x) {
        const double t0 = ((double)n0 - ((j & 1) ? 0.5 : 0.0)) * dt;  // B lags E by half a step
        double sn, cs;
        sincos(omega[j >> 1] * t0, &sn, &cs);
        rot[j] = make_float2((float)cs, (float)sn);
    }
    for (int j = tid; j < kMaxChunks * nf; j += blockDim.x) {
        double sn, cs;
        sincos(omega[j % nf] * (double)(kK * (j / nf)) * dt, &sn, &cs);
        crot[j] = make_float2((float)cs, (float)sn);
    }
    if (tid == 0) mbar_init1(bar);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                     "r"(lay.ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = tf32_idesc(kRows, n_mma);

    // the samples of the next chunk (or the next tile's first chunk) are loaded while the current
    // chunk's MMAs run
    constexpr int kHalf = kK / 2;
    float v[kHalf];
    auto load_chunk = [&](long long tile, int c) {
        const long long row = tile * kRows + trow;
        const bool live = tile < tiles && row < rows;
        const int k0 = c * kK + khalf * kHalf;
#pragma unroll
        for (int k = 0; k < kHalf; ++k) v[k] = (live && k0 + k < T) ? __ldg(blk + (size_t)(k0 + k) * rows + row) : 0.0f;
    };
    load_chunk(blockIdx.x, 0);
    uint32_t phase = 0;
    bool failed = false;
    // K-major core-matrix layout: (row / 8) * 2048 B + (k / 4) * 128 B + (row % 8) * 16 B
    const int base = (trow >> 3) * 512 + (trow & 7) * 4 + khalf * (kHalf / 4) * 32;
    for (long long tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x) {
        for (int c = 0; c < chunks; ++c) {
#pragma unroll
            for (int q = 0; q < kHalf / 4; ++q) {
                float4 h, l;
                h.x = to_tf32(v[4 * q]), h.y = to_tf32(v[4 * q + 1]), h.z = to_tf32(v[4 * q + 2]),
                h.w = to_tf32(v[4 * q + 3]);
                l.x = to_tf32(v[4 * q] - h.x), l.y = to_tf32(v[4 * q + 1] - h.y), l.z = to_tf32(v[4 * q + 2] - h.z),
                l.w = to_tf32(v[4 * q + 3] - h.w);
                *reinterpret_cast<float4*>(a_hi + base + q * 32) = h;
                *reinterpret_cast<float4*>(a_lo + base + q * 32) = l;
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic stores -> tensor-core reads
            tc_fence_before();
            __syncthreads();
            if (tid == 0) {
                tc_fence_after();
                const uint32_t acc_col = tmem + (uint32_t)(c * n_mma);
#pragma unroll
                for (int s = 0; s < kK / 8; ++s) {
                    const uint64_t ah = smem_desc(a_hi + s * 64, 128, 2048), al = smem_desc(a_lo + s * 64, 128, 2048);
                    const uint64_t bh = smem_desc(reinterpret_cast<float*>(sb_hi) + s * 64, 128, 2048),
                                   bl = smem_desc(reinterpret_cast<float*>(sb_lo) + s * 64, 128, 2048);
                    mma_tf32(acc_col, ah, bh, idesc, s > 0 ? 1u : 0u);
                    mma_tf32(acc_col, al, bh, idesc, 1u);
                    mma_tf32(acc_col, ah, bl, idesc, 1u);
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_addr(bar))
                             : "memory");
            }
            if (c + 1 < chunks) load_chunk(tile, c + 1);
            else load_chunk(tile + gridDim.x, 0);
            const bool ok = mbar_wait_bounded(bar, phase, polls);  // the MMAs have read A: it may be refilled
            phase ^= 1u;
            if (__syncthreads_or(!ok)) {
                if (tid == 0) {
                    atomicOr(err, 2u);
                    mbar_wait_bounded(bar, phase ^ 1u);  // give the MMAs in flight a bounded time to end
                }
                failed = true;
                break;
            }
        }
        if (failed) break;
        tc_fence_after();
        // epilogue: warp w owns TMEM lanes 32 (w % 4) .. +31 (tile rows) and the column groups j with
        // j % 2 == w / 4 (16 columns = 8 frequencies per load)
        const long long row = tile * kRows + (warp & 3) * 32 + lane;
        const bool live = row < rows;
        int cc = 0, i = 0;
        if (live) cc = (int)(row / points), i = (int)(row - (long long)cc * points);
        const int h = cc >= 3 ? 1 : 0;
        double2* xo = reinterpret_cast<double2*>(X) + (size_t)cc * points + i;  // + f * 6 * points
        const size_t fstride = (size_t)6 * points;
        const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
        for (int j = warp >> 2; j < n_mma / 16; j += 2) {
            float sre[8], sim[8];
            {
                float d[16];
                tmem_ld16(tmem + lane_base + (uint32_t)(j * 16), d);
#pragma unroll
                for (int p = 0; p < 8; ++p) sre[p] = d[2 * p], sim[p] = d[2 * p + 1];
            }
            for (int c = 1; c < chunks; ++c) {
                float d[16];
                tmem_ld16(tmem + lane_base + (uint32_t)(c * n_mma + j * 16), d);
#pragma unroll
                for (int p = 0; p < 8; ++p) {
                    const int f = j * 8 + p;
                    const float2 r = crot[c * nf + (f < nf ? f : 0)];
                    const float re = d[2 * p], im = d[2 * p + 1];
                    sre[p] = sre[p] + (re * r.x + im * r.y);  // (re + i im)(cos - i sin)
                    sim[p] = sim[p] + (im * r.x - re * r.y);
                }
            }
            if (!live) continue;
            // all loads of the group before any store, so the read-modify-writes overlap
            double2 acc[8];
#pragma unroll
            for (int p = 0; p < 8; ++p)
                if (j * 8 + p < nf) acc[p] = xo[(size_t)(j * 8 + p) * fstride];
#pragma unroll
            for (int p = 0; p < 8; ++p) {
                const int f = j * 8 + p;
                if (f < nf) {
                    const float2 r = rot[2 * f + h];
                    const float re = sre[p], im = sim[p];
                    const float xr = re * r.x + im * r.y, xi = im * r.x - re * r.y;
                    acc[p].x += (double)xr, acc[p].y += (double)xi;
                    xo[(size_t)f * fstride] = acc[p];
                }
            }
        }
        tc_fence_before();
        __syncthreads();  // every warp has read its accumulators before the next tile's MMAs overwrite them
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(lay.ncols) : "memory");
}

}  // namespace

int dft_tc_mma_n(int nf) { return (2 * nf + 31) / 32 * 32; }

int dft_tc_block(int nf) { return kK * tc_chunks(dft_tc_mma_n(nf)); }

void dft_tc_twiddles(int nf, const double* omega, double dt, std::vector<float>& hi, std::vector<float>& lo) {
    const int n = dft_tc_mma_n(nf);
    hi.assign((size_t)n * kK, 0.0f), lo.assign((size_t)n * kK, 0.0f);
    auto tf32 = [](float x) {  // round to nearest, ties away from zero, at 10 fraction bits (cvt.rna.tf32)
        uint32_t u;
        std::memcpy(&u, &x, 4);
        u = (u + 0x1000u) & 0xFFFFE000u;
        float y;
        std::memcpy(&y, &u, 4);
        return y;
    };
    for (int r = 0; r < 2 * nf; ++r)
        for (int k = 0; k < kK; ++k) {
            const double ph = omega[r >> 1] * dt * k;
            const double w = (r & 1) ? -std::sin(ph) : std::cos(ph);
            const float wh = tf32((float)w), wl = tf32((float)(w - (double)wh));
            const size_t at = (size_t)(r >> 3) * 512 + (size_t)(k >> 2) * 32 + (size_t)(r & 7) * 4 + (k & 3);
            hi[at] = wh, lo[at] = wl;
        }
}

bool launch_dft_fold_tc(const float* blk, int T, int points, int nf, const float* b_hi, const float* b_lo,
                        const double* omega, long long n0, double dt, double* X, unsigned* err, cudaStream_t s) {
    const int n = dft_tc_mma_n(nf);
    if (n > 256) return false;
    const TcLayout lay = tc_layout(n, nf);
    if (T < 1 || T > kK * lay.chunks) return false;
    static int max_set = 0, sms = 0, smem_sm = 0;
    static std::mutex setup;
    std::lock_guard<std::mutex> lk(setup);
    if (lay.smem > max_set) {
        int dev = 0;
        if (cudaFuncSetAttribute(dft_fold_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, lay.smem) !=
                cudaSuccess ||
            cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
            smem_sm <= 0)
            return false;
        max_set = lay.smem;
    }
    // as many CTAs per SM as shared memory and tensor memory (512 columns) allow (two at most: the
    // launch bounds cap the registers for two); the carveout asks for exactly that much shared memory
    const int per_sm = std::max(1, std::min({smem_sm / (lay.smem + 1024), 512 / lay.ncols, 2}));
    if (cudaFuncSetAttribute(dft_fold_tc_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             std::min(100, (100 * per_sm * (lay.smem + 1024) + smem_sm - 1) / smem_sm)) != cudaSuccess)
        return false;
    const long long tiles = (6ll * points + kRows - 1) / kRows;
    const int grid = (int)std::min<long long>(tiles, (long long)sms * per_sm);
    dft_fold_tc_kernel<<<grid, kThreads, lay.smem, s>>>(blk, T, points, nf, n, reinterpret_cast<const float4*>(b_hi),
                                                        reinterpret_cast<const float4*>(b_lo), omega, n0, dt, X, err,
                                                        wait_limit());
    return true;
}

}  // namespace emlab
