// dft_tc.cu - the far-field DFT fold on the 5th-generation tensor cores (sm_103a tcgen05).
//
// One fold turns a block of T <= 64 samples of every Huygens-box column (component c of node i,
// row r = c * P + i of the block) into the in-block sums S_f = sum_k F(t0 + k dt) e^{-i w_f k dt}
// and adds e^{-i w_f t0} S_f to the FP64 sums. The in-block sums are one dense contraction
//   D[r][n] = sum_k A[r][k] B[n][k],   A = samples (rows x 64), B = twiddles (N x 64),
// B rows 2f and 2f+1 holding cos(w_f k dt) and -sin(w_f k dt) (rows >= 2F are zero). It runs as
// TF32 tcgen05.mma with split-precision operands: A = A_hi + A_lo and B = B_hi + B_lo, each part
// rounded to TF32 (cvt.rna), and D = A_hi B_hi + A_lo B_hi + A_hi B_lo accumulated in FP32 in
// tensor memory; the dropped A_lo B_lo term and the rounding of the low parts leave about 2^-21 of
// each product. The twiddles come from FP64 cos/sin on the host and are split there.
//
// A CTA of four warps walks 128-row tiles: each thread loads one row's 64 samples (coalesced: the
// block is time-major, blk[k][r]), splits them, and stores them K-major in the no-swizzle canonical
// layout of 8-row x 16-byte core matrices (LBO 128 B between the core matrices along K, SBO 2048 B
// between 8-row groups); one thread issues 8 K-steps x 3 MMAs (M 128, N <= 256, K 8) and commits
// them to an mbarrier; each warp then reads its 32 TMEM lanes (= its 32 rows) with tcgen05.ld and
// applies the FP32 rotation by the block phase (cos, sin of w_f t0 evaluated in FP64 per CTA) and
// the FP64 accumulation. Every mbarrier wait is bounded; on expiry the CTA records an error,
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

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    for (int i = 0; i < (1 << 20); ++i) {
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

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

struct TcLayout {
    int n;      // MMA N (multiple of 32, <= 256)
    int ncols;  // TMEM columns allocated (power of two >= n)
    int b_off, rot_off, bar_off, smem;
};

__host__ __device__ inline TcLayout tc_layout(int n_mma, int nf) {
    TcLayout l;
    l.n = n_mma;
    l.ncols = 32;
    while (l.ncols < n_mma) l.ncols *= 2;
    l.b_off = 2 * kAbytes;
    l.rot_off = l.b_off + 2 * n_mma * kK * 4;
    l.bar_off = l.rot_off + 2 * nf * 8;
    l.smem = l.bar_off + 16;
    return l;
}

__global__ void __launch_bounds__(128) dft_fold_tc_kernel(const float* blk, int T, int points, int nf, int n_mma,
                                                          const float4* b_hi, const float4* b_lo,
                                                          const double* omega, long long n0, double dt, double* X,
                                                          unsigned* err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    const TcLayout lay = tc_layout(n_mma, nf);
    float* a_hi = reinterpret_cast<float*>(sm);
    float* a_lo = reinterpret_cast<float*>(sm + kAbytes);
    float4* sb_hi = reinterpret_cast<float4*>(sm + lay.b_off);
    float4* sb_lo = sb_hi + n_mma * kK / 4;
    float2* rot = reinterpret_cast<float2*>(sm + lay.rot_off);  // [f][E, H]: (cos w t0, sin w t0)
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + lay.bar_off);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + lay.bar_off + 8);

    const int tid = threadIdx.x, warp = tid >> 5;
    const long long rows = 6ll * points;
    const long long tiles = (rows + kRows - 1) / kRows;

    for (int j = tid; j < n_mma * kK / 4; j += blockDim.x) sb_hi[j] = b_hi[j], sb_lo[j] = b_lo[j];
    for (int j = tid; j < 2 * nf; j += blockDim.x) {
        const double t0 = ((double)n0 - ((j & 1) ? 0.5 : 0.0)) * dt;  // B lags E by half a step
        double s, c;
        sincos(omega[j >> 1] * t0, &s, &c);
        rot[j] = make_float2((float)c, (float)s);
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

    // the samples of the next tile are loaded while the current tile's MMAs and epilogue run
    float v[kK];
    auto load_rows = [&](long long tile) {
        const long long row = tile * kRows + tid;
        const bool live = tile < tiles && row < rows;
#pragma unroll
        for (int k = 0; k < kK; ++k) v[k] = (live && k < T) ? __ldg(blk + (size_t)k * rows + row) : 0.0f;
    };
    load_rows(blockIdx.x);
    uint32_t phase = 0;
    for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const long long row = tile * kRows + tid;
        const bool live = row < rows;
        // K-major core-matrix layout: (row / 8) * 2048 B + (k / 4) * 128 B + (row % 8) * 16 B
        const int base = (tid >> 3) * 512 + (tid & 7) * 4;
#pragma unroll
        for (int q = 0; q < kK / 4; ++q) {
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
#pragma unroll
            for (int s = 0; s < kK / 8; ++s) {
                const uint64_t ah = smem_desc(a_hi + s * 64, 128, 2048), al = smem_desc(a_lo + s * 64, 128, 2048);
                const uint64_t bh = smem_desc(reinterpret_cast<float*>(sb_hi) + s * 64, 128, 2048),
                               bl = smem_desc(reinterpret_cast<float*>(sb_lo) + s * 64, 128, 2048);
                mma_tf32(tmem, ah, bh, idesc, s > 0 ? 1u : 0u);
                mma_tf32(tmem, al, bh, idesc, 1u);
                mma_tf32(tmem, ah, bl, idesc, 1u);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_addr(bar))
                         : "memory");
        }
        load_rows(tile + gridDim.x);
        const bool ok = mbar_wait_bounded(bar, phase);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicOr(err, 2u);
            break;
        }
        tc_fence_after();
        int c = 0, i = 0;
        if (live) c = (int)(row / points), i = (int)(row - (long long)c * points);
        const int h = c >= 3 ? 1 : 0;
        double2* xo = reinterpret_cast<double2*>(X) + (size_t)c * points + i;  // + f * 6 * points
        const size_t fstride = (size_t)6 * points;
        for (int j = 0; j < n_mma / 32; ++j) {
            float d[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(j * 32), d);
            if (!live) continue;
            // all loads of the chunk before any store, so the 16 read-modify-writes overlap
            double2 acc[16];
#pragma unroll
            for (int p = 0; p < 16; ++p)
                if (j * 16 + p < nf) acc[p] = xo[(size_t)(j * 16 + p) * fstride];
#pragma unroll
            for (int p = 0; p < 16; ++p) {
                const int f = j * 16 + p;
                if (f < nf) {
                    const float2 r = rot[2 * f + h];
                    const float re = d[2 * p], im = d[2 * p + 1];
                    const float xr = re * r.x + im * r.y, xi = im * r.x - re * r.y;  // (re + i im)(cos - i sin)
                    acc[p].x += (double)xr, acc[p].y += (double)xi;
                    xo[(size_t)f * fstride] = acc[p];
                }
            }
        }
        tc_fence_before();
        __syncthreads();  // every warp has read D before the next tile's MMAs overwrite it
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(lay.ncols) : "memory");
}

}  // namespace

int dft_tc_mma_n(int nf) { return (2 * nf + 31) / 32 * 32; }

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
    // as many CTAs per SM as shared memory and tensor memory (512 columns) allow; the carveout asks
    // for exactly that much shared memory
    const int per_sm = std::max(1, std::min(smem_sm / (lay.smem + 1024), 512 / lay.ncols));
    if (cudaFuncSetAttribute(dft_fold_tc_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             std::min(100, (100 * per_sm * (lay.smem + 1024) + smem_sm - 1) / smem_sm)) != cudaSuccess)
        return false;
    const long long tiles = (6ll * points + kRows - 1) / kRows;
    const int grid = (int)std::min<long long>(tiles, (long long)sms * per_sm);
    dft_fold_tc_kernel<<<grid, 128, lay.smem, s>>>(blk, T, points, nf, n, reinterpret_cast<const float4*>(b_hi),
                                                   reinterpret_cast<const float4*>(b_lo), omega, n0, dt, X, err);
    return true;
}

}  // namespace emlab
