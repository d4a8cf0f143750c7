// yee.cu - the leapfrog Yee update on sm_103a.
//
// Arithmetic follows shaders/update_B.comp:31-70, shaders/update_E.comp:31-66 and
// shaders/apply_sources.comp:42-79 operation for operation (compiled with -fmad=false, so no
// multiply-add is fused and every result rounds exactly as the CPU restatement's does).
//
// Two solver variants produce identical bits:
//  * yee_fused: one pass per time step. Each CTA owns a 32 x TY column of cells and marches it
//    along z. Per z plane it stages E^n of plane z (with a one-cell halo) and z+1 in shared memory,
//    computes B^{n+1/2} for its cells plus the -x / -y halo cells that its E update needs, then
//    E^{n+1}. Reads E^n, B^n, the class index; writes E^{n+1}, B^{n+1/2} to the other buffer
//    generation: 50 bytes of HBM traffic per cell-step with a 16-bit class index.
//  * yee_split_b / yee_split_e: the reference's two in-place passes (84+ bytes per cell-step),
//    kept as the layout-for-layout counterpart and as a cross-check of the fused kernel.
#include "yee_common.cuh"

namespace emlab {

namespace {

// ----------------------------------------------------------------------------------------------
// Fused single-pass kernel.
template <typename Idx, int TY>
__global__ void __launch_bounds__(32 * TY) yee_fused(YeeArgs a) {
    constexpr int TX = 32, NT = TX * TY, W = TX + 2, H = TY + 2;
    __shared__ float sE[2][3][H][W];         // E^n of planes z and z+1, origin (x0-1, y0-1)
    __shared__ float sB[3][TY + 1][TX + 1];  // B^{n+1/2} of plane z, origin (x0-1, y0-1)

    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int zs = blockIdx.z * a.zchunk;
    const int ze = min(a.nz, zs + a.zchunk);
    if (zs >= ze) return;
    const int x = x0 + tx, y = y0 + ty;
    const bool own = x < a.nx && y < a.ny;
    // halo B cells: (x, y0-1) by the first warp, (x0-1, y0+tx) by lanes tx < TY of the second
    const bool hy = ty == 0 && x < a.nx && y0 > 0;
    const bool hx = ty == 1 && tx < TY && x0 > 0 && y0 + tx < a.ny;

    auto load_plane = [&](int buf, int z) {
        for (int t = tid; t < H * W; t += NT) {
            const int r = t / W, c = t - r * W;
            const int gx = x0 - 1 + c, gy = y0 - 1 + r;
            float vx = 0.0f, vy = 0.0f, vz = 0.0f;  // E beyond the upper faces is 0 (update_B.comp:27-29)
            if (z < a.nz && gx >= 0 && gx < a.nx && gy >= 0 && gy < a.ny) {
                const long long i = (long long)z * a.plane + (long long)gy * a.pitch + gx;
                vx = __ldg(a.ex + i), vy = __ldg(a.ey + i), vz = __ldg(a.ez + i);
            }
            sE[buf][0][r][c] = vx, sE[buf][1][r][c] = vy, sE[buf][2][r][c] = vz;
        }
    };

    int z = zs > 0 ? zs - 1 : zs;  // a chunk starting above z = 0 first rebuilds B^{n+1/2} of plane zs-1
    load_plane(0, z);
    load_plane(1, z + 1);
    float bpx = 0.0f, bpy = 0.0f;  // B^{n+1/2}(x, y, z-1).xy; B below the lower face is 0
    int cur = 0;
    for (; z < ze; ++z) {
        __syncthreads();
        const bool emit = z >= zs;
        const int nxt = cur ^ 1;
        const float e0x = sE[cur][0][ty + 1][tx + 1], e0y = sE[cur][1][ty + 1][tx + 1],
                    e0z = sE[cur][2][ty + 1][tx + 1];
        float bx = 0.0f, by = 0.0f, bz = 0.0f;
        unsigned c = 0;
        long long i = 0;
        if (own) {
            i = (long long)z * a.plane + (long long)y * a.pitch + x;
            bx = __ldg(a.bx + i), by = __ldg(a.by + i), bz = __ldg(a.bz + i);
            c = load_class<Idx>(a, i);
            b_cell(a, bx, by, bz, e0x, e0y, e0z, sE[cur][1][ty + 1][tx + 2], sE[cur][2][ty + 1][tx + 2],
                   sE[cur][0][ty + 2][tx + 1], sE[cur][2][ty + 2][tx + 1], sE[nxt][0][ty + 1][tx + 1],
                   sE[nxt][1][ty + 1][tx + 1], c, x, y, z);
            sB[0][ty + 1][tx + 1] = bx, sB[1][ty + 1][tx + 1] = by, sB[2][ty + 1][tx + 1] = bz;
            if (emit) a.nbx[i] = bx, a.nby[i] = by, a.nbz[i] = bz;
        }
        if (emit) {
            if (ty == 0) {
                float hbx = 0.0f, hby = 0.0f, hbz = 0.0f;  // B below the lower face is 0
                if (hy) {
                    const long long j = (long long)z * a.plane + (long long)(y0 - 1) * a.pitch + x;
                    hbx = __ldg(a.bx + j), hby = __ldg(a.by + j), hbz = __ldg(a.bz + j);
                    b_cell(a, hbx, hby, hbz, sE[cur][0][0][tx + 1], sE[cur][1][0][tx + 1], sE[cur][2][0][tx + 1],
                           sE[cur][1][0][tx + 2], sE[cur][2][0][tx + 2], sE[cur][0][1][tx + 1], sE[cur][2][1][tx + 1],
                           sE[nxt][0][0][tx + 1], sE[nxt][1][0][tx + 1], load_class<Idx>(a, j), x, y0 - 1, z);
                }
                sB[0][0][tx + 1] = hbx, sB[1][0][tx + 1] = hby, sB[2][0][tx + 1] = hbz;
            } else if (ty == 1 && tx < TY) {
                float hbx = 0.0f, hby = 0.0f, hbz = 0.0f;
                if (hx) {
                    const int yy = y0 + tx;
                    const long long j = (long long)z * a.plane + (long long)yy * a.pitch + (x0 - 1);
                    hbx = __ldg(a.bx + j), hby = __ldg(a.by + j), hbz = __ldg(a.bz + j);
                    b_cell(a, hbx, hby, hbz, sE[cur][0][tx + 1][0], sE[cur][1][tx + 1][0], sE[cur][2][tx + 1][0],
                           sE[cur][1][tx + 1][1], sE[cur][2][tx + 1][1], sE[cur][0][tx + 2][0], sE[cur][2][tx + 2][0],
                           sE[nxt][0][tx + 1][0], sE[nxt][1][tx + 1][0], load_class<Idx>(a, j), x0 - 1, yy, z);
                }
                sB[0][tx + 1][0] = hbx, sB[1][tx + 1][0] = hby, sB[2][tx + 1][0] = hbz;
            }
        }
        __syncthreads();
        if (emit && own) {
            const float bxm_y = sB[1][ty + 1][tx], bxm_z = sB[2][ty + 1][tx];  // B(x-1)
            const float bym_x = sB[0][ty][tx + 1], bym_z = sB[2][ty][tx + 1];  // B(y-1)
            const float cx = (bz - bym_z) - (by - bpy);
            const float cy = (bx - bpx) - (bz - bxm_z);
            const float cz = (by - bxm_y) - (bx - bym_x);
            float ex = e0x, ey = e0y, ez = e0z;
            e_cell(a, ex, ey, ez, cx, cy, cz, c, x, y, z);
            a.nex[i] = ex, a.ney[i] = ey, a.nez[i] = ez;
        }
        bpx = bx, bpy = by;
        // sE[cur] (plane z) has been read by every thread before the second barrier: refill it
        // with plane z+2, which becomes the "z+1" plane after the swap.
        if (z + 1 < ze) load_plane(cur, z + 2);
        cur = nxt;
    }
}

// ----------------------------------------------------------------------------------------------
// Reference-layout split kernels (in place, update_B.comp then update_E.comp).
template <typename Idx>
__global__ void __launch_bounds__(256) yee_split_b(YeeArgs a) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y, z = blockIdx.z;
    if (x >= a.nx || y >= a.ny) return;
    const long long i = (long long)z * a.plane + (long long)y * a.pitch + x;
    const float e0x = a.ex[i], e0y = a.ey[i], e0z = a.ez[i];
    const bool px = x + 1 < a.nx, py = y + 1 < a.ny, pz = z + 1 < a.nz;
    const float exy = px ? a.ey[i + 1] : 0.0f, exz = px ? a.ez[i + 1] : 0.0f;
    const float eyx = py ? a.ex[i + a.pitch] : 0.0f, eyz = py ? a.ez[i + a.pitch] : 0.0f;
    const float ezx = pz ? a.ex[i + a.plane] : 0.0f, ezy = pz ? a.ey[i + a.plane] : 0.0f;
    float bx = a.bx[i], by = a.by[i], bz = a.bz[i];
    b_cell(a, bx, by, bz, e0x, e0y, e0z, exy, exz, eyx, eyz, ezx, ezy, load_class<Idx>(a, i), x, y, z);
    a.wbx[i] = bx, a.wby[i] = by, a.wbz[i] = bz;
}

template <typename Idx>
__global__ void __launch_bounds__(256) yee_split_e(YeeArgs a) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y, z = blockIdx.z;
    if (x >= a.nx || y >= a.ny) return;
    const long long i = (long long)z * a.plane + (long long)y * a.pitch + x;
    const float b0x = a.bx[i], b0y = a.by[i], b0z = a.bz[i];
    const float bxy = x > 0 ? a.by[i - 1] : 0.0f, bxz = x > 0 ? a.bz[i - 1] : 0.0f;
    const float byx = y > 0 ? a.bx[i - a.pitch] : 0.0f, byz = y > 0 ? a.bz[i - a.pitch] : 0.0f;
    const float bzx = z > 0 ? a.bx[i - a.plane] : 0.0f, bzy = z > 0 ? a.by[i - a.plane] : 0.0f;
    const float cx = (b0z - byz) - (b0y - bzy);
    const float cy = (b0x - bzx) - (b0z - bxz);
    const float cz = (b0y - bxy) - (b0x - byx);
    float ex = a.ex[i], ey = a.ey[i], ez = a.ez[i];
    e_cell(a, ex, ey, ez, cx, cy, cz, load_class<Idx>(a, i), x, y, z);
    a.wex[i] = ex, a.wey[i] = ey, a.wez[i] = ez;
}

// ----------------------------------------------------------------------------------------------
// apply_sources.comp:37-40
__device__ __forceinline__ float footprint(const float4* s, float px, float py, float pz) {
    const float4 c = s[0], h = s[1], w = s[3];
    const float dx = fmaxf(fabsf(px - c.x) - h.x, 0.0f) / w.x;
    const float dy = fmaxf(fabsf(py - c.y) - h.y, 0.0f) / w.y;
    const float dz = fmaxf(fabsf(pz - c.z) - h.z, 0.0f) / w.z;
    return emlab_expf(-(dx * dx + dy * dy + dz * dz));
}

// apply_sources.comp:42-79: one thread per cell a source reaches; E^{n+1} -= Cb J^{n+1/2}.
template <typename Idx>
__global__ void __launch_bounds__(64) apply_sources(YeeArgs a, SourceArgs sa, int k) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= sa.ncells) return;
    const int4 entry = sa.cells[id];
    const int end = sa.cells[id + 1].w;
    const float cx = (float)entry.x, cy = (float)entry.y, cz = (float)entry.z;
    const float* sig = sa.signals + (long long)k * sa.nsrc;
    float jx = 0.0f, jy = 0.0f, jz = 0.0f;
    for (int q = entry.w; q < end; ++q) {
        const int si = sa.lists[q];
        const float signal = sig[si];
        if (signal == 0.0f) continue;
        const float4* s = sa.src + 4 * si;
        const float wx = footprint(s, cx + 0.5f, cy, cz);
        const float wy = footprint(s, cx, cy + 0.5f, cz);
        const float wz = footprint(s, cx, cy, cz + 0.5f);
        const float4 pa = s[2];
        const float as = pa.w * signal;
        jx = jx + (pa.x * as) * wx;
        jy = jy + (pa.y * as) * wy;
        jz = jz + (pa.z * as) * wz;
    }
    if (jx == 0.0f && jy == 0.0f && jz == 0.0f) return;
    // the footprint above is evaluated in scene coordinates; memory and absorber in grid planes
    const int x = entry.x, y = entry.y, z = entry.z + (sa.zoff ? sa.zoff[id] : 0);
    const long long i = (long long)z * a.plane + (long long)y * a.pitch + x;
    const unsigned c = load_class<Idx>(a, i);
    // the absorber of the cell's scene: in a stack of scenes with their own cross-sections its nx,
    // ny and x / y profiles (common.glsl:40-43 and 15-27 on the scene's own grid)
    int snx = a.nx, sny = a.ny;
    const float* pxy = a.pml;
    int SX = a.pml_stride;
    if (sa.scene && a.scene_xy) {
        const int sc = sa.scene[id];
        const int2 d = __ldg(a.scene_xy + sc);
        snx = d.x, sny = d.y;
        pxy = a.pml_xy + (long long)sc * a.pml_xy_scene, SX = a.pml_xy_stride;
    }
    const bool inp = x < a.L || y < a.L || x >= snx - (a.L + 1) || y >= sny - (a.L + 1) || __ldg(a.pml_z + z) != 0;
    float cbx, cby, cbz;
    if (!inp) {
        const float4 t0 = __ldg(a.tabE + 2 * c), t1 = __ldg(a.tabE + 2 * c + 1);
        cbx = t0.w, cby = t1.x, cbz = t1.y;
    } else {
        const float4 m0 = __ldg(a.tabM + 2 * c), m1 = __ldg(a.tabM + 2 * c + 1);
        const int S = a.pml_stride;
        const float ix = pxy[x], iy = pxy[SX + y], iz = a.pml[2 * S + z];
        const float hx = pxy[3 * SX + x], hy = pxy[4 * SX + y], hz = a.pml[5 * S + z];
        const float sx = m0.x + ((hx + iy) + iz), sy = m0.y + ((ix + hy) + iz), sz = m0.z + ((ix + iy) + hz);
        const float dx = a.dt / m0.w, dy = a.dt / m1.x, dz = a.dt / m1.y;
        cbx = dx * emlab_phi(sx * dx), cby = dy * emlab_phi(sy * dy), cbz = dz * emlab_phi(sz * dz);
    }
    a.wex[i] = a.wex[i] - cbx * jx;
    a.wey[i] = a.wey[i] - cby * jy;
    a.wez[i] = a.wez[i] - cbz * jz;
}

template <typename Idx>
void fused_launch(const YeeArgs& a, cudaStream_t s) {
    if (a.tile_rows == 16) {
        constexpr int TY = 16;
        const dim3 grid((a.nx + 31) / 32, (a.ny + TY - 1) / TY, (a.nz + a.zchunk - 1) / a.zchunk);
        yee_fused<Idx, TY><<<grid, dim3(32, TY), 0, s>>>(a);
    } else {
        constexpr int TY = 8;
        const dim3 grid((a.nx + 31) / 32, (a.ny + TY - 1) / TY, (a.nz + a.zchunk - 1) / a.zchunk);
        yee_fused<Idx, TY><<<grid, dim3(32, TY), 0, s>>>(a);
    }
}

}  // namespace

void launch_yee_fused(const YeeArgs& a, bool wide, cudaStream_t s) {
    if (wide) fused_launch<uint32_t>(a, s);
    else fused_launch<uint16_t>(a, s);
}

void launch_yee_split(const YeeArgs& a, bool wide, cudaStream_t s) {
    const dim3 grid((a.nx + 31) / 32, (a.ny + 7) / 8, a.nz), block(32, 8);
    if (wide) {
        yee_split_b<uint32_t><<<grid, block, 0, s>>>(a);
        yee_split_e<uint32_t><<<grid, block, 0, s>>>(a);
    } else {
        yee_split_b<uint16_t><<<grid, block, 0, s>>>(a);
        yee_split_e<uint16_t><<<grid, block, 0, s>>>(a);
    }
}

void launch_sources(const YeeArgs& a, const SourceArgs& sa, int k, bool wide, cudaStream_t s) {
    if (sa.ncells <= 0) return;
    const int blocks = (sa.ncells + 63) / 64;
    if (wide) apply_sources<uint32_t><<<blocks, 64, 0, s>>>(a, sa, k);
    else apply_sources<uint16_t><<<blocks, 64, 0, s>>>(a, sa, k);
}

}  // namespace emlab
