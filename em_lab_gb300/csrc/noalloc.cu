// noalloc.cu - Poynting flux through planes without any memory allocation.
//
// emlab_flux_planes allocates its per-workgroup partial sums with cudaMalloc and frees them again
// on every call. Some callers cannot accept that: a frame loop that measures flux every other
// frame, like the reference's, while the solver keeps stepping (cudaFree waits for the whole
// device, so every measurement would stall the solver), and applications that budget all device
// memory themselves (an allocation they did not plan for can fail part-way through a run). This
// variant keeps its scratch in fixed file-scope device arrays instead: kMaxPartials workgroup
// partials (256 KB) and kMaxPlanes FP64 sums, held by every device that loads the library until
// the process exits. The first call on a device looks their addresses up; every call shares them,
// so calls whose kernels overlap on the GPU race. The call returns once the sums are on the host.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/emlab.h"
#include "emlab_internal.h"

namespace emlab {

namespace {

constexpr int kMaxPartials = EMLAB_FLUX_NOALLOC_MAX_PARTIALS;
constexpr int kMaxPlanes = EMLAB_FLUX_NOALLOC_MAX_PLANES;
constexpr int kMaxDevices = 64;

// The scratch. In host code these names are only host-side stand-ins: the device addresses come
// from cudaGetSymbolAddress (scratch_for below) and are what the kernels receive.
static __device__ __align__(256) float g_flux_partials[kMaxPartials];
static __device__ __align__(256) double g_flux_sums[kMaxPlanes];

struct Scratch {
    float* partials = nullptr;
    double* sums = nullptr;
    bool ready = false;
};
Scratch g_scratch[kMaxDevices];
std::mutex g_scratch_mu;

// Device addresses of the scratch arrays for `device`, looked up once with that device current.
int scratch_for(int device, Scratch& out) {
    if (device < 0 || device >= kMaxDevices) return EMLAB_ERR_INVALID;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    Scratch& s = g_scratch[device];
    if (!s.ready) {
        int current = -1;
        if (cudaGetDevice(&current) != cudaSuccess || current != device) return EMLAB_ERR_CUDA;
        void* p = nullptr;
        void* q = nullptr;
        if (cudaGetSymbolAddress(&p, g_flux_partials) != cudaSuccess) return EMLAB_ERR_CUDA;
        if (cudaGetSymbolAddress(&q, g_flux_sums) != cudaSuccess) return EMLAB_ERR_CUDA;
        s.partials = static_cast<float*>(p);
        s.sums = static_cast<double*>(q);
        s.ready = true;
    }
    out = s;
    return EMLAB_OK;
}

struct PlaneSums {
    int offset[kMaxPlanes];
    int groups[kMaxPlanes];
    int n;
};

// FP64 sum of each plane's FP32 workgroup partials in workgroup order, as FieldAnalyzer::collect
// does on the host (src/FieldAnalyzer.cpp:264-269).
__global__ void flux_sum_kernel(const float* partials, PlaneSums ps, double* sums) {
    const int i = threadIdx.x;
    if (i >= ps.n) return;
    double s = 0.0;
    for (int k = 0; k < ps.groups[i]; ++k) s += (double)partials[ps.offset[i] + k];
    sums[i] = s;
}

}  // namespace

}  // namespace emlab

using namespace emlab;

extern "C" int emlab_flux_planes_noalloc(emlab_grid* g, const emlab_flux_plane* planes, int n_planes, double* out) {
    MonitorArgs m{};
    cudaStream_t stream = nullptr;
    int device = 0;
    int rc = grid_view(g, &m, &stream, &device);
    if (rc) return rc;
    if (!planes || !out || n_planes < 0) return report_error(EMLAB_ERR_INVALID, "bad flux arguments");
    if (n_planes > kMaxPlanes)
        return report_error(EMLAB_ERR_INVALID, "emlab_flux_planes_noalloc: more planes than its fixed scratch holds "
                                               "(EMLAB_FLUX_NOALLOC_MAX_PLANES)");
    if (n_planes == 0) return EMLAB_OK;
    // the rectangle clipping of FieldAnalyzer::dispatchPlane (src/FieldAnalyzer.cpp:100-124)
    const int size[3] = {m.nx, m.ny, m.nz};
    PlaneSums ps{};
    int axis[kMaxPlanes], m0[kMaxPlanes], m1[kMaxPlanes], r0[kMaxPlanes], r1[kMaxPlanes];
    int total = 0;
    for (int i = 0; i < n_planes; ++i) {
        const emlab_flux_plane& p = planes[i];
        const int a = p.axis < 0 ? 0 : (p.axis > 2 ? 2 : p.axis);
        const int u = a == 0 ? 1 : 0, v = a == 2 ? 1 : 2;
        axis[i] = a;
        m0[i] = p.rect_min[0] > 0 ? p.rect_min[0] : 0;
        m1[i] = p.rect_min[1] > 0 ? p.rect_min[1] : 0;
        r0[i] = (p.rect_max[0] < size[u] ? p.rect_max[0] : size[u]) - m0[i];
        r1[i] = (p.rect_max[1] < size[v] ? p.rect_max[1] : size[v]) - m1[i];
        long long groups = 0;
        if (p.index >= 0 && p.index < size[a] && r0[i] > 0 && r1[i] > 0)
            groups = (long long)((r0[i] + 15) / 16) * ((r1[i] + 15) / 16);
        if (total + groups > kMaxPartials)
            return report_error(EMLAB_ERR_INVALID, "emlab_flux_planes_noalloc: the planes need more workgroup partials "
                                                   "than its fixed scratch holds (EMLAB_FLUX_NOALLOC_MAX_PARTIALS)");
        ps.offset[i] = total;
        ps.groups[i] = (int)groups;
        total += (int)groups;
    }
    ps.n = n_planes;
    Scratch s;
    if (scratch_for(device, s) != EMLAB_OK)
        return report_error(EMLAB_ERR_CUDA, "emlab_flux_planes_noalloc: device scratch lookup failed");
    int launched = 0;
    for (int i = 0; i < n_planes; ++i) {
        if (!ps.groups[i]) continue;
        launch_flux_plane(m, axis[i], planes[i].index, m0[i], m1[i], r0[i], r1[i], s.partials + ps.offset[i], stream);
        ++launched;
    }
    flux_sum_kernel<<<1, kMaxPlanes, 0, stream>>>(s.partials, ps, s.sums);
    count_launches(launched + 1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return report_error(EMLAB_ERR_CUDA, cudaGetErrorString(e));
    e = cudaMemcpyAsync(out, s.sums, (size_t)n_planes * sizeof(double), cudaMemcpyDeviceToHost, stream);
    if (e != cudaSuccess) return report_error(EMLAB_ERR_CUDA, cudaGetErrorString(e));
    return emlab_grid_synchronize(g, 0);
}
