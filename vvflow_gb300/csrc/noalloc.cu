// vvgpu_velocity_points_noalloc: point velocities without any device allocation.
//
// vvgpu_velocity_points stages the query points and the results in a device buffer it
// allocates per call.  Some callers cannot allow that: a host application that gives the
// solver a fixed device-memory budget, or a probe loop that runs beside the solver every
// step and must not trigger the device-wide synchronisation that cudaMalloc and cudaFree
// imply.  This entry point stages through a fixed array in device memory instead.
//
// The array is a file-scope __device__ object of VVGPU_NOALLOC_MAX_POINTS x 4 doubles
// (512 KiB).  Every GPU that loads the library holds it until the process exits.  Host code
// cannot use the array's name as a device address, so the first call on each device, with
// that device current, looks the address up with cudaGetSymbolAddress and keeps it.  All
// calls share the one array and it keeps
// the last call's contents (every call overwrites the points and results it uses, so
// nothing needs clearing); calls whose GPU work overlaps, from different contexts or
// streams, race on it.
#include <mutex>

#include "vvgpu_internal.cuh"

namespace {

__device__ __align__(256) double g_point_scratch[4 * VVGPU_NOALLOC_MAX_POINTS];

constexpr int kMaxDevices = 64;
double* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

// Device address of the scratch array on the current device (looked up once per device).
cudaError_t scratch_address(int device, double** out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_point_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[device] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[device];
    return cudaSuccess;
}

}  // namespace

extern "C" int vvgpu_velocity_points_noalloc(vvgpu_ctx* h, int64_t n, const double* px, const double* py,
                                             double* vx, double* vy) {
    using namespace vvgpu;
    if (!h) return VVGPU_ERR_ARG;
    Ctx& c = h->c;
    try {
        if (n < 0 || (n && (!px || !py || !vx || !vy))) throw ApiError{VVGPU_ERR_ARG, "bad point arrays"};
        if (n > VVGPU_NOALLOC_MAX_POINTS)
            throw ApiError{VVGPU_ERR_LIMIT, "vvgpu_velocity_points_noalloc takes at most " +
                                                std::to_string(VVGPU_NOALLOC_MAX_POINTS) + " points per call, got " +
                                                std::to_string(n)};
        if (!c.built) throw ApiError{VVGPU_ERR_NOT_BUILT, "tree is not built"};
        if (!c.lists_full)
            throw ApiError{VVGPU_ERR_STATE, "near lists not built yet: call vvgpu_velocity_points (or vvgpu_eps, "
                                            "vvgpu_convective, vvgpu_diffusive) after vvgpu_tree_build first"};
        VV_CUDA(cudaSetDevice(c.device));
        double* base = nullptr;
        VV_CUDA(scratch_address(c.device, &base));
        if (n == 0) return VVGPU_OK;
        double* dpx = base;
        double* dpy = base + VVGPU_NOALLOC_MAX_POINTS;
        double* dvx = base + 2 * VVGPU_NOALLOC_MAX_POINTS;
        double* dvy = base + 3 * VVGPU_NOALLOC_MAX_POINTS;
        cudaStream_t s = c.st();
        VV_CUDA(cudaMemcpyAsync(dpx, px, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s));
        VV_CUDA(cudaMemcpyAsync(dpy, py, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s));
        velocity_points_on_device(c, n, dpx, dpy, dvx, dvy);
        VV_CUDA(cudaMemcpyAsync(vx, dvx, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s));
        VV_CUDA(cudaMemcpyAsync(vy, dvy, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s));
        VV_CUDA(cudaStreamSynchronize(s));
    } catch (ApiError& e) {
        c.last_error = e.msg;
        return e.code;
    } catch (CudaError& e) {
        c.last_error = std::string(e.what) + ": " + cudaGetErrorString(e.err);
        return VVGPU_ERR_CUDA;
    }
    return VVGPU_OK;
}
