// Kinetic-energy reduction (sum of m v^2) that allocates no device memory.
//
// Some callers cannot call cudaMalloc at all. Examples: a host code that runs inside a CUDA graph
// being captured, a plugin loaded into a process whose allocator owns all device memory and forbids
// outside allocations, or a real-time loop that must not block on the allocator. The regular thermo
// path (mg_thermo) keeps its per-block partial sums in a buffer the context allocates, so those
// callers cannot use it. This variant keeps the partial sums in a fixed array of this file instead,
// and works on arrays the caller already owns.
//
// The array is a file-scope __device__ variable: every GPU that loads libmisa_gb300.so holds its
// 64 KiB until the process exits, and every call on that GPU reuses it.

#include <cuda_runtime.h>

#include <mutex>

#include "../../include/misa_gb300.h"
#include "mg_internal.h"

namespace mg {
void set_global_error(const char *msg);
}

namespace {

constexpr int kThreads = 256;
constexpr int kPerThread = 16;
constexpr int kMaxBlocks = 8192;  // partial sums the scratch array holds
constexpr int64_t kMaxAtoms = (int64_t) kMaxBlocks * kThreads * kPerThread;  // 33,554,432
constexpr int kMaxDevices = 64;

// Scratch shared by all calls on one GPU: one partial sum per block of the first kernel. Each call
// writes every entry it later reads, so nothing here needs clearing between calls; the last call's
// values simply remain.
static __device__ __align__(256) double g_mvv_partials[kMaxBlocks];

std::mutex g_setup_mutex;
double *g_partials_addr[kMaxDevices] = {};  // device address of g_mvv_partials, per device

// types other than 0, 1 and 2 weigh nothing, like vacancies (the caller's arrays are not validated)
__device__ __forceinline__ double mass_of(int t) {  // src/types/atom_types.h:17-19
    return t == 0 ? 55.845 : (t == 1 ? 63.546 : (t == 2 ? 58.6934 : 0.0));
}

__device__ __forceinline__ double block_sum(double v) {
    __shared__ double warp_part[kThreads / 32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) warp_part[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < kThreads / 32; w++) s += warp_part[w];
    return s;
}

__global__ void __launch_bounds__(kThreads) k_mvv_partial(const double *vx, const double *vy, const double *vz,
                                                          const int8_t *type, int64_t n, double *partials) {
    double acc = 0.0;
    for (int64_t i = blockIdx.x * (int64_t) kThreads + threadIdx.x; i < n; i += (int64_t) gridDim.x * kThreads) {
        const int t = type[i];
        if (t < 0) continue;  // vacancy
        acc += (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]) * mass_of(t);
    }
    const double s = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kThreads) k_mvv_final(const double *partials, int nb, double *out) {
    double acc = 0.0;
    for (int b = threadIdx.x; b < nb; b += kThreads) acc += partials[b];
    const double s = block_sum(acc);
    if (threadIdx.x == 0) *out = s;
}

}  // namespace

extern "C" mg_status mg_mvv_noalloc(const double *vx, const double *vy, const double *vz, const int8_t *type,
                                    int64_t n, double *out_mvv, void *stream) {
    if (!out_mvv || n < 0 || (n > 0 && (!vx || !vy || !vz || !type))) {
        mg::set_global_error("mg_mvv_noalloc: null pointer or negative atom count");
        return MG_ERR_ARG;
    }
    if (n > kMaxAtoms) {
        mg::set_global_error("mg_mvv_noalloc: more than 33,554,432 atoms (the fixed scratch holds 8192 block sums "
                             "of 4096 atoms each); use mg_thermo for larger states");
        return MG_ERR_ARG;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        mg::set_global_error("mg_mvv_noalloc: no usable current device");
        return MG_ERR_CUDA;
    }
    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(st, &capture);
    if (e != cudaSuccess) {
        mg::set_global_error(cudaGetErrorString(e));
        return MG_ERR_CUDA;
    }
    double *partials = nullptr;
    {
        // Look up the scratch array's device address on the current device. Outside a capture the
        // address is looked up again on every call, so a device reset (which reloads the module and
        // may move the array) is picked up by the next uncaptured call; a captured call uses the
        // address of the last uncaptured call on this device and needs one to have happened.
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (capture == cudaStreamCaptureStatusNone) {
            double *p = nullptr;
            e = cudaGetSymbolAddress(reinterpret_cast<void **>(&p), g_mvv_partials);
            if (e != cudaSuccess || !p) {
                mg::set_global_error("mg_mvv_noalloc: cudaGetSymbolAddress of the scratch array failed");
                return MG_ERR_CUDA;
            }
            g_partials_addr[dev] = p;
        } else if (!g_partials_addr[dev]) {
            mg::set_global_error("mg_mvv_noalloc: the first call on a device must come before any stream capture");
            return MG_ERR_STATE;
        }
        partials = g_partials_addr[dev];
    }
    const int64_t per_block = (int64_t) kThreads * kPerThread;
    int nb = static_cast<int>((n + per_block - 1) / per_block);
    // the launches' own return codes, so an error left by unrelated earlier work is not reported here
    if (nb > 0) {
        void *args[] = {&vx, &vy, &vz, &type, &n, &partials};
        e = cudaLaunchKernel(reinterpret_cast<const void *>(k_mvv_partial), dim3(nb), dim3(kThreads), args, 0, st);
        if (e != cudaSuccess) {
            mg::set_global_error(cudaGetErrorString(e));
            return MG_ERR_CUDA;
        }
    }
    void *fargs[] = {&partials, &nb, &out_mvv};
    e = cudaLaunchKernel(reinterpret_cast<const void *>(k_mvv_final), dim3(1), dim3(kThreads), fargs, 0, st);
    if (e != cudaSuccess) {
        mg::set_global_error(cudaGetErrorString(e));
        return MG_ERR_CUDA;
    }
    return MG_OK;
}
