// Box read-back through a fixed device array (chiml_get_box_noalloc).
//
// A variant of the detector gather (k_record in fdtd_kernels.cu): that kernel
// gathers field values at listed cells into a record buffer allocated when the
// handle is created; this one gathers a box of one field component into a
// file-scope device array, so the call needs no allocation of any kind. It is
// for callers that cannot allocate device memory when they read: a run sized
// to fill HBM has no room left for a temporary, and a host application that
// runs its own memory pool does not let a library call cudaMalloc/cudaFree
// (which also synchronise the whole device) behind its back.
//
// The array's device address is looked up when a handle is created on a device
// (box_noalloc_setup, called before the handle's own uploads), once per device.
// That lookup is what loads this file's module, and with it the array, under
// lazy module loading; the gather kernels are loaded at the same time. A read
// therefore neither places the array nor loads code: it launches one kernel and
// copies.
//
// The array is shared by every call on a device and keeps the last call's
// contents. A call writes every element it copies back before the copy, so no
// element needs clearing; elements past the box hold older values and are not
// read. Calls whose kernels or copies overlap on the GPU (two host threads at
// once, on handles of the same device) race on the array.
#include <algorithm>
#include <mutex>

#include "box_noalloc.hpp"

namespace chiml {
namespace dev {

static __device__ __align__(256) double g_boxScratch[kBoxScratchCells];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setupMutex;
double* g_scratch[kMaxDevices] = {};

template <typename T>
__global__ void k_gather_box(const T* __restrict__ U, long long lx, long long lz, int x0, int y0, int z0, int bx,
                             int bz, long long n, double* __restrict__ out) {
    const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
    for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const long long x = i % bx;
        const long long r = i / bx;
        const long long z = r % bz;
        const long long y = r / bz;
        out[i] = static_cast<double>(U[(x0 + x) + lx * ((z0 + z) + lz * (y0 + y))]);
    }
}

// Device address of the array on `device` (which is current); looked up once per device.
cudaError_t scratch_address(int device, double** out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setupMutex);
    if (!g_scratch[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_boxScratch);
        if (e != cudaSuccess) return e;
        // load the gather kernels now as well, so that a read loads no code
        cudaFuncAttributes fa;
        e = cudaFuncGetAttributes(&fa, k_gather_box<float>);
        if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_gather_box<double>);
        if (e != cudaSuccess) return e;
        g_scratch[device] = static_cast<double*>(p);
    }
    *out = g_scratch[device];
    return cudaSuccess;
}

// Makes `device` current for its lifetime when it is not already, and puts the caller's
// current device back on destruction.
class DeviceGuard {
public:
    explicit DeviceGuard(int device) {
        status_ = cudaGetDevice(&prev_);
        if (status_ == cudaSuccess && prev_ != device) {
            status_ = cudaSetDevice(device);
            switched_ = status_ == cudaSuccess;
        }
    }
    ~DeviceGuard() {
        if (switched_) cudaSetDevice(prev_);
    }
    cudaError_t status() const { return status_; }

private:
    int prev_ = 0;
    bool switched_ = false;
    cudaError_t status_ = cudaSuccess;
};

}  // namespace

cudaError_t box_noalloc_setup(int device) {
    DeviceGuard guard(device);
    if (guard.status() != cudaSuccess) return guard.status();
    double* scratch = nullptr;
    return scratch_address(device, &scratch);
}

template <typename T>
cudaError_t gather_box_noalloc(int device, const T* U, int lx, int lz, const int box[6], double* hostOut,
                               cudaStream_t stream) {
    const long long n = static_cast<long long>(box[3]) * box[4] * box[5];
    if (n <= 0 || n > kBoxScratchCells) return cudaErrorInvalidValue;
    DeviceGuard guard(device);
    if (guard.status() != cudaSuccess) return guard.status();
    double* scratch = nullptr;
    cudaError_t e = scratch_address(device, &scratch);
    if (e != cudaSuccess) return e;
    const int threads = 256;
    const long long blocks = std::min<long long>((n + threads - 1) / threads, 152LL * 8);
    k_gather_box<T><<<static_cast<unsigned>(blocks), threads, 0, stream>>>(U, lx, lz, box[0], box[1], box[2], box[3],
                                                                           box[5], n, scratch);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(hostOut, scratch, static_cast<size_t>(n) * sizeof(double), cudaMemcpyDeviceToHost, stream);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(stream);
}

template cudaError_t gather_box_noalloc<float>(int, const float*, int, int, const int[6], double*, cudaStream_t);
template cudaError_t gather_box_noalloc<double>(int, const double*, int, int, const int[6], double*, cudaStream_t);

}  // namespace dev
}  // namespace chiml
