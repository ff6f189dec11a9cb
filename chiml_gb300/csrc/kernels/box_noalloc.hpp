// Box read-back that allocates no memory (chiml_get_box_noalloc, box_noalloc.cu).
#pragma once

#include <cuda_runtime.h>

namespace chiml {
namespace dev {

// Capacity of the file-scope device array the read-back stages through:
// 1,048,576 FP64 values (8 MiB) per device.
constexpr long long kBoxScratchCells = 1LL << 20;

// Looks up the device address of the array on `device` with cudaGetSymbolAddress
// (which places the array there under lazy module loading) and loads the gather
// kernels; once per device, later calls return at once. Called when a handle is
// created, before its own uploads. The caller's current device is kept.
cudaError_t box_noalloc_setup(int device);

// Gathers the box {x0, y0, z0, nx, ny, nz} of the field U (local extents
// lx, ly, lz; index x + lx*(z + lz*y)) into the device array as FP64, copies it
// to hostOut in the same x-fastest, then z, then y order, and waits for the
// copy. The caller has checked the box against the extents and the capacity.
// The caller's current device is kept.
template <typename T>
cudaError_t gather_box_noalloc(int device, const T* U, int lx, int lz, const int box[6], double* hostOut,
                               cudaStream_t stream);

}  // namespace dev
}  // namespace chiml
