// noalloc.cu — a refit entry point that allocates no device memory.
//
// dm_bvhnode2aabb_update_aabb needs num_elem-1 words of arrival flags; it
// takes them from the caller or allocates them.  Some callers can do neither:
// a real-time loop that refits a deformed mesh every frame under a no-
// allocation rule, a plugin whose host application owns the CUDA allocator,
// or an FFI caller (Rust, a game engine) with device pointers to its own
// arrays but no handle for making temporary ones.  This variant keeps the
// flags in a file-scope __device__ array instead, so the caller passes only
// inputs and outputs.
//
// The array holds kNoAllocMaxElem-1 words (16 MiB), supporting meshes of up to
// 4,194,305 triangles; every GPU that loads the library keeps it until the
// process exits.  Its device address is looked up with cudaGetSymbolAddress
// the first time the entry point runs on a device (with that device current),
// so that first call should come before any stream capture.  The address is
// kept for the life of the process: the library must not be used across a
// cudaDeviceReset of that device, which unloads the module and leaves the
// kept address stale.  All calls share
// the array: each call clears the part it uses, and calls whose work overlaps
// on the GPU (different streams, or graphs replayed concurrently) race on it.
#include <mutex>

#include "../../include/delmsh_gb300.h"
#include "dm_internal.h"

constexpr uint32_t kNoAllocMaxElem = (1u << 22) + 1;

// Arrival flags of the refit climb (one word per branch node).
static __device__ __align__(256) uint32_t g_noalloc_refit_flags[kNoAllocMaxElem - 1];

namespace {

// Device address of g_noalloc_refit_flags on the current device (looked up
// once per device).  Returns nullptr and sets *err on failure.
uint32_t* noalloc_flags(cudaError_t* err) {
  static std::mutex mu;
  static uint32_t* cache[64] = {nullptr};
  int dev = 0;
  *err = cudaGetDevice(&dev);
  if (*err != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(mu);
  if (!cache[dev]) {
    void* p = nullptr;
    *err = cudaGetSymbolAddress(&p, g_noalloc_refit_flags);
    if (*err != cudaSuccess) return nullptr;
    cache[dev] = static_cast<uint32_t*>(p);
  }
  return cache[dev];
}

}  // namespace

extern "C" int dm_bvhnode2aabb_update_aabb_noalloc(uint64_t stream_ptr, uint32_t num_bvhnode, float* bvhnode2aabb,
                                                   const uint32_t* bvhnodes, uint32_t num_elem,
                                                   const uint32_t* elem2vtx, uint32_t num_vtx,
                                                   const float* vtx2xyz0, const float* vtx2xyz1) {
  if (num_elem < 1 || num_elem > kNoAllocMaxElem)
    return dm::set_error(DM_ERR_INVALID_ARGUMENT,
                         "dm_bvhnode2aabb_update_aabb_noalloc supports 1..4194305 triangles (got %u); use "
                         "dm_bvhnode2aabb_update_aabb for larger meshes",
                         num_elem);
  if (num_bvhnode != 2 * num_elem - 1)
    return dm::set_error(DM_ERR_INVALID_ARGUMENT, "num_bvhnode (%u) must be 2*num_elem-1 (%u)", num_bvhnode,
                         2 * num_elem - 1);
  if (!bvhnode2aabb || !bvhnodes || !elem2vtx || !vtx2xyz0 || num_vtx < 1)
    return dm::set_error(DM_ERR_INVALID_ARGUMENT, "NULL argument or empty vertex array");
  cudaError_t e = cudaSuccess;
  uint32_t* flags = noalloc_flags(&e);
  if (!flags) return dm::set_error(DM_ERR_CUDA, "cudaGetSymbolAddress(flags): %s", cudaGetErrorString(e));
  cudaStream_t s = reinterpret_cast<cudaStream_t>(static_cast<uintptr_t>(stream_ptr));
  // The array keeps whatever the previous call left; the climb needs zeros.
  if (num_elem > 1) {
    e = cudaMemsetAsync(flags, 0, sizeof(uint32_t) * (num_elem - 1), s);
    if (e != cudaSuccess) return dm::set_error(DM_ERR_CUDA, "cudaMemsetAsync(flags): %s", cudaGetErrorString(e));
  }
  dm::launch_refit(s, num_elem, bvhnodes, elem2vtx, num_vtx, vtx2xyz0, vtx2xyz1, bvhnode2aabb, flags, nullptr,
                   dm::device_status_word());
  e = cudaGetLastError();
  if (e != cudaSuccess) return dm::set_error(DM_ERR_CUDA, "refit launch: %s", cudaGetErrorString(e));
  return DM_OK;
}
