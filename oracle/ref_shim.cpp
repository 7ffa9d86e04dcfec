// ref_shim.cpp — compiles the reference's own CUDA sources for this path
// (del-msh-cuda-kernels/cuda/bvhnodes_morton.cu, which includes mortons.h)
// as plain host C++, so that their Morton codes, centroids and radix-tree
// topology can be run on the CPU and used to pin the oracle.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build.py compiles this file with
// -I <reference>/del-msh-cuda-kernels/cuda into oracle/_ref/; nothing from the
// reference is copied into this repository.  The few CUDA built-ins those two
// files use are given host meanings here: __clz (count leading zeros, 32 for
// zero), int2/make_int2, and the block/thread index variables, which the
// driver loop below sets per emulated thread.
#include <climits>
#include <cmath>
#include <cstdint>

#define __device__
#define __global__
struct int2 {
  int x, y;
};
static inline int2 make_int2(int a, int b) {
  int2 r;
  r.x = a;
  r.y = b;
  return r;
}
static inline int __clz(unsigned int v) { return v == 0 ? 32 : __builtin_clz(v); }
struct ref_dim3 {
  unsigned int x, y, z;
};
static thread_local ref_dim3 blockDim = {1, 1, 1}, blockIdx = {0, 0, 0}, threadIdx = {0, 0, 0};

#include "bvhnodes_morton.cu"

extern "C" {

uint32_t ref_expand_bits3(uint32_t v) { return mortons::device_expand_bits3(v); }
uint32_t ref_morton_code3(float x, float y, float z) { return mortons::device_morton_code3(x, y, z); }
uint32_t ref_morton_code2(float x, float y) { return mortons::device_morton_code2(x, y); }

// Runs kernel_MortonCode_BVHTopology once per emulated thread, in index order.
void ref_bvh_topology(uint32_t n, const uint32_t* idx2morton, const uint32_t* idx2obj, uint32_t* bvhnodes) {
  blockDim.x = 1;
  threadIdx.x = 0;
  for (uint32_t i = 0; i < n; ++i) {
    blockIdx.x = i;
    kernel_MortonCode_BVHTopology(n, bvhnodes, idx2morton, idx2obj);
  }
}

// Runs tri2cntr once per emulated thread.
void ref_tri2cntr(uint32_t num_tri, const uint32_t* tri2vtx, const float* vtx2xyz, float* out) {
  blockDim.x = 1;
  threadIdx.x = 0;
  for (uint32_t i = 0; i < num_tri; ++i) {
    blockIdx.x = i;
    tri2cntr(out, num_tri, tri2vtx, vtx2xyz);
  }
}

}  // extern "C"
