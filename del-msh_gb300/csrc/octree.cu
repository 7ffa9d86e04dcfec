// octree.cu — quad/oct-trees from the binary radix tree of sorted, unique
// Morton codes (quad_oct_tree.cu:1-233, CPU quad_oct_tree.rs:1-234,420-451):
//
//   k_brt_depth      per branch: Karras range / split (the LBVH's), branch
//                    links (leaf children encoded num_bnode + i), and the
//                    branch's depth (common prefix of the split pair) in
//                    levels of num_dim bits
//   k_onode_count /  a branch starts an octree node when its depth differs
//   k_onode_scan /   from its parent's; bnode2onode is the exclusive prefix
//   k_onode_write    sum of those flags (three-kernel scan), and idx2bnode
//                    is each leaf's parent branch
//   k_make_tree      per leaf and per node-starting branch: the octree
//                    parent (walk up the binary tree to the branch that
//                    starts a node), the child slot from the Morton digit,
//                    centres and depths
//   k_aggregate      adds each leaf's value to every octree ancestor
//
// Everything but k_aggregate is integer work or exact float arithmetic
// (halvings of sums of 0/1), so the outputs are bit-exact; k_aggregate adds
// with atomics, as the reference kernel does.
#include "dm_device.cuh"
#include "dm_internal.h"
#include "dm_lbvh.cuh"

namespace dm {
namespace {

constexpr int kThreads = 256;
constexpr int kScanItems = 8;  // flags per thread in the scan kernels
constexpr uint32_t kScanTile = kThreads * kScanItems;

struct Codes {
  const uint32_t* p;
  __device__ __forceinline__ uint32_t operator()(uint32_t i) const { return __ldg(p + i); }
};

__global__ void __launch_bounds__(kThreads) k_brt_depth(uint32_t num_bnode, const uint32_t* __restrict__ idx2morton,
                                                       uint32_t num_dim, uint32_t max_depth, uint32_t* bnodes,
                                                       uint32_t* bnode2depth) {
  const uint32_t ib = blockIdx.x * kThreads + threadIdx.x;
  if (ib >= num_bnode) return;
  if (ib == 0) bnodes[0] = kUMax;
  uint32_t r0, r1, isplit;
  const Codes c{idx2morton};
  karras_range_split(num_bnode + 1, c, ib, r0, r1, isplit);
  uint32_t* me = bnodes + static_cast<size_t>(ib) * 3;
  if (r0 == isplit) {
    me[1] = num_bnode + isplit;
  } else {
    me[1] = isplit;
    bnodes[static_cast<size_t>(isplit) * 3] = ib;
  }
  if (r1 == isplit + 1) {
    me[2] = num_bnode + isplit + 1;
  } else {
    me[2] = isplit + 1;
    bnodes[static_cast<size_t>(isplit + 1) * 3] = ib;
  }
  const uint32_t delta = static_cast<uint32_t>(__clz(c(isplit) ^ c(isplit + 1)));
  const uint32_t offset = 32u - num_dim * max_depth;
  bnode2depth[ib] = (delta - offset) / num_dim;  // u32 arithmetic, as the CPU code
}

// flag k (k < num_bnode - 1): branch k + 1 starts an octree node
__device__ __forceinline__ uint32_t onode_flag(uint32_t k, uint32_t num_bnode, const uint32_t* __restrict__ bnodes,
                                               const uint32_t* __restrict__ bnode2depth, uint32_t* status) {
  if (k + 1 >= num_bnode) return 0u;
  const uint32_t ib = k + 1, parent = __ldg(bnodes + static_cast<size_t>(ib) * 3);
  if (parent >= num_bnode) {
    raise_status(status, kStatusBadIndex);
    return 0u;
  }
  return __ldg(bnode2depth + ib) != __ldg(bnode2depth + parent) ? 1u : 0u;
}

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* sh) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  uint32_t t = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kThreads / 32; ++w) t += sh[w];
  return t;  // thread 0
}

// Per tile of kScanTile flags: their sum; also idx2bnode.
__global__ void __launch_bounds__(kThreads) k_onode_count(uint32_t num_bnode, const uint32_t* __restrict__ bnodes,
                                                         const uint32_t* __restrict__ bnode2depth,
                                                         uint32_t* idx2bnode, uint32_t* tile_sums, uint32_t* status) {
  __shared__ uint32_t sh[kThreads / 32];
  const uint32_t base = blockIdx.x * kScanTile;
  uint32_t v = 0;
  for (int q = 0; q < kScanItems; ++q) {
    const uint32_t k = base + q * kThreads + threadIdx.x;
    if (k >= num_bnode) continue;
    v += onode_flag(k, num_bnode, bnodes, bnode2depth, status);
    for (int side = 1; side <= 2; ++side) {
      const uint32_t ch = __ldg(bnodes + static_cast<size_t>(k) * 3 + side);
      if (ch >= num_bnode) {
        const uint32_t idx = ch - num_bnode;
        if (idx <= num_bnode) idx2bnode[idx] = k;
        else raise_status(status, kStatusBadIndex);
      }
    }
  }
  const uint32_t t = block_sum(v, sh);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = t;
}

// One block: exclusive scan of the tile sums, in place.
__global__ void __launch_bounds__(1024) k_onode_scan(uint32_t num_tiles, uint32_t* tile_sums) {
  __shared__ uint32_t sh[32];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (uint32_t b = 0; b < num_tiles; b += 1024) {
    const uint32_t i = b + threadIdx.x;
    const uint32_t v = i < num_tiles ? tile_sums[i] : 0u;
    uint32_t x = v;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
      if (lane >= off) x += y;
    }
    if (lane == 31) sh[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t w = sh[lane];
      for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, w, off);
        if (lane >= off) w += y;
      }
      sh[lane] = w;
    }
    __syncthreads();
    const uint32_t excl = carry + (warp > 0 ? sh[warp - 1] : 0u) + x - v;
    if (i < num_tiles) tile_sums[i] = excl;
    __syncthreads();
    if (threadIdx.x == 1023) carry = excl + v;
    __syncthreads();
  }
}

// bnode2onode[i] = sum of flags k < i: the tile's offset plus a scan of the
// tile, kScanItems consecutive flags per thread.
__global__ void __launch_bounds__(kThreads) k_onode_write(uint32_t num_bnode, const uint32_t* __restrict__ bnodes,
                                                         const uint32_t* __restrict__ bnode2depth,
                                                         const uint32_t* __restrict__ tile_offsets,
                                                         uint32_t* bnode2onode, uint32_t* status) {
  __shared__ uint32_t sh[kThreads / 32];
  const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  uint32_t f[kScanItems], sum = 0;
#pragma unroll
  for (int q = 0; q < kScanItems; ++q) {
    f[q] = base + q < num_bnode ? onode_flag(base + q, num_bnode, bnodes, bnode2depth, status) : 0u;
    sum += f[q];
  }
  // exclusive scan of the per-thread sums over the block
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = sum;
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  uint32_t before = 0;
  for (int w = 0; w < warp; ++w) before += sh[w];
  uint32_t run = __ldg(tile_offsets + blockIdx.x) + before + x - sum;
#pragma unroll
  for (int q = 0; q < kScanItems; ++q) {
    if (base + q < num_bnode) bnode2onode[base + q] = run;
    run += f[q];
  }
}

// quad_oct_tree.rs:52-63: centre of the cell of `morton` at `depth`.
__device__ __forceinline__ void morton2center(uint32_t morton, uint32_t num_dim, uint32_t depth, uint32_t max_depth,
                                              float center[3]) {
  uint32_t key = morton >> ((max_depth - depth) * num_dim);
  for (uint32_t d = 0; d < num_dim; ++d) center[d] = 0.5f;
  for (uint32_t i = 0; i < depth; ++i)
    for (uint32_t d = 0; d < num_dim; ++d) {
      const uint32_t j = num_dim - d - 1;
      center[j] = __fmul_rn(__fadd_rn(center[j], static_cast<float>(key & 1u)), 0.5f);
      key >>= 1;
    }
}

// The octree parent of binary node `cur`: walk up to the branch that starts
// an octree node (the root, or bnode2onode changes at it).
__device__ __forceinline__ bool onode_parent(uint32_t cur, uint32_t num_bnode, const uint32_t* __restrict__ bnodes,
                                             const uint32_t* __restrict__ bnode2onode,
                                             const uint32_t* __restrict__ bnode2depth, uint32_t& onode,
                                             uint32_t& depth) {
  for (uint32_t guard = 0; guard <= num_bnode; ++guard) {
    if (cur >= num_bnode) return false;
    if (cur == 0 || __ldg(bnode2onode + cur) != __ldg(bnode2onode + cur - 1)) {
      onode = __ldg(bnode2onode + cur);
      depth = __ldg(bnode2depth + cur);
      return true;
    }
    cur = __ldg(bnodes + static_cast<size_t>(cur) * 3);
  }
  return false;
}

// quad_oct_tree.rs:127-233 / quad_oct_tree.cu make_tree_from_binary_radix_tree.
__global__ void __launch_bounds__(kThreads) k_make_tree(uint32_t num_idx, const uint32_t* __restrict__ bnodes,
                                                       const uint32_t* __restrict__ bnode2onode,
                                                       const uint32_t* __restrict__ bnode2depth,
                                                       const uint32_t* __restrict__ idx2bnode,
                                                       const uint32_t* __restrict__ idx2morton, uint32_t num_onode,
                                                       uint32_t max_depth, uint32_t num_dim, uint32_t* onodes,
                                                       uint32_t* onode2depth, float* onode2center,
                                                       uint32_t* idx2onode, float* idx2center, uint32_t* status) {
  const uint32_t i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= num_idx) return;
  const uint32_t num_bnode = num_idx - 1, num_child = 1u << num_dim, nlink = num_child + 1;
  {  // leaf i
    uint32_t op, dp;
    if (!onode_parent(__ldg(idx2bnode + i), num_bnode, bnodes, bnode2onode, bnode2depth, op, dp) || op >= num_onode ||
        dp >= max_depth) {
      raise_status(status, kStatusBadIndex);
    } else {
      const uint32_t key = __ldg(idx2morton + i);
      const uint32_t ic = (key >> ((max_depth - 1 - dp) * num_dim)) & (num_child - 1);
      onodes[static_cast<size_t>(op) * nlink + 1 + ic] = i + num_onode;
      idx2onode[i] = op;
      float center[3];
      morton2center(key, num_dim, max_depth, max_depth, center);
      for (uint32_t d = 0; d < num_dim; ++d) idx2center[static_cast<size_t>(i) * num_dim + d] = center[d];
    }
  }
  if (i + 1 >= num_idx) return;
  const uint32_t ib = i;  // branch i
  if (ib == 0) {
    for (uint32_t d = 0; d < num_dim; ++d) onode2center[d] = 0.5f;
    return;
  }
  if (__ldg(bnode2onode + ib - 1) == __ldg(bnode2onode + ib)) return;  // starts no octree node
  uint32_t op, dp;
  if (!onode_parent(__ldg(bnodes + static_cast<size_t>(ib) * 3), num_bnode, bnodes, bnode2onode, bnode2depth, op,
                    dp) ||
      op >= num_onode || dp >= max_depth) {
    raise_status(status, kStatusBadIndex);
    return;
  }
  const uint32_t morton = __ldg(idx2morton + ib);
  const uint32_t ic = (morton >> ((max_depth - 1 - dp) * num_dim)) & (num_child - 1);
  const uint32_t on = __ldg(bnode2onode + ib);
  if (on >= num_onode) {
    raise_status(status, kStatusBadIndex);
    return;
  }
  onodes[static_cast<size_t>(op) * nlink + 1 + ic] = on;
  onodes[static_cast<size_t>(on) * nlink] = op;
  const uint32_t depth = __ldg(bnode2depth + ib);
  float center[3];
  morton2center(morton, num_dim, depth, max_depth, center);
  for (uint32_t d = 0; d < num_dim; ++d) onode2center[static_cast<size_t>(on) * num_dim + d] = center[d];
  onode2depth[on] = depth;
}

// quad_oct_tree.cu aggregate / quad_oct_tree.rs:420-451.
__global__ void __launch_bounds__(kThreads) k_aggregate(uint32_t num_idx, uint32_t num_vdim,
                                                       const float* __restrict__ idx2val,
                                                       const uint32_t* __restrict__ idx2onode, uint32_t num_link,
                                                       const uint32_t* __restrict__ onodes, uint32_t num_onode,
                                                       float* onode2aggval, uint32_t* status) {
  const uint32_t idx = blockIdx.x * kThreads + threadIdx.x;
  if (idx >= num_idx) return;
  uint32_t on = __ldg(idx2onode + idx);
  for (uint32_t guard = 0; on != kUMax; ++guard) {
    if (on >= num_onode || guard > num_onode) {
      raise_status(status, kStatusBadIndex);
      return;
    }
    for (uint32_t d = 0; d < num_vdim; ++d)
      atomicAdd(onode2aggval + static_cast<size_t>(on) * num_vdim + d,
                __ldg(idx2val + static_cast<size_t>(idx) * num_vdim + d));
    on = __ldg(onodes + static_cast<size_t>(on) * num_link);
  }
}

inline uint32_t grid_of(uint32_t n) { return (n + kThreads - 1) / kThreads; }

}  // namespace

size_t octree_scratch_bytes(uint32_t num_idx) {
  const uint32_t num_bnode = num_idx > 0 ? num_idx - 1 : 0;
  return (static_cast<size_t>((num_bnode + kScanTile - 1) / kScanTile) + 1) * 4 + 256;
}

void launch_octree_brt(cudaStream_t s, uint32_t num_idx, const uint32_t* idx2morton, uint32_t num_dim,
                       uint32_t max_depth, uint32_t* bnodes, uint32_t* bnode2depth, uint32_t* bnode2onode,
                       uint32_t* idx2bnode, uint32_t* tile_sums, uint32_t* status) {
  const uint32_t num_bnode = num_idx - 1;
  if (num_bnode == 0) return;
  const uint32_t tiles = (num_bnode + kScanTile - 1) / kScanTile;
  k_brt_depth<<<grid_of(num_bnode), kThreads, 0, s>>>(num_bnode, idx2morton, num_dim, max_depth, bnodes,
                                                       bnode2depth);
  k_onode_count<<<tiles, kThreads, 0, s>>>(num_bnode, bnodes, bnode2depth, idx2bnode, tile_sums, status);
  k_onode_scan<<<1, 1024, 0, s>>>(tiles, tile_sums);
  k_onode_write<<<tiles, kThreads, 0, s>>>(num_bnode, bnodes, bnode2depth, tile_sums, bnode2onode, status);
}

void launch_octree_make(cudaStream_t s, uint32_t num_idx, const uint32_t* bnodes, const uint32_t* bnode2onode,
                        const uint32_t* bnode2depth, const uint32_t* idx2bnode, const uint32_t* idx2morton,
                        uint32_t num_onode, uint32_t max_depth, uint32_t num_dim, uint32_t* onodes,
                        uint32_t* onode2depth, float* onode2center, uint32_t* idx2onode, float* idx2center,
                        uint32_t* status) {
  if (num_idx == 0) return;
  k_make_tree<<<grid_of(num_idx), kThreads, 0, s>>>(num_idx, bnodes, bnode2onode, bnode2depth, idx2bnode, idx2morton,
                                                     num_onode, max_depth, num_dim, onodes, onode2depth, onode2center,
                                                     idx2onode, idx2center, status);
}

void launch_octree_aggregate(cudaStream_t s, uint32_t num_idx, uint32_t num_vdim, const float* idx2val,
                             const uint32_t* idx2onode, uint32_t num_link, const uint32_t* onodes, uint32_t num_onode,
                             float* onode2aggval, uint32_t* status) {
  if (num_idx == 0 || num_vdim == 0) return;
  k_aggregate<<<grid_of(num_idx), kThreads, 0, s>>>(num_idx, num_vdim, idx2val, idx2onode, num_link, onodes,
                                                     num_onode, onode2aggval, status);
}

}  // namespace dm
