// build.cu — LBVH build kernels: centroid AABB + fit transform, Morton codes
// (with the radix sort's digit histogram fused in), Karras topology and the
// bottom-up AABB refit.  All of them are HBM-bound integer / min-max work.
#include <cfloat>
#include <cuda/atomic>

#include "dm_device.cuh"
#include "dm_internal.h"
#include "dm_lbvh.cuh"

namespace dm {
namespace {

constexpr int kThreads = 256;

inline int grid_for(uint32_t n, int per_block, int max_blocks) {
  const uint32_t b = (n + per_block - 1) / per_block;
  return static_cast<int>(b < 1 ? 1 : (b > static_cast<uint32_t>(max_blocks) ? max_blocks : b));
}

// Vertex index checked against num_vtx (out of range -> vertex 0 + status).
__device__ __forceinline__ uint32_t vtx_index(const uint32_t* __restrict__ p, uint32_t num_vtx, uint32_t* status) {
  const uint32_t v = __ldg(p);
  if (v < num_vtx) return v;
  raise_status(status, kStatusBadIndex);
  return 0u;
}

__device__ __forceinline__ float3 tri_centroid(const uint32_t* __restrict__ tri2vtx, uint32_t num_vtx,
                                               const float* __restrict__ vtx2xyz, uint32_t it, uint32_t* status) {
  const uint32_t* t = tri2vtx + static_cast<size_t>(it) * 3;
  const float3 p0 = load_vtx(vtx2xyz, vtx_index(t, num_vtx, status));
  const float3 p1 = load_vtx(vtx2xyz, vtx_index(t + 1, num_vtx, status));
  const float3 p2 = load_vtx(vtx2xyz, vtx_index(t + 2, num_vtx, status));
  return make_float3(centroid1(p0.x, p1.x, p2.x), centroid1(p0.y, p1.y, p2.y), centroid1(p0.z, p1.z, p2.z));
}

// Reduction of (min, max) over 6 lanes-of-values held by each thread; NaN is
// ignored because every comparison with NaN is false.
struct MinMax {
  float lo[3], hi[3];
};

__device__ __forceinline__ void mm_merge(MinMax& a, const MinMax& b) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (b.lo[d] < a.lo[d]) a.lo[d] = b.lo[d];
    if (b.hi[d] > a.hi[d]) a.hi[d] = b.hi[d];
  }
}

__device__ __forceinline__ MinMax block_reduce_mm(MinMax v, MinMax* sh /* [kThreads/32] */) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    MinMax o;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      o.lo[d] = __shfl_down_sync(0xffffffffu, v.lo[d], off);
      o.hi[d] = __shfl_down_sync(0xffffffffu, v.hi[d], off);
    }
    mm_merge(v, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  if (warp == 0) {
    MinMax w;
    if (lane < kThreads / 32) {
      w = sh[lane];
    } else {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        w.lo[d] = INFINITY;
        w.hi[d] = -INFINITY;
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      MinMax o;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        o.lo[d] = __shfl_down_sync(0xffffffffu, w.lo[d], off);
        o.hi[d] = __shfl_down_sync(0xffffffffu, w.hi[d], off);
      }
      mm_merge(w, o);
    }
    v = w;
  }
  return v;  // valid in thread 0
}

// vtx2xyz.rs:19-37 applied to the triangle centroids, then the fit transform
// of Mat44/torch.py:120-140.  The sequential code seeds the box with the first
// centroid and widens it with strict comparisons, so a component is NaN iff
// the first centroid's is, and otherwise equals the min / max over the
// non-NaN values (the max of c + 0).  A two-level reduction with a last-block
// ticket computes exactly that.
__global__ void __launch_bounds__(kThreads) k_centroid_aabb(uint32_t num_tri, const uint32_t* __restrict__ tri2vtx,
                                                           uint32_t num_vtx, const float* __restrict__ vtx2xyz,
                                                           float* partials, uint32_t* ticket, float* aabb_out,
                                                           float* transform_out, uint32_t* status) {
  __shared__ MinMax sh[kThreads / 32];
  __shared__ bool s_last;
  MinMax v;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    v.lo[d] = INFINITY;
    v.hi[d] = -INFINITY;
  }
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < num_tri; i += gridDim.x * kThreads) {
    const float3 c = tri_centroid(tri2vtx, num_vtx, vtx2xyz, i, status);
    const float cc[3] = {c.x, c.y, c.z};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (cc[d] < v.lo[d]) v.lo[d] = cc[d];
      const float h = __fadd_rn(cc[d], 0.0f);
      if (h > v.hi[d]) v.hi[d] = h;
    }
  }
  v = block_reduce_mm(v, sh);
  if (threadIdx.x == 0) {
    float* p = partials + blockIdx.x * 6;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      p[d] = v.lo[d];
      p[d + 3] = v.hi[d];
    }
    __threadfence();
    s_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    v.lo[d] = INFINITY;
    v.hi[d] = -INFINITY;
  }
  for (uint32_t b = threadIdx.x; b < gridDim.x; b += kThreads) {
    MinMax o;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      o.lo[d] = __ldcg(partials + b * 6 + d);
      o.hi[d] = __ldcg(partials + b * 6 + 3 + d);
    }
    mm_merge(v, o);
  }
  __syncthreads();
  v = block_reduce_mm(v, sh);
  if (threadIdx.x == 0) {
    const float3 c0 = tri_centroid(tri2vtx, num_vtx, vtx2xyz, 0, status);
    const float c0a[3] = {c0.x, c0.y, c0.z};
    float lo[3], hi[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const bool nan0 = c0a[d] != c0a[d];
      lo[d] = nan0 ? c0a[d] : v.lo[d];
      hi[d] = nan0 ? c0a[d] : v.hi[d];
      if (aabb_out) {
        aabb_out[d] = lo[d];
        aabb_out[d + 3] = hi[d];
      }
    }
    float ext = __fsub_rn(hi[0], lo[0]);
    const float ey = __fsub_rn(hi[1], lo[1]), ez = __fsub_rn(hi[2], lo[2]);
    if (ey > ext) ext = ey;
    if (ez > ext) ext = ez;
    const float s = __fdiv_rn(1.0f, ext);
    float m[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) m[k] = 0.0f;
    m[0] = s;
    m[5] = s;
    m[10] = s;
    m[15] = 1.0f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float c = __fmul_rn(__fadd_rn(lo[d], hi[d]), 0.5f);
      m[12 + d] = __fadd_rn(__fmul_rn(-c, s), 0.5f);
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) transform_out[k] = m[k];
    *ticket = 0u;  // ready for the next launch
  }
}

// Centroid -> transform_homogeneous -> morton_code3 per triangle
// (bvhnodes_morton.rs:151-159 -> mortons.rs:115-138).  With kHist the four
// 8-bit digit histograms of the codes are accumulated for the radix sort.
template <bool kHist>
__global__ void __launch_bounds__(kThreads) k_morton_tri(uint32_t num_tri, const uint32_t* __restrict__ tri2vtx,
                                                        uint32_t num_vtx, const float* __restrict__ vtx2xyz,
                                                        const float* __restrict__ transform,
                                                        uint32_t* __restrict__ codes, uint32_t* __restrict__ hist,
                                                        uint32_t* status) {
  __shared__ float m[16];
  __shared__ uint32_t sh[kHist ? 4 * kRadix : 1];
  if (threadIdx.x < 16) m[threadIdx.x] = transform[threadIdx.x];
  if (kHist)
    for (int i = threadIdx.x; i < 4 * kRadix; i += kThreads) sh[i] = 0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < num_tri; i += gridDim.x * kThreads) {
    const float3 c = tri_centroid(tri2vtx, num_vtx, vtx2xyz, i, status);
    const float3 q = transform_homogeneous(m, c.x, c.y, c.z);
    const uint32_t code = morton_code3(q.x, q.y, q.z);
    codes[i] = code;
    if (kHist) {
#pragma unroll
      for (int p = 0; p < 4; ++p) atomicAdd(&sh[p * kRadix + ((code >> (8 * p)) & 0xFFu)], 1u);
    }
  }
  if (kHist) {
    __syncthreads();
    for (int i = threadIdx.x; i < 4 * kRadix; i += kThreads)
      if (sh[i]) atomicAdd(hist + i, sh[i]);
  }
}

// mortons.cu:8-37 (one code per point) with del-msh-cpu's clamping instead of
// the device asserts (mortons.rs:171-212).
__global__ void __launch_bounds__(kThreads) k_vtx2morton(uint32_t n, uint32_t num_dim, const float* __restrict__ vtx2co,
                                                        const float* __restrict__ transform, uint32_t* __restrict__ out) {
  __shared__ float m[16];
  if (threadIdx.x < 16) m[threadIdx.x] = (threadIdx.x < num_dim * num_dim + 2 * num_dim + 1) ? transform[threadIdx.x] : 0.f;
  __syncthreads();
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    if (num_dim == 3) {
      const float* p = vtx2co + static_cast<size_t>(i) * 3;
      const float3 q = transform_homogeneous(m, __ldg(p), __ldg(p + 1), __ldg(p + 2));
      out[i] = morton_code3(q.x, q.y, q.z);
    } else {
      const float* p = vtx2co + static_cast<size_t>(i) * 2;
      const float2 q = transform_homogeneous2(m, __ldg(p), __ldg(p + 1));
      out[i] = morton_code2(q.x, q.y);
    }
  }
}

// ----------------------------------------------------------------- topology

__global__ void __launch_bounds__(kThreads) k_topology(uint32_t n, const uint32_t* __restrict__ c,
                                                      const uint32_t* __restrict__ idx2obj, uint32_t* bvhnodes,
                                                      uint32_t* other_end) {
  const uint32_t ib = blockIdx.x * kThreads + threadIdx.x;
  if (ib >= n - 1) return;
  topology_node(n, Codes32{c}, Objs32{idx2obj}, bvhnodes, ib, other_end);
}

// A single object: the one-leaf tree [MAX, obj, MAX] (the reference leaves
// node 0 without children for n == 1).
__global__ void k_topology_single(const uint32_t* __restrict__ idx2obj, uint32_t* bvhnodes) {
  bvhnodes[0] = kUMax;
  bvhnodes[1] = idx2obj[0];
  bvhnodes[2] = kUMax;
}

// ------------------------------------------------------------------- refit

__device__ __forceinline__ Box leaf_box(const uint32_t* __restrict__ tri2vtx, uint32_t num_vtx,
                                        const float* __restrict__ xyz, uint32_t it, uint32_t* status) {
  const uint32_t* t = tri2vtx + static_cast<size_t>(it) * 3;
  Box b;
  box_set(b, load_vtx(xyz, vtx_index(t, num_vtx, status)), 0.0f);
  box_add(b, load_vtx(xyz, vtx_index(t + 1, num_vtx, status)), 0.0f);
  box_add(b, load_vtx(xyz, vtx_index(t + 2, num_vtx, status)), 0.0f);
  return b;
}

// One thread per leaf; each branch is merged by the second child to arrive
// (atomic arrival counter per branch, bvhnode2aabb.cu:7-65), always as
// from_two_aabbs(child0, child1).  The arrival word also carries the height
// of the first-arriving subtree, so the climb yields the tree height for free,
// and the second arriver clears the word so the flags stay zero between calls.
// The arrival is an acquire-release atomic: it publishes the arriving child's
// box (stored just before) and, for the second arriver, makes the sibling's
// box visible, without a full memory fence per level.  The climbing thread
// keeps its own child's box in registers and loads only the sibling's.
__global__ void __launch_bounds__(kThreads) k_refit(uint32_t num_tri, const uint32_t* __restrict__ bvhnodes,
                                                   const uint32_t* __restrict__ tri2vtx, uint32_t num_vtx,
                                                   const float* __restrict__ vtx2xyz0,
                                                   const float* __restrict__ vtx2xyz1, float* aabb, uint32_t* flags,
                                                   uint32_t* height_out, uint32_t* status) {
  const uint32_t ii = blockIdx.x * kThreads + threadIdx.x;
  if (ii >= num_tri) return;
  const uint32_t num_node = 2 * num_tri - 1;
  const uint32_t leaf = num_tri - 1 + ii;
  const uint32_t it = __ldg(bvhnodes + static_cast<size_t>(leaf) * 3 + 1);
  if (it >= num_tri) {
    raise_status(status, kStatusBadIndex);
    return;
  }
  Box b = leaf_box(tri2vtx, num_vtx, vtx2xyz0, it, status);
  if (vtx2xyz1) b = box_union(b, leaf_box(tri2vtx, num_vtx, vtx2xyz1, it, status));
  box_store(aabb + static_cast<size_t>(leaf) * 6, b);
  uint32_t h = 1;
  uint32_t prev = leaf;
  uint32_t node = __ldg(bvhnodes + static_cast<size_t>(leaf) * 3);
  uint32_t guard = 0;
  while (node != kUMax) {
    if (node >= num_tri - 1 || ++guard > num_node) {
      raise_status(status, kStatusBadIndex);
      return;
    }
    // the record is read-only: fetch it while the arrival atomic is in flight
    const uint32_t parent = __ldg(bvhnodes + static_cast<size_t>(node) * 3);
    const uint32_t c0 = __ldg(bvhnodes + static_cast<size_t>(node) * 3 + 1);
    const uint32_t c1 = __ldg(bvhnodes + static_cast<size_t>(node) * 3 + 2);
    cuda::atomic_ref<uint32_t, cuda::thread_scope_device> arrival(flags[node]);
    const uint32_t old = arrival.fetch_add(h, cuda::memory_order_acq_rel);
    if (old == 0u) return;  // the sibling subtree is not finished yet
    flags[node] = 0u;
    h = (old > h ? old : h) + 1;
    if (c0 >= num_node || c1 >= num_node || (c0 != prev && c1 != prev)) {
      raise_status(status, kStatusBadIndex);
      return;
    }
    const bool mine_first = (c0 == prev);
    const Box sib = box_load_cg(aabb + static_cast<size_t>(mine_first ? c1 : c0) * 6);
    b = mine_first ? box_union(b, sib) : box_union(sib, b);
    box_store(aabb + static_cast<size_t>(node) * 6, b);
    prev = node;
    node = parent;
  }
  if (height_out) *height_out = h;
}

// Windowed refit, in two kernels.
//
// k_leaf_boxes writes the box of every leaf.  k_refit_win then gives block b
// the kWinLeaves sorted leaves starting at b*kWinLeaves (global leaf order,
// across the meshes of a batch) and climbs from them.  A branch whose whole
// leaf range lies in the window (known from other_end: a branch index is one
// end of its range) gets both arrivals from this block, so its arrival
// counter and both child boxes live in shared memory and need only
// block-scope ordering; only branches whose range crosses a window edge use
// the global acquire-release arrival of k_refit.
//
// Link chains (branch j with left child leaf j and right child branch j+1; a
// run of equal Morton codes is one long chain) are not climbed level by
// level: the leaf of a link does not climb, and the thread that completes the
// branch below the chain walks the whole chain upward alone, box(j) =
// from_two(leaf j, box(j+1)), with no arrival counter, prefetching the next
// link's record and leaf box.  Values and merge order are those of k_refit.
constexpr int kWinLeaves = 512;
constexpr int kWinThreads = 256;

// Every branch whose range lies in the window has its index in the window,
// so the records and other ends of branches wA..wA+kWinLeaves-1 are loaded
// into shared memory once (coalesced) and the in-window climb reads no L2.
struct WinSmem {
  uint32_t flag[kWinLeaves];
  uint32_t rec[kWinLeaves][4];  // parent, left, right, other end
  Box leaf[kWinLeaves];
  Box node[kWinLeaves];
};

__device__ __forceinline__ uint32_t mesh_of_leaf(const Segments& seg, uint32_t i) {
  uint32_t lo = 0, hi = seg.num_mesh;  // tri_off[lo] <= i < tri_off[hi]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) / 2;
    if (__ldg(seg.tri_off + mid) <= i) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Offsets of the mesh owning global leaf i (single mesh: everything zero).
struct LeafMesh {
  uint32_t m, t0, T, v0, V;
  bool ok;
};

template <bool kBatch>
__device__ __forceinline__ LeafMesh leaf_mesh(const Segments& seg, uint32_t total_tri, uint32_t num_vtx_single,
                                              uint32_t i) {
  LeafMesh r{0, 0, total_tri, 0, num_vtx_single, true};
  if (kBatch) {
    r.m = mesh_of_leaf(seg, i);
    r.t0 = __ldg(seg.tri_off + r.m);
    r.T = __ldg(seg.tri_off + r.m + 1) - r.t0;
    r.v0 = __ldg(seg.vtx_off + r.m);
    r.V = __ldg(seg.vtx_off + r.m + 1) - r.v0;
  }
  r.ok = !(i < r.t0 || i - r.t0 >= r.T || r.T > 0x7FFFFFFFu);  // false only with invalid offsets
  return r;
}

template <bool kBatch>
__global__ void __launch_bounds__(kThreads) k_leaf_boxes(uint32_t total_tri, Segments seg, uint32_t num_vtx_single,
                                                        const uint32_t* __restrict__ bvhnodes_all,
                                                        const uint32_t* __restrict__ tri2vtx_all,
                                                        const float* __restrict__ vtx0_all,
                                                        const float* __restrict__ vtx1_all, float* aabb_all,
                                                        uint32_t* status) {
  const uint32_t i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= total_tri) return;
  const LeafMesh lm = leaf_mesh<kBatch>(seg, total_tri, num_vtx_single, i);
  if (!lm.ok) {
    raise_status(status, kStatusBadIndex);
    return;
  }
  const size_t node_off = 2ull * lm.t0 - lm.m;
  const uint32_t leaf = lm.T - 1 + (i - lm.t0);
  const uint32_t it = __ldg(bvhnodes_all + 3 * (node_off + leaf) + 1);
  if (it >= lm.T) {
    raise_status(status, kStatusBadIndex);
    return;
  }
  const uint32_t* t2v = tri2vtx_all + 3ull * lm.t0;
  Box b = leaf_box(t2v, lm.V, vtx0_all + 3ull * lm.v0, it, status);
  if (vtx1_all) b = box_union(b, leaf_box(t2v, lm.V, vtx1_all + 3ull * lm.v0, it, status));
  box_store(aabb_all + 6 * (node_off + leaf), b);
}

template <bool kBatch>
__global__ void __launch_bounds__(kWinThreads) k_refit_win(uint32_t total_tri, Segments seg, uint32_t num_vtx_single,
                                                          const uint32_t* __restrict__ bvhnodes_all,
                                                          const uint32_t* __restrict__ other_all, float* aabb_all,
                                                          uint32_t* gflags_all, uint32_t* height_out,
                                                          uint32_t* status) {
  extern __shared__ __align__(16) unsigned char win_raw[];
  WinSmem& S = *reinterpret_cast<WinSmem*>(win_raw);
  const uint32_t wA = blockIdx.x * kWinLeaves;
  for (int k = threadIdx.x; k < kWinLeaves; k += kWinThreads) {
    S.flag[k] = 0u;
    const uint32_t g = wA + k;  // position in the global leaf order
    if (g >= total_tri) continue;
    const LeafMesh lm = leaf_mesh<kBatch>(seg, total_tri, num_vtx_single, g);
    if (!lm.ok) continue;
    const size_t node_off = 2ull * lm.t0 - lm.m, int_off = static_cast<size_t>(lm.t0) - lm.m;
    const uint32_t n = g - lm.t0;  // leaf n and (if it exists) branch n of mesh m
    const float2* lb = reinterpret_cast<const float2*>(aabb_all + 6 * (node_off + lm.T - 1 + n));
    const float2 a = __ldcg(lb), bb = __ldcg(lb + 1), c = __ldcg(lb + 2);
    S.leaf[k] = Box{{a.x, a.y, bb.x}, {bb.y, c.x, c.y}};
    if (n + 1 >= lm.T) continue;
    const uint32_t* r = bvhnodes_all + 3 * (node_off + n);
    S.rec[k][0] = __ldg(r);
    S.rec[k][1] = __ldg(r + 1);
    S.rec[k][2] = __ldg(r + 2);
    S.rec[k][3] = __ldg(other_all + int_off + n);
  }
  __syncthreads();
  for (uint32_t k = threadIdx.x; k < static_cast<uint32_t>(kWinLeaves); k += kWinThreads) {
    const uint32_t i = wA + k;
    if (i >= total_tri) break;
    const LeafMesh lm = leaf_mesh<kBatch>(seg, total_tri, num_vtx_single, i);
    if (!lm.ok) continue;
    const uint32_t t0 = lm.t0, T = lm.T;
    const size_t node_off = 2ull * t0 - lm.m, int_off = static_cast<size_t>(t0) - lm.m;
    const uint32_t* bn = bvhnodes_all + 3 * node_off;
    const uint32_t* oe = other_all + int_off;
    float* aabb = aabb_all + 6 * node_off;
    uint32_t* gflags = gflags_all + int_off;
    const uint32_t num_node = 2 * T - 1;
    const uint32_t n = i - t0;
    const uint32_t leaf = T - 1 + n;
    uint32_t node = __ldg(bn + static_cast<size_t>(leaf) * 3);
    // the left leaf of a link is folded in by the chain walk, not climbed
    if (node == n && n + 1 < T - 1 && S.rec[k][1] == leaf && S.rec[k][2] == n + 1) continue;
    Box b = S.leaf[k];
    uint32_t h = 1, prev = leaf, guard = 0;
    auto in_win = [&](uint32_t x) { return t0 + x >= wA && t0 + x < wA + kWinLeaves; };
    auto record = [&](uint32_t x, uint32_t& parent, uint32_t& c0, uint32_t& c1, uint32_t& other) {
      if (in_win(x)) {
        const uint32_t* r = S.rec[t0 + x - wA];
        parent = r[0];
        c0 = r[1];
        c1 = r[2];
        other = r[3];
      } else {
        parent = __ldg(bn + static_cast<size_t>(x) * 3);
        c0 = __ldg(bn + static_cast<size_t>(x) * 3 + 1);
        c1 = __ldg(bn + static_cast<size_t>(x) * 3 + 2);
        other = __ldg(oe + x);
      }
    };
    auto leafbox = [&](uint32_t j) -> Box {
      if (in_win(j)) return S.leaf[t0 + j - wA];
      const float2* p2 = reinterpret_cast<const float2*>(aabb + static_cast<size_t>(T - 1 + j) * 6);
      const float2 a = __ldcg(p2), bb = __ldcg(p2 + 1), c = __ldcg(p2 + 2);
      return Box{{a.x, a.y, bb.x}, {bb.y, c.x, c.y}};
    };
    while (node != kUMax) {
      if (node >= T - 1 || ++guard > num_node) {
        raise_status(status, kStatusBadIndex);
        break;
      }
      uint32_t parent, c0, c1, other;
      record(node, parent, c0, c1, other);
      if (c0 == T - 1 + node && c1 == node + 1 && prev == c1) {
        // chain walk: node is a link reached from its right child
        uint32_t j = node, pj = parent;
        Box lb = leafbox(j);
        for (;;) {
          uint32_t pp = kUMax, pl = 0, pr = 0, po = 0;
          Box lbn{};
          const bool may = (pj != kUMax && pj + 1 == j && pj < T - 1);
          if (may) {  // prefetch the next link
            record(pj, pp, pl, pr, po);
            lbn = leafbox(pj);
          }
          b = box_union(lb, b);
          box_store(aabb + static_cast<size_t>(j) * 6, b);
          if (in_win(j)) S.node[t0 + j - wA] = b;
          h += 1;
          prev = j;
          if (++guard > num_node) {
            raise_status(status, kStatusBadIndex);
            pj = kUMax;
            break;
          }
          if (may && pl == T - 1 + pj && pr == j) {
            j = pj;
            pj = pp;
            lb = lbn;
            continue;
          }
          break;
        }
        node = pj;
        continue;
      }
      const uint32_t lo = node < other ? node : other, hi = node < other ? other : node;
      const bool local = (t0 + lo >= wA) && (t0 + hi < wA + kWinLeaves);
      uint32_t old;
      if (local) {
        __threadfence_block();  // this thread's shared box is visible before the arrival
        old = atomicAdd(&S.flag[t0 + node - wA], h);
        if (old == 0u) break;
        __threadfence_block();
      } else {
        cuda::atomic_ref<uint32_t, cuda::thread_scope_device> arrival(gflags[node]);
        old = arrival.fetch_add(h, cuda::memory_order_acq_rel);
        if (old == 0u) break;
        gflags[node] = 0u;
      }
      h = (old > h ? old : h) + 1;
      if (c0 >= num_node || c1 >= num_node || (c0 != prev && c1 != prev)) {
        raise_status(status, kStatusBadIndex);
        break;
      }
      const bool mine_first = (c0 == prev);
      const uint32_t sib = mine_first ? c1 : c0;
      Box sb;
      if (local) {
        // a valid tree keeps the sibling inside the window; check it anyway
        const uint32_t slot = (sib >= T - 1) ? t0 + (sib - (T - 1)) - wA : t0 + sib - wA;
        if (slot >= static_cast<uint32_t>(kWinLeaves)) {
          raise_status(status, kStatusBadIndex);
          break;
        }
        sb = (sib >= T - 1) ? S.leaf[slot] : S.node[slot];
      } else {
        sb = box_load_cg(aabb + static_cast<size_t>(sib) * 6);
      }
      b = mine_first ? box_union(b, sb) : box_union(sb, b);
      box_store(aabb + static_cast<size_t>(node) * 6, b);
      if (local) S.node[t0 + node - wA] = b;
      prev = node;
      node = parent;
    }
    if (node == kUMax && height_out) height_out[lm.m] = h;
  }
}

}  // namespace

// ------------------------------------------------------------- launchers

void launch_centroid_aabb(cudaStream_t s, uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                          const float* vtx2xyz, float* partials, uint32_t* ticket, float* aabb_out,
                          float* transform_out, uint32_t* status) {
  const int grid = grid_for(num_tri, kThreads * 8, kAabbBlocks);
  k_centroid_aabb<<<grid, kThreads, 0, s>>>(num_tri, tri2vtx, num_vtx, vtx2xyz, partials, ticket, aabb_out,
                                            transform_out, status);
}

void launch_morton_tri(cudaStream_t s, uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                       const float* vtx2xyz, const float* transform, uint32_t* codes, uint32_t* hist,
                       uint32_t* status) {
  const int grid = grid_for(num_tri, kThreads * 8, 152 * 16);
  if (hist)
    k_morton_tri<true><<<grid, kThreads, 0, s>>>(num_tri, tri2vtx, num_vtx, vtx2xyz, transform, codes, hist, status);
  else
    k_morton_tri<false><<<grid, kThreads, 0, s>>>(num_tri, tri2vtx, num_vtx, vtx2xyz, transform, codes, nullptr,
                                                  status);
}

void launch_vtx2morton(cudaStream_t s, uint32_t n, uint32_t num_dim, const float* vtx2co, const float* transform,
                       uint32_t* out) {
  const int grid = grid_for(n, kThreads * 4, 152 * 16);
  k_vtx2morton<<<grid, kThreads, 0, s>>>(n, num_dim, vtx2co, transform, out);
}

void launch_topology(cudaStream_t s, uint32_t n, const uint32_t* idx2morton, const uint32_t* idx2obj,
                     uint32_t* bvhnodes, uint32_t* other_end) {
  if (n == 1) {
    k_topology_single<<<1, 1, 0, s>>>(idx2obj, bvhnodes);
    return;
  }
  const uint32_t grid = (n - 1 + kThreads - 1) / kThreads;
  k_topology<<<grid, kThreads, 0, s>>>(n, idx2morton, idx2obj, bvhnodes, other_end);
}

void launch_refit_windowed(cudaStream_t s, uint32_t total_tri, const Segments& seg, uint32_t num_vtx_single,
                           const uint32_t* bvhnodes, const uint32_t* other_end, const uint32_t* tri2vtx,
                           const float* vtx2xyz0, const float* vtx2xyz1, float* aabb, uint32_t* flags,
                           uint32_t* height_out, uint32_t* status) {
  if (total_tri == 0) return;
  const int smem = static_cast<int>(sizeof(WinSmem));
  const uint32_t grid = (total_tri + kWinLeaves - 1) / kWinLeaves;
  const uint32_t leaf_grid = (total_tri + kThreads - 1) / kThreads;
  // the attribute is per device; set it once so that later calls (possibly
  // under stream capture) make no further runtime configuration calls
  static bool configured[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !configured[dev]) {
    cudaFuncSetAttribute(k_refit_win<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_refit_win<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    configured[dev] = true;
  }
  if (seg.tri_off) {
    k_leaf_boxes<true><<<leaf_grid, kThreads, 0, s>>>(total_tri, seg, num_vtx_single, bvhnodes, tri2vtx, vtx2xyz0,
                                                      vtx2xyz1, aabb, status);
    k_refit_win<true><<<grid, kWinThreads, smem, s>>>(total_tri, seg, num_vtx_single, bvhnodes, other_end, aabb, flags,
                                                      height_out, status);
  } else {
    k_leaf_boxes<false><<<leaf_grid, kThreads, 0, s>>>(total_tri, seg, num_vtx_single, bvhnodes, tri2vtx, vtx2xyz0,
                                                       vtx2xyz1, aabb, status);
    k_refit_win<false><<<grid, kWinThreads, smem, s>>>(total_tri, seg, num_vtx_single, bvhnodes, other_end, aabb,
                                                       flags, height_out, status);
  }
}

void launch_refit(cudaStream_t s, uint32_t num_tri, const uint32_t* bvhnodes, const uint32_t* tri2vtx,
                  uint32_t num_vtx, const float* vtx2xyz0, const float* vtx2xyz1, float* aabb, uint32_t* flags,
                  uint32_t* height_out, uint32_t* status) {
  const uint32_t grid = (num_tri + kThreads - 1) / kThreads;
  k_refit<<<grid, kThreads, 0, s>>>(num_tri, bvhnodes, tri2vtx, num_vtx, vtx2xyz0, vtx2xyz1, aabb, flags, height_out,
                                    status);
}

}  // namespace dm
