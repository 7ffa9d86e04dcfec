// build.cu — LBVH build kernels: centroid AABB + fit transform, Morton codes
// (with the radix sort's digit histogram fused in), Karras topology and the
// bottom-up AABB refit.  All of them are HBM-bound integer / min-max work.
#include <algorithm>
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

// Words of the refit header read once per block (thread 0, volatile) and
// shared: every thread reading the same L2 line would queue thousands of
// requests on one L2 slice.  Has __syncthreads.
__device__ __forceinline__ uint2 block_read_hdr(const uint32_t* w0, const uint32_t* w1) {
  __shared__ uint2 s_words;
  if (threadIdx.x == 0)
    s_words = make_uint2(*reinterpret_cast<const volatile uint32_t*>(w0),
                         w1 ? *reinterpret_cast<const volatile uint32_t*>(w1) : 0u);
  __syncthreads();
  return s_words;
}
__device__ __forceinline__ uint3 block_read_hdr3(const uint32_t* w0, const uint32_t* w1, const uint32_t* w2) {
  __shared__ uint3 s_words3;
  if (threadIdx.x == 0)
    s_words3 = make_uint3(*reinterpret_cast<const volatile uint32_t*>(w0),
                          *reinterpret_cast<const volatile uint32_t*>(w1),
                          *reinterpret_cast<const volatile uint32_t*>(w2));
  __syncthreads();
  return s_words3;
}

// A box written by an earlier kernel and not written in this one, read
// through L1 (ld.global.ca): the crossing-branch queries of neighbouring
// branches read mostly the same leaves and segment-tree nodes.  Read after
// the kernel's dependency wait, which makes the earlier kernels' writes
// visible to it.
__device__ __forceinline__ Box box_load_l1(const float* src) {
  const float2* s2 = reinterpret_cast<const float2*>(src);
  const float2 a = __ldca(s2), b = __ldca(s2 + 1), c = __ldca(s2 + 2);
  Box o;
  o.lo[0] = a.x;
  o.lo[1] = a.y;
  o.lo[2] = b.x;
  o.hi[0] = b.y;
  o.hi[1] = c.x;
  o.hi[2] = c.y;
  return o;
}

// A box stored by box_store, read through the read-only path.
__device__ __forceinline__ Box box_load_ro(const float* src) {
  const float2 a = __ldg(reinterpret_cast<const float2*>(src));
  const float2 b = __ldg(reinterpret_cast<const float2*>(src) + 1);
  const float2 c = __ldg(reinterpret_cast<const float2*>(src) + 2);
  Box o;
  o.lo[0] = a.x;
  o.lo[1] = a.y;
  o.lo[2] = b.x;
  o.hi[0] = b.y;
  o.hi[1] = c.x;
  o.hi[2] = c.y;
  return o;
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
template <bool kBox>
__global__ void __launch_bounds__(kThreads) k_centroid_aabb(uint32_t num_tri, const uint32_t* __restrict__ tri2vtx,
                                                           uint32_t num_vtx, const float* __restrict__ vtx2xyz,
                                                           float* partials, uint32_t* ticket, float* aabb_out,
                                                           float* transform_out, uint32_t* status, float* cent,
                                                           size_t stride, float* tribox) {
  __shared__ MinMax sh[kThreads / 32];
  __shared__ bool s_last;
  MinMax v;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    v.lo[d] = INFINITY;
    v.hi[d] = -INFINITY;
  }
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < num_tri; i += gridDim.x * kThreads) {
    float3 c;
    if constexpr (kBox) {
      Box tb;
      c = tri_centroid_box(tri2vtx, num_vtx, vtx2xyz, i, status, &tb);
      box_store(tribox + 6ull * i, tb);
    } else {
      c = tri_centroid(tri2vtx, num_vtx, vtx2xyz, i, status);
    }
    if (cent) {
      cent[i] = c.x;
      cent[stride + i] = c.y;
      cent[2 * stride + i] = c.z;
    }
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
    __threadfence();  // acquire: the other blocks' partials
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
// (bvhnodes_morton.rs:151-159 -> mortons.rs:115-138).  With kHist the digit
// histograms of the radix sort are accumulated: three of 10 bits (hist10) or
// four of 8 bits.
template <bool kHist>
__global__ void __launch_bounds__(kThreads) k_morton_tri(uint32_t num_tri, const uint32_t* __restrict__ tri2vtx,
                                                        uint32_t num_vtx, const float* __restrict__ vtx2xyz,
                                                        const float* __restrict__ transform,
                                                        uint32_t* __restrict__ codes, uint32_t* __restrict__ hist,
                                                        uint32_t* status, const float* cent, size_t stride,
                                                        bool hist10) {
  __shared__ float m[16];
  __shared__ uint32_t sh[kHist ? 3 * kRadix10 : 1];
  const int hist_words = hist10 ? 3 * kRadix10 : 4 * kRadix;
  // The mesh is an input of the whole build, so without stored centroids the
  // first centroid's gathers need not wait for the kernel that computes the
  // transform.
  const uint32_t i0 = blockIdx.x * kThreads + threadIdx.x;
  float3 c0 = make_float3(0.f, 0.f, 0.f);
  if (!cent && i0 < num_tri) c0 = tri_centroid(tri2vtx, num_vtx, vtx2xyz, i0, status);
  pdl_wait();
  pdl_launch_dependents();
  if (threadIdx.x < 16) m[threadIdx.x] = transform[threadIdx.x];
  if (kHist)
    for (int i = threadIdx.x; i < hist_words; i += kThreads) sh[i] = 0;
  __syncthreads();
  for (uint32_t i = i0; i < num_tri; i += gridDim.x * kThreads) {
    const float3 c = cent ? make_float3(cent[i], cent[stride + i], cent[2 * stride + i])
                          : (i == i0 ? c0 : tri_centroid(tri2vtx, num_vtx, vtx2xyz, i, status));
    const float3 q = transform_homogeneous(m, c.x, c.y, c.z);
    const uint32_t code = morton_code3(q.x, q.y, q.z);
    codes[i] = code;
    if (kHist) {
#pragma unroll
      if (hist10) {
        for (int p = 0; p < 3; ++p) atomicAdd(&sh[p * kRadix10 + ((code >> (10 * p)) & 0x3FFu)], 1u);
      } else {
        for (int p = 0; p < 4; ++p) atomicAdd(&sh[p * kRadix + ((code >> (8 * p)) & 0xFFu)], 1u);
      }
    }
  }
  if (kHist) {
    __syncthreads();
    for (int i = threadIdx.x; i < hist_words; i += kThreads)
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

template <int kTh>
__global__ void __launch_bounds__(kTh) k_topology(uint32_t n, const uint32_t* __restrict__ c,
                                                 const uint32_t* __restrict__ idx2obj, uint32_t* bvhnodes,
                                                 uint32_t* other_end) {
  pdl_wait();
  pdl_launch_dependents();
  const uint32_t ib = blockIdx.x * kTh + threadIdx.x;
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
__device__ __forceinline__ void refit_climb(uint32_t ii, uint32_t num_tri, const uint32_t* __restrict__ bvhnodes,
                                            const uint32_t* __restrict__ tri2vtx, uint32_t num_vtx,
                                            const float* __restrict__ vtx2xyz0, const float* __restrict__ vtx2xyz1,
                                            float* aabb, uint32_t* flags, uint32_t* height_out, uint32_t* status) {
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

// Grid-stride over the leaves (a leaf's climb never waits, so a thread may
// take several).
__global__ void __launch_bounds__(kThreads) k_refit(uint32_t num_tri, const uint32_t* __restrict__ bvhnodes,
                                                   const uint32_t* __restrict__ tri2vtx, uint32_t num_vtx,
                                                   const float* __restrict__ vtx2xyz0,
                                                   const float* __restrict__ vtx2xyz1, float* aabb, uint32_t* flags,
                                                   uint32_t* height_out, uint32_t* status, const uint32_t* gate) {
  // gated (drop-in refit): runs only when the tree was found not to be in
  // Karras leaf order, so that the range queries could not do the call
  if (gate != nullptr && (block_read_hdr(gate, nullptr).x & kRefitPlainClimb) == 0u) return;
  for (uint32_t ii = blockIdx.x * kThreads + threadIdx.x; ii < num_tri; ii += gridDim.x * kThreads)
    refit_climb(ii, num_tri, bvhnodes, tri2vtx, num_vtx, vtx2xyz0, vtx2xyz1, aabb, flags, height_out, status);
}

// Tree-order refit, in two kernels: the path taken when a leaf box holds NaN
// (where the merge order matters) or when tree heights are asked for; the
// range-query refit further below handles every other call, and these two
// kernels then exit at once.
//
// k_refit_win takes the windows of kRefitWindow sorted leaves (global leaf
// order, across the meshes of a batch; each block loops over windows).  It
// writes their leaf boxes and climbs from them through every branch whose
// whole leaf range lies in the window ("local": known from other_end, since
// a branch index is one end of its range).  Both arrivals at a local branch
// come from this block, so its arrival counter and child boxes live in
// shared memory and the whole local climb reads no global memory.
//
// A climb that reaches a branch whose range crosses the window edge stops
// there.  At a crossing branch it makes the global acquire-release arrival
// of k_refit; the first arriver is done, the second merges the branch and
// hands its parent to k_refit_top through a small queue.  Only the LCA of a
// window boundary can get both arrivals here, and only the link just below a
// window can be reached from a local right child, so the queue holds at most
// two entries per window.  k_refit_top climbs the remaining top of the tree
// from the queue entries with global arrivals.
//
// Link chains (branch j with left child leaf j and right child branch j+1; a
// run of equal Morton codes is one long chain) need no arrival counter: the
// leaf of a link never climbs, and the climb that completes branch j+1 folds
// the chain upward, box(j) = from_two(leaf j, box(j+1)).  In k_refit_top the
// fold prefetches eight links at a time (their records and leaf boxes sit at
// consecutive addresses).  Values and merge order are those of k_refit.
constexpr int kWinThreads = 512;
constexpr int kWinPerThread = kRefitWindow / kWinThreads;
constexpr int kFoldDepth = 8;
static_assert(kWinPerThread * kWinThreads == kRefitWindow, "window");
static_assert(kWinThreads >= kRefitWinHeap, "a thread per stored window-heap node");

// The records and other ends of branches wA..wA+kRefitWindow-1 (every local
// branch has its index in the window) are loaded into shared memory once.
struct WinSmem {
  uint32_t flag[kRefitWindow];
  uint32_t rec[kRefitWindow][4];  // parent, left, right, other end
  Box leaf[kRefitWindow];
  Box node[kRefitWindow];
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

// Hand-over queue: word 0 counts entries; entries {branch, child, height,
// global leaf} start at word kRefitQueueHdr.
__device__ __forceinline__ void queue_push(uint32_t* queue, uint32_t capacity, uint32_t node, uint32_t prev,
                                           uint32_t h, uint32_t leaf, uint32_t* status) {
  const uint32_t slot = atomicAdd(queue, 1u);
  if (slot >= capacity) {
    raise_status(status, kStatusBadIndex);
    return;
  }
  reinterpret_cast<uint4*>(queue + kRefitQueueHdr)[slot] = make_uint4(node, prev, h, leaf);
}

template <bool kBatch>
__global__ void __launch_bounds__(kWinThreads) k_refit_win(uint32_t total_tri, Segments seg, uint32_t num_vtx_single,
                                                          const uint32_t* __restrict__ bvhnodes_all,
                                                          const uint32_t* __restrict__ other_all,
                                                          const uint32_t* __restrict__ tri2vtx_all,
                                                          const float* __restrict__ vtx0_all,
                                                          const float* __restrict__ vtx1_all, float* aabb_all,
                                                          uint32_t* gflags_all, uint32_t* queue, uint32_t capacity,
                                                          uint32_t* height_out, uint32_t* status) {
  pdl_wait();
  pdl_launch_dependents();
  // runs only when the range-query refit handed over (NaN) or heights are
  // wanted, and not for a tree that is not in Karras leaf order (the plain
  // climb of k_refit does that call)
  const uint32_t climb_flag = block_read_hdr(queue + 1, nullptr).x;
  if (climb_flag == 0u || (climb_flag & kRefitPlainClimb) != 0u) return;
  extern __shared__ __align__(16) unsigned char win_raw[];
  WinSmem& S = *reinterpret_cast<WinSmem*>(win_raw);
  // persistent over the windows: when the range queries did the work, the
  // early exit above costs one wave instead of one block per window
  const uint32_t num_win = (total_tri + kRefitWindow - 1) / kRefitWindow;
  for (uint32_t win = blockIdx.x; win < num_win; win += gridDim.x) {
    const uint32_t wA = win * kRefitWindow;

    // Phase 0: leaf boxes, branch records and other ends of the window.  The
    // dependent loads (leaf record -> triangle -> vertices) of both leaves of a
    // thread are issued together.
    LeafMesh lm[kWinPerThread];
    uint32_t par[kWinPerThread];
#pragma unroll
    for (int r = 0; r < kWinPerThread; ++r) {
      const uint32_t k = threadIdx.x + r * kWinThreads, g = wA + k;
      S.flag[k] = 0u;
      lm[r] = leaf_mesh<kBatch>(seg, total_tri, num_vtx_single, g < total_tri ? g : 0u);
      if (g >= total_tri) lm[r].ok = false;
      par[r] = kUMax;
    }
    uint32_t tri[kWinPerThread];
#pragma unroll
    for (int r = 0; r < kWinPerThread; ++r) {
      const uint32_t k = threadIdx.x + r * kWinThreads;
      tri[r] = kUMax;
      if (!lm[r].ok) continue;
      const size_t node_off = 2ull * lm[r].t0 - lm[r].m;
      const uint32_t n = wA + k - lm[r].t0;
      const uint32_t* lr = bvhnodes_all + 3 * (node_off + lm[r].T - 1 + n);
      par[r] = __ldg(lr);
      tri[r] = __ldg(lr + 1);
      if (n + 1 < lm[r].T) {
        const uint32_t* br = bvhnodes_all + 3 * (node_off + n);
        S.rec[k][0] = __ldg(br);
        S.rec[k][1] = __ldg(br + 1);
        S.rec[k][2] = __ldg(br + 2);
        S.rec[k][3] = __ldg(other_all + (static_cast<size_t>(lm[r].t0) - lm[r].m) + n);
      }
    }
#pragma unroll
    for (int r = 0; r < kWinPerThread; ++r) {
      const uint32_t k = threadIdx.x + r * kWinThreads;
      if (!lm[r].ok) continue;
      if (tri[r] >= lm[r].T) {
        raise_status(status, kStatusBadIndex);
        tri[r] = 0u;
      }
      const uint32_t* t2v = tri2vtx_all + 3ull * lm[r].t0;
      const float* v0 = vtx0_all + 3ull * lm[r].v0;
      Box bx = leaf_box(t2v, lm[r].V, v0, tri[r], status);
      if (vtx1_all) bx = box_union(bx, leaf_box(t2v, lm[r].V, vtx1_all + 3ull * lm[r].v0, tri[r], status));
      S.leaf[k] = bx;
      const size_t node_off = 2ull * lm[r].t0 - lm[r].m;
      box_store(aabb_all + 6 * (node_off + lm[r].T - 1 + (wA + k - lm[r].t0)), bx);
    }
    __syncthreads();

    // Phase 1: climb the local branches.
#pragma unroll
    for (int r = 0; r < kWinPerThread; ++r) {
      if (!lm[r].ok) continue;
      const uint32_t k = threadIdx.x + r * kWinThreads;
      const uint32_t t0 = lm[r].t0, T = lm[r].T;
      const size_t node_off = 2ull * t0 - lm[r].m, int_off = static_cast<size_t>(t0) - lm[r].m;
      const uint32_t* bn = bvhnodes_all + 3 * node_off;
      float* aabb = aabb_all + 6 * node_off;
      const uint32_t num_node = 2 * T - 1;
      const uint32_t n = wA + k - t0;
      const uint32_t leaf = T - 1 + n;
      uint32_t node = par[r];
      // the left leaf of a link is folded in by the climb through the chain
      if (node == n && n + 1 < T - 1 && S.rec[k][1] == leaf && S.rec[k][2] == n + 1) continue;
      Box b = S.leaf[k];
      uint32_t h = 1, prev = leaf, guard = 0;
      while (node != kUMax) {
        if (node >= T - 1 || ++guard > num_node) {
          raise_status(status, kStatusBadIndex);
          break;
        }
        const uint32_t slot = t0 + node - wA;  // wraps to a large value below the window
        bool local = slot < static_cast<uint32_t>(kRefitWindow);
        uint32_t parent = 0, c0 = 0, c1 = 0;
        if (local) {
          parent = S.rec[slot][0];
          c0 = S.rec[slot][1];
          c1 = S.rec[slot][2];
          const uint32_t other = S.rec[slot][3];
          const uint32_t lo = node < other ? node : other, hi = node < other ? other : node;
          local = (t0 + lo >= wA) && (t0 + hi < wA + kRefitWindow);
        }
        if (!local) {
          // crossing branch: one global step, then stop
          parent = __ldg(bn + static_cast<size_t>(node) * 3);
          c0 = __ldg(bn + static_cast<size_t>(node) * 3 + 1);
          c1 = __ldg(bn + static_cast<size_t>(node) * 3 + 2);
          if (c0 == T - 1 + node && c1 == node + 1 && prev == c1) {
            queue_push(queue, capacity, node, prev, h, wA + k, status);
            break;
          }
          cuda::atomic_ref<uint32_t, cuda::thread_scope_device> arrival(gflags_all[int_off + node]);
          const uint32_t old = arrival.fetch_add(h, cuda::memory_order_acq_rel);
          if (old == 0u) break;
          gflags_all[int_off + node] = 0u;
          h = (old > h ? old : h) + 1;
          if (c0 >= num_node || c1 >= num_node || (c0 != prev && c1 != prev)) {
            raise_status(status, kStatusBadIndex);
            break;
          }
          const bool mine_first = (c0 == prev);
          const Box sb = box_load_cg(aabb + static_cast<size_t>(mine_first ? c1 : c0) * 6);
          b = mine_first ? box_union(b, sb) : box_union(sb, b);
          box_store(aabb + static_cast<size_t>(node) * 6, b);
          if (parent != kUMax) queue_push(queue, capacity, parent, node, h, wA + k, status);
          else if (height_out) height_out[lm[r].m] = h;
          break;
        }
        if (c0 == T - 1 + node && c1 == node + 1 && prev == c1) {
          // link reached from its right child: no arrival, its leaf is in the window
          b = box_union(S.leaf[slot], b);
          box_store(aabb + static_cast<size_t>(node) * 6, b);
          S.node[slot] = b;
          h += 1;
          prev = node;
          node = parent;
          continue;
        }
        __threadfence_block();  // this thread's shared box is visible before the arrival
        const uint32_t old = atomicAdd(&S.flag[slot], h);
        if (old == 0u) break;
        __threadfence_block();
        h = (old > h ? old : h) + 1;
        if (c0 >= num_node || c1 >= num_node || (c0 != prev && c1 != prev)) {
          raise_status(status, kStatusBadIndex);
          break;
        }
        const bool mine_first = (c0 == prev);
        const uint32_t sib = mine_first ? c1 : c0;
        // a valid tree keeps the sibling inside the window; check it anyway
        const uint32_t sslot = (sib >= T - 1) ? t0 + (sib - (T - 1)) - wA : t0 + sib - wA;
        if (sslot >= static_cast<uint32_t>(kRefitWindow)) {
          raise_status(status, kStatusBadIndex);
          break;
        }
        const Box sb = (sib >= T - 1) ? S.leaf[sslot] : S.node[sslot];
        b = mine_first ? box_union(b, sb) : box_union(sb, b);
        box_store(aabb + static_cast<size_t>(node) * 6, b);
        S.node[slot] = b;
        prev = node;
        node = parent;
      }
      if (node == kUMax && height_out) height_out[lm[r].m] = h;
    }
    __syncthreads();  // the next window reuses the shared arrays
  }
}

// The top of the tree: one thread per queue entry, global arrivals as in
// k_refit, link chains folded kFoldDepth links per round trip.
template <bool kBatch>
__global__ void __launch_bounds__(128) k_refit_top(uint32_t total_tri, Segments seg,
                                                   const uint32_t* __restrict__ bvhnodes_all, float* aabb_all,
                                                   uint32_t* gflags_all, const uint32_t* queue, uint32_t capacity,
                                                   uint32_t* height_out, uint32_t* status) {
  pdl_wait();
  pdl_launch_dependents();
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t count = block_read_hdr(queue, nullptr).x;
  if (e >= count || e >= capacity) return;
  const uint4 q = __ldcg(reinterpret_cast<const uint4*>(queue + kRefitQueueHdr) + e);
  const LeafMesh lm = leaf_mesh<kBatch>(seg, total_tri, 0u, q.w < total_tri ? q.w : 0u);
  if (!lm.ok || q.w >= total_tri) {
    raise_status(status, kStatusBadIndex);
    return;
  }
  const uint32_t T = lm.T, num_node = 2 * T - 1;
  const size_t node_off = 2ull * lm.t0 - lm.m;
  const uint32_t* bn = bvhnodes_all + 3 * node_off;
  float* aabb = aabb_all + 6 * node_off;
  uint32_t* gflags = gflags_all + (static_cast<size_t>(lm.t0) - lm.m);
  uint32_t node = q.x, prev = q.y, h = q.z, guard = 0;
  if (prev >= num_node) {
    raise_status(status, kStatusBadIndex);
    return;
  }
  Box b = box_load_cg(aabb + static_cast<size_t>(prev) * 6);
  while (node != kUMax) {
    if (node >= T - 1 || ++guard > num_node) {
      raise_status(status, kStatusBadIndex);
      return;
    }
    const uint32_t parent = __ldg(bn + static_cast<size_t>(node) * 3);
    const uint32_t c0 = __ldg(bn + static_cast<size_t>(node) * 3 + 1);
    const uint32_t c1 = __ldg(bn + static_cast<size_t>(node) * 3 + 2);
    if (c0 == T - 1 + node && c1 == node + 1 && prev == c1) {
      // fold the chain from link j = node upward, kFoldDepth links per round
      uint32_t j = node, pj = parent;
      for (;;) {
        Box lb[kFoldDepth];
        uint32_t rp[kFoldDepth], rl[kFoldDepth], rr[kFoldDepth];  // records of j-1-d
#pragma unroll
        for (int d = 0; d < kFoldDepth; ++d) {
          if (j >= static_cast<uint32_t>(d)) lb[d] = box_load_cg(aabb + static_cast<size_t>(T - 1 + j - d) * 6);
          if (j >= static_cast<uint32_t>(d) + 1) {
            const uint32_t* r = bn + static_cast<size_t>(j - 1 - d) * 3;
            rp[d] = __ldg(r);
            rl[d] = __ldg(r + 1);
            rr[d] = __ldg(r + 2);
          } else {
            rp[d] = rl[d] = rr[d] = kUMax;
          }
        }
        bool more = true;
#pragma unroll
        for (int d = 0; d < kFoldDepth; ++d) {
          if (!more) continue;
          const uint32_t jj = j - d;  // a link whose right child is complete
          b = box_union(lb[d], b);
          box_store(aabb + static_cast<size_t>(jj) * 6, b);
          h += 1;
          prev = jj;
          if (++guard > num_node) {
            raise_status(status, kStatusBadIndex);
            return;
          }
          const uint32_t up = (d == 0) ? pj : rp[d - 1];  // parent of jj
          node = up;
          more = jj >= 1 && up == jj - 1 && rl[d] == T - 1 + up && rr[d] == jj;
        }
        if (!more) break;
        j -= kFoldDepth;
        pj = rp[kFoldDepth - 1];
      }
      continue;
    }
    cuda::atomic_ref<uint32_t, cuda::thread_scope_device> arrival(gflags[node]);
    const uint32_t old = arrival.fetch_add(h, cuda::memory_order_acq_rel);
    if (old == 0u) return;
    gflags[node] = 0u;
    h = (old > h ? old : h) + 1;
    if (c0 >= num_node || c1 >= num_node || (c0 != prev && c1 != prev)) {
      raise_status(status, kStatusBadIndex);
      return;
    }
    const bool mine_first = (c0 == prev);
    const Box sb = box_load_cg(aabb + static_cast<size_t>(mine_first ? c1 : c0) * 6);
    b = mine_first ? box_union(b, sb) : box_union(sb, b);
    box_store(aabb + static_cast<size_t>(node) * 6, b);
    prev = node;
    node = parent;
  }
  if (height_out) height_out[lm.m] = h;
}

// ------------------------------------------------------- range-query refit
//
// Without NaN, box_union(a, b) keeps a unless b is strictly smaller (lo) /
// larger (hi), an associative operation whose fold over any tree is the
// leftmost extreme of the leaves below.  So branch i's box equals the fold of
// the leaf boxes over its leaf range [min(i, other_end[i]), max(...)], which a
// segment tree over the sorted leaf boxes answers with no climb at all.
// The tree is a perfect binary heap per kRefitWindow-leaf window (nodes of 8
// leaves and up kept), per 64-window superblock and over the superblocks; only nodes
// lying wholly inside [0, total_tri) are ever built or read.  Identity boxes
// are (+inf, -inf), which box_union returns unchanged bit for bit.
struct SegView {
  const float* wseg;  // [window][kRefitWinHeap] boxes, heap index 1..kRefitWinHeap - 1
  const float* sseg;  // [superblock][64] boxes, heap index 1..63
  const float* tseg;  // [2 << top_log] boxes, heap index 1..
  uint32_t top_log;
};

__device__ __forceinline__ const float* seg_node(const SegView& v, uint32_t lvl, uint32_t j) {
  if (lvl <= kRefitWindowLog) {
    const uint32_t sh = kRefitWindowLog - lvl;
    return v.wseg + 6 * (static_cast<size_t>(j >> sh) * kRefitWinHeap + (1u << sh) + (j & ((1u << sh) - 1)));
  }
  if (lvl <= kRefitSuperLog) {
    const uint32_t sh = kRefitSuperLog - lvl;
    return v.sseg + 6 * (static_cast<size_t>(j >> sh) * 64 + (1u << sh) + (j & ((1u << sh) - 1)));
  }
  const uint32_t sh = kRefitSuperLog + v.top_log - lvl;
  return v.tseg + 6 * ((static_cast<size_t>(1) << sh) + j);
}

__device__ __forceinline__ Box box_identity() {
  return Box{{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
}

__device__ __forceinline__ bool box_has_nan(const Box& b) {
  bool n = false;
#pragma unroll
  for (int d = 0; d < 3; ++d) n = n || (b.lo[d] != b.lo[d]) || (b.hi[d] != b.hi[d]);
  return n;
}

// heap node h (1-based) of a heap whose leaves sit at level leaf_lvl: its
// level and index within that level
__device__ __forceinline__ void heap_node(uint32_t h, uint32_t top_lvl, uint32_t& lvl, uint32_t& j) {
  const uint32_t lg = 31u - __clz(h);
  lvl = top_lvl - lg;
  j = h - (1u << lg);
}

__device__ __forceinline__ bool node_inside(uint64_t start_leaf, uint32_t lvl, uint32_t j, uint32_t total) {
  return start_leaf + ((static_cast<uint64_t>(j) + 1) << lvl) <= total;
}

// Mesh of global leaf g, walking forward from a block-wide starting mesh.
__device__ __forceinline__ uint32_t mesh_from(const Segments& seg, uint32_t m0, uint32_t g) {
  uint32_t m = m0;
  while (m + 1 < seg.num_mesh && __ldg(seg.tri_off + m + 1) <= g) ++m;
  return m;
}

constexpr int kSegWinSmem = static_cast<int>(2 * kRefitWindow * sizeof(Box));

// Window kernel: leaf boxes, the window heap, and every branch whose range
// lies inside the window.  kRuns (one mesh only): set aside the run branches
// for refit_runs (below).
template <bool kBatch, bool kRuns>
__global__ void __launch_bounds__(kWinThreads) k_refit_seg_win(uint32_t total_tri, Segments seg,
                                                              uint32_t num_vtx_single,
                                                              const uint32_t* __restrict__ bvhnodes_all,
                                                              const uint32_t* __restrict__ other_all,
                                                              const uint32_t* __restrict__ tri2vtx_all,
                                                              const float* __restrict__ vtx0_all,
                                                              const float* __restrict__ vtx1_all, float* aabb_all,
                                                              uint32_t* hdr, uint32_t* cross_list, float* wseg,
                                                              uint32_t* status, const float* __restrict__ tribox,
                                                              const uint32_t* __restrict__ leaf_tri) {
  extern __shared__ __align__(16) unsigned char seg_raw[];
  Box* tree = reinterpret_cast<Box*>(seg_raw);  // 2 * kRefitWindow boxes
  __shared__ uint32_t s_mesh, s_flag, s_bstar, s_runs;
  const uint32_t wA = blockIdx.x * kRefitWindow;
  static_assert(!(kBatch && kRuns), "run branches are set aside for one mesh only");
  if (threadIdx.x == 0) {
    if (kRuns) s_runs = 0u;
    // another block may raise the flag meanwhile: read it once for the block
    s_flag = *reinterpret_cast<volatile uint32_t*>(hdr + 1);
    if (kBatch) s_mesh = mesh_of_leaf(seg, wA);
  }
  __syncthreads();
  if (s_flag != 0u) return;  // the climb does this call
  LeafMesh lm[kWinPerThread];
  uint32_t tri[kWinPerThread], oth[kWinPerThread];
#pragma unroll
  for (int r = 0; r < kWinPerThread; ++r) {
    const uint32_t k = threadIdx.x + r * kWinThreads, g = wA + k;
    lm[r] = LeafMesh{0, 0, total_tri, 0, num_vtx_single, g < total_tri};
    if (kBatch && g < total_tri) {
      const uint32_t m = mesh_from(seg, s_mesh, g);
      lm[r].m = m;
      lm[r].t0 = __ldg(seg.tri_off + m);
      lm[r].T = __ldg(seg.tri_off + m + 1) - lm[r].t0;
      lm[r].v0 = __ldg(seg.vtx_off + m);
      lm[r].V = __ldg(seg.vtx_off + m + 1) - lm[r].v0;
      lm[r].ok = !(g < lm[r].t0 || g - lm[r].t0 >= lm[r].T || lm[r].T > 0x7FFFFFFFu);
    }
    tri[r] = 0u;
    oth[r] = kUMax;
    if (!lm[r].ok) continue;
    const uint32_t n = g - lm[r].t0;
    // the leaf's triangle: from the sorted indices when given (contiguous),
    // else from its record (12-byte stride)
    tri[r] = (!kBatch && leaf_tri) ? __ldg(leaf_tri + g)
                                   : __ldg(bvhnodes_all + 3 * (2ull * lm[r].t0 - lm[r].m + lm[r].T - 1 + n) + 1);
    if (n + 1 < lm[r].T) oth[r] = __ldg(other_all + (static_cast<size_t>(lm[r].t0) - lm[r].m) + n);
  }
  if (kRuns && threadIdx.x == kWinThreads - 1) {
    // the window's last branch, when its range starts inside the window and
    // ends beyond it: its right end b* is shared by every branch of a run of
    // equal codes that crosses the right edge
    constexpr int rl = kWinPerThread - 1;
    const uint32_t g = wA + kRefitWindow - 1;
    uint32_t bstar = kUMax;
    if (oth[rl] != kUMax) {
      const uint32_t lo = g < oth[rl] ? g : oth[rl], hi = g < oth[rl] ? oth[rl] : g;
      if (lo >= wA && hi > g && hi < total_tri) bstar = hi;
    }
    s_bstar = bstar;
  }
  bool nan = false;
#pragma unroll
  for (int r = 0; r < kWinPerThread; ++r) {
    const uint32_t k = threadIdx.x + r * kWinThreads;
    Box bx = box_identity();
    if (lm[r].ok) {
      if (tri[r] >= lm[r].T) {
        raise_status(status, kStatusBadIndex);
        tri[r] = 0u;
      }
      const uint32_t* t2v = tri2vtx_all + 3ull * lm[r].t0;
      if (tribox) {  // boxes the centroid pass computed (one mesh, one vertex state)
        bx = box_load_ro(tribox + 6ull * (lm[r].t0 + tri[r]));
      } else {
        bx = leaf_box(t2v, lm[r].V, vtx0_all + 3ull * lm[r].v0, tri[r], status);
        if (vtx1_all) bx = box_union(bx, leaf_box(t2v, lm[r].V, vtx1_all + 3ull * lm[r].v0, tri[r], status));
      }
      box_store(aabb_all + 6 * (2ull * lm[r].t0 - lm[r].m + lm[r].T - 1 + (wA + k - lm[r].t0)), bx);
      nan = nan || box_has_nan(bx);
    }
    tree[kRefitWindow + k] = bx;
  }
  if (__syncthreads_or(nan)) {
    if (threadIdx.x == 0) atomicOr(hdr + 1, 1u);  // hand the whole call to the climb
    return;
  }
  // Run branches: ranges [a, b*] with a inside the window (chain links of a
  // run of equal codes crossing the right edge).  When the window holds at
  // least kRefitRunMin of them, each gets its in-window part fold(a .. wEnd)
  // below and refit_runs folds in the shared fold(wEnd + 1 .. b*) once per
  // window; the window's heap slot 0 (otherwise unused) tells it b*.  Counted
  // here; the heap build's barriers order the count before its use.
  uint32_t run_mask = 0u;
  if (kRuns && s_bstar != kUMax) {
    const uint32_t bstar = s_bstar;
#pragma unroll
    for (int r = 0; r < kWinPerThread; ++r) {
      const uint32_t g = wA + threadIdx.x + r * kWinThreads;
      const bool run = oth[r] != kUMax && (g < oth[r] ? g : oth[r]) >= wA && (g < oth[r] ? oth[r] : g) == bstar;
      if (run) run_mask |= 1u << r;
      const uint32_t bal = __ballot_sync(0xffffffffu, run);
      if ((threadIdx.x & 31u) == 0u && bal != 0u) atomicAdd(&s_runs, static_cast<uint32_t>(__popc(bal)));
    }
  }
  // heap levels of 64 .. kRefitWindow / 2 nodes by the block, the top six
  // levels (32 .. 1 nodes) by warp 0 alone
#pragma unroll 1
  for (uint32_t half = kRefitWindow / 2; half > 32; half >>= 1) {
    for (uint32_t h = half + threadIdx.x; h < 2 * half; h += kWinThreads) tree[h] = box_union(tree[2 * h], tree[2 * h + 1]);
    __syncthreads();
  }
  if (threadIdx.x < 32) {
#pragma unroll
    for (uint32_t half = 32; half >= 1; half >>= 1) {
      if (threadIdx.x < half) tree[half + threadIdx.x] = box_union(tree[2 * (half + threadIdx.x)], tree[2 * (half + threadIdx.x) + 1]);
      __syncwarp();
    }
  }
  __syncthreads();
  // heap nodes of 8 leaves and up for the crossing queries
  if (threadIdx.x >= 1 && threadIdx.x < kRefitWinHeap) {
    uint32_t lvl, j;
    heap_node(threadIdx.x, kRefitWindowLog, lvl, j);
    if (node_inside(wA, lvl, j, total_tri)) box_store(wseg + 6 * (static_cast<size_t>(blockIdx.x) * kRefitWinHeap + threadIdx.x), tree[threadIdx.x]);
  }
  const bool runs = kRuns && s_bstar != kUMax && s_runs >= kRefitRunMin;
  if (kRuns && threadIdx.x == 0) {
    *reinterpret_cast<uint32_t*>(wseg + 6 * static_cast<size_t>(blockIdx.x) * kRefitWinHeap) = runs ? s_bstar : kUMax;
    if (runs) atomicOr(hdr + 4, 1u);  // refit_runs has work
  }
#pragma unroll
  for (int r = 0; r < kWinPerThread; ++r) {
    if (oth[r] == kUMax) continue;
    const uint32_t g = wA + threadIdx.x + r * kWinThreads, n = g - lm[r].t0;
    const uint32_t lo = n < oth[r] ? n : oth[r], hi = n < oth[r] ? oth[r] : n;
    if (hi >= lm[r].T) {
      raise_status(status, kStatusBadIndex);
      continue;
    }
    const uint32_t a = lm[r].t0 + lo, b = lm[r].t0 + hi;
    if (runs && (run_mask >> r & 1u)) {  // in-window part [a, wEnd]
      uint32_t l = a - wA + kRefitWindow, rr = 2 * kRefitWindow;
      Box L = box_identity(), R = box_identity();
      while (l < rr) {
        if (l & 1u) L = box_union(L, tree[l++]);
        if (rr & 1u) R = box_union(tree[--rr], R);
        l >>= 1;
        rr >>= 1;
      }
      box_store(aabb_all + 6 * static_cast<size_t>(n), box_union(L, R));
      continue;
    }
    if ((a >> kRefitWindowLog) != (b >> kRefitWindowLog)) {
      // crossing: listed for k_refit_seg_cross in the (zero) arrival
      // counters, which that kernel clears again as it reads them
      const uint32_t slot = atomicAdd(hdr + 3, 1u);
      if (slot < total_tri) cross_list[slot] = g + 1;  // + 1: a listed entry is never zero
      else raise_status(status, kStatusBadIndex);      // more than total_tri - 1 branches: not a tree
      continue;
    }
    uint32_t l = a - wA + kRefitWindow, rr = b - wA + kRefitWindow + 1;
    Box L = box_identity(), R = box_identity();
    while (l < rr) {
      if (l & 1u) L = box_union(L, tree[l++]);
      if (rr & 1u) R = box_union(tree[--rr], R);
      l >>= 1;
      rr >>= 1;
    }
    box_store(aabb_all + 6 * (2ull * lm[r].t0 - lm[r].m + n), box_union(L, R));
  }
}

// Superblock heaps from the window totals; the last block builds the top heap.
constexpr uint32_t kTopSmem = 256;
__global__ void __launch_bounds__(256) k_refit_seg_super(uint32_t total_tri, uint32_t* hdr, const float* wseg,
                                                         float* sseg, float* tseg, uint32_t top_log) {
  __shared__ Box t[2 * kRefitSuper];
  __shared__ Box ttop[2 * kTopSmem];  // the top heap, when it fits
  __shared__ bool s_last;
  pdl_wait();
  pdl_launch_dependents();
  if (block_read_hdr(hdr + 1, nullptr).x != 0u) return;
  const uint32_t sb = blockIdx.x;
  const uint64_t sb_start = static_cast<uint64_t>(sb) << kRefitSuperLog;
  if (threadIdx.x < kRefitSuper) {
    const uint32_t w = sb * kRefitSuper + threadIdx.x;
    t[kRefitSuper + threadIdx.x] = (static_cast<uint64_t>(w + 1) << kRefitWindowLog) <= total_tri
                                       ? box_load_cg(wseg + 6 * (static_cast<size_t>(w) * kRefitWinHeap + 1))
                                       : box_identity();
  }
  __syncthreads();
#pragma unroll 1
  for (uint32_t half = kRefitSuper / 2; half >= 1; half >>= 1) {
    if (threadIdx.x < half) {
      const uint32_t h = half + threadIdx.x;
      t[h] = box_union(t[2 * h], t[2 * h + 1]);
    }
    __syncthreads();
  }
  if (threadIdx.x >= 1 && threadIdx.x < kRefitSuper) {
    uint32_t lvl, j;
    heap_node(threadIdx.x, kRefitSuperLog, lvl, j);
    if (node_inside(sb_start, lvl, j, total_tri)) box_store(sseg + 6 * (static_cast<size_t>(sb) * 64 + threadIdx.x), t[threadIdx.x]);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();  // release: the block's heap nodes (seen through the barrier) before the ticket
    s_last = atomicAdd(hdr + 2, 1u) == gridDim.x - 1;
    __threadfence();  // acquire: the other blocks' heap nodes
  }
  __syncthreads();
  if (!s_last) return;
  const uint32_t leaves = 1u << top_log, top_lvl = kRefitSuperLog + top_log;
  if (leaves <= kTopSmem) {
    for (uint32_t s = threadIdx.x; s < leaves; s += blockDim.x)
      ttop[leaves + s] = (static_cast<uint64_t>(s + 1) << kRefitSuperLog) <= total_tri
                             ? box_load_cg(sseg + 6 * (static_cast<size_t>(s) * 64 + 1))
                             : box_identity();
    __syncthreads();
#pragma unroll 1
    for (uint32_t half = leaves / 2; half >= 1; half >>= 1) {
      for (uint32_t h = half + threadIdx.x; h < 2 * half; h += blockDim.x) ttop[h] = box_union(ttop[2 * h], ttop[2 * h + 1]);
      __syncthreads();
    }
    for (uint32_t h = 1 + threadIdx.x; h < 2 * leaves; h += blockDim.x) {
      uint32_t lvl, j;
      heap_node(h, top_lvl, lvl, j);
      if (node_inside(0, lvl, j, total_tri)) box_store(tseg + 6 * static_cast<size_t>(h), ttop[h]);
    }
    return;
  }
  for (uint32_t s = threadIdx.x; s < leaves; s += blockDim.x)
    if ((static_cast<uint64_t>(s + 1) << kRefitSuperLog) <= total_tri)
      box_store(tseg + 6 * (static_cast<size_t>(leaves) + s), box_load_cg(sseg + 6 * (static_cast<size_t>(s) * 64 + 1)));
  __syncthreads();
#pragma unroll 1
  for (uint32_t half = leaves / 2; half >= 1; half >>= 1) {
    for (uint32_t h = half + threadIdx.x; h < 2 * half; h += blockDim.x) {
      uint32_t lvl, j;
      heap_node(h, top_lvl, lvl, j);
      if (node_inside(0, lvl, j, total_tri))
        box_store(tseg + 6 * static_cast<size_t>(h),
                  box_union(box_load_cg(tseg + 12 * static_cast<size_t>(h)), box_load_cg(tseg + 12 * static_cast<size_t>(h) + 6)));
    }
    __syncthreads();
  }
}

// One crossing branch (global position g of its index): the segment-tree
// query over its leaf range.
__device__ __forceinline__ Box box_shfl_down(const Box& b, uint32_t delta, uint32_t mask) {
  Box o;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    o.lo[d] = __shfl_down_sync(mask, b.lo[d], delta, 8);
    o.hi[d] = __shfl_down_sync(mask, b.hi[d], delta, 8);
  }
  return o;
}

// Ordered union over the 8 lanes of a group, lane order ascending (kAsc) or
// descending; lane 0 of the group gets the result.  box_union keeps its left
// operand on ties, so the order of the operands is that of the leaves.
template <bool kAsc>
__device__ __forceinline__ Box group_union(Box x, uint32_t sub, uint32_t mask) {
#pragma unroll
  for (uint32_t off = 1; off < 8; off <<= 1) {
    const Box y = box_shfl_down(x, off, mask);
    if ((sub & (2 * off - 1)) == 0) x = kAsc ? box_union(x, y) : box_union(y, x);
  }
  return x;
}

// Box of branch g (global leaf position of its Karras index) whose range
// crosses a window edge, by 8 lanes: the range [l, r) of leaves is the
// ragged leaves at both ends (up to 7 each) plus, per level k >= 3 of the
// segment tree, at most one node on each side.  With L = the first and R =
// the last-plus-one level-3 index, the iterative walk (if l odd take l++; if
// r odd take --r; halve) is at level 3+j at l_j = ceil(L / 2^j) and
// r_j = floor(R / 2^j) while l_j < r_j, so every lane finds its own levels
// (4 consecutive ones) without walking the others.  In leaf order the pieces
// are: left ragged leaves, left nodes by ascending level, right nodes by
// descending level, right ragged leaves.
template <bool kBatch>
__device__ __forceinline__ void refit_cross_group(uint32_t g, uint32_t sub, uint32_t mask, uint32_t total_tri,
                                                  const Segments& seg, const uint32_t* __restrict__ other_all,
                                                  float* aabb_all, const SegView& v, uint32_t* status) {
  uint32_t m = 0, t0 = 0, T = total_tri;
  if (kBatch) {
    m = mesh_of_leaf(seg, g);
    t0 = __ldg(seg.tri_off + m);
    T = __ldg(seg.tri_off + m + 1) - t0;
  }
  const uint32_t n = g - t0;
  if (g < t0 || n + 1 >= T) {
    if (sub == 0) raise_status(status, kStatusBadIndex);
    return;
  }
  const uint32_t oth = __ldg(other_all + (static_cast<size_t>(t0) - m) + n);
  const uint32_t lo = n < oth ? n : oth, hi = n < oth ? oth : n;
  if (hi >= T) {
    if (sub == 0) raise_status(status, kStatusBadIndex);
    return;
  }
  const uint32_t l = t0 + lo, r = t0 + hi + 1;
  const float* leaf0 = aabb_all + 6 * (2ull * t0 - m + T - 1) - 6ull * t0;  // + 6*p: leaf of global position p
  const uint32_t nl = (8u - (l & 7u)) & 7u, nr = r & 7u;
  const uint32_t L = (l + nl) >> 3, R = (r - nr) >> 3;
  const float* pa = sub < nl ? leaf0 + 6ull * (l + sub) : nullptr;
  const float* pb = sub < nr ? leaf0 + 6ull * (r - nr + sub) : nullptr;
  const float* pl[4];
  const float* pr[4];
#pragma unroll
  for (uint32_t q = 0; q < 4; ++q) {
    const uint32_t j = 4 * sub + q;
    const uint32_t lj = static_cast<uint32_t>((static_cast<uint64_t>(L) + (1ull << j) - 1) >> j);
    const uint32_t rj = static_cast<uint32_t>(static_cast<uint64_t>(R) >> j);
    const bool act = lj < rj;
    pl[q] = (act && (lj & 1u)) ? seg_node(v, 3 + j, lj) : nullptr;
    pr[q] = (act && (rj & 1u)) ? seg_node(v, 3 + j, rj - 1) : nullptr;
  }
  const Box id = box_identity();
  Box A = pa ? box_load_l1(pa) : id, B = pb ? box_load_l1(pb) : id;
  Box bl[4], br[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    bl[q] = pl[q] ? box_load_l1(pl[q]) : id;
    br[q] = pr[q] ? box_load_l1(pr[q]) : id;
  }
  Box Lp = bl[0], Rp = br[3];
#pragma unroll
  for (int q = 1; q < 4; ++q) {
    Lp = box_union(Lp, bl[q]);      // ascending levels
    Rp = box_union(Rp, br[3 - q]);  // descending levels
  }
  A = group_union<true>(A, sub, mask);
  Lp = group_union<true>(Lp, sub, mask);
  Rp = group_union<false>(Rp, sub, mask);
  B = group_union<true>(B, sub, mask);
  if (sub == 0) box_store(aabb_all + 6 * (2ull * t0 - m + n), box_union(box_union(A, Lp), box_union(Rp, B)));
}

// Fold of the leaf boxes at global positions [l, r) through the segment tree
// (leaf0 + 6 p: the box of the leaf at position p), one thread, its loads
// issued four levels at a time.
__device__ __forceinline__ Box seg_fold(const float* leaf0, uint32_t l, uint32_t r, const SegView& v) {
  const float* dummy = leaf0 + 6ull * l;
  Box L = box_identity(), R = box_identity();
  {  // ragged ends: up to 7 leaves on each side
    const uint32_t nl = (8u - (l & 7u)) & 7u, nr = r & 7u;
    Box bl[7], br[7];
#pragma unroll
    for (int q = 0; q < 7; ++q) {
      bl[q] = box_load_l1(static_cast<uint32_t>(q) < nl ? leaf0 + 6ull * (l + q) : dummy);
      br[q] = box_load_l1(static_cast<uint32_t>(q) < nr ? leaf0 + 6ull * (r - 1 - q) : dummy);
    }
#pragma unroll
    for (int q = 0; q < 7; ++q) {
      if (static_cast<uint32_t>(q) < nl) L = box_union(L, bl[q]);
      if (static_cast<uint32_t>(q) < nr) R = box_union(br[q], R);
    }
    l = (l + nl) >> 3;
    r = (r - nr) >> 3;
  }
  uint32_t lvl = 3;
  while (l < r) {
    const float* pl[4];
    const float* pr[4];
    bool tl[4], tr[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      tl[q] = (l < r) && (l & 1u);
      pl[q] = tl[q] ? seg_node(v, lvl, l) : dummy;
      if (tl[q]) ++l;
      tr[q] = (l < r) && (r & 1u);
      if (tr[q]) --r;
      pr[q] = tr[q] ? seg_node(v, lvl, r) : dummy;
      l >>= 1;
      r >>= 1;
      ++lvl;
    }
    Box bl[4], br[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      bl[q] = box_load_l1(pl[q]);
      br[q] = box_load_l1(pr[q]);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (tl[q]) L = box_union(L, bl[q]);
      if (tr[q]) R = box_union(br[q], R);
    }
  }
  return box_union(L, R);
}

// One thread per branch: the query of its leaf range by seg_fold.
template <bool kBatch>
__device__ __forceinline__ void refit_cross_one(uint32_t g, uint32_t total_tri, const Segments& seg,
                                                const uint32_t* __restrict__ other_all, float* aabb_all,
                                                const SegView& v, uint32_t* status) {
  uint32_t m = 0, t0 = 0, T = total_tri;
  if (kBatch) {
    m = mesh_of_leaf(seg, g);
    t0 = __ldg(seg.tri_off + m);
    T = __ldg(seg.tri_off + m + 1) - t0;
  }
  const uint32_t n = g - t0;
  if (g < t0 || n + 1 >= T) {
    raise_status(status, kStatusBadIndex);
    return;
  }
  const uint32_t oth = __ldg(other_all + (static_cast<size_t>(t0) - m) + n);
  const uint32_t lo = n < oth ? n : oth, hi = n < oth ? oth : n;
  if (hi >= T) {
    raise_status(status, kStatusBadIndex);
    return;
  }
  const float* leaf0 = aabb_all + 6 * (2ull * t0 - m + T - 1) - 6ull * t0;  // + 6*p: leaf of global position p
  box_store(aabb_all + 6 * (2ull * t0 - m + n), seg_fold(leaf0, t0 + lo, t0 + hi + 1, v));
}


// The run branches the window kernel set aside, a window per warp: its heap
// slot 0 holds b*, or kUMax when the window had too few of them (header word
// 4 says whether any window has them).  Lane 0 folds the leaves wEnd + 1 ..
// b* once and the warp unions that into the in-window part each run branch
// holds: union(fold(a .. wEnd), fold(wEnd + 1 .. b*)) is fold(a .. b*), the
// leftmost extreme in leaf order.  The branches are found by the window
// kernel's own test on other_end.  Run by the one-thread crossing kernel,
// which then also takes the list; one mesh only.
__device__ __forceinline__ void refit_runs(uint32_t total_tri, const uint32_t* __restrict__ other_end, float* aabb,
                                           const SegView& v, uint32_t* status) {
  const uint32_t windows = (total_tri + kRefitWindow - 1) >> kRefitWindowLog;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < windows; w += nwarps) {
    const uint32_t wA = w * kRefitWindow, wEnd = wA + kRefitWindow - 1;
    uint32_t bstar = kUMax;
    if (lane == 0) bstar = __ldcg(reinterpret_cast<const uint32_t*>(v.wseg + 6 * static_cast<size_t>(w) * kRefitWinHeap));
    bstar = __shfl_sync(0xffffffffu, bstar, 0);
    if (bstar == kUMax) continue;
    if (bstar <= wEnd || bstar >= total_tri) {
      if (lane == 0) raise_status(status, kStatusBadIndex);
      continue;
    }
    Box right = box_identity();
    if (lane == 0) right = seg_fold(aabb + 6ull * (total_tri - 1), wEnd + 1, bstar + 1, v);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      right.lo[d] = __shfl_sync(0xffffffffu, right.lo[d], 0);
      right.hi[d] = __shfl_sync(0xffffffffu, right.hi[d], 0);
    }
    for (uint32_t k = lane; k < kRefitWindow; k += 32) {
      const uint32_t g = wA + k;
      if (g + 1 >= total_tri) break;  // branches are 0 .. total_tri - 2
      const uint32_t oth = __ldg(other_end + g);
      const uint32_t lo = g < oth ? g : oth, hi = g < oth ? oth : g;
      if (lo >= wA && hi == bstar) {
        float* dst = aabb + 6ull * g;
        box_store(dst, box_union(box_load_cg(dst), right));
      }
    }
  }
}

// Branches whose range crosses a window edge, from the list the window kernel
// appended, in one of two kernels chosen on the device by the list's length.
// A short list (at most `groups` branches) gets a group of 8 lanes per branch
// (k_refit_seg_cross_groups, refit_cross_group), which cuts the latency of
// each query; a long one (runs of equal codes across many windows) one
// thread per branch (k_refit_seg_cross_threads, refit_cross_one), which costs
// fewer instructions in all.  When a window set run branches aside (header
// word 4), the one-thread kernel takes the call whatever the list's length
// and runs refit_runs first.  Every list entry read is cleared, also when the
// climb took over.
template <bool kBatch, bool kRuns>
__global__ void __launch_bounds__(256, 4) k_refit_seg_cross_groups(uint32_t total_tri, Segments seg,
                                                                   const uint32_t* __restrict__ other_all,
                                                                   float* aabb_all, const uint32_t* hdr,
                                                                   uint32_t* cross_list, SegView v, uint32_t groups,
                                                                   uint32_t* status) {
  pdl_wait();
  pdl_launch_dependents();
  uint3 h;  // climb flag, list length, runs present (kRuns only)
  if constexpr (kRuns) {
    h = block_read_hdr3(hdr + 1, hdr + 3, hdr + 4);
  } else {
    const uint2 h2 = block_read_hdr(hdr + 1, hdr + 3);
    h = make_uint3(h2.x, h2.y, 0u);
  }
  const bool climb = h.x != 0u;
  uint32_t count = h.y;
  if (count > total_tri) count = total_tri;
  if (count > groups || h.z != 0u) return;  // the one-thread kernel takes it
  const uint32_t sub = threadIdx.x & 7u;
  const uint32_t mask = 0xffu << (threadIdx.x & 24u);  // the group's lanes in the warp
  const uint32_t stride = (gridDim.x * blockDim.x) >> 3;
  for (uint32_t e = (blockIdx.x * blockDim.x + threadIdx.x) >> 3; e < count; e += stride) {
    const uint32_t entry = cross_list[e];
    __syncwarp(mask);
    if (sub == 0) cross_list[e] = 0u;
    if (climb) continue;
    if (entry == 0u || entry > total_tri) {
      if (sub == 0) raise_status(status, kStatusBadIndex);
      continue;
    }
    refit_cross_group<kBatch>(entry - 1, sub, mask, total_tri, seg, other_all, aabb_all, v, status);
  }
}

template <bool kBatch, bool kRuns>
__global__ void __launch_bounds__(256) k_refit_seg_cross_threads(uint32_t total_tri, Segments seg,
                                                                 const uint32_t* __restrict__ other_all,
                                                                 float* aabb_all, const uint32_t* hdr,
                                                                 uint32_t* cross_list, SegView v, uint32_t groups,
                                                                 uint32_t* status) {
  pdl_wait();
  pdl_launch_dependents();
  uint3 h;  // climb flag, list length, runs present (kRuns only)
  if constexpr (kRuns) {
    h = block_read_hdr3(hdr + 1, hdr + 3, hdr + 4);
  } else {
    const uint2 h2 = block_read_hdr(hdr + 1, hdr + 3);
    h = make_uint3(h2.x, h2.y, 0u);
  }
  const bool climb = h.x != 0u;
  uint32_t count = h.y;
  if (count > total_tri) count = total_tri;
  if (count <= groups && h.z == 0u) return;  // the 8-lane kernel took it
  if (kRuns && !climb && h.z != 0u) refit_runs(total_tri, other_all, aabb_all, v, status);
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < count; e += gridDim.x * blockDim.x) {
    const uint32_t entry = cross_list[e];
    cross_list[e] = 0u;
    if (climb) continue;
    if (entry == 0u || entry > total_tri) {
      raise_status(status, kStatusBadIndex);
      continue;
    }
    refit_cross_one<kBatch>(entry - 1, total_tri, seg, other_all, aabb_all, v, status);
  }
}


}  // namespace

// ------------------------------------------------------------- launchers

void launch_centroid_aabb(cudaStream_t s, uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                          const float* vtx2xyz, float* partials, uint32_t* ticket, float* aabb_out,
                          float* transform_out, uint32_t* status, float* cent, size_t stride, float* tribox) {
  const int grid = grid_for(num_tri, kThreads * 8, kAabbBlocks);
  if (tribox)
    k_centroid_aabb<true><<<grid, kThreads, 0, s>>>(num_tri, tri2vtx, num_vtx, vtx2xyz, partials, ticket, aabb_out,
                                                    transform_out, status, cent, stride, tribox);
  else
    k_centroid_aabb<false><<<grid, kThreads, 0, s>>>(num_tri, tri2vtx, num_vtx, vtx2xyz, partials, ticket, aabb_out,
                                                     transform_out, status, cent, stride, nullptr);
}

void launch_morton_tri(cudaStream_t s, uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                       const float* vtx2xyz, const float* transform, uint32_t* codes, uint32_t* hist,
                       uint32_t* status, const float* cent, size_t stride, bool hist10) {
  const int grid = grid_for(num_tri, kThreads * 8, 152 * 16);
  if (hist)
    launch_pdl(k_morton_tri<true>, dim3(grid), dim3(kThreads), 0, s, num_tri, tri2vtx, num_vtx, vtx2xyz, transform,
               codes, hist, status, cent, stride, hist10);
  else
    k_morton_tri<false><<<grid, kThreads, 0, s>>>(num_tri, tri2vtx, num_vtx, vtx2xyz, transform, codes, nullptr,
                                                  status, cent, stride, false);
}

void launch_vtx2morton(cudaStream_t s, uint32_t n, uint32_t num_dim, const float* vtx2co, const float* transform,
                       uint32_t* out) {
  const int grid = grid_for(n, kThreads * 4, 152 * 16);
  k_vtx2morton<<<grid, kThreads, 0, s>>>(n, num_dim, vtx2co, transform, out);
}

void launch_topology(cudaStream_t s, uint32_t n, const uint32_t* idx2morton, const uint32_t* idx2obj,
                     uint32_t* bvhnodes, uint32_t* other_end, uint32_t threads) {
  if (n == 1) {
    k_topology_single<<<1, 1, 0, s>>>(idx2obj, bvhnodes);
    return;
  }
  const uint32_t th = threads == 128 || threads == 512 ? threads : 256u;
  const uint32_t grid = (n - 1 + th - 1) / th;
  if (th == 128) launch_pdl(k_topology<128>, dim3(grid), dim3(128), 0, s, n, idx2morton, idx2obj, bvhnodes, other_end);
  else if (th == 512) launch_pdl(k_topology<512>, dim3(grid), dim3(512), 0, s, n, idx2morton, idx2obj, bvhnodes, other_end);
  else launch_pdl(k_topology<256>, dim3(grid), dim3(256), 0, s, n, idx2morton, idx2obj, bvhnodes, other_end);
}

// The kernels after the first of this sequence are launched with launch_pdl
// and wait (pdl_wait) before touching their predecessor's data, so each is
// resident when its predecessor ends.  The first kernel triggers nothing
// early: measured on GB300, letting the range-query kernels' successors in
// while its last wave runs made the refit slower (2M triangles: 92 -> 115 us).
void launch_refit_windowed(cudaStream_t s, uint32_t total_tri, const Segments& seg, uint32_t num_vtx_single,
                           const uint32_t* bvhnodes, const uint32_t* other_end, const uint32_t* tri2vtx,
                           const float* vtx2xyz0, const float* vtx2xyz1, float* aabb, uint32_t* flags,
                           uint32_t* height_out, uint32_t* status, const float* tribox, bool header_ready,
                           const uint32_t* leaf_tri) {
  if (total_tri == 0) return;
  if (seg.tri_off || vtx2xyz1) tribox = nullptr;  // one mesh, one vertex state only
  const int smem = static_cast<int>(sizeof(WinSmem));
  const uint32_t windows = refit_num_windows(total_tri), supers = refit_num_super(total_tri);
  const uint32_t top_log = refit_top_log(total_tri);
  const uint32_t capacity = refit_queue_capacity(total_tri);
  uint32_t* queue = flags + refit_queue_offset(total_tri);  // also the header: count, climb flag, ticket
  float* segbase = reinterpret_cast<float*>(flags + refit_seg_offset(total_tri));
  SegView v{segbase, segbase + 6 * size_t{kRefitWinHeap} * windows,
            segbase + 6 * (size_t{kRefitWinHeap} * windows + size_t{64} * supers),
            top_log};
  // the attribute is per device; set it once so that later calls (possibly
  // under stream capture) make no further runtime configuration calls
  static bool configured[64] = {false};
  static int sm_count[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !configured[dev]) {
    cudaFuncSetAttribute(k_refit_win<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_refit_win<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_refit_seg_win<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSegWinSmem);
    cudaFuncSetAttribute(k_refit_seg_win<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSegWinSmem);
    cudaFuncSetAttribute(k_refit_seg_win<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSegWinSmem);
    cudaDeviceGetAttribute(&sm_count[dev], cudaDevAttrMultiProcessorCount, dev);
    configured[dev] = true;
  }
  const uint32_t sms = (dev >= 0 && dev < 64 && sm_count[dev] > 0) ? static_cast<uint32_t>(sm_count[dev]) : 152u;
  if (!header_ready) cudaMemsetAsync(queue, 0, kRefitQueueHdr * sizeof(uint32_t), s);
  if (height_out) cudaMemsetAsync(queue + 1, 1, sizeof(uint32_t), s);  // heights come from the climb
  const uint32_t top_grid = (capacity + 127) / 128;
  // persistent grids: the crossing list is short, and the climb usually exits at once
  const uint32_t cross_grid = std::min<uint32_t>((total_tri + 31) / 32, sms * 8);  // 32 branches per block
  // the 8-lane kernel loops over up to 4 rounds of its grid; longer lists
  // (the 4M soup has 3.2M crossing branches, the 2M torus 41k) take a thread each
  const uint32_t cross_groups = cross_grid * 32 * 4;
  const uint32_t cross_grid1 = std::min<uint32_t>((total_tri + 255) / 256, sms * 2);
  const uint32_t climb_grid = std::min<uint32_t>(windows, sms * 6);
  float* wseg = const_cast<float*>(v.wseg);
  float* sseg = const_cast<float*>(v.sseg);
  float* tseg = const_cast<float*>(v.tseg);
  if (seg.tri_off) {
    k_refit_seg_win<true, false><<<windows, kWinThreads, kSegWinSmem, s>>>(total_tri, seg, num_vtx_single, bvhnodes, other_end, tri2vtx,
                                                          vtx2xyz0, vtx2xyz1, aabb, queue, flags, wseg, status,
                                                          nullptr, nullptr);
    launch_pdl(k_refit_seg_super, dim3(supers), dim3(256), 0, s, total_tri, queue, wseg, sseg, tseg, top_log);
    launch_pdl(k_refit_seg_cross_groups<true, false>, dim3(cross_grid), dim3(256), 0, s, total_tri, seg, other_end, aabb,
               queue, flags, v, cross_groups, status);
    launch_pdl(k_refit_seg_cross_threads<true, false>, dim3(cross_grid1), dim3(256), 0, s, total_tri, seg, other_end, aabb,
               queue, flags, v, cross_groups, status);
    launch_pdl(k_refit_win<true>, dim3(climb_grid), dim3(kWinThreads), smem, s, total_tri, seg, num_vtx_single,
               bvhnodes, other_end, tri2vtx, vtx2xyz0, vtx2xyz1, aabb, flags, queue, capacity, height_out, status);
    launch_pdl(k_refit_top<true>, dim3(top_grid), dim3(128), 0, s, total_tri, seg, bvhnodes, aabb, flags, queue,
               capacity, height_out, status);
  } else {
    // run branches are set aside for soups (the meshes with stored triangle
    // boxes), whose clusters make runs of equal codes across windows
    if (tribox) {
      k_refit_seg_win<false, true><<<windows, kWinThreads, kSegWinSmem, s>>>(total_tri, seg, num_vtx_single, bvhnodes,
                                                                      other_end, tri2vtx, vtx2xyz0, vtx2xyz1, aabb,
                                                                      queue, flags, wseg, status, tribox, leaf_tri);
      launch_pdl(k_refit_seg_super, dim3(supers), dim3(256), 0, s, total_tri, queue, wseg, sseg, tseg, top_log);
      launch_pdl(k_refit_seg_cross_groups<false, true>, dim3(cross_grid), dim3(256), 0, s, total_tri, seg, other_end,
                 aabb, queue, flags, v, cross_groups, status);
      launch_pdl(k_refit_seg_cross_threads<false, true>, dim3(cross_grid1), dim3(256), 0, s, total_tri, seg, other_end,
                 aabb, queue, flags, v, cross_groups, status);
    } else {
      k_refit_seg_win<false, false><<<windows, kWinThreads, kSegWinSmem, s>>>(total_tri, seg, num_vtx_single, bvhnodes,
                                                                       other_end, tri2vtx, vtx2xyz0, vtx2xyz1, aabb,
                                                                       queue, flags, wseg, status, nullptr, leaf_tri);
      launch_pdl(k_refit_seg_super, dim3(supers), dim3(256), 0, s, total_tri, queue, wseg, sseg, tseg, top_log);
      launch_pdl(k_refit_seg_cross_groups<false, false>, dim3(cross_grid), dim3(256), 0, s, total_tri, seg, other_end,
                 aabb, queue, flags, v, cross_groups, status);
      launch_pdl(k_refit_seg_cross_threads<false, false>, dim3(cross_grid1), dim3(256), 0, s, total_tri, seg,
                 other_end, aabb, queue, flags, v, cross_groups, status);
    }
    launch_pdl(k_refit_win<false>, dim3(climb_grid), dim3(kWinThreads), smem, s, total_tri, seg, num_vtx_single,
               bvhnodes, other_end, tri2vtx, vtx2xyz0, vtx2xyz1, aabb, flags, queue, capacity, height_out, status);
    launch_pdl(k_refit_top<false>, dim3(top_grid), dim3(128), 0, s, total_tri, seg, bvhnodes, aabb, flags, queue,
               capacity, height_out, status);
  }
}

void launch_refit(cudaStream_t s, uint32_t num_tri, const uint32_t* bvhnodes, const uint32_t* tri2vtx,
                  uint32_t num_vtx, const float* vtx2xyz0, const float* vtx2xyz1, float* aabb, uint32_t* flags,
                  uint32_t* height_out, uint32_t* status, const uint32_t* gate) {
  uint32_t grid = (num_tri + kThreads - 1) / kThreads;
  // gated, it usually exits at once: a grid of a few blocks per SM costs
  // less to launch than one thread per leaf
  if (gate != nullptr && grid > 152u * 8u) grid = 152u * 8u;
  k_refit<<<grid, kThreads, 0, s>>>(num_tri, bvhnodes, tri2vtx, num_vtx, vtx2xyz0, vtx2xyz1, aabb, flags, height_out,
                                    status, gate);
}

// ------------------------------------------- refit of a tree given as bvhnodes
// The drop-in refit gets a tree and nothing else.  The range queries need
// each branch's leaf range.  k_refit_ends finds, for branch i with children
// c0, c1 and with bounded walks (at most kSpineWalk records each, all four
// walked together), lo(i) at the bottom of i's left spine (left child, left
// child, ...), hi(i) at the bottom of its right spine, hi(c0) at the bottom of
// c0's right spine and lo(c1) at the bottom of c1's left spine (a leaf child
// is its own position), and checks that
//   - hi(c0) + 1 == lo(c1): the children's leaf runs meet;
//   - i is lo(i) or hi(i): a branch index is one end of its range (the
//     property the window refit uses), and other_end[i] is the other end;
//   - both children name i as their parent, and the root spans 0 .. T-1.
// By induction from the leaves every subtree's leaves then form the run
// [lo, hi] in order (lo(c0) = lo(i) and hi(c1) = hi(i) hold by construction),
// so the range queries give the climb's boxes.  Anything else (a tree not in
// Karras leaf order, malformed records, or a spine longer than the walk) sets
// kRefitPlainClimb in the refit header: the range-query kernels exit at once
// and the parent-pointer climb k_refit does the call.
constexpr uint32_t kSpineWalk = 64;

__global__ void __launch_bounds__(kThreads) k_refit_ends(uint32_t num_tri, const uint32_t* __restrict__ bn,
                                                         uint32_t* __restrict__ other_end, uint32_t* hdr) {
  const uint32_t i = blockIdx.x * kThreads + threadIdx.x;
  const uint32_t nb = num_tri - 1, num_node = 2 * num_tri - 1;
  if (i >= nb) return;
  const uint32_t p = __ldg(bn + 3ull * i), c0 = __ldg(bn + 3ull * i + 1), c1 = __ldg(bn + 3ull * i + 2);
  bool bad = c0 >= num_node || c1 >= num_node;
  uint32_t lo = 0, hi = 0;
  if (!bad) {
    // four walks at once: x[0] left spine of i (from c0), x[1] right spine of
    // i (from c1), x[2] right spine of c0, x[3] left spine of c1
    uint32_t x[4] = {c0, c1, c0, c1};
    const uint32_t side[4] = {1u, 2u, 2u, 1u};
    const bool parents_ok = __ldg(bn + 3ull * c0) == i && __ldg(bn + 3ull * c1) == i;
    for (uint32_t step = 0; step < kSpineWalk; ++step) {
      bool more = false;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (x[k] < nb) {
          x[k] = __ldg(bn + 3ull * x[k] + side[k]);
          more = true;
        }
      }
      if (!more) break;
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (x[k] >= num_node) x[k] = kUMax - 1;  // a bad index: stops the walk, fails below
    }
    bool leaves = true;
#pragma unroll
    for (int k = 0; k < 4; ++k) leaves = leaves && x[k] >= nb && x[k] < num_node;
    if (!leaves || !parents_ok) {
      bad = true;
    } else {
      lo = x[0] - nb;
      hi = x[1] - nb;
      bad = (x[2] - nb) + 1 != x[3] - nb || (i != lo && i != hi) || lo >= hi;
      if (i == 0) bad = bad || p != kUMax || lo != 0 || hi != nb;
    }
  }
  other_end[i] = bad ? i : (i == lo ? hi : lo);
  if (bad) atomicOr(hdr + 1, kRefitPlainClimb);
}

void launch_refit_any_tree(cudaStream_t s, uint32_t num_tri, const uint32_t* bvhnodes, const uint32_t* tri2vtx,
                           uint32_t num_vtx, const float* vtx2xyz0, const float* vtx2xyz1, float* aabb,
                           uint32_t* other_end, uint32_t* flags, uint32_t* status) {
  if (num_tri == 0) return;
  if (num_tri == 1) {  // a single leaf: nothing to climb or query
    launch_refit(s, num_tri, bvhnodes, tri2vtx, num_vtx, vtx2xyz0, vtx2xyz1, aabb, flags, nullptr, status);
    return;
  }
  uint32_t* hdr = flags + refit_queue_offset(num_tri);
  cudaMemsetAsync(hdr, 0, kRefitQueueHdr * sizeof(uint32_t), s);
  const uint32_t grid = (num_tri - 1 + kThreads - 1) / kThreads;
  k_refit_ends<<<grid, kThreads, 0, s>>>(num_tri, bvhnodes, other_end, hdr);
  launch_refit_windowed(s, num_tri, Segments{}, num_vtx, bvhnodes, other_end, tri2vtx, vtx2xyz0, vtx2xyz1, aabb,
                        flags, nullptr, status, nullptr, /*header_ready=*/true);
  launch_refit(s, num_tri, bvhnodes, tri2vtx, num_vtx, vtx2xyz0, vtx2xyz1, aabb, flags, nullptr, status, hdr + 1);
}

}  // namespace dm
