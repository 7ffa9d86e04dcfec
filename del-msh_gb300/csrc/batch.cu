// batch.cu — LBVH build and ray cast of many independent triangle meshes of
// uneven sizes in one launch sequence (no per-mesh launches, no host sync).
//
// Meshes are stored back to back (see dm::Segments): mesh m owns triangles
// tri_off[m]..tri_off[m+1]-1 with vertex indices local to its own vertex
// block vtx_off[m]..; its tree occupies nodes 2*tri_off[m]-m .. with node and
// triangle indices local to the mesh.  Each mesh's slice of bvhnodes /
// bvhnode2aabb is therefore exactly what the single-mesh build returns for it
// alone, bit for bit.
//
// Launch sequence of a batch build:
//   k_batch_fit      one block per mesh: centroid AABB and fit transform
//   k_batch_morton   per triangle: key = (mesh << 30) | 30-bit Morton code,
//                    with the digit histograms of the key
//   k_onesweep x P   stable LSD radix sort of the 64-bit keys (P = 8-bit digits
//                    covering 30 + log2(num_mesh) bits); values = global
//                    triangle index, so ties keep ascending triangle order
//   k_batch_topology per branch of every mesh (binary search of its mesh)
//   refit            launch_refit_windowed over the global leaf order (segment-
//                    tree range queries; the tree-order climb for NaN / heights)
// and of a batch cast: the persistent traversal of dm_traverse.cuh over the
// 32-pixel tiles (8x4 by default) of every mesh's image, each lane loading its own mesh.
#include <cfloat>

#include <cooperative_groups.h>

#include "dm_lbvh.cuh"
#include "dm_traverse.cuh"

namespace dm {
namespace {

namespace cg = cooperative_groups;

constexpr int kThreads = 256;

__device__ __forceinline__ uint32_t upper_mesh(const uint32_t* __restrict__ off, uint32_t num_mesh, uint32_t i) {
  // largest m in [0, num_mesh) with off[m] <= i (off non-decreasing)
  uint32_t lo = 0, hi = num_mesh;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) / 2;
    if (__ldg(off + mid) <= i) lo = mid;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ float3 centroid_at(const uint32_t* __restrict__ t2v, const float* __restrict__ x,
                                              uint32_t num_vtx, uint32_t it, uint32_t* status) {
  const uint32_t* t = t2v + static_cast<size_t>(it) * 3;
  uint32_t v[3] = {__ldg(t), __ldg(t + 1), __ldg(t + 2)};
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (v[k] >= num_vtx) {
      raise_status(status, kStatusBadIndex);
      v[k] = 0;
    }
  const float3 p0 = load_vtx(x, v[0]), p1 = load_vtx(x, v[1]), p2 = load_vtx(x, v[2]);
  return make_float3(centroid1(p0.x, p1.x, p2.x), centroid1(p0.y, p1.y, p2.y), centroid1(p0.z, p1.z, p2.z));
}

// The fit transform of Mat44/torch.py:120-140 (uniform scale by the largest
// extent, centre to 0.5) from the centroid box lo / hi, after the
// first-centroid NaN rule of vtx2xyz.rs:19-37 (c0: the first centroid).
__device__ __forceinline__ void fit_transform(float* lo, float* hi, float3 c0, float* mo) {
  const float c0a[3] = {c0.x, c0.y, c0.z};
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if (c0a[d] != c0a[d]) lo[d] = hi[d] = c0a[d];
  float ext = __fsub_rn(hi[0], lo[0]);
  const float ey = __fsub_rn(hi[1], lo[1]), ez = __fsub_rn(hi[2], lo[2]);
  if (ey > ext) ext = ey;
  if (ez > ext) ext = ez;
  const float s = __fdiv_rn(1.0f, ext);
#pragma unroll
  for (int k = 0; k < 16; ++k) mo[k] = 0.0f;
  mo[0] = s;
  mo[5] = s;
  mo[10] = s;
  mo[15] = 1.0f;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float c = __fmul_rn(__fadd_rn(lo[d], hi[d]), 0.5f);
    mo[12 + d] = __fadd_rn(__fmul_rn(-c, s), 0.5f);
  }
}

// Per mesh: the centroid AABB of vtx2xyz.rs:19-37 (first-centroid NaN rule
// and max of c + 0, as k_centroid_aabb) and the fit transform of
// Mat44/torch.py:120-140.
__global__ void __launch_bounds__(kThreads) k_batch_fit(Segments seg, const uint32_t* __restrict__ tri2vtx,
                                                       const float* __restrict__ vtx2xyz, float* transforms,
                                                       uint32_t* status) {
  const uint32_t m = blockIdx.x;
  const uint32_t t0 = __ldg(seg.tri_off + m), T = __ldg(seg.tri_off + m + 1) - t0;
  const uint32_t v0 = __ldg(seg.vtx_off + m), V = __ldg(seg.vtx_off + m + 1) - v0;
  if (T == 0 || T > 0x7FFFFFFFu || V == 0) {  // empty or inverted mesh: invalid input, touch nothing
    if (threadIdx.x == 0) raise_status(status, kStatusBadIndex);
    return;
  }
  const uint32_t* t2v = tri2vtx + 3ull * t0;
  const float* x = vtx2xyz + 3ull * v0;
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (uint32_t i = threadIdx.x; i < T; i += kThreads) {
    const float3 c = centroid_at(t2v, x, V, i, status);
    const float cc[3] = {c.x, c.y, c.z};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (cc[d] < lo[d]) lo[d] = cc[d];
      const float h = __fadd_rn(cc[d], 0.0f);
      if (h > hi[d]) hi[d] = h;
    }
  }
  __shared__ float sh[6][kThreads / 32];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const float a = __shfl_down_sync(0xffffffffu, lo[d], off);
      const float b = __shfl_down_sync(0xffffffffu, hi[d], off);
      if (a < lo[d]) lo[d] = a;
      if (b > hi[d]) hi[d] = b;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
    for (int d = 0; d < 3; ++d) {
      sh[d][warp] = lo[d];
      sh[d + 3][warp] = hi[d];
    }
  __syncthreads();
  if (threadIdx.x != 0) return;
  for (int w = 1; w < kThreads / 32; ++w)
    for (int d = 0; d < 3; ++d) {
      if (sh[d][w] < lo[d]) lo[d] = sh[d][w];
      if (sh[d + 3][w] > hi[d]) hi[d] = sh[d + 3][w];
    }
  fit_transform(lo, hi, centroid_at(t2v, x, V, 0, status), transforms + 16ull * m);
}

// key = (mesh << 30) | morton_code3 of the centroid under the mesh's transform,
// plus the 8-bit digit histograms of the keys for num_pass passes.
__global__ void __launch_bounds__(kThreads) k_batch_morton(uint32_t total_tri, Segments seg,
                                                          const uint32_t* __restrict__ tri2vtx,
                                                          const float* __restrict__ vtx2xyz,
                                                          const float* __restrict__ transforms, uint64_t* keys,
                                                          uint32_t* hist, int num_pass, uint32_t* status) {
  __shared__ uint32_t sh[8 * kRadix];
  for (int i = threadIdx.x; i < num_pass * kRadix; i += kThreads) sh[i] = 0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < total_tri; i += gridDim.x * kThreads) {
    const uint32_t m = upper_mesh(seg.tri_off, seg.num_mesh, i);
    const uint32_t t0 = __ldg(seg.tri_off + m), T = __ldg(seg.tri_off + m + 1) - t0;
    const uint32_t v0 = __ldg(seg.vtx_off + m), V = __ldg(seg.vtx_off + m + 1) - v0;
    if (i < t0 || i - t0 >= T || V == 0) {
      raise_status(status, kStatusBadIndex);
      keys[i] = 0;
      continue;
    }
    const float3 c = centroid_at(tri2vtx + 3ull * t0, vtx2xyz + 3ull * v0, V, i - t0, status);
    const float* mt = transforms + 16ull * m;
    float mm[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) mm[k] = __ldg(mt + k);
    const float3 q = transform_homogeneous(mm, c.x, c.y, c.z);
    const uint64_t key = (static_cast<uint64_t>(m) << 30) | morton_code3(q.x, q.y, q.z);
    keys[i] = key;
    for (int p = 0; p < num_pass; ++p) atomicAdd(&sh[p * kRadix + ((key >> (8 * p)) & 0xFFu)], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < num_pass * kRadix; i += kThreads)
    if (sh[i]) atomicAdd(hist + i, sh[i]);
}

struct CodesKey {
  const uint64_t* p;
  __device__ __forceinline__ uint32_t operator()(uint32_t i) const {
    return static_cast<uint32_t>(__ldg(reinterpret_cast<const unsigned long long*>(p) + i) & 0x3FFFFFFFull);
  }
};
struct ObjsLocal {
  const uint32_t* p;
  uint32_t base;
  __device__ __forceinline__ uint32_t operator()(uint32_t i) const { return __ldg(p + i) - base; }
};

// Branch g of the batch (branches of mesh m are tri_off[m]-m ..).  Meshes of
// one triangle have no branch and get the single leaf [MAX, 0, MAX].
__global__ void __launch_bounds__(kThreads) k_batch_topology(uint32_t total_branch, Segments seg,
                                                            const uint64_t* __restrict__ keys,
                                                            const uint32_t* __restrict__ vals, uint32_t* bvhnodes_all,
                                                            uint32_t* other_all) {
  const uint32_t g = blockIdx.x * kThreads + threadIdx.x;
  if (g < seg.num_mesh) {
    const uint32_t t0 = __ldg(seg.tri_off + g), T = __ldg(seg.tri_off + g + 1) - t0;
    if (T == 1) {
      uint32_t* b = bvhnodes_all + 3 * (2ull * t0 - g);
      b[0] = kUMax;
      b[1] = 0u;
      b[2] = kUMax;
    }
  }
  if (g >= total_branch) return;
  // mesh m: largest with tri_off[m] - m <= g and a branch there (T_m > 1)
  uint32_t lo = 0, hi = seg.num_mesh;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) / 2;
    if (__ldg(seg.tri_off + mid) - mid <= g) lo = mid;
    else hi = mid;
  }
  const uint32_t m = lo;
  const uint32_t t0 = __ldg(seg.tri_off + m), T = __ldg(seg.tri_off + m + 1) - t0;
  const uint32_t ib = g - (t0 - m);
  if (T < 2 || T > 0x7FFFFFFFu || ib >= T - 1) return;  // only reachable with invalid offsets
  topology_node(T, CodesKey{keys + t0}, ObjsLocal{vals + t0, t0}, bvhnodes_all + 3 * (2ull * t0 - m), ib,
                other_all + (t0 - m));
}

// ------------------------------------------------- fused per-mesh build
// Batches whose meshes have at most kSegMaxTri triangles are built by
// k_batch_seg_build instead of the global 64-bit sort: each mesh is sorted in
// on-chip memory and never leaves it between the fit and the topology.
//
// A block holds kSegCap keys (a 30-bit code and a 16-bit triangle index) in
// two shared buffers; a mesh of up to kSegCap triangles is built by one block,
// a larger one by a cluster of kC blocks whose buffers together hold the mesh
// (an equal share of positions each, SegSplit), exchanging keys through
// distributed shared memory.  Per mesh:
//   fit      centroid AABB (the same operations as k_batch_fit), combined
//            over the cluster, and the fit transform; the centroids wait in
//            the (still empty) sort buffers
//   codes    Morton code of every centroid, stored at the triangle's position
//   4 passes stable LSD radix sort on 8-bit digits: warp ballots rank each
//            key within its warp (as k_onesweep), per-warp and per-block
//            digit counts give every key its output position in the mesh, and
//            the key is written to the block owning that position
//   topology Karras branches (topology_node) over the sorted codes, read from
//            the owning block's shared memory
// The sort is stable and starts from ascending triangle order, so the order,
// the codes and therefore the tree are those of the global sort.
constexpr int kSegThreads = 1024;
constexpr int kSegWarps = kSegThreads / 32;
constexpr uint32_t kSegCap = 16384;                         // keys per block
constexpr uint32_t kSegWarpKeys = kSegCap / kSegWarps;      // at most 512 keys per warp
constexpr int kSegSlots = static_cast<int>(kSegWarpKeys / 32);  // at most 16 keys per lane
constexpr int kSegUnroll = 2;                                 // triangles gathered together per thread
static_assert(kSegMaxTri == 4 * kSegCap, "clusters of up to four blocks");
static_assert(kSegMaxTri <= 65536, "triangle indices are held in 16 bits");

struct SegSmem {
  uint32_t code[2][kSegCap];
  uint16_t idx[2][kSegCap];
  uint16_t whist[kSegWarps][kRadix];  // per-warp digit counts, then per-warp offsets in the block
  uint32_t cnt[kRadix];               // this block's digit counts (read by the cluster)
  uint32_t off[kRadix];               // output start of this block's keys of each digit
  uint32_t scan[kSegWarps];
  float wbox[kSegWarps][6];
  float box[6];                       // this block's centroid box (read by the cluster)
  float fit[6];
  uint32_t work;
};

// The kC blocks building one mesh: a cluster, or (kC == 1) a block alone.
template <int kC>
struct SegGroup {
  __device__ static uint32_t rank() {
    if constexpr (kC == 1) return 0;
    else return cg::this_cluster().block_rank();
  }
  __device__ static void sync() {
    if constexpr (kC == 1) __syncthreads();
    else cg::this_cluster().sync();
  }
  template <typename T>
  __device__ static T* at(T* p, uint32_t r) {
    if constexpr (kC == 1) return p;
    else return cg::this_cluster().map_shared_rank(p, r);
  }
};

__device__ __forceinline__ uint32_t seg_block_scan(uint32_t v, uint32_t* s_warp) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < kSegWarps ? s_warp[lane] : 0u;
#pragma unroll
    for (int off = 1; off < kSegWarps; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, off);
      if (lane >= off) w += y;
    }
    if (lane < kSegWarps) s_warp[lane] = w;
  }
  __syncthreads();
  const uint32_t r = (warp > 0 ? s_warp[warp - 1] : 0u) + x - v;
  __syncthreads();
  return r;
}

// How the kC blocks of a group share a mesh of T triangles: block r holds
// positions r*per .. r*per+per-1, per = ceil(T / kC) (at most kSegCap).  The
// owner of a position is a multiply-high by magic = ceil(2^32 / per), exact
// for positions below 2^16 when per >= 2^12 (position times the rounding
// excess of magic*per stays below 2^32); groups of kC > 1 blocks only build
// meshes of more than kSegCap triangles, so per > kSegCap / 4 = 2^12.
template <int kC>
struct SegSplit {
  uint32_t per, magic;
  __device__ __forceinline__ explicit SegSplit(uint32_t T)
      : per((T + kC - 1) / kC), magic(kC == 1 ? 0u : 0xFFFFFFFFu / ((T + kC - 1) / kC) + 1u) {}
  __device__ __forceinline__ uint32_t owner(uint32_t i) const { return kC == 1 ? 0u : __umulhi(i, magic); }
};

// Centroid z between the fit and the codes, in the index buffers (x and y are
// in the two code buffers): 2 * kSegCap 16-bit slots hold kSegCap floats.
__device__ __forceinline__ float* seg_cz(SegSmem& S) { return reinterpret_cast<float*>(&S.idx[0][0]); }
static_assert(sizeof(SegSmem::idx) == kSegCap * sizeof(float), "centroid z fits the index buffers");

// Sorted codes / triangle indices of the mesh, read from the owning block
// (base: the buffer in this block; it has the same offset in every block).
template <int kC, typename T>
struct SegView {
  SegSplit<kC> sp;
  T* base;
  __device__ __forceinline__ uint32_t operator()(uint32_t i) const {
    const uint32_t r = sp.owner(i);
    return SegGroup<kC>::at(base, r)[i - r * sp.per];
  }
};

// One stable pass over the digit at `shift`: keys of buffer src (this block's
// n_c positions) go to buffer src ^ 1 of the block owning their output
// position.  With kIota the triangle indices are the positions themselves
// (first pass: the index buffer then still holds centroids).
template <int kC, bool kIota>
__device__ __forceinline__ void seg_pass(SegSmem& S, int src, uint32_t shift, uint32_t n_c, uint32_t rank,
                                         const SegSplit<kC>& sp) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint32_t* wh = reinterpret_cast<uint32_t*>(&S.whist[0][0]);
  for (int i = tid; i < kSegWarps * kRadix / 2; i += kSegThreads) wh[i] = 0u;
  __syncthreads();
  // the block's positions split evenly over its warps, in whole 32-key slots
  const uint32_t chunk = (n_c + kSegThreads - 1) / kSegThreads * 32u;  // <= kSegWarpKeys
  const uint32_t wpos = static_cast<uint32_t>(warp) * chunk;
  const uint32_t n_w = n_c > wpos ? min(n_c - wpos, chunk) : 0u;
  const uint32_t lt_mask = (1u << lane) - 1u;
  uint16_t* my = S.whist[warp];
  // rank in (slot, lane) order, i.e. position order; two 16-bit ranks per word
  uint32_t rk[kSegSlots / 2];
#pragma unroll
  for (int k = 0; k < kSegSlots; ++k) {
    uint32_t r = 0;
    if (static_cast<uint32_t>(k) * 32u < n_w) {
      const uint32_t p = static_cast<uint32_t>(k) * 32u + lane;
      const bool valid = p < n_w;
      const uint32_t d = valid ? (S.code[src][wpos + p] >> shift) & 0xFFu : 0u;
      const uint32_t peers = warp_peers(d, valid);
      const uint32_t before = valid ? my[d] : 0u;
      __syncwarp();
      if (valid && lane == __ffs(peers) - 1) my[d] = static_cast<uint16_t>(before + __popc(peers));
      __syncwarp();
      r = before + __popc(peers & lt_mask);
    }
    if (k & 1) rk[k / 2] |= r << 16;
    else rk[k / 2] = r;
  }
  __syncthreads();
  if (tid < kRadix) {
    uint32_t cnt = 0;
#pragma unroll
    for (int w = 0; w < kSegWarps; ++w) {
      const uint32_t v = S.whist[w][tid];
      S.whist[w][tid] = static_cast<uint16_t>(cnt);
      cnt += v;
    }
    S.cnt[tid] = cnt;
  }
  SegGroup<kC>::sync();  // every block's counts are visible
  uint32_t tot = 0, pre = 0;
  if (tid < kRadix) {
#pragma unroll
    for (int r = 0; r < kC; ++r) {
      const uint32_t v = SegGroup<kC>::at(S.cnt, r)[tid];
      tot += v;
      if (static_cast<uint32_t>(r) < rank) pre += v;
    }
  }
  const uint32_t base = seg_block_scan(tid < kRadix ? tot : 0u, S.scan);  // has __syncthreads
  if (tid < kRadix) S.off[tid] = base + pre;
  __syncthreads();
  const int dst = src ^ 1;
#pragma unroll
  for (int k = 0; k < kSegSlots; ++k) {
    const uint32_t p = static_cast<uint32_t>(k) * 32u + lane;
    if (p < n_w) {
      const uint32_t key = S.code[src][wpos + p];
      const uint16_t id = kIota ? static_cast<uint16_t>(rank * sp.per + wpos + p) : S.idx[src][wpos + p];
      const uint32_t d = (key >> shift) & 0xFFu;
      const uint32_t r = (k & 1) ? (rk[k / 2] >> 16) : (rk[k / 2] & 0xFFFFu);
      const uint32_t out = S.off[d] + S.whist[warp][d] + r;
      const uint32_t owner = sp.owner(out), q = out - owner * sp.per;
      if (owner < static_cast<uint32_t>(kC)) {  // always: the counts add up to the mesh
        SegGroup<kC>::at(&S.code[dst][0], owner)[q] = key;
        SegGroup<kC>::at(&S.idx[dst][0], owner)[q] = id;
      }
    }
  }
  SegGroup<kC>::sync();  // every key has arrived; the counts may be overwritten
}

struct SegArgs {
  Segments seg;
  const uint32_t* tri2vtx;
  const float* vtx2xyz;
  uint32_t* bvhnodes;        // all meshes' nodes
  uint32_t* other;           // all meshes' other_end (mesh m at tri_off[m] - m)
  const uint32_t* lists;     // multi-block meshes from the front, one-block meshes from the back
  const uint32_t* counts;    // [0] multi-block, [1] one-block meshes
  uint32_t* next;            // [0], [1]: work cursors
  uint32_t* status;
};
constexpr uint32_t kSegChain = 1u << 31;  // list flag: more triangles than the build was sized for

// A mesh given more triangles than max_tri_per_mesh (status already raised)
// gets a chain of branches (branch i: leaf i and branch i + 1), a valid tree
// for the refit, so that nothing downstream reads unwritten nodes.
__device__ void seg_chain(const SegArgs& a, uint32_t m) {
  const uint32_t t0 = __ldg(a.seg.tri_off + m), T = __ldg(a.seg.tri_off + m + 1) - t0;
  uint32_t* bvh = a.bvhnodes + 3 * (2ull * t0 - m);
  uint32_t* other = a.other + (t0 - m);
  const uint32_t nb = T - 1;
  for (uint32_t i = threadIdx.x; i < T; i += kSegThreads) {
    uint32_t* leaf = bvh + 3ull * (nb + i);
    leaf[0] = i < nb ? i : nb - 1;
    leaf[1] = i;
    leaf[2] = kUMax;
    if (i < nb) {
      uint32_t* b = bvh + 3ull * i;
      b[0] = i == 0 ? kUMax : i - 1;
      b[1] = nb + i;
      b[2] = i + 1 < nb ? i + 1 : nb + i + 1;
      other[i] = nb;
    }
  }
}

// Builds mesh m with the kC blocks of the group (this one is `rank`).
template <int kC>
__device__ void seg_mesh(SegSmem& S, const SegArgs& a, uint32_t m, uint32_t rank) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t t0 = __ldg(a.seg.tri_off + m), T = __ldg(a.seg.tri_off + m + 1) - t0;
  const uint32_t v0 = __ldg(a.seg.vtx_off + m), V = __ldg(a.seg.vtx_off + m + 1) - v0;
  const uint32_t* t2v = a.tri2vtx + 3ull * t0;
  const float* x = a.vtx2xyz + 3ull * v0;
  const SegSplit<kC> sp(T);
  const uint32_t p0 = rank * sp.per;
  const uint32_t n_c = T > p0 ? min(T - p0, sp.per) : 0u;

  // fit: per-thread, per-warp, per-block, then per-cluster centroid box
  // (kSegUnroll triangles per thread in flight: one block per SM holds few warps)
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (uint32_t i0 = tid; i0 < n_c; i0 += kSegUnroll * kSegThreads) {
    float3 c[kSegUnroll];
#pragma unroll
    for (int u = 0; u < kSegUnroll; ++u) {
      const uint32_t i = i0 + u * kSegThreads;
      if (i < n_c) c[u] = centroid_at(t2v, x, V, p0 + i, a.status);
    }
#pragma unroll
    for (int u = 0; u < kSegUnroll; ++u) {
      const uint32_t i = i0 + u * kSegThreads;
      if (i >= n_c) break;
      S.code[0][i] = __float_as_uint(c[u].x);  // the centroids stay on chip for the codes
      S.code[1][i] = __float_as_uint(c[u].y);
      seg_cz(S)[i] = c[u].z;
      const float cc[3] = {c[u].x, c[u].y, c[u].z};
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        if (cc[d] < lo[d]) lo[d] = cc[d];
        const float h = __fadd_rn(cc[d], 0.0f);
        if (h > hi[d]) hi[d] = h;
      }
    }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const float u = __shfl_down_sync(0xffffffffu, lo[d], off);
      const float v = __shfl_down_sync(0xffffffffu, hi[d], off);
      if (u < lo[d]) lo[d] = u;
      if (v > hi[d]) hi[d] = v;
    }
  }
  if (lane == 0)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      S.wbox[warp][d] = lo[d];
      S.wbox[warp][d + 3] = hi[d];
    }
  __syncthreads();
  if (tid < 6) {
    float v = S.wbox[0][tid];
    for (int w = 1; w < kSegWarps; ++w) {
      const float u = S.wbox[w][tid];
      if (tid < 3 ? u < v : u > v) v = u;
    }
    S.box[tid] = v;
  }
  SegGroup<kC>::sync();
  if (tid < 6) {
    float v = S.box[tid];
    for (int r = 0; r < kC; ++r) {
      if (static_cast<uint32_t>(r) == rank) continue;
      const float u = SegGroup<kC>::at(S.box, r)[tid];
      if (tid < 3 ? u < v : u > v) v = u;
    }
    S.fit[tid] = v;
  }
  __syncthreads();
  float mm[16];
  {
    float flo[3] = {S.fit[0], S.fit[1], S.fit[2]}, fhi[3] = {S.fit[3], S.fit[4], S.fit[5]};
    fit_transform(flo, fhi, centroid_at(t2v, x, V, 0, a.status), mm);
  }

  // codes at their triangle's position, over the centroid's x (each thread
  // reads and writes only its own positions; the first pass takes the
  // triangle index from the position)
  for (uint32_t i = tid; i < n_c; i += kSegThreads) {
    const float3 q = transform_homogeneous(mm, __uint_as_float(S.code[0][i]), __uint_as_float(S.code[1][i]),
                                           seg_cz(S)[i]);
    S.code[0][i] = morton_code3(q.x, q.y, q.z);
  }
  // (seg_pass starts with a __syncthreads; a cluster has synchronised above)
  seg_pass<kC, true>(S, 0, 0, n_c, rank, sp);
  seg_pass<kC, false>(S, 1, 8, n_c, rank, sp);
  seg_pass<kC, false>(S, 0, 16, n_c, rank, sp);
  seg_pass<kC, false>(S, 1, 24, n_c, rank, sp);

  // topology over the sorted buffer 0 of the group
  uint32_t* bvh = a.bvhnodes + 3 * (2ull * t0 - m);
  if (T == 1) {
    if (rank == 0 && tid == 0) {
      bvh[0] = kUMax;
      bvh[1] = 0u;
      bvh[2] = kUMax;
    }
  } else {
    const SegView<kC, uint32_t> codes{sp, &S.code[0][0]};
    const SegView<kC, uint16_t> objs{sp, &S.idx[0][0]};
    const uint32_t end = min(p0 + sp.per, T - 1);
    for (uint32_t ib = p0 + tid; ib < end; ib += kSegThreads)
      topology_node(T, codes, objs, bvh, ib, a.other + (t0 - m));
  }
  SegGroup<kC>::sync();  // the group's reads of this mesh are over
}

// Pulls mesh m's triangles and vertices toward L2 (every 128-byte line once,
// shared by the `parts` blocks of a group), so that the fit's gathers of the
// mesh after the current one find them there.
__device__ __forceinline__ void seg_prefetch(const SegArgs& a, uint32_t m, uint32_t part, uint32_t parts) {
  const uint32_t t0 = __ldg(a.seg.tri_off + m), t1 = __ldg(a.seg.tri_off + m + 1);
  const uint32_t v0 = __ldg(a.seg.vtx_off + m), v1 = __ldg(a.seg.vtx_off + m + 1);
  const char* tb = reinterpret_cast<const char*>(a.tri2vtx + 3ull * t0);
  const char* vb = reinterpret_cast<const char*>(a.vtx2xyz + 3ull * v0);
  const size_t tn = 12ull * (t1 - t0), vn = 12ull * (v1 - v0);
  const size_t first = 128ull * (part * kSegThreads + threadIdx.x), step = 128ull * parts * kSegThreads;
  for (size_t o = first; o < tn; o += step) asm volatile("prefetch.global.L2 [%0];" ::"l"(tb + o));
  for (size_t o = first; o < vn; o += step) asm volatile("prefetch.global.L2 [%0];" ::"l"(vb + o));
}

// The group's next work item from `counter` (taken by block 0, thread 0).
template <int kC>
__device__ __forceinline__ uint32_t seg_take(SegSmem& S, uint32_t* counter, uint32_t rank) {
  if (rank == 0 && threadIdx.x == 0) S.work = atomicAdd(counter, 1u);
  SegGroup<kC>::sync();
  const uint32_t j = *SegGroup<kC>::at(&S.work, 0);
  SegGroup<kC>::sync();  // read by every block before block 0 writes it again
  return j;
}

// Persistent: multi-block meshes first, each by a whole cluster, then
// one-block meshes, each by a single block.  A group takes its next mesh
// before building the current one and prefetches it.  Every loop bound is
// uniform over the group, so all its blocks reach the same barriers.
template <int kC>
__global__ void __launch_bounds__(kSegThreads, 1) k_batch_seg_build(SegArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SegSmem& S = *reinterpret_cast<SegSmem*>(smem_raw);
  if constexpr (kC > 1) {
    const uint32_t rank = SegGroup<kC>::rank();
    const uint32_t num_multi = __ldg(a.counts);
    uint32_t j = seg_take<kC>(S, a.next, rank);
    while (j < num_multi) {
      const uint32_t jn = seg_take<kC>(S, a.next, rank);
      if (jn < num_multi) seg_prefetch(a, __ldg(a.lists + jn), rank, kC);
      seg_mesh<kC>(S, a, __ldg(a.lists + j), rank);
      j = jn;
    }
  }
  const uint32_t num_one = __ldg(a.counts + 1);
  const uint32_t* one = a.lists + (a.seg.num_mesh - 1);  // one-block meshes are listed backwards
  uint32_t j = seg_take<1>(S, a.next + 1, 0);
  while (j < num_one) {
    const uint32_t jn = seg_take<1>(S, a.next + 1, 0);
    if (jn < num_one) {
      const uint32_t en = __ldg(one - jn);
      if (!(en & kSegChain)) seg_prefetch(a, en, 0, 1);
    }
    const uint32_t e = __ldg(one - j);
    if (e & kSegChain) seg_chain(a, e & ~kSegChain);
    else seg_mesh<1>(S, a, e, 0);
    j = jn;
  }
}

// Sorts the meshes into the lists of k_batch_seg_build.  Empty or inverted
// meshes are skipped (status raised, nothing written, as k_batch_fit); a mesh
// above max_tri gets a chain tree (status raised).
__global__ void __launch_bounds__(kThreads) k_batch_seg_classify(Segments seg, uint32_t max_tri, uint32_t* lists,
                                                                uint32_t* counts, uint32_t* status) {
  const uint32_t m = blockIdx.x * kThreads + threadIdx.x;
  if (m >= seg.num_mesh) return;
  const uint32_t T = __ldg(seg.tri_off + m + 1) - __ldg(seg.tri_off + m);
  const uint32_t V = __ldg(seg.vtx_off + m + 1) - __ldg(seg.vtx_off + m);
  if (T == 0 || T > 0x7FFFFFFFu || V == 0) {
    raise_status(status, kStatusBadIndex);
    return;
  }
  if (T > max_tri) {
    raise_status(status, kStatusBadIndex);
    lists[seg.num_mesh - 1 - atomicAdd(counts + 1, 1u)] = m | kSegChain;
  } else if (T > kSegCap) {
    lists[atomicAdd(counts, 1u)] = m;
  } else {
    lists[seg.num_mesh - 1 - atomicAdd(counts + 1, 1u)] = m;
  }
}

// ------------------------------------------------------------ batch cast


struct BatchJob {
  uint32_t num_work;
  Segments seg;
  const uint32_t* tri2vtx;
  const float* vtx2xyz;
  const uint32_t* bvhnodes;
  const float* aabb;
  uint32_t img_w, img_h, tiles_x, tile_w, tile_h, work_per_mesh;
  uint32_t tile_w_log;  // tile_w is a power of two
  Divider by_work_per_mesh, by_tiles_x;
  const float* transforms;  // num_mesh x 16, column-major ndc -> world
  CastOut o;

  __device__ __forceinline__ void prepare(float*) const {}

  __device__ __forceinline__ bool fetch(uint32_t w, const float*, MeshView& mv, Ray& r, uint32_t& out) const {
    const uint32_t m = by_work_per_mesh.div(w), lw = w - m * work_per_mesh;
    const uint32_t tile = lw >> 5, j = lw & 31u;
    const uint32_t ty = by_tiles_x.div(tile);
    const uint32_t px = (tile - ty * tiles_x) * tile_w + (j & (tile_w - 1u));
    const uint32_t py = ty * tile_h + (j >> tile_w_log);
    if (px >= img_w || py >= img_h) return false;
    const uint32_t t0 = __ldg(seg.tri_off + m), T = __ldg(seg.tri_off + m + 1) - t0;
    const uint32_t v0 = __ldg(seg.vtx_off + m), V = __ldg(seg.vtx_off + m + 1) - v0;
    out = m * (img_w * img_h) + py * img_w + px;
    if (T == 0 || T > 0x7FFFFFFFu || V == 0) {  // invalid (empty) mesh: report a miss
      o.hit_tri[out] = kUMax;
      if (o.hit_t) o.hit_t[out] = INFINITY;
      return false;
    }
    const size_t node_off = 2ull * t0 - m;
    mv.num_tri = T;
    mv.num_vtx = V;
    mv.tri2vtx = tri2vtx + 3ull * t0;
    mv.vtx2xyz = vtx2xyz + 3ull * v0;
    mv.bvhnodes = bvhnodes + 3 * node_off;
    mv.aabb = aabb + 6 * node_off;
    float mm[16];
    const float* mt = transforms + 16ull * m;
#pragma unroll
    for (int k = 0; k < 16; ++k) mm[k] = __ldg(mt + k);
    const uint32_t pix = py * img_w + px;
    float3 o3, d3;
    ray_for_pixel_xy(px, py, img_w, img_h, mm, o3, d3);
    r = make_ray(o3, d3);
    out = m * (img_w * img_h) + pix;
    return true;
  }

  __device__ __forceinline__ void write(uint32_t out, const MeshView&, const Ray&, const Hit& h) const {
    o.hit_tri[out] = h.id;
    if (o.hit_t) o.hit_t[out] = h.t;
  }
};

}  // namespace

int batch_num_pass(uint32_t num_mesh) {
  int bits = 30;
  uint32_t m = num_mesh > 0 ? num_mesh - 1 : 0;
  while (m) {
    ++bits;
    m >>= 1;
  }
  return (bits + 7) / 8;
}

void launch_batch_fit(cudaStream_t s, const Segments& seg, const uint32_t* tri2vtx, const float* vtx2xyz,
                      float* transforms, uint32_t* status) {
  k_batch_fit<<<seg.num_mesh, kThreads, 0, s>>>(seg, tri2vtx, vtx2xyz, transforms, status);
}

void launch_batch_morton(cudaStream_t s, uint32_t total_tri, const Segments& seg, const uint32_t* tri2vtx,
                         const float* vtx2xyz, const float* transforms, uint64_t* keys, uint32_t* hist, int num_pass,
                         uint32_t* status) {
  uint32_t grid = (total_tri + kThreads * 8 - 1) / (kThreads * 8);
  if (grid < 1) grid = 1;
  if (grid > 152 * 16) grid = 152 * 16;
  k_batch_morton<<<grid, kThreads, 0, s>>>(total_tri, seg, tri2vtx, vtx2xyz, transforms, keys, hist, num_pass, status);
}

void launch_batch_topology(cudaStream_t s, uint32_t total_tri, const Segments& seg, const uint64_t* keys,
                           const uint32_t* vals, uint32_t* bvhnodes, uint32_t* other_end) {
  const uint32_t total_branch = total_tri - seg.num_mesh;
  const uint32_t n = total_branch > seg.num_mesh ? total_branch : seg.num_mesh;
  k_batch_topology<<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(total_branch, seg, keys, vals, bvhnodes,
                                                                     other_end);
}

namespace {
// Grid of the persistent k_batch_seg_build<kC>: as many blocks (kC == 1) or
// clusters as fit on the device at once, found once per device.
template <int kC>
int seg_build_w(cudaStream_t s, const SegArgs& a) {
  auto* kernel = k_batch_seg_build<kC>;
  const size_t smem = sizeof(SegSmem);
  cudaLaunchConfig_t cfg{};
  cfg.blockDim = dim3(kSegThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kC;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = kC > 1 ? 1 : 0;
  static int grid[64] = {0};  // the attribute and the grid are per device
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 1;
  if (grid[dev] == 0) {
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) !=
        cudaSuccess)
      return 1;
    int sms = 0, per_sm = 0, clusters = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (kC == 1) {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kSegThreads, smem);
      grid[dev] = sms * per_sm;
    } else {
      cfg.gridDim = dim3(kC * sms);
      cudaOccupancyMaxActiveClusters(&clusters, kernel, &cfg);
      grid[dev] = clusters * kC;
    }
    if (grid[dev] <= 0) {
      grid[dev] = 0;
      cudaGetLastError();
      return 1;
    }
  }
  cfg.gridDim = dim3(grid[dev]);
  return cudaLaunchKernelEx(&cfg, kernel, a) == cudaSuccess ? 0 : 1;
}
}  // namespace

int launch_batch_seg_build(cudaStream_t s, const Segments& seg, uint32_t max_tri, const uint32_t* tri2vtx,
                           const float* vtx2xyz, uint32_t* bvhnodes, uint32_t* other, uint32_t* lists,
                           uint32_t* counters, uint32_t* status) {
  if (max_tri == 0 || max_tri > kSegMaxTri) return 1;
  k_batch_seg_classify<<<(seg.num_mesh + kThreads - 1) / kThreads, kThreads, 0, s>>>(seg, max_tri, lists, counters,
                                                                                      status);
  const SegArgs a{seg, tri2vtx, vtx2xyz, bvhnodes, other, lists, counters, counters + 2, status};
  // the fewest blocks that hold the largest mesh, or more if tuned so (a
  // cluster builds every mesh above one block's capacity; smaller meshes are
  // built by single blocks either way)
  const uint32_t least = get_tuning().batch_cluster;
  if (max_tri <= kSegCap && least <= 1) return seg_build_w<1>(s, a);
  if (max_tri <= 2 * kSegCap && least <= 2) return seg_build_w<2>(s, a);
  return seg_build_w<4>(s, a);
}

void launch_batch_cast_pixels(cudaStream_t s, const Segments& seg, uint32_t max_tri, const uint32_t* tri2vtx,
                              const float* vtx2xyz, const uint32_t* bvhnodes, const float* aabb, uint32_t img_w,
                              uint32_t img_h, const float* transforms, const CastOut& o, const CastScratch& sc,
                              uint32_t* status) {
  BatchJob job{};
  job.seg = seg;
  job.tri2vtx = tri2vtx;
  job.vtx2xyz = vtx2xyz;
  job.bvhnodes = bvhnodes;
  job.aabb = aabb;
  job.img_w = img_w;
  job.img_h = img_h;
  const Tuning t = get_tuning();
  job.tile_w = t.tile_w;
  job.tile_h = 32u / t.tile_w;
  job.tile_w_log = static_cast<uint32_t>(__builtin_ctz(t.tile_w));
  job.tiles_x = (img_w + job.tile_w - 1) / job.tile_w;
  job.work_per_mesh = job.tiles_x * ((img_h + job.tile_h - 1) / job.tile_h) * 32u;
  job.by_work_per_mesh = Divider::make(job.work_per_mesh);
  job.by_tiles_x = Divider::make(job.tiles_x);
  job.num_work = job.work_per_mesh * seg.num_mesh;
  job.transforms = transforms;
  job.o = o;
  cast_job(s, job, sc, max_tri, status);
}

}  // namespace dm
