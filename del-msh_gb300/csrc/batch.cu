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

#include "dm_lbvh.cuh"
#include "dm_traverse.cuh"

namespace dm {
namespace {

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
  const float3 c0 = centroid_at(t2v, x, V, 0, status);
  const float c0a[3] = {c0.x, c0.y, c0.z};
  for (int d = 0; d < 3; ++d)
    if (c0a[d] != c0a[d]) lo[d] = hi[d] = c0a[d];
  float ext = __fsub_rn(hi[0], lo[0]);
  const float ey = __fsub_rn(hi[1], lo[1]), ez = __fsub_rn(hi[2], lo[2]);
  if (ey > ext) ext = ey;
  if (ez > ext) ext = ez;
  const float s = __fdiv_rn(1.0f, ext);
  float* mo = transforms + 16ull * m;
  for (int k = 0; k < 16; ++k) mo[k] = 0.0f;
  mo[0] = s;
  mo[5] = s;
  mo[10] = s;
  mo[15] = 1.0f;
  for (int d = 0; d < 3; ++d) {
    const float c = __fmul_rn(__fadd_rn(lo[d], hi[d]), 0.5f);
    mo[12 + d] = __fadd_rn(__fmul_rn(-c, s), 0.5f);
  }
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

// ------------------------------------------------------------ batch cast


struct BatchJob {
  uint32_t num_work;
  Segments seg;
  const uint32_t* tri2vtx;
  const float* vtx2xyz;
  const uint32_t* bvhnodes;
  const float* aabb;
  uint32_t img_w, img_h, tiles_x, tile_w, tile_h, work_per_mesh;
  const float* transforms;  // num_mesh x 16, column-major ndc -> world
  CastOut o;

  __device__ __forceinline__ void prepare(float*) const {}

  __device__ __forceinline__ bool fetch(uint32_t w, const float*, MeshView& mv, Ray& r, uint32_t& out) const {
    const uint32_t m = w / work_per_mesh, lw = w - m * work_per_mesh;
    const uint32_t tile = lw >> 5, j = lw & 31u;
    const uint32_t px = (tile % tiles_x) * tile_w + (j % tile_w);
    const uint32_t py = (tile / tiles_x) * tile_h + (j / tile_w);
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
    ray_for_pixel(pix, img_w, img_h, mm, o3, d3);
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
  job.tiles_x = (img_w + job.tile_w - 1) / job.tile_w;
  job.work_per_mesh = job.tiles_x * ((img_h + job.tile_h - 1) / job.tile_h) * 32u;
  job.num_work = job.work_per_mesh * seg.num_mesh;
  job.transforms = transforms;
  job.o = o;
  cast_job(s, job, sc, max_tri, status);
}

}  // namespace dm
