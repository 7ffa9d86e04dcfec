// dm_device.cuh — device helpers shared by the LBVH build and ray-cast kernels.
//
// Every floating-point expression here is written with explicit round-to-
// nearest intrinsics (__fadd_rn, __fmul_rn, ...) in the same operation order as
// the CPU restatement of del-msh-cpu, so that Morton codes, AABBs, hit ids and
// hit distances are bit-identical to it.  The library is also compiled with
// -fmad=false so that no other expression is contracted into an FMA.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace dm {

constexpr uint32_t kUMax = 0xFFFFFFFFu;

// Bits OR-ed into the library's device status word (see capi.cu).
enum DeviceStatusBits : uint32_t {
  kStatusSpinTimeout = 1u,  // a bounded wait in a kernel gave up
  kStatusStackOverflow = 2u,  // a traversal stack tier was too small
  kStatusBadIndex = 4u,  // an index read from an input array was out of range
  kStatusSingular = 8u,  // a matrix to invert was singular (the result is NaN)
};

// Programmatic dependent launch.  A kernel launched with
// launch_pdl (dm_internal.h) may start while its predecessor in the stream
// is still running; pdl_wait() returns once the predecessor has completed
// and its writes are visible (at once for a normal launch).  Each such
// kernel calls pdl_launch_dependents() only after pdl_wait(), so when the
// next kernel starts early every kernel before this one has completed: code
// before pdl_wait() may read results of those, but nothing this kernel's
// predecessor writes, and may write nothing that it reads.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

__device__ __forceinline__ void raise_status(uint32_t* status, uint32_t bits) {
  if (status) atomicOr(status, bits);
}

// Lanes of the warp holding the same 8-bit digit, among the valid lanes: one
// ballot per digit bit.  Measured on GB300, this is several times faster than
// __match_any_sync, which made ranking the longest phase of a radix pass.
__device__ __forceinline__ uint32_t warp_peers(uint32_t d, bool valid) {
  uint32_t peers = __ballot_sync(0xffffffffu, valid);
#pragma unroll
  for (int b = 0; b < 8; ++b) {
    const bool bit = (d >> b) & 1u;
    const uint32_t bb = __ballot_sync(0xffffffffu, bit);
    peers &= bit ? bb : ~bb;
  }
  return peers;
}

// ------------------------------------------------------------- Morton codes

// mortons.rs:76-81
__device__ __forceinline__ uint32_t expand_bits3(uint32_t x) {
  x = (x | (x << 16)) & 0x030000FFu;
  x = (x | (x << 8)) & 0x0300F00Fu;
  x = (x | (x << 4)) & 0x030C30C3u;
  return (x | (x << 2)) & 0x09249249u;
}

// mortons.rs:3-8
__device__ __forceinline__ uint32_t expand_bits2(uint32_t x) {
  x = (x | (x << 8)) & 0x00ff00ffu;
  x = (x | (x << 4)) & 0x0f0f0f0fu;
  x = (x | (x << 2)) & 0x33333333u;
  return (x | (x << 1)) & 0x55555555u;
}

// Rust `v.clamp(0, hi) as u32`: NaN survives the clamp and casts to 0.
__device__ __forceinline__ uint32_t quantize(float v, float hi) {
  if (v < 0.0f) v = 0.0f;
  else if (v > hi) v = hi;
  return (v != v) ? 0u : static_cast<uint32_t>(v);
}

// mortons.rs:94-102
__device__ __forceinline__ uint32_t morton_code3(float x, float y, float z) {
  const uint32_t ix = expand_bits3(quantize(__fmul_rn(x, 1024.0f), 1023.0f));
  const uint32_t iy = expand_bits3(quantize(__fmul_rn(y, 1024.0f), 1023.0f));
  const uint32_t iz = expand_bits3(quantize(__fmul_rn(z, 1024.0f), 1023.0f));
  return ix * 4u + iy * 2u + iz;
}

// mortons.rs:20-27
__device__ __forceinline__ uint32_t morton_code2(float x, float y) {
  const uint32_t ix = expand_bits2(quantize(__fmul_rn(x, 65536.0f), 65535.0f));
  const uint32_t iy = expand_bits2(quantize(__fmul_rn(y, 65536.0f), 65535.0f));
  return ix * 2u + iy;
}

// ----------------------------------------------------------- f32 geometry

// Column-major homogeneous transform, each row summed left to right, then
// divided by w (mat4_col_major::transform_homogeneous).
__device__ __forceinline__ float3 transform_homogeneous(const float* m, float x, float y, float z) {
  const float w = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[3], x), __fmul_rn(m[7], y)), __fmul_rn(m[11], z)), m[15]);
  const float ox = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], x), __fmul_rn(m[4], y)), __fmul_rn(m[8], z)), m[12]);
  const float oy = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[1], x), __fmul_rn(m[5], y)), __fmul_rn(m[9], z)), m[13]);
  const float oz = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[2], x), __fmul_rn(m[6], y)), __fmul_rn(m[10], z)), m[14]);
  return make_float3(__fdiv_rn(ox, w), __fdiv_rn(oy, w), __fdiv_rn(oz, w));
}

// transform_homogeneous with the three divisions skipped when w is exactly
// 1, as it is for an affine matrix (bottom row 0 0 0 1) and finite input:
// x / 1 is x, so the result is the same bits.  Otherwise (a projective
// matrix, or 0 * inf = NaN in w) it divides as transform_homogeneous does.
__device__ __forceinline__ float3 transform_homogeneous_w1(const float* m, float x, float y, float z) {
  const float w = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[3], x), __fmul_rn(m[7], y)), __fmul_rn(m[11], z)), m[15]);
  const float ox = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], x), __fmul_rn(m[4], y)), __fmul_rn(m[8], z)), m[12]);
  const float oy = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[1], x), __fmul_rn(m[5], y)), __fmul_rn(m[9], z)), m[13]);
  const float oz = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[2], x), __fmul_rn(m[6], y)), __fmul_rn(m[10], z)), m[14]);
  if (w == 1.0f) return make_float3(ox, oy, oz);
  return make_float3(__fdiv_rn(ox, w), __fdiv_rn(oy, w), __fdiv_rn(oz, w));
}

__device__ __forceinline__ float2 transform_homogeneous2(const float* m, float x, float y) {
  const float w = __fadd_rn(__fadd_rn(__fmul_rn(m[2], x), __fmul_rn(m[5], y)), m[8]);
  const float ox = __fadd_rn(__fadd_rn(__fmul_rn(m[0], x), __fmul_rn(m[3], y)), m[6]);
  const float oy = __fadd_rn(__fadd_rn(__fmul_rn(m[1], x), __fmul_rn(m[4], y)), m[7]);
  return make_float2(__fdiv_rn(ox, w), __fdiv_rn(oy, w));
}

// elem2center.rs:40-53: ((0 + p0) + p1) + p2, times the f32 value of 1/3.
__device__ __forceinline__ float centroid1(float a, float b, float c) {
  return __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(0.0f, a), b), c), 1.0f / 3.0f);
}

__device__ __forceinline__ float3 sub3(float3 a, float3 b) {
  return make_float3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}
__device__ __forceinline__ float dot3(float3 a, float3 b) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
  return make_float3(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)),
                     __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
                     __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}

// Moller & Trumbore (1997), no back-face culling: det == 0 misses, edges are
// inclusive, t >= 0 hits; every comparison rejects NaN.
__device__ __forceinline__ bool tri_ray(float3 p0, float3 p1, float3 p2, float3 org, float3 dir, float& t, float& u,
                                        float& v) {
  const float3 e1 = sub3(p1, p0), e2 = sub3(p2, p0), tv = sub3(org, p0);
  const float3 pv = cross3(dir, e2);
  const float det = dot3(e1, pv);
  if (det == 0.0f) return false;
  const float inv_det = __fdiv_rn(1.0f, det);
  u = __fmul_rn(dot3(tv, pv), inv_det);
  if (!(u >= 0.0f && u <= 1.0f)) return false;
  const float3 qv = cross3(tv, e1);
  v = __fmul_rn(dot3(dir, qv), inv_det);
  if (!(v >= 0.0f && __fadd_rn(u, v) <= 1.0f)) return false;
  const float tt = __fmul_rn(dot3(e2, qv), inv_det);
  if (!(tt >= 0.0f)) return false;
  t = tt;
  return true;
}

// Slab test (Kay & Kajiya 1986; Williams et al. 2005) with precomputed 1/dir;
// entry / exit per axis and their running max / min use IEEE minNum / maxNum
// (fminf / fmaxf: a NaN operand yields the other), as the CPU restatement
// does with libm's fminf / fmaxf.  A zero direction component hits iff the
// origin lies inside that slab.  True iff t_enter <= t_exit and t_exit >= 0.
// The sign of a zero result may differ from the CPU's; every use of these
// values is a comparison, for which -0 == +0.
__device__ __forceinline__ bool slab_axis(float lo, float hi, float o, float inv, float d, float& tmin, float& tmax) {
  if (d != 0.0f) {
    const float t0 = __fmul_rn(__fsub_rn(lo, o), inv);
    const float t1 = __fmul_rn(__fsub_rn(hi, o), inv);
    tmin = fmaxf(tmin, fminf(t0, t1));
    tmax = fminf(tmax, fmaxf(t0, t1));
    return true;
  }
  return !(o < lo || o > hi);
}

__device__ __forceinline__ bool slab(const float* __restrict__ box, float3 org, float3 inv, float3 dir, float& te,
                                     float& tx) {
  const float2 a = __ldg(reinterpret_cast<const float2*>(box));
  const float2 b = __ldg(reinterpret_cast<const float2*>(box) + 1);
  const float2 c = __ldg(reinterpret_cast<const float2*>(box) + 2);
  float tmin = -INFINITY, tmax = INFINITY;
  if (!slab_axis(a.x, b.y, org.x, inv.x, dir.x, tmin, tmax)) return false;
  if (!slab_axis(a.y, c.x, org.y, inv.y, dir.y, tmin, tmax)) return false;
  if (!slab_axis(b.x, c.y, org.z, inv.z, dir.z, tmin, tmax)) return false;
  if (!(tmin <= tmax) || tmax < 0.0f) return false;
  te = tmin;
  tx = tmax;
  return true;
}

// slab() for a direction with no zero component: the same operations in the
// same order, without the per-axis test.
__device__ __forceinline__ bool slab_nz(const float* __restrict__ box, float3 org, float3 inv, float& te, float& tx) {
  const float2 a = __ldg(reinterpret_cast<const float2*>(box));
  const float2 b = __ldg(reinterpret_cast<const float2*>(box) + 1);
  const float2 c = __ldg(reinterpret_cast<const float2*>(box) + 2);
  const float x0 = __fmul_rn(__fsub_rn(a.x, org.x), inv.x), x1 = __fmul_rn(__fsub_rn(b.y, org.x), inv.x);
  const float y0 = __fmul_rn(__fsub_rn(a.y, org.y), inv.y), y1 = __fmul_rn(__fsub_rn(c.x, org.y), inv.y);
  const float z0 = __fmul_rn(__fsub_rn(b.x, org.z), inv.z), z1 = __fmul_rn(__fsub_rn(c.y, org.z), inv.z);
  float tmin = fmaxf(-INFINITY, fminf(x0, x1)), tmax = fminf(INFINITY, fmaxf(x0, x1));
  tmin = fmaxf(tmin, fminf(y0, y1));
  tmax = fminf(tmax, fmaxf(y0, y1));
  tmin = fmaxf(tmin, fminf(z0, z1));
  tmax = fminf(tmax, fmaxf(z0, z1));
  te = tmin;
  tx = tmax;
  return tmin <= tmax && !(tmax < 0.0f);
}

// Rust's lexicographic `<` on (f32, f32) tuples.
__device__ __forceinline__ bool tuple_lt(float a0, float a1, float b0, float b1) {
  return (a0 == b0) ? (a1 < b1) : (a0 < b0);
}

// ray_for_pixel.h:3-19 for the pixel in column iw, row ih.
__device__ __forceinline__ void ray_for_pixel_xy(uint32_t iw, uint32_t ih, uint32_t img_w, uint32_t img_h,
                                                 const float* m, float3& org, float3& dir) {
  const float x0 = __fsub_rn(__fdiv_rn(__fmul_rn(2.0f, __fadd_rn(static_cast<float>(iw), 0.5f)),
                                       static_cast<float>(img_w)),
                             1.0f);
  const float y0 = __fsub_rn(1.0f, __fdiv_rn(__fmul_rn(2.0f, __fadd_rn(static_cast<float>(ih), 0.5f)),
                                             static_cast<float>(img_h)));
  const float3 q0 = transform_homogeneous(m, x0, y0, 1.0f);
  const float3 q1 = transform_homogeneous(m, x0, y0, -1.0f);
  org = q0;
  dir = sub3(q1, q0);
}

// ray_for_pixel.h:3-19 for pixel i_pix (row-major).
__device__ __forceinline__ void ray_for_pixel(uint32_t i_pix, uint32_t img_w, uint32_t img_h, const float* m,
                                              float3& org, float3& dir) {
  const uint32_t ih = i_pix / img_w;
  ray_for_pixel_xy(i_pix - ih * img_w, ih, img_w, img_h, m, org, dir);
}

// n / d for any 32-bit n by a 64-bit multiply-high with magic = ceil(2^64 / d):
// n * magic / 2^64 exceeds n / d by less than n / 2^64 < 2^-32 < 1 / d, so the
// floor is exact.  For the per-ray index arithmetic of the casts.
struct Divider {
  uint32_t d;
  unsigned long long magic;  // 0 for d == 1
  __host__ static Divider make(uint32_t d) {
    return Divider{d, d <= 1 ? 0ull : ~0ull / d + 1ull};
  }
  __device__ __forceinline__ uint32_t div(uint32_t n) const {
    return d <= 1 ? n : static_cast<uint32_t>(__umul64hi(static_cast<unsigned long long>(n), magic));
  }
};

// ---------------------------------------------------------------- AABBs

// aabb3::set_as_cube / add_point with eps: box [p-eps, p+eps] widened by
// strict comparisons (the first value stays on ties).
struct Box {
  float lo[3], hi[3];
};

__device__ __forceinline__ void box_set(Box& b, float3 p, float eps) {
  b.lo[0] = __fsub_rn(p.x, eps);
  b.lo[1] = __fsub_rn(p.y, eps);
  b.lo[2] = __fsub_rn(p.z, eps);
  b.hi[0] = __fadd_rn(p.x, eps);
  b.hi[1] = __fadd_rn(p.y, eps);
  b.hi[2] = __fadd_rn(p.z, eps);
}
__device__ __forceinline__ void box_add(Box& b, float3 p, float eps) {
  const float l[3] = {__fsub_rn(p.x, eps), __fsub_rn(p.y, eps), __fsub_rn(p.z, eps)};
  const float h[3] = {__fadd_rn(p.x, eps), __fadd_rn(p.y, eps), __fadd_rn(p.z, eps)};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (l[d] < b.lo[d]) b.lo[d] = l[d];
    if (h[d] > b.hi[d]) b.hi[d] = h[d];
  }
}
// aabb3::from_two_aabbs: component-wise union, the first box wins ties.
__device__ __forceinline__ Box box_union(const Box& a, const Box& b) {
  Box o;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    o.lo[d] = (b.lo[d] < a.lo[d]) ? b.lo[d] : a.lo[d];
    o.hi[d] = (b.hi[d] > a.hi[d]) ? b.hi[d] : a.hi[d];
  }
  return o;
}

__device__ __forceinline__ void box_store(float* dst, const Box& b) {
  float2* d2 = reinterpret_cast<float2*>(dst);
  d2[0] = make_float2(b.lo[0], b.lo[1]);
  d2[1] = make_float2(b.lo[2], b.hi[0]);
  d2[2] = make_float2(b.hi[1], b.hi[2]);
}

// L2-coherent load (the box may have been written by another SM in this launch).
__device__ __forceinline__ Box box_load_cg(const float* src) {
  const float2* s2 = reinterpret_cast<const float2*>(src);
  const float2 a = __ldcg(s2), b = __ldcg(s2 + 1), c = __ldcg(s2 + 2);
  Box o;
  o.lo[0] = a.x;
  o.lo[1] = a.y;
  o.lo[2] = b.x;
  o.hi[0] = b.y;
  o.hi[1] = c.x;
  o.hi[2] = c.y;
  return o;
}

__device__ __forceinline__ float3 load_vtx(const float* __restrict__ vtx2xyz, uint32_t i) {
  const float* p = vtx2xyz + static_cast<size_t>(i) * 3;
  return make_float3(__ldg(p), __ldg(p + 1), __ldg(p + 2));
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

// tri_centroid, and the triangle's box exactly as leaf_box computes it (the
// same vertex loads, eps 0) into *box.
__device__ __forceinline__ float3 tri_centroid_box(const uint32_t* __restrict__ tri2vtx, uint32_t num_vtx,
                                                   const float* __restrict__ vtx2xyz, uint32_t it, uint32_t* status,
                                                   Box* box) {
  const uint32_t* t = tri2vtx + static_cast<size_t>(it) * 3;
  const float3 p0 = load_vtx(vtx2xyz, vtx_index(t, num_vtx, status));
  const float3 p1 = load_vtx(vtx2xyz, vtx_index(t + 1, num_vtx, status));
  const float3 p2 = load_vtx(vtx2xyz, vtx_index(t + 2, num_vtx, status));
  box_set(*box, p0, 0.0f);
  box_add(*box, p1, 0.0f);
  box_add(*box, p2, 0.0f);
  return make_float3(centroid1(p0.x, p1.x, p2.x), centroid1(p0.y, p1.y, p2.y), centroid1(p0.z, p1.z, p2.z));
}


}  // namespace dm
