// render.cu — the consumers of a pix2tri image: per-pixel depth
// (pix2depth.cu:12-97, CPU pix2depth.rs:107-146) and per-pixel interpolation
// of vertex attributes (pix2tri.cu:79-183, CPU pix2tri.rs:176-304), forward
// and backward.  One thread per pixel; the pixel ray is ray_for_pixel.h's,
// as for the cast, so a pixel's intersection is the cast's bit for bit.
//
// The forward outputs are bit-exact to the CPU restatement.  The backward
// passes accumulate into shared vertices with atomicAdd, as the reference's
// GPU kernels do, so their sums are order-dependent (equal to the sequential
// CPU sums up to float reassociation).
//
// Formulas of del-geo-core (absent from the reference checkout), restated:
// - intersection of the pixel ray with the triangle: Moller-Trumbore (the
//   cast's tri_ray); the "line" form drops the inside / t >= 0 tests;
// - backward of (t, u, v) with respect to the vertices, by implicit
//   differentiation of o + t d = p0 + u (p1-p0) + v (p2-p0): with
//   A = [-d | p1-p0 | p2-p0] and lambda = A^-T (dL/dt, dL/du, dL/dv),
//   dL/dp0 = -(1-u-v) lambda, dL/dp1 = -u lambda, dL/dp2 = -v lambda;
// - the inverse of the ndc->world matrix: Gauss-Jordan elimination with
//   partial pivoting, in f32 (mat4_col_major::try_inverse_with_pivot);
// - the Jacobian of the homogeneous transform at q:
//   d ndc_i / d q_j = (M_ij w - v_i M_3j) / w^2, v = M (q, 1), w = v_3.
#include "dm_device.cuh"
#include "dm_internal.h"

namespace dm {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float3 scale3(float3 a, float s) {
  return make_float3(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s));
}

// Moller-Trumbore on the line through the pixel ray: false only for det == 0.
__device__ __forceinline__ bool tri_line(float3 p0, float3 p1, float3 p2, float3 org, float3 dir, float& t, float& u,
                                         float& v) {
  const float3 e1 = sub3(p1, p0), e2 = sub3(p2, p0), tv = sub3(org, p0);
  const float3 pv = cross3(dir, e2);
  const float det = dot3(e1, pv);
  if (det == 0.0f) return false;
  const float inv_det = __fdiv_rn(1.0f, det);
  u = __fmul_rn(dot3(tv, pv), inv_det);
  const float3 qv = cross3(tv, e1);
  v = __fmul_rn(dot3(dir, qv), inv_det);
  t = __fmul_rn(dot3(e2, qv), inv_det);
  return true;
}

// Backward of (t, u, v) to the three vertices (see the file comment).
__device__ __forceinline__ void tri_line_bwd(float3 p0, float3 p1, float3 p2, float3 dir, float u, float v, float gt,
                                             float gu, float gv, float3& d0, float3& d1, float3& d2) {
  const float3 c0 = make_float3(-dir.x, -dir.y, -dir.z), c1 = sub3(p1, p0), c2 = sub3(p2, p0);
  const float3 x12 = cross3(c1, c2), x20 = cross3(c2, c0), x01 = cross3(c0, c1);
  const float det = dot3(c0, x12);
  const float inv = __fdiv_rn(1.0f, det);
  // lambda = (gt * x12 + gu * x20 + gv * x01) / det
  const float3 lam = scale3(make_float3(__fadd_rn(__fadd_rn(__fmul_rn(gt, x12.x), __fmul_rn(gu, x20.x)), __fmul_rn(gv, x01.x)),
                                        __fadd_rn(__fadd_rn(__fmul_rn(gt, x12.y), __fmul_rn(gu, x20.y)), __fmul_rn(gv, x01.y)),
                                        __fadd_rn(__fadd_rn(__fmul_rn(gt, x12.z), __fmul_rn(gu, x20.z)), __fmul_rn(gv, x01.z))),
                            inv);
  const float w0 = __fsub_rn(__fsub_rn(1.0f, u), v);
  d0 = scale3(lam, -w0);
  d1 = scale3(lam, -u);
  d2 = scale3(lam, -v);
}

__device__ __forceinline__ bool tri_vertices(const uint32_t* __restrict__ tri2vtx, uint32_t num_tri, uint32_t num_vtx,
                                             const float* __restrict__ vtx2xyz, uint32_t it, uint32_t iv[3], float3 p[3],
                                             uint32_t* status) {
  if (it >= num_tri) {
    raise_status(status, kStatusBadIndex);
    return false;
  }
  for (int k = 0; k < 3; ++k) {
    iv[k] = __ldg(tri2vtx + static_cast<size_t>(it) * 3 + k);
    if (iv[k] >= num_vtx) {
      raise_status(status, kStatusBadIndex);
      return false;
    }
    p[k] = load_vtx(vtx2xyz, iv[k]);
  }
  return true;
}

// One thread: world2ndc = inverse(ndc2world), Gauss-Jordan with partial
// pivoting on [M | I] (row r, column c of M at m[c*4 + r]); a zero pivot
// column raises kStatusSingular and leaves NaN.
__global__ void k_inverse4(const float* __restrict__ m, float* inv, uint32_t* status) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  // fully unrolled so that the 4x8 array stays in registers; the row swap
  // selects instead of indexing with the pivot row
  float a[4][8];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      a[r][c] = m[c * 4 + r];
      a[r][4 + c] = (r == c) ? 1.0f : 0.0f;
    }
  bool singular = false;
#pragma unroll
  for (int col = 0; col < 4; ++col) {
    int piv = col;
    float best = fabsf(a[col][col]);
#pragma unroll
    for (int r = col + 1; r < 4; ++r)
      if (fabsf(a[r][col]) > best) {
        best = fabsf(a[r][col]);
        piv = r;
      }
    singular = singular || (best == 0.0f);
#pragma unroll
    for (int r = col + 1; r < 4; ++r) {
      const bool sw = (r == piv);
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const float x = a[col][c], y = a[r][c];
        a[col][c] = sw ? y : x;
        a[r][c] = sw ? x : y;
      }
    }
    const float d = a[col][col];
#pragma unroll
    for (int c = 0; c < 8; ++c) a[col][c] = __fdiv_rn(a[col][c], d);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      if (r == col) continue;
      const float f = a[r][col];
#pragma unroll
      for (int c = 0; c < 8; ++c) a[r][c] = __fsub_rn(a[r][c], __fmul_rn(f, a[col][c]));
    }
  }
  if (singular) {
    raise_status(status, kStatusSingular);
#pragma unroll
    for (int k = 0; k < 16; ++k) inv[k] = NAN;
    return;
  }
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) inv[c * 4 + r] = a[r][4 + c];
}

// pix2depth.cu:12-50: depth = (ndc_z + 1) / 2 at the hit point; background 0;
// a pixel whose ray misses its triangle is left unchanged.
__global__ void __launch_bounds__(kThreads) k_pix2depth(uint32_t img_w, uint32_t img_h, float* __restrict__ pix2depth,
                                                       const uint32_t* __restrict__ pix2tri, uint32_t num_tri,
                                                       const uint32_t* __restrict__ tri2vtx, uint32_t num_vtx,
                                                       const float* __restrict__ vtx2xyz,
                                                       const float* __restrict__ ndc2world,
                                                       const float* __restrict__ world2ndc, uint32_t* status) {
  __shared__ float sm[32];
  if (threadIdx.x < 16) sm[threadIdx.x] = ndc2world[threadIdx.x];
  else if (threadIdx.x < 32) sm[threadIdx.x] = world2ndc[threadIdx.x - 16];
  __syncthreads();
  const uint32_t i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= img_w * img_h) return;
  const uint32_t it = pix2tri[i];
  if (it == kUMax) {
    pix2depth[i] = 0.0f;
    return;
  }
  uint32_t iv[3];
  float3 p[3];
  if (!tri_vertices(tri2vtx, num_tri, num_vtx, vtx2xyz, it, iv, p, status)) return;
  float3 o, d;
  ray_for_pixel(i, img_w, img_h, sm, o, d);
  float t, u, v;
  if (!tri_ray(p[0], p[1], p[2], o, d, t, u, v)) return;
  const float3 q = make_float3(__fadd_rn(__fmul_rn(t, d.x), o.x), __fadd_rn(__fmul_rn(t, d.y), o.y),
                               __fadd_rn(__fmul_rn(t, d.z), o.z));
  const float3 ndc = transform_homogeneous(sm + 16, q.x, q.y, q.z);
  pix2depth[i] = __fmul_rn(__fadd_rn(ndc.z, 1.0f), 0.5f);
}

// pix2depth.cu:52-97: dL/dvtx2xyz += d depth / d vertices * dL/ddepth.
__global__ void __launch_bounds__(kThreads) k_pix2depth_bwd(uint32_t img_w, uint32_t img_h, float* dldw_vtx2xyz,
                                                           const uint32_t* __restrict__ pix2tri, uint32_t num_tri,
                                                           const uint32_t* __restrict__ tri2vtx, uint32_t num_vtx,
                                                           const float* __restrict__ vtx2xyz,
                                                           const float* __restrict__ dldw_pix2depth,
                                                           const float* __restrict__ ndc2world,
                                                           const float* __restrict__ world2ndc, uint32_t* status) {
  __shared__ float sm[32];
  if (threadIdx.x < 16) sm[threadIdx.x] = ndc2world[threadIdx.x];
  else if (threadIdx.x < 32) sm[threadIdx.x] = world2ndc[threadIdx.x - 16];
  __syncthreads();
  const uint32_t i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= img_w * img_h) return;
  const uint32_t it = pix2tri[i];
  if (it == kUMax) return;
  uint32_t iv[3];
  float3 p[3];
  if (!tri_vertices(tri2vtx, num_tri, num_vtx, vtx2xyz, it, iv, p, status)) return;
  float3 o, d;
  ray_for_pixel(i, img_w, img_h, sm, o, d);
  float t, u, v;
  if (!tri_line(p[0], p[1], p[2], o, d, t, u, v)) return;
  const float* M = sm + 16;
  const float q[3] = {__fadd_rn(__fmul_rn(t, d.x), o.x), __fadd_rn(__fmul_rn(t, d.y), o.y),
                      __fadd_rn(__fmul_rn(t, d.z), o.z)};
  float vv[4];
  for (int r = 0; r < 4; ++r)
    vv[r] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(M[r], q[0]), __fmul_rn(M[4 + r], q[1])), __fmul_rn(M[8 + r], q[2])),
                      M[12 + r]);
  const float w = vv[3], ww = __fmul_rn(w, w);
  const float g_ndc[3] = {0.0f, 0.0f, __fmul_rn(0.5f, dldw_pix2depth[i])};
  float gq[3];
  for (int j = 0; j < 3; ++j) {  // gq = J^T g_ndc, J_ij = (M_ij w - v_i M_3j) / w^2
    float s = 0.0f;
    for (int r = 0; r < 3; ++r) {
      const float jij = __fdiv_rn(__fsub_rn(__fmul_rn(M[j * 4 + r], w), __fmul_rn(vv[r], M[j * 4 + 3])), ww);
      s = __fadd_rn(s, __fmul_rn(jij, g_ndc[r]));
    }
    gq[j] = s;
  }
  const float gt = __fadd_rn(__fadd_rn(__fmul_rn(gq[0], d.x), __fmul_rn(gq[1], d.y)), __fmul_rn(gq[2], d.z));
  float3 g[3];
  tri_line_bwd(p[0], p[1], p[2], d, u, v, gt, 0.0f, 0.0f, g[0], g[1], g[2]);
  for (int k = 0; k < 3; ++k) {
    atomicAdd(dldw_vtx2xyz + static_cast<size_t>(iv[k]) * 3, g[k].x);
    atomicAdd(dldw_vtx2xyz + static_cast<size_t>(iv[k]) * 3 + 1, g[k].y);
    atomicAdd(dldw_vtx2xyz + static_cast<size_t>(iv[k]) * 3 + 2, g[k].z);
  }
}

// pix2tri.cu:79-120: pix2val = bc0 v0 + bc1 v1 + bc2 v2 (0 on the background).
__global__ void __launch_bounds__(kThreads) k_interpolate(uint32_t img_w, uint32_t img_h,
                                                         const uint32_t* __restrict__ pix2tri, uint32_t num_tri,
                                                         const uint32_t* __restrict__ tri2vtx, uint32_t num_vtx,
                                                         const float* __restrict__ vtx2xyz, uint32_t num_vdim,
                                                         const float* __restrict__ vtx2val,
                                                         const float* __restrict__ ndc2world, float* pix2val,
                                                         uint32_t* status) {
  __shared__ float sm[16];
  if (threadIdx.x < 16) sm[threadIdx.x] = ndc2world[threadIdx.x];
  __syncthreads();
  const uint32_t i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= img_w * img_h) return;
  float* out = pix2val + static_cast<size_t>(i) * num_vdim;
  const uint32_t it = pix2tri[i];
  uint32_t iv[3];
  float3 p[3];
  float t = 0.f, u = 0.f, v = 0.f;
  bool ok = it != kUMax && tri_vertices(tri2vtx, num_tri, num_vtx, vtx2xyz, it, iv, p, status);
  if (ok) {
    float3 o, d;
    ray_for_pixel(i, img_w, img_h, sm, o, d);
    ok = tri_line(p[0], p[1], p[2], o, d, t, u, v);
  }
  if (!ok) {
    for (uint32_t k = 0; k < num_vdim; ++k) out[k] = 0.0f;
    return;
  }
  const float b0 = __fsub_rn(__fsub_rn(1.0f, u), v);
  for (uint32_t k = 0; k < num_vdim; ++k)
    out[k] = __fadd_rn(__fadd_rn(__fmul_rn(b0, __ldg(vtx2val + static_cast<size_t>(iv[0]) * num_vdim + k)),
                                 __fmul_rn(u, __ldg(vtx2val + static_cast<size_t>(iv[1]) * num_vdim + k))),
                       __fmul_rn(v, __ldg(vtx2val + static_cast<size_t>(iv[2]) * num_vdim + k)));
}

// pix2tri.cu:122-183: backward of the interpolation to vertex positions and
// values.
__global__ void __launch_bounds__(kThreads) k_interpolate_bwd(uint32_t img_w, uint32_t img_h,
                                                             const uint32_t* __restrict__ pix2tri, uint32_t num_tri,
                                                             const uint32_t* __restrict__ tri2vtx, uint32_t num_vtx,
                                                             const float* __restrict__ vtx2xyz, uint32_t num_vdim,
                                                             const float* __restrict__ vtx2val,
                                                             const float* __restrict__ ndc2world,
                                                             const float* __restrict__ dldw_pix2val,
                                                             float* dldw_vtx2xyz, float* dldw_vtx2val,
                                                             uint32_t* status) {
  __shared__ float sm[16];
  if (threadIdx.x < 16) sm[threadIdx.x] = ndc2world[threadIdx.x];
  __syncthreads();
  const uint32_t i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= img_w * img_h) return;
  const uint32_t it = pix2tri[i];
  if (it == kUMax) return;
  uint32_t iv[3];
  float3 p[3];
  if (!tri_vertices(tri2vtx, num_tri, num_vtx, vtx2xyz, it, iv, p, status)) return;
  const float* g = dldw_pix2val + static_cast<size_t>(i) * num_vdim;
  float gb0 = 0.0f, gb1 = 0.0f, gb2 = 0.0f;
  for (uint32_t k = 0; k < num_vdim; ++k) {
    const float gk = g[k];
    gb0 = __fadd_rn(gb0, __fmul_rn(__ldg(vtx2val + static_cast<size_t>(iv[0]) * num_vdim + k), gk));
    gb1 = __fadd_rn(gb1, __fmul_rn(__ldg(vtx2val + static_cast<size_t>(iv[1]) * num_vdim + k), gk));
    gb2 = __fadd_rn(gb2, __fmul_rn(__ldg(vtx2val + static_cast<size_t>(iv[2]) * num_vdim + k), gk));
  }
  gb1 = __fsub_rn(gb1, gb0);  // bc0 = 1 - bc1 - bc2
  gb2 = __fsub_rn(gb2, gb0);
  float3 o, d;
  ray_for_pixel(i, img_w, img_h, sm, o, d);
  float t, u, v;
  if (!tri_line(p[0], p[1], p[2], o, d, t, u, v)) return;
  float3 dp[3];
  tri_line_bwd(p[0], p[1], p[2], d, u, v, 0.0f, gb1, gb2, dp[0], dp[1], dp[2]);
  for (int k = 0; k < 3; ++k) {
    atomicAdd(dldw_vtx2xyz + static_cast<size_t>(iv[k]) * 3, dp[k].x);
    atomicAdd(dldw_vtx2xyz + static_cast<size_t>(iv[k]) * 3 + 1, dp[k].y);
    atomicAdd(dldw_vtx2xyz + static_cast<size_t>(iv[k]) * 3 + 2, dp[k].z);
  }
  const float b[3] = {__fsub_rn(__fsub_rn(1.0f, u), v), u, v};
  for (uint32_t k = 0; k < num_vdim; ++k)
    for (int j = 0; j < 3; ++j)
      atomicAdd(dldw_vtx2val + static_cast<size_t>(iv[j]) * num_vdim + k, __fmul_rn(g[k], b[j]));
}

inline uint32_t grid_of(uint32_t n) { return (n + kThreads - 1) / kThreads; }

}  // namespace

void launch_inverse4(cudaStream_t s, const float* m, float* inv, uint32_t* status) {
  k_inverse4<<<1, 32, 0, s>>>(m, inv, status);
}

void launch_pix2depth(cudaStream_t s, uint32_t img_w, uint32_t img_h, float* pix2depth, const uint32_t* pix2tri,
                      const MeshView& m, const float* ndc2world, const float* world2ndc, uint32_t* status) {
  const uint32_t n = img_w * img_h;
  if (n == 0) return;
  k_pix2depth<<<grid_of(n), kThreads, 0, s>>>(img_w, img_h, pix2depth, pix2tri, m.num_tri, m.tri2vtx, m.num_vtx,
                                               m.vtx2xyz, ndc2world, world2ndc, status);
}

void launch_pix2depth_bwd(cudaStream_t s, uint32_t img_w, uint32_t img_h, float* dldw_vtx2xyz, const uint32_t* pix2tri,
                          const MeshView& m, const float* dldw_pix2depth, const float* ndc2world,
                          const float* world2ndc, uint32_t* status) {
  const uint32_t n = img_w * img_h;
  if (n == 0) return;
  k_pix2depth_bwd<<<grid_of(n), kThreads, 0, s>>>(img_w, img_h, dldw_vtx2xyz, pix2tri, m.num_tri, m.tri2vtx,
                                                   m.num_vtx, m.vtx2xyz, dldw_pix2depth, ndc2world, world2ndc,
                                                   status);
}

void launch_interpolate(cudaStream_t s, uint32_t img_w, uint32_t img_h, const uint32_t* pix2tri, const MeshView& m,
                        uint32_t num_vdim, const float* vtx2val, const float* ndc2world, float* pix2val,
                        uint32_t* status) {
  const uint32_t n = img_w * img_h;
  if (n == 0 || num_vdim == 0) return;
  k_interpolate<<<grid_of(n), kThreads, 0, s>>>(img_w, img_h, pix2tri, m.num_tri, m.tri2vtx, m.num_vtx, m.vtx2xyz,
                                                 num_vdim, vtx2val, ndc2world, pix2val, status);
}

void launch_interpolate_bwd(cudaStream_t s, uint32_t img_w, uint32_t img_h, const uint32_t* pix2tri,
                            const MeshView& m, uint32_t num_vdim, const float* vtx2val, const float* ndc2world,
                            const float* dldw_pix2val, float* dldw_vtx2xyz, float* dldw_vtx2val, uint32_t* status) {
  const uint32_t n = img_w * img_h;
  if (n == 0 || num_vdim == 0) return;
  k_interpolate_bwd<<<grid_of(n), kThreads, 0, s>>>(img_w, img_h, pix2tri, m.num_tri, m.tri2vtx, m.num_vtx,
                                                     m.vtx2xyz, num_vdim, vtx2val, ndc2world, dldw_pix2val,
                                                     dldw_vtx2xyz, dldw_vtx2val, status);
}

}  // namespace dm
