/*
 * oracle.c — CPU restatement of del-msh-cpu's LBVH build and BVH ray cast.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h): what the CUDA path's results are
 * tested against, and the timed CPU baseline.  Built with -O2 -ffp-contract=off so that every f32
 * expression rounds exactly as the reference's Rust code does.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define OR_UMAX 0xFFFFFFFFu

/* ------------------------------------------------------------------ Morton */

/* mortons.rs:76-81 */
uint32_t or_expand_bits3(uint32_t x) {
  x = (x | (x << 16)) & 0x030000FFu;
  x = (x | (x << 8)) & 0x0300F00Fu;
  x = (x | (x << 4)) & 0x030C30C3u;
  return (x | (x << 2)) & 0x09249249u;
}

/* mortons.rs:3-8 */
static uint32_t expand_bits2(uint32_t x) {
  x = (x | (x << 8)) & 0x00ff00ffu;
  x = (x | (x << 4)) & 0x0f0f0f0fu;
  x = (x | (x << 2)) & 0x33333333u;
  return (x | (x << 1)) & 0x55555555u;
}

/* Rust `(v).clamp(0, hi) as u32`: clamp keeps NaN, and a NaN cast to u32 is 0. */
static uint32_t quantize(float v, float hi) {
  if (v < 0.0f) v = 0.0f;
  else if (v > hi) v = hi;
  if (v != v) return 0u;
  return (uint32_t)v;
}

/* mortons.rs:94-102 */
uint32_t or_morton_code3(float x, float y, float z) {
  uint32_t ix = or_expand_bits3(quantize(x * 1024.0f, 1023.0f));
  uint32_t iy = or_expand_bits3(quantize(y * 1024.0f, 1023.0f));
  uint32_t iz = or_expand_bits3(quantize(z * 1024.0f, 1023.0f));
  return ix * 4u + iy * 2u + iz;
}

/* mortons.rs:20-27 */
uint32_t or_morton_code2(float x, float y) {
  uint32_t ix = expand_bits2(quantize(x * 65536.0f, 65535.0f));
  uint32_t iy = expand_bits2(quantize(y * 65536.0f, 65535.0f));
  return ix * 2u + iy;
}

/* ------------------------------------------------------ centroids and AABB */

/* elem2center.rs:25-54: cog starts at zero, nodes are summed in order 0,1,2,
 * and the sum is multiplied by the f32 value of 1/3. */
void or_tri2cntr(uint32_t num_tri, const uint32_t* tri2vtx, const float* vtx2xyz, float* tri2cntr) {
  const float ratio = 1.0f / 3.0f;
  for (uint32_t it = 0; it < num_tri; ++it) {
    float cog[3] = {0.0f, 0.0f, 0.0f};
    for (int in = 0; in < 3; ++in) {
      const float* p = vtx2xyz + (size_t)tri2vtx[(size_t)it * 3 + in] * 3;
      for (int d = 0; d < 3; ++d) cog[d] += p[d];
    }
    for (int d = 0; d < 3; ++d) tri2cntr[(size_t)it * 3 + d] = cog[d] * ratio;
  }
}

/* aabb3::set_as_cube / add_point (del-geo-core, absent): box [p-eps, p+eps],
 * widened by strict comparisons, so among equal values the first one stays. */
static void aabb_set_as_cube(float a[6], const float p[3], float eps) {
  for (int d = 0; d < 3; ++d) {
    a[d] = p[d] - eps;
    a[d + 3] = p[d] + eps;
  }
}
static void aabb_add_point(float a[6], const float p[3], float eps) {
  for (int d = 0; d < 3; ++d) {
    const float lo = p[d] - eps, hi = p[d] + eps;
    if (lo < a[d]) a[d] = lo;
    if (hi > a[d + 3]) a[d + 3] = hi;
  }
}
/* aabb3::from_two_aabbs (del-geo-core, absent): component-wise union; the
 * first box's value stays on ties. */
static void aabb_from_two(float o[6], const float a[6], const float b[6]) {
  for (int d = 0; d < 3; ++d) {
    o[d] = (b[d] < a[d]) ? b[d] : a[d];
    o[d + 3] = (b[d + 3] > a[d + 3]) ? b[d + 3] : a[d + 3];
  }
}

/* vtx2xyz.rs:19-37 (set_as_cube from the first point, then add_point over
 * every point including the first), eps = 0 */
void or_aabb3(uint32_t num_pnt, const float* pnt2xyz, float aabb[6]) {
  aabb_set_as_cube(aabb, pnt2xyz, 0.0f);
  for (uint32_t i = 0; i < num_pnt; ++i) aabb_add_point(aabb, pnt2xyz + (size_t)i * 3, 0.0f);
}

/* Mat44/torch.py:120-140: s = 1/max extent, translation = -center*s + 0.5,
 * center = (min+max)*0.5.  Column-major 4x4. */
void or_fit_into_unit_preserve_asp(const float aabb[6], float m[16]) {
  float ext = aabb[3] - aabb[0];
  const float ey = aabb[4] - aabb[1], ez = aabb[5] - aabb[2];
  if (ey > ext) ext = ey;
  if (ez > ext) ext = ez;
  const float s = 1.0f / ext;
  memset(m, 0, sizeof(float) * 16);
  m[0] = s;
  m[5] = s;
  m[10] = s;
  m[15] = 1.0f;
  for (int d = 0; d < 3; ++d) {
    const float c = (aabb[d] + aabb[d + 3]) * 0.5f;
    m[12 + d] = -c * s + 0.5f;
  }
}

/* column-major: out_i = (m[i]x + m[4+i]y + m[8+i]z + m[12+i]) / w, summed
 * left to right. */
void or_transform_homogeneous(const float m[16], const float p[3], float out[3]) {
  const float w = m[3] * p[0] + m[7] * p[1] + m[11] * p[2] + m[15];
  for (int i = 0; i < 3; ++i) out[i] = (m[i] * p[0] + m[4 + i] * p[1] + m[8 + i] * p[2] + m[12 + i]) / w;
}

static void transform_homogeneous2(const float m[9], const float p[2], float out[2]) {
  const float w = m[2] * p[0] + m[5] * p[1] + m[8];
  for (int i = 0; i < 2; ++i) out[i] = (m[i] * p[0] + m[3 + i] * p[1] + m[6 + i]) / w;
}

/* mortons.rs:171-212 */
void or_vtx2morton(uint32_t num_vtx, uint32_t num_dim, const float* vtx2co, const float* transform,
                   uint32_t* vtx2morton) {
  for (uint32_t i = 0; i < num_vtx; ++i) {
    if (num_dim == 3) {
      float q[3];
      or_transform_homogeneous(transform, vtx2co + (size_t)i * 3, q);
      vtx2morton[i] = or_morton_code3(q[0], q[1], q[2]);
    } else {
      float q[2];
      transform_homogeneous2(transform, vtx2co + (size_t)i * 2, q);
      vtx2morton[i] = or_morton_code2(q[0], q[1]);
    }
  }
}

/* -------------------------------------------------------- stable argsort */

/* bottom-up merge sort; the result ends in a */
static void merge_sort_u64(uint64_t* a, uint64_t* tmp, size_t n) {
  uint64_t* src = a;
  uint64_t* dst = tmp;
  for (size_t w = 1; w < n; w *= 2) {
    for (size_t lo = 0; lo < n; lo += 2 * w) {
      const size_t mid = lo + w < n ? lo + w : n, hi = lo + 2 * w < n ? lo + 2 * w : n;
      size_t i = lo, j = mid, k = lo;
      while (i < mid && j < hi) dst[k++] = (src[j] < src[i]) ? src[j++] : src[i++];
      while (i < mid) dst[k++] = src[i++];
      while (j < hi) dst[k++] = src[j++];
    }
    uint64_t* t = src;
    src = dst;
    dst = t;
  }
  if (src != a) memcpy(a, src, n * sizeof(uint64_t));
}

/* mortons.rs:139-146: iota, then a stable sort_by_key on the code, then the
 * gather.  Sorting (code << 32 | index) gives the same permutation. */
void or_argsort_stable(uint32_t n, const uint32_t* vtx2morton, uint32_t* idx2vtx, uint32_t* idx2morton) {
  uint64_t* a = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
  uint64_t* t = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
  for (uint32_t i = 0; i < n; ++i) a[i] = ((uint64_t)vtx2morton[i] << 32) | i;
  merge_sort_u64(a, t, n);
  for (uint32_t i = 0; i < n; ++i) {
    idx2vtx[i] = (uint32_t)(a[i] & 0xFFFFFFFFu);
    idx2morton[i] = (uint32_t)(a[i] >> 32);
  }
  free(a);
  free(t);
}

/* ------------------------------------------------------- radix tree */

static int clz32(uint32_t v) { return v == 0 ? 32 : __builtin_clz(v); }

/* mortons.rs:216-218 */
static int64_t delta(uint32_t i0, uint32_t i1, const uint32_t* c) { return clz32(c[i0] ^ c[i1]); }

/* mortons.rs:221-288 */
void or_range_of_binary_radix_tree_node(const uint32_t* c, uint32_t n, uint32_t idx1, uint32_t* r0, uint32_t* r1) {
  if (idx1 == 0) {
    *r0 = 0;
    *r1 = n - 1;
    return;
  }
  if (idx1 == n - 1) {
    *r0 = n - 1;
    *r1 = n - 1;
    return;
  }
  const uint32_t mc0 = c[idx1 - 1], mc1 = c[idx1], mc2 = c[idx1 + 1];
  if (mc0 == mc1 && mc1 == mc2) {
    uint32_t jdx = idx1 + 1;
    while (jdx < n - 1) {
      jdx += 1;
      if (c[jdx] != mc1) {
        *r0 = idx1;
        *r1 = jdx - 1;
        return;
      }
    }
    *r0 = idx1;
    *r1 = jdx;
    return;
  }
  int64_t d = delta(idx1, idx1 + 1, c) - delta(idx1, idx1 - 1, c);
  d = d > 0 ? 1 : -1;
  const int64_t delta_min = delta(idx1, (uint32_t)((int64_t)idx1 - d), c);
  int64_t lmax = 2;
  for (;;) {
    const int64_t jdx = (int64_t)idx1 + lmax * d;
    if (jdx < 0 || jdx >= (int64_t)n) break;
    if (delta(idx1, (uint32_t)jdx, c) <= delta_min) break;
    lmax *= 2;
  }
  int64_t l = 0;
  for (int64_t t = lmax / 2; t >= 1; t /= 2) {
    const int64_t jdx = (int64_t)idx1 + (l + t) * d;
    if (jdx >= 0 && jdx < (int64_t)n && delta(idx1, (uint32_t)jdx, c) > delta_min) l += t;
  }
  const uint32_t jdx = (uint32_t)((int64_t)idx1 + l * d);
  if (idx1 <= jdx) {
    *r0 = idx1;
    *r1 = jdx;
  } else {
    *r0 = jdx;
    *r1 = idx1;
  }
}

/* mortons.rs:290-325 */
uint32_t or_split_of_binary_radix_tree_node(const uint32_t* c, uint32_t start, uint32_t end) {
  if (start == end) return OR_UMAX;
  const uint32_t mc_start = c[start];
  const int nbitcommon0 = clz32(mc_start ^ c[end]);
  if (nbitcommon0 == 32) return start;
  uint32_t split = start;
  uint32_t step = end - start;
  while (step > 1) {
    step = (step + 1) / 2;
    const uint32_t cand = split + step;
    if (cand >= end) continue;
    if (clz32(mc_start ^ c[cand]) > nbitcommon0) split = cand;
  }
  return split;
}

/* bvhnodes_morton.rs:10-50.  For n == 1 the reference leaves node 0 as a
 * branch without children; here it becomes the single leaf [MAX, obj, MAX]. */
void or_update_bvhnodes(uint32_t n, const uint32_t* idx2vtx, const uint32_t* idx2morton, uint32_t* bvhnodes) {
  bvhnodes[0] = OR_UMAX;
  if (n == 1) {
    bvhnodes[1] = idx2vtx[0];
    bvhnodes[2] = OR_UMAX;
    return;
  }
  const uint32_t num_branch = n - 1;
  for (uint32_t ib = 0; ib < num_branch; ++ib) {
    uint32_t r0, r1;
    or_range_of_binary_radix_tree_node(idx2morton, n, ib, &r0, &r1);
    const uint32_t isplit = or_split_of_binary_radix_tree_node(idx2morton, r0, r1);
    if (r0 == isplit) {
      const uint32_t a = num_branch + isplit;
      bvhnodes[ib * 3 + 1] = a;
      bvhnodes[a * 3] = ib;
      bvhnodes[a * 3 + 1] = idx2vtx[isplit];
      bvhnodes[a * 3 + 2] = OR_UMAX;
    } else {
      bvhnodes[ib * 3 + 1] = isplit;
      bvhnodes[isplit * 3] = ib;
    }
    if (r1 == isplit + 1) {
      const uint32_t b = num_branch + isplit + 1;
      bvhnodes[ib * 3 + 2] = b;
      bvhnodes[b * 3] = ib;
      bvhnodes[b * 3 + 1] = idx2vtx[isplit + 1];
      bvhnodes[b * 3 + 2] = OR_UMAX;
    } else {
      bvhnodes[ib * 3 + 2] = isplit + 1;
      bvhnodes[(isplit + 1) * 3] = ib;
    }
  }
}

void or_bvhnodes_from_triangle_mesh(uint32_t num_tri, const uint32_t* tri2vtx, const float* vtx2xyz,
                                    uint32_t* bvhnodes, float* transform_out, uint32_t* tri2morton_out,
                                    uint32_t* idx2tri_out, uint32_t* idx2morton_out) {
  float* cntr = (float*)malloc(sizeof(float) * 3 * num_tri);
  uint32_t* tri2morton = (uint32_t*)malloc(sizeof(uint32_t) * num_tri);
  uint32_t* idx2tri = (uint32_t*)malloc(sizeof(uint32_t) * num_tri);
  uint32_t* idx2morton = (uint32_t*)malloc(sizeof(uint32_t) * num_tri);
  float aabb[6], m[16];
  or_tri2cntr(num_tri, tri2vtx, vtx2xyz, cntr);
  or_aabb3(num_tri, cntr, aabb);
  or_fit_into_unit_preserve_asp(aabb, m);
  or_vtx2morton(num_tri, 3, cntr, m, tri2morton);
  or_argsort_stable(num_tri, tri2morton, idx2tri, idx2morton);
  or_update_bvhnodes(num_tri, idx2tri, idx2morton, bvhnodes);
  if (transform_out) memcpy(transform_out, m, sizeof(m));
  if (tri2morton_out) memcpy(tri2morton_out, tri2morton, sizeof(uint32_t) * num_tri);
  if (idx2tri_out) memcpy(idx2tri_out, idx2tri, sizeof(uint32_t) * num_tri);
  if (idx2morton_out) memcpy(idx2morton_out, idx2morton, sizeof(uint32_t) * num_tri);
  free(cntr);
  free(tri2morton);
  free(idx2tri);
  free(idx2morton);
}

/* -------------------------------------------------------------- refit */

/* bvhnode2aabb3.rs:68-142 (leaf: aabb3_indexed with eps 0, vtx2xyz.rs:39-61;
 * optional CCD union with vtx2xyz1; branch: from_two_aabbs(child0, child1)). */
void or_update_aabb_uniform_mesh(float* bvhnode2aabb, uint32_t i_bvhnode, const uint32_t* bvhnodes,
                                 const uint32_t* tri2vtx, const float* vtx2xyz0, const float* vtx2xyz1) {
  float* out = bvhnode2aabb + (size_t)i_bvhnode * 6;
  if (bvhnodes[i_bvhnode * 3 + 2] == OR_UMAX) {
    const uint32_t it = bvhnodes[i_bvhnode * 3 + 1];
    const uint32_t* tv = tri2vtx + (size_t)it * 3;
    float a0[6];
    aabb_set_as_cube(a0, vtx2xyz0 + (size_t)tv[0] * 3, 0.0f);
    aabb_add_point(a0, vtx2xyz0 + (size_t)tv[1] * 3, 0.0f);
    aabb_add_point(a0, vtx2xyz0 + (size_t)tv[2] * 3, 0.0f);
    if (vtx2xyz1) {
      float a1[6];
      aabb_set_as_cube(a1, vtx2xyz1 + (size_t)tv[0] * 3, 0.0f);
      aabb_add_point(a1, vtx2xyz1 + (size_t)tv[1] * 3, 0.0f);
      aabb_add_point(a1, vtx2xyz1 + (size_t)tv[2] * 3, 0.0f);
      aabb_from_two(out, a0, a1);
    } else {
      memcpy(out, a0, sizeof(a0));
    }
    return;
  }
  const uint32_t c0 = bvhnodes[i_bvhnode * 3 + 1], c1 = bvhnodes[i_bvhnode * 3 + 2];
  or_update_aabb_uniform_mesh(bvhnode2aabb, c0, bvhnodes, tri2vtx, vtx2xyz0, vtx2xyz1);
  or_update_aabb_uniform_mesh(bvhnode2aabb, c1, bvhnodes, tri2vtx, vtx2xyz0, vtx2xyz1);
  float tmp[6];
  aabb_from_two(tmp, bvhnode2aabb + (size_t)c0 * 6, bvhnode2aabb + (size_t)c1 * 6);
  memcpy(out, tmp, sizeof(tmp));
}

/* ---------------------------------------------------------- ray casting */

/* ray_for_pixel.h:3-19 */
void or_ray_for_pixel(uint32_t i_pix, uint32_t img_w, uint32_t img_h, const float t_ndc2world[16], float org[3],
                      float dir[3]) {
  const uint32_t ih = i_pix / img_w;
  const uint32_t iw = i_pix - ih * img_w;
  const float x0 = 2.0f * ((float)iw + 0.5f) / (float)img_w - 1.0f;
  const float y0 = 1.0f - 2.0f * ((float)ih + 0.5f) / (float)img_h;
  const float a[3] = {x0, y0, 1.0f}, b[3] = {x0, y0, -1.0f};
  float q0[3], q1[3];
  or_transform_homogeneous(t_ndc2world, a, q0);
  or_transform_homogeneous(t_ndc2world, b, q1);
  for (int d = 0; d < 3; ++d) {
    org[d] = q0[d];
    dir[d] = q1[d] - q0[d];
  }
}

static float dot3(const float a[3], const float b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static void cross3(float o[3], const float a[3], const float b[3]) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

/* Moller & Trumbore, "Fast, Minimum Storage Ray/Triangle Intersection"
 * (1997), without back-face culling: det == 0 is a miss, edges are
 * inclusive, t >= 0 is a hit.  All comparisons reject NaN. */
int or_tri3_ray(const float p0[3], const float p1[3], const float p2[3], const float org[3], const float dir[3],
                float* t, float bc[3]) {
  float e1[3], e2[3], tv[3], pv[3], qv[3];
  for (int d = 0; d < 3; ++d) {
    e1[d] = p1[d] - p0[d];
    e2[d] = p2[d] - p0[d];
    tv[d] = org[d] - p0[d];
  }
  cross3(pv, dir, e2);
  const float det = dot3(e1, pv);
  if (det == 0.0f) return 0;
  const float inv_det = 1.0f / det;
  const float u = dot3(tv, pv) * inv_det;
  if (!(u >= 0.0f && u <= 1.0f)) return 0;
  cross3(qv, tv, e1);
  const float v = dot3(dir, qv) * inv_det;
  if (!(v >= 0.0f && u + v <= 1.0f)) return 0;
  const float tt = dot3(e2, qv) * inv_det;
  if (!(tt >= 0.0f)) return 0;
  *t = tt;
  if (bc) {
    bc[0] = 1.0f - u - v;
    bc[1] = u;
    bc[2] = v;
  }
  return 1;
}

int or_tri3_ray_f64(const float p0[3], const float p1[3], const float p2[3], const float org[3], const float dir[3],
                    double* t) {
  double e1[3], e2[3], tv[3], pv[3], qv[3], dd[3];
  for (int d = 0; d < 3; ++d) {
    e1[d] = (double)p1[d] - (double)p0[d];
    e2[d] = (double)p2[d] - (double)p0[d];
    tv[d] = (double)org[d] - (double)p0[d];
    dd[d] = (double)dir[d];
  }
  pv[0] = dd[1] * e2[2] - dd[2] * e2[1];
  pv[1] = dd[2] * e2[0] - dd[0] * e2[2];
  pv[2] = dd[0] * e2[1] - dd[1] * e2[0];
  const double det = e1[0] * pv[0] + e1[1] * pv[1] + e1[2] * pv[2];
  if (det == 0.0) return 0;
  const double inv_det = 1.0 / det;
  qv[0] = tv[1] * e1[2] - tv[2] * e1[1];
  qv[1] = tv[2] * e1[0] - tv[0] * e1[2];
  qv[2] = tv[0] * e1[1] - tv[1] * e1[0];
  *t = (e2[0] * qv[0] + e2[1] * qv[1] + e2[2] * qv[2]) * inv_det;
  return 1;
}

/* Slab test (Kay & Kajiya 1986; Williams et al., "An Efficient and Robust
 * Ray-Box Intersection Algorithm", 2005) with precomputed 1/dir, the per-axis
 * entry / exit and their running max / min taken with IEEE 754 minNum /
 * maxNum (fminf / fmaxf: a NaN operand yields the other one).  An axis with
 * dir == 0 is a hit iff the origin lies inside the slab.  Returns 1 and
 * (t_enter, t_exit) iff t_enter <= t_exit and t_exit >= 0.  (The sign of a
 * zero result is unspecified; no decision depends on it.) */
int or_aabb3_ray(const float aabb[6], const float org[3], const float inv_dir[3], const float dir[3], float* t_enter,
                 float* t_exit) {
  float tmin = -INFINITY, tmax = INFINITY;
  for (int d = 0; d < 3; ++d) {
    if (dir[d] != 0.0f) {
      const float t0 = (aabb[d] - org[d]) * inv_dir[d];
      const float t1 = (aabb[d + 3] - org[d]) * inv_dir[d];
      tmin = fmaxf(tmin, fminf(t0, t1));
      tmax = fminf(tmax, fmaxf(t0, t1));
    } else if (org[d] < aabb[d] || org[d] > aabb[d + 3]) {
      return 0;
    }
  }
  if (!(tmin <= tmax) || tmax < 0.0f) return 0;
  *t_enter = tmin;
  *t_exit = tmax;
  return 1;
}

typedef struct {
  const uint32_t* tri2vtx;
  const float* vtx2xyz;
  const uint32_t* bvhnodes;
  const float* aabb;
  float org[3], dir[3], inv[3];
  uint64_t* n_branch; /* optional work counters (or_pix2tri_work); NULL when not counting */
  uint64_t* n_leaf;
  uint64_t* n_depth; /* optional: branches entered per depth (the root is depth 0), last bin = deeper */
  uint32_t depth, max_depth;
} RayCtx;

static void ray_ctx_init(RayCtx* c, const float org[3], const float dir[3]) {
  for (int d = 0; d < 3; ++d) {
    c->org[d] = org[d];
    c->dir[d] = dir[d];
    c->inv[d] = 1.0f / dir[d];
  }
}

static int slab(const RayCtx* c, uint32_t node, float* te, float* tx) {
  return or_aabb3_ray(c->aabb + (size_t)node * 6, c->org, c->inv, c->dir, te, tx);
}

/* Rust's lexicographic `<` on (f32, f32) tuples. */
static int tuple_lt(float a0, float a1, float b0, float b1) { return (a0 == b0) ? (a1 < b1) : (a0 < b0); }

static int tri_hit(const RayCtx* c, uint32_t it, float* t) {
  const uint32_t* tv = c->tri2vtx + (size_t)it * 3;
  return or_tri3_ray(c->vtx2xyz + (size_t)tv[0] * 3, c->vtx2xyz + (size_t)tv[1] * 3, c->vtx2xyz + (size_t)tv[2] * 3,
                     c->org, c->dir, t, NULL);
}

/* search_bvh3.rs:103-221 */
static int first_hit(const RayCtx* c, uint32_t node, float dis, float* t_out, uint32_t* tri_out) {
  float te, tx;
  if (!slab(c, node, &te, &tx)) return 0;
  const uint32_t* bn = c->bvhnodes;
  if (bn[node * 3 + 2] == OR_UMAX) {
    const uint32_t it = bn[node * 3 + 1];
    float t;
    if (c->n_leaf) ++*c->n_leaf;
    if (!tri_hit(c, it, &t)) return 0;
    if (!(t < dis)) return 0;
    *t_out = t;
    *tri_out = it;
    return 1;
  }
  const uint32_t l = bn[node * 3 + 1], r = bn[node * 3 + 2];
  if (c->n_branch) ++*c->n_branch;
  if (c->n_depth) ++c->n_depth[c->depth < c->max_depth ? c->depth : c->max_depth - 1];
  float tl0 = 0, tl1 = 0, tr0 = 0, tr1 = 0;
  const int hl = slab(c, l, &tl0, &tl1), hr = slab(c, r, &tr0, &tr1);
  int near_is_left;
  if (hl && hr) near_is_left = tuple_lt(tl0, tl1, tr0, tr1);
  else if (!hl && !hr) return 0;
  else near_is_left = hl;
  const uint32_t nn = near_is_left ? l : r, nf = near_is_left ? r : l;
  float tn = 0, tf = 0;
  uint32_t in = 0, iff = 0;
  ((RayCtx*)c)->depth++;
  const int hn = first_hit(c, nn, dis, &tn, &in);
  ((RayCtx*)c)->depth--;
  if (hn) {
    float f0, f1;
    if (slab(c, nf, &f0, &f1)) {
      if (f0 > tn) {
        *t_out = tn;
        *tri_out = in;
        return 1;
      }
    } else {
      *t_out = tn;
      *tri_out = in;
      return 1;
    }
  }
  ((RayCtx*)c)->depth++;
  const int hf = first_hit(c, nf, dis, &tf, &iff);
  ((RayCtx*)c)->depth--;
  if (hn && hf) {
    if (tn < tf) {
      *t_out = tn;
      *tri_out = in;
    } else {
      *t_out = tf;
      *tri_out = iff;
    }
    return 1;
  }
  if (hn) {
    *t_out = tn;
    *tri_out = in;
    return 1;
  }
  if (hf) {
    *t_out = tf;
    *tri_out = iff;
    return 1;
  }
  return 0;
}

int or_first_intersection_ray(const float org[3], const float dir[3], const uint32_t* tri2vtx, const float* vtx2xyz,
                              const uint32_t* bvhnodes, const float* bvhnode2aabb, uint32_t i_bvhnode, float dis,
                              float* t_out, uint32_t* tri_out) {
  RayCtx c = {tri2vtx, vtx2xyz, bvhnodes, bvhnode2aabb, {0}, {0}, {0}, NULL, NULL};
  ray_ctx_init(&c, org, dir);
  return first_hit(&c, i_bvhnode, dis, t_out, tri_out);
}

static void all_hits(const RayCtx* c, uint32_t node, float* ht, uint32_t* hi, uint32_t cap, uint32_t* cnt) {
  float te, tx;
  if (!slab(c, node, &te, &tx)) return;
  const uint32_t* bn = c->bvhnodes;
  if (bn[node * 3 + 2] == OR_UMAX) {
    float t;
    const uint32_t it = bn[node * 3 + 1];
    if (!tri_hit(c, it, &t)) return;
    if (*cnt < cap) {
      ht[*cnt] = t;
      hi[*cnt] = it;
    }
    *cnt += 1;
    return;
  }
  all_hits(c, bn[node * 3 + 1], ht, hi, cap, cnt);
  all_hits(c, bn[node * 3 + 2], ht, hi, cap, cnt);
}

/* search_bvh3.rs:12-53 */
uint32_t or_intersections_ray(const float org[3], const float dir[3], const uint32_t* tri2vtx, const float* vtx2xyz,
                              const uint32_t* bvhnodes, const float* bvhnode2aabb, float* hit_t, uint32_t* hit_tri,
                              uint32_t cap) {
  RayCtx c = {tri2vtx, vtx2xyz, bvhnodes, bvhnode2aabb, {0}, {0}, {0}, NULL, NULL};
  ray_ctx_init(&c, org, dir);
  uint32_t cnt = 0;
  all_hits(&c, 0, hit_t, hit_tri, cap, &cnt);
  return cnt;
}

/* ------------------------------------------------ multi-threaded drivers */

typedef struct {
  uint32_t num;
  int mode; /* 0: pixels, 1: ray arrays */
  uint32_t img_w, img_h;
  const float* t_ndc2world;
  const float* ray_org;
  const float* ray_dir;
  const uint32_t* tri2vtx;
  const float* vtx2xyz;
  const uint32_t* bvhnodes;
  const float* aabb;
  uint32_t* out_tri;
  float* out_t;
  uint32_t next; /* work counter, chunks of 64 */
} CastJob;

static void* cast_worker(void* arg) {
  CastJob* job = (CastJob*)arg;
  for (;;) {
    const uint32_t start = __atomic_fetch_add(&job->next, 64u, __ATOMIC_RELAXED);
    if (start >= job->num) break;
    const uint32_t end = start + 64 < job->num ? start + 64 : job->num;
    for (uint32_t i = start; i < end; ++i) {
      float org[3], dir[3];
      if (job->mode == 0) {
        or_ray_for_pixel(i, job->img_w, job->img_h, job->t_ndc2world, org, dir);
      } else {
        for (int d = 0; d < 3; ++d) {
          org[d] = job->ray_org[(size_t)i * 3 + d];
          dir[d] = job->ray_dir[(size_t)i * 3 + d];
        }
      }
      float t = INFINITY;
      uint32_t it = OR_UMAX;
      if (!or_first_intersection_ray(org, dir, job->tri2vtx, job->vtx2xyz, job->bvhnodes, job->aabb, 0, INFINITY, &t,
                                     &it)) {
        t = INFINITY;
        it = OR_UMAX;
      }
      job->out_tri[i] = it;
      if (job->out_t) job->out_t[i] = t;
    }
  }
  return NULL;
}

static void run_cast_job(CastJob* job, int num_threads) {
  if (num_threads < 1) num_threads = 1;
  if (num_threads == 1) {
    cast_worker(job);
    return;
  }
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * num_threads);
  pthread_attr_t attr;
  pthread_attr_init(&attr);
  pthread_attr_setstacksize(&attr, (size_t)64 << 20); /* deep trees recurse deeply */
  for (int i = 0; i < num_threads; ++i) pthread_create(&th[i], &attr, cast_worker, job);
  for (int i = 0; i < num_threads; ++i) pthread_join(th[i], NULL);
  pthread_attr_destroy(&attr);
  free(th);
}

/* pix2tri.rs:3-48 */
void or_pix2tri_by_raycast(uint32_t img_w, uint32_t img_h, const float t_ndc2world[16], const uint32_t* tri2vtx,
                           const float* vtx2xyz, const uint32_t* bvhnodes, const float* bvhnode2aabb,
                           uint32_t* pix2tri, float* pix2t, int num_threads) {
  CastJob job = {img_w * img_h, 0, img_w, img_h, t_ndc2world, NULL, NULL, tri2vtx, vtx2xyz,
                 bvhnodes, bvhnode2aabb, pix2tri, pix2t, 0};
  run_cast_job(&job, num_threads);
}

void or_cast_rays(uint32_t num_ray, const float* ray_org, const float* ray_dir, const uint32_t* tri2vtx,
                  const float* vtx2xyz, const uint32_t* bvhnodes, const float* bvhnode2aabb, uint32_t* hit_tri,
                  float* hit_t, int num_threads) {
  CastJob job = {num_ray, 1, 0, 0, NULL, ray_org, ray_dir, tri2vtx, vtx2xyz, bvhnodes, bvhnode2aabb, hit_tri, hit_t, 0};
  run_cast_job(&job, num_threads);
}

/* The work of first_hit over a pixel grid, one thread: out[0] rays, out[1]
 * branches entered (each tests its two children's boxes), out[2] triangles
 * tested (leaves whose box the ray enters).  The GPU traversal makes the same
 * decisions, so these are its node visits and triangle tests too. */
void or_pix2tri_work(uint32_t img_w, uint32_t img_h, const float t_ndc2world[16], const uint32_t* tri2vtx,
                     const float* vtx2xyz, const uint32_t* bvhnodes, const float* bvhnode2aabb, uint64_t out[3]) {
  or_pix2tri_work_depth(img_w, img_h, t_ndc2world, tri2vtx, vtx2xyz, bvhnodes, bvhnode2aabb, out, NULL, 0);
}

/* or_pix2tri_work, with the branches entered also counted per depth into
 * by_depth[0 .. max_depth-1] (the last bin takes every deeper entry). */
void or_pix2tri_work_depth(uint32_t img_w, uint32_t img_h, const float t_ndc2world[16], const uint32_t* tri2vtx,
                           const float* vtx2xyz, const uint32_t* bvhnodes, const float* bvhnode2aabb, uint64_t out[3],
                           uint64_t* by_depth, uint32_t max_depth) {
  uint64_t n_branch = 0, n_leaf = 0;
  if (by_depth)
    for (uint32_t k = 0; k < max_depth; ++k) by_depth[k] = 0;
  const uint32_t num = img_w * img_h;
  for (uint32_t i = 0; i < num; ++i) {
    float org[3], dir[3], t;
    uint32_t it;
    or_ray_for_pixel(i, img_w, img_h, t_ndc2world, org, dir);
    RayCtx c = {tri2vtx, vtx2xyz, bvhnodes, bvhnode2aabb, {0}, {0}, {0}, &n_branch, &n_leaf,
                by_depth && max_depth ? by_depth : NULL, 0, max_depth};
    ray_ctx_init(&c, org, dir);
    first_hit(&c, 0, INFINITY, &t, &it);
  }
  out[0] = num;
  out[1] = n_branch;
  out[2] = n_leaf;
}

/* ------------------------------------------------------------ checkers */

/* bvhnodes.rs:3-36 (iterative; a malformed tree fails instead of looping) */
int or_check_bvh_topology(const uint32_t* bvhnodes, uint32_t num_leaf) {
  const uint32_t num_node = 2 * num_leaf - 1;
  uint32_t* cnt = (uint32_t*)calloc(num_leaf, sizeof(uint32_t));
  uint32_t* stack = (uint32_t*)malloc(sizeof(uint32_t) * (num_node + 1));
  int ok = 1;
  uint32_t sp = 0, visits = 0;
  stack[sp++] = 0;
  while (sp > 0 && ok) {
    const uint32_t n = stack[--sp];
    if (n >= num_node || ++visits > num_node) {
      ok = 0;
      break;
    }
    if (bvhnodes[n * 3 + 2] == OR_UMAX) {
      const uint32_t v = bvhnodes[n * 3 + 1];
      if (v >= num_leaf) ok = 0;
      else cnt[v] += 1;
      continue;
    }
    stack[sp++] = bvhnodes[n * 3 + 2];
    stack[sp++] = bvhnodes[n * 3 + 1];
  }
  for (uint32_t i = 0; ok && i < num_leaf; ++i)
    if (cnt[i] != 1) ok = 0;
  for (uint32_t i = 0; ok && i < num_leaf; ++i)
    if (bvhnodes[(num_leaf - 1 + i) * 3 + 2] != OR_UMAX) ok = 0;
  free(cnt);
  free(stack);
  return ok;
}

/* mortons.rs:330-352 */
int or_check_morton_code_range_split(const uint32_t* c, uint32_t n) {
  for (uint32_t i = 0; i + 1 < n; ++i)
    if (c[i] > c[i + 1]) return 0;
  for (uint32_t ini = 0; ini + 1 < n; ++ini) {
    uint32_t r0, r1, a0, a1, b0, b1;
    or_range_of_binary_radix_tree_node(c, n, ini, &r0, &r1);
    const uint32_t isplit = or_split_of_binary_radix_tree_node(c, r0, r1);
    or_range_of_binary_radix_tree_node(c, n, isplit, &a0, &a1);
    or_range_of_binary_radix_tree_node(c, n, isplit + 1, &b0, &b1);
    if (r0 != a0 || r1 != b1) return 0;
    const uint32_t last1 = (isplit == r0) ? isplit : a1;
    const uint32_t first1 = (isplit + 1 == r1) ? isplit + 1 : b0;
    if (last1 + 1 != first1) return 0;
  }
  return 1;
}

uint32_t or_tree_height(const uint32_t* bvhnodes, uint32_t num_leaf) {
  const uint32_t num_node = 2 * num_leaf - 1;
  uint32_t* stack = (uint32_t*)malloc(sizeof(uint32_t) * 2 * (num_node + 1));
  uint32_t sp = 0, best = 0, visits = 0;
  stack[sp++] = 0;
  stack[sp++] = 1;
  while (sp > 0) {
    const uint32_t depth = stack[--sp];
    const uint32_t n = stack[--sp];
    if (n >= num_node || ++visits > num_node) break;
    if (depth > best) best = depth;
    if (bvhnodes[n * 3 + 2] == OR_UMAX) continue;
    stack[sp++] = bvhnodes[n * 3 + 1];
    stack[sp++] = depth + 1;
    stack[sp++] = bvhnodes[n * 3 + 2];
    stack[sp++] = depth + 1;
  }
  free(stack);
  return best;
}

/* ------------------------------------------------------------------------
 * Consumers of a pix2tri image: depth and attribute interpolation, forward
 * and backward.  pix2depth.rs:107-146 / pix2depth.cu:12-97 and
 * pix2tri.rs:176-304 / pix2tri.cu:79-183.  The formulas of the absent
 * del-geo-core crate are restated (parity unpinned against it):
 * Gauss-Jordan inverse with partial pivoting; Moller-Trumbore on the line
 * through the pixel ray; the backward of (t, u, v) by implicit
 * differentiation of o + t d = p0 + u e1 + v e2 with A = [-d | e1 | e2] and
 * lambda = A^-T g: dL/dp0 = -(1-u-v) lambda, dL/dp1 = -u lambda,
 * dL/dp2 = -v lambda; the Jacobian of the homogeneous transform
 * (M_ij w - v_i M_3j) / w^2.  The backward passes add sequentially in pixel
 * order, as the CPU reference does. */

int or_mat4_inverse_pivot(const float m[16], float inv[16]) {
  float a[4][8];
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      a[r][c] = m[c * 4 + r];
      a[r][4 + c] = (r == c) ? 1.0f : 0.0f;
    }
  for (int col = 0; col < 4; ++col) {
    int piv = col;
    float best = fabsf(a[col][col]);
    for (int r = col + 1; r < 4; ++r)
      if (fabsf(a[r][col]) > best) {
        best = fabsf(a[r][col]);
        piv = r;
      }
    if (best == 0.0f) {
      for (int k = 0; k < 16; ++k) inv[k] = NAN;
      return 0;
    }
    if (piv != col)
      for (int c = 0; c < 8; ++c) {
        const float tmp = a[col][c];
        a[col][c] = a[piv][c];
        a[piv][c] = tmp;
      }
    const float d = a[col][col];
    for (int c = 0; c < 8; ++c) a[col][c] = a[col][c] / d;
    for (int r = 0; r < 4; ++r) {
      if (r == col) continue;
      const float f = a[r][col];
      for (int c = 0; c < 8; ++c) a[r][c] = a[r][c] - f * a[col][c];
    }
  }
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) inv[c * 4 + r] = a[r][4 + c];
  return 1;
}

/* Moller-Trumbore without the inside / t >= 0 tests; 0 only for det == 0. */
static int tri3_line(const float p0[3], const float p1[3], const float p2[3], const float org[3], const float dir[3],
                     float* t, float* u, float* v) {
  float e1[3], e2[3], tv[3], pv[3], qv[3];
  for (int d = 0; d < 3; ++d) {
    e1[d] = p1[d] - p0[d];
    e2[d] = p2[d] - p0[d];
    tv[d] = org[d] - p0[d];
  }
  cross3(pv, dir, e2);
  const float det = dot3(e1, pv);
  if (det == 0.0f) return 0;
  const float inv_det = 1.0f / det;
  *u = dot3(tv, pv) * inv_det;
  cross3(qv, tv, e1);
  *v = dot3(dir, qv) * inv_det;
  *t = dot3(e2, qv) * inv_det;
  return 1;
}

static void tri3_line_bwd(const float p0[3], const float p1[3], const float p2[3], const float dir[3], float u, float v,
                          float gt, float gu, float gv, float d0[3], float d1[3], float d2[3]) {
  float c0[3], c1[3], c2[3], x12[3], x20[3], x01[3];
  for (int k = 0; k < 3; ++k) {
    c0[k] = -dir[k];
    c1[k] = p1[k] - p0[k];
    c2[k] = p2[k] - p0[k];
  }
  cross3(x12, c1, c2);
  cross3(x20, c2, c0);
  cross3(x01, c0, c1);
  const float det = dot3(c0, x12);
  const float inv = 1.0f / det;
  const float w0 = (1.0f - u) - v;
  for (int k = 0; k < 3; ++k) {
    const float lam = (gt * x12[k] + gu * x20[k] + gv * x01[k]) * inv;
    d0[k] = lam * -w0;
    d1[k] = lam * -u;
    d2[k] = lam * -v;
  }
}

static int tri_of_pixel(uint32_t it, uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                        const float* vtx2xyz, uint32_t iv[3], const float* p[3]) {
  if (it >= num_tri) return 0;
  for (int k = 0; k < 3; ++k) {
    iv[k] = tri2vtx[(size_t)it * 3 + k];
    if (iv[k] >= num_vtx) return 0;
    p[k] = vtx2xyz + (size_t)iv[k] * 3;
  }
  return 1;
}

int or_pix2depth(uint32_t img_w, uint32_t img_h, float* pix2depth, const uint32_t* pix2tri, uint32_t num_tri,
                 const uint32_t* tri2vtx, uint32_t num_vtx, const float* vtx2xyz, const float ndc2world[16]) {
  float w2n[16];
  const int ok = or_mat4_inverse_pivot(ndc2world, w2n);
  for (uint32_t i = 0; i < img_w * img_h; ++i) {
    const uint32_t it = pix2tri[i];
    if (it == OR_UMAX) {
      pix2depth[i] = 0.0f;
      continue;
    }
    uint32_t iv[3];
    const float* p[3];
    if (!tri_of_pixel(it, num_tri, tri2vtx, num_vtx, vtx2xyz, iv, p)) continue;
    float o[3], d[3], t, bc[3];
    or_ray_for_pixel(i, img_w, img_h, ndc2world, o, d);
    if (!or_tri3_ray(p[0], p[1], p[2], o, d, &t, bc)) continue;
    const float q[3] = {t * d[0] + o[0], t * d[1] + o[1], t * d[2] + o[2]};
    float ndc[3];
    or_transform_homogeneous(w2n, q, ndc);
    pix2depth[i] = (ndc[2] + 1.0f) * 0.5f;
  }
  return ok;
}

int or_pix2depth_bwd(uint32_t img_w, uint32_t img_h, float* dldw_vtx2xyz, const uint32_t* pix2tri, uint32_t num_tri,
                     const uint32_t* tri2vtx, uint32_t num_vtx, const float* vtx2xyz, const float* dldw_pix2depth,
                     const float ndc2world[16]) {
  float M[16];
  const int ok = or_mat4_inverse_pivot(ndc2world, M);
  for (uint32_t i = 0; i < img_w * img_h; ++i) {
    const uint32_t it = pix2tri[i];
    if (it == OR_UMAX) continue;
    uint32_t iv[3];
    const float* p[3];
    if (!tri_of_pixel(it, num_tri, tri2vtx, num_vtx, vtx2xyz, iv, p)) continue;
    float o[3], d[3], t, u, v;
    or_ray_for_pixel(i, img_w, img_h, ndc2world, o, d);
    if (!tri3_line(p[0], p[1], p[2], o, d, &t, &u, &v)) continue;
    const float q[3] = {t * d[0] + o[0], t * d[1] + o[1], t * d[2] + o[2]};
    float vv[4];
    for (int r = 0; r < 4; ++r) vv[r] = M[r] * q[0] + M[4 + r] * q[1] + M[8 + r] * q[2] + M[12 + r];
    const float w = vv[3], ww = w * w;
    const float g_ndc[3] = {0.0f, 0.0f, 0.5f * dldw_pix2depth[i]};
    float gq[3];
    for (int j = 0; j < 3; ++j) {
      float s = 0.0f;
      for (int r = 0; r < 3; ++r) {
        const float jij = (M[j * 4 + r] * w - vv[r] * M[j * 4 + 3]) / ww;
        s = s + jij * g_ndc[r];
      }
      gq[j] = s;
    }
    const float gt = gq[0] * d[0] + gq[1] * d[1] + gq[2] * d[2];
    float g[3][3];
    tri3_line_bwd(p[0], p[1], p[2], d, u, v, gt, 0.0f, 0.0f, g[0], g[1], g[2]);
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 3; ++c) dldw_vtx2xyz[(size_t)iv[k] * 3 + c] += g[k][c];
  }
  return ok;
}

void or_interpolate(uint32_t img_w, uint32_t img_h, const uint32_t* pix2tri, uint32_t num_tri, const uint32_t* tri2vtx,
                    uint32_t num_vtx, const float* vtx2xyz, uint32_t num_vdim, const float* vtx2val,
                    const float ndc2world[16], float* pix2val) {
  for (uint32_t i = 0; i < img_w * img_h; ++i) {
    float* out = pix2val + (size_t)i * num_vdim;
    const uint32_t it = pix2tri[i];
    uint32_t iv[3];
    const float* p[3];
    float t = 0.f, u = 0.f, v = 0.f;
    int ok = it != OR_UMAX && tri_of_pixel(it, num_tri, tri2vtx, num_vtx, vtx2xyz, iv, p);
    if (ok) {
      float o[3], d[3];
      or_ray_for_pixel(i, img_w, img_h, ndc2world, o, d);
      ok = tri3_line(p[0], p[1], p[2], o, d, &t, &u, &v);
    }
    if (!ok) {
      for (uint32_t k = 0; k < num_vdim; ++k) out[k] = 0.0f;
      continue;
    }
    const float b0 = (1.0f - u) - v;
    for (uint32_t k = 0; k < num_vdim; ++k)
      out[k] = b0 * vtx2val[(size_t)iv[0] * num_vdim + k] + u * vtx2val[(size_t)iv[1] * num_vdim + k] +
               v * vtx2val[(size_t)iv[2] * num_vdim + k];
  }
}

void or_interpolate_bwd(uint32_t img_w, uint32_t img_h, const uint32_t* pix2tri, uint32_t num_tri,
                        const uint32_t* tri2vtx, uint32_t num_vtx, const float* vtx2xyz, uint32_t num_vdim,
                        const float* vtx2val, const float ndc2world[16], const float* dldw_pix2val,
                        float* dldw_vtx2xyz, float* dldw_vtx2val) {
  for (uint32_t i = 0; i < img_w * img_h; ++i) {
    const uint32_t it = pix2tri[i];
    if (it == OR_UMAX) continue;
    uint32_t iv[3];
    const float* p[3];
    if (!tri_of_pixel(it, num_tri, tri2vtx, num_vtx, vtx2xyz, iv, p)) continue;
    const float* g = dldw_pix2val + (size_t)i * num_vdim;
    float gb0 = 0.0f, gb1 = 0.0f, gb2 = 0.0f;
    for (uint32_t k = 0; k < num_vdim; ++k) {
      gb0 = gb0 + vtx2val[(size_t)iv[0] * num_vdim + k] * g[k];
      gb1 = gb1 + vtx2val[(size_t)iv[1] * num_vdim + k] * g[k];
      gb2 = gb2 + vtx2val[(size_t)iv[2] * num_vdim + k] * g[k];
    }
    gb1 = gb1 - gb0;
    gb2 = gb2 - gb0;
    float o[3], d[3], t, u, v;
    or_ray_for_pixel(i, img_w, img_h, ndc2world, o, d);
    if (!tri3_line(p[0], p[1], p[2], o, d, &t, &u, &v)) continue;
    float dp[3][3];
    tri3_line_bwd(p[0], p[1], p[2], d, u, v, 0.0f, gb1, gb2, dp[0], dp[1], dp[2]);
    for (int c = 0; c < 3; ++c)
      for (int k = 0; k < 3; ++k) dldw_vtx2xyz[(size_t)iv[k] * 3 + c] += dp[k][c];
    const float b[3] = {(1.0f - u) - v, u, v};
    for (uint32_t k = 0; k < num_vdim; ++k)
      for (int j = 0; j < 3; ++j) dldw_vtx2val[(size_t)iv[j] * num_vdim + k] += g[k] * b[j];
  }
}

/* ------------------------------------------------------------------------
 * Quad/oct-trees from the binary radix tree of sorted unique Morton codes:
 * quad_oct_tree.rs:2-63 (binary tree + depth, morton2center), 88-125
 * (bnode2onode, idx2bnode), 127-233 (the tree), 235-338 (check_octree),
 * 420-451 (aggregate). */

void or_qot_binary_radix_tree_and_depth(uint32_t num_idx, const uint32_t* idx2morton, uint32_t num_dim,
                                        uint32_t max_depth, uint32_t* bnodes, uint32_t* bnode2depth) {
  const uint32_t num_bnode = num_idx - 1;
  bnodes[0] = OR_UMAX;
  for (uint32_t ib = 0; ib < num_bnode; ++ib) {
    uint32_t r0, r1;
    or_range_of_binary_radix_tree_node(idx2morton, num_idx, ib, &r0, &r1);
    const uint32_t isplit = or_split_of_binary_radix_tree_node(idx2morton, r0, r1);
    if (r0 == isplit) {
      bnodes[ib * 3 + 1] = num_bnode + isplit;
    } else {
      bnodes[ib * 3 + 1] = isplit;
      bnodes[isplit * 3] = ib;
    }
    if (r1 == isplit + 1) {
      bnodes[ib * 3 + 2] = num_bnode + isplit + 1;
    } else {
      bnodes[ib * 3 + 2] = isplit + 1;
      bnodes[(isplit + 1) * 3] = ib;
    }
    const uint32_t delta = (uint32_t)clz32(idx2morton[isplit] ^ idx2morton[isplit + 1]);
    const uint32_t offset = 32u - num_dim * max_depth;
    bnode2depth[ib] = (delta - offset) / num_dim;
  }
}

void or_qot_bnode2onode_and_idx2bnode(uint32_t num_idx, const uint32_t* bnodes, const uint32_t* bnode2depth,
                                      uint32_t* bnode2onode, uint32_t* idx2bnode) {
  const uint32_t num_bnode = num_idx - 1;
  uint32_t* iso = (uint32_t*)calloc(num_bnode, sizeof(uint32_t));
  for (uint32_t ib = 0; ib < num_bnode; ++ib) {
    if (bnodes[ib * 3 + 1] >= num_bnode) idx2bnode[bnodes[ib * 3 + 1] - num_bnode] = ib;
    if (bnodes[ib * 3 + 2] >= num_bnode) idx2bnode[bnodes[ib * 3 + 2] - num_bnode] = ib;
    if (ib == 0) continue;
    const uint32_t parent = bnodes[ib * 3];
    if (bnode2depth[ib] != bnode2depth[parent]) iso[ib - 1] = 1;
  }
  bnode2onode[0] = 0;
  for (uint32_t ib = 1; ib < num_bnode; ++ib) bnode2onode[ib] = bnode2onode[ib - 1] + iso[ib - 1];
  free(iso);
}

static void qot_morton2center(uint32_t morton, uint32_t num_dim, uint32_t depth, uint32_t max_depth, float c[3]) {
  uint32_t key = morton >> ((max_depth - depth) * num_dim);
  for (uint32_t d = 0; d < num_dim; ++d) c[d] = 0.5f;
  for (uint32_t i = 0; i < depth; ++i)
    for (uint32_t d = 0; d < num_dim; ++d) {
      const uint32_t j = num_dim - d - 1;
      c[j] = (c[j] + (float)(key & 1u)) * 0.5f;
      key >>= 1;
    }
}

static void qot_parent(uint32_t cur, const uint32_t* bnodes, const uint32_t* b2o, const uint32_t* b2d, uint32_t* on,
                       uint32_t* depth) {
  for (;;) {
    if (cur == 0 || b2o[cur] != b2o[cur - 1]) {
      *on = b2o[cur];
      *depth = b2d[cur];
      return;
    }
    cur = bnodes[cur * 3];
  }
}

void or_qot_make_tree(uint32_t num_idx, const uint32_t* bnodes, const uint32_t* b2o, const uint32_t* b2d,
                      const uint32_t* idx2bnode, const uint32_t* idx2morton, uint32_t num_onode, uint32_t max_depth,
                      uint32_t num_dim, uint32_t* onodes, uint32_t* onode2depth, float* onode2center,
                      uint32_t* idx2onode, float* idx2center) {
  const uint32_t num_child = 1u << num_dim, nlink = num_child + 1;
  for (uint32_t i = 0; i < num_idx; ++i) {
    uint32_t op, dp;
    qot_parent(idx2bnode[i], bnodes, b2o, b2d, &op, &dp);
    const uint32_t key = idx2morton[i];
    const uint32_t ic = (key >> ((max_depth - 1 - dp) * num_dim)) & (num_child - 1);
    onodes[op * nlink + 1 + ic] = i + num_onode;
    idx2onode[i] = op;
    float c[3];
    qot_morton2center(key, num_dim, max_depth, max_depth, c);
    for (uint32_t d = 0; d < num_dim; ++d) idx2center[i * num_dim + d] = c[d];
    if (i + 1 >= num_idx) continue;
    const uint32_t ib = i;
    if (ib == 0) {
      for (uint32_t d = 0; d < num_dim; ++d) onode2center[d] = 0.5f;
      continue;
    }
    if (b2o[ib - 1] == b2o[ib]) continue;
    qot_parent(bnodes[ib * 3], bnodes, b2o, b2d, &op, &dp);
    const uint32_t morton = idx2morton[ib];
    const uint32_t icb = (morton >> ((max_depth - 1 - dp) * num_dim)) & (num_child - 1);
    const uint32_t on = b2o[ib];
    onodes[op * nlink + 1 + icb] = on;
    onodes[on * nlink] = op;
    const uint32_t depth = b2d[ib];
    qot_morton2center(morton, num_dim, depth, max_depth, c);
    for (uint32_t d = 0; d < num_dim; ++d) onode2center[on * num_dim + d] = c[d];
    onode2depth[on] = depth;
  }
}

void or_qot_aggregate(uint32_t num_idx, uint32_t num_vdim, const float* idx2val, const uint32_t* idx2onode,
                      uint32_t num_link, const uint32_t* onodes, uint32_t num_onode, float* onode2aggval) {
  for (uint32_t k = 0; k < num_onode * num_vdim; ++k) onode2aggval[k] = 0.0f;
  for (uint32_t idx = 0; idx < num_idx; ++idx) {
    uint32_t on = idx2onode[idx];
    while (on != OR_UMAX && on < num_onode) {
      for (uint32_t d = 0; d < num_vdim; ++d) onode2aggval[on * num_vdim + d] += idx2val[idx * num_vdim + d];
      on = onodes[on * num_link];
    }
  }
}

/* quad_oct_tree.rs:235-338: every leaf reached exactly once from the root,
 * children strictly deeper than their parent and inside its cell. */
static int qot_visit(uint32_t node, uint32_t nlink, uint32_t nchild, const uint32_t* onodes, uint32_t num_onode,
                     uint32_t* seen, uint32_t num_idx, uint32_t budget) {
  if (budget == 0) return 0;
  for (uint32_t k = 0; k < nchild; ++k) {
    const uint32_t ch = onodes[node * nlink + 1 + k];
    if (ch == OR_UMAX) continue;
    if (ch >= num_onode) {
      if (ch - num_onode >= num_idx) return 0;
      seen[ch - num_onode] += 1;
    } else if (!qot_visit(ch, nlink, nchild, onodes, num_onode, seen, num_idx, budget - 1)) {
      return 0;
    }
  }
  return 1;
}

int or_qot_check(uint32_t num_idx, uint32_t num_dim, const uint32_t* idx2onode, const float* idx2center,
                 const uint32_t* onodes, const uint32_t* onode2depth, const float* onode2center, uint32_t num_onode,
                 uint32_t max_depth) {
  const uint32_t nchild = 1u << num_dim, nlink = nchild + 1;
  uint32_t* seen = (uint32_t*)calloc(num_idx, sizeof(uint32_t));
  int ok = qot_visit(0, nlink, nchild, onodes, num_onode, seen, num_idx, 64);
  for (uint32_t i = 0; ok && i < num_idx; ++i) ok = seen[i] == 1;
  free(seen);
  for (uint32_t n = 0; ok && n < num_onode + num_idx; ++n) {
    const uint32_t depth = n < num_onode ? onode2depth[n] : max_depth;
    const float h = 0.5f / (float)(1u << depth);
    const float* c = n < num_onode ? onode2center + n * num_dim : idx2center + (n - num_onode) * num_dim;
    const uint32_t p = n < num_onode ? onodes[n * nlink] : idx2onode[n - num_onode];
    if (p == OR_UMAX) continue;
    if (p >= num_onode) return 0;
    const uint32_t dp = onode2depth[p];
    if (!(depth > dp)) return 0;
    const float hp = 0.5f / (float)(1u << dp);
    for (uint32_t d = 0; d < num_dim; ++d) {
      const float dd = fabsf(c[d] - onode2center[p * num_dim + d]);
      if (!(dd + h < hp * (1.0f + 1.0e-7f))) return 0;
    }
  }
  return ok;
}

/* ------------------------------------------------------------------------
 * Self-intersection through the BVH: trimesh3_intersection.rs:10-179
 * (pair logic, search_with_bvh_between_branches, _inside_branch).  The
 * del-geo-core segment formulas are restated (parity unpinned): tri/tri by
 * the two plane-crossing segments overlapped along n_a x n_b (reported when
 * of non-zero length; coplanar pairs are not); a shared vertex by
 * Moller-Trumbore of the opposite edges (0 <= t <= 1) against the other
 * triangle.  Three shared vertices: not reported (the reference panics). */

static void lerp_cross(const float vi[3], const float vj[3], float di, float dj, float out[3]) {
  const float s = di / (di - dj);
  for (int k = 0; k < 3; ++k) out[k] = vi[k] + (vj[k] - vi[k]) * s;
}

static int plane_segment(const float* v[3], const float d[3], float s0[3], float s1[3]) {
  float pts[4][3];
  int n = 0;
  for (int k = 0; k < 3; ++k)
    if (d[k] == 0.0f) {
      memcpy(pts[n], v[k], sizeof(float) * 3);
      ++n;
    }
  for (int k = 0; k < 3; ++k) {
    const int i = k, j = (k + 1) % 3;
    if ((d[i] > 0.0f && d[j] < 0.0f) || (d[i] < 0.0f && d[j] > 0.0f)) {
      lerp_cross(v[i], v[j], d[i], d[j], pts[n]);
      ++n;
    }
  }
  if (n < 2) return 0;
  memcpy(s0, pts[0], sizeof(float) * 3);
  memcpy(s1, pts[1], sizeof(float) * 3);
  return 1;
}

static void sub3v(float o[3], const float a[3], const float b[3]) {
  for (int k = 0; k < 3; ++k) o[k] = a[k] - b[k];
}

static int tri_tri_segment(const float* a[3], const float* b[3], float p0[3], float p1[3]) {
  float e1[3], e2[3], nb[3], na[3], da[3], dbv[3];
  sub3v(e1, b[1], b[0]);
  sub3v(e2, b[2], b[0]);
  cross3(nb, e1, e2);
  const float db = -dot3(nb, b[0]);
  for (int k = 0; k < 3; ++k) da[k] = dot3(nb, a[k]) + db;
  if ((da[0] > 0.0f && da[1] > 0.0f && da[2] > 0.0f) || (da[0] < 0.0f && da[1] < 0.0f && da[2] < 0.0f)) return 0;
  if (da[0] == 0.0f && da[1] == 0.0f && da[2] == 0.0f) return 0;
  sub3v(e1, a[1], a[0]);
  sub3v(e2, a[2], a[0]);
  cross3(na, e1, e2);
  const float dA = -dot3(na, a[0]);
  for (int k = 0; k < 3; ++k) dbv[k] = dot3(na, b[k]) + dA;
  if ((dbv[0] > 0.0f && dbv[1] > 0.0f && dbv[2] > 0.0f) || (dbv[0] < 0.0f && dbv[1] < 0.0f && dbv[2] < 0.0f))
    return 0;
  float sa0[3], sa1[3], sb0[3], sb1[3], D[3];
  if (!plane_segment(a, da, sa0, sa1) || !plane_segment(b, dbv, sb0, sb1)) return 0;
  cross3(D, na, nb);
  float ta0 = dot3(D, sa0), ta1 = dot3(D, sa1), tb0 = dot3(D, sb0), tb1 = dot3(D, sb1);
  if (ta1 < ta0) {
    float t[3];
    memcpy(t, sa0, sizeof t);
    memcpy(sa0, sa1, sizeof t);
    memcpy(sa1, t, sizeof t);
    const float x = ta0;
    ta0 = ta1;
    ta1 = x;
  }
  if (tb1 < tb0) {
    float t[3];
    memcpy(t, sb0, sizeof t);
    memcpy(sb0, sb1, sizeof t);
    memcpy(sb1, t, sizeof t);
    const float x = tb0;
    tb0 = tb1;
    tb1 = x;
  }
  const float lo = ta0 >= tb0 ? ta0 : tb0, hi = ta1 <= tb1 ? ta1 : tb1;
  if (!(lo < hi)) return 0;
  memcpy(p0, ta0 >= tb0 ? sa0 : sb0, sizeof(float) * 3);
  memcpy(p1, ta1 <= tb1 ? sa1 : sb1, sizeof(float) * 3);
  return 1;
}

static int edge_tri(const float e0[3], const float e1[3], const float* t0, const float* t1, const float* t2,
                    float x[3]) {
  float dir[3], t;
  sub3v(dir, e1, e0);
  if (!or_tri3_ray(t0, t1, t2, e0, dir, &t, NULL) || !(t <= 1.0f)) return 0;
  for (int k = 0; k < 3; ++k) x[k] = e0[k] + t * dir[k];
  return 1;
}

int or_tri_pair_segment(const uint32_t* tri2vtx, const float* vtx2xyz, uint32_t it, uint32_t jt, float p0[3],
                        float p1[3]) {
  if (it == jt) return 0;
  const uint32_t* vi = tri2vtx + (size_t)it * 3;
  const uint32_t* vj = tri2vtx + (size_t)jt * 3;
  int ci[3], cj[3], shared = 0;
  for (int k = 0; k < 3; ++k) {
    ci[k] = vi[k] == vj[0] || vi[k] == vj[1] || vi[k] == vj[2];
    cj[k] = vj[k] == vi[0] || vj[k] == vi[1] || vj[k] == vi[2];
    shared += ci[k];
  }
  if (shared >= 2) return 0;
  const float* a[3];
  const float* b[3];
  for (int k = 0; k < 3; ++k) {
    a[k] = vtx2xyz + (size_t)vi[k] * 3;
    b[k] = vtx2xyz + (size_t)vj[k] * 3;
  }
  if (shared == 0) return tri_tri_segment(a, b, p0, p1);
  const int si = ci[0] ? 0 : (ci[1] ? 1 : 2), sj = cj[0] ? 0 : (cj[1] ? 1 : 2);
  const float *s = a[si], *pa = a[(si + 1) % 3], *pb = a[(si + 2) % 3], *qa = b[(sj + 1) % 3], *qb = b[(sj + 2) % 3];
  float x[3];
  if (edge_tri(qa, qb, s, pa, pb, x) || edge_tri(pa, pb, s, qa, qb, x)) {
    memcpy(p0, s, sizeof(float) * 3);
    memcpy(p1, x, sizeof(float) * 3);
    return 1;
  }
  return 0;
}

typedef struct {
  const uint32_t* tri2vtx;
  const float* vtx2xyz;
  const uint32_t* bvhnodes;
  const float* aabb;
  uint32_t cap, cnt;
  uint32_t* pairs;
  float* segs;
} SelfxCtx;

static int boxes_overlap(const float* a, const float* b) {
  return a[0] <= b[3] && b[0] <= a[3] && a[1] <= b[4] && b[1] <= a[4] && a[2] <= b[5] && b[2] <= a[5];
}

static void selfx_between(SelfxCtx* c, uint32_t n0, uint32_t n1) {
  if (!boxes_overlap(c->aabb + (size_t)n0 * 6, c->aabb + (size_t)n1 * 6)) return;
  const uint32_t a0 = c->bvhnodes[n0 * 3 + 1], a1 = c->bvhnodes[n0 * 3 + 2];
  const uint32_t b0 = c->bvhnodes[n1 * 3 + 1], b1 = c->bvhnodes[n1 * 3 + 2];
  const int la = a1 == OR_UMAX, lb = b1 == OR_UMAX;
  if (!la && !lb) {
    selfx_between(c, a0, b0);
    selfx_between(c, a1, b0);
    selfx_between(c, a0, b1);
    selfx_between(c, a1, b1);
  } else if (!la) {
    selfx_between(c, a0, n1);
    selfx_between(c, a1, n1);
  } else if (!lb) {
    selfx_between(c, n0, b0);
    selfx_between(c, n0, b1);
  } else {
    float p0[3], p1[3];
    if (or_tri_pair_segment(c->tri2vtx, c->vtx2xyz, a0, b0, p0, p1)) {
      if (c->cnt < c->cap) {
        c->pairs[c->cnt * 2] = a0;
        c->pairs[c->cnt * 2 + 1] = b0;
        memcpy(c->segs + (size_t)c->cnt * 6, p0, sizeof p0);
        memcpy(c->segs + (size_t)c->cnt * 6 + 3, p1, sizeof p1);
      }
      ++c->cnt;
    }
  }
}

static void selfx_inside(SelfxCtx* c, uint32_t n) {
  const uint32_t c0 = c->bvhnodes[n * 3 + 1], c1 = c->bvhnodes[n * 3 + 2];
  if (c1 == OR_UMAX) return;
  selfx_between(c, c0, c1);
  selfx_inside(c, c0);
  selfx_inside(c, c1);
}

uint32_t or_self_intersection(const uint32_t* tri2vtx, const float* vtx2xyz, const uint32_t* bvhnodes,
                              const float* aabb, uint32_t cap, uint32_t* pairs, float* segs) {
  SelfxCtx c = {tri2vtx, vtx2xyz, bvhnodes, aabb, cap, 0, pairs, segs};
  selfx_inside(&c, 0);
  return c.cnt;
}

uint32_t or_self_intersection_brute(uint32_t num_tri, const uint32_t* tri2vtx, const float* vtx2xyz, uint32_t cap,
                                    uint32_t* pairs, float* segs) {
  uint32_t cnt = 0;
  for (uint32_t i = 0; i < num_tri; ++i)
    for (uint32_t j = i + 1; j < num_tri; ++j) {
      float p0[3], p1[3];
      if (!or_tri_pair_segment(tri2vtx, vtx2xyz, i, j, p0, p1)) continue;
      if (cnt < cap) {
        pairs[cnt * 2] = i;
        pairs[cnt * 2 + 1] = j;
        memcpy(segs + (size_t)cnt * 6, p0, sizeof p0);
        memcpy(segs + (size_t)cnt * 6 + 3, p1, sizeof p1);
      }
      ++cnt;
    }
  return cnt;
}

/* ------------------------------------------------------------------------
 * pix2tri.rs:50-119 pix2tri_by_rasterization: every triangle is mapped to
 * pixel space through the inverse of transform_ndc2world
 * (px = ((x+1)/2 W, (1-y)/2 H)); each pixel whose centre it covers gets it
 * when its depth, the barycentric interpolation of the three ndc z, is
 * greater than the pixel's so far (pix2depth starts at -inf; strict >, so
 * the first triangle wins a tie).  Triangles with a vertex whose homogeneous
 * w is 0 are skipped, as transform_homogeneous returns None for them.
 *
 * del-geo-core's tri2_scanline (absent here) is restated from the definition
 * of a scanline walk over pixel centres: row iy is visited when its centre
 * line y = iy + 0.5 lies within the triangle's y extent; on it the triangle
 * spans x in [xl, xr] (the crossings of that line with the edges), and the
 * pixels of the row whose centres x = ix + 0.5 lie in [xl, xr] are covered.
 * barycentric_coords (also absent) is the ratio of signed areas, None for a
 * triangle of zero area. */
static float cross2(float ax, float ay, float bx, float by) { return ax * by - ay * bx; }

static int barycentric2(const float a[2], const float b[2], const float c[2], const float q[2], float w[3]) {
  const float area = cross2(b[0] - a[0], b[1] - a[1], c[0] - a[0], c[1] - a[1]);
  if (area == 0.0f) return 0;
  w[0] = cross2(b[0] - q[0], b[1] - q[1], c[0] - q[0], c[1] - q[1]) / area;
  w[1] = cross2(c[0] - q[0], c[1] - q[1], a[0] - q[0], a[1] - q[1]) / area;
  w[2] = cross2(a[0] - q[0], a[1] - q[1], b[0] - q[0], b[1] - q[1]) / area;
  return 1;
}

static int homogeneous_ok(const float m[16], const float p[3], float out[3]) {
  const float w = m[3] * p[0] + m[7] * p[1] + m[11] * p[2] + m[15];
  if (w == 0.0f) return 0;
  for (int i = 0; i < 3; ++i) out[i] = (m[i] * p[0] + m[4 + i] * p[1] + m[8 + i] * p[2] + m[12 + i]) / w;
  return 1;
}

int or_pix2tri_by_rasterization(uint32_t img_w, uint32_t img_h, const float t_ndc2world[16], uint32_t num_tri,
                                const uint32_t* tri2vtx, const float* vtx2xyz, uint32_t* pix2tri, float* pix2depth) {
  float w2n[16];
  if (!or_mat4_inverse_pivot(t_ndc2world, w2n)) return 0;
  for (size_t i = 0; i < (size_t)img_w * img_h; ++i) {
    pix2tri[i] = OR_UMAX;
    pix2depth[i] = -INFINITY;
  }
  for (uint32_t it = 0; it < num_tri; ++it) {
    float ndc[3][3], px[3][2];
    int ok = 1;
    for (int k = 0; k < 3 && ok; ++k) {
      ok = homogeneous_ok(w2n, vtx2xyz + (size_t)tri2vtx[(size_t)it * 3 + k] * 3, ndc[k]);
      px[k][0] = (ndc[k][0] + 1.0f) * 0.5f * (float)img_w;
      px[k][1] = (1.0f - ndc[k][1]) * 0.5f * (float)img_h;
    }
    if (!ok) continue;
    float ymin = px[0][1], ymax = px[0][1];
    for (int k = 1; k < 3; ++k) {
      if (px[k][1] < ymin) ymin = px[k][1];
      if (px[k][1] > ymax) ymax = px[k][1];
    }
    if (!(ymin == ymin) || !(ymax == ymax)) continue;  /* NaN vertex */
    double r0 = ceil((double)ymin - 0.5), r1 = floor((double)ymax - 0.5);
    if (r0 < 0) r0 = 0;
    if (r1 > (double)img_h - 1) r1 = (double)img_h - 1;
    for (double ry = r0; ry <= r1; ry += 1.0) {
      const uint32_t iy = (uint32_t)ry;
      const float yc = (float)iy + 0.5f;
      float xl = INFINITY, xr = -INFINITY;
      for (int e = 0; e < 3; ++e) {
        const float* p = px[e];
        const float* q = px[(e + 1) % 3];
        const float lo = p[1] < q[1] ? p[1] : q[1], hi = p[1] < q[1] ? q[1] : p[1];
        if (yc < lo || yc > hi) continue;
        if (p[1] == q[1]) { /* a horizontal edge on the centre line: both ends */
          if (p[0] < xl) xl = p[0];
          if (q[0] < xl) xl = q[0];
          if (p[0] > xr) xr = p[0];
          if (q[0] > xr) xr = q[0];
          continue;
        }
        const float x = p[0] + (yc - p[1]) * (q[0] - p[0]) / (q[1] - p[1]);
        if (x < xl) xl = x;
        if (x > xr) xr = x;
      }
      if (!(xl <= xr)) continue;
      double c0 = ceil((double)xl - 0.5), c1 = floor((double)xr - 0.5);
      if (c0 < 0) c0 = 0;
      if (c1 > (double)img_w - 1) c1 = (double)img_w - 1;
      for (double cx = c0; cx <= c1; cx += 1.0) {
        const uint32_t ix = (uint32_t)cx;
        const float centre[2] = {(float)ix + 0.5f, yc};
        float b[3];
        if (!barycentric2(px[0], px[1], px[2], centre, b)) continue;
        const float depth = b[0] * ndc[0][2] + b[1] * ndc[1][2] + b[2] * ndc[2][2];
        const size_t ip = (size_t)iy * img_w + ix;
        if (depth > pix2depth[ip]) {
          pix2depth[ip] = depth;
          pix2tri[ip] = it;
        }
      }
    }
  }
  return 1;
}
