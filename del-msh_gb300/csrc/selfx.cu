// selfx.cu — self-intersection of a triangle mesh through its BVH
// (trimesh3_intersection.rs:1-179: search_with_bvh_inside_branch and
// search_with_bvh_between_branches).  The recursion inside(root) visits, at
// every branch n, between(left(n), right(n)) and recurses; so the pairs are
// exactly the union over branches n of between(left(n), right(n)).  Each
// start pair is searched depth-first by one thread with an explicit stack of
// node pairs, in rounds: a thread that has visited kBudget pairs hands its
// remaining stack to the next round, so that the few large subtree pairs
// near the root spread over many threads instead of one.
// Every unordered pair of leaves meets at exactly one branch (their
// lowest common ancestor), with the triangle of the left subtree first, as
// in the recursion; only the order of the output list differs.
//
// Triangle pairs (trimesh3_intersection.rs:10-79): no shared vertex -> the
// segment where the two triangles cross; one shared vertex -> the segment
// from the shared vertex to where an opposite edge pierces the other
// triangle; two shared vertices -> none (three -> none here; the reference
// panics).  The segment formulas of del-geo-core are restated:
// - tri/tri: each triangle's crossing segment with the other's plane (edge
//   crossings v_i + (v_j - v_i) d_i / (d_i - d_j), plus vertices on the
//   plane), both projected on the planes' common direction n_a x n_b, and
//   their overlap [max of starts, min of ends], reported when of non-zero
//   length; coplanar pairs are not reported;
// - shared vertex: Moller-Trumbore of the opposite edge of one triangle (as
//   a segment, 0 <= t <= 1) against the other, first (q1, q2) against the
//   first triangle, then (p1, p2) against the second.
#include "dm_device.cuh"
#include "dm_internal.h"

namespace dm {
namespace {

constexpr int kThreads = 128;
constexpr int kPairStack = 192;  // node pairs on the per-thread stack

__device__ __forceinline__ float3 lerp_cross(float3 vi, float3 vj, float di, float dj) {
  const float s = __fdiv_rn(di, __fsub_rn(di, dj));
  return make_float3(__fadd_rn(vi.x, __fmul_rn(__fsub_rn(vj.x, vi.x), s)),
                     __fadd_rn(vi.y, __fmul_rn(__fsub_rn(vj.y, vi.y), s)),
                     __fadd_rn(vi.z, __fmul_rn(__fsub_rn(vj.z, vi.z), s)));
}

// The segment where triangle v crosses the plane with signed distances d.
__device__ __forceinline__ bool plane_segment(const float3 v[3], const float d[3], float3& s0, float3& s1) {
  float3 pts[4];
  int n = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (d[k] == 0.0f) pts[n++] = v[k];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int i = k, j = (k + 1) % 3;
    if ((d[i] > 0.0f && d[j] < 0.0f) || (d[i] < 0.0f && d[j] > 0.0f)) pts[n++] = lerp_cross(v[i], v[j], d[i], d[j]);
  }
  if (n < 2) return false;
  s0 = pts[0];
  s1 = pts[1];
  return true;
}

__device__ __forceinline__ bool tri_tri_segment(const float3 a[3], const float3 b[3], float3& p0, float3& p1) {
  const float3 nb = cross3(sub3(b[1], b[0]), sub3(b[2], b[0]));
  const float db = -dot3(nb, b[0]);
  float da[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) da[k] = __fadd_rn(dot3(nb, a[k]), db);
  if ((da[0] > 0.0f && da[1] > 0.0f && da[2] > 0.0f) || (da[0] < 0.0f && da[1] < 0.0f && da[2] < 0.0f)) return false;
  if (da[0] == 0.0f && da[1] == 0.0f && da[2] == 0.0f) return false;
  const float3 na = cross3(sub3(a[1], a[0]), sub3(a[2], a[0]));
  const float dA = -dot3(na, a[0]);
  float dbv[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) dbv[k] = __fadd_rn(dot3(na, b[k]), dA);
  if ((dbv[0] > 0.0f && dbv[1] > 0.0f && dbv[2] > 0.0f) || (dbv[0] < 0.0f && dbv[1] < 0.0f && dbv[2] < 0.0f))
    return false;
  float3 sa0, sa1, sb0, sb1;
  if (!plane_segment(a, da, sa0, sa1) || !plane_segment(b, dbv, sb0, sb1)) return false;
  const float3 D = cross3(na, nb);
  float ta0 = dot3(D, sa0), ta1 = dot3(D, sa1), tb0 = dot3(D, sb0), tb1 = dot3(D, sb1);
  if (ta1 < ta0) {
    const float3 t = sa0;
    sa0 = sa1;
    sa1 = t;
    const float x = ta0;
    ta0 = ta1;
    ta1 = x;
  }
  if (tb1 < tb0) {
    const float3 t = sb0;
    sb0 = sb1;
    sb1 = t;
    const float x = tb0;
    tb0 = tb1;
    tb1 = x;
  }
  const float lo = ta0 >= tb0 ? ta0 : tb0, hi = ta1 <= tb1 ? ta1 : tb1;
  if (!(lo < hi)) return false;
  p0 = ta0 >= tb0 ? sa0 : sb0;
  p1 = ta1 <= tb1 ? sa1 : sb1;
  return true;
}

// Segment (e0, e1) against triangle (t0, t1, t2): Moller-Trumbore with
// 0 <= t <= 1, inclusive edges.
__device__ __forceinline__ bool edge_tri(float3 e0, float3 e1, float3 t0, float3 t1, float3 t2, float3& x) {
  float t, u, v;
  const float3 dir = sub3(e1, e0);
  if (!tri_ray(t0, t1, t2, e0, dir, t, u, v) || !(t <= 1.0f)) return false;
  x = make_float3(__fadd_rn(e0.x, __fmul_rn(t, dir.x)), __fadd_rn(e0.y, __fmul_rn(t, dir.y)),
                  __fadd_rn(e0.z, __fmul_rn(t, dir.z)));
  return true;
}

__device__ __forceinline__ bool tri_pair(const MeshView& m, uint32_t it, uint32_t jt, float3& p0, float3& p1,
                                         uint32_t* status) {
  if (it == jt) return false;
  if (it >= m.num_tri || jt >= m.num_tri) {
    raise_status(status, kStatusBadIndex);
    return false;
  }
  uint32_t vi[3], vj[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    vi[k] = __ldg(m.tri2vtx + static_cast<size_t>(it) * 3 + k);
    vj[k] = __ldg(m.tri2vtx + static_cast<size_t>(jt) * 3 + k);
    if (vi[k] >= m.num_vtx || vj[k] >= m.num_vtx) {
      raise_status(status, kStatusBadIndex);
      return false;
    }
  }
  bool ci[3], cj[3];
  int shared = 0, si = 0, sj = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    ci[k] = vi[k] == vj[0] || vi[k] == vj[1] || vi[k] == vj[2];
    cj[k] = vj[k] == vi[0] || vj[k] == vi[1] || vj[k] == vi[2];
    shared += ci[k] ? 1 : 0;
  }
  if (shared >= 2) return false;
  float3 a[3], b[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    a[k] = load_vtx(m.vtx2xyz, vi[k]);
    b[k] = load_vtx(m.vtx2xyz, vj[k]);
  }
  if (shared == 0) return tri_tri_segment(a, b, p0, p1);
  si = ci[0] ? 0 : (ci[1] ? 1 : 2);
  sj = cj[0] ? 0 : (cj[1] ? 1 : 2);
  const float3 s = a[si], pa = a[(si + 1) % 3], pb = a[(si + 2) % 3];
  const float3 qa = b[(sj + 1) % 3], qb = b[(sj + 2) % 3];
  float3 x;
  if (edge_tri(qa, qb, s, pa, pb, x) || edge_tri(pa, pb, s, qa, qb, x)) {
    p0 = s;
    p1 = x;
    return true;
  }
  return false;
}

__device__ __forceinline__ bool boxes_overlap(const float* a, const float* b) {
  return a[0] <= b[3] && b[0] <= a[3] && a[1] <= b[4] && b[1] <= a[4] && a[2] <= b[5] && b[2] <= a[5];
}

__device__ __forceinline__ void report_pair(const MeshView& m, uint32_t a0, uint32_t b0, uint32_t capacity,
                                            uint32_t* pairs, float* segments, uint32_t* count, uint32_t* status) {
  float3 p0, p1;
  if (!tri_pair(m, a0, b0, p0, p1, status)) return;
  const uint32_t slot = atomicAdd(count, 1u);
  if (slot >= capacity) return;
  pairs[static_cast<size_t>(slot) * 2] = a0;
  pairs[static_cast<size_t>(slot) * 2 + 1] = b0;
  float* sg = segments + static_cast<size_t>(slot) * 6;
  sg[0] = p0.x;
  sg[1] = p0.y;
  sg[2] = p0.z;
  sg[3] = p1.x;
  sg[4] = p1.y;
  sg[5] = p1.z;
}

// The first round starts from (left(n), right(n)) for every branch n.
__global__ void __launch_bounds__(kThreads) k_selfx_init(MeshView m, uint2* frontier) {
  const uint32_t n = blockIdx.x * kThreads + threadIdx.x;
  if (m.num_tri < 2 || n >= m.num_tri - 1) return;
  frontier[n] = make_uint2(__ldg(m.bvhnodes + static_cast<size_t>(n) * 3 + 1),
                           __ldg(m.bvhnodes + static_cast<size_t>(n) * 3 + 2));
}

// One round: each thread searches depth-first from one start pair with an
// explicit stack; after kBudget node-pair visits it hands its remaining stack
// to the next round (when all of it fits there; otherwise it finishes alone),
// so that the few large subtree pairs near the root are split over many
// threads in the following rounds.
constexpr uint32_t kBudget = 512;

__global__ void __launch_bounds__(kThreads) k_selfx_round(MeshView m, const uint2* __restrict__ start,
                                                         uint32_t num_start, uint2* next, uint32_t* num_next,
                                                         uint64_t next_cap, uint32_t capacity, uint32_t* pairs,
                                                         float* segments, uint32_t* count, uint32_t* status) {
  const uint32_t k = blockIdx.x * kThreads + threadIdx.x;
  if (k >= num_start) return;
  const uint32_t num_node = 2 * m.num_tri - 1;
  const uint32_t* bn = m.bvhnodes;
  uint2 stack[kPairStack];
  int sp = 0;
  stack[sp++] = start[k];
  uint32_t visits = 0;
  while (sp > 0) {
    if (++visits > kBudget && sp > 1) {
      // reserve room only if the whole stack fits, so that the next round's
      // list has no unwritten holes (a bounded number of attempts)
      uint32_t cur = *reinterpret_cast<volatile uint32_t*>(num_next);
      bool handed = false;
      for (int attempt = 0; attempt < 64 && cur + static_cast<uint64_t>(sp) <= next_cap; ++attempt) {
        const uint32_t seen = atomicCAS(num_next, cur, cur + static_cast<uint32_t>(sp));
        if (seen == cur) {
          for (int q = 0; q < sp; ++q) next[cur + q] = stack[q];
          handed = true;
          break;
        }
        cur = seen;
      }
      if (handed) return;
      visits = 0;  // no room: keep going alone
    }
    const uint2 pr = stack[--sp];
    if (pr.x >= num_node || pr.y >= num_node) {
      raise_status(status, kStatusBadIndex);
      continue;
    }
    if (!boxes_overlap(m.aabb + static_cast<size_t>(pr.x) * 6, m.aabb + static_cast<size_t>(pr.y) * 6)) continue;
    const uint32_t a0 = __ldg(bn + static_cast<size_t>(pr.x) * 3 + 1), a1 = __ldg(bn + static_cast<size_t>(pr.x) * 3 + 2);
    const uint32_t b0 = __ldg(bn + static_cast<size_t>(pr.y) * 3 + 1), b1 = __ldg(bn + static_cast<size_t>(pr.y) * 3 + 2);
    const bool la = a1 == kUMax, lb = b1 == kUMax;
    if (la && lb) {
      report_pair(m, a0, b0, capacity, pairs, segments, count, status);
      continue;
    }
    const int need = (!la && !lb) ? 4 : 2;
    if (sp + need > kPairStack) {
      raise_status(status, kStatusStackOverflow);
      return;
    }
    // pushed in reverse of the recursion's order, which it then follows
    if (!la && !lb) {
      stack[sp++] = make_uint2(a1, b1);
      stack[sp++] = make_uint2(a0, b1);
      stack[sp++] = make_uint2(a1, b0);
      stack[sp++] = make_uint2(a0, b0);
    } else if (!la) {
      stack[sp++] = make_uint2(a1, pr.y);
      stack[sp++] = make_uint2(a0, pr.y);
    } else {
      stack[sp++] = make_uint2(pr.x, b1);
      stack[sp++] = make_uint2(pr.x, b0);
    }
  }
}

}  // namespace

size_t self_intersection_scratch_bytes(uint32_t num_tri) {
  const uint64_t cap = num_tri < (1u << 20) ? (1u << 20) : num_tri;  // start pairs per round
  return 256 + 2 * cap * sizeof(uint2);
}

int launch_self_intersection(cudaStream_t s, const MeshView& m, uint32_t capacity, uint32_t* pairs, float* segments,
                             uint32_t* count, void* scratch, size_t scratch_bytes, uint32_t* status) {
  if (m.num_tri < 2) return 0;
  uint32_t* num_next = static_cast<uint32_t*>(scratch);
  const uint64_t cap = (scratch_bytes - 256) / (2 * sizeof(uint2));
  uint2* fa = reinterpret_cast<uint2*>(static_cast<char*>(scratch) + 256);
  uint2* fb = fa + cap;
  uint32_t num_cur = m.num_tri - 1;
  k_selfx_init<<<(num_cur + kThreads - 1) / kThreads, kThreads, 0, s>>>(m, fa);
  // rounds until no thread hands work on (each round either finishes its
  // threads' work or splits it, so there are few; bounded here)
  for (int round = 0; round < 1000 && num_cur > 0; ++round) {
    if (cudaMemsetAsync(num_next, 0, sizeof(uint32_t), s) != cudaSuccess) return -1;
    k_selfx_round<<<(num_cur + kThreads - 1) / kThreads, kThreads, 0, s>>>(m, fa, num_cur, fb, num_next, cap,
                                                                           capacity, pairs, segments, count, status);
    uint32_t n = 0;
    if (cudaMemcpyAsync(&n, num_next, sizeof(uint32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess) return -1;
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    num_cur = n;  // every reservation was written in full
    uint2* t = fa;
    fa = fb;
    fb = t;
  }
  return 0;
}

}  // namespace dm
