// dm_lbvh.cuh — the per-branch Karras radix-tree construction shared by the
// single-mesh build (build.cu) and the batched build (batch.cu).
#pragma once
#include "dm_device.cuh"

namespace dm {

// Code / object accessors: the single-mesh arrays, or a segment of the
// batched sort's (mesh << 30 | code) keys and global triangle indices.
struct Codes32 {
  const uint32_t* p;
  __device__ __forceinline__ uint32_t operator()(uint32_t i) const { return __ldg(p + i); }
};
struct Objs32 {
  const uint32_t* p;
  __device__ __forceinline__ uint32_t operator()(uint32_t i) const { return __ldg(p + i); }
};

// Last index of the run of value v that contains position `from` (sorted c).
// Equal to the linear scan of mortons.rs:235-245, found by galloping search.
template <typename Codes>
__device__ __forceinline__ uint32_t run_end(const Codes& c, uint32_t n, uint32_t from, uint32_t v) {
  uint32_t lo = from;  // c[lo] == v
  uint32_t step = 1;
  uint32_t hi = n;     // first index known to differ (or n)
  for (;;) {
    const uint64_t probe = static_cast<uint64_t>(lo) + step;
    if (probe >= n) break;
    if (c(static_cast<uint32_t>(probe)) != v) {
      hi = static_cast<uint32_t>(probe);
      break;
    }
    lo = static_cast<uint32_t>(probe);
    step <<= 1;
  }
  while (hi - lo > 1) {  // invariant: c[lo] == v, hi == n or c[hi] != v
    const uint32_t mid = lo + (hi - lo) / 2;
    if (c(mid) == v) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Range [r0, r1] and split of branch ib of the radix tree over n sorted codes:
// mortons.rs:221-288 (range) and 290-325 (split).  The branch index is always
// one end of its range.
template <typename Codes>
__device__ __forceinline__ void karras_range_split(uint32_t n, const Codes& c, uint32_t ib, uint32_t& r0,
                                                   uint32_t& r1, uint32_t& isplit) {
  if (ib == 0) {
    r0 = 0;
    r1 = n - 1;
  } else {
    const uint32_t mc0 = c(ib - 1), mc1 = c(ib), mc2 = c(ib + 1);
    if (mc0 == mc1 && mc1 == mc2) {
      r0 = ib;
      r1 = run_end(c, n, ib + 1, mc1);
    } else {
      const int dd = __clz(mc1 ^ mc2) - __clz(mc1 ^ mc0);
      const bool up = dd > 0;  // direction d = +1 (else -1)
      const int delta_min = __clz(mc1 ^ (up ? mc0 : mc2));
      // 32-bit steps: lim is the largest step that stays inside [0, n) in
      // direction d (n < 2^30, so lmax <= 2 (lim + 1) fits), and a step s
      // lands on ib + s or ib - s
      const uint32_t lim = up ? n - 1 - ib : ib;
      uint32_t lmax = 2;
      while (lmax <= lim && __clz(mc1 ^ c(up ? ib + lmax : ib - lmax)) > delta_min) lmax *= 2;
      uint32_t l = 0;
      for (uint32_t t = lmax / 2; t >= 1; t /= 2) {
        const uint32_t s = l + t;
        if (s <= lim && __clz(mc1 ^ c(up ? ib + s : ib - s)) > delta_min) l = s;
      }
      const uint32_t j = up ? ib + l : ib - l;
      r0 = up ? ib : j;
      r1 = up ? j : ib;
    }
  }
  isplit = r0;
  const uint32_t mc_start = c(r0);
  const int common = __clz(mc_start ^ c(r1));
  if (common != 32) {
    uint32_t step = r1 - r0;
    while (step > 1) {
      step = (step + 1) / 2;
      const uint32_t cand = isplit + step;
      if (cand >= r1) continue;
      if (__clz(mc_start ^ c(cand)) > common) isplit = cand;
    }
  }
}

// One branch ib of the radix tree over n sorted codes (karras_range_split)
// written in the bvhnodes layout (bvhnodes_morton.rs:24-47).  The other end
// of the branch's range is written to other_end[ib] when other_end !=
// nullptr (used by the refit).
template <typename Codes, typename Objs>
__device__ __forceinline__ void topology_node(uint32_t n, const Codes& c, const Objs& obj, uint32_t* bvhnodes,
                                              uint32_t ib, uint32_t* other_end) {
  uint32_t r0, r1, isplit;
  karras_range_split(n, c, ib, r0, r1, isplit);
  if (other_end) other_end[ib] = (r0 == ib) ? r1 : r0;
  const uint32_t nb = n - 1;
  uint32_t* me = bvhnodes + static_cast<size_t>(ib) * 3;
  if (r0 == isplit) {
    const uint32_t a = nb + isplit;
    me[1] = a;
    uint32_t* la = bvhnodes + static_cast<size_t>(a) * 3;
    la[0] = ib;
    la[1] = obj(isplit);
    la[2] = kUMax;
  } else {
    me[1] = isplit;
    bvhnodes[static_cast<size_t>(isplit) * 3] = ib;
  }
  if (r1 == isplit + 1) {
    const uint32_t b = nb + isplit + 1;
    me[2] = b;
    uint32_t* lb = bvhnodes + static_cast<size_t>(b) * 3;
    lb[0] = ib;
    lb[1] = obj(isplit + 1);
    lb[2] = kUMax;
  } else {
    me[2] = isplit + 1;
    bvhnodes[static_cast<size_t>(isplit + 1) * 3] = ib;
  }
  if (ib == 0) me[0] = kUMax;
}

}  // namespace dm
