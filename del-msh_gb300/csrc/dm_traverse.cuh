// dm_traverse.cuh — closest-hit traversal of an LBVH in del-msh's layout
// (bvhnodes u32[(2T-1)*3] = [parent, left, right], bvhnode2aabb f32[(2T-1)*6]),
// shared by the single-mesh cast (cast.cu) and the batched cast (batch.cu).
//
// The result is, bit for bit, del-msh-cpu's recursive near-first search
// (search_bvh3.rs:103-221): at a branch the child with the smaller
// (t_enter, t_exit) tuple is searched first; the far child is skipped when the
// near result exists and the far box is missed or entered beyond it; and of
// two results the far one wins unless the near one is strictly closer.
//
// Iterative form.  Call R(n) the recursive result of node n.  "Pick" (keep
// the later of two results unless the earlier is strictly closer) is
// associative, so a run of picks is the last closest result in visit order.
// Only a branch whose two child boxes are both hit and whose near child is a
// branch needs a frame: it holds the far child, its slab entry, and the result
// accumulated so far at the enclosing level ("saved"), and the accumulator
// restarts empty, so that when the near subtree is finished the accumulator
// equals R(near) exactly — the value the far-child test of
// search_bvh3.rs:168-189 needs.  When only one child box is hit, R(n) is that
// child's result and the descent continues without a frame; a leaf near child
// is resolved inline; a far child that must be searched continues in the
// enclosing level after folding R(near) into "saved".
//
// Link chains.  A "link" branch i has the leaf i (node T-1+i) as left child
// and branch i+1 as right child; a run of k equal Morton codes is a chain of
// k-1 links.  When a link's near child is branch i+1 and both boxes are hit,
// its frame is (far = leaf i, enter, saved); along a descent through
// consecutive links every frame after the first has saved = none, so the
// whole run is kept as one chain frame (first link s, last link t, saved of
// s) and unwound leaf by leaf (t, t-1, ..., s), recomputing each far leaf's
// slab entry.  The stack then grows with the number of runs, not their
// length, and the decisions are exactly those of the uncompressed frames.
//
// Execution.  The traversal is a step function (one node entry plus the
// ascent that follows it) run by persistent warps: a lane whose ray is
// finished takes the next ray index from a global counter (one atomic per
// warp), so lanes stay busy while long rays finish.  Frames live in a
// kCastStack-entry on-chip (local) stack; a ray that needs more is appended to
// an overflow list and re-cast from scratch by a second kernel whose per-ray
// stacks are carved from a global pool (capacity chosen on the device from
// the overflow count), and anything still deeper by a third kernel with
// capacity num_tri, which no tree can exceed.  Duplicate Morton codes produce
// long chains (a run of k equal codes is a chain of height k), which is where
// the deeper tiers are used.
#pragma once
#include "dm_device.cuh"
#include "dm_internal.h"

namespace dm {

struct Hit {
  float t;
  uint32_t id;  // kUMax == none
};

// Keep `b` (the later result) unless `a` is strictly closer; none is the identity.
__device__ __forceinline__ Hit pick(Hit a, Hit b) {
  if (a.id == kUMax) return b;
  if (b.id == kUMax) return a;
  return (a.t < b.t) ? a : b;
}

struct Ray {
  float3 org, dir, inv;
};

__device__ __forceinline__ Ray make_ray(float3 o, float3 d) {
  Ray r;
  r.org = o;
  r.dir = d;
  r.inv = make_float3(__fdiv_rn(1.0f, d.x), __fdiv_rn(1.0f, d.y), __fdiv_rn(1.0f, d.z));
  return r;
}

// Leaf test: search_bvh3.rs:117-128 with dis = +inf.  Out-of-range triangle
// or vertex indices count as a miss and are reported through `bad`.
__device__ __forceinline__ bool leaf_hit(const MeshView& m, const Ray& r, uint32_t it, float& t, float& u, float& v,
                                         bool& bad) {
  if (it >= m.num_tri) {
    bad = true;
    return false;
  }
  const uint32_t* tv = m.tri2vtx + static_cast<size_t>(it) * 3;
  const uint32_t i0 = __ldg(tv), i1 = __ldg(tv + 1), i2 = __ldg(tv + 2);
  if (i0 >= m.num_vtx || i1 >= m.num_vtx || i2 >= m.num_vtx) {
    bad = true;
    return false;
  }
  const float3 p0 = load_vtx(m.vtx2xyz, i0);
  const float3 p1 = load_vtx(m.vtx2xyz, i1);
  const float3 p2 = load_vtx(m.vtx2xyz, i2);
  return tri_ray(p0, p1, p2, r.org, r.dir, t, u, v) && t < INFINITY;
}

__device__ __forceinline__ bool node_slab(const MeshView& m, const Ray& r, uint32_t n, float& te, float& tx) {
  return slab(m.aabb + static_cast<size_t>(n) * 6, r.org, r.inv, r.dir, te, tx);
}

struct LocalStack {
  uint4* p;
  __device__ __forceinline__ void store(uint32_t i, uint4 v) const { p[i] = v; }
  __device__ __forceinline__ uint4 load(uint32_t i) const { return p[i]; }
};

struct GlobalStack {
  uint4* p;
  __device__ __forceinline__ void store(uint32_t i, uint4 v) const { __stcg(p + i, v); }
  __device__ __forceinline__ uint4 load(uint32_t i) const { return __ldcg(p + i); }
};

constexpr uint32_t kChainBit = 0x80000000u;  // frame.x flag of a chain frame (node ids are < 2^31)

// Per-ray traversal state between steps.
struct Trav {
  uint32_t node;         // node to enter next
  uint32_t left, right;  // its record (bvhnodes[node*3+1], [node*3+2]), fetched ahead
  uint32_t sp;           // frames in use
  uint32_t steps;        // node entries so far (bounded by the node count)
  uint32_t chain_next;   // the link that would extend the top chain frame, or kUMax
  Hit best;              // accumulator of the current level
};

__device__ __forceinline__ void load_record(const uint32_t* __restrict__ bn, uint32_t n, uint32_t& left,
                                            uint32_t& right) {
  left = __ldg(bn + static_cast<size_t>(n) * 3 + 1);
  right = __ldg(bn + static_cast<size_t>(n) * 3 + 2);
}

enum StepResult : int { kStepContinue = 0, kStepDone = 1, kStepOverflow = 2 };

// Starts a ray: a miss of the root box finishes it immediately.
__device__ __forceinline__ bool trav_begin(const MeshView& m, const Ray& r, Trav& s) {
  s.node = 0;
  s.sp = 0;
  s.steps = 0;
  s.chain_next = kUMax;
  s.best = Hit{INFINITY, kUMax};
  load_record(m.bvhnodes, 0, s.left, s.right);
  float te, tx;
  return node_slab(m, r, 0, te, tx);
}

// One node entry and the ascent that follows it.  On kStepDone the ray's
// result is s.best.  The records of both children are fetched together with
// their boxes, so descending costs one dependent memory round trip per level.
// A malformed tree (child index out of range, or more node entries than the
// tree has nodes) finishes the ray and sets `bad`.
template <typename StackT>
__device__ __forceinline__ int trav_step(const MeshView& m, const Ray& r, StackT stack, uint32_t cap, Trav& s,
                                         bool& bad) {
  const uint32_t* __restrict__ bn = m.bvhnodes;
  const uint32_t num_node = 2 * m.num_tri - 1;
  if (++s.steps > num_node + 1) {
    bad = true;
    return kStepDone;
  }
  bool ascend = false;
  // At most one triangle test per step, issued from one place so that lanes
  // testing a root / far leaf and lanes testing a near leaf share it.
  uint32_t leaf_tri = kUMax;
  bool leaf_near = false, has_far = false;
  uint32_t nf = 0, f_l = 0, f_r = 0;
  float far_enter = 0.f;
  if (s.right == kUMax) {  // a leaf reached as the root or as a far child
    leaf_tri = s.left;
  } else {
    const uint32_t node = s.node, left = s.left, right = s.right;
    if (left >= num_node || right >= num_node) {
      bad = true;
      return kStepDone;
    }
    uint32_t ll, lr, rl, rr;
    load_record(bn, left, ll, lr);
    load_record(bn, right, rl, rr);
    float l0 = 0.f, l1 = 0.f, r0 = 0.f, r1 = 0.f;
    const bool hl = node_slab(m, r, left, l0, l1);
    const bool hr = node_slab(m, r, right, r0, r1);
    if (!hl && !hr) {
      ascend = true;
    } else {
      const bool near_left = (hl && hr) ? tuple_lt(l0, l1, r0, r1) : hl;
      const uint32_t nn = near_left ? left : right;
      nf = near_left ? right : left;
      const uint32_t n_l = near_left ? ll : rl, n_r = near_left ? lr : rr;
      f_l = near_left ? rl : ll;
      f_r = near_left ? rr : lr;
      has_far = hl && hr;
      far_enter = near_left ? r0 : l0;
      if (n_r == kUMax) {  // near child is a leaf holding triangle n_l
        leaf_tri = n_l;
        leaf_near = true;
      } else if (!has_far) {
        s.node = nn;  // R(node) == R(near): no pending decision, no frame
        s.left = n_l;
        s.right = n_r;
      } else {
        const bool link = !near_left && left == m.num_tri - 1 + node && right == node + 1;
        if (link && node == s.chain_next && s.best.id == kUMax) {
          // extend the chain frame on top: its last link becomes `node`
          const uint4 f = stack.load(s.sp - 1);
          stack.store(s.sp - 1, make_uint4(f.x, node, f.z, f.w));
        } else {
          if (s.sp >= cap) return kStepOverflow;
          if (link)
            stack.store(s.sp++, make_uint4(kChainBit | node, node, __float_as_uint(s.best.t), s.best.id));
          else
            stack.store(s.sp++, make_uint4(nf, __float_as_uint(far_enter), __float_as_uint(s.best.t), s.best.id));
        }
        s.chain_next = link ? node + 1 : kUMax;
        s.best = Hit{INFINITY, kUMax};
        s.node = nn;
        s.left = n_l;
        s.right = n_r;
      }
    }
  }
  if (leaf_tri != kUMax) {
    float t, u, v;
    const bool h = leaf_hit(m, r, leaf_tri, t, u, v, bad);
    if (h) s.best = pick(s.best, Hit{t, leaf_tri});
    if (!leaf_near || !has_far || (h && far_enter > t)) {
      ascend = true;
    } else {  // the far child of a near leaf
      s.node = nf;
      s.left = f_l;
      s.right = f_r;
    }
  }
  if (!ascend) return kStepContinue;
  s.chain_next = kUMax;
  while (s.sp > 0) {
    const uint4 f = stack.load(s.sp - 1);
    const Hit saved{__uint_as_float(f.z), f.w};
    uint32_t far;
    float far_enter;
    bool pop = true;
    if (f.x & kChainBit) {
      // level j = f.y of a chain frame: far child = leaf j, saved = none
      // unless j is the chain's first link
      const uint32_t first = f.x & ~kChainBit, j = f.y;
      far = m.num_tri - 1 + j;
      if (far >= num_node) {
        bad = true;
        return kStepDone;
      }
      float te = 0.f, tx = 0.f;
      node_slab(m, r, far, te, tx);  // hit when the frame was pushed; same value again
      far_enter = te;
      pop = j == first;
      if (pop) --s.sp;
      else stack.store(s.sp - 1, make_uint4(f.x, j - 1, f.z, f.w));
    } else {
      --s.sp;
      far = f.x;
      far_enter = __uint_as_float(f.y);
    }
    // The far test sees R(near) alone (search_bvh3.rs:168-189); only then is
    // the enclosing level's result folded in.  Deciding on the folded value
    // instead agrees only while every hit lies at or beyond its box's entry
    // t, which rounding does not guarantee (a triangle on a box face).
    const bool skip = (s.best.id != kUMax) && far_enter > s.best.t;
    if (pop) s.best = pick(saved, s.best);
    if (!skip) {
      s.node = far;
      if (s.node >= num_node) {
        bad = true;
        return kStepDone;
      }
      load_record(bn, s.node, s.left, s.right);
      return kStepContinue;
    }
  }
  return kStepDone;
}

// Barycentrics of a final hit (recomputed once per ray when asked for).
__device__ __forceinline__ void hit_bc(const MeshView& m, const Ray& r, const Hit& h, float bc[3]) {
  bc[0] = bc[1] = bc[2] = 0.0f;
  if (h.id == kUMax) return;
  float t, u, v;
  bool bad = false;
  if (leaf_hit(m, r, h.id, t, u, v, bad)) {
    bc[0] = __fsub_rn(__fsub_rn(1.0f, u), v);
    bc[1] = u;
    bc[2] = v;
  }
}

constexpr int kCastThreads = 128;

// A Job maps a work index to (mesh, ray, output slot):
//   uint32_t num_work;                              work indices are 0..num_work-1
//   __device__ void prepare(float* smem) const;    once per block, before __syncthreads
//   __device__ bool fetch(uint32_t w, const float* smem, MeshView& m, Ray& r, uint32_t& out) const;
//                                                   false: w is padding, nothing to do
//   __device__ void write(uint32_t out, const MeshView& m, const Ray& r, const Hit& h) const;

// Persistent warps with per-lane ray refill.  Rays overflowing the on-chip
// stack go to ovf_list (their work index).  kThreads threads per block and
// kStack on-chip frames per ray are tuning choices (Tuning); the register
// bound (64 registers) keeps 2048 resident threads per SM.
template <typename Job, int kThreads, int kStack>
__global__ void __launch_bounds__(kThreads, 65536 / (64 * kThreads)) k_cast_persistent(Job job, uint32_t* work_counter,
                                                                                 uint32_t* ovf_list,
                                                                                 uint32_t* ovf_count,
                                                                                 uint32_t* status) {
  __shared__ float smem[64];
  job.prepare(smem);
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t lt_mask = (1u << lane) - 1u;
  uint4 frames[kStack];
  LocalStack stack{frames};
  MeshView m{};
  Ray r{};
  Trav s{};
  uint32_t out = 0, work = kUMax;
  bool active = false, exhausted = false, bad = false;
  for (;;) {
    // refill idle lanes with consecutive work indices
    const uint32_t idle = __ballot_sync(0xffffffffu, !active);
    if (idle != 0u && !exhausted) {
      uint32_t base = 0;
      if (lane == static_cast<uint32_t>(__ffs(idle) - 1)) base = atomicAdd(work_counter, __popc(idle));
      base = __shfl_sync(0xffffffffu, base, __ffs(idle) - 1);
      if (base >= job.num_work) exhausted = true;  // warp-uniform
      if (!active) {
        const uint32_t w = base + __popc(idle & lt_mask);
        if (w < job.num_work && job.fetch(w, smem, m, r, out)) {
          work = w;
          if (trav_begin(m, r, s)) active = true;
          else job.write(out, m, r, s.best);
        }
      }
    }
    if (__all_sync(0xffffffffu, !active)) {
      if (exhausted) break;
      continue;
    }
    if (active) {
      const int rc = trav_step(m, r, stack, kStack, s, bad);
      if (rc == kStepDone) {
        job.write(out, m, r, s.best);
        active = false;
      } else if (rc == kStepOverflow) {
        ovf_list[atomicAdd(ovf_count, 1u)] = work;
        active = false;
      }
    }
  }
  if (bad) raise_status(status, kStatusBadIndex);
}

// Re-casts the work indices of list_in with stacks carved from the pool.
// cap_fixed == 0 chooses the capacity from the number of rays to process.
template <typename Job>
__global__ void __launch_bounds__(kCastThreads) k_cast_deep(Job job, const uint32_t* list_in, const uint32_t* count_in,
                                                           uint32_t* list_out, uint32_t* count_out, uint4* pool,
                                                           uint64_t pool_frames, uint32_t cap_fixed,
                                                           uint32_t max_tri, uint32_t* status) {
  __shared__ float smem[64];
  job.prepare(smem);
  __syncthreads();
  const uint32_t num = *count_in;
  if (num == 0) return;
  uint64_t cap = cap_fixed;
  if (cap == 0) {
    cap = pool_frames / num;
    if (cap < 256) cap = 256;
    const uint64_t cap_max = 2ull * max_tri;  // never more than the deepest possible tree needs
    if (cap > cap_max) cap = cap_max;
  }
  if (cap > pool_frames) cap = pool_frames;
  const uint64_t threads = static_cast<uint64_t>(gridDim.x) * kCastThreads;
  uint64_t slots = pool_frames / cap;
  if (slots > threads) slots = threads;
  const uint64_t slot = static_cast<uint64_t>(threadIdx.x) * gridDim.x + blockIdx.x;  // spread over blocks
  if (slot >= slots) return;
  GlobalStack st{pool + slot * cap};
  bool bad = false;
  for (uint64_t k = slot; k < num; k += slots) {
    const uint32_t w = list_in[k];
    MeshView m{};
    Ray r{};
    uint32_t out = 0;
    if (!job.fetch(w, smem, m, r, out)) continue;
    Trav s{};
    int rc = kStepDone;
    if (trav_begin(m, r, s)) {
      do {
        rc = trav_step(m, r, st, static_cast<uint32_t>(cap), s, bad);
      } while (rc == kStepContinue);
    }
    if (rc == kStepDone) {
      job.write(out, m, r, s.best);
    } else if (list_out) {
      list_out[atomicAdd(count_out, 1u)] = w;
    } else {
      raise_status(status, kStatusStackOverflow);
      job.write(out, m, r, Hit{INFINITY, kUMax});
    }
  }
  if (bad) raise_status(status, kStatusBadIndex);
}

// Number of resident blocks of a persistent kernel instantiation on the
// current device.
template <typename Job, int kThreads, int kStack>
inline int persistent_grid() {
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (cached[dev] == 0) {
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cast_persistent<Job, kThreads, kStack>, kThreads, 0);
    cached[dev] = (sms > 0 ? sms : 152) * (per_sm > 0 ? per_sm : 1);
  }
  return cached[dev];
}

template <typename Job, int kThreads, int kStack>
inline void launch_persistent(cudaStream_t s, const Job& job, const CastScratch& sc, uint32_t* status) {
  int grid = persistent_grid<Job, kThreads, kStack>();
  const uint32_t needed = (job.num_work + kThreads - 1) / kThreads;
  if (static_cast<uint32_t>(grid) > needed) grid = static_cast<int>(needed);
  k_cast_persistent<Job, kThreads, kStack><<<grid, kThreads, 0, s>>>(job, sc.counters, sc.list1, sc.counters + 1,
                                                                     status);
}

// The three-tier cast of every work index of `job`.  sc.counters (4 words)
// must be zero on entry: [0] work counter, [1] tier-1 overflow count, [2]
// tier-2 overflow count.  The first tier's block size and on-chip stack
// depth come from the current Tuning (kCastVariants lists the choices).
template <typename Job>
inline void cast_job(cudaStream_t s, const Job& job, const CastScratch& sc, uint32_t max_tri, uint32_t* status) {
  if (job.num_work == 0) return;
  const Tuning t = get_tuning();
  if (t.cast_threads == 64 && t.cast_stack == 64) launch_persistent<Job, 64, 64>(s, job, sc, status);
  else if (t.cast_threads == 256 && t.cast_stack == 64) launch_persistent<Job, 256, 64>(s, job, sc, status);
  else if (t.cast_threads == 128 && t.cast_stack == 32) launch_persistent<Job, 128, 32>(s, job, sc, status);
  else if (t.cast_threads == 128 && t.cast_stack == 96) launch_persistent<Job, 128, 96>(s, job, sc, status);
  else launch_persistent<Job, 128, 64>(s, job, sc, status);
  const uint64_t pool_frames = sc.pool_bytes / kFrameBytes;
  uint4* pool = static_cast<uint4*>(sc.pool);
  const uint32_t deep_grid = 152 * 4;
  k_cast_deep<Job><<<deep_grid, kCastThreads, 0, s>>>(job, sc.list1, sc.counters + 1, sc.list2, sc.counters + 2,
                                                      pool, pool_frames, 0u, max_tri, status);
  const uint32_t cap3 = max_tri < 2 ? 2u : max_tri;
  k_cast_deep<Job><<<deep_grid, kCastThreads, 0, s>>>(job, sc.list2, sc.counters + 2, nullptr, nullptr, pool,
                                                      pool_frames, cap3, max_tri, status);
}

}  // namespace dm
