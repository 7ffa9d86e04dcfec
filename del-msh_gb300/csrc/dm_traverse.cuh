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
// Execution.  The traversal is split into phases (entering a branch, testing
// a triangle, popping frames) run by persistent warps: a lane whose ray is
// finished takes the next ray index from a global counter (one atomic per
// warp), so lanes stay busy while long rays finish, and the rarer phases
// wait until several lanes need them (k_cast_persistent).  Frames live in a
// kCastStack-entry on-chip (local) stack; a ray that needs more is appended to
// an overflow list and re-cast from scratch by a second kernel whose per-ray
// stacks are carved from a global pool (capacity chosen on the device from
// the overflow count), and anything still deeper by a third kernel with
// capacity num_tri, which no tree can exceed.  Those two keep the top 64
// frames of each stack in an on-chip ring (RingStack) and only its bottom in
// the pool.  Duplicate Morton codes produce
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
  bool nz;  // no zero direction component: box tests take slab_nz
};

__device__ __forceinline__ Ray make_ray(float3 o, float3 d) {
  Ray r;
  r.org = o;
  r.dir = d;
  r.inv = make_float3(__fdiv_rn(1.0f, d.x), __fdiv_rn(1.0f, d.y), __fdiv_rn(1.0f, d.z));
  r.nz = d.x != 0.0f && d.y != 0.0f && d.z != 0.0f;
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
  const float* box = m.aabb + static_cast<size_t>(n) * 6;
  return r.nz ? slab_nz(box, r.org, r.inv, te, tx) : slab(box, r.org, r.inv, r.dir, te, tx);
}

struct LocalStack {
  uint4* p;
  __device__ __forceinline__ void store(uint32_t i, uint4 v) const { p[i] = v; }
  __device__ __forceinline__ uint4 load(uint32_t i) const { return p[i]; }
};

// A ray's stack for the overflow tiers: frames [*lo, sp) live in an on-chip
// ring of kRing frames, the frames below *lo in the ray's global area.  The
// traversal only ever reads the top frame and writes the top or the next
// slot, so a push past the ring spills the ring's oldest frame, and reading a
// top that has left the ring (the ring is then empty) brings it back.  Deep
// chains thus push and pop at on-chip latency; only their bottoms go to L2.
template <int kRing>
struct RingStack {
  static_assert((kRing & (kRing - 1)) == 0, "ring size is a power of two");
  uint4* ring;   // kRing on-chip frames
  uint4* glob;   // the ray's global frames (capacity: the tier's cap)
  uint32_t* lo;  // first frame held by the ring
  __device__ __forceinline__ void store(uint32_t i, uint4 v) const {
    if (i >= *lo + kRing) {  // a push past the ring: spill its oldest frame
      __stcg(glob + *lo, ring[*lo & (kRing - 1)]);
      ++*lo;
    }
    if (i >= *lo) ring[i & (kRing - 1)] = v;
    else __stcg(glob + i, v);
  }
  __device__ __forceinline__ uint4 load(uint32_t i) const {
    if (i >= *lo) return ring[i & (kRing - 1)];
    const uint4 v = __ldcg(glob + i);
    ring[i & (kRing - 1)] = v;  // i is the top and the ring is empty: i becomes its only frame
    *lo = i;
    return v;
  }
};

constexpr uint32_t kChainBit = 0x80000000u;  // frame.x flag of a chain frame (node ids are < 2^31)

// Per-ray traversal state between phases.
struct Trav {
  uint32_t node;         // node to enter next
  uint32_t left, right;  // its record (bvhnodes[node*3+1], [node*3+2]), fetched ahead
  uint32_t sp;           // frames in use
  uint32_t steps;        // node entries so far (bounded by the node count)
  uint32_t chain_next;   // the link that would extend the top chain frame, or kUMax
  uint32_t leaf_tri;     // triangle of a pending leaf test
  float far_enter;       // slab entry of the far child that follows a near leaf
  bool leaf_far;         // a far child (node/left/right) follows the pending leaf
  Hit best;              // accumulator of the current level
};

__device__ __forceinline__ void load_record(const uint32_t* __restrict__ bn, uint32_t n, uint32_t& left,
                                            uint32_t& right) {
  left = __ldg(bn + static_cast<size_t>(n) * 3 + 1);
  right = __ldg(bn + static_cast<size_t>(n) * 3 + 2);
}

enum StepResult : int { kStepContinue = 0, kStepDone = 1, kStepOverflow = 2 };

// What a ray does next.  A step of the recursion is split into phases so
// that the lanes of a warp can run each phase together: entering a branch
// (kLaneInner), testing one triangle (kLaneLeaf), and popping frames until a
// far child is to be searched or the ray is finished (kLaneAscend).
enum LaneState : int {
  kLaneIdle = 0,
  kLaneInner = 1,
  kLaneLeaf = 2,
  kLaneAscend = 3,
  kLaneOverflow = 4,  // the on-chip stack is full: the ray is re-cast by a deeper tier
  kLaneDone = 5,      // s.best is the ray's result
};

// Chain links: branch j whose left child is leaf j and right child branch
// j + 1 (runs of equal Morton codes build long runs of them).  The warp tier
// folds runs of at least kFoldMin links instead of walking them.
constexpr uint32_t kFoldMin = 8;

__device__ __forceinline__ bool is_link(const MeshView& m, uint32_t node, uint32_t left, uint32_t right) {
  return left == m.num_tri - 1 + node && right == node + 1;
}

// Whether a run of at least kFoldMin links starts at branch `node` (its
// record: left, right); the other records are loaded together.
__device__ __forceinline__ bool long_chain_at(const MeshView& m, uint32_t node, uint32_t left, uint32_t right) {
  if (!is_link(m, node, left, right) || node + kFoldMin > m.num_tri - 1) return false;
  bool all = true;
#pragma unroll
  for (uint32_t k = 1; k < kFoldMin; ++k) {
    uint32_t l, r;
    load_record(m.bvhnodes, node + k, l, r);
    all = all && is_link(m, node + k, l, r);
  }
  return all;
}

// Starts a ray: a miss of the root box finishes it immediately.
__device__ __forceinline__ bool trav_begin(const MeshView& m, const Ray& r, Trav& s) {
  s.node = 0;
  s.sp = 0;
  s.steps = 0;
  s.chain_next = kUMax;
  s.leaf_tri = kUMax;
  s.far_enter = 0.f;
  s.leaf_far = false;
  s.best = Hit{INFINITY, kUMax};
  load_record(m.bvhnodes, 0, s.left, s.right);
  float te, tx;
  return node_slab(m, r, 0, te, tx);
}

// Entering node s.node.  A leaf (reached as the root or as a far child)
// becomes a pending test.  A branch tests both child boxes; the records of
// both children are fetched together with their boxes, so descending costs
// one dependent memory round trip per level.  A near leaf becomes a pending
// test with the far child (if its box is hit) parked in s.node/left/right.
// A malformed tree (child index out of range, or more node entries than the
// tree has nodes) finishes the ray and sets `bad`.
template <typename StackT>
__device__ __forceinline__ int phase_inner(const MeshView& m, const Ray& r, StackT stack, uint32_t cap, Trav& s,
                                           bool& bad) {
  const uint32_t* __restrict__ bn = m.bvhnodes;
  const uint32_t num_node = 2 * m.num_tri - 1;
  if (++s.steps > num_node + 1) {
    bad = true;
    return kLaneDone;
  }
  if (s.right == kUMax) {
    s.leaf_tri = s.left;
    s.leaf_far = false;
    return kLaneLeaf;
  }
  const uint32_t node = s.node, left = s.left, right = s.right;
  if (left >= num_node || right >= num_node) {
    bad = true;
    return kLaneDone;
  }
  uint32_t ll, lr, rl, rr;
  load_record(bn, left, ll, lr);
  load_record(bn, right, rl, rr);
  float l0 = 0.f, l1 = 0.f, r0 = 0.f, r1 = 0.f;
  const bool hl = node_slab(m, r, left, l0, l1);
  const bool hr = node_slab(m, r, right, r0, r1);
  if (!hl && !hr) return kLaneAscend;
  const bool near_left = (hl && hr) ? tuple_lt(l0, l1, r0, r1) : hl;
  const uint32_t nn = near_left ? left : right, nf = near_left ? right : left;
  const uint32_t n_l = near_left ? ll : rl, n_r = near_left ? lr : rr;
  const bool has_far = hl && hr;
  const float far_enter = near_left ? r0 : l0;
  if (n_r == kUMax) {  // near child is a leaf holding triangle n_l
    s.leaf_tri = n_l;
    s.leaf_far = has_far;
    s.far_enter = far_enter;
    s.node = nf;
    s.left = near_left ? rl : ll;
    s.right = near_left ? rr : lr;
    return kLaneLeaf;
  }
  if (has_far) {
    const bool link = !near_left && left == m.num_tri - 1 + node && right == node + 1;
    if (link && node == s.chain_next && s.best.id == kUMax) {
      // extend the chain frame on top: its last link becomes `node`
      const uint4 f = stack.load(s.sp - 1);
      stack.store(s.sp - 1, make_uint4(f.x, node, f.z, f.w));
    } else {
      if (s.sp >= cap) return kLaneOverflow;
      if (link)
        stack.store(s.sp++, make_uint4(kChainBit | node, node, __float_as_uint(s.best.t), s.best.id));
      else
        stack.store(s.sp++, make_uint4(nf, __float_as_uint(far_enter), __float_as_uint(s.best.t), s.best.id));
    }
    s.chain_next = link ? node + 1 : kUMax;
    s.best = Hit{INFINITY, kUMax};
  }
  // without a far child R(node) == R(near): no pending decision, no frame
  s.node = nn;
  s.left = n_l;
  s.right = n_r;
  return kLaneInner;
}

// The pending triangle test.  After a near leaf the far child is searched
// unless the leaf was hit before the far box is entered (search_bvh3.rs:168-189).
__device__ __forceinline__ int phase_leaf(const MeshView& m, const Ray& r, Trav& s, bool& bad) {
  float t, u, v;
  const bool h = leaf_hit(m, r, s.leaf_tri, t, u, v, bad);
  if (h) s.best = pick(s.best, Hit{t, s.leaf_tri});
  if (!s.leaf_far || (h && s.far_enter > t)) return kLaneAscend;
  return kLaneInner;
}

// A frame kind that only the warp tier pushes (see ChainFold); elsewhere none.
struct NoFold {
  __device__ __forceinline__ int operator()(const uint4&, Trav&) const { return 0; }
};

// Pops frames until a far child is to be searched (kLaneInner) or the stack
// is empty (kLaneDone).  `fold` consumes the frames of its own kind (1), or
// reports a malformed one (2).
template <typename StackT, typename Fold = NoFold>
__device__ __forceinline__ int phase_ascend(const MeshView& m, const Ray& r, StackT stack, Trav& s, bool& bad,
                                            const Fold& fold = Fold{}) {
  const uint32_t num_node = 2 * m.num_tri - 1;
  s.chain_next = kUMax;
  while (s.sp > 0) {
    const uint4 f = stack.load(s.sp - 1);
    const int folded = fold(f, s);
    if (folded == 1) continue;
    if (folded == 2) {
      bad = true;
      return kLaneDone;
    }
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
        return kLaneDone;
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
        return kLaneDone;
      }
      load_record(m.bvhnodes, s.node, s.left, s.right);
      return kLaneInner;
    }
  }
  return kLaneDone;
}

// One node entry and everything up to the next one (the phases back to
// back), for one ray at a time.  On kStepDone the ray's result is s.best.
template <typename StackT>
__device__ __forceinline__ int trav_step(const MeshView& m, const Ray& r, StackT stack, uint32_t cap, Trav& s,
                                         bool& bad) {
  int st = phase_inner(m, r, stack, cap, s, bad);
  if (st == kLaneLeaf) st = phase_leaf(m, r, s, bad);
  if (st == kLaneAscend) st = phase_ascend(m, r, stack, s, bad);
  return st == kLaneInner ? kStepContinue : (st == kLaneOverflow ? kStepOverflow : kStepDone);
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
// Node entries per iteration of the persistent loop.  Measured on GB300
// (2M-triangle torus 1920x1080 cast / 4096-mesh batched cast): 1 step 0.528 / 4.94 ms, 2 steps
// 0.480 / 4.61, 3 steps 0.466 / 4.54, 4 steps 0.469 / 5.33, 6 steps 0.561 / 6.20.
constexpr int kInnerSteps = 3;
constexpr int kDeepRing = 64;  // on-chip frames per ray of the overflow tiers

// A Job maps a work index to (mesh, ray, output slot):
//   uint32_t num_work;                              work indices are 0..num_work-1
//   __device__ void prepare(float* smem) const;    once per block, before __syncthreads
//   __device__ bool fetch(uint32_t w, const float* smem, MeshView& m, Ray& r, uint32_t& out) const;
//                                                   false: w is padding, nothing to do
//   __device__ void write(uint32_t out, const MeshView& m, const Ray& r, const Hit& h) const;

// Thresholds of the phased loop: a phase runs when at least this many lanes
// of the warp wait for it, or when nothing else can run.
struct PhaseMins {
  uint32_t refill, leaf, ascend;
  uint32_t long_steps;  // node entries after which a ray is handed to the warp tier
};

// Persistent warps with per-lane ray refill, run in phases.  Each lane holds
// one ray in a LaneState; per iteration the warp enters up to kInnerSteps
// nodes in every lane that is at a branch, then runs the triangle tests, then the ascents,
// then takes new rays for its idle lanes.  The triangle test, the ascent and
// the refill each happen about once per ray but in some lane nearly every
// iteration, so running them whenever any lane needs one leaves most lanes
// idle through them; waiting until `mins` lanes need one runs each for more
// lanes at once, while the others go on entering nodes.  Once the warp's
// refill finds no more work, a waiting lane would only lengthen the warp's
// longest ray, so from then on every phase runs whenever a lane needs it.
// Every lane still makes the same decisions in the same order, so results do
// not depend on the thresholds.  Rays overflowing the on-chip stack, and
// rays past mins.long_steps node entries at a long chain once the warp's
// work is exhausted, go to ovf_list (their work index) for the warp tier.  kThreads threads per block and kStack on-chip frames per ray
// are tuning choices (Tuning); the register bound (64 registers) keeps 2048
// resident threads per SM.
template <typename Job, int kThreads, int kStack>
__global__ void __launch_bounds__(kThreads, 65536 / (64 * kThreads)) k_cast_persistent(Job job, uint32_t* work_counter,
                                                                                 uint32_t* ovf_list,
                                                                                 uint32_t* ovf_count,
                                                                                 uint32_t* status, PhaseMins mins) {
  __shared__ float smem[64];
  job.prepare(smem);
  __syncthreads();
  constexpr uint32_t kAll = 0xffffffffu;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t lt_mask = (1u << lane) - 1u;
  uint4 frames[kStack];
  LocalStack stack{frames};
  MeshView m{};
  Ray r{};
  Trav s{};
  uint32_t out = 0, work = kUMax;
  int state = kLaneIdle;
  bool exhausted = false, bad = false;
  for (;;) {
    // refill idle lanes with consecutive work indices
    const uint32_t idle = __ballot_sync(kAll, state == kLaneIdle);
    if (idle != 0u && !exhausted && (idle == kAll || static_cast<uint32_t>(__popc(idle)) >= mins.refill)) {
      uint32_t base = 0;
      if (lane == static_cast<uint32_t>(__ffs(idle) - 1)) base = atomicAdd(work_counter, __popc(idle));
      base = __shfl_sync(kAll, base, __ffs(idle) - 1);
      if (base + __popc(idle) >= job.num_work) exhausted = true;  // warp-uniform: no work after this
      if (state == kLaneIdle) {
        const uint32_t w = base + __popc(idle & lt_mask);
        if (w < job.num_work && job.fetch(w, smem, m, r, out)) {
          work = w;
          if (trav_begin(m, r, s)) state = kLaneInner;
          else job.write(out, m, r, s.best);
        }
      }
    }
    if (__all_sync(kAll, state == kLaneIdle)) {
      if (exhausted) break;
      continue;
    }
    const uint32_t leaf_min = exhausted ? 1u : mins.leaf, ascend_min = exhausted ? 1u : mins.ascend;
    // Up to kInnerSteps node entries per iteration: the warp's votes and
    // phase decisions are paid once for several entries, and a lane that
    // leaves the inner phase early waits for the others' entries.
#pragma unroll
    for (int k = 0; k < kInnerSteps; ++k)
      if (state == kLaneInner) state = phase_inner(m, r, stack, kStack, s, bad);
    uint32_t inner = __ballot_sync(kAll, state == kLaneInner);
    const uint32_t leaf = __ballot_sync(kAll, state == kLaneLeaf);
    if (leaf != 0u && (inner == 0u || static_cast<uint32_t>(__popc(leaf)) >= leaf_min)) {
      if (state == kLaneLeaf) state = phase_leaf(m, r, s, bad);
      inner = __ballot_sync(kAll, state == kLaneInner);
    }
    const uint32_t asc = __ballot_sync(kAll, state == kLaneAscend);
    if (asc != 0u && (inner == 0u || static_cast<uint32_t>(__popc(asc)) >= ascend_min)) {
      if (state == kLaneAscend) state = phase_ascend(m, r, stack, s, bad);
    }
    // Once the warp has no more rays to take, a ray past the step budget
    // that is about to enter a long chain would hold the kernel's end: it is
    // handed to the warp tier, which folds chains 32 links at a time.
    if (exhausted && state == kLaneInner && s.steps > mins.long_steps && long_chain_at(m, s.node, s.left, s.right))
      state = kLaneOverflow;
    if (state == kLaneDone) {
      job.write(out, m, r, s.best);
      state = kLaneIdle;
    } else if (state == kLaneOverflow) {
      ovf_list[atomicAdd(ovf_count, 1u)] = work;
      state = kLaneIdle;
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
  pdl_wait();
  pdl_launch_dependents();
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
  uint4 ring[kDeepRing];
  uint32_t lo = 0;
  const RingStack<kDeepRing> st{ring, pool + slot * cap, &lo};
  bool bad = false;
  for (uint64_t k = slot; k < num; k += slots) {
    lo = 0;
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

// ------------------------------------------------------------ warp tier
// Rays that overflowed the persistent cast's stack, or that were about to
// enter a long chain past its step budget once their warp had no more rays to
// take, one warp each.  Every lane runs the same serial traversal on the
// same state (the same loads, the same decisions), except at a chain: a run
// of links, branches j whose left child is leaf j and right child branch
// j + 1 (runs of equal Morton codes build them).  The recursion's result over
// a chain c0..c1 is a fold from its far end: with x = F(c1 + 1), for j = c1
// down to c0
//   x <- g_j(x):  neither child box hit: none;  only leaf j's box: h_j (its hit);
//                 only branch j+1's box: x;  both, the leaf nearer: h_j if h_j
//                 is a hit before branch j+1's entry, else pick(h_j, x);  both,
//                 the branch nearer: x if x is a hit before leaf j's entry,
//                 else pick(x, h_j)
// (the rules of phase_inner / phase_leaf / phase_ascend).  So the warp pushes
// a fold frame, searches the tail c1 + 1 on its own, and on popping the frame
// tests 32 * kFoldBatch links per round (kFoldBatch per lane) and folds them
// with shuffles.
// On the duplicate-heavy soup 96% of the long rays' node entries are links.
constexpr uint32_t kWarpAll = 0xffffffffu;

// The last link of the chain starting at link c0 (the same in every lane),
// 256 records per round (8 per lane: 2.19 ms soup cast, 4 per lane 2.22,
// 1 per lane 2.45).
__device__ __forceinline__ uint32_t chain_last(const MeshView& m, uint32_t c0, uint32_t lane) {
  const uint32_t num_branch = m.num_tri - 1;
  uint32_t last = c0;
  for (;;) {
    // lane l checks links last + 1 + 8 l .. last + 8 l + 8
    bool ok[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const uint32_t j = last + 1 + 8 * lane + q;
      ok[q] = false;
      if (j < num_branch) {
        uint32_t l, r;
        load_record(m.bvhnodes, j, l, r);
        ok[q] = is_link(m, j, l, r);
      }
    }
    uint32_t first_bad = 8;
#pragma unroll
    for (int q = 7; q >= 0; --q)
      if (!ok[q]) first_bad = q;
    const uint32_t fail = __ballot_sync(kWarpAll, first_bad < 8);
    if (fail != 0u) {
      const uint32_t l0 = static_cast<uint32_t>(__ffs(fail)) - 1u;
      const uint32_t fb = __shfl_sync(kWarpAll, first_bad, l0);
      return last + 8 * l0 + fb;
    }
    last += 256;
  }
}

// Folds links hi, hi - 1, .., lo (at most 32 * kFoldBatch) into x.  Lane k
// tests links hi - k - 32 q (q < kFoldBatch), all loads in flight together;
// the warp then applies them in order, four shuffles per link.  One batch
// per round measured fastest on the soup's cast (2.41 ms; 2 and 4 batches:
// 2.62 and 2.61 ms).
constexpr uint32_t kFoldBatch = 1;
__device__ __forceinline__ Hit fold_links(const MeshView& m, const Ray& r, uint32_t lo, uint32_t hi, Hit x,
                                          uint32_t lane, bool& bad) {
  const uint32_t n = hi - lo + 1;
  uint32_t flags[kFoldBatch];  // 1: leaf box hit, 2: branch box hit, 4: the leaf is the near child
  float far_enter[kFoldBatch];
  Hit h[kFoldBatch];
#pragma unroll
  for (uint32_t q = 0; q < kFoldBatch; ++q) {
    flags[q] = 0;
    far_enter[q] = 0.f;
    h[q] = Hit{INFINITY, kUMax};
    const uint32_t i = lane + 32 * q;
    if (i < n) {
      const uint32_t j = hi - i, leaf = m.num_tri - 1 + j;
      float a0 = 0.f, a1 = 0.f, b0 = 0.f, b1 = 0.f;
      const bool ha = node_slab(m, r, leaf, a0, a1);
      const bool hb = node_slab(m, r, j + 1, b0, b1);
      const bool near_leaf = (ha && hb) ? tuple_lt(a0, a1, b0, b1) : ha;
      flags[q] = (ha ? 1u : 0u) | (hb ? 2u : 0u) | (near_leaf ? 4u : 0u);
      far_enter[q] = near_leaf ? b0 : a0;
      if (ha) {
        const uint32_t tri = __ldg(m.bvhnodes + static_cast<size_t>(leaf) * 3 + 1);
        float t, u, v;
        if (leaf_hit(m, r, tri, t, u, v, bad)) h[q] = Hit{t, tri};
      }
    }
  }
#pragma unroll
  for (uint32_t q = 0; q < kFoldBatch; ++q) {
    for (uint32_t k = 0; k < 32 && 32 * q + k < n; ++k) {
      const uint32_t f = __shfl_sync(kWarpAll, flags[q], k);
      const float fe = __shfl_sync(kWarpAll, far_enter[q], k);
      const Hit kh{__shfl_sync(kWarpAll, h[q].t, k), __shfl_sync(kWarpAll, h[q].id, k)};
      if ((f & 3u) == 0u) {
        x = Hit{INFINITY, kUMax};
      } else if ((f & 3u) == 1u) {
        x = kh;
      } else if ((f & 3u) == 3u) {
        if (f & 4u) x = (kh.id != kUMax && fe > kh.t) ? kh : pick(kh, x);
        else x = (x.id != kUMax && fe > x.t) ? x : pick(x, kh);
      }
    }
  }
  return x;
}

// phase_inner, except that a branch starting a chain of at least kFoldMin
// links pushes a fold frame {c0 | bit, c1 | bit, saved} and searches the
// chain's tail (if its box is hit) with a fresh result.
template <typename StackT>
__device__ __forceinline__ int phase_inner_warp(const MeshView& m, const Ray& r, StackT stack, uint32_t cap, Trav& s,
                                                bool& bad, uint32_t lane) {
  if (s.right != kUMax && is_link(m, s.node, s.left, s.right)) {
    const uint32_t c0 = s.node, c1 = chain_last(m, c0, lane);
    if (c1 - c0 + 1 >= kFoldMin) {
      s.steps += 2 * (c1 - c0 + 1);  // its branches and leaves
      if (s.steps > 2 * m.num_tri) {
        bad = true;
        return kLaneDone;
      }
      if (s.sp >= cap) return kLaneOverflow;
      stack.store(s.sp++, make_uint4(kChainBit | c0, kChainBit | c1, __float_as_uint(s.best.t), s.best.id));
      s.best = Hit{INFINITY, kUMax};
      s.chain_next = kUMax;
      const uint32_t tail = c1 + 1;
      float te, tx;
      if (!node_slab(m, r, tail, te, tx)) return kLaneAscend;  // the fold ignores the tail
      s.node = tail;
      load_record(m.bvhnodes, tail, s.left, s.right);
      return kLaneInner;
    }
  }
  return phase_inner(m, r, stack, cap, s, bad);
}

constexpr uint32_t kChainPrefetch = 2;  // chunks of links prefetched ahead of the fold

// Fold frames {c0 | bit, c1 | bit, saved}: the tail's result (the current
// one) is folded through the chain, and the chain's result into `saved`.
struct ChainFold {
  const MeshView& m;
  const Ray& r;
  uint32_t lane;
  bool* bad;
  __device__ __forceinline__ int operator()(const uint4& f, Trav& s) const {
    if (!((f.x & kChainBit) && (f.y & kChainBit))) return 0;
    const uint32_t c0 = f.x & ~kChainBit, c1 = f.y & ~kChainBit;
    if (c0 > c1 || c1 + 1 >= 2 * m.num_tri - 1) return 2;
    Hit x = s.best;
    const uint32_t nb = m.num_tri - 1;
    for (uint32_t hi = c1;;) {
      const uint32_t lo = hi - c0 >= 32 * kFoldBatch - 1 ? hi - (32 * kFoldBatch - 1) : c0;
      // the links of the next kChainPrefetch chunks (lane k: one link each)
      // toward L2 while this chunk is folded: a long chain's tree does not
      // fit L2, and each chunk is otherwise a few dependent DRAM round trips
#pragma unroll
      for (uint32_t d = 0; d < kChainPrefetch; ++d) {
        const int64_t j = static_cast<int64_t>(lo) - 1 - lane - 32 * static_cast<int64_t>(d);
        if (j >= static_cast<int64_t>(c0)) {
          asm volatile("prefetch.global.L2 [%0];" ::"l"(m.bvhnodes + 3 * (nb + static_cast<uint64_t>(j))));
          asm volatile("prefetch.global.L2 [%0];" ::"l"(m.aabb + 6 * (nb + static_cast<uint64_t>(j))));
          asm volatile("prefetch.global.L2 [%0];" ::"l"(m.aabb + 6 * (static_cast<uint64_t>(j) + 1)));
        }
      }
      x = fold_links(m, r, lo, hi, x, lane, *bad);
      if (lo == c0) break;
      hi = lo - 1;
    }
    --s.sp;
    s.best = pick(Hit{__uint_as_float(f.z), f.w}, x);
    return 1;
  }
};

template <typename StackT>
__device__ __forceinline__ int trav_step_warp(const MeshView& m, const Ray& r, StackT stack, uint32_t cap, Trav& s,
                                              bool& bad, uint32_t lane) {
  int st = phase_inner_warp(m, r, stack, cap, s, bad, lane);
  if (st == kLaneLeaf) st = phase_leaf(m, r, s, bad);
  if (st == kLaneAscend) st = phase_ascend(m, r, stack, s, bad, ChainFold{m, r, lane, &bad});
  return st == kLaneInner ? kStepContinue : (st == kLaneOverflow ? kStepOverflow : kStepDone);
}

// One warp per ray of list_in; a ray whose frames outgrow the warp's slice of
// the pool goes to list_out.  Every lane keeps the same stack (the ring in its
// own local memory, the spilled frames at the same addresses of the slice).
template <typename Job>
__global__ void __launch_bounds__(kCastThreads, 4) k_cast_warp(Job job, const uint32_t* list_in, const uint32_t* count_in,
                                                           uint32_t* list_out, uint32_t* count_out, uint4* pool,
                                                           uint64_t pool_frames, uint32_t max_tri, uint32_t* status) {
  __shared__ float smem[64];
  job.prepare(smem);
  pdl_wait();
  pdl_launch_dependents();
  __syncthreads();
  const uint32_t num = *count_in;
  if (num == 0) return;
  constexpr uint32_t kWarps = kCastThreads / 32;
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t warps = static_cast<uint64_t>(gridDim.x) * kWarps;
  const uint64_t wid = static_cast<uint64_t>(blockIdx.x) * kWarps + threadIdx.x / 32;
  uint64_t cap = pool_frames / warps;
  if (cap > 2ull * max_tri) cap = 2ull * max_tri;
  uint4 ring[kDeepRing];
  uint32_t lo = 0;
  const RingStack<kDeepRing> st{ring, pool + wid * cap, &lo};
  bool bad = false;
  for (uint64_t k = wid; k < num; k += warps) {
    lo = 0;
    const uint32_t w = list_in[k];
    MeshView m{};
    Ray r{};
    uint32_t out = 0;
    if (!job.fetch(w, smem, m, r, out)) continue;
    Trav s{};
    int rc = kStepDone;
    if (trav_begin(m, r, s)) {
      do {
        rc = trav_step_warp(m, r, st, static_cast<uint32_t>(cap), s, bad, lane);
      } while (rc == kStepContinue);
    }
    if (lane == 0) {
      if (rc == kStepDone) job.write(out, m, r, s.best);
      else list_out[atomicAdd(count_out, 1u)] = w;
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
  const Tuning t = get_tuning();
  const PhaseMins mins{t.cast_refill_min, t.cast_leaf_min, t.cast_ascend_min, t.cast_long_steps};
  k_cast_persistent<Job, kThreads, kStack><<<grid, kThreads, 0, s>>>(job, sc.counters, sc.list1, sc.counters + 1,
                                                                     status, mins);
}

// The tiered cast of every work index of `job`: the persistent cast; the
// warp tier for the rays it hands over; for the rare ray whose frames outgrow
// a warp's slice, the serial tier with the pool split over those rays, then
// with unbounded frames.  sc.counters (4 words) must be zero on entry: [0]
// work counter, [1..3] the hand-over counts of tiers 1..3 (lists list1,
// list2, list1 again).  The first tier's block size and on-chip stack depth
// come from the current Tuning (kCastVariants lists the choices).
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
  launch_pdl(k_cast_warp<Job>, dim3(deep_grid), dim3(kCastThreads), 0, s, job, sc.list1, sc.counters + 1, sc.list2,
             sc.counters + 2, pool, pool_frames, max_tri, status);
  launch_pdl(k_cast_deep<Job>, dim3(deep_grid), dim3(kCastThreads), 0, s, job, sc.list2, sc.counters + 2, sc.list1,
             sc.counters + 3, pool, pool_frames, 0u, max_tri, status);
  const uint32_t cap3 = max_tri < 2 ? 2u : max_tri;
  launch_pdl(k_cast_deep<Job>, dim3(deep_grid), dim3(kCastThreads), 0, s, job, sc.list1, sc.counters + 3,
             static_cast<uint32_t*>(nullptr), static_cast<uint32_t*>(nullptr), pool, pool_frames, cap3, max_tri,
             status);
}

}  // namespace dm
