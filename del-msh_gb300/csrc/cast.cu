// cast.cu — closest-hit ray casting against an LBVH in del-msh's layout
// (bvhnodes u32[(2T-1)*3] = [parent, left, right], bvhnode2aabb f32[(2T-1)*6]).
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
// A frame is pushed only when descending into an internal near child; it
// holds the far child, its slab entry, and the result accumulated so far at
// the enclosing level ("saved"), and the accumulator restarts empty so that
// when the near subtree is finished the accumulator equals R(near) exactly —
// the value the far-child test of search_bvh3.rs:168-189 needs.  A leaf near
// child is resolved inline without a frame, and a far child that must be
// searched continues in the enclosing level after folding R(near) into
// "saved", so one frame per level with an internal near child suffices.
//
// Stack tiers.  Frames live in a 64-entry on-chip (local) stack.  A ray that
// needs more is appended to an overflow list and re-cast from scratch by a
// second kernel whose per-ray stacks are carved from a global pool (capacity
// chosen on the device from the overflow count), and anything still deeper by
// a third kernel with capacity num_tri, which no tree can exceed.  Duplicate
// Morton codes produce long chains (a run of k equal codes is a chain of
// height k), which is where the deeper tiers are used.
#include "dm_device.cuh"
#include "dm_internal.h"

namespace dm {
namespace {

constexpr uint32_t kFarMissBit = 0x80000000u;

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

// Returns false when the stack capacity was exceeded (result undefined).  A
// malformed tree (child index out of range, or more node visits than a tree
// allows) ends the ray as a miss and sets `bad`.
template <typename StackT>
__device__ bool traverse(const MeshView& m, const Ray& r, StackT stack, uint32_t cap, Hit& out, bool& bad) {
  Hit best{INFINITY, kUMax};
  float te, tx;
  out = best;
  if (!node_slab(m, r, 0, te, tx)) return true;
  const uint32_t* __restrict__ bn = m.bvhnodes;
  const uint32_t num_node = 2 * m.num_tri - 1;
  uint64_t budget = 2ull * num_node + 2;  // every node is entered at most once per ray
  uint32_t node = 0;
  uint32_t sp = 0;
  for (;;) {
    if (--budget == 0) {
      bad = true;
      return true;
    }
    bool ascend = false;
    const uint32_t right = __ldg(bn + static_cast<size_t>(node) * 3 + 2);
    if (right == kUMax) {  // a leaf reached as the root or as a far child
      const uint32_t it = __ldg(bn + static_cast<size_t>(node) * 3 + 1);
      float t, u, v;
      if (leaf_hit(m, r, it, t, u, v, bad)) best = pick(best, Hit{t, it});
      ascend = true;
    } else {
      const uint32_t left = __ldg(bn + static_cast<size_t>(node) * 3 + 1);
      if (left >= num_node || right >= num_node) {
        bad = true;
        return true;
      }
      float l0 = 0.f, l1 = 0.f, r0 = 0.f, r1 = 0.f;
      const bool hl = node_slab(m, r, left, l0, l1);
      const bool hr = node_slab(m, r, right, r0, r1);
      if (!hl && !hr) {
        ascend = true;
      } else {
        const bool near_left = (hl && hr) ? tuple_lt(l0, l1, r0, r1) : hl;
        const uint32_t nn = near_left ? left : right;
        const uint32_t nf = near_left ? right : left;
        const bool has_far = near_left ? hr : hl;
        const float far_enter = near_left ? r0 : l0;
        if (__ldg(bn + static_cast<size_t>(nn) * 3 + 2) == kUMax) {  // near child is a leaf
          const uint32_t it = __ldg(bn + static_cast<size_t>(nn) * 3 + 1);
          float t, u, v;
          const bool h = leaf_hit(m, r, it, t, u, v, bad);
          if (h) best = pick(best, Hit{t, it});
          if (!has_far || (h && far_enter > t)) ascend = true;
          else node = nf;
        } else {
          if (sp >= cap) return false;
          stack.store(sp++, make_uint4(has_far ? nf : (nf | kFarMissBit), __float_as_uint(far_enter),
                                       __float_as_uint(best.t), best.id));
          best = Hit{INFINITY, kUMax};
          node = nn;
        }
      }
    }
    if (ascend) {
      bool resumed = false;
      while (sp > 0) {
        const uint4 f = stack.load(--sp);
        const Hit saved{__uint_as_float(f.z), f.w};
        const bool has_far = (f.x & kFarMissBit) == 0u;
        const bool skip = (best.id != kUMax) ? (!has_far || __uint_as_float(f.y) > best.t) : !has_far;
        best = pick(saved, best);
        if (!skip) {
          node = f.x & ~kFarMissBit;
          resumed = true;
          break;
        }
      }
      if (!resumed) break;
    }
  }
  out = best;
  return true;
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

struct RaySource {
  // pixels (ray_for_pixel.h) when ray_org == nullptr
  uint32_t img_w, img_h;
  const float* t_ndc2world;
  const float* ray_org;
  const float* ray_dir;
};

__device__ __forceinline__ Ray load_ray(const RaySource& src, const float* m_smem, uint32_t i) {
  float3 o, d;
  if (src.ray_org == nullptr) {
    ray_for_pixel(i, src.img_w, src.img_h, m_smem, o, d);
  } else {
    const float* po = src.ray_org + static_cast<size_t>(i) * 3;
    const float* pd = src.ray_dir + static_cast<size_t>(i) * 3;
    o = make_float3(__ldg(po), __ldg(po + 1), __ldg(po + 2));
    d = make_float3(__ldg(pd), __ldg(pd + 1), __ldg(pd + 2));
  }
  return make_ray(o, d);
}

__device__ __forceinline__ void write_hit(const CastOut& o, const MeshView& m, const Ray& r, uint32_t i, const Hit& h) {
  o.hit_tri[i] = h.id;
  if (o.hit_t) o.hit_t[i] = h.t;
  if (o.hit_bc) {
    float bc0 = 0.f, bc1 = 0.f, bc2 = 0.f;
    if (h.id != kUMax) {
      float t, u, v;
      bool bad = false;
      if (leaf_hit(m, r, h.id, t, u, v, bad)) {
        bc0 = __fsub_rn(__fsub_rn(1.0f, u), v);
        bc1 = u;
        bc2 = v;
      }
    }
    o.hit_bc[static_cast<size_t>(i) * 3] = bc0;
    o.hit_bc[static_cast<size_t>(i) * 3 + 1] = bc1;
    o.hit_bc[static_cast<size_t>(i) * 3 + 2] = bc2;
  }
}

constexpr int kCastThreads = 128;

__global__ void __launch_bounds__(kCastThreads) k_cast(uint32_t num_ray, RaySource src, MeshView m, CastOut o,
                                                      uint32_t* ovf_list, uint32_t* ovf_count, uint32_t* status) {
  __shared__ float mat[16];
  if (src.ray_org == nullptr && threadIdx.x < 16) mat[threadIdx.x] = src.t_ndc2world[threadIdx.x];
  __syncthreads();
  const uint32_t i = blockIdx.x * kCastThreads + threadIdx.x;
  if (i >= num_ray) return;
  const Ray r = load_ray(src, mat, i);
  uint4 frames[kCastStack];
  Hit h;
  bool bad = false;
  if (traverse(m, r, LocalStack{frames}, kCastStack, h, bad)) {
    write_hit(o, m, r, i, h);
  } else {
    ovf_list[atomicAdd(ovf_count, 1u)] = i;
  }
  if (bad) raise_status(status, kStatusBadIndex);
}

// Re-casts the rays of list_in with stacks carved from the pool.  cap_fixed
// == 0 chooses the capacity from the number of rays to process.
__global__ void __launch_bounds__(kCastThreads) k_cast_deep(RaySource src, MeshView m, CastOut o,
                                                           const uint32_t* list_in, const uint32_t* count_in,
                                                           uint32_t* list_out, uint32_t* count_out, uint4* pool,
                                                           uint64_t pool_frames, uint32_t cap_fixed,
                                                           uint32_t* status) {
  __shared__ float mat[16];
  if (src.ray_org == nullptr && threadIdx.x < 16) mat[threadIdx.x] = src.t_ndc2world[threadIdx.x];
  __syncthreads();
  const uint32_t num = *count_in;
  if (num == 0) return;
  uint64_t cap = cap_fixed;
  if (cap == 0) {
    cap = pool_frames / num;
    if (cap < 256) cap = 256;
    const uint64_t cap_max = 2ull * m.num_tri;  // never more than the deepest possible tree needs
    if (cap > cap_max) cap = cap_max;
  }
  if (cap > pool_frames) cap = pool_frames;
  const uint64_t threads = static_cast<uint64_t>(gridDim.x) * kCastThreads;
  uint64_t slots = pool_frames / cap;
  if (slots > threads) slots = threads;
  // spread the active slots over all blocks
  const uint64_t slot = static_cast<uint64_t>(threadIdx.x) * gridDim.x + blockIdx.x;
  if (slot >= slots) return;
  GlobalStack st{pool + slot * cap};
  for (uint64_t k = slot; k < num; k += slots) {
    const uint32_t i = list_in[k];
    const Ray r = load_ray(src, mat, i);
    Hit h;
    bool bad = false;
    const bool done = traverse(m, r, st, static_cast<uint32_t>(cap), h, bad);
    if (bad) raise_status(status, kStatusBadIndex);
    if (done) {
      write_hit(o, m, r, i, h);
    } else if (list_out) {
      list_out[atomicAdd(count_out, 1u)] = i;
    } else {
      raise_status(status, kStatusStackOverflow);
      o.hit_tri[i] = kUMax;
    }
  }
}

void cast_all(cudaStream_t s, uint32_t num_ray, const RaySource& src, const MeshView& m, const CastOut& o,
              const CastScratch& sc, uint32_t* status) {
  if (num_ray == 0) return;
  const uint32_t grid = (num_ray + kCastThreads - 1) / kCastThreads;
  k_cast<<<grid, kCastThreads, 0, s>>>(num_ray, src, m, o, sc.list1, sc.counters, status);
  const uint64_t pool_frames = sc.pool_bytes / kFrameBytes;
  uint4* pool = static_cast<uint4*>(sc.pool);
  const uint32_t deep_grid = 152 * 4;
  k_cast_deep<<<deep_grid, kCastThreads, 0, s>>>(src, m, o, sc.list1, sc.counters, sc.list2, sc.counters + 1, pool,
                                                 pool_frames, 0u, status);
  const uint32_t cap3 = m.num_tri < 2 ? 2u : m.num_tri;
  k_cast_deep<<<deep_grid, kCastThreads, 0, s>>>(src, m, o, sc.list2, sc.counters + 1, nullptr, nullptr, pool,
                                                 pool_frames, cap3, status);
}

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace

size_t cast_scratch_bytes(uint32_t num_ray, uint32_t num_tri) {
  const size_t lists = align_up(static_cast<size_t>(num_ray) * 4, 256) * 2;
  const uint64_t frames = num_tri < 4096 ? 4096 : num_tri;
  size_t pool = frames * kFrameBytes;
  if (pool < (size_t{64} << 20)) pool = size_t{64} << 20;
  return 256 + lists + pool;
}

void cast_scratch_carve(void* base, uint32_t num_ray, uint32_t num_tri, CastScratch* out) {
  char* p = static_cast<char*>(base);
  out->counters = reinterpret_cast<uint32_t*>(p);
  p += 256;
  const size_t lst = align_up(static_cast<size_t>(num_ray) * 4, 256);
  out->list1 = reinterpret_cast<uint32_t*>(p);
  p += lst;
  out->list2 = reinterpret_cast<uint32_t*>(p);
  p += lst;
  out->pool = p;
  out->pool_bytes = cast_scratch_bytes(num_ray, num_tri) - 256 - 2 * lst;
}

void launch_cast_pixels(cudaStream_t s, uint32_t img_w, uint32_t img_h, const float* t_ndc2world, const MeshView& m,
                        const CastOut& o, const CastScratch& sc, uint32_t* status) {
  RaySource src{img_w, img_h, t_ndc2world, nullptr, nullptr};
  cast_all(s, img_w * img_h, src, m, o, sc, status);
}

void launch_cast_rays(cudaStream_t s, uint32_t num_ray, const float* ray_org, const float* ray_dir,
                      const MeshView& m, const CastOut& o, const CastScratch& sc, uint32_t* status) {
  RaySource src{0, 0, nullptr, ray_org, ray_dir};
  cast_all(s, num_ray, src, m, o, sc, status);
}

}  // namespace dm
