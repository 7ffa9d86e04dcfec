// front.cu — the front of the single-mesh build in one cooperative launch:
// triangle centroids, their AABB and the fit transform, 30-bit Morton codes
// and the four stable 8-bit LSD passes of the sort (with ties kept in
// triangle order, mortons.rs:139-146), for meshes whose tiles can all be
// resident on the GPU at once (about 2.5M triangles on GB300).
//
// Why one launch.  At these sizes every tile of a pass runs in the same wave,
// and a decoupled look-back then walks each tile back through its
// predecessors' aggregates a few at a time: measured on GB300, the last of
// 256 co-resident tiles finished its look-back ~8 us after the first, most of
// a 16 us pass.  Here the tiles publish their digit counts, a grid barrier
// follows, one warp per digit scans that digit's counts over the tiles
// (exclusive prefix per tile, and the digit's total), a second barrier
// follows, and every tile then knows its output offsets at once.  The same
// barriers let the centroids stay in shared memory between the AABB pass and
// the Morton codes, and the codes stay in registers into the first pass, so
// neither is written to memory and read back.
//
// Values and order of operations are those of the separate kernels it
// replaces (k_centroid_aabb, k_morton_tri, the onesweep passes): the same
// centroid sums, NaN-aware min/max, fit transform, transform_homogeneous and
// morton_code3; each pass is stable (input order within a digit), so the
// permutation is del-msh-cpu's sort_by_key over the iota.
//
// Every grid-barrier wait is bounded by the process-wide wait limit; a wait
// that gives up raises kStatusSpinTimeout and the kernel runs on (its output
// is then garbage, but nothing hangs).  Co-residency of all blocks is
// guaranteed by the cooperative launch, which is refused when the grid does
// not fit; the caller then takes the separate-kernel path.
#include <cuda/atomic>

#include "dm_device.cuh"
#include "dm_internal.h"

namespace dm {
namespace {

constexpr int kFThreads = 512;
constexpr int kFWarps = kFThreads / 32;
constexpr int kFRadix = 256;

struct FMinMax {
  float lo[3], hi[3];
};

template <int kKpt>
struct FrontSmem {
  static constexpr int kTile = kFThreads * kKpt;
  struct Sort {
    uint16_t whist[kFWarps][kFRadix];  // per-warp running counts, then per-warp exclusive offsets
    uint32_t match[kFWarps][kFRadix];  // peer masks of the rank step; zero between steps
    uint16_t rank[kTile];              // each key's rank among its warp's keys of its digit
    uint32_t keys[kTile];
    uint32_t vals[kTile];
  };
  union {
    Sort s;
    float cent[3][kTile];  // phase 0: the tile's centroids (x, y, z)
  } u;
  uint32_t tstart[kFRadix];  // start of each digit inside the tile
  uint32_t offs[kFRadix];    // output position minus tile slot, per digit
  uint32_t scan[kFWarps];
  FMinMax mm[kFWarps];
  float m[16];  // the fit transform
  uint32_t diag;  // the transform is diagonal plus translation
  uint32_t lut[1024];  // expand_bits3 of every 10-bit value
};

struct FrontArgs {
  uint32_t num_tri, num_vtx;
  const uint32_t* tri2vtx;
  const float* vtx2xyz;
  float* tribox;         // per-triangle boxes (triangle soups) or nullptr
  float* partials;       // [grid][6] AABB partials
  float* transform_out;  // 16 floats, written by block 0
  float* aabb_out;       // 6 floats or nullptr
  uint32_t* tri2morton;  // codes in triangle order, or nullptr
  uint32_t *ka, *va, *kb, *vb;       // ping-pong buffers, num_tri words each
  uint32_t *out_keys, *out_vals;     // sorted codes and triangle indices (not ka / va)
  uint32_t* counts;      // [256][grid]: per-tile digit counts, then exclusive prefixes
  uint32_t* totals;      // [256]: per-digit totals of the current pass
  uint32_t* bar;         // grid-barrier counter, zero at launch
  uint32_t* status;
  uint32_t spin_limit;
};

__device__ __forceinline__ void mm_merge(FMinMax& a, const FMinMax& b) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (b.lo[d] < a.lo[d]) a.lo[d] = b.lo[d];
    if (b.hi[d] > a.hi[d]) a.hi[d] = b.hi[d];
  }
}

__device__ __forceinline__ FMinMax mm_identity() {
  FMinMax v;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    v.lo[d] = INFINITY;
    v.hi[d] = -INFINITY;
  }
  return v;
}

__device__ __forceinline__ FMinMax mm_shfl_down(const FMinMax& v, int off) {
  FMinMax o;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    o.lo[d] = __shfl_down_sync(0xffffffffu, v.lo[d], off);
    o.hi[d] = __shfl_down_sync(0xffffffffu, v.hi[d], off);
  }
  return o;
}

// (min, max) over the block; NaN is ignored (every comparison with it is
// false).  Valid in thread 0; has __syncthreads.
__device__ __forceinline__ FMinMax block_reduce_mm512(FMinMax v, FMinMax* sh) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) mm_merge(v, mm_shfl_down(v, off));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  if (warp == 0) {
    FMinMax w = lane < kFWarps ? sh[lane] : mm_identity();
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) mm_merge(w, mm_shfl_down(w, off));
    v = w;
  }
  __syncthreads();
  return v;
}

// Exclusive scan over the block of one value per thread; has __syncthreads.
__device__ __forceinline__ uint32_t block_exclusive_scan512(uint32_t v, uint32_t* s_warp) {
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
    uint32_t w = lane < kFWarps ? s_warp[lane] : 0u;
#pragma unroll
    for (int off = 1; off < kFWarps; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, off);
      if (lane >= off) w += y;
    }
    if (lane < kFWarps) s_warp[lane] = w;
  }
  __syncthreads();
  const uint32_t r = (warp > 0 ? s_warp[warp - 1] : 0u) + x - v;
  __syncthreads();
  return r;
}

// All blocks of the (cooperative) grid arrive, then wait until the counter
// reaches epoch * gridDim.x.  The arrival is a release add by thread 0 after
// the block barrier (cumulative over the block's writes) and the wait an
// acquire load, which orders every block's writes before the barrier with
// every block's reads after it; no separate fences (measured on GB300: the
// 2M front 116.8 -> 112.5 us).  The wait is bounded.
__device__ __forceinline__ void grid_barrier(uint32_t* bar, uint32_t& epoch, uint32_t* status, uint32_t spin_limit) {
  __syncthreads();
  ++epoch;
  if (threadIdx.x == 0) {
    cuda::atomic_ref<uint32_t, cuda::thread_scope_device> b(*bar);
    b.fetch_add(1u, cuda::memory_order_release);
    const uint32_t target = epoch * gridDim.x;
    uint32_t spins = 0;
    while (b.load(cuda::memory_order_acquire) < target) {
      if (++spins > spin_limit) {
        raise_status(status, kStatusSpinTimeout);
        break;
      }
      __nanosleep(20);
    }
  }
  __syncthreads();
}

template <int kKpt, bool kBox>
__global__ void __launch_bounds__(kFThreads, 2) k_build_front(FrontArgs a) {
  static_assert(kKpt % 4 == 0, "keys per thread: a multiple of 4");
  static_assert(kFThreads * kKpt <= 65536, "ranks and per-warp offsets are 16-bit");
  using Smem = FrontSmem<kKpt>;
  constexpr int kTile = Smem::kTile;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem& S = *reinterpret_cast<Smem*>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t T = a.num_tri, nt = gridDim.x, tile = blockIdx.x;
  const uint32_t tile_base = tile * kTile;
  const uint32_t tile_n = (T - tile_base) < static_cast<uint32_t>(kTile) ? (T - tile_base) : kTile;
  uint32_t epoch = 0;
  for (int i = tid; i < 1024; i += kFThreads) S.lut[i] = expand_bits3(static_cast<uint32_t>(i));

  // ---- phase 0: centroids (kept in shared memory), the tile's AABB partial.
  // A thread takes 4 consecutive triangles at a time: their 12 vertex indices
  // are 3 uint4 loads (the tile starts at a multiple of 4 triangles), then
  // the 36 vertex coordinates are gathered together.
  {
    FMinMax v = mm_identity();
    const bool vec = (reinterpret_cast<uintptr_t>(a.tri2vtx) & 15u) == 0u;
    for (uint32_t q = 4u * tid; q < tile_n; q += 4u * kFThreads) {
      const uint32_t i0 = tile_base + q;
      uint32_t idx[12];
      if (vec && q + 4 <= tile_n) {
        const uint4* t4 = reinterpret_cast<const uint4*>(a.tri2vtx + 3ull * i0);
        const uint4 x = __ldg(t4), y = __ldg(t4 + 1), z = __ldg(t4 + 2);
        idx[0] = x.x; idx[1] = x.y; idx[2] = x.z; idx[3] = x.w;
        idx[4] = y.x; idx[5] = y.y; idx[6] = y.z; idx[7] = y.w;
        idx[8] = z.x; idx[9] = z.y; idx[10] = z.z; idx[11] = z.w;
      } else {
#pragma unroll
        for (int k = 0; k < 12; ++k) idx[k] = (q + k / 3 < tile_n) ? __ldg(a.tri2vtx + 3ull * i0 + k) : 0u;
      }
#pragma unroll
      for (int k = 0; k < 12; ++k) {
        if (idx[k] >= a.num_vtx) {  // out of range: vertex 0, as vtx_index does
          if (q + k / 3 < tile_n) raise_status(a.status, kStatusBadIndex);
          idx[k] = 0u;
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (q + u >= tile_n) break;
        const float3 p0 = load_vtx(a.vtx2xyz, idx[3 * u]);
        const float3 p1 = load_vtx(a.vtx2xyz, idx[3 * u + 1]);
        const float3 p2 = load_vtx(a.vtx2xyz, idx[3 * u + 2]);
        const float3 c = make_float3(centroid1(p0.x, p1.x, p2.x), centroid1(p0.y, p1.y, p2.y),
                                     centroid1(p0.z, p1.z, p2.z));
        if constexpr (kBox) {
          Box tb;
          box_set(tb, p0, 0.0f);
          box_add(tb, p1, 0.0f);
          box_add(tb, p2, 0.0f);
          box_store(a.tribox + 6ull * (i0 + u), tb);
        }
        S.u.cent[0][q + u] = c.x;
        S.u.cent[1][q + u] = c.y;
        S.u.cent[2][q + u] = c.z;
        const float cc[3] = {c.x, c.y, c.z};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          if (cc[d] < v.lo[d]) v.lo[d] = cc[d];
          const float h = __fadd_rn(cc[d], 0.0f);
          if (h > v.hi[d]) v.hi[d] = h;
        }
      }
    }
    v = block_reduce_mm512(v, S.mm);
    if (tid == 0) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        a.partials[6 * tile + d] = v.lo[d];
        a.partials[6 * tile + 3 + d] = v.hi[d];
      }
    }
  }
  // the first centroid decides which components are NaN (read before the
  // barrier, so its gathers overlap the wait)
  float3 c0 = make_float3(0.f, 0.f, 0.f);
  if (tid == 0) c0 = tri_centroid(a.tri2vtx, a.num_vtx, a.vtx2xyz, 0, a.status);
  grid_barrier(a.bar, epoch, a.status, a.spin_limit);
  // Every block reduces all partials and computes the same transform
  // (vtx2xyz.rs:19-37 on the centroids, then Mat44/torch.py:120-140): a
  // component is NaN iff the first centroid's is, and otherwise the min / max
  // over the non-NaN values.
  {
    FMinMax v = mm_identity();
    for (uint32_t b = tid; b < nt; b += kFThreads) {
      FMinMax o;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        o.lo[d] = __ldcg(a.partials + 6 * b + d);
        o.hi[d] = __ldcg(a.partials + 6 * b + 3 + d);
      }
      mm_merge(v, o);
    }
    v = block_reduce_mm512(v, S.mm);
    if (tid == 0) {
      const float c0a[3] = {c0.x, c0.y, c0.z};
      float lo[3], hi[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const bool nan0 = c0a[d] != c0a[d];
        lo[d] = nan0 ? c0a[d] : v.lo[d];
        hi[d] = nan0 ? c0a[d] : v.hi[d];
      }
      float ext = __fsub_rn(hi[0], lo[0]);
      const float ey = __fsub_rn(hi[1], lo[1]), ez = __fsub_rn(hi[2], lo[2]);
      if (ey > ext) ext = ey;
      if (ez > ext) ext = ez;
      const float s = __fdiv_rn(1.0f, ext);
#pragma unroll
      for (int k = 0; k < 16; ++k) S.m[k] = 0.0f;
      S.m[0] = s;
      S.m[5] = s;
      S.m[10] = s;
      S.m[15] = 1.0f;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float c = __fmul_rn(__fadd_rn(lo[d], hi[d]), 0.5f);
        S.m[12 + d] = __fadd_rn(__fmul_rn(-c, s), 0.5f);
      }
      S.diag = S.m[1] == 0.0f && S.m[2] == 0.0f && S.m[3] == 0.0f && S.m[4] == 0.0f && S.m[6] == 0.0f &&
               S.m[7] == 0.0f && S.m[8] == 0.0f && S.m[9] == 0.0f && S.m[11] == 0.0f && S.m[15] == 1.0f;
      if (tile == 0) {
#pragma unroll
        for (int k = 0; k < 16; ++k) a.transform_out[k] = S.m[k];
        if (a.aabb_out) {
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            a.aabb_out[d] = lo[d];
            a.aabb_out[d + 3] = hi[d];
          }
        }
      }
    }
    __syncthreads();
  }

  // ---- phase 1: Morton codes of the tile (warp-striped: key j of a lane is
  // local triangle warp*32*kKpt + 32 j + lane, so (j, lane) is input order)
  const uint32_t wloc = static_cast<uint32_t>(warp) * 32u * kKpt;
  {
    uint32_t codes[kKpt];
#pragma unroll
    for (int j = 0; j < kKpt; ++j) {
      const uint32_t k = wloc + 32u * j + lane;
      codes[j] = 0u;
      if (k < tile_n) {
        const float x = S.u.cent[0][k], y = S.u.cent[1][k], z = S.u.cent[2][k];
        float3 q;
        if (S.diag && isfinite(x) && isfinite(y) && isfinite(z)) {
          // the other terms of each row are zeros (0 * finite) and w is 1:
          // they can change only the sign of a zero sum, which quantizes to
          // the same cell
          q = make_float3(__fadd_rn(__fmul_rn(S.m[0], x), S.m[12]), __fadd_rn(__fmul_rn(S.m[5], y), S.m[13]),
                          __fadd_rn(__fmul_rn(S.m[10], z), S.m[14]));
        } else {
          q = transform_homogeneous_w1(S.m, x, y, z);
        }
        codes[j] = S.lut[quantize(__fmul_rn(q.x, 1024.0f), 1023.0f)] * 4u +
                   S.lut[quantize(__fmul_rn(q.y, 1024.0f), 1023.0f)] * 2u +
                   S.lut[quantize(__fmul_rn(q.z, 1024.0f), 1023.0f)];
        if (a.tri2morton) a.tri2morton[tile_base + k] = codes[j];
      }
    }
    __syncthreads();  // the centroids are dead: their space becomes the sort's
    // the codes wait in the key area, in input order, for the first pass
#pragma unroll
    for (int j = 0; j < kKpt; ++j) S.u.s.keys[wloc + 32u * j + lane] = codes[j];
  }

  // ---- the four stable 8-bit passes: computed -> A -> B -> A -> out
  const uint32_t lt_mask = (1u << lane) - 1u;
#pragma unroll 1
  for (int p = 0; p < 4; ++p) {
    const uint32_t shift = 8u * p;
    const uint32_t* kin = p == 2 ? a.kb : a.ka;
    const uint32_t* vin = p == 2 ? a.vb : a.va;
    uint32_t* kout = p == 3 ? a.out_keys : (p == 1 ? a.kb : a.ka);
    uint32_t* vout = p == 3 ? a.out_vals : (p == 1 ? a.vb : a.va);
    uint32_t keys[kKpt];
#pragma unroll
    for (int j = 0; j < kKpt; ++j) {
      const uint32_t k = wloc + 32u * j + lane;
      keys[j] = p == 0 ? S.u.s.keys[k] : (k < tile_n ? __ldcg(kin + tile_base + k) : 0u);
    }
    {
      uint4* z = reinterpret_cast<uint4*>(&S.u.s.whist[0][0]);  // whist and match (contiguous)
      constexpr int kZero = (sizeof(S.u.s.whist) + sizeof(S.u.s.match)) / 16;
      static_assert(sizeof(S.u.s.whist) % 16 == 0, "match follows whist at a 16-byte boundary");
      for (int i = tid; i < kZero; i += kFThreads) z[i] = make_uint4(0u, 0u, 0u, 0u);
    }
    __syncthreads();

    // rank inside the warp: OR the lane bit into the digit's mask slot; after
    // a __syncwarp the slot holds the peers, whose lowest lane advances the
    // warp's count of the digit and clears the slot
    uint16_t* wh = S.u.s.whist[warp];
    uint32_t* wm = S.u.s.match[warp];
#pragma unroll
    for (int j = 0; j < kKpt; ++j) {
      const uint32_t k = wloc + 32u * j + lane;
      const bool valid = k < tile_n;
      const uint32_t d = (keys[j] >> shift) & (kFRadix - 1);
      if (valid) atomicOr(wm + d, 1u << lane);
      __syncwarp();
      const uint32_t peers = valid ? wm[d] : 0u;
      const uint32_t before = valid ? wh[d] : 0u;
      __syncwarp();
      if (valid && lane == __ffs(peers) - 1) {
        wh[d] = static_cast<uint16_t>(before + __popc(peers));
        wm[d] = 0u;
      }
      __syncwarp();
      S.u.s.rank[k] = static_cast<uint16_t>(before + __popc(peers & lt_mask));
    }
    __syncthreads();

    // digit d = tid < 256: per-warp exclusive offsets and the tile count,
    // published for the column scan
    uint32_t cnt = 0;
    if (tid < kFRadix) {
#pragma unroll
      for (int w = 0; w < kFWarps; ++w) {
        const uint32_t c = S.u.s.whist[w][tid];
        S.u.s.whist[w][tid] = static_cast<uint16_t>(cnt);  // <= kTile - 1
        cnt += c;
      }
      a.counts[static_cast<size_t>(tid) * nt + tile] = cnt;
    }
    const uint32_t ts = block_exclusive_scan512(cnt, S.scan);  // has __syncthreads
    if (tid < kFRadix) S.tstart[tid] = ts;
    __syncthreads();
    // the tile in (digit, input order) in shared memory; the values are
    // loaded first, four at a time together
#pragma unroll
    for (int h = 0; h < kKpt; h += 4) {
      uint32_t vals[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const uint32_t k = wloc + 32u * (h + j) + lane;
        vals[j] = p == 0 ? tile_base + k : (k < tile_n ? __ldcg(vin + tile_base + k) : 0u);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const uint32_t k = wloc + 32u * (h + j) + lane;
        if (k < tile_n) {
          const uint32_t dg = (keys[h + j] >> shift) & (kFRadix - 1);
          const uint32_t pos = S.tstart[dg] + S.u.s.whist[warp][dg] + S.u.s.rank[k];
          S.u.s.keys[pos] = keys[h + j];
          S.u.s.vals[pos] = vals[j];
        }
      }
    }
    grid_barrier(a.bar, epoch, a.status, a.spin_limit);  // every tile's counts are published

    // one warp per digit: exclusive prefix of the digit's counts over the
    // tiles (in place) and the digit's total; lane l holds tiles l, l+32, ...
    // of a chunk of 256 tiles, loaded together
    for (uint32_t d = tile * kFWarps + warp; d < kFRadix; d += nt * kFWarps) {
      uint32_t* col = a.counts + static_cast<size_t>(d) * nt;
      uint32_t carry = 0;
      for (uint32_t r0 = 0; r0 < nt; r0 += 256) {
        uint32_t v[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const uint32_t t = r0 + 32u * i + lane;
          v[i] = t < nt ? __ldcg(col + t) : 0u;
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          uint32_t x = v[i];
#pragma unroll
          for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += y;
          }
          const uint32_t t = r0 + 32u * i + lane;
          if (t < nt) col[t] = carry + x - v[i];
          carry += __shfl_sync(0xffffffffu, x, 31);
        }
      }
      if (lane == 0) a.totals[d] = carry;
    }
    grid_barrier(a.bar, epoch, a.status, a.spin_limit);  // prefixes and totals are complete

    const uint32_t tot = tid < kFRadix ? __ldcg(a.totals + tid) : 0u;
    const uint32_t gb = block_exclusive_scan512(tot, S.scan);  // has __syncthreads
    if (tid < kFRadix)
      S.offs[tid] = gb + __ldcg(a.counts + static_cast<size_t>(tid) * nt + tile) - S.tstart[tid];  // mod 2^32
    __syncthreads();
    for (uint32_t i = tid; i < tile_n; i += kFThreads) {
      const uint32_t key = S.u.s.keys[i];
      const uint32_t g = S.offs[(key >> shift) & (kFRadix - 1)] + i;
      if (g < T) {  // always true unless a barrier wait gave up (status already raised)
        kout[g] = key;
        vout[g] = S.u.s.vals[i];
      }
    }
    if (p < 3) grid_barrier(a.bar, epoch, a.status, a.spin_limit);  // the pass's output is complete
  }
}

struct FrontVariant {
  void (*kernel)(FrontArgs);
  int kpt;
  size_t smem;
};

template <int kKpt, bool kBox>
FrontVariant front_variant() {
  return FrontVariant{k_build_front<kKpt, kBox>, kKpt, sizeof(FrontSmem<kKpt>)};
}

// Blocks of `v` that fit on the device at once (per device, looked up once).
uint32_t front_capacity(const FrontVariant& v, int slot) {
  static uint32_t cap[64][6] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
  if (cap[dev][slot] == 0) {
    int coop = 0, sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaFuncSetAttribute(v.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(v.smem)) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, v.kernel, kFThreads, v.smem) != cudaSuccess) {
      cudaGetLastError();
      per_sm = 0;
    }
    const uint32_t c = coop ? static_cast<uint32_t>(per_sm) * static_cast<uint32_t>(sms) : 0u;
    cap[dev][slot] = c > 0 ? c : 0xFFFFFFFFu;  // 0xFFFFFFFF: looked up, unusable
  }
  return cap[dev][slot] == 0xFFFFFFFFu ? 0u : cap[dev][slot];
}

}  // namespace

uint32_t front_max_tri() {
  const FrontVariant v = front_variant<16, false>();
  const uint64_t c = front_capacity(v, 4);
  const uint64_t m = c * kFThreads * 16;
  return m > 0xFFFFFFFFull ? 0xFFFFFFFFu : static_cast<uint32_t>(m);
}

bool launch_build_front(cudaStream_t s, uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                        const float* vtx2xyz, float* tribox, float* partials, uint32_t max_partials,
                        float* transform_out, float* aabb_out, uint32_t* tri2morton, uint32_t* ka, uint32_t* va,
                        uint32_t* kb, uint32_t* vb, uint32_t* out_keys, uint32_t* out_vals, uint32_t* counts,
                        uint32_t* totals, uint32_t* bar, uint32_t* status) {
  if (num_tri < 2) return false;
  const bool box = tribox != nullptr;
  const FrontVariant vs[3] = {box ? front_variant<8, true>() : front_variant<8, false>(),
                              box ? front_variant<12, true>() : front_variant<12, false>(),
                              box ? front_variant<16, true>() : front_variant<16, false>()};
  for (int k = 0; k < 3; ++k) {
    const FrontVariant& v = vs[k];
    const uint32_t tile = static_cast<uint32_t>(kFThreads * v.kpt);
    const uint32_t grid = (num_tri + tile - 1) / tile;
    const uint32_t cap = front_capacity(v, 2 * k + (box ? 1 : 0));
    if (grid > cap || grid > max_partials) continue;
    FrontArgs args{num_tri, num_vtx, tri2vtx, vtx2xyz, tribox, partials, transform_out, aabb_out, tri2morton,
                   ka, va, kb, vb, out_keys, out_vals, counts, totals, bar, status, get_wait_limit()};
    void* params[] = {&args};
    if (cudaLaunchCooperativeKernel(reinterpret_cast<void*>(v.kernel), dim3(grid), dim3(kFThreads), params, v.smem,
                                    s) != cudaSuccess) {
      cudaGetLastError();  // refused: the caller takes the separate kernels
      return false;
    }
    return true;
  }
  return false;
}

}  // namespace dm
