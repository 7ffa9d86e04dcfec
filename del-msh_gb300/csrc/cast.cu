// cast.cu — single-mesh ray casting: the pixels of one image (ray_for_pixel.h,
// as pix2tri.rs:3-48 / pix2tri.cu:13-76) or an array of explicit rays
// (search_bvh3.rs:103-221 per ray), with the traversal of dm_traverse.cuh.
//
// Pixels are handed out in tiles of 32 (8x4 by default, a tuning choice; 32
// consecutive work indices = one tile) so that the rays of a warp start close
// together and walk similar nodes.
#include "dm_traverse.cuh"

namespace dm {
namespace {

struct SingleJob {
  uint32_t num_work;
  MeshView m;
  uint32_t img_w, img_h, tiles_x, tile_w, tile_h;  // pixel mode
  uint32_t tile_w_log;                              // tile_w is a power of two
  Divider by_tiles_x;
  const float* t_ndc2world;
  const float* ray_org;  // ray mode when non-null
  const float* ray_dir;
  CastOut o;

  __device__ __forceinline__ void prepare(float* smem) const {
    if (ray_org == nullptr && threadIdx.x < 16) smem[threadIdx.x] = t_ndc2world[threadIdx.x];
  }

  __device__ __forceinline__ bool fetch(uint32_t w, const float* smem, MeshView& mv, Ray& r, uint32_t& out) const {
    mv = m;
    if (ray_org != nullptr) {
      out = w;
      const float* po = ray_org + static_cast<size_t>(w) * 3;
      const float* pd = ray_dir + static_cast<size_t>(w) * 3;
      r = make_ray(make_float3(__ldg(po), __ldg(po + 1), __ldg(po + 2)),
                   make_float3(__ldg(pd), __ldg(pd + 1), __ldg(pd + 2)));
      return true;
    }
    const uint32_t tile = w >> 5, j = w & 31u;
    const uint32_t ty = by_tiles_x.div(tile);
    const uint32_t px = (tile - ty * tiles_x) * tile_w + (j & (tile_w - 1u));
    const uint32_t py = ty * tile_h + (j >> tile_w_log);
    if (px >= img_w || py >= img_h) return false;
    out = py * img_w + px;
    float3 o3, d3;
    ray_for_pixel_xy(px, py, img_w, img_h, smem, o3, d3);
    r = make_ray(o3, d3);
    return true;
  }

  __device__ __forceinline__ void write(uint32_t out, const MeshView& mv, const Ray& r, const Hit& h) const {
    o.hit_tri[out] = h.id;
    if (o.hit_t) o.hit_t[out] = h.t;
    if (o.hit_bc) {
      float bc[3];
      hit_bc(mv, r, h, bc);
      o.hit_bc[static_cast<size_t>(out) * 3] = bc[0];
      o.hit_bc[static_cast<size_t>(out) * 3 + 1] = bc[1];
      o.hit_bc[static_cast<size_t>(out) * 3 + 2] = bc[2];
    }
  }
};

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
  SingleJob job{};
  job.m = m;
  job.img_w = img_w;
  job.img_h = img_h;
  const Tuning t = get_tuning();
  job.tile_w = t.tile_w;
  job.tile_h = 32u / t.tile_w;
  job.tile_w_log = static_cast<uint32_t>(__builtin_ctz(t.tile_w));
  job.tiles_x = (img_w + job.tile_w - 1) / job.tile_w;
  job.by_tiles_x = Divider::make(job.tiles_x);
  const uint32_t tiles_y = (img_h + job.tile_h - 1) / job.tile_h;
  job.num_work = job.tiles_x * tiles_y * 32u;
  job.t_ndc2world = t_ndc2world;
  job.o = o;
  cast_job(s, job, sc, m.num_tri, status);
}

void launch_cast_rays(cudaStream_t s, uint32_t num_ray, const float* ray_org, const float* ray_dir,
                      const MeshView& m, const CastOut& o, const CastScratch& sc, uint32_t* status) {
  SingleJob job{};
  job.m = m;
  job.num_work = num_ray;
  job.ray_org = ray_org;
  job.ray_dir = ray_dir;
  job.o = o;
  cast_job(s, job, sc, m.num_tri, status);
}

}  // namespace dm
