// dm_internal.h — host-side launchers shared between the library's
// translation units.  Not part of the public C ABI (see include/delmsh_gb300.h).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace dm {

// ----------------------------------------------------------------- capi.cu
// Records the message that dm_last_error() returns on this thread; returns code.
int set_error(int code, const char* fmt, ...);
// Device address of the library's status word on the current device (or nullptr).
uint32_t* device_status_word();
// The single-mesh build with each branch's range end kept in other_end_out
// (u32[T-1]), so later refits of the tree can use launch_refit_windowed.
int build_keep_ranges(cudaStream_t s, uint32_t T, const uint32_t* tri2vtx, uint32_t V, const float* vtx2xyz,
                      uint32_t* bvhnodes, float* aabb, uint32_t* other_end_out, void* scratch, size_t scratch_bytes);
size_t build_scratch_bytes(uint32_t T);

// ---------------------------------------------------------------- build.cu
constexpr int kAabbBlocks = 1024;  // upper bound on centroid-AABB reduction blocks

// Centroid AABB (vtx2xyz.rs:19-37 over elem2center) and the fit transform
// (16 floats, column-major).  partials: kAabbBlocks*6 floats; ticket: one u32
// that is zero on entry and left zero.  With cent != nullptr the centroids
// are also stored, x, y and z each as num_tri floats (cent, cent + stride,
// cent + 2 * stride); with tribox != nullptr each triangle's box (6 floats,
// the leaf box of the refit) too.
void launch_centroid_aabb(cudaStream_t s, uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                          const float* vtx2xyz, float* partials, uint32_t* ticket, float* aabb_out,
                          float* transform_out, uint32_t* status, float* cent = nullptr, size_t stride = 0,
                          float* tribox = nullptr);

// Triangle-centroid Morton codes; when hist != nullptr also accumulates the
// digit histograms of the radix sort (hist10: u32[3][1024] for three 10-bit
// passes, else u32[4][256]; zeroed by the caller).  With cent != nullptr the
// centroids are read from there (launch_centroid_aabb's layout) instead of
// being recomputed.
void launch_morton_tri(cudaStream_t s, uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                       const float* vtx2xyz, const float* transform, uint32_t* codes, uint32_t* hist,
                       uint32_t* status, const float* cent = nullptr, size_t stride = 0, bool hist10 = false);

// mortons.cu:8-37 semantics with the CPU's clamping (num_dim 2 or 3).
void launch_vtx2morton(cudaStream_t s, uint32_t n, uint32_t num_dim, const float* vtx2co, const float* transform,
                       uint32_t* out);

// bvhnodes_morton.rs:10-50 / bvhnodes_morton.cu:29-72.  other_end (optional,
// u32[n-1]): for each branch the end of its leaf range that is not its own
// index (a branch index is always one end of its range).
void launch_topology(cudaStream_t s, uint32_t n, const uint32_t* idx2morton, const uint32_t* idx2obj,
                     uint32_t* bvhnodes, uint32_t* other_end = nullptr, uint32_t threads = 256);

// Vertex indices >= num_vtx are replaced by 0 and raise kStatusBadIndex.
// Bottom-up refit (bvhnode2aabb.cu:7-65 semantics, values of
// bvhnode2aabb3.rs:68-142).  flags: u32[num_tri-1], zero on entry, left zero.
// height_out (optional): number of nodes on the longest root-to-leaf path.
// gate (optional): a refit header word; the climb then runs only if it has
// kRefitPlainClimb set (launch_refit_any_tree).
void launch_refit(cudaStream_t s, uint32_t num_tri, const uint32_t* bvhnodes, const uint32_t* tri2vtx,
                  uint32_t num_vtx, const float* vtx2xyz0, const float* vtx2xyz1, float* aabb, uint32_t* flags, uint32_t* height_out,
                  uint32_t* status, const uint32_t* gate = nullptr);

// Meshes of a batch stored back to back: mesh m owns triangles
// tri_off[m]..tri_off[m+1]-1 and vertices vtx_off[m]..vtx_off[m+1]-1, and its
// nodes start at node 2*tri_off[m]-m (branch words at tri_off[m]-m); indices
// stored inside a mesh's arrays are local to that mesh.  A single mesh is
// {1, nullptr, nullptr}.  Every mesh has at least one triangle.
struct Segments {
  uint32_t num_mesh;
  const uint32_t* tri_off;  // device, num_mesh+1 entries
  const uint32_t* vtx_off;  // device, num_mesh+1 entries
};

// Refit of trees built by launch_topology with other_end: the same boxes as
// launch_refit.  Without NaN in the leaf boxes, the first-wins merge of
// from_two_aabbs makes every branch box the leftmost minimum / maximum over
// its leaf range, so the boxes come from range queries on a segment tree of
// the leaf boxes (k_refit_seg_*).  With NaN, or when heights are asked for,
// the tree-order climb runs instead (k_refit_win + k_refit_top).
// flags: u32[refit_flags_words(total_tri)]; its first total_tri words are
// arrival counters, zero on entry and left zero; the rest (queue, segment
// tree) needs no initialisation.  height_out (optional) receives one height
// per mesh.
constexpr uint32_t kRefitWindowLog = 10;
constexpr uint32_t kRefitWindow = 1u << kRefitWindowLog;  // leaves per window
constexpr uint32_t kRefitWinHeap = kRefitWindow / 4;      // stored window heap: nodes of 8.. leaves, index 1..
constexpr uint32_t kRefitSuper = 64;                      // windows per superblock
// a window whose right edge is crossed by at least this many branches with a
// shared right end (a run of equal codes) folds that end once for all of them
constexpr uint32_t kRefitRunMin = 64;
constexpr uint32_t kRefitSuperLog = kRefitWindowLog + 6;  // log2(kRefitWindow * kRefitSuper)
constexpr uint32_t kRefitQueueHdr = 8;      // queue count, climb flag, ticket, crossing-list count, runs present, spare
// climb-flag bit: the tree is not in Karras leaf order (or could not be
// shown to be), so the parent-pointer climb does the refit; bit 0 hands the
// call to the tree-order climb (NaN leaf boxes, heights)
constexpr uint32_t kRefitPlainClimb = 2u;
inline uint32_t refit_num_windows(uint32_t total_tri) { return (total_tri + kRefitWindow - 1) / kRefitWindow; }
inline uint32_t refit_num_super(uint32_t total_tri) {
  return (refit_num_windows(total_tri) + kRefitSuper - 1) / kRefitSuper;
}
inline uint32_t refit_top_log(uint32_t total_tri) {
  uint32_t lg = 0;
  while ((1ull << lg) < refit_num_super(total_tri)) ++lg;
  return lg;
}
inline uint32_t refit_queue_capacity(uint32_t total_tri) { return 2 * refit_num_windows(total_tri) + 2; }
inline size_t refit_queue_offset(uint32_t total_tri) { return (static_cast<size_t>(total_tri) + 3) & ~size_t{3}; }
inline size_t refit_seg_offset(uint32_t total_tri) {
  return refit_queue_offset(total_tri) + kRefitQueueHdr + 4 * static_cast<size_t>(refit_queue_capacity(total_tri));
}
// window heaps (kRefitWinHeap boxes each), superblock heaps (64 each), top heap (2 * 2^top_log)
inline size_t refit_seg_words(uint32_t total_tri) {
  return 6 * (size_t{kRefitWinHeap} * refit_num_windows(total_tri) + size_t{64} * refit_num_super(total_tri) +
              (size_t{2} << refit_top_log(total_tri)));
}
inline size_t refit_flags_words(uint32_t total_tri) { return refit_seg_offset(total_tri) + refit_seg_words(total_tri); }
// tribox (optional, one mesh and vtx2xyz1 == nullptr only): each triangle's
// box, 6 floats in triangle order, as launch_centroid_aabb stores them; the
// leaf boxes are then read instead of gathered from the vertices.  leaf_tri
// (optional, one mesh): the triangle of each leaf position (the sort's
// values), read instead of the leaf records.
void launch_refit_windowed(cudaStream_t s, uint32_t total_tri, const Segments& seg, uint32_t num_vtx_single,
                           const uint32_t* bvhnodes, const uint32_t* other_end, const uint32_t* tri2vtx,
                           const float* vtx2xyz0, const float* vtx2xyz1, float* aabb, uint32_t* flags,
                           uint32_t* height_out, uint32_t* status, const float* tribox = nullptr,
                           bool header_ready = false, const uint32_t* leaf_tri = nullptr);
// Refit of any tree given as bvhnodes (the drop-in refit): derives every
// branch's other range end on the device and runs the range-query refit when
// the tree is in Karras leaf order, else the parent-pointer climb; the choice
// is made on the device.  other_end: u32[num_tri]; flags:
// refit_flags_words(num_tri) words whose first num_tri are zero on entry (and
// left zero).
void launch_refit_any_tree(cudaStream_t s, uint32_t num_tri, const uint32_t* bvhnodes, const uint32_t* tri2vtx,
                           uint32_t num_vtx, const float* vtx2xyz0, const float* vtx2xyz1, float* aabb,
                           uint32_t* other_end, uint32_t* flags, uint32_t* status);

// ---------------------------------------------------------------- front.cu
// Centroids, AABB + fit transform, Morton codes and the four-pass stable
// sort in one cooperative launch (see front.cu).  Returns false, having
// launched nothing, when the mesh's tiles cannot all be resident at once
// (or num_tri < 2); the caller then runs the separate kernels.  ka/va/kb/vb:
// num_tri words each; out_keys/out_vals must not be ka/va; counts:
// 256 * max_partials words; totals: 256 words; bar: one word, zero;
// partials: max_partials * 6 floats.
bool launch_build_front(cudaStream_t s, uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                        const float* vtx2xyz, float* tribox, float* partials, uint32_t max_partials,
                        float* transform_out, float* aabb_out, uint32_t* tri2morton, uint32_t* ka, uint32_t* va,
                        uint32_t* kb, uint32_t* vb, uint32_t* out_keys, uint32_t* out_vals, uint32_t* counts,
                        uint32_t* totals, uint32_t* bar, uint32_t* status);
// Largest mesh the cooperative front takes on the current device (0: none).
uint32_t front_max_tri();

// ----------------------------------------------------------------- sort.cu
constexpr int kSortTile = 3840;  // keys per onesweep tile
constexpr int kRadix = 256;

inline uint32_t sort_num_tiles(uint32_t n) { return (n + kSortTile - 1) / kSortTile; }
inline size_t sort_lookback_words(uint32_t n, int num_pass, int radix = kRadix) {
  return static_cast<size_t>(sort_num_tiles(n)) * radix * num_pass;
}

// Histogram of num_pass 8-bit digits of 32-bit keys (hist zeroed by caller).
void launch_digit_hist_u32(cudaStream_t s, uint32_t n, const uint32_t* keys, int num_pass, uint32_t* hist);
void launch_digit_hist_u64(cudaStream_t s, uint32_t n, const uint64_t* keys, int num_pass, uint32_t* hist);

// One stable onesweep pass (digit at `shift`).  vals_in == nullptr means the
// values are the input positions (iota).  lookback: sort_num_tiles(n)*256
// words and tile_counter: 1 word, both zero on entry.  With `pdl` the pass
// may start while the previous kernel runs (launch_pdl): the tile counter and
// lookback words must have been zeroed before that kernel.
void launch_onesweep_u32(cudaStream_t s, uint32_t n, uint32_t shift, const uint32_t* keys_in,
                         const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out, const uint32_t* hist,
                         uint32_t* lookback, uint32_t* tile_counter, uint32_t* status, bool pdl = false);
// A stable pass over a 10-bit digit of u32 keys (1024 digits; hist: 1024
// words, lookback: sort_lookback_words(n, 1, 1024) words); otherwise as
// launch_onesweep_u32 with pdl.  Three of them sort 30-bit Morton codes.
constexpr int kRadix10 = 1024;
// Builds of up to this many triangles sort in three 10-bit passes: fewer,
// heavier passes win while a tile's 1024 digit runs are the cost; above it
// (short runs, scattered writes) four 8-bit passes are faster (measured on
// GB300: 327k keys 44 vs 61 us, 1.3M keys 107 vs 83 us).
constexpr uint32_t kRadix10MaxKeys = 1u << 19;
void launch_onesweep10_u32(cudaStream_t s, uint32_t n, uint32_t shift, const uint32_t* keys_in,
                           const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out, const uint32_t* hist,
                           uint32_t* lookback, uint32_t* tile_counter, uint32_t* status);
void launch_onesweep_u64(cudaStream_t s, uint32_t n, uint32_t shift, const uint64_t* keys_in,
                         const uint32_t* vals_in, uint64_t* keys_out, uint32_t* vals_out, const uint32_t* hist,
                         uint32_t* lookback, uint32_t* tile_counter, uint32_t* status);
// One pass over one tile with a caller-preset tile counter (see sort.cu):
// exercises the give-up path of the look-back wait.  lookback: 2*256 words.
void launch_onesweep_wait_probe(cudaStream_t s, uint32_t n, const uint32_t* keys_in, uint32_t* keys_out,
                                uint32_t* vals_out, const uint32_t* hist, uint32_t* lookback, uint32_t* tile_counter,
                                uint32_t* status, uint32_t spin_limit);
// Polls a bounded device wait makes before it gives up (process-wide; read
// at each launch).  Default kDefaultWaitLimit.
constexpr uint32_t kDefaultWaitLimit = 1u << 22;
uint32_t get_wait_limit();
void set_wait_limit(uint32_t polls);

// ---------------------------------------------------------------- batch.cu
// Number of 8-bit passes sorting (mesh << 30 | code) keys of num_mesh meshes.
int batch_num_pass(uint32_t num_mesh);
void launch_batch_fit(cudaStream_t s, const Segments& seg, const uint32_t* tri2vtx, const float* vtx2xyz,
                      float* transforms, uint32_t* status);
void launch_batch_morton(cudaStream_t s, uint32_t total_tri, const Segments& seg, const uint32_t* tri2vtx,
                         const float* vtx2xyz, const float* transforms, uint64_t* keys, uint32_t* hist, int num_pass,
                         uint32_t* status);
void launch_batch_topology(cudaStream_t s, uint32_t total_tri, const Segments& seg, const uint64_t* keys,
                           const uint32_t* vals, uint32_t* bvhnodes, uint32_t* other_end);
// Batches whose largest mesh has at most this many triangles replace
// launch_batch_fit .. launch_batch_topology with launch_batch_seg_build: each
// mesh sorted and linked in on-chip memory by one block or one cluster.
constexpr uint32_t kSegMaxTri = 65536;
// lists: num_mesh words; counters: 4 words, zero on entry.  Returns non-zero
// (nothing launched after the failing launch) if the kernel cannot be
// launched on this device.
int launch_batch_seg_build(cudaStream_t s, const Segments& seg, uint32_t max_tri, const uint32_t* tri2vtx,
                           const float* vtx2xyz, uint32_t* bvhnodes, uint32_t* other, uint32_t* lists,
                           uint32_t* counters, uint32_t* status);

// ----------------------------------------------------------------- cast.cu
constexpr int kCastStack = 64;  // default frames of the on-chip (local) traversal stack

// Launch parameters picked by the autotuner (del_msh_gb300/autotune.py) and
// set through dm_tuning_set.  Every choice gives the same results; only the
// speed differs.  Read at each launch.
constexpr uint32_t kDefaultPhaseMin = 6;
constexpr uint32_t kDefaultLongSteps = 64;
struct Tuning {
  uint32_t cast_threads = 128;  // threads per block of the persistent cast
  uint32_t cast_stack = 64;     // on-chip frames per ray
  uint32_t tile_w = 8;          // pixel tile of one warp: tile_w x (32 / tile_w)
  uint32_t sort_window = 4;     // predecessors read per look-back round of the sort
  // lanes of a warp that must wait for a phase of the persistent cast before
  // the warp runs it (1 = whenever any lane waits): taking new rays, testing
  // triangles, popping frames
  uint32_t cast_refill_min = kDefaultPhaseMin;
  uint32_t cast_leaf_min = kDefaultPhaseMin;
  uint32_t cast_ascend_min = kDefaultPhaseMin;
  // node entries after which the persistent cast, once a warp has no more
  // rays to take, hands a ray entering a long chain to the warp tier
  uint32_t cast_long_steps = kDefaultLongSteps;
  // batched build: 0 = every mesh sorted and linked on chip when the largest
  // fits (<= kSegMaxTri triangles), 1 = the global 64-bit sort
  uint32_t batch_path = 0;
  // batched on-chip build: the least number of blocks (1, 2 or 4) that
  // build a mesh too large for one block (0 = the fewest that fit)
  uint32_t batch_cluster = 0;
};
// Single-mesh build choices for meshes of up to max_tri triangles (the
// smallest class that holds the mesh applies; none: the defaults).  Every
// choice gives the same tree and boxes.
struct BuildTuning {
  uint32_t max_tri = 0xFFFFFFFFu;
  uint32_t build_path = 0;    // 0 = the cooperative front where it fits, 1 = separate kernels
  uint32_t sort_radix = 0;    // separate kernels: 0 = 10 bits up to kRadix10MaxKeys keys, else 8; or 8 / 10
  uint32_t topo_threads = 0;  // threads per block of the topology kernel: 0 = 256, or 128 / 256 / 512
};
constexpr int kMaxBuildClasses = 8;
BuildTuning build_tuning_for(uint32_t num_tri);
bool set_build_classes(const BuildTuning* classes, uint32_t n);  // false (nothing changed) for a bad table
uint32_t get_build_classes(BuildTuning* out, uint32_t cap);
// (threads, stack) pairs compiled for the persistent cast
constexpr uint32_t kCastVariants[][2] = {{128, 64}, {64, 64}, {256, 64}, {128, 32}, {128, 96}};
Tuning get_tuning();
bool set_tuning(const Tuning& t);  // false (and nothing changed) for an unsupported choice
constexpr size_t kFrameBytes = 16;

// Launches `kernel` so that it may start before the previous kernel in the
// stream has finished (programmatic dependent launch); the kernel must call
// pdl_wait() (dm_device.cuh) before it touches that kernel's data.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

struct MeshView {
  uint32_t num_tri;
  uint32_t num_vtx;
  const uint32_t* tri2vtx;
  const float* vtx2xyz;
  const uint32_t* bvhnodes;
  const float* aabb;
};

struct CastOut {
  uint32_t* hit_tri;  // u32 per ray (MAX = miss)
  float* hit_t;       // optional
  float* hit_bc;      // optional, 3 per ray (1-u-v, u, v)
};

struct CastScratch {
  uint32_t* counters;  // 4 words, zero on entry: work counter, two overflow counts
  uint32_t* list1;     // num_ray words
  uint32_t* list2;     // num_ray words
  void* pool;          // >= 16 * max(num_tri, 4096) bytes
  size_t pool_bytes;
};

size_t cast_scratch_bytes(uint32_t num_ray, uint32_t num_tri);
void cast_scratch_carve(void* base, uint32_t num_ray, uint32_t num_tri, CastScratch* out);

// Pixels of an img_w x img_h image (ray_for_pixel.h) or explicit rays.
void launch_cast_pixels(cudaStream_t s, uint32_t img_w, uint32_t img_h, const float* t_ndc2world, const MeshView& m,
                        const CastOut& o, const CastScratch& sc, uint32_t* status);
void launch_cast_rays(cudaStream_t s, uint32_t num_ray, const float* ray_org, const float* ray_dir,
                      const MeshView& m, const CastOut& o, const CastScratch& sc, uint32_t* status);

// img_w x img_h pixels per mesh of a batch, per-mesh ndc->world transforms
// (16 floats each); output slot of pixel p of mesh m is m*img_w*img_h + p.
void launch_batch_cast_pixels(cudaStream_t s, const Segments& seg, uint32_t max_tri, const uint32_t* tri2vtx,
                              const float* vtx2xyz, const uint32_t* bvhnodes, const float* aabb, uint32_t img_w,
                              uint32_t img_h, const float* transforms, const CastOut& o, const CastScratch& sc,
                              uint32_t* status);

// --------------------------------------------------------------- render.cu
// Consumers of a pix2tri image (see render.cu): world2ndc = inverse(ndc2world)
// on the device (one thread), depth and attribute interpolation, forward and
// backward (the backward passes accumulate with atomicAdd).
void launch_inverse4(cudaStream_t s, const float* m, float* inv, uint32_t* status);
void launch_pix2depth(cudaStream_t s, uint32_t img_w, uint32_t img_h, float* pix2depth, const uint32_t* pix2tri,
                      const MeshView& m, const float* ndc2world, const float* world2ndc, uint32_t* status);
void launch_pix2depth_bwd(cudaStream_t s, uint32_t img_w, uint32_t img_h, float* dldw_vtx2xyz, const uint32_t* pix2tri,
                          const MeshView& m, const float* dldw_pix2depth, const float* ndc2world,
                          const float* world2ndc, uint32_t* status);
void launch_interpolate(cudaStream_t s, uint32_t img_w, uint32_t img_h, const uint32_t* pix2tri, const MeshView& m,
                        uint32_t num_vdim, const float* vtx2val, const float* ndc2world, float* pix2val,
                        uint32_t* status);
void launch_interpolate_bwd(cudaStream_t s, uint32_t img_w, uint32_t img_h, const uint32_t* pix2tri,
                            const MeshView& m, uint32_t num_vdim, const float* vtx2val, const float* ndc2world,
                            const float* dldw_pix2val, float* dldw_vtx2xyz, float* dldw_vtx2val, uint32_t* status);

// -------------------------------------------------------------- octree.cu
// Quad/oct-trees from the binary radix tree of sorted unique Morton codes.
size_t octree_scratch_bytes(uint32_t num_idx);
void launch_octree_brt(cudaStream_t s, uint32_t num_idx, const uint32_t* idx2morton, uint32_t num_dim,
                       uint32_t max_depth, uint32_t* bnodes, uint32_t* bnode2depth, uint32_t* bnode2onode,
                       uint32_t* idx2bnode, uint32_t* tile_sums, uint32_t* status);
void launch_octree_make(cudaStream_t s, uint32_t num_idx, const uint32_t* bnodes, const uint32_t* bnode2onode,
                        const uint32_t* bnode2depth, const uint32_t* idx2bnode, const uint32_t* idx2morton,
                        uint32_t num_onode, uint32_t max_depth, uint32_t num_dim, uint32_t* onodes,
                        uint32_t* onode2depth, float* onode2center, uint32_t* idx2onode, float* idx2center,
                        uint32_t* status);
void launch_octree_aggregate(cudaStream_t s, uint32_t num_idx, uint32_t num_vdim, const float* idx2val,
                             const uint32_t* idx2onode, uint32_t num_link, const uint32_t* onodes, uint32_t num_onode,
                             float* onode2aggval, uint32_t* status);

// --------------------------------------------------------------- selfx.cu
// Self-intersecting triangle pairs through the BVH: pairs u32[capacity][2],
// segments f32[capacity][6]; *count (zero on entry) receives the number
// found, which may exceed capacity (then only capacity are written).
// Synchronizes the stream once per round (to size the next).  scratch:
// self_intersection_scratch_bytes(num_tri).  Returns 0, or -1 on a CUDA error.
size_t self_intersection_scratch_bytes(uint32_t num_tri);
int launch_self_intersection(cudaStream_t s, const MeshView& m, uint32_t capacity, uint32_t* pairs, float* segments,
                             uint32_t* count, void* scratch, size_t scratch_bytes, uint32_t* status);

}  // namespace dm
