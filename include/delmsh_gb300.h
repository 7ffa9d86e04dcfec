/*
 * delmsh_gb300.h — C ABI of the GB300 (sm_103a) LBVH build and BVH ray cast.
 *
 * Drop-in for del-msh's LBVH / ray-cast path: the same array layouts
 *   tri2vtx      u32[num_tri*3]
 *   vtx2xyz      f32[num_vtx*3]
 *   bvhnodes     u32[(2*num_tri-1)*3]   [parent, left, right]; a leaf is
 *                                        [parent, triangle, u32::MAX]; the root
 *                                        is node 0 and its parent is u32::MAX;
 *                                        branches are 0..T-2, leaves T-1..2T-2
 *   bvhnode2aabb f32[(2*num_tri-1)*6]   [xmin, ymin, zmin, xmax, ymax, zmax]
 *   matrices     f32[16] column-major (as del-msh's kernels read them)
 * and the same results as del-msh-cpu on the same inputs (Morton codes,
 * sorted permutation with ties by index, topology and AABBs bit-exact; hit
 * triangle ids and hit t bit-exact to the CPU restatement).
 *
 * Conventions (those of the del-msh-dlpack GPU bindings):
 *   - every array argument is a DEVICE pointer; outputs are caller-allocated;
 *   - work is enqueued asynchronously on the CUDA stream `stream_ptr`
 *     (a cudaStream_t cast to u64; 0 is the legacy default stream), like the
 *     bindings' `stream_ptr: u64`;
 *   - functions return DM_OK or an error code and never abort; the message of
 *     the last error on the calling thread is dm_last_error().  Where the
 *     reference panics (assert/unwrap on shapes) these return
 *     DM_ERR_INVALID_ARGUMENT;
 *   - `scratch` may be NULL: the function then allocates its temporary memory
 *     stream-ordered (cudaMallocAsync / cudaFreeAsync on `stream_ptr`), as the
 *     reference's bindings allocate theirs.  Otherwise it must hold at least
 *     the matching *_scratch_bytes() bytes, 256-byte aligned;
 *   - calls on distinct streams may run concurrently as long as they do not
 *     share scratch memory.
 */
#ifndef DELMSH_GB300_H
#define DELMSH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DM_OK 0
#define DM_ERR_INVALID_ARGUMENT 1
#define DM_ERR_CUDA 2
#define DM_ERR_SCRATCH_TOO_SMALL 3
#define DM_ERR_UNSUPPORTED 4

/* Library version string. */
const char* dm_version(void);

/* Message of the last error returned on the calling thread ("" if none). */
const char* dm_last_error(void);

/* Reads the device status word of the current device (bits: 1 = a bounded
 * wait gave up, 2 = a traversal stack tier was too small, 4 = an index read
 * from an input array was out of range, 8 = a matrix to invert was singular).
 * Synchronizes the device.  When `clear` is non-zero the word is reset to 0.
 * No reference counterpart: the
 * reference's kernels use device asserts (mortons.cu:22-34,
 * bvhnode2aabb.cu:21-48), which this library replaces by this word. */
int dm_device_status(uint32_t* bits, int clear);

/* Launch parameters chosen by the autotuner (del_msh_gb300/autotune.py).
 * Every choice computes the same results; only speed differs.  They are read
 * at each launch (a CUDA graph keeps those of its capture).  Process-wide.
 * No reference counterpart: the reference hard-codes its launch shapes. */
typedef struct dm_tuning {
  uint32_t cast_threads; /* threads per block of the persistent cast: 64, 128 or 256 (with cast_stack 64),
                            or 128 with cast_stack 32 / 96 */
  uint32_t cast_stack;   /* on-chip traversal frames per ray before the overflow tiers */
  uint32_t tile_w;       /* pixel tile of one warp is tile_w x (32 / tile_w): 2, 4, 8, 16 or 32 */
  uint32_t sort_window;  /* predecessor tiles read per look-back round of the radix sort: 4 or 8 */
  /* The persistent cast runs a phase (taking new rays / testing triangles /
     popping frames) once this many of a warp's 32 lanes wait for it, or when
     nothing else can run: 1..32, 0 = the default (6).  Results do not depend
     on them. */
  uint32_t cast_refill_min;
  uint32_t cast_leaf_min;
  uint32_t cast_ascend_min;
  /* Node entries after which the persistent cast, once a warp has no more
     rays to take, hands a ray entering a long run of chain links to the warp
     tier, where one warp runs it and folds the links 32 at a time: 1..2^30,
     0 = the default (64).  Results do not depend on it. */
  uint32_t cast_long_steps;
  /* Batched build: 0 = every mesh sorted and linked on chip when the largest
     has at most 65536 triangles (else the global sort), 1 = the global 64-bit
     sort always. */
  uint32_t batch_path;
  /* Batched on-chip build: the least number of blocks (1, 2 or 4) that build
     a mesh too large for one block; 0 = the fewest that hold the largest
     mesh. */
  uint32_t batch_cluster;
} dm_tuning;

/* The current launch parameters. */
int dm_tuning_get(dm_tuning* out);

/* Sets the launch parameters; DM_ERR_INVALID_ARGUMENT (nothing changed) for
 * a combination that is not compiled. */
int dm_tuning_set(const dm_tuning* in);

/* Single-mesh build choices by mesh size: a build of T triangles uses the
 * first class (bounds ascending) with T <= max_tri, or the defaults (all 0)
 * when none holds it.  Every choice builds the same tree and boxes.
 * Process-wide, read at each build.  No reference counterpart. */
typedef struct dm_build_class {
  uint32_t max_tri;      /* the class holds meshes of up to this many triangles */
  uint32_t build_path;   /* 0 = centroids, codes and sort in one cooperative launch where the mesh fits on the
                            device at once, 1 = the separate kernels */
  uint32_t sort_radix;   /* separate kernels: 0 = 10-bit digits up to 2^19 keys, else 8; or 8 / 10 */
  uint32_t topo_threads; /* threads per block of the topology kernel: 0 (= 256), 128, 256 or 512 */
} dm_build_class;
int dm_build_classes_set(const dm_build_class* classes, uint32_t num_class);  /* at most 8; 0 clears */
int dm_build_classes_get(dm_build_class* out, uint32_t capacity, uint32_t* num_class);

/* Polls a bounded device wait (the radix sort's look-back) makes before it
 * gives up, raises status bit 1 and returns instead of hanging.  Process-wide,
 * read at each launch; 0 restores the default (2^22).  No reference
 * counterpart: the reference's sort (thrust) has no bounded waits. */
int dm_wait_limit_get(uint32_t* polls);
int dm_wait_limit_set(uint32_t polls);

/* Self-test of the bounded wait: one real 8-bit onesweep pass, launched as a
 * single block whose tile counter is preset so that the block draws tile 1
 * and looks back for tile 0, which nothing publishes.  The wait gives up
 * after `polls` polls (1..2^24), status bit 1 is raised and the call returns
 * (it synchronizes `stream_ptr`).  scratch: device memory of
 * dm_selftest_bounded_wait_scratch_bytes() bytes.  No reference counterpart. */
int dm_selftest_bounded_wait(uint64_t stream_ptr, uint32_t polls, void* scratch, size_t scratch_bytes);
size_t dm_selftest_bounded_wait_scratch_bytes(void);

/* Morton codes of points after a homogeneous transform (num_dim 2: 3x3, 3: 4x4
 * column-major), clamped to the unit cube as del-msh-cpu does.
 * Replaces: del-msh-dlpack/src/mortons.rs:18-77 mortons_vtx2morton_from_vtx2co
 * (kernel del-msh-cuda-kernels/cuda/mortons.cu:8-37 vtx2morton;
 * CPU del-msh-cpu/src/mortons.rs:171-212). */
int dm_mortons_vtx2morton_from_vtx2co(uint64_t stream_ptr, uint32_t num_vtx, uint32_t num_dim,
                                      const float* vtx2co, const float* transform_co2unit,
                                      uint32_t* vtx2morton);

/* Stable ascending sort of u32 values in place, writing the permutation
 * (jdx2idx[j] = original position of the j-th smallest; ties keep ascending
 * position).
 * Replaces: del-msh-dlpack/src/array1d.rs:100-154 array1d_argsort (iota +
 * thrust sort_by_key; CPU order of del-msh-cpu/src/mortons.rs:139-146). */
int dm_array1d_argsort(uint64_t stream_ptr, uint32_t n, uint32_t* idx2val, uint32_t* jdx2idx, void* scratch,
                       size_t scratch_bytes);
size_t dm_array1d_argsort_scratch_bytes(uint32_t n);

/* Karras binary radix tree over sorted Morton codes, in the bvhnodes layout;
 * n == 1 gives the single leaf [MAX, idx2obj[0], MAX].
 * Replaces: del-msh-dlpack/src/mortons.rs:80-135
 * mortons_make_bvhnodes_from_sorted_mortons (kernel
 * del-msh-cuda-kernels/cuda/bvhnodes_morton.cu:29-72;
 * CPU del-msh-cpu/src/bvhnodes_morton.rs:10-50). */
int dm_mortons_make_bvhnodes_from_sorted_mortons(uint64_t stream_ptr, uint32_t n, const uint32_t* idx2obj,
                                                 const uint32_t* idx2morton, uint32_t* bvhnodes);

/* AABB of every node of a triangle BVH (leaf = box of its triangle's three
 * vertices, branch = union of its children), optionally also enclosing
 * vtx2xyz1 (continuous collision detection; may be NULL).  This is also the
 * refit of a deformed mesh: same bvhnodes, new vertices.  Only i_bvhnode == 0
 * (the whole tree) is supported.
 * With flags_scratch == NULL (the reference binding's form) the call takes
 * stream-ordered scratch, derives every branch's leaf range from bvhnodes on
 * the device and, for a tree in Karras leaf order (every tree this library
 * or the reference builds), answers each branch by range queries over the
 * leaf boxes; any other tree, or one whose chains of right (left) children
 * are longer than 64 records, is refit by the parent-pointer climb instead,
 * chosen on the device.  Both give the reference's boxes bit for bit.
 * flags_scratch: u32[num_elem-1] that is zero before the first call and that
 * every call leaves zero; the call then uses only it and always climbs.
 * Replaces: del-msh-dlpack/src/bvhnode2aabb.rs:15-108 bvhnode2aabb_update_aabb
 * (kernel del-msh-cuda-kernels/cuda/bvhnode2aabb.cu:7-65 from_trimesh3;
 * CPU del-msh-cpu/src/bvhnode2aabb3.rs:68-142). */
int dm_bvhnode2aabb_update_aabb(uint64_t stream_ptr, uint32_t num_bvhnode, float* bvhnode2aabb,
                                uint32_t i_bvhnode, const uint32_t* bvhnodes, uint32_t num_elem,
                                const uint32_t* elem2vtx, uint32_t num_vtx, const float* vtx2xyz0,
                                const float* vtx2xyz1, uint32_t* flags_scratch);

/* dm_bvhnode2aabb_update_aabb (flags_scratch == NULL form) with caller
 * scratch of dm_bvhnode2aabb_update_aabb_scratch_bytes(num_elem) bytes,
 * zero before the first call; every call leaves it ready for the next one
 * (the words that must be zero are left zero), so a resident tree is refit
 * frame after frame with no memset and no allocation.
 * Replaces: del-msh-dlpack/src/bvhnode2aabb.rs:15-108 bvhnode2aabb_update_aabb
 * with the binding's internal flag allocation (bvhnode2aabb.rs:78-79) moved to
 * the caller. */
int dm_bvhnode2aabb_update_aabb_ex(uint64_t stream_ptr, uint32_t num_bvhnode, float* bvhnode2aabb,
                                   const uint32_t* bvhnodes, uint32_t num_elem, const uint32_t* elem2vtx,
                                   uint32_t num_vtx, const float* vtx2xyz0, const float* vtx2xyz1, void* scratch,
                                   size_t scratch_bytes);
size_t dm_bvhnode2aabb_update_aabb_scratch_bytes(uint32_t num_elem);

/* dm_bvhnode2aabb_update_aabb for callers that cannot allocate device memory
 * (a per-frame refit loop under a no-allocation rule, a plugin whose host owns
 * the CUDA allocator, an FFI caller holding only its own arrays): the arrival
 * flags live in a static device array inside the library instead of caller
 * scratch or a temporary allocation, and the call allocates nothing.  Meshes
 * of 1..4194305 triangles (16 MiB of flags, held by every GPU that loads the
 * library until exit); larger ones return DM_ERR_INVALID_ARGUMENT.  The first
 * call on a device looks up the array's address (do it before any stream
 * capture); the address is kept for the life of the process, so the library
 * must not be used across a cudaDeviceReset of that device (which unloads
 * the module and leaves the kept address stale; the device status word's
 * address is kept the same way).  Calls share the array: each clears the
 * part it uses, and calls that overlap on the GPU race.  No counterpart in
 * the reference. */
int dm_bvhnode2aabb_update_aabb_noalloc(uint64_t stream_ptr, uint32_t num_bvhnode, float* bvhnode2aabb,
                                        const uint32_t* bvhnodes, uint32_t num_elem, const uint32_t* elem2vtx,
                                        uint32_t num_vtx, const float* vtx2xyz0, const float* vtx2xyz1);

/* Whole LBVH build of a triangle mesh: centroids, centroid AABB, fit into the
 * unit cube, Morton codes, stable radix sort, topology, AABBs.
 * Replaces: del-msh-dlpack/del_msh_dlpack/TriMesh3/torch.py:233-285
 * make_bvhnodes_bvhnode2aabb (CPU: del-msh-cpu/src/bvhnodes_morton.rs:151-159
 * from_triangle_mesh + del-msh-cpu/src/bvhnode2aabb3.rs:168-195). */
int dm_trimesh3_make_bvhnodes_bvhnode2aabb(uint64_t stream_ptr, uint32_t num_tri, const uint32_t* tri2vtx,
                                           uint32_t num_vtx, const float* vtx2xyz, uint32_t* bvhnodes,
                                           float* bvhnode2aabb, void* scratch, size_t scratch_bytes);
size_t dm_trimesh3_build_scratch_bytes(uint32_t num_tri);

/* The same build with its intermediate results (each output may be NULL):
 * transform_out f32[16] (fit transform, column-major), tri2morton_out u32[T],
 * idx2tri_out / idx2morton_out u32[T] (the sorted permutation and codes, as
 * mortons.rs:115-147 returns them), height_out u32[1] (nodes on the longest
 * root-to-leaf path).  No single reference counterpart: these are the values
 * of the intermediate steps of TriMesh3/torch.py:233-285. */
int dm_trimesh3_build_ex(uint64_t stream_ptr, uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                         const float* vtx2xyz, uint32_t* bvhnodes, float* bvhnode2aabb, float* transform_out,
                         uint32_t* tri2morton_out, uint32_t* idx2tri_out, uint32_t* idx2morton_out,
                         uint32_t* height_out, void* scratch, size_t scratch_bytes);

/* The whole build with CUDA-event timing of its stages; synchronizes the
 * stream.  stage_ms (host, 4 floats): [0] centroid AABB + Morton codes (with
 * the sort's digit histogram), [1] radix sort, [2] topology, [3] AABB refit.
 * Diagnostics for benchmarks; no reference counterpart. */
int dm_trimesh3_build_profiled(uint64_t stream_ptr, uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                               const float* vtx2xyz, uint32_t* bvhnodes, float* bvhnode2aabb, void* scratch,
                               size_t scratch_bytes, float* stage_ms);

/* Closest hit per pixel of an img_w x img_h image; pixel (iw, ih) casts the
 * ray of ray_for_pixel.h (origin at ndc z=+1, towards z=-1).  pix2tri[ih*w+iw]
 * = triangle or u32::MAX; pix2t (optional) = ray coefficient t of the hit
 * (+inf on a miss).
 * Replaces: del-msh-dlpack/src/pix2tri.rs:17-94 pix2tri_by_raycast (kernel
 * del-msh-cuda-kernels/cuda/pix2tri.cu:13-76 pix_to_tri; the results are those
 * of CPU del-msh-cpu/src/pix2tri.rs:3-48). */
int dm_pix2tri_by_raycast(uint64_t stream_ptr, uint32_t img_w, uint32_t img_h, uint32_t* pix2tri, float* pix2t,
                          uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx, const float* vtx2xyz,
                          const uint32_t* bvhnodes, const float* bvhnode2aabb, const float* transform_ndc2world,
                          void* scratch, size_t scratch_bytes);

/* Closest hit of each ray (ray_org, ray_dir f32[num_ray*3]); hit_t and hit_bc
 * (barycentrics 1-u-v, u, v; f32[num_ray*3]) may be NULL.
 * Replaces: del-msh-cpu/src/search_bvh3.rs:103-221 first_intersection_ray
 * called once per ray. */
int dm_search_bvh3_first_intersection_ray(uint64_t stream_ptr, uint32_t num_ray, const float* ray_org,
                                          const float* ray_dir, uint32_t* hit_tri, float* hit_t, float* hit_bc,
                                          uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                                          const float* vtx2xyz, const uint32_t* bvhnodes,
                                          const float* bvhnode2aabb, void* scratch, size_t scratch_bytes);

/* Scratch size of dm_pix2tri_by_raycast / dm_search_bvh3_first_intersection_ray. */
size_t dm_cast_scratch_bytes(uint32_t num_ray, uint32_t num_tri);

/* ---- consumers of a pix2tri image: depth and attribute interpolation ----
 * Pixel (iw, ih) uses the cast's ray (ray_for_pixel.h) and the ray/triangle
 * intersection of its pix2tri entry; u32::MAX marks the background.  The
 * backward entries ADD into their gradient arrays with atomics, so their
 * sums may differ from a sequential sum by float reassociation. */

/* Scratch size of dm_pix2depth_update / dm_pix2depth_bwd_wrt_vtx2xyz (the
 * world->ndc matrix, inverted on the device). */
size_t dm_render_scratch_bytes(void);

/* Depth (ndc z + 1) / 2 of each pixel's hit point; 0 on the background.
 * Replaces: del-msh-dlpack/src/pix2depth.rs:15-97 pix2depth_update (kernel
 * del-msh-cuda-kernels/cuda/pix2depth.cu:12-50 fwd; CPU
 * del-msh-cpu/src/pix2depth.rs:107-146).  The inverse of the transform is
 * computed on the device (no host round trip); a singular transform raises
 * status bit 8. */
int dm_pix2depth_update(uint64_t stream_ptr, uint32_t img_w, uint32_t img_h, float* pix2depth,
                        const uint32_t* pix2tri, uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                        const float* vtx2xyz, const float* transform_ndc2world, void* scratch, size_t scratch_bytes);

/* dldw_vtx2xyz += d(pix2depth)/d(vtx2xyz)^T dldw_pix2depth.
 * Replaces: del-msh-dlpack/src/pix2depth.rs:100-189 pix2depth_bwd_wrt_vtx2xyz
 * (kernel pix2depth.cu:52-97 bwd_wrt_vtx2xyz). */
int dm_pix2depth_bwd_wrt_vtx2xyz(uint64_t stream_ptr, uint32_t img_w, uint32_t img_h, float* dldw_vtx2xyz,
                                 const uint32_t* pix2tri, uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                                 const float* vtx2xyz, const float* dldw_pix2depth, const float* transform_ndc2world,
                                 void* scratch, size_t scratch_bytes);

/* pix2val[p] = bc0 vtx2val[i0] + bc1 vtx2val[i1] + bc2 vtx2val[i2] with the
 * barycentric coordinates of the pixel ray on its triangle; 0 on the
 * background.  pix2val is f32[img_h][img_w][num_vdim].
 * Replaces: del-msh-dlpack/src/pix2tri.rs:96-177 pix2tri_interpolate (kernel
 * pix2tri.cu:79-120 interpolate; CPU del-msh-cpu/src/pix2tri.rs:176-226). */
int dm_pix2tri_interpolate(uint64_t stream_ptr, uint32_t img_w, uint32_t img_h, const uint32_t* pix2tri,
                           uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx, const float* vtx2xyz,
                           uint32_t num_vdim, const float* vtx2val, const float* transform_ndc2world, float* pix2val);

/* Backward of dm_pix2tri_interpolate: adds to dldw_vtx2xyz (f32[V][3]) and
 * dldw_vtx2val (f32[V][num_vdim]).
 * Replaces: del-msh-dlpack/src/pix2tri.rs:179-270 pix2tri_interpolate_bwd
 * (kernel pix2tri.cu:122-183 interpolate_bwd; CPU pix2tri.rs:228-304). */
int dm_pix2tri_interpolate_bwd(uint64_t stream_ptr, uint32_t img_w, uint32_t img_h, const uint32_t* pix2tri,
                               uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx, const float* vtx2xyz,
                               uint32_t num_vdim, const float* vtx2val, const float* transform_ndc2world,
                               const float* dldw_pix2val, float* dldw_vtx2xyz, float* dldw_vtx2val);

/* Self-intersecting triangle pairs of a mesh through its BVH: for each pair
 * (i, j) (the triangle of the left subtree first) the segment (p0, p1) where
 * they cross.  Pairs sharing two vertices are never reported; a pair sharing
 * one vertex reports the segment from that vertex to where an opposite edge
 * pierces the other triangle.  *count (device u32) receives the number of
 * pairs, which may exceed `capacity`, in which case only `capacity` pairs are
 * written (call again with a larger buffer).  The list is unordered.  The
 * search runs depth-first per thread (192-entry node-pair stack; status bit
 * 2 if one overflows) in rounds that rebalance the remaining work; each round
 * reads the next round's size back to the host, so the call synchronizes the
 * stream.  Its working memory (16 MB per million triangles, at least 16 MB)
 * comes from cudaMallocAsync.
 * Replaces: del-msh-cpu/src/trimesh3_intersection.rs:86-179
 * search_with_bvh_inside_branch (binding del-msh-numpy/src/mesh_intersection.rs). */
int dm_trimesh3_self_intersection(uint64_t stream_ptr, uint32_t num_tri, const uint32_t* tri2vtx, uint32_t num_vtx,
                                  const float* vtx2xyz, const uint32_t* bvhnodes, const float* bvhnode2aabb,
                                  uint32_t capacity, uint32_t* pairs, float* segments, uint32_t* count);

/* ---- quad/oct-trees from the binary radix tree of sorted unique Morton codes ----
 * Layouts of del-msh-cpu/src/quad_oct_tree.rs: bnodes u32[num_idx-1][3]
 * (branch links; a leaf child i is encoded num_idx-1+i), onodes
 * u32[num_onode][1 + 2^num_dim] (parent, then children; a leaf child idx is
 * encoded num_onode+idx, no child = u32::MAX), centres f32[.][num_dim]. */

/* Scratch size of dm_quad_oct_tree_bnodes_and_bnode2depth_and_bnode2onode_and_idx2bnode. */
size_t dm_quad_oct_tree_scratch_bytes(uint32_t num_idx);

/* Binary radix tree with per-branch depth, the branch -> octree-node map
 * (exclusive scan of "depth differs from the parent's") and each leaf's
 * parent branch.  num_onode = bnode2onode[num_idx-2] + 1.
 * Replaces: del-msh-dlpack/src/quad_oct_tree.rs:22-123 (kernels
 * quad_oct_tree.cu:26-101 + a cumsum; CPU quad_oct_tree.rs:2-50,88-125). */
int dm_quad_oct_tree_bnodes_and_bnode2depth_and_bnode2onode_and_idx2bnode(
    uint64_t stream_ptr, uint32_t num_idx, const uint32_t* idx2morton, uint32_t num_dim, uint32_t max_depth,
    uint32_t* bnodes, uint32_t* bnode2depth, uint32_t* bnode2onode, uint32_t* idx2bnode, void* scratch,
    size_t scratch_bytes);

/* The quad/oct-tree.  onodes must be filled with u32::MAX and onode2depth
 * with 0 beforehand (as the reference's wrapper does).
 * Replaces: del-msh-dlpack/src/quad_oct_tree.rs:125-224 (kernel
 * quad_oct_tree.cu:103-205; CPU quad_oct_tree.rs:127-233). */
int dm_quad_oct_tree_make_tree_from_binary_radix_tree(
    uint64_t stream_ptr, uint32_t num_idx, const uint32_t* bnodes, const uint32_t* bnode2onode,
    const uint32_t* bnode2depth, const uint32_t* idx2bnode, const uint32_t* idx2morton, uint32_t num_dim,
    uint32_t max_depth, uint32_t num_onode, uint32_t* onodes, uint32_t* onode2depth, float* onode2center,
    uint32_t* idx2onode, float* idx2center);

/* onode2aggval[n] = sum of idx2val over the leaves below octree node n
 * (zeroed first; added with atomics).
 * Replaces: del-msh-dlpack/src/quad_oct_tree.rs:226-290 (kernel
 * quad_oct_tree.cu:207-233; CPU quad_oct_tree.rs:420-451). */
int dm_quad_oct_tree_aggregate(uint64_t stream_ptr, uint32_t num_idx, uint32_t num_vdim, const float* idx2val,
                               const uint32_t* idx2onode, uint32_t num_link, const uint32_t* onodes,
                               uint32_t num_onode, float* onode2aggval);

/* ---- batches: many independent meshes of uneven sizes in one call ----
 * The meshes are stored back to back.  mesh2tri / mesh2vtx are device
 * u32[num_mesh+1] prefix offsets (mesh m owns triangles mesh2tri[m] ..
 * mesh2tri[m+1]-1 and vertices mesh2vtx[m] .. mesh2vtx[m+1]-1; every mesh has
 * at least one triangle), and tri2vtx holds vertex indices local to each
 * mesh.  Mesh m's tree occupies nodes 2*mesh2tri[m]-m .. 2*mesh2tri[m+1]-m-2
 * of bvhnodes / bvhnode2aabb, with node and triangle indices local to the
 * mesh: each slice is bit for bit what dm_trimesh3_make_bvhnodes_bvhnode2aabb
 * returns for that mesh alone.  All launches are stream-ordered with no host
 * synchronization, so a sequence of batch calls given caller scratch can be
 * captured in a CUDA graph.  No reference counterpart: the reference builds
 * and casts one mesh per call (TriMesh3/torch.py:233-285, Pix2Tri/torch.py:8-61). */

/* Builds every mesh's LBVH.  heights (optional, device u32[num_mesh]) gets
 * each tree's height.  max_tri_per_mesh bounds the largest mesh.  Up to
 * 65536, each mesh is sorted and linked in on-chip memory by one block or one
 * cluster of blocks, and a mesh with more triangles than max_tri_per_mesh
 * raises device status bit 4 and gets a placeholder tree (branch i: leaf i
 * and branch i+1).  Above 65536, all meshes go through one global sort of
 * (mesh, code) keys, which has no per-mesh bound. */
int dm_batch_trimesh3_build(uint64_t stream_ptr, uint32_t num_mesh, const uint32_t* mesh2tri,
                            const uint32_t* mesh2vtx, uint32_t total_tri, uint32_t total_vtx,
                            uint32_t max_tri_per_mesh, const uint32_t* tri2vtx, const float* vtx2xyz,
                            uint32_t* bvhnodes, float* bvhnode2aabb, uint32_t* heights, void* scratch,
                            size_t scratch_bytes);
size_t dm_batch_build_scratch_bytes(uint32_t num_mesh, uint32_t total_tri);

/* Casts an img_w x img_h image per mesh through that mesh's column-major
 * transforms_ndc2world[16*m .. 16*m+15]; pix2tri / pix2t (optional) hold
 * num_mesh images of img_h x img_w, pixel p of mesh m at m*img_w*img_h + p.
 * max_tri_per_mesh bounds the largest mesh (it sizes the deep-stack pool). */
int dm_batch_pix2tri_by_raycast(uint64_t stream_ptr, uint32_t num_mesh, const uint32_t* mesh2tri,
                                const uint32_t* mesh2vtx, uint32_t total_tri, uint32_t total_vtx,
                                uint32_t max_tri_per_mesh, const uint32_t* tri2vtx, const float* vtx2xyz,
                                const uint32_t* bvhnodes, const float* bvhnode2aabb, uint32_t img_w, uint32_t img_h,
                                const float* transforms_ndc2world, uint32_t* pix2tri, float* pix2t, void* scratch,
                                size_t scratch_bytes);
size_t dm_batch_cast_scratch_bytes(uint32_t num_ray, uint32_t max_tri_per_mesh);

/* ---- serving: a request server keeping built trees resident in HBM ----
 * No reference counterpart (del-msh has no serving loop).  A dispatcher thread
 * admits each submitted request when one of num_slots slots (a CUDA stream
 * with preallocated scratch) is free and the request's mesh is resident,
 * evicting least-recently-used idle meshes to stay under budget_bytes;
 * admitted requests run concurrently.  A mesh's tree topology is always built
 * from its rest pose and `frame` selects the vertex state (0 = rest, f > 0 =
 * rest + deform_amplitude*sin(phase_v + f + axis), phase_v a hash of the
 * mesh's deform_seed and v), so every result is a pure function of its
 * request: the same bits alone or in any mix.  Host arrays of a request must
 * stay valid until it completes (pinned memory keeps the copies
 * asynchronous). */
#define DM_REQ_BUILD_CAST 0u /* full build from the rest pose, state -> frame, pixel cast */
#define DM_REQ_REFIT_CAST 1u /* state -> frame by refitting the resident tree, pixel cast */
#define DM_REQ_CAST_RAYS 2u  /* state -> frame if needed, cast of explicit rays */

typedef struct dm_request {
  uint32_t kind;
  uint32_t mesh_id;
  uint32_t frame;
  float deform_amplitude;
  uint32_t img_w, img_h;              /* pixel casts */
  uint32_t num_ray;                   /* DM_REQ_CAST_RAYS */
  uint32_t reserved;
  const float* transform_ndc2world;   /* host, 16 floats column-major (pixel casts) */
  const float* ray_org;               /* host, num_ray*3 (DM_REQ_CAST_RAYS) */
  const float* ray_dir;               /* host, num_ray*3 */
  uint32_t* out_tri;                  /* host, one hit id per pixel / ray (u32::MAX = miss) */
  float* out_t;                       /* host, hit t per pixel / ray (+inf = miss), may be NULL */
} dm_request;

typedef struct dm_result {
  int32_t status;
  uint32_t resident_hit;              /* 1 if the mesh's tree was resident and built at admission */
  uint64_t t_submit_ns, t_admit_ns, t_done_ns;  /* steady clock */
} dm_result;

typedef struct dm_server_stats {
  uint64_t submitted, completed, resident_hits, builds, refits, evictions;
  uint64_t bytes_resident, bytes_budget, bytes_slots;
  uint32_t meshes_resident, reserved;
} dm_server_stats;

typedef struct dm_server dm_server;

/* max_tri: largest mesh to be registered; max_out: most pixels / rays of one request. */
int dm_server_create(int device, size_t budget_bytes, int num_slots, uint32_t max_tri, uint32_t max_out,
                     dm_server** out);
/* Copies the mesh into server-owned pinned host memory. */
int dm_server_register_mesh(dm_server* server, uint32_t mesh_id, const uint32_t* tri2vtx, uint32_t num_tri,
                            const float* vtx2xyz, uint32_t num_vtx, uint32_t deform_seed);
int dm_server_submit(dm_server* server, const dm_request* req, uint64_t* ticket);
/* Blocks until the request completes; returns its status. */
int dm_server_wait(dm_server* server, uint64_t ticket, dm_result* out);
/* Submits reqs[i] at arrival_s[i] seconds after the start (an open-loop
 * arrival trace), waits for all; latencies count from the scheduled arrival. */
int dm_server_run_trace(dm_server* server, uint32_t n, const dm_request* reqs, const double* arrival_s,
                        dm_result* results);
/* The same trace the straightforward way: one request at a time, each
 * uploading its mesh, building, refitting to its frame, casting and
 * downloading, synchronizing before the next; nothing stays resident. */
int dm_plain_run_trace(dm_server* server, uint32_t n, const dm_request* reqs, const double* arrival_s,
                       dm_result* results);
int dm_server_stats_get(dm_server* server, dm_server_stats* out);
int dm_server_destroy(dm_server* server);

#ifdef __cplusplus
}
#endif
#endif /* DELMSH_GB300_H */
