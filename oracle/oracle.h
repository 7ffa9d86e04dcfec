/*
 * oracle.h — CPU restatement of del-msh-cpu's LBVH build and BVH ray cast.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py may load this library, and only as
 * what results are tested against or as the timed CPU baseline.  The product (the CUDA library under
 * del-msh_gb300/) never calls it and has no CPU fallback.
 *
 * Every function names the reference file:line it follows (paths relative to
 * the del-msh repository).  Floating point is IEEE binary32 with no FMA
 * contraction (built with -ffp-contract=off), which is what Rust emits.
 *
 * Parity pins:
 *   - morton_code3 / expand_bits3: known answers of del-msh-cpu/src/mortons.rs
 *     tests, plus golden vectors produced by the reference's own
 *     del-msh-cuda-kernels/cuda/mortons.h compiled as host code (oracle/_ref).
 *   - radix-tree topology: golden vectors produced by the reference's
 *     kernel_MortonCode_BVHTopology (bvhnodes_morton.cu) compiled as host
 *     code, plus the invariant checkers of mortons.rs / bvhnodes.rs.
 *   - ray/triangle, ray/AABB, fit transform and transform_homogeneous live in
 *     the un-vendored del-geo-core crate: their f32 operation order is
 *     "parity unpinned"; the formulas below are the published methods named
 *     at each function and are the contract the GPU path matches bit for bit.
 */
#ifndef DELMSH_ORACLE_H
#define DELMSH_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* mortons.rs:76-81 */
uint32_t or_expand_bits3(uint32_t x);
/* mortons.rs:94-102 */
uint32_t or_morton_code3(float x, float y, float z);
/* mortons.rs:3-8 and 20-27 */
uint32_t or_morton_code2(float x, float y);

/* elem2center.rs:25-54 (num_node = 3, num_dim = 3) */
void or_tri2cntr(uint32_t num_tri, const uint32_t* tri2vtx, const float* vtx2xyz, float* tri2cntr);

/* vtx2xyz.rs:19-37 with eps = 0 */
void or_aabb3(uint32_t num_pnt, const float* pnt2xyz, float aabb[6]);

/* from_aabb3_fit_into_unit_preserve_asp (del-geo-core, absent); formula of
 * del-msh-dlpack/del_msh_dlpack/Mat44/torch.py:120-140.  Column-major. */
void or_fit_into_unit_preserve_asp(const float aabb[6], float m[16]);

/* mat4_col_major::transform_homogeneous (del-geo-core, absent). */
void or_transform_homogeneous(const float m[16], const float p[3], float out[3]);

/* mortons.rs:171-212 (num_dim 2 or 3; transform is column-major 3x3 / 4x4) */
void or_vtx2morton(uint32_t num_vtx, uint32_t num_dim, const float* vtx2co, const float* transform,
                   uint32_t* vtx2morton);

/* mortons.rs:139-146: stable argsort of codes (ties keep ascending index). */
void or_argsort_stable(uint32_t n, const uint32_t* vtx2morton, uint32_t* idx2vtx, uint32_t* idx2morton);

/* mortons.rs:221-288 and 290-325 */
void or_range_of_binary_radix_tree_node(const uint32_t* idx2morton, uint32_t n, uint32_t idx, uint32_t* r0,
                                        uint32_t* r1);
uint32_t or_split_of_binary_radix_tree_node(const uint32_t* idx2morton, uint32_t start, uint32_t end);

/* bvhnodes_morton.rs:10-50.  bvhnodes is u32[(2n-1)*3]. */
void or_update_bvhnodes(uint32_t n, const uint32_t* idx2vtx, const uint32_t* idx2morton, uint32_t* bvhnodes);

/* bvhnodes_morton.rs:151-185 + mortons.rs:354-382: centroids, AABB, fit,
 * Morton, stable sort, topology.  Optional outputs may be NULL. */
void or_bvhnodes_from_triangle_mesh(uint32_t num_tri, const uint32_t* tri2vtx, const float* vtx2xyz,
                                    uint32_t* bvhnodes, float* transform_out, uint32_t* tri2morton_out,
                                    uint32_t* idx2tri_out, uint32_t* idx2morton_out);

/* bvhnode2aabb3.rs:68-142 (recursive from node i_bvhnode); vtx2xyz1 may be NULL. */
void or_update_aabb_uniform_mesh(float* bvhnode2aabb, uint32_t i_bvhnode, const uint32_t* bvhnodes,
                                 const uint32_t* tri2vtx, const float* vtx2xyz0, const float* vtx2xyz1);

/* ray_for_pixel.h:3-19 (GPU twin of
 * mat4_col_major::ray_from_transform_ndc2world_and_pixel_coordinates). */
void or_ray_for_pixel(uint32_t i_pix, uint32_t img_w, uint32_t img_h, const float t_ndc2world[16], float org[3],
                      float dir[3]);

/* tri3::intersection_against_ray (del-geo-core, absent): Moller-Trumbore.
 * Returns 1 on hit and writes t (and barycentrics when bc != NULL). */
int or_tri3_ray(const float p0[3], const float p1[3], const float p2[3], const float org[3], const float dir[3],
                float* t, float bc[3]);
/* Same formula in binary64, for error reporting only. */
int or_tri3_ray_f64(const float p0[3], const float p1[3], const float p2[3], const float org[3], const float dir[3],
                    double* t);

/* aabb3::intersections_against_ray (del-geo-core, absent): slab test. */
int or_aabb3_ray(const float aabb[6], const float org[3], const float inv_dir[3], const float dir[3], float* t_enter,
                 float* t_exit);

/* search_bvh3.rs:103-221.  Returns 1 on hit. */
int or_first_intersection_ray(const float org[3], const float dir[3], const uint32_t* tri2vtx, const float* vtx2xyz,
                              const uint32_t* bvhnodes, const float* bvhnode2aabb, uint32_t i_bvhnode, float dis,
                              float* t_out, uint32_t* tri_out);

/* search_bvh3.rs:12-53: every hit along the ray (t, tri) in DFS order.
 * Returns the number of hits (writes at most cap). */
uint32_t or_intersections_ray(const float org[3], const float dir[3], const uint32_t* tri2vtx, const float* vtx2xyz,
                              const uint32_t* bvhnodes, const float* bvhnode2aabb, float* hit_t, uint32_t* hit_tri,
                              uint32_t cap);

/* pix2tri.rs:3-48 (rayon par_iter over pixels -> num_threads pthreads).
 * pix2t may be NULL; misses get u32::MAX and +inf. */
void or_pix2tri_by_raycast(uint32_t img_w, uint32_t img_h, const float t_ndc2world[16], const uint32_t* tri2vtx,
                           const float* vtx2xyz, const uint32_t* bvhnodes, const float* bvhnode2aabb,
                           uint32_t* pix2tri, float* pix2t, int num_threads);

/* first_intersection_ray over an array of rays (org/dir u32[n*3]). */
void or_cast_rays(uint32_t num_ray, const float* ray_org, const float* ray_dir, const uint32_t* tri2vtx,
                  const float* vtx2xyz, const uint32_t* bvhnodes, const float* bvhnode2aabb, uint32_t* hit_tri,
                  float* hit_t, int num_threads);

/* bvhnodes.rs:22-36 (1 = ok) */
int or_check_bvh_topology(const uint32_t* bvhnodes, uint32_t num_leaf);
/* mortons.rs:330-352 (1 = ok) */
int or_check_morton_code_range_split(const uint32_t* idx2morton, uint32_t n);

/* Height of the tree (number of nodes on the longest root-to-leaf path). */
/* first_hit's work over a pixel grid (one thread): rays, branches entered,
 * triangles tested */
void or_pix2tri_work(uint32_t img_w, uint32_t img_h, const float t_ndc2world[16], const uint32_t* tri2vtx,
                     const float* vtx2xyz, const uint32_t* bvhnodes, const float* bvhnode2aabb, uint64_t out[3]);
void or_pix2tri_work_depth(uint32_t img_w, uint32_t img_h, const float t_ndc2world[16], const uint32_t* tri2vtx,
                           const float* vtx2xyz, const uint32_t* bvhnodes, const float* bvhnode2aabb, uint64_t out[3],
                           uint64_t* by_depth, uint32_t max_depth);

/* consumers of a pix2tri image (pix2depth.rs:107-146, pix2tri.rs:176-304) */
int or_mat4_inverse_pivot(const float m[16], float inv[16]);
/* pix2tri.rs:50-119 (scanline walk over pixel centres restated); returns 0
 * when transform_ndc2world is singular. */
int or_pix2tri_by_rasterization(uint32_t img_w, uint32_t img_h, const float t_ndc2world[16], uint32_t num_tri,
                                const uint32_t* tri2vtx, const float* vtx2xyz, uint32_t* pix2tri, float* pix2depth);
int or_pix2depth(uint32_t img_w, uint32_t img_h, float* pix2depth, const uint32_t* pix2tri, uint32_t num_tri,
                 const uint32_t* tri2vtx, uint32_t num_vtx, const float* vtx2xyz, const float ndc2world[16]);
int or_pix2depth_bwd(uint32_t img_w, uint32_t img_h, float* dldw_vtx2xyz, const uint32_t* pix2tri, uint32_t num_tri,
                     const uint32_t* tri2vtx, uint32_t num_vtx, const float* vtx2xyz, const float* dldw_pix2depth,
                     const float ndc2world[16]);
void or_interpolate(uint32_t img_w, uint32_t img_h, const uint32_t* pix2tri, uint32_t num_tri, const uint32_t* tri2vtx,
                    uint32_t num_vtx, const float* vtx2xyz, uint32_t num_vdim, const float* vtx2val,
                    const float ndc2world[16], float* pix2val);
void or_interpolate_bwd(uint32_t img_w, uint32_t img_h, const uint32_t* pix2tri, uint32_t num_tri,
                        const uint32_t* tri2vtx, uint32_t num_vtx, const float* vtx2xyz, uint32_t num_vdim,
                        const float* vtx2val, const float ndc2world[16], const float* dldw_pix2val,
                        float* dldw_vtx2xyz, float* dldw_vtx2val);

/* quad/oct-trees (quad_oct_tree.rs) */
void or_qot_binary_radix_tree_and_depth(uint32_t num_idx, const uint32_t* idx2morton, uint32_t num_dim,
                                        uint32_t max_depth, uint32_t* bnodes, uint32_t* bnode2depth);
void or_qot_bnode2onode_and_idx2bnode(uint32_t num_idx, const uint32_t* bnodes, const uint32_t* bnode2depth,
                                      uint32_t* bnode2onode, uint32_t* idx2bnode);
void or_qot_make_tree(uint32_t num_idx, const uint32_t* bnodes, const uint32_t* b2o, const uint32_t* b2d,
                      const uint32_t* idx2bnode, const uint32_t* idx2morton, uint32_t num_onode, uint32_t max_depth,
                      uint32_t num_dim, uint32_t* onodes, uint32_t* onode2depth, float* onode2center,
                      uint32_t* idx2onode, float* idx2center);
void or_qot_aggregate(uint32_t num_idx, uint32_t num_vdim, const float* idx2val, const uint32_t* idx2onode,
                      uint32_t num_link, const uint32_t* onodes, uint32_t num_onode, float* onode2aggval);
int or_qot_check(uint32_t num_idx, uint32_t num_dim, const uint32_t* idx2onode, const float* idx2center,
                 const uint32_t* onodes, const uint32_t* onode2depth, const float* onode2center, uint32_t num_onode,
                 uint32_t max_depth);

/* self-intersection (trimesh3_intersection.rs) */
int or_tri_pair_segment(const uint32_t* tri2vtx, const float* vtx2xyz, uint32_t it, uint32_t jt, float p0[3],
                        float p1[3]);
uint32_t or_self_intersection(const uint32_t* tri2vtx, const float* vtx2xyz, const uint32_t* bvhnodes,
                              const float* aabb, uint32_t cap, uint32_t* pairs, float* segs);
uint32_t or_self_intersection_brute(uint32_t num_tri, const uint32_t* tri2vtx, const float* vtx2xyz, uint32_t cap,
                                    uint32_t* pairs, float* segs);

uint32_t or_tree_height(const uint32_t* bvhnodes, uint32_t num_leaf);

#ifdef __cplusplus
}
#endif
#endif
