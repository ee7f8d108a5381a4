/* rrgpu_batch.h -- uneven batches of meshes and ray sets on one GPU.
 *
 * The reference answers "many meshes, each with its own rays" with one
 * RRCollider per mesh (RRCollider::create, RRCollider/RRCollider.cpp:186-241;
 * one BSP build each, bsp.cpp:1192) and a loop of intersect() calls
 * (RRCollider.h:228), or, for objects of one scene, RRColliderMulti's loop
 * over per-object colliders (RRCollider/RRColliderMulti.cpp:103-147).  Here
 * all meshes are built in one multi-root BVH build (mesh m's root is node m;
 * every level of every mesh's tree goes through the same level loop) and all
 * rays are answered by one persistent closest-hit launch, replayed from a
 * CUDA graph.  Per-ray results are those of rrg_intersect_device on a
 * collider of the ray's own mesh alone (same hit record format, triangle
 * indices local to the mesh).
 */
#ifndef RRGPU_BATCH_H
#define RRGPU_BATCH_H
#include "rrgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rrg_batch rrg_batch;

/* Largest number of meshes in one batch. */
#define RRG_BATCH_MAX_MESHES 8192u

/* Creates a batch of nmesh meshes from host arrays.  vert_off and tri_off
 * hold nmesh+1 ascending offsets (vert_off[0] = tri_off[0] = 0): mesh m's
 * vertices are xyz[3*vert_off[m] .. 3*vert_off[m+1]) and its triangles
 * idx[3*tri_off[m] .. 3*tri_off[m+1]), with vertex indices local to the
 * mesh (0 .. vert_off[m+1]-vert_off[m]-1).  A mesh may be empty or have no
 * valid triangle (its rays then miss); an index outside its mesh is
 * RRG_ERR_INVALID.  params as for rrg_collider_create (max_leaf_size). */
RRG_API int rrg_batch_create(const float* xyz, const uint32_t* vert_off, const uint32_t* idx,
                             const uint32_t* tri_off, uint32_t nmesh, const rrg_build_params* params, int device,
                             rrg_batch** out);

RRG_API void rrg_batch_destroy(rrg_batch* b);

/* Rays fetched by a warp per work-counter atomic: 32, 64, 128 or 256
 * (default 32).  The autotuner's rays-per-warp knob. */
RRG_API int rrg_batch_set_rays_per_warp(rrg_batch* b, uint32_t rays_per_warp);

/* Traversal-stack entries per thread kept in shared memory by the batch's
 * closest-hit kernel: 0 (the whole stack in local memory, default), 8, 16
 * or 32 (deeper entries in local memory); binary trees only (the 8-wide
 * walk keeps its own stack).  The autotuner's stack-depth knob; results do
 * not depend on it. */
RRG_API int rrg_batch_set_stack_smem(rrg_batch* b, uint32_t entries);

/* Root-box queue of the batch's closest-hit kernel (binary trees; on = 1):
 * rays that enter neither child box of their mesh's root are answered at
 * once and the others traced 32 to a warp, for rays around meshes most of
 * which pass them by.  A tuning knob; results do not depend on it. */
RRG_API int rrg_batch_set_root_queue(rrg_batch* b, int on);

/* Closest hit for n device rays (float[8] each, as rrg_intersect_device);
 * ray_off_dev = nmesh+1 ascending device offsets, ray_off[nmesh] = n: ray i
 * belongs to the mesh m with ray_off[m] <= i < ray_off[m+1].  Writes one hit
 * record (float4) per ray: (hitDistance, hitTriangle local to the mesh |
 * hitFrontSide << 31, u, v), 0xFFFFFFFF = no hit.  Asynchronous on `stream`:
 * the counter reset and the persistent kernel are replayed from a CUDA graph,
 * captured on the first call and again whenever rays, offsets, n, hits or
 * the rays-per-warp or stack setting change.  Calls on the same batch must not
 * overlap on the GPU (they share its work counter).  n < 2^31. */
RRG_API int rrg_batch_intersect_device(rrg_batch* b, const float* rays_dev, const uint32_t* ray_off_dev, uint32_t n,
                                       float* hits_dev, void* stream);

/* New vertex positions for every mesh (same topology): xyz_dev in the
 * layout of rrg_batch_create's xyz (3 floats per vertex, all meshes in
 * order), copied on `stream`.  Queries of rrg_batch_intersect_device keep
 * the trees built at create; rrg_batch_rebuild_intersect_device rebuilds
 * from these positions. */
RRG_API int rrg_batch_set_vertices_device(rrg_batch* b, const float* xyz_dev, void* stream);

/* Rebuilds every mesh's tree from the batch's current vertex positions and
 * traces the rays against the new trees, both in one CUDA graph replay:
 * the build runs as a fixed sequence of launches whose counts (valid
 * triangles, tasks per tree level, nodes) stay on the device, with its
 * scratch allocated on the first call (about 350 bytes per triangle) and
 * at most 40 levels of large build tasks; then the persistent closest-hit
 * launch of rrg_batch_intersect_device on those trees.  The graph is
 * captured on the first call and again whenever rays, offsets, n, hits or
 * the rays-per-warp or stack setting change.  Binary trees only
 * (bvh_width 2): RRG_ERR_INVALID for 8-wide batches.  Results are
 * rrg_batch_intersect_device's on trees built from the same positions;
 * rrg_batch_status also reports a failed rebuild (RRG_ERR_INVALID).  The
 * reference builds each mesh's collider once on the host
 * (RRCollider::create per mesh, RRCollider.cpp:186-241; RRCollider::update
 * rebuilds one, RRCollider.h:187-190). */
RRG_API int rrg_batch_rebuild_intersect_device(rrg_batch* b, const float* rays_dev, const uint32_t* ray_off_dev,
                                               uint32_t n, float* hits_dev, void* stream);

/* Status word of the batch's traces (RRG_OK or RRG_ERR_STACK); synchronises
 * the stream and resets the word. */
RRG_API int rrg_batch_status(rrg_batch* b, void* stream);

RRG_API uint32_t rrg_batch_meshes(const rrg_batch* b);
RRG_API uint32_t rrg_batch_nodes(const rrg_batch* b);
RRG_API size_t rrg_batch_memory(const rrg_batch* b);
/* Milliseconds of device time the batch's build took (CUDA events). */
RRG_API float rrg_batch_build_ms(const rrg_batch* b);

#ifdef __cplusplus
}
#endif
#endif
