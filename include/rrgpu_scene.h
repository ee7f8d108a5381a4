/* rrgpu_scene.h -- two-level scene collider: objects = instances of the
 * meshes of a batch (rrgpu_batch.h), each with a world matrix.
 *
 * Replaces RRColliderMulti (RRCollider/RRColliderMulti.cpp:59-165), the
 * reference's collider over RRObjects, and the solver's multi-object
 * collider built by RRSolver::setStaticObjects / getCollider
 * (RRSolver/RRSolver.cpp:312,475).  Semantics per object follow
 * RRColliderMulti::intersect (RRColliderMulti.cpp:103-147): the world ray is
 * taken to object space with the object's inverse world matrix
 * (RRMatrix3x4::invertedTo, RRMath.cpp:610-628: float cofactors over the
 * float determinant), transformPosition / transformDirection
 * (RRMath.cpp:194-219), its direction is normalised with scale = |d_local|
 * and rayLengthMin/Max are multiplied by scale; the object's mesh is
 * intersected as a single collider would (IT_BSP_FASTEST fields, see
 * rrgpu.h); hitDistance is divided back by scale; the nearest hit over all
 * objects wins (RayHits::getHitOrdered, IntersectLinear.cpp:396-437) and
 * hitFrontSide is flipped for objects whose matrix has a negative
 * determinant (RayHitBackup::restoreBackupTo, IntersectLinear.cpp:309-317).
 * Instead of the reference's loop over all objects, a top-level BVH over
 * the objects' world boxes (rebuilt on the host when matrices change)
 * selects the objects a ray can reach.
 *
 * Ties: equal world distances in two objects go to the lower object index
 * (the reference keeps the first object in its object order, which is the
 * same order).  hitPlane / hitPoint3d are not produced here.
 */
#ifndef RRGPU_SCENE_H
#define RRGPU_SCENE_H
#include "rrgpu.h"
#include "rrgpu_batch.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rrg_scene rrg_scene;

/* nobj objects; obj_mesh[i] = mesh of `meshes` (0 .. meshes-1), world_3x4 =
 * nobj row-major 3 x 4 float matrices (RRMatrix3x4 layout: world = M[:, :3]
 * local + M[:, 3]).  The batch must outlive the scene.  A matrix with a zero
 * determinant (no inverse) is RRG_ERR_INVALID. */
RRG_API int rrg_scene_create(rrg_batch* meshes, uint32_t nobj, const uint32_t* obj_mesh, const float* world_3x4,
                             rrg_scene** out);
RRG_API void rrg_scene_destroy(rrg_scene* s);

/* New world matrices for all objects (objects moved): inverses and the
 * top-level BVH are rebuilt; the meshes' BVHs are untouched
 * (RRCollider::update of a multi-object collider, RRCollider.h:190). */
RRG_API int rrg_scene_set_matrices(rrg_scene* s, const float* world_3x4);

/* Objects with enabled[i] == 0 are skipped (RRObject::enabled,
 * RRColliderMulti.cpp:121). */
RRG_API int rrg_scene_set_enabled(rrg_scene* s, const uint8_t* enabled);

/* Closest hit for n device rays in world space (float[8] each, as
 * rrg_intersect_device): hits_dev one float4 per ray (hitDistance, hitTriangle
 * local to the object's mesh | hitFrontSide << 31, u, v), 0xFFFFFFFF = no
 * hit; objects_dev (may be NULL) the hit object's index (hitObject), or
 * 0xFFFFFFFF.  Asynchronous on `stream`. */
RRG_API int rrg_scene_intersect_device(rrg_scene* s, const float* rays_dev, uint32_t n, float* hits_dev,
                                       uint32_t* objects_dev, void* stream);

/* Host buffers in, host buffers out (synchronous): n rays (float[8] each)
 * -> n hit records and, when objects_host is not NULL, n hit objects, as
 * rrg_scene_intersect_device.  Staging buffers belong to the scene and grow
 * on demand; host threads that call it on one scene take turns.  Returns the
 * traces' status (RRG_ERR_STACK on a traversal overflow).  The query of
 * RRColliderMulti::intersect for callers holding rays on the host
 * (RRColliderMulti.cpp:103-147). */
RRG_API int rrg_scene_intersect_host(rrg_scene* s, const float* rays_host, uint32_t n, float* hits_host,
                                     uint32_t* objects_host);

/* Status word of the scene's traces (RRG_OK or RRG_ERR_STACK); synchronises
 * the stream and resets the word. */
RRG_API int rrg_scene_status(rrg_scene* s, void* stream);

#ifdef __cplusplus
}
#endif
#endif
