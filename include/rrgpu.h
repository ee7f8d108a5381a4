/* rrgpu.h -- C ABI of the GB300 ray-mesh collider (closest hit and any hit).
 *
 * This is the drop-in boundary for rr::RRCollider (include/Lightsprint/
 * RRCollider.h in the reference).  Everything crosses as plain pointers,
 * sizes and int status codes; no C++ or CUDA types appear in the signatures
 * (streams are passed as void* = cudaStream_t, NULL = the legacy stream).
 *
 * Ray formats
 *   device rays : float[8] per ray = ox oy oz tmin dx dy dz tmax (two float4,
 *                 16-byte aligned).  tmin/tmax are RRRay::rayLengthMin/Max.
 *   hit record  : float[4] per ray = (t, tri_bits, u, v); tri_bits is a
 *                 uint32 (read it with a bit cast): bits 0..30 = hitTriangle
 *                 (post-import index), bit 31 = hitFrontSide; 0xFFFFFFFF =
 *                 no hit.  t = hitDistance, (u, v) = hitPoint2d.
 *   rr::RRRay   : the reference's 128-byte record (rayOrigin at 0, rayDir at
 *                 16, rayLengthMin 32, rayLengthMax 36, rayFlags 40,
 *                 hitDistance 44, hitTriangle 48, hitPoint2d 52, hitPlane 60,
 *                 hitPoint3d 76, hitFrontSide 88), include/Lightsprint/
 *                 RRCollider.h:85-137.
 *
 * Output semantics follow IT_BSP_FASTEST (RRCollider/IntersectBspFast.cpp):
 * the hit triangle is the nearest one in [tmin, tmax] by a watertight test
 * (ties in distance go to the lower triangle index); hitDistance is the
 * distance to that triangle's plane, hitPoint2d its projected (u, v),
 * hitPlane its unit plane and hitFrontSide = dot(dir, normal) < 0, each
 * computed with the reference's own formulas (IntersectBspFast.cpp:130-252).
 * Triangles whose plane normal is not finite are never hit, as in the
 * reference (intersectByte 10, IntersectBspFast.cpp:182-186).
 */
#ifndef RRGPU_H
#define RRGPU_H
#include <stddef.h>
#include <stdint.h>
#if defined(_WIN32)
#define RRG_API __declspec(dllexport)
#else
#define RRG_API __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  RRCollider::create returns nullptr on failure and logs
 * (RRCollider/RRCollider.cpp:216-239); here every entry point returns one of
 * these and rrg_status_string() names it. */
enum {
	RRG_OK = 0,
	RRG_ERR_INVALID = 1,   /* bad argument (null pointer, size, alignment) */
	RRG_ERR_OOM = 2,       /* device or host allocation failed */
	RRG_ERR_CUDA = 3,      /* a CUDA call failed (rrg_last_cuda_error()) */
	RRG_ERR_STACK = 4,     /* a traversal stack overflowed (ray left unhit) */
	RRG_ERR_ABORTED = 5,   /* *aborting was set during create */
	RRG_ERR_NO_DEVICE = 6, /* no CUDA device, or not an sm_103 device */
	RRG_ERR_EMPTY = 7,     /* the mesh has no valid triangle */
	RRG_ERR_TIMEOUT = 8,   /* a bounded device wait ran out */
	RRG_ERR_TOO_LARGE = 9  /* batch above RRG_NOALLOC_MAX_RAYS (rrg_intersect_rrray_noalloc); 2^32 or more unwrap-seam runs (rrg_lightmap_filter) */
};

/* RRRay::Flags (include/Lightsprint/RRCollider.h:98-106). */
enum {
	RRG_FILL_DISTANCE = 1 << 0,
	RRG_FILL_POINT3D = 1 << 1,
	RRG_FILL_POINT2D = 1 << 2,
	RRG_FILL_PLANE = 1 << 3,
	RRG_FILL_TRIANGLE = 1 << 4,
	RRG_FILL_SIDE = 1 << 5
};

/* Build parameters, a versioned struct like the reference's BuildParams
 * (RRCollider/bsp.h:50-92), passed where RRCollider::create takes
 * `void* buildParams` (RRCollider.h:183).  size = sizeof(rrg_build_params);
 * zero fields take defaults. */
typedef struct rrg_build_params {
	uint32_t size;
	uint32_t max_leaf_size;   /* triangles per leaf, default 4, max 8 */
	uint32_t sah_bins;        /* bins per axis, default 32 (<= 32) */
	uint32_t traversal;       /* RRG_TRAVERSAL_*, 0 = default */
	uint32_t bvh_width;       /* 2 (binary) or 8 (compressed 8-wide, leaves <= 4); 0 = default */
	uint32_t reserved[3];
} rrg_build_params;

/* Traversal kernels (chosen per collider; rrg_collider_set_traversal). */
enum {
	RRG_TRAVERSAL_DEFAULT = 0,     /* RRG_TRAVERSAL_ROOT_QUEUE (on GB300: config 0 +21 %, config 1 even) */
	RRG_TRAVERSAL_IF_IF = 1,       /* warp takes 32 rays, per-thread if-if walk */
	RRG_TRAVERSAL_WHILE_WHILE = 2, /* persistent while-while, postponed leaves, per-lane refill */
	RRG_TRAVERSAL_COMPACT = 3,     /* persistent: a warp claims a block of consecutive rays and each
	                                  lane walks its share of them one after the other, with no
	                                  warp-wide step between rays; stack top in shared memory */
	RRG_TRAVERSAL_ROOT_QUEUE = 4   /* if-if, rays entering neither child box of the root answered
	                                  at once and the others queued per warp until 32 fill it
	                                  (rays around an object, most of which pass it by) */
};

typedef struct rrg_collider rrg_collider;

/* Creates a collider from host arrays: xyz = 3*nv floats, idx = 3*nt uint32
 * vertex indices (triangle i = idx[3i..3i+2], post-import numbering = i).
 * The geometry is copied to the device and a BVH is built there.  Replaces
 * RRCollider::create(mesh, nullptr, technique, aborting, ...)
 * (RRCollider.h:183, RRCollider.cpp:186-241).  `aborting` may be NULL; when
 * it becomes nonzero the build stops between levels and RRG_ERR_ABORTED is
 * returned.  device = CUDA ordinal (usually 0). */
RRG_API int rrg_collider_create(const float* xyz, uint32_t nv, const uint32_t* idx, uint32_t nt,
                        const rrg_build_params* params, const volatile int* aborting, int device,
                        rrg_collider** out);

/* Same, from device arrays (no host copy), enqueued on `stream`. */
RRG_API int rrg_collider_create_device(const float* xyz_dev, uint32_t nv, const uint32_t* idx_dev, uint32_t nt,
                               const rrg_build_params* params, const volatile int* aborting, void* stream,
                               rrg_collider** out);

/* Re-reads vertex positions (same topology) and rebuilds.  RRCollider::update
 * (RRCollider.h:187-190). */
RRG_API int rrg_collider_update(rrg_collider* c, const float* xyz_host);

RRG_API void rrg_collider_destroy(rrg_collider* c);

/* Order in which a batch's rays are traced (results do not depend on it). */
enum {
	RRG_RAY_ORDER_DEFAULT = 0,    /* binned for batches of >= 2^22 rays, else as given */
	RRG_RAY_ORDER_AS_GIVEN = 1,   /* trace ray i by ray i */
	RRG_RAY_ORDER_BINNED = 2      /* always binned: one counting-sort pass groups rays by origin
	                                 cell (8^3 over the mesh box) and direction cell (4^3) */
};
RRG_API int rrg_collider_set_ray_order(rrg_collider* c, uint32_t order);

/* Selects the traversal kernel of later queries (RRG_TRAVERSAL_*). */
RRG_API int rrg_collider_set_traversal(rrg_collider* c, uint32_t traversal);

/* Tuning of RRG_TRAVERSAL_COMPACT (the autotuner's knobs; results do not
 * depend on them):
 *   stack_smem    traversal-stack entries per thread kept in shared memory:
 *                 0, 8, 16 or 32 (deeper entries go to local memory);
 *                 RRG_COMPACT_DEFAULT = 8;
 *   rays_per_warp rays a warp claims at a time: a multiple of 32 in
 *                 32..1024; 0 = 32;
 *   blocks_per_sm 9 caps the kernel's registers (56) so that 9 blocks of
 *                 128 threads fit on an SM; 0 leaves them uncapped (62,
 *                 8 blocks); RRG_COMPACT_DEFAULT = 9. */
#define RRG_COMPACT_DEFAULT 0xFFFFFFFFu
RRG_API int rrg_collider_set_compact_tuning(rrg_collider* c, uint32_t stack_smem, uint32_t rays_per_warp,
                                            uint32_t blocks_per_sm);

/* Timing of the closest-hit traversal kernel alone (a measurement aid, no
 * reference counterpart): while enabled, each binary-tree closest-hit
 * launch of rrg_intersect_device is bracketed by CUDA events on its stream
 * (up to 256 launches).  A call returns the summed milliseconds and the
 * number of timed launches since the previous call (synchronising on their
 * events), resets them, and enables or disables the timing. */
RRG_API int rrg_collider_trace_timing(rrg_collider* c, int enable, float* total_ms, uint32_t* launches);

/* RRCollider::getMemoryOccupied (RRCollider.h:259): device bytes held. */
RRG_API size_t rrg_collider_memory(const rrg_collider* c);
RRG_API uint32_t rrg_collider_triangles(const rrg_collider* c);
RRG_API uint32_t rrg_collider_valid_triangles(const rrg_collider* c);
RRG_API uint32_t rrg_collider_nodes(const rrg_collider* c);
/* Milliseconds of device time the last build took (CUDA events). */
RRG_API float rrg_collider_build_ms(const rrg_collider* c);

/* Closest hit for n device rays -> n device hit records (float4 each).
 * planes_dev (float4 per ray) and points_dev (float[3] per ray) are optional
 * (NULL = not written; they correspond to FILL_PLANE / FILL_POINT3D).
 * Asynchronous on `stream`; the status covers launch errors only.  Batch form
 * of RRCollider::intersect(RRRay&) (RRCollider.h:228).  Launches on one
 * collider share its work counter and ray-binning scratch: do not let two of
 * them overlap on the GPU (issue them on one stream, or synchronise). */
RRG_API int rrg_intersect_device(rrg_collider* c, const float* rays_dev, uint32_t n, float* hits_dev,
                         float* planes_dev, float* points_dev, void* stream);

/* Any hit (shadow rays): occluded_dev[i] = 1 if any valid triangle is hit in
 * [tmin, tmax], else 0.  The reference answers shadow rays with intersect()
 * and a collision handler (RRSolver/gather.cpp:447,
 * RRStaticSolver/pathtracer.cpp:293); without a handler any hit suffices. */
RRG_API int rrg_occluded_device(rrg_collider* c, const float* rays_dev, uint32_t n, uint8_t* occluded_dev,
                        void* stream);

/* Host buffers in, host buffers out; synchronous.  Up to 4,194,304 rays in
 * page-locked host memory (cudaHostAlloc / cudaHostRegister, both buffers
 * 16-byte aligned): the kernel reads the rays and writes the hit records in
 * host memory directly over the host link (the if-if kernel in the given
 * order, whatever the collider's traversal setting, so that each warp
 * writes one contiguous run of records).  Otherwise the rays are copied to
 * device staging buffers owned by the collider (grown on demand), traced and
 * copied back: batches above 262,144 rays in chunks (of 4 Mi rays, or four
 * below that) whose copies overlap the tracing of the neighbouring chunks
 * (the overlap needs page-locked host buffers).  Host threads that call this or rrg_intersect_rrray on one
 * collider at once take turns. */
RRG_API int rrg_intersect_host(rrg_collider* c, const float* rays_host, uint32_t n, float* hits_host, void* stream);

/* rr::RRRay array on the host (128-byte stride): reads rayOrigin, rayDir,
 * rayLengthMin/Max and rayFlags, writes the outputs the flags request and
 * hit_host[i] = the bool RRCollider::intersect would return (hit_host may be
 * NULL).  The batch form the reference once had as intersectBatch
 * (doc/doxygen/doc.news:154).  Synchronous. */
RRG_API int rrg_intersect_rrray(rrg_collider* c, void* rrrays_host, uint32_t n, uint8_t* hit_host, void* stream);

/* One rr::RRRay on the host, from any number of host threads at once: the
 * contract of RRCollider::intersect(RRRay&), thread-safe and stateless
 * (RRCollider.h:145,217-228), whose callers run it from OpenMP loops
 * (RRSolver/gather.cpp:917, RRSolver/lightmap.cpp:368).  Calls that arrive
 * while the collider's four combining slots are busy are combined into one
 * batch, traced on a slot's own stream and buffers, so throughput grows with
 * the number of calling threads.  Reads and writes the same fields as
 * rrg_intersect_rrray; *hit_host (may be NULL) = what intersect() returns.
 * Synchronous; does not race with the other entry points of the collider.
 * RRG_ERR_STACK if a traversal stack overflowed anywhere in the batch the ray
 * went with (that ray may then be left unhit). */
RRG_API int rrg_intersect_rrray_one(rrg_collider* c, void* rrray_host, uint8_t* hit_host);

/* The next hit of one rr::RRRay after a hit that a collision handler
 * rejected: the nearest hit (t, triangle) in [rayLengthMin, rayLengthMax]
 * that comes strictly after (after_t, after_tri) in the order "t, then
 * triangle index", where t is the distance of the watertight test (the
 * order the closest hit uses; hitDistance itself is the reference's plane
 * distance, which can differ from t in the last bits).  *t_out (may be NULL)
 * receives that t, the key of the following call.  after_t = -INFINITY gives
 * the closest hit.  Replaying a handler this way offers every hit of the ray
 * once, nearest first, as IT_BSP colliders do (RRCollider.h:52-55; the
 * handler loop of RRCollider/IntersectBspFast.cpp:513 and the sorted replay
 * of RayHits::getHitOrdered, RRCollider/IntersectLinear.cpp:396-437).  Same
 * threading, fields and status as rrg_intersect_rrray_one; after_t NaN is
 * RRG_ERR_INVALID. */
RRG_API int rrg_intersect_rrray_one_after(rrg_collider* c, void* rrray_host, float after_t, uint32_t after_tri,
                                          float* t_out, uint8_t* hit_host);

/* Batches traced by rrg_intersect_rrray_one so far and the rays in them. */
RRG_API int rrg_collider_combined(const rrg_collider* c, uint64_t* batches, uint64_t* rays);

/* Same on a device copy of the RRRay array (asynchronous). */
RRG_API int rrg_intersect_rrray_device(rrg_collider* c, void* rrrays_dev, uint32_t n, uint8_t* hit_dev, void* stream);

/* Largest batch of rrg_intersect_rrray_noalloc (its static device scratch is
 * 256 + 129 * RRG_NOALLOC_MAX_RAYS bytes per device, about 2 MB). */
#define RRG_NOALLOC_MAX_RAYS 16384u

/* rrg_intersect_rrray without allocating: no counterpart in the reference.
 * Same arguments, outputs and synchronous behaviour as rrg_intersect_rrray,
 * but the device scratch (work counter, status word, staging of the records
 * and hit bytes) is one static array per device instead of buffers that the
 * collider grows with cudaFree + cudaMalloc.  For callers that must not
 * allocate device memory: a per-frame loop, where cudaFree's device-wide
 * synchronisation would stall every stream, and a process whose device memory
 * is already held (by a caching allocator such as PyTorch's, or by a bake
 * that sized its buffers to fill the GPU), where cudaMalloc would fail.
 *   - n > RRG_NOALLOC_MAX_RAYS returns RRG_ERR_TOO_LARGE and does nothing;
 *   - every call looks up the array's device address with the collider's
 *     device current (so the call keeps working after cudaDeviceReset); the
 *     first call on a device also loads the array's module there: make that
 *     first call before any stream capture begins;
 *   - the status of the trace is returned directly (RRG_ERR_STACK on a
 *     traversal overflow); rrg_collider_status() does not see it;
 *   - every call on a device shares the one array, whichever collider or
 *     stream it uses: calls that overlap on the GPU (from two host threads at
 *     once) race on it and return wrong results.  Serialise them. */
RRG_API int rrg_intersect_rrray_noalloc(rrg_collider* c, void* rrrays_host, uint32_t n, uint8_t* hit_host,
                                        void* stream);

/* Status word of the collider's last traces: RRG_OK or RRG_ERR_STACK.
 * Synchronises the stream first; resets the word. */
RRG_API int rrg_collider_status(rrg_collider* c, void* stream);

RRG_API const char* rrg_status_string(int status);
/* Text of the last CUDA error seen by this library (thread-local). */
RRG_API const char* rrg_last_cuda_error(void);
/* Library version, (major << 16) | minor. */
RRG_API uint32_t rrg_version(void);
/* Kernels this library has launched in this process so far, on every
 * device and thread (a kernel inside a CUDA graph counts once per graph
 * launch).  No reference counterpart: a profiling aid. */
RRG_API uint64_t rrg_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif
