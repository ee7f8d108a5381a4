/* rrgpu_gather.h -- C ABI of the GB300 lightmap final gather.
 *
 * Replaces, for the plain N-bounce estimator, the reference's
 * RRSolver::updateLightmaps / updateLightmap (RRSolver/lightmap.cpp:648-1163)
 * with its texel enumeration (enumerateTexelsPartial, lightmap.cpp:83-404) and
 * per-texel gather (processTexel, RRSolver/gather.cpp:600-836).  The scene is
 * the collider's mesh (rrgpu.h); materials are per-triangle diffuse albedo
 * (RRMaterial::diffuseReflectance, one-sided, RRMaterial.cpp:154-166);
 * lights are one directional and one point light with REALISTIC falloff
 * (RRLight.cpp:345-362, 450-455).  Lightmaps are `natlas` square atlases of
 * size x size texels, float RGBA per texel (RGB = irradiance in the
 * reference's physical scale, A = the texel's TexelFlags / 255 where it is
 * covered, 0 elsewhere, as the reference stores it, gather.cpp:801).
 *
 * Texel t of atlas a has global id a*size*size + y*size + x; its sample
 * streams are seeded by that id, so any subset of texels can be gathered and
 * every result is reproducible.
 */
#ifndef RRGPU_GATHER_H
#define RRGPU_GATHER_H
#include "rrgpu.h"
#include "rrgpu_cache.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct rrg_lightmapper rrg_lightmapper;

/* Scheduling of the plain gather.  Every texel's value is the same bit for
 * bit whichever runs. */
enum {
	RRG_GATHER_AUTO = 0,        /* wavefront for calls of >= 16,384 texels, else warp per texel */
	RRG_GATHER_WARP = 1,        /* one warp per texel, lanes follow whole hemisphere paths */
	RRG_GATHER_WAVEFRONT = 2,   /* paths of a batch of texels advance bounce by bounce, one thread per path */
	/* flag OR-ed into the mode: the hemisphere reads the radiosity solver of
	 * rrg_lightmapper_bake_solver at its first hit (exitance = albedo x
	 * (the triangle's direct irradiance + its corners' smoothed indirect
	 * irradiance interpolated at the hit)) and ends there, as the reference's
	 * updateLightmaps does after its first gather (useSolverDirect/
	 * IndirectSinceDepth = 0, gather.cpp:187-189; pathtracer.cpp:235-258,
	 * 326-350); warp per texel; not for the learned gather */
	RRG_GATHER_SOLVER = 4
};

/* UpdateParameters / PathTracingParameters subset (RRSolver.h:468-594,
 * 964-1001).  size = sizeof(rrg_gather_params). */
typedef struct rrg_gather_params {
	uint32_t size;
	uint32_t quality;          /* hemisphere rays per texel (UpdateParameters::quality), 1..256 */
	uint32_t max_depth;        /* diffuse bounces (PathTracingParameters::stopAtDepth); above 255 acts as 255 */
	uint32_t mode;             /* RRG_GATHER_*: how the plain gather is scheduled (results do not depend on it) */
	uint64_t seed;             /* sample streams */
	float ray_length_min;      /* 0 = the solver's minimalSafeDistance of the mesh */
	float locality;            /* UpdateParameters::locality, 0 = 100000 */
	float dir_direction[3];    /* directional light: unit direction the light travels */
	float dir_color[3];
	float point_position[3];   /* point light */
	float point_color[3];
	/* ambient occlusion (UpdateParameters::aoIntensity / aoSize, RRSolver.h:506-510):
	 * when both are > 0 the hemisphere irradiance is scaled by
	 * (rays whose first hit is farther than ao_size / rays)^ao_intensity
	 * (gather.cpp:277,306-309).  A caller built against the struct without
	 * these two fields (size 80) gets them as 0. */
	float ao_intensity;
	float ao_size;
} rrg_gather_params;

/* Enumerates sub-texels on the device.  albedo: 3 floats per triangle;
 * tri_atlas: atlas of each triangle (-1 = not lightmapped); uv: 3 corners x
 * (u, v) in [0,1] per triangle, in the triangle's vertex order.  The
 * collider must outlive the lightmapper. */
RRG_API int rrg_lightmapper_create(rrg_collider* c, const float* albedo, const int32_t* tri_atlas, const float* uv,
                                   uint32_t natlas, uint32_t size, rrg_lightmapper** out);
RRG_API void rrg_lightmapper_destroy(rrg_lightmapper* lm);
RRG_API uint64_t rrg_lightmapper_subtexels(const rrg_lightmapper* lm);
/* minimalSafeDistance used when ray_length_min = 0. */
RRG_API float rrg_lightmapper_ray_length_min(const rrg_lightmapper* lm);
/* Copies the sub-texel lists: offsets (natlas*size*size + 1 uint32) and
 * 32-byte records {uint32 triangle; float uv[3][2] in triangle space; float
 * area in map space} (may be NULL). */
RRG_API int rrg_lightmapper_copy_subtexels(const rrg_lightmapper* lm, uint32_t* offsets_host, void* subtexels_host);

/* Gathers texels [first_texel, first_texel + ntexels) into out (4 floats per
 * texel, 16-byte aligned device memory).  Asynchronous on `stream`. */
RRG_API int rrg_lightmap_gather(rrg_lightmapper* lm, const rrg_gather_params* p, uint64_t first_texel,
                                uint64_t ntexels, float* out_dev, void* stream);
/* Same, plus the bent normal of each texel when bent_dev != NULL (4 floats
 * per texel, the reference's LS_BENT_NORMALS encoding: (n + 1) / 2 of the
 * normalised sum of the lights' and the hemisphere's bent normals, w = the
 * texel's alpha; gather.cpp:274,488,811-830). */
RRG_API int rrg_lightmap_gather_ex(rrg_lightmapper* lm, const rrg_gather_params* p, uint64_t first_texel,
                                   uint64_t ntexels, float* out_dev, float* bent_dev, void* stream);
/* Same into host memory; synchronous. */
RRG_API int rrg_lightmap_gather_host(rrg_lightmapper* lm, const rrg_gather_params* p, uint64_t first_texel,
                                     uint64_t ntexels, float* out_host, void* stream);
/* Directional lightmaps (LS_DIRECTION1..3, "compatible with Unreal Engine
 * 3", gather.cpp:43-49): when any of dir1..3 is non-NULL the gather runs in
 * the reference's directional mode (gatherAllDirections, lightmap.cpp:820):
 * each hemisphere sample and light is weighted by its cosine to each of the
 * four directions of the texel's tangent basis (gather.cpp:255-272,
 * 468-486), and out (LS_LIGHTMAP) is computed that way too, as the
 * reference does when directional buffers are requested.  Each non-NULL
 * buffer: 4 floats per texel, 16-byte aligned device memory; bent_dev may
 * be NULL.  Asynchronous on `stream`. */
RRG_API int rrg_lightmap_gather_directional(rrg_lightmapper* lm, const rrg_gather_params* p, uint64_t first_texel,
                                            uint64_t ntexels, float* out_dev, float* dir1_dev, float* dir2_dev,
                                            float* dir3_dev, float* bent_dev, void* stream);
/* Number of texels that have sub-texels. */
RRG_API uint64_t rrg_lightmapper_covered(const rrg_lightmapper* lm);
/* TexelFlags of every texel (natlas*size*size bytes; RRSolver/gather.h:68-80,
 * set by the enumeration as lightmap.cpp:283-314 does).  A gathered texel's
 * alpha is its flags / 255 (gather.cpp:801), which the filters read. */
RRG_API int rrg_lightmapper_copy_flags(const rrg_lightmapper* lm, uint8_t* flags_host);

/* Post-filters that RRSolver::updateLightmap applies to each gathered
 * lightmap, in this order (RRSolver/lightmap.cpp:865-874). */
enum {
	RRG_FILTER_SMOOTH = 1,          /* RRBuffer::lightmapSmooth (RRBuffer.cpp:630-802) */
	RRG_FILTER_GROW_BILINEAR = 2,   /* lightmapGrowForBilinearInterpolation (RRBuffer.cpp:804-863) */
	RRG_FILTER_GROW = 4,            /* lightmapGrow (RRBuffer.cpp:865-962) */
	RRG_FILTER_FILL_BACKGROUND = 8, /* lightmapFillBackground (RRBuffer.cpp:964-983) */
	RRG_FILTER_ALL = 15
};

/* RRSolver::FilteringParameters (include/Lightsprint/RRSolver.h:596-621);
 * rrg_filter_defaults() fills its defaults. */
typedef struct rrg_filter_params {
	uint32_t size;               /* sizeof(rrg_filter_params) */
	uint32_t stages;             /* RRG_FILTER_* bits, run in the order above */
	float smoothing_amount;      /* smoothingAmount (default 1; 0 = off; capped at 10) */
	uint32_t spread_foreground;  /* spreadForegroundColor, in texels (default 1000) */
	float background[4];         /* backgroundColor (default 0) */
	uint32_t wrap;               /* wrap (default 0) */
	uint32_t seams;              /* 1: lightmapSmooth also averages across unwrap seams, as it
	                                does when given the object (default 1) */
} rrg_filter_params;
RRG_API void rrg_filter_defaults(rrg_filter_params* p);

/* Filters atlases [first_atlas, first_atlas + natlas) of `lightmaps_dev`
 * in place: the lightmapper's layout (atlas a, texel (x, y) at float4 index
 * (a * size + y) * size + x), RGBA with alpha as the gather writes it.
 * Asynchronous on `stream` (the grow stage synchronises it every 8 steps to
 * stop early).  Scratch (two float4 and one byte per texel of the atlases
 * filtered) is owned by the lightmapper and grown on demand; the unwrap
 * seams are found on the first call that asks for them: edges shared by two
 * triangles of an atlas (by vertex index) whose unwrap differs (UnwrapSeams,
 * RRBuffer.cpp:534-628). */
RRG_API int rrg_lightmap_filter(rrg_lightmapper* lm, const rrg_filter_params* p, uint32_t first_atlas,
                                uint32_t natlas, float* lightmaps_dev, void* stream);
/* The whole update of the lightmapper's atlases, host buffer out: every
 * texel of every atlas gathered with p (the solver-reading gather when
 * p->mode has RRG_GATHER_SOLVER, after rrg_lightmapper_bake_solver), then
 * the post-filters of f (NULL or stages 0 = none), then copied to out_host
 * (float RGBA, natlas x size x size texels, the lightmapper's layout).
 * Synchronous; the device buffer is the lightmapper's staging buffer.  What
 * RRSolver::updateLightmap does per lightmap (RRSolver/lightmap.cpp:
 * 648-930), for all atlases at once. */
RRG_API int rrg_lightmap_bake_host(rrg_lightmapper* lm, const rrg_gather_params* p, const rrg_filter_params* f,
                                   float* out_host);

/* Counting of the rays the wavefront gather traces (a measurement aid, no
 * reference counterpart): returns in *closest and *shadow (may be NULL) the
 * closest-hit and shadow rays traced since the previous call (light rounds'
 * shadow rays included), resets them, and counts from now on when enable is
 * nonzero.  Synchronises the device. */
RRG_API int rrg_lightmapper_count_rays(rrg_lightmapper* lm, int enable, uint64_t* closest, uint64_t* shadow);

/* Order in which the wavefront gather traces each bounce's closest-hit rays
 * (and the learned gather its first segments): RRG_RAY_ORDER_BINNED sorts
 * the live paths by their rays' origin and direction cell first (one
 * counting-sort pass, rrg_binning.cu); RRG_RAY_ORDER_DEFAULT and
 * RRG_RAY_ORDER_AS_GIVEN trace them in path order, where a warp's rays are
 * one texel's samples (measured 4-6 % faster than binned on GB300).
 * Results do not depend on it. */
RRG_API int rrg_lightmapper_set_ray_order(rrg_lightmapper* lm, uint32_t order);

/* Number of unwrap seams found (0 before the first filter call with seams). */
RRG_API uint64_t rrg_lightmapper_seams(const rrg_lightmapper* lm);
/* Runs of samples over all seams (a run: consecutive samples of a seam that
 * fall in the same pair of texels); 0 before the first filter call with seams. */
RRG_API uint64_t rrg_lightmapper_seam_runs(const rrg_lightmapper* lm);

/* The radiosity solver of the reference's default bake
 * (updateSolverIndirectIllumination, RRSolver/gather.cpp:1038-1117, over
 * RRStaticSolver), for gathers with RRG_GATHER_SOLVER:
 *   1. first gather per triangle (gatherPerTrianglePhysical, gather.cpp:
 *      843-952): max(1, quality / 2) / 10 + 1 light rounds from random
 *      points of the triangle -> its direct irradiance;
 *   2. rays_per_triangle (0 = quality) form-factor rays per triangle, from
 *      random points, cosine-distributed over its front side, nearest hit on
 *      either side (shotFromToHalfspace / rayTracePhoton, RRStaticSolver/
 *      rrcore.cpp:861-1050);
 *   3. `iterations` Jacobi steps of the flux balance in gathering form,
 *      E = D + (1/k) sum over the factor hits of albedo x E (the system the
 *      reference's progressive shooting solves, rrcore.cpp:1052-1297);
 *   4. indirect irradiance E - D smoothed over corners stitched at identical
 *      positions with normals within 0.01 rad, weighted by corner angle x
 *      area (Object::buildTopIVertices, interpol.cpp:78-170).
 * Uses p's lights, seed, quality and ray_length_min.  Device scratch: 4 bytes
 * per triangle per ray plus 60 bytes per triangle.  Asynchronous on stream
 * (the first call builds the stitching on the host). */
RRG_API int rrg_lightmapper_bake_solver(rrg_lightmapper* lm, const rrg_gather_params* p, uint32_t rays_per_triangle,
                                        uint32_t iterations, void* stream);
/* Copies the solver: direct irradiance (3 floats per triangle), indirect
 * irradiance before smoothing (3 floats per triangle) and smoothed corner
 * indirect irradiance (9 floats per triangle); any may be NULL.
 * Synchronous. */
RRG_API int rrg_lightmapper_copy_solver(const rrg_lightmapper* lm, float* direct_host, float* indirect_host,
                                        float* corner_host);
/* The last bake's form-factor rays: ray j of triangle t at t * rays + j, the
 * triangle whose front it hit, else 0xFFFFFFFF.  Returns their number (0
 * before a bake); copies them when cap is large enough.  Synchronous. */
RRG_API uint64_t rrg_lightmapper_copy_factor_hits(const rrg_lightmapper* lm, uint32_t* hits_host, uint64_t cap);

/* Training records for a radiance cache (rrgpu_cache.h) from the gather's
 * own paths: from every `stride`-th covered texel, paths_per_texel plain
 * paths; each of a path's first four vertices gives one record (position,
 * plane normal, albedo, outgoing radiance toward the previous vertex).  A
 * record's radiance covers the same bounces the gather traces after a
 * first hit (that vertex and max_depth more): paths are traced three
 * bounces deeper than the gather so that every record's window is whole.
 * Writes at most cap records to recs_dev (48 bytes each); *nrec_out =
 * records written. */
RRG_API int rrg_lightmap_train_samples(rrg_lightmapper* lm, const rrg_gather_params* p, uint32_t stride,
                                       uint32_t paths_per_texel, void* recs_dev, uint64_t cap, uint64_t* nrec_out,
                                       void* stream);
/* Learned gather of texels [first, first + ntexels): the light rounds as in
 * the plain gather, and for each hemisphere sample one traced segment plus a
 * cache query at its hit (in place of the remaining bounces).  Texels whose
 * samples land in cells the cache's error grid marks unreliable more often
 * than fallback_frac * quality are recomputed by the plain gather;
 * *nfallback (may be NULL) receives their number.  Synchronises the stream
 * between chunks of 2^20 texels. */
RRG_API int rrg_lightmap_gather_learned(rrg_lightmapper* lm, rrg_cache* cache, const rrg_gather_params* p,
                                        uint64_t first_texel, uint64_t ntexels, float* out_dev, float fallback_frac,
                                        uint64_t* nfallback, void* stream);

/* RRG_OK, or RRG_ERR_STACK if a traversal overflowed since the last call. */
RRG_API int rrg_lightmapper_status(rrg_lightmapper* lm, void* stream);

#ifdef __cplusplus
}
#endif
#endif
