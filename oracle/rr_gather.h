/* ORACLE: CPU restatement of the reference's lightmap final gather, for the
 * plain N-bounce estimator.  Test infrastructure only: the parity tests and
 * the CPU-baseline leg of the benchmark call it as the checker.
 *
 * Restated (file:line in the reference project):
 *   orc_enumerate      enumerateTexelsPartial: texel x triangle clipping in
 *                      triangle space, fan triangulation into sub-texels
 *                      (RRSolver/lightmap.cpp:145-330), getArea (:32-40)
 *   orc_gather         processTexel (RRSolver/gather.cpp:600-836) with
 *                      GatheredIrradianceHemisphere (:164-343) and
 *                      GatheredIrradianceLights (:356-586), HomogenousFiller2
 *                      (:57-111), getRandomEnterDirNormalized (:121-135);
 *                      PathtracerWorker::getIncidentRadiance
 *                      (RRStaticSolver/pathtracer.cpp:139-394) with
 *                      useSolver*SinceDepth = UINT_MAX (no radiosity
 *                      shortcuts), next-event shadow rays to every light and
 *                      Russian roulette on the diffuse reflectance;
 *                      RRMaterial::getResponse diffuse (RRMaterial.cpp:666-675),
 *                      RRLight::getIrradiance (RRLight.cpp:345-362),
 *                      buildBasisFromNormal (RRMesh.cpp:70-75).
 *
 * Deliberate differences from the reference, shared with the GPU kernel so
 * both run the same sample streams:
 *   - libc rand() is replaced by a counter-based hash of (seed, stream,
 *     index): the sub-texel point (rand() pair), the filler seed
 *     (rand()&0xffff), the roulette draw (RR_RAND01);
 *   - the bounce direction is cosine-weighted by Malley's method (a disk
 *     point by rejection lifted to the hemisphere) instead of the polar
 *     sin/cos form of sampleHemisphereDiffuse; the distribution is the same,
 *     and no transcendental function is needed, so CPU and GPU agree bitwise;
 *   - one shooting series per texel (every ray here is reliable).  The
 *     reference's reliability bookkeeping changes no value under its
 *     defaults: a light ray that meets a back face (hitsInside) or a hit
 *     nearer than rugDistance adds nothing, as a shadowed one does; the
 *     inside-object rejection needs hitsInside > rays * insideObjectsThreshold
 *     (default 1), which cannot happen; hemisphere rays always count as
 *     reliable (gather.cpp:283-319, 490-558, UpdateParameters defaults
 *     RRSolver.h:546-556);
 *   - the path radiance is accumulated iteratively (L += T * contribution)
 *     rather than by recursion.
 * Ambient occlusion (aoIntensity, aoSize: the hemisphere irradiance scaled
 * by (rays whose first hit is farther than aoSize / rays)^aoIntensity,
 * gather.cpp:277,306-309; the first hit's distance, pathtracer.cpp:145-177)
 * and bent normals (gather.cpp:274,488,811-830) follow the reference.
 * With fp64 = 1 the same paths are accumulated in double precision: the
 * FP64-accumulated reference that states the float accumulation error.
 *
 * Pinned against the reference's own processTexel run with no radiosity
 * solver (oracle/ref_gather.cpp, tests/golden/gather_ref.npz): bit-exact on
 * the texels whose value no random number changes, statistically (means,
 * 8x8 blocks, texel spread) on the rest.  The per-bounce counter is
 * sid * 256 + depth (depths above 255 act as 255).
 */
#ifndef RR_GATHER_H
#define RR_GATHER_H
#include <stdint.h>
#include "rr_oracle.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_subtexel {
	uint32_t tri;       /* world triangle index */
	float uv[3][2];     /* corners in triangle space (barycentric u, v) */
	float area;         /* area in map space */
} orc_subtexel;         /* 32 bytes, the GPU's sub-texel record */

typedef struct orc_gather_scene {
	const float* xyz;       /* world vertices */
	const uint32_t* idx;    /* triangles */
	uint32_t nt;
	const float* albedo;    /* nt * 3 */
	float dir_direction[3]; /* directional light: direction the light travels */
	float dir_color[3];
	float point_position[3];
	float point_color[3];
	float ray_length_min;   /* minimalSafeDistance */
	float locality;         /* UpdateParameters::locality */
	uint32_t quality;       /* hemisphere rays per texel */
	uint32_t max_depth;     /* PathTracingParameters::stopAtDepth */
	uint64_t seed;
	float ao_intensity;     /* UpdateParameters::aoIntensity (used when both are > 0) */
	float ao_size;          /* UpdateParameters::aoSize */
	const uint8_t* flags;   /* TexelFlags by texel id (alpha = flags/255, gather.cpp:801); NULL: alpha 1 */
	/* radiosity solver read at the first hit (NULL: the plain N-bounce
	 * estimator): per triangle its direct irradiance (3 floats) and the
	 * smoothed indirect irradiance at its three corners (9 floats) */
	const float* solver_direct;
	const float* solver_corner;
} orc_gather_scene;

/* Sub-texels of one atlas.  uv: n triangles x 3 corners x 2 in map space
 * [0,1]; tri: their world indices, in the order the reference visits them.
 * counts[size*size] receives sub-texels per texel; when out != NULL the
 * sub-texels are written texel by texel (offsets = exclusive scan of
 * counts, computed by the caller).  Returns the total. */
uint64_t orc_enumerate(const float* uv, const uint32_t* tri, uint32_t n, uint32_t size, uint32_t* counts,
                       const uint64_t* offsets, orc_subtexel* out);
/* Texel flags of one atlas (TexelFlags, RRSolver/gather.h:68-80, set in
 * lightmap.cpp:283-314): flags[size*size], OR over every clipped polygon of
 * every triangle in the texel.  uv as for orc_enumerate. */
void orc_texel_flags(const float* uv, uint32_t n, uint32_t size, uint8_t* flags);

/* Gathers `ntexels` texels: texel i has global id texel_id[i] (seeds its
 * sample streams) and sub-texels st[off[i] .. off[i+1]).  out: 4 floats per
 * texel (irradiance RGB, 1 if covered else 0). */
void orc_gather(const orc_bvh* bvh, const orc_gather_scene* sc, const uint64_t* texel_id, uint32_t ntexels,
                const uint64_t* off, const orc_subtexel* st, int threads, int fp64, float* out);

/* Same, plus the bent normal of each texel when bent != NULL (4 floats:
 * (n + 1) / 2 of the normalised sum of the lights' and the hemisphere's
 * bent normals, 1 if covered; gather.cpp:274,488,811-830). */
void orc_gather_ex(const orc_bvh* bvh, const orc_gather_scene* sc, const uint64_t* texel_id, uint32_t ntexels,
                   const uint64_t* off, const orc_subtexel* st, int threads, int fp64, float* out, float* bent);

/* Same in directional mode when dirs != NULL (gatherAllDirections,
 * gather.cpp:255-272,468-486; lightmap.cpp:820): out is LS_LIGHTMAP and dirs
 * 12 floats per texel, LS_DIRECTION1..3 RGBA, every output weighted by the
 * UE3 basis directions (gather.cpp:43-49) in the texel's skewed tangent
 * basis.  fp32 accumulation only. */
void orc_gather_dir(const orc_bvh* bvh, const orc_gather_scene* sc, const uint64_t* texel_id, uint32_t ntexels,
                    const uint64_t* off, const orc_subtexel* st, int threads, int fp64, float* out, float* bent,
                    float* dirs);

/* Counter-based generator shared with the GPU (and with the Python
 * generators): MurmurHash3 fmix64 of (seed, stream, index). */
uint64_t orc_hash(uint64_t seed, uint64_t stream, uint64_t index);

/* Lightmap post-filters (rr_filter.c).  rgba: width*height RGBA floats,
 * alpha = TexelFlags/255 where covered; seams: 8 floats per unwrap seam. */
uint32_t orc_unwrap_seams(const uint32_t* idx, const float* uv, uint32_t n, float* seams, uint32_t cap);
int orc_lightmap_smooth(float* rgba, uint32_t width, uint32_t height, float sigma, int wrap, const float* seams,
                        uint32_t nseams);
int orc_lightmap_grow_bilinear(float* rgba, uint32_t width, uint32_t height, int wrap);
int orc_lightmap_grow(float* rgba, uint32_t width, uint32_t height, uint32_t steps, int wrap);
void orc_lightmap_fill_background(float* rgba, uint32_t width, uint32_t height, const float* background);

/* ---- the default bake's solver (updateSolverIndirectIllumination,
 * RRSolver/gather.cpp:959-1117, and RRStaticSolver) ---- */

/* First gather per triangle (gatherPerTrianglePhysical, gather.cpp:843-952):
 * processTexel with the whole triangle as its one sub-texel at quality
 * max(1, quality / 2): (that / 10 + 1) light rounds from random points of
 * the triangle, no hemisphere rays.  direct[3 * nt]. */
void orc_bake_direct(const orc_bvh* bvh, const orc_gather_scene* sc, int threads, float* direct);
/* Form-factor rays (shotFromToHalfspace / rayTracePhoton, rrcore.cpp:861-1050):
 * k rays per triangle from random points, cosine-distributed over its front
 * half-space, nearest hit on either side (shooter skipped, tmin 1e-4);
 * hits[nt * k] = the triangle whose front side was hit (and whose diffuse
 * reflectance sums above 0.01), else 0xFFFFFFFF. */
void orc_bake_factors(const orc_bvh* bvh, const orc_gather_scene* sc, uint32_t k, int threads, uint32_t* hits);
/* Radiosity by Jacobi iteration of the gathering form of the solver's flux
 * balance: E_j <- D_j + (1/k) sum over j's hits h of albedo_h * E_h, from
 * E = D, `iterations` times.  indirect[3 * nt] = E - D. */
void orc_bake_propagate(const orc_gather_scene* sc, const float* direct, const uint32_t* hits, uint32_t k,
                        uint32_t iterations, float* indirect);
/* Corner smoothing (Object::buildTopIVertices, interpol.cpp:120-170, with
 * the stitching of RRLessVerticesFilter, RRMeshLessVertices.h:38-237, at
 * the default SmoothingParameters: identical positions, normals within
 * 0.01 rad): group[3 * nt] = each corner's stitched vertex, weight[3 * nt] =
 * its corner angle x triangle area (0 for degenerate triangles).  Returns
 * the number of groups. */
uint32_t orc_bake_stitch(const float* xyz, const uint32_t* idx, uint32_t nt, uint32_t* group, float* weight);
/* corner[9 * nt]: each corner's smoothed indirect irradiance (IVertex::
 * irradiance, interpol.cpp:78-112): the weighted mean over its group. */
void orc_bake_smooth(uint32_t nt, const uint32_t* group, const float* weight, uint32_t ngroups,
                     const float* indirect, float* corner);

#ifdef __cplusplus
}
#endif
#endif
