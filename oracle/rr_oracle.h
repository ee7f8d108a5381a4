/* ORACLE: a CPU restatement, in plain C, of the reference collider's
 * arithmetic.  Test infrastructure only: the parity tests and the CPU-baseline
 * leg of the benchmark call it as the checker; the product never links it.
 *
 * Build with -ffp-contract=off so that every float operation rounds once, as
 * the reference's own x86-64 build does; the results are then identical on
 * x86-64 and aarch64.
 *
 * Restated functions (file:line in the reference project):
 *   orc_tri_setup      TriangleSRLNP::setGeometry   RRCollider/IntersectBspFast.cpp:130-187
 *   orc_tri_fastest    intersect_triangleSRLNP +    RRCollider/IntersectBspFast.cpp:189-252
 *                      the kd-leaf plane distance   RRCollider/IntersectBspFast.cpp:344-353
 *   orc_tri_linear     intersect_triangle (Moller-Trumbore)  RRCollider/IntersectLinear.cpp:62-110
 *   orc_plane_linear   update_hitPlane              RRCollider/IntersectLinear.cpp:47-60
 *   orc_box_*          Box::init / Box::intersect   RRCollider/geometry.cpp:20-86
 *   orc_delta_bsp      DELTA_BSP                    RRCollider/IntersectLinear.cpp:129-140
 *
 * orc_collide_fastest answers IT_BSP_FASTEST queries without the BSP tree:
 * the accepted hit is the triangle with the smallest plane distance among
 * those the FASTEST triangle test accepts (ties: smaller triangle index), with
 * the FASTEST output fields.  The reference additionally lets a hit up to
 * DELTA_BSP beyond a kd split win (IntersectBspFast.cpp:397-423); those ties
 * are the only expected differences.  Acceleration is our own binned-SAH BVH,
 * with boxes inflated so that it never culls an acceptable triangle.
 */
#ifndef RR_ORACLE_H
#define RR_ORACLE_H
#include <stdint.h>
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_tri {
	float n4[4];        /* unit plane normal, d */
	float s3[3];        /* vertex0 */
	float ireal;        /* 1 / dominant 2-D cross term */
	float r3[3];        /* vertex1 - vertex0 */
	float ir3[3];       /* 1 / r3 */
	float l3[3];        /* vertex2 - vertex0 */
	unsigned char ibyte;/* projection case 0..8, 10 = degenerate */
} orc_tri;

/* Per-ray outputs, SoA; tri = 0xFFFFFFFF on a miss. */
typedef struct orc_hits {
	uint8_t* hit;
	uint32_t* tri;
	float* dist;
	float* uv;       /* 2 per ray */
	float* plane;    /* 4 per ray */
	float* point3d;  /* 3 per ray */
	uint8_t* side;
} orc_hits;

void orc_tri_setup(const float* a, const float* b, const float* c, orc_tri* t);
/* FASTEST triangle test at plane distance `dist` (hit point o + d*dist). */
int orc_tri_fastest(const orc_tri* t, const float* o, const float* d, float dist,
                    float* u, float* v, int* front);
/* FASTEST plane distance -(n.o + w) / (n.d). */
float orc_plane_distance(const orc_tri* t, const float* o, const float* d);
/* Moller-Trumbore test of IntersectLinear; returns 1 on hit in [tmin,tmax]. */
int orc_tri_linear(const float* v0, const float* v1, const float* v2, const float* o, const float* d,
                   float tmin, float tmax, float* dist, float* u, float* v, int* front);
void orc_plane_linear(const float* v0, const float* v1, const float* v2, float* plane);
float orc_delta_bsp(const float* xyz, uint32_t nv);
void orc_box_init(const float* mn, const float* mx, float* bmin, float* bmax);
int orc_box_intersect(const float* bmin, const float* bmax, const float* o, const float* d,
                      float lenmin, float lenmax, float* hmin, float* hmax);

/* Exhaustive IT_LINEAR collider: nearest Moller-Trumbore hit.  rays = n x 8
 * floats (ox oy oz tmin dx dy dz tmax).  Small cases only. */
void orc_collide_linear(const float* xyz, uint32_t nv, const uint32_t* idx, uint32_t nt,
                        const float* rays, uint32_t n, int threads, orc_hits* out);

typedef struct orc_bvh orc_bvh;
orc_bvh* orc_bvh_build(const float* xyz, uint32_t nv, const uint32_t* idx, uint32_t nt);
void orc_bvh_free(orc_bvh* b);
/* IT_BSP_FASTEST semantics over the BVH (see header comment).  any_hit=1
 * stops at the first accepted triangle (shadow rays): only hit is defined. */
void orc_collide_fastest(const orc_bvh* b, const float* rays, uint32_t n, int threads, int any_hit,
                         orc_hits* out);
/* Exact nearest hit in double precision (Moller-Trumbore in f64 over the same
 * candidate set): the FP64 reference used to state hitDistance errors. */
void orc_collide_exact64(const orc_bvh* b, const float* rays, uint32_t n, int threads,
                         uint32_t* tri, double* dist);
int orc_max_threads(void);
/* Ray cast with the final-gathering handler semantics (see rr_oracle.c). */
uint32_t orc_cast(const orc_bvh* b, const float* o, const float* d, float tmin, float tmax, int shadow,
                  uint32_t skip, float* dist, float* plane);
/* Photon ray of the radiosity solver (RRCollisionHandlerLod0): the nearest
 * hit on either side, the shooter skipped; *front = the side hit. */
uint32_t orc_cast_photon(const orc_bvh* b, const float* o, const float* d, float tmin, float tmax, uint32_t skip,
                         int* front);
/* Hemisphere cast (as orc_cast with shadow = 0) that also returns the hit's
 * barycentric u, v (hitPoint2d). */
uint32_t orc_cast_uv(const orc_bvh* b, const float* o, const float* d, float tmin, float tmax, uint32_t skip,
                     float* dist, float* uv);

#ifdef __cplusplus
}
#endif
#endif
