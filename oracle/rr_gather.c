/* ORACLE: CPU restatement of the lightmap final gather (see rr_gather.h).
 * Test infrastructure only.  Compile with -ffp-contract=off. */
#include "rr_gather.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ RNG */
static uint64_t fmix64(uint64_t k) {
	k ^= k >> 33;
	k *= 0xFF51AFD7ED558CCDULL;
	k ^= k >> 33;
	k *= 0xC4CEB9FE1A85EC53ULL;
	k ^= k >> 33;
	return k;
}

uint64_t orc_hash(uint64_t seed, uint64_t stream, uint64_t index) {
	uint64_t key = seed * 0x9E3779B97F4A7C15ULL + stream * 0xD1B54A32D192ED03ULL;
	return fmix64(fmix64(index ^ key) + 0x632BE59BD9B4E019ULL);
}

static uint32_t rng24(uint64_t seed, uint64_t stream, uint64_t index) {
	return (uint32_t)(orc_hash(seed, stream, index) >> 40);
}
static float rng01(uint64_t seed, uint64_t stream, uint64_t index) {
	return (float)rng24(seed, stream, index) * (1.0f / 16777216.0f);
}

enum { S_FILLER = 60, S_PU = 61, S_PV = 62, S_ROULETTE = 63, S_DISKX = 64, S_DISKY = 65 };
#define M24 16777215u
#define DISK_TRIES 32
/* bounce b of sample sid draws at counter sid * 256 + b; deeper limits act as 255 */
#define MAX_DEPTH 255u
#define PREVENT_INF 0.000000000137289f   /* RRLight.cpp:21 */
#define STOP_AT_VISIBILITY 0.001f        /* PathTracingParameters default, RRSolver.h:998 */

/* ------------------------------------------------------------ vectors */
typedef struct { float x, y, z; } v3;
static v3 mk(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static v3 mul(v3 a, float f) { return mk(a.x * f, a.y * f, a.z * f); }
static v3 mulv(v3 a, v3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
static v3 divf(v3 a, float f) { return mk(a.x / f, a.y / f, a.z / f); }
static v3 neg(v3 a) { return mk(-a.x, -a.y, -a.z); }
static float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static float len(v3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
static float len2(v3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static v3 normalized(v3 a) { return divf(a, len(a)); }
static float avg(v3 a) { return (a.x + a.y + a.z) * 0.33333333333333f; }
/* RRMathPrivate.h:48-58 */
static v3 ortho1(v3 a) { return fabsf(a.x) > fabsf(a.z) ? mk(-a.y, a.x, 0) : mk(0, -a.z, a.y); }
static v3 cross(v3 a, v3 b) { return mk(a.y * b.z - a.z * b.y, -a.x * b.z + a.z * b.x, a.x * b.y - a.y * b.x); }
static v3 ld3(const float* p) { return mk(p[0], p[1], p[2]); }

/* ---------------------------------------------------------- enumerate */
typedef struct { float x, y; } v2;
static v2 mk2(float x, float y) { v2 r = {x, y}; return r; }

/* RRSolver/lightmap.cpp:32-40 */
static float get_area(v2 v0, v2 v1, v2 v2_) {
	float a = sqrtf((v1.x - v0.x) * (v1.x - v0.x) + (v1.y - v0.y) * (v1.y - v0.y));
	float b = sqrtf((v2_.x - v1.x) * (v2_.x - v1.x) + (v2_.y - v1.y) * (v2_.y - v1.y));
	float c = sqrtf((v0.x - v2_.x) * (v0.x - v2_.x) + (v0.y - v2_.y) * (v0.y - v2_.y));
	float s = (a + b + c) * 0.5f;
	return sqrtf(s * (s - a) * (s - b) * (s - c));
}

static float clampf_(float a, float lo, float hi) { return a < lo ? lo : (a > hi ? hi : a); }

/* One triangle's rasterisation (lightmap.cpp:145-330): calls emit() for each
 * sub-texel in texel order, fan order. */
typedef void (*emit_fn)(void* ctx, uint32_t texel, uint32_t tri, const v2* uv, float area);

/* Texel flags of one clipped polygon (lightmap.cpp:283-314): its vertices in
 * texel space (texel centre at 0, the texel spans -0.5..0.5) mark the texel
 * edges they reach and the quadrants they fall in. */
enum { Q_X0Y0 = 1, Q_X1Y0 = 2, Q_X0Y1 = 4, Q_X1Y1 = 8, E_X0 = 16, E_X1 = 32, E_Y0 = 64, E_Y1 = 128 };

static unsigned polygon_flags(const float m[3][3], const v2* poly, unsigned n, unsigned x, unsigned y, float W,
                              float H) {
	const float err = 0.03f;   /* ERROR_IN_TEXELS */
	unsigned f = 0;
	v2 old = mk2(0, 0);
	for (unsigned k = 0; k <= n; k++) {
		v2 p = poly[(k + n - 1) % n];   /* k = 0: the last vertex, the "old" one of vertex 0 */
		v2 map = mk2(p.x * m[0][0] + p.y * m[0][1] + m[0][2], p.x * m[1][0] + p.y * m[1][1] + m[1][2]);
		v2 t = mk2(map.x * W - (float)x - 0.5f, map.y * H - (float)y - 0.5f);
		if (k) {
			if (t.x < -0.5f + err) f |= E_X0;
			if (t.x > 0.5f - err) f |= E_X1;
			if (t.y < -0.5f + err) f |= E_Y0;
			if (t.y > 0.5f - err) f |= E_Y1;
			if (t.x < 0 && t.y < 0) f |= Q_X0Y0;
			if (t.x > 0 && t.y < 0) f |= Q_X1Y0;
			if (t.x < 0 && t.y > 0) f |= Q_X0Y1;
			if (t.x > 0 && t.y > 0) f |= Q_X1Y1;
			/* an edge crossing both axes passes a quadrant without a vertex */
			if ((old.x < 0) != (t.x < 0) && (old.y < 0) != (t.y < 0)) {
				float a = (t.y - old.y) / (t.x - old.x);
				float b = t.y - a * t.x;
				f |= (b < 0) ? (Q_X0Y0 | Q_X1Y0) : (Q_X0Y1 | Q_X1Y1);
				f |= (-b / a < 0) ? (Q_X0Y0 | Q_X0Y1) : (Q_X1Y0 | Q_X1Y1);
			}
		}
		old = t;
	}
	return f;
}

static void raster_triangle(const float* uvm, uint32_t tri, uint32_t size, emit_fn emit, void* ctx,
                            uint8_t* flags) {
	const float W = (float)size, H = (float)size;
	v2 u0 = mk2(uvm[0], uvm[1]), u1 = mk2(uvm[2], uvm[3]), u2 = mk2(uvm[4], uvm[5]);
	float xmin = W * fminf(u0.x, fminf(u1.x, u2.x));
	float xmax = W * fmaxf(u0.x, fmaxf(u1.x, u2.x));
	float ymin = H * fminf(u0.y, fminf(u1.y, u2.y));
	float ymax = H * fmaxf(u0.y, fmaxf(u1.y, u2.y));
	/* the reference takes min/max with its own RR_MIN/RR_MAX; equal results
	 * for finite map coordinates */
	unsigned xminu = (unsigned)(xmin > 0.f ? xmin : 0.f);
	unsigned xmaxu = (unsigned)clampf_(xmax + 1, 0, W);
	unsigned yminu = (unsigned)(ymin > 0.f ? ymin : 0.f);
	unsigned ymaxu = (unsigned)clampf_(ymax + 1, 0, H);
	if (yminu >= ymaxu || xminu >= xmaxu) return;
	float m[3][3] = {{u1.x - u0.x, u2.x - u0.x, u0.x}, {u1.y - u0.y, u2.y - u0.y, u0.y}, {0, 0, 1}};
	float det = m[0][0] * m[1][1] * m[2][2] + m[0][1] * m[1][2] * m[2][0] + m[0][2] * m[1][0] * m[2][1] -
	            m[0][0] * m[1][2] * m[2][1] - m[0][1] * m[1][0] * m[2][2] - m[0][2] * m[1][1] * m[2][0];
	if (!det) return;
	float invdet = 1 / det;
	float inv[2][3] = {
		{(m[1][1] * m[2][2] - m[1][2] * m[2][1]) * invdet / W, (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * invdet / H,
		 (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * invdet},
		{(m[1][2] * m[2][0] - m[1][0] * m[2][2]) * invdet / W, (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * invdet / H,
		 (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * invdet}};
	float tri_area_map = get_area(u0, u1, u2);
	for (unsigned y = yminu; y < ymaxu; y++)
		for (unsigned x = xminu; x < xmaxu; x++) {
			unsigned polySize = 4;
			v2 poly[7];
#define M2T(X, Y) mk2((float)(X) * inv[0][0] + (float)(Y) * inv[0][1] + inv[0][2], \
                      (float)(X) * inv[1][0] + (float)(Y) * inv[1][1] + inv[1][2])
			poly[0] = M2T(x, y);
			poly[1] = M2T(x + 1, y);
			poly[2] = M2T(x + 1, y + 1);
			poly[3] = M2T(x, y + 1);
#undef M2T
			for (unsigned side = 0; side < 3; side++) {
				float L0 = side == 0 ? 0.f : (side == 1 ? -1.f : 1.f);
				float L1 = side == 0 ? 1.f : (side == 1 ? -1.f : 0.f);
				float L2 = side == 0 ? 0.f : (side == 1 ? 1.f : 0.f);
				int inside[7];  /* 0 inside, 1 edge, 2 outside */
				unsigned nin = 0, nout = 0;
				for (unsigned i = 0; i < polySize; i++) {
					float dd = L0 * poly[i].x + L1 * poly[i].y + L2;
					if (dd < 0) { inside[i] = 2; nout++; }
					else if (dd > 0) { inside[i] = 0; nin++; }
					else inside[i] = 1;
				}
				if (!nout) continue;
				if (!nin) { polySize = 0; break; }
				unsigned fp = 1;
				while (inside[(fp - 1) % polySize] == 0 || inside[fp % polySize] != 0) fp++;
				v2 orig[7];
				memcpy(orig, poly, sizeof(poly));
				unsigned src = fp, dst = 0;
				while (inside[src % polySize] == 0) poly[dst++] = orig[src++ % polySize];
#define ISECT(A, B)                                                                           \
	(mk2((A).x - ((B).x - (A).x) * (L0 * (A).x + L1 * (A).y + L2) /                            \
	                 (L0 * ((B).x - (A).x) + L1 * ((B).y - (A).y)),                            \
	     (A).y - ((B).y - (A).y) * (L0 * (A).x + L1 * (A).y + L2) /                            \
	                 (L0 * ((B).x - (A).x) + L1 * ((B).y - (A).y))))
				poly[dst++] = ISECT(orig[(src - 1) % polySize], orig[src % polySize]);
				poly[dst++] = ISECT(orig[(fp - 1) % polySize], orig[fp % polySize]);
#undef ISECT
				polySize = dst;
			}
			if (polySize && flags) flags[y * size + x] |= (uint8_t)polygon_flags(m, poly, polySize, x, y, W, H);
			if (polySize && emit) {
				v2 st[3];
				st[0] = poly[0];
				for (unsigned i = 0; i + 2 < polySize; i++) {
					st[1] = poly[i + 1];
					st[2] = poly[i + 2];
					float a = get_area(st[0], st[1], st[2]) * tri_area_map;
					if (isfinite(a)) emit(ctx, y * size + x, tri, st, a);
				}
			}
		}
}

typedef struct {
	uint32_t* counts;
	const uint64_t* offsets;
	uint32_t* cursor;
	orc_subtexel* out;
	uint64_t total;
} enum_ctx;

static void emit_count(void* c, uint32_t texel, uint32_t tri, const v2* uv, float area) {
	enum_ctx* e = (enum_ctx*)c;
	(void)tri; (void)uv; (void)area;
	e->counts[texel]++;
	e->total++;
}

static void emit_write(void* c, uint32_t texel, uint32_t tri, const v2* uv, float area) {
	enum_ctx* e = (enum_ctx*)c;
	orc_subtexel* s = &e->out[e->offsets[texel] + e->cursor[texel]++];
	s->tri = tri;
	for (int k = 0; k < 3; k++) { s->uv[k][0] = uv[k].x; s->uv[k][1] = uv[k].y; }
	s->area = area;
	e->total++;
}

uint64_t orc_enumerate(const float* uv, const uint32_t* tri, uint32_t n, uint32_t size, uint32_t* counts,
                       const uint64_t* offsets, orc_subtexel* out) {
	enum_ctx e = {counts, offsets, NULL, out, 0};
	if (!out) {
		memset(counts, 0, sizeof(uint32_t) * (size_t)size * size);
		for (uint32_t i = 0; i < n; i++) raster_triangle(uv + 6 * (size_t)i, tri[i], size, emit_count, &e, NULL);
		return e.total;
	}
	e.cursor = (uint32_t*)calloc((size_t)size * size, sizeof(uint32_t));
	for (uint32_t i = 0; i < n; i++) raster_triangle(uv + 6 * (size_t)i, tri[i], size, emit_write, &e, NULL);
	free(e.cursor);
	return e.total;
}

void orc_texel_flags(const float* uv, uint32_t n, uint32_t size, uint8_t* flags) {
	memset(flags, 0, (size_t)size * size);
	for (uint32_t i = 0; i < n; i++) raster_triangle(uv + 6 * (size_t)i, i, size, NULL, NULL, flags);
}

/* -------------------------------------------------------------- gather */
/* HomogenousFiller2::GetTrianglePoint (gather.cpp:65-83) */
static void filler_point(unsigned n, float* a, float* b) {
	static const float dir[4][3] = {
		{0, 0, -0.5f}, {0, 1, 0.5f}, {0.86602540378444f, -0.5f, 0.5f}, {-0.86602540378444f, -0.5f, 0.5f}};
	float x = 0, y = 0, dist = 1;
	while (n) {
		x += dist * dir[n & 3][0];
		y += dist * dir[n & 3][1];
		dist *= dir[n & 3][2];
		n >>= 2;
	}
	*a = x;
	*b = y;
}

typedef struct { double x, y, z; } d3;

static void basis_from_normal(v3 n, v3* t, v3* b) {
	*t = normalized(ortho1(n));
	*b = cross(n, *t);
}

/* point light irradiance, REALISTIC falloff (RRLight.cpp:345-362) */
static v3 point_irradiance(const orc_gather_scene* sc, v3 p) {
	v3 d = sub(p, ld3(sc->point_position));
	float att = 1 / (PREVENT_INF + len2(d));
	return mul(ld3(sc->point_color), att);
}

static v3 tri_normal(const orc_gather_scene* sc, uint32_t t, v3* v0, v3* s1, v3* s2) {
	*v0 = ld3(sc->xyz + 3 * (size_t)sc->idx[3 * t]);
	*s1 = sub(ld3(sc->xyz + 3 * (size_t)sc->idx[3 * t + 1]), *v0);
	*s2 = sub(ld3(sc->xyz + 3 * (size_t)sc->idx[3 * t + 2]), *v0);
	v3 n = cross(*s1, *s2);
	float l = len(n);
	return l ? divf(n, l) : mk(1, 0, 0);   /* normalizedSafe (RRMath.h:180) */
}

/* one hemisphere sample: getIncidentRadiance restated iteratively */
static void path(const orc_bvh* bvh, const orc_gather_scene* sc, v3 eye, v3 dir, uint32_t skip, uint64_t sid,
                 int fp64, v3* Lf, d3* Ld, float* first_t) {
	v3 T = mk(1, 1, 1);
	d3 Td = {1, 1, 1};
	v3 L = mk(0, 0, 0);
	d3 LD = {0, 0, 0};
	float tmax = sc->locality;
	const float tmin = sc->ray_length_min;
	if (sc->solver_direct) {
		/* the solver read at the first hit: direct from the triangle, indirect
		 * interpolated from its corners, times the albedo; the diffuse path
		 * ends there (pathtracer.cpp:235-258, 326-350; rrcore.cpp:262-277) */
		float dist, uv[2];
		uint32_t tri = orc_cast_uv(bvh, &eye.x, &dir.x, tmin, tmax, skip, &dist, uv);
		if (tri != 0xFFFFFFFFu) {
			*first_t = dist;
			const float* c = sc->solver_corner + 9 * (size_t)tri;
			float w = 1 - uv[0] - uv[1];
			v3 ind = add(add(mul(ld3(c), w), mul(ld3(c + 3), uv[0])), mul(ld3(c + 6), uv[1]));
			v3 alb = ld3(sc->albedo + 3 * (size_t)tri);
			L = add(mulv(ld3(sc->solver_direct + 3 * (size_t)tri), alb), mulv(ind, alb));
			LD.x = L.x;
			LD.y = L.y;
			LD.z = L.z;
		}
		*Lf = L;
		*Ld = LD;
		return;
	}
	for (uint32_t depth = 0;; depth++) {
		float dist, plane[4];
		uint32_t tri = orc_cast(bvh, &eye.x, &dir.x, tmin, tmax, 0, skip, &dist, plane);
		if (tri == 0xFFFFFFFFu) break;
		if (depth == 0) *first_t = dist;
		v3 p = add(eye, mul(dir, dist));
		v3 n = mk(plane[0], plane[1], plane[2]);
		v3 alb = ld3(sc->albedo + 3 * (size_t)tri);
		for (int li = 0; li < 2; li++) {
			v3 sdir;
			float smax;
			if (li == 0) {
				sdir = neg(ld3(sc->dir_direction));
				smax = 1e10f;
			} else {
				v3 d = sub(ld3(sc->point_position), p);
				sdir = normalized(d);
				smax = len(d);
			}
			if (!(dot(n, sdir) > 0)) continue;
			v3 unob = li == 0 ? ld3(sc->dir_color) : point_irradiance(sc, p);
			float dif = -dot(neg(sdir), n);
			dif = clampf_(dif, 0, 1);
			v3 contrib = mulv(unob, mul(alb, dif));
			if (contrib.x == 0 && contrib.y == 0 && contrib.z == 0) continue;
			if (orc_cast(bvh, &p.x, &sdir.x, tmin, smax, 1, tri, NULL, NULL) != 0xFFFFFFFFu) continue;
			if (fp64) {
				LD.x += Td.x * contrib.x;
				LD.y += Td.y * contrib.y;
				LD.z += Td.z * contrib.z;
			} else {
				L = add(L, mulv(T, contrib));
			}
		}
		tmax = 1e10f;
		float pdiff = avg(alb);
		if (pdiff < 0) pdiff = 0;
		float pstop = 1 - pdiff;
		if (pstop < 0) pstop = 0;
		float r = rng01(sc->seed, S_ROULETTE, sid * (MAX_DEPTH + 1) + depth);
		if (!(r < pdiff && depth < (sc->max_depth < MAX_DEPTH ? sc->max_depth : MAX_DEPTH))) break;
		float intensity = (pdiff + pstop) / pdiff;
		float x = 0, y = 0;
		for (uint32_t j = 0; j < DISK_TRIES; j++) {
			uint64_t c = (sid * (MAX_DEPTH + 1) + depth) * DISK_TRIES + j;
			float a = rng01(sc->seed, S_DISKX, c) * 2.0f - 1.0f;
			float b = rng01(sc->seed, S_DISKY, c) * 2.0f - 1.0f;
			if (a * a + b * b < 1.0f) { x = a; y = b; break; }
		}
		float cosT = sqrtf(1.0f - (x * x + y * y));
		v3 tg, bt;
		basis_from_normal(n, &tg, &bt);
		v3 s = add(add(mul(n, cosT), mul(tg, x)), mul(bt, y));
		float pdf = cosT;
		v3 dirIn = neg(s);
		float dif = clampf_(-dot(dirIn, n), 0, 1);
		v3 colorOut = mul(alb, dif);
		if (!(pdf > 0 && dot(dirIn, n) < 0)) break;
		v3 rs = mul(colorOut, intensity / pdf);
		if (!(avg(rs) > STOP_AT_VISIBILITY)) break;
		T = mulv(T, rs);
		Td.x *= rs.x;
		Td.y *= rs.y;
		Td.z *= rs.z;
		eye = p;
		dir = s;
		skip = tri;
	}
	*Lf = L;
	*Ld = LD;
}

/* RRVec3::abs().avg() (RRMath.h:170-171) */
static float absavg(v3 v) { return (fabsf(v.x) + fabsf(v.y) + fabsf(v.z)) * 0.33333333333333f; }

/* Directional lightmaps, compatible with Unreal Engine 3 (gather.cpp:43-49):
 * LS_LIGHTMAP and LS_DIRECTION1..3 in tangent space. */
static void lightmap_directions(float D[4][3]) {
	const float s6 = sqrtf(6.0f), s3 = sqrtf(3.0f), s2 = sqrtf(2.0f);
	D[0][0] = 0; D[0][1] = 0; D[0][2] = 1;
	D[1][0] = 0; D[1][1] = s6 / 3; D[1][2] = 1 / s3;
	D[2][0] = -1 / s2; D[2][1] = -1 / s6; D[2][2] = 1 / s3;
	D[3][0] = 1 / s2; D[3][1] = -1 / s6; D[3][2] = 1 / s3;
}

static void gather_texel(const orc_bvh* bvh, const orc_gather_scene* sc, uint64_t tid, const orc_subtexel* S,
                         uint32_t m, int fp64, float* out, float* bent, float* dirs) {
	if (bent) bent[0] = bent[1] = bent[2] = bent[3] = 0;
	if (dirs)
		for (int i = 0; i < 12; i++) dirs[i] = 0;
	if (!m) {
		out[0] = out[1] = out[2] = out[3] = 0;
		return;
	}
	for (uint32_t i = 0; i < m; i++)
		if (S[i].tri >= sc->nt) {   /* malformed input: no answer rather than a wild read */
			out[0] = out[1] = out[2] = out[3] = NAN;
			return;
		}
	v3 bentH = mk(0, 0, 0), bentL = mk(0, 0, 0);
	uint32_t distant = 0;
	const uint32_t Q = sc->quality ? sc->quality : 1;
	const uint32_t rounds = Q / 10 + 1;
	const uint32_t N = Q > rounds ? Q : rounds;
	float areaMax = 0;
	for (uint32_t i = 0; i < m; i++) areaMax += S[i].area;
	float areaStep = areaMax / ((float)N + 0.91f);
	float areaAccu = -S[0].area;
	uint32_t it = 0;
	unsigned num = (unsigned)(orc_hash(sc->seed, S_FILLER, tid) & 0xffff);
	v3 hemi = mk(0, 0, 0), lights = mk(0, 0, 0);
	d3 hemiD = {0, 0, 0}, lightsD = {0, 0, 0};
	/* directional mode (gatherAllDirections, lightmap.cpp:820): all four
	 * outputs weighted by the UE3 basis (gather.cpp:255-272, 468-486) */
	float D[4][3];
	lightmap_directions(D);
	v3 hemiI[4], lightsI[4];
	for (int i = 0; i < 4; i++) hemiI[i] = lightsI[i] = mk(0, 0, 0);
	uint32_t gl = 0, shotRounds = 0;
	const float tmin = sc->ray_length_min;
	for (uint32_t k = 0; k < N; k++) {
		areaAccu += areaStep;
		while (areaAccu > 0) {
			it++;
			if (it == m) it = 0;
			areaAccu -= S[it].area;
		}
		const orc_subtexel* st = &S[it];
		v3 v0, s1, s2;
		v3 fn = tri_normal(sc, st->tri, &v0, &s1, &s2);
		/* interpolated vertex normals at the sub-texel centre (gather.cpp:725-730) */
		float cu = (st->uv[0][0] + st->uv[1][0] + st->uv[2][0]) * 0.333333333f;
		float cv = (st->uv[0][1] + st->uv[1][1] + st->uv[2][1]) * 0.333333333f;
		float w = 1 - cu - cv;
		v3 nrm = normalized(add(add(mul(fn, w), mul(fn, cu)), mul(fn, cv)));
		v3 tg, bt;
		basis_from_normal(nrm, &tg, &bt);
		/* the skewed basis (gather.cpp:725-730): the vertices' bases (each the
		 * plane normal's, RRMesh.cpp:77-91) interpolated and normalised, and the
		 * four lightmap directions in it */
		v3 ldir[4];
		if (dirs) {
			v3 ft, fb;
			basis_from_normal(fn, &ft, &fb);
			v3 ts = normalized(add(add(mul(ft, w), mul(ft, cu)), mul(ft, cv)));
			v3 bs = normalized(add(add(mul(fb, w), mul(fb, cu)), mul(fb, cv)));
			for (int i = 0; i < 4; i++)
				ldir[i] = normalized(add(add(mul(ts, D[i][0]), mul(bs, D[i][1])), mul(nrm, D[i][2])));
		}
		/* random point in the sub-texel (gather.cpp:742-752) */
		uint64_t sid = tid * N + k;
		uint32_t ru = rng24(sc->seed, S_PU, sid), rv = rng24(sc->seed, S_PV, sid);
		if (ru + rv > M24) { ru = M24 - ru; rv = M24 - rv; }
		float fu = (float)ru / (float)M24, fv = (float)rv / (float)M24;
		float pu = (st->uv[0][0] + (st->uv[1][0] - st->uv[0][0]) * fu) + (st->uv[2][0] - st->uv[0][0]) * fv;
		float pv = (st->uv[0][1] + (st->uv[1][1] - st->uv[0][1]) * fu) + (st->uv[2][1] - st->uv[0][1]) * fv;
		v3 origin = add(add(v0, mul(s1, pu)), mul(s2, pv));
		if (k < Q) {
			/* hemisphere ray (gather.cpp:230-279) */
			float x, y, dd;
			do {
				filler_point(num++, &x, &y);
			} while ((dd = x * x + y * y) >= 1);
			float cosa = sqrtf(1 - dd);
			v3 dir = add(add(mul(nrm, cosa), mul(tg, x)), mul(bt, y));
			v3 L;
			d3 LD;
			float first_t = 1e10f;
			path(bvh, sc, origin, dir, st->tri, sid, fp64, &L, &LD, &first_t);
			if (first_t > sc->ao_size) distant++;
			bentH = add(bentH, mul(dir, absavg(L)));
			hemi = add(hemi, L);
			if (dirs) {
				float ni1 = dot(dir, nrm);
				if (ni1 > 0) {
					float inv = 1 / ni1;
					for (int i = 0; i < 4; i++) {
						float ni2 = dot(dir, ldir[i]);
						if (ni2 > 0) hemiI[i] = add(hemiI[i], mul(L, ni2 * inv));
					}
				}
			}
			hemiD.x += LD.x;
			hemiD.y += LD.y;
			hemiD.z += LD.z;
		}
		if ((uint64_t)gl * (N - 1) < (uint64_t)rounds * k || rounds >= Q) {
			gl++;
			for (int li = 0; li < 2; li++) {
				v3 d = li == 0 ? neg(ld3(sc->dir_direction)) : sub(ld3(sc->point_position), origin);
				float dsize = len(d);
				d = divf(d, dsize);
				if (li == 0) dsize *= sc->locality;
				float ni = dot(d, nrm);
				if (ni <= 0 || !isfinite(ni)) continue;
				if (orc_cast(bvh, &origin.x, &d.x, tmin, dsize, 1, st->tri, NULL, NULL) != 0xFFFFFFFFu) continue;
				v3 irr = li == 0 ? ld3(sc->dir_color) : point_irradiance(sc, origin);
				bentL = add(bentL, mul(d, absavg(irr) * ni));
				lights = add(lights, mul(irr, ni));
				if (dirs)
					for (int i = 0; i < 4; i++) {
						float ni2 = dot(d, ldir[i]);
						if (ni2 > 0) lightsI[i] = add(lightsI[i], mul(irr, ni2));
					}
				lightsD.x += (double)irr.x * ni;
				lightsD.y += (double)irr.y * ni;
				lightsD.z += (double)irr.z * ni;
			}
			shotRounds++;
		}
	}
	const int ao = sc->ao_intensity > 0 && sc->ao_size > 0;
	const float aof = ao ? powf((float)distant / (float)Q, sc->ao_intensity) : 1.0f;
	if (fp64) {
		double f = 1.0 / (double)Q * aof;
		out[0] = (float)(lightsD.x / shotRounds + hemiD.x * f);
		out[1] = (float)(lightsD.y / shotRounds + hemiD.y * f);
		out[2] = (float)(lightsD.z / shotRounds + hemiD.z * f);
	} else {
		float f = 1 / (float)Q;
		if (ao) f = f * aof;
		lights = divf(lights, (float)shotRounds);
		hemi = mul(hemi, f);
		v3 r = add(lights, hemi);
		out[0] = r.x;
		out[1] = r.y;
		out[2] = r.z;
	}
	out[3] = sc->flags ? (float)sc->flags[tid] / 255.f : 1.f;
	if (dirs) {
		float f = 1 / (float)Q;
		if (ao) f = f * aof;
		for (int i = 0; i < 4; i++) {
			v3 r = add(divf(lightsI[i], (float)shotRounds), mul(hemiI[i], f));
			float* o = i == 0 ? out : dirs + 4 * (i - 1);
			o[0] = r.x;
			o[1] = r.y;
			o[2] = r.z;
			o[3] = out[3];
		}
	}
	if (bent) {
		v3 b = add(bentL, bentH);
		if (b.x != 0 || b.y != 0 || b.z != 0) b = divf(b, len(b));
		bent[0] = (b.x + 1) * 0.5f;
		bent[1] = (b.y + 1) * 0.5f;
		bent[2] = (b.z + 1) * 0.5f;
		bent[3] = out[3];
	}
}

void orc_gather_dir(const orc_bvh* bvh, const orc_gather_scene* sc, const uint64_t* texel_id, uint32_t ntexels,
                    const uint64_t* off, const orc_subtexel* st, int threads, int fp64, float* out, float* bent,
                    float* dirs) {
#ifdef _OPENMP
	if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
	for (long i = 0; i < (long)ntexels; i++)
		gather_texel(bvh, sc, texel_id[i], st + off[i], (uint32_t)(off[i + 1] - off[i]), fp64, out + 4 * (size_t)i,
		             bent ? bent + 4 * (size_t)i : NULL, dirs ? dirs + 12 * (size_t)i : NULL);
}

void orc_gather_ex(const orc_bvh* bvh, const orc_gather_scene* sc, const uint64_t* texel_id, uint32_t ntexels,
                   const uint64_t* off, const orc_subtexel* st, int threads, int fp64, float* out, float* bent) {
	orc_gather_dir(bvh, sc, texel_id, ntexels, off, st, threads, fp64, out, bent, NULL);
}

void orc_gather(const orc_bvh* bvh, const orc_gather_scene* sc, const uint64_t* texel_id, uint32_t ntexels,
                const uint64_t* off, const orc_subtexel* st, int threads, int fp64, float* out) {
	orc_gather_ex(bvh, sc, texel_id, ntexels, off, st, threads, fp64, out, NULL);
}

/* ---------------------------------------------------------------- bake */
/* The default bake's radiosity solver.  Deliberate differences from the
 * reference, shared with the GPU: the same hash streams instead of rand()
 * and boost::rand48; factor-ray directions by Malley's method (the
 * distribution of rrcore.cpp:1026-1038); the converged solution of the flux
 * balance by Jacobi iteration of its gathering form (each triangle's own
 * rays estimate the form factors it receives through; by reciprocity the
 * same system the reference's progressive shooting solves, rrcore.cpp:
 * 1052-1297), where the reference stops at its accuracy target. */
enum { S_TRI_PU = 80, S_TRI_PV = 81, S_FF_PU = 82, S_FF_PV = 83, S_FF_DX = 84, S_FF_DY = 85 };
#define SHOT_OFFSET 1e-4f   /* geometry_v.h:30 */
#define BIG_REAL 1e20f      /* geometry_v.h:28 */

/* a random point of the triangle (gather.cpp:742-749 with the whole
 * triangle as sub-texel; rrcore.cpp:1016-1024) */
static void tri_point(uint64_t seed, uint64_t su, uint64_t sv, uint64_t i, float* pu, float* pv) {
	uint32_t ru = rng24(seed, su, i), rv = rng24(seed, sv, i);
	if (ru + rv > M24) { ru = M24 - ru; rv = M24 - rv; }
	*pu = (float)ru / (float)M24;
	*pv = (float)rv / (float)M24;
}

static float sum3(v3 a) { return a.x + a.y + a.z; }

void orc_bake_direct(const orc_bvh* bvh, const orc_gather_scene* sc, int threads, float* direct) {
	const uint32_t qh = sc->quality / 2 ? sc->quality / 2 : 1;
	const uint32_t rounds = qh / 10 + 1;
	if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 64)
	for (int64_t ti = 0; ti < (int64_t)sc->nt; ti++) {
		const uint32_t t = (uint32_t)ti;
		v3 v0, s1, s2;
		v3 n = tri_normal(sc, t, &v0, &s1, &s2);
		v3 acc = mk(0, 0, 0);
		for (uint32_t r = 0; r < rounds; r++) {
			float pu, pv;
			tri_point(sc->seed, S_TRI_PU, S_TRI_PV, (uint64_t)t * rounds + r, &pu, &pv);
			v3 o = add(add(v0, mul(s1, pu)), mul(s2, pv));
			for (int li = 0; li < 2; li++) {
				v3 d = li == 0 ? neg(ld3(sc->dir_direction)) : sub(ld3(sc->point_position), o);
				float dsize = len(d);
				d = divf(d, dsize);
				if (li == 0) dsize *= sc->locality;
				float ni = dot(d, n);
				if (ni <= 0 || !isfinite(ni)) continue;
				if (orc_cast(bvh, &o.x, &d.x, sc->ray_length_min, dsize, 1, t, NULL, NULL) != 0xFFFFFFFFu) continue;
				v3 irr = li == 0 ? ld3(sc->dir_color) : point_irradiance(sc, o);
				acc = add(acc, mul(irr, ni));
			}
		}
		acc = divf(acc, (float)rounds);
		direct[3 * (size_t)t] = acc.x;
		direct[3 * (size_t)t + 1] = acc.y;
		direct[3 * (size_t)t + 2] = acc.z;
	}
}

void orc_bake_factors(const orc_bvh* bvh, const orc_gather_scene* sc, uint32_t k, int threads, uint32_t* hits) {
	if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 64)
	for (int64_t ti = 0; ti < (int64_t)sc->nt; ti++) {
		const uint32_t t = (uint32_t)ti;
		v3 v0, s1, s2;
		v3 n = tri_normal(sc, t, &v0, &s1, &s2);
		v3 tg, bt;
		basis_from_normal(n, &tg, &bt);
		for (uint32_t j = 0; j < k; j++) {
			const uint64_t i = (uint64_t)t * k + j;
			float pu, pv;
			tri_point(sc->seed, S_FF_PU, S_FF_PV, i, &pu, &pv);
			v3 o = add(add(v0, mul(s1, pu)), mul(s2, pv));
			float x = 0, y = 0;
			for (uint32_t q = 0; q < DISK_TRIES; q++) {
				uint64_t c = i * DISK_TRIES + q;
				float a = rng01(sc->seed, S_FF_DX, c) * 2.0f - 1.0f;
				float b = rng01(sc->seed, S_FF_DY, c) * 2.0f - 1.0f;
				if (a * a + b * b < 1.0f) { x = a; y = b; break; }
			}
			float cosa = sqrtf(1.0f - (x * x + y * y));
			v3 d = add(add(mul(n, cosa), mul(tg, x)), mul(bt, y));
			int front = 0;
			uint32_t h = orc_cast_photon(bvh, &o.x, &d.x, SHOT_OFFSET, BIG_REAL, t, &front);
			hits[i] = (h != 0xFFFFFFFFu && front && sum3(ld3(sc->albedo + 3 * (size_t)h)) > 0.01f) ? h : 0xFFFFFFFFu;
		}
	}
}

void orc_bake_propagate(const orc_gather_scene* sc, const float* direct, const uint32_t* hits, uint32_t k,
                        uint32_t iterations, float* indirect) {
	const size_t n3 = 3 * (size_t)sc->nt;
	float* e = (float*)malloc(n3 * sizeof(float));
	float* f = (float*)malloc(n3 * sizeof(float));
	memcpy(e, direct, n3 * sizeof(float));
	const float inv = 1.0f / (float)(k ? k : 1);
	for (uint32_t it = 0; it < iterations; it++) {
#pragma omp parallel for schedule(static)
		for (int64_t ti = 0; ti < (int64_t)sc->nt; ti++) {
			v3 acc = mk(0, 0, 0);
			for (uint32_t j = 0; j < k; j++) {
				const uint32_t h = hits[(size_t)ti * k + j];
				if (h == 0xFFFFFFFFu) continue;
				acc = add(acc, mulv(ld3(sc->albedo + 3 * (size_t)h), ld3(e + 3 * (size_t)h)));
			}
			v3 r = add(ld3(direct + 3 * ti), mul(acc, inv));
			f[3 * ti] = r.x;
			f[3 * ti + 1] = r.y;
			f[3 * ti + 2] = r.z;
		}
		float* tmp = e;
		e = f;
		f = tmp;
	}
	for (size_t i = 0; i < n3; i++) indirect[i] = e[i] - direct[i];
	free(e);
	free(f);
}

/* Abramowitz & Stegun 4.4.45, as geometry_v.h:114-129 applies it (over the
 * whole [-1, 1]) */
static float as_acos(float x) {
	float root = sqrtf(1.0f - x);
	float r = -0.0187293f;
	r *= x;
	r += 0.0742610f;
	r *= x;
	r -= 0.2121144f;
	r *= x;
	r += 1.5707288f;
	return r * root;
}

/* rrcore.cpp:105-111 */
static float tri_area(v3 s1, v3 s2) {
	float a = len2(s1), b = len2(s2), c = len2(sub(s2, s1));
	return sqrtf(2 * b * c + 2 * c * a + 2 * a * b - a * a - b * b - c * c) / 4;
}

typedef struct { float p[3], n[3]; uint32_t c; } corner_key;

static int cmp_corner(const void* x, const void* y) {
	const corner_key* a = (const corner_key*)x;
	const corner_key* b = (const corner_key*)y;
	for (int i = 0; i < 3; i++)
		if (a->p[i] != b->p[i]) return a->p[i] < b->p[i] ? -1 : 1;
	for (int i = 0; i < 3; i++)
		if (a->n[i] != b->n[i]) return a->n[i] < b->n[i] ? -1 : 1;
	return a->c < b->c ? -1 : (a->c > b->c);
}

uint32_t orc_bake_stitch(const float* xyz, const uint32_t* idx, uint32_t nt, uint32_t* group, float* weight) {
	/* every corner is a vertex of its own with its face's normal (the mesh
	 * has flat normals); RRLessVerticesFilter merges identical positions
	 * whose normals are within 0.01 rad, greedily in (position, normal) order
	 * against the unique vertices found so far, newest first */
	const uint32_t nc = 3 * nt;
	corner_key* k = (corner_key*)malloc((size_t)(nc ? nc : 1) * sizeof(corner_key));
	for (uint32_t t = 0; t < nt; t++) {
		v3 p0 = ld3(xyz + 3 * (size_t)idx[3 * t]);
		v3 n = cross(sub(ld3(xyz + 3 * (size_t)idx[3 * t + 1]), p0), sub(ld3(xyz + 3 * (size_t)idx[3 * t + 2]), p0));
		float l = len(n);
		if (l > 0) n = divf(n, l);
		for (int i = 0; i < 3; i++) {
			corner_key* c = &k[3 * t + i];
			const float* p = xyz + 3 * (size_t)idx[3 * t + i];
			c->p[0] = p[0]; c->p[1] = p[1]; c->p[2] = p[2];
			c->n[0] = n.x; c->n[1] = n.y; c->n[2] = n.z;
			c->c = 3 * t + i;
		}
	}
	qsort(k, nc, sizeof(corner_key), cmp_corner);
	uint32_t* rep = (uint32_t*)malloc((size_t)(nc ? nc : 1) * sizeof(uint32_t));   /* unique -> sorted slot */
	uint32_t nu = 0;
	const float min_dot = cosf(0.01f);
	for (uint32_t s = 0; s < nc; s++) {
		const corner_key* d = &k[s];
		uint32_t g = 0xFFFFFFFFu;
		for (uint32_t u = nu; u--;) {
			const corner_key* r = &k[rep[u]];
			if (!(fabsf(d->p[0] - r->p[0]) <= 0.0f)) break;
			if (fabsf(d->p[1] - r->p[1]) <= 0.0f && fabsf(d->p[2] - r->p[2]) <= 0.0f &&
			    d->n[0] * r->n[0] + d->n[1] * r->n[1] + d->n[2] * r->n[2] >= min_dot) {
				g = u;
				break;
			}
		}
		if (g == 0xFFFFFFFFu) {
			rep[nu] = s;
			g = nu++;
		}
		group[d->c] = g;
	}
	/* Object::buildTopIVertices (interpol.cpp:120-170): corner weight =
	 * corner angle x triangle area; triangles that stitching degenerates or
	 * that have no area get none */
	for (uint32_t t = 0; t < nt; t++) {
		v3 p[3];
		for (int i = 0; i < 3; i++) p[i] = ld3(xyz + 3 * (size_t)idx[3 * t + i]);
		float area = tri_area(sub(p[1], p[0]), sub(p[2], p[0]));
		const uint32_t* g = group + 3 * t;
		int ok = area > 0 && g[0] != g[1] && g[0] != g[2] && g[1] != g[2];
		for (int i = 0; i < 3; i++) {
			float w = 0;
			if (ok) {
				v3 a = normalized(sub(p[(i + 1) % 3], p[i])), b = normalized(sub(p[(i + 2) % 3], p[i]));
				float dd = dot(a, b);
				dd = dd < -1 ? -1 : (dd > 1 ? 1 : dd);
				w = as_acos(dd) * area;
			}
			weight[3 * t + i] = w;
		}
	}
	free(rep);
	free(k);
	return nu;
}

void orc_bake_smooth(uint32_t nt, const uint32_t* group, const float* weight, uint32_t ngroups,
                     const float* indirect, float* corner) {
	float* num = (float*)calloc(3 * (size_t)(ngroups ? ngroups : 1), sizeof(float));
	float* den = (float*)calloc((size_t)(ngroups ? ngroups : 1), sizeof(float));
	for (uint32_t c = 0; c < 3 * nt; c++) {
		const uint32_t g = group[c];
		const float w = weight[c];
		if (w == 0) continue;
		const float* I = indirect + 3 * (size_t)(c / 3);
		num[3 * (size_t)g] += I[0] * w;
		num[3 * (size_t)g + 1] += I[1] * w;
		num[3 * (size_t)g + 2] += I[2] * w;
		den[g] += w;
	}
	for (uint32_t c = 0; c < 3 * nt; c++) {
		const uint32_t g = group[c];
		for (int i = 0; i < 3; i++) {
			float v = den[g] > 0 ? num[3 * (size_t)g + i] / den[g] : 0;
			corner[3 * (size_t)c + i] = v > 0 ? v : 0;   /* clampToZero (interpol.cpp:104) */
		}
	}
	free(num);
	free(den);
}
