/* ORACLE: CPU restatement of the reference collider arithmetic.  Test
 * infrastructure only (see rr_oracle.h for what is restated from where).
 * Compile with -ffp-contract=off: every float operation must round once. */
#include "rr_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static float minf_(float a, float b) { return a < b ? a : b; }
static float maxf_(float a, float b) { return a > b ? a : b; }
static int finitef_(float x) { return isfinite(x); }

int orc_max_threads(void) {
#ifdef _OPENMP
	return omp_get_max_threads();
#else
	return 1;
#endif
}

/* RRCollider/IntersectBspFast.cpp:130-187 */
void orc_tri_setup(const float* a, const float* b, const float* c, orc_tri* t) {
	for (int k = 0; k < 3; k++) {
		t->s3[k] = a[k];
		t->r3[k] = b[k] - a[k];
		t->l3[k] = c[k] - a[k];
	}
	for (int k = 0; k < 3; k++) t->ir3[k] = 1.0f / t->r3[k];
	const float* r3 = t->r3;
	const float* l3 = t->l3;
	float rxy = l3[1] * r3[0] - l3[0] * r3[1];
	float ryz = l3[2] * r3[1] - l3[1] * r3[2];
	float rzx = l3[0] * r3[2] - l3[2] * r3[0];
	unsigned char ib;
	if (fabsf(rxy) >= fabsf(ryz)) {
		if (fabsf(rxy) >= fabsf(rzx)) { ib = 0; t->ireal = 1.0f / rxy; }
		else { ib = 2; t->ireal = 1.0f / rzx; }
	} else {
		if (fabsf(ryz) >= fabsf(rzx)) { ib = 1; t->ireal = 1.0f / ryz; }
		else { ib = 2; t->ireal = 1.0f / rzx; }
	}
	if (fabsf(r3[0]) >= fabsf(r3[1])) {
		if (fabsf(r3[0]) >= fabsf(r3[2])) ib += 3;
	} else {
		if (fabsf(r3[1]) >= fabsf(r3[2])) ib += 6;
	}
	/* n = normalized(r3 x l3); components written as the reference's
	 * orthogonalTo(a,b) (RRMathPrivate.h:55-58) */
	float nx = r3[1] * l3[2] - r3[2] * l3[1];
	float ny = -r3[0] * l3[2] + r3[2] * l3[0];
	float nz = r3[0] * l3[1] - r3[1] * l3[0];
	float sz = sqrtf(nx * nx + ny * ny + nz * nz);
	t->n4[0] = nx / sz;
	t->n4[1] = ny / sz;
	t->n4[2] = nz / sz;
	t->n4[3] = -(t->s3[0] * t->n4[0] + t->s3[1] * t->n4[1] + t->s3[2] * t->n4[2]);
	if (!(finitef_(t->n4[0]) && finitef_(t->n4[1]) && finitef_(t->n4[2]))) ib = 10;
	t->ibyte = ib;
}

/* RRCollider/IntersectBspFast.cpp:344-347 */
float orc_plane_distance(const orc_tri* t, const float* o, const float* d) {
	const float* n = t->n4;
	float nDotDir = d[0] * n[0] + d[1] * n[1] + d[2] * n[2];
	float nDotOrigin = o[0] * n[0] + o[1] * n[1] + o[2] * n[2] + n[3];
	return -nDotOrigin / nDotDir;
}

/* RRCollider/IntersectBspFast.cpp:189-252, hit point from
 * IntersectLinear.cpp:40-45 (update_hitPoint3d) */
int orc_tri_fastest(const orc_tri* t, const float* o, const float* d, float dist,
                    float* uo, float* vo, int* front) {
	static const unsigned char tab[11][3] = {{0, 1, 2}, {1, 2, 2}, {2, 0, 2}, {0, 1, 0}, {1, 2, 0}, {2, 0, 0},
	                                         {0, 1, 1}, {1, 2, 1}, {2, 0, 1}, {2, 0, 1}, {2, 0, 1}};
	float hp[3];
	for (int k = 0; k < 3; k++) hp[k] = o[k] + d[k] * dist;
	int X = tab[t->ibyte][0], Y = tab[t->ibyte][1], Z = tab[t->ibyte][2];
	float v = ((hp[Y] - t->s3[Y]) * t->r3[X] - (hp[X] - t->s3[X]) * t->r3[Y]) * t->ireal;
	if (v < 0 || v > 1) return 0;
	float u = (hp[Z] - t->s3[Z] - t->l3[Z] * v) * t->ir3[Z];
	if (u < 0 || u + v > 1) return 0;
	if (t->ibyte > 8) return 0;
	*front = (d[0] * t->n4[0] + d[1] * t->n4[1] + d[2] * t->n4[2]) < 0;
	*uo = u;
	*vo = v;
	return 1;
}

/* RRCollider/IntersectLinear.cpp:62-110 */
int orc_tri_linear(const float* v0, const float* v1, const float* v2, const float* o, const float* d,
                   float tmin, float tmax, float* dist, float* uo, float* vo, int* front) {
	float s1[3], s2[3], tv[3], p[3], q[3];
	for (int k = 0; k < 3; k++) { s1[k] = v1[k] - v0[k]; s2[k] = v2[k] - v0[k]; }
	p[0] = d[1] * s2[2] - d[2] * s2[1];
	p[1] = -d[0] * s2[2] + d[2] * s2[0];
	p[2] = d[0] * s2[1] - d[1] * s2[0];
	float det = s1[0] * p[0] + s1[1] * p[1] + s1[2] * p[2];
	int fr = det > 0;
	if (det == 0) return 0;
	for (int k = 0; k < 3; k++) tv[k] = o[k] - v0[k];
	float u = (tv[0] * p[0] + tv[1] * p[1] + tv[2] * p[2]) / det;
	if (u < 0 || u > 1) return 0;
	q[0] = tv[1] * s1[2] - tv[2] * s1[1];
	q[1] = -tv[0] * s1[2] + tv[2] * s1[0];
	q[2] = tv[0] * s1[1] - tv[1] * s1[0];
	float v = (d[0] * q[0] + d[1] * q[1] + d[2] * q[2]) / det;
	if (v < 0 || u + v > 1) return 0;
	float t = (s2[0] * q[0] + s2[1] * q[1] + s2[2] * q[2]) / det;
	if (t < tmin || t > tmax) return 0;
	*dist = t;
	*uo = u;
	*vo = v;
	*front = fr;
	return 1;
}

/* RRCollider/IntersectLinear.cpp:47-60 */
void orc_plane_linear(const float* v0, const float* v1, const float* v2, float* pl) {
	float s1[3], s2[3];
	for (int k = 0; k < 3; k++) { s1[k] = v1[k] - v0[k]; s2[k] = v2[k] - v0[k]; }
	float nx = s1[1] * s2[2] - s1[2] * s2[1];
	float ny = s1[2] * s2[0] - s1[0] * s2[2];
	float nz = s1[0] * s2[1] - s1[1] * s2[0];
	float siz = sqrtf(nx * nx + ny * ny + nz * nz);
	pl[0] = nx / siz;
	pl[1] = ny / siz;
	pl[2] = nz / siz;
	pl[3] = -(v0[0] * pl[0] + v0[1] * pl[1] + v0[2] * pl[2]);
}

/* RRCollider/geometry.cpp:20-31 */
void orc_box_init(const float* mn, const float* mx, float* bmin, float* bmax) {
	float dd = (mx[0] - mn[0] + mx[1] - mn[1] + mx[2] - mn[2]) * 1e-5f;
	for (int k = 0; k < 3; k++) { bmin[k] = mn[k] - dd; bmax[k] = mx[k] + dd; }
}

/* RRCollider/geometry.cpp:38-86 (the non-SSE path used on Linux) */
int orc_box_intersect(const float* bmin, const float* bmax, const float* o, const float* d,
                      float lenmin, float lenmax, float* hmin, float* hmax) {
	float l1 = (bmin[0] - o[0]) / d[0], l2 = (bmax[0] - o[0]) / d[0];
	float lmin = minf_(l1, l2), lmax = maxf_(l1, l2);
	l1 = (bmin[1] - o[1]) / d[1];
	l2 = (bmax[1] - o[1]) / d[1];
	lmin = maxf_(minf_(l1, l2), lmin);
	lmax = minf_(maxf_(l1, l2), lmax);
	l1 = (bmin[2] - o[2]) / d[2];
	l2 = (bmax[2] - o[2]) / d[2];
	lmin = maxf_(minf_(l1, l2), lmin);
	lmax = minf_(maxf_(l1, l2), lmax);
	lmin = maxf_(lenmin, lmin);
	lmax = minf_(lenmax, lmax);
	*hmin = lmin;
	*hmax = lmax;
	return (lmax >= 0.f) & (lmax >= lmin);
}

static void mesh_aabb(const float* xyz, const uint32_t* idx, uint32_t nt, float* mn, float* mx) {
	for (int k = 0; k < 3; k++) { mn[k] = INFINITY; mx[k] = -INFINITY; }
	for (size_t i = 0; i < 3 * (size_t)nt; i++) {
		const float* p = xyz + 3 * (size_t)idx[i];
		for (int k = 0; k < 3; k++) {
			if (p[k] < mn[k]) mn[k] = p[k];
			if (p[k] > mx[k]) mx[k] = p[k];
		}
	}
}

/* RRCollider/IntersectLinear.cpp:129-140: 1e-5 * max |coordinate| of the
 * inflated box */
float orc_delta_bsp(const float* xyz, uint32_t nv) {
	float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
	for (size_t i = 0; i < nv; i++)
		for (int k = 0; k < 3; k++) {
			float v = xyz[3 * i + k];
			if (v < mn[k]) mn[k] = v;
			if (v > mx[k]) mx[k] = v;
		}
	float bmin[3], bmax[3];
	orc_box_init(mn, mx, bmin, bmax);
	float m = 0;
	for (int k = 0; k < 3; k++) {
		float a = fabsf(bmax[k]) > fabsf(bmin[k]) ? fabsf(bmax[k]) : fabsf(bmin[k]);
		if (a > m) m = a;
	}
	if (m == 0 || isnan(m)) m = 1;
	return m * 1e-5f;
}

static void set_miss(orc_hits* o, size_t i) {
	o->hit[i] = 0;
	o->tri[i] = 0xFFFFFFFFu;
	o->dist[i] = 0;
	o->uv[2 * i] = o->uv[2 * i + 1] = 0;
	for (int k = 0; k < 4; k++) o->plane[4 * i + k] = 0;
	for (int k = 0; k < 3; k++) o->point3d[3 * i + k] = 0;
	o->side[i] = 0;
}

/* RRCollider/IntersectLinear.cpp:161-273: box clip, then every triangle in
 * index order; hitDistanceMax shrinks to each accepted hit, so among equal
 * distances the later triangle wins. */
void orc_collide_linear(const float* xyz, uint32_t nv, const uint32_t* idx, uint32_t nt,
                        const float* rays, uint32_t n, int threads, orc_hits* out) {
	(void)nv;
	float mn[3], mx[3], bmin[3], bmax[3];
	mesh_aabb(xyz, idx, nt, mn, mx);
	orc_box_init(mn, mx, bmin, bmax);
#ifdef _OPENMP
	if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
	for (long i = 0; i < (long)n; i++) {
		const float* r = rays + 8 * (size_t)i;
		const float* o = r;
		const float* d = r + 4;
		float hmin, hmax;
		set_miss(out, i);
		if (!nt || !orc_box_intersect(bmin, bmax, o, d, r[3], r[7], &hmin, &hmax)) continue;
		int hit = 0;
		for (uint32_t t = 0; t < nt; t++) {
			const float* v0 = xyz + 3 * (size_t)idx[3 * t];
			const float* v1 = xyz + 3 * (size_t)idx[3 * t + 1];
			const float* v2 = xyz + 3 * (size_t)idx[3 * t + 2];
			float dist, u, v;
			int fr;
			if (orc_tri_linear(v0, v1, v2, o, d, hmin, hmax, &dist, &u, &v, &fr)) {
				hit = 1;
				hmax = dist;
				out->tri[i] = t;
				out->dist[i] = dist;
				out->uv[2 * i] = u;
				out->uv[2 * i + 1] = v;
				out->side[i] = (uint8_t)fr;
			}
		}
		if (hit) {
			uint32_t t = out->tri[i];
			out->hit[i] = 1;
			orc_plane_linear(xyz + 3 * (size_t)idx[3 * t], xyz + 3 * (size_t)idx[3 * t + 1],
			                 xyz + 3 * (size_t)idx[3 * t + 2], out->plane + 4 * (size_t)i);
			for (int k = 0; k < 3; k++) out->point3d[3 * i + k] = o[k] + d[k] * out->dist[i];
		}
	}
}

/* ------------------------------------------------------------------------
 * Acceleration for the oracle: our own binned-SAH binary BVH over the valid
 * (ibyte < 10) triangles.  It only decides which triangles are tested; the
 * accepted hit is defined by the restated FASTEST arithmetic above. */
typedef struct { float mn[3], mx[3]; int32_t left, right; uint32_t first, count; } onode;
struct orc_bvh {
	onode* nodes;
	uint32_t nnodes;
	uint32_t* prims;   /* triangle ids in leaf order */
	orc_tri* tris;     /* per original triangle */
	const float* xyz;
	const uint32_t* idx;
	uint32_t nt;
	float bmin[3], bmax[3]; /* Box::init of the mesh AABB */
	float pad;              /* node inflation */
};

typedef struct { float mn[3], mx[3], c[3]; } pinfo;

static void grow(float* mn, float* mx, const float* a, const float* b) {
	for (int k = 0; k < 3; k++) {
		if (a[k] < mn[k]) mn[k] = a[k];
		if (b[k] > mx[k]) mx[k] = b[k];
	}
}
static float area(const float* mn, const float* mx) {
	float e0 = mx[0] - mn[0], e1 = mx[1] - mn[1], e2 = mx[2] - mn[2];
	if (e0 < 0) return 0;
	return e0 * e1 + e1 * e2 + e2 * e0;
}

#define OBINS 16
static uint32_t build_rec(orc_bvh* b, pinfo* pi, uint32_t* ids, uint32_t first, uint32_t count,
                          uint32_t* cap) {
	uint32_t me = b->nnodes++;
	if (b->nnodes > *cap) {
		*cap *= 2;
		b->nodes = (onode*)realloc(b->nodes, sizeof(onode) * (*cap));
	}
	float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
	float cmn[3] = {INFINITY, INFINITY, INFINITY}, cmx[3] = {-INFINITY, -INFINITY, -INFINITY};
	for (uint32_t i = first; i < first + count; i++) {
		grow(mn, mx, pi[ids[i]].mn, pi[ids[i]].mx);
		grow(cmn, cmx, pi[ids[i]].c, pi[ids[i]].c);
	}
	onode nd;
	for (int k = 0; k < 3; k++) { nd.mn[k] = mn[k] - b->pad; nd.mx[k] = mx[k] + b->pad; }
	nd.left = nd.right = -1;
	nd.first = first;
	nd.count = count;
	int best_axis = -1, best_bin = -1;
	float best_cost = INFINITY;
	if (count > 2) {
		for (int ax = 0; ax < 3; ax++) {
			float ext = cmx[ax] - cmn[ax];
			if (!(ext > 0)) continue;
			uint32_t cnt[OBINS] = {0};
			float bmn[OBINS][3], bmx[OBINS][3];
			for (int q = 0; q < OBINS; q++)
				for (int k = 0; k < 3; k++) { bmn[q][k] = INFINITY; bmx[q][k] = -INFINITY; }
			for (uint32_t i = first; i < first + count; i++) {
				int q = (int)((pi[ids[i]].c[ax] - cmn[ax]) / ext * OBINS);
				if (q >= OBINS) q = OBINS - 1;
				if (q < 0) q = 0;
				cnt[q]++;
				grow(bmn[q], bmx[q], pi[ids[i]].mn, pi[ids[i]].mx);
			}
			float ra[OBINS];
			uint32_t rc[OBINS];
			float amn[3] = {INFINITY, INFINITY, INFINITY}, amx[3] = {-INFINITY, -INFINITY, -INFINITY};
			uint32_t ac = 0;
			for (int q = OBINS - 1; q > 0; q--) {
				grow(amn, amx, bmn[q], bmx[q]);
				ac += cnt[q];
				ra[q] = area(amn, amx);
				rc[q] = ac;
			}
			for (int k = 0; k < 3; k++) { amn[k] = INFINITY; amx[k] = -INFINITY; }
			ac = 0;
			for (int q = 0; q < OBINS - 1; q++) {
				grow(amn, amx, bmn[q], bmx[q]);
				ac += cnt[q];
				if (!ac || !rc[q + 1]) continue;
				float cost = area(amn, amx) * ac + ra[q + 1] * rc[q + 1];
				if (cost < best_cost) { best_cost = cost; best_axis = ax; best_bin = q; }
			}
		}
	}
	float leaf_cost = area(mn, mx) * count;
	if (count <= 2 || (count <= 8 && best_cost >= leaf_cost) || best_axis < 0) {
		if (count > 8) {  /* all centroids equal: split by index */
			uint32_t h = count / 2;
			b->nodes[me] = nd;
			uint32_t l = build_rec(b, pi, ids, first, h, cap);
			uint32_t r = build_rec(b, pi, ids, first + h, count - h, cap);
			b->nodes[me].left = (int32_t)l;
			b->nodes[me].right = (int32_t)r;
			return me;
		}
		b->nodes[me] = nd;
		return me;
	}
	/* partition */
	float ext = cmx[best_axis] - cmn[best_axis];
	uint32_t i = first, j = first + count;
	while (i < j) {
		int q = (int)((pi[ids[i]].c[best_axis] - cmn[best_axis]) / ext * OBINS);
		if (q >= OBINS) q = OBINS - 1;
		if (q <= best_bin) i++;
		else { uint32_t tmp = ids[i]; ids[i] = ids[--j]; ids[j] = tmp; }
	}
	uint32_t nl = i - first;
	b->nodes[me] = nd;
	uint32_t l = build_rec(b, pi, ids, first, nl, cap);
	uint32_t r = build_rec(b, pi, ids, first + nl, count - nl, cap);
	b->nodes[me].left = (int32_t)l;
	b->nodes[me].right = (int32_t)r;
	return me;
}

orc_bvh* orc_bvh_build(const float* xyz, uint32_t nv, const uint32_t* idx, uint32_t nt) {
	orc_bvh* b = (orc_bvh*)calloc(1, sizeof(orc_bvh));
	b->xyz = xyz;
	b->idx = idx;
	b->nt = nt;
	b->tris = (orc_tri*)malloc(sizeof(orc_tri) * (nt ? nt : 1));
	float mn[3], mx[3];
	mesh_aabb(xyz, idx, nt, mn, mx);
	orc_box_init(mn, mx, b->bmin, b->bmax);
	b->pad = orc_delta_bsp(xyz, nv) * 10.0f;
	pinfo* pi = (pinfo*)malloc(sizeof(pinfo) * (nt ? nt : 1));
	uint32_t* ids = (uint32_t*)malloc(sizeof(uint32_t) * (nt ? nt : 1));
	uint32_t nvalid = 0;
	for (uint32_t t = 0; t < nt; t++) {
		const float* a = xyz + 3 * (size_t)idx[3 * t];
		const float* bb = xyz + 3 * (size_t)idx[3 * t + 1];
		const float* c = xyz + 3 * (size_t)idx[3 * t + 2];
		orc_tri_setup(a, bb, c, &b->tris[t]);
		if (b->tris[t].ibyte >= 10) continue;
		for (int k = 0; k < 3; k++) {
			float lo = a[k] < bb[k] ? a[k] : bb[k];
			lo = c[k] < lo ? c[k] : lo;
			float hi = a[k] > bb[k] ? a[k] : bb[k];
			hi = c[k] > hi ? c[k] : hi;
			pi[t].mn[k] = lo;
			pi[t].mx[k] = hi;
			pi[t].c[k] = 0.5f * (lo + hi);
		}
		if (!(isfinite(pi[t].mn[0]) && isfinite(pi[t].mn[1]) && isfinite(pi[t].mn[2]) &&
		      isfinite(pi[t].mx[0]) && isfinite(pi[t].mx[1]) && isfinite(pi[t].mx[2]))) {
			b->tris[t].ibyte = 10;
			continue;
		}
		ids[nvalid++] = t;
	}
	uint32_t cap = 1024;
	b->nodes = (onode*)malloc(sizeof(onode) * cap);
	b->nnodes = 0;
	if (nvalid) build_rec(b, pi, ids, 0, nvalid, &cap);
	b->prims = ids;
	free(pi);
	return b;
}

void orc_bvh_free(orc_bvh* b) {
	if (!b) return;
	free(b->nodes);
	free(b->prims);
	free(b->tris);
	free(b);
}

static int slab(const onode* nd, const float* o, const float* inv, float t0, float t1) {
	float lo = t0, hi = t1;
	for (int k = 0; k < 3; k++) {
		float a = (nd->mn[k] - o[k]) * inv[k];
		float c = (nd->mx[k] - o[k]) * inv[k];
		float n0 = a < c ? a : c, f0 = a < c ? c : a;
		if (isnan(a) || isnan(c)) { n0 = -INFINITY; f0 = INFINITY; }  /* origin on a slab plane, d=0 */
		if (n0 > lo) lo = n0;
		if (f0 < hi) hi = f0;
	}
	return lo <= hi;
}

/* Visits candidate triangles front to back; mode 0 = FASTEST nearest,
 * mode 1 = FASTEST any hit, mode 2 = exact f64 nearest. */
static void trace_one(const orc_bvh* b, const float* r, int mode, orc_hits* out, size_t i,
                      uint32_t* tri64, double* dist64) {
	const float* o = r;
	const float* d = r + 4;
	float hmin, hmax;
	if (out) set_miss(out, i);
	if (tri64) { tri64[i] = 0xFFFFFFFFu; dist64[i] = 0; }
	if (!b->nnodes) return;
	if (mode != 2 && !orc_box_intersect(b->bmin, b->bmax, o, d, r[3], r[7], &hmin, &hmax)) return;
	if (mode == 2) { hmin = r[3]; hmax = r[7]; }
	float inv[3] = {1.0f / d[0], 1.0f / d[1], 1.0f / d[2]};
	uint32_t stack[128];
	int sp = 0;
	stack[sp++] = 0;
	float best = hmax;
	uint32_t best_tri = 0xFFFFFFFFu;
	float bu = 0, bv = 0;
	int bfront = 0;
	double best64 = (double)hmax;
	while (sp) {
		const onode* nd = &b->nodes[stack[--sp]];
		float slack = 1e-6f * (fabsf(best) + fabsf(hmin)) + b->pad;
		if (!slab(nd, o, inv, hmin - slack, best + slack)) continue;
		if (nd->left < 0) {
			for (uint32_t k = nd->first; k < nd->first + nd->count; k++) {
				uint32_t t = b->prims[k];
				const orc_tri* tr = &b->tris[t];
				if (mode == 2) {
					const float* A = b->xyz + 3 * (size_t)b->idx[3 * t];
					const float* B = b->xyz + 3 * (size_t)b->idx[3 * t + 1];
					const float* C = b->xyz + 3 * (size_t)b->idx[3 * t + 2];
					double s1[3], s2[3], tv[3], p[3], q[3];
					for (int m = 0; m < 3; m++) {
						s1[m] = (double)B[m] - A[m];
						s2[m] = (double)C[m] - A[m];
						tv[m] = (double)o[m] - A[m];
					}
					p[0] = d[1] * s2[2] - d[2] * s2[1];
					p[1] = d[2] * s2[0] - d[0] * s2[2];
					p[2] = d[0] * s2[1] - d[1] * s2[0];
					double det = s1[0] * p[0] + s1[1] * p[1] + s1[2] * p[2];
					if (det == 0) continue;
					double u = (tv[0] * p[0] + tv[1] * p[1] + tv[2] * p[2]) / det;
					if (u < 0 || u > 1) continue;
					q[0] = tv[1] * s1[2] - tv[2] * s1[1];
					q[1] = tv[2] * s1[0] - tv[0] * s1[2];
					q[2] = tv[0] * s1[1] - tv[1] * s1[0];
					double v = (d[0] * q[0] + d[1] * q[1] + d[2] * q[2]) / det;
					if (v < 0 || u + v > 1) continue;
					double tt = (s2[0] * q[0] + s2[1] * q[1] + s2[2] * q[2]) / det;
					if (tt < hmin || tt > best64) continue;
					if (tt < best64 || t < best_tri) {
						best64 = tt;
						best_tri = t;
						best = (float)tt;
					}
					continue;
				}
				float dp = orc_plane_distance(tr, o, d);
				if (!(dp >= hmin && dp <= best)) continue;
				float u, v;
				int fr;
				if (!orc_tri_fastest(tr, o, d, dp, &u, &v, &fr)) continue;
				if (dp < best || t < best_tri) {
					best = dp;
					best_tri = t;
					bu = u;
					bv = v;
					bfront = fr;
				}
				if (mode == 1) { sp = 0; break; }
			}
		} else {
			const onode* l = &b->nodes[nd->left];
			const onode* rr = &b->nodes[nd->right];
			/* push the far child first */
			float dl = (l->mn[0] + l->mx[0]) * d[0] + (l->mn[1] + l->mx[1]) * d[1] + (l->mn[2] + l->mx[2]) * d[2];
			float dr = (rr->mn[0] + rr->mx[0]) * d[0] + (rr->mn[1] + rr->mx[1]) * d[1] + (rr->mn[2] + rr->mx[2]) * d[2];
			if (sp + 2 > 128) continue;  /* cannot happen for depth < 64 */
			if (dl <= dr) { stack[sp++] = (uint32_t)nd->right; stack[sp++] = (uint32_t)nd->left; }
			else { stack[sp++] = (uint32_t)nd->left; stack[sp++] = (uint32_t)nd->right; }
		}
	}
	if (mode == 2) {
		if (best_tri != 0xFFFFFFFFu) { tri64[i] = best_tri; dist64[i] = best64; }
		return;
	}
	if (best_tri == 0xFFFFFFFFu) return;
	const orc_tri* tr = &b->tris[best_tri];
	out->hit[i] = 1;
	out->tri[i] = best_tri;
	out->dist[i] = best;
	out->uv[2 * i] = bu;
	out->uv[2 * i + 1] = bv;
	for (int k = 0; k < 4; k++) out->plane[4 * i + k] = tr->n4[k];
	for (int k = 0; k < 3; k++) out->point3d[3 * i + k] = o[k] + d[k] * best;
	out->side[i] = (uint8_t)bfront;
}

void orc_collide_fastest(const orc_bvh* b, const float* rays, uint32_t n, int threads, int any_hit,
                         orc_hits* out) {
#ifdef _OPENMP
	if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1024)
#endif
	for (long i = 0; i < (long)n; i++) trace_one(b, rays + 8 * (size_t)i, any_hit ? 1 : 0, out, i, NULL, NULL);
}

void orc_collide_exact64(const orc_bvh* b, const float* rays, uint32_t n, int threads, uint32_t* tri,
                         double* dist) {
#ifdef _OPENMP
	if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1024)
#endif
	for (long i = 0; i < (long)n; i++) trace_one(b, rays + 8 * (size_t)i, 2, NULL, i, tri, dist);
}

/* ------------------------------------------------------------------------
 * Ray cast with the final-gathering collision handler
 * (RRStaticSolver/pathtracer.h:117-242) for opaque one-sided diffuse
 * materials (RRMaterial::reset(false), RRObject/RRMaterial.cpp:154-166):
 *   - the shooter triangle `skip` is never hit;
 *   - a triangle with the same three vertices as the shooter is not hit at
 *     distances below 1000 * tmin (pathtracer.h:138-161);
 *   - hemisphere rays (shadow = 0) see only front sides (back renderFrom = 0);
 *   - shadow rays (shadow = 1) are stopped by either side; any hit ends them.
 * Hits reach the handler nearest first, so the result is the nearest
 * accepted hit.  Returns its triangle (or 0xFFFFFFFF), FASTEST distance and
 * plane. */
static int same_vertices(const orc_bvh* b, uint32_t t, uint32_t s) {
	for (int i = 0; i < 3; i++) {
		const float* p = b->xyz + 3 * (size_t)b->idx[3 * t + i];
		int found = 0;
		for (int j = 0; j < 3 && !found; j++) {
			const float* q = b->xyz + 3 * (size_t)b->idx[3 * s + j];
			found = p[0] == q[0] && p[1] == q[1] && p[2] == q[2];
		}
		if (!found) return 0;
	}
	return 1;
}

/* mode 0: hemisphere, 1: shadow, 2: photon (RRCollisionHandlerLod0,
 * rrcore.cpp:670-723: every side collides, only the shooter is skipped) */
static uint32_t cast_impl(const orc_bvh* b, const float* o, const float* d, float tmin, float tmax, int shadow,
                          uint32_t skip, float* dist_out, float* plane_out, int* front_out, float* uv_out) {
	float hmin, hmax;
	if (!b->nnodes) return 0xFFFFFFFFu;
	if (!orc_box_intersect(b->bmin, b->bmax, o, d, tmin, tmax, &hmin, &hmax)) return 0xFFFFFFFFu;
	float inv[3] = {1.0f / d[0], 1.0f / d[1], 1.0f / d[2]};
	uint32_t stack[128];
	int sp = 0;
	stack[sp++] = 0;
	float best = hmax;
	uint32_t best_tri = 0xFFFFFFFFu;
	int best_fr = 0;
	float best_u = 0, best_v = 0;
	while (sp) {
		const onode* nd = &b->nodes[stack[--sp]];
		float slack = 1e-6f * (fabsf(best) + fabsf(hmin)) + b->pad;
		if (!slab(nd, o, inv, hmin - slack, best + slack)) continue;
		if (nd->left < 0) {
			for (uint32_t k = nd->first; k < nd->first + nd->count; k++) {
				uint32_t t = b->prims[k];
				const orc_tri* tr = &b->tris[t];
				float dp = orc_plane_distance(tr, o, d);
				if (!(dp >= hmin && dp <= best)) continue;
				float u, v;
				int fr;
				if (!orc_tri_fastest(tr, o, d, dp, &u, &v, &fr)) continue;
				if (t == skip) continue;
				if (shadow != 2 && skip != 0xFFFFFFFFu && dp < 1000 * tmin && same_vertices(b, t, skip)) continue;
				if (!shadow && !fr) continue;
				if (dp < best || t < best_tri) {
					best = dp;
					best_tri = t;
					best_fr = fr;
					best_u = u;
					best_v = v;
				}
				if (shadow == 1) { sp = 0; break; }
			}
		} else {
			const onode* l = &b->nodes[nd->left];
			const onode* rr = &b->nodes[nd->right];
			float dl = (l->mn[0] + l->mx[0]) * d[0] + (l->mn[1] + l->mx[1]) * d[1] + (l->mn[2] + l->mx[2]) * d[2];
			float dr = (rr->mn[0] + rr->mx[0]) * d[0] + (rr->mn[1] + rr->mx[1]) * d[1] + (rr->mn[2] + rr->mx[2]) * d[2];
			if (sp + 2 > 128) continue;
			if (dl <= dr) { stack[sp++] = (uint32_t)nd->right; stack[sp++] = (uint32_t)nd->left; }
			else { stack[sp++] = (uint32_t)nd->left; stack[sp++] = (uint32_t)nd->right; }
		}
	}
	if (best_tri != 0xFFFFFFFFu) {
		if (dist_out) *dist_out = best;
		if (plane_out)
			for (int k = 0; k < 4; k++) plane_out[k] = b->tris[best_tri].n4[k];
		if (front_out) *front_out = best_fr;
		if (uv_out) { uv_out[0] = best_u; uv_out[1] = best_v; }
	}
	return best_tri;
}

uint32_t orc_cast(const orc_bvh* b, const float* o, const float* d, float tmin, float tmax, int shadow,
                  uint32_t skip, float* dist_out, float* plane_out) {
	return cast_impl(b, o, d, tmin, tmax, shadow ? 1 : 0, skip, dist_out, plane_out, NULL, NULL);
}

uint32_t orc_cast_uv(const orc_bvh* b, const float* o, const float* d, float tmin, float tmax, uint32_t skip,
                     float* dist, float* uv) {
	return cast_impl(b, o, d, tmin, tmax, 0, skip, dist, NULL, NULL, uv);
}

uint32_t orc_cast_photon(const orc_bvh* b, const float* o, const float* d, float tmin, float tmax, uint32_t skip,
                         int* front) {
	*front = 0;
	return cast_impl(b, o, d, tmin, tmax, 2, skip, NULL, NULL, front, NULL);
}
