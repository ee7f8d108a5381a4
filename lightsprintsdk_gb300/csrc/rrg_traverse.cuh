// Device-side traversal shared by the collider kernels and the lightmap
// gather: ray set-up, slab test, watertight triangle test (Woop, Benthin,
// Wald, JCGT 2(1), 2013), the reference's FASTEST output fields, and the
// stack traversal of the binary BVH with optional gathering filters.
#pragma once
#include "rrg_internal.cuh"

namespace rrg {

constexpr int kTraceThreads = 128;

struct RayState {
	float ox, oy, oz, tmin, dx, dy, dz, tmax;
	float ix, iy, iz;       // 1/d (zero components replaced by +-1e-30)
	float oix, oiy, oiz;    // o * (1/d)
	// shear rows (watertight): A' = M (v - o)
	float m0x, m0y, m0z, m1x, m1y, m1z, m2x, m2y, m2z;
	float4 d_kz;            // unused padding for alignment
};

__device__ __forceinline__ float safe_inv(float d) {
	return 1.0f / (fabsf(d) > 1e-30f ? d : copysignf(1e-30f, d));
}

__device__ __forceinline__ void ray_setup(RayState& r) {
	r.ix = safe_inv(r.dx);
	r.iy = safe_inv(r.dy);
	r.iz = safe_inv(r.dz);
	r.oix = r.ox * r.ix;
	r.oiy = r.oy * r.iy;
	r.oiz = r.oz * r.iz;
	float ax = fabsf(r.dx), ay = fabsf(r.dy), az = fabsf(r.dz);
	int kz = (ax >= ay) ? (ax >= az ? 0 : 2) : (ay >= az ? 1 : 2);
	int kx = kz == 2 ? 0 : kz + 1;
	int ky = kx == 2 ? 0 : kx + 1;
	float dkz = kz == 0 ? r.dx : (kz == 1 ? r.dy : r.dz);
	if (dkz < 0.f) { int t = kx; kx = ky; ky = t; }
	float dkx = kx == 0 ? r.dx : (kx == 1 ? r.dy : r.dz);
	float dky = ky == 0 ? r.dx : (ky == 1 ? r.dy : r.dz);
	float Sx = dkx / dkz, Sy = dky / dkz, Sz = 1.0f / dkz;
	// row 0: e_kx - Sx e_kz ; row 1: e_ky - Sy e_kz ; row 2: Sz e_kz
	r.m0x = (kx == 0) ? 1.f : (kz == 0 ? -Sx : 0.f);
	r.m0y = (kx == 1) ? 1.f : (kz == 1 ? -Sx : 0.f);
	r.m0z = (kx == 2) ? 1.f : (kz == 2 ? -Sx : 0.f);
	r.m1x = (ky == 0) ? 1.f : (kz == 0 ? -Sy : 0.f);
	r.m1y = (ky == 1) ? 1.f : (kz == 1 ? -Sy : 0.f);
	r.m1z = (ky == 2) ? 1.f : (kz == 2 ? -Sy : 0.f);
	r.m2x = (kz == 0) ? Sz : 0.f;
	r.m2y = (kz == 1) ? Sz : 0.f;
	r.m2z = (kz == 2) ? Sz : 0.f;
}

// slab test against one child box; returns entry distance or +inf on miss
__device__ __forceinline__ float box_enter(const RayState& r, float lox, float hix, float loy, float hiy, float loz,
                                           float hiz, float tbest) {
	float tx0 = fmaf(lox, r.ix, -r.oix), tx1 = fmaf(hix, r.ix, -r.oix);
	float ty0 = fmaf(loy, r.iy, -r.oiy), ty1 = fmaf(hiy, r.iy, -r.oiy);
	float tz0 = fmaf(loz, r.iz, -r.oiz), tz1 = fmaf(hiz, r.iz, -r.oiz);
	float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), r.tmin));
	float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tbest));
	// conservative: never reject a box the exact test would accept
	return tn <= tf * 1.0000004f ? tn : INFINITY;
}

struct Shear { float x, y, z; };

__device__ __forceinline__ Shear shear(const RayState& r, float4 v) {
	float ax = v.x - r.ox, ay = v.y - r.oy, az = v.z - r.oz;
	Shear s;
	s.x = fmaf(r.m0x, ax, fmaf(r.m0y, ay, r.m0z * az));
	s.y = fmaf(r.m1x, ax, fmaf(r.m1y, ay, r.m1z * az));
	s.z = fmaf(r.m2x, ax, fmaf(r.m2y, ay, r.m2z * az));
	return s;
}

// edge function p.x*q.y - p.y*q.x with one rounding per product and difference
__device__ __forceinline__ float edge(float px, float py, float qx, float qy) {
	return __fsub_rn(__fmul_rn(px, qy), __fmul_rn(py, qx));
}

// Watertight test; on hit in [tmin, tbest] (ties: lower tri id) returns t.
__device__ __forceinline__ bool tri_test(const RayState& r, float4 a, float4 b, float4 c, float tbest, uint32_t tri,
                                         uint32_t best_tri, float& t_out) {
	Shear A = shear(r, a), B = shear(r, b), C = shear(r, c);
	float U = edge(C.x, C.y, B.x, B.y);
	float V = edge(A.x, A.y, C.x, C.y);
	float W = edge(B.x, B.y, A.x, A.y);
	if (U == 0.f || V == 0.f || W == 0.f) {
		U = (float)((double)C.x * (double)B.y - (double)C.y * (double)B.x);
		V = (float)((double)A.x * (double)C.y - (double)A.y * (double)C.x);
		W = (float)((double)B.x * (double)A.y - (double)B.y * (double)A.x);
	}
	if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
	float det = U + V + W;
	if (det == 0.f) return false;
	float T = U * A.z + V * B.z + W * C.z;
	float t = T / det;
	if (!(t >= r.tmin && t <= tbest)) return false;
	if (t == tbest && tri >= best_tri) return false;
	t_out = t;
	return true;
}

// FASTEST output fields for one triangle (IntersectBspFast.cpp:130-252 and
// the plane distance of :344-347), one rounding per operation.
struct Fastest {
	float dist, u, v;
	float n[4];
	bool front;
};

__device__ __forceinline__ float sel3(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

__device__ inline Fastest fastest_fields(const RayState& r, float4 a, float4 b, float4 c) {
	Fastest f;
	float r0 = __fsub_rn(b.x, a.x), r1 = __fsub_rn(b.y, a.y), r2 = __fsub_rn(b.z, a.z);
	float l0 = __fsub_rn(c.x, a.x), l1 = __fsub_rn(c.y, a.y), l2 = __fsub_rn(c.z, a.z);
	float ir0 = __fdiv_rn(1.f, r0), ir1 = __fdiv_rn(1.f, r1), ir2 = __fdiv_rn(1.f, r2);
	float rxy = __fsub_rn(__fmul_rn(l1, r0), __fmul_rn(l0, r1));
	float ryz = __fsub_rn(__fmul_rn(l2, r1), __fmul_rn(l1, r2));
	float rzx = __fsub_rn(__fmul_rn(l0, r2), __fmul_rn(l2, r0));
	int ib;
	float ireal;
	if (fabsf(rxy) >= fabsf(ryz)) {
		if (fabsf(rxy) >= fabsf(rzx)) { ib = 0; ireal = __fdiv_rn(1.f, rxy); }
		else { ib = 2; ireal = __fdiv_rn(1.f, rzx); }
	} else {
		if (fabsf(ryz) >= fabsf(rzx)) { ib = 1; ireal = __fdiv_rn(1.f, ryz); }
		else { ib = 2; ireal = __fdiv_rn(1.f, rzx); }
	}
	if (fabsf(r0) >= fabsf(r1)) {
		if (fabsf(r0) >= fabsf(r2)) ib += 3;
	} else {
		if (fabsf(r1) >= fabsf(r2)) ib += 6;
	}
	float nx = __fsub_rn(__fmul_rn(r1, l2), __fmul_rn(r2, l1));
	float ny = __fadd_rn(__fmul_rn(-r0, l2), __fmul_rn(r2, l0));
	float nz = __fsub_rn(__fmul_rn(r0, l1), __fmul_rn(r1, l0));
	float sz = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)), __fmul_rn(nz, nz)));
	f.n[0] = __fdiv_rn(nx, sz);
	f.n[1] = __fdiv_rn(ny, sz);
	f.n[2] = __fdiv_rn(nz, sz);
	f.n[3] = -__fadd_rn(__fadd_rn(__fmul_rn(a.x, f.n[0]), __fmul_rn(a.y, f.n[1])), __fmul_rn(a.z, f.n[2]));
	float ndd = __fadd_rn(__fadd_rn(__fmul_rn(r.dx, f.n[0]), __fmul_rn(r.dy, f.n[1])), __fmul_rn(r.dz, f.n[2]));
	float ndo = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(r.ox, f.n[0]), __fmul_rn(r.oy, f.n[1])), __fmul_rn(r.oz, f.n[2])),
	                      f.n[3]);
	f.dist = __fdiv_rn(-ndo, ndd);
	float hx = __fadd_rn(r.ox, __fmul_rn(r.dx, f.dist));
	float hy = __fadd_rn(r.oy, __fmul_rn(r.dy, f.dist));
	float hz = __fadd_rn(r.oz, __fmul_rn(r.dz, f.dist));
	// projection case table of intersect_triangleSRLNP
	const int X = (ib % 3 == 0) ? 0 : (ib % 3 == 1 ? 1 : 2);
	const int Y = (ib % 3 == 0) ? 1 : (ib % 3 == 1 ? 2 : 0);
	const int Z = ib < 3 ? 2 : (ib < 6 ? 0 : 1);
	float hpY = sel3(hx, hy, hz, Y), hpX = sel3(hx, hy, hz, X), hpZ = sel3(hx, hy, hz, Z);
	float s3Y = sel3(a.x, a.y, a.z, Y), s3X = sel3(a.x, a.y, a.z, X), s3Z = sel3(a.x, a.y, a.z, Z);
	float r3X = sel3(r0, r1, r2, X), r3Y = sel3(r0, r1, r2, Y);
	float l3Z = sel3(l0, l1, l2, Z), ir3Z = sel3(ir0, ir1, ir2, Z);
	f.v = __fmul_rn(__fsub_rn(__fmul_rn(__fsub_rn(hpY, s3Y), r3X), __fmul_rn(__fsub_rn(hpX, s3X), r3Y)), ireal);
	f.u = __fmul_rn(__fsub_rn(__fsub_rn(hpZ, s3Z), __fmul_rn(l3Z, f.v)), ir3Z);
	f.front = ndd < 0.f;
	return f;
}

__device__ __forceinline__ void load_tri(const float4* __restrict__ tris, int slot, float4& a, float4& b, float4& c) {
	a = __ldg(tris + 3 * slot);
	b = __ldg(tris + 3 * slot + 1);
	c = __ldg(tris + 3 * slot + 2);
}

// Traverses one ray.  ANY: stop at the first accepted triangle.
// Returns best slot (>= 0) or -1; tbest updated; sets *err on stack overflow.
constexpr uint32_t kMaxSteps = 1u << 22;   // per-ray bound on visited nodes + leaves

// Acceptance filter of the final-gathering collision handler
// (RRStaticSolver/pathtracer.h:117-242) for opaque one-sided materials:
// never the shooter triangle, nor a triangle with the shooter's three
// vertices closer than ident_t (= 1000 * rayLengthMin); front sides only when
// front_only (hemisphere rays; shadow rays are stopped by either side).
struct GatherFilter {
	uint32_t skip;
	float ident_t;
	bool front_only;
	float4 s0, s1, s2;   // shooter vertices
};

__device__ __forceinline__ bool same_point(float4 p, float4 q) { return p.x == q.x && p.y == q.y && p.z == q.z; }
__device__ __forceinline__ bool in_set(float4 p, const GatherFilter& f) {
	return same_point(p, f.s0) || same_point(p, f.s1) || same_point(p, f.s2);
}

// front side: dot(dir, (b-a) x (c-a)) < 0, one rounding per operation
__device__ __forceinline__ bool front_facing(const RayState& r, float4 a, float4 b, float4 c) {
	float r0 = __fsub_rn(b.x, a.x), r1 = __fsub_rn(b.y, a.y), r2 = __fsub_rn(b.z, a.z);
	float l0 = __fsub_rn(c.x, a.x), l1 = __fsub_rn(c.y, a.y), l2 = __fsub_rn(c.z, a.z);
	float nx = __fsub_rn(__fmul_rn(r1, l2), __fmul_rn(r2, l1));
	float ny = __fadd_rn(__fmul_rn(-r0, l2), __fmul_rn(r2, l0));
	float nz = __fsub_rn(__fmul_rn(r0, l1), __fmul_rn(r1, l0));
	return __fadd_rn(__fadd_rn(__fmul_rn(r.dx, nx), __fmul_rn(r.dy, ny)), __fmul_rn(r.dz, nz)) < 0.f;
}

// KEYED: only hits after (key_t, key_tri) in the order (t, triangle index)
// count, for replaying a collision handler hit by hit.  The caller raises
// r.tmin to key_t, so boxes and triangles nearer than key_t are culled as
// usual; a triangle at exactly key_t is taken only above key_tri.
template <bool ANY, bool FILTER = false, bool KEYED = false>
__device__ int traverse(const TNode* __restrict__ nodes, const float4* __restrict__ tris, const RayState& r,
                        int nnodes, int ntris, float& tbest, uint32_t& best_tri, bool& overflow,
                        const GatherFilter* flt = nullptr, int root = 0, float key_t = 0.f,
                        uint32_t key_tri = 0) {
	int stack[kStackSize];
	int sp = 0;
	int ref = root;
	int best_slot = -1;
	for (uint32_t steps = 0;; steps++) {
		if (steps >= kMaxSteps) { overflow = true; break; }
		if (ref >= 0) {
			if (ref >= nnodes) { overflow = true; break; }
			const float4* np = reinterpret_cast<const float4*>(nodes + ref);
			float4 na = __ldg(np), nb = __ldg(np + 1), nc = __ldg(np + 2);
			int4 nd = __ldg(reinterpret_cast<const int4*>(np + 3));
			float t0 = nd.x != kEmptyRef ? box_enter(r, na.x, na.y, na.z, na.w, nc.x, nc.y, tbest) : INFINITY;
			float t1 = nd.y != kEmptyRef ? box_enter(r, nb.x, nb.y, nb.z, nb.w, nc.z, nc.w, tbest) : INFINITY;
			bool h0 = t0 != INFINITY, h1 = t1 != INFINITY;
			if (h0 && h1) {
				int nearr = t0 <= t1 ? nd.x : nd.y;
				int farr = t0 <= t1 ? nd.y : nd.x;
				if (sp < kStackSize) stack[sp++] = farr;
				else overflow = true;
				ref = nearr;
				continue;
			}
			if (h0) { ref = nd.x; continue; }
			if (h1) { ref = nd.y; continue; }
		} else {
			int first = ref & 0x07FFFFFF;
			int count = ((ref >> 27) & 15) + 1;
			if (first + count > ntris) { overflow = true; break; }
			for (int k = 0; k < count; k++) {
				float4 a, b, c;
				load_tri(tris, first + k, a, b, c);
				uint32_t tri = (uint32_t)__float_as_int(a.w);
				float t;
				if (tri_test(r, a, b, c, tbest, tri, best_tri, t)) {
					if (KEYED && t == key_t && tri <= key_tri) continue;
					if (FILTER) {
						if (tri == flt->skip) continue;
						if (t < flt->ident_t && in_set(a, *flt) && in_set(b, *flt) && in_set(c, *flt)) continue;
						if (flt->front_only && !front_facing(r, a, b, c)) continue;
					}
					tbest = t;
					best_tri = tri;
					best_slot = first + k;
					if (ANY) return best_slot;
				}
			}
		}
		if (sp == 0) break;
		ref = stack[--sp];
	}
	return best_slot;
}


// traverse() with a split stack: the top SDEPTH entries of the thread's
// stack in shared memory at sst[d * kTraceThreads] (sst = the block's stack
// array + threadIdx.x, so a warp's lanes touch 32 consecutive words), the
// deeper ones in a local array.  Same visits and results as traverse().
template <bool ANY, int SDEPTH>
__device__ __forceinline__ int traverse_split(const TNode* __restrict__ nodes, const float4* __restrict__ tris,
                                              const RayState& r, int nnodes, int ntris, float& tbest,
                                              uint32_t& best_tri, bool& overflow, int* sst, int root = 0) {
	int spill[kStackSize - SDEPTH];
	int sp = 0;
	int ref = root;
	int best_slot = -1;
	for (uint32_t steps = 0;; steps++) {
		if (steps >= kMaxSteps) { overflow = true; break; }
		if (ref >= 0) {
			if (ref >= nnodes) { overflow = true; break; }
			const float4* np = reinterpret_cast<const float4*>(nodes + ref);
			const float4 na = __ldg(np), nb = __ldg(np + 1), nc = __ldg(np + 2);
			const int4 nd = __ldg(reinterpret_cast<const int4*>(np + 3));
			const float t0 = nd.x != kEmptyRef ? box_enter(r, na.x, na.y, na.z, na.w, nc.x, nc.y, tbest) : INFINITY;
			const float t1 = nd.y != kEmptyRef ? box_enter(r, nb.x, nb.y, nb.z, nb.w, nc.z, nc.w, tbest) : INFINITY;
			const bool h0 = t0 != INFINITY, h1 = t1 != INFINITY;
			if (h0 && h1) {
				const int nearr = t0 <= t1 ? nd.x : nd.y;
				const int farr = t0 <= t1 ? nd.y : nd.x;
				if (sp < SDEPTH) sst[sp++ * kTraceThreads] = farr;
				else if (sp < kStackSize) { spill[sp - SDEPTH] = farr; sp++; }
				else overflow = true;
				ref = nearr;
				continue;
			}
			if (h0) { ref = nd.x; continue; }
			if (h1) { ref = nd.y; continue; }
		} else {
			const int first = ref & 0x07FFFFFF;
			const int count = ((ref >> 27) & 15) + 1;
			if (first + count > ntris) { overflow = true; break; }
			for (int k = 0; k < count; k++) {
				float4 a, b, c;
				load_tri(tris, first + k, a, b, c);
				const uint32_t tri = (uint32_t)__float_as_int(a.w);
				float t;
				if (tri_test(r, a, b, c, tbest, tri, best_tri, t)) {
					tbest = t;
					best_tri = tri;
					best_slot = first + k;
					if (ANY) return best_slot;
				}
			}
		}
		if (sp == 0) break;
		--sp;
		ref = sp < SDEPTH ? sst[sp * kTraceThreads] : spill[sp - SDEPTH];
	}
	return best_slot;
}

// ------------------------------------------------------------ 8-wide BVH
// Header of the node being walked: child/triangle bases and the slot codes.
struct WideHdr {
	uint32_t child_base, tri_base, meta_lo, meta_hi;
};

__device__ __forceinline__ uint32_t ray_octant(const RayState& r) {
	return (r.dx < 0.f ? 1u : 0u) | (r.dy < 0.f ? 2u : 0u) | (r.dz < 0.f ? 4u : 0u);
}

// Byte s of an 8-byte quantised bound as a float, without an integer to
// float conversion: one byte permute builds the bits of 2^23 + q, and
// subtracting 2^23 is exact.
__device__ __forceinline__ float qbyte(uint32_t lo4, uint32_t hi4, int s) {
	const uint32_t bits = __byte_perm(s < 4 ? lo4 : hi4, 0x4B000000u, (uint32_t)(s & 3) | 0x7540u);
	return __uint_as_float(bits) - 8388608.0f;
}

// Tests the ray against the eight child boxes of wide node `node`; returns
// the hit children as a mask in visiting order (bit i = slot i ^ oct) and
// the node header.  Each quantised bound is p + q 2^e, so its ray distance
// is fma(q, 2^e / d, (p - o) / d): one FMA per bound after per-node set-up.
__device__ __forceinline__ uint32_t wide_visit(const uint4* __restrict__ wn, uint32_t node, const RayState& r,
                                               uint32_t oct, float tbest, WideHdr& h) {
	const uint4* np = wn + 5 * (size_t)node;
	const uint4 w0 = __ldg(np), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3), w4 = __ldg(np + 4);
	h.child_base = w1.x;
	h.tri_base = w1.y;
	h.meta_lo = w1.z;
	h.meta_hi = w1.w;
	const uint32_t ev = w0.w;
	const float sx = __uint_as_float((ev & 0xFFu) << 23);
	const float sy = __uint_as_float(((ev >> 8) & 0xFFu) << 23);
	const float sz = __uint_as_float(((ev >> 16) & 0xFFu) << 23);
	const uint32_t valid = ev >> 24;
	const float ax = sx * r.ix, ay = sy * r.iy, az = sz * r.iz;
	const float bx = fmaf(__uint_as_float(w0.x), r.ix, -r.oix);
	const float by = fmaf(__uint_as_float(w0.y), r.iy, -r.oiy);
	const float bz = fmaf(__uint_as_float(w0.z), r.iz, -r.oiz);
	uint32_t mask = 0;
#pragma unroll
	for (int s = 0; s < 8; s++) {
		const float tx0 = fmaf(qbyte(w2.x, w2.y, s), ax, bx), tx1 = fmaf(qbyte(w3.z, w3.w, s), ax, bx);
		const float ty0 = fmaf(qbyte(w2.z, w2.w, s), ay, by), ty1 = fmaf(qbyte(w4.x, w4.y, s), ay, by);
		const float tz0 = fmaf(qbyte(w3.x, w3.y, s), az, bz), tz1 = fmaf(qbyte(w4.z, w4.w, s), az, bz);
		const float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), r.tmin));
		const float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tbest));
		const bool hit = ((valid >> s) & 1u) && tn <= tf * 1.0000004f;
		mask |= (hit ? 1u : 0u) << (s ^ oct);
	}
	return mask;
}

// Closest (ANY = any) hit over the 8-wide tree from root node `root`.  The
// current node's remaining hit children are a mask; when an inner child is
// entered, the rest of the mask is pushed as one 32-bit entry (24-bit node
// index, 8-bit mask), so the stack holds at most one entry per level.
template <bool ANY>
__device__ int traverse_wide(const uint4* __restrict__ wn, const float4* __restrict__ tris, const RayState& r,
                             int nwnodes, int ntris, float& tbest, uint32_t& best_tri, bool& overflow, int root = 0) {
	uint32_t stack[kStackSize];
	int sp = 0;
	int best_slot = -1;
	const uint32_t oct = ray_octant(r);
	if (root < 0 || root >= nwnodes) { overflow = true; return -1; }
	uint32_t node = (uint32_t)root;
	WideHdr h;
	uint32_t mask = wide_visit(wn, node, r, oct, tbest, h);
	for (uint32_t steps = 0;; steps++) {
		if (steps >= kMaxSteps) { overflow = true; break; }
		if (mask) {
			const uint32_t i = __ffs(mask) - 1;
			mask &= mask - 1;
			const uint32_t slot = i ^ oct;
			const uint32_t m = ((slot < 4 ? h.meta_lo : h.meta_hi) >> (8 * (slot & 3))) & 0xFFu;
			if (m & 0x80u) {
				const uint32_t child = h.child_base + (m & 7u);
				if (child >= (uint32_t)nwnodes) { overflow = true; break; }
				if (mask) {
					if (sp < kStackSize) stack[sp++] = node | (mask << 24);
					else { overflow = true; break; }
				}
				node = child;
				mask = wide_visit(wn, node, r, oct, tbest, h);
			} else {
				const int first = (int)(h.tri_base + (m & 31u));
				const int count = (int)(m >> 5) + 1;
				if (first + count > ntris) { overflow = true; break; }
				for (int k = 0; k < count; k++) {
					float4 a, b, c;
					load_tri(tris, first + k, a, b, c);
					const uint32_t tri = (uint32_t)__float_as_int(a.w);
					float t;
					if (tri_test(r, a, b, c, tbest, tri, best_tri, t)) {
						tbest = t;
						best_tri = tri;
						best_slot = first + k;
						if (ANY) return best_slot;
					}
				}
			}
			continue;
		}
		if (sp == 0) break;
		const uint32_t e = stack[--sp];
		node = e & 0xFFFFFFu;
		mask = e >> 24;
		const uint4 w1 = __ldg(wn + 5 * (size_t)node + 1);
		h.child_base = w1.x;
		h.tri_base = w1.y;
		h.meta_lo = w1.z;
		h.meta_hi = w1.w;
	}
	return best_slot;
}

}  // namespace rrg
