// Lightmap final gather on the GPU: texel enumeration and the plain N-bounce
// gather, behind the C ABI of include/rrgpu_gather.h.
//
// Reference path: RRSolver::updateLightmaps -> updateLightmap ->
// enumerateTexelsFull/Partial -> processTexel (RRSolver/lightmap.cpp:83-454,
// 648-930; RRSolver/gather.cpp:600-836) with
// PathtracerWorker::getIncidentRadiance (RRStaticSolver/pathtracer.cpp:139-394).
//
// 1. enumeration: one warp per triangle; lanes walk the texels of the
//    triangle's lightmap bounding box, clip each texel square by the
//    triangle's three edges in triangle space and fan the polygon into
//    sub-texels (lightmap.cpp:145-330), first counting per texel, then (after
//    a device-wide scan) writing; each texel's list is then sorted by
//    (triangle, fan index), the order in which the reference appends them.
// 2. gather: one warp per texel.  The 64 hemisphere samples of a texel are
//    the 32 lanes x 2; each lane selects its sub-texel by the reference's
//    area stepping, takes its point and its HomogenousFiller2 direction (the
//    filler's accepted points are found cooperatively with a ballot), and
//    traces an N-bounce path with next-event shadow rays.  Light rounds
//    (quality/10+1, interleaved as gather.cpp:773-785) add direct light.
//    Lane 0 sums the samples in the reference's order.
// Every floating-point step mirrors the C oracle (oracle/rr_gather.c) with
// one rounding per operation (__f*_rn), so both produce the same values from
// the same counter-based sample streams.
#include "rrg_traverse.cuh"

#include <stddef.h>
#include "../../include/rrgpu_gather.h"
#include "../../include/rrgpu_cache.h"
#include "rrg_mlp.cuh"

#include <algorithm>
#include <type_traits>
#include <vector>

namespace rrg {

// ------------------------------------------------------------------ RNG
__device__ __forceinline__ uint64_t fmix64(uint64_t k) {
	k ^= k >> 33;
	k *= 0xFF51AFD7ED558CCDULL;
	k ^= k >> 33;
	k *= 0xC4CEB9FE1A85EC53ULL;
	k ^= k >> 33;
	return k;
}
__device__ __forceinline__ uint64_t hash64(uint64_t seed, uint64_t stream, uint64_t index) {
	uint64_t key = seed * 0x9E3779B97F4A7C15ULL + stream * 0xD1B54A32D192ED03ULL;
	return fmix64(fmix64(index ^ key) + 0x632BE59BD9B4E019ULL);
}
__device__ __forceinline__ uint32_t rng24(uint64_t seed, uint64_t stream, uint64_t index) {
	return (uint32_t)(hash64(seed, stream, index) >> 40);
}
__device__ __forceinline__ float rng01(uint64_t seed, uint64_t stream, uint64_t index) {
	return __fmul_rn((float)rng24(seed, stream, index), 1.0f / 16777216.0f);
}

enum { S_FILLER = 60, S_PU = 61, S_PV = 62, S_ROULETTE = 63, S_DISKX = 64, S_DISKY = 65 };
constexpr uint32_t kM24 = 16777215u;
constexpr int kDiskTries = 32;
// Bounce b of sample sid draws its numbers at counter sid * 256 + b, so a
// path has 256 bounces of its own; deeper limits act as 255.
constexpr uint32_t kMaxDepth = 255;
constexpr float kPreventInf = 0.000000000137289f;   // RRLight.cpp:21
constexpr float kStopAtVisibility = 0.001f;         // PathTracingParameters default

// -------------------------------------------------------------- vectors
struct V3 {
	float x, y, z;
};
__host__ __device__ __forceinline__ V3 mk(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return mk(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)); }
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return mk(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)); }
__device__ __forceinline__ V3 mul(V3 a, float f) { return mk(__fmul_rn(a.x, f), __fmul_rn(a.y, f), __fmul_rn(a.z, f)); }
__device__ __forceinline__ V3 mulv(V3 a, V3 b) { return mk(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z)); }
__device__ __forceinline__ V3 divf(V3 a, float f) { return mk(__fdiv_rn(a.x, f), __fdiv_rn(a.y, f), __fdiv_rn(a.z, f)); }
__device__ __forceinline__ V3 neg(V3 a) { return mk(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float dot(V3 a, V3 b) {
	return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ float len(V3 a) { return __fsqrt_rn(dot(a, a)); }
__device__ __forceinline__ V3 normalized(V3 a) { return divf(a, len(a)); }
__device__ __forceinline__ float avg3(V3 a) { return __fmul_rn(__fadd_rn(__fadd_rn(a.x, a.y), a.z), 0.33333333333333f); }
__device__ __forceinline__ V3 ortho1(V3 a) { return fabsf(a.x) > fabsf(a.z) ? mk(-a.y, a.x, 0.f) : mk(0.f, -a.z, a.y); }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
	return mk(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)), __fadd_rn(__fmul_rn(-a.x, b.z), __fmul_rn(a.z, b.x)),
	          __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ float clampf(float a, float lo, float hi) { return a < lo ? lo : (a > hi ? hi : a); }

// ---------------------------------------------------------- enumeration
struct Sub {            // one sub-texel, 32 bytes (matches orc_subtexel)
	uint32_t tri;
	float uv[6];
	float area;
};

struct V2 {
	float x, y;
};

__device__ __forceinline__ float get_area(V2 v0, V2 v1, V2 v2) {
	auto l = [](V2 p, V2 q) {
		float dx = __fsub_rn(q.x, p.x), dy = __fsub_rn(q.y, p.y);
		return __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
	};
	float a = l(v0, v1), b = l(v1, v2), c = l(v2, v0);
	float s = __fmul_rn(__fadd_rn(__fadd_rn(a, b), c), 0.5f);
	return __fsqrt_rn(__fmul_rn(__fmul_rn(__fmul_rn(s, __fsub_rn(s, a)), __fsub_rn(s, b)), __fsub_rn(s, c)));
}

struct Raster {
	unsigned x0, x1, y0, y1;   // texel bbox [x0,x1) x [y0,y1)
	float m[2][3];             // triangle space -> map space
	float inv[2][3];
	float tri_area;
	bool ok;
};

// bounding box and map -> triangle space matrix (lightmap.cpp:155-205)
__device__ Raster raster_setup(const float* uvm, unsigned size) {
	Raster R;
	R.ok = false;
	const float W = (float)size, H = (float)size;
	V2 u0{uvm[0], uvm[1]}, u1{uvm[2], uvm[3]}, u2{uvm[4], uvm[5]};
	float xmin = __fmul_rn(W, fminf(u0.x, fminf(u1.x, u2.x)));
	float xmax = __fmul_rn(W, fmaxf(u0.x, fmaxf(u1.x, u2.x)));
	float ymin = __fmul_rn(H, fminf(u0.y, fminf(u1.y, u2.y)));
	float ymax = __fmul_rn(H, fmaxf(u0.y, fmaxf(u1.y, u2.y)));
	R.x0 = (unsigned)(xmin > 0.f ? xmin : 0.f);
	R.x1 = (unsigned)clampf(__fadd_rn(xmax, 1.f), 0.f, W);
	R.y0 = (unsigned)(ymin > 0.f ? ymin : 0.f);
	R.y1 = (unsigned)clampf(__fadd_rn(ymax, 1.f), 0.f, H);
	if (R.y0 >= R.y1 || R.x0 >= R.x1) return R;
	float m00 = __fsub_rn(u1.x, u0.x), m01 = __fsub_rn(u2.x, u0.x), m02 = u0.x;
	float m10 = __fsub_rn(u1.y, u0.y), m11 = __fsub_rn(u2.y, u0.y), m12 = u0.y;
	const float m20 = 0.f, m21 = 0.f, m22 = 1.f;
	float det = __fsub_rn(
	    __fsub_rn(__fsub_rn(__fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(m00, m11), m22), __fmul_rn(__fmul_rn(m01, m12), m20)),
	                                  __fmul_rn(__fmul_rn(m02, m10), m21)),
	                        __fmul_rn(__fmul_rn(m00, m12), m21)),
	              __fmul_rn(__fmul_rn(m01, m10), m22)),
	    __fmul_rn(__fmul_rn(m02, m11), m20));
	if (!(det != 0.f)) return R;
	float invdet = __fdiv_rn(1.f, det);
	R.inv[0][0] = __fdiv_rn(__fmul_rn(__fsub_rn(__fmul_rn(m11, m22), __fmul_rn(m12, m21)), invdet), W);
	R.inv[0][1] = __fdiv_rn(__fmul_rn(__fsub_rn(__fmul_rn(m02, m21), __fmul_rn(m01, m22)), invdet), H);
	R.inv[0][2] = __fmul_rn(__fsub_rn(__fmul_rn(m01, m12), __fmul_rn(m02, m11)), invdet);
	R.inv[1][0] = __fdiv_rn(__fmul_rn(__fsub_rn(__fmul_rn(m12, m20), __fmul_rn(m10, m22)), invdet), W);
	R.inv[1][1] = __fdiv_rn(__fmul_rn(__fsub_rn(__fmul_rn(m00, m22), __fmul_rn(m02, m20)), invdet), H);
	R.inv[1][2] = __fmul_rn(__fsub_rn(__fmul_rn(m02, m10), __fmul_rn(m00, m12)), invdet);
	R.m[0][0] = m00; R.m[0][1] = m01; R.m[0][2] = m02;
	R.m[1][0] = m10; R.m[1][1] = m11; R.m[1][2] = m12;
	R.tri_area = get_area(u0, u1, u2);
	R.ok = true;
	return R;
}

// clips texel (x, y) by the triangle; returns the polygon size (0..7)
__device__ int clip_texel(const Raster& R, unsigned x, unsigned y, V2* poly) {
	auto m2t = [&](unsigned X, unsigned Y) {
		float fx = (float)X, fy = (float)Y;
		return V2{__fadd_rn(__fadd_rn(__fmul_rn(fx, R.inv[0][0]), __fmul_rn(fy, R.inv[0][1])), R.inv[0][2]),
		          __fadd_rn(__fadd_rn(__fmul_rn(fx, R.inv[1][0]), __fmul_rn(fy, R.inv[1][1])), R.inv[1][2])};
	};
	unsigned n = 4;
	poly[0] = m2t(x, y);
	poly[1] = m2t(x + 1, y);
	poly[2] = m2t(x + 1, y + 1);
	poly[3] = m2t(x, y + 1);
	for (int side = 0; side < 3; side++) {
		float L0 = side == 0 ? 0.f : (side == 1 ? -1.f : 1.f);
		float L1 = side == 0 ? 1.f : (side == 1 ? -1.f : 0.f);
		float L2 = side == 0 ? 0.f : (side == 1 ? 1.f : 0.f);
		int inside[7];
		unsigned nin = 0, nout = 0;
		for (unsigned i = 0; i < n; i++) {
			float dd = __fadd_rn(__fadd_rn(__fmul_rn(L0, poly[i].x), __fmul_rn(L1, poly[i].y)), L2);
			if (dd < 0.f) { inside[i] = 2; nout++; }
			else if (dd > 0.f) { inside[i] = 0; nin++; }
			else inside[i] = 1;
		}
		if (!nout) continue;
		if (!nin) return 0;
		unsigned fp = 1;
		while (inside[(fp - 1) % n] == 0 || inside[fp % n] != 0) fp++;
		V2 orig[7];
		for (int i = 0; i < 7; i++) orig[i] = poly[i];
		unsigned src = fp, dst = 0;
		while (inside[src % n] == 0 && dst < 7) poly[dst++] = orig[src++ % n];
		auto isect = [&](V2 A, V2 B) {
			float dA = __fadd_rn(__fadd_rn(__fmul_rn(L0, A.x), __fmul_rn(L1, A.y)), L2);
			float den = __fadd_rn(__fmul_rn(L0, __fsub_rn(B.x, A.x)), __fmul_rn(L1, __fsub_rn(B.y, A.y)));
			return V2{__fsub_rn(A.x, __fdiv_rn(__fmul_rn(__fsub_rn(B.x, A.x), dA), den)),
			          __fsub_rn(A.y, __fdiv_rn(__fmul_rn(__fsub_rn(B.y, A.y), dA), den))};
		};
		if (dst + 2 > 7) return 0;   // cannot happen for a convex quad cut three times
		poly[dst++] = isect(orig[(src - 1) % n], orig[src % n]);
		poly[dst++] = isect(orig[(fp - 1) % n], orig[fp % n]);
		n = dst;
	}
	return (int)n;
}

// TexelFlags (RRSolver/gather.h:68-80) of one clipped polygon, set as in
// lightmap.cpp:283-314: its vertices in texel space (texel centre at 0,
// spanning -0.5..0.5) mark the texel edges they reach (within 0.03 texel)
// and the quadrants they fall in; an edge that crosses both axes also marks
// the quadrants it passes without a vertex.
constexpr unsigned kQ00 = 1, kQ10 = 2, kQ01 = 4, kQ11 = 8, kEX0 = 16, kEX1 = 32, kEY0 = 64, kEY1 = 128;

__device__ unsigned polygon_flags(const Raster& R, const V2* poly, int n, unsigned x, unsigned y, float W, float H) {
	const float lo = __fadd_rn(-0.5f, 0.03f), hi = __fsub_rn(0.5f, 0.03f);
	unsigned f = 0;
	V2 old{0.f, 0.f};
	for (int k = 0; k <= n; k++) {
		const V2 p = poly[(k + n - 1) % n];   // k = 0: the last vertex, "old" of vertex 0
		const float mx = __fadd_rn(__fadd_rn(__fmul_rn(p.x, R.m[0][0]), __fmul_rn(p.y, R.m[0][1])), R.m[0][2]);
		const float my = __fadd_rn(__fadd_rn(__fmul_rn(p.x, R.m[1][0]), __fmul_rn(p.y, R.m[1][1])), R.m[1][2]);
		const V2 t{__fsub_rn(__fsub_rn(__fmul_rn(mx, W), (float)x), 0.5f),
		           __fsub_rn(__fsub_rn(__fmul_rn(my, H), (float)y), 0.5f)};
		if (k) {
			if (t.x < lo) f |= kEX0;
			if (t.x > hi) f |= kEX1;
			if (t.y < lo) f |= kEY0;
			if (t.y > hi) f |= kEY1;
			if (t.x < 0.f && t.y < 0.f) f |= kQ00;
			if (t.x > 0.f && t.y < 0.f) f |= kQ10;
			if (t.x < 0.f && t.y > 0.f) f |= kQ01;
			if (t.x > 0.f && t.y > 0.f) f |= kQ11;
			if ((old.x < 0.f) != (t.x < 0.f) && (old.y < 0.f) != (t.y < 0.f)) {
				const float a = __fdiv_rn(__fsub_rn(t.y, old.y), __fsub_rn(t.x, old.x));
				const float b = __fsub_rn(t.y, __fmul_rn(a, t.x));
				f |= (b < 0.f) ? (kQ00 | kQ10) : (kQ01 | kQ11);
				f |= (__fdiv_rn(-b, a) < 0.f) ? (kQ00 | kQ01) : (kQ10 | kQ11);
			}
		}
		old = t;
	}
	return f;
}

// One warp per triangle.  COUNT: counts[texel] += sub-texels and the texel's
// flags (4 per word) |= the polygon's.  Otherwise
// writes them at off[texel] + cursor, with the fan index in .tri's top bits
// replaced later by the sort.
template <bool COUNT>
__global__ void k_enumerate(const float* __restrict__ uv, const int32_t* __restrict__ tri_atlas, uint32_t nt,
                            uint32_t size, uint32_t natlas, uint32_t* __restrict__ counts,
                            const uint32_t* __restrict__ off, uint32_t* __restrict__ cursor, Sub* __restrict__ out,
                            uint32_t* __restrict__ fan_out, uint64_t cap, uint32_t* err,
                            uint32_t* __restrict__ flags) {
	const int lane = threadIdx.x & 31;
	const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
	for (uint32_t t = warp; t < nt; t += nwarps) {
		int a = tri_atlas[t];
		if (a < 0 || (uint32_t)a >= natlas) continue;
		Raster R = raster_setup(uv + 6 * (size_t)t, size);
		if (!R.ok) continue;
		const uint32_t bw = R.x1 - R.x0, bh = R.y1 - R.y0;
		const uint64_t nb = (uint64_t)bw * bh;
		const uint64_t abase = (uint64_t)a * size * size;
		for (uint64_t j = lane; j < nb; j += 32) {
			unsigned x = R.x0 + (unsigned)(j % bw), y = R.y0 + (unsigned)(j / bw);
			V2 poly[7];
			int n = clip_texel(R, x, y, poly);
			if (n < 3) continue;
			uint64_t texel = abase + (uint64_t)y * size + x;
			if (COUNT && flags) {
				const unsigned f = polygon_flags(R, poly, n, x, y, (float)size, (float)size);
				if (f) atomicOr(&flags[texel >> 2], f << (8 * (unsigned)(texel & 3)));
			}
			float areas[5];
			int valid = 0;
			for (int i = 0; i + 2 < n; i++) {
				float ar = __fmul_rn(get_area(poly[0], poly[i + 1], poly[i + 2]), R.tri_area);
				areas[i] = ar;
				if (isfinite(ar)) valid++;
			}
			if (!valid) continue;
			if (COUNT) {
				atomicAdd(&counts[texel], (uint32_t)valid);
			} else {
				uint32_t base = off[texel] + atomicAdd(&cursor[texel], (uint32_t)valid);
				int w = 0;
				for (int i = 0; i + 2 < n; i++) {
					if (!isfinite(areas[i])) continue;
					uint64_t pos = (uint64_t)base + w;
					if (pos >= cap) { atomicOr(err, 1u); break; }
					Sub s;
					s.tri = t;
					s.uv[0] = poly[0].x; s.uv[1] = poly[0].y;
					s.uv[2] = poly[i + 1].x; s.uv[3] = poly[i + 1].y;
					s.uv[4] = poly[i + 2].x; s.uv[5] = poly[i + 2].y;
					s.area = areas[i];
					out[pos] = s;
					fan_out[pos] = (uint32_t)i;
					w++;
				}
			}
		}
	}
}

// per texel: insertion sort of its sub-texels by (triangle, fan)
__global__ void k_sort_texels(const uint32_t* __restrict__ off, uint64_t ntexels, Sub* __restrict__ st,
                              uint32_t* __restrict__ fan) {
	for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < ntexels; t += (uint64_t)gridDim.x * blockDim.x) {
		uint32_t b = off[t], e = off[t + 1];
		for (uint32_t i = b + 1; i < e; i++) {
			Sub s = st[i];
			uint32_t f = fan[i];
			uint64_t key = ((uint64_t)s.tri << 8) | f;
			uint32_t j = i;
			while (j > b && ((((uint64_t)st[j - 1].tri) << 8) | fan[j - 1]) > key) {
				st[j] = st[j - 1];
				fan[j] = fan[j - 1];
				j--;
			}
			st[j] = s;
			fan[j] = f;
		}
	}
}

// exclusive scan of n uint32 (total < 2^32) -> off[0..n]
constexpr int kScanBT = 256, kScanPer = 4096;
__global__ void k_scan_sums(const uint32_t* __restrict__ in, uint64_t n, uint32_t* __restrict__ bsum) {
	__shared__ uint32_t ws[kScanBT / 32];
	uint64_t base = (uint64_t)blockIdx.x * kScanPer;
	uint32_t s = 0;
	for (int k = threadIdx.x; k < kScanPer; k += kScanBT)
		if (base + k < n) s += in[base + k];
	for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
	if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
	__syncthreads();
	if (threadIdx.x == 0) {
		uint32_t t = 0;
		for (int w = 0; w < kScanBT / 32; w++) t += ws[w];
		bsum[blockIdx.x] = t;
	}
}
__global__ void k_scan_top(uint32_t* __restrict__ bsum, uint32_t nb) {
	if (threadIdx.x) return;
	uint32_t s = 0;
	for (uint32_t i = 0; i < nb; i++) {
		uint32_t v = bsum[i];
		bsum[i] = s;
		s += v;
	}
	bsum[nb] = s;
}
__global__ void k_scan_apply(const uint32_t* __restrict__ in, uint64_t n, const uint32_t* __restrict__ bsum,
                             uint32_t* __restrict__ out) {
	__shared__ uint32_t ws[kScanBT / 32];
	__shared__ uint32_t carry;
	uint64_t base = (uint64_t)blockIdx.x * kScanPer;
	if (threadIdx.x == 0) carry = bsum[blockIdx.x];
	__syncthreads();
	const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
	for (int k0 = 0; k0 < kScanPer; k0 += kScanBT) {
		uint64_t i = base + k0 + threadIdx.x;
		uint32_t v = i < n ? in[i] : 0;
		uint32_t x = v;
		for (int o = 1; o < 32; o <<= 1) {
			uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
			if (lane >= o) x += y;
		}
		if (lane == 31) ws[w] = x;
		__syncthreads();
		uint32_t wo = 0, tot = 0;
		for (int q = 0; q < kScanBT / 32; q++) {
			if (q < w) wo += ws[q];
			tot += ws[q];
		}
		if (i < n) out[i] = carry + wo + x - v;
		__syncthreads();
		if (threadIdx.x == 0) carry += tot;
		__syncthreads();
	}
	if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = bsum[gridDim.x];
}

__global__ void k_covered_flags(const uint32_t* __restrict__ off, uint64_t n, uint32_t* __restrict__ flag) {
	for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x)
		flag[t] = off[t + 1] > off[t] ? 1u : 0u;
}
__global__ void k_covered_scatter(const uint32_t* __restrict__ flag, const uint32_t* __restrict__ pos, uint64_t n,
                                  uint32_t* __restrict__ list) {
	for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x)
		if (flag[t]) list[pos[t]] = (uint32_t)t;
}

// ---------------------------------------------------------------- gather
struct GatherScene {
	const TNode* nodes;
	const float4* tris;
	int nnodes, ntris;
	const float* xyz;
	const uint32_t* idx;
	const float* albedo;
	V3 dir_direction, dir_color, point_position, point_color;
	float tmin, locality;
	uint32_t quality, max_depth;
	uint64_t seed;
	float ao_intensity, ao_size;   // both > 0: ambient occlusion on the hemisphere part
	const uint8_t* flags;          // TexelFlags per texel
	float ldir[4][3];              // LS_LIGHTMAP, LS_DIRECTION1..3 in tangent space (gather.cpp:43-49)
	// the bake's radiosity solver, read at the first hit when set: per
	// triangle its direct irradiance (3 floats) and the smoothed indirect
	// irradiance at its corners (9 floats)
	const float* solver_direct;
	const float* solver_corner;
};

// Outputs of the directional mode (LS_DIRECTION1..3, each may be null).
struct DirOut {
	float4* d[3];
};

// Alpha of a gathered texel: its TexelFlags / 255 (TEXELFLAGS_TO_FLOAT,
// gather.cpp:801,814), which the lightmap filters read back.
__device__ __forceinline__ float texel_alpha(const GatherScene& g, uint64_t tid) {
	return __fdiv_rn((float)g.flags[tid], 255.f);
}

__device__ __forceinline__ V3 ld3(const float* p) { return mk(p[0], p[1], p[2]); }

__device__ V3 tri_normal(const GatherScene& g, uint32_t t, V3& v0, V3& s1, V3& s2) {
	v0 = ld3(g.xyz + 3 * (size_t)g.idx[3 * t]);
	s1 = sub(ld3(g.xyz + 3 * (size_t)g.idx[3 * t + 1]), v0);
	s2 = sub(ld3(g.xyz + 3 * (size_t)g.idx[3 * t + 2]), v0);
	V3 n = cross(s1, s2);
	float l = len(n);
	return l != 0.f ? divf(n, l) : mk(1.f, 0.f, 0.f);
}

__device__ __forceinline__ V3 point_irr(const GatherScene& g, V3 p) {
	V3 d = sub(p, g.point_position);
	float att = __fdiv_rn(1.f, __fadd_rn(kPreventInf, dot(d, d)));
	return mul(g.point_color, att);
}

__device__ __forceinline__ void basis_from_normal(V3 n, V3& t, V3& b) {
	t = normalized(ortho1(n));
	b = cross(n, t);
}

__device__ __forceinline__ void set_ray(RayState& r, V3 o, V3 d, float tmin, float tmax) {
	r.ox = o.x; r.oy = o.y; r.oz = o.z; r.tmin = tmin;
	r.dx = d.x; r.dy = d.y; r.dz = d.z; r.tmax = tmax;
	ray_setup(r);
}

__device__ GatherFilter make_filter(const GatherScene& g, uint32_t skip, bool front_only) {
	GatherFilter f;
	f.skip = skip;
	f.ident_t = __fmul_rn(1000.f, g.tmin);
	f.front_only = front_only;
	const float* a = g.xyz + 3 * (size_t)g.idx[3 * skip];
	const float* b = g.xyz + 3 * (size_t)g.idx[3 * skip + 1];
	const float* c = g.xyz + 3 * (size_t)g.idx[3 * skip + 2];
	f.s0 = make_float4(a[0], a[1], a[2], 0.f);
	f.s1 = make_float4(b[0], b[1], b[2], 0.f);
	f.s2 = make_float4(c[0], c[1], c[2], 0.f);
	return f;
}

// shadow ray: any accepted hit blocks
__device__ bool occluded(const GatherScene& g, V3 o, V3 d, float tmin, float tmax, uint32_t skip, bool& overflow) {
	RayState r;
	set_ray(r, o, d, tmin, tmax);
	GatherFilter f = make_filter(g, skip, false);
	float tb = r.tmax;
	uint32_t bt = 0xFFFFFFFFu;
	return traverse<true, true>(g.nodes, g.tris, r, g.nnodes, g.ntris, tb, bt, overflow, &f) >= 0;
}

// Per-vertex record of a path, for training the radiance cache.
constexpr int kMaxVerts = 17;
struct PathLog {
	int n;
	V3 p[kMaxVerts], nrm[kMaxVerts], alb[kMaxVerts], nee[kMaxVerts], rs[kMaxVerts];
	bool cont[kMaxVerts];
};

// one hemisphere sample: getIncidentRadiance restated iteratively
template <bool LOG = false>
__device__ V3 trace_path(const GatherScene& g, V3 eye, V3 dir, uint32_t skip, uint64_t sid, bool& overflow,
                         PathLog* log = nullptr, float* first_t = nullptr) {
	V3 T = mk(1.f, 1.f, 1.f), L = mk(0.f, 0.f, 0.f);
	if (LOG) log->n = 0;
	float tmax = g.locality;
	if (!LOG && g.solver_direct) {
		// the solver read at the first hit: the triangle's direct irradiance
		// and its corners' smoothed indirect, interpolated, times the albedo;
		// the diffuse path ends there (pathtracer.cpp:235-258, 326-350;
		// Triangle::getPointMeasure, rrcore.cpp:262-277)
		RayState r;
		set_ray(r, eye, dir, g.tmin, tmax);
		GatherFilter f = make_filter(g, skip, true);
		float tb = r.tmax;
		uint32_t tri = 0xFFFFFFFFu;
		int slot = traverse<false, true>(g.nodes, g.tris, r, g.nnodes, g.ntris, tb, tri, overflow, &f);
		if (slot >= 0) {
			float4 a, b, c;
			load_tri(g.tris, slot, a, b, c);
			Fastest fs = fastest_fields(r, a, b, c);
			if (first_t) *first_t = fs.dist;
			const float* c9 = g.solver_corner + 9 * (size_t)tri;
			float w = __fsub_rn(__fsub_rn(1.f, fs.u), fs.v);
			V3 ind = add(add(mul(ld3(c9), w), mul(ld3(c9 + 3), fs.u)), mul(ld3(c9 + 6), fs.v));
			V3 alb = ld3(g.albedo + 3 * (size_t)tri);
			L = add(mulv(ld3(g.solver_direct + 3 * (size_t)tri), alb), mulv(ind, alb));
		}
		return L;
	}
	for (uint32_t depth = 0;; depth++) {
		RayState r;
		set_ray(r, eye, dir, g.tmin, tmax);
		GatherFilter f = make_filter(g, skip, true);
		float tb = r.tmax;
		uint32_t tri = 0xFFFFFFFFu;
		int slot = traverse<false, true>(g.nodes, g.tris, r, g.nnodes, g.ntris, tb, tri, overflow, &f);
		if (slot < 0) break;
		float4 a, b, c;
		load_tri(g.tris, slot, a, b, c);
		Fastest fs = fastest_fields(r, a, b, c);
		if (depth == 0 && first_t) *first_t = fs.dist;   // the first hit's distance, for ambient occlusion
		V3 p = add(eye, mul(dir, fs.dist));
		V3 n = mk(fs.n[0], fs.n[1], fs.n[2]);
		V3 alb = ld3(g.albedo + 3 * (size_t)tri);
		V3 nee = mk(0.f, 0.f, 0.f);
		for (int li = 0; li < 2; li++) {
			V3 sdir;
			float smax;
			if (li == 0) {
				sdir = neg(g.dir_direction);
				smax = 1e10f;
			} else {
				V3 d = sub(g.point_position, p);
				sdir = normalized(d);
				smax = len(d);
			}
			if (!(dot(n, sdir) > 0.f)) continue;
			V3 unob = li == 0 ? g.dir_color : point_irr(g, p);
			float dif = clampf(-dot(neg(sdir), n), 0.f, 1.f);
			V3 contrib = mulv(unob, mul(alb, dif));
			if (contrib.x == 0.f && contrib.y == 0.f && contrib.z == 0.f) continue;
			if (occluded(g, p, sdir, g.tmin, smax, tri, overflow)) continue;
			L = add(L, mulv(T, contrib));
			if (LOG) nee = add(nee, contrib);
		}
		const int vi = LOG ? log->n : 0;
		if (LOG && vi < kMaxVerts) {
			log->p[vi] = p; log->nrm[vi] = n; log->alb[vi] = alb; log->nee[vi] = nee; log->cont[vi] = false;
			log->n = vi + 1;
		}
		tmax = 1e10f;
		float pdiff = avg3(alb);
		if (pdiff < 0.f) pdiff = 0.f;
		float pstop = __fsub_rn(1.f, pdiff);
		if (pstop < 0.f) pstop = 0.f;
		float rr = rng01(g.seed, S_ROULETTE, sid * (kMaxDepth + 1) + depth);
		if (!(rr < pdiff && depth < g.max_depth)) break;
		float intensity = __fdiv_rn(__fadd_rn(pdiff, pstop), pdiff);
		float x = 0.f, y = 0.f;
		for (int j = 0; j < kDiskTries; j++) {
			uint64_t cc = (sid * (kMaxDepth + 1) + depth) * kDiskTries + j;
			float ax = __fsub_rn(__fmul_rn(rng01(g.seed, S_DISKX, cc), 2.0f), 1.0f);
			float by = __fsub_rn(__fmul_rn(rng01(g.seed, S_DISKY, cc), 2.0f), 1.0f);
			if (__fadd_rn(__fmul_rn(ax, ax), __fmul_rn(by, by)) < 1.0f) { x = ax; y = by; break; }
		}
		float cosT = __fsqrt_rn(__fsub_rn(1.0f, __fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y))));
		V3 tg, bt;
		basis_from_normal(n, tg, bt);
		V3 s = add(add(mul(n, cosT), mul(tg, x)), mul(bt, y));
		float pdf = cosT;
		V3 dirIn = neg(s);
		float dif = clampf(-dot(dirIn, n), 0.f, 1.f);
		V3 colorOut = mul(alb, dif);
		if (!(pdf > 0.f && dot(dirIn, n) < 0.f)) break;
		V3 rs = mul(colorOut, __fdiv_rn(intensity, pdf));
		if (!(avg3(rs) > kStopAtVisibility)) break;
		T = mulv(T, rs);
		if (LOG && vi < kMaxVerts) { log->rs[vi] = rs; log->cont[vi] = true; }
		eye = p;
		dir = s;
		skip = tri;
	}
	return L;
}

// first segment of a hemisphere sample (learned gather): the hit point,
// plane and albedo as a cache query record; t[0] = 1 marks a hit
__device__ CacheRec first_hit(const GatherScene& g, V3 eye, V3 dir, uint32_t skip, bool& overflow) {
	CacheRec r;
	RayState rs;
	set_ray(rs, eye, dir, g.tmin, g.locality);
	GatherFilter f = make_filter(g, skip, true);
	float tb = rs.tmax;
	uint32_t tri = 0xFFFFFFFFu;
	int slot = traverse<false, true>(g.nodes, g.tris, rs, g.nnodes, g.ntris, tb, tri, overflow, &f);
	if (slot < 0) {
		for (int k = 0; k < 3; k++) { r.p[k] = 0.f; r.n[k] = 0.f; r.alb[k] = 0.f; r.t[k] = 0.f; }
		return r;
	}
	float4 a, b, c;
	load_tri(g.tris, slot, a, b, c);
	Fastest fs = fastest_fields(rs, a, b, c);
	V3 p = add(eye, mul(dir, fs.dist));
	const float* al = g.albedo + 3 * (size_t)tri;
	r.p[0] = p.x; r.p[1] = p.y; r.p[2] = p.z;
	r.n[0] = fs.n[0]; r.n[1] = fs.n[1]; r.n[2] = fs.n[2];
	r.alb[0] = al[0]; r.alb[1] = al[1]; r.alb[2] = al[2];
	r.t[0] = 1.f; r.t[1] = 0.f; r.t[2] = 0.f;
	return r;
}

// HomogenousFiller2::GetTrianglePoint (gather.cpp:65-83)
__device__ __forceinline__ void filler_point(unsigned n, float& a, float& b) {
	float x = 0.f, y = 0.f, dist = 1.f;
	while (n) {
		unsigned q = n & 3;
		float dx = q == 0 ? 0.f : (q == 1 ? 0.f : (q == 2 ? 0.86602540378444f : -0.86602540378444f));
		float dy = q == 0 ? 0.f : (q == 1 ? 1.f : -0.5f);
		float dm = q == 0 ? -0.5f : 0.5f;
		x = __fadd_rn(x, __fmul_rn(dist, dx));
		y = __fadd_rn(y, __fmul_rn(dist, dy));
		dist = __fmul_rn(dist, dm);
		n >>= 2;
	}
	a = x;
	b = y;
}

constexpr int kGatherWarps = 4;
constexpr int kMaxQuality = 256;
constexpr int kMaxRounds = kMaxQuality / 10 + 1;

struct WarpSmem {
	float fx[kMaxQuality], fy[kMaxQuality], fd[kMaxQuality];
	V3 hemi[kMaxQuality];
	V3 light[kMaxRounds][2];
	V3 lbent[kMaxRounds][2];          // the light rounds' bent-normal terms
	unsigned char lit[kMaxRounds][2];
	unsigned char distant[kMaxQuality];   // first hit farther than ao_size
	unsigned next;   // next unclaimed sample of the texel
};

// ---------------------------------------------------------------- wavefront
// The plain gather as a wavefront: the hemisphere paths of a batch of texels
// advance bounce by bounce, one thread per live path, instead of one warp per
// texel following its lanes' paths to the end (where the warp waits for its
// longest path: about 5 of 32 lanes busy).  Each bounce is trace_path's loop
// body split into kernels: k_wf_closest (the closest hit and its fields,
// then the contributions toward the lights, wf_nee), k_wf_shadow (one thread
// per shadow ray), k_wf_shade (the unoccluded contributions added in light order,
// roulette, next direction), with the same arithmetic in the same order, so
// every path's radiance is bit-identical to trace_path's; k_wf_reduce sums
// each texel's samples in the order the warp-per-texel kernel does.  Path
// state is structure-of-arrays in HBM.
struct WfState {
	float4* eye;           // eye.xyz, skip triangle (bits)
	float4* dir;           // dir.xyz, depth (bits)
	float4* T;             // throughput.xyz, first hit distance
	float4* L;             // radiance.xyz
	float4* dir0;          // first direction.xyz (bent normals)
	float4* hitp;          // hit point.xyz, hit triangle (bits)
	float4* hitn;          // hit plane normal.xyz
	float4* slot_lights;   // per texel of the batch: the light rounds' average (xyz)
	float4* slot_bl;       // per texel of the batch: the light rounds' bent-normal sum (xyz)
	uint64_t* slot_tid;    // per texel of the batch: texel id (~0: uncovered)
	float4* nee;           // 2 x cap: next-event contribution toward light li of path p at [2p + li];
	                       // w = 1: a shadow ray decides, 2: unoccluded, 0: nothing to add
	uint32_t* live;        // 2 x cap: live path lists, ping-pong
	uint32_t* hits;        // cap: paths that hit in this bounce
	uint32_t* shadow;      // 2 x cap: shadow rays of this bounce (2p + li)
	uint32_t* counts;      // [0], [1]: live counts (ping-pong), [2]: hits, [3]: shadow rays,
	                       // [4]: the light rounds' shadow rays
	uint32_t cap;          // paths
	uint32_t Q, N;
	// the light rounds of a batch's texels: slot (ti x shot + round) x 2 + light
	float4* lr_light;      // the round's contribution (xyz); w = 1 once its shadow ray found the light
	float4* lr_bent;       // its bent-normal term (xyz)
	float4* lr_ray;        // 2 per shadow ray: (origin, shooter triangle bits), (direction, length)
	uint32_t* lr_slot;     // the slot of each shadow ray
	uint32_t shot;         // light rounds per texel
	unsigned long long* rays = nullptr;   // optional counts of traced rays: [0] closest, [1] shadow
};

// Adds the rays traced by the calling lanes to a counter (one atomic per
// converged group of lanes).
__device__ __forceinline__ void count_ray(unsigned long long* c) {
	const unsigned m = __activemask();
	if ((threadIdx.x & 31) == (unsigned)(__ffs(m) - 1)) atomicAdd(c, (unsigned long long)__popc(m));
}

// Directional mode (gatherAllDirections, lightmap.cpp:820): each hemisphere
// sample's weights for the four lightmap directions (its cosine to the
// direction over its cosine to the normal; < 0: not added,
// gather.cpp:255-272), and each light's irradiance and cosines to the
// directions (gather.cpp:468-486).
struct WarpSmemDir {
	float wgt[kMaxQuality][4];
	V3 lirr[kMaxRounds][2];
	float lw[kMaxRounds][2][4];
};

// RRVec3::abs().avg() (RRMath.h:170-171), one rounding per operation
__device__ __forceinline__ float absavg3(V3 a) {
	return __fmul_rn(__fadd_rn(__fadd_rn(fabsf(a.x), fabsf(a.y)), fabsf(a.z)), 0.33333333333333f);
}

// LEARNED = false: the plain gather, out[tid - out_base] = texel RGBA.
// LEARNED = true : first segments only; recs[(tid - out_base) * Q + k] get the
// cache queries and out[tid - out_base] the light rounds' average (the plain
// texel's first term) with w = 1.  list (may be null) selects texel ids.
// WF = true: the set-up of the wavefront gather (k_wf_*): texel ti of the
// launch writes its Q paths' first rays (path ti * Q + k) and its light
// rounds' sums instead of tracing the paths.
template <bool LEARNED, bool DIR = false, bool WF = false>
__global__ void __launch_bounds__(kGatherWarps * 32, 6) k_gather(GatherScene g, const uint32_t* __restrict__ off,
                                                              const Sub* __restrict__ st, uint64_t first,
                                                              uint64_t count, const uint32_t* __restrict__ list,
                                                              uint64_t out_base, float4* __restrict__ out,
                                                              CacheRec* __restrict__ recs, uint32_t* counter,
                                                              uint32_t* status, float4* __restrict__ bent_out,
                                                              DirOut dout = DirOut{}, WfState wf = WfState{}) {
	__shared__ WarpSmem sm_all[kGatherWarps];
	WarpSmem& sm = sm_all[threadIdx.x >> 5];
	__shared__ typename std::conditional<DIR, WarpSmemDir, char>::type smd_all[kGatherWarps];
	auto& smd = smd_all[threadIdx.x >> 5];
	const int lane = threadIdx.x & 31;
	const uint32_t Q = g.quality;
	const uint32_t rounds = Q / 10 + 1;
	const uint32_t N = Q > rounds ? Q : rounds;
	bool overflow = false;
	while (true) {
		uint64_t ti = 0;
		if (lane == 0) ti = atomicAdd((unsigned long long*)counter, 1ull);
		ti = __shfl_sync(0xFFFFFFFFu, ti, 0);
		if (ti >= count) break;
		const uint64_t tid = list ? (uint64_t)list[ti] : first + ti;
		const uint64_t oi = tid - out_base;
		const uint32_t b = off[tid], m = off[tid + 1] - b;
		if (m == 0) {
			if (WF && lane == 0) wf.slot_tid[ti] = ~0ull;
			if (lane == 0) out[oi] = make_float4(0.f, 0.f, 0.f, 0.f);
			if (lane == 0 && bent_out) bent_out[oi] = make_float4(0.f, 0.f, 0.f, 0.f);
			if (DIR && lane == 0)
				for (int i = 0; i < 3; i++)
					if (dout.d[i]) dout.d[i][oi] = make_float4(0.f, 0.f, 0.f, 0.f);
			continue;
		}
		const Sub* S = st + b;
		for (int q = lane; q < kMaxRounds * 2; q += 32) sm.lit[q >> 1][q & 1] = 0;
		if (WF)   // the wavefront traces the light rounds' shadow rays later (k_wf_light_trace)
			for (uint32_t q = lane; q < 2 * wf.shot; q += 32)
				wf.lr_light[(size_t)ti * 2 * wf.shot + q] = make_float4(0.f, 0.f, 0.f, 0.f);
		// HomogenousFiller2 points: candidate num = reset + j, the k-th accepted one
		// serves hemisphere ray k (gather.cpp:88-93)
		const unsigned reset = (unsigned)(hash64(g.seed, S_FILLER, tid) & 0xffffu);
		uint32_t found = 0;
		for (uint32_t j0 = 0; found < Q; j0 += 32) {
			float x, y;
			filler_point(reset + j0 + lane, x, y);
			float dd = __fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y));
			bool ok = dd < 1.f;
			unsigned m32 = __ballot_sync(0xFFFFFFFFu, ok);
			uint32_t slot = found + __popc(m32 & ((1u << lane) - 1));
			if (ok && slot < Q) { sm.fx[slot] = x; sm.fy[slot] = y; sm.fd[slot] = dd; }
			found += __popc(m32);
		}
		__syncwarp();
		float areaMax = 0.f;
		for (uint32_t i = 0; i < m; i++) areaMax = __fadd_rn(areaMax, S[i].area);
		const float areaStep = __fdiv_rn(areaMax, __fadd_rn((float)N, 0.91f));
		if (lane == 0) sm.next = 32;
		__syncwarp();
		// samples are claimed dynamically: a lane whose path ended early takes
		// the next unclaimed one (results are stored per sample index and
		// summed in index order, so the texel does not depend on who traced what)
		for (uint32_t k = lane; k < N; k = atomicAdd(&sm.next, 1u)) {
			// area stepping (gather.cpp:665-688), replayed up to shooter k
			float areaAccu = -S[0].area;
			uint32_t it = 0;
			uint32_t gl = 0, round = 0;
			bool fires = false;
			for (uint32_t q = 0; q <= k; q++) {
				areaAccu = __fadd_rn(areaAccu, areaStep);
				while (areaAccu > 0.f) {
					it++;
					if (it == m) it = 0;
					areaAccu = __fsub_rn(areaAccu, S[it].area);
				}
				bool f = (uint64_t)gl * (N - 1) < (uint64_t)rounds * q || rounds >= Q;
				if (q == k) { fires = f; round = gl; }
				if (f) gl++;
			}
			const Sub& s = S[it];
			V3 v0, s1, s2;
			V3 fn = tri_normal(g, s.tri, v0, s1, s2);
			float cu = __fmul_rn(__fadd_rn(__fadd_rn(s.uv[0], s.uv[2]), s.uv[4]), 0.333333333f);
			float cv = __fmul_rn(__fadd_rn(__fadd_rn(s.uv[1], s.uv[3]), s.uv[5]), 0.333333333f);
			float w = __fsub_rn(__fsub_rn(1.f, cu), cv);
			V3 nrm = normalized(add(add(mul(fn, w), mul(fn, cu)), mul(fn, cv)));
			V3 tg, bt;
			basis_from_normal(nrm, tg, bt);
			// directional mode: the skewed basis (gather.cpp:725-730; the vertices'
			// bases are the plane normal's, RRMesh.cpp:77-91) and the four
			// lightmap directions in it
			V3 ldir[4];
			if (DIR) {
				V3 ft, fb;
				basis_from_normal(fn, ft, fb);
				const V3 ts = normalized(add(add(mul(ft, w), mul(ft, cu)), mul(ft, cv)));
				const V3 bs = normalized(add(add(mul(fb, w), mul(fb, cu)), mul(fb, cv)));
				for (int i = 0; i < 4; i++)
					ldir[i] = normalized(add(add(mul(ts, g.ldir[i][0]), mul(bs, g.ldir[i][1])), mul(nrm, g.ldir[i][2])));
			}
			const uint64_t sid = tid * N + k;
			uint32_t ru = rng24(g.seed, S_PU, sid), rv = rng24(g.seed, S_PV, sid);
			if (ru + rv > kM24) { ru = kM24 - ru; rv = kM24 - rv; }
			float fu = __fdiv_rn((float)ru, (float)kM24), fv = __fdiv_rn((float)rv, (float)kM24);
			float pu = __fadd_rn(__fadd_rn(s.uv[0], __fmul_rn(__fsub_rn(s.uv[2], s.uv[0]), fu)),
			                     __fmul_rn(__fsub_rn(s.uv[4], s.uv[0]), fv));
			float pv = __fadd_rn(__fadd_rn(s.uv[1], __fmul_rn(__fsub_rn(s.uv[3], s.uv[1]), fu)),
			                     __fmul_rn(__fsub_rn(s.uv[5], s.uv[1]), fv));
			V3 origin = add(add(v0, mul(s1, pu)), mul(s2, pv));
			if (k < Q) {
				float cosa = __fsqrt_rn(__fsub_rn(1.f, sm.fd[k]));
				V3 dir = add(add(mul(nrm, cosa), mul(tg, sm.fx[k])), mul(bt, sm.fy[k]));
				if (LEARNED) {
					recs[oi * Q + k] = first_hit(g, origin, dir, s.tri, overflow);
				} else if (WF) {
					const uint32_t pth = (uint32_t)ti * Q + k;
					wf.eye[pth] = make_float4(origin.x, origin.y, origin.z, __uint_as_float(s.tri));
					wf.dir[pth] = make_float4(dir.x, dir.y, dir.z, __uint_as_float(0u));
					wf.T[pth] = make_float4(1.f, 1.f, 1.f, 1e10f);
					wf.L[pth] = make_float4(0.f, 0.f, 0.f, 0.f);
					wf.dir0[pth] = make_float4(dir.x, dir.y, dir.z, 0.f);
					wf.live[atomicAdd(&wf.counts[0], 1u)] = pth;
				} else {
					float ft = 1e10f;
					const V3 Lk = trace_path(g, origin, dir, s.tri, sid, overflow, nullptr, &ft);
					sm.hemi[k] = Lk;
					sm.distant[k] = ft > g.ao_size ? 1 : 0;
					// the filler point of sample k is used up: its slots hold the
					// sample's bent-normal term dir * |L|.avg (gather.cpp:274)
					const V3 bk = mul(dir, absavg3(Lk));
					sm.fx[k] = bk.x;
					sm.fy[k] = bk.y;
					sm.fd[k] = bk.z;
					if constexpr (DIR) {
						const float ni1 = dot(dir, nrm);
						const float inv = ni1 > 0.f ? __fdiv_rn(1.f, ni1) : 0.f;
						for (int i = 0; i < 4; i++) {
							const float ni2 = dot(dir, ldir[i]);
							smd.wgt[k][i] = (ni1 > 0.f && ni2 > 0.f) ? __fmul_rn(ni2, inv) : -1.f;
						}
					}
				}
			}
			if (WF && fires && round < wf.shot) {
				// the round's contributions, and its shadow rays for k_wf_light_trace
				for (int li = 0; li < 2; li++) {
					const size_t slot = ((size_t)ti * wf.shot + round) * 2 + li;
					V3 d = li == 0 ? neg(g.dir_direction) : sub(g.point_position, origin);
					float dsize = len(d);
					d = divf(d, dsize);
					if (li == 0) dsize = __fmul_rn(dsize, g.locality);
					float ni = dot(d, nrm);
					if (ni <= 0.f || !isfinite(ni)) continue;
					V3 irr = li == 0 ? g.dir_color : point_irr(g, origin);
					const V3 lc = mul(irr, ni), lb = mul(d, __fmul_rn(absavg3(irr), ni));   // gather.cpp:488
					wf.lr_light[slot] = make_float4(lc.x, lc.y, lc.z, 0.f);
					wf.lr_bent[slot] = make_float4(lb.x, lb.y, lb.z, 0.f);
					const uint32_t j = atomicAdd(&wf.counts[4], 1u);
					wf.lr_ray[2 * (size_t)j] = make_float4(origin.x, origin.y, origin.z, __uint_as_float(s.tri));
					wf.lr_ray[2 * (size_t)j + 1] = make_float4(d.x, d.y, d.z, dsize);
					wf.lr_slot[j] = (uint32_t)slot;
				}
			} else if (fires && round < (uint32_t)kMaxRounds) {
				for (int li = 0; li < 2; li++) {
					sm.lit[round][li] = 0;
					V3 d = li == 0 ? neg(g.dir_direction) : sub(g.point_position, origin);
					float dsize = len(d);
					d = divf(d, dsize);
					if (li == 0) dsize = __fmul_rn(dsize, g.locality);
					float ni = dot(d, nrm);
					if (ni <= 0.f || !isfinite(ni)) continue;
					if (WF && wf.rays) count_ray(wf.rays + 1);
					if (occluded(g, origin, d, g.tmin, dsize, s.tri, overflow)) continue;
					V3 irr = li == 0 ? g.dir_color : point_irr(g, origin);
					sm.light[round][li] = mul(irr, ni);
					sm.lbent[round][li] = mul(d, __fmul_rn(absavg3(irr), ni));   // gather.cpp:488
					if constexpr (DIR) {
						smd.lirr[round][li] = irr;
						for (int i = 0; i < 4; i++) {
							const float ni2 = dot(d, ldir[i]);
							smd.lw[round][li][i] = ni2 > 0.f ? ni2 : -1.f;
						}
					}
					sm.lit[round][li] = 1;
				}
			}
		}
		__syncwarp();
		if (lane == 0) {
			V3 hemi = mk(0.f, 0.f, 0.f), lights = mk(0.f, 0.f, 0.f);
			if (!LEARNED && !WF)
				for (uint32_t k = 0; k < Q; k++) hemi = add(hemi, sm.hemi[k]);
			uint32_t shot = rounds < (uint32_t)kMaxRounds ? rounds : (uint32_t)kMaxRounds;
			for (uint32_t r = 0; r < shot; r++)
				for (int li = 0; li < 2; li++)
					if (sm.lit[r][li]) lights = add(lights, sm.light[r][li]);
			lights = divf(lights, (float)shot);
			if (WF) {
				wf.slot_tid[ti] = tid;   // the light rounds are summed by k_wf_light_sum
			} else if (LEARNED) {
				out[oi] = make_float4(lights.x, lights.y, lights.z, texel_alpha(g, tid));
			} else {
				float f = __fdiv_rn(1.f, (float)Q);
				if (g.ao_intensity > 0.f && g.ao_size > 0.f) {
					uint32_t nd = 0;
					for (uint32_t k = 0; k < Q; k++) nd += sm.distant[k];
					f = __fmul_rn(f, powf(__fdiv_rn((float)nd, (float)Q), g.ao_intensity));
				}
				hemi = mul(hemi, f);
				V3 res = add(lights, hemi);
				if constexpr (DIR) {
					// every output weighted by its direction, summed in sample order
					for (int i = 0; i < 4; i++) {
						V3 hi = mk(0.f, 0.f, 0.f), li_ = mk(0.f, 0.f, 0.f);
						for (uint32_t k = 0; k < Q; k++)
							if (smd.wgt[k][i] >= 0.f) hi = add(hi, mul(sm.hemi[k], smd.wgt[k][i]));
						for (uint32_t r = 0; r < shot; r++)
							for (int l = 0; l < 2; l++)
								if (sm.lit[r][l] && smd.lw[r][l][i] >= 0.f) li_ = add(li_, mul(smd.lirr[r][l], smd.lw[r][l][i]));
						const V3 ri = add(divf(li_, (float)shot), mul(hi, f));
						if (i == 0)
							res = ri;
						else if (dout.d[i - 1])
							dout.d[i - 1][oi] = make_float4(ri.x, ri.y, ri.z, texel_alpha(g, tid));
					}
				}
				out[oi] = make_float4(res.x, res.y, res.z, texel_alpha(g, tid));
				if (bent_out) {
					V3 bl = mk(0.f, 0.f, 0.f), bh = mk(0.f, 0.f, 0.f);
					for (uint32_t r = 0; r < shot; r++)
						for (int li = 0; li < 2; li++)
							if (sm.lit[r][li]) bl = add(bl, sm.lbent[r][li]);
					for (uint32_t k = 0; k < Q; k++) bh = add(bh, mk(sm.fx[k], sm.fy[k], sm.fd[k]));
					V3 b = add(bl, bh);
					if (b.x != 0.f || b.y != 0.f || b.z != 0.f) b = divf(b, len(b));
					bent_out[oi] = make_float4(__fmul_rn(__fadd_rn(b.x, 1.f), 0.5f), __fmul_rn(__fadd_rn(b.y, 1.f), 0.5f),
					                           __fmul_rn(__fadd_rn(b.z, 1.f), 0.5f), texel_alpha(g, tid));
				}
			}
		}
		__syncwarp();
	}
	if (overflow) atomicOr(status, (uint32_t)RRG_ERR_STACK);
}

// Next event estimation of path p at its hit (trace_path's loop body after
// the closest hit): the contribution toward each light, and a shadow ray
// where the light is above the surface and the contribution is not zero.
// Called by k_wf_closest right after the hit, with the hit in registers.
__device__ __forceinline__ void wf_nee(const GatherScene& g, const WfState& w, uint32_t p, V3 pnt, V3 nrm,
                                       uint32_t tri) {
	const V3 alb = ld3(g.albedo + 3 * (size_t)tri);
	for (int li = 0; li < 2; li++) {
		float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
		V3 sdir;
		if (li == 0) {
			sdir = neg(g.dir_direction);
		} else {
			V3 dd = sub(g.point_position, pnt);
			sdir = normalized(dd);
		}
		if (dot(nrm, sdir) > 0.f) {
			V3 unob = li == 0 ? g.dir_color : point_irr(g, pnt);
			float dif = clampf(-dot(neg(sdir), nrm), 0.f, 1.f);
			V3 contrib = mulv(unob, mul(alb, dif));
			if (!(contrib.x == 0.f && contrib.y == 0.f && contrib.z == 0.f)) {
				e = make_float4(contrib.x, contrib.y, contrib.z, 1.f);
				w.shadow[atomicAdd(&w.counts[3], 1u)] = 2 * p + (uint32_t)li;
			}
		}
		w.nee[2 * (size_t)p + li] = e;
	}
}

// (The wavefront's traversal kernels are capped at 7 blocks of 128 per SM:
// 72 registers, no spills in k_wf_closest; measured 1 % faster over the
// config-2 bake than 8 blocks with 64 registers and spills.)
// Closest hit of every live path (trace_path's traversal and hit fields),
// in the order of `order` (the live paths sorted by their rays' key) or of
// the live list.
__global__ void __launch_bounds__(128, 7) k_wf_closest(GatherScene g, WfState w, int cur, const uint32_t* order,
                                                     uint32_t* status) {
	const uint32_t n = w.counts[cur];
	const uint32_t* live = order ? order : w.live + (size_t)cur * w.cap;
	bool overflow = false;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const uint32_t p = live[i];
		const float4 e = w.eye[p], d = w.dir[p];
		const V3 eye = mk(e.x, e.y, e.z), dir = mk(d.x, d.y, d.z);
		const uint32_t skip = __float_as_uint(e.w), depth = __float_as_uint(d.w);
		RayState r;
		set_ray(r, eye, dir, g.tmin, depth == 0 ? g.locality : 1e10f);
		GatherFilter f = make_filter(g, skip, true);
		float tb = r.tmax;
		uint32_t tri = 0xFFFFFFFFu;
		const int slot = traverse<false, true>(g.nodes, g.tris, r, g.nnodes, g.ntris, tb, tri, overflow, &f);
		if (slot < 0) continue;   // the path ends with what it has gathered
		float4 a, b, c;
		load_tri(g.tris, slot, a, b, c);
		const Fastest fs = fastest_fields(r, a, b, c);
		if (depth == 0) w.T[p].w = fs.dist;   // the first hit's distance, for ambient occlusion
		const V3 hp = add(eye, mul(dir, fs.dist));
		w.hitp[p] = make_float4(hp.x, hp.y, hp.z, __uint_as_float(tri));
		w.hitn[p] = make_float4(fs.n[0], fs.n[1], fs.n[2], 0.f);
		w.hits[atomicAdd(&w.counts[2], 1u)] = p;
		wf_nee(g, w, p, hp, mk(fs.n[0], fs.n[1], fs.n[2]), tri);
	}
	if (overflow) atomicOr(status, (uint32_t)RRG_ERR_STACK);
}

// The learned gather's first segments on the wavefront: one thread per path
// the set-up (k_gather<0, 0, 1>) started, each path's first hit as a cache
// query record (first_hit, as the warp-per-texel learned kernel writes it),
// record of path p = ti * Q + k at recs[p] (recs = the batch's first texel's
// records).
__global__ void __launch_bounds__(128, 7) k_wf_first_hit(GatherScene g, WfState w, const uint32_t* order,
                                                       CacheRec* __restrict__ recs, uint32_t* status) {
	const uint32_t n = w.counts[0];
	const uint32_t* live = order ? order : w.live;
	bool overflow = false;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const uint32_t p = live[i];
		const float4 e = w.eye[p], d = w.dir[p];
		recs[p] = first_hit(g, mk(e.x, e.y, e.z), mk(d.x, d.y, d.z), __float_as_uint(e.w), overflow);
	}
	if (overflow) atomicOr(status, (uint32_t)RRG_ERR_STACK);
}

// The learned texel's first term, the light rounds' average, as the
// warp-per-texel learned kernel writes it (uncovered texels: the set-up wrote 0).
__global__ void k_wf_learned_out(GatherScene g, WfState w, uint32_t nb, uint64_t out_base, float4* __restrict__ out) {
	const uint32_t ti = blockIdx.x * blockDim.x + threadIdx.x;
	if (ti >= nb) return;
	const uint64_t tid = w.slot_tid[ti];
	if (tid == ~0ull) return;
	const float4 l = w.slot_lights[ti];
	out[tid - out_base] = make_float4(l.x, l.y, l.z, texel_alpha(g, tid));
}

// The shadow rays of this bounce, one thread each (the same ray and test as
// trace_path's occluded() call).
__global__ void __launch_bounds__(128, 7) k_wf_shadow(GatherScene g, WfState w, uint32_t* status) {
	const uint32_t n = w.counts[3];
	bool overflow = false;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const uint32_t q = w.shadow[i], p = q >> 1, li = q & 1u;
		const float4 hp4 = w.hitp[p];
		const V3 pnt = mk(hp4.x, hp4.y, hp4.z);
		const uint32_t tri = __float_as_uint(hp4.w);
		V3 sdir;
		float smax;
		if (li == 0) {
			sdir = neg(g.dir_direction);
			smax = 1e10f;
		} else {
			V3 dd = sub(g.point_position, pnt);
			sdir = normalized(dd);
			smax = len(dd);
		}
		if (!occluded(g, pnt, sdir, g.tmin, smax, tri, overflow)) w.nee[q].w = 2.f;
	}
	if (overflow) atomicOr(status, (uint32_t)RRG_ERR_STACK);
}

// The light rounds' shadow rays of a batch, one thread each (the set-up
// made them: processTexel's light rounds, gather.cpp:421-559 via
// GatheredIrradianceLights::shotRay): a ray that reaches its light marks the
// round's contribution.
__global__ void __launch_bounds__(128, 7) k_wf_light_trace(GatherScene g, WfState w, uint32_t* status) {
	const uint32_t n = w.counts[4];
	bool overflow = false;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const float4 o4 = w.lr_ray[2 * (size_t)i], d4 = w.lr_ray[2 * (size_t)i + 1];
		if (w.rays) count_ray(w.rays + 1);
		if (!occluded(g, mk(o4.x, o4.y, o4.z), mk(d4.x, d4.y, d4.z), g.tmin, d4.w, __float_as_uint(o4.w), overflow))
			w.lr_light[w.lr_slot[i]].w = 1.f;
	}
	if (overflow) atomicOr(status, (uint32_t)RRG_ERR_STACK);
}

// Each texel's light rounds, averaged in round and light order as the
// warp-per-texel kernel sums them (gather.cpp:541-559), and their
// bent-normal terms.
__global__ void k_wf_light_sum(WfState w, uint32_t nb) {
	const uint32_t ti = blockIdx.x * blockDim.x + threadIdx.x;
	if (ti >= nb || w.slot_tid[ti] == ~0ull) return;
	V3 lights = mk(0.f, 0.f, 0.f), bl = mk(0.f, 0.f, 0.f);
	for (uint32_t r = 0; r < w.shot; r++)
		for (int li = 0; li < 2; li++) {
			const size_t slot = ((size_t)ti * w.shot + r) * 2 + li;
			const float4 l = w.lr_light[slot];
			if (l.w > 0.f) {
				lights = add(lights, mk(l.x, l.y, l.z));
				const float4 b = w.lr_bent[slot];
				bl = add(bl, mk(b.x, b.y, b.z));
			}
		}
	lights = divf(lights, (float)w.shot);
	w.slot_lights[ti] = make_float4(lights.x, lights.y, lights.z, 0.f);
	w.slot_bl[ti] = make_float4(bl.x, bl.y, bl.z, 0.f);
}

// The rest of trace_path's loop body for every path that hit: the unoccluded
// contributions added in light order, Russian roulette, the next direction.
// Paths that continue go to the other live list.
__global__ void __launch_bounds__(128) k_wf_shade(GatherScene g, WfState w, int cur) {
	const uint32_t n = w.counts[2];
	if (w.rays && blockIdx.x == 0 && threadIdx.x == 0) {
		atomicAdd(w.rays, (unsigned long long)w.counts[cur]);       // this bounce's closest-hit rays
		atomicAdd(w.rays + 1, (unsigned long long)w.counts[3]);     // and its shadow rays
	}
	uint32_t* next = w.live + (size_t)(cur ^ 1) * w.cap;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const uint32_t p = w.hits[i];
		const float4 hp4 = w.hitp[p], hn4 = w.hitn[p], T4 = w.T[p], L4 = w.L[p], d4 = w.dir[p];
		const V3 pnt = mk(hp4.x, hp4.y, hp4.z), nrm = mk(hn4.x, hn4.y, hn4.z);
		const uint32_t tri = __float_as_uint(hp4.w), depth = __float_as_uint(d4.w);
		V3 T = mk(T4.x, T4.y, T4.z), L = mk(L4.x, L4.y, L4.z);
		const uint64_t sid = w.slot_tid[p / w.Q] * w.N + p % w.Q;
		const V3 alb = ld3(g.albedo + 3 * (size_t)tri);
		for (int li = 0; li < 2; li++) {
			const float4 e = w.nee[2 * (size_t)p + li];
			if (e.w == 2.f) L = add(L, mulv(T, mk(e.x, e.y, e.z)));
		}
		w.L[p] = make_float4(L.x, L.y, L.z, 0.f);
		float pdiff = avg3(alb);
		if (pdiff < 0.f) pdiff = 0.f;
		float pstop = __fsub_rn(1.f, pdiff);
		if (pstop < 0.f) pstop = 0.f;
		float rr = rng01(g.seed, S_ROULETTE, sid * (kMaxDepth + 1) + depth);
		if (!(rr < pdiff && depth < g.max_depth)) continue;
		float intensity = __fdiv_rn(__fadd_rn(pdiff, pstop), pdiff);
		float x = 0.f, y = 0.f;
		for (int j = 0; j < kDiskTries; j++) {
			uint64_t cc = (sid * (kMaxDepth + 1) + depth) * kDiskTries + j;
			float ax = __fsub_rn(__fmul_rn(rng01(g.seed, S_DISKX, cc), 2.0f), 1.0f);
			float by = __fsub_rn(__fmul_rn(rng01(g.seed, S_DISKY, cc), 2.0f), 1.0f);
			if (__fadd_rn(__fmul_rn(ax, ax), __fmul_rn(by, by)) < 1.0f) { x = ax; y = by; break; }
		}
		float cosT = __fsqrt_rn(__fsub_rn(1.0f, __fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y))));
		V3 tg, bt;
		basis_from_normal(nrm, tg, bt);
		V3 s = add(add(mul(nrm, cosT), mul(tg, x)), mul(bt, y));
		float pdf = cosT;
		V3 dirIn = neg(s);
		float dif = clampf(-dot(dirIn, nrm), 0.f, 1.f);
		V3 colorOut = mul(alb, dif);
		if (!(pdf > 0.f && dot(dirIn, nrm) < 0.f)) continue;
		V3 rs = mul(colorOut, __fdiv_rn(intensity, pdf));
		if (!(avg3(rs) > kStopAtVisibility)) continue;
		T = mulv(T, rs);
		w.T[p] = make_float4(T.x, T.y, T.z, T4.w);
		w.eye[p] = make_float4(pnt.x, pnt.y, pnt.z, __uint_as_float(tri));
		w.dir[p] = make_float4(s.x, s.y, s.z, __uint_as_float(depth + 1));
		next[atomicAdd(&w.counts[cur ^ 1], 1u)] = p;
	}
}

// Texel sums (the warp-per-texel kernel's lane-0 tail): the samples' radiance
// in sample order, the ambient-occlusion factor, the bent normal.
__global__ void k_wf_reduce(GatherScene g, WfState w, uint32_t nslots, uint64_t out_base, float4* __restrict__ out,
                            float4* __restrict__ bent_out) {
	const uint32_t Q = w.Q;
	for (uint32_t sl = blockIdx.x * blockDim.x + threadIdx.x; sl < nslots; sl += gridDim.x * blockDim.x) {
		const uint64_t tid = w.slot_tid[sl];
		if (tid == ~0ull) continue;   // uncovered: written by the set-up
		const uint64_t oi = tid - out_base;
		V3 hemi = mk(0.f, 0.f, 0.f);
		uint32_t nd = 0;
		for (uint32_t k = 0; k < Q; k++) {
			const float4 l = w.L[(size_t)sl * Q + k];
			hemi = add(hemi, mk(l.x, l.y, l.z));
			nd += w.T[(size_t)sl * Q + k].w > g.ao_size ? 1u : 0u;
		}
		const float4 l4 = w.slot_lights[sl];
		const V3 lights = mk(l4.x, l4.y, l4.z);
		float f = __fdiv_rn(1.f, (float)Q);
		if (g.ao_intensity > 0.f && g.ao_size > 0.f) f = __fmul_rn(f, powf(__fdiv_rn((float)nd, (float)Q), g.ao_intensity));
		hemi = mul(hemi, f);
		const V3 res = add(lights, hemi);
		out[oi] = make_float4(res.x, res.y, res.z, texel_alpha(g, tid));
		if (bent_out) {
			const float4 b4 = w.slot_bl[sl];
			V3 bl = mk(b4.x, b4.y, b4.z), bh = mk(0.f, 0.f, 0.f);
			for (uint32_t k = 0; k < Q; k++) {
				const float4 l = w.L[(size_t)sl * Q + k], d0 = w.dir0[(size_t)sl * Q + k];
				bh = add(bh, mul(mk(d0.x, d0.y, d0.z), absavg3(mk(l.x, l.y, l.z))));
			}
			V3 b = add(bl, bh);
			if (b.x != 0.f || b.y != 0.f || b.z != 0.f) b = divf(b, len(b));
			bent_out[oi] = make_float4(__fmul_rn(__fadd_rn(b.x, 1.f), 0.5f), __fmul_rn(__fadd_rn(b.y, 1.f), 0.5f),
			                           __fmul_rn(__fadd_rn(b.z, 1.f), 0.5f), texel_alpha(g, tid));
		}
	}
}

// Training paths for the radiance cache: path i starts at covered texel
// covered[(i / spt) * stride] (spt paths per texel) from a random point of a
// random sub-texel in a cosine direction, traces a plain path and writes one
// record for each of its first kTrainRecords vertices: position, plane
// normal, albedo and the outgoing radiance toward the previous vertex.
// The learned gather asks the cache at a hemisphere sample's first hit for
// what the plain gather gets there: the light of that vertex and of the
// `window` bounces after it (stopAtDepth), L = sum_j T_kj nee_j over
// j = k .. k + window.  So every record's target is that same window: the
// path is traced kTrainRecords - 1 bounces deeper than the gather's (g's
// max_depth is the gather's plus that), and record k sums vertices
// k .. k + window only.  (Summing each vertex's whole path tail instead
// gives vertex k only window - k bounces, and the cache learned too little
// light: 2.5 to 8 % on the config-2 atlases.)
constexpr int kTrainRecords = 4;

__global__ void __launch_bounds__(128) k_train_paths(GatherScene g, const uint32_t* __restrict__ off,
                                                     const Sub* __restrict__ st, const uint32_t* __restrict__ covered,
                                                     uint32_t ncov, uint32_t stride, uint32_t spt, uint64_t npaths,
                                                     uint64_t seed, CacheRec* __restrict__ recs, uint64_t cap,
                                                     unsigned long long* count, uint32_t* status, uint32_t window) {
	bool overflow = false;
	PathLog log;
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < npaths;
	     i += (uint64_t)gridDim.x * blockDim.x) {
		uint64_t ci = (i / spt) * stride;
		if (ci >= ncov) continue;
		const uint64_t tid = covered[ci];
		const uint32_t b = off[tid], m = off[tid + 1] - b;
		if (!m) continue;
		const Sub& s = st[b + (uint32_t)(hash64(seed, 70, i) % m)];
		V3 v0, s1, s2;
		V3 nrm = tri_normal(g, s.tri, v0, s1, s2);
		uint32_t ru = rng24(seed, 71, i), rv = rng24(seed, 72, i);
		if (ru + rv > kM24) { ru = kM24 - ru; rv = kM24 - rv; }
		float fu = __fdiv_rn((float)ru, (float)kM24), fv = __fdiv_rn((float)rv, (float)kM24);
		float pu = s.uv[0] + (s.uv[2] - s.uv[0]) * fu + (s.uv[4] - s.uv[0]) * fv;
		float pv = s.uv[1] + (s.uv[3] - s.uv[1]) * fu + (s.uv[5] - s.uv[1]) * fv;
		V3 origin = add(add(v0, mul(s1, pu)), mul(s2, pv));
		float x = 0.f, y = 0.f;
		for (int j = 0; j < kDiskTries; j++) {
			float ax = rng01(seed, 73, i * kDiskTries + j) * 2.f - 1.f;
			float by = rng01(seed, 74, i * kDiskTries + j) * 2.f - 1.f;
			if (ax * ax + by * by < 1.f) { x = ax; y = by; break; }
		}
		V3 tg, bt;
		basis_from_normal(nrm, tg, bt);
		V3 dir = add(add(mul(nrm, sqrtf(fmaxf(0.f, 1.f - x * x - y * y))), mul(tg, x)), mul(bt, y));
		trace_path<true>(g, origin, dir, s.tri, (seed << 20) ^ (i + 0x9E37ull), overflow, &log);
		const int nk = log.n < kTrainRecords ? log.n : kTrainRecords;
		for (int k = 0; k < nk; k++) {
			// L_k over vertices k .. k + window, the throughput carried along
			V3 Lk = mk(0.f, 0.f, 0.f), T = mk(1.f, 1.f, 1.f);
			const int last = k + (int)window < log.n - 1 ? k + (int)window : log.n - 1;
			for (int j = k; j <= last; j++) {
				Lk = add(Lk, mulv(T, log.nee[j]));
				if (!log.cont[j]) break;
				T = mulv(T, log.rs[j]);
			}
			unsigned long long slot = atomicAdd(count, 1ull);
			if (slot >= cap) continue;
			CacheRec r;
			r.p[0] = log.p[k].x; r.p[1] = log.p[k].y; r.p[2] = log.p[k].z;
			r.n[0] = log.nrm[k].x; r.n[1] = log.nrm[k].y; r.n[2] = log.nrm[k].z;
			r.alb[0] = log.alb[k].x; r.alb[1] = log.alb[k].y; r.alb[2] = log.alb[k].z;
			r.t[0] = Lk.x; r.t[1] = Lk.y; r.t[2] = Lk.z;
			recs[slot] = r;
		}
	}
	if (overflow) atomicOr(status, (uint32_t)RRG_ERR_STACK);
}

// Learned texel = light rounds' average + mean of the cache over the Q
// hemisphere samples (summed in sample order).  Texels whose samples fall in
// unreliable cache cells more often than `frac` go to the fallback list.
__global__ void k_learned_reduce(const uint32_t* __restrict__ off, uint64_t first, uint64_t count, uint32_t Q,
                                 const CacheRec* __restrict__ recs, const float4* __restrict__ rad,
                                 float4* __restrict__ out, const uint8_t* __restrict__ reliable, int res,
                                 float lo0, float lo1, float lo2, float ie0, float ie1, float ie2, float frac,
                                 uint32_t* __restrict__ fb_list, unsigned int* fb_count) {
	uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	if (i >= count) return;
	const uint64_t tid = first + i;
	if (off[tid + 1] == off[tid]) return;   // uncovered: the first pass wrote 0
	V3 hemi = mk(0.f, 0.f, 0.f);
	uint32_t bad = 0;
	for (uint32_t k = 0; k < Q; k++) {
		const float4 r = rad[i * Q + k];
		hemi = add(hemi, mk(r.x, r.y, r.z));
		if (reliable && r.w > 0.f) {
			const CacheRec& c = recs[i * Q + k];
			int vx = min(res - 1, max(0, (int)((c.p[0] - lo0) * ie0 * res)));
			int vy = min(res - 1, max(0, (int)((c.p[1] - lo1) * ie1 * res)));
			int vz = min(res - 1, max(0, (int)((c.p[2] - lo2) * ie2 * res)));
			if (!reliable[((size_t)vz * res + vy) * res + vx]) bad++;
		}
	}
	hemi = mul(hemi, __fdiv_rn(1.f, (float)Q));
	float4 l = out[i];
	out[i] = make_float4(__fadd_rn(l.x, hemi.x), __fadd_rn(l.y, hemi.y), __fadd_rn(l.z, hemi.z), l.w);
	if (fb_list && (float)bad > frac * (float)Q) fb_list[atomicAdd(fb_count, 1u)] = (uint32_t)tid;
}

// ------------------------------------------------------------ lightmapper
struct Lightmapper {
	Collider* c = nullptr;
	uint32_t natlas = 0, size = 0;
	uint64_t ntexels = 0, nsub = 0;
	float* d_albedo = nullptr;
	uint32_t* d_off = nullptr;    // ntexels + 1
	Sub* d_sub = nullptr;
	uint64_t* d_counter = nullptr;
	uint32_t* d_status = nullptr;
	unsigned long long* d_rays = nullptr;   // traced-ray counters of the wavefront gather (when counting)
	bool count_rays = false;
	float* d_stage = nullptr;
	size_t stage_bytes = 0;
	float tmin_default = 0.f;
	uint32_t* d_covered = nullptr;   // ids of texels with sub-texels
	uint8_t* d_flags = nullptr;      // TexelFlags per texel (ntexels rounded up to 4)
	// host copies of the unwrap (for the lightmap filters' seam search)
	std::vector<float> h_uv;
	std::vector<int32_t> h_atlas;
	LightmapFilter* filter = nullptr;   // filter scratch and seams (rrg_filter.cu)
	// wavefront gather state (grown on demand): 7 float4 per path, 2 float4 +
	// 1 id per texel of a batch, 3 path lists, 3 counters
	void* d_wf = nullptr;
	size_t wf_bytes = 0;
	uint32_t ray_order = RRG_RAY_ORDER_DEFAULT;   // wavefront rays in path order, or in key order (BINNED)
	uint64_t ncovered = 0;
	// learned-gather work buffers (grown on demand)
	CacheRec* d_recs = nullptr;
	float4* d_rad = nullptr;
	uint32_t* d_fb = nullptr;
	unsigned int* d_fbcount = nullptr;
	// the bake's radiosity solver (rrg_lightmapper_bake_solver): per triangle
	// direct irradiance and smoothed corner indirect; the corner stitching
	// (built on the first bake) as groups of corners
	float* d_solver_direct = nullptr;   // 3 per triangle
	float* d_solver_corner = nullptr;   // 9 per triangle
	uint32_t* d_corner_group = nullptr; // 3 per triangle
	uint32_t* d_group_off = nullptr;    // ngroups + 1
	uint32_t* d_group_corner = nullptr; // weighted corners, group by group, corner order
	float* d_corner_weight = nullptr;   // 3 per triangle
	uint32_t ngroups = 0;
	uint32_t* d_bake_hits = nullptr;    // rays x triangles (ray j of triangle t at j * triangles + t)
	size_t bake_hits_cap = 0;
	uint64_t bake_hits_used = 0;
	uint32_t bake_k = 0;
	float* d_bake_e = nullptr;          // E, E' (3 per triangle each), group values (3 per group)
	float4* d_bake_re = nullptr;        // albedo * E, two per triangle (ping-pong)
	const float* d_bake_final = nullptr;  // the converged E (one of the two above)
	uint64_t lg_cap = 0;             // texels
	uint64_t lg_cap_samples = 0;     // texels x samples per texel
};

static void free_lm(Lightmapper* L) {
	if (!L) return;
	filter_free(L->filter);
	cudaFree(L->d_wf);
	cudaFree(L->d_albedo);
	cudaFree(L->d_flags);
	cudaFree(L->d_off);
	cudaFree(L->d_sub);
	cudaFree(L->d_counter);
	cudaFree(L->d_status);
	cudaFree(L->d_rays);
	cudaFree(L->d_stage);
	cudaFree(L->d_covered);
	cudaFree(L->d_recs);
	cudaFree(L->d_rad);
	cudaFree(L->d_fb);
	cudaFree(L->d_fbcount);
	cudaFree(L->d_solver_direct);
	cudaFree(L->d_solver_corner);
	cudaFree(L->d_corner_group);
	cudaFree(L->d_group_off);
	cudaFree(L->d_group_corner);
	cudaFree(L->d_corner_weight);
	cudaFree(L->d_bake_hits);
	cudaFree(L->d_bake_e);
	cudaFree(L->d_bake_re);
	delete L;
}

static int make_scene(Lightmapper* L, const rrg_gather_params* p, GatherScene& g) {
	// a caller built against the struct without the ambient-occlusion fields
	// passes the smaller size; those fields then read as 0
	if (!p || p->size < offsetof(rrg_gather_params, ao_intensity)) return RRG_ERR_INVALID;
	if (p->quality == 0 || p->quality > (uint32_t)kMaxQuality) return RRG_ERR_INVALID;
	Collider* c = L->c;
	g.nodes = c->d_nodes;
	g.tris = c->d_tris;
	g.nnodes = (int)c->nnodes;
	g.ntris = (int)c->nvalid;
	g.xyz = c->d_xyz;
	g.idx = c->d_idx;
	g.albedo = L->d_albedo;
	g.flags = L->d_flags;
	{   // UE3 lightmap directions, gather.cpp:43-49 (host sqrtf, as the reference's static table)
		const float s6 = sqrtf(6.0f), s3 = sqrtf(3.0f), s2 = sqrtf(2.0f);
		const float D[4][3] = {{0.f, 0.f, 1.f}, {0.f, s6 / 3, 1 / s3}, {-1 / s2, -1 / s6, 1 / s3}, {1 / s2, -1 / s6, 1 / s3}};
		memcpy(g.ldir, D, sizeof(D));
	}
	g.dir_direction = mk(p->dir_direction[0], p->dir_direction[1], p->dir_direction[2]);
	g.dir_color = mk(p->dir_color[0], p->dir_color[1], p->dir_color[2]);
	g.point_position = mk(p->point_position[0], p->point_position[1], p->point_position[2]);
	g.point_color = mk(p->point_color[0], p->point_color[1], p->point_color[2]);
	g.tmin = p->ray_length_min > 0.f ? p->ray_length_min : L->tmin_default;
	g.locality = p->locality > 0.f ? p->locality : 100000.f;
	g.quality = p->quality;
	g.max_depth = p->max_depth < kMaxDepth ? p->max_depth : kMaxDepth;
	g.seed = p->seed;
	const bool has_ao = p->size >= sizeof(rrg_gather_params);
	g.ao_intensity = has_ao ? p->ao_intensity : 0.f;
	g.ao_size = has_ao ? p->ao_size : 0.f;
	if (!(g.ao_intensity >= 0.f) || !(g.ao_size >= 0.f)) return RRG_ERR_INVALID;
	if ((p->mode & 3u) > RRG_GATHER_WAVEFRONT || (p->mode & ~(3u | RRG_GATHER_SOLVER))) return RRG_ERR_INVALID;
	g.solver_direct = nullptr;
	g.solver_corner = nullptr;
	if (p->mode & RRG_GATHER_SOLVER) {
		if (!L->d_solver_direct) return RRG_ERR_INVALID;   // no solver baked yet
		g.solver_direct = L->d_solver_direct;
		g.solver_corner = L->d_solver_corner;
	}
	return RRG_OK;
}

template <bool LEARNED, bool DIR = false>
static int launch_gather_kernel(Lightmapper* L, const GatherScene& g, uint64_t first, uint64_t count,
                                const uint32_t* list, uint64_t out_base, float4* out, CacheRec* recs, cudaStream_t s,
                                float4* bent = nullptr, DirOut dout = DirOut{}) {
	if (!count) return RRG_OK;
	RRG_CUDA(cudaMemsetAsync(L->d_counter, 0, 8, s));
	int per_sm = 0;
	RRG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gather<LEARNED, DIR>, kGatherWarps * 32, 0));
	uint64_t want = (count + kGatherWarps - 1) / kGatherWarps;
	uint64_t cap = (uint64_t)(per_sm > 0 ? per_sm : 1) * L->c->num_sms;
	int grid = (int)(want < cap ? want : cap);
	rrg::note_launch(), k_gather<LEARNED, DIR><<<grid, kGatherWarps * 32, 0, s>>>(g, L->d_off, L->d_sub, first, count, list, out_base, out,
	                                                          recs, reinterpret_cast<uint32_t*>(L->d_counter), L->d_status,
	                                                          LEARNED ? nullptr : bent, dout);
	RRG_CUDA(cudaGetLastError());
	return RRG_OK;
}

// The wavefront gather of texels [first, first + count): batches of texels,
// each set up by k_gather<0, 0, 1> (first rays and light rounds), advanced
// bounce by bounce (k_wf_closest with each hit's next-event estimation,
// k_wf_shadow, k_wf_shade; the
// path counts stay on the device) and summed (k_wf_reduce).
// The lightmapper's device scratch (the wavefront's path state; the bake's
// triangle-major form-factor hits between k_bake_factors and the transpose),
// grown on demand.
static int grow_scratch(Lightmapper* L, size_t bytes) {
	if (bytes <= L->wf_bytes) return RRG_OK;
	cudaFree(L->d_wf);
	L->d_wf = nullptr;
	L->wf_bytes = 0;
	RRG_CUDA(cudaMalloc(&L->d_wf, bytes));
	L->wf_bytes = bytes;
	return RRG_OK;
}

constexpr uint64_t kWfMinTexels = 16384;
// paths per batch: 2^25 (6 GB of path state at about 180 B a path) keeps the
// deep bounces' launches full; on the config-2 scene 2^23 measured 4 %
// slower and 2^24 1 % slower
constexpr uint64_t kWfMaxPaths = 1ull << 25;

// recs: the learned gather's first segments instead (the records of texel
// first + i at recs + i * Q, out = the light rounds' average).
static int gather_wavefront(Lightmapper* L, const GatherScene& g, uint64_t first, uint64_t count, float4* out,
                            float4* bent, cudaStream_t s, CacheRec* recs = nullptr) {
	const uint32_t Q = g.quality;
	const uint32_t rounds = Q / 10 + 1;
	const uint32_t N = Q > rounds ? Q : rounds;
	const uint64_t B = std::min<uint64_t>(count, kWfMaxPaths / Q);   // texels per batch
	const uint64_t cap = B * Q;                                       // paths per batch
	const uint32_t shot = rounds < (uint32_t)kMaxRounds ? rounds : (uint32_t)kMaxRounds;
	const uint64_t nslot = B * shot * 2;   // light rounds of a batch
	const size_t base_bytes = (9 * 16 * cap + 2 * 16 * B + 8 * B + 5 * 4 * cap + 32 + 255) / 256 * 256;
	const size_t state_bytes = base_bytes + (4 * 16 * nslot + 4 * nslot + 255) / 256 * 256;
	// binned order (RRG_RAY_ORDER_BINNED): the live paths sorted by their
	// rays' key before each closest-hit pass, with the sort's scratch after
	// the state.  Not the default: on the config-2 scene it measured 4-6 %
	// slower than path order, whose warps already hold one texel's rays.
	const bool binned = L->ray_order == RRG_RAY_ORDER_BINNED;
	const size_t order_bytes = binned ? (4 * cap + 255) / 256 * 256 : 0;
	const size_t bin_bytes = binned ? bin_paths_bytes(L->c, (uint32_t)cap) : 0;
	if (int st = grow_scratch(L, state_bytes + order_bytes + bin_bytes)) return st;
	WfState w;
	float4* f4 = reinterpret_cast<float4*>(L->d_wf);
	w.eye = f4;
	w.dir = f4 + cap;
	w.T = f4 + 2 * cap;
	w.L = f4 + 3 * cap;
	w.dir0 = f4 + 4 * cap;
	w.hitp = f4 + 5 * cap;
	w.hitn = f4 + 6 * cap;
	w.nee = f4 + 7 * cap;
	w.slot_lights = f4 + 9 * cap;
	w.slot_bl = f4 + 9 * cap + B;
	w.slot_tid = reinterpret_cast<uint64_t*>(f4 + 9 * cap + 2 * B);
	w.live = reinterpret_cast<uint32_t*>(w.slot_tid + B);
	w.hits = w.live + 2 * cap;
	w.shadow = w.hits + cap;
	w.counts = w.shadow + 2 * cap;
	float4* lr = reinterpret_cast<float4*>(reinterpret_cast<uint8_t*>(L->d_wf) + base_bytes);
	w.lr_light = lr;
	w.lr_bent = lr + nslot;
	w.lr_ray = lr + 2 * nslot;
	w.lr_slot = reinterpret_cast<uint32_t*>(lr + 4 * nslot);
	w.shot = shot;
	w.cap = (uint32_t)cap;
	w.Q = Q;
	w.N = N;
	w.rays = L->count_rays ? L->d_rays : nullptr;
	uint32_t* order = binned ? reinterpret_cast<uint32_t*>(reinterpret_cast<uint8_t*>(L->d_wf) + state_bytes) : nullptr;
	void* bin_scratch = binned ? reinterpret_cast<uint8_t*>(L->d_wf) + state_bytes + order_bytes : nullptr;
	int per_sm = 0;
	RRG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gather<false, false, true>, kGatherWarps * 32, 0));
	int per_sm_c = 0;
	RRG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_c, k_wf_closest, 128, 0));
	const int grid_c = std::max(1, per_sm_c) * L->c->num_sms;
	for (uint64_t b0 = 0; b0 < count; b0 += B) {
		const uint64_t nb = std::min<uint64_t>(B, count - b0);
		RRG_CUDA(cudaMemsetAsync(L->d_counter, 0, 8, s));
		RRG_CUDA(cudaMemsetAsync(w.counts, 0, 5 * sizeof(uint32_t), s));
		const uint64_t want = (nb + kGatherWarps - 1) / kGatherWarps;
		const uint64_t capb = (uint64_t)(per_sm > 0 ? per_sm : 1) * L->c->num_sms;
		const int grid = (int)(want < capb ? want : capb);
		rrg::note_launch(), k_gather<false, false, true><<<grid, kGatherWarps * 32, 0, s>>>(
		    g, L->d_off, L->d_sub, first + b0, nb, nullptr, first, out, nullptr, reinterpret_cast<uint32_t*>(L->d_counter),
		    L->d_status, nullptr, DirOut{}, w);
		rrg::note_launch(), k_wf_light_trace<<<grid_c, 128, 0, s>>>(g, w, L->d_status);
		rrg::note_launch(), k_wf_light_sum<<<(int)((nb + 127) / 128), 128, 0, s>>>(w, (uint32_t)nb);
		RRG_CUDA(cudaGetLastError());
		if (recs) {
			if (binned) {
				if (int st = bin_paths(L->c, w.eye, w.dir, w.live, w.counts, (uint32_t)cap, bin_scratch, order, s))
					return st;
			}
			rrg::note_launch(), k_wf_first_hit<<<grid_c, 128, 0, s>>>(g, w, order, recs + b0 * Q, L->d_status);
			rrg::note_launch(), k_wf_learned_out<<<(int)((nb + 127) / 128), 128, 0, s>>>(g, w, (uint32_t)nb, first, out);
			RRG_CUDA(cudaGetLastError());
			continue;
		}
		int cur = 0;
		for (uint32_t depth = 0; depth <= g.max_depth; depth++) {
			RRG_CUDA(cudaMemsetAsync(w.counts + 2, 0, 2 * sizeof(uint32_t), s));
			RRG_CUDA(cudaMemsetAsync(w.counts + (cur ^ 1), 0, sizeof(uint32_t), s));
			if (binned) {
				if (int st = bin_paths(L->c, w.eye, w.dir, w.live + (size_t)cur * cap, w.counts + cur, (uint32_t)cap,
				                       bin_scratch, order, s))
					return st;
			}
			rrg::note_launch(), k_wf_closest<<<grid_c, 128, 0, s>>>(g, w, cur, order, L->d_status);
			rrg::note_launch(), k_wf_shadow<<<grid_c, 128, 0, s>>>(g, w, L->d_status);
			rrg::note_launch(), k_wf_shade<<<grid_c, 128, 0, s>>>(g, w, cur);
			cur ^= 1;
		}
		rrg::note_launch(), k_wf_reduce<<<(int)((nb + 127) / 128), 128, 0, s>>>(g, w, (uint32_t)nb, first, out, bent);
		RRG_CUDA(cudaGetLastError());
	}
	return RRG_OK;
}

// ------------------------------------------------------------ bake solver
// The default bake's radiosity solver (updateSolverIndirectIllumination,
// RRSolver/gather.cpp:1038-1117, over RRStaticSolver): the first gather per
// triangle at half quality, form-factor rays, the flux balance solved by
// Jacobi iteration of its gathering form, corner smoothing.  The same sample
// streams as the oracle, so the two agree to float rounding.
enum { S_TRI_PU = 80, S_TRI_PV = 81, S_FF_PU = 82, S_FF_PV = 83, S_FF_DX = 84, S_FF_DY = 85 };
constexpr float kShotOffset = 1e-4f;   // SHOT_OFFSET, geometry_v.h:30
constexpr float kBigReal = 1e20f;      // BIG_REAL, geometry_v.h:28

// a random point of the triangle (the whole triangle as the sub-texel,
// gather.cpp:742-749; rrcore.cpp:1016-1024)
__device__ __forceinline__ void tri_point(uint64_t seed, uint64_t su, uint64_t sv, uint64_t i, float& pu, float& pv) {
	uint32_t ru = rng24(seed, su, i), rv = rng24(seed, sv, i);
	if (ru + rv > kM24) { ru = kM24 - ru; rv = kM24 - rv; }
	pu = __fdiv_rn((float)ru, (float)kM24);
	pv = __fdiv_rn((float)rv, (float)kM24);
}

// First gather per triangle (gatherPerTrianglePhysical, gather.cpp:843-952):
// `rounds` light rounds from random points of the triangle, no hemisphere.
__global__ void __launch_bounds__(128) k_bake_direct(GatherScene g, uint32_t nt, uint32_t rounds, float* __restrict__ direct,
                                                     uint32_t* status) {
	bool overflow = false;
	for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
		V3 v0, s1, s2;
		const V3 n = tri_normal(g, t, v0, s1, s2);
		V3 acc = mk(0.f, 0.f, 0.f);
		for (uint32_t r = 0; r < rounds; r++) {
			float pu, pv;
			tri_point(g.seed, S_TRI_PU, S_TRI_PV, (uint64_t)t * rounds + r, pu, pv);
			const V3 o = add(add(v0, mul(s1, pu)), mul(s2, pv));
			for (int li = 0; li < 2; li++) {
				V3 d = li == 0 ? neg(g.dir_direction) : sub(g.point_position, o);
				float dsize = len(d);
				d = divf(d, dsize);
				if (li == 0) dsize = __fmul_rn(dsize, g.locality);
				const float ni = dot(d, n);
				if (!(ni > 0.f) || !isfinite(ni)) continue;
				if (occluded(g, o, d, g.tmin, dsize, t, overflow)) continue;
				const V3 irr = li == 0 ? g.dir_color : point_irr(g, o);
				acc = add(acc, mul(irr, ni));
			}
		}
		acc = divf(acc, (float)rounds);
		direct[3 * (size_t)t] = acc.x;
		direct[3 * (size_t)t + 1] = acc.y;
		direct[3 * (size_t)t + 2] = acc.z;
	}
	if (overflow) atomicOr(status, (uint32_t)RRG_ERR_STACK);
}

// Form-factor rays (shotFromToHalfspace / rayTracePhoton, rrcore.cpp:
// 861-1050): ray i of triangle i / k from a random point, cosine-distributed
// over the front half-space (Malley's method), nearest hit on either side
// with only the shooter skipped (RRCollisionHandlerLod0, rrcore.cpp:670-723);
// a front hit on a triangle whose albedo sums above 0.01 is a factor.
__global__ void __launch_bounds__(128, 8) k_bake_factors(GatherScene g, uint32_t nt, uint32_t k,
                                                         uint32_t* __restrict__ hits, uint32_t* status) {
	bool overflow = false;
	const uint64_t total = (uint64_t)nt * k;
	// thread i traces ray j = i % k of triangle t = i / k (a warp's rays leave
	// one triangle: coherent traversal); hits are written triangle-major and
	// transposed for the iteration by k_bake_transpose
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
		const uint32_t t = (uint32_t)(i / k);
		V3 v0, s1, s2;
		const V3 n = tri_normal(g, t, v0, s1, s2);
		V3 tg, bt;
		basis_from_normal(n, tg, bt);
		float pu, pv;
		tri_point(g.seed, S_FF_PU, S_FF_PV, i, pu, pv);
		const V3 o = add(add(v0, mul(s1, pu)), mul(s2, pv));
		float x = 0.f, y = 0.f;
		for (int q = 0; q < kDiskTries; q++) {
			const uint64_t c = i * kDiskTries + q;
			float a = __fsub_rn(__fmul_rn(rng01(g.seed, S_FF_DX, c), 2.0f), 1.0f);
			float b = __fsub_rn(__fmul_rn(rng01(g.seed, S_FF_DY, c), 2.0f), 1.0f);
			if (__fadd_rn(__fmul_rn(a, a), __fmul_rn(b, b)) < 1.0f) { x = a; y = b; break; }
		}
		const float cosa = __fsqrt_rn(__fsub_rn(1.0f, __fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y))));
		const V3 d = add(add(mul(n, cosa), mul(tg, x)), mul(bt, y));
		RayState r;
		set_ray(r, o, d, kShotOffset, kBigReal);
		GatherFilter f = make_filter(g, t, false);
		f.ident_t = -1.f;   // every side collides, only the shooter is skipped
		float tb = r.tmax;
		uint32_t tri = 0xFFFFFFFFu;
		const int slot = traverse<false, true>(g.nodes, g.tris, r, g.nnodes, g.ntris, tb, tri, overflow, &f);
		uint32_t h = 0xFFFFFFFFu;
		if (slot >= 0) {
			float4 a, b, c;
			load_tri(g.tris, slot, a, b, c);
			const V3 alb = ld3(g.albedo + 3 * (size_t)tri);
			if (front_facing(r, a, b, c) && __fadd_rn(__fadd_rn(alb.x, alb.y), alb.z) > 0.01f) h = tri;
		}
		hits[i] = h;
	}
	if (overflow) atomicOr(status, (uint32_t)RRG_ERR_STACK);
}

// Triangle-major hits (t * k + j) to ray-major (j * nt + t) through a 32 x 32
// tile in shared memory, both sides coalesced.  Block 32 x 8.
__global__ void k_bake_transpose(const uint32_t* __restrict__ in, uint32_t nt, uint32_t k, uint32_t* __restrict__ out) {
	__shared__ uint32_t tile[32][33];
	const uint32_t t0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
	for (uint32_t y = threadIdx.y; y < 32; y += 8) {
		const uint32_t t = t0 + y, j = j0 + threadIdx.x;
		if (t < nt && j < k) tile[y][threadIdx.x] = in[(size_t)t * k + j];
	}
	__syncthreads();
	for (uint32_t y = threadIdx.y; y < 32; y += 8) {
		const uint32_t j = j0 + y, t = t0 + threadIdx.x;
		if (t < nt && j < k) out[(size_t)j * nt + t] = tile[threadIdx.x][y];
	}
}

// One Jacobi step of E_j = D_j + (1/k) sum over j's factor hits h of
// albedo_h * E_h (the flux balance of rrcore.cpp:1052-1086 in gathering
// form).  re holds albedo * E of every triangle (one 16-byte load per hit);
// the step writes E' and albedo * E' for the next.
__global__ void __launch_bounds__(128) k_bake_iterate(const float* __restrict__ direct, const float* __restrict__ albedo,
                                                      const uint32_t* __restrict__ hits, uint32_t nt, uint32_t k,
                                                      float inv, const float4* __restrict__ re,
                                                      float* __restrict__ e2, float4* __restrict__ re2) {
	for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
		V3 acc = mk(0.f, 0.f, 0.f);
		for (uint32_t j = 0; j < k; j++) {
			const uint32_t h = hits[(size_t)j * nt + t];
			if (h == 0xFFFFFFFFu) continue;
			const float4 r = re[h];
			acc = add(acc, mk(r.x, r.y, r.z));
		}
		const V3 r = add(ld3(direct + 3 * (size_t)t), mul(acc, inv));
		e2[3 * (size_t)t] = r.x;
		e2[3 * (size_t)t + 1] = r.y;
		e2[3 * (size_t)t + 2] = r.z;
		const V3 q = mulv(ld3(albedo + 3 * (size_t)t), r);
		re2[t] = make_float4(q.x, q.y, q.z, 0.f);
	}
}

// albedo * D: the propagation's first source term
__global__ void k_bake_re_init(const float* __restrict__ direct, const float* __restrict__ albedo, uint32_t nt,
                               float4* __restrict__ re) {
	for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
		const V3 q = mulv(ld3(albedo + 3 * (size_t)t), ld3(direct + 3 * (size_t)t));
		re[t] = make_float4(q.x, q.y, q.z, 0.f);
	}
}

// Smoothed indirect of each stitched vertex (IVertex::irradiance,
// interpol.cpp:78-112): the corner-weighted mean of its triangles' indirect
// irradiance (E - D), summed in corner order, clamped at zero; written to
// every corner of the group.
__global__ void k_bake_smooth(const uint32_t* __restrict__ group_off, const uint32_t* __restrict__ group_corner,
                              const float* __restrict__ weight, const float* __restrict__ e,
                              const float* __restrict__ direct, uint32_t ngroups, float* __restrict__ gval) {
	for (uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x; gi < ngroups; gi += gridDim.x * blockDim.x) {
		V3 num = mk(0.f, 0.f, 0.f);
		float den = 0.f;
		for (uint32_t q = group_off[gi]; q < group_off[gi + 1]; q++) {
			const uint32_t c = group_corner[q];
			const float w = weight[c];
			const size_t t3 = 3 * (size_t)(c / 3);
			const V3 ind = sub(ld3(e + t3), ld3(direct + t3));
			num = add(num, mul(ind, w));
			den = __fadd_rn(den, w);
		}
		V3 v = den > 0.f ? divf(num, den) : mk(0.f, 0.f, 0.f);
		gval[3 * (size_t)gi] = v.x > 0.f ? v.x : 0.f;
		gval[3 * (size_t)gi + 1] = v.y > 0.f ? v.y : 0.f;
		gval[3 * (size_t)gi + 2] = v.z > 0.f ? v.z : 0.f;
	}
}

__global__ void k_bake_corners(const uint32_t* __restrict__ group, const float* __restrict__ gval, uint32_t ncorner,
                               float* __restrict__ corner) {
	for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < ncorner; c += gridDim.x * blockDim.x) {
		const uint32_t gi = group[c];
		corner[3 * (size_t)c] = gval[3 * (size_t)gi];
		corner[3 * (size_t)c + 1] = gval[3 * (size_t)gi + 1];
		corner[3 * (size_t)c + 2] = gval[3 * (size_t)gi + 2];
	}
}

// Abramowitz & Stegun 4.4.45, as geometry_v.h:114-129 applies it (over the
// whole [-1, 1])
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

// Corner stitching and weights (Object::buildTopIVertices, interpol.cpp:
// 120-170, over RRLessVerticesFilter, RRMeshLessVertices.h:38-237, at the
// default SmoothingParameters): every corner is a vertex with its face's
// normal; identical positions whose normals are within 0.01 rad merge,
// greedily in (position, normal) order against the unique vertices found so
// far, newest first.  A corner weighs its angle (the published polynomial
// above) times its triangle's area (rrcore.cpp:105-111); triangles that
// stitching degenerates weigh nothing.
static uint32_t bake_stitch(const std::vector<float>& xyz, const std::vector<uint32_t>& idx, uint32_t nt,
                            std::vector<uint32_t>& group, std::vector<float>& weight) {
	struct Key {
		float p[3], n[3];
		uint32_t c;
	};
	const uint32_t nc = 3 * nt;
	std::vector<Key> k(nc);
	auto P = [&](uint32_t t, int i) { return &xyz[3 * (size_t)idx[3 * (size_t)t + i]]; };
	for (uint32_t t = 0; t < nt; t++) {
		const float *p0 = P(t, 0), *p1 = P(t, 1), *p2 = P(t, 2);
		const float a0 = p1[0] - p0[0], a1 = p1[1] - p0[1], a2 = p1[2] - p0[2];
		const float b0 = p2[0] - p0[0], b1 = p2[1] - p0[1], b2 = p2[2] - p0[2];
		float n0 = a1 * b2 - a2 * b1, n1 = -a0 * b2 + a2 * b0, n2 = a0 * b1 - a1 * b0;
		const float l = sqrtf(n0 * n0 + n1 * n1 + n2 * n2);
		if (l > 0) { n0 = n0 / l; n1 = n1 / l; n2 = n2 / l; }
		for (int i = 0; i < 3; i++) {
			Key& q = k[3 * (size_t)t + i];
			const float* p = P(t, i);
			q.p[0] = p[0]; q.p[1] = p[1]; q.p[2] = p[2];
			q.n[0] = n0; q.n[1] = n1; q.n[2] = n2;
			q.c = 3 * t + i;
		}
	}
	std::sort(k.begin(), k.end(), [](const Key& a, const Key& b) {
		for (int i = 0; i < 3; i++)
			if (a.p[i] != b.p[i]) return a.p[i] < b.p[i];
		for (int i = 0; i < 3; i++)
			if (a.n[i] != b.n[i]) return a.n[i] < b.n[i];
		return a.c < b.c;
	});
	std::vector<uint32_t> rep;
	rep.reserve(nc);
	group.assign(nc, 0);
	const float min_dot = cosf(0.01f);
	// The reference scans, newest first, every unique vertex with the same x
	// (quadratic on axis-aligned planes).  With weld distance 0 only an
	// identical position can merge, and after the sort identical positions
	// are contiguous, so the scan over the unique vertices of the current
	// position finds the same first match.
	uint32_t block = 0;   // first unique vertex of the current position
	for (uint32_t s = 0; s < nc; s++) {
		const Key& d = k[s];
		if (s == 0 || d.p[0] != k[s - 1].p[0] || d.p[1] != k[s - 1].p[1] || d.p[2] != k[s - 1].p[2])
			block = (uint32_t)rep.size();
		uint32_t g = 0xFFFFFFFFu;
		for (uint32_t u = (uint32_t)rep.size(); u-- > block;) {
			const Key& r = k[rep[u]];
			if (d.n[0] * r.n[0] + d.n[1] * r.n[1] + d.n[2] * r.n[2] >= min_dot) {
				g = u;
				break;
			}
		}
		if (g == 0xFFFFFFFFu) {
			g = (uint32_t)rep.size();
			rep.push_back(s);
		}
		group[d.c] = g;
	}
	weight.assign(nc, 0.f);
	for (uint32_t t = 0; t < nt; t++) {
		float p[3][3];
		for (int i = 0; i < 3; i++)
			for (int j = 0; j < 3; j++) p[i][j] = P(t, i)[j];
		auto len2 = [](const float* v) { return v[0] * v[0] + v[1] * v[1] + v[2] * v[2]; };
		const float s1[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
		const float s2[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
		const float s21[3] = {s2[0] - s1[0], s2[1] - s1[1], s2[2] - s1[2]};
		const float a = len2(s1), b = len2(s2), c = len2(s21);
		const float area = sqrtf(2 * b * c + 2 * c * a + 2 * a * b - a * a - b * b - c * c) / 4;
		const uint32_t* gg = &group[3 * (size_t)t];
		if (!(area > 0) || gg[0] == gg[1] || gg[0] == gg[2] || gg[1] == gg[2]) continue;
		for (int i = 0; i < 3; i++) {
			const float* q0 = p[i];
			const float* q1 = p[(i + 1) % 3];
			const float* q2 = p[(i + 2) % 3];
			float u[3] = {q1[0] - q0[0], q1[1] - q0[1], q1[2] - q0[2]};
			float v[3] = {q2[0] - q0[0], q2[1] - q0[1], q2[2] - q0[2]};
			const float lu = sqrtf(len2(u)), lv = sqrtf(len2(v));
			for (int j = 0; j < 3; j++) { u[j] = u[j] / lu; v[j] = v[j] / lv; }
			float dd = u[0] * v[0] + u[1] * v[1] + u[2] * v[2];
			dd = dd < -1 ? -1 : (dd > 1 ? 1 : dd);
			weight[3 * (size_t)t + i] = as_acos(dd) * area;
		}
	}
	return (uint32_t)rep.size();
}

// device memory freed unless released
struct DevBuf {
	void* p = nullptr;
	~DevBuf() { cudaFree(p); }
	void* release() {
		void* r = p;
		p = nullptr;
		return r;
	}
};

static int bake_solver(Lightmapper* L, const rrg_gather_params* p, uint32_t k, uint32_t iterations, cudaStream_t s) {
	if (!p || p->size < offsetof(rrg_gather_params, ao_intensity)) return RRG_ERR_INVALID;
	rrg_gather_params q{};
	memcpy(&q, p, p->size < sizeof(q) ? p->size : sizeof(q));
	q.mode &= 3u;   // the solver is what this builds
	GatherScene g;
	int st = make_scene(L, &q, g);
	if (st) return st;
	Collider* c = L->c;
	const uint32_t nt = c->nt;
	if (!k) k = q.quality;
	if (!nt || k > 4096 || iterations > 1024) return RRG_ERR_INVALID;
	if (!L->d_corner_group) {   // the stitching depends on the mesh only: built once
		std::vector<float> xyz(3 * (size_t)c->nv);
		std::vector<uint32_t> idx(3 * (size_t)nt);
		RRG_CUDA(cudaMemcpy(xyz.data(), c->d_xyz, xyz.size() * sizeof(float), cudaMemcpyDeviceToHost));
		RRG_CUDA(cudaMemcpy(idx.data(), c->d_idx, idx.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
		for (uint32_t v : idx)
			if (v >= c->nv) return RRG_ERR_INVALID;
		std::vector<uint32_t> group;
		std::vector<float> weight;
		const uint32_t ng = bake_stitch(xyz, idx, nt, group, weight);
		std::vector<uint32_t> off(ng + 1, 0), list;
		for (uint32_t cc = 0; cc < 3 * nt; cc++)
			if (weight[cc] != 0.f) off[group[cc] + 1]++;
		for (uint32_t i = 0; i < ng; i++) off[i + 1] += off[i];
		list.resize(off[ng] ? off[ng] : 1);
		std::vector<uint32_t> cur(off.begin(), off.end() - 1);
		for (uint32_t cc = 0; cc < 3 * nt; cc++)
			if (weight[cc] != 0.f) list[cur[group[cc]]++] = cc;
		DevBuf dg, dw, doff, dl;
		RRG_CUDA(cudaMalloc(&dg.p, group.size() * 4));
		RRG_CUDA(cudaMalloc(&dw.p, weight.size() * 4));
		RRG_CUDA(cudaMalloc(&doff.p, off.size() * 4));
		RRG_CUDA(cudaMalloc(&dl.p, list.size() * 4));
		RRG_CUDA(cudaMemcpy(dg.p, group.data(), group.size() * 4, cudaMemcpyHostToDevice));
		RRG_CUDA(cudaMemcpy(dw.p, weight.data(), weight.size() * 4, cudaMemcpyHostToDevice));
		RRG_CUDA(cudaMemcpy(doff.p, off.data(), off.size() * 4, cudaMemcpyHostToDevice));
		RRG_CUDA(cudaMemcpy(dl.p, list.data(), list.size() * 4, cudaMemcpyHostToDevice));
		L->d_corner_group = (uint32_t*)dg.release();
		L->d_corner_weight = (float*)dw.release();
		L->d_group_off = (uint32_t*)doff.release();
		L->d_group_corner = (uint32_t*)dl.release();
		L->ngroups = ng;
	}
	if (!L->d_solver_direct) {
		DevBuf dd, dc, de, dr;
		RRG_CUDA(cudaMalloc(&dd.p, 3 * (size_t)nt * sizeof(float)));
		RRG_CUDA(cudaMalloc(&dc.p, 9 * (size_t)nt * sizeof(float)));
		RRG_CUDA(cudaMalloc(&de.p, (6 * (size_t)nt + 3 * (size_t)L->ngroups) * sizeof(float)));
		RRG_CUDA(cudaMalloc(&dr.p, 2 * (size_t)nt * sizeof(float4)));
		L->d_solver_direct = (float*)dd.release();
		L->d_solver_corner = (float*)dc.release();
		L->d_bake_e = (float*)de.release();
		L->d_bake_re = (float4*)dr.release();
	}
	const size_t nhits = (size_t)nt * k;
	if (nhits > L->bake_hits_cap) {
		cudaFree(L->d_bake_hits);
		L->d_bake_hits = nullptr;
		L->bake_hits_cap = 0;
		RRG_CUDA(cudaMalloc(&L->d_bake_hits, nhits * sizeof(uint32_t)));
		L->bake_hits_cap = nhits;
	}
	// the rays write their hits triangle-major into the lightmapper's
	// scratch (which the final gather reuses for its path state); the
	// transpose leaves the ray-major copy the Jacobi steps read
	if (int st = grow_scratch(L, nhits * sizeof(uint32_t))) return st;
	uint32_t* hits_tm = reinterpret_cast<uint32_t*>(L->d_wf);
	L->bake_hits_used = nhits;
	L->bake_k = k;
	const uint32_t qh = q.quality / 2 ? q.quality / 2 : 1;
	const uint32_t rounds = qh / 10 + 1;
	const int tgrid = (int)std::min<uint64_t>((nt + 127) / 128, (uint64_t)c->num_sms * 16);
	rrg::note_launch(), k_bake_direct<<<tgrid, 128, 0, s>>>(g, nt, rounds, L->d_solver_direct, L->d_status);
	RRG_CUDA(cudaGetLastError());
	const int fgrid = (int)std::min<uint64_t>((nhits + 127) / 128, (uint64_t)c->num_sms * 64);
	rrg::note_launch(), k_bake_factors<<<fgrid, 128, 0, s>>>(g, nt, k, hits_tm, L->d_status);
	RRG_CUDA(cudaGetLastError());
	rrg::note_launch(), k_bake_transpose<<<dim3((nt + 31) / 32, (k + 31) / 32), dim3(32, 8), 0, s>>>(hits_tm, nt, k, L->d_bake_hits);
	RRG_CUDA(cudaGetLastError());
	float* e = L->d_bake_e;
	float* e2 = e + 3 * (size_t)nt;
	float* gval = e + 6 * (size_t)nt;
	float4* re = L->d_bake_re;
	float4* re2 = re + nt;
	RRG_CUDA(cudaMemcpyAsync(e, L->d_solver_direct, 3 * (size_t)nt * sizeof(float), cudaMemcpyDeviceToDevice, s));
	rrg::note_launch(), k_bake_re_init<<<tgrid, 128, 0, s>>>(L->d_solver_direct, L->d_albedo, nt, re);
	const float inv = 1.0f / (float)k;
	for (uint32_t it = 0; it < iterations; it++) {
		rrg::note_launch(), k_bake_iterate<<<tgrid, 128, 0, s>>>(L->d_solver_direct, L->d_albedo, L->d_bake_hits, nt, k,
		                                                         inv, re, e2, re2);
		std::swap(e, e2);
		std::swap(re, re2);
	}
	RRG_CUDA(cudaGetLastError());
	const int ggrid = (int)std::min<uint64_t>((L->ngroups + 127) / 128 + 1, (uint64_t)c->num_sms * 16);
	L->d_bake_final = e;
	rrg::note_launch(), k_bake_smooth<<<ggrid, 128, 0, s>>>(L->d_group_off, L->d_group_corner, L->d_corner_weight, e,
	                                                        L->d_solver_direct, L->ngroups, gval);
	const int cgrid = (int)std::min<uint64_t>((3 * (uint64_t)nt + 127) / 128, (uint64_t)c->num_sms * 16);
	rrg::note_launch(), k_bake_corners<<<cgrid, 128, 0, s>>>(L->d_corner_group, gval, 3 * nt, L->d_solver_corner);
	RRG_CUDA(cudaGetLastError());
	return RRG_OK;
}

static int gather_launch(Lightmapper* L, const rrg_gather_params* p, uint64_t first, uint64_t count, float* out_dev,
                         cudaStream_t s, float* bent_dev = nullptr, const DirOut* dirs = nullptr) {
	GatherScene g;
	int st = make_scene(L, p, g);
	if (st) return st;
	if (first + count > L->ntexels) return RRG_ERR_INVALID;
	const uint32_t sched = p->mode & 3u;
	const bool directional = dirs && (dirs->d[0] || dirs->d[1] || dirs->d[2]);
	// reading the solver ends every path at its first hit: one ray per
	// sample, which the warp-per-texel kernel keeps busy
	if (!directional && count && !g.solver_direct &&
	    (sched == RRG_GATHER_WAVEFRONT || (sched == RRG_GATHER_AUTO && count >= kWfMinTexels)))
		return gather_wavefront(L, g, first, count, reinterpret_cast<float4*>(out_dev),
		                        reinterpret_cast<float4*>(bent_dev), s);
	if (directional)
		return launch_gather_kernel<false, true>(L, g, first, count, nullptr, first, reinterpret_cast<float4*>(out_dev),
		                                         nullptr, s, reinterpret_cast<float4*>(bent_dev), *dirs);
	return launch_gather_kernel<false>(L, g, first, count, nullptr, first, reinterpret_cast<float4*>(out_dev), nullptr,
	                                   s, reinterpret_cast<float4*>(bent_dev));
}

}  // namespace rrg

using namespace rrg;

LightmapView rrg::lightmapper_view(::rrg_lightmapper* h) {
	Lightmapper* L = reinterpret_cast<Lightmapper*>(h);
	LightmapView v{};
	if (!L) return v;
	v.c = L->c;
	v.natlas = L->natlas;
	v.size = L->size;
	v.nt = L->c->nt;
	v.uv = L->h_uv.data();
	v.atlas = L->h_atlas.data();
	v.filter = &L->filter;
	return v;
}

extern "C" {

int rrg_lightmapper_create(rrg_collider* ch, const float* albedo, const int32_t* tri_atlas, const float* uv,
                           uint32_t natlas, uint32_t size, rrg_lightmapper** out) {
	if (!out) return RRG_ERR_INVALID;
	*out = nullptr;
	Collider* c = reinterpret_cast<Collider*>(ch);
	if (!c || !albedo || !tri_atlas || !uv || !natlas || !size || size > 16384) return RRG_ERR_INVALID;
	const uint64_t ntexels = (uint64_t)natlas * size * size;
	if (ntexels >= (1ull << 32)) return RRG_ERR_INVALID;
	RRG_CUDA(cudaSetDevice(c->device));
	Lightmapper* L = new Lightmapper();
	L->c = c;
	L->natlas = natlas;
	L->size = size;
	L->ntexels = ntexels;
	const uint32_t nt = c->nt;
	L->h_uv.assign(uv, uv + 6 * (size_t)nt);
	L->h_atlas.assign(tri_atlas, tri_atlas + nt);
	float *d_uv = nullptr;
	int32_t* d_atlas = nullptr;
	uint32_t *d_counts = nullptr, *d_cursor = nullptr, *d_bsum = nullptr, *d_err = nullptr, *d_fan = nullptr;
	auto fail = [&](cudaError_t e) {
		cudaFree(d_uv); cudaFree(d_atlas); cudaFree(d_counts); cudaFree(d_cursor); cudaFree(d_bsum);
		cudaFree(d_err); cudaFree(d_fan);
		free_lm(L);
		return cuda_fail(e);
	};
	cudaError_t e;
	if ((e = cudaMalloc(&L->d_albedo, sizeof(float) * 3 * (size_t)nt)) != cudaSuccess) return fail(e);
	if ((e = cudaMemcpy(L->d_albedo, albedo, sizeof(float) * 3 * (size_t)nt, cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e);
	if ((e = cudaMalloc(&d_uv, sizeof(float) * 6 * (size_t)nt)) != cudaSuccess) return fail(e);
	if ((e = cudaMemcpy(d_uv, uv, sizeof(float) * 6 * (size_t)nt, cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e);
	if ((e = cudaMalloc(&d_atlas, sizeof(int32_t) * (size_t)nt)) != cudaSuccess) return fail(e);
	if ((e = cudaMemcpy(d_atlas, tri_atlas, sizeof(int32_t) * (size_t)nt, cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e);
	if ((e = cudaMalloc(&d_counts, sizeof(uint32_t) * ntexels)) != cudaSuccess) return fail(e);
	if ((e = cudaMemset(d_counts, 0, sizeof(uint32_t) * ntexels)) != cudaSuccess) return fail(e);
	if ((e = cudaMalloc(&d_err, 4)) != cudaSuccess) return fail(e);
	if ((e = cudaMemset(d_err, 0, 4)) != cudaSuccess) return fail(e);
	const int grid = c->num_sms * 16;
	if ((e = cudaMalloc(&L->d_flags, (ntexels + 3) / 4 * 4)) != cudaSuccess) return fail(e);
	if ((e = cudaMemset(L->d_flags, 0, (ntexels + 3) / 4 * 4)) != cudaSuccess) return fail(e);
	rrg::note_launch(), k_enumerate<true><<<grid, 256>>>(d_uv, d_atlas, nt, size, natlas, d_counts, nullptr, nullptr, nullptr, nullptr, 0, d_err,
	                                 reinterpret_cast<uint32_t*>(L->d_flags));
	if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
	const uint32_t nb = (uint32_t)((ntexels + kScanPer - 1) / kScanPer);
	if ((e = cudaMalloc(&d_bsum, sizeof(uint32_t) * (nb + 1))) != cudaSuccess) return fail(e);
	if ((e = cudaMalloc(&L->d_off, sizeof(uint32_t) * (ntexels + 1))) != cudaSuccess) return fail(e);
	rrg::note_launch(), k_scan_sums<<<nb, kScanBT>>>(d_counts, ntexels, d_bsum);
	rrg::note_launch(), k_scan_top<<<1, 32>>>(d_bsum, nb);
	rrg::note_launch(), k_scan_apply<<<nb, kScanBT>>>(d_counts, ntexels, d_bsum, L->d_off);
	if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
	uint32_t total = 0;
	if ((e = cudaMemcpy(&total, L->d_off + ntexels, 4, cudaMemcpyDeviceToHost)) != cudaSuccess) return fail(e);
	L->nsub = total;
	if ((e = cudaMalloc(&L->d_sub, sizeof(Sub) * (total ? total : 1))) != cudaSuccess) return fail(e);
	if ((e = cudaMalloc(&d_fan, sizeof(uint32_t) * (total ? total : 1))) != cudaSuccess) return fail(e);
	if ((e = cudaMalloc(&d_cursor, sizeof(uint32_t) * ntexels)) != cudaSuccess) return fail(e);
	if ((e = cudaMemset(d_cursor, 0, sizeof(uint32_t) * ntexels)) != cudaSuccess) return fail(e);
	rrg::note_launch(), k_enumerate<false><<<grid, 256>>>(d_uv, d_atlas, nt, size, natlas, nullptr, L->d_off, d_cursor, L->d_sub, d_fan, total, d_err,
	                                  nullptr);
	rrg::note_launch(), k_sort_texels<<<grid, 256>>>(L->d_off, ntexels, L->d_sub, d_fan);
	if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
	uint32_t herr = 0;
	if ((e = cudaMemcpy(&herr, d_err, 4, cudaMemcpyDeviceToHost)) != cudaSuccess) return fail(e);
	cudaFree(d_uv); cudaFree(d_atlas); cudaFree(d_counts); cudaFree(d_cursor); cudaFree(d_bsum); cudaFree(d_err);
	cudaFree(d_fan);
	d_uv = nullptr; d_atlas = nullptr; d_counts = d_cursor = d_bsum = d_err = d_fan = nullptr;
	if (herr) { free_lm(L); return RRG_ERR_INVALID; }
	if ((e = cudaMalloc(&L->d_counter, 8)) != cudaSuccess) return fail(e);
	if ((e = cudaMalloc(&L->d_status, 4)) != cudaSuccess) return fail(e);
	if ((e = cudaMemset(L->d_status, 0, 4)) != cudaSuccess) return fail(e);
	{   // covered texel list (deterministic order: flags, scan, scatter)
		uint32_t *flag = nullptr, *pos = nullptr, *bs = nullptr;
		if ((e = cudaMalloc(&flag, sizeof(uint32_t) * ntexels)) != cudaSuccess) return fail(e);
		if ((e = cudaMalloc(&pos, sizeof(uint32_t) * (ntexels + 1))) != cudaSuccess) { cudaFree(flag); return fail(e); }
		if ((e = cudaMalloc(&bs, sizeof(uint32_t) * (nb + 1))) != cudaSuccess) { cudaFree(flag); cudaFree(pos); return fail(e); }
		rrg::note_launch(), k_covered_flags<<<grid, 256>>>(L->d_off, ntexels, flag);
		rrg::note_launch(), k_scan_sums<<<nb, kScanBT>>>(flag, ntexels, bs);
		rrg::note_launch(), k_scan_top<<<1, 32>>>(bs, nb);
		rrg::note_launch(), k_scan_apply<<<nb, kScanBT>>>(flag, ntexels, bs, pos);
		uint32_t ncov = 0;
		e = cudaMemcpy(&ncov, pos + ntexels, 4, cudaMemcpyDeviceToHost);
		if (e == cudaSuccess) e = cudaMalloc(&L->d_covered, sizeof(uint32_t) * (ncov ? ncov : 1));
		if (e == cudaSuccess) {
			rrg::note_launch(), k_covered_scatter<<<grid, 256>>>(flag, pos, ntexels, L->d_covered);
			e = cudaGetLastError();
		}
		cudaFree(flag);
		cudaFree(pos);
		cudaFree(bs);
		if (e != cudaSuccess) return fail(e);
		L->ncovered = ncov;
	}
	// minimalSafeDistance = (aabb max - min).avg() * 1e-6 (RRSolver.cpp:329-334)
	float ex = c->aabb_hi[0] - c->aabb_lo[0], ey = c->aabb_hi[1] - c->aabb_lo[1], ez = c->aabb_hi[2] - c->aabb_lo[2];
	L->tmin_default = ((ex + ey) + ez) * 0.33333333333333f * 1e-6f;
	*out = reinterpret_cast<rrg_lightmapper*>(L);
	return RRG_OK;
}

void rrg_lightmapper_destroy(rrg_lightmapper* h) {
	Lightmapper* L = reinterpret_cast<Lightmapper*>(h);
	if (!L) return;
	cudaSetDevice(L->c->device);
	cudaDeviceSynchronize();
	free_lm(L);
}

uint64_t rrg_lightmapper_subtexels(const rrg_lightmapper* h) {
	const Lightmapper* L = reinterpret_cast<const Lightmapper*>(h);
	return L ? L->nsub : 0;
}

float rrg_lightmapper_ray_length_min(const rrg_lightmapper* h) {
	const Lightmapper* L = reinterpret_cast<const Lightmapper*>(h);
	return L ? L->tmin_default : 0.f;
}

int rrg_lightmapper_copy_subtexels(const rrg_lightmapper* h, uint32_t* offsets_host, void* subtexels_host) {
	const Lightmapper* L = reinterpret_cast<const Lightmapper*>(h);
	if (!L || !offsets_host) return RRG_ERR_INVALID;
	RRG_CUDA(cudaMemcpy(offsets_host, L->d_off, sizeof(uint32_t) * (L->ntexels + 1), cudaMemcpyDeviceToHost));
	if (subtexels_host && L->nsub)
		RRG_CUDA(cudaMemcpy(subtexels_host, L->d_sub, sizeof(Sub) * L->nsub, cudaMemcpyDeviceToHost));
	return RRG_OK;
}

int rrg_lightmapper_copy_flags(const rrg_lightmapper* h, uint8_t* flags_host) {
	const Lightmapper* L = reinterpret_cast<const Lightmapper*>(h);
	if (!L || !flags_host) return RRG_ERR_INVALID;
	RRG_CUDA(cudaMemcpy(flags_host, L->d_flags, L->ntexels, cudaMemcpyDeviceToHost));
	return RRG_OK;
}

int rrg_lightmap_gather(rrg_lightmapper* h, const rrg_gather_params* p, uint64_t first_texel, uint64_t ntexels,
                        float* out_dev, void* stream) {
	Lightmapper* L = reinterpret_cast<Lightmapper*>(h);
	if (!L || !out_dev || ((uintptr_t)out_dev & 15)) return RRG_ERR_INVALID;
	return gather_launch(L, p, first_texel, ntexels, out_dev, (cudaStream_t)stream);
}

int rrg_lightmap_gather_ex(rrg_lightmapper* h, const rrg_gather_params* p, uint64_t first_texel, uint64_t ntexels,
                           float* out_dev, float* bent_dev, void* stream) {
	Lightmapper* L = reinterpret_cast<Lightmapper*>(h);
	if (!L || !out_dev || ((uintptr_t)out_dev & 15) || ((uintptr_t)bent_dev & 15)) return RRG_ERR_INVALID;
	return gather_launch(L, p, first_texel, ntexels, out_dev, (cudaStream_t)stream, bent_dev);
}

int rrg_lightmap_gather_directional(rrg_lightmapper* h, const rrg_gather_params* p, uint64_t first_texel,
                                    uint64_t ntexels, float* out_dev, float* dir1_dev, float* dir2_dev, float* dir3_dev,
                                    float* bent_dev, void* stream) {
	Lightmapper* L = reinterpret_cast<Lightmapper*>(h);
	if (!L || !out_dev || ((uintptr_t)out_dev & 15) || ((uintptr_t)bent_dev & 15) || ((uintptr_t)dir1_dev & 15) ||
	    ((uintptr_t)dir2_dev & 15) || ((uintptr_t)dir3_dev & 15))
		return RRG_ERR_INVALID;
	const DirOut d{{reinterpret_cast<float4*>(dir1_dev), reinterpret_cast<float4*>(dir2_dev),
	                reinterpret_cast<float4*>(dir3_dev)}};
	return gather_launch(L, p, first_texel, ntexels, out_dev, (cudaStream_t)stream, bent_dev, &d);
}

int rrg_lightmap_gather_host(rrg_lightmapper* h, const rrg_gather_params* p, uint64_t first_texel, uint64_t ntexels,
                             float* out_host, void* stream) {
	Lightmapper* L = reinterpret_cast<Lightmapper*>(h);
	if (!L || !out_host) return RRG_ERR_INVALID;
	RRG_CUDA(cudaSetDevice(L->c->device));
	size_t bytes = 16 * (size_t)ntexels;
	if (bytes > L->stage_bytes) {
		cudaFree(L->d_stage);
		L->d_stage = nullptr;
		L->stage_bytes = 0;
		RRG_CUDA(cudaMalloc(&L->d_stage, bytes));
		L->stage_bytes = bytes;
	}
	cudaStream_t s = (cudaStream_t)stream;
	int st = gather_launch(L, p, first_texel, ntexels, L->d_stage, s);
	if (st) return st;
	RRG_CUDA(cudaMemcpyAsync(out_host, L->d_stage, bytes, cudaMemcpyDeviceToHost, s));
	RRG_CUDA(cudaStreamSynchronize(s));
	return RRG_OK;
}

int rrg_lightmap_bake_host(rrg_lightmapper* h, const rrg_gather_params* p, const rrg_filter_params* f,
                           float* out_host) {
	Lightmapper* L = reinterpret_cast<Lightmapper*>(h);
	if (!L || !p || !out_host) return RRG_ERR_INVALID;
	const uint64_t n = (uint64_t)L->natlas * L->size * L->size;
	if (!n) return RRG_OK;
	RRG_CUDA(cudaSetDevice(L->c->device));
	const size_t bytes = 16 * (size_t)n;
	if (bytes > L->stage_bytes) {
		cudaFree(L->d_stage);
		L->d_stage = nullptr;
		L->stage_bytes = 0;
		RRG_CUDA(cudaMalloc(&L->d_stage, bytes));
		L->stage_bytes = bytes;
	}
	cudaStream_t s = nullptr;
	int st = gather_launch(L, p, 0, n, L->d_stage, s);
	if (st) return st;
	if (f && f->stages) {
		st = rrg_lightmap_filter(h, f, 0, L->natlas, L->d_stage, s);
		if (st) return st;
	}
	RRG_CUDA(cudaMemcpyAsync(out_host, L->d_stage, bytes, cudaMemcpyDeviceToHost, s));
	RRG_CUDA(cudaStreamSynchronize(s));
	return rrg_lightmapper_status(h, s);
}

int rrg_lightmapper_set_ray_order(rrg_lightmapper* h, uint32_t order) {
	Lightmapper* L = reinterpret_cast<Lightmapper*>(h);
	if (!L || order > RRG_RAY_ORDER_BINNED) return RRG_ERR_INVALID;
	L->ray_order = order;
	return RRG_OK;
}

int rrg_lightmapper_count_rays(rrg_lightmapper* h, int enable, uint64_t* closest, uint64_t* shadow) {
	Lightmapper* L = reinterpret_cast<Lightmapper*>(h);
	if (!L) return RRG_ERR_INVALID;
	RRG_CUDA(cudaSetDevice(L->c->device));
	if (!L->d_rays) {
		RRG_CUDA(cudaMalloc(&L->d_rays, 2 * sizeof(unsigned long long)));
		RRG_CUDA(cudaMemset(L->d_rays, 0, 2 * sizeof(unsigned long long)));
	}
	unsigned long long h2[2] = {0, 0};
	RRG_CUDA(cudaDeviceSynchronize());
	RRG_CUDA(cudaMemcpy(h2, L->d_rays, sizeof(h2), cudaMemcpyDeviceToHost));
	RRG_CUDA(cudaMemset(L->d_rays, 0, sizeof(h2)));
	if (closest) *closest = h2[0];
	if (shadow) *shadow = h2[1];
	L->count_rays = enable != 0;
	return RRG_OK;
}

uint64_t rrg_lightmapper_covered(const rrg_lightmapper* h) {
	const Lightmapper* L = reinterpret_cast<const Lightmapper*>(h);
	return L ? L->ncovered : 0;
}

int rrg_lightmapper_bake_solver(rrg_lightmapper* h, const rrg_gather_params* p, uint32_t rays_per_triangle,
                                uint32_t iterations, void* stream) {
	Lightmapper* L = reinterpret_cast<Lightmapper*>(h);
	if (!L) return RRG_ERR_INVALID;
	RRG_CUDA(cudaSetDevice(L->c->device));
	return bake_solver(L, p, rays_per_triangle, iterations, (cudaStream_t)stream);
}

int rrg_lightmapper_copy_solver(const rrg_lightmapper* h, float* direct_host, float* indirect_host,
                                float* corner_host) {
	const Lightmapper* L = reinterpret_cast<const Lightmapper*>(h);
	if (!L || !L->d_solver_direct || !L->d_bake_final) return RRG_ERR_INVALID;
	RRG_CUDA(cudaSetDevice(L->c->device));
	const size_t nt = L->c->nt;
	if (direct_host)
		RRG_CUDA(cudaMemcpy(direct_host, L->d_solver_direct, 3 * nt * sizeof(float), cudaMemcpyDeviceToHost));
	if (indirect_host) {   // E - D, as the smoothing reads it
		std::vector<float> e(3 * nt), d(3 * nt);
		RRG_CUDA(cudaMemcpy(e.data(), L->d_bake_final, 3 * nt * sizeof(float), cudaMemcpyDeviceToHost));
		RRG_CUDA(cudaMemcpy(d.data(), L->d_solver_direct, 3 * nt * sizeof(float), cudaMemcpyDeviceToHost));
		for (size_t i = 0; i < 3 * nt; i++) indirect_host[i] = e[i] - d[i];
	}
	if (corner_host)
		RRG_CUDA(cudaMemcpy(corner_host, L->d_solver_corner, 9 * nt * sizeof(float), cudaMemcpyDeviceToHost));
	return RRG_OK;
}

uint64_t rrg_lightmapper_copy_factor_hits(const rrg_lightmapper* h, uint32_t* hits_host, uint64_t cap) {
	const Lightmapper* L = reinterpret_cast<const Lightmapper*>(h);
	if (!L || !L->d_bake_hits || !L->d_bake_final) return 0;
	if (cudaSetDevice(L->c->device) != cudaSuccess) return 0;
	const uint64_t n = L->bake_hits_used;
	if (hits_host && cap >= n) {
		// ray-major on the device (ray j of triangle t at j * nt + t), triangle-major here
		std::vector<uint32_t> rm(n);
		if (cudaMemcpy(rm.data(), L->d_bake_hits, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return 0;
		const uint64_t k = L->bake_k, nt = k ? n / k : 0;
		for (uint64_t j = 0; j < k; j++)
			for (uint64_t t = 0; t < nt; t++) hits_host[t * k + j] = rm[j * nt + t];
	}
	return n;
}

int rrg_lightmap_train_samples(rrg_lightmapper* h, const rrg_gather_params* p, uint32_t stride,
                               uint32_t paths_per_texel, void* recs_dev, uint64_t cap, uint64_t* nrec_out,
                               void* stream) {
	Lightmapper* L = reinterpret_cast<Lightmapper*>(h);
	if (!L || !recs_dev || !stride || !paths_per_texel || !cap) return RRG_ERR_INVALID;
	if (p && (p->mode & RRG_GATHER_SOLVER)) return RRG_ERR_INVALID;   // plain paths only
	GatherScene g;
	int st = make_scene(L, p, g);
	if (st) return st;
	cudaStream_t s = (cudaStream_t)stream;
	const uint64_t npaths = (L->ncovered + stride - 1) / stride * paths_per_texel;
	RRG_CUDA(cudaMemsetAsync(L->d_counter, 0, 8, s));
	int grid = L->c->num_sms * 8;
	// traced deeper than the gather so that every record's window is whole
	const uint32_t window = g.max_depth;
	g.max_depth = g.max_depth + (uint32_t)(kTrainRecords - 1) < kMaxDepth ? g.max_depth + (uint32_t)(kTrainRecords - 1)
	                                                                       : kMaxDepth;
	rrg::note_launch(), k_train_paths<<<grid, 128, 0, s>>>(g, L->d_off, L->d_sub, L->d_covered, (uint32_t)L->ncovered, stride,
	                                   paths_per_texel, npaths, p->seed ^ 0x7A1Dull, reinterpret_cast<CacheRec*>(recs_dev),
	                                   cap, reinterpret_cast<unsigned long long*>(L->d_counter), L->d_status, window);
	RRG_CUDA(cudaGetLastError());
	uint64_t n = 0;
	RRG_CUDA(cudaMemcpyAsync(&n, L->d_counter, 8, cudaMemcpyDeviceToHost, s));
	RRG_CUDA(cudaStreamSynchronize(s));
	if (nrec_out) *nrec_out = n < cap ? n : cap;
	return RRG_OK;
}

int rrg_lightmap_gather_learned(rrg_lightmapper* h, rrg_cache* cache, const rrg_gather_params* p, uint64_t first,
                                uint64_t count, float* out_dev, float fallback_frac, uint64_t* nfallback,
                                void* stream) {
	Lightmapper* L = reinterpret_cast<Lightmapper*>(h);
	if (!L || !cache || !out_dev || ((uintptr_t)out_dev & 15)) return RRG_ERR_INVALID;
	if (p && (p->mode & RRG_GATHER_SOLVER)) return RRG_ERR_INVALID;   // the cache replaces the plain paths only
	GatherScene g;
	int st = make_scene(L, p, g);
	if (st) return st;
	if (first + count > L->ntexels) return RRG_ERR_INVALID;
	cudaStream_t s = (cudaStream_t)stream;
	const uint32_t Q = p->quality;
	const uint64_t chunk = (uint64_t)1 << 20;
	const uint64_t need = count < chunk ? count : chunk;
	// records and radiances hold Q samples per texel: the capacity check is
	// on both the texel count and the sample count
	if (need > L->lg_cap || need * Q > L->lg_cap_samples) {
		cudaFree(L->d_recs); cudaFree(L->d_rad); cudaFree(L->d_fb); cudaFree(L->d_fbcount);
		L->d_recs = nullptr; L->d_rad = nullptr; L->d_fb = nullptr; L->d_fbcount = nullptr;
		L->lg_cap = 0;
		L->lg_cap_samples = 0;
		RRG_CUDA(cudaMalloc(&L->d_recs, sizeof(CacheRec) * need * Q));
		RRG_CUDA(cudaMalloc(&L->d_rad, sizeof(float4) * need * Q));
		RRG_CUDA(cudaMalloc(&L->d_fb, sizeof(uint32_t) * need));
		RRG_CUDA(cudaMalloc(&L->d_fbcount, sizeof(unsigned int)));
		L->lg_cap = need;
		L->lg_cap_samples = need * Q;
	}
	const uint8_t* grid = nullptr;
	int res = 0;
	float lo[3] = {0, 0, 0}, ie[3] = {0, 0, 0};
	cache_grid(cache, &grid, &res, lo, ie);
	uint64_t total_fb = 0;
	float4* out = reinterpret_cast<float4*>(out_dev);
	for (uint64_t c0 = first; c0 < first + count; c0 += chunk) {
		const uint64_t n = (first + count - c0) < chunk ? (first + count - c0) : chunk;
		float4* oc = out + (c0 - first);
		const uint32_t sched = p->mode & 3u;
		if (sched == RRG_GATHER_WAVEFRONT || (sched == RRG_GATHER_AUTO && n >= kWfMinTexels))
			st = gather_wavefront(L, g, c0, n, oc, nullptr, s, L->d_recs);
		else
			st = launch_gather_kernel<true>(L, g, c0, n, nullptr, c0, oc, L->d_recs, s);
		if (st) return st;
		st = rrg_cache_infer(cache, L->d_recs, n * Q, reinterpret_cast<float*>(L->d_rad), stream);
		if (st) return st;
		RRG_CUDA(cudaMemsetAsync(L->d_fbcount, 0, sizeof(unsigned int), s));
		rrg::note_launch(), k_learned_reduce<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
		    L->d_off, c0, n, Q, L->d_recs, L->d_rad, oc, grid, res, lo[0], lo[1], lo[2], ie[0], ie[1], ie[2],
		    fallback_frac, grid ? L->d_fb : nullptr, L->d_fbcount);
		RRG_CUDA(cudaGetLastError());
		unsigned int nf = 0;
		if (grid) {
			RRG_CUDA(cudaMemcpyAsync(&nf, L->d_fbcount, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
			RRG_CUDA(cudaStreamSynchronize(s));
		}
		if (nf) {
			st = launch_gather_kernel<false>(L, g, 0, nf, L->d_fb, c0, oc, nullptr, s);
			if (st) return st;
		}
		total_fb += nf;
	}
	if (nfallback) *nfallback = total_fb;
	return RRG_OK;
}

int rrg_lightmapper_status(rrg_lightmapper* h, void* stream) {
	Lightmapper* L = reinterpret_cast<Lightmapper*>(h);
	if (!L) return RRG_ERR_INVALID;
	uint32_t w = 0;
	cudaStream_t s = (cudaStream_t)stream;
	RRG_CUDA(cudaMemcpyAsync(&w, L->d_status, 4, cudaMemcpyDeviceToHost, s));
	RRG_CUDA(cudaStreamSynchronize(s));
	RRG_CUDA(cudaMemsetAsync(L->d_status, 0, 4, s));
	return w ? RRG_ERR_STACK : RRG_OK;
}

}  // extern "C"
