// rrg_filter.cu -- the lightmap post-filters of RRSolver::updateLightmap
// (RRSolver/lightmap.cpp:865-874) on gathered atlases in device memory,
// behind rrg_lightmap_filter (include/rrgpu_gather.h):
//
//   smooth           RRBuffer::lightmapSmooth (RRBuffer/RRBuffer.cpp:630-802):
//                    blur passes of at most 0.34 sigma^2 each over the 8
//                    neighbours the texel flags allow, then, per pass, the
//                    averaging along unwrap seams (UnwrapSeams, :534-628)
//   grow bilinear    lightmapGrowForBilinearInterpolation (:804-863)
//   grow             lightmapGrow (:865-962), ping-pong steps until nothing
//                    changes or the step budget is spent, per atlas
//   fill background  lightmapFillBackground (:964-983)
//
// Every per-texel filter is one thread per texel over all atlases of the
// call (HBM-bound stencils).  The seam pass is sequential by nature: the
// reference walks each seam's 1,001 samples in order, overwriting a texel
// whenever a run of samples leaves it, and later samples read what earlier
// runs wrote.  It runs as one warp per atlas: the 32 lanes place 32 samples
// at a time, runs of samples in the same texel pair are found with ballots,
// and lanes 0..7 each carry one float component of the two accumulators, so
// the sums are the reference's sequential float sums, bit for bit.
#include "rrg_internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/rrgpu_gather.h"

namespace rrg {

struct Seam {
	float4 e1;   // edge1[0].xy, edge1[1].xy (map space)
	float4 e2;   // edge2[0].xy, edge2[1].xy
};

struct LightmapFilter {
	float4* d_a = nullptr;
	float4* d_b = nullptr;
	uint8_t* d_bits = nullptr;        // blur-neighbour bits per texel
	uint64_t cap = 0;                 // texels
	uint32_t* d_chg = nullptr;        // grow: 2 x (atlases + 1) change flags
	uint32_t* h_any = nullptr;        // page-locked copy of the "any atlas changed" word
	uint32_t chg_cap = 0;
	bool seams_built = false;
	Seam* d_seams = nullptr;
	uint32_t* d_seam_off = nullptr;   // natlas + 1
	uint64_t nseams = 0;
};

void filter_free(LightmapFilter* f) {
	if (!f) return;
	cudaFree(f->d_a);
	cudaFree(f->d_b);
	cudaFree(f->d_bits);
	cudaFree(f->d_chg);
	cudaFreeHost(f->h_any);
	cudaFree(f->d_seams);
	cudaFree(f->d_seam_off);
	delete f;
}

// FLOAT_TO_TEXELFLAGS (RRSolver/gather.h:79)
__device__ __forceinline__ unsigned texel_flags(float a) { return (unsigned)__fadd_rn(__fmul_rn(a, 255.f), 0.5f); }

constexpr unsigned kQ00 = 1, kQ10 = 2, kQ01 = 4, kQ11 = 8, kEX0 = 16, kEX1 = 32, kEY0 = 64, kEY1 = 128;

__device__ __forceinline__ float4 f4add(float4 a, float4 b) {
	return make_float4(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z), __fadd_rn(a.w, b.w));
}
__device__ __forceinline__ float4 f4mul(float4 a, float f) {
	return make_float4(__fmul_rn(a.x, f), __fmul_rn(a.y, f), __fmul_rn(a.z, f), __fmul_rn(a.w, f));
}
__device__ __forceinline__ float4 f4div(float4 a, float f) {
	return make_float4(__fdiv_rn(a.x, f), __fdiv_rn(a.y, f), __fdiv_rn(a.z, f), __fdiv_rn(a.w, f));
}

// ------------------------------------------------------------------ smooth
// Blur bits (RRBuffer.cpp:665-699) and the working copy with alpha 0 or 1.
__global__ void k_smooth_prep(const float4* __restrict__ lm, float4* __restrict__ work, uint8_t* __restrict__ bits,
                              uint32_t size, uint64_t n, int wrap) {
	const uint64_t S = (uint64_t)size * size;
	for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
		const uint64_t base = k / S * S;
		const int i = (int)((k - base) % size), j = (int)((k - base) / size);
		const float4 c = lm[k];
		const unsigned center = texel_flags(c.w);
		unsigned bit = 1, b = 0;
		for (int jj = -1; jj < 2; jj++)
			for (int ii = -1; ii < 2; ii++)
				if (ii || jj) {
					int x = i + ii, y = j + jj;
					if (wrap) {
						x = (int)(((unsigned)x + size) % size);
						y = (int)(((unsigned)y + size) % size);
					}
					if (x >= 0 && x < (int)size && y >= 0 && y < (int)size) {
						const unsigned nb = texel_flags(lm[base + (uint64_t)y * size + x].w);
						if ((ii >= 0 || ((center & kEX0) && (nb & kEX1))) && (ii <= 0 || ((center & kEX1) && (nb & kEX0))) &&
						    (jj >= 0 || ((center & kEY0) && (nb & kEY1))) && (jj <= 0 || ((center & kEY1) && (nb & kEY0))))
							b |= bit;
					}
					bit *= 2;
				}
		bits[k] = (uint8_t)b;
		work[k] = make_float4(c.x, c.y, c.z, c.w > 0.f ? 1.f : 0.f);
	}
}

// One blur pass (RRBuffer.cpp:719-742); neighbours wrap at the atlas border
// (weight 0 where the bits forbid), as the reference indexes them.
__global__ void k_smooth_pass(const float4* __restrict__ src, float4* __restrict__ dst, const uint8_t* __restrict__ bits,
                              uint32_t size, uint64_t n, float k1, float k2) {
	const uint64_t S = (uint64_t)size * size;
	for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
		float4 c = src[k];
		if (c.w != 0.f) {
			const uint64_t base = k / S * S;
			const uint32_t i = (uint32_t)((k - base) % size), j = (uint32_t)((k - base) / size);
			const unsigned f = bits[k];
			const uint32_t im = (i - 1 + size) % size, ip = (i + 1) % size;
			const uint32_t jm = (j - 1 + size) % size, jp = (j + 1) % size;
			const float4* a = src + base;
			c = f4mul(c, 1.f);
			c = f4add(c, f4mul(a[im + jm * size], (f & 1) ? k2 : 0.f));
			c = f4add(c, f4mul(a[i + jm * size], (f & 2) ? k1 : 0.f));
			c = f4add(c, f4mul(a[ip + jm * size], (f & 4) ? k2 : 0.f));
			c = f4add(c, f4mul(a[im + j * size], (f & 8) ? k1 : 0.f));
			c = f4add(c, f4mul(a[ip + j * size], (f & 16) ? k1 : 0.f));
			c = f4add(c, f4mul(a[im + jp * size], (f & 32) ? k2 : 0.f));
			c = f4add(c, f4mul(a[i + jp * size], (f & 64) ? k1 : 0.f));
			c = f4add(c, f4mul(a[ip + jp * size], (f & 128) ? k2 : 0.f));
			c = f4div(c, c.w);
		}
		dst[k] = c;
	}
}

// Seam averaging of one pass (RRBuffer.cpp:744-786), one warp per atlas,
// seams in order.  Lane l < 8 carries component (l & 3) of accumulator
// (l >> 2) (acc1, acc2 of the reference).  Texels with alpha 0 are never
// written and written texels get alpha 1, so whether a sample counts (both
// its texels have alpha != 0) does not change during the pass and is read
// up front, 32 samples at a time.
__global__ void __launch_bounds__(32) k_smooth_seams(float4* __restrict__ work, const Seam* __restrict__ seams,
                                                     const uint32_t* __restrict__ seam_off, uint32_t first_atlas,
                                                     uint32_t size) {
	const uint32_t t = blockIdx.x;   // atlas of this call
	const uint32_t a = first_atlas + t;
	const int lane = threadIdx.x;
	const unsigned kFull = 0xFFFFFFFFu;
	const uint32_t kNone = 0xFFFFFFFFu;
	float4* img = work + (uint64_t)t * size * size;
	float* imgf = reinterpret_cast<float*>(img);
	const int comp = lane & 3;
	const bool carrier = lane < 8;
	const bool first_acc = lane < 4;
	const float fs = (float)size;
	for (uint32_t s = seam_off[a]; s < seam_off[a + 1]; s++) {
		const Seam sm = seams[s];
		uint32_t last1 = kNone, last2 = kNone;
		float acc = 0.f, v = 0.f;
		for (unsigned c0 = 0; c0 <= 1000; c0 += 32) {
			const unsigned si = c0 + (unsigned)lane;
			bool ok = false;
			uint32_t i1 = 0, i2 = 0;
			if (si <= 1000) {
				const float b = __fmul_rn((float)si, 0.001f), am = __fsub_rn(1.f, b);
				const float u1x = __fadd_rn(__fmul_rn(sm.e1.x, am), __fmul_rn(sm.e1.z, b));
				const float u1y = __fadd_rn(__fmul_rn(sm.e1.y, am), __fmul_rn(sm.e1.w, b));
				const float u2x = __fadd_rn(__fmul_rn(sm.e2.x, am), __fmul_rn(sm.e2.z, b));
				const float u2y = __fadd_rn(__fmul_rn(sm.e2.y, am), __fmul_rn(sm.e2.w, b));
				if (u1x >= 0.f && u1x < 1.f && u1y >= 0.f && u1y < 1.f && u2x >= 0.f && u2x < 1.f && u2y >= 0.f &&
				    u2y < 1.f) {
					i1 = (unsigned)__fmul_rn(u1x, fs) + (unsigned)__fmul_rn(u1y, fs) * size;
					i2 = (unsigned)__fmul_rn(u2x, fs) + (unsigned)__fmul_rn(u2y, fs) * size;
					ok = img[i1].w != 0.f && img[i2].w != 0.f;
				}
			}
			const unsigned M = __ballot_sync(kFull, ok);
			if (!M) continue;
			// previous counted sample: the nearest lower lane in M, or the
			// state carried from the earlier chunks
			const unsigned below = M & ((1u << lane) - 1u);
			const int p = below ? 31 - __clz(below) : lane;
			const uint32_t q1 = __shfl_sync(kFull, i1, p), q2 = __shfl_sync(kFull, i2, p);
			const uint32_t p1 = below ? q1 : last1, p2 = below ? q2 : last2;
			const unsigned starts = __ballot_sync(kFull, ok && (i1 != p1 || i2 != p2));
			// samples before the first run start continue the carried run
			const unsigned pre = starts ? (starts & (0u - starts)) - 1u : kFull;
			unsigned n = __popc(M & pre);
			if (carrier)
				for (unsigned r = 0; r < n; r++) acc = __fadd_rn(acc, v);
			unsigned rest = starts;
			while (rest) {
				const int k = __ffs(rest) - 1;
				rest &= rest - 1u;
				const uint32_t k1 = __shfl_sync(kFull, i1, k), k2 = __shfl_sync(kFull, i2, k);
				const float w1 = __shfl_sync(kFull, acc, 3), w2 = __shfl_sync(kFull, acc, 7);
				if (k1 != last1) {
					if (last1 != kNone && first_acc) imgf[4 * (size_t)last1 + comp] = __fdiv_rn(acc, w1);
					last1 = k1;
					if (first_acc) acc = 0.f;
				}
				__syncwarp();
				if (k2 != last2) {
					if (last2 != kNone && carrier && !first_acc) imgf[4 * (size_t)last2 + comp] = __fdiv_rn(acc, w2);
					last2 = k2;
					if (carrier && !first_acc) acc = 0.f;
				}
				__syncwarp();
				if (carrier) v = __fadd_rn(imgf[4 * (size_t)k1 + comp], imgf[4 * (size_t)k2 + comp]);
				// this run's samples in the chunk: from k up to the next start
				const unsigned upto = rest ? (rest & (0u - rest)) - 1u : kFull;
				n = __popc(M & upto & ~((1u << k) - 1u));
				if (carrier)
					for (unsigned r = 0; r < n; r++) acc = __fadd_rn(acc, v);
			}
		}
		const float w1 = __shfl_sync(kFull, acc, 3), w2 = __shfl_sync(kFull, acc, 7);
		if (last1 != kNone && first_acc) imgf[4 * (size_t)last1 + comp] = __fdiv_rn(acc, w1);
		__syncwarp();
		if (last2 != kNone && carrier && !first_acc) imgf[4 * (size_t)last2 + comp] = __fdiv_rn(acc, w2);
		__syncwarp();
	}
}

// Copy back where the smoothed texel is used, keeping the original alpha.
__global__ void k_smooth_store(float4* __restrict__ lm, const float4* __restrict__ work, uint64_t n) {
	for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
		const float4 s = work[k];
		if (s.w > 0.f) lm[k] = make_float4(s.x, s.y, s.z, lm[k].w);
	}
}

// -------------------------------------------------------------------- grow
// lightmapGrowForBilinearInterpolation (RRBuffer.cpp:804-863): an empty texel
// (alpha <= 0.002) takes the weighted mean of the neighbours whose quadrant
// flags reach towards it, with alpha 0.001.  Reads a copy taken before the
// pass: the reference writes in place, but what it writes has alpha 0.001,
// whose flags are 0, so an earlier write never counts as a neighbour and the
// order does not matter.
__global__ void k_grow_bilinear(const float4* __restrict__ in, float4* __restrict__ lm, uint32_t size, uint64_t n,
                                int wrap) {
	const uint64_t S = (uint64_t)size * size;
	for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
		if (in[k].w > 0.002f) continue;
		const uint64_t base = k / S * S;
		const int i = (int)((k - base) % size), j = (int)((k - base) / size);
		float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
		for (int jj = -1; jj < 2; jj++)
			for (int ii = -1; ii < 2; ii++) {
				int x = i + ii, y = j + jj;
				if (wrap) {
					x = (int)(((unsigned)x + size) % size);
					y = (int)(((unsigned)y + size) % size);
				} else if (x < 0 || x >= (int)size || y < 0 || y >= (int)size)
					continue;
				const float4 c = in[base + (uint64_t)y * size + x];
				const unsigned f = texel_flags(c.w);
				if ((ii < 1 && jj < 1 && (f & kQ11)) || (ii > -1 && jj > -1 && (f & kQ00)) ||
				    (ii < 1 && jj > -1 && (f & kQ10)) || (ii > -1 && jj < 1 && (f & kQ01))) {
					const float wgt = (ii && jj) ? 1.f : 1.6f;
					sum = f4add(sum, f4mul(make_float4(c.x, c.y, c.z, 1.f), wgt));
				}
			}
		if (sum.w != 0.f)
			lm[k] = make_float4(__fdiv_rn(sum.x, sum.w), __fdiv_rn(sum.y, sum.w), __fdiv_rn(sum.z, sum.w), 0.001f);
	}
}

// lightmapGrow working copy: used texels (alpha > 0) with alpha 1, others 0.
__global__ void k_grow_prep(const float4* __restrict__ lm, float4* __restrict__ work, uint64_t n) {
	for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
		const float4 c = lm[k];
		work[k] = c.w > 0.f ? make_float4(c.x, c.y, c.z, 1.f) : make_float4(0.f, 0.f, 0.f, 0.f);
	}
}

// One grow step (RRBuffer.cpp:897-945) of every atlas still growing: an
// empty texel takes the mean of its 4 edge neighbours (weight 1.6) and 4
// corner neighbours.  An atlas whose previous step changed nothing is copied
// through.  With wrap the reference indexes neighbours modulo the texel count
// in unsigned arithmetic, which this repeats.
__global__ void k_grow_step(const float4* __restrict__ src, float4* __restrict__ dst, uint32_t size, uint64_t n,
                            int wrap, const uint32_t* __restrict__ prev, uint32_t* __restrict__ cur, int first) {
	const uint64_t S = (uint64_t)size * size;
	const uint32_t nat = (uint32_t)(n / S);
	for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
		const uint32_t t = (uint32_t)(k / S);
		float4 c = src[k];
		if (c.w == 0.f && (first || prev[t])) {
			const uint64_t base = (uint64_t)t * S;
			const float4* a = src + base;
			const uint32_t sz = (uint32_t)S;
			float4 d;
			if (wrap) {
				const int i = (int)(k - base), w = (int)size;
				const float4 s4 = f4add(f4add(f4add(a[(unsigned)(i + 1) % sz], a[(unsigned)(i - 1) % sz]),
				                              a[(unsigned)(i + w) % sz]), a[(unsigned)(i - w) % sz]);
				const float4 s8 = f4add(f4add(f4add(a[(unsigned)(i + 1 + w) % sz], a[(unsigned)(i + 1 - w) % sz]),
				                              a[(unsigned)(i - 1 + w) % sz]), a[(unsigned)(i - 1 - w) % sz]);
				d = f4add(f4mul(s4, 1.6f), s8);
			} else {
				const int x = (int)((k - base) % size), y = (int)((k - base) / size), w = (int)size, h = (int)size;
				const int xp = min(x + 1, w - 1), xm = max(x - 1, 0), yp = min(y + 1, h - 1), ym = max(y - 1, 0);
				const float4 s4 = f4add(f4add(f4add(a[xp + y * w], a[xm + y * w]), a[x + yp * w]), a[x + ym * w]);
				const float4 s8 = f4add(f4add(f4add(a[xp + yp * w], a[xp + ym * w]), a[xm + yp * w]), a[xm + ym * w]);
				d = f4add(f4mul(s4, 1.6f), s8);
			}
			if (d.w != 0.f) {
				c = f4div(d, d.w);
				cur[t] = 1u;
				cur[nat] = 1u;
			}
		}
		dst[k] = c;
	}
}

// Copy back texels the growing reached (alpha 0.001), lightmapGrow's end.
__global__ void k_grow_store(float4* __restrict__ lm, const float4* __restrict__ work, uint64_t n) {
	for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
		const float4 s = work[k];
		if (s.w > 0.f && lm[k].w == 0.f) lm[k] = make_float4(s.x, s.y, s.z, 0.001f);
	}
}

// lightmapFillBackground: unused texels (alpha <= 0) get the background.
__global__ void k_fill_background(float4* __restrict__ lm, uint64_t n, float4 bg) {
	for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
		if (lm[k].w <= 0.f) lm[k] = bg;
}

// ------------------------------------------------------------------- seams
// UnwrapSeams (RRBuffer.cpp:534-628) of every atlas: for each triangle t1 of
// the atlas (ascending index) and each of its edges v1-v2, every later
// triangle t2 of the atlas sharing both vertices (found by merging the two
// vertices' ascending triangle lists, as the reference does) whose unwrap of
// the edge differs.  Vertices are shared by index (the reference first
// stitches equal positions whose normals differ by at most 1 degree, which a
// mesh with one vertex per position already is).  Host code, run once per
// lightmapper: it is mesh preprocessing, O(triangles).
static int build_seams(const LightmapView& v, LightmapFilter* F) {
	const uint32_t nt = v.nt, natlas = v.natlas;
	std::vector<uint32_t> idx(3 * (size_t)nt);
	RRG_CUDA(cudaMemcpy(idx.data(), v.c->d_idx, sizeof(uint32_t) * idx.size(), cudaMemcpyDeviceToHost));
	uint32_t nv = 0;
	for (uint32_t x : idx) nv = x + 1 > nv ? x + 1 : nv;
	// triangles of each atlas, ascending
	std::vector<uint32_t> aoff(natlas + 1, 0), tris;
	for (uint32_t t = 0; t < nt; t++)
		if (v.atlas[t] >= 0 && (uint32_t)v.atlas[t] < natlas) aoff[v.atlas[t] + 1]++;
	for (uint32_t a = 0; a < natlas; a++) aoff[a + 1] += aoff[a];
	tris.resize(aoff[natlas]);
	{
		std::vector<uint32_t> cur(aoff.begin(), aoff.end() - 1);
		for (uint32_t t = 0; t < nt; t++)
			if (v.atlas[t] >= 0 && (uint32_t)v.atlas[t] < natlas) tris[cur[v.atlas[t]]++] = t;
	}
	std::vector<uint32_t> cnt(nv + 1, 0), start(nv, 0), fill(nv, 0), touched, tiv;
	std::vector<Seam> seams;
	std::vector<uint32_t> soff(natlas + 1, 0);
	for (uint32_t a = 0; a < natlas; a++) {
		const uint32_t* T = tris.data() + aoff[a];
		const uint32_t n = aoff[a + 1] - aoff[a];
		touched.clear();
		for (uint32_t l = 0; l < n; l++)
			for (int c = 0; c < 3; c++) {
				const uint32_t vi = idx[3 * (size_t)T[l] + c];
				if (!cnt[vi]++) touched.push_back(vi);
			}
		uint32_t run = 0;
		for (uint32_t vi : touched) {
			start[vi] = run;
			run += cnt[vi];
		}
		tiv.resize(run);
		for (uint32_t l = 0; l < n; l++)
			for (int c = 0; c < 3; c++) {
				const uint32_t vi = idx[3 * (size_t)T[l] + c];
				tiv[start[vi] + fill[vi]++] = l;
			}
		for (uint32_t l1 = 0; l1 < n; l1++) {
			const uint32_t* tv1 = idx.data() + 3 * (size_t)T[l1];
			const float* uv1 = v.uv + 6 * (size_t)T[l1];
			for (unsigned e = 0; e < 3; e++) {
				const uint32_t v1 = tv1[e], v2 = tv1[(e + 1) % 3];
				const float* a0 = uv1 + 2 * e;
				const float* a1 = uv1 + 2 * ((e + 1) % 3);
				const uint32_t* L1 = tiv.data() + start[v1];
				const uint32_t* L2 = tiv.data() + start[v2];
				const uint32_t n1 = cnt[v1], n2 = cnt[v2];
				uint32_t i1 = 0;
				for (uint32_t i2 = 0; i2 < n2; i2++)
					if (L2[i2] > l1) {
						while (i1 + 1 < n1 && L1[i1] < L2[i2]) i1++;
						if (L1[i1] != L2[i2]) continue;
						const uint32_t t2 = T[L2[i2]];
						const uint32_t* tv2 = idx.data() + 3 * (size_t)t2;
						const unsigned c1 = (tv2[0] == v1) ? 0 : ((tv2[1] == v1) ? 1 : 2);
						const unsigned c2 = (tv2[0] == v2) ? 0 : ((tv2[1] == v2) ? 1 : 2);
						const float* b0 = v.uv + 6 * (size_t)t2 + 2 * c1;
						const float* b1 = v.uv + 6 * (size_t)t2 + 2 * c2;
						if (a0[0] != b0[0] || a0[1] != b0[1] || a1[0] != b1[0] || a1[1] != b1[1])
							seams.push_back(Seam{make_float4(a0[0], a0[1], a1[0], a1[1]),
							                     make_float4(b0[0], b0[1], b1[0], b1[1])});
					}
			}
		}
		for (uint32_t vi : touched) cnt[vi] = fill[vi] = 0;
		soff[a + 1] = (uint32_t)seams.size();
	}
	RRG_CUDA(cudaMalloc(&F->d_seam_off, sizeof(uint32_t) * (natlas + 1)));
	RRG_CUDA(cudaMemcpy(F->d_seam_off, soff.data(), sizeof(uint32_t) * (natlas + 1), cudaMemcpyHostToDevice));
	RRG_CUDA(cudaMalloc(&F->d_seams, sizeof(Seam) * (seams.size() ? seams.size() : 1)));
	if (!seams.empty())
		RRG_CUDA(cudaMemcpy(F->d_seams, seams.data(), sizeof(Seam) * seams.size(), cudaMemcpyHostToDevice));
	F->nseams = seams.size();
	F->seams_built = true;
	return RRG_OK;
}

static int reserve(LightmapFilter* F, uint64_t texels, uint32_t natlas) {
	if (texels > F->cap) {
		cudaFree(F->d_a);
		cudaFree(F->d_b);
		cudaFree(F->d_bits);
		F->d_a = F->d_b = nullptr;
		F->d_bits = nullptr;
		F->cap = 0;
		RRG_CUDA(cudaMalloc(&F->d_a, sizeof(float4) * texels));
		RRG_CUDA(cudaMalloc(&F->d_b, sizeof(float4) * texels));
		RRG_CUDA(cudaMalloc(&F->d_bits, texels));
		F->cap = texels;
	}
	if (natlas + 1 > F->chg_cap) {
		cudaFree(F->d_chg);
		F->d_chg = nullptr;
		F->chg_cap = 0;
		RRG_CUDA(cudaMalloc(&F->d_chg, sizeof(uint32_t) * 2 * (natlas + 1)));
		F->chg_cap = natlas + 1;
	}
	if (!F->h_any) RRG_CUDA(cudaHostAlloc(&F->h_any, sizeof(uint32_t), cudaHostAllocDefault));
	return RRG_OK;
}

}  // namespace rrg

using namespace rrg;

extern "C" {

void rrg_filter_defaults(rrg_filter_params* p) {
	if (!p) return;
	memset(p, 0, sizeof(*p));
	p->size = sizeof(*p);
	p->stages = RRG_FILTER_ALL;
	p->smoothing_amount = 1.f;
	p->spread_foreground = 1000;
	p->seams = 1;
}

int rrg_lightmap_filter(rrg_lightmapper* h, const rrg_filter_params* p, uint32_t first_atlas, uint32_t natlas,
                        float* lightmaps_dev, void* stream) {
	LightmapView v = lightmapper_view(h);
	if (!v.c || !p || p->size != sizeof(rrg_filter_params) || !lightmaps_dev || ((uintptr_t)lightmaps_dev & 15))
		return RRG_ERR_INVALID;
	if (first_atlas > v.natlas || natlas > v.natlas - first_atlas) return RRG_ERR_INVALID;
	if (!(p->smoothing_amount == p->smoothing_amount)) return RRG_ERR_INVALID;
	if (!natlas) return RRG_OK;
	RRG_CUDA(cudaSetDevice(v.c->device));
	if (!*v.filter) {
		*v.filter = new (std::nothrow) LightmapFilter();
		if (!*v.filter) return RRG_ERR_OOM;
	}
	LightmapFilter* F = *v.filter;
	const uint64_t S = (uint64_t)v.size * v.size, n = S * natlas;
	int st = reserve(F, n, natlas);
	if (st) return st;
	cudaStream_t s = (cudaStream_t)stream;
	float4* lm = reinterpret_cast<float4*>(lightmaps_dev) + (uint64_t)first_atlas * S;
	const int threads = 256;
	const int grid = (int)std::min<uint64_t>((n + threads - 1) / threads, (uint64_t)v.c->num_sms * 16);
	const int wrap = p->wrap ? 1 : 0;

	// lightmapSmooth: sigma < 0 or 0 does nothing; at most 10
	float sigma = p->smoothing_amount;
	if ((p->stages & RRG_FILTER_SMOOTH) && sigma > 0.f) {
		if (p->seams && !F->seams_built) {
			st = build_seams(v, F);
			if (st) return st;
		}
		const bool seams = p->seams && F->nseams;
		k_smooth_prep<<<grid, threads, 0, s>>>(lm, F->d_a, F->d_bits, v.size, n, wrap);
		if (sigma > 10.f) sigma = 10.f;
		float sum = sigma * sigma;
		float4* src = F->d_a;
		float4* dst = F->d_b;
		while (sum > 0.f) {
			const float s2 = sum < 0.34f ? sum : 0.34f;
			// the kernel weights come from the host's expf, as the reference's do
			const float k1 = expf(-0.5f / s2), k2 = expf(-1.f / s2);
			sum -= s2;
			k_smooth_pass<<<grid, threads, 0, s>>>(src, dst, F->d_bits, v.size, n, k1, k2);
			if (seams) k_smooth_seams<<<natlas, 32, 0, s>>>(dst, F->d_seams, F->d_seam_off, first_atlas, v.size);
			std::swap(src, dst);
		}
		k_smooth_store<<<grid, threads, 0, s>>>(lm, src, n);
		RRG_CUDA(cudaGetLastError());
	}
	if (p->stages & RRG_FILTER_GROW_BILINEAR) {
		RRG_CUDA(cudaMemcpyAsync(F->d_a, lm, sizeof(float4) * n, cudaMemcpyDeviceToDevice, s));
		k_grow_bilinear<<<grid, threads, 0, s>>>(F->d_a, lm, v.size, n, wrap);
		RRG_CUDA(cudaGetLastError());
	}
	if ((p->stages & RRG_FILTER_GROW) && p->spread_foreground) {
		k_grow_prep<<<grid, threads, 0, s>>>(lm, F->d_a, n);
		float4* src = F->d_a;
		float4* dst = F->d_b;
		uint32_t* chg[2] = {F->d_chg, F->d_chg + (natlas + 1)};
		for (uint32_t step = 0; step < p->spread_foreground; step++) {
			uint32_t* cur = chg[step & 1];
			const uint32_t* prev = chg[(step + 1) & 1];
			RRG_CUDA(cudaMemsetAsync(cur, 0, sizeof(uint32_t) * (natlas + 1), s));
			k_grow_step<<<grid, threads, 0, s>>>(src, dst, v.size, n, wrap, prev, cur, step == 0);
			std::swap(src, dst);
			// stop once a step changed nothing anywhere (checked every 8 steps)
			if ((step & 7) == 7 || step + 1 == p->spread_foreground) {
				RRG_CUDA(cudaMemcpyAsync(F->h_any, cur + natlas, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
				RRG_CUDA(cudaStreamSynchronize(s));
				if (!*F->h_any) break;
			}
		}
		k_grow_store<<<grid, threads, 0, s>>>(lm, src, n);
		RRG_CUDA(cudaGetLastError());
	}
	if (p->stages & RRG_FILTER_FILL_BACKGROUND) {
		k_fill_background<<<grid, threads, 0, s>>>(lm, n, make_float4(p->background[0], p->background[1],
		                                                              p->background[2], p->background[3]));
		RRG_CUDA(cudaGetLastError());
	}
	return RRG_OK;
}

uint64_t rrg_lightmapper_seams(const rrg_lightmapper* h) {
	LightmapView v = lightmapper_view(const_cast<rrg_lightmapper*>(h));
	return (v.filter && *v.filter) ? (*v.filter)->nseams : 0;
}

}  // extern "C"
