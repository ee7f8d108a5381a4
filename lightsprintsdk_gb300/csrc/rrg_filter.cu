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
// whenever a run of samples leaves it, and later seams read what earlier
// ones wrote (on the finely tessellated atlases nearly every seam depends on
// the one before).  So it runs as one warp per atlas over the atlas's seams,
// and each seam is made cheap: its runs of samples in one texel pair are
// found once, from the geometry, and loaded a seam ahead; the used flags of
// the atlas sit in shared memory; a seam's texel values are loaded in one
// round trip; a seam of at most 32 runs whose runs read no texel it wrote
// before them sums each texel group's runs on its own four lanes, eight
// groups at a time (seam_parallel, seam_parallel_runs); any other walks its
// runs with lanes 0..7 carrying the components of the two accumulators; a
// run's repeated value is added in
// closed form per binade, so the sums are the reference's sequential float
// sums, bit for bit.
#include "rrg_internal.cuh"
#include "rrg_add_repeat.cuh"

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
	uint32_t* d_seam_off = nullptr;   // natlas + 1: each atlas's seams
	uint32_t* d_run_off = nullptr;    // nseams + 1: each seam's runs
	uint32_t* d_runs = nullptr;       // 3 words per run
	uint64_t nseams = 0, nruns = 0;
};

void filter_free(LightmapFilter* f) {
	if (!f) return;
	cudaFree(f->d_a);
	cudaFree(f->d_b);
	cudaFree(f->d_bits);
	cudaFree(f->d_chg);
	cudaFreeHost(f->h_any);
	cudaFree(f->d_seam_off);
	cudaFree(f->d_run_off);
	cudaFree(f->d_runs);
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

// Texels of sample si (0..1000) of a seam's two edges, with the reference's
// float arithmetic (RRBuffer.cpp:752-760); false where either lies outside
// the map.
__device__ __forceinline__ bool seam_sample(const Seam& e, int si, float fs, uint32_t size, uint32_t& i1,
                                            uint32_t& i2) {
	if (si < 0 || si > 1000) return false;
	const float b = __fmul_rn((float)si, 0.001f), am = __fsub_rn(1.f, b);
	const float u1x = __fadd_rn(__fmul_rn(e.e1.x, am), __fmul_rn(e.e1.z, b));
	const float u1y = __fadd_rn(__fmul_rn(e.e1.y, am), __fmul_rn(e.e1.w, b));
	const float u2x = __fadd_rn(__fmul_rn(e.e2.x, am), __fmul_rn(e.e2.z, b));
	const float u2y = __fadd_rn(__fmul_rn(e.e2.y, am), __fmul_rn(e.e2.w, b));
	if (!(u1x >= 0.f && u1x < 1.f && u1y >= 0.f && u1y < 1.f && u2x >= 0.f && u2x < 1.f && u2y >= 0.f && u2y < 1.f))
		return false;
	i1 = (unsigned)__fmul_rn(u1x, fs) + (unsigned)__fmul_rn(u1y, fs) * size;
	i2 = (unsigned)__fmul_rn(u2x, fs) + (unsigned)__fmul_rn(u2y, fs) * size;
	return true;
}

constexpr uint32_t kNoTexel = 0xFFFFFFFFu;

// The runs of each seam's samples: maximal runs of consecutive samples inside
// the map whose two texels stay the same, as (texel on edge 1, texel on
// edge 2, samples), in sample order.  They depend on the geometry only, so
// they are found once.  One warp per seam; a lane ends a run where the next
// sample leaves it.  COUNT: counts[s]; else the runs at 3 * off[s].
template <bool COUNT>
__global__ void k_seam_runs(const Seam* __restrict__ seams, uint64_t nseams, uint32_t size,
                            uint32_t* __restrict__ counts, const uint32_t* __restrict__ off,
                            uint32_t* __restrict__ runs) {
	const int lane = threadIdx.x & 31;
	const unsigned kFull = 0xFFFFFFFFu;
	const unsigned le = (2u << lane) - 1u;   // lanes <= this one (lane 31: all)
	const unsigned lt = (1u << lane) - 1u;
	const float fs = (float)size;
	for (uint64_t s = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; s < nseams;
	     s += ((uint64_t)gridDim.x * blockDim.x) >> 5) {
		const Seam e = seams[s];
		uint32_t n = 0;
		int last_start = 0;   // start of the run open at the end of the previous chunk
		for (int c0 = 0; c0 <= 1000; c0 += 32) {
			const int si = c0 + lane;
			uint32_t a1 = 0, a2 = 0, b1 = 0, b2 = 0, c1 = 0, c2 = 0;
			const bool in = seam_sample(e, si, fs, size, b1, b2);
			const bool in_prev = seam_sample(e, si - 1, fs, size, a1, a2);
			const bool in_next = seam_sample(e, si + 1, fs, size, c1, c2);
			const bool start = in && !(in_prev && a1 == b1 && a2 == b2);
			const bool end = in && !(in_next && c1 == b1 && c2 == b2);
			const unsigned S = __ballot_sync(kFull, start), E = __ballot_sync(kFull, end);
			const unsigned my_starts = S & le;
			const int st = my_starts ? c0 + 31 - __clz(my_starts) : last_start;
			if (!COUNT && end) {
				uint32_t* r = runs + 3 * ((uint64_t)off[s] + n + __popc(E & lt));
				r[0] = b1;
				r[1] = b2;
				r[2] = (uint32_t)(si - st + 1);
			}
			n += __popc(E);
			if (S) last_start = c0 + 31 - __clz(S);
		}
		if (COUNT && lane == 0) counts[s] = n;
	}
}

// Seam averaging of one pass (RRBuffer.cpp:744-786): one warp per atlas, its
// seams in order (each seam reads what the earlier ones wrote, so an atlas's
// seams are sequential).  Per seam, the lanes take 32 runs at a time: whether
// a run counts (both its texels used, alpha != 0; texels with alpha 0 are
// never written and written texels keep alpha 1, so this does not change
// during the pass) and the runs' texel values, loaded together.  Then the
// reference's walk over the runs, with lanes 0..7 each carrying one float
// component of its two accumulators (lane l: component l & 3 of accumulator
// l >> 2): where a texel's run ends, the texel gets its accumulator's
// average; a run of c samples adds its texels' sum c times, in the
// reference's order (a run's c additions in closed form, add_repeat), so
// every value is the reference's sequential float result, bit for bit.  A
// texel this seam wrote and reads again is read back from memory where the
// atlas's flags sit in shared memory (a flag per texel marks this seam's
// writes, cleared when the seam ends), else taken from a log of its writes.
constexpr int kSeamLog = 2048;                 // >= the writes of one seam (2 per run)
constexpr uint32_t kUsedSmemMax = 128 * 1024;  // used flags of atlases up to 362^2 texels in shared memory
constexpr uint8_t kUsed = 1, kWritten = 2;     // per-texel flags in shared memory: used; written by this seam

constexpr int kChains = 8;               // texel groups summed at once on the parallel path (4 lanes each)
constexpr uint32_t kParallelRuns = 32;   // runs of a seam on the parallel path (one lane each)

struct SeamLog {
	uint32_t key[kSeamLog];
	float4 val[kSeamLog];
	// the parallel path: per run its texel sum and samples; per group (seams
	// of at most kChains runs) the run that ends it, its texel and write order
	float4 run_v[kParallelRuns];
	uint32_t run_cnt[kParallelRuns];
	uint32_t chain_end[kChains], chain_tex[kChains], chain_key[kChains];
};

// Latest value this seam wrote to `key`, if any (the last of the log's n
// entries that matches).
__device__ __forceinline__ bool seam_log_find(const SeamLog& lg, unsigned n, uint32_t key, int lane, float4& out) {
	const unsigned kFull = 0xFFFFFFFFu;
	int found = -1;
	for (unsigned j0 = 0; j0 < n; j0 += 32) {
		const unsigned j = j0 + (unsigned)lane;
		const unsigned m = __ballot_sync(kFull, j < n && lg.key[j] == key);
		if (m) found = (int)(j0 + 31 - __clz(m));
	}
	if (found < 0) return false;
	out = lg.val[found];
	return true;
}

__device__ __forceinline__ float4 shfl4(float4 x, int k) {
	const unsigned kFull = 0xFFFFFFFFu;
	return make_float4(__shfl_sync(kFull, x.x, k), __shfl_sync(kFull, x.y, k), __shfl_sync(kFull, x.z, k),
	                   __shfl_sync(kFull, x.w, k));
}

__device__ __forceinline__ float comp4(const float4& x, int c) {
	return c == 0 ? x.x : (c == 1 ? x.y : (c == 2 ? x.z : x.w));
}

// One seam on the parallel path, when it has at most kChains runs; false
// (nothing written) where the seam needs the sequential walk.  In the
// reference's walk (RRBuffer.cpp:764-781) an accumulator restarts when its
// edge's texel changes, and the texel it leaves gets its average; so each
// accumulator's sums split into groups of consecutive counting runs with
// one texel, whose sums are independent of one another as long as no run
// reads a texel that this seam wrote before it.  Then every group is one
// chain of additions from zero over its runs (four lanes: one component
// each), and every group's texel is written at once, a texel that two groups
// write taking the later group's value, as in the reference's order (at a
// run boundary edge 1's texel before edge 2's).  A seam with a run that
// reads a texel written before it in the seam, or with more than kChains
// groups, goes to the sequential walk.
// Lane j < m holds run j (texels i1, i2, samples cnt).
__device__ __forceinline__ bool seam_parallel(const float4* __restrict__ img, float* __restrict__ imgf,
                                              const uint8_t* __restrict__ used, int used_in_smem, uint32_t i1,
                                              uint32_t i2, uint32_t cnt, uint32_t m, SeamLog& lg, int lane) {
	const unsigned kFull = 0xFFFFFFFFu;
	bool ok = false;
	float4 x1 = make_float4(0.f, 0.f, 0.f, 0.f), x2 = x1;
	if ((uint32_t)lane < m) {
		ok = used_in_smem ? (used[i1] & used[i2] & kUsed) != 0 : (img[i1].w != 0.f && img[i2].w != 0.f);
		if (ok) {
			x1 = img[i1];
			x2 = img[i2];
		}
	}
	const unsigned O = __ballot_sync(kFull, ok);   // counting runs
	if (!O) return true;                            // nothing is written
	// groups: a counting run starts one where its texel differs from the
	// previous counting run's, and ends one where the next counting run starts
	// one (or none follows)
	const unsigned below = O & ((1u << lane) - 1u);
	const int prev = below ? 31 - __clz(below) : lane;
	const uint32_t p1 = __shfl_sync(kFull, i1, prev), p2 = __shfl_sync(kFull, i2, prev);
	const unsigned S1 = __ballot_sync(kFull, ok && (!below || i1 != p1));
	const unsigned S2 = __ballot_sync(kFull, ok && (!below || i2 != p2));
	const unsigned above = lane < 31 ? O & ~((2u << lane) - 1u) : 0u;
	const int next = above ? __ffs(above) - 1 : -1;
	const unsigned E1 = __ballot_sync(kFull, ok && (next < 0 || ((S1 >> next) & 1u)));
	const unsigned E2 = __ballot_sync(kFull, ok && (next < 0 || ((S2 >> next) & 1u)));
	const int n1 = __popc(E1), nch = n1 + __popc(E2);
	if (nch > kChains) return false;
	if (ok)
		lg.run_v[lane] = make_float4(__fadd_rn(x1.x, x2.x), __fadd_rn(x1.y, x2.y), __fadd_rn(x1.z, x2.z),
		                             __fadd_rn(x1.w, x2.w));
	if ((uint32_t)lane < m) lg.run_cnt[lane] = cnt;
	// this lane's chain: group k (edge 1's groups first, in run order), component c
	const int k = lane >> 2, c = lane & 3;
	const bool mine = k < nch;
	const bool edge1 = k < n1;
	int end = 0, start = 0;
	if (mine) {
		unsigned E = edge1 ? E1 : E2;
		for (int t = edge1 ? k : k - n1; t > 0; t--) E &= E - 1u;
		end = __ffs(E) - 1;
		const unsigned starts = (edge1 ? S1 : S2) & ((2u << end) - 1u);   // end < kChains
		start = 31 - __clz(starts);
	}
	const uint32_t end_i1 = __shfl_sync(kFull, i1, end), end_i2 = __shfl_sync(kFull, i2, end);
	const uint32_t tex = mine ? (edge1 ? end_i1 : end_i2) : kNoTexel;
	// writes in the reference's order: group ending at run q, edge e -> 2q + e
	const uint32_t key = 2u * (uint32_t)end + (edge1 ? 0u : 1u);
	if (mine && c == 0) {
		lg.chain_end[k] = (uint32_t)end;
		lg.chain_tex[k] = tex;
		lg.chain_key[k] = key;
	}
	__syncwarp();
	// a counting run that reads a texel written before it: sequential walk
	bool dirty = false, later = false;
	for (int t = 0; t < nch; t++) {
		const uint32_t te = lg.chain_tex[t];
		if (ok && (int)lg.chain_end[t] < lane && (te == i1 || te == i2)) dirty = true;
		if (mine && lg.chain_key[t] > key && te == tex) later = true;
	}
	if (__any_sync(kFull, dirty)) return false;
	float acc = 0.f;
	if (mine) {
		uint32_t done = 0;   // additions so far: the first kPlainSteps are plain
		for (int r = start; r <= end; r++) {
			if (!((O >> r) & 1u)) continue;
			const uint32_t n = lg.run_cnt[r];
			const float v = comp4(lg.run_v[r], c);
			acc = add_repeat(acc, v, n, done < kPlainSteps ? kPlainSteps - done : 0u);
			done += n;
		}
	}
	const float w = __shfl_sync(kFull, acc, lane | 3);
	if (mine && !later) imgf[4 * (size_t)tex + c] = __fdiv_rn(acc, w);
	return true;
}

// seam_parallel for seams of kChains + 1 .. kParallelRuns runs: the same
// texel groups, summed kChains groups at a time, with the checks (a run that
// reads a texel written before it; a group's texel written again by a later
// group) made in one pass over the runs rather than over the groups, which
// is cheaper for many groups and dearer for few (seams of up to 8 runs took
// 15 % longer this way on the config-2 atlases).  False (nothing written)
// where the seam needs the sequential walk.  Lane j < m holds run j.
__device__ __forceinline__ bool seam_parallel_runs(const float4* __restrict__ img, float* __restrict__ imgf,
                                              const uint8_t* __restrict__ used, int used_in_smem, uint32_t i1,
                                              uint32_t i2, uint32_t cnt, uint32_t m, SeamLog& lg, int lane) {
	const unsigned kFull = 0xFFFFFFFFu;
	bool ok = false;
	float4 x1 = make_float4(0.f, 0.f, 0.f, 0.f), x2 = x1;
	if ((uint32_t)lane < m) {
		ok = used_in_smem ? (used[i1] & used[i2] & kUsed) != 0 : (img[i1].w != 0.f && img[i2].w != 0.f);
		if (ok) {
			x1 = img[i1];
			x2 = img[i2];
		}
	}
	const unsigned O = __ballot_sync(kFull, ok);   // counting runs
	if (!O) return true;                            // nothing is written
	// groups: a counting run starts one where its texel differs from the
	// previous counting run's, and ends one where the next counting run starts
	// one (or none follows)
	const unsigned below = O & ((1u << lane) - 1u);
	const int prev = below ? 31 - __clz(below) : lane;
	const uint32_t p1 = __shfl_sync(kFull, i1, prev), p2 = __shfl_sync(kFull, i2, prev);
	const unsigned S1 = __ballot_sync(kFull, ok && (!below || i1 != p1));
	const unsigned S2 = __ballot_sync(kFull, ok && (!below || i2 != p2));
	const unsigned above = lane < 31 ? O & ~((2u << lane) - 1u) : 0u;
	const int next = above ? __ffs(above) - 1 : -1;
	const unsigned E1 = __ballot_sync(kFull, ok && (next < 0 || ((S1 >> next) & 1u)));
	const unsigned E2 = __ballot_sync(kFull, ok && (next < 0 || ((S2 >> next) & 1u)));
	// over the runs q: whether this lane's run reads a texel that a group
	// ending before it writes (dirty), and whether the texel its edge-1 /
	// edge-2 group writes is written again by a later group (key 2q + edge)
	const bool my_e1 = (E1 >> lane) & 1u, my_e2 = (E2 >> lane) & 1u;
	bool dirty = false, later1 = false, later2 = false;
	for (uint32_t q = 0; q < m; q++) {
		const uint32_t t1 = __shfl_sync(kFull, i1, (int)q), t2 = __shfl_sync(kFull, i2, (int)q);
		const bool e1 = (E1 >> q) & 1u, e2 = (E2 >> q) & 1u;
		if ((int)q < lane)
			dirty |= ok && ((e1 && (t1 == i1 || t1 == i2)) || (e2 && (t2 == i1 || t2 == i2)));
		else if ((int)q > lane) {
			later1 |= my_e1 && ((e1 && t1 == i1) || (e2 && t2 == i1));
			later2 |= my_e2 && ((e1 && t1 == i2) || (e2 && t2 == i2));
		} else
			later1 |= my_e1 && e2 && t2 == i1;
	}
	if (__any_sync(kFull, dirty)) return false;
	const unsigned L1 = __ballot_sync(kFull, later1), L2 = __ballot_sync(kFull, later2);
	if (ok)
		lg.run_v[lane] = make_float4(__fadd_rn(x1.x, x2.x), __fadd_rn(x1.y, x2.y), __fadd_rn(x1.z, x2.z),
		                             __fadd_rn(x1.w, x2.w));
	if ((uint32_t)lane < m) lg.run_cnt[lane] = cnt;
	__syncwarp();
	const int n1 = __popc(E1), nch = n1 + __popc(E2);
	for (int base = 0; base < nch; base += kChains) {
		// this lane's group: k (edge 1's groups first, in run order), component c
		const int k = base + (lane >> 2), c = lane & 3;
		const bool mine = k < nch;
		const bool edge1 = k < n1;
		int end = 0, start = 0;
		if (mine) {
			unsigned E = edge1 ? E1 : E2;
			for (int t = edge1 ? k : k - n1; t > 0; t--) E &= E - 1u;
			end = __ffs(E) - 1;
			start = 31 - __clz((edge1 ? S1 : S2) & ((2u << end) - 1u));
		}
		const uint32_t end_i1 = __shfl_sync(kFull, i1, end), end_i2 = __shfl_sync(kFull, i2, end);
		const bool write = mine && !(((edge1 ? L1 : L2) >> end) & 1u);
		float acc = 0.f;
		if (mine) {
			uint32_t done = 0;   // additions so far: the first kPlainSteps are plain
			for (int r = start; r <= end; r++) {
				if (!((O >> r) & 1u)) continue;
				const uint32_t n = lg.run_cnt[r];
				const float v = comp4(lg.run_v[r], c);
				acc = add_repeat(acc, v, n, done < kPlainSteps ? kPlainSteps - done : 0u);
				done += n;
			}
		}
		const float w = __shfl_sync(kFull, acc, lane | 3);
		if (write) imgf[4 * (size_t)(edge1 ? end_i1 : end_i2) + c] = __fdiv_rn(acc, w);
	}
	return true;
}

__global__ void __launch_bounds__(32) k_smooth_seams(float4* __restrict__ work, const uint32_t* __restrict__ runs,
                                                     const uint32_t* __restrict__ run_off,
                                                     const uint32_t* __restrict__ seam_off, uint32_t first_atlas,
                                                     uint32_t size, int used_in_smem) {
	extern __shared__ __align__(16) unsigned char seam_smem[];
	SeamLog& lg = *reinterpret_cast<SeamLog*>(seam_smem);
	uint8_t* used = seam_smem + sizeof(SeamLog);
	const uint32_t t = blockIdx.x;   // atlas of this call
	const uint32_t a = first_atlas + t;
	const int lane = threadIdx.x;
	const unsigned kFull = 0xFFFFFFFFu;
	const uint64_t S = (uint64_t)size * size;
	float4* img = work + (uint64_t)t * S;
	float* imgf = reinterpret_cast<float*>(img);
	const int comp = lane & 3;
	const bool carrier = lane < 8;
	const bool first_acc = lane < 4;
	if (used_in_smem)
		for (uint64_t k = lane; k < S; k += 32) used[k] = img[k].w != 0.f ? kUsed : 0;
	__syncwarp();
	// A seam's run offsets and runs do not depend on texel values, so they are
	// loaded one seam ahead (the offsets two): q0..q1 are the runs of the seam
	// about to start, q2 the end of the one after, and lane j holds run j of
	// the seam about to start (the first 32).
	const uint32_t s_begin = seam_off[a], s_end = seam_off[a + 1];
	uint32_t q0 = 0, q1 = 0, q2 = 0, n1 = 0, n2 = 0, nc = 0;
	if (s_begin < s_end) {
		q0 = run_off[s_begin];
		q1 = run_off[s_begin + 1];
		q2 = s_begin + 1 < s_end ? run_off[s_begin + 2] : q1;
	}
	if (q0 + (uint32_t)lane < q1) {
		const uint32_t* r = runs + 3 * ((uint64_t)q0 + (uint32_t)lane);
		n1 = r[0];
		n2 = r[1];
		nc = r[2];
	}
	for (uint32_t s = s_begin; s < s_end; s++) {
		const uint64_t r0 = q0;
		const uint32_t m = q1 - q0;
		const uint32_t f1 = n1, f2 = n2, fc = nc;   // run `lane` of this seam
		q0 = q1;
		q1 = q2;
		if (s + 2 < s_end) q2 = run_off[s + 3];
		n1 = n2 = nc = 0;
		if (q0 + (uint32_t)lane < q1) {
			const uint32_t* r = runs + 3 * ((uint64_t)q0 + (uint32_t)lane);
			n1 = r[0];
			n2 = r[1];
			nc = r[2];
		}
		if (m <= kParallelRuns) {
			const bool done = m <= (uint32_t)kChains
			                      ? seam_parallel(img, imgf, used, used_in_smem, f1, f2, fc, m, lg, lane)
			                      : seam_parallel_runs(img, imgf, used, used_in_smem, f1, f2, fc, m, lg, lane);
			__syncwarp();
			if (done) continue;
		}
		uint32_t last1 = kNoTexel, last2 = kNoTexel;
		unsigned nlog = 0;   // the same in every lane
		float acc = 0.f, v = 0.f;
		for (uint32_t c0 = 0; c0 < m; c0 += 32) {
			const uint32_t j = c0 + (uint32_t)lane;
			bool ok = false;
			uint32_t i1 = 0, i2 = 0, cnt = 0;
			float4 x1 = make_float4(0.f, 0.f, 0.f, 0.f), x2 = x1;
			if (j < m) {
				if (c0 == 0) {
					i1 = f1;
					i2 = f2;
					cnt = fc;
				} else {
					const uint32_t* r = runs + 3 * (r0 + j);
					i1 = r[0];
					i2 = r[1];
					cnt = r[2];
				}
				ok = used_in_smem ? (used[i1] & used[i2] & kUsed) != 0 : (img[i1].w != 0.f && img[i2].w != 0.f);
				if (ok) {
					x1 = img[i1];
					x2 = img[i2];
				}
			}
			unsigned M = __ballot_sync(kFull, ok);
			while (M) {
				const int k = __ffs(M) - 1;
				M &= M - 1u;
				const uint32_t k1 = __shfl_sync(kFull, i1, k), k2 = __shfl_sync(kFull, i2, k);
				const uint32_t kc = __shfl_sync(kFull, cnt, k);
				const float4 y1 = shfl4(x1, k), y2 = shfl4(x2, k);
				const float w1 = __shfl_sync(kFull, acc, 3), w2 = __shfl_sync(kFull, acc, 7);
				bool changed = false;
				if (k1 != last1) {
					if (last1 != kNoTexel) {
						if (first_acc) {
							const float q = __fdiv_rn(acc, w1);
							imgf[4 * (size_t)last1 + comp] = q;
							if (!used_in_smem) reinterpret_cast<float*>(&lg.val[nlog])[comp] = q;
						}
						if (lane == 0) {
							lg.key[nlog] = last1;
							if (used_in_smem) used[last1] |= kWritten;
						}
						nlog++;
					}
					last1 = k1;
					if (first_acc) acc = 0.f;
					changed = true;
				}
				__syncwarp();
				if (k2 != last2) {
					if (last2 != kNoTexel) {
						if (carrier && !first_acc) {
							const float q = __fdiv_rn(acc, w2);
							imgf[4 * (size_t)last2 + comp] = q;
							if (!used_in_smem) reinterpret_cast<float*>(&lg.val[nlog])[comp] = q;
						}
						if (lane == 0) {
							lg.key[nlog] = last2;
							if (used_in_smem) used[last2] |= kWritten;
						}
						nlog++;
					}
					last2 = k2;
					if (carrier && !first_acc) acc = 0.f;
					changed = true;
				}
				__syncwarp();
				if (changed) {
					// the pair's values: this seam's writes, else as loaded
					float4 z1 = y1, z2 = y2, l;
					if (used_in_smem) {
						if (used[k1] & kWritten) z1 = img[k1];
						if (used[k2] & kWritten) z2 = img[k2];
					} else {
						if (seam_log_find(lg, nlog, k1, lane, l)) z1 = l;
						if (seam_log_find(lg, nlog, k2, lane, l)) z2 = l;
					}
					v = __fadd_rn(comp4(z1, comp), comp4(z2, comp));
				}
				if (carrier) acc = add_repeat(acc, v, kc);
			}
		}
		const float w1 = __shfl_sync(kFull, acc, 3), w2 = __shfl_sync(kFull, acc, 7);
		if (last1 != kNoTexel && first_acc) imgf[4 * (size_t)last1 + comp] = __fdiv_rn(acc, w1);
		__syncwarp();
		if (last2 != kNoTexel && carrier && !first_acc) imgf[4 * (size_t)last2 + comp] = __fdiv_rn(acc, w2);
		if (used_in_smem)
			for (unsigned j = (unsigned)lane; j < nlog; j += 32) used[lg.key[j]] &= kUsed;
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
// lightmapper: it is mesh preprocessing, O(triangles); the runs of each
// seam's samples then come from the GPU (k_seam_runs).
// Runs of all seams (k_seam_runs): offsets and runs, on the device.
static int seam_runs(LightmapFilter* F, const std::vector<Seam>& seams, uint32_t size, int num_sms) {
	struct Dev {
		void* p = nullptr;
		~Dev() { cudaFree(p); }
	} dseams, cnt;
	const uint64_t ns = seams.size();
	RRG_CUDA(cudaMalloc(&dseams.p, sizeof(Seam) * ns));
	RRG_CUDA(cudaMemcpy(dseams.p, seams.data(), sizeof(Seam) * ns, cudaMemcpyHostToDevice));
	RRG_CUDA(cudaMalloc(&cnt.p, sizeof(uint32_t) * ns));
	const int grid = (int)std::min<uint64_t>((ns * 32 + 255) / 256, (uint64_t)num_sms * 16);
	rrg::note_launch(), k_seam_runs<true><<<grid, 256>>>((const Seam*)dseams.p, ns, size, (uint32_t*)cnt.p, nullptr, nullptr);
	RRG_CUDA(cudaGetLastError());
	std::vector<uint32_t> counts(ns);
	RRG_CUDA(cudaMemcpy(counts.data(), cnt.p, sizeof(uint32_t) * ns, cudaMemcpyDeviceToHost));
	std::vector<uint32_t> off(ns + 1, 0);
	uint64_t total = 0;
	for (uint64_t k = 0; k < ns; k++) {
		total += counts[k];
		if (total >= (1ull << 32)) return RRG_ERR_TOO_LARGE;   // run offsets are 32-bit
		off[k + 1] = (uint32_t)total;
	}
	F->nruns = total;
	RRG_CUDA(cudaMalloc(&F->d_run_off, sizeof(uint32_t) * (ns + 1)));
	RRG_CUDA(cudaMemcpy(F->d_run_off, off.data(), sizeof(uint32_t) * (ns + 1), cudaMemcpyHostToDevice));
	RRG_CUDA(cudaMalloc(&F->d_runs, sizeof(uint32_t) * 3 * (off[ns] ? off[ns] : 1)));
	rrg::note_launch(), k_seam_runs<false><<<grid, 256>>>((const Seam*)dseams.p, ns, size, nullptr, F->d_run_off, F->d_runs);
	RRG_CUDA(cudaGetLastError());
	RRG_CUDA(cudaDeviceSynchronize());
	return RRG_OK;
}

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
	F->nseams = seams.size();
	RRG_CUDA(cudaMalloc(&F->d_seam_off, sizeof(uint32_t) * (natlas + 1)));
	RRG_CUDA(cudaMemcpy(F->d_seam_off, soff.data(), sizeof(uint32_t) * (natlas + 1), cudaMemcpyHostToDevice));
	if (!seams.empty()) {
		int st = seam_runs(F, seams, v.size, v.c->num_sms);
		if (st) return st;
	}
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
		const int used_in_smem = S <= kUsedSmemMax ? 1 : 0;
		const size_t seam_smem = sizeof(SeamLog) + (used_in_smem ? (size_t)S : 0);
		if (seams)
			RRG_CUDA(cudaFuncSetAttribute(k_smooth_seams, cudaFuncAttributeMaxDynamicSharedMemorySize,
			                              (int)seam_smem));
		rrg::note_launch(), k_smooth_prep<<<grid, threads, 0, s>>>(lm, F->d_a, F->d_bits, v.size, n, wrap);
		if (sigma > 10.f) sigma = 10.f;
		float sum = sigma * sigma;
		float4* src = F->d_a;
		float4* dst = F->d_b;
		while (sum > 0.f) {
			const float s2 = sum < 0.34f ? sum : 0.34f;
			// the kernel weights come from the host's expf, as the reference's do
			const float k1 = expf(-0.5f / s2), k2 = expf(-1.f / s2);
			sum -= s2;
			rrg::note_launch(), k_smooth_pass<<<grid, threads, 0, s>>>(src, dst, F->d_bits, v.size, n, k1, k2);
			if (seams)
				rrg::note_launch(), k_smooth_seams<<<natlas, 32, seam_smem, s>>>(dst, F->d_runs, F->d_run_off, F->d_seam_off, first_atlas,
				                                             v.size, used_in_smem);
			std::swap(src, dst);
		}
		rrg::note_launch(), k_smooth_store<<<grid, threads, 0, s>>>(lm, src, n);
		RRG_CUDA(cudaGetLastError());
	}
	if (p->stages & RRG_FILTER_GROW_BILINEAR) {
		RRG_CUDA(cudaMemcpyAsync(F->d_a, lm, sizeof(float4) * n, cudaMemcpyDeviceToDevice, s));
		rrg::note_launch(), k_grow_bilinear<<<grid, threads, 0, s>>>(F->d_a, lm, v.size, n, wrap);
		RRG_CUDA(cudaGetLastError());
	}
	if ((p->stages & RRG_FILTER_GROW) && p->spread_foreground) {
		rrg::note_launch(), k_grow_prep<<<grid, threads, 0, s>>>(lm, F->d_a, n);
		float4* src = F->d_a;
		float4* dst = F->d_b;
		uint32_t* chg[2] = {F->d_chg, F->d_chg + (natlas + 1)};
		for (uint32_t step = 0; step < p->spread_foreground; step++) {
			uint32_t* cur = chg[step & 1];
			const uint32_t* prev = chg[(step + 1) & 1];
			RRG_CUDA(cudaMemsetAsync(cur, 0, sizeof(uint32_t) * (natlas + 1), s));
			rrg::note_launch(), k_grow_step<<<grid, threads, 0, s>>>(src, dst, v.size, n, wrap, prev, cur, step == 0);
			std::swap(src, dst);
			// stop once a step changed nothing anywhere (checked every 8 steps)
			if ((step & 7) == 7 || step + 1 == p->spread_foreground) {
				RRG_CUDA(cudaMemcpyAsync(F->h_any, cur + natlas, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
				RRG_CUDA(cudaStreamSynchronize(s));
				if (!*F->h_any) break;
			}
		}
		rrg::note_launch(), k_grow_store<<<grid, threads, 0, s>>>(lm, src, n);
		RRG_CUDA(cudaGetLastError());
	}
	if (p->stages & RRG_FILTER_FILL_BACKGROUND) {
		rrg::note_launch(), k_fill_background<<<grid, threads, 0, s>>>(lm, n, make_float4(p->background[0], p->background[1],
		                                                              p->background[2], p->background[3]));
		RRG_CUDA(cudaGetLastError());
	}
	return RRG_OK;
}

uint64_t rrg_lightmapper_seams(const rrg_lightmapper* h) {
	LightmapView v = lightmapper_view(const_cast<rrg_lightmapper*>(h));
	return (v.filter && *v.filter) ? (*v.filter)->nseams : 0;
}

uint64_t rrg_lightmapper_seam_runs(const rrg_lightmapper* h) {
	LightmapView v = lightmapper_view(const_cast<rrg_lightmapper*>(h));
	return (v.filter && *v.filter) ? (*v.filter)->nruns : 0;
}

}  // extern "C"
