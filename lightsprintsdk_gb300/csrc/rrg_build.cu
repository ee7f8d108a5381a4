// GPU binned-SAH BVH build for the collider.
//
// Replaces the reference's single-threaded BSP/kd builder
// (RRCollider/bsp.cpp:388-1192) with a top-down binned SAH build that runs
// entirely on the device:
//   1. prep     : per triangle, the FASTEST validity rule (finite unit normal,
//                 RRCollider/IntersectBspFast.cpp:178-186), its AABB;
//   2. compact  : valid triangle ids in index order (device-wide scan);
//   3. large    : level-synchronous splitting of tasks > kSmall triangles,
//                 each task spread over CTAs of kChunk triangles that bin
//                 centroids (kBins per axis) into shared memory and merge into
//                 per-task global bins; one CTA per task evaluates the SAH; a
//                 stable chunked partition writes the children's ranges;
//   4. small    : one CTA builds the whole subtree of each task of <= kSmall
//                 triangles in shared memory (smaller child first, so the
//                 pending stack stays <= log2(kSmall) deep);
//   5. emit     : binary traversal nodes with both child boxes in the parent,
//                 and the triangles copied into leaf order.
// Depth is bounded: below depth kMedianDepth splits fall back to the object
// median, so the tree is never deeper than kStackSize-1 and traversal stacks
// cannot overflow on valid input.
#include "rrg_internal.cuh"

#include <new>

#include <vector>

namespace rrg {

constexpr int kBins = 32;
constexpr int kChunk = 2048;
constexpr int kSmall = 2048;
constexpr int kBT = 256;            // build threads per CTA
constexpr int kBinInts = 13;        // count, lo[3], hi[3], clo[3], chi[3]
constexpr int kAxisInts = kBins * kBinInts;
constexpr int kTaskBinInts = 3 * kAxisInts;
constexpr int kMedianDepth = 32;
constexpr float kCt = 1.0f;         // SAH traversal cost (triangle test = 1)

__device__ __forceinline__ int f2o(float f) {
	int i = __float_as_int(f);
	return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float o2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF); }

struct Task {
	int node, begin, count, depth;
	float cmin[3], cmax[3];
	int buf;                   // which ids buffer holds the range
	int chunk_base, nchunks;   // large path only
};

struct Split {
	int axis;        // -1 = object median by position
	int bin;         // left = bin <= this
	int nleft;
	float cmin, scale;
};

struct Chunk {
	int task, begin, count;
};

struct BuildState {
	int node_count;
	int nlarge_next;
	int nsmall;
	int nchunks;
	int error;
	int ntasks;     // large tasks of the current level (the graph-replayed build)
	int pad[2];
};

// ------------------------------------------------------------------ prep
// FASTEST unit normal with one rounding per operation, as
// TriangleSRLNP::setGeometry computes it (IntersectBspFast.cpp:130-187).
__device__ __forceinline__ bool fastest_normal_finite(float3 a, float3 b, float3 c) {
	float r0 = __fsub_rn(b.x, a.x), r1 = __fsub_rn(b.y, a.y), r2 = __fsub_rn(b.z, a.z);
	float l0 = __fsub_rn(c.x, a.x), l1 = __fsub_rn(c.y, a.y), l2 = __fsub_rn(c.z, a.z);
	float nx = __fsub_rn(__fmul_rn(r1, l2), __fmul_rn(r2, l1));
	float ny = __fadd_rn(__fmul_rn(-r0, l2), __fmul_rn(r2, l0));
	float nz = __fsub_rn(__fmul_rn(r0, l1), __fmul_rn(r1, l0));
	float sz = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)), __fmul_rn(nz, nz)));
	float x = __fdiv_rn(nx, sz), y = __fdiv_rn(ny, sz), z = __fdiv_rn(nz, sz);
	return isfinite(x) && isfinite(y) && isfinite(z);
}

__global__ void k_prep(const float* __restrict__ xyz, uint32_t nv, const uint32_t* __restrict__ idx, uint32_t nt,
                       float4* __restrict__ plo, float4* __restrict__ phi, uint32_t* __restrict__ valid,
                       BuildState* st) {
	uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= nt) return;
	uint32_t i0 = idx[3 * t], i1 = idx[3 * t + 1], i2 = idx[3 * t + 2];
	if (i0 >= nv || i1 >= nv || i2 >= nv) {
		atomicOr(&st->error, 1);
		valid[t] = 0;
		return;
	}
	float3 a = make_float3(xyz[3 * i0], xyz[3 * i0 + 1], xyz[3 * i0 + 2]);
	float3 b = make_float3(xyz[3 * i1], xyz[3 * i1 + 1], xyz[3 * i1 + 2]);
	float3 c = make_float3(xyz[3 * i2], xyz[3 * i2 + 1], xyz[3 * i2 + 2]);
	bool ok = isfinite(a.x) && isfinite(a.y) && isfinite(a.z) && isfinite(b.x) && isfinite(b.y) && isfinite(b.z) &&
	          isfinite(c.x) && isfinite(c.y) && isfinite(c.z) && fastest_normal_finite(a, b, c);
	valid[t] = ok ? 1u : 0u;
	plo[t] = make_float4(fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z)), 0.f);
	phi[t] = make_float4(fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z)), 0.f);
}

// AABB of all vertices (RRMesh::getAABB), as ordered ints
__global__ void k_vertex_aabb(const float* __restrict__ xyz, uint32_t nv, int* __restrict__ rb) {
	float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x)
		for (int k = 0; k < 3; k++) {
			float v = xyz[3 * (size_t)i + k];
			if (v < lo[k]) lo[k] = v;   // NaN never compares: skipped, as getAABB's comparisons skip it
			if (v > hi[k]) hi[k] = v;
		}
	for (int k = 0; k < 3; k++) {
		float a = lo[k], b = hi[k];
		for (int o = 16; o; o >>= 1) {
			a = fminf(a, __shfl_xor_sync(0xFFFFFFFFu, a, o));
			b = fmaxf(b, __shfl_xor_sync(0xFFFFFFFFu, b, o));
		}
		if ((threadIdx.x & 31) == 0) {
			atomicMin(&rb[k], f2o(a));
			atomicMax(&rb[3 + k], f2o(b));
		}
	}
}

// ------------------------------------------------------------ compaction
constexpr int kScanItems = 1024;   // flags per scan block (256 threads x 4)

__global__ void k_block_count(const uint32_t* __restrict__ flags, uint32_t n, uint32_t* __restrict__ bsum) {
	__shared__ uint32_t ws[kBT / 32];
	uint32_t base = blockIdx.x * kScanItems;
	uint32_t c = 0;
	for (int k = 0; k < kScanItems / kBT; k++) {
		uint32_t i = base + k * kBT + threadIdx.x;
		if (i < n) c += flags[i];
	}
	for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
	if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
	__syncthreads();
	if (threadIdx.x == 0) {
		uint32_t s = 0;
		for (int w = 0; w < kBT / 32; w++) s += ws[w];
		bsum[blockIdx.x] = s;
	}
}

// exclusive scan of nb block sums by one CTA; total -> *total
__global__ void k_scan_blocks(uint32_t* __restrict__ bsum, uint32_t nb, uint32_t* __restrict__ total) {
	__shared__ uint32_t carry;
	__shared__ uint32_t ws[kBT / 32];
	if (threadIdx.x == 0) carry = 0;
	__syncthreads();
	for (uint32_t base = 0; base < nb; base += kBT) {
		uint32_t i = base + threadIdx.x;
		uint32_t v = i < nb ? bsum[i] : 0;
		uint32_t x = v;
		int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
		for (int o = 1; o < 32; o <<= 1) {
			uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
			if (lane >= o) x += y;
		}
		if (lane == 31) ws[w] = x;
		__syncthreads();
		uint32_t wo = 0;
		for (int k = 0; k < w; k++) wo += ws[k];
		uint32_t incl = x + wo + carry;
		if (i < nb) bsum[i] = incl - v;
		__syncthreads();
		if (threadIdx.x == kBT - 1) carry = incl;
		__syncthreads();
	}
	if (threadIdx.x == 0) *total = carry;
}

__global__ void k_compact(const uint32_t* __restrict__ flags, uint32_t n, const uint32_t* __restrict__ boff,
                          int* __restrict__ ids) {
	__shared__ uint32_t ws[kBT / 32];
	__shared__ uint32_t carry;
	if (threadIdx.x == 0) carry = boff[blockIdx.x];
	__syncthreads();
	uint32_t base = blockIdx.x * kScanItems;
	int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
	for (int k = 0; k < kScanItems / kBT; k++) {
		uint32_t i = base + k * kBT + threadIdx.x;
		uint32_t f = i < n ? flags[i] : 0;
		uint32_t m = __ballot_sync(0xFFFFFFFFu, f);
		uint32_t r = __popc(m & ((1u << lane) - 1));
		if (lane == 0) ws[w] = __popc(m);
		__syncthreads();
		uint32_t wo = 0, tot = 0;
		for (int q = 0; q < kBT / 32; q++) {
			if (q < w) wo += ws[q];
			tot += ws[q];
		}
		if (f) ids[carry + wo + r] = (int)i;
		__syncthreads();
		if (threadIdx.x == 0) carry += tot;
		__syncthreads();
	}
}

// ------------------------------------------------------------ root stats
__global__ void k_root_bounds(const int* __restrict__ ids, uint32_t n, const float4* __restrict__ plo,
                              const float4* __restrict__ phi, int* __restrict__ rb) {
	// rb: lo[3], hi[3], clo[3], chi[3] as ordered ints
	float v[12];
	for (int k = 0; k < 3; k++) {
		v[k] = INFINITY; v[3 + k] = -INFINITY; v[6 + k] = INFINITY; v[9 + k] = -INFINITY;
	}
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		int t = ids[i];
		float4 lo = plo[t], hi = phi[t];
		float l[3] = {lo.x, lo.y, lo.z}, h[3] = {hi.x, hi.y, hi.z};
		for (int k = 0; k < 3; k++) {
			float c = 0.5f * (l[k] + h[k]);
			v[k] = fminf(v[k], l[k]);
			v[3 + k] = fmaxf(v[3 + k], h[k]);
			v[6 + k] = fminf(v[6 + k], c);
			v[9 + k] = fmaxf(v[9 + k], c);
		}
	}
	for (int k = 0; k < 12; k++) {
		bool mx = (k >= 3 && k < 6) || k >= 9;
		float x = v[k];
		for (int o = 16; o; o >>= 1) {
			float y = __shfl_xor_sync(0xFFFFFFFFu, x, o);
			x = mx ? fmaxf(x, y) : fminf(x, y);
		}
		if ((threadIdx.x & 31) == 0) {
			if (mx) atomicMax(&rb[k], f2o(x));
			else atomicMin(&rb[k], f2o(x));
		}
	}
}

__global__ void k_root_init(const int* __restrict__ rb, uint32_t n, BNode* nodes, Task* large, Task* small,
                            BuildState* st) {
	BNode r;
	for (int k = 0; k < 3; k++) { r.lo[k] = o2f(rb[k]); r.hi[k] = o2f(rb[3 + k]); }
	r.left = r.right = -1;
	r.begin = 0;
	r.count = (int)n;
	nodes[0] = r;
	Task t;
	t.node = 0; t.begin = 0; t.count = (int)n; t.depth = 0; t.buf = 0;
	t.chunk_base = 0; t.nchunks = 0;
	for (int k = 0; k < 3; k++) { t.cmin[k] = o2f(rb[6 + k]); t.cmax[k] = o2f(rb[9 + k]); }
	st->node_count = 1;
	if ((int)n > kSmall) {
		large[0] = t;
		st->nlarge_next = 1;
		st->nsmall = 0;
	} else {
		small[0] = t;
		st->nlarge_next = 0;
		st->nsmall = 1;
	}
}

// ------------------------------------------------------ batches of meshes
// A batch builds one tree per mesh in the same level loop: mesh m's root is
// node m, its triangles occupy positions [pos[m], pos[m+1]) of the
// compacted id list (ids ascend, so each mesh's valid triangles are
// contiguous there), and its subtree never mixes with another mesh's.

// pos[m] = first position in the ascending id list holding a triangle id
// >= tri_off[m] (m = 0..nroots).
// n_dev (may be null): read n there instead (the graph-replayed build, where
// the count of valid triangles stays on the device).  The same holds for the
// n_dev / ntasks_dev / nnodes_dev arguments of the kernels below.
__global__ void k_mesh_ranges(const int* __restrict__ ids, uint32_t n, const uint32_t* __restrict__ tri_off,
                              uint32_t nroots, uint32_t* __restrict__ pos, const uint32_t* n_dev = nullptr) {
	uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
	if (m > nroots) return;
	if (n_dev) n = *n_dev;
	const int key = (int)tri_off[m];
	uint32_t lo = 0, hi = n;
	while (lo < hi) {
		uint32_t mid = (lo + hi) >> 1;
		if (ids[mid] < key) lo = mid + 1;
		else hi = mid;
	}
	pos[m] = lo;
}

// rb[12 m ..] = identities of (lo[3] min, hi[3] max, clo[3] min, chi[3] max)
__global__ void k_fill_root_bounds(int* __restrict__ rb, uint32_t nroots) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= 12 * nroots) return;
	const int k = (int)(i % 12);
	const bool mx = (k >= 3 && k < 6) || k >= 9;
	rb[i] = mx ? f2o(-INFINITY) : f2o(INFINITY);
}

// Per-mesh root bounds and centroid bounds.  A warp covers 32 consecutive
// positions; when they all belong to one mesh (the usual case) it reduces
// in registers and issues one atomic per field.
__global__ void k_root_bounds_multi(const int* __restrict__ ids, uint32_t n, const float4* __restrict__ plo,
                                    const float4* __restrict__ phi, const uint32_t* __restrict__ pos,
                                    uint32_t nroots, int* __restrict__ rb, const uint32_t* n_dev = nullptr) {
	const int lane = threadIdx.x & 31;
	if (n_dev) n = *n_dev;
	const uint32_t stride = gridDim.x * blockDim.x;
	for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < n; base += stride) {
		const uint32_t i = base + lane;
		const bool ok = i < n;
		float v[12];
		for (int k = 0; k < 3; k++) {
			v[k] = INFINITY; v[3 + k] = -INFINITY; v[6 + k] = INFINITY; v[9 + k] = -INFINITY;
		}
		int m = -1;
		if (ok) {
			m = (int)segment_of(pos, nroots, i);
			const int t = ids[i];
			float4 lo = plo[t], hi = phi[t];
			float l[3] = {lo.x, lo.y, lo.z}, h[3] = {hi.x, hi.y, hi.z};
			for (int k = 0; k < 3; k++) {
				float c = 0.5f * (l[k] + h[k]);
				v[k] = l[k]; v[3 + k] = h[k]; v[6 + k] = c; v[9 + k] = c;
			}
		}
		const int m0 = __shfl_sync(0xFFFFFFFFu, m, 0);
		const bool uniform = __all_sync(0xFFFFFFFFu, !ok || m == m0);
		for (int k = 0; k < 12; k++) {
			const bool mx = (k >= 3 && k < 6) || k >= 9;
			float x = v[k];
			if (uniform) {
				for (int o = 16; o; o >>= 1) {
					float y = __shfl_xor_sync(0xFFFFFFFFu, x, o);
					x = mx ? fmaxf(x, y) : fminf(x, y);
				}
				if (lane == 0) {
					if (mx) atomicMax(&rb[12 * m0 + k], f2o(x));
					else atomicMin(&rb[12 * m0 + k], f2o(x));
				}
			} else if (ok) {
				if (mx) atomicMax(&rb[12 * m + k], f2o(x));
				else atomicMin(&rb[12 * m + k], f2o(x));
			}
		}
	}
}

// Root node m and its task (large or small list) for every non-empty mesh.
__global__ void k_root_init_multi(const int* __restrict__ rb, const uint32_t* __restrict__ pos, uint32_t nroots,
                                  BNode* nodes, Task* large, Task* small, BuildState* st) {
	uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
	if (m == 0) st->node_count = (int)nroots;
	if (m >= nroots) return;
	const int* b = rb + 12 * m;
	BNode r;
	for (int k = 0; k < 3; k++) { r.lo[k] = o2f(b[k]); r.hi[k] = o2f(b[3 + k]); }
	r.left = r.right = -1;
	r.begin = (int)pos[m];
	r.count = (int)(pos[m + 1] - pos[m]);
	nodes[m] = r;
	if (r.count == 0) return;
	Task t;
	t.node = (int)m; t.begin = r.begin; t.count = r.count; t.depth = 0; t.buf = 0;
	t.chunk_base = 0; t.nchunks = 0;
	for (int k = 0; k < 3; k++) { t.cmin[k] = o2f(b[6 + k]); t.cmax[k] = o2f(b[9 + k]); }
	if (t.count > kSmall) large[atomicAdd(&st->nlarge_next, 1)] = t;
	else small[atomicAdd(&st->nsmall, 1)] = t;
}

// Globalises a batch's per-mesh vertex indices: idx of mesh m's triangles
// += vert_off[m]; an index outside its mesh's vertices becomes 0xFFFFFFFF,
// which the build reports as invalid input.
__global__ void k_globalize_indices(uint32_t* __restrict__ idx, uint32_t nt, const uint32_t* __restrict__ tri_off,
                                    const uint32_t* __restrict__ vert_off, uint32_t nroots) {
	uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= nt) return;
	const uint32_t m = segment_of(tri_off, nroots, t);
	const uint32_t nvm = vert_off[m + 1] - vert_off[m];
	for (int k = 0; k < 3; k++) {
		uint32_t v = idx[3 * t + k];
		idx[3 * t + k] = v < nvm ? v + vert_off[m] : 0xFFFFFFFFu;
	}
}

int globalize_batch_indices(Collider* c, const uint32_t* d_vert_off, cudaStream_t s) {
	rrg::note_launch(), k_globalize_indices<<<(c->nt + 255) / 256, 256, 0, s>>>(c->d_idx, c->nt, c->d_tri_off, d_vert_off, c->nroots);
	RRG_CUDA(cudaGetLastError());
	return RRG_OK;
}

// Scene pad of the node boxes: 2^-20 of the largest root coordinate (empty
// meshes skipped).
__global__ void k_root_pad(const BNode* __restrict__ bn, uint32_t nroots, float* __restrict__ pad) {
	__shared__ float red[32];
	float mx = 0.f;
	for (uint32_t m = threadIdx.x; m < nroots; m += blockDim.x) {
		const BNode r = bn[m];
		if (r.left < 0 && r.count == 0) continue;
		for (int k = 0; k < 3; k++) mx = fmaxf(mx, fmaxf(fabsf(r.lo[k]), fabsf(r.hi[k])));
	}
	for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, o));
	if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
	__syncthreads();
	if (threadIdx.x == 0) {
		for (int w = 1; w < (int)(blockDim.x >> 5); w++) mx = fmaxf(mx, red[w]);
		*pad = mx * 9.5367431640625e-07f + 1e-30f;
	}
}

// --------------------------------------------------------- shared binning
__device__ __forceinline__ void bins_clear(int* b, int n_ints) {
	for (int i = threadIdx.x; i < n_ints; i += blockDim.x) {
		int f = i % kBinInts;
		int v;
		if (f == 0) v = 0;
		else if ((f >= 1 && f <= 3) || (f >= 7 && f <= 9)) v = f2o(INFINITY);
		else v = f2o(-INFINITY);
		b[i] = v;
	}
}

__device__ __forceinline__ int bin_of(float c, float cmin, float scale) {
	int q = (int)((c - cmin) * scale);
	return q < 0 ? 0 : (q >= kBins ? kBins - 1 : q);
}

// Bins one primitive into shared bins for the axes with positive extent.
__device__ __forceinline__ void bin_prim(int* sb, float4 lo, float4 hi, const float* cmin, const float* scale) {
	float l[3] = {lo.x, lo.y, lo.z}, h[3] = {hi.x, hi.y, hi.z};
	float c[3] = {0.5f * (l[0] + h[0]), 0.5f * (l[1] + h[1]), 0.5f * (l[2] + h[2])};
	for (int a = 0; a < 3; a++) {
		if (!(scale[a] > 0)) continue;
		int* b = sb + a * kAxisInts + bin_of(c[a], cmin[a], scale[a]) * kBinInts;
		atomicAdd(&b[0], 1);
		for (int k = 0; k < 3; k++) {
			atomicMin(&b[1 + k], f2o(l[k]));
			atomicMax(&b[4 + k], f2o(h[k]));
			atomicMin(&b[7 + k], f2o(c[k]));
			atomicMax(&b[10 + k], f2o(c[k]));
		}
	}
}

__device__ __forceinline__ float half_area(const float* lo, const float* hi) {
	float e0 = hi[0] - lo[0], e1 = hi[1] - lo[1], e2 = hi[2] - lo[2];
	if (!(e0 >= 0.f)) return 0.f;
	return e0 * e1 + e1 * e2 + e2 * e0;
}

struct Decision {
	int axis, bin;      // axis -1: no binned split available
	float cost;         // unnormalised sum A_L N_L + A_R N_R
};

// SAH sweep by warp `a` (< 3) over the bins of axis a; lane q = bin q.
// Writes the best (cost, bin) of the axis to out[a].
__device__ void sah_axis(const int* sb, int a, bool usable, Decision* out) {
	int lane = threadIdx.x & 31;
	const int* b = sb + a * kAxisInts + lane * kBinInts;
	int cnt = usable ? b[0] : 0;
	float lo[3], hi[3];
	for (int k = 0; k < 3; k++) {
		lo[k] = cnt ? o2f(b[1 + k]) : INFINITY;
		hi[k] = cnt ? o2f(b[4 + k]) : -INFINITY;
	}
	// inclusive prefix from the left
	int lc = cnt;
	float llo[3] = {lo[0], lo[1], lo[2]}, lhi[3] = {hi[0], hi[1], hi[2]};
	for (int o = 1; o < 32; o <<= 1) {
		int yc = __shfl_up_sync(0xFFFFFFFFu, lc, o);
		float ylo[3], yhi[3];
		for (int k = 0; k < 3; k++) {
			ylo[k] = __shfl_up_sync(0xFFFFFFFFu, llo[k], o);
			yhi[k] = __shfl_up_sync(0xFFFFFFFFu, lhi[k], o);
		}
		if (lane >= o) {
			lc += yc;
			for (int k = 0; k < 3; k++) { llo[k] = fminf(llo[k], ylo[k]); lhi[k] = fmaxf(lhi[k], yhi[k]); }
		}
	}
	// inclusive suffix from the right
	int rc = cnt;
	float rlo[3] = {lo[0], lo[1], lo[2]}, rhi[3] = {hi[0], hi[1], hi[2]};
	for (int o = 1; o < 32; o <<= 1) {
		int yc = __shfl_down_sync(0xFFFFFFFFu, rc, o);
		float ylo[3], yhi[3];
		for (int k = 0; k < 3; k++) {
			ylo[k] = __shfl_down_sync(0xFFFFFFFFu, rlo[k], o);
			yhi[k] = __shfl_down_sync(0xFFFFFFFFu, rhi[k], o);
		}
		if (lane + o < 32) {
			rc += yc;
			for (int k = 0; k < 3; k++) { rlo[k] = fminf(rlo[k], ylo[k]); rhi[k] = fmaxf(rhi[k], yhi[k]); }
		}
	}
	// split after bin `lane`: left = prefix(lane), right = suffix(lane+1)
	int nrc = __shfl_down_sync(0xFFFFFFFFu, rc, 1);
	float nrlo[3], nrhi[3];
	for (int k = 0; k < 3; k++) {
		nrlo[k] = __shfl_down_sync(0xFFFFFFFFu, rlo[k], 1);
		nrhi[k] = __shfl_down_sync(0xFFFFFFFFu, rhi[k], 1);
	}
	float cost = INFINITY;
	if (usable && lane < 31 && lc > 0 && nrc > 0)
		cost = half_area(llo, lhi) * (float)lc + half_area(nrlo, nrhi) * (float)nrc;
	int best = lane;
	for (int o = 16; o; o >>= 1) {
		float oc = __shfl_xor_sync(0xFFFFFFFFu, cost, o);
		int ob = __shfl_xor_sync(0xFFFFFFFFu, best, o);
		if (oc < cost || (oc == cost && ob < best)) { cost = oc; best = ob; }
	}
	if (lane == 0) { out[a].axis = isfinite(cost) ? a : -1; out[a].bin = best; out[a].cost = cost; }
}

// union of bins [q0, q1] of axis a: box, centroid box, count
__device__ void bins_union(const int* sb, int a, int q0, int q1, float* lo, float* hi, float* clo, float* chi, int* cnt) {
	*cnt = 0;
	for (int k = 0; k < 3; k++) { lo[k] = INFINITY; hi[k] = -INFINITY; clo[k] = INFINITY; chi[k] = -INFINITY; }
	for (int q = q0; q <= q1; q++) {
		const int* b = sb + a * kAxisInts + q * kBinInts;
		if (!b[0]) continue;
		*cnt += b[0];
		for (int k = 0; k < 3; k++) {
			lo[k] = fminf(lo[k], o2f(b[1 + k]));
			hi[k] = fmaxf(hi[k], o2f(b[4 + k]));
			clo[k] = fminf(clo[k], o2f(b[7 + k]));
			chi[k] = fmaxf(chi[k], o2f(b[10 + k]));
		}
	}
}

__device__ __forceinline__ void axis_scales(const Task& t, float* scale) {
	for (int a = 0; a < 3; a++) {
		float e = t.cmax[a] - t.cmin[a];
		scale[a] = (e > 0.f && isfinite(e)) ? (float)kBins / e : 0.f;
	}
}

// ------------------------------------------------------------ large path
__global__ void k_level_setup(Task* tasks, int ntasks, int* __restrict__ gbins, Chunk* chunks, BuildState* st,
                              const int* ntasks_dev = nullptr) {
	__shared__ int base;
	if (ntasks_dev) ntasks = *ntasks_dev;
	for (int ti = blockIdx.x; ti < ntasks; ti += gridDim.x) {
		bins_clear(gbins + (size_t)ti * kTaskBinInts, kTaskBinInts);
		Task t = tasks[ti];
		int nc = (t.count + kChunk - 1) / kChunk;
		if (threadIdx.x == 0) {
			base = atomicAdd(&st->nchunks, nc);
			tasks[ti].chunk_base = base;
			tasks[ti].nchunks = nc;
		}
		__syncthreads();
		for (int k = threadIdx.x; k < nc; k += blockDim.x) {
			Chunk c;
			c.task = ti;
			c.begin = t.begin + k * kChunk;
			c.count = min(kChunk, t.begin + t.count - c.begin);
			chunks[base + k] = c;
		}
		__syncthreads();
	}
}

__global__ void __launch_bounds__(kBT) k_bin_chunks(const Task* __restrict__ tasks, const Chunk* __restrict__ chunks,
                                                    const BuildState* st, int* const* ids_bufs,
                                                    const float4* __restrict__ plo, const float4* __restrict__ phi,
                                                    int* __restrict__ gbins) {
	__shared__ int sb[kTaskBinInts];
	int nchunks = st->nchunks;
	for (int ci = blockIdx.x; ci < nchunks; ci += gridDim.x) {
		Chunk c = chunks[ci];
		Task t = tasks[c.task];
		float scale[3];
		axis_scales(t, scale);
		bins_clear(sb, kTaskBinInts);
		__syncthreads();
		const int* ids = ids_bufs[t.buf];
		for (int i = threadIdx.x; i < c.count; i += blockDim.x) {
			int p = ids[c.begin + i];
			bin_prim(sb, plo[p], phi[p], t.cmin, scale);
		}
		__syncthreads();
		int* gb = gbins + (size_t)c.task * kTaskBinInts;
		for (int i = threadIdx.x; i < kTaskBinInts; i += blockDim.x) {
			int bin = i / kBinInts, f = i % kBinInts;
			if (!sb[bin * kBinInts]) continue;
			if (f == 0) atomicAdd(&gb[i], sb[i]);
			else if ((f >= 1 && f <= 3) || (f >= 7 && f <= 9)) atomicMin(&gb[i], sb[i]);
			else atomicMax(&gb[i], sb[i]);
		}
		__syncthreads();
	}
}

// Creates a child task (large list or small list) and its node box.
__device__ void emit_child(int node, int begin, int count, int depth, int buf, const float* lo, const float* hi,
                           const float* clo, const float* chi, BNode* nodes, Task* next_large, Task* small,
                           BuildState* st) {
	BNode n;
	for (int k = 0; k < 3; k++) { n.lo[k] = lo[k]; n.hi[k] = hi[k]; }
	n.left = n.right = -1;
	n.begin = begin;
	n.count = count;
	nodes[node] = n;
	Task t;
	t.node = node; t.begin = begin; t.count = count; t.depth = depth; t.buf = buf;
	t.chunk_base = 0; t.nchunks = 0;
	for (int k = 0; k < 3; k++) { t.cmin[k] = clo[k]; t.cmax[k] = chi[k]; }
	if (count > kSmall) next_large[atomicAdd(&st->nlarge_next, 1)] = t;
	else small[atomicAdd(&st->nsmall, 1)] = t;
}

// One CTA (>= 96 threads) per large task: SAH decision, children.
__global__ void k_decide_large(const Task* __restrict__ tasks, int ntasks, const int* __restrict__ gbins,
                               Split* __restrict__ splits, BNode* nodes, Task* next_large, Task* small,
                               BuildState* st, const int* ntasks_dev = nullptr) {
	__shared__ int sb[kTaskBinInts];
	__shared__ Decision dec[3];
	if (ntasks_dev) ntasks = *ntasks_dev;
	for (int ti = blockIdx.x; ti < ntasks; ti += gridDim.x) {
		Task t = tasks[ti];
		const int* gb = gbins + (size_t)ti * kTaskBinInts;
		for (int i = threadIdx.x; i < kTaskBinInts; i += blockDim.x) sb[i] = gb[i];
		__syncthreads();
		float scale[3];
		axis_scales(t, scale);
		int w = threadIdx.x >> 5;
		if (w < 3) sah_axis(sb, w, scale[w] > 0 && t.depth < kMedianDepth, dec);
		__syncthreads();
		if (threadIdx.x == 0) {
			int ba = -1;
			float bc = INFINITY;
			for (int a = 0; a < 3; a++)
				if (dec[a].axis >= 0 && dec[a].cost < bc) { bc = dec[a].cost; ba = a; }
			const BNode& me = nodes[t.node];
			Split sp;
			float llo[3], lhi[3], lclo[3], lchi[3], rlo[3], rhi[3], rclo[3], rchi[3];
			int nl, nr;
			if (ba >= 0) {
				sp.axis = ba;
				sp.bin = dec[ba].bin;
				sp.cmin = t.cmin[ba];
				sp.scale = scale[ba];
				bins_union(sb, ba, 0, sp.bin, llo, lhi, lclo, lchi, &nl);
				bins_union(sb, ba, sp.bin + 1, kBins - 1, rlo, rhi, rclo, rchi, &nr);
			} else {
				sp.axis = -1; sp.bin = 0; sp.cmin = 0; sp.scale = 0;
				nl = t.count / 2;
				nr = t.count - nl;
				for (int k = 0; k < 3; k++) {
					llo[k] = rlo[k] = me.lo[k];
					lhi[k] = rhi[k] = me.hi[k];
					lclo[k] = rclo[k] = t.cmin[k];
					lchi[k] = rchi[k] = t.cmax[k];
				}
			}
			sp.nleft = nl;
			splits[ti] = sp;
			int c0 = atomicAdd(&st->node_count, 2);
			nodes[t.node].left = c0;
			nodes[t.node].right = c0 + 1;
			int nb = t.buf ^ 1;
			emit_child(c0, t.begin, nl, t.depth + 1, nb, llo, lhi, lclo, lchi, nodes, next_large, small, st);
			emit_child(c0 + 1, t.begin + nl, nr, t.depth + 1, nb, rlo, rhi, rclo, rchi, nodes, next_large, small, st);
		}
		__syncthreads();
	}
}

__device__ __forceinline__ bool goes_left(const Split& sp, int pos_in_task, float4 lo, float4 hi) {
	if (sp.axis < 0) return pos_in_task < sp.nleft;
	float l = sp.axis == 0 ? lo.x : (sp.axis == 1 ? lo.y : lo.z);
	float h = sp.axis == 0 ? hi.x : (sp.axis == 1 ? hi.y : hi.z);
	return bin_of(0.5f * (l + h), sp.cmin, sp.scale) <= sp.bin;
}

__global__ void k_part_count(const Task* __restrict__ tasks, const Chunk* __restrict__ chunks, const BuildState* st,
                             const Split* __restrict__ splits, int* const* ids_bufs, const float4* __restrict__ plo,
                             const float4* __restrict__ phi, int* __restrict__ chunk_left) {
	__shared__ int ws[kBT / 32];
	int nchunks = st->nchunks;
	for (int ci = blockIdx.x; ci < nchunks; ci += gridDim.x) {
		Chunk c = chunks[ci];
		Task t = tasks[c.task];
		Split sp = splits[c.task];
		const int* ids = ids_bufs[t.buf];
		int cnt = 0;
		for (int i = threadIdx.x; i < c.count; i += blockDim.x) {
			int p = ids[c.begin + i];
			cnt += goes_left(sp, c.begin + i - t.begin, plo[p], phi[p]) ? 1 : 0;
		}
		for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(0xFFFFFFFFu, cnt, o);
		if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = cnt;
		__syncthreads();
		if (threadIdx.x == 0) {
			int s = 0;
			for (int w = 0; w < kBT / 32; w++) s += ws[w];
			chunk_left[ci] = s;
		}
		__syncthreads();
	}
}

// per task: exclusive scan of its chunks' left counts (chunks of a task are
// contiguous and in range order)
__global__ void k_part_scan(const Task* __restrict__ tasks, int ntasks, int* __restrict__ chunk_left,
                            const int* ntasks_dev = nullptr) {
	int ti = blockIdx.x * blockDim.x + threadIdx.x;
	if (ntasks_dev) ntasks = *ntasks_dev;
	if (ti >= ntasks) return;
	Task t = tasks[ti];
	int s = 0;
	for (int k = 0; k < t.nchunks; k++) {
		int v = chunk_left[t.chunk_base + k];
		chunk_left[t.chunk_base + k] = s;
		s += v;
	}
}

__global__ void __launch_bounds__(kBT) k_part_scatter(const Task* __restrict__ tasks, const Chunk* __restrict__ chunks,
                                                      const BuildState* st, const Split* __restrict__ splits,
                                                      int* const* ids_bufs, const float4* __restrict__ plo,
                                                      const float4* __restrict__ phi,
                                                      const int* __restrict__ chunk_left, BuildState* stw) {
	__shared__ int ws[kBT / 32];
	__shared__ int lcar, rcar;
	int nchunks = st->nchunks;
	int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
	for (int ci = blockIdx.x; ci < nchunks; ci += gridDim.x) {
		Chunk c = chunks[ci];
		Task t = tasks[c.task];
		Split sp = splits[c.task];
		const int* in = ids_bufs[t.buf];
		int* out = ids_bufs[t.buf ^ 1];
		if (threadIdx.x == 0) {
			lcar = chunk_left[ci];
			rcar = (c.begin - t.begin) - chunk_left[ci];
		}
		__syncthreads();
		for (int b0 = 0; b0 < c.count; b0 += kBT) {
			int i = b0 + threadIdx.x;
			bool act = i < c.count;
			int p = act ? in[c.begin + i] : 0;
			bool left = act && goes_left(sp, c.begin + i - t.begin, plo[p], phi[p]);
			unsigned m = __ballot_sync(0xFFFFFFFFu, left);
			if (lane == 0) ws[w] = __popc(m);
			__syncthreads();
			int wo = 0, tot = 0;
			for (int q = 0; q < kBT / 32; q++) {
				if (q < w) wo += ws[q];
				tot += ws[q];
			}
			int lrank = wo + __popc(m & ((1u << lane) - 1));
			int before = (w * 32 + lane);      // items before me in this block round
			int rrank = before - lrank;
			if (act) {
				int dst = left ? lcar + lrank : sp.nleft + rcar + rrank;
				if (dst >= 0 && dst < t.count) out[t.begin + dst] = p;
				else atomicOr(&stw->error, 4);
			}
			__syncthreads();
			if (threadIdx.x == 0) {
				int nact = min(kBT, c.count - b0);
				lcar += tot;
				rcar += nact - tot;
			}
			__syncthreads();
		}
	}
}

// ------------------------------------------------------------ small path
struct SubTask {
	int node, begin, count, depth, buf;
	float cmin[3], cmax[3];
};

constexpr int kSmallThreads = 128;
constexpr int kPend = 16;   // pending stack: smaller child first => <= log2(kSmall)+1

__global__ void __launch_bounds__(kSmallThreads) k_small(const Task* __restrict__ tasks, const BuildState* st,
                                                         int* const* ids_bufs, const float4* __restrict__ plo,
                                                         const float4* __restrict__ phi, BNode* nodes,
                                                         int* __restrict__ final_ids, int max_leaf,
                                                         BuildState* stw) {
	__shared__ int ids[2][kSmall];
	__shared__ int sb[kTaskBinInts];
	__shared__ SubTask pend[kPend];
	__shared__ int npend;
	__shared__ SubTask cur;
	__shared__ Decision dec[3];
	__shared__ int ws[kSmallThreads / 32];
	__shared__ int split_axis, split_bin, split_nl, leaf_flag, lcar, rcar, have;
	__shared__ float split_cmin, split_scale;
	int nsmall = st->nsmall;
	int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
	for (int ti = blockIdx.x; ti < nsmall; ti += gridDim.x) {
		Task t = tasks[ti];
		if (t.count > kSmall || t.count < 1) {
			if (threadIdx.x == 0) atomicOr(&stw->error, 8);
			continue;
		}
		const int* src = ids_bufs[t.buf];
		for (int i = threadIdx.x; i < t.count; i += blockDim.x) ids[0][i] = src[t.begin + i];
		if (threadIdx.x == 0) {
			SubTask s;
			s.node = t.node; s.begin = 0; s.count = t.count; s.depth = t.depth; s.buf = 0;
			for (int k = 0; k < 3; k++) { s.cmin[k] = t.cmin[k]; s.cmax[k] = t.cmax[k]; }
			pend[0] = s;
			npend = 1;
		}
		__syncthreads();
		while (true) {
			if (threadIdx.x == 0) {
				have = npend > 0;
				if (have) cur = pend[--npend];
			}
			__syncthreads();
			if (!have) break;
			SubTask s = cur;
			float scale[3];
			for (int a = 0; a < 3; a++) {
				float e = s.cmax[a] - s.cmin[a];
				scale[a] = (e > 0.f && isfinite(e)) ? (float)kBins / e : 0.f;
			}
			bool can_bin = s.count > 1 && s.depth < kMedianDepth;
			if (can_bin) {
				bins_clear(sb, kTaskBinInts);
				__syncthreads();
				for (int i = threadIdx.x; i < s.count; i += blockDim.x) {
					int p = ids[s.buf][s.begin + i];
					bin_prim(sb, plo[p], phi[p], s.cmin, scale);
				}
				__syncthreads();
				if (w < 3) sah_axis(sb, w, scale[w] > 0, dec);
				__syncthreads();
			}
			if (threadIdx.x == 0) {
				const BNode& me = nodes[s.node];
				float area = half_area(me.lo, me.hi);
				int ba = -1;
				float bc = INFINITY;
				if (can_bin)
					for (int a = 0; a < 3; a++)
						if (dec[a].axis >= 0 && dec[a].cost < bc) { bc = dec[a].cost; ba = a; }
				float leaf_cost = (float)s.count;
				float split_cost = area > 0.f ? kCt + bc / area : INFINITY;
				int leaf = s.count <= 1 || (s.count <= max_leaf && (ba < 0 || leaf_cost <= split_cost));
				leaf_flag = leaf;
				if (!leaf) {
					float llo[3], lhi[3], lclo[3], lchi[3], rlo[3], rhi[3], rclo[3], rchi[3];
					int nl, nr;
					if (ba >= 0) {
						split_axis = ba;
						split_bin = dec[ba].bin;
						split_cmin = s.cmin[ba];
						split_scale = scale[ba];
						bins_union(sb, ba, 0, split_bin, llo, lhi, lclo, lchi, &nl);
						bins_union(sb, ba, split_bin + 1, kBins - 1, rlo, rhi, rclo, rchi, &nr);
					} else {
						split_axis = -1; split_bin = 0; split_cmin = 0; split_scale = 0;
						nl = s.count / 2;
						nr = s.count - nl;
						for (int k = 0; k < 3; k++) {
							llo[k] = rlo[k] = me.lo[k];
							lhi[k] = rhi[k] = me.hi[k];
							lclo[k] = rclo[k] = s.cmin[k];
							lchi[k] = rchi[k] = s.cmax[k];
						}
					}
					split_nl = nl;
					int c0 = atomicAdd(&stw->node_count, 2);
					nodes[s.node].left = c0;
					nodes[s.node].right = c0 + 1;
					BNode L, R;
					for (int k = 0; k < 3; k++) { L.lo[k] = llo[k]; L.hi[k] = lhi[k]; R.lo[k] = rlo[k]; R.hi[k] = rhi[k]; }
					L.left = L.right = R.left = R.right = -1;
					L.begin = t.begin + s.begin; L.count = nl;
					R.begin = t.begin + s.begin + nl; R.count = nr;
					nodes[c0] = L;
					nodes[c0 + 1] = R;
					SubTask a, b;
					a.node = c0; a.begin = s.begin; a.count = nl; a.depth = s.depth + 1; a.buf = s.buf ^ 1;
					b.node = c0 + 1; b.begin = s.begin + nl; b.count = nr; b.depth = s.depth + 1; b.buf = s.buf ^ 1;
					for (int k = 0; k < 3; k++) {
						a.cmin[k] = lclo[k]; a.cmax[k] = lchi[k];
						b.cmin[k] = rclo[k]; b.cmax[k] = rchi[k];
					}
					// larger child deeper in the stack: the smaller is processed next
					if (npend + 2 > kPend) {
						atomicOr(&stw->error, 2);
						npend = 0;
					} else if (nl <= nr) {
						pend[npend++] = b;
						pend[npend++] = a;
					} else {
						pend[npend++] = a;
						pend[npend++] = b;
					}
					lcar = 0;
					rcar = 0;
				} else {
					nodes[s.node].left = -1;
					nodes[s.node].right = -1;
					nodes[s.node].begin = t.begin + s.begin;
					nodes[s.node].count = s.count;
				}
			}
			__syncthreads();
			if (leaf_flag) {
				for (int i = threadIdx.x; i < s.count; i += blockDim.x)
					final_ids[t.begin + s.begin + i] = ids[s.buf][s.begin + i];
			} else {
				Split sp;
				sp.axis = split_axis; sp.bin = split_bin; sp.nleft = split_nl; sp.cmin = split_cmin; sp.scale = split_scale;
				const int* in = ids[s.buf];
				int* out = ids[s.buf ^ 1];
				for (int b0 = 0; b0 < s.count; b0 += blockDim.x) {
					int i = b0 + threadIdx.x;
					bool act = i < s.count;
					int p = act ? in[s.begin + i] : 0;
					bool left = act && goes_left(sp, i, plo[p], phi[p]);
					unsigned m = __ballot_sync(0xFFFFFFFFu, left);
					if (lane == 0) ws[w] = __popc(m);
					__syncthreads();
					int wo = 0, tot = 0;
					for (int q = 0; q < kSmallThreads / 32; q++) {
						if (q < w) wo += ws[q];
						tot += ws[q];
					}
					int lrank = wo + __popc(m & ((1u << lane) - 1));
					int rrank = (w * 32 + lane) - lrank;
					if (act) {
						int dst = left ? lcar + lrank : sp.nleft + rcar + rrank;
						if (dst >= 0 && dst < s.count) out[s.begin + dst] = p;
						else atomicOr(&stw->error, 4);
					}
					__syncthreads();
					if (threadIdx.x == 0) {
						int nact = min((int)blockDim.x, s.count - b0);
						lcar += tot;
						rcar += nact - tot;
					}
					__syncthreads();
				}
			}
			__syncthreads();
		}
		__syncthreads();
	}
}

// ------------------------------------------------------------------ emit
// Child boxes are widened by 2^-20 of each coordinate's magnitude plus
// 2^-20 of the scene's largest coordinate, so that a ray lying exactly on a
// box face (an axis-aligned ray with a zero direction component, common in
// architectural scenes) still enters the box and reaches triangles on its
// boundary.
__device__ __forceinline__ void widen(BNode& n, float pad) {
	for (int k = 0; k < 3; k++) {
		n.lo[k] = n.lo[k] - (fabsf(n.lo[k]) * 9.5367431640625e-07f + pad);
		n.hi[k] = n.hi[k] + (fabsf(n.hi[k]) * 9.5367431640625e-07f + pad);
	}
}

__global__ void k_emit_nodes(const BNode* __restrict__ bn, int nnodes, int nroots, const float* __restrict__ pad_ptr,
                             TNode* __restrict__ tn, const int* nnodes_dev = nullptr) {
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (nnodes_dev) nnodes = *nnodes_dev;
	if (i >= nnodes) return;
	BNode n = bn[i];
	const float pad = *pad_ptr;
	TNode o;
	if (n.left < 0) {
		if (i >= nroots) return;   // leaves live in their parent's child refs
		if (n.count == 0) {        // a mesh without valid triangles
			o.a = make_float4(INFINITY, -INFINITY, INFINITY, -INFINITY);
			o.b = o.a;
			o.c = o.a;
			o.d = make_int4(kEmptyRef, kEmptyRef, 0, 0);
			tn[i] = o;
			return;
		}
		// a root that is a leaf: wrap it in a one-child inner node
		widen(n, pad);
		o.a = make_float4(n.lo[0], n.hi[0], n.lo[1], n.hi[1]);
		o.b = make_float4(INFINITY, -INFINITY, INFINITY, -INFINITY);
		o.c = make_float4(n.lo[2], n.hi[2], INFINITY, -INFINITY);
		o.d = make_int4(leaf_ref(n.begin, n.count), kEmptyRef, 0, 0);
		tn[i] = o;
		return;
	}
	if (n.left >= nnodes || n.right >= nnodes) return;
	BNode l = bn[n.left], r = bn[n.right];
	const int lleft = l.left, rleft = r.left;
	widen(l, pad);
	widen(r, pad);
	o.a = make_float4(l.lo[0], l.hi[0], l.lo[1], l.hi[1]);
	o.b = make_float4(r.lo[0], r.hi[0], r.lo[1], r.hi[1]);
	o.c = make_float4(l.lo[2], l.hi[2], r.lo[2], r.hi[2]);
	int r0 = lleft < 0 ? leaf_ref(l.begin, l.count) : n.left;
	int r1 = rleft < 0 ? leaf_ref(r.begin, r.count) : n.right;
	o.d = make_int4(r0, r1, 0, 0);
	tn[i] = o;
}

__global__ void k_emit_tris(const int* __restrict__ final_ids, uint32_t n, const float* __restrict__ xyz,
                            const uint32_t* __restrict__ idx, float4* __restrict__ tris, const uint32_t* n_dev = nullptr) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (n_dev) n = *n_dev;
	if (i >= n) return;
	int t = final_ids[i];
	uint32_t i0 = idx[3 * t], i1 = idx[3 * t + 1], i2 = idx[3 * t + 2];
	tris[3 * i] = make_float4(xyz[3 * i0], xyz[3 * i0 + 1], xyz[3 * i0 + 2], __int_as_float(t));
	tris[3 * i + 1] = make_float4(xyz[3 * i1], xyz[3 * i1 + 1], xyz[3 * i1 + 2], 0.f);
	tris[3 * i + 2] = make_float4(xyz[3 * i2], xyz[3 * i2 + 1], xyz[3 * i2 + 2], 0.f);
}

// ------------------------------------------------------------------ host
template <class T>
static cudaError_t dalloc(T** p, size_t n) {
	return cudaMalloc((void**)p, sizeof(T) * (n ? n : 1));
}

struct Scratch {
	std::vector<void*> ptrs;
	~Scratch() {
		for (void* p : ptrs) cudaFree(p);
	}
	template <class T>
	cudaError_t get(T** p, size_t n) {
		cudaError_t e = dalloc(p, n);
		if (e == cudaSuccess) ptrs.push_back(*p);
		return e;
	}
};

int build_bvh(Collider* c, cudaStream_t s, const volatile int* aborting) {
	const uint32_t nt = c->nt;
	int max_leaf = c->params.max_leaf_size ? (int)c->params.max_leaf_size : 4;
	if (max_leaf > kMaxLeaf) max_leaf = kMaxLeaf;
	if (max_leaf < 1) max_leaf = 1;
	cudaEvent_t e0, e1;
	RRG_CUDA(cudaEventCreate(&e0));
	RRG_CUDA(cudaEventCreate(&e1));
	RRG_CUDA(cudaEventRecord(e0, s));

	Scratch sc;
	float4 *plo, *phi;
	uint32_t *valid, *bsum, *total;
	int *idsA, *idsB, *final_ids, *rb;
	BuildState* st;
	RRG_CUDA(sc.get(&plo, nt));
	RRG_CUDA(sc.get(&phi, nt));
	RRG_CUDA(sc.get(&valid, nt));
	uint32_t nb = (nt + kScanItems - 1) / kScanItems;
	RRG_CUDA(sc.get(&bsum, nb));
	RRG_CUDA(sc.get(&total, 1));
	RRG_CUDA(sc.get(&st, 1));
	RRG_CUDA(sc.get(&rb, 12));
	RRG_CUDA(cudaMemsetAsync(st, 0, sizeof(BuildState), s));

	rrg::note_launch(), k_prep<<<(nt + 255) / 256, 256, 0, s>>>(c->d_xyz, c->nv, c->d_idx, nt, plo, phi, valid, st);
	rrg::note_launch(), k_block_count<<<nb, kBT, 0, s>>>(valid, nt, bsum);
	rrg::note_launch(), k_scan_blocks<<<1, kBT, 0, s>>>(bsum, nb, total);
	RRG_CUDA(cudaGetLastError());
	uint32_t nvalid = 0;
	BuildState hst;
	RRG_CUDA(cudaMemcpyAsync(&nvalid, total, 4, cudaMemcpyDeviceToHost, s));
	RRG_CUDA(cudaMemcpyAsync(&hst, st, sizeof(hst), cudaMemcpyDeviceToHost, s));
	RRG_CUDA(cudaStreamSynchronize(s));
	if (hst.error & 1) return RRG_ERR_INVALID;
	if (nvalid == 0) return RRG_ERR_EMPTY;
	if (nvalid >= (1u << 27)) return RRG_ERR_INVALID;   // leaf refs address 2^27 slots
	c->nvalid = nvalid;

	RRG_CUDA(sc.get(&idsA, nvalid));
	RRG_CUDA(sc.get(&idsB, nvalid));
	RRG_CUDA(sc.get(&final_ids, nvalid));
	rrg::note_launch(), k_compact<<<nb, kBT, 0, s>>>(valid, nt, bsum, idsA);

	const uint32_t nroots = c->d_tri_off ? c->nroots : 1;
	const int max_nodes = 2 * (int)nvalid + (int)nroots;
	BNode* bnodes;
	RRG_CUDA(sc.get(&bnodes, max_nodes));
	// task lists: large tasks per level <= nvalid / kSmall * 2, small <= nvalid
	const int max_large = 2 * ((int)nvalid / kSmall + 2);
	const int max_chunks = (int)nvalid / kChunk + max_large + 2;
	const int max_small = (int)nvalid / 1 + 2;
	Task *largeA, *largeB, *small;
	Split* splits;
	Chunk* chunks;
	int *gbins, *chunk_left;
	RRG_CUDA(sc.get(&largeA, max_large));
	RRG_CUDA(sc.get(&largeB, max_large));
	RRG_CUDA(sc.get(&small, max_small < (int)nvalid ? max_small : (int)nvalid + 2));
	RRG_CUDA(sc.get(&splits, max_large));
	RRG_CUDA(sc.get(&chunks, max_chunks));
	RRG_CUDA(sc.get(&chunk_left, max_chunks));
	RRG_CUDA(sc.get(&gbins, (size_t)max_large * kTaskBinInts));
	int** ids_bufs;
	RRG_CUDA(sc.get(&ids_bufs, 2));
	int* hbufs[2] = {idsA, idsB};
	RRG_CUDA(cudaMemcpyAsync(ids_bufs, hbufs, sizeof(hbufs), cudaMemcpyHostToDevice, s));

	int rb_init[12];
	{
		// ordered-int encodings of +inf (mins) and -inf (maxs)
		float pinf = INFINITY, ninf = -INFINITY;
		int ip, in;
		memcpy(&ip, &pinf, 4);
		memcpy(&in, &ninf, 4);
		in ^= 0x7FFFFFFF;
		for (int k = 0; k < 3; k++) { rb_init[k] = ip; rb_init[3 + k] = in; rb_init[6 + k] = ip; rb_init[9 + k] = in; }
	}
	RRG_CUDA(cudaMemcpyAsync(rb, rb_init, sizeof(rb_init), cudaMemcpyHostToDevice, s));
	{
		int vgrid = (int)((c->nv + 255) / 256);
		if (vgrid > 4 * 152) vgrid = 4 * 152;
		rrg::note_launch(), k_vertex_aabb<<<vgrid, 256, 0, s>>>(c->d_xyz, c->nv, rb);
		int hb[6];
		RRG_CUDA(cudaMemcpyAsync(hb, rb, sizeof(hb), cudaMemcpyDeviceToHost, s));
		RRG_CUDA(cudaStreamSynchronize(s));
		for (int k = 0; k < 3; k++) {
			int lo = hb[k] >= 0 ? hb[k] : hb[k] ^ 0x7FFFFFFF, hi = hb[3 + k] >= 0 ? hb[3 + k] : hb[3 + k] ^ 0x7FFFFFFF;
			memcpy(&c->aabb_lo[k], &lo, 4);
			memcpy(&c->aabb_hi[k], &hi, 4);
		}
		RRG_CUDA(cudaMemcpyAsync(rb, rb_init, sizeof(rb_init), cudaMemcpyHostToDevice, s));
	}
	int rgrid = (int)((nvalid + 255) / 256);
	if (rgrid > 4 * 152) rgrid = 4 * 152;
	if (c->d_tri_off) {
		uint32_t* pos;
		int* rbm;
		RRG_CUDA(sc.get(&pos, nroots + 1));
		RRG_CUDA(sc.get(&rbm, 12 * (size_t)nroots));
		rrg::note_launch(), k_mesh_ranges<<<(nroots + 1 + 255) / 256, 256, 0, s>>>(idsA, nvalid, c->d_tri_off, nroots, pos);
		rrg::note_launch(), k_fill_root_bounds<<<(12 * nroots + 255) / 256, 256, 0, s>>>(rbm, nroots);
		rrg::note_launch(), k_root_bounds_multi<<<rgrid, 256, 0, s>>>(idsA, nvalid, plo, phi, pos, nroots, rbm);
		rrg::note_launch(), k_root_init_multi<<<(nroots + 255) / 256, 256, 0, s>>>(rbm, pos, nroots, bnodes, largeA, small, st);
	} else {
		rrg::note_launch(), k_root_bounds<<<rgrid, 256, 0, s>>>(idsA, nvalid, plo, phi, rb);
		rrg::note_launch(), k_root_init<<<1, 1, 0, s>>>(rb, nvalid, bnodes, largeA, small, st);
	}
	RRG_CUDA(cudaGetLastError());

	Task* cur = largeA;
	Task* nxt = largeB;
	int grid = c->num_sms * 8;
	for (int level = 0; level < 4096; level++) {
		RRG_CUDA(cudaMemcpyAsync(&hst, st, sizeof(hst), cudaMemcpyDeviceToHost, s));
		RRG_CUDA(cudaStreamSynchronize(s));
		if (aborting && *aborting) return RRG_ERR_ABORTED;
		int ntasks = hst.nlarge_next;
		if (ntasks == 0) break;
		if (ntasks > max_large) return RRG_ERR_INVALID;
		// reset per-level counters (keep node_count and nsmall)
		RRG_CUDA(cudaMemsetAsync(&st->nlarge_next, 0, 4, s));
		RRG_CUDA(cudaMemsetAsync(&st->nchunks, 0, 4, s));
		rrg::note_launch(), k_level_setup<<<ntasks < grid ? ntasks : grid, kBT, 0, s>>>(cur, ntasks, gbins, chunks, st);
		rrg::note_launch(), k_bin_chunks<<<grid, kBT, 0, s>>>(cur, chunks, st, ids_bufs, plo, phi, gbins);
		rrg::note_launch(), k_decide_large<<<ntasks < grid ? ntasks : grid, 128, 0, s>>>(cur, ntasks, gbins, splits, bnodes, nxt, small, st);
		rrg::note_launch(), k_part_count<<<grid, kBT, 0, s>>>(cur, chunks, st, splits, ids_bufs, plo, phi, chunk_left);
		rrg::note_launch(), k_part_scan<<<(ntasks + 127) / 128, 128, 0, s>>>(cur, ntasks, chunk_left);
		rrg::note_launch(), k_part_scatter<<<grid, kBT, 0, s>>>(cur, chunks, st, splits, ids_bufs, plo, phi, chunk_left, st);
		RRG_CUDA(cudaGetLastError());
		Task* tmp = cur;
		cur = nxt;
		nxt = tmp;
	}
	RRG_CUDA(cudaMemcpyAsync(&hst, st, sizeof(hst), cudaMemcpyDeviceToHost, s));
	RRG_CUDA(cudaStreamSynchronize(s));
	if (aborting && *aborting) return RRG_ERR_ABORTED;
	if (hst.nsmall > 0) {
		int sgrid = hst.nsmall < c->num_sms * 8 ? hst.nsmall : c->num_sms * 8;
		rrg::note_launch(), k_small<<<sgrid, kSmallThreads, 0, s>>>(small, st, ids_bufs, plo, phi, bnodes, final_ids, max_leaf, st);
		RRG_CUDA(cudaGetLastError());
	}
	RRG_CUDA(cudaMemcpyAsync(&hst, st, sizeof(hst), cudaMemcpyDeviceToHost, s));
	RRG_CUDA(cudaStreamSynchronize(s));
	if (hst.error) return RRG_ERR_INVALID;
	int nnodes = hst.node_count;
	if (nnodes > max_nodes) return RRG_ERR_INVALID;

	// final device arrays
	if (c->d_nodes) cudaFree(c->d_nodes);
	if (c->d_tris) cudaFree(c->d_tris);
	c->d_nodes = nullptr;
	c->d_tris = nullptr;
	RRG_CUDA(dalloc(&c->d_nodes, nnodes));
	RRG_CUDA(dalloc(&c->d_tris, 3 * (size_t)nvalid));
	float* pad;
	RRG_CUDA(sc.get(&pad, 1));
	rrg::note_launch(), k_root_pad<<<1, 256, 0, s>>>(bnodes, nroots, pad);
	rrg::note_launch(), k_emit_nodes<<<(nnodes + 255) / 256, 256, 0, s>>>(bnodes, nnodes, (int)nroots, pad, c->d_nodes);
	rrg::note_launch(), k_emit_tris<<<(nvalid + 255) / 256, 256, 0, s>>>(final_ids, nvalid, c->d_xyz, c->d_idx, c->d_tris);
	RRG_CUDA(cudaGetLastError());
	if (c->width == 8) {
		int wst = build_wide(c, bnodes, nnodes, pad, s);
		if (wst) return wst;
	}
	RRG_CUDA(cudaEventRecord(e1, s));
	RRG_CUDA(cudaEventSynchronize(e1));
	float ms = 0;
	cudaEventElapsedTime(&ms, e0, e1);
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	c->build_ms = ms;
	c->nnodes = (uint32_t)nnodes;
	return RRG_OK;
}

// ------------------------------------------------------- graph rebuild
// The build of a batch (binary tree, one root per mesh) as a fixed sequence
// of launches that a CUDA graph can hold: every count the host build reads
// back (valid triangles, large tasks per level, small tasks, nodes) stays on
// the device and the kernels read it there; the scratch is allocated once at
// its largest (every triangle valid: 2 nt + roots nodes); the level loop runs
// kGraphLevels times, a level with no large task costing seven empty
// launches; the error word collects what the host build returns as errors
// (bit 1 invalid vertex index, 8 bad small task, 16 levels exhausted, 32 too
// many large tasks).  The result is a tree of the same algorithm over the
// same input; it may number its nodes differently (the build's task lists
// fill by atomics), which no query result depends on.
constexpr int kGraphLevels = 40;

struct GraphBuild {
	uint32_t nt = 0, nroots = 0, max_nodes = 0;
	int max_large = 0, max_chunks = 0, max_leaf = 4, grid = 0, rgrid = 0, nb = 0;
	Scratch sc;
	float4 *plo = nullptr, *phi = nullptr;
	uint32_t *valid = nullptr, *bsum = nullptr, *total = nullptr, *pos = nullptr;
	int *idsA = nullptr, *idsB = nullptr, *final_ids = nullptr, *gbins = nullptr, *chunk_left = nullptr, *rbm = nullptr;
	int** ids_bufs = nullptr;
	BuildState* st = nullptr;
	BNode* bnodes = nullptr;
	Task *largeA = nullptr, *largeB = nullptr, *small = nullptr;
	Split* splits = nullptr;
	Chunk* chunks = nullptr;
	float* pad = nullptr;
	TNode* nodes = nullptr;
	float4* tris = nullptr;
};

__global__ void k_level_begin(BuildState* st, int max_large) {
	int n = st->nlarge_next;
	if (n > max_large) {
		st->error |= 32;
		n = 0;
	}
	st->ntasks = n;
	st->nlarge_next = 0;
	st->nchunks = 0;
}

__global__ void k_level_end(BuildState* st) {
	if (st->nlarge_next > 0) st->error |= 16;
}

int graph_build_new(Collider* c, GraphBuild** out) {
	*out = nullptr;
	if (!c->d_tri_off || c->width == 8) return RRG_ERR_INVALID;
	GraphBuild* g = new (std::nothrow) GraphBuild();
	if (!g) return RRG_ERR_OOM;
	const uint32_t nt = c->nt, nroots = c->nroots;
	g->nt = nt;
	g->nroots = nroots;
	g->max_leaf = c->params.max_leaf_size ? (int)c->params.max_leaf_size : 4;
	if (g->max_leaf > kMaxLeaf) g->max_leaf = kMaxLeaf;
	g->max_nodes = 2 * nt + nroots;
	g->max_large = 2 * ((int)nt / kSmall + 2);
	g->max_chunks = (int)nt / kChunk + g->max_large + 2;
	g->nb = (int)((nt + kScanItems - 1) / kScanItems);
	g->grid = c->num_sms * 8;
	g->rgrid = (int)((nt + 255) / 256) < 4 * c->num_sms ? (int)((nt + 255) / 256) : 4 * c->num_sms;
	cudaError_t e = cudaSuccess;
	Scratch& sc = g->sc;
	if (e == cudaSuccess) e = sc.get(&g->plo, nt);
	if (e == cudaSuccess) e = sc.get(&g->phi, nt);
	if (e == cudaSuccess) e = sc.get(&g->valid, nt);
	if (e == cudaSuccess) e = sc.get(&g->bsum, (size_t)g->nb);
	if (e == cudaSuccess) e = sc.get(&g->total, 1);
	if (e == cudaSuccess) e = sc.get(&g->st, 1);
	if (e == cudaSuccess) e = sc.get(&g->idsA, nt);
	if (e == cudaSuccess) e = sc.get(&g->idsB, nt);
	if (e == cudaSuccess) e = sc.get(&g->final_ids, nt);
	if (e == cudaSuccess) e = sc.get(&g->bnodes, g->max_nodes);
	if (e == cudaSuccess) e = sc.get(&g->largeA, (size_t)g->max_large);
	if (e == cudaSuccess) e = sc.get(&g->largeB, (size_t)g->max_large);
	if (e == cudaSuccess) e = sc.get(&g->small, (size_t)nt + 2);
	if (e == cudaSuccess) e = sc.get(&g->splits, (size_t)g->max_large);
	if (e == cudaSuccess) e = sc.get(&g->chunks, (size_t)g->max_chunks);
	if (e == cudaSuccess) e = sc.get(&g->chunk_left, (size_t)g->max_chunks);
	if (e == cudaSuccess) e = sc.get(&g->gbins, (size_t)g->max_large * kTaskBinInts);
	if (e == cudaSuccess) e = sc.get(&g->ids_bufs, 2);
	if (e == cudaSuccess) e = sc.get(&g->pos, (size_t)nroots + 1);
	if (e == cudaSuccess) e = sc.get(&g->rbm, 12 * (size_t)nroots);
	if (e == cudaSuccess) e = sc.get(&g->pad, 1);
	if (e == cudaSuccess) e = sc.get(&g->nodes, g->max_nodes);
	if (e == cudaSuccess) e = sc.get(&g->tris, 3 * (size_t)nt);
	if (e == cudaSuccess) {
		int* hbufs[2] = {g->idsA, g->idsB};
		e = cudaMemcpy(g->ids_bufs, hbufs, sizeof(hbufs), cudaMemcpyHostToDevice);
	}
	if (e != cudaSuccess) {
		delete g;
		return cuda_fail(e);
	}
	*out = g;
	return RRG_OK;
}

void graph_build_free(GraphBuild* g) { delete g; }
const TNode* graph_build_nodes(const GraphBuild* g) { return g->nodes; }
const float4* graph_build_tris(const GraphBuild* g) { return g->tris; }
uint32_t graph_build_max_nodes(const GraphBuild* g) { return g->max_nodes; }

// Enqueues the whole build of c's current vertex positions (c->d_xyz,
// c->d_idx) on stream s, reading nothing back.
int graph_build_enqueue(Collider* c, GraphBuild* g, cudaStream_t s) {
	const uint32_t nt = g->nt, nroots = g->nroots;
	BuildState* st = g->st;
	RRG_CUDA(cudaMemsetAsync(st, 0, sizeof(BuildState), s));
	rrg::note_launch(), k_prep<<<(nt + 255) / 256, 256, 0, s>>>(c->d_xyz, c->nv, c->d_idx, nt, g->plo, g->phi, g->valid, st);
	rrg::note_launch(), k_block_count<<<g->nb, kBT, 0, s>>>(g->valid, nt, g->bsum);
	rrg::note_launch(), k_scan_blocks<<<1, kBT, 0, s>>>(g->bsum, (uint32_t)g->nb, g->total);
	rrg::note_launch(), k_compact<<<g->nb, kBT, 0, s>>>(g->valid, nt, g->bsum, g->idsA);
	rrg::note_launch(), k_mesh_ranges<<<(nroots + 1 + 255) / 256, 256, 0, s>>>(g->idsA, 0, c->d_tri_off, nroots, g->pos,
	                                                                           g->total);
	rrg::note_launch(), k_fill_root_bounds<<<(12 * nroots + 255) / 256, 256, 0, s>>>(g->rbm, nroots);
	rrg::note_launch(), k_root_bounds_multi<<<g->rgrid, 256, 0, s>>>(g->idsA, 0, g->plo, g->phi, g->pos, nroots, g->rbm,
	                                                                g->total);
	rrg::note_launch(), k_root_init_multi<<<(nroots + 255) / 256, 256, 0, s>>>(g->rbm, g->pos, nroots, g->bnodes, g->largeA,
	                                                                          g->small, st);
	RRG_CUDA(cudaGetLastError());
	Task* cur = g->largeA;
	Task* nxt = g->largeB;
	const int grid = g->grid;
	for (int level = 0; level < kGraphLevels; level++) {
		rrg::note_launch(), k_level_begin<<<1, 1, 0, s>>>(st, g->max_large);
		rrg::note_launch(), k_level_setup<<<grid, kBT, 0, s>>>(cur, 0, g->gbins, g->chunks, st, &st->ntasks);
		rrg::note_launch(), k_bin_chunks<<<grid, kBT, 0, s>>>(cur, g->chunks, st, g->ids_bufs, g->plo, g->phi, g->gbins);
		rrg::note_launch(), k_decide_large<<<grid, 128, 0, s>>>(cur, 0, g->gbins, g->splits, g->bnodes, nxt, g->small, st,
		                                                       &st->ntasks);
		rrg::note_launch(), k_part_count<<<grid, kBT, 0, s>>>(cur, g->chunks, st, g->splits, g->ids_bufs, g->plo, g->phi,
		                                                     g->chunk_left);
		rrg::note_launch(), k_part_scan<<<(g->max_large + 127) / 128, 128, 0, s>>>(cur, 0, g->chunk_left, &st->ntasks);
		rrg::note_launch(), k_part_scatter<<<grid, kBT, 0, s>>>(cur, g->chunks, st, g->splits, g->ids_bufs, g->plo, g->phi,
		                                                       g->chunk_left, st);
		Task* tmp = cur;
		cur = nxt;
		nxt = tmp;
	}
	rrg::note_launch(), k_level_end<<<1, 1, 0, s>>>(st);
	rrg::note_launch(), k_small<<<grid, kSmallThreads, 0, s>>>(g->small, st, g->ids_bufs, g->plo, g->phi, g->bnodes,
	                                                          g->final_ids, g->max_leaf, st);
	rrg::note_launch(), k_root_pad<<<1, 256, 0, s>>>(g->bnodes, nroots, g->pad);
	rrg::note_launch(), k_emit_nodes<<<(g->max_nodes + 255) / 256, 256, 0, s>>>(g->bnodes, 0, (int)nroots, g->pad, g->nodes,
	                                                                           &st->node_count);
	rrg::note_launch(), k_emit_tris<<<(nt + 255) / 256, 256, 0, s>>>(g->final_ids, 0, c->d_xyz, c->d_idx, g->tris, g->total);
	RRG_CUDA(cudaGetLastError());
	return RRG_OK;
}

// The error word of the last enqueued build (synchronises s): RRG_OK, or
// RRG_ERR_INVALID when the build reported an error.
int graph_build_status(GraphBuild* g, cudaStream_t s) {
	BuildState h;
	RRG_CUDA(cudaMemcpyAsync(&h, g->st, sizeof(h), cudaMemcpyDeviceToHost, s));
	RRG_CUDA(cudaStreamSynchronize(s));
	return h.error ? RRG_ERR_INVALID : RRG_OK;
}

}  // namespace rrg
