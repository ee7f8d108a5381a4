// Ray binning before traversal: one counting-sort pass groups the rays of a
// large batch by a 15-bit key (origin cell of a 8 x 8 x 8 grid over the
// scene box, Morton-interleaved, then direction cell of a 4 x 4 x 4 grid
// over [-1, 1]^3), so that the rays a warp takes next start near each other
// and point the same way.  The trace kernels then read rays and write hits
// through the permutation; each ray's result does not depend on the order,
// so binning changes speed only.
//
//   k_bin_hist    : block-local histogram in shared memory (one shared
//                   atomic per ray: measured faster than warp-aggregating
//                   them with match_any), written bin-major to
//                   hist[bin][block]; the 16-bit keys are kept for the
//                   second pass
//   k_scan_*      : exclusive scan of hist (bins x blocks)
//   k_bin_scatter : each block walks its range again and writes ray ids to
//                   perm at its bins' scanned cursors
#include "rrg_internal.cuh"

namespace rrg {

namespace {

constexpr int kBinBits = 15;
constexpr int kBins = 1 << kBinBits;
constexpr int kBinThreads = 1024;
constexpr int kScanThreads = 1024;

__device__ __forceinline__ uint32_t spread3(uint32_t x) {   // 3 bits -> positions 0, 3, 6
	return (x & 1u) | ((x & 2u) << 2) | ((x & 4u) << 4);
}

__device__ __forceinline__ uint32_t key_od(float4 a, float4 b, float lo0, float lo1, float lo2, float s0, float s1,
                                           float s2) {
	auto cell = [](float v, float lo, float s, int n) {
		float q = (v - lo) * s;
		int c = (int)q;
		return (uint32_t)(c < 0 ? 0 : (c > n - 1 ? n - 1 : c));
	};
	const uint32_t ox = cell(a.x, lo0, s0, 8), oy = cell(a.y, lo1, s1, 8), oz = cell(a.z, lo2, s2, 8);
	const uint32_t dx = cell(b.x, -1.f, 2.f, 4), dy = cell(b.y, -1.f, 2.f, 4), dz = cell(b.z, -1.f, 2.f, 4);
	const uint32_t ko = spread3(ox) | (spread3(oy) << 1) | (spread3(oz) << 2);              // 9 bits
	const uint32_t kd = (dx & 1u) | ((dy & 1u) << 1) | ((dz & 1u) << 2) | ((dx & 2u) << 2) |
	                    ((dy & 2u) << 3) | ((dz & 2u) << 4);                                   // 6 bits
	return (ko << 6) | kd;
}

__device__ __forceinline__ uint32_t ray_key(const float4* __restrict__ rays, uint32_t i, float lo0, float lo1,
                                            float lo2, float s0, float s1, float s2) {
	return key_od(__ldg(rays + 2 * (size_t)i), __ldg(rays + 2 * (size_t)i + 1), lo0, lo1, lo2, s0, s1, s2);
}

__global__ void __launch_bounds__(kBinThreads) k_bin_hist(const float4* __restrict__ rays, uint32_t n, uint32_t chunk,
                                                          float lo0, float lo1, float lo2, float s0, float s1,
                                                          float s2, uint16_t* __restrict__ keys,
                                                          uint32_t* __restrict__ hist, uint32_t nblocks) {
	extern __shared__ uint32_t sh[];
	for (int b = threadIdx.x; b < kBins; b += blockDim.x) sh[b] = 0;
	__syncthreads();
	const uint32_t begin = blockIdx.x * chunk;
	const uint32_t end = min(n, begin + chunk);
	for (uint32_t base = begin; base < end; base += blockDim.x) {
		const uint32_t i = base + threadIdx.x;
		const bool ok = i < end;
		if (ok) {
			const uint32_t k = ray_key(rays, i, lo0, lo1, lo2, s0, s1, s2);
			keys[i] = (uint16_t)k;
			atomicAdd(&sh[k], 1u);   // shared-memory atomic per ray
		}
	}
	__syncthreads();
	for (int b = threadIdx.x; b < kBins; b += blockDim.x) hist[(size_t)b * nblocks + blockIdx.x] = sh[b];
}

__global__ void __launch_bounds__(kBinThreads) k_bin_scatter(const uint16_t* __restrict__ keys, uint32_t n,
                                                             uint32_t chunk, const uint32_t* __restrict__ offs,
                                                             uint32_t nblocks, uint32_t* __restrict__ perm) {
	extern __shared__ uint32_t cur[];
	for (int b = threadIdx.x; b < kBins; b += blockDim.x) cur[b] = offs[(size_t)b * nblocks + blockIdx.x];
	__syncthreads();
	const uint32_t begin = blockIdx.x * chunk;
	const uint32_t end = min(n, begin + chunk);
	for (uint32_t base = begin; base < end; base += blockDim.x) {
		const uint32_t i = base + threadIdx.x;
		if (i < end) perm[atomicAdd(&cur[keys[i]], 1u)] = i;
	}
}

// exclusive scan of n uint32 values in place: per-block sums, a single-block
// scan of the block sums, then the per-block scans with their offsets
__global__ void __launch_bounds__(kScanThreads) k_scan_block_sums(const uint32_t* __restrict__ v, uint64_t n,
                                                                  uint32_t* __restrict__ bsum) {
	__shared__ uint32_t red[kScanThreads / 32];
	const uint64_t i = blockIdx.x * (uint64_t)kScanThreads + threadIdx.x;
	uint32_t x = i < n ? v[i] : 0u;
	for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xFFFFFFFFu, x, o);
	if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
	__syncthreads();
	if (threadIdx.x < 32) {
		uint32_t y = threadIdx.x < kScanThreads / 32 ? red[threadIdx.x] : 0u;
		for (int o = 16; o; o >>= 1) y += __shfl_xor_sync(0xFFFFFFFFu, y, o);
		if (threadIdx.x == 0) bsum[blockIdx.x] = y;
	}
}

__global__ void __launch_bounds__(kScanThreads) k_scan_sums_exclusive(uint32_t* __restrict__ bsum, uint32_t nb) {
	__shared__ uint32_t carry;
	__shared__ uint32_t wsum[kScanThreads / 32];
	if (threadIdx.x == 0) carry = 0;
	__syncthreads();
	for (uint32_t base = 0; base < nb; base += kScanThreads) {
		const uint32_t i = base + threadIdx.x;
		const uint32_t x = i < nb ? bsum[i] : 0u;
		uint32_t incl = x;
		const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
		for (int o = 1; o < 32; o <<= 1) {
			uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
			if (lane >= o) incl += y;
		}
		if (lane == 31) wsum[w] = incl;
		__syncthreads();
		if (w == 0) {
			uint32_t s = lane < kScanThreads / 32 ? wsum[lane] : 0u;
			for (int o = 1; o < 32; o <<= 1) {
				uint32_t y = __shfl_up_sync(0xFFFFFFFFu, s, o);
				if (lane >= o) s += y;
			}
			if (lane < kScanThreads / 32) wsum[lane] = s;
		}
		__syncthreads();
		const uint32_t before = (w ? wsum[w - 1] : 0u) + carry;
		if (i < nb) bsum[i] = before + incl - x;
		__syncthreads();
		if (threadIdx.x == kScanThreads - 1) carry = before + incl;
		__syncthreads();
	}
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply_exclusive(uint32_t* __restrict__ v, uint64_t n,
                                                                       const uint32_t* __restrict__ bsum) {
	__shared__ uint32_t wsum[kScanThreads / 32];
	const uint64_t i = blockIdx.x * (uint64_t)kScanThreads + threadIdx.x;
	const uint32_t x = i < n ? v[i] : 0u;
	uint32_t incl = x;
	const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
	for (int o = 1; o < 32; o <<= 1) {
		uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
		if (lane >= o) incl += y;
	}
	if (lane == 31) wsum[w] = incl;
	__syncthreads();
	if (w == 0) {
		uint32_t s = lane < kScanThreads / 32 ? wsum[lane] : 0u;
		for (int o = 1; o < 32; o <<= 1) {
			uint32_t y = __shfl_up_sync(0xFFFFFFFFu, s, o);
			if (lane >= o) s += y;
		}
		if (lane < kScanThreads / 32) wsum[lane] = s;
	}
	__syncthreads();
	if (i < n) v[i] = bsum[blockIdx.x] + (w ? wsum[w - 1] : 0u) + incl - x;
}

// The same two passes over a list of path ids whose count stays on the
// device (the wavefront gather's live paths): path p's ray is (eye[p],
// dir[p]); the scatter writes the path ids themselves in key order.
__global__ void __launch_bounds__(kBinThreads) k_bin_hist_paths(const float4* __restrict__ eye,
                                                                const float4* __restrict__ dir,
                                                                const uint32_t* __restrict__ list,
                                                                const uint32_t* __restrict__ n_dev, float lo0,
                                                                float lo1, float lo2, float s0, float s1, float s2,
                                                                uint16_t* __restrict__ keys,
                                                                uint32_t* __restrict__ hist, uint32_t nblocks) {
	extern __shared__ uint32_t sh[];
	for (int b = threadIdx.x; b < kBins; b += blockDim.x) sh[b] = 0;
	__syncthreads();
	const uint32_t n = *n_dev;
	const uint32_t chunk = (n + gridDim.x - 1) / gridDim.x;
	const uint32_t begin = min(n, blockIdx.x * chunk);
	const uint32_t end = min(n, begin + chunk);
	for (uint32_t base = begin; base < end; base += blockDim.x) {
		const uint32_t i = base + threadIdx.x;
		const bool ok = i < end;
		if (ok) {
			const uint32_t p = list[i];
			const uint32_t k = key_od(eye[p], dir[p], lo0, lo1, lo2, s0, s1, s2);
			keys[i] = (uint16_t)k;
			atomicAdd(&sh[k], 1u);
		}
	}
	__syncthreads();
	for (int b = threadIdx.x; b < kBins; b += blockDim.x) hist[(size_t)b * nblocks + blockIdx.x] = sh[b];
}

__global__ void __launch_bounds__(kBinThreads) k_bin_scatter_paths(const uint16_t* __restrict__ keys,
                                                                   const uint32_t* __restrict__ list,
                                                                   const uint32_t* __restrict__ n_dev,
                                                                   const uint32_t* __restrict__ offs, uint32_t nblocks,
                                                                   uint32_t* __restrict__ out) {
	extern __shared__ uint32_t cur[];
	for (int b = threadIdx.x; b < kBins; b += blockDim.x) cur[b] = offs[(size_t)b * nblocks + blockIdx.x];
	__syncthreads();
	const uint32_t n = *n_dev;
	const uint32_t chunk = (n + gridDim.x - 1) / gridDim.x;
	const uint32_t begin = min(n, blockIdx.x * chunk);
	const uint32_t end = min(n, begin + chunk);
	for (uint32_t base = begin; base < end; base += blockDim.x) {
		const uint32_t i = base + threadIdx.x;
		if (i < end) out[atomicAdd(&cur[keys[i]], 1u)] = list[i];
	}
}

}  // namespace

// The binning kernels' shared-memory allowance (128 KB of bins), set on the
// collider's device the first time it bins.
static int bin_attrs(Collider* c) {
	if (c->bin_attr) return RRG_OK;
	const int smem = (int)(kBins * sizeof(uint32_t));
	RRG_CUDA(cudaFuncSetAttribute(k_bin_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
	RRG_CUDA(cudaFuncSetAttribute(k_bin_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
	RRG_CUDA(cudaFuncSetAttribute(k_bin_hist_paths, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
	RRG_CUDA(cudaFuncSetAttribute(k_bin_scatter_paths, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
	c->bin_attr = true;
	return RRG_OK;
}

// Bytes of scratch bin_paths needs for lists of up to cap paths.
size_t bin_paths_bytes(const Collider* c, uint32_t cap) {
	const uint64_t nh = (uint64_t)kBins * (uint32_t)c->num_sms;
	const uint64_t nsum = (nh + kScanThreads - 1) / kScanThreads;
	return sizeof(uint32_t) * (size_t)cap + sizeof(uint32_t) * nh + sizeof(uint32_t) * nsum + 256 +
	       sizeof(uint16_t) * (size_t)cap;
}

// Sorts the *n_dev path ids of list by the key of their rays (eye, dir)
// into out (cap entries), with scratch of bin_paths_bytes(c, cap) bytes.
int bin_paths(Collider* c, const float4* eye, const float4* dir, const uint32_t* list, const uint32_t* n_dev,
              uint32_t cap, void* scratch, uint32_t* out, cudaStream_t s) {
	const uint32_t nblocks = (uint32_t)c->num_sms;
	const uint64_t nh = (uint64_t)kBins * nblocks;
	const uint64_t nsum = (nh + kScanThreads - 1) / kScanThreads;
	if (int st = bin_attrs(c)) return st;
	uint8_t* p = reinterpret_cast<uint8_t*>(scratch);
	p += sizeof(uint32_t) * (size_t)cap;   // (unused: keeps the layout of bin_rays)
	uint32_t* hist = reinterpret_cast<uint32_t*>(p);
	p += sizeof(uint32_t) * nh;
	uint32_t* bsum = reinterpret_cast<uint32_t*>(p);
	p += sizeof(uint32_t) * nsum;
	p = reinterpret_cast<uint8_t*>(((uintptr_t)p + 255) & ~(uintptr_t)255);
	uint16_t* keys = reinterpret_cast<uint16_t*>(p);
	float s3[3];
	for (int k = 0; k < 3; k++) {
		const float ext = c->aabb_hi[k] - c->aabb_lo[k];
		s3[k] = ext > 0.f ? 8.f / ext : 0.f;
	}
	const size_t smem = kBins * sizeof(uint32_t);
	rrg::note_launch(), k_bin_hist_paths<<<nblocks, kBinThreads, smem, s>>>(eye, dir, list, n_dev, c->aabb_lo[0],
	                                                                        c->aabb_lo[1], c->aabb_lo[2], s3[0], s3[1],
	                                                                        s3[2], keys, hist, nblocks);
	rrg::note_launch(), k_scan_block_sums<<<(unsigned)nsum, kScanThreads, 0, s>>>(hist, nh, bsum);
	rrg::note_launch(), k_scan_sums_exclusive<<<1, kScanThreads, 0, s>>>(bsum, (uint32_t)nsum);
	rrg::note_launch(), k_scan_apply_exclusive<<<(unsigned)nsum, kScanThreads, 0, s>>>(hist, nh, bsum);
	rrg::note_launch(), k_bin_scatter_paths<<<nblocks, kBinThreads, smem, s>>>(keys, list, n_dev, hist, nblocks, out);
	RRG_CUDA(cudaGetLastError());
	return RRG_OK;
}

int bin_rays(Collider* c, const float4* rays, uint32_t n, cudaStream_t s, int slot, const uint32_t** perm_out) {
	*perm_out = nullptr;
	if (slot < 0 || slot > 3) return RRG_ERR_INVALID;
	const uint32_t nblocks = (uint32_t)c->num_sms;
	const uint32_t chunk = (n + nblocks - 1) / nblocks;
	const uint64_t nh = (uint64_t)kBins * nblocks;
	const uint64_t nsum = (nh + kScanThreads - 1) / kScanThreads;
	if (nsum > 65535u * 16) return RRG_ERR_INVALID;
	const size_t need = sizeof(uint32_t) * (size_t)n + sizeof(uint16_t) * (size_t)n + sizeof(uint32_t) * nh +
	                    sizeof(uint32_t) * nsum + 256 * 4;
	if (need > c->bin_bytes[slot]) {
		cudaFree(c->d_bin[slot]);
		c->d_bin[slot] = nullptr;
		c->bin_bytes[slot] = 0;
		RRG_CUDA(cudaMalloc(&c->d_bin[slot], need));
		c->bin_bytes[slot] = need;
		account_collider(c);
	}
	if (int st = bin_attrs(c)) return st;
	uint8_t* p = reinterpret_cast<uint8_t*>(c->d_bin[slot]);
	uint32_t* perm = reinterpret_cast<uint32_t*>(p);
	p += sizeof(uint32_t) * (size_t)n;
	uint32_t* hist = reinterpret_cast<uint32_t*>(p);
	p += sizeof(uint32_t) * nh;
	uint32_t* bsum = reinterpret_cast<uint32_t*>(p);
	p += sizeof(uint32_t) * nsum;
	p = reinterpret_cast<uint8_t*>(((uintptr_t)p + 255) & ~(uintptr_t)255);
	uint16_t* keys = reinterpret_cast<uint16_t*>(p);
	float s3[3];
	for (int k = 0; k < 3; k++) {
		const float ext = c->aabb_hi[k] - c->aabb_lo[k];
		s3[k] = ext > 0.f ? 8.f / ext : 0.f;
	}
	const size_t smem = kBins * sizeof(uint32_t);
	rrg::note_launch(), k_bin_hist<<<nblocks, kBinThreads, smem, s>>>(rays, n, chunk, c->aabb_lo[0], c->aabb_lo[1], c->aabb_lo[2], s3[0],
	                                              s3[1], s3[2], keys, hist, nblocks);
	rrg::note_launch(), k_scan_block_sums<<<(unsigned)nsum, kScanThreads, 0, s>>>(hist, nh, bsum);
	rrg::note_launch(), k_scan_sums_exclusive<<<1, kScanThreads, 0, s>>>(bsum, (uint32_t)nsum);
	rrg::note_launch(), k_scan_apply_exclusive<<<(unsigned)nsum, kScanThreads, 0, s>>>(hist, nh, bsum);
	rrg::note_launch(), k_bin_scatter<<<nblocks, kBinThreads, smem, s>>>(keys, n, chunk, hist, nblocks, perm);
	RRG_CUDA(cudaGetLastError());
	*perm_out = perm;
	return RRG_OK;
}

}  // namespace rrg
