// Compacting traversal of the binary BVH (RRG_TRAVERSAL_COMPACT): closest
// hit and any hit for batches of rays, with the same results as k_closest /
// k_occluded (rrg_trace.cu) but fewer idle lanes and no local-memory stack.
//
// In k_closest a warp takes 32 rays and walks them until its last ray is
// done; lanes whose ray finished early idle until then (ncu on the
// config-1 interior: 13.4 of 32 lanes active per issued instruction).
// Here:
//   * each warp claims a block of 32 x fetch consecutive rays of the launch
//     (in the binned order when the batch is binned, rrg_binning.cu), so
//     the rays a warp holds stay neighbours in origin and direction;
//   * lane l walks rays l, l + 32, l + 64, ... of the block one after the
//     other, each to its end, with no warp-wide step in between: a lane
//     whose ray ends goes straight on to its next ray (the warp's lanes are
//     compacted onto the block's remaining rays), and the warp waits for its
//     slowest lane once per block instead of once per 32 rays;
//   * each thread's traversal stack keeps its top SDEPTH entries in shared
//     memory, entry d of thread t at s_stack[d * kTraceThreads + t] (a
//     warp's 32 lanes touch 32 consecutive words, one bank each), and the
//     deeper entries in a per-thread local array, so the stack traffic of
//     the usual shallow stacks stays out of the L1 cache that holds the
//     tree.
// (A variant that refilled idle lanes from the block after a warp vote on
// every node step measured 1.6x slower on the config-1 interior: the vote
// forces the node and leaf paths of the warp to reconverge at every step.)
// Every visit, triangle test, tie rule and output field is that of
// traverse() and k_closest (rrg_traverse.cuh), so results are bit-identical
// to the other traversal kernels; only the order in which rays are walked
// differs.
#include "rrg_traverse.cuh"

namespace rrg {

// MINB > 0 caps registers so that MINB blocks fit on an SM (occupancy
// against spills: a tuning knob).
template <bool ANY, bool PERM, int SDEPTH, int MINB>
__global__ void __launch_bounds__(kTraceThreads, MINB) k_trace_compact(
    const TNode* __restrict__ nodes, int nnodes, const float4* __restrict__ tris, int ntris,
    const float4* __restrict__ rays, uint32_t n, float4* __restrict__ hits, float4* __restrict__ planes,
    float* __restrict__ points, uint8_t* __restrict__ occ, uint32_t* counter, const uint32_t* __restrict__ perm,
    int fetch) {
	__shared__ int s_stack[(SDEPTH > 0 ? SDEPTH : 1) * kTraceThreads];
	int* const sst = s_stack + threadIdx.x;
	const int lane = threadIdx.x & 31;
	const uint32_t per_fetch = 32u * (uint32_t)fetch;
	bool overflow = false;
	while (true) {
		uint32_t base = 0;
		if (lane == 0) base = atomicAdd(counter, per_fetch);
		base = __shfl_sync(0xFFFFFFFFu, base, 0);
		if (base >= n) break;
		for (int k = 0; k < fetch; k++) {
			const uint32_t j = base + 32u * (uint32_t)k + (uint32_t)lane;
			if (j >= n) break;
			const uint32_t i = PERM ? __ldg(perm + j) : j;
			RayState r;
			const float4 ra = __ldg(rays + 2 * (size_t)i), rb = __ldg(rays + 2 * (size_t)i + 1);
			r.ox = ra.x; r.oy = ra.y; r.oz = ra.z; r.tmin = ra.w;
			r.dx = rb.x; r.dy = rb.y; r.dz = rb.z; r.tmax = rb.w;
			ray_setup(r);
			float tbest = r.tmax;
			uint32_t best_tri = 0xFFFFFFFFu;
			int slot = -1;
			if (r.tmin <= r.tmax)
				slot = traverse_split<ANY, SDEPTH>(nodes, tris, r, nnodes, ntris, tbest, best_tri, overflow, sst);
			if (ANY) {
				occ[i] = slot >= 0 ? 1 : 0;
			} else if (slot < 0) {
				hits[i] = make_float4(0.f, __int_as_float((int)0xFFFFFFFFu), 0.f, 0.f);
				if (planes) planes[i] = make_float4(0.f, 0.f, 0.f, 0.f);
				if (points) {
					points[3 * (size_t)i] = 0.f;
					points[3 * (size_t)i + 1] = 0.f;
					points[3 * (size_t)i + 2] = 0.f;
				}
			} else {
				float4 a, b, c;
				load_tri(tris, slot, a, b, c);
				const Fastest f = fastest_fields(r, a, b, c);
				hits[i] = make_float4(f.dist, __int_as_float((int)(best_tri | (f.front ? 0x80000000u : 0u))), f.u, f.v);
				if (planes) planes[i] = make_float4(f.n[0], f.n[1], f.n[2], f.n[3]);
				if (points) {
					points[3 * (size_t)i] = __fadd_rn(r.ox, __fmul_rn(r.dx, f.dist));
					points[3 * (size_t)i + 1] = __fadd_rn(r.oy, __fmul_rn(r.dy, f.dist));
					points[3 * (size_t)i + 2] = __fadd_rn(r.oz, __fmul_rn(r.dz, f.dist));
				}
			}
		}
	}
	if (overflow) atomicOr(counter + 1, (uint32_t)RRG_ERR_STACK);
}

namespace {

using CompactKernel = void (*)(const TNode*, int, const float4*, int, const float4*, uint32_t, float4*, float4*,
                               float*, uint8_t*, uint32_t*, const uint32_t*, int);

template <bool ANY, bool PERM, int MINB>
CompactKernel pick_depth(uint32_t sdepth) {
	switch (sdepth) {
		case 0: return k_trace_compact<ANY, PERM, 0, MINB>;
		case 8: return k_trace_compact<ANY, PERM, 8, MINB>;
		case 32: return k_trace_compact<ANY, PERM, 32, MINB>;
		default: return k_trace_compact<ANY, PERM, 16, MINB>;
	}
}

template <bool ANY, bool PERM>
CompactKernel pick_minb(uint32_t sdepth, uint32_t minb) {
	return minb ? pick_depth<ANY, PERM, 9>(sdepth) : pick_depth<ANY, PERM, 0>(sdepth);
}

CompactKernel pick(bool any, bool perm, uint32_t sdepth, uint32_t minb) {
	if (any) return perm ? pick_minb<true, true>(sdepth, minb) : pick_minb<true, false>(sdepth, minb);
	return perm ? pick_minb<false, true>(sdepth, minb) : pick_minb<false, false>(sdepth, minb);
}

}  // namespace

bool compact_depth_ok(uint32_t sdepth) { return sdepth == 0 || sdepth == 8 || sdepth == 16 || sdepth == 32; }

// Clears the work counter (words[0]) and launches the compacting kernel on
// stream s: closest hit when occ is null, else any hit.  Grid: the kernel's
// resident blocks per SM times the SMs (persistent), fewer for small batches.
int launch_compact(Collider* c, const float4* rays, uint32_t n, float4* hits, float4* planes, float* points,
                   uint8_t* occ, uint32_t* words, const uint32_t* perm, cudaStream_t s) {
	if (!n) return RRG_OK;
	const CompactKernel k = pick(occ != nullptr, perm != nullptr, c->compact_sdepth, c->compact_minb);
	const int slot = (c->compact_minb ? 16 : 0) + (occ ? 8 : 0) + (perm ? 4 : 0) +
	                 (c->compact_sdepth == 0 ? 0 : c->compact_sdepth == 8 ? 1 : c->compact_sdepth == 32 ? 3 : 2);
	if (!c->compact_blocks[slot]) {
		int per_sm = 0;
		RRG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kTraceThreads, 0));
		c->compact_blocks[slot] = (per_sm > 0 ? per_sm : 1) * c->num_sms;
	}
	const uint32_t blocks = (uint32_t)c->compact_blocks[slot];
	const uint32_t per_block = 32u * (uint32_t)c->compact_fetch * (kTraceThreads / 32);
	const uint32_t want = (uint32_t)(((uint64_t)n + per_block - 1) / per_block);
	const int grid = (int)(want < blocks ? want : blocks);
	RRG_CUDA(cudaMemsetAsync(words, 0, 4, s));
	rrg::note_launch(), k<<<grid, kTraceThreads, 0, s>>>(c->d_nodes, (int)c->nnodes, c->d_tris, (int)c->nvalid, rays, n,
	                                                   hits, planes, points, occ, words, perm, (int)c->compact_fetch);
	RRG_CUDA(cudaGetLastError());
	return RRG_OK;
}

}  // namespace rrg
