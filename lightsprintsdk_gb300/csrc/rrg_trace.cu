// Closest-hit and any-hit traversal of the binary BVH.
//
// Replaces IntersectBspFast::intersect (RRCollider/IntersectBspFast.cpp:795-845)
// and its BSP walk (:302-535) for batches of rays:
//   * persistent CTAs; each warp takes 32 rays at a time from a global counter;
//   * a stack per thread; both child boxes are tested from one 64-byte node
//     fetch (four float4 __ldg loads), the nearer child is visited first;
//   * watertight ray/triangle test (Woop, Benthin, Wald: "Watertight
//     Ray/Triangle Intersection", JCGT 2(1), 2013): per-ray shear to the
//     dominant axis, 2-D edge functions evaluated without contraction
//     (__fmul_rn/__fsub_rn) so that a shared edge gives opposite values in
//     both triangles, with a double-precision retry when an edge value is 0;
//   * nearest hit in [rayLengthMin, rayLengthMax]; equal distances resolve to
//     the lower triangle index, so results do not depend on the tree;
//   * the reported fields are then recomputed for the chosen triangle with
//     the reference's own float formulas (IntersectBspFast.cpp:130-252, one
//     rounding per operation), so hitDistance, hitPoint2d, hitPlane and
//     hitFrontSide are the values IT_BSP_FASTEST reports for that triangle.
#include "rrg_traverse.cuh"

namespace rrg {

__device__ __forceinline__ void load_ray(const float4* __restrict__ rays, uint32_t i, RayState& r) {
	float4 a = __ldg(rays + 2 * (size_t)i), b = __ldg(rays + 2 * (size_t)i + 1);
	r.ox = a.x; r.oy = a.y; r.oz = a.z; r.tmin = a.w;
	r.dx = b.x; r.dy = b.y; r.dz = b.z; r.tmax = b.w;
	ray_setup(r);
}

// Persistent work distribution: each warp takes 32 consecutive rays.
__device__ __forceinline__ uint32_t warp_fetch(uint32_t* counter) {
	uint32_t base = 0;
	if ((threadIdx.x & 31) == 0) base = atomicAdd(counter, 32u);
	return __shfl_sync(0xFFFFFFFFu, base, 0);
}

// Whether the first step of traverse() from node 0 enters either child box
// (a ray that enters neither ends there as a miss).
__device__ __forceinline__ bool root_enter(const TNode* __restrict__ nodes, int nnodes, const RayState& r) {
	if (nnodes <= 0) return true;   // traverse() reports the malformed tree
	const float4* np = reinterpret_cast<const float4*>(nodes);
	const float4 na = __ldg(np), nb = __ldg(np + 1), nc = __ldg(np + 2);
	const int4 nd = __ldg(reinterpret_cast<const int4*>(np + 3));
	const float t0 = nd.x != kEmptyRef ? box_enter(r, na.x, na.y, na.z, na.w, nc.x, nc.y, r.tmax) : INFINITY;
	const float t1 = nd.y != kEmptyRef ? box_enter(r, nb.x, nb.y, nb.z, nb.w, nc.z, nc.w, r.tmax) : INFINITY;
	return t0 != INFINITY || t1 != INFINITY;
}

__device__ __forceinline__ void write_miss(uint32_t i, float4* __restrict__ hits, float4* __restrict__ planes,
                                           float* __restrict__ points) {
	hits[i] = make_float4(0.f, __int_as_float((int)0xFFFFFFFFu), 0.f, 0.f);
	if (planes) planes[i] = make_float4(0.f, 0.f, 0.f, 0.f);
	if (points) { points[3 * (size_t)i] = 0.f; points[3 * (size_t)i + 1] = 0.f; points[3 * (size_t)i + 2] = 0.f; }
}

// Root-box queue (RRG_TRAVERSAL_ROOT_QUEUE): a warp takes batches of 32
// rays, answers at once the rays that enter neither child box of the root
// (or have tmin > tmax), and queues the others in shared memory until 32
// of them fill the warp; a batch whose 32 rays all enter is traced at once.
// Where most rays pass the mesh by (rays around an object), a warp then
// traces 32 rays that enter the tree instead of a few among 32.  Returns
// the ray index this lane traces next (0xFFFFFFFF: none), or sets done when
// the launch's rays and the queue are exhausted.  The same rays get the
// same answers as without the queue; only the order they are walked in
// changes.
template <bool PERM>
__device__ __forceinline__ uint32_t next_queued(const TNode* __restrict__ nodes, int nnodes,
                                                const float4* __restrict__ rays, uint32_t n,
                                                const uint32_t* __restrict__ perm, uint32_t* counter,
                                                uint32_t* q, int& qn, bool& exhausted, bool& done,
                                                float4* __restrict__ hits, float4* __restrict__ planes,
                                                float* __restrict__ points, uint8_t* __restrict__ occ) {
	const int lane = threadIdx.x & 31;
	while (!exhausted) {
		const uint32_t base = warp_fetch(counter);
		if (base >= n) { exhausted = true; break; }
		const uint32_t j = base + lane;
		const bool valid = j < n;
		uint32_t i = 0;
		bool enter = false;
		if (valid) {
			i = PERM ? __ldg(perm + j) : j;
			RayState r;
			load_ray(rays, i, r);
			enter = r.tmin <= r.tmax && root_enter(nodes, nnodes, r);
			if (!enter) {
				if (occ) occ[i] = 0;
				else write_miss(i, hits, planes, points);
			}
		}
		const uint32_t mask = __ballot_sync(0xFFFFFFFFu, enter);
		if (mask == 0xFFFFFFFFu && qn == 0) return i;   // a full batch: trace it as it is
		if (enter) q[qn + __popc(mask & ((1u << lane) - 1u))] = i;
		qn += __popc(mask);
		__syncwarp();
		if (qn >= 32) break;
	}
	if (qn == 0) {
		done = true;
		return 0xFFFFFFFFu;
	}
	const int take = qn < 32 ? qn : 32;
	const uint32_t i = lane < take ? q[qn - take + lane] : 0xFFFFFFFFu;
	__syncwarp();
	qn -= take;
	return i;
}

// PERM: ray j of the launch is ray perm[j] of the batch (binned order, see
// rrg_binning.cu); hits are written at the ray's own index.  QUEUE: rays
// come through the root-box queue (next_queued).
template <bool PERM, bool QUEUE>
__global__ void __launch_bounds__(kTraceThreads, QUEUE ? 9 : 0) k_closest(const TNode* __restrict__ nodes, int nnodes,
                                                           const float4* __restrict__ tris, int ntris,
                                                           const float4* __restrict__ rays, uint32_t n,
                                                           float4* __restrict__ hits, float4* __restrict__ planes,
                                                           float* __restrict__ points, uint32_t* counter,
                                                           const uint32_t* __restrict__ perm) {
	__shared__ uint32_t s_q[QUEUE ? kTraceThreads / 32 : 1][64];
	uint32_t* q = s_q[QUEUE ? threadIdx.x >> 5 : 0];
	int qn = 0;
	bool exhausted = false, done = false;
	const int lane = threadIdx.x & 31;
	while (true) {
		uint32_t i;
		if (QUEUE) {
			i = next_queued<PERM>(nodes, nnodes, rays, n, perm, counter, q, qn, exhausted, done, hits, planes, points,
			                      nullptr);
			if (done) break;
			if (i == 0xFFFFFFFFu) continue;
		} else {
			uint32_t base = warp_fetch(counter);
			if (base >= n) break;
			const uint32_t j = base + lane;
			if (j >= n) continue;
			i = PERM ? __ldg(perm + j) : j;
		}
		RayState r;
		load_ray(rays, i, r);
		float tbest = r.tmax;
		uint32_t best_tri = 0xFFFFFFFFu;
		bool overflow = false;
		int slot = -1;
		if (r.tmin <= r.tmax) slot = traverse<false>(nodes, tris, r, nnodes, ntris, tbest, best_tri, overflow);
		if (overflow) atomicOr(counter + 1, (uint32_t)RRG_ERR_STACK);
		if (slot < 0) {
			write_miss(i, hits, planes, points);
			continue;
		}
		float4 a, b, c;
		load_tri(tris, slot, a, b, c);
		Fastest f = fastest_fields(r, a, b, c);
		uint32_t bits = best_tri | (f.front ? 0x80000000u : 0u);
		hits[i] = make_float4(f.dist, __int_as_float((int)bits), f.u, f.v);
		if (planes) planes[i] = make_float4(f.n[0], f.n[1], f.n[2], f.n[3]);
		if (points) {
			points[3 * (size_t)i] = __fadd_rn(r.ox, __fmul_rn(r.dx, f.dist));
			points[3 * (size_t)i + 1] = __fadd_rn(r.oy, __fmul_rn(r.dy, f.dist));
			points[3 * (size_t)i + 2] = __fadd_rn(r.oz, __fmul_rn(r.dz, f.dist));
		}
	}
}

template <bool PERM, bool QUEUE>
__global__ void __launch_bounds__(kTraceThreads) k_occluded(const TNode* __restrict__ nodes, int nnodes,
                                                            const float4* __restrict__ tris, int ntris,
                                                            const float4* __restrict__ rays, uint32_t n,
                                                            uint8_t* __restrict__ occ, uint32_t* counter,
                                                            const uint32_t* __restrict__ perm) {
	__shared__ uint32_t s_q[QUEUE ? kTraceThreads / 32 : 1][64];
	uint32_t* q = s_q[QUEUE ? threadIdx.x >> 5 : 0];
	int qn = 0;
	bool exhausted = false, done = false;
	const int lane = threadIdx.x & 31;
	while (true) {
		uint32_t i;
		if (QUEUE) {
			i = next_queued<PERM>(nodes, nnodes, rays, n, perm, counter, q, qn, exhausted, done, nullptr, nullptr,
			                      nullptr, occ);
			if (done) break;
			if (i == 0xFFFFFFFFu) continue;
		} else {
			uint32_t base = warp_fetch(counter);
			if (base >= n) break;
			const uint32_t j = base + lane;
			if (j >= n) continue;
			i = PERM ? __ldg(perm + j) : j;
		}
		RayState r;
		load_ray(rays, i, r);
		float tbest = r.tmax;
		uint32_t best_tri = 0xFFFFFFFFu;
		bool overflow = false;
		int slot = -1;
		if (r.tmin <= r.tmax) slot = traverse<true>(nodes, tris, r, nnodes, ntris, tbest, best_tri, overflow);
		if (overflow) atomicOr(counter + 1, (uint32_t)RRG_ERR_STACK);
		occ[i] = slot >= 0 ? 1 : 0;
	}
}

// The same two kernels over the 8-wide tree (traverse_wide).
__global__ void __launch_bounds__(kTraceThreads, 8) k_closest_w(const uint4* __restrict__ wn, int nwnodes,
                                                             const float4* __restrict__ tris, int ntris,
                                                             const float4* __restrict__ rays, uint32_t n,
                                                             float4* __restrict__ hits, float4* __restrict__ planes,
                                                             float* __restrict__ points, uint32_t* counter) {
	const int lane = threadIdx.x & 31;
	while (true) {
		uint32_t base = warp_fetch(counter);
		if (base >= n) break;
		uint32_t i = base + lane;
		if (i >= n) continue;
		RayState r;
		load_ray(rays, i, r);
		float tbest = r.tmax;
		uint32_t best_tri = 0xFFFFFFFFu;
		bool overflow = false;
		int slot = -1;
		if (r.tmin <= r.tmax) slot = traverse_wide<false>(wn, tris, r, nwnodes, ntris, tbest, best_tri, overflow);
		if (overflow) atomicOr(counter + 1, (uint32_t)RRG_ERR_STACK);
		if (slot < 0) {
			hits[i] = make_float4(0.f, __int_as_float((int)0xFFFFFFFFu), 0.f, 0.f);
			if (planes) planes[i] = make_float4(0.f, 0.f, 0.f, 0.f);
			if (points) { points[3 * (size_t)i] = 0.f; points[3 * (size_t)i + 1] = 0.f; points[3 * (size_t)i + 2] = 0.f; }
			continue;
		}
		float4 a, b, c;
		load_tri(tris, slot, a, b, c);
		Fastest f = fastest_fields(r, a, b, c);
		uint32_t bits = best_tri | (f.front ? 0x80000000u : 0u);
		hits[i] = make_float4(f.dist, __int_as_float((int)bits), f.u, f.v);
		if (planes) planes[i] = make_float4(f.n[0], f.n[1], f.n[2], f.n[3]);
		if (points) {
			points[3 * (size_t)i] = __fadd_rn(r.ox, __fmul_rn(r.dx, f.dist));
			points[3 * (size_t)i + 1] = __fadd_rn(r.oy, __fmul_rn(r.dy, f.dist));
			points[3 * (size_t)i + 2] = __fadd_rn(r.oz, __fmul_rn(r.dz, f.dist));
		}
	}
}

__global__ void __launch_bounds__(kTraceThreads, 8) k_occluded_w(const uint4* __restrict__ wn, int nwnodes,
                                                              const float4* __restrict__ tris, int ntris,
                                                              const float4* __restrict__ rays, uint32_t n,
                                                              uint8_t* __restrict__ occ, uint32_t* counter) {
	const int lane = threadIdx.x & 31;
	while (true) {
		uint32_t base = warp_fetch(counter);
		if (base >= n) break;
		uint32_t i = base + lane;
		if (i >= n) continue;
		RayState r;
		load_ray(rays, i, r);
		float tbest = r.tmax;
		uint32_t best_tri = 0xFFFFFFFFu;
		bool overflow = false;
		int slot = -1;
		if (r.tmin <= r.tmax) slot = traverse_wide<true>(wn, tris, r, nwnodes, ntris, tbest, best_tri, overflow);
		if (overflow) atomicOr(counter + 1, (uint32_t)RRG_ERR_STACK);
		occ[i] = slot >= 0 ? 1 : 0;
	}
}

// Closest hit over a batch of meshes in one persistent launch.  Ray i
// belongs to mesh m = segment_of(ray_off, nmesh, i) (offsets staged in
// shared memory) and is traced from that mesh's root, node m; its hit
// triangle is reported as an index local to mesh m.  A warp takes
// 32 * fetch consecutive rays per atomic (the rays-per-warp knob).
// QUEUE: the rays of a claimed block pass through the root-box queue
// (next_queued's scheme, with each ray's own mesh root): rays entering
// neither child box of their mesh's root are answered at once, the others
// traced 32 at a time.  Capped at 9 blocks per SM (56 registers; the
// queue variant spills 16 bytes): 2 % faster on config 3 than 8 blocks.
template <bool WIDE, int SDEPTH>
__device__ __forceinline__ void batch_trace_ray(const TNode* __restrict__ nodes, int nnodes,
                                                const uint4* __restrict__ wn, int nwnodes,
                                                const float4* __restrict__ tris, int ntris,
                                                const float4* __restrict__ rays, uint32_t i, uint32_t m,
                                                const uint32_t* __restrict__ tri_off, float4* __restrict__ hits,
                                                uint32_t* counter, int* sst) {
	RayState r;
	load_ray(rays, i, r);
	float tbest = r.tmax;
	uint32_t best_tri = 0xFFFFFFFFu;
	bool overflow = false;
	int slot = -1;
	if (r.tmin <= r.tmax) {
		if (WIDE) slot = traverse_wide<false>(wn, tris, r, nwnodes, ntris, tbest, best_tri, overflow, (int)m);
		else if (SDEPTH > 0)
			slot = traverse_split<false, SDEPTH>(nodes, tris, r, nnodes, ntris, tbest, best_tri, overflow, sst, (int)m);
		else slot = traverse<false>(nodes, tris, r, nnodes, ntris, tbest, best_tri, overflow, nullptr, (int)m);
	}
	if (overflow) atomicOr(counter + 1, (uint32_t)RRG_ERR_STACK);
	if (slot < 0) {
		hits[i] = make_float4(0.f, __int_as_float((int)0xFFFFFFFFu), 0.f, 0.f);
		return;
	}
	float4 a, b, c;
	load_tri(tris, slot, a, b, c);
	Fastest f = fastest_fields(r, a, b, c);
	const uint32_t bits = (best_tri - __ldg(tri_off + m)) | (f.front ? 0x80000000u : 0u);
	hits[i] = make_float4(f.dist, __int_as_float((int)bits), f.u, f.v);
}

template <bool WIDE, int SDEPTH, bool QUEUE>
__global__ void __launch_bounds__(kTraceThreads, 9) k_batch_closest(const TNode* __restrict__ nodes, int nnodes,
                                                                 const uint4* __restrict__ wn, int nwnodes,
                                                                 const float4* __restrict__ tris, int ntris,
                                                                 const float4* __restrict__ rays, uint32_t n,
                                                                 const uint32_t* __restrict__ ray_off,
                                                                 const uint32_t* __restrict__ tri_off,
                                                                 uint32_t nmesh, int fetch,
                                                                 float4* __restrict__ hits, uint32_t* counter) {
	extern __shared__ uint32_t s_off[];
	__shared__ int s_stack[(SDEPTH > 0 ? SDEPTH : 1) * kTraceThreads];
	__shared__ uint32_t s_q[QUEUE ? kTraceThreads / 32 : 1][64];
	int* const sst = s_stack + threadIdx.x;
	for (uint32_t k = threadIdx.x; k <= nmesh; k += blockDim.x) s_off[k] = ray_off[k];
	__syncthreads();
	const int lane = threadIdx.x & 31;
	const uint32_t per_fetch = 32u * (uint32_t)fetch;
	if (!QUEUE) {
		while (true) {
			uint32_t base = 0;
			if (lane == 0) base = atomicAdd(counter, per_fetch);
			base = __shfl_sync(0xFFFFFFFFu, base, 0);
			if (base >= n) break;
			for (int j = 0; j < fetch; j++) {
				const uint32_t i = base + 32u * (uint32_t)j + (uint32_t)lane;
				if (i >= n) break;
				batch_trace_ray<WIDE, SDEPTH>(nodes, nnodes, wn, nwnodes, tris, ntris, rays, i,
				                              segment_of(s_off, nmesh, i), tri_off, hits, counter, sst);
			}
		}
		return;
	}
	uint32_t* q = s_q[QUEUE ? threadIdx.x >> 5 : 0];
	int qn = 0;
	bool exhausted = false;
	uint32_t blk = 0, blk_end = 0;   // the warp's claimed block of rays (warp-uniform)
	while (true) {
		uint32_t i = 0xFFFFFFFFu;
		bool direct = false;
		while (!exhausted) {
			if (blk >= blk_end) {
				uint32_t base = 0;
				if (lane == 0) base = atomicAdd(counter, per_fetch);
				base = __shfl_sync(0xFFFFFFFFu, base, 0);
				if (base >= n) {
					exhausted = true;
					break;
				}
				blk = base;
				blk_end = n - base < per_fetch ? n : base + per_fetch;
			}
			const uint32_t ri = blk + (uint32_t)lane;
			blk += 32;
			bool enter = false;
			if (ri < blk_end) {
				const uint32_t m = segment_of(s_off, nmesh, ri);
				RayState r;
				load_ray(rays, ri, r);
				enter = r.tmin <= r.tmax && root_enter(nodes + m, nnodes - (int)m, r);
				if (!enter) hits[ri] = make_float4(0.f, __int_as_float((int)0xFFFFFFFFu), 0.f, 0.f);
			}
			const uint32_t mask = __ballot_sync(0xFFFFFFFFu, enter);
			if (mask == 0xFFFFFFFFu && qn == 0) {   // a full batch: trace it as it is
				i = ri;
				direct = true;
				break;
			}
			if (enter) q[qn + __popc(mask & ((1u << lane) - 1u))] = ri;
			qn += __popc(mask);
			__syncwarp();
			if (qn >= 32) break;
		}
		if (!direct) {
			if (qn == 0) break;   // rays and queue exhausted
			const int take = qn < 32 ? qn : 32;
			if (lane < take) i = q[qn - take + lane];
			__syncwarp();
			qn -= take;
		}
		if (i != 0xFFFFFFFFu)
			batch_trace_ray<WIDE, SDEPTH>(nodes, nnodes, wn, nwnodes, tris, ntris, rays, i, segment_of(s_off, nmesh, i),
			                              tri_off, hits, counter, sst);
	}
}

// rr::RRRay records (128-byte stride) in device memory: offsets of
// include/Lightsprint/RRCollider.h:85-137 on LP64.
constexpr int kRRRayStride = 128;

// keyed: each record carries a replay key in its hitPadding1 bytes (the
// reference also keeps collider scratch there, RRCollider/config.h:55):
// float key_t at byte 92, uint32 key_tri at 96; only hits after
// (key_t, key_tri) in the order (t, triangle) count, and the hit's own
// watertight t is written at byte 100.  Records of non-keyed launches are
// read and written at bytes 0..91 only.
__global__ void __launch_bounds__(kTraceThreads) k_rrray(const TNode* __restrict__ nodes, int nnodes,
                                                         const float4* __restrict__ tris, int ntris, uint8_t* rrrays,
                                                         uint32_t n, uint8_t* __restrict__ hit_out,
                                                         uint32_t* counter, int keyed) {
	const int lane = threadIdx.x & 31;
	while (true) {
		uint32_t base = warp_fetch(counter);
		if (base >= n) break;
		uint32_t i = base + lane;
		if (i >= n) continue;
		uint8_t* rec = rrrays + (size_t)i * kRRRayStride;
		float4 o = *reinterpret_cast<const float4*>(rec);
		float4 d = *reinterpret_cast<const float4*>(rec + 16);
		float4 lf = *reinterpret_cast<const float4*>(rec + 32);   // lengthMin, lengthMax, flags, hitDistance
		uint32_t flags = (uint32_t)__float_as_int(lf.z);
		RayState r;
		r.ox = o.x; r.oy = o.y; r.oz = o.z; r.tmin = lf.x;
		r.dx = d.x; r.dy = d.y; r.dz = d.z; r.tmax = lf.y;
		ray_setup(r);
		float tbest = r.tmax;
		uint32_t best_tri = 0xFFFFFFFFu;
		bool overflow = false;
		int slot = -1;
		if (keyed) {
			const float key_t = *reinterpret_cast<const float*>(rec + 92);
			const uint32_t key_tri = *reinterpret_cast<const uint32_t*>(rec + 96);
			if (key_t > r.tmin) r.tmin = key_t;
			if (r.tmin <= r.tmax)
				slot = traverse<false, false, true>(nodes, tris, r, nnodes, ntris, tbest, best_tri, overflow, nullptr,
				                                    0, key_t, key_tri);
			*reinterpret_cast<float*>(rec + 100) = tbest;
		} else if (r.tmin <= r.tmax) {
			slot = traverse<false>(nodes, tris, r, nnodes, ntris, tbest, best_tri, overflow);
		}
		if (overflow) atomicOr(counter + 1, (uint32_t)RRG_ERR_STACK);
		if (hit_out) hit_out[i] = slot >= 0 ? 1 : 0;
		if (slot < 0) continue;   // outputs undefined after a negative test (RRCollider.h:123)
		float4 a, b, c;
		load_tri(tris, slot, a, b, c);
		Fastest f = fastest_fields(r, a, b, c);
		float* rf = reinterpret_cast<float*>(rec);
		if (flags & RRG_FILL_DISTANCE) rf[11] = f.dist;
		if (flags & RRG_FILL_TRIANGLE) reinterpret_cast<uint32_t*>(rec)[12] = best_tri;
		if (flags & RRG_FILL_POINT2D) { rf[13] = f.u; rf[14] = f.v; }
		if (flags & RRG_FILL_PLANE) { rf[15] = f.n[0]; rf[16] = f.n[1]; rf[17] = f.n[2]; rf[18] = f.n[3]; }
		if (flags & RRG_FILL_POINT3D) {
			rf[19] = __fadd_rn(r.ox, __fmul_rn(r.dx, f.dist));
			rf[20] = __fadd_rn(r.oy, __fmul_rn(r.dy, f.dist));
			rf[21] = __fadd_rn(r.oz, __fmul_rn(r.dz, f.dist));
		}
		if (flags & RRG_FILL_SIDE) rec[88] = f.front ? 1 : 0;
	}
}

// ---------------------------------------------------------------------------
// Persistent while-while traversal with postponed leaves and per-lane refill
// (after Aila & Laine, "Understanding the efficiency of ray traversal on
// GPUs", HPG 2009): a lane that finishes its ray takes the next one at the
// top of the loop while the other lanes keep their traversal state; inner
// nodes are walked until every active lane holds a leaf, then the leaves are
// tested; stack entries carry their entry distance and are skipped once a
// closer hit is known.
constexpr int kSent = 0x7FFFFFFF;   // no current node

__device__ __forceinline__ int pop_entry(const int2* stack, int& sp, float tbest) {
	while (sp > 0) {
		int2 e = stack[--sp];
		if (__int_as_float(e.y) <= tbest) return e.x;
	}
	return kSent;
}

template <bool ANY>
__global__ void __launch_bounds__(kTraceThreads) k_trace_ww(const TNode* __restrict__ nodes, int nnodes,
                                                            const float4* __restrict__ tris, int ntris,
                                                            const float4* __restrict__ rays, uint32_t n,
                                                            float4* __restrict__ hits, float4* __restrict__ planes,
                                                            float* __restrict__ points, uint8_t* __restrict__ occ,
                                                            uint32_t* counter) {
	const int lane = threadIdx.x & 31;
	const unsigned lt = (1u << lane) - 1u;
	int2 stack[kStackSize];
	int sp = 0;
	RayState r;
	uint32_t ray = 0xFFFFFFFFu;
	int ref = kSent, leaf = kSent;
	float tbest = 0.f;
	uint32_t best_tri = 0xFFFFFFFFu;
	int best_slot = -1;
	bool overflow = false;
	bool exhausted = false;
	uint32_t steps = 0;
	while (true) {
		const bool done = (ref == kSent) && (leaf == kSent);
		if (done && ray != 0xFFFFFFFFu) {
			if (ANY) {
				occ[ray] = best_slot >= 0 ? 1 : 0;
			} else if (best_slot < 0) {
				hits[ray] = make_float4(0.f, __int_as_float((int)0xFFFFFFFFu), 0.f, 0.f);
				if (planes) planes[ray] = make_float4(0.f, 0.f, 0.f, 0.f);
				if (points) { points[3 * (size_t)ray] = 0.f; points[3 * (size_t)ray + 1] = 0.f; points[3 * (size_t)ray + 2] = 0.f; }
			} else {
				float4 a, b, c;
				load_tri(tris, best_slot, a, b, c);
				Fastest f = fastest_fields(r, a, b, c);
				hits[ray] = make_float4(f.dist, __int_as_float((int)(best_tri | (f.front ? 0x80000000u : 0u))), f.u, f.v);
				if (planes) planes[ray] = make_float4(f.n[0], f.n[1], f.n[2], f.n[3]);
				if (points) {
					points[3 * (size_t)ray] = __fadd_rn(r.ox, __fmul_rn(r.dx, f.dist));
					points[3 * (size_t)ray + 1] = __fadd_rn(r.oy, __fmul_rn(r.dy, f.dist));
					points[3 * (size_t)ray + 2] = __fadd_rn(r.oz, __fmul_rn(r.dz, f.dist));
				}
			}
			ray = 0xFFFFFFFFu;
		}
		const unsigned dmask = __ballot_sync(0xFFFFFFFFu, done);
		if (dmask && !exhausted) {
			const int cnt = __popc(dmask);
			uint32_t base = 0;
			if (lane == 0) base = atomicAdd(counter, (uint32_t)cnt);
			base = __shfl_sync(0xFFFFFFFFu, base, 0);
			if (done) {
				const uint32_t i = base + __popc(dmask & lt);
				if (i < n) {
					ray = i;
					float4 ra = __ldg(rays + 2 * (size_t)i), rb = __ldg(rays + 2 * (size_t)i + 1);
					r.ox = ra.x; r.oy = ra.y; r.oz = ra.z; r.tmin = ra.w;
					r.dx = rb.x; r.dy = rb.y; r.dz = rb.z; r.tmax = rb.w;
					ray_setup(r);
					tbest = r.tmax;
					best_tri = 0xFFFFFFFFu;
					best_slot = -1;
					sp = 0;
					steps = 0;
					ref = r.tmin <= r.tmax ? 0 : kSent;
					leaf = kSent;
				}
			}
			if (base + (uint32_t)cnt >= n) exhausted = true;
		}
		const bool active = !((ref == kSent) && (leaf == kSent));
		if (!__any_sync(0xFFFFFFFFu, active)) {
			if (exhausted) break;
			continue;
		}
		// inner nodes until every active lane holds a postponed leaf
		while (ref != kSent && ref >= 0) {
			if (ref >= nnodes || ++steps > kMaxSteps) { overflow = true; ref = kSent; leaf = kSent; break; }
			const float4* np = reinterpret_cast<const float4*>(nodes + ref);
			const float4 na = __ldg(np), nb = __ldg(np + 1), nc = __ldg(np + 2);
			const int4 nd = __ldg(reinterpret_cast<const int4*>(np + 3));
			const float t0 = nd.x != kEmptyRef ? box_enter(r, na.x, na.y, na.z, na.w, nc.x, nc.y, tbest) : INFINITY;
			const float t1 = nd.y != kEmptyRef ? box_enter(r, nb.x, nb.y, nb.z, nb.w, nc.z, nc.w, tbest) : INFINITY;
			const bool h0 = t0 != INFINITY, h1 = t1 != INFINITY;
			if (h0 && h1) {
				const bool first0 = t0 <= t1;
				if (sp < kStackSize) stack[sp++] = make_int2(first0 ? nd.y : nd.x, __float_as_int(first0 ? t1 : t0));
				else overflow = true;
				ref = first0 ? nd.x : nd.y;
			} else if (h0) {
				ref = nd.x;
			} else if (h1) {
				ref = nd.y;
			} else {
				ref = pop_entry(stack, sp, tbest);
			}
			if (ref != kSent && ref < 0 && leaf == kSent) {
				leaf = ref;
				ref = pop_entry(stack, sp, tbest);
			}
			if (__all_sync(__activemask(), leaf != kSent)) break;
		}
		// leaves
		while (leaf != kSent) {
			const int first = leaf & 0x07FFFFFF;
			const int count = ((leaf >> 27) & 15) + 1;
			leaf = kSent;
			if (first + count > ntris) { overflow = true; ref = kSent; break; }
			bool stop = false;
			for (int k = 0; k < count; k++) {
				float4 a, b, c;
				load_tri(tris, first + k, a, b, c);
				const uint32_t tri = (uint32_t)__float_as_int(a.w);
				float t;
				if (tri_test(r, a, b, c, tbest, tri, best_tri, t)) {
					tbest = t;
					best_tri = tri;
					best_slot = first + k;
					if (ANY) { stop = true; break; }
				}
			}
			if (stop) { ref = kSent; break; }
			if (ref != kSent && ref < 0) {
				leaf = ref;
				ref = pop_entry(stack, sp, tbest);
			}
		}
	}
	if (overflow) atomicOr(counter + 1, (uint32_t)RRG_ERR_STACK);
}

int trace_occupancy(Collider* c) {
	int per_sm = 0;
	RRG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_closest<false, false>, kTraceThreads, 0));
	c->trace_blocks = (per_sm > 0 ? per_sm : 1) * c->num_sms;
	RRG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_occluded<false, false>, kTraceThreads, 0));
	c->occl_blocks = (per_sm > 0 ? per_sm : 1) * c->num_sms;
	RRG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_ww<false>, kTraceThreads, 0));
	c->ww_blocks = (per_sm > 0 ? per_sm : 1) * c->num_sms;
	RRG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_closest_w, kTraceThreads, 0));
	c->wide_blocks = (per_sm > 0 ? per_sm : 1) * c->num_sms;
	return RRG_OK;
}

// Batches this large are binned first (rrg_binning.cu) unless the caller
// asked for the given order.
constexpr uint32_t kBinMinRays = 1u << 22;

static bool use_binning(const Collider* c, uint32_t n) {
	if (c->ray_order == RRG_RAY_ORDER_AS_GIVEN) return false;
	if (c->ray_order == RRG_RAY_ORDER_BINNED) return n >= 1024;
	return n >= kBinMinRays;
}

// words[0] = the launch's work counter (cleared here), words[1] = its status;
// bin_slot selects the binning scratch (one per concurrently running caller).
int launch_closest_on(Collider* c, const float4* rays, uint32_t n, float4* hits, float4* planes, float* points,
                      uint32_t* words, cudaStream_t s, int bin_slot) {
	if (!n) return RRG_OK;
	RRG_CUDA(cudaMemsetAsync(words, 0, 4, s));
	uint32_t want = (n + 31) / 32 * 32 / kTraceThreads + 1;
	if (c->width == 8 && c->d_wnodes) {
		int grid = (int)(want < (uint32_t)c->wide_blocks ? want : (uint32_t)c->wide_blocks);
		int st = trace_event(c, s, false);
		if (st) return st;
		rrg::note_launch(), k_closest_w<<<grid, kTraceThreads, 0, s>>>(c->d_wnodes, (int)c->nwnodes, c->d_wtris, (int)c->nvalid, rays, n,
		                                           hits, planes, points, words);
		RRG_CUDA(cudaGetLastError());
		return trace_event(c, s, true);
	}
	if (c->traversal == RRG_TRAVERSAL_COMPACT) {
		const uint32_t* perm = nullptr;
		if (use_binning(c, n)) {
			int st = bin_rays(c, rays, n, s, bin_slot, &perm);
			if (st) return st;
		}
		int st = trace_event(c, s, false);
		if (!st) st = launch_compact(c, rays, n, hits, planes, points, nullptr, words, perm, s);
		return st ? st : trace_event(c, s, true);
	}
	if (c->traversal == RRG_TRAVERSAL_WHILE_WHILE) {
		int grid = (int)(want < (uint32_t)c->ww_blocks ? want : (uint32_t)c->ww_blocks);
		int st = trace_event(c, s, false);
		if (st) return st;
		rrg::note_launch(), k_trace_ww<false><<<grid, kTraceThreads, 0, s>>>(c->d_nodes, (int)c->nnodes, c->d_tris, (int)c->nvalid, rays,
		                                                  n, hits, planes, points, nullptr, words);
		RRG_CUDA(cudaGetLastError());
		return trace_event(c, s, true);
	}
	int grid = (int)(want < (uint32_t)c->trace_blocks ? want : (uint32_t)c->trace_blocks);
	const bool queue = c->traversal == RRG_TRAVERSAL_ROOT_QUEUE;
	const uint32_t* perm = nullptr;
	if (use_binning(c, n)) {
		int st = bin_rays(c, rays, n, s, bin_slot, &perm);
		if (st) return st;
	}
	auto kernel = perm ? (queue ? k_closest<true, true> : k_closest<true, false>)
	                   : (queue ? k_closest<false, true> : k_closest<false, false>);
	int st = trace_event(c, s, false);
	if (st) return st;
	rrg::note_launch(), kernel<<<grid, kTraceThreads, 0, s>>>(c->d_nodes, (int)c->nnodes, c->d_tris, (int)c->nvalid, rays, n,
	                                                          hits, planes, points, words, perm);
	RRG_CUDA(cudaGetLastError());
	return trace_event(c, s, true);
}

int trace_event(Collider* c, cudaStream_t s, bool end) {
	if (!c->timing || c->tev_n >= 256) return RRG_OK;
	cudaEvent_t& e = c->tev[2 * c->tev_n + (end ? 1 : 0)];
	if (!e) RRG_CUDA(cudaEventCreate(&e));
	RRG_CUDA(cudaEventRecord(e, s));
	if (end) c->tev_n++;
	return RRG_OK;
}

// Rays and hit records in page-locked host memory, read and written by the
// kernel over the host link: the if-if kernel in the given order, so that a
// warp writes its 32 hit records as one contiguous 512-byte run (the
// root-box queue's and the binned order's scattered 16-byte writes cost
// more over the link than they save: 3.3 against 4.0 Grays/s on config 0).
int launch_closest_mapped(Collider* c, const float4* rays, uint32_t n, float4* hits, cudaStream_t s) {
	if (!n) return RRG_OK;
	if (c->width == 8 && c->d_wnodes) return launch_closest(c, rays, n, hits, nullptr, nullptr, s);
	uint32_t* words = c->d_counter;
	RRG_CUDA(cudaMemsetAsync(words, 0, 4, s));
	const uint32_t want = (n + 31) / 32 * 32 / kTraceThreads + 1;
	const int grid = (int)(want < (uint32_t)c->trace_blocks ? want : (uint32_t)c->trace_blocks);
	int st = trace_event(c, s, false);
	if (st) return st;
	rrg::note_launch(), k_closest<false, false><<<grid, kTraceThreads, 0, s>>>(
	    c->d_nodes, (int)c->nnodes, c->d_tris, (int)c->nvalid, rays, n, hits, nullptr, nullptr, words, nullptr);
	RRG_CUDA(cudaGetLastError());
	return trace_event(c, s, true);
}

int launch_closest(Collider* c, const float4* rays, uint32_t n, float4* hits, float4* planes, float* points,
                   cudaStream_t s) {
	return launch_closest_on(c, rays, n, hits, planes, points, c->d_counter, s, 3);
}

int launch_occluded(Collider* c, const float4* rays, uint32_t n, uint8_t* occ, cudaStream_t s) {
	if (!n) return RRG_OK;
	if (c->traversal == RRG_TRAVERSAL_COMPACT && !(c->width == 8 && c->d_wnodes)) {
		const uint32_t* perm = nullptr;
		if (use_binning(c, n)) {
			int st = bin_rays(c, rays, n, s, 3, &perm);
			if (st) return st;
		}
		return launch_compact(c, rays, n, nullptr, nullptr, nullptr, occ, c->d_counter, perm, s);
	}
	RRG_CUDA(cudaMemsetAsync(c->d_counter, 0, 4, s));
	uint32_t want = (n + 31) / 32 * 32 / kTraceThreads + 1;
	if (c->width == 8 && c->d_wnodes) {
		int grid = (int)(want < (uint32_t)c->wide_blocks ? want : (uint32_t)c->wide_blocks);
		rrg::note_launch(), k_occluded_w<<<grid, kTraceThreads, 0, s>>>(c->d_wnodes, (int)c->nwnodes, c->d_wtris, (int)c->nvalid, rays,
		                                            n, occ, c->d_counter);
		RRG_CUDA(cudaGetLastError());
		return RRG_OK;
	}
	if (c->traversal == RRG_TRAVERSAL_WHILE_WHILE) {
		int grid = (int)(want < (uint32_t)c->ww_blocks ? want : (uint32_t)c->ww_blocks);
		rrg::note_launch(), k_trace_ww<true><<<grid, kTraceThreads, 0, s>>>(c->d_nodes, (int)c->nnodes, c->d_tris, (int)c->nvalid, rays,
		                                                 n, nullptr, nullptr, nullptr, occ, c->d_counter);
		RRG_CUDA(cudaGetLastError());
		return RRG_OK;
	}
	int grid = (int)(want < (uint32_t)c->occl_blocks ? want : (uint32_t)c->occl_blocks);
	const bool queue = c->traversal == RRG_TRAVERSAL_ROOT_QUEUE;
	const uint32_t* perm = nullptr;
	if (use_binning(c, n)) {
		int st = bin_rays(c, rays, n, s, 3, &perm);
		if (st) return st;
	}
	auto kernel = perm ? (queue ? k_occluded<true, true> : k_occluded<true, false>)
	                   : (queue ? k_occluded<false, true> : k_occluded<false, false>);
	rrg::note_launch(), kernel<<<grid, kTraceThreads, 0, s>>>(c->d_nodes, (int)c->nnodes, c->d_tris, (int)c->nvalid, rays, n,
	                                                          occ, c->d_counter, perm);
	RRG_CUDA(cudaGetLastError());
	return RRG_OK;
}

int launch_rrray(Collider* c, void* rrrays_dev, uint32_t n, uint8_t* hit_dev, cudaStream_t s) {
	if (!n) return RRG_OK;
	RRG_CUDA(cudaMemsetAsync(c->d_counter, 0, 4, s));
	uint32_t want = (n + 31) / 32 * 32 / kTraceThreads + 1;
	int grid = (int)(want < (uint32_t)c->trace_blocks ? want : (uint32_t)c->trace_blocks);
	rrg::note_launch(), k_rrray<<<grid, kTraceThreads, 0, s>>>(c->d_nodes, (int)c->nnodes, c->d_tris, (int)c->nvalid, (uint8_t*)rrrays_dev, n, hit_dev, c->d_counter, 0);
	RRG_CUDA(cudaGetLastError());
	return RRG_OK;
}

// k_rrray on caller-owned scratch words ([0] work counter, [1] status), which
// the caller has cleared on stream s; keyed as k_rrray's argument.
int launch_rrray_scratch(Collider* c, void* rrrays_dev, uint32_t n, uint8_t* hit_dev, uint32_t* words,
                         cudaStream_t s, int keyed) {
	if (!n) return RRG_OK;
	uint32_t want = (n + 31) / 32 * 32 / kTraceThreads + 1;
	int grid = (int)(want < (uint32_t)c->trace_blocks ? want : (uint32_t)c->trace_blocks);
	rrg::note_launch(), k_rrray<<<grid, kTraceThreads, 0, s>>>(c->d_nodes, (int)c->nnodes, c->d_tris, (int)c->nvalid, (uint8_t*)rrrays_dev, n, hit_dev, words, keyed);
	RRG_CUDA(cudaGetLastError());
	return RRG_OK;
}

using BatchKernel = void (*)(const TNode*, int, const uint4*, int, const float4*, int, const float4*, uint32_t,
                             const uint32_t*, const uint32_t*, uint32_t, int, float4*, uint32_t*);

// k_batch_closest for the tree width and the shared-memory stack depth
// (0, 8, 16 or 32 entries; the wide walk keeps its own local stack);
// mode = entries | kBatchRootQueue for the root-box queue (binary tree)
static BatchKernel binary_batch_kernel(uint32_t mode) {
	const bool q = (mode & kBatchRootQueue) != 0;
	switch (mode & ~kBatchRootQueue) {
		case 8: return q ? k_batch_closest<false, 8, true> : k_batch_closest<false, 8, false>;
		case 16: return q ? k_batch_closest<false, 16, true> : k_batch_closest<false, 16, false>;
		case 32: return q ? k_batch_closest<false, 32, true> : k_batch_closest<false, 32, false>;
		default: return q ? k_batch_closest<false, 0, true> : k_batch_closest<false, 0, false>;
	}
}

static BatchKernel batch_kernel(const Collider* c, uint32_t mode) {
	if (c->width == 8 && c->d_wnodes) return k_batch_closest<true, 0, false>;
	return binary_batch_kernel(mode);
}

int batch_trace_blocks(Collider* c, uint32_t nmesh, uint32_t sdepth, int* blocks) {
	int per_sm = 0;
	RRG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel(c, sdepth), kTraceThreads,
	                                                       sizeof(uint32_t) * (nmesh + 1)));
	*blocks = (per_sm > 0 ? per_sm : 1) * c->num_sms;
	return RRG_OK;
}

// Clears the work counter and launches k_batch_closest on stream s (both
// stream-ordered, so the pair can be captured in a CUDA graph).
int launch_batch_closest_on(Collider* c, const TNode* nodes, int nnodes, const float4* tris, int ntris,
                            const float4* rays, uint32_t n, const uint32_t* ray_off, uint32_t nmesh, int fetch,
                            int blocks, uint32_t sdepth, float4* hits, cudaStream_t s) {
	if (!n) return RRG_OK;
	RRG_CUDA(cudaMemsetAsync(c->d_counter, 0, 4, s));
	const uint32_t per_fetch = 32u * (uint32_t)fetch;
	const uint32_t want = (uint32_t)(((uint64_t)n + per_fetch - 1) / per_fetch * 32 / kTraceThreads + 1);
	const int grid = (int)(want < (uint32_t)blocks ? want : (uint32_t)blocks);
	const size_t smem = sizeof(uint32_t) * (nmesh + 1);
	BatchKernel k = binary_batch_kernel(sdepth);
	rrg::note_launch(), k<<<grid, kTraceThreads, smem, s>>>(nodes, nnodes, nullptr, 0, tris, ntris, rays, n, ray_off,
	                                                      c->d_tri_off, nmesh, fetch, hits, c->d_counter);
	RRG_CUDA(cudaGetLastError());
	return RRG_OK;
}

int launch_batch_closest(Collider* c, const float4* rays, uint32_t n, const uint32_t* ray_off, uint32_t nmesh,
                         int fetch, int blocks, uint32_t sdepth, float4* hits, cudaStream_t s) {
	if (!n) return RRG_OK;
	RRG_CUDA(cudaMemsetAsync(c->d_counter, 0, 4, s));
	const uint32_t per_fetch = 32u * (uint32_t)fetch;
	const uint32_t want = (uint32_t)(((uint64_t)n + per_fetch - 1) / per_fetch * 32 / kTraceThreads + 1);
	const int grid = (int)(want < (uint32_t)blocks ? want : (uint32_t)blocks);
	const size_t smem = sizeof(uint32_t) * (nmesh + 1);
	const bool wide = c->width == 8 && c->d_wnodes;
	rrg::note_launch(), batch_kernel(c, sdepth)<<<grid, kTraceThreads, smem, s>>>(
	    c->d_nodes, (int)c->nnodes, c->d_wnodes, (int)c->nwnodes, wide ? c->d_wtris : c->d_tris, (int)c->nvalid, rays,
	    n, ray_off, c->d_tri_off, nmesh, fetch, hits, c->d_counter);
	RRG_CUDA(cudaGetLastError());
	return RRG_OK;
}

}  // namespace rrg
