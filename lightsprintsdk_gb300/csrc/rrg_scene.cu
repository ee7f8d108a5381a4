// Two-level scene collider (include/rrgpu_scene.h): objects are instances of
// a batch's meshes under world matrices; a top-level BVH over the objects'
// world boxes, built on the host, selects the objects a ray reaches, and
// each reached object is intersected in its own space from its mesh's root
// in the batch's multi-root tree.
#include "rrg_traverse.cuh"

#include "../../include/rrgpu_scene.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <new>
#include <vector>

namespace rrg {

// Per object, 64 bytes: inverse world matrix (row-major 3 x 4), mesh (=
// root node), 1 if the matrix has a negative determinant, the mesh's first
// triangle in the batch.
struct SceneObj {
	float inv[12];
	uint32_t mesh;
	uint32_t neg;
	uint32_t tri_base;
	uint32_t pad;
};

struct Scene {
	::rrg_batch* batch = nullptr;
	Collider* c = nullptr;            // the batch's geometry (not owned)
	uint32_t nobj = 0;
	std::vector<uint32_t> obj_mesh;
	std::vector<float> world;         // 12 per object
	std::vector<uint8_t> enabled;
	std::vector<float> mesh_lo, mesh_hi;   // local box of each mesh (3 per mesh)
	SceneObj* d_obj = nullptr;
	TNode* d_tl = nullptr;            // top-level nodes
	uint32_t* d_tl_obj = nullptr;     // objects in top-level leaf order
	uint32_t ntl = 0, ntl_obj = 0;
	size_t cap_tl = 0, cap_tl_obj = 0;
	uint32_t* d_counter = nullptr;    // [0] work counter, [1] status
	int blocks = 0;
	// host-buffer queries (rrg_scene_intersect_host): one staging buffer
	// (rays, then hits, then objects), grown on demand; callers take turns
	std::mutex host_mu;
	void* d_stage = nullptr;
	uint32_t stage_cap = 0;
	cudaStream_t s_host = nullptr;
};

// RRMatrix3x4::determinant3x3 and invertedTo (RRMath.cpp:605-628) in float,
// in the same order of operations (the library is compiled without
// floating-point contraction), so that object-space rays match the
// reference's.
static float det3x3(const float* m) {
	return m[0] * (m[5] * m[10] - m[9] * m[6]) + m[1] * (m[6] * m[8] - m[10] * m[4]) +
	       m[2] * (m[4] * m[9] - m[8] * m[5]);
}

static bool invert3x4(const float* m, float* d) {
	const float det = det3x3(m);
	if (!det || !isfinite(det)) return false;
	d[0] = +(m[10] * m[5] - m[9] * m[6]) / det;
	d[1] = -(m[10] * m[1] - m[9] * m[2]) / det;
	d[2] = +(m[6] * m[1] - m[5] * m[2]) / det;
	d[4] = -(m[10] * m[4] - m[8] * m[6]) / det;
	d[5] = +(m[10] * m[0] - m[8] * m[2]) / det;
	d[6] = -(m[6] * m[0] - m[4] * m[2]) / det;
	d[8] = +(m[9] * m[4] - m[8] * m[5]) / det;
	d[9] = -(m[9] * m[0] - m[8] * m[1]) / det;
	d[10] = +(m[5] * m[0] - m[4] * m[1]) / det;
	d[3] = -m[3] * d[0] - m[7] * d[1] - m[11] * d[2];
	d[7] = -m[3] * d[4] - m[7] * d[5] - m[11] * d[6];
	d[11] = -m[3] * d[8] - m[7] * d[9] - m[11] * d[10];
	return true;
}

struct HBox {
	float lo[3], hi[3];
};

static HBox box_union(const HBox& a, const HBox& b) {
	HBox r;
	for (int k = 0; k < 3; k++) {
		r.lo[k] = std::min(a.lo[k], b.lo[k]);
		r.hi[k] = std::max(a.hi[k], b.hi[k]);
	}
	return r;
}

static HBox box_empty() {
	HBox r;
	for (int k = 0; k < 3; k++) { r.lo[k] = INFINITY; r.hi[k] = -INFINITY; }
	return r;
}

// Top-level BVH over object boxes: object-median splits on the longest axis
// of the centroids, leaves of at most 2 objects, emitted as TNodes (root =
// node 0); returns the subtree's reference and box.
struct TlasBuilder {
	const std::vector<HBox>& boxes;
	std::vector<TNode> nodes;
	std::vector<uint32_t> leaf_objs;
	explicit TlasBuilder(const std::vector<HBox>& b) : boxes(b) {}

	int build(uint32_t* ids, int n, HBox& out) {
		out = box_empty();
		for (int i = 0; i < n; i++) out = box_union(out, boxes[ids[i]]);
		if (n <= 2) {
			const int first = (int)leaf_objs.size();
			for (int i = 0; i < n; i++) leaf_objs.push_back(ids[i]);
			return leaf_ref(first, n);
		}
		float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
		for (int i = 0; i < n; i++)
			for (int k = 0; k < 3; k++) {
				const float c = 0.5f * (boxes[ids[i]].lo[k] + boxes[ids[i]].hi[k]);
				clo[k] = std::min(clo[k], c);
				chi[k] = std::max(chi[k], c);
			}
		int axis = 0;
		for (int k = 1; k < 3; k++)
			if (chi[k] - clo[k] > chi[axis] - clo[axis]) axis = k;
		const int mid = n / 2;
		std::nth_element(ids, ids + mid, ids + n, [&](uint32_t a, uint32_t b) {
			const float ca = boxes[a].lo[axis] + boxes[a].hi[axis], cb = boxes[b].lo[axis] + boxes[b].hi[axis];
			return ca < cb || (ca == cb && a < b);
		});
		const int idx = (int)nodes.size();
		nodes.push_back(TNode{});
		HBox lb, rb;
		const int l = build(ids, mid, lb);
		const int r = build(ids + mid, n - mid, rb);
		TNode t;
		t.a = make_float4(lb.lo[0], lb.hi[0], lb.lo[1], lb.hi[1]);
		t.b = make_float4(rb.lo[0], rb.hi[0], rb.lo[1], rb.hi[1]);
		t.c = make_float4(lb.lo[2], lb.hi[2], rb.lo[2], rb.hi[2]);
		t.d = make_int4(l, r, 0, 0);
		nodes[idx] = t;
		return idx;
	}
};

// Object-space ray of RRColliderMulti::intersect (RRColliderMulti.cpp:121-131):
// o' = inv o (RRMatrix3x4::transformPosition), d' = inv d (transformDirection),
// scale = |d'|, d' /= scale, lengths *= scale; one rounding per operation.
__device__ __forceinline__ float local_ray(const SceneObj& so, const RayState& w, RayState& r) {
	const float* m = so.inv;
	r.ox = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(w.ox, m[0]), __fmul_rn(w.oy, m[1])), __fmul_rn(w.oz, m[2])), m[3]);
	r.oy = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(w.ox, m[4]), __fmul_rn(w.oy, m[5])), __fmul_rn(w.oz, m[6])), m[7]);
	r.oz = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(w.ox, m[8]), __fmul_rn(w.oy, m[9])), __fmul_rn(w.oz, m[10])), m[11]);
	float dx = __fadd_rn(__fadd_rn(__fmul_rn(w.dx, m[0]), __fmul_rn(w.dy, m[1])), __fmul_rn(w.dz, m[2]));
	float dy = __fadd_rn(__fadd_rn(__fmul_rn(w.dx, m[4]), __fmul_rn(w.dy, m[5])), __fmul_rn(w.dz, m[6]));
	float dz = __fadd_rn(__fadd_rn(__fmul_rn(w.dx, m[8]), __fmul_rn(w.dy, m[9])), __fmul_rn(w.dz, m[10]));
	const float scale = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
	r.dx = __fdiv_rn(dx, scale);
	r.dy = __fdiv_rn(dy, scale);
	r.dz = __fdiv_rn(dz, scale);
	r.tmin = __fmul_rn(w.tmin, scale);
	r.tmax = __fmul_rn(w.tmax, scale);
	ray_setup(r);
	return scale;
}

__device__ __forceinline__ void load_obj(const SceneObj* __restrict__ objs, uint32_t o, SceneObj& so) {
	const float4* p = reinterpret_cast<const float4*>(objs + o);
	const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3);
	so.inv[0] = a.x; so.inv[1] = a.y; so.inv[2] = a.z; so.inv[3] = a.w;
	so.inv[4] = b.x; so.inv[5] = b.y; so.inv[6] = b.z; so.inv[7] = b.w;
	so.inv[8] = c.x; so.inv[9] = c.y; so.inv[10] = c.z; so.inv[11] = c.w;
	so.mesh = __float_as_uint(d.x);
	so.neg = __float_as_uint(d.y);
	so.tri_base = __float_as_uint(d.z);
}

constexpr int kTopStack = 32;

// Closest hit over the scene.  The top-level walk prunes with the world
// distance of the best hit so far; each reached object is traced from its
// mesh's root with the local bound tbest * scale (enlarged by 2^-20 so no
// hit that can still win is pruned by the rounding of the product), and
// its candidate competes on world distance t / scale (ties: lower object).
// The reported fields are the FASTEST fields of the winner in its object
// space, the distance divided by scale, the side flipped for a mirroring
// matrix.
__global__ void __launch_bounds__(kTraceThreads) k_scene_closest(
    const TNode* __restrict__ tl, int ntl, const uint32_t* __restrict__ tl_obj, int ntl_obj,
    const SceneObj* __restrict__ objs, int nobj, const TNode* __restrict__ nodes, int nnodes,
    const float4* __restrict__ tris, int ntris, const float4* __restrict__ rays, uint32_t n,
    float4* __restrict__ hits, uint32_t* __restrict__ hit_obj, uint32_t* counter) {
	const int lane = threadIdx.x & 31;
	while (true) {
		uint32_t base = 0;
		if (lane == 0) base = atomicAdd(counter, 32u);
		base = __shfl_sync(0xFFFFFFFFu, base, 0);
		if (base >= n) break;
		const uint32_t i = base + lane;
		if (i >= n) continue;
		RayState w;
		{
			const float4 a = __ldg(rays + 2 * (size_t)i), b = __ldg(rays + 2 * (size_t)i + 1);
			w.ox = a.x; w.oy = a.y; w.oz = a.z; w.tmin = a.w;
			w.dx = b.x; w.dy = b.y; w.dz = b.z; w.tmax = b.w;
			ray_setup(w);
		}
		float tbest = w.tmax;
		int best_obj = -1, best_slot = -1;
		uint32_t best_tri = 0xFFFFFFFFu;
		bool overflow = false;
		if (ntl > 0 && w.tmin <= w.tmax) {
			int stack[kTopStack];
			int sp = 0;
			int ref = 0;
			for (uint32_t steps = 0;; steps++) {
				if (steps >= kMaxSteps) { overflow = true; break; }
				if (ref >= 0) {
					if (ref >= ntl) { overflow = true; break; }
					const float4* np = reinterpret_cast<const float4*>(tl + ref);
					const float4 na = __ldg(np), nb = __ldg(np + 1), nc = __ldg(np + 2);
					const int4 nd = __ldg(reinterpret_cast<const int4*>(np + 3));
					const float t0 = nd.x != kEmptyRef ? box_enter(w, na.x, na.y, na.z, na.w, nc.x, nc.y, tbest) : INFINITY;
					const float t1 = nd.y != kEmptyRef ? box_enter(w, nb.x, nb.y, nb.z, nb.w, nc.z, nc.w, tbest) : INFINITY;
					const bool h0 = t0 != INFINITY, h1 = t1 != INFINITY;
					if (h0 && h1) {
						if (sp < kTopStack) stack[sp++] = t0 <= t1 ? nd.y : nd.x;
						else { overflow = true; break; }
						ref = t0 <= t1 ? nd.x : nd.y;
						continue;
					}
					if (h0) { ref = nd.x; continue; }
					if (h1) { ref = nd.y; continue; }
				} else {
					const int first = ref & 0x07FFFFFF;
					const int count = ((ref >> 27) & 15) + 1;
					if (first + count > ntl_obj) { overflow = true; break; }
					for (int k = 0; k < count; k++) {
						const uint32_t o = __ldg(tl_obj + first + k);
						if (o >= (uint32_t)nobj) { overflow = true; break; }
						SceneObj so;
						load_obj(objs, o, so);
						RayState r;
						const float scale = local_ray(so, w, r);
						if (!(scale > 0.f) || !isfinite(scale)) continue;
						float tb = fminf(r.tmax, __fmul_rn(__fmul_rn(tbest, scale), 1.00000095367431640625f));
						uint32_t bt = 0xFFFFFFFFu;
						const int slot = traverse<false>(nodes, tris, r, nnodes, ntris, tb, bt, overflow, nullptr,
						                                 (int)so.mesh);
						if (slot < 0) continue;
						const float tw = __fdiv_rn(tb, scale);
						if (tw < tbest || (tw == tbest && (int)o < best_obj)) {
							tbest = tw;
							best_obj = (int)o;
							best_slot = slot;
							best_tri = bt;
						}
					}
				}
				if (sp == 0) break;
				ref = stack[--sp];
			}
		}
		if (overflow) atomicOr(counter + 1, (uint32_t)RRG_ERR_STACK);
		if (best_obj < 0) {
			hits[i] = make_float4(0.f, __int_as_float((int)0xFFFFFFFFu), 0.f, 0.f);
			if (hit_obj) hit_obj[i] = 0xFFFFFFFFu;
			continue;
		}
		SceneObj so;
		load_obj(objs, (uint32_t)best_obj, so);
		RayState r;
		const float scale = local_ray(so, w, r);
		float4 a, b, c;
		load_tri(tris, best_slot, a, b, c);
		const Fastest f = fastest_fields(r, a, b, c);
		const bool front = so.neg ? !f.front : f.front;
		const uint32_t bits = (best_tri - so.tri_base) | (front ? 0x80000000u : 0u);
		hits[i] = make_float4(__fdiv_rn(f.dist, scale), __int_as_float((int)bits), f.u, f.v);
		if (hit_obj) hit_obj[i] = (uint32_t)best_obj;
	}
}

// Inverses, object records and the top-level tree from the current
// matrices and enabled flags; uploads them.
static int rebuild(Scene* S) {
	const uint32_t nobj = S->nobj;
	std::vector<SceneObj> objs(nobj);
	std::vector<HBox> boxes(nobj);
	std::vector<uint32_t> ids;
	std::vector<uint32_t> tri_off(S->c->nroots + 1);
	RRG_CUDA(cudaMemcpy(tri_off.data(), S->c->d_tri_off, sizeof(uint32_t) * tri_off.size(), cudaMemcpyDeviceToHost));
	double maxc = 0.0;
	for (uint32_t o = 0; o < nobj; o++) {
		const float* m = &S->world[12 * (size_t)o];
		SceneObj& so = objs[o];
		memset(&so, 0, sizeof(so));
		if (!invert3x4(m, so.inv)) return RRG_ERR_INVALID;
		const uint32_t mesh = S->obj_mesh[o];
		so.mesh = mesh;
		so.neg = det3x3(m) < 0.f ? 1u : 0u;
		so.tri_base = tri_off[mesh];
		// world box: the 8 corners of the mesh's local box
		HBox wb = box_empty();
		const float* lo = &S->mesh_lo[3 * (size_t)mesh];
		const float* hi = &S->mesh_hi[3 * (size_t)mesh];
		if (!(lo[0] <= hi[0] && lo[1] <= hi[1] && lo[2] <= hi[2])) continue;   // mesh without valid triangles
		double wlo[3] = {INFINITY, INFINITY, INFINITY}, whi[3] = {-INFINITY, -INFINITY, -INFINITY};
		for (int k = 0; k < 8; k++) {
			const double p[3] = {(k & 1) ? hi[0] : lo[0], (k & 2) ? hi[1] : lo[1], (k & 4) ? hi[2] : lo[2]};
			for (int r = 0; r < 3; r++) {
				const double v = (double)m[4 * r] * p[0] + (double)m[4 * r + 1] * p[1] + (double)m[4 * r + 2] * p[2] +
				                 (double)m[4 * r + 3];
				wlo[r] = std::min(wlo[r], v);
				whi[r] = std::max(whi[r], v);
			}
		}
		for (int r = 0; r < 3; r++) {
			wb.lo[r] = (float)wlo[r];
			wb.hi[r] = (float)whi[r];
			maxc = std::max(maxc, std::max(fabs(wlo[r]), fabs(whi[r])));
		}
		boxes[o] = wb;
		if (S->enabled[o]) ids.push_back(o);
	}
	// widen each box by 2^-20 of its coordinates and of the scene's largest
	// coordinate, rounding outward: the object-space transform of a ray that
	// grazes a box is rounded, the box test must not reject it
	const double pad = maxc * 9.5367431640625e-07;
	for (uint32_t o : ids) {
		HBox& b = boxes[o];
		for (int r = 0; r < 3; r++) {
			b.lo[r] = nextafterf((float)(b.lo[r] - (fabs(b.lo[r]) * 9.5367431640625e-07 + pad)), -INFINITY);
			b.hi[r] = nextafterf((float)(b.hi[r] + (fabs(b.hi[r]) * 9.5367431640625e-07 + pad)), INFINITY);
		}
	}
	TlasBuilder tb(boxes);
	if (!ids.empty()) {
		HBox rootb;
		const int root = tb.build(ids.data(), (int)ids.size(), rootb);
		if (root < 0) {   // a root that is a leaf: wrap it in a one-child node
			TNode t;
			t.a = make_float4(rootb.lo[0], rootb.hi[0], rootb.lo[1], rootb.hi[1]);
			t.b = make_float4(INFINITY, -INFINITY, INFINITY, -INFINITY);
			t.c = make_float4(rootb.lo[2], rootb.hi[2], INFINITY, -INFINITY);
			t.d = make_int4(root, kEmptyRef, 0, 0);
			tb.nodes.push_back(t);
		}
	}
	RRG_CUDA(cudaMemcpy(S->d_obj, objs.data(), sizeof(SceneObj) * nobj, cudaMemcpyHostToDevice));
	if (tb.nodes.size() > S->cap_tl) {
		cudaFree(S->d_tl);
		S->d_tl = nullptr;
		S->cap_tl = 0;
		RRG_CUDA(cudaMalloc(&S->d_tl, sizeof(TNode) * tb.nodes.size()));
		S->cap_tl = tb.nodes.size();
	}
	if (tb.leaf_objs.size() > S->cap_tl_obj) {
		cudaFree(S->d_tl_obj);
		S->d_tl_obj = nullptr;
		S->cap_tl_obj = 0;
		RRG_CUDA(cudaMalloc(&S->d_tl_obj, sizeof(uint32_t) * tb.leaf_objs.size()));
		S->cap_tl_obj = tb.leaf_objs.size();
	}
	if (!tb.nodes.empty())
		RRG_CUDA(cudaMemcpy(S->d_tl, tb.nodes.data(), sizeof(TNode) * tb.nodes.size(), cudaMemcpyHostToDevice));
	if (!tb.leaf_objs.empty())
		RRG_CUDA(cudaMemcpy(S->d_tl_obj, tb.leaf_objs.data(), sizeof(uint32_t) * tb.leaf_objs.size(),
		                    cudaMemcpyHostToDevice));
	S->ntl = (uint32_t)tb.nodes.size();
	S->ntl_obj = (uint32_t)tb.leaf_objs.size();
	return RRG_OK;
}

static void free_scene(Scene* S) {
	if (!S) return;
	cudaFree(S->d_obj);
	cudaFree(S->d_tl);
	cudaFree(S->d_tl_obj);
	cudaFree(S->d_counter);
	cudaFree(S->d_stage);
	if (S->s_host) cudaStreamDestroy(S->s_host);
	delete S;
}

}  // namespace rrg

using namespace rrg;

extern "C" {

int rrg_scene_create(rrg_batch* meshes, uint32_t nobj, const uint32_t* obj_mesh, const float* world_3x4,
                     rrg_scene** out) {
	if (!out) return RRG_ERR_INVALID;
	*out = nullptr;
	Collider* c = batch_collider(meshes);
	if (!c || !nobj || !obj_mesh || !world_3x4) return RRG_ERR_INVALID;
	for (uint32_t o = 0; o < nobj; o++)
		if (obj_mesh[o] >= c->nroots) return RRG_ERR_INVALID;
	RRG_CUDA(cudaSetDevice(c->device));
	Scene* S = new (std::nothrow) Scene();
	if (!S) return RRG_ERR_OOM;
	S->batch = meshes;
	S->c = c;
	S->nobj = nobj;
	S->obj_mesh.assign(obj_mesh, obj_mesh + nobj);
	S->world.assign(world_3x4, world_3x4 + 12 * (size_t)nobj);
	S->enabled.assign(nobj, 1);
	// local box of each mesh: the union of its root node's child boxes
	const uint32_t M = c->nroots;
	std::vector<TNode> roots(M);
	int st = RRG_OK;
	cudaError_t e = cudaMemcpy(roots.data(), c->d_nodes, sizeof(TNode) * M, cudaMemcpyDeviceToHost);
	if (e != cudaSuccess) st = cuda_fail(e);
	S->mesh_lo.assign(3 * (size_t)M, INFINITY);
	S->mesh_hi.assign(3 * (size_t)M, -INFINITY);
	for (uint32_t m = 0; m < M && !st; m++) {
		const TNode& t = roots[m];
		const float cb[2][6] = {{t.a.x, t.a.y, t.a.z, t.a.w, t.c.x, t.c.y}, {t.b.x, t.b.y, t.b.z, t.b.w, t.c.z, t.c.w}};
		const int refs[2] = {t.d.x, t.d.y};
		for (int k = 0; k < 2; k++) {
			if (refs[k] == kEmptyRef) continue;
			for (int a = 0; a < 3; a++) {
				S->mesh_lo[3 * m + a] = std::min(S->mesh_lo[3 * m + a], cb[k][2 * a]);
				S->mesh_hi[3 * m + a] = std::max(S->mesh_hi[3 * m + a], cb[k][2 * a + 1]);
			}
		}
	}
	if (!st) {
		e = cudaMalloc(&S->d_obj, sizeof(SceneObj) * nobj);
		if (e == cudaSuccess) e = cudaMalloc(&S->d_counter, 64);
		if (e == cudaSuccess) e = cudaMemset(S->d_counter, 0, 64);
		if (e != cudaSuccess) st = cuda_fail(e);
	}
	if (!st) st = rebuild(S);
	if (!st) {
		int per_sm = 0;
		e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_scene_closest, kTraceThreads, 0);
		if (e != cudaSuccess) st = cuda_fail(e);
		S->blocks = (per_sm > 0 ? per_sm : 1) * c->num_sms;
	}
	if (st) {
		free_scene(S);
		return st;
	}
	*out = reinterpret_cast<rrg_scene*>(S);
	return RRG_OK;
}

void rrg_scene_destroy(rrg_scene* h) {
	Scene* S = reinterpret_cast<Scene*>(h);
	if (!S) return;
	cudaSetDevice(S->c->device);
	cudaDeviceSynchronize();
	free_scene(S);
}

int rrg_scene_set_matrices(rrg_scene* h, const float* world_3x4) {
	Scene* S = reinterpret_cast<Scene*>(h);
	if (!S || !world_3x4) return RRG_ERR_INVALID;
	RRG_CUDA(cudaSetDevice(S->c->device));
	RRG_CUDA(cudaDeviceSynchronize());   // traces in flight read the old records
	std::vector<float> old = S->world;
	S->world.assign(world_3x4, world_3x4 + 12 * (size_t)S->nobj);
	int st = rebuild(S);
	if (st) {
		S->world = old;
		rebuild(S);
	}
	return st;
}

int rrg_scene_set_enabled(rrg_scene* h, const uint8_t* enabled) {
	Scene* S = reinterpret_cast<Scene*>(h);
	if (!S || !enabled) return RRG_ERR_INVALID;
	RRG_CUDA(cudaSetDevice(S->c->device));
	RRG_CUDA(cudaDeviceSynchronize());
	S->enabled.assign(enabled, enabled + S->nobj);
	return rebuild(S);
}

int rrg_scene_intersect_device(rrg_scene* h, const float* rays_dev, uint32_t n, float* hits_dev,
                               uint32_t* objects_dev, void* stream) {
	Scene* S = reinterpret_cast<Scene*>(h);
	if (!S) return RRG_ERR_INVALID;
	if (n == 0) return RRG_OK;
	if (!rays_dev || !hits_dev || ((uintptr_t)rays_dev & 15) || ((uintptr_t)hits_dev & 15) || n >= 0x80000000u)
		return RRG_ERR_INVALID;
	RRG_CUDA(cudaSetDevice(S->c->device));
	cudaStream_t s = (cudaStream_t)stream;
	RRG_CUDA(cudaMemsetAsync(S->d_counter, 0, 4, s));
	const uint32_t want = (n + 31) / 32 * 32 / kTraceThreads + 1;
	const int grid = (int)(want < (uint32_t)S->blocks ? want : (uint32_t)S->blocks);
	const Collider* c = S->c;
	rrg::note_launch(), k_scene_closest<<<grid, kTraceThreads, 0, s>>>(S->d_tl, (int)S->ntl, S->d_tl_obj, (int)S->ntl_obj, S->d_obj,
	                                               (int)S->nobj, c->d_nodes, (int)c->nnodes, c->d_tris,
	                                               (int)c->nvalid, reinterpret_cast<const float4*>(rays_dev), n,
	                                               reinterpret_cast<float4*>(hits_dev), objects_dev, S->d_counter);
	RRG_CUDA(cudaGetLastError());
	return RRG_OK;
}

int rrg_scene_intersect_host(rrg_scene* h, const float* rays_host, uint32_t n, float* hits_host,
                             uint32_t* objects_host) {
	Scene* S = reinterpret_cast<Scene*>(h);
	if (!S || (n && (!rays_host || !hits_host)) || n >= 0x80000000u) return RRG_ERR_INVALID;
	if (!n) return RRG_OK;
	std::lock_guard<std::mutex> lk(S->host_mu);
	RRG_CUDA(cudaSetDevice(S->c->device));
	if (!S->s_host) RRG_CUDA(cudaStreamCreateWithFlags(&S->s_host, cudaStreamNonBlocking));
	const size_t per = 32 + 16 + 4;   // ray, hit record, object
	if (n > S->stage_cap) {
		uint32_t cap = S->stage_cap ? S->stage_cap : 256;
		while (cap < n) cap = cap > 0x40000000u ? n : cap * 2;
		cudaFree(S->d_stage);
		S->d_stage = nullptr;
		S->stage_cap = 0;
		RRG_CUDA(cudaMalloc(&S->d_stage, per * (size_t)cap));
		S->stage_cap = cap;
	}
	uint8_t* base = static_cast<uint8_t*>(S->d_stage);
	float* d_rays = reinterpret_cast<float*>(base);
	float* d_hits = reinterpret_cast<float*>(base + 32 * (size_t)S->stage_cap);
	uint32_t* d_obj = reinterpret_cast<uint32_t*>(base + 48 * (size_t)S->stage_cap);
	cudaStream_t s = S->s_host;
	RRG_CUDA(cudaMemcpyAsync(d_rays, rays_host, 32 * (size_t)n, cudaMemcpyHostToDevice, s));
	int st = rrg_scene_intersect_device(h, d_rays, n, d_hits, objects_host ? d_obj : nullptr, s);
	if (st) return st;
	RRG_CUDA(cudaMemcpyAsync(hits_host, d_hits, 16 * (size_t)n, cudaMemcpyDeviceToHost, s));
	if (objects_host) RRG_CUDA(cudaMemcpyAsync(objects_host, d_obj, 4 * (size_t)n, cudaMemcpyDeviceToHost, s));
	return rrg_scene_status(h, s);
}

int rrg_scene_status(rrg_scene* h, void* stream) {
	Scene* S = reinterpret_cast<Scene*>(h);
	if (!S) return RRG_ERR_INVALID;
	uint32_t w = 0;
	cudaStream_t s = (cudaStream_t)stream;
	RRG_CUDA(cudaMemcpyAsync(&w, S->d_counter + 1, 4, cudaMemcpyDeviceToHost, s));
	RRG_CUDA(cudaStreamSynchronize(s));
	RRG_CUDA(cudaMemsetAsync(S->d_counter + 1, 0, 4, s));
	return w ? RRG_ERR_STACK : RRG_OK;
}

}  // extern "C"
