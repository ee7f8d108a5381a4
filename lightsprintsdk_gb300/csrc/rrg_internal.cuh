// Internal declarations shared by the collider's translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include <atomic>
#include <mutex>

#include "../../include/rrgpu.h"

typedef struct rrg_batch rrg_batch;
typedef struct rrg_lightmapper rrg_lightmapper;

namespace rrg {

// ---------------------------------------------------------------- layout
// Build node (one per BVH node, root = 0).  Leaves: left < 0, prims
// [begin, begin+count) of the leaf-ordered triangle array.
struct BNode {
	float lo[3];
	float hi[3];
	int left, right;
	int begin, count;
};

// Binary traversal node: both children's boxes in the parent (64 bytes):
//   a = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   b = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   c = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   d = (ref0, ref1, 0, 0)
// ref >= 0: inner node index; ref with bit 31 set: leaf, bits 27..30 =
// count-1, bits 0..26 = first slot; kEmptyRef: no child.
struct TNode {
	float4 a, b, c;
	int4 d;
};

constexpr int kLeafBit = (int)0x80000000u;
constexpr int kEmptyRef = (int)0xFFFFFFFFu;   // leaf bit set, count 16: never produced
constexpr int kMaxLeaf = 8;
constexpr int kStackSize = 64;

// Compressed 8-wide node (80 bytes = 5 x uint4), built from the binary tree
// (rrg_wide.cu) for the closest/any-hit kernels:
//   w[0] = (p.x, p.y, p.z as float bits, e.x | e.y << 8 | e.z << 16 | valid << 24)
//   w[1] = (child_base, tri_base, meta[0..3], meta[4..7])
//   w[2] = (qlo.x[0..7], qlo.y[0..7]) bytes, w[3] = (qlo.z, qhi.x), w[4] = (qhi.y, qhi.z)
// Child slot s spans p + q[s] * 2^(e-127) on each axis (q in 0..255,
// rounded outward, so the box contains the child's widened box).  meta[s]:
// internal child 0x80 | k -> node child_base + k; leaf (count-1) << 5 |
// offset -> triangles tri_base + offset .. + count-1 (count <= 4).  The
// slots of a node are assigned so that visiting slot i ^ octant(ray) for
// i = 0..7 goes roughly near to far.
constexpr int kWideLeafMax = 4;
constexpr uint32_t kWideMaxNodes = 1u << 24;   // stack entries pack a node index in 24 bits

__host__ __device__ inline int leaf_ref(int first, int count) {
	return kLeafBit | ((count - 1) << 27) | first;
}

// Index m of the segment holding item i, for ascending offsets off[0..n]
// with off[0] = 0 and i < off[n]: the largest m < n with off[m] <= i (empty
// segments, whose offsets repeat, are skipped).
__device__ __forceinline__ uint32_t segment_of(const uint32_t* off, uint32_t n, uint32_t i) {
	uint32_t lo = 0, hi = n;
	while (hi - lo > 1) {
		uint32_t mid = (lo + hi) >> 1;
		if (off[mid] <= i) lo = mid;
		else hi = mid;
	}
	return lo;
}

// Triangles in leaf order: 3 x float4 = (v0.xyz, original index bits),
// (v1.xyz, 0), (v2.xyz, 0); vertices in the mesh's own order.

// -------------------------------------------------------------- collider
struct Combiner;

struct Collider {
	int device = 0;
	uint32_t nv = 0, nt = 0, nvalid = 0, nnodes = 0;
	float* d_xyz = nullptr;       // 3*nv
	uint32_t* d_idx = nullptr;    // 3*nt
	TNode* d_nodes = nullptr;
	float4* d_tris = nullptr;     // 3*nvalid
	uint32_t* d_counter = nullptr;// scratch (16 words): [0] ray counter, [1] status word; pipelined
	                              // host calls use [4k], [4k+1] for staging slot k
	size_t bytes = 0;
	float build_ms = 0;
	float aabb_lo[3] = {0, 0, 0}, aabb_hi[3] = {0, 0, 0};   // all vertices
	rrg_build_params params{};
	// host-call staging (rrg_intersect_host / rrg_intersect_rrray)
	void* d_stage_in = nullptr;
	void* d_stage_out = nullptr;
	size_t stage_in_bytes = 0, stage_out_bytes = 0;
	int num_sms = 0;
	int trace_blocks = 0;
	int occl_blocks = 0;
	int ww_blocks = 0;
	int wide_blocks = 0;
	uint32_t traversal = RRG_TRAVERSAL_ROOT_QUEUE;
	// RRG_TRAVERSAL_COMPACT tuning (rrg_collider_set_compact_tuning) and its
	// persistent grid per kernel variant (filled on first use)
	uint32_t compact_sdepth = 8, compact_fetch = 1, compact_minb = 9;
	int compact_blocks[32] = {};
	// batches of meshes (rrg_batch): one BVH root per mesh, nodes 0..nroots-1;
	// d_tri_off = nroots+1 offsets of each mesh's triangles in d_idx
	uint32_t nroots = 1;
	uint32_t* d_tri_off = nullptr;
	// 8-wide form (bvh_width 8): nodes 0..nroots-1 are roots; triangles in
	// wide-leaf order, same 3 x float4 layout as d_tris
	uint32_t width = 2;
	// pipelined host calls: copy-in and copy-out streams, one event set per
	// staging slot (created on first use)
	cudaStream_t s_in = nullptr, s_out = nullptr, s_comp = nullptr;
	cudaEvent_t ev_in[3] = {nullptr, nullptr, nullptr};
	cudaEvent_t ev_done[3] = {nullptr, nullptr, nullptr};
	cudaEvent_t ev_out[3] = {nullptr, nullptr, nullptr};
	cudaEvent_t ev_start = nullptr;
	// ray binning scratch, one per concurrently running caller: slots 0..2 for
	// the pipelined host path's staging slots, 3 for direct launches
	uint32_t ray_order = RRG_RAY_ORDER_DEFAULT;
	void* d_bin[4] = {nullptr, nullptr, nullptr, nullptr};
	size_t bin_bytes[4] = {0, 0, 0, 0};
	bool bin_attr = false;
	uint4* d_wnodes = nullptr;    // 5 per node
	float4* d_wtris = nullptr;    // 3*nvalid
	uint32_t nwnodes = 0;
	// host threads calling the staging entry points (rrg_intersect_host,
	// rrg_intersect_rrray) take turns on this lock
	std::mutex host_mu;
	// single-ray queries combined across host threads (rrg_combine.cu)
	Combiner* comb = nullptr;
	// optional CUDA-event pairs around each closest-hit traversal launch
	// (rrg_collider_trace_timing); tev_n pairs recorded since the reset
	bool timing = false;
	cudaEvent_t tev[2 * 256] = {};
	uint32_t tev_n = 0;
};
// records the start (end = false) or end of a timed traversal launch
int trace_event(Collider* c, cudaStream_t s, bool end);

// build (rrg_build.cu)
int build_bvh(Collider* c, cudaStream_t s, const volatile int* aborting);
int globalize_batch_indices(Collider* c, const uint32_t* d_vert_off, cudaStream_t s);
// wide (rrg_wide.cu): collapses the binary build nodes into d_wnodes/d_wtris
int build_wide(Collider* c, const BNode* bnodes, int nnodes, const float* pad, cudaStream_t s);

// trace (rrg_trace.cu)
int launch_closest(Collider* c, const float4* rays, uint32_t n, float4* hits, float4* planes, float* points,
                   cudaStream_t s);
int launch_closest_on(Collider* c, const float4* rays, uint32_t n, float4* hits, float4* planes, float* points,
                      uint32_t* words, cudaStream_t s, int bin_slot);
// binning (rrg_binning.cu): permutation of the n rays into binned order in
// scratch slot bin_slot (0..3) of the collider
int bin_rays(Collider* c, const float4* rays, uint32_t n, cudaStream_t s, int bin_slot, const uint32_t** perm_out);
// the wavefront gather's live paths sorted by their rays' key (device count)
size_t bin_paths_bytes(const Collider* c, uint32_t cap);
int bin_paths(Collider* c, const float4* eye, const float4* dir, const uint32_t* list, const uint32_t* n_dev,
              uint32_t cap, void* scratch, uint32_t* out, cudaStream_t s);
int launch_occluded(Collider* c, const float4* rays, uint32_t n, uint8_t* occ, cudaStream_t s);
int launch_rrray(Collider* c, void* rrrays_dev, uint32_t n, uint8_t* hit_dev, cudaStream_t s);
int launch_rrray_scratch(Collider* c, void* rrrays_dev, uint32_t n, uint8_t* hit_dev, uint32_t* words,
                         cudaStream_t s, int keyed = 0);
int trace_occupancy(Collider* c);
// compacting traversal (rrg_compact.cu): closest hit (occ null) or any hit;
// perm = binned order or null; words[0] work counter (cleared here), [1] status
int launch_compact(Collider* c, const float4* rays, uint32_t n, float4* hits, float4* planes, float* points,
                   uint8_t* occ, uint32_t* words, const uint32_t* perm, cudaStream_t s);
bool compact_depth_ok(uint32_t sdepth);
// batches (nmesh roots): ray i belongs to mesh segment_of(ray_off, nmesh, i)
constexpr uint32_t kBatchMaxMeshes = 8192;
// the collider holding a batch's meshes (rrg_batch.cu)
Collider* batch_collider(::rrg_batch* b);
// the batch build as a graph-capturable launch sequence (rrg_build.cu)
struct GraphBuild;
int graph_build_new(Collider* c, GraphBuild** out);
void graph_build_free(GraphBuild* g);
int graph_build_enqueue(Collider* c, GraphBuild* g, cudaStream_t s);
int graph_build_status(GraphBuild* g, cudaStream_t s);
const TNode* graph_build_nodes(const GraphBuild* g);
const float4* graph_build_tris(const GraphBuild* g);
uint32_t graph_build_max_nodes(const GraphBuild* g);
// a batch trace's mode word: shared-memory stack entries (0, 8, 16, 32),
// or-ed with kBatchRootQueue for the root-box queue
constexpr uint32_t kBatchRootQueue = 0x10000u;
int batch_trace_blocks(Collider* c, uint32_t nmesh, uint32_t sdepth, int* blocks);
// closest hit with rays and hits in page-locked host memory (rrg_intersect_host)
int launch_closest_mapped(Collider* c, const float4* rays, uint32_t n, float4* hits, cudaStream_t s);
// launch_batch_closest on explicit binary-tree buffers (a graph build's)
int launch_batch_closest_on(Collider* c, const TNode* nodes, int nnodes, const float4* tris, int ntris,
                            const float4* rays, uint32_t n, const uint32_t* ray_off, uint32_t nmesh, int fetch,
                            int blocks, uint32_t sdepth, float4* hits, cudaStream_t s);
int launch_batch_closest(Collider* c, const float4* rays, uint32_t n, const uint32_t* ray_off, uint32_t nmesh,
                         int fetch, int blocks, uint32_t sdepth, float4* hits, cudaStream_t s);

// combined single-ray queries (rrg_combine.cu)
Combiner* combiner_new();
void combiner_free(Combiner* k);

// lightmaps (rrg_gather.cu, rrg_filter.cu)
struct LightmapFilter;
void filter_free(LightmapFilter* f);
struct LightmapView {
	Collider* c;
	uint32_t natlas, size, nt;
	const float* uv;          // host, 6 per triangle
	const int32_t* atlas;     // host, per triangle
	LightmapFilter** filter;  // the lightmapper's filter state
};
LightmapView lightmapper_view(::rrg_lightmapper* lm);

// api (rrg_api.cu)
// Kernels this library has launched in the process (rrg_launch_count):
// every launch site bumps it through note_launch(); launches recorded into a
// CUDA graph are counted when the graph is launched, not while it is captured.
extern std::atomic<uint64_t> g_launches;
extern thread_local int t_capturing;
inline void note_launch() {
	if (!t_capturing) g_launches.fetch_add(1, std::memory_order_relaxed);
}
inline void note_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
int cuda_fail(cudaError_t e);
int init_collider(Collider* c, const rrg_build_params* params);
void free_collider(Collider* c);
void account_collider(Collider* c);

}  // namespace rrg

#define RRG_CUDA(x)                                  \
	do {                                             \
		cudaError_t e_ = (x);                        \
		if (e_ != cudaSuccess) return rrg::cuda_fail(e_); \
	} while (0)
