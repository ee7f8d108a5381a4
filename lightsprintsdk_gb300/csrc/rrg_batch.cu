// C ABI of uneven mesh batches (include/rrgpu_batch.h): one multi-root BVH
// build over all meshes and one persistent closest-hit launch over all
// rays, replayed from a CUDA graph.
#include "rrg_internal.cuh"

#include "../../include/rrgpu_batch.h"

#include <new>
#include <vector>

namespace rrg {

struct Batch {
	Collider* c = nullptr;          // all meshes' geometry; c->nroots = meshes
	uint32_t nmesh = 0;
	int fetch = 1;                  // rays per warp / 32
	uint32_t sdepth = 0;            // mode word: stack entries in shared memory | kBatchRootQueue
	int blocks = 0;                 // persistent grid (occupancy x SMs) of the current kernel variant
	cudaStream_t cap = nullptr;     // private stream the graph is captured on
	cudaGraphExec_t exec = nullptr;
	uint32_t graph_kernels = 0;   // kernel nodes of exec
	// arguments the captured graph was made for
	const void* g_rays = nullptr;
	const void* g_off = nullptr;
	void* g_hits = nullptr;
	uint32_t g_n = 0;
	int g_fetch = 0;
	uint32_t g_sdepth = 0;
	// rebuild + trace in one graph (rrg_batch_rebuild_intersect_device)
	GraphBuild* gb = nullptr;
	cudaGraphExec_t exec_rb = nullptr;
	uint32_t rb_kernels = 0;
	const void* r_rays = nullptr;
	const void* r_off = nullptr;
	void* r_hits = nullptr;
	uint32_t r_n = 0;
	int r_fetch = 0;
	uint32_t r_sdepth = 0;
};

static void free_batch(Batch* b) {
	if (!b) return;
	if (b->exec) cudaGraphExecDestroy(b->exec);
	if (b->exec_rb) cudaGraphExecDestroy(b->exec_rb);
	graph_build_free(b->gb);
	if (b->cap) cudaStreamDestroy(b->cap);
	free_collider(b->c);
	delete b;
}

Collider* batch_collider(rrg_batch* h) {
	Batch* b = reinterpret_cast<Batch*>(h);
	return b ? b->c : nullptr;
}

static bool ascending(const uint32_t* off, uint32_t n) {
	if (off[0] != 0) return false;
	for (uint32_t m = 0; m < n; m++)
		if (off[m + 1] < off[m]) return false;
	return true;
}

// Captures on the batch's private stream either the trace alone or the
// rebuild of every mesh's tree followed by the trace (rebuild), and
// instantiates it; *kernels = the kernel nodes of the graph.
static int capture(Batch* b, bool rebuild, const float* rays_dev, const uint32_t* ray_off_dev, uint32_t n,
                   float* hits_dev, cudaGraphExec_t* exec, uint32_t* kernels) {
	cudaGraph_t g = nullptr;
	RRG_CUDA(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
	t_capturing = 1;   // recorded, not launched: counted per graph launch
	int st = RRG_OK;
	if (rebuild) {
		st = graph_build_enqueue(b->c, b->gb, b->cap);
		if (!st)
			st = launch_batch_closest_on(b->c, graph_build_nodes(b->gb), (int)graph_build_max_nodes(b->gb),
			                             graph_build_tris(b->gb), (int)b->c->nt,
			                             reinterpret_cast<const float4*>(rays_dev), n, ray_off_dev, b->nmesh, b->fetch,
			                             b->blocks, b->sdepth, reinterpret_cast<float4*>(hits_dev), b->cap);
	} else {
		st = launch_batch_closest(b->c, reinterpret_cast<const float4*>(rays_dev), n, ray_off_dev, b->nmesh, b->fetch,
		                          b->blocks, b->sdepth, reinterpret_cast<float4*>(hits_dev), b->cap);
	}
	t_capturing = 0;
	cudaError_t e = cudaStreamEndCapture(b->cap, &g);
	if (st) {
		if (g) cudaGraphDestroy(g);
		return st;
	}
	if (e != cudaSuccess) return cuda_fail(e);
	*kernels = 0;
	size_t nn = 0;
	if (cudaGraphGetNodes(g, nullptr, &nn) == cudaSuccess && nn) {
		std::vector<cudaGraphNode_t> nodes(nn);
		if (cudaGraphGetNodes(g, nodes.data(), &nn) == cudaSuccess)
			for (size_t i = 0; i < nn; i++) {
				cudaGraphNodeType t;
				if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) (*kernels)++;
			}
	}
	e = cudaGraphInstantiate(exec, g, 0);
	cudaGraphDestroy(g);
	if (e != cudaSuccess) {
		*exec = nullptr;
		return cuda_fail(e);
	}
	return RRG_OK;
}

}  // namespace rrg

using namespace rrg;

extern "C" {

int rrg_batch_create(const float* xyz, const uint32_t* vert_off, const uint32_t* idx, const uint32_t* tri_off,
                     uint32_t nmesh, const rrg_build_params* params, int device, rrg_batch** out) {
	if (!out) return RRG_ERR_INVALID;
	*out = nullptr;
	if (!vert_off || !tri_off || nmesh == 0 || nmesh > RRG_BATCH_MAX_MESHES) return RRG_ERR_INVALID;
	if (!ascending(vert_off, nmesh) || !ascending(tri_off, nmesh)) return RRG_ERR_INVALID;
	const uint32_t nv = vert_off[nmesh], nt = tri_off[nmesh];
	if (nt == 0) return RRG_ERR_EMPTY;
	if (!xyz || !idx || !nv) return RRG_ERR_INVALID;
	if ((uint64_t)nt * 3 > 0xFFFFFFFFull || (uint64_t)nv * 3 > 0xFFFFFFFFull || nt >= 0x80000000u)
		return RRG_ERR_INVALID;
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return RRG_ERR_NO_DEVICE;
	if (device < 0 || device >= ndev) return RRG_ERR_INVALID;
	RRG_CUDA(cudaSetDevice(device));
	Batch* b = new (std::nothrow) Batch();
	if (!b) return RRG_ERR_OOM;
	Collider* c = b->c = new (std::nothrow) Collider();
	if (!c) {
		delete b;
		return RRG_ERR_OOM;
	}
	int st = init_collider(c, params);
	uint32_t* d_vert_off = nullptr;
	cudaError_t e = cudaSuccess;
	if (!st) {
		c->nv = nv;
		c->nt = nt;
		c->nroots = nmesh;
		e = cudaMalloc((void**)&c->d_xyz, sizeof(float) * 3 * (size_t)nv);
		if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_idx, sizeof(uint32_t) * 3 * (size_t)nt);
		if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_tri_off, sizeof(uint32_t) * (nmesh + 1));
		if (e == cudaSuccess) e = cudaMalloc((void**)&d_vert_off, sizeof(uint32_t) * (nmesh + 1));
		if (e == cudaSuccess) e = cudaMemcpy(c->d_xyz, xyz, sizeof(float) * 3 * (size_t)nv, cudaMemcpyHostToDevice);
		if (e == cudaSuccess) e = cudaMemcpy(c->d_idx, idx, sizeof(uint32_t) * 3 * (size_t)nt, cudaMemcpyHostToDevice);
		if (e == cudaSuccess)
			e = cudaMemcpy(c->d_tri_off, tri_off, sizeof(uint32_t) * (nmesh + 1), cudaMemcpyHostToDevice);
		if (e == cudaSuccess)
			e = cudaMemcpy(d_vert_off, vert_off, sizeof(uint32_t) * (nmesh + 1), cudaMemcpyHostToDevice);
		if (e != cudaSuccess) st = cuda_fail(e);
	}
	if (!st) st = globalize_batch_indices(c, d_vert_off, nullptr);
	if (!st) st = build_bvh(c, nullptr, nullptr);
	cudaFree(d_vert_off);
	if (!st) st = batch_trace_blocks(c, nmesh, 0, &b->blocks);
	if (!st) {
		e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
		if (e != cudaSuccess) st = cuda_fail(e);
	}
	if (st) {
		free_batch(b);
		return st;
	}
	b->nmesh = nmesh;
	account_collider(c);
	*out = reinterpret_cast<rrg_batch*>(b);
	return RRG_OK;
}

void rrg_batch_destroy(rrg_batch* h) {
	Batch* b = reinterpret_cast<Batch*>(h);
	if (!b) return;
	cudaSetDevice(b->c->device);
	cudaDeviceSynchronize();
	free_batch(b);
}

int rrg_batch_set_rays_per_warp(rrg_batch* h, uint32_t rays_per_warp) {
	Batch* b = reinterpret_cast<Batch*>(h);
	if (!b) return RRG_ERR_INVALID;
	if (rays_per_warp != 32 && rays_per_warp != 64 && rays_per_warp != 128 && rays_per_warp != 256)
		return RRG_ERR_INVALID;
	b->fetch = (int)(rays_per_warp / 32);
	return RRG_OK;
}

int rrg_batch_set_stack_smem(rrg_batch* h, uint32_t entries) {
	Batch* b = reinterpret_cast<Batch*>(h);
	if (!b) return RRG_ERR_INVALID;
	if (entries != 0 && entries != 8 && entries != 16 && entries != 32) return RRG_ERR_INVALID;
	RRG_CUDA(cudaSetDevice(b->c->device));
	int blocks = 0;
	const uint32_t mode = entries | (b->sdepth & kBatchRootQueue);
	int st = batch_trace_blocks(b->c, b->nmesh, mode, &blocks);
	if (st) return st;
	b->sdepth = mode;
	b->blocks = blocks;
	return RRG_OK;
}

int rrg_batch_set_root_queue(rrg_batch* h, int on) {
	Batch* b = reinterpret_cast<Batch*>(h);
	if (!b) return RRG_ERR_INVALID;
	RRG_CUDA(cudaSetDevice(b->c->device));
	int blocks = 0;
	const uint32_t mode = (b->sdepth & ~kBatchRootQueue) | (on ? kBatchRootQueue : 0u);
	int st = batch_trace_blocks(b->c, b->nmesh, mode, &blocks);
	if (st) return st;
	b->sdepth = mode;
	b->blocks = blocks;
	return RRG_OK;
}

int rrg_batch_intersect_device(rrg_batch* h, const float* rays_dev, const uint32_t* ray_off_dev, uint32_t n,
                               float* hits_dev, void* stream) {
	Batch* b = reinterpret_cast<Batch*>(h);
	if (!b) return RRG_ERR_INVALID;
	if (n == 0) return RRG_OK;
	if (!rays_dev || !ray_off_dev || !hits_dev || ((uintptr_t)rays_dev & 15) || ((uintptr_t)hits_dev & 15) ||
	    ((uintptr_t)ray_off_dev & 3) || n >= 0x80000000u)
		return RRG_ERR_INVALID;
	RRG_CUDA(cudaSetDevice(b->c->device));
	if (!b->exec || b->g_rays != rays_dev || b->g_off != ray_off_dev || b->g_hits != hits_dev || b->g_n != n ||
	    b->g_fetch != b->fetch || b->g_sdepth != b->sdepth) {
		if (b->exec) {
			// the previous graph may still be running on the caller's stream
			RRG_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
			cudaGraphExecDestroy(b->exec);
			b->exec = nullptr;
		}
		int st = capture(b, false, rays_dev, ray_off_dev, n, hits_dev, &b->exec, &b->graph_kernels);
		if (st) return st;
		b->g_rays = rays_dev;
		b->g_off = ray_off_dev;
		b->g_hits = hits_dev;
		b->g_n = n;
		b->g_fetch = b->fetch;
		b->g_sdepth = b->sdepth;
	}
	RRG_CUDA(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
	note_launches(b->graph_kernels);
	return RRG_OK;
}

int rrg_batch_set_vertices_device(rrg_batch* h, const float* xyz_dev, void* stream) {
	Batch* b = reinterpret_cast<Batch*>(h);
	if (!b || !xyz_dev) return RRG_ERR_INVALID;
	RRG_CUDA(cudaSetDevice(b->c->device));
	RRG_CUDA(cudaMemcpyAsync(b->c->d_xyz, xyz_dev, sizeof(float) * 3 * (size_t)b->c->nv, cudaMemcpyDeviceToDevice,
	                         (cudaStream_t)stream));
	return RRG_OK;
}

int rrg_batch_rebuild_intersect_device(rrg_batch* h, const float* rays_dev, const uint32_t* ray_off_dev, uint32_t n,
                                       float* hits_dev, void* stream) {
	Batch* b = reinterpret_cast<Batch*>(h);
	if (!b) return RRG_ERR_INVALID;
	if (!rays_dev || !ray_off_dev || !hits_dev || ((uintptr_t)rays_dev & 15) || ((uintptr_t)hits_dev & 15) ||
	    ((uintptr_t)ray_off_dev & 3) || n == 0 || n >= 0x80000000u)
		return RRG_ERR_INVALID;
	if (b->c->width == 8) return RRG_ERR_INVALID;
	RRG_CUDA(cudaSetDevice(b->c->device));
	if (!b->gb) {
		int st = graph_build_new(b->c, &b->gb);
		if (st) return st;
	}
	if (!b->exec_rb || b->r_rays != rays_dev || b->r_off != ray_off_dev || b->r_hits != hits_dev || b->r_n != n ||
	    b->r_fetch != b->fetch || b->r_sdepth != b->sdepth) {
		if (b->exec_rb) {
			RRG_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
			cudaGraphExecDestroy(b->exec_rb);
			b->exec_rb = nullptr;
		}
		int st = capture(b, true, rays_dev, ray_off_dev, n, hits_dev, &b->exec_rb, &b->rb_kernels);
		if (st) return st;
		b->r_rays = rays_dev;
		b->r_off = ray_off_dev;
		b->r_hits = hits_dev;
		b->r_n = n;
		b->r_fetch = b->fetch;
		b->r_sdepth = b->sdepth;
	}
	RRG_CUDA(cudaGraphLaunch(b->exec_rb, (cudaStream_t)stream));
	note_launches(b->rb_kernels);
	return RRG_OK;
}

int rrg_batch_status(rrg_batch* h, void* stream) {
	Batch* b = reinterpret_cast<Batch*>(h);
	if (!b) return RRG_ERR_INVALID;
	uint32_t w = 0;
	cudaStream_t s = (cudaStream_t)stream;
	RRG_CUDA(cudaMemcpyAsync(&w, b->c->d_counter + 1, 4, cudaMemcpyDeviceToHost, s));
	RRG_CUDA(cudaStreamSynchronize(s));
	RRG_CUDA(cudaMemsetAsync(b->c->d_counter + 1, 0, 4, s));
	if (b->gb && b->exec_rb) {
		const int gs = graph_build_status(b->gb, s);
		if (gs) return gs;
	}
	return w ? RRG_ERR_STACK : RRG_OK;
}

uint32_t rrg_batch_meshes(const rrg_batch* h) {
	const Batch* b = reinterpret_cast<const Batch*>(h);
	return b ? b->nmesh : 0;
}
uint32_t rrg_batch_nodes(const rrg_batch* h) {
	const Batch* b = reinterpret_cast<const Batch*>(h);
	return b ? b->c->nnodes : 0;
}
size_t rrg_batch_memory(const rrg_batch* h) {
	const Batch* b = reinterpret_cast<const Batch*>(h);
	return b ? b->c->bytes + sizeof(uint32_t) * (b->nmesh + 1) : 0;
}
float rrg_batch_build_ms(const rrg_batch* h) {
	const Batch* b = reinterpret_cast<const Batch*>(h);
	return b ? b->c->build_ms : 0.f;
}

}  // extern "C"
