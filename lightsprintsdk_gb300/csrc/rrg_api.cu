// C ABI of the collider (include/rrgpu.h): argument checks, device memory,
// streams and status codes.  The reference equivalents are
// RRCollider::create / defaultBuilder (RRCollider/RRCollider.cpp:87-241) and
// the IntersectBspFast members (RRCollider/IntersectBspFast.h:55-74).
#include "rrg_internal.cuh"

#include <stdio.h>
#include <string.h>
#include <new>
#include <algorithm>
#include <vector>

namespace rrg {

static thread_local char g_cuda_err[256] = "";

int cuda_fail(cudaError_t e) {
	snprintf(g_cuda_err, sizeof(g_cuda_err), "%s: %s", cudaGetErrorName(e), cudaGetErrorString(e));
	if (e == cudaErrorMemoryAllocation) return RRG_ERR_OOM;
	if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver || e == cudaErrorNoKernelImageForDevice)
		return RRG_ERR_NO_DEVICE;
	return RRG_ERR_CUDA;
}

void free_collider(Collider* c) {
	if (!c) return;
	cudaFree(c->d_tri_off);
	cudaFree(c->d_wnodes);
	cudaFree(c->d_wtris);
	for (int k = 0; k < 3; k++) {
		if (c->ev_in[k]) cudaEventDestroy(c->ev_in[k]);
		if (c->ev_done[k]) cudaEventDestroy(c->ev_done[k]);
		if (c->ev_out[k]) cudaEventDestroy(c->ev_out[k]);
	}
	if (c->ev_start) cudaEventDestroy(c->ev_start);
	for (cudaEvent_t e : c->tev)
		if (e) cudaEventDestroy(e);
	if (c->s_in) cudaStreamDestroy(c->s_in);
	if (c->s_out) cudaStreamDestroy(c->s_out);
	if (c->s_comp) cudaStreamDestroy(c->s_comp);
	cudaFree(c->d_xyz);
	cudaFree(c->d_idx);
	cudaFree(c->d_nodes);
	cudaFree(c->d_tris);
	cudaFree(c->d_counter);
	cudaFree(c->d_stage_in);
	cudaFree(c->d_stage_out);
	for (int k = 0; k < 4; k++) cudaFree(c->d_bin[k]);
	combiner_free(c->comb);
	delete c;
}

int init_collider(Collider* c, const rrg_build_params* params) {
	memset(&c->params, 0, sizeof(c->params));
	if (params) {
		if (params->size < sizeof(uint32_t) || params->size > sizeof(rrg_build_params)) return RRG_ERR_INVALID;
		memcpy(&c->params, params, params->size);
	}
	c->params.size = sizeof(rrg_build_params);
	if (c->params.max_leaf_size > (uint32_t)kMaxLeaf) return RRG_ERR_INVALID;
	if (c->params.traversal > RRG_TRAVERSAL_ROOT_QUEUE) return RRG_ERR_INVALID;
	if (c->params.bvh_width != 0 && c->params.bvh_width != 2 && c->params.bvh_width != 8) return RRG_ERR_INVALID;
	c->width = c->params.bvh_width ? c->params.bvh_width : 2;
	if (c->width == 8 && c->params.max_leaf_size > (uint32_t)kWideLeafMax) return RRG_ERR_INVALID;
	c->traversal = c->params.traversal ? c->params.traversal : RRG_TRAVERSAL_ROOT_QUEUE;
	RRG_CUDA(cudaGetDevice(&c->device));
	cudaDeviceProp prop;
	RRG_CUDA(cudaGetDeviceProperties(&prop, c->device));
	c->num_sms = prop.multiProcessorCount;
	RRG_CUDA(cudaMalloc((void**)&c->d_counter, 64));
	RRG_CUDA(cudaMemset(c->d_counter, 0, 64));
	c->comb = combiner_new();
	if (!c->comb) return RRG_ERR_OOM;
	return trace_occupancy(c);
}

void account_collider(Collider* c) {
	c->bytes = sizeof(float) * 3 * (size_t)c->nv + sizeof(uint32_t) * 3 * (size_t)c->nt + sizeof(TNode) * (size_t)c->nnodes +
	           sizeof(float4) * 3 * (size_t)c->nvalid + 64 + c->stage_in_bytes + c->stage_out_bytes +
	           (c->d_wnodes ? sizeof(uint4) * 5 * (size_t)c->nwnodes + sizeof(float4) * 3 * (size_t)c->nvalid : 0) +
	           c->bin_bytes[0] + c->bin_bytes[1] + c->bin_bytes[2] + c->bin_bytes[3];
}

static int ensure_stage(Collider* c, size_t in_bytes, size_t out_bytes) {
	if (in_bytes > c->stage_in_bytes) {
		cudaFree(c->d_stage_in);
		c->d_stage_in = nullptr;
		c->stage_in_bytes = 0;
		RRG_CUDA(cudaMalloc(&c->d_stage_in, in_bytes));
		c->stage_in_bytes = in_bytes;
	}
	if (out_bytes > c->stage_out_bytes) {
		cudaFree(c->d_stage_out);
		c->d_stage_out = nullptr;
		c->stage_out_bytes = 0;
		RRG_CUDA(cudaMalloc(&c->d_stage_out, out_bytes));
		c->stage_out_bytes = out_bytes;
	}
	account_collider(c);
	return RRG_OK;
}

static int ensure_pipeline(Collider* c) {
	if (c->s_in) return RRG_OK;
	RRG_CUDA(cudaStreamCreateWithFlags(&c->s_out, cudaStreamNonBlocking));
	RRG_CUDA(cudaStreamCreateWithFlags(&c->s_comp, cudaStreamNonBlocking));
	for (int k = 0; k < 3; k++) {
		RRG_CUDA(cudaEventCreateWithFlags(&c->ev_in[k], cudaEventDisableTiming));
		RRG_CUDA(cudaEventCreateWithFlags(&c->ev_done[k], cudaEventDisableTiming));
		RRG_CUDA(cudaEventCreateWithFlags(&c->ev_out[k], cudaEventDisableTiming));
	}
	RRG_CUDA(cudaEventCreateWithFlags(&c->ev_start, cudaEventDisableTiming));
	RRG_CUDA(cudaStreamCreateWithFlags(&c->s_in, cudaStreamNonBlocking));   // last: marks the set complete
	return RRG_OK;
}

// Pipelined host calls (rrg_intersect_host).  Calls of up to kHostSingle
// rays go up, through and back in one piece; page-locked calls of up to
// kHostChunk rays are traced in place in host memory; the others are cut
// into chunks (chunk_schedule) whose copies overlap the tracing.
constexpr uint32_t kHostChunk = 1u << 22;
constexpr uint32_t kHostSingle = 1u << 18;

// Chunk sizes of a pipelined call: kHostChunk rays each (128 MiB of rays in,
// 64 MiB of hits out, binned), or four equal chunks below that.  (On config
// 1 on GB300 both a ramp of 1, 2, 4, 8 ... 8, 4, 2, 1 Mi rays, which
// shortens the unhidden first copy-in and last copy-out, and 4, 8, 8, 8, 4
// Mi rays, which bins larger chunks, measured slower end to end: 3.31 and
// 3.35 against 3.43 Grays/s.)
static void chunk_schedule(uint32_t n, std::vector<uint32_t>& sizes) {
	const uint32_t chunk = n > kHostChunk ? kHostChunk : ((n + 3) / 4 + 255) / 256 * 256;
	sizes.clear();
	for (uint32_t done = 0; done < n; done += chunk) sizes.push_back(n - done < chunk ? n - done : chunk);
}

std::atomic<uint64_t> g_launches{0};
thread_local int t_capturing = 0;

}  // namespace rrg

using namespace rrg;

extern "C" {

uint32_t rrg_version(void) { return (1u << 16) | 0u; }

uint64_t rrg_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

const char* rrg_last_cuda_error(void) { return g_cuda_err; }

const char* rrg_status_string(int s) {
	switch (s) {
		case RRG_OK: return "ok";
		case RRG_ERR_INVALID: return "invalid argument";
		case RRG_ERR_OOM: return "out of memory";
		case RRG_ERR_CUDA: return "CUDA error";
		case RRG_ERR_STACK: return "traversal stack overflow";
		case RRG_ERR_ABORTED: return "aborted";
		case RRG_ERR_NO_DEVICE: return "no usable CUDA device";
		case RRG_ERR_EMPTY: return "mesh has no valid triangle";
		case RRG_ERR_TIMEOUT: return "device wait timed out";
		case RRG_ERR_TOO_LARGE: return "batch larger than RRG_NOALLOC_MAX_RAYS (static scratch limit)";
		default: return "unknown status";
	}
}

int rrg_collider_create_device(const float* xyz_dev, uint32_t nv, const uint32_t* idx_dev, uint32_t nt,
                               const rrg_build_params* params, const volatile int* aborting, void* stream,
                               rrg_collider** out) {
	if (!out) return RRG_ERR_INVALID;
	*out = nullptr;
	if (!xyz_dev || !idx_dev || !nv || !nt) return (nt == 0 && out) ? RRG_ERR_EMPTY : RRG_ERR_INVALID;
	if ((uint64_t)nt * 3 > 0xFFFFFFFFull || (uint64_t)nv * 3 > 0xFFFFFFFFull) return RRG_ERR_INVALID;
	Collider* c = new (std::nothrow) Collider();
	if (!c) return RRG_ERR_OOM;
	int st = init_collider(c, params);
	if (st) { free_collider(c); return st; }
	cudaStream_t s = (cudaStream_t)stream;
	c->nv = nv;
	c->nt = nt;
	cudaError_t e = cudaMalloc((void**)&c->d_xyz, sizeof(float) * 3 * (size_t)nv);
	if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_idx, sizeof(uint32_t) * 3 * (size_t)nt);
	if (e == cudaSuccess) e = cudaMemcpyAsync(c->d_xyz, xyz_dev, sizeof(float) * 3 * (size_t)nv, cudaMemcpyDeviceToDevice, s);
	if (e == cudaSuccess) e = cudaMemcpyAsync(c->d_idx, idx_dev, sizeof(uint32_t) * 3 * (size_t)nt, cudaMemcpyDeviceToDevice, s);
	if (e != cudaSuccess) { free_collider(c); return cuda_fail(e); }
	st = build_bvh(c, s, aborting);
	if (st) { free_collider(c); return st; }
	account_collider(c);
	*out = reinterpret_cast<rrg_collider*>(c);
	return RRG_OK;
}

int rrg_collider_create(const float* xyz, uint32_t nv, const uint32_t* idx, uint32_t nt,
                        const rrg_build_params* params, const volatile int* aborting, int device,
                        rrg_collider** out) {
	if (!out) return RRG_ERR_INVALID;
	*out = nullptr;
	if (nt == 0) return RRG_ERR_EMPTY;
	if (!xyz || !idx || !nv) return RRG_ERR_INVALID;
	if ((uint64_t)nt * 3 > 0xFFFFFFFFull || (uint64_t)nv * 3 > 0xFFFFFFFFull) return RRG_ERR_INVALID;
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return RRG_ERR_NO_DEVICE;
	if (device < 0 || device >= ndev) return RRG_ERR_INVALID;
	RRG_CUDA(cudaSetDevice(device));
	float* dx = nullptr;
	uint32_t* di = nullptr;
	cudaError_t e = cudaMalloc((void**)&dx, sizeof(float) * 3 * (size_t)nv);
	if (e == cudaSuccess) e = cudaMalloc((void**)&di, sizeof(uint32_t) * 3 * (size_t)nt);
	if (e == cudaSuccess) e = cudaMemcpy(dx, xyz, sizeof(float) * 3 * (size_t)nv, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(di, idx, sizeof(uint32_t) * 3 * (size_t)nt, cudaMemcpyHostToDevice);
	if (e != cudaSuccess) {
		cudaFree(dx);
		cudaFree(di);
		return cuda_fail(e);
	}
	int st = rrg_collider_create_device(dx, nv, di, nt, params, aborting, nullptr, out);
	cudaDeviceSynchronize();
	cudaFree(dx);
	cudaFree(di);
	return st;
}

int rrg_collider_update(rrg_collider* h, const float* xyz_host) {
	Collider* c = reinterpret_cast<Collider*>(h);
	if (!c || !xyz_host) return RRG_ERR_INVALID;
	RRG_CUDA(cudaSetDevice(c->device));
	RRG_CUDA(cudaMemcpy(c->d_xyz, xyz_host, sizeof(float) * 3 * (size_t)c->nv, cudaMemcpyHostToDevice));
	int st = build_bvh(c, nullptr, nullptr);
	account_collider(c);
	return st;
}

void rrg_collider_destroy(rrg_collider* h) {
	Collider* c = reinterpret_cast<Collider*>(h);
	if (!c) return;
	cudaSetDevice(c->device);
	cudaDeviceSynchronize();
	free_collider(c);
}

int rrg_collider_set_ray_order(rrg_collider* h, uint32_t order) {
	Collider* c = reinterpret_cast<Collider*>(h);
	if (!c || order > RRG_RAY_ORDER_BINNED) return RRG_ERR_INVALID;
	c->ray_order = order;
	return RRG_OK;
}

int rrg_collider_set_traversal(rrg_collider* h, uint32_t traversal) {
	Collider* c = reinterpret_cast<Collider*>(h);
	if (!c || traversal > RRG_TRAVERSAL_ROOT_QUEUE) return RRG_ERR_INVALID;
	c->traversal = traversal ? traversal : RRG_TRAVERSAL_ROOT_QUEUE;
	return RRG_OK;
}

int rrg_collider_set_compact_tuning(rrg_collider* h, uint32_t stack_smem, uint32_t rays_per_warp,
                                    uint32_t blocks_per_sm) {
	Collider* c = reinterpret_cast<Collider*>(h);
	if (!c) return RRG_ERR_INVALID;
	const uint32_t depth = stack_smem == RRG_COMPACT_DEFAULT ? 8u : stack_smem;
	const uint32_t rays = rays_per_warp ? rays_per_warp : 32u;
	const uint32_t minb = blocks_per_sm == RRG_COMPACT_DEFAULT ? 9u : blocks_per_sm;
	if (!compact_depth_ok(depth) || rays % 32 || rays < 32 || rays > 1024 || (minb && minb != 9))
		return RRG_ERR_INVALID;
	c->compact_sdepth = depth;
	c->compact_fetch = rays / 32;
	c->compact_minb = minb;
	return RRG_OK;
}

int rrg_collider_trace_timing(rrg_collider* h, int enable, float* total_ms, uint32_t* launches) {
	Collider* c = reinterpret_cast<Collider*>(h);
	if (!c) return RRG_ERR_INVALID;
	float sum = 0.f;
	for (uint32_t i = 0; i < c->tev_n; i++) {
		RRG_CUDA(cudaEventSynchronize(c->tev[2 * i + 1]));
		float ms = 0.f;
		RRG_CUDA(cudaEventElapsedTime(&ms, c->tev[2 * i], c->tev[2 * i + 1]));
		sum += ms;
	}
	if (total_ms) *total_ms = sum;
	if (launches) *launches = c->tev_n;
	c->tev_n = 0;
	c->timing = enable != 0;
	return RRG_OK;
}

size_t rrg_collider_memory(const rrg_collider* h) {
	const Collider* c = reinterpret_cast<const Collider*>(h);
	return c ? c->bytes : 0;
}
uint32_t rrg_collider_triangles(const rrg_collider* h) {
	const Collider* c = reinterpret_cast<const Collider*>(h);
	return c ? c->nt : 0;
}
uint32_t rrg_collider_valid_triangles(const rrg_collider* h) {
	const Collider* c = reinterpret_cast<const Collider*>(h);
	return c ? c->nvalid : 0;
}
uint32_t rrg_collider_nodes(const rrg_collider* h) {
	const Collider* c = reinterpret_cast<const Collider*>(h);
	return c ? c->nnodes : 0;
}
float rrg_collider_build_ms(const rrg_collider* h) {
	const Collider* c = reinterpret_cast<const Collider*>(h);
	return c ? c->build_ms : 0.f;
}

static bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

int rrg_intersect_device(rrg_collider* h, const float* rays_dev, uint32_t n, float* hits_dev, float* planes_dev,
                         float* points_dev, void* stream) {
	Collider* c = reinterpret_cast<Collider*>(h);
	if (!c) return RRG_ERR_INVALID;
	if (n == 0) return RRG_OK;
	if (!rays_dev || !hits_dev || !aligned16(rays_dev) || !aligned16(hits_dev)) return RRG_ERR_INVALID;
	if (planes_dev && !aligned16(planes_dev)) return RRG_ERR_INVALID;
	return launch_closest(c, reinterpret_cast<const float4*>(rays_dev), n, reinterpret_cast<float4*>(hits_dev),
	                      reinterpret_cast<float4*>(planes_dev), points_dev, (cudaStream_t)stream);
}

int rrg_occluded_device(rrg_collider* h, const float* rays_dev, uint32_t n, uint8_t* occ_dev, void* stream) {
	Collider* c = reinterpret_cast<Collider*>(h);
	if (!c) return RRG_ERR_INVALID;
	if (n == 0) return RRG_OK;
	if (!rays_dev || !occ_dev || !aligned16(rays_dev)) return RRG_ERR_INVALID;
	return launch_occluded(c, reinterpret_cast<const float4*>(rays_dev), n, occ_dev, (cudaStream_t)stream);
}

// The device address of page-locked (registered or cudaHostAlloc'ed) host
// memory, which kernels can read and write in place over the host link; null
// for pageable memory or on any error (the caller then copies).
static const void* mapped_host(const void* p) {
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
		cudaGetLastError();
		return nullptr;
	}
	if (a.type != cudaMemoryTypeHost || !a.devicePointer || ((uintptr_t)a.devicePointer & 15)) return nullptr;
	return a.devicePointer;
}

int rrg_intersect_host(rrg_collider* h, const float* rays_host, uint32_t n, float* hits_host, void* stream) {
	Collider* c = reinterpret_cast<Collider*>(h);
	if (!c) return RRG_ERR_INVALID;
	if (n == 0) return RRG_OK;
	if (!rays_host || !hits_host) return RRG_ERR_INVALID;
	std::lock_guard<std::mutex> lk(c->host_mu);
	RRG_CUDA(cudaSetDevice(c->device));
	cudaStream_t s = (cudaStream_t)stream;
	if (n <= kHostChunk) {
		// page-locked rays and hits up to one chunk: the kernel reads the
		// rays and writes the hits in host memory itself (no staging copies,
		// no chunk bookkeeping)
		const void* rd = mapped_host(rays_host);
		void* hd = rd ? const_cast<void*>(mapped_host(hits_host)) : nullptr;
		if (rd && hd) {
			int st = launch_closest_mapped(c, reinterpret_cast<const float4*>(rd), n, reinterpret_cast<float4*>(hd), s);
			if (st) return st;
			RRG_CUDA(cudaStreamSynchronize(s));
			return RRG_OK;
		}
	}
	if (n <= kHostSingle) {
		int st = ensure_stage(c, 32 * (size_t)n, 16 * (size_t)n);
		if (st) return st;
		RRG_CUDA(cudaMemcpyAsync(c->d_stage_in, rays_host, 32 * (size_t)n, cudaMemcpyHostToDevice, s));
		st = launch_closest(c, reinterpret_cast<const float4*>(c->d_stage_in), n,
		                    reinterpret_cast<float4*>(c->d_stage_out), nullptr, nullptr, s);
		if (st) return st;
		RRG_CUDA(cudaMemcpyAsync(hits_host, c->d_stage_out, 16 * (size_t)n, cudaMemcpyDeviceToHost, s));
		RRG_CUDA(cudaStreamSynchronize(s));
		return RRG_OK;
	}
	// Large batches: chunks (chunk_schedule) through a ring of three staging
	// slots, rays copied in on s_in, traced alternately on the caller's
	// stream and s_comp (each slot with its own work counter, so a chunk's
	// kernel can start in the previous one's tail), hits copied out on
	// s_out: the copies of one chunk overlap the tracing of its neighbours.
	// (Writing the hit records of binned chunks straight into page-locked
	// host memory instead measured 25-50 % slower on GB300: the binned order
	// scatters them in 16-byte pieces over the host link.)
	std::vector<uint32_t> sizes;
	chunk_schedule(n, sizes);
	const uint32_t chunk = *std::max_element(sizes.begin(), sizes.end());
	int st = ensure_stage(c, 3 * 32 * (size_t)chunk, 3 * 16 * (size_t)chunk);
	if (!st) st = ensure_pipeline(c);
	if (st) return st;
	RRG_CUDA(cudaEventRecord(c->ev_start, s));   // after the caller's earlier work on s
	RRG_CUDA(cudaStreamWaitEvent(c->s_in, c->ev_start, 0));
	RRG_CUDA(cudaStreamWaitEvent(c->s_comp, c->ev_start, 0));
	size_t base = 0;
	for (uint32_t k = 0; k < (uint32_t)sizes.size(); k++) {
		const int slot = (int)(k % 3);
		const uint32_t m = sizes[k];
		float4* in = reinterpret_cast<float4*>(c->d_stage_in) + 2 * (size_t)chunk * slot;
		float4* out = reinterpret_cast<float4*>(c->d_stage_out) + (size_t)chunk * slot;
		if (k >= 3) RRG_CUDA(cudaStreamWaitEvent(c->s_in, c->ev_out[slot], 0));   // slot free again
		RRG_CUDA(cudaMemcpyAsync(in, rays_host + 8 * base, 32 * (size_t)m, cudaMemcpyHostToDevice, c->s_in));
		RRG_CUDA(cudaEventRecord(c->ev_in[slot], c->s_in));
		cudaStream_t cs = (k & 1) ? c->s_comp : s;
		RRG_CUDA(cudaStreamWaitEvent(cs, c->ev_in[slot], 0));
		st = launch_closest_on(c, in, m, out, nullptr, nullptr, c->d_counter + 4 * slot, cs, slot);
		if (st) return st;
		RRG_CUDA(cudaEventRecord(c->ev_done[slot], cs));
		RRG_CUDA(cudaStreamWaitEvent(c->s_out, c->ev_done[slot], 0));
		RRG_CUDA(cudaMemcpyAsync(hits_host + 4 * base, out, 16 * (size_t)m, cudaMemcpyDeviceToHost, c->s_out));
		RRG_CUDA(cudaEventRecord(c->ev_out[slot], c->s_out));
		base += m;
	}
	RRG_CUDA(cudaStreamSynchronize(c->s_out));
	RRG_CUDA(cudaStreamSynchronize(c->s_comp));
	RRG_CUDA(cudaStreamSynchronize(s));
	return RRG_OK;
}

int rrg_intersect_rrray_device(rrg_collider* h, void* rrrays_dev, uint32_t n, uint8_t* hit_dev, void* stream) {
	Collider* c = reinterpret_cast<Collider*>(h);
	if (!c) return RRG_ERR_INVALID;
	if (n == 0) return RRG_OK;
	if (!rrrays_dev || !aligned16(rrrays_dev)) return RRG_ERR_INVALID;
	return launch_rrray(c, rrrays_dev, n, hit_dev, (cudaStream_t)stream);
}

int rrg_intersect_rrray(rrg_collider* h, void* rrrays_host, uint32_t n, uint8_t* hit_host, void* stream) {
	Collider* c = reinterpret_cast<Collider*>(h);
	if (!c) return RRG_ERR_INVALID;
	if (n == 0) return RRG_OK;
	if (!rrrays_host) return RRG_ERR_INVALID;
	std::lock_guard<std::mutex> lk(c->host_mu);
	RRG_CUDA(cudaSetDevice(c->device));
	int st = ensure_stage(c, 128 * (size_t)n, (size_t)n);
	if (st) return st;
	cudaStream_t s = (cudaStream_t)stream;
	// bytes 0..91 of each record go up (inputs, and the output fields so that
	// fields the flags do not request come back unchanged); 44..91 come back
	RRG_CUDA(cudaMemcpy2DAsync(c->d_stage_in, 128, rrrays_host, 128, 92, n, cudaMemcpyHostToDevice, s));
	st = launch_rrray(c, c->d_stage_in, n, (uint8_t*)c->d_stage_out, s);
	if (st) return st;
	RRG_CUDA(cudaMemcpy2DAsync((uint8_t*)rrrays_host + 44, 128, (uint8_t*)c->d_stage_in + 44, 128, 48, n,
	                           cudaMemcpyDeviceToHost, s));
	if (hit_host) RRG_CUDA(cudaMemcpyAsync(hit_host, c->d_stage_out, n, cudaMemcpyDeviceToHost, s));
	RRG_CUDA(cudaStreamSynchronize(s));
	return RRG_OK;
}

int rrg_collider_status(rrg_collider* h, void* stream) {
	Collider* c = reinterpret_cast<Collider*>(h);
	if (!c) return RRG_ERR_INVALID;
	uint32_t w[12] = {0};
	cudaStream_t s = (cudaStream_t)stream;
	RRG_CUDA(cudaMemcpyAsync(w, c->d_counter, sizeof(w), cudaMemcpyDeviceToHost, s));
	RRG_CUDA(cudaStreamSynchronize(s));
	// status words of the direct launches ([1]) and of the pipelined slots ([5], [9])
	for (int k = 0; k < 3; k++) RRG_CUDA(cudaMemsetAsync(c->d_counter + 4 * k + 1, 0, 4, s));
	return (w[1] | w[5] | w[9]) ? RRG_ERR_STACK : RRG_OK;
}

}  // extern "C"
