// rrg_intersect_rrray_noalloc: the RRRay batch query (k_rrray, the kernel
// behind rrg_intersect_rrray) with every byte of its device scratch in one
// static device array, so that a call allocates no device memory.
//
// Who needs it.  rrg_intersect_rrray keeps its staging buffers in the
// collider and grows them with cudaFree + cudaMalloc when a batch is larger
// than any before.  Two kinds of caller cannot take that:
//   * a per-frame loop (a realtime indirect-illumination update that casts
//     its rays every frame): cudaFree synchronises the whole device, so a
//     growing buffer stalls every stream of the process for that frame;
//   * a process whose device memory is already spoken for: a caching
//     allocator (PyTorch's) holding the free memory in its pools, or a bake
//     that sized its atlases and colliders to fill the GPU.  There cudaMalloc
//     fails with out-of-memory although the caller's work would fit.
// This entry point calls no cudaMalloc, cudaFree or allocating library
// routine; the price is a fixed batch limit and one scratch array per device
// shared by all calls.
//
// Scratch layout (kScratchBytes, 256-byte aligned):
//   [0, 4)        work counter of the persistent kernel  (cleared every call)
//   [4, 8)        status word (RRG_ERR_STACK on overflow) (cleared every call)
//   [256, ...)    RRG_NOALLOC_MAX_RAYS rr::RRRay records, 128 bytes each
//   [..., +max)   one hit byte per ray
// Records and hit bytes are overwritten for the rays of the call before the
// kernel reads them; bytes beyond the call's n keep the last call's contents
// and are never read.
#include "rrg_internal.cuh"

namespace rrg {
namespace {

constexpr size_t kRecordBytes = 128;
constexpr size_t kRecordsOffset = 256;
constexpr size_t kHitsOffset = kRecordsOffset + kRecordBytes * RRG_NOALLOC_MAX_RAYS;
constexpr size_t kScratchBytes = kHitsOffset + RRG_NOALLOC_MAX_RAYS;   // 2,113,792 bytes
static_assert(kHitsOffset % 16 == 0, "hit bytes follow whole records");

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// The device address of g_scratch on the current device.  Looked up on every
// call rather than cached: a context made after cudaDeviceReset may place the
// array elsewhere, and a cached address would then point at freed memory.
// The lookup allocates nothing; the first one on a device loads this file's
// module there (the set-up), which is why the first call should come before
// any stream capture.
int scratch_on(unsigned char** out) {
	void* sym = nullptr;
	RRG_CUDA(cudaGetSymbolAddress(&sym, g_scratch));
	*out = static_cast<unsigned char*>(sym);
	return RRG_OK;
}

}  // namespace
}  // namespace rrg

using namespace rrg;

extern "C" {

int rrg_intersect_rrray_noalloc(rrg_collider* h, void* rrrays_host, uint32_t n, uint8_t* hit_host, void* stream) {
	Collider* c = reinterpret_cast<Collider*>(h);
	if (!c) return RRG_ERR_INVALID;
	if (n == 0) return RRG_OK;
	if (!rrrays_host) return RRG_ERR_INVALID;
	if (n > RRG_NOALLOC_MAX_RAYS) return RRG_ERR_TOO_LARGE;
	RRG_CUDA(cudaSetDevice(c->device));
	unsigned char* base = nullptr;
	int st = scratch_on(&base);
	if (st) return st;
	uint32_t* words = reinterpret_cast<uint32_t*>(base);
	uint8_t* recs = base + kRecordsOffset;
	uint8_t* hits = base + kHitsOffset;
	cudaStream_t s = (cudaStream_t)stream;
	// the counter and the status word must start at zero; the array keeps
	// whatever the previous call left there
	RRG_CUDA(cudaMemsetAsync(words, 0, 2 * sizeof(uint32_t), s));
	// bytes 0..91 of each record go up, 44..91 (the outputs) come back, as in
	// rrg_intersect_rrray
	RRG_CUDA(cudaMemcpy2DAsync(recs, kRecordBytes, rrrays_host, kRecordBytes, 92, n, cudaMemcpyHostToDevice, s));
	st = launch_rrray_scratch(c, recs, n, hits, words, s);
	if (st) return st;
	RRG_CUDA(cudaMemcpy2DAsync((uint8_t*)rrrays_host + 44, kRecordBytes, recs + 44, kRecordBytes, 48, n,
	                           cudaMemcpyDeviceToHost, s));
	if (hit_host) RRG_CUDA(cudaMemcpyAsync(hit_host, hits, n, cudaMemcpyDeviceToHost, s));
	uint32_t status = 0;
	RRG_CUDA(cudaMemcpyAsync(&status, words + 1, sizeof(status), cudaMemcpyDeviceToHost, s));
	RRG_CUDA(cudaStreamSynchronize(s));
	return status ? RRG_ERR_STACK : RRG_OK;
}

}  // extern "C"
