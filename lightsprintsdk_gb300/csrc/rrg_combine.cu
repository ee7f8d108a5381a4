// rrg_combine.cu -- single-ray queries from many host threads at once:
// rrg_intersect_rrray_one, behind the C ABI of include/rrgpu.h.
//
// rr::RRCollider::intersect(RRRay&) is documented thread-safe and callable
// from any number of host threads (include/Lightsprint/RRCollider.h:145,
// 217-228); the reference's own callers use it that way from OpenMP loops
// (RRSolver/gather.cpp:917, RRSolver/lightmap.cpp:368,
// samples/BunnyBenchmark/BunnyBenchmark.cpp:70-106).  On the GPU one ray per
// device round trip would both waste the round trip (~10 us) and make every
// thread contend for the collider's staging buffers.  Calls are therefore
// combined: a caller queues its ray; if one of the collider's kSlots
// combining slots is free it becomes that slot's combiner, takes every
// queued ray (its own and those that arrived meanwhile), traces them as one
// batch on the slot's own stream and buffers, copies each ray's outputs back
// into its record and wakes the waiters.  Otherwise it sleeps until its ray
// is done, or until a slot frees and it can combine what has queued since.
// The batch size thus follows the number of threads that call at once, and
// at most kSlots small batches of one collider are on the GPU together.
#include "rrg_internal.cuh"

#include <cmath>
#include <condition_variable>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

namespace rrg {

namespace {

struct Request {
	void* ray;        // one 128-byte rr::RRRay on the host
	uint8_t* hit;     // optional
	int status;
	bool done;
	float key_t;      // only hits after (key_t, key_tri) in (t, triangle) order;
	uint32_t key_tri; // key_t = -inf: every hit
	float* t_out;     // optional: the hit's watertight t
};

constexpr size_t kRecBytes = 128;   // sizeof(rr::RRRay)
constexpr size_t kInBytes = 92;     // bytes 0..91: inputs and the output fields
constexpr size_t kOutOffset = 44;   // hitDistance .. hitFrontSide
constexpr size_t kOutBytes = 48;
constexpr size_t kKeyOffset = 92;   // staged copy only: key_t, key_tri, then the hit's t (k_rrray, keyed)

}  // namespace

constexpr int kSlots = 4;

// Owned by the thread that marked the slot busy.
struct Slot {
	std::vector<Request*> batch;
	// one buffer each side, so that a batch costs one copy up and one down:
	// [16 B: work counter, status word, 0, 0][kRecBytes per ray][1 hit byte per ray]
	cudaStream_t s = nullptr;
	uint8_t* h_buf = nullptr;      // page-locked
	uint8_t* d_buf = nullptr;
	uint32_t cap = 0;
};

struct Combiner {
	std::mutex m;
	std::condition_variable cv;
	std::vector<Request*> queue;   // guarded by m
	bool busy[kSlots] = {};        // guarded by m
	Slot slot[kSlots];
	uint64_t batches = 0, rays = 0;   // guarded by m
};

Combiner* combiner_new() { return new (std::nothrow) Combiner(); }

void combiner_free(Combiner* k) {
	if (!k) return;
	for (Slot& sl : k->slot) {
		if (sl.s) cudaStreamDestroy(sl.s);
		cudaFreeHost(sl.h_buf);
		cudaFree(sl.d_buf);
	}
	delete k;
}

constexpr size_t kHead = 16;

// Buffers for n rays (grown by doubling, from 256).
static int reserve(Slot* k, uint32_t n) {
	if (!k->s) RRG_CUDA(cudaStreamCreateWithFlags(&k->s, cudaStreamNonBlocking));
	if (n <= k->cap) return RRG_OK;
	uint32_t cap = k->cap ? k->cap : 256;
	while (cap < n) cap *= 2;
	cudaFreeHost(k->h_buf);
	cudaFree(k->d_buf);
	k->h_buf = k->d_buf = nullptr;
	k->cap = 0;
	const size_t bytes = kHead + (kRecBytes + 1) * (size_t)cap;
	RRG_CUDA(cudaHostAlloc(&k->h_buf, bytes, cudaHostAllocDefault));
	RRG_CUDA(cudaMalloc(&k->d_buf, bytes));
	k->cap = cap;
	return RRG_OK;
}

// Traces k->batch; RRG_ERR_STACK if a traversal stack overflowed in it.
static int run_batch(Collider* c, Slot* k) {
	const uint32_t n = (uint32_t)k->batch.size();
	int st = reserve(k, n);
	if (st) return st;
	uint8_t* h_recs = k->h_buf + kHead;
	uint8_t* d_recs = k->d_buf + kHead;
	uint32_t* h_words = reinterpret_cast<uint32_t*>(k->h_buf);
	const size_t bytes = kHead + (kRecBytes + 1) * (size_t)n;
	// the words go up cleared with the records
	memset(k->h_buf, 0, kHead);
	for (uint32_t i = 0; i < n; i++) {
		uint8_t* rec = h_recs + kRecBytes * i;
		memcpy(rec, k->batch[i]->ray, kInBytes);
		memcpy(rec + kKeyOffset, &k->batch[i]->key_t, 4);
		memcpy(rec + kKeyOffset + 4, &k->batch[i]->key_tri, 4);
	}
	RRG_CUDA(cudaMemcpyAsync(k->d_buf, k->h_buf, kHead + kRecBytes * (size_t)n, cudaMemcpyHostToDevice, k->s));
	st = launch_rrray_scratch(c, d_recs, n, d_recs + kRecBytes * (size_t)n, reinterpret_cast<uint32_t*>(k->d_buf),
	                          k->s, 1);
	if (st) return st;
	RRG_CUDA(cudaMemcpyAsync(k->h_buf, k->d_buf, bytes, cudaMemcpyDeviceToHost, k->s));
	RRG_CUDA(cudaStreamSynchronize(k->s));
	const uint8_t* h_hit = h_recs + kRecBytes * (size_t)n;
	for (uint32_t i = 0; i < n; i++) {
		Request* r = k->batch[i];
		memcpy(static_cast<uint8_t*>(r->ray) + kOutOffset, h_recs + kRecBytes * i + kOutOffset, kOutBytes);
		if (r->hit) *r->hit = h_hit[i];
		if (r->t_out) memcpy(r->t_out, h_recs + kRecBytes * i + kKeyOffset + 8, 4);
	}
	return h_words[1] ? RRG_ERR_STACK : RRG_OK;
}

}  // namespace rrg

using namespace rrg;

extern "C" {

static int submit(Collider* c, Request& me) {
	Combiner* k = c->comb;
	if (!k) return RRG_ERR_OOM;
	std::unique_lock<std::mutex> lk(k->m);
	k->queue.push_back(&me);
	while (!me.done) {
		int free = -1;
		for (int j = 0; j < kSlots && free < 0; j++)
			if (!k->busy[j]) free = j;
		// nothing to combine (this call's ray is already in a batch) or no slot
		if (k->queue.empty() || free < 0) {
			k->cv.wait(lk);
			continue;
		}
		// combine everything queued so far, usually this call's ray included
		Slot* sl = &k->slot[free];
		k->busy[free] = true;
		sl->batch.swap(k->queue);
		lk.unlock();
		const cudaError_t e = cudaSetDevice(c->device);
		const int st = e == cudaSuccess ? run_batch(c, sl) : cuda_fail(e);
		lk.lock();
		for (Request* r : sl->batch) {
			r->status = st;
			r->done = true;
		}
		k->batches++;
		k->rays += sl->batch.size();
		sl->batch.clear();
		k->busy[free] = false;
		k->cv.notify_all();
	}
	return me.status;
}

int rrg_intersect_rrray_one(rrg_collider* h, void* rrray_host, uint8_t* hit_host) {
	Collider* c = reinterpret_cast<Collider*>(h);
	if (!c || !rrray_host) return RRG_ERR_INVALID;
	Request me{rrray_host, hit_host, RRG_OK, false, -INFINITY, 0u, nullptr};
	return submit(c, me);
}

int rrg_intersect_rrray_one_after(rrg_collider* h, void* rrray_host, float after_t, uint32_t after_tri,
                                  float* t_out, uint8_t* hit_host) {
	Collider* c = reinterpret_cast<Collider*>(h);
	if (!c || !rrray_host || after_t != after_t) return RRG_ERR_INVALID;
	Request me{rrray_host, hit_host, RRG_OK, false, after_t, after_tri, t_out};
	return submit(c, me);
}

int rrg_collider_combined(const rrg_collider* h, uint64_t* batches, uint64_t* rays) {
	const Collider* c = reinterpret_cast<const Collider*>(h);
	if (!c || !c->comb) return RRG_ERR_INVALID;
	std::lock_guard<std::mutex> lk(c->comb->m);
	if (batches) *batches = c->comb->batches;
	if (rays) *rays = c->comb->rays;
	return RRG_OK;
}

}  // extern "C"
