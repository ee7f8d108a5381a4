// The reference collider behind a small C interface, so that the benchmark
// times it in-process on the same ray arrays as the GPU collider (no files,
// no re-launch per step).  Test infrastructure: built into
// oracle/_ref/libref_bench.so from the reference's own library; only the
// benchmark's reference arm and CPU-baseline leg load it.
//
// The mesh and collider are made as samples/BunnyBenchmark/BunnyBenchmark.cpp
// :45-60 makes them (RRMesh over the caller's arrays, RRCollider::create with
// the asked technique), except that the mesh is indexed without vertex
// stitching so triangle numbers stay as given, and the collider cache is off
// so every create builds its tree.  Rays are cast as in BunnyBenchmark.cpp
// :66-106: an OpenMP parallel region, one RRRay per thread, re-filled for
// each ray and passed to RRCollider::intersect.
#include "Lightsprint/RRCollider.h"
#include <omp.h>
#include <chrono>
#include <cstring>
#include <vector>

using namespace rr;

namespace {

struct RefCollider {
	std::vector<float> xyz;
	std::vector<unsigned> idx;
	RRMesh* mesh = nullptr;
	RRCollider* collider = nullptr;
};

}  // namespace

extern "C" {

// technique: RRCollider::IntersectTechnique (IT_LINEAR 0 .. IT_BSP_FASTEST 4,
// include/Lightsprint/RRCollider.h:156-166).  *build_s = seconds of create().
__attribute__((visibility("default"))) void* refb_create(const float* xyz, unsigned nv, const unsigned* idx,
                                                         unsigned nt, int technique, double* build_s) {
	RefCollider* h = new RefCollider();
	h->xyz.assign(xyz, xyz + 3 * (size_t)nv);
	h->idx.assign(idx, idx + 3 * (size_t)nt);
	h->mesh = RRMesh::createIndexed(RRMesh::TRI_LIST, RRMesh::FLOAT32, h->xyz.data(), nv, 12, RRMesh::UINT32,
	                                h->idx.data(), 3 * nt, -1);
	if (!h->mesh) {
		delete h;
		return nullptr;
	}
	bool aborting = false;
	auto t0 = std::chrono::steady_clock::now();
	// cacheLocation + hash + extension names the cache file
	// (RRHash/RRHash.cpp:198-227); a directory that cannot exist makes the
	// read and the write fail, so the tree is always built.
	h->collider = RRCollider::create(h->mesh, nullptr, (RRCollider::IntersectTechnique)technique, aborting,
	                                 "/proc/no-collider-cache/");
	auto t1 = std::chrono::steady_clock::now();
	if (build_s) *build_s = std::chrono::duration<double>(t1 - t0).count();
	if (!h->collider) {
		delete h->mesh;
		delete h;
		return nullptr;
	}
	return h;
}

__attribute__((visibility("default"))) int refb_technique(void* p) {
	return (int)static_cast<RefCollider*>(p)->collider->getTechnique();
}

__attribute__((visibility("default"))) size_t refb_memory(void* p) {
	return static_cast<RefCollider*>(p)->collider->getMemoryOccupied();
}

// Closest hit for n rays (float[8] each: ox oy oz tmin dx dy dz tmax) on
// `threads` OpenMP threads (0 = every core).  hit/tri/dist/uv may be NULL;
// a missed ray gets tri 0xFFFFFFFF and zeros.  Returns the seconds the
// parallel loop took, or -1.
__attribute__((visibility("default"))) double refb_trace(void* p, const float* rays, size_t n, unsigned flags,
                                                         int threads, unsigned char* hit, unsigned* tri,
                                                         float* dist, float* uv) {
	RefCollider* h = static_cast<RefCollider*>(p);
	const RRCollider* collider = h->collider;
	const int nth = threads > 0 ? threads : omp_get_max_threads();
	auto t0 = std::chrono::steady_clock::now();
#pragma omp parallel num_threads(nth)
	{
		RRRay ray;
		ray.collisionHandler = nullptr;
#pragma omp for schedule(dynamic, 4096)
		for (long long i = 0; i < (long long)n; i++) {
			const float* r = rays + 8 * (size_t)i;
			ray.rayOrigin[0] = r[0];
			ray.rayOrigin[1] = r[1];
			ray.rayOrigin[2] = r[2];
			ray.rayLengthMin = r[3];
			ray.rayDir[0] = r[4];
			ray.rayDir[1] = r[5];
			ray.rayDir[2] = r[6];
			ray.rayLengthMax = r[7];
			ray.rayFlags = flags;
			const bool hh = collider->intersect(ray);
			if (hit) hit[i] = hh ? 1 : 0;
			if (tri) tri[i] = hh ? ray.hitTriangle : 0xFFFFFFFFu;
			if (dist) dist[i] = hh ? ray.hitDistance : 0.f;
			if (uv) {
				uv[2 * i] = hh ? ray.hitPoint2d[0] : 0.f;
				uv[2 * i + 1] = hh ? ray.hitPoint2d[1] : 0.f;
			}
		}
	}
	auto t1 = std::chrono::steady_clock::now();
	return std::chrono::duration<double>(t1 - t0).count();
}

__attribute__((visibility("default"))) void refb_destroy(void* p) {
	RefCollider* h = static_cast<RefCollider*>(p);
	if (!h) return;
	delete h->collider;
	delete h->mesh;
	delete h;
}

}  // extern "C"
