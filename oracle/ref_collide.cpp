// Runs the reference collider (built from the reference's own sources into
// oracle/_ref) on one mesh and one ray batch, and writes every ray's outputs.
// Test infrastructure only: it produces the golden vectors the GPU collider
// is checked against, and times the reference CPU collider.
//
//   ref_collide MESH RAYS OUT TECHNIQUE THREADS [FLAGS] [REPEAT]
//
// MESH : "RGM1", u32 nv, u32 nt, f32 xyz[nv*3], u32 idx[nt*3]
// RAYS : "RGR1", u32 n, f32 [n*8] = ox oy oz tmin dx dy dz tmax
// OUT  : "RGH1", u32 n, then arrays hit u8[n], tri u32[n], dist f32[n],
//        uv f32[2n], plane f32[4n], point3d f32[3n], side u8[n]
//        (OUT "-" writes nothing; only the timing line is printed)
// TECHNIQUE : linear | bsp_fast | bsp_fastest (RRCollider::IntersectTechnique,
//             include/Lightsprint/RRCollider.h:156-166)
// FLAGS : RRRay::rayFlags bit mask, default FILL_DISTANCE|FILL_POINT2D|
//         FILL_PLANE|FILL_TRIANGLE|FILL_SIDE|FILL_POINT3D
//
// Mirrors samples/BunnyBenchmark/BunnyBenchmark.cpp:59-113: mesh via
// RRMesh::createIndexed (no vertex stitching so indices stay as given),
// collider via RRCollider::create, rays traced in an OpenMP parallel for.
#include "Lightsprint/RRCollider.h"
#include <omp.h>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace rr;

static bool readFile(const char* path, std::vector<char>& buf) {
	FILE* f = fopen(path, "rb");
	if (!f) return false;
	fseek(f, 0, SEEK_END);
	long n = ftell(f);
	fseek(f, 0, SEEK_SET);
	buf.resize(n);
	bool ok = fread(buf.data(), 1, n, f) == (size_t)n;
	fclose(f);
	return ok;
}

int main(int argc, char** argv) {
	if (argc < 6) {
		fprintf(stderr, "usage: ref_collide MESH RAYS OUT TECHNIQUE THREADS [FLAGS] [REPEAT]\n");
		return 2;
	}
	std::vector<char> mb, rb;
	if (!readFile(argv[1], mb) || memcmp(mb.data(), "RGM1", 4)) { fprintf(stderr, "bad mesh\n"); return 2; }
	if (!readFile(argv[2], rb) || memcmp(rb.data(), "RGR1", 4)) { fprintf(stderr, "bad rays\n"); return 2; }
	unsigned nv, nt, n;
	memcpy(&nv, mb.data() + 4, 4);
	memcpy(&nt, mb.data() + 8, 4);
	memcpy(&n, rb.data() + 4, 4);
	float* xyz = (float*)(mb.data() + 12);
	unsigned* idx = (unsigned*)(mb.data() + 12 + 12 * (size_t)nv);
	const float* rays = (const float*)(rb.data() + 8);
	std::string tech = argv[4];
	int threads = atoi(argv[5]);
	unsigned flags = argc > 6 ? (unsigned)strtoul(argv[6], nullptr, 0)
	                          : (RRRay::FILL_DISTANCE | RRRay::FILL_POINT2D | RRRay::FILL_PLANE |
	                             RRRay::FILL_TRIANGLE | RRRay::FILL_SIDE | RRRay::FILL_POINT3D);
	int repeat = argc > 7 ? atoi(argv[7]) : 1;
	RRCollider::IntersectTechnique it =
		tech == "linear" ? RRCollider::IT_LINEAR :
		tech == "bsp_fast" ? RRCollider::IT_BSP_FAST :
		tech == "bsp_compact" ? RRCollider::IT_BSP_COMPACT :
		RRCollider::IT_BSP_FASTEST;

	RRMesh* mesh = RRMesh::createIndexed(RRMesh::TRI_LIST, RRMesh::FLOAT32, xyz, nv, 12,
	                                     RRMesh::UINT32, idx, 3 * nt, -1);
	if (!mesh) { fprintf(stderr, "createIndexed failed\n"); return 1; }
	bool aborting = false;
	auto t0 = std::chrono::steady_clock::now();
	// The cache file name is cacheLocation + hash + extension
	// (RRHash/RRHash.cpp:198-227); a directory that cannot exist makes both
	// the cache read and the cache write fail, so every run builds the tree.
	RRCollider* collider = RRCollider::create(mesh, nullptr, it, aborting, "/proc/no-collider-cache/");
	auto t1 = std::chrono::steady_clock::now();
	if (!collider) { fprintf(stderr, "create failed\n"); return 1; }

	std::vector<unsigned char> hit(n), side(n);
	std::vector<unsigned> tri(n);
	std::vector<float> dist(n), uv(2 * (size_t)n), plane(4 * (size_t)n), p3(3 * (size_t)n);
	if (threads > 0) omp_set_num_threads(threads);
	double best = 1e30;
	for (int rep = 0; rep < repeat; rep++) {
		auto a = std::chrono::steady_clock::now();
#pragma omp parallel
		{
			RRRay* ray = RRRay::create();
#pragma omp for schedule(dynamic, 4096)
			for (long i = 0; i < (long)n; i++) {
				const float* r = rays + 8 * (size_t)i;
				ray->rayOrigin = RRVec3(r[0], r[1], r[2]);
				ray->rayDir = RRVec3(r[4], r[5], r[6]);
				ray->rayLengthMin = r[3];
				ray->rayLengthMax = r[7];
				ray->rayFlags = flags;
				ray->collisionHandler = nullptr;
				bool h = collider->intersect(*ray);
				hit[i] = h;
				if (h) {
					tri[i] = ray->hitTriangle;
					dist[i] = ray->hitDistance;
					uv[2 * i] = ray->hitPoint2d[0];
					uv[2 * i + 1] = ray->hitPoint2d[1];
					for (int k = 0; k < 4; k++) plane[4 * i + k] = ray->hitPlane[k];
					for (int k = 0; k < 3; k++) p3[3 * i + k] = ray->hitPoint3d[k];
					side[i] = ray->hitFrontSide;
				} else {
					tri[i] = 0xFFFFFFFFu;
					dist[i] = 0;
					uv[2 * i] = uv[2 * i + 1] = 0;
					for (int k = 0; k < 4; k++) plane[4 * i + k] = 0;
					for (int k = 0; k < 3; k++) p3[3 * i + k] = 0;
					side[i] = 0;
				}
			}
			delete ray;
		}
		auto b = std::chrono::steady_clock::now();
		double s = std::chrono::duration<double>(b - a).count();
		if (s < best) best = s;
	}
	size_t hits = 0;
	for (unsigned i = 0; i < n; i++) hits += hit[i];
	int used = threads > 0 ? threads : omp_get_max_threads();
	printf("{\"technique\": \"%s\", \"got_technique\": %d, \"triangles\": %u, \"rays\": %u, \"threads\": %d, "
	       "\"build_s\": %.6f, \"trace_s\": %.6f, \"rays_per_s\": %.1f, \"hits\": %zu, \"memory\": %zu}\n",
	       tech.c_str(), (int)collider->getTechnique(), nt, n, used,
	       std::chrono::duration<double>(t1 - t0).count(), best, n / best, hits,
	       collider->getMemoryOccupied());
	if (strcmp(argv[3], "-")) {
		FILE* f = fopen(argv[3], "wb");
		if (!f) return 1;
		fwrite("RGH1", 1, 4, f);
		fwrite(&n, 4, 1, f);
		fwrite(hit.data(), 1, n, f);
		fwrite(tri.data(), 4, n, f);
		fwrite(dist.data(), 4, n, f);
		fwrite(uv.data(), 4, 2 * (size_t)n, f);
		fwrite(plane.data(), 4, 4 * (size_t)n, f);
		fwrite(p3.data(), 4, 3 * (size_t)n, f);
		fwrite(side.data(), 1, n, f);
		fclose(f);
	}
	delete collider;
	delete mesh;
	return 0;
}
