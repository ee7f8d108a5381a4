// Builds against the reference's own headers and library and goes through
// RRCollider::registerTechnique / create / intersect.
//
//   plugin_check
//     registers the GPU technique and runs the HelloCollider query
//     (samples/HelloCollider/HelloCollider.cpp:15-42) through
//     RRCollider::create / intersect; prints the technique create() returned
//     and the hit.  Without a GPU the builder returns nullptr and the
//     reference falls back to IT_LINEAR (RRCollider/RRCollider.cpp:236-239).
//
//   plugin_check handler MESH RAYS OUT ACCEPT_AT
//     one RRMesh (RRMesh::createIndexed, no vertex stitching) and two
//     colliders over it: the GPU technique and the reference's
//     IT_BSP_FASTEST.  Every ray is cast through each collider twice with a
//     collision handler that logs each hit offered to collides():
//       pass 1 rejects every hit, so the log is the whole sequence of hits
//              in the order the collider offers them;
//       pass 2 accepts the hit offered at position ACCEPT_AT (0-based) and
//              rejects those before it; intersect() then returns done(),
//              and the ray's fields are those of the accepted hit.
//     MESH and RAYS use the formats of oracle/refio.py ("RGM1", "RGR1").
//     OUT.<gpu|ref>: per ray u32 count, count x (u32 tri, f32 dist), then
//     pass 2 as u8 result, u32 hitTriangle, f32 hitDistance, f32 u, f32 v,
//     f32 plane[4], f32 point3d[3], u8 hitFrontSide, u32 offers.
#include "Lightsprint/RRCollider.h"
#include "rrgpu_rrcollider_plugin.hpp"
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace rr;

namespace {

class LogHandler : public RRCollisionHandler {
public:
	unsigned accept_at = ~0u;
	std::vector<unsigned> tri;
	std::vector<float> dist;
	void init(RRRay&) override {
		tri.clear();
		dist.clear();
	}
	bool collides(const RRRay& ray) override {
		tri.push_back(ray.hitTriangle);
		dist.push_back(ray.hitDistance);
		return tri.size() > accept_at;
	}
	bool done() override { return tri.size() > accept_at; }
};

bool read_file(const char* path, std::vector<char>& buf) {
	FILE* f = fopen(path, "rb");
	if (!f) return false;
	fseek(f, 0, SEEK_END);
	const long n = ftell(f);
	fseek(f, 0, SEEK_SET);
	buf.resize(n);
	const bool ok = fread(buf.data(), 1, n, f) == (size_t)n;
	fclose(f);
	return ok;
}

int hello() {
	rrgpu_plugin::registerGpuTechnique();
	float vertexArray[18] = {-1, 0, 0, 1, 0, 0, 0, 1, 0, 1, 0, 0, -1, 0, 0, 0, 0, 1};
	RRMesh* mesh = RRMesh::create(RRMesh::TRI_LIST, RRMesh::FLOAT32, vertexArray, 6, 3 * sizeof(float));
	bool aborting = false;
	RRCollider* collider = RRCollider::create(mesh, nullptr, (RRCollider::IntersectTechnique)rrgpu_plugin::IT_GPU,
	                                          aborting, "/proc/no-collider-cache/");
	RRRay ray;
	ray.rayOrigin = RRVec3(0, -1, 0.3f);
	ray.rayDir = RRVec3(0, 1, 0);
	ray.rayLengthMin = 0;
	ray.rayLengthMax = 1000;
	bool hit = collider->intersect(ray);
	printf("technique=%d hit=%d tri=%u dist=%g u=%g v=%g front=%d\n", (int)collider->getTechnique(), (int)hit,
	       ray.hitTriangle, ray.hitDistance, ray.hitPoint2d[0], ray.hitPoint2d[1], (int)ray.hitFrontSide);
	delete collider;
	delete mesh;
	return 0;
}

void cast_all(const RRCollider* collider, const float* rays, unsigned n, unsigned accept_at, const char* path) {
	std::vector<std::vector<unsigned>> seq_tri(n), pass2_tri(n);
	std::vector<std::vector<float>> seq_dist(n);
	struct Rec {
		unsigned char result, side;
		unsigned tri, offers;
		float dist, u, v, plane[4], p3[3];
	};
	std::vector<Rec> rec(n);
#pragma omp parallel
	{
		LogHandler h;
		RRRay ray;
#pragma omp for schedule(dynamic, 16)
		for (long long i = 0; i < (long long)n; i++) {
			const float* r = rays + 8 * (size_t)i;
			for (int pass = 0; pass < 2; pass++) {
				ray.rayOrigin = RRVec3(r[0], r[1], r[2]);
				ray.rayDir = RRVec3(r[4], r[5], r[6]);
				ray.rayLengthMin = r[3];
				ray.rayLengthMax = r[7];
				ray.rayFlags = RRRay::FILL_DISTANCE | RRRay::FILL_TRIANGLE | RRRay::FILL_POINT2D | RRRay::FILL_SIDE;
				ray.hitTriangle = ~0u;
				ray.collisionHandler = &h;
				h.accept_at = pass == 0 ? ~0u : accept_at;
				const bool res = collider->intersect(ray);
				if (pass == 0) {
					seq_tri[i] = h.tri;
					seq_dist[i] = h.dist;
				} else {
					Rec& q = rec[i];
					q.result = res ? 1 : 0;
					q.tri = ray.hitTriangle;
					q.dist = ray.hitDistance;
					q.u = ray.hitPoint2d[0];
					q.v = ray.hitPoint2d[1];
					for (int k = 0; k < 4; k++) q.plane[k] = ray.hitPlane[k];
					for (int k = 0; k < 3; k++) q.p3[k] = ray.hitPoint3d[k];
					q.side = ray.hitFrontSide ? 1 : 0;
					q.offers = (unsigned)h.tri.size();
				}
			}
		}
	}
	FILE* f = fopen(path, "wb");
	if (!f) return;
	for (unsigned i = 0; i < n; i++) {
		const unsigned c = (unsigned)seq_tri[i].size();
		fwrite(&c, 4, 1, f);
		for (unsigned k = 0; k < c; k++) {
			fwrite(&seq_tri[i][k], 4, 1, f);
			fwrite(&seq_dist[i][k], 4, 1, f);
		}
	}
	for (unsigned i = 0; i < n; i++) {
		const Rec& q = rec[i];
		fwrite(&q.result, 1, 1, f);
		fwrite(&q.tri, 4, 1, f);
		fwrite(&q.dist, 4, 1, f);
		fwrite(&q.u, 4, 1, f);
		fwrite(&q.v, 4, 1, f);
		fwrite(q.plane, 4, 4, f);
		fwrite(q.p3, 4, 3, f);
		fwrite(&q.side, 1, 1, f);
		fwrite(&q.offers, 4, 1, f);
	}
	fclose(f);
}

int handler(int argc, char** argv) {
	if (argc < 6) return 2;
	std::vector<char> mb, rb;
	if (!read_file(argv[2], mb) || memcmp(mb.data(), "RGM1", 4)) return 2;
	if (!read_file(argv[3], rb) || memcmp(rb.data(), "RGR1", 4)) return 2;
	unsigned nv, nt, n;
	memcpy(&nv, mb.data() + 4, 4);
	memcpy(&nt, mb.data() + 8, 4);
	memcpy(&n, rb.data() + 4, 4);
	float* xyz = reinterpret_cast<float*>(mb.data() + 12);
	unsigned* idx = reinterpret_cast<unsigned*>(mb.data() + 12 + 12 * (size_t)nv);
	const float* rays = reinterpret_cast<const float*>(rb.data() + 8);
	const unsigned accept_at = (unsigned)atoi(argv[5]);
	rrgpu_plugin::registerGpuTechnique();
	RRMesh* mesh = RRMesh::createIndexed(RRMesh::TRI_LIST, RRMesh::FLOAT32, xyz, nv, 12, RRMesh::UINT32, idx, 3 * nt,
	                                     -1);
	if (!mesh) return 1;
	bool aborting = false;
	RRCollider* gpu = RRCollider::create(mesh, nullptr, (RRCollider::IntersectTechnique)rrgpu_plugin::IT_GPU, aborting,
	                                     "/proc/no-collider-cache/");
	RRCollider* ref = RRCollider::create(mesh, nullptr, RRCollider::IT_BSP_FASTEST, aborting,
	                                     "/proc/no-collider-cache/");
	if (!gpu || !ref) return 1;
	printf("{\"gpu_technique\": %d, \"ref_technique\": %d, \"rays\": %u, \"triangles\": %u}\n",
	       (int)gpu->getTechnique(), (int)ref->getTechnique(), n, nt);
	std::string out = argv[4];
	cast_all(gpu, rays, n, accept_at, (out + ".gpu").c_str());
	cast_all(ref, rays, n, accept_at, (out + ".ref").c_str());
	delete gpu;
	delete ref;
	delete mesh;
	return 0;
}

}  // namespace

int main(int argc, char** argv) {
	if (argc > 1 && !strcmp(argv[1], "handler")) return handler(argc, argv);
	return hello();
}
