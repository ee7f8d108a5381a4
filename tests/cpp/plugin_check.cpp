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
//
//   plugin_check multi SCENE RAYS OUT
//     RRObjects over a few meshes (each object's collider IT_BSP_FASTEST,
//     its world matrix, its enabled flag) and two multi-object colliders
//     over them, RRCollider::create(nullptr, &objects, technique): the GPU
//     technique and the reference's own RRColliderMulti (IT_LINEAR builder,
//     RRCollider.cpp:87-92).  Every ray once through each without a handler,
//     and once with a handler that accepts the second hit.
//     SCENE "RGO1": u32 nmesh, per mesh u32 nv, u32 nt, f32 xyz[3nv],
//     u32 idx[3nt]; u32 nobj, per object u32 mesh, u32 enabled, f32 m[12].
//     OUT.<gpu|ref>: per ray u8 hit, i32 object, u32 tri, f32 dist, f32 u,
//     f32 v, u8 side, then per ray of the handler pass u8 result, i32
//     object, u32 tri, u32 offers.
//
//   plugin_check lightmaps SCENE OUT plain|bake SEED
//     the scene of oracle/ref_gather.cpp ("RGS1", one object per atlas, its
//     triangles with their own vertices and face normals, one diffuse
//     material per triangle, one directional and one point light) in an
//     RRSolver whose static objects' collider is the GPU technique; lightmap
//     buffers (RGBA float, size x size) in layer 0 of the SCENE's output
//     atlases; then rrgpu_plugin::updateLightmaps (include/
//     rrgpu_update_lightmaps.hpp) with UpdateParameters(quality):
//     useCurrentSolution = true for "plain" (the plain N-bounce gather),
//     false for "bake" (the default bake), and FilteringParameters with
//     smoothing and spreading off.  OUT: "RGG1" as ref_gather writes it.
//     OUT.<gpu|ref>: per ray u32 count, count x (u32 tri, f32 dist), then
//     pass 2 as u8 result, u32 hitTriangle, f32 hitDistance, f32 u, f32 v,
//     f32 plane[4], f32 point3d[3], u8 hitFrontSide, u32 offers.
#include "Lightsprint/RRCollider.h"
#include "Lightsprint/RRLight.h"
#include "Lightsprint/RRSolver.h"
#include "rrgpu_rrcollider_plugin.hpp"
#include "rrgpu_update_lightmaps.hpp"
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

int object_index(const RRObjects& objects, const RRObject* o) {
	for (unsigned i = 0; i < objects.size(); i++)
		if (objects[i] == o) return (int)i;
	return -1;
}

void cast_multi(const RRCollider* collider, const RRObjects& objects, const float* rays, unsigned n,
                const char* path) {
	struct Rec {
		unsigned char hit, side;
		int obj;
		unsigned tri;
		float dist, u, v;
		unsigned char hres;
		int hobj;
		unsigned htri, hoffers;
	};
	std::vector<Rec> rec(n);
#pragma omp parallel
	{
		LogHandler h;
		RRRay ray;
#pragma omp for schedule(dynamic, 64)
		for (long long i = 0; i < (long long)n; i++) {
			const float* r = rays + 8 * (size_t)i;
			Rec& q = rec[i];
			for (int pass = 0; pass < 2; pass++) {
				ray.rayOrigin = RRVec3(r[0], r[1], r[2]);
				ray.rayDir = RRVec3(r[4], r[5], r[6]);
				ray.rayLengthMin = r[3];
				ray.rayLengthMax = r[7];
				ray.rayFlags = RRRay::FILL_DISTANCE | RRRay::FILL_TRIANGLE | RRRay::FILL_POINT2D | RRRay::FILL_SIDE;
				ray.hitObject = nullptr;
				ray.collisionHandler = pass ? &h : nullptr;
				h.accept_at = 1;
				const bool res = collider->intersect(ray);
				if (!pass) {
					q.hit = res ? 1 : 0;
					q.obj = res ? object_index(objects, ray.hitObject) : -1;
					q.tri = res ? ray.hitTriangle : ~0u;
					q.dist = res ? ray.hitDistance : 0.f;
					q.u = res ? ray.hitPoint2d[0] : 0.f;
					q.v = res ? ray.hitPoint2d[1] : 0.f;
					q.side = res && ray.hitFrontSide ? 1 : 0;
				} else {
					q.hres = res ? 1 : 0;
					q.hobj = res ? object_index(objects, ray.hitObject) : -1;
					q.htri = res ? ray.hitTriangle : ~0u;
					q.hoffers = (unsigned)h.tri.size();
				}
			}
		}
	}
	FILE* f = fopen(path, "wb");
	if (!f) return;
	for (unsigned i = 0; i < n; i++) {
		const Rec& q = rec[i];
		fwrite(&q.hit, 1, 1, f);
		fwrite(&q.obj, 4, 1, f);
		fwrite(&q.tri, 4, 1, f);
		fwrite(&q.dist, 4, 1, f);
		fwrite(&q.u, 4, 1, f);
		fwrite(&q.v, 4, 1, f);
		fwrite(&q.side, 1, 1, f);
	}
	for (unsigned i = 0; i < n; i++) {
		const Rec& q = rec[i];
		fwrite(&q.hres, 1, 1, f);
		fwrite(&q.hobj, 4, 1, f);
		fwrite(&q.htri, 4, 1, f);
		fwrite(&q.hoffers, 4, 1, f);
	}
	fclose(f);
}

int multi(int argc, char** argv) {
	if (argc < 5) return 2;
	std::vector<char> sb, rb;
	if (!read_file(argv[2], sb) || memcmp(sb.data(), "RGO1", 4)) return 2;
	if (!read_file(argv[3], rb) || memcmp(rb.data(), "RGR1", 4)) return 2;
	const char* p = sb.data() + 4;
	auto u32 = [&p]() {
		unsigned v;
		memcpy(&v, p, 4);
		p += 4;
		return v;
	};
	const unsigned nmesh = u32();
	std::vector<RRMesh*> meshes;
	bool aborting = false;
	rrgpu_plugin::registerGpuTechnique();
	std::vector<RRCollider*> own;
	for (unsigned m = 0; m < nmesh; m++) {
		const unsigned nv = u32(), nt = u32();
		float* xyz = (float*)p;
		p += 12 * (size_t)nv;
		unsigned* idx = (unsigned*)p;
		p += 12 * (size_t)nt;
		meshes.push_back(RRMesh::createIndexed(RRMesh::TRI_LIST, RRMesh::FLOAT32, xyz, nv, 12, RRMesh::UINT32, idx,
		                                       3 * nt, -1));
		own.push_back(RRCollider::create(meshes.back(), nullptr, RRCollider::IT_BSP_FASTEST, aborting,
		                                 "/proc/no-collider-cache/"));
	}
	const unsigned nobj = u32();
	RRObjects objects;
	std::vector<RRObject*> store;
	for (unsigned o = 0; o < nobj; o++) {
		const unsigned m = u32(), en = u32();
		float w[12];
		memcpy(w, p, 48);
		p += 48;
		RRObject* obj = new RRObject();
		obj->setCollider(own[m]);
		RRMatrix3x4 mat;
		for (int r = 0; r < 3; r++)
			for (int c = 0; c < 4; c++) mat.m[r][c] = w[4 * r + c];
		obj->setWorldMatrix(&mat);
		obj->enabled = en != 0;
		objects.push_back(obj);
		store.push_back(obj);
	}
	unsigned n;
	memcpy(&n, rb.data() + 4, 4);
	const float* rays = reinterpret_cast<const float*>(rb.data() + 8);
	RRCollider* gpu = RRCollider::create(nullptr, &objects, (RRCollider::IntersectTechnique)rrgpu_plugin::IT_GPU,
	                                     aborting);
	RRCollider* ref = RRCollider::create(nullptr, &objects, RRCollider::IT_LINEAR, aborting);
	if (!gpu || !ref) return 1;
	printf("{\"gpu_technique\": %d, \"ref_technique\": %d, \"rays\": %u, \"objects\": %u}\n",
	       (int)gpu->getTechnique(), (int)ref->getTechnique(), n, nobj);
	std::string out = argv[4];
	cast_multi(gpu, objects, rays, n, (out + ".gpu").c_str());
	cast_multi(ref, objects, rays, n, (out + ".ref").c_str());
	delete gpu;
	delete ref;
	for (RRObject* o : store) delete o;   // RRObject does not own its collider (RRObject.cpp:133-136)
	for (RRCollider* c : own) delete c;
	for (RRMesh* m : meshes) delete m;
	return 0;
}

int lightmaps(int argc, char** argv) {
	if (argc < 6) return 2;
	std::vector<char> sb;
	if (!read_file(argv[2], sb) || sb.size() < 32 || memcmp(sb.data(), "RGS1", 4)) return 2;
	unsigned hdr[7];
	memcpy(hdr, sb.data() + 4, sizeof(hdr));
	const unsigned nv = hdr[0], nt = hdr[1], natlas = hdr[2], size = hdr[3], quality = hdr[4], nout = hdr[5];
	const float* xyz = (const float*)(sb.data() + 32);
	const unsigned* idx = (const unsigned*)(xyz + 3 * (size_t)nv);
	const float* uv = (const float*)(idx + 3 * (size_t)nt);
	const float* albedo = uv + 6 * (size_t)nt;
	const int* atlas = (const int*)(albedo + 3 * (size_t)nt);
	const float* L = (const float*)(atlas + nt);
	const unsigned* out_atlas = (const unsigned*)(L + 12);
	const bool bake = !strcmp(argv[4], "bake");
	rrgpu_plugin::registerGpuTechnique();
	RRObjects objects;
	bool aborting = false;
	for (unsigned a = 0; a <= natlas; a++) {
		std::vector<unsigned> tris;
		for (unsigned t = 0; t < nt; t++)
			if (a < natlas ? atlas[t] == (int)a : atlas[t] < 0) tris.push_back(t);
		if (a == natlas && tris.empty()) break;
		const unsigned n = (unsigned)tris.size();
		RRMeshArrays* mesh = new RRMeshArrays();
		RRVector<unsigned> channels;
		channels.push_back(0);
		if (!mesh->resizeMesh(n, 3 * n, &channels, false, false)) return 3;
		RRMaterial* mats = new RRMaterial[n ? n : 1];
		RRObject* object = new RRObject();
		for (unsigned k = 0; k < n; k++) {
			const unsigned t = tris[k];
			RRVec3 p[3];
			for (unsigned c = 0; c < 3; c++) {
				const unsigned v = idx[3 * t + c];
				p[c] = RRVec3(xyz[3 * v], xyz[3 * v + 1], xyz[3 * v + 2]);
			}
			const RRVec3 nrm = (p[1] - p[0]).cross(p[2] - p[0]).normalized();
			for (unsigned c = 0; c < 3; c++) {
				mesh->triangle[k][c] = 3 * k + c;
				mesh->position[3 * k + c] = p[c];
				mesh->normal[3 * k + c] = nrm;
				mesh->texcoord[0][3 * k + c] = RRVec2(uv[6 * t + 2 * c], uv[6 * t + 2 * c + 1]);
			}
			mats[k].reset(false);
			mats[k].diffuseReflectance.color = RRVec3(albedo[3 * t], albedo[3 * t + 1], albedo[3 * t + 2]);
			mats[k].diffuseReflectance.colorLinear = mats[k].diffuseReflectance.color;
			mats[k].lightmap.texcoord = 0;
			object->faceGroups.push_back(RRObject::FaceGroup(&mats[k], 1));
		}
		object->setCollider(RRCollider::create(mesh, nullptr, RRCollider::IT_LINEAR, aborting));
		objects.push_back(object);
	}
	RRSolver* solver = new RRSolver();
	solver->setColorSpace(nullptr);
	solver->setStaticObjects(objects, nullptr, "/proc/no-collider-cache/",
	                         (RRCollider::IntersectTechnique)rrgpu_plugin::IT_GPU);
	RRLights lights;
	lights.push_back(RRLight::createDirectionalLight(RRVec3(L[0], L[1], L[2]), RRVec3(L[3], L[4], L[5]), true));
	lights.push_back(RRLight::createPointLight(RRVec3(L[6], L[7], L[8]), RRVec3(L[9], L[10], L[11])));
	solver->setLights(lights);
	std::vector<RRBuffer*> bufs;
	for (unsigned o = 0; o < nout; o++) {
		const unsigned a = out_atlas[o];
		if (a >= natlas) return 6;
		RRBuffer* b = RRBuffer::create(BT_2D_TEXTURE, size, size, 1, BF_RGBAF, false, nullptr);
		objects[a]->illumination.getLayer(0) = b;
		bufs.push_back(b);
	}
	RRSolver::UpdateParameters params(quality);
	params.useCurrentSolution = !bake;
	RRSolver::FilteringParameters filtering;
	filtering.smoothingAmount = 0;
	filtering.spreadForegroundColor = 0;
	rrgpu_plugin::UpdateLightmapsOptions opt;
	opt.seed = (uint64_t)strtoull(argv[5], nullptr, 0);
	const unsigned updated = rrgpu_plugin::updateLightmaps(solver, 0, &params, &filtering, opt);
	printf("{\"updated\": %u, \"multi_technique\": %d}\n", updated,
	       (int)solver->getMultiObject()->getCollider()->getTechnique());
	if (updated != nout) return 8;
	FILE* f = fopen(argv[3], "wb");
	if (!f) return 5;
	fwrite("RGG1", 1, 4, f);
	fwrite(&nout, 4, 1, f);
	fwrite(&size, 4, 1, f);
	for (unsigned o = 0; o < nout; o++) {
		std::vector<float> px((size_t)size * size * 4);
		for (unsigned i = 0; i < size * size; i++) {
			const RRVec4 e = bufs[o]->getElement(i, nullptr);
			for (int c = 0; c < 4; c++) px[4 * (size_t)i + c] = e[c];
		}
		fwrite(px.data(), sizeof(float), px.size(), f);
	}
	fclose(f);
	return 0;
}

}  // namespace

int main(int argc, char** argv) {
	if (argc > 1 && !strcmp(argv[1], "lightmaps")) return lightmaps(argc, argv);
	if (argc > 1 && !strcmp(argv[1], "handler")) return handler(argc, argv);
	if (argc > 1 && !strcmp(argv[1], "multi")) return multi(argc, argv);
	return hello();
}
