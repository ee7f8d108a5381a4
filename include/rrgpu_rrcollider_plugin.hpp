// rrgpu_rrcollider_plugin.hpp -- the reference-side binding: an
// rr::RRCollider implemented by the GB300 collider, registered as a new
// intersect technique.  Include it in a program (or in LightsprintCore) that
// builds against the reference's headers and link librrgpu.so:
//
//   #include "Lightsprint/RRCollider.h"
//   #include "rrgpu_rrcollider_plugin.hpp"
//   rrgpu_plugin::registerGpuTechnique();            // once
//   RRCollider* c = RRCollider::create(mesh, nullptr,
//       (RRCollider::IntersectTechnique)rrgpu_plugin::IT_GPU, aborting);
//
// The plug point is RRCollider::registerTechnique(unsigned, Builder*)
// (include/Lightsprint/RRCollider.h:169-171); create() dispatches on the
// technique number (RRCollider/RRCollider.cpp:204), so no header of the
// reference changes.  Semantics:
//   * the mesh is flattened once (getVertex/getTriangle, RRMesh.h:151,172)
//     and copied to the device; post-import triangle numbers are kept;
//   * intersect(RRRay&) without a collision handler is one device query,
//     thread-safe like the reference's (RRCollider.h:145): calls from many
//     host threads at once are combined into one batch
//     (rrg_intersect_rrray_one);
//   * with a collision handler, hits are offered to collides() nearest first
//     (the IT_BSP contract, RRCollider.h:52-55), each hit once: after a
//     rejection the next query asks for the nearest hit after the rejected
//     one in the order (watertight t, triangle index)
//     (rrg_intersect_rrray_one_after), so hits at equal distances are all
//     offered and none twice.  As in the reference's handler path
//     (IntersectBspFast.cpp:500-515 with intersect_triangleSRLNP :189-252),
//     hitDistance, hitTriangle, hitPoint2d, hitPlane and hitPoint3d are
//     filled for every offered hit, hitFrontSide when FILL_SIDE asks;
//   * RRObjects input (create(nullptr, &objects, ...), the multi-object
//     collider of RRCollider.cpp:87-92 and of RRSolver::getCollider,
//     RRSolver.cpp:445-475) builds GpuMultiCollider: the objects' meshes
//     (getCollider()->getMesh(), shared meshes once) in one multi-root BVH
//     and a two-level scene over the objects' world matrices and enabled
//     flags (rrgpu_scene.h).  A ray without a collision handler is one scene
//     query: RRColliderMulti's semantics (RRColliderMulti.cpp:103-147) with
//     hitObject, hitTriangle local to the object's mesh, hitDistance in
//     world space, hitPoint2d and hitFrontSide (flipped for mirroring
//     matrices); hitPlane and hitPoint3d are not filled.  A ray with a
//     handler goes to the reference's own RRColliderMulti over the objects'
//     own colliders (created with IT_LINEAR, which keeps the objects'
//     colliders as they are), so the handler sees exactly the reference's
//     ordered replay.  Like the reference's Embree scene collider, it reads
//     matrices and enabled flags at build and on update().
#ifndef RRGPU_RRCOLLIDER_PLUGIN_HPP
#define RRGPU_RRCOLLIDER_PLUGIN_HPP

#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "Lightsprint/RRCollider.h"
#include "Lightsprint/RRObject.h"
#include "rrgpu.h"
#include "rrgpu_scene.h"

namespace rrgpu_plugin {

enum { IT_GPU = 100 };

class GpuMultiCollider;

class GpuCollider : public rr::RRCollider {
public:
	static rr::RRCollider* build(const rr::RRMesh* mesh, const rr::RRObjects* objects, IntersectTechnique,
	                             bool& aborting, const char*, void*);
	static rr::RRCollider* build_mesh(const rr::RRMesh* mesh, bool& aborting) {
		if (!mesh) return nullptr;
		std::vector<float> xyz;
		std::vector<unsigned> idx;
		flatten(mesh, xyz, idx);
		rrg_collider* h = nullptr;
		volatile int ab = aborting ? 1 : 0;
		if (rrg_collider_create(xyz.data(), mesh->getNumVertices(), idx.data(), mesh->getNumTriangles(), nullptr,
		                        &ab, 0, &h) != RRG_OK)
			return nullptr;
		return new GpuCollider(mesh, h, mesh->getNumTriangles());
	}

	virtual void update() override {
		std::vector<float> xyz;
		std::vector<unsigned> idx;
		flatten(mesh_, xyz, idx);
		rrg_collider_update(h_, xyz.data());
	}

	virtual bool intersect(rr::RRRay& ray) const override {
		rr::RRCollisionHandler* handler = ray.collisionHandler;
		if (!handler) {
			uint8_t hit = 0;
			return rrg_intersect_rrray_one(h_, &ray, &hit) == RRG_OK && hit;
		}
		handler->init(ray);
		const unsigned flags = ray.rayFlags;   // after init, which may add flags (RRCollider.h:45-47)
		ray.rayFlags = flags | rr::RRRay::FILL_DISTANCE | rr::RRRay::FILL_TRIANGLE | rr::RRRay::FILL_POINT2D |
		               rr::RRRay::FILL_PLANE | rr::RRRay::FILL_POINT3D;
		float key_t = -INFINITY;
		unsigned key_tri = 0;
		// every round moves strictly forward in a finite order, so this ends
		// after at most one round per triangle
		for (unsigned round = 0; round <= nt_; round++) {
			uint8_t hit = 0;
			float t = 0;
			ray.collisionHandler = nullptr;
			const int st = rrg_intersect_rrray_one_after(h_, &ray, key_t, key_tri, &t, &hit);
			ray.collisionHandler = handler;
			if (st != RRG_OK || !hit) break;
			if (handler->collides(ray)) break;
			key_t = t;
			key_tri = ray.hitTriangle;
		}
		ray.rayFlags = flags;
		return handler->done();
	}

	virtual const rr::RRMesh* getMesh() const override { return mesh_; }
	virtual IntersectTechnique getTechnique() const override { return (IntersectTechnique)IT_GPU; }
	virtual size_t getMemoryOccupied() const override { return sizeof(*this) + rrg_collider_memory(h_); }
	virtual ~GpuCollider() { rrg_collider_destroy(h_); }
	// the C-ABI collider behind it (for other C-ABI calls on the same geometry)
	rrg_collider* handle() const { return h_; }

	// Batch form for callers that own many rays (rays without handlers).
	bool intersectBatch(rr::RRRay* rays, unsigned n, unsigned char* hit) const {
		return rrg_intersect_rrray(h_, rays, n, hit, nullptr) == RRG_OK && rrg_collider_status(h_, nullptr) == RRG_OK;
	}

	static void flatten(const rr::RRMesh* mesh, std::vector<float>& xyz, std::vector<unsigned>& idx) {
		unsigned nv = mesh->getNumVertices(), nt = mesh->getNumTriangles();
		xyz.resize(3 * (size_t)nv);
		idx.resize(3 * (size_t)nt);
		for (unsigned v = 0; v < nv; v++) {
			rr::RRMesh::Vertex p;
			mesh->getVertex(v, p);
			xyz[3 * (size_t)v] = p[0];
			xyz[3 * (size_t)v + 1] = p[1];
			xyz[3 * (size_t)v + 2] = p[2];
		}
		for (unsigned t = 0; t < nt; t++) {
			rr::RRMesh::Triangle tr;
			mesh->getTriangle(t, tr);
			idx[3 * (size_t)t] = tr[0];
			idx[3 * (size_t)t + 1] = tr[1];
			idx[3 * (size_t)t + 2] = tr[2];
		}
	}

private:
	GpuCollider(const rr::RRMesh* m, rrg_collider* h, unsigned nt) : mesh_(m), h_(h), nt_(nt) {}
	const rr::RRMesh* mesh_;
	rrg_collider* h_;
	unsigned nt_;
};

class GpuMultiCollider : public rr::RRCollider {
public:
	static rr::RRCollider* build(const rr::RRObjects& objects, bool& aborting) {
		const unsigned n = objects.size();
		if (!n) return nullptr;
		std::vector<const rr::RRMesh*> meshes;
		std::map<const rr::RRMesh*, unsigned> index;
		std::vector<uint32_t> obj_mesh(n);
		for (unsigned i = 0; i < n; i++) {
			const rr::RRCollider* oc = objects[i] ? objects[i]->getCollider() : nullptr;
			const rr::RRMesh* m = oc ? oc->getMesh() : nullptr;
			if (!m) return nullptr;
			auto it = index.find(m);
			if (it == index.end()) {
				it = index.emplace(m, (unsigned)meshes.size()).first;
				meshes.push_back(m);
			}
			obj_mesh[i] = it->second;
		}
		std::vector<float> xyz;
		std::vector<unsigned> idx;
		std::vector<uint32_t> vert_off(1, 0), tri_off(1, 0);
		for (const rr::RRMesh* m : meshes) {
			std::vector<float> x;
			std::vector<unsigned> t;
			GpuCollider::flatten(m, x, t);
			xyz.insert(xyz.end(), x.begin(), x.end());
			idx.insert(idx.end(), t.begin(), t.end());
			vert_off.push_back(vert_off.back() + (uint32_t)(x.size() / 3));
			tri_off.push_back(tri_off.back() + (uint32_t)(t.size() / 3));
		}
		if (aborting) return nullptr;
		rrg_batch* b = nullptr;
		if (rrg_batch_create(xyz.data(), vert_off.data(), idx.data(), tri_off.data(), (uint32_t)meshes.size(), nullptr,
		                     0, &b) != RRG_OK)
			return nullptr;
		std::vector<float> world;
		std::vector<uint8_t> enabled;
		read_objects(objects, world, enabled);
		rrg_scene* sc = nullptr;
		if (rrg_scene_create(b, n, obj_mesh.data(), world.data(), &sc) != RRG_OK ||
		    rrg_scene_set_enabled(sc, enabled.data()) != RRG_OK) {
			rrg_scene_destroy(sc);
			rrg_batch_destroy(b);
			return nullptr;
		}
		// rays with a collision handler: the reference's RRColliderMulti
		// (defaultBuilder with no mesh, RRCollider.cpp:87-92)
		rr::RRCollider* replay = rr::RRCollider::create(nullptr, &objects, rr::RRCollider::IT_LINEAR, aborting);
		return new GpuMultiCollider(objects, b, sc, replay);
	}

	virtual void update() override {
		std::vector<float> world;
		std::vector<uint8_t> enabled;
		read_objects(objects_, world, enabled);
		rrg_scene_set_matrices(scene_, world.data());
		rrg_scene_set_enabled(scene_, enabled.data());
		if (replay_) replay_->update();
	}

	virtual bool intersect(rr::RRRay& ray) const override {
		if (ray.collisionHandler) return replay_ && replay_->intersect(ray);
		const float r[8] = {ray.rayOrigin[0], ray.rayOrigin[1], ray.rayOrigin[2], ray.rayLengthMin,
		                    ray.rayDir[0],    ray.rayDir[1],    ray.rayDir[2],    ray.rayLengthMax};
		float h[4];
		uint32_t obj = 0;
		if (rrg_scene_intersect_host(scene_, r, 1, h, &obj) != RRG_OK) return false;
		uint32_t bits;
		memcpy(&bits, &h[1], 4);
		if (bits == 0xFFFFFFFFu || obj >= objects_.size()) return false;
		const unsigned f = ray.rayFlags;
		if (f & rr::RRRay::FILL_DISTANCE) ray.hitDistance = h[0];
		if (f & rr::RRRay::FILL_TRIANGLE) ray.hitTriangle = bits & 0x7FFFFFFFu;
		if (f & rr::RRRay::FILL_POINT2D) {
			ray.hitPoint2d[0] = h[2];
			ray.hitPoint2d[1] = h[3];
		}
		if (f & rr::RRRay::FILL_SIDE) ray.hitFrontSide = (bits >> 31) != 0;
		ray.hitObject = objects_[obj];
		return true;
	}

	virtual const rr::RRMesh* getMesh() const override { return nullptr; }
	virtual IntersectTechnique getTechnique() const override { return (IntersectTechnique)IT_GPU; }
	virtual size_t getMemoryOccupied() const override { return sizeof(*this) + rrg_batch_memory(batch_); }
	virtual ~GpuMultiCollider() {
		delete replay_;
		rrg_scene_destroy(scene_);
		rrg_batch_destroy(batch_);
	}

private:
	GpuMultiCollider(const rr::RRObjects& o, rrg_batch* b, rrg_scene* s, rr::RRCollider* replay)
	    : objects_(o), batch_(b), scene_(s), replay_(replay) {}
	static void read_objects(const rr::RRObjects& objects, std::vector<float>& world, std::vector<uint8_t>& enabled) {
		const unsigned n = objects.size();
		world.assign(12 * (size_t)n, 0.f);
		enabled.assign(n, 0);
		for (unsigned i = 0; i < n; i++) {
			const rr::RRMatrix3x4Ex* w = objects[i]->getWorldMatrix();   // nullptr = identity (RRObject.h:194)
			for (int r = 0; r < 3; r++)
				for (int c = 0; c < 4; c++) world[12 * (size_t)i + 4 * r + c] = w ? w->m[r][c] : (r == c ? 1.f : 0.f);
			enabled[i] = objects[i]->enabled ? 1 : 0;
		}
	}
	rr::RRObjects objects_;
	rrg_batch* batch_;
	rrg_scene* scene_;
	rr::RRCollider* replay_;
};

inline rr::RRCollider* GpuCollider::build(const rr::RRMesh* mesh, const rr::RRObjects* objects, IntersectTechnique,
                                          bool& aborting, const char*, void*) {
	if (mesh) return build_mesh(mesh, aborting);
	return objects ? GpuMultiCollider::build(*objects, aborting) : nullptr;
}

// RRCollider::create registers the built-in builders only while its registry
// is empty (RRCollider/RRCollider.cpp:189-202); registering first would leave
// IT_LINEAR unregistered and break the reference's fallback (:236-239).  A
// create() with no mesh and no objects fills the registry and returns nullptr
// (defaultBuilder, :89-92) before the GPU technique is added.
inline void registerGpuTechnique() {
	bool aborting = false;
	rr::RRCollider::create(nullptr, nullptr, rr::RRCollider::IT_LINEAR, aborting);
	rr::RRCollider::registerTechnique(IT_GPU, &GpuCollider::build);
}

}  // namespace rrgpu_plugin

#endif
