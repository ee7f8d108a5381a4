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
//   * RRObjects input (multi-object colliders) is not handled here: the
//     builder returns nullptr and the reference falls back as it does for
//     any failed builder (RRCollider.cpp:236-239).
#ifndef RRGPU_RRCOLLIDER_PLUGIN_HPP
#define RRGPU_RRCOLLIDER_PLUGIN_HPP

#include <cmath>
#include <cstring>
#include <vector>

#include "Lightsprint/RRCollider.h"
#include "rrgpu.h"

namespace rrgpu_plugin {

enum { IT_GPU = 100 };

class GpuCollider : public rr::RRCollider {
public:
	static rr::RRCollider* build(const rr::RRMesh* mesh, const rr::RRObjects* objects, IntersectTechnique,
	                             bool& aborting, const char*, void*) {
		if (!mesh || objects) return nullptr;
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

	// Batch form for callers that own many rays (rays without handlers).
	bool intersectBatch(rr::RRRay* rays, unsigned n, unsigned char* hit) const {
		return rrg_intersect_rrray(h_, rays, n, hit, nullptr) == RRG_OK && rrg_collider_status(h_, nullptr) == RRG_OK;
	}

private:
	GpuCollider(const rr::RRMesh* m, rrg_collider* h, unsigned nt) : mesh_(m), h_(h), nt_(nt) {}
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
	const rr::RRMesh* mesh_;
	rrg_collider* h_;
	unsigned nt_;
};

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
