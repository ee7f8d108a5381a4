// RRColliderGPU.hpp -- C++ host API of the GB300 collider, header-only over
// the C ABI (rrgpu.h).  It mirrors rr::RRCollider (include/Lightsprint/
// RRCollider.h in the reference) for programs that do not link the reference:
//
//   reference                                   here
//   RRCollider::create(mesh,0,tech,aborting)    RRColliderGPU::create(xyz,nv,idx,nt,aborting)   (RRCollider.h:183)
//   RRCollider::intersect(RRRay&) const         RRColliderGPU::intersect(RRRay&) const            (RRCollider.h:228)
//   (removed) RRCollider::intersectBatch        RRColliderGPU::intersectBatch(RRRay*,n) const     (doc.news:154)
//   RRCollider::update()                        RRColliderGPU::update(xyz)                        (RRCollider.h:190)
//   RRCollider::getMemoryOccupied() const       RRColliderGPU::getMemoryOccupied() const          (RRCollider.h:259)
//   RRCollider::getTechnique() const            RRColliderGPU::getTechnique() const               (RRCollider.h:250)
//   rr::RRRay (128 bytes)                       rrgpu::RRRay, same layout (static_asserts below)  (RRCollider.h:85-137)
//
// Unlike the reference, a failed create returns nullptr and leaves the status
// in *status; there is no IT_LINEAR fallback (RRCollider.cpp:236-239), the
// caller decides.  Collision handlers are not supported here; the
// reference-side plugin (rrgpu_rrcollider_plugin.hpp) replays them.
#ifndef RRCOLLIDERGPU_HPP
#define RRCOLLIDERGPU_HPP

#include <cstddef>
#include <cstdint>

#include "rrgpu.h"

namespace rrgpu {

// rr::RRRay, LP64 layout.
struct alignas(16) RRRay {
	enum Flags {
		FILL_DISTANCE = RRG_FILL_DISTANCE,
		FILL_POINT3D = RRG_FILL_POINT3D,
		FILL_POINT2D = RRG_FILL_POINT2D,
		FILL_PLANE = RRG_FILL_PLANE,
		FILL_TRIANGLE = RRG_FILL_TRIANGLE,
		FILL_SIDE = RRG_FILL_SIDE
	};
	float rayOrigin[4];      // w = 1
	float rayDir[4];         // normalized
	float rayLengthMin;
	float rayLengthMax;
	unsigned rayFlags;
	float hitDistance;
	unsigned hitTriangle;
	float hitPoint2d[2];
	float hitPlane[4];
	float hitPoint3d[3];
	bool hitFrontSide;
	float hitPadding1[3];
	float hitPadding2[2];
	const void* hitObject;
	void* collisionHandler;

	// RRRay::RRRay (RRCollider/RRRay.cpp:19-26): zeroed, all FILL flags on.
	RRRay() {
		unsigned char* p = reinterpret_cast<unsigned char*>(this);
		for (size_t i = 0; i < sizeof(RRRay); i++) p[i] = 0;
		rayOrigin[3] = 1;
		rayFlags = FILL_DISTANCE | FILL_POINT3D | FILL_POINT2D | FILL_PLANE | FILL_TRIANGLE | FILL_SIDE;
	}
};
static_assert(sizeof(RRRay) == 128, "rr::RRRay is 128 bytes");
static_assert(offsetof(RRRay, rayLengthMin) == 32 && offsetof(RRRay, rayFlags) == 40, "rr::RRRay inputs");
static_assert(offsetof(RRRay, hitDistance) == 44 && offsetof(RRRay, hitTriangle) == 48, "rr::RRRay outputs");
static_assert(offsetof(RRRay, hitPoint2d) == 52 && offsetof(RRRay, hitPlane) == 60, "rr::RRRay outputs");
static_assert(offsetof(RRRay, hitPoint3d) == 76 && offsetof(RRRay, hitFrontSide) == 88, "rr::RRRay outputs");
static_assert(offsetof(RRRay, hitObject) == 112 && offsetof(RRRay, collisionHandler) == 120, "rr::RRRay tail");

class RRColliderGPU {
public:
	// Technique number registered with RRCollider::registerTechnique.
	enum { IT_GPU = 100 };

	static RRColliderGPU* create(const float* xyz, unsigned nv, const unsigned* idx, unsigned nt, bool& aborting,
	                             const rrg_build_params* params = nullptr, int device = 0, int* status = nullptr) {
		rrg_collider* h = nullptr;
		volatile int abort_flag = aborting ? 1 : 0;
		int st = rrg_collider_create(xyz, nv, idx, nt, params, &abort_flag, device, &h);
		if (status) *status = st;
		if (st != RRG_OK) return nullptr;
		return new RRColliderGPU(h, nv);
	}

	// One ray; a blocking round trip to the device.  Thread-safe: calls from
	// many host threads at once are traced together as one batch.  Use
	// intersectBatch for throughput from one thread.
	bool intersect(RRRay& ray) const {
		uint8_t hit = 0;
		const int st = rrg_intersect_rrray_one(h_, &ray, &hit);
		last_status_ = st;
		return st == RRG_OK && hit;
	}

	// n rays in place; hit[i] (optional) = what intersect() would return.
	bool intersectBatch(RRRay* rays, unsigned n, unsigned char* hit = nullptr) const {
		last_status_ = rrg_intersect_rrray(h_, rays, n, hit, nullptr);
		if (last_status_ == RRG_OK) last_status_ = rrg_collider_status(h_, nullptr);
		return last_status_ == RRG_OK;
	}

	void update(const float* xyz) { last_status_ = rrg_collider_update(h_, xyz); }
	size_t getMemoryOccupied() const { return sizeof(*this) + rrg_collider_memory(h_); }
	unsigned getTechnique() const { return IT_GPU; }
	int lastStatus() const { return last_status_; }
	rrg_collider* handle() const { return h_; }
	~RRColliderGPU() { rrg_collider_destroy(h_); }

	RRColliderGPU(const RRColliderGPU&) = delete;
	RRColliderGPU& operator=(const RRColliderGPU&) = delete;

private:
	RRColliderGPU(rrg_collider* h, unsigned nv) : h_(h), nv_(nv) {}
	rrg_collider* h_;
	unsigned nv_;
	mutable int last_status_ = RRG_OK;
};

}  // namespace rrgpu

#endif
