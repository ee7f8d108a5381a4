// Builds against the reference's own headers and library: registers the GPU
// technique through RRCollider::registerTechnique and runs the HelloCollider
// query (samples/HelloCollider/HelloCollider.cpp:15-42) through
// RRCollider::create / intersect.  Prints the technique create() returned and
// the hit.  Without a GPU the builder returns nullptr and the reference falls
// back to IT_LINEAR (RRCollider/RRCollider.cpp:236-239).
#include "Lightsprint/RRCollider.h"
#include "rrgpu_rrcollider_plugin.hpp"
#include <cstdio>

using namespace rr;

int main() {
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
