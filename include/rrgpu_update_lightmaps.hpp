// rrgpu_update_lightmaps.hpp -- the reference-side binding of the lightmap
// bake: RRSolver::updateLightmaps on the GB300 gather.  Include it in a
// program that builds against the reference's headers and links
// librrgpu.so, next to rrgpu_rrcollider_plugin.hpp:
//
//   solver->setStaticObjects(objects, ...);   solver->setLights(lights);
//   objects[i]->illumination.getLayer(layer) = RRBuffer::create(BT_2D_TEXTURE, size, size, ...);
//   unsigned n = rrgpu_plugin::updateLightmaps(solver, layer, &params, &filtering);
//
// It replaces RRSolver::updateLightmaps(layer, -1, -1, &params, &filtering)
// (RRSolver/lightmap.cpp:943-1163) and returns what that returns: the number
// of lightmaps updated.  What it reads from the solver, as the reference's
// updateLightmap does (lightmap.cpp:83-404, 648-930):
//   * the static scene: the multi-object's world-space mesh
//     (getMultiObject()->getCollider()->getMesh(), RRSolver.cpp:312), copied
//     to the GPU once per call (or the GPU collider itself when the
//     multi-object's collider is the GPU technique);
//   * per static object s and each post-import triangle of its mesh: the
//     multi-object triangle it became (getPostImportTriangle of
//     (s, getPreImportTriangle(...).index), lightmap.cpp:115-120), the
//     triangle's material (getTriangleMaterial) -- its diffuse reflectance
//     colorLinear as the albedo -- and its unwrap (getTriangleMapping in the
//     material's lightmap.texcoord channel, lightmap.cpp:127-131);
//   * the lightmaps: each static object's buffer in `layer`
//     (illumination.getLayer, lightmap.cpp:985), 2D RGBA float textures;
//     objects of one buffer size are baked together, one atlas per object;
//   * the lights (getLights): at most one directional and one point light
//     with realistic distance attenuation (RRLight.cpp:345-362, 450-455);
//   * UpdateParameters: quality, locality, aoIntensity, aoSize and
//     useCurrentSolution;  FilteringParameters: smoothingAmount,
//     spreadForegroundColor, backgroundColor, wrap.
// What runs, by the reference's own rule (lightmap.cpp:979, 1039-1056):
//   * quality > 0 and !useCurrentSolution (UpdateParameters' default): the
//     whole default bake -- the first gather per triangle and the radiosity
//     propagation (rrg_lightmapper_bake_solver) and then each lightmap's
//     final gather reading that solution at the first hit
//     (RRG_GATHER_SOLVER);
//   * useCurrentSolution with no solution computed by the GPU: the plain
//     N-bounce gather (PathTracingParameters::stopAtDepth bounces).  A
//     solution the reference's own solver computed earlier (calculate())
//     is not read.
// Then the post-filters of updateLightmap (lightmap.cpp:865-874) on the GPU
// (rrg_lightmap_filter), and the result is written into the buffers.
// Returns 0 (and updates nothing) for what the GPU gather does not cover:
// other light types or more than one light of a kind, non-square or
// non-2D buffers, directional lightmaps or bent normals (the layers those
// take are not parameters here), a quality above 256, and errors of the
// library.  The reference's sample streams are libc rand(), ours are
// counter-based: results agree statistically, not bit for bit.
#ifndef RRGPU_UPDATE_LIGHTMAPS_HPP
#define RRGPU_UPDATE_LIGHTMAPS_HPP

#include <climits>
#include <cstdint>
#include <cstring>
#include <map>
#include <vector>

#include "Lightsprint/RRBuffer.h"
#include "Lightsprint/RRLight.h"
#include "Lightsprint/RRObject.h"
#include "Lightsprint/RRSolver.h"
#include "rrgpu.h"
#include "rrgpu_gather.h"
#include "rrgpu_rrcollider_plugin.hpp"

namespace rrgpu_plugin {

struct UpdateLightmapsOptions {
	uint64_t seed = 0x5EED;        // first sample-stream seed (texel streams are seeded by texel id on top)
	uint32_t solver_iterations = 32;
};

inline unsigned updateLightmaps(rr::RRSolver* solver, int layer, const rr::RRSolver::UpdateParameters* params_in,
                                const rr::RRSolver::FilteringParameters* filtering,
                                const UpdateLightmapsOptions& opt = UpdateLightmapsOptions()) {
	if (!solver || layer < 0) return 0;
	rr::RRSolver::UpdateParameters params;
	if (params_in) params = *params_in;
	if (!params.quality || params.quality > 256) return 0;
	const rr::RRObject* multi = solver->getMultiObject();
	if (!multi || !multi->getCollider() || !multi->getCollider()->getMesh()) return 0;
	const rr::RRMesh* mm = multi->getCollider()->getMesh();
	const rr::RRObjects& objects = solver->getStaticObjects();
	const unsigned nt = mm->getNumTriangles();

	// lights: one directional, one point (realistic falloff)
	rrg_gather_params gp;
	memset(&gp, 0, sizeof(gp));
	gp.size = sizeof(gp);
	gp.quality = params.quality;
	gp.max_depth = rr::RRSolver::PathTracingParameters().stopAtDepth;   // updateLightmaps' path tracer: the defaults
	gp.seed = opt.seed;
	gp.locality = params.locality;
	gp.ao_intensity = params.aoIntensity;
	gp.ao_size = params.aoSize;
	bool have_dir = false, have_point = false;
	const rr::RRLights& lights = solver->getLights();
	for (unsigned i = 0; i < lights.size(); i++) {
		const rr::RRLight* L = lights[i];
		if (!L || !L->enabled) continue;
		if (L->type == rr::RRLight::DIRECTIONAL && !have_dir) {
			for (int k = 0; k < 3; k++) gp.dir_direction[k] = L->direction[k];
			for (int k = 0; k < 3; k++) gp.dir_color[k] = L->color[k];
			have_dir = true;
		} else if (L->type == rr::RRLight::POINT && L->distanceAttenuationType == rr::RRLight::REALISTIC &&
		           !have_point) {
			for (int k = 0; k < 3; k++) gp.point_position[k] = L->position[k];
			for (int k = 0; k < 3; k++) gp.point_color[k] = L->color[k];
			have_point = true;
		} else {
			return 0;
		}
	}

	// per multi-object triangle: albedo, unwrap, object (lightmapped ones)
	std::vector<float> albedo(3 * (size_t)nt, 0.f), uv(6 * (size_t)nt, 0.f);
	std::vector<int> owner(nt, -1);
	for (unsigned t = 0; t < nt; t++) {
		const rr::RRMaterial* m = multi->getTriangleMaterial(t, nullptr, nullptr);
		if (m)
			for (int k = 0; k < 3; k++) albedo[3 * (size_t)t + k] = m->diffuseReflectance.colorLinear[k];
	}
	std::map<unsigned, std::vector<unsigned>> by_size;   // buffer size -> objects
	for (unsigned o = 0; o < objects.size(); o++) {
		rr::RRBuffer* b = objects[o]->illumination.getLayer(layer);
		if (!b) continue;
		if (b->getType() != rr::BT_2D_TEXTURE || b->getWidth() != b->getHeight() || !b->getWidth()) return 0;
		by_size[b->getWidth()].push_back(o);
	}
	if (by_size.empty()) return 0;
	for (unsigned o = 0; o < objects.size(); o++) {
		const rr::RRObject* so = objects[o];
		const rr::RRMesh* sm = so->getCollider()->getMesh();
		const bool lit = so->illumination.getLayer(layer) != nullptr;
		for (unsigned s = 0; s < sm->getNumTriangles(); s++) {
			rr::RRMesh::PreImportNumber pre;
			pre.object = o;
			pre.index = sm->getPreImportTriangle(s).index;
			const unsigned t = mm->getPostImportTriangle(pre);
			if (t >= nt) continue;
			const rr::RRMaterial* m = so->getTriangleMaterial(s, nullptr, nullptr);
			if (m)
				for (int k = 0; k < 3; k++) albedo[3 * (size_t)t + k] = m->diffuseReflectance.colorLinear[k];
			if (!lit) continue;
			rr::RRMesh::TriangleMapping map;
			const unsigned channel = m ? m->lightmap.texcoord : UINT_MAX;
			if (!sm->getTriangleMapping(s, map, channel)) continue;
			for (int c = 0; c < 3; c++) {
				uv[6 * (size_t)t + 2 * c] = map.uv[c][0];
				uv[6 * (size_t)t + 2 * c + 1] = map.uv[c][1];
			}
			owner[t] = (int)o;
		}
	}

	// the collider: the multi-object's own when it is the GPU technique
	rrg_collider* col = nullptr;
	bool own_collider = false;
	if (const GpuCollider* g = dynamic_cast<const GpuCollider*>(multi->getCollider())) col = g->handle();
	if (!col) {
		std::vector<float> xyz;
		std::vector<unsigned> idx;
		GpuCollider::flatten(mm, xyz, idx);
		if (rrg_collider_create(xyz.data(), mm->getNumVertices(), idx.data(), nt, nullptr, nullptr, 0, &col) != RRG_OK)
			return 0;
		own_collider = true;
	}

	rrg_filter_params fp;
	rrg_filter_defaults(&fp);
	if (filtering) {
		fp.smoothing_amount = filtering->smoothingAmount;
		fp.spread_foreground = filtering->spreadForegroundColor;
		for (int k = 0; k < 4; k++) fp.background[k] = filtering->backgroundColor[k];
		fp.wrap = filtering->wrap ? 1 : 0;
	}
	const bool bake = !params.useCurrentSolution;
	unsigned updated = 0;
	bool failed = false;
	for (const auto& group : by_size) {
		const unsigned size = group.first;
		const std::vector<unsigned>& objs = group.second;
		std::vector<int32_t> tri_atlas(nt, -1);
		std::map<unsigned, int32_t> atlas_of;
		for (unsigned a = 0; a < objs.size(); a++) atlas_of[objs[a]] = (int32_t)a;
		for (unsigned t = 0; t < nt; t++)
			if (owner[t] >= 0 && atlas_of.count((unsigned)owner[t])) tri_atlas[t] = atlas_of[(unsigned)owner[t]];
		rrg_lightmapper* lm = nullptr;
		if (rrg_lightmapper_create(col, albedo.data(), tri_atlas.data(), uv.data(), (uint32_t)objs.size(), size, &lm) !=
		    RRG_OK) {
			failed = true;
			break;
		}
		const uint64_t S = (uint64_t)size * size, n = S * objs.size();
		std::vector<float> px(4 * (size_t)n);
		rrg_gather_params g2 = gp;
		int st = RRG_OK;
		if (bake) {
			st = rrg_lightmapper_bake_solver(lm, &gp, 0, opt.solver_iterations, nullptr);
			g2.mode = RRG_GATHER_SOLVER;
		}
		if (!st) st = rrg_lightmap_bake_host(lm, &g2, &fp, px.data());
		rrg_lightmapper_destroy(lm);
		if (st) {
			failed = true;
			break;
		}
		for (unsigned a = 0; a < objs.size(); a++) {
			rr::RRBuffer* b = objects[objs[a]]->illumination.getLayer(layer);
			for (uint64_t i = 0; i < S; i++) {
				const float* q = &px[4 * (size_t)(a * S + i)];
				b->setElement((unsigned)i, rr::RRVec4(q[0], q[1], q[2], q[3]), nullptr);
			}
			updated++;
		}
	}
	if (own_collider) rrg_collider_destroy(col);
	return failed ? 0 : updated;
}

}  // namespace rrgpu_plugin

#endif
