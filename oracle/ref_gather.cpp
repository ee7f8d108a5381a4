// Runs the reference's own per-texel gather (processTexel, RRSolver/gather.cpp:
// 600-836, called by enumerateTexelsPartial, RRSolver/lightmap.cpp:83-404, as
// updateLightmap does at lightmap.cpp:823) on a scene of unwrapped objects,
// built from the reference's sources into oracle/_ref.  Test infrastructure
// only: the golden vectors that pin the plain N-bounce estimator of the
// oracle (oracle/rr_gather.c) and of the GPU gather statistically.
//
//   ref_gather SCENE OUT [THREADS] [bake]
//
// SCENE : "RGS1", u32 nv, u32 nt, u32 natlas, u32 size, u32 quality,
//         u32 nout, u32 seed, f32 xyz[3nv], u32 idx[3nt], f32 uv[6nt]
//         (lightmap uv of each triangle corner), f32 albedo[3nt],
//         i32 atlas[nt], f32 lights[12] (directional light: direction the
//         light travels, colour; point light: position, colour),
//         u32 out_atlas[nout]
// OUT   : "RGG1", u32 nout, u32 size, then per output atlas
//         f32 rgba[size*size*4] (alpha = TexelFlags / 255 where covered)
// OUT.solver (bake only): "RGB1", u32 nt, then per triangle (our order)
//         f32 direct[3], indirect[3] (flat), corner indirect[3][3] (smoothed)
//
// Atlas a is object a (its triangles in index order, three vertices of their
// own each, vertex normal = the face normal (v1-v0)x(v2-v0), one one-sided
// diffuse material per triangle); all objects are the solver's static
// objects, IT_BSP_FASTEST.  The architect solver is never created (no
// calculateCore, no updateSolver*), so the hemisphere's PathtracerWorker
// finds no solver triangles (pathtracer.cpp:74) and, at every hit, shoots
// shadow rays to the lights (pathtracer.cpp:254-300) and continues the path
// by Russian roulette (pathtracer.cpp:352-381) up to the default
// PathTracingParameters::stopAtDepth (20) and stopAtVisibility (0.001):
// the plain N-bounce estimator.  UpdateParameters: quality as given,
// useCurrentSolution = true (so the hemisphere shoots, gather.cpp:197), the
// rest default (locality 100000, no AO, multipliers 1).
//
// With "bake" the reference's whole default bake runs instead:
// RRSolver::updateLightmaps(layer 0, -1, -1, UpdateParameters(quality),
// filtering) (lightmap.cpp:943-1163): the first gather per triangle at half
// quality and the radiosity propagation (updateSolverIndirectIllumination,
// gather.cpp:1038-1117), then each requested atlas's final gather reading
// the solver at the first hit.  Filtering: smoothingAmount 0 and
// spreadForegroundColor 0, so covered texels keep their gathered values
// (growForBilinear and the background fill touch only empty texels).
#include "Lightsprint/RRCollider.h"
#include "Lightsprint/RRLight.h"
#include "Lightsprint/RRMesh.h"
#include "Lightsprint/RRObject.h"
#include "Lightsprint/RRSolver.h"
#include "RRSolver/gather.h"
#include <omp.h>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace rr {
// The statistics record enumerateTexelsPartial fills; it is defined inside
// lightmap.cpp (lightmap.cpp:47-81), so the same fields are declared here to
// call it.
struct UnwrapStatistics {
	bool subtexelsInMapSpace = false;
	unsigned numTrianglesWithoutUnwrap = 0;
	unsigned numTrianglesWithUnwrap = 0;
	unsigned pass = 0;
	unsigned numTrianglesWithUnwrapOutOfRange = 0;
	float areaOfAllTriangles = 0;
	float areaOfAllTrianglesInRange = 0;
	unsigned numTexelsProcessed = 0;
};
bool enumerateTexelsPartial(const RRObject* multiObject, unsigned objectNumber, unsigned mapWidth, unsigned mapHeight,
                            unsigned rectXMin, unsigned rectYMin, unsigned rectXMaxPlus1, unsigned rectYMaxPlus1,
                            ProcessTexelResult(callback)(const struct ProcessTexelParams& pti), const LightmapperJob& lmj,
                            RRReal minimalSafeDistance, UnwrapStatistics& unwrapStatistics, int onlyTriangleNumber);
}  // namespace rr

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
	if (argc < 3) {
		fprintf(stderr, "usage: ref_gather SCENE OUT [THREADS]\n");
		return 2;
	}
	std::vector<char> sb;
	if (!readFile(argv[1], sb) || sb.size() < 32 || memcmp(sb.data(), "RGS1", 4)) {
		fprintf(stderr, "bad scene\n");
		return 2;
	}
	unsigned hdr[7];
	memcpy(hdr, sb.data() + 4, sizeof(hdr));
	const unsigned nv = hdr[0], nt = hdr[1], natlas = hdr[2], size = hdr[3], quality = hdr[4], nout = hdr[5],
	               seed = hdr[6];
	const float* xyz = (const float*)(sb.data() + 32);
	const unsigned* idx = (const unsigned*)(xyz + 3 * (size_t)nv);
	const float* uv = (const float*)(idx + 3 * (size_t)nt);
	const float* albedo = uv + 6 * (size_t)nt;
	const int* atlas = (const int*)(albedo + 3 * (size_t)nt);
	const float* L = (const float*)(atlas + nt);
	const unsigned* out_atlas = (const unsigned*)(L + 12);
	if (argc > 3 && atoi(argv[3]) > 0) omp_set_num_threads(atoi(argv[3]));
	srand(seed);

	// one object per atlas (triangles in index order), then the triangles of no atlas
	RRObjects objects;
	bool aborting = false;
	std::vector<unsigned> multi_of(nt);   // our triangle -> the multi-object's
	unsigned nmulti = 0;
	for (unsigned a = 0; a <= natlas; a++) {
		std::vector<unsigned> tris;
		for (unsigned t = 0; t < nt; t++)
			if (a < natlas ? atlas[t] == (int)a : atlas[t] < 0) tris.push_back(t);
		for (unsigned t : tris) multi_of[t] = nmulti++;
		if (a == natlas && tris.empty()) break;
		const unsigned n = (unsigned)tris.size();
		RRMeshArrays* mesh = new RRMeshArrays();
		RRVector<unsigned> channels;
		channels.push_back(0);
		if (!mesh->resizeMesh(n, 3 * n, &channels, false, false)) { fprintf(stderr, "mesh\n"); return 3; }
		RRMaterial* mats = new RRMaterial[n ? n : 1];
		RRObject* object = new RRObject();
		for (unsigned k = 0; k < n; k++) {
			const unsigned t = tris[k];
			RRVec3 p[3];
			for (unsigned c = 0; c < 3; c++) {
				const unsigned v = idx[3 * t + c];
				p[c] = RRVec3(xyz[3 * v], xyz[3 * v + 1], xyz[3 * v + 2]);
			}
			RRVec3 nrm = (p[1] - p[0]).cross(p[2] - p[0]).normalized();
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
	solver->setStaticObjects(objects, nullptr, "/proc/no-collider-cache/", RRCollider::IT_BSP_FASTEST);
	RRLights lights;
	lights.push_back(RRLight::createDirectionalLight(RRVec3(L[0], L[1], L[2]), RRVec3(L[3], L[4], L[5]), true));
	lights.push_back(RRLight::createPointLight(RRVec3(L[6], L[7], L[8]), RRVec3(L[9], L[10], L[11])));
	solver->setLights(lights);
	const RRObject* multi = solver->getMultiObject();
	if (!multi || multi->getCollider()->getMesh()->getNumTriangles() != nt) {
		fprintf(stderr, "multi-object lost triangles\n");
		return 4;
	}
	// minimalSafeDistance as setStaticObjects computes it (RRSolver.cpp:329-334)
	RRVec3 mini, maxi, center;
	multi->getCollider()->getMesh()->getAABB(&mini, &maxi, &center);
	const float msd = (maxi - mini).avg() * 1e-6f;

	const bool bake = argc > 4 && !strcmp(argv[4], "bake");
	if (bake) {
		std::vector<RRBuffer*> bufs;
		for (unsigned o = 0; o < nout; o++) {
			const unsigned a = out_atlas[o];
			if (a >= natlas) { fprintf(stderr, "bad atlas\n"); return 6; }
			RRBuffer* b = RRBuffer::create(BT_2D_TEXTURE, size, size, 1, BF_RGBAF, false, nullptr);
			objects[a]->illumination.getLayer(0) = b;
			bufs.push_back(b);
		}
		RRSolver::UpdateParameters params(quality);
		RRSolver::FilteringParameters filtering;
		filtering.smoothingAmount = 0;
		filtering.spreadForegroundColor = 0;
		const unsigned updated = solver->updateLightmaps(0, -1, -1, &params, &filtering);
		if (updated != nout) { fprintf(stderr, "updated %u of %u\n", updated, nout); return 8; }
		FILE* f = fopen(argv[2], "wb");
		if (!f) return 5;
		fwrite("RGG1", 1, 4, f);
		fwrite(&nout, 4, 1, f);
		fwrite(&size, 4, 1, f);
		for (unsigned o = 0; o < nout; o++) {
			std::vector<float> px((size_t)size * size * 4);
			for (unsigned i = 0; i < size * size; i++) {
				RRVec4 e = bufs[o]->getElement(i, nullptr);
				for (int c = 0; c < 4; c++) px[4 * (size_t)i + c] = e[c];
			}
			fwrite(px.data(), sizeof(float), px.size(), f);
		}
		fclose(f);
		// the solver the final gather read, per triangle of ours: direct and
		// indirect irradiance (flat) and the smoothed indirect at each corner
		std::string sp = std::string(argv[2]) + ".solver";
		f = fopen(sp.c_str(), "wb");
		if (!f) return 5;
		fwrite("RGB1", 1, 4, f);
		fwrite(&nt, 4, 1, f);
		for (unsigned t = 0; t < nt; t++) {
			float rec[15];
			RRVec3 v;
			RRRadiometricMeasure md(0, 0, 0, 1, 0), mi(0, 0, 0, 0, 1);
			md.smoothed = 0;
			RRRadiometricMeasure mif = mi;
			mif.smoothed = 0;
			solver->getTriangleMeasure(multi_of[t], 3, md, v);
			for (int c = 0; c < 3; c++) rec[c] = v[c];
			solver->getTriangleMeasure(multi_of[t], 3, mif, v);
			for (int c = 0; c < 3; c++) rec[3 + c] = v[c];
			for (unsigned k = 0; k < 3; k++) {
				solver->getTriangleMeasure(multi_of[t], k, mi, v);
				for (int c = 0; c < 3; c++) rec[6 + 3 * k + c] = v[c];
			}
			fwrite(rec, sizeof(float), 15, f);
		}
		fclose(f);
		printf("ok bake\n");
		return 0;
	}

	RRSolver::UpdateParameters params(quality);
	params.useCurrentSolution = true;
	FILE* f = fopen(argv[2], "wb");
	if (!f) return 5;
	fwrite("RGG1", 1, 4, f);
	fwrite(&nout, 4, 1, f);
	fwrite(&size, 4, 1, f);
	for (unsigned o = 0; o < nout; o++) {
		const unsigned a = out_atlas[o];
		if (a >= natlas) { fprintf(stderr, "bad atlas\n"); return 6; }
		LightmapperJob job(solver, params);
		job.pixelBuffers[LS_LIGHTMAP] = RRBuffer::create(BT_2D_TEXTURE, size, size, 1, BF_RGBAF, false, nullptr);
		job.pixelBuffers[LS_LIGHTMAP]->clear();
		job.singleObjectReceiver = objects[a];
		job.gatherAllDirections = false;
		UnwrapStatistics us;
		if (!enumerateTexelsPartial(multi, a, size, size, 0, 0, size, size, processTexel, job, msd, us, -1)) {
			fprintf(stderr, "gather failed\n");
			return 7;
		}
		std::vector<float> px((size_t)size * size * 4);
		for (unsigned i = 0; i < size * size; i++) {
			RRVec4 e = job.pixelBuffers[LS_LIGHTMAP]->getElement(i, nullptr);
			for (int c = 0; c < 4; c++) px[4 * (size_t)i + c] = e[c];
		}
		fwrite(px.data(), sizeof(float), px.size(), f);
		delete job.pixelBuffers[LS_LIGHTMAP];
		printf("atlas %u texels %u\n", a, us.numTexelsProcessed);
	}
	fclose(f);
	printf("ok\n");
	return 0;
}
