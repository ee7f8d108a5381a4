// Runs the reference's texel enumeration (enumerateTexelsPartial,
// RRSolver/lightmap.cpp:83-404, built from the reference's own sources into
// oracle/_ref) on one unwrapped mesh and writes every texel's TexelFlags and
// sub-texels.  Test infrastructure only: the golden vectors of the GPU
// enumeration and of the oracle's restatement (oracle/rr_gather.c).
//
//   ref_enumerate UNWRAP SIZE OUT
//
// UNWRAP : "RGU1", u32 nv, u32 nt, f32 xyz[3nv], f32 normal[3nv],
//          u32 idx[3nt], f32 uv[6nt] (lightmap uv of each triangle corner)
// OUT    : "RGE1", u32 size, u32 total, u8 flags[size*size],
//          u32 count[size*size], then total records {u32 tri, f32 uv[6],
//          f32 area} texel by texel in the reference's order
//
// The enumeration is called the way updateLightmap calls it for one object
// (lightmap.cpp:823) but with no solver (it then takes the object as its own
// multi-object and processes every texel, lightmap.cpp:115,381) and a
// callback that records each texel instead of gathering it.
#include "Lightsprint/RRCollider.h"
#include "Lightsprint/RRMesh.h"
#include "Lightsprint/RRObject.h"
#include "RRSolver/gather.h"
#include <cstdio>
#include <cstdlib>
#include <cstring>
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

struct Rec {
	unsigned tri;
	float uv[6];
	float area;
};
static unsigned g_size = 0;
static std::vector<unsigned char> g_flags;
static std::vector<std::vector<Rec>> g_texels;

// Called from the enumeration's OpenMP loop, once per covered texel.
static ProcessTexelResult record(const ProcessTexelParams& p) {
	const unsigned k = p.uv[0] + p.uv[1] * g_size;
	g_flags[k] = p.subTexels->texelFlags;
	std::vector<Rec>& out = g_texels[k];
	for (TexelSubTexels::const_iterator i = p.subTexels->begin(); i != p.subTexels->end(); ++i) {
		Rec r;
		r.tri = i->multiObjPostImportTriIndex;
		for (int c = 0; c < 3; c++) {
			r.uv[2 * c] = i->uvInTriangleSpace[c][0];
			r.uv[2 * c + 1] = i->uvInTriangleSpace[c][1];
		}
		r.area = i->areaInMapSpace;
		out.push_back(r);
	}
	return ProcessTexelResult();
}

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
	if (argc != 4) {
		fprintf(stderr, "usage: ref_enumerate UNWRAP SIZE OUT\n");
		return 2;
	}
	std::vector<char> mb;
	if (!readFile(argv[1], mb) || memcmp(mb.data(), "RGU1", 4)) { fprintf(stderr, "bad mesh\n"); return 2; }
	unsigned nv, nt;
	memcpy(&nv, mb.data() + 4, 4);
	memcpy(&nt, mb.data() + 8, 4);
	const float* xyz = (const float*)(mb.data() + 12);
	const float* nrm = xyz + 3 * (size_t)nv;
	const unsigned* idx = (const unsigned*)(nrm + 3 * (size_t)nv);
	const float* uv = (const float*)(idx + 3 * (size_t)nt);
	g_size = (unsigned)atoi(argv[2]);
	g_flags.assign((size_t)g_size * g_size, 0);
	g_texels.assign((size_t)g_size * g_size, std::vector<Rec>());

	RRMeshArrays* mesh = new RRMeshArrays();
	RRVector<unsigned> channels;
	channels.push_back(0);
	if (!mesh->resizeMesh(nt, 3 * nt, &channels, false, false)) { fprintf(stderr, "mesh\n"); return 3; }
	for (unsigned t = 0; t < nt; t++)
		for (unsigned c = 0; c < 3; c++) {
			const unsigned v = idx[3 * t + c], k = 3 * t + c;
			mesh->triangle[t][c] = k;
			mesh->position[k] = RRVec3(xyz[3 * v], xyz[3 * v + 1], xyz[3 * v + 2]);
			mesh->normal[k] = RRVec3(nrm[3 * v], nrm[3 * v + 1], nrm[3 * v + 2]);
			mesh->texcoord[0][k] = RRVec2(uv[6 * t + 2 * c], uv[6 * t + 2 * c + 1]);
		}
	bool aborting = false;
	RRCollider* collider = RRCollider::create(mesh, nullptr, RRCollider::IT_LINEAR, aborting);
	RRMaterial material;
	material.reset(false);
	material.lightmap.texcoord = 0;
	RRObject* object = new RRObject();
	object->faceGroups.push_back(RRObject::FaceGroup(&material, nt));
	object->setCollider(collider);

	RRSolver::UpdateParameters params;
	LightmapperJob job(nullptr, params);
	UnwrapStatistics us;
	if (!enumerateTexelsPartial(object, 0, g_size, g_size, 0, 0, g_size, g_size, record, job, 0.f, us, -1)) {
		fprintf(stderr, "enumeration failed\n");
		return 4;
	}
	FILE* f = fopen(argv[3], "wb");
	if (!f) return 5;
	unsigned total = 0;
	for (auto& v : g_texels) total += (unsigned)v.size();
	fwrite("RGE1", 1, 4, f);
	fwrite(&g_size, 4, 1, f);
	fwrite(&total, 4, 1, f);
	fwrite(g_flags.data(), 1, g_flags.size(), f);
	for (auto& v : g_texels) {
		unsigned c = (unsigned)v.size();
		fwrite(&c, 4, 1, f);
	}
	for (auto& v : g_texels)
		if (!v.empty()) fwrite(v.data(), sizeof(Rec), v.size(), f);
	fclose(f);
	printf("ok %u\n", total);
	return 0;
}
