// Runs the reference's lightmap post-filters (built from the reference's own
// sources into oracle/_ref) on one RGBA float lightmap and writes the result.
// Test infrastructure only: it produces the golden vectors that the filter
// oracle (oracle/rr_filter.c) and the GPU filters are checked against.
//
//   ref_filter IN OUT SIGMA WRAP SPREAD STAGES [MESH]
//
// IN, OUT : "RGL1", u32 width, u32 height, f32 rgba[width*height*4]
// STAGES  : bit mask, 1 lightmapSmooth, 2 lightmapGrowForBilinearInterpolation,
//           4 lightmapGrow, 8 lightmapFillBackground (background 0), run in
//           the order of RRSolver::updateLightmap (RRSolver/lightmap.cpp:865-874)
// MESH    : optional "RGU1", u32 nv, u32 nt, f32 xyz[3nv], f32 normal[3nv],
//           u32 idx[3nt], f32 uv[6nt] (lightmap uv of each triangle corner).
//           With it lightmapSmooth is given an object, so it also averages
//           across unwrap seams (RRBuffer.cpp:534-628,744-786).  The object's
//           mesh has one vertex per triangle corner, each with its source
//           vertex's position and normal, as an unwrapped mesh is stored
//           (RRMeshArrays keeps uv per vertex); the reference's seam search
//           stitches them back (createOptimizedVertices(0, 1 degree, 0)).
#include "Lightsprint/RRBuffer.h"
#include "Lightsprint/RRCollider.h"
#include "Lightsprint/RRMesh.h"
#include "Lightsprint/RRObject.h"
#include <cstdio>
#include <cstdlib>
#include <cstring>
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

// The object given to lightmapSmooth: one vertex per triangle corner.
static RRMeshArrays* unwrapped_mesh(const std::vector<char>& mb, unsigned& nt) {
	unsigned nv;
	memcpy(&nv, mb.data() + 4, 4);
	memcpy(&nt, mb.data() + 8, 4);
	const float* xyz = (const float*)(mb.data() + 12);
	const float* nrm = xyz + 3 * (size_t)nv;
	const unsigned* idx = (const unsigned*)(nrm + 3 * (size_t)nv);
	const float* uv = (const float*)(idx + 3 * (size_t)nt);
	RRMeshArrays* mesh = new RRMeshArrays();
	RRVector<unsigned> channels;
	channels.push_back(0);
	if (!mesh->resizeMesh(nt, 3 * nt, &channels, false, false)) return nullptr;
	for (unsigned t = 0; t < nt; t++)
		for (unsigned c = 0; c < 3; c++) {
			const unsigned v = idx[3 * t + c], k = 3 * t + c;
			mesh->triangle[t][c] = k;
			mesh->position[k] = RRVec3(xyz[3 * v], xyz[3 * v + 1], xyz[3 * v + 2]);
			mesh->normal[k] = RRVec3(nrm[3 * v], nrm[3 * v + 1], nrm[3 * v + 2]);
			mesh->texcoord[0][k] = RRVec2(uv[6 * t + 2 * c], uv[6 * t + 2 * c + 1]);
		}
	return mesh;
}

int main(int argc, char** argv) {
	if (argc < 7) {
		fprintf(stderr, "usage: ref_filter IN OUT SIGMA WRAP SPREAD STAGES [MESH]\n");
		return 2;
	}
	std::vector<char> ib;
	if (!readFile(argv[1], ib) || ib.size() < 12 || memcmp(ib.data(), "RGL1", 4)) { fprintf(stderr, "bad image\n"); return 2; }
	unsigned w, h;
	memcpy(&w, ib.data() + 4, 4);
	memcpy(&h, ib.data() + 8, 4);
	if (ib.size() != 12 + 16 * (size_t)w * h) { fprintf(stderr, "bad image size\n"); return 2; }
	const float sigma = (float)atof(argv[3]);
	const bool wrap = atoi(argv[4]) != 0;
	const unsigned spread = (unsigned)atoi(argv[5]);
	const unsigned stages = (unsigned)atoi(argv[6]);

	RRBuffer* buf = RRBuffer::create(BT_2D_TEXTURE, w, h, 1, BF_RGBAF, false, (const unsigned char*)(ib.data() + 12));
	if (!buf) { fprintf(stderr, "buffer\n"); return 3; }

	RRMeshArrays* mesh = nullptr;
	RRCollider* collider = nullptr;
	RRObject* object = nullptr;
	RRMaterial material;
	if (argc > 7) {
		std::vector<char> mb;
		if (!readFile(argv[7], mb) || memcmp(mb.data(), "RGU1", 4)) { fprintf(stderr, "bad mesh\n"); return 2; }
		unsigned nt = 0;
		mesh = unwrapped_mesh(mb, nt);
		if (!mesh) { fprintf(stderr, "mesh\n"); return 3; }
		bool aborting = false;
		collider = RRCollider::create(mesh, nullptr, RRCollider::IT_LINEAR, aborting);
		material.reset(false);
		material.lightmap.texcoord = 0;
		object = new RRObject();
		object->faceGroups.push_back(RRObject::FaceGroup(&material, nt));
		object->setCollider(collider);
	}

	bool aborting = false;
	if (stages & 1) buf->lightmapSmooth(sigma, wrap, object);
	if (stages & 2) buf->lightmapGrowForBilinearInterpolation(wrap);
	if (stages & 4) buf->lightmapGrow(spread, wrap, aborting);
	if (stages & 8) buf->lightmapFillBackground(RRVec4(0));

	FILE* f = fopen(argv[2], "wb");
	if (!f) return 4;
	fwrite("RGL1", 1, 4, f);
	fwrite(&w, 4, 1, f);
	fwrite(&h, 4, 1, f);
	for (unsigned i = 0; i < w * h; i++) {
		RRVec4 c = buf->getElement(i, nullptr);
		fwrite(&c, 4, 4, f);
	}
	fclose(f);
	printf("ok\n");
	delete object;
	delete collider;
	delete mesh;
	delete buf;
	return 0;
}
