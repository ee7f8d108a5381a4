/* rr_filter.c -- ORACLE (test infrastructure only): CPU restatement of the
 * lightmap post-filters that RRSolver::updateLightmap runs on each gathered
 * lightmap (RRSolver/lightmap.cpp:865-874), and of the unwrap-seam search
 * that lightmapSmooth uses.  Only tests/, the smoke check and the bench's
 * CPU leg call it.  Single-threaded, in the reference's loop order, float
 * arithmetic with one rounding per operation (built -ffp-contract=off).
 *
 *   orc_unwrap_seams     UnwrapSeams (RRBuffer/RRBuffer.cpp:534-628), with
 *                        vertices shared by index (see below)
 *   orc_lightmap_smooth  RRBuffer::lightmapSmooth (RRBuffer.cpp:630-802)
 *   orc_lightmap_grow_bilinear
 *                        RRBuffer::lightmapGrowForBilinearInterpolation
 *                        (RRBuffer.cpp:804-863)
 *   orc_lightmap_grow    RRBuffer::lightmapGrow (RRBuffer.cpp:865-962)
 *   orc_lightmap_fill_background
 *                        RRBuffer::lightmapFillBackground (RRBuffer.cpp:964-983)
 *
 * Pinned bit-exact against the reference's own functions, run from its
 * sources (oracle/ref_filter.cpp, tests/golden/lightmap_ref.npz).
 *
 * A lightmap is width*height RGBA floats, texel (i, j) at i + j*width, alpha
 * = TexelFlags/255 where the gather covered the texel (gather.cpp:801).
 *
 * Seams: the reference first stitches vertices of equal position whose
 * normals differ by at most 1 degree (createOptimizedVertices(0, 1deg, 0),
 * RRBuffer.cpp:558) and then looks for edges shared by two triangles whose
 * unwrap differs.  Here two triangles share a vertex when they share its
 * index; for a mesh that keeps one vertex per position (as the stitch leaves
 * it) both find the same edges, in the same order. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "rr_gather.h"

typedef struct { float x, y, z, w; } v4;

static v4 v4mk(float x, float y, float z, float w) { v4 r = {x, y, z, w}; return r; }
static v4 v4add(v4 a, v4 b) { return v4mk(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
static v4 v4mul(v4 a, float f) { return v4mk(a.x * f, a.y * f, a.z * f, a.w * f); }
static v4 v4div(v4 a, float f) { return v4mk(a.x / f, a.y / f, a.z / f, a.w / f); }
static v4 ld4(const float* p) { return v4mk(p[0], p[1], p[2], p[3]); }
static void st4(float* p, v4 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; p[3] = v.w; }

/* FLOAT_TO_TEXELFLAGS (RRSolver/gather.h:79) */
static unsigned texel_flags(float a) { return (unsigned)(a * 255 + 0.5f); }

enum { Q_X0Y0 = 1, Q_X1Y0 = 2, Q_X0Y1 = 4, Q_X1Y1 = 8, E_X0 = 16, E_X1 = 32, E_Y0 = 64, E_Y1 = 128 };

/* ------------------------------------------------------------------ seams */
uint32_t orc_unwrap_seams(const uint32_t* idx, const float* uv, uint32_t n, float* seams, uint32_t cap) {
	/* idx: 3 vertex indices per triangle, uv: 6 floats per triangle (map space),
	 * both in the object's triangle order.  seams: 8 floats per seam
	 * (edge1[0], edge1[1], edge2[0], edge2[1]); returns the number found
	 * (writes at most cap). */
	uint32_t maxv = 0;
	for (uint32_t k = 0; k < 3 * n; k++)
		if (idx[k] + 1 > maxv) maxv = idx[k] + 1;
	uint32_t* cnt = (uint32_t*)calloc((size_t)maxv + 1, sizeof(uint32_t));
	uint32_t* tiv = (uint32_t*)malloc(sizeof(uint32_t) * (3 * (size_t)n + 1));
	uint32_t* fill = (uint32_t*)calloc((size_t)maxv + 1, sizeof(uint32_t));
	for (uint32_t k = 0; k < 3 * n; k++) cnt[idx[k] + 1]++;
	for (uint32_t v = 0; v < maxv; v++) cnt[v + 1] += cnt[v];
	/* trianglesInVertex, each list in ascending triangle order */
	for (uint32_t t = 0; t < n; t++)
		for (int v = 0; v < 3; v++) {
			uint32_t vi = idx[3 * (size_t)t + v];
			tiv[cnt[vi] + fill[vi]++] = t;
		}
	uint32_t found = 0;
	for (uint32_t t1 = 0; t1 < n; t1++) {
		const uint32_t* tv1 = idx + 3 * (size_t)t1;
		for (unsigned e = 0; e < 3; e++) {
			uint32_t v1 = tv1[e], v2 = tv1[(e + 1) % 3];
			const float* a0 = uv + 6 * (size_t)t1 + 2 * e;
			const float* a1 = uv + 6 * (size_t)t1 + 2 * ((e + 1) % 3);
			const uint32_t* l1 = tiv + cnt[v1];
			const uint32_t n1 = cnt[v1 + 1] - cnt[v1];
			const uint32_t* l2 = tiv + cnt[v2];
			const uint32_t n2 = cnt[v2 + 1] - cnt[v2];
			uint32_t i1 = 0;
			for (uint32_t i2 = 0; i2 < n2; i2++)
				if (l2[i2] > t1) {
					while (i1 + 1 < n1 && l1[i1] < l2[i2]) i1++;
					if (l1[i1] == l2[i2]) {
						uint32_t t2 = l2[i2];
						const uint32_t* tv2 = idx + 3 * (size_t)t2;
						unsigned c1 = (tv2[0] == v1) ? 0 : ((tv2[1] == v1) ? 1 : 2);
						unsigned c2 = (tv2[0] == v2) ? 0 : ((tv2[1] == v2) ? 1 : 2);
						const float* b0 = uv + 6 * (size_t)t2 + 2 * c1;
						const float* b1 = uv + 6 * (size_t)t2 + 2 * c2;
						if (a0[0] != b0[0] || a0[1] != b0[1] || a1[0] != b1[0] || a1[1] != b1[1]) {
							if (found < cap) {
								float* s = seams + 8 * (size_t)found;
								s[0] = a0[0]; s[1] = a0[1]; s[2] = a1[0]; s[3] = a1[1];
								s[4] = b0[0]; s[5] = b0[1]; s[6] = b1[0]; s[7] = b1[1];
							}
							found++;
						}
					}
				}
		}
	}
	free(cnt);
	free(tiv);
	free(fill);
	return found;
}

/* ------------------------------------------------------------------ smooth */
/* One pass over the seams (RRBuffer.cpp:744-786): along both edges of a seam,
 * 1001 samples; each run of samples in one texel averages the two edges'
 * texels and, when the run ends, overwrites its texel. */
static void smooth_seams(v4* dst, uint32_t width, uint32_t height, const float* seams, uint32_t nseams) {
	for (uint32_t s = 0; s < nseams; s++) {
		const float* sm = seams + 8 * (size_t)s;
		uint32_t last1 = UINT32_MAX, last2 = UINT32_MAX;
		v4 acc1 = v4mk(0, 0, 0, 0), acc2 = v4mk(0, 0, 0, 0);
		for (unsigned i = 0; i <= 1000; i++) {
			float b = (float)i * 0.001f, a = 1 - b;
			float u1x = sm[0] * a + sm[2] * b, u1y = sm[1] * a + sm[3] * b;
			float u2x = sm[4] * a + sm[6] * b, u2y = sm[5] * a + sm[7] * b;
			if (!(u1x >= 0 && u1x < 1 && u1y >= 0 && u1y < 1)) continue;
			if (!(u2x >= 0 && u2x < 1 && u2y >= 0 && u2y < 1)) continue;
			uint32_t i1 = (unsigned)(u1x * (float)width) + (unsigned)(u1y * (float)height) * width;
			uint32_t i2 = (unsigned)(u2x * (float)width) + (unsigned)(u2y * (float)height) * width;
			if (!(dst[i1].w != 0 && dst[i2].w != 0)) continue;
			if (i1 != last1) {
				if (last1 != UINT32_MAX) dst[last1] = v4div(acc1, acc1.w);
				last1 = i1;
				acc1 = v4mk(0, 0, 0, 0);
			}
			if (i2 != last2) {
				if (last2 != UINT32_MAX) dst[last2] = v4div(acc2, acc2.w);
				last2 = i2;
				acc2 = v4mk(0, 0, 0, 0);
			}
			acc1 = v4add(acc1, v4add(dst[i1], dst[i2]));
			acc2 = v4add(acc2, v4add(dst[i1], dst[i2]));
		}
		if (last1 != UINT32_MAX) dst[last1] = v4div(acc1, acc1.w);
		if (last2 != UINT32_MAX) dst[last2] = v4div(acc2, acc2.w);
	}
}

/* Blur-flag bits of texel (i, j): which of the 8 neighbours it may blur with
 * (RRBuffer.cpp:665-699).  Bit order: (-1,-1) (0,-1) (1,-1) (-1,0) (1,0)
 * (-1,1) (0,1) (1,1). */
static unsigned blur_bits(const v4* src, uint32_t width, uint32_t height, int wrap, int i, int j) {
	unsigned center = texel_flags(src[i + j * width].w);
	unsigned bit = 1, bits = 0;
	for (int jj = -1; jj < 2; jj++)
		for (int ii = -1; ii < 2; ii++)
			if (ii || jj) {
				int x = i + ii, y = j + jj;
				if (wrap) {
					x = (int)(((unsigned)x + width) % width);
					y = (int)(((unsigned)y + height) % height);
				}
				if (x >= 0 && x < (int)width && y >= 0 && y < (int)height) {
					unsigned nb = texel_flags(src[x + y * width].w);
					if ((ii >= 0 || ((center & E_X0) && (nb & E_X1))) && (ii <= 0 || ((center & E_X1) && (nb & E_X0))) &&
					    (jj >= 0 || ((center & E_Y0) && (nb & E_Y1))) && (jj <= 0 || ((center & E_Y1) && (nb & E_Y0))))
						bits |= bit;
				}
				bit *= 2;
			}
	return bits;
}

int orc_lightmap_smooth(float* rgba, uint32_t width, uint32_t height, float sigma, int wrap, const float* seams,
                        uint32_t nseams) {
	if (sigma < 0) return 0;
	if (sigma == 0) return 1;
	const size_t size = (size_t)width * height;
	v4* src = (v4*)malloc(sizeof(v4) * size);
	v4* dst = (v4*)malloc(sizeof(v4) * size);
	unsigned char* bf = (unsigned char*)malloc(size);
	for (size_t k = 0; k < size; k++) src[k] = ld4(rgba + 4 * k);
	for (uint32_t j = 0; j < height; j++)
		for (uint32_t i = 0; i < width; i++) bf[i + j * width] = (unsigned char)blur_bits(src, width, height, wrap, (int)i, (int)j);
	for (size_t k = 0; k < size; k++) src[k].w = src[k].w > 0 ? 1.f : 0.f;
	if (sigma > 10) sigma = 10;
	float sum = sigma * sigma;
	while (sum > 0) {
		float s2 = sum < 0.34f ? sum : 0.34f;
		float k0 = 1, k1 = expf(-0.5f / s2), k2 = expf(-1 / s2);
		sum -= s2;
		for (uint32_t j = 0; j < height; j++)
			for (uint32_t i = 0; i < width; i++) {
				uint32_t k = i + j * width;
				v4 c = src[k];
				if (c.w != 0) {
					unsigned f = bf[k];
					uint32_t im = (i - 1 + width) % width, ip = (i + 1) % width;
					uint32_t jm = (j - 1 + height) % height, jp = (j + 1) % height;
					c = v4mul(c, k0);
					c = v4add(c, v4mul(src[im + jm * width], (f & 1) ? k2 : 0));
					c = v4add(c, v4mul(src[i + jm * width], (f & 2) ? k1 : 0));
					c = v4add(c, v4mul(src[ip + jm * width], (f & 4) ? k2 : 0));
					c = v4add(c, v4mul(src[im + j * width], (f & 8) ? k1 : 0));
					c = v4add(c, v4mul(src[ip + j * width], (f & 16) ? k1 : 0));
					c = v4add(c, v4mul(src[im + jp * width], (f & 32) ? k2 : 0));
					c = v4add(c, v4mul(src[i + jp * width], (f & 64) ? k1 : 0));
					c = v4add(c, v4mul(src[ip + jp * width], (f & 128) ? k2 : 0));
					c = v4div(c, c.w);
				}
				dst[k] = c;
			}
		smooth_seams(dst, width, height, seams, nseams);
		v4* t = src;
		src = dst;
		dst = t;
	}
	for (size_t k = 0; k < size; k++)
		if (src[k].w > 0) {
			rgba[4 * k] = src[k].x;
			rgba[4 * k + 1] = src[k].y;
			rgba[4 * k + 2] = src[k].z;
		}
	free(src);
	free(dst);
	free(bf);
	return 1;
}

/* ------------------------------------------------------------------- grow */
int orc_lightmap_grow_bilinear(float* rgba, uint32_t width, uint32_t height, int wrap) {
	/* in place, in the reference's scan order: a texel written here gets
	 * alpha 0.001, whose flags are 0, so it never counts as a good neighbour */
	int not_empty = 0;
	for (uint32_t j = 0; j < height; j++)
		for (uint32_t i = 0; i < width; i++) {
			if (rgba[4 * ((size_t)i + (size_t)j * width) + 3] > 0.002f) {
				not_empty = 1;
				continue;
			}
			v4 sum = v4mk(0, 0, 0, 0);
			for (int jj = -1; jj < 2; jj++)
				for (int ii = -1; ii < 2; ii++) {
					int x = (int)i + ii, y = (int)j + jj;
					if (wrap) {
						x = (int)(((unsigned)x + width) % width);
						y = (int)(((unsigned)y + height) % height);
					} else if (x < 0 || x >= (int)width || y < 0 || y >= (int)height)
						continue;
					v4 c = ld4(rgba + 4 * ((size_t)x + (size_t)y * width));
					unsigned f = texel_flags(c.w);
					if ((ii < 1 && jj < 1 && (f & Q_X1Y1)) || (ii > -1 && jj > -1 && (f & Q_X0Y0)) ||
					    (ii < 1 && jj > -1 && (f & Q_X1Y0)) || (ii > -1 && jj < 1 && (f & Q_X0Y1))) {
						float wgt = (ii && jj) ? 1 : 1.6f;
						sum = v4add(sum, v4mul(v4mk(c.x, c.y, c.z, 1), wgt));
					}
				}
			if (sum.w != 0)
				st4(rgba + 4 * ((size_t)i + (size_t)j * width), v4mk(sum.x / sum.w, sum.y / sum.w, sum.z / sum.w, 0.001f));
		}
	return not_empty;
}

int orc_lightmap_grow(float* rgba, uint32_t width, uint32_t height, uint32_t steps, int wrap) {
	if (steps == 0) return 1;
	const uint32_t size = width * height;
	v4* src = (v4*)malloc(sizeof(v4) * size);
	v4* dst = (v4*)malloc(sizeof(v4) * size);
	for (uint32_t k = 0; k < size; k++) {
		v4 c = ld4(rgba + 4 * (size_t)k);
		src[k] = c.w > 0 ? v4mk(c.x, c.y, c.z, 1) : v4mk(0, 0, 0, 0);
	}
	while (steps--) {
		int changed = 0;
		for (uint32_t k = 0; k < size; k++) {
			v4 c = src[k];
			if (c.w == 0) {
				v4 d;
				if (wrap) {
					/* unsigned index arithmetic modulo the texel count, as the
					 * reference's int-with-unsigned expressions do */
					const int i = (int)k, w = (int)width;
					v4 s4 = v4add(v4add(v4add(src[(unsigned)(i + 1) % size], src[(unsigned)(i - 1) % size]),
					                    src[(unsigned)(i + w) % size]), src[(unsigned)(i - w) % size]);
					v4 s8 = v4add(v4add(v4add(src[(unsigned)(i + 1 + w) % size], src[(unsigned)(i + 1 - w) % size]),
					                    src[(unsigned)(i - 1 + w) % size]), src[(unsigned)(i - 1 - w) % size]);
					d = v4add(v4mul(s4, 1.6f), s8);
				} else {
					int x = (int)(k % width), y = (int)(k / width), w = (int)width, h = (int)height;
					int xp = x + 1 < w - 1 ? x + 1 : w - 1, xm = x - 1 > 0 ? x - 1 : 0;
					int yp = y + 1 < h - 1 ? y + 1 : h - 1, ym = y - 1 > 0 ? y - 1 : 0;
					v4 s4 = v4add(v4add(v4add(src[xp + y * w], src[xm + y * w]), src[x + yp * w]), src[x + ym * w]);
					v4 s8 = v4add(v4add(v4add(src[xp + yp * w], src[xp + ym * w]), src[xm + yp * w]), src[xm + ym * w]);
					d = v4add(v4mul(s4, 1.6f), s8);
				}
				if (d.w != 0) {
					c = v4div(d, d.w);
					changed = 1;
				}
			}
			dst[k] = c;
		}
		if (!changed) steps = 0;
		v4* t = src;
		src = dst;
		dst = t;
	}
	for (uint32_t k = 0; k < size; k++)
		if (src[k].w > 0 && rgba[4 * (size_t)k + 3] == 0) st4(rgba + 4 * (size_t)k, v4mk(src[k].x, src[k].y, src[k].z, 0.001f));
	free(src);
	free(dst);
	return 1;
}

void orc_lightmap_fill_background(float* rgba, uint32_t width, uint32_t height, const float* background) {
	for (size_t k = 0; k < (size_t)width * height; k++)
		if (rgba[4 * k + 3] <= 0) memcpy(rgba + 4 * k, background, 4 * sizeof(float));
}
