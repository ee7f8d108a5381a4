/* ORACLE: double-precision restatement of the radiance-cache network (the
 * learned part of the gather, which has no counterpart in the reference).
 * Test infrastructure only: the GPU's BF16 tensor-core forward and backward
 * kernels are checked against it.
 *
 * Network (shared with lightsprintsdk_gb300/csrc/rrg_mlp.cu):
 *   x  = encode(p, n, albedo)            64 features
 *   h1 = relu(x  W1)  h2 = relu(h1 W2)  h3 = relu(h2 W3)  h4 = relu(h3 W4)
 *   y  = h4 W5                           16 outputs, the first 3 = RGB
 *   W1..W4: 64 x 64, W5: 64 x 16, row = input feature, column = output;
 *   parameters stored layer after layer, row-major (17,408 floats).
 * Encoding: u = clamp((p - lo) / (hi - lo), 0, 1); for axis j, frequency k
 *   (0..7): x[16j + 2k] = sin(2^k pi u_j), x[16j + 2k + 1] = cos(2^k pi u_j);
 *   x[48..50] = n, x[51..53] = albedo, x[54] = 1, x[55..63] = 0.
 * Loss (relative L2 of neural radiance caching, Mueller et al. 2021):
 *   L = (1/B) sum_i sum_{c<3} (y_ic - t_ic)^2 / (y_ic^2 + 0.01), the
 *   denominator held constant for the gradient:
 *   dL/dy_ic = 2 (y_ic - t_ic) / (y_ic^2 + 0.01) / B.
 * With bf16 = 1 the oracle rounds to bfloat16 where the GPU does (inputs,
 * weights, post-activation values, output gradients and back-propagated
 * deltas), so only the accumulation order differs. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define NIN 64
#define NH 64
#define NOUT 16
#define NPARAM (4 * 64 * 64 + 64 * 16)

static const double kPi = 3.14159265358979323846;

double orc_bf16(double x) {
	float f = (float)x;
	uint32_t u;
	memcpy(&u, &f, 4);
	if ((u & 0x7F800000u) == 0x7F800000u) return f;    /* inf / nan unchanged */
	uint32_t r = 0x7FFFu + ((u >> 16) & 1u);            /* round to nearest even */
	u = (u + r) & 0xFFFF0000u;
	memcpy(&f, &u, 4);
	return f;
}

void orc_mlp_encode(const float* p, const float* n, const float* alb, const float* lo, const float* hi,
                    double* x) {
	for (int j = 0; j < 3; j++) {
		double u = ((double)p[j] - lo[j]) / ((double)hi[j] - lo[j]);
		if (u < 0) u = 0;
		if (u > 1) u = 1;
		for (int k = 0; k < 8; k++) {
			double f = (double)(1 << k) * kPi * u;
			x[16 * j + 2 * k] = sin(f);
			x[16 * j + 2 * k + 1] = cos(f);
		}
	}
	for (int j = 0; j < 3; j++) {
		x[48 + j] = n[j];
		x[51 + j] = alb[j];
	}
	x[54] = 1;
	for (int j = 55; j < 64; j++) x[j] = 0;
}

static const int kLayerIn[5] = {64, 64, 64, 64, 64};
static const int kLayerOut[5] = {64, 64, 64, 64, 16};
static int layer_off(int l) { return l * 4096; }

/* Forward and backward over B samples.  W: NPARAM floats.  X: B x 64
 * encoded inputs (float).  T: B x 3 targets.  dW (NPARAM doubles, zeroed
 * here) receives the gradient of the mean loss; *loss the mean loss; Y
 * (B x 3, may be NULL) the outputs. */
void orc_mlp_grad(const float* W, const float* X, const float* T, int B, int bf16, double* dW, double* loss,
                  float* Y) {
	double* w = (double*)malloc(sizeof(double) * NPARAM);
	for (int i = 0; i < NPARAM; i++) w[i] = bf16 ? orc_bf16(W[i]) : W[i];
	memset(dW, 0, sizeof(double) * NPARAM);
	double L = 0;
	double act[5][64], z[5][64], d[5][64], dn[64];
	for (int b = 0; b < B; b++) {
		for (int i = 0; i < 64; i++) act[0][i] = bf16 ? orc_bf16(X[64 * b + i]) : X[64 * b + i];
		double y[16];
		for (int l = 0; l < 5; l++) {
			const double* in = act[l];
			int no = kLayerOut[l];
			for (int o = 0; o < no; o++) {
				double s = 0;
				for (int i = 0; i < kLayerIn[l]; i++) s += in[i] * w[layer_off(l) + i * no + o];
				z[l][o] = s;
			}
			if (l < 4)
				for (int o = 0; o < 64; o++) {
					double h = z[l][o] > 0 ? z[l][o] : 0;
					act[l + 1][o] = bf16 ? orc_bf16(h) : h;
				}
			else
				for (int o = 0; o < 16; o++) y[o] = z[l][o];
		}
		double dy[16];
		for (int c = 0; c < 16; c++) dy[c] = 0;
		for (int c = 0; c < 3; c++) {
			double t = T[3 * b + c];
			double den = y[c] * y[c] + 0.01;
			L += (y[c] - t) * (y[c] - t) / den / B;
			dy[c] = 2 * (y[c] - t) / den / B;
			if (Y) Y[3 * b + c] = (float)y[c];
		}
		for (int c = 0; c < 16; c++) d[4][c] = bf16 ? orc_bf16(dy[c]) : dy[c];
		for (int l = 4; l >= 0; l--) {
			int ni = kLayerIn[l], no = kLayerOut[l];
			for (int i = 0; i < ni; i++)
				for (int o = 0; o < no; o++) dW[layer_off(l) + i * no + o] += act[l][i] * d[l][o];
			if (l == 0) break;
			for (int i = 0; i < ni; i++) {
				double s = 0;
				for (int o = 0; o < no; o++) s += d[l][o] * w[layer_off(l) + i * no + o];
				dn[i] = (act[l][i] > 0) ? s : 0;   /* relu'(z) = [h > 0] */
			}
			for (int i = 0; i < ni; i++) d[l - 1][i] = bf16 ? orc_bf16(dn[i]) : dn[i];
		}
	}
	*loss = L;
	free(w);
}

/* ---------------------------------------------------------------- hash grid
 * Encoding 1 ("hash grid", a multiresolution hash encoding after Mueller,
 * Evans, Schied, Keller, "Instant Neural Graphics Primitives with a
 * Multiresolution Hash Encoding", SIGGRAPH 2022):
 *   u = clamp((p - lo) * ie, 0, 1) in float (ie = 1 / (hi - lo), float);
 *   for level l (0..15) with resolution N_l (an integer, res[l]):
 *     x = u N_l (float), x0 = clamp(floor(x), 0, N_l - 1), w = x - x0;
 *     corner c = (x0 + cx, y0 + cy, z0 + cz), weight prod of (c ? w : 1 - w);
 *     index = dense (ix + iy (N+1) + iz (N+1)^2) when (N+1)^3 <= T, else
 *     (ix ^ iy 2654435761 ^ iz 805459861) mod T (uint32 arithmetic);
 *     x[2l + k] = sum_c weight_c table[(l T + index_c) 2 + k], k = 0, 1;
 *   x[32 + 8j + 2k] = sin(2^k pi u_j), x[32 + 8j + 2k + 1] = cos(2^k pi u_j)
 *     for axis j, k = 0..3;
 *   x[56..58] = n, x[59..61] = albedo, x[62] = 1, x[63] = 0.
 * The table is trained with the network: dL/dtable is the input gradient
 * dL/dx[2l + k] = sum_o d1[o] W1[2l + k][o] scattered to the 8 corners with
 * their weights. */
static uint32_t hg_index(int l, const int* res, uint32_t T, uint32_t ix, uint32_t iy, uint32_t iz) {
	const uint64_t n1 = (uint64_t)res[l] + 1;
	if (n1 * n1 * n1 <= T) return (uint32_t)(ix + iy * n1 + iz * n1 * n1);
	return (ix ^ (iy * 2654435761u) ^ (iz * 805459861u)) & (T - 1u);
}

/* Corner indices (within level l's T entries) and weights of one sample. */
static void hg_corners(const float* p, const float* lo, const float* ie, const int* res, uint32_t T, int l,
                       uint32_t* idx, float* wt) {
	float u[3], w[3];
	uint32_t x0[3];
	for (int j = 0; j < 3; j++) {
		float v = (p[j] - lo[j]) * ie[j];
		u[j] = v < 0.f ? 0.f : (v > 1.f ? 1.f : v);
		float x = u[j] * (float)res[l];
		int f = (int)floorf(x);
		if (f < 0) f = 0;
		if (f > res[l] - 1) f = res[l] - 1;
		x0[j] = (uint32_t)f;
		w[j] = x - (float)f;
	}
	for (int c = 0; c < 8; c++) {
		const int cx = c & 1, cy = (c >> 1) & 1, cz = (c >> 2) & 1;
		idx[c] = hg_index(l, res, T, x0[0] + cx, x0[1] + cy, x0[2] + cz);
		wt[c] = ((cx ? w[0] : 1.f - w[0]) * (cy ? w[1] : 1.f - w[1])) * (cz ? w[2] : 1.f - w[2]);
	}
}

void orc_mlp_encode_hash(const float* p, const float* n, const float* alb, const float* lo, const float* ie,
                         const float* table, const int* res, uint32_t T, double* x) {
	for (int l = 0; l < 16; l++) {
		uint32_t idx[8];
		float wt[8];
		hg_corners(p, lo, ie, res, T, l, idx, wt);
		for (int k = 0; k < 2; k++) {
			double s = 0;
			for (int c = 0; c < 8; c++) s += (double)wt[c] * table[((size_t)l * T + idx[c]) * 2 + k];
			x[2 * l + k] = s;
		}
	}
	for (int j = 0; j < 3; j++) {
		float v = (p[j] - lo[j]) * ie[j];
		double u = v < 0.f ? 0.f : (v > 1.f ? 1.f : v);
		for (int k = 0; k < 4; k++) {
			double f = (double)(1 << k) * kPi * u;
			x[32 + 8 * j + 2 * k] = sin(f);
			x[32 + 8 * j + 2 * k + 1] = cos(f);
		}
	}
	for (int j = 0; j < 3; j++) {
		x[56 + j] = n[j];
		x[59 + j] = alb[j];
	}
	x[62] = 1;
	x[63] = 0;
}

/* orc_mlp_grad with the hash-grid encoding computed here from the records
 * (P, N, A: B x 3 floats; T3: B x 3 targets): dW as orc_mlp_grad, and
 * dTable (levels x T x 2 doubles, zeroed here) the table gradient; Y (B x 3
 * doubles, may be NULL) the outputs.  With
 * bf16 the encoded inputs, weights and deltas are rounded as on the GPU. */
void orc_mlp_grad_hash(const float* W, const float* table, const int* res, uint32_t T, const float* lo,
                       const float* ie, const float* P, const float* N, const float* A, const float* T3, int B,
                       int bf16, double* dW, double* dTable, double* loss, double* Y) {
	double* w = (double*)malloc(sizeof(double) * NPARAM);
	for (int i = 0; i < NPARAM; i++) w[i] = bf16 ? orc_bf16(W[i]) : W[i];
	memset(dW, 0, sizeof(double) * NPARAM);
	memset(dTable, 0, sizeof(double) * 16 * (size_t)T * 2);
	double L = 0;
	double act[5][64], z[5][64], d[5][64], dn[64], x[64];
	for (int b = 0; b < B; b++) {
		orc_mlp_encode_hash(P + 3 * b, N + 3 * b, A + 3 * b, lo, ie, table, res, T, x);
		for (int i = 0; i < 64; i++) act[0][i] = bf16 ? orc_bf16((float)x[i]) : x[i];
		double y[16];
		for (int l = 0; l < 5; l++) {
			const double* in = act[l];
			int no = kLayerOut[l];
			for (int o = 0; o < no; o++) {
				double s = 0;
				for (int i = 0; i < kLayerIn[l]; i++) s += in[i] * w[layer_off(l) + i * no + o];
				z[l][o] = s;
			}
			if (l < 4)
				for (int o = 0; o < 64; o++) {
					double h = z[l][o] > 0 ? z[l][o] : 0;
					act[l + 1][o] = bf16 ? orc_bf16(h) : h;
				}
			else
				for (int o = 0; o < 16; o++) y[o] = z[l][o];
		}
		double dy[16];
		for (int c = 0; c < 16; c++) dy[c] = 0;
		for (int c = 0; c < 3; c++) {
			double t = T3[3 * b + c];
			double den = y[c] * y[c] + 0.01;
			L += (y[c] - t) * (y[c] - t) / den / B;
			dy[c] = 2 * (y[c] - t) / den / B;
			if (Y) Y[3 * b + c] = y[c];
		}
		for (int c = 0; c < 16; c++) d[4][c] = bf16 ? orc_bf16(dy[c]) : dy[c];
		for (int l = 4; l >= 0; l--) {
			int ni = kLayerIn[l], no = kLayerOut[l];
			for (int i = 0; i < ni; i++)
				for (int o = 0; o < no; o++) dW[layer_off(l) + i * no + o] += act[l][i] * d[l][o];
			if (l == 0) break;
			for (int i = 0; i < ni; i++) {
				double s = 0;
				for (int o = 0; o < no; o++) s += d[l][o] * w[layer_off(l) + i * no + o];
				dn[i] = (act[l][i] > 0) ? s : 0;
			}
			for (int i = 0; i < ni; i++) d[l - 1][i] = bf16 ? orc_bf16(dn[i]) : dn[i];
		}
		/* input gradient of the 32 hash features, scattered to the corners */
		for (int lv = 0; lv < 16; lv++) {
			uint32_t idx[8];
			float wt[8];
			hg_corners(P + 3 * b, lo, ie, res, T, lv, idx, wt);
			for (int k = 0; k < 2; k++) {
				double s = 0;
				for (int o = 0; o < 64; o++) s += d[0][o] * w[layer_off(0) + (2 * lv + k) * 64 + o];
				for (int c = 0; c < 8; c++) dTable[((size_t)lv * T + idx[c]) * 2 + k] += (double)wt[c] * s;
			}
		}
	}
	*loss = L;
	free(w);
}
