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
