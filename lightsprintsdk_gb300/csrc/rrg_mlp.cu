// Training and inference kernels of the radiance-cache network (rrg_mlp.cuh)
// and the C ABI of include/rrgpu_cache.h.
//
// One training step (captured in a CUDA graph by the caller if wanted):
//   k_mlp_fwd_bwd : warp per 16 samples: gather the batch's records, encode,
//                   forward through 5 BF16 mma layers, relative-L2 loss
//                   gradient, back-propagate the deltas through W^T; stores the
//                   encoded inputs, activations and deltas (BF16) for
//   k_mlp_wgrad   : dW_l = In_l^T dZ_l, a K = batch reduction: one CTA per
//                   (layer, 128-row chunk), warp per 16 input features,
//                   partial sums added to the FP32 gradient atomically;
//   k_mlp_adam    : Adam on the FP32 masters, gradient reset;
//   k_mlp_pack    : BF16 fragment copies of W and W^T.
// Inference: k_mlp_infer, warp per 16 samples, weights staged in shared
// memory, activations in registers from input to output.
#include "rrg_internal.cuh"
#include "rrg_mlp.cuh"

#include <math.h>
#include "../../include/rrgpu_cache.h"

namespace rrg {

__device__ __forceinline__ uint64_t mlp_mix(uint64_t k) {
	k ^= k >> 33;
	k *= 0xFF51AFD7ED558CCDULL;
	k ^= k >> 33;
	k *= 0xC4CEB9FE1A85EC53ULL;
	k ^= k >> 33;
	return k;
}

__global__ void k_mlp_init(float* __restrict__ w, uint64_t seed) {
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= kMlpParams) return;
	int l = i < 16384 ? i / 4096 : 4;
	float fan = l < 4 ? 128.f : 80.f;
	float s = sqrtf(6.f / fan);
	uint64_t h = mlp_mix(mlp_mix((uint64_t)i ^ (seed * 0x9E3779B97F4A7C15ULL)) + 0x632BE59BD9B4E019ULL);
	float u = (float)(h >> 40) * (1.0f / 16777216.0f);
	w[i] = (2.f * u - 1.f) * s;
}

// fragment packing: word f of layer l -> two bf16 of W (fwd) or W^T (bwd)
__global__ void k_mlp_pack(const float* __restrict__ w, uint32_t* __restrict__ fwd, uint32_t* __restrict__ bwd) {
	int f = blockIdx.x * blockDim.x + threadIdx.x;
	if (f >= kMlpFragWords) return;
	int l = f < 8192 ? f / 2048 : 4;
	int local = f - mlp_frag_off(l);
	const int no = mlp_layer_out(l);
	const float* W = w + mlp_layer_off(l);
	int r = local & 1, lane = (local >> 1) & 31, tile = local >> 6;
	int g = lane >> 2, q = lane & 3;
	{   // forward: K = 64 inputs, N = no outputs, NT = no / 8
		int NT = no / 8;
		int kt = tile / NT, nt = tile % NT;
		int k0 = 16 * kt + 8 * r + 2 * q, n = 8 * nt + g;
		fwd[f] = pack_bf16(W[k0 * no + n], W[(k0 + 1) * no + n]);
	}
	{   // backward: K = no outputs, N = 64 inputs, NT = 8
		int kt = tile / 8, nt = tile % 8;
		int k0 = 16 * kt + 8 * r + 2 * q, n = 8 * nt + g;
		bwd[f] = pack_bf16(W[n * no + k0], W[n * no + k0 + 1]);
	}
}

struct MlpBuffers {
	uint32_t* X;          // [B][32] words (64 bf16)
	uint32_t* H[4];       // inputs of layers 1..4
	uint32_t* dZ[5];      // [B][32] words for layers 0..3, [B][8] for layer 4
	float* grad;          // kMlpParams
	float* loss;          // 1
};

__device__ __forceinline__ void store_a_rows(uint32_t* base, int row0, const uint32_t* a, int kt) {
	const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
	base[(row0 + g) * 32 + 8 * kt + q] = a[0];
	base[(row0 + g + 8) * 32 + 8 * kt + q] = a[1];
	base[(row0 + g) * 32 + 8 * kt + 4 + q] = a[2];
	base[(row0 + g + 8) * 32 + 8 * kt + 4 + q] = a[3];
}

// relu' mask of a C-layout fragment from the stored bf16 activations H
__device__ __forceinline__ void mask_c(const uint32_t* H, int row0, int nt, float* c) {
	const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
	uint32_t w0 = H[(row0 + g) * 32 + 4 * nt + q], w1 = H[(row0 + g + 8) * 32 + 4 * nt + q];
	if (!(bf16_lo(w0) > 0.f)) c[0] = 0.f;
	if (!(bf16_hi(w0) > 0.f)) c[1] = 0.f;
	if (!(bf16_lo(w1) > 0.f)) c[2] = 0.f;
	if (!(bf16_hi(w1) > 0.f)) c[3] = 0.f;
}

__device__ __forceinline__ uint32_t batch_index(uint64_t seed, uint64_t step, uint32_t row, uint32_t nrec,
                                                const uint32_t* order) {
	if (order) return order[row];
	uint64_t h = mlp_mix(mlp_mix(((uint64_t)row << 20) ^ (step * 0xD1B54A32D192ED03ULL) ^ seed) + 0x9E3779B97F4A7C15ULL);
	return (uint32_t)(h % nrec);
}

__global__ void k_mlp_fwd_bwd(const CacheRec* __restrict__ recs, uint32_t nrec, uint32_t B, uint64_t seed, uint64_t step,
                              const uint32_t* __restrict__ order, const uint32_t* __restrict__ fwd,
                              const uint32_t* __restrict__ bwd, MlpBuffers buf, float lo0, float lo1, float lo2,
                              float ie0, float ie1, float ie2, float* __restrict__ pred, HashGrid hg) {
	const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
	const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const uint32_t ntiles = B / 16;
	if (warp >= ntiles) return;
	const int row0 = warp * 16;
	const float lo[3] = {lo0, lo1, lo2}, ie[3] = {ie0, ie1, ie2};
	{   // encode 16 samples: lane -> row lane&15, half lane>>4
		int r = lane & 15;
		uint32_t idx = batch_index(seed, step, row0 + r, nrec, order);
		const CacheRec rec = recs[idx];
		if (hg.table) mlp_encode_half_hash(rec.p, rec.n, rec.alb, lo, ie, hg, lane >> 4, buf.X + (size_t)(row0 + r) * 32);
		else mlp_encode_half(rec.p, rec.n, rec.alb, lo, ie, lane >> 4, buf.X + (size_t)(row0 + r) * 32);
	}
	__syncwarp();
	uint32_t a[4][4];
	float acc[8][4];
#pragma unroll
	for (int kt = 0; kt < 4; kt++) load_a(buf.X + (size_t)row0 * 32, 32, kt, a[kt]);
#pragma unroll
	for (int l = 0; l < 4; l++) {
		mlp_layer<8>(a, fwd + mlp_frag_off(l), acc);
#pragma unroll
		for (int kt = 0; kt < 4; kt++) {
			c_to_a<true>(acc[2 * kt], acc[2 * kt + 1], a[kt]);
			store_a_rows(buf.H[l], row0, a[kt], kt);
		}
	}
	float y[2][4];
	mlp_layer<2>(a, fwd + mlp_frag_off(4), y);
	// relative L2 loss gradient on channels 0..2
	uint32_t ia = batch_index(seed, step, row0 + g, nrec, order);
	uint32_t ib = batch_index(seed, step, row0 + g + 8, nrec, order);
	float dy[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
	float lsum = 0.f;
	const float invB = 1.f / (float)B;
#pragma unroll
	for (int e = 0; e < 4; e++) {
		int c = 2 * q + (e & 1);
		if (c < 3) {
			float t = (e < 2) ? recs[ia].t[c] : recs[ib].t[c];
			float yv = y[0][e];
			float den = yv * yv + 0.01f;
			dy[0][e] = 2.f * (yv - t) / den * invB;
			lsum += (yv - t) * (yv - t) / den * invB;
			if (pred) pred[(size_t)(row0 + g + (e >= 2 ? 8 : 0)) * 3 + c] = yv;
		}
	}
	for (int o = 16; o; o >>= 1) lsum += __shfl_xor_sync(0xFFFFFFFFu, lsum, o);
	if (lane == 0) atomicAdd(buf.loss, lsum);
	// dZ5 (16 wide) -> one A k-tile; store [B][8] words
	uint32_t d5[4];
	c_to_a<false>(dy[0], dy[1], d5);
	buf.dZ[4][(row0 + g) * 8 + q] = d5[0];
	buf.dZ[4][(row0 + g + 8) * 8 + q] = d5[1];
	buf.dZ[4][(row0 + g) * 8 + 4 + q] = d5[2];
	buf.dZ[4][(row0 + g + 8) * 8 + 4 + q] = d5[3];
	// dH4 = dZ5 W5^T (K = 16)
#pragma unroll
	for (int nt = 0; nt < 8; nt++) {
		acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
		const uint2 b = *reinterpret_cast<const uint2*>(bwd + mlp_frag_off(4) + (nt * 32 + lane) * 2);
		mma16816(acc[nt], d5, b.x, b.y);
	}
	__syncwarp();
	// layers 3, 2, 1, 0: mask with the layer's input activation, store dZ, propagate
#pragma unroll
	for (int l = 3; l >= 0; l--) {
#pragma unroll
		for (int nt = 0; nt < 8; nt++) mask_c(buf.H[l], row0, nt, acc[nt]);
#pragma unroll
		for (int kt = 0; kt < 4; kt++) {
			c_to_a<false>(acc[2 * kt], acc[2 * kt + 1], a[kt]);
			store_a_rows(buf.dZ[l], row0, a[kt], kt);
		}
		if (l == 0) {
			if (hg.table) {
				// input gradient of the 32 hash features, dX = dZ_0 W_0^T
				// (columns 0..31 = n-tiles 0..3), scattered to the table:
				// n-tile nt holds level 4 nt + q for rows g and g + 8
#pragma unroll
				for (int nt = 0; nt < 4; nt++) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll
				for (int kt = 0; kt < 4; kt++)
#pragma unroll
					for (int nt = 0; nt < 4; nt++) {
						const uint2 b = *reinterpret_cast<const uint2*>(bwd + mlp_frag_off(0) + ((kt * 8 + nt) * 32 + lane) * 2);
						mma16816(acc[nt], a[kt], b.x, b.y);
					}
#pragma unroll
				for (int nt = 0; nt < 4; nt++) {
					hash_backward(recs[ia].p, lo, ie, hg, 4 * nt + q, acc[nt][0], acc[nt][1]);
					hash_backward(recs[ib].p, lo, ie, hg, 4 * nt + q, acc[nt][2], acc[nt][3]);
				}
			}
			break;
		}
		// dH_l = dZ_l W_l^T (K = 64)
#pragma unroll
		for (int nt = 0; nt < 8; nt++) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll
		for (int kt = 0; kt < 4; kt++)
#pragma unroll
			for (int nt = 0; nt < 8; nt++) {
				const uint2 b = *reinterpret_cast<const uint2*>(bwd + mlp_frag_off(l) + ((kt * 8 + nt) * 32 + lane) * 2);
				mma16816(acc[nt], a[kt], b.x, b.y);
			}
	}
}

// dW_l (64 x no) += In_l^T (64 x R) * dZ_l (R x no) over a 128-row chunk.
// In_l rows are 32 words; dZ rows are 32 words (no = 64) or 8 (no = 16).
constexpr int kWgRows = 128;

template <int NO>
__device__ void wgrad_chunk(const uint32_t* __restrict__ In, const uint32_t* __restrict__ dZ, int row0,
                            float* __restrict__ grad, uint16_t (*sIn)[64], uint16_t (*sZ)[64]) {
	const int dzw = NO / 2;   // words per dZ row
	for (int i = threadIdx.x; i < kWgRows * 32; i += blockDim.x) {
		int r = i / 32, w = i % 32;
		uint32_t v = In[(size_t)(row0 + r) * 32 + w];
		sIn[r][2 * w] = (uint16_t)(v & 0xFFFFu);
		sIn[r][2 * w + 1] = (uint16_t)(v >> 16);
	}
	for (int i = threadIdx.x; i < kWgRows * dzw; i += blockDim.x) {
		int r = i / dzw, w = i % dzw;
		uint32_t v = dZ[(size_t)(row0 + r) * dzw + w];
		sZ[r][2 * w] = (uint16_t)(v & 0xFFFFu);
		sZ[r][2 * w + 1] = (uint16_t)(v >> 16);
	}
	__syncthreads();
	const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3, w = threadIdx.x >> 5;
	constexpr int NT = NO / 8;
	float acc[NT][4];
#pragma unroll
	for (int nt = 0; nt < NT; nt++) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
	const int m0 = 16 * w;
	for (int ks = 0; ks < kWgRows / 16; ks++) {
		const int k0 = 16 * ks;
		uint32_t a[4];
		a[0] = sIn[k0 + 2 * q][m0 + g] | ((uint32_t)sIn[k0 + 2 * q + 1][m0 + g] << 16);
		a[1] = sIn[k0 + 2 * q][m0 + g + 8] | ((uint32_t)sIn[k0 + 2 * q + 1][m0 + g + 8] << 16);
		a[2] = sIn[k0 + 8 + 2 * q][m0 + g] | ((uint32_t)sIn[k0 + 8 + 2 * q + 1][m0 + g] << 16);
		a[3] = sIn[k0 + 8 + 2 * q][m0 + g + 8] | ((uint32_t)sIn[k0 + 8 + 2 * q + 1][m0 + g + 8] << 16);
#pragma unroll
		for (int nt = 0; nt < NT; nt++) {
			uint32_t b0 = sZ[k0 + 2 * q][8 * nt + g] | ((uint32_t)sZ[k0 + 2 * q + 1][8 * nt + g] << 16);
			uint32_t b1 = sZ[k0 + 8 + 2 * q][8 * nt + g] | ((uint32_t)sZ[k0 + 8 + 2 * q + 1][8 * nt + g] << 16);
			mma16816(acc[nt], a, b0, b1);
		}
	}
#pragma unroll
	for (int nt = 0; nt < NT; nt++) {
		// columns n and n + 1 are adjacent (n even): one 8-byte atomic per row
		int n = 8 * nt + 2 * q;
		atomicAdd(reinterpret_cast<float2*>(&grad[(m0 + g) * NO + n]), make_float2(acc[nt][0], acc[nt][1]));
		atomicAdd(reinterpret_cast<float2*>(&grad[(m0 + g + 8) * NO + n]), make_float2(acc[nt][2], acc[nt][3]));
	}
}

__global__ void __launch_bounds__(128) k_mlp_wgrad(MlpBuffers buf, uint32_t B) {
	const int nchunk = B / kWgRows;
	const int l = blockIdx.x / nchunk, chunk = blockIdx.x % nchunk;
	__shared__ uint16_t sIn[kWgRows][64];
	__shared__ uint16_t sZ[kWgRows][64];
	const uint32_t* In = l == 0 ? buf.X : buf.H[l - 1];
	if (l < 4) wgrad_chunk<64>(In, buf.dZ[l], chunk * kWgRows, buf.grad + mlp_layer_off(l), sIn, sZ);
	else wgrad_chunk<16>(In, buf.dZ[4], chunk * kWgRows, buf.grad + mlp_layer_off(4), sIn, sZ);
}

__global__ void k_mlp_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                           float* __restrict__ grad, float lr, float b1, float b2, float eps, float c1, float c2) {
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= kMlpParams) return;
	float gr = grad[i];
	grad[i] = 0.f;
	if (!isfinite(gr)) return;
	float mi = b1 * m[i] + (1.f - b1) * gr;
	float vi = b2 * v[i] + (1.f - b2) * gr * gr;
	m[i] = mi;
	v[i] = vi;
	w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// Hash table: uniform in [-1e-4, 1e-4] (the initialisation of the hash
// encoding's paper), and Adam with the network's hyper-parameters.
__global__ void k_table_init(float* __restrict__ t, uint64_t n, uint64_t seed) {
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
		uint64_t h = mlp_mix(mlp_mix(i ^ (seed * 0xD1B54A32D192ED03ULL)) + 0x632BE59BD9B4E019ULL);
		float u = (float)(h >> 40) * (1.0f / 16777216.0f);
		t[i] = (2.f * u - 1.f) * 1e-4f;
	}
}

// One Adam step of a table entry (entries whose gradient is not finite keep
// their state).
__device__ __forceinline__ void adam_entry(float gr, float& mi, float& vi, float& wi, float lr, float b1, float b2,
                                           float eps, float c1, float c2) {
	if (!isfinite(gr)) return;
	mi = b1 * mi + (1.f - b1) * gr;
	vi = b2 * vi + (1.f - b2) * gr * gr;
	wi -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// Adam over the whole table (every entry's moments decay each step), four
// entries per thread and iteration with all four arrays read up front: the
// kernel is a stream over 32 B per entry, bound by HBM.
__global__ void k_table_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                             float* __restrict__ grad, uint64_t n, float lr, float b1, float b2, float eps, float c1,
                             float c2) {
	const uint64_t n4 = n / 4, stride = (uint64_t)gridDim.x * blockDim.x;
	float4* w4 = reinterpret_cast<float4*>(w);
	float4* m4 = reinterpret_cast<float4*>(m);
	float4* v4 = reinterpret_cast<float4*>(v);
	float4* g4 = reinterpret_cast<float4*>(grad);
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n4; i += stride) {
		const float4 gr = g4[i];
		float4 mm = m4[i], vv = v4[i], ww = w4[i];
		g4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
		adam_entry(gr.x, mm.x, vv.x, ww.x, lr, b1, b2, eps, c1, c2);
		adam_entry(gr.y, mm.y, vv.y, ww.y, lr, b1, b2, eps, c1, c2);
		adam_entry(gr.z, mm.z, vv.z, ww.z, lr, b1, b2, eps, c1, c2);
		adam_entry(gr.w, mm.w, vv.w, ww.w, lr, b1, b2, eps, c1, c2);
		m4[i] = mm;
		v4[i] = vv;
		w4[i] = ww;
	}
	for (uint64_t i = 4 * n4 + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
		const float gr = grad[i];
		grad[i] = 0.f;
		float mi = m[i], vi = v[i], wi = w[i];
		adam_entry(gr, mi, vi, wi, lr, b1, b2, eps, c1, c2);
		m[i] = mi;
		v[i] = vi;
		w[i] = wi;
	}
}

// Inference: warp per 16 records.  out[i] = (rgb clamped >= 0, valid flag).
constexpr int kInferWarps = 8;
__global__ void __launch_bounds__(kInferWarps * 32) k_mlp_infer(const CacheRec* __restrict__ recs, uint64_t n,
                                                                const uint32_t* __restrict__ fwd_g, float lo0,
                                                                float lo1, float lo2, float ie0, float ie1, float ie2,
                                                                float4* __restrict__ out, HashGrid hg,
                                                                int all_valid) {
	extern __shared__ uint32_t smem[];
	uint32_t* fwd = smem;                                   // kMlpFragWords
	uint32_t* tiles = smem + kMlpFragWords;                  // kInferWarps x 16 x 32 words
	for (int i = threadIdx.x; i < kMlpFragWords; i += blockDim.x) fwd[i] = fwd_g[i];
	__syncthreads();
	const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3, w = threadIdx.x >> 5;
	uint32_t* tile = tiles + w * 16 * 32;
	const float lo[3] = {lo0, lo1, lo2}, ie[3] = {ie0, ie1, ie2};
	const uint64_t ntiles = (n + 15) / 16;
	for (uint64_t t = (uint64_t)blockIdx.x * kInferWarps + w; t < ntiles; t += (uint64_t)gridDim.x * kInferWarps) {
		const uint64_t r0 = t * 16;
		{
			int r = lane & 15;
			uint64_t i = r0 + r;
			CacheRec rec;
			if (i < n) rec = recs[i];
			else {
				for (int k = 0; k < 3; k++) { rec.p[k] = lo[k]; rec.n[k] = 0.f; rec.alb[k] = 0.f; rec.t[k] = 0.f; }
			}
			if (hg.table) mlp_encode_half_hash(rec.p, rec.n, rec.alb, lo, ie, hg, lane >> 4, tile + r * 32);
			else mlp_encode_half(rec.p, rec.n, rec.alb, lo, ie, lane >> 4, tile + r * 32);
		}
		__syncwarp();
		uint32_t x[4][4];
#pragma unroll
		for (int kt = 0; kt < 4; kt++) load_a(tile, 32, kt, x[kt]);
		float y[2][4];
		mlp_forward_tile(x, fwd, y);
		// channels 0..2 live in n-tile 0 at columns 2q, 2q+1 (q = 0, 1)
		__syncwarp();
		float* ftile = reinterpret_cast<float*>(tile);   // reuse as [16][4] floats
		if (q < 2) {
			ftile[g * 4 + 2 * q] = y[0][0];
			if (2 * q + 1 < 3) ftile[g * 4 + 2 * q + 1] = y[0][1];
			ftile[(g + 8) * 4 + 2 * q] = y[0][2];
			if (2 * q + 1 < 3) ftile[(g + 8) * 4 + 2 * q + 1] = y[0][3];
		}
		__syncwarp();
		if (lane < 16 && r0 + lane < n) {
			// queries mark validity in t[0]; training records (the error
			// grid's input) carry targets there, all of them valid
			float valid = all_valid ? 1.f : recs[r0 + lane].t[0];
			float4 o;
			o.x = valid > 0.f ? fmaxf(ftile[lane * 4 + 0], 0.f) : 0.f;
			o.y = valid > 0.f ? fmaxf(ftile[lane * 4 + 1], 0.f) : 0.f;
			o.z = valid > 0.f ? fmaxf(ftile[lane * 4 + 2], 0.f) : 0.f;
			o.w = valid;
			out[r0 + lane] = o;
		}
		__syncwarp();
	}
}

// ------------------------------------------------------------------ cache
struct RadianceCache {
	int device = 0;
	int num_sms = 0;
	float lo[3], ie[3];
	float* w = nullptr;       // masters
	float* m = nullptr;
	float* v = nullptr;
	uint32_t* fwd = nullptr;
	uint32_t* bwd = nullptr;
	MlpBuffers buf{};
	uint32_t capB = 0;
	uint64_t steps = 0;
	uint8_t* grid = nullptr;       // reliability per cell
	int grid_res = 0;
	float lr = 5e-3f, b1 = 0.9f, b2 = 0.99f, eps = 1e-8f;
	// hash-grid encoding (hg.table == nullptr: frequency encoding)
	HashGrid hg{};
	float* table = nullptr;        // kHashLevels x T x 2
	float* tm = nullptr;
	float* tv = nullptr;
	float* tgrad = nullptr;
	uint64_t table_floats = 0;
	int infer_per_sm = 0;          // resident k_mlp_infer blocks per SM (0: not yet known)
};

static void free_cache(RadianceCache* C) {
	if (!C) return;
	cudaFree(C->w); cudaFree(C->m); cudaFree(C->v); cudaFree(C->fwd); cudaFree(C->bwd);
	cudaFree(C->buf.X);
	for (int i = 0; i < 4; i++) cudaFree(C->buf.H[i]);
	for (int i = 0; i < 5; i++) cudaFree(C->buf.dZ[i]);
	cudaFree(C->buf.grad); cudaFree(C->buf.loss);
	cudaFree(C->grid);
	cudaFree(C->table); cudaFree(C->tm); cudaFree(C->tv); cudaFree(C->tgrad);
	delete C;
}

static int ensure_batch(RadianceCache* C, uint32_t B) {
	if (B <= C->capB) return RRG_OK;
	cudaFree(C->buf.X);
	for (int i = 0; i < 4; i++) cudaFree(C->buf.H[i]);
	for (int i = 0; i < 5; i++) cudaFree(C->buf.dZ[i]);
	C->buf.X = nullptr;
	for (int i = 0; i < 4; i++) C->buf.H[i] = nullptr;
	for (int i = 0; i < 5; i++) C->buf.dZ[i] = nullptr;
	C->capB = 0;
	RRG_CUDA(cudaMalloc(&C->buf.X, (size_t)B * 128));
	for (int i = 0; i < 4; i++) RRG_CUDA(cudaMalloc(&C->buf.H[i], (size_t)B * 128));
	for (int i = 0; i < 4; i++) RRG_CUDA(cudaMalloc(&C->buf.dZ[i], (size_t)B * 128));
	RRG_CUDA(cudaMalloc(&C->buf.dZ[4], (size_t)B * 32));
	C->capB = B;
	return RRG_OK;
}

static int pack(RadianceCache* C, cudaStream_t s) {
	rrg::note_launch(), k_mlp_pack<<<(kMlpFragWords + 255) / 256, 256, 0, s>>>(C->w, C->fwd, C->bwd);
	RRG_CUDA(cudaGetLastError());
	return RRG_OK;
}

// one forward/backward over B records (B multiple of 128); grad accumulates
static int fwd_bwd(RadianceCache* C, const CacheRec* recs, uint32_t nrec, uint32_t B, uint64_t seed,
                   const uint32_t* order, float* pred, cudaStream_t s) {
	int st = ensure_batch(C, B);
	if (st) return st;
	const int warps = B / 16;
	rrg::note_launch(), k_mlp_fwd_bwd<<<(warps + 3) / 4, 128, 0, s>>>(recs, nrec, B, seed, C->steps, order, C->fwd, C->bwd, C->buf,
	                                              C->lo[0], C->lo[1], C->lo[2], C->ie[0], C->ie[1], C->ie[2], pred,
	                                              C->hg);
	rrg::note_launch(), k_mlp_wgrad<<<5 * (B / kWgRows), 128, 0, s>>>(C->buf, B);
	RRG_CUDA(cudaGetLastError());
	return RRG_OK;
}

// error grid: per cell sums of target and prediction (mean over RGB) and counts
__global__ void k_grid_accum(const CacheRec* __restrict__ recs, const float4* __restrict__ pred, uint64_t n, int res,
                             float lo0, float lo1, float lo2, float ie0, float ie1, float ie2, float* __restrict__ st,
                             float* __restrict__ sp, float* __restrict__ cnt) {
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
		const CacheRec& r = recs[i];
		int vx = min(res - 1, max(0, (int)((r.p[0] - lo0) * ie0 * res)));
		int vy = min(res - 1, max(0, (int)((r.p[1] - lo1) * ie1 * res)));
		int vz = min(res - 1, max(0, (int)((r.p[2] - lo2) * ie2 * res)));
		size_t c = ((size_t)vz * res + vy) * res + vx;
		float4 p = pred[i];
		float tm = (r.t[0] + r.t[1] + r.t[2]) * (1.f / 3.f);
		atomicAdd(&st[c], tm);
		atomicAdd(&sp[c], (p.x + p.y + p.z) * (1.f / 3.f));
		atomicAdd(&cnt[c], 1.f);
		atomicAdd(&st[c + 3 * (size_t)res * res * res], tm * tm);
	}
}

// A cell is reliable when it holds >= min_count records and the mean
// prediction differs from the mean target by at most max(thr * mean target,
// 3 standard errors of that mean): the targets are single-path estimates, so
// their own noise bounds what the test can resolve.
__global__ void k_grid_flags(const float* __restrict__ st, const float* __restrict__ sp, const float* __restrict__ cnt,
                             const float* __restrict__ st2, size_t ncell, float thr, float min_count,
                             float plain_samples, uint8_t* __restrict__ flags, unsigned int* __restrict__ nrel) {
	size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
	if (c >= ncell) return;
	float n = cnt[c];
	bool ok = false;
	if (n >= min_count) {
		float mt = st[c] / n, mp = sp[c] / n;
		float var = fmaxf(st2[c] / n - mt * mt, 0.f);
		float se = sqrtf(var / n);
		float tol = fmaxf(thr * fmaxf(mt, 1e-4f), 3.f * se);
		// a bias below the noise of a plain_samples-sample mean of these
		// paths costs less than falling back to that mean
		if (plain_samples > 0.f) tol = fmaxf(tol, sqrtf(var / plain_samples));
		ok = fabsf(mp - mt) <= tol;
	}
	flags[c] = ok ? 1 : 0;
	if (ok) atomicAdd(nrel, 1u);
}

void cache_grid(rrg_cache* h, const uint8_t** flags, int* res, float* lo, float* ie) {
	RadianceCache* C = reinterpret_cast<RadianceCache*>(h);
	*flags = C ? C->grid : nullptr;
	*res = C ? C->grid_res : 0;
	for (int k = 0; k < 3; k++) {
		lo[k] = C ? C->lo[k] : 0.f;
		ie[k] = C ? C->ie[k] : 0.f;
	}
}

}  // namespace rrg

using namespace rrg;

static int infer_impl(RadianceCache* C, const void* recs_dev, uint64_t n, float* out_dev, int all_valid,
                      cudaStream_t stream) {
	if (!C || !recs_dev || !out_dev || ((uintptr_t)out_dev & 15)) return RRG_ERR_INVALID;
	if (!n) return RRG_OK;
	const size_t smem = sizeof(uint32_t) * (kMlpFragWords + kInferWarps * 16 * 32);
	if (!C->infer_per_sm) {   // on the cache's device, once
		int per_sm = 0;
		RRG_CUDA(cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
		RRG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mlp_infer, kInferWarps * 32, smem));
		C->infer_per_sm = per_sm < 1 ? 1 : per_sm;
	}
	const int per_sm = C->infer_per_sm;
	uint64_t ntiles = (n + 15) / 16;
	uint64_t blocks = (ntiles + kInferWarps - 1) / kInferWarps;
	uint64_t cap = (uint64_t)C->num_sms * per_sm;   // one wave of resident blocks, grid-stride over the tiles
	rrg::note_launch(), k_mlp_infer<<<(int)(blocks < cap ? blocks : cap), kInferWarps * 32, smem, (cudaStream_t)stream>>>(
	    reinterpret_cast<const CacheRec*>(recs_dev), n, C->fwd, C->lo[0], C->lo[1], C->lo[2], C->ie[0], C->ie[1],
	    C->ie[2], reinterpret_cast<float4*>(out_dev), C->hg, all_valid);
	RRG_CUDA(cudaGetLastError());
	return RRG_OK;
}

extern "C" {

int rrg_cache_build_error_grid(rrg_cache* h, const void* recs_dev, uint64_t nrec, uint32_t res, float rel_threshold,
                               uint32_t min_count, uint32_t* nreliable, void* stream) {
	return rrg_cache_build_error_grid_ex(h, recs_dev, nrec, res, rel_threshold, min_count, 0.f, nreliable, stream);
}

int rrg_cache_build_error_grid_ex(rrg_cache* h, const void* recs_dev, uint64_t nrec, uint32_t res,
                                  float rel_threshold, uint32_t min_count, float plain_samples, uint32_t* nreliable,
                                  void* stream) {
	RadianceCache* C = reinterpret_cast<RadianceCache*>(h);
	if (!C || !recs_dev || !nrec || res < 1 || res > 256 || !(plain_samples >= 0.f)) return RRG_ERR_INVALID;
	cudaStream_t s = (cudaStream_t)stream;
	const size_t ncell = (size_t)res * res * res;
	float4* pred = nullptr;
	float* sums = nullptr;
	unsigned int* nrel = nullptr;
	RRG_CUDA(cudaMalloc(&pred, sizeof(float4) * nrec));
	RRG_CUDA(cudaMalloc(&sums, sizeof(float) * 4 * ncell));
	RRG_CUDA(cudaMalloc(&nrel, sizeof(unsigned int)));
	if (C->grid_res != (int)res) {
		cudaFree(C->grid);
		C->grid = nullptr;
		C->grid_res = 0;
		RRG_CUDA(cudaMalloc(&C->grid, ncell));
		C->grid_res = (int)res;
	}
	RRG_CUDA(cudaMemsetAsync(sums, 0, sizeof(float) * 4 * ncell, s));
	RRG_CUDA(cudaMemsetAsync(nrel, 0, sizeof(unsigned int), s));
	int st = infer_impl(C, recs_dev, nrec, reinterpret_cast<float*>(pred), 1, s);
	if (!st) {
		rrg::note_launch(), k_grid_accum<<<C->num_sms * 8, 256, 0, s>>>(reinterpret_cast<const CacheRec*>(recs_dev), pred, nrec, (int)res,
		                                             C->lo[0], C->lo[1], C->lo[2], C->ie[0], C->ie[1], C->ie[2], sums,
		                                             sums + ncell, sums + 2 * ncell);
		rrg::note_launch(), k_grid_flags<<<(unsigned)((ncell + 255) / 256), 256, 0, s>>>(sums, sums + ncell, sums + 2 * ncell,
		                                                            sums + 3 * ncell, ncell, rel_threshold,
		                                                            (float)min_count, plain_samples, C->grid, nrel);
		cudaError_t e = cudaGetLastError();
		if (e != cudaSuccess) st = cuda_fail(e);
	}
	unsigned int hn = 0;
	if (!st) {
		cudaMemcpyAsync(&hn, nrel, sizeof(unsigned int), cudaMemcpyDeviceToHost, s);
		cudaStreamSynchronize(s);
	}
	if (nreliable) *nreliable = hn;
	cudaFree(pred);
	cudaFree(sums);
	cudaFree(nrel);
	return st;
}

int rrg_cache_create(const float* lo, const float* hi, uint64_t seed, rrg_cache** out) {
	if (!lo || !hi) return RRG_ERR_INVALID;
	rrg_cache_params p{};
	p.size = sizeof(p);
	for (int k = 0; k < 3; k++) { p.lo[k] = lo[k]; p.hi[k] = hi[k]; }
	p.seed = seed;
	p.encoding = RRG_CACHE_FREQUENCY;
	return rrg_cache_create_ex(&p, out);
}

int rrg_cache_create_ex(const rrg_cache_params* params, rrg_cache** out) {
	if (!out || !params) return RRG_ERR_INVALID;
	*out = nullptr;
	if (params->size < sizeof(rrg_cache_params)) return RRG_ERR_INVALID;
	if (params->encoding != RRG_CACHE_FREQUENCY && params->encoding != RRG_CACHE_HASHGRID) return RRG_ERR_INVALID;
	const float* lo = params->lo;
	const float* hi = params->hi;
	const uint64_t seed = params->seed;
	const uint32_t log2T = params->log2_table ? params->log2_table : 19;
	const float min_res = params->min_res > 0.f ? params->min_res : 16.f;
	const float max_res = params->max_res > 0.f ? params->max_res : 1024.f;
	if (params->encoding == RRG_CACHE_HASHGRID && (log2T < 10 || log2T > 24 || !(max_res >= min_res) || min_res < 2.f))
		return RRG_ERR_INVALID;
	RadianceCache* C = new RadianceCache();
	RRG_CUDA(cudaGetDevice(&C->device));
	cudaDeviceProp prop;
	RRG_CUDA(cudaGetDeviceProperties(&prop, C->device));
	C->num_sms = prop.multiProcessorCount;
	for (int k = 0; k < 3; k++) {
		float e = hi[k] - lo[k];
		if (!(e > 0.f)) { delete C; return RRG_ERR_INVALID; }
		C->lo[k] = lo[k];
		C->ie[k] = 1.f / e;
	}
	cudaError_t e = cudaSuccess;
	if (e == cudaSuccess) e = cudaMalloc(&C->w, sizeof(float) * kMlpParams);
	if (e == cudaSuccess) e = cudaMalloc(&C->m, sizeof(float) * kMlpParams);
	if (e == cudaSuccess) e = cudaMalloc(&C->v, sizeof(float) * kMlpParams);
	if (e == cudaSuccess) e = cudaMalloc(&C->fwd, sizeof(uint32_t) * kMlpFragWords);
	if (e == cudaSuccess) e = cudaMalloc(&C->bwd, sizeof(uint32_t) * kMlpFragWords);
	if (e == cudaSuccess) e = cudaMalloc(&C->buf.grad, sizeof(float) * kMlpParams);
	if (e == cudaSuccess) e = cudaMalloc(&C->buf.loss, sizeof(float));
	if (e == cudaSuccess) e = cudaMemset(C->m, 0, sizeof(float) * kMlpParams);
	if (e == cudaSuccess) e = cudaMemset(C->v, 0, sizeof(float) * kMlpParams);
	if (e == cudaSuccess) e = cudaMemset(C->buf.grad, 0, sizeof(float) * kMlpParams);
	if (e != cudaSuccess) { free_cache(C); return cuda_fail(e); }
	rrg::note_launch(), k_mlp_init<<<(kMlpParams + 255) / 256, 256>>>(C->w, seed);
	if (params->encoding == RRG_CACHE_HASHGRID) {
		const uint32_t T = 1u << log2T;
		C->table_floats = (uint64_t)kHashLevels * T * 2;
		const size_t bytes = sizeof(float) * C->table_floats;
		e = cudaMalloc(&C->table, bytes);
		if (e == cudaSuccess) e = cudaMalloc(&C->tm, bytes);
		if (e == cudaSuccess) e = cudaMalloc(&C->tv, bytes);
		if (e == cudaSuccess) e = cudaMalloc(&C->tgrad, bytes);
		if (e == cudaSuccess) e = cudaMemset(C->tm, 0, bytes);
		if (e == cudaSuccess) e = cudaMemset(C->tv, 0, bytes);
		if (e == cudaSuccess) e = cudaMemset(C->tgrad, 0, bytes);
		if (e != cudaSuccess) { free_cache(C); return cuda_fail(e); }
		rrg::note_launch(), k_table_init<<<C->num_sms * 8, 256>>>(C->table, C->table_floats, seed);
		C->hg.table = reinterpret_cast<const float2*>(C->table);
		C->hg.tgrad = C->tgrad;
		C->hg.T = T;
		C->hg.dense = 0;
		// resolutions floor(min_res b^l), b = (max_res / min_res)^(1/15), as
		// oracle/rr_mlp.c and oracle/orc.py::hashgrid_res compute them
		const double b = exp((log((double)max_res) - log((double)min_res)) / (kHashLevels - 1));
		for (int l = 0; l < kHashLevels; l++) {
			const double r = floor((double)min_res * pow(b, (double)l));
			C->hg.res[l] = (float)r;
			const double n1 = r + 1.0;
			if (n1 * n1 * n1 <= (double)T) C->hg.dense |= 1u << l;
		}
	}
	int st = pack(C, nullptr);
	if (st) { free_cache(C); return st; }
	*out = reinterpret_cast<rrg_cache*>(C);
	return RRG_OK;
}

uint64_t rrg_cache_table_floats(const rrg_cache* h) {
	const RadianceCache* C = reinterpret_cast<const RadianceCache*>(h);
	return C ? C->table_floats : 0;
}

int rrg_cache_get_table(rrg_cache* h, float* host) {
	RadianceCache* C = reinterpret_cast<RadianceCache*>(h);
	if (!C || !host || !C->table) return RRG_ERR_INVALID;
	RRG_CUDA(cudaMemcpy(host, C->table, sizeof(float) * C->table_floats, cudaMemcpyDeviceToHost));
	return RRG_OK;
}

int rrg_cache_set_table(rrg_cache* h, const float* host) {
	RadianceCache* C = reinterpret_cast<RadianceCache*>(h);
	if (!C || !host || !C->table) return RRG_ERR_INVALID;
	RRG_CUDA(cudaMemcpy(C->table, host, sizeof(float) * C->table_floats, cudaMemcpyHostToDevice));
	return RRG_OK;
}

int rrg_cache_get_resolutions(const rrg_cache* h, float* res16) {
	const RadianceCache* C = reinterpret_cast<const RadianceCache*>(h);
	if (!C || !res16 || !C->table) return RRG_ERR_INVALID;
	for (int l = 0; l < kHashLevels; l++) res16[l] = C->hg.res[l];
	return RRG_OK;
}

void rrg_cache_destroy(rrg_cache* h) {
	RadianceCache* C = reinterpret_cast<RadianceCache*>(h);
	if (!C) return;
	cudaSetDevice(C->device);
	cudaDeviceSynchronize();
	free_cache(C);
}

int rrg_cache_set_weights(rrg_cache* h, const float* w_host) {
	RadianceCache* C = reinterpret_cast<RadianceCache*>(h);
	if (!C || !w_host) return RRG_ERR_INVALID;
	RRG_CUDA(cudaMemcpy(C->w, w_host, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice));
	return pack(C, nullptr);
}

int rrg_cache_get_weights(rrg_cache* h, float* w_host) {
	RadianceCache* C = reinterpret_cast<RadianceCache*>(h);
	if (!C || !w_host) return RRG_ERR_INVALID;
	RRG_CUDA(cudaMemcpy(w_host, C->w, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
	return RRG_OK;
}

int rrg_cache_set_adam(rrg_cache* h, float lr, float beta1, float beta2, float eps) {
	RadianceCache* C = reinterpret_cast<RadianceCache*>(h);
	if (!C || !(lr > 0.f)) return RRG_ERR_INVALID;
	C->lr = lr; C->b1 = beta1; C->b2 = beta2; C->eps = eps;
	return RRG_OK;
}

int rrg_cache_gradient(rrg_cache* h, const void* recs_host, uint32_t B, float* grad_host, float* loss_host,
                       float* pred_host) {
	return rrg_cache_gradient_ex(h, recs_host, B, grad_host, nullptr, loss_host, pred_host);
}

int rrg_cache_gradient_ex(rrg_cache* h, const void* recs_host, uint32_t B, float* grad_host, float* table_grad_host,
                          float* loss_host, float* pred_host) {
	RadianceCache* C = reinterpret_cast<RadianceCache*>(h);
	if (!C || !recs_host || !grad_host || B == 0 || B % kWgRows) return RRG_ERR_INVALID;
	if (table_grad_host && !C->table) return RRG_ERR_INVALID;
	if (C->tgrad) RRG_CUDA(cudaMemset(C->tgrad, 0, sizeof(float) * C->table_floats));
	CacheRec* d = nullptr;
	uint32_t* order = nullptr;
	float* pred = nullptr;
	RRG_CUDA(cudaMalloc(&d, sizeof(CacheRec) * B));
	RRG_CUDA(cudaMalloc(&order, sizeof(uint32_t) * B));
	RRG_CUDA(cudaMalloc(&pred, sizeof(float) * 3 * B));
	RRG_CUDA(cudaMemcpy(d, recs_host, sizeof(CacheRec) * B, cudaMemcpyHostToDevice));
	uint32_t* ho = new uint32_t[B];
	for (uint32_t i = 0; i < B; i++) ho[i] = i;
	cudaMemcpy(order, ho, sizeof(uint32_t) * B, cudaMemcpyHostToDevice);
	delete[] ho;
	RRG_CUDA(cudaMemset(C->buf.grad, 0, sizeof(float) * kMlpParams));
	RRG_CUDA(cudaMemset(C->buf.loss, 0, sizeof(float)));
	int st = fwd_bwd(C, d, B, B, 0, order, pred, nullptr);
	if (!st) {
		RRG_CUDA(cudaMemcpy(grad_host, C->buf.grad, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
		if (loss_host) RRG_CUDA(cudaMemcpy(loss_host, C->buf.loss, sizeof(float), cudaMemcpyDeviceToHost));
		if (pred_host) RRG_CUDA(cudaMemcpy(pred_host, pred, sizeof(float) * 3 * B, cudaMemcpyDeviceToHost));
		if (table_grad_host)
			RRG_CUDA(cudaMemcpy(table_grad_host, C->tgrad, sizeof(float) * C->table_floats, cudaMemcpyDeviceToHost));
		RRG_CUDA(cudaMemset(C->buf.grad, 0, sizeof(float) * kMlpParams));
		if (C->tgrad) RRG_CUDA(cudaMemset(C->tgrad, 0, sizeof(float) * C->table_floats));
	}
	cudaFree(d);
	cudaFree(order);
	cudaFree(pred);
	return st;
}

int rrg_cache_train(rrg_cache* h, const void* recs_dev, uint32_t nrec, uint32_t batch, uint32_t steps,
                    float* last_loss, void* stream) {
	RadianceCache* C = reinterpret_cast<RadianceCache*>(h);
	if (!C || !recs_dev || nrec == 0 || batch == 0 || batch % kWgRows) return RRG_ERR_INVALID;
	cudaStream_t s = (cudaStream_t)stream;
	for (uint32_t i = 0; i < steps; i++) {
		RRG_CUDA(cudaMemsetAsync(C->buf.loss, 0, sizeof(float), s));
		int st = fwd_bwd(C, reinterpret_cast<const CacheRec*>(recs_dev), nrec, batch, 0x5EEDull, nullptr, nullptr, s);
		if (st) return st;
		C->steps++;
		float c1 = 1.f - powf(C->b1, (float)C->steps), c2 = 1.f - powf(C->b2, (float)C->steps);
		rrg::note_launch(), k_mlp_adam<<<(kMlpParams + 255) / 256, 256, 0, s>>>(C->w, C->m, C->v, C->buf.grad, C->lr, C->b1, C->b2,
		                                                    C->eps, c1, c2);
		if (C->table)
			rrg::note_launch(), k_table_adam<<<C->num_sms * 8, 256, 0, s>>>(C->table, C->tm, C->tv, C->tgrad, C->table_floats, C->lr,
			                                           C->b1, C->b2, C->eps, c1, c2);
		st = pack(C, s);
		if (st) return st;
	}
	RRG_CUDA(cudaGetLastError());
	if (last_loss) {
		RRG_CUDA(cudaMemcpyAsync(last_loss, C->buf.loss, sizeof(float), cudaMemcpyDeviceToHost, s));
		RRG_CUDA(cudaStreamSynchronize(s));
	}
	return RRG_OK;
}

int rrg_cache_infer(rrg_cache* h, const void* recs_dev, uint64_t n, float* out_dev, void* stream) {
	return infer_impl(reinterpret_cast<RadianceCache*>(h), recs_dev, n, out_dev, 0, (cudaStream_t)stream);
}


uint64_t rrg_cache_steps(const rrg_cache* h) {
	const RadianceCache* C = reinterpret_cast<const RadianceCache*>(h);
	return C ? C->steps : 0;
}

}  // extern "C"
