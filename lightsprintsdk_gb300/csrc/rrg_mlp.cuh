// Radiance-cache network on BF16 tensor cores (FP32 accumulation).
//
// The network and its loss are specified in oracle/rr_mlp.c (the FP64
// oracle the gradients are checked against):
//   x(64) -> relu(W1) 64 -> relu(W2) 64 -> relu(W3) 64 -> relu(W4) 64 -> W5 -> 16 (RGB = first 3)
// Weights live in three forms: FP32 masters (row = input, column = output,
// layer after layer, 17,408 floats) updated by Adam, and two BF16 copies
// pre-arranged in the register-fragment order of mma.m16n8k16: W for the
// forward pass and W^T for back-propagation.  A warp computes 16 samples at
// a time; a layer's FP32 accumulator fragments become the next layer's BF16
// A fragments without leaving registers (the C layout of two adjacent
// n-tiles is the A layout of one k-tile).
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace rrg {

constexpr int kMlpIn = 64;
constexpr int kMlpOut = 16;
constexpr int kMlpParams = 4 * 64 * 64 + 64 * 16;     // 17,408
constexpr int kMlpFragWords = 4 * (4 * 8 * 32 * 2) + 4 * 2 * 32 * 2;   // 8,704 uint32 (fwd); bwd same

__host__ __device__ constexpr int mlp_layer_off(int l) { return l * 4096; }
__host__ __device__ constexpr int mlp_layer_out(int l) { return l < 4 ? 64 : 16; }
// fragment word offset of layer l (forward: K = 64 in, N = out; backward: K = out, N = 64 in)
__host__ __device__ constexpr int mlp_frag_off(int l) { return l * 2048; }

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
	__nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
	return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float bf16_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }

// D += A(16x16, row) * B(16x8, col); bf16 in, fp32 accumulate
__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
	asm volatile(
	    "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
	    "{%0,%1,%2,%3};\n"
	    : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
	    : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// C fragments of n-tiles 2kt, 2kt+1 (after relu when RELU) -> A fragment of k-tile kt
template <bool RELU>
__device__ __forceinline__ void c_to_a(const float* c0, const float* c1, uint32_t* a) {
	auto f = [](float x) { return RELU ? fmaxf(x, 0.f) : x; };
	a[0] = pack_bf16(f(c0[0]), f(c0[1]));
	a[1] = pack_bf16(f(c0[2]), f(c0[3]));
	a[2] = pack_bf16(f(c1[0]), f(c1[1]));
	a[3] = pack_bf16(f(c1[2]), f(c1[3]));
}

// A fragments of a 16 x 64 bf16 row-major tile (row stride in uint32 words)
__device__ __forceinline__ void load_a(const uint32_t* tile, int stride_words, int kt, uint32_t* a) {
	const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
	a[0] = tile[g * stride_words + 8 * kt + q];
	a[1] = tile[(g + 8) * stride_words + 8 * kt + q];
	a[2] = tile[g * stride_words + 8 * kt + 4 + q];
	a[3] = tile[(g + 8) * stride_words + 8 * kt + 4 + q];
}

// One 64-input layer on 4 A k-tiles; NT n-tiles of B fragments at frag.
template <int NT>
__device__ __forceinline__ void mlp_layer(const uint32_t (*a)[4], const uint32_t* __restrict__ frag, float (*acc)[4]) {
	const int lane = threadIdx.x & 31;
#pragma unroll
	for (int nt = 0; nt < NT; nt++) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll
	for (int kt = 0; kt < 4; kt++) {
#pragma unroll
		for (int nt = 0; nt < NT; nt++) {
			const uint2 b = *reinterpret_cast<const uint2*>(frag + ((kt * NT + nt) * 32 + lane) * 2);
			mma16816(acc[nt], a[kt], b.x, b.y);
		}
	}
}

// Forward of one 16-row tile: x = A fragments of the encoded inputs.
// Leaves the 16 x 16 output in out (C layout, 2 n-tiles).
__device__ __forceinline__ void mlp_forward_tile(const uint32_t (*x)[4], const uint32_t* __restrict__ fwd,
                                                 float (*out)[4]) {
	uint32_t a[4][4];
	float acc[8][4];
#pragma unroll
	for (int kt = 0; kt < 4; kt++)
#pragma unroll
		for (int r = 0; r < 4; r++) a[kt][r] = x[kt][r];
#pragma unroll
	for (int l = 0; l < 4; l++) {
		mlp_layer<8>(a, fwd + mlp_frag_off(l), acc);
#pragma unroll
		for (int kt = 0; kt < 4; kt++) c_to_a<true>(acc[2 * kt], acc[2 * kt + 1], a[kt]);
	}
	mlp_layer<2>(a, fwd + mlp_frag_off(4), out);
}

// Frequency encoding of one sample into 64 bf16 features (see oracle/rr_mlp.c);
// `half` 0 writes words 0..15 (features 0..31), 1 words 16..31.
__device__ __forceinline__ void mlp_encode_half(const float* p, const float* n, const float* alb, const float* lo,
                                                const float* inv_ext, int half, uint32_t* row_words) {
	if (half == 0) {
#pragma unroll
		for (int j = 0; j < 2; j++) {
			float u = fminf(fmaxf((p[j] - lo[j]) * inv_ext[j], 0.f), 1.f);
#pragma unroll
			for (int k = 0; k < 8; k++) {
				float s, c;
				sincospif((float)(1 << k) * u, &s, &c);
				row_words[8 * j + k] = pack_bf16(s, c);
			}
		}
	} else {
		float u = fminf(fmaxf((p[2] - lo[2]) * inv_ext[2], 0.f), 1.f);
#pragma unroll
		for (int k = 0; k < 8; k++) {
			float s, c;
			sincospif((float)(1 << k) * u, &s, &c);
			row_words[16 + k] = pack_bf16(s, c);
		}
		row_words[24] = pack_bf16(n[0], n[1]);
		row_words[25] = pack_bf16(n[2], alb[0]);
		row_words[26] = pack_bf16(alb[1], alb[2]);
		row_words[27] = pack_bf16(1.f, 0.f);
		row_words[28] = 0u;
		row_words[29] = 0u;
		row_words[30] = 0u;
		row_words[31] = 0u;
	}
}

// Sample record shared by training and inference: position, normal, albedo,
// and the target (training) or a validity flag in w (inference).
struct CacheRec {
	float p[3], n[3], alb[3], t[3];
};

// ------------------------------------------------------ hash-grid encoding
// Multiresolution hash encoding (specified in oracle/rr_mlp.c): 16 levels x
// 2 features from trilinearly interpolated table entries, 4 octaves of
// frequency encoding, normal, albedo, bias.  table == nullptr selects the
// frequency encoding above.
constexpr int kHashLevels = 16;

struct HashGrid {
	const float2* table;   // kHashLevels x T entries of 2 features
	float* tgrad;          // same layout, gradient (training only)
	uint32_t T;            // entries per level (power of two)
	uint32_t dense;        // bit l: level l indexed densely ((res+1)^3 <= T)
	float res[kHashLevels];
};

// Corner c (0..7) of level l: table index (within the level) and weight.
struct HashCorners {
	uint32_t x0[3];
	float w[3];
};

// the position scaled to the cache box and clamped to [0, 1]
__device__ __forceinline__ float hash_unit(float p, float lo, float ie) {
	return fminf(fmaxf(__fmul_rn(__fsub_rn(p, lo), ie), 0.f), 1.f);
}

__device__ __forceinline__ HashCorners hash_cell_u(const float* u, float res) {
	HashCorners h;
	const int n = (int)res;
#pragma unroll
	for (int j = 0; j < 3; j++) {
		float x = __fmul_rn(u[j], res);
		int f = (int)floorf(x);
		f = f < 0 ? 0 : (f > n - 1 ? n - 1 : f);
		h.x0[j] = (uint32_t)f;
		h.w[j] = __fsub_rn(x, (float)f);
	}
	return h;
}

__device__ __forceinline__ HashCorners hash_cell(const float* p, const float* lo, const float* ie, float res) {
	const float u[3] = {hash_unit(p[0], lo[0], ie[0]), hash_unit(p[1], lo[1], ie[1]), hash_unit(p[2], lo[2], ie[2])};
	return hash_cell_u(u, res);
}

// index within a level: dense levels ((res+1)^3 <= T) by position, the
// others by the spatial hash
__device__ __forceinline__ uint32_t hash_index_r(bool dense, float res, uint32_t T, uint32_t ix, uint32_t iy,
                                                 uint32_t iz) {
	if (dense) {
		const uint32_t n1 = (uint32_t)res + 1u;
		return ix + iy * n1 + iz * n1 * n1;
	}
	return (ix ^ (iy * 2654435761u) ^ (iz * 805459861u)) & (T - 1u);
}

__device__ __forceinline__ uint32_t hash_index(const HashGrid& g, int l, uint32_t ix, uint32_t iy, uint32_t iz) {
	return hash_index_r((g.dense >> l) & 1u, g.res[l], g.T, ix, iy, iz);
}

__device__ __forceinline__ float hash_weight(const HashCorners& h, int c) {
	const float wx = (c & 1) ? h.w[0] : __fsub_rn(1.f, h.w[0]);
	const float wy = (c & 2) ? h.w[1] : __fsub_rn(1.f, h.w[1]);
	const float wz = (c & 4) ? h.w[2] : __fsub_rn(1.f, h.w[2]);
	return __fmul_rn(__fmul_rn(wx, wy), wz);
}

// Encoding with the hash grid, split evenly between the two lanes of a
// sample: `half` 0 writes the even levels' feature pairs (words 0, 2, .., 14)
// and the x and y octaves (words 16..23), `half` 1 the odd levels' (words 1,
// 3, .., 15), the z octaves (24..27), normal, albedo and bias (28..31).  Each
// lane's eight levels are unrolled so their 64 table reads are in flight
// together; the level's resolution is picked from two kernel-parameter
// constants (no indexed parameter array, which would live in local memory).
__device__ __forceinline__ void mlp_encode_half_hash(const float* p, const float* n, const float* alb,
                                                     const float* lo, const float* ie, const HashGrid& g, int half,
                                                     uint32_t* row_words) {
	const float u[3] = {hash_unit(p[0], lo[0], ie[0]), hash_unit(p[1], lo[1], ie[1]), hash_unit(p[2], lo[2], ie[2])};
#pragma unroll
	for (int i = 0; i < kHashLevels / 2; i++) {
		const int l = 2 * i + half;
		const float res = half ? g.res[2 * i + 1] : g.res[2 * i];
		const HashCorners h = hash_cell_u(u, res);
		const float2* tl = g.table + (size_t)l * g.T;
		const bool dense = (g.dense >> l) & 1u;
		float f0 = 0.f, f1 = 0.f;
#pragma unroll
		for (int c = 0; c < 8; c++) {
			const uint32_t idx = hash_index_r(dense, res, g.T, h.x0[0] + (c & 1), h.x0[1] + ((c >> 1) & 1),
			                                  h.x0[2] + ((c >> 2) & 1));
			const float wc = hash_weight(h, c);
			const float2 e = __ldg(tl + idx);
			f0 = fmaf(wc, e.x, f0);
			f1 = fmaf(wc, e.y, f1);
		}
		row_words[l] = pack_bf16(f0, f1);
	}
	const int j0 = half ? 2 : 0, j1 = half ? 3 : 2;
	for (int j = j0; j < j1; j++) {
#pragma unroll
		for (int k = 0; k < 4; k++) {
			float s, c;
			sincospif((float)(1 << k) * u[j], &s, &c);
			row_words[16 + 4 * j + k] = pack_bf16(s, c);
		}
	}
	if (half) {
		row_words[28] = pack_bf16(n[0], n[1]);
		row_words[29] = pack_bf16(n[2], alb[0]);
		row_words[30] = pack_bf16(alb[1], alb[2]);
		row_words[31] = pack_bf16(1.f, 0.f);
	}
}

// Scatter of the input gradient of level l's two features for one sample
// to the 8 corners (atomics; the table gradient is zeroed by the optimiser).
__device__ __forceinline__ void hash_backward(const float* p, const float* lo, const float* ie, const HashGrid& g,
                                              int l, float d0, float d1) {
	const HashCorners h = hash_cell(p, lo, ie, g.res[l]);
	// the entry's two features are adjacent: one 8-byte atomic for both
	float2* tl = reinterpret_cast<float2*>(g.tgrad + (size_t)l * g.T * 2);
#pragma unroll
	for (int c = 0; c < 8; c++) {
		const uint32_t idx = hash_index(g, l, h.x0[0] + (c & 1), h.x0[1] + ((c >> 1) & 1), h.x0[2] + ((c >> 2) & 1));
		const float wc = hash_weight(h, c);
		atomicAdd(tl + idx, make_float2(wc * d0, wc * d1));
	}
}

}  // namespace rrg

typedef struct rrg_cache rrg_cache;
namespace rrg {
// The cache's reliability grid (res^3 cells over its box; null if not built).
void cache_grid(rrg_cache* c, const uint8_t** flags, int* res, float* lo, float* ie);

}  // namespace rrg
