// rrg_add_repeat.cuh -- k additions of one float value, each rounded to
// nearest even, in fewer dependent additions: the seam averaging of
// RRBuffer::lightmapSmooth (RRBuffer/RRBuffer.cpp:764-781) adds a run's
// texel sum once per edge sample, and the kernel (rrg_filter.cu) reproduces
// those sums bit for bit with this.  The header compiles as device code under
// nvcc and as plain C++ elsewhere, so the CPU tests check this same source
// against the loop of single additions (tests/test_add_repeat.py).
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define RRG_AR_FN __device__ __forceinline__
#define RRG_AR_ADD(a, b) __fadd_rn(a, b)
#define RRG_AR_BITS(x) __float_as_uint(x)
#define RRG_AR_FLOAT(u) __uint_as_float(u)
#ifndef RRG_AR_DIV
#define RRG_AR_DIV(a, b) __fdividef(a, b)
#endif
// float to unsigned, saturating (d == 0 gives 0 or 2^32 - 1, replaced below)
#define RRG_AR_QUOT(room, d) __float2uint_rz(RRG_AR_DIV((float)(room), (float)(d)))
#else
#include <string.h>
#define RRG_AR_FN static inline
// plain float addition: one rounding to nearest even (no contraction: no product)
static inline float rrg_ar_add(float a, float b) { return a + b; }
static inline uint32_t rrg_ar_bits(float x) {
	uint32_t u;
	memcpy(&u, &x, 4);
	return u;
}
static inline float rrg_ar_float(uint32_t u) {
	float x;
	memcpy(&x, &u, 4);
	return x;
}
#define RRG_AR_ADD(a, b) rrg_ar_add(a, b)
#define RRG_AR_BITS(x) rrg_ar_bits(x)
#define RRG_AR_FLOAT(u) rrg_ar_float(u)
#ifndef RRG_AR_DIV
#define RRG_AR_DIV(a, b) ((a) / (b))
#endif
// a quotient in [0, 2^23 + 1]: the conversion stays in range
#define RRG_AR_QUOT(room, d) ((uint32_t)RRG_AR_DIV((float)(room), (float)((d) ? (d) : 1u)))
#endif

namespace rrg {

// Plain additions before the closed form: an accumulator that starts at zero
// crosses a binade every few steps there, and one pass of the loop below
// costs about as much as a few dozen additions (timed on the config-2
// atlases, 256 of 256^2 texels: 1.99 s with 64 plain steps, 2.02-2.06 s with
// 32 or 48, 2.16 s with 16, 2.28 s with 8 and with none of the closed form).
constexpr uint32_t kPlainSteps = 64;

// x after k steps of x = x + v, each rounded to nearest even.  While the sums
// stay in one binade (one exponent, same sign) every step adds the same
// number d of units in the last place: v rounded to that spacing, and where v
// falls exactly half-way, the choice that keeps the significand even (so from
// a rounded, even significand the choice repeats).  So after three real steps
// inside one binade, the next n steps add n * d to the bit pattern, n as many
// as stay below the binade's top; then real steps cross into the next
// binade.  Zero and subnormal binades take the real steps.  The loop has no
// branch but its exit, as the 8 lanes that carry components run it together:
// the quotient room / d comes from a float division within one of the true
// one (RRG_AR_DIV) and is corrected with exact products.  `plain` sets how
// many of the k steps are plain additions first (an accumulator that already
// holds many additions of a like value needs none).
RRG_AR_FN float add_repeat(float x, float v, uint32_t k, uint32_t plain = kPlainSteps) {
	const uint32_t p = k < plain ? k : plain;
	for (uint32_t q = 0; q < p; q++) x = RRG_AR_ADD(x, v);
	k -= p;
	while (k >= 4u) {
		const float y = RRG_AR_ADD(x, v);
		const float z = RRG_AR_ADD(y, v);
		const float w = RRG_AR_ADD(z, v);
		k -= 3u;
		const uint32_t by = RRG_AR_BITS(y), bz = RRG_AR_BITS(z), bw = RRG_AR_BITS(w);
		const uint32_t e = bw >> 23;   // sign and exponent
		const bool same = (by >> 23) == e && (bz >> 23) == e && (e & 0xFFu) != 0u;
		const uint32_t d = bw - bz;
		const uint32_t room = 0x7FFFFFu - (bw & 0x7FFFFFu);
		uint32_t q = RRG_AR_QUOT(room, d);   // room < 2^23
		if ((uint64_t)q * d > room) q--;
		else if ((uint64_t)(q + 1u) * d <= room) q++;
		uint32_t n = d == 0u ? k : (q < k ? q : k);
		n = same ? n : 0u;
		x = RRG_AR_FLOAT(bw + n * d);
		k -= n;
	}
	for (; k; k--) x = RRG_AR_ADD(x, v);
	return x;
}

}  // namespace rrg
