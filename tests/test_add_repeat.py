"""The closed form of repeated rounded additions used by the seam averaging
(lightsprintsdk_gb300/csrc/rrg_add_repeat.cuh, RRBuffer.cpp:764-781 adds a
run's texel sum once per edge sample): the same header compiled as C++ on
the CPU, against the loop of single float additions, bit for bit, over
random accumulators and values (ties to even, sums crossing many binades,
negative values, zeros, subnormals, infinities and NaN; the default and
random numbers of leading plain additions), once with the exact
quotient and once with a quotient perturbed by up to one (the kernel's
approximate division), which the correction must absorb."""
import os
import shutil
import subprocess

import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "lightsprintsdk_gb300", "csrc")

DRIVER = r"""
#include <stdio.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
static uint64_t g_s = 88172645463325252ull;
static uint64_t rnd() { g_s ^= g_s << 13; g_s ^= g_s >> 7; g_s ^= g_s << 17; return g_s; }
#ifdef PERTURB
// a quotient off by up to one either way, as an approximate division may be
static float perturbed_div(float a, float b) {
	const float q = a / b;
	const int r = (int)(rnd() % 3) - 1;
	const float p = q + (float)r * ((rnd() & 1) ? 1.0f : 0.999f);
	return p > 0.f ? p : 0.f;
}
#define RRG_AR_DIV(a, b) perturbed_div(a, b)
#endif
#include "rrg_add_repeat.cuh"
static inline uint32_t fb(float x) { uint32_t u; memcpy(&u, &x, 4); return u; }
static inline float bf(uint32_t u) { float x; memcpy(&x, &u, 4); return x; }
static float add_loop(float x, float v, uint32_t k) { while (k--) { volatile float r = x + v; x = r; } return x; }
int main(int argc, char** argv) {
	const long cases = argc > 1 ? strtol(argv[1], 0, 10) : 1000000;
	long bad = 0, n = 0;
	for (long it = 0; it < cases; it++) {
		float x, v;
		const int mode = (int)(rnd() % 8);
		v = bf(((uint32_t)(rnd() % 60 + 100) << 23) | (uint32_t)(rnd() & 0x7FFFFF));
		if (mode == 0) x = 0.f;                                            // a fresh accumulator
		else if (mode == 1) x = v * (float)(rnd() % 2000);                 // a running sum
		else if (mode == 2) {                                              // few significant bits: ties
			v = bf(fb(v) & 0xFFFF0000u);
			x = bf((fb(v) + ((uint32_t)(rnd() % 12) << 23)) | (uint32_t)(rnd() & 0x7FFFFF));
		} else if (mode == 3) {
			v = bf(fb(v) & 0xFFFFFFF0u);
			x = bf(fb(v) + ((uint32_t)(rnd() % 24) << 23) + (uint32_t)(rnd() & 0xFF));
		} else if (mode == 4) { v = 2.f; x = (float)(2 * (rnd() % 3000)); }  // an alpha sum
		else if (mode == 5) x = bf((fb(v) + ((uint32_t)(rnd() % 30) << 23)) | 0x7FFF00u);  // near a binade's top
		else if (mode == 6) { x = -bf(fb(v) + ((uint32_t)(rnd() % 5) << 23)); if (rnd() & 1) v = -v; }
		else { v = bf((uint32_t)(rnd() % 0x7F800000u)); x = bf((uint32_t)(rnd() % 0x7F800000u)); }
		const uint32_t k = (uint32_t)(rnd() % 1200);
		const uint32_t plain = (it & 1) ? rrg::kPlainSteps : (uint32_t)(rnd() % 80);   // leading plain additions
		const float a = add_loop(x, v, k), b = rrg::add_repeat(x, v, k, plain);
		n++;
		if (fb(a) != fb(b)) {
			if (bad < 5) printf("mismatch x=%a v=%a k=%u loop=%a closed=%a\n", x, v, k, a, b);
			bad++;
		}
	}
	const float inf = 1.f / 0.f;
	const float sp[] = {0.f, -0.f, 1e-40f, -1e-40f, inf, -inf, 3.4e38f, -3.4e38f, 1.17549435e-38f, inf - inf};
	for (int i = 0; i < 10; i++)
		for (int j = 0; j < 10; j++)
			for (uint32_t k = 0; k < 200; k += 1 + k / 8) {
				const float a = add_loop(sp[i], sp[j], k), b = rrg::add_repeat(sp[i], sp[j], k);
				n++;
				if (fb(a) != fb(b) && !(a != a && b != b)) {
					if (bad < 10) printf("special mismatch x=%a v=%a k=%u loop=%a closed=%a\n", sp[i], sp[j], k, a, b);
					bad++;
				}
			}
	printf("%ld cases, %ld mismatches\n", n, bad);
	return bad != 0;
}
"""


@pytest.mark.parametrize("perturb", [False, True])
def test_add_repeat_equals_single_additions(tmp_path, perturb):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    src = tmp_path / "drv.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "drv"
    cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I", CSRC, str(src), "-o", str(exe)]
    if perturb:
        cmd.insert(1, "-DPERTURB")
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe), "1500000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:]
    assert "0 mismatches" in r.stdout
