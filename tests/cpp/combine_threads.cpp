// Native host threads calling rrg_intersect_rrray_one at once, the way the
// reference's OpenMP loops call RRCollider::intersect(RRRay&)
// (RRSolver/gather.cpp:917).  Used by tests/test_collider_gpu.py:
//   combine_threads <dir> <threads>
// reads <dir>/xyz.f32, <dir>/idx.u32, <dir>/rays.rrray (128-byte records),
// traces every record with one call per ray, thread t taking records
// t, t + threads, ..., and writes <dir>/out.rrray, <dir>/hit.u8 and one line
// "rays batches seconds" on stdout.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <thread>
#include <vector>

#include "rrgpu.h"

static std::vector<char> slurp(const std::string& path) {
	std::vector<char> b;
	FILE* f = fopen(path.c_str(), "rb");
	if (!f) return b;
	fseek(f, 0, SEEK_END);
	b.resize((size_t)ftell(f));
	fseek(f, 0, SEEK_SET);
	if (fread(b.data(), 1, b.size(), f) != b.size()) b.clear();
	fclose(f);
	return b;
}

int main(int argc, char** argv) {
	if (argc != 3) return 2;
	const std::string dir = argv[1];
	const int nthreads = atoi(argv[2]);
	std::vector<char> xyz = slurp(dir + "/xyz.f32"), idx = slurp(dir + "/idx.u32"), rays = slurp(dir + "/rays.rrray");
	if (xyz.empty() || idx.empty() || rays.empty() || nthreads < 1) return 3;
	rrg_collider* c = nullptr;
	int st = rrg_collider_create(reinterpret_cast<const float*>(xyz.data()), (uint32_t)(xyz.size() / 12),
	                             reinterpret_cast<const uint32_t*>(idx.data()), (uint32_t)(idx.size() / 12), nullptr,
	                             nullptr, 0, &c);
	if (st != RRG_OK) {
		fprintf(stderr, "create: %s\n", rrg_status_string(st));
		return 4;
	}
	const size_t n = rays.size() / 128;
	std::vector<unsigned char> hit(n, 0);
	std::vector<int> status(nthreads, RRG_OK);
	auto work = [&](int t) {
		for (size_t i = (size_t)t; i < n; i += (size_t)nthreads) {
			int s = rrg_intersect_rrray_one(c, rays.data() + 128 * i, &hit[i]);
			if (s != RRG_OK) status[t] = s;
		}
	};
	const auto t0 = std::chrono::steady_clock::now();
	std::vector<std::thread> pool;
	for (int t = 0; t < nthreads; t++) pool.emplace_back(work, t);
	for (auto& th : pool) th.join();
	const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
	for (int t = 0; t < nthreads; t++)
		if (status[t] != RRG_OK) {
			fprintf(stderr, "thread %d: %s\n", t, rrg_status_string(status[t]));
			return 5;
		}
	uint64_t batches = 0, traced = 0;
	rrg_collider_combined(c, &batches, &traced);
	FILE* f = fopen((dir + "/out.rrray").c_str(), "wb");
	FILE* g = fopen((dir + "/hit.u8").c_str(), "wb");
	if (!f || !g) return 6;
	fwrite(rays.data(), 1, rays.size(), f);
	fwrite(hit.data(), 1, hit.size(), g);
	fclose(f);
	fclose(g);
	printf("%llu %llu %.6f\n", (unsigned long long)traced, (unsigned long long)batches, secs);
	rrg_collider_destroy(c);
	return 0;
}
