// Compressed 8-wide BVH, collapsed on the device from the binary binned-SAH
// tree of rrg_build.cu.  The node format follows the idea of Ylitie,
// Karras and Laine, "Efficient Incoherent Ray Traversal on GPUs Through
// Compressed Wide BVHs" (HPG 2017): child boxes quantised to 8 bits on a
// per-node power-of-two grid, children ordered by ray octant so that a
// traversal needs no sort, and one stack entry per visited node.  The
// layout, the collapse (greedy: open the largest-area inner child until
// eight children) and the slot assignment (greedy on the octant-corner
// dot product) are this library's own; the format is in rrg_internal.cuh.
#include "rrg_internal.cuh"

#include <math.h>

namespace rrg {

namespace {

struct WideTask {
	int w;   // wide node index
	int b;   // binary build node it is made from
};

struct WideCounters {
	int nodes;    // wide nodes allocated
	int tris;     // wide triangle slots allocated
	int next;     // tasks of the next level
	int error;    // 1 = node budget exceeded, 2 = leaf too large, 4 = bad child
};

__device__ __forceinline__ float half_area_b(const BNode& n) {
	float e0 = n.hi[0] - n.lo[0], e1 = n.hi[1] - n.lo[1], e2 = n.hi[2] - n.lo[2];
	if (!(e0 >= 0.f)) return 0.f;
	return e0 * e1 + e1 * e2 + e2 * e0;
}

// the box widening of the binary emission (rrg_build.cu, widen())
__device__ __forceinline__ void widen_box(float* lo, float* hi, float pad) {
	for (int k = 0; k < 3; k++) {
		lo[k] = lo[k] - (fabsf(lo[k]) * 9.5367431640625e-07f + pad);
		hi[k] = hi[k] + (fabsf(hi[k]) * 9.5367431640625e-07f + pad);
	}
}

// smallest exponent x in [-126, 127] with ext <= 255 * 2^x
__device__ __forceinline__ int grid_exponent(float ext) {
	if (!(ext > 0.f)) return -126;
	int x;
	frexp((double)ext / 255.0, &x);   // ext/255 = m 2^x, m in [0.5, 1)
	while (x > -126 && (double)ext <= 255.0 * ldexp(1.0, x - 1)) x--;
	while ((double)ext > 255.0 * ldexp(1.0, x)) x++;
	return x < -126 ? -126 : (x > 127 ? 127 : x);
}

__global__ void k_wide_level(const BNode* __restrict__ bn, int nnodes, const WideTask* __restrict__ cur, int ncur,
                             WideTask* __restrict__ nxt, WideCounters* cnt, const float* __restrict__ pad_ptr,
                             const float4* __restrict__ tris_bin, int nvalid, uint4* __restrict__ wn, int max_wnodes,
                             float4* __restrict__ wtris) {
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= ncur) return;
	const WideTask task = cur[t];
	const float pad = *pad_ptr;
	int ch[8];
	int nch = 0;
	const BNode b = bn[task.b];
	if (b.left < 0) {
		if (b.count > 0) ch[nch++] = task.b;   // a root that is a leaf
	} else {
		ch[nch++] = b.left;
		ch[nch++] = b.right;
	}
	// open the inner child of largest surface area until there are eight
	while (nch < 8) {
		int best = -1;
		float ba = -1.f;
		for (int k = 0; k < nch; k++) {
			if (ch[k] < 0 || ch[k] >= nnodes) { atomicOr(&cnt->error, 4); return; }
			const BNode& c = bn[ch[k]];
			if (c.left >= 0) {
				float a = half_area_b(c);
				if (a > ba) { ba = a; best = k; }
			}
		}
		if (best < 0) break;
		const BNode c = bn[ch[best]];
		ch[best] = c.left;
		ch[nch++] = c.right;
	}
	float clo[8][3], chi[8][3];
	float plo[3] = {INFINITY, INFINITY, INFINITY}, phi[3] = {-INFINITY, -INFINITY, -INFINITY};
	bool inner[8];
	int count[8];
	for (int k = 0; k < nch; k++) {
		if (ch[k] < 0 || ch[k] >= nnodes) { atomicOr(&cnt->error, 4); return; }
		const BNode c = bn[ch[k]];
		inner[k] = c.left >= 0;
		count[k] = c.count;
		if (!inner[k] && (c.count < 1 || c.count > kWideLeafMax || c.begin < 0 || c.begin + c.count > nvalid)) {
			atomicOr(&cnt->error, 2);
			return;
		}
		for (int a = 0; a < 3; a++) { clo[k][a] = c.lo[a]; chi[k][a] = c.hi[a]; }
		widen_box(clo[k], chi[k], pad);
		for (int a = 0; a < 3; a++) { plo[a] = fminf(plo[a], clo[k][a]); phi[a] = fmaxf(phi[a], chi[k][a]); }
	}
	// slots: child most towards octant corner s goes to slot s (greedy)
	int child_in[8];
	for (int s = 0; s < 8; s++) child_in[s] = -1;
	{
		float cc[8][3];
		for (int k = 0; k < nch; k++)
			for (int a = 0; a < 3; a++)
				cc[k][a] = 0.5f * (clo[k][a] + chi[k][a]) - 0.5f * (plo[a] + phi[a]);
		unsigned used_c = 0, used_s = 0;
		for (int it = 0; it < nch; it++) {
			float best = -INFINITY;
			int bc = -1, bs = -1;
			for (int k = 0; k < nch; k++) {
				if (used_c >> k & 1) continue;
				for (int s = 0; s < 8; s++) {
					if (used_s >> s & 1) continue;
					float d = ((s & 1) ? cc[k][0] : -cc[k][0]) + ((s & 2) ? cc[k][1] : -cc[k][1]) +
					          ((s & 4) ? cc[k][2] : -cc[k][2]);
					if (d > best || bc < 0) { best = d; bc = k; bs = s; }
				}
			}
			used_c |= 1u << bc;
			used_s |= 1u << bs;
			child_in[bs] = bc;
		}
	}
	int nint = 0, ntri = 0;
	for (int k = 0; k < nch; k++) {
		if (inner[k]) nint++;
		else ntri += count[k];
	}
	const int child_base = nint ? atomicAdd(&cnt->nodes, nint) : 0;
	if (child_base + nint > max_wnodes) { atomicOr(&cnt->error, 1); return; }
	const int tri_base = ntri ? atomicAdd(&cnt->tris, ntri) : 0;
	if (tri_base + ntri > nvalid) { atomicOr(&cnt->error, 2); return; }
	const int next_base = nint ? atomicAdd(&cnt->next, nint) : 0;
	// grid
	int ex[3];
	double scale[3];
	for (int a = 0; a < 3; a++) {
		ex[a] = nch ? grid_exponent(phi[a] - plo[a]) : -126;
		scale[a] = ldexp(1.0, ex[a]);
	}
	uint32_t meta[2] = {0u, 0u};
	uint32_t q[6][2] = {{0u, 0u}, {0u, 0u}, {0u, 0u}, {0u, 0u}, {0u, 0u}, {0u, 0u}};
	uint32_t valid = 0;
	int k_int = 0, off = 0;
	for (int s = 0; s < 8; s++) {
		const int k = child_in[s];
		if (k < 0) continue;
		valid |= 1u << s;
		uint32_t m;
		if (inner[k]) {
			m = 0x80u | (uint32_t)k_int;
			nxt[next_base + k_int] = WideTask{child_base + k_int, ch[k]};
			k_int++;
		} else {
			m = ((uint32_t)(count[k] - 1) << 5) | (uint32_t)off;
			const BNode c = bn[ch[k]];
			for (int j = 0; j < count[k]; j++)
				for (int r = 0; r < 3; r++)
					wtris[3 * (size_t)(tri_base + off + j) + r] = tris_bin[3 * (size_t)(c.begin + j) + r];
			off += count[k];
		}
		meta[s >> 2] |= m << (8 * (s & 3));
		for (int a = 0; a < 3; a++) {
			const double p = (double)plo[a];
			double ql = floor(((double)clo[k][a] - p) / scale[a]);
			double qh = ceil(((double)chi[k][a] - p) / scale[a]);
			ql = ql < 0.0 ? 0.0 : (ql > 255.0 ? 255.0 : ql);
			qh = qh < 0.0 ? 0.0 : (qh > 255.0 ? 255.0 : qh);
			while (ql > 0.0 && p + ql * scale[a] > (double)clo[k][a]) ql -= 1.0;
			while (qh < 255.0 && p + qh * scale[a] < (double)chi[k][a]) qh += 1.0;
			q[a][s >> 2] |= (uint32_t)ql << (8 * (s & 3));
			q[3 + a][s >> 2] |= (uint32_t)qh << (8 * (s & 3));
		}
	}
	const uint32_t ebits = (uint32_t)(ex[0] + 127) | ((uint32_t)(ex[1] + 127) << 8) |
	                       ((uint32_t)(ex[2] + 127) << 16) | (valid << 24);
	uint4* o = wn + 5 * (size_t)task.w;
	o[0] = make_uint4(__float_as_uint(nch ? plo[0] : 0.f), __float_as_uint(nch ? plo[1] : 0.f),
	                  __float_as_uint(nch ? plo[2] : 0.f), ebits);
	o[1] = make_uint4((uint32_t)child_base, (uint32_t)tri_base, meta[0], meta[1]);
	o[2] = make_uint4(q[0][0], q[0][1], q[1][0], q[1][1]);
	o[3] = make_uint4(q[2][0], q[2][1], q[3][0], q[3][1]);
	o[4] = make_uint4(q[4][0], q[4][1], q[5][0], q[5][1]);
}

__global__ void k_wide_roots(WideTask* cur, int nroots, WideCounters* cnt) {
	int m = blockIdx.x * blockDim.x + threadIdx.x;
	if (m == 0) { cnt->nodes = nroots; cnt->tris = 0; cnt->next = 0; cnt->error = 0; }
	if (m < nroots) cur[m] = WideTask{m, m};
}

}  // namespace

int build_wide(Collider* c, const BNode* bnodes, int nnodes, const float* pad, cudaStream_t s) {
	const int nroots = (int)(c->d_tri_off ? c->nroots : 1);
	// every wide node is made from a distinct binary node
	int max_wnodes = nnodes < (int)kWideMaxNodes ? nnodes : (int)kWideMaxNodes;
	if (max_wnodes < nroots) return RRG_ERR_INVALID;
	WideTask *cur = nullptr, *nxt = nullptr;
	WideCounters* cnt = nullptr;
	uint4* wn = nullptr;
	float4* wt = nullptr;
	int st = RRG_OK;
	cudaError_t e = cudaMalloc(&cur, sizeof(WideTask) * (size_t)max_wnodes);
	if (e == cudaSuccess) e = cudaMalloc(&nxt, sizeof(WideTask) * (size_t)max_wnodes);
	if (e == cudaSuccess) e = cudaMalloc(&cnt, sizeof(WideCounters));
	if (e == cudaSuccess) e = cudaMalloc(&wn, sizeof(uint4) * 5 * (size_t)max_wnodes);
	if (e == cudaSuccess) e = cudaMalloc(&wt, sizeof(float4) * 3 * (size_t)c->nvalid);
	if (e != cudaSuccess) st = cuda_fail(e);
	int ncur = nroots;
	WideCounters h{};
	if (!st) {
		rrg::note_launch(), k_wide_roots<<<(nroots + 255) / 256, 256, 0, s>>>(cur, nroots, cnt);
		for (int level = 0; level < 128 && ncur > 0; level++) {
			e = cudaMemsetAsync(&cnt->next, 0, sizeof(int), s);
			if (e != cudaSuccess) { st = cuda_fail(e); break; }
			rrg::note_launch(), k_wide_level<<<(ncur + 127) / 128, 128, 0, s>>>(bnodes, nnodes, cur, ncur, nxt, cnt, pad, c->d_tris,
			                                               (int)c->nvalid, wn, max_wnodes, wt);
			e = cudaGetLastError();
			if (e == cudaSuccess) e = cudaMemcpyAsync(&h, cnt, sizeof(h), cudaMemcpyDeviceToHost, s);
			if (e == cudaSuccess) e = cudaStreamSynchronize(s);
			if (e != cudaSuccess) { st = cuda_fail(e); break; }
			if (h.error) { st = RRG_ERR_INVALID; break; }
			ncur = h.next;
			WideTask* tmp = cur;
			cur = nxt;
			nxt = tmp;
		}
		if (!st && (ncur > 0 || h.tris != (int)c->nvalid)) st = RRG_ERR_INVALID;
	}
	cudaFree(cur);
	cudaFree(nxt);
	cudaFree(cnt);
	if (st) {
		cudaFree(wn);
		cudaFree(wt);
		return st;
	}
	// keep only the nodes in use
	uint4* fit = nullptr;
	if (cudaMalloc(&fit, sizeof(uint4) * 5 * (size_t)h.nodes) == cudaSuccess &&
	    cudaMemcpyAsync(fit, wn, sizeof(uint4) * 5 * (size_t)h.nodes, cudaMemcpyDeviceToDevice, s) == cudaSuccess &&
	    cudaStreamSynchronize(s) == cudaSuccess) {
		cudaFree(wn);
		wn = fit;
	} else {
		cudaFree(fit);
		cudaGetLastError();
	}
	cudaFree(c->d_wnodes);
	cudaFree(c->d_wtris);
	c->d_wnodes = wn;
	c->d_wtris = wt;
	c->nwnodes = (uint32_t)h.nodes;
	return RRG_OK;
}

}  // namespace rrg
