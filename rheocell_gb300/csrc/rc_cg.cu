// Viscous solve of the wet models on the device: matrix-free, Jacobi-
// preconditioned conjugate gradient for both velocity components at once.
//
// Reference: WetModel::begin_energy_computation assembles, per velocity
// component, the SPD system over the stacked patch sites (WetModel.cpp:279-347;
// WetPolarModel.cpp:309-337) and solves it with
// Eigen::ConjugateGradient<SparseMatrix<double>, Upper> (:361-376).  The
// operator is
//     (A v)_j = (xi + eta * D_j) v_j - eta * sum_{k' in N4(k_j)} sum_{i covers k'} v_i
// with k_j the box site of patch site j, N4 the four box neighbours and
// D_j = sum_{k' in N4(k_j)} n(k') the patches covering them.  It is applied
// here without assembling it: a box-grid sum P = S p over the cover lists, a
// four-neighbour sum of P, and a per-site diagonal.  The diagonal is formed as
// the reference's triplet sum (xi, then +eta once per covering patch site), so
// it and the Jacobi preconditioner 1/diag are bit-identical.
//
// The iteration follows Eigen's ConjugateGradient step for step: r = b - A x
// (x = 0 on a cold start), threshold max(tol^2 |b|^2, DBL_MIN), p = M^-1 r,
// then alpha = r.z / p.Ap, x += alpha p, r -= alpha Ap, stop when |r|^2 <
// threshold, beta = r'.z' / r.z, p = z' + beta p; at most 2n iterations.  The
// x and y systems share the operator and run in the same sweep, each with its
// own scalars and its own stopping point, which gives the same iterates as two
// sequential solves.
//
// The solve is one persistent cooperative kernel: every phase is a grid-stride
// loop, and phases are separated by a grid barrier.  Barrier waits are bounded;
// on timeout the kernel records ERR_BARRIER and returns.  Dot products are
// summed in a fixed order (per-block tree, then every block sums the block
// partials in block order), so results are bit-reproducible.
#include "rc_kernels.cuh"

#include <float.h>

namespace rc {

constexpr int CG_THREADS = 512;
constexpr int CG_MAX_D = 4 * STORE_MAX;
constexpr long long BARRIER_SPIN_LIMIT = 4000000;  // about 1-2 s with 64 ns naps

// Scalars block (global): [0..7] reduction results.
enum { SC_RED = 0 };

__device__ __forceinline__ double ldcg(const double *p) { return __ldcg(p); }

struct CGShared {
	double T[CG_MAX_D + 1], iT[CG_MAX_D + 1];
	double red[8 * (CG_THREADS / 32 + 1)];  // block_sum<8> scratch
	double tot[8];
	double rz[2], thr[2], bn2[2], rn2[2], alpha[2], beta[2];
	double pap[2], scale[2];  // learned path: p.Ap of the sweep, residual scale
	float Tf[CG_MAX_D + 1], iTf[CG_MAX_D + 1];  // FP32 copies of T, 1/T (learned path)
	int act[2], it[2], first, zero[2];
	int site_first, site_step, site_end;  // by-site phases: this block's box sites
	int hbase, hm;            // harvesting: first slot of this solve, points taken
	long long jlo, S;         // this solve's unknowns [jlo, jlo + S) (a member's, for ensembles)
	int cold;                 // cold start
	unsigned long long tmark; // diagnostic phase timers: last mark (block 0, thread 0)
	unsigned epoch;           // grid barriers passed (the same count in every block)
	int fail;                 // a barrier wait ran out (sticky)
};

// Grid-wide barrier with an optional fixed-order reduction of nv <= 8
// doubles.  v[i] holds this block's partial sums (valid in thread 0); on
// return sh.tot[i] holds the grid totals.  Every block arrives once on a
// monotonic counter (a.bar[0], zero at launch) and waits for it to reach
// (barriers passed + 1) * blocks; then every block sums the partials itself,
// in block order, so all blocks obtain the same, reproducible totals.  The
// partials alternate between two buffers by barrier parity, so a block that
// runs ahead never overwrites sums another block is still reading.  Returns
// false if the wait ran out (then ERR_BARRIER is set).
__device__ __forceinline__ bool grid_reduce(const CGArgs &a, CGShared &sh, int nv, const double *v) {
	const unsigned nb = gridDim.x;
	__syncthreads();  // the whole block's writes of this phase precede the arrival
	if(threadIdx.x == 0) {
		const unsigned e = sh.epoch;
		double *part = a.partials + (size_t) (e & 1u) * 8 * nb;
		for(int i = 0; i < nv; i++) part[(size_t) i * nb + blockIdx.x] = v[i];
		const unsigned target = (e + 1u) * nb + (e == 0u ? (unsigned) a.barrier_extra : 0u);
		const long long limit = a.spin_limit > 0 ? a.spin_limit : BARRIER_SPIN_LIMIT;
		__threadfence();
		atomicAdd(&a.bar[0], 1u);
		long long spins = 0;
		unsigned c;
		while(true) {
			asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(c) : "l"(a.bar) : "memory");
			if((int) (c - target) >= 0) break;
			if(++spins > limit) {
				atomicOr(&a.st->err, ERR_BARRIER);
				sh.fail = 1;
				break;
			}
			__nanosleep(20);
		}
		sh.epoch = e + 1u;
	}
	__syncthreads();
	if(nv > 0) {
		// one warp: lane l sums partials l, l + 32, ... in order, then a fixed
		// shuffle tree (FP64 warp instructions are expensive on GB300: no
		// other warp repeats this work)
		if(threadIdx.x < 32) {
			const double *part = a.partials + (size_t) ((sh.epoch - 1u) & 1u) * 8 * nb;
			const int lane = threadIdx.x;
#pragma unroll
			for(int i = 0; i < 8; i++) {
				if(i >= nv) break;
				double t = 0.0;
				for(unsigned b = lane; b < nb; b += 32) t += ldcg(&part[(size_t) i * nb + b]);
#pragma unroll
				for(int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
				if(lane == 0) sh.tot[i] = t;
			}
		}
		__syncthreads();
	}
	return !sh.fail;
}

__device__ __forceinline__ int box_deg(const int *cnt, int k, int L) {
	const int x = k % L, y = k / L;
	const int kr = (x == L - 1) ? k - (L - 1) : k + 1;
	const int kl = (x == 0) ? k + (L - 1) : k - 1;
	const int ku = (y == L - 1) ? k - (L - 1) * L : k + L;
	const int kd = (y == 0) ? k + (L - 1) * L : k - L;
	return cnt[kd] + cnt[kl] + cnt[kr] + cnt[ku];
}

template<typename T>
__device__ __forceinline__ double box_n4(const T *P, int k, int L) {
	const int x = k % L, y = k / L;
	const int kr = (x == L - 1) ? k - (L - 1) : k + 1;
	const int kl = (x == 0) ? k + (L - 1) : k - 1;
	const int ku = (y == L - 1) ? k - (L - 1) * L : k + L;
	const int kd = (y == 0) ? k + (L - 1) * L : k - L;
	return (double) P[kd] + (double) P[kl] + (double) P[kr] + (double) P[ku];
}


__device__ __forceinline__ unsigned long long gtimer() {
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

// Diagnostic phase timers: block 0's thread 0 charges the time since the
// previous mark (including its wait at the barrier that ended the phase) to
// phase k.  Phases: 0 refinement update and true residual before a flexible
// CG run, 1 first layer, 2-4 tensor-core layers of levels 0-2, 5 last layer
// (all network layers when the network runs in FP32), 6 flexible CG phase E,
// 7 phase AB, 8 start of a solve (cover lists, first true residual), 9 phase
// C, 10 everything else.
enum { PH_INIT, PH_E0A, PH_TC0, PH_TC1, PH_TC2, PH_OUT, PH_Z, PH_AB, PH_START, PH_C, PH_OTHER, PH_COUNT };
__device__ __forceinline__ void pmark(const CGArgs &a, CGShared &sh, int k) {
	if(a.phase_ns && blockIdx.x == 0 && threadIdx.x == 0) {
		const unsigned long long t = gtimer();
		a.phase_ns[k] += t - sh.tmark;
		sh.tmark = t;
	}
}

// Cover lists in CSR form for this solve: cov_off[k] = sum of n over box
// sites before k, cov_idx[cov_off[k] + i] = cover[i][k] (unknowns covering k,
// in cell order).  Block b scans the contiguous box range it owns; the block
// totals meet through one grid barrier.
__device__ __forceinline__ bool build_csr(const CGArgs &a, CGShared &sh) {
	const long long L2 = (long long) a.L * a.L;
	const long long chunk = (L2 + gridDim.x - 1) / gridDim.x;
	const long long lo = blockIdx.x * chunk, hi = min(L2, lo + chunk);
	__shared__ int s_scan[CG_THREADS];
	__shared__ long long s_base;
	// per-thread contiguous sub-range of the block's range
	const long long per = (chunk + blockDim.x - 1) / blockDim.x;
	const long long tlo = min(hi, lo + threadIdx.x * per), thi = min(hi, tlo + per);
	int tsum = 0;
	for(long long k = tlo; k < thi; k++) tsum += a.cnt[k];
	s_scan[threadIdx.x] = tsum;
	__syncthreads();
	for(int o = 1; o < (int) blockDim.x; o <<= 1) {
		const int add = (threadIdx.x >= (unsigned) o) ? s_scan[threadIdx.x - o] : 0;
		__syncthreads();
		s_scan[threadIdx.x] += add;
		__syncthreads();
	}
	const int block_total = s_scan[blockDim.x - 1];
	double v[1] = {(double) block_total};
	if(threadIdx.x == 0) a.partials[(size_t) 7 * gridDim.x + blockIdx.x] = v[0];
	if(!grid_reduce(a, sh, 0, nullptr)) return false;
	{
		double acc[1] = {0.0};
		for(unsigned b = threadIdx.x; b < blockIdx.x; b += blockDim.x) acc[0] += ldcg(&a.partials[(size_t) 7 * gridDim.x + b]);
		block_sum<1>(acc, sh.red);
		if(threadIdx.x == 0) s_base = (long long) acc[0];
		__syncthreads();
	}
	long long off = s_base + s_scan[threadIdx.x] - tsum;
	for(long long k = tlo; k < thi; k++) {
		const int n = a.cnt[k];
		a.cov_off[k] = (int) off;
		for(int i = 0; i < n; i++) a.cov_idx[off + i] = a.cover[(size_t) i * L2 + k];
		off += n;
	}
	if(blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) a.cov_off[L2] = (int) off;
	return grid_reduce(a, sh, 0, nullptr);
}

// Warp-segmented sum of v over consecutive lanes with equal key (keys sorted
// within the warp); returns the segment's partial sum in its last lane of
// this warp (others: unused), and whether this lane is that tail.
template<typename T>
__device__ __forceinline__ T seg_sum(T v, int key, bool &tail) {
	const int lane = threadIdx.x & 31;
#pragma unroll
	for(int d = 1; d < 32; d <<= 1) {
		const T u = __shfl_up_sync(0xffffffffu, v, d);
		const int kd = __shfl_up_sync(0xffffffffu, key, d);
		if(lane >= d && kd == key) v += u;
	}
	const int kn = __shfl_down_sync(0xffffffffu, key, 1);
	tail = (lane == 31) || (kn != key);
	return v;
}

// W(k) = n(k) / T(k), the network's second input channel.
__device__ __forceinline__ float box_w(const CGArgs &a, const CGShared &sh, int k, int L) {
	const int n = a.cnt[k];
	return n ? (float) ((double) n * sh.iT[box_deg(a.cnt, k, L)]) : 0.f;
}

// FP32 copies of the residual made by true_residual.
enum { RES_FP64 = 0, RES_FLOAT_COVER = 1 };

// r = b - A x for both components (x = 0 when `x_zero`), written in FP64,
// by box site: thread k forms the box sums of x at k (first pass), then the
// four-neighbour sum and the diagonal once for the unknowns covering k.
// fmode RES_FLOAT_COVER also rounds r to FP32 and clears the correction,
// both in cover order (rxf[e], exf[e] for cov_idx[e] = j; the flexible CG's
// layout), and writes the network input of
// its first application: x0 = (sum over the unknowns at k of r / T, W(k))
// per component, unscaled.  Reduces |b|^2, |r|^2 and r.M^-1 r (the latter
// on the stored precision of r) into sh.tot[0..5], each thread's partial
// sums in box-site order, so the totals are reproducible.
// want_b: also |b|^2 (needed once per solve); want_rz: also r.M^-1 r (not
// needed by the flexible CG, which forms its own).  Unrequested sums are 0.
// GB300 issues FP64 at a small fraction of the FP32 rate, so the residual
// does no FP64 work it does not need.
// add_e: first x += e, the FP32 correction of the last refinement sweep
// (exf/eyf, in cover order; RES_FLOAT_COVER only), fused into the pass that
// forms the box sums of x.
// NB: unknowns of a site whose index and value loads are issued together
// (one dependent load chain per NB unknowns instead of per unknown); the
// arithmetic runs unknown by unknown in cover order whatever NB is, so the
// result does not depend on it.
template<int fmode, int NB = 1>
__device__ __forceinline__ bool true_residual(const CGArgs &a, CGShared &sh, bool x_zero, bool want_b = true, bool want_rz = true,
                                              bool add_e = false) {
	const int L = a.L;
	const long long L2 = (long long) L * L;
	const double neta = -a.eta * 1.0;
	const long long gtid = blockIdx.x * (long long) blockDim.x + threadIdx.x;
	const long long gstride = (long long) gridDim.x * blockDim.x;
	const int *cov_idx = a.cov_idx, *cov_off = a.cov_off;
	if(!x_zero) {
		for(long long k = gtid; k < L2; k += gstride) {
			const int e0 = cov_off[k], e1 = cov_off[k + 1];
			double sx = 0.0, sy = 0.0;
#pragma unroll 1
			for(int e = e0; e < e1; e += NB) {
				int js[NB];
				double uxv[NB], uyv[NB];
				float exv[NB], eyv[NB];
#pragma unroll
				for(int u = 0; u < NB; u++) js[u] = e + u < e1 ? cov_idx[e + u] : -1;
#pragma unroll
				for(int u = 0; u < NB; u++) {
					const int j = js[u];
					uxv[u] = j >= 0 ? a.vx[j] : 0.0;
					uyv[u] = j >= 0 ? a.vy[j] : 0.0;
					if(fmode == RES_FLOAT_COVER && add_e) {
						exv[u] = j >= 0 ? a.exf[e + u] : 0.0f;
						eyv[u] = j >= 0 ? a.eyf[e + u] : 0.0f;
					}
				}
#pragma unroll
				for(int u = 0; u < NB; u++) {
					const int j = js[u];
					if(j < 0) break;
					double ux = uxv[u], uy = uyv[u];
					if(fmode == RES_FLOAT_COVER && add_e) {
						ux += (double) exv[u];
						uy += (double) eyv[u];
						a.vx[j] = ux;
						a.vy[j] = uy;
					}
					sx += ux;
					sy += uy;
				}
			}
			a.Px[k] = sx;
			a.Py[k] = sy;
		}
		if(!grid_reduce(a, sh, 0, nullptr)) return false;
	}
	double v[6] = {0, 0, 0, 0, 0, 0};
	for(long long k = gtid; k < L2; k += gstride) {
		const int e0 = cov_off[k], e1 = cov_off[k + 1];
		float Rx = 0.f, Ry = 0.f;
		if(e1 > e0) {
			const int D = box_deg(a.cnt, (int) k, L);
			const double T = sh.T[D], iT = sh.iT[D];
			const float iTf = (float) iT;
			const double qx = x_zero ? 0.0 : neta * box_n4(a.Px, (int) k, L);
			const double qy = x_zero ? 0.0 : neta * box_n4(a.Py, (int) k, L);
#pragma unroll 1
			for(int e0b = e0; e0b < e1; e0b += NB) {
				int js[NB];
				double bxv[NB], byv[NB], uxv[NB], uyv[NB];
#pragma unroll
				for(int u = 0; u < NB; u++) js[u] = e0b + u < e1 ? cov_idx[e0b + u] : -1;
#pragma unroll
				for(int u = 0; u < NB; u++) {
					const int j = js[u];
					bxv[u] = j >= 0 ? a.fx[j] : 0.0;
					byv[u] = j >= 0 ? a.fy[j] : 0.0;
					uxv[u] = (j >= 0 && !x_zero) ? a.vx[j] : 0.0;
					uyv[u] = (j >= 0 && !x_zero) ? a.vy[j] : 0.0;
				}
#pragma unroll
				for(int u = 0; u < NB; u++) {
					const int j = js[u];
					if(j < 0) break;
					const int e = e0b + u;
					const double bx = bxv[u], by = byv[u];
					double rx, ry;
					if(x_zero) {
						rx = bx - 0.0;
						ry = by - 0.0;
					}
					else {
						rx = bx - __fma_rn(T, uxv[u], qx);
						ry = by - __fma_rn(T, uyv[u], qy);
					}
					if(fmode != RES_FLOAT_COVER) {
						// the learned path never reads the FP64 residual (its FP64
						// fallback recomputes it)
						a.rx[j] = rx;
						a.ry[j] = ry;
					}
					if(want_b) {
						v[0] = __fma_rn(bx, bx, v[0]);
						v[1] = __fma_rn(by, by, v[1]);
					}
					v[2] = __fma_rn(rx, rx, v[2]);
					v[3] = __fma_rn(ry, ry, v[3]);
					if(fmode != RES_FP64) {
						const float fx = (float) rx, fy = (float) ry;
						a.rxf[e] = fx;
						a.ryf[e] = fy;
						a.exf[e] = 0.0f;
						a.eyf[e] = 0.0f;
						if(want_rz) {
							v[4] += (double) fx * (iT * (double) fx);
							v[5] += (double) fy * (iT * (double) fy);
						}
						Rx += fx * iTf;
						Ry += fy * iTf;
					}
					else if(want_rz) {
						v[4] += rx * (iT * rx);
						v[5] += ry * (iT * ry);
					}
				}
			}
		}
		if(fmode == RES_FLOAT_COVER && a.unet_params) {
			const float wv = box_w(a, sh, (int) k, L);
			a.unet.x0[k * 2] = Rx;
			a.unet.x0[k * 2 + 1] = wv;
			a.unet.x0[(L2 + k) * 2] = Ry;
			a.unet.x0[(L2 + k) * 2 + 1] = wv;
		}
	}
	block_sum<6>(v, sh.red);
	return grid_reduce(a, sh, 6, v);
}

// Shuffle tree within each warp in the vectors' own precision (lane 0 ends
// with the warp's sum).
template<typename T, int NV>
__device__ __forceinline__ void warp_tree(T (&w)[NV]) {
#pragma unroll
	for(int i = 0; i < NV; i++) {
#pragma unroll
		for(int o = 16; o > 0; o >>= 1) w[i] += __shfl_down_sync(0xffffffffu, w[i], o);
	}
}

// Block sum of values already reduced within each warp (valid in lane 0),
// FP64 across warps; result in every thread.
template<int NV>
__device__ inline void block_sum_warps(double (&v)[NV], double *scratch) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	__syncthreads();
	if(lane == 0) {
#pragma unroll
		for(int i = 0; i < NV; i++) scratch[i * nw + warp] = v[i];
	}
	__syncthreads();
	if(warp == 0) {
#pragma unroll
		for(int i = 0; i < NV; i++) {
			double t = lane < nw ? scratch[i * nw + lane] : 0.0;
#pragma unroll
			for(int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
			if(lane == 0) scratch[NV * nw + i] = t;
		}
	}
	__syncthreads();
#pragma unroll
	for(int i = 0; i < NV; i++) v[i] = scratch[NV * nw + i];
	__syncthreads();
}

__device__ __forceinline__ bool harvest_point(const CGArgs &a, CGShared &sh, const double *ux, const double *uy, const double *rx,
                              const double *ry, int m);


template<typename T>
__device__ __forceinline__ T box_n4T(const T *P, int k, int L) {
	const int x = k % L, y = k / L;
	const int kr = (x == L - 1) ? k - (L - 1) : k + 1;
	const int kl = (x == 0) ? k + (L - 1) : k - 1;
	const int ku = (y == L - 1) ? k - (L - 1) * L : k + L;
	const int kd = (y == 0) ? k + (L - 1) * L : k - L;
	return P[kd] + P[kl] + P[kr] + P[ku];
}

// Vectors of one FP64 CG run: residual r, scaled direction q = T p, box sums
// P of p, solution x.
struct CGVecs {
	double *rx, *ry, *qx, *qy, *Pbx, *Pby, *ux, *uy;
};

// The Jacobi preconditioner is constant on a box site (every unknown at k has
// the diagonal T(k)), so the plain solve carries q = T p in place of Eigen's
// direction p.  Eigen's p = z + beta p with z = r / T becomes q = r + beta q,
// and every other 1/T factor is taken once per site instead of once per
// unknown.  With P(k) = sum of p over the unknowns at k:
//   p.Ap = sum_k (1/T) sum q^2 - eta sum_k P(k) N4(P)(k)
//   Ap = q - eta N4(P),  x += (alpha / T) q,  r.z = sum_k (1/T) sum r^2,
// so no pass reads or writes an Ap vector: phase A forms q, P and the first
// term of p.Ap; phase B is a pass over box sites only (the second term);
// phase C forms Ap on the fly.  Per unknown and component-iteration that is
// 64 B of vector traffic (r, q read and q written; q, r, x read and r, x
// written) and seven FP64 operations -- GB300 issues FP64 at a small fraction
// of its FP32 rate and the solve is bound by that issue and by HBM.  The
// iterates are Eigen's up to rounding (the solve is not bitwise Eigen's in
// any case: its reductions run in a different order).

// First box site k in [0, L2] with cov_off[k] >= t (cov_off is
// nondecreasing, cov_off[L2] = the number of cover entries >= t).
__device__ __forceinline__ long long first_site_from(const int *cov_off, long long L2, long long t) {
	long long lo = 0, hi = L2;
	while(lo < hi) {
		const long long mid = (lo + hi) >> 1;
		if((long long) __ldcg(&cov_off[mid]) >= t) hi = mid;
		else lo = mid + 1;
	}
	return lo;
}

// The box sites of this block in the by-site phases (thread 0 only): the
// thread (or warp) at offset t of the block takes sites site_first + t,
// + site_step, ... below site_end.  On boxes with fewer than four sites per
// thread of the grid the block takes a contiguous run of sites holding an
// equal share of the cover entries (the unknowns): a grid-stride split would
// leave whole blocks (SMs) without sites there while others walk long cover
// lists.  Larger boxes keep the grid-stride split, balanced by itself.
__device__ __forceinline__ void block_site_range(const CGArgs &a, CGShared &sh) {
	const long long L2 = (long long) a.L * a.L;
	const long long nb = gridDim.x, b = blockIdx.x, threads = nb * blockDim.x;
	if(L2 >= 4 * threads) {
		sh.site_first = (int) (b * blockDim.x);
		sh.site_step = (int) threads;
		sh.site_end = (int) L2;
		return;
	}
	const long long E = __ldcg(&a.cov_off[L2]);
	sh.site_first = (int) first_site_from(a.cov_off, L2, E * b / nb);
	sh.site_step = blockDim.x;
	sh.site_end = (int) (b + 1 == nb ? L2 : first_site_from(a.cov_off, L2, E * (b + 1) / nb));
}

// Phase A by box site: thread k walks its cover list in order, updates q
// there, stores P(k) (every site written, so P needs no clearing) and sums
// (1/T) sum q^2 into sh.tot[0..1].
// NB: unknowns of a site whose loads are issued together (their indices
// first, then their values), summed in the same order; 2 in the two-CTA
// build, 4 where one CTA per SM leaves the registers for it.
template<int NB>
__device__ __forceinline__ bool cg_phase_a_sites(const CGArgs &a, CGShared &sh, const CGVecs &V) {
	const int L = a.L;
	const int ax = sh.act[0], ay = sh.act[1], first = sh.first;
	const double bx = sh.beta[0], by = sh.beta[1];
	const double *rx = V.rx, *ry = V.ry;
	double *qx = V.qx, *qy = V.qy, *Pbx = V.Pbx, *Pby = V.Pby;
	const int *cov_idx = a.cov_idx, *cov_off = a.cov_off, *cnt = a.cnt;
	double w0 = 0.0, w1 = 0.0;
	for(long long k = sh.site_first + threadIdx.x; k < sh.site_end; k += sh.site_step) {
		const int e0 = cov_off[k], e1 = cov_off[k + 1];
		double sx = 0.0, sy = 0.0;
		if(e1 > e0) {
			double hx = 0.0, hy = 0.0;
			for(int e = e0; e < e1; e += NB) {
				int js[NB];
				double rxv[NB], ryv[NB], qxv[NB], qyv[NB];
#pragma unroll
				for(int u = 0; u < NB; u++) js[u] = e + u < e1 ? cov_idx[e + u] : -1;
#pragma unroll
				for(int u = 0; u < NB; u++) {
					const int j = js[u];
					const bool v = j >= 0;
					rxv[u] = (v && ax) ? rx[j] : 0.0;
					qxv[u] = (v && ax && !first) ? qx[j] : 0.0;
					ryv[u] = (v && ay) ? ry[j] : 0.0;
					qyv[u] = (v && ay && !first) ? qy[j] : 0.0;
				}
#pragma unroll
				for(int u = 0; u < NB; u++) {
					const int j = js[u];
					if(j < 0) break;
					if(ax) {
						const double q = first ? rxv[u] : __fma_rn(bx, qxv[u], rxv[u]);
						qx[j] = q;
						sx += q;
						hx = __fma_rn(q, q, hx);
					}
					if(ay) {
						const double q = first ? ryv[u] : __fma_rn(by, qyv[u], ryv[u]);
						qy[j] = q;
						sy += q;
						hy = __fma_rn(q, q, hy);
					}
				}
			}
			const double id = sh.iT[box_deg(cnt, (int) k, L)];
			sx *= id;
			sy *= id;
			w0 = __fma_rn(id, hx, w0);
			w1 = __fma_rn(id, hy, w1);
		}
		if(ax) Pbx[k] = sx;
		if(ay) Pby[k] = sy;
	}
	double w[2] = {w0, w1};
	warp_tree<double, 2>(w);
	double v[2] = {w[0], w[1]};
	block_sum_warps<2>(v, sh.red);
	return grid_reduce(a, sh, 2, v);
}

// Phase B over box sites: sum_k P(k) N4(P)(k) = 2 sum_k P(k) (P(k + x) +
// P(k + y)) on the periodic box, into sh.tot[0..1].
__device__ __forceinline__ bool cg_phase_b_sites(const CGArgs &a, CGShared &sh, const CGVecs &V) {
	const int L = a.L;
	const long long L2 = (long long) L * L;
	const long long gtid = blockIdx.x * (long long) blockDim.x + threadIdx.x;
	const long long gstride = (long long) gridDim.x * blockDim.x;
	const int ax = sh.act[0], ay = sh.act[1];
	const double *Pbx = V.Pbx, *Pby = V.Pby;
	double w0 = 0.0, w1 = 0.0;
	for(long long k = gtid; k < L2; k += gstride) {
		const int x = (int) (k % L);
		const long long kr = (x == L - 1) ? k - (L - 1) : k + 1;
		const long long ku = (k >= L2 - L) ? k - (L2 - L) : k + L;
		if(ax) w0 = __fma_rn(Pbx[k], Pbx[kr] + Pbx[ku], w0);
		if(ay) w1 = __fma_rn(Pby[k], Pby[kr] + Pby[ku], w1);
	}
	double w[2] = {w0, w1};
	warp_tree<double, 2>(w);
	double v[2] = {w[0], w[1]};
	block_sum_warps<2>(v, sh.red);
	return grid_reduce(a, sh, 2, v);
}

// Phase C by box site: Ap = q - eta N4(P), x += (alpha / T) q, r -= alpha Ap
// for the unknowns at k and the site's sum of r^2, giving |r|^2 and
// r.z = sum_k (1/T) sum r^2 into sh.tot[0..3].
template<int NB>
__device__ __forceinline__ bool cg_phase_c_sites(const CGArgs &a, CGShared &sh, const CGVecs &V) {
	const int L = a.L;
	const double neta = -a.eta * 1.0;
	const int ax = sh.act[0], ay = sh.act[1];
	const double alx = sh.alpha[0], aly = sh.alpha[1];
	const double *qx = V.qx, *qy = V.qy, *Pbx = V.Pbx, *Pby = V.Pby;
	double *rx = V.rx, *ry = V.ry, *ux = V.ux, *uy = V.uy;
	const int *cov_idx = a.cov_idx, *cov_off = a.cov_off, *cnt = a.cnt;
	double w[4] = {0.0, 0.0, 0.0, 0.0};
	for(long long k = sh.site_first + threadIdx.x; k < sh.site_end; k += sh.site_step) {
		const int e0 = cov_off[k], e1 = cov_off[k + 1];
		if(e1 == e0) continue;
		const double id = sh.iT[box_deg(cnt, (int) k, L)];
		const double gx = alx * id, gy = aly * id;
		const double nx = ax ? neta * box_n4T<double>(Pbx, (int) k, L) : 0.0;
		const double ny = ay ? neta * box_n4T<double>(Pby, (int) k, L) : 0.0;
		double sx = 0.0, sy = 0.0;
		for(int e = e0; e < e1; e += NB) {
			int js[NB];
			double qxv[NB], rxv[NB], uxv[NB], qyv[NB], ryv[NB], uyv[NB];
#pragma unroll
			for(int u = 0; u < NB; u++) js[u] = e + u < e1 ? cov_idx[e + u] : -1;
#pragma unroll
			for(int u = 0; u < NB; u++) {
				const int j = js[u];
				const bool vx = j >= 0 && ax, vy = j >= 0 && ay;
				qxv[u] = vx ? qx[j] : 0.0;
				rxv[u] = vx ? rx[j] : 0.0;
				uxv[u] = vx ? ux[j] : 0.0;
				qyv[u] = vy ? qy[j] : 0.0;
				ryv[u] = vy ? ry[j] : 0.0;
				uyv[u] = vy ? uy[j] : 0.0;
			}
#pragma unroll
			for(int u = 0; u < NB; u++) {
				const int j = js[u];
				if(j < 0) break;
				if(ax) {
					ux[j] = __fma_rn(gx, qxv[u], uxv[u]);
					const double r = __fma_rn(-alx, qxv[u] + nx, rxv[u]);
					rx[j] = r;
					sx = __fma_rn(r, r, sx);
				}
				if(ay) {
					uy[j] = __fma_rn(gy, qyv[u], uyv[u]);
					const double r = __fma_rn(-aly, qyv[u] + ny, ryv[u]);
					ry[j] = r;
					sy = __fma_rn(r, r, sy);
				}
			}
		}
		w[0] += sx;
		w[1] += sy;
		w[2] = __fma_rn(id, sx, w[2]);
		w[3] = __fma_rn(id, sy, w[3]);
	}
	double v[4] = {w[0], w[1], w[2], w[3]};
	block_sum<4>(v, sh.red);
	return grid_reduce(a, sh, 4, v);
}

// Jacobi-preconditioned CG iterations from the state in sh (act, rz, thr) and
// the residual in V.rx, V.ry: Eigen's loop, in FP64 and on the scaled
// direction q = T p (the plain solve and the FP64 fallback of the
// mixed-precision refinement); every thread's partial dot products, in
// box-site order, are summed for the block and grid reductions.
template<int NB = 1>
__device__ __forceinline__ bool cg_iterate(const CGArgs &a, CGShared &sh, const CGVecs &V, long long max_it) {
	// phase A writes P at every site for each active component
	if(threadIdx.x == 0) {
		block_site_range(a, sh);
		sh.first = 1;
	}
	__syncthreads();
	long long sweep = 0;
	while(sh.act[0] || sh.act[1]) {
		if(a.harv_in && !a.mixed && sh.hm < a.harv_per_solve && sweep % a.harv_every == 0 &&
		   sh.hbase + 2LL * (sh.hm + 1) <= a.harv_cap) {
			if(!harvest_point(a, sh, V.ux, V.uy, V.rx, V.ry, sh.hm)) return false;
			if(threadIdx.x == 0) sh.hm++;
			__syncthreads();
		}
		sweep++;
		const int ax = sh.act[0], ay = sh.act[1];
		if(!cg_phase_a_sites<NB>(a, sh, V)) return false;
		if(threadIdx.x == 0) {
			sh.pap[0] = sh.tot[0];
			sh.pap[1] = sh.tot[1];
		}
		if(!cg_phase_b_sites(a, sh, V)) return false;
		if(threadIdx.x == 0) {
			const double neta2 = -2.0 * a.eta;
			if(ax) sh.alpha[0] = sh.rz[0] / __fma_rn(neta2, sh.tot[0], sh.pap[0]);
			if(ay) sh.alpha[1] = sh.rz[1] / __fma_rn(neta2, sh.tot[1], sh.pap[1]);
		}
		__syncthreads();
		// phase C holds six values per unknown: the two-CTA build has the
		// registers for one unknown in flight
		if(!cg_phase_c_sites<(NB >= 4 ? NB : 1)>(a, sh, V)) return false;
		if(threadIdx.x == 0) {
			for(int c = 0; c < 2; c++) {
				if(!sh.act[c]) continue;
				sh.rn2[c] = sh.tot[c];
				if(sh.rn2[c] < sh.thr[c]) {
					sh.act[c] = 0;
					continue;
				}
				// a NaN/Inf right-hand side: stop now (Eigen would run to its
				// iteration cap, twice the unknowns) and report it
				if(!isfinite(sh.rn2[c])) {
					sh.act[c] = 0;
					atomicOr(&a.st->err, ERR_NONFINITE);
					continue;
				}
				const double rz_new = sh.tot[2 + c];
				sh.beta[c] = rz_new / sh.rz[c];
				sh.rz[c] = rz_new;
				sh.it[c]++;
				if(sh.it[c] >= max_it) sh.act[c] = 0;
			}
			sh.first = 0;
		}
		__syncthreads();
	}
	return true;
}

// ---------------------------------------------------------------------------
// Training samples for the learned preconditioner, taken from the FP64 solve.
//
// Eliminating the patch unknowns at one box site k (they share T = xi + eta
// D(k)) turns A v = r into a box-grid system: with R[k] = sum_{j at k} r_j / T
// and V = S v (box sums), V - eta W (N4 V) = R where W[k] = n(k) / T(k), and
// then v_j = (r_j + eta (N4 V)[k_j]) / T_j exactly.  The network learns
// R -> V.  At iteration k of the plain solve, with x_k the iterate and r_k
// its residual, the error e_k = x* - x_k solves A e_k = r_k, so the pair is
// (R_k, V = S x* - S x_k).  Inputs and targets are divided by the residual
// scale s = sqrt(|r_k|^2 / S), the same normalisation the solve applies.

// Record harvest point m: box sums of x (into the target slot) and of r/T
// (into the input slot) for both components; slots hbase + 2m + c.
__device__ __forceinline__ bool harvest_point(const CGArgs &a, CGShared &sh, const double *ux, const double *uy, const double *rx,
                              const double *ry, int m) {
	const int L = a.L;
	const long long L2 = (long long) L * L;
	const long long gtid = blockIdx.x * (long long) blockDim.x + threadIdx.x;
	const long long gstride = (long long) gridDim.x * blockDim.x;
	const long long q0 = sh.hbase + 2LL * m;
	for(long long k = gtid; k < L2; k += gstride) {
		const float w = box_w(a, sh, (int) k, L);
		for(int c = 0; c < 2; c++) {
			a.harv_in[((q0 + c) * L2 + k) * 2] = 0.f;
			a.harv_in[((q0 + c) * L2 + k) * 2 + 1] = w;
			a.harv_tgt[(q0 + c) * L2 + k] = 0.f;
		}
	}
	if(blockIdx.x == 0 && threadIdx.x < 2) {
		const int c = threadIdx.x;
		a.harv_s[q0 + c] = sh.act[c] ? (float) sqrt(sh.rn2[c] / (double) sh.S) : 0.f;
	}
	if(!grid_reduce(a, sh, 0, nullptr)) return false;
	const long long E = __ldcg(&a.cov_off[L2]);
	const long long gwarp = gtid >> 5, nwarps = gstride >> 5;
	const int lane = threadIdx.x & 31;
	for(long long base = gwarp * 32; base < E; base += nwarps * 32) {
		const long long t = base + lane;
		const bool valid = t < E;
		const int j = valid ? a.cov_idx[t] : 0;
		const int key = valid ? a.mapg[j] : -1;
		const double id = valid ? sh.iT[box_deg(a.cnt, key, L)] : 0.0;
		bool t0, t1, t2, t3;
		const double sx = seg_sum<double>(valid ? ux[j] : 0.0, key, t0);
		const double sy = seg_sum<double>(valid ? uy[j] : 0.0, key, t1);
		const double rxs = seg_sum<double>(valid ? rx[j] * id : 0.0, key, t2);
		const double rys = seg_sum<double>(valid ? ry[j] * id : 0.0, key, t3);
		if(valid && t0) {
			atomicAdd(&a.harv_tgt[q0 * L2 + key], (float) sx);
			atomicAdd(&a.harv_tgt[(q0 + 1) * L2 + key], (float) sy);
			atomicAdd(&a.harv_in[(q0 * L2 + key) * 2], (float) rxs);
			atomicAdd(&a.harv_in[((q0 + 1) * L2 + key) * 2], (float) rys);
		}
	}
	return grid_reduce(a, sh, 0, nullptr);
}

// After the solve: targets (S x* - S x_k) / s and inputs R / s for the
// points taken, then publish the new sample count.
__device__ __forceinline__ bool harvest_finish(const CGArgs &a, CGShared &sh, const double *ux, const double *uy) {
	const int L = a.L;
	const long long L2 = (long long) L * L;
	const long long gtid = blockIdx.x * (long long) blockDim.x + threadIdx.x;
	const long long gstride = (long long) gridDim.x * blockDim.x;
	for(long long k = gtid; k < L2; k += gstride) {
		a.Px[k] = 0.0;
		a.Py[k] = 0.0;
	}
	if(!grid_reduce(a, sh, 0, nullptr)) return false;
	const long long E = __ldcg(&a.cov_off[L2]);
	const long long gwarp = gtid >> 5, nwarps = gstride >> 5;
	const int lane = threadIdx.x & 31;
	for(long long base = gwarp * 32; base < E; base += nwarps * 32) {
		const long long t = base + lane;
		const bool valid = t < E;
		const int j = valid ? a.cov_idx[t] : 0;
		const int key = valid ? a.mapg[j] : -1;
		bool t0, t1;
		const double sx = seg_sum<double>(valid ? ux[j] : 0.0, key, t0);
		const double sy = seg_sum<double>(valid ? uy[j] : 0.0, key, t1);
		if(valid && t0) {
			atomicAdd(&a.Px[key], sx);
			atomicAdd(&a.Py[key], sy);
		}
	}
	if(!grid_reduce(a, sh, 0, nullptr)) return false;
	const long long n = 2LL * sh.hm;
	for(long long e = gtid; e < n * L2; e += gstride) {
		const long long q = sh.hbase + e / L2, k = e % L2;
		const float sc = __ldcg(&a.harv_s[q]);
		if(sc > 0.f) {
			const double xs = ((e / L2) & 1) ? a.Py[k] : a.Px[k];
			a.harv_tgt[q * L2 + k] = (float) ((xs - (double) a.harv_tgt[q * L2 + k]) / (double) sc);
			a.harv_in[(q * L2 + k) * 2] = a.harv_in[(q * L2 + k) * 2] / sc;
		}
	}
	if(blockIdx.x == 0 && threadIdx.x == 0) *a.harv_count = sh.hbase + 2 * sh.hm;
	return true;
}

// ---------------------------------------------------------------------------
// Learned preconditioner inside flexible CG.
//
// The FP32 vectors of the flexible CG (r, z, p, Ap, e) are stored in cover
// order: entry e is the unknown cov_idx[e], and the entries of box site k are
// [cov_off[k], cov_off[k+1]).  Every phase is a loop over box sites in which
// a thread walks its site's contiguous entries: no index indirection, box
// sums stored without atomics, all sums in a fixed order.
//
// One iteration (both components at once, each with its own scalars):
//   network  V = N(R / s, W)                (input R written by phase C)
//   phase E  z = (r + eta s N4V) / T, Z = S z, r.z and z.Ap_old
//   phase AB p = z + beta p with beta = -z.Ap_old / p.Ap_old (Notay's
//            FCG(1)); P' = S p; Ap = T p - eta N4(P'), the neighbours' P'
//            taken as Z + beta P (linearity, so no barrier); p.Ap
//   phase C  e += alpha p, r -= alpha Ap, |r|^2, R = sum r / T
// with alpha = r.z / p.Ap.  P alternates between two box buffers.

// The network on both components: V (a.unet.out, FP32) from x0.
__device__ __noinline__ bool precond_network(const CGArgs &a, CGShared &sh, TcCtx &tc) {
	float *wsm = reinterpret_cast<float *>(tc.sm);
	pmark(a, sh, PH_OTHER);
	const int L = a.L;
	const long long L2 = (long long) L * L;
	const long long gtid = blockIdx.x * (long long) blockDim.x + threadIdx.x;
	const long long gstride = (long long) gridDim.x * blockDim.x;
	const float sc[2] = {sh.scale[0] > 0.0 ? (float) (1.0 / sh.scale[0]) : 0.f,
	                     sh.scale[1] > 0.0 ? (float) (1.0 / sh.scale[1]) : 0.f};
	// the tensor-core path evaluates the first layer while staging the
	// second's rows when the box side allows strips
	const bool fused_first = a.unet_tc && L % 128 == 0;
	if(!fused_first) {
		const int nw = 9 * 2 * 16 + 16;
		__syncthreads();
		for(int k = threadIdx.x; k < nw; k += blockDim.x) wsm[k] = a.unet_params[unet_weight_offset(L_E0A) + k];
		__syncthreads();
		for(long long p = gtid; p < 2 * L2; p += gstride) {
			const int n = p >= L2;
			const int r = (int) (p - n * L2);
			const int i = r / L, j = r - (r / L) * L;
			float y[16];
			e0a_pixel(a.unet.x0, wsm, n, i, j, L, sc[n], y);
			if(a.unet_tc) {
				uint4 o0, o1;
				o0.x = f2bf(y[0], y[1]);
				o0.y = f2bf(y[2], y[3]);
				o0.z = f2bf(y[4], y[5]);
				o0.w = f2bf(y[6], y[7]);
				o1.x = f2bf(y[8], y[9]);
				o1.y = f2bf(y[10], y[11]);
				o1.z = f2bf(y[12], y[13]);
				o1.w = f2bf(y[14], y[15]);
				uint4 *o = reinterpret_cast<uint4 *>(a.unet_bf.e0a + p * 16);
				o[0] = o0;
				o[1] = o1;
			}
			else {
				float4 *o = reinterpret_cast<float4 *>(a.unet.e0a + p * 16);
#pragma unroll
				for(int q = 0; q < 4; q++) o[q] = make_float4(y[4 * q], y[4 * q + 1], y[4 * q + 2], y[4 * q + 3]);
			}
		}
		if(!grid_reduce(a, sh, 0, nullptr)) return false;
		pmark(a, sh, PH_E0A);
	}
	if(a.unet_tc) {
		// nine tensor-core layers; last layer (FP32, CUDA cores) -> V
		for(int l = L_E0B; l <= L_D0B; l++) {
			TcSrc src = unet_tc_src(l, a.unet_bf);
			if(l == L_E0B && fused_first) {
				src.mode = IN_FIRST;
				src.x = a.unet.x0;
				src.w0 = a.unet_params + unet_weight_offset(L_E0A);
				src.sc[0] = sc[0];
				src.sc[1] = sc[1];
			}
			if(!tc_conv_layer(l, src, a.unet_wpack + unet_pack_offset(l),
			                  a.unet_params + unet_weight_offset(l), a.unet_params + unet_bias_offset(l),
			                  unet_tc_dst(l, a.unet_bf), 2, L >> unet_layer(l).level, tc))
				return false;
			if(!grid_reduce(a, sh, 0, nullptr)) return false;
			pmark(a, sh, PH_TC0 + unet_layer(l).level);
		}
		__syncthreads();
		const int nw = 9 * 16 + 1;
		for(int k = threadIdx.x; k < nw; k += blockDim.x) wsm[k] = a.unet_params[unet_weight_offset(L_OUT) + k];
		__syncthreads();
		out_range(a.unet_bf.t0, wsm, a.unet.out, 2, L, gtid, gstride);
		if(!grid_reduce(a, sh, 0, nullptr)) return false;
		pmark(a, sh, PH_OUT);
	}
	else {
		for(int l = L_E0B; l < UNET_LAYERS; l++) {
			const UNetLayerDesc d = unet_layer(l);
			const int nw = 9 * d.ci * d.co + d.co;
			const float *src = a.unet_params + unet_weight_offset(l);
			__syncthreads();
			for(int k = threadIdx.x; k < nw; k += blockDim.x) wsm[k] = src[k];
			__syncthreads();
			conv_layer_range(l, unet_src(l, a.unet), wsm, wsm + 9 * d.ci * d.co, unet_dst(l, a.unet), 2, L >> d.level,
			                 gtid, gstride);
			if(!grid_reduce(a, sh, 0, nullptr)) return false;
		}
		pmark(a, sh, PH_OUT);
	}
	return true;
}

// Warp-cooperative walk over the entries of 32 consecutive box sites: lane l
// owns site k0 + l (entries [e0, e1) of it); the warp then streams the
// entries [E0, E1) of its 32 sites in coalesced chunks of 32.  For an entry,
// `s` is the lane owning its site (found by a five-step search over the
// lanes' e0), `same[i]` whether the entry 2^i lanes below belongs to the same
// site and `tail` whether it is the last entry of its site in this chunk;
// per-site sums are formed by a segmented scan in the chunk and added by the
// tail lane to the owner's slot of a per-warp accumulator, chunk after chunk,
// so all sums have a fixed order.
constexpr int FCG_BATCH = 4;  // chunks whose loads are in flight together (phase C: eight streams)
constexpr int FCG_BATCH_EA = 8;  // the same for phases E and AB (four streams)

struct SegLane {
	int s;
	bool valid, tail;
	bool same[5];
};

__device__ __forceinline__ SegLane seg_lane(int e, int E1, int e0) {
	SegLane g;
	const int lane = threadIdx.x & 31;
	g.valid = e < E1;
	int s = 0;
#pragma unroll
	for(int step = 16; step > 0; step >>= 1) {
		const int v = __shfl_sync(0xffffffffu, e0, s + step);
		if(v <= e) s += step;
	}
	g.s = g.valid ? s : 32;
#pragma unroll
	for(int i = 0; i < 5; i++) {
		const int ks = __shfl_up_sync(0xffffffffu, g.s, 1 << i);
		g.same[i] = lane >= (1 << i) && ks == g.s;
	}
	const int kn = __shfl_down_sync(0xffffffffu, g.s, 1);
	g.tail = g.valid && (lane == 31 || kn != g.s);
	return g;
}

__device__ __forceinline__ float seg_scan(float v, const SegLane &g) {
#pragma unroll
	for(int i = 0; i < 5; i++) {
		const float u = __shfl_up_sync(0xffffffffu, v, 1 << i);
		if(g.same[i]) v += u;
	}
	return v;
}

// Phase E: z = (r + eta s N4V) / T, Z = S z; r.z, and z.Ap of the previous
// direction (not on the first sweep) into sh.tot[0..3].  wacc: 2 x blockDim
// floats of shared memory.
__device__ __noinline__ bool fcg_phase_e(const CGArgs &a, CGShared &sh, bool first, float *wacc) {
	const int L = a.L;
	const long long L2 = (long long) L * L;
	const int lane = threadIdx.x & 31;
	const int ax = sh.act[0], ay = sh.act[1];
	const float es0 = (float) (a.eta * sh.scale[0]), es1 = (float) (a.eta * sh.scale[1]);
	const bool net = a.unet_params != nullptr;  // without a network: z = r / T (Jacobi)
	const float *V = a.unet.out;
	const float *rx = a.rxf, *ry = a.ryf, *apx = a.apxf, *apy = a.apyf;
	float *zx = a.zxf, *zy = a.zyf;
	const int *cov_off = a.cov_off;
	const int Eend = __ldcg(&cov_off[sh.site_end]);
	float *accx = wacc, *accy = wacc + blockDim.x;
	float w[4] = {0.f, 0.f, 0.f, 0.f};
	// per-site values of a group of 32 sites, loaded one group ahead so that
	// their round trips overlap the previous group's entries
	int pe0 = Eend, pe1 = Eend, pdeg = 0;
	float pvx = 0.f, pvy = 0.f;
	auto prefetch = [&](long long kk) {
		const bool v = kk < sh.site_end;
		pe0 = v ? cov_off[kk] : Eend;
		pe1 = v ? cov_off[kk + 1] : Eend;
		pdeg = v ? box_deg(a.cnt, (int) kk, L) : 0;
		pvx = (v && net && ax) ? box_n4T<float>(V, (int) kk, L) : 0.f;
		pvy = (v && net && ay) ? box_n4T<float>(V + L2, (int) kk, L) : 0.f;
	};
	// warps take runs of 32 of the block's sites; lanes past the last site
	// hold the empty entry range at Eend
	const long long kfirst = sh.site_first + (threadIdx.x & ~31);
	if(kfirst < sh.site_end) prefetch(kfirst + lane);
	for(long long k0 = kfirst; k0 < sh.site_end; k0 += sh.site_step) {
		const long long k = k0 + lane;
		const bool kv = k < sh.site_end;
		const int e0 = pe0, e1 = pe1;
		float id = 0.f, nvx = 0.f, nvy = 0.f;
		if(e1 > e0) {
			id = sh.iTf[pdeg];
			if(net && ax) nvx = es0 * pvx;
			if(net && ay) nvy = es1 * pvy;
		}
		if(k0 + sh.site_step < sh.site_end) prefetch(k0 + sh.site_step + lane);
		accx[threadIdx.x] = 0.f;
		accy[threadIdx.x] = 0.f;
		__syncwarp();
		const int E0 = __shfl_sync(0xffffffffu, e0, 0), E1 = __shfl_sync(0xffffffffu, e1, 31);
		// chunks in batches of FCG_BATCH: all loads of a batch are issued first
		for(int c0 = E0; c0 < E1; c0 += 32 * FCG_BATCH_EA) {
			float r0[FCG_BATCH_EA], q0[FCG_BATCH_EA], r1[FCG_BATCH_EA], q1[FCG_BATCH_EA];
#pragma unroll
			for(int u = 0; u < FCG_BATCH_EA; u++) {
				const int e = c0 + 32 * u + lane;
				const bool v = e < E1;
				r0[u] = (v && ax) ? rx[e] : 0.f;
				q0[u] = (v && ax && !first) ? apx[e] : 0.f;
				r1[u] = (v && ay) ? ry[e] : 0.f;
				q1[u] = (v && ay && !first) ? apy[e] : 0.f;
			}
#pragma unroll
			for(int u = 0; u < FCG_BATCH_EA; u++) {
				if(c0 + 32 * u >= E1) break;
				const int e = c0 + 32 * u + lane;
				const SegLane sg = seg_lane(e, E1, e0);
				const int src = sg.s & 31;
				const float ids = __shfl_sync(0xffffffffu, id, src);
				const int slot = (threadIdx.x & ~31) + src;
				if(ax) {
					const float nv = __shfl_sync(0xffffffffu, nvx, src);
					float z = 0.f;
					if(sg.valid) {
						z = ids * (r0[u] + nv);
						zx[e] = z;
						w[0] = __fmaf_rn(r0[u], z, w[0]);
						w[2] = __fmaf_rn(z, q0[u], w[2]);
					}
					const float t = seg_scan(z, sg);
					if(sg.tail) accx[slot] += t;
				}
				if(ay) {
					const float nv = __shfl_sync(0xffffffffu, nvy, src);
					float z = 0.f;
					if(sg.valid) {
						z = ids * (r1[u] + nv);
						zy[e] = z;
						w[1] = __fmaf_rn(r1[u], z, w[1]);
						w[3] = __fmaf_rn(z, q1[u], w[3]);
					}
					const float t = seg_scan(z, sg);
					if(sg.tail) accy[slot] += t;
				}
				__syncwarp();
			}
		}
		if(kv) {
			if(ax) a.Zxf[k] = accx[threadIdx.x];
			if(ay) a.Zyf[k] = accy[threadIdx.x];
		}
		__syncwarp();
	}
	warp_tree<float, 4>(w);
	double v[4] = {(double) w[0], (double) w[1], (double) w[2], (double) w[3]};
	block_sum_warps<4>(v, sh.red);
	return grid_reduce(a, sh, 4, v);
}

// Phase AB: p = z + beta p, box sums into Pn, Ap = T p - eta N4(Pn) with the
// neighbours' Pn = Z + beta Po; p.Ap into sh.tot[0..1].
__device__ __noinline__ bool fcg_phase_ab(const CGArgs &a, CGShared &sh, bool first, const float *Pox, const float *Poy,
                                          float *Pnx, float *Pny, float *wacc) {
	const int L = a.L;
	const int lane = threadIdx.x & 31;
	const int ax = sh.act[0], ay = sh.act[1];
	const float bx = (float) sh.beta[0], by = (float) sh.beta[1];
	const float neta = (float) (-a.eta * 1.0);
	const float *zx = a.zxf, *zy = a.zyf, *Zx = a.Zxf, *Zy = a.Zyf;
	float *px = a.pxf, *py = a.pyf, *apx = a.apxf, *apy = a.apyf;
	const int *cov_off = a.cov_off;
	const int Eend = __ldcg(&cov_off[sh.site_end]);
	float *accx = wacc, *accy = wacc + blockDim.x;
	float w[2] = {0.f, 0.f};
	// per-site values of a group of 32 sites, loaded one group ahead (their
	// round trips overlap the previous group's entries)
	int pe0 = Eend, pe1 = Eend, pdeg = 0;
	float pzx = 0.f, pzy = 0.f, pox = 0.f, poy = 0.f;
	auto prefetch = [&](long long kk) {
		const bool v = kk < sh.site_end;
		pe0 = v ? cov_off[kk] : Eend;
		pe1 = v ? cov_off[kk + 1] : Eend;
		pdeg = v ? box_deg(a.cnt, (int) kk, L) : 0;
		pzx = (v && ax) ? box_n4T<float>(Zx, (int) kk, L) : 0.f;
		pzy = (v && ay) ? box_n4T<float>(Zy, (int) kk, L) : 0.f;
		pox = (v && ax && !first) ? box_n4T<float>(Pox, (int) kk, L) : 0.f;
		poy = (v && ay && !first) ? box_n4T<float>(Poy, (int) kk, L) : 0.f;
	};
	// warps take runs of 32 of the block's sites; lanes past the last site
	// hold the empty entry range at Eend
	const long long kfirst = sh.site_first + (threadIdx.x & ~31);
	if(kfirst < sh.site_end) prefetch(kfirst + lane);
	for(long long k0 = kfirst; k0 < sh.site_end; k0 += sh.site_step) {
		const long long k = k0 + lane;
		const bool kv = k < sh.site_end;
		const int e0 = pe0, e1 = pe1;
		float d = 0.f, qx = 0.f, qy = 0.f;
		if(e1 > e0) {
			d = sh.Tf[pdeg];
			if(ax) qx = neta * (first ? pzx : __fmaf_rn(bx, pox, pzx));
			if(ay) qy = neta * (first ? pzy : __fmaf_rn(by, poy, pzy));
		}
		if(k0 + sh.site_step < sh.site_end) prefetch(k0 + sh.site_step + lane);
		accx[threadIdx.x] = 0.f;
		accy[threadIdx.x] = 0.f;
		__syncwarp();
		const int E0 = __shfl_sync(0xffffffffu, e0, 0), E1 = __shfl_sync(0xffffffffu, e1, 31);
		for(int c0 = E0; c0 < E1; c0 += 32 * FCG_BATCH_EA) {
			float z0[FCG_BATCH_EA], p0[FCG_BATCH_EA], z1[FCG_BATCH_EA], p1[FCG_BATCH_EA];
#pragma unroll
			for(int u = 0; u < FCG_BATCH_EA; u++) {
				const int e = c0 + 32 * u + lane;
				const bool v = e < E1;
				z0[u] = (v && ax) ? zx[e] : 0.f;
				p0[u] = (v && ax && !first) ? px[e] : 0.f;
				z1[u] = (v && ay) ? zy[e] : 0.f;
				p1[u] = (v && ay && !first) ? py[e] : 0.f;
			}
#pragma unroll
			for(int u = 0; u < FCG_BATCH_EA; u++) {
				if(c0 + 32 * u >= E1) break;
				const int e = c0 + 32 * u + lane;
				const SegLane sg = seg_lane(e, E1, e0);
				const int src = sg.s & 31;
				const float ds = __shfl_sync(0xffffffffu, d, src);
				const int slot = (threadIdx.x & ~31) + src;
				if(ax) {
					const float q = __shfl_sync(0xffffffffu, qx, src);
					float p = 0.f;
					if(sg.valid) {
						p = first ? z0[u] : __fmaf_rn(bx, p0[u], z0[u]);
						px[e] = p;
						const float ap = __fmaf_rn(ds, p, q);
						apx[e] = ap;
						w[0] = __fmaf_rn(p, ap, w[0]);
					}
					const float t = seg_scan(p, sg);
					if(sg.tail) accx[slot] += t;
				}
				if(ay) {
					const float q = __shfl_sync(0xffffffffu, qy, src);
					float p = 0.f;
					if(sg.valid) {
						p = first ? z1[u] : __fmaf_rn(by, p1[u], z1[u]);
						py[e] = p;
						const float ap = __fmaf_rn(ds, p, q);
						apy[e] = ap;
						w[1] = __fmaf_rn(p, ap, w[1]);
					}
					const float t = seg_scan(p, sg);
					if(sg.tail) accy[slot] += t;
				}
				__syncwarp();
			}
		}
		if(kv) {
			if(ax) Pnx[k] = accx[threadIdx.x];
			if(ay) Pny[k] = accy[threadIdx.x];
		}
		__syncwarp();
	}
	warp_tree<float, 2>(w);
	double v[2] = {(double) w[0], (double) w[1]};
	block_sum_warps<2>(v, sh.red);
	return grid_reduce(a, sh, 2, v);
}

// Phase C: e += alpha p, r -= alpha Ap, |r|^2 into sh.tot[0..1]; the next
// network input R = sum over the site's unknowns of r / T (unscaled).
__device__ __noinline__ bool fcg_phase_c(const CGArgs &a, CGShared &sh, float *wacc) {
	const int L = a.L;
	const long long L2 = (long long) L * L;
	const int lane = threadIdx.x & 31;
	const int ax = sh.act[0], ay = sh.act[1];
	const float alx = (float) sh.alpha[0], aly = (float) sh.alpha[1];
	const float *px = a.pxf, *py = a.pyf, *apx = a.apxf, *apy = a.apyf;
	float *ex = a.exf, *ey = a.eyf, *rx = a.rxf, *ry = a.ryf, *x0 = a.unet.x0;
	const bool net = a.unet_params != nullptr;
	const int *cov_off = a.cov_off;
	const int Eend = __ldcg(&cov_off[sh.site_end]);
	float *accx = wacc, *accy = wacc + blockDim.x;
	float w[2] = {0.f, 0.f};
	// per-site values of a group of 32 sites, loaded one group ahead
	int pe0 = Eend, pe1 = Eend, pdeg = 0;
	auto prefetch = [&](long long kk) {
		const bool v = kk < sh.site_end;
		pe0 = v ? cov_off[kk] : Eend;
		pe1 = v ? cov_off[kk + 1] : Eend;
		pdeg = v ? box_deg(a.cnt, (int) kk, L) : 0;
	};
	// warps take runs of 32 of the block's sites; lanes past the last site
	// hold the empty entry range at Eend
	const long long kfirst = sh.site_first + (threadIdx.x & ~31);
	if(kfirst < sh.site_end) prefetch(kfirst + lane);
	for(long long k0 = kfirst; k0 < sh.site_end; k0 += sh.site_step) {
		const long long k = k0 + lane;
		const bool kv = k < sh.site_end;
		const int e0 = pe0, e1 = pe1;
		const float id = (e1 > e0) ? sh.iTf[pdeg] : 0.f;
		if(k0 + sh.site_step < sh.site_end) prefetch(k0 + sh.site_step + lane);
		accx[threadIdx.x] = 0.f;
		accy[threadIdx.x] = 0.f;
		__syncwarp();
		const int E0 = __shfl_sync(0xffffffffu, e0, 0), E1 = __shfl_sync(0xffffffffu, e1, 31);
		for(int c0 = E0; c0 < E1; c0 += 32 * FCG_BATCH) {
			float e0v[FCG_BATCH], p0[FCG_BATCH], r0[FCG_BATCH], q0[FCG_BATCH];
			float e1v[FCG_BATCH], p1[FCG_BATCH], r1[FCG_BATCH], q1[FCG_BATCH];
#pragma unroll
			for(int u = 0; u < FCG_BATCH; u++) {
				const int e = c0 + 32 * u + lane;
				const bool v = e < E1;
				e0v[u] = (v && ax) ? ex[e] : 0.f;
				p0[u] = (v && ax) ? px[e] : 0.f;
				r0[u] = (v && ax) ? rx[e] : 0.f;
				q0[u] = (v && ax) ? apx[e] : 0.f;
				e1v[u] = (v && ay) ? ey[e] : 0.f;
				p1[u] = (v && ay) ? py[e] : 0.f;
				r1[u] = (v && ay) ? ry[e] : 0.f;
				q1[u] = (v && ay) ? apy[e] : 0.f;
			}
#pragma unroll
			for(int u = 0; u < FCG_BATCH; u++) {
				if(c0 + 32 * u >= E1) break;
				const int e = c0 + 32 * u + lane;
				const SegLane sg = seg_lane(e, E1, e0);
				const int src = sg.s & 31;
				const float ids = __shfl_sync(0xffffffffu, id, src);
				const int slot = (threadIdx.x & ~31) + src;
				if(ax) {
					float rv = 0.f;
					if(sg.valid) {
						ex[e] = __fmaf_rn(alx, p0[u], e0v[u]);
						const float r = __fmaf_rn(-alx, q0[u], r0[u]);
						rx[e] = r;
						w[0] = __fmaf_rn(r, r, w[0]);
						rv = r * ids;
					}
					if(net) {
						const float t = seg_scan(rv, sg);
						if(sg.tail) accx[slot] += t;
					}
				}
				if(ay) {
					float rv = 0.f;
					if(sg.valid) {
						ey[e] = __fmaf_rn(aly, p1[u], e1v[u]);
						const float r = __fmaf_rn(-aly, q1[u], r1[u]);
						ry[e] = r;
						w[1] = __fmaf_rn(r, r, w[1]);
						rv = r * ids;
					}
					if(net) {
						const float t = seg_scan(rv, sg);
						if(sg.tail) accy[slot] += t;
					}
				}
				__syncwarp();
			}
		}
		if(kv && net) {
			if(ax) x0[k * 2] = accx[threadIdx.x];
			if(ay) x0[(L2 + k) * 2] = accy[threadIdx.x];
		}
		__syncwarp();
	}
	warp_tree<float, 2>(w);
	double v[2] = {(double) w[0], (double) w[1]};
	block_sum_warps<2>(v, sh.red);
	return grid_reduce(a, sh, 2, v);
}

// Flexible CG on the FP32 correction system A e = r of one refinement sweep,
// preconditioned by the network; r and e in cover order (rxf, exf ...) and
// the network input x0 as true_residual(RES_FLOAT_COVER) leaves them.  Stops
// a component at |r|^2 < thr.
__device__ __noinline__ bool fcg_iterate(const CGArgs &a, CGShared &sh, TcCtx &tc, long long max_it) {
	const long long S = sh.S;
	for(int d = threadIdx.x; d <= CG_MAX_D; d += blockDim.x) {
		sh.Tf[d] = (float) sh.T[d];
		sh.iTf[d] = (float) sh.iT[d];
	}
	if(threadIdx.x == 0) {
		for(int c = 0; c < 2; c++) sh.scale[c] = sqrt(sh.rn2[c] / (double) S);
		block_site_range(a, sh);
	}
	__syncthreads();
	pmark(a, sh, PH_INIT);
	bool first = true;
	int par = 0;
	while(sh.act[0] || sh.act[1]) {
		if(a.unet_params && !precond_network(a, sh, tc)) return false;
		if(!fcg_phase_e(a, sh, first, reinterpret_cast<float *>(tc.sm))) return false;
		pmark(a, sh, PH_Z);
		if(threadIdx.x == 0) {
			for(int c = 0; c < 2; c++) {
				if(!sh.act[c]) continue;
				sh.rz[c] = sh.tot[c];
				sh.beta[c] = first ? 0.0 : -sh.tot[2 + c] / sh.pap[c];
			}
		}
		__syncthreads();
		float *Pox = par ? a.Pxf2 : a.Pxf, *Poy = par ? a.Pyf2 : a.Pyf;
		float *Pnx = par ? a.Pxf : a.Pxf2, *Pny = par ? a.Pyf : a.Pyf2;
		if(!fcg_phase_ab(a, sh, first, Pox, Poy, Pnx, Pny, reinterpret_cast<float *>(tc.sm))) return false;
		pmark(a, sh, PH_AB);
		if(threadIdx.x == 0) {
			for(int c = 0; c < 2; c++) {
				if(!sh.act[c]) continue;
				sh.pap[c] = sh.tot[c];
				sh.alpha[c] = sh.rz[c] / sh.tot[c];
			}
		}
		__syncthreads();
		if(!fcg_phase_c(a, sh, reinterpret_cast<float *>(tc.sm))) return false;
		pmark(a, sh, PH_C);
		if(threadIdx.x == 0) {
			for(int c = 0; c < 2; c++) {
				if(!sh.act[c]) continue;
				sh.rn2[c] = sh.tot[c];
				sh.it[c]++;
				if(sh.rn2[c] < sh.thr[c] || sh.it[c] >= max_it || !isfinite(sh.rn2[c])) sh.act[c] = 0;
				sh.scale[c] = sqrt(sh.rn2[c] / (double) S);
			}
		}
		__syncthreads();
		first = false;
		par ^= 1;
	}
	return true;
}

template<bool LEARNED, int NB>
__device__ __forceinline__ void cg_body(const CGArgs &a, CGShared &sh, TcCtx &tc) {
	const double eta = a.eta;
	if(threadIdx.x == 0) {
		if(a.layer >= 0) {
			// a member of an ensemble: its cells' sites are contiguous
			const LayerDev &ly = a.layers[a.layer];
			const CellDev &c0 = a.cells[ly.cell_lo];
			const CellDev &c1 = a.cells[ly.cell_hi - 1];
			sh.jlo = ly.cell_hi > ly.cell_lo ? c0.start : 0;
			sh.S = ly.cell_hi > ly.cell_lo ? (long long) c1.start + c1.n - c0.start : 0;
			sh.cold = a.lsolve[a.layer].cg_cold;
		}
		else {
			sh.jlo = 0;
			sh.S = a.st->S;
			sh.cold = a.st->cg_cold;
		}
	}
	__syncthreads();
	const long long S = sh.S, jlo = sh.jlo;
	const int cold = sh.cold;
	const long long gtid = blockIdx.x * (long long) blockDim.x + threadIdx.x;
	const long long gstride = (long long) gridDim.x * blockDim.x;
	if(threadIdx.x == 0) {
		sh.T[0] = a.xi;
		for(int d = 1; d <= CG_MAX_D; d++) sh.T[d] = sh.T[d - 1] + eta * 1.0;
		for(int d = 0; d <= CG_MAX_D; d++) sh.iT[d] = sh.T[d] != 0.0 ? 1.0 / sh.T[d] : 1.0;
		sh.beta[0] = sh.beta[1] = 0.0;
		sh.hm = 0;
		sh.hbase = a.harv_count ? __ldcg(a.harv_count) : 0;
	}
	__syncthreads();
	if(cold) {
		for(long long j = jlo + gtid; j < jlo + S; j += gstride) {
			a.vx[j] = 0.0;
			a.vy[j] = 0.0;
		}
	}
	if(!build_csr(a, sh)) return;
	// the flexible-CG kernel runs every mixed-precision solve (with or
	// without a network); the plain kernel only FP64 ones
	if constexpr(LEARNED) {
		if(!true_residual<RES_FLOAT_COVER, 4>(a, sh, cold != 0, true, false)) return;
	}
	else {
		if(!true_residual<RES_FP64, (NB >= 4 ? NB : 1)>(a, sh, cold != 0)) return;
	}
	pmark(a, sh, PH_START);
	if(threadIdx.x == 0) {
		for(int c = 0; c < 2; c++) {
			sh.bn2[c] = sh.tot[c];
			sh.rn2[c] = sh.tot[2 + c];
			sh.rz[c] = sh.tot[4 + c];
			sh.it[c] = 0;
			sh.zero[c] = 0;
			sh.thr[c] = fmax(a.tol * a.tol * sh.bn2[c], DBL_MIN);
			if(sh.bn2[c] == 0.0) {
				sh.act[c] = 0;
				sh.zero[c] = 1;
			}
			else sh.act[c] = (sh.rn2[c] < sh.thr[c]) ? 0 : 1;
		}
	}
	__syncthreads();
	if(sh.zero[0] || sh.zero[1]) {
		for(long long j = jlo + gtid; j < jlo + S; j += gstride) {
			if(sh.zero[0]) a.vx[j] = 0.0;
			if(sh.zero[1]) a.vy[j] = 0.0;
		}
	}
	const long long max_it = a.max_iters > 0 ? a.max_iters : 2 * S;
	int refinements = 0, fell_back = 0;
	if constexpr(!LEARNED) {
		if(!cg_iterate<NB>(a, sh, CGVecs{a.rx, a.ry, a.px, a.py, a.Px, a.Py, a.vx, a.vy}, max_it)) return;
		if(a.harv_in && sh.hm > 0 && !harvest_finish(a, sh, a.vx, a.vy)) return;
	}
	else {
		// Iterative refinement: FP32 flexible CG (network or Jacobi
		// preconditioner) for the correction A e = r, stopped at
		// inner_tol * |r|, then x += e and r = b - A x in FP64.  A sweep that
		// fails to reduce |r| by 2x hands over to FP64 CG.
		__shared__ double s_goal[2], s_prev[2];
		__shared__ int s_fallback;
		if(threadIdx.x == 0) {
			for(int c = 0; c < 2; c++) s_goal[c] = sh.thr[c];
			s_fallback = 0;
		}
		__syncthreads();
		for(int sweep = 0; sweep < 64 && (sh.act[0] || sh.act[1]); sweep++) {
			if(threadIdx.x == 0) {
				for(int c = 0; c < 2; c++) {
					s_prev[c] = sh.rn2[c];
					if(sh.act[c]) sh.thr[c] = fmax(a.inner_tol * a.inner_tol * sh.rn2[c], s_goal[c]);
				}
			}
			__syncthreads();
			if(!fcg_iterate(a, sh, tc, max_it < 1000 ? max_it : 1000)) return;
			refinements++;
			// x += e and r = b - A x
			if(!true_residual<RES_FLOAT_COVER, 4>(a, sh, false, false, false, true)) return;
			if(threadIdx.x == 0) {
				for(int c = 0; c < 2; c++) {
					sh.rn2[c] = sh.tot[2 + c];
					sh.rz[c] = sh.tot[4 + c];
					sh.beta[c] = 0.0;
					if(sh.zero[c]) continue;
					sh.act[c] = (sh.rn2[c] < s_goal[c]) ? 0 : 1;
					if(sh.act[c] && !(sh.rn2[c] <= 0.25 * s_prev[c])) s_fallback = 1;
				}
			}
			__syncthreads();
			if(s_fallback) break;
		}
		if(s_fallback || sh.act[0] || sh.act[1]) {
			// plain FP64 CG from the current x (the residual is in rx, ry)
			fell_back = 1;
			if(!true_residual<RES_FP64, 4>(a, sh, false, false, true)) return;
			if(threadIdx.x == 0) {
				for(int c = 0; c < 2; c++) {
					sh.rn2[c] = sh.tot[2 + c];
					sh.rz[c] = sh.tot[4 + c];
					sh.thr[c] = s_goal[c];
					sh.beta[c] = 0.0;
					sh.act[c] = (!sh.zero[c] && sh.rn2[c] >= s_goal[c]) ? 1 : 0;
				}
			}
			__syncthreads();
			if(!cg_iterate<1>(a, sh, CGVecs{a.rx, a.ry, a.px, a.py, a.Px, a.Py, a.vx, a.vy}, max_it)) return;
		}
	}
	if(blockIdx.x == 0 && threadIdx.x == 0) {
		DevStatus *st = a.st;
		st->cg_solves += 2;
		st->cg_iters += sh.it[0] + sh.it[1];
		st->cg_max_iters = max(st->cg_max_iters, max(sh.it[0], sh.it[1]));
		st->refinements += refinements;
		st->fallbacks += fell_back;
		for(int c = 0; c < 2; c++) {
			const double rel = sh.bn2[c] > 0 ? sqrt(sh.rn2[c] / sh.bn2[c]) : 0.0;
			st->cg_max_rel = fmax(st->cg_max_rel, rel);
			// stopped at the cap (or on a non-finite residual) above the
			// tolerance; sh.thr is the FP64 goal here on every path (the
			// mixed sweeps leave a looser inner threshold only when they
			// reached the goal)
			if(a.fail_noconv && !sh.zero[c] && !(sh.rn2[c] < sh.thr[c])) atomicOr(&st->err, ERR_NOCONV);
		}
		int &restart = a.layer >= 0 ? a.lsolve[a.layer].restart : st->restart;
		if(cold) restart = 0;
		else restart += 1;
	}
}

constexpr size_t LEARNED_SMEM = TC_SMEM > sizeof(float) * UNET_MAX_LAYER_PARAMS ? TC_SMEM : sizeof(float) * UNET_MAX_LAYER_PARAMS;

// The plain solve keeps two CTAs per SM (64 registers); the learned one
// needs the whole register file of one CTA.
// MINB: CTAs per SM the kernel is built for.  The plain solve has a two-CTA
// build (64 registers; box-site phases batch the loads of two unknowns) and,
// for the small boxes that run one CTA per SM, a one-CTA build whose spare
// registers hold the loads of four.
template<bool LEARNED, int MINB = (LEARNED ? 1 : 2)>
__global__ void __launch_bounds__(CG_THREADS, MINB) cg_kernel(const __grid_constant__ CGArgs a) {
	__shared__ CGShared sh;
	extern __shared__ __align__(1024) unsigned char dsm[];
	TcCtx tc{dsm, 0u, {0u, 0u}, &a.st->err, ERR_MMA, a.phase_ns ? a.phase_ns + PH_COUNT : nullptr};
	if(threadIdx.x == 0) {
		sh.epoch = 0u;
		sh.fail = 0;
	}
	__syncthreads();
	if(a.phase_ns && blockIdx.x == 0 && threadIdx.x == 0) sh.tmark = gtimer();
	if constexpr(LEARNED) {
		if(a.unet_tc) {
			uint32_t *hold = reinterpret_cast<uint32_t *>(dsm + TC_HOLD_OFF);
			if(threadIdx.x < 32) tc_alloc(hold, TC_COLS);
			if(threadIdx.x == 0)
				for(int k = 0; k < TC_NMBAR; k++) mbar_init(reinterpret_cast<uint64_t *>(dsm + TC_MBAR_OFF) + k, 1);
			tc_fence_before();
			__syncthreads();
			tc_fence_after();
			tc.tmem = *hold;
		}
	}
	cg_body<LEARNED, LEARNED ? 1 : (MINB == 1 ? 4 : 2)>(a, sh, tc);
	pmark(a, sh, PH_OTHER);
	if constexpr(LEARNED) {
		if(a.unet_tc) {
			tc_fence_before();
			__syncthreads();
			if(threadIdx.x < 32) tc_dealloc(tc.tmem, TC_COLS);
		}
	}
}

// Blocks of the persistent solve.  The plain solve runs two CTAs per SM,
// except on boxes with fewer sites than that grid has threads: there the box-
// site phases leave most threads idle and one CTA per SM, with half the block
// partials to combine at every grid barrier, is faster (256^2: 8.9 against
// 10.4 ms per step; 512^2: 35.7 against 25.2, the other way round).
int cg_grid_blocks(int device, bool learned, long long box_sites) {
	int sms = 0, per_sm = 0;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
	if(learned) {
		cudaFuncSetAttribute(cg_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) LEARNED_SMEM);
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cg_kernel<true>, CG_THREADS, LEARNED_SMEM);
	}
	else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cg_kernel<false>, CG_THREADS, 0);
	if(per_sm < 1) per_sm = 1;
	if(per_sm > 2) per_sm = 2;
	// the learned solve holds all of an SM's TMEM columns: one CTA per SM, or
	// a second CTA would wait in its allocation for one that waits for it
	if(learned) per_sm = 1;
	else if(box_sites < 2LL * sms * CG_THREADS) per_sm = 1;
	const int blocks = sms * per_sm;
	return blocks < 2048 ? blocks : 2048;  // partial sums: 2 x 8 x blocks doubles
}

cudaError_t launch_cg(const CGArgs &a, int blocks, cudaStream_t s) {
	// cooperative launch (all blocks co-resident, required by the grid
	// barriers); cudaLaunchKernelEx form so that it can be captured in a graph
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(blocks);
	cfg.blockDim = dim3(CG_THREADS);
	const bool learned = a.fcg != 0;
	cfg.dynamicSmemBytes = learned ? LEARNED_SMEM : 0;
	cfg.stream = s;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeCooperative;
	attr[0].val.cooperative = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	if(learned) return cudaLaunchKernelEx(&cfg, cg_kernel<true>, a);
	static int sms = 0;
	if(!sms) {
		int dev = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	}
	if(blocks <= sms) return cudaLaunchKernelEx(&cfg, cg_kernel<false, 1>, a);
	return cudaLaunchKernelEx(&cfg, cg_kernel<false, 2>, a);
}

}  // namespace rc
