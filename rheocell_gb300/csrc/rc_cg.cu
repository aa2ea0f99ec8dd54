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
// summed in a fixed order (per-block tree, then the last block to arrive sums
// the block partials in block order), so results are bit-reproducible.
#include "rc_kernels.cuh"

#include <float.h>

namespace rc {

constexpr int CG_THREADS = 512;
constexpr int CG_MAX_D = 4 * STORE_MAX;
constexpr long long BARRIER_SPIN_LIMIT = 4000000;  // about 1-2 s with 64 ns naps

// Scalars block (global): [0..7] reduction results.
enum { SC_RED = 0 };

__device__ __forceinline__ double ldcg(const double *p) { return __ldcg(p); }

// Grid-wide barrier with an optional fixed-order reduction of nv doubles.
// v[i] must hold this block's partial sums (valid in thread 0).  On return,
// out[i] (shared) holds the grid totals in every thread.  Returns false if
// the barrier timed out anywhere.
__device__ bool grid_reduce(const CGArgs &a, int nv, const double *v, double *out, double *red) {
	__shared__ int s_last;
	__shared__ unsigned s_gen;
	__shared__ int s_fail;
	const unsigned nb = gridDim.x;
	if(threadIdx.x == 0) {
		for(int i = 0; i < nv; i++) a.partials[(size_t) i * nb + blockIdx.x] = v[i];
		s_gen = atomicAdd(&a.bar[1], 0u);
		__threadfence();
		const unsigned prev = atomicAdd(&a.bar[0], 1u);
		s_last = (prev == nb - 1);
		s_fail = 0;
	}
	__syncthreads();
	if(s_last) {
		for(int i = 0; i < nv; i++) {
			double acc[1] = {0.0};
			for(unsigned b = threadIdx.x; b < nb; b += blockDim.x) acc[0] += ldcg(&a.partials[(size_t) i * nb + b]);
			block_sum<1>(acc, red);
			if(threadIdx.x == 0) a.scalars[SC_RED + i] = acc[0];
		}
		if(threadIdx.x == 0) {
			__threadfence();
			atomicExch(&a.bar[0], 0u);
			__threadfence();
			atomicAdd(&a.bar[1], 1u);
		}
	}
	else if(threadIdx.x == 0) {
		long long spins = 0;
		while(atomicAdd(&a.bar[1], 0u) == s_gen) {
			if(++spins > BARRIER_SPIN_LIMIT) {
				atomicOr(&a.st->err, ERR_BARRIER);
				s_fail = 1;
				break;
			}
			__nanosleep(64);
		}
		__threadfence();
	}
	__syncthreads();
	if(threadIdx.x == 0 && (atomicAdd(&a.st->err, 0) & ERR_BARRIER)) s_fail = 1;
	__syncthreads();
	for(int i = threadIdx.x; i < nv; i += blockDim.x) out[i] = ldcg(&a.scalars[SC_RED + i]);
	__syncthreads();
	return !s_fail;
}

__device__ __forceinline__ int box_deg(const int *cnt, int k, int L) {
	const int x = k % L, y = k / L;
	const int kr = (x == L - 1) ? k - (L - 1) : k + 1;
	const int kl = (x == 0) ? k + (L - 1) : k - 1;
	const int ku = (y == L - 1) ? k - (L - 1) * L : k + L;
	const int kd = (y == 0) ? k + (L - 1) * L : k - L;
	return cnt[kd] + cnt[kl] + cnt[kr] + cnt[ku];
}

__device__ __forceinline__ double box_n4(const double *P, int k, int L) {
	const int x = k % L, y = k / L;
	const int kr = (x == L - 1) ? k - (L - 1) : k + 1;
	const int kl = (x == 0) ? k + (L - 1) : k - 1;
	const int ku = (y == L - 1) ? k - (L - 1) * L : k + L;
	const int kd = (y == 0) ? k + (L - 1) * L : k - L;
	return P[kd] + P[kl] + P[kr] + P[ku];
}

__global__ void __launch_bounds__(CG_THREADS) cg_kernel(const CGArgs a) {
	__shared__ double T[CG_MAX_D + 1], iT[CG_MAX_D + 1];
	__shared__ double red[8 * (CG_THREADS / 32)];
	__shared__ double tot[8];
	__shared__ double s_rz[2], s_thr[2], s_bn2[2], s_rn2[2], s_alpha[2], s_beta[2];
	__shared__ int s_act[2], s_it[2], s_first, s_zero[2];
	if(threadIdx.x < 2) s_beta[threadIdx.x] = 0.0;
	const int L = a.L;
	const long long L2 = (long long) L * L;
	const long long S = a.st->S;
	const int cold = a.st->cg_cold;
	const double eta = a.eta;
	const double neta = -eta * 1.0;
	const long long gtid = blockIdx.x * (long long) blockDim.x + threadIdx.x;
	const long long gstride = (long long) gridDim.x * blockDim.x;
	if(threadIdx.x == 0) {
		T[0] = a.xi;
		for(int d = 1; d <= CG_MAX_D; d++) T[d] = T[d - 1] + eta * 1.0;
		for(int d = 0; d <= CG_MAX_D; d++) iT[d] = T[d] != 0.0 ? 1.0 / T[d] : 1.0;
	}
	__syncthreads();

	// r = b - A x
	if(!cold) {
		for(long long k = gtid; k < L2; k += gstride) {
			const int n = a.cnt[k];
			double sx = 0.0, sy = 0.0;
			for(int i = 0; i < n; i++) {
				const int j = a.cover[(size_t) i * L2 + k];
				sx += a.vx[j];
				sy += a.vy[j];
			}
			a.Px[k] = sx;
			a.Py[k] = sy;
		}
		if(!grid_reduce(a, 0, nullptr, tot, red)) return;
	}
	{
		double v[6] = {0, 0, 0, 0, 0, 0};
		for(long long j = gtid; j < S; j += gstride) {
			const int k = a.mapg[j];
			const int D = box_deg(a.cnt, k, L);
			const double bx = a.fx[j], by = a.fy[j];
			double rx, ry;
			if(cold) {
				a.vx[j] = 0.0;
				a.vy[j] = 0.0;
				rx = bx - 0.0;
				ry = by - 0.0;
			}
			else {
				const double ax = T[D] * a.vx[j] + neta * box_n4(a.Px, k, L);
				const double ay = T[D] * a.vy[j] + neta * box_n4(a.Py, k, L);
				rx = bx - ax;
				ry = by - ay;
			}
			a.rx[j] = rx;
			a.ry[j] = ry;
			v[0] += bx * bx;
			v[1] += by * by;
			v[2] += rx * rx;
			v[3] += ry * ry;
			v[4] += rx * (iT[D] * rx);
			v[5] += ry * (iT[D] * ry);
		}
		block_sum<6>(v, red);
		if(!grid_reduce(a, 6, v, tot, red)) return;
	}
	if(threadIdx.x == 0) {
		for(int c = 0; c < 2; c++) {
			s_bn2[c] = tot[c];
			s_rn2[c] = tot[2 + c];
			s_rz[c] = tot[4 + c];
			s_it[c] = 0;
			s_zero[c] = 0;
			s_thr[c] = fmax(a.tol * a.tol * s_bn2[c], DBL_MIN);
			if(s_bn2[c] == 0.0) {
				s_act[c] = 0;
				s_zero[c] = 1;
			}
			else s_act[c] = (s_rn2[c] < s_thr[c]) ? 0 : 1;
		}
		s_first = 1;
	}
	__syncthreads();
	if(s_zero[0] || s_zero[1]) {
		for(long long j = gtid; j < S; j += gstride) {
			if(s_zero[0]) a.vx[j] = 0.0;
			if(s_zero[1]) a.vy[j] = 0.0;
		}
	}

	const long long max_it = 2 * S;
	while(s_act[0] || s_act[1]) {
		const int ax = s_act[0], ay = s_act[1], first = s_first;
		const double bx = s_beta[0], by = s_beta[1];
		// Phase A: p = z + beta p (p = z on the first sweep), P = S p
		for(long long k = gtid; k < L2; k += gstride) {
			const int n = a.cnt[k];
			if(n == 0) {
				if(ax) a.Px[k] = 0.0;
				if(ay) a.Py[k] = 0.0;
				continue;
			}
			const double id = iT[box_deg(a.cnt, k, L)];
			double sx = 0.0, sy = 0.0;
			for(int i = 0; i < n; i++) {
				const int j = a.cover[(size_t) i * L2 + k];
				if(ax) {
					const double z = id * a.rx[j];
					const double p = first ? z : z + bx * a.px[j];
					a.px[j] = p;
					sx += p;
				}
				if(ay) {
					const double z = id * a.ry[j];
					const double p = first ? z : z + by * a.py[j];
					a.py[j] = p;
					sy += p;
				}
			}
			if(ax) a.Px[k] = sx;
			if(ay) a.Py[k] = sy;
		}
		if(!grid_reduce(a, 0, nullptr, tot, red)) return;
		// Phase B: p.Ap
		{
			double v[2] = {0, 0};
			for(long long j = gtid; j < S; j += gstride) {
				const int k = a.mapg[j];
				const double d = T[box_deg(a.cnt, k, L)];
				if(ax) {
					const double p = a.px[j];
					v[0] += p * (d * p + neta * box_n4(a.Px, k, L));
				}
				if(ay) {
					const double p = a.py[j];
					v[1] += p * (d * p + neta * box_n4(a.Py, k, L));
				}
			}
			block_sum<2>(v, red);
			if(!grid_reduce(a, 2, v, tot, red)) return;
		}
		if(threadIdx.x == 0) {
			if(ax) s_alpha[0] = s_rz[0] / tot[0];
			if(ay) s_alpha[1] = s_rz[1] / tot[1];
		}
		__syncthreads();
		// Phase C: x += alpha p; r -= alpha Ap; |r|^2 and r.z
		{
			const double alx = s_alpha[0], aly = s_alpha[1];
			double v[4] = {0, 0, 0, 0};
			for(long long j = gtid; j < S; j += gstride) {
				const int k = a.mapg[j];
				const int D = box_deg(a.cnt, k, L);
				const double d = T[D], id = iT[D];
				if(ax) {
					const double p = a.px[j];
					const double ap = d * p + neta * box_n4(a.Px, k, L);
					a.vx[j] = a.vx[j] + alx * p;
					const double r = a.rx[j] - alx * ap;
					a.rx[j] = r;
					v[0] += r * r;
					v[2] += r * (id * r);
				}
				if(ay) {
					const double p = a.py[j];
					const double ap = d * p + neta * box_n4(a.Py, k, L);
					a.vy[j] = a.vy[j] + aly * p;
					const double r = a.ry[j] - aly * ap;
					a.ry[j] = r;
					v[1] += r * r;
					v[3] += r * (id * r);
				}
			}
			block_sum<4>(v, red);
			if(!grid_reduce(a, 4, v, tot, red)) return;
		}
		if(threadIdx.x == 0) {
			for(int c = 0; c < 2; c++) {
				if(!s_act[c]) continue;
				s_rn2[c] = tot[c];
				if(s_rn2[c] < s_thr[c]) {
					s_act[c] = 0;
					continue;
				}
				const double rz_new = tot[2 + c];
				s_beta[c] = rz_new / s_rz[c];
				s_rz[c] = rz_new;
				s_it[c]++;
				if(s_it[c] >= max_it) s_act[c] = 0;
			}
			s_first = 0;
		}
		__syncthreads();
	}
	if(blockIdx.x == 0 && threadIdx.x == 0) {
		DevStatus *st = a.st;
		st->cg_solves += 2;
		st->cg_iters += s_it[0] + s_it[1];
		st->cg_max_iters = max(st->cg_max_iters, max(s_it[0], s_it[1]));
		for(int c = 0; c < 2; c++) {
			const double rel = s_bn2[c] > 0 ? sqrt(s_rn2[c] / s_bn2[c]) : 0.0;
			st->cg_max_rel = fmax(st->cg_max_rel, rel);
		}
		if(cold) st->restart = 0;
		else st->restart += 1;
	}
}

int cg_grid_blocks(int device) {
	int sms = 0, per_sm = 0;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cg_kernel, CG_THREADS, 0);
	if(per_sm < 1) per_sm = 1;
	if(per_sm > 2) per_sm = 2;
	return sms * per_sm;
}

cudaError_t launch_cg(const CGArgs &a, int blocks, cudaStream_t s) {
	void *args[] = {(void *) &a};
	return cudaLaunchCooperativeKernel((const void *) cg_kernel, dim3(blocks), dim3(CG_THREADS), args, 0, s);
}

}  // namespace rc
