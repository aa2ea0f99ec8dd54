// FP32 cell kernels of the GB300 multi-phase-field engine
// (RC_PRECISION_FLOAT): the stages of the FP64 cell kernels (rc_cells.cu)
// with FP32 site arithmetic, for the polar model (wetpolarmodel, dry or wet)
// and the wet nematic model (wetmodel).
//
// Reference functions re-designed here (paths relative to the reference's src/):
//   FD_CPUBackend::first_step ........ Backends/FD_CPUBackend.cpp:44-120
//   f_interaction (chemical potential) WetPolarModel.cpp:262-301, WetModel.cpp:487-613
//   calc_internal_forces ............. WetPolarModel.cpp:304-339, WetModel.cpp:616-694
//
// The force evaluation's mu and gradients, which only the FP32 update reads,
// are kept in FP32 arrays (muf, dxf, dyf): 12 B per site instead of 24, and
// no conversions on either side; downloads and observables widen them.
//
// Precision pattern: the patch, chemical potential, stresses, forces and the
// Heun update run in FP32 (shared memory in FP32); phi, the velocities and
// the right-hand side stay stored in FP64 (the box gather and the viscous
// solve read them unchanged), converted on the integer pipes (on GB300 the conversion instructions issue
// on the narrow FP64 pipe).  The area integral sum(phi^2) that drives the
// area constraint accumulates in double-float (near FP64); the other per-cell
// sums come from FP32 per-thread partials combined in FP64.  This
// translation unit is compiled with FMA contraction: its results are close
// to, not bitwise equal to, the FP64 kernels'.
//
// The wet nematic model's passive force (WetModel.cpp:634-637) is the
// divergence of the stress sigma_xx = f_d - mu phi + 2 gamma lambda (d_x phi)^2,
// sigma_yy = f_d - mu phi + 2 gamma lambda (d_y phi)^2,
// sigma_xy = 2 gamma lambda d_x phi d_y phi, taken by central differences at
// the patch neighbours:
//   F_x = -1/2 (sigma_xx[r] - sigma_xx[l]) - 1/2 (sigma_xy[u] - sigma_xy[d])
//   F_y = -1/2 (sigma_yy[u] - sigma_yy[d]) - 1/2 (sigma_xy[r] - sigma_xy[l]),
// the same terms as the reference's expression, grouped per site: stage 1
// forms the three stress components once per site in shared memory.
#include "rc_cell_dev.cuh"
#include "rc_tc.cuh"

namespace rc {

// Shared-memory float arrays of a kernel: none for an update alone (it
// streams its sites); else phi and, per model,
//   polar: mu, Repulsion;
//   wetmodel: sigma_xx, sigma_yy, sigma_xy, and mu when the update follows
//   the evaluation in the same kernel (dry phases).
__host__ __device__ constexpr int f32_arrays(int model, int eval) {
	return eval == EV_NONE ? 0 : model == M_POLAR ? 3 : (eval == EV_WET_RHS ? 4 : 5);
}

template<int MODEL, int EVAL, int UPD, int BLOCK>
__global__ void __launch_bounds__(BLOCK) cell_kernel_f32(const CellArgs a) {
	static_assert(MODEL == M_POLAR || MODEL == M_WET, "FP32 kernels: polar and wet nematic models");
	extern __shared__ __align__(16) unsigned char smem_raw[];
	__shared__ CellDev c;
	__shared__ double red[12 * (BLOCK / 32 + 1)];
	__shared__ int ired[2 * (BLOCK / 32)];
	const int ci = blockIdx.x;
	{
		const int *src = reinterpret_cast<const int *>(&a.cells[ci]);
		int *dst = reinterpret_cast<int *>(&c);
		for(int i = threadIdx.x; i < (int) (sizeof(CellDev) / 4); i += blockDim.x) dst[i] = src[i];
	}
	__syncthreads();
	const LayerDev lay = a.layers[c.layer];
	const int n = c.n, lx = c.lx, ly = c.ly, L = lay.L, start = c.start;
	const double *phi2 = a.phi2 + lay.box_off;
	const double *sq00 = a.sq00 + lay.box_off;
	const double *sq01 = a.sq01 + lay.box_off;
	const int cx0 = c.corner % L, cy0 = c.corner / L;
	// box coordinates of patch site (x, y): GetSubIndex without divisions
	auto box_xy = [&](int x, int y, int &bx, int &by) {
		int px = x + c.offx;
		if(px >= lx) px -= lx;
		int py = y + c.offy;
		if(py >= ly) py -= ly;
		bx = cx0 + px;
		if(bx >= L) bx -= L;
		by = cy0 + py;
		if(by >= L) by -= L;
	};
	if(n > a.smem_n) {
		if(threadIdx.x == 0) {
			atomicOr(&a.st->err, ERR_CAPACITY);
			a.st->err_where = ci;
		}
		return;
	}
	// polar: phi | mu | Repulsion; wetmodel: phi | sigma_xx | sigma_yy | sigma_xy [| mu]
	float *sphi = reinterpret_cast<float *>(smem_raw);
	float *smu = sphi + a.smem_n;
	float *saux = smu + a.smem_n;
	float *sxy = saux + a.smem_n;
	float *smw = sxy + a.smem_n;
	const DevParams &P = a.P;
	const PhaseParams &pe = a.pe;
	// Per-cell constants, formed once by thread 0: on GB300 an FP64 warp
	// instruction (a division is ~10 of them) costs tens of issue cycles, too
	// many to repeat in every thread.
	enum { K_GAMMA, K_LAMBDA, K_OMEGA, K_RLAMBDA, K_AC, K_REPC, K_J0, K_HDT, K_ZS, K_ZI, K_ALPHA, K_RFR, K_Q00, K_Q01,
	       K_BETA, K_HAS_BETA, K_HAS_OMEGA, K_CHD, K_GL, K_AD, K_KL, K_G2, K_N };
	__shared__ float kc[K_N];
	__shared__ double s_perim;
	if(threadIdx.x == 0) {
		kc[K_GAMMA] = (float) P.gamma;
		kc[K_LAMBDA] = (float) P.lambda;
		kc[K_OMEGA] = (float) P.omega;
		kc[K_RLAMBDA] = (float) (1.0 / P.lambda);
		kc[K_AC] = (float) (-4 * (P.mu / P.a0) * (1 - c.area / P.a0));
		kc[K_REPC] = (float) (4 * (P.kappa / P.lambda));
		kc[K_J0] = (float) P.J0;
		kc[K_HDT] = (float) (P.dt * .5);
		kc[K_ZS] = (float) pe.zs;
		kc[K_ZI] = (float) pe.zi;
		kc[K_ALPHA] = (float) P.passive_alpha;
		kc[K_RFR] = (float) (1.0 / pe.friction);
		kc[K_Q00] = (float) c.q00;
		kc[K_Q01] = (float) c.q01;
		kc[K_HAS_BETA] = (MODEL == M_POLAR && pe.beta != 0.0) ? 1.f : 0.f;
		kc[K_HAS_OMEGA] = P.omega != 0.0 ? 1.f : 0.f;
		// wetmodel free-energy density (WetModel.cpp:607-611)
		kc[K_CHD] = (float) ((P.gamma / P.lambda) * 4);
		kc[K_GL] = (float) (P.gamma * P.lambda);
		kc[K_AD] = (float) (-P.mu / P.a0);
		kc[K_KL] = (float) (P.kappa / P.lambda);
		kc[K_G2] = (float) (2 * P.gamma * P.lambda);
	}
	__syncthreads();
	const float gamma = kc[K_GAMMA], lambda = kc[K_LAMBDA], omega = kc[K_OMEGA];
	const float rlambda = kc[K_RLAMBDA], two_lambda = 2.f * lambda;
	const float A_c = kc[K_AC], Rep_c = kc[K_REPC];
	double perim = 0.0;
	const bool has_beta = kc[K_HAS_BETA] != 0.f, has_omega = kc[K_HAS_OMEGA] != 0.f;
	if(EVAL != EV_NONE) {
		for(int q = threadIdx.x; q < n; q += blockDim.x) sphi[q] = d2f_int(a.phi_eval[start + q]);
		__syncthreads();
		if(MODEL == M_POLAR && has_beta) {
			float pp = 0.f;
			for(PatchWalk w(lx); w.q < n; w.next()) {
				const int q = w.q, x = w.x, y = w.y;
				const Nb nb = patch_nb(q, x, y, lx, ly);
				const float dx = .5f * (sphi[nb.r] - sphi[nb.l]);
				const float dy = .5f * (sphi[nb.u] - sphi[nb.d]);
				pp += dx * dx + dy * dy;
			}
#pragma unroll
			for(int o = 16; o > 0; o >>= 1) pp += __shfl_down_sync(0xffffffffu, pp, o);
			__shared__ float s_pp[BLOCK / 32];
			if((threadIdx.x & 31) == 0) s_pp[threadIdx.x >> 5] = pp;
			__syncthreads();
			if(threadIdx.x == 0) {
				double t = 0.0;
				for(int w = 0; w < (int) (blockDim.x >> 5); w++) t += (double) s_pp[w];
				s_perim = t;
				kc[K_BETA] = (float) (4 * (pe.beta / 12.) * (1 - t / 12.));
			}
			__syncthreads();
			perim = s_perim;
		}
		const float beta_t = has_beta ? kc[K_BETA] : 0.f;
		const float CHd_c = kc[K_CHD], gl_c = kc[K_GL], Ad_c = kc[K_AD], kl_c = kc[K_KL], g2 = kc[K_G2];
		// Stage 1: chemical potential (and the wetmodel's stress) per site.
		for(PatchWalk w(lx); w.q < n; w.next()) {
			const int q = w.q, x = w.x, y = w.y;
			const Nb nb = patch_nb(q, x, y, lx, ly);
			const float phi = sphi[q];
			const float pr = sphi[nb.r], pl = sphi[nb.l], pu_ = sphi[nb.u], pd = sphi[nb.d];
			int bx, by;
			box_xy(x, y, bx, by);
			const int k = bx + by * L;
			const float p2 = d2f_int(phi2[k]);
			const float lap = pu_ + pd + pr + pl - 4.f * phi;
			const float dx = .5f * (pr - pl), dy = .5f * (pu_ - pd);
			const float CH = gamma * (8.f * phi * (1.f - phi) * (1.f - 2.f * phi) * rlambda - two_lambda * lap);
			const float Rep = Rep_c * phi * (p2 - phi * phi);
			float V = CH + A_c * phi + Rep;
			if(has_omega) {
				const int kr = (bx == L - 1) ? k - (L - 1) : k + 1, kl = (bx == 0) ? k + (L - 1) : k - 1;
				const int ku = (by == L - 1) ? k - (L - 1) * L : k + L, kd = (by == 0) ? k + (L - 1) * L : k - L;
				const float ls = (float) (phi2[kr] + phi2[ku] + phi2[kl] + phi2[kd] - 4. * phi2[k]);
				const float lsq = 2.f * phi * lap + 2.f * (dx * dx + dy * dy);
				const float sup = (ls - lsq) * rsqrtf(1.f + (ls - lsq) * (ls - lsq));
				V = V + (-4.f * lambda * omega * sup * phi);
			}
			if(MODEL == M_POLAR && has_beta) V = V + beta_t * lap;
			if(EVAL == EV_STORE || EVAL == EV_WET_RHS) {
				a.muf[start + q] = V;
				a.dxf[start + q] = dx;
				a.dyf[start + q] = dy;
				a.mapg[start + q] = k;
			}
			if(MODEL == M_POLAR) {
				if(a.rep_on) {
					const float r = d2f_int(a.rep[start + q]) + Rep;
					if(a.accumulate_rep) a.rep[start + q] = f2d_int(r);
					saux[q] = r;
				}
				smu[q] = V;
			}
			else {
				const float pp = phi * phi;
				const float fd = CHd_c * pp * (1.f - phi) * (1.f - phi) + gl_c * (dx * dx + dy * dy) + Ad_c * pp +
				                 kl_c * pp * (p2 - pp);
				const float s = fd - V * phi;
				smu[q] = s + g2 * dx * dx;
				saux[q] = s + g2 * dy * dy;
				sxy[q] = g2 * dx * dy;
				if(f32_arrays(MODEL, EVAL) == 5) smw[q] = V;
			}
		}
		__syncthreads();
	}
	float af[12];
#pragma unroll
	for(int i = 0; i < 12; i++) af[i] = 0.f;
	int imin[2] = {lx, ly};
	float area_s = 0.f, area_c = 0.f;
	const float J0 = kc[K_J0], hdt = kc[K_HDT];
	const bool conserved = P.conserved != 0;
	const float zs = kc[K_ZS], zi = kc[K_ZI], alpha = kc[K_ALPHA], lam = lambda;
	const float rfr = kc[K_RFR];
	const int tb = table_base(lx), tby = table_base(ly);
	const float q00 = kc[K_Q00], q01 = kc[K_Q01];
	// The update of a site (first_step) from its dphi inputs; shared by the
	// batched update-only loop and the evaluate-and-update loop below.
	auto update_site = [&](int q, int x, int y, float dphi, float phi_pre, float dphi_prev) {
		float phi_new;
		if(UPD == UP_PRED) {
			a.dphif[start + q] = dphi;
			phi_new = phi_pre + hdt * (dphi + dphi);
		}
		else {
			phi_new = phi_pre + hdt * (dphi + dphi_prev);
		}
		a.phi_out[start + q] = f2d_int(phi_new);
		acc_square(phi_new, area_s, area_c);
		af[1] += phi_new;
		int lxx = x + c.offx;
		if(lxx >= lx) lxx -= lx;
		int lyy = y + c.offy;
		if(lyy >= ly) lyy -= ly;
		af[2] += phi_new * a.tab_cosf[tb + lxx];
		af[3] += phi_new * a.tab_sinf[tb + lxx];
		af[4] += phi_new * a.tab_cosf[tby + lyy];
		af[5] += phi_new * a.tab_sinf[tby + lyy];
		if(UPD == UP_CORR && phi_new < 0.09f && phi_new > 0.01f) {
			imin[0] = min(imin[0], lxx);
			imin[1] = min(imin[1], lyy);
		}
	};
	// Stage 2: forces (calc_internal_forces) and the update (first_step).
	// (The wet models' update alone after the solve is cell_update_bulk
	// below; this kernel runs it only for conserved dynamics.)
	for(PatchWalk w(lx); w.q < n; w.next()) {
		const int q = w.q, x = w.x, y = w.y;
		float mu = 0.f, vx = 0.f, vy = 0.f, dx, dy, phi_e = 0.f;
		if(EVAL != EV_NONE) {
			const Nb nb = patch_nb(q, x, y, lx, ly);
			phi_e = sphi[q];
			dx = .5f * (sphi[nb.r] - sphi[nb.l]);
			dy = .5f * (sphi[nb.u] - sphi[nb.d]);
			float fx, fy;
			if(MODEL == M_POLAR) {
				mu = smu[q];
				const float fpx = -.5f * (smu[nb.r] - smu[nb.l]);
				const float fpy = -.5f * (smu[nb.u] - smu[nb.d]);
				if(a.rep_on) {
					af[8] += -.5f * (saux[nb.r] - saux[nb.l]) * phi_e;
					af[9] += -.5f * (saux[nb.u] - saux[nb.d]) * phi_e;
				}
				const float sx = -dx * q00, sy = -dy * q01;
				const float fsx = sx < 0.f ? 0.f : lam * sx * q00;
				const float fsy = sy < 0.f ? 0.f : lam * sy * q01;
				fx = fpx * alpha + fsx * zs;
				fy = fpy * alpha + fsy * zs;
				af[10] += fx * phi_e;
				af[11] += fy * phi_e;
			}
			else {
				// self and inter nematic forces (WetModel.cpp:641-656) from the
				// cell's Q and the box sums of phi Q at the box neighbours
				int bx, by;
				box_xy(x, y, bx, by);
				const int k = bx + by * L;
				const int kr = (bx == L - 1) ? k - (L - 1) : k + 1, kl = (bx == 0) ? k + (L - 1) : k - 1;
				const int ku = (by == L - 1) ? k - (L - 1) * L : k + L, kd = (by == 0) ? k + (L - 1) * L : k - L;
				const float a0r = d2f_int(sq00[kr]), a0l = d2f_int(sq00[kl]), a0u = d2f_int(sq00[ku]),
				            a0d = d2f_int(sq00[kd]);
				const float a1r = d2f_int(sq01[kr]), a1l = d2f_int(sq01[kl]), a1u = d2f_int(sq01[ku]),
				            a1d = d2f_int(sq01[kd]);
				const float fsx = -(q00 * dx + q01 * dy);
				const float fsy = -(q01 * dx - q00 * dy);
				const float fix = -(.5f * (a0r - a0l) + .5f * (a1u - a1d)) - fsx;
				const float fiy = -(.5f * (a1r - a1l) - .5f * (a0u - a0d)) - fsy;
				const float fpx = -.5f * (smu[nb.r] - smu[nb.l]) - .5f * (sxy[nb.u] - sxy[nb.d]);
				const float fpy = -.5f * (saux[nb.u] - saux[nb.d]) - .5f * (sxy[nb.r] - sxy[nb.l]);
				fx = fpx * alpha + fsx * zs + fix * zi;
				fy = fpy * alpha + fsy * zs + fiy * zi;
				if(f32_arrays(MODEL, EVAL) == 5) mu = smw[q];
			}
			if(EVAL == EV_WET_RHS) {
				a.fxg[start + q] = f2d_int(fx);
				a.fyg[start + q] = f2d_int(fy);
			}
			else {
				vx = fx * rfr;
				vy = fy * rfr;
				if(EVAL == EV_STORE) {
					a.vxg[start + q] = f2d_int(vx);
					a.vyg[start + q] = f2d_int(vy);
				}
			}
		}
		else {
			mu = a.muf[start + q];
			vx = d2f_int(a.vxg[start + q]);
			vy = d2f_int(a.vyg[start + q]);
			dx = a.dxf[start + q];
			dy = a.dyf[start + q];
		}
		if(UPD == UP_NONE) continue;
		float dphi;
		if(conserved) {
			// FD_CH (FD_CHBackend.cpp:63-68); the polar and wet models keep every
			// neighbour's freeEnergy through the loop (WetPolarModel.cpp:130,
			// WetModel.cpp:167)
			const Nb nb = patch_nb(q, x, y, lx, ly);
			auto fe = [&](int s_) {
				if(EVAL == EV_NONE) return a.muf[start + s_];
				return MODEL == M_POLAR ? smu[s_] : smw[s_];
			};
			const float lmu = fe(nb.r) + fe(nb.u) + fe(nb.l) + fe(nb.d) - 4.f * mu;
			dphi = J0 * lmu - vx * dx - vy * dy;
		}
		else
			dphi = -J0 * mu - vx * dx - vy * dy;
		if(UPD == UP_PRED) update_site(q, x, y, dphi, (EVAL != EV_NONE) ? phi_e : d2f_int(a.phi_eval[start + q]), 0.f);
		else update_site(q, x, y, dphi, d2f_int(a.phi_old[start + q]), a.dphif[start + q]);
		af[6] += -.5f * (dx * dx - dy * dy);
		af[7] += -dx * dy;
	}
	if(a.split) {
		// per-warp partials for the epilogue kernel: FP32 warp trees, the area
		// as a double-float pair, converted once per warp
		const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
		for(int o = 16; o > 0; o >>= 1) {
			const float s2 = __shfl_down_sync(0xffffffffu, area_s, o);
			const float c2 = __shfl_down_sync(0xffffffffu, area_c, o);
			add_df(area_s, area_c, s2, c2);
#pragma unroll
			for(int i = 1; i < 12; i++) af[i] += __shfl_down_sync(0xffffffffu, af[i], o);
		}
		if(UPD == UP_CORR) block_min<2>(imin, ired);
		CellSum &o = a.csum[ci];
		if(lane == 0) {
			o.area[warp] = (double) area_s + (double) area_c;
#pragma unroll
			for(int i = 1; i < 12; i++) o.part[warp][i] = af[i];
		}
		if(threadIdx.x == 0) {
			o.imin[0] = imin[0];
			o.imin[1] = imin[1];
			o.nw = BLOCK / 32;
			o.perim = perim;
		}
		return;
	}
	double acc[12];
	acc[0] = (double) area_s + (double) area_c;
	// per-cell sums: warp trees in FP32 (the area term in FP64), then the
	// warps' partial sums in FP64 by one warp; the totals are needed by thread 0 only
	{
		const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
		for(int o = 16; o > 0; o >>= 1) {
			acc[0] += __shfl_down_sync(0xffffffffu, acc[0], o);
#pragma unroll
			for(int i = 1; i < 12; i++) af[i] += __shfl_down_sync(0xffffffffu, af[i], o);
		}
		if(lane == 0) {
			red[warp] = acc[0];
#pragma unroll
			for(int i = 1; i < 12; i++) red[i * nw + warp] = (double) af[i];
		}
		__syncthreads();
		if(warp == 0) {
#pragma unroll
			for(int i = 0; i < 12; i++) {
				double t = lane < nw ? red[i * nw + lane] : 0.0;
#pragma unroll
				for(int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
				acc[i] = t;
			}
		}
	}
	if(UPD == UP_CORR) block_min<2>(imin, ired);
	if(threadIdx.x == 0) cell_finish<MODEL, EVAL, UPD>(c, acc, imin, perim, a, lay, ci);
	__syncthreads();
	{
		const int *src = reinterpret_cast<const int *>(&c);
		int *dst = reinterpret_cast<int *>(&a.cells[ci]);
		for(int i = threadIdx.x; i < (int) (sizeof(CellDev) / 4); i += blockDim.x) dst[i] = src[i];
	}
}

// The wet models' update alone, after the viscous solve (first_step,
// FD_CPUBackend.cpp:44-120): dphi = -J0 mu - v . grad phi from the last
// evaluation's mu and gradient, phi* = phi + dt dphi (predictor) or
// phi^{n+1} = phi^n + dt/2 (dphi + dphi^n) (corrector), and the per-cell
// sums of the new phi, one CTA per cell.
//
// A pure stream, staged by the Tensor Memory Accelerator: thread 0 moves
// each chunk of CH sites of every input array into shared memory with one
// bulk copy per array (cp.async.bulk, completion counted in bytes on the
// stage's mbarrier), NST chunks ahead of the threads, so the bytes in flight
// do not depend on how many loads each thread keeps outstanding.  The copies
// move 16-byte aligned windows around the chunk (up to 3 floats or 1 double
// of slack at each end; the engine pads the arrays by 8 elements so that a
// window never leaves its allocation); values in the slack belong to
// neighbouring sites and are never used.  In the corrector phi^n is read and
// phi^{n+1} written in place: a site's new value is written only after its
// chunk has landed, and no site's value is read from another chunk's
// window.  Every completion wait is bounded (ERR_COPY).
//
// Per site: no set-up beyond the patch's trig rows (centre-of-mass sums),
// staged once per cell already rotated by the patch offset; the double ->
// float conversions in the short integer form (d2f_fast); the area sum in
// double-float.  Per-warp partial sums go to the epilogue kernel
// (cell_finish_kernel), which every FP32 wet engine runs.
constexpr long long UPD_WAIT_LIMIT = 1LL << 22;  // mbarrier polls

template<int UPD>
struct UpdStage {
	static constexpr int NF = UPD == UP_CORR ? 4 : 3;  // FP32 inputs: mu, d_x phi, d_y phi [, dphi^n]
};

template<int UPD, int BLOCK, int CH, int NST>
__global__ void __launch_bounds__(BLOCK) cell_update_bulk(const CellArgs a) {
	static_assert(CH % BLOCK == 0, "a chunk is a whole number of thread strides");
	constexpr int NF = UpdStage<UPD>::NF;
	constexpr int FW = CH + 8, DW = CH + 4;  // window capacities (floats, doubles)
	constexpr int STAGE = NF * FW * 4 + 3 * DW * 8;
	static_assert((FW * 4) % 16 == 0 && (DW * 8) % 16 == 0 && STAGE % 16 == 0, "16-byte aligned windows");
	extern __shared__ __align__(16) unsigned char stage_mem[];
	__shared__ float2 trow[2 * MAX_TABLE_SIDE];
	__shared__ __align__(8) uint64_t full[NST];
	const int ci = blockIdx.x;
	const CellDev *cp = a.cells + ci;
	const int lx = cp->lx, ly = cp->ly, n = cp->n;
	const long long start = cp->start;
	const int nch = (n + CH - 1) / CH;
	const double *pin = UPD == UP_PRED ? a.phi_eval : a.phi_old;
	// chunk c into stage s: the float windows, then vx, vy, phi
	auto issue = [&](int c, int s) {
		const long long i0 = start + (long long) c * CH;
		const int cnt = min(CH, n - c * CH);
		const long long fa = i0 & ~3LL, fe = (i0 + cnt + 3) & ~3LL;
		const long long da = i0 & ~1LL, de = (i0 + cnt + 1) & ~1LL;
		const uint32_t fb = (uint32_t) (fe - fa) * 4u, db = (uint32_t) (de - da) * 8u;
		unsigned char *base = stage_mem + (size_t) s * STAGE;
		mbar_expect_tx(&full[s], NF * fb + 3 * db);
		bulk_g2s(base, a.muf + fa, fb, &full[s]);
		bulk_g2s(base + FW * 4, a.dxf + fa, fb, &full[s]);
		bulk_g2s(base + 2 * FW * 4, a.dyf + fa, fb, &full[s]);
		if(UPD == UP_CORR) bulk_g2s(base + 3 * FW * 4, a.dphif + fa, fb, &full[s]);
		bulk_g2s(base + NF * FW * 4, a.vxg + da, db, &full[s]);
		bulk_g2s(base + NF * FW * 4 + DW * 8, a.vyg + da, db, &full[s]);
		bulk_g2s(base + NF * FW * 4 + 2 * DW * 8, pin + da, db, &full[s]);
	};
	if(threadIdx.x == 0) {
		for(int s = 0; s < NST; s++) mbar_init(&full[s], 1);
		for(int c = 0; c < min(NST, nch); c++) issue(c, c);
	}
	{
		const int offx = cp->offx, offy = cp->offy, tb = table_base(lx), tby = table_base(ly);
		for(int i = threadIdx.x; i < lx + ly; i += BLOCK) {
			int t;
			if(i < lx) {
				int j = i + offx;
				if(j >= lx) j -= lx;
				t = tb + j;
			}
			else {
				int j = i - lx + offy;
				if(j >= ly) j -= ly;
				t = tby + j;
			}
			trow[i] = make_float2(a.tab_cosf[t], a.tab_sinf[t]);
		}
	}
	const float J0 = d2f_int(a.P.J0), hdt = .5f * d2f_int(a.P.dt);
	float *dold = a.dphif + start;
	double *pout = a.phi_out + start;
	float sm[8];
#pragma unroll
	for(int i = 0; i < 8; i++) sm[i] = 0.f;
	float area_s = 0.f, area_c = 0.f;
	int imx = lx, imy = ly;
	const int sy = BLOCK / lx, sx = BLOCK - sy * lx;
	int y = (int) threadIdx.x / lx, x = (int) threadIdx.x - y * lx;
	bool ok = true;
	__syncthreads();  // barriers initialised, trig rows staged
	int c_stop = nch;  // first chunk not consumed
	for(int c = 0; c < nch; c++) {
		const int s = c % NST;
		// every thread acquires the stage itself; a timeout anywhere stops all
		const bool got = mbar_wait(&full[s], (uint32_t) ((c / NST) & 1), UPD_WAIT_LIMIT);
		if(__syncthreads_or(!got)) {
			ok = false;
			c_stop = c;
			break;
		}
		const long long i0 = start + (long long) c * CH;
		const unsigned char *base = stage_mem + (size_t) s * STAGE;
		const float *smu = reinterpret_cast<const float *>(base) + (i0 & 3);
		const float *sdx = smu + FW, *sdy = smu + 2 * FW, *sdp = smu + 3 * FW;
		const double *svx = reinterpret_cast<const double *>(base + NF * FW * 4) + (i0 & 1);
		const double *svy = svx + DW, *sph = svx + 2 * DW;
#pragma unroll
		for(int u = 0; u < CH / BLOCK; u++) {
			const int j = (int) threadIdx.x + u * BLOCK, q = c * CH + j;
			if(q < n) {
				const float dx = sdx[j], dy = sdy[j];
				const float dphi = -J0 * smu[j] - d2f_fast(svx[j]) * dx - d2f_fast(svy[j]) * dy;
				float pn;
				if(UPD == UP_PRED) {
					dold[q] = dphi;
					pn = d2f_fast(sph[j]) + hdt * (dphi + dphi);
				}
				else {
					pn = d2f_fast(sph[j]) + hdt * (dphi + sdp[j]);
				}
				pout[q] = f2d_int(pn);
				acc_square(pn, area_s, area_c);
				sm[1] += pn;
				const float2 cx = trow[x], cy = trow[lx + y];
				sm[2] += pn * cx.x;
				sm[3] += pn * cx.y;
				sm[4] += pn * cy.x;
				sm[5] += pn * cy.y;
				if(UPD == UP_CORR && pn < 0.09f && pn > 0.01f) {
					int lxx = x + cp->offx, lyy = y + cp->offy;
					if(lxx >= lx) lxx -= lx;
					if(lyy >= ly) lyy -= ly;
					imx = min(imx, lxx);
					imy = min(imy, lyy);
				}
				sm[6] += -.5f * (dx * dx - dy * dy);
				sm[7] += -dx * dy;
			}
			x += sx;
			y += sy;
			if(x >= lx) {
				x -= lx;
				y += 1;
			}
		}
		__syncthreads();  // stage s read by every thread: refill it
		if(threadIdx.x == 0 && c + NST < nch) issue(c + NST, s);
	}
	if(!ok) {
		// a completion wait ran out: report, then let the copies still in
		// flight land (bounded) before the shared memory is released
		if(threadIdx.x == 0) {
			atomicOr(&a.st->err, ERR_COPY);
			a.st->err_where = ci;
			for(int c = c_stop; c < min(nch, c_stop + NST); c++)
				mbar_wait(&full[c % NST], (uint32_t) ((c / NST) & 1), UPD_WAIT_LIMIT);
		}
		return;
	}
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
	for(int o = 16; o > 0; o >>= 1) {
		const float s2 = __shfl_down_sync(0xffffffffu, area_s, o);
		const float c2 = __shfl_down_sync(0xffffffffu, area_c, o);
		add_df(area_s, area_c, s2, c2);
#pragma unroll
		for(int i = 1; i < 8; i++) sm[i] += __shfl_down_sync(0xffffffffu, sm[i], o);
	}
	CellSum &o = a.csum[ci];
	if(lane == 0) {
		o.area[warp] = (double) area_s + (double) area_c;
#pragma unroll
		for(int i = 1; i < 8; i++) o.part[warp][i] = sm[i];
#pragma unroll
		for(int i = 8; i < 12; i++) o.part[warp][i] = 0.f;
	}
	if(UPD == UP_CORR) {
		__shared__ int ired[2 * (BLOCK / 32)];
		int im[2] = {imx, imy};
		block_min<2>(im, ired);
		imx = im[0];
		imy = im[1];
	}
	if(threadIdx.x == 0) {
		o.imin[0] = imx;
		o.imin[1] = imy;
		o.nw = BLOCK / 32;
		o.perim = 0.0;
	}
}

constexpr int UPD_BULK_BLOCK = 128, UPD_BULK_CH = 512, UPD_BULK_NST = 2;

template<int UPD>
constexpr size_t upd_bulk_smem() {
	return (size_t) UPD_BULK_NST *
	       (UpdStage<UPD>::NF * (UPD_BULK_CH + 8) * 4 + 3 * (UPD_BULK_CH + 4) * 8);
}

// The update's inputs are engine allocations (cudaMalloc: 256-byte aligned),
// as the bulk copies need.
static void launch_update_bulk(int upd, const CellArgs &a, cudaStream_t s) {
	constexpr int B = UPD_BULK_BLOCK, CH = UPD_BULK_CH, NST = UPD_BULK_NST;
	if(upd == UP_PRED) cell_update_bulk<UP_PRED, B, CH, NST><<<a.N, B, upd_bulk_smem<UP_PRED>(), s>>>(a);
	else cell_update_bulk<UP_CORR, B, CH, NST><<<a.N, B, upd_bulk_smem<UP_CORR>(), s>>>(a);
}

// (eval, upd) pairs with an FP32 kernel, for every model and tile
#define RC_F32_MODES(X)      \
	X(EV_LOCAL, UP_PRED)     \
	X(EV_LOCAL, UP_CORR)     \
	X(EV_NONE, UP_PRED)      \
	X(EV_NONE, UP_CORR)      \
	X(EV_STORE, UP_NONE)     \
	X(EV_WET_RHS, UP_NONE)

template<int MODEL, int BLOCK>
static bool launch_f32_mb(int eval, int upd, const CellArgs &a, cudaStream_t s) {
	const size_t smem = sizeof(float) * (size_t) f32_arrays(MODEL, eval) * (size_t) a.smem_n;
#define RC_LAUNCH(EV, UP)                                                          \
	if(eval == EV && upd == UP) {                                                  \
		cell_kernel_f32<MODEL, EV, UP, BLOCK><<<a.N, BLOCK, smem, s>>>(a);         \
		return true;                                                               \
	}
	RC_F32_MODES(RC_LAUNCH)
#undef RC_LAUNCH
	return false;
}

template<int MODEL>
static bool launch_f32_m(int eval, int upd, const CellArgs &a, cudaStream_t s, int block) {
	if(block == 128) return launch_f32_mb<MODEL, 128>(eval, upd, a, s);
	if(block == 512) return launch_f32_mb<MODEL, 512>(eval, upd, a, s);
	return launch_f32_mb<MODEL, 256>(eval, upd, a, s);
}

bool launch_cell_kernel_f32(int model, int eval, int upd, const CellArgs &a, cudaStream_t s, int block) {
	if((model == M_POLAR || model == M_WET) && eval == EV_NONE && upd != UP_NONE && a.split && !a.P.conserved) {
		if(a.N > 0) launch_update_bulk(upd, a, s);
		return true;
	}
	if(model == M_POLAR) {
		if(a.N <= 0) return true;
		return launch_f32_m<M_POLAR>(eval, upd, a, s, block);
	}
	if(model == M_WET) {
		if(a.N <= 0) return true;
		return launch_f32_m<M_WET>(eval, upd, a, s, block);
	}
	return false;
}

template<int MODEL, int BLOCK>
static cudaError_t configure_f32_mb() {
	cudaError_t e = cudaSuccess, c;
	const int mx = 200 * 1024;
#define RC_CFG(EV, UP)                                                                                              \
	if((c = cudaFuncSetAttribute(cell_kernel_f32<MODEL, EV, UP, BLOCK>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
	                             mx)) != cudaSuccess)                                                                \
		e = c;
	RC_F32_MODES(RC_CFG)
#undef RC_CFG
	return e;
}

cudaError_t configure_kernels_f32() {
	cudaError_t e = cudaSuccess, c;
	if((c = configure_f32_mb<M_POLAR, 128>()) != cudaSuccess) e = c;
	if((c = configure_f32_mb<M_POLAR, 256>()) != cudaSuccess) e = c;
	if((c = configure_f32_mb<M_POLAR, 512>()) != cudaSuccess) e = c;
	if((c = configure_f32_mb<M_WET, 128>()) != cudaSuccess) e = c;
	if((c = configure_f32_mb<M_WET, 256>()) != cudaSuccess) e = c;
	if((c = configure_f32_mb<M_WET, 512>()) != cudaSuccess) e = c;
	return e;
}

}  // namespace rc
