// Per-cell kernels of the GB300 multi-phase-field engine: force evaluation,
// Heun predictor/corrector update, per-cell reductions and the per-cell
// scalar dynamics, fused in one CTA per cell with the patch in shared memory.
//
// Reference functions re-designed here (paths relative to the reference's src/):
//   FD_CPUBackend::first_step ........ Backends/FD_CPUBackend.cpp:44-120
//   computeGlobalSums stencils ....... Interactions/*::computeGlobalSums and
//                                      BaseInteraction.h:196-263
//   f_interaction (chemical potential) SimpleMultiField.cpp:141-184,
//                                      ActiveNematic.cpp:176-230,
//                                      WetPolarModel.cpp:381-420, WetModel.cpp:487-613
//   calc_internal_forces ............. ActiveNematic.cpp:233-254,
//                                      WetPolarModel.cpp:423-458, WetModel.cpp:616-694
//   updateDirectedActiveForces ....... WetPolarModel.cpp:461-533,
//                                      WetModel.cpp:697-747, ActiveNematic.cpp:257-289
//   set_positions / check_borders .... Fields/MultiPhaseField.cpp:223-344
//   Utils::gaussian (drand48 stream) . Utilities/Utils.h:210-236
//
// The patch of a cell is a periodic torus (Fields/MultiPhaseField.cpp:188-208),
// so one CTA holding the whole patch needs no halo from any other cell; the
// only coupling between cells goes through the box arrays (phi^2, phi*Q sums),
// which the box gather (rc_box.cu) produces before each evaluation.
//
// Arithmetic is IEEE FP64 in the reference's order of operations and the
// library is compiled without FMA contraction, so a single evaluation is
// bit-identical to the reference's exact build; per-cell sums use a fixed
// tree instead of the reference's sequential loop (last-bit differences).
#include "rc_kernels.cuh"

#include <math.h>

namespace rc {

#define RC_PI_F 3.141592653589793238462643f

enum { EVB = 0 };

__device__ inline int box_el(int site, int dx, int dy, int L) {
	return wrapi(site % L + dx, L) + wrapi(site / L + dy, L) * L;
}

// Correctly rounded x / b from rb = RN(1/b): q = RN(x rb), the exact
// remainder x - q b by FMA, and one correction q + rem rb (Markstein's
// reciprocal-based division, P. Markstein, IBM J. Res. Dev. 34 (1990) 111-119).
// Three FP64 instructions instead of a full division; the result equals the
// IEEE quotient, which tests/test_gpu_parity.py checks bitwise against the
// CPU restatement's divisions on whole force evaluations.
__device__ __forceinline__ double div_rn(double x, double b, double rb) {
	const double q = x * rb;
	const double rem = __fma_rn(-q, b, x);
	return __fma_rn(rem, rb, q);
}

struct Nb {
	int r, l, u, d;
};

__device__ inline Nb patch_nb(int q, int x, int y, int lx, int ly) {
	Nb nb;
	nb.r = (x == lx - 1) ? q - (lx - 1) : q + 1;
	nb.l = (x == 0) ? q + (lx - 1) : q - 1;
	nb.u = (y == ly - 1) ? q - (ly - 1) * lx : q + lx;
	nb.d = (y == 0) ? q + (ly - 1) * lx : q - lx;
	return nb;
}

struct BoxNb {
	int r, l, u, d;
};

__device__ inline BoxNb box_nb(int k, int L) {
	const int x = k % L, y = k / L;
	BoxNb b;
	b.r = (x == L - 1) ? k - (L - 1) : k + 1;
	b.l = (x == 0) ? k + (L - 1) : k - 1;
	b.u = (y == L - 1) ? k - (L - 1) * L : k + L;
	b.d = (y == 0) ? k + (L - 1) * L : k - L;
	return b;
}

// Appends cell ci to the bins its patch rectangle overlaps (periodic).
__device__ void append_bins(const CellDev &c, int ci, const LayerDev &ly, int *bin_count_all, int *bin_cells_all,
                            DevStatus *st) {
	const int L = ly.L, nbx = ly.nbx;
	int *bin_count = bin_count_all + ly.bin_off;
	int *bin_cells = bin_cells_all + (size_t) ly.bin_off * BIN_CAP;
	// patch sides are <= MAX_TABLE_SIDE (128): at most 5 x-bins and 17 y-bins
	int bxs[8], bys[24];
	int nbxs = 0, nbys = 0;
	{
		int x = c.corner % L, rem = c.lx;
		while(rem > 0 && nbxs < 8) {
			const int b = x / BIN_X;
			int end = min((b + 1) * BIN_X, L);
			int run = min(rem, end - x);
			bool seen = false;
			for(int i = 0; i < nbxs; i++) seen |= (bxs[i] == b);
			if(!seen) bxs[nbxs++] = b;
			rem -= run;
			x += run;
			if(x >= L) x = 0;
		}
	}
	{
		int y = c.corner / L, rem = c.ly;
		while(rem > 0 && nbys < 24) {
			const int b = y / BIN_Y;
			int end = min((b + 1) * BIN_Y, L);
			int run = min(rem, end - y);
			bool seen = false;
			for(int i = 0; i < nbys; i++) seen |= (bys[i] == b);
			if(!seen) bys[nbys++] = b;
			rem -= run;
			y += run;
			if(y >= L) y = 0;
		}
	}
	for(int j = 0; j < nbys; j++)
		for(int i = 0; i < nbxs; i++) {
			const int b = bxs[i] + bys[j] * nbx;
			const int slot = atomicAdd(&bin_count[b], 1);
			if(slot < BIN_CAP) bin_cells[(size_t) b * BIN_CAP + slot] = ci;
			else atomicOr(&st->err, ERR_BIN);
		}
}

// set_positions (Fields/MultiPhaseField.cpp:223-310).  The resize branch only
// records the new geometry; the field copy runs in the repack kernels.
__device__ void set_positions_dev(CellDev &c, const DevParams &P, int L, DevStatus *st, int ci) {
	const int border = P.border;
	if(c.xl >= border && c.yb >= border) {
		const int site = box_el(c.corner, (int) c.comx, (int) c.comy, L);
		c.comy = (int) (site / L) + (c.comy - (int) c.comy);
		c.comx = (int) (site - (int) (site / L) * L) + (c.comx - (int) c.comx);
		const double cox = c.corner % L, coy = c.corner / L;
		const int ncorner = box_el(site, (int) -c.lx / 2, (int) -c.ly / 2, L);
		const double cnx = ncorner % L, cny = ncorner / L;
		const double d0 = cnx - cox - rint((cnx - cox) / L) * L;
		const double d1 = cny - coy - rint((cny - coy) / L) * L;
		c.unrapx += d0;
		c.unrapy += d1;
		c.offx = (int) (c.offx + c.lx - d0) % c.lx;
		c.offy = (int) (c.offy + c.ly - d1) % c.ly;
		c.corner = ncorner;
		c.resized = 0;
		return;
	}
	const int nlx = c.lx - (2 * c.xl) + (2 * border);
	const int nly = c.ly - (2 * c.yb) + (2 * border);
	if(nlx <= 0 || nly <= 0 || nlx > L || nly > L || nlx > MAX_TABLE_SIDE || nly > MAX_TABLE_SIDE ||
	   nlx * nly > MAX_PATCH_SITES) {
		atomicOr(&st->err, ERR_CAPACITY);
		st->err_where = ci;
		c.resized = 0;
		return;
	}
	const int ncorner = box_el(c.corner, -(-(2 * c.xl) + (2 * border)) / 2, -(-(2 * c.yb) + (2 * border)) / 2, L);
	c.old_lx = c.lx;
	c.old_ly = c.ly;
	c.old_offx = c.offx;
	c.old_offy = c.offy;
	c.old_corner = c.corner;
	{
		const double ox = c.corner % L, oy = c.corner / L;
		const double nx = ncorner % L, ny = ncorner / L;
		c.unrapx += nx - ox - rint((nx - ox) / L) * L;
		c.unrapy += ny - oy - rint((ny - oy) / L) * L;
	}
	c.lx = nlx;
	c.ly = nly;
	c.n = nlx * nly;
	c.corner = ncorner;
	c.offx = c.offy = 0;
	const int site = box_el(c.corner, c.lx / 2, c.ly / 2, L);
	c.comy = (int) (site / L);
	c.comx = (int) (site - (int) (site / L) * L);
	c.resized = 1;
	atomicAdd(&st->resized, 1);
	atomicAdd(&st->resized_total, 1);
}

__device__ void directed_forces_dev(CellDev &c, const DevParams &P, const PhaseParams &pu, int store, DevStatus *st,
                                    int ci) {
	const double dt = P.dt, JQ = pu.JQ;
	if(P.model == M_POLAR) {
		if(store) c.thq_old = c.thq + sqrt(dt) * pu.zi * c.gauss;
		const double f0 = c.trx, f1 = c.try_;
		c.thq = c.thq_old - dt * JQ * (atan2(f0 * c.q01 - f1 * c.q00, f0 * c.q00 + f1 * c.q01));
		c.q00 = cos(c.thq);
		c.q01 = sin(c.thq);
	}
	else if(P.model == M_WET) {
		const double smod = sqrt(c.s00 * c.s00 + c.s01 * c.s01);
		if(store) {
			c.nq_oldx = c.nqx;
			c.nq_oldy = c.nqy;
		}
		if(smod > 0.00000001) {
			const double t = 0.5 * atan2(c.s01, c.s00);
			const double d0 = cos(t), d1 = sin(t);
			const double sgn = (d0 * c.nqx + d1 * c.nqy > 0.0) ? 1.0 : -1.0;
			c.nqx = c.nq_oldx + dt * JQ * (sgn * d0 - c.nqx);
			c.nqy = c.nq_oldy + dt * JQ * (sgn * d1 - c.nqy);
			c.q00 = 0.5 * (c.nqx * c.nqx - c.nqy * c.nqy);
			c.q01 = c.nqx * c.nqy;
		}
	}
	else if(P.model == M_NEMATIC) {
		if(store) {
			c.nq_oldx = c.nqx;
			c.nq_oldy = c.nqy;
		}
		if(c.type == 0) {
			c.nqx = c.nq_oldx;
			c.nqy = c.nq_oldy;
		}
		else if(c.type == 1) {
			const double t = 0.5 * atan2(c.s01, c.s00);
			const double d0 = cos(t), d1 = sin(t);
			const double sgn = (d0 * c.nqx + d1 * c.nqy > 0.0) ? 1.0 : -1.0;
			c.nqx = c.nq_oldx + dt * JQ * (sgn * d0 - c.nqx);
			c.nqy = c.nq_oldy + dt * JQ * (sgn * d1 - c.nqy);
			c.q00 = 0.5 * (c.nqx * c.nqx - c.nqy * c.nqy);
			c.q01 = c.nqx * c.nqy;
		}
		else {
			atomicOr(&st->err, ERR_TYPE);
			st->err_where = ci;
		}
	}
}

// Per-cell epilogue of an evaluation / update (one thread): cell outputs,
// area, centre of mass, set_positions, the per-cell scalar dynamics and the
// bins of the next gather.  Shared by the FP64 and FP32 cell kernels.
template<int MODEL, int EVAL, int UPD>
__device__ __forceinline__ void cell_finish(CellDev &c, const double (&acc)[12], const int (&imin)[2], double perim,
                                            const CellArgs &a, const LayerDev &lay, int ci) {
	const DevParams &P = a.P;
	const PhaseParams &pu = a.pu;
	const int lx = c.lx, ly = c.ly, L = lay.L;
	(void) lx;
	(void) ly;
	if(EVAL != EV_NONE) {
		// per-cell outputs of the evaluation (perimeter, force totals)
		c.perim = (MODEL == M_POLAR) ? perim : 0.0;
		if(MODEL == M_POLAR) {
			c.trx = acc[8];
			c.try_ = acc[9];
			c.tfx = acc[10];
			c.tfy = acc[11];
		}
		else {
			c.trx = c.try_ = c.tfx = c.tfy = 0.0;
		}
	}
	if(UPD != UP_NONE) {
		if(UPD == UP_PRED) {
			c.com_oldx = c.comx;
			c.com_oldy = c.comy;
			c.area_old = c.area;
			c.sumf_old = c.sumf;
		}
		c.area = acc[0];
		c.sumf = acc[1];
		c.s00 = acc[6];
		c.s01 = acc[7];
		c.perim = 0.0;
		c.xl = (UPD == UP_CORR) ? imin[0] : lx;
		c.yb = (UPD == UP_CORR) ? imin[1] : ly;
		c.comx = c.lx * (atan2(-acc[3] / c.sumf, -acc[2] / c.sumf) + RC_PI_F) / (2 * RC_PI_F);
		c.comy = c.ly * (atan2(-acc[5] / c.sumf, -acc[4] / c.sumf) + RC_PI_F) / (2 * RC_PI_F);
		if(!isfinite(c.area) || !isfinite(c.sumf) || !isfinite(c.comx) || !isfinite(c.comy)) {
			atomicOr(&a.st->err, ERR_NONFINITE);
			a.st->err_where = ci;
		}
		if(UPD == UP_CORR) set_positions_dev(c, P, L, a.st, ci);
		directed_forces_dev(c, P, pu, UPD == UP_PRED, a.st, ci);
		if(UPD == UP_CORR) {
			append_bins(c, ci, lay, a.bin_count, a.bin_cells, a.st);
			atomicMax(&a.st->max_n, c.n);
		}
	}
}

// Forces of one site from the shared-memory patch (stage 2 of the evaluation)
// and the update of that site.  Kept as one templated kernel so that the fused
// (dry) and split (wet) variants share every line of arithmetic.
template<int MODEL, int EVAL, int UPD>
__global__ void __launch_bounds__(CELL_THREADS) cell_kernel(const CellArgs a) {
	extern __shared__ double smem[];
	__shared__ CellDev c;
	__shared__ double red[12 * (CELL_THREADS / 32 + 1)];
	__shared__ int ired[2 * (CELL_THREADS / 32)];

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
	if(n > a.smem_n) {
		if(threadIdx.x == 0) {
			atomicOr(&a.st->err, ERR_CAPACITY);
			a.st->err_where = ci;
		}
		return;
	}
	// shared layout: phi | mu | aux (Repulsion or f_d) | ext (second chain of
	// the sequential polar totals); cell_smem_bytes sizes it per model
	double *sphi = smem;
	double *smu = smem + a.smem_n;
	double *saux = smem + 2 * a.smem_n;
	double *sext = smem + 3 * a.smem_n;
	const DevParams &P = a.P;
	const PhaseParams &pe = a.pe;
	const double gamma = P.gamma, lambda = P.lambda, mu_c = P.mu, kappa = P.kappa, omega = P.omega, a0 = P.a0;
	const bool dry = (MODEL == M_NEMATIC) || (MODEL == M_SIMPLE) || pe.friction_cell == 0;

	// Per-cell constant factors of the reference's left-to-right products
	// (hoisting a leading sub-product leaves every rounding unchanged), formed
	// once by thread 0: FP64 divisions are expensive on GB300.
	__shared__ double kd[8];
	if(threadIdx.x == 0) {
		kd[0] = 1.0 / lambda;
		if(MODEL == M_SIMPLE || MODEL == M_NEMATIC) {
			kd[1] = -4 * mu_c / a0 * (1 - c.area / a0);
			kd[2] = 4 * kappa / lambda;
			kd[3] = 0.0;
			kd[4] = 0.0;
		}
		else {
			kd[1] = -4 * (mu_c / a0) * (1 - c.area / a0);
			kd[2] = 4 * (kappa / lambda);
			kd[3] = -mu_c / a0;
			kd[4] = (gamma / lambda) * 4;
		}
		kd[5] = kappa / lambda;
		kd[6] = 1.0 / pe.friction;
	}
	__syncthreads();
	const double rlambda = kd[0];
	const double two_lambda = 2 * lambda;
	const double A_c = kd[1], Rep_c = kd[2], Ad_c = kd[3], CHd_c = kd[4], gl_c = gamma * lambda;
	const double kl_c = kd[5];
	double perim = 0.0;
	if(EVAL != EV_NONE) {
		for(int q = threadIdx.x; q < n; q += blockDim.x) sphi[q] = a.phi_eval[start + q];
		__syncthreads();
		if(MODEL == M_POLAR && (pe.beta != 0.0 || EVAL == EV_STORE || EVAL == EV_WET_RHS)) {
			double v[1] = {0.0};
			for(int q = threadIdx.x; q < n; q += blockDim.x) {
				const int y = q / lx, x = q - y * lx;
				const Nb nb = patch_nb(q, x, y, lx, ly);
				const double dx = .5 * (sphi[nb.r] - sphi[nb.l]);
				const double dy = .5 * (sphi[nb.u] - sphi[nb.d]);
				v[0] += dx * dx + dy * dy;
			}
			block_sum<1>(v, red);
			perim = v[0];
		}
		// Stage 1: chemical potential (f_interaction).
		for(int q = threadIdx.x; q < n; q += blockDim.x) {
			const int y = q / lx, x = q - y * lx;
			const Nb nb = patch_nb(q, x, y, lx, ly);
			const double phi = sphi[q];
			const double pr = sphi[nb.r], pl = sphi[nb.l], pu_ = sphi[nb.u], pd = sphi[nb.d];
			const double dx = .5 * (pr - pl), dy = .5 * (pu_ - pd);
			const int k = box_site(c, x, y, L);
			const double p2 = phi2[k];
			double ls = 0.0;
			if(omega != 0.0 && MODEL != M_SIMPLE) {
				const BoxNb kb = box_nb(k, L);
				ls = phi2[kb.r] + phi2[kb.u] + phi2[kb.l] + phi2[kb.d] - 4. * p2;
			}
			double mu = 0.0;
			if(MODEL == M_SIMPLE) {
				const double lap = pu_ + pd + pr + pl - 4 * phi;
				const double CH = gamma * (div_rn(8 * phi * (1 - phi) * (1 - 2 * phi), lambda, rlambda) - two_lambda * lap);
				const double A = A_c * phi;
				const double Rep = Rep_c * phi * (p2 - phi * phi);
				mu = CH + A + Rep + 0.;
				if(a.fsplit) {  // SimpleMultiField.cpp:158-181: pressure and free-energy density
					a.fsplit[4 * a.fsplit_stride + start + q] = Rep - CH - A;
					const double dx = .5 * (pr - pl), dy = .5 * (pu_ - pd);
					const double CHd = (gamma / lambda) * 4 * phi * phi * (1 - phi) * (1 - phi) + gamma * lambda * (dx * dx + dy * dy);
					const double Ad = -P.mu / P.a0 * phi * phi;
					const double Repd = (P.kappa / lambda) * phi * phi * (p2 - phi * phi);
					a.fsplit[5 * a.fsplit_stride + start + q] = CHd + Ad + Repd;
				}
			}
			else if(MODEL == M_NEMATIC) {
				const double lap = pr + pu_ + pl + pd - 4. * phi;
				const double CH = +gamma * (div_rn(8 * phi * (1 - phi) * (1 - 2 * phi), lambda, rlambda) - two_lambda * lap);
				const double A = A_c * phi;
				const double Rep = Rep_c * phi * (p2 - phi * phi);
				double V = CH + A + Rep;
				if(omega != 0.0) {
					const double lsq = 2 * phi * lap + 2 * (dx * dx + dy * dy);
					const double sup = (ls - lsq) / sqrt(1 + (ls - lsq) * (ls - lsq));
					V = V + (-4 * lambda * omega * sup * phi);
				}
				mu = V;
				if(a.fsplit) {  // ActiveNematic.cpp:225; no free-energy density
					a.fsplit[4 * a.fsplit_stride + start + q] = Rep - CH - A;
					a.fsplit[5 * a.fsplit_stride + start + q] = 0.0;
				}
			}
			else {
				const double lap = pu_ + pd + pr + pl - 4 * phi;
				const double CH = gamma * (div_rn(8 * phi * (1 - phi) * (1 - 2 * phi), lambda, rlambda) - two_lambda * lap);
				const double A = A_c * phi;
				const double Rep = Rep_c * phi * (p2 - phi * phi);
				double V = CH + A + Rep;
				if(omega != 0.0) {
					const double lsq = 2 * phi * lap + 2 * (dx * dx + dy * dy);
					const double sup = (ls - lsq) / sqrt(1 + (ls - lsq) * (ls - lsq));
					V = V + (-4 * lambda * omega * sup * phi);
				}
				if(a.fsplit) a.fsplit[4 * a.fsplit_stride + start + q] = Rep - CH - A;  // WetModel.cpp:605, WetPolarModel.cpp:298
				if(MODEL == M_POLAR) {
					if(pe.beta != 0.0) {
						const double p0 = 12.;
						V = V + 4 * (pe.beta / p0) * (1 - perim / p0) * lap;
					}
					if(a.rep_on) {
						double r = a.rep[start + q] + Rep;
						if(a.accumulate_rep) a.rep[start + q] = r;
						saux[q] = r;
					}
				}
				else {
					const double CHd = CHd_c * phi * phi * (1 - phi) * (1 - phi) + gl_c * (dx * dx + dy * dy);
					const double Ad = Ad_c * phi * phi;
					const double Repd = kl_c * phi * phi * (p2 - phi * phi);
					saux[q] = CHd + Ad + Repd;
					if(a.fsplit) a.fsplit[5 * a.fsplit_stride + start + q] = saux[q];  // WetModel.cpp:607
				}
				if(MODEL == M_POLAR && a.fsplit) a.fsplit[5 * a.fsplit_stride + start + q] = 0.0;
				mu = V;
			}
			smu[q] = mu;
			if(EVAL == EV_STORE || EVAL == EV_WET_RHS) {
				a.mu[start + q] = mu;
				a.dxg[start + q] = dx;
				a.dyg[start + q] = dy;
				a.mapg[start + q] = k;
			}
		}
		__syncthreads();
	}

	// Stage 2: forces (calc_internal_forces) and the update (first_step).
	double acc[12];
#pragma unroll
	for(int i = 0; i < 12; i++) acc[i] = 0.0;
	int imin[2] = {lx, ly};
	const PhaseParams &pu = a.pu;
	const double J0 = P.J0, hdt = P.dt * .5;
	const double zs = pe.zs, zi = pe.zi, fr = pe.friction, alpha = P.passive_alpha;
	const double rfr = kd[6];
	const int tb = table_base(lx), tby = table_base(ly);

	for(int q = threadIdx.x; q < n; q += blockDim.x) {
		const int y = q / lx, x = q - y * lx;
		double mu, vx = 0.0, vy = 0.0, dx, dy, phi_e = 0.0;
		if(EVAL != EV_NONE) {
			const Nb nb = patch_nb(q, x, y, lx, ly);
			phi_e = sphi[q];
			dx = .5 * (sphi[nb.r] - sphi[nb.l]);
			dy = .5 * (sphi[nb.u] - sphi[nb.d]);
			mu = smu[q];
			if(MODEL == M_SIMPLE) {
				vx = 0.0;
				vy = 0.0;
				if(a.fsplit)
					for(int f = 0; f < 4; f++) a.fsplit[f * a.fsplit_stride + start + q] = 0.0;
			}
			else if(MODEL == M_NEMATIC || MODEL == M_WET) {
				const int k = box_site(c, x, y, L);
				const BoxNb kb = box_nb(k, L);
				const double fsx = -(c.q00 * dx + c.q01 * dy);
				const double fsy = -(c.q01 * dx - c.q00 * dy);
				const double fix = -(0.5 * (sq00[kb.r] - sq00[kb.l]) + 0.5 * (sq01[kb.u] - sq01[kb.d])) - fsx;
				const double fiy = -(0.5 * (sq01[kb.r] - sq01[kb.l]) - 0.5 * (sq00[kb.u] - sq00[kb.d])) - fsy;
				if(MODEL == M_NEMATIC) {
					vx = div_rn(mu * dx + fsx * zs + fix * zi, fr, rfr);
					vy = div_rn(mu * dy + fsy * zs + fiy * zi, fr, rfr);
					if(a.fsplit) {  // ActiveNematic.cpp:239-240,249-250
						double *fs = a.fsplit + start + q;
						fs[0] = mu * dx;
						fs[a.fsplit_stride] = mu * dy;
						fs[2 * a.fsplit_stride] = zs * fsx + zi * fix;
						fs[3 * a.fsplit_stride] = zs * fsy + zi * fiy;
					}
				}
				else {
					// Passive stress of WetModel.cpp:634-635 from neighbours' mu, f_d and gradients.
					const double g2 = 2 * gamma * lambda;
					auto grad_x = [&](int s, int sx, int sy) {
						const Nb b = patch_nb(s, sx, sy, lx, ly);
						return .5 * (sphi[b.r] - sphi[b.l]);
					};
					auto grad_y = [&](int s, int sx, int sy) {
						const Nb b = patch_nb(s, sx, sy, lx, ly);
						return .5 * (sphi[b.u] - sphi[b.d]);
					};
					const int xr = (x == lx - 1) ? 0 : x + 1, xl_ = (x == 0) ? lx - 1 : x - 1;
					const int yu = (y == ly - 1) ? 0 : y + 1, yd = (y == 0) ? ly - 1 : y - 1;
					const Nb nb2 = patch_nb(q, x, y, lx, ly);
					const double dxr = grad_x(nb2.r, xr, y), dxl = grad_x(nb2.l, xl_, y);
					const double dxu = grad_x(nb2.u, x, yu), dxd = grad_x(nb2.d, x, yd);
					const double dyu = grad_y(nb2.u, x, yu), dyd = grad_y(nb2.d, x, yd);
					const double dyr = grad_y(nb2.r, xr, y), dyl = grad_y(nb2.l, xl_, y);
					const double fgxr = g2 * dxr, fgxl = g2 * dxl, fgyu = g2 * dyu, fgyd = g2 * dyd;
					const double fgyu_x = g2 * dyu, fgyd_x = g2 * dyd;  // freeEnergyDensityGradient_y at u, d
					const double fgxr_y = g2 * dxr, fgxl_y = g2 * dxl;  // freeEnergyDensityGradient_x at r, l
					const double fpx = -0.5 * ((saux[nb2.r] - smu[nb2.r] * sphi[nb2.r] + dxr * fgxr) - (saux[nb2.l] - smu[nb2.l] * sphi[nb2.l] + dxl * fgxl))
					                   - 0.5 * ((dxu * fgyu_x) - (dxd * fgyd_x));
					const double fpy = -0.5 * ((saux[nb2.u] - smu[nb2.u] * sphi[nb2.u] + dyu * fgyu) - (saux[nb2.d] - smu[nb2.d] * sphi[nb2.d] + dyd * fgyd))
					                   - 0.5 * ((dyr * fgxr_y) - (dyl * fgxl_y));
					const double fx = fpx * alpha + fsx * zs + fix * zi;
					const double fy = fpy * alpha + fsy * zs + fiy * zi;
					if(a.fsplit) {  // WetModel.cpp:636-637,655-656
						double *fs = a.fsplit + start + q;
						fs[0] = fpx * alpha;
						fs[a.fsplit_stride] = fpy * alpha;
						fs[2 * a.fsplit_stride] = zs * fsx + zi * fix;
						fs[3 * a.fsplit_stride] = zs * fsy + zi * fiy;
					}
					if(EVAL == EV_WET_RHS) {
						a.fxg[start + q] = fx;
						a.fyg[start + q] = fy;
					}
					else {
						vx = div_rn(fx, fr, rfr);
						vy = div_rn(fy, fr, rfr);
					}
				}
			}
			else {  // M_POLAR
				const Nb nb = patch_nb(q, x, y, lx, ly);
				const double fpx = (-1) * 0.5 * (smu[nb.r] - smu[nb.l]);
				const double fpy = (-1) * 0.5 * (smu[nb.u] - smu[nb.d]);
				if(a.rep_on) {
					acc[8] += (-1) * 0.5 * (saux[nb.r] - saux[nb.l]) * phi_e;
					acc[9] += (-1) * 0.5 * (saux[nb.u] - saux[nb.d]) * phi_e;
				}
				double th = (-dx * c.q00) < 0 ? 0.0 : 1.0;
				const double fsx = lambda * (-dx * c.q00) * th * c.q00;
				th = (-dy * c.q01) < 0 ? 0.0 : 1.0;
				const double fsy = lambda * (-dy * c.q01) * th * c.q01;
				const double fx = fpx * alpha + fsx * zs;
				const double fy = fpy * alpha + fsy * zs;
				if(a.fsplit) {  // WetPolarModel.cpp:311-312,325-326
					double *fs = a.fsplit + start + q;
					fs[0] = fpx * alpha;
					fs[a.fsplit_stride] = fpy * alpha;
					fs[2 * a.fsplit_stride] = zs * fsx;
					fs[3 * a.fsplit_stride] = zs * fsy;
				}
				acc[10] += fx * phi_e;
				acc[11] += fy * phi_e;
				if(EVAL == EV_WET_RHS) {
					a.fxg[start + q] = fx;
					a.fyg[start + q] = fy;
				}
				else {
					vx = div_rn(fx, fr, rfr);
					vy = div_rn(fy, fr, rfr);
				}
			}
			if(EVAL == EV_STORE && dry) {
				a.vxg[start + q] = vx;
				a.vyg[start + q] = vy;
			}
		}
		else {
			mu = a.mu[start + q];
			vx = a.vxg[start + q];
			vy = a.vyg[start + q];
			dx = a.dxg[start + q];
			dy = a.dyg[start + q];
		}
		if(UPD != UP_NONE) {
			double dphi;
			if(P.conserved) {
				// FD_CHBackend::first_step (FD_CHBackend.cpp:63-68): J0 lap(mu) - v.grad(phi).
				// For the simple and nematic models the reference resets
				// freeEnergy[q'] to the external term (0) as each site q' is updated
				// (BaseInteraction::updateFieldProperties, BaseInteraction.cpp:62-69),
				// so neighbours earlier in storage order enter the Laplacian as 0; the
				// polar and wet models' updateFieldProperties (WetPolarModel.cpp:130,
				// WetModel.cpp:167) keep it.
				const Nb nb = patch_nb(q, x, y, lx, ly);
				auto fe = [&](int s_) {
					if((MODEL == M_SIMPLE || MODEL == M_NEMATIC) && s_ < q) return 0.0;
					return (EVAL != EV_NONE) ? smu[s_] : a.mu[start + s_];
				};
				const double lmu = fe(nb.r) + fe(nb.u) + fe(nb.l) + fe(nb.d) - 4. * mu;
				dphi = J0 * lmu - vx * dx - vy * dy;
			}
			else
				dphi = -J0 * mu - vx * dx - vy * dy;
			double phi_new;
			if(UPD == UP_PRED) {
				const double phi_old = (EVAL != EV_NONE) ? phi_e : a.phi_eval[start + q];
				a.dphi_old[start + q] = dphi;
				phi_new = phi_old + hdt * (dphi + dphi);
			}
			else {
				const double phi_old = a.phi_old[start + q];
				const double dold = a.dphi_old[start + q];
				phi_new = phi_old + hdt * (dphi + dold);
			}
			a.phi_out[start + q] = phi_new;
			acc[0] += phi_new * phi_new;
			acc[1] += phi_new;
			int lxx = x + c.offx;
			if(lxx >= lx) lxx -= lx;
			int lyy = y + c.offy;
			if(lyy >= ly) lyy -= ly;
			acc[2] += phi_new * a.tab_cos[tb + lxx];
			acc[3] += phi_new * a.tab_sin[tb + lxx];
			acc[4] += phi_new * a.tab_cos[tby + lyy];
			acc[5] += phi_new * a.tab_sin[tby + lyy];
			if(UPD == UP_CORR && phi_new < 0.09 && phi_new > 0.01) {
				imin[0] = min(imin[0], lxx);
				imin[1] = min(imin[1], lyy);
			}
			acc[6] += -0.5 * (dx * dx - dy * dy);
			acc[7] += -dx * dy;
		}
	}

	// Sums whose terms cancel and whose direction drives the dynamics -- the
	// shape tensor of the nematic models (director alignment) and the polar
	// repulsion-force totals (torque when J_Q != 0) -- are formed sequentially
	// in storage order, as the reference's loops form them; a tree order
	// changes them by more than the 1e-10 parity bar.  Well-conditioned sums
	// (area, sums of phi, centre-of-mass sums) use the block tree.
	// (Only needed when J_Q != 0: otherwise neither sum affects the dynamics.)
	// On GB300 an FP64 warp instruction occupies the FP64 pipe for tens of
	// cycles, so all threads first form the terms into shared memory, and one
	// warp instruction per term then carries both dependent add chains.
	const bool seq_shape = (MODEL == M_NEMATIC || MODEL == M_WET) && UPD != UP_NONE && pu.JQ != 0.0;
	const bool seq_rep = (MODEL == M_POLAR) && (EVAL != EV_NONE) && a.rep_on;
	double *chain0 = saux, *chain1 = smu;  // terms of the two chains (free after stage 2)
	if(seq_shape || seq_rep) __syncthreads();
	if(seq_shape) {
		for(int q = threadIdx.x; q < n; q += blockDim.x) {
			double dx, dy;
			if(EVAL != EV_NONE) {
				const int y = q / lx, x = q - y * lx;
				const Nb nb = patch_nb(q, x, y, lx, ly);
				dx = .5 * (sphi[nb.r] - sphi[nb.l]);
				dy = .5 * (sphi[nb.u] - sphi[nb.d]);
			}
			else {
				dx = a.dxg[start + q];
				dy = a.dyg[start + q];
			}
			chain0[q] = -0.5 * (dx * dx - dy * dy);
			chain1[q] = -dx * dy;
		}
	}
	if(seq_rep) {
		// saux holds the Repulsion accumulator (read at neighbours): terms go to
		// smu and the fourth array
		chain0 = smu;
		chain1 = sext;
		for(int q = threadIdx.x; q < n; q += blockDim.x) {
			const int y = q / lx, x = q - y * lx;
			const Nb nb = patch_nb(q, x, y, lx, ly);
			chain0[q] = (-1) * 0.5 * (saux[nb.r] - saux[nb.l]) * sphi[q];
			chain1[q] = (-1) * 0.5 * (saux[nb.u] - saux[nb.d]) * sphi[q];
		}
	}
	if(UPD != UP_NONE) {
		block_sum<12>(acc, red);
		if(UPD == UP_CORR) block_min<2>(imin, ired);
	}
	else if(MODEL == M_POLAR && EVAL != EV_NONE) {
		double v4[4] = {acc[8], acc[9], acc[10], acc[11]};
		block_sum<4>(v4, red);
		acc[8] = v4[0];
		acc[9] = v4[1];
		acc[10] = v4[2];
		acc[11] = v4[3];
	}
	if(seq_shape || seq_rep) {
		__shared__ double s_seq[2];
		__syncthreads();
		if(threadIdx.x < 2) {
			const double *terms = (threadIdx.x == 0) ? chain0 : chain1;
			double sum = 0.0;
			for(int q = 0; q < n; q++) sum += terms[q];
			s_seq[threadIdx.x] = sum;
		}
		__syncthreads();
		if(threadIdx.x == 0) {
			if(seq_shape) {
				acc[6] = s_seq[0];
				acc[7] = s_seq[1];
			}
			else {
				acc[8] = s_seq[0];
				acc[9] = s_seq[1];
			}
		}
	}

	if(a.split) {
		if(threadIdx.x == 0) {
			CellSum &o = a.csum[ci];
#pragma unroll
			for(int i = 0; i < 12; i++) o.acc[i] = acc[i];
			o.imin[0] = imin[0];
			o.imin[1] = imin[1];
			o.perim = perim;
		}
		return;
	}
	if(threadIdx.x == 0) cell_finish<MODEL, EVAL, UPD>(c, acc, imin, perim, a, lay, ci);
	__syncthreads();
	{
		const int *src = reinterpret_cast<const int *>(&c);
		int *dst = reinterpret_cast<int *>(&a.cells[ci]);
		for(int i = threadIdx.x; i < (int) (sizeof(CellDev) / 4); i += blockDim.x) dst[i] = src[i];
	}
}

// ---------------------------------------------------------------- FP32 ---
// Double-float accumulation of x*x: (s, c) holds the running sum with its
// error term (exact product by FMA, Knuth's TwoSum), close to FP64 accuracy
// with FP32 arithmetic only.
__device__ __forceinline__ void acc_square(float x, float &s, float &c) {
	const float p = x * x;
	const float ep = __fmaf_rn(x, x, -p);
	const float t = s + p;
	const float bp = t - s;
	const float err = (s - (t - bp)) + (p - bp);
	s = t;
	c += err + ep;
}

// The dry polar model (wetpolarmodel with friction_cell = 0, the
// ensemble's model) with FP32 site arithmetic: the patch, chemical
// potential, forces and the update in FP32 (shared memory in FP32, fields
// stored in FP64); the area integral sum(phi^2) that drives the area
// constraint accumulates in double-float (near FP64), the other per-cell
// sums from FP32 per-thread partials in FP64.  Same stages, expressions and per-cell
// epilogue as cell_kernel<M_POLAR, ...>; not bitwise the reference.
// Patch coordinates of q = threadIdx.x, threadIdx.x + blockDim.x, ... without
// a per-site division: the stride's row and column steps are fixed per cell.
struct PatchWalk {
	int q, x, y, sx, sy, lx;
	__device__ __forceinline__ PatchWalk(int lx_) : lx(lx_) {
		q = threadIdx.x;
		y = q / lx;
		x = q - y * lx;
		sy = (int) blockDim.x / lx;
		sx = (int) blockDim.x - sy * lx;
	}
	__device__ __forceinline__ void next() {
		q += blockDim.x;
		x += sx;
		y += sy;
		if(x >= lx) {
			x -= lx;
			y += 1;
		}
	}
};

template<int EVAL, int UPD, int BLOCK>
__global__ void __launch_bounds__(BLOCK) cell_kernel_f32(const CellArgs a) {
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
	const int cx0 = c.corner % L, cy0 = c.corner / L;
	// box site of patch site (x, y): GetSubIndex without divisions
	auto site_of = [&](int x, int y) {
		int px = x + c.offx;
		if(px >= lx) px -= lx;
		int py = y + c.offy;
		if(py >= ly) py -= ly;
		int bx = cx0 + px;
		if(bx >= L) bx -= L;
		int by = cy0 + py;
		if(by >= L) by -= L;
		return bx + by * L;
	};
	if(n > a.smem_n) {
		if(threadIdx.x == 0) {
			atomicOr(&a.st->err, ERR_CAPACITY);
			a.st->err_where = ci;
		}
		return;
	}
	float *sphi = reinterpret_cast<float *>(smem_raw);
	float *smu = sphi + a.smem_n;
	float *saux = smu + a.smem_n;
	const DevParams &P = a.P;
	const PhaseParams &pe = a.pe;
	// Per-cell constants, formed once by thread 0: on GB300 an FP64 warp
	// instruction (a division is ~10 of them) costs tens of issue cycles, too
	// many to repeat in every thread.
	enum { K_GAMMA, K_LAMBDA, K_OMEGA, K_RLAMBDA, K_AC, K_REPC, K_J0, K_HDT, K_ZS, K_ALPHA, K_RFR, K_Q00, K_Q01, K_BETA,
	       K_HAS_BETA, K_HAS_OMEGA, K_N };
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
		kc[K_ALPHA] = (float) P.passive_alpha;
		kc[K_RFR] = (float) (1.0 / pe.friction);
		kc[K_Q00] = (float) c.q00;
		kc[K_Q01] = (float) c.q01;
		kc[K_HAS_BETA] = pe.beta != 0.0 ? 1.f : 0.f;
		kc[K_HAS_OMEGA] = P.omega != 0.0 ? 1.f : 0.f;
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
		if(has_beta) {
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
		for(PatchWalk w(lx); w.q < n; w.next()) {
			const int q = w.q, x = w.x, y = w.y;
			const Nb nb = patch_nb(q, x, y, lx, ly);
			const float phi = sphi[q];
			const float pr = sphi[nb.r], pl = sphi[nb.l], pu_ = sphi[nb.u], pd = sphi[nb.d];
			const int k = site_of(x, y);
			const float p2 = d2f_int(phi2[k]);
			const float lap = pu_ + pd + pr + pl - 4.f * phi;
			const float CH = gamma * (8.f * phi * (1.f - phi) * (1.f - 2.f * phi) * rlambda - two_lambda * lap);
			const float Rep = Rep_c * phi * (p2 - phi * phi);
			float V = CH + A_c * phi + Rep;
			if(has_omega) {
				const BoxNb kb = box_nb(k, L);
				const float ls = (float) (phi2[kb.r] + phi2[kb.u] + phi2[kb.l] + phi2[kb.d] - 4. * phi2[k]);
				const float dx = .5f * (pr - pl), dy = .5f * (pu_ - pd);
				const float lsq = 2.f * phi * lap + 2.f * (dx * dx + dy * dy);
				const float sup = (ls - lsq) * rsqrtf(1.f + (ls - lsq) * (ls - lsq));
				V = V + (-4.f * lambda * omega * sup * phi);
			}
			if(has_beta) V = V + beta_t * lap;
			if(EVAL == EV_STORE) {
				a.mu[start + q] = f2d_int(V);
				a.dxg[start + q] = f2d_int(.5f * (pr - pl));
				a.dyg[start + q] = f2d_int(.5f * (pu_ - pd));
				a.mapg[start + q] = k;
			}
			if(a.rep_on) {
				const float r = d2f_int(a.rep[start + q]) + Rep;
				if(a.accumulate_rep) a.rep[start + q] = f2d_int(r);
				saux[q] = r;
			}
			smu[q] = V;
		}
		__syncthreads();
	}
	double acc[12];
#pragma unroll
	for(int i = 0; i < 12; i++) acc[i] = 0.0;
	float af[12];
#pragma unroll
	for(int i = 0; i < 12; i++) af[i] = 0.f;
	int imin[2] = {lx, ly};
	float area_s = 0.f, area_c = 0.f;
	const float J0 = kc[K_J0], hdt = kc[K_HDT];
	const bool conserved = P.conserved != 0;
	const float zs = kc[K_ZS], alpha = kc[K_ALPHA], lam = lambda;
	const float rfr = kc[K_RFR];
	const int tb = table_base(lx), tby = table_base(ly);
	const float q00 = kc[K_Q00], q01 = kc[K_Q01];
	for(PatchWalk w(lx); w.q < n; w.next()) {
		const int q = w.q, x = w.x, y = w.y;
		float mu, vx, vy, dx, dy, phi_e = 0.f;
		if(EVAL != EV_NONE) {
			const Nb nb = patch_nb(q, x, y, lx, ly);
			phi_e = sphi[q];
			dx = .5f * (sphi[nb.r] - sphi[nb.l]);
			dy = .5f * (sphi[nb.u] - sphi[nb.d]);
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
			const float fx = fpx * alpha + fsx * zs;
			const float fy = fpy * alpha + fsy * zs;
			af[10] += fx * phi_e;
			af[11] += fy * phi_e;
			vx = fx * rfr;
			vy = fy * rfr;
			if(EVAL == EV_STORE) {
				a.vxg[start + q] = f2d_int(vx);
				a.vyg[start + q] = f2d_int(vy);
			}
		}
		else {
			mu = d2f_int(a.mu[start + q]);
			vx = d2f_int(a.vxg[start + q]);
			vy = d2f_int(a.vyg[start + q]);
			dx = d2f_int(a.dxg[start + q]);
			dy = d2f_int(a.dyg[start + q]);
		}
		if(UPD == UP_NONE) continue;
		float dphi;
		if(conserved) {
			// FD_CH (FD_CHBackend.cpp:63-68); the polar model keeps every
			// neighbour's freeEnergy through the loop (WetPolarModel.cpp:130)
			const Nb nb = patch_nb(q, x, y, lx, ly);
			auto fe = [&](int s_) {
				return (EVAL != EV_NONE) ? smu[s_] : d2f_int(a.mu[start + s_]);
			};
			const float lmu = fe(nb.r) + fe(nb.u) + fe(nb.l) + fe(nb.d) - 4.f * mu;
			dphi = J0 * lmu - vx * dx - vy * dy;
		}
		else
			dphi = -J0 * mu - vx * dx - vy * dy;
		float phi_new;
		if(UPD == UP_PRED) {
			const float phi_old = (EVAL != EV_NONE) ? phi_e : d2f_int(a.phi_eval[start + q]);
			a.dphi_old[start + q] = f2d_int(dphi);
			phi_new = phi_old + hdt * (dphi + dphi);
		}
		else {
			phi_new = d2f_int(a.phi_old[start + q]) + hdt * (dphi + d2f_int(a.dphi_old[start + q]));
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
			const float t = area_s + s2, bp = t - area_s;
			area_c += ((area_s - (t - bp)) + (s2 - bp)) + c2;
			area_s = t;
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
	if(threadIdx.x == 0) cell_finish<M_POLAR, EVAL, UPD>(c, acc, imin, perim, a, lay, ci);
	__syncthreads();
	{
		const int *src = reinterpret_cast<const int *>(&c);
		int *dst = reinterpret_cast<int *>(&a.cells[ci]);
		for(int i = threadIdx.x; i < (int) (sizeof(CellDev) / 4); i += blockDim.x) dst[i] = src[i];
	}
}

template<int BLOCK>
static bool launch_f32_block(int eval, int upd, const CellArgs &a, cudaStream_t s) {
	const size_t smem = sizeof(float) * 3 * (size_t) a.smem_n;
	if(eval == EV_LOCAL && upd == UP_PRED) cell_kernel_f32<EV_LOCAL, UP_PRED, BLOCK><<<a.N, BLOCK, smem, s>>>(a);
	else if(eval == EV_LOCAL && upd == UP_CORR) cell_kernel_f32<EV_LOCAL, UP_CORR, BLOCK><<<a.N, BLOCK, smem, s>>>(a);
	else if(eval == EV_NONE && upd == UP_PRED) cell_kernel_f32<EV_NONE, UP_PRED, BLOCK><<<a.N, BLOCK, smem, s>>>(a);
	else if(eval == EV_STORE && upd == UP_NONE) cell_kernel_f32<EV_STORE, UP_NONE, BLOCK><<<a.N, BLOCK, smem, s>>>(a);
	else return false;
	return true;
}

bool launch_cell_kernel_f32(int eval, int upd, const CellArgs &a, cudaStream_t s, int block) {
	if(a.N <= 0) return true;
	if(block == 128) return launch_f32_block<128>(eval, upd, a, s);
	if(block == 512) return launch_f32_block<512>(eval, upd, a, s);
	return launch_f32_block<256>(eval, upd, a, s);
}

template<int BLOCK>
static cudaError_t configure_f32_block() {
	cudaError_t e = cudaSuccess, c;
	const int mx = 200 * 1024;
	if((c = cudaFuncSetAttribute(cell_kernel_f32<EV_LOCAL, UP_PRED, BLOCK>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx)) !=
	   cudaSuccess)
		e = c;
	if((c = cudaFuncSetAttribute(cell_kernel_f32<EV_LOCAL, UP_CORR, BLOCK>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx)) !=
	   cudaSuccess)
		e = c;
	if((c = cudaFuncSetAttribute(cell_kernel_f32<EV_NONE, UP_PRED, BLOCK>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx)) !=
	   cudaSuccess)
		e = c;
	if((c = cudaFuncSetAttribute(cell_kernel_f32<EV_STORE, UP_NONE, BLOCK>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx)) !=
	   cudaSuccess)
		e = c;
	return e;
}

static cudaError_t configure_f32() {
	cudaError_t e = cudaSuccess, c;
	if((c = configure_f32_block<128>()) != cudaSuccess) e = c;
	if((c = configure_f32_block<256>()) != cudaSuccess) e = c;
	if((c = configure_f32_block<512>()) != cudaSuccess) e = c;
	return e;
}

// Split mode: the per-cell epilogue with one thread per cell, so that 32
// cells share every FP64 instruction of the centre-of-mass, re-centering and
// per-cell dynamics code (the same cell_finish the fused kernels run).
template<int MODEL, int EVAL, int UPD, bool F32>
__global__ void __launch_bounds__(128) cell_finish_kernel(const CellArgs a) {
	const int ci = blockIdx.x * blockDim.x + threadIdx.x;
	if(ci >= a.N) return;
	CellDev c = a.cells[ci];
	const CellSum &sm = a.csum[ci];
	double acc[12];
	if(F32) {
		const int nw = sm.nw;
		double t = 0.0;
		for(int w = 0; w < nw; w++) t += sm.area[w];
		acc[0] = t;
#pragma unroll
		for(int i = 1; i < 12; i++) {
			double u = 0.0;
			for(int w = 0; w < nw; w++) u += (double) sm.part[w][i];
			acc[i] = u;
		}
	}
	else {
#pragma unroll
		for(int i = 0; i < 12; i++) acc[i] = sm.acc[i];
	}
	const int imin[2] = {sm.imin[0], sm.imin[1]};
	const LayerDev lay = a.layers[c.layer];
	cell_finish<MODEL, EVAL, UPD>(c, acc, imin, sm.perim, a, lay, ci);
	a.cells[ci] = c;
}

template<int MODEL, bool F32>
static void launch_finish_m(int eval, int upd, const CellArgs &a, cudaStream_t s) {
	const int g = (a.N + 127) / 128;
	if(eval == EV_STORE && upd == UP_NONE) cell_finish_kernel<MODEL, EV_STORE, UP_NONE, F32><<<g, 128, 0, s>>>(a);
	else if(eval == EV_WET_RHS && upd == UP_NONE) cell_finish_kernel<MODEL, EV_WET_RHS, UP_NONE, F32><<<g, 128, 0, s>>>(a);
	else if(eval == EV_LOCAL && upd == UP_PRED) cell_finish_kernel<MODEL, EV_LOCAL, UP_PRED, F32><<<g, 128, 0, s>>>(a);
	else if(eval == EV_LOCAL && upd == UP_CORR) cell_finish_kernel<MODEL, EV_LOCAL, UP_CORR, F32><<<g, 128, 0, s>>>(a);
	else if(eval == EV_NONE && upd == UP_PRED) cell_finish_kernel<MODEL, EV_NONE, UP_PRED, F32><<<g, 128, 0, s>>>(a);
	else if(eval == EV_NONE && upd == UP_CORR) cell_finish_kernel<MODEL, EV_NONE, UP_CORR, F32><<<g, 128, 0, s>>>(a);
}

void launch_cell_finish(int model, int eval, int upd, bool f32, const CellArgs &a, cudaStream_t s) {
	if(a.N <= 0) return;
	if(f32) {
		const int g = (a.N + 127) / 128;
		if(eval == EV_LOCAL && upd == UP_PRED) cell_finish_kernel<M_POLAR, EV_LOCAL, UP_PRED, true><<<g, 128, 0, s>>>(a);
		else if(eval == EV_LOCAL && upd == UP_CORR) cell_finish_kernel<M_POLAR, EV_LOCAL, UP_CORR, true><<<g, 128, 0, s>>>(a);
		else if(eval == EV_STORE && upd == UP_NONE) cell_finish_kernel<M_POLAR, EV_STORE, UP_NONE, true><<<g, 128, 0, s>>>(a);
		else cell_finish_kernel<M_POLAR, EV_NONE, UP_PRED, true><<<g, 128, 0, s>>>(a);
		return;
	}
	switch(model) {
		case M_SIMPLE: launch_finish_m<M_SIMPLE, false>(eval, upd, a, s); break;
		case M_NEMATIC: launch_finish_m<M_NEMATIC, false>(eval, upd, a, s); break;
		case M_POLAR: launch_finish_m<M_POLAR, false>(eval, upd, a, s); break;
		default: launch_finish_m<M_WET, false>(eval, upd, a, s); break;
	}
}

int cell_smem_arrays(int model) {
	switch(model) {
		case M_SIMPLE: return 2;
		case M_NEMATIC: return 3;  // phi, mu, and the shape-tensor chain
		case M_POLAR: return 4;    // phi, mu, Repulsion, and the second torque chain
		default: return 3;         // phi, mu, f_d
	}
}

size_t cell_smem_bytes(int model, int smem_n) {
	return sizeof(double) * (size_t) cell_smem_arrays(model) * (size_t) smem_n;
}

template<int MODEL, int EVAL, int UPD>
static void launch_t(const CellArgs &a, cudaStream_t s) {
	const size_t smem = cell_smem_bytes(MODEL, a.smem_n);
	cell_kernel<MODEL, EVAL, UPD><<<a.N, CELL_THREADS, smem, s>>>(a);
}

template<int MODEL>
static cudaError_t configure_m() {
	cudaError_t e = cudaSuccess, c;
#define RC_CFG(EV, UP)                                                                                             \
	c = cudaFuncSetAttribute(cell_kernel<MODEL, EV, UP>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024); \
	if(c != cudaSuccess) e = c;
	RC_CFG(EV_STORE, UP_NONE)
	RC_CFG(EV_WET_RHS, UP_NONE)
	RC_CFG(EV_LOCAL, UP_PRED)
	RC_CFG(EV_LOCAL, UP_CORR)
	RC_CFG(EV_NONE, UP_PRED)
	RC_CFG(EV_NONE, UP_CORR)
#undef RC_CFG
	return e;
}

template<int MODEL>
static void launch_m(int eval, int upd, const CellArgs &a, cudaStream_t s) {
	if(eval == EV_STORE && upd == UP_NONE) launch_t<MODEL, EV_STORE, UP_NONE>(a, s);
	else if(eval == EV_WET_RHS && upd == UP_NONE) launch_t<MODEL, EV_WET_RHS, UP_NONE>(a, s);
	else if(eval == EV_LOCAL && upd == UP_PRED) launch_t<MODEL, EV_LOCAL, UP_PRED>(a, s);
	else if(eval == EV_LOCAL && upd == UP_CORR) launch_t<MODEL, EV_LOCAL, UP_CORR>(a, s);
	else if(eval == EV_NONE && upd == UP_PRED) launch_t<MODEL, EV_NONE, UP_PRED>(a, s);
	else if(eval == EV_NONE && upd == UP_CORR) launch_t<MODEL, EV_NONE, UP_CORR>(a, s);
}

void launch_cell_kernel(int model, int eval, int upd, const CellArgs &a, cudaStream_t s) {
	if(a.N <= 0) return;
	switch(model) {
		case M_SIMPLE: launch_m<M_SIMPLE>(eval, upd, a, s); break;
		case M_NEMATIC: launch_m<M_NEMATIC>(eval, upd, a, s); break;
		case M_POLAR: launch_m<M_POLAR>(eval, upd, a, s); break;
		default: launch_m<M_WET>(eval, upd, a, s); break;
	}
}

// ------------------------------------------------------------------ RNG ---
// Utils::gaussian over the drand48 stream, one deviate per cell in cell
// order, as the reference draws them in updateDirectedActiveForces(store).
// Pairs of draws are tested in parallel (jump-ahead of the LCG); the accepted
// pairs are consumed in stream order.
__constant__ unsigned long long c_jumpA[2 * CELL_THREADS + 1];
__constant__ unsigned long long c_jumpC[2 * CELL_THREADS + 1];

__global__ void __launch_bounds__(CELL_THREADS) rng_kernel(CellDev *cells_all, LayerDev *layers, DevStatus *st) {
	LayerDev *lay = &layers[blockIdx.x];
	CellDev *cells = cells_all + lay->cell_lo;
	const int N = lay->cell_hi - lay->cell_lo;
	__shared__ int s_scan[CELL_THREADS];
	__shared__ unsigned long long s_state;
	__shared__ int s_produced, s_has, s_last;
	__shared__ double s_cached;
	const unsigned long long M = (1ULL << 48) - 1;
	const int t = threadIdx.x;
	if(t == 0) {
		s_state = lay->rng_state;
		s_has = lay->rng_has;
		s_cached = lay->rng_cached;
		s_produced = 0;
		if(s_has && N > 0) {
			cells[0].gauss = s_cached;
			s_has = 0;
			s_produced = 1;
		}
	}
	__syncthreads();
	int rounds = 0;
	while(s_produced < N && rounds++ < (1 << 20)) {
		const unsigned long long X0 = s_state;
		const unsigned long long X1 = (c_jumpA[2 * t + 1] * X0 + c_jumpC[2 * t + 1]) & M;
		const unsigned long long X2 = (c_jumpA[2 * t + 2] * X0 + c_jumpC[2 * t + 2]) & M;
		const double u = 2. * ((double) X1 * (1.0 / 281474976710656.0)) - 1.0;
		const double v = 2. * ((double) X2 * (1.0 / 281474976710656.0)) - 1.0;
		const double w = u * u + v * v;
		const int acc = (w < 1.0) ? 1 : 0;
		s_scan[t] = acc;
		__syncthreads();
		for(int o = 1; o < CELL_THREADS; o <<= 1) {  // inclusive scan
			int add = (t >= o) ? s_scan[t - o] : 0;
			__syncthreads();
			s_scan[t] += add;
			__syncthreads();
		}
		const int produced = s_produced;
		const int need = N - produced;
		const int pairs_needed = (need + 1) / 2;
		const int total = s_scan[CELL_THREADS - 1];
		const int rank = s_scan[t] - acc;
		if(t == 0) s_last = -1;
		__syncthreads();
		if(acc && rank < pairs_needed) {
			const double sc = sqrt((-2. * log(w)) / w);
			const int pos = produced + 2 * rank;
			cells[pos].gauss = u * sc;
			if(pos + 1 < N) cells[pos + 1].gauss = v * sc;
			if(rank == pairs_needed - 1) {
				s_last = t;
				if(pos + 1 >= N) {
					s_has = 1;
					s_cached = v * sc;
				}
			}
		}
		__syncthreads();
		if(t == 0) {
			if(total >= pairs_needed) {
				const int k = 2 * (s_last + 1);
				s_state = (c_jumpA[k] * X0 + c_jumpC[k]) & M;
				s_produced = N;
			}
			else {
				s_state = (c_jumpA[2 * CELL_THREADS] * X0 + c_jumpC[2 * CELL_THREADS]) & M;
				s_produced = produced + 2 * total;
			}
		}
		__syncthreads();
	}
	if(t == 0) {
		if(s_produced < N) atomicOr(&st->err, ERR_NONFINITE);
		lay->rng_state = s_state;
		lay->rng_has = s_has;
		lay->rng_cached = s_cached;
	}
}

void launch_rng(CellDev *cells, LayerDev *layers, int n_layers, DevStatus *st, cudaStream_t s) {
	if(n_layers > 0) rng_kernel<<<n_layers, CELL_THREADS, 0, s>>>(cells, layers, st);
}

// One-time, per-device set-up that must not happen inside stream capture:
// shared-memory limits of the cell kernels and the LCG jump-ahead table.
cudaError_t configure_kernels() {
	cudaError_t e = cudaSuccess, c;
	if((c = configure_m<M_SIMPLE>()) != cudaSuccess) e = c;
	if((c = configure_m<M_NEMATIC>()) != cudaSuccess) e = c;
	if((c = configure_m<M_POLAR>()) != cudaSuccess) e = c;
	if((c = configure_m<M_WET>()) != cudaSuccess) e = c;
	if((c = configure_f32()) != cudaSuccess) e = c;
	unsigned long long A[2 * CELL_THREADS + 1], Cc[2 * CELL_THREADS + 1];
	const unsigned long long a = 0x5DEECE66DULL, cc = 0xBULL, M = (1ULL << 48) - 1;
	A[0] = 1;
	Cc[0] = 0;
	for(int k = 1; k <= 2 * CELL_THREADS; k++) {
		A[k] = (A[k - 1] * a) & M;
		Cc[k] = (Cc[k - 1] * a + cc) & M;
	}
	if((c = cudaMemcpyToSymbol(c_jumpA, A, sizeof(A))) != cudaSuccess) e = c;
	if((c = cudaMemcpyToSymbol(c_jumpC, Cc, sizeof(Cc))) != cudaSuccess) e = c;
	return e;
}

// ----------------------------------------------------------------- bins ---
__global__ void bins_kernel(const CellDev *cells, const LayerDev *layers, int N, int *bin_count, int *bin_cells,
                            DevStatus *st) {
	const int ci = blockIdx.x * blockDim.x + threadIdx.x;
	if(ci >= N) return;
	CellDev c = cells[ci];
	append_bins(c, ci, layers[c.layer], bin_count, bin_cells, st);
	atomicMax(&st->max_n, c.n);
}

void launch_bins(CellDev *cells, const LayerDev *layers, int N, int *bin_count, int *bin_cells, int total_bins,
                 DevStatus *st, cudaStream_t s) {
	cudaMemsetAsync(bin_count, 0, sizeof(int) * (size_t) total_bins, s);
	if(N > 0) bins_kernel<<<(N + 127) / 128, 128, 0, s>>>(cells, layers, N, bin_count, bin_cells, st);
}

// --------------------------------------------------------------- repack ---
// After a corrector in which patches were resized (st->resized > 0): new
// flat offsets, the resized patches' field copy with the reference's loop
// (MultiPhaseField.cpp:250-303, including its copy bounds and its area sum),
// and std::vector::resize semantics for the Repulsion accumulator.  All three
// kernels return at once when nothing was resized.
__global__ void repack_scan_kernel(CellDev *cells, int N, DevStatus *st, int *new_start, long long cap) {
	if(st->resized == 0) return;
	if(threadIdx.x == 0) {
		long long acc = 0;
		for(int i = 0; i < N; i++) {
			new_start[i] = (int) acc;
			acc += cells[i].n;
		}
		st->S = acc;
		if(acc > cap) {
			atomicOr(&st->err, ERR_CAPACITY);
		}
	}
}

__global__ void repack_copy_kernel(CellDev *cells, const LayerDev *layers, int N, DevStatus *st, const int *new_start,
                                   const double *phi, double *out_phi, const double *rep, double *out_rep, int rep_on,
                                   long long cap) {
	if(st->resized == 0 || (st->err & ERR_CAPACITY)) return;
	const int ci = blockIdx.x;
	const CellDev &c = cells[ci];
	const int ns = new_start[ci];
	if(!c.resized) {
		for(int q = threadIdx.x; q < c.n; q += blockDim.x) {
			out_phi[ns + q] = phi[c.start + q];
			if(rep_on) out_rep[ns + q] = rep[c.start + q];
		}
		return;
	}
	const int nlx = c.lx, nly = c.ly, nn = c.n, olx = c.old_lx, oly = c.old_ly;
	const int L = layers[c.layer].L;
	for(int q = threadIdx.x; q < nn; q += blockDim.x) {
		out_phi[ns + q] = 0.0;
		if(rep_on) out_rep[ns + q] = (q < olx * oly) ? rep[c.start + q] : 0.0;
	}
	__syncthreads();
	if(threadIdx.x == 0) {
		double area = 0;
		int sy, dimy, sx, dimx;
		if(nly < oly) {
			sy = (oly - nly) / 2;
			dimy = nly;
		}
		else {
			sy = 0;
			dimy = oly;
		}
		if(nlx < olx) {
			sx = (olx - nlx) / 2;
			dimx = nlx;
		}
		else {
			sx = 0;
			dimx = olx;
		}
		const int ncorner = c.corner, ocorner = c.old_corner;
		for(int i = sy; i < dimy; i++) {
			const int yy = wrapi(ocorner / L + i, L);
			int offy = i - c.old_offy;
			if(offy < 0) offy += oly;
			for(int j = sx; j < dimx; j++) {
				const int xx = wrapi(ocorner % L + j, L);
				int dx = (ncorner - (ncorner / L) * L) - xx;
				if(dx > L / 2) dx -= L;
				else if(dx < -L / 2) dx += L;
				int dy = (ncorner / L) - yy;
				if(dy > L / 2) dy -= L;
				else if(dy < -L / 2) dy += L;
				int offx = j - c.old_offx;
				if(offx < 0) offx += olx;
				const double v = phi[c.start + offx + offy * olx];
				const int dst = abs(dx) + abs(dy) * nlx;
				if(dst < nn) out_phi[ns + dst] = v;
				area += v * v;
			}
		}
		cells[ci].area = area;
	}
}

__global__ void repack_finish_kernel(CellDev *cells, int N, DevStatus *st, const int *new_start, double *phi,
                                     const double *in_phi, double *rep, const double *in_rep, int rep_on) {
	if(st->resized == 0 || (st->err & ERR_CAPACITY)) return;
	const long long S = st->S;
	for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < S; i += (long long) gridDim.x * blockDim.x) {
		phi[i] = in_phi[i];
		if(rep_on) rep[i] = in_rep[i];
	}
}

__global__ void repack_done_kernel(CellDev *cells, int N, DevStatus *st, const int *new_start) {
	if(st->resized == 0) return;
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
		cells[i].start = new_start[i];
		cells[i].resized = 0;
	}
}

__global__ void repack_clear_kernel(DevStatus *st) { st->resized = 0; }

void launch_repack(CellArgs a, double *scratch_phi, double *scratch_rep, long long cap, cudaStream_t s) {
	// new_start lives behind the scratch buffers' tail (allocated by the engine)
	int *new_start = reinterpret_cast<int *>(scratch_phi + cap);
	repack_scan_kernel<<<1, 32, 0, s>>>(a.cells, a.N, a.st, new_start, cap);
	repack_copy_kernel<<<a.N, CELL_THREADS, 0, s>>>(a.cells, a.layers, a.N, a.st, new_start, a.phi_out, scratch_phi,
	                                                 a.rep, scratch_rep, a.rep_on, cap);
	repack_finish_kernel<<<304, 256, 0, s>>>(a.cells, a.N, a.st, new_start, a.phi_out, scratch_phi, a.rep, scratch_rep,
	                                         a.rep_on);
	repack_done_kernel<<<(a.N + 255) / 256, 256, 0, s>>>(a.cells, a.N, a.st, new_start);
	repack_clear_kernel<<<1, 1, 0, s>>>(a.st);
}

}  // namespace rc
