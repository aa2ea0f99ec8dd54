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
#include "rc_cell_dev.cuh"

namespace rc {

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

// Wall boxes.  A box site is open when its wall value is below wall_slip
// (BaseInteraction.h:196-263 test getWalls(k) < wall_slip); open_nb packs
// the four box neighbours of k: bit 0 right, 1 left, 2 up, 3 down.
__device__ __forceinline__ int open_nb(const double *walls, double slip, int k, int L) {
	const BoxNb b = box_nb(k, L);
	return (walls[b.r] < slip ? 1 : 0) | (walls[b.l] < slip ? 2 : 0) | (walls[b.u] < slip ? 4 : 0) |
	       (walls[b.d] < slip ? 8 : 0);
}

// BaseInteraction::derivX, derivY and Laplacian (BaseInteraction.h:196-263)
// of the shared patch at q, whose covering box site has open neighbours f:
// the central differences vanish across a wall, and the Laplacian doubles
// the open side of a direction that has one wall (the reference's branch
// order and expressions, for bitwise equal results).
__device__ __forceinline__ void wall_stencil(const double *sphi, const Nb &nb, int q, int f, double &dx, double &dy,
                                             double &lap) {
	const double phi = sphi[q], r = sphi[nb.r], l = sphi[nb.l], u = sphi[nb.u], d = sphi[nb.d];
	const bool R = f & 1, Lf = f & 2, U = f & 4, D = f & 8;
	dx = (R && Lf) ? .5 * (r - l) : 0.;
	dy = (U && D) ? .5 * (u - d) : 0.;
	if(U && D) {
		if(R && Lf) lap = u + d + r + l - 4 * phi;
		else if(R) lap = u + d + 2 * r - 4 * phi;
		else if(Lf) lap = u + d + 2 * l - 4 * phi;
		else lap = u + d - 2 * phi;
	}
	else if(U || D) {
		const double v = U ? u : d;
		if(R && Lf) lap = 2 * v + r + l - 4 * phi;
		else if(R) lap = 2 * v + 2 * r - 4 * phi;
		else if(Lf) lap = 2 * v + 2 * l - 4 * phi;
		else lap = 2 * v - 2 * phi;
	}
	else lap = 0.;
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
	const double *walls = a.walls ? a.walls + lay.box_off : nullptr;  // wall boxes (null: periodic)
	const double slip = a.P.wall_slip;
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
				double dx = .5 * (sphi[nb.r] - sphi[nb.l]);
				double dy = .5 * (sphi[nb.u] - sphi[nb.d]);
				if(walls) {
					double lw;
					wall_stencil(sphi, nb, q, open_nb(walls, slip, box_site(c, x, y, L), L), dx, dy, lw);
				}
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
			double dx = .5 * (pr - pl), dy = .5 * (pu_ - pd);
			const int k = box_site(c, x, y, L);
			const double p2 = phi2[k];
			// wall boxes: the stencils of every model but activenematic, whose
			// own plain differences ignore walls (ActiveNematic.cpp:176-230)
			double lapw = 0.0;
			const bool walled = MODEL != M_NEMATIC && walls != nullptr;
			if(walled) wall_stencil(sphi, nb, q, open_nb(walls, slip, k, L), dx, dy, lapw);
			double ls = 0.0;
			if(omega != 0.0 && MODEL != M_SIMPLE) {
				const BoxNb kb = box_nb(k, L);
				// at a wall site the polar and wet models keep the x terms
				// (WetModel.cpp:531-536, WetPolarModel.cpp:267-272)
				if(walled && !(walls[k] < slip)) ls = phi2[kb.r] + phi2[kb.l] - 2. * p2;
				else ls = phi2[kb.r] + phi2[kb.u] + phi2[kb.l] + phi2[kb.d] - 4. * p2;
			}
			double mu = 0.0;
			if(MODEL == M_SIMPLE) {
				const double lap = walled ? lapw : pu_ + pd + pr + pl - 4 * phi;
				const double CH = gamma * (div_rn(8 * phi * (1 - phi) * (1 - 2 * phi), lambda, rlambda) - two_lambda * lap);
				const double A = A_c * phi;
				const double Rep = Rep_c * phi * (p2 - phi * phi);
				mu = CH + A + Rep + 0.;
				if(a.fsplit) {  // SimpleMultiField.cpp:158-181: pressure and free-energy density
					a.fsplit[4 * a.fsplit_stride + start + q] = Rep - CH - A;
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
				const double lap = walled ? lapw : pu_ + pd + pr + pl - 4 * phi;
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
			// wall boxes: stored gradients (not activenematic's), and the polar
			// and wet forces vanish on wall sites (WetPolarModel.cpp:329-337,
			// WetModel.cpp:664-690)
			bool open_q = true;
			if(MODEL != M_NEMATIC && walls != nullptr) {
				const int kq = box_site(c, x, y, L);
				double lw;
				wall_stencil(sphi, nb, q, open_nb(walls, slip, kq, L), dx, dy, lw);
				open_q = walls[kq] < slip;
			}
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
					// the neighbours' stored gradients, with the wall branches of
					// their own box sites
					auto grad_x = [&](int s, int sx, int sy) {
						const Nb b = patch_nb(s, sx, sy, lx, ly);
						if(walls != nullptr && (open_nb(walls, slip, box_site(c, sx, sy, L), L) & 3) != 3) return 0.;
						return .5 * (sphi[b.r] - sphi[b.l]);
					};
					auto grad_y = [&](int s, int sx, int sy) {
						const Nb b = patch_nb(s, sx, sy, lx, ly);
						if(walls != nullptr && (open_nb(walls, slip, box_site(c, sx, sy, L), L) & 12) != 12) return 0.;
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
					const double fx = open_q ? fpx * alpha + fsx * zs + fix * zi : 0.;
					const double fy = open_q ? fpy * alpha + fsy * zs + fiy * zi : 0.;
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
				const double fx = open_q ? fpx * alpha + fsx * zs : 0.;
				const double fy = open_q ? fpy * alpha + fsy * zs : 0.;
				if(a.fsplit) {  // WetPolarModel.cpp:311-312,325-326
					double *fs = a.fsplit + start + q;
					fs[0] = fpx * alpha;
					fs[a.fsplit_stride] = fpy * alpha;
					fs[2 * a.fsplit_stride] = zs * fsx;
					fs[3 * a.fsplit_stride] = zs * fsy;
				}
				if(open_q) {
					acc[10] += fx * phi_e;
					acc[11] += fy * phi_e;
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
				if(MODEL == M_WET && walls != nullptr) {
					double lw;
					wall_stencil(sphi, nb, q, open_nb(walls, slip, box_site(c, x, y, L), L), dx, dy, lw);
				}
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
		if(model == M_POLAR) launch_finish_m<M_POLAR, true>(eval, upd, a, s);
		else launch_finish_m<M_WET, true>(eval, upd, a, s);
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
	if((c = configure_kernels_f32()) != cudaSuccess) e = c;
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
__global__ void widen3_kernel(const float *a, const float *b, const float *c, double *x, double *y, double *z,
                              long long n) {
	for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
		x[i] = (double) a[i];
		y[i] = (double) b[i];
		z[i] = (double) c[i];
	}
}

void launch_widen3(const float *a, const float *b, const float *c, double *x, double *y, double *z, long long n,
                   cudaStream_t s) {
	if(n <= 0) return;
	const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 16);
	widen3_kernel<<<(int) blocks, 256, 0, s>>>(a, b, c, x, y, z, n);
}

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
