// Device code shared by the FP64 cell kernels (rc_cells.cu) and the FP32
// cell kernels (rc_cells_f32.cu): patch and box neighbours, the bins of the
// box gather, set_positions, the directed active forces and the per-cell
// epilogue of an update.
//
// Reference functions re-designed here (paths relative to the reference's src/):
//   set_positions / check_borders .... Fields/MultiPhaseField.cpp:223-344
//   updateDirectedActiveForces ....... WetPolarModel.cpp:342-414,
//                                      WetModel.cpp:697-747, ActiveNematic.cpp:257-289
//   FD_CPUBackend::first_step sums ... Backends/FD_CPUBackend.cpp:85-120
#pragma once

#include "rc_kernels.cuh"

#include <math.h>

namespace rc {

#define RC_PI_F 3.141592653589793238462643f

__device__ inline int box_el(int site, int dx, int dy, int L) {
	return wrapi(site % L + dx, L) + wrapi(site / L + dy, L) * L;
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
static __device__ void append_bins(const CellDev &c, int ci, const LayerDev &ly, int *bin_count_all, int *bin_cells_all,
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
static __device__ void set_positions_dev(CellDev &c, const DevParams &P, int L, DevStatus *st, int ci) {
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

static __device__ void directed_forces_dev(CellDev &c, const DevParams &P, const PhaseParams &pu, int store, DevStatus *st,
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


// Double-float accumulation of x*x: (s, c) holds the running sum with its
// error term (exact product by FMA, Knuth's TwoSum), close to FP64 accuracy
// with FP32 arithmetic only.  Written with rounding intrinsics, which the
// compiler never fuses, so the error terms stay exact where FMA contraction
// is enabled.
__device__ __forceinline__ void acc_square(float x, float &s, float &c) {
	const float p = __fmul_rn(x, x);
	const float ep = __fmaf_rn(x, x, -p);
	const float t = __fadd_rn(s, p);
	const float bp = __fsub_rn(t, s);
	const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
	s = t;
	c = __fadd_rn(c, __fadd_rn(err, ep));
}

// TwoSum of two double-float partials (s, c) += (s2, c2), the same way.
__device__ __forceinline__ void add_df(float &s, float &c, float s2, float c2) {
	const float t = __fadd_rn(s, s2), bp = __fsub_rn(t, s);
	c = __fadd_rn(c, __fadd_rn(__fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(s2, bp)), c2));
	s = t;
}

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


}  // namespace rc
