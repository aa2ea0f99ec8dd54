/*
 * CPU restatement of RheoCell's time-step hot path -- TEST INFRASTRUCTURE
 * (the checker; see rc_oracle.h).  Serial, FP64, in the reference's order of
 * evaluation, so that with -ffp-contract=off it reproduces the exact build of
 * the reference bit for bit (pinned by tests/test_oracle_golden.py).
 *
 * Functions restated (paths relative to the reference's src/):
 *   first_step ............ Backends/FD_CPUBackend.cpp:44-120
 *   sim_step .............. Backends/FD_CPUBackend.cpp:134-160
 *   init (first forces) ... Backends/FD_CPUBackend.cpp:19-42
 *   stencils .............. Interactions/BaseInteraction.h:196-263 (square box,
 *                           no walls: the wall branches are not taken)
 *   patch neighbours ...... Fields/MultiPhaseField.cpp:188-208
 *   trig tables ........... Fields/MultiPhaseField.cpp:54-65
 *   set_positions ......... Fields/MultiPhaseField.cpp:223-310
 *   check_borders ......... Fields/MultiPhaseField.cpp:334-344
 *   GetSubIndex ........... Fields/MultiPhaseField.cpp:348-358, Boxes/SquareBox.cpp:31-45
 *   min_image ............. Boxes/SquareBox.cpp:71-76
 *   simplefield ........... Interactions/SimpleMultiField.cpp:78-184
 *   activenematic ......... Interactions/ActiveNematic.cpp:101-289
 *   wetpolarmodel ......... Interactions/WetPolarModel.cpp:232-414
 *   wetmodel .............. Interactions/WetModel.cpp:126-747
 *   viscous solve ......... the operator assembled at WetModel.cpp:279-347 /
 *                           WetPolarModel.cpp:309-337, solved with Jacobi-
 *                           preconditioned CG as Eigen::ConjugateGradient
 *                           documents (restated in oracle/eigen_shim/Eigen/Sparse),
 *                           applied matrix-free
 *   drand48 ............... POSIX 48-bit LCG (a = 0x5DEECE66D, c = 0xB)
 *   gaussian .............. Utilities/Utils.h:210-236 (polar Marsaglia, cached pair)
 */
#include "rc_oracle.h"

#include <float.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define PI_F 3.141592653589793238462643f
#define STORE_MAX 20

typedef struct {
	int lx, ly, n;
	int off[2];
	int corner, corner_old;
	int type;
	double com[2], com_old[2], unrap[2];
	double q00, q01, thq, thq_old, nq[2], nq_old[2];
	double area, area_old, sumf, sumf_old, perim, s00, s01;
	int xl, yb;
	double tfx, tfy, trx, try_;
	double *phi, *phi_old, *dphi_old, *mu, *fed, *fgx, *fgy, *dx, *dy, *lap, *rep, *vx, *vy;
	int *map;
	double *ctx, *stx, *cty, *sty;
} ocell;

struct orc_sim {
	rc_params P;
	int phase;
	int L, N;
	ocell *c;
	double *phi2, *sq00, *sq01, *sphi;
	int *cnt, *cover;
	long long *start;
	long long size_rows, size_rows_old;
	int restart;
	double *vvx, *vvy, *vfx, *vfy;
	long long vcap;
	unsigned long long rng;
	int has_g;
	double next_g;
	char err[512];
	rc_step_stats st;
	double *walls;  /* box->getWalls(k), NULL for the periodic square box */
};

static int fail(orc_sim *s, int code, const char *fmt, ...) {
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(s->err, sizeof(s->err), fmt, ap);
	va_end(ap);
	return code;
}

/* ---------------------------------------------------------------- RNG --- */
static double rng_drand48(orc_sim *s) {
	s->rng = (0x5DEECE66DULL * s->rng + 0xBULL) & 0xFFFFFFFFFFFFULL;
	return (double) s->rng * (1.0 / 281474976710656.0);
}

static double rng_gaussian(orc_sim *s) {
	double u, v, w;
	if(s->has_g) {
		s->has_g = 0;
		return s->next_g;
	}
	w = 2.;
	while(w >= 1.0) {
		u = 2. * rng_drand48(s) - 1.0;
		v = 2. * rng_drand48(s) - 1.0;
		w = u * u + v * v;
	}
	w = sqrt((-2. * log(w)) / w);
	s->next_g = v * w;
	s->has_g = 1;
	return u * w;
}

/* ---------------------------------------------------------- geometry --- */
static inline int wrap(int v, int L) {
	v %= L;
	return v < 0 ? v + L : v;
}
static inline int box_x(const orc_sim *s, int site, int d) { return wrap(site % s->L + d, s->L); }
static inline int box_y(const orc_sim *s, int site, int d) { return wrap(site / s->L + d, s->L); }
static inline int box_el(const orc_sim *s, int site, int dx, int dy) {
	return box_x(s, site, dx) + box_y(s, site, dy) * s->L;
}
/* box->neighbors[j + 9k] for j = 1 (down), 3 (left), 5 (right), 7 (up) */
static inline int box_nb(const orc_sim *s, int k, int j) {
	int x = k % s->L, y = k / s->L;
	switch(j) {
		case 1: return x + wrap(y - 1, s->L) * s->L;
		case 3: return wrap(x - 1, s->L) + y * s->L;
		case 5: return wrap(x + 1, s->L) + y * s->L;
		default: return x + wrap(y + 1, s->L) * s->L;
	}
}
/* neighbors_sub[j + 9q] on the periodic patch torus */
static inline int patch_nb(const ocell *c, int q, int j) {
	int y = q / c->lx, x = q - y * c->lx;
	switch(j) {
		case 1: return x + (y == 0 ? c->ly - 1 : y - 1) * c->lx;
		case 3: return (x == 0 ? c->lx - 1 : x - 1) + y * c->lx;
		case 5: return (x == c->lx - 1 ? 0 : x + 1) + y * c->lx;
		default: return x + (y == c->ly - 1 ? 0 : y + 1) * c->lx;
	}
}
static inline int sub_index(const orc_sim *s, const ocell *c, int q) {
	int lxs = q - (q / c->lx) * c->lx, lys = q / c->lx;
	return box_el(s, c->corner, (lxs + c->off[0]) % c->lx, (lys + c->off[1]) % c->ly);
}

/* ------------------------------------------------------------- walls --- */
/* A box site is open when it has no walls or its wall value is below
 * wall_slip (BaseInteraction.h:196-263 tests getWalls(k) < wall_slip). */
static inline int open_site(const orc_sim *s, int k) { return !s->walls || s->walls[k] < s->P.wall_slip; }

/* BaseInteraction::derivX, derivY and Laplacian (BaseInteraction.h:196-263)
 * at patch site q of cell c covering box site k: the central differences
 * and the five-point Laplacian, with the reference's one-sided forms where
 * a box neighbour of k is a wall site. */
static void wall_stencils(const orc_sim *s, const ocell *c, int q, int k, double *dx, double *dy, double *lap) {
	const double phi = c->phi[q];
	const double r = c->phi[patch_nb(c, q, 5)], l = c->phi[patch_nb(c, q, 3)];
	const double u = c->phi[patch_nb(c, q, 7)], d = c->phi[patch_nb(c, q, 1)];
	const int R = open_site(s, box_nb(s, k, 5)), Lf = open_site(s, box_nb(s, k, 3));
	const int U = open_site(s, box_nb(s, k, 7)), D = open_site(s, box_nb(s, k, 1));
	*dx = (R && Lf) ? .5 * (r - l) : 0.;
	*dy = (U && D) ? .5 * (u - d) : 0.;
	if(!lap) return;
	if(U && D) {
		if(R && Lf) *lap = u + d + r + l - 4 * phi;
		else if(R) *lap = u + d + 2 * r - 4 * phi;
		else if(Lf) *lap = u + d + 2 * l - 4 * phi;
		else *lap = u + d - 2 * phi;
	}
	else if(U) {
		if(R && Lf) *lap = 2 * u + r + l - 4 * phi;
		else if(R) *lap = 2 * u + 2 * r - 4 * phi;
		else if(Lf) *lap = 2 * u + 2 * l - 4 * phi;
		else *lap = 2 * u - 2 * phi;
	}
	else if(D) {
		if(R && Lf) *lap = 2 * d + r + l - 4 * phi;
		else if(R) *lap = 2 * d + 2 * r - 4 * phi;
		else if(Lf) *lap = 2 * d + 2 * l - 4 * phi;
		else *lap = 2 * d - 2 * phi;
	}
	else *lap = 0.;
}

static void make_tables(ocell *c) {
	c->ctx = (double *) realloc(c->ctx, sizeof(double) * (size_t) c->lx);
	c->stx = (double *) realloc(c->stx, sizeof(double) * (size_t) c->lx);
	c->cty = (double *) realloc(c->cty, sizeof(double) * (size_t) c->ly);
	c->sty = (double *) realloc(c->sty, sizeof(double) * (size_t) c->ly);
	for(int i = 0; i < c->lx; i++) {
		float a = (2.0f * PI_F * (float) i) / (float) c->lx;
		c->ctx[i] = cos((double) a);
		c->stx[i] = sin((double) a);
	}
	for(int i = 0; i < c->ly; i++) {
		float a = (2.0f * PI_F * (float) i) / (float) c->ly;
		c->cty[i] = cos((double) a);
		c->sty[i] = sin((double) a);
	}
}

/* std::vector::resize semantics: keep the first min(old, new) values, zero the rest. */
static double *vresize(double *p, int oldn, int newn) {
	double *q = (double *) realloc(p, sizeof(double) * (size_t) (newn > 0 ? newn : 1));
	for(int i = oldn; i < newn; i++) q[i] = 0.0;
	return q;
}

static void cell_resize(ocell *c, int oldn, int newn) {
	double **arrs[] = {&c->phi, &c->phi_old, &c->dphi_old, &c->mu, &c->fed, &c->fgx, &c->fgy,
	                   &c->dx, &c->dy, &c->lap, &c->rep, &c->vx, &c->vy};
	for(size_t i = 0; i < sizeof(arrs) / sizeof(arrs[0]); i++) *arrs[i] = vresize(*arrs[i], oldn, newn);
	int *m = (int *) realloc(c->map, sizeof(int) * (size_t) (newn > 0 ? newn : 1));
	for(int i = oldn; i < newn; i++) m[i] = 0;
	c->map = m;
	make_tables(c);
}

/* ------------------------------------------------------- parameters --- */
#define PRM(s, f) ((s)->P.f[(s)->phase])
static inline double a0_of(const orc_sim *s) {
	float a = PI_F * (float) s->P.R * (float) s->P.R; /* PI is a float literal: float arithmetic */
	return (double) a;
}
static inline int is_wet_model(const orc_sim *s) { return s->P.model == RC_WETMODEL || s->P.model == RC_WETPOLARMODEL; }
static inline double vel_x(const orc_sim *s, const ocell *c, int ci, int q) {
	return is_wet_model(s) ? s->vvx[s->start[ci] + q] : c->vx[q];
}
static inline double vel_y(const orc_sim *s, const ocell *c, int ci, int q) {
	return is_wet_model(s) ? s->vvy[s->start[ci] + q] : c->vy[q];
}

/* ----------------------------------------------------- init stencils --- */
/* begin_energy_computation() of each model: initFieldProperties. */
static void init_field_properties(orc_sim *s) {
	for(int ci = 0; ci < s->N; ci++) {
		ocell *c = &s->c[ci];
		for(int q = 0; q < c->n; q++) {
			c->tfx = c->tfy = c->trx = c->try_ = 0.;
			c->mu[q] = 0.;
			c->fed[q] = 0.;
			double dx = .5 * (c->phi[patch_nb(c, q, 5)] - c->phi[patch_nb(c, q, 3)]);
			double dy = .5 * (c->phi[patch_nb(c, q, 7)] - c->phi[patch_nb(c, q, 1)]);
			/* derivX/derivY (SimpleMultiField.cpp:97-98, WetModel.cpp:154-155,
			 * WetPolarModel.cpp:119-120); ActiveNematic.cpp:127-128 keeps the
			 * plain differences */
			if(s->walls && s->P.model != RC_ACTIVENEMATIC) wall_stencils(s, c, q, sub_index(s, c, q), &dx, &dy, NULL);
			c->dx[q] = dx;
			c->dy[q] = dy;
			c->s00 += -0.5 * (dx * dx - dy * dy);
			c->s01 += -dx * dy;
		}
	}
}

/* ----------------------------------------------------------- forces --- */
static int ensure_vectors(orc_sim *s) {
	if(s->size_rows > s->vcap) {
		long long n = s->size_rows;
		s->vvx = (double *) realloc(s->vvx, sizeof(double) * (size_t) n);
		s->vvy = (double *) realloc(s->vvy, sizeof(double) * (size_t) n);
		s->vfx = (double *) realloc(s->vfx, sizeof(double) * (size_t) n);
		s->vfy = (double *) realloc(s->vfy, sizeof(double) * (size_t) n);
		if(!s->vvx || !s->vvy || !s->vfx || !s->vfy) return fail(s, RC_ERR_OOM, "out of memory");
		s->vcap = n;
	}
	return RC_OK;
}

/* The per-site part of computeGlobalSums (box scatter, map, stencils). */
static int global_sums(orc_sim *s) {
	const int model = s->P.model;
	const size_t L2 = (size_t) s->L * (size_t) s->L;
	memset(s->phi2, 0, sizeof(double) * L2);
	memset(s->sq00, 0, sizeof(double) * L2);
	memset(s->sq01, 0, sizeof(double) * L2);
	memset(s->sphi, 0, sizeof(double) * L2);
	memset(s->cnt, 0, sizeof(int) * L2);
	long long rows = 0;
	for(int ci = 0; ci < s->N; ci++) {
		ocell *c = &s->c[ci];
		s->start[ci] = rows;
		rows += c->n;
		for(int q = 0; q < c->n; q++) {
			const int k = sub_index(s, c, q);
			const double phi = c->phi[q];
			s->phi2[k] += phi * phi;
			if(model == RC_WETMODEL || model == RC_WETPOLARMODEL) s->sphi[k] += phi;
			if(model == RC_WETMODEL || model == RC_ACTIVENEMATIC) {
				s->sq00[k] += phi * c->q00;
				s->sq01[k] += phi * c->q01;
			}
			c->map[q] = k;
			if(model == RC_ACTIVENEMATIC) continue;
			const double r = c->phi[patch_nb(c, q, 5)], l = c->phi[patch_nb(c, q, 3)];
			const double u = c->phi[patch_nb(c, q, 7)], d = c->phi[patch_nb(c, q, 1)];
			c->dx[q] = .5 * (r - l);
			c->dy[q] = .5 * (u - d);
			if(model != RC_SIMPLEFIELD) c->lap[q] = u + d + r + l - 4 * phi;
			if(s->walls) wall_stencils(s, c, q, k, &c->dx[q], &c->dy[q], &c->lap[q]);
			if(model == RC_WETPOLARMODEL) c->perim += c->dx[q] * c->dx[q] + c->dy[q] * c->dy[q];
			c->tfx = c->tfy = c->trx = c->try_ = 0.;
			c->mu[q] = 0.;
			c->fed[q] = 0.;
			if(model == RC_WETMODEL || model == RC_WETPOLARMODEL) {
				if(s->cnt[k] >= STORE_MAX)
					return fail(s, RC_ERR_OVERLAP, "Too many field patches overlap: cell %d, box site %d", ci, k);
				s->cover[(size_t) k * STORE_MAX + (size_t) s->cnt[k]] = (int) (s->start[ci] + q);
				s->cnt[k]++;
			}
		}
	}
	s->size_rows = rows;
	return RC_OK;
}

static inline double lap_square(const orc_sim *s, int k) {
	return s->phi2[box_nb(s, k, 5)] + s->phi2[box_nb(s, k, 7)] + s->phi2[box_nb(s, k, 3)] + s->phi2[box_nb(s, k, 1)] - 4. * s->phi2[k];
}
/* the wet and polar models' laplacianSquare at a wall site keeps the x terms
 * (WetModel.cpp:531-536, WetPolarModel.cpp:267-272) */
static inline double lap_square_walls(const orc_sim *s, int k) {
	if(open_site(s, k)) return lap_square(s, k);
	return s->phi2[box_nb(s, k, 5)] + s->phi2[box_nb(s, k, 3)] - 2. * s->phi2[k];
}

static void f_interaction(orc_sim *s) {
	const int model = s->P.model;
	const double gamma = s->P.gamma, lambda = s->P.lambda, mu = s->P.mu, kappa = s->P.kappa;
	const double omega = s->P.omega, a0 = a0_of(s);
	for(int ci = 0; ci < s->N; ci++) {
		ocell *c = &s->c[ci];
		for(int q = 0; q < c->n; q++) {
			const int k = c->map[q];
			const double phi = c->phi[q];
			if(model == RC_SIMPLEFIELD) {
				double lap = c->phi[patch_nb(c, q, 7)] + c->phi[patch_nb(c, q, 1)] + c->phi[patch_nb(c, q, 5)] + c->phi[patch_nb(c, q, 3)] - 4 * phi;
				if(s->walls) {
					double dxw, dyw;
					wall_stencils(s, c, q, k, &dxw, &dyw, &lap);
				}
				const double CH = gamma * (8 * phi * (1 - phi) * (1 - 2 * phi) / lambda - 2 * lambda * lap);
				const double A = -4 * mu / a0 * (1 - c->area / a0) * phi;
				const double Rep = 4 * kappa / lambda * phi * (s->phi2[k] - phi * phi);
				const double Adh = 0.;
				const double V = CH + A + Rep + Adh;
				c->mu[q] += V;
			}
			else if(model == RC_ACTIVENEMATIC) {
				const double r = c->phi[patch_nb(c, q, 5)], l = c->phi[patch_nb(c, q, 3)];
				const double u = c->phi[patch_nb(c, q, 7)], d = c->phi[patch_nb(c, q, 1)];
				const double dx = .5 * (r - l), dy = .5 * (u - d);
				c->dx[q] = dx;
				c->dy[q] = dy;
				const double lap = r + u + l + d - 4. * phi;
				const double ls = lap_square(s, k);
				const double CH = +gamma * (8 * phi * (1 - phi) * (1 - 2 * phi) / lambda - 2 * lambda * lap);
				const double A = -4 * mu / a0 * (1 - c->area / a0) * phi;
				const double Rep = +4 * kappa / lambda * phi * (s->phi2[k] - phi * phi);
				const double lsq = 2 * phi * lap + 2 * (dx * dx + dy * dy);
				const double sup = (ls - lsq) / sqrt(1 + (ls - lsq) * (ls - lsq));
				const double Adh = -4 * lambda * omega * sup * phi;
				const double V = CH + A + Rep + Adh;
				c->mu[q] += V;
			}
			else {
				const double lap = c->lap[q];
				const double ls = lap_square_walls(s, k);
				const double CH = gamma * (8 * phi * (1 - phi) * (1 - 2 * phi) / lambda - 2 * lambda * lap);
				const double A = -4 * (mu / a0) * (1 - c->area / a0) * phi;
				const double Rep = 4 * (kappa / lambda) * phi * (s->phi2[k] - phi * phi);
				const double dx = c->dx[q], dy = c->dy[q];
				const double lsq = 2 * phi * lap + 2 * (dx * dx + dy * dy);
				const double sup = (ls - lsq) / sqrt(1 + (ls - lsq) * (ls - lsq));
				const double Adh = -4 * lambda * omega * sup * phi;
				if(model == RC_WETPOLARMODEL) {
					const double p0 = 12.;
					const double P = 4 * (PRM(s, beta) / p0) * (1 - c->perim / p0) * lap;
					const double V = CH + A + Rep + Adh + P;
					c->mu[q] += V;
					c->rep[q] += Rep;
				}
				else {
					const double CHd = (gamma / lambda) * 4 * phi * phi * (1 - phi) * (1 - phi) + gamma * lambda * (dx * dx + dy * dy);
					const double Ad = -mu / a0 * phi * phi;
					const double Repd = (kappa / lambda) * phi * phi * (s->phi2[k] - phi * phi);
					const double V = CH + A + Rep + Adh;
					c->mu[q] += V;
					c->fed[q] += CHd + Ad + Repd;
					c->fgx[q] = 2 * gamma * lambda * dx;
					c->fgy[q] = 2 * gamma * lambda * dy;
				}
			}
		}
	}
}

static void internal_forces(orc_sim *s) {
	const int model = s->P.model;
	const double lambda = s->P.lambda, alpha = s->P.passive_alpha;
	const double zs = PRM(s, zetaQ_self), zi = PRM(s, zetaQ_inter), fr = PRM(s, friction);
	const int dry = PRM(s, friction_cell) == 0;
	for(int ci = 0; ci < s->N; ci++) {
		ocell *c = &s->c[ci];
		for(int q = 0; q < c->n; q++) {
			const int k = c->map[q];
			const int r = patch_nb(c, q, 5), l = patch_nb(c, q, 3), u = patch_nb(c, q, 7), d = patch_nb(c, q, 1);
			const double phi = c->phi[q], dx = c->dx[q], dy = c->dy[q];
			if(model == RC_ACTIVENEMATIC) {
				const int kr = box_nb(s, k, 5), kl = box_nb(s, k, 3), ku = box_nb(s, k, 7), kd = box_nb(s, k, 1);
				const double fsx = -(c->q00 * dx + c->q01 * dy);
				const double fsy = -(c->q01 * dx - c->q00 * dy);
				const double fix = -(0.5 * (s->sq00[kr] - s->sq00[kl]) + 0.5 * (s->sq01[ku] - s->sq01[kd])) - fsx;
				const double fiy = -(0.5 * (s->sq01[kr] - s->sq01[kl]) - 0.5 * (s->sq00[ku] - s->sq00[kd])) - fsy;
				c->vx[q] = (c->mu[q] * dx + fsx * zs + fix * zi) / fr;
				c->vy[q] = (c->mu[q] * dy + fsy * zs + fiy * zi) / fr;
				continue;
			}
			const long long g = s->start[ci] + q;
			double fx, fy;
			if(model == RC_WETPOLARMODEL) {
				const double fpx = (-1) * 0.5 * (c->mu[r] - c->mu[l]);
				const double fpy = (-1) * 0.5 * (c->mu[u] - c->mu[d]);
				c->trx += (-1) * 0.5 * (c->rep[r] - c->rep[l]) * phi;
				c->try_ += (-1) * 0.5 * (c->rep[u] - c->rep[d]) * phi;
				double th = (-dx * c->q00) < 0 ? 0.0 : 1.0;
				const double fsx = lambda * (-dx * c->q00) * th * c->q00;
				th = (-dy * c->q01) < 0 ? 0.0 : 1.0;
				const double fsy = lambda * (-dy * c->q01) * th * c->q01;
				fx = fpx * alpha + fsx * zs;
				fy = fpy * alpha + fsy * zs;
				if(open_site(s, k)) {
					c->tfx += fx * phi;
					c->tfy += fy * phi;
				}
			}
			else { /* RC_WETMODEL */
				const int kr = box_nb(s, k, 5), kl = box_nb(s, k, 3), ku = box_nb(s, k, 7), kd = box_nb(s, k, 1);
				const double fpx = -0.5 * ((c->fed[r] - c->mu[r] * c->phi[r] + c->dx[r] * c->fgx[r]) - (c->fed[l] - c->mu[l] * c->phi[l] + c->dx[l] * c->fgx[l])) - 0.5 * ((c->dx[u] * c->fgy[u]) - (c->dx[d] * c->fgy[d]));
				const double fpy = -0.5 * ((c->fed[u] - c->mu[u] * c->phi[u] + c->dy[u] * c->fgy[u]) - (c->fed[d] - c->mu[d] * c->phi[d] + c->dy[d] * c->fgy[d])) - 0.5 * ((c->dy[r] * c->fgx[r]) - (c->dy[l] * c->fgx[l]));
				const double fsx = -(c->q00 * dx + c->q01 * dy);
				const double fsy = -(c->q01 * dx - c->q00 * dy);
				const double fix = -(0.5 * (s->sq00[kr] - s->sq00[kl]) + 0.5 * (s->sq01[ku] - s->sq01[kd])) - fsx;
				const double fiy = -(0.5 * (s->sq01[kr] - s->sq01[kl]) - 0.5 * (s->sq00[ku] - s->sq00[kd])) - fsy;
				fx = fpx * alpha + fsx * zs + fix * zi;
				fy = fpy * alpha + fsy * zs + fiy * zi;
			}
			if(!open_site(s, k)) fx = fy = 0.; /* WetModel.cpp:686-689, WetPolarModel.cpp:334-337 */
			s->vfx[g] = fx;
			s->vfy[g] = fy;
			if(dry) {
				s->vvx[g] = fx / fr;
				s->vvy[g] = fy / fr;
			}
		}
	}
}

/* Matrix-free product with the operator the reference assembles from
 * triplets: diagonal xi + eta * sum_{4 box neighbours} n(k'), off-diagonal
 * -eta for every patch site covering a box neighbour. */
static void cg_apply(const orc_sim *s, const double *diag, const double *p, double *y) {
	const double eta = PRM(s, friction_cell);
	for(int ci = 0; ci < s->N; ci++) {
		const ocell *c = &s->c[ci];
		for(int q = 0; q < c->n; q++) {
			const long long g = s->start[ci] + q;
			const int k = c->map[q];
			double acc = diag[g] * p[g];
			static const int nbs[4] = {1, 3, 5, 7};
			for(int j = 0; j < 4; j++) {
				const int kk = box_nb(s, k, nbs[j]);
				const int *cov = &s->cover[(size_t) kk * STORE_MAX];
				for(int i = 0; i < s->cnt[kk]; i++) acc += (-eta * 1.0) * p[cov[i]];
			}
			y[g] = acc;
		}
	}
}

static double dotv(const double *a, const double *b, long long n) {
	double r = 0;
	for(long long i = 0; i < n; i++) r += a[i] * b[i];
	return r;
}

/* Eigen::ConjugateGradient semantics (see the file header). */
static int cg_solve(orc_sim *s, const double *diag, const double *invdiag, const double *b, double *x, int cold,
                    double *r, double *p, double *z, double *tmp) {
	const long long n = s->size_rows;
	const double tol = s->P.cg_tolerance > 0 ? s->P.cg_tolerance : DBL_EPSILON;
	if(cold) memset(x, 0, sizeof(double) * (size_t) n);
	cg_apply(s, diag, x, tmp);
	for(long long i = 0; i < n; i++) r[i] = b[i] - tmp[i];
	const double bn2 = dotv(b, b, n);
	s->st.cg_solves++;
	if(bn2 == 0) {
		memset(x, 0, sizeof(double) * (size_t) n);
		return RC_OK;
	}
	const double thr = fmax(tol * tol * bn2, DBL_MIN);
	double rn2 = dotv(r, r, n);
	if(rn2 < thr) {
		double rel = sqrt(rn2 / bn2);
		if(rel > s->st.cg_max_rel_residual) s->st.cg_max_rel_residual = rel;
		return RC_OK;
	}
	for(long long i = 0; i < n; i++) p[i] = invdiag[i] * r[i];
	double abs_new = dotv(r, p, n);
	long long it = 0;
	while(it < 2 * n) {
		cg_apply(s, diag, p, tmp);
		const double alpha = abs_new / dotv(p, tmp, n);
		for(long long i = 0; i < n; i++) x[i] += alpha * p[i];
		for(long long i = 0; i < n; i++) r[i] -= alpha * tmp[i];
		rn2 = dotv(r, r, n);
		if(rn2 < thr) break;
		for(long long i = 0; i < n; i++) z[i] = invdiag[i] * r[i];
		const double abs_old = abs_new;
		abs_new = dotv(r, z, n);
		const double beta = abs_new / abs_old;
		for(long long i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
		it++;
	}
	s->st.cg_iterations += (int) it;
	if(it > s->st.cg_max_iterations) s->st.cg_max_iterations = (int) it;
	double rel = sqrt(rn2 / bn2);
	if(rel > s->st.cg_max_rel_residual) s->st.cg_max_rel_residual = rel;
	return RC_OK;
}

static int viscous_solve(orc_sim *s) {
	const long long n = s->size_rows;
	const double xi = PRM(s, friction), eta = PRM(s, friction_cell);
	double *diag = (double *) malloc(sizeof(double) * (size_t) n);
	double *inv = (double *) malloc(sizeof(double) * (size_t) n);
	double *w = (double *) malloc(sizeof(double) * (size_t) n * 4);
	if(!diag || !inv || !w) {
		free(diag);
		free(inv);
		free(w);
		return fail(s, RC_ERR_OOM, "out of memory");
	}
	for(int ci = 0; ci < s->N; ci++) {
		const ocell *c = &s->c[ci];
		for(int q = 0; q < c->n; q++) {
			const long long g = s->start[ci] + q;
			const int k = c->map[q];
			double dsum = xi; /* duplicate triplets summed in insertion order */
			static const int nbs[4] = {1, 3, 5, 7};
			for(int j = 0; j < 4; j++) {
				const int kk = box_nb(s, k, nbs[j]);
				for(int i = 0; i < s->cnt[kk]; i++) dsum += eta * 1.0;
			}
			diag[g] = dsum;
			inv[g] = dsum != 0.0 ? 1.0 / dsum : 1.0;
		}
	}
	const int cold = s->size_rows != s->size_rows_old;
	int rc = cg_solve(s, diag, inv, s->vfx, s->vvx, cold, w, w + n, w + 2 * n, w + 3 * n);
	if(rc == RC_OK) rc = cg_solve(s, diag, inv, s->vfy, s->vvy, cold, w, w + n, w + 2 * n, w + 3 * n);
	if(cold) s->restart = 0;
	else s->restart += 1;
	free(diag);
	free(inv);
	free(w);
	return rc;
}

/* interaction->begin_energy_computation(fields) for the selected model. */
static int compute_forces(orc_sim *s) {
	const int wet_model = is_wet_model(s);
	if(wet_model) {
		const int every = s->P.cg_restart_every;
		if(s->restart < every) s->size_rows_old = s->size_rows;
		else {
			s->size_rows_old = 0;
			s->restart = 0;
		}
	}
	int rc = global_sums(s);
	if(rc) return rc;
	if(wet_model) {
		rc = ensure_vectors(s);
		if(rc) return rc;
		if(s->size_rows != s->size_rows_old) {
			/* Eigen resize: contents undefined; the shim zero-fills */
			memset(s->vvx, 0, sizeof(double) * (size_t) s->size_rows);
			memset(s->vvy, 0, sizeof(double) * (size_t) s->size_rows);
			memset(s->vfx, 0, sizeof(double) * (size_t) s->size_rows);
			memset(s->vfy, 0, sizeof(double) * (size_t) s->size_rows);
		}
	}
	f_interaction(s);
	if(s->P.model == RC_SIMPLEFIELD) return RC_OK;
	internal_forces(s);
	if(wet_model && PRM(s, friction_cell) != 0) return viscous_solve(s);
	return RC_OK;
}

/* ------------------------------------------------------ first_step --- */
static void set_positions(orc_sim *s, ocell *c) {
	const int L = s->L, border = s->P.border;
	if(c->xl >= border && c->yb >= border) {
		const int site = box_el(s, c->corner, (int) c->com[0], (int) c->com[1]);
		c->com[1] = (int) (site / L) + (c->com[1] - (int) c->com[1]);
		c->com[0] = (int) (site - (int) (site / L) * L) + (c->com[0] - (int) c->com[0]);
		const double cox = box_x(s, c->corner, 0), coy = box_y(s, c->corner, 0);
		c->corner_old = c->corner;
		c->corner = box_el(s, site, (int) -c->lx / 2, (int) -c->ly / 2);
		const double cnx = box_x(s, c->corner, 0), cny = box_y(s, c->corner, 0);
		const double d0 = cnx - cox - rint((cnx - cox) / L) * L;
		const double d1 = cny - coy - rint((cny - coy) / L) * L;
		c->unrap[0] += d0;
		c->unrap[1] += d1;
		c->off[0] = (int) (c->off[0] + c->lx - d0) % c->lx;
		c->off[1] = (int) (c->off[1] + c->ly - d1) % c->ly;
		return;
	}
	const int nlx = c->lx - (2 * c->xl) + (2 * border);
	const int nly = c->ly - (2 * c->yb) + (2 * border);
	const int nn = nlx * nly;
	const int ncorner = box_el(s, c->corner, -(-(2 * c->xl) + (2 * border)) / 2, -(-(2 * c->yb) + (2 * border)) / 2);
	double *nphi = (double *) calloc((size_t) (nn > 0 ? nn : 1), sizeof(double));
	c->area = 0;
	int sy, dimy, sx, dimx;
	if(nly < c->ly) { sy = (c->ly - nly) / 2; dimy = nly; }
	else { sy = 0; dimy = c->ly; }
	if(nlx < c->lx) { sx = (c->lx - nlx) / 2; dimx = nlx; }
	else { sx = 0; dimx = c->lx; }
	for(int i = sy; i < dimy; i++) {
		const int yy = box_y(s, c->corner, i);
		int offy = i - c->off[1];
		if(offy < 0) offy += c->ly;
		for(int j = sx; j < dimx; j++) {
			const int xx = box_x(s, c->corner, j);
			int dx = (ncorner - (ncorner / L) * L) - xx;
			if(dx > L / 2) dx -= L;
			else if(dx < -L / 2) dx += L;
			int dy = (ncorner / L) - yy;
			if(dy > L / 2) dy -= L;
			else if(dy < -L / 2) dy += L;
			int offx = j - c->off[0];
			if(offx < 0) offx += c->lx;
			const double v = c->phi[offx + offy * c->lx];
			nphi[abs(dx) + abs(dy) * nlx] = v;
			c->area += v * v;
		}
	}
	{
		const double ox = box_x(s, c->corner, 0), oy = box_y(s, c->corner, 0);
		const double nx = box_x(s, ncorner, 0), ny = box_y(s, ncorner, 0);
		c->unrap[0] += nx - ox - rint((nx - ox) / L) * L;
		c->unrap[1] += ny - oy - rint((ny - oy) / L) * L;
	}
	const int oldn = c->n;
	c->lx = nlx;
	c->ly = nly;
	c->corner_old = c->corner;
	c->corner = ncorner;
	c->off[0] = c->off[1] = 0;
	c->n = nn;
	cell_resize(c, oldn, nn);
	memcpy(c->phi, nphi, sizeof(double) * (size_t) nn);
	free(nphi);
	const int site = box_el(s, c->corner, c->lx / 2, c->ly / 2);
	c->com[1] = (int) (site / L);
	c->com[0] = (int) (site - (int) (site / L) * L);
	s->st.resized_cells++;
}

static int directed_active_forces(orc_sim *s, ocell *c, int store) {
	const double dt = s->P.dt, JQ = PRM(s, J_Q);
	switch(s->P.model) {
		case RC_WETPOLARMODEL: {
			if(store) c->thq_old = c->thq + sqrt(dt) * PRM(s, zetaQ_inter) * rng_gaussian(s);
			const double f0 = c->trx, f1 = c->try_;
			c->thq = c->thq_old - dt * JQ * (atan2(f0 * c->q01 - f1 * c->q00, f0 * c->q00 + f1 * c->q01));
			c->q00 = cos(c->thq);
			c->q01 = sin(c->thq);
			break;
		}
		case RC_WETMODEL: {
			const double smod = sqrt(c->s00 * c->s00 + c->s01 * c->s01);
			if(store) {
				c->nq_old[0] = c->nq[0];
				c->nq_old[1] = c->nq[1];
			}
			if(smod > 0.00000001) {
				const double t = 0.5 * atan2(c->s01, c->s00);
				const double d0 = cos(t), d1 = sin(t);
				const double sgn = (d0 * c->nq[0] + d1 * c->nq[1] > 0.0) ? 1.0 : -1.0;
				c->nq[0] = c->nq_old[0] + dt * JQ * (sgn * d0 - c->nq[0]);
				c->nq[1] = c->nq_old[1] + dt * JQ * (sgn * d1 - c->nq[1]);
				c->q00 = 0.5 * (c->nq[0] * c->nq[0] - c->nq[1] * c->nq[1]);
				c->q01 = c->nq[0] * c->nq[1];
			}
			break;
		}
		case RC_ACTIVENEMATIC: {
			if(store) {
				c->nq_old[0] = c->nq[0];
				c->nq_old[1] = c->nq[1];
			}
			if(c->type == 0) {
				c->nq[0] = c->nq_old[0];
				c->nq[1] = c->nq_old[1];
			}
			else if(c->type == 1) {
				const double t = 0.5 * atan2(c->s01, c->s00);
				const double d0 = cos(t), d1 = sin(t);
				const double sgn = (d0 * c->nq[0] + d1 * c->nq[1] > 0.0) ? 1.0 : -1.0;
				c->nq[0] = c->nq_old[0] + dt * JQ * (sgn * d0 - c->nq[0]);
				c->nq[1] = c->nq_old[1] + dt * JQ * (sgn * d1 - c->nq[1]);
				c->q00 = 0.5 * (c->nq[0] * c->nq[0] - c->nq[1] * c->nq[1]);
				c->q01 = c->nq[0] * c->nq[1];
			}
			else return fail(s, RC_ERR_INVALID, "Too many field types");
			break;
		}
		default: break;
	}
	return RC_OK;
}

static int first_step(orc_sim *s, int store) {
	const int model = s->P.model;
	const double J0 = s->P.J0, dt = s->P.dt;
	for(int ci = 0; ci < s->N; ci++) {
		ocell *c = &s->c[ci];
		double t0 = 0, t1 = 0, t2 = 0, t3 = 0;
		if(store) {
			c->com_old[0] = c->com[0];
			c->com_old[1] = c->com[1];
			c->area_old = c->area;
			c->sumf_old = c->sumf;
		}
		c->s00 = c->s01 = 0;
		c->xl = c->lx;
		c->yb = c->ly;
		c->area = 0;
		c->perim = 0;
		c->sumf = 0;
		c->com[0] = c->com[1] = 0.;
		for(int q = 0; q < c->n; q++) {
			double dphi;
			if(s->P.conserved) {
				/* FD_CHBackend::first_step (FD_CHBackend.cpp:63-68).  For the simple and
				 * nematic models the freeEnergy of the sites already updated in this loop
				 * has been reset to the external term (0) by updateFieldProperties
				 * (BaseInteraction.cpp:62-69), as mu[] is below; the wet models'
				 * updateFieldProperties (WetModel.cpp:167, WetPolarModel.cpp:130) keeps it. */
				const int nr = patch_nb(c, q, 5), nu = patch_nb(c, q, 7), nl = patch_nb(c, q, 3), nd = patch_nb(c, q, 1);
				const double lmu = c->mu[nr] + c->mu[nu] + c->mu[nl] + c->mu[nd] - 4. * c->mu[q];
				dphi = J0 * lmu - vel_x(s, c, ci, q) * c->dx[q] - vel_y(s, c, ci, q) * c->dy[q];
			}
			else
				dphi = -J0 * c->mu[q] - vel_x(s, c, ci, q) * c->dx[q] - vel_y(s, c, ci, q) * c->dy[q];
			if(store) {
				c->phi_old[q] = c->phi[q];
				c->dphi_old[q] = dphi;
			}
			const double phi = c->phi_old[q] + dt * .5 * (dphi + c->dphi_old[q]);
			c->phi[q] = phi;
			c->area += phi * phi;
			c->sumf += phi;
			const int x = ((q - (q / c->lx) * c->lx) + c->off[0]) % c->lx;
			const int y = ((q / c->lx) + c->off[1]) % c->ly;
			t0 += phi * c->ctx[x];
			t1 += phi * c->stx[x];
			t2 += phi * c->cty[y];
			t3 += phi * c->sty[y];
			if(!store && phi < 0.09 && phi > 0.01) {
				if(x < c->xl) c->xl = x;
				if(y < c->yb) c->yb = y;
			}
			if(model == RC_SIMPLEFIELD || model == RC_ACTIVENEMATIC) {
				c->tfx = c->tfy = c->trx = c->try_ = 0.;
				c->mu[q] = 0.;
				c->fed[q] = 0.;
			}
			c->s00 += -0.5 * (c->dx[q] * c->dx[q] - c->dy[q] * c->dy[q]);
			c->s01 += -c->dx[q] * c->dy[q];
		}
		c->com[0] = c->lx * (atan2(-t1 / c->sumf, -t0 / c->sumf) + PI_F) / (2 * PI_F);
		c->com[1] = c->ly * (atan2(-t3 / c->sumf, -t2 / c->sumf) + PI_F) / (2 * PI_F);
		if(!store) {
			if(!(c->xl >= s->P.border && c->yb >= s->P.border)) {
				const int nlx = c->lx - 2 * c->xl + 2 * s->P.border, nly = c->ly - 2 * c->yb + 2 * s->P.border;
				if(nlx <= 0 || nly <= 0 || nlx > s->L || nly > s->L)
					return fail(s, RC_ERR_CAPACITY, "patch of cell %d cannot be resized to %dx%d", ci, nlx, nly);
			}
			set_positions(s, c);
		}
		int rc = directed_active_forces(s, c, store);
		if(rc) return rc;
	}
	return RC_OK;
}

/* ---------------------------------------------------------- public --- */
int orc_create(const rc_params *params, const rc_box *box, int n_cells, const rc_cell_host *cells, orc_sim **out) {
	*out = NULL;
	orc_sim *s = (orc_sim *) calloc(1, sizeof(orc_sim));
	if(!s) return RC_ERR_OOM;
	*out = s;
	s->P = *params;
	s->phase = 0;
	if(box->Lx != box->Ly || box->Lx <= 2) return fail(s, RC_ERR_INVALID, "the box must be square (got %dx%d)", box->Lx, box->Ly);
	if(params->model < RC_SIMPLEFIELD || params->model > RC_WETMODEL) return fail(s, RC_ERR_INVALID, "unknown model %d", params->model);
	s->L = box->Lx;
	s->N = n_cells;
	if(box->walls) {
		const int wet = (params->model == RC_WETMODEL || params->model == RC_WETPOLARMODEL) &&
		                (params->friction_cell[0] != 0.0 || params->friction_cell[1] != 0.0);
		if(wet) return fail(s, RC_ERR_UNSUPPORTED, "walls with a viscous solve are not provided");
		s->walls = (double *) malloc(sizeof(double) * (size_t) s->L * (size_t) s->L);
		if(!s->walls) return fail(s, RC_ERR_OOM, "out of memory");
		memcpy(s->walls, box->walls, sizeof(double) * (size_t) s->L * (size_t) s->L);
	}
	s->rng = params->rng_state & 0xFFFFFFFFFFFFULL;
	s->has_g = params->rng_has_cached;
	s->next_g = params->rng_cached;
	const size_t L2 = (size_t) s->L * (size_t) s->L;
	s->phi2 = (double *) calloc(L2, sizeof(double));
	s->sq00 = (double *) calloc(L2, sizeof(double));
	s->sq01 = (double *) calloc(L2, sizeof(double));
	s->sphi = (double *) calloc(L2, sizeof(double));
	s->cnt = (int *) calloc(L2, sizeof(int));
	s->cover = (int *) calloc(L2 * STORE_MAX, sizeof(int));
	s->start = (long long *) calloc((size_t) (n_cells > 0 ? n_cells : 1), sizeof(long long));
	s->c = (ocell *) calloc((size_t) (n_cells > 0 ? n_cells : 1), sizeof(ocell));
	if(!s->phi2 || !s->sq00 || !s->sq01 || !s->sphi || !s->cnt || !s->cover || !s->start || !s->c)
		return fail(s, RC_ERR_OOM, "out of memory");
	for(int i = 0; i < n_cells; i++) {
		const rc_cell_host *h = &cells[i];
		ocell *c = &s->c[i];
		if(h->lsub_x <= 0 || h->lsub_y <= 0 || h->lsub_x > s->L || h->lsub_y > s->L)
			return fail(s, RC_ERR_INVALID, "cell %d: bad patch size %dx%d", i, h->lsub_x, h->lsub_y);
		c->lx = h->lsub_x;
		c->ly = h->lsub_y;
		c->n = c->lx * c->ly;
		c->off[0] = h->offset_x;
		c->off[1] = h->offset_y;
		c->corner = c->corner_old = h->corner;
		c->type = h->type;
		c->com[0] = c->com_old[0] = h->com_x;
		c->com[1] = c->com_old[1] = h->com_y;
		c->unrap[0] = h->unrap_x;
		c->unrap[1] = h->unrap_y;
		c->q00 = h->q00;
		c->q01 = h->q01;
		c->thq = h->theta_q;
		c->thq_old = h->theta_q_old;
		c->nq[0] = h->nemq_x;
		c->nq[1] = h->nemq_y;
		c->nq_old[0] = h->nemq_old_x;
		c->nq_old[1] = h->nemq_old_y;
		cell_resize(c, 0, c->n);
		memcpy(c->phi, h->phi, sizeof(double) * (size_t) c->n);
		c->area = 0;
		c->sumf = 0;
		for(int q = 0; q < c->n; q++) {
			c->area += c->phi[q] * c->phi[q];
			c->sumf += c->phi[q];
		}
	}
	init_field_properties(s);
	int rc = compute_forces(s);
	if(rc) return rc;
	return RC_OK;
}

int orc_step(orc_sim *s, int n_steps, rc_step_stats *stats) {
	memset(&s->st, 0, sizeof(s->st));
	for(int i = 0; i < n_steps; i++) {
		int rc = first_step(s, 1);
		if(!rc) rc = compute_forces(s);
		if(!rc) rc = first_step(s, 0);
		if(!rc) rc = compute_forces(s);
		if(rc) {
			if(stats) *stats = s->st;
			return rc;
		}
		s->st.steps_done++;
	}
	if(stats) *stats = s->st;
	return RC_OK;
}

int orc_set_phase(orc_sim *s, int active) {
	s->phase = active ? 1 : 0;
	return RC_OK;
}

int orc_get_sizes(const orc_sim *s, int *n_cells, int *lsub_x, int *lsub_y) {
	if(n_cells) *n_cells = s->N;
	for(int i = 0; i < s->N; i++) {
		if(lsub_x) lsub_x[i] = s->c[i].lx;
		if(lsub_y) lsub_y[i] = s->c[i].ly;
	}
	return RC_OK;
}

long long orc_site_count(const orc_sim *s) {
	long long n = 0;
	for(int i = 0; i < s->N; i++) n += s->c[i].n;
	return n;
}

unsigned long long orc_rng_state(const orc_sim *s) { return s->rng; }

int orc_download(const orc_sim *s, rc_cell_host *cells, unsigned mask) {
	for(int i = 0; i < s->N; i++) {
		const ocell *c = &s->c[i];
		rc_cell_host *h = &cells[i];
		if(mask & RC_FIELD_SCALARS) {
			h->lsub_x = c->lx;
			h->lsub_y = c->ly;
			h->offset_x = c->off[0];
			h->offset_y = c->off[1];
			h->corner = c->corner;
			h->type = c->type;
			h->com_x = c->com[0];
			h->com_y = c->com[1];
			h->unrap_x = c->unrap[0];
			h->unrap_y = c->unrap[1];
			h->q00 = c->q00;
			h->q01 = c->q01;
			h->theta_q = c->thq;
			h->theta_q_old = c->thq_old;
			h->nemq_x = c->nq[0];
			h->nemq_y = c->nq[1];
			h->nemq_old_x = c->nq_old[0];
			h->nemq_old_y = c->nq_old[1];
			h->area = c->area;
			h->sum_f = c->sumf;
			h->perimeter = c->perim;
			h->s00 = c->s00;
			h->s01 = c->s01;
			h->force_rep_x = c->trx;
			h->force_rep_y = c->try_;
		}
		if((mask & ~RC_FIELD_SCALARS) && h->capacity < c->n) return RC_ERR_INVALID;
		for(int q = 0; q < c->n; q++) {
			if((mask & RC_FIELD_PHI) && h->phi) h->phi[q] = c->phi[q];
			if(mask & RC_FIELD_VEL) {
				if(h->vx) h->vx[q] = s->P.model == RC_SIMPLEFIELD ? 0.0 : vel_x(s, c, i, q);
				if(h->vy) h->vy[q] = s->P.model == RC_SIMPLEFIELD ? 0.0 : vel_y(s, c, i, q);
			}
			if((mask & RC_FIELD_MU) && h->mu) h->mu[q] = c->mu[q];
			if(mask & RC_FIELD_GRAD) {
				if(h->dx) h->dx[q] = c->dx[q];
				if(h->dy) h->dy[q] = c->dy[q];
			}
			if((mask & RC_FIELD_MAP) && h->box_index) h->box_index[q] = c->map[q];
		}
	}
	return RC_OK;
}

const char *orc_last_error(const orc_sim *s) { return s ? s->err : "no simulation"; }

void orc_destroy(orc_sim *s) {
	if(!s) return;
	for(int i = 0; i < s->N && s->c; i++) {
		ocell *c = &s->c[i];
		double *arrs[] = {c->phi, c->phi_old, c->dphi_old, c->mu, c->fed, c->fgx, c->fgy, c->dx, c->dy,
		                  c->lap, c->rep, c->vx, c->vy, c->ctx, c->stx, c->cty, c->sty};
		for(size_t k = 0; k < sizeof(arrs) / sizeof(arrs[0]); k++) free(arrs[k]);
		free(c->map);
	}
	free(s->c);
	free(s->walls);
	free(s->phi2);
	free(s->sq00);
	free(s->sq01);
	free(s->sphi);
	free(s->cnt);
	free(s->cover);
	free(s->start);
	free(s->vvx);
	free(s->vvy);
	free(s->vfx);
	free(s->vfy);
	free(s);
}
