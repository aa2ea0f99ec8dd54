// Diagnostic observables on the device.
//
// Box fields of the reference's field observables (paths relative to its
// src/):
//   VelocityField::calc_field  Observables/VelocityField.cpp:69-78
//   ShapeField::calc_field     Observables/ShapeField.cpp:69-78 (S00, S01 of each cell)
//   NematicField::calc_field   Observables/NematicField.cpp:69-78 (Q00, Q01 of each cell)
// F[k] = sum over the visible cells, in index order, of g(cell, q) * phi(q)
// at the patch site q that maps to box site k, and the coarse-grained field
// (VelocityField.cpp:105-121): the mean over a size_grid x size_grid periodic
// window, each term divided by size_grid^2 as the reference writes it.  As in
// the box gather, each box site visits the cells covering it in ascending
// index, so the fields are formed in the reference's order.
//
// Per-cell shape statistics (the reference's analysis script
// scripts/calcAvgShape.py:274-336): with a = sum dx^2, b = sum dy^2,
// c = sum dx dy over the patch (current gradients), S00 = -(a - b)/2,
// S01 = -c, elongation |S| = sqrt(S00^2 + S01^2), orientation
// theta = atan2(S01, S00)/2, aspect ratio sqrt(s1/s2) - 1 with s1, s2 the
// eigenvalues (a + b)/2 +- |S| of [[a, c], [c, b]].  The unwrapped centre of
// mass (the position an MSD or speed uses, scripts/MSD_calc.py) is the
// unwrapped patch corner plus the centre of mass's offset from the corner.
#include "rc_kernels.cuh"

namespace rc {

struct ObsArgs {
	const CellDev *cells;
	const LayerDev *layers;
	const int *bin_count, *bin_cells;
	const double *phi, *vx, *vy;
	int kind, layer, only_type;
	double *fx, *fy;
	double scale;  // OBS_SITES: per-site values are multiplied by it first; OBS_THERMO: 2 gamma lambda
	// OBS_THERMO: free-energy density, chemical potential and gradients per
	// site; sub 0: (xx, yy), 1: (xy, mu), 2: (mu^2, phi)
	const double *fd, *mu, *dxg, *dyg;
	int sub;
};

// OBS_SITES: f0 += (vx[j] * scale) * phi, f1 += (vy[j] * scale) * phi, or
// f1 += phi when vy is null -- ForceField / StressField::calc_field
// (ForceField.cpp:79-96, StressField.cpp:84-100): total force (v times the
// friction, get_total_force_x/y), passive and active forces, pressure with
// the phi field.
// OBS_THERMO: ThermodynamicStressField::calc_field (ThermodynamicStressField.cpp:75-99),
// unweighted per-site sums: xx += f_d - mu phi + dx g_x, yy likewise with y,
// xy += dx g_y, with g = 2 gamma lambda grad(phi) (WetModel.cpp:608-609;
// zero for the models that do not set it), and the sums of mu, mu^2, phi.
enum { OBS_VELOCITY = 0, OBS_SHAPE = 1, OBS_NEMATIC = 2, OBS_SITES = 3, OBS_THERMO = 4 };

__global__ void __launch_bounds__(BIN_X *BIN_Y) obs_field_kernel(const ObsArgs a) {
	__shared__ int s_ids[BIN_CAP];
	__shared__ int s_sorted[BIN_CAP];
	__shared__ int s_cx[BIN_CAP], s_cy[BIN_CAP], s_lx[BIN_CAP], s_ly[BIN_CAP], s_ox[BIN_CAP], s_oy[BIN_CAP],
	    s_start[BIN_CAP], s_vis[BIN_CAP];
	__shared__ double s_g0[BIN_CAP], s_g1[BIN_CAP];
	const LayerDev lay = a.layers[a.layer];
	const int b = lay.bin_off + blockIdx.x;
	const int bxi = blockIdx.x % lay.nbx, byi = blockIdx.x / lay.nbx;
	const int L = lay.L;
	int count = a.bin_count[b];
	if(count > BIN_CAP) count = BIN_CAP;
	const int t = threadIdx.x;
	if(t < count) s_ids[t] = a.bin_cells[(size_t) b * BIN_CAP + t];
	__syncthreads();
	if(t < count) {
		const int id = s_ids[t];
		int rank = 0;
		for(int j = 0; j < count; j++) rank += (s_ids[j] < id);
		s_sorted[rank] = id;
	}
	__syncthreads();
	if(t < count) {
		const CellDev &c = a.cells[s_sorted[t]];
		s_cx[t] = c.corner % L;
		s_cy[t] = c.corner / L;
		s_lx[t] = c.lx;
		s_ly[t] = c.ly;
		s_ox[t] = c.offx;
		s_oy[t] = c.offy;
		s_start[t] = c.start;
		s_vis[t] = (a.only_type < 0 || c.type == a.only_type);
		s_g0[t] = a.kind == OBS_SHAPE ? c.s00 : c.q00;
		s_g1[t] = a.kind == OBS_SHAPE ? c.s01 : c.q01;
	}
	__syncthreads();
	const int x = bxi * BIN_X + (t % BIN_X);
	const int y = byi * BIN_Y + (t / BIN_X);
	if(x >= L || y >= L) return;
	double f0 = 0.0, f1 = 0.0;
	for(int i = 0; i < count; i++) {
		if(!s_vis[i]) continue;
		int rx = x - s_cx[i];
		if(rx < 0) rx += L;
		int ry = y - s_cy[i];
		if(ry < 0) ry += L;
		if(rx >= s_lx[i] || ry >= s_ly[i]) continue;
		int sx = rx - s_ox[i];
		if(sx < 0) sx += s_lx[i];
		int sy = ry - s_oy[i];
		if(sy < 0) sy += s_ly[i];
		const int j = s_start[i] + sy * s_lx[i] + sx;
		const double phi = a.phi[j];
		if(a.kind == OBS_VELOCITY) {
			f0 += a.vx[j] * phi;
			f1 += a.vy[j] * phi;
		}
		else if(a.kind == OBS_SITES) {
			f0 += (a.vx[j] * a.scale) * phi;
			f1 += a.vy ? (a.vy[j] * a.scale) * phi : phi;
		}
		else if(a.kind == OBS_THERMO) {
			const double mu = a.mu[j], dx = a.dxg[j], dy = a.dyg[j];
			const double gx = a.scale * dx, gy = a.scale * dy;
			if(a.sub == 0) {
				f0 += a.fd[j] - mu * phi + dx * gx;
				f1 += a.fd[j] - mu * phi + dy * gy;
			}
			else if(a.sub == 1) {
				f0 += dx * gy;
				f1 += mu;
			}
			else {
				f0 += mu * mu;
				f1 += phi;
			}
		}
		else {
			f0 += s_g0[i] * phi;
			f1 += s_g1[i] * phi;
		}
	}
	a.fx[x + y * L] = f0;
	a.fy[x + y * L] = f1;
}

// Coarse-grained field: per site the reference's window loop (rows outer,
// columns inner), each term divided by size_grid^2.
__global__ void obs_coarse_kernel(const double *f, double *out, int L, int sg) {
	const int site = blockIdx.x * blockDim.x + threadIdx.x;
	if(site >= L * L) return;
	const int i = site / L, j = site - (site / L) * L;
	const double den = (double) (sg * sg);
	double acc = 0.0;
	for(int k = 0; k < sg; k++)
		for(int l = 0; l < sg; l++) {
			const int xx = (((j - sg / 2 + L) % L) + l) % L;
			const int yy = (((i - sg / 2 + L) % L) + k) % L;
			acc += f[xx + yy * L] / den;
		}
	out[site] = acc;
}

// StressField's coarse stress (StressField.cpp:171-199): per site, over the
// size_grid^2 window in the reference's order (rows outer, columns inner),
// with r the periodic offset of the window site from the centre and
// e = -r / |r| (the centre itself skipped):
//   xx += fx * ex / sg^2, yy += fy * ey / sg^2,
//   xy += (fx * ey + fy * ex) / (2 sg^2)  (xy null: not formed).
__global__ void obs_stress_kernel(const double *fx, const double *fy, double *xx, double *yy, double *xy, int L, int sg) {
	const int site = blockIdx.x * blockDim.x + threadIdx.x;
	if(site >= L * L) return;
	const int i = site / L, j = site - (site / L) * L;
	double axx = 0.0, ayy = 0.0, axy = 0.0;
	for(int k = 0; k < sg; k++)
		for(int l = 0; l < sg; l++) {
			const int xx_ = (((j - sg / 2 + L) % L) + l) % L;
			const int yy_ = (((i - sg / 2 + L) % L) + k) % L;
			const int ss = xx_ + yy_ * L;
			double rx = j - xx_, ry = i - yy_;
			if(rx >= L / 2) rx -= L;
			if(rx <= -L / 2) rx += L;
			if(ry >= L / 2) ry -= L;
			if(ry <= -L / 2) ry += L;
			const double r = sqrt(rx * rx + ry * ry);
			if(r != 0) {
				const double ex = -rx / r, ey = -ry / r;
				axx += (fx[ss] * ex) / (sg * sg);
				ayy += (fy[ss] * ey) / (sg * sg);
				if(xy) axy += ((fx[ss] * ey + fy[ss] * ex)) / (2 * sg * sg);
			}
		}
	xx[site] = axx;
	yy[site] = ayy;
	if(xy) xy[site] = axy;
}

// Per-cell statistics (one CTA per cell): x, y, area, elongation, aspect, theta.
__global__ void __launch_bounds__(256) obs_cells_kernel(const CellDev *cells, const LayerDev *layers, const double *dxg,
                                                        const double *dyg, double *out) {
	__shared__ double red[3 * (256 / 32 + 1)];
	const int ci = blockIdx.x;
	const CellDev &c = cells[ci];
	double v[3] = {0.0, 0.0, 0.0};
	for(int q = threadIdx.x; q < c.n; q += blockDim.x) {
		const double dx = dxg[c.start + q], dy = dyg[c.start + q];
		v[0] += dx * dx;
		v[1] += dy * dy;
		v[2] += dx * dy;
	}
	block_sum<3>(v, red);
	if(threadIdx.x == 0) {
		const int L = layers[c.layer].L;
		double ox = c.comx - (double) (c.corner % L), oy = c.comy - (double) (c.corner / L);
		if(ox < 0) ox += L;
		if(oy < 0) oy += L;
		const double s00 = -0.5 * (v[0] - v[1]), s01 = -v[2];
		const double D = sqrt(s00 * s00 + s01 * s01);
		const double T = 0.5 * (v[0] + v[1]);
		double *o = out + (size_t) ci * 6;
		o[0] = c.unrapx + ox;
		o[1] = c.unrapy + oy;
		o[2] = c.area;
		o[3] = D;
		o[4] = (T - D) > 0.0 ? sqrt((T + D) / (T - D)) - 1.0 : 0.0;
		o[5] = 0.5 * atan2(s01, s00);
	}
}

// Per-member means in cell order (one thread per member): mean area, area
// variance, mean elongation, mean aspect ratio.
__global__ void obs_layers_kernel(const LayerDev *layers, int n_layers, const double *cell_obs, double *out) {
	const int l = blockIdx.x * blockDim.x + threadIdx.x;
	if(l >= n_layers) return;
	const int lo = layers[l].cell_lo, hi = layers[l].cell_hi, n = hi - lo;
	double sa = 0.0, se = 0.0, sr = 0.0;
	for(int i = lo; i < hi; i++) {
		sa += cell_obs[(size_t) i * 6 + 2];
		se += cell_obs[(size_t) i * 6 + 3];
		sr += cell_obs[(size_t) i * 6 + 4];
	}
	const double ma = n ? sa / n : 0.0;
	double va = 0.0;
	for(int i = lo; i < hi; i++) {
		const double d = cell_obs[(size_t) i * 6 + 2] - ma;
		va += d * d;
	}
	out[(size_t) l * 4 + 0] = ma;
	out[(size_t) l * 4 + 1] = n ? va / n : 0.0;
	out[(size_t) l * 4 + 2] = n ? se / n : 0.0;
	out[(size_t) l * 4 + 3] = n ? sr / n : 0.0;
}

void launch_obs_field(const CellDev *cells, const LayerDev *layers, const LayerDev &lay_h, const int *bin_count,
                      const int *bin_cells, const double *phi, const double *vx, const double *vy, int kind, int layer,
                      int only_type, double *fx, double *fy, cudaStream_t s) {
	ObsArgs a;
	memset(&a, 0, sizeof(a));
	a.cells = cells;
	a.layers = layers;
	a.bin_count = bin_count;
	a.bin_cells = bin_cells;
	a.phi = phi;
	a.vx = vx;
	a.vy = vy;
	a.kind = kind;
	a.layer = layer;
	a.only_type = only_type;
	a.fx = fx;
	a.fy = fy;
	a.scale = 1.0;
	obs_field_kernel<<<lay_h.nbx * lay_h.nby, BIN_X * BIN_Y, 0, s>>>(a);
}

void launch_obs_sites(const CellDev *cells, const LayerDev *layers, const LayerDev &lay_h, const int *bin_count,
                      const int *bin_cells, const double *phi, const double *g0, const double *g1, double scale, int layer,
                      int only_type, double *fx, double *fy, cudaStream_t s) {
	ObsArgs a;
	memset(&a, 0, sizeof(a));
	a.cells = cells;
	a.layers = layers;
	a.bin_count = bin_count;
	a.bin_cells = bin_cells;
	a.phi = phi;
	a.vx = g0;
	a.vy = g1;
	a.kind = OBS_SITES;
	a.layer = layer;
	a.only_type = only_type;
	a.fx = fx;
	a.fy = fy;
	a.scale = scale;
	obs_field_kernel<<<lay_h.nbx * lay_h.nby, BIN_X * BIN_Y, 0, s>>>(a);
}

void launch_obs_thermo(const CellDev *cells, const LayerDev *layers, const LayerDev &lay_h, const int *bin_count,
                       const int *bin_cells, const double *phi, const double *fd, const double *mu, const double *dxg,
                       const double *dyg, double g2, int sub, int layer, int only_type, double *fx, double *fy,
                       cudaStream_t s) {
	ObsArgs a;
	memset(&a, 0, sizeof(a));
	a.cells = cells;
	a.layers = layers;
	a.bin_count = bin_count;
	a.bin_cells = bin_cells;
	a.phi = phi;
	a.kind = OBS_THERMO;
	a.layer = layer;
	a.only_type = only_type;
	a.fx = fx;
	a.fy = fy;
	a.scale = g2;
	a.fd = fd;
	a.mu = mu;
	a.dxg = dxg;
	a.dyg = dyg;
	a.sub = sub;
	obs_field_kernel<<<lay_h.nbx * lay_h.nby, BIN_X * BIN_Y, 0, s>>>(a);
}

void launch_obs_stress(const double *fx, const double *fy, double *xx, double *yy, double *xy, int L, int sg, cudaStream_t s) {
	obs_stress_kernel<<<(L * L + 255) / 256, 256, 0, s>>>(fx, fy, xx, yy, xy, L, sg);
}

void launch_obs_coarse(const double *f, double *out, int L, int sg, cudaStream_t s) {
	obs_coarse_kernel<<<(L * L + 255) / 256, 256, 0, s>>>(f, out, L, sg);
}

void launch_obs_cells(const CellDev *cells, const LayerDev *layers, int N, int n_layers, const double *dxg,
                      const double *dyg, double *cell_obs, double *layer_obs, cudaStream_t s) {
	if(N > 0) obs_cells_kernel<<<N, 256, 0, s>>>(cells, layers, dxg, dyg, cell_obs);
	obs_layers_kernel<<<(n_layers + 63) / 64, 64, 0, s>>>(layers, n_layers, cell_obs, layer_obs);
}

}  // namespace rc
