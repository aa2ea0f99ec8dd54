// Box-grid gather: for every box site, the sums over the patches covering it
// (phi^2, phi*Q00, phi*Q01) and, for the wet models, the cover list of the
// viscous operator.
//
// Reference: the scatter half of computeGlobalSums
// (src/Interactions/WetModel.cpp:440-485, WetPolarModel.cpp:355-379,
// ActiveNematic.cpp:166-174, SimpleMultiField.cpp:108-120), which loops over
// cells in index order and adds each patch site into its box site.  Here each
// box site instead gathers from the cells covering it, visited in ascending
// cell index, so every sum is formed in the reference's order (bit-identical
// for identical phi) and the result is deterministic without atomics.
//
// Covering cells are found through bins of BIN_X x BIN_Y box sites: each bin
// lists the cells whose patch rectangle overlaps it (filled by the cell
// kernels' epilogue).  One CTA handles one bin: it sorts the bin's list,
// stages the cells' geometry in shared memory and tests containment per site.
// Consecutive threads are consecutive box sites along x, which map to
// consecutive patch storage sites of the same cell, so the phi reads coalesce.
#include "rc_kernels.cuh"

namespace rc {


// F32: for the FP32 engines (dry polar, phi^2 only): conversions on the
// integer pipes and FP32 sums in the same cell order, stored exactly as
// doubles; the FP32 cell kernel reads them back in FP32.
template<bool F32>
__global__ void __launch_bounds__(BIN_X *BIN_Y) box_gather_kernel(const BoxArgs a) {
	__shared__ int s_ids[BIN_CAP];
	__shared__ int s_sorted[BIN_CAP];
	__shared__ int s_cx[BIN_CAP], s_cy[BIN_CAP], s_lx[BIN_CAP], s_ly[BIN_CAP], s_ox[BIN_CAP], s_oy[BIN_CAP],
	    s_start[BIN_CAP];
	__shared__ double s_q00[BIN_CAP], s_q01[BIN_CAP];
	const LayerDev lay = a.layers[a.bin_layer[blockIdx.x]];
	const int b = blockIdx.x;
	const int lb = b - lay.bin_off;
	const int bxi = lb % lay.nbx, byi = lb / lay.nbx;
	const int L = lay.L;
	int count = a.bin_count[b];
	if(count > BIN_CAP) count = BIN_CAP;  // overflow already flagged by the appender
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
		s_q00[t] = c.q00;
		s_q01[t] = c.q01;
	}
	__syncthreads();
	if(a.st->err & ERR_CAPACITY) return;
	const int x = bxi * BIN_X + (t % BIN_X);
	const int y = byi * BIN_Y + (t / BIN_X);
	if(x >= L || y >= L) return;
	const int kl = x + y * L;                      // site in the layer's box
	const long long k = lay.box_off + kl;          // index into the batch's box arrays
	const size_t L2 = (size_t) L * (size_t) L;
	auto site_in = [&](int i) {
		int rx = x - s_cx[i];
		if(rx < 0) rx += L;
		int ry = y - s_cy[i];
		if(ry < 0) ry += L;
		if(rx >= s_lx[i] || ry >= s_ly[i]) return -1;
		int sx = rx - s_ox[i];
		if(sx < 0) sx += s_lx[i];
		int sy = ry - s_oy[i];
		if(sy < 0) sy += s_ly[i];
		return s_start[i] + sy * s_lx[i] + sx;
	};
	if constexpr(F32) {
		float p2f = 0.f;
		int n = 0;
		for(int i = 0; i < count; i++) {
			const int j = site_in(i);
			if(j < 0) continue;
			const float phi = d2f_int(a.phi[j]);
			p2f = __fmaf_rn(phi, phi, p2f);
			n++;
		}
		a.phi2[k] = f2d_int(p2f);
		if(a.check_overlap && n > STORE_MAX) {
			atomicOr(&a.st->err, ERR_OVERLAP);
			a.st->err_where = k;
		}
		return;
	}
	double p2 = 0.0, q0 = 0.0, q1 = 0.0;
	int n = 0;
	for(int i = 0; i < count; i++) {
		const int j = site_in(i);
		if(j < 0) continue;
		const double phi = a.phi[j];
		p2 += phi * phi;
		if(a.want_q) {
			q0 += phi * s_q00[i];
			q1 += phi * s_q01[i];
		}
		if(a.want_cover) {
			// a member's cover lists are [slot][its L x L sites] from STORE_MAX * box_off
			if(n < STORE_MAX) a.cover[(size_t) STORE_MAX * lay.box_off + (size_t) n * L2 + kl] = j;
			else {
				atomicOr(&a.st->err, ERR_OVERLAP);
				a.st->err_where = k;
			}
		}
		n++;
	}
	a.phi2[k] = p2;
	if(a.want_q) {
		a.sq00[k] = q0;
		a.sq01[k] = q1;
	}
	if(a.want_cover) a.cnt[k] = n > STORE_MAX ? STORE_MAX : n;
	else if(a.check_overlap && n > STORE_MAX) {
		// the reference's cover-list bound applies to the wet models' dry phase too
		atomicOr(&a.st->err, ERR_OVERLAP);
		a.st->err_where = k;
	}
}

// Solver bookkeeping of the wet models, once per evaluation
// (WetModel.cpp:195-209,366-375; WetPolarModel.cpp:270-285,342-351).
__global__ void bookkeeping_kernel(DevStatus *st, int restart_every, int solve_follows) {
	long long rows_old;
	if(st->restart < restart_every) rows_old = st->S_rows;
	else {
		rows_old = 0;
		st->restart = 0;
	}
	st->S_rows = st->S;
	if(solve_follows) st->cg_cold = (st->S_rows != rows_old) ? 1 : 0;
}

// The same bookkeeping for every member of a wet ensemble, one thread per
// member: a member's unknowns are its cells' sites.
__global__ void bookkeeping_layers_kernel(const CellDev *cells, const LayerDev *layers, int n_layers, LayerSolve *ls,
                                          int restart_every, int solve_follows) {
	const int l = blockIdx.x * blockDim.x + threadIdx.x;
	if(l >= n_layers) return;
	const LayerDev &ly = layers[l];
	const long long S = ly.cell_hi > ly.cell_lo
	                        ? (long long) cells[ly.cell_hi - 1].start + cells[ly.cell_hi - 1].n - cells[ly.cell_lo].start
	                        : 0;
	LayerSolve &b = ls[l];
	long long rows_old;
	if(b.restart < restart_every) rows_old = b.S_rows;
	else {
		rows_old = 0;
		b.restart = 0;
	}
	b.S_rows = S;
	if(solve_follows) b.cg_cold = (b.S_rows != rows_old) ? 1 : 0;
}

void launch_box_gather(const BoxArgs &a, cudaStream_t s) {
	if(a.f32) box_gather_kernel<true><<<a.total_bins, BIN_X * BIN_Y, 0, s>>>(a);
	else box_gather_kernel<false><<<a.total_bins, BIN_X * BIN_Y, 0, s>>>(a);
	if(a.bookkeeping) {
		if(a.lsolve)
			bookkeeping_layers_kernel<<<(a.n_layers + 127) / 128, 128, 0, s>>>(a.cells, a.layers, a.n_layers, a.lsolve,
			                                                                   a.restart_every, a.solve_follows);
		else bookkeeping_kernel<<<1, 1, 0, s>>>(a.st, a.restart_every, a.solve_follows);
	}
}

}  // namespace rc
