// Shared device-side definitions of the GB300 multi-phase-field engine.
//
// State layout in HBM (all FP64 unless noted):
//   * per-site arrays, "flat": the patches of all cells concatenated in cell
//     order, each patch in storage order (LsubX fastest).  This is exactly the
//     order of the reference's stacked viscous-solve unknowns
//     (field_start_index, src/Interactions/WetModel.cpp:203-209), so the
//     solver's warm start has the same meaning as the reference's.
//   * per-cell records (CellDev, one 288-byte struct per cell);
//   * box arrays of L*L entries (phi^2 sum, phi*Q sums, patch counts) and the
//     cover lists of the wet models, slot-major ([slot][box site]) so that
//     consecutive box sites read consecutive addresses.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace rc {

constexpr int STORE_MAX = 20;        // store_max_size (src/Interactions/WetModel.cpp:58)
constexpr int MAX_TABLE_SIDE = 128;  // patch sides with precomputed trig tables
constexpr int MAX_PATCH_SITES = 16384;
constexpr int BIN_X = 32, BIN_Y = 8; // box bins for the cover search (one CTA each)
constexpr int BIN_CAP = 128;         // cells listed per bin
constexpr int CELL_THREADS = 256;
// FP32 cell kernel: threads per cell patch, chosen among these by rc_autotune
constexpr int CELL_MAX_THREADS = 512;
constexpr int CELL_F32_BLOCKS[3] = {128, 256, 512};
constexpr int OVERFLOW_SLOTS = 64;   // cells per launch whose patch exceeds shared memory

enum Model { M_SIMPLE = 0, M_NEMATIC = 1, M_POLAR = 2, M_WET = 3 };

// Error bits accumulated on the device and reported by rc_step.
enum ErrBits {
	ERR_OVERLAP = 1,    // > STORE_MAX patches on one box site (WetModel.cpp:475-480)
	ERR_CAPACITY = 2,   // patch or site capacity exceeded
	ERR_NONFINITE = 4,  // NaN/Inf in a cell's sums
	ERR_BIN = 8,        // bin list overflow
	ERR_BARRIER = 16,   // a grid barrier timed out
	ERR_TYPE = 32,      // activenematic type other than 0/1
	ERR_MMA = 64,       // a tensor-core completion wait timed out
	ERR_NOCONV = 128,   // a viscous solve stopped at its iteration cap above the tolerance
	ERR_COPY = 256,     // a bulk-copy completion wait timed out
};

// Phase-dependent parameters (see rc_params in the C header).
struct PhaseParams {
	double friction, friction_cell, zs, zi, JQ, beta;
};

struct DevParams {
	int model, L, border, conserved;  // conserved: FD_CH dynamics
	double dt, J0, gamma, lambda, omega, mu, kappa, passive_alpha, a0, cg_tol;
	double wall_slip;  // open box sites have a wall value below it (wall boxes only)
};

struct CellDev {
	int lx, ly, offx, offy;
	int corner, type, start, n;
	int xl, yb, resized, old_lx;
	int old_ly, old_offx, old_offy, old_corner;
	int layer, pad_i;
	double comx, comy, com_oldx, com_oldy;
	double unrapx, unrapy, q00, q01;
	double thq, thq_old, nqx, nqy;
	double nq_oldx, nq_oldy, area, area_old;
	double sumf, sumf_old, perim, s00;
	double s01, trx, try_, tfx;
	double tfy, gauss, pad0, pad1;
};

// One monolayer of a batch: its own periodic box, box arrays at box_off,
// bins at bin_off, cells [cell_lo, cell_hi), and its own drand48 stream.
struct LayerDev {
	int L, nbx, nby, bin_off;
	long long box_off;
	int cell_lo, cell_hi;
	unsigned long long rng_state;
	int rng_has, pad;
	double rng_cached;
};

// Device status word block (one per engine).
struct DevStatus {
	int err;
	int err_where;
	int resized;      // patches resized by the last corrector
	int max_n;        // largest patch (sites) after the last corrector
	long long S;      // sites = sum of patch sizes (= viscous unknowns)
	long long S_rows; // size_rows of the last evaluation (solver bookkeeping)
	int restart;      // restart_solver
	int cg_cold;      // the next solve starts from zero
	// counters since the last status read (zeroed together, one memset)
	int cg_solves;
	int cg_iters;
	int cg_max_iters;
	int refinements;
	int fallbacks;    // mixed/learned solves finished by the plain FP64 CG
	int pad_fb;
	double cg_max_rel;
	int resized_total;
	int overflow_used;
	unsigned long long rng_state;
	int rng_has;
	int pad2;
	double rng_cached;
};

// Solver bookkeeping of one member of a wet ensemble (the single-monolayer
// engine keeps it in DevStatus): size_rows, restart_solver and the cold-start
// flag of its next solve (WetModel.cpp:195-209).
struct LayerSolve {
	long long S_rows;
	int restart;
	int cg_cold;
};

__host__ __device__ inline int wrapi(int v, int L) {
	v %= L;
	return v < 0 ? v + L : v;
}

// Box site of patch storage site (sx, sy) (GetSubIndex, MultiPhaseField.cpp:348-350).
__device__ inline int box_site(const CellDev &c, int sx, int sy, int L) {
	int lx = sx + c.offx;
	if(lx >= c.lx) lx -= c.lx;
	int ly = sy + c.offy;
	if(ly >= c.ly) ly -= c.ly;
	int x = c.corner % L + lx;
	if(x >= L) x -= L;
	int y = c.corner / L + ly;
	if(y >= L) y -= L;
	return x + y * L;
}

// Trig table index of patch side l (tables for sides 1..MAX_TABLE_SIDE packed).
__host__ __device__ inline int table_base(int l) { return (l * (l - 1)) / 2; }

// Deterministic block-wide sum of NV doubles per thread (fixed shuffle tree).
// `scratch` holds NV * (blockDim/32 + 1) doubles.  Result valid in every thread.
// Only warp 0 combines the per-warp partials: on GB300 every FP64 warp
// instruction is expensive, so no thread repeats that work.
template<int NV>
__device__ inline void block_sum(double (&v)[NV], double *scratch) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
	for(int i = 0; i < NV; i++) {
#pragma unroll
		for(int o = 16; o > 0; o >>= 1) v[i] += __shfl_down_sync(0xffffffffu, v[i], o);
	}
	__syncthreads();
	if(lane == 0) {
#pragma unroll
		for(int i = 0; i < NV; i++) scratch[i * nw + warp] = v[i];
	}
	__syncthreads();
	if(warp == 0) {
#pragma unroll
		for(int i = 0; i < NV; i++) {
			double s = lane < nw ? scratch[i * nw + lane] : 0.0;
#pragma unroll
			for(int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
			if(lane == 0) scratch[NV * nw + i] = s;
		}
	}
	__syncthreads();
#pragma unroll
	for(int i = 0; i < NV; i++) v[i] = scratch[NV * nw + i];
	__syncthreads();
}

template<int NV>
__device__ inline void block_min(int (&v)[NV], int *scratch) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
	for(int i = 0; i < NV; i++) {
#pragma unroll
		for(int o = 16; o > 0; o >>= 1) v[i] = min(v[i], __shfl_down_sync(0xffffffffu, v[i], o));
	}
	__syncthreads();
	if(lane == 0) {
#pragma unroll
		for(int i = 0; i < NV; i++) scratch[i * nw + warp] = v[i];
	}
	__syncthreads();
#pragma unroll
	for(int i = 0; i < NV; i++) {
		int s = scratch[i * nw];
		for(int w = 1; w < nw; w++) s = min(s, scratch[i * nw + w]);
		v[i] = s;
	}
	__syncthreads();
}

// double <-> float conversions on the integer pipes (on GB300 the conversion
// instructions issue on the narrow FP64 pipe).  Round to nearest even;
// magnitudes below the FP32 normal range become zero and the fields' values
// never reach the FP32 overflow range.
__device__ __forceinline__ float d2f_int(double v) {
	const unsigned hi = (unsigned) __double2hiint(v), lo = (unsigned) __double2loint(v);
	const unsigned sign = hi & 0x80000000u;
	const int e = (int) ((hi >> 20) & 0x7FFu) - 896;  // FP32 biased exponent
	if(e <= 0) return __uint_as_float(sign);
	unsigned m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
	const unsigned r = lo & 0x1FFFFFFFu;
	unsigned bits = sign | ((unsigned) e << 23);
	bits += m;
	if(r > 0x10000000u || (r == 0x10000000u && (m & 1u))) bits += 1u;  // carries into the exponent
	return __uint_as_float(bits);
}

// The short form for streams: one funnel shift takes the low 9 exponent bits
// and the top 23 mantissa bits together, a subtraction of 384 << 23 rebiases
// the exponent modulo 2^9 (exact for every FP32 normal), and the first
// dropped bit is added (round to nearest, ties away from zero: differs from
// d2f_int on exact ties only).  Below the FP32 normal range -> signed zero;
// beyond the FP32 range, infinities and NaN -> NaN, so a non-finite input
// stays non-finite.
__device__ __forceinline__ float d2f_fast(double v) {
	const unsigned hi = (unsigned) __double2hiint(v), lo = (unsigned) __double2loint(v);
	const unsigned mag = hi & 0x7FFFFFFFu, sign = hi ^ mag;
	unsigned b = __funnelshift_l(lo, hi, 3) - (384u << 23) + ((lo >> 28) & 1u);
	b = mag < (897u << 20) ? 0u : b;
	b = mag >= (1151u << 20) ? 0x7FC00000u : b;
	return __uint_as_float(b | sign);
}

__device__ __forceinline__ double f2d_int(float v) {
	const unsigned b = __float_as_uint(v);
	const unsigned sign = b & 0x80000000u, e = (b >> 23) & 0xFFu, m = b & 0x7FFFFFu;
	if(e == 0u) return __hiloint2double((int) sign, 0);
	return __hiloint2double((int) (sign | ((e + 896u) << 20) | (m >> 3)), (int) (m << 29));
}

}  // namespace rc
