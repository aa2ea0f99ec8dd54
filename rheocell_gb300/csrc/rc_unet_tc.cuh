// Inference of the learned preconditioner's network on the tensor cores:
// BF16 activations (channel-last, 16 channels = 32 bytes per pixel), FP32
// accumulation in TMEM.  The nine 16->16 and 32->16 layers are implicit
// GEMMs (M = 128 pixels, N = 16 output channels, K = 16 input channels per
// instruction, nine taps); the first (2 -> 16) and last (16 -> 1) layers are
// light and run on the CUDA cores in FP32.
#pragma once

#include "rc_tc.cuh"
#include "rc_unet.cuh"

#include <cuda_bf16.h>

namespace rc {

typedef __nv_bfloat16 bf16;

// BF16 activations of one forward pass (layouts as UNetActs).
struct UNetActsBF {
	bf16 *e0a, *s0, *d0a, *t0;  // level 0
	bf16 *e1a, *s1, *d1a, *t1;  // level 1
	bf16 *b0, *t2;              // level 2
};

struct TcSrc {
	int mode;
	const bf16 *a;
	const bf16 *b;
};

__host__ __device__ inline TcSrc unet_tc_src(int l, const UNetActsBF &A) {
	switch(l) {
	case L_E0B: return TcSrc{IN_DIRECT, A.e0a, nullptr};
	case L_E1A: return TcSrc{IN_POOL, A.s0, nullptr};
	case L_E1B: return TcSrc{IN_DIRECT, A.e1a, nullptr};
	case L_B0: return TcSrc{IN_POOL, A.s1, nullptr};
	case L_B1: return TcSrc{IN_DIRECT, A.b0, nullptr};
	case L_D1A: return TcSrc{IN_UPCAT, A.t2, A.s1};
	case L_D1B: return TcSrc{IN_DIRECT, A.d1a, nullptr};
	case L_D0A: return TcSrc{IN_UPCAT, A.t1, A.s0};
	case L_D0B: return TcSrc{IN_DIRECT, A.d0a, nullptr};
	default: return TcSrc{IN_DIRECT, nullptr, nullptr};
	}
}

__host__ __device__ inline bf16 *unet_tc_dst(int l, const UNetActsBF &A) {
	switch(l) {
	case L_E0A: return A.e0a;
	case L_E0B: return A.s0;
	case L_E1A: return A.e1a;
	case L_E1B: return A.s1;
	case L_B0: return A.b0;
	case L_B1: return A.t2;
	case L_D1A: return A.d1a;
	case L_D1B: return A.t1;
	case L_D0A: return A.d0a;
	case L_D0B: return A.t0;
	default: return nullptr;
	}
}

// Packed BF16 weights: layer l at element offset unet_pack_offset(l) (the
// FP32 weight offsets without the biases); within a tensor-core layer the
// order is [tap][kc][co][8] (kc = input channels / 8), the K-major B
// operand in core matrices.
__host__ __device__ constexpr int unet_pack_offset(int l) {
	int off = 0;
	for(int k = 0; k < l; k++) off += 9 * unet_layer(k).ci * unet_layer(k).co;
	return off;
}
constexpr int UNET_PACKED = unet_pack_offset(UNET_LAYERS);

constexpr int TC_RT = 2;       // tiles (of 128 pixels) per round, gathered operands
constexpr int TC_RT_ROWS = 4;  // tiles per round, row-halo operands
constexpr int TC_COLS = 64;    // TMEM columns: up to TC_RT_ROWS accumulators of 16
constexpr int TC_HALO = 130;   // staged positions per row: 128 pixels and a periodic neighbour on each side
constexpr size_t TC_A_GATHER = (size_t) TC_RT * 9 * 4 * 128 * 16;
constexpr size_t TC_A_ROWS = (size_t) TC_RT_ROWS * 4 * 3 * TC_HALO * 16;
constexpr size_t TC_A_BYTES = TC_A_GATHER > TC_A_ROWS ? TC_A_GATHER : TC_A_ROWS;
constexpr size_t TC_B_OFF = TC_A_BYTES;
constexpr size_t TC_B_BYTES = 9 * 4 * 16 * 16;
constexpr size_t TC_BIAS_OFF = TC_B_OFF + TC_B_BYTES;
constexpr size_t TC_TILE_OFF = TC_BIAS_OFF + 64;        // per-tile (n, y, x0), row mode
constexpr size_t TC_MBAR_OFF = TC_TILE_OFF + 16 * TC_RT_ROWS;
constexpr size_t TC_HOLD_OFF = TC_MBAR_OFF + 8;
constexpr size_t TC_SMEM = TC_HOLD_OFF + 8;
constexpr uint32_t TC_IDESC = tc_idesc_bf16(128, 16);
constexpr long long TC_WAIT_LIMIT = 2000000;  // mbarrier polls (each a bounded hardware wait)

__device__ __forceinline__ float2 bf2f(uint32_t u) {
	__nv_bfloat162 h = *reinterpret_cast<__nv_bfloat162 *>(&u);
	return __bfloat1622float2(h);
}
__device__ __forceinline__ uint32_t f2bf(float a, float b) {
	__nv_bfloat162 h = __floats2bfloat162_rn(a, b);
	return *reinterpret_cast<uint32_t *>(&h);
}

// Input channels [8 kc, 8 kc + 8) of a layer's input at (n, i, j), side L.
__device__ __forceinline__ uint4 tc_load_chunk(const TcSrc &s, int ci, int n, int i, int j, int L, int kc) {
	if(s.mode == IN_DIRECT) return *reinterpret_cast<const uint4 *>(s.a + ((size_t) (n * L + i) * L + j) * ci + kc * 8);
	if(s.mode == IN_POOL) {
		const int L2 = 2 * L;
		float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
		for(int q = 0; q < 4; q++) {
			const uint4 v = *reinterpret_cast<const uint4 *>(
			    s.a + ((size_t) (n * L2 + 2 * i + (q >> 1)) * L2 + 2 * j + (q & 1)) * ci + kc * 8);
			const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
			for(int e = 0; e < 4; e++) {
				const float2 f = bf2f(w[e]);
				acc[2 * e] += f.x;
				acc[2 * e + 1] += f.y;
			}
		}
		uint4 o;
		o.x = f2bf(0.25f * acc[0], 0.25f * acc[1]);
		o.y = f2bf(0.25f * acc[2], 0.25f * acc[3]);
		o.z = f2bf(0.25f * acc[4], 0.25f * acc[5]);
		o.w = f2bf(0.25f * acc[6], 0.25f * acc[7]);
		return o;
	}
	if(kc < 2) {
		const int Lh = L / 2;
		return *reinterpret_cast<const uint4 *>(s.a + ((size_t) (n * Lh + i / 2) * Lh + j / 2) * 16 + kc * 8);
	}
	return *reinterpret_cast<const uint4 *>(s.b + ((size_t) (n * L + i) * L + j) * 16 + (kc - 2) * 8);
}

// Row-mode operand staging of nt tiles (KC = input channels / 8): chunk
// c = r * RB + (kc * 3 + row) * TC_HALO + pos holds channels 8 kc .. of input
// pixel (n, y + row - 1, x0 + pos - 1) of tile r (coordinates in tile[r]).
template<int KC>
__device__ __forceinline__ void tc_stage_rows(const TcSrc &src, const int4 *tile, int nt, int L, uint4 *As) {
	constexpr int RB = KC * 3 * TC_HALO;
	const int nchunk = nt * RB;
	if(src.mode != IN_POOL) {
		for(int c = threadIdx.x; c < nchunk; c += blockDim.x) {
			const int r = c / RB, rem = c - r * RB;
			const int kc = rem / (3 * TC_HALO), rem2 = rem - kc * (3 * TC_HALO);
			const int row = rem2 / TC_HALO, pos = rem2 - row * TC_HALO;
			const int4 tl = tile[r];
			const int ii = wrap(tl.y + row - 1, L), jj = wrap(tl.z + pos - 1, L);
			const bf16 *g;
			if(src.mode == IN_DIRECT) g = src.a + ((size_t) (tl.x * L + ii) * L + jj) * (KC * 8) + kc * 8;
			else if(kc < 2) g = src.a + ((size_t) (tl.x * (L / 2) + ii / 2) * (L / 2) + jj / 2) * 16 + kc * 8;
			else g = src.b + ((size_t) (tl.x * L + ii) * L + jj) * 16 + (kc - 2) * 8;
			cp_async16(As + c, g, 16u);
		}
		cp_async_wait_all();
	}
	else {
		for(int c0 = threadIdx.x; c0 < nchunk; c0 += 3 * blockDim.x) {
			uint4 v[3];
#pragma unroll
			for(int u = 0; u < 3; u++) {
				const int c = c0 + u * blockDim.x;
				v[u] = make_uint4(0u, 0u, 0u, 0u);
				if(c < nchunk) {
					const int r = c / RB, rem = c - r * RB;
					const int kc = rem / (3 * TC_HALO), rem2 = rem - kc * (3 * TC_HALO);
					const int row = rem2 / TC_HALO, pos = rem2 - row * TC_HALO;
					const int4 tl = tile[r];
					v[u] = tc_load_chunk(src, KC * 8, tl.x, wrap(tl.y + row - 1, L), wrap(tl.z + pos - 1, L), L, kc);
				}
			}
#pragma unroll
			for(int u = 0; u < 3; u++) {
				const int c = c0 + u * blockDim.x;
				if(c < nchunk) As[c] = v[u];
			}
		}
	}
}

// One tensor-core layer (ci = 16 or 32 -> 16 channels, ReLU) over all
// 128-pixel tiles of `batch` samples at side L.  Tile t is pixels
// [128 t, 128 t + 128) in (sample, row, column) order.  When L is a multiple
// of 128 a tile is a row segment: its three input rows, each with the
// periodic neighbour on either side (130 positions), are staged once, and the
// nine taps are nine shifted descriptors into them (TC_RT_ROWS tiles per
// round).  Otherwise each tap's operand is gathered pixel by pixel (TC_RT
// tiles per round).  sm: TC_SMEM bytes of shared memory (mbarrier at TC_MBAR_OFF
// initialised with count 1), tmem: TC_COLS allocated columns, phase: the
// mbarrier's current parity (advanced here).  Returns false (and sets
// *err |= err_bit) if an MMA completion wait ran out; the caller then stops.
// tns (diagnostics, may be null): block 0 adds the time of weight staging,
// operand staging, MMA issue and completion, and the epilogue to tns[0..3].
static __device__ __noinline__ bool tc_conv_layer(int l, const TcSrc &src, const bf16 *wpack, const float *bias, bf16 *dst,
                                                  int batch, int L, unsigned char *sm, uint32_t tmem, uint32_t &phase, int *err,
                                                  int err_bit, unsigned long long *tns) {
	const bool timed = tns && blockIdx.x == 0 && threadIdx.x == 0;
	unsigned long long tm = 0;
	if(timed) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(tm));
	auto mark = [&](int k) {
		if(timed) {
			unsigned long long t;
			asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
			tns[k] += t - tm;
			tm = t;
		}
	};
	const UNetLayerDesc d = unet_layer(l);
	const int KC = d.ci / 8;
	const long long npix = (long long) batch * L * L;
	const long long ntiles = (npix + 127) / 128;
	uint4 *As = reinterpret_cast<uint4 *>(sm);
	uint4 *Bs = reinterpret_cast<uint4 *>(sm + TC_B_OFF);
	float *bs = reinterpret_cast<float *>(sm + TC_BIAS_OFF);
	uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + TC_MBAR_OFF);
	__syncthreads();  // the previous user of the shared buffers is done
	for(int c = threadIdx.x; c < 9 * KC * 16; c += blockDim.x) Bs[c] = reinterpret_cast<const uint4 *>(wpack)[c];
	if(threadIdx.x < 16) bs[threadIdx.x] = bias[threadIdx.x];
	const uint32_t a_base = smem_u32(As), b_base = smem_u32(Bs);
	const long long LL = (long long) L * L;
	mark(0);
	const bool rowmode = (L % 128) == 0;
	const int RT = rowmode ? TC_RT_ROWS : TC_RT;
	const int RB = KC * 3 * TC_HALO;  // row mode: 16-byte chunks per tile
	for(long long t0 = (long long) blockIdx.x * RT; t0 < ntiles; t0 += (long long) gridDim.x * RT) {
		const int nt = (int) (ntiles - t0 < RT ? ntiles - t0 : RT);
		if(rowmode) {
			int4 *tile = reinterpret_cast<int4 *>(sm + TC_TILE_OFF);
			if(threadIdx.x < (unsigned) nt) {
				const int P0 = (int) ((t0 + threadIdx.x) * 128);
				const int n = P0 / (int) LL, rr = P0 - n * (int) LL;
				tile[threadIdx.x] = make_int4(n, rr / L, rr - (rr / L) * L, 0);
			}
			__syncthreads();
			if(KC == 4) tc_stage_rows<4>(src, tile, nt, L, As);
			else tc_stage_rows<2>(src, tile, nt, L, As);
		}
		else
		// staging: thread -> (tile r, pixel p, half of the (tap, kc) chunks);
		// requires 512 threads.  Copies go straight to shared memory
		// (cp.async, all in flight); pooled inputs are averaged in registers.
		{
			const int pix = threadIdx.x & 255, half = threadIdx.x >> 8;
			const int r = pix >> 7, p = pix & 127;
			if(r < nt) {
				const long long P = (t0 + r) * 128 + p;
				const bool valid = P < npix;
				int n = 0, y = 0, x = 0;
				if(valid) {
					n = (int) P / (int) LL;
					const int rr = (int) P - n * (int) LL;
					y = rr / L;
					x = rr - y * L;
				}
				const int ys[3] = {wrap(y - 1, L), y, wrap(y + 1, L)};
				const int xs[3] = {wrap(x - 1, L), x, wrap(x + 1, L)};
				uint4 *dst_base = As + (size_t) r * 9 * KC * 128 + p;
				const int lgk = KC == 4 ? 2 : 1;
				if(src.mode != IN_POOL) {
					for(int q = half; q < 9 * KC; q += 2) {
						const int t = q >> lgk, kc = q & (KC - 1);
						const int ii = ys[t / 3], jj = xs[t % 3];
						const bf16 *g;
						if(src.mode == IN_DIRECT) g = src.a + ((size_t) (n * L + ii) * L + jj) * d.ci + kc * 8;
						else if(kc < 2) g = src.a + ((size_t) (n * (L / 2) + ii / 2) * (L / 2) + jj / 2) * 16 + kc * 8;
						else g = src.b + ((size_t) (n * L + ii) * L + jj) * 16 + (kc - 2) * 8;
						cp_async16(dst_base + (size_t) q * 128, valid ? (const void *) g : (const void *) src.a, valid ? 16u : 0u);
					}
					cp_async_wait_all();
				}
				else {
					for(int q0 = half; q0 < 9 * KC; q0 += 6) {
						uint4 v[3];
#pragma unroll
						for(int u = 0; u < 3; u++) {
							const int q = q0 + 2 * u;
							v[u] = make_uint4(0u, 0u, 0u, 0u);
							if(q < 9 * KC && valid) {
								const int t = q >> lgk, kc = q & (KC - 1);
								v[u] = tc_load_chunk(src, d.ci, n, ys[t / 3], xs[t % 3], L, kc);
							}
						}
#pragma unroll
						for(int u = 0; u < 3; u++) {
							const int q = q0 + 2 * u;
							if(q < 9 * KC) dst_base[(size_t) q * 128] = v[u];
						}
					}
				}
			}
		}
		fence_async_smem();
		__syncthreads();
		mark(1);
		if(threadIdx.x == 0) {
			tc_fence_after();
			// descriptors as base + offset: the start-address field counts 16-byte
			// units and shared addresses stay below 256 KB, so offsets (in
			// 16-byte chunks) add without carrying out of the field
			const uint64_t ad0 = rowmode ? tc_sdesc(a_base, 3 * TC_HALO * 16, 128) : tc_sdesc(a_base, 128 * 16, 128);
			const uint64_t bd0 = tc_sdesc(b_base, 16 * 16, 128);
			const int nks = KC / 2;
			// taps outer, tiles inner: consecutive MMAs go to different accumulators
#pragma unroll
			for(int t = 0; t < 9; t++) {
				for(int ks = 0; ks < nks; ks++) {
					const uint32_t boff = (uint32_t) ((t * KC + 2 * ks) * 16);
					for(int r = 0; r < nt; r++) {
						const uint32_t aoff = rowmode ? (uint32_t) (r * RB + ((2 * ks) * 3 + t / 3) * TC_HALO + t % 3)
						                              : (uint32_t) (((r * 9 + t) * KC + 2 * ks) * 128);
						tc_mma(tmem + (uint32_t) (r * 16), ad0 + aoff, bd0 + boff, TC_IDESC, (t | ks) != 0);
					}
				}
			}
			tc_commit(mbar);
		}
		bool ok = mbar_wait(mbar, phase, TC_WAIT_LIMIT);
		if(!ok) {
			if(threadIdx.x == 0) atomicOr(err, err_bit);
			ok = mbar_wait(mbar, phase, TC_WAIT_LIMIT);  // let the MMAs in flight finish before returning
			return false;
		}
		phase ^= 1u;
		tc_fence_after();
		mark(2);
		const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
		if(w < 4 * nt) {
			const int r = w >> 2, q = w & 3;
			float v[16];
			tc_ld16(tmem + ((uint32_t) (32 * q) << 16) + (uint32_t) (r * 16), v);
			const long long P = (t0 + r) * 128 + 32 * q + lane;
			if(P < npix) {
				uint4 o0, o1;
				o0.x = f2bf(fmaxf(v[0] + bs[0], 0.f), fmaxf(v[1] + bs[1], 0.f));
				o0.y = f2bf(fmaxf(v[2] + bs[2], 0.f), fmaxf(v[3] + bs[3], 0.f));
				o0.z = f2bf(fmaxf(v[4] + bs[4], 0.f), fmaxf(v[5] + bs[5], 0.f));
				o0.w = f2bf(fmaxf(v[6] + bs[6], 0.f), fmaxf(v[7] + bs[7], 0.f));
				o1.x = f2bf(fmaxf(v[8] + bs[8], 0.f), fmaxf(v[9] + bs[9], 0.f));
				o1.y = f2bf(fmaxf(v[10] + bs[10], 0.f), fmaxf(v[11] + bs[11], 0.f));
				o1.z = f2bf(fmaxf(v[12] + bs[12], 0.f), fmaxf(v[13] + bs[13], 0.f));
				o1.w = f2bf(fmaxf(v[14] + bs[14], 0.f), fmaxf(v[15] + bs[15], 0.f));
				uint4 *o = reinterpret_cast<uint4 *>(dst + P * 16);
				o[0] = o0;
				o[1] = o1;
			}
		}
		tc_fence_before();
		__syncthreads();
		mark(3);
	}
	return true;
}

// First layer (2 -> 16, ReLU) on the CUDA cores: FP32 input [R/s, W], BF16 output.
// w: FP32 [9][2][16] then 16 biases (shared memory).
static __device__ __noinline__ void e0a_range(const float *x0, const float *w, bf16 *dst, int batch, int L, long long first,
                                          long long stride) {
	const long long npix = (long long) batch * L * L;
	const float *bias = w + 9 * 2 * 16;
	const ConvSrc s{IN_DIRECT, x0, nullptr};
	for(long long p = first; p < npix; p += stride) {
		const int n = (int) (p / ((long long) L * L));
		const int r = (int) (p - (long long) n * L * L);
		const int i = r / L, j = r - (r / L) * L;
		float y[16];
		conv_pixel<2, 16>(s, w, bias, n, i, j, L, true, y);
		uint4 o0, o1;
		o0.x = f2bf(y[0], y[1]);
		o0.y = f2bf(y[2], y[3]);
		o0.z = f2bf(y[4], y[5]);
		o0.w = f2bf(y[6], y[7]);
		o1.x = f2bf(y[8], y[9]);
		o1.y = f2bf(y[10], y[11]);
		o1.z = f2bf(y[12], y[13]);
		o1.w = f2bf(y[14], y[15]);
		uint4 *o = reinterpret_cast<uint4 *>(dst + p * 16);
		o[0] = o0;
		o[1] = o1;
	}
}

// Last layer (16 -> 1, no activation) on the CUDA cores: BF16 input, FP32
// output.  w: FP32 [9][16][1] then 1 bias (shared memory).
static __device__ __noinline__ void out_range(const bf16 *t0, const float *w, float *dst, int batch, int L, long long first,
                                          long long stride) {
	const long long npix = (long long) batch * L * L;
	for(long long p = first; p < npix; p += stride) {
		const int n = (int) (p / ((long long) L * L));
		const int r = (int) (p - (long long) n * L * L);
		const int i = r / L, j = r - (r / L) * L;
		float acc = w[9 * 16];
#pragma unroll 3
		for(int t = 0; t < 9; t++) {
			const int ii = wrap(i + t / 3 - 1, L), jj = wrap(j + t % 3 - 1, L);
			const uint4 *q = reinterpret_cast<const uint4 *>(t0 + ((size_t) (n * L + ii) * L + jj) * 16);
			const uint4 u0 = q[0], u1 = q[1];
			const uint32_t u[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
			const float *wt = w + t * 16;
#pragma unroll
			for(int e = 0; e < 8; e++) {
				const float2 f = bf2f(u[e]);
				acc = fmaf(f.x, wt[2 * e], acc);
				acc = fmaf(f.y, wt[2 * e + 1], acc);
			}
		}
		dst[p] = acc;
	}
}

}  // namespace rc
