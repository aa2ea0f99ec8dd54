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

// Input of a tensor-core layer: BF16 activations (IN_DIRECT, IN_POOL,
// IN_UPCAT as for the FP32 layers), or IN_FIRST: the first layer (2 -> 16,
// ReLU) evaluated while staging, from the FP32 network input x (channel 0
// multiplied by sc[sample]) with the FP32 weights w0 ([9][2][16] + 16 biases).
enum { IN_FIRST = 3 };
struct TcSrc {
	int mode;
	const bf16 *a;
	const bf16 *b;
	const float *x = nullptr;
	const float *w0 = nullptr;
	float sc[2] = {1.f, 1.f};
};

// First layer (2 -> 16, ReLU) at one pixel of sample n, FP32: channel 0 of
// the input (R) is multiplied by sc (1/s of the component) as it is read.
// w: [9][2][16] then 16 biases.
__device__ __forceinline__ void e0a_pixel(const float *x0, const float *w, int n, int i, int j, int L, float sc, float *y) {
#pragma unroll
	for(int o = 0; o < 16; o++) y[o] = w[9 * 2 * 16 + o];
#pragma unroll
	for(int t = 0; t < 9; t++) {
		const int ii = wrap(i + t / 3 - 1, L), jj = wrap(j + t % 3 - 1, L);
		const float2 in = *reinterpret_cast<const float2 *>(x0 + ((size_t) (n * L + ii) * L + jj) * 2);
		const float r = in.x * sc, wv = in.y;
		const float *wt = w + t * 32;
#pragma unroll
		for(int o = 0; o < 16; o++) y[o] = fmaf(r, wt[o], y[o]);
#pragma unroll
		for(int o = 0; o < 16; o++) y[o] = fmaf(wv, wt[16 + o], y[o]);
	}
#pragma unroll
	for(int o = 0; o < 16; o++) y[o] = fmaxf(y[o], 0.f);
}


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

// Shared memory and TMEM of the tensor-core layers.
//
// Strip mode (level side a multiple of 128): a CTA streams the rows of a
// column strip of T tiles of 128 pixels.  Each staged input row rho (its
// W = 128 T pixels plus the periodic neighbour on either side, channel
// chunks of 8 in planes [kc][position]) is consumed by 3 x KS MMAs per tile,
// one per horizontal tap dx (the A descriptor shifted by dx) and channel
// pair: A = 128 pixels x 16 channels, B = the three vertical taps' weights
// stacked along N (N = 48: dy = +1, 0, -1), D = the accumulators of output
// rows rho - 1, rho, rho + 1, which sit in consecutive 16-column slots of a
// ring of R = 32 / T - 2 slots per tile in TMEM; the ring is followed by two
// overflow slots, so the three slots of an MMA are always contiguous (what
// lands in slot R or R + 1 belongs to logical slot 0 or 1 and is added by
// the epilogue).  An output row is complete once
// input row + 1 has been multiplied; the epilogue reads it, writes BF16
// (bias, ReLU) and zeroes the slot for reuse.  Rows are pipelined: the MMAs
// of input row i run while output row i - 3 is written out and input row
// i + 1 is staged.  An MMA is costed by the tensor core at about the same
// time whatever N is (16 to 256), so stacking the vertical taps along N cuts
// the instruction count threefold against one MMA per tap.
//
// Gather mode (other sides, small levels only): each tap's operand is
// gathered pixel by pixel for one tile of 128 pixels (K-major A), nine taps
// times KC/2 MMAs of N = 16 into one accumulator.
constexpr int TC_STRIP_T = 4;   // strip mode: at most 4 tiles (512 pixels) per strip
constexpr int TC_COLS = 512;    // TMEM columns: T x R slots of 16
constexpr int TC_HW_MAX = TC_STRIP_T * 128 + 2;
constexpr size_t TC_A_GATHER = (size_t) 9 * 4 * 128 * 16;  // gather mode: one tile's operands
constexpr size_t TC_A_STRIP = (size_t) 3 * 4 * TC_HW_MAX * 16;  // three input-row buffers, up to 4 channel chunks
constexpr size_t TC_A_BYTES = TC_A_GATHER > TC_A_STRIP ? TC_A_GATHER : TC_A_STRIP;
constexpr size_t TC_B_OFF = TC_A_BYTES;
constexpr size_t TC_B_BYTES = 9 * 4 * 16 * 16;  // either layout: 9 taps x 32 channels x 16 outputs, BF16
constexpr size_t TC_BIAS_OFF = TC_B_OFF + TC_B_BYTES;
constexpr size_t TC_W0_OFF = TC_BIAS_OFF + 64;  // first layer's FP32 weights (IN_FIRST)
constexpr int TC_NMBAR = 6;  // [0] gather mode, [1] spare, [2..5] strip mode's MMA completions
constexpr size_t TC_MBAR_OFF = TC_W0_OFF + sizeof(float) * (9 * 2 * 16 + 16);
constexpr size_t TC_CTRL_OFF = TC_MBAR_OFF + 8 * TC_NMBAR;  // strip mode: rows staged, rows written, abort, MMAs issued
constexpr size_t TC_HOLD_OFF = TC_CTRL_OFF + 16;
constexpr size_t TC_SMEM = TC_HOLD_OFF + 16;
constexpr uint32_t TC_IDESC = tc_idesc_bf16(128, 16);
constexpr uint32_t TC_IDESC48 = tc_idesc_bf16(128, 48);
constexpr long long TC_WAIT_LIMIT = 2000000;  // mbarrier polls (each a bounded hardware wait)

// Per-CTA state of the tensor-core layers: shared memory (TC_SMEM bytes,
// the TC_NMBAR mbarriers at TC_MBAR_OFF initialised with count 1), the TMEM
// allocation (TC_COLS columns) and the parities the mbarriers wait for next.
// err/err_bit: where a wait that ran out is recorded.  tns (diagnostics, may
// be null): block 0 adds times to tns[0..3] -- in gather mode weight
// staging, operand staging, MMA completion waits and the epilogue; in strip
// mode, as seen by the first write-out thread, weight staging, band set-up,
// waits for MMA completion and the write-out work.
struct TcCtx {
	unsigned char *sm;
	uint32_t tmem;
	uint32_t phase[2];
	int *err;
	int err_bit;
	unsigned long long *tns;
	unsigned long long mma_rows = 0;  // strip mode: input rows multiplied so far (indexes the MMA mbarriers)
};

// Shared-memory flags between the roles of the strip pipeline.
__device__ __forceinline__ int ld_acquire_s32(const int *p) {
	int v;
	asm volatile("ld.acquire.cta.shared::cta.b32 %0, [%1];" : "=r"(v) : "r"(smem_u32(p)) : "memory");
	return v;
}
__device__ __forceinline__ void st_release_s32(int *p, int v) {
	asm volatile("st.release.cta.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(p)), "r"(v) : "memory");
}
// Barrier among `n` threads (a multiple of 32) under id (1 - 15).
__device__ __forceinline__ void bar_named(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
// The same, returning whether any participant passed v = true.
__device__ __forceinline__ bool bar_named_or(int id, int n, bool v) {
	uint32_t r;
	asm volatile(
	    "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, %2, %3, p;\n\tselp.u32 %0, 1, 0, q;\n\t}"
	    : "=r"(r)
	    : "r"((uint32_t) v), "r"(id), "r"(n)
	    : "memory");
	return r != 0;
}
// Bounded wait for an mbarrier phase that also gives up once *abort is set.
__device__ __forceinline__ bool mbar_wait_abort(uint64_t *mbar, uint32_t parity, const volatile int *abort, long long limit) {
	for(long long i = 0; i < limit; i++) {
		if(mbar_try_wait(mbar, parity)) return true;
		if((i & 31) == 31 && *abort) return false;
	}
	return false;
}

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

// Source of input chunk kc of pixel (n, i, j) for a plain copy (direct and
// up-sampled/concatenated inputs).
__device__ __forceinline__ const bf16 *tc_chunk_ptr(const TcSrc &s, int ci, int n, int i, int j, int L, int kc) {
	if(s.mode == IN_DIRECT) return s.a + ((size_t) (n * L + i) * L + j) * ci + kc * 8;
	if(kc < 2) return s.a + ((size_t) (n * (L / 2) + i / 2) * (L / 2) + j / 2) * 16 + kc * 8;
	return s.b + ((size_t) (n * L + i) * L + j) * 16 + (kc - 2) * 8;
}

// Stage input row `row` of sample n, pixels x0 - 1 .. x0 + W (periodic), into
// buf[kc * HW + position] (HW = W + 2).  Consecutive threads take
// consecutive 16-byte chunks of global memory (kc fastest).  Plain inputs go
// by cp.async (the caller waits); pooled inputs are averaged in registers;
// IN_FIRST rows are computed from the network input (w0s: the first layer's
// weights in shared memory).
__device__ __forceinline__ void tc_stage_strip_row(const TcSrc &src, int KC, int n, int row, int x0, int HW, int L, uint4 *buf,
                                                   const float *w0s, int t0, int nthr) {
	const int nchunk = KC * HW;
	if(src.mode == IN_FIRST) {
		for(int pos = t0; pos < HW; pos += nthr) {
			float y[16];
			e0a_pixel(src.x, w0s, n, row, wrap(x0 - 1 + pos, L), L, src.sc[n], y);
			buf[pos] = make_uint4(f2bf(y[0], y[1]), f2bf(y[2], y[3]), f2bf(y[4], y[5]), f2bf(y[6], y[7]));
			buf[HW + pos] = make_uint4(f2bf(y[8], y[9]), f2bf(y[10], y[11]), f2bf(y[12], y[13]), f2bf(y[14], y[15]));
		}
	}
	else if(src.mode != IN_POOL) {
		for(int c = t0; c < nchunk; c += nthr) {
			const int pos = c / KC, kc = c - pos * KC;
			const int x = wrap(x0 - 1 + pos, L);
			cp_async16(buf + kc * HW + pos, tc_chunk_ptr(src, KC * 8, n, row, x, L, kc), 16u);
		}
	}
	else {
		for(int c = t0; c < nchunk; c += nthr) {
			const int pos = c / KC, kc = c - pos * KC;
			buf[kc * HW + pos] = tc_load_chunk(src, KC * 8, n, row, wrap(x0 - 1 + pos, L), L, kc);
		}
	}
}

// 16 consecutive TMEM columns of this thread's lane set to zero.
__device__ __forceinline__ void tc_st16_zero(uint32_t taddr) {
	const uint32_t z = 0u;
	asm volatile(
	    "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1};" ::"r"(
	        taddr),
	    "r"(z)
	    : "memory");
}
__device__ __forceinline__ void tc_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// Bias, ReLU and BF16 conversion of one pixel's 16 accumulators; 32-byte store.
__device__ __forceinline__ void tc_store_pixel(const float (&v)[16], const float *bs, bf16 *dst, long long P) {
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

struct TcTimer {
	bool on;
	unsigned long long t;
	unsigned long long *tns;
	__device__ __forceinline__ TcTimer(unsigned long long *p, unsigned who = 0)
	    : on(p && blockIdx.x == 0 && threadIdx.x == who), t(0), tns(p) {
		if(on) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	}
	__device__ __forceinline__ void mark(int k) {
		if(on) {
			unsigned long long u;
			asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(u));
			tns[k] += u - t;
			t = u;
		}
	}
};


// Strip mode (L a multiple of 128); requires 512 threads in three roles that
// run decoupled: warp 0 issues the MMAs, warps 1 - 7 stage input rows into a
// ring of three buffers, warps 8 - 15 write finished output rows out of TMEM.
// Rows pass between the roles through release/acquire counters in shared
// memory (rows staged, rows written out) and the MMA completion mbarriers;
// every wait is bounded and gives up when any role has set the abort flag,
// and the roles' own barriers are reached by all of their threads or none.  wl: the layer's
// FP32 weights [tap = (dy + 1) * 3 + dx + 1][ci][16]; bias: 16 FP32.
static __device__ __noinline__ bool tc_conv_strip(int l, const TcSrc &src, const float *wl, const float *bias, bf16 *dst,
                                                  int batch, int L, TcCtx &c) {
	TcTimer tm(c.tns, 256);  // block 0's first write-out thread
	const UNetLayerDesc d = unet_layer(l);
	const int KC = d.ci / 8, KS = KC / 2;
	const int ntile = L / 128;
	int T = TC_STRIP_T;
	while(ntile % T) T >>= 1;
	const int R = TC_COLS / 16 / T - 2;  // output-row slots per tile, plus two overflow slots
	const int W = T * 128, HW = W + 2;
	const int NS = ntile / T;
	const long long U = (long long) batch * NS * L;  // (sample, strip, row) units
	uint4 *Abuf = reinterpret_cast<uint4 *>(c.sm);
	bf16 *Bh = reinterpret_cast<bf16 *>(c.sm + TC_B_OFF);
	float *bs = reinterpret_cast<float *>(c.sm + TC_BIAS_OFF);
	uint64_t *mbar = reinterpret_cast<uint64_t *>(c.sm + TC_MBAR_OFF);
	__syncthreads();  // the previous user of the shared buffers is done
	// B of (dx, channel pair ks): rows n = 16 j + co hold the weights of
	// dy = 1 - j; K-major core matrices, LBO 768 B (K halves), SBO 128 B
	const int nB = 3 * KS * 2 * 48 * 8;
	for(int idx = threadIdx.x; idx < nB; idx += blockDim.x) {
		const int e = idx & 7, rest = idx >> 3;
		const int n = rest % 48, hq = rest / 48;
		const int h = hq & 1, q = hq >> 1;
		const int ks = q % KS, dxi = q / KS;
		const int j = n >> 4, co = n & 15;
		const int t = (2 - j) * 3 + dxi;
		Bh[idx] = __float2bfloat16_rn(wl[(t * d.ci + 16 * ks + 8 * h + e) * 16 + co]);
	}
	if(threadIdx.x < 16) bs[threadIdx.x] = bias[threadIdx.x];
	float *w0s = reinterpret_cast<float *>(c.sm + TC_W0_OFF);
	if(src.mode == IN_FIRST)
		for(int k = threadIdx.x; k < 9 * 2 * 16 + 16; k += blockDim.x) w0s[k] = src.w0[k];
	if(threadIdx.x == 0) reinterpret_cast<int *>(c.sm + TC_CTRL_OFF)[2] = 0;
	fence_async_smem();
	__syncthreads();
	tm.mark(0);
	const uint32_t a_base = smem_u32(Abuf), b_base = smem_u32(Bh);
	const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
	int *ctrl = reinterpret_cast<int *>(c.sm + TC_CTRL_OFF);  // [0] rows staged, [1] rows written, [2] abort, [3] MMAs issued
	const volatile int *abort = ctrl + 2;
	uint64_t *acc = mbar + 2;  // MMA completion of input row g on acc[g & 3], phase (g >> 2) & 1
	const long long per = (U + gridDim.x - 1) / gridDim.x;
	const long long u0 = blockIdx.x * per, u1 = u0 + per < U ? u0 + per : U;
	for(long long u = u0; u < u1;) {
		const long long col = u / L;
		const int y0 = (int) (u - col * L);
		const int y1 = (int) ((u1 - col * L) < L ? (u1 - col * L) : L);  // exclusive
		const int n = (int) (col / NS), x0 = (int) (col - (long long) n * NS) * W;
		const int nin = y1 - y0 + 2;  // input rows y0 - 1 .. y1; output rows y0 - 2 .. y1 - 1
		// all slots zero (by the warps that will write them out), counters reset
		if(w >= 8)
			for(int r = (w - 8) >> 2; r < T; r += 2)
				for(int sl = 0; sl < R + 2; sl++)
					tc_st16_zero(c.tmem + ((uint32_t) (32 * (w & 3)) << 16) + (uint32_t) ((r * (R + 2) + sl) * 16));
		tc_wait_st();
		if(threadIdx.x == 0) {
			ctrl[0] = 0;
			ctrl[1] = 0;
			ctrl[3] = 0;
		}
		tc_fence_before();
		__syncthreads();
		tc_fence_after();
		tm.mark(1);
		const unsigned long long G = c.mma_rows;
		if(w == 0) {
			// MMA warp: input row i (buffer i % 3) once it is staged and output
			// row i - 4 has been written out (its slot is reused and the MMA
			// mbarriers stay at most one phase ahead of their waiters)
			if(lane == 0) {
				TcTimer tmm(c.tns, 0);  // block 0's MMA thread: [4] waits for staged rows and free slots, [5] issue
				for(int i = 0; i < nin; i++) {
					bool ok = false;
					for(long long t = 0; t < TC_WAIT_LIMIT; t++) {
						if(ld_acquire_s32(&ctrl[0]) >= i + 1 && ld_acquire_s32(&ctrl[1]) >= i - 3) {
							ok = true;
							break;
						}
						if(*abort) break;
					}
					tmm.mark(4);
					if(!ok) {
						ctrl[2] = 1;
						break;
					}
					tc_fence_after();
					fence_async_smem();
					const uint32_t abuf = a_base + (uint32_t) ((i % 3) * KC * HW * 16);
					const int s0 = i % R;
					for(int r = 0; r < T; r++) {
						const uint32_t dcol = c.tmem + (uint32_t) ((r * (R + 2) + s0) * 16);
						for(int dxi = 0; dxi < 3; dxi++) {
							for(int ks = 0; ks < KS; ks++) {
								const uint64_t ad =
								    tc_sdesc(abuf + (uint32_t) (((2 * ks) * HW + r * 128 + dxi) * 16), (uint32_t) (HW * 16), 128);
								const uint32_t bq = b_base + (uint32_t) ((dxi * KS + ks) * 1536);
								tc_mma(dcol, ad, tc_sdesc(bq, 768, 128), TC_IDESC48, 1u);
							}
						}
					}
					tc_commit(&acc[(G + i) & 3]);
					ctrl[3] = i + 1;
					tmm.mark(5);
				}
			}
			__syncwarp();
		}
		else if(w < 8) {
			// staging warps: row r into buffer r % 3 once the MMAs of row r - 3
			// (the buffer's previous row) are done
			const int pt = threadIdx.x - 32, np = 224;
			TcTimer tst(c.tns, 32);  // block 0's first staging thread: [6] waits for buffer reuse, [7] loading
			for(int r = 0; r < nin; r++) {
				bool ok = true;
				if(r >= 3 && pt == 0) {
					const unsigned long long g = G + r - 3;
					ok = mbar_wait_abort(&acc[g & 3], (uint32_t) ((g >> 2) & 1), abort, TC_WAIT_LIMIT);
					if(!ok) ctrl[2] = 1;
				}
				if(bar_named_or(1, np, !ok || *abort != 0)) break;
				tst.mark(6);
				tc_stage_strip_row(src, KC, n, wrap(y0 - 1 + r, L), x0, HW, L, Abuf + (r % 3) * KC * HW, w0s, pt, np);
				cp_async_wait_all();
				fence_async_smem();
				bar_named(1, np);
				if(pt == 0) st_release_s32(&ctrl[0], r + 1);
				tst.mark(7);
			}
		}
		else {
			// write-out warps: output row y0 - 2 + m once the MMAs of input row
			// m are done (bias, ReLU, BF16; rows above the band only cleared)
			const int et = threadIdx.x - 256;
			for(int m = 0; m < nin; m++) {
				const unsigned long long g = G + m;
				const bool ok = mbar_wait_abort(&acc[g & 3], (uint32_t) ((g >> 2) & 1), abort, TC_WAIT_LIMIT);
				if(!ok) ctrl[2] = 1;
				if(bar_named_or(2, 256, !ok || *abort != 0)) break;
				tc_fence_after();
				tm.mark(2);
				const int y = y0 - 2 + m, sl = m % R;
				for(int r = (w - 8) >> 2; r < T; r += 2) {
					const uint32_t ta = c.tmem + ((uint32_t) (32 * (w & 3)) << 16) + (uint32_t) ((r * (R + 2) + sl) * 16);
					if(y >= y0) {
						float v[16];
						tc_ld16(ta, v);
						if(sl < 2) {
							float o[16];
							tc_ld16(ta + (uint32_t) (R * 16), o);
#pragma unroll
							for(int k = 0; k < 16; k++) v[k] += o[k];
						}
						tc_store_pixel(v, bs, dst, ((long long) n * L + y) * L + x0 + r * 128 + 32 * (w & 3) + lane);
					}
					tc_st16_zero(ta);
					if(sl < 2) tc_st16_zero(ta + (uint32_t) (R * 16));
				}
				tc_wait_st();
				tc_fence_before();
				bar_named(2, 256);
				if(et == 0) st_release_s32(&ctrl[1], m + 1);
				tm.mark(3);
			}
		}
		__syncthreads();
		if(ctrl[2]) {
			// let the MMAs in flight finish before giving up
			if(threadIdx.x == 0) {
				atomicOr(c.err, c.err_bit);
				const int issued = ctrl[3];
				if(issued > 0) {
					const unsigned long long g = G + issued - 1;
					mbar_wait(&acc[g & 3], (uint32_t) ((g >> 2) & 1), TC_WAIT_LIMIT);
				}
			}
			cp_async_wait_all();
			__syncthreads();
			return false;
		}
		c.mma_rows += nin;
		u += y1 - y0;
	}
	return true;
}

// Gather mode: one tile of 128 pixels per round, operands gathered pixel by
// pixel; wpack: the layer's packed BF16 weights [tap][kc][co][8].  Inputs
// IN_DIRECT, IN_POOL and IN_UPCAT (not IN_FIRST).
static __device__ __noinline__ bool tc_conv_gather(int l, const TcSrc &src, const bf16 *wpack, const float *bias, bf16 *dst,
                                                   int batch, int L, TcCtx &c) {
	TcTimer tm(c.tns);
	const UNetLayerDesc d = unet_layer(l);
	const int KC = d.ci / 8;
	const long long npix = (long long) batch * L * L;
	const long long ntiles = (npix + 127) / 128;
	uint4 *As = reinterpret_cast<uint4 *>(c.sm);
	uint4 *Bs = reinterpret_cast<uint4 *>(c.sm + TC_B_OFF);
	float *bs = reinterpret_cast<float *>(c.sm + TC_BIAS_OFF);
	uint64_t *mbar = reinterpret_cast<uint64_t *>(c.sm + TC_MBAR_OFF);
	__syncthreads();
	for(int k = threadIdx.x; k < 9 * KC * 16; k += blockDim.x) Bs[k] = reinterpret_cast<const uint4 *>(wpack)[k];
	if(threadIdx.x < 16) bs[threadIdx.x] = bias[threadIdx.x];
	const uint32_t a_base = smem_u32(As), b_base = smem_u32(Bs);
	const long long LL = (long long) L * L;
	tm.mark(0);
	const int lgk = KC == 4 ? 2 : 1;
	for(long long t0 = blockIdx.x; t0 < ntiles; t0 += gridDim.x) {
		// thread -> (pixel p, half of the (tap, kc) chunks)
		{
			const int p = threadIdx.x & 127, part = threadIdx.x >> 7;
			const long long P = t0 * 128 + p;
			const bool valid = P < npix;
			int n = 0, y = 0, x = 0;
			if(valid) {
				n = (int) (P / LL);
				const int rr = (int) (P - n * LL);
				y = rr / L;
				x = rr - y * L;
			}
			const int ys[3] = {wrap(y - 1, L), y, wrap(y + 1, L)};
			const int xs[3] = {wrap(x - 1, L), x, wrap(x + 1, L)};
			uint4 *dst_base = As + p;
			for(int q = part; q < 9 * KC; q += 4) {
				const int t = q >> lgk, kc = q & (KC - 1);
				if(src.mode != IN_POOL) {
					const bf16 *g = valid ? tc_chunk_ptr(src, d.ci, n, ys[t / 3], xs[t % 3], L, kc) : src.a;
					cp_async16(dst_base + (size_t) q * 128, g, valid ? 16u : 0u);
				}
				else dst_base[(size_t) q * 128] = valid ? tc_load_chunk(src, d.ci, n, ys[t / 3], xs[t % 3], L, kc) : make_uint4(0u, 0u, 0u, 0u);
			}
			cp_async_wait_all();
		}
		fence_async_smem();
		__syncthreads();
		tm.mark(1);
		if(threadIdx.x == 0) {
			tc_fence_after();
			const uint64_t ad0 = tc_sdesc(a_base, 128 * 16, 128);
			const uint64_t bd0 = tc_sdesc(b_base, 16 * 16, 128);
			const int nks = KC / 2;
#pragma unroll
			for(int t = 0; t < 9; t++) {
				for(int ks = 0; ks < nks; ks++) {
					const uint32_t boff = (uint32_t) ((t * KC + 2 * ks) * 16);
					const uint32_t aoff = (uint32_t) ((t * KC + 2 * ks) * 128);
					tc_mma(c.tmem, ad0 + aoff, bd0 + boff, TC_IDESC, (t | ks) != 0);
				}
			}
			tc_commit(&mbar[0]);
		}
		const bool ok = mbar_wait(&mbar[0], c.phase[0], TC_WAIT_LIMIT);
		c.phase[0] ^= 1u;
		tc_fence_after();
		if(__syncthreads_or(!ok)) {
			if(threadIdx.x == 0) atomicOr(c.err, c.err_bit);
			return false;
		}
		tm.mark(2);
		const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
		if(w < 4) {
			float v[16];
			tc_ld16(c.tmem + ((uint32_t) (32 * w) << 16), v);
			const long long P = t0 * 128 + 32 * w + lane;
			if(P < npix) tc_store_pixel(v, bs, dst, P);
		}
		tc_fence_before();
		__syncthreads();
		tm.mark(3);
	}
	return true;
}

// One tensor-core layer (ci = 16 or 32 -> 16 channels, ReLU) over `batch`
// samples at side L.  Returns false (and sets *c.err |= c.err_bit) if an MMA
// completion wait ran out; the caller then stops.
__device__ __forceinline__ bool tc_conv_layer(int l, const TcSrc &src, const bf16 *wpack, const float *wl, const float *bias,
                                              bf16 *dst, int batch, int L, TcCtx &c) {
	if(L % 128 == 0) return tc_conv_strip(l, src, wl, bias, dst, batch, L, c);
	return tc_conv_gather(l, src, wpack, bias, dst, batch, L, c);
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
// output.  w: FP32 [9][16][1] then 1 bias (shared memory).  A work item is
// one column j of OUT_ROWS consecutive output rows of one sample; its input
// rows are loaded once each (three pixels, j - 1 .. j + 1) and folded at
// once into the outputs they feed: row r adds its dy = -1 taps to output
// r + 1, its dy = 0 taps to r, its dy = +1 taps to r - 1.  Every output thus
// receives its taps in the order dy, dx, channel, as a per-pixel loop would,
// with (OUT_ROWS + 2) * 3 / OUT_ROWS pixel loads per output instead of nine;
// consecutive threads take consecutive columns (coalesced).  L must be a
// multiple of OUT_ROWS (the learned solver requires L % 4 == 0).
constexpr int OUT_ROWS = 4;
static __device__ __noinline__ void out_range(const bf16 *t0, const float *w, float *dst, int batch, int L, long long first,
                                          long long stride) {
	const int nrb = L / OUT_ROWS;
	const long long nitems = (long long) batch * nrb * L;
	for(long long it = first; it < nitems; it += stride) {
		const int j = (int) (it % L);
		const long long rest = it / L;
		const int rb = (int) (rest % nrb), n = (int) (rest / nrb);
		const int i0 = rb * OUT_ROWS;
		const int cols[3] = {wrap(j - 1, L), j, wrap(j + 1, L)};
		float acc[OUT_ROWS];
#pragma unroll
		for(int o = 0; o < OUT_ROWS; o++) acc[o] = w[9 * 16];
#pragma unroll
		for(int r = -1; r <= OUT_ROWS; r++) {
			uint4 px[3][2];
			const uint4 *row = reinterpret_cast<const uint4 *>(t0 + (size_t) (n * L + wrap(i0 + r, L)) * L * 16);
#pragma unroll
			for(int d = 0; d < 3; d++) {
				px[d][0] = row[cols[d] * 2];
				px[d][1] = row[cols[d] * 2 + 1];
			}
			// tap rows ty = 0, 1, 2 (dy = ty - 1) feed output row r - ty + 1
#pragma unroll
			for(int ty = 0; ty < 3; ty++) {
				const int o = r - ty + 1;
				if(o < 0 || o >= OUT_ROWS) continue;
#pragma unroll
				for(int d = 0; d < 3; d++) {
					const uint32_t u[8] = {px[d][0].x, px[d][0].y, px[d][0].z, px[d][0].w,
					                       px[d][1].x, px[d][1].y, px[d][1].z, px[d][1].w};
					const float *wt = w + (ty * 3 + d) * 16;
#pragma unroll
					for(int e = 0; e < 8; e++) {
						const float2 f = bf2f(u[e]);
						acc[o] = fmaf(f.x, wt[2 * e], acc[o]);
						acc[o] = fmaf(f.y, wt[2 * e + 1], acc[o]);
					}
				}
			}
			if(r >= 1) dst[((size_t) n * L + i0 + r - 1) * L + j] = acc[r - 1];
			// one input row in registers at a time: keep the next row's loads
			// from being hoisted above this row's arithmetic
			asm volatile("" ::: "memory");
		}
	}
}

}  // namespace rc
