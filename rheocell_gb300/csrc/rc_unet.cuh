// The learned preconditioner's network: a 3-level U-Net on the periodic box
// grid (channel-last float arrays, [sample][y][x][channel]).  The layer
// table, the parameter layout and the FP32 convolution used both by the
// training kernels (rc_unet.cu) and by the preconditioned solve (rc_cg.cu).
//
//   e0a 2->16, e0b 16->16 = s0            (L)    input [R/s, W]
//   e1a 16->16, e1b 16->16 = s1           (L/2)  input avgpool2(s0)
//   b0 16->16, b1 16->16 = t2             (L/4)  input avgpool2(s1)
//   d1a 32->16, d1b 16->16 = t1           (L/2)  input [upsample2(t2), s1]
//   d0a 32->16, d0b 16->16 = t0           (L)    input [upsample2(t1), s0]
//   out 16->1                             (L)    no activation
//
// Every layer is a 3x3 convolution with periodic wrap plus a bias, then ReLU
// (except `out`).  Weights w[tap][ci][co], tap = (dy + 1) * 3 + (dx + 1),
// y(i, j) += x((i + dy) mod L, (j + dx) mod L) * w[tap].
#pragma once

#include <cuda_runtime.h>

namespace rc {

constexpr int UNET_LAYERS = 11;
constexpr int UNET_C = 16;

enum { L_E0A, L_E0B, L_E1A, L_E1B, L_B0, L_B1, L_D1A, L_D1B, L_D0A, L_D0B, L_OUT };

// input modes of a convolution
enum { IN_DIRECT = 0, IN_POOL = 1, IN_UPCAT = 2 };

struct UNetLayerDesc {
	int ci, co, relu, level, mode;
};

__host__ __device__ constexpr UNetLayerDesc unet_layer(int l) {
	return l == L_E0A   ? UNetLayerDesc{2, 16, 1, 0, IN_DIRECT}
	       : l == L_E0B ? UNetLayerDesc{16, 16, 1, 0, IN_DIRECT}
	       : l == L_E1A ? UNetLayerDesc{16, 16, 1, 1, IN_POOL}
	       : l == L_E1B ? UNetLayerDesc{16, 16, 1, 1, IN_DIRECT}
	       : l == L_B0  ? UNetLayerDesc{16, 16, 1, 2, IN_POOL}
	       : l == L_B1  ? UNetLayerDesc{16, 16, 1, 2, IN_DIRECT}
	       : l == L_D1A ? UNetLayerDesc{32, 16, 1, 1, IN_UPCAT}
	       : l == L_D1B ? UNetLayerDesc{16, 16, 1, 1, IN_DIRECT}
	       : l == L_D0A ? UNetLayerDesc{32, 16, 1, 0, IN_UPCAT}
	       : l == L_D0B ? UNetLayerDesc{16, 16, 1, 0, IN_DIRECT}
	                    : UNetLayerDesc{16, 1, 0, 0, IN_DIRECT};
}

// offsets in the flat parameter vector: per layer 9*ci*co weights, then co biases
__host__ __device__ constexpr int unet_weight_offset(int l) {
	int off = 0;
	for(int k = 0; k < l; k++) off += 9 * unet_layer(k).ci * unet_layer(k).co + unet_layer(k).co;
	return off;
}
__host__ __device__ constexpr int unet_bias_offset(int l) {
	return unet_weight_offset(l) + 9 * unet_layer(l).ci * unet_layer(l).co;
}
constexpr int UNET_PARAMS = unet_weight_offset(UNET_LAYERS);
static_assert(UNET_PARAMS == 25937, "parameter count of the network");

// largest 9*ci*co + co of any layer (d1a/d0a: 9*32*16 + 16)
constexpr int UNET_MAX_LAYER_PARAMS = 9 * 32 * 16 + 16;

// Source of a convolution's input at level side L:
//   IN_DIRECT: a[(n, i, j)][0..ci)          (side L, ci channels)
//   IN_POOL:   mean of a over the 2x2 block  (a at side 2L, ci channels)
//   IN_UPCAT:  channels 0..15 from a[(n, i/2, j/2)] (side L/2, 16 channels),
//              16..31 from b[(n, i, j)] (side L, 16 channels)
struct ConvSrc {
	int mode;
	const float *a;
	const float *b;
};

__device__ __forceinline__ int wrap(int v, int L) { return v < 0 ? v + L : (v >= L ? v - L : v); }

template<int CI>
__device__ __forceinline__ void load_input(const ConvSrc &s, int n, int i, int j, int L, float (&x)[CI]) {
	if(s.mode == IN_DIRECT) {
		const float *p = s.a + ((size_t) (n * L + i) * L + j) * CI;
		if constexpr(CI % 4 == 0) {
#pragma unroll
			for(int c = 0; c < CI; c += 4) {
				const float4 v = *reinterpret_cast<const float4 *>(p + c);
				x[c] = v.x;
				x[c + 1] = v.y;
				x[c + 2] = v.z;
				x[c + 3] = v.w;
			}
		}
		else {
#pragma unroll
			for(int c = 0; c < CI; c++) x[c] = p[c];
		}
	}
	else if constexpr(CI % 4 != 0) {
		// only the first layer has CI % 4 != 0, and it reads directly
	}
	else if(s.mode == IN_POOL) {
		const int L2 = 2 * L;
#pragma unroll
		for(int c = 0; c < CI; c++) x[c] = 0.f;
#pragma unroll
		for(int q = 0; q < 4; q++) {
			const float *p = s.a + ((size_t) (n * L2 + 2 * i + (q >> 1)) * L2 + 2 * j + (q & 1)) * CI;
#pragma unroll
			for(int c = 0; c < CI; c += 4) {
				const float4 v = *reinterpret_cast<const float4 *>(p + c);
				x[c] += v.x;
				x[c + 1] += v.y;
				x[c + 2] += v.z;
				x[c + 3] += v.w;
			}
		}
#pragma unroll
		for(int c = 0; c < CI; c++) x[c] *= 0.25f;
	}
	else if constexpr(CI >= 16) {
		const int Lh = L / 2;
		const float *p = s.a + ((size_t) (n * Lh + i / 2) * Lh + j / 2) * 16;
		const float *q = s.b + ((size_t) (n * L + i) * L + j) * 16;
#pragma unroll
		for(int c = 0; c < 16; c += 4) {
			const float4 v = *reinterpret_cast<const float4 *>(p + c);
			const float4 u = *reinterpret_cast<const float4 *>(q + c);
			x[c] = v.x;
			x[c + 1] = v.y;
			x[c + 2] = v.z;
			x[c + 3] = v.w;
			if constexpr(CI == 32) {
				x[16 + c] = u.x;
				x[17 + c] = u.y;
				x[18 + c] = u.z;
				x[19 + c] = u.w;
			}
		}
	}
}

// Channel c of a convolution's input at (n, i, j), side L (ci channels).
__device__ __forceinline__ float input_scalar(const ConvSrc &s, int ci, int n, int i, int j, int L, int c) {
	if(s.mode == IN_DIRECT) return s.a[((size_t) (n * L + i) * L + j) * ci + c];
	if(s.mode == IN_POOL) {
		const int L2 = 2 * L;
		const float *p = s.a + ((size_t) (n * L2 + 2 * i) * L2 + 2 * j) * ci + c;
		return 0.25f * (((p[0] + p[ci]) + p[(size_t) L2 * ci]) + p[(size_t) L2 * ci + ci]);
	}
	if(c < 16) {
		const int Lh = L / 2;
		return s.a[((size_t) (n * Lh + i / 2) * Lh + j / 2) * 16 + c];
	}
	return s.b[((size_t) (n * L + i) * L + j) * 16 + (c - 16)];
}

// One output pixel of a layer: y[0..CO) = bias + sum over taps and inputs.
// w: [9][CI][CO], bias: [CO] (shared memory).
template<int CI, int CO>
__device__ __forceinline__ void conv_pixel(const ConvSrc &s, const float *w, const float *bias, int n, int i, int j,
                                           int L, bool relu, float *out) {
	float acc[CO];
#pragma unroll
	for(int o = 0; o < CO; o++) acc[o] = bias[o];
#pragma unroll(CI <= 2 ? 9 : 1)
	for(int t = 0; t < 9; t++) {
		const int ii = wrap(i + t / 3 - 1, L), jj = wrap(j + t % 3 - 1, L);
		float x[CI];
		load_input<CI>(s, n, ii, jj, L, x);
		const float *wt = w + t * CI * CO;
#pragma unroll
		for(int c = 0; c < CI; c++) {
#pragma unroll
			for(int o = 0; o < CO; o++) acc[o] = fmaf(x[c], wt[c * CO + o], acc[o]);
		}
	}
	if constexpr(CO % 4 == 0) {
#pragma unroll
		for(int o = 0; o < CO; o += 4) {
			float4 v;
			v.x = relu ? fmaxf(acc[o], 0.f) : acc[o];
			v.y = relu ? fmaxf(acc[o + 1], 0.f) : acc[o + 1];
			v.z = relu ? fmaxf(acc[o + 2], 0.f) : acc[o + 2];
			v.w = relu ? fmaxf(acc[o + 3], 0.f) : acc[o + 3];
			*reinterpret_cast<float4 *>(out + o) = v;
		}
	}
	else {
#pragma unroll
		for(int o = 0; o < CO; o++) out[o] = relu ? fmaxf(acc[o], 0.f) : acc[o];
	}
}

// All output pixels of layer l for `batch` samples at level side L, strided
// over [first, first + stride, ...).  w/bias already in shared memory.
__device__ __forceinline__ void conv_layer_range(int l, const ConvSrc &s, const float *w, const float *bias, float *y,
                                                 int batch, int L, long long first, long long stride) {
	const long long npix = (long long) batch * L * L;
	const UNetLayerDesc d = unet_layer(l);
	for(long long p = first; p < npix; p += stride) {
		const int n = (int) (p / ((long long) L * L));
		const int r = (int) (p - (long long) n * L * L);
		const int i = r / L, j = r - (r / L) * L;
		if(d.ci == 2) conv_pixel<2, 16>(s, w, bias, n, i, j, L, d.relu, y + p * 16);
		else if(d.ci == 32) conv_pixel<32, 16>(s, w, bias, n, i, j, L, d.relu, y + p * 16);
		else if(d.co == 16) conv_pixel<16, 16>(s, w, bias, n, i, j, L, d.relu, y + p * 16);
		else conv_pixel<16, 1>(s, w, bias, n, i, j, L, d.relu, y + p);
	}
}

// Activation buffers of one forward pass (batch samples at side L; level
// k has side L >> k).  Each pointer holds batch*(L>>k)^2*channels floats.
struct UNetActs {
	float *x0;                 // [R/s, W], 2 channels, level 0
	float *e0a, *s0, *d0a, *t0; // level 0, 16 channels
	float *out;                // level 0, 1 channel
	float *e1a, *s1, *d1a, *t1; // level 1
	float *b0, *t2;            // level 2
};

__host__ __device__ inline ConvSrc unet_src(int l, const UNetActs &A) {
	switch(l) {
	case L_E0A: return ConvSrc{IN_DIRECT, A.x0, nullptr};
	case L_E0B: return ConvSrc{IN_DIRECT, A.e0a, nullptr};
	case L_E1A: return ConvSrc{IN_POOL, A.s0, nullptr};
	case L_E1B: return ConvSrc{IN_DIRECT, A.e1a, nullptr};
	case L_B0: return ConvSrc{IN_POOL, A.s1, nullptr};
	case L_B1: return ConvSrc{IN_DIRECT, A.b0, nullptr};
	case L_D1A: return ConvSrc{IN_UPCAT, A.t2, A.s1};
	case L_D1B: return ConvSrc{IN_DIRECT, A.d1a, nullptr};
	case L_D0A: return ConvSrc{IN_UPCAT, A.t1, A.s0};
	case L_D0B: return ConvSrc{IN_DIRECT, A.d0a, nullptr};
	default: return ConvSrc{IN_DIRECT, A.t0, nullptr};
	}
}

__host__ __device__ inline float *unet_dst(int l, const UNetActs &A) {
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
	default: return A.out;
	}
}

}  // namespace rc
