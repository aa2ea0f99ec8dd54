// Training of the learned preconditioner's network on the device: FP32
// forward (the same convolution code the solve uses), relative-L2 loss,
// backward through every layer, Adam.  All reductions are in a fixed order,
// so a training run is reproducible bit for bit.
#include "rc_unet.cuh"
#include "rc_unet_train.cuh"
#include "rc_unet_tc.cuh"
#include "../../include/rheocell_gb300.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

namespace rc {

namespace {

constexpr int FWD_THREADS = 256;
constexpr int DW_CHUNK = 1024;  // pixels per weight-gradient block

__global__ void __launch_bounds__(FWD_THREADS) conv_fwd_kernel(int l, ConvSrc s, const float *params, float *y,
                                                                int batch, int L) {
	__shared__ float w[UNET_MAX_LAYER_PARAMS];
	const UNetLayerDesc d = unet_layer(l);
	const int nw = 9 * d.ci * d.co + d.co;
	const float *src = params + unet_weight_offset(l);
	for(int k = threadIdx.x; k < nw; k += blockDim.x) w[k] = src[k];
	__syncthreads();
	conv_layer_range(l, s, w, w + 9 * d.ci * d.co, y, batch, L, blockIdx.x * (long long) blockDim.x + threadIdx.x,
	                 (long long) gridDim.x * blockDim.x);
}

// per-sample sums |y - t|^2 and |t|^2 (one block per sample, fixed order)
__global__ void __launch_bounds__(1024) loss_sums_kernel(const float *y, const float *t, int L, double *num,
                                                          double *den) {
	__shared__ double sa[1024], sb[1024];
	const int n = blockIdx.x;
	const long long P = (long long) L * L;
	double a = 0.0, b = 0.0;
	for(long long p = threadIdx.x; p < P; p += blockDim.x) {
		const double tv = t[n * P + p], d = (double) y[n * P + p] - tv;
		a += d * d;
		b += tv * tv;
	}
	sa[threadIdx.x] = a;
	sb[threadIdx.x] = b;
	__syncthreads();
	for(int h = blockDim.x / 2; h > 0; h >>= 1) {
		if(threadIdx.x < h) {
			sa[threadIdx.x] += sa[threadIdx.x + h];
			sb[threadIdx.x] += sb[threadIdx.x + h];
		}
		__syncthreads();
	}
	if(threadIdx.x == 0) {
		num[n] = sa[0];
		den[n] = sb[0];
	}
}

__global__ void loss_grad_kernel(const float *y, const float *t, const double *den, int batch, int L, float *g) {
	const long long P = (long long) L * L, tot = P * batch;
	for(long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < tot; k += (long long) gridDim.x * blockDim.x) {
		const int n = (int) (k / P);
		const double dn = den[n] > 1e-300 ? den[n] : 1e-300;
		g[k] = (float) (2.0 * ((double) y[k] - t[k]) / ((double) batch * dn));
	}
}

__global__ void relu_mask_kernel(const float *g, const float *a, float *gz, long long n, int relu) {
	for(long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < n; k += (long long) gridDim.x * blockDim.x)
		gz[k] = (!relu || a[k] > 0.f) ? g[k] : 0.f;
}

// gx[(n, i, j)][c] = sum_t sum_o gz[(n, i - dy, j - dx)][o] w[t][c][o]
template<int CI, int CO>
__global__ void __launch_bounds__(FWD_THREADS) conv_dx_kernel(int l, const float *gz, const float *params, float *gx,
                                                               int batch, int L) {
	__shared__ float w[9 * CI * CO];
	const float *src = params + unet_weight_offset(l);
	for(int k = threadIdx.x; k < 9 * CI * CO; k += blockDim.x) w[k] = src[k];
	__syncthreads();
	const long long npix = (long long) batch * L * L;
	for(long long p = blockIdx.x * (long long) blockDim.x + threadIdx.x; p < npix; p += (long long) gridDim.x * blockDim.x) {
		const int n = (int) (p / ((long long) L * L));
		const int r = (int) (p - (long long) n * L * L);
		const int i = r / L, j = r - (r / L) * L;
		float acc[CI];
#pragma unroll
		for(int c = 0; c < CI; c++) acc[c] = 0.f;
#pragma unroll 1
		for(int t = 0; t < 9; t++) {
			const int ii = wrap(i - (t / 3 - 1), L), jj = wrap(j - (t % 3 - 1), L);
			const float *g = gz + ((size_t) (n * L + ii) * L + jj) * CO;
			float gv[CO];
#pragma unroll
			for(int o = 0; o < CO; o++) gv[o] = g[o];
			const float *wt = w + t * CI * CO;
#pragma unroll
			for(int c = 0; c < CI; c++) {
#pragma unroll
				for(int o = 0; o < CO; o++) acc[c] = fmaf(gv[o], wt[c * CO + o], acc[c]);
			}
		}
		float *out = gx + p * CI;
#pragma unroll
		for(int c = 0; c < CI; c++) out[c] = acc[c];
	}
}

// partial weight and bias gradients of layer l over one chunk of pixels:
// part[blk][t*CI*CO + c*CO + o] and part[blk][9*CI*CO + o]
template<int CO>
__global__ void conv_dw_kernel(int l, ConvSrc s, const float *gz, float *part, int batch, int L) {
	__shared__ float gs[128 * 16];
	const UNetLayerDesc d = unet_layer(l);
	const int ci = d.ci;
	const int nthr = 9 * ci + 1;
	const int k = threadIdx.x;
	const int t = k / ci, c = k - (k / ci) * ci;
	const long long npix = (long long) batch * L * L;
	const long long p0 = (long long) blockIdx.x * DW_CHUNK;
	const long long p1 = p0 + DW_CHUNK < npix ? p0 + DW_CHUNK : npix;
	float acc[CO];
#pragma unroll
	for(int o = 0; o < CO; o++) acc[o] = 0.f;
	for(long long q0 = p0; q0 < p1; q0 += 128) {
		const int cnt = (int) (p1 - q0 < 128 ? p1 - q0 : 128);
		__syncthreads();
		for(int e = threadIdx.x; e < cnt * CO; e += blockDim.x) gs[e] = gz[q0 * CO + e];
		__syncthreads();
		if(k < nthr) {
			for(int q = 0; q < cnt; q++) {
				const long long p = q0 + q;
				float x = 1.f;
				if(k < 9 * ci) {
					const int n = (int) (p / ((long long) L * L));
					const int r = (int) (p - (long long) n * L * L);
					const int i = r / L, j = r - (r / L) * L;
					x = input_scalar(s, ci, n, wrap(i + t / 3 - 1, L), wrap(j + t % 3 - 1, L), L, c);
				}
#pragma unroll
				for(int o = 0; o < CO; o++) acc[o] = fmaf(x, gs[q * CO + o], acc[o]);
			}
		}
	}
	if(k < nthr) {
		const int stride = 9 * ci * CO + CO;
		float *out = part + (size_t) blockIdx.x * stride + (k < 9 * ci ? (t * ci + c) * CO : 9 * ci * CO);
#pragma unroll
		for(int o = 0; o < CO; o++) out[o] = acc[o];
	}
}

__global__ void dw_reduce_kernel(const float *part, int nblk, int stride, float *grad) {
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= stride) return;
	double s = 0.0;
	for(int b = 0; b < nblk; b++) s += part[(size_t) b * stride + k];
	grad[k] = (float) s;
}

// g_src (side 2L) += pool backward of gx (side L), ci channels
__global__ void pool_back_kernel(const float *gx, float *ga, int batch, int L, int ci) {
	const int L2 = 2 * L;
	const long long tot = (long long) batch * L2 * L2 * ci;
	for(long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < tot; k += (long long) gridDim.x * blockDim.x) {
		const int c = (int) (k % ci);
		const long long p = k / ci;
		const int n = (int) (p / ((long long) L2 * L2));
		const int r = (int) (p - (long long) n * L2 * L2);
		const int I = r / L2, J = r - (r / L2) * L2;
		ga[k] += 0.25f * gx[((size_t) (n * L + I / 2) * L + J / 2) * ci + c];
	}
}

// gx (side L, 32 channels) -> ga (side L/2, channels 0..15, sum of 4) and gb (side L, channels 16..31)
__global__ void upcat_back_kernel(const float *gx, float *ga, float *gb, int batch, int L) {
	const int Lh = L / 2;
	const long long tb = (long long) batch * L * L * 16;
	for(long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < tb; k += (long long) gridDim.x * blockDim.x) {
		const int c = (int) (k % 16);
		const long long p = k / 16;
		gb[k] += gx[p * 32 + 16 + c];
	}
	const long long ta = (long long) batch * Lh * Lh * 16;
	for(long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < ta; k += (long long) gridDim.x * blockDim.x) {
		const int c = (int) (k % 16);
		const long long p = k / 16;
		const int n = (int) (p / ((long long) Lh * Lh));
		const int r = (int) (p - (long long) n * Lh * Lh);
		const int i = r / Lh, j = r - (r / Lh) * Lh;
		const float *g = gx + ((size_t) (n * L + 2 * i) * L + 2 * j) * 32 + c;
		ga[k] += ((g[0] + g[32]) + g[(size_t) L * 32]) + g[(size_t) L * 32 + 32];
	}
}

__global__ void add_kernel(const float *x, float *y, long long n) {
	for(long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < n; k += (long long) gridDim.x * blockDim.x)
		y[k] += x[k];
}

__global__ void adam_kernel(float *p, const float *g, float *m, float *v, int n, float lr, float b1, float b2, float eps,
                            float c1, float c2) {
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= n) return;
	const float gk = g[k];
	const float mk = b1 * m[k] + (1.f - b1) * gk;
	const float vk = b2 * v[k] + (1.f - b2) * gk * gk;
	m[k] = mk;
	v[k] = vk;
	p[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
}

__global__ void gather_kernel(const float *hin, const float *htgt, const int *idx, int n, long long L2, float *x0,
                              float *tgt) {
	const long long tot = (long long) n * L2;
	for(long long e = blockIdx.x * (long long) blockDim.x + threadIdx.x; e < tot; e += (long long) gridDim.x * blockDim.x) {
		const long long b = e / L2, k = e - b * L2;
		const long long q = idx[b];
		const float2 v = *reinterpret_cast<const float2 *>(hin + (q * L2 + k) * 2);
		*reinterpret_cast<float2 *>(x0 + e * 2) = v;
		tgt[e] = htgt[q * L2 + k];
	}
}

// acc[0] += sum over the batch of |f - y|^2 / |y|^2 (one thread, sample order)
__global__ void loss_acc_kernel(const double *sums, int batch, double *acc) {
	if(threadIdx.x || blockIdx.x) return;
	double s = 0.0;
	for(int n = 0; n < batch; n++) s += sums[n] / (sums[batch + n] > 1e-300 ? sums[batch + n] : 1e-300);
	acc[0] += s;
}

int grid_for(long long n, int threads) {
	long long b = (n + threads - 1) / threads;
	if(b > 65536) b = 65536;
	return (int) (b < 1 ? 1 : b);
}

size_t level_pix(const UNetTrainer &T, int level) { return (size_t) T.batch * (T.L >> level) * (T.L >> level); }

}  // namespace

// --- allocation -------------------------------------------------------------

static int talloc(UNetTrainer &T, float **p, size_t n) {
	void *q = nullptr;
	if(cudaMalloc(&q, sizeof(float) * (n ? n : 1)) != cudaSuccess) return -1;
	cudaMemset(q, 0, sizeof(float) * (n ? n : 1));
	T.allocs.push_back(q);
	*p = (float *) q;
	return 0;
}

static int alloc_acts(UNetTrainer &T, UNetActs &A) {
	const size_t p0 = level_pix(T, 0), p1 = level_pix(T, 1), p2 = level_pix(T, 2);
	int rc = 0;
	rc |= talloc(T, &A.x0, p0 * 2);
	rc |= talloc(T, &A.e0a, p0 * 16);
	rc |= talloc(T, &A.s0, p0 * 16);
	rc |= talloc(T, &A.d0a, p0 * 16);
	rc |= talloc(T, &A.t0, p0 * 16);
	rc |= talloc(T, &A.out, p0);
	rc |= talloc(T, &A.e1a, p1 * 16);
	rc |= talloc(T, &A.s1, p1 * 16);
	rc |= talloc(T, &A.d1a, p1 * 16);
	rc |= talloc(T, &A.t1, p1 * 16);
	rc |= talloc(T, &A.b0, p2 * 16);
	rc |= talloc(T, &A.t2, p2 * 16);
	return rc;
}

int unet_trainer_init(UNetTrainer &T, int L, int batch) {
	if(L < 8 || L % 4 != 0 || batch < 1) return -2;
	T.L = L;
	T.batch = batch;
	const size_t p0 = level_pix(T, 0);
	T.dw_blocks = (int) ((p0 + DW_CHUNK - 1) / DW_CHUNK);
	int rc = 0;
	rc |= talloc(T, &T.params, UNET_PARAMS);
	rc |= talloc(T, &T.grad, UNET_PARAMS);
	rc |= talloc(T, &T.m, UNET_PARAMS);
	rc |= talloc(T, &T.v, UNET_PARAMS);
	rc |= alloc_acts(T, T.A);
	rc |= alloc_acts(T, T.G);
	rc |= talloc(T, &T.gz, p0 * 16);
	rc |= talloc(T, &T.gx, p0 * 32);
	rc |= talloc(T, &T.target, p0);
	rc |= talloc(T, &T.part, (size_t) T.dw_blocks * UNET_MAX_LAYER_PARAMS);
	void *q = nullptr;
	if(cudaMalloc(&q, sizeof(double) * 2 * batch) != cudaSuccess) rc |= -1;
	else {
		T.allocs.push_back(q);
		T.sums = (double *) q;
	}
	T.step = 0;
	return rc ? -1 : 0;
}

void unet_trainer_free(UNetTrainer &T) {
	for(void *p : T.allocs) cudaFree(p);
	T.allocs.clear();
}

// --- passes -----------------------------------------------------------------

void unet_forward(UNetTrainer &T, const float *params, cudaStream_t s) {
	for(int l = 0; l < UNET_LAYERS; l++) {
		const int Ll = T.L >> unet_layer(l).level;
		const long long npix = (long long) T.batch * Ll * Ll;
		conv_fwd_kernel<<<grid_for(npix, FWD_THREADS), FWD_THREADS, 0, s>>>(l, unet_src(l, T.A), params,
		                                                                    unet_dst(l, T.A), T.batch, Ll);
	}
}

void unet_loss(UNetTrainer &T, cudaStream_t s) {
	loss_sums_kernel<<<T.batch, 1024, 0, s>>>(T.A.out, T.target, T.L, T.sums, T.sums + T.batch);
	loss_grad_kernel<<<grid_for(level_pix(T, 0), 256), 256, 0, s>>>(T.A.out, T.target, T.sums + T.batch, T.batch, T.L,
	                                                                 T.G.out);
}

static void layer_dw(UNetTrainer &T, int l, cudaStream_t s) {
	const UNetLayerDesc d = unet_layer(l);
	const int Ll = T.L >> d.level;
	const long long npix = (long long) T.batch * Ll * Ll;
	const int nblk = (int) ((npix + DW_CHUNK - 1) / DW_CHUNK);
	const int thr = ((9 * d.ci + 1) + 31) / 32 * 32;
	if(d.co == 16) conv_dw_kernel<16><<<nblk, thr, 0, s>>>(l, unet_src(l, T.A), T.gz, T.part, T.batch, Ll);
	else conv_dw_kernel<1><<<nblk, thr, 0, s>>>(l, unet_src(l, T.A), T.gz, T.part, T.batch, Ll);
	const int stride = 9 * d.ci * d.co + d.co;
	dw_reduce_kernel<<<(stride + 255) / 256, 256, 0, s>>>(T.part, nblk, stride, T.grad + unet_weight_offset(l));
}

static void layer_dx(UNetTrainer &T, int l, const float *params, cudaStream_t s) {
	const UNetLayerDesc d = unet_layer(l);
	const int Ll = T.L >> d.level;
	const long long npix = (long long) T.batch * Ll * Ll;
	const int g = grid_for(npix, FWD_THREADS);
	if(d.ci == 32) conv_dx_kernel<32, 16><<<g, FWD_THREADS, 0, s>>>(l, T.gz, params, T.gx, T.batch, Ll);
	else if(d.co == 1) conv_dx_kernel<16, 1><<<g, FWD_THREADS, 0, s>>>(l, T.gz, params, T.gx, T.batch, Ll);
	else conv_dx_kernel<16, 16><<<g, FWD_THREADS, 0, s>>>(l, T.gz, params, T.gx, T.batch, Ll);
	// hand gx to the gradients of the layer's sources
	const ConvSrc src = unet_src(l, T.A);
	const ConvSrc gsrc = unet_src(l, T.G);
	if(d.mode == IN_DIRECT) {
		add_kernel<<<grid_for(npix * d.ci, 256), 256, 0, s>>>(T.gx, (float *) gsrc.a, npix * d.ci);
	}
	else if(d.mode == IN_POOL) {
		const long long n2 = (long long) T.batch * (2 * Ll) * (2 * Ll) * d.ci;
		pool_back_kernel<<<grid_for(n2, 256), 256, 0, s>>>(T.gx, (float *) gsrc.a, T.batch, Ll, d.ci);
	}
	else {
		upcat_back_kernel<<<grid_for(npix * 16, 256), 256, 0, s>>>(T.gx, (float *) gsrc.a, (float *) gsrc.b, T.batch, Ll);
	}
	(void) src;
}

void unet_backward(UNetTrainer &T, const float *params, cudaStream_t s) {
	// gradients w.r.t. every activation except the output start at zero
	const size_t p0 = level_pix(T, 0), p1 = level_pix(T, 1), p2 = level_pix(T, 2);
	cudaMemsetAsync(T.G.e0a, 0, sizeof(float) * p0 * 16, s);
	cudaMemsetAsync(T.G.s0, 0, sizeof(float) * p0 * 16, s);
	cudaMemsetAsync(T.G.d0a, 0, sizeof(float) * p0 * 16, s);
	cudaMemsetAsync(T.G.t0, 0, sizeof(float) * p0 * 16, s);
	cudaMemsetAsync(T.G.e1a, 0, sizeof(float) * p1 * 16, s);
	cudaMemsetAsync(T.G.s1, 0, sizeof(float) * p1 * 16, s);
	cudaMemsetAsync(T.G.d1a, 0, sizeof(float) * p1 * 16, s);
	cudaMemsetAsync(T.G.t1, 0, sizeof(float) * p1 * 16, s);
	cudaMemsetAsync(T.G.b0, 0, sizeof(float) * p2 * 16, s);
	cudaMemsetAsync(T.G.t2, 0, sizeof(float) * p2 * 16, s);
	for(int l = UNET_LAYERS - 1; l >= 0; l--) {
		const UNetLayerDesc d = unet_layer(l);
		const int Ll = T.L >> d.level;
		const long long n = (long long) T.batch * Ll * Ll * d.co;
		relu_mask_kernel<<<grid_for(n, 256), 256, 0, s>>>(unet_dst(l, T.G), unet_dst(l, T.A), T.gz, n, d.relu);
		layer_dw(T, l, s);
		if(l > 0) layer_dx(T, l, params, s);
	}
}

void unet_adam(UNetTrainer &T, float lr, cudaStream_t s) {
	T.step += 1;
	const float b1 = 0.9f, b2 = 0.999f;
	const float c1 = 1.f - powf(b1, (float) T.step), c2 = 1.f - powf(b2, (float) T.step);
	adam_kernel<<<(UNET_PARAMS + 255) / 256, 256, 0, s>>>(T.params, T.grad, T.m, T.v, UNET_PARAMS, lr, b1, b2, 1e-8f, c1,
	                                                      c2);
}

void unet_gather(UNetTrainer &T, const float *hin, const float *htgt, const int *idx, int n, cudaStream_t s) {
	const long long L2 = (long long) T.L * T.L;
	gather_kernel<<<grid_for(n * L2, 256), 256, 0, s>>>(hin, htgt, idx, n, L2, T.A.x0, T.target);
}

void unet_accumulate_loss(UNetTrainer &T, double *acc, cudaStream_t s) {
	loss_acc_kernel<<<1, 32, 0, s>>>(T.sums, T.batch, acc);
}

double unet_read_loss(UNetTrainer &T, cudaStream_t s) {
	std::vector<double> h((size_t) 2 * T.batch);
	cudaMemcpyAsync(h.data(), T.sums, sizeof(double) * 2 * T.batch, cudaMemcpyDeviceToHost, s);
	cudaStreamSynchronize(s);
	double acc = 0.0;
	for(int n = 0; n < T.batch; n++) acc += h[(size_t) n] / (h[(size_t) T.batch + n] > 1e-300 ? h[(size_t) T.batch + n] : 1e-300);
	return acc / T.batch;
}

}  // namespace rc

// --- tensor-core inference ----------------------------------------------------

namespace rc {

namespace {

__global__ void pack_bf16_kernel(const float *params, bf16 *packed) {
	for(int l = 0; l < UNET_LAYERS; l++) {
		const UNetLayerDesc d = unet_layer(l);
		if(d.co != 16 || d.ci < 16) continue;
		const int KC = d.ci / 8, n = 9 * d.ci * 16;
		const float *w = params + unet_weight_offset(l);
		bf16 *o = packed + unet_pack_offset(l);
		for(int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
			const int e = idx & 7, co = (idx >> 3) & 15;
			const int tk = idx >> 7, kc = tk % KC, t = tk / KC;
			o[idx] = __float2bfloat16_rn(w[(t * d.ci + kc * 8 + e) * 16 + co]);
		}
	}
}

// One CTA per SM (the TMEM allocation is the whole of an SM's 512 columns).
__global__ void __launch_bounds__(512, 1) tc_layer_kernel(int l, TcSrc src, const bf16 *packed, const float *params,
                                                           bf16 *dst, int batch, int L, int *err) {
	extern __shared__ __align__(1024) unsigned char tsm[];
	uint32_t *hold = reinterpret_cast<uint32_t *>(tsm + TC_HOLD_OFF);
	uint64_t *mbar = reinterpret_cast<uint64_t *>(tsm + TC_MBAR_OFF);
	if(threadIdx.x < 32) tc_alloc(hold, TC_COLS);
	if(threadIdx.x == 0)
		for(int k = 0; k < TC_NMBAR; k++) mbar_init(mbar + k, 1);
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	TcCtx c{tsm, *hold, {0u, 0u}, err, 1, nullptr};
	tc_conv_layer(l, src, packed + unet_pack_offset(l), params + unet_weight_offset(l), params + unet_bias_offset(l), dst,
	              batch, L, c);
	tc_fence_before();
	__syncthreads();
	if(threadIdx.x < 32) tc_dealloc(c.tmem, TC_COLS);
}

__global__ void e0a_kernel(const float *x0, const float *params, bf16 *dst, int batch, int L) {
	__shared__ float w[9 * 2 * 16 + 16];
	for(int k = threadIdx.x; k < 9 * 2 * 16 + 16; k += blockDim.x) w[k] = params[unet_weight_offset(L_E0A) + k];
	__syncthreads();
	e0a_range(x0, w, dst, batch, L, blockIdx.x * (long long) blockDim.x + threadIdx.x, (long long) gridDim.x * blockDim.x);
}

__global__ void out_kernel(const bf16 *t0, const float *params, float *dst, int batch, int L) {
	__shared__ float w[9 * 16 + 1];
	for(int k = threadIdx.x; k < 9 * 16 + 1; k += blockDim.x) w[k] = params[unet_weight_offset(L_OUT) + k];
	__syncthreads();
	out_range(t0, w, dst, batch, L, blockIdx.x * (long long) blockDim.x + threadIdx.x, (long long) gridDim.x * blockDim.x);
}

}  // namespace

void unet_pack_bf16(const float *params, bf16 *packed, cudaStream_t s) { pack_bf16_kernel<<<64, 256, 0, s>>>(params, packed); }

cudaError_t unet_tc_configure() {
	return cudaFuncSetAttribute(tc_layer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) TC_SMEM);
}

// Forward pass with the tensor-core layers (separate launches): x0 (FP32) ->
// out (FP32) through the BF16 activations A.
void unet_tc_forward(const float *params, const bf16 *packed, const float *x0, const UNetActsBF &A, float *out, int batch,
                     int L, int sms, int *err, cudaStream_t s) {
	const long long p0 = (long long) batch * L * L;
	// as in the solve: the first layer is evaluated while the second stages
	// its rows when L allows strips
	const bool fused_first = L % 128 == 0;
	if(!fused_first) e0a_kernel<<<grid_for(p0, 256), 256, 0, s>>>(x0, params, A.e0a, batch, L);
	for(int l = L_E0B; l <= L_D0B; l++) {
		const int Ll = L >> unet_layer(l).level;
		const long long tiles = ((long long) batch * Ll * Ll + 127) / 128;
		long long g = tiles;
		if(g > sms) g = sms;
		TcSrc src = unet_tc_src(l, A);
		if(l == L_E0B && fused_first) {
			src.mode = IN_FIRST;
			src.x = x0;
			src.w0 = params + unet_weight_offset(L_E0A);
		}
		tc_layer_kernel<<<(int) g, 512, TC_SMEM, s>>>(l, src, packed, params, unet_tc_dst(l, A), batch, Ll, err);
	}
	out_kernel<<<grid_for(p0, 256), 256, 0, s>>>(A.t0, params, out, batch, L);
}

}  // namespace rc

extern "C" int rc_unet_forward_tc(int L, int batch, const double *params, const double *input, double *output,
                                  int device) {
	using namespace rc;
	if(!params || !input || !output || batch < 1 || L < 8 || L % 4 != 0) return RC_ERR_INVALID;
	if(cudaSetDevice(device) != cudaSuccess) return RC_ERR_CUDA;
	if(unet_tc_configure() != cudaSuccess) return RC_ERR_CUDA;
	int sms = 0;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
	const size_t p0 = (size_t) batch * L * L, p1 = p0 / 4, p2 = p0 / 16;
	std::vector<void *> al;
	auto get = [&](size_t bytes) -> void * {
		void *q = nullptr;
		if(cudaMalloc(&q, bytes ? bytes : 16) != cudaSuccess) return nullptr;
		cudaMemset(q, 0, bytes ? bytes : 16);
		al.push_back(q);
		return q;
	};
	float *dp = (float *) get(sizeof(float) * UNET_PARAMS);
	bf16 *pk = (bf16 *) get(sizeof(bf16) * UNET_PACKED);
	float *x0 = (float *) get(sizeof(float) * p0 * 2);
	float *out = (float *) get(sizeof(float) * p0);
	int *err = (int *) get(sizeof(int));
	UNetActsBF A;
	A.e0a = (bf16 *) get(2 * p0 * 16);
	A.s0 = (bf16 *) get(2 * p0 * 16);
	A.d0a = (bf16 *) get(2 * p0 * 16);
	A.t0 = (bf16 *) get(2 * p0 * 16);
	A.e1a = (bf16 *) get(2 * p1 * 16);
	A.s1 = (bf16 *) get(2 * p1 * 16);
	A.d1a = (bf16 *) get(2 * p1 * 16);
	A.t1 = (bf16 *) get(2 * p1 * 16);
	A.b0 = (bf16 *) get(2 * p2 * 16);
	A.t2 = (bf16 *) get(2 * p2 * 16);
	bool okalloc = true;
	for(void *q : al) okalloc = okalloc && q;
	int rc = RC_OK;
	if(!okalloc || al.size() != 15) rc = RC_ERR_OOM;
	else {
		std::vector<float> hp(UNET_PARAMS), hx(p0 * 2), hy(p0);
		for(int k = 0; k < UNET_PARAMS; k++) hp[(size_t) k] = (float) params[k];
		for(size_t k = 0; k < 2 * p0; k++) hx[k] = (float) input[k];
		cudaMemcpy(dp, hp.data(), sizeof(float) * UNET_PARAMS, cudaMemcpyHostToDevice);
		cudaMemcpy(x0, hx.data(), sizeof(float) * 2 * p0, cudaMemcpyHostToDevice);
		unet_pack_bf16(dp, pk, nullptr);
		unet_tc_forward(dp, pk, x0, A, out, batch, L, sms, err, nullptr);
		const cudaError_t ce = cudaDeviceSynchronize();
		int herr = 0;
		cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost);
		cudaMemcpy(hy.data(), out, sizeof(float) * p0, cudaMemcpyDeviceToHost);
		if(ce != cudaSuccess) rc = RC_ERR_CUDA;
		else if(herr) rc = RC_ERR_CG;
		else
			for(size_t k = 0; k < p0; k++) output[k] = hy[k];
	}
	for(void *q : al)
		if(q) cudaFree(q);
	return rc;
}

// --- C ABI: one forward/loss/backward pass on host data ----------------------

extern "C" int rc_unet_loss_grad(int L, int batch, const double *params, const double *input, const double *target,
                                 double *loss, double *grad, double *output, int device) {
	using namespace rc;
	if(!params || !input || !target || batch < 1) return RC_ERR_INVALID;
	if(cudaSetDevice(device) != cudaSuccess) return RC_ERR_CUDA;
	UNetTrainer T;
	const int rc0 = unet_trainer_init(T, L, batch);
	if(rc0) {
		unet_trainer_free(T);
		return rc0 == -2 ? RC_ERR_INVALID : RC_ERR_OOM;
	}
	const size_t P = (size_t) batch * L * L;
	std::vector<float> hp(UNET_PARAMS), hx(P * 2), ht(P), hy(P), hg(UNET_PARAMS);
	for(int k = 0; k < UNET_PARAMS; k++) hp[(size_t) k] = (float) params[k];
	for(size_t k = 0; k < 2 * P; k++) hx[k] = (float) input[k];
	for(size_t k = 0; k < P; k++) ht[k] = (float) target[k];
	cudaStream_t s = nullptr;
	cudaMemcpy(T.params, hp.data(), sizeof(float) * UNET_PARAMS, cudaMemcpyHostToDevice);
	cudaMemcpy(T.A.x0, hx.data(), sizeof(float) * 2 * P, cudaMemcpyHostToDevice);
	cudaMemcpy(T.target, ht.data(), sizeof(float) * P, cudaMemcpyHostToDevice);
	unet_forward(T, T.params, s);
	unet_loss(T, s);
	unet_backward(T, T.params, s);
	const double l = unet_read_loss(T, s);
	cudaMemcpy(hy.data(), T.A.out, sizeof(float) * P, cudaMemcpyDeviceToHost);
	cudaMemcpy(hg.data(), T.grad, sizeof(float) * UNET_PARAMS, cudaMemcpyDeviceToHost);
	const cudaError_t err = cudaDeviceSynchronize();
	unet_trainer_free(T);
	if(err != cudaSuccess) return RC_ERR_CUDA;
	if(loss) *loss = l;
	if(grad)
		for(int k = 0; k < UNET_PARAMS; k++) grad[k] = hg[(size_t) k];
	if(output)
		for(size_t k = 0; k < P; k++) output[k] = hy[k];
	return RC_OK;
}
