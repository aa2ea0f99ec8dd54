// Device training state of the learned preconditioner's network (rc_unet.cu).
#pragma once

#include "rc_unet.cuh"
#include "rc_unet_tc.cuh"

#include <cuda_runtime.h>

#include <vector>

namespace rc {

struct UNetTrainer {
	int L = 0, batch = 0;
	int dw_blocks = 0;
	long long step = 0;
	float *params = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;  // FP32 master copy and Adam moments
	UNetActs A{};                                                          // activations of the last forward
	UNetActs G{};                                                          // gradients w.r.t. them
	float *gz = nullptr, *gx = nullptr;                                    // per-layer scratch
	float *target = nullptr;                                               // [batch][L][L]
	float *part = nullptr;                                                 // weight-gradient partial sums
	double *sums = nullptr;                                                // per-sample |f-y|^2, |y|^2
	std::vector<void *> allocs;
};

// 0 on success; -2 for an unsupported size (L % 4 != 0 or L < 8); -1 out of memory
int unet_trainer_init(UNetTrainer &T, int L, int batch);
void unet_trainer_free(UNetTrainer &T);
// input in T.A.x0 ([R/s, W] per pixel), target in T.target
void unet_forward(UNetTrainer &T, const float *params, cudaStream_t s);
void unet_loss(UNetTrainer &T, cudaStream_t s);
void unet_backward(UNetTrainer &T, const float *params, cudaStream_t s);
void unet_adam(UNetTrainer &T, float lr, cudaStream_t s);
double unet_read_loss(UNetTrainer &T, cudaStream_t s);
// samples idx[0..n) of a harvested set into T.A.x0 / T.target (n <= T.batch)
void unet_gather(UNetTrainer &T, const float *hin, const float *htgt, const int *idx, int n, cudaStream_t s);
// acc[0] += sum over the last loss evaluation's samples of |f - y|^2 / |y|^2
void unet_accumulate_loss(UNetTrainer &T, double *acc, cudaStream_t s);
// BF16 copy of the tensor-core layers' weights in the B-operand order
void unet_pack_bf16(const float *params, bf16 *packed, cudaStream_t s);
cudaError_t unet_tc_configure();

}  // namespace rc
