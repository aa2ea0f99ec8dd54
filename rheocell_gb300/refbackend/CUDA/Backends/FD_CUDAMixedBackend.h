/*
 * CUDAMixedBackend -- the factory's default CUDA backend when the reference
 * is built without CUDA_DOUBLE_PRECISION (backend_precision = mixed, the
 * value BackendFactory.cpp:41-46 picks when the key is absent).  It is the
 * GB300 engine with RC_PRECISION_MIXED: FP64 fields and per-cell integrals,
 * the wet models' viscous solve with FP32 inner iterations inside FP64
 * iterative refinement (true FP64 residual below CGtolerance).
 */
#ifndef FD_CUDAMIXEDBACKEND_H_
#define FD_CUDAMIXEDBACKEND_H_

#include "FD_CUDABackend.h"

class CUDAMixedBackend: public FD_CUDABackend {
protected:
	std::string precision_name() const override { return "mixed"; }
};

#endif /* FD_CUDAMIXEDBACKEND_H_ */
