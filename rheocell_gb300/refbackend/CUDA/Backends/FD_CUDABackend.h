/*
 * FD_CUDABackend -- the `backend = CUDA` slot of the reference's backend
 * factory (src/Backends/BackendFactory.cpp:5-10 includes this header,
 * :37-65 constructs the class), filled by the GB300 engine.
 *
 * It is an FDBackend like the reference's FD_CPUBackend
 * (src/Backends/FD_CPUBackend.h): SimBackend reads the input, topology and
 * configuration exactly as for the CPU backend (same drand48 draws), then the
 * whole time step -- FD_CPUBackend::sim_step (FD_CPUBackend.cpp:134-160) with
 * the interaction's force evaluation and the wet models' viscous solve -- runs
 * on the GPU through the engine's C ABI (include/rheocell_gb300.h).  The
 * BaseField objects become host mirrors of the device state, refreshed by
 * apply_simulation_data_changes(), which SimBackend calls before every print
 * (SimBackend.cpp:356,389,399,404).
 *
 * Build: compile the reference's sources without -DNOCUDA, with this
 * directory's parent (.../refbackend/CUDA) and the engine's include/ on the
 * include path, so that "../CUDA/Backends/FD_CUDABackend.h" resolves here;
 * add -DCUDA_DOUBLE_PRECISION for the build whose CUDA backend is FP64
 * (backend_precision = double), and link librheocell_gb300.so.
 */
#ifndef FD_CUDABACKEND_H_
#define FD_CUDABACKEND_H_

#include "Backends/FDBackend.h"
#include "rheocell_gb300.h"

#include <string>
#include <vector>

class FD_CUDABackend: public FDBackend {
public:
	FD_CUDABackend();
	virtual ~FD_CUDABackend();

	void get_settings(input_file &inp) override;
	void init() override;
	void sim_step() override;
	void apply_simulation_data_changes() override;
	void apply_changes_to_simulation_data() override;
	void apply_simulation_changes_after_equilibration() override;

	/// the engine handle, for observables that call rc_observe_* themselves
	rc_engine *engine() { return engine_; }

protected:
	/// backend_precision this class stands for in the factory's mapping
	/// (BackendFactory.cpp:38-63): "double" in a CUDA_DOUBLE_PRECISION build,
	/// "float" otherwise
	virtual std::string precision_name() const;
	void check(int rc, const char *what);

	rc_params params_ = {};
	rc_engine *engine_ = nullptr;
	rc_step_stats stats_ = {};
	int device_ = 0;
	bool in_sync_ = false;                    ///< mirrors hold the device state
	std::vector<std::vector<number>> phi_seen_; ///< phi as the device last had it (host edits are diffs against it)
};

#endif /* FD_CUDABACKEND_H_ */
