// Test driver for the unmodified reference (deppinto/RheoCell), compiled
// out-of-tree by oracle/Makefile into oracle/_ref/.  Test infrastructure only:
// it produces golden dumps and CPU timings; nothing in the product links it.
//
// It reproduces the order of SimManager::load_options / init / run
// (src/Managers/SimManager.cpp:53-178): srand48(seed), backend factory,
// get_settings, init (which performs the passive first force evaluation,
// src/Backends/FD_CPUBackend.cpp:19-42), the equilibration steps, then
// apply_simulation_changes_after_equilibration (SimManager.cpp:144) and the
// main loop of sim_step calls.  Observables and configuration printing are
// skipped: they do not feed back into the dynamics.
//
// Usage:
//   ref_driver dump  <out.bin> <steps,csv> <input> [key=value ...]
//   ref_driver time  <n_steps>             <input> [key=value ...]
//   ref_driver observe <out.txt> <step>:<type>:<size_grid> <input> [key=value ...]
//     after <step> main-loop steps, the output string of the reference's
//     own field observable <type> (force_field, stress_field or
//     thermodynamic_stress_field) with that
//     size_grid, as its ObservableOutput would print it
//
// Dump record layout (little endian), one record per requested step (step 0 is
// the state right after init and equilibration, before the main loop):
//   int32 magic 0x50444352 ("RCDP"), int32 step, int32 N, int32 box side
//   per cell:
//     int32 LsubX, LsubY, offset_x, offset_y, sub_corner_bottom_left, type
//     double CoM_x, CoM_y, unrap_x, unrap_y, Q00, Q01, thetaQ, nemQ_x, nemQ_y,
//            area, sumF, perimeter, S00, S01, total_force_repulsion_x/_y
//     double phi[subSize]; int32 map_sub_to_box[subSize];
//     double vx[subSize], vy[subSize], freeEnergy[subSize], dx[subSize], dy[subSize]
#include "defs.h"
#include "Observables/ForceField.h"
#include "Observables/StressField.h"
#include "Observables/ThermodynamicStressField.h"
#include "Backends/BackendFactory.h"
#include "Backends/SimBackend.h"
#include "Interactions/BaseInteraction.h"
#include "Utilities/ConfigInfo.h"
#include "Utilities/RCexception.h"
#include "Utilities/Timings.h"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <set>
#include <sstream>
#include <string>
#include <vector>

static void write_i32(FILE *f, int v) { fwrite(&v, sizeof(int), 1, f); }
static void write_f64(FILE *f, double v) { fwrite(&v, sizeof(double), 1, f); }

static void dump_state(FILE *f, long long step) {
	auto ci = ConfigInfo::instance();
	std::vector<BaseField *> &fields = ci->fields();
	BaseInteraction *inter = ci->interaction;
	write_i32(f, 0x50444352);
	write_i32(f, (int) step);
	write_i32(f, (int) fields.size());
	write_i32(f, ci->box->getXsize());
	for(BaseField *p : fields) {
		write_i32(f, p->LsubX);
		write_i32(f, p->LsubY);
		write_i32(f, p->offset[0]);
		write_i32(f, p->offset[1]);
		write_i32(f, p->sub_corner_bottom_left);
		write_i32(f, p->type);
		write_f64(f, p->CoM[0]);
		write_f64(f, p->CoM[1]);
		write_f64(f, p->unrap_sub_corner_bottom_left_x);
		write_f64(f, p->unrap_sub_corner_bottom_left_y);
		write_f64(f, p->Q00);
		write_f64(f, p->Q01);
		write_f64(f, p->thetaQ);
		write_f64(f, p->nemQ[0]);
		write_f64(f, p->nemQ[1]);
		write_f64(f, p->area);
		write_f64(f, p->sumF);
		write_f64(f, p->perimeter);
		write_f64(f, p->S00);
		write_f64(f, p->S01);
		write_f64(f, p->total_force_repulsion_x);
		write_f64(f, p->total_force_repulsion_y);
		const int n = p->subSize;
		fwrite(p->fieldScalar.data(), sizeof(double), n, f);
		fwrite(p->map_sub_to_box.data(), sizeof(int), n, f);
		for(int q = 0; q < n; q++) write_f64(f, inter->get_velocity_x(p, q));
		for(int q = 0; q < n; q++) write_f64(f, inter->get_velocity_y(p, q));
		fwrite(p->freeEnergy.data(), sizeof(double), n, f);
		fwrite(p->fieldDX.data(), sizeof(double), n, f);
		fwrite(p->fieldDY.data(), sizeof(double), n, f);
	}
}

int main(int argc, char *argv[]) {
	const std::string mode = argc > 1 ? argv[1] : "";
	if(argc < (mode == "time" ? 4 : 5)) {
		fprintf(stderr, "usage: %s dump <out> <steps,csv> <input> [k=v...] | time <n> <input> [k=v...]\n", argv[0]);
		return 2;
	}
	try {
		Logger::init();
		TimingManager::init();

		// the parser takes (program, input file, key=value ...): the argument
		// before the input file stands in for the program name
		const int skip = mode == "time" ? 2 : 3;
		input_file input(true);
		input.init_from_command_line_args(argc - skip, argv + skip);

		long long steps = 0, eq_steps = 0;
		int seed = 1;
		getInputLLInt(&input, "steps", &steps, 0);
		getInputLLInt(&input, "equilibration_steps", &eq_steps, 0);
		getInputInt(&input, "seed", &seed, 1);

		std::set<long long> dump_steps;
		FILE *out = nullptr;
		if(mode == "dump") {
			std::stringstream ss(argv[3]);
			std::string tok;
			while(std::getline(ss, tok, ',')) dump_steps.insert(std::atoll(tok.c_str()));
			out = fopen(argv[2], "wb");
			if(!out) throw RCexception("cannot open dump file %s", argv[2]);
			steps = 0;
			for(long long s : dump_steps) steps = std::max(steps, s);
		}
		else if(mode == "time") {
			steps = std::atoll(argv[2]);
		}
		else if(mode == "observe") {
			steps = std::atoll(argv[3]);
		}
		else {
			throw RCexception("unknown mode %s", mode.c_str());
		}

		srand48(seed);
		std::shared_ptr<SimBackend> backend = BackendFactory::make_backend(input);
		backend->get_settings(input);
		backend->init();
		backend->apply_changes_to_simulation_data();
		for(long long s = 0; s < eq_steps; s++) backend->sim_step();
		backend->apply_simulation_changes_after_equilibration();
		if(out && dump_steps.count(0)) dump_state(out, 0);

		auto t0 = std::chrono::steady_clock::now();
		for(long long s = 1; s <= steps; s++) {
			backend->sim_step();
			backend->increment_current_step();
			if(out && dump_steps.count(s)) dump_state(out, s);
		}
		auto t1 = std::chrono::steady_clock::now();
		if(out) fclose(out);
		if(mode == "observe") {
			// <step>:<type>:<size_grid>; the backend's fields hold the state
			// and the forces of the last evaluation, as when SimBackend prints
			std::string spec = argv[3];
			const size_t c1 = spec.find(':'), c2 = spec.find(':', c1 + 1);
			const std::string type = spec.substr(c1 + 1, c2 - c1 - 1);
			input_file oi;
			oi.init_from_string("type = " + type + "\nsize_grid = " + spec.substr(c2 + 1) + "\n");
			std::shared_ptr<BaseObservable> obs;
			if(type == "force_field") obs = std::make_shared<ForceField>();
			else if(type == "stress_field") obs = std::make_shared<StressField>();
			else if(type == "thermodynamic_stress_field") obs = std::make_shared<ThermodynamicStressField>();
			else throw RCexception("unknown observable %s", type.c_str());
			obs->get_settings(oi, input);
			obs->init();
			FILE *o = fopen(argv[2], "w");
			if(!o) throw RCexception("cannot open %s", argv[2]);
			const std::string text = obs->get_output_string(steps);
			fwrite(text.data(), 1, text.size(), o);
			fclose(o);
		}
		if(mode == "time") {
			double secs = std::chrono::duration<double>(t1 - t0).count();
			printf("{\"steps\": %lld, \"seconds\": %.9f}\n", steps, secs);
		}
	}
	catch(RCexception &e) {
		fprintf(stderr, "RCexception: %s\n", e.what());
		return 1;
	}
	return 0;
}
