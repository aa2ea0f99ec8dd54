/*
 * FD_CUDABackend: the reference's FD time step on the GB300 engine.  See the
 * header for the place of this class in the reference; this file maps the
 * reference's state and input keys onto the engine's C ABI.
 */
#include "FD_CUDABackend.h"

#include "Fields/BaseField.h"
#include "Utilities/RCexception.h"
#include "Utilities/Timings.h"
#include "Utilities/parse_input/parse_input.h"

#include <cstdlib>
#include <cstring>

FD_CUDABackend::FD_CUDABackend() :
				FDBackend() {
}

FD_CUDABackend::~FD_CUDABackend() {
	if(engine_) rc_destroy(engine_);
}

std::string FD_CUDABackend::precision_name() const {
#ifdef CUDA_DOUBLE_PRECISION
	return "double";
#else
	return "float";
#endif
}

void FD_CUDABackend::check(int rc, const char *what) {
	if(rc != RC_OK) throw RCexception("GB300 engine, %s: %s", what, rc_last_error(engine_));
}

namespace {

// The interaction parameters in force before apply_changes_after_equilibration
// are each interaction's constructor values; after it, the input keys.
struct ModelDefaults {
	int model;
	double gamma, lambda, omega, mu, kappa;
};

// Constructor values of the four interactions (SimpleMultiField.cpp:4-12,
// ActiveNematic.cpp:4-16, WetPolarModel.cpp:4-21, WetModel.cpp:4-21).
bool model_defaults(const std::string &name, ModelDefaults &d) {
	if(name == "simplefield") d = {RC_SIMPLEFIELD, 0.01, 2.5, 0.0, 3.0, 0.1};
	else if(name == "activenematic") d = {RC_ACTIVENEMATIC, 0.01, 2.5, 0.004, 3.0, 0.1};
	else if(name == "wetpolarmodel") d = {RC_WETPOLARMODEL, 0.06, 2.5, 0.004, 20.0, 0.1};
	else if(name == "wetmodel") d = {RC_WETMODEL, 0.01, 2.5, 0.004, 3.0, 0.1};
	else return false;
	return true;
}

double number_or(input_file &inp, const char *key, double def, int mandatory = 0) {
	number v = def;
	getInputNumber(&inp, key, &v, mandatory);
	return (double) v;
}

}  // namespace

void FD_CUDABackend::get_settings(input_file &inp) {
	// SimBackend: interaction, box, conf/trajectory files, seed, max_io;
	// FDBackend: dt and the box type (FDBackend.cpp:19-44)
	FDBackend::get_settings(inp);

	const std::string prec = precision_name();
	params_.precision = prec == "double" ? RC_PRECISION_DOUBLE : (prec == "mixed" ? RC_PRECISION_MIXED : RC_PRECISION_FLOAT);

	std::string sim_type("FD_CPU");
	getInputString(&inp, "sim_type", sim_type, 0);
	params_.conserved = sim_type == "FD_CH" ? 1 : 0;
	if(lees_edwards) throw RCexception("GB300 engine: Lees-Edwards boundaries are not provided");
	std::string box_type("square");
	getInputString(&inp, "box", box_type, 0);
	if(box_type != "square")
		throw RCexception("GB300 engine: box '%s' is not provided (square boxes, with or without walls, only)", box_type.c_str());
	params_.wall_slip = number_or(inp, "wall_slip", 0.5);  // BaseInteraction.cpp:10,23
	bool ext = false;
	getInputBool(&inp, "external_forces", &ext, 0);
	if(ext) throw RCexception("GB300 engine: external forces are not provided");

	std::string name;
	getInputString(&inp, "interaction_type", name, 1);
	ModelDefaults d;
	if(!model_defaults(name, d)) throw RCexception("GB300 engine: interaction_type '%s' is not provided", name.c_str());
	params_.model = d.model;
	int R = 8;
	getInputInt(&inp, "R", &R, 1);
	params_.R = R;
	params_.border = 4;  // BaseField.cpp:5
	params_.dt = (double) dt;
	params_.J0 = number_or(inp, "J0", 1.0);
	params_.gamma = number_or(inp, "gamma", d.gamma);
	// SimpleMultiField::get_settings does not read lambda (SimpleMultiField.cpp:19-27)
	params_.lambda = d.model == RC_SIMPLEFIELD ? d.lambda : number_or(inp, "lambda", d.lambda);
	params_.omega = number_or(inp, "omega", d.omega);
	params_.mu = number_or(inp, "mu", d.mu);
	params_.kappa = number_or(inp, "kappa", d.kappa);
	const bool wet_model = d.model == RC_WETMODEL || d.model == RC_WETPOLARMODEL;
	params_.passive_alpha = wet_model ? number_or(inp, "passive_alpha", 1.0) : 1.0;
	params_.cg_tolerance = wet_model ? number_or(inp, "CGtolerance", 0.0001) : 0.0;
	params_.cg_restart_every = d.model == RC_WETPOLARMODEL ? 10 : 100;  // WetPolarModel.cpp:152, WetModel.cpp:195-201
	auto both = [](double *a, double before, double after) {
		a[0] = before;
		a[1] = after;
	};
	if(d.model == RC_SIMPLEFIELD) {
		both(params_.friction, 1.0, 1.0);
	}
	else if(d.model == RC_ACTIVENEMATIC) {
		const double fr = number_or(inp, "friction", 2.0);
		both(params_.friction, fr, fr);
		both(params_.zetaQ_self, 0.0, number_or(inp, "zetaQ_self", 0.0, 1));
		both(params_.zetaQ_inter, 0.0, number_or(inp, "zetaQ_inter", 0.0, 1));
		both(params_.J_Q, 0.0, number_or(inp, "J_Q", 0.0, 1));
	}
	else {
		both(params_.friction, 1.0, number_or(inp, "friction", 0.0, 1));
		both(params_.friction_cell, 0.0, number_or(inp, "friction_cell", 0.0, 1));
		both(params_.zetaQ_self, 0.0, number_or(inp, "zetaQ_self", 0.0, 1));
		both(params_.zetaQ_inter, 0.0, number_or(inp, "zetaQ_inter", 0.0, 1));
		both(params_.J_Q, 0.0, number_or(inp, "J_Q", 0.0, 1));
		if(d.model == RC_WETPOLARMODEL) both(params_.beta, 0.0, number_or(inp, "beta", 0.0, 1));
	}
	getInputInt(&inp, "CUDA_device", &device_, 0);
}

void FD_CUDABackend::init() {
	// SimBackend::init: topology, configuration and the drand48 draws of
	// read_topology and MultiPhaseField::init, unchanged; FDBackend::init: timers
	FDBackend::init();

	std::vector<rc_cell_host> cells(fields.size());
	for(size_t i = 0; i < fields.size(); i++) {
		BaseField *p = fields[i];
		rc_cell_host &h = cells[i];
		memset(&h, 0, sizeof(h));
		h.lsub_x = p->LsubX;
		h.lsub_y = p->LsubY;
		h.offset_x = p->offset[0];
		h.offset_y = p->offset[1];
		h.corner = p->sub_corner_bottom_left;
		h.type = p->type;
		h.com_x = p->CoM[0];
		h.com_y = p->CoM[1];
		h.unrap_x = p->unrap_sub_corner_bottom_left_x;
		h.unrap_y = p->unrap_sub_corner_bottom_left_y;
		h.q00 = p->Q00;
		h.q01 = p->Q01;
		h.theta_q = p->thetaQ;
		h.theta_q_old = p->thetaQ_old;
		h.nemq_x = p->nemQ[0];
		h.nemq_y = p->nemQ[1];
		h.nemq_old_x = p->nemQ_old[0];
		h.nemq_old_y = p->nemQ_old[1];
		h.area = p->area;
		h.sum_f = p->sumF;
		h.capacity = p->subSize;
		h.phi = p->fieldScalar.data();
	}
	// drand48's state after those draws (seed48 returns it and installs the
	// probe; the second call puts it back), continued by the device's polar
	// noise stream
	unsigned short probe[3] = {0, 0, 0}, cur[3];
	memcpy(cur, seed48(probe), sizeof(cur));
	seed48(cur);
	params_.rng_state = (unsigned long long) cur[0] | ((unsigned long long) cur[1] << 16) | ((unsigned long long) cur[2] << 32);
	params_.rng_has_cached = 0;
	params_.rng_cached = 0.0;

	rc_box b = {box->getXsize(), box->getYsize(), nullptr};
	// the box's wall values (SquareWalls, CircleWalls, TriangleWalls; zero for
	// the periodic SquareBox, whose sites are all open unless wall_slip <= 0)
	std::vector<double> walls((size_t) b.Lx * (size_t) b.Ly);
	bool any_wall = params_.wall_slip <= 0.0;
	for(size_t k = 0; k < walls.size(); k++) {
		walls[k] = (double) box->getWalls((int) k);
		any_wall |= walls[k] != 0.0;
	}
	if(any_wall) b.walls = walls.data();
	// the first force evaluation of FD_CPUBackend::init (FD_CPUBackend.cpp:19-42)
	// runs inside rc_create
	const int rc = rc_create(&params_, &b, (int) cells.size(), cells.data(), device_, &engine_);
	if(rc != RC_OK) {
		const std::string m = rc_last_error(engine_);
		if(engine_) rc_destroy(engine_);
		engine_ = nullptr;
		throw RCexception("GB300 engine: %s", m.c_str());
	}
	phi_seen_.resize(fields.size());
	for(size_t i = 0; i < fields.size(); i++) phi_seen_[i] = fields[i]->fieldScalar;
	in_sync_ = true;
}

void FD_CUDABackend::sim_step() {
	mytimer->resume();
	check(rc_step(engine_, 1, &stats_), "rc_step");
	in_sync_ = false;
	mytimer->pause();
}

void FD_CUDABackend::apply_simulation_changes_after_equilibration() {
	SimBackend::apply_simulation_changes_after_equilibration();
	check(rc_set_phase(engine_, 1), "rc_set_phase");
}

void FD_CUDABackend::apply_simulation_data_changes() {
	if(in_sync_) return;
	const size_t n = fields.size();
	std::vector<int> lx(n), ly(n);
	check(rc_get_sizes(engine_, nullptr, lx.data(), ly.data()), "rc_get_sizes");
	std::vector<rc_cell_host> cells(n);
	for(size_t i = 0; i < n; i++) {
		BaseField *p = fields[i];
		const int m = lx[i] * ly[i];
		if(p->LsubX != lx[i] || p->LsubY != ly[i] || (int) p->fieldScalar.size() != m) {
			// a patch the engine grew (MultiPhaseField::resizing): resize the mirrors
			p->LsubX = lx[i];
			p->LsubY = ly[i];
			p->subSize = m;
			p->fieldScalar.resize(m);
			p->map_sub_to_box.resize(m);
			p->map_sub_to_box_x.resize(m);
			p->map_sub_to_box_y.resize(m);
			p->freeEnergy.resize(m);
			p->fieldDX.resize(m);
			p->fieldDY.resize(m);
		}
		p->velocityX.resize(m);
		p->velocityY.resize(m);
		rc_cell_host &h = cells[i];
		memset(&h, 0, sizeof(h));
		h.capacity = m;
		h.phi = p->fieldScalar.data();
		h.box_index = p->map_sub_to_box.data();
		h.mu = p->freeEnergy.data();
		h.dx = p->fieldDX.data();
		h.dy = p->fieldDY.data();
		h.vx = p->velocityX.data();
		h.vy = p->velocityY.data();
	}
	check(rc_download(engine_, cells.data(), RC_FIELD_ALL), "rc_download");
	const int Lx = box->getXsize();
	for(size_t i = 0; i < n; i++) {
		BaseField *p = fields[i];
		const rc_cell_host &h = cells[i];
		p->offset[0] = h.offset_x;
		p->offset[1] = h.offset_y;
		p->sub_corner_bottom_left = h.corner;
		p->CoM[0] = h.com_x;
		p->CoM[1] = h.com_y;
		p->unrap_sub_corner_bottom_left_x = h.unrap_x;
		p->unrap_sub_corner_bottom_left_y = h.unrap_y;
		p->Q00 = h.q00;
		p->Q01 = h.q01;
		p->thetaQ = h.theta_q;
		p->thetaQ_old = h.theta_q_old;
		p->nemQ[0] = h.nemq_x;
		p->nemQ[1] = h.nemq_y;
		p->nemQ_old[0] = h.nemq_old_x;
		p->nemQ_old[1] = h.nemq_old_y;
		p->area = h.area;
		p->sumF = h.sum_f;
		p->perimeter = h.perimeter;
		p->S00 = h.s00;
		p->S01 = h.s01;
		p->total_force_repulsion_x = h.force_rep_x;
		p->total_force_repulsion_y = h.force_rep_y;
		for(int q = 0; q < p->subSize; q++) {
			p->map_sub_to_box_y[q] = p->map_sub_to_box[q] / Lx;
			p->map_sub_to_box_x[q] = p->map_sub_to_box[q] - p->map_sub_to_box_y[q] * Lx;
		}
		phi_seen_[i] = p->fieldScalar;
	}
	in_sync_ = true;
}

void FD_CUDABackend::apply_changes_to_simulation_data() {
	// Only mirrors that hold the device's current state can carry edits; an
	// edited phi is sent back (rc_upload: the next step uses the forces of
	// the last evaluation, as the CPU backend does).
	if(!engine_ || !in_sync_) return;
	bool edited = false;
	for(size_t i = 0; i < fields.size() && !edited; i++) edited = fields[i]->fieldScalar != phi_seen_[i];
	if(!edited) return;
	std::vector<rc_cell_host> cells(fields.size());
	for(size_t i = 0; i < fields.size(); i++) {
		BaseField *p = fields[i];
		if((int) p->fieldScalar.size() != (int) phi_seen_[i].size())
			throw RCexception("GB300 engine: patch %d changed size on the host", (int) i);
		memset(&cells[i], 0, sizeof(rc_cell_host));
		cells[i].capacity = p->subSize;
		cells[i].phi = p->fieldScalar.data();
	}
	check(rc_upload(engine_, cells.data(), RC_FIELD_PHI), "rc_upload");
	for(size_t i = 0; i < fields.size(); i++) phi_seen_[i] = fields[i]->fieldScalar;
}
