// rheocell -- command-line driver of the GB300 engine, a drop-in for the
// reference's `rheoCell input [key=value ...]` (src/rheoCell.cpp:13-49).
//
// It keeps the reference's input keys, topology and configuration formats and
// run loop, and replaces the backend: FD_CUDABackend below plays the role of
// the slot BackendFactory reserves for `backend = CUDA`
// (src/Backends/BackendFactory.cpp:37-65) and calls the engine through its C
// ABI (include/rheocell_gb300.h).  Host-side pieces mirrored here:
//   input file ........ key = value lines, '#' comments, command-line
//                       overrides (src/Utilities/parse_input/parse_input.cpp:117-160)
//   run loop .......... SimManager::load_options / init / run
//                       (src/Managers/SimManager.cpp:53-178)
//   RNG seeding ....... srand48(seed) then the draws of read_topology and
//                       MultiPhaseField::init (WetPolarModel.cpp:191,
//                       Fields/MultiPhaseField.cpp:79-95), with the C library's drand48
//   configuration ..... SimBackend::read_next_configuration (SimBackend.cpp:220-314)
//                       and Configuration::headers/field (Observables/Configuration.cpp:36-56)
//   output ............ trajectory (appended), last_conf (overwritten),
//                       equilibrated_conf (ObservableOutput.cpp:86-190,
//                       SimBackend.cpp:398-410); the I/O-rate limit max_io
//                       (SimBackend.cpp:157-166, 366-376)
//
// Output runs on a writer thread: at a print point the state is downloaded
// into a host snapshot, the snapshot is queued, and stepping continues while
// the thread formats and writes it (at most two snapshots in flight).
//
// Extra keys (not read by the reference): backend_precision = float (dry
// polar model), CUDA_device, and the learned preconditioner of the wet
// models' viscous solve -- cg_solver = learned with learned_harvest_steps
// (plain-CG steps that collect training samples, default 40),
// learned_train_epochs (default 20), learned_params_file (parameters to load
// instead of training, or to save after training).
#include "../../include/rheocell_gb300.h"

#include <chrono>
#include <cmath>
#include <condition_variable>
#include <csignal>
#include <deque>
#include <mutex>
#include <thread>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>
#include <atomic>

namespace {

const float PI_F = 3.141592653589793238462643f;
volatile std::sig_atomic_t g_stop = 0;
void on_signal(int) { g_stop = 1; }

struct RCexception : std::runtime_error {
	using std::runtime_error::runtime_error;
};

std::string trim(const std::string &s) {
	size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
	return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

// ---------------------------------------------------------------- input ---
class InputFile {
public:
	void add_line(std::string line) {
		size_t c = line.find('#');
		if(c != std::string::npos) line.erase(c);
		size_t eq = line.find('=');
		if(eq == std::string::npos) return;
		std::string k = trim(line.substr(0, eq)), v = trim(line.substr(eq + 1));
		if(!k.empty()) keys_[k] = v;
	}
	void load(const std::string &path) {
		std::ifstream f(path);
		if(!f.good()) throw RCexception("Input file '" + path + "' not found");
		std::string line;
		while(std::getline(f, line)) add_line(line);
	}
	bool has(const std::string &k) const { return keys_.count(k) > 0; }
	std::string str(const std::string &k, const std::string &def = "", bool required = false) const {
		auto it = keys_.find(k);
		if(it == keys_.end()) {
			if(required) throw RCexception("Mandatory key `" + k + "' not found");
			return def;
		}
		return it->second;
	}
	double num(const std::string &k, double def = 0, bool required = false) const {
		return has(k) ? std::stod(str(k)) : (required ? (str(k, "", true), 0.0) : def);
	}
	long long integer(const std::string &k, long long def = 0, bool required = false) const {
		return has(k) ? (long long) std::llround(std::stod(str(k))) : (required ? (str(k, "", true), 0LL) : def);
	}
	bool boolean(const std::string &k, bool def = false) const {
		if(!has(k)) return def;
		std::string v = str(k);
		for(auto &ch : v) ch = (char) tolower(ch);
		return v == "1" || v == "true" || v == "yes" || v == "yup" || v == "of course";
	}

private:
	std::map<std::string, std::string> keys_;
};

// --------------------------------------------------------------- fields ---
struct Field {  // host mirror of one patch (BaseField's public state)
	rc_cell_host h;
	std::vector<double> phi;
	std::vector<int> map;
};

// ------------------------------------------------------------- backend ---
class FD_CUDABackend {
public:
	~FD_CUDABackend() {
		if(engine_) rc_destroy(engine_);
	}

	void get_settings(const InputFile &inp) {
		std::string backend = inp.str("backend", "", true);
		if(backend != "CUDA" && backend != "CPU")
			throw RCexception("Backend '" + backend + "' not supported");
		std::string sim_type = inp.str("sim_type", "FD_CPU");
		if(sim_type != "FD_CPU" && sim_type != "FD_CH")
			throw RCexception("sim_type '" + sim_type + "' is not provided by the GB300 engine");
		params_.conserved = sim_type == "FD_CH" ? 1 : 0;
		std::string prec = inp.str("backend_precision", "double");
		if(prec == "double") params_.precision = RC_PRECISION_DOUBLE;
		else if(prec == "mixed") params_.precision = RC_PRECISION_MIXED;
		else if(prec == "float") params_.precision = RC_PRECISION_FLOAT;
		else throw RCexception("Backend precision '" + prec + "' is not allowed");
		cell_tile_ = inp.integer("cell_tile", 0);
		if(cell_tile_ != 0 && cell_tile_ != 128 && cell_tile_ != 256 && cell_tile_ != 512)
			throw RCexception("cell_tile must be 128, 256 or 512");
		if(inp.str("box", "square") != "square") throw RCexception("only the periodic square box is provided");
		if(inp.integer("external_forces", 0) != 0) throw RCexception("external forces are not provided");
		// wall boxes run through the library (rc_box.walls) from the reference's
		// own rheoCell with backend = CUDA; this driver runs the periodic box
		if(inp.str("type", "none").find("walls") != std::string::npos || (inp.has("wall_slip") && inp.num("wall_slip") <= 0))
			throw RCexception("wall boxes are run by the reference's rheoCell with backend = CUDA, not by this driver");
		params_.wall_slip = inp.has("wall_slip") ? inp.num("wall_slip") : 0.5;
		if(inp.boolean("anchoring")) throw RCexception("anchoring is not provided");

		interaction_ = inp.str("interaction_type", "", true);
		struct D {
			double gamma, lambda, omega, mu, kappa;
		} d;
		if(interaction_ == "simplefield") {
			params_.model = RC_SIMPLEFIELD;
			d = {0.01, 2.5, 0.0, 3.0, 0.1};
		}
		else if(interaction_ == "activenematic") {
			params_.model = RC_ACTIVENEMATIC;
			d = {0.01, 2.5, 0.004, 3.0, 0.1};
		}
		else if(interaction_ == "wetpolarmodel") {
			params_.model = RC_WETPOLARMODEL;
			d = {0.06, 2.5, 0.004, 20.0, 0.1};
		}
		else if(interaction_ == "wetmodel") {
			params_.model = RC_WETMODEL;
			d = {0.01, 2.5, 0.004, 3.0, 0.1};
		}
		else throw RCexception("interaction_type '" + interaction_ + "' is not provided by the GB300 engine");
		params_.R = (int) inp.integer("R", 8, true);
		params_.border = 4;
		params_.dt = inp.num("dt", 0, true);
		params_.J0 = inp.num("J0", 1.0);
		params_.gamma = inp.num("gamma", d.gamma);
		params_.lambda = interaction_ == "simplefield" ? d.lambda : inp.num("lambda", d.lambda);
		params_.omega = inp.num("omega", d.omega);
		params_.mu = inp.num("mu", d.mu);
		params_.kappa = inp.num("kappa", d.kappa);
		const bool wet = params_.model == RC_WETMODEL || params_.model == RC_WETPOLARMODEL;
		params_.passive_alpha = wet ? inp.num("passive_alpha", 1.0) : 1.0;
		params_.cg_tolerance = wet ? inp.num("CGtolerance", 0.0001) : 0.0;
		params_.cg_restart_every = params_.model == RC_WETPOLARMODEL ? 10 : 100;
		auto both = [](double *a, double p, double q) {
			a[0] = p;
			a[1] = q;
		};
		if(params_.model == RC_SIMPLEFIELD) {
			both(params_.friction, 1, 1);
		}
		else if(params_.model == RC_ACTIVENEMATIC) {
			double fr = inp.num("friction", 2.0);
			both(params_.friction, fr, fr);
			both(params_.zetaQ_self, 0, inp.num("zetaQ_self", 0, true));
			both(params_.zetaQ_inter, 0, inp.num("zetaQ_inter", 0, true));
			both(params_.J_Q, 0, inp.num("J_Q", 0, true));
		}
		else {
			both(params_.friction, 1.0, inp.num("friction", 0, true));
			both(params_.friction_cell, 0.0, inp.num("friction_cell", 0, true));
			both(params_.zetaQ_self, 0, inp.num("zetaQ_self", 0, true));
			both(params_.zetaQ_inter, 0, inp.num("zetaQ_inter", 0, true));
			both(params_.J_Q, 0, inp.num("J_Q", 0, true));
			if(params_.model == RC_WETPOLARMODEL) both(params_.beta, 0, inp.num("beta", 0, true));
		}
		topology_ = inp.str("topology", "", true);
		conf_file_ = inp.str("conf_file", "", true);
		if(inp.integer("confs_to_skip", 0) != 0) throw RCexception("confs_to_skip is not provided");
		restart_step_counter_ = inp.boolean("restart_step_counter", false);
		device_ = (int) inp.integer("CUDA_device", 0);
		const std::string solver = inp.str("cg_solver", "plain");
		if(solver != "plain" && solver != "learned") throw RCexception("cg_solver '" + solver + "' is not provided");
		learned_ = solver == "learned";
		if(learned_ && !wet) throw RCexception("cg_solver = learned needs a wet model (friction_cell != 0)");
		harvest_steps_ = inp.integer("learned_harvest_steps", 40);
		train_epochs_ = (int) inp.integer("learned_train_epochs", 20);
		params_file_ = inp.str("learned_params_file", "");
	}

	bool learned() const { return learned_; }
	long long harvest_steps() const { return harvest_steps_; }

	// Learned solver: parameters from learned_params_file when it exists,
	// otherwise harvesting during the first learned_harvest_steps steps.
	// Returns true when harvesting was started.
	bool start_learned() {
		if(!params_file_.empty()) {
			std::ifstream f(params_file_);
			if(f.good()) {
				std::vector<double> p(RC_UNET_PARAMS);
				for(auto &v : p)
					if(!(f >> v)) throw RCexception("learned_params_file " + params_file_ + ": too few values");
				check(rc_learned_set_params(engine_, p.data()));
				check(rc_set_solver(engine_, RC_SOLVER_LEARNED));
				fprintf(stderr, "INFO: learned preconditioner parameters read from %s\n", params_file_.c_str());
				return false;
			}
		}
		check(rc_learned_harvest(engine_, 4000, 3, 6));
		return true;
	}

	void finish_learned() {
		rc_train_options o = {};
		o.epochs = train_epochs_;
		o.batch = 8;
		o.learning_rate = 2e-3;
		o.learning_rate_final = 1e-4;
		o.validation = 0.1;
		o.seed = 1;
		o.init = 1;
		rc_train_report r = {};
		check(rc_learned_train(engine_, &o, &r));
		check(rc_learned_harvest(engine_, 0, 0, 0));
		check(rc_set_solver(engine_, RC_SOLVER_LEARNED));
		fprintf(stderr, "INFO: learned preconditioner trained on %d samples in %.1f s, validation loss %.4g -> %.4g\n",
		        r.samples, r.ms * 1e-3, r.validation_loss_init, r.validation_loss);
		if(!params_file_.empty()) {
			std::vector<double> p(RC_UNET_PARAMS);
			check(rc_learned_get_params(engine_, p.data()));
			std::ofstream f(params_file_);
			f.precision(17);
			for(double v : p) f << v << "\n";
		}
	}

	// SimBackend::init + FD_CPUBackend::init
	void init() {
		read_topology();
		read_configuration();
		params_.rng_state = 0;
		// drand48's state after the draws above, carried to the device stream
		unsigned short probe[3];
		unsigned short *cur = seed48(probe);  // returns the previous state, sets probe
		memcpy(probe, cur, sizeof(probe));
		seed48(probe);                        // restore it
		params_.rng_state = (unsigned long long) probe[0] | ((unsigned long long) probe[1] << 16) |
		                    ((unsigned long long) probe[2] << 32);
		params_.rng_has_cached = 0;
		params_.rng_cached = 0;
		rc_box box = {L_, L_};
		std::vector<rc_cell_host> hc;
		for(auto &f : fields_) hc.push_back(f.h);
		int rc = rc_create(&params_, &box, (int) hc.size(), hc.data(), device_, &engine_);
		if(rc) throw RCexception(std::string("GB300 engine: ") + rc_last_error(engine_));
		if(cell_tile_) check(rc_set_cell_threads(engine_, cell_tile_));
	}

	void sim_step() { check(rc_step(engine_, 1, &stats_)); }
	void sim_steps(int n) { check(rc_step(engine_, n, &stats_)); }
	void apply_simulation_changes_after_equilibration() { check(rc_set_phase(engine_, 1)); }

	// device state -> host mirrors (SimBackend::apply_simulation_data_changes)
	void apply_simulation_data_changes() {
		std::vector<int> lx(fields_.size()), ly(fields_.size());
		check(rc_get_sizes(engine_, nullptr, lx.data(), ly.data()));
		std::vector<rc_cell_host> hc(fields_.size());
		for(size_t i = 0; i < fields_.size(); i++) {
			Field &f = fields_[i];
			const size_t n = (size_t) lx[i] * ly[i];
			f.phi.resize(n);
			f.map.resize(n);
			memset(&hc[i], 0, sizeof(rc_cell_host));
			hc[i].capacity = (int) n;
			hc[i].phi = f.phi.data();
			hc[i].box_index = f.map.data();
		}
		check(rc_download(engine_, hc.data(), RC_FIELD_SCALARS | RC_FIELD_PHI | RC_FIELD_MAP));
		for(size_t i = 0; i < fields_.size(); i++) {
			hc[i].phi = fields_[i].phi.data();
			hc[i].box_index = fields_[i].map.data();
			fields_[i].h = hc[i];
		}
	}

	// host snapshot of the configuration (Configuration::headers/field)
	struct Snapshot {
		long long step;
		int L;
		std::vector<rc_cell_host> h;
		std::vector<std::vector<double>> phi;
		std::vector<std::vector<int>> map;
	};

	Snapshot snapshot(long long step) const {
		Snapshot sn;
		sn.step = step;
		sn.L = L_;
		for(const auto &f : fields_) {
			sn.h.push_back(f.h);
			sn.phi.push_back(f.phi);
			sn.map.push_back(f.map);
		}
		return sn;
	}

	static std::string format(const Snapshot &sn) {
		std::stringstream conf;
		conf.precision(15);
		conf << "t = " << sn.step << std::endl;
		conf << "b = " << sn.L << " " << sn.L << std::endl;
		for(size_t i = 0; i < sn.h.size(); i++) {
			const rc_cell_host &h = sn.h[i];
			if(i > 0) conf << std::endl;
			conf << h.lsub_x << " " << h.lsub_y << " " << h.com_x << " " << h.com_y << " " << h.offset_x << " "
			     << h.offset_y << " " << h.corner << " " << h.unrap_x << " " << h.unrap_y << " " << h.q00 << " "
			     << h.q01 << " ";
			for(size_t q = 0; q < sn.phi[i].size(); q++) conf << sn.map[i][q] << " " << sn.phi[i][q] << " ";
		}
		conf << std::endl;
		return conf.str();
	}

	std::string configuration(long long step) const { return format(snapshot(step)); }

	long long start_step() const { return restart_step_counter_ ? 0 : conf_step_; }
	const rc_step_stats &stats() const { return stats_; }

private:
	void check(int rc) {
		if(rc) throw RCexception(std::string("GB300 engine: ") + rc_last_error(engine_));
	}

	void read_topology() {
		std::ifstream t(topology_);
		if(!t.good()) throw RCexception("Can't read topology file '" + topology_ + "'. Aborting");
		int n = 0;
		t >> n;
		std::string rest;
		std::getline(t, rest);
		std::string line2;
		std::getline(t, line2);
		std::stringstream ss(line2);
		types_.assign((size_t) n, 0);
		for(int i = 0; i < n && (ss >> types_[(size_t) i]); i++) {
		}
		fields_.resize((size_t) n);
		if(params_.model == RC_WETPOLARMODEL)
			for(int i = 0; i < n; i++) (void) drand48();  // run_clock draw of read_topology
	}

	void read_configuration() {
		std::ifstream c(conf_file_);
		if(!c.good()) throw RCexception("Can't read configuration file '" + conf_file_ + "'");
		std::string line;
		std::getline(c, line);
		if(sscanf(line.c_str(), "t = %lld", &conf_step_) != 1) throw RCexception("Malformed headers found in an input configuration");
		std::getline(c, line);
		double Lx = 0, Ly = 0;
		if(sscanf(line.c_str(), "b = %lf %lf", &Lx, &Ly) != 2) throw RCexception("Malformed headers found in an input configuration");
		if(Lx != Ly) throw RCexception("The box in the configuration file is not a square");
		L_ = (int) Lx;
		size_t i = 0;
		while(i < fields_.size() && std::getline(c, line)) {
			std::vector<double> v;
			const char *p = line.c_str();
			char *end = nullptr;
			for(;;) {
				double x = strtod(p, &end);
				if(end == p) break;
				v.push_back(x);
				p = end;
			}
			if(v.size() < 11) continue;
			Field &f = fields_[i];
			rc_cell_host &h = f.h;
			memset(&h, 0, sizeof(h));
			// MultiPhaseField::init(Lx, Ly): one draw seeds the nematic director
			double theta = (double) PI_F * (1 - 2 * drand48());
			double q00 = cos(2 * theta), q01 = sin(2 * theta);
			double mod = sqrt(q00 * q00 + q01 * q01);
			double sgn = q01 > 0 ? 1 : (q01 < 0 ? -1 : 0);
			h.nemq_x = h.nemq_old_x = sqrt((1 + q00 / mod) / 2);
			h.nemq_y = h.nemq_old_y = sgn * sqrt((1 - q00 / mod) / 2);
			h.lsub_x = (int) v[0];
			h.lsub_y = (int) v[1];
			h.com_x = v[2];
			h.com_y = v[3];
			h.offset_x = (int) v[4];
			h.offset_y = (int) v[5];
			h.corner = (int) v[6];
			h.unrap_x = (int) v[7];
			h.unrap_y = (int) v[8];
			h.q00 = v[9];
			h.q01 = v[10];
			h.theta_q = h.theta_q_old = 0.5 * atan2(2 * h.q01, 2 * h.q00);
			h.type = types_[i];
			const size_t n = (size_t) h.lsub_x * h.lsub_y;
			if(v.size() < 11 + 2 * n) throw RCexception("configuration line too short");
			f.phi.resize(n);
			f.map.resize(n);
			for(size_t q = 0; q < n; q++) {
				f.map[q] = (int) v[11 + 2 * q];
				f.phi[q] = v[11 + 2 * q + 1];
			}
			h.capacity = (int) n;
			h.phi = f.phi.data();
			i++;
		}
		if(i != fields_.size())
			throw RCexception("The number of lines found in configuration file doesn't match the parsed number of particles");
	}

	rc_params params_ = {};
	rc_engine *engine_ = nullptr;
	rc_step_stats stats_ = {};
	std::string interaction_, topology_, conf_file_;
	std::vector<int> types_;
	std::vector<Field> fields_;
	int L_ = 0;
	long long conf_step_ = 0;
	bool restart_step_counter_ = false;
	int device_ = 0;
	int cell_tile_ = 0;  // FP32 cell kernel tile (patch sites per CTA); 0: the engine's default
	bool learned_ = false;
	long long harvest_steps_ = 40;
	int train_epochs_ = 20;
	std::string params_file_;
};

void write_file(const std::string &path, const std::string &text, bool append) {
	std::ofstream f(path, append ? std::ios::app : std::ios::trunc);
	if(!f.good()) throw RCexception("Stream " + path + " not writable");
	f << text;
}

// Formats and writes configuration snapshots in order on its own thread
// (trajectory appended, last_conf overwritten); at most two snapshots wait.
class ConfWriter {
public:
	ConfWriter(std::string traj, std::string last) : traj_(std::move(traj)), last_(std::move(last)) {
		th_ = std::thread([this] { run(); });
	}
	~ConfWriter() { close(); }

	void push(FD_CUDABackend::Snapshot &&sn) {
		std::unique_lock<std::mutex> lk(mu_);
		cv_.wait(lk, [this] { return q_.size() < 2 || !err_.empty(); });
		if(!err_.empty()) throw RCexception(err_);
		q_.push_back(std::move(sn));
		cv_.notify_all();
	}

	// waits for the queue to drain; rethrows a writer error
	void close() {
		{
			std::unique_lock<std::mutex> lk(mu_);
			done_ = true;
			cv_.notify_all();
		}
		if(th_.joinable()) th_.join();
		if(!err_.empty()) {
			std::string e = err_;
			err_.clear();
			throw RCexception(e);
		}
	}

	long long bytes() const { return bytes_.load(); }

private:
	void run() {
		while(true) {
			FD_CUDABackend::Snapshot sn;
			{
				std::unique_lock<std::mutex> lk(mu_);
				cv_.wait(lk, [this] { return !q_.empty() || done_; });
				if(q_.empty()) return;
				sn = std::move(q_.front());
				q_.pop_front();
				cv_.notify_all();
			}
			try {
				const std::string c = FD_CUDABackend::format(sn);
				write_file(traj_, c, true);
				write_file(last_, c, false);
				bytes_ += (long long) c.size();
			}
			catch(std::exception &e) {
				std::unique_lock<std::mutex> lk(mu_);
				err_ = e.what();
				cv_.notify_all();
				return;
			}
		}
	}

	std::string traj_, last_;
	std::thread th_;
	std::mutex mu_;
	std::condition_variable cv_;
	std::deque<FD_CUDABackend::Snapshot> q_;
	bool done_ = false;
	std::string err_;
	std::atomic<long long> bytes_{0};
};

}  // namespace

int main(int argc, char *argv[]) {
	try {
		if(argc < 2) throw RCexception(std::string("Usage is '") + argv[0] + " input_file'");
		InputFile input;
		input.load(argv[1]);
		for(int i = 2; i < argc; i++) input.add_line(argv[i]);

		// SimManager::load_options
		const long long steps = input.integer("steps", 0, true);
		const long long eq_steps = input.integer("equilibration_steps", 0);
		if(!input.boolean("restart_step_counter") && eq_steps > 0)
			throw RCexception("if equilibration_steps > 0, restart_step_counter must be set to true");
		if(eq_steps < 0) throw RCexception("Equilibration steps can not be < 0. Aborting");
		if(!input.has("seed")) throw RCexception("seed must be given (the GB300 driver does not draw one)");
		const int seed = (int) input.integer("seed");
		const std::string ts = input.str("time_scale", "", true);
		if(ts != "linear") throw RCexception("Time scale '" + ts + "' not supported");
		const long long interval = input.integer("print_conf_interval", 0, true);
		const std::string traj = input.str("trajectory_file", "", true);
		const std::string last_conf = input.str("lastconf_file", "last_conf.dat");
		const std::string eq_conf = input.str("equilibratedconf_file", "equilibrated_conf.dat");
		double max_io = 1.0;  // MB/s, the reference's default
		if(input.has("max_io")) {
			max_io = input.num("max_io");
			if(max_io < 0) throw RCexception("Cannot run with a negative I/O limit. Set the max_io key to something > 0");
		}

		// SimManager::init
		srand48(seed);
		FD_CUDABackend backend;
		backend.get_settings(input);
		signal(SIGTERM, on_signal);
		signal(SIGINT, on_signal);
		signal(SIGUSR2, on_signal);
		backend.init();
		long long cur = backend.start_step();
		long long next_print = cur + interval - (cur % interval);
		write_file(traj, "", false);

		// SimManager::run
		for(long long s = 0; s < eq_steps && !g_stop; s++) backend.sim_step();
		backend.apply_simulation_data_changes();
		write_file(eq_conf, backend.configuration(cur), false);
		backend.apply_simulation_changes_after_equilibration();
		long long learn_at = -1;  // main-loop step at which the network is trained
		if(backend.learned() && backend.start_learned()) learn_at = backend.harvest_steps();
		const auto t_start = std::chrono::steady_clock::now();
		ConfWriter writer(traj, last_conf);
		auto print = [&]() {
			backend.apply_simulation_data_changes();
			writer.push(backend.snapshot(cur));
			// SimBackend::print_observables: data-rate limit after 30 s
			const double t = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
			if(t > 30) {
				const double MBps = ((double) writer.bytes() / (1024. * 1024.)) / t;
				if(MBps > max_io) {
					char msg[512];
					snprintf(msg, sizeof(msg),
					         "Aborting because the program is generating too much data (%g MB/s).\n\t\t\tThe current "
					         "limit is set to %g MB/s;\n\t\t\tyou can change it by setting max_io=<float> in the input "
					         "file.",
					         MBps, max_io);
					throw RCexception(msg);
				}
			}
		};
		long long run = 0;
		while(run < steps && !g_stop) {
			if(cur == next_print) {
				if(run > 0) print();
				next_print += interval;
			}
			// advance to the next print point (or the training point) in one call
			long long chunk = std::min(steps - run, next_print - cur);
			if(learn_at > run) chunk = std::min(chunk, learn_at - run);
			if(chunk < 1) chunk = 1;
			backend.sim_steps((int) chunk);
			cur += chunk;
			run += chunk;
			if(run == learn_at) backend.finish_learned();
		}
		if(cur == next_print && run > 0) print();
		writer.close();
		backend.apply_simulation_data_changes();
		write_file(last_conf, backend.configuration(cur), false);
		fprintf(stderr, "INFO: END OF THE SIMULATION, everything went OK! (%lld steps)\n", run);
	}
	catch(std::exception &e) {
		fprintf(stderr, "ERROR: %s\n", e.what());
		return 1;
	}
	return 0;
}
