// confgenerator -- initial configurations in the reference's format, a
// drop-in for the reference's `confGenerator input [side|density|NNxNN]`
// (src/confGenerator.cpp:9-42).
//
// Mirrored from the reference (paths relative to its src/):
//   GeneratorManager::GeneratorManager/load_options/init/generate
//                              Managers/GeneratorManager.cpp:6-158
//   random / lattice / cluster placement
//                              Interactions/BaseInteraction.cpp:102-294
//   MultiPhaseField::init() (30x30 patch, disc of radius R/2, nematic angle)
//                              Fields/MultiPhaseField.cpp:110-158
//   set_positions_initial      Fields/MultiPhaseField.cpp:211-221
//   drand48 order: srand48(seed); wetpolarmodel's read_topology draws one per
//   cell (WetPolarModel.cpp:191); placement draws; one per cell in init().
// With the default keys the output file is byte-identical to the
// reference's.  Extra keys (not read by the reference) produce the benchmark
// initial conditions instead: `patch_size = 41`, `profile = tanh`,
// `tanh_width` (default 2) and `tanh_radius` (default R) give
// phi = (1 - tanh((|x - CoM| - radius) / width)) / 2 on the patch.
#include <cmath>
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

namespace {

const float PI_F = 3.141592653589793238462643f;

struct Error : std::runtime_error {
	using std::runtime_error::runtime_error;
};

std::string trim(const std::string &s) {
	size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
	return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

struct Input {
	std::map<std::string, std::string> kv;
	void add(std::string line) {
		size_t c = line.find('#');
		if(c != std::string::npos) line.erase(c);
		size_t e = line.find('=');
		if(e == std::string::npos) return;
		std::string k = trim(line.substr(0, e));
		if(!k.empty()) kv[k] = trim(line.substr(e + 1));
	}
	bool has(const std::string &k) const { return kv.count(k) > 0; }
	std::string str(const std::string &k, const std::string &d = "", bool req = false) const {
		auto it = kv.find(k);
		if(it == kv.end()) {
			if(req) throw Error("Mandatory key `" + k + "' not found");
			return d;
		}
		return it->second;
	}
	double num(const std::string &k, double d) const { return has(k) ? std::stod(str(k)) : d; }
	int integer(const std::string &k, int d, bool req = false) const {
		if(!has(k)) {
			if(req) throw Error("Mandatory key `" + k + "' not found");
			return d;
		}
		return (int) std::lround(std::stod(str(k)));
	}
};

struct Box {
	int side;
	int x(int site, int d) const {
		int v = (site - (site / side) * side) + d;
		while(v < 0) v += side;
		while(v >= side) v -= side;
		return v;
	}
	int y(int site, int d) const {
		int v = site / side + d;
		while(v < 0) v += side;
		while(v >= side) v -= side;
		return v;
	}
	int el(int site, int dx, int dy) const { return x(site, dx) + y(site, dy) * side; }
	double sqr_min_image(const double *a, const double *b) const {
		double dx = b[0] - a[0] - rint((b[0] - a[0]) / side) * side;
		double dy = b[1] - a[1] - rint((b[1] - a[1]) / side) * side;
		return dx * dx + dy * dy;
	}
};

struct Cell {
	int lx = 30, ly = 30;
	double com[2] = {0, 0};
	int corner = 0;
	double unrap[2] = {0, 0};
	double q00 = 0, q01 = 0;
	std::vector<double> phi;
	void set_positions_initial(const Box &b) {
		int xx = (int) com[0], yy = (int) com[1];
		int site = xx + yy * b.side;
		xx = b.x(site, (int) -lx / 2);
		yy = b.y(site, (int) -ly / 2);
		corner = xx + yy * b.side;
		unrap[0] = xx;
		unrap[1] = yy;
	}
	int sub_index(const Box &b, int q) const { return b.el(corner, q % lx, q / lx); }
};

}  // namespace

int main(int argc, char *argv[]) {
	try {
		if(argc < 3) throw Error(std::string("Usage is '") + argv[0] + " input_file [box_size|density]'");
		Input in;
		{
			std::ifstream f(argv[1]);
			if(!f.good()) throw Error(std::string("Input file '") + argv[1] + "' not found");
			std::string line;
			while(std::getline(f, line)) in.add(line);
			for(int i = 3; i < argc; i++) in.add(argv[i]);
		}
		// third argument: side, density (< 2) or NNxNN
		std::string third = argv[2];
		bool use_density = false;
		double density = -1, side_x = -1, side_y = -1;
		if(third.find('x') != std::string::npos) {
			side_x = atof(third.substr(0, third.find('x')).c_str());
			side_y = atof(third.substr(third.find('x') + 1).c_str());
		}
		else {
			double v = atof(third.c_str());
			if(v <= 0.) throw Error("Refusing to run with box_side/density = " + third);
			if(v < 2.) {
				use_density = true;
				density = v;
			}
			else side_x = side_y = v;
		}
		in.str("trajectory_file", "", true);
		const std::string out_conf = in.str("conf_file", "", true);
		const std::string type = in.str("initial_configuration_type", "random");
		int n_rows = 0, n_columns = 0;
		if(type == "lattice") {
			n_rows = in.integer("n_rows", 0, true);
			n_columns = in.integer("n_columns", 0, true);
		}
		if(!in.has("seed")) throw Error("seed must be given (the GB300 generator does not draw one)");
		srand48((long int) in.integer("seed", 0));
		const std::string interaction = in.str("interaction_type", "", true);
		const int R = in.integer("R", 8, true);
		// topology: N, and wetpolarmodel's one draw per cell in read_topology
		int N = 0;
		{
			std::ifstream t(in.str("topology", "", true));
			if(!t.good()) throw Error("Can't read topology file");
			t >> N;
		}
		if(interaction == "wetpolarmodel")
			for(int i = 0; i < N; i++) (void) drand48();
		if(use_density) side_x = side_y = pow(N / density, 1. / 2.);
		if((int) side_x != (int) side_y) throw Error("The box in the configuration file is not a square");
		Box box{(int) side_x};

		const int patch = in.integer("patch_size", 30);
		const bool tanh_profile = in.str("profile", "disc") == "tanh";
		const double width = in.num("tanh_width", 2.0), radius = in.num("tanh_radius", (double) R);
		std::vector<Cell> cells((size_t) N);
		for(auto &c : cells) {
			c.lx = c.ly = patch;
		}
		auto overlap = [&](const Cell &p, const Cell &q, double sqr_rcut) {
			return !(box.sqr_min_image(p.com, q.com) >= 2. * sqr_rcut);
		};
		if(type == "lattice") {
			const double a = 2 * R - 2, b = 2 * R - 2;
			const double theta = 60.0 * M_PI / 180.0;
			const double ax = a, ay = 0, bx = b * cos(theta), by = b * sin(theta);
			const double cx = box.side / 2.0, cy = box.side / 2.0;
			const double sx = cx - 0.5 * ((n_columns - 1) * ax + (n_rows - 1) * bx);
			const double sy = cy - 0.5 * ((n_columns - 1) * ay + (n_rows - 1) * by);
			int placed = 0;
			for(int r = 0; r < n_rows && placed < N; ++r)
				for(int c = 0; c < n_columns && placed < N; ++c) {
					Cell &p = cells[(size_t) placed++];
					p.com[0] = sx + c * ax + r * bx + 0.0;
					p.com[1] = sy + c * ay + r * by + 0.0;
					p.set_positions_initial(box);
				}
		}
		else {
			const bool cluster = type == "cluster";
			for(auto &p : cells) {
				p.com[0] = drand48() * box.side;
				p.com[1] = drand48() * box.side;
			}
			const double rcut = cluster ? (double) R - 1 : (double) R - 3;
			const double sqr_rcut = rcut * rcut;
			const double cluster_radius = R * R * N;
			const double ref[2] = {box.side / 2., box.side / 2.};
			for(int i = 0; i < N; i++) {
				Cell &p = cells[(size_t) i];
				bool inserted = false;
				long long attempts = 0;
				do {
					p.com[0] = drand48() * box.side;
					p.com[1] = drand48() * box.side;
					p.set_positions_initial(box);
					inserted = true;
					if(cluster && box.sqr_min_image(p.com, ref) > cluster_radius) inserted = false;
					for(int n = 0; n < i; n++)
						if(overlap(p, cells[(size_t) n], sqr_rcut)) inserted = false;
					if(++attempts > 100000000LL) throw Error("could not place all cells");
				} while(!inserted);
			}
		}
		// MultiPhaseField::init() and set_positions_initial per cell
		const int init_radius = R / 2, init_radius2 = init_radius * init_radius;
		for(auto &p : cells) {
			const int n = p.lx * p.ly;
			double theta = (double) PI_F * (1 - 2 * drand48());
			p.q00 = cos(2 * theta);
			p.q01 = sin(2 * theta);
			p.phi.assign((size_t) n, 0.0);
			const double fx = p.com[0] - (int) p.com[0], fy = p.com[1] - (int) p.com[1];
			for(int i = 0; i < n; i++) {
				if(tanh_profile) {
					const double dx = (i % p.lx) - p.lx / 2 - fx, dy = (i / p.lx) - p.ly / 2 - fy;
					p.phi[(size_t) i] = 0.5 * (1 - tanh((sqrt(dx * dx + dy * dy) - radius) / width));
				}
				else {
					const int y = p.ly / 2 - i / p.lx;
					const int x = p.lx / 2 - (i - (i / p.lx) * p.lx);
					p.phi[(size_t) i] = (x * x + y * y < init_radius2 + 0.5) ? 1. : 0.;
				}
			}
			p.set_positions_initial(box);
		}
		std::ofstream conf(out_conf);
		if(!conf.good()) throw Error("cannot write " + out_conf);
		conf.precision(15);
		conf << "t = 0" << std::endl;
		conf << "b = " << side_x << " " << side_y << std::endl;
		for(const auto &p : cells) {
			conf << p.lx << " " << p.ly << " " << p.com[0] << " " << p.com[1] << " " << 0 << " " << 0 << " " << p.corner
			     << " " << p.unrap[0] << " " << p.unrap[1] << " " << p.q00 << " " << p.q01 << " ";
			for(int q = 0; q < p.lx * p.ly; q++) conf << p.sub_index(box, q) << " " << p.phi[(size_t) q] << " ";
			conf << std::endl;
		}
	}
	catch(std::exception &e) {
		fprintf(stderr, "ERROR: %s\n", e.what());
		return 1;
	}
	return 0;
}
