// driver.cpp — ch_<DIM>D, the reference's command-line program running the
// GB300 engine: `ch_2D input.toml`.
//
// It reads the reference's TOML keys, builds the model and the initial
// density, and runs the output cadence and file formats of src/main.cpp:20-200
// and src/utils/Printer.cpp (init_/last_ snapshots, traj_ appends, energy.dat
// and the same line on stdout), with every time step executed by libchgb on
// the GPU (include/chgb.h).  Consecutive steps between two outputs are queued
// as one chgb_step call.  Observables are reduced on the device
// (chgb_observables).  Log messages go to stderr; stdout carries only the
// energy lines.
//
// Deliberate differences from the reference:
// * `use_CUDA` is read and ignored: every step runs on the GPU.
// * The `bailo` integrator and the ricci/generic Wertheim models are outside
//   this engine and stop with a message.
// * `output.print_pressure` follows the reference (src/main.cpp:114-126,
//   140-162; src/utils/Printer.cpp:33-45,157-168), its quirks included: the
//   `pressure_<i>` trajectories hold the density (Printer::add_to_trajectory
//   writes the state's rho whatever field it is given), and the log cadence
//   fires once, at round(log_n0), because the printed count never advances.
// * `load_from_full_3d = true` (a key the reference does not have) reads all
//   N*N lines of a 3D configuration; by default the reference's behaviour of
//   reading N lines (src/CahnHilliard.cpp:87,124) is kept.
// * `output.full_precision = true` (a key the reference does not have) writes
//   the native init_/last_/traj_ files with 17 significant digits instead of
//   std::ostream's 6, so a `load_from` restart continues from the exact state
//   (bit-for-bit for the explicit integrators when distance_scaling_factor is
//   1); the default keeps the reference's 6-digit text.
#include <sys/stat.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include <chgb.h>

#include "toml_lite.h"

#ifndef DIM
#define DIM 2
#endif

namespace ch {

using tomllite::Table;
using tomllite::Value;

[[noreturn]] void critical(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::fprintf(stderr, "[critical] ");
    std::vfprintf(stderr, fmt, ap);
    std::fprintf(stderr, "\n");
    va_end(ap);
    std::exit(1);
}

void info(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::fprintf(stderr, "[info] ");
    std::vfprintf(stderr, fmt, ap);
    std::fprintf(stderr, "\n");
    va_end(ap);
}

// fmt's "{:.P}" of a double as the reference prints it: general format with
// trailing zeros kept (e.g. 0.0000, 11.100, 1.2346e+05).
std::string fmt_g(double v, int prec) {
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%#.*g", prec, v);
    return buf;
}

// std::ostream << double with the default precision.
std::string ostream_g(double v) {
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%g", v);
    return buf;
}

// Shortest form that reads back to the same double (17 significant digits).
std::string full_g(double v) {
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.17g", v);
    return buf;
}

bool is_dir(const std::string &p) {
    struct stat st;
    return stat(p.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

std::string join(const std::string &dir, const std::string &name) {
    if(dir.empty() || dir == ".") return name;
    return dir.back() == '/' ? dir + name : dir + "/" + name;
}

// The reference's TOML getters (src/Object.h:32-90).
struct Config {
    Table root;

    const Value *node(const std::string &path) const { return tomllite::find(root, path); }
    bool has(const std::string &path) const { return node(path) != nullptr; }

    double get_double(const std::string &path) const {
        const Value *v = node(path);
        if(!v) critical("Mandatory option '%s' not found", path.c_str());
        auto d = v->as_double();
        if(!d) critical("Option '%s' is not a number", path.c_str());
        return *d;
    }
    long long get_int(const std::string &path) const {
        const Value *v = node(path);
        if(!v) critical("Mandatory option '%s' not found", path.c_str());
        auto i = v->as_integer();
        if(!i) critical("Option '%s' is not an integer", path.c_str());
        return *i;
    }
    std::string get_string(const std::string &path) const {
        const Value *v = node(path);
        if(!v) critical("Mandatory option '%s' not found", path.c_str());
        auto s = v->as_string();
        if(!s) critical("Option '%s' is not a string", path.c_str());
        return *s;
    }
    double opt_double(const std::string &path, double def) const {
        const Value *v = node(path);
        if(!v) return def;
        return v->as_double().value_or(def);
    }
    long long opt_int(const std::string &path, long long def) const {
        const Value *v = node(path);
        if(!v) return def;
        return v->as_integer().value_or(def);
    }
    bool opt_bool(const std::string &path, bool def) const {
        const Value *v = node(path);
        if(!v) return def;
        return v->as_bool().value_or(def);
    }
    std::string opt_string(const std::string &path, const std::string &def) const {
        const Value *v = node(path);
        if(!v) return def;
        return v->as_string().value_or(def);
    }
    // _config_array_values: a scalar of the exact type broadcasts, else an array of that type
    std::vector<double> array_double(const std::string &path, size_t size) const {
        const Value *v = node(path);
        if(!v) critical("Mandatory option '%s' not found", path.c_str());
        std::vector<double> out;
        if(v->type == Value::FLOAT) out.assign(size, v->f);
        else if(v->type == Value::ARRAY) {
            for(auto &e : v->arr) {
                if(e.type != Value::FLOAT) critical("Option '%s': cannot convert element", path.c_str());
                out.push_back(e.f);
            }
        }
        if(out.size() != size)
            critical("Option '%s' should be a single value or an array of size %zu, not %zu", path.c_str(), size,
                     out.size());
        return out;
    }
    std::vector<long long> array_int(const std::string &path, size_t size) const {
        const Value *v = node(path);
        if(!v) critical("Mandatory option '%s' not found", path.c_str());
        std::vector<long long> out;
        if(v->type == Value::INTEGER) out.assign(size, v->i);
        else if(v->type == Value::ARRAY) {
            for(auto &e : v->arr) {
                if(e.type != Value::INTEGER) critical("Option '%s': cannot convert element", path.c_str());
                out.push_back(e.i);
            }
        }
        if(out.size() != size)
            critical("Option '%s' should be a single value or an array of size %zu, not %zu", path.c_str(), size,
                     out.size());
        return out;
    }
};

// Delta from a number or a {T, deltaH, deltaS, salt, sticky_size} table, src/utils/Delta.cpp:15-42.
double delta_value(const Config &cfg, const std::string &path) {
    const Value *v = cfg.node(path);
    if(!v) critical("Mandatory option '%s' not found", path.c_str());
    if(v->is_number()) return *v->as_double();
    if(v->type == Value::TABLE) {
        Config sub;
        sub.root = *v->tbl;
        double d = sub.opt_double("value", 0.0);
        if(d == 0.0) {
            double T = sub.get_double("T");
            double salt = sub.opt_double("salt", 1.0);
            long long L_DNA = sub.opt_int("sticky_size", 6);
            double dH = sub.get_double("deltaH");
            double dS = sub.get_double("deltaS");
            double dS_salt = 0.368 * (L_DNA - 1.0) * std::log(salt);
            double dG = dH - T * (dS + dS_salt);
            const double k_B = 1.9872036;
            d = 1.6606 * std::exp(-dG / (k_B * T));
        }
        return d;
    }
    critical("A delta must be specified either as a single number or as a table of values (%s)", path.c_str());
}

// POSIX drand48 (seeded as src/main.cpp:36).
struct Rand48 {
    unsigned long long x = 0x330E;
    void seed(long long s) { x = (((unsigned long long) s & 0xFFFFFFFFull) << 16) | 0x330Eull; }
    double next() {
        x = (0x5DEECE66Dull * x + 0xBull) & 0xFFFFFFFFFFFFull;
        return std::ldexp((double) x, -48);
    }
};

// Trajectory / snapshot writer, src/utils/Printer.cpp.
struct Printer {
    int N, S;
    double dt, dx, internal_to_user;
    std::string strategy;
    long long traj_every = 0, last_every = 0;
    int log_n0 = 0;
    double log_fact = 1.0;
    int traj_printed = 0;  // never advanced, as in the reference (Printer.h:72)
    bool print_vtk = false;
    bool full_precision = false;
    bool print_pressure = false;
    std::string pressure_strategy;
    long long pressure_every = 0;
    std::string out_path, traj_path;

    Printer(const Config &cfg, int species, bool loading) : S(species) {
        N = (int) cfg.get_int("N");
        dt = cfg.get_double("dt");
        dx = cfg.opt_double("dx", 1.0);
        strategy = cfg.opt_string("print_trajectory_strategy", "linear");
        if(strategy == "linear") {
            traj_every = cfg.opt_int("print_trajectory_every", 0);
            last_every = cfg.opt_int("print_last_every", traj_every);
        }
        else if(strategy == "log") {
            log_n0 = (int) cfg.get_int("output.log_n0");
            log_fact = cfg.get_double("output.log_fact");
            last_every = cfg.get_int("print_last_every");
        }
        else {
            critical("Unsupported trajectory printing strategy '%s'", strategy.c_str());
        }
        // src/utils/Printer.cpp:33-45
        print_pressure = cfg.opt_bool("output.print_pressure", false);
        if(print_pressure) {
            pressure_strategy = cfg.opt_string("output.print_pressure_strategy", "linear");
            if(pressure_strategy == "linear") {
                pressure_every = cfg.get_int("output.print_pressure_every");
            }
            else if(pressure_strategy == "log") {
                log_n0 = (int) cfg.get_int("output.log_n0");
                log_fact = cfg.get_double("output.log_fact");
            }
            else {
                critical("Unsupported pressure printing strategy '%s'", pressure_strategy.c_str());
            }
        }
        out_path = cfg.opt_string("output.path", ".");
        if(!is_dir(out_path)) critical("Output path '%s' does not exist or is not a directory", out_path.c_str());
        print_vtk = cfg.opt_bool("output.print_vtk", false);
        full_precision = cfg.opt_bool("output.full_precision", false);
        traj_path = print_vtk ? cfg.get_string("output.trajectory_path") : cfg.opt_string("output.trajectory_path", out_path);
        if(!is_dir(traj_path)) critical("Trajectory output path '%s' does not exist or is not a directory", traj_path.c_str());
        if(!print_vtk && !loading) {
            for(int i = 0; i < S; i++) {
                for(const char *prefix : {"mu", "pressure", "traj"}) {
                    std::ofstream(join(traj_path, std::string(prefix) + "_" + std::to_string(i) + ".dat"));
                }
            }
        }
    }

    bool should_print_last(long long t) const { return last_every > 0 && t % last_every == 0; }
    bool should_print_traj(long long t) const {
        if(strategy == "linear") return traj_every > 0 && t % traj_every == 0;
        long long next_t = (long long) std::round(log_n0 * std::pow(log_fact, traj_printed));
        return next_t == t;
    }
    bool should_print_pressure(long long t) const {
        if(!print_pressure) return false;
        if(pressure_strategy == "linear") return pressure_every > 0 && t % pressure_every == 0;
        long long next_t = (long long) std::round(log_n0 * std::pow(log_fact, traj_printed));
        return next_t == t;
    }

    void write_native(std::ostream &out, const std::vector<double> &rho, double factor, int species, long long t,
                      const char *obs = "density") const {
        int nx = N, ny = DIM >= 2 ? N : 1, nz = DIM >= 3 ? N : 1;
        size_t bins = (size_t) nx * ny * nz;
        out << "# step = " << t << ", t = " << fmt_g(t * dt, 5) << ", size = " << nx << "x" << ny << "x" << nz
            << " | " << obs << "\n";
        std::string line;
        for(size_t idx = 0; idx < bins; idx++) {
            if(idx > 0 && idx % ny == 0) {
                out << line << "\n";
                line.clear();
            }
            double v = 0.0;
            if(species == -1) {
                for(int s = 0; s < S; s++) v += rho[s * bins + idx];
            }
            else {
                v = rho[species * bins + idx];
            }
            line += full_precision ? full_g(v * factor) : ostream_g(v * factor);
            line += ' ';
        }
        out << line << "\n";
    }

    void write_vtk(const std::string &filename, const std::vector<double> &rho, double factor, int species,
                   long long t, const char *obs = "density") const {
        if(!print_vtk) return;
        if(DIM == 1) critical("VTK output is not supported for 1D simulations");
        std::ofstream out(filename);
        int nx = N, ny = DIM >= 2 ? N : 1, nz = DIM >= 3 ? N : 1;
        size_t bins = (size_t) nx * ny * nz;
        double s = dx * internal_to_user;
        out << "# vtk DataFile Version 3.0\n";
        out << "step = " << t << ", t = " << fmt_g(t * dt, 5) << ", size = " << nx << "x" << ny << "x" << nz
            << " | " << obs << "\n";
        out << "ASCII\nDATASET STRUCTURED_POINTS\n";
        out << "DIMENSIONS " << nx << " " << ny << " " << nz << "\n";
        out << "ORIGIN 0 0 0\n";
        out << "SPACING " << ostream_g(s) << " " << ostream_g(s) << " " << ostream_g(s) << "\n";
        out << "POINT_DATA " << bins << "\n";
        out << "SCALARS species_" << species << " double 1\n";
        out << "LOOKUP_TABLE default\n";
        char buf[64];
        for(size_t idx = 0; idx < bins; idx++) {
            double v = 0.0;
            if(species == -1) {
                for(int q = 0; q < S; q++) v += rho[q * bins + idx];
            }
            else {
                v = rho[species * bins + idx];
            }
            std::snprintf(buf, sizeof(buf), "%e\n", v * factor);
            out << buf;
        }
    }

    void print_current_state(const std::string &prefix, long long t, const std::vector<double> &rho, double factor) const {
        for(int i = 0; i < S; i++) {
            std::ofstream out(join(out_path, prefix + std::to_string(i) + ".dat"));
            write_native(out, rho, factor, i, t);
            write_vtk(join(out_path, prefix + std::to_string(i) + ".vtk"), rho, factor, i, t);
        }
        std::ofstream out(join(out_path, prefix + "density.dat"));
        write_native(out, rho, factor, -1, t);
        write_vtk(join(out_path, prefix + "density.vtk"), rho, factor, -1, t);
    }

    // `prefix` is "traj" (observable "density") or "pressure" (observable
    // "pressure"); the values written are the density in both cases, as in the
    // reference (src/utils/Printer.cpp:118-136 writes _sim_state.rho).
    void add_to_trajectory(const std::string &prefix, const char *obs, const std::vector<double> &rho, double factor,
                           int species, long long t) const {
        if(print_vtk) {
            write_vtk(join(traj_path, prefix + "_" + std::to_string(species) + "_" + std::to_string(t) + ".vtk"), rho,
                      factor, species, t, obs);
        }
        else {
            std::ofstream out(join(traj_path, prefix + "_" + std::to_string(species) + ".dat"), std::ios_base::app);
            write_native(out, rho, factor, species, t, obs);
        }
    }

    // The pressure snapshots of src/main.cpp:140-162: one file per species when
    // there are several, then the total.
    void print_pressure_state(const std::string &prefix, long long t, const std::vector<double> &p, double factor) const {
        if(S > 1) {
            for(int i = 0; i < S; i++) {
                std::ofstream out(join(out_path, prefix + std::to_string(i) + "_pressure.dat"));
                write_native(out, p, factor, i, t, "pressure");
                write_vtk(join(out_path, prefix + std::to_string(i) + "_pressure.vtk"), p, factor, i, t, "pressure");
            }
        }
        std::ofstream out(join(out_path, prefix + "pressure.dat"));
        write_native(out, p, factor, -1, t, "pressure");
        write_vtk(join(out_path, prefix + "pressure.vtk"), p, factor, -1, t, "pressure");
    }
};

void split_ws(const std::string &line, std::vector<std::string> &out) {
    out.clear();
    std::istringstream ss(line);
    std::string tok;
    while(ss >> tok) out.push_back(tok);
}

class Manager {
public:
    explicit Manager(const Config &cfg) : cfg_(cfg) {
        steps_ = cfg.get_int("steps");
        if(steps_ < 0) critical("steps should be a number larger than 0");
        internal_to_user_ = cfg.opt_double("distance_scaling_factor", 1.0);
        u_ = 1.0 / internal_to_user_;
        print_every_ = cfg.opt_int("print_every", 0);
        print_pressure_ = cfg.opt_bool("output.print_pressure", false);
        rng_.seed(cfg.opt_int("seed", (long long) std::time(nullptr)));
        output_path_ = cfg.opt_string("output_path", ".");
        if(!is_dir(output_path_)) critical("Output path '%s' does not exist or is not a directory", output_path_.c_str());

        build_model();
        build_system();
        loading_ = cfg.has("load_from");
        printer_ = new Printer(cfg, S_, loading_);
        printer_->internal_to_user = internal_to_user_;
        if(loading_) {
            std::ifstream in(cfg.get_string("load_from"));
            std::string line;
            std::getline(in, line);
            std::vector<std::string> spl;
            split_ws(line, spl);
            if(spl.size() > 3 && spl[0] == "#" && spl[1] == "step" && spl[2] == "=") {
                initial_t_ = std::stoll(spl[3]);
                info("Initial time step (as parsed from the 'load_from' file): %lld", initial_t_);
            }
            else {
                info("The header line of the 'load_from' file does not contain information about the time step");
            }
        }
    }

    ~Manager() {
        if(h_) chgb_destroy(h_);
        delete printer_;
    }

    // Parameters as handed to chgb_create, without touching the GPU.
    static void print_params(const Config &cfg) {
        Manager m(cfg, true);
        const chgb_params &p = m.params_;
        const chgb_model_params &q = p.model;
        std::printf("{\"dims\": %d, \"N\": %d, \"integrator\": %d, \"mobility_type\": %d, \"dt\": %.17g, "
                    "\"dx\": %.17g, \"k\": [%.17g, %.17g, %.17g], \"M\": %.17g, \"splitting_S\": %.17g, "
                    "\"use_dealias\": %d, \"kind\": %d, \"n_species\": %d, \"epsilon\": %.17g, \"valence\": %d, "
                    "\"saleh_valence\": [%d, %d, %d], \"B2\": %.17g, \"B3\": %.17g, \"delta\": %.17g, "
                    "\"regularisation_delta\": %.17g, \"delta_AA\": %.17g, \"delta_BB\": %.17g, "
                    "\"density_conversion_factor\": %.17g, \"steps\": %lld, \"rho_sum\": %.17g, "
                    "\"rho_min\": %.17g, \"gel\": [%.17g, %.17g, %.17g, %.17g]}\n",
                    p.dims, p.N, p.integrator, p.mobility_type, p.dt, p.dx, p.k[0], p.k[1], p.k[2], p.M,
                    p.splitting_S, p.use_dealias, q.kind, q.n_species, q.epsilon, q.valence, q.saleh_valence[0],
                    q.saleh_valence[1], q.saleh_valence[2], q.B2, q.B3, q.delta, q.regularisation_delta, q.delta_AA,
                    q.delta_BB, q.density_conversion_factor, m.steps_, m.rho_sum(), p.rho_min, p.gel_phi_critical,
                    p.gel_c0, p.gel_M_c, p.gel_beta_delta_F);
    }

private:
    Manager(const Config &cfg, bool dry) : cfg_(cfg), dry_(dry) {
        steps_ = cfg.get_int("steps");
        internal_to_user_ = cfg.opt_double("distance_scaling_factor", 1.0);
        u_ = 1.0 / internal_to_user_;
        rng_.seed(cfg.opt_int("seed", (long long) std::time(nullptr)));
        build_model();
        build_system();
    }

    double rho_sum() const {
        double s = 0.0;
        for(double r : rho_) s += r;
        return s;
    }

public:

    void run() {
        print_state("init_", 0);
        double rho_factor = u_ * u_ * u_;  // density_to_user(1.0)
        std::ofstream energy(join(output_path_, "energy.dat"), loading_ ? std::ios_base::app : std::ios_base::out);
        long long t = initial_t_;
        const long long end = initial_t_ + steps_;
        while(t < end) {
            if(printer_->should_print_last(t)) print_state("last_", t);
            if(printer_->should_print_traj(t)) {
                sync();
                for(int i = 0; i < S_; i++) printer_->add_to_trajectory("traj", "density", rho_, rho_factor, i, t);
            }
            if(printer_->should_print_pressure(t)) {
                // src/main.cpp:114-119: the pressure is computed, but the trajectory receives the density
                sync();
                for(int i = 0; i < S_; i++) printer_->add_to_trajectory("pressure", "pressure", rho_, rho_factor, i, t);
            }
            if(print_every_ > 0 && t % print_every_ == 0) {
                double mass = 0, fe = 0;
                int32_t nan = 0;
                int r = chgb_observables(h_, &mass, &fe, &nan);
                if(nan) critical("Encountered a nan while computing the total free energy or mass (step %lld)", t);
                if(r != CHGB_OK) critical("%s", chgb_last_error(h_));
                std::string line = fmt_g(t * dt_, 5) + " " + fmt_g(fe, 8) + " " + fmt_g(mass, 5) + " " +
                                   std::to_string(t);
                if(print_pressure_) line += " " + fmt_g(average_pressure(), 5);
                energy << line << std::endl;
                std::printf("%s\n", line.c_str());
                std::fflush(stdout);
            }
            // queue every step up to the next output event as one call
            long long next = t + 1;
            while(next < end && !event_at(next)) next++;
            step(next - t);
            t = next;
        }
        energy.close();
        print_state("last_", steps_);  // src/main.cpp:133 uses steps, not t0 + steps
    }

private:
    bool event_at(long long t) const {
        return printer_->should_print_last(t) || printer_->should_print_traj(t) ||
               printer_->should_print_pressure(t) || (print_every_ > 0 && t % print_every_ == 0);
    }

    // chgb_pressure; for a model without a pressure the reference stops in
    // FreeEnergyModel::pressure() (src/models/FreeEnergyModel.h:43-44).
    int pressure_status(double *field, double *avg) {
        int r = chgb_pressure(h_, field, avg);
        if(r == CHGB_ERR_UNSUPPORTED) critical("this model does not support the pressure coupling");
        if(r != CHGB_OK) critical("%s", chgb_last_error(h_));
        return r;
    }

    double average_pressure() {
        double avg = 0.0;
        pressure_status(nullptr, &avg);
        return avg;
    }

    void step(long long n) {
        if(chgb_step(h_, n) != CHGB_OK) critical("%s", chgb_last_error(h_));
        synced_ = false;
    }

    void sync() {
        if(synced_) return;
        if(chgb_download(h_, rho_.data(), nullptr) != CHGB_OK) critical("%s", chgb_last_error(h_));
        synced_ = true;
    }

    void print_state(const std::string &prefix, long long t) {
        sync();
        printer_->print_current_state(prefix, t, rho_, u_ * u_ * u_);
        if(print_pressure_) {
            pressure_.resize(rho_.size());
            pressure_status(pressure_.data(), nullptr);
            printer_->print_pressure_state(prefix, t, pressure_, u_ * u_ * u_);
        }
    }

    void build_model() {
        std::string name = cfg_.get_string("free_energy");
        chgb_model_params &m = params_.model;
        std::memset(&m, 0, sizeof(m));
        double u3 = u_ * u_ * u_;
        m.density_conversion_factor = u3;
        if(name == "landau") {
            // src/models/Landau.cpp:16-36
            m.kind = CHGB_MODEL_LANDAU;
            m.n_species = 1;
            if(cfg_.has("landau.epsilon")) m.epsilon = cfg_.get_double("landau.epsilon");
            else if(cfg_.has("landau.T")) m.epsilon = 1 - cfg_.get_double("landau.T");
            else critical("The Landau free energy requires either 'epsilon' or 'T' to be set");
            if(u_ != 1.0) critical("The Landau free energy does not support distance_scaling_factor values different from 1.0");
        }
        else if(name == "simple_wertheim") {
            // src/models/SimpleWertheim.cpp:20-34
            m.kind = CHGB_MODEL_SIMPLE_WERTHEIM;
            m.n_species = 1;
            m.valence = (int32_t) cfg_.get_int("wertheim.valence");
            m.B2 = cfg_.get_double("wertheim.B2") * u3;
            m.regularisation_delta = cfg_.opt_double("wertheim.regularisation_delta", 0.0) / u3;
            m.delta = delta_value(cfg_, "wertheim.delta") * u3;
        }
        else if(name == "saleh") {
            // src/models/SalehWertheim.cpp:19-41
            m.kind = CHGB_MODEL_SALEH;
            m.n_species = 3;
            m.B2 = cfg_.get_double("saleh.B2") * u3;
            m.B3 = cfg_.opt_double("saleh.B3", 0.0) * u3 * u3;
            m.delta_AA = delta_value(cfg_, "saleh.delta_AA") * u3;
            m.delta_BB = delta_value(cfg_, "saleh.delta_BB") * u3;
            auto v = cfg_.array_int("saleh.valence", 3);
            for(int i = 0; i < 3; i++) m.saleh_valence[i] = (int32_t) v[i];
        }
        else if(name == "generic_wertheim" || name == "ricci") {
            critical("The free energy model '%s' is not supported by the GB300 engine", name.c_str());
        }
        else {
            critical("Unsupported free energy model '%s'", name.c_str());
        }
        S_ = m.n_species;
    }

    void build_system() {
        // src/CahnHilliard.cpp:34-229
        int N = (int) cfg_.get_int("N");
        double l2 = std::log2((double) N);
        if(N <= 0 || std::ceil(l2) != std::floor(l2)) critical("N should be a power of 2");
        params_.dims = DIM;
        params_.N = N;
        auto k = cfg_.array_double("k", S_);
        dt_ = cfg_.get_double("dt");
        double dx = cfg_.opt_double("dx", 1.0);
        std::string integ = cfg_.opt_string("integrator", "euler");
        if(cfg_.opt_bool("use_CUDA", false) == false) info("use_CUDA = false: the GB300 engine runs every step on the GPU");

        size_t bins = 1;
        for(int d = 0; d < DIM; d++) bins *= N;
        rho_.assign(bins * S_, 0.0);
        if(!cfg_.has("initial_density") && !cfg_.has("load_from")) {
            critical("Either 'initial_density' or 'load_from' should be specified");
        }
        if(cfg_.has("load_from")) {
            load_from(cfg_.get_string("load_from"), N, bins);
        }
        else {
            auto densities = cfg_.array_double("initial_density", S_);
            double A = cfg_.opt_double("initial_A", 1e-2);
            long long peaks = cfg_.opt_int("initial_N_peaks", 0);
            double initial_k = 2 * M_PI * peaks / (double) N;
            for(size_t bin = 0; bin < bins; bin++) {
                double modulation = A * std::cos(initial_k * (double) bin);
                for(int i = 0; i < S_; i++) {
                    double rf = (peaks == 0) ? (rng_.next() - 0.5) : 1.0 + 0.02 * (rng_.next() - 0.5);
                    double avg = densities[i];
                    rho_[i * bins + bin] = (avg != 0.0) ? avg * (1.0 + 2.0 * modulation * rf) : 2.0 * modulation * rf;
                }
            }
        }
        dx *= u_;
        for(auto &kv : k) kv *= std::pow(u_, 5);
        double u3 = u_ * u_ * u_;
        for(auto &r : rho_) r /= u3;
        params_.dt = dt_;
        params_.dx = dx;
        for(int s = 0; s < S_; s++) params_.k[s] = k[s];

        // src/mobility/IMobility.cpp:18-57
        std::string mob = cfg_.opt_string("mobility.type", "constant");
        double M = cfg_.opt_double("mobility.M", 1.0);
        if(mob == "constant") params_.mobility_type = CHGB_MOBILITY_CONSTANT;
        else if(mob == "free_energy") params_.mobility_type = CHGB_MOBILITY_FREE_ENERGY;
        else if(mob == "regularised") {
            params_.mobility_type = CHGB_MOBILITY_REGULARISED;
            if(!cfg_.has("mobility.rho_min")) critical("For 'regularised' mobility, 'rho_min' must be specified");
            params_.rho_min = cfg_.get_double("mobility.rho_min") / u_;
        }
        else if(mob == "gel") {
            params_.mobility_type = CHGB_MOBILITY_GEL;
            if(!cfg_.has("mobility.phi_critical") || !cfg_.has("mobility.c_0") || !cfg_.has("mobility.M_c") ||
               !cfg_.has("landau.epsilon"))
                critical("For 'gel' mobility, 'phi_critical', 'c_0', 'M_c', and 'landau.epsilon' must be specified");
            params_.gel_phi_critical = cfg_.get_double("mobility.phi_critical");
            params_.gel_c0 = cfg_.get_double("mobility.c_0");
            params_.gel_M_c = cfg_.get_double("mobility.M_c") / u_;
            params_.gel_beta_delta_F = 10.0 / (1.0 - cfg_.get_double("landau.epsilon")) - std::log(24000.0);
        }
        else critical("Unknown mobility type: %s", mob.c_str());
        params_.M = M / u_;

        if(integ == "euler") params_.integrator = CHGB_INTEGRATOR_EULER;
        else if(integ == "euler_mobility") params_.integrator = CHGB_INTEGRATOR_EULER_MOBILITY;
        else if(integ == "pseudospectral") params_.integrator = CHGB_INTEGRATOR_PSEUDOSPECTRAL;
        else if(integ == "pseudospectral_mobility") params_.integrator = CHGB_INTEGRATOR_PSEUDOSPECTRAL_MOBILITY;
        else if(integ == "bailo") critical("Unsupported CUDA integrator %s", integ.c_str());
        else critical("Unsupported integrator %s", integ.c_str());
        if(integ == "pseudospectral_mobility") {
            // src/integrators/PseudospectralMobilityCPU.cpp:204-208
            params_.use_gmres = cfg_.opt_bool("pseudospectral.use_gmres", false) ? 1 : 0;
            params_.gmres_restart = (int32_t) cfg_.opt_int("pseudospectral.gmres_restart", 30);
            params_.gmres_max_iter = (int32_t) cfg_.opt_int("pseudospectral.gmres_max_iter", 200);
            params_.gmres_tol = cfg_.opt_double("pseudospectral.gmres_tol", 1e-10);
        }
        // src/integrators/PseudospectralCPU.cpp:24 scales S; PseudospectralMobilityCPU.cpp:22 does not
        params_.splitting_S = cfg_.opt_double("pseudospectral.S", 0.0) *
                              (params_.integrator == CHGB_INTEGRATOR_PSEUDOSPECTRAL_MOBILITY ? 1.0 : u3);
        params_.use_dealias = cfg_.opt_bool("pseudospectral.use_dealias", false) ? 1 : 0;
        if(params_.mobility_type != CHGB_MOBILITY_CONSTANT && params_.integrator != CHGB_INTEGRATOR_EULER_MOBILITY &&
           params_.integrator != CHGB_INTEGRATOR_PSEUDOSPECTRAL_MOBILITY)
            critical("The selected integrator only supports constant mobility");
        if(dry_) return;

        if(chgb_create(&params_, &h_) != CHGB_OK) critical("%s", chgb_last_error(nullptr));
        if(chgb_upload(h_, rho_.data(), nullptr) != CHGB_OK) critical("%s", chgb_last_error(h_));
        synced_ = true;
        info("Running a simulation with N = %d, dt = %g, dx = %g, integrator = %s on the GB300 engine", N, dt_, dx,
             integ.c_str());
    }

    // src/CahnHilliard.cpp:72-132
    void load_from(const std::string &filename, int N, size_t bins) {
        std::ifstream in(filename);
        if(!in.good()) critical("The initial conditions file '%s' is not readable", filename.c_str());
        bool full3d = cfg_.opt_bool("load_from_full_3d", false);
        int want = (DIM == 3 && full3d) ? N * N : N;
        std::string line;
        std::vector<std::string> spl;
        int lines = 0;
        for(int s = 0; s < S_; s++) {
            int ok = 0;
            while(ok < want && in.good()) {
                std::getline(in, line);
                size_t a = line.find_first_not_of(" \t\r\n");
                size_t b = line.find_last_not_of(" \t\r\n");
                line = (a == std::string::npos) ? "" : line.substr(a, b - a + 1);
                split_ws(line, spl);
                if(!line.empty() && line[0] != '#') {
                    if(DIM == 1) {
                        if(spl.size() != 1) critical("Line n. %d in the initial configuration file contains %zu fields, should be 1", lines, spl.size());
                        rho_[s * bins + ok] = std::stod(line);
                    }
                    else {
                        if((int) spl.size() != N)
                            critical("Line n. %d in the initial configuration file contains only %zu fields, should be %d", lines, spl.size(), N);
                        size_t y = (DIM == 2) ? ok : ok % N;
                        size_t z = (DIM == 2) ? 0 : ok / N;
                        for(int x = 0; x < N; x++) rho_[s * bins + x + N * y + (size_t) N * N * z] = std::stod(spl[x]);
                    }
                    ok++;
                }
                lines++;
            }
            if(ok != want) critical("The initial configuration file contains only %d valid lines for species %d, should be %d", ok, s, want);
        }
    }

    const Config &cfg_;
    long long steps_ = 0, print_every_ = 0, initial_t_ = 0;
    double internal_to_user_ = 1.0, u_ = 1.0, dt_ = 0.0;
    std::string output_path_;
    Rand48 rng_;
    chgb_params params_{};
    chgb_handle *h_ = nullptr;
    int S_ = 1;
    std::vector<double> rho_, pressure_;
    bool synced_ = false, loading_ = false, dry_ = false, print_pressure_ = false;
    Printer *printer_ = nullptr;
};

}  // namespace ch

int main(int argc, char *argv[]) {
    if(argc < 2) {
        std::fprintf(stderr, "Usage is %s configuration_file\n", argv[0]);
        return 0;
    }
    bool print_params = std::strcmp(argv[1], "--print-params") == 0;
    const char *path = print_params ? (argc > 2 ? argv[2] : "") : argv[1];
    ch::Config cfg;
    try {
        cfg.root = tomllite::parse_file(path);
    }
    catch(const tomllite::ParseError &e) {
        std::fprintf(stderr, "Parsing failed with error '%s'\n", e.what());
        return 1;
    }
    if(print_params) {
        ch::Manager::print_params(cfg);
        return 0;
    }
    ch::Manager manager(cfg);
    manager.run();
    return 0;
}
