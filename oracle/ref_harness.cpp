/*
 * ref_harness.cpp — drives the reference's own CPU integrators and dumps the
 * density at full FP64 precision.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile against the
 * reference sources where they lie (never copied into this repository); the
 * binaries go to oracle/_ref/.  The reference's native writer keeps six
 * significant digits (src/utils/Printer.cpp:183-192), too few for a 1e-12
 * comparison, hence this harness.
 *
 * It builds the objects in the order of src/main.cpp:22-65 (srand48 before
 * the model and the CahnHilliard object, so the drand48 draws of the initial
 * density are the same), then calls CahnHilliard<DIM>::evolve() `steps`
 * times (src/CahnHilliard.cpp:278-282) and writes raw little-endian doubles:
 *   <prefix>_init.bin, <prefix>_final.bin, <prefix>_mobility.bin,
 *   <prefix>_obs.txt  (mass and free energy before/after, %.17g),
 * and, for the Landau model (the one model whose pressure() does not stop the
 * program, src/models/FreeEnergyModel.h:43-44), <prefix>_pressure.bin with
 * CahnHilliard::pressure() of the final state and <prefix>_pressure.txt with
 * average_pressure() before/after (src/CahnHilliard.cpp:321-356); it prints
 * the evolve-loop wall time.
 *
 * usage: ref_harness_<D>D config.toml steps prefix
 */
#include "CahnHilliard.h"
#include "SimulationState.h"
#include "models/Landau.h"
#include "models/SalehWertheim.h"
#include "models/SimpleWertheim.h"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>

static void dump(const std::string &fn, const ch::MultiField<double> &f) {
    FILE *fp = std::fopen(fn.c_str(), "wb");
    if(!fp) {
        std::perror(fn.c_str());
        std::exit(2);
    }
    std::fwrite(f.data(), sizeof(double), (size_t) f.size(), fp);
    std::fclose(fp);
}

int main(int argc, char *argv[]) {
    if(argc < 4) {
        std::fprintf(stderr, "usage: %s config.toml steps prefix\n", argv[0]);
        return 1;
    }
    toml::parse_result res = toml::parse_file(argv[1]);
    if(!res) {
        std::fprintf(stderr, "TOML parse error\n");
        return 1;
    }
    toml::table config = std::move(res).table();
    long long steps = std::atoll(argv[2]);
    std::string prefix = argv[3];

    ch::SimulationState<DIM> state;
    state.internal_to_user = config["distance_scaling_factor"].value_or(1.0);
    state.user_to_internal = 1.0 / state.internal_to_user;
    srand48(config["seed"].value_or<long long>(0));

    std::string model_name = config["free_energy"].value_or(std::string("landau"));
    if(model_name == "landau") state.model = std::make_unique<ch::Landau>(config);
    else if(model_name == "simple_wertheim") state.model = std::make_unique<ch::SimpleWertheim>(config);
    else if(model_name == "saleh") state.model = std::make_unique<ch::SalehWertheim>(config);
    else {
        std::fprintf(stderr, "unsupported model %s\n", model_name.c_str());
        return 1;
    }

    ch::CahnHilliard<DIM> system(state, state.model.get(), config);
    const bool landau = model_name == "landau";
    FILE *obs = std::fopen((prefix + "_obs.txt").c_str(), "w");
    FILE *prs = landau ? std::fopen((prefix + "_pressure.txt").c_str(), "w") : nullptr;
    dump(prefix + "_init.bin", state.rho);
    std::fprintf(obs, "%.17g %.17g\n", system.average_mass(), system.average_free_energy());
    if(prs) std::fprintf(prs, "%.17g\n", system.average_pressure());

    auto t0 = std::chrono::steady_clock::now();
    for(long long t = 0; t < steps; t++) system.evolve();
    auto t1 = std::chrono::steady_clock::now();
    system.integrator->sync();

    dump(prefix + "_final.bin", state.rho);
    dump(prefix + "_mobility.bin", state.mobility);
    std::fprintf(obs, "%.17g %.17g\n", system.average_mass(), system.average_free_energy());
    std::fclose(obs);
    if(prs) {
        std::fprintf(prs, "%.17g\n", system.average_pressure());
        std::fclose(prs);
        dump(prefix + "_pressure.bin", system.pressure());
    }
    double secs = std::chrono::duration<double>(t1 - t0).count();
    std::printf("evolve_seconds %.9f cells %d steps %lld\n", secs, system.grid_size, steps);
    return 0;
}
