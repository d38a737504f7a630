/*
 * gb300_dropin.cpp — the reference's own simulation object driven by the GB300
 * engine through cahn-hilliard_gb300/host/GB300Integrator.h.
 *
 * Compiled by oracle/Makefile (`make -C oracle dropin`) against the
 * reference's sources where they lie and linked with libchgb.so; binaries go
 * to oracle/_ref/.  It shows that the reference-side binding compiles and
 * links against the reference's Integrator<dims> interface
 * (src/integrators/Integrator.h:10-41): it builds the model and the
 * CahnHilliard<DIM> object in the order of src/main.cpp:22-65, swaps in
 * GB300Integrator (and the no-op host mobility), calls
 * CahnHilliard<DIM>::evolve() `steps` times (src/CahnHilliard.cpp:278-282),
 * syncs, and writes the final density as raw doubles plus the reference's own
 * host observables (average_mass / average_free_energy, %.17g).
 *
 * usage: gb300_dropin_<D>D config.toml steps prefix
 *        gb300_dropin_<D>D --print-params config.toml
 *            (the chgb_params the integrator builds, as JSON, without a GPU)
 */
#include "CahnHilliard.h"
#include "SimulationState.h"
#include "models/Landau.h"
#include "models/SalehWertheim.h"
#include "models/SimpleWertheim.h"

#include "GB300Integrator.h"

#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>

static void print_params(const chgb_params &p) {
    const chgb_model_params &q = p.model;
    std::printf("{\"dims\": %d, \"N\": %d, \"integrator\": %d, \"mobility_type\": %d, \"dt\": %.17g, "
                "\"dx\": %.17g, \"k\": [%.17g, %.17g, %.17g], \"M\": %.17g, \"splitting_S\": %.17g, "
                "\"use_dealias\": %d, \"kind\": %d, \"n_species\": %d, \"epsilon\": %.17g, \"valence\": %d, "
                "\"saleh_valence\": [%d, %d, %d], \"B2\": %.17g, \"B3\": %.17g, \"delta\": %.17g, "
                "\"regularisation_delta\": %.17g, \"delta_AA\": %.17g, \"delta_BB\": %.17g, "
                "\"density_conversion_factor\": %.17g, \"rho_min\": %.17g, \"gel\": [%.17g, %.17g, %.17g, %.17g], "
                "\"gmres\": [%d, %d, %d, %.17g]}\n",
                p.dims, p.N, p.integrator, p.mobility_type, p.dt, p.dx, p.k[0], p.k[1], p.k[2], p.M, p.splitting_S,
                p.use_dealias, q.kind, q.n_species, q.epsilon, q.valence, q.saleh_valence[0], q.saleh_valence[1],
                q.saleh_valence[2], q.B2, q.B3, q.delta, q.regularisation_delta, q.delta_AA, q.delta_BB,
                q.density_conversion_factor, p.rho_min, p.gel_phi_critical, p.gel_c0, p.gel_M_c, p.gel_beta_delta_F,
                p.use_gmres, p.gmres_restart, p.gmres_max_iter, p.gmres_tol);
}

int main(int argc, char *argv[]) {
    const bool params_only = argc == 3 && std::string(argv[1]) == "--print-params";
    if(argc < 4 && !params_only) {
        std::fprintf(stderr, "usage: %s config.toml steps prefix | --print-params config.toml\n", argv[0]);
        return 1;
    }
    toml::parse_result res = toml::parse_file(argv[params_only ? 2 : 1]);
    if(!res) {
        std::fprintf(stderr, "TOML parse error\n");
        return 1;
    }
    toml::table config = std::move(res).table();
    long long steps = params_only ? 0 : std::atoll(argv[2]);
    std::string prefix = params_only ? "" : argv[3];

    ch::SimulationState<DIM> state;
    state.internal_to_user = config["distance_scaling_factor"].value_or(1.0);
    state.user_to_internal = 1.0 / state.internal_to_user;
    state.use_CUDA = false;   // the reference's own CUDA path stays out; the engine is the integrator
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
    if(params_only) {
        ch::GB300Integrator<DIM> probe(state, state.model.get(), config, false);
        print_params(probe.params());
        return 0;
    }
    ch::install<DIM>(system, state, state.model.get(), config);

    for(long long t = 0; t < steps; t++) system.evolve();
    system.integrator->sync();

    FILE *fp = std::fopen((prefix + "_final.bin").c_str(), "wb");
    if(!fp) {
        std::perror(prefix.c_str());
        return 2;
    }
    std::fwrite(state.rho.data(), sizeof(double), (size_t) state.rho.size(), fp);
    std::fclose(fp);
    FILE *obs = std::fopen((prefix + "_obs.txt").c_str(), "w");
    std::fprintf(obs, "%.17g %.17g\n", system.average_mass(), system.average_free_energy());
    std::fclose(obs);
    return 0;
}
