/*
 * GB300Integrator.h — the drop-in integrator for the reference program
 * (lorenzo-rovigatti/cahn-hilliard), running every time step in libchgb.
 *
 * It subclasses the reference's plugin interface `Integrator<dims>`
 * (src/integrators/Integrator.h:10-41) and is compiled against the
 * reference's own headers (src/ on the include path) and include/chgb.h,
 * linked with libchgb.so.  The reference's factory
 * (src/CahnHilliard.cpp:169-223) would construct it where it constructs the
 * CUDA integrators when `use_CUDA = true`; CahnHilliard::integrator and
 * CahnHilliard::mobility are public, so a program can also swap it into an
 * existing CahnHilliard object (install() below) without touching the
 * reference.
 *
 * What it does:
 * * constructor: fills a chgb_params from the reference's TOML keys, scaled to
 *   internal units exactly as the reference's constructors scale them
 *   (Integrator.cpp:8-25 for dt, dx, k; Landau.cpp:16-36, SimpleWertheim.cpp:
 *   20-34, SalehWertheim.cpp:19-41 for the model constants; FreeEnergyModel.h:
 *   18-22 for the density conversion; ConstantMobility.h:18-22,
 *   FreeEnergyMobility.h:18-22, RegularisedMobility.h:18-22,
 *   GelMobility.h:20-27 and IMobility.cpp:18-57 for the mobility;
 *   PseudospectralCPU.cpp:23-25 and PseudospectralMobilityCPU.cpp:22-23,
 *   204-208 for the pseudospectral keys), then chgb_create + chgb_upload of
 *   the host density (CUDAIntegrator::_CPU_GPU, src/CUDA/integrators/
 *   CUDAIntegrator.cu:43-53);
 * * evolve(): chgb_step(h, 1) -- one CahnHilliard::evolve(), whose mobility
 *   update (src/CahnHilliard.cpp:278-282) the engine performs on the device
 *   from the step's own input, so the host mobility object must do nothing
 *   (install() puts a no-op one in place);
 * * sync(): chgb_download of the density and the mobility into the
 *   SimulationState when the host copy is stale (CUDAIntegrator::sync,
 *   CUDAIntegrator.cu:56-70);
 * * _supports_nonconstant_mobility(): true for `euler_mobility` and
 *   `pseudospectral_mobility`, so validate() rejects the same combinations as
 *   the reference (Integrator.cpp:38-42).
 * Errors become the reference's critical() (log and exit) with the engine's
 * message.
 */
#ifndef CHGB_GB300_INTEGRATOR_H
#define CHGB_GB300_INTEGRATOR_H

#include "integrators/Integrator.h"
#include "mobility/IMobility.h"
#include "utils/Delta.h"

#include <chgb.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

namespace ch {

template<int dims>
class GB300Integrator : public Integrator<dims> {
public:
    // create_handle = false fills params() only (no device work), for checking the translation.
    GB300Integrator(SimulationState<dims> &sim_state, FreeEnergyModel *model, toml::table &config,
                    bool create_handle = true) :
            Integrator<dims>(sim_state, model, config) {
        std::memset(&_p, 0, sizeof(_p));
        const double u = sim_state.user_to_internal;
        const double u3 = u * u * u;
        _p.dims = dims;
        _p.N = this->_N_per_dim;
        _p.dt = this->_dt;
        _p.dx = this->_dx;                                   // already times user_to_internal
        for(int s = 0; s < this->_N_species && s < CHGB_MAX_SPECIES; s++) _p.k[s] = this->_k_laplacian[s];
        _p.kernel_variant = 0;                               // the engine times its kernel variants once

        _integrator = this->template _config_optional_value<std::string>(config, "integrator", "euler");
        if(_integrator == "euler") _p.integrator = CHGB_INTEGRATOR_EULER;
        else if(_integrator == "euler_mobility") _p.integrator = CHGB_INTEGRATOR_EULER_MOBILITY;
        else if(_integrator == "pseudospectral") _p.integrator = CHGB_INTEGRATOR_PSEUDOSPECTRAL;
        else if(_integrator == "pseudospectral_mobility") _p.integrator = CHGB_INTEGRATOR_PSEUDOSPECTRAL_MOBILITY;
        else this->critical("Unsupported GB300 integrator {}", _integrator);

        // pseudospectral: S is scaled by u^3 there and not for the mobility variant
        double S = this->template _config_optional_value<double>(config, "pseudospectral.S", 0.0);
        _p.splitting_S = (_p.integrator == CHGB_INTEGRATOR_PSEUDOSPECTRAL_MOBILITY) ? S : S * u3;
        _p.use_dealias = this->template _config_optional_value<bool>(config, "pseudospectral.use_dealias", false);
        _p.use_gmres = this->template _config_optional_value<bool>(config, "pseudospectral.use_gmres", false);
        _p.gmres_restart = this->template _config_optional_value<int>(config, "pseudospectral.gmres_restart", 30);
        _p.gmres_max_iter = this->template _config_optional_value<int>(config, "pseudospectral.gmres_max_iter", 200);
        _p.gmres_tol = this->template _config_optional_value<double>(config, "pseudospectral.gmres_tol", 1e-10);

        _fill_model(config, u3);
        _fill_mobility(config, u);

        if(!create_handle) return;
        if(chgb_create(&_p, &_h) != CHGB_OK) this->critical("{}", chgb_last_error(nullptr));
        if(chgb_upload(_h, this->_rho.data(), nullptr) != CHGB_OK) this->critical("{}", chgb_last_error(_h));
        _output_ready = true;
    }

    ~GB300Integrator() override {
        if(_h) chgb_destroy(_h);
    }

    void evolve() override {
        if(chgb_step(_h, 1) != CHGB_OK) this->critical("{}", chgb_last_error(_h));
        _output_ready = false;
    }

    void sync() override {
        if(_output_ready) return;
        if(chgb_download(_h, this->_rho.data(), this->_sim_state.mobility.data()) != CHGB_OK)
            this->critical("{}", chgb_last_error(_h));
        _output_ready = true;
    }

    // The engine's handle, for chgb_observables / chgb_pressure / chgb_structure_factor.
    chgb_handle *handle() const { return _h; }
    const chgb_params &params() const { return _p; }

    GET_NAME(GB300Integrator)

protected:
    bool _supports_nonconstant_mobility() const override {
        return _p.integrator == CHGB_INTEGRATOR_EULER_MOBILITY ||
               _p.integrator == CHGB_INTEGRATOR_PSEUDOSPECTRAL_MOBILITY;
    }

private:
    void _fill_model(toml::table &config, double u3) {
        chgb_model_params &m = _p.model;
        m.density_conversion_factor = u3;
        const std::string name = this->template _config_value<std::string>(config, "free_energy");
        if(name == "landau") {
            m.kind = CHGB_MODEL_LANDAU;
            m.n_species = 1;
            if(config["landau"]["epsilon"]) m.epsilon = this->template _config_value<double>(config, "landau.epsilon");
            else m.epsilon = 1.0 - this->template _config_value<double>(config, "landau.T");
        }
        else if(name == "simple_wertheim") {
            m.kind = CHGB_MODEL_SIMPLE_WERTHEIM;
            m.n_species = 1;
            m.valence = this->template _config_value<int>(config, "wertheim.valence");
            m.B2 = this->template _config_value<double>(config, "wertheim.B2") * u3;
            m.regularisation_delta =
                    this->template _config_optional_value<double>(config, "wertheim.regularisation_delta", 0.0) / u3;
            m.delta = (double) Delta(config, "wertheim.delta") * u3;
        }
        else if(name == "saleh") {
            m.kind = CHGB_MODEL_SALEH;
            m.n_species = 3;
            m.B2 = this->template _config_value<double>(config, "saleh.B2") * u3;
            m.B3 = this->template _config_optional_value<double>(config, "saleh.B3", 0.0) * u3 * u3;
            m.delta_AA = (double) Delta(config, "saleh.delta_AA") * u3;
            m.delta_BB = (double) Delta(config, "saleh.delta_BB") * u3;
            std::vector<int> v = this->template _config_array_values<int>(config, "saleh.valence", 3);
            for(int i = 0; i < 3; i++) m.saleh_valence[i] = v[i];
        }
        else {
            this->critical("The free energy model '{}' is not supported by the GB300 engine", name);
        }
    }

    void _fill_mobility(toml::table &config, double u) {
        const double M = config["mobility"]["M"].value_or(1.0);
        _p.M = M / u;
        const std::string &type = this->_mobility_type;
        if(type == "constant") _p.mobility_type = CHGB_MOBILITY_CONSTANT;
        else if(type == "free_energy") _p.mobility_type = CHGB_MOBILITY_FREE_ENERGY;
        else if(type == "regularised") {
            _p.mobility_type = CHGB_MOBILITY_REGULARISED;
            _p.rho_min = this->template _config_value<double>(config, "mobility.rho_min") / u;
        }
        else if(type == "gel") {
            _p.mobility_type = CHGB_MOBILITY_GEL;
            _p.gel_phi_critical = this->template _config_value<double>(config, "mobility.phi_critical");
            _p.gel_c0 = this->template _config_value<double>(config, "mobility.c_0");
            _p.gel_M_c = this->template _config_value<double>(config, "mobility.M_c") / u;
            const double eps = this->template _config_value<double>(config, "landau.epsilon");
            _p.gel_beta_delta_F = 10.0 / (1.0 - eps) - std::log(24000.0);
        }
        else {
            this->critical("Unknown mobility type: {}", type);
        }
    }

    chgb_params _p;
    chgb_handle *_h = nullptr;
    bool _output_ready = true;
    std::string _integrator;
};

// The host-side mobility object of a CahnHilliard driven by GB300Integrator:
// the engine updates the mobility on the device inside every chgb_step.
template<int dims>
class GB300DeviceMobility : public IMobility<dims> {
public:
    explicit GB300DeviceMobility(SimulationState<dims> &state) : IMobility<dims>(state) {}
    void update_mobility() override {}
    GET_NAME(GB300DeviceMobility)
};

// Replace the integrator and the mobility object of a constructed
// CahnHilliard<dims> (both public members) with the GB300 ones, then run the
// reference's validate(), as its factory does (src/CahnHilliard.cpp:221-223).
template<int dims, class System>
GB300Integrator<dims> *install(System &system, SimulationState<dims> &state, FreeEnergyModel *model,
                               toml::table &config) {
    auto integ = std::make_unique<GB300Integrator<dims>>(state, model, config);
    GB300Integrator<dims> *raw = integ.get();
    system.integrator = std::move(integ);
    system.mobility = std::make_unique<GB300DeviceMobility<dims>>(state);
    system.integrator->validate();
    state.integrator = raw;
    return raw;
}

} /* namespace ch */

#endif /* CHGB_GB300_INTEGRATOR_H */
