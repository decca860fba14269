// measures.hpp — measure_energy (src/measures/energy.cpp:6-26) and
// measure_spectrum (src/measures/spectrum.cpp:13-21) on the GPU-computed
// ed_cache.
#pragma once
#include <vector>

#include "configuration.hpp"

namespace fk {

struct measure_energy {
    double beta;
    configuration_t& config;
    std::vector<double>& _energies;
    std::vector<double>& _d2energies;
    std::vector<double>& _c_energies;
    int _Z = 0;
    double _average_energy = 0.0, _average_d2energy = 0.0;
    measure_energy(double beta, configuration_t& in, std::vector<double>& energies, std::vector<double>& d2energies,
                   std::vector<double>& c_energies)
        : beta(beta), config(in), _energies(energies), _d2energies(d2energies), _c_energies(c_energies) {}
    void accumulate(double) {
        config.calc_ed(false);
        const auto& spectrum = config.ed_data_.cached_spectrum;
        const auto& exp_e = config.ed_data_.cached_exp;
        _Z++;
        double e_c = 0.0, d2e = 0.0;
        for (std::size_t i = 0; i < spectrum.size(); ++i) {
            e_c += spectrum[i] / (1.0 + exp_e[i]);
            d2e += spectrum[i] * spectrum[i] / (1.0 + 0.5 * (exp_e[i] + 1. / exp_e[i]));
        }
        const double e_val = e_c - double(config.params_.mu_f) * config.get_nf() + config.calc_ff_energy();
        _average_energy += e_val;
        _average_d2energy += d2e / 2.0;
        _energies.push_back(e_val);
        _d2energies.push_back(d2e / 2.0);
        _c_energies.push_back(e_c);
    }
};

struct measure_spectrum {
    configuration_t& config;
    std::vector<double>& _average_spectrum;
    int _Z = 0;
    measure_spectrum(configuration_t& in, std::vector<double>& average_spectrum)
        : config(in), _average_spectrum(average_spectrum) {
        _average_spectrum.resize(config.lattice_.msize(), 0.0);
    }
    void accumulate(double) {
        config.calc_ed(false);
        const auto& spectrum = config.ed_data_.cached_spectrum;
        for (std::size_t i = 0; i < _average_spectrum.size(); i++)
            _average_spectrum[i] = (_average_spectrum[i] * _Z + spectrum[i]) / (_Z + 1);
        _Z++;
    }
};

}  // namespace fk
