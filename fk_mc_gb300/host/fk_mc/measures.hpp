// measures.hpp — measure_energy (src/measures/energy.cpp:6-26) and
// measure_spectrum (src/measures/spectrum.cpp:13-21) on the GPU-computed
// ed_cache; measure_ipr (include/fk_mc/measures/ipr.hpp) and
// measure_stiffness (include/fk_mc/measures/stiffness.hpp) computed on the GPU
// from calc_ed(true) (fkg_measure_ipr, fkg_measure_stiffness);
// measure_spectrum_history (src/measures/spectrum_history.cpp:7-19),
// measure_focc (src/measures/focc_history.cpp:7-12) and measure_nf0pi
// (include/fk_mc/measures/fsusc0pi.hpp:10-44) record the series that the
// statistics stage (data_save.hpp) bins.
#pragma once
#include <cmath>
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

// measure_ipr (include/fk_mc/measures/ipr.hpp:13-56): every accumulate()
// appends ipr_k = ||x_k||_4 / ||x_k||_2^2 of each eigenvector k (ascending
// eigenvalues) of the current configuration to ipr_vals[k].
template <typename lattice_t>
struct measure_ipr {
    const lattice_t& lattice_;
    configuration_t& config_;
    int _Z = 0;
    std::vector<std::vector<double>>& ipr_vals_;
    measure_ipr(configuration_t& in, const lattice_t& lattice, std::vector<std::vector<double>>& ipr_vals)
        : lattice_(lattice), config_(in), ipr_vals_(ipr_vals) {
        ipr_vals_.resize(config_.lattice_.volume());
    }
    void accumulate(double) {
        gpu_backend& g = gpu_backend::instance();
        const int id = g.lattice_id(config_.lattice_);
        const std::vector<double>& diag = config_.calc_hamiltonian();
        std::vector<double> ipr(diag.size());
        double beta = config_.params().beta;
        g.check(fkg_measure_ipr(g.ctx(), 1, &id, diag.data(), &beta, ipr.data()), "fkg_measure_ipr");
        for (std::size_t i = 0; i < ipr.size() && i < ipr_vals_.size(); ++i) ipr_vals_[i].push_back(ipr[i]);
        _Z++;
    }
};

// measure_stiffness (include/fk_mc/measures/stiffness.hpp:49-187): the
// kinetic and current operators along the lattice's first axis are built once
// (periodic left/right neighbours, -t and -/+1) and registered with the
// library; every accumulate() appends the configuration's Drude stiffness to
// stiffness_vals and, for each frequency of wgrid, the sum of its resonant
// terms (width offset) to cond_history.
template <typename lattice_t>
struct measure_stiffness {
    const lattice_t& lattice_;
    configuration_t& config_;
    std::vector<double>& stiffness_vals_;
    std::vector<std::vector<double>>& cond_history_;
    double t_ = 1.;
    std::vector<double> wgrid_;
    double offset_;
    measure_stiffness(configuration_t& in, const lattice_t& lattice, std::vector<double>& stiffness_vals,
                      std::vector<std::vector<double>>& cond_history, std::vector<double> wgrid, double offset)
        : lattice_(lattice), config_(in), stiffness_vals_(stiffness_vals), cond_history_(cond_history),
          wgrid_(std::move(wgrid)), offset_(offset) {
        cond_history_.resize(wgrid_.size());
    }
    void accumulate(double) {
        gpu_backend& g = gpu_backend::instance();
        const int id = g.lattice_id(config_.lattice_);
        if (registered_id_ != id || registered_version_ != g.registrations()) register_ops(g, id);
        const std::vector<double>& diag = config_.calc_hamiltonian();
        double beta = config_.params().beta, st = 0.0;
        std::vector<double> cond(wgrid_.size());
        g.check(fkg_measure_stiffness(g.ctx(), 1, &id, diag.data(), &beta, &st, (int)wgrid_.size(),
                                      wgrid_.empty() ? nullptr : wgrid_.data(), offset_,
                                      wgrid_.empty() ? nullptr : cond.data()),
                "fkg_measure_stiffness");
        stiffness_vals_.push_back(st);
        for (std::size_t w = 0; w < wgrid_.size(); ++w) cond_history_[w].push_back(cond[w]);
    }

private:
    int registered_id_ = -1;
    unsigned long registered_version_ = 0;
    void register_ops(gpu_backend& g, int id) {
        const auto dims = lattice_.dims();
        const int Lx = dims[0];
        const std::size_t n = lattice_.msize();
        std::vector<int32_t> rowptr(n + 1, 0), col;
        std::vector<double> tv, jv;
        for (std::size_t i = 0; i < n; ++i) {
            auto p0 = lattice_.index_to_pos(i), pl = p0, pr = p0;
            pl[0] = ((p0[0] - 1) + Lx) % Lx;
            pr[0] = ((p0[0] + 1) + Lx) % Lx;
            const int il = (int)lattice_.pos_to_index(pl), ir = (int)lattice_.pos_to_index(pr);
            if (il == ir) {  // L = 2: the two triplets coincide and are summed
                col.push_back(il); tv.push_back(-2.0 * t_); jv.push_back(0.0);
            } else {
                const int a = il < ir ? il : ir, b = il < ir ? ir : il;
                col.push_back(a); tv.push_back(-t_); jv.push_back(a == il ? -1.0 : 1.0);
                col.push_back(b); tv.push_back(-t_); jv.push_back(b == il ? -1.0 : 1.0);
            }
            rowptr[i + 1] = (int32_t)col.size();
        }
        g.check(fkg_set_stiffness_ops(g.ctx(), id, (int)n, rowptr.data(), col.data(), tv.data(), jv.data()),
                "fkg_set_stiffness_ops");
        registered_id_ = id;
        registered_version_ = g.registrations();
    }
};

// every accumulate() appends eigenvalue i of the current configuration to
// spectrum_history[i]
struct measure_spectrum_history {
    configuration_t& config;
    std::vector<std::vector<double>>& _spectrum_history;
    int _Z = 0;
    measure_spectrum_history(configuration_t& in, std::vector<std::vector<double>>& spectrum_history)
        : config(in), _spectrum_history(spectrum_history) {
        _spectrum_history.resize(config.lattice_.msize());
    }
    void accumulate(double) {
        config.calc_ed(false);
        const auto& spectrum = config.ed_data_.cached_spectrum;
        for (std::size_t i = 0; i < spectrum.size(); ++i) _spectrum_history[i].push_back(spectrum[i]);
        _Z++;
    }
};

// every accumulate() appends f_i of the current configuration to focc[i]
struct measure_focc {
    configuration_t& config;
    std::vector<std::vector<double>>& focc_;
    int _Z = 0;
    measure_focc(configuration_t& in, std::vector<std::vector<double>>& focc) : config(in), focc_(focc) {
        focc_.resize(config.lattice_.volume());
    }
    void accumulate(double) {
        for (std::size_t i = 0; i < config.f_config_.size(); ++i) focc_[i].push_back(config.f_config_[i]);
        _Z++;
    }
};

// n_f(q=0) = sum_i f_i and n_f(q=pi) = |sum_i f_i (-1)^(sum of coordinates)|
template <typename lattice_t>
struct measure_nf0pi {
    const configuration_t& config_;
    const lattice_t& lattice_;
    int _Z = 0;
    double average_nf0_ = 0.0, average_nfpi_ = 0.0;
    std::vector<double>& n0_;
    std::vector<double>& npi_;
    measure_nf0pi(const configuration_t& in, const lattice_t& lattice, std::vector<double>& n0, std::vector<double>& npi)
        : config_(in), lattice_(lattice), n0_(n0), npi_(npi) {}
    void accumulate(double) {
        const double n0 = (double)config_.get_nf();
        const double npi = std::abs((double)lattice_.FFT_pi(config_.f_config_));
        average_nf0_ += n0;
        average_nfpi_ += npi;
        n0_.push_back(n0);
        npi_.push_back(npi);
        _Z++;
    }
};

}  // namespace fk
