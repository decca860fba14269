// moves.hpp — move_flip, move_randomize, move_addremove with the reference's
// interface and random-draw order (include/fk_mc/moves.hpp:11-47,
// src/moves.cpp:5-67). The eigen-solves inside attempt() run on the GPU.
#pragma once
#include <cmath>

#include "configuration.hpp"

namespace fk {

struct move_flip {
    typedef double mc_weight_type;
    double beta;
    configuration_t& config;
    configuration_t new_config;
    random_generator& RND;
    move_flip(double beta, configuration_t& current_config, random_generator& RND_)
        : beta(beta), config(current_config), new_config(current_config), RND(RND_) {}
    virtual ~move_flip() = default;

    virtual mc_weight_type attempt() {  // src/moves.cpp:5-21
        std::uniform_int_distribution<> distr(0, (int)config.lattice_.volume() - 1);
        if (config.get_nf() == 0 || config.get_nf() == config.lattice_.msize()) return 0;
        new_config = config;
        std::size_t from = distr(RND);
        while (new_config.f_config_[from] == 0) from = distr(RND);
        std::size_t to = distr(RND);
        while (new_config.f_config_[to] == 1) to = distr(RND);
        config.calc_ed(false);
        new_config.f_config_[from] = 0;
        new_config.f_config_[to] = 1;
        new_config.calc_hamiltonian();
        new_config.calc_ed(false);
        return std::exp(new_config.ed_data_.logZ - config.ed_data_.logZ);
    }
    mc_weight_type accept() { config = new_config; return 1.0; }  // src/moves.cpp:23-28
    void reject() {}
};

struct move_randomize : move_flip {
    using move_flip::move_flip;
    mc_weight_type attempt() override {  // src/moves.cpp:35-49
        new_config = config;
        new_config.randomize_f(RND);
        new_config.calc_hamiltonian();
        config.calc_ed(false);
        new_config.calc_ed(false);
        const double log_ratio = new_config.ed_data_.logZ - config.ed_data_.logZ;
        const double ff_diff = new_config.calc_ff_energy() - config.calc_ff_energy();
        // the reference subtracts two size_t counts (a decrease wraps around)
        const double dnf = (double)(new_config.get_nf() - config.get_nf());
        const double mu_f = config.params_.mu_f;
        if (beta * mu_f * dnf - ff_diff > 2.7182818 - log_ratio) return 1;
        else if (beta * mu_f * dnf - ff_diff + log_ratio < 0) return 0;
        return std::exp(log_ratio) * std::exp(beta * (mu_f * dnf - ff_diff));
    }
};

struct move_addremove : move_flip {
    double exp_beta_mu_f;
    int last_site = -1;
    move_addremove(double beta, configuration_t& current_config, random_generator& RND_)
        : move_flip(beta, current_config, RND_), exp_beta_mu_f(std::exp(beta * current_config.params_.mu_f)) {}
    mc_weight_type attempt() override {  // src/moves.cpp:52-67
        std::uniform_int_distribution<> distr(0, (int)config.lattice_.volume() - 1);
        new_config = config;
        const std::size_t to = distr(RND);
        last_site = (int)to;
        new_config.f_config_[to] = 1 - config.f_config_[to];
        config.calc_ed(false);
        new_config.calc_hamiltonian();
        new_config.calc_ed(false);
        const double ff_diff = new_config.calc_ff_energy() - config.calc_ff_energy();
        const double ratio = std::exp(new_config.ed_data_.logZ - config.ed_data_.logZ);
        return (new_config.f_config_[to] ? ratio * exp_beta_mu_f : ratio / exp_beta_mu_f) * std::exp(-beta * ff_diff);
    }
};

// move_addremove with the proposal's spectrum from the rank-one update of
// the current eigen-decomposition (fkg_rank1_logz) instead of a re-solve: the
// same random draws and weight as move_addremove (src/moves.cpp:52-67). The
// current configuration's eigenvectors come from calc_ed(true) (cached until
// a proposal is accepted); they must be FP64-accurate, so the context runs
// the FP64 path for that solve. A rejected proposal costs O(n^2).
struct move_addremove_rank1 : move_addremove {
    using move_addremove::move_addremove;
    mc_weight_type attempt() override {
        std::uniform_int_distribution<> distr(0, (int)config.lattice_.volume() - 1);
        new_config = config;
        const std::size_t to = distr(RND);
        last_site = (int)to;
        new_config.f_config_[to] = 1 - config.f_config_[to];
        gpu_backend& g = gpu_backend::instance();
        if (config.ed_data_.status != ed_cache::full) {
            g.check(fkg_set_precision(g.ctx(), FKG_PREC_F64), "fkg_set_precision");
            config.calc_ed(true);
        }
        const std::size_t n = config.lattice_.msize();
        std::vector<double> z(n), ev(n);
        for (std::size_t k = 0; k < n; ++k) z[k] = config.ed_data_.cached_evecs[to + k * n];  // row `to`
        const double rho = new_config.f_config_[to] ? config.params_.U : -config.params_.U;
        double beta = config.params_.beta, logz = 0.0;
        g.check(fkg_rank1_logz(g.ctx(), 1, (int)n, config.ed_data_.cached_spectrum.data(), z.data(), &rho, &beta,
                               &logz, ev.data()),
                "fkg_rank1_logz");
        new_config.calc_hamiltonian();
        new_config.set_spectrum(ev, logz);
        const double ff_diff = new_config.calc_ff_energy() - config.calc_ff_energy();
        const double ratio = std::exp(new_config.ed_data_.logZ - config.ed_data_.logZ);
        return (new_config.f_config_[to] ? ratio * exp_beta_mu_f : ratio / exp_beta_mu_f) * std::exp(-beta * ff_diff);
    }
};

}  // namespace fk
