// moves_chebyshev.hpp — chebyshev::move_flip, move_randomize and
// move_addremove with the reference's interface and order of calls and
// random draws (include/fk_mc/moves_chebyshev.hpp:11-55,
// src/moves_chebyshev.cpp:6-72): the moves of moves.hpp with logZ from the
// Chebyshev expansion (calc_chebyshev on the GPU) in place of calc_ed.
#pragma once
#include <cmath>

#include "chebyshev.hpp"
#include "configuration.hpp"
#include "moves.hpp"

namespace fk {
namespace chebyshev {

struct move_flip : fk::move_flip {
    const chebyshev_eval& cheb_;
    move_flip(double beta, configuration_t& current_config, const chebyshev_eval& cheb, random_generator& RND_)
        : fk::move_flip(beta, current_config, RND_), cheb_(cheb) {}

    mc_weight_type attempt() override {  // src/moves_chebyshev.cpp:6-25
        config.calc_chebyshev(cheb_);
        if (config.get_nf() == 0 || config.get_nf() == config.lattice_.msize()) return 0;
        std::uniform_int_distribution<> distr(0, (int)config.lattice_.msize() - 1);
        new_config = config;
        std::size_t from = distr(RND);
        while (new_config.f_config_[from] == 0) from = distr(RND);
        std::size_t to = distr(RND);
        while (new_config.f_config_[to] == 1) to = distr(RND);
        new_config.f_config_[from] = 0;
        new_config.f_config_[to] = 1;
        new_config.calc_hamiltonian();
        new_config.calc_chebyshev(cheb_);
        const double ff_diff = new_config.calc_ff_energy() - config.calc_ff_energy();
        return std::exp(new_config.cheb_data_.logZ - config.cheb_data_.logZ - beta * ff_diff);
    }
};

struct move_randomize : move_flip {
    using move_flip::move_flip;
    mc_weight_type attempt() override {  // src/moves_chebyshev.cpp:38-51
        config.calc_chebyshev(cheb_);
        new_config = config;
        new_config.randomize_f(RND);
        new_config.calc_hamiltonian();
        new_config.calc_chebyshev(cheb_);
        const double log_ratio = new_config.cheb_data_.logZ - config.cheb_data_.logZ;
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
    move_addremove(double beta, configuration_t& current_config, const chebyshev_eval& cheb, random_generator& RND_)
        : move_flip(beta, current_config, cheb, RND_), exp_beta_mu_f(std::exp(beta * current_config.params_.mu_f)) {}
    mc_weight_type attempt() override {  // src/moves_chebyshev.cpp:54-72
        std::uniform_int_distribution<> distr(0, (int)config.lattice_.msize() - 1);
        config.calc_chebyshev(cheb_);
        new_config = config;
        const std::size_t to = distr(RND);
        last_site = (int)to;
        new_config.f_config_[to] = 1 - config.f_config_[to];
        new_config.calc_hamiltonian();
        new_config.calc_chebyshev(cheb_);
        const double ff_diff = new_config.calc_ff_energy() - config.calc_ff_energy();
        const double ratio = std::exp(new_config.cheb_data_.logZ - config.cheb_data_.logZ);
        return (new_config.f_config_[to] ? ratio * exp_beta_mu_f : ratio / exp_beta_mu_f) * std::exp(-beta * ff_diff);
    }
};

}  // namespace chebyshev
}  // namespace fk
