// batched_mc.hpp — B independent Markov chains on one GPU, each one what a
// reference MPI rank runs (mc_metropolis seeded SEED + rank,
// src/mc_metropolis.cpp:25, with move_addremove as its only move,
// include/fk_mc/fk_mc.hxx:71-74). For single-site flips the random draws of a
// proposal (move index, site, Metropolis uniform — src/mc_metropolis.cpp:41-43,
// src/moves.cpp:55-57) do not depend on the chain's state, so the host draws
// them from each chain's own std::mt19937 and the GPU runs one batched
// propose/solve/accept step for all chains (fkg_propose_accept). With
// cheb_size > 0 the chains take logZ from the Chebyshev expansion
// (chebyshev::move_addremove, src/moves_chebyshev.cpp:54-72, which draws the
// same numbers in the same order) through FKG_METHOD_CHEBYSHEV.
#pragma once
#include <cmath>
#include <random>
#include <stdexcept>
#include <vector>

#include "configuration.hpp"

namespace fk {

struct batched_mc {
    batched_mc(const abstract_lattice& lattice, double beta, double U, double mu_c, double mu_f,
               const std::vector<long>& seeds, int nf_start, int precision = FKG_PREC_F64, int cheb_size = 0,
               int cheb_grid = 0)
        : lattice_(lattice), beta_(beta), U_(U), mu_c_(mu_c), mu_f_(mu_f), B_((int)seeds.size()), cheb_(cheb_size > 0) {
        gpu_backend& g = gpu_backend::instance();
        g.check(fkg_set_precision(g.ctx(), precision), "fkg_set_precision");
        if (cheb_) g.set_chebyshev(cheb_size, cheb_grid);
        g.check(fkg_set_method(g.ctx(), cheb_ ? FKG_METHOD_CHEBYSHEV : FKG_METHOD_ED), "fkg_set_method");
        const int id = g.lattice_id(lattice);
        const int V = (int)lattice.volume();
        std::vector<int> f((size_t)B_ * V);
        for (int c = 0; c < B_; ++c) {
            rngs_.emplace_back((std::mt19937::result_type)seeds[c]);
            configuration_t cfg(lattice, beta, U, mu_c, mu_f);
            cfg.randomize_f(rngs_.back(), nf_start);  // fk_mc::initialize (include/fk_mc/fk_mc.hxx:46)
            std::copy(cfg.f_config_.begin(), cfg.f_config_.end(), f.begin() + (size_t)c * V);
            const double w1[1] = {1.0};
            move_distrib_.emplace_back(w1, w1 + 1);
        }
        f_initial_ = f;
        std::vector<int> ids(B_, id);
        std::vector<double> Us(B_, U), mcs(B_, mu_c), mfs(B_, mu_f), bs(B_, beta);
        g.check(fkg_chains_init(g.ctx(), B_, ids.data(), f.data(), Us.data(), mcs.data(), mfs.data(), bs.data()),
                "fkg_chains_init");
    }

    // one sweep of sweep_len proposals on every chain; appends the accept flags
    void update(int sweep_len, std::vector<int>* accepted = nullptr, std::vector<int>* sites = nullptr) {
        gpu_backend& g = gpu_backend::instance();
        std::vector<int> site(B_), acc(B_);
        std::vector<double> u(B_), dl(B_);
        std::uniform_int_distribution<> distr(0, (int)lattice_.volume() - 1);
        std::uniform_real_distribution<> metropolis(0, 1);
        for (int m = 0; m < sweep_len; ++m) {
            for (int c = 0; c < B_; ++c) {
                move_distrib_[c](rngs_[c]);       // move choice (one registered move)
                site[c] = distr(rngs_[c]);        // move_addremove::attempt
                u[c] = metropolis(rngs_[c]);      // mc_metropolis::update
            }
            g.check(fkg_propose_accept(g.ctx(), 1, site.data(), u.data(), acc.data(), dl.data()), "fkg_propose_accept");
            if (accepted) accepted->insert(accepted->end(), acc.begin(), acc.end());
            if (sites) sites->insert(sites->end(), site.begin(), site.end());
        }
    }

    // measure_energy::accumulate (src/measures/energy.cpp:6-26) on every chain
    void measure_energy(std::vector<double>& e, std::vector<double>& d2e, std::vector<double>& ec) {
        gpu_backend& g = gpu_backend::instance();
        const int V = (int)lattice_.volume();
        std::vector<int> f((size_t)B_ * V);
        std::vector<double> logz(B_), w((size_t)B_ * V);
        g.check(fkg_chains_get(g.ctx(), f.data(), logz.data(), w.data()), "fkg_chains_get");
        for (int c = 0; c < B_; ++c) {
            double s = 0.0, s2 = 0.0, nf = 0.0;
            for (int i = 0; i < V; ++i) {
                const double eps = w[(size_t)c * V + i], ex = std::exp(beta_ * eps);
                s += eps / (1.0 + ex);
                s2 += eps * eps / (1.0 + 0.5 * (ex + 1. / ex));
                nf += f[(size_t)c * V + i];
            }
            ec.push_back(s);
            e.push_back(s - mu_f_ * nf);
            d2e.push_back(s2 / 2.0);
        }
    }

    void get_state(std::vector<int>& f, std::vector<double>& logz) {
        gpu_backend& g = gpu_backend::instance();
        f.resize((size_t)B_ * lattice_.volume());
        logz.resize(B_);
        g.check(fkg_chains_get(g.ctx(), f.data(), logz.data(), nullptr), "fkg_chains_get");
    }

    ~batched_mc() {  // the thread's context goes back to the eigen-solve for other users
        if (cheb_) fkg_set_method(gpu_backend::instance().ctx(), FKG_METHOD_ED);
    }

    const abstract_lattice& lattice_;
    double beta_, U_, mu_c_, mu_f_;
    int B_;
    bool cheb_;
    std::vector<std::mt19937> rngs_;
    std::vector<std::discrete_distribution<>> move_distrib_;
    std::vector<int> f_initial_;
};

}  // namespace fk
