// configuration.hpp — configuration_t with the reference's interface
// (include/fk_mc/configuration.hpp:52-87); calc_ed runs on the GPU through the
// C ABI of include/fkg.h instead of Eigen::SelfAdjointEigenSolver
// (src/configuration.cpp:208-246). The ed_cache fields, their meaning and the
// cache status machine are the reference's.
#pragma once
#include <numeric>
#include <random>
#include <vector>

#include "chebyshev.hpp"
#include "gpu_backend.hpp"
#include "lattice.hpp"

namespace fk {

typedef std::mt19937 random_generator;  // include/fk_mc/common.hpp:18

struct config_params {
    double beta, U, mu_c, mu_f;
    std::vector<double> W;
    bool operator==(const config_params& rhs) const {
        const double tol = std::numeric_limits<double>::epsilon();
        return std::abs(beta - rhs.beta) < tol && std::abs(U - rhs.U) < tol && std::abs(mu_c - rhs.mu_c) < tol &&
               std::abs(mu_f - rhs.mu_f) < tol;
    }
};

struct ed_cache {
    enum status_eval { empty, spectrum, full };
    status_eval status = empty;
    std::vector<double> cached_spectrum, cached_exp, cached_fermi;
    std::vector<double> cached_evecs;  // column-major msize x msize when status == full
    double logZ = 0.0;
};

// include/fk_mc/configuration.hpp:36-50 (the scaled matrix x stays on the GPU)
struct chebyshev_cache {
    enum status_eval { empty, logz };
    status_eval status = empty;
    double e_max = 0.0, e_min = 0.0;
    double a = 0.0;  // (e_max - e_min)/2
    double b = 0.0;  // (e_max + e_min)/2
    std::vector<double> moments;
    double logZ = 0.0;
};

struct configuration_t {
    typedef std::vector<double> real_array_t;
    typedef std::vector<int> int_array_t;

    configuration_t(const abstract_lattice& lattice, double beta, double U, double mu_c, double mu_f,
                    std::vector<double> W = {})
        : lattice_(lattice), params_({beta, U, mu_c, mu_f, W}), f_config_(lattice.volume(), 0) {}
    configuration_t(const configuration_t&) = default;
    configuration_t& operator=(const configuration_t& rhs) {  // src/configuration.cpp:32-40
        f_config_ = rhs.f_config_;
        diag_ = rhs.diag_;
        ed_data_ = rhs.ed_data_;
        cheb_data_ = rhs.cheb_data_;
        if (!(params_ == rhs.params_)) throw std::logic_error("Mismatched parameters in config assignment");
        return *this;
    }

    std::size_t get_nf() const { return std::accumulate(f_config_.begin(), f_config_.end(), (std::size_t)0); }

    void randomize_f(random_generator& rnd, std::size_t nf = 0) {  // src/configuration.cpp:47-56
        std::uniform_int_distribution<> distr(0, (int)lattice_.volume() - 1);
        if (!nf) nf = distr(rnd);
        std::fill(f_config_.begin(), f_config_.end(), 0);
        for (std::size_t i = 0; i < nf; ++i) {
            std::size_t ind = distr(rnd);
            while (f_config_[ind] == 1) ind = distr(rnd);
            f_config_[ind] = 1;
        }
    }

    double calc_ff_energy() const {  // src/configuration.cpp:59-77
        if (lattice_.ndim() != 1) return 0;
        double e = 0;
        const int V = (int)lattice_.volume();
        for (int i = 0; i < V; ++i) {
            if (!f_config_[i]) continue;
            for (int l = 0; l < (int)params_.W.size(); ++l) {
                const int left = (i - l + V) % V, right = (i + l) % V;
                e += params_.W[l] * f_config_[left];
                e += params_.W[l] * f_config_[right] * (l > 0);
            }
        }
        return e;
    }

    // H = hopping + diag(-mu_c + U f) (src/configuration.cpp:79-91): the
    // hopping part lives on the GPU, the diagonal is kept here.
    const std::vector<double>& calc_hamiltonian() {
        reset_cache();
        const std::size_t norbs = lattice_.norbs();
        diag_.assign(lattice_.msize(), 0.0);
        for (std::size_t i = 0; i < lattice_.volume(); ++i)
            for (std::size_t o = 0; o < norbs; ++o) diag_[i * norbs + o] = -params_.mu_c + params_.U * f_config_[i];
        return diag_;
    }
    void reset_cache() {
        ed_data_.status = ed_cache::empty;
        cheb_data_.status = chebyshev_cache::empty;
    }

    // src/configuration.cpp:94-205 on the GPU (fkg_chebyshev_logz, batch 1):
    // spectral bounds, moments and logZ of the Chebyshev expansion
    void calc_chebyshev(const chebyshev::chebyshev_eval& cheb) {
        if (cheb_data_.status == chebyshev_cache::logz) return;
        if (diag_.size() != lattice_.msize()) calc_hamiltonian();
        gpu_backend& g = gpu_backend::instance();
        const int id = g.lattice_id(lattice_);
        g.set_chebyshev(cheb.cheb_size(), cheb.grid_size());
        cheb_data_.moments.resize(cheb.cheb_size());
        double beta = params_.beta;
        g.check(fkg_chebyshev_logz(g.ctx(), 1, &id, diag_.data(), &beta, &cheb_data_.logZ, &cheb_data_.e_min,
                                   &cheb_data_.e_max, cheb_data_.moments.data(), nullptr),
                "fkg_chebyshev_logz");
        cheb_data_.a = (cheb_data_.e_max - cheb_data_.e_min) / 2.;
        cheb_data_.b = (cheb_data_.e_max + cheb_data_.e_min) / 2.;
        cheb_data_.status = chebyshev_cache::logz;
    }
    const chebyshev_cache& cheb_data() const { return cheb_data_; }

    // src/configuration.cpp:208-246 on the GPU (fkg_eigh_logz, batch 1)
    void calc_ed(bool calc_evecs = false) {
        if ((ed_data_.status == ed_cache::spectrum && !calc_evecs) || (ed_data_.status == ed_cache::full && calc_evecs))
            return;
        if (diag_.size() != lattice_.msize()) calc_hamiltonian();
        gpu_backend& g = gpu_backend::instance();
        const int id = g.lattice_id(lattice_);
        const std::size_t n = lattice_.msize();
        ed_data_.cached_spectrum.resize(n);
        ed_data_.cached_exp.resize(n);
        ed_data_.cached_fermi.resize(n);
        if (calc_evecs) ed_data_.cached_evecs.resize(n * n);
        double beta = params_.beta;
        g.check(fkg_eigh_logz(g.ctx(), 1, &id, diag_.data(), &beta, ed_data_.cached_spectrum.data(),
                              ed_data_.cached_exp.data(), ed_data_.cached_fermi.data(),
                              calc_evecs ? ed_data_.cached_evecs.data() : nullptr, &ed_data_.logZ),
                "fkg_eigh_logz");
        ed_data_.status = calc_evecs ? ed_cache::full : ed_cache::spectrum;
    }

    // a spectrum computed elsewhere (the rank-one update): ed_cache filled as
    // calc_ed fills it (src/configuration.cpp:224-245), without eigenvectors
    void set_spectrum(const std::vector<double>& spectrum, double logz) {
        const std::size_t n = spectrum.size();
        ed_data_.cached_spectrum = spectrum;
        ed_data_.cached_exp.resize(n);
        ed_data_.cached_fermi.resize(n);
        for (std::size_t i = 0; i < n; ++i) {
            ed_data_.cached_exp[i] = std::exp(params_.beta * spectrum[i]);
            ed_data_.cached_fermi[i] = 1.0 / (1.0 + ed_data_.cached_exp[i]);
        }
        ed_data_.logZ = logz;
        ed_data_.status = ed_cache::spectrum;
    }

    const config_params& params() const { return params_; }
    const ed_cache& ed_data() const { return ed_data_; }

    const abstract_lattice& lattice_;
    const config_params params_;
    int_array_t f_config_;
    std::vector<double> diag_;  // diagonal of H (the hopping part is shared on the GPU)
    ed_cache ed_data_;
    chebyshev_cache cheb_data_;
};

}  // namespace fk
