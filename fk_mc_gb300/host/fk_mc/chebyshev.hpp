// chebyshev.hpp — chebyshev::chebyshev_eval with the reference's interface
// (include/fk_mc/chebyshev.hpp:8-66): the number of Chebyshev moments (rounded
// up to even) and the Lobatto grid x_i = -cos(pi theta_i), theta uniform on
// [0, 1], on which the coefficients are integrated by the trapezoid rule in
// theta. moment_f evaluates a coefficient on the host; configuration_t's
// calc_chebyshev passes cheb_size() and grid_size() to the GPU, which
// evaluates the same coefficients for logZ.
#pragma once
#include <cmath>
#include <cstddef>
#include <stdexcept>
#include <vector>

namespace fk {
namespace chebyshev {

inline double chebyshev_t(double x, std::size_t n) {
    if (!(std::abs(x) <= 1)) throw std::logic_error("chebyshev_t argument outside [-1, 1]");
    return std::cos(n * std::acos(x));
}

struct chebyshev_eval {
    int cheb_size() const { return M_; }
    int grid_size() const { return (int)angle_grid_.size(); }

    chebyshev_eval(int max_moment, int grid_size) : M_(max_moment + max_moment % 2) {
        if (max_moment < 1 || grid_size < 2) throw std::logic_error("chebyshev_eval needs max_moment >= 1, grid_size >= 2");
        const double step = 1.0 / (double)(grid_size - 1);
        for (int i = 0; i < grid_size; ++i) {
            angle_grid_.push_back((double)i * step);
            lobatto_grid_.push_back(-std::cos(M_PI * angle_grid_.back()));
        }
        chebt_cache_.resize((std::size_t)M_ * grid_size);
        for (int k = 0; k < M_; ++k)
            for (int i = 0; i < grid_size; ++i)
                chebt_cache_[(std::size_t)k * grid_size + i] = chebyshev_t(lobatto_grid_[i], (std::size_t)k);
    }

    template <typename F>
    double moment_f(const F& op, int order) const {
        std::vector<double> vals(angle_grid_.size());
        for (std::size_t i = 0; i < angle_grid_.size(); ++i) vals[i] = op(lobatto_grid_[i]);
        return moment(vals, order);
    }

    template <class V>
    double moment(const V& in, int order) const {
        const int G = grid_size();
        double s = 0.0;
        for (int i = 0; i + 1 < G; ++i)
            s += (in[i + 1] * chebt_cache_[(std::size_t)order * G + i + 1] + in[i] * chebt_cache_[(std::size_t)order * G + i]) *
                 (angle_grid_[i + 1] - angle_grid_[i]);
        return s * 0.5;
    }

private:
    int M_;
    std::vector<double> angle_grid_, lobatto_grid_, chebt_cache_;
};

}  // namespace chebyshev
}  // namespace fk
