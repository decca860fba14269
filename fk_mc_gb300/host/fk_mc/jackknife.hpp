// jackknife.hpp — jackknife estimate of a function F(<x_1>, <x_2>, ...) of
// the means of several time series, as the reference's
// include/fk_mc/jackknife.hpp defines it (jackknife_adapter::jack,
// jackknife.hpp:47-80):
//   * every series is binned at the same depth (binning.hpp);
//   * U_0 = F(means); U_j = F(means with bin j left out), the left-out mean
//     being (size * mean - x_j) / (size - 1);
//   * with U_bar and err_U the mean and sqrt(var / size) of the U_j, the
//     estimate is U_0 - (size - 1) (U_bar - U_0) with error
//     dU = (size - 1) err_U, and the returned statistics are
//     (size, estimate, dU^2 * size, dU).
// accumulate_jackknife returns those for depths 0..max_depth
// (jackknife.hpp:85-115, 148-157). F takes a std::vector<double> of the means.
#pragma once

#include <functional>
#include <stdexcept>
#include <utility>
#include <vector>

#include "binning.hpp"

namespace fk {
namespace jackknife {

using binning::bin_data_t;
using binning::bin_stats_t;

typedef std::function<double(const std::vector<double>&)> function_t;

// jackknife over already-binned series (all of the same length)
inline bin_stats_t jack_binned(const function_t& F, const std::vector<std::vector<double>>& x) {
    if (x.empty()) throw std::logic_error("jackknife of no series");
    const std::size_t L = x.size(), size = x[0].size();
    for (const auto& s : x)
        if (s.size() != size) throw std::logic_error("Argument size mismatch for jackknife");
    std::vector<double> x_means(L);
    for (std::size_t i = 0; i < L; ++i) x_means[i] = std::get<binning::_MEAN>(binning::calc_stats(x[i].begin(), x[i].end()));
    const double U_0 = F(x_means);
    std::vector<double> U(size), loo(L);
    for (std::size_t j = 0; j < size; ++j) {
        for (std::size_t i = 0; i < L; ++i) loo[i] = (double(size) * x_means[i] - x[i][j]) / (double(size - 1));
        U[j] = F(loo);
    }
    const bin_stats_t U_stats = binning::calc_stats(U.begin(), U.end());
    const double U_bar = std::get<binning::_MEAN>(U_stats);
    const double U_average = U_0 - (size - 1) * (U_bar - U_0);
    const double dU = (size - 1) * std::get<binning::_SQERROR>(U_stats);
    return std::make_tuple(size, U_average, dU * dU * size, dU);
}

// series given as iterator pairs (forward or reverse), binned at `depth`
template <typename iter_t>
bin_stats_t jack(const function_t& F, const std::vector<std::pair<iter_t, iter_t>>& in, std::size_t depth) {
    std::vector<std::vector<double>> x;
    x.reserve(in.size());
    for (const auto& r : in) x.push_back(binning::binned_values(r.first, r.second, depth));
    return jack_binned(F, x);
}

inline bin_stats_t jack(const function_t& F, const std::vector<std::vector<double>>& in, std::size_t depth) {
    typedef std::vector<double>::const_iterator it_t;
    std::vector<std::pair<it_t, it_t>> r;
    for (const auto& s : in) r.emplace_back(s.begin(), s.end());
    return jack(F, r, depth);
}

template <typename iter_t>
bin_data_t accumulate_jackknife(const function_t& F, const std::vector<std::pair<iter_t, iter_t>>& in,
                                std::size_t max_depth) {
    if (max_depth > binning::kMaxDepth)
        throw std::logic_error("bin_depth =" + std::to_string(max_depth) + "> compiled bin size");
    bin_data_t out;
    for (std::size_t d = 0; d <= max_depth; ++d) out.push_back(jack(F, in, d));
    return out;
}

inline bin_data_t accumulate_jackknife(const function_t& F, const std::vector<std::vector<double>>& in,
                                       std::size_t max_depth) {
    typedef std::vector<double>::const_iterator it_t;
    std::vector<std::pair<it_t, it_t>> r;
    for (const auto& s : in) r.emplace_back(s.begin(), s.end());
    return accumulate_jackknife(F, r, max_depth);
}

}  // namespace jackknife
}  // namespace fk
