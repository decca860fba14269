// binning.hpp — binning analysis of a Monte Carlo time series, as the
// reference's include/fk_mc/binning.hpp defines it:
//   * a bin of depth D is the average of 2^D consecutive samples, formed by
//     repeated pairwise averaging ((a + b) / 2 of the two bins of depth D-1,
//     binning.hpp:37-38), and a series of `size` samples gives size / 2^D
//     bins (calc_bin_size, binning.hpp:70-78; the incomplete tail is dropped);
//   * the statistics of a set of bins are (size, mean, variance with the
//     size-1 denominator, sqrt(variance / size)) (calc_stats, binning.hpp:90-97);
//   * accumulate_binning returns those statistics for depths 0..max_depth
//     (binning.hpp:106-130, 146-160);
//   * the correlation-length estimate of depth i is
//     0.5 * (2^i * var_i / var_0 - 1) (calc_cor_length, binning.hpp:168-176).
// The series is read through any random-access iterator pair, so the
// reference's reversed reads (energies.rbegin(), prog/data_save.hxx:171) are
// a pair of reverse iterators here too. A depth whose bin is longer than the
// series throws, like FKMC_ERROR (binning.hpp:72-75).
#pragma once

#include <cmath>
#include <cstddef>
#include <iterator>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

namespace fk {
namespace binning {

enum bin_m : std::size_t { _SIZE, _MEAN, _DISP, _SQERROR };
typedef std::tuple<std::size_t, double, double, double> bin_stats_t;
typedef std::vector<bin_stats_t> bin_data_t;

// the deepest bin the reference compiles (BINNING_RANGE, binning.hpp:17)
constexpr std::size_t kMaxDepth = 15;

inline std::size_t calc_bin_size(std::size_t size, std::size_t bin_step) {
    if (bin_step > size)
        throw std::logic_error("Can't bin with binning step(" + std::to_string(bin_step) + ")> container size (" +
                               std::to_string(size) + ")");
    return size / bin_step;
}

// Bins of depth `depth` of [begin, end): level d is built from level d-1 by
// (x[2k] + x[2k+1]) / 2, the same operations in the same order as the
// reference's recursive dereference.
template <typename iter_t>
std::vector<double> binned_values(iter_t begin, iter_t end, std::size_t depth) {
    if (depth > kMaxDepth) throw std::logic_error("bin_depth =" + std::to_string(depth) + "> compiled bin size");
    const std::size_t size = (std::size_t)std::distance(begin, end);
    const std::size_t nbins = calc_bin_size(size, std::size_t(1) << depth);
    std::vector<double> level(begin, begin + (std::ptrdiff_t)(nbins << depth));
    for (std::size_t d = 0; d < depth; ++d) {
        const std::size_t half = level.size() / 2;
        for (std::size_t k = 0; k < half; ++k) level[k] = (level[2 * k] + level[2 * k + 1]) / 2.;
        level.resize(half);
    }
    return level;
}

template <typename iter_t>
bin_stats_t calc_stats(iter_t begin, iter_t end, std::size_t size = 0) {
    if (!size) size = (std::size_t)std::distance(begin, end);
    double sum = 0.0;
    for (iter_t it = begin; it != end; ++it) sum += *it;
    const double mean = sum / size;
    double sq = 0.0;
    for (iter_t it = begin; it != end; ++it) sq += (*it - mean) * (*it - mean);
    const double variance = sq / (size - 1);
    return std::make_tuple(size, mean, variance, std::sqrt(variance / size));
}

template <typename iter_t>
bin_stats_t bin(iter_t begin, iter_t end, std::size_t depth) {
    const std::vector<double> v = binned_values(begin, end, depth);
    return calc_stats(v.begin(), v.end());
}

template <typename container_t>
bin_stats_t bin(const container_t& in, std::size_t depth) {
    return bin(in.begin(), in.end(), depth);
}

template <typename iter_t>
bin_data_t accumulate_binning(iter_t begin, iter_t end, std::size_t max_depth) {
    if (max_depth > kMaxDepth) throw std::logic_error("bin_depth =" + std::to_string(max_depth) + "> compiled bin size");
    bin_data_t out;
    out.reserve(max_depth + 1);
    for (std::size_t d = 0; d <= max_depth; ++d) out.push_back(bin(begin, end, d));
    return out;
}

template <typename container_t>
bin_data_t accumulate_binning(const container_t& in, std::size_t max_depth) {
    return accumulate_binning(in.begin(), in.end(), max_depth);
}

inline std::vector<double> calc_cor_length(const bin_data_t& in) {
    std::vector<double> out(in.size());
    if (in.empty()) return out;
    const double sigma = std::get<_DISP>(in[0]);
    for (std::size_t i = 0; i < in.size(); ++i) out[i] = 0.5 * (std::pow(2., (double)i) * std::get<_DISP>(in[i]) / sigma - 1);
    return out;
}

// The depth at which the error bar has saturated: walking down from the
// deepest bin while consecutive errors differ by less than 5% and the
// difference keeps shrinking (estimate_bin, prog/data_save.hpp:108-122).
inline std::size_t estimate_bin(const bin_data_t& data) {
    if (data.empty()) return 0;
    double rel_error = 1.;
    std::size_t ind = data.size() - 1;
    bool f = true;
    while (f && ind > 0) {
        const double cur = std::abs(std::get<_SQERROR>(data[ind - 1]) / std::get<_SQERROR>(data[ind]) - 1.);
        f = (cur < 0.05 && cur < rel_error);
        if (f) {
            rel_error = cur;
            ind--;
        }
    }
    return ind;
}

}  // namespace binning
}  // namespace fk
