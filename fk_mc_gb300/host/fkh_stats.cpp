// fkh_stats.cpp — C entry points of the statistics and output stage
// (include/fk_mc_host.h): binning and jackknife (include/fk_mc/binning.hpp,
// jackknife.hpp), estimate_bin and save_all (prog/data_save.hpp,
// prog/data_save.hxx), and the graph-lattice loader (src/lattice/graph.cpp).
// None of them touches the GPU.
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "../../include/fk_mc_host.h"
#include "fk_mc/binning.hpp"
#include "fk_mc/data_save.hpp"
#include "fk_mc/jackknife.hpp"
#include "fk_mc/lattice.hpp"

namespace {

int report(const std::exception& e, char* errbuf, int errlen) {
    if (errbuf && errlen > 0) {
        std::strncpy(errbuf, e.what(), (size_t)errlen - 1);
        errbuf[errlen - 1] = '\0';
    }
    return -1;
}

void check_depth(long long n, int max_bin) {
    if (n < 1) throw std::logic_error("empty series");
    if (max_bin < 0 || max_bin > (int)fk::binning::kMaxDepth) throw std::logic_error("max_bin must be in [0, 15]");
}

fk::jackknife::function_t jack_function(int func, int nseries, const double* fparams) {
    switch (func) {
        case FKH_JACK_MEAN:
            if (nseries != 1) throw std::logic_error("FKH_JACK_MEAN takes one series");
            return [](const std::vector<double>& x) { return x[0]; };
        case FKH_JACK_CV: {
            if (nseries != 3 || !fparams) throw std::logic_error("FKH_JACK_CV takes three series and {beta, volume}");
            const double beta = fparams[0], vol = fparams[1];
            return [beta, vol](const std::vector<double>& x) { return beta * beta * (x[1] - x[2] - x[0] * x[0]) / vol; };
        }
        case FKH_JACK_DISP:
            if (nseries != 2) throw std::logic_error("FKH_JACK_DISP takes two series");
            return [](const std::vector<double>& x) { return x[1] - x[0] * x[0]; };
        case FKH_JACK_BINDER:
            if (nseries != 2) throw std::logic_error("FKH_JACK_BINDER takes two series");
            return [](const std::vector<double>& x) { return 1. - x[1] / 3. / x[0] / x[0]; };
        case FKH_JACK_LINEAR: {
            if (nseries < 1 || !fparams) throw std::logic_error("FKH_JACK_LINEAR needs its coefficients");
            std::vector<double> c(fparams, fparams + nseries);
            return [c](const std::vector<double>& x) {
                double s = 0.0;
                for (std::size_t i = 0; i < c.size(); ++i) s += c[i] * x[i];
                return s;
            };
        }
        default: throw std::logic_error("unknown jackknife function");
    }
}

std::vector<std::vector<double>> state_major(const double* p, std::size_t states, std::size_t n) {
    std::vector<std::vector<double>> out;
    if (!p) return out;
    out.assign(states, std::vector<double>(n));
    for (std::size_t i = 0; i < states; ++i)
        for (std::size_t m = 0; m < n; ++m) out[i][m] = p[i * n + m];
    return out;
}

}  // namespace

extern "C" int fkh_binning(const double* x, long long n, int reverse, int max_bin, double* rows, char* errbuf,
                           int errlen) {
    try {
        if (!x || !rows) throw std::logic_error("null argument");
        check_depth(n, max_bin);
        const std::vector<double> v(x, x + n);
        const fk::binning::bin_data_t b = reverse ? fk::binning::accumulate_binning(v.rbegin(), v.rend(), max_bin)
                                                  : fk::binning::accumulate_binning(v.begin(), v.end(), max_bin);
        const std::vector<double> cor = fk::binning::calc_cor_length(b);
        for (std::size_t d = 0; d < b.size(); ++d) {
            rows[5 * d + 0] = (double)std::get<fk::binning::_SIZE>(b[d]);
            rows[5 * d + 1] = std::get<fk::binning::_MEAN>(b[d]);
            rows[5 * d + 2] = std::get<fk::binning::_DISP>(b[d]);
            rows[5 * d + 3] = std::get<fk::binning::_SQERROR>(b[d]);
            rows[5 * d + 4] = cor[d];
        }
        return 0;
    } catch (const std::exception& e) {
        return report(e, errbuf, errlen);
    }
}

extern "C" int fkh_estimate_bin(const double* rows, int nrows, int stride) {
    if (!rows || nrows < 1 || stride < 4) return -1;
    fk::binning::bin_data_t b;
    for (int i = 0; i < nrows; ++i)
        b.emplace_back((std::size_t)rows[i * stride], rows[i * stride + 1], rows[i * stride + 2], rows[i * stride + 3]);
    return (int)fk::binning::estimate_bin(b);
}

extern "C" int fkh_jackknife(int func, int nseries, const double* const* series, long long n, int reverse, int max_bin,
                             const double* fparams, double* rows, char* errbuf, int errlen) {
    try {
        if (!series || !rows || nseries < 1) throw std::logic_error("null argument");
        check_depth(n, max_bin);
        const fk::jackknife::function_t F = jack_function(func, nseries, fparams);
        std::vector<std::vector<double>> data(nseries);
        for (int i = 0; i < nseries; ++i) {
            if (!series[i]) throw std::logic_error("null series");
            data[i].assign(series[i], series[i] + n);
        }
        fk::binning::bin_data_t b;
        if (reverse) {
            typedef std::vector<double>::const_reverse_iterator it_t;
            std::vector<std::pair<it_t, it_t>> r;
            for (const auto& s : data) r.emplace_back(s.crbegin(), s.crend());
            b = fk::jackknife::accumulate_jackknife(F, r, max_bin);
        } else {
            b = fk::jackknife::accumulate_jackknife(F, data, max_bin);
        }
        for (std::size_t d = 0; d < b.size(); ++d) {
            rows[4 * d + 0] = (double)std::get<fk::binning::_SIZE>(b[d]);
            rows[4 * d + 1] = std::get<fk::binning::_MEAN>(b[d]);
            rows[4 * d + 2] = std::get<fk::binning::_DISP>(b[d]);
            rows[4 * d + 3] = std::get<fk::binning::_SQERROR>(b[d]);
        }
        return 0;
    } catch (const std::exception& e) {
        return report(e, errbuf, errlen);
    }
}

extern "C" int fkh_save_stats(const char* dir, const fkh_params* p, const fkh_observables* obs,
                              const fkh_save_options* opt, char* errbuf, int errlen) {
    try {
        if (!dir || !obs || !opt) throw std::logic_error("null argument");
        if (obs->n_meas < 0 || obs->volume < 0) throw std::logic_error("negative sizes");
        const std::size_t M = (std::size_t)obs->n_meas, V = (std::size_t)obs->volume;
        fk::observables_t o;
        auto series = [M](const double* x) { return x ? std::vector<double>(x, x + M) : std::vector<double>(); };
        o.energies = series(obs->energies);
        o.d2energies = series(obs->d2energies);
        o.c_energies = series(obs->c_energies);
        o.nf0 = series(obs->nf0);
        o.nfpi = series(obs->nfpi);
        o.stiffness = series(obs->stiffness);
        if (obs->spectrum) o.spectrum.assign(obs->spectrum, obs->spectrum + obs->n_spectrum);
        o.spectrum_history = state_major(obs->spectrum_history, V, M);
        o.ipr_history = state_major(obs->ipr_history, V, M);
        o.focc_history = state_major(obs->focc_history, V, M);
        o.cond_history = state_major(obs->cond_history, obs->cond_history ? (std::size_t)obs->nw : 0, M);
        if (!o.energies.empty() && o.d2energies.empty()) throw std::logic_error("energies need d2energies");
        fk::save_options so;
        so.beta = opt->beta;
        so.volume = V;
        so.measure_history = opt->measure_history != 0;
        so.measure_ipr = opt->measure_ipr != 0;
        so.measure_stiffness = opt->measure_stiffness != 0;
        so.dos_npts = opt->dos_npts;
        so.dos_width = opt->dos_width;
        so.dos_offset = opt->dos_offset;
        so.max_bin = opt->max_bin;
        if (obs->wgrid_cond && obs->nw > 0) so.wgrid_cond.assign(obs->wgrid_cond, obs->wgrid_cond + obs->nw);
        if (p) {
            so.parameters = {{"lattice_kind", (double)p->lattice_kind}, {"L", (double)p->L}, {"t", p->t}, {"tp", p->tp},
                             {"beta", p->beta}, {"U", p->U}, {"mu_c", p->mu_c}, {"mu_f", p->mu_f},
                             {"random_seed", (double)p->seed}, {"nsweeps", (double)p->nsweeps},
                             {"sweep_len", (double)p->sweep_len}, {"ntherm_sweeps", (double)p->ntherm_sweeps},
                             {"mc_flip", p->mc_flip}, {"mc_add_remove", p->mc_add_remove},
                             {"mc_reshuffle", p->mc_reshuffle}, {"Nf_start", (double)p->nf_start}};
        }
        so.parameters.push_back({"dos_npts", (double)opt->dos_npts});
        so.parameters.push_back({"dos_width", opt->dos_width});
        so.parameters.push_back({"dos_offset", opt->dos_offset});
        fk::data_saver saver(o, so);
        saver.save_all(dir);
        return 0;
    } catch (const std::exception& e) {
        return report(e, errbuf, errlen);
    }
}

extern "C" int fkh_graph_lattice_csr(const char* lattice_dir, int cap_n, int cap_nnz, int* n, int* nnz,
                                     int32_t* rowptr, int32_t* col, double* val, char* errbuf, int errlen) {
    try {
        if (!lattice_dir || !n || !nnz) throw std::logic_error("null argument");
        const fk::graph_lattice l = fk::read_lattice_npy(lattice_dir);
        const fk::csr_matrix& h = l.hopping_m();
        *n = h.rows;
        *nnz = (int)h.val.size();
        if (cap_n < h.rows + 1 || cap_nnz < (int)h.val.size() || !rowptr || !col || !val) return 1;
        for (int i = 0; i <= h.rows; ++i) rowptr[i] = h.rowptr[i];
        for (std::size_t k = 0; k < h.val.size(); ++k) { col[k] = h.col[k]; val[k] = h.val[k]; }
        return 0;
    } catch (const std::exception& e) {
        return report(e, errbuf, errlen);
    }
}
