// data_save.hpp — the statistics and output stage of a run, as the
// reference's data_saver does it (prog/data_save.hpp:30-161,
// prog/data_save.hxx:32-530), with one .npy file per HDF5 dataset: the HDF5
// group "/mc_data" becomes the directory <dir>/mc_data, "/binning" becomes
// <dir>/binning, "/stats" becomes <dir>/stats, and "/parameters" becomes
// <dir>/parameters.json. <dir>/stats.json repeats every /stats entry with its
// bin depth, for reading by eye.
//
// What is written, per reference function:
//   save_measurements (data_save.hxx:104-153): the measured series;
//   save_energy (:157-199): binning of energy, d2energy, c_energy and the
//     jackknifed specific heat cv = beta^2 (<E^2> - <d2E> - <E>^2) / volume;
//   save_fstats (:202-236): binning of nf(q=0), nf(q=pi), the jackknifed
//     susceptibilities <n^2> - <n>^2 and Binder cumulants 1 - <n^4>/(3<n^2>^2);
//   save_glocal (:266-345): the local density of states at w = 0 (binned),
//     on a real grid (dos_err) and its integral against the Fermi function (nc);
//   save_ipr (:486-530): the Lorentzian-weighted inverse participation ratio
//     at w = 0 (binned) and on the real grid (ipr_err);
//   save_conductivity (:425-484): binning of the Drude stiffness, w*sigma(w)
//     with error bars (wcond_err), the dc limit (cond0), sigma(w) (cond_err)
//     and sigma(w) - sigma(0) (cond_dynamic).
// Every binned quantity is saved as the reference's save_binning does
// (prog/data_save.hpp:137-156): the rows (size, mean, variance, error,
// correlation length) for every depth under /binning and the row at the depth
// estimate_bin picks under /stats.
//
// Where the reference would fail this one does not: it takes the number of
// measurements from nf(q=pi) (data_save.hpp:89), and with no nf(q=pi)
// series its binning of the density of states throws; here the number of
// energy measurements is used instead.
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <fstream>
#include <map>
#include <string>
#include <sys/stat.h>
#include <utility>
#include <vector>

#include "binning.hpp"
#include "jackknife.hpp"
#include "npy.hpp"

namespace fk {

// The measured series (include/fk_mc/fk_mc.hpp:13-34); histories are
// indexed [state][measurement] as the reference stores them.
struct observables_t {
    std::vector<double> energies, c_energies, d2energies, nf0, nfpi, spectrum, stiffness;
    std::vector<std::vector<double>> spectrum_history, ipr_history, cond_history, focc_history;
};

struct save_options {
    double beta = 1.0;
    std::size_t volume = 0;                 // lattice msize
    bool measure_history = true, measure_ipr = false, measure_stiffness = false;
    int dos_npts = 240;                     // prog/fk_mc_exec.cpp:205-207
    double dos_width = 6.0, dos_offset = 0.05;
    std::vector<double> wgrid_cond;         // conductivity frequencies
    int max_bin = -1;                       // < 0: the reference's rule (data_save.hpp:90)
    std::vector<std::pair<std::string, double>> parameters;  // written to parameters.json
};

// The reference's default maximal bin depth for n measurements
// (data_save.hpp:90): min(15, max(int(log2(n / 16) - 1), 1)).
inline int default_max_bin(std::size_t n) {
    if (n == 0) return 1;
    const double v = std::log(double(n) / 16) / std::log(2.) - 1;
    return std::min(15, std::max(v < -1e9 ? 1 : int(v), 1));
}

namespace detail {

inline void make_dir(const std::string& d) {
    if (::mkdir(d.c_str(), 0755) != 0) {
        struct stat st;
        if (::stat(d.c_str(), &st) != 0 || !S_ISDIR(st.st_mode)) throw std::runtime_error("cannot create directory " + d);
    }
}

inline std::string json_number(double v) {
    if (!std::isfinite(v)) return "null";
    char buf[40];
    std::snprintf(buf, sizeof buf, "%.17g", v);
    return buf;
}

}  // namespace detail

class data_saver {
public:
    typedef binning::bin_data_t bin_data_t;
    typedef binning::bin_stats_t bin_stats_t;

    data_saver(const observables_t& obs, save_options opt) : obs_(obs), opt_(std::move(opt)) {
        nmeasures_ = obs_.nfpi.size() ? obs_.nfpi.size() : obs_.energies.size();
        max_bin_ = opt_.max_bin >= 0 ? opt_.max_bin : default_max_bin(nmeasures_);
        volume_ = opt_.volume;
    }

    int max_bin() const { return max_bin_; }
    std::size_t nmeasures() const { return nmeasures_; }

    // results, also kept in memory: name -> rows of every depth, name ->
    // (depth, statistics), name -> table (rows of columns)
    std::map<std::string, bin_data_t> binning_out;
    std::map<std::string, std::pair<int, bin_stats_t>> stats_out;
    std::map<std::string, std::vector<std::vector<double>>> tables_out;

    // compute everything; write it under `dir` when dir is not empty
    void save_all(const std::string& dir) {
        dir_ = dir;
        if (!dir_.empty()) {
            detail::make_dir(dir_);
            for (const char* g : {"mc_data", "binning", "stats"}) detail::make_dir(dir_ + "/" + g);
            save_parameters();
            save_measurements();
        }
        if (!obs_.energies.empty()) save_energy();
        if (!obs_.nf0.empty() && !obs_.nfpi.empty()) save_fstats();
        std::vector<double> grid_real(opt_.dos_npts);
        for (int i = 0; i < opt_.dos_npts; ++i) grid_real[i] = -opt_.dos_width + 2. * opt_.dos_width * i / (1. * opt_.dos_npts);
        if (opt_.measure_history && !obs_.spectrum_history.empty()) save_glocal(grid_real);
        if (opt_.measure_ipr && !obs_.ipr_history.empty() && !obs_.spectrum_history.empty()) save_ipr(grid_real);
        if (opt_.measure_stiffness && !obs_.stiffness.empty()) save_conductivity(opt_.wgrid_cond);
        if (!dir_.empty()) write_stats_json();
    }

private:
    const observables_t& obs_;
    save_options opt_;
    std::size_t nmeasures_ = 0, volume_ = 0;
    int max_bin_ = 1;
    std::string dir_;

    void save_parameters() {
        std::ofstream out(dir_ + "/parameters.json");
        out << "{";
        for (std::size_t i = 0; i < opt_.parameters.size(); ++i)
            out << (i ? ", " : "") << "\"" << opt_.parameters[i].first << "\": " << detail::json_number(opt_.parameters[i].second);
        out << "}\n";
    }

    void write_npy(const std::string& group, const std::string& name, const std::vector<double>& v) {
        if (!dir_.empty()) npy::write(dir_ + "/" + group + "/" + name + ".npy", v);
    }
    void write_npy(const std::string& group, const std::string& name, const std::vector<std::vector<double>>& m) {
        if (!dir_.empty()) npy::write(dir_ + "/" + group + "/" + name + ".npy", m);
    }

    void save_measurements() {
        const std::pair<const char*, const std::vector<double>*> series[] = {
            {"energies", &obs_.energies}, {"d2energies", &obs_.d2energies}, {"c_energies", &obs_.c_energies},
            {"nf0", &obs_.nf0},           {"nfpi", &obs_.nfpi},             {"stiffness", &obs_.stiffness},
            {"spectrum", &obs_.spectrum}};
        for (const auto& s : series)
            if (!s.second->empty()) write_npy("mc_data", s.first, *s.second);
        if (opt_.measure_history) {
            if (!obs_.spectrum_history.empty()) write_npy("mc_data", "spectrum_history", obs_.spectrum_history);
            if (!obs_.focc_history.empty()) write_npy("mc_data", "focc_history", obs_.focc_history);
            if (opt_.measure_ipr && !obs_.ipr_history.empty()) write_npy("mc_data", "ipr_history", obs_.ipr_history);
        }
        if (opt_.measure_stiffness && !obs_.cond_history.empty()) write_npy("mc_data", "cond_history", obs_.cond_history);
    }

    void save_bin_data(const bin_stats_t& s, const std::string& name, int bin) {
        stats_out[name] = {bin, s};
        write_npy("stats", name, std::vector<double>{double(std::get<binning::_SIZE>(s)), std::get<binning::_MEAN>(s),
                                                     std::get<binning::_DISP>(s), std::get<binning::_SQERROR>(s)});
    }

    void save_binning(const bin_data_t& data, const std::string& name) {
        binning_out[name] = data;
        const std::vector<double> cor = binning::calc_cor_length(data);
        std::vector<std::vector<double>> rows;
        for (std::size_t i = 0; i < data.size(); ++i)
            rows.push_back({double(std::get<binning::_SIZE>(data[i])), std::get<binning::_MEAN>(data[i]),
                            std::get<binning::_DISP>(data[i]), std::get<binning::_SQERROR>(data[i]), cor[i]});
        write_npy("binning", name, rows);
        const std::size_t b = binning::estimate_bin(data);
        save_bin_data(data[b], name, (int)b);
    }

    void save_table(const std::string& name, const std::vector<std::vector<double>>& rows) {
        tables_out[name] = rows;
        write_npy("stats", name, rows);
    }

    void save_energy() {
        const auto& e = obs_.energies;
        save_binning(binning::accumulate_binning(e.rbegin(), e.rend(), max_bin_), "energy");
        save_binning(binning::accumulate_binning(obs_.d2energies.rbegin(), obs_.d2energies.rend(), max_bin_), "d2energy");
        if (!obs_.c_energies.empty())
            save_binning(binning::accumulate_binning(obs_.c_energies.rbegin(), obs_.c_energies.rend(), max_bin_), "c_energy");
        std::vector<double> e2(e.size());
        for (std::size_t i = 0; i < e.size(); ++i) e2[i] = e[i] * e[i];
        const double beta = opt_.beta, vol = double(volume_);
        jackknife::function_t cv = [beta, vol](const std::vector<double>& x) {
            return beta * beta * (x[1] - x[2] - x[0] * x[0]) / vol;
        };
        typedef std::vector<double>::const_reverse_iterator it_t;
        std::vector<std::pair<it_t, it_t>> data = {{e.rbegin(), e.rend()}, {e2.crbegin(), e2.crend()},
                                                   {obs_.d2energies.rbegin(), obs_.d2energies.rend()}};
        save_binning(jackknife::accumulate_jackknife(cv, data, max_bin_), "cv");
    }

    void save_fstats() {
        const auto& nf0 = obs_.nf0;
        const auto& nfpi = obs_.nfpi;
        std::vector<double> nn_0(nf0.size()), nn_pi(nfpi.size()), n4_0(nf0.size()), n4_pi(nfpi.size());
        for (std::size_t i = 0; i < nf0.size(); ++i) { nn_0[i] = nf0[i] * nf0[i]; n4_0[i] = nf0[i] * nf0[i] * nf0[i] * nf0[i]; }
        for (std::size_t i = 0; i < nfpi.size(); ++i) { nn_pi[i] = nfpi[i] * nfpi[i]; n4_pi[i] = nfpi[i] * nfpi[i] * nfpi[i] * nfpi[i]; }
        jackknife::function_t disp = [](const std::vector<double>& x) { return x[1] - x[0] * x[0]; };
        save_binning(binning::accumulate_binning(nf0.rbegin(), nf0.rend(), max_bin_), "nf_0");
        save_binning(binning::accumulate_binning(nfpi.rbegin(), nfpi.rend(), max_bin_), "nf_pi");
        const bin_data_t fsusc0 = jackknife::accumulate_jackknife(disp, {nf0, nn_0}, max_bin_);
        save_binning(fsusc0, "fsusc_0");
        save_binning(jackknife::accumulate_jackknife(disp, {nfpi, nn_pi}, max_bin_), "fsusc_pi");
        jackknife::function_t binder = [](const std::vector<double>& x) { return 1. - x[1] / 3. / x[0] / x[0]; };
        const std::size_t nf_bin = binning::estimate_bin(fsusc0);
        save_bin_data(jackknife::jack(binder, {nn_0, n4_0}, nf_bin), "binder_0", (int)nf_bin);
        save_bin_data(jackknife::jack(binder, {nn_pi, n4_pi}, nf_bin), "binder_pi", (int)nf_bin);
    }

    // spectrum of measurement m (the history is stored [state][measurement])
    std::vector<double> spectrum_of(std::size_t m) const {
        std::vector<double> s(volume_);
        for (std::size_t i = 0; i < volume_; ++i) s[i] = obs_.spectrum_history.at(i).at(m);
        return s;
    }

    void save_glocal(const std::vector<double>& grid_real) {
        const double offset = opt_.dos_offset, beta = opt_.beta;
        const std::size_t vol = volume_;
        auto dos0_f = [offset, vol](const std::vector<double>& spec, double z) {
            std::complex<double> d = 0.0;
            for (std::size_t i = 0; i < spec.size(); ++i) d += 1. / (std::complex<double>(z, 0.) - spec[i] + std::complex<double>(0., offset));
            return -(std::imag(d) / (double)vol) / M_PI;
        };
        std::vector<std::vector<double>> specs(nmeasures_);
        for (std::size_t m = 0; m < nmeasures_; ++m) specs[m] = spectrum_of(m);
        std::vector<double> dos(nmeasures_);
        for (std::size_t m = 0; m < nmeasures_; ++m) dos[m] = dos0_f(specs[m], 0.0);
        const bin_data_t dos0 = binning::accumulate_binning(dos.rbegin(), dos.rend(), max_bin_);
        save_binning(dos0, "dos0");
        const std::size_t dos_bin = binning::estimate_bin(dos0);
        std::vector<std::vector<double>> dos_ev(grid_real.size(), std::vector<double>(3));
        for (std::size_t i = 0; i < grid_real.size(); ++i) {
            for (std::size_t m = 0; m < nmeasures_; ++m) dos[m] = dos0_f(specs[m], grid_real[i]);
            const bin_stats_t b = binning::bin(dos.rbegin(), dos.rend(), dos_bin);
            dos_ev[i] = {grid_real[i], std::get<binning::_MEAN>(b), std::get<binning::_SQERROR>(b)};
        }
        save_table("dos_err", dos_ev);
        // n_c = integral of dos(w) f(w) over the grid, error from the squared
        // errors; trapezoid rule on the grid points
        double nc = 0.0, nc_err2 = 0.0;
        auto fermi = [beta](double w) { return 1.0 / (1.0 + std::exp(beta * w)); };
        for (std::size_t i = 0; i + 1 < grid_real.size(); ++i) {
            const double h = grid_real[i + 1] - grid_real[i];
            const double f0 = fermi(grid_real[i]), f1 = fermi(grid_real[i + 1]);
            nc += 0.5 * h * (dos_ev[i][1] * f0 + dos_ev[i + 1][1] * f1);
            nc_err2 += 0.5 * h * (std::pow(dos_ev[i][2] * f0, 2) + std::pow(dos_ev[i + 1][2] * f1, 2));
        }
        save_bin_data(std::make_tuple(std::size_t(0), nc, 0.0, std::sqrt(nc_err2)), "nc", (int)dos_bin);
    }

    void save_ipr(const std::vector<double>& grid_real) {
        const double offset = opt_.dos_offset;
        const std::size_t vol = volume_;
        // Lorentzian-weighted average of the per-state IPR; the stored value is
        // the ratio of norms measure_ipr records, raised to the 4th power as
        // the reference does (data_save.hxx:491-503)
        auto ipr_f = [offset, vol](const std::vector<double>& spec, const std::vector<double>& ipr, double z) {
            double nom = 0.0, denom = 0.0;
            for (std::size_t i = 0; i < vol; ++i) {
                const double p = ipr[i] * ipr[i], state = p * p;
                const double wme = z - spec[i];
                const double lorentz = offset / (wme * wme + offset * offset);
                denom += lorentz;
                nom += lorentz * state;
            }
            return nom / denom;
        };
        std::vector<std::vector<double>> specs(nmeasures_), iprs(nmeasures_, std::vector<double>(vol));
        for (std::size_t m = 0; m < nmeasures_; ++m) {
            specs[m] = spectrum_of(m);
            for (std::size_t i = 0; i < vol; ++i) iprs[m][i] = obs_.ipr_history.at(i).at(m);
        }
        std::vector<double> data(nmeasures_);
        for (std::size_t m = 0; m < nmeasures_; ++m) data[m] = ipr_f(specs[m], iprs[m], 0.0);
        const bin_data_t ipr0 = binning::accumulate_binning(data.rbegin(), data.rend(), max_bin_);
        save_binning(ipr0, "ipr0");
        const std::size_t b0 = binning::estimate_bin(ipr0);
        std::vector<std::vector<double>> ev(grid_real.size(), std::vector<double>(3));
        for (std::size_t i = 0; i < grid_real.size(); ++i) {
            for (std::size_t m = 0; m < nmeasures_; ++m) data[m] = ipr_f(specs[m], iprs[m], grid_real[i]);
            const bin_stats_t b = binning::bin(data.rbegin(), data.rend(), b0);
            ev[i] = {grid_real[i], std::get<binning::_MEAN>(b), std::get<binning::_SQERROR>(b)};
        }
        save_table("ipr_err", ev);
    }

    void save_conductivity(const std::vector<double>& wgrid) {
        const auto& st = obs_.stiffness;
        save_binning(binning::accumulate_binning(st.rbegin(), st.rend(), max_bin_), "stiffness");
        if (wgrid.size() < 3 || obs_.cond_history.size() != wgrid.size()) return;
        const auto& ch = obs_.cond_history;
        const bin_data_t cs0 = binning::accumulate_binning(ch[wgrid.size() / 2].begin(), ch[wgrid.size() / 2].end(), max_bin_);
        const std::size_t cbin = binning::estimate_bin(cs0);
        std::vector<std::vector<double>> wcond(wgrid.size(), std::vector<double>(3));
        for (std::size_t i = 0; i < wgrid.size(); ++i) {
            const bin_stats_t b = binning::bin(ch[i].begin(), ch[i].end(), cbin);
            wcond[i] = {wgrid[i], std::get<binning::_MEAN>(b), std::get<binning::_SQERROR>(b)};
        }
        save_table("wcond_err", wcond);
        const std::size_t iz = (wgrid.size() - 1) / 2;
        const double cond_left = -wcond[iz - 1][1] / wgrid[iz - 1];
        const double cond_right = -wcond[iz + 1][1] / wgrid[iz + 1];
        const double cond0 = (cond_left + cond_right) / 2;
        const double cond0_err = wcond[iz + 1][2] / wgrid[iz + 1];
        const double size0 = double(std::get<binning::_SIZE>(cs0[cbin]));
        stats_out["cond0"] = {(int)cbin, std::make_tuple(std::get<binning::_SIZE>(cs0[cbin]), cond0, size0 * cond0_err * cond0_err, cond0_err)};
        write_npy("stats", "cond0", std::vector<double>{size0, cond0, size0 * cond0_err * cond0_err, cond0_err});
        std::vector<std::vector<double>> cond_ev(wcond), cond_dyn(wcond);
        for (std::size_t i = 0; i < wgrid.size(); ++i) {
            cond_ev[i][1] = -wcond[i][1] / wgrid[i];
            cond_ev[i][2] = -wcond[i][2] / wgrid[i];
            cond_dyn[i][1] = cond_ev[i][1] - cond0;
            cond_dyn[i][2] = cond_ev[i][2];
        }
        save_table("cond_err", cond_ev);
        save_table("cond_dynamic", cond_dyn);
    }

    void write_stats_json() {
        std::ofstream out(dir_ + "/stats.json");
        out << "{";
        bool first = true;
        for (const auto& kv : stats_out) {
            const bin_stats_t& s = kv.second.second;
            out << (first ? "" : ",") << "\n  \"" << kv.first << "\": {\"bin\": " << kv.second.first
                << ", \"size\": " << std::get<binning::_SIZE>(s) << ", \"mean\": " << detail::json_number(std::get<binning::_MEAN>(s))
                << ", \"disp\": " << detail::json_number(std::get<binning::_DISP>(s))
                << ", \"error\": " << detail::json_number(std::get<binning::_SQERROR>(s)) << "}";
            first = false;
        }
        out << "\n}\n";
    }
};

}  // namespace fk
