// fkh_capi.cpp — C entry points of the host adapter (include/fk_mc_host.h):
// a chain set up and run as fk_mc<L>::initialize + mc.run do
// (include/fk_mc/fk_mc.hxx:35-125, prog/fk_mc_exec.cpp:124-151).
#include <cmath>
#include <cstring>
#include <exception>
#include <limits>
#include <memory>

#include "../../include/fk_mc_host.h"
#include "fk_mc/batched_mc.hpp"
#include "fk_mc/configuration.hpp"
#include "fk_mc/lattice.hpp"
#include "fk_mc/mc_metropolis.hpp"
#include "fk_mc/measures.hpp"
#include "fk_mc/moves.hpp"
#include "fk_mc/moves_chebyshev.hpp"

namespace {

std::unique_ptr<fk::abstract_lattice> make_lattice(int kind, int L, double t, double tp) {
    switch (kind) {
        case 1: { auto l = std::make_unique<fk::hypercubic_lattice<1>>(L); fk::fill_nearest_neighbors(*l, t); return l; }
        case 2: { auto l = std::make_unique<fk::hypercubic_lattice<2>>(L); fk::fill_nearest_neighbors(*l, t); return l; }
        case 3: { auto l = std::make_unique<fk::hypercubic_lattice<3>>(L); fk::fill_nearest_neighbors(*l, t); return l; }
        case 4: { auto l = std::make_unique<fk::hypercubic_lattice<2>>(L); fk::fill_triangular(*l, t, tp); return l; }
        default: throw std::logic_error("unknown lattice kind");
    }
}

int report(const std::exception& e, char* errbuf, int errlen) {
    if (errbuf && errlen > 0) {
        std::strncpy(errbuf, e.what(), (size_t)errlen - 1);
        errbuf[errlen - 1] = '\0';
    }
    return -1;
}

}  // namespace

namespace {

// One chain through the reference's classes on `lattice` (fk_mc<L>::initialize
// and mc.run, include/fk_mc/fk_mc.hxx:35-125).
template <typename lattice_t>
void run_chain(const lattice_t& lattice, const fkh_params* p, fkh_out* out) {
    fk::gpu_backend& g = fk::gpu_backend::instance();
    g.check(fkg_set_precision(g.ctx(), p->precision), "fkg_set_precision");
    fk::mc_metropolis mc(p->seed, p->nsweeps, p->sweep_len, p->ntherm_sweeps);
    fk::configuration_t config(lattice, p->beta, p->U, p->mu_c, p->mu_f);
    config.randomize_f(mc.rng(), p->nf_start);
    const std::size_t V = lattice.volume();
    if (out && out->f_initial) std::copy(config.f_config_.begin(), config.f_config_.end(), out->f_initial);
    config.calc_hamiltonian();
    const double eps = std::numeric_limits<double>::epsilon();
    int kinds[3], nm = 0;
    // include/fk_mc/fk_mc.hxx:59-78: the Chebyshev evaluator and moves
    std::unique_ptr<fk::chebyshev::chebyshev_eval> cheb;
    if (p->cheb_moves) {
        int cs = int(std::log((double)lattice.msize()) * p->cheb_prefactor);
        cs += cs % 2;
        cheb.reset(new fk::chebyshev::chebyshev_eval(cs, std::max(cs * 2, 10)));
    }
    if (p->mc_flip > eps) {
        if (cheb) mc.add_move(std::make_shared<fk::chebyshev::move_flip>(p->beta, config, *cheb, mc.rng()), "flip", p->mc_flip);
        else mc.add_move(std::make_shared<fk::move_flip>(p->beta, config, mc.rng()), "flip", p->mc_flip);
        kinds[nm++] = 0;
    }
    if (p->mc_add_remove > eps) {
        if (cheb) mc.add_move(std::make_shared<fk::chebyshev::move_addremove>(p->beta, config, *cheb, mc.rng()), "add_remove", p->mc_add_remove);
        else if (p->rank1_moves) mc.add_move(std::make_shared<fk::move_addremove_rank1>(p->beta, config, mc.rng()), "add_remove", p->mc_add_remove);
        else mc.add_move(std::make_shared<fk::move_addremove>(p->beta, config, mc.rng()), "add_remove", p->mc_add_remove);
        kinds[nm++] = 1;
    }
    if (p->mc_reshuffle > eps) {
        if (cheb) mc.add_move(std::make_shared<fk::chebyshev::move_randomize>(p->beta, config, *cheb, mc.rng()), "reshuffle", p->mc_reshuffle);
        else mc.add_move(std::make_shared<fk::move_randomize>(p->beta, config, mc.rng()), "reshuffle", p->mc_reshuffle);
        kinds[nm++] = 2;
    }
    std::vector<double> energies, d2energies, c_energies, nf0, nfpi;
    std::vector<std::vector<double>> spectrum_history, focc_history;
    if (!cheb) {  // with the Chebyshev moves the reference registers no energy measure
        auto me = std::make_shared<fk::measure_energy>(p->beta, config, energies, d2energies, c_energies);
        mc.add_measure([me](double ph) { me->accumulate(ph); }, "energy");
    }
    auto mn = std::make_shared<fk::measure_nf0pi<lattice_t>>(config, lattice, nf0, nfpi);
    mc.add_measure([mn](double ph) { mn->accumulate(ph); }, "nf0pi");
    if (out && out->spectrum_history) {
        auto ms = std::make_shared<fk::measure_spectrum_history>(config, spectrum_history);
        mc.add_measure([ms](double ph) { ms->accumulate(ph); }, "spectrum_history");
    }
    if (out && out->focc_history) {
        auto mf = std::make_shared<fk::measure_focc>(config, focc_history);
        mc.add_measure([mf](double ph) { mf->accumulate(ph); }, "focc_history");
    }
    long k = 0, naccept = 0;
    mc.on_proposal = [&](int idx, double w, double u, bool acc) {
        if (out) {
            if (out->move_index) out->move_index[k] = kinds[idx];
            if (out->accepted) out->accepted[k] = acc;
            if (out->weight) out->weight[k] = w;
            if (out->uniform) out->uniform[k] = u;
        }
        naccept += acc;
        ++k;
    };
    mc.run();
    if (out) {
        const std::size_t M = nf0.size();
        for (std::size_t m = 0; m < M; ++m) {
            if (m < energies.size()) {
                if (out->energy) out->energy[m] = energies[m];
                if (out->d2energy) out->d2energy[m] = d2energies[m];
                if (out->c_energy) out->c_energy[m] = c_energies[m];
            }
            if (out->nf0) out->nf0[m] = nf0[m];
            if (out->nfpi) out->nfpi[m] = nfpi[m];
        }
        // histories: state-major [i * nsweeps + m], as the reference stores them
        if (out->spectrum_history)
            for (std::size_t i = 0; i < spectrum_history.size(); ++i)
                for (std::size_t m = 0; m < M; ++m) out->spectrum_history[i * M + m] = spectrum_history[i][m];
        if (out->focc_history)
            for (std::size_t i = 0; i < focc_history.size(); ++i)
                for (std::size_t m = 0; m < M; ++m) out->focc_history[i * M + m] = (int32_t)focc_history[i][m];
        if (out->f_final) std::copy(config.f_config_.begin(), config.f_config_.begin() + V, out->f_final);
        out->naccept = naccept;
    }
}

}  // namespace

extern "C" int fkh_run_chain(const fkh_params* p, fkh_out* out, char* errbuf, int errlen) {
    try {
        if (!p) throw std::logic_error("null parameters");
        switch (p->lattice_kind) {
            case 1: { fk::hypercubic_lattice<1> l(p->L); fk::fill_nearest_neighbors(l, p->t); run_chain(l, p, out); break; }
            case 2: { fk::hypercubic_lattice<2> l(p->L); fk::fill_nearest_neighbors(l, p->t); run_chain(l, p, out); break; }
            case 3: { fk::hypercubic_lattice<3> l(p->L); fk::fill_nearest_neighbors(l, p->t); run_chain(l, p, out); break; }
            case 4: { fk::hypercubic_lattice<2> l(p->L); fk::fill_triangular(l, p->t, p->tp); run_chain(l, p, out); break; }
            default: throw std::logic_error("unknown lattice kind");
        }
        return 0;
    } catch (const std::exception& e) {
        return report(e, errbuf, errlen);
    }
}

extern "C" int fkh_run_chain_graph(const char* lattice_dir, const fkh_params* p, fkh_out* out, char* errbuf,
                                   int errlen) {
    try {
        if (!p || !lattice_dir) throw std::logic_error("null argument");
        const fk::graph_lattice l = fk::read_lattice_npy(lattice_dir);
        run_chain(l, p, out);
        return 0;
    } catch (const std::exception& e) {
        return report(e, errbuf, errlen);
    }
}

extern "C" int fkh_run_batched(const fkh_params* p, int batch, fkh_out* out, char* errbuf, int errlen) {
    try {
        if (!p || batch < 1) throw std::logic_error("bad parameters");
        auto lattice = make_lattice(p->lattice_kind, p->L, p->t, p->tp);
        std::vector<long> seeds(batch);
        for (int c = 0; c < batch; ++c) seeds[c] = (long)(p->seed + c);
        int cs = 0;
        if (p->cheb_moves) {  // include/fk_mc/fk_mc.hxx:59-64
            cs = int(std::log((double)lattice->msize()) * p->cheb_prefactor);
            cs += cs % 2;
        }
        fk::batched_mc bmc(*lattice, p->beta, p->U, p->mu_c, p->mu_f, seeds, p->nf_start, p->precision, cs,
                           std::max(cs * 2, 10));
        const int V = (int)lattice->volume();
        const long nprop = (long)(p->nsweeps + p->ntherm_sweeps) * p->sweep_len;
        std::vector<int> acc;  // step-major [k][c]
        std::vector<double> e, d2e, ec;  // measurement-major [m][c]
        for (int s = 0; s < p->nsweeps + p->ntherm_sweeps; ++s) {
            bmc.update(p->sweep_len, &acc);
            if (s >= p->ntherm_sweeps && !p->cheb_moves) bmc.measure_energy(e, d2e, ec);
        }
        std::vector<int> f;
        std::vector<double> logz;
        bmc.get_state(f, logz);
        if (out) {
            long naccept = 0;
            for (long k = 0; k < nprop; ++k)
                for (int c = 0; c < batch; ++c) {
                    naccept += acc[(size_t)k * batch + c];
                    if (out->accepted) out->accepted[(size_t)c * nprop + k] = acc[(size_t)k * batch + c];
                }
            for (int m = 0; m < (p->cheb_moves ? 0 : p->nsweeps); ++m)
                for (int c = 0; c < batch; ++c) {
                    if (out->energy) out->energy[(size_t)c * p->nsweeps + m] = e[(size_t)m * batch + c];
                    if (out->d2energy) out->d2energy[(size_t)c * p->nsweeps + m] = d2e[(size_t)m * batch + c];
                    if (out->c_energy) out->c_energy[(size_t)c * p->nsweeps + m] = ec[(size_t)m * batch + c];
                }
            if (out->f_initial) std::copy(bmc.f_initial_.begin(), bmc.f_initial_.end(), out->f_initial);
            if (out->f_final) std::copy(f.begin(), f.end(), out->f_final);
            out->naccept = naccept;
        }
        (void)V;
        return 0;
    } catch (const std::exception& e) {
        return report(e, errbuf, errlen);
    }
}

namespace {

template <typename lattice_t>
void measure_eigen(const lattice_t& lattice, const fkh_params* p, const int32_t* f, int nw, const double* wgrid,
                   double eta, double* stiffness, double* cond, double* ipr) {
    fk::gpu_backend& g = fk::gpu_backend::instance();
    g.check(fkg_set_precision(g.ctx(), p->precision), "fkg_set_precision");
    fk::configuration_t config(lattice, p->beta, p->U, p->mu_c, p->mu_f);
    for (std::size_t i = 0; i < lattice.volume(); ++i) config.f_config_[i] = f[i];
    config.calc_hamiltonian();
    std::vector<double> stiffness_vals;
    std::vector<std::vector<double>> cond_history;
    fk::measure_stiffness<lattice_t> ms(config, lattice, stiffness_vals, cond_history,
                                        std::vector<double>(wgrid, wgrid + nw), eta);
    ms.accumulate(1.0);
    *stiffness = stiffness_vals.at(0);
    for (int w = 0; w < nw; ++w) cond[w] = cond_history[w].at(0);
    if (ipr) {
        std::vector<std::vector<double>> ipr_vals;
        fk::measure_ipr<lattice_t> mi(config, lattice, ipr_vals);
        mi.accumulate(1.0);
        for (std::size_t k = 0; k < ipr_vals.size(); ++k) ipr[k] = ipr_vals[k].at(0);
    }
}

}  // namespace

extern "C" int fkh_measure_eigen(const fkh_params* p, const int32_t* f, int nw, const double* wgrid, double eta,
                                 double* stiffness, double* cond, double* ipr, char* errbuf, int errlen) {
    try {
        if (!p || !f || !stiffness || nw < 0 || (nw > 0 && (!wgrid || !cond))) throw std::logic_error("bad arguments");
        switch (p->lattice_kind) {
            case 1: { fk::hypercubic_lattice<1> l(p->L); fk::fill_nearest_neighbors(l, p->t);
                      measure_eigen(l, p, f, nw, wgrid, eta, stiffness, cond, ipr); break; }
            case 2: { fk::hypercubic_lattice<2> l(p->L); fk::fill_nearest_neighbors(l, p->t);
                      measure_eigen(l, p, f, nw, wgrid, eta, stiffness, cond, ipr); break; }
            case 3: { fk::hypercubic_lattice<3> l(p->L); fk::fill_nearest_neighbors(l, p->t);
                      measure_eigen(l, p, f, nw, wgrid, eta, stiffness, cond, ipr); break; }
            case 4: { fk::hypercubic_lattice<2> l(p->L); fk::fill_triangular(l, p->t, p->tp);
                      measure_eigen(l, p, f, nw, wgrid, eta, stiffness, cond, ipr); break; }
            default: throw std::logic_error("unknown lattice kind");
        }
        return 0;
    } catch (const std::exception& e) {
        return report(e, errbuf, errlen);
    }
}
