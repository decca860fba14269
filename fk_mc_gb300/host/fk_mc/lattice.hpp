// lattice.hpp — the reference's lattice interface without Eigen/FFTW:
// abstract_lattice holds the hopping matrix as CSR (include/fk_mc/lattice.hpp:12-46),
// hypercubic_lattice<D> numbers sites with the last coordinate fastest
// (src/lattice/hypercubic.cpp:30-51), fill_nearest_neighbors puts -t on every
// periodic bond (src/lattice/hypercubic.cpp:115-131) and fill_triangular adds
// -tp on the (-1,-1)/(+1,+1) diagonal (src/lattice/hypercubic.cpp:137-155).
// graph_lattice and read_lattice_npy load a lattice given by its site
// coordinates and a list of hopping elements (src/lattice/graph.cpp:7-80),
// from .npy files instead of an HDF5 group.
#pragma once
#include <array>
#include <atomic>
#include <cmath>
#include <cstddef>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "npy.hpp"

namespace fk {

struct csr_matrix {
    int rows = 0;
    std::vector<int> rowptr, col;
    std::vector<double> val;
};

struct abstract_lattice {
    explicit abstract_lattice(std::size_t msize = 0, std::size_t norbitals = 1)
        : entries_(msize), msize_(msize), norbs_(norbitals), serial_(next_serial()) {}
    abstract_lattice(const abstract_lattice& rhs)
        : entries_(rhs.entries_), msize_(rhs.msize_), norbs_(rhs.norbs_), serial_(next_serial()) {}
    virtual ~abstract_lattice() = default;
    // identity of this lattice's hopping matrix: unique per object, bumped by every add_hopping
    std::pair<unsigned long, unsigned long> identity() const { return {serial_, version_}; }
    std::size_t msize() const { return msize_; }
    std::size_t norbs() const { return norbs_; }
    std::size_t volume() const { return msize_ / norbs_; }
    virtual std::size_t ndim() const = 0;
    // add_hopping (src/lattice.cpp:9-16); a repeated entry is summed
    abstract_lattice& add_hopping(std::size_t l, std::size_t r, double v, bool symmetrize = false) {
        entries_.at(l)[(int)r] += v;
        if (symmetrize) entries_.at(r)[(int)l] += v;
        csr_valid_ = false;
        ++version_;
        return *this;
    }
    // one element set (not summed), as hopping_m.coeffRef(l, r) = v does
    abstract_lattice& set_hopping(std::size_t l, std::size_t r, double v) {
        entries_.at(l)[(int)r] = v;
        csr_valid_ = false;
        ++version_;
        return *this;
    }
    const csr_matrix& hopping_m() const {
        if (!csr_valid_) {
            csr_ = csr_matrix();
            csr_.rows = (int)msize_;
            csr_.rowptr.assign(msize_ + 1, 0);
            for (std::size_t i = 0; i < msize_; ++i) {
                csr_.rowptr[i + 1] = csr_.rowptr[i] + (int)entries_[i].size();
                for (auto& kv : entries_[i]) { csr_.col.push_back(kv.first); csr_.val.push_back(kv.second); }
            }
            csr_valid_ = true;
        }
        return csr_;
    }

protected:
    std::vector<std::map<int, double>> entries_;
    std::size_t msize_, norbs_;
    mutable csr_matrix csr_;
    mutable bool csr_valid_ = false;
    unsigned long serial_, version_ = 0;
    static unsigned long next_serial() {
        static std::atomic<unsigned long> counter{1};
        return counter++;
    }
};

template <std::size_t D>
struct hypercubic_lattice : abstract_lattice {
    static constexpr std::size_t Ndim = D;
    explicit hypercubic_lattice(std::size_t L) : abstract_lattice(ipow(L)) { dims_.fill((int)L); }
    std::size_t ndim() const override { return D; }
    const std::array<int, D>& dims() const { return dims_; }
    std::array<int, D> index_to_pos(std::size_t index) const {
        std::array<int, D> out;
        for (int i = (int)D - 1; i >= 0; --i) { out[i] = (int)(index % dims_[i]); index /= dims_[i]; }
        return out;
    }
    std::size_t pos_to_index(std::array<int, D> pos) const {
        std::size_t out = 0, mult = 1;
        for (int i = (int)D - 1; i >= 0; --i) { out += pos[i] * mult; mult *= dims_[i]; }
        return out;
    }
    // sum_i f_i exp(i pi sum_d x_d) (FFT_pi, src/lattice/hypercubic.cpp:78-83
    // with phase_array(pi), :17-28): the phase is (-1)^(sum of coordinates),
    // so the rounded sum is formed in integers
    template <typename array_t>
    int FFT_pi(const array_t& f) const {
        long s = 0;
        for (std::size_t i = 0; i < volume(); ++i) {
            const auto pos = index_to_pos(i);
            int parity = 0;
            for (int p : pos) parity += p;
            s += (parity % 2 ? -1 : 1) * (long)f[i];
        }
        return (int)s;
    }

private:
    static std::size_t ipow(std::size_t L) { std::size_t v = 1; for (std::size_t i = 0; i < D; ++i) v *= L; return v; }
    std::array<int, D> dims_;
};

template <std::size_t D>
hypercubic_lattice<D>& fill_nearest_neighbors(hypercubic_lattice<D>& l, double t) {
    for (std::size_t i = 0; i < l.volume(); ++i) {
        auto cur = l.index_to_pos(i);
        for (std::size_t n = 0; n < D; ++n) {
            auto pl = cur, pr = cur;
            pl[n] = cur[n] > 0 ? cur[n] - 1 : l.dims()[n] - 1;
            pr[n] = cur[n] < l.dims()[n] - 1 ? cur[n] + 1 : 0;
            l.add_hopping(i, l.pos_to_index(pl), -1.0 * t);
            l.add_hopping(i, l.pos_to_index(pr), -1.0 * t);
        }
    }
    return l;
}

inline hypercubic_lattice<2>& fill_triangular(hypercubic_lattice<2>& l, double t, double tp) {
    fill_nearest_neighbors(l, t);
    for (std::size_t i = 0; i < l.volume(); ++i) {
        auto cur = l.index_to_pos(i);
        auto pl = cur, pr = cur;
        for (std::size_t n = 0; n < 2; ++n) {
            pl[n] = cur[n] > 0 ? cur[n] - 1 : l.dims()[n] - 1;
            pr[n] = cur[n] < l.dims()[n] - 1 ? cur[n] + 1 : 0;
        }
        l.add_hopping(i, l.pos_to_index(pl), -1.0 * tp);
        l.add_hopping(i, l.pos_to_index(pr), -1.0 * tp);
    }
    return l;
}

// A lattice given by the coordinates of its sites and an explicit hopping
// matrix (include/fk_mc/lattice/graph.hpp, src/lattice/graph.cpp:7-21).
struct graph_lattice : abstract_lattice {
    typedef std::vector<int> pos_t;
    graph_lattice(std::size_t msize, std::vector<pos_t> sites, std::vector<int> dims, std::size_t norbs)
        : abstract_lattice(msize, norbs), sites_(std::move(sites)), dims_(std::move(dims)) {
        for (const auto& p : sites_)
            if (p.size() != dims_.size()) throw std::logic_error("site coordinate of the wrong dimension");
        if (sites_.size() * norbs != msize) throw std::logic_error("sites x orbitals != matrix size");
    }
    std::size_t ndim() const override { return dims_.size(); }
    const std::vector<int>& dims() const { return dims_; }
    const std::vector<pos_t>& sites() const { return sites_; }
    // sum_i f_i (-1)^(sum of the coordinates of site i), as for hypercubic_lattice
    template <typename array_t>
    int FFT_pi(const array_t& f) const {
        long s = 0;
        for (std::size_t i = 0; i < volume(); ++i) {
            int parity = 0;
            for (int p : sites_[i]) parity += p;
            s += ((parity % 2 + 2) % 2 ? -1 : 1) * (long)f[i];
        }
        return (int)s;
    }

private:
    std::vector<pos_t> sites_;
    std::vector<int> dims_;
};

// read_lattice_hdf5 (src/lattice/graph.cpp:52-80) with each dataset of the
// group as <dir>/<name>.npy: dims (the lattice extents, whose product is the
// number of sites), norbitals (a scalar), coordinates (sites x ndim) and
// hopping (rows (p1, p2, m), real or complex; element (p1, p2) is set to m,
// a later row for the same element replacing an earlier one). Matrix
// elements must be real: the eigensolver is the real symmetric one.
inline graph_lattice read_lattice_npy(const std::string& dir) {
    const npy::array dims = npy::read(dir + "/dims.npy");
    const npy::array norb = npy::read(dir + "/norbitals.npy");
    const npy::array coords = npy::read(dir + "/coordinates.npy");
    const npy::array hop = npy::read(dir + "/hopping.npy");
    if (norb.size() != 1) throw std::runtime_error("norbitals must be a scalar");
    const int norbs = (int)norb.data[0];
    std::size_t npts = 1;
    std::vector<int> d;
    for (double x : dims.data) { d.push_back((int)x); npts *= (std::size_t)x; }
    if (norbs < 1 || d.empty()) throw std::runtime_error("bad dims or norbitals");
    if (coords.shape.size() != 2 || coords.shape[0] != npts || coords.shape[1] != d.size())
        throw std::runtime_error("coordinates must be (number of sites) x (number of dimensions)");
    std::vector<graph_lattice::pos_t> sites(npts);
    for (std::size_t i = 0; i < npts; ++i)
        for (std::size_t k = 0; k < d.size(); ++k) sites[i].push_back((int)coords.data[i * d.size() + k]);
    const std::size_t msize = npts * (std::size_t)norbs;
    graph_lattice l(msize, sites, d, (std::size_t)norbs);
    if (hop.shape.size() != 2 || hop.shape[1] != 3) throw std::runtime_error("hopping must be rows of (p1, p2, m)");
    for (std::size_t r = 0; r < hop.shape[0]; ++r) {
        const long p1 = std::lround(hop.data[3 * r]), p2 = std::lround(hop.data[3 * r + 1]);
        if (p1 < 0 || p2 < 0 || (std::size_t)p1 >= msize || (std::size_t)p2 >= msize)
            throw std::runtime_error("hopping index out of range");
        if (!hop.imag.empty() && hop.imag[3 * r + 2] != 0.0)
            throw std::runtime_error("complex hopping elements are not supported by the real symmetric solver");
        l.set_hopping((std::size_t)p1, (std::size_t)p2, hop.data[3 * r + 2]);
    }
    return l;
}

}  // namespace fk
