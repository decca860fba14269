// lattice.hpp — the reference's lattice interface without Eigen/FFTW:
// abstract_lattice holds the hopping matrix as CSR (include/fk_mc/lattice.hpp:12-46),
// hypercubic_lattice<D> numbers sites with the last coordinate fastest
// (src/lattice/hypercubic.cpp:30-51), fill_nearest_neighbors puts -t on every
// periodic bond (src/lattice/hypercubic.cpp:115-131) and fill_triangular adds
// -tp on the (-1,-1)/(+1,+1) diagonal (src/lattice/hypercubic.cpp:137-155).
#pragma once
#include <array>
#include <atomic>
#include <cstddef>
#include <map>
#include <stdexcept>
#include <vector>

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

}  // namespace fk
