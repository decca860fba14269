// gpu_backend.hpp — one libfkg context per host thread, shared by every
// configuration_t of that thread, and the mapping lattice -> registered CSR.
// Errors of the C ABI come back as std::logic_error, the exception type the
// reference throws through FKMC_ERROR (include/fk_mc/common.hpp:49-59).
#pragma once
#include <iterator>
#include <map>
#include <stdexcept>
#include <string>

#include "../../../include/fkg.h"
#include "lattice.hpp"

namespace fk {

class gpu_backend {
public:
    static gpu_backend& instance() {
        thread_local gpu_backend b;
        return b;
    }
    fkg_ctx* ctx() { return ctx_; }
    // lattice id of `l`, registering its hopping matrix on first use (keyed by
    // the lattice's identity, not its address: a new lattice may reuse the
    // address of a destroyed one). When all 64 slots are taken they are
    // recycled from the start.
    int lattice_id(const abstract_lattice& l) {
        auto it = ids_.find(l.identity());
        if (it != ids_.end()) return it->second;
        if (next_slot_ >= 64) { ids_.clear(); next_slot_ = 0; }
        const csr_matrix& h = l.hopping_m();
        const int id = next_slot_++;
        for (auto jt = ids_.begin(); jt != ids_.end();)  // slot reuse drops the old owner
            jt = jt->second == id ? ids_.erase(jt) : std::next(jt);
        check(fkg_set_hopping(ctx_, id, h.rows, h.rowptr.data(), h.col.data(), h.val.data()), "fkg_set_hopping");
        ids_[l.identity()] = id;
        ++registrations_;
        return id;
    }
    // counts hopping registrations: a registration drops the slot's measure
    // operators, which their owners then register again
    unsigned long registrations() const { return registrations_; }
    // moments and grid of the context's Chebyshev expansion, set on change
    void set_chebyshev(int cheb_size, int grid_size) {
        if (cheb_size == cheb_size_ && grid_size == grid_size_) return;
        check(fkg_set_chebyshev(ctx_, cheb_size, grid_size), "fkg_set_chebyshev");
        cheb_size_ = cheb_size;
        grid_size_ = grid_size;
    }
    void check(int rc, const char* what) {
        if (rc != FKG_OK) throw std::logic_error(std::string(what) + ": " + fkg_last_error(ctx_));
    }
    ~gpu_backend() { if (ctx_) fkg_destroy(ctx_); }

private:
    gpu_backend() : ctx_(fkg_create(1024, 1, 0)) {
        if (!ctx_) throw std::logic_error("fkg_create failed: no CUDA device");
    }
    fkg_ctx* ctx_;
    std::map<std::pair<unsigned long, unsigned long>, int> ids_;
    int next_slot_ = 0;
    unsigned long registrations_ = 0;
    int cheb_size_ = 0, grid_size_ = 0;
};

}  // namespace fk
