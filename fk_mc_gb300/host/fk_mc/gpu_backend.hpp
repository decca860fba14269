// gpu_backend.hpp — one libfkg context per host thread, shared by every
// configuration_t of that thread, and the mapping lattice -> registered CSR.
// Errors of the C ABI come back as std::logic_error, the exception type the
// reference throws through FKMC_ERROR (include/fk_mc/common.hpp:49-59).
#pragma once
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
    // lattice id of `l`, registering its hopping matrix on first use
    int lattice_id(const abstract_lattice& l) {
        auto it = ids_.find(&l);
        if (it != ids_.end()) return it->second;
        if ((int)ids_.size() >= 64) throw std::logic_error("fkg: more than 64 lattices in one thread");
        const csr_matrix& h = l.hopping_m();
        int id = (int)ids_.size();
        check(fkg_set_hopping(ctx_, id, h.rows, h.rowptr.data(), h.col.data(), h.val.data()), "fkg_set_hopping");
        ids_[&l] = id;
        return id;
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
    std::map<const abstract_lattice*, int> ids_;
};

}  // namespace fk
