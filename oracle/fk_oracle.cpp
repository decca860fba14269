// fk_oracle.cpp — CPU oracle for the fk_mc exact-diagonalisation Metropolis path.
//
// TEST INFRASTRUCTURE ONLY. This file restates, in plain C++ (no Eigen, no
// ALPSCore, no Boost), the reference algorithm of aeantipov/fk_mc for the path
// that the GPU library replaces. Only tests/, __graft_entry__.smoke() and the
// CPU-baseline legs of bench.py load it, and only as the checker / the timed
// CPU baseline. The product (fk_mc_gb300/) never links or calls it.
//
// What is restated, with the reference lines it follows:
//   * lattices: hypercubic index maps and periodic nearest-neighbour hopping
//     (-t per bond), triangular diagonal bonds (-tp)
//       src/lattice/hypercubic.cpp:30-51, 115-131, 137-155
//   * configuration_t: randomize_f, calc_ff_energy, calc_hamiltonian, calc_ed
//       src/configuration.cpp:47-56, 59-77, 79-91, 208-246
//     The dense eigensolve at src/configuration.cpp:213 is Eigen 3's
//     SelfAdjointEigenSolver (third party, version unpinned:
//     cmake/CommonDefs.cmake:98). Its published algorithm — Householder
//     tridiagonalisation followed by implicit symmetric QR with a Wilkinson
//     shift and an ascending sort — is restated here from Golub & Van Loan,
//     "Matrix Computations", 4th ed., Alg. 8.3.1 / 8.3.3.
//   * moves: move_flip, move_randomize, move_addremove
//       src/moves.cpp:5-67, include/fk_mc/moves.hpp:11-47
//   * mc_metropolis: update/measure and the order of random draws
//       src/mc_metropolis.cpp:21-61, include/fk_mc/mc_metropolis.hpp:140-143,176-183
//     driven as fk_mc::initialize does (include/fk_mc/fk_mc.hxx:35-125)
//   * measure_energy::accumulate        src/measures/energy.cpp:6-26
//   * measure_stiffness::accumulate     include/fk_mc/measures/stiffness.hpp:129-187
//   * measure_ipr::accumulate           include/fk_mc/measures/ipr.hpp:39-56
//   * calc_chebyshev, chebyshev_eval and the Chebyshev moves
//       src/configuration.cpp:94-205, include/fk_mc/chebyshev.hpp:16-66,
//       src/moves_chebyshev.cpp:6-72 (spectral bounds from the dense
//       eigensolve where the reference asks ARPACK)
//
// Random numbers: std::mt19937 with the libstdc++ distributions, used exactly
// as the reference uses them (same objects, same order of draws), so a
// libstdc++ build of the reference and this oracle consume identical streams.
//
// Build: see oracle/build_oracle.py (g++ -O3 -shared -fPIC, no -march flags).

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace orc {

typedef std::mt19937 random_generator;  // include/fk_mc/common.hpp:18

// ---------------------------------------------------------------------------
// Lattices (sparse hopping in CSR, rows sorted by column).
// ---------------------------------------------------------------------------
struct csr_t {
    int n = 0;
    std::vector<int> rowptr, col;
    std::vector<double> val;
};

struct triplets_t {
    int n;
    std::vector<std::map<int, double>> rows;
    explicit triplets_t(int n_) : n(n_), rows(n_) {}
    // abstract_lattice::add_hopping (src/lattice.cpp:9-16) inserts one entry;
    // an entry that already exists is summed (Eigen's insert would assert).
    void add(int i, int j, double v) { rows[i][j] += v; }
    csr_t to_csr() const {
        csr_t c;
        c.n = n;
        c.rowptr.assign(n + 1, 0);
        for (int i = 0; i < n; ++i) {
            c.rowptr[i + 1] = c.rowptr[i] + (int)rows[i].size();
            for (auto& kv : rows[i]) { c.col.push_back(kv.first); c.val.push_back(kv.second); }
        }
        return c;
    }
};

// hypercubic_lattice<D>::index_to_pos / pos_to_index: last coordinate fastest
// (src/lattice/hypercubic.cpp:30-51).
static std::vector<int> index_to_pos(int D, int L, int index) {
    std::vector<int> pos(D);
    for (int i = D - 1; i >= 0; --i) { pos[i] = index % L; index /= L; }
    return pos;
}
static int pos_to_index(int D, int L, const std::vector<int>& pos) {
    int out = 0, mult = 1;
    for (int i = D - 1; i >= 0; --i) { out += pos[i] * mult; mult *= L; }
    return out;
}
static int ipow(int L, int D) { int v = 1; for (int i = 0; i < D; ++i) v *= L; return v; }

// fill_nearest_neighbors (src/lattice/hypercubic.cpp:115-131): for every site
// and every axis, left and right periodic neighbours get -t.
static void fill_nearest_neighbors(triplets_t& h, int D, int L, double t) {
    int V = ipow(L, D);
    for (int i = 0; i < V; ++i) {
        auto cur = index_to_pos(D, L, i);
        for (int n = 0; n < D; ++n) {
            auto pl = cur, pr = cur;
            pl[n] = cur[n] > 0 ? cur[n] - 1 : L - 1;
            pr[n] = cur[n] < L - 1 ? cur[n] + 1 : 0;
            h.add(i, pos_to_index(D, L, pl), -1.0 * t);
            h.add(i, pos_to_index(D, L, pr), -1.0 * t);
        }
    }
}

// fill_triangular (src/lattice/hypercubic.cpp:137-155): square lattice plus the
// (-1,-1) and (+1,+1) diagonal with -tp.
static void fill_triangular(triplets_t& h, int L, double t, double tp) {
    fill_nearest_neighbors(h, 2, L, t);
    int V = L * L;
    for (int i = 0; i < V; ++i) {
        auto cur = index_to_pos(2, L, i);
        auto pl = cur, pr = cur;
        for (int n = 0; n < 2; ++n) {
            pl[n] = cur[n] > 0 ? cur[n] - 1 : L - 1;
            pr[n] = cur[n] < L - 1 ? cur[n] + 1 : 0;
        }
        h.add(i, pos_to_index(2, L, pl), -1.0 * tp);
        h.add(i, pos_to_index(2, L, pr), -1.0 * tp);
    }
}

// kind: 1,2,3 = cubic1d/2d/3d; 4 = triangular.
static csr_t make_lattice(int kind, int L, double t, double tp) {
    if (kind >= 1 && kind <= 3) {
        triplets_t h(ipow(L, kind));
        fill_nearest_neighbors(h, kind, L, t);
        return h.to_csr();
    }
    if (kind == 4) {
        triplets_t h(L * L);
        fill_triangular(h, L, t, tp);
        return h.to_csr();
    }
    throw std::invalid_argument("unknown lattice kind");
}
static int lattice_ndim(int kind) { return kind == 4 ? 2 : kind; }

// ---------------------------------------------------------------------------
// Dense symmetric eigensolver (restatement of the published algorithm of
// Eigen::SelfAdjointEigenSolver used at src/configuration.cpp:213).
// ---------------------------------------------------------------------------

// Householder tridiagonalisation of the lower triangle of A (column-major,
// leading dimension n): A = Q T Q^T, Q = H_0 H_1 ... H_{n-3},
// H_k = I - tau_k v_k v_k^T, v_k(k+1) = 1, v_k(k+2:) stored in A(k+2:, k).
// Symmetric rank-2 updates touch the lower triangle only (GVL Alg. 8.3.1).
static void tridiagonalize(int n, double* A, double* d, double* e, double* tau) {
    std::vector<double> v(n), p(n), w(n);
    for (int k = 0; k + 2 < n; ++k) {
        double* col = A + (size_t)k * n;
        const int s = k + 1;
        double alpha = col[s];
        double sigma = 0.0;
        for (int i = s + 1; i < n; ++i) sigma += col[i] * col[i];
        if (sigma == 0.0) {
            tau[k] = 0.0;
            e[k] = alpha;
            continue;
        }
        double xnorm = std::sqrt(alpha * alpha + sigma);
        double beta = alpha >= 0.0 ? -xnorm : xnorm;
        double t = (beta - alpha) / beta;
        double scale = 1.0 / (alpha - beta);
        v[s] = 1.0;
        for (int i = s + 1; i < n; ++i) { v[i] = col[i] * scale; col[i] = v[i]; }
        col[s] = beta;
        tau[k] = t;
        e[k] = beta;
        // p = t * A22 * v using the lower triangle of A22 = A(s:, s:)
        for (int i = s; i < n; ++i) p[i] = 0.0;
        for (int j = s; j < n; ++j) {
            const double* aj = A + (size_t)j * n;
            double vj = v[j];
            double acc = aj[j] * vj;
            for (int i = j + 1; i < n; ++i) {
                p[i] += aj[i] * vj;
                acc += aj[i] * v[i];
            }
            p[j] += acc;
        }
        double pv = 0.0;
        for (int i = s; i < n; ++i) { p[i] *= t; pv += p[i] * v[i]; }
        double K = 0.5 * t * pv;
        for (int i = s; i < n; ++i) w[i] = p[i] - K * v[i];
        // A22 -= v w^T + w v^T (lower)
        for (int j = s; j < n; ++j) {
            double* aj = A + (size_t)j * n;
            double vj = v[j], wj = w[j];
            for (int i = j; i < n; ++i) aj[i] -= v[i] * wj + w[i] * vj;
        }
    }
    for (int k = 0; k < n; ++k) d[k] = A[(size_t)k * n + k];
    if (n >= 2) e[n - 2] = A[(size_t)(n - 2) * n + (n - 1)];
    if (n >= 2) tau[n - 2] = 0.0;
}

// Q = H_0 ... H_{n-3} formed explicitly by backward accumulation.
static void form_q(int n, const double* A, const double* tau, double* Q) {
    std::fill(Q, Q + (size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) Q[(size_t)i * n + i] = 1.0;
    std::vector<double> v(n), r(n);
    for (int k = n - 3; k >= 0; --k) {
        if (tau[k] == 0.0) continue;
        const int s = k + 1;
        v[s] = 1.0;
        for (int i = s + 1; i < n; ++i) v[i] = A[(size_t)k * n + i];
        // Q(s:, s:) = (I - tau v v^T) Q(s:, s:)
        for (int j = s; j < n; ++j) {
            double* qj = Q + (size_t)j * n;
            double dot = 0.0;
            for (int i = s; i < n; ++i) dot += v[i] * qj[i];
            dot *= tau[k];
            for (int i = s; i < n; ++i) qj[i] -= dot * v[i];
        }
    }
}

// Implicit symmetric QR with Wilkinson shift on the unreduced blocks of the
// tridiagonal (d, e); rotations accumulated into the columns of Z (n x n,
// column-major) when Z is non-null. Returns 0 on success.
static int tridiag_qr(int n, double* d, double* e, double* Z) {
    const double eps = std::numeric_limits<double>::epsilon();
    const double tiny = std::numeric_limits<double>::min();
    int end = n - 1;
    long iter = 0, maxiter = 30L * n + 30;
    while (end > 0) {
        for (int i = 0; i < end; ++i)
            if (std::abs(e[i]) <= eps * (std::abs(d[i]) + std::abs(d[i + 1])) || std::abs(e[i]) < tiny)
                e[i] = 0.0;
        while (end > 0 && e[end - 1] == 0.0) --end;
        if (end <= 0) break;
        if (++iter > maxiter) return -1;
        int start = end - 1;
        while (start > 0 && e[start - 1] != 0.0) --start;
        // Wilkinson shift: eigenvalue of the trailing 2x2 closer to d[end]
        double td = 0.5 * (d[end - 1] - d[end]);
        double e2 = e[end - 1];
        double mu;
        if (td == 0.0) mu = d[end] - std::abs(e2);
        else {
            double h = std::hypot(td, e2);
            mu = d[end] - e2 * (e2 / (td + (td > 0 ? h : -h)));
        }
        double x = d[start] - mu, z = e[start];
        for (int k = start; k < end; ++k) {
            double r = std::hypot(x, z);
            double c = 1.0, s = 0.0;
            if (r != 0.0) { c = x / r; s = z / r; }
            if (k > start) e[k - 1] = r;
            double a = d[k], b = e[k], cc = d[k + 1];
            d[k] = c * c * a + 2.0 * c * s * b + s * s * cc;
            d[k + 1] = s * s * a - 2.0 * c * s * b + c * c * cc;
            e[k] = c * s * (cc - a) + (c * c - s * s) * b;
            if (k + 1 < end) {
                z = s * e[k + 1];
                e[k + 1] = c * e[k + 1];
            }
            x = e[k];
            if (Z) {
                double* zk = Z + (size_t)k * n;
                double* zk1 = Z + (size_t)(k + 1) * n;
                for (int i = 0; i < n; ++i) {
                    double a0 = zk[i], a1 = zk1[i];
                    zk[i] = c * a0 + s * a1;
                    zk1[i] = -s * a0 + c * a1;
                }
            }
        }
    }
    return 0;
}

// Full eigensolve: ascending eigenvalues w, optional eigenvectors (columns of Z).
static int eigh(int n, const double* Ain, double* w, double* Z) {
    if (n <= 0) return 0;
    std::vector<double> A(Ain, Ain + (size_t)n * n), e(std::max(n, 1), 0.0), tau(std::max(n, 1), 0.0);
    if (n == 1) {
        w[0] = A[0];
        if (Z) Z[0] = 1.0;
        return 0;
    }
    tridiagonalize(n, A.data(), w, e.data(), tau.data());
    if (Z) form_q(n, A.data(), tau.data(), Z);
    int rc = tridiag_qr(n, w, e.data(), Z);
    if (rc) return rc;
    // ascending selection sort, swapping eigenvector columns with it
    for (int i = 0; i + 1 < n; ++i) {
        int m = (int)(std::min_element(w + i, w + n) - w);
        if (m != i) {
            std::swap(w[i], w[m]);
            if (Z) std::swap_ranges(Z + (size_t)i * n, Z + (size_t)(i + 1) * n, Z + (size_t)m * n);
        }
    }
    return 0;
}

// ---------------------------------------------------------------------------
// configuration_t (include/fk_mc/configuration.hpp:52-87)
// ---------------------------------------------------------------------------
struct config_params {
    double beta, U, mu_c, mu_f;
    std::vector<double> W;
};

struct ed_cache {
    enum status_eval { empty, spectrum, full };
    status_eval status = empty;
    std::vector<double> cached_spectrum, cached_exp, cached_fermi, cached_evecs;
    double logZ = 0.0;
};

struct lattice_t {
    int kind, L, ndim, V;
    csr_t hop;
};

// chebyshev::chebyshev_eval (include/fk_mc/chebyshev.hpp:16-66): Lobatto
// grid x_i = -cos(pi theta_i), theta uniform on [0, 1], T_k(x_i) =
// cos(k acos(x_i)); moment() is the trapezoid rule in theta.
struct chebyshev_eval {
    int M, G;
    std::vector<double> theta, x, T;  // T[k * G + i]
    chebyshev_eval(int max_moment, int grid_size) : M(max_moment + max_moment % 2), G(grid_size) {
        const double step = 1.0 / (double)(G - 1);
        for (int i = 0; i < G; ++i) {
            theta.push_back((double)i * step);
            x.push_back(-std::cos(M_PI * theta.back()));
        }
        T.resize((size_t)M * G);
        for (int k = 0; k < M; ++k)
            for (int i = 0; i < G; ++i) T[(size_t)k * G + i] = std::cos((double)k * std::acos(x[i]));
    }
    template <typename F>
    double moment_f(const F& f, int order) const {
        std::vector<double> v(G);
        for (int i = 0; i < G; ++i) v[i] = f(x[i]);
        double s = 0.0;
        for (int i = 0; i + 1 < G; ++i)
            s += (v[i + 1] * T[(size_t)order * G + i + 1] + v[i] * T[(size_t)order * G + i]) * (theta[i + 1] - theta[i]);
        return s * 0.5;
    }
};

// include/fk_mc/configuration.hpp:36-50
struct chebyshev_cache {
    enum status_eval { empty, logz };
    status_eval status = empty;
    double e_max = 0, e_min = 0, a = 0, b = 0;
    std::vector<double> moments;
    double logZ = 0.0;
};

struct configuration_t {
    const lattice_t* lattice_;
    config_params params_;
    std::vector<int> f_config_;
    std::vector<double> hamilt_dense_;  // dense copy of H (src/configuration.cpp:212)
    ed_cache ed_data_;
    chebyshev_cache cheb_data_;

    configuration_t(const lattice_t& l, double beta, double U, double mu_c, double mu_f, std::vector<double> W = {})
        : lattice_(&l), params_{beta, U, mu_c, mu_f, W}, f_config_(l.V, 0) {}

    size_t get_nf() const {  // src/configuration.cpp:42-45
        size_t s = 0;
        for (int x : f_config_) s += x;
        return s;
    }
    // src/configuration.cpp:47-56
    void randomize_f(random_generator& rnd, size_t nf = 0) {
        std::uniform_int_distribution<> distr(0, lattice_->V - 1);
        if (!nf) nf = distr(rnd);
        std::fill(f_config_.begin(), f_config_.end(), 0);
        for (size_t i = 0; i < nf; ++i) {
            size_t ind = distr(rnd);
            while (f_config_[ind] == 1) ind = distr(rnd);
            f_config_[ind] = 1;
        }
    }
    // src/configuration.cpp:59-77 (only 1D lattices carry f-f interactions)
    double calc_ff_energy() const {
        if (lattice_->ndim != 1) return 0;
        double e = 0;
        int V = lattice_->V;
        for (int i = 0; i < V; ++i) {
            if (!f_config_[i]) continue;
            for (int l = 0; l < (int)params_.W.size(); ++l) {
                int left = (i - l + V) % V;
                int right = (i + l) % V;
                double el = params_.W[l] * f_config_[left];
                double er = params_.W[l] * f_config_[right];
                e += el;
                e += er * (l > 0);
            }
        }
        return e;
    }
    // src/configuration.cpp:79-91: H = hopping + diag(-mu_c + U f_i)
    void calc_hamiltonian() {
        ed_data_.status = ed_cache::empty;
        cheb_data_.status = chebyshev_cache::empty;
        int n = lattice_->hop.n;
        hamilt_dense_.assign((size_t)n * n, 0.0);
        const csr_t& h = lattice_->hop;
        for (int i = 0; i < n; ++i)
            for (int p = h.rowptr[i]; p < h.rowptr[i + 1]; ++p) hamilt_dense_[(size_t)h.col[p] * n + i] += h.val[p];
        for (int i = 0; i < n; ++i) hamilt_dense_[(size_t)i * n + i] += -params_.mu_c + params_.U * f_config_[i];
    }
    // src/configuration.cpp:208-246
    void calc_ed(bool calc_evecs = false) {
        if ((ed_data_.status == ed_cache::spectrum && !calc_evecs) || (ed_data_.status == ed_cache::full && calc_evecs))
            return;
        int n = lattice_->hop.n;
        ed_data_.cached_spectrum.assign(n, 0.0);
        if (calc_evecs) ed_data_.cached_evecs.assign((size_t)n * n, 0.0);
        if (eigh(n, hamilt_dense_.data(), ed_data_.cached_spectrum.data(),
                 calc_evecs ? ed_data_.cached_evecs.data() : nullptr))
            throw std::runtime_error("eigensolver did not converge");
        ed_data_.status = calc_evecs ? ed_cache::full : ed_cache::spectrum;
        const auto& spec = ed_data_.cached_spectrum;
        double beta = params_.beta;
        double e0 = spec[0];
        double logw0 = beta * e0;
        double weight0 = std::exp(logw0);
        ed_data_.cached_exp.resize(n);
        ed_data_.cached_fermi.resize(n);
        double logz = 0.0;
        for (int i = 0; i < n; ++i) {
            double e = spec[i];
            double w = std::exp(-beta * (e - e0));
            ed_data_.cached_exp[i] = std::exp(beta * e);
            ed_data_.cached_fermi[i] = 1.0 / (1.0 + ed_data_.cached_exp[i]);
            logz += std::log(weight0 + w) - logw0;
        }
        ed_data_.logZ = logz;
    }
    // src/configuration.cpp:94-205: bounds (the reference asks ARPACK for the
    // extreme eigenvalues; here they come from the dense eigensolve), x =
    // (H - b)/a, moments Tr T_m(x)/N (recursion for m <= M/2, products for
    // the rest, in the reference's order), logZ = sum (2 - [m=0]) c_m mu_m.
    void calc_chebyshev(const chebyshev_eval& cheb) {
        if (cheb_data_.status == chebyshev_cache::logz) return;
        const int n = lattice_->hop.n;
        std::vector<double> w(n);
        if (eigh(n, hamilt_dense_.data(), w.data(), nullptr)) throw std::runtime_error("eigensolver did not converge");
        const double e_min = w[0], e_max = w[n - 1];
        const double a = (e_max - e_min) / 2., b = (e_max + e_min) / 2.;
        cheb_data_.e_min = e_min;
        cheb_data_.e_max = e_max;
        cheb_data_.a = a;
        cheb_data_.b = b;
        std::vector<double> x(hamilt_dense_);
        for (int i = 0; i < n; ++i) x[(size_t)i * n + i] += -b;
        for (double& v : x) v /= a;
        const int M = cheb.M;
        auto trace = [n](const std::vector<double>& A) { double s = 0; for (int i = 0; i < n; ++i) s += A[(size_t)i * n + i]; return s; };
        auto dot = [](const std::vector<double>& A, const std::vector<double>& B) { double s = 0; for (size_t k = 0; k < A.size(); ++k) s += A[k] * B[k]; return s; };
        std::vector<double> c0((size_t)n * n, 0.0), c1(x), tmp((size_t)n * n);
        for (int i = 0; i < n; ++i) c0[(size_t)i * n + i] = 1.0;
        std::vector<double> mu(M, 0.0);
        std::vector<bool> is_set(M, false);
        mu[0] = 1.0;
        is_set[0] = true;
        const double trx = trace(x);
        if (M > 1) { mu[1] = trace(c1) / n; is_set[1] = true; }
        for (int m = 2; m <= M / 2; ++m) {
            // tmp = 2 x c1 - c0 (all matrices symmetric, column-major)
            for (int j = 0; j < n; ++j)
                for (int i = 0; i < n; ++i) {
                    double s = 0.0;
                    for (int k = 0; k < n; ++k) s += x[(size_t)k * n + i] * c1[(size_t)j * n + k];
                    tmp[(size_t)j * n + i] = 2. * s - c0[(size_t)j * n + i];
                }
            c0.swap(c1);
            c1.swap(tmp);
            if (!is_set[m]) { mu[m] = trace(c1) / n; is_set[m] = true; }
            int k = 2 * m - 1;
            if (k < M && k >= M / 2) {
                mu[k] = (dot(c0, c1) * 2. - trx) / n;
                is_set[k] = true;
                if (k != M - 1) {
                    ++k;
                    mu[k] = dot(c1, c1) / n * 2. - 1.0;
                    is_set[k] = true;
                }
            }
        }
        cheb_data_.moments = mu;
        const double beta = params_.beta;
        auto logz_f = [a, b, beta, n](double wv) { return n * std::log(1. + std::exp(-beta * (a * wv + b))); };
        double s = cheb.moment_f(logz_f, 0);
        for (int m = 1; m < M; ++m) s += 2. * cheb.moment_f(logz_f, m) * mu[m];
        cheb_data_.logZ = s;
        cheb_data_.status = chebyshev_cache::logz;
    }
};

// ---------------------------------------------------------------------------
// moves (src/moves.cpp:5-67)
// ---------------------------------------------------------------------------
struct move_base {
    double beta;
    configuration_t& config;
    configuration_t new_config;
    random_generator& RND;
    int last_site = -1;  // site flipped by the last add/remove attempt (-1 for the other moves)
    move_base(double b, configuration_t& c, random_generator& r) : beta(b), config(c), new_config(c), RND(r) {}
    virtual ~move_base() {}
    virtual double attempt() = 0;
    double accept() { config = new_config; return 1.0; }  // src/moves.cpp:23-28
    void reject() {}
};

struct move_flip : move_base {  // src/moves.cpp:5-21
    using move_base::move_base;
    double attempt() override {
        std::uniform_int_distribution<> distr(0, config.lattice_->V - 1);
        if (config.get_nf() == 0 || config.get_nf() == (size_t)config.lattice_->hop.n) return 0;
        new_config = config;
        size_t from = distr(RND);
        while (new_config.f_config_[from] == 0) from = distr(RND);
        size_t to = distr(RND);
        while (new_config.f_config_[to] == 1) to = distr(RND);
        config.calc_ed(false);
        new_config.f_config_[from] = 0;
        new_config.f_config_[to] = 1;
        new_config.calc_hamiltonian();
        new_config.calc_ed(false);
        return std::exp(new_config.ed_data_.logZ - config.ed_data_.logZ);
    }
};

struct move_randomize : move_base {  // src/moves.cpp:35-49
    using move_base::move_base;
    double attempt() override {
        new_config = config;
        new_config.randomize_f(RND);
        new_config.calc_hamiltonian();
        config.calc_ed(false);
        new_config.calc_ed(false);
        double log_ratio = new_config.ed_data_.logZ - config.ed_data_.logZ;
        double ff_diff = new_config.calc_ff_energy() - config.calc_ff_energy();
        // The reference subtracts two size_t counts: a decrease wraps to a
        // huge unsigned value. Restated as written.
        double dnf = (double)(new_config.get_nf() - config.get_nf());
        double mu_f = config.params_.mu_f;
        if (beta * mu_f * dnf - ff_diff > 2.7182818 - log_ratio) return 1;
        else if (beta * mu_f * dnf - ff_diff + log_ratio < 0) return 0;
        else return std::exp(log_ratio) * std::exp(beta * (mu_f * dnf - ff_diff));
    }
};

struct move_addremove : move_base {  // src/moves.cpp:52-67
    double exp_beta_mu_f;
    move_addremove(double b, configuration_t& c, random_generator& r)
        : move_base(b, c, r), exp_beta_mu_f(std::exp(b * c.params_.mu_f)) {}
    double attempt() override {
        std::uniform_int_distribution<> distr(0, config.lattice_->V - 1);
        new_config = config;
        size_t to = distr(RND);
        last_site = (int)to;
        new_config.f_config_[to] = 1 - config.f_config_[to];
        config.calc_ed(false);
        new_config.calc_hamiltonian();
        new_config.calc_ed(false);
        double ff_diff = new_config.calc_ff_energy() - config.calc_ff_energy();
        double ratio = std::exp(new_config.ed_data_.logZ - config.ed_data_.logZ);
        return (new_config.f_config_[to] ? ratio * exp_beta_mu_f : ratio / exp_beta_mu_f) * std::exp(-beta * ff_diff);
    }
};

// chebyshev::move_flip / move_randomize / move_addremove
// (src/moves_chebyshev.cpp:6-72): the ED moves with calc_chebyshev in place
// of calc_ed, in the reference's order of calls and random draws.
struct cheb_move_flip : move_base {
    const chebyshev_eval& cheb_;
    cheb_move_flip(double b, configuration_t& c, const chebyshev_eval& ch, random_generator& r) : move_base(b, c, r), cheb_(ch) {}
    double attempt() override {
        config.calc_chebyshev(cheb_);
        if (config.get_nf() == 0 || config.get_nf() == (size_t)config.lattice_->hop.n) return 0;
        std::uniform_int_distribution<> distr(0, config.lattice_->hop.n - 1);
        new_config = config;
        size_t from = distr(RND);
        while (new_config.f_config_[from] == 0) from = distr(RND);
        size_t to = distr(RND);
        while (new_config.f_config_[to] == 1) to = distr(RND);
        new_config.f_config_[from] = 0;
        new_config.f_config_[to] = 1;
        new_config.calc_hamiltonian();
        new_config.calc_chebyshev(cheb_);
        double ff_diff = new_config.calc_ff_energy() - config.calc_ff_energy();
        return std::exp(new_config.cheb_data_.logZ - config.cheb_data_.logZ - beta * ff_diff);
    }
};

struct cheb_move_randomize : move_base {
    const chebyshev_eval& cheb_;
    cheb_move_randomize(double b, configuration_t& c, const chebyshev_eval& ch, random_generator& r) : move_base(b, c, r), cheb_(ch) {}
    double attempt() override {
        config.calc_chebyshev(cheb_);
        new_config = config;
        new_config.randomize_f(RND);
        new_config.calc_hamiltonian();
        new_config.calc_chebyshev(cheb_);
        double log_ratio = new_config.cheb_data_.logZ - config.cheb_data_.logZ;
        double ff_diff = new_config.calc_ff_energy() - config.calc_ff_energy();
        double dnf = (double)(new_config.get_nf() - config.get_nf());  // size_t difference, as written
        double mu_f = config.params_.mu_f;
        if (beta * mu_f * dnf - ff_diff > 2.7182818 - log_ratio) return 1;
        else if (beta * mu_f * dnf - ff_diff + log_ratio < 0) return 0;
        else return std::exp(log_ratio) * std::exp(beta * (mu_f * dnf - ff_diff));
    }
};

struct cheb_move_addremove : move_base {
    const chebyshev_eval& cheb_;
    double exp_beta_mu_f;
    cheb_move_addremove(double b, configuration_t& c, const chebyshev_eval& ch, random_generator& r)
        : move_base(b, c, r), cheb_(ch), exp_beta_mu_f(std::exp(b * c.params_.mu_f)) {}
    double attempt() override {
        std::uniform_int_distribution<> distr(0, config.lattice_->hop.n - 1);
        config.calc_chebyshev(cheb_);
        new_config = config;
        size_t to = distr(RND);
        last_site = (int)to;
        new_config.f_config_[to] = 1 - config.f_config_[to];
        new_config.calc_hamiltonian();
        new_config.calc_chebyshev(cheb_);
        double ff_diff = new_config.calc_ff_energy() - config.calc_ff_energy();
        double ratio = std::exp(new_config.cheb_data_.logZ - config.cheb_data_.logZ);
        return (new_config.f_config_[to] ? ratio * exp_beta_mu_f : ratio / exp_beta_mu_f) * std::exp(-beta * ff_diff);
    }
};

// measure_energy::accumulate (src/measures/energy.cpp:6-26)
static void energy_estimators(configuration_t& config, double* e_val, double* d2e_val, double* e_val_c) {
    config.calc_ed(false);
    const auto& spectrum = config.ed_data_.cached_spectrum;
    const auto& exp_e = config.ed_data_.cached_exp;
    double se = 0.0, sd2 = 0.0;
    for (size_t i = 0; i < spectrum.size(); ++i) {
        se += spectrum[i] / (1.0 + exp_e[i]);
        sd2 += spectrum[i] * spectrum[i] / (1.0 + 0.5 * (exp_e[i] + 1. / exp_e[i]));
    }
    *e_val_c = se;
    *e_val = se - double(config.params_.mu_f) * config.get_nf() + config.calc_ff_energy();
    *d2e_val = sd2 / 2.0;
}

}  // namespace orc

// ---------------------------------------------------------------------------
// C ABI used by the Python tests and by bench.py's CPU-baseline legs.
// ---------------------------------------------------------------------------
using namespace orc;

extern "C" {

// Lattice hopping in CSR. Returns nnz (>= 0) or -1 on bad arguments. Call with
// null arrays to query n (written to *n_out) and nnz.
int orc_lattice_csr(int kind, int L, double t, double tp, int* n_out, int* rowptr, int* col, double* val) {
    try {
        csr_t c = make_lattice(kind, L, t, tp);
        if (n_out) *n_out = c.n;
        if (rowptr) std::copy(c.rowptr.begin(), c.rowptr.end(), rowptr);
        if (col) std::copy(c.col.begin(), c.col.end(), col);
        if (val) std::copy(c.val.begin(), c.val.end(), val);
        return (int)c.col.size();
    } catch (...) {
        return -1;
    }
}

// Dense symmetric eigensolve of a column-major n x n matrix (lower triangle read).
int orc_eigh(int n, const double* A, double* w, double* Z) { return eigh(n, A, w, Z); }

// Householder tridiagonal (d[n], e[n-1]) of a column-major n x n matrix.
int orc_tridiag(int n, const double* Ain, double* d, double* e) {
    std::vector<double> A(Ain, Ain + (size_t)n * n), tau(std::max(n, 1)), ee(std::max(n, 1));
    if (n == 1) { d[0] = A[0]; return 0; }
    tridiagonalize(n, A.data(), d, ee.data(), tau.data());
    std::copy(ee.begin(), ee.begin() + (n - 1), e);
    return 0;
}

// One configuration_t::calc_ed on lattice (kind, L, t, tp) with f-occupations
// f[V]. Outputs are the ed_cache fields; evecs may be null.
int orc_calc_ed(int kind, int L, double t, double tp, const int* f, double beta, double U, double mu_c,
                int calc_evecs, double* spectrum, double* exp_e, double* fermi, double* evecs, double* logz) {
    try {
        lattice_t lat{kind, L, lattice_ndim(kind), 0, make_lattice(kind, L, t, tp)};
        lat.V = lat.hop.n;
        configuration_t c(lat, beta, U, mu_c, mu_c);
        std::copy(f, f + lat.V, c.f_config_.begin());
        c.calc_hamiltonian();
        c.calc_ed(calc_evecs != 0);
        int n = lat.V;
        std::copy(c.ed_data_.cached_spectrum.begin(), c.ed_data_.cached_spectrum.end(), spectrum);
        if (exp_e) std::copy(c.ed_data_.cached_exp.begin(), c.ed_data_.cached_exp.end(), exp_e);
        if (fermi) std::copy(c.ed_data_.cached_fermi.begin(), c.ed_data_.cached_fermi.end(), fermi);
        if (evecs && calc_evecs) std::copy(c.ed_data_.cached_evecs.begin(), c.ed_data_.cached_evecs.begin() + (size_t)n * n, evecs);
        if (logz) *logz = c.ed_data_.logZ;
        return 0;
    } catch (...) {
        return -1;
    }
}

// logZ of a given ascending spectrum, exactly as src/configuration.cpp:224-245.
double orc_logz_of_spectrum(int n, const double* spec, double beta) {
    double e0 = spec[0], logw0 = beta * e0, weight0 = std::exp(logw0), logz = 0.0;
    for (int i = 0; i < n; ++i) logz += std::log(weight0 + std::exp(-beta * (spec[i] - e0))) - logw0;
    return logz;
}

// measure_stiffness::accumulate on a 2D square lattice of side L, hopping t,
// for the f-configuration f (include/fk_mc/measures/stiffness.hpp:49-187 and
// the set-up of test/stiffness_test.cpp:12-33). Returns the stiffness.
double orc_stiffness(int L, double t, double U, double beta, const int* f) {
    lattice_t lat{2, L, 2, 0, make_lattice(2, L, t, 0.0)};
    lat.V = lat.hop.n;
    int n = lat.V;
    double mu = U / 2;
    configuration_t c(lat, beta, U, mu, mu);
    std::copy(f, f + n, c.f_config_.begin());
    c.calc_hamiltonian();
    c.calc_ed(true);
    const auto& X = c.ed_data_.cached_evecs;
    const auto& ev = c.ed_data_.cached_spectrum;
    const auto& fermi = c.ed_data_.cached_fermi;
    // T and J along axis 0 (pos[0]), t_ = 1 as in the reference measure.
    const double t_ = 1.0;
    std::vector<std::map<int, double>> Tm(n), Jm(n);
    for (int i = 0; i < n; ++i) {
        auto p0 = index_to_pos(2, L, i), pl = p0, pr = p0;
        pl[0] = ((p0[0] - 1) + L) % L;
        pr[0] = ((p0[0] + 1) + L) % L;
        int il = pos_to_index(2, L, pl), ir = pos_to_index(2, L, pr);
        Tm[i][il] += -t_;
        Tm[i][ir] += -t_;
        Jm[i][il] += -1;
        Jm[i][ir] += 1;
    }
    // JX = Jm * X, TX = Tm * X; mJ = X^T J X; T = -pi * sum_k (x_k^T Tm x_k) f_k
    std::vector<double> JX((size_t)n * n, 0.0);
    double T = 0.0;
    for (int k = 0; k < n; ++k) {
        const double* xk = &X[(size_t)k * n];
        double tk = 0.0;
        for (int i = 0; i < n; ++i) {
            double sj = 0.0, st = 0.0;
            for (auto& kv : Jm[i]) sj += kv.second * xk[kv.first];
            for (auto& kv : Tm[i]) st += kv.second * xk[kv.first];
            JX[(size_t)k * n + i] = sj;
            tk += xk[i] * st;
        }
        T += tk * fermi[k];
    }
    T *= -M_PI;
    std::vector<double> mJ((size_t)n * n, 0.0);  // mJ(a,b) = x_a^T J x_b
    for (int b = 0; b < n; ++b)
        for (int a = 0; a < n; ++a) {
            double s = 0.0;
            for (int i = 0; i < n; ++i) s += X[(size_t)a * n + i] * JX[(size_t)b * n + i];
            mJ[(size_t)b * n + a] = s;
        }
    double V = 0.0;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j) {
            bool neq = std::abs(ev[i] - ev[j]) > 1e-12;
            if (neq) {
                double sigma_v = M_PI * (fermi[j] - fermi[i]) * mJ[(size_t)i * n + j] * mJ[(size_t)j * n + i];
                double V_val = 2. * sigma_v / (ev[i] - ev[j]);
                if (std::abs(sigma_v) > 1e-13) V += V_val;
            }
        }
    return (V + T) / n;
}

// measure_ipr::accumulate (include/fk_mc/measures/ipr.hpp:39-56) on given
// eigenvectors (column-major n x n): ipr_k = ||x_k||_4 / ||x_k||_2^2.
void orc_ipr(int n, const double* X, double* ipr) {
    for (int k = 0; k < n; ++k) {
        double s2 = 0, s4 = 0;
        for (int i = 0; i < n; ++i) { double x = X[(size_t)k * n + i]; s2 += x * x; s4 += x * x * x * x; }
        ipr[k] = std::pow(s4, 0.25) / s2;
    }
}

// Parameters of one Markov chain run, as fk_mc::define_parameters /
// mc_metropolis::define_parameters name them.
struct orc_mc_params {
    int kind, L;
    double t, tp;
    double beta, U, mu_c, mu_f;
    long long seed;         // SEED + rank
    int nsweeps, sweep_len, ntherm_sweeps;
    double mc_flip, mc_add_remove, mc_reshuffle;
    int nf_start;           // randomize_f(rng, Nf_start); < 0 => use f_init as is
    const int* f_init;      // used when nf_start < 0
    int cheb_moves;         // the Chebyshev moves (include/fk_mc/fk_mc.hxx:55-78)
    double cheb_prefactor;  // cheb_size = int(log(V) * cheb_prefactor), even
};

// Output arrays sized by the caller:
//   move_index, accepted, site: (nsweeps+ntherm)*sweep_len entries
//   weight: same (the |w| compared with the uniform), uniform: same
//   energy, d2energy, c_energy: nsweeps entries;  f_final: V entries
struct orc_mc_out {
    int* move_index;
    int* accepted;
    int* site;
    double* weight;
    double* uniform;
    double* energy;
    double* d2energy;
    double* c_energy;
    int* f_final;
    int* f_initial;  // configuration after randomize_f, before the first sweep
    long long naccept;
};

// One chain driven as fk_mc::initialize + alps::mcbase::run would drive it:
// update() then measure() until sweep_count reaches nsweeps + ntherm_sweeps.
int orc_mc_run(const orc_mc_params* P, orc_mc_out* O) {
    try {
        lattice_t lat{P->kind, P->L, lattice_ndim(P->kind), 0, make_lattice(P->kind, P->L, P->t, P->tp)};
        lat.V = lat.hop.n;
        random_generator random((random_generator::result_type)P->seed);  // src/mc_metropolis.cpp:25
        configuration_t config(lat, P->beta, P->U, P->mu_c, P->mu_f);
        if (P->nf_start >= 0) config.randomize_f(random, P->nf_start);
        else std::copy(P->f_init, P->f_init + lat.V, config.f_config_.begin());
        if (O && O->f_initial) std::copy(config.f_config_.begin(), config.f_config_.end(), O->f_initial);
        config.calc_hamiltonian();
        std::vector<std::unique_ptr<move_base>> moves;
        std::vector<double> probs;
        std::vector<int> kinds;
        const double eps = std::numeric_limits<double>::epsilon();
        // include/fk_mc/fk_mc.hxx:59-64: cheb_size and the grid of the evaluator
        std::unique_ptr<chebyshev_eval> cheb;
        if (P->cheb_moves) {
            int cs = int(std::log((double)lat.V) * P->cheb_prefactor);
            cs += cs % 2;
            cheb.reset(new chebyshev_eval(cs, std::max(cs * 2, 10)));
        }
        if (P->mc_flip > eps) {
            if (cheb) moves.emplace_back(new cheb_move_flip(P->beta, config, *cheb, random));
            else moves.emplace_back(new move_flip(P->beta, config, random));
            probs.push_back(P->mc_flip); kinds.push_back(0);
        }
        if (P->mc_add_remove > eps) {
            if (cheb) moves.emplace_back(new cheb_move_addremove(P->beta, config, *cheb, random));
            else moves.emplace_back(new move_addremove(P->beta, config, random));
            probs.push_back(P->mc_add_remove); kinds.push_back(1);
        }
        if (P->mc_reshuffle > eps) {
            if (cheb) moves.emplace_back(new cheb_move_randomize(P->beta, config, *cheb, random));
            else moves.emplace_back(new move_randomize(P->beta, config, random));
            probs.push_back(P->mc_reshuffle); kinds.push_back(2);
        }
        if (moves.empty()) return -2;
        std::discrete_distribution<> move_distrib(probs.begin(), probs.end());
        std::uniform_real_distribution<> metropolis_distrib(0, 1);
        long sweep_count = 0, measure_count = 0, naccept = 0, prop = 0, meas = 0;
        double phase = 1.0;
        long total = (long)P->nsweeps + P->ntherm_sweeps;
        do {
            for (int m = 0; m < P->sweep_len; ++m) {  // src/mc_metropolis.cpp:34-52
                int idx = move_distrib(random);
                double weight = moves[idx]->attempt();
                double u = metropolis_distrib(random);
                bool acc = std::abs(weight) > u;
                if (acc) {
                    weight *= moves[idx]->accept();
                    naccept++;
                    phase *= (0.0 < weight) - (weight < 0.0);
                } else moves[idx]->reject();
                if (O) {
                    if (O->move_index) O->move_index[prop] = kinds[idx];
                    if (O->accepted) O->accepted[prop] = acc;
                    if (O->weight) O->weight[prop] = weight;
                    if (O->uniform) O->uniform[prop] = u;
                    if (O->site) O->site[prop] = moves[idx]->last_site;
                }
                ++prop;
            }
            sweep_count++;
            // with the Chebyshev moves the reference registers no energy measure
            // (include/fk_mc/fk_mc.hxx:94-114)
            if (measure_count >= P->ntherm_sweeps && !P->cheb_moves) {  // src/mc_metropolis.cpp:54-61
                double e, d2e, ec;
                energy_estimators(config, &e, &d2e, &ec);
                if (O && O->energy) { O->energy[meas] = e; O->d2energy[meas] = d2e; O->c_energy[meas] = ec; }
                ++meas;
            }
            measure_count++;
        } while ((double)sweep_count / (double)total < 1.0);
        if (O) {
            if (O->f_final) std::copy(config.f_config_.begin(), config.f_config_.end(), O->f_final);
            O->naccept = naccept;
        }
        return 0;
    } catch (...) {
        return -1;
    }
}

// CPU baseline: single-site-flip proposals (one calc_ed each, plus the
// Metropolis decision) on independent chains, one chain per std::thread, for
// about `seconds` of wall time. Chain c starts from Bernoulli(0.5) f drawn from
// std::mt19937(seed + c) and uses that generator for its moves. Returns the
// number of proposals completed; *elapsed gets the wall time in seconds.
long long orc_bench_proposals(int kind, int L, double t, double tp, double beta, double U, double mu_c,
                              double mu_f, long long seed, int threads, double seconds, int max_props_per_thread,
                              double* elapsed) {
    lattice_t lat{kind, L, lattice_ndim(kind), 0, make_lattice(kind, L, t, tp)};
    lat.V = lat.hop.n;
    std::atomic<long long> total{0};
    auto t0 = std::chrono::steady_clock::now();
    auto worker = [&](int c) {
        random_generator rng((random_generator::result_type)(seed + c));
        configuration_t config(lat, beta, U, mu_c, mu_f);
        std::bernoulli_distribution bern(0.5);
        for (int i = 0; i < lat.V; ++i) config.f_config_[i] = bern(rng);
        config.calc_hamiltonian();
        move_addremove mv(beta, config, rng);
        std::uniform_real_distribution<> ud(0, 1);
        long long done = 0;
        while (done < max_props_per_thread) {
            double w = mv.attempt();
            if (std::abs(w) > ud(rng)) mv.accept(); else mv.reject();
            ++done;
            double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (el > seconds) break;
        }
        total += done;
    };
    std::vector<std::thread> th;
    for (int c = 0; c < threads; ++c) th.emplace_back(worker, c);
    for (auto& x : th) x.join();
    if (elapsed) *elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return total.load();
}

}  // extern "C"

extern "C" {

// Steady-state CPU timing of running chains: `threads` independent chains
// (chain c from Bernoulli(0.5) f of std::mt19937(seed + c)) each do `warmup`
// untimed single-site-flip proposals — the first one also solves the starting
// configuration, which a running chain has cached — then wait at a common
// start line; from there each does `steps` proposals (one calc_ed of the
// proposed configuration and the Metropolis decision each). *elapsed gets the
// wall time from the start line to the last chain's end; the return value is
// the number of timed proposals (threads * steps).
long long orc_bench_steps(int kind, int L, double t, double tp, double beta, double U, double mu_c, double mu_f,
                          long long seed, int threads, int warmup, int steps, double* elapsed) {
    lattice_t lat{kind, L, lattice_ndim(kind), 0, make_lattice(kind, L, t, tp)};
    lat.V = lat.hop.n;
    std::atomic<int> ready{0};
    std::atomic<bool> go{false};
    std::atomic<long long> total{0};
    auto worker = [&](int c) {
        random_generator rng((random_generator::result_type)(seed + c));
        configuration_t config(lat, beta, U, mu_c, mu_f);
        std::bernoulli_distribution bern(0.5);
        for (int i = 0; i < lat.V; ++i) config.f_config_[i] = bern(rng);
        config.calc_hamiltonian();
        move_addremove mv(beta, config, rng);
        std::uniform_real_distribution<> ud(0, 1);
        auto one = [&]() {
            double w = mv.attempt();
            if (std::abs(w) > ud(rng)) mv.accept(); else mv.reject();
        };
        for (int k = 0; k < std::max(warmup, 1); ++k) one();
        ready.fetch_add(1);
        while (!go.load()) std::this_thread::yield();
        for (int k = 0; k < steps; ++k) one();
        total += steps;
    };
    std::vector<std::thread> th;
    for (int c = 0; c < threads; ++c) th.emplace_back(worker, c);
    while (ready.load() < threads) std::this_thread::yield();
    auto t0 = std::chrono::steady_clock::now();
    go.store(true);
    for (auto& x : th) x.join();
    if (elapsed) *elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return total.load();
}

}  // extern "C"
