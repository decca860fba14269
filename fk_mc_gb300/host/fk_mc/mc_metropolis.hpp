// mc_metropolis.hpp — the Metropolis engine of include/fk_mc/mc_metropolis.hpp
// (move/measure registry, update/measure, random-draw order), without the
// ALPSCore base class: run() alternates update() and measure() until
// nsweeps + ntherm_sweeps sweeps are done, as alps::mcbase::run does with
// fraction_completed() (src/mc_metropolis.cpp:62-84).
#pragma once
#include <functional>
#include <map>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

namespace fk {

typedef double mc_weight_t;

struct mc_metropolis {
    typedef std::mt19937 random_generator;

    mc_metropolis(long seed, long nsweeps = 1024, long sweep_len = 16, long ntherm_sweeps = 1)
        : random((random_generator::result_type)seed), measure_sweeps_(nsweeps), sweep_len_(sweep_len),
          thermalization_sweeps_(ntherm_sweeps) {}

    template <typename Move_t>
    bool add_move(std::shared_ptr<Move_t> move, std::string name, double move_prob = 1.0) {
        moves_.push_back({[move]() { return move->attempt(); }, [move]() { return move->accept(); },
                          [move]() { move->reject(); }});
        move_names_.push_back(name);
        move_probs_.push_back(move_prob);
        move_distrib_ = std::discrete_distribution<>(move_probs_.begin(), move_probs_.end());
        return true;
    }
    bool add_measure(std::function<void(mc_weight_t)> accumulate, std::string name) {
        measures_.emplace(name, accumulate);
        return true;
    }

    // one sweep: sweep_len proposals (src/mc_metropolis.cpp:34-52)
    void update() {
        if (moves_.empty()) throw std::logic_error("No registered moves");
        for (long m = 0; m < sweep_len_; m++) {
            const int move_index = move_distrib_(random);
            mc_weight_t weight = moves_[move_index].attempt();
            const double u = metropolis_distrib_(random);
            const bool acc = std::abs(weight) > u;
            if (acc) {
                weight *= moves_[move_index].accept();
                naccept_++;
                phase_ *= (0.0 < weight) - (weight < 0.0);
            } else moves_[move_index].reject();
            if (on_proposal) on_proposal(move_index, weight, u, acc);
        }
        sweep_count_++;
    }
    void measure() {  // src/mc_metropolis.cpp:54-61
        if (measure_count_ >= thermalization_sweeps_)
            for (auto& m : measures_) m.second(phase_);
        measure_count_++;
    }
    double fraction_completed() const {
        return double(sweep_count_) / double(measure_sweeps_ + thermalization_sweeps_);
    }
    void run() {
        do {
            update();
            measure();
        } while (fraction_completed() < 1.);
    }
    double acceptance_rate() const { return double(naccept_) / double(sweep_count_ * sweep_len_); }
    random_generator& rng() { return random; }

    // optional observer of every proposal (move index, weight, uniform, accepted)
    std::function<void(int, double, double, bool)> on_proposal;

protected:
    struct move_wrap {
        std::function<mc_weight_t()> attempt, accept;
        std::function<void()> reject;
    };
    std::vector<move_wrap> moves_;
    std::vector<std::string> move_names_;
    std::vector<double> move_probs_;
    std::map<std::string, std::function<void(mc_weight_t)>> measures_;
    random_generator random;
    long measure_sweeps_, sweep_len_, thermalization_sweeps_;
    long sweep_count_ = 0, measure_count_ = 0, naccept_ = 0;
    std::discrete_distribution<> move_distrib_;
    std::uniform_real_distribution<> metropolis_distrib_ = std::uniform_real_distribution<>(0, 1);
    mc_weight_t phase_ = 1.0;
};

}  // namespace fk
