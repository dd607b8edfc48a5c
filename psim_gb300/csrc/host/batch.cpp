#include "batch.hpp"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <exception>
#include <map>
#include <mutex>
#include <stdexcept>
#include <thread>

#include "../device/engine.hpp"
#include "model.hpp"

namespace psim {

namespace {

// Runs f(i) for i in [0, n) on up to `workers` threads; rethrows the first failure.
template<typename F> void parallel_for(std::size_t n, int workers, F f) {
    std::atomic<std::size_t> next{ 0 };
    std::mutex err_mu;
    std::exception_ptr first_error;
    std::atomic<bool> failed{ false };
    auto work = [&]() {
        try {
            while (!failed.load()) {
                const std::size_t i = next.fetch_add(1);
                if (i >= n) { break; }
                f(i);
            }
        } catch (...) {
            std::lock_guard<std::mutex> lock(err_mu);
            if (!first_error) { first_error = std::current_exception(); }
            failed.store(true);
        }
    };
    const int t = std::max(1, std::min<int>(workers, static_cast<int>(n)));
    std::vector<std::thread> pool;
    pool.reserve(static_cast<std::size_t>(t));
    for (int w = 0; w < t; ++w) { pool.emplace_back(work); }
    for (auto& th : pool) { th.join(); }
    if (first_error) { std::rethrow_exception(first_error); }
}

// Every model on its own: worker threads with a CUDA stream each.
std::uint64_t run_each(const std::vector<HostModel*>& models, const BatchOptions& opt) {
    if (models.empty()) { return 0; }
    const int workers = std::max(1, std::min<int>(opt.workers, static_cast<int>(models.size())));
    std::atomic<std::size_t> next{ 0 };
    std::atomic<std::uint64_t> steps{ 0 };
    std::mutex err_mu;
    std::exception_ptr first_error;
    std::atomic<bool> failed{ false };
    auto work = [&]() {
        void* stream = nullptr;
        try {
            stream = gpu::create_stream();
            while (!failed.load()) {
                const std::size_t i = next.fetch_add(1);
                if (i >= models.size()) { break; }
                HostModel& m = *models[i];
                void* const old_stream = m.stream();
                const int old_grid = m.grid();
                m.set_stream(stream);
                m.set_grid(opt.max_blocks);
                try {
                    m.run();
                } catch (...) {
                    m.set_stream(old_stream);
                    m.set_grid(old_grid);
                    throw;
                }
                m.set_stream(old_stream);
                m.set_grid(old_grid);
                steps.fetch_add(m.counters().phonon_steps);
            }
        } catch (...) {
            std::lock_guard<std::mutex> lock(err_mu);
            if (!first_error) { first_error = std::current_exception(); }
            failed.store(true);
        }
        gpu::destroy_stream(stream);
    };
    std::vector<std::thread> pool;
    pool.reserve(static_cast<std::size_t>(workers));
    for (int w = 0; w < workers; ++w) { pool.emplace_back(work); }
    for (auto& t : pool) { t.join(); }
    if (first_error) { std::rethrow_exception(first_error); }
    return steps.load();
}

// The models' transports in batched launches, grouped by their number of steps; run by run
// (models with more runs go on alone after the others finish theirs).
std::uint64_t run_queued(const std::vector<HostModel*>& models, const BatchOptions& opt) {
    std::map<std::size_t, std::vector<HostModel*>> groups;
    for (HostModel* m : models) { groups[m->n_steps()].push_back(m); }
    std::uint64_t steps = 0;
    void* stream = gpu::create_stream();
    try {
        for (auto& [n_steps, group] : groups) {
            (void)n_steps;
            for (HostModel* m : group) { m->begin_runs(); }
            std::size_t max_runs = 0;
            for (HostModel* m : group) { max_runs = std::max(max_runs, m->n_runs()); }
            for (std::size_t r = 0; r < max_runs; ++r) {
                std::vector<HostModel*> members;
                for (HostModel* m : group) {
                    if (m->n_runs() > r) { members.push_back(m); }
                }
                parallel_for(members.size(), opt.workers, [&](std::size_t i) { members[i]->prepare_run(r); });
                std::vector<gpu::Engine*> engines;
                for (HostModel* m : members) { engines.push_back(m->engine()); }
                if (!gpu::Engine::run_batched(engines, stream, static_cast<std::uint32_t>(std::max(1, opt.per_thread)))) {
                    for (HostModel* m : members) { m->engine()->run(m->precision(), stream); }
                }
                parallel_for(members.size(), opt.workers, [&](std::size_t i) { members[i]->finish_run(); });
            }
            for (HostModel* m : group) {
                m->end_runs();
                steps += m->counters().phonon_steps;
            }
        }
    } catch (...) {
        gpu::destroy_stream(stream);
        throw;
    }
    gpu::destroy_stream(stream);
    return steps;
}

}// namespace

BatchResult run_batch(const std::vector<HostModel*>& models, const BatchOptions& opt) {
    if (opt.workers < 1) { throw std::invalid_argument("a batch needs at least one worker"); }
    if (opt.max_blocks < 0) { throw std::invalid_argument("blocks per launch must not be negative"); }
    if (opt.per_thread < 1) { throw std::invalid_argument("a work item needs at least one phonon per thread"); }
    for (const HostModel* m : models) {
        if (m == nullptr) { throw std::invalid_argument("null model in the batch"); }
    }
    for (std::size_t i = 0; i < models.size(); ++i) {
        for (std::size_t j = i + 1; j < models.size(); ++j) {
            if (models[i] == models[j]) { throw std::invalid_argument("a model appears twice in the batch"); }
        }
    }
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<HostModel*> queued;
    std::vector<HostModel*> alone;
    for (HostModel* m : models) { (opt.device_queue != 0 && m->precision() == 0 && !m->steady_stop() ? queued : alone).push_back(m); }
    BatchResult r;
    r.phonon_steps = run_queued(queued, opt) + run_each(alone, opt);
    r.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return r;
}

BatchOptions autotune_batch(const std::vector<HostModel*>& models, int sample, double* best_rate) {
    if (models.empty()) { throw std::invalid_argument("empty batch"); }
    const std::size_t k = std::min<std::size_t>(models.size(), static_cast<std::size_t>(std::max(1, sample)));
    const std::vector<HostModel*> pilot(models.begin(), models.begin() + static_cast<std::ptrdiff_t>(k));
    // The batched launches gain with the number of models they spread over the multiprocessors,
    // and a few models favour small work items that a large batch does not need: they are timed
    // on up to four times the pilot's models, against the best worker-thread options of the pilot.
    const std::size_t k2 = std::min<std::size_t>(models.size(), 4U * k);
    const std::vector<HostModel*> wider(models.begin(), models.begin() + static_cast<std::ptrdiff_t>(k2));
    const int sms = gpu::sm_count();
    auto rate_of = [](const std::vector<HostModel*>& ms, const BatchOptions& o) {
        const BatchResult r = run_batch(ms, o);
        return r.seconds > 0. ? static_cast<double>(r.phonon_steps) / r.seconds : 0.;
    };
    BatchOptions best_alone;
    double alone_r = -1.;
    for (const int workers : { 4, 8, 16, 32 }) {// every model on its own
        for (const int div : { 8, 4, 2, 1 }) {
            BatchOptions o;
            o.workers = workers;
            o.device_queue = 0;
            o.max_blocks = std::max(1, sms / div);
            const double rate = rate_of(pilot, o);
            if (rate > alone_r) {
                alone_r = rate;
                best_alone = o;
            }
        }
    }
    if (k2 > k) { alone_r = rate_of(wider, best_alone); }
    BatchOptions best_queue;
    double queue_r = -1.;
    for (const int per_thread : { 4, 8, 16, 32 }) {// batched launches
        BatchOptions o;
        o.workers = 16;
        o.device_queue = 1;
        o.per_thread = per_thread;
        const double rate = rate_of(wider, o);
        if (rate > queue_r) {
            queue_r = rate;
            best_queue = o;
        }
    }
    if (best_rate != nullptr) { *best_rate = std::max(queue_r, alone_r); }
    return queue_r >= alone_r ? best_queue : best_alone;
}

}// namespace psim
