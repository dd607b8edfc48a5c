#include "batch.hpp"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <exception>
#include <mutex>
#include <stdexcept>
#include <thread>

#include "../device/engine.hpp"
#include "model.hpp"

namespace psim {

BatchResult run_batch(const std::vector<HostModel*>& models, const BatchOptions& opt) {
    if (opt.workers < 1) { throw std::invalid_argument("a batch needs at least one worker"); }
    if (opt.max_blocks < 0) { throw std::invalid_argument("blocks per launch must not be negative"); }
    for (const HostModel* m : models) {
        if (m == nullptr) { throw std::invalid_argument("null model in the batch"); }
    }
    for (std::size_t i = 0; i < models.size(); ++i) {
        for (std::size_t j = i + 1; j < models.size(); ++j) {
            if (models[i] == models[j]) { throw std::invalid_argument("a model appears twice in the batch"); }
        }
    }
    const int workers = std::max(1, std::min<int>(opt.workers, static_cast<int>(models.size())));
    std::atomic<std::size_t> next{ 0 };
    std::atomic<std::uint64_t> steps{ 0 };
    std::mutex err_mu;
    std::exception_ptr first_error;
    std::atomic<bool> failed{ false };
    const auto t0 = std::chrono::steady_clock::now();
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
    BatchResult r;
    r.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    r.phonon_steps = steps.load();
    return r;
}

BatchOptions autotune_batch(const std::vector<HostModel*>& models, int sample, double* best_rate) {
    if (models.empty()) { throw std::invalid_argument("empty batch"); }
    const std::size_t k = std::min<std::size_t>(models.size(), static_cast<std::size_t>(std::max(1, sample)));
    const std::vector<HostModel*> pilot(models.begin(), models.begin() + static_cast<std::ptrdiff_t>(k));
    const int sms = gpu::sm_count();
    BatchOptions best;
    double best_r = -1.;
    for (const int workers : { 4, 8, 16, 32 }) {
        for (const int div : { 8, 4, 2, 1 }) {
            BatchOptions o;
            o.workers = workers;
            o.max_blocks = std::max(1, sms / div);
            const BatchResult r = run_batch(pilot, o);
            const double rate = r.seconds > 0. ? static_cast<double>(r.phonon_steps) / r.seconds : 0.;
            if (rate > best_r) {
                best_r = rate;
                best = o;
            }
        }
    }
    if (best_rate != nullptr) { *best_rate = best_r; }
    return best;
}

}// namespace psim
