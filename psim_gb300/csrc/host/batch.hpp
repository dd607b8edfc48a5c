// Many independent models on one GPU (the batched workload: uneven cell and phonon counts).
//
// psim runs one model per process.  Here a host work queue hands models to worker threads,
// each with its own non-blocking CUDA stream; every model's run is the usual CUDA graph of
// transport launches on its worker's stream, with its launches limited to `max_blocks` thread
// blocks so that small models occupy a few multiprocessors and several run at once.  A model's
// results do not depend on the stream, the grid or what runs beside it.
#pragma once

#include <cstdint>
#include <vector>

namespace psim {

class HostModel;

struct BatchOptions {
    int workers{ 8 };     // host threads, one CUDA stream each
    int max_blocks{ 0 };  // thread blocks per transport launch (0: one per multiprocessor)
};

struct BatchResult {
    double seconds{ 0. };            // wall time of the batch
    std::uint64_t phonon_steps{ 0 }; // over every model's run
};

// Runs every model once (Model::runSimulation with each model's own seed and precision).
// Throws the first failure after every worker has stopped.
BatchResult run_batch(const std::vector<HostModel*>& models, const BatchOptions& opt);

// The autotuner: times the batch's first `sample` models (full runs) under each candidate of
// workers x blocks per launch and returns the fastest, by phonon-steps per second.
BatchOptions autotune_batch(const std::vector<HostModel*>& models, int sample, double* best_rate);

}// namespace psim
