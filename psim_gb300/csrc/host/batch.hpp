// Many independent models on one GPU (the batched workload: uneven cell and phonon counts).
//
// psim runs one model per process.  Here the FP32 models of a batch that have the same number of
// steps run their transport together: one CUDA graph of batched launches, each covering the same
// window of steps for every model, whose persistent blocks take runs of one model's phonons from
// a device work queue and stage that model's tables in shared memory (gpu::Engine::run_batched).
// Worker threads prepare the runs (tables, phonon builders) and interpret them afterwards.  Models
// that cannot share launches (FP64, a steady-state stop, tables beyond the kernel's shared
// memory) run on the worker threads instead, each with its own CUDA stream and its launches
// limited to `max_blocks` blocks.  A model's results do not depend on the batch, the stream or
// the grid: a phonon's random stream is keyed by (seed, step, id) and tallies are exact sums.
#pragma once

#include <cstdint>
#include <vector>

namespace psim {

class HostModel;

struct BatchOptions {
    int workers{ 8 };       // host threads, one CUDA stream each
    int max_blocks{ 0 };    // thread blocks per transport launch of a model run on its own (0: one per multiprocessor)
    int device_queue{ 1 };  // 1: batched launches fed by a device work queue where models allow; 0: every model on its own
    int per_thread{ 16 };   // batched launches: phonons per thread in one work item
};

struct BatchResult {
    double seconds{ 0. };            // wall time of the batch
    std::uint64_t phonon_steps{ 0 }; // over every model's run
};

// Runs every model once (Model::runSimulation with each model's own seed and precision).
// Throws the first failure after every worker has stopped.
BatchResult run_batch(const std::vector<HostModel*>& models, const BatchOptions& opt);

// The autotuner: models on their own under workers {4, 8, 16, 32} x blocks per launch {1/8, 1/4,
// 1/2, 1} of the multiprocessors, timed on the batch's first `sample` models (full runs), the
// fastest of them again on up to 4 x `sample` models; batched launches with 4, 8, 16 or 32 phonons
// per thread in a work item, timed on those 4 x `sample` models.  Returns the fastest, by
// phonon-steps per second.
BatchOptions autotune_batch(const std::vector<HostModel*>& models, int sample, double* best_rate);

}// namespace psim
