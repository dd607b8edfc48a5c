/*
 * psim_gb300 C ABI: the GPU phonon-simulation phase of psim behind plain C calls.
 *
 * All functions return a status code (PSIM_OK = 0) and never throw; the message
 * for the last failure on the calling thread is available from psim_last_error().
 * Handles are not reentrant: use one handle per host thread.  Device memory is
 * owned by the handle that allocated it.  There is no CPU fallback: when the CUDA
 * device is missing every call that needs it fails with PSIM_ERR_CUDA.
 *
 * Reference interfaces replaced (paths relative to the psim project):
 *   psim_model_*   InputManager::deserialize (psim/include/psim/inputManager.h:17) and
 *                  Model::runSimulation / Model::exportResults (psim/include/psim/model.h:109-110),
 *                  i.e. what the CLI does for one input file (psim/src/main.cpp:10-31).
 *   psim_sim_*     ModelSimulator (psim/include/psim/modelSimulator.h:12-41): the
 *                  phonon step loop that Model drives (psim/src/model.cpp:160-161).
 *   psim_interpret SensorInterpreter::scaleHeatParams / getFinalTemp
 *                  (psim/include/psim/sensorInterpreter.h:17-20).
 *   psim_geom_*    Geometry::Line::getIntersection, Line::contains(Point),
 *                  Triangle::contains(Point) (psim/include/psim/geometry.h:44-75)
 *                  evaluated by the GPU in FP64.
 */
#ifndef PSIM_GB300_H
#define PSIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PSIM_OK 0
#define PSIM_ERR_INVALID 1 /* invalid input (model, sizes, arguments) */
#define PSIM_ERR_CUDA 2    /* CUDA error or no device */
#define PSIM_ERR_IO 3      /* file could not be read or written */
#define PSIM_ERR_LIMIT 4   /* a device-side bound was exceeded (reported, run aborted) */

/* Arithmetic of the phonon transport kernels. */
#define PSIM_PRECISION_FP32 0 /* FP32 cell-local drift/intersection/sampling */
#define PSIM_PRECISION_FP64 1 /* FP64 with the reference's segment-intersection geometry */

/* Material table layout: NUM_FREQ_BINS bins (psim/include/psim/material.h:14). */
#define PSIM_NUM_FREQ_BINS 1000

const char* psim_last_error(void);
/* Library version string. */
const char* psim_version(void);
/* Number of visible CUDA devices (0 when none); never fails. */
int psim_device_count(void);

/* ------------------------------------------------------------------------------------------
 * Model level: one psim JSON input file, run on the GPU, results in psim's output format.
 * ------------------------------------------------------------------------------------------ */
typedef struct psim_model psim_model;

typedef struct psim_run_counters {
    uint64_t phonons;        /* phonons created in the last run (cell origin + emitted) */
    uint64_t phonon_steps;   /* phonons alive at a measurement boundary, summed over boundaries */
    uint64_t kernel_launches;/* kernels launched by the last run */
    double eff_energy;       /* energy per phonon used to scale the last run's results */
    double seconds;          /* wall time of Model::runSimulation's equivalent, last call */
    double kernel_ms;        /* device time of the phonon transport kernels, last run */
    uint64_t max_population; /* largest number of phonons in flight at one step */
    uint64_t limit_hits;     /* phonons relocated by the 100-collision rule */
    uint64_t event_limit_hits; /* phonon-steps cut short by the per-step event bound (numerical corner cases) */
    uint64_t h2d_bytes;      /* host-to-device bytes copied by the last run */
    uint64_t d2h_bytes;      /* device-to-host bytes copied by the last run and its read-outs */
    uint64_t transport_launches; /* launches of the phonon transport kernel (an FP32 launch covers several steps) */
    uint64_t steps_per_launch;   /* measurement steps per transport launch in the last run (FP64: 1) */
    uint64_t backscatters;       /* phonons sent back at an interface between two materials because their
                                    frequency exceeds the other material's branch maximum (last run) */
    uint64_t state_bytes;        /* device bytes of the phonon state buffers the last run used */
} psim_run_counters;

/* InputManager::deserialize (psim/src/inputManager.cpp:14-115): reads and validates the model
 * (cell overlap checks, transition surfaces, emitting-surface placement).  Fails with
 * PSIM_ERR_IO / PSIM_ERR_INVALID and a message on bad input. */
int psim_model_load_json(const char* json_path, psim_model** out);
/* Seed of the counter-based random streams, kernel precision (PSIM_PRECISION_*), and
 * the CUDA stream (cudaStream_t; NULL for the handle's own stream) used by later runs. */
int psim_model_set_options(psim_model* m, uint64_t seed, int32_t precision, void* cuda_stream);
/* Model::runSimulation (psim/src/model.cpp:141-182): every run of the model on the GPU,
 * including the per-run energy rescaling the reference applies after its stability check. */
int psim_model_run(psim_model* m);
/* Sizes: sensors, recorded steps per sensor, cells, measurement steps, runs. */
int psim_model_shape(const psim_model* m, int64_t* n_sensors, int64_t* n_recorded, int64_t* n_cells,
                     int64_t* n_steps, int64_t* n_runs);
/* Per-sensor results averaged over runs (OutputManager::calculateAverages,
 * psim/src/outputManager.cpp:40-70): stats[S][6] = T, SE(T), fx, SE(fx), fy, SE(fy). */
int psim_model_measurements(const psim_model* m, double* stats);
/* Per-step series of one run: temps[S][K] and fluxes[S][K][2] (SensorMeasurements::final_*). */
int psim_model_series(const psim_model* m, int64_t run, double* temps, double* fluxes);
/* OutputManager::addMeasurement for every sensor of `runs` runs (psim/src/outputManager.cpp:116-118):
 * replaces the model's per-run results with statistics made elsewhere, stats[runs][S][6] (T, SE,
 * flux x, SE, flux y, SE per sensor), for example runs combined from several processes.
 * psim_model_measurements and psim_model_export then report them; they carry no per-step series,
 * so a periodic export of them fails with PSIM_ERR_INVALID. */
int psim_model_set_measurements(psim_model* m, const double* stats, int64_t runs);
/* Raw tallies of the last run: energy[S][K] (sum of phonon signs) and flux[S][K][2]
 * (sum of sign * velocity, m/s) as Sensor::inc_energy_ / inc_flux_ (psim/src/sensor.cpp:43-52). */
int psim_model_tallies(const psim_model* m, int64_t* energy, double* flux);
int psim_model_counters(const psim_model* m, psim_run_counters* out);
/* Phonons in flight (alive plus newly born) at each measurement step of the last run: out[n_steps]. */
int psim_model_population(const psim_model* m, uint32_t* out);
/* Forward declarations of the seam descriptions (defined below). */
struct psim_sim_desc;
struct psim_interp_desc;
/* The flattened model this file describes, as handed to the simulator seam: arrays point into
 * the model and stay valid until psim_model_destroy.  Host only (no GPU needed). */
int psim_model_sim_desc(const psim_model* m, struct psim_sim_desc* out);
/* The interpreter description of the model (areas, heat capacities, temperature grid, bounds)
 * with the given energy per phonon (<= 0: the model's initial total energy / num_phonons).
 * Arrays point into the model (valid until the next call on it).  Host only. */
int psim_model_interp_desc(const psim_model* m, double eff_energy, struct psim_interp_desc* out);
/* Warm start (no counterpart in the reference, whose runs start from the JSON's "t_init"): the
 * temperature each sensor starts later runs from, in file order (temps[S]; NULL restores the
 * file's).  It sets the cells' initial phonon energy and the first recorded temperature; the
 * material tables and heat capacities stay at the file's t_init, so a warm run solves the same
 * linearised problem as a cold one and reaches the same steady state.  Deviational models only
 * (t_eq > 0); each temperature positive and finite.  psim_model_start_temps: out[S]. */
int psim_model_start_temps(const psim_model* m, double* out);
int psim_model_set_start_temps(psim_model* m, const double* temps);
/* OutputManager::exportResults (psim/src/outputManager.cpp:13-38): writes ss_<name>.txt or
 * per_<name>.txt next to json_path with the given time in the header. */
int psim_model_export(const psim_model* m, const char* json_path, double seconds);
void psim_model_destroy(psim_model* m);

/* ------------------------------------------------------------------------------------------
 * The warm-start surrogate: a multilayer perceptron on the GPU (no counterpart in the
 * reference).  widths[0] inputs, widths[1..n-2] GELU hidden layers, widths[n-1] linear outputs;
 * BF16 parameters and activations, FP32 accumulation, mean-squared-error loss, Adam (beta 0.9 /
 * 0.999) on FP32 master weights.  Parameters are laid out per layer as W[in][out] then b[out].
 * Rows are float32 x[n][in], y[n][out].
 * ------------------------------------------------------------------------------------------ */
typedef struct psim_mlp psim_mlp;
int psim_mlp_create(const int32_t* widths, int32_t n_widths, uint64_t seed, psim_mlp** out);
int psim_mlp_n_params(const psim_mlp* net, uint64_t* n);
int psim_mlp_get_params(const psim_mlp* net, float* out);
int psim_mlp_set_params(psim_mlp* net, const float* in);
/* Loss over the n rows and its gradient for every parameter (grads may be NULL). */
int psim_mlp_gradients(psim_mlp* net, const float* x, const float* y, int32_t n, float* loss, float* grads);
/* Adam over shuffled whole batches for `epochs` passes; final_loss (may be NULL): the last
 * epoch's mean batch loss. */
int psim_mlp_train(psim_mlp* net, const float* x, const float* y, int32_t n, int32_t batch, int32_t epochs, float lr,
                   uint64_t seed, float* final_loss);
int psim_mlp_predict(psim_mlp* net, const float* x, int32_t n, float* y);
void psim_mlp_destroy(psim_mlp* net);

/* ------------------------------------------------------------------------------------------
 * Many independent models on one GPU.  No counterpart in the reference, which runs one model
 * per process (psim/src/main.cpp:10-31 loops over its input files).  Each model runs as
 * psim_model_run would (its own seed, precision and steady-state stop).  With device_queue set,
 * the FP32 models of the batch that have the same number of steps share their transport: one
 * CUDA graph of batched launches, each covering one window of steps for every model, whose
 * persistent thread blocks take runs of `per_thread` x 1024 phonons of one model at a time from
 * a device work queue and stage that model's tables in shared memory.  Worker threads prepare
 * and interpret the runs.  The other models (FP64, a steady-state stop, tables beyond the
 * kernel's shared memory, or device_queue 0) run on `workers` host threads, each with its own
 * CUDA stream, their transport launches limited to `max_blocks` thread blocks.  A model's
 * results do not depend on the batch it ran in.
 * ------------------------------------------------------------------------------------------ */
typedef struct psim_batch_options {
    int32_t workers;      /* host threads (>= 1) */
    int32_t max_blocks;   /* thread blocks per transport launch of a model run on its own (0: one per multiprocessor) */
    int32_t device_queue; /* 1: batched launches fed by a device work queue where the models allow */
    int32_t per_thread;   /* batched launches: phonons per thread in one work item (>= 1) */
} psim_batch_options;
/* Runs every model once; fails with the first model's failure after the others stopped.
 * seconds (may be NULL): wall time; phonon_steps (may be NULL): over all models. */
int psim_batch_run(psim_model* const* models, int32_t n, const psim_batch_options* opt, double* seconds,
                   uint64_t* phonon_steps);
/* The autotuner: models on their own under workers 4, 8, 16, 32 x blocks per launch 1/8, 1/4, 1/2
 * and all of the multiprocessors, timed on the first `sample` models, the fastest of them again on
 * up to 4 x `sample` models; batched launches with 4, 8, 16 or 32 phonons per thread in a work
 * item, timed on those 4 x `sample` models.  Returns the fastest options and their rate
 * (phonon-steps/s; may be NULL). */
int psim_batch_autotune(psim_model* const* models, int32_t n, int32_t sample, psim_batch_options* out,
                        double* best_rate);

/* ------------------------------------------------------------------------------------------
 * Simulator seam: ModelSimulator (psim/include/psim/modelSimulator.h:12-41).
 * The caller keeps ownership of every array in the description; psim_sim_create copies it.
 * Indices are 0-based positions in the caller's arrays.
 * ------------------------------------------------------------------------------------------ */
typedef struct psim_sim psim_sim;

#define PSIM_SUB_TRANSITION 0 /* TransitionSurface: target = neighbour cell */
#define PSIM_SUB_EMIT 1       /* EmitSurface: target = emitter */

#define PSIM_SIM_STEADY 0
#define PSIM_SIM_PERIODIC 1
#define PSIM_SIM_TRANSIENT 2

typedef struct psim_sim_desc {
    /* ModelSimulator(measurement_steps, simulation_time, phasor_sim) */
    uint64_t measurement_steps;
    double simulation_time; /* ns */
    int32_t phasor_sim;
    int32_t sim_type;          /* PSIM_SIM_*; selects which steps are tallied */
    uint64_t step_adjustment;  /* ModelSimulator::setStepAdjustment */
    uint64_t recorded_steps;   /* tally slots per sensor (Sensor::inc_energy_.size()) */
    int32_t full_simulation;   /* Material::setFullSimulation: bin-centre frequencies (t_eq == 0) */

    /* Materials (Material, psim/include/psim/material.h) */
    uint32_t n_materials;
    const double* mat_freq;    /* [n_materials][1000] bin centres, rad/s */
    const double* mat_vel;     /* [n_materials][2][1000] LA then TA group velocity, m/s */
    const double* mat_params;  /* [n_materials][8]: b_l b_tn b_tu b_i w freq_width w_max_la w_max_ta */

    /* Cumulative tables (Material::Table): [n_tables][1000][2] = (cumulative probability, LA fraction) */
    uint32_t n_tables;
    const double* tables;

    /* Sensors (Sensor / SensorController) */
    uint32_t n_sensors;
    const uint32_t* sensor_material;      /* [n_sensors] */
    const double* sensor_temp;            /* [n_sensors] temperature for scattering rates (getSteadyTemp) */
    const uint32_t* sensor_base_table;    /* [n_sensors] table for cell-origin phonons */
    const uint32_t* sensor_scatter_table; /* [n_sensors] table for scattering resamples */

    /* Cells (Cell): triangle p1 p2 p3; edges 0,1,2 = p1p2, p2p3, p3p1 */
    uint32_t n_cells;
    const double* cell_vertices; /* [n_cells][6] nm */
    const uint32_t* cell_sensor; /* [n_cells] */
    const double* cell_spec;     /* [n_cells] specularity of the cell's boundary surfaces, in [0,1] */
    /* Sub-surfaces of each edge in CompositeSurface order (transition surfaces first, then
     * emitting surfaces): edge e of cell c owns subs [edge_sub_begin[3c+e], edge_sub_begin[3c+e+1]). */
    const uint32_t* edge_sub_begin; /* [n_cells*3+1] */
    uint32_t n_subs;
    const int32_t* sub_kind;    /* [n_subs] PSIM_SUB_* */
    const uint32_t* sub_target; /* [n_subs] neighbour cell or emitter index */
    const double* sub_line;     /* [n_subs][4] x1 y1 x2 y2 of the sub-surface line */

    /* Emitting surfaces (EmitSurface) */
    uint32_t n_emitters;
    const uint32_t* emit_cell;   /* [n_emitters] owning cell */
    const uint32_t* emit_edge;   /* [n_emitters] edge of the owning cell (0..2) */
    const double* emit_line;     /* [n_emitters][4] */
    const double* emit_temp;     /* [n_emitters] K */
    const double* emit_start;    /* [n_emitters] ns */
    const double* emit_duration; /* [n_emitters] ns */
    const uint32_t* emit_table;  /* [n_emitters] emit table index */
} psim_sim_desc;

int psim_sim_create(const psim_sim_desc* desc, psim_sim** out);
/* ModelSimulator::initPhononBuilders (psim/src/modelSimulator.cpp:43-85): phonon counts
 * floor(E/eff_energy) + Bernoulli(frac) for each cell's initial energy and each emitter's
 * energy (both supplied by the caller, Cell::getInitEnergy and the emitter energy
 * formula), drawn from seed.  sensor_init_temp[S] (Sensor::getInitTemp) sets the sign of
 * cell-origin phonons.  Returns the total through total_phonons (may be NULL). */
int psim_sim_init_phonon_builders(psim_sim* s, double t_eq, double eff_energy, const double* cell_energy,
                                  const double* emit_energy, const double* sensor_init_temp, uint64_t seed,
                                  uint64_t* total_phonons);
/* ModelSimulator::runSimulation: all measurement steps on the GPU.  Tallies accumulate
 * into the handle (cleared by psim_sim_reset). */
int psim_sim_run(psim_sim* s, double t_eq, int32_t precision, void* cuda_stream);
/* ModelSimulator::reset plus the tally reset of Sensor::reset. */
int psim_sim_reset(psim_sim* s);
/* ModelSimulator::setStepAdjustment */
int psim_sim_set_step_adjustment(psim_sim* s, uint64_t step_adjustment);
/* energy[S][K] and flux[S][K][2] as in psim_model_tallies. */
int psim_sim_tallies(const psim_sim* s, int64_t* energy, double* flux);
int psim_sim_counters(const psim_sim* s, psim_run_counters* out);
/* Phonons in flight at each measurement step of the last run: out[measurement_steps]. */
int psim_sim_population(const psim_sim* s, uint32_t* out);
void psim_sim_destroy(psim_sim* s);

/* ------------------------------------------------------------------------------------------
 * SensorInterpreter (psim/src/sensorInterpreter.cpp) on the GPU in FP64.
 * ------------------------------------------------------------------------------------------ */
typedef struct psim_interp_desc {
    uint32_t n_sensors;
    uint64_t recorded_steps;    /* K */
    double t_eq;                /* 0 = full simulation (bisection), else deviational */
    double eff_energy;
    double lower_bound, upper_bound; /* SensorInterpreter::setBounds */
    const double* sensor_area;  /* [S] */
    const double* sensor_heat_capacity; /* [S] heat capacity (SensorController::getHeatCapacity; constant over a run) */
    const double* sensor_init_temp;     /* [S] value written over the first temperature */
    const uint32_t* sensor_material;    /* [S] */
    /* Tabulated energy per material for the full-simulation inversion: temperature grid and the
     * base table sums (Material::theoreticalEnergy). */
    uint32_t n_materials;
    const uint64_t* mat_temp_begin; /* [n_materials+1] offsets into temps/energies */
    const double* temps;
    const double* energies;
} psim_interp_desc;

/* scaleHeatParams for every sensor: temps[S][K], fluxes[S][K][2] (may be NULL) and
 * stats[S][6].  energy[S][K] and flux[S][K][2] are raw tallies. */
int psim_interpret(const psim_interp_desc* d, const int64_t* energy, const double* flux, double* temps,
                   double* fluxes, double* stats);
/* getFinalTemp(sensor, start_step) for every sensor: out[S]. */
int psim_final_temps(const psim_interp_desc* d, const int64_t* energy, uint64_t start_step, double* out);

/* ------------------------------------------------------------------------------------------
 * Steady-state detection.  No counterpart in the reference: psim runs for the time the user
 * gives, and its README (Steady-State Detection) proposes stopping once each cell's flux stays
 * constant within a margin for some time.  The criterion here: each sensor's per-step energy
 * count and flux components are cut into windows of `window` steps, each window into `batches`
 * equal batches; a window's standard error is the spread of its batch means over sqrt(batches)
 * (per-step tallies are correlated: a phonon stays in a sensor's cells for several steps); a
 * window agrees with an anchor window when every mean differs by at most z combined standard
 * errors; a sensor is steady from window j when the `patience` windows after j all agree with
 * window j (a window that disagrees becomes the next anchor) and, with drift_z > 0, the least-
 * squares slope of each quantity's means over those patience + 1 windows lies within drift_z of
 * its standard error (a slope beyond it also makes the latest window the anchor); the onset is
 * the largest over the sensors, in steps (-1: not steady).  Evaluated by a GPU kernel on the
 * exact integer tallies.  window must be a multiple of batches, batches >= 2, z > 0,
 * patience >= 1, drift_z >= 0 (PSIM_ERR_INVALID otherwise).
 * ------------------------------------------------------------------------------------------ */
/* On raw tallies energy[S][K] and flux[S][K][2] (as psim_sim_tallies returns them); flux is taken
 * at 2^-20 m/s resolution.  per_sensor[S] may be NULL. */
int psim_steady_state(const int64_t* energy, const double* flux, uint32_t n_sensors, uint64_t recorded_steps,
                      uint32_t window, uint32_t batches, double z, uint32_t patience, double drift_z,
                      int64_t* onset_step, int64_t* per_sensor);
/* On the recorded steps of the simulator's / model's last run (its tallies stay on the GPU). */
int psim_sim_steady_state(const psim_sim* s, uint32_t window, uint32_t batches, double z, uint32_t patience,
                          double drift_z, int64_t* onset_step, int64_t* per_sensor);
int psim_model_steady_state(const psim_model* m, uint32_t window, uint32_t batches, double z, uint32_t patience,
                            double drift_z, int64_t* onset_step, int64_t* per_sensor);
/* Stop later runs once their recorded steps are steady by the criterion above, checked every
 * check_every steps (0: every (patience + 1) x window steps) between launches; enable = 0 turns
 * it off.  Only for runs that record every step: a single-run periodic or transient model, or a
 * simulator whose step adjustment is 0 (a run fails with PSIM_ERR_INVALID otherwise).  The
 * results of a stopped run cover the steps it simulated: psim_model_shape reports them as the
 * recorded steps, and psim_model_series / psim_model_tallies return that many. */
int psim_model_set_steady_stop(psim_model* m, int32_t enable, uint32_t window, uint32_t batches, double z,
                               uint32_t patience, double drift_z, uint64_t check_every);
int psim_sim_set_steady_stop(psim_sim* s, int32_t enable, uint32_t window, uint32_t batches, double z,
                             uint32_t patience, double drift_z, uint64_t check_every);
/* Measurement steps the last run simulated. */
int psim_model_steps_run(const psim_model* m, uint64_t* steps);
int psim_sim_steps_run(const psim_sim* s, uint64_t* steps);

/* psim_final_temps without any allocation.  This has no counterpart in the reference.
 * It is for hosts that must not allocate device memory inside a call: a host that keeps
 * all device memory in its own pool, or that runs under a hard device-memory quota.
 *
 * energy_dev[S][K] (raw tallies) and out_dev[S] are DEVICE pointers owned by the caller; the
 * work is enqueued on cuda_stream (a cudaStream_t of the current device, NULL = legacy default
 * stream) and the call returns without waiting for it.  The descriptor's host arrays are copied
 * to the device with cudaMemcpyAsync: from pageable memory they may be reused once the call
 * returns, from pinned memory only once the stream has passed the call.  Results equal
 * psim_final_temps on the same tallies.
 *
 * Limit: the tables plus the per-step temperatures (S x (K - start_step) x 8 bytes, each part
 * rounded up to 256 bytes) must fit in one fixed device scratch of
 * psim_final_temps_noalloc_max_bytes() bytes (8 MiB); larger inputs fail with PSIM_ERR_LIMIT
 * before anything is enqueued.  The scratch is one per device and per process: calls whose GPU
 * work overlaps (different streams, or several host threads) race on it and give wrong results;
 * order them on one stream or with events.  The first call on each device looks up the
 * scratch's address (and may load the module onto that device): make it before any stream
 * capture.  Whether the call can be captured in a CUDA graph is not covered here.  The address is
 * kept per device ordinal for the life of the process, so hosts that reset a device
 * (cudaDeviceReset) or run in a context other than the device's primary one are not supported. */
int psim_final_temps_noalloc(const psim_interp_desc* d, const int64_t* energy_dev, uint64_t start_step,
                             double* out_dev, void* cuda_stream);
/* Size in bytes of the fixed scratch behind psim_final_temps_noalloc. */
uint64_t psim_final_temps_noalloc_max_bytes(void);

/* ------------------------------------------------------------------------------------------
 * FP64 geometry on the GPU, bit-exact with the reference routines.
 * ------------------------------------------------------------------------------------------ */
/* Line(a).getIntersection(Line(b)) for n segment pairs a[n][4], b[n][4]:
 * has[n] = 1 with poi[n][2], 0 for none, -1 when a segment is degenerate (LineError). */
int psim_geom_intersect(int64_t n, const double* a, const double* b, double* poi, int32_t* has);
/* Line(lines[i]).contains(pts[i]) -> out[i] in {0,1}; -1 for a degenerate line. */
int psim_geom_on_line(int64_t n, const double* lines, const double* pts, int32_t* out);
/* Triangle(tris[i]).contains(pts[i]) -> out[i] in {0,1}. */
int psim_geom_tri_contains(int64_t n, const double* tris, const double* pts, int32_t* out);
/* Cell::handleSurfaceCollision edge choice: index (0..2) of the first edge of tris[i] whose line
 * contains pts[i], or -1. */
int psim_geom_edge_index(int64_t n, const double* tris, const double* pts, int32_t* out);

/* ------------------------------------------------------------------------------------------
 * Scattering rates on the GPU, for checks.
 * ------------------------------------------------------------------------------------------ */
/* Material::relaxRates(temp, freq, polarization) (psim/src/material.cpp:54-62,207-239) as the
 * transport kernels evaluate it: out[n][3] = normal, Umklapp and impurity rates (1/s) of one
 * material for the cases (T[i] K, freq[i] rad/s, pol[i] 0 LA / 1 TA).  mat_params holds the
 * material as psim_sim_desc.mat_params does: b_l, b_tn, b_tu, b_i, w, bin width, w_max LA,
 * w_max TA.  precision PSIM_PRECISION_FP32 takes the FP32 kernel's rate function (frequency
 * rounded to float in units of 1e13 rad/s, temperature factors rounded to float as each
 * sensor's are), PSIM_PRECISION_FP64 the FP64 kernel's.  At most 2^24 cases per call. */
int psim_rates(const double* mat_params, int64_t n, const double* T, const double* freq, const int32_t* pol,
               int precision, double* out);

/* ------------------------------------------------------------------------------------------
 * The frequency sampler, for checks (host only, no GPU needed).
 * ------------------------------------------------------------------------------------------ */
/* Material::freqIndex (psim/src/material.cpp:64-75) draws bin h with the probability
 * cum[h] - cum[h-1] of a cumulative table (bin 1 also takes bin 0's mass, bin 999 the rest
 * above cum[998]) and LA with probability la_frac[h].  The kernels draw the same (bin,
 * polarization) outcomes from the Walker alias table the engine builds from that table;
 * this returns it.  table[1000][2] = (cumulative probability, LA fraction); out[2048], one word
 * per column: acceptance threshold (21 bits) << 11 | alias column.  Outcome 2h is bin h LA,
 * 2h + 1 bin h TA; a 32-bit random word picks column (word >> 21) and keeps it when
 * (word & 0x1FFFFF) is below the threshold, else takes the alias. */
int psim_sampling_alias_table(const double* table, uint32_t* out);

#ifdef __cplusplus
}
#endif

#endif /* PSIM_GB300_H */
