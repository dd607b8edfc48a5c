// Host-side interface of the GPU engine (implemented in engine.cu).  No CUDA types
// appear here so plain C++ translation units can use it.
#pragma once

#include <array>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

namespace psim::gpu {

struct StepParams;

constexpr std::uint32_t kMaxMaterialsHost = 16;

// Owning copy of psim_sim_desc (include/psim_gb300.h).
struct SimDesc {
    std::uint64_t steps{ 0 };
    double sim_time{ 0. };
    bool phasor{ false };
    int sim_type{ 0 };
    std::uint64_t step_adj{ 0 };
    std::uint64_t recorded{ 0 };
    bool full{ false };
    std::uint32_t n_materials{ 0 };
    std::vector<double> mat_freq;   // [M][1000]
    std::vector<double> mat_vel;    // [M][2][1000]
    std::vector<double> mat_params; // [M][8]
    std::uint32_t n_tables{ 0 };
    std::vector<double> tables;     // [T][1000][2]
    std::uint32_t n_sensors{ 0 };
    std::vector<std::uint32_t> sensor_material, sensor_base_table, sensor_scatter_table;
    std::vector<double> sensor_temp;
    std::uint32_t n_cells{ 0 };
    std::vector<double> cell_vertices;// [C][6]
    std::vector<std::uint32_t> cell_sensor;
    std::vector<double> cell_spec;
    std::vector<std::uint32_t> edge_sub_begin;// [3C+1]
    std::vector<std::int32_t> sub_kind;
    std::vector<std::uint32_t> sub_target;
    std::vector<double> sub_line;// [n_subs][4]
    std::uint32_t n_emitters{ 0 };
    std::vector<std::uint32_t> emit_cell, emit_edge, emit_table;
    std::vector<double> emit_line, emit_temp, emit_start, emit_duration;
};

struct RunCounters {
    std::uint64_t phonons{ 0 };
    std::uint64_t phonon_steps{ 0 };
    std::uint64_t kernel_launches{ 0 };
    std::uint64_t relocations{ 0 };
    std::uint64_t overflow{ 0 };
    std::uint64_t max_population{ 0 };
    std::uint64_t event_limits{ 0 };
    std::uint64_t h2d_bytes{ 0 };
    std::uint64_t d2h_bytes{ 0 };
    std::uint64_t transport_launches{ 0 };
    std::uint64_t steps_per_launch{ 0 };
    std::uint64_t backscatters{ 0 };
    std::uint64_t state_bytes{ 0 };
    double kernel_ms{ 0. };
};

// Interpreter inputs (SensorInterpreter state plus the per-sensor quantities it reads).
struct InterpDesc {
    std::uint32_t n_sensors{ 0 };
    std::uint64_t recorded{ 0 };
    double t_eq{ 0. };
    double eff_energy{ 0. };
    double lb{ 0. }, ub{ 0. };
    std::vector<double> area, heat_capacity, init_temp;
    std::vector<std::uint32_t> material;
    std::vector<std::uint64_t> mat_temp_begin;// [M+1]
    std::vector<double> temps, energies;
};

// Steady-state criterion over windows of recorded steps (device/steady.cu).
struct SteadyCriterion {
    std::uint32_t window{ 250 }; // steps per window
    std::uint32_t batches{ 5 };  // batch means per window (window is a multiple of it)
    double z{ 3. };              // agreement tolerance in combined standard errors
    std::uint32_t patience{ 3 }; // consecutive agreeing windows
    double drift_z{ 0. };        // trend test over the anchor and its agreeing windows (0: none)
};

class Engine {
public:
    explicit Engine(const SimDesc& desc);
    ~Engine();
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;

    // Phonon counts per cell and emitter (initPhononBuilders) and the birth schedule.
    std::uint64_t init_builders(double t_eq, double eff_energy, const double* cell_energy, const double* emit_energy,
                                const double* sensor_init_temp, std::uint64_t seed);
    // Every measurement step; stream may be null (the engine's own stream).
    void run(int precision, void* stream);
    void reset();
    void set_step_adjustment(std::uint64_t adj) { desc_.step_adj = adj; }
    void set_use_graph(bool on) { use_graph_ = on; }
    void set_grid(int blocks) { grid_override_ = blocks; }
    // Stage cells and tables into shared memory in the FP32 kernel when they fit (default on).
    void set_stage_tables(bool on) { stage_tables_ = on; }
    // FP32 kernel: plain step boundaries are crossed in a warp-uniform loop while at least this
    // many of a warp's 32 lanes cross one (0: every boundary takes the general segment).
    void set_coast_lanes(std::uint32_t lanes) { coast_lanes_ = lanes > 32U ? 32U : lanes; }
    std::uint32_t last_stage_mask() const noexcept { return last_stage_mask_; }
    // Measurement steps per FP32 launch in the last run (1 for FP64).
    std::uint32_t last_fused() const noexcept { return last_fused_; }

    // Phonons in flight at each measurement step of the last run (alive + born), [steps].
    void population(std::uint32_t* out) const;
    // Raw tallies (host) of the first K recorded steps (all of them by default): energy[S][K],
    // flux[S][K][2].
    void tallies(std::int64_t* energy, double* flux, std::uint64_t K = UINT64_MAX) const;
    // Device-resident interpretation of the current tallies.
    void interpret(const InterpDesc& d, double* temps, double* fluxes, double* stats) const;
    void final_temps(const InterpDesc& d, std::uint64_t start, double* out) const;
    // Steady-state onset over the last run's recorded steps (-1: not steady).
    long long steady_onset(const SteadyCriterion& c, long long* per_sensor) const;
    // Stop runs once the recorded steps are steady, checked every check_every steps (rounded up
    // to whole launches; 0 = every patience x window steps).  Needs every step recorded
    // (periodic or transient); run() throws otherwise.
    void set_steady_stop(bool on, const SteadyCriterion& c, std::uint64_t check_every);
    // Measurement steps the last run simulated (all of them unless it stopped at steady state).
    std::uint64_t steps_run() const noexcept { return steps_run_; }

    const RunCounters& counters() const noexcept { return counters_; }
    // bytes copied host->device when the model was created (geometry, tables, materials)
    std::uint64_t model_bytes() const noexcept { return model_bytes_; }
    void add_h2d(std::uint64_t bytes) const noexcept { counters_.h2d_bytes += bytes; }
    const SimDesc& desc() const noexcept { return desc_; }
    void* stream() const noexcept { return stream_; }

    // Runs the transport of every engine's prepared run (init_builders done) in one sequence of
    // batched launches on `stream`: each launch covers the same window of steps for every model,
    // and its blocks take runs of one model's phonons from a device work queue (FP32 kernel,
    // `per_thread` phonons per thread in a work item).  Returns false, having run nothing, when the
    // engines cannot share launches (different step counts, a steady-state stop, or a model whose
    // tables and tallies do not fit the batched kernel's shared memory).  Each engine's run then
    // finishes as after run(): its counters hold its own phonon-steps, and kernel_ms the batch's
    // device time split by phonon-steps.
    static bool run_batched(const std::vector<Engine*>& engines, void* stream, std::uint32_t per_thread = 16);

private:
    void ensure_capacity(std::uint64_t need, std::uint64_t live_front, std::uint64_t live_back, int cur, std::size_t rec_bytes,
                         bool grow_ahead, void* stream);
    void base_params(StepParams& P) const;
    void window_params(StepParams& P, std::uint64_t w, std::uint64_t s0, std::uint32_t tw) const;
    std::uint32_t window_steps(std::uint64_t s0, std::uint32_t cap, std::uint64_t capacity) const;
    void finish_run(double ms, std::uint64_t launches, std::uint64_t transport_launches, std::uint32_t fused);

    struct Impl;
    SimDesc desc_;
    std::unique_ptr<Impl> impl_;
    void* stream_{ nullptr };
    mutable RunCounters counters_;
    std::uint64_t model_bytes_{ 0 };
    bool use_graph_{ true };
    bool stage_tables_{ true };
    std::uint32_t coast_lanes_{ 0 };
    std::uint32_t last_stage_mask_{ 0 };
    std::uint32_t last_fused_{ 1 };
    bool stop_on_{ false };
    SteadyCriterion stop_crit_{};
    std::uint64_t stop_check_{ 0 };
    std::uint64_t steps_run_{ 0 };
    int grid_override_{ 0 };
};

void validate_steady(const SteadyCriterion& c);
// Onset step of steady state over the first k_used recorded steps of device tallies [K][S]
// (TallySlot records), or -1; per_sensor[S] (may be null) gets each sensor's onset.
long long steady_onset_device(const void* tally, std::uint32_t S, std::uint64_t k_used, const SteadyCriterion& c,
                              long long* per_sensor, void* stream);
// The same on host tallies energy[S][K], flux[S][K][2].
long long steady_onset_host(const std::int64_t* energy, const double* flux, std::uint32_t S, std::uint64_t K,
                            const SteadyCriterion& c, long long* per_sensor);

// Device buffers an engine keeps for its interpretations (device/interpret.cu).
struct InterpCache;
InterpCache* interp_cache_create();
void interp_cache_destroy(InterpCache* c) noexcept;

// Stand-alone interpreter on host arrays (psim_interpret / psim_final_temps).
void interpret_host(const InterpDesc& d, const std::int64_t* energy, const double* flux, double* temps, double* fluxes,
                    double* stats);
void final_temps_host(const InterpDesc& d, const std::int64_t* energy, std::uint64_t start, double* out);

// Interpreter inputs as the caller's own host arrays, for the call that allocates nothing.
struct InterpView {
    std::uint32_t n_sensors{ 0 };
    std::uint64_t recorded{ 0 };
    double t_eq{ 0. }, eff_energy{ 0. }, lb{ 0. }, ub{ 0. };
    const double* area{ nullptr };
    const double* heat_capacity{ nullptr };
    const std::uint32_t* material{ nullptr };
    std::uint32_t n_materials{ 0 };
    const std::uint64_t* mat_temp_begin{ nullptr };// [n_materials + 1]
    const double* temps{ nullptr };
    const double* energies{ nullptr };
};

// Size of the fixed device scratch behind final_temps_noalloc.
constexpr std::size_t kFinalTempsScratchBytes = std::size_t{ 8 } << 20;
// Scratch bytes final_temps_noalloc needs for these inputs (tables plus S x (K - start) doubles).
std::size_t final_temps_scratch_bytes(const InterpView& d, std::uint64_t start);
// getFinalTemp for every sensor with device-resident tallies energy_dev[S][K] and result
// out_dev[S], enqueued on `stream` (a cudaStream_t; NULL = legacy default stream).  Uses the
// module's static scratch instead of allocating; throws std::length_error past its size.
void final_temps_noalloc(const InterpView& d, const std::int64_t* energy_dev, std::uint64_t start, double* out_dev,
                         void* stream);

// FP64 geometry kernels (bit-exact with the reference routines).
void geom_intersect(std::int64_t n, const double* a, const double* b, double* poi, std::int32_t* has);
void geom_on_line(std::int64_t n, const double* lines, const double* pts, std::int32_t* out);
void geom_tri_contains(std::int64_t n, const double* tris, const double* pts, std::int32_t* out);
void geom_edge_index(std::int64_t n, const double* tris, const double* pts, std::int32_t* out);

// Device material record from (b_l, b_tn, b_tu, b_i, w, bin width, w_max LA, w_max TA), and a
// sensor's FP32 rate factors of its temperature T (T^3, T^4, hbar 1e13 / (k T)).
struct MaterialDev;
struct SensorDev;
MaterialDev material_dev(const double* params);
void sensor_rate_factors(double T, SensorDev& sd);
// Material::relaxRates on the GPU for n cases (T[i], f[i] rad/s, pol[i] 0 LA / 1 TA) of one
// material: out[n][3] = N, U, I rates (1/s) from the FP32 (precision 0) or FP64 kernel's rates.
void rates_probe(const double* mat_params, std::int64_t n, const double* T, const double* f, const std::int32_t* pol,
                 int precision, double* out);

// The Walker alias table the engine uploads for one cumulative table (tab[1000][2]): 2048 words.
std::vector<std::uint32_t> alias_table_of(const double* tab);

int device_count() noexcept;
// A non-blocking CUDA stream of the current device (as void*), and its release.
void* create_stream();
void destroy_stream(void* stream) noexcept;
// Multiprocessors of the current device.
int sm_count();

}// namespace psim::gpu
