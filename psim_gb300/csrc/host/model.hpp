// Host-side psim model: JSON input, model assembly and validation, run orchestration
// around the GPU engine, and the ss_/per_ output tables.
//
// This mirrors the reference's InputManager (psim/src/inputManager.cpp), Model
// (psim/src/model.cpp), Cell/CompositeSurface assembly (psim/src/cell.cpp,
// psim/src/compositeSurface.cpp) and OutputManager (psim/src/outputManager.cpp).
#pragma once

#include <array>
#include <chrono>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "../device/engine.hpp"
#include "geom64.hpp"
#include "material.hpp"

namespace psim {

enum class SimType { SteadyState = 0, Periodic = 1, Transient = 2 };

struct SubSurface {// TransitionSurface or EmitSurface placed on a cell edge
    int kind{ 0 };   // 0 transition, 1 emit
    std::uint32_t target{ 0 };// neighbour cell or emitter
    Seg64 line{};
    double length{ 0. };
};

struct EdgeRec {// CompositeSurface
    Seg64 main{};
    double length{ 0. };
    std::vector<SubSurface> trans;
    std::vector<SubSurface> emits;
};

struct CellRec {
    P2 v[3]{};
    std::uint32_t sensor{ 0 };
    double spec{ 0. };
    double area{ 0. };
    int nsign{ 1 };
    std::array<EdgeRec, 3> edge{};
    P2 lo{}, hi{};// bounding box
};

struct SensorRec {
    std::uint64_t id{ 0 };
    std::uint32_t material{ 0 };
    double t_init{ 0. };
    double t_steady{ 0. };
    double area{ 0. };
    double heat_cap{ 0. };
    std::size_t temp_index{ 0 };
};

struct EmitterRec {
    std::uint32_t cell{ 0 }, edge{ 0 };
    Seg64 line{};
    double length{ 0. };
    double temp{ 0. }, duration{ 0. }, start{ 0. };
};

struct Measurement {// SensorMeasurements (psim/include/psim/sensor.h:59-71)
    std::uint64_t id{ 0 };
    std::array<double, 6> stats{};
    std::vector<double> temps;
    std::vector<double> fluxes;// [K][2]
};

class HostModel {
public:
    static std::unique_ptr<HostModel> from_json(const std::string& path);
    ~HostModel();

    void set_options(std::uint64_t seed, int precision, void* stream) {
        seed_ = seed;
        precision_ = precision;
        stream_ = stream;
    }
    void set_stream(void* stream) noexcept { stream_ = stream; }
    void* stream() const noexcept { return stream_; }
    // Thread blocks per transport launch (0: one per multiprocessor, the default).
    void set_grid(int blocks) noexcept { grid_ = blocks; }
    int grid() const noexcept { return grid_; }
    // Stop each run once its recorded steps are steady (single-run periodic or transient models).
    void set_steady_stop(bool on, const gpu::SteadyCriterion& c, std::uint64_t check_every) {
        if (on) { gpu::validate_steady(c); }
        stop_on_ = on;
        stop_crit_ = c;
        stop_check_ = check_every;
    }
    // Warm start (deviational models): the temperatures runs start from, per sensor in file
    // order (an empty list restores the file's).  They set the cells' initial phonon energy and the first recorded
    // temperature; the material tables and heat capacities stay at the file's t_init, so a warm
    // run solves the same linearised problem as a cold one and reaches the same steady state.
    void set_start_temps(const std::vector<double>& temps);
    std::vector<double> start_temps() const;
    void run();// Model::runSimulation
    // run() in parts, for transports run elsewhere (a batch): begin_runs(), then per run r
    // prepare_run(r) (tables, engine, phonon builders), the engine's transport, finish_run()
    // (interpretation and results); end_runs() at the end.
    void begin_runs();
    void prepare_run(std::size_t run);
    void finish_run();
    void end_runs();
    int precision() const noexcept { return precision_; }
    bool steady_stop() const noexcept { return stop_on_; }
    void export_results(const std::string& json_path, double seconds) const;

    std::size_t n_sensors() const noexcept { return sensors_.size(); }
    std::size_t n_cells() const noexcept { return cells_.size(); }
    // Recorded steps of the results: all the model records, or those simulated before a stop at
    // steady state.
    std::size_t n_recorded() const noexcept { return recorded_; }
    std::size_t n_steps() const noexcept { return steps_; }
    std::size_t n_runs() const noexcept { return num_runs_; }
    SimType type() const noexcept { return type_; }
    const std::vector<std::vector<Measurement>>& measurements() const noexcept { return runs_; }
    std::vector<std::array<double, 6>> averaged() const;
    // Replaces the per-run results with given statistics stats[runs][S][6] (no per-step series).
    void set_measurements(const double* stats, std::size_t runs);
    void tallies(std::int64_t* energy, double* flux) const;
    const gpu::RunCounters& counters() const;
    double last_seconds() const noexcept { return last_seconds_; }
    double last_eff_energy() const noexcept { return eff_energy_; }
    // The simulator description this model hands to the GPU engine (the C ABI seam).
    const gpu::SimDesc& sim_desc() const noexcept { return desc_; }
    // Interpreter description with the given energy per phonon (<= 0: initial total energy / phonons).
    gpu::InterpDesc interp_for(double eff) const { return interp_desc(eff > 0. ? eff : initial_eff_); }
    gpu::Engine* engine() const noexcept { return engine_.get(); }
    // Energies ModelSimulator::initPhononBuilders turns into phonon counts (cell.cpp:38-41,
    // modelSimulator.cpp:66-70), for the current sensor temperatures.
    std::vector<double> cell_energies() const;
    std::vector<double> emit_energies() const;
    std::vector<double> sensor_init_temps() const;
    double t_eq() const noexcept { return t_eq_; }
    double initial_eff_energy() const noexcept { return initial_eff_; }

private:
    HostModel() = default;

    // settings
    std::size_t num_runs_{ 1 }, steps_{ 0 }, num_phonons_{ 0 }, step_interval_{ 0 };
    double sim_time_{ 0. }, t_eq_{ 0. };
    bool phasor_{ false };
    SimType type_{ SimType::SteadyState };
    std::size_t start_step_{ 0 }, step_adj_{ 0 }, recorded_{ 0 };
    double lb_{ 0. }, ub_{ 0. }, eff_energy_{ 0. }, initial_eff_{ 0. };

    std::vector<MaterialSpec> mat_specs_;
    std::vector<MaterialTables> mats_;
    std::vector<SensorRec> sensors_;
    std::vector<CellRec> cells_;
    std::vector<EmitterRec> emitters_;

    std::uint64_t seed_{ 1 };
    int precision_{ 0 };
    void* stream_{ nullptr };
    int grid_{ 0 };
    std::vector<double> t_start_;// warm-start temperatures (empty: the file's)
    bool stop_on_{ false };
    gpu::SteadyCriterion stop_crit_{};
    std::uint64_t stop_check_{ 0 };

    gpu::SimDesc desc_;
    std::unique_ptr<gpu::Engine> engine_;
    std::vector<std::vector<Measurement>> runs_;
    double last_seconds_{ 0. };
    std::chrono::steady_clock::time_point run_t0_{};

    // assembly
    void set_type(SimType t, std::size_t interval);
    void add_sensor(std::uint64_t id, std::uint32_t material, double t_init);
    void add_cell(P2 p1, P2 p2, P2 p3, std::uint64_t sensor_id, double spec);
    bool set_emit(P2 p1, P2 p2, double temp, double duration, double start);
    bool edge_accepts(const EdgeRec& e, const Seg64& line, double len) const;
    bool add_transition(std::uint32_t cell, const Seg64& line, double len, std::uint32_t target);
    std::size_t sensor_index(std::uint64_t id) const;

    // run helpers
    double init_temp(const SensorRec& s) const;
    double start_temp(std::size_t s) const;// the warm-start temperature, else init_temp
    double cell_init_energy(std::size_t c) const;
    double cell_emit_energy(std::size_t c) const;
    double total_energy() const;
    std::pair<double, double> bounds();
    void build_tables(double lo, double hi);
    void build_desc();
    gpu::InterpDesc interp_desc(double eff) const;
};

}// namespace psim
