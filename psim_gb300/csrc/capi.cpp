// C ABI of psim_gb300 (declared in include/psim_gb300.h).  Every entry point catches
// exceptions and returns a status code; the message is kept per thread.
#include "../../include/psim_gb300.h"

#include <algorithm>
#include <cstring>
#include <exception>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>

#include "device/engine.hpp"
#include "device/mlp.hpp"
#include "host/batch.hpp"
#include "host/model.hpp"

struct psim_model {
    std::unique_ptr<psim::HostModel> m;
    psim::gpu::InterpDesc interp_cache;// storage behind psim_model_interp_desc
};

struct psim_sim {
    std::unique_ptr<psim::gpu::Engine> e;
};

struct psim_mlp {
    std::unique_ptr<psim::gpu::Mlp> net;
};

namespace {

thread_local std::string g_error;

int fail(int code, const std::string& msg) {
    g_error = msg;
    return code;
}

bool is_cuda_error(const std::string& msg) {
    return msg.find("CUDA") != std::string::npos || msg.find("cuda") != std::string::npos
           || msg.find("no CUDA device") != std::string::npos;
}

template<typename F> int guard(F f) {
    try {
        f();
        return PSIM_OK;
    } catch (const std::invalid_argument& e) {
        return fail(PSIM_ERR_INVALID, e.what());
    } catch (const std::length_error& e) {
        return fail(PSIM_ERR_LIMIT, e.what());
    } catch (const std::bad_alloc&) {
        return fail(PSIM_ERR_LIMIT, "out of host memory");
    } catch (const std::exception& e) {
        const std::string msg = e.what();
        if (msg.rfind("Error opening file", 0) == 0 || msg.rfind("cannot write", 0) == 0) { return fail(PSIM_ERR_IO, msg); }
        if (is_cuda_error(msg)) { return fail(PSIM_ERR_CUDA, msg); }
        return fail(PSIM_ERR_INVALID, msg);
    } catch (...) {
        return fail(PSIM_ERR_INVALID, "unknown error");
    }
}

template<typename T> std::vector<T> copy_of(const T* p, std::size_t n, const char* what) {
    if (n > 0 && p == nullptr) { throw std::invalid_argument(std::string("missing array: ") + what); }
    return n > 0 ? std::vector<T>(p, p + n) : std::vector<T>{};
}

// The ABI views of the flattened model and of its interpreter description: pointers into d.
void fill_sim_desc(const psim::gpu::SimDesc& d, psim_sim_desc* out) {
    *out = psim_sim_desc{};
    out->measurement_steps = d.steps;
    out->simulation_time = d.sim_time;
    out->phasor_sim = d.phasor ? 1 : 0;
    out->sim_type = d.sim_type;
    out->step_adjustment = d.step_adj;
    out->recorded_steps = d.recorded;
    out->full_simulation = d.full ? 1 : 0;
    out->n_materials = d.n_materials;
    out->mat_freq = d.mat_freq.data();
    out->mat_vel = d.mat_vel.data();
    out->mat_params = d.mat_params.data();
    out->n_tables = d.n_tables;
    out->tables = d.tables.data();
    out->n_sensors = d.n_sensors;
    out->sensor_material = d.sensor_material.data();
    out->sensor_temp = d.sensor_temp.data();
    out->sensor_base_table = d.sensor_base_table.data();
    out->sensor_scatter_table = d.sensor_scatter_table.data();
    out->n_cells = d.n_cells;
    out->cell_vertices = d.cell_vertices.data();
    out->cell_sensor = d.cell_sensor.data();
    out->cell_spec = d.cell_spec.data();
    out->edge_sub_begin = d.edge_sub_begin.data();
    out->n_subs = static_cast<uint32_t>(d.sub_kind.size());
    out->sub_kind = d.sub_kind.data();
    out->sub_target = d.sub_target.data();
    out->sub_line = d.sub_line.data();
    out->n_emitters = d.n_emitters;
    out->emit_cell = d.emit_cell.data();
    out->emit_edge = d.emit_edge.data();
    out->emit_line = d.emit_line.data();
    out->emit_temp = d.emit_temp.data();
    out->emit_start = d.emit_start.data();
    out->emit_duration = d.emit_duration.data();
    out->emit_table = d.emit_table.data();
}

void fill_interp_desc(const psim::gpu::InterpDesc& d, psim_interp_desc* out) {
    *out = psim_interp_desc{};
    out->n_sensors = d.n_sensors;
    out->recorded_steps = d.recorded;
    out->t_eq = d.t_eq;
    out->eff_energy = d.eff_energy;
    out->lower_bound = d.lb;
    out->upper_bound = d.ub;
    out->sensor_area = d.area.data();
    out->sensor_heat_capacity = d.heat_capacity.data();
    out->sensor_init_temp = d.init_temp.data();
    out->sensor_material = d.material.data();
    out->n_materials = static_cast<uint32_t>(d.mat_temp_begin.size() - 1);
    out->mat_temp_begin = d.mat_temp_begin.data();
    out->temps = d.temps.data();
    out->energies = d.energies.data();
}

}// namespace

extern "C" {

const char* psim_last_error(void) { return g_error.c_str(); }

const char* psim_version(void) { return "psim_gb300 0.1 (sm_103a)"; }

int psim_device_count(void) { return psim::gpu::device_count(); }

// ------------------------------------------------------------------ model level
int psim_model_load_json(const char* json_path, psim_model** out) {
    if (json_path == nullptr || out == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    return guard([&]() {
        auto h = std::make_unique<psim_model>();
        h->m = psim::HostModel::from_json(json_path);
        *out = h.release();
    });
}

int psim_model_set_options(psim_model* m, uint64_t seed, int32_t precision, void* cuda_stream) {
    if (m == nullptr) { return fail(PSIM_ERR_INVALID, "null model"); }
    if (precision != PSIM_PRECISION_FP32 && precision != PSIM_PRECISION_FP64) { return fail(PSIM_ERR_INVALID, "unknown precision"); }
    m->m->set_options(seed, precision, cuda_stream);
    return PSIM_OK;
}

int psim_model_run(psim_model* m) {
    if (m == nullptr) { return fail(PSIM_ERR_INVALID, "null model"); }
    return guard([&]() { m->m->run(); });
}

int psim_model_shape(const psim_model* m, int64_t* n_sensors, int64_t* n_recorded, int64_t* n_cells, int64_t* n_steps,
                     int64_t* n_runs) {
    if (m == nullptr) { return fail(PSIM_ERR_INVALID, "null model"); }
    if (n_sensors != nullptr) { *n_sensors = static_cast<int64_t>(m->m->n_sensors()); }
    if (n_recorded != nullptr) { *n_recorded = static_cast<int64_t>(m->m->n_recorded()); }
    if (n_cells != nullptr) { *n_cells = static_cast<int64_t>(m->m->n_cells()); }
    if (n_steps != nullptr) { *n_steps = static_cast<int64_t>(m->m->n_steps()); }
    if (n_runs != nullptr) { *n_runs = static_cast<int64_t>(m->m->n_runs()); }
    return PSIM_OK;
}

int psim_model_set_measurements(psim_model* m, const double* stats, int64_t runs) {
    if (m == nullptr || stats == nullptr || runs < 1) { return fail(PSIM_ERR_INVALID, "bad arguments"); }
    return guard([&]() { m->m->set_measurements(stats, static_cast<std::size_t>(runs)); });
}

int psim_model_measurements(const psim_model* m, double* stats) {
    if (m == nullptr || stats == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    if (m->m->measurements().empty()) { return fail(PSIM_ERR_INVALID, "the model has not been run"); }
    return guard([&]() {
        const auto a = m->m->averaged();
        for (std::size_t i = 0; i < a.size(); ++i) { std::memcpy(stats + 6 * i, a[i].data(), 6 * sizeof(double)); }
    });
}

int psim_model_series(const psim_model* m, int64_t run, double* temps, double* fluxes) {
    if (m == nullptr) { return fail(PSIM_ERR_INVALID, "null model"); }
    const auto& runs = m->m->measurements();
    if (run < 0 || static_cast<std::size_t>(run) >= runs.size()) { return fail(PSIM_ERR_INVALID, "run index out of range"); }
    const auto& r = runs[static_cast<std::size_t>(run)];
    const std::size_t K = m->m->n_recorded();
    for (std::size_t s = 0; s < r.size(); ++s) {
        if (temps != nullptr && K > 0) { std::memcpy(temps + s * K, r[s].temps.data(), K * sizeof(double)); }
        if (fluxes != nullptr && K > 0) { std::memcpy(fluxes + 2 * s * K, r[s].fluxes.data(), 2 * K * sizeof(double)); }
    }
    return PSIM_OK;
}

int psim_model_tallies(const psim_model* m, int64_t* energy, double* flux) {
    if (m == nullptr) { return fail(PSIM_ERR_INVALID, "null model"); }
    return guard([&]() { m->m->tallies(energy, flux); });
}

int psim_model_counters(const psim_model* m, psim_run_counters* out) {
    if (m == nullptr || out == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    const auto& c = m->m->counters();
    out->phonons = c.phonons;
    out->phonon_steps = c.phonon_steps;
    out->kernel_launches = c.kernel_launches;
    out->eff_energy = m->m->last_eff_energy();
    out->seconds = m->m->last_seconds();
    out->kernel_ms = c.kernel_ms;
    out->max_population = c.max_population;
    out->limit_hits = c.relocations;
    out->event_limit_hits = c.event_limits;
    out->h2d_bytes = c.h2d_bytes;
    out->d2h_bytes = c.d2h_bytes;
    out->transport_launches = c.transport_launches;
    out->steps_per_launch = c.steps_per_launch;
    out->backscatters = c.backscatters;
    out->state_bytes = c.state_bytes;
    return PSIM_OK;
}

int psim_model_population(const psim_model* m, uint32_t* out) {
    if (m == nullptr || out == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    if (m->m->engine() == nullptr) { return fail(PSIM_ERR_INVALID, "the model has not been run"); }
    return guard([&]() { m->m->engine()->population(out); });
}

int psim_model_start_temps(const psim_model* m, double* out) {
    if (m == nullptr || out == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    return guard([&]() {
        const auto t = m->m->start_temps();
        std::copy(t.begin(), t.end(), out);
    });
}

int psim_model_set_start_temps(psim_model* m, const double* temps) {
    if (m == nullptr) { return fail(PSIM_ERR_INVALID, "null model"); }
    return guard([&]() {
        m->m->set_start_temps(temps == nullptr ? std::vector<double>{} : std::vector<double>(temps, temps + m->m->n_sensors()));
    });
}

int psim_model_export(const psim_model* m, const char* json_path, double seconds) {
    if (m == nullptr || json_path == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    if (m->m->measurements().empty()) { return fail(PSIM_ERR_INVALID, "the model has not been run"); }
    return guard([&]() { m->m->export_results(json_path, seconds); });
}

int psim_model_sim_desc(const psim_model* m, psim_sim_desc* out) {
    if (m == nullptr || out == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    return guard([&]() { fill_sim_desc(m->m->sim_desc(), out); });
}

int psim_model_interp_desc(const psim_model* m, double eff_energy, psim_interp_desc* out) {
    if (m == nullptr || out == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    auto* mm = const_cast<psim_model*>(m);
    return guard([&]() {
        mm->interp_cache = m->m->interp_for(eff_energy);
        fill_interp_desc(mm->interp_cache, out);
    });
}

void psim_model_destroy(psim_model* m) { delete m; }

// ------------------------------------------------------------------ simulator seam
int psim_sim_create(const psim_sim_desc* d, psim_sim** out) {
    if (d == nullptr || out == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    return guard([&]() {
        constexpr std::size_t B = PSIM_NUM_FREQ_BINS;
        psim::gpu::SimDesc s;
        s.steps = d->measurement_steps;
        s.sim_time = d->simulation_time;
        s.phasor = d->phasor_sim != 0;
        s.sim_type = d->sim_type;
        s.step_adj = d->step_adjustment;
        s.recorded = d->recorded_steps;
        s.full = d->full_simulation != 0;
        if (s.steps == 0 || !(s.sim_time > 0.)) { throw std::invalid_argument("measurement_steps and simulation_time must be positive"); }
        if (s.recorded + s.step_adj < s.steps) { throw std::invalid_argument("recorded_steps + step_adjustment must cover the measurement steps"); }
        s.n_materials = d->n_materials;
        s.mat_freq = copy_of(d->mat_freq, static_cast<std::size_t>(d->n_materials) * B, "mat_freq");
        s.mat_vel = copy_of(d->mat_vel, static_cast<std::size_t>(d->n_materials) * 2 * B, "mat_vel");
        s.mat_params = copy_of(d->mat_params, static_cast<std::size_t>(d->n_materials) * 8, "mat_params");
        s.n_tables = d->n_tables;
        s.tables = copy_of(d->tables, static_cast<std::size_t>(d->n_tables) * B * 2, "tables");
        s.n_sensors = d->n_sensors;
        s.sensor_material = copy_of(d->sensor_material, d->n_sensors, "sensor_material");
        s.sensor_temp = copy_of(d->sensor_temp, d->n_sensors, "sensor_temp");
        s.sensor_base_table = copy_of(d->sensor_base_table, d->n_sensors, "sensor_base_table");
        s.sensor_scatter_table = copy_of(d->sensor_scatter_table, d->n_sensors, "sensor_scatter_table");
        s.n_cells = d->n_cells;
        s.cell_vertices = copy_of(d->cell_vertices, static_cast<std::size_t>(d->n_cells) * 6, "cell_vertices");
        s.cell_sensor = copy_of(d->cell_sensor, d->n_cells, "cell_sensor");
        s.cell_spec = copy_of(d->cell_spec, d->n_cells, "cell_spec");
        s.edge_sub_begin = copy_of(d->edge_sub_begin, static_cast<std::size_t>(d->n_cells) * 3 + 1, "edge_sub_begin");
        if (s.edge_sub_begin.front() != 0 || s.edge_sub_begin.back() != d->n_subs) { throw std::invalid_argument("edge_sub_begin must run from 0 to n_subs"); }
        for (std::size_t i = 1; i < s.edge_sub_begin.size(); ++i) {
            if (s.edge_sub_begin[i] < s.edge_sub_begin[i - 1]) { throw std::invalid_argument("edge_sub_begin must be non-decreasing"); }
        }
        s.sub_kind = copy_of(d->sub_kind, d->n_subs, "sub_kind");
        s.sub_target = copy_of(d->sub_target, d->n_subs, "sub_target");
        s.sub_line = copy_of(d->sub_line, static_cast<std::size_t>(d->n_subs) * 4, "sub_line");
        s.n_emitters = d->n_emitters;
        s.emit_cell = copy_of(d->emit_cell, d->n_emitters, "emit_cell");
        s.emit_edge = copy_of(d->emit_edge, d->n_emitters, "emit_edge");
        s.emit_line = copy_of(d->emit_line, static_cast<std::size_t>(d->n_emitters) * 4, "emit_line");
        s.emit_temp = copy_of(d->emit_temp, d->n_emitters, "emit_temp");
        s.emit_start = copy_of(d->emit_start, d->n_emitters, "emit_start");
        s.emit_duration = copy_of(d->emit_duration, d->n_emitters, "emit_duration");
        s.emit_table = copy_of(d->emit_table, d->n_emitters, "emit_table");
        auto h = std::make_unique<psim_sim>();
        h->e = std::make_unique<psim::gpu::Engine>(s);
        *out = h.release();
    });
}

int psim_sim_init_phonon_builders(psim_sim* s, double t_eq, double eff_energy, const double* cell_energy,
                                  const double* emit_energy, const double* sensor_init_temp, uint64_t seed,
                                  uint64_t* total_phonons) {
    if (s == nullptr || cell_energy == nullptr || sensor_init_temp == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    if (emit_energy == nullptr && s->e->desc().n_emitters > 0) { return fail(PSIM_ERR_INVALID, "null emit_energy"); }
    return guard([&]() {
        const std::uint64_t n = s->e->init_builders(t_eq, eff_energy, cell_energy, emit_energy, sensor_init_temp, seed);
        if (total_phonons != nullptr) { *total_phonons = n; }
    });
}

int psim_sim_run(psim_sim* s, double /*t_eq*/, int32_t precision, void* cuda_stream) {
    if (s == nullptr) { return fail(PSIM_ERR_INVALID, "null simulator"); }
    if (precision != PSIM_PRECISION_FP32 && precision != PSIM_PRECISION_FP64) { return fail(PSIM_ERR_INVALID, "unknown precision"); }
    return guard([&]() { s->e->run(precision, cuda_stream); });
}

int psim_sim_reset(psim_sim* s) {
    if (s == nullptr) { return fail(PSIM_ERR_INVALID, "null simulator"); }
    return guard([&]() { s->e->reset(); });
}

int psim_sim_set_step_adjustment(psim_sim* s, uint64_t step_adjustment) {
    if (s == nullptr) { return fail(PSIM_ERR_INVALID, "null simulator"); }
    if (step_adjustment > s->e->desc().steps) { return fail(PSIM_ERR_INVALID, "step adjustment beyond the measurement steps"); }
    s->e->set_step_adjustment(step_adjustment);
    return PSIM_OK;
}

int psim_sim_tallies(const psim_sim* s, int64_t* energy, double* flux) {
    if (s == nullptr) { return fail(PSIM_ERR_INVALID, "null simulator"); }
    return guard([&]() { s->e->tallies(energy, flux); });
}

int psim_sim_counters(const psim_sim* s, psim_run_counters* out) {
    if (s == nullptr || out == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    const auto& c = s->e->counters();
    *out = psim_run_counters{};
    out->phonons = c.phonons;
    out->phonon_steps = c.phonon_steps;
    out->kernel_launches = c.kernel_launches;
    out->kernel_ms = c.kernel_ms;
    out->max_population = c.max_population;
    out->limit_hits = c.relocations;
    out->event_limit_hits = c.event_limits;
    out->h2d_bytes = c.h2d_bytes;
    out->d2h_bytes = c.d2h_bytes;
    out->transport_launches = c.transport_launches;
    out->steps_per_launch = c.steps_per_launch;
    out->backscatters = c.backscatters;
    out->state_bytes = c.state_bytes;
    return PSIM_OK;
}

int psim_sim_population(const psim_sim* s, uint32_t* out) {
    if (s == nullptr || out == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    return guard([&]() { s->e->population(out); });
}

void psim_sim_destroy(psim_sim* s) { delete s; }

// ------------------------------------------------------------------ interpreter
namespace {
psim::gpu::InterpDesc interp_from(const psim_interp_desc* d) {
    psim::gpu::InterpDesc o;
    o.n_sensors = d->n_sensors;
    o.recorded = d->recorded_steps;
    o.t_eq = d->t_eq;
    o.eff_energy = d->eff_energy;
    o.lb = d->lower_bound;
    o.ub = d->upper_bound;
    o.area = copy_of(d->sensor_area, d->n_sensors, "sensor_area");
    o.heat_capacity = copy_of(d->sensor_heat_capacity, d->n_sensors, "sensor_heat_capacity");
    o.init_temp = copy_of(d->sensor_init_temp, d->n_sensors, "sensor_init_temp");
    o.material = copy_of(d->sensor_material, d->n_sensors, "sensor_material");
    o.mat_temp_begin = copy_of(d->mat_temp_begin, static_cast<std::size_t>(d->n_materials) + 1, "mat_temp_begin");
    const std::size_t nt = o.mat_temp_begin.empty() ? 0 : static_cast<std::size_t>(o.mat_temp_begin.back());
    o.temps = copy_of(d->temps, nt, "temps");
    o.energies = copy_of(d->energies, nt, "energies");
    for (std::size_t m = 0; m + 1 < o.mat_temp_begin.size(); ++m) {
        if (o.mat_temp_begin[m + 1] < o.mat_temp_begin[m]) { throw std::invalid_argument("mat_temp_begin decreases"); }
    }
    for (auto m : o.material) {
        if (m >= d->n_materials) { throw std::invalid_argument("sensor material out of range"); }
        if (o.mat_temp_begin[m + 1] <= o.mat_temp_begin[m]) { throw std::invalid_argument("material has an empty temperature grid"); }
    }
    return o;
}
}// namespace

int psim_interpret(const psim_interp_desc* d, const int64_t* energy, const double* flux, double* temps, double* fluxes,
                   double* stats) {
    if (d == nullptr || energy == nullptr || flux == nullptr || stats == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    return guard([&]() { psim::gpu::interpret_host(interp_from(d), energy, flux, temps, fluxes, stats); });
}

int psim_final_temps(const psim_interp_desc* d, const int64_t* energy, uint64_t start_step, double* out) {
    if (d == nullptr || energy == nullptr || out == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    return guard([&]() { psim::gpu::final_temps_host(interp_from(d), energy, start_step, out); });
}

// ------------------------------------------------------------------ steady-state detection
namespace {
psim::gpu::SteadyCriterion criterion(uint32_t window, uint32_t batches, double z, uint32_t patience, double drift_z) {
    psim::gpu::SteadyCriterion c;
    c.window = window;
    c.batches = batches;
    c.z = z;
    c.patience = patience;
    c.drift_z = drift_z;
    psim::gpu::validate_steady(c);
    return c;
}
}// namespace

int psim_steady_state(const int64_t* energy, const double* flux, uint32_t n_sensors, uint64_t recorded_steps, uint32_t window,
                      uint32_t batches, double z, uint32_t patience, double drift_z, int64_t* onset_step, int64_t* per_sensor) {
    if (onset_step == nullptr || (n_sensors > 0 && recorded_steps > 0 && (energy == nullptr || flux == nullptr))) {
        return fail(PSIM_ERR_INVALID, "null argument");
    }
    return guard([&]() {
        const auto c = criterion(window, batches, z, patience, drift_z);
        *onset_step = psim::gpu::steady_onset_host(energy, flux, n_sensors, recorded_steps, c, reinterpret_cast<long long*>(per_sensor));
    });
}

int psim_sim_steady_state(const psim_sim* s, uint32_t window, uint32_t batches, double z, uint32_t patience, double drift_z,
                          int64_t* onset_step,
                          int64_t* per_sensor) {
    if (s == nullptr || onset_step == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    return guard([&]() {
        *onset_step = s->e->steady_onset(criterion(window, batches, z, patience, drift_z), reinterpret_cast<long long*>(per_sensor));
    });
}

int psim_model_steady_state(const psim_model* m, uint32_t window, uint32_t batches, double z, uint32_t patience, double drift_z,
                            int64_t* onset_step, int64_t* per_sensor) {
    if (m == nullptr || onset_step == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    if (m->m->engine() == nullptr) { return fail(PSIM_ERR_INVALID, "the model has not been run"); }
    return guard([&]() {
        *onset_step = m->m->engine()->steady_onset(criterion(window, batches, z, patience, drift_z),
                                                   reinterpret_cast<long long*>(per_sensor));
    });
}

int psim_model_set_steady_stop(psim_model* m, int32_t enable, uint32_t window, uint32_t batches, double z, uint32_t patience,
                               double drift_z,
                               uint64_t check_every) {
    if (m == nullptr) { return fail(PSIM_ERR_INVALID, "null model"); }
    return guard([&]() {
        psim::gpu::SteadyCriterion c;
        if (enable != 0) { c = criterion(window, batches, z, patience, drift_z); }
        m->m->set_steady_stop(enable != 0, c, check_every);
    });
}

int psim_sim_set_steady_stop(psim_sim* s, int32_t enable, uint32_t window, uint32_t batches, double z, uint32_t patience,
                             double drift_z,
                             uint64_t check_every) {
    if (s == nullptr) { return fail(PSIM_ERR_INVALID, "null simulator"); }
    return guard([&]() {
        psim::gpu::SteadyCriterion c;
        if (enable != 0) { c = criterion(window, batches, z, patience, drift_z); }
        s->e->set_steady_stop(enable != 0, c, check_every);
    });
}

int psim_model_steps_run(const psim_model* m, uint64_t* steps) {
    if (m == nullptr || steps == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    if (m->m->engine() == nullptr) { return fail(PSIM_ERR_INVALID, "the model has not been run"); }
    *steps = m->m->engine()->steps_run();
    return PSIM_OK;
}

int psim_sim_steps_run(const psim_sim* s, uint64_t* steps) {
    if (s == nullptr || steps == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    *steps = s->e->steps_run();
    return PSIM_OK;
}

// ------------------------------------------------------------------ the surrogate MLP
int psim_mlp_create(const int32_t* widths, int32_t n_widths, uint64_t seed, psim_mlp** out) {
    if (widths == nullptr || out == nullptr || n_widths < 2) { return fail(PSIM_ERR_INVALID, "bad arguments"); }
    return guard([&]() {
        auto h = std::make_unique<psim_mlp>();
        h->net = std::make_unique<psim::gpu::Mlp>(std::vector<int>(widths, widths + n_widths), seed);
        *out = h.release();
    });
}

int psim_mlp_n_params(const psim_mlp* net, uint64_t* n) {
    if (net == nullptr || n == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    *n = net->net->n_params();
    return PSIM_OK;
}

int psim_mlp_get_params(const psim_mlp* net, float* out) {
    if (net == nullptr || out == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    return guard([&]() { net->net->get_params(out); });
}

int psim_mlp_set_params(psim_mlp* net, const float* in) {
    if (net == nullptr || in == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    return guard([&]() { net->net->set_params(in); });
}

int psim_mlp_gradients(psim_mlp* net, const float* x, const float* y, int32_t n, float* loss, float* grads) {
    if (net == nullptr || x == nullptr || y == nullptr || n < 1) { return fail(PSIM_ERR_INVALID, "bad arguments"); }
    return guard([&]() {
        const float l = net->net->gradients(x, y, n, grads);
        if (loss != nullptr) { *loss = l; }
    });
}

int psim_mlp_train(psim_mlp* net, const float* x, const float* y, int32_t n, int32_t batch, int32_t epochs, float lr, uint64_t seed,
                   float* final_loss) {
    if (net == nullptr || x == nullptr || y == nullptr || n < 1 || batch < 1 || epochs < 0 || !(lr > 0.f)) {
        return fail(PSIM_ERR_INVALID, "bad arguments");
    }
    return guard([&]() {
        const float l = net->net->train(x, y, n, batch, epochs, lr, seed);
        if (final_loss != nullptr) { *final_loss = l; }
    });
}

int psim_mlp_predict(psim_mlp* net, const float* x, int32_t n, float* y) {
    if (net == nullptr || x == nullptr || y == nullptr || n < 0) { return fail(PSIM_ERR_INVALID, "bad arguments"); }
    return guard([&]() { net->net->predict(x, n, y); });
}

void psim_mlp_destroy(psim_mlp* net) { delete net; }

// ------------------------------------------------------------------ batches of models
namespace {
std::vector<psim::HostModel*> batch_models(psim_model* const* models, int32_t n) {
    if (n < 0 || (n > 0 && models == nullptr)) { throw std::invalid_argument("bad model list"); }
    std::vector<psim::HostModel*> v;
    for (int32_t i = 0; i < n; ++i) {
        if (models[i] == nullptr) { throw std::invalid_argument("null model in the batch"); }
        v.push_back(models[i]->m.get());
    }
    return v;
}
}// namespace

int psim_batch_run(psim_model* const* models, int32_t n, const psim_batch_options* opt, double* seconds, uint64_t* phonon_steps) {
    if (opt == nullptr) { return fail(PSIM_ERR_INVALID, "null options"); }
    return guard([&]() {
        psim::BatchOptions o;
        o.workers = opt->workers;
        o.max_blocks = opt->max_blocks;
        o.device_queue = opt->device_queue;
        o.per_thread = opt->per_thread;
        const psim::BatchResult r = psim::run_batch(batch_models(models, n), o);
        if (seconds != nullptr) { *seconds = r.seconds; }
        if (phonon_steps != nullptr) { *phonon_steps = r.phonon_steps; }
    });
}

int psim_batch_autotune(psim_model* const* models, int32_t n, int32_t sample, psim_batch_options* out, double* best_rate) {
    if (out == nullptr) { return fail(PSIM_ERR_INVALID, "null options"); }
    return guard([&]() {
        const psim::BatchOptions o = psim::autotune_batch(batch_models(models, n), sample, best_rate);
        out->workers = o.workers;
        out->max_blocks = o.max_blocks;
        out->device_queue = o.device_queue;
        out->per_thread = o.per_thread;
    });
}

int psim_final_temps_noalloc(const psim_interp_desc* d, const int64_t* energy_dev, uint64_t start_step, double* out_dev,
                             void* cuda_stream) {
    if (d == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    return guard([&]() {
        psim::gpu::InterpView v;
        v.n_sensors = d->n_sensors;
        v.recorded = d->recorded_steps;
        v.t_eq = d->t_eq;
        v.eff_energy = d->eff_energy;
        v.lb = d->lower_bound;
        v.ub = d->upper_bound;
        v.area = d->sensor_area;
        v.heat_capacity = d->sensor_heat_capacity;
        v.material = d->sensor_material;
        v.n_materials = d->n_materials;
        v.mat_temp_begin = d->mat_temp_begin;
        v.temps = d->temps;
        v.energies = d->energies;
        psim::gpu::final_temps_noalloc(v, energy_dev, start_step, out_dev, cuda_stream);
    });
}

uint64_t psim_final_temps_noalloc_max_bytes(void) { return psim::gpu::kFinalTempsScratchBytes; }

// ------------------------------------------------------------------ geometry
int psim_geom_intersect(int64_t n, const double* a, const double* b, double* poi, int32_t* has) {
    if (n < 0 || (n > 0 && (a == nullptr || b == nullptr || poi == nullptr || has == nullptr))) { return fail(PSIM_ERR_INVALID, "bad arguments"); }
    return guard([&]() { psim::gpu::geom_intersect(n, a, b, poi, has); });
}
int psim_geom_on_line(int64_t n, const double* lines, const double* pts, int32_t* out) {
    if (n < 0 || (n > 0 && (lines == nullptr || pts == nullptr || out == nullptr))) { return fail(PSIM_ERR_INVALID, "bad arguments"); }
    return guard([&]() { psim::gpu::geom_on_line(n, lines, pts, out); });
}
int psim_geom_tri_contains(int64_t n, const double* tris, const double* pts, int32_t* out) {
    if (n < 0 || (n > 0 && (tris == nullptr || pts == nullptr || out == nullptr))) { return fail(PSIM_ERR_INVALID, "bad arguments"); }
    return guard([&]() { psim::gpu::geom_tri_contains(n, tris, pts, out); });
}
int psim_geom_edge_index(int64_t n, const double* tris, const double* pts, int32_t* out) {
    if (n < 0 || (n > 0 && (tris == nullptr || pts == nullptr || out == nullptr))) { return fail(PSIM_ERR_INVALID, "bad arguments"); }
    return guard([&]() { psim::gpu::geom_edge_index(n, tris, pts, out); });
}

int psim_rates(const double* mat_params, int64_t n, const double* T, const double* freq, const int32_t* pol, int precision,
               double* out) {
    if (n < 0 || mat_params == nullptr || (n > 0 && (T == nullptr || freq == nullptr || pol == nullptr || out == nullptr))
        || (precision != PSIM_PRECISION_FP32 && precision != PSIM_PRECISION_FP64)) {
        return fail(PSIM_ERR_INVALID, "bad arguments");
    }
    return guard([&]() { psim::gpu::rates_probe(mat_params, n, T, freq, pol, precision, out); });
}

int psim_sampling_alias_table(const double* table, uint32_t* out) {
    if (table == nullptr || out == nullptr) { return fail(PSIM_ERR_INVALID, "null argument"); }
    return guard([&]() {
        const auto t = psim::gpu::alias_table_of(table);
        std::copy(t.begin(), t.end(), out);
    });
}

}// extern "C"
