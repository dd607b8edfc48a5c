// Test-oracle driver for the reference psim sources (built by oracle/ref_recipe/Makefile).
//
// The reference reads models with nlohmann::json (psim/src/inputManager.cpp),
// which is not available here.  This driver parses the same JSON schema with the
// project's own reader and builds the reference Model through its public API in
// the order inputManager.cpp:79-105 uses, then runs and dumps results.  Private
// members are opened only in this translation unit, to read tallies and tables
// for golden vectors.
//
// Subcommands:
//   run    <model.json> <dump.json> [export.json-path]   run the model, dump tallies/measurements
//   tables <model.json> <dump.bin>                       material tables after initializeTables
//   geom   <cases.txt> <out.txt>                         geometry known answers
//   invert <model.json> <counts.txt> <out.txt>           E->T inversion of given counts
//   topology <model.json> <out.txt>                      assembled cells and edge sub-surfaces
//   rates  <model.json> <cases.bin> <out.bin>            Material::relaxRates of every material on
//                                                        given (T, frequency, polarization) triples
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <execution>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <optional>
#include <sstream>
#include <stack>
#include <string>
#include <unordered_map>
#include <variant>
#include <vector>

#include "../../psim_gb300/csrc/host/json.hpp"

#define private public
#define protected public
#include "psim/cell.h"
#include "psim/geometry.h"
#include "psim/material.h"
#include "psim/model.h"
#include "psim/sensor.h"
#include "psim/sensorInterpreter.h"
#undef private
#undef protected

using psim_json::Value;
using Geometry::Line;
using Geometry::Point;
using Geometry::Triangle;

namespace {

Point getPoint(const Value& v) { return Point{ v.at("x").as_double(), v.at("y").as_double() }; }

std::unique_ptr<Model> buildModel(const Value& j) {
    const Value& settings = j.at("settings");
    const Value& sensors = j.at("sensors");
    const Value& cells = j.at("cells");
    const double t_eq = settings.at("t_eq").as_double();
    ModelParams params{ 1,
        cells.size(),
        sensors.size(),
        static_cast<std::size_t>(settings.at("num_measurements").as_int()),
        static_cast<std::size_t>(settings.at("num_phonons").as_int()),
        settings.at("sim_time").as_double(),
        t_eq,
        settings.at("phasor_sim").kind() == Value::Kind::Bool && settings.at("phasor_sim").as_bool() };
    if (settings.contains("num_runs")) { params.num_runs = static_cast<std::size_t>(settings.at("num_runs").as_int()); }
    auto model = std::make_unique<Model>(params);
    SimulationType type = SimulationType::SteadyState;
    const auto st = settings.at("sim_type").as_int();
    if (st == 1) { type = SimulationType::Periodic; }
    if (st == 2) { type = SimulationType::Transient; }
    if (type == SimulationType::SteadyState) {
        model->setSimulationType(type);
    } else {
        model->setSimulationType(type, static_cast<std::size_t>(settings.at("step_interval").as_int()));
    }
    std::size_t material_id = 0;
    for (const Value& m : j.at("materials").items()) {
        const Value& d = m.at("d_data");
        const Value& r = m.at("r_data");
        const std::array<double, 3> la{ d.at("la_data").at(0).as_double(), d.at("la_data").at(1).as_double(),
            d.at("la_data").at(2).as_double() };
        const std::array<double, 3> ta{ d.at("ta_data").at(0).as_double(), d.at("ta_data").at(1).as_double(),
            d.at("ta_data").at(2).as_double() };
        const DispersionData dd{ la, ta, d.at("max_freq_la").as_double(), d.at("max_freq_ta").as_double() };
        const RelaxationData rd{ r.at("b_l").as_double(), r.at("b_tn").as_double(), r.at("b_tu").as_double(),
            r.at("b_i").as_double(), r.at("w").as_double() };
        auto material = Material(material_id++, dd, rd);
        if (t_eq == 0.) { material.setFullSimulation(); }
        model->addMaterial(m.at("name").as_string(), material);
    }
    for (const Value& s : sensors.items()) {
        model->addSensor(static_cast<std::size_t>(s.at("id").as_int()), s.at("material").as_string(),
            s.at("t_init").as_double(), type);
    }
    for (const Value& c : cells.items()) {
        const Value& t = c.at("triangle");
        Triangle tri{ getPoint(t.at("p1")), getPoint(t.at("p2")), getPoint(t.at("p3")) };
        model->addCell(std::move(tri), static_cast<std::size_t>(c.at("sensorID").as_int()),
            c.at("specularity").as_double());
    }
    for (const Value& e : j.at("emit_surfaces").items()) {
        if (!model->setEmitSurface(getPoint(e.at("p1")), getPoint(e.at("p2")), e.at("temp").as_double(),
                e.at("duration").as_double(), e.at("start_time").as_double())) {
            throw std::runtime_error("Unable to add emitting surface.");
        }
    }
    return model;
}

void put(std::ostream& os, double v) { os << std::setprecision(17) << v; }

template<typename T> void putArray(std::ostream& os, const std::vector<T>& v) {
    os << '[';
    for (std::size_t i = 0; i < v.size(); ++i) {
        if (i) { os << ','; }
        if constexpr (std::is_floating_point_v<T>) {
            put(os, v[i]);
        } else {
            os << v[i];
        }
    }
    os << ']';
}

int cmdRun(const std::string& model_path, const std::string& dump_path, const std::string& export_path) {
    const Value j = psim_json::parse_file(model_path);
    auto model = buildModel(j);
    model->runSimulation();
    if (!export_path.empty()) { model->exportResults(export_path, 0.0); }
    std::ofstream os(dump_path);
    os << "{\"total_phonons_last_run\":" << model->simulator_.total_phonons_;
    os << ",\"t_eq\":";
    put(os, model->t_eq_);
    os << ",\"sensors\":[";
    for (std::size_t i = 0; i < model->sensors_.size(); ++i) {
        const Sensor& s = model->sensors_[i];
        if (i) { os << ','; }
        os << "{\"id\":" << s.getID() << ",\"area\":";
        put(os, s.getArea());
        os << ",\"heat_capacity\":";
        put(os, s.getHeatCapacity());
        os << ",\"energies\":";
        putArray(os, s.getEnergies());
        std::vector<double> fx;
        std::vector<double> fy;
        for (const auto& f : s.getFluxes()) {
            fx.push_back(f[0]);
            fy.push_back(f[1]);
        }
        os << ",\"flux_x\":";
        putArray(os, fx);
        os << ",\"flux_y\":";
        putArray(os, fy);
        os << '}';
    }
    os << "],\"runs\":[";
    bool first_run = true;
    std::vector<std::size_t> run_ids;
    for (const auto& kv : model->outputManager_.measurements_) { run_ids.push_back(kv.first); }
    std::sort(run_ids.begin(), run_ids.end());
    for (const auto run_id : run_ids) {
        if (!first_run) { os << ','; }
        first_run = false;
        os << '[';
        const auto& ms = model->outputManager_.measurements_.at(run_id);
        for (std::size_t i = 0; i < ms.size(); ++i) {
            const auto& m = ms[i];
            if (i) { os << ','; }
            os << "{\"id\":" << m.id << ",\"stats\":[";
            put(os, m.t_steady);
            os << ',';
            put(os, m.std_t_steady);
            os << ',';
            put(os, m.x_flux);
            os << ',';
            put(os, m.std_x_flux);
            os << ',';
            put(os, m.y_flux);
            os << ',';
            put(os, m.std_y_flux);
            os << "],\"final_temps\":";
            putArray(os, m.final_temps);
            std::vector<double> fx;
            std::vector<double> fy;
            for (const auto& f : m.final_fluxes) {
                fx.push_back(f[0]);
                fy.push_back(f[1]);
            }
            os << ",\"final_flux_x\":";
            putArray(os, fx);
            os << ",\"final_flux_y\":";
            putArray(os, fy);
            os << '}';
        }
        os << ']';
    }
    os << "]}\n";
    return 0;
}

// Binary dump of every material's tables after Model::initializeMaterialTables.
int cmdTables(const std::string& model_path, const std::string& out_path) {
    const Value j = psim_json::parse_file(model_path);
    auto model = buildModel(j);
    const auto [lo, hi] = model->setTemperatureBounds();
    model->initializeMaterialTables(lo, hi);
    std::ofstream os(out_path, std::ios::binary);
    auto wd = [&os](double v) { os.write(reinterpret_cast<const char*>(&v), sizeof v); };
    auto wu = [&os](std::uint64_t v) { os.write(reinterpret_cast<const char*>(&v), sizeof v); };
    // Materials in JSON order (the reference stores them in an unordered_map keyed by name).
    for (const Value& m : j.at("materials").items()) {
        const Material& mat = model->materials_.at(m.at("name").as_string());
        wu(mat.temps_.size());
        for (double t : mat.temps_) { wd(t); }
        for (double v : mat.frequencies_) { wd(v); }
        for (double v : mat.velocities_la_) { wd(v); }
        for (double v : mat.velocities_ta_) { wd(v); }
        for (double v : mat.densities_la_) { wd(v); }
        for (double v : mat.densities_ta_) { wd(v); }
        for (const auto* tabs : { &mat.base_tables_, &mat.emit_tables_, &mat.scatter_tables_ }) {
            for (const auto& td : *tabs) {
                wd(td.cumul_sum);
                for (const auto& e : td.table) {
                    wd(e.first);
                    wd(e.second);
                }
            }
        }
    }
    // Interpreter bounds
    wd(model->interpreter_.lb_);
    wd(model->interpreter_.ub_);
    return 0;
}

// Geometry known answers.  Each input line is one case:
//   I ax1 ay1 ax2 ay2 bx1 by1 bx2 by2     -> Line(a).getIntersection(Line(b)): "1 x y" or "0"
//   C tx1 ty1 tx2 ty2 tx3 ty3 px py       -> Triangle(t).contains(Point p): "0|1"
//   L ax1 ay1 ax2 ay2 px py               -> Line(a).contains(Point p): "0|1"
//   S ax1 ay1 ax2 ay2 bx1 by1 bx2 by2     -> Line(a).contains(Line b) and overlaps: "c o"
//   N tx1 ty1 tx2 ty2 tx3 ty3             -> clockwise flag, area, and the 3 edge normals with the cell's sign
//   R tx1 ty1 tx2 ty2 tx3 ty3 r1 r2       -> Triangle::getRandPoint(r1, r2)
// Values are written with 17 significant digits (round-trip exact).
int cmdGeom(const std::string& in_path, const std::string& out_path) {
    std::ifstream is(in_path);
    std::ofstream os(out_path);
    os << std::setprecision(17);
    std::string line;
    while (std::getline(is, line)) {
        if (line.empty()) { continue; }
        std::istringstream ls(line);
        char op = 0;
        ls >> op;
        std::vector<double> v;
        double x = 0;
        while (ls >> x) { v.push_back(x); }
        try {
            if (op == 'I') {
                const Line a{ { v[0], v[1] }, { v[2], v[3] } };
                const Line b{ { v[4], v[5] }, { v[6], v[7] } };
                const auto poi = a.getIntersection(b);
                if (poi) {
                    os << "1 " << poi->x << ' ' << poi->y << '\n';
                } else {
                    os << "0\n";
                }
            } else if (op == 'C') {
                const Triangle t{ { v[0], v[1] }, { v[2], v[3] }, { v[4], v[5] } };
                os << (t.contains(Point{ v[6], v[7] }) ? 1 : 0) << '\n';
            } else if (op == 'L') {
                const Line a{ { v[0], v[1] }, { v[2], v[3] } };
                os << (a.contains(Point{ v[4], v[5] }) ? 1 : 0) << '\n';
            } else if (op == 'S') {
                const Line a{ { v[0], v[1] }, { v[2], v[3] } };
                const Line b{ { v[4], v[5] }, { v[6], v[7] } };
                os << (a.contains(b) ? 1 : 0) << ' ' << (a.overlaps(b) ? 1 : 0) << '\n';
            } else if (op == 'N') {
                const Triangle t{ { v[0], v[1] }, { v[2], v[3] }, { v[4], v[5] } };
                const int sign = t.isClockwise() ? 1 : -1;
                os << (t.isClockwise() ? 1 : 0) << ' ' << t.area();
                for (const auto& l : t.lines()) {
                    const auto n = l.normal(sign);
                    os << ' ' << n.x << ' ' << n.y;
                }
                os << '\n';
            } else if (op == 'R') {
                const Triangle t{ { v[0], v[1] }, { v[2], v[3] }, { v[4], v[5] } };
                const auto p = t.getRandPoint(v[6], v[7]);
                os << p.x << ' ' << p.y << '\n';
            } else {
                os << "E\n";
            }
        } catch (const std::exception&) { os << "X\n"; }
    }
    return 0;
}

// E->T inversion known answers.  counts.txt holds one line per sensor: "<sensor_index> K c0 c1 ... cK-1".
// eff_energy is the one Model::runSimulation computes for the model (total energy / num_phonons).
int cmdInvert(const std::string& model_path, const std::string& counts_path, const std::string& out_path) {
    const Value j = psim_json::parse_file(model_path);
    auto model = buildModel(j);
    const auto [lo, hi] = model->setTemperatureBounds();
    model->initializeMaterialTables(lo, hi);
    const double total_energy = model->getTotalInitialEnergy();
    const double eff = total_energy / static_cast<double>(model->num_phonons_);
    model->interpreter_.setParams(model->t_eq_, eff);
    std::ifstream is(counts_path);
    std::ofstream os(out_path);
    os << std::setprecision(17);
    os << "eff " << eff << '\n';
    std::string line;
    while (std::getline(is, line)) {
        if (line.empty()) { continue; }
        std::istringstream ls(line);
        std::size_t si = 0;
        std::size_t k = 0;
        ls >> si >> k;
        Sensor& s = model->sensors_.at(si);
        for (std::size_t i = 0; i < k && i < s.inc_energy_.size(); ++i) {
            long long c = 0;
            ls >> c;
            s.inc_energy_[i] = static_cast<int>(c);
            s.inc_flux_[i] = { static_cast<double>(c) * 1000.5, static_cast<double>(-c) * 250.25 };
        }
        const auto m = model->interpreter_.scaleHeatParams(s);
        os << si << ' ' << m.t_steady << ' ' << m.std_t_steady << ' ' << m.x_flux << ' ' << m.std_x_flux << ' '
           << m.y_flux << ' ' << m.std_y_flux;
        for (double t : m.final_temps) { os << ' ' << t; }
        os << '\n';
    }
    return 0;
}

// The assembled model: cells after Model::addCell's neighbour search (Cell::findTransitionSurface)
// and the emitting surfaces after Model::setEmitSurface.  One line per cell, then one per
// sub-surface of its edges in CompositeSurface order (transition surfaces, then emitting ones):
//   c <sensor index> <x1> <y1> <x2> <y2> <x3> <y3> <spec of edge 0> <edge 1> <edge 2>
//   t <cell> <edge> <neighbour cell> <x1> <y1> <x2> <y2>
//   e <cell> <edge> <owning cell> <temp> <duration> <start time> <x1> <y1> <x2> <y2>
// Cells and sensors are numbered by their position in the model (file order).
int cmdTopology(const std::string& model_path, const std::string& out_path) {
    const Value j = psim_json::parse_file(model_path);
    auto model = buildModel(j);
    const Cell* cells = model->cells_.data();
    const Sensor* sensors = model->sensors_.data();
    std::ofstream os(out_path);
    os << std::setprecision(17);
    auto put_line = [&os](const Line& l) { os << ' ' << l.p1.x << ' ' << l.p1.y << ' ' << l.p2.x << ' ' << l.p2.y; };
    for (std::size_t c = 0; c < model->cells_.size(); ++c) {
        const Cell& cell = model->cells_[c];
        os << "c " << (&cell.sensor_ - sensors);
        for (const Point& p : { cell.cell_.p1, cell.cell_.p2, cell.cell_.p3 }) { os << ' ' << p.x << ' ' << p.y; }
        for (const auto& b : cell.boundaries_) { os << ' ' << b.main_surface_.getSpecularity(); }
        os << '\n';
        for (std::size_t e = 0; e < 3; ++e) {
            const CompositeSurface& b = cell.boundaries_[e];
            for (const auto& t : b.transition_sub_surfaces_) {
                os << "t " << c << ' ' << e << ' ' << (&t.cell_ - cells);
                put_line(t.getSurfaceLine());
                os << '\n';
            }
            for (const auto& s : b.emit_sub_surfaces_) {
                os << "e " << c << ' ' << e << ' ' << (&s.cell_ - cells) << ' ' << s.temp_ << ' ' << s.duration_ << ' '
                   << s.start_time_;
                put_line(s.getSurfaceLine());
                os << '\n';
            }
        }
    }
    return 0;
}

// Material::relaxRates(temp, freq, polar) (psim/src/material.cpp:54-62,207-239) of every
// material of the model, in JSON order, on the cases in 'cases_path': float64 triples (T, freq,
// polarization 0 LA / 1 TA).  Writes [material][case][N, U, I] float64.
int cmdRates(const std::string& model_path, const std::string& cases_path, const std::string& out_path) {
    const Value j = psim_json::parse_file(model_path);
    auto model = buildModel(j);
    std::ifstream is(cases_path, std::ios::binary);
    std::vector<double> cases;
    double v = 0.;
    while (is.read(reinterpret_cast<char*>(&v), sizeof v)) { cases.push_back(v); }
    std::ofstream os(out_path, std::ios::binary);
    for (const Value& m : j.at("materials").items()) {
        const Material& mat = model->materials_.at(m.at("name").as_string());
        for (std::size_t i = 0; i + 2 < cases.size(); i += 3) {
            const auto pol = cases[i + 2] == 0. ? Material::Polar::LA : Material::Polar::TA;
            const auto r = mat.relaxRates(cases[i], cases[i + 1], pol);
            for (double x : r) { os.write(reinterpret_cast<const char*>(&x), sizeof x); }
        }
    }
    return 0;
}

}// namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::cerr << "usage: ref_driver run|tables|geom|invert|topology|rates ...\n";
        return 2;
    }
    const std::string cmd = argv[1];
    try {
        if (cmd == "run" && argc >= 4) { return cmdRun(argv[2], argv[3], argc >= 5 ? argv[4] : ""); }
        if (cmd == "tables" && argc >= 4) { return cmdTables(argv[2], argv[3]); }
        if (cmd == "geom" && argc >= 4) { return cmdGeom(argv[2], argv[3]); }
        if (cmd == "invert" && argc >= 5) { return cmdInvert(argv[2], argv[3], argv[4]); }
        if (cmd == "topology" && argc >= 4) { return cmdTopology(argv[2], argv[3]); }
        if (cmd == "rates" && argc >= 5) { return cmdRates(argv[2], argv[3], argv[4]); }
    } catch (const std::exception& e) {
        std::cerr << "ref_driver error: " << e.what() << '\n';
        return 1;
    }
    std::cerr << "bad arguments\n";
    return 2;
}
