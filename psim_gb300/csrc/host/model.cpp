#include "model.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <ctime>
#include <fstream>
#include <iomanip>
#include <map>
#include <sstream>
#include <stdexcept>

#include "json.hpp"

namespace psim {
namespace {

// Model constants (psim/src/model.cpp:11-25)
constexpr double kTempBoundEps = 10.;
constexpr double kPhasorTempBoundEps = kTempBoundEps * 100.;
constexpr double kSsStepsPercent = 0.1;

Seg64 seg(P2 a, P2 b) {
    bool ok = false;
    Seg64 s = make_seg(a, b, &ok);
    if (!ok) {
        std::ostringstream os;
        os << "Cannot create a line using 2 identical points -> Point (" << a.x << ", " << a.y << ") Point (" << b.x
           << ", " << b.y << ')';
        throw std::runtime_error(os.str());
    }
    return s;
}

// Line::contains(Line): psim/src/geometry.cpp:75-86
bool seg_contains(const Seg64& s, double s_len, const Seg64& o, double o_len) {
    if (on_line(s, o.a) && on_line(s, o.b) && s_len >= o_len) {
        const double l1xmin = std::min(s.a.x, s.b.x);
        const double l1xmax = std::max(s.a.x, s.b.x);
        const double l2xmin = std::min(o.a.x, o.b.x);
        const double l2xmax = std::max(o.a.x, o.b.x);
        const double l1ymin = std::min(s.a.y, s.b.y);
        const double l1ymax = std::max(s.a.y, s.b.y);
        const double l2ymin = std::min(o.a.y, o.b.y);
        const double l2ymax = std::max(o.a.y, o.b.y);
        return l1xmax >= l2xmax - kGeoEps && l1xmin <= l2xmin + kGeoEps && l1ymax >= l2ymax - kGeoEps
               && l1ymin <= l2ymin + kGeoEps;
    }
    return false;
}

// Line::overlaps (parallel lines overlapping at more than a point): geometry.cpp:56-72
bool seg_overlaps(const Seg64& s, const Seg64& o) {
    if (coincide(s.a, o.a) && coincide(s.b, o.b)) { return true; }
    auto order = [](P2 p, P2 q) {
        return (p.x + p.y - (q.x + q.y) >= 0.) ? std::pair<P2, P2>{ q, p } : std::pair<P2, P2>{ p, q };
    };
    const auto [pa, pb] = order(s.a, s.b);
    const auto [pc, pd] = order(o.a, o.b);
    if (!(coincide(pd, pa) || coincide(pb, pc))) {
        return (pd.x + pd.y - (pa.x + pa.y) >= 0.) && (pb.x + pb.y - (pc.x + pc.y) >= 0.);
    }
    return false;
}

// Triangle::intersects: geometry.cpp:167-188
bool tri_intersects(const CellRec& t, const CellRec& o) {
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) {
            P2 poi{};
            const Seg64& l1 = t.edge[i].main;
            const Seg64& l2 = o.edge[j].main;
            if (intersection(l1, l2, &poi)) {
                if (!(coincide(poi, l1.a) || coincide(poi, l1.b) || coincide(poi, l2.a) || coincide(poi, l2.b))) { return true; }
            }
        }
    }
    return false;
}

bool tri_contains_tri(const CellRec& t, const CellRec& o) {// geometry.cpp:262-264
    return tri_contains(t.v[0], t.v[1], t.v[2], o.v[0]) || tri_contains(t.v[0], t.v[1], t.v[2], o.v[1])
           || tri_contains(t.v[0], t.v[1], t.v[2], o.v[2]);
}

bool tri_same(const CellRec& t, const CellRec& o) {// Triangle::operator==: geometry.cpp:244-248
    auto has = [](const CellRec& r, P2 p) { return coincide(p, r.v[0]) || coincide(p, r.v[1]) || coincide(p, r.v[2]); };
    return has(o, t.v[0]) && has(o, t.v[1]) && has(o, t.v[2]);
}

std::string tri_text(const CellRec& c) {
    std::ostringstream os;
    os << "Triangle: [Point (" << c.v[0].x << ", " << c.v[0].y << "), Point (" << c.v[1].x << ", " << c.v[1].y
       << "), Point (" << c.v[2].x << ", " << c.v[2].y << ")]";
    return os.str();
}

// libstdc++'s std::reduce / transform_reduce order for random-access ranges (groups of four).
template<typename F> double grouped_sum(std::size_t n, F f) {
    double init = 0.;
    std::size_t i = 0;
    while (n - i >= 4) {
        const double v1 = f(i) + f(i + 1);
        const double v2 = f(i + 2) + f(i + 3);
        const double v3 = v1 + v2;
        init = init + v3;
        i += 4;
    }
    for (; i < n; ++i) { init = init + f(i); }
    return init;
}

}// namespace

HostModel::~HostModel() = default;

std::size_t HostModel::sensor_index(std::uint64_t id) const {
    for (std::size_t i = 0; i < sensors_.size(); ++i) {
        if (sensors_[i].id == id) { return i; }
    }
    throw std::runtime_error("Sensor does not exist");
}

void HostModel::set_type(SimType t, std::size_t interval) {// Model::setSimulationType: model.cpp:46-70
    type_ = t;
    if (t == SimType::Transient || t == SimType::Periodic) {
        start_step_ = static_cast<std::size_t>(static_cast<double>(steps_) - static_cast<double>(steps_) * kSsStepsPercent);
        if (interval == 0) { throw std::runtime_error("Step interval of 0 is invalid for transient and periodic simulations."); }
    }
    if (t == SimType::Transient && t_eq_ == 0) { throw std::runtime_error("Transient simulations must be run using the deviational approach."); }
    if (t == SimType::SteadyState) {
        step_adj_ = static_cast<std::size_t>(static_cast<double>(steps_) - static_cast<double>(steps_) * kSsStepsPercent);
        if (interval > 0) { throw std::runtime_error("Step interval > 0 is invalid for steady-state simulations"); }
    }
    step_interval_ = interval;
    recorded_ = (t == SimType::SteadyState) ? static_cast<std::size_t>(static_cast<double>(steps_) * kSsStepsPercent) : steps_;
}

void HostModel::add_sensor(std::uint64_t id, std::uint32_t material, double t_init) {// model.cpp:81-96
    // the scattering rates take the sensor's temperature: it must be a temperature
    if (!(t_init > 0.) || !std::isfinite(t_init)) {
        throw std::runtime_error("Sensor temperature must be positive and finite: sensor " + std::to_string(id));
    }
    for (const auto& s : sensors_) {
        if (s.id == id) { throw std::runtime_error("Sensor with this ID already exists"); }
    }
    SensorRec s;
    s.id = id;
    s.material = material;
    s.t_init = t_init;
    s.t_steady = t_init;
    sensors_.push_back(s);
}

bool HostModel::edge_accepts(const EdgeRec& e, const Seg64& line, double len) const {// compositeSurface.cpp:66-85
    if (seg_contains(e.main, e.length, line, len)) {
        for (const auto& t : e.trans) {
            if (seg_overlaps(line, t.line)) { throw std::runtime_error("An existing surface conflicts with the location of the incoming surface."); }
        }
        for (const auto& t : e.emits) {
            if (seg_overlaps(line, t.line)) { throw std::runtime_error("An existing surface conflicts with the location of the incoming surface."); }
        }
        return true;
    }
    return false;
}

bool HostModel::add_transition(std::uint32_t cell, const Seg64& line, double len, std::uint32_t target) {// cell.cpp:126-132
    for (auto& e : cells_[cell].edge) {
        if (edge_accepts(e, line, len)) {
            e.trans.push_back(SubSurface{ 0, target, line, len });
            return true;
        }
    }
    return false;
}

// Model::addCell (psim/src/model.cpp:98-113) with Cell::validate and findTransitionSurface
// (psim/src/cell.cpp:21-25, 81-98).  Only cells whose bounding boxes come within a margin
// of the new cell can intersect, contain or share an edge with it, so the pairwise checks
// run over those candidates, in the same (increasing) order as the reference's full scan.
void HostModel::add_cell(P2 p1, P2 p2, P2 p3, std::uint64_t sensor_id, double spec) {
    if (!tri_valid(p1, p2, p3)) {
        std::ostringstream os;
        os << "These 3 points do not allow for a valid triangle -> Triangle: [Point (" << p1.x << ", " << p1.y
           << "), Point (" << p2.x << ", " << p2.y << "), Point (" << p3.x << ", " << p3.y << ")]";
        throw std::runtime_error(os.str());
    }
    CellRec c;
    c.v[0] = p1;
    c.v[1] = p2;
    c.v[2] = p3;
    c.sensor = static_cast<std::uint32_t>(sensor_index(sensor_id));
    c.spec = std::min(std::max(spec, 0.), 1.);
    c.nsign = tri_clockwise(p1, p2, p3) ? 1 : -1;
    for (int e = 0; e < 3; ++e) {
        c.edge[e].main = seg(c.v[e], c.v[(e + 1) % 3]);
        c.edge[e].length = dist2(c.v[e], c.v[(e + 1) % 3]);
    }
    c.area = tri_area(p1, p2, p3);
    c.lo = P2{ std::min({ p1.x, p2.x, p3.x }), std::min({ p1.y, p2.y, p3.y }) };
    c.hi = P2{ std::max({ p1.x, p2.x, p3.x }), std::max({ p1.y, p2.y, p3.y }) };
    sensors_[c.sensor].area += c.area;
    cells_.push_back(c);
    const auto inc = static_cast<std::uint32_t>(cells_.size() - 1);
    const CellRec& ci = cells_[inc];
    const double margin = 1e-6 + 1e-6 * std::max(ci.hi.x - ci.lo.x, ci.hi.y - ci.lo.y);
    std::size_t identical = 0;
    for (std::uint32_t k = 0; k < cells_.size(); ++k) {
        const CellRec& ck = cells_[k];
        if (k != inc) {
            const double m = margin + 1e-6 * std::max(ck.hi.x - ck.lo.x, ck.hi.y - ck.lo.y);
            if (ck.lo.x > ci.hi.x + m || ck.hi.x < ci.lo.x - m || ck.lo.y > ci.hi.y + m || ck.hi.y < ci.lo.y - m) { continue; }
        }
        if (!tri_same(cells_[inc], ck)) {
            if (tri_intersects(cells_[inc], ck)) { throw std::runtime_error("Incoming " + tri_text(cells_[inc]) + "\nintersects\nExisting" + tri_text(ck)); }
            if (tri_contains_tri(cells_[inc], ck)) { throw std::runtime_error(tri_text(ck) + "\nis contained within\n" + tri_text(cells_[inc])); }
            if (tri_contains_tri(ck, cells_[inc])) { throw std::runtime_error(tri_text(cells_[inc]) + "\nis contained within\n" + tri_text(ck)); }
            for (int i = 0; i < 3; ++i) {
                for (int j = 0; j < 3; ++j) {
                    const EdgeRec& l1 = cells_[inc].edge[i];
                    const EdgeRec& l2 = cells_[k].edge[j];
                    if (seg_contains(l1.main, l1.length, l2.main, l2.length)) {
                        const Seg64 line = l2.main;
                        const double len = l2.length;
                        if (!add_transition(inc, line, len, k) || !add_transition(k, line, len, inc)) {
                            throw std::runtime_error("An existing surface conflicts with the location of the incoming surface.");
                        }
                    } else if (seg_contains(l2.main, l2.length, l1.main, l1.length)) {
                        const Seg64 line = l1.main;
                        const double len = l1.length;
                        if (!add_transition(inc, line, len, k) || !add_transition(k, line, len, inc)) {
                            throw std::runtime_error("An existing surface conflicts with the location of the incoming surface.");
                        }
                    }
                }
            }
        } else if (++identical == 2) {
            throw std::runtime_error("Duplicate cell detected.");
        }
    }
}

// Model::setEmitSurface / Cell::setEmitSurface / CompositeSurface::addEmitSurface
// (psim/src/model.cpp:125-138, cell.cpp:29-35, compositeSurface.cpp:17-31)
bool HostModel::set_emit(P2 p1, P2 p2, double temp, double duration, double start) {
    if (!(temp > 0.) || !std::isfinite(temp)) { throw std::runtime_error("Emitting surface temperature must be positive and finite."); }
    if ((start < 0. || start >= sim_time_) || (duration < 0. || duration > sim_time_ - start)) {
        throw std::runtime_error("Transient Surface start_time or duration specifications are invalid.");
    }
    if ((start > 0. || duration < sim_time_) && type_ != SimType::Transient) {
        throw std::runtime_error("Cannot add a transient surface to a non transient simulation.");
    }
    const Seg64 line = seg(p1, p2);
    const double len = dist2(p1, p2);
    for (std::uint32_t c = 0; c < cells_.size(); ++c) {
        for (std::uint32_t e = 0; e < 3; ++e) {
            if (edge_accepts(cells_[c].edge[e], line, len)) {
                const auto id = static_cast<std::uint32_t>(emitters_.size());
                cells_[c].edge[e].emits.push_back(SubSurface{ 1, id, line, len });
                emitters_.push_back(EmitterRec{ c, e, line, len, temp, duration, start });
                return true;
            }
        }
    }
    return false;
}

std::unique_ptr<HostModel> HostModel::from_json(const std::string& path) {// InputManager::deserialize
    std::ifstream probe(path);
    if (!probe.is_open()) { throw std::runtime_error("Error opening file at " + path); }
    probe.close();
    const psim_json::Value j = psim_json::parse_file(path);
    std::unique_ptr<HostModel> m(new HostModel());
    const auto& st = j.at("settings");
    m->steps_ = static_cast<std::size_t>(st.at("num_measurements").as_int());
    m->num_phonons_ = static_cast<std::size_t>(st.at("num_phonons").as_int());
    m->sim_time_ = st.at("sim_time").as_double();
    m->t_eq_ = st.at("t_eq").as_double();
    const auto& ph = st.at("phasor_sim");
    m->phasor_ = ph.kind() == psim_json::Value::Kind::Bool && ph.as_bool();
    if (st.contains("num_runs")) { m->num_runs_ = static_cast<std::size_t>(st.at("num_runs").as_int()); }
    if (m->steps_ == 0) { throw std::runtime_error("num_measurements must be positive"); }
    if (m->num_phonons_ == 0) { throw std::runtime_error("num_phonons must be positive"); }
    if (m->num_runs_ == 0) { throw std::runtime_error("num_runs must be positive"); }
    const auto ty = st.at("sim_type").as_int();
    const SimType t = ty == 1 ? SimType::Periodic : (ty == 2 ? SimType::Transient : SimType::SteadyState);
    m->set_type(t, t == SimType::SteadyState ? 0 : static_cast<std::size_t>(st.at("step_interval").as_int()));
    std::map<std::string, std::uint32_t> by_name;
    for (const auto& mj : j.at("materials").items()) {
        MaterialSpec sp;
        sp.name = mj.at("name").as_string();
        if (by_name.count(sp.name) != 0) { throw std::runtime_error("A duplicate material name was detected."); }
        const auto& d = mj.at("d_data");
        const auto& r = mj.at("r_data");
        for (std::size_t i = 0; i < 3; ++i) {
            sp.la[i] = d.at("la_data").at(i).as_double();
            sp.ta[i] = d.at("ta_data").at(i).as_double();
        }
        sp.w_max_la = d.at("max_freq_la").as_double();
        sp.w_max_ta = d.at("max_freq_ta").as_double();
        sp.b_l = r.at("b_l").as_double();
        sp.b_tn = r.at("b_tn").as_double();
        sp.b_tu = r.at("b_tu").as_double();
        sp.b_i = r.at("b_i").as_double();
        sp.w = r.at("w").as_double();
        // the rates must stay finite and non-negative for every event loop to end
        for (const double b : { sp.b_l, sp.b_tn, sp.b_tu, sp.b_i }) {
            if (!std::isfinite(b) || b < 0.) {
                throw std::runtime_error("Relaxation coefficients must be finite and non-negative: " + sp.name);
            }
        }
        if (!std::isfinite(sp.w)) { throw std::runtime_error("Relaxation cut-off frequency must be finite: " + sp.name); }
        by_name[sp.name] = static_cast<std::uint32_t>(m->mat_specs_.size());
        m->mat_specs_.push_back(sp);
        m->mats_.emplace_back(sp, m->t_eq_ == 0.);
    }
    if (m->mat_specs_.size() > gpu::kMaxMaterialsHost) { throw std::runtime_error("at most 16 materials are supported"); }
    for (const auto& s : j.at("sensors").items()) {
        const auto it = by_name.find(s.at("material").as_string());
        if (it == by_name.end()) { throw std::runtime_error("Sensor material does not exist: " + s.at("material").as_string()); }
        m->add_sensor(static_cast<std::uint64_t>(s.at("id").as_int()), it->second, s.at("t_init").as_double());
    }
    auto pt = [](const psim_json::Value& v) { return P2{ v.at("x").as_double(), v.at("y").as_double() }; };
    for (const auto& c : j.at("cells").items()) {
        const auto& t3 = c.at("triangle");
        m->add_cell(pt(t3.at("p1")), pt(t3.at("p2")), pt(t3.at("p3")), static_cast<std::uint64_t>(c.at("sensorID").as_int()),
                    c.at("specularity").as_double());
    }
    for (const auto& e : j.at("emit_surfaces").items()) {
        if (!m->set_emit(pt(e.at("p1")), pt(e.at("p2")), e.at("temp").as_double(), e.at("duration").as_double(),
                         e.at("start_time").as_double())) {
            throw std::runtime_error("Unable to add emitting surface.");
        }
    }
    if (m->cells_.empty()) { throw std::runtime_error("the model has no cells"); }
    // Tables and the flattened description for the first run (Model::runSimulation builds
    // them from the same initial temperatures at the start of every run).
    const auto [mn, mx] = m->bounds();
    m->build_tables(mn, mx);
    m->initial_eff_ = m->total_energy() / static_cast<double>(m->num_phonons_);
    m->build_desc();
    return m;
}

void HostModel::set_start_temps(const std::vector<double>& temps) {
    if (!temps.empty() && temps.size() != sensors_.size()) { throw std::invalid_argument("one start temperature per sensor"); }
    if (!temps.empty() && t_eq_ == 0.) { throw std::invalid_argument("start temperatures need a deviational model (t_eq > 0)"); }
    for (double t : temps) {
        if (!(t > 0.) || !std::isfinite(t)) { throw std::invalid_argument("start temperatures must be positive and finite"); }
    }
    t_start_ = temps;
}

std::vector<double> HostModel::start_temps() const {
    std::vector<double> out;
    for (std::size_t s = 0; s < sensors_.size(); ++s) { out.push_back(start_temp(s)); }
    return out;
}

// ---------------------------------------------------------------- run orchestration
double HostModel::init_temp(const SensorRec& s) const { return type_ == SimType::SteadyState ? s.t_steady : s.t_init; }

double HostModel::start_temp(std::size_t s) const { return t_start_.empty() ? init_temp(sensors_[s]) : t_start_[s]; }

double HostModel::cell_init_energy(std::size_t c) const {// Cell::getInitEnergy: cell.cpp:38-41
    const SensorRec& s = sensors_[cells_[c].sensor];
    const double e = cells_[c].area * s.heat_cap;
    return (t_eq_ == 0.) ? e : e * std::fabs(start_temp(cells_[c].sensor) - t_eq_);
}

double HostModel::cell_emit_energy(std::size_t c) const {// Cell::getEmitEnergy: cell.cpp:45-63
    double total = 0.;
    const MaterialTables& m = mats_[sensors_[cells_[c].sensor].material];
    for (const auto& e : cells_[c].edge) {
        total += grouped_sum(e.emits.size(), [&](std::size_t i) {
            const EmitterRec& em = emitters_[e.emits[i].target];
            const double en = em.length * em.duration * m.emit(m.temp_index(em.temp)).sum / 4.;
            return (t_eq_ == 0.) ? en : en * std::fabs(em.temp - t_eq_);
        });
    }
    return total;
}

double HostModel::total_energy() const {// Model::getTotalInitialEnergy: model.cpp:196-201
    return grouped_sum(cells_.size(), [&](std::size_t c) { return cell_init_energy(c) + cell_emit_energy(c); });
}

std::pair<double, double> HostModel::bounds() {// Model::setTemperatureBounds: model.cpp:203-218
    double mn = 0.;
    double mx = 0.;
    bool first = true;
    auto take = [&](double t) {
        if (first) {
            mn = mx = t;
            first = false;
        } else {
            mn = std::min(mn, t);
            mx = std::max(mx, t);
        }
    };
    for (const auto& c : cells_) {
        take(init_temp(sensors_[c.sensor]));
        for (const auto& e : c.edge) {
            for (const auto& s : e.emits) { take(emitters_[s.target].temp); }
        }
    }
    const double b = phasor_ ? kPhasorTempBoundEps : kTempBoundEps;
    lb_ = std::max(mn - b, 0.);
    ub_ = mx + b;
    return { mn, mx };
}

void HostModel::build_tables(double lo, double hi) {// Model::initializeMaterialTables: model.cpp:221-227
    for (auto& m : mats_) { m.build_tables(lo, hi); }
    for (auto& s : sensors_) {
        const MaterialTables& m = mats_[s.material];
        s.temp_index = m.temp_index(s.t_init);
        s.heat_cap = m.base(s.temp_index).sum;
    }
}

// Flatten the assembled model into the simulator description (include/psim_gb300.h).
void HostModel::build_desc() {
    gpu::SimDesc d;
    d.steps = steps_;
    d.sim_time = sim_time_;
    d.phasor = phasor_;
    d.sim_type = static_cast<int>(type_);
    d.step_adj = step_adj_;
    d.recorded = recorded_;
    d.full = (t_eq_ == 0.);
    d.n_materials = static_cast<std::uint32_t>(mats_.size());
    for (const auto& m : mats_) {
        d.mat_freq.insert(d.mat_freq.end(), m.freq().begin(), m.freq().end());
        d.mat_vel.insert(d.mat_vel.end(), m.vel(kLA).begin(), m.vel(kLA).end());
        d.mat_vel.insert(d.mat_vel.end(), m.vel(kTA).begin(), m.vel(kTA).end());
        const auto& sp = m.spec();
        const double p[8] = { sp.b_l, sp.b_tn, sp.b_tu, sp.b_i, sp.w, m.width(), sp.w_max_la, sp.w_max_ta };
        d.mat_params.insert(d.mat_params.end(), p, p + 8);
    }
    // Tables: one per (material, kind, temperature index) that a sensor or emitter uses.
    std::map<std::array<std::size_t, 3>, std::uint32_t> index;
    auto table = [&](std::size_t mat, std::size_t kind, std::size_t ti) {
        const std::array<std::size_t, 3> key{ mat, kind, ti };
        const auto it = index.find(key);
        if (it != index.end()) { return it->second; }
        const MaterialTables& m = mats_[mat];
        const CumTable& t = kind == 0 ? m.base(ti) : (kind == 1 ? m.scatter(ti) : m.emit(ti));
        for (std::size_t b = 0; b < kBins; ++b) {
            d.tables.push_back(t.cum[b]);
            d.tables.push_back(t.la_frac[b]);
        }
        const auto id = d.n_tables++;
        index[key] = id;
        return id;
    };
    d.n_sensors = static_cast<std::uint32_t>(sensors_.size());
    for (const auto& s : sensors_) {
        d.sensor_material.push_back(s.material);
        d.sensor_temp.push_back(s.t_init);
        d.sensor_base_table.push_back(table(s.material, 0, s.temp_index));
        d.sensor_scatter_table.push_back(table(s.material, 1, s.temp_index));
    }
    d.n_cells = static_cast<std::uint32_t>(cells_.size());
    d.edge_sub_begin.push_back(0);
    for (const auto& c : cells_) {
        for (int i = 0; i < 3; ++i) {
            d.cell_vertices.push_back(c.v[i].x);
            d.cell_vertices.push_back(c.v[i].y);
        }
        d.cell_sensor.push_back(c.sensor);
        d.cell_spec.push_back(c.spec);
        for (const auto& e : c.edge) {
            for (const auto* list : { &e.trans, &e.emits }) {
                for (const auto& s : *list) {
                    d.sub_kind.push_back(s.kind);
                    d.sub_target.push_back(s.target);
                    d.sub_line.insert(d.sub_line.end(), { s.line.a.x, s.line.a.y, s.line.b.x, s.line.b.y });
                }
            }
            d.edge_sub_begin.push_back(static_cast<std::uint32_t>(d.sub_kind.size()));
        }
    }
    d.n_emitters = static_cast<std::uint32_t>(emitters_.size());
    for (const auto& e : emitters_) {
        d.emit_cell.push_back(e.cell);
        d.emit_edge.push_back(e.edge);
        d.emit_line.insert(d.emit_line.end(), { e.line.a.x, e.line.a.y, e.line.b.x, e.line.b.y });
        d.emit_temp.push_back(e.temp);
        d.emit_start.push_back(e.start);
        d.emit_duration.push_back(e.duration);
        const MaterialTables& m = mats_[sensors_[cells_[e.cell].sensor].material];
        d.emit_table.push_back(table(sensors_[cells_[e.cell].sensor].material, 2, m.temp_index(e.temp)));
    }
    desc_ = std::move(d);
}

gpu::InterpDesc HostModel::interp_desc(double eff) const {
    gpu::InterpDesc d;
    d.n_sensors = static_cast<std::uint32_t>(sensors_.size());
    d.recorded = recorded_;
    d.t_eq = t_eq_;
    d.eff_energy = eff;
    d.lb = lb_;
    d.ub = ub_;
    for (const auto& s : sensors_) {
        d.area.push_back(s.area);
        d.heat_capacity.push_back(s.heat_cap);
        d.init_temp.push_back(start_temp(static_cast<std::size_t>(&s - sensors_.data())));
        d.material.push_back(s.material);
    }
    d.mat_temp_begin.push_back(0);
    for (const auto& m : mats_) {
        for (std::size_t i = 0; i < m.temps().size(); ++i) {
            d.temps.push_back(m.temps()[i]);
            d.energies.push_back(m.base(i).sum);
        }
        d.mat_temp_begin.push_back(d.temps.size());
    }
    return d;
}

// Model::runSimulation (psim/src/model.cpp:141-182) with the GPU simulator.  After each run the
// reference's stability check stores every sensor's mean temperature as its steady temperature
// (model.cpp:250-272, sensorController.cpp:57-62) and the energy per phonon is recomputed from
// it before the results are scaled (model.cpp:171); with MAX_ITERS = 1 no re-run follows.
void HostModel::begin_runs() {
    run_t0_ = std::chrono::steady_clock::now();
    if (stop_on_ && (num_runs_ != 1 || type_ == SimType::SteadyState)) {
        throw std::invalid_argument("stopping at steady state needs a single-run periodic or transient model");
    }
    runs_.clear();
    recorded_ = desc_.recorded;
}

void HostModel::prepare_run(std::size_t run) {
    const auto [mn, mx] = bounds();
    build_tables(mn, mx);
    eff_energy_ = total_energy() / static_cast<double>(num_phonons_);
    const bool fresh = !engine_;
    if (fresh) { engine_ = std::make_unique<gpu::Engine>(desc_); }
    engine_->reset();
    if (fresh) { engine_->add_h2d(engine_->model_bytes()); }
    const std::vector<double> cell_energy = cell_energies();
    const std::vector<double> emit_energy = emit_energies();
    const std::vector<double> sensor_t0 = sensor_init_temps();
    const std::uint64_t run_seed = seed_ * 0x9E3779B97F4A7C15ULL + run * 0xD1B54A32D192ED03ULL + 1;
    engine_->init_builders(t_eq_, eff_energy_, cell_energy.data(), emit_energy.data(), sensor_t0.data(), run_seed);
    engine_->set_steady_stop(stop_on_, stop_crit_, stop_check_);
    engine_->set_grid(grid_);
}

void HostModel::finish_run() {
    recorded_ = std::min<std::size_t>(desc_.recorded, engine_->steps_run());
    if (type_ == SimType::SteadyState) {
        std::vector<double> finals(sensors_.size());
        engine_->final_temps(interp_desc(eff_energy_), start_step_, finals.data());
        for (std::size_t s = 0; s < sensors_.size(); ++s) { sensors_[s].t_steady = finals[s]; }
        eff_energy_ = total_energy() / static_cast<double>(num_phonons_);
    }
    std::vector<Measurement> ms(sensors_.size());
    std::vector<double> temps(sensors_.size() * recorded_);
    std::vector<double> fluxes(sensors_.size() * recorded_ * 2);
    std::vector<double> stats(sensors_.size() * 6);
    engine_->interpret(interp_desc(eff_energy_), temps.data(), fluxes.data(), stats.data());
    for (std::size_t s = 0; s < sensors_.size(); ++s) {
        Measurement& m = ms[s];
        m.id = sensors_[s].id;
        std::copy(stats.begin() + static_cast<std::ptrdiff_t>(6 * s), stats.begin() + static_cast<std::ptrdiff_t>(6 * s + 6), m.stats.begin());
        m.temps.assign(temps.begin() + static_cast<std::ptrdiff_t>(s * recorded_), temps.begin() + static_cast<std::ptrdiff_t>((s + 1) * recorded_));
        m.fluxes.assign(fluxes.begin() + static_cast<std::ptrdiff_t>(2 * s * recorded_), fluxes.begin() + static_cast<std::ptrdiff_t>(2 * (s + 1) * recorded_));
    }
    std::sort(ms.begin(), ms.end(), [](const Measurement& a, const Measurement& b) { return a.id < b.id; });
    runs_.push_back(std::move(ms));
    for (auto& s : sensors_) { s.t_steady = s.t_init; }// Model::reset(true) before the next run
}

void HostModel::end_runs() { last_seconds_ = std::chrono::duration<double>(std::chrono::steady_clock::now() - run_t0_).count(); }

void HostModel::run() {
    begin_runs();
    for (std::size_t run = 0; run < num_runs_; ++run) {
        prepare_run(run);
        engine_->run(precision_, stream_);
        finish_run();
    }
    end_runs();
}

std::vector<double> HostModel::cell_energies() const {
    std::vector<double> out(cells_.size());
    for (std::size_t c = 0; c < cells_.size(); ++c) { out[c] = cell_init_energy(c); }
    return out;
}

std::vector<double> HostModel::emit_energies() const {// ModelSimulator::initPhononBuilders: modelSimulator.cpp:66-70
    std::vector<double> out(emitters_.size());
    for (std::size_t e = 0; e < emitters_.size(); ++e) {
        const EmitterRec& em = emitters_[e];
        const MaterialTables& m = mats_[sensors_[cells_[em.cell].sensor].material];
        const double factor = m.emit(m.temp_index(em.temp)).sum * em.duration * em.length / 4.;
        out[e] = (t_eq_ == 0.) ? factor : factor * std::fabs(t_eq_ - em.temp);
    }
    return out;
}

std::vector<double> HostModel::sensor_init_temps() const {
    std::vector<double> out(sensors_.size());
    for (std::size_t s = 0; s < sensors_.size(); ++s) { out[s] = start_temp(s); }
    return out;
}

std::vector<std::array<double, 6>> HostModel::averaged() const {// OutputManager::calculateAverages
    std::vector<std::array<double, 6>> out(sensors_.size(), std::array<double, 6>{});
    for (const auto& r : runs_) {
        for (std::size_t i = 0; i < r.size() && i < out.size(); ++i) {
            for (int k = 0; k < 6; ++k) { out[i][k] += r[i].stats[k]; }
        }
    }
    const auto n = static_cast<double>(runs_.size());
    for (auto& o : out) {
        for (auto& v : o) { v /= n; }
    }
    return out;
}

// OutputManager::addMeasurement for every sensor of every run (psim/src/outputManager.cpp:116-118),
// from statistics made elsewhere.
void HostModel::set_measurements(const double* stats, std::size_t runs) {
    const std::size_t S = sensors_.size();
    std::vector<std::vector<Measurement>> r(runs, std::vector<Measurement>(S));
    for (std::size_t k = 0; k < runs; ++k) {
        for (std::size_t s = 0; s < S; ++s) {
            r[k][s].id = s;
            std::copy(stats + (k * S + s) * 6, stats + (k * S + s) * 6 + 6, r[k][s].stats.begin());
        }
    }
    runs_ = std::move(r);
}

void HostModel::tallies(std::int64_t* energy, double* flux) const {
    if (!engine_) { throw std::runtime_error("the model has not been run"); }
    engine_->tallies(energy, flux, recorded_);
}

const gpu::RunCounters& HostModel::counters() const {
    static const gpu::RunCounters empty{};
    return engine_ ? engine_->counters() : empty;
}

// OutputManager::exportResults (psim/src/outputManager.cpp:13-38, 72-114).  The per_ table
// averages each step over the runs' per-step series (the reference's calculateAverages does
// not carry the series, psim/src/outputManager.cpp:40-70, so its periodic writer reads an
// empty vector); for one run the numbers are the run's own.
void HostModel::export_results(const std::string& json_path, double seconds) const {
    std::string dir;
    std::string name = json_path;
    const auto slash = json_path.find_last_of('/');
    if (slash != std::string::npos) {
        dir = json_path.substr(0, slash + 1);
        name = json_path.substr(slash + 1);
    }
    const bool ss = type_ == SimType::SteadyState;
    std::string stem = name;
    const auto dot = stem.find_last_of('.');
    if (dot != std::string::npos && dot != 0) { stem = stem.substr(0, dot); }
    const std::string out_path = dir + (ss ? "ss_" : "per_") + stem + ".txt";
    std::ofstream out(out_path, std::ios_base::trunc);
    if (!out.is_open()) { throw std::runtime_error("cannot write " + out_path); }
    const auto now = std::chrono::system_clock::to_time_t(std::chrono::system_clock::now());
    std::tm tm_time{};
    localtime_r(&now, &tm_time);
    std::ostringstream when;
    when << std::put_time(&tm_time, "%Y-%m-%d %X");
    out << (ss ? "Steady State" : "Periodic") << " Results from " << std::quoted(name) << " @ " << when.str()
        << " - Time Taken " << seconds << "[s] over " << num_runs_ << " runs\n";
    if (ss) {
        for (const auto& a : averaged()) {
            out << a[0] << ' ' << a[1] << ' ' << a[2] << ' ' << a[3] << ' ' << a[4] << ' ' << a[5] << '\n';
        }
        return;
    }
    const std::size_t S = sensors_.size();
    const std::size_t K = recorded_;
    for (const auto& r : runs_) {
        for (const auto& m : r) {
            if (m.temps.size() < K || m.fluxes.size() < 2 * K) { throw std::runtime_error("the runs carry no per-step series to export"); }
        }
    }
    std::vector<double> t(S * K, 0.);
    std::vector<double> f(S * K * 2, 0.);
    for (const auto& r : runs_) {
        for (std::size_t s = 0; s < S; ++s) {
            for (std::size_t k = 0; k < K; ++k) {
                t[s * K + k] += r[s].temps[k];
                f[(s * K + k) * 2] += r[s].fluxes[2 * k];
                f[(s * K + k) * 2 + 1] += r[s].fluxes[2 * k + 1];
            }
        }
    }
    const auto runs = static_cast<double>(runs_.size());
    for (auto& v : t) { v /= runs; }
    for (auto& v : f) { v /= runs; }
    const std::size_t iv = step_interval_;
    for (std::size_t step = 0; iv > 0 && step + iv <= K; step += iv) {
        out << step + iv / 2 << '\n' << S << '\n';
        for (std::size_t s = 0; s < S; ++s) {
            double ts = 0.;
            for (std::size_t k = step; k < step + iv; ++k) { ts += t[s * K + k]; }
            const double temp = ts / static_cast<double>(iv);
            const double fx = grouped_sum(iv, [&](std::size_t i) { return f[(s * K + step + i) * 2]; }) / static_cast<double>(iv);
            const double fy = grouped_sum(iv, [&](std::size_t i) { return f[(s * K + step + i) * 2 + 1]; }) / static_cast<double>(iv);
            out << temp << ' ' << fx << ' ' << fy << '\n';
        }
    }
}

}// namespace psim
