// psim CPU oracle: a restatement of the reference psim Monte Carlo phonon
// simulation, used ONLY as a test oracle and as the timed CPU baseline.
// Nothing in the product (psim_gb300/) links, imports or runs this file.
//
// It restates, in its own structure, the algorithms of the reference files
// cited per function below (paths relative to the reference project).  It draws
// random numbers exactly as the reference does (a std::mt19937 per thread fed
// through std::uniform_real_distribution(0, nextafter(1, 2)),
// psim/include/psim/utils.h:16-21, and a std::random_device-shaped engine for the
// phonon shuffle, psim/src/modelSimulator.cpp:239) and consumes them in the same
// order, so with one thread and the same PSIM seed it reproduces the reference
// built with oracle/ref_recipe/seed_shim.h bit for bit.  With several threads the
// phonons are split across threads, each thread with its own engine; the result
// is then the same process with a different random stream (used for timing).
//
// Floating-point expressions keep the reference's operation order; compile with
// -ffp-contract=off so no fused multiply-add changes a rounding.
#include <algorithm>
#include <array>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <limits>
#include <map>
#include <memory>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../psim_gb300/csrc/host/json.hpp"

namespace oracle {

// ---------------------------------------------------------------- constants
// psim/include/psim/utils.h:10-11
constexpr double GEOEPS = std::numeric_limits<double>::epsilon() * 1E9;
constexpr double PI = 3.1415926535897932384626433832795028841971693993751058209749445923;
// psim/src/material.cpp:13-14, psim/include/psim/material.h:14
constexpr double HBAR = 1.054517e-34;
constexpr double BOLTZ = 1.38065e-23;
constexpr std::size_t NBINS = 1000;
// psim/src/modelSimulator.cpp:17-25
constexpr double SCALING_FACTOR = 1e9;
constexpr std::size_t PHONON_CUTOFF = 5'000'000;
constexpr std::size_t BUILDER_MAX_PHONONS = 100'000;
constexpr double VELOCITY_EPS = 0.01;
constexpr std::size_t MAX_COLLISIONS = 100;
// psim/src/model.cpp:11-25
constexpr double TEMP_BOUND_EPS = 10.;
constexpr double PHASOR_TEMP_BOUND_EPS = TEMP_BOUND_EPS * 100.;
constexpr double SS_STEPS_PERCENT = 0.1;
constexpr float TEMP_INTERVAL = .1F;
// psim/src/sensorInterpreter.cpp:9-10
constexpr double INV_EPS = .0001;
constexpr std::size_t INV_MAX_ITERS = 40;

enum class SimType { SteadyState = 0, Periodic = 1, Transient = 2 };
enum Polar : int { LA = 0, TA = 1 };

// ---------------------------------------------------------------- random numbers
// One engine per thread; thread 0 is seeded with the run seed exactly like the
// reference shim, other threads with seed + thread index.
struct Rng {
    std::mt19937 gen;
    explicit Rng(std::uint32_t seed) : gen(seed) {}
    double u() {
        std::uniform_real_distribution<double> dist(0., std::nextafter(1., 2.));
        return dist(gen);
    }
};

// Uniform random bit generator with std::random_device's range, used for the
// phonon shuffle (the shim's seeded stand-in for std::random_device).
struct ShuffleDevice {
    using result_type = unsigned int;
    std::mt19937* engine;
    static constexpr result_type min() { return 0U; }
    static constexpr result_type max() { return UINT_MAX; }
    result_type operator()() { return static_cast<result_type>((*engine)()); }
};

// ---------------------------------------------------------------- geometry (psim/src/geometry.cpp)
struct Pt {
    double x, y;
};

// Point equality within GEOEPS: geometry.cpp:34-39
inline bool same(const Pt& a, const Pt& b) {
    const double dx = a.x - b.x;
    const double dy = a.y - b.y;
    return dx * dx + dy * dy < GEOEPS * GEOEPS;
}

inline double cross(const Pt& a, const Pt& b) { return a.x * b.y - b.x * a.y; }// geometry.cpp:310-312
inline double dot(const Pt& a, const Pt& b) { return a.x * b.x + a.y * b.y; }  // geometry.cpp:314-316
inline bool nearly(double a, double b) { return std::abs(a - b) < GEOEPS; }    // utils.h:67-69
// Slope, 0 for a vertical line: geometry.cpp:325-327
inline double slopeOf(const Pt& a, const Pt& b) { return nearly(a.x, b.x) ? 0. : (a.y - b.y) / (a.x - b.x); }

struct Seg {
    Pt a, b;
    double m, c;// slope and intercept
    Pt lo, hi;  // bounding box
    double len;
};

// Line constructor: geometry.cpp:45-53 (+ findBoundingBox :271-282, getLineLength :318-322)
inline Seg makeSeg(Pt a, Pt b) {
    Seg s{};
    s.a = a;
    s.b = b;
    s.m = slopeOf(a, b);
    s.c = a.y - s.m * a.x;
    double lx = a.x;
    double ly = a.y;
    double hx = b.x;
    double hy = b.y;
    if (b.x <= a.x) { std::swap(lx, hx); }
    if (b.y <= a.y) { std::swap(ly, hy); }
    s.lo = { lx, ly };
    s.hi = { hx, hy };
    s.len = std::sqrt((b.x - a.x) * (b.x - a.x) + (b.y - a.y) * (b.y - a.y));
    if (same(a, b)) { throw std::runtime_error("Cannot create a line using 2 identical points"); }
    return s;
}

inline bool onLine(const Seg& s, const Pt& p) {// isPointOnLine: geometry.cpp:295-298
    return std::fabs(cross({ s.b.x - s.a.x, s.b.y - s.a.y }, { p.x - s.a.x, p.y - s.a.y })) < GEOEPS;
}
inline bool rightOf(const Seg& s, const Pt& p) {// isPointRightOfLine: geometry.cpp:300-303
    return cross({ s.b.x - s.a.x, s.b.y - s.a.y }, { p.x - s.a.x, p.y - s.a.y }) < 0.;
}
inline bool crossesLine(const Seg& l1, const Seg& l2) {// doesSegmentCrossLine: geometry.cpp:305-308
    return onLine(l1, l2.a) || onLine(l1, l2.b) || ((rightOf(l1, l2.a) ^ rightOf(l1, l2.b)) != 0);
}
inline bool boxesMeet(const Seg& s, const Seg& o) {// boxesIntersect: geometry.cpp:284-292
    return s.lo.x <= o.hi.x - GEOEPS && s.hi.x >= o.lo.x + GEOEPS && s.lo.y <= o.hi.y - GEOEPS
           && s.hi.y >= o.lo.y + GEOEPS;
}
inline bool segIntersects(const Seg& s, const Seg& o) {// Line::intersects: geometry.cpp:92-95
    return boxesMeet(s, o) && crossesLine(s, o) && crossesLine(o, s);
}

// Line::getIntersection: geometry.cpp:104-138
inline bool segIntersection(const Seg& s, const Seg& o, Pt& poi) {
    if (!segIntersects(s, o)) { return false; }
    auto eq = [](double a, double b) { return std::fabs(a - b) <= ((std::fabs(a) < std::fabs(b) ? std::fabs(b) : std::fabs(a)) * GEOEPS); };
    auto vert = [&](const Pt& p1, const Pt& p3, const Pt& p4) {
        if (eq(p3.x, p4.x)) { return false; }
        const double m = slopeOf(p3, p4);
        const double c = p3.y - m * p3.x;
        poi = { p1.x, m * p1.x + c };
        return true;
    };
    if (eq(s.a.x, s.b.x)) { return vert(s.a, o.a, o.b); }
    if (eq(o.a.x, o.b.x)) { return vert(o.a, s.a, s.b); }
    if (eq(s.m, o.m)) { return false; }
    const double x = (o.c - s.c) / (s.m - o.m);
    poi = { x, s.m * x + s.c };
    return true;
}

// Line::contains(Line): geometry.cpp:75-86
inline bool segContains(const Seg& s, const Seg& o) {
    if (onLine(s, o.a) && onLine(s, o.b) && s.len >= o.len) {
        const double l1xmin = std::min(s.a.x, s.b.x);
        const double l1xmax = std::max(s.a.x, s.b.x);
        const double l2xmin = std::min(o.a.x, o.b.x);
        const double l2xmax = std::max(o.a.x, o.b.x);
        const double l1ymin = std::min(s.a.y, s.b.y);
        const double l1ymax = std::max(s.a.y, s.b.y);
        const double l2ymin = std::min(o.a.y, o.b.y);
        const double l2ymax = std::max(o.a.y, o.b.y);
        return l1xmax >= l2xmax - GEOEPS && l1xmin <= l2xmin + GEOEPS && l1ymax >= l2ymax - GEOEPS
               && l1ymin <= l2ymin + GEOEPS;
    }
    return false;
}

// Line::overlaps (for parallel lines): geometry.cpp:56-72
inline bool segOverlaps(const Seg& s, const Seg& o) {
    if (same(s.a, o.a) && same(s.b, o.b)) { return true; }
    auto order = [](const Pt& p, const Pt& q) {
        return (p.x + p.y - (q.x + q.y) >= 0.) ? std::pair<Pt, Pt>{ q, p } : std::pair<Pt, Pt>{ p, q };
    };
    const auto [pa, pb] = order(s.a, s.b);
    const auto [pc, pd] = order(o.a, o.b);
    if (!(same(pd, pa) || same(pb, pc))) {
        if ((pd.x + pd.y - (pa.x + pa.y) >= 0.) && (pb.x + pb.y - (pc.x + pc.y) >= 0.)) { return true; }
    }
    return false;
}

struct Vec {
    double x, y;
};
// Line::normal: geometry.cpp:97-100
inline Vec segNormal(const Seg& s, int sign) {
    sign = (sign >= 0) ? 1 : -1;
    return { sign * (s.b.y - s.a.y) / s.len, -sign * (s.b.x - s.a.x) / s.len };
}

struct Tri {
    Pt p1, p2, p3;
};

inline std::array<Seg, 3> triLines(const Tri& t) { return { makeSeg(t.p1, t.p2), makeSeg(t.p2, t.p3), makeSeg(t.p3, t.p1) }; }

// Triangle constructor validity: geometry.cpp:150-158
inline bool triValid(const Tri& t) {
    const double s12 = std::fabs(slopeOf(t.p1, t.p2));
    const double s23 = std::fabs(slopeOf(t.p2, t.p3));
    const double s31 = std::fabs(slopeOf(t.p3, t.p1));
    return !((s12 == s23 && s23 == s31) || same(t.p1, t.p2) || same(t.p2, t.p3) || same(t.p3, t.p1));
}

// Triangle::area (Heron): geometry.cpp:250-257
inline double triArea(const Tri& t) {
    const auto l = triLines(t);
    const double a = l[0].len;
    const double b = l[1].len;
    const double c = l[2].len;
    const double p = (a + b + c) / 2.;
    return std::sqrt(p * (p - a) * (p - b) * (p - c));
}

// Triangle::isClockwise: geometry.cpp:217-222
inline bool triClockwise(const Tri& t) {
    const double ax = t.p2.x - t.p1.x;
    const double ay = t.p2.y + t.p1.y;
    const double bx = t.p3.x - t.p2.x;
    const double by = t.p3.y + t.p2.y;
    const double cx = t.p1.x - t.p3.x;
    const double cy = t.p1.y + t.p3.y;
    return ax * ay + bx * by + cx * cy >= 0.;
}

// Triangle::contains(Point), including its area test as written: geometry.cpp:190-215
inline bool triContains(const Tri& t, const Pt& p) {
    auto area = [](Pt a, Pt b, Pt c) {
        const Tri s{ a, b, c };
        if (!triValid(s)) { return 0.; }
        return triArea(s);
    };
    const Pt bp1{ t.p2.x - t.p1.x, t.p2.y - t.p1.y };
    const Pt bp2{ t.p3.x - t.p1.x, t.p3.y - t.p1.y };
    const double d00 = dot(bp1, bp1);
    const double d01 = dot(bp1, bp2);
    const double d11 = dot(bp2, bp2);
    const double denom = d00 * d11 - d01 * d01;
    const Pt bp3{ p.x - t.p1.x, p.y - t.p1.y };
    const double d20 = dot(bp3, bp1);
    const double d21 = dot(bp3, bp2);
    const double u = (d11 * d20 - d01 * d21) / denom;
    const double v = (d00 * d21 - d01 * d20) / denom;
    if (u >= GEOEPS && u <= 1. + GEOEPS && v >= GEOEPS && v <= 1. + GEOEPS && u + v <= 1. + GEOEPS) {
        if ((triArea(t) - area(p, t.p2, t.p3) + area(t.p1, p, t.p3) + area(t.p1, t.p2, p)) < GEOEPS) { return true; }
    }
    return false;
}

// Triangle::intersects: geometry.cpp:167-188
inline bool triIntersects(const Tri& t, const Tri& o) {
    const auto a = triLines(t);
    const auto b = triLines(o);
    for (const auto& l1 : a) {
        for (const auto& l2 : b) {
            Pt poi{};
            if (segIntersection(l1, l2, poi)) {
                if (!(same(poi, l1.a) || same(poi, l1.b) || same(poi, l2.a) || same(poi, l2.b))) { return true; }
            }
        }
    }
    return false;
}

inline bool triContainsTri(const Tri& t, const Tri& o) {// geometry.cpp:262-264
    return triContains(t, o.p1) || triContains(t, o.p2) || triContains(t, o.p3);
}

inline bool triSame(const Tri& t, const Tri& o) {// Triangle::operator==: geometry.cpp:244-248
    auto has = [](const Tri& r, const Pt& p) { return same(p, r.p1) || same(p, r.p2) || same(p, r.p3); };
    return has(o, t.p1) && has(o, t.p2) && has(o, t.p3);
}

// Triangle::getRandPoint: geometry.cpp:234-242
inline Pt triRandPoint(const Tri& t, double r1, double r2) {
    if (r1 + r2 > 1.) {
        r1 = 1 - r1;
        r2 = 1 - r2;
    }
    return { t.p1.x + (t.p2.x - t.p1.x) * r1 + (t.p3.x - t.p1.x) * r2,
        t.p1.y + (t.p2.y - t.p1.y) * r1 + (t.p3.y - t.p1.y) * r2 };
}

// Line::getRandPoint: geometry.cpp:140-143
inline Pt segRandPoint(const Seg& s, double r1) {
    const double r2 = 1. - r1;
    return { s.a.x * r1 + s.b.x * r2, s.a.y * r1 + s.b.y * r2 };
}

// ---------------------------------------------------------------- material (psim/src/material.cpp)
using Arr = std::array<double, NBINS>;
struct Table {
    std::array<double, NBINS> cum{};
    std::array<double, NBINS> la_frac{};
    double sum{ 0. };
};

struct Material {
    std::string name;
    std::array<double, 3> la{}, ta{};
    double w_max_la{}, w_max_ta{};
    double b_l{}, b_tn{}, b_tu{}, b_i{}, w{};
    double width{};
    bool full{ false };
    Arr freq{}, dens_la{}, dens_ta{}, vel_la{}, vel_ta{};
    std::vector<double> temps;
    std::vector<Table> base, emit, scat;

    // getK / getGv: material.cpp:86-95
    static double waveNumber(double f, const std::array<double, 3>& c) {
        const double d = std::pow(c[1], 2) - 4. * c[0] * (c[2] - f);
        const double a = (-c[1] - std::sqrt(d)) / (2. * c[0]);
        const double b = (-c[1] + std::sqrt(d)) / (2. * c[0]);
        return (a < b) ? a : b;
    }
    static double groupVel(double f, const std::array<double, 3>& c) { return 2. * c[0] * waveNumber(f, c) + c[1]; }

    // Material constructor: material.cpp:20-51
    void build() {
        width = std::max(w_max_la, w_max_ta) / NBINS;
        for (std::size_t i = 0; i < NBINS; ++i) { freq[i] = static_cast<double>(static_cast<int>(2 * i + 1)) * width / 2.; }
        for (std::size_t i = 0; i < NBINS; ++i) {
            const double la_gv = groupVel(freq[i], la);
            vel_la[i] = la_gv;
            dens_la[i] = std::pow(waveNumber(freq[i], la), 2) / 2. / std::pow(PI, 2) / la_gv;
            const double ta_gv = groupVel(freq[i], ta);
            if (!std::isnan(ta_gv)) {
                vel_ta[i] = ta_gv;
                dens_ta[i] = std::pow(waveNumber(freq[i], ta), 2) / std::pow(PI, 2) / ta_gv;
            }
        }
    }

    // tauNInv / tauUInv / tauIInv: material.cpp:207-239
    double rateN(double T, double f, int pol) const {
        if (pol == LA) { return b_l * f * f * std::pow(T, 3); }
        return (f < w) ? b_tn * f * std::pow(T, 4) : 0.;
    }
    double rateU(double T, double f, int pol) const {
        if (pol == LA) { return b_l * f * f * std::pow(T, 3); }
        return (f >= w) ? b_tu * f * f / std::sinh(HBAR * f / (T * BOLTZ)) : 0.;
    }
    double rateI(double f) const { return b_i * std::pow(f, 4); }
    std::array<double, 3> rates(double T, double f, int pol) const { return { rateN(T, f, pol), rateU(T, f, pol), rateI(f) }; }

    // phononDist: material.cpp:184-204
    Arr dist(double T, int pol) const {
        Arr out{};
        const Arr& dens = (pol == LA) ? dens_la : dens_ta;
        const double k = HBAR / (BOLTZ * T);
        for (std::size_t i = 0; i < NBINS; ++i) {
            const double f = freq[i];
            double d = f * HBAR / std::expm1(k * f) * width * dens[i];
            if (!full) { d *= k * f * std::exp(k * f) / (std::expm1(k * f) * T); }
            out[i] = d;
        }
        return out;
    }

    static double plainSum(const Arr& a) {// std::accumulate: sequential left fold
        double s = 0.;
        for (double v : a) { s += v; }
        return s;
    }

    // buildCumulDist: material.cpp:170-179
    static Table cumulative(const Arr& t1, const Arr& t2) {
        Table t;
        const double total = plainSum(t1) + plainSum(t2);
        t.cum[0] = (t1[0] + t2[0]) / total;
        t.la_frac[0] = t1[0] / (t1[0] + t2[0]);
        for (std::size_t i = 1; i < NBINS; ++i) {
            t.cum[i] = t.cum[i - 1] + (t1[i] + t2[i]) / total;
            t.la_frac[i] = t1[i] / (t1[i] + t2[i]);
        }
        return t;
    }

    // initializeTables: material.cpp:101-123 (+ cumulDistEmit/Scatter :140-168)
    void initTables(double lo, double hi) {
        const auto n = static_cast<std::size_t>((hi - lo) / static_cast<double>(TEMP_INTERVAL));
        temps.assign(n, 0.);
        double k = -1.;
        for (auto& t : temps) { t = lo + static_cast<double>(TEMP_INTERVAL) * (k += 1); }
        temps.push_back(hi);
        base.clear();
        emit.clear();
        scat.clear();
        for (const double T : temps) {
            const Arr la_d = dist(T, LA);
            const Arr ta_d = dist(T, TA);
            Table b = cumulative(la_d, ta_d);
            b.sum = plainSum(la_d) + plainSum(ta_d);
            base.push_back(b);
            Arr la_e = la_d;
            Arr ta_e = ta_d;
            for (std::size_t i = 0; i < NBINS; ++i) {
                la_e[i] = la_e[i] * vel_la[i];
                ta_e[i] = ta_e[i] * vel_ta[i];
            }
            Table e = cumulative(la_e, ta_e);
            e.sum = plainSum(la_e) + plainSum(ta_e);
            emit.push_back(e);
            Arr la_s = la_d;
            Arr ta_s = ta_d;
            for (std::size_t i = 0; i < NBINS; ++i) {
                const auto rl = rates(T, freq[i], LA);
                la_s[i] = la_s[i] * (((0. + rl[0]) + rl[1]) + rl[2]);
                const auto rt = rates(T, freq[i], TA);
                ta_s[i] = ta_s[i] * (((0. + rt[0]) + rt[1]) + rt[2]);
            }
            Table s = cumulative(la_s, ta_s);
            s.sum = plainSum(la_s) + plainSum(ta_s);
            scat.push_back(s);
        }
    }

    // getTempIndex: material.cpp:241-246
    std::size_t tempIndex(double T) const {
        const auto idx = static_cast<std::size_t>(std::lower_bound(temps.begin(), temps.end(), T) - temps.begin());
        return std::min(idx, temps.size() - 1);
    }

    // getFreq: material.cpp:77-80
    double sampleFreq(std::size_t bin, Rng& r) const {
        return full ? freq[bin] : freq[bin] + (2. * r.u() - 1.) * width / 2.;
    }
    double vel(std::size_t bin, int pol) const { return pol == LA ? vel_la[bin] : vel_ta[bin]; }
};

// freqIndex: material.cpp:64-75
inline std::pair<std::size_t, int> sampleBin(const Table& t, Rng& r) {
    std::size_t lo = 0;
    std::size_t hi = NBINS - 1;
    std::size_t mid = lo + (hi - lo) / 2;
    const double u = r.u();
    while (hi - lo > 1) {
        if (u < t.cum[mid]) {
            hi = mid;
        } else {
            lo = mid;
        }
        mid = (lo + hi) / 2;
    }
    return { hi, (r.u() <= t.la_frac[hi]) ? LA : TA };
}

// ---------------------------------------------------------------- model structures
struct Sensor {
    std::size_t id{};
    std::size_t mat{};
    double t_init{};
    double t_steady{};
    double area{ 0. };
    double heat_cap{ 0. };
    const Table* base{ nullptr };
    const Table* scat{ nullptr };
    std::vector<double> steady_temps;// transient only
    std::vector<const Table*> scat_steps;
    std::vector<double> heat_caps;
    std::vector<int> energy;
    std::vector<std::array<double, 2>> flux;
};

struct Surface {// Surface / TransitionSurface / EmitSurface: psim/src/surface.cpp
    Seg line;
    Vec normal;
    double spec{ 0. };
    std::size_t target{ 0 };// transition: neighbour cell
    // emit surfaces
    double temp{ 0. }, duration{ 0. }, start{ 0. };
    const Table* table{ nullptr };
};

struct Edge {// CompositeSurface: psim/src/compositeSurface.cpp
    Surface main;
    std::vector<Surface> trans;
    std::vector<Surface> emits;
};

struct Cell {
    Tri tri;
    std::size_t sensor{};
    double area{};
    int nsign{ 1 };
    std::array<Edge, 3> edges;
};

struct Phonon {// psim/include/psim/phonon.h:90-104
    signed char sign{ 1 };
    double lifetime{ 0. };
    std::size_t lifestep{ 0 };
    double px{ 0. }, py{ 0. }, dx{ 0. }, dy{ 0. };
    std::size_t bin{ 0 };
    double freq{ 0. }, vel{ 0. };
    int pol{ LA };
    long cell{ -1 };// -1 = absorbed (outside any cell)
};

struct Measurement {
    std::size_t id{};
    double t{}, st{}, fx{}, sfx{}, fy{}, sfy{};
    std::vector<double> temps;
    std::vector<std::array<double, 2>> fluxes;
};

struct Builder {// the three builder kinds of psim/include/psim/phononBuilder.h
    int kind{ 0 };// 0 cell origin, 1 surface origin, 2 phasor
    std::vector<std::pair<std::size_t, std::size_t>> stack;// cell origin: (cell, remaining), used LIFO
    std::size_t cell{ 0 }, edge{ 0 }, emit{ 0 }, remaining{ 0 };
    std::size_t total{ 0 };
};

// libstdc++'s std::reduce / std::transform_reduce order for random-access ranges
// (4-way grouped, then a sequential tail); psim calls these with execution::seq.
template<typename F> double groupedSum(std::size_t n, double init, F f) {
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

class Model {
public:
    // settings
    std::size_t num_runs{ 1 }, steps{ 0 }, num_phonons{ 0 }, step_interval{ 0 };
    double sim_time{ 0. }, t_eq{ 0. };
    bool phasor{ false };
    SimType type{ SimType::SteadyState };
    std::size_t start_step{ 0 }, step_adj{ 0 };
    double step_time{ 0. };
    std::vector<double> step_times;
    double lb{ 0. }, ub{ 0. }, eff_energy{ 0. };

    std::vector<Material> mats;
    std::vector<Sensor> sensors;
    std::vector<Cell> cells;
    std::map<std::size_t, std::vector<Measurement>> measurements;

    // simulator state
    std::vector<Builder> builders;
    std::size_t total_phonons{ 0 };

    // counters (oracle instrumentation)
    std::uint64_t phonon_steps{ 0 };
    std::uint64_t phonons_simulated{ 0 };

    int threads{ 1 };
    std::uint32_t seed{ 5489U };
    std::unique_ptr<Rng> rng;// thread 0 engine; also used by the host-side steps
    std::unique_ptr<std::mt19937> shuffle_engine;

    // ------------------------------------------------ construction (psim/src/inputManager.cpp, model.cpp)
    std::size_t sensorIndex(std::size_t id) const {
        for (std::size_t i = 0; i < sensors.size(); ++i) {
            if (sensors[i].id == id) { return i; }
        }
        throw std::runtime_error("Sensor does not exist");
    }
    const Material& matOf(std::size_t cell) const { return mats[sensors[cells[cell].sensor].mat]; }

    void setType(SimType t, std::size_t interval) {// Model::setSimulationType: model.cpp:46-70
        type = t;
        if (t == SimType::Transient || t == SimType::Periodic) {
            start_step = static_cast<std::size_t>(static_cast<double>(steps) - static_cast<double>(steps) * SS_STEPS_PERCENT);
            if (interval == 0) { throw std::runtime_error("Step interval of 0 is invalid for transient and periodic simulations."); }
        }
        if (t == SimType::Transient && t_eq == 0) { throw std::runtime_error("Transient simulations must be run using the deviational approach."); }
        if (t == SimType::SteadyState) {
            step_adj = static_cast<std::size_t>(static_cast<double>(steps) - static_cast<double>(steps) * SS_STEPS_PERCENT);
            if (interval > 0) { throw std::runtime_error("Step interval > 0 is invalid for steady-state simulations"); }
        }
        step_interval = interval;
    }

    void addSensor(std::size_t id, std::size_t mat, double t_init) {// model.cpp:81-96
        for (const auto& s : sensors) {
            if (s.id == id) { throw std::runtime_error("Sensor with this ID already exists"); }
        }
        Sensor s;
        s.id = id;
        s.mat = mat;
        s.t_init = t_init;
        s.t_steady = t_init;
        const std::size_t rec = (type == SimType::SteadyState)
                                    ? static_cast<std::size_t>(static_cast<double>(steps) * SS_STEPS_PERCENT)
                                    : steps;
        s.energy.assign(rec, 0);
        s.flux.assign(rec, { 0., 0. });
        if (type == SimType::Transient) {
            s.steady_temps.assign(rec, 0.);
            s.scat_steps.assign(rec, nullptr);
            s.heat_caps.assign(rec, 0.);
        }
        sensors.push_back(std::move(s));
    }

    static Surface makeSurface(const Seg& line, double spec, int nsign) {
        Surface s;
        s.line = line;
        s.normal = segNormal(line, nsign);
        s.spec = spec;
        return s;
    }

    // CompositeSurface::verifySurfaceLine: compositeSurface.cpp:66-85
    static bool edgeAccepts(const Edge& e, const Seg& line) {
        if (segContains(e.main.line, line)) {
            for (const auto& t : e.trans) {
                if (segOverlaps(line, t.line)) { throw std::runtime_error("An existing surface conflicts with the location of the incoming surface."); }
            }
            for (const auto& t : e.emits) {
                if (segOverlaps(line, t.line)) { throw std::runtime_error("An existing surface conflicts with the location of the incoming surface."); }
            }
            return true;
        }
        return false;
    }

    bool addTransition(std::size_t c, const Seg& line, std::size_t target) {// Cell::setTransitionSurface: cell.cpp:126-132
        for (auto& e : cells[c].edges) {
            if (edgeAccepts(e, line)) {
                Surface s = makeSurface(line, 0., cells[c].nsign);
                s.target = target;
                e.trans.push_back(s);
                return true;
            }
        }
        return false;
    }

    void addCell(const Tri& t, std::size_t sensor_id, double spec) {// Model::addCell: model.cpp:98-113
        if (!triValid(t)) { throw std::runtime_error("These 3 points do not allow for a valid triangle"); }
        Cell c;
        c.tri = t;
        c.sensor = sensorIndex(sensor_id);
        spec = std::min(std::max(spec, 0.), 1.);
        c.nsign = triClockwise(t) ? 1 : -1;
        const auto lines = triLines(t);
        for (std::size_t i = 0; i < 3; ++i) { c.edges[i].main = makeSurface(lines[i], spec, c.nsign); }
        c.area = triArea(t);
        sensors[c.sensor].area += c.area;
        cells.push_back(std::move(c));
        const std::size_t inc = cells.size() - 1;
        std::size_t identical = 0;
        for (std::size_t k = 0; k < cells.size(); ++k) {
            if (!triSame(cells[inc].tri, cells[k].tri)) {
                // Cell::validate: cell.cpp:21-25
                if (triIntersects(cells[inc].tri, cells[k].tri)) { throw std::runtime_error("Incoming triangle intersects an existing triangle"); }
                if (triContainsTri(cells[inc].tri, cells[k].tri)) { throw std::runtime_error("Triangle is contained within another"); }
                if (triContainsTri(cells[k].tri, cells[inc].tri)) { throw std::runtime_error("Triangle is contained within another"); }
                // Cell::findTransitionSurface: cell.cpp:81-98
                const auto l1s = triLines(cells[inc].tri);
                const auto l2s = triLines(cells[k].tri);
                for (const auto& l1 : l1s) {
                    for (const auto& l2 : l2s) {
                        if (segContains(l1, l2)) {
                            if (!addTransition(inc, l2, k) || !addTransition(k, l2, inc)) { throw std::runtime_error("transition surface conflict"); }
                        } else if (segContains(l2, l1)) {
                            if (!addTransition(inc, l1, k) || !addTransition(k, l1, inc)) { throw std::runtime_error("transition surface conflict"); }
                        }
                    }
                }
            } else if (++identical == 2) {
                throw std::runtime_error("Duplicate cell detected.");
            }
        }
    }

    bool setEmit(Pt p1, Pt p2, double temp, double duration, double start) {// Model::setEmitSurface: model.cpp:125-138
        if ((start < 0. || start >= sim_time) || (duration < 0. || duration > sim_time - start)) {
            throw std::runtime_error("Transient Surface start_time or duration specifications are invalid.");
        }
        if ((start > 0. || duration < sim_time) && type != SimType::Transient) {
            throw std::runtime_error("Cannot add a transient surface to a non transient simulation.");
        }
        const Seg line = makeSeg(p1, p2);
        for (auto& c : cells) {
            for (auto& e : c.edges) {// Cell::setEmitSurface / CompositeSurface::addEmitSurface
                if (edgeAccepts(e, line)) {
                    Surface s = makeSurface(line, e.main.spec, c.nsign);
                    s.normal = e.main.normal;
                    s.temp = temp;
                    s.duration = duration;
                    s.start = start;
                    e.emits.push_back(s);
                    return true;
                }
            }
        }
        return false;
    }

    void load(const psim_json::Value& j) {// InputManager::deserialize: inputManager.cpp:14-115
        const auto& st = j.at("settings");
        steps = static_cast<std::size_t>(st.at("num_measurements").as_int());
        num_phonons = static_cast<std::size_t>(st.at("num_phonons").as_int());
        sim_time = st.at("sim_time").as_double();
        t_eq = st.at("t_eq").as_double();
        phasor = st.at("phasor_sim").kind() == psim_json::Value::Kind::Bool && st.at("phasor_sim").as_bool();
        if (st.contains("num_runs")) { num_runs = static_cast<std::size_t>(st.at("num_runs").as_int()); }
        step_time = sim_time / static_cast<double>(steps);
        step_times.resize(steps);
        for (std::size_t n = 1; n <= steps; ++n) { step_times[n - 1] = static_cast<double>(static_cast<int>(n)) * sim_time / static_cast<double>(steps); }
        const auto ty = st.at("sim_type").as_int();
        const SimType t = ty == 1 ? SimType::Periodic : (ty == 2 ? SimType::Transient : SimType::SteadyState);
        setType(t, t == SimType::SteadyState ? 0 : static_cast<std::size_t>(st.at("step_interval").as_int()));
        std::map<std::string, std::size_t> by_name;
        for (const auto& m : j.at("materials").items()) {
            Material mat;
            mat.name = m.at("name").as_string();
            if (by_name.count(mat.name) != 0) { throw std::runtime_error("A duplicate material name was detected."); }
            const auto& d = m.at("d_data");
            const auto& r = m.at("r_data");
            for (int i = 0; i < 3; ++i) {
                mat.la[i] = d.at("la_data").at(i).as_double();
                mat.ta[i] = d.at("ta_data").at(i).as_double();
            }
            mat.w_max_la = d.at("max_freq_la").as_double();
            mat.w_max_ta = d.at("max_freq_ta").as_double();
            mat.b_l = r.at("b_l").as_double();
            mat.b_tn = r.at("b_tn").as_double();
            mat.b_tu = r.at("b_tu").as_double();
            mat.b_i = r.at("b_i").as_double();
            mat.w = r.at("w").as_double();
            mat.full = (t_eq == 0.);
            mat.build();
            by_name[mat.name] = mats.size();
            mats.push_back(std::move(mat));
        }
        for (const auto& s : j.at("sensors").items()) {
            addSensor(static_cast<std::size_t>(s.at("id").as_int()), by_name.at(s.at("material").as_string()), s.at("t_init").as_double());
        }
        const auto& cs = j.at("cells");
        for (const auto& c : cs.items()) {
            const auto& t = c.at("triangle");
            auto pt = [](const psim_json::Value& v) { return Pt{ v.at("x").as_double(), v.at("y").as_double() }; };
            addCell(Tri{ pt(t.at("p1")), pt(t.at("p2")), pt(t.at("p3")) }, static_cast<std::size_t>(c.at("sensorID").as_int()), c.at("specularity").as_double());
        }
        for (const auto& e : j.at("emit_surfaces").items()) {
            auto pt = [](const psim_json::Value& v) { return Pt{ v.at("x").as_double(), v.at("y").as_double() }; };
            if (!setEmit(pt(e.at("p1")), pt(e.at("p2")), e.at("temp").as_double(), e.at("duration").as_double(), e.at("start_time").as_double())) {
                throw std::runtime_error("Unable to add emitting surface.");
            }
        }
    }

    // ------------------------------------------------ controllers (psim/src/sensorController.cpp)
    double initTemp(const Sensor& s) const { return type == SimType::SteadyState ? s.t_steady : s.t_init; }
    double steadyTemp(const Sensor& s, std::size_t step) const {
        if (type == SimType::Transient) { return step == 0 ? s.t_init : s.steady_temps[step]; }
        return s.t_steady;
    }
    double heatCap(const Sensor& s, std::size_t step) const { return type == SimType::Transient ? s.heat_caps[step] : s.heat_cap; }

    void updateTables(Sensor& s) {// SensorController::updateTables: sensorController.cpp:38-50
        const Material& m = mats[s.mat];
        const std::size_t k = m.tempIndex(s.t_init);
        s.base = &m.base[k];
        s.heat_cap = m.base[k].sum;
        s.scat = &m.scat[k];
        if (type == SimType::Transient) {
            std::fill(s.scat_steps.begin(), s.scat_steps.end(), s.scat);
            std::fill(s.heat_caps.begin(), s.heat_caps.end(), s.heat_cap);
            std::fill(s.steady_temps.begin(), s.steady_temps.end(), s.t_init);
        }
    }

    // ------------------------------------------------ energies (cell.cpp:38-63, model.cpp:196-201)
    double cellInitEnergy(std::size_t c) const {
        const Sensor& s = sensors[cells[c].sensor];
        const double e = cells[c].area * s.heat_cap;
        return (t_eq == 0.) ? e : e * std::fabs(initTemp(s) - t_eq);
    }
    double cellEmitEnergy(std::size_t c) const {
        double total = 0.;
        const Material& m = matOf(c);
        for (const auto& e : cells[c].edges) {
            total += groupedSum(e.emits.size(), 0., [&](std::size_t i) {
                const Surface& s = e.emits[i];
                const double en = s.line.len * s.duration * m.emit[m.tempIndex(s.temp)].sum / 4.;
                return (t_eq == 0.) ? en : en * std::fabs(s.temp - t_eq);
            });
        }
        return total;
    }
    double totalEnergy() const {
        return groupedSum(cells.size(), 0., [&](std::size_t c) { return cellInitEnergy(c) + cellEmitEnergy(c); });
    }

    // ------------------------------------------------ builders (modelSimulator.cpp:43-85, phononBuilder.cpp)
    void initBuilders(double eff) {
        auto count = [&](double energy) {
            double whole = 0;
            const double frac = std::modf(energy / eff, &whole);
            auto n = static_cast<std::size_t>(whole);
            return (rng->u() < frac) ? n + 1 : n;
        };
        Builder cb;
        cb.kind = 0;
        for (std::size_t c = 0; c < cells.size(); ++c) {
            const std::size_t n = count(cellInitEnergy(c));
            if (n > 0) {
                total_phonons += n;
                if (cb.total + n > BUILDER_MAX_PHONONS / 2 && cb.total != 0) {
                    builders.push_back(cb);
                    cb = Builder{};
                    cb.kind = 0;
                }
                cb.total += n;
                cb.stack.emplace_back(c, n);
            }
            const Material& m = matOf(c);
            for (std::size_t ei = 0; ei < 3; ++ei) {
                const Edge& e = cells[c].edges[ei];
                for (std::size_t k = 0; k < e.emits.size(); ++k) {
                    const Surface& s = e.emits[k];
                    const double factor = m.emit[m.tempIndex(s.temp)].sum * s.duration * s.line.len / 4.;
                    const double energy = (t_eq == 0.) ? factor : factor * std::fabs(t_eq - s.temp);
                    std::size_t n2 = count(energy);
                    total_phonons += n2;
                    auto push = [&](std::size_t amount) {
                        Builder b;
                        b.kind = phasor ? 2 : 1;
                        b.cell = c;
                        b.edge = ei;
                        b.emit = k;
                        b.remaining = amount;
                        b.total = amount;
                        builders.push_back(b);
                    };
                    while (n2 > BUILDER_MAX_PHONONS) {
                        push(BUILDER_MAX_PHONONS);
                        n2 -= BUILDER_MAX_PHONONS;
                    }
                    push(n2);
                }
            }
        }
        if (!cb.stack.empty()) { builders.push_back(cb); }
    }

    bool hasPhonons(const Builder& b) const { return b.kind == 0 ? !b.stack.empty() : b.remaining > 0; }

    // Phonon::setRandDirection: phonon.cpp:28-31
    static void randDirection(Phonon& p, Rng& r) {
        p.dx = 2. * r.u() - 1.;
        p.dy = std::sqrt(1. - p.dx * p.dx) * std::cos(2. * PI * r.u());
    }
    // Surface::redirectPhonon: surface.cpp:23-30
    static void redirect(const Surface& s, Phonon& p, Rng& r) {
        const double u = r.u();
        const double ndx = std::sqrt(u);
        const double ndy = std::sqrt(1. - u) * std::cos(2. * PI * r.u());
        p.dx = s.normal.x * ndx - s.normal.y * ndy;
        p.dy = s.normal.y * ndx + s.normal.x * ndy;
    }
    // SensorController::initialUpdate / scatterUpdate: sensorController.cpp:28-36,52-55
    void resample(Phonon& p, const Material& m, const Table& t, Rng& r) const {
        const auto [bin, pol] = sampleBin(t, r);
        p.bin = bin;
        p.freq = m.sampleFreq(bin, r);
        p.vel = m.vel(bin, pol);
        p.pol = pol;
    }

    Phonon build(Builder& b, Rng& r) {
        Phonon p;
        if (b.kind == 0) {// CellOriginBuilder::operator(): phononBuilder.cpp:6-16
            auto& top = b.stack.back();
            const std::size_t c = top.first;
            const Sensor& s = sensors[cells[c].sensor];
            p.sign = (initTemp(s) > t_eq) ? 1 : -1;
            p.lifetime = 0.;
            p.cell = static_cast<long>(c);
            resample(p, matOf(c), *s.base, r);
            // getRandPoint(urand(), urand()): GCC evaluates these call arguments right to left.
            const double r2 = r.u();
            const double r1 = r.u();
            const Pt q = triRandPoint(cells[c].tri, r1, r2);
            p.px = q.x;
            p.py = q.y;
            randDirection(p, r);
            if (--top.second == 0) { b.stack.pop_back(); }
            return p;
        }
        // SurfaceOriginBuilder / PhasorBuilder: phononBuilder.cpp:31-49
        --b.remaining;
        const Surface& s = cells[b.cell].edges[b.edge].emits[b.emit];
        p.sign = (s.temp > t_eq) ? 1 : -1;
        p.lifetime = s.start + s.duration * r.u();// EmitSurface::getPhononTime: surface.cpp:67-69
        p.cell = static_cast<long>(b.cell);
        const Material& m = matOf(b.cell);
        resample(p, m, m.emit[m.tempIndex(s.temp)], r);
        const Pt q = segRandPoint(s.line, r.u());
        p.px = q.x;
        p.py = q.y;
        redirect(s, p, r);
        if (b.kind == 2) {
            p.bin = 1;
            p.freq = 1;
            p.vel = 1000;
            p.pol = LA;
            p.dx = s.normal.x;
            p.dy = s.normal.y;
        }
        return p;
    }

    // ------------------------------------------------ phonon transport (modelSimulator.cpp, cell.cpp, surface.cpp)
    struct Tally {
        std::vector<std::vector<int>> energy;
        std::vector<std::vector<std::array<double, 2>>> flux;
        std::uint64_t steps{ 0 };
    };

    // Surface::boundaryHandlePhonon: surface.cpp:32-44
    static void boundary(const Surface& s, Phonon& p, Rng& r) {
        if (s.spec == 1. || r.u() < s.spec) {
            const double nx = s.normal.x;
            const double ny = s.normal.y;
            const double ndx = -p.dx * nx - p.dy * ny;
            const double ndy = -p.dx * ny + p.dy * nx;
            p.dx = nx * ndx - ny * ndy;
            p.dy = ny * ndx + nx * ndy;
        } else {
            redirect(s, p, r);
        }
    }

    // Cell::handleSurfaceCollision -> CompositeSurface::handlePhonon: cell.cpp:103-108, compositeSurface.cpp:47-66
    void collide(Phonon& p, const Pt& poi, Rng& r) const {
        const Cell& c = cells[static_cast<std::size_t>(p.cell)];
        for (const auto& e : c.edges) {
            if (!onLine(e.main.line, poi)) { continue; }
            for (const auto& t : e.trans) {
                if (onLine(t.line, poi)) {// TransitionSurface::handlePhonon: surface.cpp:71-109
                    const Material& to = matOf(t.target);
                    if (sensors[c.sensor].mat == sensors[cells[t.target].sensor].mat) {
                        p.cell = static_cast<long>(t.target);
                    } else {
                        const double max_freq = (p.pol == LA) ? to.w_max_la : to.w_max_ta;
                        if (p.freq > max_freq) {
                            redirect(t, p, r);
                        } else {
                            p.cell = static_cast<long>(t.target);
                        }
                    }
                    return;
                }
            }
            for (const auto& s : e.emits) {
                if (onLine(s.line, poi)) {// EmitSurface::handlePhonon: surface.cpp:61-65
                    const double pt = static_cast<double>(p.lifestep) * step_time;
                    if (pt < s.start || pt + step_time > s.start + s.duration) {
                        boundary(s, p, r);
                    } else {
                        p.cell = -1;
                    }
                    return;
                }
            }
            boundary(e.main, p, r);
            return;
        }
    }

    // ModelSimulator::nextImpact: modelSimulator.cpp:87-122
    bool nextImpact(Phonon& p, double time, double& out, Rng& r) const {
        const double vx = p.dx * p.vel;
        const double vy = p.dy * p.vel;
        const Pt start{ p.px, p.py };
        const Pt end{ p.px + time * vx, p.py + time * vy };
        const Cell& c = cells[static_cast<std::size_t>(p.cell)];
        if (same(start, end)) { return false; }
        const Seg path = makeSeg(start, end);
        auto timeTo = [](double s, double e, double v, double mx) {
            return (v > VELOCITY_EPS || v < -VELOCITY_EPS) ? (e - s) / v : mx;
        };
        bool hit = false;
        Pt best{};
        for (const auto& e : c.edges) {
            Pt poi{};
            if (segIntersection(e.main.line, path, poi) && !same(poi, start)) {
                const double tx = timeTo(start.x, poi.x, vx, time);
                const double ty = timeTo(start.y, poi.y, vy, time);
                const double t = (tx <= ty) ? tx : ty;
                if (t <= time) {
                    time = t;
                    best = poi;
                    hit = true;
                }
            }
        }
        if (hit) {
            p.px = best.x;
            p.py = best.y;
            collide(p, best, r);
            out = time;
            return true;
        }
        return false;
    }

    // ModelSimulator::handleImpacts: modelSimulator.cpp:205-225.  Returns false when absorbed.
    bool impacts(Phonon& p, double drift, std::size_t sensor, double& drifted, Rng& r) const {
        double t = 0.;
        bool more = nextImpact(p, drift, t, r);
        drifted = 0.;
        std::size_t n = 0;
        while (more) {
            if (p.cell < 0) { return false; }
            drifted += t;
            if (++n > MAX_COLLISIONS) {
                // setRandPoint(urand(), urand()): arguments evaluated right to left.
                const double r2 = r.u();
                const double r1 = r.u();
                const Pt q = triRandPoint(cells[static_cast<std::size_t>(p.cell)].tri, r1, r2);
                p.px = q.x;
                p.py = q.y;
                drifted = drift;
                return true;
            }
            if (cells[static_cast<std::size_t>(p.cell)].sensor != sensor) { return true; }
            more = nextImpact(p, drift - drifted, t, r);
        }
        return p.cell >= 0;
    }

    std::array<double, 3> relaxRates(const Phonon& p, std::size_t step) const {// Phonon::getRelaxRates: phonon.cpp:55-60
        const Sensor& s = sensors[cells[static_cast<std::size_t>(p.cell)].sensor];
        return mats[s.mat].rates(steadyTemp(s, step), p.freq, p.pol);
    }

    // ModelSimulator::scatter: modelSimulator.cpp:124-137
    void scatter(Phonon& p, const std::array<double, 3>& rr, Rng& r) const {
        const double tau = ((0. + rr[0]) + rr[1]) + rr[2];
        const double u = r.u();
        if (u <= (rr[0] + rr[1]) / tau) {
            const Sensor& s = sensors[cells[static_cast<std::size_t>(p.cell)].sensor];
            const Table& t = (type == SimType::Transient) ? *s.scat_steps[p.lifestep] : *s.scat;
            resample(p, mats[s.mat], t, r);
            if (u > rr[0] / tau) { randDirection(p, r); }
        } else if (rr[2] > 0.) {
            randDirection(p, r);
        }
    }

    // ModelSimulator::simulatePhonon: modelSimulator.cpp:139-198
    void simulate(Phonon p, Tally& tally, Rng& r) const {
        bool alive = true;
        double age = p.lifetime;
        auto step = static_cast<std::size_t>(age / step_time);
        p.lifestep = step;
        std::array<double, 3> rr{};
        double tts = 0.;
        double ttm = 0.;
        while (alive) {
            if (tts <= 0.) {
                rr = relaxRates(p, step);
                tts = SCALING_FACTOR * -std::log(r.u()) / (((0. + rr[0]) + rr[1]) + rr[2]);
            }
            if (ttm <= 0.) { ttm = step_times[step] - age; }
            double drift = std::min(tts, ttm);
            const std::size_t sensor = cells[static_cast<std::size_t>(p.cell)].sensor;
            double drifted = 0.;
            if (impacts(p, drift, sensor, drifted, r)) {
                if (cells[static_cast<std::size_t>(p.cell)].sensor != sensor) { drift = drifted; }
                const double factor = p.vel * (drift - drifted);// Phonon::drift: phonon.cpp:22-26
                p.px += p.dx * factor;
                p.py += p.dy * factor;
                age += drift;
                ttm -= drift;
                tts -= drift;
                if (ttm == 0.) {
                    ++tally.steps;// one phonon-step: the phonon reached a measurement boundary alive
                    if (++step < steps) {
                        p.lifestep = step;
                        if (step >= step_adj) {// Sensor::updateHeatParams: sensor.cpp:43-52
                            const std::size_t si = cells[static_cast<std::size_t>(p.cell)].sensor;
                            const std::size_t k = step - step_adj;
                            tally.energy[si][k] += p.sign;
                            tally.flux[si][k][0] += (p.dx * p.vel) * p.sign;
                            tally.flux[si][k][1] += (p.dy * p.vel) * p.sign;
                        }
                    } else {
                        alive = false;
                    }
                } else if (!phasor && tts == 0.) {
                    scatter(p, rr, r);
                } else {
                    tts = 0.;
                }
            } else {
                alive = false;
            }
        }
    }

    Tally newTally() const {
        Tally t;
        t.energy.resize(sensors.size());
        t.flux.resize(sensors.size());
        for (std::size_t i = 0; i < sensors.size(); ++i) {
            t.energy[i].assign(sensors[i].energy.size(), 0);
            t.flux[i].assign(sensors[i].flux.size(), { 0., 0. });
        }
        return t;
    }
    void merge(const Tally& t) {
        for (std::size_t i = 0; i < sensors.size(); ++i) {
            for (std::size_t k = 0; k < sensors[i].energy.size(); ++k) {
                sensors[i].energy[k] += t.energy[i][k];
                sensors[i].flux[k][0] += t.flux[i][k][0];
                sensors[i].flux[k][1] += t.flux[i][k][1];
            }
        }
        phonon_steps += t.steps;
    }

    // ModelSimulator::runSimulation / runPhononByPhonon / runUsingBuilders: modelSimulator.cpp:39-41,227-254
    void runSimulator() {
        if (total_phonons < PHONON_CUTOFF) {
            std::vector<Phonon> ph;
            ph.reserve(total_phonons);
            for (auto& b : builders) {
                while (hasPhonons(b)) { ph.push_back(build(b, *rng)); }
            }
            ShuffleDevice dev{ shuffle_engine.get() };
            std::ranges::shuffle(ph, dev);
            phonons_simulated += ph.size();
            if (threads <= 1) {
                Tally t = newTally();
                for (const auto& p : ph) { simulate(p, t, *rng); }
                merge(t);
            } else {
                std::vector<Tally> ts(static_cast<std::size_t>(threads), newTally());
                std::vector<std::thread> pool;
                std::atomic<std::size_t> next{ 0 };
                for (int w = 0; w < threads; ++w) {
                    pool.emplace_back([&, w]() {
                        Rng local(seed + 7919U * static_cast<std::uint32_t>(w + 1));
                        Rng& rr = (w == 0) ? *rng : local;
                        constexpr std::size_t CHUNK = 256;
                        while (true) {
                            const std::size_t lo = next.fetch_add(CHUNK);
                            if (lo >= ph.size()) { break; }
                            const std::size_t hi = std::min(ph.size(), lo + CHUNK);
                            for (std::size_t i = lo; i < hi; ++i) { simulate(ph[i], ts[static_cast<std::size_t>(w)], rr); }
                        }
                    });
                }
                for (auto& th : pool) { th.join(); }
                for (const auto& t : ts) { merge(t); }
            }
        } else {
            if (threads <= 1) {
                Tally t = newTally();
                for (auto& b : builders) {
                    while (hasPhonons(b)) {
                        simulate(build(b, *rng), t, *rng);
                        ++phonons_simulated;
                    }
                }
                merge(t);
            } else {
                std::vector<Tally> ts(static_cast<std::size_t>(threads), newTally());
                std::vector<std::thread> pool;
                std::atomic<std::size_t> next{ 0 };
                std::atomic<std::uint64_t> simulated{ 0 };
                for (int w = 0; w < threads; ++w) {
                    pool.emplace_back([&, w]() {
                        Rng local(seed + 7919U * static_cast<std::uint32_t>(w + 1));
                        Rng& rr = (w == 0) ? *rng : local;
                        while (true) {
                            const std::size_t bi = next.fetch_add(1);
                            if (bi >= builders.size()) { break; }
                            while (hasPhonons(builders[bi])) {
                                simulate(build(builders[bi], rr), ts[static_cast<std::size_t>(w)], rr);
                                simulated.fetch_add(1, std::memory_order_relaxed);
                            }
                        }
                    });
                }
                for (auto& th : pool) { th.join(); }
                for (const auto& t : ts) { merge(t); }
                phonons_simulated += simulated.load();
            }
        }
    }

    // ------------------------------------------------ interpretation (psim/src/sensorInterpreter.cpp)
    std::vector<double> findTemps(const Sensor& s, std::size_t start, double eff) const {
        const std::size_t n = s.energy.size() - start;
        std::vector<double> out(n);
        const Material& m = mats[s.mat];
        for (std::size_t i = 0; i < n; ++i) {
            const double energy = eff * s.energy[start + i];
            if (t_eq != 0.) {
                out[i] = energy / (s.area * heatCap(s, i)) + t_eq;
            } else {
                double temp = 0.;
                double hi = ub;
                double lo = lb;
                std::size_t iter = 0;
                while ((hi - lo >= INV_EPS) && (++iter != INV_MAX_ITERS)) {
                    temp = (hi + lo) / 2.;
                    const double de = (m.base[m.tempIndex(temp)].sum * s.area) - energy;
                    if (de < 0.) {
                        lo = temp;
                    } else {
                        hi = temp;
                    }
                }
                out[i] = temp;
            }
        }
        return out;
    }

    double finalTemp(const Sensor& s, std::size_t start, double eff) const {// getFinalTemp: sensorInterpreter.cpp:68-74
        if (s.area == 0.) { return 0.; }
        const auto temps = findTemps(s, start, eff);
        double sum = 0.;
        for (double t : temps) { sum += t; }
        return sum / static_cast<double>(s.energy.size() - start);
    }

    static std::pair<double, double> meanAndError(const std::vector<double>& d) {// sensorInterpreter.cpp:35-46
        const auto n = static_cast<double>(d.size());
        const double avg = groupedSum(d.size(), 0., [&](std::size_t i) { return d[i]; }) / n;
        const double sd = std::sqrt(groupedSum(d.size(), 0., [&](std::size_t i) { return (avg - d[i]) * (avg - d[i]); }) / n);
        return { avg, sd / std::sqrt(n) };
    }

    Measurement scale(const Sensor& s, double eff) const {// scaleHeatParams: sensorInterpreter.cpp:19-66
        Measurement m;
        m.id = s.id;
        m.temps = findTemps(s, 0, eff);
        if (!m.temps.empty()) { m.temps.front() = initTemp(s); }
        const double f = eff / s.area;
        m.fluxes.resize(s.flux.size());
        for (std::size_t k = 0; k < s.flux.size(); ++k) { m.fluxes[k] = { s.flux[k][0] * f, s.flux[k][1] * f }; }
        std::vector<double> fx(m.fluxes.size());
        std::vector<double> fy(m.fluxes.size());
        for (std::size_t k = 0; k < m.fluxes.size(); ++k) {
            fx[k] = m.fluxes[k][0];
            fy[k] = m.fluxes[k][1];
        }
        std::tie(m.t, m.st) = meanAndError(m.temps);
        std::tie(m.fx, m.sfx) = meanAndError(fx);
        std::tie(m.fy, m.sfy) = meanAndError(fy);
        return m;
    }

    // ------------------------------------------------ run orchestration (psim/src/model.cpp:141-283)
    std::pair<double, double> bounds() {// setTemperatureBounds: model.cpp:203-218
        std::vector<double> temps;
        for (const auto& c : cells) {
            temps.push_back(initTemp(sensors[c.sensor]));
            for (const auto& e : c.edges) {
                for (const auto& s : e.emits) { temps.push_back(s.temp); }
            }
        }
        const auto [mn, mx] = std::minmax_element(temps.begin(), temps.end());
        const double b = phasor ? PHASOR_TEMP_BOUND_EPS : TEMP_BOUND_EPS;
        lb = std::max(*mn - b, 0.);
        ub = *mx + b;
        return { *mn, *mx };
    }

    void initTables(double lo, double hi) {// initializeMaterialTables: model.cpp:221-227
        for (auto& m : mats) { m.initTables(lo, hi); }
        for (auto& s : sensors) { updateTables(s); }
        for (auto& c : cells) {
            const Material& m = mats[sensors[c.sensor].mat];
            for (auto& e : c.edges) {
                for (auto& s : e.emits) { s.table = &m.emit[m.tempIndex(s.temp)]; }
            }
        }
    }

    void run() {// Model::runSimulation
        rng = std::make_unique<Rng>(seed);
        shuffle_engine = std::make_unique<std::mt19937>(seed ^ 0x9E3779B9U);
        for (std::size_t run = 0; run < num_runs; ++run) {
            const auto [mn, mx] = bounds();
            initTables(mn, mx);
            eff_energy = totalEnergy() / static_cast<double>(num_phonons);
            initBuilders(eff_energy);
            runSimulator();
            // Model::resetRequired updates each controller's steady temperature (model.cpp:250-272,
            // sensorController.cpp:57-62,90-99); MAX_ITERS = 1 so no re-run follows.
            for (auto& s : sensors) {
                if (type != SimType::Transient) {
                    s.t_steady = finalTemp(s, start_step, eff_energy);
                } else {
                    s.steady_temps = findTemps(s, 0, eff_energy);
                }
            }
            eff_energy = totalEnergy() / static_cast<double>(num_phonons);
            auto& ms = measurements[run];
            for (const auto& s : sensors) { ms.push_back(scale(s, eff_energy)); }
            std::sort(ms.begin(), ms.end(), [](const Measurement& a, const Measurement& b) { return a.id < b.id; });
            if (run + 1 < num_runs) {// Model::reset(true)
                builders.clear();
                total_phonons = 0;
                for (auto& s : sensors) {
                    s.t_steady = s.t_init;
                    const Material& m = mats[s.mat];
                    const std::size_t k = m.tempIndex(s.t_steady);
                    s.base = &m.base[k];
                    if (type == SimType::SteadyState) { s.heat_cap = m.base[k].sum; }
                    s.scat = &m.scat[k];
                    if (type == SimType::Transient) {
                        std::fill(s.scat_steps.begin(), s.scat_steps.end(), s.scat);
                        std::fill(s.heat_caps.begin(), s.heat_caps.end(), s.heat_cap);
                        std::fill(s.steady_temps.begin(), s.steady_temps.end(), s.t_init);
                    }
                    std::fill(s.energy.begin(), s.energy.end(), 0);
                    std::fill(s.flux.begin(), s.flux.end(), std::array<double, 2>{ 0., 0. });
                }
            }
        }
    }
};

}// namespace oracle

// ---------------------------------------------------------------- C interface for tests and the CPU baseline
namespace {
thread_local std::string g_error;
}

extern "C" {

const char* oracle_last_error(void) { return g_error.c_str(); }

// Runs a model file.  Outputs (caller-allocated, may be null):
//   stats[n_sensors*6]      per sensor: T, SE(T), fx, SE(fx), fy, SE(fy) averaged over runs
//   energy[n_sensors*K], flux[n_sensors*K*2]  raw tallies of the last run
//   counters[4]             total phonons of the last run, phonons simulated, phonon-steps, eff_energy bits
// Returns 0 on success.
int oracle_run(const char* json_path, unsigned seed, int threads, int* n_sensors, int* n_recorded, double* stats,
    long long* energy, double* flux, unsigned long long* counters, double* seconds) {
    try {
        oracle::Model m;
        m.load(psim_json::parse_file(json_path));
        m.seed = seed;
        m.threads = threads < 1 ? 1 : threads;
        const auto t0 = std::chrono::steady_clock::now();
        m.run();
        const auto t1 = std::chrono::steady_clock::now();
        if (seconds != nullptr) { *seconds = std::chrono::duration<double>(t1 - t0).count(); }
        const std::size_t S = m.sensors.size();
        const std::size_t K = S > 0 ? m.sensors[0].energy.size() : 0;
        if (n_sensors != nullptr) { *n_sensors = static_cast<int>(S); }
        if (n_recorded != nullptr) { *n_recorded = static_cast<int>(K); }
        if (stats != nullptr) {
            std::vector<double> acc(S * 6, 0.);
            for (const auto& [run, ms] : m.measurements) {
                for (std::size_t i = 0; i < ms.size(); ++i) {
                    acc[i * 6 + 0] += ms[i].t;
                    acc[i * 6 + 1] += ms[i].st;
                    acc[i * 6 + 2] += ms[i].fx;
                    acc[i * 6 + 3] += ms[i].sfx;
                    acc[i * 6 + 4] += ms[i].fy;
                    acc[i * 6 + 5] += ms[i].sfy;
                }
            }
            const auto runs = static_cast<double>(m.measurements.size());
            for (std::size_t i = 0; i < S * 6; ++i) { stats[i] = acc[i] / runs; }
        }
        for (std::size_t i = 0; i < S; ++i) {
            for (std::size_t k = 0; k < K; ++k) {
                if (energy != nullptr) { energy[i * K + k] = m.sensors[i].energy[k]; }
                if (flux != nullptr) {
                    flux[(i * K + k) * 2 + 0] = m.sensors[i].flux[k][0];
                    flux[(i * K + k) * 2 + 1] = m.sensors[i].flux[k][1];
                }
            }
        }
        if (counters != nullptr) {
            counters[0] = m.total_phonons;
            counters[1] = m.phonons_simulated;
            counters[2] = m.phonon_steps;
            std::memcpy(&counters[3], &m.eff_energy, sizeof(double));
        }
        return 0;
    } catch (const std::exception& e) {
        g_error = e.what();
        return 1;
    }
}

// Model shape only: number of sensors and recorded steps, without running.
int oracle_shape(const char* json_path, int* n_sensors, int* n_recorded, int* n_cells) {
    try {
        oracle::Model m;
        m.load(psim_json::parse_file(json_path));
        *n_sensors = static_cast<int>(m.sensors.size());
        *n_recorded = m.sensors.empty() ? 0 : static_cast<int>(m.sensors[0].energy.size());
        *n_cells = static_cast<int>(m.cells.size());
        return 0;
    } catch (const std::exception& e) {
        g_error = e.what();
        return 1;
    }
}

// Segment intersection known answers: segs_a/segs_b [n][4]; out_poi [n][2]; out_has [n].
void oracle_intersect(int n, const double* a, const double* b, double* poi, int* has) {
    for (int i = 0; i < n; ++i) {
        try {
            const auto sa = oracle::makeSeg({ a[4 * i], a[4 * i + 1] }, { a[4 * i + 2], a[4 * i + 3] });
            const auto sb = oracle::makeSeg({ b[4 * i], b[4 * i + 1] }, { b[4 * i + 2], b[4 * i + 3] });
            oracle::Pt p{};
            has[i] = oracle::segIntersection(sa, sb, p) ? 1 : 0;
            poi[2 * i] = has[i] ? p.x : 0.;
            poi[2 * i + 1] = has[i] ? p.y : 0.;
        } catch (const std::exception&) {
            has[i] = -1;
            poi[2 * i] = 0.;
            poi[2 * i + 1] = 0.;
        }
    }
}

// Point-on-line (Line::contains(Point)) known answers: lines [n][4], pts [n][2].
void oracle_on_line(int n, const double* lines, const double* pts, int* out) {
    for (int i = 0; i < n; ++i) {
        try {
            const auto s = oracle::makeSeg({ lines[4 * i], lines[4 * i + 1] }, { lines[4 * i + 2], lines[4 * i + 3] });
            out[i] = oracle::onLine(s, { pts[2 * i], pts[2 * i + 1] }) ? 1 : 0;
        } catch (const std::exception&) { out[i] = -1; }
    }
}

// Triangle::contains(Point) known answers: tris [n][6], pts [n][2].
void oracle_tri_contains(int n, const double* tris, const double* pts, int* out) {
    for (int i = 0; i < n; ++i) {
        const oracle::Tri t{ { tris[6 * i], tris[6 * i + 1] }, { tris[6 * i + 2], tris[6 * i + 3] }, { tris[6 * i + 4], tris[6 * i + 5] } };
        try {
            out[i] = oracle::triContains(t, { pts[2 * i], pts[2 * i + 1] }) ? 1 : 0;
        } catch (const std::exception&) { out[i] = -1; }
    }
}

// Material tables for a model file after initializeTables (all materials in JSON order):
// writes the same binary layout as ref_driver's "tables" command into out_path.
int oracle_tables(const char* json_path, const char* out_path) {
    try {
        oracle::Model m;
        m.load(psim_json::parse_file(json_path));
        const auto [lo, hi] = m.bounds();
        m.initTables(lo, hi);
        std::ofstream os(out_path, std::ios::binary);
        auto wd = [&os](double v) { os.write(reinterpret_cast<const char*>(&v), sizeof v); };
        auto wu = [&os](std::uint64_t v) { os.write(reinterpret_cast<const char*>(&v), sizeof v); };
        for (const auto& mat : m.mats) {
            wu(mat.temps.size());
            for (double t : mat.temps) { wd(t); }
            for (double v : mat.freq) { wd(v); }
            for (double v : mat.vel_la) { wd(v); }
            for (double v : mat.vel_ta) { wd(v); }
            for (double v : mat.dens_la) { wd(v); }
            for (double v : mat.dens_ta) { wd(v); }
            for (const auto* tabs : { &mat.base, &mat.emit, &mat.scat }) {
                for (const auto& td : *tabs) {
                    wd(td.sum);
                    for (std::size_t i = 0; i < oracle::NBINS; ++i) {
                        wd(td.cum[i]);
                        wd(td.la_frac[i]);
                    }
                }
            }
        }
        wd(m.lb);
        wd(m.ub);
        return 0;
    } catch (const std::exception& e) {
        g_error = e.what();
        return 1;
    }
}

}// extern "C"
