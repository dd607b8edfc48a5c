// FP64 planar geometry with psim's exact semantics, for host model assembly and
// for the FP64 GPU kernels (functions are __host__ __device__ under nvcc).
//
// The tolerances, slope-intercept formulation and operation order follow
// psim/src/geometry.cpp so that results are bit-identical to the reference on the
// same inputs.  Device translation units that include this header are compiled
// with -fmad=false and host ones with -ffp-contract=off: a fused multiply-add
// would change roundings.
#pragma once

#include <cmath>
#include <cfloat>

#if defined(__CUDACC__)
#define PSIM_HD __host__ __device__ __forceinline__
#else
#define PSIM_HD inline
#endif

namespace psim {

// GEOEPS = DBL_EPSILON * 1e9 (psim/include/psim/utils.h:10)
constexpr double kGeoEps = DBL_EPSILON * 1E9;
constexpr double kPi = 3.1415926535897932384626433832795028841971693993751058209749445923;

struct P2 {
    double x, y;
};

// Point equality: squared distance below GEOEPS^2 (geometry.cpp:34-39).
PSIM_HD bool coincide(P2 a, P2 b) {
    const double dx = a.x - b.x;
    const double dy = a.y - b.y;
    return dx * dx + dy * dy < kGeoEps * kGeoEps;
}

PSIM_HD double cross2(P2 a, P2 b) { return a.x * b.y - b.x * a.y; }
PSIM_HD double dot2(P2 a, P2 b) { return a.x * b.x + a.y * b.y; }
PSIM_HD double absd(double v) { return v < 0. ? -v : v; }

// Slope of p->q, 0 when the x coordinates agree within GEOEPS (geometry.cpp:325-327).
PSIM_HD double slope(P2 p, P2 q) { return (absd(p.x - q.x) < kGeoEps) ? 0. : (p.y - q.y) / (p.x - q.x); }

// A segment in the reference's Line form: end points, slope, intercept, bounding box.
struct Seg64 {
    P2 a, b;
    double m, c;
    P2 lo, hi;
};

// Line constructor without the length (geometry.cpp:45-53, findBoundingBox :271-282).
// valid is false for coincident end points (the reference throws LineError).
PSIM_HD Seg64 make_seg(P2 a, P2 b, bool* valid) {
    Seg64 s;
    s.a = a;
    s.b = b;
    s.m = slope(a, b);
    s.c = a.y - s.m * a.x;
    double lx = a.x;
    double ly = a.y;
    double hx = b.x;
    double hy = b.y;
    if (b.x <= a.x) {
        const double t = lx;
        lx = hx;
        hx = t;
    }
    if (b.y <= a.y) {
        const double t = ly;
        ly = hy;
        hy = t;
    }
    s.lo = P2{ lx, ly };
    s.hi = P2{ hx, hy };
    if (valid != nullptr) { *valid = !coincide(a, b); }
    return s;
}

PSIM_HD double seg_length(const Seg64& s) {// getLineLength: geometry.cpp:318-322
    return sqrt((s.b.x - s.a.x) * (s.b.x - s.a.x) + (s.b.y - s.a.y) * (s.b.y - s.a.y));
}

// isPointOnLine (infinite line through the segment): geometry.cpp:295-298
PSIM_HD bool on_line(const Seg64& s, P2 p) {
    return absd(cross2(P2{ s.b.x - s.a.x, s.b.y - s.a.y }, P2{ p.x - s.a.x, p.y - s.a.y })) < kGeoEps;
}
PSIM_HD bool right_of(const Seg64& s, P2 p) {// isPointRightOfLine: geometry.cpp:300-303
    return cross2(P2{ s.b.x - s.a.x, s.b.y - s.a.y }, P2{ p.x - s.a.x, p.y - s.a.y }) < 0.;
}
PSIM_HD bool crosses_line(const Seg64& l1, const Seg64& l2) {// doesSegmentCrossLine: geometry.cpp:305-308
    return on_line(l1, l2.a) || on_line(l1, l2.b) || (right_of(l1, l2.a) != right_of(l1, l2.b));
}
PSIM_HD bool boxes_overlap(const Seg64& s, const Seg64& o) {// boxesIntersect: geometry.cpp:284-292
    return s.lo.x <= o.hi.x - kGeoEps && s.hi.x >= o.lo.x + kGeoEps && s.lo.y <= o.hi.y - kGeoEps
           && s.hi.y >= o.lo.y + kGeoEps;
}

PSIM_HD bool rel_equal(double a, double b) {// the 'equals' helper of geometry.cpp:107-109
    const double fa = absd(a);
    const double fb = absd(b);
    return absd(a - b) <= ((fa < fb ? fb : fa) * kGeoEps);
}

// Line::getIntersection (geometry.cpp:104-138): parallel or collinear lines have none.
PSIM_HD bool intersection(const Seg64& s, const Seg64& o, P2* poi) {
    if (!(boxes_overlap(s, o) && crosses_line(s, o) && crosses_line(o, s))) { return false; }
    P2 base;
    P2 q3;
    P2 q4;
    if (rel_equal(s.a.x, s.b.x)) {
        base = s.a;
        q3 = o.a;
        q4 = o.b;
    } else if (rel_equal(o.a.x, o.b.x)) {
        base = o.a;
        q3 = s.a;
        q4 = s.b;
    } else {
        if (rel_equal(s.m, o.m)) { return false; }
        const double x = (o.c - s.c) / (s.m - o.m);
        *poi = P2{ x, s.m * x + s.c };
        return true;
    }
    // One of the lines is vertical: evaluate the other line at its x.
    if (rel_equal(q3.x, q4.x)) { return false; }
    const double m = slope(q3, q4);
    const double c = q3.y - m * q3.x;
    *poi = P2{ base.x, m * base.x + c };
    return true;
}

// Triangle helpers (geometry.cpp:150-257)
PSIM_HD bool tri_valid(P2 p1, P2 p2, P2 p3) {
    const double s12 = absd(slope(p1, p2));
    const double s23 = absd(slope(p2, p3));
    const double s31 = absd(slope(p3, p1));
    return !((s12 == s23 && s23 == s31) || coincide(p1, p2) || coincide(p2, p3) || coincide(p3, p1));
}

PSIM_HD double dist2(P2 a, P2 b) { return sqrt((b.x - a.x) * (b.x - a.x) + (b.y - a.y) * (b.y - a.y)); }

PSIM_HD double tri_area(P2 p1, P2 p2, P2 p3) {// Heron's formula on the three edge lengths
    const double a = dist2(p1, p2);
    const double b = dist2(p2, p3);
    const double c = dist2(p3, p1);
    const double p = (a + b + c) / 2.;
    return sqrt(p * (p - a) * (p - b) * (p - c));
}

PSIM_HD bool tri_clockwise(P2 p1, P2 p2, P2 p3) {
    const double ax = p2.x - p1.x;
    const double ay = p2.y + p1.y;
    const double bx = p3.x - p2.x;
    const double by = p3.y + p2.y;
    const double cx = p1.x - p3.x;
    const double cy = p1.y + p3.y;
    return ax * ay + bx * by + cx * cy >= 0.;
}

// Triangle::contains(Point): barycentric window plus the area expression exactly as the
// reference writes it (geometry.cpp:190-215).
PSIM_HD bool tri_contains(P2 p1, P2 p2, P2 p3, P2 p) {
    const P2 bp1{ p2.x - p1.x, p2.y - p1.y };
    const P2 bp2{ p3.x - p1.x, p3.y - p1.y };
    const double d00 = dot2(bp1, bp1);
    const double d01 = dot2(bp1, bp2);
    const double d11 = dot2(bp2, bp2);
    const double denom = d00 * d11 - d01 * d01;
    const P2 bp3{ p.x - p1.x, p.y - p1.y };
    const double d20 = dot2(bp3, bp1);
    const double d21 = dot2(bp3, bp2);
    const double u = (d11 * d20 - d01 * d21) / denom;
    const double v = (d00 * d21 - d01 * d20) / denom;
    if (u >= kGeoEps && u <= 1. + kGeoEps && v >= kGeoEps && v <= 1. + kGeoEps && u + v <= 1. + kGeoEps) {
        const double a1 = tri_valid(p, p2, p3) ? tri_area(p, p2, p3) : 0.;
        const double a2 = tri_valid(p1, p, p3) ? tri_area(p1, p, p3) : 0.;
        const double a3 = tri_valid(p1, p2, p) ? tri_area(p1, p2, p) : 0.;
        if ((tri_area(p1, p2, p3) - a1 + a2 + a3) < kGeoEps) { return true; }
    }
    return false;
}

// Triangle::getRandPoint by reflection (geometry.cpp:234-242)
PSIM_HD P2 tri_point(P2 p1, P2 p2, P2 p3, double r1, double r2) {
    if (r1 + r2 > 1.) {
        r1 = 1 - r1;
        r2 = 1 - r2;
    }
    return P2{ p1.x + (p2.x - p1.x) * r1 + (p3.x - p1.x) * r2, p1.y + (p2.y - p1.y) * r1 + (p3.y - p1.y) * r2 };
}

// Line::normal(sign): geometry.cpp:97-100
PSIM_HD P2 seg_normal(P2 a, P2 b, int sign) {
    const double len = dist2(a, b);
    const double sg = (sign >= 0) ? 1. : -1.;
    return P2{ sg * (b.y - a.y) / len, -sg * (b.x - a.x) / len };
}

}// namespace psim
