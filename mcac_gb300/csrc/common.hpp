// Shared definitions for the MCAC GB300 library: field layout, status codes,
// and the exact FP64 geometry used by both the host mirror and the kernels.
//
// Every FP64 routine here follows the operation order of the reference
// (giraldeau/MCAC) so results are bit-identical. Both compilers must run with
// FP contraction off (-ffp-contract=off on the host, -fmad=false on the
// device); build() passes those flags.
#pragma once
#include <cmath>
#include <cstdint>
#include <limits>

#if defined(__CUDACC__)
#define MCACG_HD __host__ __device__ __forceinline__
#define MCACG_UNROLL _Pragma("unroll")
#else
#define MCACG_HD inline
#define MCACG_UNROLL
#endif

namespace mcacg {

// Sphere storage columns (include/constants.hpp:34-45 of the reference).
enum SphereField : int {
    SPH_X, SPH_Y, SPH_Z, SPH_R, SPH_VOLUME, SPH_SURFACE, SPH_RX, SPH_RY, SPH_RZ, SPH_NFIELDS
};
// Aggregate storage columns (include/constants.hpp:46-69 of the reference).
enum AggField : int {
    AGG_RG, AGG_F_AGG, AGG_LPM, AGG_TIME_STEP, AGG_RMAX, AGG_VOLUME, AGG_SURFACE,
    AGG_X, AGG_Y, AGG_Z, AGG_RX, AGG_RY, AGG_RZ, AGG_TIME, AGG_DP, AGG_DG_OVER_DP,
    AGG_OVERLAPPING, AGG_COORDINATION_NUMBER, AGG_ELECTRIC_CHARGE, AGG_D_M, AGG_CH_RATIO,
    AGG_NFIELDS
};
// Volume/surface methods (include/constants.hpp:113-120).
enum VolSurf : int { VS_CAPS = 0, VS_SBL = 1, VS_ARVO = 2, VS_ALPHAS = 3, VS_NONE = 4, VS_INVALID = 5 };

// Physical constants (include/constants.hpp:123-139).
constexpr double kBoltzmann = 1.38066E-23;
constexpr double kFluidMeanFreePathRef = 66.5E-9;
constexpr double kTemperatureRef = 293.15;
constexpr double kSutherland = 110;
constexpr double kPressureRef = 101300;
constexpr double kViscosityRef = 18.203E-6;
constexpr double kContactEpsilon = 1e-28;
constexpr double kCoordinationEpsilon = 1e-10;

MCACG_HD double pi_value() { return 3.141592653589793115997963468544185161590576171875; }

// --- periodic helpers (include/physical_model/physical_model.hpp:99-126) ---
// The reference wraps with unbounded while loops. Here each loop is capped:
// inside the cap (any value within 64 box lengths) the result is the
// reference's, operation for operation; beyond it (or for inf/NaN) the value
// is reduced with floor() instead, so no input can make a kernel spin.
constexpr int kWrapCap = 64;
MCACG_HD double periodic_distance(double d, double dim) {
    double half = 0.5 * dim;
    int guard = 0;
    while (d < -half && guard < kWrapCap) d += dim, ++guard;
    while (d >= half && guard < kWrapCap) d -= dim, ++guard;
    if (guard >= kWrapCap) d = d - dim * floor(d / dim + 0.5);
    return d;
}
MCACG_HD double periodic_position(double p, double dim) {
    int guard = 0;
    while (p < 0 && guard < kWrapCap) p += dim, ++guard;
    while (p >= dim && guard < kWrapCap) p -= dim, ++guard;
    if (guard >= kWrapCap) p = p - dim * floor(p / dim);
    return p;
}
MCACG_HD int periodic_cell(int i, int n) {
    i %= n;
    return i < 0 ? i + n : i;
}
MCACG_HD double dmin(double a, double b) { return (b < a) ? b : a; }  // std::min
MCACG_HD double dmax(double a, double b) { return (a < b) ? b : a; }  // std::max

struct Vec3 {
    double x, y, z;
};

// Periodic squared distance (spheres/sphere_distances.cpp:68-76).
MCACG_HD double periodic_distance_2(Vec3 a, Vec3 b, double L) {
    double dx = periodic_distance(a.x - b.x, L);
    double dy = periodic_distance(a.y - b.y, L);
    double dz = periodic_distance(a.z - b.z, L);
    return dx * dx + dy * dy + dz * dz;
}

// Sphere-sphere contact test with the 1e-28 tolerance
// (spheres/sphere_distances.cpp:81-90).
MCACG_HD bool spheres_in_contact(Vec3 p1, double r1, Vec3 p2, double r2, double L) {
    double d2 = periodic_distance_2(p1, p2, L);
    double s = r1 + r2;
    return d2 - s * s <= kContactEpsilon;
}

// Travel distance along 'dir' before sphere 1 touches sphere 2, +inf when
// they do not meet within 'dist' -- the swept test of
// spheres/sphere_contact.cpp:47-125, operation for operation. Returns 0 when
// the spheres already touch. 'dir' is a unit vector.
MCACG_HD double sweep_contact_distance(Vec3 p1, double r1, Vec3 p2, double r2, Vec3 dir, double dist,
                                       double L) {
    const double dc = r1 + r2;
    const double dc2 = dc * dc;
    if (periodic_distance_2(p1, p2, L) <= dc2) return 0.0;
    const double tx = dir.x * dist, ty = dir.y * dist, tz = dir.z * dist;
    double q[3], zone[3];
    int nper[3];
    const double pa[3] = {p1.x, p1.y, p1.z};
    const double pb[3] = {p2.x, p2.y, p2.z};
    const double td[3] = {tx, ty, tz};
MCACG_UNROLL
    for (int l = 0; l < 3; ++l) {
        double moved = pa[l] + td[l];
        double base = dmin(pa[l], moved) - dc;
        double end = dmax(pa[l], moved) + dc;
        zone[l] = end - base;
        double w = fmod(pb[l] - base, L);
        if (w < 0) w += L;
        q[l] = w + base;
        // images to visit; the cap only bites for sweeps longer than 16 boxes
        double np = floor(zone[l] / L);
        nper[l] = (np >= 0 && np <= 16) ? static_cast<int>(np) : (np > 16 ? 16 : 0);
    }
    double res = std::numeric_limits<double>::infinity();
    for (int i = 0; i <= nper[0]; i++) {
        for (int j = 0; j <= nper[1]; j++) {
            for (int k = 0; k <= nper[2]; k++) {
                double p3x = q[0] + i * L, p3y = q[1] + j * L, p3z = q[2] + k * L;
                double dx = p3x - p1.x, dy = p3y - p1.y, dz = p3z - p1.z;
                if (fabs(dx) > zone[0]) continue;
                if (fabs(dy) > zone[1]) continue;
                if (fabs(dz) > zone[2]) continue;
                double proj = dx * dir.x + dy * dir.y + dz * dir.z;
                if (proj < 0) continue;
                double ex = (p1.x + tx) - p3x, ey = (p1.y + ty) - p3y, ez = (p1.z + tz) - p3z;
                bool end_contact = ex * ex + ey * ey + ez * ez <= dc2;
                if ((!end_contact) && dist < proj) continue;
                double cx = dy * dir.z - dz * dir.y;
                double cy = dz * dir.x - dx * dir.z;
                double cz = dx * dir.y - dy * dir.x;
                double axis = cx * cx + cy * cy + cz * cz;
                if (axis > dc2) continue;
                res = dmin(res, proj - sqrt(dc2 - axis));
            }
        }
    }
    return res;
}

// Verlet cell of a position (aggregats/aggregat.cpp:699-705): step is
// double(n_div) / box_length.
MCACG_HD int verlet_coord(double x, double step) { return static_cast<int>(floor(x * step)); }

// Bounds of Verlet::get_neighborhood (verlet/verlet.cpp:52-78): inclusive cell
// ranges [lo, hi] per axis, before periodic wrapping.
struct CellRange {
    int lo[3], hi[3];
};
// Intersection (spheres/sphere_intersection.cpp:29-66): the volume and
// surface of the cap that sphere 1 loses to sphere 2 at centre distance
// 'dist' (v1, s1) and the other way round (v2, s2); a sphere inside the
// other loses all of itself (its stored volume and surface).
struct SphereCaps {
    double v1, v2, s1, s2;
};
MCACG_HD SphereCaps sphere_caps(double r1, double vol1, double sur1, double r2, double vol2, double sur2,
                                double dist) {
    SphereCaps c{0., 0., 0., 0.};
    if (dist <= 0) return c;
    if (dist < r1 + r2) {
        const double fd = r1 > r2 ? r1 - r2 : 0.0;  // std::fdim
        if (dist >= fd) {
            const double pi = pi_value();
            const double a = r1 - dist, bb = r2 - dist;
            const double h1 = (r2 * r2 - a * a) / (2. * dist);
            const double h2 = (r1 * r1 - bb * bb) / (2. * dist);
            c.v1 = pi * (h1 * h1) * (3 * r1 - h1) / 3.;
            c.v2 = pi * (h2 * h2) * (3 * r2 - h2) / 3.;
            c.s1 = 2 * pi * r1 * h1;
            c.s2 = 2 * pi * r2 * h2;
        } else if (r1 < r2) {
            c.v1 = vol1;
            c.s1 = sur1;
        } else {
            c.v2 = vol2;
            c.s2 = sur2;
        }
    }
    return c;
}
// volume_alpha_correction / surface_alpha_correction (aggregat.cpp:289-319)
MCACG_HD double volume_alpha(double cn, double c20, double c30, double min_cn, double extreme) {
    const double d = fabs(cn - min_cn);
    double corr = 0.25 * (3.0 * c20 - c30) * cn - c30 * d * 0.62741833 - pow(d, 1.5) * 0.00332425;
    if (corr < 0.0) corr = 1.0;
    corr = dmin(corr, 1.0);
    return dmax(1.0 - corr, extreme);
}
MCACG_HD double surface_alpha(double cn, double c10, double min_cn, double extreme) {
    const double d = fabs(cn - min_cn);
    double corr = 0.5 * c10 * cn - (c10 * c10) * d * 0.70132500 - (d * d) * 0.00450000;
    if (corr < 0.0) corr = 1.0;
    corr = dmin(corr, 1.0);
    return dmax(1.0 - corr, extreme);
}
// The sums of the "alphas" method over one contact of sphere i (radius r1)
// with sphere j (radius r2) at distance d (aggregat.cpp:394-413).
struct AlphaSums {
    double overlapping, c_s10, c_v20, c_v30, vp_sum, sp_sum;
};
MCACG_HD void alpha_add(AlphaSums &a, double r1, double r2, double d) {
    const double c = (r1 + r2 - d) / (r1 + r2);
    const double vp1 = pow(r1, 3), vp2 = pow(r2, 3);
    const double sp1 = r1 * r1, sp2 = r2 * r2;
    a.vp_sum += (vp1 + vp2);
    a.sp_sum += (sp1 + sp2);
    a.overlapping += c;
    a.c_s10 += c * (sp1 + sp2);
    a.c_v20 += (c * c) * (vp1 + vp2);
    a.c_v30 += pow(c, 3) * (vp1 + vp2);
}
// The end of the "alphas" method: averages, coordination, and the corrected
// volume and surface (aggregat.cpp:414-425); n spheres, 'entries' map
// entries (each contact counted from both spheres).
MCACG_HD void alpha_finish(const AlphaSums &a0, int n, int entries, double *volume, double *surface,
                           double *overlapping, double *coordination) {
    *overlapping = a0.overlapping;
    if (entries > 0) {
        const double c_s10 = a0.c_s10 / a0.sp_sum, c_v20 = a0.c_v20 / a0.vp_sum, c_v30 = a0.c_v30 / a0.vp_sum;
        const double min_cn = 2 * (1.0 - 1.0 / static_cast<double>(n));
        *overlapping = a0.overlapping / static_cast<double>(entries);
        *coordination = static_cast<double>(entries) / static_cast<double>(n);
        const double extreme = 1.0 / static_cast<double>(n);
        *volume *= volume_alpha(*coordination, c_v20, c_v30, min_cn, extreme);
        *surface *= surface_alpha(*coordination, c_s10, min_cn, extreme);
    }
}

// floor(a / w) as the reference computes it (the correctly rounded quotient,
// then floor) from the product a * inv_w, inv_w = 1 / w rounded: the product
// is within 2 ulp of the quotient, so the two floors agree unless an integer
// lies within 4 ulp of the product; then the division decides.
MCACG_HD double floor_div(double a, double w, double inv_w) {
    const double q = a * inv_w;
    const double f = floor(q);
    const double tol = fabs(q) * 0x1p-50 + 0x1p-50;
    const double g = q - f;  // exact
    if (g > tol && g < 1.0 - tol) return f;
    return floor(a / w);
}
// One axis of Verlet::get_neighborhood (verlet/verlet.cpp:52-78): the
// inclusive cell range [lo, hi] before periodic wrapping, the whole axis
// when it spans n_div cells or more (or is not finite).
MCACG_HD void neighborhood_axis(double s, double v, double distance, int n_div, double width, double inv_width,
                                int *lo_out, int *hi_out) {
    const double p = s + distance + dmax(v, 0.);
    const double m = s - distance + dmin(v, 0.);
    const double lo = floor_div(static_cast<double>(n_div) * m, width, inv_width);
    const double hi = floor_div(static_cast<double>(n_div) * p, width, inv_width) + 1;
    if (!(hi - lo < n_div) || !(lo > -1e9) || !(hi < 1e9) || int(hi) - int(lo) >= n_div) {
        *lo_out = 0;
        *hi_out = n_div - 1;
        return;
    }
    *lo_out = static_cast<int>(lo);
    *hi_out = static_cast<int>(hi);
}
MCACG_HD CellRange neighborhood_range(Vec3 src, Vec3 vec, double distance, int n_div, double width) {
    const double s[3] = {src.x, src.y, src.z};
    const double v[3] = {vec.x, vec.y, vec.z};
    CellRange r;
MCACG_UNROLL
    for (int l = 0; l < 3; ++l) neighborhood_axis(s[l], v[l], distance, n_div, width, 1.0 / width, &r.lo[l], &r.hi[l]);
    return r;
}

// Status codes: 0-11 mirror the reference's ErrorCodes
// (include/constants.hpp:70-83); 100+ are this library's own.
enum Status : int {
    ST_OK = 0,
    ST_UNKNOWN = 1,
    ST_IO = 2,
    ST_VERLET = 3,
    ST_INPUT = 4,
    ST_ABANDON = 5,
    ST_TOO_DENSE = 6,
    ST_SBL = 7,
    ST_VOL_SURF = 8,
    ST_MERGE = 9,
    ST_ARVO = 10,
    ST_INTERPOTENTIAL = 11,
    ST_CUDA = 100,
    ST_CAPACITY = 101,
    ST_TIMEOUT = 102,
    ST_BAD_ARGUMENT = 103,
    ST_NO_DEVICE = 104,
};

}  // namespace mcacg
