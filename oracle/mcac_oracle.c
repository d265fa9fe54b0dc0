/*
 * mcac_oracle.c -- CPU restatement of the MCAC MC loop (collisions, surface
 * growth and oxidation).
 *
 * TEST INFRASTRUCTURE: the oracle of the test suite and the CPU baseline of
 * bench.py. Never linked by the product. Each function names the reference
 * code it restates (paths relative to the reference repository). Compiled
 * with -ffp-contract=off so every FP64 expression rounds like the reference
 * build with contraction off.
 */
#include "mcac_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------ constants */
/* include/constants.hpp:123-139 */
#define PI 3.141592653589793115997963468544185161590576171875
static const double kBoltzmann = 1.38066E-23;
static const double kContactEpsilon = 1e-28;
static const double kCoordinationEpsilon = 1e-10;

enum { S_X, S_Y, S_Z, S_R, S_VOL, S_SURF, S_RX, S_RY, S_RZ };
enum {
    A_RG, A_F_AGG, A_LPM, A_TIME_STEP, A_RMAX, A_VOLUME, A_SURFACE, A_X, A_Y, A_Z, A_RX, A_RY, A_RZ, A_TIME,
    A_DP, A_DG_OVER_DP, A_OVERLAPPING, A_COORDINATION, A_CHARGE, A_D_M, A_CH_RATIO
};

/* ------------------------------------------------------- small vectors */
typedef struct {
    int64_t *v;
    int64_t n, cap;
} ivec;

static void iv_reserve(ivec *a, int64_t cap) {
    if (cap <= a->cap) return;
    int64_t c = a->cap ? a->cap : 4;
    while (c < cap) c *= 2;
    a->v = (int64_t *)realloc(a->v, (size_t)c * sizeof(int64_t));
    a->cap = c;
}
static void iv_push(ivec *a, int64_t x) {
    iv_reserve(a, a->n + 1);
    a->v[a->n++] = x;
}
/* sorted-set helpers: std::set<size_t> of a Verlet cell (verlet/verlet.hpp:29) */
static int64_t iv_lower_bound(const ivec *a, int64_t x) {
    int64_t lo = 0, hi = a->n;
    while (lo < hi) {
        int64_t mid = (lo + hi) / 2;
        if (a->v[mid] < x) lo = mid + 1; else hi = mid;
    }
    return lo;
}
static void set_insert(ivec *a, int64_t x) {
    int64_t k = iv_lower_bound(a, x);
    if (k < a->n && a->v[k] == x) return;
    iv_reserve(a, a->n + 1);
    memmove(a->v + k + 1, a->v + k, (size_t)(a->n - k) * sizeof(int64_t));
    a->v[k] = x;
    a->n++;
}
static void set_erase(ivec *a, int64_t x) {
    int64_t k = iv_lower_bound(a, x);
    if (k >= a->n || a->v[k] != x) return;
    memmove(a->v + k, a->v + k + 1, (size_t)(a->n - k - 1) * sizeof(int64_t));
    a->n--;
}

/* ---------------------------------------------------------------- box */
struct mo_box {
    mo_params p;
    double L, time, maxradius, max_time_step, avg_npp;
    int n_div;
    int64_t ns, na;
    double *sph[9];
    double *volw;  /* each sphere's volume as the last Aggregate::update counted it */
    int64_t *sph_label;
    double *agg[21];  /* by label (positional list, aggregat_list.hpp:29) */
    int64_t *agg_n;
    int64_t *agg_uid; /* identity of each aggregate (the reference's weak pointers) */
    int64_t next_uid;
    ivec *members;
    int64_t (*vidx)[3];
    ivec *cells;
    int64_t *index_sorted;
    double *cumulative, *tp;
    int64_t n_iter_without_event;
    int event;
};

#define SPH(b, f, s) ((b)->sph[f][s])
#define AGG(b, f, a) ((b)->agg[f][a])

/* -------------------------------------------------- periodic helpers */
/* include/physical_model/physical_model.hpp:99-126 */
static double periodic_distance(double d, double dim) {
    double half = 0.5 * dim;
    while (d < -half) d += dim;
    while (d >= half) d -= dim;
    return d;
}
static double periodic_position(double p, double dim) {
    while (p < 0) p += dim;
    while (p >= dim) p -= dim;
    return p;
}
static int periodic_int(int i, int n) {
    while (i < 0) i += n;
    while (i >= n) i -= n;
    return i;
}
static double dmin(double a, double b) { return (b < a) ? b : a; }
static double dmax(double a, double b) { return (a < b) ? b : a; }

/* spheres/sphere_distances.cpp:68-90 */
static double distance_2(const double a[3], const double b[3], double L) {
    double dx = periodic_distance(a[0] - b[0], L);
    double dy = periodic_distance(a[1] - b[1], L);
    double dz = periodic_distance(a[2] - b[2], L);
    return dx * dx + dy * dy + dz * dz;
}
static int contact(const double a[3], double ra, const double b[3], double rb, double L) {
    double d = distance_2(a, b, L);
    double dc = (ra + rb) * (ra + rb);
    return d - dc <= kContactEpsilon;
}

/* spheres/sphere_contact.cpp:47-125: swept sphere-sphere contact distance */
static double sweep(const double p1[3], double r1, const double p2in[3], double r2, const double dir[3], double dist,
                    double L) {
    double dc = r1 + r2;
    double dc2 = dc * dc;
    if (distance_2(p1, p2in, L) <= dc2) return 0.;
    double td[3] = {dir[0] * dist, dir[1] * dist, dir[2] * dist};
    double p2[3], zone[3];
    int nper[3];
    for (int l = 0; l < 3; ++l) {
        double base = dmin(p1[l], p1[l] + td[l]) - dc;
        double end = dmax(p1[l], p1[l] + td[l]) + dc;
        zone[l] = end - base;
        p2[l] = fmod((p2in[l] - base), L);
        if (p2[l] < 0) p2[l] += L;
        p2[l] += base;
        nper[l] = (int)floor(zone[l] / L);
    }
    double res = INFINITY;
    for (int i = 0; i <= nper[0]; i++)
        for (int j = 0; j <= nper[1]; j++)
            for (int k = 0; k <= nper[2]; k++) {
                double p3[3] = {p2[0] + i * L, p2[1] + j * L, p2[2] + k * L};
                double diff[3] = {p3[0] - p1[0], p3[1] - p1[1], p3[2] - p1[2]};
                if (fabs(diff[0]) > zone[0]) continue;
                if (fabs(diff[1]) > zone[1]) continue;
                if (fabs(diff[2]) > zone[2]) continue;
                double proj = diff[0] * dir[0] + diff[1] * dir[1] + diff[2] * dir[2];
                if (proj < 0) continue;
                double e[3] = {(p1[0] + td[0]) - p3[0], (p1[1] + td[1]) - p3[1], (p1[2] + td[2]) - p3[2]};
                int end_contact = e[0] * e[0] + e[1] * e[1] + e[2] * e[2] <= dc2;
                if ((!end_contact) && dist < proj) continue;
                double c0 = diff[1] * dir[2] - diff[2] * dir[1];
                double c1 = diff[2] * dir[0] - diff[0] * dir[2];
                double c2 = diff[0] * dir[1] - diff[1] * dir[0];
                double axis = c0 * c0 + c1 * c1 + c2 * c2;
                if (axis > dc2) continue;
                res = dmin(res, proj - sqrt(dc2 - axis));
            }
    return res;
}

/* ------------------------------------------------------------ Verlet */
static ivec *cell(mo_box *b, const int64_t idx[3]) {
    return &b->cells[(idx[0] * b->n_div + idx[1]) * b->n_div + idx[2]];
}
/* aggregats/aggregat.cpp:699-705 */
static void verlet_index(const mo_box *b, int64_t a, int64_t out[3]) {
    double step = (double)b->n_div / b->L;
    out[0] = (int64_t)floor(AGG(b, A_X, a) * step);
    out[1] = (int64_t)floor(AGG(b, A_Y, a) * step);
    out[2] = (int64_t)floor(AGG(b, A_Z, a) * step);
    for (int l = 0; l < 3; ++l) {  /* a position rounding onto the box edge */
        if (out[l] >= b->n_div) out[l] = b->n_div - 1;
        if (out[l] < 0) out[l] = 0;
    }
}
/* aggregats/aggregat.cpp:706-717 */
static void update_verlet(mo_box *b, int64_t a) {
    int64_t ni[3];
    verlet_index(b, a, ni);
    if (ni[0] != b->vidx[a][0] || ni[1] != b->vidx[a][1] || ni[2] != b->vidx[a][2]) {
        set_erase(cell(b, b->vidx[a]), a);
        memcpy(b->vidx[a], ni, sizeof ni);
        set_insert(cell(b, ni), a);
    }
}
/* aggregats/aggregat.cpp:109-118 */
static void set_position(mo_box *b, int64_t a, const double pos[3]) {
    AGG(b, A_X, a) = periodic_position(pos[0], b->L);
    AGG(b, A_Y, a) = periodic_position(pos[1], b->L);
    AGG(b, A_Z, a) = periodic_position(pos[2], b->L);
    update_verlet(b, a);
}
/* verlet/verlet.cpp:52-98: labels of the cells around a swept sphere */
static void neighborhood(const mo_box *b, const double src[3], const double vec[3], double distance, ivec *out) {
    int lo[3], hi[3];
    for (int l = 0; l < 3; ++l) {
        double p = src[l] + distance + dmax(vec[l], 0.);
        double m = src[l] - distance + dmin(vec[l], 0.);
        lo[l] = (int)floor((double)b->n_div * m / b->L);
        hi[l] = (int)(floor((double)b->n_div * p / b->L) + 1);
        if (hi[l] - lo[l] >= b->n_div) {
            lo[l] = 0;
            hi[l] = b->n_div - 1;
        }
    }
    out->n = 0;
    for (int i = lo[0]; i <= hi[0]; i++)
        for (int j = lo[1]; j <= hi[1]; j++)
            for (int k = lo[2]; k <= hi[2]; k++) {
                int64_t idx[3] = {periodic_int(i, b->n_div), periodic_int(j, b->n_div), periodic_int(k, b->n_div)};
                const ivec *c = &b->cells[(idx[0] * b->n_div + idx[1]) * b->n_div + idx[2]];
                iv_reserve(out, out->n + c->n);
                memcpy(out->v + out->n, c->v, (size_t)c->n * sizeof(int64_t));
                out->n += c->n;
            }
}

/* ------------------------------------------------------------ physics */
/* physical_model.cpp:550-617 */
static double cunningham(const mo_params *p, double r) {
    double a = 1.142, bb = 0.558, c = 0.999;
    return 1.0 + a * p->gaz_mean_free_path / r + bb * p->gaz_mean_free_path / r * exp(-c * r / p->gaz_mean_free_path);
}
static double friction_exponent(const mo_params *p, double r) {
    return 0.689 * (1. + erf(((p->gaz_mean_free_path / r) + 4.454) / 10.628));
}
static double friction_coeff(const mo_params *p, double V, double v, double r) {
    double fe = friction_exponent(p, r);
    double cc = cunningham(p, r);
    return (6. * PI * p->viscosity * r / cc) * pow(V / v, fe / p->fractal_dimension);
}
static double mobility_diameter(const mo_params *p, double V, double v, double r) {
    double fe = friction_exponent(p, r);
    double ar = r * pow(V / v, fe / p->fractal_dimension / 2.0);
    double cc_pp = cunningham(p, r);
    double cc_a = cunningham(p, ar);
    return (cc_a / cc_pp) * 2.0 * r * pow(V / v, fe / p->fractal_dimension);
}

/* Aggregate::update (aggregat.cpp:247-288, 321-483, 719-764), method
 * "none": all FP64 sums in list order; with 'partial', update_partial
 * (aggregat.cpp:247-282): no overlap or volume pass, the centre of mass and
 * Rg weighed with the sphere volumes the last update counted, the
 * aggregate's volume as it was. Returns 0 or the VolSurfError code. */
static int update_aggregate_part(mo_box *b, int64_t a, int partial);
static int update_aggregate(mo_box *b, int64_t a) { return update_aggregate_part(b, a, 0); }
static int update_aggregate_part(mo_box *b, int64_t a, int partial) {
    const ivec *m = &b->members[a];
    const int64_t n = m->n;
    double V = AGG(b, A_VOLUME, a);
    if (!partial) {
        double overlapping = 0.0, coordination = 0.0;
        int64_t inter = 0;
        for (int64_t i = 0; i < n; i++)
            for (int64_t j = i + 1; j < n; j++) {
                int64_t si = m->v[i], sj = m->v[j];
                double dx = SPH(b, S_RX, si) - SPH(b, S_RX, sj), dy = SPH(b, S_RY, si) - SPH(b, S_RY, sj),
                       dz = SPH(b, S_RZ, si) - SPH(b, S_RZ, sj);
                double dist = sqrt(dx * dx + dy * dy + dz * dz);
                if (dist <= (1. + kCoordinationEpsilon) * (SPH(b, S_R, si) + SPH(b, S_R, sj))) {
                    double cij = (SPH(b, S_R, si) + SPH(b, S_R, sj) - dist) / (SPH(b, S_R, si) + SPH(b, S_R, sj));
                    overlapping += 2.0 * cij;
                    inter += 2;
                }
            }
        if (inter > 0) {
            overlapping /= (double)inter;
            coordination = (double)inter / (double)n;
        }
        double Sf = 0.0;
        V = 0.0;
        for (int64_t i = 0; i < n; i++) {
            V = V + SPH(b, S_VOL, m->v[i]);
            Sf = Sf + SPH(b, S_SURF, m->v[i]);
            b->volw[m->v[i]] = SPH(b, S_VOL, m->v[i]);
        }
        AGG(b, A_VOLUME, a) = V;
        AGG(b, A_SURFACE, a) = Sf;
        AGG(b, A_OVERLAPPING, a) = overlapping;
        AGG(b, A_COORDINATION, a) = coordination;
        if (V <= 0 || Sf <= 0) return 8;
    }
    double r[3] = {0., 0., 0.};
    for (int64_t i = 0; i < n; i++) {
        int64_t s = m->v[i];
        double vol = b->volw[s];
        r[0] += SPH(b, S_RX, s) * vol;
        r[1] += SPH(b, S_RY, s) * vol;
        r[2] += SPH(b, S_RZ, s) * vol;
    }
    r[0] /= V;
    r[1] /= V;
    r[2] /= V;
    double *dcen = (double *)malloc((size_t)n * sizeof(double));
    for (int64_t i = 0; i < n; i++) {
        int64_t s = m->v[i];
        double dx = SPH(b, S_RX, s) - r[0], dy = SPH(b, S_RY, s) - r[1], dz = SPH(b, S_RZ, s) - r[2];
        dcen[i] = sqrt(dx * dx + dy * dy + dz * dz);
    }
    int64_t s0 = m->v[0];
    double pos[3] = {SPH(b, S_X, s0) + r[0], SPH(b, S_Y, s0) + r[1], SPH(b, S_Z, s0) + r[2]};
    set_position(b, a, pos);
    AGG(b, A_RX, a) = r[0];
    AGG(b, A_RY, a) = r[1];
    AGG(b, A_RZ, a) = r[2];
    double rmax = 0.0;
    for (int64_t i = 0; i < n; i++) rmax = dmax(rmax, SPH(b, S_R, m->v[i]) + dcen[i]);
    AGG(b, A_RMAX, a) = rmax;
    double arg = 0., brg = 0.;
    for (int64_t i = 0; i < n; i++) {
        double vol = b->volw[m->v[i]], rs = SPH(b, S_R, m->v[i]);
        arg = arg + vol * (dcen[i] * dcen[i]);
        brg = brg + vol * (rs * rs);
    }
    free(dcen);
    double rg = sqrt(fabs((arg + 3. / 5. * brg) / V));
    AGG(b, A_RG, a) = rg;
    double dp = 0., vol_pp = 0.;
    for (int64_t i = 0; i < n; i++) {
        vol_pp += SPH(b, S_VOL, m->v[i]);
        dp += SPH(b, S_R, m->v[i]);
    }
    dp = 2 * dp / (double)n;
    vol_pp = vol_pp / (double)n;
    AGG(b, A_DP, a) = dp;
    const mo_params *p = &b->p;
    double f = friction_coeff(p, V, vol_pp, 0.5 * dp);
    AGG(b, A_F_AGG, a) = f;
    AGG(b, A_D_M, a) = mobility_diameter(p, V, vol_pp, 0.5 * dp);
    double masse = p->density * V;
    double relax = masse / f;
    AGG(b, A_TIME_STEP, a) = 3. * relax;
    double diffusivity = kBoltzmann * p->temperature / f;
    AGG(b, A_LPM, a) = sqrt(6. * diffusivity * AGG(b, A_TIME_STEP, a));
    AGG(b, A_DG_OVER_DP, a) = 2 * rg / dp;
    if (rmax > b->maxradius) b->maxradius = rmax;
    return 0;
}

/* ------------------------------------------------------------ random */
/* tools/tools.cpp:59-107 on the C library generator */
static double rnd(void) {
    double v = rand();
    v = v / RAND_MAX;
    return v;
}
static double inverfc(double p) {
    if (p >= 2.) return -100.;
    if (p <= 0.0) return 100.;
    double pp = (p < 1.0) ? p : 2. - p;
    double t = sqrt(-2. * log(pp / 2.));
    double x = -0.70711 * ((2.30753 + t * 0.27061) / (1. + t * (0.99229 + t * 0.04481)) - t);
    for (int j = 0; j < 2; j++) {
        double err = erfc(x) - pp;
        x += err / (1.12837916709551257 * exp(-(x * x)) - x * err);
    }
    return (p < 1.0 ? x : -x);
}
static double inverf(double p) { return inverfc(1. - p); }
static void random_direction(double out[3]) {
    double theta = rnd() * 2 * PI;
    double phi = acos(1 - 2 * rnd());
    out[0] = sin(phi) * cos(theta);
    out[1] = sin(phi) * sin(theta);
    out[2] = cos(phi);
}
/* physical_model.cpp:557-578 */
static int random_diameter(const mo_params *p, double *d) {
    double x;
    if (p->initialisation_mode == 1) {
        x = p->mean_diameter + sqrt(2.) * p->dispersion_diameter * inverf(2. * rnd() - 1.0);
    } else {
        if (p->dispersion_diameter < 1.0) return 4;
        x = p->mean_diameter * pow(p->dispersion_diameter, sqrt(2.) * inverf(2. * rnd() - 1.0));
    }
    if (x <= 0) x = p->mean_diameter;
    *d = x * 1E-9;
    return 0;
}

/* --------------------------------------------------------- allocation */
static mo_box *alloc_box(const mo_params *p, int64_t ns, int64_t na, int n_div, double L) {
    mo_box *b = (mo_box *)calloc(1, sizeof(mo_box));
    b->p = *p;
    b->L = L;
    b->n_div = n_div;
    b->ns = ns;
    b->na = na;
    for (int f = 0; f < 9; ++f) b->sph[f] = (double *)calloc((size_t)ns, sizeof(double));
    b->volw = (double *)calloc((size_t)ns, sizeof(double));
    b->sph_label = (int64_t *)calloc((size_t)ns, sizeof(int64_t));
    /* room for an aggregate per sphere: oxidation splits append aggregates */
    const int64_t cap = na > ns ? na : ns;
    for (int f = 0; f < 21; ++f) b->agg[f] = (double *)calloc((size_t)cap, sizeof(double));
    b->agg_n = (int64_t *)calloc((size_t)cap, sizeof(int64_t));
    b->agg_uid = (int64_t *)calloc((size_t)cap, sizeof(int64_t));
    for (int64_t a = 0; a < na; ++a) b->agg_uid[a] = a;
    b->next_uid = na;
    b->members = (ivec *)calloc((size_t)cap, sizeof(ivec));
    b->vidx = (int64_t(*)[3])calloc((size_t)cap, sizeof(int64_t[3]));
    b->cells = (ivec *)calloc((size_t)n_div * n_div * n_div, sizeof(ivec));
    b->index_sorted = (int64_t *)calloc((size_t)cap, sizeof(int64_t));
    b->cumulative = (double *)calloc((size_t)cap, sizeof(double));
    b->tp = (double *)calloc((size_t)cap, sizeof(double));
    b->event = 1;
    return b;
}

void mo_box_free(mo_box *b) {
    if (!b) return;
    for (int f = 0; f < 9; ++f) free(b->sph[f]);
    free(b->volw);
    free(b->sph_label);
    for (int f = 0; f < 21; ++f) free(b->agg[f]);
    free(b->agg_n);
    free(b->agg_uid);
    for (int64_t a = 0; a < b->na; ++a) free(b->members[a].v);
    free(b->members);
    free(b->vidx);
    for (int64_t c = 0; c < (int64_t)b->n_div * b->n_div * b->n_div; ++c) free(b->cells[c].v);
    free(b->cells);
    free(b->index_sorted);
    free(b->cumulative);
    free(b->tp);
    free(b);
}

int64_t mo_size(const mo_box *b) { return b->na; }
int64_t mo_n_spheres(const mo_box *b) { return b->ns; }
double mo_time(const mo_box *b) { return b->time; }
void mo_set_time(mo_box *b, double t) { b->time = t; }
void mo_set_aggregate_limit(mo_box *b, int64_t limit) { b->p.number_of_aggregates_limit = limit; }

/* Derived box length and gas properties (physical_model.cpp:228-262,
 * 536-546). */
void mo_params_derive(mo_params *p, double pressure) {
    const double n = (double)p->n_monomeres;
    double mean_massic_radius;
    if (p->initialisation_mode == 1) {
        p->box_length = p->mean_diameter * 1E-9 *
                        pow(n * PI / 6. / p->volume_fraction *
                                (1. + 3. * pow(p->dispersion_diameter / p->mean_diameter, 2)),
                            1. / 3.);
        mean_massic_radius = 0.5 * 1E-9 *
                             (pow(p->mean_diameter, 4) + 6 * pow(p->mean_diameter, 2) * pow(p->dispersion_diameter, 2) +
                              3 * pow(p->dispersion_diameter, 4)) /
                             (pow(p->mean_diameter, 3) + 3 * p->mean_diameter * pow(p->dispersion_diameter, 2));
    } else {
        p->box_length = p->mean_diameter * 1E-9 *
                        pow(n * PI / 6. / p->volume_fraction * exp(9. / 2. * pow(log(p->dispersion_diameter), 2)),
                            1. / 3.);
        mean_massic_radius = 0.5 * p->mean_diameter * 1E-9 * exp(1.5 * pow(log(p->dispersion_diameter), 2));
    }
    (void)mean_massic_radius;
    const double T = p->temperature, Tref = 293.15, Sc = 110, Pref = 101300;
    p->viscosity = 18.203E-6 * (Sc + Tref) / (Sc + T) * pow(T / Tref, 1.5);
    p->gaz_mean_free_path = 66.5E-9 * (Pref / pressure) * (T / Tref) * (1. + Sc / Tref) / (1. + Sc / T);
    p->u_sg = p->flux_surfgrowth / p->density; /* physical_model.cpp:264 */
}

/* AggregatList::refresh (aggregat_list.cpp:100-108) */
void mo_refresh(mo_box *b) {
    if (b->na < 1) return;
    b->max_time_step = AGG(b, A_TIME_STEP, 0);
    for (int64_t a = 0; a < b->na; ++a) b->max_time_step = dmax(AGG(b, A_TIME_STEP, a), b->max_time_step);
    b->avg_npp = (double)b->ns / (double)b->na;
}

/* AggregatList::AggregatList (aggregat_list_storage.cpp:52-88) with
 * Aggregate::init (aggregat.cpp:162-229) and test_free_space
 * (aggregat_list.cpp:534-548). */
int mo_box_new_random(const mo_params *p, mo_box **out) {
    const int64_t N = p->n_monomeres;
    const double L = p->box_length;
    mo_box *b = alloc_box(p, N, N, (int)p->n_verlet_divisions, L);
    b->time = p->initial_time;
    srand((unsigned)(p->random_seed < 0 ? 0 : p->random_seed));
    const double vf = 4 * PI / 3, sf = 4 * PI;
    ivec nb = {0, 0, 0};
    for (int64_t i = 0; i < N; ++i) {
        AGG(b, A_TIME, i) = b->time;
        double diameter;
        int rc = random_diameter(p, &diameter);
        if (rc) {
            free(nb.v);
            mo_box_free(b);
            return rc;
        }
        const double radius = diameter * 0.5;
        int placed = 0;
        for (int64_t n_try = 0; n_try < N; n_try++) {
            double pos[3];
            pos[0] = rnd() * L;
            pos[1] = rnd() * L;
            pos[2] = rnd() * L;
            const double zero[3] = {0, 0, 0};
            neighborhood(b, pos, zero, radius + b->maxradius, &nb);
            int busy = 0;
            for (int64_t k = 0; k < nb.n && !busy; ++k) {
                int64_t j = nb.v[k];
                double ca[3] = {AGG(b, A_X, j), AGG(b, A_Y, j), AGG(b, A_Z, j)};
                if (!contact(pos, radius, ca, AGG(b, A_RMAX, j), L)) continue;
                for (int64_t m = 0; m < b->members[j].n; ++m) {
                    int64_t s = b->members[j].v[m];
                    double cs[3] = {SPH(b, S_X, s), SPH(b, S_Y, s), SPH(b, S_Z, s)};
                    if (contact(pos, radius, cs, SPH(b, S_R, s), L)) {
                        busy = 1;
                        break;
                    }
                }
            }
            if (busy) continue;
            /* Aggregate::init(...): set_position, set_verlet, sphere, update */
            AGG(b, A_X, i) = periodic_position(pos[0], L);
            AGG(b, A_Y, i) = periodic_position(pos[1], L);
            AGG(b, A_Z, i) = periodic_position(pos[2], L);
            verlet_index(b, i, b->vidx[i]);
            set_insert(cell(b, b->vidx[i]), i);
            b->sph_label[i] = i;
            SPH(b, S_X, i) = pos[0];
            SPH(b, S_Y, i) = pos[1];
            SPH(b, S_Z, i) = pos[2];
            SPH(b, S_R, i) = radius;
            SPH(b, S_RX, i) = SPH(b, S_RY, i) = SPH(b, S_RZ, i) = 0.;
            SPH(b, S_VOL, i) = vf * pow(radius, 3);
            SPH(b, S_SURF, i) = sf * pow(radius, 2);
            iv_push(&b->members[i], i);
            b->agg_n[i] = 1;
            AGG(b, A_D_M, i) = diameter;
            rc = update_aggregate(b, i);
            if (rc) {
                free(nb.v);
                mo_box_free(b);
                return rc;
            }
            placed = 1;
            break;
        }
        if (!placed) {
            free(nb.v);
            mo_box_free(b);
            return 6; /* TooDenseError */
        }
    }
    free(nb.v);
    mo_refresh(b);
    if (p->enforce_volume_fraction) {
        double cur = 0.0;
        for (int64_t a = 0; a < N; ++a) cur += AGG(b, A_VOLUME, a);
        double pres = p->volume_fraction * pow(L, 3);
        double corr = pow(pres / cur, 1. / 3.);
        for (int64_t s = 0; s < N; ++s) {
            SPH(b, S_R, s) = SPH(b, S_R, s) * corr;
            SPH(b, S_VOL, s) = vf * pow(SPH(b, S_R, s), 3);
            SPH(b, S_SURF, s) = sf * pow(SPH(b, S_R, s), 2);
            b->volw[s] = SPH(b, S_VOL, s); /* compute_volume_surface's per-sphere volumes */
        }
        for (int64_t a = 0; a < N; ++a) {
            double V = 0.0, S = 0.0;
            for (int64_t m = 0; m < b->members[a].n; ++m) {
                V = V + SPH(b, S_VOL, b->members[a].v[m]);
                S = S + SPH(b, S_SURF, b->members[a].v[m]);
            }
            AGG(b, A_VOLUME, a) = V;
            AGG(b, A_SURFACE, a) = S;
        }
    }
    *out = b;
    return 0;
}

int mo_box_new_state(const mo_params *p, int64_t ns, int64_t na, int64_t n_div, double box_length, double maxradius,
                     double time, const double *spheres, const int64_t *sphere_label, const double *aggregates,
                     const int64_t *n_spheres, const int64_t *members, mo_box **out) {
    mo_box *b = alloc_box(p, ns, na, (int)n_div, box_length);
    b->time = time;
    b->maxradius = maxradius;
    for (int f = 0; f < 9; ++f) memcpy(b->sph[f], spheres + (size_t)f * ns, (size_t)ns * sizeof(double));
    memcpy(b->volw, b->sph[S_VOL], (size_t)ns * sizeof(double));
    memcpy(b->sph_label, sphere_label, (size_t)ns * sizeof(int64_t));
    for (int f = 0; f < 21; ++f) memcpy(b->agg[f], aggregates + (size_t)f * na, (size_t)na * sizeof(double));
    int64_t off = 0;
    for (int64_t a = 0; a < na; ++a) {
        b->agg_n[a] = n_spheres[a];
        for (int64_t k = 0; k < n_spheres[a]; ++k) iv_push(&b->members[a], members[off + k]);
        off += n_spheres[a];
        verlet_index(b, a, b->vidx[a]);
        set_insert(cell(b, b->vidx[a]), a);
    }
    mo_refresh(b);
    *out = b;
    return 0;
}

void mo_store(const mo_box *b, double *spheres, int64_t *sphere_label, double *aggregates, int64_t *n_spheres,
              int64_t *members, double *scalars3) {
    for (int f = 0; f < 9; ++f) memcpy(spheres + (size_t)f * b->ns, b->sph[f], (size_t)b->ns * sizeof(double));
    memcpy(sphere_label, b->sph_label, (size_t)b->ns * sizeof(int64_t));
    for (int f = 0; f < 21; ++f) memcpy(aggregates + (size_t)f * b->na, b->agg[f], (size_t)b->na * sizeof(double));
    int64_t off = 0;
    for (int64_t a = 0; a < b->na; ++a) {
        n_spheres[a] = b->members[a].n;
        memcpy(members + off, b->members[a].v, (size_t)b->members[a].n * sizeof(int64_t));
        off += b->members[a].n;
    }
    scalars3[0] = b->maxradius;
    scalars3[1] = b->time;
    scalars3[2] = b->L;
}

/* ------------------------------------------------------ contact search */
/* AggregatList::distance_to_next_contact (aggregat_list.cpp:447-532) with
 * distance_to_contact(Aggregate, Aggregate) (aggregat_distance.cpp:24-44). */
typedef struct {
    double d;
    int64_t label;
} keyed;

int mo_distance_to_next_contact(mo_box *b, int64_t source, const double dir[3], double distance, mo_contact *out) {
    out->distance = INFINITY;
    out->moving_sphere = out->other_sphere = out->moving_aggregate = out->other_aggregate = -1;
    const double mindist = AGG(b, A_RMAX, source) + b->maxradius;
    const double src[3] = {AGG(b, A_X, source), AGG(b, A_Y, source), AGG(b, A_Z, source)};
    const double vec[3] = {distance * dir[0], distance * dir[1], distance * dir[2]};
    ivec nb = {0, 0, 0};
    neighborhood(b, src, vec, mindist, &nb);
    int64_t found = -1;
    for (int64_t i = 0; i < nb.n; ++i)
        if (nb.v[i] == source) {
            found = i;
            break;
        }
    if (found < 0) {
        free(nb.v);
        return 3; /* VerletError */
    }
    memmove(nb.v + found, nb.v + found + 1, (size_t)(nb.n - found - 1) * sizeof(int64_t));
    nb.n--;
    /* filter_neighborhood: multimap ordered by bounding distance, ties in
     * insertion order */
    keyed *mm = (keyed *)malloc((size_t)(nb.n + 1) * sizeof(keyed));
    int64_t nm = 0;
    const double rs = AGG(b, A_RMAX, source);
    for (int64_t i = 0; i < nb.n; ++i) {
        int64_t o = nb.v[i];
        double po[3] = {AGG(b, A_X, o), AGG(b, A_Y, o), AGG(b, A_Z, o)};
        double d = sweep(src, rs, po, AGG(b, A_RMAX, o), dir, distance, b->L);
        if (d < distance) {
            int64_t k = nm;
            while (k > 0 && mm[k - 1].d > d) {  /* upper bound: after equal keys */
                mm[k] = mm[k - 1];
                --k;
            }
            mm[k].d = d;
            mm[k].label = o;
            nm++;
        }
    }
    free(nb.v);
    const ivec *mov = &b->members[source];
    for (int64_t c = 0; c < nm; ++c) {
        if (out->distance <= 0.) break;
        if (out->distance < mm[c].d) break;
        const int64_t o = mm[c].label;
        const ivec *oth = &b->members[o];
        double best = INFINITY;
        int64_t bi = -1, bj = -1;
        for (int64_t i = 0; i < mov->n; ++i) {
            int64_t si = mov->v[i];
            double p1[3] = {SPH(b, S_X, si), SPH(b, S_Y, si), SPH(b, S_Z, si)};
            double half = INFINITY;
            int64_t hj = -1;
            for (int64_t j = 0; j < oth->n; ++j) {
                int64_t sj = oth->v[j];
                double p2[3] = {SPH(b, S_X, sj), SPH(b, S_Y, sj), SPH(b, S_Z, sj)};
                double r = sweep(p1, SPH(b, S_R, si), p2, SPH(b, S_R, sj), dir, distance, b->L);
                if (r < half) {
                    half = r;
                    hj = sj;
                }
            }
            if (half < best) {
                best = half;
                bi = si;
                bj = hj;
            }
        }
        if (best < out->distance) {
            out->distance = best;
            out->moving_sphere = bi;
            out->other_sphere = bj;
            out->moving_aggregate = source;
            out->other_aggregate = o;
        }
    }
    free(mm);
    return 0;
}

/* Aggregate::translate (aggregat.cpp:148-161) */
void mo_translate(mo_box *b, int64_t a, const double v[3]) {
    double pos[3] = {AGG(b, A_X, a) + v[0], AGG(b, A_Y, a) + v[1], AGG(b, A_Z, a) + v[2]};
    set_position(b, a, pos);
    double ref[3] = {AGG(b, A_X, a) - AGG(b, A_RX, a), AGG(b, A_Y, a) - AGG(b, A_RY, a),
                     AGG(b, A_Z, a) - AGG(b, A_RZ, a)};
    const ivec *m = &b->members[a];
    for (int64_t k = 0; k < m->n; ++k) {
        int64_t s = m->v[k];
        SPH(b, S_X, s) = ref[0] + SPH(b, S_RX, s);
        SPH(b, S_Y, s) = ref[1] + SPH(b, S_RY, s);
        SPH(b, S_Z, s) = ref[2] + SPH(b, S_RZ, s);
    }
}

/* AggregatList::remove (aggregat_list_storage.cpp:37-44) with
 * ListStorage::remove (list_storage_methods.hpp:78-87) and
 * Aggregate::decrease_label (aggregat.cpp:80-91): every later aggregate is
 * renumbered and re-keyed in the Verlet grid. */
static void remove_aggregate(mo_box *b, int64_t a) {
    set_erase(cell(b, b->vidx[a]), a);
    free(b->members[a].v);
    int64_t tail = b->na - a - 1;
    for (int f = 0; f < 21; ++f) memmove(b->agg[f] + a, b->agg[f] + a + 1, (size_t)tail * sizeof(double));
    memmove(b->agg_n + a, b->agg_n + a + 1, (size_t)tail * sizeof(int64_t));
    memmove(b->agg_uid + a, b->agg_uid + a + 1, (size_t)tail * sizeof(int64_t));
    memmove(b->members + a, b->members + a + 1, (size_t)tail * sizeof(ivec));
    memmove(b->vidx + a, b->vidx + a + 1, (size_t)tail * sizeof(int64_t[3]));
    b->na--;
    memset(&b->members[b->na], 0, sizeof(ivec));
    for (int64_t i = a; i < b->na; ++i) {
        ivec *c = cell(b, b->vidx[i]);
        set_erase(c, i + 1);
        for (int64_t k = 0; k < b->members[i].n; ++k) b->sph_label[b->members[i].v[k]]--;
        set_insert(c, i);
    }
}

/* AggregatList::merge (aggregat_list.cpp:367-410) and Aggregate::merge
 * (aggregat.cpp:486-544) */
int mo_merge(mo_box *b, const mo_contact *c, int32_t *merged) {
    *merged = 0;
    if (c->moving_sphere < 0 || c->other_sphere < 0) return 0;
    const int64_t ms = c->moving_sphere, os = c->other_sphere;
    double pm[3] = {SPH(b, S_X, ms), SPH(b, S_Y, ms), SPH(b, S_Z, ms)};
    double po[3] = {SPH(b, S_X, os), SPH(b, S_Y, os), SPH(b, S_Z, os)};
    if (!contact(pm, SPH(b, S_R, ms), po, SPH(b, S_R, os), b->L)) return 0;
    /* an aggregate of the contact that split or disappeared since the query
     * (aggregat.cpp:488-493): the reference's merge refuses */
    if (c->moving_aggregate < 0 || c->other_aggregate < 0) return 9; /* MergeError */
    int64_t la = b->sph_label[ms], lb = b->sph_label[os];
    int64_t keep = la < lb ? la : lb, removed = la < lb ? lb : la;
    double newtime = AGG(b, A_TIME, keep) + AGG(b, A_TIME, removed) - b->time;
    int64_t my, oth;
    if (c->moving_aggregate == keep) {
        my = ms;
        oth = os;
    } else if (c->other_aggregate == keep) {
        my = os;
        oth = ms;
    } else {
        return 9; /* MergeError */
    }
    int64_t s0 = b->members[keep].v[0];
    double refpos[3] = {SPH(b, S_X, s0), SPH(b, S_Y, s0), SPH(b, S_Z, s0)};
    double dcx = periodic_distance(SPH(b, S_X, oth) - SPH(b, S_X, my), b->L);
    double dcy = periodic_distance(SPH(b, S_Y, oth) - SPH(b, S_Y, my), b->L);
    double dcz = periodic_distance(SPH(b, S_Z, oth) - SPH(b, S_Z, my), b->L);
    double diff[3] = {SPH(b, S_RX, my) + dcx - SPH(b, S_RX, oth), SPH(b, S_RY, my) + dcy - SPH(b, S_RY, oth),
                      SPH(b, S_RZ, my) + dcz - SPH(b, S_RZ, oth)};
    ivec *rm = &b->members[removed];
    for (int64_t k = 0; k < rm->n; ++k) {
        int64_t s = rm->v[k];
        b->sph_label[s] = keep;
        SPH(b, S_RX, s) += diff[0];
        SPH(b, S_RY, s) += diff[1];
        SPH(b, S_RZ, s) += diff[2];
        SPH(b, S_X, s) = SPH(b, S_RX, s) + refpos[0];
        SPH(b, S_Y, s) = SPH(b, S_RY, s) + refpos[1];
        SPH(b, S_Z, s) = SPH(b, S_RZ, s) + refpos[2];
    }
    for (int64_t k = 0; k < rm->n; ++k) iv_push(&b->members[keep], rm->v[k]);
    b->agg_n[keep] = b->members[keep].n;
    int rc = update_aggregate(b, keep);
    if (rc) return rc;
    remove_aggregate(b, removed);
    AGG(b, A_TIME, keep) = newtime;
    *merged = 1;
    return 0;
}

/* --------------------------------------------------------- std::sort */
/* The element order of libstdc++'s std::sort (introsort: median-of-three
 * pivot, unguarded partition, heapsort below the depth limit, final
 * insertion sort with threshold 16). sort_time_steps sorts label indices by
 * time-step weight with it, and ties (identical monomers) keep the order
 * this algorithm leaves them in, so the pick depends on reproducing it. */
typedef struct {
    const double *k;
} cmpctx;
#define LESS(a, b) (ctx->k[a] < ctx->k[b])

static void iswap(int64_t *a, int64_t *b) {
    int64_t t = *a;
    *a = *b;
    *b = t;
}
static void median_to_first(const cmpctx *ctx, int64_t *res, int64_t *a, int64_t *b, int64_t *c) {
    if (LESS(*a, *b)) {
        if (LESS(*b, *c)) iswap(res, b);
        else if (LESS(*a, *c)) iswap(res, c);
        else iswap(res, a);
    } else if (LESS(*a, *c)) iswap(res, a);
    else if (LESS(*b, *c)) iswap(res, c);
    else iswap(res, b);
}
static int64_t *unguarded_partition(const cmpctx *ctx, int64_t *first, int64_t *last, int64_t *pivot) {
    for (;;) {
        while (LESS(*first, *pivot)) ++first;
        --last;
        while (LESS(*pivot, *last)) --last;
        if (!(first < last)) return first;
        iswap(first, last);
        ++first;
    }
}
static void push_heap(const cmpctx *ctx, int64_t *first, int64_t hole, int64_t top, int64_t value) {
    int64_t parent = (hole - 1) / 2;
    while (hole > top && LESS(first[parent], value)) {
        first[hole] = first[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    first[hole] = value;
}
static void adjust_heap(const cmpctx *ctx, int64_t *first, int64_t hole, int64_t len, int64_t value) {
    const int64_t top = hole;
    int64_t child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (LESS(first[child], first[child - 1])) child--;
        first[hole] = first[child];
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        first[hole] = first[child - 1];
        hole = child - 1;
    }
    push_heap(ctx, first, hole, top, value);
}
static void heap_sort(const cmpctx *ctx, int64_t *first, int64_t *last) {
    int64_t len = last - first;
    if (len >= 2) {
        for (int64_t parent = (len - 2) / 2;; --parent) {
            adjust_heap(ctx, first, parent, len, first[parent]);
            if (parent == 0) break;
        }
    }
    while (last - first > 1) {
        --last;
        int64_t value = *last;
        *last = *first;
        adjust_heap(ctx, first, 0, last - first, value);
    }
}
static void introsort_loop(const cmpctx *ctx, int64_t *first, int64_t *last, int64_t depth) {
    while (last - first > 16) {
        if (depth == 0) {
            heap_sort(ctx, first, last);
            return;
        }
        --depth;
        int64_t *mid = first + (last - first) / 2;
        median_to_first(ctx, first, first + 1, mid, last - 1);
        int64_t *cut = unguarded_partition(ctx, first + 1, last, first);
        introsort_loop(ctx, cut, last, depth);
        last = cut;
    }
}
static void linear_insert(const cmpctx *ctx, int64_t *last) {
    int64_t val = *last;
    int64_t *next = last - 1;
    while (LESS(val, *next)) {
        *last = *next;
        last = next;
        --next;
    }
    *last = val;
}
static void insertion_sort(const cmpctx *ctx, int64_t *first, int64_t *last) {
    if (first == last) return;
    for (int64_t *i = first + 1; i != last; ++i) {
        if (LESS(*i, *first)) {
            int64_t val = *i;
            memmove(first + 1, first, (size_t)(i - first) * sizeof(int64_t));
            *first = val;
        } else {
            linear_insert(ctx, i);
        }
    }
}
void mo_sort_indices(const double *keys, int64_t *idx, int64_t n) {
    cmpctx c = {keys};
    const cmpctx *ctx = &c;
    for (int64_t i = 0; i < n; ++i) idx[i] = i;
    if (n == 0) return;
    int64_t lg = 63 - __builtin_clzll((unsigned long long)n);
    introsort_loop(ctx, idx, idx + n, 2 * lg);
    if (n > 16) {
        insertion_sort(ctx, idx, idx + 16);
        for (int64_t *i = idx + 16; i != idx + n; ++i) linear_insert(ctx, i);
    } else {
        insertion_sort(ctx, idx, idx + n);
    }
}

/* AggregatList::sort_time_steps / pick_random / get_time_step
 * (aggregat_list.cpp:54-66, 124-141) */
void mo_sort_time_steps(mo_box *b, double factor) {
    for (int64_t i = 0; i < b->na; ++i) b->tp[i] = factor / AGG(b, A_TIME_STEP, i);
    mo_sort_indices(b->tp, b->index_sorted, b->na);
    b->cumulative[0] = b->tp[b->index_sorted[0]];
    for (int64_t i = 1; i < b->na; ++i) b->cumulative[i] = b->cumulative[i - 1] + b->tp[b->index_sorted[i]];
}
int64_t mo_pick_random(mo_box *b) {
    double val = rnd() * b->cumulative[b->na - 1];
    int64_t lo = 0, hi = b->na;
    while (lo < hi) { /* std::lower_bound */
        int64_t mid = lo + (hi - lo) / 2;
        if (b->cumulative[mid] < val) lo = mid + 1; else hi = mid;
    }
    return b->index_sorted[lo];
}
double mo_get_time_step(const mo_box *b, double max) { return max / b->cumulative[b->na - 1]; }

/* PhysicalModel::finished (physical_model.cpp:288-337) without the STOPCODE
 * file and CPU-time checks */
static int finished(const mo_box *b) {
    const mo_params *p = &b->p;
    if (b->na < 1) return 1;
    if ((uint64_t)b->na <= (uint64_t)p->number_of_aggregates_limit) return 1;
    if (p->n_iter_without_event_limit > 0 && b->n_iter_without_event >= p->n_iter_without_event_limit) return 1;
    if (p->physical_time_limit > 0 && b->time >= p->physical_time_limit) return 1;
    if (p->mean_monomere_per_aggregate_limit > 0 && b->avg_npp >= (double)p->mean_monomere_per_aggregate_limit)
        return 1;
    return 0;
}

/* Sphere::croissance_surface (sphere.cpp:113-120) of one aggregate's
 * spheres: r + u_sg dt, volume and surface from the new radius. */
static void grow_aggregate(mo_box *b, int64_t a, double dt) {
    const ivec *m = &b->members[a];
    for (int64_t i = 0; i < m->n; i++) {
        const int64_t s = m->v[i];
        const double r = SPH(b, S_R, s) + b->p.u_sg * dt;
        const double r2 = r * r, r3 = r2 * r;
        SPH(b, S_R, s) = r;
        SPH(b, S_VOL, s) = 4 * PI / 3 * r3;
        SPH(b, S_SURF, s) = 4 * PI * r2;
    }
}

/* ---------------------------------------------------------- oxidation */
/* spheres.remove(id) (list_storage_methods.hpp:78-87): the later spheres move
 * down one index; member lists and the tracked sphere references follow
 * (a reference to the removed sphere becomes -1, as an expired weak pointer). */
static void remove_sphere_storage(mo_box *b, int64_t id, int64_t **refs, int nrefs) {
    const int64_t tail = b->ns - id - 1;
    for (int f = 0; f < 9; ++f) memmove(b->sph[f] + id, b->sph[f] + id + 1, (size_t)tail * sizeof(double));
    memmove(b->volw + id, b->volw + id + 1, (size_t)tail * sizeof(double));
    memmove(b->sph_label + id, b->sph_label + id + 1, (size_t)tail * sizeof(int64_t));
    b->ns--;
    for (int64_t a = 0; a < b->na; ++a)
        for (int64_t k = 0; k < b->members[a].n; ++k)
            if (b->members[a].v[k] > id) b->members[a].v[k]--;
    for (int r = 0; r < nrefs; ++r) {
        if (*refs[r] == id) *refs[r] = -1;
        else if (*refs[r] > id) (*refs[r])--;
    }
}

/* Relative positions from the first sphere, Aggregate::update, then every
 * sphere placed back from the aggregate's position (remove_sphere and
 * split, aggregat.cpp:596-609, 641-654). */
static int rebase_update_place(mo_box *b, int64_t a) {
    const ivec *m = &b->members[a];
    const int64_t s0 = m->v[0];
    const double ref0[3] = {SPH(b, S_X, s0), SPH(b, S_Y, s0), SPH(b, S_Z, s0)};
    for (int64_t k = 0; k < m->n; ++k) {
        const int64_t s = m->v[k];
        SPH(b, S_RX, s) = SPH(b, S_X, s) - ref0[0];
        SPH(b, S_RY, s) = SPH(b, S_Y, s) - ref0[1];
        SPH(b, S_RZ, s) = SPH(b, S_Z, s) - ref0[2];
    }
    int rc = update_aggregate(b, a);
    if (rc) return rc;
    const double ref[3] = {AGG(b, A_X, a) - AGG(b, A_RX, a), AGG(b, A_Y, a) - AGG(b, A_RY, a),
                           AGG(b, A_Z, a) - AGG(b, A_RZ, a)};
    for (int64_t k = 0; k < m->n; ++k) {
        const int64_t s = m->v[k];
        SPH(b, S_X, s) = ref[0] + SPH(b, S_RX, s);
        SPH(b, S_Y, s) = ref[1] + SPH(b, S_RY, s);
        SPH(b, S_Z, s) = ref[2] + SPH(b, S_RZ, s);
    }
    return 0;
}

/* Aggregate::croissance_surface (aggregat.cpp:230-243) with remove_sphere
 * (aggregat.cpp:629-655): the spheres shrink, each one at or below rp_min
 * leaves (the list keeps its order) and the aggregate is updated after each
 * removal. *empty is set when no sphere is left. */
static int oxidize_aggregate(mo_box *b, int64_t a, double dt, double rp_min, int64_t **refs, int nrefs, int *empty) {
    grow_aggregate(b, a, dt);
    ivec *m = &b->members[a];
    for (int64_t k = 0; k < m->n;) {
        const int64_t id = m->v[k];
        if (!(SPH(b, S_R, id) <= rp_min)) {
            ++k;
            continue;
        }
        memmove(m->v + k, m->v + k + 1, (size_t)(m->n - k - 1) * sizeof(int64_t));
        m->n--;
        remove_sphere_storage(b, id, refs, nrefs);
        b->agg_n[a] = m->n;
        if (m->n > 0) {
            int rc = rebase_update_place(b, a);
            if (rc) return rc;
        }
    }
    *empty = m->n == 0;
    return 0;
}

/* Aggregate::split (aggregat.cpp:545-628): the connected parts of the
 * aggregate's contact network, found as the reference walks it (the first
 * unvisited sphere starts a part; the last discovered sphere is explored
 * next against the unvisited ones in order), each appended as a copy of the
 * aggregate's record with its own spheres in discovery order, updated;
 * then AggregatList::remove of the aggregate. *did is set when it split. */
static int split_aggregate(mo_box *b, int64_t a, int *did) {
    *did = 0;
    const ivec *m = &b->members[a];
    const int64_t n = m->n;
    if (n < 2) return 0;
    int64_t *unvisited = (int64_t *)malloc((size_t)n * sizeof(int64_t));
    int64_t *order = (int64_t *)malloc((size_t)n * sizeof(int64_t));  /* parts back to back */
    int64_t *part_end = (int64_t *)malloc((size_t)(n + 1) * sizeof(int64_t));
    int64_t *stack = (int64_t *)malloc((size_t)n * sizeof(int64_t));
    int64_t nu = n, no = 0, np = 0;
    for (int64_t i = 0; i < n; ++i) unvisited[i] = i;
    while (nu > 0) {
        int64_t first = unvisited[0];
        memmove(unvisited, unvisited + 1, (size_t)(nu - 1) * sizeof(int64_t));
        nu--;
        order[no++] = first;
        int64_t ns_ = 0;
        stack[ns_++] = first;
        while (ns_ > 0) {
            const int64_t s1 = m->v[stack[--ns_]];
            const double p1[3] = {SPH(b, S_X, s1), SPH(b, S_Y, s1), SPH(b, S_Z, s1)};
            for (int64_t idx = 0; idx < nu;) {
                const int64_t s2 = m->v[unvisited[idx]];
                const double p2[3] = {SPH(b, S_X, s2), SPH(b, S_Y, s2), SPH(b, S_Z, s2)};
                if (contact(p1, SPH(b, S_R, s1), p2, SPH(b, S_R, s2), b->L)) {
                    order[no++] = unvisited[idx];
                    stack[ns_++] = unvisited[idx];
                    memmove(unvisited + idx, unvisited + idx + 1, (size_t)(nu - idx - 1) * sizeof(int64_t));
                    nu--;
                } else {
                    ++idx;
                }
            }
        }
        part_end[np++] = no;
    }
    int rc = 0;
    if (np > 1) {
        *did = 1;
        for (int64_t c = 0; c < np && !rc; ++c) {
            const int64_t beg = c == 0 ? 0 : part_end[c - 1];
            const int64_t L = b->na;
            for (int f = 0; f < 21; ++f) AGG(b, f, L) = AGG(b, f, a);
            b->agg_uid[L] = b->next_uid++;
            memset(&b->members[L], 0, sizeof(ivec));
            for (int64_t k = beg; k < part_end[c]; ++k) {
                const int64_t s = b->members[a].v[order[k]];
                iv_push(&b->members[L], s);
                b->sph_label[s] = L;
            }
            b->agg_n[L] = b->members[L].n;
            b->na++;
            verlet_index(b, L, b->vidx[L]);
            set_insert(cell(b, b->vidx[L]), L);
            rc = rebase_update_place(b, L);
        }
        if (!rc) remove_aggregate(b, a);
    }
    free(unvisited);
    free(order);
    free(part_end);
    free(stack);
    return rc;
}

/* calcul (src/calcul.cpp:66-281): collisions, with surface growth or
 * oxidation when the parameters ask for it */
int mo_calcul(mo_box *b, int64_t max_steps, mo_step_record *trace, int64_t cap, mo_stats *stats) {
    int64_t steps = 0, events = 0;
    const int surface = b->p.with_surface_reactions != 0;
    const int individual = surface && b->p.individual_surf_reactions != 0;
    const int oxidation = surface && b->p.u_sg < 0.0;
    while (!finished(b)) {
        if (max_steps > 0 && steps >= max_steps) break;
        double max = b->max_time_step;
        if (b->event || surface) mo_sort_time_steps(b, max);
        int64_t label = mo_pick_random(b);
        double deltatemps = mo_get_time_step(b, max);
        const double deltatemps_pick = deltatemps;
        double deltatemps_indiv = AGG(b, A_TIME_STEP, label);
        double full = AGG(b, A_LPM, label);
        double dir[3];
        random_direction(dir);
        double move = full;
        int n_try = 1, contact_flag = 0;
        mo_contact c = {INFINITY, -1, -1, -1, -1};
        if (b->p.with_collisions) {
            int rc = mo_distance_to_next_contact(b, label, dir, full, &c);
            if (rc) return rc;
            contact_flag = c.distance <= full;
            if (contact_flag) move = c.distance;
        }
        double v[3] = {dir[0] * move, dir[1] * move, dir[2] * move};
        mo_translate(b, label, v);
        deltatemps = deltatemps * (move / full + (double)(n_try - 1));
        deltatemps_indiv = deltatemps_indiv * (move / full + (double)(n_try - 1));
        AGG(b, A_TIME, label) += deltatemps;
        b->time = b->time + deltatemps;
        /* surface reactions before the merge (calcul.cpp:157-170) */
        int split = 0, disappear = 0;
        const int64_t moving_uid = b->agg_uid[label];
        const int64_t other_uid = contact_flag && c.other_aggregate >= 0 ? b->agg_uid[c.other_aggregate] : -1;
        if (oxidation) {
            int64_t *refs[2] = {&c.moving_sphere, &c.other_sphere};
            const double rp_min = b->p.rp_min_oxid;
            if (individual) {
                int empty = 0;
                int rc = oxidize_aggregate(b, label, deltatemps_indiv, rp_min, refs, 2, &empty);
                if (rc) return rc;
                if (empty) {
                    remove_aggregate(b, label);
                    disappear = 1;
                } else {
                    rc = split_aggregate(b, label, &split);
                    if (rc) return rc;
                }
            } else {
                for (int64_t a = 0; a < b->na;) {
                    int empty = 0;
                    int rc = oxidize_aggregate(b, a, deltatemps, rp_min, refs, 2, &empty);
                    if (rc) return rc;
                    if (empty) {
                        remove_aggregate(b, a);
                        disappear = 1;
                    } else {
                        ++a;
                    }
                }
                for (int64_t a = 0; a < b->na;) {
                    int did = 0;
                    int rc = split_aggregate(b, a, &did);
                    if (rc) return rc;
                    if (did) split = 1;
                    else ++a;
                }
            }
        } else if (individual) {
            grow_aggregate(b, label, deltatemps_indiv);
        } else if (surface) {
            for (int64_t a = 0; a < b->na; ++a) grow_aggregate(b, a, deltatemps);
        }
        int32_t merged = 0;
        if (contact_flag && (!individual || !(split || disappear))) {
            if (oxidation) {
                /* the aggregates of the contact where they are now (-1 when
                 * split or gone: the reference's expired weak pointers) */
                c.moving_aggregate = c.other_aggregate = -1;
                for (int64_t a = 0; a < b->na; ++a) {
                    if (b->agg_uid[a] == moving_uid) c.moving_aggregate = a;
                    if (b->agg_uid[a] == other_uid) c.other_aggregate = a;
                }
            }
            int rc = mo_merge(b, &c, &merged);
            if (rc) return rc;
        }
        if (surface) {
            /* update() every full_aggregate_update_frequency-th step without
             * event, else update_partial(); the moved aggregate alone in the
             * individual mode unless there was a merge (calcul.cpp:180-206) */
            const int64_t every = b->p.full_aggregate_update_frequency > 0 ? b->p.full_aggregate_update_frequency : 1;
            const int partial = b->n_iter_without_event % every != 0;
            if (individual && !merged && !split && !disappear) {
                int rc = update_aggregate_part(b, label, partial);
                if (rc) return rc;
            } else {
                for (int64_t a = 0; a < b->na; ++a) {
                    int rc = update_aggregate_part(b, a, partial);
                    if (rc) return rc;
                }
            }
        }
        b->event = merged || split || disappear;
        if (b->event) {
            b->n_iter_without_event = 0;
            ++events;
            mo_refresh(b);
        } else {
            b->n_iter_without_event++;
        }
        if (trace && steps < cap) {
            mo_step_record *r = &trace[steps];
            r->step = steps;
            r->picked = label;
            r->contact = contact_flag;
            r->merged = merged;
            r->moving_sphere = c.moving_sphere;
            r->other_sphere = c.other_sphere;
            r->moving_agg = c.moving_aggregate;
            r->other_agg = c.other_aggregate;
            r->n_agg_after = b->na;
            r->deltatemps = deltatemps_pick;
            r->full_distance = full;
            r->dir[0] = dir[0];
            r->dir[1] = dir[1];
            r->dir[2] = dir[2];
            r->contact_distance = c.distance;
            r->move_distance = move;
            r->time_after = b->time;
            r->reserved = 0;
        }
        ++steps;
    }
    if (stats) {
        stats->steps = steps;
        stats->events = events;
        stats->n_aggregates = b->na;
        stats->time = b->time;
        stats->finished = finished(b);
        stats->reserved = 0;
    }
    return 0;
}
