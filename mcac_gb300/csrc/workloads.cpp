// Seeded synthetic box states for the contact-search benchmark: aggregates
// grown by ballistic sticking, placed without overlap in a periodic cube
// sized for the requested volume fraction. The reference has no such
// generator; the aggregate fields are those of its update()
// (host_update_aggregate).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <thread>
#include <vector>

#include "common.hpp"
#include "host_box.hpp"
#include "physics.hpp"
#include "rng.hpp"

namespace mcacg {

namespace {

struct Sph {
    double x, y, z, r;
};

double lognormal_diameter(RandStream &rs, double mean, double sigma_geo) {
    // the reference's LogNormal draw (physical_model.cpp:564-568) on rs
    double u = rs.uniform();
    double d = mean * std::pow(sigma_geo, std::sqrt(2.) * inverf(2. * u - 1.0));
    if (!(d > 0)) d = mean;
    return d * 1e-9;
}

void unit_vector(RandStream &rs, double out[3]) {
    double theta = rs.uniform() * 2 * pi_value();
    double phi = std::acos(1 - 2 * rs.uniform());
    out[0] = std::sin(phi) * std::cos(theta);
    out[1] = std::sin(phi) * std::sin(theta);
    out[2] = std::cos(phi);
}

// One aggregate of n spheres by ballistic sticking: each new sphere comes
// from far away along a random direction u on the line through a random
// member m and stops at its first contact with the aggregate. On that line a
// member o is reached at s_o = (o - m).u - sqrt((r + r_o)^2 - perp_o^2), perp_o
// being the distance from o to the line; the sphere is placed at m + u min s_o,
// tangent to the first member hit and clear of every other one.
std::vector<Sph> grow(RandStream &rs, int n, double mean_d, double sigma_geo) {
    std::vector<Sph> s;
    s.reserve(size_t(n));
    s.push_back(Sph{0, 0, 0, 0.5 * lognormal_diameter(rs, mean_d, sigma_geo)});
    while (int(s.size()) < n) {
        const double r = 0.5 * lognormal_diameter(rs, mean_d, sigma_geo);
        const Sph &m = s[size_t(rs.next_int()) % s.size()];
        double u[3];
        unit_vector(rs, u);
        double best = HUGE_VAL;
        for (const Sph &o : s) {
            double dx = o.x - m.x, dy = o.y - m.y, dz = o.z - m.z;
            double proj = dx * u[0] + dy * u[1] + dz * u[2];
            double perp2 = dx * dx + dy * dy + dz * dz - proj * proj;
            double rs2 = (r + o.r) * (r + o.r);
            if (perp2 < rs2) best = std::min(best, proj - std::sqrt(rs2 - perp2));
        }
        // the line passes through m, so best is finite
        s.push_back(Sph{m.x + best * u[0], m.y + best * u[1], m.z + best * u[2], r});
    }
    return s;
}

}  // namespace

int make_synthetic_state(const mcacg_params &p, int n_aggregates, int max_size, HostState *st, std::string *err) {
    const int64_t n_total = p.n_monomeres;
    if (n_aggregates < 1 || n_total < n_aggregates || max_size < 1 || int64_t(max_size) * n_aggregates < n_total) {
        if (err) *err = "inconsistent synthetic box sizes";
        return ST_BAD_ARGUMENT;
    }
    RandStream master;
    master.seed(uint32_t(p.random_seed < 0 ? 0 : p.random_seed));
    // sizes: log-normal with a log-sd of 1.2 and the requested mean, clipped
    // to [1, max_size], then nudged one sphere at a time to the exact total
    const double mean = double(n_total) / n_aggregates;
    const double sigma = 1.2, mu = std::log(mean) - 0.5 * sigma * sigma;
    std::vector<int> size(static_cast<size_t>(n_aggregates));
    int64_t sum = 0;
    for (int a = 0; a < n_aggregates; ++a) {
        double z = std::sqrt(2.) * inverf(2. * master.uniform() - 1.);
        double v = std::exp(mu + sigma * z);
        size[size_t(a)] = (v >= max_size) ? max_size : std::max(1, int(std::lround(v)));
        sum += size[size_t(a)];
    }
    for (int64_t guard = 0; sum != n_total && guard < 1000000000; ++guard) {
        int a = int(uint32_t(master.next_int()) % uint32_t(n_aggregates));
        if (sum < n_total && size[size_t(a)] < max_size) {
            ++size[size_t(a)];
            ++sum;
        } else if (sum > n_total && size[size_t(a)] > 1) {
            --size[size_t(a)];
            --sum;
        }
    }
    // grow every aggregate (parallel; one private stream per aggregate)
    std::vector<std::vector<Sph>> aggs(static_cast<size_t>(n_aggregates));
    std::atomic<int> next{0};
    unsigned nt = std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nt; ++t)
        pool.emplace_back([&] {
            for (int a = next++; a < n_aggregates; a = next++) {
                RandStream rs;
                rs.seed(uint32_t(p.random_seed) * 2654435761u + uint32_t(a) + 1u);
                aggs[size_t(a)] = grow(rs, size[size_t(a)], p.mean_diameter, p.dispersion_diameter);
            }
        });
    for (auto &th : pool) th.join();
    int64_t ns = 0;
    double vol = 0.0;
    for (const auto &g : aggs) {
        ns += int64_t(g.size());
        for (const Sph &s : g) vol += 4.0 / 3.0 * pi_value() * s.r * s.r * s.r;
    }
    const double L = std::cbrt(vol / p.volume_fraction);
    // place aggregates at random offsets, rejecting overlaps (spatial hash)
    double rmax_sphere = 0;
    for (const auto &g : aggs)
        for (const Sph &s : g) rmax_sphere = std::max(rmax_sphere, s.r);
    const double cell = std::max(2.0 * rmax_sphere, L / 512.0);
    const int G = std::max(1, int(L / cell));
    const double h = L / G;
    std::vector<int> head(size_t(G) * G * G, -1), nxt(size_t(ns), -1);
    std::vector<Sph> placed(static_cast<size_t>(ns));
    int64_t used = 0;
    auto cell_id = [&](double x) {
        int c = int(std::floor(x / h));
        return periodic_cell(c, G);
    };
    st->ns = int(ns);
    st->nslots = n_aggregates;
    st->n_div = int(p.n_verlet_divisions);
    st->box_length = L;
    st->time = p.initial_time;
    st->maxradius = 0;
    st->sph.assign(9 * size_t(ns), 0.0);
    st->sph_slot.assign(size_t(ns), 0);
    st->agg.assign(21 * size_t(n_aggregates), 0.0);
    st->agg_n.assign(size_t(n_aggregates), 0);
    st->members.clear();
    st->members.reserve(size_t(n_aggregates), size_t(ns));
    for (int a = 0; a < n_aggregates; ++a) {
        const auto &g = aggs[size_t(a)];
        bool ok = false;
        double off[3] = {0, 0, 0};
        for (int attempt = 0; attempt < 100000 && !ok; ++attempt) {
            off[0] = master.uniform() * L;
            off[1] = master.uniform() * L;
            off[2] = master.uniform() * L;
            ok = true;
            for (const Sph &s : g) {
                double c[3] = {s.x + off[0], s.y + off[1], s.z + off[2]};
                for (int dx = -1; dx <= 1 && ok; ++dx)
                    for (int dy = -1; dy <= 1 && ok; ++dy)
                        for (int dz = -1; dz <= 1 && ok; ++dz) {
                            int ci = periodic_cell(cell_id(c[0]) + dx, G), cj = periodic_cell(cell_id(c[1]) + dy, G),
                                ck = periodic_cell(cell_id(c[2]) + dz, G);
                            for (int o = head[(size_t(ci) * G + cj) * G + ck]; o >= 0; o = nxt[size_t(o)]) {
                                const Sph &q = placed[size_t(o)];
                                double ex = periodic_distance(c[0] - q.x, L), ey = periodic_distance(c[1] - q.y, L),
                                       ez = periodic_distance(c[2] - q.z, L);
                                double lim = (s.r + q.r) * (1.0 + 1e-9);
                                if (ex * ex + ey * ey + ez * ez < lim * lim) {
                                    ok = false;
                                    break;
                                }
                            }
                        }
                if (!ok) break;
            }
        }
        if (!ok) {
            if (err) *err = "synthetic box too dense to place every aggregate";
            return ST_TOO_DENSE;
        }
        const double pi = pi_value();
        for (size_t k = 0; k < g.size(); ++k) {
            const int s_id = int(used);
            Sph q{g[k].x + off[0], g[k].y + off[1], g[k].z + off[2], g[k].r};
            placed[size_t(used)] = q;
            int ci = cell_id(q.x), cj = cell_id(q.y), ck = cell_id(q.z);
            size_t c = (size_t(ci) * G + cj) * G + ck;
            nxt[size_t(used)] = head[c];
            head[c] = int(used);
            ++used;
            auto S = [&](int f) -> double & { return st->sph[size_t(f) * size_t(ns) + size_t(s_id)]; };
            S(SPH_X) = q.x;
            S(SPH_Y) = q.y;
            S(SPH_Z) = q.z;
            S(SPH_R) = q.r;
            S(SPH_VOLUME) = 4 * pi / 3 * std::pow(q.r, 3);
            S(SPH_SURFACE) = 4 * pi * std::pow(q.r, 2);
            S(SPH_RX) = g[k].x - g[0].x;
            S(SPH_RY) = g[k].y - g[0].y;
            S(SPH_RZ) = g[k].z - g[0].z;
            st->sph_slot[size_t(s_id)] = a;
        }
        // this aggregate's spheres are the last g.size() ids placed, in order
        for (int k = 0; k < int(g.size()); ++k) st->members.ids.push_back(int(used) - int(g.size()) + k);
        st->members.off.push_back(int(st->members.ids.size()));
        st->agg_n[size_t(a)] = int(g.size());
        double f[21] = {0};
        f[AGG_TIME] = p.initial_time;
        int rc = host_update_aggregate(p, *st, st->members[size_t(a)], f, &st->maxradius);
        if (rc != ST_OK) {
            if (err) *err = "volume/surface error in a synthetic aggregate";
            return rc;
        }
        for (int k = 0; k < 21; ++k) st->agg[size_t(k) * n_aggregates + a] = f[k];
    }
    return ST_OK;
}

}  // namespace mcacg
