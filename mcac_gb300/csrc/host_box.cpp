// Host side of one box; see host_box.hpp. Compiled with -ffp-contract=off.
#include "host_box.hpp"

#include <algorithm>
#include <array>
#include <fstream>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>

#include "common.hpp"
#include "physics.hpp"
#include "rng.hpp"
#include "batch.hpp"

namespace mcacg {

namespace {

inline double &SF(HostState &st, int field, int s) { return st.sph[size_t(field) * size_t(st.ns) + size_t(s)]; }
inline double SF(const HostState &st, int field, int s) { return st.sph[size_t(field) * size_t(st.ns) + size_t(s)]; }
inline double &AF(HostState &st, int field, int a) { return st.agg[size_t(field) * size_t(st.nslots) + size_t(a)]; }

// Spatial hash used by the free-space test of the initial placement.
struct PlacementGrid {
    double h = 1, L = 1;
    int G = 1;
    std::vector<int> head, next;
    void init(double box, double cell, int n) {
        L = box;
        G = std::max(1, std::min(512, int(box / cell)));
        h = box / G;
        head.assign(size_t(G) * G * G, -1);
        next.assign(size_t(n), -1);
    }
    int coord(double x) const { return std::min(std::max(int(std::floor(x / h)), 0), G - 1); }
    void insert(int id, const double p[3]) {
        size_t c = (size_t(coord(p[0])) * G + coord(p[1])) * G + coord(p[2]);
        next[size_t(id)] = head[c];
        head[c] = id;
    }
    template <class F>
    bool any(const double p[3], double reach, F &&f) const {
        int lo[3], cnt[3];
        for (int l = 0; l < 3; ++l) {
            lo[l] = int(std::floor((p[l] - reach) / h));
            int hi = int(std::floor((p[l] + reach) / h));
            cnt[l] = hi - lo[l] + 1;
            if (cnt[l] >= G) {
                lo[l] = 0;
                cnt[l] = G;
            }
        }
        for (int a = 0; a < cnt[0]; ++a)
            for (int b = 0; b < cnt[1]; ++b)
                for (int c = 0; c < cnt[2]; ++c) {
                    int i = periodic_cell(lo[0] + a, G), j = periodic_cell(lo[1] + b, G), k = periodic_cell(lo[2] + c, G);
                    for (int id = head[(size_t(i) * G + j) * G + k]; id >= 0; id = next[size_t(id)])
                        if (f(id)) return true;
                }
        return false;
    }
};

}  // namespace

namespace {
// update_distances_and_overlapping (aggregat.cpp:719-764)
void overlap_fields(const HostState &st, MemberLists::View members, double *overlapping_out, double *coordination_out) {
    const int n = members.size();
    double overlapping = 0.0, coordination = 0.0;
    int intersections = 0;
    for (int i = 0; i < n; i++) {
        int si = members[size_t(i)];
        for (int j = i + 1; j < n; j++) {
            int sj = members[size_t(j)];
            double dx = SF(st, SPH_RX, si) - SF(st, SPH_RX, sj);
            double dy = SF(st, SPH_RY, si) - SF(st, SPH_RY, sj);
            double dz = SF(st, SPH_RZ, si) - SF(st, SPH_RZ, sj);
            double dist = std::sqrt(dx * dx + dy * dy + dz * dz);
            double rsum = SF(st, SPH_R, si) + SF(st, SPH_R, sj);
            if (dist <= (1. + kCoordinationEpsilon) * rsum) {
                double c = (rsum - dist) / rsum;
                overlapping += 2.0 * c;
                intersections += 2;
            }
        }
    }
    if (intersections > 0) {
        overlapping /= static_cast<double>(intersections);
        coordination = static_cast<double>(intersections) / static_cast<double>(n);
    }
    *overlapping_out = overlapping;
    *coordination_out = coordination;
}
}  // namespace

void host_refresh_overlap(HostState *st) {
    for (int a = 0; a < st->nslots; ++a) {
        if (st->agg_n[size_t(a)] == 0) continue;
        double ov = 0.0, co = 0.0;
        overlap_fields(*st, st->members[size_t(a)], &ov, &co);
        AF(*st, AGG_OVERLAPPING, a) = ov;
        AF(*st, AGG_COORDINATION_NUMBER, a) = co;
    }
}

int host_update_aggregate(const mcacg_params &p, const HostState &st, MemberLists::View members, double fields[21],
                          double *maxradius) {
    const int n = members.size();
    // update_distances_and_overlapping (aggregat.cpp:719-764): the contact
    // pairs i < j in (i, j) order, and each sphere's contacts in key order
    struct Contact {
        int j;
        double d;
    };
    std::vector<std::vector<Contact>> adj(static_cast<size_t>(n));
    double overlapping = 0.0, coordination = 0.0;
    int intersections = 0;
    for (int i = 0; i < n; i++) {
        const int si = members[size_t(i)];
        for (int j = i + 1; j < n; j++) {
            const int sj = members[size_t(j)];
            const double dx = SF(st, SPH_RX, si) - SF(st, SPH_RX, sj);
            const double dy = SF(st, SPH_RY, si) - SF(st, SPH_RY, sj);
            const double dz = SF(st, SPH_RZ, si) - SF(st, SPH_RZ, sj);
            const double dist = std::sqrt(dx * dx + dy * dy + dz * dz);
            const double rsum = SF(st, SPH_R, si) + SF(st, SPH_R, sj);
            if (dist <= (1. + kCoordinationEpsilon) * rsum) {
                adj[size_t(i)].push_back(Contact{j, dist});
                adj[size_t(j)].push_back(Contact{i, dist});
                const double c = (rsum - dist) / rsum;
                overlapping += 2.0 * c;
                intersections += 2;
            }
        }
    }
    if (intersections > 0) {
        overlapping /= static_cast<double>(intersections);
        coordination = static_cast<double>(intersections) / static_cast<double>(n);
    }
    // the exact SBL and ARVO back-ends are optional libraries of the
    // reference, which stops with their error codes when they are absent
    // (aggregat.cpp:329-346)
    if (p.volsurf_method == VS_SBL) return ST_SBL;
    if (p.volsurf_method == VS_ARVO) return ST_ARVO;
    if (p.volsurf_method != VS_NONE && p.volsurf_method != VS_CAPS && p.volsurf_method != VS_ALPHAS)
        return ST_INPUT;
    // compute_volume_surface (aggregat.cpp:321-430): per-sphere volumes and
    // surfaces, cut by the spherical caps of each contact for "caps" (the
    // contacts of a sphere with later ones in key order), then summed; the
    // "alphas" corrections act on the sums
    std::vector<double> vols(static_cast<size_t>(n)), surfs(static_cast<size_t>(n));
    for (int i = 0; i < n; i++) {
        vols[size_t(i)] = SF(st, SPH_VOLUME, members[size_t(i)]);
        surfs[size_t(i)] = SF(st, SPH_SURFACE, members[size_t(i)]);
    }
    if (p.volsurf_method == VS_CAPS) {
        for (int i = 0; i < n; i++) {
            const int si = members[size_t(i)];
            for (const Contact &c : adj[size_t(i)]) {
                if (c.j <= i) continue;
                const int sj = members[size_t(c.j)];
                const SphereCaps k = sphere_caps(SF(st, SPH_R, si), SF(st, SPH_VOLUME, si), SF(st, SPH_SURFACE, si),
                                                 SF(st, SPH_R, sj), SF(st, SPH_VOLUME, sj), SF(st, SPH_SURFACE, sj), c.d);
                vols[size_t(i)] = vols[size_t(i)] - k.v1;
                surfs[size_t(i)] = surfs[size_t(i)] - k.s1;
                vols[size_t(c.j)] = vols[size_t(c.j)] - k.v2;
                surfs[size_t(c.j)] = surfs[size_t(c.j)] - k.s2;
            }
            vols[size_t(i)] = std::max(vols[size_t(i)], 0.0);
            surfs[size_t(i)] = std::max(surfs[size_t(i)], 0.0);
        }
    }
    double volume = 0.0, surface = 0.0;
    for (int i = 0; i < n; i++) {
        volume = volume + vols[size_t(i)];
        surface = surface + surfs[size_t(i)];
    }
    if (p.volsurf_method == VS_ALPHAS) {
        AlphaSums a{0., 0., 0., 0., 0., 0.};
        int entries = 0;
        for (int i = 0; i < n; i++) {
            const double r1 = SF(st, SPH_R, members[size_t(i)]);
            for (const Contact &c : adj[size_t(i)]) alpha_add(a, r1, SF(st, SPH_R, members[size_t(c.j)]), c.d);
            entries += int(adj[size_t(i)].size());
        }
        alpha_finish(a, n, entries, &volume, &surface, &overlapping, &coordination);
    }
    if (volume <= 0 || surface <= 0) return ST_VOL_SURF;
    // compute_mass_center (aggregat.cpp:431-452), with the per-sphere volumes
    // of compute_volume_surface
    double r[3] = {0., 0., 0.};
    for (int i = 0; i < n; i++) {
        int s = members[size_t(i)];
        double vol = vols[size_t(i)];
        r[0] += SF(st, SPH_RX, s) * vol;
        r[1] += SF(st, SPH_RY, s) * vol;
        r[2] += SF(st, SPH_RZ, s) * vol;
    }
    r[0] /= volume;
    r[1] /= volume;
    r[2] /= volume;
    std::vector<double> dcen(static_cast<size_t>(n), 0.0);
    for (int i = 0; i < n; i++) {
        int s = members[size_t(i)];
        double dx = SF(st, SPH_RX, s) - r[0], dy = SF(st, SPH_RY, s) - r[1], dz = SF(st, SPH_RZ, s) - r[2];
        dcen[size_t(i)] = std::sqrt(dx * dx + dy * dy + dz * dz);
    }
    int s0 = members[0];
    fields[AGG_X] = periodic_position(SF(st, SPH_X, s0) + r[0], st.box_length);
    fields[AGG_Y] = periodic_position(SF(st, SPH_Y, s0) + r[1], st.box_length);
    fields[AGG_Z] = periodic_position(SF(st, SPH_Z, s0) + r[2], st.box_length);
    fields[AGG_RX] = r[0];
    fields[AGG_RY] = r[1];
    fields[AGG_RZ] = r[2];
    // compute_max_radius, compute_giration_radius (aggregat.cpp:453-483)
    double rmax = 0.0, arg = 0., brg = 0.;
    for (int i = 0; i < n; i++) {
        int s = members[size_t(i)];
        rmax = dmax(rmax, SF(st, SPH_R, s) + dcen[size_t(i)]);
    }
    for (int i = 0; i < n; i++) {
        int s = members[size_t(i)];
        double vol = vols[size_t(i)];
        double rs = SF(st, SPH_R, s);
        arg = arg + vol * (dcen[size_t(i)] * dcen[size_t(i)]);
        brg = brg + vol * (rs * rs);
    }
    double rg = std::sqrt(std::abs((arg + (3. / 5.) * brg) / volume));
    // update_partial (aggregat.cpp:253-281)
    double dp = 0., vol_pp = 0.;
    for (int i = 0; i < n; i++) {
        vol_pp += SF(st, SPH_VOLUME, members[size_t(i)]);
        dp += SF(st, SPH_R, members[size_t(i)]);
    }
    dp = 2 * dp / static_cast<double>(n);
    vol_pp = vol_pp / static_cast<double>(n);
    AggregatePhysics ph = aggregate_physics(p, volume, vol_pp, dp, rg);
    fields[AGG_RG] = rg;
    fields[AGG_F_AGG] = ph.f_agg;
    fields[AGG_LPM] = ph.lpm;
    fields[AGG_TIME_STEP] = ph.time_step;
    fields[AGG_RMAX] = rmax;
    fields[AGG_VOLUME] = volume;
    fields[AGG_SURFACE] = surface;
    fields[AGG_DP] = dp;
    fields[AGG_DG_OVER_DP] = ph.dg_over_dp;
    fields[AGG_OVERLAPPING] = overlapping;
    fields[AGG_COORDINATION_NUMBER] = coordination;
    fields[AGG_D_M] = ph.d_m;
    if (rmax > *maxradius) *maxradius = rmax;
    return ST_OK;
}

int init_random_state(const mcacg_params &p, HostState *st, std::string *err) {
    const int N = int(p.n_monomeres);
    if (N < 1) {
        if (err) *err = "number of monomers must be positive";
        return ST_INPUT;
    }
    const double L = p.box_length;
    const double pi = pi_value();
    const double volume_factor = 4 * pi / 3;
    const double surface_factor = 4 * pi;
    init_random(p.random_seed);
    st->n_div = int(p.n_verlet_divisions);
    st->box_length = L;
    st->maxradius = 0.;
    st->time = p.initial_time;
    st->ns = st->nslots = N;
    st->sph.assign(9 * size_t(N), 0.);
    st->sph_slot.assign(size_t(N), -1);
    st->agg.assign(21 * size_t(N), 0.);
    st->agg_n.assign(size_t(N), 0);
    st->members.clear();
    st->members.reserve(size_t(N), size_t(N));
    PlacementGrid grid;
    grid.init(L, 4.0 * p.mean_diameter * 1e-9, N);
    for (int i = 0; i < N; ++i) {
        AF(*st, AGG_TIME, i) = st->time;
        double diameter = 0;
        int rc = random_diameter(p, p.mean_diameter, p.dispersion_diameter, &diameter);
        if (rc != ST_OK) {
            if (err) *err = "dispersion_diameter cannot be lower than 1";
            return rc;
        }
        const double radius = diameter * 0.5;
        bool placed = false;
        for (int n_try = 0; n_try < N; n_try++) {
            double pos[3];
            pos[0] = random_uniform() * L;
            pos[1] = random_uniform() * L;
            pos[2] = random_uniform() * L;
            // AggregatList::test_free_space (aggregat_list.cpp:534-548)
            const double reach = radius + st->maxradius + 1e-3 * grid.h;
            bool busy = grid.any(pos, reach, [&](int j) {
                Vec3 q{pos[0], pos[1], pos[2]};
                Vec3 ca{AF(*st, AGG_X, j), AF(*st, AGG_Y, j), AF(*st, AGG_Z, j)};
                if (!spheres_in_contact(q, radius, ca, AF(*st, AGG_RMAX, j), L)) return false;
                Vec3 cs{SF(*st, SPH_X, j), SF(*st, SPH_Y, j), SF(*st, SPH_Z, j)};
                return spheres_in_contact(q, radius, cs, SF(*st, SPH_R, j), L);
            });
            if (busy) continue;
            // Aggregate::init(...) (aggregat.cpp:194-229)
            AF(*st, AGG_X, i) = periodic_position(pos[0], L);
            AF(*st, AGG_Y, i) = periodic_position(pos[1], L);
            AF(*st, AGG_Z, i) = periodic_position(pos[2], L);
            st->sph_slot[size_t(i)] = i;
            SF(*st, SPH_X, i) = pos[0];
            SF(*st, SPH_Y, i) = pos[1];
            SF(*st, SPH_Z, i) = pos[2];
            SF(*st, SPH_R, i) = radius;
            SF(*st, SPH_RX, i) = 0.;
            SF(*st, SPH_RY, i) = 0.;
            SF(*st, SPH_RZ, i) = 0.;
            SF(*st, SPH_VOLUME, i) = volume_factor * std::pow(radius, 3);
            SF(*st, SPH_SURFACE, i) = surface_factor * std::pow(radius, 2);
            st->members.push_single(i);
            st->agg_n[size_t(i)] = 1;
            AF(*st, AGG_D_M, i) = diameter;
            double f[21];
            for (int k = 0; k < 21; ++k) f[k] = AF(*st, k, i);
            rc = host_update_aggregate(p, *st, st->members[size_t(i)], f, &st->maxradius);
            if (rc != ST_OK) {
                if (err) *err = "volume/surface error during placement";
                return rc;
            }
            for (int k = 0; k < 21; ++k) AF(*st, k, i) = f[k];
            double cp[3] = {AF(*st, AGG_X, i), AF(*st, AGG_Y, i), AF(*st, AGG_Z, i)};
            grid.insert(i, cp);
            placed = true;
            break;
        }
        if (!placed) {
            if (err) *err = "Too dense: could not place a monomer";
            return ST_TOO_DENSE;
        }
    }
    if (p.enforce_volume_fraction) {
        // aggregat_list_storage.cpp:75-87
        double current = 0.0;
        for (int a = 0; a < N; ++a) current += AF(*st, AGG_VOLUME, a);
        double prescribed = p.volume_fraction * std::pow(L, 3);
        double correction = std::pow(prescribed / current, 1. / 3.);
        for (int s = 0; s < N; ++s) {
            double r = SF(*st, SPH_R, s) * correction;
            SF(*st, SPH_R, s) = r;
            SF(*st, SPH_VOLUME, s) = volume_factor * std::pow(r, 3);
            SF(*st, SPH_SURFACE, s) = surface_factor * std::pow(r, 2);
        }
        for (int a = 0; a < N; ++a) {
            // compute_volume_surface only (method "none": sums of sphere values)
            double v = 0.0, s = 0.0;
            for (int m : st->members[size_t(a)]) {
                v = v + SF(*st, SPH_VOLUME, m);
                s = s + SF(*st, SPH_SURFACE, m);
            }
            AF(*st, AGG_VOLUME, a) = v;
            AF(*st, AGG_SURFACE, a) = s;
        }
    }
    return ST_OK;
}

int init_random_state_private(const mcacg_params &p, HostState *st, std::string *err) {
    RandStream rs;
    rs.seed(uint32_t(p.random_seed < 0 ? 0 : p.random_seed));
    set_thread_stream(&rs);
    int rc = init_random_state(p, st, err);
    set_thread_stream(nullptr);
    return rc;
}

// ------------------------------------------------------------------ HostBox
int HostBox::upload(const HostState &st, void *stream, std::string *err) {
    ns_ = st.ns;
    nslots_ = st.nslots;
    agg_ = st.agg;
    agg_n_ = st.agg_n;
    alive_.clear();
    for (int a = 0; a < nslots_; ++a)
        if (agg_n_[size_t(a)] > 0) alive_.push_back(a);
    uid_.resize(alive_.size());
    std::iota(uid_.begin(), uid_.end(), int64_t(0));
    next_uid_ = int64_t(alive_.size());
    cpu_last_event_ = cpu_start_ = std::clock();  // physical_model.cpp:286
    maxradius_ = st.maxradius;
    time_ = st.time;
    DeviceBox *d = nullptr;
    int rc = DeviceBox::create(st, stream, &d, err);
    if (rc != ST_OK) return rc;
    dev_.reset(d);
    rc = dev_->set_volsurf(p_.volsurf_method);
    if (rc != ST_OK) {
        if (err) *err = "volsurf_method not available";
        return rc;
    }
    refresh();
    init_model_values();
    return ST_OK;
}

// PhysicalModel's concentrations before the first update
// (physical_model.cpp:266-267) and its input volume fraction.
void HostBox::init_model_values() {
    aggregate_concentration_ = static_cast<double>(p_.n_monomeres) / p_.box_volume;
    monomer_concentration_ = aggregate_concentration_;
    volume_fraction_ = p_.volume_fraction;
}

// PhysicalModel::time_to_write (physical_model.cpp:338-356).
bool HostBox::time_to_write() {
    if (p_.write_delta_t > 0) {
        const uint64_t timestep = static_cast<uint64_t>(std::floor(time_ / p_.write_delta_t));
        if (timestep > last_timestep_written_) {
            last_timestep_written_ = timestep;
            return true;
        }
    }
    const uint64_t every_event = static_cast<uint64_t>(p_.write_events_frequency);
    const uint64_t every_step = static_cast<uint64_t>(p_.write_between_event_frequency);
    if (n_iter_without_event_ == 0 && static_cast<uint64_t>(total_events_) % every_event == 0) return true;
    if (n_iter_without_event_ > 0 && static_cast<uint64_t>(n_iter_without_event_) % every_step == 0) return true;
    return false;
}

// save_advancement (calcul.cpp:29-43): one line appended, default stream
// formatting (6 significant digits), the values of the physical model.
void HostBox::save_advancement(const char *path) const {
    std::ofstream outfile;
    outfile.open(path, std::ios_base::app);
    outfile << time_;
    outfile << " " << aggregate_concentration_;
    outfile << " " << volume_fraction_;
    outfile << " " << avg_npp_;
    outfile << " " << p_.temperature;
    outfile << " " << p_.box_volume;
    outfile << " " << monomer_concentration_;
    outfile << " " << p_.u_sg;
    outfile << " " << 0.0;  // flux_nucleation: nucleation is outside this library's path
    outfile << std::endl;
    outfile.close();
}

int HostBox::create_random(const mcacg_params &p, void *stream, std::unique_ptr<HostBox> *out, std::string *err) {
    if (p.with_nucleation || p.with_potentials || p.with_flame_coupling || p.with_electric_charges) {
        if (err) *err = "nucleation, potentials, flame coupling and charges are outside this library's path";
        return ST_INPUT;
    }
    std::unique_ptr<HostBox> hb(new HostBox());
    hb->p_ = p;
    HostState st;
    int rc = init_random_state(p, &st, err);
    if (rc != ST_OK) return rc;
    rc = hb->upload(st, stream, err);
    if (rc != ST_OK) return rc;
    *out = std::move(hb);
    return ST_OK;
}

int HostBox::create_from_state(const mcacg_params &p, const mcacg_state &in, void *stream,
                               std::unique_ptr<HostBox> *out, std::string *err) {
    if (in.n_spheres <= 0 || in.n_aggregates <= 0 || !in.spheres || !in.sphere_label || !in.aggregates ||
        !in.n_spheres_per_aggregate || !in.members) {
        if (err) *err = "incomplete state";
        return ST_BAD_ARGUMENT;
    }
    std::unique_ptr<HostBox> hb(new HostBox());
    hb->p_ = p;
    hb->p_.box_length = in.box_length;
    hb->p_.box_volume = std::pow(in.box_length, 3);
    hb->p_.n_verlet_divisions = in.n_verlet_divisions;
    HostState st;
    int rc = state_to_host(in, &st, err);
    if (rc != ST_OK) return rc;
    rc = hb->upload(st, stream, err);
    if (rc != ST_OK) return rc;
    *out = std::move(hb);
    return ST_OK;
}

int state_to_host(const mcacg_state &in, HostState *out, std::string *err) {
    if (in.n_spheres <= 0 || in.n_aggregates <= 0 || !in.spheres || !in.sphere_label || !in.aggregates ||
        !in.n_spheres_per_aggregate || !in.members) {
        if (err) *err = "incomplete state";
        return ST_BAD_ARGUMENT;
    }
    HostState &st = *out;
    st.n_div = int(in.n_verlet_divisions);
    st.box_length = in.box_length;
    st.maxradius = in.maxradius;
    st.time = in.time;
    st.ns = int(in.n_spheres);
    st.nslots = int(in.n_aggregates);
    st.sph.assign(in.spheres, in.spheres + 9 * size_t(st.ns));
    st.sph_slot.resize(size_t(st.ns));
    for (int s = 0; s < st.ns; ++s) {
        int64_t l = in.sphere_label[s];
        if (l < 0 || l >= st.nslots) {
            if (err) *err = "sphere label out of range";
            return ST_BAD_ARGUMENT;
        }
        st.sph_slot[size_t(s)] = int(l);
    }
    st.agg.assign(in.aggregates, in.aggregates + 21 * size_t(st.nslots));
    st.agg_n.resize(size_t(st.nslots));
    st.members.off.resize(size_t(st.nslots) + 1);
    st.members.off[0] = 0;
    int64_t off = 0;
    for (int a = 0; a < st.nslots; ++a) {
        int64_t n = in.n_spheres_per_aggregate[a];
        if (n <= 0) {
            if (err) *err = "empty aggregate in state";
            return ST_BAD_ARGUMENT;
        }
        st.agg_n[size_t(a)] = int(n);
        off += n;
        if (off > st.ns) {
            if (err) *err = "member lists do not cover every sphere once";
            return ST_BAD_ARGUMENT;
        }
        st.members.off[size_t(a) + 1] = int(off);
    }
    if (off != st.ns) {
        if (err) *err = "member lists do not cover every sphere once";
        return ST_BAD_ARGUMENT;
    }
    st.members.ids.resize(size_t(st.ns));
    for (int a = 0; a < st.nslots; ++a) {
        for (int k = st.members.off[size_t(a)]; k < st.members.off[size_t(a) + 1]; ++k) {
            int64_t s = in.members[k];
            if (s < 0 || s >= st.ns || st.sph_slot[size_t(s)] != a) {
                if (err) *err = "member list inconsistent with sphere labels";
                return ST_BAD_ARGUMENT;
            }
            st.members.ids[size_t(k)] = int(s);
        }
    }
    return ST_OK;
}

int64_t HostBox::label_of(int slot) const {
    auto it = std::lower_bound(alive_.begin(), alive_.end(), slot);
    if (it == alive_.end() || *it != slot) return -1;
    return int64_t(it - alive_.begin());
}

int HostBox::distance_to_next_contact(int64_t label, const double dir[3], double distance, mcacg_contact *out,
                                      std::string *err) {
    if (label < 0 || label >= int64_t(alive_.size())) {
        if (err) *err = "label out of range";
        return ST_BAD_ARGUMENT;
    }
    QueryResult q;
    int rc = dev_->query(alive_[size_t(label)], dir, distance, &q, err);
    if (rc != ST_OK) return rc;
    out->distance = q.distance;
    out->moving_sphere = -1;
    out->other_sphere = -1;
    out->moving_aggregate = -1;
    out->other_aggregate = -1;
    if (q.moving_sphere >= 0) {
        out->moving_sphere = q.moving_sphere;
        out->other_sphere = q.other_sphere;
        out->moving_aggregate = label;
        out->other_aggregate = label_of(q.other_slot);
    }
    return ST_OK;
}

int HostBox::distance_to_next_contacts(int n, const int64_t *labels, const double *dirs, const double *distances,
                                       mcacg_contact *out, double *kernel_ms, std::string *err) {
    if (n < 0) {
        if (err) *err = "negative query count";
        return ST_BAD_ARGUMENT;
    }
    std::vector<int> slots(static_cast<size_t>(n));
    for (int k = 0; k < n; ++k) {
        if (labels[k] < 0 || labels[k] >= int64_t(alive_.size())) {
            if (err) *err = "label out of range in query " + std::to_string(k);
            return ST_BAD_ARGUMENT;
        }
        slots[size_t(k)] = alive_[size_t(labels[k])];
    }
    std::vector<QueryResult> q(static_cast<size_t>(n));
    int rc = dev_->query_batch(n, slots.data(), dirs, distances, q.data(), kernel_ms, err);
    for (int k = 0; k < n; ++k) {
        const QueryResult &r = q[size_t(k)];
        mcacg_contact &c = out[k];
        c.distance = r.distance;
        c.moving_sphere = -1;
        c.other_sphere = -1;
        c.moving_aggregate = -1;
        c.other_aggregate = -1;
        if (rc == ST_OK && r.moving_sphere >= 0) {
            c.moving_sphere = r.moving_sphere;
            c.other_sphere = r.other_sphere;
            c.moving_aggregate = labels[k];
            c.other_aggregate = label_of(r.other_slot);
        }
    }
    return rc;
}

int HostBox::translate(int64_t label, const double v[3], std::string *err) {
    if (label < 0 || label >= int64_t(alive_.size())) {
        if (err) *err = "label out of range";
        return ST_BAD_ARGUMENT;
    }
    invalidate_device_run();
    int slot = alive_[size_t(label)];
    F(AGG_X, slot) = periodic_position(F(AGG_X, slot) + v[0], p_.box_length);
    F(AGG_Y, slot) = periodic_position(F(AGG_Y, slot) + v[1], p_.box_length);
    F(AGG_Z, slot) = periodic_position(F(AGG_Z, slot) + v[2], p_.box_length);
    return dev_->translate(slot, v, err);
}

int HostBox::time_forward(int64_t label, double dt, std::string *err) {
    if (label < 0 || label >= int64_t(alive_.size())) {
        if (err) *err = "label out of range";
        return ST_BAD_ARGUMENT;
    }
    invalidate_device_run();
    F(AGG_TIME, alive_[size_t(label)]) += dt;
    return ST_OK;
}

int HostBox::merge(const mcacg_contact &c, int32_t *merged, std::string *err) {
    *merged = 0;
    // a sphere of the contact that is gone (oxidation): nothing to merge
    // (aggregat_list.cpp:369-374)
    if (c.moving_sphere < 0 || c.other_sphere < 0) return ST_OK;
    if (c.moving_aggregate >= int64_t(alive_.size()) || c.other_aggregate >= int64_t(alive_.size()) ||
        c.moving_sphere >= ns_ || c.other_sphere >= ns_) {
        if (err) *err = "contact refers to an unknown aggregate or sphere";
        return ST_BAD_ARGUMENT;
    }
    invalidate_device_run();
    // an aggregate of the contact that is gone (-1, oxidation split it):
    // the device merge refuses with MergeError if the spheres still touch,
    // as the reference does (aggregat.cpp:488-504)
    const int mslot = c.moving_aggregate >= 0 ? alive_[size_t(c.moving_aggregate)] : -1;
    const int oslot = c.other_aggregate >= 0 ? alive_[size_t(c.other_aggregate)] : -1;
    MergeResult m;
    int rc = dev_->merge(int(c.moving_sphere), int(c.other_sphere), mslot, oslot, &m, err);
    if (rc != ST_OK) return rc;
    if (!m.merged) return ST_OK;
    const int keep = m.keep, removed = m.removed;
    // proper time keeping the global time constant (aggregat_list.cpp:385-387)
    double newtime = F(AGG_TIME, keep) + F(AGG_TIME, removed) - time_;
    dt_order_erase(keep, F(AGG_TIME_STEP, keep));
    dt_order_erase(removed, F(AGG_TIME_STEP, removed));
    AggregatePhysics ph = aggregate_physics(p_, m.fields[AGG_VOLUME], m.vol_pp, m.fields[AGG_DP], m.fields[AGG_RG]);
    const int geometry[] = {AGG_RG, AGG_RMAX, AGG_VOLUME, AGG_SURFACE, AGG_X, AGG_Y, AGG_Z, AGG_RX, AGG_RY, AGG_RZ,
                            AGG_DP, AGG_OVERLAPPING, AGG_COORDINATION_NUMBER};
    for (int f : geometry) F(f, keep) = m.fields[f];
    F(AGG_F_AGG, keep) = ph.f_agg;
    F(AGG_D_M, keep) = ph.d_m;
    F(AGG_TIME_STEP, keep) = ph.time_step;
    dt_order_insert(keep, ph.time_step);
    F(AGG_LPM, keep) = ph.lpm;
    F(AGG_DG_OVER_DP, keep) = ph.dg_over_dp;
    F(AGG_TIME, keep) = newtime;
    agg_n_[size_t(keep)] = m.n;
    agg_n_[size_t(removed)] = 0;
    maxradius_ = m.maxradius;
    auto it = std::lower_bound(alive_.begin(), alive_.end(), removed);
    if (it != alive_.end() && *it == removed) {
        uid_.erase(uid_.begin() + (it - alive_.begin()));
        alive_.erase(it);
    }
    double upd[21];
    for (int f = 0; f < 21; ++f) upd[f] = F(f, keep);
    unsigned mask = (1u << AGG_F_AGG) | (1u << AGG_D_M) | (1u << AGG_TIME_STEP) | (1u << AGG_LPM) |
                    (1u << AGG_DG_OVER_DP) | (1u << AGG_TIME);
    rc = dev_->set_fields(keep, upd, mask, err);
    if (rc != ST_OK) return rc;
    *merged = 1;
    return ST_OK;
}

void HostBox::build_dt_order() {
    by_dt_.clear();
    by_dt_.reserve(alive_.size());
    for (int slot : alive_) by_dt_.emplace_back(F(AGG_TIME_STEP, slot), slot);
    std::sort(by_dt_.begin(), by_dt_.end(), [](const std::pair<double, int> &a, const std::pair<double, int> &b) {
        return a.first > b.first || (a.first == b.first && a.second < b.second);
    });
    dt_order_valid_ = true;
}

void HostBox::dt_order_erase(int slot, double dt) {
    if (!dt_order_valid_) return;
    auto cmp = [](const std::pair<double, int> &a, const std::pair<double, int> &b) {
        return a.first > b.first || (a.first == b.first && a.second < b.second);
    };
    auto it = std::lower_bound(by_dt_.begin(), by_dt_.end(), std::make_pair(dt, slot), cmp);
    if (it != by_dt_.end() && it->second == slot) {
        by_dt_.erase(it);
    } else {
        dt_order_valid_ = false;
    }
}

void HostBox::dt_order_insert(int slot, double dt) {
    if (!dt_order_valid_) return;
    auto cmp = [](const std::pair<double, int> &a, const std::pair<double, int> &b) {
        return a.first > b.first || (a.first == b.first && a.second < b.second);
    };
    auto pr = std::make_pair(dt, slot);
    by_dt_.insert(std::lower_bound(by_dt_.begin(), by_dt_.end(), pr, cmp), pr);
}

void HostBox::sort_time_steps(double factor) {
    // aggregat_list.cpp:109-141: std::sort of label indices by factor/time_step,
    // then the sequential cumulative sum.
    //
    // factor/time_step is non-increasing in time_step (correctly rounded
    // division is monotone), so the aggregates ordered by decreasing time
    // step are in non-decreasing weight order; that order is kept up to date
    // at every merge instead of re-sorting. Every sorted order has the same
    // sequence of weights, hence the same cumulative sums, bit for bit: the
    // orders differ only in which label sits at each position of a run of
    // equal weights. So the cumulative sums come from the kept order, and the
    // reference's own order (std::sort's placement of equal keys) is only
    // needed when a pick lands inside such a run (pick_random); it is then
    // computed from the weights as they were at this call.
    const size_t n = alive_.size();
    if (!dt_order_valid_ || by_dt_.size() != n) build_dt_order();
    if (slot_label_.size() != size_t(nslots_)) slot_label_.assign(size_t(nslots_), -1);
    for (size_t l = 0; l < n; ++l) slot_label_[size_t(alive_[l])] = int(l);
    index_sorted_.resize(n);
    cumulative_.resize(n);
    weights_.resize(n);
    tp_by_label_.resize(n);
    ties_ = false;
    ref_order_valid_ = false;
    double prev = -std::numeric_limits<double>::infinity();
    for (size_t k = 0; k < n; ++k) {
        const int slot = by_dt_[k].second;
        const double tp = factor / F(AGG_TIME_STEP, slot);
        ties_ = ties_ || !(tp > prev);
        prev = tp;
        const int label = slot_label_[size_t(slot)];
        index_sorted_[k] = size_t(label);
        weights_[k] = tp;
        tp_by_label_[size_t(label)] = tp;
        cumulative_[k] = (k == 0) ? tp : cumulative_[k - 1] + tp;
    }
}

void HostBox::reference_sort_order() {
    // aggregat_list.cpp:109-123: indices 0..n-1 sorted by weight with std::sort
    const size_t n = tp_by_label_.size();
    index_ref_.resize(n);
    std::iota(index_ref_.begin(), index_ref_.end(), size_t(0));
    const std::vector<double> &tp = tp_by_label_;
    std::sort(index_ref_.begin(), index_ref_.end(), [&tp](size_t a, size_t b) { return tp[a] < tp[b]; });
    ref_order_valid_ = true;
}

int64_t HostBox::pick_random() {
    // aggregat_list.cpp:59-66
    double val = random_uniform() * cumulative_[alive_.size() - 1];
    size_t k = size_t(std::lower_bound(cumulative_.begin(), cumulative_.end(), val) - cumulative_.begin());
    if (k >= cumulative_.size()) k = cumulative_.size() - 1;  // unreachable for finite weights
    const bool in_run = ties_ && ((k > 0 && weights_[k - 1] == weights_[k]) ||
                                  (k + 1 < weights_.size() && weights_[k + 1] == weights_[k]));
    if (!in_run) return int64_t(index_sorted_[k]);
    if (!ref_order_valid_) reference_sort_order();
    return int64_t(index_ref_[k]);
}

void HostBox::refresh() {
    if (alive_.empty()) return;  // every sphere oxidised
    max_time_step_ = F(AGG_TIME_STEP, alive_[0]);
    for (int slot : alive_) max_time_step_ = std::max(F(AGG_TIME_STEP, slot), max_time_step_);
    avg_npp_ = static_cast<double>(ns_) / static_cast<double>(alive_.size());
}

double HostBox::total_volume() const {
    double v = 0.0;
    for (int slot : alive_) v += F(AGG_VOLUME, slot);
    return v;
}
double HostBox::total_surface() const {
    double v = 0.0;
    for (int slot : alive_) v += F(AGG_SURFACE, slot);
    return v;
}

const double *HostBox::fields(int64_t label, double out[21]) const {
    int slot = alive_[size_t(label)];
    for (int f = 0; f < 21; ++f) out[f] = F(f, slot);
    return out;
}

bool HostBox::finished() const {
    const uint64_t n = alive_.size();
    if (n < 1) return true;
    if (n <= static_cast<uint64_t>(p_.number_of_aggregates_limit)) return true;
    if (p_.n_iter_without_event_limit > 0 && n_iter_without_event_ >= p_.n_iter_without_event_limit) return true;
    // processor time since the box was made, and since the last event
    // (physical_model.cpp:311-326)
    if (p_.cpu_limit > 0 && double(std::clock() - cpu_start_) / CLOCKS_PER_SEC >= p_.cpu_limit) return true;
    if (p_.cpu_event_limit > 0 && double(std::clock() - cpu_last_event_) / CLOCKS_PER_SEC >= p_.cpu_event_limit)
        return true;
    if (p_.physical_time_limit > 0 && time_ >= p_.physical_time_limit) return true;
    if (p_.mean_monomere_per_aggregate_limit > 0 && avg_npp_ >= double(p_.mean_monomere_per_aggregate_limit))
        return true;
    return false;
}

// Aggregate::update, or update_partial, of one aggregate (slot >= 0) or of
// every one after surface growth (calcul.cpp:180-206): the geometry on the
// device, the physics fields here with the C library's functions (as the
// reference computes them), then back to the device with the list's
// maxradius; the pick order is rebuilt at the next sort.
int HostBox::update_aggregates(int slot, bool full, std::string *err) {
    std::vector<double> agg, vol_pp;
    int rc = dev_->update_geometry(slot, full, &agg, &vol_pp, err);
    if (rc != ST_OK) return rc;
    // the geometry the device recomputed (the proper times live here only)
    const int geometry[] = {AGG_RG, AGG_RMAX, AGG_VOLUME, AGG_SURFACE, AGG_X, AGG_Y, AGG_Z, AGG_RX, AGG_RY, AGG_RZ,
                            AGG_DP, AGG_OVERLAPPING, AGG_COORDINATION_NUMBER};
    auto physics = [&](int a) {
        for (int f : geometry) F(f, a) = agg[size_t(f) * size_t(nslots_) + size_t(a)];
        const AggregatePhysics ph = aggregate_physics(p_, F(AGG_VOLUME, a), vol_pp[size_t(a)], F(AGG_DP, a), F(AGG_RG, a));
        F(AGG_F_AGG, a) = ph.f_agg;
        F(AGG_D_M, a) = ph.d_m;
        F(AGG_TIME_STEP, a) = ph.time_step;
        F(AGG_LPM, a) = ph.lpm;
        F(AGG_DG_OVER_DP, a) = ph.dg_over_dp;
        if (F(AGG_RMAX, a) > maxradius_) maxradius_ = F(AGG_RMAX, a);
    };
    if (slot >= 0) {
        physics(slot);
    } else {
        for (int a : alive_) physics(a);
    }
    dt_order_valid_ = false;
    rc = dev_->upload_aggregates(agg_, err);
    if (rc != ST_OK) return rc;
    return dev_->set_maxradius(maxradius_, err);
}

namespace {
// A box in the reference's own order, for oxidation: aggregates by label,
// spheres by storage index, both renumbered as the reference renumbers them.
struct LabelBox {
    HostState st;                           // spheres ([9][ns]); st.ns
    std::vector<std::array<double, 21>> f;  // fields by label
    std::vector<std::vector<int>> mem;      // members by label, list order
    std::vector<int64_t> uid;
};

// spheres.remove(id) (list_storage_methods.hpp:78-87): later spheres move
// down one index; member lists and the contact's sphere references follow
// (a reference to the removed sphere becomes -1, an expired weak pointer).
void remove_storage(LabelBox &w, int id, int64_t *refs[], int nrefs) {
    const int ns = w.st.ns;
    std::vector<double> sph(size_t(9) * size_t(ns - 1));
    for (int f = 0; f < 9; ++f) {
        const double *src = w.st.sph.data() + size_t(f) * size_t(ns);
        double *dst = sph.data() + size_t(f) * size_t(ns - 1);
        std::copy(src, src + id, dst);
        std::copy(src + id + 1, src + ns, dst + id);
    }
    w.st.sph.swap(sph);
    w.st.ns = ns - 1;
    for (auto &m : w.mem)
        for (int &x : m)
            if (x > id) --x;
    for (int r = 0; r < nrefs; ++r) {
        if (*refs[r] == id) *refs[r] = -1;
        else if (*refs[r] > id) --(*refs[r]);
    }
}
}  // namespace

// Relative positions from the first sphere, Aggregate::update, then each
// sphere placed back from the aggregate's position (remove_sphere and split,
// aggregat.cpp:596-609, 641-654); all on the host, as the reference.
static int rebase_update_place(const mcacg_params &p, LabelBox &w, int a, double *maxradius) {
    HostState &st = w.st;
    const std::vector<int> &m = w.mem[size_t(a)];
    auto SFr = [&](int f, int s) -> double & { return st.sph[size_t(f) * size_t(st.ns) + size_t(s)]; };
    const int s0 = m[0];
    const double r0[3] = {SFr(SPH_X, s0), SFr(SPH_Y, s0), SFr(SPH_Z, s0)};
    for (int s : m) {
        SFr(SPH_RX, s) = SFr(SPH_X, s) - r0[0];
        SFr(SPH_RY, s) = SFr(SPH_Y, s) - r0[1];
        SFr(SPH_RZ, s) = SFr(SPH_Z, s) - r0[2];
    }
    int rc = host_update_aggregate(p, st, MemberLists::View{m.data(), int(m.size())}, w.f[size_t(a)].data(), maxradius);
    if (rc != ST_OK) return rc;
    const double *F = w.f[size_t(a)].data();
    const double ref[3] = {F[AGG_X] - F[AGG_RX], F[AGG_Y] - F[AGG_RY], F[AGG_Z] - F[AGG_RZ]};
    for (int s : m) {
        SFr(SPH_X, s) = ref[0] + SFr(SPH_RX, s);
        SFr(SPH_Y, s) = ref[1] + SFr(SPH_RY, s);
        SFr(SPH_Z, s) = ref[2] + SFr(SPH_RZ, s);
    }
    return ST_OK;
}

int64_t HostBox::label_of_uid(int64_t uid) const {
    for (size_t l = 0; l < uid_.size(); ++l)
        if (uid_[l] == uid) return int64_t(l);
    return -1;
}

// The box's state replaced by one in label order (slot = label), for the
// spheres and aggregates oxidation renumbered: a new device box, the host
// mirrors from it. Nothing else changes (the pick factor and mean size stay
// as the last event left them).
int HostBox::replace_state(const HostState &st, std::string *err) {
    invalidate_device_run();
    DeviceBox *d = nullptr;
    void *stream = dev_->owns_stream() ? nullptr : dev_->stream();
    int rc = DeviceBox::create(st, stream, &d, err);
    if (rc != ST_OK) return rc;
    dev_.reset(d);
    rc = dev_->set_volsurf(p_.volsurf_method);
    if (rc != ST_OK) {
        if (err) *err = "volsurf_method not available";
        return rc;
    }
    ns_ = st.ns;
    nslots_ = st.nslots;
    agg_ = st.agg;
    agg_n_ = st.agg_n;
    alive_.resize(size_t(st.nslots));
    std::iota(alive_.begin(), alive_.end(), 0);
    maxradius_ = st.maxradius;
    dt_order_valid_ = false;
    return ST_OK;
}

// Oxidation after the spheres shrank on the device (calcul.cpp:157-170):
// Aggregate::croissance_surface with remove_sphere (aggregat.cpp:230-243,
// 629-655) and AggregatList::croissance_surface (aggregat_list.cpp:549-579),
// then Aggregate::split (aggregat.cpp:545-628, aggregat_list.cpp:409-446) of
// every aggregate, or of the moved one (label >= 0, the individual mode).
// Worked on the host in the reference's own order, every step being
// sequential and exact; when anything changed the device box is rebuilt in
// that order. The contact's sphere references are renumbered.
int HostBox::oxidize(int64_t label, mcacg_contact *c, bool *split, bool *disappear, std::string *err) {
    *split = *disappear = false;
    HostState cur;
    int rc = dev_->download(&cur, err);
    if (rc != ST_OK) return rc;
    LabelBox w;
    w.st.n_div = cur.n_div;
    w.st.box_length = cur.box_length;
    w.st.ns = cur.ns;
    w.st.sph.swap(cur.sph);
    const size_t na = alive_.size();
    w.f.resize(na);
    w.mem.resize(na);
    w.uid = uid_;
    for (size_t l = 0; l < na; ++l) {
        const int slot = alive_[l];
        for (int f = 0; f < 21; ++f) w.f[l][size_t(f)] = F(f, slot);
        const auto v = cur.members[size_t(slot)];
        w.mem[l].assign(v.begin(), v.end());
    }
    const double L = w.st.box_length, rp_min = p_.rp_min_oxid;
    double maxr = maxradius_;
    bool changed = false;
    int64_t *refs[2] = {&c->moving_sphere, &c->other_sphere};
    auto R = [&](int s) { return w.st.sph[size_t(SPH_R) * size_t(w.st.ns) + size_t(s)]; };
    auto P = [&](int s) {
        const size_t ns = size_t(w.st.ns);
        return Vec3{w.st.sph[size_t(SPH_X) * ns + size_t(s)], w.st.sph[size_t(SPH_Y) * ns + size_t(s)],
                    w.st.sph[size_t(SPH_Z) * ns + size_t(s)]};
    };
    // removal in one aggregate; true when it is left empty
    auto remove_small = [&](int a, int *status) {
        std::vector<int> &m = w.mem[size_t(a)];
        for (size_t k = 0; k < m.size();) {
            const int id = m[k];
            if (!(R(id) <= rp_min)) {
                ++k;
                continue;
            }
            m.erase(m.begin() + long(k));
            remove_storage(w, id, refs, 2);
            changed = true;
            if (!m.empty()) {
                const int r2 = rebase_update_place(p_, w, a, &maxr);
                if (r2 != ST_OK) {
                    *status = r2;
                    return false;
                }
            }
        }
        return m.empty();
    };
    auto erase_label = [&](int a) {
        w.f.erase(w.f.begin() + a);
        w.mem.erase(w.mem.begin() + a);
        w.uid.erase(w.uid.begin() + a);
        changed = true;
        *disappear = true;
    };
    // Aggregate::split of label a: parts as the reference walks them, each
    // appended as a copy of a's record with its spheres in discovery order
    // and updated, then a removed. Returns true when it split.
    auto split_one = [&](int a, int *status) {
        const std::vector<int> m = w.mem[size_t(a)];
        const int n = int(m.size());
        if (n < 2) return false;
        std::vector<int> unvisited(static_cast<size_t>(n));
        std::iota(unvisited.begin(), unvisited.end(), 0);
        std::vector<std::vector<int>> parts;
        while (!unvisited.empty()) {
            std::vector<int> part{unvisited.front()};
            unvisited.erase(unvisited.begin());
            std::vector<int> discovered = part;
            while (!discovered.empty()) {
                const int i1 = discovered.back();
                discovered.pop_back();
                for (size_t idx = 0; idx < unvisited.size();) {
                    const int i2 = unvisited[idx];
                    if (spheres_in_contact(P(m[size_t(i1)]), R(m[size_t(i1)]), P(m[size_t(i2)]), R(m[size_t(i2)]), L)) {
                        part.push_back(i2);
                        discovered.push_back(i2);
                        unvisited.erase(unvisited.begin() + long(idx));
                    } else {
                        ++idx;
                    }
                }
            }
            parts.push_back(std::move(part));
        }
        if (parts.size() < 2) return false;
        const std::array<double, 21> fa = w.f[size_t(a)];
        for (const auto &part : parts) {
            w.f.push_back(fa);
            w.uid.push_back(next_uid_++);
            std::vector<int> pm;
            for (int i : part) pm.push_back(m[size_t(i)]);
            w.mem.push_back(std::move(pm));
            const int r2 = rebase_update_place(p_, w, int(w.mem.size()) - 1, &maxr);
            if (r2 != ST_OK) {
                *status = r2;
                return true;
            }
        }
        erase_label(a);
        *disappear = false;  // a split, not a disappearance
        changed = true;
        return true;
    };
    int status = ST_OK;
    bool any_disappear = false;
    if (label >= 0) {
        if (remove_small(int(label), &status)) {
            erase_label(int(label));
            any_disappear = true;
        } else if (status == ST_OK) {
            *split = split_one(int(label), &status);
        }
    } else {
        for (int a = 0; a < int(w.mem.size()) && status == ST_OK;) {
            if (remove_small(a, &status)) {
                erase_label(a);
                any_disappear = true;
            } else {
                ++a;
            }
        }
        for (int a = 0; a < int(w.mem.size()) && status == ST_OK;) {
            if (split_one(a, &status)) *split = true;
            else ++a;
        }
    }
    *disappear = any_disappear;
    if (status != ST_OK) {
        if (err) *err = "volume/surface error in an oxidised aggregate";
        return status;
    }
    if (!changed) return ST_OK;
    // the state in label order (slot = label)
    HostState st;
    st.n_div = w.st.n_div;
    st.box_length = w.st.box_length;
    st.maxradius = maxr;
    st.time = time_;
    st.ns = w.st.ns;
    st.nslots = int(w.mem.size());
    st.sph.swap(w.st.sph);
    st.sph_slot.assign(size_t(st.ns), -1);
    st.agg.assign(size_t(21) * size_t(st.nslots), 0.0);
    st.agg_n.assign(size_t(st.nslots), 0);
    st.members.clear();
    for (int l = 0; l < st.nslots; ++l) {
        for (int f = 0; f < 21; ++f) st.agg[size_t(f) * size_t(st.nslots) + size_t(l)] = w.f[size_t(l)][size_t(f)];
        st.agg_n[size_t(l)] = int(w.mem[size_t(l)].size());
        st.members.push_list(w.mem[size_t(l)].data(), int(w.mem[size_t(l)].size()));
        for (int s : w.mem[size_t(l)]) st.sph_slot[size_t(s)] = l;
    }
    if (st.nslots == 0) {  // every sphere gone: an empty box
        alive_.clear();
        uid_.clear();
        ns_ = st.ns;
        maxradius_ = maxr;
        return ST_OK;
    }
    rc = replace_state(st, err);
    if (rc != ST_OK) return rc;
    uid_ = w.uid;
    return ST_OK;
}

int HostBox::calcul(const mcacg_run_opts &opts, mcacg_run_stats *stats, std::string *err) {
    const bool surface = p_.with_surface_reactions != 0;
    const bool individual = surface && p_.individual_surf_reactions != 0;
    const bool oxidation = surface && p_.u_sg < 0.0;
    if (p_.with_domain_duplication || p_.with_domain_reduction || p_.pick_method != MCACG_PICK_RANDOM ||
        (oxidation && p_.full_aggregate_update_frequency > 1)) {
        if (err) *err = "the host-driven loop covers collisions with optional surface reactions (no domain "
                        "duplication/reduction, pick_method=random; oxidation with a full update every step)";
        return ST_INPUT;
    }
    if (opts.advancement_path && (p_.write_events_frequency <= 0 || p_.write_between_event_frequency <= 0)) {
        if (err) *err = "write_events_frequency and write_between_event_frequency must be positive";
        return ST_INPUT;
    }
    int64_t steps = 0, events = 0;
    while (!finished()) {
        if (opts.max_steps > 0 && steps >= opts.max_steps) break;
        if (time_to_write() && opts.advancement_path) save_advancement(opts.advancement_path);
        double max = max_time_step_;
        if (event_ || surface) sort_time_steps(max);  // every step when time steps change (calcul.cpp:100-102)
        const int64_t label = pick_random();
        double deltatemps = get_time_step(max);
        const double deltatemps_pick = deltatemps;
        const int slot = alive_[size_t(label)];
        double deltatemps_indiv = F(AGG_TIME_STEP, slot);
        const double full_distance = F(AGG_LPM, slot);
        double dir[3];
        random_direction(dir);
        double move_distance = full_distance;
        const int n_try = 1;
        bool contact = false;
        mcacg_contact c{std::numeric_limits<double>::infinity(), -1, -1, -1, -1};
        if (p_.with_collisions) {
            int rc = distance_to_next_contact(label, dir, full_distance, &c, err);
            if (rc != ST_OK) return rc;
            contact = c.distance <= full_distance;
            if (contact) move_distance = c.distance;
        }
        double v[3] = {dir[0] * move_distance, dir[1] * move_distance, dir[2] * move_distance};
        int rc = translate(label, v, err);
        if (rc != ST_OK) return rc;
        deltatemps = deltatemps * (move_distance / full_distance + static_cast<double>(n_try - 1));
        deltatemps_indiv = deltatemps_indiv * (move_distance / full_distance + static_cast<double>(n_try - 1));
        time_forward(label, deltatemps, err);
        time_ = time_ + deltatemps;
        // surface reactions before the merge (calcul.cpp:157-170): every
        // sphere, or the moved aggregate's by its own time step, grows or
        // shrinks; with oxidation spheres leave, aggregates disappear or split
        const int64_t moving_uid = oxidation ? uid_[size_t(label)] : -1;
        const int64_t other_uid = oxidation && contact && c.other_aggregate >= 0 ? uid_[size_t(c.other_aggregate)] : -1;
        bool split = false, disappear = false;
        if (surface) {
            rc = individual ? dev_->grow(slot, p_.u_sg * deltatemps_indiv, err)
                            : dev_->grow(-1, p_.u_sg * deltatemps, err);
            if (rc != ST_OK) return rc;
        }
        if (oxidation) {
            rc = oxidize(individual ? label : -1, &c, &split, &disappear, err);
            if (rc != ST_OK) return rc;
        }
        int32_t merged = 0;
        if (contact && (!individual || !(split || disappear))) {
            if (oxidation) {
                // the contact's aggregates where they are now (-1: split or gone)
                c.moving_aggregate = label_of_uid(moving_uid);
                c.other_aggregate = label_of_uid(other_uid);
            }
            rc = merge(c, &merged, err);
            if (rc != ST_OK) return rc;
        }
        if (surface && !alive_.empty()) {
            // update() every full_aggregate_update_frequency-th step without
            // event, else update_partial(); the moved aggregate alone in the
            // individual mode unless there was an event (calcul.cpp:180-206)
            const int64_t every = std::max<int64_t>(1, p_.full_aggregate_update_frequency);
            const bool full = n_iter_without_event_ % every == 0;
            const bool alone = individual && !merged && !split && !disappear;
            rc = update_aggregates(alone ? alive_[size_t(label)] : -1, full, err);
            if (rc != ST_OK) return rc;
        }
        event_ = merged != 0 || split || disappear;
        if (event_) {
            n_iter_without_event_ = 0;
            ++events;
            ++total_events_;
            refresh();
            cpu_last_event_ = std::clock();  // calcul.cpp:238
        } else {
            n_iter_without_event_++;
        }
        if (event_ || surface) {
            // PhysicalModel::update after an event or with surface reactions
            // (calcul.cpp:274-279)
            aggregate_concentration_ = static_cast<double>(alive_.size()) / p_.box_volume;
            monomer_concentration_ = static_cast<double>(ns_) / p_.box_volume;
            volume_fraction_ = total_volume() / p_.box_volume;
        }
        if (opts.trace && steps < opts.trace_capacity) {
            mcacg_step_record &r = opts.trace[steps];
            r.step = steps;
            r.picked = label;
            r.contact = contact;
            r.merged = merged;
            r.moving_sphere = c.moving_sphere;
            r.other_sphere = c.other_sphere;
            r.moving_agg = c.moving_aggregate;
            r.other_agg = c.other_aggregate;
            r.n_agg_after = int64_t(alive_.size());
            r.deltatemps = deltatemps_pick;
            r.full_distance = full_distance;
            r.dir[0] = dir[0];
            r.dir[1] = dir[1];
            r.dir[2] = dir[2];
            r.contact_distance = c.distance;
            r.move_distance = move_distance;
            r.time_after = time_;
            r.reserved = 0;
        }
        ++steps;
    }
    // the final line, once, when the run has met its stop criteria (calcul.cpp:282)
    if (opts.advancement_path && finished() && !advancement_closed_) {
        save_advancement(opts.advancement_path);
        advancement_closed_ = true;
    }
    if (stats) {
        stats->steps = steps;
        stats->events = events;
        stats->n_aggregates = int64_t(alive_.size());
        stats->time = time_;
        stats->finished = finished() ? 1 : 0;
    }
    return ST_OK;
}

int HostBox::store(mcacg_state *out, std::string *err) {
    HostState st;
    int rc = dev_->download(&st, err);
    if (rc != ST_OK) return rc;

    const int na = int(alive_.size());
    if (out->n_spheres < ns_ || out->n_aggregates < na) {
        if (err) *err = "state buffers too small";
        return ST_BAD_ARGUMENT;
    }
    out->n_spheres = ns_;
    out->n_aggregates = na;
    out->n_verlet_divisions = st.n_div;
    out->box_length = st.box_length;
    out->maxradius = maxradius_;
    out->time = time_;
    if (out->spheres) {
        for (int f = 0; f < 9; ++f)
            std::memcpy(out->spheres + size_t(f) * ns_, st.sph.data() + size_t(f) * ns_, sizeof(double) * size_t(ns_));
    }
    if (out->sphere_label)
        for (int s = 0; s < ns_; ++s) out->sphere_label[s] = label_of(st.sph_slot[size_t(s)]);
    if (out->aggregates)
        for (int f = 0; f < 21; ++f)
            for (int l = 0; l < na; ++l) out->aggregates[size_t(f) * na + l] = F(f, alive_[size_t(l)]);
    int64_t off = 0;
    for (int l = 0; l < na; ++l) {
        const auto &m = st.members[size_t(alive_[size_t(l)])];
        if (out->n_spheres_per_aggregate) out->n_spheres_per_aggregate[l] = int64_t(m.size());
        if (out->members)
            for (size_t k = 0; k < m.size(); ++k) out->members[off + int64_t(k)] = m[k];
        off += int64_t(m.size());
    }
    return ST_OK;
}

}  // namespace mcacg

// ------------------------------------------------------- device-loop runs
namespace mcacg {

HostBox::HostBox() = default;
// the device-loop runner works on dev_'s stream and memory: it goes first
HostBox::~HostBox() { runner_.reset(); }

void HostBox::set_time(double t) {
    time_ = t;
    invalidate_device_run();
}

void HostBox::invalidate_device_run() {
    runner_.reset();
    runner_steps_ = runner_events_ = 0;
}

int HostBox::refresh_from_device(std::string *err) {
    HostState st;
    int rc = dev_->download(&st, err);
    if (rc != ST_OK) return rc;
    agg_ = st.agg;
    agg_n_ = st.agg_n;
    alive_.clear();
    for (int a = 0; a < nslots_; ++a)
        if (agg_n_[size_t(a)] > 0) alive_.push_back(a);
    maxradius_ = st.maxradius;
    event_ = true;
    dt_order_valid_ = false;
    if (!alive_.empty()) refresh();
    return ST_OK;
}

int HostBox::run_device(int64_t max_steps, mcacg_run_stats *stats, std::string *err) {
    if (!runner_) {
        // the host mirror holds the authoritative aggregate fields (proper
        // times and physics) after host-driven steps
        int up = dev_->upload_aggregates(agg_, err);
        if (up != ST_OK) return up;
        std::unique_ptr<BatchRunner> r;
        int rc = BatchRunner::attach({p_}, {dev_.get()}, {time_}, dev_->stream(), &r, err);
        if (rc != ST_OK) return rc;
        runner_ = std::move(r);
        runner_steps_ = runner_events_ = 0;
    }
    int rc = runner_->run(max_steps, 20000, err);
    if (rc != ST_OK) return rc;
    std::vector<BoxRunStats> s;
    rc = runner_->stats(&s, err);
    if (rc != ST_OK) return rc;
    const BoxRunStats &b = s[0];
    if (b.status != ST_OK) {
        if (err) *err = "device loop stopped with status " + std::to_string(b.status);
        return b.status;
    }
    time_ = b.time;
    rc = refresh_from_device(err);
    if (rc != ST_OK) return rc;
    if (stats) {
        stats->steps = b.steps - runner_steps_;
        stats->events = b.events - runner_events_;
        stats->n_aggregates = int64_t(alive_.size());
        stats->time = time_;
        stats->finished = b.finished;
    }
    runner_steps_ = b.steps;
    runner_events_ = b.events;
    return ST_OK;
}

}  // namespace mcacg
