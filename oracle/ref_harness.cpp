// Oracle harness around the reference MCAC objects (oracle/_ref/libmcac_ref.a).
// Test infrastructure only: it produces golden vectors from the reference
// itself and is never part of the product. It opens the reference classes'
// private members (a #define placed before the reference headers) so it can
// read and fill the reference's SoA storage directly.
//
// Modes
//   meta    <ini>                         print PhysicalModel-derived values
//   trace   <ini> <prefix> [step ...]     run the MC loop of src/calcul.cpp:66-281
//                                         (collisions only), write per-step records,
//                                         the initial/final state and states before
//                                         the listed steps
//   calcul  <ini> <prefix>                run the reference's own mcac::calcul and
//                                         write its final state (validates 'trace')
//   calcul_from <ini> <snap> <prefix>     load a state, run mcac::calcul on it with
//                                         the INI's parameters (e.g. oxidation) and
//                                         write its final state
//   queries <ini> <snap> <nq> <seed> <out> [update]
//                                         load a state, answer nq seeded
//                                         distance_to_next_contact queries
//   merges  <ini> <snap> <queries.bin> <out>
//                                         for each query record with a contact,
//                                         reload the state, translate, merge and
//                                         write the merged aggregate record
//
// Snapshot layout (little endian, written by write_snapshot): see
// mcac_gb300/snapshot.py, which reads and writes the same layout.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <experimental/filesystem>
#include <fstream>
#include <functional>
#include <iostream>
#include <limits>
#include <list>
#include <map>
#include <memory>
#include <numeric>
#include <set>
#include <sstream>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>
// Open the reference classes' members to this translation unit only; the
// standard headers above are included first so their access is unchanged.
#define private public
#define protected public
#include "aggregats/aggregat_list.hpp"
#include "aggregats/aggregat_distance.hpp"
#include "calcul.hpp"
#include "physical_model/physical_model.hpp"
#include "spheres/sphere.hpp"
#include "spheres/sphere_contact.hpp"
#include "spheres/sphere_distance.hpp"
#include "tools/tools.hpp"
#include "exceptions.hpp"
#include <inipp.h>

using namespace mcac;

namespace {

const char kMagic[8] = {'M', 'C', 'S', 'N', 'A', 'P', '0', '1'};

struct Writer {
    FILE *f;
    explicit Writer(const std::string &path) : f(std::fopen(path.c_str(), "wb")) {
        if (!f) { std::perror(path.c_str()); std::exit(2); }
    }
    ~Writer() { std::fclose(f); }
    void raw(const void *p, size_t n) { std::fwrite(p, 1, n, f); }
    void i64(int64_t v) { raw(&v, 8); }
    void f64(double v) { raw(&v, 8); }
};

struct Reader {
    FILE *f;
    explicit Reader(const std::string &path) : f(std::fopen(path.c_str(), "rb")) {
        if (!f) { std::perror(path.c_str()); std::exit(2); }
    }
    ~Reader() { std::fclose(f); }
    void raw(void *p, size_t n) {
        if (std::fread(p, 1, n, f) != n) { std::fprintf(stderr, "short read\n"); std::exit(2); }
    }
    int64_t i64() { int64_t v; raw(&v, 8); return v; }
    double f64() { double v; raw(&v, 8); return v; }
};

// Snapshot: header, sphere SoA (9 fields), sphere labels, aggregate SoA
// (21 fields), per-aggregate sphere counts, member lists (concatenated, in
// list order), per-aggregate Verlet cell, physics scalars.
void write_snapshot(const std::string &path, PhysicalModel &pm, AggregatList &al) {
    Writer w(path);
    w.raw(kMagic, 8);
    const int64_t ns = int64_t(al.spheres.size());
    const int64_t na = int64_t(al.size());
    w.i64(ns);
    w.i64(na);
    w.i64(int64_t(pm.n_verlet_divisions));
    w.f64(pm.box_length);
    w.f64(al.maxradius);
    w.f64(pm.time);
    // physics scalars used by update_partial
    w.f64(pm.temperature);
    w.f64(pm.pressure);
    w.f64(pm.density);
    w.f64(pm.viscosity);
    w.f64(pm.gaz_mean_free_path);
    w.f64(pm.fractal_dimension);
    w.f64(pm.fractal_prefactor);
    w.f64(pm.mean_massic_radius);
    w.f64(pm.friction_exponnant);
    w.i64(int64_t(pm.volsurf_method));
    for (int fld = 0; fld < SPHERE_NFIELDS; ++fld)
        for (int64_t s = 0; s < ns; ++s) w.f64((*al.spheres.storage)[fld][size_t(s)]);
    for (int64_t s = 0; s < ns; ++s) w.i64(int64_t(al.spheres[size_t(s)]->agg_label));
    for (int fld = 0; fld < AGGREGAT_NFIELDS; ++fld)
        for (int64_t a = 0; a < na; ++a) w.f64((*al.storage)[fld][size_t(a)]);
    for (int64_t a = 0; a < na; ++a) w.i64(int64_t(al[size_t(a)]->n_spheres));
    for (int64_t a = 0; a < na; ++a)
        for (const auto &sph : al[size_t(a)]->myspheres) w.i64(int64_t(sph->get_index()));
    for (int64_t a = 0; a < na; ++a)
        for (int k = 0; k < 3; ++k) w.i64(int64_t(al[size_t(a)]->index_verlet[size_t(k)]));
}

struct Snapshot {
    int64_t ns = 0, na = 0, n_div = 0;
    double box_length = 0, maxradius = 0, time = 0;
    std::vector<double> sph[SPHERE_NFIELDS];
    std::vector<int64_t> sph_label;
    std::vector<double> agg[AGGREGAT_NFIELDS];
    std::vector<int64_t> n_spheres, members, cells;
};

Snapshot read_snapshot(const std::string &path) {
    Reader r(path);
    char magic[8];
    r.raw(magic, 8);
    if (std::memcmp(magic, kMagic, 8) != 0) { std::fprintf(stderr, "bad snapshot\n"); std::exit(2); }
    Snapshot s;
    s.ns = r.i64();
    s.na = r.i64();
    s.n_div = r.i64();
    s.box_length = r.f64();
    s.maxradius = r.f64();
    s.time = r.f64();
    for (int k = 0; k < 9; ++k) r.f64();  // physics scalars (recomputed from the INI)
    r.i64();
    for (auto &col : s.sph) { col.resize(size_t(s.ns)); r.raw(col.data(), 8 * size_t(s.ns)); }
    s.sph_label.resize(size_t(s.ns));
    r.raw(s.sph_label.data(), 8 * size_t(s.ns));
    for (auto &col : s.agg) { col.resize(size_t(s.na)); r.raw(col.data(), 8 * size_t(s.na)); }
    s.n_spheres.resize(size_t(s.na));
    r.raw(s.n_spheres.data(), 8 * size_t(s.na));
    int64_t tot = 0;
    for (auto n : s.n_spheres) tot += n;
    s.members.resize(size_t(tot));
    r.raw(s.members.data(), 8 * size_t(tot));
    s.cells.resize(size_t(3 * s.na));
    r.raw(s.cells.data(), 8 * size_t(3 * s.na));
    return s;
}

// The AggregatList constructor always places n_monomeres random monomers;
// a snapshot load starts from a single one in a box of the snapshot's size.
void prepare_for_snapshot(PhysicalModel &pm, const Snapshot &s) {
    pm.n_monomeres = 1;
    pm.box_length = s.box_length;
    pm.box_volume = std::pow(s.box_length, 3);
    pm.n_verlet_divisions = size_t(s.n_div);
}

// Fill a freshly constructed AggregatList (built from an INI with number=1)
// with a snapshot. When 'update' is set, every aggregate is recomputed with
// Aggregate::update() (synthetic snapshots that only carry sphere data).
void load_snapshot(const Snapshot &s, PhysicalModel &pm, AggregatList &al, bool update) {
    for (const auto &agg : al.list) agg->unset_verlet();
    pm.box_length = s.box_length;
    pm.box_volume = std::pow(s.box_length, 3);
    pm.n_verlet_divisions = size_t(s.n_div);
    pm.time = s.time;
    al.verlet = Verlet(size_t(s.n_div), s.box_length);
    if (s.ns > 1) al.spheres.add(size_t(s.ns - 1), al.spheres);
    al.spheres.setpointers();
    if (s.na > 1) al.ListStorage<AGGREGAT_NFIELDS, Aggregate>::add(size_t(s.na - 1), al);
    al.setpointers();
    for (int64_t i = 0; i < s.ns; ++i) {
        for (int fld = 0; fld < SPHERE_NFIELDS; ++fld) (*al.spheres.storage)[fld][size_t(i)] = s.sph[fld][size_t(i)];
        al.spheres[size_t(i)]->agg_label = long(s.sph_label[size_t(i)]);
        al.spheres[size_t(i)]->physicalmodel = &pm;
    }
    al.spheres.setpointers();
    for (const auto &sph : al.spheres) sph->setpointers();
    int64_t off = 0;
    for (int64_t a = 0; a < s.na; ++a) {
        auto &agg = al.list[size_t(a)];
        agg->label = size_t(a);
        agg->index_in_storage = size_t(a);
        agg->physicalmodel = &pm;
        agg->setpointers();
        std::vector<size_t> idx;
        for (int64_t k = 0; k < s.n_spheres[size_t(a)]; ++k) idx.push_back(size_t(s.members[size_t(off + k)]));
        off += s.n_spheres[size_t(a)];
        agg->myspheres = SphereList(&al.spheres, idx);
        agg->n_spheres = agg->myspheres.size();
        agg->alpha_vs_extreme = 1.0 / double(agg->n_spheres);
        agg->electric_charge = 0;
        agg->bulk_density = pm.density;
        for (int fld = 0; fld < AGGREGAT_NFIELDS; ++fld) (*al.storage)[fld][size_t(a)] = s.agg[fld][size_t(a)];
    }
    al.maxradius = s.maxradius;
    for (const auto &agg : al.list) {
        if (update) {
            agg->update();
        } else {
            // internal caches used by merge/update are rebuilt by update();
            // queries only need positions, rmax and the member lists.
        }
        agg->set_verlet(&al.verlet);
    }
    al.refresh();
}


// The reference PhysicalModel constructor prompts on stdin when its output
// directory already exists (physical_model/physical_model.cpp:196-210); the
// harness removes that directory first so construction never blocks.
PhysicalModel &fresh_model(const std::string &ini, std::unique_ptr<PhysicalModel> &holder) {
    inipp::Ini<char> parsed;
    std::ifstream is(ini);
    parsed.parse(is);
    std::string out = "MCAC_output";
    inipp::extract(parsed.sections["output"]["output_dir"], out);
    std::experimental::filesystem::path dir = extract_path(ini) / out;
    std::error_code ec;
    std::experimental::filesystem::remove_all(dir, ec);
    holder = std::make_unique<PhysicalModel>(ini);
    return *holder;
}

// One fixed-size record per MC step.
struct StepRecord {
    int64_t step;
    int64_t picked;           // label picked by pick_random
    int64_t contact;          // next_contact <= full_distance
    int64_t merged;           // AggregatList::merge returned true
    int64_t moving_sphere;    // storage index, -1 if none
    int64_t other_sphere;
    int64_t moving_agg;       // label at query time, -1 if none
    int64_t other_agg;
    int64_t n_agg_after;
    double deltatemps;        // get_time_step(max) before scaling
    double full_distance;     // lpm of the picked aggregate
    double dir[3];
    double contact_distance;  // +inf if none
    double move_distance;
    double time_after;
    double u_pick_unused;     // reserved
};
static_assert(sizeof(StepRecord) == 18 * 8, "record layout");

int64_t sphere_index(const std::weak_ptr<Sphere> &w) {
    auto p = w.lock();
    return p ? int64_t(p->get_index()) : -1;
}
int64_t agg_label(const std::weak_ptr<Aggregate> &w) {
    auto p = w.lock();
    return p ? int64_t(p->get_label()) : -1;
}

int mode_meta(const std::string &ini) {
    std::unique_ptr<PhysicalModel> pm_holder;
    PhysicalModel &pm = fresh_model(ini, pm_holder);
    std::printf("box_length %.17g\n", pm.box_length);
    std::printf("box_volume %.17g\n", pm.box_volume);
    std::printf("gaz_mean_free_path %.17g\n", pm.gaz_mean_free_path);
    std::printf("viscosity %.17g\n", pm.viscosity);
    std::printf("mean_massic_radius %.17g\n", pm.mean_massic_radius);
    std::printf("friction_exponnant %.17g\n", pm.friction_exponnant);
    std::printf("u_sg %.17g\n", pm.u_sg);
    std::printf("aggregate_concentration %.17g\n", pm.aggregate_concentration);
    std::printf("fractal_dimension %.17g\n", pm.fractal_dimension);
    std::printf("fractal_prefactor %.17g\n", pm.fractal_prefactor);
    std::printf("temperature %.17g\n", pm.temperature);
    std::printf("pressure %.17g\n", pm.pressure);
    std::printf("density %.17g\n", pm.density);
    std::printf("n_monomeres %zu\n", pm.n_monomeres);
    std::printf("volume_fraction %.17g\n", pm.volume_fraction);
    std::printf("flux_surfgrowth %.17g\n", pm.flux_surfgrowth);
    std::printf("mean_diameter %.17g\n", pm.mean_diameter);
    std::printf("dispersion_diameter %.17g\n", pm.dispersion_diameter);
    std::printf("volsurf_method %d\n", int(pm.volsurf_method));
    std::printf("random_seed %d\n", pm.random_seed);
    std::printf("n_verlet_divisions %zu\n", pm.n_verlet_divisions);
    return 0;
}

int mode_trace(const std::string &ini, const std::string &prefix, const std::set<int64_t> &snap_steps) {
    std::unique_ptr<PhysicalModel> pm_holder;
    PhysicalModel &pm = fresh_model(ini, pm_holder);
    if (pm.with_surface_reactions || pm.with_nucleation || pm.with_potentials || pm.with_flame_coupling ||
        pm.with_domain_duplication || pm.with_domain_reduction || pm.pick_method != PickMethods::PICK_RANDOM) {
        std::fprintf(stderr, "trace mode covers the collision-only loop\n");
        return 2;
    }
    AggregatList al(&pm);
    write_snapshot(prefix + "_init.snap", pm, al);
    Writer tw(prefix + "_trace.bin");
    Writer mw(prefix + "_merges.bin");
    bool event = true;
    int64_t step = 0;
    while (!pm.finished(al.size(), al.get_avg_npp())) {
        if (snap_steps.count(step)) write_snapshot(prefix + "_step" + std::to_string(step) + ".snap", pm, al);
        StepRecord rec{};
        rec.step = step;
        double max = al.get_max_time_step();
        if (event) al.sort_time_steps(max);
        size_t num_agg = al.pick_random();
        double deltatemps = al.get_time_step(max);
        double full_distance = al[num_agg]->get_lpm();
        rec.picked = int64_t(num_agg);
        rec.deltatemps = deltatemps;
        rec.full_distance = full_distance;
        std::array<double, 3> vectdir = random_direction();
        double move_distance = full_distance;
        int n_try = 1;
        bool contact = false;
        AggregateContactInfo next_contact;
        if (pm.with_collisions) {
            next_contact = al.distance_to_next_contact(num_agg, vectdir, full_distance);
            contact = next_contact <= full_distance;
            if (contact) move_distance = next_contact.distance;
        }
        rec.dir[0] = vectdir[0];
        rec.dir[1] = vectdir[1];
        rec.dir[2] = vectdir[2];
        rec.contact = contact;
        rec.contact_distance = next_contact.distance;
        rec.moving_sphere = sphere_index(next_contact.moving_sphere);
        rec.other_sphere = sphere_index(next_contact.other_sphere);
        rec.moving_agg = agg_label(next_contact.moving_aggregate);
        rec.other_agg = agg_label(next_contact.other_aggregate);
        rec.move_distance = move_distance;
        al[num_agg]->translate(vectdir * move_distance);
        deltatemps = deltatemps * (move_distance / full_distance + static_cast<double>(n_try - 1));
        al[num_agg]->time_forward(deltatemps);
        pm.time = pm.time + deltatemps;
        bool merge = false;
        if (contact) merge = al.merge(next_contact);
        rec.merged = merge;
        event = merge;
        if (event) {
            pm.n_iter_without_event = 0;
        } else {
            pm.n_iter_without_event++;
        }
        if (event) al.refresh();
        if (event) pm.update(al.size(), al.spheres.size(), al.get_total_volume(), al.get_total_surface());
        rec.n_agg_after = int64_t(al.size());
        rec.time_after = pm.time;
        tw.raw(&rec, sizeof rec);
        if (merge) {
            // merged aggregate = min label of the two; record all fields.
            size_t keep = size_t(std::min(rec.moving_agg, rec.other_agg));
            mw.i64(step);
            mw.i64(int64_t(keep));
            mw.i64(int64_t(al[keep]->n_spheres));
            for (int fld = 0; fld < AGGREGAT_NFIELDS; ++fld) mw.f64((*al.storage)[fld][keep]);
            mw.f64(al.maxradius);
        }
        ++step;
    }
    write_snapshot(prefix + "_final.snap", pm, al);
    std::printf("steps %lld n_agg %zu time %.17g\n", (long long)step, al.size(), pm.time);
    return 0;
}

int mode_calcul(const std::string &ini, const std::string &prefix) {
    std::unique_ptr<PhysicalModel> pm_holder;
    PhysicalModel &pm = fresh_model(ini, pm_holder);
    AggregatList al(&pm);
    {
        // the reference prints a progress table; keep it out of the harness output
        std::ofstream devnull("/dev/null");
        auto *old = std::cout.rdbuf(devnull.rdbuf());
        calcul(pm, al);
        std::cout.rdbuf(old);
    }
    write_snapshot(prefix + "_final.snap", pm, al);
    std::printf("n_agg %zu time %.17g\n", al.size(), pm.time);
    return 0;
}

int mode_calcul_from(const std::string &ini, const std::string &snap, const std::string &prefix) {
    std::unique_ptr<PhysicalModel> pm_holder;
    PhysicalModel &pm = fresh_model(ini, pm_holder);
    Snapshot s = read_snapshot(snap);
    prepare_for_snapshot(pm, s);
    AggregatList al(&pm);
    load_snapshot(s, pm, al, true);
    {
        std::ofstream devnull("/dev/null");
        auto *old = std::cout.rdbuf(devnull.rdbuf());
        calcul(pm, al);
        std::cout.rdbuf(old);
    }
    write_snapshot(prefix + "_final.snap", pm, al);
    std::printf("n_agg %zu n_spheres %zu time %.17g\n", al.size(), al.spheres.size(), pm.time);
    return 0;
}

// Query record: inputs and the reference answer.
struct QueryRecord {
    int64_t label;
    int64_t moving_sphere;
    int64_t other_sphere;
    int64_t moving_agg;
    int64_t other_agg;
    int64_t contact;
    double dir[3];
    double distance;
    double contact_distance;
    double pad;
};
static_assert(sizeof(QueryRecord) == 6 * 8 + 6 * 8, "query layout");

int mode_queries(const std::string &ini, const std::string &snap, int64_t nq, int seed, const std::string &out,
                 bool update) {
    std::unique_ptr<PhysicalModel> pm_holder;
    PhysicalModel &pm = fresh_model(ini, pm_holder);
    Snapshot s = read_snapshot(snap);
    prepare_for_snapshot(pm, s);
    AggregatList al(&pm);
    load_snapshot(s, pm, al, update);
    if (update) write_snapshot(out + ".snap", pm, al);
    srand(unsigned(seed));
    Writer w(out);
    for (int64_t q = 0; q < nq; ++q) {
        QueryRecord rec{};
        size_t label = size_t(mcac::random() * double(al.size()));
        if (label >= al.size()) label = al.size() - 1;
        std::array<double, 3> dir = random_direction();
        double dist = al[label]->get_lpm();
        AggregateContactInfo info = al.distance_to_next_contact(label, dir, dist);
        rec.label = int64_t(label);
        rec.dir[0] = dir[0];
        rec.dir[1] = dir[1];
        rec.dir[2] = dir[2];
        rec.distance = dist;
        rec.contact_distance = info.distance;
        rec.contact = info <= dist;
        rec.moving_sphere = sphere_index(info.moving_sphere);
        rec.other_sphere = sphere_index(info.other_sphere);
        rec.moving_agg = agg_label(info.moving_aggregate);
        rec.other_agg = agg_label(info.other_aggregate);
        w.raw(&rec, sizeof rec);
    }
    return 0;
}

int mode_merges(const std::string &ini, const std::string &snap, const std::string &qpath, const std::string &out) {
    Snapshot s = read_snapshot(snap);
    std::vector<QueryRecord> qs;
    {
        Reader r(qpath);
        QueryRecord rec;
        while (std::fread(&rec, sizeof rec, 1, r.f) == 1) qs.push_back(rec);
    }
    Writer w(out);
    for (size_t q = 0; q < qs.size(); ++q) {
        if (!qs[q].contact) continue;
        std::unique_ptr<PhysicalModel> pm_holder;
        PhysicalModel &pm = fresh_model(ini, pm_holder);
        prepare_for_snapshot(pm, s);
        AggregatList al(&pm);
        // the merged aggregate is rebuilt from its spheres by the reference's
        // own Aggregate::update(); the others are used as stored.
        load_snapshot(s, pm, al, false);
        std::array<double, 3> dir{qs[q].dir[0], qs[q].dir[1], qs[q].dir[2]};
        size_t label = size_t(qs[q].label);
        AggregateContactInfo info = al.distance_to_next_contact(label, dir, qs[q].distance);
        if (!(info <= qs[q].distance)) continue;
        al[label]->translate(dir * info.distance);
        double newtime_ref = pm.time;
        bool merged = al.merge(info);
        size_t keep = size_t(std::min(qs[q].moving_agg, qs[q].other_agg));
        w.i64(int64_t(q));
        w.i64(merged);
        w.i64(int64_t(keep));
        w.i64(int64_t(al[keep]->n_spheres));
        for (int fld = 0; fld < AGGREGAT_NFIELDS; ++fld) w.f64((*al.storage)[fld][keep]);
        w.f64(al.maxradius);
        w.f64(newtime_ref);
        // the merged aggregate's sphere rows, in list order
        for (const auto &sph : al[keep]->myspheres) {
            w.i64(int64_t(sph->get_index()));
            for (int fld = 0; fld < SPHERE_NFIELDS; ++fld) w.f64((*al.spheres.storage)[fld][sph->get_index()]);
        }
    }
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s meta|trace|calcul|queries|merges ...\n", argv[0]);
        return 2;
    }
    std::string mode = argv[1];
    try {
        if (mode == "meta") return mode_meta(argv[2]);
        if (mode == "trace" && argc >= 4) {
            std::set<int64_t> steps;
            for (int i = 4; i < argc; ++i) steps.insert(std::atoll(argv[i]));
            std::ofstream devnull("/dev/null");
            auto *old = std::cout.rdbuf(devnull.rdbuf());
            int rc = mode_trace(argv[2], argv[3], steps);
            std::cout.rdbuf(old);
            return rc;
        }
        if (mode == "calcul" && argc >= 4) return mode_calcul(argv[2], argv[3]);
        if (mode == "calcul_from" && argc >= 5) return mode_calcul_from(argv[2], argv[3], argv[4]);
        if (mode == "queries" && argc >= 7) {
            std::ofstream devnull("/dev/null");
            auto *old = std::cout.rdbuf(devnull.rdbuf());
            int rc = mode_queries(argv[2], argv[3], std::atoll(argv[4]), std::atoi(argv[5]), argv[6],
                                  argc >= 8 && std::string(argv[7]) == "update");
            std::cout.rdbuf(old);
            return rc;
        }
        if (mode == "merges" && argc >= 6) {
            std::ofstream devnull("/dev/null");
            auto *old = std::cout.rdbuf(devnull.rdbuf());
            int rc = mode_merges(argv[2], argv[3], argv[4], argv[5]);
            std::cout.rdbuf(old);
            return rc;
        }
    } catch (const BaseException &e) {
        std::fprintf(stderr, "reference error %d: %s\n", int(e.code), e.what());
        return int(e.code);
    }
    std::fprintf(stderr, "bad arguments\n");
    return 2;
}
