// extern "C" entry points of include/mcacg.h. No exception crosses this
// boundary: every call returns a status code and records a message for
// mcacg_last_error().
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <atomic>
#include <thread>
#include <vector>
#include <exception>
#include <fstream>
#include <memory>
#include <new>
#include <sstream>
#include <string>

#include "../../include/mcacg.h"
#include "common.hpp"
#include "batch.hpp"
#include "host_box.hpp"
#include "physics.hpp"
#include "static_query.hpp"
#include "host_parallel.hpp"

struct mcacg_box {
    std::unique_ptr<mcacg::HostBox> impl;
};

struct mcacg_batch {
    std::unique_ptr<mcacg::BatchRunner> impl;
    std::vector<mcacg_params> params;
};

struct mcacg_server {
    std::unique_ptr<mcacg::Server> impl;
    std::vector<mcacg::Completion> unread;
};

namespace {

// A slot-ordered device state as the C-ABI's label-ordered arrays.
int store_host_state(const mcacg::HostState &st, mcacg_state *out, std::string *err) {
    std::vector<int> label_of(size_t(st.nslots), -1);
    int na = 0;
    for (int a = 0; a < st.nslots; ++a)
        if (st.agg_n[size_t(a)] > 0) label_of[size_t(a)] = na++;
    if (out->n_spheres < st.ns || out->n_aggregates < na) {
        if (err) *err = "state buffers too small";
        return mcacg::ST_BAD_ARGUMENT;
    }
    out->n_spheres = st.ns;
    out->n_aggregates = na;
    out->n_verlet_divisions = st.n_div;
    out->box_length = st.box_length;
    out->maxradius = st.maxradius;
    out->time = st.time;
    if (out->spheres) std::copy(st.sph.begin(), st.sph.end(), out->spheres);
    if (out->sphere_label)
        for (int s = 0; s < st.ns; ++s) {
            const int a = st.sph_slot[size_t(s)];
            out->sphere_label[s] = a >= 0 && a < st.nslots ? label_of[size_t(a)] : -1;
        }
    int64_t off = 0;
    for (int a = 0; a < st.nslots; ++a) {
        int l = label_of[size_t(a)];
        if (l < 0) continue;
        if (out->aggregates)
            for (int f = 0; f < 21; ++f) out->aggregates[size_t(f) * na + l] = st.agg[size_t(f) * st.nslots + a];
        const auto &m = st.members[size_t(a)];
        if (out->n_spheres_per_aggregate) out->n_spheres_per_aggregate[l] = int64_t(m.size());
        if (out->members)
            for (size_t k = 0; k < m.size(); ++k) out->members[off + int64_t(k)] = m[k];
        off += int64_t(m.size());
    }
    return mcacg::ST_OK;
}

// Spheres taken out by oxidation (label -1) leave a stored state, as they
// leave the reference's sphere storage (aggregat.cpp:629-641): the others
// keep their order, the tables are packed as [9][n_spheres], and the member
// lists are renumbered.
void drop_removed_spheres(mcacg_state *out) {
    const int64_t ns = out->n_spheres;
    if (!out->sphere_label || !out->spheres) return;
    bool any = false;
    for (int64_t s = 0; s < ns && !any; ++s) any = out->sphere_label[s] < 0;
    if (!any) return;
    std::vector<int64_t> new_index(static_cast<size_t>(ns), -1);
    int64_t live = 0;
    for (int64_t s = 0; s < ns; ++s)
        if (out->sphere_label[s] >= 0) new_index[size_t(s)] = live++;
    // destinations never pass their sources: in place, in increasing order
    for (int64_t f = 0; f < 9; ++f)
        for (int64_t s = 0; s < ns; ++s)
            if (new_index[size_t(s)] >= 0) out->spheres[f * live + new_index[size_t(s)]] = out->spheres[f * ns + s];
    for (int64_t s = 0; s < ns; ++s)
        if (new_index[size_t(s)] >= 0) out->sphere_label[new_index[size_t(s)]] = out->sphere_label[s];
    if (out->members && out->n_spheres_per_aggregate) {
        int64_t total = 0;
        for (int64_t a = 0; a < out->n_aggregates; ++a) total += out->n_spheres_per_aggregate[a];
        for (int64_t k = 0; k < total && k < ns; ++k) {
            const int64_t m = out->members[k];
            out->members[k] = m >= 0 && m < ns ? new_index[size_t(m)] : -1;
        }
    }
    out->n_spheres = live;
}

thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

template <class F>
int guarded(F &&f) {
    try {
        g_last_error.clear();
        return f();
    } catch (const std::bad_alloc &) {
        return fail(mcacg::ST_CAPACITY, "host allocation failed");
    } catch (const std::exception &e) {
        return fail(mcacg::ST_UNKNOWN, e.what());
    } catch (...) {
        return fail(mcacg::ST_UNKNOWN, "unknown error");
    }
}

int finish(int rc, const std::string &err) {
    if (rc != mcacg::ST_OK) g_last_error = err.empty() ? "error " + std::to_string(rc) : err;
    return rc;
}

}  // namespace

extern "C" {

int mcacg_abi_version(void) { return MCACG_ABI_VERSION; }

const char *mcacg_last_error(void) { return g_last_error.c_str(); }

int mcacg_device_count(int *count) {
    return guarded([&] {
        if (!count) return fail(MCACG_ERR_BAD_ARGUMENT, "null count");
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess) n = 0;
        cudaGetLastError();
        *count = n;
        return 0;
    });
}

int mcacg_params_default(mcacg_params *params) {
    return guarded([&] {
        if (!params) return fail(MCACG_ERR_BAD_ARGUMENT, "null params");
        mcacg::params_defaults(params);
        mcacg::params_derive(params);
        return 0;
    });
}

int mcacg_params_from_ini_text(const char *text, mcacg_params *params) {
    return guarded([&] {
        if (!text || !params) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        std::string err;
        int rc = mcacg::params_from_ini(mcacg::parse_ini_text(text), params, &err);
        return finish(rc, err);
    });
}

int mcacg_params_from_ini(const char *path, mcacg_params *params) {
    return guarded([&] {
        if (!path || !params) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        std::ifstream is(path);
        if (!is) return fail(mcacg::ST_INPUT, std::string("File does not exist: ") + path);
        std::stringstream ss;
        ss << is.rdbuf();
        std::string err;
        int rc = mcacg::params_from_ini(mcacg::parse_ini_text(ss.str()), params, &err);
        return finish(rc, err);
    });
}

int mcacg_state_init_random(const mcacg_params *params, mcacg_state *state) {
    return guarded([&] {
        if (!params || !state || !state->spheres || !state->sphere_label || !state->aggregates ||
            !state->n_spheres_per_aggregate || !state->members)
            return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        if (state->n_spheres < params->n_monomeres || state->n_aggregates < params->n_monomeres)
            return fail(MCACG_ERR_BAD_ARGUMENT, "state buffers smaller than n_monomeres");
        mcacg::HostState st;
        std::string err;
        int rc = mcacg::init_random_state(*params, &st, &err);
        if (rc != 0) return finish(rc, err);
        state->n_spheres = st.ns;
        state->n_aggregates = st.nslots;
        state->n_verlet_divisions = st.n_div;
        state->box_length = st.box_length;
        state->maxradius = st.maxradius;
        state->time = st.time;
        std::copy(st.sph.begin(), st.sph.end(), state->spheres);
        for (int s = 0; s < st.ns; ++s) state->sphere_label[s] = st.sph_slot[size_t(s)];
        std::copy(st.agg.begin(), st.agg.end(), state->aggregates);
        int64_t off = 0;
        for (int a = 0; a < st.nslots; ++a) {
            state->n_spheres_per_aggregate[a] = int64_t(st.members[size_t(a)].size());
            for (int m : st.members[size_t(a)]) state->members[off++] = m;
        }
        return 0;
    });
}

int mcacg_state_synthetic(const mcacg_params *params, int32_t n_aggregates, int32_t max_size, mcacg_state *state) {
    return guarded([&] {
        if (!params || !state || !state->spheres || !state->sphere_label || !state->aggregates ||
            !state->n_spheres_per_aggregate || !state->members)
            return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        if (params->n_monomeres > INT32_MAX) return fail(MCACG_ERR_BAD_ARGUMENT, "too many spheres");
        if (state->n_spheres < params->n_monomeres || state->n_aggregates < n_aggregates)
            return fail(MCACG_ERR_BAD_ARGUMENT, "state buffers too small");
        mcacg::HostState st;
        std::string err;
        int rc = mcacg::make_synthetic_state(*params, n_aggregates, max_size, &st, &err);
        if (rc != 0) return finish(rc, err);
        const int rc2 = store_host_state(st, state, &err);
        if (rc2 == 0) drop_removed_spheres(state);
        return finish(rc2, err);
    });
}

int mcacg_box_create(const mcacg_params *params, mcacg_box **box) {
    return guarded([&] {
        if (!params || !box) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        *box = nullptr;
        std::unique_ptr<mcacg_box> b(new mcacg_box());
        std::string err;
        int rc = mcacg::HostBox::create_random(*params, nullptr, &b->impl, &err);
        if (rc != 0) return finish(rc, err);
        *box = b.release();
        return 0;
    });
}

int mcacg_box_create_from_state(const mcacg_params *params, const mcacg_state *state, mcacg_box **box) {
    return guarded([&] {
        if (!params || !state || !box) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        *box = nullptr;
        std::unique_ptr<mcacg_box> b(new mcacg_box());
        std::string err;
        int rc = mcacg::HostBox::create_from_state(*params, *state, nullptr, &b->impl, &err);
        if (rc != 0) return finish(rc, err);
        *box = b.release();
        return 0;
    });
}

int mcacg_box_destroy(mcacg_box *box) {
    return guarded([&] {
        delete box;
        return 0;
    });
}

int mcacg_box_set_stream(mcacg_box *box, void *cuda_stream) {
    return guarded([&] {
        if (!box) return fail(MCACG_ERR_BAD_ARGUMENT, "null box");
        return box->impl->device().set_stream(cuda_stream);
    });
}

int mcacg_box_sizes(const mcacg_box *box, int64_t *n_spheres, int64_t *n_aggregates) {
    return guarded([&] {
        if (!box) return fail(MCACG_ERR_BAD_ARGUMENT, "null box");
        if (n_spheres) *n_spheres = box->impl->n_spheres();
        if (n_aggregates) *n_aggregates = box->impl->size();
        return 0;
    });
}

int mcacg_box_store_state(mcacg_box *box, mcacg_state *state) {
    return guarded([&] {
        if (!box || !state) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        std::string err;
        return finish(box->impl->store(state, &err), err);
    });
}

int mcacg_box_get_time(const mcacg_box *box, double *time) {
    return guarded([&] {
        if (!box || !time) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        *time = box->impl->time();
        return 0;
    });
}

int mcacg_box_set_profiling(mcacg_box *box, int enable) {
    return guarded([&] {
        if (!box) return fail(MCACG_ERR_BAD_ARGUMENT, "null box");
        box->impl->device().set_profiling(enable != 0);
        return 0;
    });
}

int mcacg_box_take_profile(mcacg_box *box, mcacg_profile *out) {
    return guarded([&] {
        if (!box || !out) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        mcacg::Profile p = box->impl->device().take_profile();
        out->queries = p.queries;
        out->merges = p.merges;
        out->translates = p.translates;
        out->query_ms = p.query_ms;
        out->merge_ms = p.merge_ms;
        out->mov_spheres = p.mov_spheres;
        out->scanned = p.scanned;
        out->cells = p.cells;
        out->candidates = p.candidates;
        out->cand_spheres = p.cand_spheres;
        out->refined = p.refined;
        out->merged_spheres = p.merged_spheres;
        out->merge_pairs = p.merge_pairs;
        return 0;
    });
}

int mcacg_box_set_time(mcacg_box *box, double time) {
    return guarded([&] {
        if (!box) return fail(MCACG_ERR_BAD_ARGUMENT, "null box");
        box->impl->set_time(time);
        return 0;
    });
}

int mcacg_distance_to_next_contact(mcacg_box *box, int64_t source, const double direction[3], double distance,
                                   mcacg_contact *out) {
    return guarded([&] {
        if (!box || !direction || !out) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        std::string err;
        return finish(box->impl->distance_to_next_contact(source, direction, distance, out, &err), err);
    });
}

int mcacg_distance_to_next_contacts(mcacg_box *box, int32_t n, const int64_t *sources, const double *directions,
                                    const double *distances, mcacg_contact *out, double *kernel_ms) {
    return guarded([&] {
        if (!box || n < 0 || (n > 0 && (!sources || !directions || !distances || !out)))
            return fail(MCACG_ERR_BAD_ARGUMENT, "null argument or negative count");
        std::string err;
        return finish(box->impl->distance_to_next_contacts(n, sources, directions, distances, out, kernel_ms, &err),
                      err);
    });
}

int mcacg_distance_to_next_contacts_static(mcacg_box *box, int32_t n, const int64_t *sources,
                                           const double *directions, const double *distances, mcacg_contact *out) {
    return guarded([&] {
        if (!box || n < 0 || (n > 0 && (!sources || !directions || !distances || !out)))
            return fail(MCACG_ERR_BAD_ARGUMENT, "null argument or negative count");
        // labels to slots here, on the host, from the box's live-slot list
        const mcacg::HostBox &hb = *box->impl;
        std::vector<int> slots(static_cast<size_t>(n));
        for (int k = 0; k < n; ++k) {
            if (sources[k] < 0 || sources[k] >= int64_t(hb.size()))
                return fail(MCACG_ERR_BAD_ARGUMENT, "label out of range in query " + std::to_string(k));
            slots[size_t(k)] = hb.slot_of(sources[k]);
        }
        std::string err;
        const int rc = mcacg::query_batch_static(box->impl->device(), n, slots.data(), directions, distances, out, &err);
        for (int k = 0; k < n && rc == 0; ++k) {
            mcacg_contact &c = out[k];
            if (c.moving_sphere >= 0) {
                c.moving_aggregate = sources[k];
                c.other_aggregate = hb.label_of(int(c.other_aggregate));  // the kernel wrote the slot
            } else {
                c.moving_aggregate = -1;
                c.other_aggregate = -1;
            }
        }
        return finish(rc, err);
    });
}

int mcacg_translate(mcacg_box *box, int64_t label, const double vector[3]) {
    return guarded([&] {
        if (!box || !vector) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        std::string err;
        return finish(box->impl->translate(label, vector, &err), err);
    });
}

int mcacg_time_forward(mcacg_box *box, int64_t label, double deltatemps) {
    return guarded([&] {
        if (!box) return fail(MCACG_ERR_BAD_ARGUMENT, "null box");
        std::string err;
        return finish(box->impl->time_forward(label, deltatemps, &err), err);
    });
}

int mcacg_merge(mcacg_box *box, const mcacg_contact *contact, int32_t *merged) {
    return guarded([&] {
        if (!box || !contact || !merged) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        std::string err;
        return finish(box->impl->merge(*contact, merged, &err), err);
    });
}

int mcacg_sort_time_steps(mcacg_box *box, double factor) {
    return guarded([&] {
        if (!box) return fail(MCACG_ERR_BAD_ARGUMENT, "null box");
        box->impl->sort_time_steps(factor);
        return 0;
    });
}

int mcacg_pick_random(mcacg_box *box, int64_t *label) {
    return guarded([&] {
        if (!box || !label) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        *label = box->impl->pick_random();
        return 0;
    });
}

int mcacg_get_time_step(const mcacg_box *box, double max, double *deltatemps) {
    return guarded([&] {
        if (!box || !deltatemps) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        *deltatemps = box->impl->get_time_step(max);
        return 0;
    });
}

int mcacg_get_max_time_step(const mcacg_box *box, double *max) {
    return guarded([&] {
        if (!box || !max) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        *max = box->impl->max_time_step();
        return 0;
    });
}

int mcacg_refresh(mcacg_box *box) {
    return guarded([&] {
        if (!box) return fail(MCACG_ERR_BAD_ARGUMENT, "null box");
        box->impl->refresh();
        return 0;
    });
}

int mcacg_size(const mcacg_box *box, int64_t *n_aggregates) {
    return guarded([&] {
        if (!box || !n_aggregates) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        *n_aggregates = box->impl->size();
        return 0;
    });
}

int mcacg_get_avg_npp(const mcacg_box *box, double *avg_npp) {
    return guarded([&] {
        if (!box || !avg_npp) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        *avg_npp = box->impl->avg_npp();
        return 0;
    });
}

int mcacg_get_total_volume(const mcacg_box *box, double *volume) {
    return guarded([&] {
        if (!box || !volume) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        *volume = box->impl->total_volume();
        return 0;
    });
}

int mcacg_get_total_surface(const mcacg_box *box, double *surface) {
    return guarded([&] {
        if (!box || !surface) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        *surface = box->impl->total_surface();
        return 0;
    });
}

int mcacg_get_aggregate(const mcacg_box *box, int64_t label, double fields[21], int64_t *n_spheres) {
    return guarded([&] {
        if (!box || !fields) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        if (label < 0 || label >= box->impl->size()) return fail(MCACG_ERR_BAD_ARGUMENT, "label out of range");
        box->impl->fields(label, fields);
        if (n_spheres) *n_spheres = box->impl->n_spheres_of(label);
        return 0;
    });
}

int mcacg_calcul(mcacg_box *box, const mcacg_run_opts *opts, mcacg_run_stats *stats) {
    return guarded([&] {
        if (!box) return fail(MCACG_ERR_BAD_ARGUMENT, "null box");
        mcacg_run_opts o{};
        if (opts) o = *opts;
        mcacg_run_stats s{};
        std::string err;
        int rc = box->impl->calcul(o, &s, &err);
        if (stats) *stats = s;
        return finish(rc, err);
    });
}

int mcacg_run_device(mcacg_box *box, int64_t max_steps, mcacg_run_stats *stats) {
    return guarded([&] {
        if (!box) return fail(MCACG_ERR_BAD_ARGUMENT, "null box");
        mcacg_run_stats s{};
        std::string err;
        int rc = box->impl->run_device(max_steps, &s, &err);
        if (stats) *stats = s;
        return finish(rc, err);
    });
}

int mcacg_batch_create(const mcacg_params *params, int32_t n_boxes, void *cuda_stream, mcacg_batch **batch) {
    return guarded([&] {
        if (!params || !batch || n_boxes <= 0) return fail(MCACG_ERR_BAD_ARGUMENT, "bad argument");
        *batch = nullptr;
        std::vector<mcacg_params> ps(params, params + n_boxes);
        for (const auto &p : ps)
            if (p.with_nucleation || p.with_potentials || p.with_flame_coupling || p.with_electric_charges)
                return fail(mcacg::ST_INPUT, "batched boxes cover collisions with optional surface reactions");
        // placements in parallel: each box draws from its own copy of the C
        // library stream, so the result equals a sequential placement
        std::vector<mcacg::HostState> states(static_cast<size_t>(n_boxes));
        std::vector<int> rcs(static_cast<size_t>(n_boxes), 0);
        std::vector<std::string> errs(static_cast<size_t>(n_boxes));
        mcacg::parallel_for(n_boxes, [&](int i) {
            rcs[size_t(i)] = mcacg::init_random_state_private(ps[size_t(i)], &states[size_t(i)], &errs[size_t(i)]);
        });
        for (int i = 0; i < n_boxes; ++i)
            if (rcs[size_t(i)] != 0) return fail(rcs[size_t(i)], "box " + std::to_string(i) + ": " + errs[size_t(i)]);
        std::unique_ptr<mcacg_batch> b(new mcacg_batch());
        std::string err;
        int rc = mcacg::BatchRunner::create(ps, std::move(states), cuda_stream, &b->impl, &err);
        if (rc != 0) return finish(rc, err);
        b->params = ps;
        *batch = b.release();
        return 0;
    });
}

int mcacg_batch_create_from_states(const mcacg_params *params, const mcacg_state *states, int32_t n_boxes,
                                   void *cuda_stream, mcacg_batch **batch) {
    return guarded([&] {
        if (!params || !states || !batch || n_boxes <= 0) return fail(MCACG_ERR_BAD_ARGUMENT, "bad argument");
        *batch = nullptr;
        std::vector<mcacg_params> ps(params, params + n_boxes);
        for (const auto &p : ps)
            if (p.with_nucleation || p.with_potentials || p.with_flame_coupling || p.with_electric_charges)
                return fail(mcacg::ST_INPUT, "batched boxes cover collisions with optional surface reactions");
        // the boxes load straight from the caller's arrays (by DMA when they
        // are page-locked); the device checks labels, counts and member lists
        std::vector<mcacg::StateView> views(static_cast<size_t>(n_boxes));
        // a box that oxidises needs a slot for every sphere (splits): its
        // aggregate table is copied into one with dead slots after the live ones
        std::vector<std::vector<double>> pad_agg(static_cast<size_t>(n_boxes));
        std::vector<std::vector<int64_t>> pad_count(static_cast<size_t>(n_boxes));
        bool padded = false;
        for (int i = 0; i < n_boxes; ++i) {
            const mcacg_state &in = states[i];
            if (in.n_spheres <= 0 || in.n_aggregates <= 0 || in.n_spheres > INT32_MAX ||
                in.n_aggregates > in.n_spheres || !in.spheres || !in.sphere_label || !in.aggregates ||
                !in.n_spheres_per_aggregate || !in.members || in.n_verlet_divisions <= 0 ||
                in.n_verlet_divisions > 1024 || !(in.box_length > 0.0))
                return fail(mcacg::ST_BAD_ARGUMENT, "box " + std::to_string(i) + ": incomplete state");
            mcacg::StateView &v = views[size_t(i)];
            v.n_div = int(in.n_verlet_divisions);
            v.box_length = in.box_length;
            v.maxradius = in.maxradius;
            v.time = in.time;
            v.ns = int(in.n_spheres);
            v.nslots = int(in.n_aggregates);
            v.sph = in.spheres;
            v.agg = in.aggregates;
            v.sph_slot = in.sphere_label;
            v.agg_n = in.n_spheres_per_aggregate;
            v.members = in.members;
            v.wide = true;
            v.dead_slots = false;
            ps[size_t(i)].box_length = in.box_length;
            ps[size_t(i)].n_verlet_divisions = in.n_verlet_divisions;
            const mcacg_params &p = ps[size_t(i)];
            if (p.with_surface_reactions && p.u_sg < 0.0 && v.nslots < v.ns) {
                const size_t ns = size_t(v.ns), na = size_t(v.nslots);
                std::vector<double> &agg = pad_agg[size_t(i)];
                agg.assign(21 * ns, 0.0);
                for (size_t f = 0; f < 21; ++f)
                    std::copy(in.aggregates + f * na, in.aggregates + (f + 1) * na, agg.begin() + long(f * ns));
                pad_count[size_t(i)].assign(ns, 0);
                std::copy(in.n_spheres_per_aggregate, in.n_spheres_per_aggregate + na, pad_count[size_t(i)].begin());
                v.nslots = v.ns;
                v.agg = agg.data();
                v.agg_n = pad_count[size_t(i)].data();
                padded = true;
            }
        }
        if (padded)
            for (auto &v : views) v.dead_slots = true;
        std::string err;
        std::unique_ptr<mcacg_batch> b(new mcacg_batch());
        int rc = mcacg::BatchRunner::create(ps, views, cuda_stream, &b->impl, &err);
        if (rc != 0) return finish(rc, err);
        b->params = ps;
        *batch = b.release();
        return 0;
    });
}

int mcacg_batch_destroy(mcacg_batch *batch) {
    return guarded([&] {
        delete batch;
        return 0;
    });
}

int mcacg_batch_run(mcacg_batch *batch, int64_t max_steps, int64_t steps_per_launch) {
    return guarded([&] {
        if (!batch) return fail(MCACG_ERR_BAD_ARGUMENT, "null batch");
        std::string err;
        return finish(batch->impl->run(max_steps, steps_per_launch, &err), err);
    });
}

int mcacg_batch_run_timed(mcacg_batch *batch, double wall_ms) {
    return guarded([&] {
        if (!batch || !(wall_ms >= 0.0)) return fail(MCACG_ERR_BAD_ARGUMENT, "bad argument");
        std::string err;
        return finish(batch->impl->run_timed(wall_ms, &err), err);
    });
}

int mcacg_batch_stats(mcacg_batch *batch, mcacg_run_stats *stats) {
    return guarded([&] {
        if (!batch || !stats) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        std::vector<mcacg::BoxRunStats> s;
        std::string err;
        int rc = batch->impl->stats(&s, &err);
        if (rc != 0) return finish(rc, err);
        for (size_t i = 0; i < s.size(); ++i) {
            stats[i].steps = s[i].steps;
            stats[i].events = s[i].events;
            stats[i].n_aggregates = s[i].n_alive;
            stats[i].time = s[i].time;
            stats[i].finished = s[i].finished;
            stats[i].reserved = s[i].status;
        }
        return 0;
    });
}

int mcacg_batch_size(const mcacg_batch *batch, int32_t *n_boxes) {
    return guarded([&] {
        if (!batch || !n_boxes) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        *n_boxes = batch->impl->size();
        return 0;
    });
}

int mcacg_batch_box_sizes(mcacg_batch *batch, int32_t box, int64_t *n_spheres, int64_t *n_aggregates) {
    return guarded([&] {
        if (!batch || box < 0 || box >= batch->impl->size()) return fail(MCACG_ERR_BAD_ARGUMENT, "bad box");
        std::string err;
        int alive = 0;
        int rc = batch->impl->box(box).n_alive(&alive, &err);
        if (rc != 0) return finish(rc, err);
        if (n_spheres) *n_spheres = batch->impl->box(box).ns();
        if (n_aggregates) *n_aggregates = alive;
        return 0;
    });
}

int mcacg_batch_store_state(mcacg_batch *batch, int32_t box, mcacg_state *state) {
    return guarded([&] {
        if (!batch || !state || box < 0 || box >= batch->impl->size())
            return fail(MCACG_ERR_BAD_ARGUMENT, "bad argument");
        std::string err;
        if (!batch->impl->refresh_overlap(box)) {
            std::vector<double> times;
            int rc = batch->impl->times(&times, &err);
            if (rc == 0) rc = batch->impl->box(box).store(state, &err);
            if (rc == 0) state->time = times[size_t(box)];
            if (rc == 0) drop_removed_spheres(state);
            return finish(rc, err);
        }
        mcacg::HostState st;
        int rc = batch->impl->download(box, &st, &err);
        if (rc != 0) return finish(rc, err);
        const int rc2 = store_host_state(st, state, &err);
        if (rc2 == 0) drop_removed_spheres(state);
        return finish(rc2, err);
    });
}

int mcacg_batch_store_states(mcacg_batch *batch, mcacg_state *states, int32_t n_boxes) {
    return guarded([&] {
        if (!batch || !states || n_boxes != batch->impl->size()) return fail(MCACG_ERR_BAD_ARGUMENT, "bad argument");
        std::vector<double> times;
        std::string err;
        int rc = batch->impl->times(&times, &err);
        if (rc != 0) return finish(rc, err);
        // boxes whose device fields are current (all but growth with volsurf
        // "none"): packed on the device and copied straight into the
        // caller's arrays, all boxes at once
        std::vector<int> direct, grown;
        for (int i = 0; i < n_boxes; ++i) (batch->impl->refresh_overlap(i) ? grown : direct).push_back(i);
        std::vector<mcacg::DeviceBox *> boxes;
        std::vector<mcacg_state *> outs;
        for (int i : direct) {
            boxes.push_back(&batch->impl->box(i));
            outs.push_back(&states[i]);
        }
        std::vector<int> rcs;
        std::vector<std::string> errs;
        rc = mcacg::DeviceBox::store_many(boxes, outs, batch->impl->stream(), &rcs, &errs, &err);
        if (rc != 0) return finish(rc, err);
        for (size_t k = 0; k < direct.size(); ++k) {
            if (rcs[k] != 0) return fail(rcs[k], "box " + std::to_string(direct[k]) + ": " + errs[k]);
            states[direct[k]].time = times[size_t(direct[k])];
            drop_removed_spheres(&states[direct[k]]);
        }
        // growing boxes with volsurf "none": overlap and coordination
        // refreshed on the host, one copy stream per worker thread
        struct CopyStream {
            cudaStream_t s = nullptr;
            ~CopyStream() {
                if (s) cudaStreamDestroy(s);
            }
        };
        rcs.assign(grown.size(), 0);
        errs.assign(grown.size(), std::string());
        mcacg::parallel_for(int(grown.size()), [&](int k) {
            thread_local CopyStream cs;
            if (!cs.s) cudaStreamCreateWithFlags(&cs.s, cudaStreamNonBlocking);
            const int i = grown[size_t(k)];
            mcacg::HostState st;
            rcs[size_t(k)] = batch->impl->box(i).download(&st, &errs[size_t(k)], cs.s);
            if (rcs[size_t(k)] != 0) return;
            mcacg::host_refresh_overlap(&st);
            st.time = times[size_t(i)];
            rcs[size_t(k)] = store_host_state(st, &states[i], &errs[size_t(k)]);
            if (rcs[size_t(k)] == 0) drop_removed_spheres(&states[i]);
        });
        for (size_t k = 0; k < grown.size(); ++k)
            if (rcs[k] != 0) return fail(rcs[k], "box " + std::to_string(grown[k]) + ": " + errs[k]);
        return 0;
    });
}

int mcacg_set_merge_grid_min(int32_t n_spheres, int32_t *previous) {
    return guarded([&] {
        if (n_spheres < 1) return fail(MCACG_ERR_BAD_ARGUMENT, "n_spheres must be positive");
        int old = mcacg::set_merge_grid_min(n_spheres);
        if (previous) *previous = old;
        return 0;
    });
}

int mcacg_set_live_list_max(int32_t n_aggregates, int32_t *previous) {
    return guarded([&] {
        if (n_aggregates < 0 || n_aggregates > 128) return fail(MCACG_ERR_BAD_ARGUMENT, "n_aggregates must be 0..128");
        int old = mcacg::set_live_list_max(n_aggregates);
        if (previous) *previous = old;
        return 0;
    });
}

int mcacg_host_alloc(int64_t bytes, void **ptr) {
    return guarded([&] {
        if (!ptr || bytes <= 0) return fail(MCACG_ERR_BAD_ARGUMENT, "bad argument");
        *ptr = nullptr;
        cudaError_t e = cudaHostAlloc(ptr, size_t(bytes), cudaHostAllocPortable);
        if (e != cudaSuccess) {
            *ptr = nullptr;
            return fail(mcacg::ST_CUDA, std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
        }
        return 0;
    });
}

int mcacg_host_free(void *ptr) {
    return guarded([&] {
        if (ptr) cudaFreeHost(ptr);
        return 0;
    });
}

int mcacg_resident_boxes(int32_t threads, int32_t *boxes) {
    return guarded([&] {
        if (!boxes) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        int n = 0;
        std::string err;
        int rc = mcacg::BatchRunner::resident_boxes(threads, &n, &err);
        if (rc != 0) return finish(rc, err);
        *boxes = n;
        return 0;
    });
}

int mcacg_batch_set_threads(mcacg_batch *batch, int32_t threads) {
    return guarded([&] {
        if (!batch) return fail(MCACG_ERR_BAD_ARGUMENT, "null batch");
        if (batch->impl->set_threads(threads) != 0)
            return fail(MCACG_ERR_BAD_ARGUMENT, "threads per box must be 0, 32, 64, 128, 256 or 512");
        return 0;
    });
}

int mcacg_batch_set_aggregate_limit(mcacg_batch *batch, int64_t limit) {
    return guarded([&] {
        if (!batch) return fail(MCACG_ERR_BAD_ARGUMENT, "null batch");
        std::string err;
        const int rc = batch->impl->set_aggregate_limit(limit, &err);
        if (rc != 0) return fail(rc, err);
        return 0;
    });
}

int mcacg_batch_pick_histogram(mcacg_batch *batch, int32_t box, int64_t n_picks, uint32_t seed, int64_t *counts,
                               int64_t capacity, int64_t *n_labels, int64_t *picks_done) {
    return guarded([&] {
        if (!batch || !counts || !n_labels || !picks_done) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        std::vector<int64_t> by_label;
        std::string err;
        int64_t done = 0;
        const int rc = batch->impl->pick_histogram(box, n_picks, seed, &by_label, &done, &err);
        if (rc != 0) return finish(rc, err);
        if (int64_t(by_label.size()) > capacity) return fail(MCACG_ERR_BAD_ARGUMENT, "counts array too small");
        std::copy(by_label.begin(), by_label.end(), counts);
        *n_labels = int64_t(by_label.size());
        *picks_done = done;
        return 0;
    });
}

int mcacg_draw_directions(int64_t n, uint32_t seed, double *out) {
    return guarded([&] {
        if (n < 0 || (n > 0 && !out)) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument or negative count");
        int count = 0;
        if (cudaGetDeviceCount(&count) != cudaSuccess || count < 1) {
            cudaGetLastError();
            return fail(MCACG_ERR_NO_DEVICE, "no CUDA device");
        }
        std::string err;
        return finish(mcacg::BatchRunner::draw_directions(n, seed, out, &err), err);
    });
}

int mcacg_batch_set_speculation(mcacg_batch *batch, int32_t ctas_per_box) {
    return guarded([&] {
        if (!batch) return fail(MCACG_ERR_BAD_ARGUMENT, "null batch");
        if (batch->impl->set_speculation(ctas_per_box) != 0)
            return fail(MCACG_ERR_BAD_ARGUMENT, "CTAs per box must be 0, 1, 2, 4 or 8");
        return 0;
    });
}

int mcacg_batch_speculation(const mcacg_batch *batch, int32_t *ctas_per_box) {
    return guarded([&] {
        if (!batch || !ctas_per_box) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        *ctas_per_box = batch->impl->speculation();
        return 0;
    });
}

int mcacg_batch_threads(const mcacg_batch *batch, int32_t *threads) {
    return guarded([&] {
        if (!batch || !threads) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        *threads = batch->impl->threads();
        return 0;
    });
}

namespace {
void add_work(const mcacg::BoxRunStats &x, mcacg_profile *out) {
    out->queries += x.queries;
    out->merges += x.events;
    out->translates += x.steps;
    out->mov_spheres += x.mov;
    out->scanned += x.scanned;
    out->cells += x.cells;
    out->candidates += x.candidates;
    out->cand_spheres += x.cand_spheres;
    out->refined += x.refined;
    out->merged_spheres += x.merged_spheres;
    out->merge_pairs += x.merge_pairs;
    out->cycles_pick += x.cyc_pick;
    out->cycles_query += x.cyc_query;
    out->cycles_move += x.cyc_move;
    out->cycles_merge += x.cyc_merge;
    out->cycles_query_scan += x.cyc_qscan;
    out->cycles_query_pairs += x.cyc_qpairs;
}
}  // namespace

int mcacg_batch_work(mcacg_batch *batch, mcacg_profile *out) {
    return guarded([&] {
        if (!batch || !out) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        std::vector<mcacg::BoxRunStats> s;
        std::string err;
        int rc = batch->impl->stats(&s, &err);
        if (rc != 0) return finish(rc, err);
        *out = mcacg_profile{};
        for (const auto &x : s) add_work(x, out);
        return 0;
    });
}

int mcacg_batch_box_work(mcacg_batch *batch, int32_t box, mcacg_profile *out) {
    return guarded([&] {
        if (!batch || !out || box < 0 || box >= batch->impl->size()) return fail(MCACG_ERR_BAD_ARGUMENT, "bad argument");
        std::vector<mcacg::BoxRunStats> s;
        std::string err;
        int rc = batch->impl->stats(&s, &err);
        if (rc != 0) return finish(rc, err);
        *out = mcacg_profile{};
        add_work(s[size_t(box)], out);
        return 0;
    });
}

int mcacg_server_create(int32_t capacity, int64_t memory_budget_bytes, void *cuda_stream, int32_t keep_final_states,
                        mcacg_server **server) {
    return guarded([&] {
        if (!server) return fail(MCACG_ERR_BAD_ARGUMENT, "null server");
        *server = nullptr;
        std::unique_ptr<mcacg_server> s(new mcacg_server());
        std::string err;
        int rc = mcacg::Server::create(capacity, memory_budget_bytes, cuda_stream, keep_final_states != 0, &s->impl,
                                       &err);
        if (rc != 0) return finish(rc, err);
        *server = s.release();
        return 0;
    });
}

int mcacg_server_destroy(mcacg_server *server) {
    return guarded([&] {
        delete server;
        return 0;
    });
}

int mcacg_server_set_epoch_ms(mcacg_server *server, double ms) {
    return guarded([&] {
        if (!server || !(ms >= 0.0)) return fail(MCACG_ERR_BAD_ARGUMENT, "bad argument");
        server->impl->set_epoch_ms(ms);
        return 0;
    });
}

int mcacg_server_set_threads(mcacg_server *server, int32_t threads) {
    return guarded([&] {
        if (!server) return fail(MCACG_ERR_BAD_ARGUMENT, "null server");
        if (server->impl->set_threads(threads) != 0)
            return fail(MCACG_ERR_BAD_ARGUMENT, "threads per box must be 0, 32, 64, 128, 256 or 512");
        return 0;
    });
}

int mcacg_server_submit(mcacg_server *server, const mcacg_params *params, int64_t *id) {
    return guarded([&] {
        if (!server || !params || !id) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        std::string err;
        return finish(server->impl->submit(*params, id, &err), err);
    });
}

int mcacg_server_step(mcacg_server *server, int64_t epoch_steps, int32_t *n_active, int32_t *n_pending) {
    return guarded([&] {
        if (!server) return fail(MCACG_ERR_BAD_ARGUMENT, "null server");
        std::string err;
        int rc = server->impl->step(epoch_steps, &err);
        if (n_active) *n_active = server->impl->n_active();
        if (n_pending) *n_pending = server->impl->n_pending();
        return finish(rc, err);
    });
}

int mcacg_server_poll(mcacg_server *server, mcacg_completion *out, int32_t capacity, int32_t *n_out) {
    return guarded([&] {
        if (!server || !n_out || (capacity > 0 && !out)) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        for (auto &c : server->impl->poll()) server->unread.push_back(c);
        int32_t n = std::min<int32_t>(capacity, int32_t(server->unread.size()));
        for (int32_t i = 0; i < n; ++i) {
            const auto &c = server->unread[size_t(i)];
            out[i] = mcacg_completion{c.id, c.steps, c.events, c.n_alive, c.time, c.status, c.finished,
                                      c.submit_s, c.admit_s, c.finish_s};
        }
        server->unread.erase(server->unread.begin(), server->unread.begin() + n);
        *n_out = n;
        return 0;
    });
}

int mcacg_server_final_sizes(mcacg_server *server, int64_t id, int64_t *n_spheres, int64_t *n_aggregates) {
    return guarded([&] {
        if (!server) return fail(MCACG_ERR_BAD_ARGUMENT, "null server");
        mcacg::HostState st;
        if (server->impl->final_state(id, &st) != 0) return fail(MCACG_ERR_BAD_ARGUMENT, "no final state for id");
        int na = 0;
        for (int n : st.agg_n) na += n > 0;
        if (n_spheres) *n_spheres = st.ns;
        if (n_aggregates) *n_aggregates = na;
        return 0;
    });
}

int mcacg_server_final_state(mcacg_server *server, int64_t id, mcacg_state *state) {
    return guarded([&] {
        if (!server || !state) return fail(MCACG_ERR_BAD_ARGUMENT, "null argument");
        mcacg::HostState st;
        if (server->impl->final_state(id, &st) != 0) return fail(MCACG_ERR_BAD_ARGUMENT, "no final state for id");
        std::string err;
        const int rc2 = store_host_state(st, state, &err);
        if (rc2 == 0) drop_removed_spheres(state);
        return finish(rc2, err);
    });
}

int mcacg_server_kernel_time(const mcacg_server *server, double *kernel_ms, int32_t *launches) {
    return guarded([&] {
        if (!server) return fail(MCACG_ERR_BAD_ARGUMENT, "null server");
        if (kernel_ms) *kernel_ms = server->impl->kernel_ms();
        if (launches) *launches = server->impl->launches();
        return 0;
    });
}

int mcacg_batch_last_run(const mcacg_batch *batch, double *kernel_ms, int32_t *launches) {
    return guarded([&] {
        if (!batch) return fail(MCACG_ERR_BAD_ARGUMENT, "null batch");
        if (kernel_ms) *kernel_ms = batch->impl->last_kernel_ms();
        if (launches) *launches = batch->impl->launches();
        return 0;
    });
}

}  // extern "C"
