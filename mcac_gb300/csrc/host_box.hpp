// Host side of one box: the AggregatList interface of the reference
// (include/aggregats/aggregat_list.hpp:29-116) over a device-resident state.
//
// The host keeps a mirror of the 21 aggregate fields (small) and the label
// order; the spheres, member lists and Verlet grid live on the GPU. Every
// per-step operation of src/calcul.cpp maps to one method here.
#pragma once
#include <ctime>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "../../include/mcacg.h"
#include "device_box.hpp"

namespace mcacg {

class BatchRunner;

class HostBox {
  public:
    // AggregatList::AggregatList: seeded random placement (host), then upload.
    static int create_random(const mcacg_params &p, void *stream, std::unique_ptr<HostBox> *out, std::string *err);
    // From a complete state (labels in order, all aggregates alive).
    static int create_from_state(const mcacg_params &p, const mcacg_state &st, void *stream,
                                 std::unique_ptr<HostBox> *out, std::string *err);

    int size() const { return int(alive_.size()); }
    int n_spheres() const { return ns_; }
    double time() const { return time_; }
    void set_time(double t);
    const mcacg_params &params() const { return p_; }
    DeviceBox &device() { return *dev_; }

    // per-step interface
    int distance_to_next_contact(int64_t label, const double dir[3], double distance, mcacg_contact *out,
                                 std::string *err);
    // n independent queries on the current state, run concurrently on the
    // device; *kernel_ms (may be null) gets the kernel time.
    int distance_to_next_contacts(int n, const int64_t *labels, const double *dirs, const double *distances,
                                  mcacg_contact *out, double *kernel_ms, std::string *err);
    int translate(int64_t label, const double v[3], std::string *err);
    int time_forward(int64_t label, double dt, std::string *err);
    int merge(const mcacg_contact &c, int32_t *merged, std::string *err);
    void sort_time_steps(double factor);
    int64_t pick_random();
    double get_time_step(double max) const { return max / cumulative_[alive_.size() - 1]; }
    double max_time_step() const { return max_time_step_; }
    double avg_npp() const { return avg_npp_; }
    void refresh();
    double total_volume() const;
    double total_surface() const;
    const double *fields(int64_t label, double out[21]) const;
    int n_spheres_of(int64_t label) const { return agg_n_[size_t(alive_[size_t(label)])]; }
    int slot_of(int64_t label) const { return alive_[size_t(label)]; }
    int64_t label_of(int slot) const;

    // the reference's stop criteria (physical_model.cpp:288-337, without the
    // STOPCODE file: this library writes no output directory)
    bool finished() const;
    // one run of the MC loop of src/calcul.cpp:66-281 (collisions, with
    // surface growth when the parameters ask for it)
    int calcul(const mcacg_run_opts &opts, mcacg_run_stats *stats, std::string *err);

    // whole state (store) in label order
    int store(mcacg_state *st, std::string *err);

    // the device-resident loop on this machine (see BatchRunner)
    int run_device(int64_t max_steps, mcacg_run_stats *stats, std::string *err);

  private:
    int update_aggregates(int slot, bool full, std::string *err);
    int oxidize(int64_t label, mcacg_contact *c, bool *split, bool *disappear, std::string *err);
    int replace_state(const HostState &st, std::string *err);
    int64_t label_of_uid(int64_t uid) const;
    void invalidate_device_run();
    int refresh_from_device(std::string *err);
    std::unique_ptr<BatchRunner> runner_;
    int64_t runner_steps_ = 0, runner_events_ = 0;
    HostBox();
  public:
    ~HostBox();

  private:
    int upload(const HostState &st, void *stream, std::string *err);
    double &F(int field, int slot) { return agg_[size_t(field) * size_t(nslots_) + size_t(slot)]; }
    double F(int field, int slot) const { return agg_[size_t(field) * size_t(nslots_) + size_t(slot)]; }

    mcacg_params p_{};
    double time_ = 0;
    int64_t n_iter_without_event_ = 0;
    bool event_ = true;
    int ns_ = 0, nslots_ = 0;
    std::vector<double> agg_;   // [21][nslots] mirror
    std::vector<int> agg_n_;    // members per slot (0: dead)
    std::vector<int> alive_;    // slot of each label
    std::vector<int64_t> uid_;  // identity of each label's aggregate (the reference's weak pointers)
    // processor time at the box's creation and at the last event, for the
    // cpu and cpu_event limits (PhysicalModel::cpu_start, cpu_last_event)
    std::clock_t cpu_start_ = 0, cpu_last_event_ = 0;
    int64_t next_uid_ = 0;
    double maxradius_ = 0;
    double max_time_step_ = 0, avg_npp_ = 1;
    std::vector<size_t> index_sorted_;
    std::vector<double> cumulative_;
    std::vector<double> weights_;      // weights in sorted order
    std::vector<double> tp_by_label_;  // weights by label at the last sort
    std::vector<size_t> index_ref_;    // the reference's std::sort order, on demand
    bool ties_ = false, ref_order_valid_ = false;
    void reference_sort_order();
    // live slots ordered by decreasing time step (kept across merges)
    std::vector<std::pair<double, int>> by_dt_;
    bool dt_order_valid_ = false;
    std::vector<int> slot_label_;
    void build_dt_order();
    void dt_order_erase(int slot, double dt);
    void dt_order_insert(int slot, double dt);
    std::unique_ptr<DeviceBox> dev_;
    // The PhysicalModel values that the reference's advancement.dat lines
    // print (physical_model.cpp:266-267, 489-498) and its write bookkeeping
    // (physical_model.cpp:338-356, calcul.cpp:60-68).
    int64_t total_events_ = 0;
    uint64_t last_timestep_written_ = 0;
    double aggregate_concentration_ = 0, monomer_concentration_ = 0, volume_fraction_ = 0;
    bool advancement_closed_ = false;  // the final line is written
    void init_model_values();
    bool time_to_write();
    void save_advancement(const char *path) const;
};

// Random placement of the reference's AggregatList constructor into 'st'
// (aggregat.cpp:162-229, aggregat_list_storage.cpp:52-88). Seeds the C
// library generator. Uses a fine spatial hash for the free-space test; the
// answer of that test does not depend on the grid, so the placements are the
// reference's.
int init_random_state(const mcacg_params &p, HostState *st, std::string *err);
// The same placement drawing from a private copy of the C library stream
// seeded with p.random_seed: identical result, safe to run on many threads.
int init_random_state_private(const mcacg_params &p, HostState *st, std::string *err);

// A C-ABI state (labels in order) as a slot-ordered host state, validated.
int state_to_host(const mcacg_state &in, HostState *out, std::string *err);

// Aggregate::update for an aggregate given by its members (host, used for
// initial monomers and for loading states): writes all 21 fields except the
// position-independent proper time and charge, and raises 'maxradius'.
int host_update_aggregate(const mcacg_params &p, const HostState &st, MemberLists::View members, double fields[21],
                          double *maxradius);

// The overlap and coordination fields of every live aggregate from its
// spheres (update_distances_and_overlapping, aggregat.cpp:719-764): the
// device loop with surface growth leaves them to the read-back.
void host_refresh_overlap(HostState *st);

// A seeded synthetic snapshot for the contact-search benchmark:
// p.n_monomeres spheres (diameters drawn like initialisation_mode=lognormal)
// in n_aggregates aggregates of 1..max_size spheres grown by ballistic
// sticking, placed without overlap in a periodic cube whose length makes the
// sphere volume fraction p.volume_fraction. Deterministic for a given
// p.random_seed (workloads.cpp).
int make_synthetic_state(const mcacg_params &p, int n_aggregates, int max_size, HostState *st, std::string *err);

}  // namespace mcacg
