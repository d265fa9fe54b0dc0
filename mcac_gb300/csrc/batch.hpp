// Host side of the device-resident MC loop: many boxes advanced by one
// persistent kernel launch, one thread block per box.
#pragma once
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/mcacg.h"
#include "device_box.hpp"

namespace mcacg {

// Process-wide: the device loop keeps a list of the live slots in shared
// memory once at most this many aggregates are left (0: never; at most 128),
// read by boxes set up afterwards. Results do not depend on it.
int live_list_max();
int set_live_list_max(int n);  // returns the previous value

struct BoxRunStats {
    int64_t steps, events, n_alive;
    double time;
    int finished, status;
    // work counters since creation
    int64_t queries, mov, scanned, cells, candidates, cand_spheres, refined, merged_spheres, merge_pairs;
    int64_t cyc_pick, cyc_query, cyc_move, cyc_merge;  // SM cycles per phase of the step
    int64_t cyc_qscan, cyc_qpairs;                     // parts of cyc_query
};

class BatchRunner {
  public:
    // One box per state; params[i] gives box i's physics, stop criteria and
    // seed (its device rand() stream is seeded with params[i].random_seed).
    static int create(const std::vector<mcacg_params> &params, std::vector<HostState> &&states, void *stream,
                      std::unique_ptr<BatchRunner> *out, std::string *err);
    // The same from states in host memory that the caller keeps (page-locked
    // arrays are copied by DMA, without a host-side copy).
    static int create(const std::vector<mcacg_params> &params, const std::vector<StateView> &states, void *stream,
                      std::unique_ptr<BatchRunner> *out, std::string *err);
    // Runs existing device boxes (owned elsewhere) with the device loop.
    static int attach(const std::vector<mcacg_params> &params, const std::vector<DeviceBox *> &boxes,
                      const std::vector<double> &times, void *stream, std::unique_ptr<BatchRunner> *out,
                      std::string *err);
    ~BatchRunner();
    // Boxes the device loop keeps resident at once on the current device
    // (thread blocks per SM at its register and shared-memory use x SMs).
    static int resident_boxes(int threads, int *boxes, std::string *err);
    // Threads per box (32, 64, 128, 256 or 512; 0: the largest at which all
    // unfinished boxes are resident, chosen at the next run and again when
    // half of the running boxes have finished).
    int set_threads(int threads);
    int threads() const { return threads_; }
    // CTAs per box of the loop's speculative rounds (spec.cuh): 1 (none, the
    // default; 0 means the same), 2, 4 or 8. Results do not depend on it.
    int set_speculation(int k);
    int speculation() const { return spec_max_ > 0 && spec_max_ < spec_k_ ? spec_max_ : spec_k_; }

    int size() const { return int(boxes_.size()); }
    // Advances every unfinished box by at most max_steps MC steps (<= 0: until
    // every box meets its stop criterion) in launches of 'chunk' steps.
    int run(int64_t max_steps, int64_t chunk, std::string *err);
    // Runs every unfinished box for about wall_ms milliseconds of wall time
    // (launches of at most 200 ms in which each box does as many steps as
    // fit), returning early when all have met their stop criteria.
    int run_timed(double wall_ms, std::string *err);
    int stats(std::vector<BoxRunStats> *out, std::string *err);
    // Replaces every box's number_of_aggregates stop criterion; boxes that
    // stopped without an error are re-armed and re-check all their criteria
    // before their next step.
    int set_aggregate_limit(int64_t limit, std::string *err);
    // Diagnostics of the loop's random draws. pick_histogram: at least n_picks
    // picks of box 'box''s current pick tree (nothing moves; 256 warps with
    // rand() streams seeded seed, seed + 1, ...), counted per label;
    // *picks_done gets the picks made. draw_directions: n directions of the
    // loop's direction draw (thread t's stream seeded seed + t) into host
    // memory, 3 doubles each.
    int pick_histogram(int box, int64_t n_picks, uint32_t seed, std::vector<int64_t> *by_label,
                       int64_t *picks_done, std::string *err);
    static int draw_directions(int64_t n, uint32_t seed, double *out, std::string *err);
    int download(int box, HostState *st, std::string *err);
    // Physical time of every box.
    int times(std::vector<double> *out, std::string *err);
    // Box i grows by surface reactions (its overlap fields are refreshed on read-back).
    bool grows(int i) const { return growth_.size() > size_t(i) && growth_[size_t(i)]; }
    // Box i's overlap and coordination fields are stale on the device (growth
    // with volsurf "none") and are recomputed on read-back.
    bool refresh_overlap(int i) const {
        return grows(i) && volsurf_.size() > size_t(i) && volsurf_[size_t(i)] == MCACG_VOLSURF_NONE;
    }
    DeviceBox &box(int i) { return *boxes_[size_t(i)]; }
    void *stream() const { return stream_; }
    // Kernel time of the last run() (CUDA events on the stream).
    double last_kernel_ms() const { return last_ms_; }
    int launches() const { return launches_; }

  private:
    BatchRunner() = default;
    int init_stream(void *stream, std::string *err);
    int init(const std::vector<mcacg_params> &params, const std::vector<double> &times, std::string *err);
    std::vector<std::unique_ptr<DeviceBox>> owned_;
    std::vector<DeviceBox *> boxes_;
    void *stream_ = nullptr;
    bool own_stream_ = false;
    void *runs_dev_ = nullptr;    // BoxRun[n]
    void *states_dev_ = nullptr;  // RunState[n]
    void *sc_dev_ = nullptr;      // DevScalars[n], gathered by stats()
    std::vector<void *> trees_;
    double last_ms_ = 0;
    int launches_ = 0;
    int threads_ = 0;
    bool auto_threads_ = true;
    std::vector<char> growth_;  // per box: surface reactions on
    std::vector<int> volsurf_;  // per box: VolSurfMethods
    int tuned_active_ = 0;  // unfinished boxes at the last tuning
    int tune(int64_t budget, int64_t *done, float *ms_total, std::string *err, bool one_wave);
    int spec_room(std::string *err);
    cudaError_t launch_run(int nt, int k, long long steps, long long budget_ns);
    int spec_k_ = 1;          // CTAs per box in use
    int spec_max_ = 0;        // CTAs per box the helper scratch allows (0: not set up yet)
    void *spec_mem_ = nullptr;  // helper query scratch
    void *spec_tab_ = nullptr;  // SpecScratch[n * (kSpecMax - 1)]
    void *order_dev_ = nullptr; // int[n]: the box of each block of a launch, largest first
};

// Continuous-batching request loop: 'capacity' block slots; between kernel
// epochs finished boxes leave and pending requests are admitted while a free
// slot and the device-memory budget allow. A box's trajectory depends only on
// its own state and rand() stream, so it is the same alone and in any mix.
struct Completion {
    int64_t id;
    int64_t steps, events, n_alive;
    double time;
    int status, finished;
    double submit_s, admit_s, finish_s;  // host clock, seconds since the server started
};

class Server {
  public:
    static int create(int capacity, int64_t memory_budget, void *stream, bool keep_final_states,
                      std::unique_ptr<Server> *out, std::string *err);
    ~Server();
    int submit(const mcacg_params &p, int64_t *id, std::string *err);
    // admit, one kernel epoch of at most 'epoch_steps' steps per box, retire
    int step(int64_t epoch_steps, std::string *err);
    // Threads per box of the epochs (32, 64, 128, 256 or 512; default 256;
    // 0: at each epoch the largest size at which every active box is
    // resident at once).
    int set_threads(int threads);
    int last_threads() const { return last_threads_; }
    // Wall-time cap of an epoch in milliseconds (0: epochs end by steps only).
    void set_epoch_ms(double ms) { epoch_budget_ns_ = ms > 0 ? (long long)(ms * 1e6) : 0; }
    int n_active() const;
    int n_pending() const { return int(pending_.size()); }
    std::vector<Completion> poll();
    int final_state(int64_t id, HostState *st) const;
    double kernel_ms() const { return kernel_ms_; }
    int launches() const { return launches_; }
    int64_t memory_in_use() const { return mem_in_use_; }

  private:
    Server() = default;
    static int64_t footprint(const mcacg_params &p);
    double now() const;
    struct Request {
        int64_t id;
        mcacg_params p;
        double submit_s;
    };
    struct Slot {
        std::unique_ptr<DeviceBox> box;
        void *tree = nullptr;
        int64_t id = -1;
        int64_t bytes = 0;
        double submit_s = 0, admit_s = 0;
        bool growth = false;
        int volsurf = MCACG_VOLSURF_NONE;
    };
    int admit(std::string *err);
    int retire(std::string *err);
    int capacity_ = 0;
    int threads_ = 256;
    int last_threads_ = 0;           // threads per box of the last epoch
    long long epoch_budget_ns_ = 0;  // wall-time cap of an epoch (0: steps only)
    int64_t budget_ = 0, mem_in_use_ = 0, next_id_ = 0;
    bool keep_ = false;
    void *stream_ = nullptr;
    bool own_stream_ = false;
    void *runs_dev_ = nullptr, *states_dev_ = nullptr;
    std::vector<Slot> slots_;
    std::vector<Request> pending_;
    std::vector<Completion> done_;
    std::vector<std::pair<int64_t, HostState>> finals_;
    double t0_ = 0, kernel_ms_ = 0;
    int launches_ = 0;
};

}  // namespace mcacg
