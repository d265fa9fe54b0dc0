// Host side of the device-resident MC loop: many boxes advanced by one
// persistent kernel launch, one thread block per box.
#pragma once
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "../../include/mcacg.h"
#include "device_box.hpp"

namespace mcacg {

struct BoxRunStats {
    int64_t steps, events, n_alive;
    double time;
    int finished, status;
    // work counters since creation
    int64_t queries, mov, scanned, cells, candidates, cand_spheres, refined, merged_spheres, merge_pairs;
};

class BatchRunner {
  public:
    // One box per state; params[i] gives box i's physics, stop criteria and
    // seed (its device rand() stream is seeded with params[i].random_seed).
    static int create(const std::vector<mcacg_params> &params, std::vector<HostState> &&states, void *stream,
                      std::unique_ptr<BatchRunner> *out, std::string *err);
    // Runs existing device boxes (owned elsewhere) with the device loop.
    static int attach(const std::vector<mcacg_params> &params, const std::vector<DeviceBox *> &boxes,
                      const std::vector<double> &times, void *stream, std::unique_ptr<BatchRunner> *out,
                      std::string *err);
    ~BatchRunner();

    int size() const { return int(boxes_.size()); }
    // Advances every unfinished box by at most max_steps MC steps (<= 0: until
    // every box meets its stop criterion) in launches of 'chunk' steps.
    int run(int64_t max_steps, int64_t chunk, std::string *err);
    int stats(std::vector<BoxRunStats> *out, std::string *err);
    int download(int box, HostState *st, std::string *err);
    DeviceBox &box(int i) { return *boxes_[size_t(i)]; }
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
    std::vector<void *> trees_;
    double last_ms_ = 0;
    int launches_ = 0;
};

}  // namespace mcacg
