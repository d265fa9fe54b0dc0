// Persistent device loop over many boxes; see batch.hpp and run.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <thread>
#include <type_traits>

#include "batch.hpp"
#include "host_parallel.hpp"
#include "host_box.hpp"
#include "run.cuh"
#include "spec.cuh"

namespace mcacg {

constexpr int kRunThreads = 256;  // serving loop
// Block sizes of the batched loop. Most of an MC step is a chain of
// dependent loads and block barriers, so smaller blocks (more boxes per SM)
// often finish more steps per second; BatchRunner::run picks one by timing.
// Every variant keeps to 128 registers a thread (512 / NT blocks per SM).
// (Holding one warp per box to fewer registers, for 20 boxes per SM, spilled
// and ran slower.)
// Large blocks pay off late in a run, when few boxes are left and each holds
// big aggregates (long pair searches and merges).
constexpr int kRunThreadChoices[] = {32, 64, 128, 256, 512};

// One warp per box uses the small shared-memory plan, so that 16 boxes fit
// an SM (shared memory being the limit there, not registers).
template <int NT>
using RunSmemFor = typename std::conditional<(NT <= 32), RunSmemSmall, RunSmem>::type;
// wall time of one launch when boxes run to their stop criteria
constexpr long long kRunLaunchBudgetNs = 200LL * 1000 * 1000;


// Each block advances its box by at most max_steps steps; with budget_ns > 0
// it also stops after that much wall time, so that boxes of very different
// cost do not wait for one another between launches.
template <int NT>
__global__ void __launch_bounds__(NT, 512 / NT) k_run(const BoxRun *runs, int n, long long max_steps,
                                                      long long budget_ns, const int *order) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    RunSmemFor<NT> &sm = *reinterpret_cast<RunSmemFor<NT> *>(smem_raw);
    __shared__ __align__(16) BoxRun R;
    __shared__ __align__(16) RunState st;  // the box's loop state, kept on chip for the launch
    if (int(blockIdx.x) >= n) return;
    const int box = order != nullptr ? order[blockIdx.x] : int(blockIdx.x);
    RunState *st_global = runs[box].st;
    if (st_global == nullptr) return;  // an empty serving slot
    {
        const int words = int(sizeof(BoxRun) / sizeof(int));
        const int *src = reinterpret_cast<const int *>(&runs[box]);
        int *dst = reinterpret_cast<int *>(&R);
        for (int k = threadIdx.x; k < words; k += NT) dst[k] = src[k];
        const int swords = int(sizeof(RunState) / sizeof(int));
        const int *ssrc = reinterpret_cast<const int *>(st_global);
        int *sdst = reinterpret_cast<int *>(&st);
        for (int k = threadIdx.x; k < swords; k += NT) sdst[k] = ssrc[k];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        R.st = &st;
        // every step starts only before the deadline (a step is never cut)
        sm.deadline = budget_ns > 0 ? global_ns() + (unsigned long long)budget_ns : 0ULL;
    }
    if (threadIdx.x == 0) {
        sm.live.allow = decltype(sm.live)::kCap > 1 ? 1 : 0;
        sm.live.max = R.live_max;
        sm.live.on = 0;
    }
    __syncthreads();
    tree_cache_load(R, sm.tree);
    live_load(R, sm.live, sm.u.q.warp_tmp);
    for (long long s = 0; s < max_steps; ++s)
        if (!block_mc_step(R, sm)) break;
    __syncthreads();
    {
        const int swords = int(sizeof(RunState) / sizeof(int));
        const int *ssrc = reinterpret_cast<const int *>(&st);
        int *sdst = reinterpret_cast<int *>(st_global);
        for (int k = threadIdx.x; k < swords; k += NT) sdst[k] = ssrc[k];
    }
}

// The same loop with speculative rounds (spec.cuh): a cluster of K CTAs per
// box (grid n * K, clusters of K consecutive blocks), K steps per round,
// committed in order by the leader CTA (rank 0). helpers[box * (kSpecMax -
// 1) + rank - 1] is the query scratch of helper rank 'rank'.
template <int NT>
__global__ void __launch_bounds__(NT, 512 / NT) k_run_spec(const BoxRun *runs, const SpecScratch *helpers, int n,
                                                           long long max_steps, long long budget_ns,
                                                           const int *order) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const int K = int(cluster.num_blocks());
    const int rank = int(cluster.block_rank());
    const int box = order != nullptr ? order[int(blockIdx.x) / K] : int(blockIdx.x) / K;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    RunSmemFor<NT> &sm = *reinterpret_cast<RunSmemFor<NT> *>(smem_raw);
    __shared__ __align__(16) BoxRun R;
    __shared__ __align__(16) RunState st;
    __shared__ __align__(16) SpecShared sh;
    // the same for every CTA of a cluster (one box per cluster)
    if (box >= n || runs[box].st == nullptr) return;
    RunState *st_global = runs[box].st;
    {
        const int words = int(sizeof(BoxRun) / sizeof(int));
        const int *src = reinterpret_cast<const int *>(&runs[box]);
        int *dst = reinterpret_cast<int *>(&R);
        for (int k = threadIdx.x; k < words; k += NT) dst[k] = src[k];
        if (rank == 0) {
            const int swords = int(sizeof(RunState) / sizeof(int));
            const int *ssrc = reinterpret_cast<const int *>(st_global);
            int *sdst = reinterpret_cast<int *>(&st);
            for (int k = threadIdx.x; k < swords; k += NT) sdst[k] = ssrc[k];
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (rank == 0) {
            R.st = &st;
            sm.deadline = budget_ns > 0 ? global_ns() + (unsigned long long)budget_ns : 0ULL;
            sh.tree_gen = 0;
        }
        sm.live.allow = 0;  // the rounds pick from the tree (every CTA keeps a copy of its top)
        sm.live.on = 0;
        sm.live.max = 0;
        if (rank != 0) {
            const SpecScratch &h = helpers[size_t(box) * (kSpecMax - 1) + size_t(rank - 1)];
            R.box.cand_db = h.cand_db;
            R.box.cand_key = h.cand_key;
            R.box.cand_slot = h.cand_slot;
            R.box.cand_order = h.cand_order;
            R.box.cand_prefix = h.cand_prefix;
            R.box.best_res = h.best_res;
            R.box.best_ij = h.best_ij;
            R.box.surv = h.surv;
            R.box.surv_res = h.surv_res;
            R.box.surv_cap = h.surv_cap;
        }
    }
    __syncthreads();
    tree_cache_load(R, sm.tree);
    SpecShared *lead = cluster.map_shared_rank(&sh, 0);
    int gen = 0;
    long long done = 0, t0 = 0;
    for (;;) {
        if (rank == 0) {
            if (threadIdx.x == 0) t0 = clock64();
            spec_prepare(R, sm, sh, K, max_steps - done);
        }
        cluster.sync();
        const int stop = lead->stop, njobs = lead->n_jobs, tgen = lead->tree_gen;
        if (stop) break;
        if (rank < njobs) {
            if (rank != 0 && tgen != gen) {
                tree_cache_load(R, sm.tree);  // the leader's merges changed the tree
                gen = tgen;
            }
            spec_query(R, sm, &lead->job[rank], &lead->res[rank]);
        }
        cluster.sync();
        if (rank == 0) {
            if (threadIdx.x == 0) st.cyc_query += clock64() - t0;
            done += spec_commit(R, sm, sh, njobs);
        }
    }
    cluster.sync();  // no CTA leaves while another may still read its shared memory
    if (rank == 0) {
        const int swords = int(sizeof(RunState) / sizeof(int));
        const int *ssrc = reinterpret_cast<const int *>(&st);
        int *sdst = reinterpret_cast<int *>(st_global);
        for (int k = threadIdx.x; k < swords; k += NT) sdst[k] = ssrc[k];
    }
}

// The scalars of n boxes in one array.
__global__ void k_gather_run_scalars(const BoxRun *runs, int n, DevScalars *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = *runs[i].box.sc;
}

// A new aggregate-count stop criterion for n boxes: boxes that stopped
// without an error run again and re-check every criterion before their next
// step.
__global__ void k_set_aggregate_limit(BoxRun *runs, int n, long long limit) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    runs[i].lim.number_of_aggregates_limit = limit;
    RunState *st = runs[i].st;
    if (st != nullptr && st->status == ST_OK) st->finished = 0;
}

// Diagnostics of the device loop's random draws (one warp per block): the
// pick's descent of box 'box''s sum tree for per_warp targets per warp, each
// warp with its own rand() stream (seed + block), counted per slot.
__global__ void __launch_bounds__(32) k_pick_histogram(const BoxRun *runs, int box, long long per_warp,
                                                       unsigned seed, unsigned long long *counts) {
    __shared__ TreeCache cache;
    const BoxRun &R = runs[box];
    tree_cache_load(R, cache);
    RandStream rng;
    if (threadIdx.x == 0) rng.seed(seed + blockIdx.x);
    const unsigned long long total = R.st->tree_total;
    for (long long k = 0; k < per_warp; ++k) {
        unsigned long long t = 0;
        if (threadIdx.x == 0) t = pick_target(rng, total);
        t = __shfl_sync(0xffffffffu, t, 0);
        const int slot = tree_sample(R, cache, t);
        if (threadIdx.x == 0 && slot >= 0 && slot < R.box.nslots) atomicAdd(&counts[slot], 1ULL);
    }
}
// The counts of the live slots in slot order, i.e. by label (one thread).
__global__ void k_counts_by_label(const int *agg_n, int nslots, const unsigned long long *by_slot,
                                  long long *by_label, int *n_live) {
    int r = 0;
    for (int s = 0; s < nslots; ++s)
        if (agg_n[s] > 0) by_label[r++] = (long long)by_slot[s];
    *n_live = r;
}
// The device loop's directions: thread t draws directions t, t + T, t + 2T,
// ... (T threads in all) from its own rand() stream (seed + t).
__global__ void k_directions(long long n, unsigned seed, double *out) {
    const long long T = (long long)gridDim.x * blockDim.x;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    RandStream rng;
    rng.seed(seed + unsigned(t));
    for (long long i = t; i < n; i += T) {
        double d[3];
        draw_direction(rng, d);
        out[3 * i] = d[0];
        out[3 * i + 1] = d[1];
        out[3 * i + 2] = d[2];
    }
}

// The pick trees of n boxes from their time steps, one block per box
// (block_tree_build); the total weight goes to each box's loop state.
__global__ void __launch_bounds__(256) k_tree_build(const BoxRun *runs, int n) {
    if (int(blockIdx.x) >= n) return;
    block_tree_build(runs[blockIdx.x]);
}

namespace {
std::atomic<int> g_live_list_max{kLiveMax};
}  // namespace

int live_list_max() { return g_live_list_max.load(std::memory_order_relaxed); }
int set_live_list_max(int n) { return g_live_list_max.exchange(n); }

namespace {

bool ok_cuda(cudaError_t e, std::string *err, const char *what) {
    if (e == cudaSuccess) return true;
    if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
}

template <int NT>
cudaError_t prepare_k_run() {
    cudaError_t e =
        cudaFuncSetAttribute(k_run<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(RunSmemFor<NT>)));
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_run<NT>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
}
cudaError_t prepare_all_k_run() {
    cudaError_t e = prepare_k_run<32>();
    if (e == cudaSuccess) e = prepare_k_run<64>();
    if (e == cudaSuccess) e = prepare_k_run<128>();
    if (e == cudaSuccess) e = prepare_k_run<256>();
    if (e == cudaSuccess) e = prepare_k_run<512>();
    return e;
}
// order (may be null): the box each block takes, block b box order[b].
cudaError_t launch_k_run(int nt, int grid, cudaStream_t s, const BoxRun *runs, int n, long long steps,
                         long long budget_ns = 0, const int *order = nullptr) {
    switch (nt) {
        case 32: k_run<32><<<grid, 32, sizeof(RunSmemFor<32>), s>>>(runs, n, steps, budget_ns, order); break;
        case 64: k_run<64><<<grid, 64, sizeof(RunSmem), s>>>(runs, n, steps, budget_ns, order); break;
        case 128: k_run<128><<<grid, 128, sizeof(RunSmem), s>>>(runs, n, steps, budget_ns, order); break;
        case 512: k_run<512><<<grid, 512, sizeof(RunSmem), s>>>(runs, n, steps, budget_ns, order); break;
        default: k_run<256><<<grid, 256, sizeof(RunSmem), s>>>(runs, n, steps, budget_ns, order); break;
    }
    return cudaGetLastError();
}
template <int NT>
cudaLaunchConfig_t spec_config(int k, int n, cudaStream_t s, cudaLaunchAttribute *attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(unsigned(n) * unsigned(k));
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = sizeof(RunSmemFor<NT>);
    cfg.stream = s;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = unsigned(k);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}
template <int NT>
cudaError_t launch_spec_t(int k, int n, cudaStream_t s, const BoxRun *runs, const SpecScratch *h, long long steps,
                          long long budget_ns, const int *order) {
    static bool prepared = false;
    if (!prepared) {
        cudaError_t e = cudaFuncSetAttribute(k_run_spec<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             int(sizeof(RunSmemFor<NT>)));
        if (e != cudaSuccess) return e;
        prepared = true;
    }
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = spec_config<NT>(k, n, s, attr);
    return cudaLaunchKernelEx(&cfg, k_run_spec<NT>, runs, h, n, steps, budget_ns, order);
}
cudaError_t launch_spec(int nt, int k, int n, cudaStream_t s, const BoxRun *runs, const SpecScratch *h,
                        long long steps, long long budget_ns, const int *order) {
    switch (nt) {
        case 32: return launch_spec_t<32>(k, n, s, runs, h, steps, budget_ns, order);
        case 64: return launch_spec_t<64>(k, n, s, runs, h, steps, budget_ns, order);
        case 128: return launch_spec_t<128>(k, n, s, runs, h, steps, budget_ns, order);
        case 512: return launch_spec_t<512>(k, n, s, runs, h, steps, budget_ns, order);
        default: return launch_spec_t<256>(k, n, s, runs, h, steps, budget_ns, order);
    }
}
// Clusters of k CTAs of nt threads the device keeps resident at once.
template <int NT>
cudaError_t spec_clusters_t(int k, int *clusters) {
    cudaError_t e = cudaFuncSetAttribute(k_run_spec<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         int(sizeof(RunSmemFor<NT>)));
    if (e != cudaSuccess) return e;
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = spec_config<NT>(k, 1, nullptr, attr);
    return cudaOccupancyMaxActiveClusters(clusters, k_run_spec<NT>, &cfg);
}
cudaError_t spec_clusters(int nt, int k, int *clusters) {
    switch (nt) {
        case 32: return spec_clusters_t<32>(k, clusters);
        case 64: return spec_clusters_t<64>(k, clusters);
        case 128: return spec_clusters_t<128>(k, clusters);
        case 512: return spec_clusters_t<512>(k, clusters);
        default: return spec_clusters_t<256>(k, clusters);
    }
}
int occupancy_k_run(int nt, int *per_sm) {
    cudaError_t e;
    switch (nt) {
        case 32: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_run<32>, 32, sizeof(RunSmemFor<32>)); break;
        case 64: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_run<64>, 64, sizeof(RunSmem)); break;
        case 128: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_run<128>, 128, sizeof(RunSmem)); break;
        case 512: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_run<512>, 512, sizeof(RunSmem)); break;
        default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_run<256>, 256, sizeof(RunSmem)); break;
    }
    return e == cudaSuccess ? ST_OK : ST_CUDA;
}

// 32-ary sum tree over per-slot weights (leaves first, top level <= 32 entries).
struct TreeLayout {
    int levels = 0;
    int off[kMaxTreeLevels] = {0};
    int len[kMaxTreeLevels] = {0};
    int total = 0;
};

TreeLayout tree_layout(int nslots) {
    TreeLayout t;
    int len = std::max(nslots, 1);
    for (;;) {
        t.off[t.levels] = t.total;
        t.len[t.levels] = len;
        t.total += len;
        t.levels += 1;
        if (len <= kTreeFan || t.levels == kMaxTreeLevels) break;
        len = (len + kTreeFan - 1) / kTreeFan;
    }
    return t;
}

// The loop state and the launch record of one box; 'tree' (tree_layout's
// total doubles of device memory) receives the sum tree, built by
// k_tree_build from the box's time steps once the records are on the device.
int make_box_run(const DevBox &b, const mcacg_params &p, double time, RunState *state_dev, BoxRun *run,
                 RunState *state, unsigned long long *tree) {
    const TreeLayout tl = tree_layout(b.nslots);
    std::memset(state, 0, sizeof(*state));
    state->rng.seed(uint32_t(p.random_seed < 0 ? 0 : p.random_seed));
    state->time = time;
    state->weight_total = 0.0;  // set by k_tree_build
    std::memset(run, 0, sizeof(*run));
    run->box = b;
    run->phys = PhysParams{p.viscosity,
                           p.gaz_mean_free_path,
                           p.fractal_dimension,
                           p.density,
                           p.temperature,
                           p.with_surface_reactions ? p.u_sg : 0.0,
                           1.0 / p.gaz_mean_free_path,
                           1.0 / p.fractal_dimension,
                           p.with_surface_reactions ? 1 : 0,
                           p.with_surface_reactions && p.individual_surf_reactions ? 1 : 0,
                           int(std::max<int64_t>(1, p.full_aggregate_update_frequency)),
                           p.with_surface_reactions && p.u_sg < 0.0 ? 1 : 0,
                           p.rp_min_oxid};
    run->lim.number_of_aggregates_limit = p.number_of_aggregates_limit;
    run->lim.n_iter_without_event_limit = p.n_iter_without_event_limit;
    run->lim.mean_monomere_per_aggregate_limit = p.mean_monomere_per_aggregate_limit;
    run->lim.physical_time_limit = p.physical_time_limit;
    run->lim.with_collisions = p.with_collisions;
    run->st = state_dev;
    run->tree = tree;
    run->tree_levels = tl.levels;
    run->live_max = live_list_max();
    for (int k = 0; k < kMaxTreeLevels; ++k) {
        run->tree_off[k] = tl.off[k];
        run->tree_len[k] = tl.len[k];
    }
    return ST_OK;
}

}  // namespace

BatchRunner::~BatchRunner() {
    if (stream_) cudaStreamSynchronize(static_cast<cudaStream_t>(stream_));
    for (void *p : trees_) cudaFree(p);
    if (spec_mem_) cudaFree(spec_mem_);
    if (spec_tab_) cudaFree(spec_tab_);
    if (order_dev_) cudaFree(order_dev_);
    if (runs_dev_) cudaFree(runs_dev_);
    if (states_dev_) cudaFree(states_dev_);
    if (sc_dev_) cudaFree(sc_dev_);
    owned_.clear();
    if (own_stream_ && stream_) cudaStreamDestroy(static_cast<cudaStream_t>(stream_));
}

int BatchRunner::resident_boxes(int threads, int *boxes, std::string *err) {
    if (threads != 32 && threads != 64 && threads != 128 && threads != 256 && threads != 512) {
        if (err) *err = "threads per box must be 32, 64, 128, 256 or 512";
        return ST_BAD_ARGUMENT;
    }
    int dev = 0, n_sm = 0, per_sm = 0;
    if (!ok_cuda(cudaGetDevice(&dev), err, "cudaGetDevice") ||
        !ok_cuda(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev), err, "device attribute") ||
        !ok_cuda(prepare_all_k_run(), err, "cudaFuncSetAttribute"))
        return ST_CUDA;
    if (occupancy_k_run(threads, &per_sm) != ST_OK) {
        if (err) *err = "occupancy query failed";
        return ST_CUDA;
    }
    *boxes = std::max(1, per_sm) * n_sm;
    return ST_OK;
}

int BatchRunner::create(const std::vector<mcacg_params> &params, std::vector<HostState> &&states, void *stream,
                        std::unique_ptr<BatchRunner> *out, std::string *err) {
    std::vector<StateView> views(states.size());
    std::vector<std::vector<int>> compact(states.size());
    parallel_for(int(states.size()), [&](int i) { views[size_t(i)] = view_of(states[size_t(i)], &compact[size_t(i)]); });
    return create(params, views, stream, out, err);
}

int BatchRunner::create(const std::vector<mcacg_params> &params, const std::vector<StateView> &states, void *stream,
                        std::unique_ptr<BatchRunner> *out, std::string *err) {
    if (params.size() != states.size() || params.empty()) {
        if (err) *err = "one parameter set per state is needed";
        return ST_BAD_ARGUMENT;
    }
    std::unique_ptr<BatchRunner> r(new BatchRunner());
    int rc = r->init_stream(stream, err);
    if (rc != ST_OK) return rc;
    rc = DeviceBox::create_many(states, r->stream_, &r->owned_, err);
    if (rc != ST_OK) return rc;
    std::vector<double> times(states.size());
    for (size_t i = 0; i < states.size(); ++i) {
        times[i] = states[i].time;
        r->boxes_.push_back(r->owned_[i].get());
    }
    rc = r->init(params, times, err);
    if (rc != ST_OK) return rc;
    *out = std::move(r);
    return ST_OK;
}

int BatchRunner::attach(const std::vector<mcacg_params> &params, const std::vector<DeviceBox *> &boxes,
                        const std::vector<double> &times, void *stream, std::unique_ptr<BatchRunner> *out,
                        std::string *err) {
    if (params.size() != boxes.size() || boxes.empty() || times.size() != boxes.size()) {
        if (err) *err = "one parameter set and time per box is needed";
        return ST_BAD_ARGUMENT;
    }
    std::unique_ptr<BatchRunner> r(new BatchRunner());
    r->boxes_ = boxes;
    int rc = r->init_stream(stream, err);
    if (rc != ST_OK) return rc;
    rc = r->init(params, times, err);
    if (rc != ST_OK) return rc;
    *out = std::move(r);
    return ST_OK;
}

int BatchRunner::init_stream(void *stream, std::string *err) {
    if (stream) {
        stream_ = stream;
        return ST_OK;
    }
    cudaStream_t s;
    if (!ok_cuda(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), err, "cudaStreamCreate")) return ST_CUDA;
    stream_ = s;
    own_stream_ = true;
    return ST_OK;
}

int BatchRunner::init(const std::vector<mcacg_params> &params, const std::vector<double> &times, std::string *err) {
    const int n = int(boxes_.size());
    growth_.assign(static_cast<size_t>(n), 0);
    volsurf_.assign(static_cast<size_t>(n), VS_NONE);
    for (int i = 0; i < n; ++i) {
        growth_[size_t(i)] = params[size_t(i)].with_surface_reactions ? 1 : 0;
        volsurf_[size_t(i)] = params[size_t(i)].volsurf_method;
        const int rc = boxes_[size_t(i)]->set_volsurf(params[size_t(i)].volsurf_method);
        if (rc != ST_OK) {
            if (err) *err = "box " + std::to_string(i) + ": volsurf_method not available";
            return rc;
        }
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    for (DeviceBox *d : boxes_)
        if (d->sync(err) != ST_OK) return ST_CUDA;
    std::vector<BoxRun> runs(static_cast<size_t>(n));
    std::vector<RunState> states(static_cast<size_t>(n));
    if (!ok_cuda(cudaMalloc(&runs_dev_, sizeof(BoxRun) * size_t(n)), err, "cudaMalloc")) return ST_CUDA;
    if (!ok_cuda(cudaMalloc(&states_dev_, sizeof(RunState) * size_t(n)), err, "cudaMalloc")) return ST_CUDA;
    if (!ok_cuda(cudaMalloc(&sc_dev_, sizeof(DevScalars) * size_t(n)), err, "cudaMalloc")) return ST_CUDA;
    RunState *states_dev = static_cast<RunState *>(states_dev_);
    // the pick trees of all boxes in one allocation, built on the device
    std::vector<size_t> tree_off(static_cast<size_t>(n) + 1, 0);
    for (int i = 0; i < n; ++i) {
        const DevBox &b = *static_cast<DevBox *>(boxes_[size_t(i)]->devbox_ptr());
        tree_off[size_t(i) + 1] = tree_off[size_t(i)] + size_t(tree_layout(b.nslots).total);
    }
    void *trees = nullptr;
    if (!ok_cuda(cudaMalloc(&trees, sizeof(unsigned long long) * tree_off[size_t(n)]), err, "cudaMalloc"))
        return ST_CUDA;
    trees_.push_back(trees);
    for (int i = 0; i < n; ++i) {
        const DevBox &b = *static_cast<DevBox *>(boxes_[size_t(i)]->devbox_ptr());
        int rc = make_box_run(b, params[size_t(i)], times[size_t(i)], states_dev + i, &runs[size_t(i)],
                              &states[size_t(i)], static_cast<unsigned long long *>(trees) + tree_off[size_t(i)]);
        if (rc != ST_OK) return rc;
    }
    if (!ok_cuda(cudaMemcpyAsync(runs_dev_, runs.data(), sizeof(BoxRun) * size_t(n), cudaMemcpyHostToDevice, s), err,
                 "upload"))
        return ST_CUDA;
    if (!ok_cuda(cudaMemcpyAsync(states_dev_, states.data(), sizeof(RunState) * size_t(n), cudaMemcpyHostToDevice, s),
                 err, "upload"))
        return ST_CUDA;
    k_tree_build<<<n, 256, 0, s>>>(static_cast<const BoxRun *>(runs_dev_), n);
    if (!ok_cuda(cudaGetLastError(), err, "k_tree_build")) return ST_CUDA;
    // Launch order, largest box first: blocks are handed to the SMs in index
    // order, one per SM before a second, so the largest boxes -- the longest
    // chains of steps -- start on SMs of their own and share them only with
    // smaller boxes (which finish first). Each box's result does not depend
    // on where it runs.
    {
        std::vector<int> order(static_cast<size_t>(n));
        for (int i = 0; i < n; ++i) order[size_t(i)] = i;
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int c) { return boxes_[size_t(a)]->ns() > boxes_[size_t(c)]->ns(); });
        if (!ok_cuda(cudaMalloc(&order_dev_, sizeof(int) * size_t(n)), err, "cudaMalloc") ||
            !ok_cuda(cudaMemcpyAsync(order_dev_, order.data(), sizeof(int) * size_t(n), cudaMemcpyHostToDevice, s),
                     err, "upload"))
            return ST_CUDA;
    }
    if (!ok_cuda(prepare_all_k_run(), err, "cudaFuncSetAttribute")) return ST_CUDA;
    if (!ok_cuda(cudaStreamSynchronize(s), err, "sync")) return ST_CUDA;
    return ST_OK;
}

int BatchRunner::set_speculation(int k) {
    if (k != 0 && k != 1 && k != 2 && k != 4 && k != 8) return ST_BAD_ARGUMENT;
    spec_k_ = k == 0 ? 1 : k;
    if (auto_threads_) threads_ = 0;  // the block size is chosen again for the new cluster size
    return ST_OK;
}

// Helper-CTA scratch for speculative rounds, once: for each box, the query
// lists of up to kSpecMax - 1 helpers (fewer when the device lacks room).
// Returns the most CTAs per box it allows (1: none).
int BatchRunner::spec_room(std::string *err) {
    if (spec_max_ > 0) return spec_max_;
    spec_max_ = 1;
    const int n = int(boxes_.size());
    auto r256 = [](size_t x) { return (x + 255) & ~size_t(255); };
    std::vector<size_t> set_bytes(static_cast<size_t>(n));
    size_t per_helper = 0;
    for (int i = 0; i < n; ++i) {
        const size_t nc1 = size_t(boxes_[size_t(i)]->nslots()) + 1;
        set_bytes[size_t(i)] = 4 * r256(8 * nc1) + 3 * r256(4 * nc1) + r256(sizeof(int4) * kSpecSurvivors) +
                               r256(sizeof(double) * kSpecSurvivors);
        per_helper += set_bytes[size_t(i)];
    }
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return spec_max_;
    }
    int kmax = kSpecMax;
    while (kmax > 1 && per_helper * size_t(kmax - 1) > free_b / 2) kmax /= 2;
    if (kmax < 2) return spec_max_;
    std::vector<SpecScratch> tab(size_t(n) * (kSpecMax - 1));
    if (!ok_cuda(cudaMalloc(&spec_mem_, per_helper * size_t(kmax - 1)), err, "cudaMalloc") ||
        !ok_cuda(cudaMalloc(&spec_tab_, sizeof(SpecScratch) * tab.size()), err, "cudaMalloc")) {
        if (spec_mem_) cudaFree(spec_mem_);
        spec_mem_ = nullptr;
        cudaGetLastError();
        return spec_max_;
    }
    char *p = static_cast<char *>(spec_mem_);
    for (int i = 0; i < n; ++i) {
        const size_t nc1 = size_t(boxes_[size_t(i)]->nslots()) + 1;
        for (int h = 0; h < kmax - 1; ++h) {
            SpecScratch &t = tab[size_t(i) * (kSpecMax - 1) + size_t(h)];
            char *q = p;
            auto take = [&](size_t bytes) {
                char *r = q;
                q += r256(bytes);
                return r;
            };
            t.cand_db = reinterpret_cast<double *>(take(8 * nc1));
            t.cand_key = reinterpret_cast<long long *>(take(8 * nc1));
            t.best_res = reinterpret_cast<unsigned long long *>(take(8 * nc1));
            t.best_ij = reinterpret_cast<unsigned long long *>(take(8 * nc1));
            t.cand_slot = reinterpret_cast<int *>(take(4 * nc1));
            t.cand_order = reinterpret_cast<int *>(take(4 * nc1));
            t.cand_prefix = reinterpret_cast<int *>(take(4 * nc1));
            t.surv = reinterpret_cast<int4 *>(take(sizeof(int4) * kSpecSurvivors));
            t.surv_res = reinterpret_cast<double *>(take(sizeof(double) * kSpecSurvivors));
            t.surv_cap = kSpecSurvivors;
            t.pad = 0;
            p += set_bytes[size_t(i)];
        }
    }
    if (!ok_cuda(cudaMemcpy(spec_tab_, tab.data(), sizeof(SpecScratch) * tab.size(), cudaMemcpyHostToDevice), err,
                 "upload"))
        return spec_max_;
    spec_max_ = kmax;
    return spec_max_;
}

// One launch of the loop at nt threads per CTA and k CTAs per box.
cudaError_t BatchRunner::launch_run(int nt, int k, long long steps, long long budget_ns) {
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    const int n = int(boxes_.size());
    const BoxRun *runs = static_cast<const BoxRun *>(runs_dev_);
    if (k > 1) k = std::min(k, spec_room(nullptr));  // helper scratch set up at the first such launch
    const int *order = static_cast<const int *>(order_dev_);
    if (k <= 1 || !spec_tab_) return launch_k_run(nt, n, s, runs, n, steps, budget_ns, order);
    return launch_spec(nt, k, n, s, runs, static_cast<const SpecScratch *>(spec_tab_), steps, budget_ns, order);
}

int BatchRunner::set_threads(int threads) {
    if (threads != 0 && threads != 32 && threads != 64 && threads != 128 && threads != 256 && threads != 512)
        return ST_BAD_ARGUMENT;
    threads_ = threads;
    auto_threads_ = threads == 0;
    return ST_OK;
}

// Chooses the threads per box for the unfinished boxes (tuned_active_ of
// them): the largest block size at which every one of them is resident at
// once. A run's wall time is the chain of steps of its slowest boxes, and a
// box's step is a chain of dependent loads and block barriers whose parallel
// parts (the neighbour scan, the sphere-pair search, the merge's pair
// search) shorten with more threads; a second wave of blocks, though, would
// wait for the first (and time-capped launches give each block its budget
// from its own start, so a second wave also halves every box's share of a
// launch). Timing a few steps of each size, as this once did, chose by the
// boxes' cheap first steps and, late in a run, spent seconds on steps of the
// large aggregates run with 32 threads. Speculative rounds (spec.cuh) stay
// off unless set (set_speculation): clusters of several blocks per box
// leave fewer boxes resident at a given block size, and measured on the
// benchmark ensemble they gained at most 10% on its slowest chains. Returns
// ST_OK (nothing is run).
int BatchRunner::tune(int64_t, int64_t *, float *, std::string *err, bool) {
    if (!auto_threads_ && threads_ != 0) return ST_OK;
    int best = kRunThreadChoices[0];
    for (int nt : kRunThreadChoices) {
        int resident = 0;
        if (spec_k_ > 1) {
            if (spec_clusters(nt, spec_k_, &resident) != cudaSuccess) {
                cudaGetLastError();
                resident = 0;
            }
        } else if (resident_boxes(nt, &resident, err) != ST_OK) {
            return ST_CUDA;
        }
        if (resident >= tuned_active_) best = nt;
    }
    threads_ = best;
    return ST_OK;
}

int BatchRunner::run(int64_t max_steps, int64_t chunk, std::string *err) {
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    const int n = int(boxes_.size());
    const BoxRun *runs = static_cast<const BoxRun *>(runs_dev_);
    if (chunk <= 0) chunk = 20000;
    launches_ = 0;
    int64_t done = 0;
    int rc = ST_OK;
    float ms_total = 0.f;
    auto count_active = [&](int *active) -> int {
        std::vector<BoxRunStats> st;
        int r = stats(&st, err);
        if (r != ST_OK) return r;
        int a = 0;
        for (const auto &x : st) a += !(x.finished || x.status != ST_OK);
        *active = a;
        return ST_OK;
    };
    if (auto_threads_ && threads_ == 0) {
        rc = count_active(&tuned_active_);
        if (rc == ST_OK) rc = tune(max_steps, &done, &ms_total, err, max_steps <= 0);
        if (rc != ST_OK) return rc;
    }
    const float ms_tune = ms_total;
    ms_total = 0.f;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (;;) {
        int64_t steps = max_steps > 0 ? std::min(chunk, max_steps - done) : chunk;
        if (steps <= 0) break;
        const int nt = threads_ ? threads_ : 256;
        // to the stop criteria: launches of a fixed wall time, each box
        // doing as many steps as it can in it
        const long long budget = max_steps <= 0 ? kRunLaunchBudgetNs : 0;
        cudaEventRecord(e0, s);
        if (!ok_cuda(launch_run(nt, spec_k_, (long long)steps, budget), err, "k_run")) {
            rc = ST_CUDA;
            break;
        }
        cudaEventRecord(e1, s);
        if (!ok_cuda(cudaEventSynchronize(e1), err, "k_run")) {
            rc = ST_CUDA;
            break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        ms_total += ms;
        ++launches_;
        done += steps;
        if (max_steps > 0 && done >= max_steps) break;
        {
            // until every box has met its stop criterion (or failed), or the
            // step count; when half of the boxes running at the last choice
            // have finished, the block size is chosen again
            int active = 0;
            rc = count_active(&active);
            if (rc != ST_OK) break;
            if (active == 0) break;
            if (auto_threads_ && active * 2 <= tuned_active_) {
                tuned_active_ = active;
                float mt = 0.f;
                rc = tune(0, &done, &mt, err, true);
                ms_total += mt;
                if (rc != ST_OK) break;
            }
        }
    }
    last_ms_ = ms_total + ms_tune;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

int BatchRunner::run_timed(double wall_ms, std::string *err) {
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    const int n = int(boxes_.size());
    const BoxRun *runs = static_cast<const BoxRun *>(runs_dev_);
    const auto t0 = std::chrono::steady_clock::now();
    auto elapsed_ms = [&] {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    };
    launches_ = 0;
    float ms_total = 0.f;
    int64_t done = 0;
    auto count_active = [&](int *active) -> int {
        std::vector<BoxRunStats> st;
        int r = stats(&st, err);
        if (r != ST_OK) return r;
        int a = 0;
        for (const auto &x : st) a += !(x.finished || x.status != ST_OK);
        *active = a;
        return ST_OK;
    };
    int active = 0;
    int rc = count_active(&active);
    if (rc != ST_OK) return rc;
    int resident_now = 0;
    if (threads_ != 0 && resident_boxes(threads_, &resident_now, err) != ST_OK) return ST_CUDA;
    if (auto_threads_ && (threads_ == 0 || active * 2 <= tuned_active_ || resident_now < active) && active > 0) {
        tuned_active_ = active;
        rc = tune(0, &done, &ms_total, err, true);
        if (rc != ST_OK) return rc;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    while (active > 0) {
        const double left = wall_ms - elapsed_ms();
        if (left <= 0.0) break;
        const long long budget = std::max(1LL, std::min(kRunLaunchBudgetNs, (long long)(left * 1e6)));
        const int nt = threads_ ? threads_ : 256;
        cudaEventRecord(e0, s);
        if (!ok_cuda(launch_run(nt, spec_k_, 1LL << 50, budget), err, "k_run")) {
            rc = ST_CUDA;
            break;
        }
        cudaEventRecord(e1, s);
        if (!ok_cuda(cudaEventSynchronize(e1), err, "k_run")) {
            rc = ST_CUDA;
            break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        ms_total += ms;
        ++launches_;
        rc = count_active(&active);
        if (rc != ST_OK) break;
        if (auto_threads_ && active > 0 && active * 2 <= tuned_active_) {
            tuned_active_ = active;
            rc = tune(0, &done, &ms_total, err, true);
            if (rc != ST_OK) break;
        }
    }
    last_ms_ = ms_total;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

int BatchRunner::pick_histogram(int box, int64_t n_picks, uint32_t seed, std::vector<int64_t> *by_label,
                                int64_t *picks_done, std::string *err) {
    if (box < 0 || box >= size() || n_picks <= 0) {
        if (err) *err = "box out of range or no picks asked";
        return ST_BAD_ARGUMENT;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    const DevBox &b = *static_cast<const DevBox *>(boxes_[size_t(box)]->devbox_ptr());
    const int nslots = b.nslots;
    constexpr int kWarps = 256;
    const long long per_warp = (n_picks + kWarps - 1) / kWarps;
    void *mem = nullptr;
    const size_t bytes = sizeof(unsigned long long) * size_t(nslots) * 2 + 256;
    if (!ok_cuda(cudaMalloc(&mem, bytes), err, "cudaMalloc")) return ST_CUDA;
    auto *by_slot = static_cast<unsigned long long *>(mem);
    auto *lab = reinterpret_cast<long long *>(by_slot + nslots);
    int *n_live_dev = reinterpret_cast<int *>(lab + nslots);
    int n_live = 0;
    by_label->assign(size_t(nslots), 0);
    bool ok = ok_cuda(cudaMemsetAsync(by_slot, 0, sizeof(unsigned long long) * size_t(nslots), s), err, "memset");
    if (ok) {
        k_pick_histogram<<<kWarps, 32, 0, s>>>(static_cast<const BoxRun *>(runs_dev_), box, per_warp, seed, by_slot);
        k_counts_by_label<<<1, 1, 0, s>>>(b.agg_n, nslots, by_slot, lab, n_live_dev);
        ok = ok_cuda(cudaGetLastError(), err, "k_pick_histogram") &&
             ok_cuda(cudaMemcpyAsync(by_label->data(), lab, sizeof(long long) * size_t(nslots), cudaMemcpyDeviceToHost,
                                     s),
                     err, "download") &&
             ok_cuda(cudaMemcpyAsync(&n_live, n_live_dev, sizeof(int), cudaMemcpyDeviceToHost, s), err, "download") &&
             ok_cuda(cudaStreamSynchronize(s), err, "k_pick_histogram");
    }
    cudaFree(mem);
    if (!ok) return ST_CUDA;
    by_label->resize(size_t(n_live));
    *picks_done = per_warp * kWarps;
    return ST_OK;
}

int BatchRunner::draw_directions(int64_t n, uint32_t seed, double *out, std::string *err) {
    if (n <= 0) return ST_OK;
    void *mem = nullptr;
    if (!ok_cuda(cudaMalloc(&mem, sizeof(double) * 3 * size_t(n)), err, "cudaMalloc")) return ST_CUDA;
    const long long threads = std::min<long long>(n, 1 << 16);
    k_directions<<<unsigned((threads + 255) / 256), 256>>>(n, seed, static_cast<double *>(mem));
    const bool ok = ok_cuda(cudaGetLastError(), err, "k_directions") &&
                    ok_cuda(cudaMemcpy(out, mem, sizeof(double) * 3 * size_t(n), cudaMemcpyDeviceToHost), err,
                            "download");
    cudaFree(mem);
    return ok ? ST_OK : ST_CUDA;
}

int BatchRunner::set_aggregate_limit(int64_t limit, std::string *err) {
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    const int n = int(boxes_.size());
    if (n == 0) return ST_OK;
    k_set_aggregate_limit<<<(n + 255) / 256, 256, 0, s>>>(static_cast<BoxRun *>(runs_dev_), n, (long long)limit);
    if (!ok_cuda(cudaGetLastError(), err, "k_set_aggregate_limit")) return ST_CUDA;
    return ST_OK;
}

int BatchRunner::stats(std::vector<BoxRunStats> *out, std::string *err) {
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    const int n = int(boxes_.size());
    std::vector<RunState> st(static_cast<size_t>(n));
    if (!ok_cuda(cudaMemcpyAsync(st.data(), states_dev_, sizeof(RunState) * size_t(n), cudaMemcpyDeviceToHost, s),
                 err, "download"))
        return ST_CUDA;
    // the boxes' scalars gathered on the device, then one copy
    std::vector<DevScalars> sc(static_cast<size_t>(n));
    k_gather_run_scalars<<<(n + 255) / 256, 256, 0, s>>>(static_cast<const BoxRun *>(runs_dev_), n,
                                                          static_cast<DevScalars *>(sc_dev_));
    if (!ok_cuda(cudaGetLastError(), err, "k_gather_run_scalars") ||
        !ok_cuda(cudaMemcpyAsync(sc.data(), sc_dev_, sizeof(DevScalars) * size_t(n), cudaMemcpyDeviceToHost, s), err,
                 "download") ||
        !ok_cuda(cudaStreamSynchronize(s), err, "sync"))
        return ST_CUDA;
    out->resize(size_t(n));
    for (int i = 0; i < n; ++i) {
        BoxRunStats &o = (*out)[size_t(i)];
        o.steps = st[size_t(i)].steps;
        o.events = st[size_t(i)].events;
        o.time = st[size_t(i)].time;
        o.finished = st[size_t(i)].finished;
        o.status = st[size_t(i)].status != ST_OK ? st[size_t(i)].status : sc[size_t(i)].status;
        o.n_alive = sc[size_t(i)].n_alive;
        const RunState &r = st[size_t(i)];
        o.queries = r.c_queries;
        o.mov = r.c_mov;
        o.scanned = r.c_scanned;
        o.cells = r.c_cells;
        o.candidates = r.c_candidates;
        o.cand_spheres = r.c_cand_spheres;
        o.refined = r.c_refined;
        o.merged_spheres = r.c_merged_spheres;
        o.merge_pairs = r.c_merge_pairs;
        o.cyc_pick = r.cyc_pick;
        o.cyc_query = r.cyc_query;
        o.cyc_move = r.cyc_move;
        o.cyc_merge = r.cyc_merge;
        o.cyc_qscan = r.cyc_qscan;
        o.cyc_qpairs = r.cyc_qpairs;
    }
    return ST_OK;
}

int BatchRunner::download(int box, HostState *st, std::string *err) {
    if (box < 0 || box >= size()) return ST_BAD_ARGUMENT;
    int rc = boxes_[size_t(box)]->download(st, err);
    if (rc != ST_OK) return rc;
    if (refresh_overlap(box)) host_refresh_overlap(st);
    RunState r;
    if (!ok_cuda(cudaMemcpy(&r, static_cast<RunState *>(states_dev_) + box, sizeof(r), cudaMemcpyDeviceToHost), err,
                 "download"))
        return ST_CUDA;
    st->time = r.time;
    return ST_OK;
}

int BatchRunner::times(std::vector<double> *out, std::string *err) {
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    const int n = size();
    std::vector<RunState> st(static_cast<size_t>(n));
    if (!ok_cuda(cudaMemcpyAsync(st.data(), states_dev_, sizeof(RunState) * size_t(n), cudaMemcpyDeviceToHost, s),
                 err, "download") ||
        !ok_cuda(cudaStreamSynchronize(s), err, "sync"))
        return ST_CUDA;
    out->resize(size_t(n));
    for (int i = 0; i < n; ++i) (*out)[size_t(i)] = st[size_t(i)].time;
    return ST_OK;
}

// ------------------------------------------------------------------ Server
double Server::now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count() - t0_;
}

int64_t Server::footprint(const mcacg_params &p) {
    // device bytes of one box (DeviceBox::create's arrays plus the sum tree)
    const int64_t n = p.n_monomeres;
    const int64_t cells = p.n_verlet_divisions * p.n_verlet_divisions * p.n_verlet_divisions;
    const int64_t fine_cells = int64_t(kFineMaxDiv) * kFineMaxDiv * kFineMaxDiv;  // upper bound
    return n * 760 + cells * 4 * 80 + fine_cells * 4 + (3 << 20);
}

int Server::create(int capacity, int64_t memory_budget, void *stream, bool keep_final_states,
                   std::unique_ptr<Server> *out, std::string *err) {
    if (capacity <= 0) {
        if (err) *err = "capacity must be positive";
        return ST_BAD_ARGUMENT;
    }
    std::unique_ptr<Server> s(new Server());
    s->capacity_ = capacity;
    s->budget_ = memory_budget > 0 ? memory_budget : (int64_t(1) << 40);
    s->keep_ = keep_final_states;
    s->t0_ = 0;
    s->t0_ = s->now();
    if (stream) {
        s->stream_ = stream;
    } else {
        cudaStream_t st;
        if (!ok_cuda(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), err, "cudaStreamCreate")) return ST_CUDA;
        s->stream_ = st;
        s->own_stream_ = true;
    }
    s->slots_.resize(size_t(capacity));
    if (!ok_cuda(cudaMalloc(&s->runs_dev_, sizeof(BoxRun) * size_t(capacity)), err, "cudaMalloc")) return ST_CUDA;
    if (!ok_cuda(cudaMalloc(&s->states_dev_, sizeof(RunState) * size_t(capacity)), err, "cudaMalloc")) return ST_CUDA;
    if (!ok_cuda(cudaMemset(s->runs_dev_, 0, sizeof(BoxRun) * size_t(capacity)), err, "cudaMemset")) return ST_CUDA;
    if (!ok_cuda(prepare_all_k_run(), err, "cudaFuncSetAttribute")) return ST_CUDA;
    *out = std::move(s);
    return ST_OK;
}

int Server::set_threads(int threads) {
    if (threads != 0 && threads != 32 && threads != 64 && threads != 128 && threads != 256 && threads != 512)
        return ST_BAD_ARGUMENT;
    threads_ = threads;
    return ST_OK;
}

Server::~Server() {
    if (stream_) cudaStreamSynchronize(static_cast<cudaStream_t>(stream_));
    for (auto &sl : slots_)
        if (sl.tree) cudaFree(sl.tree);
    slots_.clear();
    if (runs_dev_) cudaFree(runs_dev_);
    if (states_dev_) cudaFree(states_dev_);
    if (own_stream_ && stream_) cudaStreamDestroy(static_cast<cudaStream_t>(stream_));
}

int Server::submit(const mcacg_params &p, int64_t *id, std::string *err) {
    if (p.with_nucleation || p.with_potentials || p.with_flame_coupling || p.with_electric_charges) {
        if (err) *err = "served boxes cover collisions with optional surface reactions";
        return ST_INPUT;
    }
    if (footprint(p) > budget_) {
        if (err) *err = "request larger than the device-memory budget";
        return ST_CAPACITY;
    }
    *id = next_id_++;
    pending_.push_back(Request{*id, p, now()});
    return ST_OK;
}

int Server::n_active() const {
    int n = 0;
    for (const auto &sl : slots_) n += sl.id >= 0;
    return n;
}

int Server::admit(std::string *err) {
    // free slots and requests that fit, first come first served
    std::vector<int> free_slots;
    for (int i = 0; i < capacity_; ++i)
        if (slots_[size_t(i)].id < 0) free_slots.push_back(i);
    std::vector<Request> take;
    size_t k = 0;
    int64_t mem = mem_in_use_;
    while (k < pending_.size() && take.size() < free_slots.size()) {
        int64_t need = footprint(pending_[k].p);
        if (mem + need > budget_) break;  // keep arrival order: wait for memory
        mem += need;
        take.push_back(pending_[k]);
        ++k;
    }
    pending_.erase(pending_.begin(), pending_.begin() + long(k));
    if (take.empty()) return ST_OK;
    // reference placements in parallel (private rand() streams)
    std::vector<HostState> states(take.size());
    std::vector<int> rcs(take.size(), 0);
    std::vector<std::string> errs(take.size());
    std::atomic<int> next{0};
    unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), unsigned(take.size())));
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nt; ++t)
        pool.emplace_back([&] {
            for (int i = next++; i < int(take.size()); i = next++)
                rcs[size_t(i)] = init_random_state_private(take[size_t(i)].p, &states[size_t(i)], &errs[size_t(i)]);
        });
    for (auto &th : pool) th.join();
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    BoxRun *runs_dev = static_cast<BoxRun *>(runs_dev_);
    RunState *states_dev = static_cast<RunState *>(states_dev_);
    for (size_t i = 0; i < take.size(); ++i) {
        const int slot = free_slots[i];
        Slot &sl = slots_[size_t(slot)];
        const double t_admit = now();
        if (rcs[i] != ST_OK) {
            done_.push_back(Completion{take[i].id, 0, 0, 0, 0.0, rcs[i], 0, take[i].submit_s, t_admit, t_admit});
            continue;
        }
        DeviceBox *d = nullptr;
        int rc = DeviceBox::create(states[i], stream_, &d, err);
        if (rc != ST_OK) return rc;
        sl.box.reset(d);
        rc = d->set_volsurf(take[i].p.volsurf_method);
        if (rc != ST_OK) {
            const double t_fail = now();
            done_.push_back(Completion{take[i].id, 0, 0, 0, 0.0, rc, 0, take[i].submit_s, t_fail, t_fail});
            sl.box.reset();
            continue;
        }
        BoxRun run;
        RunState st;
        const DevBox &db = *static_cast<DevBox *>(d->devbox_ptr());
        if (!ok_cuda(cudaMalloc(&sl.tree, sizeof(unsigned long long) * size_t(tree_layout(db.nslots).total)), err,
                     "cudaMalloc"))
            return ST_CUDA;
        rc = make_box_run(db, take[i].p, states[i].time, states_dev + slot, &run, &st,
                          static_cast<unsigned long long *>(sl.tree));
        if (rc != ST_OK) return rc;
        if (!ok_cuda(cudaMemcpyAsync(states_dev + slot, &st, sizeof(st), cudaMemcpyHostToDevice, s), err, "upload") ||
            !ok_cuda(cudaMemcpyAsync(runs_dev + slot, &run, sizeof(run), cudaMemcpyHostToDevice, s), err, "upload"))
            return ST_CUDA;
        k_tree_build<<<1, 256, 0, s>>>(runs_dev + slot, 1);
        if (!ok_cuda(cudaGetLastError(), err, "k_tree_build") || !ok_cuda(cudaStreamSynchronize(s), err, "sync"))
            return ST_CUDA;
        sl.id = take[i].id;
        sl.growth = take[i].p.with_surface_reactions != 0;
        sl.volsurf = take[i].p.volsurf_method;
        sl.bytes = footprint(take[i].p);
        sl.submit_s = take[i].submit_s;
        sl.admit_s = t_admit;
        mem_in_use_ += sl.bytes;
        states[i] = HostState();
    }
    return ST_OK;
}

int Server::retire(std::string *err) {
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    std::vector<RunState> st(static_cast<size_t>(capacity_));
    if (!ok_cuda(cudaMemcpyAsync(st.data(), states_dev_, sizeof(RunState) * size_t(capacity_), cudaMemcpyDeviceToHost,
                                 s), err, "download") ||
        !ok_cuda(cudaStreamSynchronize(s), err, "sync"))
        return ST_CUDA;
    BoxRun *runs_dev = static_cast<BoxRun *>(runs_dev_);
    for (int i = 0; i < capacity_; ++i) {
        Slot &sl = slots_[size_t(i)];
        if (sl.id < 0) continue;
        const RunState &r = st[size_t(i)];
        if (!r.finished && r.status == ST_OK) continue;
        HostState final_state;
        if (keep_) {
            int rc = sl.box->download(&final_state, err);
            if (rc == ST_OK && sl.growth && sl.volsurf == VS_NONE) host_refresh_overlap(&final_state);
            if (rc != ST_OK) return rc;
            final_state.time = r.time;
        }
        DevScalars sc;
        const DevBox &b = *static_cast<DevBox *>(sl.box->devbox_ptr());
        if (!ok_cuda(cudaMemcpy(&sc, b.sc, sizeof(sc), cudaMemcpyDeviceToHost), err, "download")) return ST_CUDA;
        done_.push_back(Completion{sl.id, r.steps, r.events, sc.n_alive, r.time, r.status, r.finished, sl.submit_s,
                                   sl.admit_s, now()});
        if (keep_) finals_.emplace_back(sl.id, std::move(final_state));
        BoxRun empty;
        std::memset(&empty, 0, sizeof(empty));
        if (!ok_cuda(cudaMemcpyAsync(runs_dev + i, &empty, sizeof(empty), cudaMemcpyHostToDevice, s), err, "upload") ||
            !ok_cuda(cudaStreamSynchronize(s), err, "sync"))
            return ST_CUDA;
        sl.box.reset();
        if (sl.tree) cudaFree(sl.tree);
        sl.tree = nullptr;
        mem_in_use_ -= sl.bytes;
        sl = Slot();
    }
    return ST_OK;
}

int Server::step(int64_t epoch_steps, std::string *err) {
    int rc = admit(err);
    if (rc != ST_OK) return rc;
    if (n_active() > 0) {
        cudaStream_t s = static_cast<cudaStream_t>(stream_);
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        // threads per box: as set, or (0) the largest size at which every
        // active box is resident at once (empty slots leave at once)
        int nt = threads_;
        if (nt == 0) {
            const int active = n_active();
            nt = kRunThreadChoices[0];
            for (int c : kRunThreadChoices) {
                int resident = 0;
                if (BatchRunner::resident_boxes(c, &resident, err) != ST_OK) return ST_CUDA;
                if (resident >= active) nt = c;
            }
        }
        last_threads_ = nt;
        cudaEventRecord(e0, s);
        const cudaError_t le = launch_k_run(nt, capacity_, s, static_cast<const BoxRun *>(runs_dev_), capacity_,
                                            (long long)epoch_steps, epoch_budget_ns_);
        ++launches_;
        cudaEventRecord(e1, s);
        if (!ok_cuda(le, err, "k_run") || !ok_cuda(cudaEventSynchronize(e1), err, "k_run")) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return ST_CUDA;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        kernel_ms_ += ms;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    return retire(err);
}

std::vector<Completion> Server::poll() {
    std::vector<Completion> out;
    out.swap(done_);
    return out;
}

int Server::final_state(int64_t id, HostState *st) const {
    for (const auto &f : finals_)
        if (f.first == id) {
            *st = f.second;
            return ST_OK;
        }
    return ST_BAD_ARGUMENT;
}

}  // namespace mcacg
