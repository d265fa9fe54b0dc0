// Persistent device loop over many boxes; see batch.hpp and run.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "batch.hpp"
#include "run.cuh"

namespace mcacg {

constexpr int kRunThreads = 256;

template <int NT>
__global__ void __launch_bounds__(NT) k_run(const BoxRun *runs, int n, long long max_steps) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    RunSmem &sm = *reinterpret_cast<RunSmem *>(smem_raw);
    __shared__ __align__(16) BoxRun R;
    const int box = blockIdx.x;
    if (box >= n) return;
    const int words = int(sizeof(BoxRun) / sizeof(int));
    const int *src = reinterpret_cast<const int *>(&runs[box]);
    int *dst = reinterpret_cast<int *>(&R);
    for (int k = threadIdx.x; k < words; k += NT) dst[k] = src[k];
    __syncthreads();
    for (long long s = 0; s < max_steps; ++s)
        if (!block_mc_step(R, sm)) break;
}

namespace {

bool ok_cuda(cudaError_t e, std::string *err, const char *what) {
    if (e == cudaSuccess) return true;
    if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
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

}  // namespace

BatchRunner::~BatchRunner() {
    if (stream_) cudaStreamSynchronize(static_cast<cudaStream_t>(stream_));
    for (void *p : trees_) cudaFree(p);
    if (runs_dev_) cudaFree(runs_dev_);
    if (states_dev_) cudaFree(states_dev_);
    owned_.clear();
    if (own_stream_ && stream_) cudaStreamDestroy(static_cast<cudaStream_t>(stream_));
}

int BatchRunner::create(const std::vector<mcacg_params> &params, std::vector<HostState> &&states, void *stream,
                        std::unique_ptr<BatchRunner> *out, std::string *err) {
    if (params.size() != states.size() || params.empty()) {
        if (err) *err = "one parameter set per state is needed";
        return ST_BAD_ARGUMENT;
    }
    std::unique_ptr<BatchRunner> r(new BatchRunner());
    std::vector<double> times;
    for (size_t i = 0; i < states.size(); ++i) {
        DeviceBox *d = nullptr;
        int rc = DeviceBox::create(states[i], stream, &d, err);
        if (rc != ST_OK) return rc;
        r->owned_.emplace_back(d);
        r->boxes_.push_back(d);
        times.push_back(states[i].time);
        states[i] = HostState();  // release host memory early
    }
    int rc = r->init_stream(stream, err);
    if (rc != ST_OK) return rc;
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
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    for (DeviceBox *d : boxes_)
        if (d->sync(err) != ST_OK) return ST_CUDA;
    std::vector<BoxRun> runs(static_cast<size_t>(n));
    std::vector<RunState> states(static_cast<size_t>(n));
    if (!ok_cuda(cudaMalloc(&runs_dev_, sizeof(BoxRun) * size_t(n)), err, "cudaMalloc")) return ST_CUDA;
    if (!ok_cuda(cudaMalloc(&states_dev_, sizeof(RunState) * size_t(n)), err, "cudaMalloc")) return ST_CUDA;
    RunState *states_dev = static_cast<RunState *>(states_dev_);
    for (int i = 0; i < n; ++i) {
        const DevBox &b = *static_cast<DevBox *>(boxes_[size_t(i)]->devbox_ptr());
        const mcacg_params &p = params[size_t(i)];
        // leaves: 1 / time_step of every live slot
        std::vector<double> ts(size_t(b.nslots));
        std::vector<int> alive(size_t(b.nslots));
        if (!ok_cuda(cudaMemcpy(ts.data(), b.agg + size_t(AGG_TIME_STEP) * b.nslots, sizeof(double) * ts.size(),
                                cudaMemcpyDeviceToHost), err, "download"))
            return ST_CUDA;
        if (!ok_cuda(cudaMemcpy(alive.data(), b.agg_n, sizeof(int) * alive.size(), cudaMemcpyDeviceToHost), err,
                     "download"))
            return ST_CUDA;
        TreeLayout tl = tree_layout(b.nslots);
        std::vector<double> tree(size_t(tl.total), 0.0);
        for (int a = 0; a < b.nslots; ++a) tree[size_t(a)] = alive[size_t(a)] > 0 ? 1.0 / ts[size_t(a)] : 0.0;
        for (int lev = 1; lev < tl.levels; ++lev)
            for (int g = 0; g < tl.len[lev]; ++g) {
                double sum = 0.0;
                for (int k = 0; k < kTreeFan; ++k) {
                    int c = g * kTreeFan + k;
                    if (c < tl.len[lev - 1]) sum += tree[size_t(tl.off[lev - 1] + c)];
                }
                tree[size_t(tl.off[lev] + g)] = sum;
            }
        double total = 0.0;
        for (int k = 0; k < tl.len[tl.levels - 1]; ++k) total += tree[size_t(tl.off[tl.levels - 1] + k)];
        void *tree_dev = nullptr;
        if (!ok_cuda(cudaMalloc(&tree_dev, sizeof(double) * tree.size()), err, "cudaMalloc")) return ST_CUDA;
        trees_.push_back(tree_dev);
        if (!ok_cuda(cudaMemcpy(tree_dev, tree.data(), sizeof(double) * tree.size(), cudaMemcpyHostToDevice), err,
                     "upload"))
            return ST_CUDA;
        RunState &st = states[size_t(i)];
        std::memset(&st, 0, sizeof(st));
        st.rng.seed(uint32_t(p.random_seed < 0 ? 0 : p.random_seed));
        st.time = times[size_t(i)];
        st.weight_total = total;
        BoxRun &R = runs[size_t(i)];
        std::memset(&R, 0, sizeof(R));
        R.box = b;
        R.phys = PhysParams{p.viscosity, p.gaz_mean_free_path, p.fractal_dimension, p.density, p.temperature};
        R.lim.number_of_aggregates_limit = p.number_of_aggregates_limit;
        R.lim.n_iter_without_event_limit = p.n_iter_without_event_limit;
        R.lim.mean_monomere_per_aggregate_limit = p.mean_monomere_per_aggregate_limit;
        R.lim.physical_time_limit = p.physical_time_limit;
        R.lim.with_collisions = p.with_collisions;
        R.st = states_dev + i;
        R.tree = static_cast<double *>(tree_dev);
        R.tree_levels = tl.levels;
        for (int k = 0; k < kMaxTreeLevels; ++k) {
            R.tree_off[k] = tl.off[k];
            R.tree_len[k] = tl.len[k];
        }
    }
    if (!ok_cuda(cudaMemcpyAsync(runs_dev_, runs.data(), sizeof(BoxRun) * size_t(n), cudaMemcpyHostToDevice, s), err,
                 "upload"))
        return ST_CUDA;
    if (!ok_cuda(cudaMemcpyAsync(states_dev_, states.data(), sizeof(RunState) * size_t(n), cudaMemcpyHostToDevice, s),
                 err, "upload"))
        return ST_CUDA;
    if (!ok_cuda(cudaFuncSetAttribute(k_run<kRunThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      int(sizeof(RunSmem))), err, "cudaFuncSetAttribute"))
        return ST_CUDA;
    if (!ok_cuda(cudaStreamSynchronize(s), err, "sync")) return ST_CUDA;
    return ST_OK;
}

int BatchRunner::run(int64_t max_steps, int64_t chunk, std::string *err) {
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    const int n = int(boxes_.size());
    if (chunk <= 0) chunk = 20000;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    launches_ = 0;
    int64_t done = 0;
    int rc = ST_OK;
    for (;;) {
        int64_t steps = max_steps > 0 ? std::min(chunk, max_steps - done) : chunk;
        if (steps <= 0) break;
        k_run<kRunThreads><<<n, kRunThreads, sizeof(RunSmem), s>>>(static_cast<const BoxRun *>(runs_dev_), n,
                                                                   (long long)steps);
        ++launches_;
        if (!ok_cuda(cudaGetLastError(), err, "k_run")) {
            rc = ST_CUDA;
            break;
        }
        done += steps;
        if (max_steps > 0 && done >= max_steps) break;
        if (max_steps <= 0) {
            // until every box has met its stop criterion (or failed)
            std::vector<BoxRunStats> st;
            rc = stats(&st, err);
            if (rc != ST_OK) break;
            bool all = true;
            for (const auto &x : st) all = all && (x.finished || x.status != ST_OK);
            if (all) break;
        }
    }
    cudaEventRecord(e1, s);
    if (!ok_cuda(cudaEventSynchronize(e1), err, "k_run")) rc = ST_CUDA;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    last_ms_ = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

int BatchRunner::stats(std::vector<BoxRunStats> *out, std::string *err) {
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    const int n = int(boxes_.size());
    std::vector<RunState> st(static_cast<size_t>(n));
    if (!ok_cuda(cudaMemcpyAsync(st.data(), states_dev_, sizeof(RunState) * size_t(n), cudaMemcpyDeviceToHost, s),
                 err, "download"))
        return ST_CUDA;
    std::vector<DevScalars> sc(static_cast<size_t>(n));
    for (int i = 0; i < n; ++i) {
        const DevBox &b = *static_cast<DevBox *>(boxes_[size_t(i)]->devbox_ptr());
        if (!ok_cuda(cudaMemcpyAsync(&sc[size_t(i)], b.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, s), err,
                     "download"))
            return ST_CUDA;
    }
    if (!ok_cuda(cudaStreamSynchronize(s), err, "sync")) return ST_CUDA;
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
    }
    return ST_OK;
}

int BatchRunner::download(int box, HostState *st, std::string *err) {
    if (box < 0 || box >= size()) return ST_BAD_ARGUMENT;
    int rc = boxes_[size_t(box)]->download(st, err);
    if (rc != ST_OK) return rc;
    std::vector<BoxRunStats> s;
    rc = stats(&s, err);
    if (rc != ST_OK) return rc;
    st->time = s[size_t(box)].time;
    return ST_OK;
}

}  // namespace mcacg
