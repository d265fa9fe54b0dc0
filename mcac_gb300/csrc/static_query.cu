// Batched contact queries that allocate no device memory.
//
// Some callers cannot allocate device memory while they run: a serving loop
// that has handed the whole device to its own pool, a caller that must not
// add the implicit device synchronisation of cudaMalloc/cudaFree to its
// step, or one that runs under a fixed memory budget. For them,
// mcacg_distance_to_next_contacts_static answers the same queries as
// mcacg_distance_to_next_contacts with all of its device scratch (the query
// inputs, the results and each thread block's candidate and survivor lists)
// in one file-scope __device__ array of kStaticScratchBytes, created with
// the module. The library calls no cudaMalloc, cudaFree or other allocating
// routine on this path.
//
// Limits: at most kStaticMaxQueries queries per call; a box whose candidate
// lists (44 bytes per aggregate slot per block) do not fit the array even
// for one block is refused; fewer blocks run concurrently than on the
// allocating path when the box is large.
//
// Set-up: the first call on each device looks up the array's address with
// cudaGetSymbolAddress, with that device current, and keeps it; make that
// first call before any stream capture begins. Every call then clears the
// two words that must start at zero (the query counter and the status) with
// cudaMemsetAsync, copies the queries in, runs the kernel, copies the
// results out and waits for its stream.
//
// The array is shared by every box on a device. Calls that overlapped would
// race on it; this file serialises them with a process-wide lock, so
// concurrent calls from several host threads wait for each other.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "../../include/mcacg.h"
#include "box.cuh"
#include "device_box.hpp"
#include "static_query.hpp"

namespace mcacg {

constexpr size_t kStaticScratchBytes = size_t(32) << 20;  // 32 MiB
constexpr int kStaticMaxQueries = 1 << 16;
constexpr int kStaticSurvivors = 1 << 12;  // HBM survivors per block
constexpr int kStaticMaxDevices = 64;

namespace {

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

struct StaticScratch {
    int *header;  // [0] next query, [1] first failing status: zero at launch
    const long long *sources;
    const double *dirs;
    const double *dists;
    mcacg_contact *out;
    size_t stride;  // candidate entries per block (nslots + 1)
    char *blocks;   // per-block slices
    size_t block_bytes;
    size_t o_key, o_slot, o_order, o_prefix, o_res, o_ij, o_surv, o_sres;
};

// Slot of the live aggregate with the given label: labels are the ranks of
// the live slots in slot order. Block-wide; every thread gets the answer.
__device__ int block_slot_of_label(const DevBox &b, long long label, int *warp_tmp, int *found) {
    const int NT = blockDim.x, tid = threadIdx.x;
    const int chunk = (b.nslots + NT - 1) / NT;
    const int lo = min(b.nslots, tid * chunk), hi = min(b.nslots, lo + chunk);
    int c = 0;
    for (int i = lo; i < hi; ++i) c += b.agg_n[i] > 0;
    if (tid == 0) *found = -1;
    int total = 0;
    const int before = block_exclusive_scan(c, warp_tmp, total);
    if (label >= before && label < before + c) {
        long long r = before;
        for (int i = lo; i < hi; ++i) {
            if (b.agg_n[i] > 0) {
                if (r == label) {
                    *found = i;
                    break;
                }
                ++r;
            }
        }
    }
    __syncthreads();
    const int slot = *found;
    __syncthreads();
    return slot;
}

// Number of live slots below 'slot' (the label of a live slot).
__device__ int block_live_before(const DevBox &b, int slot, int *warp_tmp) {
    int c = 0;
    for (int i = threadIdx.x; i < slot; i += blockDim.x) c += b.agg_n[i] > 0;
    int total = 0;
    block_exclusive_scan(c, warp_tmp, total);
    return total;
}

__global__ void __launch_bounds__(kQueryThreads) k_query_static(DevBox b, StaticScratch s, int n) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    QuerySmem &sm = *reinterpret_cast<QuerySmem *>(smem_raw);
    __shared__ int q_cur, found;
    __shared__ int warp_tmp[32];
    char *mine = s.blocks + size_t(blockIdx.x) * s.block_bytes;
    b.cand_db = reinterpret_cast<double *>(mine);
    b.cand_key = reinterpret_cast<long long *>(mine + s.o_key);
    b.cand_slot = reinterpret_cast<int *>(mine + s.o_slot);
    b.cand_order = reinterpret_cast<int *>(mine + s.o_order);
    b.cand_prefix = reinterpret_cast<int *>(mine + s.o_prefix);
    b.best_res = reinterpret_cast<unsigned long long *>(mine + s.o_res);
    b.best_ij = reinterpret_cast<unsigned long long *>(mine + s.o_ij);
    b.surv = reinterpret_cast<int4 *>(mine + s.o_surv);
    b.surv_res = reinterpret_cast<double *>(mine + s.o_sres);
    b.surv_cap = kStaticSurvivors;
    for (;;) {
        if (threadIdx.x == 0) q_cur = atomicAdd(&s.header[0], 1);
        __syncthreads();
        const int q = q_cur;
        if (q >= n) break;  // block-uniform
        const long long label = s.sources[q];
        const int slot = block_slot_of_label(b, label, warp_tmp, &found);
        mcacg_contact c{CUDART_INF, -1, -1, -1, -1};
        if (slot < 0) {
            if (threadIdx.x == 0) atomicCAS(&s.header[1], 0, int(ST_BAD_ARGUMENT));
        } else {
            block_query(b, slot, Vec3{s.dirs[3 * q], s.dirs[3 * q + 1], s.dirs[3 * q + 2]}, s.dists[q], sm);
            __syncthreads();
            const QueryOut o = sm.out;
            c.distance = o.distance;
            if (o.status != ST_OK && threadIdx.x == 0) atomicCAS(&s.header[1], 0, o.status);
            if (o.moving_sphere >= 0) {
                const int other = block_live_before(b, o.other_slot, warp_tmp);
                c.moving_sphere = o.moving_sphere;
                c.other_sphere = o.other_sphere;
                c.moving_aggregate = label;
                c.other_aggregate = other;
            }
        }
        if (threadIdx.x == 0) s.out[q] = c;
        __syncthreads();
    }
}

bool ok_or(cudaError_t e, std::string *err, const char *what) {
    if (e == cudaSuccess) return true;
    if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
}

size_t round256(size_t x) { return (x + 255) & ~size_t(255); }

std::mutex g_static_lock;
void *g_static_ptr[kStaticMaxDevices] = {};

}  // namespace

int query_batch_static(DeviceBox &dev, int n_alive, int n, const int64_t *sources, const double *dirs,
                       const double *dists, mcacg_contact *out, std::string *err) {
    if (n < 0) {
        if (err) *err = "negative query count";
        return ST_BAD_ARGUMENT;
    }
    if (n > kStaticMaxQueries) {
        if (err) *err = "at most " + std::to_string(kStaticMaxQueries) + " queries per call on the static-scratch path";
        return ST_CAPACITY;
    }
    for (int k = 0; k < n; ++k)
        if (sources[k] < 0 || sources[k] >= n_alive) {
            if (err) *err = "label out of range in query " + std::to_string(k);
            return ST_BAD_ARGUMENT;
        }
    if (n == 0) return ST_OK;
    std::lock_guard<std::mutex> hold(g_static_lock);
    int device = 0;
    if (!ok_or(cudaGetDevice(&device), err, "cudaGetDevice")) return ST_CUDA;
    if (device < 0 || device >= kStaticMaxDevices) {
        if (err) *err = "device index beyond the static-scratch table";
        return ST_CAPACITY;
    }
    if (!g_static_ptr[device]) {
        void *p = nullptr;
        if (!ok_or(cudaGetSymbolAddress(&p, g_static_scratch), err, "cudaGetSymbolAddress")) return ST_CUDA;
        g_static_ptr[device] = p;
    }
    char *base = static_cast<char *>(g_static_ptr[device]);
    const DevBox &b = *static_cast<const DevBox *>(dev.devbox_ptr());
    cudaStream_t stream = static_cast<cudaStream_t>(dev.stream());

    // layout: header, inputs, results, then one slice per block
    StaticScratch s{};
    size_t off = 0;
    const size_t o_header = off;
    off += 256;
    const size_t o_src = off;
    off += round256(sizeof(int64_t) * size_t(n));
    const size_t o_dirs = off;
    off += round256(3 * sizeof(double) * size_t(n));
    const size_t o_dists = off;
    off += round256(sizeof(double) * size_t(n));
    const size_t o_out = off;
    off += round256(sizeof(mcacg_contact) * size_t(n));
    s.stride = size_t(dev.nslots()) + 1;
    size_t bo = round256(8 * s.stride);
    s.o_key = bo;
    bo += round256(8 * s.stride);
    s.o_slot = bo;
    bo += round256(4 * s.stride);
    s.o_order = bo;
    bo += round256(4 * s.stride);
    s.o_prefix = bo;
    bo += round256(4 * s.stride);
    s.o_res = bo;
    bo += round256(8 * s.stride);
    s.o_ij = bo;
    bo += round256(8 * s.stride);
    s.o_surv = bo;
    bo += round256(sizeof(int4) * size_t(kStaticSurvivors));
    s.o_sres = bo;
    bo += round256(sizeof(double) * size_t(kStaticSurvivors));
    s.block_bytes = bo;
    const size_t fit = off < kStaticScratchBytes ? (kStaticScratchBytes - off) / s.block_bytes : 0;
    if (fit < 1) {
        if (err)
            *err = "box too large for the static scratch: " + std::to_string(s.block_bytes) +
                   " bytes per block after " + std::to_string(off) + " bytes of queries, " +
                   std::to_string(kStaticScratchBytes) + " in all";
        return ST_CAPACITY;
    }
    int n_sm = 0, per_sm = 0;
    if (!ok_or(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, device), err, "device attribute"))
        return ST_CUDA;
    if (!ok_or(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_query_static, kQueryThreads,
                                                             sizeof(QuerySmem)),
               err, "occupancy"))
        return ST_CUDA;
    size_t blocks = size_t(std::max(1, per_sm)) * size_t(std::max(1, n_sm));
    blocks = std::min(blocks, std::min(fit, size_t(n)));
    s.header = reinterpret_cast<int *>(base + o_header);
    s.sources = reinterpret_cast<const long long *>(base + o_src);
    s.dirs = reinterpret_cast<const double *>(base + o_dirs);
    s.dists = reinterpret_cast<const double *>(base + o_dists);
    s.out = reinterpret_cast<mcacg_contact *>(base + o_out);
    s.blocks = base + off;

    int status = 0;
    bool ok = ok_or(cudaMemsetAsync(base + o_header, 0, 2 * sizeof(int), stream), err, "clear counter") &&
              ok_or(cudaMemcpyAsync(base + o_src, sources, sizeof(int64_t) * size_t(n), cudaMemcpyHostToDevice,
                                    stream),
                    err, "upload sources") &&
              ok_or(cudaMemcpyAsync(base + o_dirs, dirs, 3 * sizeof(double) * size_t(n), cudaMemcpyHostToDevice,
                                    stream),
                    err, "upload directions") &&
              ok_or(cudaMemcpyAsync(base + o_dists, dists, sizeof(double) * size_t(n), cudaMemcpyHostToDevice,
                                    stream),
                    err, "upload distances");
    if (ok) {
        k_query_static<<<unsigned(blocks), kQueryThreads, sizeof(QuerySmem), stream>>>(b, s, n);
        ok = ok_or(cudaGetLastError(), err, "k_query_static") &&
             ok_or(cudaMemcpyAsync(out, base + o_out, sizeof(mcacg_contact) * size_t(n), cudaMemcpyDeviceToHost,
                                   stream),
                   err, "download results") &&
             ok_or(cudaMemcpyAsync(&status, base + o_header + sizeof(int), sizeof(int), cudaMemcpyDeviceToHost,
                                   stream),
                   err, "download status") &&
             ok_or(cudaStreamSynchronize(stream), err, "k_query_static");
    }
    if (!ok) return ST_CUDA;
    if (status != ST_OK && err) *err = "a contact query failed with status " + std::to_string(status);
    return status;
}

}  // namespace mcacg
