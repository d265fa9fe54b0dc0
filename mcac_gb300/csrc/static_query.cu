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
// Limits: at most kStaticMaxQueries queries per call; each thread block
// keeps kStaticSurvivors refined sphere pairs in the array, as many as the
// allocating path keeps, so a query fails with MCACG_ERR_CAPACITY here
// exactly when it does there; a box whose candidate lists (44 bytes per
// aggregate slot) and survivor lists (384 KiB) do not fit the array for one
// block is refused; fewer blocks run concurrently than on the allocating
// path (about 32 MiB / (384 KiB + 44 B x slots)).
//
// Set-up: every call looks up the array's address on the current device
// with cudaGetSymbolAddress (it allocates nothing, and a context made again
// after a device reset gets the new address); the first call on a device
// also loads the module, so make it before any stream capture begins. The
// labels are turned into slots on the host before the call and the hit
// slot back into a label after it. Every call then clears the two words
// that must start at zero (the query counter and the status) with
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
constexpr int kStaticSurvivors = 1 << 14;  // HBM survivors per block, as on the allocating path

namespace {

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

struct StaticScratch {
    int *header;  // [0] next query, [1] first failing status: zero at launch
    const int *slots;
    const double *dirs;
    const double *dists;
    mcacg_contact *out;
    size_t stride;  // candidate entries per block (nslots + 1)
    char *blocks;   // per-block slices
    size_t block_bytes;
    size_t o_key, o_slot, o_order, o_prefix, o_res, o_ij, o_surv, o_sres;
};

__global__ void __launch_bounds__(kQueryThreads) k_query_static(DevBox b, StaticScratch s, int n) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    QuerySmem &sm = *reinterpret_cast<QuerySmem *>(smem_raw);
    __shared__ int q_cur;
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
        const int slot = s.slots[q];
        // the host fills in the labels: moving_aggregate from the query,
        // other_aggregate from the hit slot written here
        mcacg_contact c{CUDART_INF, -1, -1, -1, -1};
        block_query(b, slot, Vec3{s.dirs[3 * q], s.dirs[3 * q + 1], s.dirs[3 * q + 2]}, s.dists[q], sm);
        __syncthreads();
        const QueryOut o = sm.out;
        c.distance = o.distance;
        if (o.status != ST_OK && threadIdx.x == 0) atomicCAS(&s.header[1], 0, o.status);
        if (o.moving_sphere >= 0) {
            c.moving_sphere = o.moving_sphere;
            c.other_sphere = o.other_sphere;
            c.other_aggregate = o.other_slot;
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

}  // namespace

int query_batch_static(DeviceBox &dev, int n, const int *slots, const double *dirs, const double *dists,
                       mcacg_contact *out, std::string *err) {
    if (n < 0) {
        if (err) *err = "negative query count";
        return ST_BAD_ARGUMENT;
    }
    if (n > kStaticMaxQueries) {
        if (err) *err = "at most " + std::to_string(kStaticMaxQueries) + " queries per call on the static-scratch path";
        return ST_CAPACITY;
    }
    for (int k = 0; k < n; ++k)
        if (slots[k] < 0 || slots[k] >= dev.nslots()) {
            if (err) *err = "slot out of range in query " + std::to_string(k);
            return ST_BAD_ARGUMENT;
        }
    if (n == 0) return ST_OK;
    std::lock_guard<std::mutex> hold(g_static_lock);
    int device = 0;
    if (!ok_or(cudaGetDevice(&device), err, "cudaGetDevice")) return ST_CUDA;
    // the array's address in the current context (no allocation)
    void *addr = nullptr;
    if (!ok_or(cudaGetSymbolAddress(&addr, g_static_scratch), err, "cudaGetSymbolAddress")) return ST_CUDA;
    char *base = static_cast<char *>(addr);
    const DevBox &b = *static_cast<const DevBox *>(dev.devbox_ptr());
    cudaStream_t stream = static_cast<cudaStream_t>(dev.stream());

    // layout: header, inputs, results, then one slice per block
    StaticScratch s{};
    size_t off = 0;
    const size_t o_header = off;
    off += 256;
    const size_t o_src = off;
    off += round256(sizeof(int) * size_t(n));
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
    s.slots = reinterpret_cast<const int *>(base + o_src);
    s.dirs = reinterpret_cast<const double *>(base + o_dirs);
    s.dists = reinterpret_cast<const double *>(base + o_dists);
    s.out = reinterpret_cast<mcacg_contact *>(base + o_out);
    s.blocks = base + off;

    int status = 0;
    bool ok = ok_or(cudaMemsetAsync(base + o_header, 0, 2 * sizeof(int), stream), err, "clear counter") &&
              ok_or(cudaMemcpyAsync(base + o_src, slots, sizeof(int) * size_t(n), cudaMemcpyHostToDevice, stream),
                    err, "upload slots") &&
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
