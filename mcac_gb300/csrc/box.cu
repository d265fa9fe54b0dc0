// Single-box kernels and the host-side management of a device-resident box.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>

#include "box.cuh"
#include "device_box.hpp"
#include "merge.cuh"

namespace mcacg {

// ------------------------------------------------------------------ kernels
__global__ void __launch_bounds__(kQueryThreads) k_query(DevBox b, int src, double dx, double dy, double dz,
                                                         double dist, QueryOut *out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    QuerySmem &sm = *reinterpret_cast<QuerySmem *>(smem_raw);
    block_query(b, src, Vec3{dx, dy, dz}, dist, sm);
    if (threadIdx.x == 0) *out = sm.out;
}

// Many independent contact queries on one unchanged box. Each block takes
// the next query from a shared counter (queries differ widely in cost) and
// runs it with its own slice of the candidate and survivor scratch; the box
// state is only read.
struct QueryIn {
    double dx, dy, dz, dist;
    int slot, pad;
};
struct BatchScratch {
    int *next;      // query counter, zero at launch
    size_t stride;  // candidate entries per block (nslots + 1)
    int surv_cap;   // HBM survivors per block
    double *cand_db;
    long long *cand_key;
    int *cand_slot, *cand_order, *cand_prefix;
    unsigned long long *best_res, *best_ij;
    int4 *surv;
    double *surv_res;
};
constexpr int kBatchThreads = 256;  // two blocks per SM at 128 registers a thread
template <int NT>
__global__ void __launch_bounds__(NT) k_query_batch(DevBox b, BatchScratch s, int n, const QueryIn *in,
                                                    QueryOut *out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    QuerySmem &sm = *reinterpret_cast<QuerySmem *>(smem_raw);
    __shared__ int q_cur;
    const size_t c0 = size_t(blockIdx.x) * s.stride;
    b.cand_db = s.cand_db + c0;
    b.cand_key = s.cand_key + c0;
    b.cand_slot = s.cand_slot + c0;
    b.cand_order = s.cand_order + c0;
    b.cand_prefix = s.cand_prefix + c0;
    b.best_res = s.best_res + c0;
    b.best_ij = s.best_ij + c0;
    b.surv = s.surv + size_t(blockIdx.x) * size_t(s.surv_cap);
    b.surv_res = s.surv_res + size_t(blockIdx.x) * size_t(s.surv_cap);
    b.surv_cap = s.surv_cap;
    for (;;) {
        if (threadIdx.x == 0) q_cur = atomicAdd(s.next, 1);
        __syncthreads();
        const int q = q_cur;
        if (q >= n) break;  // block-uniform
        const QueryIn qi = in[q];
        block_query(b, qi.slot, Vec3{qi.dx, qi.dy, qi.dz}, qi.dist, sm);
        if (threadIdx.x == 0) out[q] = sm.out;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kQueryThreads) k_translate(DevBox b, int slot, double vx, double vy, double vz) {
    __shared__ double refpos[3];
    block_translate(b, slot, Vec3{vx, vy, vz}, refpos);
}

__global__ void __launch_bounds__(kQueryThreads) k_merge(DevBox b, int ms, int os, int mslot, int oslot,
                                                         MergeOut *out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    MergeSmem &sm = *reinterpret_cast<MergeSmem *>(smem_raw);
    block_merge(b, ms, os, mslot, oslot, sm, out);
}

struct FieldUpdate {
    double v[21];
};
__global__ void k_set_fields(DevBox b, int slot, FieldUpdate u, unsigned mask) {
    int f = threadIdx.x;
    if (f < AGG_NFIELDS && (mask >> f) & 1u) A(b, f, slot) = u.v[f];
}

// Verlet and fine grids from the aggregate positions: clear the cells, drop
// every live slot into its cells (in any order: the scan key restores the
// reference's order), then link the fine lists backwards.
__global__ void k_grid_clear(DevBox b) {
    const int stride = gridDim.x * blockDim.x, t = blockIdx.x * blockDim.x + threadIdx.x;
    for (int c = t; c < b.n_cells; c += stride) b.cell_n[c] = 0;
    if (b.fine_div > 0) {
        const int nf3 = b.fine_div * b.fine_div * b.fine_div;
        for (int c = t; c < nf3; c += stride) b.fine_head[c] = -1;
        for (int a = t; a < b.nslots; a += stride) b.fine_cell[a] = -1;
    }
}
__global__ void k_grid_fill(DevBox b) {
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < b.nslots; a += gridDim.x * blockDim.x) {
        if (b.agg_n[a] == 0) continue;
        const int c = cell_of(b, agg_pos(b, a));
        b.agg_cell[a] = c;
        b.agg_f4[a] = make_float4(float(A(b, AGG_X, a)), float(A(b, AGG_Y, a)), float(A(b, AGG_Z, a)),
                                  float(A(b, AGG_RMAX, a)));
        const int k = atomicAdd(&b.cell_n[c], 1);
        if (k < b.cell_cap) {
            b.cell_items[size_t(c) * b.cell_cap + k] = a;
            b.cell_pos[a] = k;
        } else {
            b.sc->cell_overflow = 1;
            b.sc->status = ST_CAPACITY;
        }
        if (b.fine_div > 0) {
            const int fc = fine_cell_of(b, agg_pos(b, a));
            b.fine_cell[a] = fc;
            b.fine_next[a] = atomicExch(&b.fine_head[fc], a);
        }
    }
}
// back links of the fine lists built by k_grid_fill
__global__ void k_fine_link(DevBox b) {
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < b.nslots; a += gridDim.x * blockDim.x) {
        const int c = b.fine_cell[a];
        if (c < 0) continue;
        const int n = b.fine_next[a];
        if (n >= 0) b.fine_prev[n] = a;
        if (b.fine_head[c] == a) b.fine_prev[a] = -1;
    }
}
__global__ void k_refresh_f4(DevBox b) {
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < b.nslots; a += gridDim.x * blockDim.x)
        b.agg_f4[a] = make_float4(float(A(b, AGG_X, a)), float(A(b, AGG_Y, a)), float(A(b, AGG_Z, a)),
                                  float(A(b, AGG_RMAX, a)));
}

// Loading a state: the sphere and aggregate tables go straight to their
// places; the integer arrays (owning slot per sphere, spheres per slot,
// member lists in slot order) are staged as 32- or 64-bit values and
// converted here, with the pool built from the member lists. Inconsistent
// input is flagged (sc->pad[0] = the LoadError, status BAD_ARGUMENT) and
// never read out of bounds.
enum LoadError { LOAD_OK = 0, LOAD_LABEL = 1, LOAD_COUNT = 2, LOAD_COVER = 3, LOAD_MEMBER = 4 };
struct LoadStage {
    const void *label, *count, *members;
    int wide;     // 64-bit integers
    int dead_ok;  // slots without spheres are allowed
};
__device__ __forceinline__ long long load_int(const void *p, int wide, int i) {
    return wide ? static_cast<const long long *>(p)[i] : static_cast<long long>(static_cast<const int *>(p)[i]);
}
__device__ __forceinline__ void load_fail(DevBox &b, int code) {
    atomicCAS(&b.sc->pad[0], 0, code);
    b.sc->status = ST_BAD_ARGUMENT;
}
constexpr int kLoadScanThreads = 1024;
// spheres per slot, pool offsets (exclusive sum in slot order), live count
__global__ void __launch_bounds__(kLoadScanThreads) k_load_counts(DevBox b, LoadStage in) {
    __shared__ long long part[kLoadScanThreads];
    __shared__ int alive[kLoadScanThreads];
    __shared__ int bad;
    const int t = threadIdx.x;
    if (t == 0) bad = 0;
    __syncthreads();
    const int chunk = (b.nslots + kLoadScanThreads - 1) / kLoadScanThreads;
    const int a0 = min(b.nslots, t * chunk), a1 = min(b.nslots, a0 + chunk);
    long long sum = 0;
    int live = 0, flag = 0;
    for (int a = a0; a < a1; ++a) {
        long long n = load_int(in.count, in.wide, a);
        if (n < 0 || n > b.ns || (n == 0 && !in.dead_ok)) {
            flag = 1;
            n = 0;
        }
        sum += n;
        live += n > 0;
    }
    part[t] = sum;
    alive[t] = live;
    if (flag) atomicOr(&bad, 1);
    __syncthreads();
    if (t == 0) {
        if (bad) load_fail(b, LOAD_COUNT);
        long long run = 0;
        int n_alive = 0;
        for (int k = 0; k < kLoadScanThreads; ++k) {
            const long long v = part[k];
            part[k] = run;
            run += v;
            n_alive += alive[k];
        }
        b.sc->n_alive = n_alive;
        b.sc->pool_top = b.ns;
        if (run != b.ns) load_fail(b, LOAD_COVER);
    }
    __syncthreads();
    long long off = part[t];
    for (int a = a0; a < a1; ++a) {
        long long n = load_int(in.count, in.wide, a);
        if (n < 0 || n > b.ns || (n == 0 && !in.dead_ok)) n = 0;
        b.agg_n[a] = int(n);
        b.agg_off[a] = int(min(off, (long long)b.ns));
        off += n;
    }
}
// owning slots, pool ids and pool positions (pool entry k = member k)
__global__ void k_load_spheres(DevBox b, LoadStage in) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < b.ns; s += gridDim.x * blockDim.x) {
        long long l = load_int(in.label, in.wide, s);
        if (l < 0 || l >= b.nslots) {
            load_fail(b, LOAD_LABEL);
            l = 0;
        }
        b.sph_slot[s] = int(l);
        long long m = load_int(in.members, in.wide, s);
        if (m < 0 || m >= b.ns) {
            load_fail(b, LOAD_MEMBER);
            m = 0;
        }
        b.pool_id[0][s] = int(m);
        b.pool_pos[0][s] = make_float4(float(S(b, SPH_X, int(m))), float(S(b, SPH_Y, int(m))),
                                       float(S(b, SPH_Z, int(m))), float(S(b, SPH_R, int(m))));
    }
    for (int k = b.ns + blockIdx.x * blockDim.x + threadIdx.x; k < b.pool_cap; k += gridDim.x * blockDim.x) {
        b.pool_id[0][k] = 0;
        b.pool_pos[0][k] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}
// Storing a state: the live slots are packed in slot order (label = rank
// among the live slots, as the reference's list has them), with their member
// lists back to back, into the staging area; the host copies the pieces out.
struct PackStage {
    double *agg;       // [21][na]
    long long *count;  // [na]
    long long *label;  // [ns]
    long long *members;// [ns]
    int *rank;         // [nslots]
    int *moff;         // [nslots] first member of the slot in 'members'
    int na;
    int sel;           // live pool buffer
};
__global__ void __launch_bounds__(kLoadScanThreads) k_pack_ranks(DevBox b, PackStage out) {
    __shared__ int live_part[kLoadScanThreads];
    __shared__ int mem_part[kLoadScanThreads];
    const int t = threadIdx.x;
    const int chunk = (b.nslots + kLoadScanThreads - 1) / kLoadScanThreads;
    const int a0 = min(b.nslots, t * chunk), a1 = min(b.nslots, a0 + chunk);
    int live = 0, mem = 0;
    for (int a = a0; a < a1; ++a) {
        const int n = b.agg_n[a];
        live += n > 0;
        mem += n;
    }
    live_part[t] = live;
    mem_part[t] = mem;
    __syncthreads();
    if (t == 0) {
        int rl = 0, rm = 0;
        for (int k = 0; k < kLoadScanThreads; ++k) {
            const int l = live_part[k], m = mem_part[k];
            live_part[k] = rl;
            mem_part[k] = rm;
            rl += l;
            rm += m;
        }
    }
    __syncthreads();
    int r = live_part[t], o = mem_part[t];
    for (int a = a0; a < a1; ++a) {
        const int n = b.agg_n[a];
        out.rank[a] = n > 0 ? r : -1;
        out.moff[a] = o;
        r += n > 0;
        o += n;
    }
}
__global__ void k_pack(DevBox b, PackStage out) {
    const int stride = gridDim.x * blockDim.x, t = blockIdx.x * blockDim.x + threadIdx.x;
    const int *pool = b.pool_id[out.sel];
    for (int a = t; a < b.nslots; a += stride) {
        const int r = out.rank[a];
        if (r < 0 || r >= out.na) continue;
        const int n = b.agg_n[a];
        out.count[r] = n;
        for (int f = 0; f < AGG_NFIELDS; ++f) out.agg[size_t(f) * out.na + r] = A(b, f, a);
        const int src = b.agg_off[a], dst = out.moff[a];
        for (int k = 0; k < n && dst + k < b.ns && src + k < b.pool_cap; ++k) out.members[dst + k] = pool[src + k];
    }
    for (int s = t; s < b.ns; s += stride) out.label[s] = out.rank[b.sph_slot[s]];
}

// every member of slot a is owned by slot a
__global__ void k_load_check(DevBox b) {
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < b.nslots; a += gridDim.x * blockDim.x) {
        const int o = b.agg_off[a], e = min(b.ns, o + b.agg_n[a]);
        for (int k = o; k < e; ++k)
            if (b.sph_slot[b.pool_id[0][k]] != a) {
                load_fail(b, LOAD_MEMBER);
                break;
            }
    }
}
// ------------------------------------------------------------------- host
namespace {

bool cuda_ok(cudaError_t e, std::string *err, const char *what) {
    if (e == cudaSuccess) return true;
    if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
}

struct OutBuffers {
    QueryOut query;
    MergeOut merge;
};

}  // namespace

StateView view_of(const HostState &st, std::vector<int> *compact) {
    StateView v;
    v.n_div = st.n_div;
    v.box_length = st.box_length;
    v.maxradius = st.maxradius;
    v.time = st.time;
    v.ns = st.ns;
    v.nslots = st.nslots;
    v.sph = st.sph.data();
    v.agg = st.agg.data();
    v.sph_slot = st.sph_slot.data();
    v.agg_n = st.agg_n.data();
    v.wide = false;
    v.dead_slots = true;
    // the member lists are usually stored back to back in slot order, dead
    // slots empty; otherwise they are gathered
    bool packed = st.members.count() == size_t(st.nslots) && st.members.ids.size() == size_t(st.ns);
    for (int a = 0; packed && a < st.nslots; ++a)
        packed = st.members[size_t(a)].size() == st.agg_n[size_t(a)];
    if (packed) {
        v.members = st.members.ids.data();
    } else {
        compact->clear();
        compact->reserve(size_t(st.ns));
        for (int a = 0; a < st.nslots && a < int(st.members.count()); ++a)
            if (st.agg_n[size_t(a)] > 0)
                for (int s : st.members[size_t(a)]) compact->push_back(s);
        compact->resize(size_t(st.ns), -1);  // a short list is flagged by the load check
        v.members = compact->data();
    }
    return v;
}

int DeviceBox::create(const HostState &st, void *stream, DeviceBox **out, std::string *err) {
    std::vector<int> compact;
    const StateView v = view_of(st, &compact);
    return create(v, stream, out, err);
}

int DeviceBox::create(const StateView &st, void *stream, DeviceBox **out, std::string *err) {
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        if (err) *err = "no CUDA device";
        return ST_NO_DEVICE;
    }
    if (st.ns <= 0 || st.nslots <= 0 || st.nslots > st.ns || !st.sph || !st.agg || !st.sph_slot || !st.agg_n ||
        !st.members || !(st.box_length > 0.0) || st.n_div <= 0) {
        if (err) *err = "incomplete state";
        return ST_BAD_ARGUMENT;
    }
    DeviceBox *d = new DeviceBox();
    d->ns_ = st.ns;
    d->nslots_ = st.nslots;
    DevBox b{};
    b.L = st.box_length;
    b.n_div = st.n_div;
    b.step = double(st.n_div) / st.box_length;
    b.n_cells = st.n_div * st.n_div * st.n_div;
    b.ns = st.ns;
    b.nslots = st.nslots;
    const double *agg = st.agg;
    auto AF = [&](int f, int a) { return agg[size_t(f) * size_t(st.nslots) + size_t(a)]; };
    // FP32 screening margin: coordinates are bounded by the box plus the
    // largest aggregate; 2^-17 of that bound is >10x the FP32 error of the
    // capsule test.
    // one pass over the live slots: largest r_max, the means of lpm and
    // r_max, and the Verlet cell counts (for the cell capacity)
    double rmax_all = st.maxradius, lpm_sum = 0.0, rmax_sum = 0.0;
    int live = 0, maxc = 0;
    std::vector<int> cell_n(size_t(b.n_cells), 0);
    for (int a = 0; a < st.nslots; ++a) {
        if (st.count(a) <= 0) continue;
        const double rm = AF(AGG_RMAX, a);
        rmax_all = std::max(rmax_all, rm);
        lpm_sum += AF(AGG_LPM, a);
        rmax_sum += rm;
        ++live;
        const int ix = std::min(std::max(verlet_coord(AF(AGG_X, a), b.step), 0), b.n_div - 1);
        const int iy = std::min(std::max(verlet_coord(AF(AGG_Y, a), b.step), 0), b.n_div - 1);
        const int iz = std::min(std::max(verlet_coord(AF(AGG_Z, a), b.step), 0), b.n_div - 1);
        maxc = std::max(maxc, ++cell_n[size_t((ix * b.n_div + iy) * b.n_div + iz)]);
    }
    b.margin = (3.0 * st.box_length + 4.0 * rmax_all) * (1.0 / 131072.0);
    // fine discovery grid, when finer than the Verlet grid: a query visits
    // the cells covering its swept box, about lpm/2 + 2 (r_max + max r_max)
    // per axis on average; cells of 0.6 of that balance the cells visited
    // against the aggregates screened. At least 2 max r_max and L/128.
    {
        const double extent = live ? 0.5 * lpm_sum / live + 2.0 * (rmax_sum / live + rmax_all) : 0.0;
        const double h = std::max({2.0 * rmax_all, st.box_length / double(kFineMaxDiv), 0.6 * extent});
        const double nf = std::floor(st.box_length / h);
        b.fine_div = (nf > double(st.n_div) && nf <= double(kFineMaxDiv)) ? int(nf) : 0;
        b.fine_step = b.fine_div > 0 ? double(b.fine_div) / st.box_length : 0.0;
    }
    // grid capacity
    int avg = (st.nslots + b.n_cells - 1) / b.n_cells;
    b.cell_cap = std::max({64, 2 * maxc, 8 * avg});
    b.pool_cap = 2 * st.ns + 1024;
    b.surv_cap = 1 << 16;
    // contact pairs inside one aggregate: equal spheres touch at most 12
    // others (the kissing number), so at most 6 pairs per sphere; the
    // merge reports a capacity error beyond 8 per sphere
    b.pair_cap = 8 * st.ns + 1024;

    // all arrays of the box are carved from one allocation: a sizing pass,
    // one cudaMalloc, then the carving pass
    size_t arena_bytes = 0;
    char *arena = nullptr;
    bool sizing = true;
    auto alloc = [&](void **p, size_t bytes) -> bool {
        size_t need = (std::max<size_t>(bytes, 16) + 255) & ~size_t(255);
        if (sizing) {
            *p = nullptr;
        } else {
            *p = arena + arena_bytes;
        }
        arena_bytes += need;
        return true;
    };
    bool ok = true;
    for (int pass = 0; pass < 2; ++pass) {
    if (pass == 1) {
        if (!cuda_ok(cudaMalloc((void **)&arena, arena_bytes), err, "cudaMalloc")) {
            delete d;
            return ST_CUDA;
        }
        d->allocations_.push_back(arena);
        sizing = false;
        arena_bytes = 0;
    }
    ok = ok && alloc((void **)&b.sph, sizeof(double) * 9 * size_t(st.ns));
    ok = ok && alloc((void **)&b.sph_slot, sizeof(int) * size_t(st.ns));
    ok = ok && alloc((void **)&b.agg, sizeof(double) * 21 * size_t(st.nslots));
    ok = ok && alloc((void **)&b.agg_n, sizeof(int) * size_t(st.nslots));
    ok = ok && alloc((void **)&b.agg_off, sizeof(int) * size_t(st.nslots));
    ok = ok && alloc((void **)&b.agg_cell, sizeof(int) * size_t(st.nslots));
    ok = ok && alloc((void **)&b.agg_f4, sizeof(float4) * size_t(st.nslots));
    for (int k = 0; k < 2; ++k) {
        ok = ok && alloc((void **)&b.pool_id[k], sizeof(int) * size_t(b.pool_cap));
        ok = ok && alloc((void **)&b.pool_pos[k], sizeof(float4) * size_t(b.pool_cap));
    }
    ok = ok && alloc((void **)&b.cell_n, sizeof(int) * size_t(b.n_cells));
    ok = ok && alloc((void **)&b.cell_pos, sizeof(int) * size_t(st.nslots));
    if (b.fine_div > 0) {
        const size_t nf3 = size_t(b.fine_div) * size_t(b.fine_div) * size_t(b.fine_div);
        ok = ok && alloc((void **)&b.fine_head, sizeof(int) * nf3);
        ok = ok && alloc((void **)&b.fine_next, sizeof(int) * size_t(st.nslots));
        ok = ok && alloc((void **)&b.fine_prev, sizeof(int) * size_t(st.nslots));
        ok = ok && alloc((void **)&b.fine_cell, sizeof(int) * size_t(st.nslots));
    }
    ok = ok && alloc((void **)&b.cell_items, sizeof(int) * size_t(b.n_cells) * size_t(b.cell_cap));
    ok = ok && alloc((void **)&b.sc, sizeof(DevScalars));
    ok = ok && alloc((void **)&b.surv, sizeof(int4) * size_t(b.surv_cap));
    ok = ok && alloc((void **)&b.surv_res, sizeof(double) * size_t(b.surv_cap));
    // the merge's pair scratch is one block (32 B per pair), which also
    // stages a packed state on its way to the host
    {
        char *pairs = nullptr;
        const size_t pc = size_t(b.pair_cap);
        ok = ok && alloc((void **)&pairs, 32 * pc);
        b.pair_i = reinterpret_cast<int *>(pairs);
        b.pair_j = b.pair_i + pc;
        b.pair_tmp_i = b.pair_j + pc;
        b.pair_tmp_j = b.pair_tmp_i + pc;
        b.pair_d = reinterpret_cast<double *>(pairs + 16 * pc);
        b.pair_tmp_d = b.pair_d + pc;
        d->stage_ = pairs;
        d->stage_bytes_ = 32 * pc;
    }
    ok = ok && alloc((void **)&b.row_cnt, sizeof(int) * (size_t(std::max(st.ns, st.nslots)) + 2));
    ok = ok && alloc((void **)&b.work, sizeof(double) * 8 * size_t(st.ns));
    ok = ok && alloc((void **)&b.counters, sizeof(int) * 8);
    const size_t nc1 = size_t(st.nslots) + 1;
    ok = ok && alloc((void **)&b.cand_db, sizeof(double) * nc1);
    ok = ok && alloc((void **)&b.cand_key, sizeof(long long) * nc1);
    ok = ok && alloc((void **)&b.cand_slot, sizeof(int) * nc1);
    ok = ok && alloc((void **)&b.cand_order, sizeof(int) * nc1);
    ok = ok && alloc((void **)&b.cand_prefix, sizeof(int) * nc1);
    ok = ok && alloc((void **)&b.best_res, sizeof(unsigned long long) * nc1);
    ok = ok && alloc((void **)&b.best_ij, sizeof(unsigned long long) * nc1);
    }  // sizing / carving passes
    if (stream) {
        d->stream_ = stream;
    } else {
        cudaStream_t s;
        if (!cuda_ok(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), err, "cudaStreamCreate")) {
            delete d;
            return ST_CUDA;
        }
        d->stream_ = s;
        d->own_stream_ = true;
    }
    // upload: the tables straight to their places, the integer arrays to
    // the box's work area (64 B per sphere; 16 B per sphere and 8 B per slot
    // at most are needed), converted and checked there by the load kernels
    DevScalars sc{};
    sc.maxradius = st.maxradius;
    sc.time = st.time;
    sc.pool_sel = 0;
    const size_t iw = st.wide ? 8 : 4;
    char *stage = reinterpret_cast<char *>(b.work);
    LoadStage in{stage, stage + 2 * iw * size_t(st.ns), stage + iw * size_t(st.ns), st.wide ? 1 : 0,
                 st.dead_slots ? 1 : 0};
    // copies on the box's own stream (boxes of a batch are built in parallel,
    // each on a stream of its own); the host arrays stay alive until the
    // status read below synchronises the stream
    cudaStream_t s = static_cast<cudaStream_t>(d->stream_);
    auto put = [&](const void *dst, const void *src, size_t bytes) {
        return cuda_ok(cudaMemcpyAsync(const_cast<void *>(dst), src, bytes, cudaMemcpyHostToDevice, s), err, "upload");
    };
    ok = ok && put(b.sph, st.sph, sizeof(double) * 9 * size_t(st.ns)) &&
         put(b.agg, st.agg, sizeof(double) * 21 * size_t(st.nslots)) && put(in.label, st.sph_slot, iw * size_t(st.ns)) &&
         put(in.members, st.members, iw * size_t(st.ns)) && put(in.count, st.agg_n, iw * size_t(st.nslots)) &&
         put(b.sc, &sc, sizeof(sc));
    if (!ok) {
        delete d;
        return ST_CUDA;
    }
    {
        const int blocks = std::min(1024, (std::max(st.ns, st.nslots) + 255) / 256);
        k_load_counts<<<1, kLoadScanThreads, 0, s>>>(b, in);
        k_load_spheres<<<blocks, 256, 0, s>>>(b, in);
        k_load_check<<<blocks, 256, 0, s>>>(b);
        if (!cuda_ok(cudaGetLastError(), err, "state load")) {
            delete d;
            return ST_CUDA;
        }
        DevScalars got;
        if (!cuda_ok(cudaMemcpyAsync(&got, b.sc, sizeof(got), cudaMemcpyDeviceToHost, s), err, "status") ||
            !cuda_ok(cudaStreamSynchronize(s), err, "sync")) {
            delete d;
            return ST_CUDA;
        }
        if (got.status != ST_OK) {
            static const char *const what[] = {"state rejected", "sphere label out of range",
                                                "bad sphere count of an aggregate",
                                                "member lists do not cover every sphere once",
                                                "member list inconsistent with sphere labels"};
            const int code = got.pad[0];
            if (err) *err = what[(code >= 0 && code <= LOAD_MEMBER) ? code : 0];
            delete d;
            return ST_BAD_ARGUMENT;
        }
    }
    d->devbox_ = new DevBox(b);
    int rc = d->rebuild_grid(b.cell_cap, err);
    if (rc != ST_OK) {
        delete d;
        return rc;
    }
    *out = d;
    return ST_OK;
}

void DeviceBox::set_profiling(bool on) {
    if (on && !ev_[0]) {
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        ev_[0] = a;
        ev_[1] = b;
    }
    profiling_ = on;
}

Profile DeviceBox::take_profile() {
    Profile p = prof_;
    prof_ = Profile();
    return p;
}

DeviceBox::~DeviceBox() {
    if (stream_) cudaStreamSynchronize(static_cast<cudaStream_t>(stream_));
    for (void *e : ev_)
        if (e) cudaEventDestroy(static_cast<cudaEvent_t>(e));
    for (void *p : allocations_) cudaFree(p);
    if (batch_mem_) cudaFree(batch_mem_);
    if (host_out_) cudaFreeHost(host_out_);
    if (own_stream_ && stream_) cudaStreamDestroy(static_cast<cudaStream_t>(stream_));
    delete static_cast<DevBox *>(devbox_);
}

int DeviceBox::set_stream(void *stream) {
    if (stream_) cudaStreamSynchronize(static_cast<cudaStream_t>(stream_));
    if (own_stream_ && stream_) cudaStreamDestroy(static_cast<cudaStream_t>(stream_));
    own_stream_ = false;
    stream_ = stream;
    if (!stream_) {
        cudaStream_t s;
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return ST_CUDA;
        stream_ = s;
        own_stream_ = true;
    }
    return ST_OK;
}

int DeviceBox::sync(std::string *err) {
    if (!cuda_ok(cudaStreamSynchronize(static_cast<cudaStream_t>(stream_)), err, "sync")) return ST_CUDA;
    return ST_OK;
}

int DeviceBox::check_status(std::string *err) {
    DevBox &b = *static_cast<DevBox *>(devbox_);
    DevScalars sc;
    if (!cuda_ok(cudaMemcpyAsync(&sc, b.sc, sizeof(sc), cudaMemcpyDeviceToHost, static_cast<cudaStream_t>(stream_)), err,
                 "status"))
        return ST_CUDA;
    if (!cuda_ok(cudaStreamSynchronize(static_cast<cudaStream_t>(stream_)), err, "sync")) return ST_CUDA;
    return sc.status;
}

int DeviceBox::rebuild_grid(int cap, std::string *err) {
    DevBox &b = *static_cast<DevBox *>(devbox_);
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    if (cap != b.cell_cap) {
        int *items = nullptr;
        if (!cuda_ok(cudaMalloc(&items, sizeof(int) * size_t(b.n_cells) * size_t(cap)), err, "cudaMalloc")) return ST_CUDA;
        // the first grid lives in the box's arena; a regrown one is its own allocation
        auto it = std::find(allocations_.begin(), allocations_.end(), (void *)b.cell_items);
        if (it != allocations_.end()) {
            cudaFree(*it);
            *it = items;
        } else {
            allocations_.push_back(items);
        }
        b.cell_items = items;
        b.cell_cap = cap;
    }
    // clear the overflow flag and status
    DevScalars sc;
    if (!cuda_ok(cudaMemcpyAsync(&sc, b.sc, sizeof(sc), cudaMemcpyDeviceToHost, s), err, "status")) return ST_CUDA;
    if (!cuda_ok(cudaStreamSynchronize(s), err, "sync")) return ST_CUDA;
    sc.cell_overflow = 0;
    if (sc.status == ST_CAPACITY) sc.status = ST_OK;
    if (!cuda_ok(cudaMemcpyAsync(b.sc, &sc, sizeof(sc), cudaMemcpyHostToDevice, s), err, "status")) return ST_CUDA;
    const int slot_blocks = std::min(1024, (b.nslots + 255) / 256);
    const int nf3 = b.fine_div * b.fine_div * b.fine_div;
    const int clear_blocks = std::min(1024, (std::max({b.n_cells, nf3, b.nslots}) + 255) / 256);
    k_grid_clear<<<clear_blocks, 256, 0, s>>>(b);
    k_grid_fill<<<slot_blocks, 256, 0, s>>>(b);
    if (b.fine_div > 0) k_fine_link<<<slot_blocks, 256, 0, s>>>(b);
    if (!cuda_ok(cudaGetLastError(), err, "grid build")) return ST_CUDA;
    int st = check_status(err);
    if (st == ST_CAPACITY) return rebuild_grid(cap * 2, err);
    return st;
}

// The mapped host buffer of the one-at-a-time query and merge results, made
// on first use (a batch's boxes never need one), and the kernels' shared
// memory limits, set once per process.
int DeviceBox::ensure_out_buffers(std::string *err) {
    if (host_out_) return ST_OK;
    static bool attrs = false;
    if (!attrs) {
        if (!cuda_ok(cudaFuncSetAttribute(k_query, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(QuerySmem))),
                     err, "cudaFuncSetAttribute") ||
            !cuda_ok(cudaFuncSetAttribute(k_merge, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(MergeSmem))),
                     err, "cudaFuncSetAttribute"))
            return ST_CUDA;
        attrs = true;
    }
    if (!cuda_ok(cudaHostAlloc(&host_out_, sizeof(OutBuffers), cudaHostAllocMapped), err, "cudaHostAlloc")) {
        host_out_ = nullptr;
        return ST_CUDA;
    }
    if (!cuda_ok(cudaHostGetDevicePointer(&dev_out_, host_out_, 0), err, "cudaHostGetDevicePointer")) return ST_CUDA;
    return ST_OK;
}

int DeviceBox::query(int src_slot, const double dir[3], double dist, QueryResult *out, std::string *err) {
    if (ensure_out_buffers(err) != ST_OK) return ST_CUDA;
    DevBox &b = *static_cast<DevBox *>(devbox_);
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    OutBuffers *ho = static_cast<OutBuffers *>(host_out_);
    OutBuffers *dout = static_cast<OutBuffers *>(dev_out_);
    if (profiling_) cudaEventRecord(static_cast<cudaEvent_t>(ev_[0]), s);
    k_query<<<1, kQueryThreads, sizeof(QuerySmem), s>>>(b, src_slot, dir[0], dir[1], dir[2], dist, &dout->query);
    if (profiling_) cudaEventRecord(static_cast<cudaEvent_t>(ev_[1]), s);
    if (!cuda_ok(cudaGetLastError(), err, "k_query")) return ST_CUDA;
    if (!cuda_ok(cudaStreamSynchronize(s), err, "k_query")) return ST_CUDA;
    const QueryOut &q = ho->query;
    if (profiling_) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, static_cast<cudaEvent_t>(ev_[0]), static_cast<cudaEvent_t>(ev_[1]));
        prof_.queries += 1;
        prof_.query_ms += ms;
        prof_.mov_spheres += q.n_mov;
        prof_.scanned += q.n_scanned;
        prof_.cells += q.n_cells;
        prof_.candidates += q.n_candidates;
        prof_.cand_spheres += q.n_cand_spheres;
        prof_.refined += q.n_pairs_refined;
    }
    out->n_scanned = q.n_scanned;
    out->n_cells = q.n_cells;
    out->n_cand_spheres = q.n_cand_spheres;
    out->n_mov = q.n_mov;
    out->distance = q.distance;
    out->moving_sphere = q.moving_sphere;
    out->other_sphere = q.other_sphere;
    out->other_slot = q.other_slot;
    out->status = q.status;
    out->n_candidates = q.n_candidates;
    out->n_pairs_refined = q.n_pairs_refined;
    if (q.status != ST_OK && err) *err = "contact query failed with status " + std::to_string(q.status);
    return q.status;
}

int DeviceBox::query_batch(int n, const int *slots, const double *dirs, const double *dists, QueryResult *out,
                           double *kernel_ms, std::string *err) {
    if (kernel_ms) *kernel_ms = 0.0;
    if (n <= 0) return ST_OK;
    for (int k = 0; k < n; ++k)
        if (slots[k] < 0 || slots[k] >= nslots_) {
            if (err) *err = "query slot out of range";
            return ST_BAD_ARGUMENT;
        }
    DevBox &b = *static_cast<DevBox *>(devbox_);
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    int dev = 0, n_sm = 0, per_sm = 0;
    if (!cuda_ok(cudaGetDevice(&dev), err, "cudaGetDevice")) return ST_CUDA;
    if (!cuda_ok(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev), err, "device attribute"))
        return ST_CUDA;
    if (!cuda_ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_query_batch<kBatchThreads>, kBatchThreads,
                                                               sizeof(QuerySmem)),
                 err, "occupancy"))
        return ST_CUDA;
    const int blocks = std::max(1, std::min(n, std::max(1, per_sm) * std::max(1, n_sm)));

    // scratch layout: counter, inputs, outputs, then per-block candidate and
    // survivor slices
    BatchScratch sc{};
    sc.stride = size_t(nslots_) + 1;
    sc.surv_cap = 1 << 14;
    const size_t nb = size_t(blocks), ncand = nb * sc.stride, nsurv = nb * size_t(sc.surv_cap);
    size_t off = 0;
    auto carve = [&](size_t bytes) {
        size_t at = off;
        off += (std::max<size_t>(bytes, 16) + 255) & ~size_t(255);
        return at;
    };
    const size_t o_next = carve(sizeof(int)), o_in = carve(sizeof(QueryIn) * size_t(n)),
                 o_out = carve(sizeof(QueryOut) * size_t(n)), o_db = carve(8 * ncand), o_key = carve(8 * ncand),
                 o_slot = carve(4 * ncand), o_order = carve(4 * ncand), o_prefix = carve(4 * ncand),
                 o_res = carve(8 * ncand), o_ij = carve(8 * ncand), o_surv = carve(sizeof(int4) * nsurv),
                 o_sres = carve(8 * nsurv);
    if (off > batch_bytes_) {
        if (batch_mem_) {
            cudaStreamSynchronize(s);
            cudaFree(batch_mem_);
            batch_mem_ = nullptr;
            batch_bytes_ = 0;
        }
        if (!cuda_ok(cudaMalloc(&batch_mem_, off), err, "cudaMalloc (query batch)")) return ST_CUDA;
        batch_bytes_ = off;
    }
    char *base = static_cast<char *>(batch_mem_);
    sc.next = reinterpret_cast<int *>(base + o_next);
    sc.cand_db = reinterpret_cast<double *>(base + o_db);
    sc.cand_key = reinterpret_cast<long long *>(base + o_key);
    sc.cand_slot = reinterpret_cast<int *>(base + o_slot);
    sc.cand_order = reinterpret_cast<int *>(base + o_order);
    sc.cand_prefix = reinterpret_cast<int *>(base + o_prefix);
    sc.best_res = reinterpret_cast<unsigned long long *>(base + o_res);
    sc.best_ij = reinterpret_cast<unsigned long long *>(base + o_ij);
    sc.surv = reinterpret_cast<int4 *>(base + o_surv);
    sc.surv_res = reinterpret_cast<double *>(base + o_sres);
    QueryIn *d_in = reinterpret_cast<QueryIn *>(base + o_in);
    QueryOut *d_out = reinterpret_cast<QueryOut *>(base + o_out);

    std::vector<QueryIn> hin(static_cast<size_t>(n));
    for (int k = 0; k < n; ++k)
        hin[size_t(k)] = QueryIn{dirs[3 * k], dirs[3 * k + 1], dirs[3 * k + 2], dists[k], slots[k], 0};
    std::vector<QueryOut> hout(static_cast<size_t>(n));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (!cuda_ok(cudaEventCreate(&e0), err, "cudaEventCreate")) return ST_CUDA;
    if (!cuda_ok(cudaEventCreate(&e1), err, "cudaEventCreate")) {
        cudaEventDestroy(e0);
        return ST_CUDA;
    }
    bool ok = cuda_ok(cudaMemcpyAsync(d_in, hin.data(), sizeof(QueryIn) * size_t(n), cudaMemcpyHostToDevice, s), err,
                      "query upload") &&
              cuda_ok(cudaMemsetAsync(sc.next, 0, sizeof(int), s), err, "query counter");
    if (ok) {
        cudaEventRecord(e0, s);
        k_query_batch<kBatchThreads><<<blocks, kBatchThreads, sizeof(QuerySmem), s>>>(b, sc, n, d_in, d_out);
        cudaEventRecord(e1, s);
        ok = cuda_ok(cudaGetLastError(), err, "k_query_batch") &&
             cuda_ok(cudaMemcpyAsync(hout.data(), d_out, sizeof(QueryOut) * size_t(n), cudaMemcpyDeviceToHost, s),
                     err, "query download") &&
             cuda_ok(cudaStreamSynchronize(s), err, "k_query_batch");
    }
    float ms = 0.f;
    if (ok) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!ok) return ST_CUDA;
    if (kernel_ms) *kernel_ms = double(ms);
    int status = ST_OK;
    for (int k = 0; k < n; ++k) {
        const QueryOut &q = hout[size_t(k)];
        QueryResult &r = out[k];
        r.distance = q.distance;
        r.moving_sphere = q.moving_sphere;
        r.other_sphere = q.other_sphere;
        r.other_slot = q.other_slot;
        r.status = q.status;
        r.n_candidates = q.n_candidates;
        r.n_pairs_refined = q.n_pairs_refined;
        r.n_scanned = q.n_scanned;
        r.n_cells = q.n_cells;
        r.n_cand_spheres = q.n_cand_spheres;
        r.n_mov = q.n_mov;
        if (q.status != ST_OK && status == ST_OK) {
            status = q.status;
            if (err) *err = "contact query " + std::to_string(k) + " failed with status " + std::to_string(q.status);
        }
        if (profiling_) {
            prof_.queries += 1;
            prof_.mov_spheres += q.n_mov;
            prof_.scanned += q.n_scanned;
            prof_.cells += q.n_cells;
            prof_.candidates += q.n_candidates;
            prof_.cand_spheres += q.n_cand_spheres;
            prof_.refined += q.n_pairs_refined;
        }
    }
    if (profiling_) prof_.query_ms += double(ms);
    return status;
}

int DeviceBox::translate(int slot, const double v[3], std::string *err) {
    DevBox &b = *static_cast<DevBox *>(devbox_);
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    k_translate<<<1, kQueryThreads, 0, s>>>(b, slot, v[0], v[1], v[2]);
    prof_.translates += profiling_ ? 1 : 0;
    if (!cuda_ok(cudaGetLastError(), err, "k_translate")) return ST_CUDA;
    return ST_OK;
}

int DeviceBox::merge(int ms, int os, int mslot, int oslot, MergeResult *out, std::string *err) {
    if (ensure_out_buffers(err) != ST_OK) return ST_CUDA;
    DevBox &b = *static_cast<DevBox *>(devbox_);
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    OutBuffers *ho = static_cast<OutBuffers *>(host_out_);
    OutBuffers *dout = static_cast<OutBuffers *>(dev_out_);
    if (profiling_) cudaEventRecord(static_cast<cudaEvent_t>(ev_[0]), s);
    k_merge<<<1, kQueryThreads, sizeof(MergeSmem), s>>>(b, ms, os, mslot, oslot, &dout->merge);
    if (profiling_) cudaEventRecord(static_cast<cudaEvent_t>(ev_[1]), s);
    if (!cuda_ok(cudaGetLastError(), err, "k_merge")) return ST_CUDA;
    if (!cuda_ok(cudaStreamSynchronize(s), err, "k_merge")) return ST_CUDA;
    const MergeOut &m = ho->merge;
    if (profiling_) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, static_cast<cudaEvent_t>(ev_[0]), static_cast<cudaEvent_t>(ev_[1]));
        prof_.merges += 1;
        prof_.merge_ms += ms;
        if (m.merged) {
            prof_.merged_spheres += m.n;
            prof_.merge_pairs += m.n_pairs;
        }
    }
    out->merged = m.merged;
    out->status = m.status;
    out->keep = m.keep;
    out->removed = m.removed;
    out->n = m.n;
    out->n_pairs = m.n_pairs;
    std::memcpy(out->fields, m.fields, sizeof(out->fields));
    out->vol_pp = m.vol_pp;
    out->maxradius = m.maxradius;
    int st = m.status;
    if (st == ST_OK) {
        // a Verlet cell may have overflowed during the merge
        int cs = check_status(err);
        if (cs == ST_CAPACITY) {
            DevBox &bb = *static_cast<DevBox *>(devbox_);
            cs = rebuild_grid(bb.cell_cap * 2, err);
        }
        st = cs;
    }
    if (st != ST_OK && err && err->empty()) *err = "merge failed with status " + std::to_string(st);
    return st;
}

int DeviceBox::set_fields(int slot, const double fields[21], unsigned mask, std::string *err) {
    DevBox &b = *static_cast<DevBox *>(devbox_);
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    FieldUpdate u;
    std::memcpy(u.v, fields, sizeof(u.v));
    k_set_fields<<<1, 32, 0, s>>>(b, slot, u, mask);
    if (!cuda_ok(cudaGetLastError(), err, "k_set_fields")) return ST_CUDA;
    return ST_OK;
}

int DeviceBox::upload_aggregates(const std::vector<double> &agg, std::string *err) {
    DevBox &b = *static_cast<DevBox *>(devbox_);
    if (agg.size() != size_t(21) * size_t(b.nslots)) return ST_BAD_ARGUMENT;
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    if (!cuda_ok(cudaMemcpyAsync(b.agg, agg.data(), sizeof(double) * agg.size(), cudaMemcpyHostToDevice, s), err,
                 "upload"))
        return ST_CUDA;
    k_refresh_f4<<<std::min(1024, (b.nslots + 255) / 256), 256, 0, s>>>(b);
    if (!cuda_ok(cudaGetLastError(), err, "k_refresh_f4")) return ST_CUDA;
    if (!cuda_ok(cudaStreamSynchronize(s), err, "sync")) return ST_CUDA;
    return ST_OK;
}

int DeviceBox::download(HostState *st, std::string *err, void *copy_stream) {
    DevBox &b = *static_cast<DevBox *>(devbox_);
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    cudaStream_t cs = copy_stream ? static_cast<cudaStream_t>(copy_stream) : s;
    if (!cuda_ok(cudaStreamSynchronize(s), err, "sync")) return ST_CUDA;
    DevScalars sc;
    st->ns = b.ns;
    st->nslots = b.nslots;
    st->n_div = b.n_div;
    st->box_length = b.L;
    st->sph.resize(9 * size_t(b.ns));
    st->sph_slot.resize(size_t(b.ns));
    st->agg.resize(21 * size_t(b.nslots));
    st->agg_n.resize(size_t(b.nslots));
    std::vector<int> off(static_cast<size_t>(b.nslots));
    auto get = [&](void *dst, const void *src, size_t bytes) {
        return cuda_ok(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, cs), err, "download");
    };
    bool ok = get(&sc, b.sc, sizeof(sc)) && cuda_ok(cudaStreamSynchronize(cs), err, "download") &&
              get(st->sph.data(), b.sph, sizeof(double) * 9 * size_t(b.ns)) &&
              get(st->sph_slot.data(), b.sph_slot, sizeof(int) * size_t(b.ns)) &&
              get(st->agg.data(), b.agg, sizeof(double) * 21 * size_t(b.nslots)) &&
              get(st->agg_n.data(), b.agg_n, sizeof(int) * size_t(b.nslots)) &&
              get(off.data(), b.agg_off, sizeof(int) * size_t(b.nslots));
    std::vector<int> pool(static_cast<size_t>(b.pool_cap));
    ok = ok && get(pool.data(), b.pool_id[sc.pool_sel], sizeof(int) * size_t(b.pool_cap)) &&
         cuda_ok(cudaStreamSynchronize(cs), err, "download");
    if (!ok) return ST_CUDA;
    st->members.clear();
    st->members.reserve(size_t(b.nslots), size_t(b.ns));
    for (int a = 0; a < b.nslots; ++a) st->members.push_list(pool.data() + off[size_t(a)], st->agg_n[size_t(a)]);
    st->maxradius = sc.maxradius;
    st->time = sc.time;
    return ST_OK;
}

int DeviceBox::store(mcacg_state *out, std::string *err, void *copy_stream) {
    DevBox &b = *static_cast<DevBox *>(devbox_);
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    cudaStream_t cs = copy_stream ? static_cast<cudaStream_t>(copy_stream) : s;
    if (!out->spheres || !out->sphere_label || !out->aggregates || !out->n_spheres_per_aggregate || !out->members) {
        if (err) *err = "incomplete state buffers";
        return ST_BAD_ARGUMENT;
    }
    if (!cuda_ok(cudaStreamSynchronize(s), err, "sync")) return ST_CUDA;
    DevScalars sc;
    if (!cuda_ok(cudaMemcpyAsync(&sc, b.sc, sizeof(sc), cudaMemcpyDeviceToHost, cs), err, "store") ||
        !cuda_ok(cudaStreamSynchronize(cs), err, "store"))
        return ST_CUDA;
    const int na = sc.n_alive;
    if (out->n_spheres < b.ns || out->n_aggregates < na || na < 1) {
        if (err) *err = "state buffers too small";
        return ST_BAD_ARGUMENT;
    }
    const size_t need = 176 * size_t(na) + 16 * size_t(b.ns) + 8 * size_t(b.nslots);
    if (need > stage_bytes_) {
        if (err) *err = "store staging area too small";
        return ST_CAPACITY;
    }
    char *p = static_cast<char *>(stage_);
    PackStage ps;
    ps.agg = reinterpret_cast<double *>(p);
    ps.count = reinterpret_cast<long long *>(p + 168 * size_t(na));
    ps.label = reinterpret_cast<long long *>(p + 176 * size_t(na));
    ps.members = ps.label + b.ns;
    ps.rank = reinterpret_cast<int *>(ps.members + b.ns);
    ps.moff = ps.rank + b.nslots;
    ps.na = na;
    ps.sel = sc.pool_sel;
    const int blocks = std::min(1024, (std::max(b.ns, b.nslots) + 255) / 256);
    k_pack_ranks<<<1, kLoadScanThreads, 0, cs>>>(b, ps);
    k_pack<<<blocks, 256, 0, cs>>>(b, ps);
    if (!cuda_ok(cudaGetLastError(), err, "store")) return ST_CUDA;
    auto get = [&](void *dst, const void *src, size_t bytes) {
        return cuda_ok(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, cs), err, "store");
    };
    const bool ok = get(out->spheres, b.sph, sizeof(double) * 9 * size_t(b.ns)) &&
                    get(out->sphere_label, ps.label, 8 * size_t(b.ns)) &&
                    get(out->aggregates, ps.agg, 168 * size_t(na)) &&
                    get(out->n_spheres_per_aggregate, ps.count, 8 * size_t(na)) &&
                    get(out->members, ps.members, 8 * size_t(b.ns)) && cuda_ok(cudaStreamSynchronize(cs), err, "store");
    if (!ok) return ST_CUDA;
    out->n_spheres = b.ns;
    out->n_aggregates = na;
    out->n_verlet_divisions = b.n_div;
    out->box_length = b.L;
    out->maxradius = sc.maxradius;
    out->time = sc.time;
    return ST_OK;
}

}  // namespace mcacg
