// Single-box kernels and the host-side management of a device-resident box.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "box.cuh"
#include "device_box.hpp"
#include "host_parallel.hpp"
#include "merge.cuh"

#include <atomic>

namespace mcacg {

namespace {
std::atomic<int> g_merge_grid_min{2048};
}

int merge_grid_min() { return g_merge_grid_min.load(std::memory_order_relaxed); }
int set_merge_grid_min(int n) { return g_merge_grid_min.exchange(n); }


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
// Threads per query block: 64, 128 or 256 (8, 4 or 2 blocks per SM at 128
// registers a thread); the first large batch of a box times each and keeps
// the fastest (results do not depend on it).
constexpr int kBatchThreadChoices[] = {64, 128, 256};
template <int NT>
__global__ void __launch_bounds__(NT, 512 / NT) k_query_batch(DevBox b, BatchScratch s, int n, const QueryIn *in,
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

// Surface growth of the host-driven loop (Sphere::croissance_surface,
// sphere.cpp:113-120): every sphere of one slot (slot >= 0) or of every live
// slot becomes r + du, its volume and surface from the new radius.
__global__ void k_grow(DevBox b, int slot, double du) {
    const double pi = pi_value();
    const double vf = 4. * pi / 3., sf = 4. * pi;
    const int *pool_id = b.pool_id[b.sc->pool_sel];
    float4 *pool_pos = b.pool_pos[b.sc->pool_sel];
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    const int k0 = slot >= 0 ? b.agg_off[slot] : 0;
    const int k1 = slot >= 0 ? k0 + b.agg_n[slot] : b.sc->pool_top;
    for (int k = k0 + t0; k < k1; k += stride) {
        const int s = pool_id[k];
        if (s < 0 || s >= b.ns) continue;
        const int a = b.sph_slot[s];
        if (a < 0 || a >= b.nslots) continue;
        const int rel = k - b.agg_off[a];
        if (b.agg_n[a] == 0 || rel < 0 || rel >= b.agg_n[a]) continue;  // a stale pool entry
        const double r = S(b, SPH_R, s) + du;
        const double r2 = r * r, r3 = r2 * r;
        S(b, SPH_R, s) = r;
        S(b, SPH_VOLUME, s) = vf * r3;
        S(b, SPH_SURFACE, s) = sf * r2;
        pool_pos[k].w = float(r);
    }
}

// The geometry of every live slot (slot < 0) or of one (Aggregate::update
// when 'full', with the overlap and coordination fields, else
// update_partial; without the physics fields), one thread per slot; vol_pp[a] receives update_partial's mean sphere volume. Slots
// whose Verlet or fine cell changed are listed in moved[] (count in
// counters[5]) for k_regrid_moved.
__global__ void k_update_geometry(DevBox b, int slot, int full, double *vol_pp, int *moved) {
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    const int a0 = slot >= 0 ? slot : 0, a1 = slot >= 0 ? slot + 1 : b.nslots;
    for (int a = a0 + t0; a < a1; a += stride) {
        if (b.agg_n[a] == 0) continue;
        double vp = 0.0;
        thread_update_geometry(b, a, full != 0, &vp, true);
        vol_pp[a] = vp;
        const Vec3 p = agg_pos(b, a);
        if (cell_of(b, p) != b.agg_cell[a] || (b.fine_div > 0 && fine_cell_of(b, p) != b.fine_cell[a]))
            moved[atomicAdd(&b.counters[5], 1)] = a;
    }
}
// The listed slots follow their new positions in the grids (one thread; the
// grid lists are unordered, so the order of the moves sets no result).
__global__ void k_regrid_moved(DevBox b, const int *moved) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const int n = b.counters[5];
    for (int k = 0; k < n && k < b.nslots; ++k) regrid(b, moved[k], agg_pos(b, moved[k]));
    b.counters[5] = 0;
}

struct FieldUpdate {
    double v[21];
};
__global__ void k_set_fields(DevBox b, int slot, FieldUpdate u, unsigned mask) {
    int f = threadIdx.x;
    if (f < AGG_NFIELDS && (mask >> f) & 1u) A(b, f, slot) = u.v[f];
}

// The kernels below run on one box (single-box launches) or on many boxes at
// once (k_boxes: per_box blocks for each box, whose DevBox is read into
// shared memory). Their bodies take the thread's index among the box's
// threads and the number of those threads.
//
// Verlet and fine grids from the aggregate positions: clear the cells, drop
// every live slot into its cells (in any order: the scan key restores the
// reference's order), then link the fine lists backwards.
__device__ void grid_clear_range(const DevBox &b, int t, int stride) {
    for (int c = t; c < b.n_cells; c += stride) b.cell_n[c] = 0;
    if (b.fine_div > 0) {
        const int nf3 = b.fine_div * b.fine_div * b.fine_div;
        for (int c = t; c < nf3; c += stride) b.fine_head[c] = -1;
        for (int a = t; a < b.nslots; a += stride) b.fine_cell[a] = -1;
    }
}
__device__ void grid_fill_range(const DevBox &b, int t, int stride) {
    for (int a = t; a < b.nslots; a += stride) {
        if (b.agg_n[a] == 0) continue;
        const int key = cell_of(b, agg_pos(b, a));
        const int c = cell_index(b, key);
        b.agg_cell[a] = key;
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
// back links of the fine lists built by grid_fill_range
__device__ void fine_link_range(const DevBox &b, int t, int stride) {
    if (b.fine_div == 0) return;
    for (int a = t; a < b.nslots; a += stride) {
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
// member lists in slot order) are staged in the box's work area (64 B per
// sphere; 16 B per sphere and 8 B per slot at most are used) as 32- or 64-bit
// values and converted here, with the pool built from the member lists.
// Inconsistent input is flagged (sc->pad[0] = the LoadError, status
// BAD_ARGUMENT) and never read out of bounds.
enum LoadError { LOAD_OK = 0, LOAD_LABEL = 1, LOAD_COUNT = 2, LOAD_COVER = 3, LOAD_MEMBER = 4 };
struct LoadStage {
    const void *label, *count, *members;
    int wide;     // 64-bit integers
    int dead_ok;  // slots without spheres are allowed
};
__host__ __device__ inline LoadStage load_stage(const DevBox &b, int wide, int dead_ok) {
    const size_t iw = wide ? 8 : 4;
    const char *stage = reinterpret_cast<const char *>(b.work);
    return LoadStage{stage, stage + 2 * iw * size_t(b.ns), stage + iw * size_t(b.ns), wide, dead_ok};
}
__device__ __forceinline__ long long load_int(const void *p, int wide, int i) {
    return wide ? static_cast<const long long *>(p)[i] : static_cast<long long>(static_cast<const int *>(p)[i]);
}
__device__ __forceinline__ void load_fail(const DevBox &b, int code) {
    atomicCAS(&b.sc->pad[0], 0, code);
    b.sc->status = ST_BAD_ARGUMENT;
}
constexpr int kScanThreads = 1024;
// spheres per slot, pool offsets (exclusive sum in slot order), live count;
// one block of kScanThreads threads per box
__device__ void load_counts_block(const DevBox &b, const LoadStage &in) {
    __shared__ long long part[kScanThreads];
    __shared__ int alive[kScanThreads];
    __shared__ int bad;
    const int t = threadIdx.x;
    if (t == 0) bad = 0;
    __syncthreads();
    const int chunk = (b.nslots + kScanThreads - 1) / kScanThreads;
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
        for (int k = 0; k < kScanThreads; ++k) {
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
__device__ void load_spheres_range(const DevBox &b, const LoadStage &in, int t, int stride) {
    for (int s = t; s < b.ns; s += stride) {
        long long l = load_int(in.label, in.wide, s);
        if (l < 0 || l >= b.nslots) {
            load_fail(b, LOAD_LABEL);
            l = 0;
        }
        b.sph_slot[s] = int(l);
        b.sph_volw[s] = S(b, SPH_VOLUME, s);
        long long m = load_int(in.members, in.wide, s);
        if (m < 0 || m >= b.ns) {
            load_fail(b, LOAD_MEMBER);
            m = 0;
        }
        b.pool_id[0][s] = int(m);
        b.pool_pos[0][s] = make_float4(float(S(b, SPH_X, int(m))), float(S(b, SPH_Y, int(m))),
                                       float(S(b, SPH_Z, int(m))), float(S(b, SPH_R, int(m))));
    }
    for (int k = b.ns + t; k < b.pool_cap; k += stride) {
        b.pool_id[0][k] = 0;
        b.pool_pos[0][k] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}
// every member of slot a is owned by slot a
__device__ void load_check_range(const DevBox &b, int t, int stride) {
    for (int a = t; a < b.nslots; a += stride) {
        const int o = b.agg_off[a], e = min(b.ns, o + b.agg_n[a]);
        for (int k = o; k < e; ++k)
            if (b.sph_slot[b.pool_id[0][k]] != a) {
                load_fail(b, LOAD_MEMBER);
                break;
            }
    }
}

// Storing a state: the live slots are packed in slot order (label = rank
// among the live slots, as the reference's list has them), with their member
// lists back to back, into the merge's pair scratch; the host copies the
// pieces out (PackLayout gives the offsets).
struct PackStage {
    double *agg;         // [21][na]
    long long *count;    // [na]
    long long *label;    // [ns]
    long long *members;  // [ns]
    int *rank;           // [nslots]
    int *moff;           // [nslots] first member of the slot in 'members'
    int na;
    int sel;             // live pool buffer
};
__host__ __device__ inline PackStage pack_stage(const DevBox &b, int na, int sel) {
    char *p = reinterpret_cast<char *>(b.pair_i);
    const PackLayout l = pack_layout(na, b.ns, b.nslots);
    return PackStage{reinterpret_cast<double *>(p + l.agg),      reinterpret_cast<long long *>(p + l.count),
                     reinterpret_cast<long long *>(p + l.label), reinterpret_cast<long long *>(p + l.members),
                     reinterpret_cast<int *>(p + l.rank),        reinterpret_cast<int *>(p + l.moff),
                     na,
                     sel};
}
// ranks of the live slots and member offsets; one block of kScanThreads
__device__ void pack_ranks_block(const DevBox &b, const PackStage &out) {
    __shared__ int live_part[kScanThreads];
    __shared__ int mem_part[kScanThreads];
    const int t = threadIdx.x;
    const int chunk = (b.nslots + kScanThreads - 1) / kScanThreads;
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
        for (int k = 0; k < kScanThreads; ++k) {
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
__device__ void pack_range(const DevBox &b, const PackStage &out, int t, int stride) {
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
    for (int s = t; s < b.ns; s += stride) {
        const int a = b.sph_slot[s];
        out.label[s] = (a >= 0 && a < b.nslots) ? out.rank[a] : -1;
    }
}

enum BoxOp { OP_GRID_CLEAR, OP_GRID_FILL, OP_FINE_LINK, OP_LOAD_COUNTS, OP_LOAD_SPHERES, OP_LOAD_CHECK, OP_PACK_RANKS,
             OP_PACK };
// Per-box arguments of k_boxes: the load flags, or the live count (< 0:
// skip the box) and live pool buffer of a store.
struct BoxArg {
    int a, b;
};
template <int OP>
__device__ __forceinline__ void box_op(const DevBox &b, BoxArg arg, int t, int stride) {
    if (OP == OP_GRID_CLEAR) grid_clear_range(b, t, stride);
    if (OP == OP_GRID_FILL) grid_fill_range(b, t, stride);
    if (OP == OP_FINE_LINK) fine_link_range(b, t, stride);
    if (OP == OP_LOAD_COUNTS) load_counts_block(b, load_stage(b, arg.a, arg.b));
    if (OP == OP_LOAD_SPHERES) load_spheres_range(b, load_stage(b, arg.a, arg.b), t, stride);
    if (OP == OP_LOAD_CHECK) load_check_range(b, t, stride);
    if (OP == OP_PACK_RANKS) pack_ranks_block(b, pack_stage(b, arg.a, arg.b));
    if (OP == OP_PACK) pack_range(b, pack_stage(b, arg.a, arg.b), t, stride);
}
template <int OP>
__global__ void __launch_bounds__(kScanThreads) k_box(DevBox b, BoxArg arg) {
    box_op<OP>(b, arg, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}
template <int OP>
__global__ void __launch_bounds__(kScanThreads) k_boxes(const DevBox *boxes, const BoxArg *args, int n, int per_box) {
    __shared__ DevBox b;
    __shared__ BoxArg arg;
    const int box = blockIdx.x / per_box;
    if (box >= n) return;  // block-uniform
    if (threadIdx.x == 0) {
        b = boxes[box];
        arg = args[box];
    }
    __syncthreads();
    if ((OP == OP_PACK_RANKS || OP == OP_PACK) && arg.a < 0) return;  // block-uniform
    box_op<OP>(b, arg, (blockIdx.x % per_box) * blockDim.x + threadIdx.x, per_box * blockDim.x);
}
// the scalars of many boxes, gathered for one copy to the host
__global__ void k_gather_scalars(const DevBox *boxes, int n, DevScalars *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = *boxes[i].sc;
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

namespace {

bool view_ok(const StateView &st) {
    return st.ns > 0 && st.nslots > 0 && st.nslots <= st.ns && st.sph && st.agg && st.sph_slot && st.agg_n &&
           st.members && st.box_length > 0.0 && st.n_div > 0 && st.n_div <= 1024;
}

// Sizes, grids and capacities of a box from its state, by host arithmetic
// over the live slots: one pass gives the largest r_max, the means of lpm and
// r_max, and the Verlet cell counts. No pointer is set.
// What a box's sizes and fixed parameters need: the state's counts and box
// alone (no pass over its arrays).
DevBox plan_fixed(const StateView &st) {
    DevBox b{};
    b.volsurf = VS_NONE;
    b.L = st.box_length;
    b.n_div = st.n_div;
    b.step = double(st.n_div) / st.box_length;
    b.n_cells = st.n_div * st.n_div * st.n_div;
    b.ns = st.ns;
    b.nslots = st.nslots;
    b.inv_L = 1.0 / st.box_length;
    b.Lf = float(st.box_length);
    b.inv_Lf = 1.0f / b.Lf;
    b.inv_cells = 1.0f / float(b.n_cells);
    b.pool_cap = 2 * st.ns + 1024;
    b.surv_cap = 1 << 16;
    // contact pairs inside one aggregate: equal spheres touch at most 12
    // others (the kissing number), so at most 6 pairs per sphere; the
    // merge reports a capacity error beyond 8 per sphere
    b.pair_cap = 8 * st.ns + 1024;
    b.grid_pairs_min = merge_grid_min();
    return b;
}

// The grids from one pass over the live slots: largest r_max, the means of
// lpm and r_max, and the Verlet cell counts (host arithmetic).
void plan_grids(const StateView &st, DevBox &b) {
    const double *agg = st.agg;
    auto AF = [&](int f, int a) { return agg[size_t(f) * size_t(st.nslots) + size_t(a)]; };
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
    // FP32 screening margin: coordinates are bounded by the box plus the
    // largest aggregate; 2^-17 of that bound is >10x the FP32 error of the
    // capsule test.
    b.margin = (3.0 * st.box_length + 4.0 * rmax_all) * (1.0 / 131072.0);
    // fine discovery grid, when finer than the Verlet grid: a query visits
    // the cells covering its swept box, about lpm/2 + 2 (r_max + max r_max)
    // per axis on average; cells of 0.6 of that balance the cells visited
    // against the aggregates screened. At least 2 max r_max and L/128.
    const double extent = live ? 0.5 * lpm_sum / live + 2.0 * (rmax_sum / live + rmax_all) : 0.0;
    const double h = std::max({2.0 * rmax_all, st.box_length / double(kFineMaxDiv), 0.6 * extent});
    const double nf = std::floor(st.box_length / h);
    b.fine_div = (nf > double(st.n_div) && nf <= double(kFineMaxDiv)) ? int(nf) : 0;
    b.fine_step = b.fine_div > 0 ? double(b.fine_div) / st.box_length : 0.0;
    b.margin_f = float(b.margin);
    b.fine_step_f = float(b.fine_step);
    b.inv_fine_cells = b.fine_div > 0 ? 1.0f / float(double(b.fine_div) * b.fine_div * b.fine_div) : 0.0f;
    const int avg = (st.nslots + b.n_cells - 1) / b.n_cells;
    b.cell_cap = std::max({64, 2 * maxc, 8 * avg});
}

DevBox plan_box(const StateView &st) {
    DevBox b = plan_fixed(st);
    plan_grids(st, b);
    return b;
}

// Places the box's arrays (nullptr: sizes them only, leaving the pointers
// null) and returns the bytes used; every array starts on a 256-byte
// boundary. The fixed part depends on the counts alone; the grid part
// (fine lists, Verlet cell lists) on plan_grids.
size_t carve_take(char *arena, size_t *used, void **p, size_t bytes) {
    *p = arena ? arena + *used : nullptr;
    *used += (std::max<size_t>(bytes, 16) + 255) & ~size_t(255);
    return *used;
}
size_t carve_fixed(DevBox &b, char *arena) {
    size_t used = 0;
    auto take = [&](void **p, size_t bytes) { carve_take(arena, &used, p, bytes); };
    const size_t ns = size_t(b.ns), nslots = size_t(b.nslots);
    take((void **)&b.sph, sizeof(double) * 9 * ns);
    take((void **)&b.sph_slot, sizeof(int) * ns);
    take((void **)&b.sph_volw, sizeof(double) * ns);
    take((void **)&b.agg, sizeof(double) * 21 * nslots);
    take((void **)&b.agg_n, sizeof(int) * nslots);
    take((void **)&b.agg_off, sizeof(int) * nslots);
    take((void **)&b.agg_cell, sizeof(int) * nslots);
    take((void **)&b.agg_f4, sizeof(float4) * nslots);
    for (int k = 0; k < 2; ++k) {
        take((void **)&b.pool_id[k], sizeof(int) * size_t(b.pool_cap));
        take((void **)&b.pool_pos[k], sizeof(float4) * size_t(b.pool_cap));
    }
    take((void **)&b.cell_n, sizeof(int) * size_t(b.n_cells));
    take((void **)&b.cell_pos, sizeof(int) * nslots);
    take((void **)&b.sc, sizeof(DevScalars));
    take((void **)&b.surv, sizeof(int4) * size_t(b.surv_cap));
    take((void **)&b.surv_res, sizeof(double) * size_t(b.surv_cap));
    // the merge's pair scratch is one block (32 B per pair), which also
    // stages a packed state on its way to the host
    {
        char *pairs = nullptr;
        const size_t pc = size_t(b.pair_cap);
        take((void **)&pairs, 32 * pc);
        b.pair_i = reinterpret_cast<int *>(pairs);
        b.pair_j = pairs ? b.pair_i + pc : nullptr;
        b.pair_tmp_i = pairs ? b.pair_j + pc : nullptr;
        b.pair_tmp_j = pairs ? b.pair_tmp_i + pc : nullptr;
        b.pair_d = pairs ? reinterpret_cast<double *>(pairs + 16 * pc) : nullptr;
        b.pair_tmp_d = pairs ? b.pair_d + pc : nullptr;
    }
    take((void **)&b.row_cnt, sizeof(int) * (std::max(ns, nslots) + 2));
    // 64 B per sphere: the merge sums' per-sphere terms, and the merge's
    // cell-grid pair search (at most 52 B per merged sphere + 4, merge.cuh)
    take((void **)&b.work, sizeof(double) * 8 * ns);
    take((void **)&b.counters, sizeof(int) * 8);
    const size_t nc1 = nslots + 1;
    take((void **)&b.cand_db, sizeof(double) * nc1);
    take((void **)&b.cand_key, sizeof(long long) * nc1);
    take((void **)&b.cand_slot, sizeof(int) * nc1);
    take((void **)&b.cand_order, sizeof(int) * nc1);
    take((void **)&b.cand_prefix, sizeof(int) * nc1);
    take((void **)&b.best_res, sizeof(unsigned long long) * nc1);
    take((void **)&b.best_ij, sizeof(unsigned long long) * nc1);
    return used;
}
size_t carve_grids(DevBox &b, char *arena) {
    size_t used = 0;
    auto take = [&](void **p, size_t bytes) { carve_take(arena, &used, p, bytes); };
    const size_t nslots = size_t(b.nslots);
    b.fine_head = b.fine_next = b.fine_prev = b.fine_cell = nullptr;
    if (b.fine_div > 0) {
        const size_t nf3 = size_t(b.fine_div) * size_t(b.fine_div) * size_t(b.fine_div);
        take((void **)&b.fine_head, sizeof(int) * nf3);
        take((void **)&b.fine_next, sizeof(int) * nslots);
        take((void **)&b.fine_prev, sizeof(int) * nslots);
        take((void **)&b.fine_cell, sizeof(int) * nslots);
    }
    take((void **)&b.cell_items, sizeof(int) * size_t(b.n_cells) * size_t(b.cell_cap));
    return used;
}
size_t carve_box(DevBox &b, char *arena) {
    const size_t fixed = carve_fixed(b, arena);
    return fixed + carve_grids(b, arena ? arena + fixed : nullptr);
}

// The copies of a state into a carved box on stream s: the tables to their
// places, the integer arrays to the load stage (load_stage).
bool upload_state(const DevBox &b, const StateView &st, cudaStream_t s, std::string *err) {
    DevScalars sc{};
    sc.maxradius = st.maxradius;
    sc.time = st.time;
    sc.pool_sel = 0;
    const size_t iw = st.wide ? 8 : 4;
    const LoadStage in = load_stage(b, st.wide ? 1 : 0, st.dead_slots ? 1 : 0);
    auto put = [&](const void *dst, const void *src, size_t bytes) {
        return cuda_ok(cudaMemcpyAsync(const_cast<void *>(dst), src, bytes, cudaMemcpyHostToDevice, s), err, "upload");
    };
    return put(b.sph, st.sph, sizeof(double) * 9 * size_t(st.ns)) &&
           put(b.agg, st.agg, sizeof(double) * 21 * size_t(st.nslots)) && put(in.label, st.sph_slot, iw * size_t(st.ns)) &&
           put(in.members, st.members, iw * size_t(st.ns)) && put(in.count, st.agg_n, iw * size_t(st.nslots)) &&
           put(b.sc, &sc, sizeof(sc));
}

const char *load_error_text(int code) {
    switch (code) {
        case LOAD_LABEL: return "sphere label out of range";
        case LOAD_COUNT: return "bad sphere count of an aggregate";
        case LOAD_COVER: return "member lists do not cover every sphere once";
        case LOAD_MEMBER: return "member list inconsistent with sphere labels";
        default: return "state rejected";
    }
}

// blocks per box of the many-box kernels: enough to fill the GPU
int blocks_per_box(int n_boxes, int max_items) {
    int dev = 0, n_sm = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n_sm <= 0) n_sm = 152;
    const int want = (8 * n_sm + n_boxes - 1) / std::max(1, n_boxes);
    return std::max(1, std::min({want, 256, (max_items + 255) / 256}));
}

// A few streams that share the copies of many boxes (several copy engines
// at work, their per-copy latencies overlapped), forked from and joined back
// into a main stream.
class CopyStreams {
  public:
    explicit CopyStreams(int n) {
        for (int i = 0; i < n; ++i) {
            cudaStream_t st = nullptr;
            if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) break;
            streams_.push_back(st);
        }
    }
    ~CopyStreams() {
        for (cudaStream_t st : streams_) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
        if (ev_) cudaEventDestroy(ev_);
    }
    CopyStreams(const CopyStreams &) = delete;
    CopyStreams &operator=(const CopyStreams &) = delete;
    // stream k of the set (the main stream when none could be made)
    cudaStream_t at(size_t k, cudaStream_t main) const {
        return streams_.empty() ? main : streams_[k % streams_.size()];
    }
    // the set's streams start after the work queued on 'main' so far
    bool fork(cudaStream_t main) {
        if (streams_.empty()) return true;
        if (!ev_ && cudaEventCreateWithFlags(&ev_, cudaEventDisableTiming) != cudaSuccess) return false;
        if (cudaEventRecord(ev_, main) != cudaSuccess) return false;
        for (cudaStream_t st : streams_)
            if (cudaStreamWaitEvent(st, ev_, 0) != cudaSuccess) return false;
        return true;
    }
    // 'main' continues after the work queued on the set so far
    bool join(cudaStream_t main) {
        for (cudaStream_t st : streams_) {
            cudaEvent_t e = nullptr;
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return false;
            const bool ok = cudaEventRecord(e, st) == cudaSuccess && cudaStreamWaitEvent(main, e, 0) == cudaSuccess;
            cudaEventDestroy(e);
            if (!ok) return false;
        }
        return true;
    }

  private:
    std::vector<cudaStream_t> streams_;
    cudaEvent_t ev_ = nullptr;
};
constexpr int kCopyStreams = 4;

}  // namespace

int DeviceBox::create(const StateView &st, void *stream, DeviceBox **out, std::string *err) {
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        if (err) *err = "no CUDA device";
        return ST_NO_DEVICE;
    }
    if (!view_ok(st)) {
        if (err) *err = "incomplete state";
        return ST_BAD_ARGUMENT;
    }
    DevBox b = plan_box(st);
    const size_t bytes = carve_box(b, nullptr);
    std::unique_ptr<DeviceBox> d(new DeviceBox());
    d->ns_ = st.ns;
    d->nslots_ = st.nslots;
    char *arena = nullptr;
    if (!cuda_ok(cudaMalloc((void **)&arena, bytes), err, "cudaMalloc")) return ST_CUDA;
    d->allocations_.push_back(arena);
    carve_box(b, arena);
    d->stage_ = b.pair_i;
    d->stage_bytes_ = 32 * size_t(b.pair_cap);
    if (stream) {
        d->stream_ = stream;
    } else {
        cudaStream_t s;
        if (!cuda_ok(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), err, "cudaStreamCreate")) return ST_CUDA;
        d->stream_ = s;
        d->own_stream_ = true;
    }
    // the host arrays stay alive until the status read below synchronises
    cudaStream_t s = static_cast<cudaStream_t>(d->stream_);
    if (!upload_state(b, st, s, err)) return ST_CUDA;
    const BoxArg la{st.wide ? 1 : 0, st.dead_slots ? 1 : 0};
    const int blocks = std::min(1024, (std::max(st.ns, st.nslots) + 255) / 256);
    k_box<OP_LOAD_COUNTS><<<1, kScanThreads, 0, s>>>(b, la);
    k_box<OP_LOAD_SPHERES><<<blocks, 256, 0, s>>>(b, la);
    k_box<OP_LOAD_CHECK><<<blocks, 256, 0, s>>>(b, la);
    if (!cuda_ok(cudaGetLastError(), err, "state load")) return ST_CUDA;
    DevScalars got;
    if (!cuda_ok(cudaMemcpyAsync(&got, b.sc, sizeof(got), cudaMemcpyDeviceToHost, s), err, "status") ||
        !cuda_ok(cudaStreamSynchronize(s), err, "sync"))
        return ST_CUDA;
    if (got.status != ST_OK) {
        if (err) *err = load_error_text(got.pad[0]);
        return ST_BAD_ARGUMENT;
    }
    d->devbox_ = new DevBox(b);
    int rc = d->rebuild_grid(b.cell_cap, err);
    if (rc != ST_OK) return rc;
    *out = d.release();
    return ST_OK;
}

int DeviceBox::create_many(const std::vector<StateView> &views, void *stream,
                           std::vector<std::unique_ptr<DeviceBox>> *out, std::string *err) {
    out->clear();
    const int n = int(views.size());
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        if (err) *err = "no CUDA device";
        return ST_NO_DEVICE;
    }
    bool same_kind = true;
    for (int i = 0; i < n; ++i) {
        if (!view_ok(views[size_t(i)])) {
            if (err) *err = "box " + std::to_string(i) + ": incomplete state";
            return ST_BAD_ARGUMENT;
        }
        same_kind = same_kind && views[size_t(i)].wide == views[0].wide &&
                    views[size_t(i)].dead_slots == views[0].dead_slots;
    }
    if (n == 0) return ST_OK;
    if (!same_kind) {
        if (err) *err = "states of one batch must have the same integer width";
        return ST_BAD_ARGUMENT;
    }
    // The fixed part of every box in one allocation, sized from the counts
    // alone, so the copies start at once; the grids are planned on the host
    // threads (one pass over each state's live slots) while they run, then
    // get a second allocation.
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::vector<DevBox> plans(static_cast<size_t>(n));
    std::vector<size_t> off(static_cast<size_t>(n) + 1, 0);
    int max_items = 0;
    for (int i = 0; i < n; ++i) {
        plans[size_t(i)] = plan_fixed(views[size_t(i)]);
        off[size_t(i) + 1] = off[size_t(i)] + carve_fixed(plans[size_t(i)], nullptr);
        max_items = std::max({max_items, plans[size_t(i)].ns, plans[size_t(i)].nslots});
    }
    char *arena = nullptr;
    if (!cuda_ok(cudaMalloc((void **)&arena, off[size_t(n)]), err, "cudaMalloc")) {
        if (err) *err += " (" + std::to_string(off[size_t(n)] >> 20) + " MiB for " + std::to_string(n) + " boxes)";
        return ST_CUDA;
    }
    std::shared_ptr<void> shared(arena, [](void *p) { cudaFree(p); });
    for (int i = 0; i < n; ++i) carve_fixed(plans[size_t(i)], arena + off[size_t(i)]);
    // the copies, spread over a few streams, then joined into the main one
    CopyStreams copies(kCopyStreams);
    if (!copies.fork(s)) {
        if (err) *err = "copy streams";
        return ST_CUDA;
    }
    for (int i = 0; i < n; ++i)
        if (!upload_state(plans[size_t(i)], views[size_t(i)], copies.at(size_t(i), s), err)) {
            if (err) *err = "box " + std::to_string(i) + ": " + *err;
            return ST_CUDA;  // the copy streams are synchronised on the way out
        }
    if (!copies.join(s)) {
        if (err) *err = "copy streams";
        return ST_CUDA;
    }
    parallel_for(n, [&](int i) { plan_grids(views[size_t(i)], plans[size_t(i)]); });
    std::vector<size_t> goff(static_cast<size_t>(n) + 1, 0);
    for (int i = 0; i < n; ++i) goff[size_t(i) + 1] = goff[size_t(i)] + carve_grids(plans[size_t(i)], nullptr);
    char *grid_arena = nullptr;
    if (!cuda_ok(cudaMalloc((void **)&grid_arena, goff[size_t(n)]), err, "cudaMalloc")) {
        cudaStreamSynchronize(s);
        return ST_CUDA;
    }
    std::shared_ptr<void> shared_grids(grid_arena, [](void *p) { cudaFree(p); });
    std::vector<std::unique_ptr<DeviceBox>> boxes(static_cast<size_t>(n));
    for (int i = 0; i < n; ++i) {
        DevBox &b = plans[size_t(i)];
        carve_grids(b, grid_arena + goff[size_t(i)]);
        std::unique_ptr<DeviceBox> d(new DeviceBox());
        d->ns_ = b.ns;
        d->nslots_ = b.nslots;
        d->arena_ = shared;
        d->arena_grids_ = shared_grids;
        d->stage_ = b.pair_i;
        d->stage_bytes_ = 32 * size_t(b.pair_cap);
        d->stream_ = s;
        d->devbox_ = new DevBox(b);
        boxes[size_t(i)] = std::move(d);
    }
    // the load and grid kernels over all boxes at once
    const size_t tb = (sizeof(DevBox) * size_t(n) + 255) & ~size_t(255);
    const size_t ta = (sizeof(BoxArg) * size_t(n) + 255) & ~size_t(255);
    char *tmp = nullptr;
    if (!cuda_ok(cudaMalloc((void **)&tmp, tb + ta + sizeof(DevScalars) * size_t(n)), err, "cudaMalloc")) return ST_CUDA;
    std::unique_ptr<char, void (*)(char *)> tmp_owner(tmp, [](char *p) { cudaFree(p); });
    DevBox *dboxes = reinterpret_cast<DevBox *>(tmp);
    BoxArg *dargs = reinterpret_cast<BoxArg *>(tmp + tb);
    DevScalars *dsc = reinterpret_cast<DevScalars *>(tmp + tb + ta);
    std::vector<BoxArg> args(static_cast<size_t>(n), BoxArg{views[0].wide ? 1 : 0, views[0].dead_slots ? 1 : 0});
    std::vector<DevScalars> sc(static_cast<size_t>(n));
    const int per = blocks_per_box(n, max_items);
    if (!cuda_ok(cudaMemcpyAsync(dboxes, plans.data(), sizeof(DevBox) * size_t(n), cudaMemcpyHostToDevice, s), err,
                 "upload") ||
        !cuda_ok(cudaMemcpyAsync(dargs, args.data(), sizeof(BoxArg) * size_t(n), cudaMemcpyHostToDevice, s), err,
                 "upload"))
        return ST_CUDA;
    k_boxes<OP_LOAD_COUNTS><<<n, kScanThreads, 0, s>>>(dboxes, dargs, n, 1);
    k_boxes<OP_LOAD_SPHERES><<<n * per, 256, 0, s>>>(dboxes, dargs, n, per);
    k_boxes<OP_LOAD_CHECK><<<n * per, 256, 0, s>>>(dboxes, dargs, n, per);
    k_boxes<OP_GRID_CLEAR><<<n * per, 256, 0, s>>>(dboxes, dargs, n, per);
    k_boxes<OP_GRID_FILL><<<n * per, 256, 0, s>>>(dboxes, dargs, n, per);
    k_boxes<OP_FINE_LINK><<<n * per, 256, 0, s>>>(dboxes, dargs, n, per);
    k_gather_scalars<<<(n + 255) / 256, 256, 0, s>>>(dboxes, n, dsc);
    if (!cuda_ok(cudaGetLastError(), err, "state load") ||
        !cuda_ok(cudaMemcpyAsync(sc.data(), dsc, sizeof(DevScalars) * size_t(n), cudaMemcpyDeviceToHost, s), err,
                 "status") ||
        !cuda_ok(cudaStreamSynchronize(s), err, "sync"))
        return ST_CUDA;
    for (int i = 0; i < n; ++i) {
        const DevScalars &c = sc[size_t(i)];
        if (c.status == ST_BAD_ARGUMENT) {
            if (err) *err = "box " + std::to_string(i) + ": " + load_error_text(c.pad[0]);
            return ST_BAD_ARGUMENT;
        }
        if (c.status == ST_CAPACITY || c.cell_overflow) {  // a crowded Verlet cell: a larger grid for this box
            int rc = boxes[size_t(i)]->rebuild_grid(2 * plans[size_t(i)].cell_cap, err);
            if (rc != ST_OK) {
                if (err) *err = "box " + std::to_string(i) + ": " + *err;
                return rc;
            }
        } else if (c.status != ST_OK) {
            if (err) *err = "box " + std::to_string(i) + ": status " + std::to_string(c.status);
            return c.status;
        }
    }
    *out = std::move(boxes);
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

int DeviceBox::set_volsurf(int method) {
    // the exact SBL and ARVO back-ends are optional libraries of the
    // reference, which stops with their error codes when they are absent
    // (aggregat.cpp:329-346)
    if (method == VS_SBL) return ST_SBL;
    if (method == VS_ARVO) return ST_ARVO;
    if (method != VS_NONE && method != VS_CAPS && method != VS_ALPHAS) return ST_INPUT;
    static_cast<DevBox *>(devbox_)->volsurf = method;
    return ST_OK;
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
    k_box<OP_GRID_CLEAR><<<clear_blocks, 256, 0, s>>>(b, BoxArg{0, 0});
    k_box<OP_GRID_FILL><<<slot_blocks, 256, 0, s>>>(b, BoxArg{0, 0});
    if (b.fine_div > 0) k_box<OP_FINE_LINK><<<slot_blocks, 256, 0, s>>>(b, BoxArg{0, 0});
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
    int dev = 0, n_sm = 0;
    if (!cuda_ok(cudaGetDevice(&dev), err, "cudaGetDevice")) return ST_CUDA;
    if (!cuda_ok(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev), err, "device attribute"))
        return ST_CUDA;
    static bool attrs = false;
    if (!attrs) {
        auto set = [&](const void *k) {
            return cuda_ok(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(QuerySmem))),
                           err, "cudaFuncSetAttribute") &&
                   cuda_ok(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100), err,
                           "cudaFuncSetAttribute");
        };
        if (!set((const void *)k_query_batch<64>) || !set((const void *)k_query_batch<128>) ||
            !set((const void *)k_query_batch<256>))
            return ST_CUDA;
        attrs = true;
    }
    // blocks of each size the GPU holds at once; the scratch is sized for
    // the most of them
    auto resident = [&](int nt, int *blocks) {
        int per_sm = 0;
        cudaError_t e = nt == 64    ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_query_batch<64>, 64,
                                                                                    sizeof(QuerySmem))
                        : nt == 128 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_query_batch<128>, 128,
                                                                                    sizeof(QuerySmem))
                                    : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_query_batch<256>, 256,
                                                                                    sizeof(QuerySmem));
        *blocks = std::max(1, std::min(n, std::max(1, per_sm) * std::max(1, n_sm)));
        return cuda_ok(e, err, "occupancy");
    };
    int blocks = 1;
    for (int nt : kBatchThreadChoices) {
        int nb = 1;
        if (!resident(nt, &nb)) return ST_CUDA;
        blocks = std::max(blocks, nb);
    }

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
    auto launch = [&](int nt, float *ms) {
        int nb = 1;
        if (!resident(nt, &nb)) return false;
        if (!cuda_ok(cudaMemsetAsync(sc.next, 0, sizeof(int), s), err, "query counter")) return false;
        cudaEventRecord(e0, s);
        if (nt == 64)
            k_query_batch<64><<<nb, 64, sizeof(QuerySmem), s>>>(b, sc, n, d_in, d_out);
        else if (nt == 128)
            k_query_batch<128><<<nb, 128, sizeof(QuerySmem), s>>>(b, sc, n, d_in, d_out);
        else
            k_query_batch<256><<<nb, 256, sizeof(QuerySmem), s>>>(b, sc, n, d_in, d_out);
        cudaEventRecord(e1, s);
        if (!cuda_ok(cudaGetLastError(), err, "k_query_batch") || !cuda_ok(cudaEventSynchronize(e1), err, "k_query_batch"))
            return false;
        cudaEventElapsedTime(ms, e0, e1);
        return true;
    };
    float ms = 0.f;
    if (ok && batch_threads_ == 0 && n >= 1024) {
        // the first large batch: each block size on the same queries (they
        // only read the box), the fastest kept
        float best = 0.f;
        for (int nt : kBatchThreadChoices) {
            float t = 0.f;
            ok = ok && launch(nt, &t);
            if (ok && (best == 0.f || t < best)) {
                best = t;
                batch_threads_ = nt;
            }
        }
        ms = best;
    } else if (ok) {
        ok = launch(batch_threads_ ? batch_threads_ : 256, &ms);
    }
    ok = ok &&
         cuda_ok(cudaMemcpyAsync(hout.data(), d_out, sizeof(QueryOut) * size_t(n), cudaMemcpyDeviceToHost, s), err,
                 "query download") &&
         cuda_ok(cudaStreamSynchronize(s), err, "k_query_batch");
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

int DeviceBox::grow(int slot, double du, std::string *err) {
    DevBox &b = *static_cast<DevBox *>(devbox_);
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    k_grow<<<slot >= 0 ? 1 : std::max(1, std::min(1024, (b.pool_cap + 255) / 256)), 256, 0, s>>>(b, slot, du);
    if (!cuda_ok(cudaGetLastError(), err, "k_grow")) return ST_CUDA;
    return ST_OK;
}

int DeviceBox::update_geometry(int slot, bool full, std::vector<double> *agg, std::vector<double> *vol_pp,
                               std::string *err) {
    DevBox &b = *static_cast<DevBox *>(devbox_);
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    const int slot_blocks = std::max(1, std::min(1024, (b.nslots + 255) / 256));
    // query scratch, free between queries: the mean sphere volumes and the moved slots
    if (!cuda_ok(cudaMemsetAsync(b.counters + 5, 0, sizeof(int), s), err, "memset")) return ST_CUDA;
    k_update_geometry<<<slot >= 0 ? 1 : slot_blocks, 256, 0, s>>>(b, slot, full ? 1 : 0, b.cand_db, b.cand_slot);
    k_regrid_moved<<<1, 1, 0, s>>>(b, b.cand_slot);
    if (!cuda_ok(cudaGetLastError(), err, "k_update_geometry")) return ST_CUDA;
    agg->resize(size_t(21) * size_t(b.nslots));
    vol_pp->resize(size_t(b.nslots));
    if (!cuda_ok(cudaMemcpyAsync(agg->data(), b.agg, sizeof(double) * agg->size(), cudaMemcpyDeviceToHost, s), err,
                 "download") ||
        !cuda_ok(cudaMemcpyAsync(vol_pp->data(), b.cand_db, sizeof(double) * vol_pp->size(), cudaMemcpyDeviceToHost,
                                 s),
                 err, "download") ||
        !cuda_ok(cudaStreamSynchronize(s), err, "sync"))
        return ST_CUDA;
    return check_status(err);
}

int DeviceBox::set_maxradius(double r, std::string *err) {
    DevBox &b = *static_cast<DevBox *>(devbox_);
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    // the value is read before the call returns (synchronised below)
    if (!cuda_ok(cudaMemcpyAsync(&b.sc->maxradius, &r, sizeof(double), cudaMemcpyHostToDevice, s), err, "upload") ||
        !cuda_ok(cudaStreamSynchronize(s), err, "sync"))
        return ST_CUDA;
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

int DeviceBox::n_alive(int *n, std::string *err) {
    DevBox &b = *static_cast<DevBox *>(devbox_);
    cudaStream_t s = static_cast<cudaStream_t>(stream_);
    DevScalars sc;
    if (!cuda_ok(cudaMemcpyAsync(&sc, b.sc, sizeof(sc), cudaMemcpyDeviceToHost, s), err, "download") ||
        !cuda_ok(cudaStreamSynchronize(s), err, "sync"))
        return ST_CUDA;
    *n = sc.n_alive;
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
    if (na == 0) {  // every sphere oxidised: an empty state
        out->n_spheres = 0;
        out->n_aggregates = 0;
        out->n_verlet_divisions = b.n_div;
        out->box_length = b.L;
        out->maxradius = sc.maxradius;
        out->time = sc.time;
        return ST_OK;
    }
    if (out->n_spheres < b.ns || out->n_aggregates < na || na < 1) {
        if (err) *err = "state buffers too small";
        return ST_BAD_ARGUMENT;
    }
    if (pack_layout(na, b.ns, b.nslots).total > stage_bytes_) {
        if (err) *err = "store staging area too small";
        return ST_CAPACITY;
    }
    const PackStage ps = pack_stage(b, na, sc.pool_sel);
    const BoxArg pa{na, sc.pool_sel};
    const int blocks = std::min(1024, (std::max(b.ns, b.nslots) + 255) / 256);
    k_box<OP_PACK_RANKS><<<1, kScanThreads, 0, cs>>>(b, pa);
    k_box<OP_PACK><<<blocks, 256, 0, cs>>>(b, pa);
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

int DeviceBox::store_many(const std::vector<DeviceBox *> &boxes, const std::vector<mcacg_state *> &outs,
                          void *stream, std::vector<int> *rcs, std::vector<std::string> *errs, std::string *err) {
    const int n = int(boxes.size());
    rcs->assign(size_t(n), ST_OK);
    errs->assign(size_t(n), std::string());
    if (n == 0) return ST_OK;
    if (outs.size() != boxes.size()) {
        if (err) *err = "one state per box is needed";
        return ST_BAD_ARGUMENT;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::vector<DevBox> host_boxes(static_cast<size_t>(n));
    int max_items = 0;
    for (int i = 0; i < n; ++i) {
        if (!cuda_ok(cudaStreamSynchronize(static_cast<cudaStream_t>(boxes[size_t(i)]->stream_)), err, "sync"))
            return ST_CUDA;
        host_boxes[size_t(i)] = *static_cast<DevBox *>(boxes[size_t(i)]->devbox_);
        max_items = std::max({max_items, host_boxes[size_t(i)].ns, host_boxes[size_t(i)].nslots});
    }
    const size_t tb = (sizeof(DevBox) * size_t(n) + 255) & ~size_t(255);
    const size_t ta = (sizeof(BoxArg) * size_t(n) + 255) & ~size_t(255);
    char *tmp = nullptr;
    if (!cuda_ok(cudaMalloc((void **)&tmp, tb + ta + sizeof(DevScalars) * size_t(n)), err, "cudaMalloc")) return ST_CUDA;
    std::unique_ptr<char, void (*)(char *)> tmp_owner(tmp, [](char *p) { cudaFree(p); });
    DevBox *dboxes = reinterpret_cast<DevBox *>(tmp);
    BoxArg *dargs = reinterpret_cast<BoxArg *>(tmp + tb);
    DevScalars *dsc = reinterpret_cast<DevScalars *>(tmp + tb + ta);
    std::vector<DevScalars> sc(static_cast<size_t>(n));
    if (!cuda_ok(cudaMemcpyAsync(dboxes, host_boxes.data(), sizeof(DevBox) * size_t(n), cudaMemcpyHostToDevice, s),
                 err, "store"))
        return ST_CUDA;
    k_gather_scalars<<<(n + 255) / 256, 256, 0, s>>>(dboxes, n, dsc);
    if (!cuda_ok(cudaGetLastError(), err, "store") ||
        !cuda_ok(cudaMemcpyAsync(sc.data(), dsc, sizeof(DevScalars) * size_t(n), cudaMemcpyDeviceToHost, s), err,
                 "store") ||
        !cuda_ok(cudaStreamSynchronize(s), err, "sync"))
        return ST_CUDA;
    // per box: the live count, or -1 for a box that cannot be stored or has
    // no aggregate left (every sphere oxidised: an empty state)
    std::vector<BoxArg> args(static_cast<size_t>(n));
    std::vector<char> empty(static_cast<size_t>(n), 0);
    for (int i = 0; i < n; ++i) {
        const DevBox &b = host_boxes[size_t(i)];
        const mcacg_state *o = outs[size_t(i)];
        const int na = sc[size_t(i)].n_alive;
        args[size_t(i)] = BoxArg{-1, sc[size_t(i)].pool_sel};
        if (!o || !o->spheres || !o->sphere_label || !o->aggregates || !o->n_spheres_per_aggregate || !o->members) {
            (*rcs)[size_t(i)] = ST_BAD_ARGUMENT;
            (*errs)[size_t(i)] = "incomplete state buffers";
        } else if (na == 0) {
            empty[size_t(i)] = 1;
        } else if (o->n_spheres < b.ns || o->n_aggregates < na || na < 1) {
            (*rcs)[size_t(i)] = ST_BAD_ARGUMENT;
            (*errs)[size_t(i)] = "state buffers too small";
        } else if (pack_layout(na, b.ns, b.nslots).total > boxes[size_t(i)]->stage_bytes_) {
            (*rcs)[size_t(i)] = ST_CAPACITY;
            (*errs)[size_t(i)] = "store staging area too small";
        } else {
            args[size_t(i)].a = na;
        }
    }
    const int per = blocks_per_box(n, max_items);
    if (!cuda_ok(cudaMemcpyAsync(dargs, args.data(), sizeof(BoxArg) * size_t(n), cudaMemcpyHostToDevice, s), err,
                 "store"))
        return ST_CUDA;
    k_boxes<OP_PACK_RANKS><<<n, kScanThreads, 0, s>>>(dboxes, dargs, n, 1);
    k_boxes<OP_PACK><<<n * per, 256, 0, s>>>(dboxes, dargs, n, per);
    if (!cuda_ok(cudaGetLastError(), err, "store")) return ST_CUDA;
    // the copies, spread over a few streams after the packing
    CopyStreams copies(kCopyStreams);
    if (!copies.fork(s)) {
        if (err) *err = "copy streams";
        return ST_CUDA;
    }
    cudaStream_t cs = s;
    auto get = [&](void *dst, const void *src, size_t bytes) {
        return cuda_ok(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, cs), err, "store");
    };
    for (int i = 0; i < n; ++i) {
        const int na = args[size_t(i)].a;
        if (na < 0) continue;
        const DevBox &b = host_boxes[size_t(i)];
        const PackStage ps = pack_stage(b, na, args[size_t(i)].b);
        mcacg_state *o = outs[size_t(i)];
        cs = copies.at(size_t(i), s);
        if (!(get(o->spheres, b.sph, sizeof(double) * 9 * size_t(b.ns)) &&
              get(o->sphere_label, ps.label, 8 * size_t(b.ns)) && get(o->aggregates, ps.agg, 168 * size_t(na)) &&
              get(o->n_spheres_per_aggregate, ps.count, 8 * size_t(na)) &&
              get(o->members, ps.members, 8 * size_t(b.ns))))
            return ST_CUDA;
    }
    if (!copies.join(s) || !cuda_ok(cudaStreamSynchronize(s), err, "sync")) return ST_CUDA;
    for (int i = 0; i < n; ++i) {
        if (args[size_t(i)].a < 0 && !empty[size_t(i)]) continue;
        const DevBox &b = host_boxes[size_t(i)];
        mcacg_state *o = outs[size_t(i)];
        o->n_spheres = empty[size_t(i)] ? 0 : b.ns;
        o->n_aggregates = empty[size_t(i)] ? 0 : args[size_t(i)].a;
        o->n_verlet_divisions = b.n_div;
        o->box_length = b.L;
        o->maxradius = sc[size_t(i)].maxradius;
        o->time = sc[size_t(i)].time;
    }
    return ST_OK;
}

}  // namespace mcacg
