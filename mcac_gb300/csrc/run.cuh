// Device-resident MC loop: one thread block advances one box for many steps
// without returning to the host (the batched / served form).
//
// Per step (src/calcul.cpp:94-281):
//   pick   a slot with probability 1/time_step / sum(1/time_step), by a
//          descent of a 32-ary FP64 sum tree (warp-wide scans), and advance
//          time by 1 / sum(1/time_step) -- the reference's
//          max / sum(max / time_step), rearranged;
//   move   random direction from the box's own C-library rand() stream,
//          contact search (block_query), translation (block_translate);
//   merge  block_merge, then the aggregate physics of update_partial
//          (erf/exp/pow from CUDA's libm) and two tree updates;
//   with surface reactions, the spheres grow or shrink before the merge
//   (oxidation: removals, disappearances, splits) and the aggregates are
//   updated after it.
// The contact search and merge geometry are the exact kernels of the
// single-box path; pick order and libm differ from the reference, so runs
// agree with it statistically, not step by step (the host-driven loop is the
// bit-exact form).
#pragma once
#include "box.cuh"
#include "merge.cuh"
#include "rng.hpp"

namespace mcacg {

constexpr int kTreeFan = 32;
constexpr int kMaxTreeLevels = 8;

struct PhysParams {
    double viscosity, lambda, fractal_dimension, density, temperature;
    double u_sg;        // surface growth velocity dr/dt (m/s)
    double inv_lambda, inv_fractal_dimension;
    int growth;         // with_surface_reactions
    int individual;     // individual_surf_reactions: only the moved aggregate grows and is updated
    int full_update_every;  // full_aggregate_update_frequency
    int oxidation;      // growth with u_sg < 0: spheres at or below rp_min leave, aggregates split
    double rp_min;      // rp_min_oxid (m)
};

struct RunLimits {
    long long number_of_aggregates_limit, n_iter_without_event_limit, mean_monomere_per_aggregate_limit;
    double physical_time_limit;
    int with_collisions;
    int pad;
};

// Mutable loop state of one box (device memory).
struct RunState {
    RandStream rng;
    double time;
    double weight_total;     // sum over live slots of 1/time_step
    double inv_weight;       // 1 / weight_total (the step's time increment)
    double tree_scale;       // pick tree weights are round(scale / time_step), scale a power of 2
    double inv_tree_scale;
    unsigned long long tree_total;  // the pick tree's integer total
    long long steps, events, n_iter_without_event;
    int finished;
    int status;
    int removed_spheres;  // spheres taken out by oxidation
    int splits;           // aggregates split by oxidation
    // work counters of the contact queries and merges (algorithmic bytes)
    long long c_queries, c_mov, c_scanned, c_cells, c_candidates, c_cand_spheres, c_refined;
    long long c_merged_spheres, c_merge_pairs;
    // SM clock cycles spent by the block in each phase of the step
    long long cyc_pick, cyc_query, cyc_move, cyc_merge;
    long long cyc_qscan, cyc_qpairs;  // parts of cyc_query
};
static_assert(sizeof(RunState) % sizeof(int) == 0, "RunState is copied as ints");

struct BoxRun {
    DevBox box;
    PhysParams phys;
    RunLimits lim;
    RunState *st;
    unsigned long long *tree;  // all levels, leaves first (fixed-point weights)
    int tree_levels;
    int live_max;  // the loop keeps a live list from this many live aggregates down (0: never)
    int tree_off[kMaxTreeLevels];
    int tree_len[kMaxTreeLevels];
};

constexpr int kMovedCap = 64;  // grid moves listed per update of all aggregates

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The top levels of a box's pick tree (up to kTreeCache entries) are kept in
// shared memory for a launch: the descent then reads global memory only for
// the lower levels. coff[lev] is the level's offset in the copy, -1 if the
// level is not kept.
template <int N>
struct TreeCacheT {
    static constexpr int kCap = N;
    unsigned long long v[N];
    int coff[kMaxTreeLevels];
};
// one warp per box (16 boxes an SM): 128 entries; larger blocks: 640, so
// that the two levels above the leaves of a box of up to ~20 000 slots stay
// on chip and a pick reads one level of the tree from device memory
using TreeCache = TreeCacheT<128>;
using TreeCacheLarge = TreeCacheT<640>;
// The tree's weights are integers: the live slots' 1/time_step times a power
// of 2 chosen at each rebuild so that the total stays below 2^62, rounded,
// and at least 1 (relative rounding below 1e-13 at 1e5 slots). Sums are then
// exact in any order and the descent runs on the integer pipes: FP64 is
// scarce on this GPU. The pick follows the weights as the FP64 sums did, up
// to that rounding (the device loop follows the reference statistically).
constexpr unsigned long long kTreeHeadroom = 1ULL << 62;


template <class QS, class MS, class TC, class LL>
struct RunSmemT {
    union {
        QS q;
        MS m;
    } u;
    MergeOut mout;
    double refpos[3];
    double dir[3];
    unsigned long long t_pick;  // pick target in the tree's fixed point
    unsigned long long deadline;  // %globaltimer time after which no step starts (0: none)
    double dt, full, move;
    int slot, contact, stop, merged, rescale;
    int keep, removed;
    int ms, os, oslot;  // contact of this step: spheres and the other slot
    unsigned long long tree_tmp;  // block reduction scratch
    double step_dt;               // this step's time increment
    double dt_indiv, step_dt_indiv;  // the moved aggregate's own time step, and its increment
    int n_moved;                  // slots whose grid cell changed in the update of all aggregates
    int moved[kMovedCap];
    TC tree;                      // top levels of the pick tree
    LL live;                      // the live slots when few are left (box.cuh)
    int split, disappear;         // this step's oxidation events
};
using RunSmem = RunSmemT<QuerySmem, MergeSmem, TreeCacheLarge, LiveList>;
using RunSmemSmall = RunSmemT<QuerySmemSmall, MergeSmemSmall, TreeCache, LiveListNone>;

// ------------------------------------------------------------ sum tree
// Marks the kept levels and copies them (all threads).
template <class TC>
__device__ inline void tree_cache_load(const BoxRun &R, TC &c) {
    if (threadIdx.x == 0) {
        int used = 0;
        for (int lev = kMaxTreeLevels - 1; lev >= 0; --lev) c.coff[lev] = -1;
        for (int lev = R.tree_levels - 1; lev >= 0; --lev) {
            if (used + R.tree_len[lev] > TC::kCap) break;
            c.coff[lev] = used;
            used += R.tree_len[lev];
        }
    }
    __syncthreads();
    for (int lev = 0; lev < R.tree_levels; ++lev) {
        if (c.coff[lev] < 0) continue;
        for (int k = threadIdx.x; k < R.tree_len[lev]; k += blockDim.x) c.v[c.coff[lev] + k] = R.tree[R.tree_off[lev] + k];
    }
    __syncthreads();
}

// Warp 0: descend from the top level to a leaf holding the target 't'
// (0 <= t < total).
template <class TC>
__device__ inline int tree_sample(const BoxRun &R, const TC &c, unsigned long long t) {
    const int lane = threadIdx.x & 31;
    int node = 0;  // index within the current level
    for (int lev = R.tree_levels - 1; lev >= 0; --lev) {
        const int base = node * kTreeFan;
        const int len = R.tree_len[lev];
        const int co = c.coff[lev];
        const unsigned long long v =
            (base + lane < len) ? (co >= 0 ? c.v[co + base + lane] : R.tree[R.tree_off[lev] + base + lane]) : 0ULL;
        // inclusive scan over the 32 children (fixed order)
        unsigned long long incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const unsigned over = __ballot_sync(0xffffffffu, incl > t && v > 0ULL);
        const unsigned nonzero = __ballot_sync(0xffffffffu, v > 0ULL);
        const int pick = over ? __ffs(over) - 1 : (nonzero ? 31 - __clz(nonzero) : 0);
        t -= __shfl_sync(0xffffffffu, incl - v, pick);
        node = base + pick;
    }
    return node;
}

// The pick's target in the tree's fixed point from one rand() value r:
// floor(total * r / 2^31), below the total.
__device__ __forceinline__ unsigned long long pick_target(RandStream &rng, unsigned long long total) {
    const unsigned long long r = static_cast<unsigned long long>(rng.next_int());
    return (__umul64hi(r, total) << 33) | ((r * total) >> 31);
}

// random_direction (tools.cpp:82-89): theta = 2 pi u1, phi = acos(1 - 2 u2),
// from two rand() values. cos(phi) is 1 - 2 u2 itself and sin(phi) =
// 2 sqrt(u2 (1 - u2)). The angles are drawn in FP32 (the device loop follows
// the reference statistically; FP64 is scarce on this GPU) and the vector is
// brought to unit length in FP64 by one Newton step on its norm: with
// |d|^2 = 1 + e, e ~ 1e-7, the factor 1.5 - 0.5 |d|^2 leaves
// |d| - 1 ~ 3e^2/8 < 1e-13, far inside the 1e-10 contact tolerance of the
// merge.
__device__ __forceinline__ void direction_from(int r1, int r2, double d[3]) {
    const float u1 = float(r1) * (1.0f / 2147483647.0f), u2 = float(r2) * (1.0f / 2147483647.0f);
    const float cpf = 1.f - 2.f * u2;
    const float spf = 2.f * sqrtf(u2 * (1.f - u2));
    float sth, cth;
    sincospif(2.f * u1, &sth, &cth);
    const double dx = double(spf * cth), dy = double(spf * sth), dz = double(cpf);
    const double k = 1.5 - 0.5 * (dx * dx + dy * dy + dz * dz);
    d[0] = dx * k;
    d[1] = dy * k;
    d[2] = dz * k;
}
// The same from the stream's next two values (u1 first).
__device__ __forceinline__ void draw_direction(RandStream &rng, double d[3]) {
    const int r1 = rng.next_int();
    const int r2 = rng.next_int();
    direction_from(r1, r2, d);
}

// The fixed-point weight of a slot with this time step (live slots only).
__device__ __forceinline__ unsigned long long tree_weight(const RunState &st, double time_step) {
    const double w = fmin((1.0 / time_step) * st.tree_scale, double(kTreeHeadroom));
    const unsigned long long q = __double2ull_rn(w);
    return q > 0ULL ? q : 1ULL;
}

// Warp 0: set leaf 'slot' to 'w' and refresh its ancestors (in global
// memory and in the kept copy); returns the new total.
template <class TC>
__device__ inline unsigned long long tree_set(const BoxRun &R, TC &c, int slot, unsigned long long w) {
    const int lane = threadIdx.x & 31;
    if (lane == 0) {
        R.tree[R.tree_off[0] + slot] = w;
        if (c.coff[0] >= 0) c.v[c.coff[0] + slot] = w;
    }
    __syncwarp();
    int idx = slot;
    unsigned long long total = 0ULL;
    for (int lev = 0; lev < R.tree_levels; ++lev) {
        const int g = idx / kTreeFan;
        const int len = R.tree_len[lev];
        const int co = c.coff[lev];
        const int k = g * kTreeFan + lane;
        unsigned long long v = (k < len) ? (co >= 0 ? c.v[co + k] : R.tree[R.tree_off[lev] + k]) : 0ULL;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lev + 1 < R.tree_levels) {
            if (lane == 0) {
                R.tree[R.tree_off[lev + 1] + g] = v;
                if (c.coff[lev + 1] >= 0) c.v[c.coff[lev + 1] + g] = v;
            }
            __syncwarp();
        } else {
            total = v;
        }
        idx = g;
    }
    return total;
}

// The loop state's FP64 total weight and its inverse (the time increment of
// a step) from the tree's integer total.
__device__ __forceinline__ void tree_total_to_state(RunState &st, unsigned long long total) {
    st.tree_total = total;
    st.weight_total = double(total) * st.inv_tree_scale;
    st.inv_weight = 1.0 / st.weight_total;
}

// ------------------------------------------------------------ live list
// (Re)builds the list of live slots in slot order with their tree leaf
// weights when at most live.max aggregates are left (all threads); turns it
// off otherwise. The pick and the query then read the list.
template <class LL>
__device__ inline void live_load(const BoxRun &R, LL &L, int *warp_tmp) {
    const DevBox &b = R.box;
    const int tid = threadIdx.x, NT = blockDim.x;
    const int n_alive = b.sc->n_alive;
    const bool want = L.allow && !R.phys.growth && n_alive <= L.max && L.max <= LL::kCap;
    __syncthreads();
    if (!want) {
        if (tid == 0) L.on = 0;
        __syncthreads();
        return;
    }
    // ordered compaction: each thread a contiguous run of slots
    const int per = (b.nslots + NT - 1) / NT;
    const int lo = min(b.nslots, tid * per), hi = min(b.nslots, lo + per);
    int c = 0;
    for (int a = lo; a < hi; ++a) c += b.agg_n[a] > 0;
    int total = 0;
    int k = block_exclusive_scan(c, warp_tmp, total);
    if (total <= LL::kCap) {
        for (int a = lo; a < hi; ++a) {
            if (b.agg_n[a] > 0) {
                L.slot[k] = a;
                L.w[k] = R.tree[R.tree_off[0] + a];
                ++k;
            }
        }
    }
    if (tid == 0) {
        L.n = total;
        L.on = total <= LL::kCap ? 1 : 0;
    }
    __syncthreads();
}

// Warp 0: the first listed slot whose running weight (in slot order)
// exceeds t -- the leaf the tree's descent reaches for the same target,
// the weights being the tree's exact integers.
template <class LL>
__device__ inline int live_sample(const LL &L, unsigned long long t) {
    static_assert(LL::kCap <= 128, "four entries a lane");
    const int lane = threadIdx.x & 31;
    unsigned long long v[4];
    unsigned long long sum = 0ULL;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int i = 4 * lane + j;
        v[j] = i < L.n ? L.w[i] : 0ULL;
        sum += v[j];
    }
    unsigned long long incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    const unsigned over = __ballot_sync(0xffffffffu, incl > t);
    const int src = over ? __ffs(over) - 1 : 31;
    int idx = -1;
    if (lane == src) {
        unsigned long long run = incl - sum;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            run += v[j];
            if (idx < 0 && v[j] > 0ULL && run > t) idx = 4 * lane + j;
        }
    }
    idx = __shfl_sync(0xffffffffu, idx, src);
    return (idx >= 0 && idx < L.n) ? L.slot[idx] : -1;
}

// After a merge (thread 0): the removed slot leaves the list, the kept one
// takes its new weight.
template <class LL>
__device__ inline void live_merge(LL &L, int keep, int removed, unsigned long long w_keep) {
    int j = 0;
    for (int i = 0; i < L.n; ++i) {
        const int s = L.slot[i];
        if (s == removed) continue;
        L.slot[j] = s;
        L.w[j] = s == keep ? w_keep : L.w[i];
        ++j;
    }
    L.n = j;
}

// ------------------------------------------------------------ physics
// update_partial's physics (aggregat.cpp:264-276, physical_model.cpp:550-617):
// friction, mobility diameter, time step and mean free path, in FP32 with
// CUDA's erff / expf / powf. FP64 runs at 1/64 of the FP32 rate on this
// part, and one merge's physics took ~10 us of FP64 (four transcendental
// functions, divisions and a square root on one thread); these values only
// set the loop's rates, which it follows statistically. Relative error of
// the results about 1e-6 (a few FP32 roundings and the functions' 1-2 ulp);
// the values stay far inside FP32's range (f ~1e-12..1e-6 kg/s, time steps
// ~1e-9..1e-2 s). The common factors are taken once: one pow (its square
// root form squared) and the reciprocals of the gas mean free path and of
// the fractal dimension from the host. dg/dp, a geometric ratio, stays FP64.
__device__ inline void device_physics(const PhysParams &p, double V, double vol_pp, double dp, double rg, double *f_agg,
                               double *d_m, double *time_step, double *lpm, double *dg_over_dp) {
    const float r = float(0.5 * dp);
    const float a = 1.142f, b = 0.558f, c = 0.999f;
    const float lambda = float(p.lambda), inv_lambda = float(p.inv_lambda);
    const float lr = lambda / r;
    const float fe = 0.689f * (1.f + erff((lr + 4.454f) * (1.f / 10.628f)));
    const float cc = 1.f + lr * (a + b * expf(-c * r * inv_lambda));
    const float ratio = float(V) / float(vol_pp);
    const float pw2 = powf(ratio, 0.5f * fe * float(p.inv_fractal_dimension));
    const float pw = pw2 * pw2;
    const float f = (6.f * float(pi_value()) * float(p.viscosity) * r / cc) * pw;
    const float ar = r * pw2;
    const float cc_a = 1.f + (lambda / ar) * (a + b * expf(-c * ar * inv_lambda));
    const float ts = 3.f * (float(p.density) * float(V)) / f;
    *f_agg = double(f);
    *d_m = double((cc_a / cc) * 2.f * r * pw);
    *time_step = double(ts);
    *lpm = double(sqrtf(6.f * float(kBoltzmann) * float(p.temperature) / f * ts));
    *dg_over_dp = rg / (0.5 * dp);
}

__device__ __forceinline__ bool run_finished(const BoxRun &R, const RunState &st, int n_alive) {
    const RunLimits &L = R.lim;
    if (n_alive < 1) return true;
    if (static_cast<unsigned long long>(n_alive) <= static_cast<unsigned long long>(L.number_of_aggregates_limit))
        return true;
    if (L.n_iter_without_event_limit > 0 && st.n_iter_without_event >= L.n_iter_without_event_limit) return true;
    if (L.physical_time_limit > 0 && st.time >= L.physical_time_limit) return true;
    if (L.mean_monomere_per_aggregate_limit > 0 &&
        double(R.box.ns - st.removed_spheres) / double(n_alive) >= double(L.mean_monomere_per_aggregate_limit))
        return true;
    return false;
}

// One MC step of one box by the whole block. Returns false when the box is
// finished or in error (then nothing was done).
// ------------------------------------------------------ surface growth
// Sphere::croissance_surface (sphere.cpp:113-120) for every sphere of the box:
// r += u_sg dt, volume and surface from the new radius. Each sphere is found
// once through the live segments of the member pool, whose FP32 copy is
// refreshed too.
// With oxidation, b.counters[3] is set when a sphere ends at or below rp_min.
__device__ inline void block_grow_spheres(const BoxRun &R, double dt) {
    const DevBox &b = R.box;
    const double pi = pi_value();
    const double vf = 4. * pi / 3., sf = 4. * pi;
    const int *pool_id = b.pool_id[b.sc->pool_sel];
    float4 *pool_pos = b.pool_pos[b.sc->pool_sel];
    const int top = b.sc->pool_top;
    for (int k = threadIdx.x; k < top; k += blockDim.x) {
        const int s = pool_id[k];
        if (s < 0 || s >= b.ns) continue;
        const int a = b.sph_slot[s];
        if (a < 0 || a >= b.nslots) continue;  // a sphere removed by oxidation
        const int rel = k - b.agg_off[a];
        if (b.agg_n[a] == 0 || rel < 0 || rel >= b.agg_n[a]) continue;  // a stale pool entry
        const double r = S(b, SPH_R, s) + R.phys.u_sg * dt;                // PhysicalModel::grow
        const double r2 = r * r, r3 = r2 * r;
        S(b, SPH_R, s) = r;
        S(b, SPH_VOLUME, s) = vf * r3;
        S(b, SPH_SURFACE, s) = sf * r2;
        pool_pos[k].w = float(r);
        if (R.phys.oxidation && r <= R.phys.rp_min) b.counters[3] = 1;
    }
}

// SphereList::croissance_surface (sphere_list.cpp:81-87) of one slot's
// spheres: the individual mode grows only the moved aggregate, by its own
// time step (calcul.cpp:108, 148, 159-160).
__device__ inline void block_grow_slot(const BoxRun &R, int slot, double dt) {
    const DevBox &b = R.box;
    const double pi = pi_value();
    const double vf = 4. * pi / 3., sf = 4. * pi;
    const int *pool_id = b.pool_id[b.sc->pool_sel];
    float4 *pool_pos = b.pool_pos[b.sc->pool_sel];
    const int off = b.agg_off[slot], n = b.agg_n[slot];
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const int s = pool_id[off + k];
        const double r = S(b, SPH_R, s) + R.phys.u_sg * dt;  // PhysicalModel::grow
        const double r2 = r * r, r3 = r2 * r;
        S(b, SPH_R, s) = r;
        S(b, SPH_VOLUME, s) = vf * r3;
        S(b, SPH_SURFACE, s) = sf * r2;
        pool_pos[off + k].w = float(r);
    }
}

// Aggregate::update / update_partial (aggregat.cpp:247-288) of one slot by
// one thread: the geometry (thread_update_geometry), then the physics fields
// in FP32 (device_physics). Returns r_max.
__device__ inline double thread_update_aggregate(const BoxRun &R, int a, bool full) {
    const DevBox &b = R.box;
    double vol_pp = 0.0;
    const double rmax = thread_update_geometry(b, a, full, &vol_pp);
    double f, dm, ts, lpm, dgdp;
    device_physics(R.phys, A(b, AGG_VOLUME, a), vol_pp, A(b, AGG_DP, a), A(b, AGG_RG, a), &f, &dm, &ts, &lpm, &dgdp);
    A(b, AGG_F_AGG, a) = f;
    A(b, AGG_D_M, a) = dm;
    A(b, AGG_TIME_STEP, a) = ts;
    A(b, AGG_LPM, a) = lpm;
    A(b, AGG_DG_OVER_DP, a) = dgdp;
    return rmax;
}

// The pick tree from the time steps: the scale from the largest weight and
// the live count, leaves of the live slots (0 elsewhere), then each level
// from the one below, and the total into the loop state. The FP64 weights
// sit in the leaves (as bits) between the two passes.
__device__ inline void block_tree_build(const BoxRun &R) {
    const DevBox &b = R.box;
    const int tid = threadIdx.x, NT = blockDim.x;
    __shared__ unsigned long long max_bits;
    __shared__ int n_live;
    if (tid == 0) {
        max_bits = 0ULL;
        n_live = 0;
    }
    __syncthreads();
    unsigned long long mb = 0ULL;  // non-negative doubles order like their bits
    int live = 0;
    for (int a = tid; a < R.tree_len[0]; a += NT) {
        double w = 0.0;
        if (a < b.nslots && b.agg_n[a] > 0) {
            w = 1.0 / A(b, AGG_TIME_STEP, a);
            ++live;
        }
        const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(w));
        R.tree[R.tree_off[0] + a] = bits;
        mb = bits > mb ? bits : mb;
    }
    atomicMax(&max_bits, mb);
    atomicAdd(&n_live, live);
    __syncthreads();
    if (tid == 0) {
        // n_live * max weight * scale < 2^62
        int e = 0;
        frexp(double(n_live > 0 ? n_live : 1) * __longlong_as_double(static_cast<long long>(max_bits)), &e);
        const int k = max(-1000, min(1000, 62 - e));
        R.st->tree_scale = ldexp(1.0, k);
        R.st->inv_tree_scale = ldexp(1.0, -k);
    }
    __syncthreads();
    const double scale = R.st->tree_scale;
    for (int a = tid; a < R.tree_len[0]; a += NT) {
        const double w = __longlong_as_double(static_cast<long long>(R.tree[R.tree_off[0] + a]));
        unsigned long long q = 0ULL;
        if (w > 0.0) {
            q = __double2ull_rn(fmin(w * scale, double(kTreeHeadroom)));
            q = q > 0ULL ? q : 1ULL;
        }
        R.tree[R.tree_off[0] + a] = q;
    }
    __syncthreads();
    for (int lev = 1; lev < R.tree_levels; ++lev) {
        for (int g = tid; g < R.tree_len[lev]; g += NT) {
            unsigned long long sum = 0ULL;
            for (int k = 0; k < kTreeFan; ++k) {
                const int c = g * kTreeFan + k;
                if (c < R.tree_len[lev - 1]) sum += R.tree[R.tree_off[lev - 1] + c];
            }
            R.tree[R.tree_off[lev] + g] = sum;
        }
        __syncthreads();
    }
    if (tid == 0) {
        const int top = R.tree_levels - 1;
        unsigned long long total = 0ULL;
        for (int k = 0; k < R.tree_len[top]; ++k) total += R.tree[R.tree_off[top] + k];
        tree_total_to_state(*R.st, total);
    }
    __syncthreads();
}

// The per-step update of every aggregate after growth (calcul.cpp:180-206):
// fields, Verlet and fine cells (centres move as spheres grow unevenly),
// maxradius, and the pick tree rebuilt from the new time steps.
template <class RS>
__device__ inline void block_update_all(const BoxRun &R, RS &sm, bool full) {
    const DevBox &b = R.box;
    const int tid = threadIdx.x, NT = blockDim.x;
    double rmax_d = 0.0;
    if (tid == 0) sm.n_moved = 0;
    __syncthreads();
    for (int a = tid; a < b.nslots; a += NT) {
        if (b.agg_n[a] == 0) continue;
        const double rm = thread_update_aggregate(R, a, full);
        rmax_d = dmax(rmax_d, rm);
        // the centre moves a little when spheres grow unevenly: note the
        // slots whose Verlet or fine cell changed
        const Vec3 pa = agg_pos(b, a);
        if (cell_of(b, pa) != b.agg_cell[a] || (b.fine_div > 0 && fine_cell_of(b, pa) != b.fine_cell[a])) {
            const int k = atomicAdd(&sm.n_moved, 1);
            if (k < kMovedCap) sm.moved[k] = a;
        }
    }
    // block max of r_max (bits of a non-negative double order like integers)
    unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(rmax_d));
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(0xffffffffu, bits, o);
        bits = other > bits ? other : bits;
    }
    if (tid == 0) sm.tree_tmp = 0ULL;
    __syncthreads();
    if ((tid & 31) == 0) atomicMax(&sm.tree_tmp, bits);
    __syncthreads();
    if (tid == 0) {
        const double m = __longlong_as_double(static_cast<long long>(sm.tree_tmp));
        if (m > b.sc->maxradius) b.sc->maxradius = m;
        // the grid lists change one slot at a time, as in the translation
        if (sm.n_moved <= kMovedCap) {
            for (int k = 0; k < sm.n_moved; ++k) regrid(b, sm.moved[k], agg_pos(b, sm.moved[k]));
        } else {
            for (int a = 0; a < b.nslots; ++a)
                if (b.agg_n[a] > 0) regrid(b, a, agg_pos(b, a));
        }
    }
    __syncthreads();
    block_tree_build(R);
    tree_cache_load(R, sm.tree);
}

// The update after growth: every aggregate (slot < 0) or one slot (the
// individual mode): its fields, grid cells, maxradius and pick-tree leaf.
template <class RS>
__device__ inline void block_update_one_or_all(const BoxRun &R, RS &sm, int slot, bool full) {
    if (slot < 0) {
        block_update_all(R, sm, full);
        return;
    }
    const DevBox &b = R.box;
    if (threadIdx.x == 0) {
        const double rm = thread_update_aggregate(R, slot, full);
        if (rm > b.sc->maxradius) b.sc->maxradius = rm;
        regrid(b, slot, agg_pos(b, slot));
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const unsigned long long total =
            tree_set(R, sm.tree, slot, tree_weight(*R.st, A(b, AGG_TIME_STEP, slot)));
        if (threadIdx.x == 0) {
            tree_total_to_state(*R.st, total);
            sm.rescale = total > kTreeHeadroom;
        }
    }
    __syncthreads();
    if (sm.rescale) {
        block_tree_build(R);
        tree_cache_load(R, sm.tree);
    }
}

// ---------------------------------------------------------------- oxidation
// With u_sg < 0 the spheres shrink (block_grow_*). Then, as in
// Aggregate::croissance_surface (aggregat.cpp:230-243), a sphere whose radius
// is at or below rp_min leaves its aggregate (remove_sphere,
// aggregat.cpp:629-655: the list keeps its order, relative positions are
// taken again from the first sphere left, the aggregate is updated); an
// aggregate left without spheres disappears (aggregat_list.cpp:549-579);
// and an aggregate whose spheres no longer form one network of contacts
// splits into one aggregate per connected part (Aggregate::split,
// aggregat.cpp:545-628; AggregatList::split, aggregat_list.cpp:409-446).
// Slots stay where they are: the part holding the first sphere keeps the
// slot, the others take free slots (a box that oxidises has a slot for every
// sphere), each part's spheres in list order, with the split aggregate's
// record (its proper time) before their own update. A removed sphere keeps
// its index with the slot -1.

// Relative positions from the first member (remove_sphere and split:
// position minus the first sphere's position); one thread.
__device__ inline void thread_rebase(const DevBox &b, const int *mem, int n) {
    const int s0 = mem[0];
    const double x0 = S(b, SPH_X, s0), y0 = S(b, SPH_Y, s0), z0 = S(b, SPH_Z, s0);
    for (int k = 0; k < n; ++k) {
        const int s = mem[k];
        S(b, SPH_RX, s) = S(b, SPH_X, s) - x0;
        S(b, SPH_RY, s) = S(b, SPH_Y, s) - y0;
        S(b, SPH_RZ, s) = S(b, SPH_Z, s) - z0;
    }
}

// One slot's spheres at or below rp_min leave its list, the others keep
// their order (one thread). Returns how many left.
__device__ inline int thread_remove_small(const BoxRun &R, int a) {
    const DevBox &b = R.box;
    const int off = b.agg_off[a], n = b.agg_n[a];
    int *pid = b.pool_id[b.sc->pool_sel] + off;
    float4 *pp = b.pool_pos[b.sc->pool_sel] + off;
    int w = 0;
    for (int k = 0; k < n; ++k) {
        const int s = pid[k];
        if (S(b, SPH_R, s) <= R.phys.rp_min) {
            b.sph_slot[s] = -1;
            continue;
        }
        if (w != k) {
            pid[w] = s;
            pp[w] = pp[k];
        }
        ++w;
    }
    b.agg_n[a] = w;
    if (w > 0 && w < n) {
        thread_rebase(b, pid, w);
        thread_update_aggregate(R, a, true);
    }
    return n - w;
}

// Removal in one slot (slot >= 0) or in every slot once a sphere reached
// rp_min; slots left empty leave the grids. Sets sm.disappear.
template <class RS>
__device__ inline void block_remove_small(const BoxRun &R, RS &sm, int slot) {
    const DevBox &b = R.box;
    DevScalars *sc = b.sc;
    const int tid = threadIdx.x, NT = blockDim.x;
    int *emptied = b.row_cnt;  // per slot: 1 when this step left it empty
    if (slot >= 0) {
        if (tid == 0) {
            const int gone = thread_remove_small(R, slot);
            R.st->removed_spheres += gone;
            if (gone > 0 && b.agg_n[slot] == 0) {
                cell_remove(b, cell_index(b, b.agg_cell[slot]), slot);
                if (b.fine_div > 0) fine_unlink(b, slot);
                sc->n_alive -= 1;
                sm.disappear = 1;
            }
        }
        __syncthreads();
        return;
    }
    if (b.counters[3] == 0) return;  // no sphere reached rp_min (set by the growth pass)
    __syncthreads();
    if (tid == 0) {
        b.counters[1] = 0;
        b.counters[2] = 0;
    }
    for (int a = tid; a < b.nslots; a += NT) emptied[a] = 0;
    __syncthreads();
    for (int a = tid; a < b.nslots; a += NT) {
        const int n = b.agg_n[a];
        if (n == 0) continue;
        const int *mem = b.pool_id[sc->pool_sel] + b.agg_off[a];
        bool any = false;
        for (int k = 0; k < n && !any; ++k) any = S(b, SPH_R, mem[k]) <= R.phys.rp_min;
        if (!any) continue;
        const int gone = thread_remove_small(R, a);
        atomicAdd(&b.counters[2], gone);
        if (gone == n) {
            emptied[a] = 1;
            atomicAdd(&b.counters[1], 1);
        }
    }
    __syncthreads();
    if (tid == 0) {
        const int n_empty = b.counters[1];
        R.st->removed_spheres += b.counters[2];
        // the grids' lists change one slot at a time, in slot order
        for (int a = 0, left = n_empty; a < b.nslots && left > 0; ++a) {
            if (!emptied[a]) continue;
            cell_remove(b, cell_index(b, b.agg_cell[a]), a);
            if (b.fine_div > 0) fine_unlink(b, a);
            --left;
        }
        sc->n_alive -= n_empty;
        if (n_empty > 0) sm.disappear = 1;
        b.counters[3] = 0;
    }
    __syncthreads();
}

// Disjoint-set forest over an aggregate's spheres: each root is the
// smallest index of its set (a larger root is hooked under a smaller one),
// so a parent never exceeds its child and every walk ends.
__device__ __forceinline__ int uf_find(int *parent, int x) {
    volatile int *p = parent;
    for (;;) {
        const int up = p[x];
        if (up == x) return x;
        const int gp = p[up];
        if (gp != up) p[x] = gp;  // path halving (still an ancestor)
        x = up;
    }
}
// Returns false when the retries ran out (they cannot: each failed hook
// means another root was hooked, at most n - 1 times).
__device__ __forceinline__ bool uf_unite(int *parent, int i, int j, int n) {
    for (int it = 0; it <= n + 1; ++it) {
        int ri = uf_find(parent, i), rj = uf_find(parent, j);
        if (ri == rj) return true;
        if (ri < rj) {
            const int t = ri;
            ri = rj;
            rj = t;
        }
        if (atomicCAS(&parent[ri], ri, rj) == ri) return true;
    }
    return false;
}

// Aggregate::split of one slot (all threads): its contact network's
// connected parts (sphere_distances.cpp:81-90, the 1e-28 tolerance), one
// aggregate each. Sets sm.split when it splits.
template <class RS>
__device__ inline void block_split_slot(const BoxRun &R, RS &sm, int a) {
    const DevBox &b = R.box;
    DevScalars *sc = b.sc;
    const int tid = threadIdx.x, NT = blockDim.x;
    const int n = b.agg_n[a];
    if (n < 2) return;
    const int *mem = b.pool_id[sc->pool_sel] + b.agg_off[a];
    if (tid == 0) {
        b.counters[0] = 0;
        b.counters[4] = 0;
    }
    // spheres in contact: |d| <= r_i + r_j + 1e-14 m, inside the scan's reach
    block_pair_scan(b, mem, n, sm.u.m, 2e-14f, [&](int i, int j) {
        const int si = mem[i], sj = mem[j];
        if (!spheres_in_contact(sph_pos(b, si), S(b, SPH_R, si), sph_pos(b, sj), S(b, SPH_R, sj), b.L)) return;
        const int p = atomicAdd(&b.counters[0], 1);
        if (p < b.pair_cap) {
            b.pair_tmp_i[p] = i;
            b.pair_tmp_j[p] = j;
        }
    });
    const int P = b.counters[0];
    if (P > b.pair_cap) {
        if (tid == 0) sc->status = ST_CAPACITY;
        __syncthreads();
        return;
    }
    int *parent = b.row_cnt;
    for (int i = tid; i < n; i += NT) parent[i] = i;
    __syncthreads();
    for (int p = tid; p < P; p += NT)
        if (!uf_unite(parent, b.pair_tmp_i[p], b.pair_tmp_j[p], n)) b.counters[4] = 1;
    __syncthreads();
    for (int i = tid; i < n; i += NT) parent[i] = uf_find(parent, i);
    __syncthreads();
    if (b.counters[4] != 0) {
        if (tid == 0) sc->status = ST_UNKNOWN;
        __syncthreads();
        return;
    }
    // parts in the order of their first sphere
    int *rank = reinterpret_cast<int *>(b.work);  // n + 1
    for (int i = tid; i < n; i += NT) rank[i] = parent[i] == i ? 1 : 0;
    __syncthreads();
    const int K = block_scan_global(rank, n, sm.u.m.warp_tmp);
    if (K < 2) return;
    int *cnt = rank + n + 1;   // K + 1: part sizes, then ends
    int *part = cnt + K + 1;   // n: part of each member
    int *ord = part + n;       // n: members grouped by part, list order kept
    float4 *ordf = reinterpret_cast<float4 *>(b.work + ((size_t(ord + n - rank) * sizeof(int) + 15) / 16) * 2);
    for (int c = tid; c <= K; c += NT) cnt[c] = 0;
    __syncthreads();
    for (int i = tid; i < n; i += NT) {
        const int c = rank[parent[i]];
        part[i] = c;
        atomicAdd(&cnt[c], 1);
    }
    __syncthreads();
    block_scan_global(cnt, K + 1, sm.u.m.warp_tmp);  // starts
    const float4 *pp0 = b.pool_pos[sc->pool_sel] + b.agg_off[a];
    if (tid == 0) {
        for (int i = 0; i < n; ++i) {
            const int q = cnt[part[i]]++;  // cnt[c] ends as the end of part c
            ord[q] = mem[i];
            ordf[q] = pp0[i];
        }
    }
    // free slots for parts 1..K-1, in slot order
    int *freef = b.cand_prefix;
    int *freelist = b.cand_slot;
    for (int x = tid; x < b.nslots; x += NT) freef[x] = b.agg_n[x] == 0 ? 1 : 0;
    __syncthreads();
    const int nfree = block_scan_global(freef, b.nslots, sm.u.m.warp_tmp);
    if (nfree < K - 1) {
        if (tid == 0) sc->status = ST_CAPACITY;
        __syncthreads();
        return;
    }
    for (int x = tid; x < b.nslots; x += NT)
        if (b.agg_n[x] == 0 && freef[x] < K - 1) freelist[freef[x]] = x;
    const int n0 = cnt[0];
    if (sc->pool_top + (n - n0) > b.pool_cap) block_compact_pool(b, sm.u.m.warp_tmp);
    __syncthreads();
    const int off0 = b.agg_off[a], base = sc->pool_top;
    int *pid = b.pool_id[sc->pool_sel];
    float4 *pp = b.pool_pos[sc->pool_sel];
    for (int q = tid; q < n; q += NT) {
        int lo = 0, hi = K - 1;  // the part of position q: the first end above q
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (cnt[mid] > q) hi = mid; else lo = mid + 1;
        }
        const int s = ord[q];
        if (lo == 0) {
            pid[off0 + q] = s;
            pp[off0 + q] = ordf[q];
        } else {
            pid[base + q - n0] = s;
            pp[base + q - n0] = ordf[q];
            b.sph_slot[s] = freelist[lo - 1];
        }
    }
    for (int t = tid; t < (K - 1) * AGG_NFIELDS; t += NT)
        A(b, t % AGG_NFIELDS, freelist[t / AGG_NFIELDS]) = A(b, t % AGG_NFIELDS, a);
    __syncthreads();
    if (tid == 0) {
        b.agg_n[a] = n0;
        for (int c = 1; c < K; ++c) {
            const int x = freelist[c - 1];
            b.agg_off[x] = base + cnt[c - 1] - n0;
            b.agg_n[x] = cnt[c] - cnt[c - 1];
        }
        sc->pool_top = base + (n - n0);
        sc->n_alive += K - 1;
    }
    __syncthreads();
    for (int c = tid; c < K; c += NT) {
        const int x = c == 0 ? a : freelist[c - 1];
        thread_rebase(b, pid + b.agg_off[x], b.agg_n[x]);
        thread_update_aggregate(R, x, true);
    }
    __syncthreads();
    if (tid == 0) {
        regrid(b, a, agg_pos(b, a));
        for (int c = 1; c < K; ++c) {
            const int x = freelist[c - 1];
            const Vec3 p = agg_pos(b, x);
            const int key = cell_of(b, p);
            cell_insert(b, cell_index(b, key), x);
            b.agg_cell[x] = key;
            if (b.fine_div > 0) fine_link(b, x, fine_cell_of(b, p));
        }
        R.st->splits += 1;
        sm.split = 1;
    }
    __syncthreads();
}

// The oxidation of a step (all threads), after the spheres shrank: removals
// and disappearances, then splits -- of the moved aggregate (slot >= 0, the
// individual mode, calcul.cpp:159-163) or of every aggregate (calcul.cpp:
// 165-169). Sets sm.split and sm.disappear. Out of line: the loop's steps
// without oxidation keep their code compact.
template <class RS>
__device__ __noinline__ void block_oxidize(const BoxRun &R, RS &sm, int slot) {
    const DevBox &b = R.box;
    const int tid = threadIdx.x, NT = blockDim.x;
    if (tid == 0) {
        sm.split = 0;
        sm.disappear = 0;
    }
    __syncthreads();
    block_remove_small(R, sm, slot);
    if (slot >= 0) {
        if (!sm.disappear) block_split_slot(R, sm, slot);
        return;
    }
    // the aggregates of two or more spheres, in slot order (the parts made
    // by a split are connected and are not visited)
    int *flag = b.cand_order;
    long long *list = b.cand_key;
    for (int a = tid; a < b.nslots; a += NT) flag[a] = b.agg_n[a] >= 2 ? 1 : 0;
    __syncthreads();
    const int m = block_scan_global(flag, b.nslots, sm.u.m.warp_tmp);
    for (int a = tid; a < b.nslots; a += NT)
        if (b.agg_n[a] >= 2) list[flag[a]] = a;
    __syncthreads();
    for (int k = 0; k < m; ++k) {
        block_split_slot(R, sm, int(list[k]));
        if (b.sc->status != ST_OK) break;
    }
    __syncthreads();
}

// The query's answer into the step's shared state and the box's counters
// (thread 0).
template <class RS>
__device__ inline void apply_query(RunState &st, RS &sm, const QueryOut &q) {
    if (q.status != ST_OK) {
        st.status = q.status;
        sm.stop = 1;
    }
    sm.contact = q.distance <= sm.full;
    sm.move = sm.contact ? q.distance : sm.full;
    sm.ms = q.moving_sphere;
    sm.os = q.other_sphere;
    sm.oslot = q.other_slot;
    st.c_queries += 1;
    st.c_mov += q.n_mov;
    st.c_scanned += q.n_scanned;
    st.c_cells += q.n_cells;
    st.c_candidates += q.n_candidates;
    st.c_cand_spheres += q.n_cand_spheres;
    st.c_refined += q.n_pairs_refined;
    st.cyc_qscan += q.cyc_scan;
    st.cyc_qpairs += q.cyc_pairs;
}

// The rest of a step once its pick (sm.slot, sm.dir, sm.dt, sm.full,
// sm.dt_indiv) and its query's answer (sm.contact, sm.move, sm.ms, sm.os,
// sm.oslot) are known: translation, time, surface reactions, merge, pick
// tree, counters and the stop criteria (all threads). Returns false when
// the box stopped on an error.
template <class RS>
__device__ inline bool step_commit(const BoxRun &R, RS &sm, long long &t_phase) {
    const int tid = threadIdx.x;
    const DevBox &b = R.box;
    RunState &st = *R.st;
    const int slot = sm.slot;
    const Vec3 dir{sm.dir[0], sm.dir[1], sm.dir[2]};
    const int ms = sm.ms, os = sm.os, oslot = sm.oslot;
    block_translate(b, slot, Vec3{dir.x * sm.move, dir.y * sm.move, dir.z * sm.move}, sm.refpos);
    if (tid == 0) {
        const long long t = clock64();
        st.cyc_move += t - t_phase;
        t_phase = t;
        // without contact the move is the full lpm and the ratio is 1
        double dt = sm.contact ? sm.dt * (sm.move / sm.full + 0.0) : sm.dt;
        A(b, AGG_TIME, slot) += dt;
        st.time = st.time + dt;
        sm.merged = 0;
        sm.step_dt = dt;
        sm.step_dt_indiv = sm.contact ? sm.dt_indiv * (sm.move / sm.full + 0.0) : sm.dt_indiv;
    }
    __syncthreads();
    // surface reactions before the merge (calcul.cpp:157-172)
    if (R.phys.growth) {
        if (R.phys.individual)
            block_grow_slot(R, slot, sm.step_dt_indiv);
        else
            block_grow_spheres(R, sm.step_dt);
    }
    __syncthreads();
    bool try_merge = sm.contact;
    int mslot = slot, cslot = oslot;
    if (R.phys.oxidation) {
        block_oxidize(R, sm, R.phys.individual ? slot : -1);
        if (tid == 0 && b.sc->status != ST_OK) {
            st.status = b.sc->status;
            sm.stop = 1;
        }
        __syncthreads();
        if (sm.stop) return false;
        // AggregatList::merge takes the two spheres where they are now, and
        // merges nothing when one is gone or they no longer touch
        // (aggregat_list.cpp:367-378); the individual mode merges nothing
        // after a split or a disappearance (calcul.cpp:173-178)
        if (try_merge) {
            mslot = b.sph_slot[ms];
            cslot = b.sph_slot[os];
            if (mslot < 0 || cslot < 0 || mslot == cslot) try_merge = false;
            if (R.phys.individual && (sm.split || sm.disappear)) try_merge = false;
        }
    }
    if (try_merge) {
        block_merge(b, ms, os, mslot, cslot, sm.u.m, &sm.mout);
        if (tid == 0) {
            if (sm.mout.status != ST_OK) {
                st.status = sm.mout.status;
                sm.stop = 1;
            } else if (sm.mout.merged) {
                const int keep = sm.mout.keep, removed = sm.mout.removed;
                double f, dm, ts, lpm, dgdp;
                device_physics(R.phys, sm.mout.fields[AGG_VOLUME], sm.mout.vol_pp, sm.mout.fields[AGG_DP],
                               sm.mout.fields[AGG_RG], &f, &dm, &ts, &lpm, &dgdp);
                A(b, AGG_F_AGG, keep) = f;
                A(b, AGG_D_M, keep) = dm;
                A(b, AGG_TIME_STEP, keep) = ts;
                A(b, AGG_LPM, keep) = lpm;
                A(b, AGG_DG_OVER_DP, keep) = dgdp;
                A(b, AGG_TIME, keep) = A(b, AGG_TIME, keep) + A(b, AGG_TIME, removed) - st.time;
                sm.merged = 1;
                sm.keep = keep;
                sm.removed = removed;
                st.c_merged_spheres += sm.mout.n;
                st.c_merge_pairs += sm.mout.n_pairs;
            }
        }
        __syncthreads();
        if (sm.stop) return false;
        if (sm.merged && tid < 32 && !R.phys.growth) {
            tree_set(R, sm.tree, sm.removed, 0ULL);
            const unsigned long long wk = tree_weight(st, A(b, AGG_TIME_STEP, sm.keep));
            const unsigned long long total = tree_set(R, sm.tree, sm.keep, wk);
            if (tid == 0) {
                tree_total_to_state(st, total);
                sm.rescale = total > kTreeHeadroom;  // a new scale keeps the total clear of 2^64
                if (sm.live.on) live_merge(sm.live, sm.keep, sm.removed, wk);
            }
        }
        __syncthreads();
        if (sm.merged && !R.phys.growth && sm.rescale) {
            block_tree_build(R);
            tree_cache_load(R, sm.tree);
            live_load(R, sm.live, sm.u.q.warp_tmp);  // every weight changed
        } else if (sm.merged && !R.phys.growth && !sm.live.on && sm.live.allow &&
                   b.sc->n_alive <= sm.live.max) {
            live_load(R, sm.live, sm.u.q.warp_tmp);  // few enough left now
        }
    }
    if (R.phys.growth) {
        // every aggregate after growth (and merge): update() on every
        // full_aggregate_update_frequency-th step without event, else
        // update_partial() (calcul.cpp:180-206); in the individual mode only
        // the moved aggregate, unless there was a merge
        __syncthreads();
        const long long every = R.phys.full_update_every > 0 ? R.phys.full_update_every : 1;
        const bool full = st.n_iter_without_event % every == 0;
        const bool event = sm.merged || (R.phys.oxidation && (sm.split || sm.disappear));
        if (!R.phys.individual || event)
            block_update_one_or_all(R, sm, -1, full);
        else
            block_update_one_or_all(R, sm, slot, full);
    }
    if (tid == 0) {
        st.cyc_merge += clock64() - t_phase;
        st.steps += 1;
        if (sm.merged || (R.phys.oxidation && (sm.split || sm.disappear))) {
            st.events += 1;
            st.n_iter_without_event = 0;
        } else {
            st.n_iter_without_event += 1;
        }
        if (run_finished(R, st, b.sc->n_alive)) st.finished = 1;
    }
    __syncthreads();
    return true;
}

// One MC step of one box by the whole block. Returns false when the box is
// finished or in error (then nothing was done).
template <class RS>
__device__ inline bool block_mc_step(const BoxRun &R, RS &sm) {
    const int tid = threadIdx.x;
    const DevBox &b = R.box;
    RunState &st = *R.st;
    long long t_phase = 0;
    if (tid == 0) {
        t_phase = clock64();
        sm.stop = st.finished || st.status != ST_OK;
        if (!sm.stop && run_finished(R, st, b.sc->n_alive)) {
            st.finished = 1;
            sm.stop = 1;
        }
        // a time-capped launch: checked before every step, so that a box of
        // expensive steps does not hold the launch (and the other boxes,
        // which wait for it) past the cap
        if (!sm.stop && sm.deadline != 0ULL && global_ns() >= sm.deadline) sm.stop = 1;
        if (!sm.stop) sm.t_pick = pick_target(st.rng, st.tree_total);
    }
    __syncthreads();
    if (sm.stop) return false;
    if (tid < 32) {
        int slot = sm.live.on ? live_sample(sm.live, sm.t_pick) : tree_sample(R, sm.tree, sm.t_pick);
        if (tid == 0) {
            if (slot < 0 || slot >= b.nslots || b.agg_n[slot] == 0) {
                st.status = ST_UNKNOWN;  // the tree lost a live slot: stop this box
                sm.stop = 1;
                slot = 0;
            }
            sm.slot = slot;
            sm.dt = st.inv_weight;
            sm.full = A(b, AGG_LPM, slot);
            sm.dt_indiv = A(b, AGG_TIME_STEP, slot);
            draw_direction(st.rng, sm.dir);
        }
    }
    __syncthreads();
    if (sm.stop) return false;
    if (tid == 0) {
        const long long t = clock64();
        st.cyc_pick += t - t_phase;
        t_phase = t;
    }
    if (R.lim.with_collisions) {
        block_query(b, sm.slot, Vec3{sm.dir[0], sm.dir[1], sm.dir[2]}, sm.full, sm.u.q, &sm.live);
        if (tid == 0) apply_query(st, sm, sm.u.q.out);
    } else if (tid == 0) {
        sm.contact = 0;
        sm.move = sm.full;
    }
    __syncthreads();
    if (sm.stop) return false;
    if (tid == 0) {
        const long long t = clock64();
        st.cyc_query += t - t_phase;
        t_phase = t;
    }
    return step_commit(R, sm, t_phase);
}

}  // namespace mcacg
