// Device-resident MCAC box and the block-level algorithms of the hot path.
//
// One thread block works on one box at a time. The same __device__ routines
// serve the single-box kernels behind the C-ABI and the persistent batched
// kernel (many boxes, one block each).
//
// Layout in HBM (per box):
//   spheres     FP64 [9][ns] field-major (reference SoA, constants.hpp:34-45)
//               + int owning slot
//   aggregates  FP64 [21][nslots] field-major by stable slot; slot order is
//               label order, so label = number of live slots before it
//   members     per aggregate a contiguous segment of a pool: sphere id (int)
//               and an FP32 (x, y, z, r) copy used by the screening passes;
//               merges append keep++removed at the pool top, a compaction
//               pass reclaims space
//   Verlet grid n_div^3 cells of unordered slot lists (+ each slot's place in
//               its list, so moves are O(1)); the reference's order inside a
//               cell (std::set<size_t> of labels, verlet.hpp:29) is restored
//               by the scan key (cell rank in the scan, slot)
//   fine grid   fine_div^3 cells (fine_div > n_div) of doubly linked slot
//               lists, used only to find the neighbours of a query faster;
//               which neighbours count, and their order, stay the Verlet
//               grid's
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <math_constants.h>

#include "common.hpp"

namespace mcacg {

constexpr int kQueryThreads = 512;
constexpr int kFineMaxCells = 4096;    // fine cells a query may visit before the Verlet cells are used
constexpr int kFineMaxDiv = 128;       // fine cells per axis at most
constexpr int kCullCands = 16;         // candidates whose extents cull the moving spheres

// Mutable per-box scalars, in device memory.
struct DevScalars {
    double maxradius;     // AggregatList::maxradius (monotone)
    double time;          // physical time (device-driven runs)
    int pool_top;         // first free pool entry
    int pool_sel;         // which pool buffer is live
    int n_alive;          // aggregates alive
    int status;           // sticky error (Status)
    int cell_overflow;    // a Verlet cell ran out of room
    int survivors_overflow;
    int pad[2];
};

struct DevBox {
    double L;        // box_length
    double step;     // double(n_div) / box_length
    double margin;   // FP32 screening margin (absolute, metres)
    double inv_L;    // 1 / box_length
    // FP32 copies for the screens and the fine grid
    float Lf, inv_Lf, margin_f, fine_step_f;
    float inv_fine_cells, inv_cells;  // 1 / fine_div^3, 1 / n_cells
    int n_div;
    int n_cells;
    int ns;          // spheres
    int nslots;      // aggregate slots (initial aggregate count)
    int cell_cap;    // room per Verlet cell
    int pool_cap;    // entries per pool buffer
    int surv_cap;    // survivors in global scratch
    int pair_cap;    // intra-aggregate contact pairs in global scratch
    int grid_pairs_min;  // merged aggregates from this size find their pairs on a cell grid
    double *sph;     // [9][ns]
    int *sph_slot;   // owning slot
    // each sphere's entry of its aggregate's per-sphere volumes at the last
    // compute_volume_surface (Aggregate::volumes, aggregat.cpp:321-430): the
    // sphere's volume, less its spherical caps for "caps"; update_partial
    // weighs the centre of mass and Rg with it (aggregat.cpp:431-483)
    double *sph_volw;
    int volsurf;     // VolSurfMethods of the box (VS_NONE, VS_CAPS, VS_ALPHAS)
    double *agg;     // [21][nslots]
    int *agg_n;      // members (0: dead slot)
    int *agg_off;    // segment offset in the live pool
    int *agg_cell;   // Verlet cell (cell_key)
    float4 *agg_f4;  // FP32 (x, y, z, rmax) of each slot, for the neighbour screen
    int *pool_id[2];
    float4 *pool_pos[2];
    int *cell_n;     // [n_cells]
    int *cell_items; // [n_cells][cell_cap], unordered
    int *cell_pos;   // [nslots] index of each live slot in its cell's list
    int fine_div;    // fine grid cells per axis (0: no fine grid)
    double fine_step;  // fine_div / box_length
    int *fine_head;  // [fine_div^3] first slot of each fine cell, -1 if empty
    int *fine_next, *fine_prev;  // [nslots] list links, -1 at the ends
    int *fine_cell;  // [nslots] fine cell of each live slot, -1 if none
    DevScalars *sc;
    // global scratch (one box handled by one block at a time)
    int4 *surv;          // survivors: candidate, i, j, unused
    double *surv_res;
    int *pair_i, *pair_j;   // intra-aggregate contact pairs
    double *pair_d;
    int *pair_tmp_i, *pair_tmp_j;
    double *pair_tmp_d;
    int *row_cnt;        // [ns + 1]
    double *work;        // [8][ns] per-sphere terms of the merge sums
    int *counters;       // [8]
    // contact-query candidates (at most one per aggregate slot)
    double *cand_db;
    long long *cand_key;  // Verlet scan position: cell rank in the scan x nslots + slot
    int *cand_slot, *cand_order, *cand_prefix;
    unsigned long long *best_res, *best_ij;
};

// Byte offsets of a packed state (na live aggregates) in the merge's pair
// scratch (32 B per pair, 8 ns + 1024 pairs: 200 B per sphere at most are used):
// aggregates [21][na] f64, sphere counts [na] i64, labels [ns] i64, members
// [ns] i64, then the ranks and member offsets of the slots [nslots] i32 each.
struct PackLayout {
    size_t agg, count, label, members, rank, moff, total;
};
__host__ __device__ inline PackLayout pack_layout(int na, int ns, int nslots) {
    PackLayout l;
    l.agg = 0;
    l.count = 168 * size_t(na);
    l.label = 176 * size_t(na);
    l.members = l.label + 8 * size_t(ns);
    l.rank = l.members + 8 * size_t(ns);
    l.moff = l.rank + 4 * size_t(nslots);
    l.total = l.moff + 4 * size_t(nslots);
    return l;
}

__device__ __forceinline__ double &A(const DevBox &b, int field, int slot) {
    return b.agg[size_t(field) * size_t(b.nslots) + size_t(slot)];
}
__device__ __forceinline__ double &S(const DevBox &b, int field, int s) {
    return b.sph[size_t(field) * size_t(b.ns) + size_t(s)];
}

// Result of a contact query.
struct QueryOut {
    double distance;
    int moving_sphere;  // storage index or -1
    int other_sphere;
    int other_slot;
    int status;
    int n_candidates;     // aggregates passing the bounding-sphere filter
    int n_pairs_refined;  // sphere pairs evaluated in FP64
    int n_scanned;        // aggregates read from the Verlet cells
    int n_cells;          // Verlet cells scanned
    int n_cand_spheres;   // spheres of the candidates
    int n_mov;            // spheres of the moving aggregate
    long long cyc_scan;   // SM cycles: neighbourhood and bounding-sphere filter
    long long cyc_pairs;  // SM cycles: candidate order, pair search, walk
};

// Merge result returned to the host (geometry; physics done by the caller).
struct MergeOut {
    int merged;       // 0: the spheres no longer touch
    int status;
    int keep;         // slot kept
    int removed;      // slot removed
    int n;            // spheres in the merged aggregate
    int n_pairs;      // contact pairs found
    double fields[21];
    double vol_pp;
    double maxradius;
};

// ---------------------------------------------------------------- helpers
__device__ __forceinline__ Vec3 agg_pos(const DevBox &b, int slot) {
    return Vec3{A(b, AGG_X, slot), A(b, AGG_Y, slot), A(b, AGG_Z, slot)};
}
__device__ __forceinline__ Vec3 sph_pos(const DevBox &b, int s) {
    return Vec3{S(b, SPH_X, s), S(b, SPH_Y, s), S(b, SPH_Z, s)};
}
// A Verlet cell is kept as its coordinates packed in one int (10 bits each,
// n_div <= 1024), so the neighbourhood test needs no division; the cell
// lists are indexed by the linear cell.
__device__ __forceinline__ int cell_key(int ix, int iy, int iz) { return ix | (iy << 10) | (iz << 20); }
__device__ __forceinline__ int cell_index(const DevBox &b, int key) {
    return ((key & 1023) * b.n_div + ((key >> 10) & 1023)) * b.n_div + (key >> 20);
}
__device__ __forceinline__ int cell_of(const DevBox &b, Vec3 p) {
    int ix = verlet_coord(p.x, b.step), iy = verlet_coord(p.y, b.step), iz = verlet_coord(p.z, b.step);
    ix = min(max(ix, 0), b.n_div - 1);
    iy = min(max(iy, 0), b.n_div - 1);
    iz = min(max(iz, 0), b.n_div - 1);
    return cell_key(ix, iy, iz);
}
// i mod n for i in [-2n, 3n)
__device__ __forceinline__ int wrap_cell(int i, int n) {
    i += i < 0 ? n : 0;
    i += i < 0 ? n : 0;
    i -= i >= n ? n : 0;
    i -= i >= n ? n : 0;
    return i;
}

// Order-preserving map of a double to an unsigned 64-bit key.
__device__ __forceinline__ unsigned long long dkey(double v) {
    unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(v));
    return (u & 0x8000000000000000ULL) ? ~u : (u | 0x8000000000000000ULL);
}
__device__ __forceinline__ double dkey_inv(unsigned long long k) {
    unsigned long long u = (k & 0x8000000000000000ULL) ? (k & 0x7fffffffffffffffULL) : ~k;
    return __longlong_as_double(static_cast<long long>(u));
}

// Conservative FP32 capsule test: can a sphere at p2 (radius folded into
// 'reach') come within 'reach' of the segment p1 -> p1 + dist*u under the
// periodic box? False means the FP64 swept test of sweep_contact_distance
// returns +inf for this pair. When the swept zone (|dist*u_l| + 2*reach)
// approaches the box size several periodic images can matter and the test
// always passes; otherwise only the image nearest to the segment centre can
// be within reach and it is the one tested. 'reach' already holds the margin.
struct Sweep32 {
    float px, py, pz;     // segment start
    float ux, uy, uz;     // unit direction
    float dist;           // length
    float cx, cy, cz;     // segment centre offset (dist*u/2)
    float L, invL;
    float zmax;           // max_l |dist * u_l|
    float margin;
};
__device__ __forceinline__ bool capsule_hit(const Sweep32 &w, float qx, float qy, float qz, float reach) {
    if (w.zmax + 2.f * reach + 8.f * w.margin >= w.L) return true;
    float ex = qx - w.px, ey = qy - w.py, ez = qz - w.pz;
    ex -= w.L * rintf((ex - w.cx) * w.invL);
    ey -= w.L * rintf((ey - w.cy) * w.invL);
    ez -= w.L * rintf((ez - w.cz) * w.invL);
    float t = __fmaf_rn(ex, w.ux, __fmaf_rn(ey, w.uy, ez * w.uz));
    t = fminf(fmaxf(t, 0.f), w.dist);
    float dx = __fmaf_rn(-t, w.ux, ex), dy = __fmaf_rn(-t, w.uy, ey), dz = __fmaf_rn(-t, w.uz, ez);
    float d2 = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, dz * dz));
    return d2 <= reach * reach;
}

// ------------------------------------------------------------ block scans
__device__ __forceinline__ int block_exclusive_scan(int v, int *warp_tmp, int &total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int NT = blockDim.x;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tmp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int w = (lane < NT / 32) ? warp_tmp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < NT / 32) warp_tmp[lane] = w;
    }
    __syncthreads();
    int base = (wid > 0) ? warp_tmp[wid - 1] : 0;
    total = warp_tmp[NT / 32 - 1];
    __syncthreads();
    return base + x - v;
}

// ------------------------------------------------------ shared memory plans
// CellChunk: Verlet cells scanned per chunk (also the cross-motion grid's
// room); MoveTile: moving spheres staged per pass; SurvSmem: refined pairs
// kept in shared memory (the rest in HBM). The small plan lets 16 boxes
// share an SM.
template <int CellChunk, int MoveTile, int SurvSmem, int CandCache>
struct QuerySmemT {
    static constexpr int kCellChunk = CellChunk;
    static constexpr int kMoveTile = MoveTile;
    static constexpr int kSurv = SurvSmem;
    static constexpr int kCandCache = CandCache;
    static_assert(CandCache <= 32, "the cache is filled by the lanes of one warp");
    static constexpr int kGridMax = CellChunk >= 1024 ? 32 : (CellChunk >= 256 ? 16 : 11);  // grid cells per axis
    static_assert(kGridMax * kGridMax <= CellChunk, "grid must fit the cell arrays");
    int cell_prefix[kCellChunk + 1];
    int cell_lin[kCellChunk];
    // candidate arrays live in the machine's HBM scratch (one entry per slot at most)
    double *cand_db;
    long long *cand_key;
    int *cand_slot;
    int *cand_order;   // sorted position -> candidate
    int *cand_prefix;
    unsigned long long *best_res;
    unsigned long long *best_ij;
    float4 mov[kMoveTile];
    short mov_sel[kMoveTile];  // moving spheres of the tile that can reach a candidate
    // up to kCandCache candidates (the usual case) their sorted sphere
    // prefix, slots and pool offsets are kept here too, so the pair search
    // reads them from shared memory instead of chasing cand_order ->
    // cand_slot -> agg_off in device memory for every candidate sphere
    int c_pre[CandCache + 1];
    int c_slot[CandCache];
    int c_off[CandCache];
    float4 cand_c[kCullCands];  // candidate centre (FP32)
    float cand_ext[kCullCands]; // candidate extent from that centre (max |q - c| + r_q)
    int n_sel;
    // 2D grid of a moving tile across the direction of motion
    float grid_h, grid_half, grid_rmax, grid_span;
    int grid_g, grid_on;
    float basis[6];  // two unit vectors orthogonal to the direction
    int4 surv[kSurv];
    double surv_res[kSurv];
    int warp_tmp[32];
    float warp_f[32];
    float warp_f2[32];
    int n_cand;
    int n_screen;  // neighbours passing the FP32 screen, before the FP64 filter
    int n_surv;
    int found_source;
    int flat_base;
    int n_refined;
    int use_fine;     // neighbours found through the fine grid
    long long t_q0;   // clock at the start of the query
    int fine_lo[3], fine_n[3];
    float mov_reach;
    CellRange range;
    QueryOut out;
};
using QuerySmem = QuerySmemT<1024, 512, 256, 32>;
// the one-warp plan: 16 boxes an SM leave 14.25 KB of shared memory a box
using QuerySmemSmall = QuerySmemT<256, 256, 128, 4>;

// The live slots of a box with few aggregates left, in ascending slot order,
// with their pick weights (kept in shared memory by the device loop). With
// it a query reads its neighbours from the list instead of walking the
// Verlet cells around it (late in a run most of those cells are empty), and
// the pick scans the list instead of descending the tree from HBM.
constexpr int kLiveMax = 128;
template <int N>
struct LiveListT {
    static constexpr int kCap = N;
    int on;      // the list is in use
    int n;       // live slots listed
    int allow;   // the kernel may use a list (0: never)
    int max;     // use a list from this many live aggregates down (<= kCap)
    int slot[N];
    unsigned long long w[N];
};
using LiveList = LiveListT<kLiveMax>;
// one warp per box keeps no list: its shared memory holds 16 boxes an SM
using LiveListNone = LiveListT<1>;

// -------------------------------------------------------------- the query
// AggregatList::distance_to_next_contact (aggregats/aggregat_list.cpp:447-532):
//  1. neighbourhood = aggregates in the Verlet cells covering the swept
//     bounding sphere (verlet.cpp:52-98), in the reference's scan order;
//  2. bounding-sphere filter d_b < distance, ordered by (d_b, scan order)
//     like the reference's std::multimap;
//  3. every moving-sphere x candidate-sphere pair that the FP32 capsule
//     screen keeps is refined with the exact FP64 swept test; each candidate
//     keeps its first minimum in (moving index, other index) order;
//  4. the candidates are walked in filter order with the reference's two
//     early exits.
// Must be called by all threads of the block.
template <class SM, class LL = LiveList>
__device__ inline void block_query(const DevBox &b, int src, Vec3 dir, double dist, SM &sm,
                                   const LL *live = nullptr) {
    constexpr int kCellChunk = SM::kCellChunk;
    constexpr int kMoveTile = SM::kMoveTile;
    constexpr int kMaxSurvivorsSmem = SM::kSurv;
    const int tid = threadIdx.x;
    const int NT = blockDim.x;
    const DevScalars *sc = b.sc;
    const int *pool_id = b.pool_id[sc->pool_sel];
    const float4 *pool_pos = b.pool_pos[sc->pool_sel];

    const Vec3 sp = agg_pos(b, src);
    const double rmax_src = A(b, AGG_RMAX, src);
    const float4 src_f = b.agg_f4[src];  // FP32 centre and r_max of the source
    // Lanes 0-2 of warp 0 take one axis each (FP64 work costs the same for
    // one lane as for the warp): the reference's Verlet cell range, and the
    // fine range. The fine grid finds the same neighbours when every
    // aggregate that can pass the bounding-sphere filter lies in the fine
    // cells visited: its centre is within rmax_src + rmax <= mindist of the
    // path. The fine range is computed in FP32 and widened by 2e-3 of a fine
    // cell: its rounding (and that of the aggregates' FP32 fine cells) stays
    // below 1e-4 of a cell while it spans less than the box, and a range of
    // the box or more is the whole axis.
    if (tid < 32) {
        int lo = 0, hi = 0, flo = 0, fn = 0;
        if (tid < 3) {
            const double mindist = rmax_src + sc->maxradius;
            const double sl = tid == 0 ? sp.x : (tid == 1 ? sp.y : sp.z);
            const double vl = dist * (tid == 0 ? dir.x : (tid == 1 ? dir.y : dir.z));
            neighborhood_axis(sl, vl, mindist, b.n_div, b.L, b.inv_L, &lo, &hi);
            sm.range.lo[tid] = lo;
            sm.range.hi[tid] = hi;
            if (b.fine_div > 0) {
                const float pf = tid == 0 ? src_f.x : (tid == 1 ? src_f.y : src_f.z);
                const float mf = float(mindist), vf = float(vl);
                const float flof = floorf((pf - mf + fminf(vf, 0.f)) * b.fine_step_f - 2e-3f);
                const float fhif = floorf((pf + mf + fmaxf(vf, 0.f)) * b.fine_step_f + 2e-3f);
                const bool part = (fhif - flof + 1.f < float(b.fine_div)) && flof > -1e6f && fhif < 1e6f;
                flo = part ? int(flof) : 0;
                fn = part ? int(fhif - flof + 1.f) : b.fine_div;
                sm.fine_lo[tid] = flo;
                sm.fine_n[tid] = fn;
            }
        }
        const int nc = hi - lo + 1;
        const int nc1 = __shfl_sync(0xffffffffu, nc, 1), nc2 = __shfl_sync(0xffffffffu, nc, 2);
        const int fn1 = __shfl_sync(0xffffffffu, fn, 1), fn2 = __shfl_sync(0xffffffffu, fn, 2);
        if (tid == 0) {
            sm.use_fine = 0;
            if (b.fine_div > 0) {
                // visit the grid that reads fewer cells and list entries
                const int n_fine = fn * fn1 * fn2;
                const float alive = float(sc->n_alive);
                const float cost_fine = float(n_fine) * (1.f + alive * b.inv_fine_cells);
                const float cost_coarse = float(nc) * float(nc1) * float(nc2) * (1.f + alive * b.inv_cells);
                sm.use_fine = (n_fine <= kFineMaxCells) && (cost_fine < cost_coarse);
            }
        }
    }
    if (tid == 0) {
        sm.n_cand = 0;
        sm.n_screen = 0;
        sm.n_surv = 0;
        sm.found_source = 0;
        sm.flat_base = 0;
        sm.n_refined = 0;
        sm.out.distance = CUDART_INF;
        sm.out.moving_sphere = -1;
        sm.out.other_sphere = -1;
        sm.out.other_slot = -1;
        sm.out.status = ST_OK;
        sm.out.n_candidates = 0;
        sm.out.n_pairs_refined = 0;
        sm.out.n_scanned = 0;
        sm.out.n_cells = 0;
        sm.out.n_cand_spheres = 0;
        sm.out.n_mov = b.agg_n[src];
        sm.out.cyc_scan = 0;
        sm.out.cyc_pairs = 0;
        sm.t_q0 = clock64();
        sm.cand_db = b.cand_db;
        sm.cand_key = b.cand_key;
        sm.cand_slot = b.cand_slot;
        sm.cand_order = b.cand_order;
        sm.cand_prefix = b.cand_prefix;
        sm.best_res = b.best_res;
        sm.best_ij = b.best_ij;
    }
    __syncthreads();

    // FP32 sweep of the bounding sphere of the source.
    Sweep32 w;
    w.px = src_f.x;
    w.py = src_f.y;
    w.pz = src_f.z;
    w.ux = float(dir.x);
    w.uy = float(dir.y);
    w.uz = float(dir.z);
    w.dist = float(dist);
    w.cx = 0.5f * w.dist * w.ux;
    w.cy = 0.5f * w.dist * w.uy;
    w.cz = 0.5f * w.dist * w.uz;
    w.L = b.Lf;
    w.invL = b.inv_Lf;
    // b.margin and 1e-6 dist, each rounded to FP32 (the screen keeps them
    // conservative: both bound errors far smaller than themselves)
    const float margin = b.margin_f + 1e-6f * w.dist;
    w.zmax = fmaxf(fabsf(w.dist * w.ux), fmaxf(fabsf(w.dist * w.uy), fabsf(w.dist * w.uz)));
    w.margin = margin;

    // ---- 1+2: neighbourhood and bounding-sphere filter
    const CellRange rg = sm.range;
    const int nx = rg.hi[0] - rg.lo[0] + 1, ny = rg.hi[1] - rg.lo[1] + 1, nz = rg.hi[2] - rg.lo[2] + 1;
    const int n_scan = nx * ny * nz;
    // bounding-sphere filter of one neighbour, first part: the FP32 screen;
    // 'key' is its position in the reference's neighbour list order (Verlet
    // cell rank in the scan, then slot). Those passing wait (in the
    // candidates' prefix and key scratch, free until the pair search) for
    // the FP64 test after the scan: one copy of that code, run densely.
    long long *screen_key = reinterpret_cast<long long *>(sm.best_ij);
    auto consider = [&](int slot, long long key, float4 of) {
        if (!capsule_hit(w, of.x, of.y, of.z, src_f.w + of.w + margin)) return;
        const int k = atomicAdd(&sm.n_screen, 1);  // < nslots: one entry per aggregate
        sm.cand_prefix[k] = slot;
        screen_key[k] = key;
    };
    int n_cells_visited = n_scan;
    if (live != nullptr && live->on) {
        // few aggregates left: the live list in slot order, each aggregate
        // kept when its Verlet cell is in the reference's neighbourhood, with
        // the scan key of the fine walk below (the same set, the same keys)
        const int nd = b.n_div;
        const int rlo0 = rg.lo[0], rlo1 = rg.lo[1], rlo2 = rg.lo[2];
        for (int k = tid; k < live->n; k += NT) {
            const int slot = live->slot[k];
            const int key = b.agg_cell[slot];
            const int oa = wrap_cell((key & 1023) - rlo0, nd);
            const int ob = wrap_cell(((key >> 10) & 1023) - rlo1, nd);
            const int oc = wrap_cell((key >> 20) - rlo2, nd);
            if (!(oa < nx && ob < ny && oc < nz)) continue;
            if (slot == src) {
                sm.found_source = 1;
            } else {
                consider(slot, (long long)((oa * ny + ob) * nz + oc) * b.nslots + slot, b.agg_f4[slot]);
            }
        }
        if (tid == 0) sm.flat_base = live->n;
        n_cells_visited = 0;
        __syncthreads();
    } else if (sm.use_fine) {
        // walk the fine cells; keep the aggregates whose Verlet cell is in
        // the reference's neighbourhood
        const int fny = sm.fine_n[1], fnz = sm.fine_n[2];
        const int n_f = sm.fine_n[0] * fny * fnz;
        const int nf = b.fine_div, nd = b.n_div;
        // g -> (a, bb, c) by FP32 reciprocals: g < 2^21 and divisors <= 128^2
        // keep (g + 1/2) / d at least 1/(2 d) from an integer, far above the
        // FP32 error, so the floors are exact
        const int fyz = fny * fnz;
        const float inv_yz = 1.f / float(fyz), inv_z = 1.f / float(fnz);
        const int flo0 = sm.fine_lo[0], flo1 = sm.fine_lo[1], flo2 = sm.fine_lo[2];
        const int rlo0 = rg.lo[0], rlo1 = rg.lo[1], rlo2 = rg.lo[2];
        n_cells_visited = n_f;
        int visited = 0;
        constexpr int kHeads = 4;  // list heads fetched together per thread
        for (int g0 = 0; g0 < n_f; g0 += kHeads * NT) {
            int heads[kHeads];
#pragma unroll
            for (int u = 0; u < kHeads; ++u) {
                const int g = g0 + u * NT + tid;
                heads[u] = -1;
                if (g < n_f) {
                    const int a = int((float(g) + 0.5f) * inv_yz), r = g - a * fyz;
                    const int bb = int((float(r) + 0.5f) * inv_z), c = r - bb * fnz;
                    const int fi = wrap_cell(flo0 + a, nf);
                    const int fj = wrap_cell(flo1 + bb, nf);
                    const int fk = wrap_cell(flo2 + c, nf);
                    heads[u] = b.fine_head[(size_t(fi) * nf + fj) * nf + fk];
                }
            }
#pragma unroll 1
            for (int u = 0; u < kHeads; ++u) {
                int slot = u == 0 ? heads[0] : (u == 1 ? heads[1] : (u == 2 ? heads[2] : heads[3]));
                for (int guard = 0; slot >= 0 && guard < b.nslots; ++guard) {
                    // the three loads of a list entry are independent
                    const int nxt = b.fine_next[slot];
                    const int key = b.agg_cell[slot];
                    const float4 of = b.agg_f4[slot];
                    ++visited;
                    if (slot == src) {
                        sm.found_source = 1;
                    } else {
                        const int oa = wrap_cell((key & 1023) - rlo0, nd);
                        const int ob = wrap_cell(((key >> 10) & 1023) - rlo1, nd);
                        const int oc = wrap_cell((key >> 20) - rlo2, nd);
                        if (oa < nx && ob < ny && oc < nz)
                            consider(slot, (long long)((oa * ny + ob) * nz + oc) * b.nslots + slot, of);
                    }
                    slot = nxt;
                }
            }
        }
        if (visited) atomicAdd(&sm.flat_base, visited);
        __syncthreads();
    } else {
    for (int c0 = 0; c0 < n_scan; c0 += kCellChunk) {
        const int nch = min(kCellChunk, n_scan - c0);
        int cnt_local = 0;
        // each thread owns a contiguous run of cells so the block scan keeps scan order
        const int per = (nch + NT - 1) / NT;
        const int my0 = tid * per;
        for (int k = 0; k < per; ++k) {
            int s = my0 + k;
            if (s < nch) {
                int g = c0 + s;
                int a = g / (ny * nz), r = g % (ny * nz), bb = r / nz, c = r % nz;
                int ii = periodic_cell(rg.lo[0] + a, b.n_div);
                int jj = periodic_cell(rg.lo[1] + bb, b.n_div);
                int kk = periodic_cell(rg.lo[2] + c, b.n_div);
                int lin = (ii * b.n_div + jj) * b.n_div + kk;
                sm.cell_lin[s] = lin;
                cnt_local += b.cell_n[lin];
            }
        }
        int total;
        int base = block_exclusive_scan(cnt_local, sm.warp_tmp, total);
        {
            int run = base;
            for (int k = 0; k < per; ++k) {
                int s = my0 + k;
                if (s < nch) {
                    sm.cell_prefix[s] = run;
                    run += b.cell_n[sm.cell_lin[s]];
                }
            }
            if (tid == 0) sm.cell_prefix[nch] = total;
        }
        __syncthreads();
        for (int f = tid; f < total; f += NT) {
            // cell of flat item f: last prefix <= f
            int lo = 0, hi = nch - 1;
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (sm.cell_prefix[mid] <= f) lo = mid; else hi = mid - 1;
            }
            const int lin = sm.cell_lin[lo];
            const int slot = b.cell_items[size_t(lin) * b.cell_cap + (f - sm.cell_prefix[lo])];
            if (slot == src) {
                sm.found_source = 1;
                continue;
            }
            consider(slot, (long long)(c0 + lo) * b.nslots + slot, b.agg_f4[slot]);
        }
        __syncthreads();
        if (tid == 0) sm.flat_base += total;
        __syncthreads();
    }
    }
    if (tid == 0) {
        sm.out.n_scanned = sm.flat_base;
        sm.out.n_cells = n_cells_visited;
    }
    if (!sm.found_source) {
        if (tid == 0) sm.out.status = ST_VERLET;  // "Aggregate not on the verlet list"
        __syncthreads();
        return;
    }
    // bounding-sphere filter, second part: the exact FP64 sweep
    {
        const int n_screen = sm.n_screen;
        for (int k = tid; k < n_screen; k += NT) {
            const int slot = sm.cand_prefix[k];
            const long long key = screen_key[k];
            const double ox = A(b, AGG_X, slot), oy = A(b, AGG_Y, slot), oz = A(b, AGG_Z, slot);
            const double orm = A(b, AGG_RMAX, slot);
            const double db = sweep_contact_distance(sp, rmax_src, Vec3{ox, oy, oz}, orm, dir, dist, b.L);
            if (db < dist) {
                const int j = atomicAdd(&sm.n_cand, 1);
                sm.cand_db[j] = db;
                sm.cand_key[j] = key;
                sm.cand_slot[j] = slot;
            }
        }
        __syncthreads();
        if (tid == 0) {
            sm.out.n_candidates = sm.n_cand;
            sm.out.cyc_scan = clock64() - sm.t_q0;
        }
    }
    const int nc = sm.n_cand;
    if (nc == 0) {
        __syncthreads();
        return;
    }

    // order candidates by (d_b, scan position): rank sort
    for (int k = tid; k < nc; k += NT) {
        double dk = sm.cand_db[k];
        long long fk = sm.cand_key[k];
        int rank = 0;
        for (int m = 0; m < nc; ++m) {
            double dm = sm.cand_db[m];
            rank += (dm < dk) || (dm == dk && sm.cand_key[m] < fk);
        }
        sm.cand_order[rank] = k;
    }
    __syncthreads();
    // per-candidate sphere prefix (in sorted order) and best keys; up to 32
    // candidates the counts are read by the lanes of warp 0 at once and
    // scanned there (the chain of dependent loads of one thread otherwise)
    if (nc <= 32) {
        if (tid < 32) {
            const int cs = tid < nc ? sm.cand_slot[sm.cand_order[tid]] : 0;
            const int cnt = tid < nc ? b.agg_n[cs] : 0;
            const int coff = tid < nc ? b.agg_off[cs] : 0;
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (tid >= o) incl += y;
            }
            if (tid < nc) {
                sm.cand_prefix[tid] = incl - cnt;
                if (tid < SM::kCandCache) {
                    sm.c_pre[tid] = incl - cnt;
                    sm.c_slot[tid] = cs;
                    sm.c_off[tid] = coff;
                }
            }
            if (tid == nc - 1) {
                sm.cand_prefix[nc] = incl;
                if (nc <= SM::kCandCache) sm.c_pre[nc] = incl;
            }
        }
    } else if (tid == 0) {
        int run = 0;
        for (int r = 0; r < nc; ++r) {
            sm.cand_prefix[r] = run;
            run += b.agg_n[sm.cand_slot[sm.cand_order[r]]];
        }
        sm.cand_prefix[nc] = run;
    }
    for (int r = tid; r < nc; r += NT) {
        sm.best_res[r] = ~0ULL;
        sm.best_ij[r] = ~0ULL;
    }
    __syncthreads();

    // ---- 3: pair search
    const int n_mov = b.agg_n[src];
    const int off_m = b.agg_off[src];
    // the candidates' sorted prefix, slots and pool offsets: shared memory up
    // to kCandCache candidates, device memory beyond
    const bool small_nc = nc <= SM::kCandCache;
    const int *cpre = small_nc ? sm.c_pre : sm.cand_prefix;
    auto cand_slot_of = [&](int r) { return small_nc ? sm.c_slot[r] : sm.cand_slot[sm.cand_order[r]]; };
    auto cand_off_of = [&](int r) { return small_nc ? sm.c_off[r] : b.agg_off[sm.cand_slot[sm.cand_order[r]]]; };
    const int n_other = cpre[nc];
    if (tid == 0) sm.out.n_cand_spheres = n_other;
    // With few candidates and a large moving aggregate, the moving spheres
    // that cannot come within reach of any candidate's spheres are dropped
    // before the pair loop. Each candidate's extent is measured from its own
    // FP32 spheres (the stored r_max of a monomer can be smaller than its
    // radius), and the test keeps two screening margins: a moving sphere
    // whose sweep reaches a candidate sphere always reaches the ball around
    // the candidate centre that holds all its spheres.
    const bool cull = nc <= kCullCands && n_mov >= 8;
    if (cull) {
        for (int r = tid; r < nc; r += NT) {
            sm.cand_c[r] = b.agg_f4[cand_slot_of(r)];
            sm.cand_ext[r] = 0.f;
        }
        __syncthreads();
        for (int f = tid; f < n_other; f += NT) {
            int r = 0;
            while (r + 1 < nc && cpre[r + 1] <= f) ++r;
            const float4 q = pool_pos[cand_off_of(r) + (f - cpre[r])];
            const float4 c = sm.cand_c[r];
            float ex = q.x - c.x, ey = q.y - c.y, ez = q.z - c.z;
            ex -= w.L * rintf(ex * w.invL);
            ey -= w.L * rintf(ey * w.invL);
            ez -= w.L * rintf(ez * w.invL);
            const float e = sqrtf(ex * ex + ey * ey + ez * ez) + q.w;
            atomicMax(reinterpret_cast<int *>(&sm.cand_ext[r]), __float_as_int(e));  // e >= 0
        }
        __syncthreads();
    }
    // one candidate sphere against one moving sphere of the tile: FP32
    // capsule screen, exact FP64 swept test, the candidate's running minimum
    auto try_pair = [&](int t0, int i, const float4 &q, int pj, int r, int jl) {
        const float4 p = sm.mov[i];
        Sweep32 wi = w;
        wi.px = p.x;
        wi.py = p.y;
        wi.pz = p.z;
        if (!capsule_hit(wi, q.x, q.y, q.z, p.w + q.w + margin)) return;
        const int si = pool_id[off_m + t0 + i];
        const int sj = pool_id[pj];
        double res = sweep_contact_distance(sph_pos(b, si), S(b, SPH_R, si), sph_pos(b, sj), S(b, SPH_R, sj), dir,
                                            dist, b.L);
        atomicAdd(&sm.n_refined, 1);
        if (!(res < CUDART_INF)) return;
        unsigned long long key = dkey(res);
        atomicMin(&sm.best_res[r], key);
        int k = atomicAdd(&sm.n_surv, 1);
        int4 rec = make_int4(r, t0 + i, jl, 0);
        if (k < kMaxSurvivorsSmem) {
            sm.surv[k] = rec;
            sm.surv_res[k] = res;
        } else if (k - kMaxSurvivorsSmem < b.surv_cap) {
            b.surv[k - kMaxSurvivorsSmem] = rec;
            b.surv_res[k - kMaxSurvivorsSmem] = res;
        }
    };
    if (tid == 0) {
        // basis across the motion: u1 = dir x (axis least aligned), u2 = dir x u1
        const float ax = fabsf(w.ux), ay = fabsf(w.uy), az = fabsf(w.uz);
        float ex = 0.f, ey = 0.f, ez = 0.f;
        if (ax <= ay && ax <= az) ex = 1.f; else if (ay <= az) ey = 1.f; else ez = 1.f;
        float u1x = w.uy * ez - w.uz * ey, u1y = w.uz * ex - w.ux * ez, u1z = w.ux * ey - w.uy * ex;
        const float inv = rsqrtf(u1x * u1x + u1y * u1y + u1z * u1z);
        u1x *= inv;
        u1y *= inv;
        u1z *= inv;
        sm.basis[0] = u1x;
        sm.basis[1] = u1y;
        sm.basis[2] = u1z;
        sm.basis[3] = w.uy * u1z - w.uz * u1y;
        sm.basis[4] = w.uz * u1x - w.ux * u1z;
        sm.basis[5] = w.ux * u1y - w.uy * u1x;
    }
    for (int t0 = 0; t0 < n_mov; t0 += kMoveTile) {
        const int nt = min(kMoveTile, n_mov - t0);
        float reach_local = 0.f, rad_local = 0.f, span_local = 0.f;
        for (int i = tid; i < nt; i += NT) {
            float4 p = pool_pos[off_m + t0 + i];
            sm.mov[i] = p;
            // distance of this moving sphere from the source centre, + radius
            float ex = p.x - w.px, ey = p.y - w.py, ez = p.z - w.pz;
            // unreduced: member positions are stored around the centre
            span_local = fmaxf(span_local, sqrtf(ex * ex + ey * ey + ez * ez) + p.w);
            ex -= w.L * rintf(ex * w.invL);
            ey -= w.L * rintf(ey * w.invL);
            ez -= w.L * rintf(ez * w.invL);
            reach_local = fmaxf(reach_local, sqrtf(ex * ex + ey * ey + ez * ez) + p.w);
            rad_local = fmaxf(rad_local, p.w);
        }
        // block max of the moving tile's extent and of its radii
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            reach_local = fmaxf(reach_local, __shfl_xor_sync(0xffffffffu, reach_local, o));
            rad_local = fmaxf(rad_local, __shfl_xor_sync(0xffffffffu, rad_local, o));
            span_local = fmaxf(span_local, __shfl_xor_sync(0xffffffffu, span_local, o));
        }
        if ((tid & 31) == 0) {
            sm.warp_f[tid >> 5] = reach_local;
            sm.warp_tmp[tid >> 5] = __float_as_int(rad_local);  // non-negative: int order is float order
            sm.warp_f2[tid >> 5] = span_local;
        }
        __syncthreads();
        if (tid == 0) {
            float m = 0.f, rr = 0.f, sp = 0.f;
            for (int k = 0; k < NT / 32; ++k) {
                m = fmaxf(m, sm.warp_f[k]);
                rr = fmaxf(rr, __int_as_float(sm.warp_tmp[k]));
                sp = fmaxf(sp, sm.warp_f2[k]);
            }
            sm.mov_reach = m;
            sm.grid_span = sp;
            // Moving spheres binned on a grid across the motion. A pair can
            // pass the capsule test only if the candidate sphere lies within
            // r_p + r_q + margin of the moving sphere's line of motion, so
            // with cells at least that wide the 3 x 3 cells around the
            // candidate's position hold every moving sphere it can meet.
            // Used for large pair counts; at most kGridMax^2 cells.
            const bool big = nt >= 32 && (long long)nt * n_other >= 16384;
            sm.grid_on = big;
            if (big) {
                const float h = (2.f * rr + margin) * 1.001f + margin;
                const float span = 2.f * (sp + margin);
                const int g = max(1, min(SM::kGridMax, int(span / h) + 1));
                sm.grid_g = g;
                sm.grid_h = fmaxf(h, span / float(g));
                sm.grid_half = 0.5f * float(g) * sm.grid_h;
                sm.grid_rmax = rr;
            }
        }
        __syncthreads();
        const float mov_reach = sm.mov_reach + margin;
        const bool grid = sm.grid_on;
        int n_sel = nt;
        if (grid) {
            // counting sort of the tile's spheres by grid cell
            const int g = sm.grid_g, g2 = g * g;
            const float gh = sm.grid_h, ghalf = sm.grid_half;
            const float b0 = sm.basis[0], b1 = sm.basis[1], b2 = sm.basis[2];
            const float b3 = sm.basis[3], b4 = sm.basis[4], b5 = sm.basis[5];
            auto cell_of_mov = [&](int i) {
                // member positions are stored unwrapped around the aggregate
                // centre, so p - centre is the true offset
                const float4 p = sm.mov[i];
                const float ex = p.x - w.px, ey = p.y - w.py, ez = p.z - w.pz;
                const float a1 = ex * b0 + ey * b1 + ez * b2, a2 = ex * b3 + ey * b4 + ez * b5;
                const int c1 = min(g - 1, max(0, int(floorf((a1 + ghalf) / gh))));
                const int c2 = min(g - 1, max(0, int(floorf((a2 + ghalf) / gh))));
                return c1 * g + c2;
            };
            for (int c = tid; c <= g2; c += NT) sm.cell_prefix[c] = 0;
            __syncthreads();
            for (int i = tid; i < nt; i += NT) atomicAdd(&sm.cell_prefix[cell_of_mov(i)], 1);
            __syncthreads();
            {
                const int per = (g2 + NT - 1) / NT, my0 = tid * per;
                int cnt = 0;
                for (int k = 0; k < per; ++k)
                    if (my0 + k < g2) cnt += sm.cell_prefix[my0 + k];
                int total;
                int run = block_exclusive_scan(cnt, sm.warp_tmp, total);
                for (int k = 0; k < per; ++k)
                    if (my0 + k < g2) {
                        const int v = sm.cell_prefix[my0 + k];
                        sm.cell_prefix[my0 + k] = run;
                        sm.cell_lin[my0 + k] = run;
                        run += v;
                    }
                if (tid == 0) sm.cell_prefix[g2] = total;
            }
            __syncthreads();
            for (int i = tid; i < nt; i += NT) sm.mov_sel[atomicAdd(&sm.cell_lin[cell_of_mov(i)], 1)] = short(i);
            __syncthreads();
        } else if (cull) {
            if (tid == 0) sm.n_sel = 0;
            __syncthreads();
            for (int i = tid; i < nt; i += NT) {
                const float4 p = sm.mov[i];
                Sweep32 wi = w;
                wi.px = p.x;
                wi.py = p.y;
                wi.pz = p.z;
                bool hit = false;
                for (int r = 0; r < nc && !hit; ++r) {
                    const float4 c = sm.cand_c[r];
                    const float e = sm.cand_ext[r];
                    hit = !(e < 0.25f * w.L) || capsule_hit(wi, c.x, c.y, c.z, p.w + e + 2.f * margin);
                }
                if (hit) sm.mov_sel[atomicAdd(&sm.n_sel, 1)] = short(i);
            }
            __syncthreads();
            n_sel = sm.n_sel;
        }
        for (int f = tid; f < n_other && n_sel > 0; f += NT) {
            int lo = 0, hi = nc - 1;
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (cpre[mid] <= f) lo = mid; else hi = mid - 1;
            }
            const int r = lo;
            const int jl = f - cpre[r];
            const int pj = cand_off_of(r) + jl;
            const float4 q = pool_pos[pj];
            // can any moving sphere reach this one?
            if (!capsule_hit(w, q.x, q.y, q.z, mov_reach + q.w)) continue;
            // the grid needs the pair's reach within a cell, and a swept zone
            // short of the box (else the capsule test passes every pair)
            if (grid && q.w <= sm.grid_rmax + margin &&
                w.zmax + 2.f * (sm.grid_rmax + q.w + margin) + 8.f * margin < w.L) {
                const int g = sm.grid_g;
                const float mr = sm.grid_span + 2.f * margin;  // bound of |moving sphere - centre|
                const float dx = q.x - w.px, dy = q.y - w.py, dz = q.z - w.pz;
                // periodic shifts k the capsule test can give this sphere
                // against a moving sphere: rint((q - p_i - c) / L), p_i within mr
                const int kx0 = int(rintf((dx - w.cx - mr) * w.invL)), kx1 = int(rintf((dx - w.cx + mr) * w.invL));
                const int ky0 = int(rintf((dy - w.cy - mr) * w.invL)), ky1 = int(rintf((dy - w.cy + mr) * w.invL));
                const int kz0 = int(rintf((dz - w.cz - mr) * w.invL)), kz1 = int(rintf((dz - w.cz + mr) * w.invL));
                for (int kx = kx0; kx <= kx1; ++kx)
                    for (int ky = ky0; ky <= ky1; ++ky)
                        for (int kz = kz0; kz <= kz1; ++kz) {
                            const float ex = dx - w.L * float(kx), ey = dy - w.L * float(ky), ez = dz - w.L * float(kz);
                            const float a1 = ex * sm.basis[0] + ey * sm.basis[1] + ez * sm.basis[2];
                            const float a2 = ex * sm.basis[3] + ey * sm.basis[4] + ez * sm.basis[5];
                            const int c1 = int(floorf((a1 + sm.grid_half) / sm.grid_h));
                            const int c2 = int(floorf((a2 + sm.grid_half) / sm.grid_h));
                            for (int x1 = max(0, c1 - 1); x1 <= min(g - 1, c1 + 1); ++x1)
                                for (int x2 = max(0, c2 - 1); x2 <= min(g - 1, c2 + 1); ++x2) {
                                    const int cell = x1 * g + x2;
                                    for (int k = sm.cell_prefix[cell]; k < sm.cell_prefix[cell + 1]; ++k) {
                                        const int i = int(sm.mov_sel[k]);
                                        const float4 p = sm.mov[i];
                                        // the shift the capsule test will use for this pair
                                        // (same expression): each pair is tried once
                                        if (int(rintf(((q.x - p.x) - w.cx) * w.invL)) != kx ||
                                            int(rintf(((q.y - p.y) - w.cy) * w.invL)) != ky ||
                                            int(rintf(((q.z - p.z) - w.cz) * w.invL)) != kz)
                                            continue;
                                        try_pair(t0, i, q, pj, r, jl);
                                    }
                                }
                        }
            } else {
                for (int ii = 0; ii < n_sel; ++ii) try_pair(t0, (cull && !grid) ? int(sm.mov_sel[ii]) : ii, q, pj, r, jl);
            }
        }
        __syncthreads();
    }
    const int n_surv = sm.n_surv;
    if (n_surv > kMaxSurvivorsSmem + b.surv_cap) {
        if (tid == 0) sm.out.status = ST_CAPACITY;
        __syncthreads();
        return;
    }
    // lexicographic (moving index, other index) among each candidate's minima
    for (int k = tid; k < n_surv; k += NT) {
        int4 rec = (k < kMaxSurvivorsSmem) ? sm.surv[k] : b.surv[k - kMaxSurvivorsSmem];
        double res = (k < kMaxSurvivorsSmem) ? sm.surv_res[k] : b.surv_res[k - kMaxSurvivorsSmem];
        if (dkey(res) == sm.best_res[rec.x]) {
            unsigned long long ij = (static_cast<unsigned long long>(rec.y) << 32) | static_cast<unsigned>(rec.z);
            atomicMin(&sm.best_ij[rec.x], ij);
        }
    }
    __syncthreads();

    // ---- 4: the reference's ordered walk with early exits (warp 0; up to
    // 32 candidates their values are read by the lanes at once and the walk
    // goes through them by shuffles)
    if (tid < 32) {
        double best = CUDART_INF;
        int best_r = -1;
        if (nc <= 32) {
            const double db_l = tid < nc ? sm.cand_db[sm.cand_order[tid]] : 0.0;
            const unsigned long long br_l = tid < nc ? sm.best_res[tid] : ~0ULL;
            for (int r = 0; r < nc; ++r) {
                const double db_r = __shfl_sync(0xffffffffu, db_l, r);
                const unsigned long long br_r = __shfl_sync(0xffffffffu, br_l, r);
                if (best <= 0.) break;
                if (best < db_r) break;
                if (br_r == ~0ULL) continue;  // no finite pair: +inf never wins
                const double res = dkey_inv(br_r);
                if (res < best) {
                    best = res;
                    best_r = r;
                }
            }
        } else if (tid == 0) {
            for (int r = 0; r < nc; ++r) {
                if (best <= 0.) break;
                if (best < sm.cand_db[sm.cand_order[r]]) break;
                if (sm.best_res[r] == ~0ULL) continue;  // no finite pair: +inf never wins
                double res = dkey_inv(sm.best_res[r]);
                if (res < best) {
                    best = res;
                    best_r = r;
                }
            }
        }
        if (tid == 0) {
            sm.out.distance = best;
            if (best_r >= 0) {
                unsigned long long ij = sm.best_ij[best_r];
                int i = int(ij >> 32), j = int(ij & 0xffffffffu);
                int cslot = cand_slot_of(best_r);
                sm.out.moving_sphere = pool_id[off_m + i];
                sm.out.other_sphere = pool_id[b.agg_off[cslot] + j];
                sm.out.other_slot = cslot;
            }
            sm.out.n_pairs_refined = sm.n_refined;
            sm.out.cyc_pairs = clock64() - sm.t_q0 - sm.out.cyc_scan;
        }
    }
    __syncthreads();
}

// ------------------------------------------------------------- Verlet grid
// Remove / insert a slot in a cell's unordered list (one thread, O(1)).
__device__ __forceinline__ void cell_remove(const DevBox &b, int cell, int slot) {
    const int n = b.cell_n[cell];
    int *items = b.cell_items + size_t(cell) * b.cell_cap;
    int k = b.cell_pos[slot];
    if (k < 0 || k >= n || items[k] != slot) {  // not where recorded: search
        k = 0;
        while (k < n && items[k] != slot) ++k;
        if (k == n) return;
    }
    const int last = items[n - 1];
    items[k] = last;
    b.cell_pos[last] = k;
    b.cell_pos[slot] = -1;
    b.cell_n[cell] = n - 1;
}
__device__ __forceinline__ void cell_insert(const DevBox &b, int cell, int slot) {
    const int n = b.cell_n[cell];
    if (n >= b.cell_cap) {
        b.sc->cell_overflow = 1;
        b.sc->status = ST_CAPACITY;
        return;
    }
    b.cell_items[size_t(cell) * b.cell_cap + n] = slot;
    b.cell_pos[slot] = n;
    b.cell_n[cell] = n + 1;
}
// Fine grid cells, in FP32: the fine grid is this library's own search
// structure (the neighbours that count are the Verlet grid's), so a cell only
// has to agree with the query's fine range, which is widened by far more
// than the FP32 rounding. Periodic index of one coordinate (a position that
// rounds to L falls in cell 0, its periodic image).
__device__ __forceinline__ int fine_index(float x, float step, int n) {
    float f = floorf(x * step);
    if (!(f > -1e6f && f < 1e6f)) f = 0.f;
    return periodic_cell(static_cast<int>(f), n);
}
__device__ __forceinline__ int fine_cell_of(const DevBox &b, float x, float y, float z) {
    const int n = b.fine_div;
    return (fine_index(x, b.fine_step_f, n) * n + fine_index(y, b.fine_step_f, n)) * n +
           fine_index(z, b.fine_step_f, n);
}
__device__ __forceinline__ int fine_cell_of(const DevBox &b, Vec3 p) {
    return fine_cell_of(b, float(p.x), float(p.y), float(p.z));
}
// Take a slot out of its fine cell's list / put it at the head of one (one thread).
__device__ __forceinline__ void fine_unlink(const DevBox &b, int slot) {
    const int c = b.fine_cell[slot];
    if (c < 0) return;
    const int p = b.fine_prev[slot], n = b.fine_next[slot];
    if (p >= 0) b.fine_next[p] = n; else b.fine_head[c] = n;
    if (n >= 0) b.fine_prev[n] = p;
    b.fine_cell[slot] = -1;
}
__device__ __forceinline__ void fine_link(const DevBox &b, int slot, int c) {
    const int n = b.fine_head[c];
    b.fine_next[slot] = n;
    b.fine_prev[slot] = -1;
    if (n >= 0) b.fine_prev[n] = slot;
    b.fine_head[c] = slot;
    b.fine_cell[slot] = c;
}
// Aggregate::update_verlet (aggregat.cpp:706-717) for a new position, and
// the same move in the fine grid (one thread). The loads that do not depend
// on one another are issued first: a move costs three rounds of memory
// latency instead of one per list operation.
__device__ __forceinline__ void regrid_to(const DevBox &b, int slot, int key, int fc) {
    const bool fine = b.fine_div > 0;
    const int c = cell_index(b, key);
    // pass 1: everything indexed by the slot or by the new cells
    const int old_key = b.agg_cell[slot];
    const int old = cell_index(b, old_key);
    const int k = b.cell_pos[slot];
    const int n_new = b.cell_n[c];
    const int fold = fine ? b.fine_cell[slot] : -1;
    const int fprev = fine ? b.fine_prev[slot] : -1;
    const int fnext = fine ? b.fine_next[slot] : -1;
    const int fhead = fine ? b.fine_head[fc] : -1;
    if (key != old_key) {
        // passes 2 and 3: the old cell's length, then its last item
        const int n_old = b.cell_n[old];
        int *items = b.cell_items + size_t(old) * b.cell_cap;
        int kk = k;
        if (kk < 0 || kk >= n_old || items[kk] != slot) {  // not where recorded: search
            kk = 0;
            while (kk < n_old && items[kk] != slot) ++kk;
        }
        if (kk < n_old) {
            const int last = items[n_old - 1];
            items[kk] = last;
            b.cell_pos[last] = kk;
            b.cell_n[old] = n_old - 1;
        }
        if (n_new >= b.cell_cap) {
            b.sc->cell_overflow = 1;
            b.sc->status = ST_CAPACITY;
            b.cell_pos[slot] = -1;
        } else {
            b.cell_items[size_t(c) * b.cell_cap + n_new] = slot;
            b.cell_pos[slot] = n_new;
            b.cell_n[c] = n_new + 1;
        }
        b.agg_cell[slot] = key;
    }
    if (fine && fc != fold) {
        // unlink from the old fine cell, link at the head of the new one (the
        // two lists are distinct, so the loads above stay valid)
        if (fold >= 0) {
            if (fprev >= 0) b.fine_next[fprev] = fnext; else b.fine_head[fold] = fnext;
            if (fnext >= 0) b.fine_prev[fnext] = fprev;
        }
        b.fine_next[slot] = fhead;
        b.fine_prev[slot] = -1;
        if (fhead >= 0) b.fine_prev[fhead] = slot;
        b.fine_head[fc] = slot;
        b.fine_cell[slot] = fc;
    }
}

__device__ __forceinline__ void regrid(const DevBox &b, int slot, Vec3 p) {
    regrid_to(b, slot, cell_of(b, p), b.fine_div > 0 ? fine_cell_of(b, p) : -1);
}

// --------------------------------------------------------------- translate
// Aggregate::translate (aggregats/aggregat.cpp:148-161). Lanes 0-2 of warp 0
// take one axis each (the FP64 work of one lane costs as much as that of the
// warp), lane 0 then moves the slot in the grids.
__device__ inline void block_translate(const DevBox &b, int slot, Vec3 v, double *refpos_sm) {
    const int tid = threadIdx.x;
    if (tid < 32) {
        double x = 0.0;
        float xf = 0.f;
        int vc = 0, fc = 0;
        if (tid < 3) {
            const double vl = tid == 0 ? v.x : (tid == 1 ? v.y : v.z);
            x = periodic_position(A(b, AGG_X + tid, slot) + vl, b.L);
            A(b, AGG_X + tid, slot) = x;
            refpos_sm[tid] = x - A(b, AGG_RX + tid, slot);
            xf = float(x);
            vc = min(max(verlet_coord(x, b.step), 0), b.n_div - 1);
            if (b.fine_div > 0) fc = fine_index(xf, b.fine_step_f, b.fine_div);
        }
        const float yf = __shfl_sync(0xffffffffu, xf, 1), zf = __shfl_sync(0xffffffffu, xf, 2);
        const int vy = __shfl_sync(0xffffffffu, vc, 1), vz = __shfl_sync(0xffffffffu, vc, 2);
        const int fy = __shfl_sync(0xffffffffu, fc, 1), fz = __shfl_sync(0xffffffffu, fc, 2);
        if (tid == 0) {
            const float rm = b.agg_f4[slot].w;  // r_max is unchanged by a move
            b.agg_f4[slot] = make_float4(xf, yf, zf, rm);
            const int n = b.fine_div;
            regrid_to(b, slot, cell_key(vc, vy, vz), n > 0 ? (fc * n + fy) * n + fz : -1);
        }
    }
    __syncthreads();
    const double rx = refpos_sm[0], ry = refpos_sm[1], rz = refpos_sm[2];
    const int n = b.agg_n[slot], off = b.agg_off[slot];
    int *pool_id = b.pool_id[b.sc->pool_sel];
    float4 *pool_pos = b.pool_pos[b.sc->pool_sel];
    for (int k = tid; k < n; k += blockDim.x) {
        int s = pool_id[off + k];
        double x = rx + S(b, SPH_RX, s);
        double y = ry + S(b, SPH_RY, s);
        double z = rz + S(b, SPH_RZ, s);
        S(b, SPH_X, s) = x;
        S(b, SPH_Y, s) = y;
        S(b, SPH_Z, s) = z;
        pool_pos[off + k] = make_float4(float(x), float(y), float(z), float(S(b, SPH_R, s)));
    }
    __syncthreads();
}

}  // namespace mcacg
