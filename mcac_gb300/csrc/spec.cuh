// Speculative steps of the device loop: one box advanced by a thread-block
// cluster of K CTAs, K MC steps per round.
//
// Between two events (merges) the pick tree does not change, so the picks
// and directions of the next K steps are fixed by the box's rand() stream
// alone (one value for the pick, two for the direction, per step). The
// leader CTA draws them; each CTA of the cluster answers one step's contact
// query on the state at the start of the round, with its own scratch. The
// leader then commits the steps in order with the sequential loop's own
// code (translation, time, merge, pick tree, counters, stop criteria), and
// stops at the first step whose answer could differ from the sequential
// one: a step of an aggregate already moved in this round, or one whose
// swept bounding capsule comes within reach of the sweep of a step
// committed before it in the round, or one after an event (the tree
// changes). Everything not committed is drawn again next round from the
// same place of the stream, so the run is the sequential loop's, bit for bit
// (the aggregates a query can hit are those whose bounding spheres reach its
// swept bounding sphere: an aggregate whose whole move stays out of that
// reach is not a candidate before or after its move, and nothing else a
// query reads changes without an event).
//
// Cluster synchronisation is the hardware cluster barrier; every CTA of a
// cluster passes the same number of barriers (the loop's exit is decided by
// a flag read by all after the same barrier), and no CTA leaves while
// another may still read its shared memory.
#pragma once
#include <cooperative_groups.h>

#include "run.cuh"

namespace mcacg {

constexpr int kSpecMax = 8;               // CTAs per box at most (the portable cluster size)
constexpr int kSpecSurvivors = 1 << 14;   // refined pairs in HBM per helper CTA

// The query scratch of one helper CTA (device memory, sized for its box).
struct SpecScratch {
    double *cand_db;
    long long *cand_key;
    int *cand_slot, *cand_order, *cand_prefix;
    unsigned long long *best_res, *best_ij;
    int4 *surv;
    double *surv_res;
    int surv_cap;
    int pad;
};

struct SpecJob {
    unsigned long long target;  // pick target in the tree's fixed point
    int r1, r2;                 // the direction's two rand() values
};

struct SpecResult {
    QueryOut q;
    int slot;  // -1: the pick found no live slot
    int pad;
    double dir[3];
    double full, dt_indiv, rmax;
    double pos[3];  // the aggregate's centre at the start of the round
};

// The round's shared record; the leader's copy is the one in use.
struct SpecShared {
    int stop, n_jobs, tree_gen, ok;
    double dt;  // the steps' time increment (the tree's, unchanged in a round)
    SpecJob job[kSpecMax];
    SpecResult res[kSpecMax];
    double move[kSpecMax];
    RandStream rng0;  // the leader's stream at the start of the round
};

// Could the committed step 'a' (its aggregate swept from a.pos along a.dir
// for move_a) be a candidate of query 'b' (b.pos along b.dir for b.full) at
// any point of its move? Conservative: true when the two sweeps come within
// the two bounding radii (plus a margin far above the FP64 rounding of the
// reference's own bounding-sphere test), when they are long enough for a
// second periodic image to matter, and for the same aggregate.
__device__ inline bool spec_conflict(const SpecResult &a, double move_a, const SpecResult &b, double L) {
    if (a.slot == b.slot) return true;
    const double reach = a.rmax + b.rmax;
    const double ext = move_a + b.full;
    if (!(ext + reach < 0.45 * L)) return true;
    // w0 = start of b's sweep minus start of a's, minimum image: with all
    // extents below L/2 no other image can come within reach
    const double w0x = -periodic_distance(a.pos[0] - b.pos[0], L);
    const double w0y = -periodic_distance(a.pos[1] - b.pos[1], L);
    const double w0z = -periodic_distance(a.pos[2] - b.pos[2], L);
    const double ux = b.dir[0] * b.full, uy = b.dir[1] * b.full, uz = b.dir[2] * b.full;
    const double vx = a.dir[0] * move_a, vy = a.dir[1] * move_a, vz = a.dir[2] * move_a;
    // closest points of the segments w0 + s u and t v (s, t in [0, 1])
    const double aa = ux * ux + uy * uy + uz * uz;
    const double bb = ux * vx + uy * vy + uz * vz;
    const double cc = vx * vx + vy * vy + vz * vz;
    const double dd = ux * w0x + uy * w0y + uz * w0z;
    const double ee = vx * w0x + vy * w0y + vz * w0z;
    double s = 0.0, t = 0.0;
    if (aa > 0.0 && cc > 0.0) {
        const double den = aa * cc - bb * bb;
        s = den > 0.0 ? fmin(fmax((bb * ee - cc * dd) / den, 0.0), 1.0) : 0.0;
        t = (bb * s + ee) / cc;
        if (t < 0.0) {
            t = 0.0;
            s = fmin(fmax(-dd / aa, 0.0), 1.0);
        } else if (t > 1.0) {
            t = 1.0;
            s = fmin(fmax((bb - dd) / aa, 0.0), 1.0);
        }
    } else if (aa > 0.0) {
        s = fmin(fmax(-dd / aa, 0.0), 1.0);
    } else if (cc > 0.0) {
        t = fmin(fmax(ee / cc, 0.0), 1.0);
    }
    const double px = w0x + s * ux - t * vx, py = w0y + s * uy - t * vy, pz = w0z + s * uz - t * vz;
    const double lim = reach * (1.0 + 1e-6) + 1e-9 * L;
    return px * px + py * py + pz * pz <= lim * lim;
}

// The leader's round set-up (all threads of the leader CTA): the stop
// checks of a step's start, then the picks and directions of up to K steps
// from the stream (the stream's state at the start is kept).
template <class RS>
__device__ inline void spec_prepare(const BoxRun &R, RS &sm, SpecShared &sh, int K, long long left) {
    if (threadIdx.x == 0) {
        RunState &st = *R.st;
        int stop = st.finished || st.status != ST_OK;
        if (!stop && run_finished(R, st, R.box.sc->n_alive)) {
            st.finished = 1;
            stop = 1;
        }
        if (!stop && sm.deadline != 0ULL && global_ns() >= sm.deadline) stop = 1;
        if (!stop && left <= 0) stop = 1;
        sh.stop = stop;
        sh.n_jobs = 0;
        if (!stop) {
            int nj = left < K ? int(left) : K;
            if (R.phys.growth) nj = 1;  // each step of a growing box changes every radius
            sh.rng0 = st.rng;
            for (int i = 0; i < nj; ++i) {
                sh.job[i].target = pick_target(st.rng, st.tree_total);
                sh.job[i].r1 = st.rng.next_int();
                sh.job[i].r2 = st.rng.next_int();
            }
            sh.n_jobs = nj;
            sh.dt = st.inv_weight;
        }
    }
    __syncthreads();
}

// One CTA's step of the round (all its threads): the pick's tree descent,
// the direction and the contact query on the round's starting state; the
// answer goes to the leader's record.
template <class RS>
__device__ inline void spec_query(const BoxRun &R, RS &sm, const SpecJob *job, SpecResult *out) {
    const DevBox &b = R.box;
    if (threadIdx.x < 32) {
        const unsigned long long t = job->target;
        const int slot = tree_sample(R, sm.tree, t);
        if (threadIdx.x == 0) {
            const bool live = slot >= 0 && slot < b.nslots && b.agg_n[slot] > 0;
            sm.slot = live ? slot : -1;
            if (live) {
                direction_from(job->r1, job->r2, sm.dir);
                sm.full = A(b, AGG_LPM, slot);
            }
        }
    }
    __syncthreads();
    const int slot = sm.slot;
    if (slot >= 0 && R.lim.with_collisions) block_query(b, slot, Vec3{sm.dir[0], sm.dir[1], sm.dir[2]}, sm.full, sm.u.q);
    if (threadIdx.x == 0) {
        SpecResult r;
        r.slot = slot;
        r.pad = 0;
        if (slot >= 0 && R.lim.with_collisions) {
            r.q = sm.u.q.out;
        } else {
            r.q = QueryOut{};
            r.q.distance = CUDART_INF;
            r.q.moving_sphere = r.q.other_sphere = r.q.other_slot = -1;
            r.q.status = ST_OK;
        }
        if (slot >= 0) {
            r.dir[0] = sm.dir[0];
            r.dir[1] = sm.dir[1];
            r.dir[2] = sm.dir[2];
            r.full = sm.full;
            r.dt_indiv = A(b, AGG_TIME_STEP, slot);
            r.rmax = A(b, AGG_RMAX, slot);
            r.pos[0] = A(b, AGG_X, slot);
            r.pos[1] = A(b, AGG_Y, slot);
            r.pos[2] = A(b, AGG_Z, slot);
        }
        *out = r;
    }
    __syncthreads();
}

// The leader commits the round's steps in order (all threads of the leader
// CTA); returns the number committed. The stream is left after the
// committed steps' draws.
template <class RS>
__device__ inline int spec_commit(const BoxRun &R, RS &sm, SpecShared &sh, int nj) {
    const DevBox &b = R.box;
    RunState &st = *R.st;
    int committed = 0;
    for (int i = 0; i < nj; ++i) {
        if (threadIdx.x == 0) {
            const SpecResult &r = sh.res[i];
            int ok = 1;
            if (st.finished || st.status != ST_OK) {
                ok = 0;
            } else if (run_finished(R, st, b.sc->n_alive)) {
                st.finished = 1;
                ok = 0;
            } else if (r.slot < 0) {
                if (i == 0) st.status = ST_UNKNOWN;  // the tree lost a live slot: stop this box
                ok = 0;
            } else if (i > 0 && r.q.status != ST_OK) {
                ok = 0;  // a helper's answer failed (its scratch): the leader asks again next round
            } else {
                for (int j = 0; j < i && ok; ++j)
                    if (spec_conflict(sh.res[j], sh.move[j], r, b.L)) ok = 0;
            }
            sm.stop = 0;
            if (ok) {
                sm.slot = r.slot;
                sm.dir[0] = r.dir[0];
                sm.dir[1] = r.dir[1];
                sm.dir[2] = r.dir[2];
                sm.dt = sh.dt;
                sm.full = r.full;
                sm.dt_indiv = r.dt_indiv;
                if (R.lim.with_collisions) {
                    apply_query(st, sm, r.q);
                } else {
                    sm.contact = 0;
                    sm.move = sm.full;
                }
                sh.move[i] = sm.move;
            }
            sh.ok = ok;
        }
        __syncthreads();
        if (!sh.ok || sm.stop) break;
        long long t_phase = clock64();
        if (!step_commit(R, sm, t_phase)) break;
        ++committed;
        if (sm.merged) {
            if (threadIdx.x == 0) sh.tree_gen += 1;  // the helpers' copies of the tree are stale
            break;
        }
    }
    if (threadIdx.x == 0) {
        st.rng = sh.rng0;
        for (int k = 0; k < 3 * committed; ++k) st.rng.next_int();
    }
    __syncthreads();
    return committed;
}

}  // namespace mcacg
