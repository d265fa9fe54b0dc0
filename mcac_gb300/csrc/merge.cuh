// Merge of two aggregates on the device: relabel, pool segment, and the
// geometry part of Aggregate::update (aggregats/aggregat.cpp:247-288,
// 321-483, 486-544, 719-764).
//
// The reference accumulates every aggregate sum sequentially in sphere-list
// order. To stay bit-identical the per-sphere terms are formed in parallel
// (one rounding each, as in the reference) and each sum is then accumulated
// in list order by one thread; the seven sums run on seven lanes of the
// first warp, in step (any block size of 32 threads or more works). The
// O(n^2) intra-aggregate contact search is screened in FP32 and refined in
// FP64; its pairs are put back in (i, j) order before they are summed.
#pragma once
#include "box.cuh"

namespace mcacg {

constexpr int kSumSeries = 8;

// PairTile: spheres staged per pass of the intra-aggregate pair search.
template <int PairTile>
struct MergeSmemT {
    static constexpr int kPairTile = PairTile;
    double refpos[3];
    double diffpos[3];
    double r_cm[3];
    double sums[kSumSeries];
    double vol_raw, overlap, coord;
    float ext, rmax_f;  // bound of |relative position| + r, largest radius (FP32)
    double rmax_warp[32];
    float tile_f[kPairTile * 4];
    int warp_tmp[32];
    float warp_f[32];
    int keep, removed, mysph, othsph;
    int n_keep, n_rem, off_keep, off_rem, new_off, n;
    int n_pairs;
    int status;
    int merged;
    float margin;
};
using MergeSmem = MergeSmemT<1024>;
using MergeSmemSmall = MergeSmemT<256>;

// exclusive scan of a global int array in place (block-wide, chunked);
// returns the total.
__device__ inline int block_scan_global(int *data, int n, int *warp_tmp) {
    const int NT = blockDim.x;
    int carry = 0;
    for (int c0 = 0; c0 < n; c0 += NT) {
        int idx = c0 + threadIdx.x;
        int v = (idx < n) ? data[idx] : 0;
        int total;
        // generic warp scan for any block size multiple of 32
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = NT >> 5;
        int x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tmp[wid] = x;
        __syncthreads();
        if (wid == 0) {
            int wv = (lane < nw) ? warp_tmp[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, wv, o);
                if (lane >= o) wv += y;
            }
            if (lane < nw) warp_tmp[lane] = wv;
        }
        __syncthreads();
        int base = (wid > 0) ? warp_tmp[wid - 1] : 0;
        total = warp_tmp[nw - 1];
        if (idx < n) data[idx] = carry + base + x - v;
        carry += total;
        __syncthreads();
    }
    return carry;
}

// Move every live segment to the front of the other pool buffer, in slot
// order. Uses counters[] and row_cnt[] as scratch.
__device__ inline void block_compact_pool(const DevBox &b, int *warp_tmp) {
    DevScalars *sc = b.sc;
    const int from = sc->pool_sel, to = 1 - from;
    // prefix of member counts over slots, staged in row_cnt (size >= nslots+1)
    int *pref = b.row_cnt;
    for (int a = threadIdx.x; a < b.nslots; a += blockDim.x) pref[a] = b.agg_n[a];
    __syncthreads();
    int total = block_scan_global(pref, b.nslots, warp_tmp);
    for (int a = threadIdx.x; a < b.nslots; a += blockDim.x) {
        int n = b.agg_n[a];
        if (n == 0) continue;
        int src = b.agg_off[a], dst = pref[a];
        for (int k = 0; k < n; ++k) {
            b.pool_id[to][dst + k] = b.pool_id[from][src + k];
            b.pool_pos[to][dst + k] = b.pool_pos[from][src + k];
        }
    }
    __syncthreads();
    for (int a = threadIdx.x; a < b.nslots; a += blockDim.x)
        if (b.agg_n[a] > 0) b.agg_off[a] = pref[a];
    __syncthreads();
    if (threadIdx.x == 0) {
        sc->pool_sel = to;
        sc->pool_top = total;
    }
    __syncthreads();
}

// Sequential (list-order) sum of one work series, as the reference's loops.
__device__ __forceinline__ double ordered_sum(const double *v, int n) {
    double acc = 0.0;
    for (int i = 0; i < n; ++i) acc = acc + v[i];
    return acc;
}

// Every pair i < j of the n spheres mem[0..n) of one aggregate whose FP32
// relative positions pass the screen |rel_i - rel_j| <= (r_i + r_j) 1.0001 +
// margin + extra goes to test(i, j) (any thread, any order); the margin is
// 1e-5 of the aggregate's extent, far above the FP32 rounding, so every pair
// within (r_i + r_j)(1 + 1e-4) + extra in FP64 is handed over. All threads
// call it; b.work holds the staging (52 n + 4 bytes at most).
template <class SM, class F>
__device__ inline void block_pair_scan(const DevBox &b, const int *mem, int n, SM &sm, float extra, F &&test) {
    constexpr int kPairTile = SM::kPairTile;
    const int tid = threadIdx.x, NT = blockDim.x;
    // stage relative positions (FP32) and the extent for the screening margin
    float4 *relf = reinterpret_cast<float4 *>(b.work);  // reuse: n float4 fit in work[0..n/2)
    float ext = 0.f, rmx = 0.f;
    for (int k = tid; k < n; k += NT) {
        int s = mem[k];
        float4 v = make_float4(float(S(b, SPH_RX, s)), float(S(b, SPH_RY, s)), float(S(b, SPH_RZ, s)),
                               float(S(b, SPH_R, s)));
        relf[k] = v;
        ext = fmaxf(ext, fabsf(v.x) + fabsf(v.y) + fabsf(v.z) + v.w);
        rmx = fmaxf(rmx, v.w);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ext = fmaxf(ext, __shfl_xor_sync(0xffffffffu, ext, o));
        rmx = fmaxf(rmx, __shfl_xor_sync(0xffffffffu, rmx, o));
    }
    if ((tid & 31) == 0) {
        sm.warp_f[tid >> 5] = ext;
        sm.warp_tmp[tid >> 5] = __float_as_int(rmx);  // non-negative: int order is float order
    }
    __syncthreads();
    if (tid == 0) {
        float m = 0.f, r = 0.f;
        for (int k = 0; k < NT / 32; ++k) {
            m = fmaxf(m, sm.warp_f[k]);
            r = fmaxf(r, __int_as_float(sm.warp_tmp[k]));
        }
        sm.margin = 1.0e-5f * m;  // FP32 error of |rel_i - rel_j| is ~1e-7 of the extent
        sm.ext = m;
        sm.rmax_f = r;
    }
    __syncthreads();
    const float pm_margin = sm.margin + extra;
    // the FP32 screen of one pair i < j; the survivors go to 'test'
    auto pair_test = [&](int i, int j, const float4 &pi_, const float4 &pj_) {
        const float dx = pi_.x - pj_.x, dy = pi_.y - pj_.y, dz = pi_.z - pj_.z;
        const float reach = (pi_.w + pj_.w) * 1.0001f + pm_margin;
        if (__fmaf_rn(dx, dx, __fmaf_rn(dy, dy, dz * dz)) > reach * reach) return;
        test(i, j);
    };
    if (n >= b.grid_pairs_min) {
        // Large aggregates: a hashed cell grid over the relative positions
        // (cells wider than any pair's screening reach, 2 r_max 1.0001 +
        // margin, by one more margin -- 100 times the FP32 rounding of the
        // cell coordinates -- and 0.1%), so that every pair
        // that can pass the screen sits in neighbouring cells; each sphere
        // meets the spheres of its 27 cells with a larger index. The same
        // pairs as the all-pairs loop, found in O(n) (a merge of two
        // 8000-sphere aggregates needs 10^8 pair tests otherwise).
        // Scratch after the n float4 of relf: cell coordinates (int4, n),
        // bucket counts/starts (2^k + 1 >= 2n + 1), sorted sphere indices (n).
        // With nb < 4n that is 16n + 16n + 4(nb + 1) + 4n <= 52n + 4 bytes,
        // inside the work area of 8 doubles (64 B) per sphere of the box
        // (n <= ns); a larger carve needs a larger work area.
        int4 *cellc = reinterpret_cast<int4 *>(relf + n);
        int nb = 1;
        while (nb < 2 * n) nb <<= 1;
        int *bstart = reinterpret_cast<int *>(cellc + n);
        int *sorted = bstart + nb + 1;
        const float h = ((2.f * sm.rmax_f) * 1.0001f + 2.f * pm_margin) * 1.001f;
        const float inv_h = 1.f / h, e0 = sm.ext;
        auto bucket_of = [&](int cx, int cy, int cz) {
            const unsigned hsh = (unsigned(cx) * 73856093u) ^ (unsigned(cy) * 19349663u) ^ (unsigned(cz) * 83492791u);
            return int(hsh & unsigned(nb - 1));
        };
        for (int k = tid; k <= nb; k += NT) bstart[k] = 0;
        __syncthreads();
        for (int k = tid; k < n; k += NT) {
            const float4 v = relf[k];
            const int cx = int(floorf((v.x + e0) * inv_h)), cy = int(floorf((v.y + e0) * inv_h)),
                      cz = int(floorf((v.z + e0) * inv_h));
            const int bk = bucket_of(cx, cy, cz);
            cellc[k] = make_int4(cx, cy, cz, bk);
            atomicAdd(&bstart[bk], 1);
        }
        __syncthreads();
        block_scan_global(bstart, nb + 1, sm.warp_tmp);  // bstart[nb] = n
        __syncthreads();
        // scatter (bstart[bk] advances to the bucket's end; starts are then
        // bstart[bk - 1], or 0)
        for (int k = tid; k < n; k += NT) sorted[atomicAdd(&bstart[cellc[k].w], 1)] = k;
        __syncthreads();
        for (int i = tid; i < n; i += NT) {
            const float4 pi_ = relf[i];
            const int4 ci = cellc[i];
            for (int ox = -1; ox <= 1; ++ox)
                for (int oy = -1; oy <= 1; ++oy)
                    for (int oz = -1; oz <= 1; ++oz) {
                        const int cx = ci.x + ox, cy = ci.y + oy, cz = ci.z + oz;
                        const int bk = bucket_of(cx, cy, cz);
                        const int beg = bk == 0 ? 0 : bstart[bk - 1], end = bstart[bk];
                        for (int t = beg; t < end; ++t) {
                            const int j = sorted[t];
                            if (j <= i) continue;
                            const int4 cj = cellc[j];
                            if (cj.x != cx || cj.y != cy || cj.z != cz) continue;  // another cell in the bucket
                            pair_test(i, j, pi_, relf[j]);
                        }
                    }
        }
        __syncthreads();
    } else {
    for (int j0 = 0; j0 < n; j0 += kPairTile) {
        const int nt = min(kPairTile, n - j0);
        for (int k = tid; k < nt; k += NT) {
            float4 v = relf[j0 + k];
            sm.tile_f[4 * k + 0] = v.x;
            sm.tile_f[4 * k + 1] = v.y;
            sm.tile_f[4 * k + 2] = v.z;
            sm.tile_f[4 * k + 3] = v.w;
        }
        __syncthreads();
        for (int i = tid; i < min(n, j0 + nt); i += NT) {
            const float4 pi_ = relf[i];
            int jstart = max(i + 1, j0) - j0;
            for (int jj = jstart; jj < nt; ++jj) {
                const float4 pj_ = make_float4(sm.tile_f[4 * jj + 0], sm.tile_f[4 * jj + 1], sm.tile_f[4 * jj + 2],
                                               sm.tile_f[4 * jj + 3]);
                pair_test(i, j0 + jj, pi_, pj_);
            }
        }
        __syncthreads();
    }
    }  // all pairs: both branches end on a barrier
}

// AggregatList::merge + Aggregate::merge + Aggregate::update (geometry).
// ms / os: moving / other sphere; mslot / oslot: their aggregates at query
// time. The physics fields (f_agg, d_m, time_step, lpm, dg_over_dp), the
// proper time and the charge are left to the caller.
template <class SM>
__device__ inline void block_merge(const DevBox &b, int ms, int os, int mslot, int oslot, SM &sm, MergeOut *out) {
    const int tid = threadIdx.x, NT = blockDim.x;
    DevScalars *sc = b.sc;
    if (tid == 0) {
        sm.status = ST_OK;
        sm.merged = 0;
        sm.n_pairs = 0;
        Vec3 pm = sph_pos(b, ms), po = sph_pos(b, os);
        if (!spheres_in_contact(pm, S(b, SPH_R, ms), po, S(b, SPH_R, os), b.L)) {
            sm.merged = 0;
        } else {
            int la = b.sph_slot[ms], lb = b.sph_slot[os];
            int keep = min(la, lb), removed = max(la, lb);
            int my = -1, oth = -1;
            if (mslot == keep) {
                my = ms;
                oth = os;
            } else if (oslot == keep) {
                my = os;
                oth = ms;
            }
            if (my < 0 || keep == removed) {
                sm.status = ST_MERGE;  // "ListAggregate want to merge but the aggregate refuses"
            } else {
                sm.merged = 1;
                sm.keep = keep;
                sm.removed = removed;
                sm.mysph = my;
                sm.othsph = oth;
                sm.n_keep = b.agg_n[keep];
                sm.n_rem = b.agg_n[removed];
                sm.n = sm.n_keep + sm.n_rem;
                const int *pid = b.pool_id[sc->pool_sel];
                int s0 = pid[b.agg_off[keep]];
                sm.refpos[0] = S(b, SPH_X, s0);
                sm.refpos[1] = S(b, SPH_Y, s0);
                sm.refpos[2] = S(b, SPH_Z, s0);
                Vec3 pmy = sph_pos(b, my), poth = sph_pos(b, oth);
                double dcx = periodic_distance(poth.x - pmy.x, b.L);
                double dcy = periodic_distance(poth.y - pmy.y, b.L);
                double dcz = periodic_distance(poth.z - pmy.z, b.L);
                sm.diffpos[0] = S(b, SPH_RX, my) + dcx - S(b, SPH_RX, oth);
                sm.diffpos[1] = S(b, SPH_RY, my) + dcy - S(b, SPH_RY, oth);
                sm.diffpos[2] = S(b, SPH_RZ, my) + dcz - S(b, SPH_RZ, oth);
            }
        }
    }
    __syncthreads();
    if (!sm.merged || sm.status != ST_OK) {
        if (tid == 0) {
            out->merged = 0;
            out->status = sm.status;
        }
        __syncthreads();
        return;
    }
    const int keep = sm.keep, removed = sm.removed, n = sm.n, n_keep = sm.n_keep, n_rem = sm.n_rem;
    // room for the merged segment
    if (sc->pool_top + n > b.pool_cap) block_compact_pool(b, sm.warp_tmp);
    if (tid == 0) {
        sm.off_keep = b.agg_off[keep];
        sm.off_rem = b.agg_off[removed];
        sm.new_off = sc->pool_top;
    }
    __syncthreads();
    int *pool_id = b.pool_id[sc->pool_sel];
    float4 *pool_pos = b.pool_pos[sc->pool_sel];
    const int off_keep = sm.off_keep, off_rem = sm.off_rem, new_off = sm.new_off;
    // relabel and shift the removed aggregate's spheres; build keep ++ removed
    for (int k = tid; k < n; k += NT) {
        if (k < n_keep) {
            pool_id[new_off + k] = pool_id[off_keep + k];
            pool_pos[new_off + k] = pool_pos[off_keep + k];
        } else {
            int s = pool_id[off_rem + (k - n_keep)];
            b.sph_slot[s] = keep;
            double rx = S(b, SPH_RX, s) + sm.diffpos[0];
            double ry = S(b, SPH_RY, s) + sm.diffpos[1];
            double rz = S(b, SPH_RZ, s) + sm.diffpos[2];
            S(b, SPH_RX, s) = rx;
            S(b, SPH_RY, s) = ry;
            S(b, SPH_RZ, s) = rz;
            double x = rx + sm.refpos[0], y = ry + sm.refpos[1], z = rz + sm.refpos[2];
            S(b, SPH_X, s) = x;
            S(b, SPH_Y, s) = y;
            S(b, SPH_Z, s) = z;
            pool_id[new_off + k] = s;
            pool_pos[new_off + k] = make_float4(float(x), float(y), float(z), float(S(b, SPH_R, s)));
        }
    }
    __syncthreads();
    if (tid == 0) {
        b.agg_off[keep] = new_off;
        b.agg_n[keep] = n;
        b.agg_n[removed] = 0;
        sc->pool_top = new_off + n;
        sc->n_alive -= 1;
    }
    __syncthreads();
    const int *mem = pool_id + new_off;

    // ---- update_distances_and_overlapping: contact pairs i < j
    for (int k = tid; k <= n; k += NT) b.row_cnt[k] = 0;
    if (tid == 0) b.counters[0] = 0;
    block_pair_scan(b, mem, n, sm, 0.f, [&](int i, int j) {
        const int si = mem[i], sj = mem[j];
        double ex = S(b, SPH_RX, si) - S(b, SPH_RX, sj);
        double ey = S(b, SPH_RY, si) - S(b, SPH_RY, sj);
        double ez = S(b, SPH_RZ, si) - S(b, SPH_RZ, sj);
        double dist = sqrt(ex * ex + ey * ey + ez * ez);
        double rsum = S(b, SPH_R, si) + S(b, SPH_R, sj);
        if (dist <= (1. + kCoordinationEpsilon) * rsum) {
            int p = atomicAdd(&b.counters[0], 1);
            if (p < b.pair_cap) {
                b.pair_tmp_i[p] = i;
                b.pair_tmp_j[p] = j;
                b.pair_tmp_d[p] = dist;
                atomicAdd(&b.row_cnt[i], 1);
            }
        }
    });
    const int P = b.counters[0];
    if (P > b.pair_cap) {
        if (tid == 0) {
            sc->status = ST_CAPACITY;
            out->merged = 1;
            out->status = ST_CAPACITY;
        }
        __syncthreads();
        return;
    }
    // counting sort of the pairs by i, then by j within a row
    block_scan_global(b.row_cnt, n + 1, sm.warp_tmp);
    for (int p = tid; p < P; p += NT) {
        int i = b.pair_tmp_i[p];
        int dst = atomicAdd(&b.row_cnt[i], 1);
        b.pair_i[dst] = i;
        b.pair_j[dst] = b.pair_tmp_j[p];
        b.pair_d[dst] = b.pair_tmp_d[p];
    }
    __syncthreads();
    // row_cnt[i] now holds the end of row i; row i starts at row_cnt[i-1]
    for (int i = tid; i < n; i += NT) {
        int beg = (i == 0) ? 0 : b.row_cnt[i - 1];
        int end = b.row_cnt[i];
        for (int x = beg + 1; x < end; ++x) {
            int jv = b.pair_j[x];
            double dv = b.pair_d[x];
            int y = x;
            while (y > beg && b.pair_j[y - 1] > jv) {
                b.pair_j[y] = b.pair_j[y - 1];
                b.pair_d[y] = b.pair_d[y - 1];
                --y;
            }
            b.pair_j[y] = jv;
            b.pair_d[y] = dv;
        }
    }
    __syncthreads();

    // ---- per-sphere terms (one rounding each, as in the reference)
    // work[0] volume, [1] surface, [2..4] rel * volume, [5] volume * r^2,
    // [6] r, [7] volume * dcenter^2 (after the centre of mass is known)
    double *wv = b.work;
    const size_t W = size_t(b.ns);
    for (int k = tid; k < n; k += NT) {
        int s = mem[k];
        wv[0 * W + k] = S(b, SPH_VOLUME, s);
        wv[1 * W + k] = S(b, SPH_SURFACE, s);
        wv[6 * W + k] = S(b, SPH_R, s);
    }
    __syncthreads();
    if (b.volsurf == VS_CAPS && tid == 0) {
        // compute_volume_surface, "caps" (aggregat.cpp:358-388): each
        // sphere's contacts with later ones, in (i, j) order, take their caps
        // off both spheres; a sphere is clamped at 0 once its own contacts
        // are done. The reference visits a sphere's contacts in its hash
        // map's order; here they go by index.
        for (int p = 0; p < P; ++p) {
            const int i = b.pair_i[p], j = b.pair_j[p];
            const int si = mem[i], sj = mem[j];
            const SphereCaps k = sphere_caps(S(b, SPH_R, si), S(b, SPH_VOLUME, si), S(b, SPH_SURFACE, si),
                                             S(b, SPH_R, sj), S(b, SPH_VOLUME, sj), S(b, SPH_SURFACE, sj), b.pair_d[p]);
            wv[0 * W + i] = wv[0 * W + i] - k.v1;
            wv[1 * W + i] = wv[1 * W + i] - k.s1;
            wv[0 * W + j] = wv[0 * W + j] - k.v2;
            wv[1 * W + j] = wv[1 * W + j] - k.s2;
        }
        // the clamps: a sphere's value is final once its row is done, and
        // later rows never touch it
        for (int i = 0; i < n; ++i) {
            wv[0 * W + i] = dmax(wv[0 * W + i], 0.0);
            wv[1 * W + i] = dmax(wv[1 * W + i], 0.0);
        }
    }
    __syncthreads();
    for (int k = tid; k < n; k += NT) {
        const int s = mem[k];
        const double vol = wv[0 * W + k];
        const double r = wv[6 * W + k];
        wv[2 * W + k] = S(b, SPH_RX, s) * vol;
        wv[3 * W + k] = S(b, SPH_RY, s) * vol;
        wv[4 * W + k] = S(b, SPH_RZ, s) * vol;
        wv[5 * W + k] = vol * (r * r);
        b.sph_volw[s] = vol;
    }
    __syncthreads();
    // overlapping's terms (rsum - d) / rsum of the (i, j)-ordered pairs, formed
    // in parallel (each one rounding as in the reference); summed in pair
    // order below. The pair sort's scratch is free by now.
    double *ov_terms = b.pair_tmp_d;
    for (int p = tid; p < P; p += NT) {
        const double rsum = S(b, SPH_R, mem[b.pair_i[p]]) + S(b, SPH_R, mem[b.pair_j[p]]);
        ov_terms[p] = (rsum - b.pair_d[p]) / rsum;
    }
    __syncthreads();
    {
        // seven independent ordered sums, one per lane of the first warp
        if (tid < 7) sm.sums[tid] = ordered_sum(wv + size_t(tid) * W, n);
        // the overlap sum, sequential over the pairs, on the second warp
        // when there is one (beside the seven)
        if (tid == (NT > 32 ? 32 : 0)) {
            double ov = 0.0;
            for (int p = 0; p < P; ++p) ov += 2.0 * ov_terms[p];
            sm.sums[7] = ov;
            sm.n_pairs = P;
        }
    }
    __syncthreads();
    if (tid == 0) {
        // the plain sum of the sphere volumes (update_partial's vol_pp)
        sm.vol_raw = sm.sums[0];
        if (b.volsurf == VS_CAPS) {
            double v = 0.0;
            for (int k = 0; k < n; ++k) v = v + S(b, SPH_VOLUME, mem[k]);
            sm.vol_raw = v;
        }
        sm.overlap = 0.0;
        sm.coord = 0.0;
        if (P > 0) {
            sm.overlap = sm.sums[7] / static_cast<double>(2 * P);
            sm.coord = static_cast<double>(2 * P) / static_cast<double>(n);
        }
        if (b.volsurf == VS_ALPHAS) {
            // compute_volume_surface, "alphas" (aggregat.cpp:391-426): the
            // sums over every contact seen from both spheres (here each pair
            // twice in a row, in (i, j) order), then the corrections
            AlphaSums a{0., 0., 0., 0., 0., 0.};
            for (int p = 0; p < P; ++p) {
                const double ri = S(b, SPH_R, mem[b.pair_i[p]]), rj = S(b, SPH_R, mem[b.pair_j[p]]);
                alpha_add(a, ri, rj, b.pair_d[p]);
                alpha_add(a, rj, ri, b.pair_d[p]);
            }
            alpha_finish(a, n, 2 * P, &sm.sums[0], &sm.sums[1], &sm.overlap, &sm.coord);
        }
    }
    __syncthreads();
    const double V = sm.sums[0], Sf = sm.sums[1];
    if (tid == 0) {
        if (V <= 0 || Sf <= 0) sm.status = ST_VOL_SURF;
        double cx = sm.sums[2] / V, cy = sm.sums[3] / V, cz = sm.sums[4] / V;
        sm.r_cm[0] = cx;
        sm.r_cm[1] = cy;
        sm.r_cm[2] = cz;
    }
    __syncthreads();
    if (sm.status != ST_OK) {
        if (tid == 0) {
            sc->status = sm.status;
            out->merged = 1;
            out->status = sm.status;
        }
        __syncthreads();
        return;
    }
    // distances to the centre of mass, r_max, Rg terms
    double rmax_local = 0.0;
    for (int k = tid; k < n; k += NT) {
        int s = mem[k];
        double dx = S(b, SPH_RX, s) - sm.r_cm[0];
        double dy = S(b, SPH_RY, s) - sm.r_cm[1];
        double dz = S(b, SPH_RZ, s) - sm.r_cm[2];
        double dcen = sqrt(dx * dx + dy * dy + dz * dz);
        wv[7 * W + k] = wv[0 * W + k] * (dcen * dcen);
        rmax_local = dmax(rmax_local, S(b, SPH_R, s) + dcen);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rmax_local = dmax(rmax_local, __shfl_xor_sync(0xffffffffu, rmax_local, o));
    if ((tid & 31) == 0) sm.rmax_warp[tid >> 5] = rmax_local;
    __syncthreads();
    // the removed slot leaves the grids on the second warp, beside the sums
    // below (the grid lists are unordered: the order of their updates sets
    // no result); with one warp, thread 0 does it after them
    const int grid_thread = NT > 32 ? 32 : 0;
    if (grid_thread != 0 && tid == grid_thread) {
        cell_remove(b, cell_index(b, b.agg_cell[removed]), removed);
        if (b.fine_div > 0) fine_unlink(b, removed);
    }
    double x = 0.0, y = 0.0, z = 0.0, rmax = 0.0, vol_pp = 0.0;
    if (tid == 0) {
        for (int k = 0; k < NT / 32; ++k) rmax = dmax(rmax, sm.rmax_warp[k]);
        double arg = ordered_sum(wv + 7 * W, n);
        double brg = sm.sums[5];
        double rg = sqrt(fabs((arg + (3. / 5.) * brg) / V));
        double dp = 2 * sm.sums[6] / static_cast<double>(n);
        vol_pp = sm.vol_raw / static_cast<double>(n);
        const double overlapping = sm.overlap, coordination = sm.coord;
        const int s0 = mem[0];
        x = periodic_position(S(b, SPH_X, s0) + sm.r_cm[0], b.L);
        y = periodic_position(S(b, SPH_Y, s0) + sm.r_cm[1], b.L);
        z = periodic_position(S(b, SPH_Z, s0) + sm.r_cm[2], b.L);
        A(b, AGG_RG, keep) = rg;
        A(b, AGG_RMAX, keep) = rmax;
        A(b, AGG_VOLUME, keep) = V;
        A(b, AGG_SURFACE, keep) = Sf;
        A(b, AGG_X, keep) = x;
        A(b, AGG_Y, keep) = y;
        A(b, AGG_Z, keep) = z;
        A(b, AGG_RX, keep) = sm.r_cm[0];
        A(b, AGG_RY, keep) = sm.r_cm[1];
        A(b, AGG_RZ, keep) = sm.r_cm[2];
        A(b, AGG_DP, keep) = dp;
        A(b, AGG_OVERLAPPING, keep) = overlapping;
        A(b, AGG_COORDINATION_NUMBER, keep) = coordination;
        b.agg_f4[keep] = make_float4(float(x), float(y), float(z), float(rmax));
    }
    __syncthreads();
    if (tid == 0) {
        if (grid_thread == 0) {
            cell_remove(b, cell_index(b, b.agg_cell[removed]), removed);
            if (b.fine_div > 0) fine_unlink(b, removed);
        }
        regrid(b, keep, Vec3{x, y, z});
        if (rmax > sc->maxradius) sc->maxradius = rmax;
        out->merged = 1;
        out->status = ST_OK;
        out->keep = keep;
        out->removed = removed;
        out->n = n;
        out->n_pairs = P;
        for (int f = 0; f < AGG_NFIELDS; ++f) out->fields[f] = A(b, f, keep);
        out->vol_pp = vol_pp;
        out->maxradius = sc->maxradius;
    }
    __syncthreads();
}

// The geometry of Aggregate::update / update_partial (aggregat.cpp:247-288,
// 321-483) of one slot by one thread, sums in list order, without the
// physics fields (friction, mobility diameter, time step, lpm, Rg/dp).
// Returns r_max, and the mean sphere volume of update_partial in *vol_pp_out.
// 'full' is update(): compute_volume_surface refreshes the aggregate's
// volume and surface and each sphere's entry of the per-sphere volumes
// (sph_volw); update_partial weighs the centre of mass and Rg with those
// entries as last set, as the reference does. For "none" the overlap and
// coordination fields, which need every pair of the aggregate and do not act
// on the dynamics, are left to the merge and to the read-back unless
// 'overlap' asks for them; "caps" and "alphas" need the pairs for the volume
// and set them here.
__device__ inline double thread_update_geometry(const DevBox &b, int a, bool full, double *vol_pp_out,
                                                bool overlap = false) {
    const int n = b.agg_n[a];
    const int *mem = b.pool_id[b.sc->pool_sel] + b.agg_off[a];
    double volume = A(b, AGG_VOLUME, a);
    if (full && b.volsurf == VS_NONE && !overlap) {
        double v = 0.0, sfc = 0.0;
        for (int i = 0; i < n; ++i) {
            const double vi = S(b, SPH_VOLUME, mem[i]);
            v = v + vi;
            sfc = sfc + S(b, SPH_SURFACE, mem[i]);
            b.sph_volw[mem[i]] = vi;
        }
        volume = v;
        A(b, AGG_VOLUME, a) = v;
        A(b, AGG_SURFACE, a) = sfc;
    } else if (full) {
        // update_distances_and_overlapping, then compute_volume_surface
        // ("caps": sph_volw and the work area hold the per-sphere volumes and
        // surfaces as the caps come off; "alphas": sums over the pairs, each
        // pair twice in a row, in (i, j) order)
        double *surf_w = b.work;  // by sphere index; free outside a merge
        for (int i = 0; i < n; ++i) {
            b.sph_volw[mem[i]] = S(b, SPH_VOLUME, mem[i]);
            surf_w[mem[i]] = S(b, SPH_SURFACE, mem[i]);
        }
        double ov = 0.0;
        int inter = 0;
        AlphaSums al{0., 0., 0., 0., 0., 0.};
        for (int i = 0; i < n; ++i) {
            const int si = mem[i];
            const double ri = S(b, SPH_R, si);
            for (int j = i + 1; j < n; ++j) {
                const int sj = mem[j];
                const double ex = S(b, SPH_RX, si) - S(b, SPH_RX, sj);
                const double ey = S(b, SPH_RY, si) - S(b, SPH_RY, sj);
                const double ez = S(b, SPH_RZ, si) - S(b, SPH_RZ, sj);
                const double dist = sqrt(ex * ex + ey * ey + ez * ez);
                const double rj = S(b, SPH_R, sj);
                const double rsum = ri + rj;
                if (!(dist <= (1. + kCoordinationEpsilon) * rsum)) continue;
                ov += 2.0 * ((rsum - dist) / rsum);
                inter += 2;
                if (b.volsurf == VS_CAPS) {
                    const SphereCaps k = sphere_caps(ri, S(b, SPH_VOLUME, si), S(b, SPH_SURFACE, si), rj,
                                                     S(b, SPH_VOLUME, sj), S(b, SPH_SURFACE, sj), dist);
                    b.sph_volw[si] = b.sph_volw[si] - k.v1;
                    surf_w[si] = surf_w[si] - k.s1;
                    b.sph_volw[sj] = b.sph_volw[sj] - k.v2;
                    surf_w[sj] = surf_w[sj] - k.s2;
                } else if (b.volsurf == VS_ALPHAS) {
                    alpha_add(al, ri, rj, dist);
                    alpha_add(al, rj, ri, dist);
                }
            }
            if (b.volsurf == VS_CAPS) {
                b.sph_volw[si] = dmax(b.sph_volw[si], 0.0);
                surf_w[si] = dmax(surf_w[si], 0.0);
            }
        }
        double overlapping = 0.0, coordination = 0.0;
        if (inter > 0) {
            overlapping = ov / static_cast<double>(inter);
            coordination = static_cast<double>(inter) / static_cast<double>(n);
        }
        double v = 0.0, sfc = 0.0;
        for (int i = 0; i < n; ++i) {
            v = v + b.sph_volw[mem[i]];
            sfc = sfc + surf_w[mem[i]];
        }
        if (b.volsurf == VS_ALPHAS) alpha_finish(al, n, inter, &v, &sfc, &overlapping, &coordination);
        volume = v;
        A(b, AGG_VOLUME, a) = v;
        A(b, AGG_SURFACE, a) = sfc;
        A(b, AGG_OVERLAPPING, a) = overlapping;
        A(b, AGG_COORDINATION_NUMBER, a) = coordination;
    }
    // compute_mass_center (aggregat.cpp:431-452)
    double rx = 0., ry = 0., rz = 0.;
    for (int i = 0; i < n; ++i) {
        const int s = mem[i];
        const double vol = b.sph_volw[s];
        rx += S(b, SPH_RX, s) * vol;
        ry += S(b, SPH_RY, s) * vol;
        rz += S(b, SPH_RZ, s) * vol;
    }
    rx /= volume;
    ry /= volume;
    rz /= volume;
    // compute_max_radius, compute_giration_radius (aggregat.cpp:453-483),
    // and update_partial's mean radius and mean sphere volume
    double rmax = 0.0, arg = 0., brg = 0., dp = 0., vol_pp = 0.;
    for (int i = 0; i < n; ++i) {
        const int s = mem[i];
        const double dx = S(b, SPH_RX, s) - rx, dy = S(b, SPH_RY, s) - ry, dz = S(b, SPH_RZ, s) - rz;
        const double dc = sqrt(dx * dx + dy * dy + dz * dz);
        const double rs = S(b, SPH_R, s), volw = b.sph_volw[s];
        rmax = dmax(rmax, rs + dc);
        arg = arg + volw * (dc * dc);
        brg = brg + volw * (rs * rs);
        vol_pp += S(b, SPH_VOLUME, s);
        dp += rs;
    }
    const double rg = sqrt(fabs((arg + (3. / 5.) * brg) / volume));
    dp = 2 * dp / double(n);
    vol_pp = vol_pp / double(n);
    // the aggregate's position (aggregat.cpp:431-452, as in the merge)
    const int s0 = mem[0];
    const double x = periodic_position(S(b, SPH_X, s0) + rx, b.L);
    const double y = periodic_position(S(b, SPH_Y, s0) + ry, b.L);
    const double z = periodic_position(S(b, SPH_Z, s0) + rz, b.L);
    A(b, AGG_RX, a) = rx;
    A(b, AGG_RY, a) = ry;
    A(b, AGG_RZ, a) = rz;
    A(b, AGG_X, a) = x;
    A(b, AGG_Y, a) = y;
    A(b, AGG_Z, a) = z;
    A(b, AGG_RMAX, a) = rmax;
    A(b, AGG_RG, a) = rg;
    A(b, AGG_DP, a) = dp;
    b.agg_f4[a] = make_float4(float(x), float(y), float(z), float(rmax));
    *vol_pp_out = vol_pp;
    return rmax;
}

}  // namespace mcacg
