// Host-side handle of one box resident on the GPU (allocation, upload,
// download, launches of the single-box kernels).
#pragma once
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "../../include/mcacg.h"

namespace mcacg {

struct QueryOut;
struct MergeOut;

// Member lists of all aggregate slots in one array (list a is
// ids[off[a] .. off[a+1]), in list order); built slot by slot in order.
struct MemberLists {
    std::vector<int> off{0};
    std::vector<int> ids;
    struct View {
        const int *p;
        int n;
        int size() const { return n; }
        const int &operator[](size_t k) const { return p[k]; }
        const int *begin() const { return p; }
        const int *end() const { return p + n; }
    };
    View operator[](size_t a) const { return View{ids.data() + off[a], off[a + 1] - off[a]}; }
    size_t count() const { return off.size() - 1; }
    void clear() {
        off.assign(1, 0);
        ids.clear();
    }
    void reserve(size_t lists, size_t items) {
        off.reserve(lists + 1);
        ids.reserve(items);
    }
    void push_list(const int *b, int n) {
        ids.insert(ids.end(), b, b + n);
        off.push_back(int(ids.size()));
    }
    void push_single(int x) {
        ids.push_back(x);
        off.push_back(int(ids.size()));
    }
};

// Complete box state in host memory, by stable aggregate slot.
struct HostState {
    int n_div = 10;
    double box_length = 0;
    double maxradius = 0;
    double time = 0;
    int ns = 0;
    int nslots = 0;
    std::vector<double> sph;          // [9][ns]
    std::vector<int> sph_slot;        // [ns]
    std::vector<double> agg;          // [21][nslots]
    std::vector<int> agg_n;           // [nslots], 0 for a dead slot
    MemberLists members;              // per slot, list order
};

// A box state in host memory, not owned: the tables of HostState or of an
// mcacg_state. The integer arrays are 32-bit (HostState) or 64-bit
// (mcacg_state, wide). Page-locked arrays are copied by DMA.
struct StateView {
    int n_div = 10;
    double box_length = 0;
    double maxradius = 0;
    double time = 0;
    int ns = 0;
    int nslots = 0;
    const double *sph = nullptr;    // [9][ns]
    const double *agg = nullptr;    // [21][nslots]
    const void *sph_slot = nullptr; // [ns] owning slot
    const void *agg_n = nullptr;    // [nslots] spheres per slot (0: dead slot)
    const void *members = nullptr;  // [ns] member lists of the slots, concatenated in slot order
    bool wide = false;
    bool dead_slots = true;         // slots without spheres are allowed
    long long count(int a) const {
        return wide ? static_cast<const long long *>(agg_n)[a] : static_cast<const int *>(agg_n)[a];
    }
};

// The view of a HostState; 'compact' receives the member ids when the lists
// are not stored back to back in slot order.
StateView view_of(const HostState &st, std::vector<int> *compact);

struct QueryResult {
    double distance;
    int moving_sphere, other_sphere, other_slot;
    int status;
    int n_candidates;
    int n_pairs_refined;
    int n_scanned, n_cells, n_cand_spheres, n_mov;
};

// Per-kernel timings (CUDA events on the box's stream) and the counts the
// algorithmic-byte model of the contact query uses.
struct Profile {
    int64_t queries = 0, merges = 0, translates = 0;
    double query_ms = 0, merge_ms = 0;
    int64_t mov_spheres = 0, scanned = 0, cells = 0, candidates = 0, cand_spheres = 0, refined = 0;
    int64_t merged_spheres = 0, merge_pairs = 0;
};

struct MergeResult {
    int merged, status, keep, removed, n, n_pairs;
    double fields[21];
    double vol_pp;
    double maxradius;
};

// Merged aggregates of at least this many spheres find their contact pairs
// on a hashed cell grid, smaller ones by testing all pairs (the same pairs
// either way). Process-wide; read when a box is created. Default 2048.
int merge_grid_min();
int set_merge_grid_min(int n);  // returns the previous value

class DeviceBox {
  public:
    // Uploads a state to the current device. Returns a status code; an
    // inconsistent state (labels, counts, member lists) gives BAD_ARGUMENT.
    // The host arrays must stay valid until this returns.
    static int create(const HostState &st, void *stream, DeviceBox **out, std::string *err);
    static int create(const StateView &v, void *stream, DeviceBox **out, std::string *err);
    // Many boxes on one stream: one device allocation holds them all (freed
    // with the last of them), the copies go in one stream and the load and
    // grid kernels run over all boxes at once. States of one call have the
    // same integer width. On error, *err names the failing box.
    static int create_many(const std::vector<StateView> &views, void *stream,
                           std::vector<std::unique_ptr<DeviceBox>> *out, std::string *err);
    ~DeviceBox();
    DeviceBox(const DeviceBox &) = delete;
    DeviceBox &operator=(const DeviceBox &) = delete;

    int set_stream(void *stream);
    // VolSurfMethods used by the merges and updates of this box
    // (MCACG_VOLSURF_NONE, _CAPS or _ALPHAS); set before the box runs.
    int set_volsurf(int method);
    void *stream() const { return stream_; }
    bool owns_stream() const { return own_stream_; }
    int query(int src_slot, const double dir[3], double dist, QueryResult *out, std::string *err);
    // n independent queries on the current state (nothing is moved): slots[k],
    // dirs[3k..3k+2], dists[k] -> out[k]. The queries run concurrently, one
    // per thread block. Returns the first failing status, or ST_OK;
    // *kernel_ms (may be null) gets the kernel's CUDA-event time.
    int query_batch(int n, const int *slots, const double *dirs, const double *dists, QueryResult *out,
                    double *kernel_ms, std::string *err);
    int translate(int slot, const double v[3], std::string *err);
    int merge(int ms, int os, int mslot, int oslot, MergeResult *out, std::string *err);
    // Writes aggregate fields of one slot: fields[f] for every f with bit f of mask set.
    int set_fields(int slot, const double fields[21], unsigned mask, std::string *err);
    // Overwrites the whole aggregate table ([21][nslots], slot order).
    int upload_aggregates(const std::vector<double> &agg, std::string *err);
    // Surface growth for the host-driven loop: the spheres of one slot
    // (slot >= 0) or of every live slot grow by du.
    int grow(int slot, double du, std::string *err);
    // The geometry of one slot (slot >= 0) or of every live slot
    // (Aggregate::update when 'full', else update_partial, without the
    // physics fields); the slots follow their positions in the grids. *agg
    // receives the whole table ([21][nslots]) and *vol_pp each slot's mean
    // sphere volume.
    int update_geometry(int slot, bool full, std::vector<double> *agg, std::vector<double> *vol_pp,
                        std::string *err);
    int set_maxradius(double r, std::string *err);
    // Copies the whole state back (spheres, aggregates, members, scalars),
    // on copy_stream when given (so several boxes can come back at once),
    // else on the box's stream.
    int download(HostState *st, std::string *err, void *copy_stream = nullptr);
    // Stores the state straight into caller arrays in the layout of
    // mcacg_state (live aggregates packed in slot order, labels = their
    // ranks): packed on the device, then copied (by DMA into page-locked
    // arrays). The overlap and coordination fields are those on the device.
    // Capacities are out->n_spheres and out->n_aggregates; the scalars are
    // set on return.
    int store(mcacg_state *out, std::string *err, void *copy_stream = nullptr);
    // store() for many boxes at once on 'stream': their scalars in one copy,
    // the packing kernels over all boxes, the pieces copied in one stream.
    // (*rcs)[i] and (*errs)[i] report box i; the return value reports the
    // call itself.
    static int store_many(const std::vector<DeviceBox *> &boxes, const std::vector<mcacg_state *> &outs,
                          void *stream, std::vector<int> *rcs, std::vector<std::string> *errs, std::string *err);
    // Rebuilds the Verlet grid from the aggregate positions with 'cap' rooms per cell.
    int rebuild_grid(int cap, std::string *err);
    int sync(std::string *err);
    void set_profiling(bool on);
    Profile take_profile();
    // Live aggregates (after the work queued on the box's stream).
    int n_alive(int *n, std::string *err);
    int ns() const { return ns_; }
    int nslots() const { return nslots_; }
    void *devbox_ptr() { return devbox_; }  // DevBox* (opaque to host code)

  private:
    DeviceBox() = default;
    int check_status(std::string *err);
    int ensure_out_buffers(std::string *err);
    void *devbox_ = nullptr;  // DevBox (host copy with device pointers)
    void *stream_ = nullptr;
    bool own_stream_ = false;
    int ns_ = 0, nslots_ = 0;
    std::vector<void *> allocations_;
    std::shared_ptr<void> arena_;        // the allocations shared by boxes made together:
    std::shared_ptr<void> arena_grids_;  // fixed parts, and grids
    void *host_out_ = nullptr;  // mapped pinned result buffer
    void *dev_out_ = nullptr;
    bool profiling_ = false;
    void *ev_[2] = {nullptr, nullptr};
    void *batch_mem_ = nullptr;  // query_batch scratch, grown on demand
    size_t batch_bytes_ = 0;
    int batch_threads_ = 0;      // query_batch block size (0: timed at the first large batch)
    void *stage_ = nullptr;      // the merge's pair scratch, also the store staging area
    size_t stage_bytes_ = 0;
    Profile prof_;
};

}  // namespace mcacg
