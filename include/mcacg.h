/*
 * mcacg.h -- C-ABI of the MCAC GB300 library.
 *
 * The library keeps one or many MCAC boxes resident on one GB300 and runs the
 * per-step collision search and merge update of MCAC (giraldeau/MCAC) there.
 * The entry points below are what a host program binds to replace the
 * reference's C++ member interface that src/calcul.cpp calls each step.
 * Plain C types only; no exception crosses this boundary. Every function
 * returns a status code: 0-11 are the reference's ErrorCodes
 * (include/constants.hpp:70-83), 100+ are this library's own
 * (MCACG_ERR_*). mcacg_last_error() gives the message of the last failure on
 * the calling thread.
 *
 * Labels are the reference's aggregate labels: the position of the aggregate
 * in AggregatList, renumbered after every merge (keep = min label). Sphere
 * indices are storage indices (Sphere::index_in_storage), stable unless
 * oxidation removes spheres (see mcacg_batch_store_state).
 */
#ifndef MCACG_H
#define MCACG_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCACG_ABI_VERSION 2

/* status codes beyond the reference's ErrorCodes */
#define MCACG_ERR_CUDA 100         /* a CUDA call failed */
#define MCACG_ERR_CAPACITY 101     /* a fixed device capacity was exceeded */
#define MCACG_ERR_TIMEOUT 102      /* a bounded device wait gave up */
#define MCACG_ERR_BAD_ARGUMENT 103 /* invalid argument (null pointer, label out of range, ...) */
#define MCACG_ERR_NO_DEVICE 104    /* no CUDA device */

/* initialisation modes and methods, numbered like the reference enums */
#define MCACG_INIT_LOGNORMAL 0 /* MonomeresInitialisationMode, constants.hpp:104-108 */
#define MCACG_INIT_NORMAL 1
#define MCACG_VOLSURF_CAPS 0   /* VolSurfMethods, constants.hpp:113-120 */
#define MCACG_VOLSURF_SBL 1
#define MCACG_VOLSURF_ARVO 2
#define MCACG_VOLSURF_ALPHAS 3
#define MCACG_VOLSURF_NONE 4
#define MCACG_PICK_RANDOM 0    /* PickMethods, constants.hpp:98-102 */
#define MCACG_PICK_LAST 1

/* The PhysicalModel subset of one box (physical_model.hpp:29-97). Filled by
 * mcacg_params_from_ini / mcacg_params_default; the "derived" block is
 * computed by the library. */
typedef struct mcacg_params {
    /* [monomers] */
    int64_t n_monomeres;
    double density;
    double mean_diameter;       /* nm */
    double dispersion_diameter; /* nm (normal) or geometric sigma (lognormal) */
    int32_t initialisation_mode;
    int32_t pick_method;
    /* [environment] */
    double initial_time;
    double volume_fraction;
    double temperature;
    double pressure;
    double fractal_prefactor;
    double fractal_dimension;
    /* [surface_growth] / [oxidation] */
    int32_t with_surface_reactions;
    int32_t volsurf_method;
    double flux_surfgrowth;
    double rp_min_oxid;
    int64_t full_aggregate_update_frequency;
    /* [limits] */
    int64_t number_of_aggregates_limit;
    int64_t n_iter_without_event_limit; /* <= 0: none */
    double cpu_limit;                   /* <= 0: none; CPU seconds (mcacg_calcul only) */
    double physical_time_limit;         /* <= 0: none */
    int64_t mean_monomere_per_aggregate_limit; /* <= 0: none */
    /* [numerics] */
    int32_t with_domain_duplication;
    int32_t with_domain_reduction;
    int32_t with_collisions;
    int32_t enforce_volume_fraction;
    int32_t individual_surf_reactions;
    int32_t random_seed;
    int64_t n_verlet_divisions;
    /* features outside the collision-only path; must be 0 */
    int32_t with_nucleation;
    int32_t with_potentials;
    int32_t with_flame_coupling;
    int32_t with_electric_charges;
    /* derived (physical_model.cpp:228-269, 536-546) */
    double box_length;
    double box_volume;
    double viscosity;
    double gaz_mean_free_path;
    double mean_massic_radius;
    double friction_exponnant;
    double u_sg;
    /* [output] (physical_model.cpp:185-187): when calcul appends a line to
     * advancement.dat (PhysicalModel::time_to_write, physical_model.cpp:338-356) */
    int64_t write_events_frequency;        /* default 1 */
    int64_t write_between_event_frequency; /* default 100 */
    double write_delta_t;                  /* seconds; <= 0: none (default -1) */
    /* [limits] cpu_event (physical_model.cpp:153): CPU seconds since the last
     * event; with cpu_limit, a stop criterion of mcacg_calcul only */
    double cpu_event_limit;                /* <= 0: none (default -1) */
} mcacg_params;

/* Result of a contact search: AggregateContactInfo
 * (include/tools/contact_info.hpp:73-85) with the weak pointers replaced by
 * indices. */
typedef struct mcacg_contact {
    double distance;          /* travel distance to first contact; +inf: none */
    int64_t moving_sphere;    /* sphere storage index; -1: none */
    int64_t other_sphere;     /* sphere storage index; -1: none */
    int64_t moving_aggregate; /* label; -1: none */
    int64_t other_aggregate;  /* label; -1: none */
} mcacg_contact;

/* Box state arrays (host memory), field-major like the reference's SoA
 * storage (constants.hpp:34-69). Used to load and to store a box. */
typedef struct mcacg_state {
    int64_t n_spheres;
    int64_t n_aggregates;
    int64_t n_verlet_divisions;
    double box_length;
    double maxradius;
    double time;
    double *spheres;                 /* [9][n_spheres] */
    int64_t *sphere_label;           /* [n_spheres]: label of the owning aggregate */
    double *aggregates;              /* [21][n_aggregates] */
    int64_t *n_spheres_per_aggregate;/* [n_aggregates] */
    int64_t *members;                /* sphere indices of each aggregate, in list order, concatenated */
} mcacg_state;

/* One MC step of a traced run; layout of mcac_gb300.snapshot.STEP_DTYPE. */
typedef struct mcacg_step_record {
    int64_t step, picked, contact, merged, moving_sphere, other_sphere, moving_agg, other_agg, n_agg_after;
    double deltatemps, full_distance, dir[3], contact_distance, move_distance, time_after, reserved;
} mcacg_step_record;

typedef struct mcacg_run_opts {
    int64_t max_steps;          /* stop after this many MC steps; <= 0: only the stop criteria */
    mcacg_step_record *trace;   /* optional per-step records (host memory) */
    int64_t trace_capacity;
    /* optional: the file the reference's calcul appends its time-resolved
     * lines to (advancement.dat, calcul.cpp:29-43), written at the same steps
     * with the same values and formatting */
    const char *advancement_path;
} mcacg_run_opts;

typedef struct mcacg_run_stats {
    int64_t steps;        /* MC steps done by this call */
    int64_t events;       /* merges done by this call */
    int64_t n_aggregates; /* aggregates left */
    double time;          /* physical time */
    int32_t finished;     /* a stop criterion of the parameters was met */
    int32_t reserved;
} mcacg_run_stats;

/* Kernel timings and work counts of one box since the last read (profiling
 * must be on). Times are CUDA-event durations on the box's stream. */
typedef struct mcacg_profile {
    int64_t queries, merges, translates;
    double query_ms, merge_ms;
    int64_t mov_spheres;  /* spheres of the moving aggregates */
    int64_t scanned;      /* aggregates read from the Verlet cells */
    int64_t cells;        /* Verlet cells scanned */
    int64_t candidates;   /* aggregates passing the bounding-sphere filter */
    int64_t cand_spheres; /* spheres of those candidates */
    int64_t refined;      /* sphere pairs evaluated in FP64 */
    int64_t merged_spheres, merge_pairs;
    /* device-resident loop only: SM clock cycles its thread blocks spent in
     * each phase of the MC step (pick + direction, contact query,
     * translation + time, merge + pick-tree update), summed over boxes */
    int64_t cycles_pick, cycles_query, cycles_move, cycles_merge;
    /* the query cycles split: neighbourhood + bounding-sphere filter, and
     * candidate order + sphere-pair search + ordered walk */
    int64_t cycles_query_scan, cycles_query_pairs;
} mcacg_profile;

typedef struct mcacg_box mcacg_box;

/* ---- library ---- */
int mcacg_abi_version(void);
/* Message of the last failing call on this thread (empty if none). */
const char *mcacg_last_error(void);
/* Number of CUDA devices visible (0 on a machine without a GPU). */
int mcacg_device_count(int *count);

/* ---- parameter file (PhysicalModel::PhysicalModel, physical_model.cpp:32-287) ---- */
int mcacg_params_default(mcacg_params *params);
/* Parse an INI parameter file with the reference's keys and defaults. Unlike
 * the reference constructor it creates no output directory and does not seed
 * the random generator (mcacg_box_create does). */
int mcacg_params_from_ini(const char *path, mcacg_params *params);
int mcacg_params_from_ini_text(const char *text, mcacg_params *params);

/* ---- host-only state construction (no GPU needed) ---- */
/* The random placement of AggregatList::AggregatList
 * (aggregats/aggregat_list_storage.cpp:52-88, aggregat.cpp:162-229) into
 * caller-owned arrays sized for params->n_monomeres spheres and aggregates:
 * seeds the C library generator with random_seed, places the monomers
 * without overlap, computes every aggregate field and applies
 * enforce_volume_fraction. Bit-identical with the reference. */
int mcacg_state_init_random(const mcacg_params *params, mcacg_state *state);
/* A seeded synthetic snapshot for contact-search benchmarks (no counterpart
 * in the reference, which has no state generator): params->n_monomeres
 * spheres, diameters drawn like initialisation_mode=lognormal from
 * mean_diameter and dispersion_diameter, grouped into n_aggregates
 * aggregates of 1..max_size spheres (log-normal sizes, mean
 * n_monomeres/n_aggregates) grown by ballistic sticking, placed without
 * overlap in a periodic cube sized so that the spheres fill
 * params->volume_fraction. Aggregate fields follow Aggregate::update
 * (aggregat.cpp:284-288). Caller-owned arrays sized for n_monomeres spheres
 * and n_aggregates aggregates. Deterministic in random_seed. */
int mcacg_state_synthetic(const mcacg_params *params, int32_t n_aggregates, int32_t max_size, mcacg_state *state);

/* ---- boxes ---- */
/* AggregatList::AggregatList (aggregats/aggregat_list_storage.cpp:52-88):
 * seeds the C library generator with random_seed, places n_monomeres
 * monomers without overlap exactly as the reference does, and uploads the
 * box to the current CUDA device. */
int mcacg_box_create(const mcacg_params *params, mcacg_box **box);
/* Builds a box from a state (no random placement). Aggregate fields are used
 * as given. */
int mcacg_box_create_from_state(const mcacg_params *params, const mcacg_state *state, mcacg_box **box);
int mcacg_box_destroy(mcacg_box *box);
/* Launch the box's kernels on this CUDA stream (cudaStream_t; NULL: the
 * library's own stream). */
int mcacg_box_set_stream(mcacg_box *box, void *cuda_stream);
int mcacg_box_sizes(const mcacg_box *box, int64_t *n_spheres, int64_t *n_aggregates);
/* Copies the whole state to host arrays sized by mcacg_box_sizes. */
int mcacg_box_store_state(mcacg_box *box, mcacg_state *state);
int mcacg_box_get_time(const mcacg_box *box, double *time);
/* Turns per-kernel CUDA-event timing on or off (no counterpart in the
 * reference: instrumentation of this library). */
int mcacg_box_set_profiling(mcacg_box *box, int enable);
/* Reads and resets the counters of mcacg_profile. */
int mcacg_box_take_profile(mcacg_box *box, mcacg_profile *out);
int mcacg_box_set_time(mcacg_box *box, double time);

/* ---- the per-step interface (include/aggregats/aggregat_list.hpp:29-116) ---- */
/* AggregatList::distance_to_next_contact (aggregat_list.hpp:69-71,
 * aggregat_list.cpp:447-484): first contact of aggregate 'source' moving
 * along the unit vector 'direction' for at most 'distance'. */
int mcacg_distance_to_next_contact(mcacg_box *box, int64_t source, const double direction[3], double distance,
                                   mcacg_contact *out);
/* n independent AggregatList::distance_to_next_contact queries on the
 * current state, run concurrently on the GPU (one thread block per query):
 * sources[k], directions[3k..3k+2], distances[k] -> out[k]. Nothing is
 * moved; each result is that of mcacg_distance_to_next_contact on the same
 * state. kernel_ms (may be NULL) receives the kernel's GPU time. No
 * counterpart in the reference, which answers one query at a time. */
int mcacg_distance_to_next_contacts(mcacg_box *box, int32_t n, const int64_t *sources, const double *directions,
                                    const double *distances, mcacg_contact *out, double *kernel_ms);
/* The queries of mcacg_distance_to_next_contacts with no device memory
 * allocated: for callers that cannot allocate while they run (a loop that
 * gave the device to its own memory pool, one that must not take the
 * device-wide synchronisation of cudaMalloc/cudaFree, one under a fixed
 * memory budget). All device scratch is one 32 MiB __device__ array of the
 * library. At most 65536 queries per call (MCACG_ERR_CAPACITY beyond); each
 * thread block keeps up to 16384 refined sphere pairs, as the allocating
 * entry point does (a query refining more fails with MCACG_ERR_CAPACITY on
 * both); a box whose per-block lists (44 bytes per aggregate slot plus
 * 384 KiB of refined pairs) do not fit the array is refused with
 * MCACG_ERR_CAPACITY. Every call looks the array up on the current device
 * (cudaGetSymbolAddress, which allocates nothing); the first call on a
 * device also loads the library's module there, so make it before any
 * stream capture begins. Each call zeroes its query counter and status
 * word, copies the queries in, runs on the box's stream and waits for it.
 * The array is shared by all boxes on a device: overlapping calls would race
 * on it, so the library serialises them with a lock. No counterpart in the
 * reference. */
int mcacg_distance_to_next_contacts_static(mcacg_box *box, int32_t n, const int64_t *sources,
                                           const double *directions, const double *distances, mcacg_contact *out);
/* Aggregate::translate (aggregat.hpp:108, aggregat.cpp:148-161). */
int mcacg_translate(mcacg_box *box, int64_t label, const double vector[3]);
/* Aggregate::time_forward (aggregat.cpp:106-108). */
int mcacg_time_forward(mcacg_box *box, int64_t label, double deltatemps);
/* AggregatList::merge (aggregat_list.hpp:63, aggregat_list.cpp:367-410):
 * *merged = 0 when the two spheres are no longer in contact. Uses the box
 * time for the merged proper time. Throws the reference's MergeError /
 * VolSurfError as status codes 9 / 8. */
int mcacg_merge(mcacg_box *box, const mcacg_contact *contact, int32_t *merged);
/* AggregatList::sort_time_steps / pick_random / get_time_step /
 * get_max_time_step / refresh (aggregat_list.cpp:50-66, 100-141).
 * pick_random draws one number from the C library generator. */
int mcacg_sort_time_steps(mcacg_box *box, double factor);
int mcacg_pick_random(mcacg_box *box, int64_t *label);
int mcacg_get_time_step(const mcacg_box *box, double max, double *deltatemps);
int mcacg_get_max_time_step(const mcacg_box *box, double *max);
int mcacg_refresh(mcacg_box *box);
/* AggregatList::size, get_avg_npp, get_total_volume, get_total_surface. */
int mcacg_size(const mcacg_box *box, int64_t *n_aggregates);
int mcacg_get_avg_npp(const mcacg_box *box, double *avg_npp);
int mcacg_get_total_volume(const mcacg_box *box, double *volume);
int mcacg_get_total_surface(const mcacg_box *box, double *surface);
/* The 21 storage fields of aggregate 'label' and its sphere count. */
int mcacg_get_aggregate(const mcacg_box *box, int64_t label, double fields[21], int64_t *n_spheres);

/* ---- whole runs ---- */
/* The MC loop of mcac::calcul (src/calcul.cpp:66-281) for collisions, with
 * surface reactions when the parameters ask for them (with_surface_reactions:
 * every sphere or the moved aggregate's grows or, u_sg < 0, shrinks; with
 * oxidation spheres at or below rp_min_oxid leave, empty aggregates
 * disappear and disconnected ones split; then the aggregates are updated,
 * calcul.cpp:157-206), driven from the host one step at a time through the
 * entry points above: results are bit-identical with the reference binary
 * built with FP contraction off. Oxidation renumbers spheres and labels as
 * the reference does; it needs a full update every step
 * (full_aggregate_update_frequency 1, else MCACG_ERR_INPUT_ERROR). */
int mcacg_calcul(mcacg_box *box, const mcacg_run_opts *opts, mcacg_run_stats *stats);

/* ---- device-resident runs (batched and served forms) ----
 * The same MC loop with every step on the GPU: one thread block per box,
 * many steps per launch, no host round trip. Contact search, translation and
 * merge geometry are the exact kernels of the calls above; the pick walks a
 * sum tree of 1/time_step (same probabilities as the reference's sorted CDF,
 * different order) and directions and aggregate physics use CUDA's libm, so
 * these runs follow the reference statistically, not step by step. Each box
 * draws from its own copy of the C library rand() stream seeded with its
 * random_seed, continued across consecutive device runs. No counterpart in
 * the reference (it has no batched mode). */
typedef struct mcacg_batch mcacg_batch;
/* Advances one box on the GPU by at most max_steps steps (<= 0: until a stop
 * criterion of its parameters). */
int mcacg_run_device(mcacg_box *box, int64_t max_steps, mcacg_run_stats *stats);
/* n_boxes independent boxes, box i placed as mcacg_box_create would place it
 * with params[i] (size, seed, physics and stop criteria per box).
 * Surface reactions run here in both directions: growth (u_sg >= 0), and
 * oxidation (u_sg < 0: spheres shrink; a sphere at or below rp_min_oxid
 * leaves its aggregate, an aggregate left empty disappears and one whose
 * spheres no longer form one network of contacts splits into one aggregate
 * per connected part; aggregat.cpp:230-243, 545-655). Nucleation,
 * potentials, flame coupling and electric charges give MCACG_ERR_INPUT_ERROR. */
int mcacg_batch_create(const mcacg_params *params, int32_t n_boxes, void *cuda_stream, mcacg_batch **batch);
/* n_boxes boxes from host states (states[i] as for mcacg_box_create_from_state);
 * params[i] gives box i's physics, stop criteria and device stream seed. The
 * arrays are read in place (by DMA when they are page-locked, e.g. from
 * mcacg_host_alloc) and checked on the device: an inconsistent state gives
 * MCACG_ERR_BAD_ARGUMENT. A box that oxidises gets a slot for every sphere
 * (its aggregate table is copied into a larger one), room for any split. */
int mcacg_batch_create_from_states(const mcacg_params *params, const mcacg_state *states, int32_t n_boxes,
                                   void *cuda_stream, mcacg_batch **batch);
/* Page-locked host memory (freed by mcacg_host_free), for state arrays that
 * are loaded and stored by DMA. */
int mcacg_host_alloc(int64_t bytes, void **ptr);
/* Merged aggregates of at least n_spheres spheres find their intra-aggregate
 * contact pairs on a hashed cell grid (O(n)), smaller ones by testing all
 * pairs (O(n^2)); both give the same pairs. Process-wide, read by boxes
 * created afterwards; default 2048. *previous (may be NULL) gets the old value. */
int mcacg_set_merge_grid_min(int32_t n_spheres, int32_t *previous);
/* Once at most n_aggregates aggregates of a box are left (0: never; at most
 * 128; default 128), the device-resident loop at 64 or more threads per box
 * keeps the list of its live aggregates in shared memory: the pick scans the list instead of descending
 * the pick tree in device memory, and a contact query takes its neighbours
 * from it instead of walking the Verlet cells around the moving aggregate
 * (the same neighbours, the same order). Process-wide, read by batches and
 * servers created afterwards; results do not depend on it. *previous (may be
 * NULL) gets the old value. */
int mcacg_set_live_list_max(int32_t n_aggregates, int32_t *previous);
int mcacg_host_free(void *ptr);
int mcacg_batch_destroy(mcacg_batch *batch);
/* Boxes the device-resident loop runs at once on the current device with
 * 'threads' threads per box (32, 64, 128, 256 or 512): its thread blocks per SM x
 * SMs. Batches up to this size take one wave. */
int mcacg_resident_boxes(int32_t threads, int32_t *boxes);
/* Threads per box of the batch's loop: 32, 64, 128, 256 or 512, or 0 (the
 * default): the largest size at which every unfinished box is resident at
 * once, chosen at the start of a run and again whenever half of the boxes
 * running at the last choice have finished. Results do not depend on it. */
int mcacg_batch_set_threads(mcacg_batch *batch, int32_t threads);
int mcacg_batch_threads(const mcacg_batch *batch, int32_t *threads);
/* Speculative rounds of the batch's loop: a cluster of ctas_per_box thread
 * blocks per box (1, the default, or 0: none; 2, 4 or 8). Between two merges the pick tree is
 * fixed, so the picks and directions of the next steps depend on the box's
 * rand() stream alone: each block of the cluster answers one of the next
 * steps' contact queries at once, and the steps are committed in order up
 * to the first one whose answer a committed move could change (same
 * aggregate, or swept bounding capsules within reach) or the first merge;
 * the rest is drawn again. Results do not depend on it: every run is the
 * one-block loop's, bit for bit. The helper blocks' query scratch is
 * allocated once per batch (about 44 bytes per aggregate slot and 384 KiB
 * per helper and box), only when it fits half of the free device memory;
 * boxes with surface reactions always run one step at a time. No
 * counterpart in the reference, whose loop is sequential. */
int mcacg_batch_set_speculation(mcacg_batch *batch, int32_t ctas_per_box);
int mcacg_batch_speculation(const mcacg_batch *batch, int32_t *ctas_per_box);
/* Advances every unfinished box by at most max_steps steps (<= 0: until all
 * meet their stop criteria) in kernel launches of steps_per_launch steps. */
int mcacg_batch_run(mcacg_batch *batch, int64_t max_steps, int64_t steps_per_launch);
/* Advances every unfinished box for about wall_ms milliseconds: launches of
 * at most 200 ms in which each box does as many steps as fit, so boxes of
 * very different cost never wait for one another. Returns early once every
 * box has met its stop criteria. */
int mcacg_batch_run_timed(mcacg_batch *batch, double wall_ms);
/* Sets every box's number_of_aggregates stop criterion
 * (PhysicalModel::finished, physical_model.cpp:288-337) to 'limit'. Boxes
 * that stopped without an error are re-armed: each re-checks all of its
 * criteria before its next step, so a box that has already met the new
 * limit or another criterion does no further step. Lets one batch run a
 * stage of its runs (say, down to 100 aggregates) and then the rest. No
 * counterpart in the reference. */
int mcacg_batch_set_aggregate_limit(mcacg_batch *batch, int64_t limit);
/* Diagnostics of the device loop's random draws (no counterpart in the
 * reference; they check the loop's statistics against the reference's
 * AggregatList::pick_random, aggregat_list.cpp:59-66, 124-141, and
 * random_direction, tools.cpp:82-89).
 * mcacg_batch_pick_histogram: at least n_picks picks (*picks_done gets the
 * number) from box 'box''s current pick tree by the loop's own descent,
 * nothing moved, drawn from rand() streams seeded seed, seed + 1, ...;
 * counts[label] for the live aggregates (*n_labels of them, at most
 * 'capacity'). mcacg_draw_directions: n unit vectors by the loop's direction
 * draw, out[3k..3k+2] (stream of thread t seeded seed + t). */
int mcacg_batch_pick_histogram(mcacg_batch *batch, int32_t box, int64_t n_picks, uint32_t seed, int64_t *counts,
                               int64_t capacity, int64_t *n_labels, int64_t *picks_done);
int mcacg_draw_directions(int64_t n, uint32_t seed, double *out);
/* Per-box counters since creation (arrays of n_boxes). */
int mcacg_batch_stats(mcacg_batch *batch, mcacg_run_stats *stats);
int mcacg_batch_size(const mcacg_batch *batch, int32_t *n_boxes);
int mcacg_batch_box_sizes(mcacg_batch *batch, int32_t box, int64_t *n_spheres, int64_t *n_aggregates);
/* The state of one box in label order. Spheres removed by oxidation leave
 * the stored state as they leave the reference's storage: the others keep
 * their order and n_spheres shrinks (the tables are packed as
 * [9][n_spheres] and [21][n_aggregates]); a box whose spheres all went
 * stores an empty state (no spheres, no aggregates). */
int mcacg_batch_store_state(mcacg_batch *batch, int32_t box, mcacg_state *state);
/* mcacg_batch_store_state for every box at once (states[i] for box i, all
 * n_boxes of them), the conversions spread over the host's cores. */
int mcacg_batch_store_states(mcacg_batch *batch, mcacg_state *states, int32_t n_boxes);
/* Work counters of all boxes since creation, summed (the query and merge
 * fields of mcacg_profile; times are left at 0). */
int mcacg_batch_work(mcacg_batch *batch, mcacg_profile *out);
/* The same counters for one box of the batch. */
int mcacg_batch_box_work(mcacg_batch *batch, int32_t box, mcacg_profile *out);
/* GPU time (CUDA events) and kernel launches of the last mcacg_batch_run. */
int mcacg_batch_last_run(const mcacg_batch *batch, double *kernel_ms, int32_t *launches);

/* ---- serving: continuous batching of aggregation runs ----
 * A request is one box (its parameters; placed like mcacg_box_create). The
 * server keeps 'capacity' thread-block slots on the GPU; each
 * mcacg_server_step admits pending requests in arrival order while a slot is
 * free and the device-memory budget holds their footprint, runs one kernel
 * epoch of at most epoch_steps MC steps per active box, and retires the
 * boxes that met a stop criterion. A box's run depends only on its own state
 * and rand() stream: it is the same alone and in any mix. No counterpart in
 * the reference. */
typedef struct mcacg_server mcacg_server;
typedef struct mcacg_completion {
    int64_t id;
    int64_t steps, events, n_aggregates;
    double time;                        /* physical time reached */
    int32_t status, finished;
    double submit_s, admit_s, finish_s; /* host clock, seconds since the server was created */
} mcacg_completion;
int mcacg_server_create(int32_t capacity, int64_t memory_budget_bytes, void *cuda_stream, int32_t keep_final_states,
                        mcacg_server **server);
int mcacg_server_destroy(mcacg_server *server);
/* Threads per box of the server's epochs: 32, 64, 128, 256 (default) or 512,
 * or 0: at each epoch the largest size at which every active run is resident
 * at once.
 * With smaller blocks more slots fit on the GPU at once
 * (mcacg_resident_boxes); results do not depend on it. */
int mcacg_server_set_threads(mcacg_server *server, int32_t threads);
/* Wall-time cap of one epoch in milliseconds: each box then does as many of
 * its epoch_steps as fit (0, the default: every box does epoch_steps). */
int mcacg_server_set_epoch_ms(mcacg_server *server, double ms);
int mcacg_server_submit(mcacg_server *server, const mcacg_params *params, int64_t *id);
int mcacg_server_step(mcacg_server *server, int64_t epoch_steps, int32_t *n_active, int32_t *n_pending);
/* Moves up to 'capacity' completions (oldest first) into 'out'. */
int mcacg_server_poll(mcacg_server *server, mcacg_completion *out, int32_t capacity, int32_t *n_out);
/* Final state of a completed request (when created with keep_final_states). */
int mcacg_server_final_sizes(mcacg_server *server, int64_t id, int64_t *n_spheres, int64_t *n_aggregates);
int mcacg_server_final_state(mcacg_server *server, int64_t id, mcacg_state *state);
/* GPU time (CUDA events) and kernel launches since creation. */
int mcacg_server_kernel_time(const mcacg_server *server, double *kernel_ms, int32_t *launches);

#ifdef __cplusplus
}
#endif
#endif /* MCACG_H */
