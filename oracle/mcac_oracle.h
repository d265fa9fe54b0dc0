/*
 * mcac_oracle.h -- CPU restatement of the MCAC hot path (test infrastructure).
 *
 * This is the oracle of the test suite and the CPU baseline of bench.py: a
 * plain-C restatement of the reference algorithm (giraldeau/MCAC) for the
 * MC loop -- initial placement, the Verlet grid of aggregate labels, the
 * contact search, translation, merge with label renumbering, the pick CDF,
 * surface growth, and oxidation with sphere removal and splits. It keeps the reference's data structures where they set the
 * result or the cost (sorted label sets per cell, a positional aggregate list
 * renumbered on every removal, an introsort with libstdc++'s element order).
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU arms use it; the
 * product never links it.
 */
#ifndef MCAC_ORACLE_H
#define MCAC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mo_params {
    int64_t n_monomeres;
    double density, mean_diameter, dispersion_diameter;
    int32_t initialisation_mode; /* 0 lognormal, 1 normal */
    int32_t random_seed;
    double initial_time, volume_fraction, temperature;
    double fractal_dimension;
    double viscosity, gaz_mean_free_path; /* derived gas properties */
    double box_length;
    int64_t n_verlet_divisions;
    int32_t enforce_volume_fraction, with_collisions;
    int64_t number_of_aggregates_limit, n_iter_without_event_limit, mean_monomere_per_aggregate_limit;
    double physical_time_limit;
    /* [surface_growth] (flux < 0: oxidation) and [oxidation]; u_sg is derived */
    int32_t with_surface_reactions, individual_surf_reactions;
    double flux_surfgrowth, u_sg;
    int64_t full_aggregate_update_frequency;
    double rp_min_oxid;
} mo_params;

typedef struct mo_contact {
    double distance;
    int64_t moving_sphere, other_sphere, moving_aggregate, other_aggregate;
} mo_contact;

/* same layout as mcacg_step_record / STEP_DTYPE */
typedef struct mo_step_record {
    int64_t step, picked, contact, merged, moving_sphere, other_sphere, moving_agg, other_agg, n_agg_after;
    double deltatemps, full_distance, dir[3], contact_distance, move_distance, time_after, reserved;
} mo_step_record;

typedef struct mo_stats {
    int64_t steps, events, n_aggregates;
    double time;
    int32_t finished, reserved;
} mo_stats;

typedef struct mo_box mo_box;

/* Fills box_length, viscosity, gaz_mean_free_path and u_sg from the raw fields. */
void mo_params_derive(mo_params *p, double pressure);

/* AggregatList::AggregatList: seeds rand() and places n_monomeres monomers. */
int mo_box_new_random(const mo_params *p, mo_box **out);
/* From a state in the snapshot layout (field-major SoA, labels in order). */
int mo_box_new_state(const mo_params *p, int64_t ns, int64_t na, int64_t n_div, double box_length,
                     double maxradius, double time, const double *spheres, const int64_t *sphere_label,
                     const double *aggregates, const int64_t *n_spheres, const int64_t *members, mo_box **out);
void mo_box_free(mo_box *b);
int64_t mo_size(const mo_box *b);
int64_t mo_n_spheres(const mo_box *b);
/* Writes the state in the same layout (arrays sized by mo_n_spheres / mo_size). */
void mo_store(const mo_box *b, double *spheres, int64_t *sphere_label, double *aggregates, int64_t *n_spheres,
              int64_t *members, double *scalars3 /* maxradius, time, box_length */);

int mo_distance_to_next_contact(mo_box *b, int64_t source, const double dir[3], double distance, mo_contact *out);
void mo_translate(mo_box *b, int64_t label, const double v[3]);
int mo_merge(mo_box *b, const mo_contact *c, int32_t *merged);
void mo_sort_time_steps(mo_box *b, double factor);
int64_t mo_pick_random(mo_box *b);
double mo_get_time_step(const mo_box *b, double max);
void mo_refresh(mo_box *b);
double mo_time(const mo_box *b);
void mo_set_time(mo_box *b, double t);
/* Replaces the number_of_aggregates stop criterion (a benchmark runs a box in
 * stages: down to some aggregate count, then on). */
void mo_set_aggregate_limit(mo_box *b, int64_t limit);

/* The MC loop of src/calcul.cpp:66-281 (collisions, with surface growth or
 * oxidation when the parameters ask for them). Stops at the parameters'
 * criteria or after max_steps (> 0). */
int mo_calcul(mo_box *b, int64_t max_steps, mo_step_record *trace, int64_t trace_capacity, mo_stats *stats);

/* libstdc++ std::sort order of indices 0..n-1 by 'keys' (ascending); the
 * restatement used by sort_time_steps, exposed for its own test. */
void mo_sort_indices(const double *keys, int64_t *idx, int64_t n);

#ifdef __cplusplus
}
#endif
#endif
