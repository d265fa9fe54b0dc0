// Parameter-file reader and the physical model of an MCAC box, host side.
//
// Mirrors PhysicalModel (src/physical_model/physical_model.cpp:32-287 and
// 536-617 of the reference): INI keys and defaults, derived box length and gas
// properties, and the friction / mobility / Cunningham formulas used when an
// aggregate is updated. Formulas keep the reference's operation order so the
// host results are bit-identical with glibc's libm.
#pragma once
#include <map>
#include <string>

#include "../../include/mcacg.h"

namespace mcacg {

// INI contents: section -> key -> value. The first definition of a key wins.
using IniData = std::map<std::string, std::map<std::string, std::string>>;

// Parses INI text. Lines starting with ';' or '#' are comments.
IniData parse_ini_text(const std::string &text);

// Fills 'p' from INI data with the reference's defaults and semantics.
// Returns a status code (ST_INPUT for an invalid enumeration value).
int params_from_ini(const IniData &ini, mcacg_params *p, std::string *error);

// Default parameters (physical_model.cpp:32-98).
void params_defaults(mcacg_params *p);

// Derived quantities: box length, gas properties, friction exponent,
// surface-growth velocity (physical_model.cpp:228-269, 536-546).
void params_derive(mcacg_params *p);

// Gas properties at a temperature (physical_model.cpp:536-546).
void update_temperature(mcacg_params *p, double temperature);

// Physics of an aggregate (physical_model.cpp:550-617).
double cunningham(const mcacg_params &p, double r);
double friction_exponent(const mcacg_params &p, double sphere_radius);
double friction_coeff(const mcacg_params &p, double aggregate_volume, double sphere_volume, double sphere_radius);
double mobility_diameter(const mcacg_params &p, double aggregate_volume, double sphere_volume, double sphere_radius);

// Random monomer diameter in metres (physical_model.cpp:557-578); draws from
// the C library generator like the reference. Returns ST_INPUT on bad params.
int random_diameter(const mcacg_params &p, double mean, double dispersion, double *diameter);

// The reference's RNG helpers (src/tools/tools.cpp:41-107), on the C library
// generator.
void init_random(int seed);
double random_uniform();
// Makes this thread's draws come from 'stream' (a bit-identical copy of the C
// library generator) instead of the process-wide rand(); nullptr restores it.
struct RandStream;
void set_thread_stream(RandStream *stream);
void random_direction(double out[3]);
double inverfc(double p);
double inverf(double p);

// Physics fields of an aggregate from its geometry (aggregat.cpp:264-276):
// writes f_agg, d_m, time_step, lpm, dg_over_dp.
struct AggregatePhysics {
    double f_agg, d_m, time_step, lpm, dg_over_dp;
};
AggregatePhysics aggregate_physics(const mcacg_params &p, double volume, double vol_pp, double dp, double rg);

}  // namespace mcacg
