// Host physics of an MCAC box; see physics.hpp. Compiled with
// -ffp-contract=off so every expression rounds like the reference build.
#include "physics.hpp"

#include <cmath>
#include <cstdlib>
#include <sstream>

#include "common.hpp"
#include "rng.hpp"

namespace mcacg {

namespace {

std::string trim(const std::string &s) {
    const char *ws = " \t\r\n\f\v";
    size_t b = s.find_first_not_of(ws);
    if (b == std::string::npos) return std::string();
    size_t e = s.find_last_not_of(ws);
    return s.substr(b, e - b + 1);
}

// Value of [section] key, "" when absent (the reference indexes
// ini.sections[...][...], which yields an empty string for missing keys).
std::string value_of(const IniData &ini, const char *section, const char *key) {
    auto s = ini.find(section);
    if (s == ini.end()) return std::string();
    auto k = s->second.find(key);
    if (k == s->second.end()) return std::string();
    return k->second;
}

// inipp::extract semantics: the destination changes only when the whole
// value parses (std::boolalpha for booleans).
template <class T>
void extract(const std::string &value, T &dst) {
    std::istringstream is(value);
    T result;
    char c;
    if ((is >> std::boolalpha >> result) && !(is >> c)) dst = result;
}
void extract_bool(const std::string &value, int32_t &dst) {
    bool b = dst != 0;
    extract(value, b);
    dst = b ? 1 : 0;
}

}  // namespace

IniData parse_ini_text(const std::string &text) {
    IniData ini;
    std::istringstream is(text);
    std::string line, section;
    while (std::getline(is, line)) {
        std::string t = trim(line);
        if (t.empty() || t[0] == ';' || t[0] == '#') continue;
        if (t[0] == '[') {
            size_t close = t.find(']');
            if (close != std::string::npos) section = trim(t.substr(1, close - 1));
            continue;
        }
        size_t eq = t.find('=');
        if (eq == std::string::npos) continue;
        ini[section].emplace(trim(t.substr(0, eq)), trim(t.substr(eq + 1)));
    }
    return ini;
}

void params_defaults(mcacg_params *p) {
    *p = mcacg_params{};
    p->n_monomeres = 2500;
    p->density = 1800.;
    p->mean_diameter = 30.;
    p->dispersion_diameter = 1.0;
    p->initialisation_mode = MCACG_INIT_LOGNORMAL;
    p->pick_method = MCACG_PICK_RANDOM;
    p->initial_time = 0.;
    p->volume_fraction = 1e-3;
    p->temperature = kTemperatureRef;
    p->pressure = kPressureRef;
    // the reference initialises these two swapped (physical_model.cpp:33-34)
    p->fractal_dimension = 1.4;
    p->fractal_prefactor = 1.8;
    p->with_surface_reactions = 0;
    p->volsurf_method = MCACG_VOLSURF_NONE;
    p->flux_surfgrowth = 0.;
    p->rp_min_oxid = 0.166e-09;
    p->full_aggregate_update_frequency = 1;
    p->number_of_aggregates_limit = 1;
    p->n_iter_without_event_limit = -1;
    p->cpu_limit = -1;
    p->cpu_event_limit = -1;
    p->physical_time_limit = -1;
    p->mean_monomere_per_aggregate_limit = -1;
    p->with_domain_duplication = 1;
    p->with_domain_reduction = 0;
    p->with_collisions = 1;
    p->enforce_volume_fraction = 1;
    p->individual_surf_reactions = 0;
    p->random_seed = -1;
    p->n_verlet_divisions = 10;
    p->gaz_mean_free_path = kFluidMeanFreePathRef;
    p->viscosity = kViscosityRef;
    p->write_events_frequency = 1;
    p->write_between_event_frequency = 100;
    p->write_delta_t = -1;
}

int params_from_ini(const IniData &ini, mcacg_params *p, std::string *error) {
    params_defaults(p);
    std::string mode;
    extract(value_of(ini, "monomers", "number"), p->n_monomeres);
    extract(value_of(ini, "monomers", "density"), p->density);
    extract(value_of(ini, "monomers", "dispersion_diameter"), p->dispersion_diameter);
    extract(value_of(ini, "monomers", "mean_diameter"), p->mean_diameter);
    mode = value_of(ini, "monomers", "initialisation_mode");
    if (!mode.empty()) {
        if (mode == "lognormal") {
            p->initialisation_mode = MCACG_INIT_LOGNORMAL;
        } else if (mode == "normal") {
            p->initialisation_mode = MCACG_INIT_NORMAL;
        } else {
            if (error) *error = "Monomere initialisation mode unknown: " + mode;
            return ST_INPUT;
        }
    }
    extract(value_of(ini, "environment", "initial_time"), p->initial_time);
    extract(value_of(ini, "environment", "volume_fraction"), p->volume_fraction);
    extract(value_of(ini, "environment", "temperature"), p->temperature);
    extract(value_of(ini, "environment", "pressure"), p->pressure);
    extract(value_of(ini, "environment", "fractal_prefactor"), p->fractal_prefactor);
    extract(value_of(ini, "environment", "fractal_dimension"), p->fractal_dimension);
    extract_bool(value_of(ini, "surface_growth", "with_surface_reactions"), p->with_surface_reactions);
    extract(value_of(ini, "surface_growth", "flux_surfgrowth"), p->flux_surfgrowth);
    mode = value_of(ini, "surface_growth", "volsurf_method");
    if (!mode.empty()) {
        const char *names[] = {"caps", "sbl", "arvo", "alphas", "none"};
        int found = VS_INVALID;
        for (int i = 0; i < 5; ++i)
            if (mode == names[i]) found = i;
        if (found == VS_INVALID) {
            if (error) *error = "Invalid method to calculate Vols/Surf: " + mode;
            return ST_INPUT;
        }
        p->volsurf_method = found;
    }
    extract(value_of(ini, "surface_growth", "full_aggregate_update_frequency"), p->full_aggregate_update_frequency);
    extract(value_of(ini, "oxidation", "rp_min"), p->rp_min_oxid);
    extract_bool(value_of(ini, "nucleation", "with_nucleation"), p->with_nucleation);
    extract(value_of(ini, "limits", "number_of_aggregates"), p->number_of_aggregates_limit);
    extract(value_of(ini, "limits", "n_iter_without_event"), p->n_iter_without_event_limit);
    extract(value_of(ini, "limits", "cpu"), p->cpu_limit);
    extract(value_of(ini, "limits", "cpu_event"), p->cpu_event_limit);
    extract(value_of(ini, "limits", "physical_time"), p->physical_time_limit);
    extract(value_of(ini, "limits", "mean_monomere_per_aggregate"), p->mean_monomere_per_aggregate_limit);
    extract_bool(value_of(ini, "numerics", "with_domain_duplication"), p->with_domain_duplication);
    extract_bool(value_of(ini, "numerics", "with_domain_reduction"), p->with_domain_reduction);
    extract_bool(value_of(ini, "numerics", "individual_surf_reactions"), p->individual_surf_reactions);
    extract_bool(value_of(ini, "numerics", "with_collisions"), p->with_collisions);
    extract_bool(value_of(ini, "numerics", "enforce_volume_fraction"), p->enforce_volume_fraction);
    extract(value_of(ini, "numerics", "n_verlet_divisions"), p->n_verlet_divisions);
    mode = value_of(ini, "numerics", "pick_method");
    extract(value_of(ini, "numerics", "random_seed"), p->random_seed);
    if (!mode.empty()) {
        if (mode == "random") {
            p->pick_method = MCACG_PICK_RANDOM;
        } else if (mode == "last") {
            p->pick_method = MCACG_PICK_LAST;
        } else {
            if (error) *error = "Invalid pick method: " + mode;
            return ST_INPUT;
        }
    }
    extract_bool(value_of(ini, "inter_potential", "with_potentials"), p->with_potentials);
    extract_bool(value_of(ini, "inter_potential", "with_electric_charges"), p->with_electric_charges);
    extract_bool(value_of(ini, "flame_coupling", "with_flame_coupling"), p->with_flame_coupling);
    extract(value_of(ini, "output", "write_between_event_frequency"), p->write_between_event_frequency);
    extract(value_of(ini, "output", "write_events_frequency"), p->write_events_frequency);
    extract(value_of(ini, "output", "write_Delta_t"), p->write_delta_t);
    params_derive(p);
    return ST_OK;
}

void update_temperature(mcacg_params *p, double temperature) {
    p->temperature = temperature;
    p->viscosity = kViscosityRef * (kSutherland + kTemperatureRef) / (kSutherland + p->temperature) *
                   std::pow(p->temperature / kTemperatureRef, 1.5);
    p->gaz_mean_free_path = kFluidMeanFreePathRef * (kPressureRef / p->pressure) *
                            (p->temperature / kTemperatureRef) * (1. + kSutherland / kTemperatureRef) /
                            (1. + kSutherland / p->temperature);
    p->friction_exponnant =
        0.689 * (1. + std::erf(((p->gaz_mean_free_path / p->mean_massic_radius) + 4.454) / 10.628));
}

void params_derive(mcacg_params *p) {
    const double pi = pi_value();
    const double n = static_cast<double>(p->n_monomeres);
    if (p->initialisation_mode == MCACG_INIT_NORMAL) {
        p->box_length = p->mean_diameter * 1E-9 *
                        std::pow(n * pi / 6. / p->volume_fraction *
                                     (1. + 3. * std::pow(p->dispersion_diameter / p->mean_diameter, 2)),
                                 1. / 3.);
        p->mean_massic_radius =
            0.5 * 1E-9 *
            (std::pow(p->mean_diameter, 4) + 6 * std::pow(p->mean_diameter, 2) * std::pow(p->dispersion_diameter, 2) +
             3 * std::pow(p->dispersion_diameter, 4)) /
            (std::pow(p->mean_diameter, 3) + 3 * p->mean_diameter * std::pow(p->dispersion_diameter, 2));
    } else {
        p->box_length = p->mean_diameter * 1E-9 *
                        std::pow(n * pi / 6. / p->volume_fraction *
                                     std::exp(9. / 2. * std::pow(std::log(p->dispersion_diameter), 2)),
                                 1. / 3.);
        p->mean_massic_radius =
            0.5 * p->mean_diameter * 1E-9 * std::exp(1.5 * std::pow(std::log(p->dispersion_diameter), 2));
    }
    p->box_volume = std::pow(p->box_length, 3);
    update_temperature(p, p->temperature);
    p->u_sg = p->flux_surfgrowth / p->density;
}

double cunningham(const mcacg_params &p, double r) {
    const double a = 1.142;
    const double b = 0.558;
    const double c = 0.999;
    const double lambda = p.gaz_mean_free_path;
    return 1.0 + a * lambda / r + b * lambda / r * std::exp(-c * r / lambda);
}

double friction_exponent(const mcacg_params &p, double sphere_radius) {
    return 0.689 * (1. + std::erf(((p.gaz_mean_free_path / sphere_radius) + 4.454) / 10.628));
}

double friction_coeff(const mcacg_params &p, double aggregate_volume, double sphere_volume, double sphere_radius) {
    double friction_exp = friction_exponent(p, sphere_radius);
    double cc = cunningham(p, sphere_radius);
    return (6. * pi_value() * p.viscosity * sphere_radius / cc) *
           std::pow(aggregate_volume / sphere_volume, friction_exp / p.fractal_dimension);
}

double mobility_diameter(const mcacg_params &p, double aggregate_volume, double sphere_volume, double sphere_radius) {
    double friction_exp = friction_exponent(p, sphere_radius);
    double aggregate_radius =
        sphere_radius * std::pow(aggregate_volume / sphere_volume, friction_exp / p.fractal_dimension / 2.0);
    double cc_pp = cunningham(p, sphere_radius);
    double cc_a = cunningham(p, aggregate_radius);
    return (cc_a / cc_pp) * 2.0 * sphere_radius *
           std::pow(aggregate_volume / sphere_volume, friction_exp / p.fractal_dimension);
}

AggregatePhysics aggregate_physics(const mcacg_params &p, double volume, double vol_pp, double dp, double rg) {
    AggregatePhysics out;
    out.f_agg = friction_coeff(p, volume, vol_pp, 0.5 * dp);
    out.d_m = mobility_diameter(p, volume, vol_pp, 0.5 * dp);
    double masse = p.density * volume;
    double relax_time = masse / out.f_agg;
    out.time_step = 3. * relax_time;
    double diffusivity = kBoltzmann * p.temperature / out.f_agg;
    out.lpm = std::sqrt(6. * diffusivity * out.time_step);
    out.dg_over_dp = 2 * rg / dp;
    return out;
}

namespace {
// when set, this thread draws from its own copy of the C library stream
thread_local RandStream *t_stream = nullptr;
}  // namespace

void init_random(int seed) {
    if (t_stream) {
        t_stream->seed(static_cast<unsigned>(seed < 0 ? 0 : seed));
        return;
    }
    // a negative seed means "from the clock" in the reference
    // (tools.cpp:41-52); runs here are always seeded explicitly.
    if (seed < 0) seed = 0;
    std::srand(static_cast<unsigned>(seed));
}

void set_thread_stream(RandStream *stream) { t_stream = stream; }

double random_uniform() {
    if (t_stream) return t_stream->uniform();
    double v = std::rand();
    v = v / RAND_MAX;
    return v;
}

double inverfc(double p) {
    if (p >= 2.) return -100.;
    if (p <= 0.0) return 100.;
    double pp = (p < 1.0) ? p : 2. - p;
    double t = std::sqrt(-2. * std::log(pp / 2.));
    double x = -0.70711 * ((2.30753 + t * 0.27061) / (1. + t * (0.99229 + t * 0.04481)) - t);
    for (int j = 0; j < 2; j++) {
        double err = std::erfc(x) - pp;
        x += err / (1.12837916709551257 * std::exp(-(x * x)) - x * err);
    }
    return (p < 1.0 ? x : -x);
}

double inverf(double p) { return inverfc(1. - p); }

void random_direction(double out[3]) {
    double theta = random_uniform() * 2 * pi_value();
    double phi = std::acos(1 - 2 * random_uniform());
    out[0] = std::sin(phi) * std::cos(theta);
    out[1] = std::sin(phi) * std::sin(theta);
    out[2] = std::cos(phi);
}

int random_diameter(const mcacg_params &p, double mean, double dispersion, double *diameter) {
    double d = 0;
    if (p.initialisation_mode == MCACG_INIT_NORMAL) {
        d = mean + std::sqrt(2.) * dispersion * inverf(2. * random_uniform() - 1.0);
    } else if (p.initialisation_mode == MCACG_INIT_LOGNORMAL) {
        if (dispersion < 1.0) return ST_INPUT;
        d = mean * std::pow(dispersion, std::sqrt(2.) * inverf(2. * random_uniform() - 1.0));
    } else {
        return ST_INPUT;
    }
    if (d <= 0) d = mean;
    *diameter = d * 1E-9;
    return ST_OK;
}

}  // namespace mcacg
