// config.ini reader: the reference's schema, defaults, unit conversion and
// validation (src/params.cpp:8-260, src/units.cpp:16-65, include/units.h:18-220,
// libs/inireader.cpp semantics), producing the hot-path pimdb_config.
//
// The reader keeps the reference's error messages; errors are reported as
// PIMDB_ERR_CONFIG (the reference's std::invalid_argument) or PIMDB_ERR_PARSE
// (file unreadable).  Keys outside the hot path (steps, sfreq, threshold,
// output and observables sections) are accepted and ignored here.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <regex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/pimdb_gb300.h"
#include "pimdb_host.hpp"
#include "units.hpp"

namespace pimdb_host {

// ---------------------------------------------------------------- INI reader
// Sections and names are case-insensitive, values are trimmed, ';' and '#'
// start a comment line, ';' preceded by whitespace starts an inline comment,
// a repeated key appends "\n" + value (inih / INIReader conventions).
class IniFile {
public:
    explicit IniFile(const std::string& path) {
        std::ifstream in(path);
        if (!in.is_open()) {
            error_ = -1;
            return;
        }
        std::string line, section;
        int lineno = 0;
        while (std::getline(in, line)) {
            ++lineno;
            if (lineno == 1 && line.size() >= 3 && (unsigned char)line[0] == 0xEF && (unsigned char)line[1] == 0xBB &&
                (unsigned char)line[2] == 0xBF)
                line = line.substr(3);
            std::string t = trim(strip_inline_comment(line));
            if (t.empty() || t[0] == ';' || t[0] == '#') continue;
            if (t[0] == '[') {
                const size_t e = t.find(']');
                if (e == std::string::npos) {
                    if (!error_) error_ = lineno;
                    continue;
                }
                section = lower(trim(t.substr(1, e - 1)));
                continue;
            }
            size_t eq = t.find_first_of("=:");
            if (eq == std::string::npos) {
                if (!error_) error_ = lineno;
                continue;
            }
            const std::string key = section + "=" + lower(trim(t.substr(0, eq)));
            const std::string val = trim(t.substr(eq + 1));
            auto it = values_.find(key);
            if (it == values_.end()) values_[key] = val;
            else it->second += "\n" + val;
        }
    }
    int ParseError() const { return error_; }
    std::string Get(const std::string& sec, const std::string& name, const std::string& dflt) const {
        auto it = values_.find(lower(sec) + "=" + lower(name));
        return it == values_.end() ? dflt : it->second;
    }
    std::string GetString(const std::string& sec, const std::string& name, const std::string& dflt) const {
        std::string v = Get(sec, name, "");
        return v.empty() ? dflt : v;
    }
    long GetLong(const std::string& sec, const std::string& name, long dflt) const {
        std::string v = Get(sec, name, "");
        const char* b = v.c_str();
        char* e = nullptr;
        long n = std::strtol(b, &e, 0);
        return e > b ? n : dflt;
    }
    int GetInteger(const std::string& sec, const std::string& name, int dflt) const {
        return (int)GetLong(sec, name, dflt);
    }
    double GetReal(const std::string& sec, const std::string& name, double dflt) const {
        std::string v = Get(sec, name, "");
        const char* b = v.c_str();
        char* e = nullptr;
        double n = std::strtod(b, &e);
        return e > b ? n : dflt;
    }
    bool GetBoolean(const std::string& sec, const std::string& name, bool dflt) const {
        std::string v = lower(Get(sec, name, ""));
        if (v == "true" || v == "yes" || v == "on" || v == "1") return true;
        if (v == "false" || v == "no" || v == "off" || v == "0") return false;
        return dflt;
    }

private:
    static std::string lower(std::string s) {
        for (char& c : s) c = (char)std::tolower((unsigned char)c);
        return s;
    }
    static std::string trim(const std::string& s) {
        size_t b = 0, e = s.size();
        while (b < e && std::isspace((unsigned char)s[b])) ++b;
        while (e > b && std::isspace((unsigned char)s[e - 1])) --e;
        return s.substr(b, e - b);
    }
    static std::string strip_inline_comment(const std::string& s) {
        for (size_t i = 1; i < s.size(); ++i)
            if (s[i] == ';' && std::isspace((unsigned char)s[i - 1])) return s.substr(0, i);
        return s;
    }
    std::map<std::string, std::string> values_;
    int error_ = 0;
};

// "<number> <unit>" -> internal units (params.cpp:281-308)
static double get_quantity(const std::string& family, const std::string& input) {
    std::istringstream iss(input);
    double value;
    std::string unit;
    if (!(iss >> value >> std::ws >> unit)) throw std::invalid_argument("Invalid input format");
    return Units::convertToInternal(family, unit, value);
}

// "token(value)" (params.cpp:311-330)
static bool parse_token_parentheses(const std::string& input, std::string& token, std::string& value) {
    static const std::regex pattern(R"(\s*(\w+)\((.*)\)\s*|\s*(\w+)\s*)");
    std::smatch m;
    if (std::regex_match(input, m, pattern) && (m[1].matched || m[3].matched)) {
        token = m[1].matched ? m[1].str() : m[3].str();
        value = m[2].str();
        return true;
    }
    return false;
}

static std::string fmt3(double v) {
    char b[64];
    std::snprintf(b, sizeof b, "%4.3f", v);
    return b;
}

static void read_config(const IniFile& r, int ndim, pimdb_config& c, RunParams& run) {
    using std::invalid_argument;
    pimdb_config_default(&c);
    c.ndim = ndim;
    const std::string SIM = "simulation", SYS = "system", INT = "interaction_potential", EXT = "external_potential";

    c.dt = get_quantity("time", r.Get(SIM, "dt", "1.0 femtosecond"));
    run.threshold = r.GetReal(SIM, "threshold", 0.1);
    c.gamma = r.GetReal(SIM, "gamma", -1.0);
    if (c.gamma < 0) c.gamma = 1 / (100.0 * c.dt);
    const int nchains = r.GetInteger(SIM, "nchains", 4);
    if (nchains < 1)
        throw invalid_argument("The specified number of Nose-Hoover chains (" + std::to_string(nchains) +
                               ") is less than one!");
    run.steps = (long)std::stod(r.Get(SIM, "steps", "1e5"));
    run.sfreq = r.GetLong(SIM, "sfreq", 1000);
    c.nbeads = r.GetInteger(SIM, "nbeads", 4);
    if (c.nbeads < 1)
        throw invalid_argument("The specified number of beads (" + std::to_string(c.nbeads) + ") is less than one!");
    c.seed = (unsigned int)std::stod(r.Get(SIM, "seed", "1234"));

    const bool bosonic = r.GetBoolean(SIM, "bosonic", false);
    c.bosonic = bosonic;
    c.fixcom = r.GetBoolean(SIM, "fixcom", true);
    c.pbc = r.GetBoolean(SIM, "pbc", false);
    const bool nmthermostat = r.GetBoolean(SIM, "nmthermostat", false);
    c.nmthermostat = nmthermostat;

    std::string tok, spec;
    if (!parse_token_parentheses(r.Get(SIM, "initial_position", "random"), tok, spec))
        throw invalid_argument("The coordinate initialization method format is invalid!");
    if (tok != "random" && tok != "xyz" && tok != "grid")
        throw invalid_argument("The specified coordinate initialization method (" + tok + ") is not supported!");
    run.init_pos_type = tok;
    run.init_pos_spec = spec;
    if (!parse_token_parentheses(r.Get(SIM, "initial_velocity", "random"), tok, spec))
        throw invalid_argument("The velocity initialization method format is invalid!");
    if (tok != "random" && tok != "manual")
        throw invalid_argument("The specified velocity initialization method (" + tok + ") is not supported!");
    run.init_vel_type = tok;
    run.init_vel_spec = spec;
    run.output_positions = r.Get("output", "positions", "off");
    run.output_velocities = r.Get("output", "velocities", "off");
    run.output_forces = r.Get("output", "forces", "off");
    // params.cpp:256-259
    run.obs_energy = r.Get("observables", "energy", "kelvin");
    run.obs_classical = r.Get("observables", "classical", "off");
    run.obs_bosonic = r.Get("observables", "bosonic", "off");
    run.obs_gsf = r.Get("observables", "gsf", "off");

    const std::string propagator = r.GetString(SIM, "propagator", "cartesian");
    if (bosonic && propagator == "normal_modes")
        throw invalid_argument("Normal modes propogation is currently not available for bosons!");
    if (propagator != "cartesian" && propagator != "normal_modes")
        throw invalid_argument("The specified time propagator (" + propagator + ") is not supported!");
    c.propagator = propagator == "normal_modes" ? PIMDB_PROP_NORMAL_MODES : PIMDB_PROP_CARTESIAN;

    const std::string thermostat = r.GetString(SIM, "thermostat", "error");
    if (thermostat == "error") throw invalid_argument("Thermostat must be specified!");
    if (nmthermostat && thermostat == "none") throw invalid_argument("nmthermostat cannot be used in nve ensemble!");
    if (r.GetInteger(SIM, "nchains", -1) != -1 && (thermostat == "none" || thermostat == "langevin"))
        throw invalid_argument("nchains can only be used with Nose-Hoover thermostats!");
    if (thermostat != "langevin" && thermostat != "nose_hoover" && thermostat != "nose_hoover_np" &&
        thermostat != "nose_hoover_np_dim" && thermostat != "none")
        throw invalid_argument("The specified thermostat (" + propagator + ") is not supported!");
    c.thermostat = thermostat == "langevin"             ? PIMDB_THERMO_LANGEVIN
                   : thermostat == "nose_hoover"        ? PIMDB_THERMO_NOSE_HOOVER
                   : thermostat == "nose_hoover_np"     ? PIMDB_THERMO_NOSE_HOOVER_NP
                   : thermostat == "nose_hoover_np_dim" ? PIMDB_THERMO_NOSE_HOOVER_NP_DIM
                                                        : PIMDB_THERMO_NONE;
    c.nchains = nchains;

    c.temperature = get_quantity("temperature", r.Get(SYS, "temperature", "1.0 kelvin"));
    if (c.temperature <= 0.0)
        throw invalid_argument("The specified temperature (" + fmt3(c.temperature) + " kelvin) is unphysical!");
    c.natoms = r.GetInteger(SYS, "natoms", 1);
    if (c.natoms < 1)
        throw invalid_argument("The specified number of particles (" + std::to_string(c.natoms) +
                               ") is smaller than one!");
    c.mass = get_quantity("mass", r.Get(SYS, "mass", "1.0 dalton"));
    if (c.mass <= 0.0) throw invalid_argument("The provided mass (" + fmt3(c.mass) + ") is unphysical!");
    c.size = get_quantity("length", r.Get(SYS, "size", "1.0 picometer"));
    if (c.size <= 0.0) throw invalid_argument("The provided system size (" + fmt3(c.size) + ") is unphysical!");

    const std::string iname = r.GetString(INT, "name", "free");
    if (iname != "aziz" && iname != "free" && iname != "harmonic" && iname != "dipole")
        throw invalid_argument("The specified interaction potential (" + iname + ") is not supported!");
    c.cutoff = get_quantity("length", r.Get(INT, "cutoff", "-1.0 angstrom"));
    c.int_kind = PIMDB_POT_FREE;
    if (iname == "free") {
        c.cutoff = 0.0;
    } else if (iname == "harmonic") {
        c.int_kind = PIMDB_POT_HARMONIC;
        c.int_params[0] = get_quantity("energy", r.Get(INT, "omega", "1.0 millielectronvolt"));
    } else if (iname == "dipole") {
        c.int_kind = PIMDB_POT_DIPOLE;
        c.int_params[0] = r.GetReal(INT, "strength", 1.0);
    } else if (iname == "aziz") {
        c.int_kind = PIMDB_POT_AZIZ;
    }

    const std::string ename = r.GetString(EXT, "name", "free");
    if (ename != "free" && ename != "harmonic" && ename != "double_well" && ename != "cosine")
        throw invalid_argument("The specified external potential (" + ename + ") is not supported!");
    c.ext_kind = PIMDB_POT_FREE;
    if (ename == "harmonic") {
        c.ext_kind = PIMDB_POT_HARMONIC;
        c.ext_params[0] = get_quantity("energy", r.Get(EXT, "omega", "1.0 millielectronvolt"));
    } else if (ename == "double_well") {
        c.ext_kind = PIMDB_POT_DOUBLE_WELL;
        c.ext_params[0] = get_quantity("energy", r.Get(EXT, "strength", "1.0 millielectronvolt"));
        c.ext_params[1] = get_quantity("length", r.Get(EXT, "location", "1.0 angstrom"));
    } else if (ename == "cosine") {
        c.ext_kind = PIMDB_POT_COSINE;
        c.ext_params[0] = get_quantity("energy", r.Get(EXT, "amplitude", "1.0 millielectronvolt"));
        c.ext_params[1] = r.GetReal(EXT, "phase", 1.0);
    }
}

void read_params(const std::string& path, int ndim, pimdb_config& cfg, RunParams& run) {
    if (ndim < 1 || ndim > 3) throw std::invalid_argument("ndim must be 1, 2 or 3");
    IniFile r(path);
    if (r.ParseError() < 0) throw std::invalid_argument("Unable to read the configuration file " + path);
    read_config(r, ndim, cfg, run);
}

}  // namespace pimdb_host

extern "C" int pimdb_config_from_ini(const char* path, int ndim, pimdb_config* cfg, char* err, int err_len) {
    auto report = [&](const std::string& m) {
        if (err && err_len > 0) std::snprintf(err, (size_t)err_len, "%s", m.c_str());
    };
    if (!path || !cfg) return PIMDB_ERR_ARG;
    if (ndim < 1 || ndim > 3) {
        report("ndim must be 1, 2 or 3");
        return PIMDB_ERR_CONFIG;
    }
    pimdb_host::IniFile r(path);
    if (r.ParseError() < 0) {
        report(std::string("Unable to read the configuration file ") + path);
        return PIMDB_ERR_PARSE;
    }
    try {
        pimdb_host::RunParams run;
        pimdb_host::read_config(r, ndim, *cfg, run);
    } catch (const std::exception& ex) {
        report(ex.what());
        return PIMDB_ERR_CONFIG;
    }
    report("");
    return PIMDB_OK;
}
