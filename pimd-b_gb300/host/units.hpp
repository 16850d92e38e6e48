// Unit conversion to Hartree atomic units.  The table is the reference's
// (include/units.h:51-210, itself from i-PI's units.py); the conversion
// strips metric prefixes the way src/units.cpp:16-60 does (the last prefix
// matched before the base unit is the one applied).
#pragma once

#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

namespace pimdb_host {
namespace Units {

inline const std::vector<std::pair<std::string, double>>& prefixes() {
    static const std::vector<std::pair<std::string, double>> p = {
        {"yotta", 1e24}, {"zetta", 1e21}, {"exa", 1e18},   {"peta", 1e15},  {"tera", 1e12},
        {"giga", 1e9},   {"mega", 1e6},   {"kilo", 1e3},   {"hecto", 1e2},  {"deci", 1e-1},
        {"centi", 1e-2}, {"milli", 1e-3}, {"micro", 1e-6}, {"nano", 1e-9},  {"pico", 1e-12},
        {"femto", 1e-15}, {"atto", 1e-18}, {"zepto", 1e-21}, {"yocto", 1e-24}};
    return p;
}

inline const std::unordered_map<std::string, std::unordered_map<std::string, double>>& table() {
    static const std::unordered_map<std::string, std::unordered_map<std::string, double>> t = {
        {"undefined", {}},
        {"energy", {{"electronvolt", 0.036749326}, {"j/mol", 0.00000038087989}, {"cal/mol", 0.0000015946679},
                    {"kelvin", 3.1668152e-06}}},
        {"temperature", {{"kelvin", 3.1668152e-06}}},
        {"time", {{"second", 4.1341373e16}}},
        {"frequency", {{"inversecm", 4.5563353e-06}, {"hertz*rad", 2.4188843e-17}, {"hertz", 1.5198298e-16}}},
        {"ms-momentum", {}},
        {"length", {{"angstrom", 1.8897261}, {"meter", 1.8897261e10}, {"radian", 1.00},
                    {"degree", 0.017453292519943295}}},
        {"volume", {{"angstrom3", 6.748334231}}},
        {"velocity", {{"angstrom/ps", 4.5710289e-5}, {"m/s", 4.5710289e-7}}},
        {"momentum", {}},
        {"mass", {{"dalton", 1822.8885}, {"amu", 1822.8885}, {"electronmass", 1.00}}},
        {"pressure", {{"bar", 3.398827377e-9}, {"atmosphere", 3.44386184e-9}, {"pascal", 3.398827377e-14},
                      {"ev/ang3", 0.0054456877}}},
        {"density", {{"g/cm3", 162.67263}}},
        {"force", {{"newton", 12137805}, {"ev/ang", 0.019446904}}},
        {"hessian", {{"ev/ang^2", 0.010290858}}},
    };
    return t;
}

inline double convertToInternal(const std::string& family, const std::string& unit, double number) {
    if (family == "number") return number;
    auto fam = table().find(family);
    if (fam == table().end()) throw std::invalid_argument(family + " is an undefined units kind.");
    std::string rest = unit;
    double scale = 1.0;
    for (bool more = true; more;) {
        more = false;
        for (const auto& [name, val] : prefixes()) {
            if (rest.compare(0, name.size(), name) == 0) {
                rest = rest.substr(name.size());
                scale = val;
                more = true;
                break;
            }
        }
    }
    if (rest.empty() || rest == "automatic" || rest == "atomic_unit") return number * 1.0 * scale;
    auto base = fam->second.find(rest);
    if (base == fam->second.end()) throw std::invalid_argument(rest + " is an undefined unit for kind " + family + ".");
    return number * base->second * scale;
}

inline double convertToUser(const std::string& family, const std::string& unit, double number) {
    return number / convertToInternal(family, unit, 1.0);
}

}  // namespace Units
}  // namespace pimdb_host
