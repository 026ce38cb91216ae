// INI configuration of the rans library.
//
// The reader follows tiny::config (libs/headeronly/tinyconfig.hpp:152-221):
// "[section]" lines, "key = value" lines, and "<k = v, ...>" list entries on
// one line or spread over several lines; all whitespace is stripped from keys
// and values.  Settings::import_config_file (src/rans/include/rans/core.h:
// 238-272) is then applied with the same required keys and the same errors.
// Keys this library adds are optional: [rans-gas] mu_L/Pr_L/Pr_T and
// [rans-solver] precision/limiter/airfoil_name.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <sstream>
#include <unordered_map>

#include "afx_host.hpp"

namespace afx {

namespace {

struct Ini {
    std::unordered_map<std::string, std::unordered_map<std::string, std::string>> config;
    std::unordered_map<std::string, std::vector<std::unordered_map<std::string, std::string>>> config_vec;

    static std::string clean(std::string s) {
        s.erase(std::remove_if(s.begin(), s.end(), [](unsigned char c) { return std::isspace(c); }), s.end());
        return s;
    }
    static void extract(std::unordered_map<std::string, std::string>& map, const std::string& line, size_t sep,
                        size_t end, int line_nb) {
        if (sep == std::string::npos) return;
        if (end == std::string::npos)
            throw Error(2, "Closing character is missing on line: " + std::to_string(line_nb));
        map[clean(line.substr(0, sep))] = clean(line.substr(sep + 1, end - sep - 1));
    }

    void read(const std::string& text) {  // tinyconfig.hpp:186-221
        std::istringstream f(text);
        std::string line, section = "_";
        const std::string ws(" \t\f\v\n\r");
        int line_nb = 0;
        while (std::getline(f, line)) {
            line_nb++;
            auto fb = line.find('[');
            if (fb != std::string::npos) {
                auto sb = line.find(']');
                if (sb == std::string::npos)
                    throw Error(2, "Closing character is missing on line: " + std::to_string(line_nb));
                section = clean(line.substr(fb + 1, sb - fb - 1));
                config[section];
                continue;
            }
            auto fa = line.find('<');
            if (fa != std::string::npos) {
                std::unordered_map<std::string, std::string> entry;
                if (fa == line.find_last_not_of(ws)) {
                    while (std::getline(f, line) && line.find('>') == std::string::npos) {
                        line_nb++;
                        extract(entry, line, line.find('='), line.find(','), line_nb);
                    }
                } else if (line.find('>') != std::string::npos) {
                    line = line.substr(fa + 1);
                    auto comma = line.find(',');
                    while (comma != std::string::npos) {
                        extract(entry, line, line.find('='), comma, line_nb);
                        line = line.substr(comma + 1);
                        comma = line.find(',');
                    }
                    extract(entry, line, line.find('='), line.find('>'), line_nb);
                }
                config_vec[section].push_back(std::move(entry));
                continue;
            }
            extract(config[section], line, line.find('='), line.length(), line_nb);
        }
    }

    const std::string& get(const std::string& sec, const std::string& key) const {
        auto s = config.find(sec);
        if (s == config.end()) throw Error(2, "Section [" + sec + "] not found");
        auto k = s->second.find(key);
        if (k == s->second.end()) throw Error(2, "Setting (" + key + ") not found");
        return k->second;
    }
    const std::string* find(const std::string& sec, const std::string& key) const {
        auto s = config.find(sec);
        if (s == config.end()) return nullptr;
        auto k = s->second.find(key);
        return k == s->second.end() ? nullptr : &k->second;
    }
    int how_many(const std::string& sec) const {
        auto s = config_vec.find(sec);
        if (s == config_vec.end()) throw Error(2, "Section [" + sec + "] not found");
        return (int)s->second.size();
    }
    const std::string& get_i(const std::string& sec, const std::string& key, int i) const {
        auto s = config_vec.find(sec);
        if (s == config_vec.end()) throw Error(2, "Section [" + sec + "] not found");
        auto k = s->second.at(i).find(key);
        if (k == s->second.at(i).end()) throw Error(2, "Setting (" + key + ") not found");
        return k->second;
    }
};

// convert_value<T> (tinyconfig.hpp:61-84): istringstream extraction (0 on failure).
double as_double(const std::string& s) {
    double v = 0;
    std::istringstream(s) >> v;
    return v;
}
int as_int(const std::string& s) {
    int v = 0;
    std::istringstream(s) >> v;
    return v;
}
bool as_bool(std::string s) {
    std::transform(s.begin(), s.end(), s.begin(), ::tolower);
    if (s == "1" || s == "true" || s == "yes" || s == "on") return true;
    if (s == "0" || s == "false" || s == "no" || s == "off") return false;
    throw Error(2, "'" + s + "' is not a valid boolean value.");
}

}  // namespace

int Settings::viscosity_code() const {
    if (viscosity == "laminar") return VISC_LAMINAR;
    if (viscosity == "spalart-allmaras") return VISC_SA;
    if (viscosity == "spallart-allmaras") return VISC_SA_MISSPELLED;
    return VISC_INVISCID;
}

int Settings::bc_code(const std::string& t) {
    if (t == "farfield") return BC_FARFIELD;
    if (t == "slip-wall") return BC_SLIP_WALL;
    if (t == "wall") return BC_WALL;
    if (t == "inlet-outlet") return BC_INLET_OUTLET;
    return BC_INTERNAL;
}

void conservative(const Settings& s, const FarfieldVars& v, double out[4]) {  // core.h:73-83
    double c = std::sqrt(s.gamma * s.R * v.T);
    double u = v.mach * c * std::cos(v.angle);
    double w = v.mach * c * std::sin(v.angle);
    double rho = v.p / (s.R * v.T);
    double rhoE = v.p / (s.gamma - 1) + 0.5 * rho * (u * u + w * w);
    out[0] = rho;
    out[1] = rho * u;
    out[2] = rho * w;
    out[3] = rhoE;
}

void import_ini(Settings& st, const std::string& text) {
    Ini io;
    io.read(text);
    if (io.how_many("rans-bc") != 2) throw Error(2, "[RANS] Invalid number of boundary conditions");
    st.gamma = as_double(io.get("rans-gas", "gamma"));
    st.R = as_double(io.get("rans-gas", "R"));
    if (auto v = io.find("rans-gas", "mu_L")) st.mu_L = as_double(*v);
    if (auto v = io.find("rans-gas", "Pr_L")) st.Pr_L = as_double(*v);
    if (auto v = io.find("rans-gas", "Pr_T")) st.Pr_T = as_double(*v);
    for (int i = 0; i < io.how_many("rans-bc"); ++i) {
        std::string type = io.get_i("rans-bc", "type", i);
        std::string name = io.get_i("rans-bc", "name", i);
        if (!st.bcs.count(name)) st.bc_order.push_back(name);
        auto& bc = st.bcs[name];
        bc.type = type;
        if (type == "farfield") {
            bc.vars.T = as_double(io.get_i("rans-bc", "T", i));
            bc.vars.mach = as_double(io.get_i("rans-bc", "mach", i));
            bc.vars.angle = as_double(io.get_i("rans-bc", "angle", i));
            bc.vars.p = as_double(io.get_i("rans-bc", "p", i));
        }
    }
    // set_solver_type / set_gradient_scheme / set_viscosity_model leave the
    // field unchanged on an unknown string (core.h:203-227)
    const std::string sv = io.get("rans-solver", "solver");
    if (sv == "explicit" || sv == "implicit") st.solver = sv;
    const std::string gr = io.get("rans-solver", "gradient");
    if (gr == "least-squares" || gr == "green-gauss") st.gradient = gr;
    const std::string vi = io.get("rans-solver", "viscosity");
    if (vi == "inviscid" || vi == "laminar" || vi == "spallart-allmaras" || vi == "spalart-allmaras")
        st.viscosity = vi;
    st.second_order = as_bool(io.get("rans-solver", "second_order"));
    st.relaxation = as_double(io.get("rans-solver", "relaxation"));
    st.start_cfl = as_double(io.get("rans-solver", "start_cfl"));
    st.slope_cfl = as_double(io.get("rans-solver", "slope_cfl"));
    st.max_cfl = as_double(io.get("rans-solver", "max_cfl"));
    st.tolerance = as_double(io.get("rans-solver", "tolerance"));
    st.rhs_iterations = as_int(io.get("rans-solver", "rhs_iterations"));
    st.max_iterations = as_int(io.get("rans-solver", "max_iterations"));
    st.limiter_k = as_double(io.get("rans-solver", "limiter_k"));
    if (auto v = io.find("rans-solver", "precision")) {
        if (*v != "fp64" && *v != "fp32-mixed") throw Error(2, "precision must be fp64 or fp32-mixed");
        st.precision = *v;
    }
    if (auto v = io.find("rans-solver", "limiter")) {
        if (*v != "venkatakrishnan" && *v != "michalak") throw Error(2, "limiter must be venkatakrishnan or michalak");
        st.limiter = *v;
    }
    if (auto v = io.find("rans-solver", "airfoil_name")) st.airfoil_name = *v;
    st.alpha_start = as_double(io.get("rans-alphas", "alpha_start"));
    st.alpha_end = as_double(io.get("rans-alphas", "alpha_end"));
    st.alpha_step = as_double(io.get("rans-alphas", "alpha_step"));
}

}  // namespace afx
