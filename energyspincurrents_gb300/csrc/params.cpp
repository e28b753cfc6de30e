// params.cpp -- reference input-file parser.
//
// Same semantics as ConstVariables (src/ParametersEngine.h:53-149) and its matchers
// matchstring / matchstring2 (:157-229): each line is split at the first '='; the part before
// must equal the key exactly (no trimming); the value is read with operator>> (a number for
// numeric keys, a whitespace-delimited token for string keys); the first line that matches AND
// parses wins; a missing mandatory key is an error "<Key>= argument is missing in the input
// file!".  Numeric values are read as double and converted as the reference converts them
// (int(...) truncation, bool(...) = nonzero).  Keys added by this library are optional and
// default to the reference's hard-wired constants.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "esc_internal.h"

namespace {

struct ParseError : std::invalid_argument {
    using std::invalid_argument::invalid_argument;
};

bool match_number(const std::string& file, const std::string& key, double* out) {
    std::ifstream f(file);
    std::string line, test;
    while (std::getline(f, line)) {
        std::istringstream iss(line);
        if (std::getline(iss, test, '=')) {
            double v;
            if ((iss >> v) && test == key) { *out = v; return true; }
        }
    }
    return false;
}

bool match_string(const std::string& file, const std::string& key, std::string* out) {
    std::ifstream f(file);
    std::string line, test;
    while (std::getline(f, line)) {
        std::istringstream iss(line);
        if (std::getline(iss, test, '=')) {
            std::string v;
            if ((iss >> v) && test == key) { *out = v; return true; }
        }
    }
    return false;
}

double need_number(const std::string& file, const char* key) {
    double v;
    if (!match_number(file, key, &v)) throw ParseError(std::string(key) + "= argument is missing in the input file!");
    return v;
}
std::string need_string(const std::string& file, const char* key) {
    std::string v;
    if (!match_string(file, key, &v)) throw ParseError(std::string(key) + "= argument is missing in the input file!");
    return v;
}
double opt_number(const std::string& file, const char* key, double dflt) {
    double v;
    return match_number(file, key, &v) ? v : dflt;
}

void copy_str(char* dst, size_t cap, const std::string& s) {
    std::snprintf(dst, cap, "%s", s.c_str());
}

}  // namespace

extern "C" esc_status esc_params_default(esc_params* p) {
    if (!p) return ESC_ERR_PARAM;
    std::memset(p, 0, sizeof(*p));
    p->Lx = 3; p->Ly = 4; p->pbcx = 1; p->pbcy = 1;
    copy_str(p->model, sizeof(p->model), "Kitaev");
    copy_str(p->solver, sizeof(p->solver), "none");
    copy_str(p->lanctype, sizeof(p->lanctype), "All");
    p->Kxx = p->Kyy = p->Kzz = 1.0;
    p->lanczos_steps = 200;       // src/ParametersEngine.h:85-90
    p->threads = 1;
    p->omega_steps = 1000;        // src/dynamics.h:231-233, :354-356, :72-74
    p->domega = 0.002;
    p->eta = 0.005;
    p->dyn_mode = ESC_DYNMODE_RITZ;
    p->dyn_lanczos_steps = 0;     // 0 = LanczosSteps
    p->precision = 0;
    p->start_vector = ESC_START_REFUNIFORM;
    p->reortho = 1;
    return ESC_OK;
}

extern "C" esc_status esc_params_from_file(const char* path, esc_params* p, char* errbuf, size_t errlen) {
    auto fail = [&](const std::string& msg) {
        if (errbuf && errlen) std::snprintf(errbuf, errlen, "%s", msg.c_str());
        return ESC_ERR_PARAM;
    };
    if (!path || !p) return fail("null argument");
    {
        std::ifstream probe(path);
        if (!probe.good()) return fail(std::string("cannot open input file ") + path);
    }
    try {
        esc_params_default(p);
        const std::string f(path);
        p->Lx = int(need_number(f, "NumberofSitesLx"));
        p->Ly = int(need_number(f, "NumberofSitesLy"));
        p->seed = int(need_number(f, "RandomSeed"));
        copy_str(p->model, sizeof(p->model), need_string(f, "Model"));
        copy_str(p->solver, sizeof(p->solver), need_string(f, "Solver"));
        p->Kxx = need_number(f, "Kxx");
        p->Kyy = need_number(f, "Kyy");
        p->Kzz = need_number(f, "Kzz");
        p->Bxx = need_number(f, "Bxx");
        p->Byy = need_number(f, "Byy");
        p->Bzz = need_number(f, "Bzz");
        p->temperature = need_number(f, "Temperature");
        p->lanczos_eps = need_number(f, "LanczosEps");
        p->pbcx = bool(need_number(f, "IsPeriodicX"));
        p->pbcy = bool(need_number(f, "IsPeriodicY"));
        copy_str(p->lanctype, sizeof(p->lanctype), need_string(f, "LancType"));
        p->threads = int(need_number(f, "Threads"));
        p->lanczos_steps = int(opt_number(f, "LanczosSteps", 200));
        const bool all = std::string(p->lanctype) == "All";
        const char* dyn_err = "You need to set LancType=All for Dynamical calculations --- you dummy!";
        p->local_skw = bool(opt_number(f, "LocalSkw", 0));
        if (p->local_skw && !all) return fail(dyn_err);
        p->spin_curr_dyn = bool(opt_number(f, "SpinCurrDynamics", 0));
        if (p->spin_curr_dyn && !all) return fail(dyn_err);
        p->energy_curr_dyn = bool(opt_number(f, "EnergyCurrDynamics", 0));
        if (p->energy_curr_dyn && !all) return fail(dyn_err);
        // ---- keys added by this library (optional) ----
        p->jheis = opt_number(f, "Jheis", 0.0);
        p->omega_steps = int(opt_number(f, "OmegaSteps", 1000));
        p->domega = opt_number(f, "DOmega", 0.002);
        double omax;
        if (match_number(f, "OmegaMax", &omax)) p->domega = omax / (p->omega_steps > 0 ? p->omega_steps : 1);
        p->eta = opt_number(f, "Eta", 0.005);
        std::string s;
        if (match_string(f, "DynMode", &s)) {
            if (s == "Ritz") p->dyn_mode = ESC_DYNMODE_RITZ;
            else if (s == "CF") p->dyn_mode = ESC_DYNMODE_CF;
            else return fail("DynMode must be Ritz or CF");
        }
        p->dyn_lanczos_steps = int(opt_number(f, "DynLanczosSteps", 0));
        if (match_string(f, "Precision", &s)) {
            if (s == "fp64") p->precision = 0;
            else if (s == "mixed") p->precision = 1;
            else return fail("Precision must be fp64 or mixed");
        }
        if (match_string(f, "StartVector", &s)) {
            if (s == "RefUniform") p->start_vector = ESC_START_REFUNIFORM;
            else if (s == "Normal") p->start_vector = ESC_START_NORMAL;
            else return fail("StartVector must be RefUniform or Normal");
        }
        p->local_szsz_dyn = bool(opt_number(f, "LocalSzSzDynamics", 0));
        if (p->local_szsz_dyn && !all) return fail(dyn_err);
        // `Reortho=` appears in the reference's example input but is never read there: full
        // reorthogonalisation is always on except for LancType=OnlyEgs
        // (src/DynLanczosSolver.h:105-107).  It is ignored here too; the opt-out key of this
        // library is FullReortho=0.
        p->reortho = std::string(p->lanctype) == "OnlyEgs" ? 0 : 1;
        double r;
        if (match_number(f, "FullReortho", &r) && r == 0.0) p->reortho = 0;
        return ESC_OK;
    } catch (std::exception& e) {
        return fail(e.what());
    }
}
