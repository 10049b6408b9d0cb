// redgb_run -- command-line driver with red's interface, over libredgb.
//
// Replays red's run_simulation (src/red.cuda/main.cu:403-640) on the C ABI of
// libredgb: it reads red's option flags (options.cpp:60-170), its parameter
// file (parameter.cpp:60-257), its analytic gas disk file
// (analytic_gas_disk.cu:90-291) and its start files, body and info records
// (file_util.cpp:325-390, 562-633), integrates, and writes red's output files:
// the numbered snapshots data_NNNNNNNNN.{txt,dat} with their .info files,
// start_files.txt, info.txt, integral.txt, integral.event.txt, event.txt and
// dump files.  Record layouts and number formats are red's, so red's tools read
// the output and a run can restart from it.
//
//   redgb_run -idir <dir> -odir <dir> -p <parameter file> [-i start_files.txt]
//             [-ga <analytic gas disk file>] [-ef] [-v] [-pts] [-id_dev <n>]
//             [-prec mixed|fp64|fp64_exact|fp32]
//
// -cpu, -gpu and -n_chg are accepted and ignored: the integration always runs
// on the GPU.  Every integrator of red's parameter file is taken (Euler and
// RK2 at the fixed initial step, as red's constructors).  The FARGO gas disk
// (-gf) is refused, as red's own constructor fails on it
// (fargo_gas_disk.cu:35, 259-261).
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "redgb.h"

namespace {

const double kGauss = 0.01720209895;            // red_macro.h:13
const double kYearToDay = 365.25;
const double kSolarToGram = 1.0e3 * 1.98911e30; // red_constants.h:142-143
const double kAuToMeter = 1.495978707e11;       // red_constants.h:162
const int kOrdinalWidth = 9;                    // red_macro.h:11

struct Fail {
    std::string msg;
};

struct Options {
    std::string idir = ".", odir = ".", start = "start_files.txt", param, gas;
    bool ef = false, verbose = false, pts = false;
    int device = 0;
    int precision = RED_PREC_MIXED;
};

struct Param {
    std::string name, desc;
    bool binary = false;
    int integrator = RED_INTEGRATOR_RUNGEKUTTAFEHLBERG78;
    bool adaptive = true;
    double tolerance = 1.0e-10;
    bool eftp = false;
    double length = 0.0, output_interval = 0.0;   // code units (k day)
    double info_dt = 5.0, dump_dt = 3600.0;       // wall-clock seconds
    double threshold[RED_THRESHOLD_N] = {0.0, 0.0, 0.0};
};

std::string trim(const std::string& s)
{
    const size_t a = s.find_first_not_of(" \t\r\n");
    if (a == std::string::npos) return "";
    const size_t b = s.find_last_not_of(" \t\r\n");
    return s.substr(a, b - a + 1);
}

std::string path_join(const std::string& dir, const std::string& fn)
{
    if (dir.empty() || dir == ".") return fn;
    return dir.back() == '/' ? dir + fn : dir + "/" + fn;
}

std::string read_text(const std::string& path)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) throw Fail{"Cannot open " + path + "."};
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

// Tokens of s between any of the delimiter characters, empty ones skipped
// (the Tokenizer red's parsers use, red.cuda.utility/tokenizer.cpp:60-85).
std::vector<std::string> tokens(const std::string& s, const char* delims)
{
    std::vector<std::string> out;
    size_t i = 0;
    while (i < s.size()) {
        while (i < s.size() && strchr(delims, s[i])) i++;
        size_t j = i;
        while (j < s.size() && !strchr(delims, s[j])) j++;
        if (j > i) out.push_back(s.substr(i, j - i));
        i = j;
    }
    return out;
}

std::string lower(std::string s)
{
    for (char& c : s) c = (char)tolower((unsigned char)c);
    return s;
}

// "key = value" lines as parameter::parse / set_param read them
// (parameter.cpp:60-100, 108-112; analytic_gas_disk.cu:50-97 alike): every
// non-empty line must hold a key and a value separated by '=', else the file
// is rejected; the key is trimmed and lower-cased, the value trimmed.
std::vector<std::pair<std::string, std::string>> key_values(const std::string& text)
{
    std::vector<std::pair<std::string, std::string>> kv;
    for (const std::string& line : tokens(text, "\r\n")) {
        const std::vector<std::string> t = tokens(line, "=");
        if (t.size() < 2) throw Fail{"Invalid key/value pair: " + line + "."};
        kv.emplace_back(lower(trim(t[0])), trim(t[1]));
    }
    return kv;
}

// tools::is_number (tools.cpp:29-43) then atof, as red reads its numbers
double number(const std::string& key, const std::string& v)
{
    for (char c : v)
        if (!(isdigit((unsigned char)c) || c == 'e' || c == 'E' || c == '.' || c == '-' || c == '+'))
            throw Fail{"Invalid number at: " + key};
    return atof(v.c_str());
}

// parameter::set_param (parameter.cpp:108-240) and transform_time (:250-257)
Param read_param(const std::string& path)
{
    Param p;
    for (const auto& [key, value] : key_values(read_text(path))) {
        if (key == "name") p.name = value;
        else if (key == "description") p.desc = value;
        else if (key == "output data representation" || key == "odr") {
            const std::string lv = lower(value);
            if (lv == "t" || lv == "text") p.binary = false;
            else if (lv == "b" || lv == "binary") p.binary = true;
            else throw Fail{"Invalid data type: " + lv};
        } else if (key == "integrator") {
            const std::string lv = lower(value);
            if (lv == "euler" || lv == "e") p.integrator = RED_INTEGRATOR_EULER;
            else if (lv == "runge-kutta2" || lv == "rk2") p.integrator = RED_INTEGRATOR_RUNGEKUTTA2;
            else if (lv == "runge-kutta4" || lv == "rk4") p.integrator = RED_INTEGRATOR_RUNGEKUTTA4;
            else if (lv == "runge-kutta-fehlberg8" || lv == "rkf8") p.integrator = RED_INTEGRATOR_RUNGEKUTTAFEHLBERG78;
            else throw Fail{"Invalid integrator type: " + lv};
        } else if (key == "tolerance") {
            p.tolerance = number(key, value);
            p.adaptive = true;
        } else if (key == "error check for tp") {
            if (value == "true") p.eftp = true;
            else if (value == "false") p.eftp = false;
            else throw Fail{"Invalid value at: " + key};
        } else if (key == "length") p.length = number(key, value) * kYearToDay * kGauss;
        else if (key == "output interval") p.output_interval = number(key, value) * kYearToDay * kGauss;
        else if (key == "info dt") p.info_dt = number(key, value);
        else if (key == "dump dt" || key == "ddt") p.dump_dt = number(key, value);
        else if (key == "ejection") p.threshold[RED_THRESHOLD_EJECTION_DISTANCE] = number(key, value);
        else if (key == "hit centrum") p.threshold[RED_THRESHOLD_HIT_CENTRUM_DISTANCE] = number(key, value);
        else if (key == "radii enhance factor" || key == "collision factor")
            p.threshold[RED_THRESHOLD_RADII_ENHANCE_FACTOR] = number(key, value);
        else throw Fail{"Invalid parameter: " + key + "."};
    }
    return p;
}

// analytic_gas_disk::set_param + calc + transform_time (analytic_gas_disk.cu:90-291)
red_gas_params_t read_gas(const std::string& path)
{
    red_gas_params_t g;
    memset(&g, 0, sizeof(g));
    const double gram_to_solar = 1.0 / kSolarToGram;
    const double cm_au = 1.0e-2 / kAuToMeter;
    const double gcm3 = gram_to_solar / (cm_au * cm_au * cm_au);
    const double kday = kYearToDay * kGauss;
    for (const auto& [key, value] : key_values(read_text(path))) {
        if (key == "name" || key == "description") continue;
        if (key == "time_dependence") {
            if (value == "constant" || value == "const") g.gas_decrease = 0;
            else if (value == "linear" || value == "lin") g.gas_decrease = 1;
            else if (value == "exponential" || value == "exp") g.gas_decrease = 2;
            else throw Fail{"Invalid value at: " + key + "."};
            continue;
        }
        const double x = number(key, value);
        if (key == "eta_c") g.eta[0] = x;
        else if (key == "eta_p") g.eta[1] = x;
        else if (key == "rho_c") g.rho[0] = x * gcm3;
        else if (key == "rho_p") g.rho[1] = x;
        else if (key == "sch_c") g.sch[0] = x;
        else if (key == "sch_p") g.sch[1] = x;
        else if (key == "tau_c") g.tau[0] = x;
        else if (key == "tau_p") g.tau[1] = x;
        else if (key == "mmw") g.mean_molecular_weight = x * gram_to_solar;
        else if (key == "diameter") g.particle_diameter = x / kAuToMeter;
        else if (key == "alpha") g.alpha = x;
        else if (key == "t0") g.t0 = x * kday;
        else if (key == "t1") g.t1 = x * kday;
        else if (key == "e_folding_time") g.e_folding_time = x * kday;
        else throw Fail{"Invalid parameter :" + key + "."};
    }
    return g;
}

// ---------------------------------------------------------------------------
// red's body and info records (file_util.cpp:325-390, 562-633)
// ---------------------------------------------------------------------------
struct Bodies {
    std::vector<std::string> name;
    std::vector<red_var4_t> r, v;
    std::vector<red_param_t> p;
    std::vector<red_body_metadata_t> md;
    uint32_t counts[RED_BODY_N] = {0};
    double t = 0.0, dt = 0.0;
    uint32_t dt_cpu = 0;
};

bool ends_with(const std::string& s, const std::string& e)
{
    return s.size() >= e.size() && s.compare(s.size() - e.size(), e.size(), e) == 0;
}

void read_info(const std::string& path, Bodies& b)
{
    const std::string raw = read_text(path);
    if (ends_with(path, ".dat")) {
        if (raw.size() < 48) throw Fail{"Short binary info record: " + path};
        memcpy(&b.t, raw.data(), 8);
        memcpy(&b.dt, raw.data() + 8, 8);
        memcpy(&b.dt_cpu, raw.data() + 16, 4);
        memcpy(b.counts, raw.data() + 20, 4 * RED_BODY_N);
        return;
    }
    std::istringstream in(raw);
    in >> b.t >> b.dt >> b.dt_cpu;
    for (int k = 0; k < RED_BODY_N; k++) in >> b.counts[k];
    if (!in) throw Fail{"Invalid info record: " + path};
}

void read_data(const std::string& path, Bodies& b)
{
    uint32_t n = 0;
    for (int k = 0; k < RED_BODY_N; k++) n += b.counts[k];
    b.name.resize(n);
    b.r.assign(n, red_var4_t{});
    b.v.assign(n, red_var4_t{});
    b.p.assign(n, red_param_t{});
    b.md.assign(n, red_body_metadata_t{});
    const std::string raw = read_text(path);
    if (ends_with(path, ".dat")) {
        const size_t rec = 30 + 24 + 32 + 48;
        if (raw.size() < rec * n) throw Fail{"Short binary data file: " + path};
        for (uint32_t i = 0; i < n; i++) {
            const char* q = raw.data() + rec * i;
            b.name[i] = std::string(q, strnlen(q, 30));
            memcpy(&b.md[i], q + 30, 24);
            memcpy(&b.p[i], q + 54, 32);
            double x[6];
            memcpy(x, q + 86, 48);
            b.r[i] = red_var4_t{x[0], x[1], x[2], 0.0};
            b.v[i] = red_var4_t{x[3], x[4], x[5], 0.0};
        }
        return;
    }
    std::istringstream in(raw);
    for (uint32_t i = 0; i < n; i++) {
        in >> b.name[i] >> b.md[i].id >> b.md[i].body_type >> b.md[i].mig_type >> b.md[i].mig_stop_at >> b.p[i].mass >>
            b.p[i].radius >> b.p[i].density >> b.p[i].cd >> b.r[i].x >> b.r[i].y >> b.r[i].z >> b.v[i].x >> b.v[i].y >>
            b.v[i].z;
        if (!in) throw Fail{"Invalid body record " + std::to_string(i) + " in " + path};
    }
}

void write_info(const std::string& path, bool binary, double t, double dt, uint32_t dt_cpu, const uint32_t* active)
{
    FILE* f = fopen(path.c_str(), binary ? "wb" : "w");
    if (!f) throw Fail{"Cannot open " + path + "."};
    if (binary) {
        fwrite(&t, 8, 1, f);
        fwrite(&dt, 8, 1, f);
        fwrite(&dt_cpu, 4, 1, f);
        fwrite(active, 4, RED_BODY_N, f);
    } else {
        fprintf(f, "%25.16e %25.16e %10u ", t, dt, dt_cpu);
        for (int k = 0; k < RED_BODY_N; k++) fprintf(f, "%8u ", active[k]);
    }
    fclose(f);
}

void write_data(const std::string& path, bool binary, const Bodies& b)
{
    FILE* f = fopen(path.c_str(), binary ? "wb" : "w");
    if (!f) throw Fail{"Cannot open " + path + "."};
    for (size_t i = 0; i < b.md.size(); i++) {
        if (b.md[i].id < 0) continue;   // inactive bodies are not written
        if (binary) {
            char name[30];
            memset(name, 0, sizeof(name));
            memcpy(name, b.name[i].data(), std::min<size_t>(30, b.name[i].size()));
            fwrite(name, 1, 30, f);
            fwrite(&b.md[i], 24, 1, f);
            fwrite(&b.p[i], 32, 1, f);
            const double x[6] = {b.r[i].x, b.r[i].y, b.r[i].z, b.v[i].x, b.v[i].y, b.v[i].z};
            fwrite(x, 8, 6, f);
        } else {
            fprintf(f, "%30s %8d %2d %2d %25.16e %25.16e %25.16e %25.16e %25.16e %25.16e %25.16e %25.16e %25.16e %25.16e %25.16e\n",
                    b.name[i].c_str(), b.md[i].id, b.md[i].body_type, b.md[i].mig_type, b.md[i].mig_stop_at, b.p[i].mass,
                    b.p[i].radius, b.p[i].density, b.p[i].cd, b.r[i].x, b.r[i].y, b.r[i].z, b.v[i].x, b.v[i].y, b.v[i].z);
        }
    }
    fclose(f);
}

// ---------------------------------------------------------------------------
// the run (main.cu:403-640)
// ---------------------------------------------------------------------------
void check(int rc)
{
    if (rc != RED_OK) throw Fail{std::string("libredgb: ") + red_last_error()};
}

struct Run {
    Options opt;
    Param par;
    red_sim* sim = nullptr;
    std::map<int32_t, std::string> names;   // red's body names by |id|
    std::string prefix, ext;
    std::string path_info, path_integral, path_integral_event, path_event;
    uint32_t n_print = 0;
    double wall0 = 0.0;

    static double now()
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
    }

    // the bodies of the handle as red's records (names re-attached by id)
    Bodies state()
    {
        red_system_info_t info;
        check(red_get_system_info(sim, 0, &info));
        Bodies b;
        const uint32_t n = info.n_total;
        b.r.resize(n);
        b.v.resize(n);
        b.p.resize(n);
        b.md.resize(n);
        b.name.resize(n);
        check(red_get_state(sim, 0, b.r.data(), b.v.data(), b.p.data(), b.md.data()));
        for (uint32_t i = 0; i < n; i++) {
            const auto it = names.find(std::abs(b.md[i].id));
            b.name[i] = it != names.end() ? it->second : "body" + std::to_string(i);
        }
        b.t = info.t;
        b.dt = info.dt_did;
        b.dt_cpu = (uint32_t)(now() - wall0);
        return b;
    }

    static void active_counts(const Bodies& b, uint32_t* out)
    {
        for (int k = 0; k < RED_BODY_N; k++) out[k] = 0;
        for (const auto& m : b.md)
            if (m.id >= 0 && m.body_type >= 0 && m.body_type < RED_BODY_N) out[m.body_type]++;
    }

    void write_snapshot(const std::string& stem)
    {
        const Bodies b = state();
        uint32_t act[RED_BODY_N];
        active_counts(b, act);
        const std::string fn_data = prefix + stem + "." + ext, fn_info = prefix + stem + ".info." + ext;
        write_data(path_join(opt.odir, fn_data), par.binary, b);
        write_info(path_join(opt.odir, fn_info), par.binary, b.t, b.dt, b.dt_cpu, act);
        std::ofstream s(path_join(opt.odir, "start_files.txt"));
        if (!s) throw Fail{"Cannot open start_files.txt in " + opt.odir};
        s << fn_info << "\n" << fn_data << "\n";
    }

    // pp_disk::print_integral_data (pp_disk.cu:2096-2124)
    void write_integral(const std::string& path)
    {
        red_integral_t I;
        check(red_calc_integral(sim, 0, &I));
        red_system_info_t info;
        check(red_get_system_info(sim, 0, &info));
        FILE* f = fopen(path.c_str(), "a");
        if (!f) throw Fail{"Cannot open " + path + "."};
        const double v[11] = {info.t / kGauss, I.R.x, I.R.y, I.R.z, I.V.x * kGauss, I.V.y * kGauss, I.V.z * kGauss,
                              I.C.x * kGauss, I.C.y * kGauss, I.C.z * kGauss, I.E * kGauss * kGauss};
        for (double x : v) fprintf(f, "%25.16e ", x);
        fprintf(f, "\n");
        fclose(f);
    }

    // print_data (main.cu:194-220): the numbered snapshot, start files, an integral line
    void print_data()
    {
        char num[32];
        snprintf(num, sizeof(num), "%0*u", kOrdinalWidth, n_print);
        write_snapshot(std::string("data_") + num);
        n_print++;
        write_integral(path_integral);
    }

    void print_dump() { write_snapshot("dump"); }

    // pp_disk::print_event_data (pp_disk.cu:2008-2085)
    void write_events(const std::vector<red_event_t>& ev)
    {
        static const char* names_ev[] = {"NONE", "HIT_CENTRUM", "EJECTION", "COLLISION"};
        FILE* f = fopen(path_event.c_str(), "a");
        if (!f) throw Fail{"Cannot open " + path_event + "."};
        for (const red_event_t& e : ev) {
            fprintf(f, "%16s %25.16e %25.16e %8d %8d %8d ", names_ev[e.event_name & 3], e.t, e.d, e.id0, e.id1, e.id2);
            const red_param_t* ps[4] = {&e.p0, &e.p1, &e.p2, &e.ps};
            const red_var4_t* rs[4] = {&e.r0, &e.r1, &e.r2, &e.rs};
            const red_var4_t* vs[4] = {&e.v0, &e.v1, &e.v2, &e.vs};
            for (int k = 0; k < 4; k++)
                fprintf(f, "%25.16e %25.16e %25.16e %25.16e %25.16e %25.16e %25.16e %25.16e %25.16e ", ps[k]->mass,
                        ps[k]->density, ps[k]->radius, rs[k]->x, rs[k]->y, rs[k]->z, vs[k]->x, vs[k]->y, vs[k]->z);
            fprintf(f, "\n");
        }
        fclose(f);
    }

    // print_info (main.cu:133-192): one CSV line per call
    void print_info(double dt, double dT, bool first)
    {
        red_system_info_t info;
        check(red_get_system_info(sim, 0, &info));
        FILE* f = fopen(path_info.c_str(), "a");
        if (!f) throw Fail{"Cannot open " + path_info + "."};
        if (first)
            fprintf(f, "dev,date      ,time    ,t [d]      ,dt [d]     ,dt_avg [d] ,dT [s]     ,dT_avg [s] ,Nc   ,Ne   ,"
                       "Nh   ,nb_p ,nb_i,nb_r ,ns_t    ,ns_p    ,ns_f    ,ns_a,ns_r  ,ngp_a,ngp_r,nrp_a,nrp_r,npp_a,"
                       "npp_r,nspl_a,nspl_r,npl_a,npl_r,ntp_a,ntp_r\n");
        const time_t tt = time(nullptr);
        char stamp[64];
        strftime(stamp, sizeof(stamp), "%Y-%m-%d,%H:%M:%S", localtime(&tt));
        const double np = info.n_passed ? (double)info.n_passed : 1.0;
        uint32_t playing = 0, inactive = 0, removed = 0;
        for (int k = 0; k < RED_BODY_N; k++) {
            playing += info.playing[k];
            inactive += info.inactive[k];
            removed += info.removed[k];
        }
        fprintf(f, "GPU,%s,%.4e,%.4e,%.4e,%.4e,%.4e,%u,%u,%u,%u,%u,%u,%llu,%llu,%llu", stamp, info.t / kGauss,
                dt / kGauss, info.t / kGauss / np, dT, (now() - wall0) / np, info.n_collision[0], info.n_ejection[0],
                info.n_hit_centrum[0], playing, inactive, removed, (unsigned long long)info.n_tried,
                (unsigned long long)info.n_passed, (unsigned long long)info.n_failed);
        for (int k = 0; k < RED_BODY_N; k++) fprintf(f, ",%u,%u", info.playing[k] - info.inactive[k], info.removed[k]);
        fprintf(f, "\n");
        fclose(f);
        if (opt.pts || opt.verbose)
            printf("[GPU] t: %10.4e, dt: %10.4e [d], N: %u (%u, %u), nt: %llu, np: %llu, nf: %llu\n", info.t / kGauss,
                   dt / kGauss, playing, inactive, removed, (unsigned long long)info.n_tried,
                   (unsigned long long)info.n_passed, (unsigned long long)info.n_failed);
    }

    int run()
    {
        wall0 = now();
        par = read_param(path_join(opt.idir, opt.param));
        // start files: the info record on line 1, the body records on line 2 (main.cu:206-214)
        std::istringstream sf(read_text(path_join(opt.idir, opt.start)));
        std::string fn_info, fn_data;
        std::getline(sf, fn_info);
        std::getline(sf, fn_data);
        fn_info = trim(fn_info);
        fn_data = trim(fn_data);
        Bodies b;
        read_info(path_join(opt.idir, fn_info), b);
        read_data(path_join(opt.idir, fn_data), b);
        for (size_t i = 0; i < b.md.size(); i++) names[std::abs(b.md[i].id)] = b.name[i];

        red_config_t cfg;
        memset(&cfg, 0, sizeof(cfg));
        cfg.integrator = par.integrator;
        cfg.adaptive = par.adaptive ? 1 : 0;
        cfg.tolerance = par.tolerance;
        cfg.error_check_for_tp = par.eftp ? 1 : 0;
        cfg.precision = opt.precision;
        for (int k = 0; k < RED_THRESHOLD_N; k++) cfg.threshold[k] = par.threshold[k];
        cfg.output_interval = par.output_interval;
        // red steps while the integrated time is within the length: one step when it is zero
        cfg.length = par.length > 0.0 ? par.length : 1.0e-300;
        if (!opt.gas.empty()) {
            cfg.gas_disk = 1;
            cfg.gas = read_gas(path_join(opt.idir, opt.gas));
        }
        cfg.device = opt.device;
        const double t0 = b.t;
        const double dt0 = b.dt > 0.0 ? b.dt : (par.output_interval > 0.0 ? par.output_interval : kGauss);
        check(red_create(&cfg, 1, b.counts, b.r.data(), b.v.data(), b.p.data(), b.md.data(), &t0, &dt0, &sim));

        // output names (main.cu:101-131, 405-411)
        if (opt.ef)
            prefix = std::string("R_gpu_") + (par.adaptive ? "as" : "fs") + "_" +
                     (par.integrator == RED_INTEGRATOR_RUNGEKUTTA4 ? "RK4" : "RKF7") + "_";
        ext = par.binary ? "dat" : "txt";
        path_info = path_join(opt.odir, prefix + "info.txt");
        path_integral = path_join(opt.odir, prefix + "integral.txt");
        path_integral_event = path_join(opt.odir, prefix + "integral.event.txt");
        path_event = path_join(opt.odir, prefix + "event.txt");

        // a restart from snapshot data_N continues the numbering (main.cu:431-447)
        if (fn_data.size() >= 4 && fn_data.compare(0, 4, "data") == 0) {
            const size_t pos = fn_data.find('_');
            if (pos != std::string::npos) n_print = (uint32_t)atoi(fn_data.substr(pos + 1, kOrdinalWidth).c_str()) + 1;
        }
        if (n_print == 0 && fn_data.compare(0, 4, "dump") != 0) print_data();

        double ps = 0.0, dt = 0.0, last_dump = now(), last_info = now(), step_wall = 0.0;
        bool first_info = true;
        red_system_info_t info;
        check(red_get_system_info(sim, 0, &info));
        while (info.active) {
            const double w0 = now();
            check(red_step(sim, &dt));
            step_wall = now() - w0;
            ps += dt;
            check(red_get_system_info(sim, 0, &info));
            if (info.halted) {
                // collisions, ejections, hits of the centre: integrals before and after,
                // the event records, a dump (main.cu:499-569)
                write_integral(path_integral_event);
                std::vector<red_event_t> ev(4096);
                uint32_t n_ev = 0;
                check(red_handle_events(sim, ev.data(), (uint32_t)ev.size(), &n_ev));
                ev.resize(std::min<uint32_t>(n_ev, (uint32_t)ev.size()));
                write_integral(path_integral_event);
                write_events(ev);
                print_dump();
                last_dump = now();
                check(red_get_system_info(sim, 0, &info));
            }
            if (par.output_interval > 0.0 && par.output_interval <= std::fabs(ps)) {
                ps = 0.0;
                print_data();
            }
            if (par.dump_dt < now() - last_dump) {
                last_dump = now();
                print_dump();
            }
            if (par.info_dt < now() - last_info) {
                last_info = now();
                print_info(dt, step_wall, first_info);
                first_info = false;
            }
            if (info.status != RED_OK) throw Fail{std::string("integration stopped: ") + red_last_error()};
        }
        print_info(dt, step_wall, first_info);
        if (0.0 < std::fabs(ps)) print_data();   // the final state, unless just written
        red_destroy(sim);
        sim = nullptr;
        return 0;
    }
};

void usage()
{
    printf("usage: redgb_run -idir <dir> -odir <dir> -p <parameter file> [-i <start files>] [-ga <gas disk file>]\n"
           "                 [-ef] [-v] [-pts] [-id_dev <n>] [-prec mixed|fp64|fp64_exact|fp32]\n");
}

}  // namespace

int main(int argc, char** argv)
{
    Run R;
    try {
        for (int i = 1; i < argc; i++) {
            const std::string a = argv[i];
            auto next = [&]() -> std::string {
                if (i + 1 >= argc) throw Fail{"missing value after " + a};
                return argv[++i];
            };
            if (a == "-idir") R.opt.idir = next();
            else if (a == "-odir") R.opt.odir = next();
            else if (a == "-i") R.opt.start = next();
            else if (a == "-p") R.opt.param = next();
            else if (a == "-ga") R.opt.gas = next();
            else if (a == "-gf") throw Fail{"the FARGO gas disk is not on this path"};
            else if (a == "-ef") R.opt.ef = true;
            else if (a == "-v") R.opt.verbose = true;
            else if (a == "-pts") R.opt.pts = true;
            else if (a == "-id_dev") R.opt.device = atoi(next().c_str());
            else if (a == "-n_chg") next();
            else if (a == "-t" || a == "-pe" || a == "-cpu" || a == "-gpu") continue;
            else if (a == "-prec") {
                const std::string p = next();
                if (p == "mixed") R.opt.precision = RED_PREC_MIXED;
                else if (p == "fp64") R.opt.precision = RED_PREC_FP64;
                else if (p == "fp64_exact") R.opt.precision = RED_PREC_FP64_EXACT;
                else if (p == "fp32") R.opt.precision = RED_PREC_FP32;
                else throw Fail{"invalid precision: " + p};
            } else if (a == "-h") {
                usage();
                return 0;
            } else throw Fail{"invalid option: " + a};
        }
        if (R.opt.param.empty()) {
            usage();
            throw Fail{"a parameter file (-p) is required"};
        }
        return R.run();
    } catch (const Fail& f) {
        fprintf(stderr, "redgb_run: %s\n", f.msg.c_str());
        if (R.sim) red_destroy(R.sim);
        return 1;
    }
}
