// ref_harness.cu -- drives the reference's own CPU code (TEST INFRASTRUCTURE).
//
// Built by oracle/ref_build.sh against the unmodified sources of
// suliaron/red.cuda (src/red.cuda, src/red.cuda.utility, red.type) into
// oracle/_ref/ref_harness.  It loads a red input (info + data file pair) with
// pp_disk's own file constructor (pp_disk.cu:1546-1575) and calls the public
// pp_disk / rungekutta4 / rungekutta8 methods on the CPU, writing raw doubles
// so that tests/golden/make_golden.py can store the reference's answers as
// fixtures.  pp_disk's private members are reached by compiling this unit with
// 'private' mapped to 'public' (the class layout is unchanged).
//
// usage: ref_harness key=value ...
//   dir=  info=  data=            red input files (ASCII .txt or binary .dat)
//   out=                          output file (raw little-endian records)
//   mode=accel|run|coll|ejhc|integral|dump
//   integrator=1|2|4|8 (Euler, RK2, RK4, RKF78) adaptive=0|1 tol= nsteps= eftp=0|1   (mode=run)
//   factor= t=                    (mode=coll)
//   ej= hc=                       (mode=ejhc)
//   gasdir= gas= t=               (mode=accel: adds drag on NSI bodies)
//   odir=                         (mode=dump: red's own print_data/print_data_info)
//   dev=cpu|gpu                   gpu: red's own GPU path (pp_disk on COMPUTING_DEVICE_GPU,
//                                 copy_to_device, the n_tpb search of run_simulation,
//                                 main.cu:449-463); accel writes red's gravity + drag as one
//                                 array, run times the step loop, coll writes the raw events
//   tpb=                          (dev=gpu) threads per block instead of red's search
//   tout=                         (dev=gpu, mode=run) file for the step loop's wall time
//
// With dev=gpu the binary must be built on the machine that has the GPU
// (oracle/ref_build.sh, from a staged copy of the unmodified sources).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>
#include <fstream>

#define private public
#include "pp_disk.h"
#include "integrator.h"
#include "int_euler.h"
#include "int_rungekutta2.h"
#include "int_rungekutta4.h"
#include "int_rungekutta8.h"
#undef private
#include "redutilcu.h"
#include "red_constants.h"

using namespace std;

static map<string, string> args;

static string arg(const char* k, const char* def = "")
{
    map<string, string>::iterator it = args.find(k);
    return it == args.end() ? string(def) : it->second;
}

static void put(FILE* f, const void* p, size_t n) { fwrite(p, 1, n, f); }

static void put_state(FILE* f, pp_disk* ppd)
{
    uint32_t n = ppd->n_bodies->get_n_total_playing();
    put(f, &n, 4);
    put(f, ppd->n_bodies->playing, 7 * 4);
    put(f, ppd->n_bodies->inactive, 7 * 4);
    put(f, &ppd->t, 8);
    put(f, ppd->sim_data->h_y[0], n * sizeof(var4_t));
    put(f, ppd->sim_data->h_y[1], n * sizeof(var4_t));
    put(f, ppd->sim_data->h_p, n * sizeof(pp_disk_t::param_t));
    put(f, ppd->sim_data->h_body_md, n * sizeof(pp_disk_t::body_metadata_t));
}

static void put_events(FILE* f, const vector<pp_disk_t::event_data_t>& ev)
{
    uint32_t n = (uint32_t)ev.size();
    put(f, &n, 4);
    for (uint32_t i = 0; i < n; i++) put(f, &ev[i], sizeof(pp_disk_t::event_data_t));
}

int main(int argc, char** argv)
{
    for (int i = 1; i < argc; i++) {
        string s = argv[i];
        size_t p = s.find('=');
        if (p != string::npos) args[s.substr(0, p)] = s.substr(p + 1);
    }
    try {
        string dir = arg("dir"), info = arg("info"), data = arg("data");
        string path_data = redutilcu::file::combine_path(dir, data);
        string path_info = redutilcu::file::combine_path(dir, info);
        var_t thr[THRESHOLD_N] = {0.0, 0.0, 0.0};
        thr[THRESHOLD_HIT_CENTRUM_DISTANCE] = atof(arg("hc", "0").c_str());
        thr[THRESHOLD_EJECTION_DISTANCE] = atof(arg("ej", "0").c_str());
        thr[THRESHOLD_RADII_ENHANCE_FACTOR] = atof(arg("factor", "0").c_str());
        string gas = arg("gas");
        gas_disk_model_t gdm = gas.empty() ? GAS_DISK_MODEL_NONE : GAS_DISK_MODEL_ANALYTIC;
        const bool gpu = arg("dev", "cpu") == "gpu";
        const computing_device_t cdev = gpu ? COMPUTING_DEVICE_GPU : COMPUTING_DEVICE_CPU;
        pp_disk* ppd = new pp_disk(path_data, path_info, gdm, 0, cdev, thr);
        if (!gas.empty()) {
            string gdir = arg("gasdir");
            ppd->a_gd = new analytic_gas_disk(gdir, gas, false);
            ppd->a_gd->calc(ppd->get_mass_of_star());
        }
        if (gpu) {
            // options::create_pp_disk (options.cpp:239-242), then run_simulation's
            // thread-per-block search (main.cu:449-463)
            ppd->copy_to_device();
            const int tpb = atoi(arg("tpb", "0").c_str());
            ppd->set_n_tpb(tpb > 0 ? (uint32_t)tpb : ppd->benchmark(false));
        }
        string mode = arg("mode", "run");
        FILE* f = fopen(arg("out").c_str(), "wb");
        if (!f && mode != "dump") throw string("cannot open out");
        const uint32_t n = ppd->n_bodies->get_n_total_playing();

        if (mode == "accel" && gpu) {
            // red's calc_dydx(1, ...) on the device: the SI, NSI and NI launches of
            // calc_grav_accel_naive, then calc_drag_accel_NSI (pp_disk.cu:1450-1502, 1014-1060)
            vector<var4_t> a(n);
            var_t t = atof(arg("t", "0").c_str());
            var4_t* d_dy = 0;
            if (cudaMalloc((void**)&d_dy, n * sizeof(var4_t)) != cudaSuccess) throw string("cudaMalloc");
            cudaMemset(d_dy, 0, n * sizeof(var4_t));
            ppd->calc_dydx(1, 0, t, ppd->sim_data->y[0], ppd->sim_data->y[1], d_dy);
            if (cudaMemcpy(&a[0], d_dy, n * sizeof(var4_t), cudaMemcpyDeviceToHost) != cudaSuccess)
                throw string("cudaMemcpy");
            int grav_ok = 1;
            put(f, &grav_ok, 4);
            put(f, &a[0], n * sizeof(var4_t));
        } else if (mode == "accel") {
            // gravity through red's CPU path (SI symmetric + NI), then drag on the NSI bodies
            vector<var4_t> a(n), d(n);
            var_t t = atof(arg("t", "0").c_str());
            memset(&a[0], 0, n * sizeof(var4_t));
            memset(&d[0], 0, n * sizeof(var4_t));
            int grav_ok = 1;
            if (ppd->n_bodies->get_n_NSI() == 0) {
                ppd->cpu_calc_grav_accel(t, ppd->sim_data->h_y[0], ppd->sim_data->h_y[1], &a[0]);
            } else {
                grav_ok = 0;
            }
            if (!gas.empty()) {
                interaction_bound b = ppd->n_bodies->get_bound_GD();
                ppd->cpu_calc_drag_accel_NSI(t, b, ppd->sim_data->h_body_md, ppd->sim_data->h_p,
                                             ppd->sim_data->h_y[0], ppd->sim_data->h_y[1], &d[0]);
            }
            put(f, &grav_ok, 4);
            put(f, &a[0], n * sizeof(var4_t));
            put(f, &d[0], n * sizeof(var4_t));
        } else if (mode == "run") {
            int kind = atoi(arg("integrator", "4").c_str());
            bool adaptive = atoi(arg("adaptive", "0").c_str()) != 0;
            var_t tol = atof(arg("tol", "1e-10").c_str());
            int nsteps = atoi(arg("nsteps", "1").c_str());
            integrator* ig = 0;
            if (kind == 1) ig = new euler(ppd, ppd->dt, cdev);
            else if (kind == 2) ig = new rungekutta2(ppd, ppd->dt, cdev);
            else if (kind == 4) ig = new rungekutta4(ppd, ppd->dt, adaptive, tol, cdev);
            else ig = new rungekutta8(ppd, ppd->dt, adaptive, tol, cdev);
            ig->error_check_for_tp = atoi(arg("eftp", "0").c_str()) != 0;
            put(f, &nsteps, 4);
            // the step loop's wall time (dev=gpu: every launch of red's path ends in a
            // device synchronisation, red_macro.h:33, 62-90)
            if (gpu) cudaDeviceSynchronize();
            const auto t_start = std::chrono::steady_clock::now();
            double t_steps = 0.0;
            for (int s = 0; s < nsteps; s++) {
                ttt_t dt = ig->step();
                ttt_t dtn = ig->get_dt_next();
                uint64_t c[3] = {ig->get_n_tried_step(), ig->get_n_passed_step(), ig->get_n_failed_step()};
                put(f, &ppd->t, 8);
                put(f, &dt, 8);
                put(f, &dtn, 8);
                put(f, c, 24);
            }
            if (gpu) cudaDeviceSynchronize();
            t_steps = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
            if (!arg("tout").empty()) {
                FILE* ft = fopen(arg("tout").c_str(), "w");
                if (!ft) throw string("cannot open tout");
                fprintf(ft, "%.9f %u\n", t_steps, (unsigned)ppd->n_tpb);
                fclose(ft);
            }
            if (gpu) ppd->copy_to_host();
            put_state(f, ppd);
            pp_disk_t::integral_t I;
            ppd->calc_integral(false, I);
            put(f, &I, sizeof(I));
        } else if (mode == "coll" && gpu) {
            // red's GPU check (pp_disk.cu:320-371, 1203-1218): the caller has counted the
            // pairs beforehand, so the unchecked event buffer of n records
            // (pp_disk.cu:1623-1628) holds them
            ppd->t = atof(arg("t", "0").c_str());
            ppd->check_for_collision();
            ppd->copy_event_data_to_host();
            vector<pp_disk_t::event_data_t> raw(ppd->events, ppd->events + ppd->event_counter);
            put_events(f, raw);
        } else if (mode == "coll") {
            ppd->t = atof(arg("t", "0").c_str());
            ppd->check_for_collision();
            vector<pp_disk_t::event_data_t> raw(ppd->events, ppd->events + ppd->event_counter);
            put_events(f, raw);
            if (ppd->event_counter) ppd->handle_collision();
            put_events(f, ppd->sp_events);
            put_state(f, ppd);
        } else if (mode == "ejhc") {
            ppd->t = atof(arg("t", "0").c_str());
            ppd->check_for_ejection_hit_centrum();
            vector<pp_disk_t::event_data_t> raw(ppd->events, ppd->events + ppd->event_counter);
            put_events(f, raw);
            if (ppd->event_counter) ppd->handle_ejection_hit_centrum();
            put_state(f, ppd);
            ppd->rebuild_vectors();
            put_state(f, ppd);
        } else if (mode == "integral") {
            pp_disk_t::integral_t I;
            ppd->calc_integral(false, I);
            put(f, &I, sizeof(I));
        } else if (mode == "dump") {
            string odir = arg("odir");
            string pa = redutilcu::file::combine_path(odir, "ref_data.txt");
            string pai = redutilcu::file::combine_path(odir, "ref_data.info.txt");
            string pb = redutilcu::file::combine_path(odir, "ref_data.dat");
            string pbi = redutilcu::file::combine_path(odir, "ref_data.info.dat");
            ppd->print_data(pa, DATA_REPRESENTATION_ASCII);
            ppd->print_data_info(pai, DATA_REPRESENTATION_ASCII);
            ppd->print_data(pb, DATA_REPRESENTATION_BINARY);
            ppd->print_data_info(pbi, DATA_REPRESENTATION_BINARY);
        } else {
            throw string("unknown mode");
        }
        if (f) fclose(f);
        // ppd is not deleted: pp_disk's destructor frees device vectors that a
        // CPU-only instance never allocated (util.cu:292-300 via pp_disk.cu:1577-1586).
    } catch (const string& msg) {
        fprintf(stderr, "Error: %s\n", msg.c_str());
        return 2;
    }
    return 0;
}
