// initial_harness.cu -- drives the reference's own initial-condition generator
// (TEST INFRASTRUCTURE).
//
// Built by oracle/ref_build.sh from the unmodified sources of suliaron/red.cuda
// (src/red.cuda.initial: distribution.cpp, util_init.cpp, nebula.cpp and the
// functions of main.cu, which this unit includes with its main() renamed).  It
// reads a disk specification, builds red's body_disk_t from it exactly as
// red's scenario functions do (one distribution object per drawn quantity,
// each with its own seed: e.g. set_parameters::n_pl, main.cu:1059-1112), and
// runs red's own pipeline of such a scenario (main.cu:2741-2800):
// populate_disk (main.cu:251-314), the radius / density fix-up, calculate_phase
// (main.cu:317-342), tools::transform_to_bc, transform_time and
// transform_velocity.  The resulting records go to a raw file that
// tests/golden/make_golden.py stores as a fixture.
//
// usage: initial_harness <spec file> <out file>
// spec lines:
//   n <body type> <count>
//   pp <body type> <mass|radius|density|cd> <distribution> <seed> <parameters...>
//   oe <body type> <sma|ecc|inc|peri|node|mean> <distribution> <seed> <parameters...>
// distributions: uniform x_min x_max | rayleigh sigma | power x_min x_max power |
//                exponential lambda | normal mean variance
#define main red_initial_main
#include "main.cu"
#undef main

#include <cstdio>
#include <fstream>
#include <sstream>

static distribution_base* make_dist(const std::string& kind, uint32_t seed, std::istringstream& in)
{
    double a = 0.0, b = 0.0, c = 0.0;
    if (kind == "uniform") {
        in >> a >> b;
        return new uniform_distribution(seed, a, b);
    }
    if (kind == "rayleigh") {
        in >> a;
        return new rayleigh_distribution(seed, a);
    }
    if (kind == "power") {
        in >> a >> b >> c;
        return new power_law_distribution(seed, a, b, c);
    }
    if (kind == "exponential") {
        in >> a;
        return new exponential_distribution(seed, a);
    }
    if (kind == "normal") {
        in >> a >> b;
        return new normal_distribution(seed, a, b);
    }
    throw std::string("unknown distribution " + kind);
}

int main(int argc, char** argv)
{
    if (argc < 3) {
        fprintf(stderr, "usage: initial_harness <spec> <out>\n");
        return 1;
    }
    try {
        body_disk_t disk;
        std::ifstream f(argv[1]);
        if (!f) throw std::string("cannot open spec");
        std::string line;
        const char* pp_names[4] = {"mass", "radius", "density", "cd"};
        const char* oe_names[6] = {"sma", "ecc", "inc", "peri", "node", "mean"};
        while (std::getline(f, line)) {
            std::istringstream in(line);
            std::string what;
            if (!(in >> what)) continue;
            int type = 0;
            in >> type;
            if (what == "n") {
                in >> disk.nBody[type];
                continue;
            }
            std::string item, kind;
            uint32_t seed = 0;
            in >> item >> kind >> seed;
            if (what == "pp") {
                int k = -1;
                for (int q = 0; q < 4; q++)
                    if (item == pp_names[q]) k = q;
                if (k < 0) throw std::string("unknown physical property " + item);
                disk.pp_d[type].item[k] = make_dist(kind, seed, in);
            } else if (what == "oe") {
                int k = -1;
                for (int q = 0; q < 6; q++)
                    if (item == oe_names[q]) k = q;
                if (k < 0) throw std::string("unknown orbital element " + item);
                disk.oe_d[type].item[k] = make_dist(kind, seed, in);
            } else {
                throw std::string("bad spec line: " + line);
            }
        }
        const uint32_t n_body = calc_number_of_bodies(disk);
        disk.mig_type = new migration_type_t[n_body];
        disk.stop_at = new var_t[n_body];
        for (uint32_t i = 0; i < n_body; i++) {
            disk.mig_type[i] = MIGRATION_TYPE_NO;
            disk.stop_at[i] = 0.0;
        }
        ttt_t t0 = 0.0;
        pp_disk_t::sim_data_t* sd = new pp_disk_t::sim_data_t;
        allocate_host_storage(sd, n_body);
        populate_disk(t0, disk, sd);
        // the fix-up every scenario applies after populate_disk (main.cu:2764-2781)
        uint32_t bodyIdx = 0;
        for (int type = BODY_TYPE_STAR; type < BODY_TYPE_N; type++) {
            for (unsigned int i = 0; i < disk.nBody[type]; i++, bodyIdx++) {
                if (sd->h_p[bodyIdx].mass > 0.0) {
                    if (disk.pp_d[type].item[DENSITY] == 0x0 && disk.pp_d[type].item[RADIUS] != 0x0)
                        sd->h_p[bodyIdx].density = tools::calc_density(sd->h_p[bodyIdx].mass, sd->h_p[bodyIdx].radius);
                    if (disk.pp_d[type].item[RADIUS] == 0x0 && disk.pp_d[type].item[DENSITY] != 0x0)
                        sd->h_p[bodyIdx].radius = tools::calc_radius(sd->h_p[bodyIdx].mass, sd->h_p[bodyIdx].density);
                }
            }
        }
        ttt_t dt = 0.0;
        calculate_phase(sd, n_body, dt);
        tools::transform_to_bc(n_body, sd);
        tools::transform_time(n_body, sd);
        tools::transform_velocity(n_body, sd);
        dt *= constants::Gauss;
        FILE* o = fopen(argv[2], "wb");
        if (!o) throw std::string("cannot open out");
        fwrite(&n_body, 4, 1, o);
        fwrite(&dt, 8, 1, o);
        fwrite(sd->h_y[0], sizeof(var4_t), n_body, o);
        fwrite(sd->h_y[1], sizeof(var4_t), n_body, o);
        fwrite(sd->h_p, sizeof(pp_disk_t::param_t), n_body, o);
        fwrite(sd->h_body_md, sizeof(pp_disk_t::body_metadata_t), n_body, o);
        fwrite(sd->h_oe, sizeof(orbelem_t), n_body, o);
        fclose(o);
    } catch (const std::string& msg) {
        fprintf(stderr, "Error: %s\n", msg.c_str());
        return 2;
    }
    return 0;
}
