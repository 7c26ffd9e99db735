// main_total_force.cpp -- drop-in replacement of the reference executable
// total_force_cuda.x (src/total_force_cuda.cpp:28-179): same config file,
// same per-step call order, same trajectory / restart / CV outputs, driven
// through the C ABI.  Steps without output run as captured CUDA graphs.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "isspa_gb300.h"

namespace {

int fail(const char *what, int rc) {
    std::fprintf(stderr, "%s: %s (%d)\n", what, isspa_strerror(rc), rc);
    return 1;
}

// atom_class.cpp:248-290: "%d\n%d\n" header, "C %10.6f %10.6f %10.6f\n" rows
void write_xyz(FILE *f, const std::vector<float> &v, int n) {
    if (!f) return;
    std::fprintf(f, "%d\n%d\n", n, n);
    for (int i = 0; i < n; ++i) std::fprintf(f, "C %10.6f %10.6f %10.6f\n", v[4 * i], v[4 * i + 1], v[4 * i + 2]);
    std::fflush(f);
}

// atom_class.cpp:259-268 (ISSPA_force.xyz): positions and the IS-SPA force
// buffer, which the reference zeroes every step and never fills
// (isspa_force_cuda.cu:343, :323-325).
void write_isspaf(FILE *f, const std::vector<float> &pos, int n) {
    if (!f) return;
    std::fprintf(f, "%d\n%d\n", n, n);
    for (int i = 0; i < n; ++i)
        std::fprintf(f, "C %10.6f %10.6f %10.6f %16.8e %16.8e %16.8e\n", pos[4 * i], pos[4 * i + 1], pos[4 * i + 2],
                     0.0, 0.0, 0.0);
    std::fflush(f);
}

// atom_class.cpp:292-328: 6F12.7 pairs of atoms, then the box line
void write_rst(const char *path, const char *title, const std::vector<float> &v, int n, float box) {
    FILE *f = std::fopen(path, "w");
    if (!f) return;
    std::fprintf(f, "%s\n%d\n", title, n);
    for (int i = 0; i < n; i += 2) {
        std::fprintf(f, "%12.7f%12.7f%12.7f", v[4 * i], v[4 * i + 1], v[4 * i + 2]);
        if (i + 1 < n) std::fprintf(f, "%12.7f%12.7f%12.7f\n", v[4 * i + 4], v[4 * i + 5], v[4 * i + 6]);
        else std::fprintf(f, "\n");
    }
    std::fprintf(f, "%12.7f%12.7f%12.7f%12.7f%12.7f%12.7f\n", box, box, box, 90.0, 90.0, 90.0);
    std::fclose(f);
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s config.txt\n", argv[0]);
        return 2;
    }
    isspa_run_config cfg;
    int rc = isspa_read_run_config(argv[1], &cfg);
    if (rc) return fail("reading config", rc);
    if (!cfg.pnu_set) std::printf("pnu not set in config: Andersen thermostat off (pnu = 0)\n");
    isspa_host_system *sys = nullptr;
    if ((rc = isspa_system_load(&cfg, nullptr, &sys))) return fail("reading inputs", rc);
    char cv_name[512] = {0};
    if (cfg.us == 1 && (rc = isspa_read_us_config(sys, cfg.us_cfg, cv_name, sizeof cv_name)))
        return fail("reading US config", rc);
    isspa_system_desc d;
    isspa_system_describe(sys, &d);
    isspa_engine *e = nullptr;
    if ((rc = isspa_engine_create(&d, 1, nullptr, &e))) return fail("creating engine", rc);
    if (cfg.n_steps >= 1000) {  // worth a fraction of a second: time the launch-shape candidates once
        int shape[ISSPA_SHAPE_COUNT];
        if ((rc = isspa_autotune(e, 3, shape))) return fail("autotuning", rc);
        std::printf("launch shapes: field split %d, force chunk %d points (last items %d), %d atom(s) per force thread, "
                    "step integrator %d, programmatic launches %d, fused field + force %d\n",
                    shape[0], shape[2], shape[8], shape[7], shape[11], shape[15], shape[16]);
    }
    const int n = d.n_atoms;
    std::vector<float> pos(4 * (size_t)n), vel(4 * (size_t)n), frc(4 * (size_t)n);
    FILE *ff = std::fopen(cfg.for_out, "w"), *fp = std::fopen(cfg.pos_out, "w"), *fv = std::fopen(cfg.vel_out, "w");
    FILE *fi = std::fopen("ISSPA_force.xyz", "w");
    FILE *fcv = cfg.us == 1 ? std::fopen(cv_name, "w") : nullptr;
    const int dw = cfg.delta_write > 0 ? cfg.delta_write : cfg.n_steps + 1;
    auto t0 = std::chrono::steady_clock::now();
    for (int step = 0; step < cfg.n_steps;) {
        if (step % dw == 0) {
            // output step: per-term calls in the reference order, then write
            if ((rc = isspa_zero_forces(e)) || (rc = bond_force_cuda(e, nullptr)) ||
                (rc = angle_force_cuda(e, nullptr)) || (rc = dih_force_cuda(e, nullptr)) ||
                (rc = isspa_force_cuda(e, nullptr)) || (rc = nonbond_force_cuda(e, nullptr)) ||
                (cfg.us == 1 && (rc = us_force_cuda(e, nullptr))))
                return fail("force step", rc);
            isspa_get_positions(e, pos.data(), n);
            isspa_get_velocities(e, vel.data(), n);
            isspa_get_forces(e, frc.data(), n);
            write_isspaf(fi, pos, n);
            write_xyz(ff, frc, n);
            write_xyz(fp, pos, n);
            write_xyz(fv, vel, n);
            if (fcv) {
                double cv = 0.0;
                isspa_get_us_com(e, nullptr, &cv);
                std::fprintf(fcv, "%8d  %8.3f\n", step, cv);  // us_class.cpp:132
                std::fflush(fcv);
            }
            if ((rc = leapfrog_cuda(e, nullptr))) return fail("leapfrog", rc);
            ++step;
            continue;
        }
        int run = dw - step % dw;
        if (step + run > cfg.n_steps) run = cfg.n_steps - step;
        if ((rc = isspa_step(e, run))) return fail("step", rc);
        step += run;
    }
    if ((rc = isspa_synchronize(e))) return fail("run", rc);
    auto t1 = std::chrono::steady_clock::now();
    isspa_get_positions(e, pos.data(), n);
    isspa_get_velocities(e, vel.data(), n);
    write_rst(cfg.pos_rst_file, "Restart Positions from ISSPA CUDA Code", pos, n, cfg.box);
    write_rst(cfg.vel_rst_file, "Restart Velocities from ISSPA CUDA Code", vel, n, cfg.box);
    const double ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    const double ns = cfg.n_steps * cfg.dt_ps * 1.0e-3;
    std::printf("Elapsed CPU/GPU time = %10.2f ms\n", ms);
    std::printf("Simulation time = %10.2f ns\n", ns);
    std::printf("Average ns/day = %10.2f\n", ns / (ms * 1e-3 / 86400.0));  // timing_class.cpp:57-58
    for (FILE *f : {ff, fp, fv, fi, fcv})
        if (f) std::fclose(f);
    isspa_engine_destroy(e);
    isspa_system_free(sys);
    return 0;
}
