// ebb_solve.cpp -- command-line driver with ebb-solve's interface (app/solver.d:430-470):
//
//   ebb-solve -c config.json [-s save_prefix] [--precision fp64|split|df] [--device N]
//
// Reads the JSON config and the gmsh mesh it names, runs the time loop of
// runIntegrator (app/solver.d:38-277) on the GPU through the C ABI, and writes what the
// reference writes: save_<k>_0.esln every saveIter iterations, final_0.esln, and
// boundaryForces.frc (big-endian f64 triples t, drag, lift per iteration).  -s P
// restarts from P + "0.esln" (rank 0's file, app/solver.d:455-458).  SIGINT and SIGUSR1
// stop the loop after the current chunk and still write the final solution.
#include <signal.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/ebb_gb300.h"

namespace {

volatile sig_atomic_t g_interrupted = 0;
void on_signal(int) { g_interrupted = 1; }

const char *flux_name(int f) { return f == EBB_FLUX_ROE ? "roeFlux" : "rusanovFlux"; }
const char *int_name(int i)
{
    switch (i) {
    case EBB_INT_RK2: return "RK2";
    case EBB_INT_RK2_TVD: return "RK2_TVD";
    case EBB_INT_RK4: return "RK4";
    default: return "Euler";
    }
}

void put_be(std::vector<unsigned char> &b, double d)
{
    uint64_t v;
    std::memcpy(&v, &d, 8);
    for (int k = 7; k >= 0; k--) b.push_back((unsigned char)(v >> (8 * k)));
}

int fail(const char *what, int code, ebb_solver *s)
{
    char msg[256] = {0};
    int32_t kind = 0;
    int64_t idx = -1;
    if (s) ebb_last_error(s, &kind, &idx, msg, sizeof msg);
    std::printf("Solver encountered an error: %s (status %d)%s%s", what, code, msg[0] ? ": " : "", msg);
    if (idx >= 0) std::printf(" [index %lld]", (long long)idx);
    std::printf("\n");
    return 1;
}

}  // namespace

int main(int argc, char **argv)
{
    std::string cfg_path, save_prefix;
    int precision = EBB_PREC_FP64, device = 0;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        auto next = [&]() -> std::string { return i + 1 < argc ? std::string(argv[++i]) : std::string(); };
        if (a == "-c" || a == "--config")
            cfg_path = next();
        else if (a == "-s" || a == "--save")
            save_prefix = next();
        else if (a == "--precision") {
            const std::string p = next();
            if (p == "fp64")
                precision = EBB_PREC_FP64;
            else if (p == "split")
                precision = EBB_PREC_SPLIT;
            else if (p == "df")
                precision = EBB_PREC_DF;
            else {
                std::fprintf(stderr, "unknown precision form '%s' (fp64, split or df)\n", p.c_str());
                return 2;
            }
        }
        else if (a == "--device")
            device = std::atoi(next().c_str());
        else {
            std::fprintf(stderr, "usage: ebb-solve -c config.json [-s save_prefix] [--precision fp64|split|df] [--device N]\n");
            return 2;
        }
    }
    if (cfg_path.empty()) {
        std::fprintf(stderr, "usage: ebb-solve -c config.json [-s save_prefix]\n");
        return 2;
    }
    signal(SIGINT, on_signal);
    signal(SIGUSR1, on_signal);
    const auto t_start = std::chrono::steady_clock::now();

    std::ifstream f(cfg_path);
    if (!f) {
        std::printf("Solver encountered an error: cannot read %s\n", cfg_path.c_str());
        return 1;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    ebb_config cfg;
    char err[512] = {0};
    int r = ebb_config_parse(ss.str().c_str(), &cfg, err, sizeof err);
    if (r) {
        std::printf("Solver encountered an error: %s\n", err);
        return 1;
    }
    ebb_set_device(device);
    ebb_mesh *mesh = nullptr;
    if ((r = ebb_mesh_import(cfg.mesh_file, &mesh, err, sizeof err))) {
        std::printf("Solver encountered an error: %s\n", err);
        return 1;
    }
    ebb_mesh_info info;
    ebb_mesh_get_info(mesh, &info);
    ebb_solver *s = nullptr;
    if ((r = ebb_solver_create(mesh, &cfg, precision, &s, err, sizeof err))) {
        std::printf("Solver encountered an error: %s\n", err);
        ebb_mesh_free(mesh);
        return 1;
    }
    if (!save_prefix.empty()) {
        std::string sf = save_prefix + "0.esln";
        if ((r = ebb_load_solution(s, sf.c_str()))) {
            std::printf("Solver encountered an error: Failed to load solution %s\n", sf.c_str());
            return 1;
        }
    }
    std::printf("Running 2D finite volume solver\n-limited: %s\n-order: %lld\n-flux: %s\n-integrator: %s\n",
                cfg.limited ? "true" : "false", (long long)cfg.order, flux_name(cfg.flux), int_name(cfg.integrator));

    FILE *frc = std::fopen("boundaryForces.frc", "wb");
    std::vector<unsigned char> fbuf;
    const int64_t plot = cfg.plot_iter, save = cfg.save_iter;
    int64_t iterations = 0, save_k = 0;
    ebb_step_record last{};
    bool have_last = false;
    const auto t_solve = std::chrono::steady_clock::now();
    std::vector<ebb_step_record> rec(4096);
    int rc = 0;
    while (!g_interrupted) {
        // run up to the next iteration that prints or saves (at most 4096 steps per chunk)
        int64_t chunk = 4096;
        for (int64_t k = 0; k < chunk; k++) {
            int64_t it = iterations + k;
            if ((plot > 0 && it % plot == 0) || (save > 0 && it % save == 0)) {
                chunk = k + 1;
                break;
            }
        }
        int64_t n = 0;
        r = ebb_run(s, chunk, rec.data(), &n);
        for (int64_t k = 0; k < n; k++) {
            const ebb_step_record &R = rec[k];
            const int64_t it = iterations + k;
            put_be(fbuf, R.t);
            put_be(fbuf, R.drag);
            put_be(fbuf, R.lift);
            if (plot > 0 && it % plot == 0) {
                std::printf("lift force = %f\t drag force = %f\t t = %f\n", R.lift, R.drag, R.t);
                std::printf("rho_RMS = %.10e\tu_RMS = %.10e\tv_RMS = %.10e\tE_RMS = %.10e\tFlux_R = %.10e\t dt = %10.10f\n",
                            R.resid[0], R.resid[1], R.resid[2], R.resid[3], R.rmax, R.dt);
            }
            last = R;
            have_last = true;
        }
        if (r) {
            rc = fail("solver step failed", r, s);
            break;
        }
        if (n > 0 && save > 0 && (iterations + n - 1) % save == 0) {
            char name[64];
            std::snprintf(name, sizeof name, "save_%lld_0.esln", (long long)save_k++);
            if (ebb_save_solution(s, name, last.t, last.dt)) rc = fail("saving a solution failed", EBB_ERR_IO, s);
        }
        iterations += n;
        if (n < chunk) break;  // t reached tEnd
    }
    const double elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_solve).count();
    if (frc) {
        std::fwrite(fbuf.data(), 1, fbuf.size(), frc);
        std::fclose(frc);
    }
    double t = 0, dt = 0;
    int64_t iters = 0;
    ebb_get_time(s, &t, &dt, &iters);
    if (ebb_save_solution(s, "final_0.esln", t, dt)) rc = fail("saving the final solution failed", EBB_ERR_IO, s);
    if (have_last) {
        std::printf("lift force = %f\t drag force = %f\t t = %f\n", last.lift, last.drag, t);
        std::printf("rho_RMS = %.10e\tu_RMS = %.10e\tv_RMS = %.10e\tE_RMS = %.10e\tFlux_R = %.10e\t dt = %10.10f\n",
                    last.resid[0], last.resid[1], last.resid[2], last.resid[3], last.rmax, dt);
    }
    std::printf("total solver time: %g s\n", elapsed);
    if (iterations > 0) {
        const double per_it = elapsed / (double)iterations;
        std::printf("average time per iteration: %g s\n", per_it);
        std::printf("average time per cell: %g us\n", per_it / (double)(info.n_cells + info.n_ghost) * 1e6);
    }
    std::printf("exiting\n");
    ebb_solver_destroy(s);
    ebb_mesh_free(mesh);
    std::printf("total run time: %g\n", std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count());
    return rc;
}
