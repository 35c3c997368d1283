// ebb_reconstruct.cpp -- command-line driver with ebb-reconstruct's interface
// (app/reconstruct.d:236-424):
//
//   ebb-reconstruct config.json save_N_0.esln [save_N_1.esln ...] [--precision fp64|split] [--device K]
//
// Reads the config and the mesh it names (relative to the config's directory), loads
// the solution files (one per rank of the saving run, cells placed by global id),
// and writes recon_<mesh name>.mmsh and recon_save_<N>.esln in the working directory.
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/ebb_gb300.h"

namespace {

// trailing number of "..._<k>.esln" (the rank), the reference's sort key
long rank_of(const std::string &f)
{
    std::string b = f;
    if (b.size() >= 5 && b.compare(b.size() - 5, 5, ".esln") == 0) b.resize(b.size() - 5);
    const size_t u = b.rfind('_');
    return std::strtol(b.c_str() + (u == std::string::npos ? 0 : u + 1), nullptr, 10);
}

std::vector<std::string> split(const std::string &s, char c)
{
    std::vector<std::string> out;
    size_t a = 0;
    for (;;) {
        size_t b = s.find(c, a);
        out.push_back(s.substr(a, b == std::string::npos ? std::string::npos : b - a));
        if (b == std::string::npos) return out;
        a = b + 1;
    }
}

int fail(const char *what, const char *detail)
{
    std::printf("Solver encountered an error: %s%s%s\n", what, detail && detail[0] ? ": " : "", detail ? detail : "");
    return 1;
}

}  // namespace

int main(int argc, char **argv)
{
    std::vector<std::string> pos;
    int precision = EBB_PREC_FP64, device = 0;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        if (a == "--precision" && i + 1 < argc)
            precision = std::string(argv[++i]) == "split" ? EBB_PREC_SPLIT : EBB_PREC_FP64;
        else if (a == "--device" && i + 1 < argc)
            device = std::atoi(argv[++i]);
        else
            pos.push_back(a);
    }
    if (pos.size() < 2) {
        std::printf("Not enough input arguments\nUsage: ebb-reconstruct configFile save_#_*\n");
        return 255;
    }
    const std::string cfg_file = pos[0];
    std::vector<std::string> sln(pos.begin() + 1, pos.end());
    std::stable_sort(sln.begin(), sln.end(), [](const std::string &a, const std::string &b) { return rank_of(a) < rank_of(b); });
    const std::vector<std::string> parts = split(sln[0], '_');
    const std::string save_num = parts.size() >= 2 ? parts[parts.size() - 2] : "0";
    std::printf("saveNum: %s\n", save_num.c_str());

    std::ifstream f(cfg_file);
    if (!f) return fail("cannot read", cfg_file.c_str());
    std::stringstream ss;
    ss << f.rdbuf();
    ebb_config cfg;
    char err[512] = {0};
    if (ebb_config_parse(ss.str().c_str(), &cfg, err, sizeof err)) return fail("config", err);
    // the mesh path is relative to the config file's directory (reconstruct.d:265-273)
    char absbuf[PATH_MAX];
    std::string dir = ".";
    if (realpath(cfg_file.c_str(), absbuf)) {
        dir = absbuf;
        dir = dir.substr(0, dir.rfind('/'));
    }
    const std::string mesh_file = dir + "/" + cfg.mesh_file;
    ebb_set_device(device);
    ebb_mesh *mesh = nullptr;
    if (ebb_mesh_import(mesh_file.c_str(), &mesh, err, sizeof err)) return fail("mesh", err);
    ebb_solver *s = nullptr;
    if (ebb_solver_create(mesh, &cfg, precision, &s, err, sizeof err)) {
        ebb_mesh_free(mesh);
        return fail("setup", err);
    }
    std::vector<const char *> paths;
    for (const std::string &p : sln) paths.push_back(p.c_str());
    int rc = 0;
    if (ebb_load_solution_parts(s, (int32_t)paths.size(), paths.data())) {
        rc = fail("Failed to load solution file", sln[0].c_str());
    } else {
        double t = 0, dt = 0;
        int64_t it = 0, n = 0;
        ebb_get_time(s, &t, &dt, &it);
        const std::string base = split(std::string(cfg.mesh_file), '.')[0];
        const std::string mmsh = "recon_" + base + ".mmsh", esln = "recon_save_" + save_num + ".esln";
        const int r = ebb_reconstruct(s, mesh, mmsh.c_str(), esln.c_str(), t, dt, nullptr, &n);
        if (r) {
            char msg[256] = {0};
            int32_t kind = 0;
            int64_t idx = -1;
            ebb_last_error(s, &kind, &idx, msg, sizeof msg);
            rc = fail("reconstruction failed", msg);
        } else {
            std::printf("wrote %s and %s (%lld points)\nexiting\n", mmsh.c_str(), esln.c_str(), (long long)n);
        }
    }
    ebb_solver_destroy(s);
    ebb_mesh_free(mesh);
    return rc;
}
