// rrsph_run — runs an experiment directory with the GPU step, the way RRSPH's
// main() runs the experiment and dump layer the user picks (sources/SPH.cpp:49-74,
// RRSPH_COMMON/src/CLI.cpp:13-46), without the interactive prompts.
//
//   rrsph_run <experiment_dir> [--dump <layer.csv>] [--precision fp64|mixed]
//             [--max-steps N]
//
// The start layer defaults to the latest dump/<t>.csv. Layers are written to
// <experiment_dir>/data and <experiment_dir>/dump as the reference does.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <string>
#include <vector>

#include "../../include/rrsph_cuda.h"

namespace fs = std::filesystem;

static int fail(const char* what) {
    std::fprintf(stderr, "rrsph_run: %s: %s\n", what, rrsph_last_error());
    return 1;
}

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s <experiment_dir> [--dump <layer.csv>] [--precision fp64|mixed] [--max-steps N]\n",
                     argv[0]);
        return 2;
    }
    const fs::path dir = argv[1];
    std::string dump;
    int precision = RRSPH_PRECISION_MIXED;
    uint64_t max_steps = UINT64_MAX;
    for (int i = 2; i < argc; i++) {
        if (!std::strcmp(argv[i], "--dump") && i + 1 < argc) dump = argv[++i];
        else if (!std::strcmp(argv[i], "--precision") && i + 1 < argc) {
            const std::string v = argv[++i];
            precision = v == "fp64" ? RRSPH_PRECISION_FP64 : RRSPH_PRECISION_MIXED;
        } else if (!std::strcmp(argv[i], "--max-steps") && i + 1 < argc) {
            max_steps = std::strtoull(argv[++i], nullptr, 10);
        } else {
            std::fprintf(stderr, "rrsph_run: unknown argument %s\n", argv[i]);
            return 2;
        }
    }
    rrsph_params p;
    if (rrsph_params_defaults(&p) || rrsph_experiment_load_params(dir.c_str(), &p)) return fail("params");
    if (dump.empty()) {  // the latest dump layer
        double best = -1;
        std::error_code ec;
        for (const auto& e : fs::directory_iterator(dir / "dump", ec)) {
            if (e.path().extension() != ".csv") continue;
            double t;
            if (rrsph_layer_time_from_path(e.path().c_str(), &t) == RRSPH_OK && t > best) {
                best = t;
                dump = e.path().string();
            }
        }
        if (dump.empty()) {
            std::fprintf(stderr, "rrsph_run: no dump layer in %s/dump\n", dir.c_str());
            return 1;
        }
    }
    if (rrsph_layer_time_from_path(dump.c_str(), &p.start_simulation_time)) return fail("dump name");
    const size_t n = p.ntotal, dim = p.dim;
    std::vector<double> r(n * dim), v(n * dim), rho(n), pres(n);
    std::vector<int32_t> itype(n);
    if (rrsph_layer_read(dump.c_str(), &p, r.data(), (uint32_t)dim, v.data(), rho.data(), pres.data(), itype.data()))
        return fail("dump layer");
    if (rrsph_params_derive(&p, r.data(), (uint32_t)dim)) return fail("derive");
    rrsph_solver* s = nullptr;
    if (rrsph_create(&p, precision, &s)) return fail("create");
    if (rrsph_upload(s, r.data(), (uint32_t)dim, v.data(), rho.data(), nullptr, itype.data())) return fail("upload");
    double t = p.start_simulation_time;
    uint64_t steps = 0;
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = rrsph_run(s, dir.c_str(), &t, max_steps, &steps);
    const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("rrsph_run: %s, %zu particles, %llu steps, t = %.6f s, wall %.3f s (%s)\n",
                precision == RRSPH_PRECISION_FP64 ? "fp64" : "mixed", n, (unsigned long long)steps, t, wall,
                rc ? rrsph_last_error() : "ok");
    rrsph_destroy(s);
    return rc ? 1 : 0;
}
