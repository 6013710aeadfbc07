/*
 * accel_main.cpp -- drop-in for the reference's accel binary
 * (src/gpu/main.cpp:61-327): same flags, same files, same exit codes.
 *
 *   accel [-i input.xml] [-d data.xml] [-o output.xml] [-g gpuspec]
 *         [-hs f|d] [-ds f|d] [-dt f|d] [-S n] [-F seed] [-q] [-v]
 *         [--list-devices] [-h]
 *
 * One estimation at a time, through the C ABI of libpcs.so.  Differences
 * from the reference, all deliberate:
 *   -g    the first listed device is used (one GPU); its queue count sets the
 *         number of proposal batches in flight.  Further devices are ignored
 *         with a note.
 *   -ds d the forward model computes in float only; "-ds d" is rejected.
 *   -hs   the population is always kept in double; "-hs f" is accepted and
 *         noted.
 *   -F n  seeds the random streams with n (the reference passes the flag's
 *         boolean instead of n, main.cpp:93-98, so every -F run used seed 1).
 * On failure it prints "Top-level exception: <type>" and the messages and
 * returns 1, as main.cpp:143-159 does.
 */
#include <unistd.h>

#include <chrono>
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <random>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/pcs.h"

namespace {

struct Config {
    bool list_devices = false;
    std::string input = "./input.xml";
    std::string data;
    std::string output;
    char host_scalar = 'd', dev_scalar = 'f', dist_type = 'f';
    int verbosity = 0;
    std::string gpu_spec = "1/30";
    unsigned long max_iter = 0;
    bool fixed_seed = false;
    uint32_t seed_value = 0;
};

struct CliError : std::runtime_error {
    std::string type;
    CliError(const std::string& t, const std::string& m) : std::runtime_error(m), type(t) {}
};

void help(FILE* f, const char* self)
{
    std::fprintf(f, "Synopsis: %s [--flags...]\n\n", self);
    std::fprintf(f,
                 "Flags:\n"
                 "  --input, -i file         : select input XML file\n"
                 "  --data, -d file          : override data XML file location(*)\n"
                 "  --output, -o file        : override output XML file destination(*)\n"
                 "\n"
                 "  --gpus, -g gpuspec       : select GPU and queues\n"
                 "\n"
                 "  --host-scalar, -hs {f,d} : select host code scalar type (float or double)\n"
                 "  --dev-scalar, -ds {f,d}  : select device code scalar type (float or double)\n"
                 "  --dist-type, -dt {f,d}   : select distance type (float or double)\n"
                 "\n"
                 "  --max-steps, -S n        : abort after n steps\n"
                 "  --fixed-seed, -F n       : use a fixed seed n for random number generation\n"
                 "\n"
                 "  --quiet, -q              : decrease verbosity\n"
                 "  --verbose, -v            : increase verbosity (repeat for further increases)\n"
                 "\n"
                 "  --help, -h               : print this help and exit\n"
                 "  --list-devices           : list compute devices and exit\n");
    std::fprintf(f,
                 "\ngpuspec is a comma separated list of GPU IDs (as shown by --list-devices).\n"
                 "Optionally, a queue count can be added to each GPU ID by appending a \"/N\".\n"
                 "accel runs on the first listed GPU.\n"
                 "\n(*) If specified, the -d/-o options override the paths given in the input XML\n"
                 "    for the data and for the output XML, respectively.\n");
}

Config parse(int argc, char** argv)
{
    Config c;
    for (int a = 1; a < argc; ++a) {
        auto flag = [&](const char* m, const char* alt = nullptr) {
            return std::strcmp(m, argv[a]) == 0 || (alt && std::strcmp(alt, argv[a]) == 0);
        };
        auto arg = [&](const char* m, const char* alt, std::string& out) {
            if (!flag(m, alt)) return false;
            if (a + 1 >= argc) throw CliError("std::runtime_error", std::string("Command line argument ") + argv[a] + " requires an additional argument");
            out = argv[++a];
            return true;
        };
        auto scalar = [&](char& out) {
            if (a + 1 >= argc) throw CliError("std::runtime_error", std::string("Command line argument ") + argv[a] + " requires an additional argument f or d");
            if (std::strcmp(argv[a + 1], "f") == 0)
                out = 'f';
            else if (std::strcmp(argv[a + 1], "d") == 0)
                out = 'd';
            else
                throw CliError("std::runtime_error", std::string("Scalar type must be either 'f' (float) or 'd' (double) and not '") + argv[a + 1] + "'");
            ++a;
        };
        if (flag("--help", "-h")) {
            help(stdout, argv[0]);
            std::exit(0);
        } else if (flag("--quiet", "-q")) {
            --c.verbosity;
        } else if (flag("--verbose", "-v")) {
            ++c.verbosity;
        } else if (arg("--input", "-i", c.input)) {
        } else if (arg("--data", "-d", c.data)) {
        } else if (arg("--output", "-o", c.output)) {
        } else if (arg("--gpus", "-g", c.gpu_spec)) {
        } else if (flag("--host-scalar", "-hs")) {
            scalar(c.host_scalar);
        } else if (flag("--dev-scalar", "-ds")) {
            scalar(c.dev_scalar);
        } else if (flag("--dist-type", "-dt")) {
            scalar(c.dist_type);
        } else if (flag("--max-steps", "-S")) {
            if (a + 1 >= argc) throw CliError("std::runtime_error", std::string("Command line argument ") + argv[a] + " requires an additional integer argument");
            char dummy;
            if (std::sscanf(argv[a + 1], "%lu%c", &c.max_iter, &dummy) != 1)
                throw CliError("std::runtime_error", std::string("Command line argument ") + argv[a] + " requires an additional positive integer argument and not " + argv[a + 1]);
            ++a;
        } else if (flag("--fixed-seed", "-F")) {
            if (a + 1 >= argc) throw CliError("std::runtime_error", std::string("Command line argument ") + argv[a] + " requires an additional integer argument");
            char dummy;
            unsigned v = 0;
            if (std::sscanf(argv[a + 1], "%u%c", &v, &dummy) != 1)
                throw CliError("std::runtime_error", std::string("Command line argument ") + argv[a] + " requires an additional integer argument and not " + argv[a + 1]);
            c.seed_value = v;
            c.fixed_seed = true;
            ++a;
        } else if (flag("--list-devices")) {
            c.list_devices = true;
        } else {
            throw CliError("std::runtime_error", std::string("Unknown command line argument '") + argv[a] + "'");
        }
    }
    return c;
}

/* gpuspec "dev[/queues],..." (detail/simulation_impl.inl:631-682), 1-based ids */
std::pair<int, int> parse_gpuspec(const std::string& spec, int verbosity)
{
    int first_dev = -1, first_q = 1, count = 0;
    const char* s = spec.c_str();
    while (s) {
        unsigned dev = 0, q = 1;
        int r = std::sscanf(s, "%u/%u", &dev, &q);
        if (r != 1 && r != 2) throw CliError("error::InvalidGPUSpec", "Don't understand provided gpuspec");
        if (dev == 0) throw CliError("error::InvalidGPUSpec", "GPU ids in gpuspec start at 1");
        if (count == 0) {
            first_dev = (int)dev - 1;
            first_q = (int)(q ? q : 1);
        } else if (verbosity >= 0) {
            std::fprintf(stderr, "Note: accel uses one GPU; ignoring GPU %u in gpuspec\n", dev);
        }
        ++count;
        const char* x = std::strchr(s, ',');
        s = x ? x + 1 : nullptr;
    }
    if (count == 0) throw CliError("error::InvalidGPUSpec", "No GPU queues were created! Check gpuspec.");
    return {first_dev, first_q};
}

void list_devices()
{
    std::vector<char> buf(1 << 16);
    pcs_device_report(buf.data(), buf.size());
    std::fputs(buf.data(), stdout);
}

void fail(pcs_status s, const char* what)
{
    if (s == PCS_OK) return;
    std::string type = "error::RuntimeError";
    const char* msg = pcs_last_error();
    if (s == PCS_ERR_XML) type = "error::XMLLoadError";
    if (s == PCS_ERR_CUDA || s == PCS_ERR_DEVICE) type = "error::CudaError";
    throw CliError(type, std::string(what) + ": " + pcs_status_string(s) + ": " + msg);
}

std::string now_str(std::chrono::system_clock::time_point t)
{
    std::time_t tt = std::chrono::system_clock::to_time_t(t);
    char buf[256];
    std::strftime(buf, 255, "%F %T%z", std::localtime(&tt));
    return buf;
}

} // namespace

int main(int argc, char** argv)
{
    try {
        Config cfg = parse(argc, argv);
        if (cfg.list_devices) {
            list_devices();
            return 0;
        }
        if (cfg.dev_scalar == 'd')
            throw CliError("std::runtime_error", "Device scalar type double is not supported (the forward model computes in float)");
        if (cfg.host_scalar == 'f' && cfg.verbosity >= 0)
            std::fprintf(stderr, "Note: -hs f accepted; the population is kept in double\n");
        const auto gs = parse_gpuspec(cfg.gpu_spec, cfg.verbosity);

        pcs_input* in = nullptr;
        fail(pcs_input_load(cfg.input.c_str(), cfg.data.empty() ? nullptr : cfg.data.c_str(), &in), "input::load");
        pcs_params params;
        pcs_observed obs;
        const char* out_path = nullptr;
        fail(pcs_input_params(in, &params, &obs, &out_path), "input");
        std::string output_path = cfg.output.empty() ? std::string(out_path) : cfg.output;
        params.distance_double = cfg.dist_type == 'd' ? 1 : 0;

        uint64_t seed;
        if (cfg.fixed_seed) {
            seed = cfg.seed_value;
        } else {
            std::random_device rd;
            seed = ((uint64_t)rd() << 32) ^ rd();
        }

        pcs_ctx* ctx = nullptr;
        fail(pcs_open(gs.first, gs.second, &ctx), "open");
        pcs_job* job = nullptr;
        fail(pcs_job_create(ctx, &params, &obs, seed, &job), "make_simulation");
        if (cfg.verbosity >= 0) std::printf("Begin main iterations...\n");

        const auto start = std::chrono::system_clock::now();
        fail(pcs_job_run(job, (uint32_t)cfg.max_iter), "run");
        const auto end = std::chrono::system_clock::now();

        pcs_job_info info{};
        fail(pcs_job_info_get(job, &info), "info");
        const size_t N = info.abc_sample_count, C = info.component_count, Z = info.z_component_count;
        std::vector<double> m(N * C), s(N * C), c(N * C), az(N * Z), dist(N), w(N);
        fail(pcs_job_output(job, m.data(), s.data(), c.data(), az.data(), dist.data(), w.data()), "output");
        if (cfg.verbosity >= 0)
            std::printf("Done: %u iterations, %" PRIu64 " simulations, gamma = %g, converged = %s\n", info.iterations,
                        info.simulations, info.gamma, info.converged ? "true" : "false");

        /* meta (detail/simulation_impl.inl:483-497, main.cpp:106-134) */
        char host[256] = {};
        std::vector<std::pair<std::string, std::string>> meta = {
            {"simulator", "gpu"},
            {"iterations", std::to_string(info.iterations)},
            {"simulations", std::to_string(info.simulations)},
            {"gpus", "1"},
            {"gpu0_id", std::to_string(gs.first + 1)},
            {"gpu0_queues", std::to_string(gs.second)},
            {"hostScalarType", "d"},
            {"deviceScalarType", "f"},
            {"distanceType", cfg.dist_type == 'd' ? "d" : "f"},
            {"runtime_ms", std::to_string((unsigned long long)std::chrono::duration_cast<std::chrono::milliseconds>(end - start).count())},
            {"started_at", now_str(start)},
            {"finished_at", now_str(end)},
        };
        if (::gethostname(host, 255) == 0) meta.push_back({"machine", host});
#ifdef NDEBUG
        meta.push_back({"debug", "false"});
#else
        meta.push_back({"debug", "true"});
#endif
        meta.push_back({"input_file", cfg.input});
        if (!cfg.data.empty()) meta.push_back({"data_file", cfg.data});
        std::vector<pcs_output_meta> mv;
        for (auto& kv : meta) mv.push_back(pcs_output_meta{kv.first.c_str(), kv.second.c_str()});
        const bool lognormal = params.model == PCS_MODEL_LOGNORMAL;
        fail(pcs_output_write(output_path.c_str(), params.model, params.weighting_scheme, N, C, Z, mv.data(), mv.size(),
                              (int)info.converged, info.gamma, m.data(), m.size(), lognormal ? s.data() : nullptr,
                              lognormal ? s.size() : 0, c.data(), c.size(), az.data(), az.size(), dist.data(), dist.size(),
                              w.data(), w.size()),
             "output::write");
        pcs_job_destroy(job);
        pcs_close(ctx);
        pcs_input_free(in);
        return 0;
    } catch (const CliError& e) {
        std::fprintf(stderr, "Top-level exception: %s\n", e.type.c_str());
        std::fprintf(stderr, "  - %s\n", e.what());
        return 1;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "Top-level exception: std::exception\n");
        std::fprintf(stderr, "  - %s\n", e.what());
        return 1;
    }
}
