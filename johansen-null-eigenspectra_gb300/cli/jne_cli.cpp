// jne_cli.cpp -- command-line driver with the reference's flags (cli.rs:56-132,
// main.rs:44-136): for every dim in [--dim-start, --dim-end] run the resumable
// simulation of every model of --model into data/eigenvalues_model*_dim*_steps*.dat
// (all models of a dim from one pass over the paths) and, unless --quiet, print
// the trace and max-eigenvalue percentile tables.
// The runs go to the GPU through the C ABI of libjne_gb300.so; --threads is
// accepted and validated as in the reference (it sized the CPU thread pool
// there and has no effect here).  Extra flags: --precision fp64|mixed,
// --device N, --data-dir D.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/jne.h"

namespace {

struct Config {
  long long threads = -1, steps = 10000, runs = 10000000, dim_start = 1, dim_end = 12;
  std::vector<int> models = {0, 1, 2, 3, 4};
  bool quiet = false;
  int precision = JNE_PREC_MIXED, device = 0;
  std::string data_dir = "data";
};

// JohansenModel's Display text (johansen_models.rs:54-68, 137-141)
const char* kModelNames[5] = {
    "Model 0: No intercept, no trend", "Model 1: Intercept, no trend, intercept in cointegration",
    "Model 2: Intercept, no trend, intercept not fully explained by cointegration",
    "Model 3: Intercept, trend, trend in cointegration",
    "Model 4: Intercept, trend, intercept and trend not fully explained by cointegration"};

std::string with_commas(long long v) {
  std::string s = std::to_string(v), out;
  int n = 0;
  for (auto it = s.rbegin(); it != s.rend(); ++it) {
    if (n && n % 3 == 0 && *it != '-') out.insert(out.begin(), ',');
    out.insert(out.begin(), *it);
    n++;
  }
  return out;
}

// cli.rs parse_next_arg: a non-negative integer, commas allowed
bool parse_count(int argc, char** argv, int i, const char* name, long long* out) {
  if (i + 1 >= argc) {
    std::fprintf(stderr, "Error: %s parameter requires a value\n", name);
    return false;
  }
  std::string s;
  for (const char* p = argv[i + 1]; *p; p++)
    if (*p != ',') s.push_back(*p);
  char* end = nullptr;
  const long long v = s.empty() || s[0] == '-' ? -1 : std::strtoll(s.c_str(), &end, 10);
  if (v < 0 || !end || *end) {
    std::fprintf(stderr, "Error: %s parameter must be a positive integer (commas allowed, e.g., 1,000,000)\n", name);
    return false;
  }
  *out = v;
  return true;
}

bool parse_models(const char* s, std::vector<int>* out) {
  out->clear();
  std::string part;
  for (const char* p = s;; p++) {
    if (*p == ',' || !*p) {
      size_t a = part.find_first_not_of(" \t"), b = part.find_last_not_of(" \t");
      if (a != std::string::npos) {
        const std::string t = part.substr(a, b - a + 1);
        char* end = nullptr;
        const long v = std::strtol(t.c_str(), &end, 10);
        if (*end || v < 0 || v > 4) {
          std::fprintf(stderr, "Error: invalid model number: %s\n", t.c_str());
          return false;
        }
        bool seen = false;  // a repeated model would only find its file complete
        for (int m : *out) seen = seen || m == (int)v;
        if (!seen) out->push_back((int)v);
      }
      part.clear();
      if (!*p) break;
    } else {
      part.push_back(*p);
    }
  }
  if (out->empty()) {
    std::fprintf(stderr, "Error: the model list must not be empty\n");
    return false;
  }
  return true;
}

void help(const char* prog) {
  std::printf("Johansen null-eigenspectra simulation (GB300 engine)\n\n");
  std::printf("Usage: %s [options]\n\nOptions:\n", prog);
  std::printf("  --threads <int>      accepted for compatibility; the runs go to the GPU (default: %u)\n",
              std::thread::hardware_concurrency());
  std::printf("  --steps <int>        number of simulation steps (default: 10,000)\n");
  std::printf("  --runs <int>         number of runs per model (default: 10,000,000)\n");
  std::printf("  --dim-start <int>    starting matrix dimension (default: 1)\n");
  std::printf("  --dim-end <int>      ending matrix dimension (default: 12)\n");
  std::printf("  --dim <int>          run a single dimension (sets start and end to the same value)\n");
  std::printf("  --model <list>       comma separated list of model numbers to compute (default: 0,1,2,3,4)\n");
  std::printf("  --quiet              suppress progress and tables\n");
  std::printf("  --precision <p>      fp64 or mixed (default: mixed)\n");
  std::printf("  --device <int>       CUDA device (default: 0)\n");
  std::printf("  --data-dir <dir>     output directory (default: data)\n");
  std::printf("  --version, -v        print the version\n  --help, -h           print this help\n");
}

// display_utils.rs:234-290: the percentile table of one statistic
void table(const char* model, const char* stat, const std::vector<double>& ps, const std::vector<double>& vals,
           long long n) {
  std::printf("%s for model %s:\nTotal calculated %s values\n", stat, model, with_commas(n).c_str());
  size_t pw = std::strlen("Percentile"), vw = std::strlen("Value");
  char buf[64];
  for (double p : ps) pw = std::max(pw, (size_t)std::snprintf(buf, sizeof buf, "%.1fth", p * 100.0));
  for (double v : vals) vw = std::max(vw, (size_t)std::snprintf(buf, sizeof buf, "%.6f", v));
  std::printf("%-*s %*s\n", (int)pw, "Percentile", (int)vw, "Value");
  std::printf("%s\n", std::string(pw + vw + 1, '-').c_str());
  for (size_t i = 0; i < ps.size(); i++) {
    std::snprintf(buf, sizeof buf, "%.1fth", ps[i] * 100.0);
    std::printf("%-*s %*.6f\n", (int)pw, buf, (int)vw, vals[i]);
  }
}

int report(const Config& cfg, int model, int dim) {
  char path[4096];
  if (jne_simulation_filename(cfg.data_dir.c_str(), model, dim, (int)cfg.steps, path, sizeof path)) return 1;
  int m = 0, d = 0, k = 0;
  uint32_t steps = 0;
  int64_t n = 0;
  if (jne_dat_read(path, &m, &d, &steps, &n, &k, nullptr, nullptr, 0)) return 1;
  std::vector<uint32_t> seeds((size_t)n);
  std::vector<double> eigs((size_t)n * k);
  if (n && jne_dat_read(path, nullptr, nullptr, nullptr, &n, &k, seeds.data(), eigs.data(), n)) return 1;
  // read_data (simulation.rs:61-87): the records with seed <= num_runs
  std::vector<double> kept;
  long long cnt = 0;
  for (int64_t r = 0; r < n; r++)
    if (seeds[(size_t)r] >= 1 && (long long)seeds[(size_t)r] <= cfg.runs) {
      kept.insert(kept.end(), eigs.begin() + r * k, eigs.begin() + (r + 1) * k);
      cnt++;
    }
  const std::vector<double> ps = {0.5, 0.75, 0.8, 0.85, 0.9, 0.95, 0.975, 0.99};
  std::vector<double> tr(ps.size()), mx(ps.size());
  if (jne_percentiles(kept.data(), cnt, k, 0, ps.data(), (int)ps.size(), tr.data()) ||
      jne_percentiles(kept.data(), cnt, k, 1, ps.data(), (int)ps.size(), mx.data()))
    return 1;
  table(kModelNames[model], "Trace", ps, tr, cnt);
  std::printf("\n");
  table(kModelNames[model], "MaxEig", ps, mx, cnt);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  Config cfg;
  if (argc > 1 && (!std::strcmp(argv[1], "--help") || !std::strcmp(argv[1], "-h"))) {
    help(argv[0]);
    return 0;
  }
  if (argc > 1 && (!std::strcmp(argv[1], "--version") || !std::strcmp(argv[1], "-v"))) {
    const int v = jne_version();  // cli.rs print_version: "<name> version <x.y.z>"
    std::printf("jne_gb300 version %d.%d.%d\n", v / 10000, v / 100 % 100, v % 100);
    return 0;
  }
  for (int i = 1; i < argc;) {
    const std::string a = argv[i];
    long long v = 0;
    if (a == "--threads" || a == "--steps" || a == "--runs" || a == "--dim-start" || a == "--dim-end" ||
        a == "--dim" || a == "--device") {
      if (!parse_count(argc, argv, i, a.c_str(), &v)) return 1;
      if (a == "--threads") cfg.threads = v;
      else if (a == "--steps") cfg.steps = v;
      else if (a == "--runs") cfg.runs = v;
      else if (a == "--dim-start") cfg.dim_start = v;
      else if (a == "--dim-end") cfg.dim_end = v;
      else if (a == "--device") cfg.device = (int)v;
      else cfg.dim_start = cfg.dim_end = v;
      i += 2;
    } else if (a == "--model") {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "Error: --model parameter requires a value\n");
        return 1;
      }
      if (!parse_models(argv[i + 1], &cfg.models)) return 1;
      i += 2;
    } else if (a == "--precision" || a == "--data-dir") {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "Error: %s parameter requires a value\n", a.c_str());
        return 1;
      }
      const std::string val = argv[i + 1];
      if (a == "--data-dir") {
        cfg.data_dir = val;
      } else if (val == "fp64" || val == "mixed") {
        cfg.precision = val == "fp64" ? JNE_PREC_FP64 : JNE_PREC_MIXED;
      } else {
        std::fprintf(stderr, "Error: --precision must be fp64 or mixed\n");
        return 1;
      }
      i += 2;
    } else if (a == "--quiet") {
      cfg.quiet = true;
      i += 1;
    } else {
      std::fprintf(stderr, "Error: unknown argument '%s'\nUse --help to see available options\n", a.c_str());
      return 1;
    }
  }
  // cli.rs validate
  if (cfg.dim_start > cfg.dim_end) {
    std::fprintf(stderr, "Error: dimension start (%lld) cannot be greater than end (%lld)\n", cfg.dim_start,
                 cfg.dim_end);
    return 1;
  }
  if (cfg.steps == 0 || cfg.runs == 0 || cfg.dim_start == 0) {
    std::fprintf(stderr, "Error: steps, runs, and dimension parameters must be greater than 0\n");
    return 1;
  }
  const long long cores = std::thread::hardware_concurrency();
  if (cfg.threads == 0 || (cfg.threads > 0 && cfg.threads > 2 * cores)) {
    std::fprintf(stderr, "Error: thread count must be between 1 and %lld\n", 2 * cores);
    return 1;
  }
  if (cfg.dim_end > JNE_MAX_DIM) {
    std::fprintf(stderr, "Error: dimensions above %d are not supported by this engine\n", JNE_MAX_DIM);
    return 1;
  }
  jne_context* ctx = nullptr;
  if (jne_open(cfg.device, 0, &ctx) != JNE_OK) {
    std::fprintf(stderr, "Error: cannot open CUDA device %d\n", cfg.device);
    return 1;
  }
  if (!cfg.quiet) {
    std::printf("=== Large-scale Simulation Demo ===\n");
    std::printf("Starting simulation (supports resuming from checkpoint)...\nConfiguration:\n");
    std::printf("  Steps: %s\n  Runs: %s\n  Dimension range: %lld - %lld\n", with_commas(cfg.steps).c_str(),
                with_commas(cfg.runs).c_str(), cfg.dim_start, cfg.dim_end);
    std::printf("  Precision: %s\n\n", cfg.precision == JNE_PREC_FP64 ? "fp64" : "mixed");
  }
  int rc = 0;
  for (long long dim = cfg.dim_start; dim <= cfg.dim_end && !rc; dim++) {
    if (!cfg.quiet)
      std::printf("Simulation config: %lld dimensions, %s steps, %s runs\n", dim, with_commas(cfg.steps).c_str(),
                  with_commas(cfg.runs).c_str());
    // every model of this dim from one pass over the paths (the path of a seed does not depend on the model)
    rc = jne_simulation_run_models(ctx, cfg.data_dir.c_str(), cfg.models.data(), (int)cfg.models.size(), (int)dim,
                                   (int)cfg.steps, cfg.runs, cfg.precision, JNE_DEFAULT_BASE_SEED, cfg.quiet ? 1 : 0);
    if (rc) {
      std::fprintf(stderr, "Error: dim %lld: %s\n", dim, jne_dat_last_error());
      break;
    }
    for (int model : cfg.models) {
      if (!cfg.quiet && report(cfg, model, (int)dim)) {
        std::fprintf(stderr, "Error: reading results: %s\n", jne_dat_last_error());
        rc = 1;
        break;
      }
      if (!cfg.quiet) std::printf("\n");
    }
  }
  jne_close(ctx);
  return rc ? 1 : 0;
}
