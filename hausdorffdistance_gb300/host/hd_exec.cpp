// hd_exec — command-line driver with the reference's flags
// (src/flags.cc:1-58, src/main.cpp:33-152, src/run_hausdorff_distance.cu:53-402)
// over libhdgpu.so.  Prints "Time: <avg> ms" and
// "HausdorffDistance: distance is <d>" and writes the reference's JSON keys.
//
// -execution cpu runs the CPU early-break of cpu_early_break.h (the
// reference's CPU path, on -parallelism threads, every host thread when it is
// not positive), and -check re-runs it on all host threads and compares, as the
// reference does (run_hausdorff_distance.cu:366-389).  Each file, and both
// together, get the reference's "Grid", "MBR" and "Density" statistics
// (run_hausdorff_distance.cu:150-185) from hd_compute_stats on the GPU.
// Differences: -undirected computes max(h(A,B), h(B,A)) in one call;
// -input_type also accepts "bin" (the reference's point-cache layout), and
// "image" reads NIfTI-1 (.nii) and MetaImage (.mha/.mhd) files without ITK;
// -variant accepts eb | hybrid | auto | rt | lbvh | grid | bf16 | brute; the
// grid statistics' "NonEmptyCells" is the non-empty fraction as a real number
// (the reference divides two integers there, which truncates it to 0).
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "cpu_early_break.h"
#include "hausdorff_distance.h"
#include "hd_gpu.h"
#include "json.h"
#include "loaders.h"

namespace {

struct Flags {
  std::map<std::string, std::string> v;
  std::string get(const std::string& k, const std::string& def) const {
    auto it = v.find(k);
    return it == v.end() ? def : it->second;
  }
  long long geti(const std::string& k, long long def) const {
    auto it = v.find(k);
    return it == v.end() ? def : std::atoll(it->second.c_str());
  }
  double getd(const std::string& k, double def) const {
    auto it = v.find(k);
    return it == v.end() ? def : std::atof(it->second.c_str());
  }
  // gflags' boolean values: 1/t/true/y/yes and 0/f/false/n/no, any case.
  bool getb(const std::string& k, bool def) const {
    auto it = v.find(k);
    if (it == v.end()) return def;
    std::string s = it->second;
    for (auto& ch : s) ch = (char) std::tolower((unsigned char) ch);
    return !(s == "false" || s == "0" || s == "no" || s == "f" || s == "n");
  }
};

const char* kBoolFlags[] = {"is_double", "normalize", "auto_tune", "auto_tune_eb_only_threshold",
                            "auto_tune_n_points_cell", "auto_tune_max_hit", "fast_build_bvh",
                            "rebuild_bvh", "rt_prune", "rt_eb", "overwrite", "check",
                            "vary_params", "undirected"};

bool is_bool_flag(const std::string& k) {
  for (const char* b : kBoolFlags)
    if (k == b) return true;
  return false;
}

// gflags syntax: -name=value, --name=value, -name value, -boolflag,
// -noboolflag.
Flags parse(int argc, char** argv) {
  Flags f;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    if (a.size() < 2 || a[0] != '-') {
      std::fprintf(stderr, "unexpected argument %s\n", a.c_str());
      std::exit(1);
    }
    a = a.substr(a[1] == '-' ? 2 : 1);
    const size_t eq = a.find('=');
    if (eq != std::string::npos) {
      f.v[a.substr(0, eq)] = a.substr(eq + 1);
    } else if (is_bool_flag(a)) {
      f.v[a] = "true";
    } else if (a.rfind("no", 0) == 0 && is_bool_flag(a.substr(2))) {
      f.v[a.substr(2)] = "false";
    } else if (i + 1 < argc) {
      f.v[a] = argv[++i];
    } else {
      std::fprintf(stderr, "flag -%s needs a value\n", a.c_str());
      std::exit(1);
    }
  }
  return f;
}

std::string lower(std::string s) {
  for (auto& ch : s) ch = (char) std::tolower((unsigned char) ch);
  return s;
}

std::string now_string() {
  std::time_t t = std::time(nullptr);
  std::tm tmv;
  localtime_r(&t, &tmv);
  char buf[64];
  std::strftime(buf, sizeof(buf), "%Y-%m-%d %H:%M:%S", &tmv);
  return buf;
}

void usage(const char* argv0) {
  std::fprintf(stderr,
               "Usage: %s -input1 A -input2 B -input_type wkt|off|ply|image|bin -n_dims 2|3|<d> "
               "[-variant eb|hybrid|rt|lbvh|grid|bf16|brute] [-execution gpu|cpu] [-repeat 5] "
               "[-seed 0] [-check] [-json out.json] [-serialize dir] [-limit n] [-normalize] "
               "[-translate r] [-undirected] [-sample_rate 0.01] [-n_points_cell 8] "
               "[-eb_only_threshold 0] [-max_hit 256] [-auto_tune] [-device 0] [-parallelism n] "
               "[-stats_n_points_cell 10]\n",
               argv0);
}

// -max_hit as an LBVH traversal budget: 0 means no cap, as in the reference.
uint32_t budget_from_max_hit(long long max_hit) {
  if (max_hit <= 0 || max_hit >= 0xFFFFFFFFll) return 0xFFFFFFFFu;
  return (uint32_t) max_hit;
}

std::vector<double> split_doubles(const std::string& s) {
  std::vector<double> out;
  std::stringstream ss(s);
  std::string tok;
  while (std::getline(ss, tok, ','))
    if (!tok.empty()) out.push_back(std::atof(tok.c_str()));
  return out;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc == 1) {
    usage(argv[0]);
    return 1;
  }
  Flags fl = parse(argc, argv);
  const std::string input1 = fl.get("input1", ""), input2 = fl.get("input2", "");
  const std::string input_type = lower(fl.get("input_type", ""));
  if (input_type != "wkt" && input_type != "off" && input_type != "ply" && input_type != "image" &&
      input_type != "bin") {
    std::fprintf(stderr, "Unsupported input type: %s\n", input_type.c_str());
    return 1;
  }
  const int dims = (int) fl.geti("n_dims", 0);
  if (dims < 1 || dims > 128) {
    std::fprintf(stderr, "Wrong number of dimensions: %d\n", dims);
    return 1;
  }
  if (input_type != "bin" && dims != 2 && dims != 3) {
    std::fprintf(stderr, "%s inputs have 2 or 3 dimensions\n", input_type.c_str());
    return 1;
  }
  // -is_double: coordinates parsed and solved in FP64 (hd_solve_f64; the
  // reference's disabled double dispatch, run_hausdorff_distance.cu:56-62).
  const bool is_double = fl.getb("is_double", false);
  const std::string execution = lower(fl.get("execution", "gpu"));
  if (execution != "gpu" && execution != "cpu") {
    std::fprintf(stderr, "Unknown execution: %s\n", execution.c_str());
    return 1;
  }
  const std::string vname = lower(fl.get("variant", "eb"));
  int variant;
  if (vname == "eb") variant = HD_VARIANT_EB;
  else if (vname == "hybrid" || vname == "auto") variant = HD_VARIANT_AUTO;
  else if (vname == "rt" || vname == "lbvh") variant = HD_VARIANT_LBVH;
  else if (vname == "grid") variant = HD_VARIANT_GRID;
  else if (vname == "bf16") variant = HD_VARIANT_BF16;
  else if (vname == "brute") variant = HD_VARIANT_BRUTE;
  else {
    std::fprintf(stderr, "Unknown or unsupported variant: %s\n", vname.c_str());
    return 1;
  }
  const long long limit = fl.geti("limit", 0x7FFFFFFF);
  const int repeat = (int) std::max<long long>(1, fl.geti("repeat", 5));
  const bool undirected = fl.getb("undirected", false);
  const bool check = fl.getb("check", true);

  hd::PointSet pa, pb;
  try {
    pa = hd::LoadPoints(input1, input_type, dims, limit, fl.get("serialize", ""), is_double);
    pb = hd::LoadPoints(input2, input_type, dims, limit, fl.get("serialize", ""), is_double);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  if (pa.size() == 0 || pb.size() == 0) {
    std::fprintf(stderr, "empty input: %s has %zu points, %s has %zu\n", input1.c_str(), pa.size(),
                 input2.c_str(), pb.size());
    return 1;
  }
  const bool normalize = fl.getb("normalize", false);
  const double translate = fl.getd("translate", 0.0);
  if (normalize) {
    hd::NormalizePoints(pa);
    hd::NormalizePoints(pb);
  }
  if (translate != 0.0) hd::TranslatePoints(pb, 0, translate);
  for (size_t i = 0; i < std::min<size_t>(10, std::min(pa.size(), pb.size())); ++i) {
    std::printf("%zu A", i);
    for (int k = 0; k < std::min(dims, 3); ++k) std::printf("%s%.6f", k ? "," : " ", pa.xyz[i * dims + k]);
    std::printf(" B");
    for (int k = 0; k < std::min(dims, 3); ++k) std::printf("%s%.6f", k ? "," : " ", pb.xyz[i * dims + k]);
    std::printf("\n");
  }

  hd_options opt;
  hd_default_options(&opt);
  opt.device = (int) fl.geti("device", 0);
  opt.seed = (uint64_t) fl.geti("seed", 0);
  opt.sample_rate = fl.getd("sample_rate", 0.01);
  opt.n_points_cell = (uint32_t) fl.geti("n_points_cell", 8);
  opt.eb_only_threshold = (uint32_t) fl.geti("eb_only_threshold", 0);
  // The hybrid's RT knobs (hausdorff_distance_hybrid.h:286-295,708-778):
  // -max_hit caps the index work of one query before it falls back to the
  // early-break scan, 0 meaning no cap; here it caps the nodes and leaves an
  // LBVH packet visits before its open queries go to the deferred pass.
  // Without the flag, and under -auto_tune / -auto_tune_max_hit (the
  // reference's model predictions), the tuned table decides; likewise
  // -auto_tune / -auto_tune_eb_only_threshold leave the EB-only choice to it.
  // -fast_build_bvh, -rebuild_bvh, -rt_prune, -rt_eb, -max_reg and -bit_count
  // configure OptiX builds and are logged only.
  const bool auto_tune = fl.getb("auto_tune", false);
  if (auto_tune || fl.getb("auto_tune_eb_only_threshold", false)) opt.eb_only_threshold = 0;
  const long long max_hit = fl.geti("max_hit", 256);
  if (fl.v.count("max_hit") && !auto_tune && !fl.getb("auto_tune_max_hit", false))
    opt.lbvh_budget = budget_from_max_hit(max_hit);

  hd::Json stats = hd::Json::Object();
  int dev = opt.device;
  cudaDeviceProp prop;
  // -execution cpu runs without a GPU too (then without the GPU statistics).
  const bool have_gpu =
      cudaSetDevice(dev) == cudaSuccess && cudaGetDeviceProperties(&prop, dev) == cudaSuccess;
  if (!have_gpu && execution == "gpu") {
    std::fprintf(stderr, "no CUDA device %d\n", dev);
    return 1;
  }
  if (have_gpu) {
    stats["GPU"]["Device"] = dev;
    stats["GPU"]["name"] = prop.name;
  }
  stats["DateTime"] = now_string();
  hd::Json& input = stats["Input"];
  hd::Json files = hd::Json::Array();
  hd::Json f1 = hd::Json::Object(), f2 = hd::Json::Object();
  f1["Path"] = input1;
  f1["NumPoints"] = (unsigned long long) pa.size();
  f2["Path"] = input2;
  f2["NumPoints"] = (unsigned long long) pb.size();
  files.push_back(f1);
  files.push_back(f2);
  input["Files"] = files;
  input["Normalize"] = normalize;
  input["Translate"] = translate;
  input["SerializationPrefix"] = fl.get("serialize", "");
  input["Limit"] = limit;
  input["NumDims"] = dims;
  input["Type"] = is_double ? "Double" : "Float";

  // Per-file and combined point statistics on the GPU (the reference's
  // write_points_stats).
  const uint32_t stats_npc = (uint32_t) std::max<long long>(1, fl.geti("stats_n_points_cell", 10));
  if (have_gpu && (dims == 2 || dims == 3)) {
    hd_ctx* sctx = nullptr;
    if (hd_create(&sctx, &opt) != HD_OK) {
      std::fprintf(stderr, "hd_create failed\n");
      return 1;
    }
    auto write_stats = [&](hd::Json& j, const std::vector<float>& xyz) -> bool {
      hd_point_stats ps;
      const hd_status st = hd_compute_stats(sctx, xyz.data(), xyz.size() / dims, dims, stats_npc,
                                            0u, &ps);
      if (st != HD_OK) {
        std::fprintf(stderr, "hd_compute_stats: %s: %s\n", hd_status_string(st),
                     hd_last_error(sctx));
        return false;
      }
      hd::Json grid = hd::Json::Object();
      grid["TotalCells"] = (unsigned long long) ps.total_cells;
      grid["NonEmptyCells"] = (double) ps.nonempty_cells / (double) ps.total_cells;
      grid["MaxPoints"] = (unsigned long long) ps.max_points;
      grid["GiniIndex"] = ps.gini_index;
      grid["BuildTime"] = ps.build_ms;
      hd::Json gsize = hd::Json::Array();
      for (int k = 0; k < dims; ++k) gsize.push_back((unsigned long long) ps.grid_size[k]);
      grid["GridSize"] = gsize;
      grid["CellDiagonalLength"] = ps.cell_diagonal;
      grid["MedianPointsPerCell"] = (unsigned long long) ps.median_points;
      hd::Json hist = hd::Json::Array();
      for (uint32_t r = 0; r < ps.n_hist; ++r) {
        // The reference parses HdrHistogram's printed table back
        // (running_stats.h:106-140): the percentile carries the six
        // decimals of "%f".
        char pct[64];
        std::snprintf(pct, sizeof(pct), "%f", ps.hist_percentile[r]);
        hd::Json row = hd::Json::Object();
        row["value"] = ps.hist_value[r];
        row["percentile"] = std::strtod(pct, nullptr);
        row["count"] = (unsigned long long) ps.hist_count[r];
        hist.push_back(row);
      }
      grid["Histogram"] = hist;
      j["Grid"] = grid;
      j["StatsGridNumPointsPerCell"] = (unsigned long long) stats_npc;
      hd::Json mbr = hd::Json::Array();
      for (int k = 0; k < dims; ++k) {
        hd::Json e = hd::Json::Object();
        e["Lower"] = ps.lower[k];
        e["Upper"] = ps.upper[k];
        mbr.push_back(e);
      }
      j["MBR"] = mbr;
      j["Density"] = ps.density;
      return true;
    };
    hd::Json& jf = input["Files"];
    std::vector<float> both = pa.xyz;
    both.insert(both.end(), pb.xyz.begin(), pb.xyz.end());
    const bool ok = write_stats(jf.element(0), pa.xyz) && write_stats(jf.element(1), pb.xyz) &&
                    write_stats(input, both);
    hd_destroy(sctx);
    if (!ok) return 1;
  }

  // Inputs go to the device once, before the repeat loop, as in the
  // reference (run_hausdorff_distance.cu:148); ReportedTime excludes them.
  // With -is_double the device copies hold the doubles.
  void *dA = nullptr, *dB = nullptr;
  const size_t esz = is_double ? sizeof(double) : sizeof(float);
  const void* hA = is_double ? (const void*) pa.xyz64.data() : (const void*) pa.xyz.data();
  const void* hB = is_double ? (const void*) pb.xyz64.data() : (const void*) pb.xyz.data();
  if (have_gpu && (cudaMalloc(&dA, pa.xyz.size() * esz) != cudaSuccess ||
      cudaMalloc(&dB, pb.xyz.size() * esz) != cudaSuccess ||
      cudaMemcpy(dA, hA, pa.xyz.size() * esz, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dB, hB, pb.xyz.size() * esz, cudaMemcpyHostToDevice) != cudaSuccess)) {
    std::fprintf(stderr, "device allocation or copy failed\n");
    return 1;
  }
  // Distances are printed with the digits their type needs.
  auto print_dist = [&](double d) {
    if (is_double)
      std::printf("HausdorffDistance: distance is %.17g\n", d);
    else
      std::printf("HausdorffDistance: distance is %.9g\n", d);
  };

  // The configuration keys the reference writes into "Running" whatever the
  // execution (run_hausdorff_distance.cu:206-215), plus this driver's own.
  auto write_run_config = [&](hd::Json& run_json, const hd_options& o) {
    run_json["Seed"] = (unsigned long long) o.seed;
    run_json["FastBuildBVH"] = fl.getb("fast_build_bvh", false);
    run_json["RebuildBVH"] = fl.getb("rebuild_bvh", false);
    run_json["SampleRate"] = o.sample_rate;
    run_json["NumPointsPerCell"] = o.n_points_cell;
    run_json["MaxHit"] = max_hit;
    run_json["EBOnlyThreshold"] = o.eb_only_threshold;
    run_json["AutoTune"] = auto_tune;
    run_json["LBVHBudget"] = (unsigned long long) o.lbvh_budget;  // 0: tuned table
    run_json["Undirected"] = undirected;
  };

  auto run = [&](const hd_options& o, hd::Json& run_json, double* out_dist) -> int {
    hd_ctx* ctx = nullptr;
    hd_status s = hd_create(&ctx, &o);
    if (s != HD_OK) {
      std::fprintf(stderr, "hd_create: %s\n", hd_status_string(s));
      return 1;
    }
    double total = 0.0;
    hd::Json repeats = hd::Json::Array();
    hd_result r{};
    const auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < repeat; ++i) {
      const uint32_t sflags =
          HD_DEVICE_PTRS | HD_TIMING | HD_COUNT_PAIRS | (undirected ? HD_UNDIRECTED : 0u);
      s = is_double ? hd_solve_f64(ctx, (const double*) dA, pa.size(), (const double*) dB,
                                   pb.size(), dims, sflags, variant, &r)
                    : hd_solve(ctx, (const float*) dA, pa.size(), (const float*) dB, pb.size(),
                               dims, sflags, variant, &r);
      if (s != HD_OK) {
        std::fprintf(stderr, "%s: %s: %s\n", is_double ? "hd_solve_f64" : "hd_solve",
                     hd_status_string(s), hd_last_error(ctx));
        hd_destroy(ctx);
        return 1;
      }
      static const char* names[] = {"Hybrid", "Early Break", "Uniform Grid", "LBVH", "Split BF16",
                                    "Brute Force"};
      hd::Json rep = hd::Json::Object();
      rep["Repeat"] = i + 1;
      rep["Algorithm"] = names[variant];
      rep["VariantUsed"] = names[r.variant_used];
      rep["Execution"] = "GPU";
      rep["ReportedTime"] = r.ms;
      rep["ComparedPairs"] = (unsigned long long) r.visited_pairs;
      rep["HD64"] = r.hd;
      total += r.ms;
      repeats.push_back(rep);
    }
    const double wall =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    write_run_config(run_json, o);
    run_json["Repeats"] = repeats;
    run_json["AvgTime"] = total / repeat;
    run_json["AvgWallTime"] = wall / repeat;
    std::printf("Time: %f ms\n", total / repeat);
    *out_dist = is_double ? r.hd : (double) r.hd_f32;
    hd_destroy(ctx);
    return 0;
  };

  // The CPU early-break on all host threads (or -parallelism of them); both
  // directions for -undirected.
  auto cpu_eb = [&](const hd::PointSet& x, const hd::PointSet& y, unsigned threads) {
    return is_double ? hd::CpuEarlyBreak(x.xyz64.data(), x.size(), y.xyz64.data(), y.size(), dims,
                                         (uint32_t) opt.seed, threads)
                     : hd::CpuEarlyBreak(x.xyz.data(), x.size(), y.xyz.data(), y.size(), dims,
                                         (uint32_t) opt.seed, threads);
  };
  auto cpu_distance = [&](unsigned threads, double* compute_ms, unsigned long long* pairs,
                          double* shuffle_ms) {
    hd::CpuEarlyBreakResult ab = cpu_eb(pa, pb, threads);
    double d = ab.distance;
    *compute_ms = ab.compute_ms;
    *pairs = ab.compared_pairs;
    *shuffle_ms = ab.shuffle_ms;
    if (undirected) {
      hd::CpuEarlyBreakResult ba = cpu_eb(pb, pa, threads);
      d = std::max(d, ba.distance);
      *compute_ms += ba.compute_ms;
      *pairs += ba.compared_pairs;
      *shuffle_ms += ba.shuffle_ms;
    }
    return d;
  };
  const long long parallelism = fl.geti("parallelism", -1);
  const unsigned all_threads = std::max(1u, std::thread::hardware_concurrency());
  const unsigned cpu_threads = parallelism > 0 ? (unsigned) parallelism : all_threads;

  const std::string json_path = fl.get("json", "");
  if (execution == "cpu") {
    hd::Json& run_json = stats["Running"];
    hd::Json repeats = hd::Json::Array();
    double total = 0.0;
    double dist = 0.0;
    for (int i = 0; i < repeat; ++i) {
      double ms = 0.0, shuffle_ms = 0.0;
      unsigned long long pairs = 0;
      dist = cpu_distance(cpu_threads, &ms, &pairs, &shuffle_ms);
      // The keys of the reference's CPU early-break stats
      // (hausdorff_distance_early_break.h:104-112).
      hd::Json rep = hd::Json::Object();
      rep["Repeat"] = i + 1;
      rep["Algorithm"] = "Early Break";
      rep["Execution"] = "CPU";
      rep["Threads"] = (unsigned long long) cpu_threads;
      rep["ComparedPairs"] = pairs;
      rep["ShuffleTime"] = shuffle_ms;
      rep["ComputeTime"] = ms;
      rep["ReportedTime"] = ms;
      total += ms;
      repeats.push_back(rep);
    }
    write_run_config(run_json, opt);
    run_json["Repeats"] = repeats;
    run_json["AvgTime"] = total / repeat;
    stats["HDResult"] = dist;
    std::printf("Time: %f ms\n", total / repeat);
    print_dist(dist);
    if (!json_path.empty()) {
      const bool exists = access(json_path.c_str(), R_OK) == 0;
      if (!exists || fl.getb("overwrite", false)) std::ofstream(json_path) << stats.dump(4);
    }
    if (have_gpu) {
      cudaFree(dA);
      cudaFree(dB);
    }
    return 0;
  }
  if (fl.getb("vary_params", false)) {
    // Parameter sweep over the selector's knobs (the reference's
    // autotune_hausdorff_distance.cu:208-299), one JSON file per combination.
    const auto rates = split_doubles(fl.get("sample_rate_list", "0.01"));
    const auto thresholds = split_doubles(fl.get("eb_only_threshold_list", "0"));
    const auto cells = split_doubles(fl.get("n_points_cell_list", "8"));
    const auto hits = split_doubles(fl.get("max_hit_list", "256"));
    for (double sr : rates)
      for (double th : thresholds)
        for (double np : cells)
          for (double mh : hits) {
            hd_options o = opt;
            o.sample_rate = sr;
            o.eb_only_threshold = (uint32_t) th;
            o.n_points_cell = (uint32_t) np;
            o.lbvh_budget = budget_from_max_hit((long long) mh);
            hd::Json st = stats;
            double dist = 0.0;
            if (run(o, st["Running"], &dist)) return 1;
            st["Running"]["MaxHit"] = (long long) mh;
            st["HDResult"] = dist;
            if (!json_path.empty()) {
              std::ostringstream name;
              name << json_path << "_sr" << sr << "_th" << th << "_np" << np << "_mh" << mh
                   << ".json";
              std::ofstream(name.str()) << st.dump(4);
            }
          }
    return 0;
  }

  double dist = 0.0;
  if (run(opt, stats["Running"], &dist)) return 1;
  stats["HDResult"] = dist;
  print_dist(dist);

  if (check) {
    // The reference re-runs its CPU early-break on every host thread.
    double ms = 0.0, shuffle_ms = 0.0;
    unsigned long long pairs = 0;
    const double answer = cpu_distance(all_threads, &ms, &pairs, &shuffle_ms);
    hd::Json& ck = stats["Check"];
    ck["HDAnswer"] = answer;
    ck["Diff"] = answer - dist;
    ck["Pass"] = answer == dist;
    if (answer != dist) {
      std::fprintf(stderr, "Wrong HausdorffDistance. Result: %.8f Answer: %.8f Diff: %.8f\n", dist,
                   answer, answer - dist);
    } else {
      std::printf("HausdorffDistance is checked\n");
    }
  }
  if (!json_path.empty()) {
    const bool exists = access(json_path.c_str(), R_OK) == 0;
    if (!exists || fl.getb("overwrite", false)) {
      std::ofstream(json_path) << stats.dump(4);
    } else {
      std::fprintf(stderr, "Skip writing to JSON file %s\n", json_path.c_str());
    }
  }
  cudaFree(dA);
  cudaFree(dB);
  return 0;
}
