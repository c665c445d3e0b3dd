// gfaz - command-line front end of the GB300 GFAz build, written purely
// against the C ABI (include/gfaz_gb300.h).
//
// Commands, options, default output names and error behaviour follow the
// reference CLI (src/cli/gfaz_cli.cpp, compress_command.cpp,
// decompress_command.cpp, extract_path_command.cpp, extract_walk_command.cpp,
// add_haplotypes_command.cpp, growth_command.cpp, pav_command.cpp): "Error: <message>" on stderr and exit code 1
// on failure, extracted lines on stdout.  The transform always runs on the
// GPU; --gpu is accepted for compatibility.
#include <getopt.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cerrno>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "../../../include/gfaz_gb300.h"

namespace {

using Clock = std::chrono::steady_clock;

int fail(const char *what = nullptr) {
  std::cerr << "Error: " << (what ? what : gfz_last_error()) << std::endl;
  return 1;
}

void usage() {
  std::cout << "gfaz - GFA Compression Tool (GB300 transform)\n\nUSAGE:\n"
               "    gfaz compress [OPTIONS] <input.gfa> [output.gfaz]\n"
               "    gfaz decompress [OPTIONS] <input.gfaz> [output.gfa]\n"
               "    gfaz extract-path [OPTIONS] <input.gfaz> <path_name> [path_name ...]\n"
               "    gfaz extract-walk [OPTIONS] <input.gfaz>\n"
               "                      <sample_id> <hap_index> <seq_id> <seq_start> <seq_end> [...]\n"
               "    gfaz add-haplotypes [OPTIONS] <input.gfaz> <paths_or_walks.gfa> [output.gfaz]\n"
               "    gfaz growth [-j N] [-G path|sample-hap-seq|sample-hap|sample] <input.gfaz>\n"
               "    gfaz pav -i <input.gfaz> -b <ranges.bed> [-S|-H] [-M] [-B T] [-t N]\n\n"
               "compress options:   -r/--rounds N (8)  -d/--delta N (1)  -t/--threshold N (2)\n"
               "                    -j/--threads N (0 = auto)  -g/--gpu  -s/--stats  --debug\n"
               "                    --gpu-rolling-input-chunk-mb N (alias --gpu-chunk-mb)  --gpu-legacy\n"
               "decompress options: -j/--threads N  -l/--legacy  -g/--gpu  -s/--stats  --debug\n"
               "                    --gpu-rolling-output-chunk-mb N (alias --gpu-max-expanded-chunk-mb)\n"
               "                    --gpu-legacy\n"
               "other commands:     -j/--threads N\n";
}

long file_size(const std::string &p) {
  FILE *f = std::fopen(p.c_str(), "rb");
  if (!f) return 0;
  std::fseek(f, 0, SEEK_END);
  long n = std::ftell(f);
  std::fclose(f);
  return n;
}

// Long-only options of the reference CLI (src/cli/common.hpp values).
constexpr int kOptInputChunkMb = 1000;
constexpr int kOptGpuLegacy = 1001;
constexpr int kOptDebug = 1003;
constexpr int kOptOutputChunkMb = 1004;
// The reference's default rolling output chunk of the GPU decompressor, MiB.
constexpr unsigned long long kDefaultOutputChunkMb = 1024;

// A positive decimal integer, as the reference's parse_ull_arg takes it.
bool positive_ull(const char *name, const char *value, unsigned long long &out) {
  errno = 0;
  char *end = nullptr;
  out = std::strtoull(value, &end, 10);
  if (errno != 0 || end == value || *end != '\0' || out == 0) {
    std::cerr << "Error: Invalid value for " << name << ": " << value << std::endl;
    return false;
  }
  return true;
}

// --debug: the library's phase timers (GFA_COMPRESSION_DEBUG, read once, on
// the first library call that looks at it).
void enable_debug() { setenv("GFA_COMPRESSION_DEBUG", "1", 1); }

// A context carrying one option, or none (the library's default context).
struct CliContext {
  gfz_context *ctx = nullptr;
  ~CliContext() {
    if (ctx) gfz_context_destroy(ctx);
  }
  bool set(const char *name, int64_t value) {
    if (!ctx && gfz_context_create(0, nullptr, &ctx) != GFZ_OK) return false;
    return gfz_context_set_option(ctx, name, value) == GFZ_OK;
  }
};

const char *threads_line(int threads, std::string &buf) {
  buf = threads == 0 ? std::string("auto") : threads < 0 ? std::string("inherit OpenMP") : std::to_string(threads);
  return buf.c_str();
}

// compress_command.cpp:21-271.  The transform always runs on the GPU and is
// bit-exact with the reference's CPU compressor, so --delta and --threshold
// are honoured with or without --gpu.  --gpu-rolling-input-chunk-mb N
// streams host-resident steps through HBM in chunks of N MiB (same bytes);
// --gpu-legacy selects the whole-device path, which is this build's default
// (it changes nothing); both require --gpu, as in the reference.
int do_compress(int argc, char **argv) {
  int rounds = 8, delta = 1, threshold = 2, threads = 0;
  bool stats = false, use_gpu = false, gpu_legacy = false, debug = false;
  unsigned long long chunk_mb = 0;
  static struct option lo[] = {{"rounds", required_argument, 0, 'r'},
                               {"delta", required_argument, 0, 'd'},
                               {"threshold", required_argument, 0, 't'},
                               {"threads", required_argument, 0, 'j'},
                               {"gpu", no_argument, 0, 'g'},
                               {"gpu-rolling-input-chunk-mb", required_argument, 0, kOptInputChunkMb},
                               {"gpu-chunk-mb", required_argument, 0, kOptInputChunkMb},
                               {"gpu-legacy", no_argument, 0, kOptGpuLegacy},
                               {"stats", no_argument, 0, 's'},
                               {"debug", no_argument, 0, kOptDebug},
                               {"help", no_argument, 0, 'h'},
                               {0, 0, 0, 0}};
  int opt;
  optind = 1;
  while ((opt = getopt_long(argc, argv, "r:d:t:j:gsh", lo, nullptr)) != -1) {
    switch (opt) {
      case 'r': rounds = std::atoi(optarg); break;
      case 'd':
        delta = std::atoi(optarg);
        if (delta < 0) {
          std::cerr << "Warning: --delta must be >= 0, clamping to 0" << std::endl;
          delta = 0;
        }
        break;
      case 't': threshold = std::atoi(optarg); break;
      case 'j': threads = std::atoi(optarg); break;
      case 'g': use_gpu = true; break;
      case kOptInputChunkMb:
        if (!positive_ull("--gpu-rolling-input-chunk-mb", optarg, chunk_mb)) return 1;
        break;
      case kOptGpuLegacy: gpu_legacy = true; break;
      case 's': stats = true; break;
      case kOptDebug: debug = true; break;
      case 'h': usage(); return 0;
      default: usage(); return 1;
    }
  }
  if (optind >= argc) {
    std::cerr << "Error: No input file specified\n";
    return 1;
  }
  const std::string in = argv[optind];
  const std::string out = optind + 1 < argc ? argv[optind + 1] : in + ".gfaz";
  if (!use_gpu && (chunk_mb > 0 || gpu_legacy)) {
    std::cerr << "Error: --gpu-rolling-input-chunk-mb and --gpu-legacy require --gpu\n";
    return 1;
  }
  if (gpu_legacy && chunk_mb > 0) {
    std::cerr << "Note: --gpu-rolling-input-chunk-mb is ignored with --gpu-legacy." << std::endl;
    chunk_mb = 0;
  }
  std::string tb;
  std::cout << "=== GFAZ Compress ===\nInput:  " << in << "\nOutput: " << out << "\nBackend: GPU\nStats: "
            << (stats ? "on" : "off") << "\nDebug: " << (debug ? "on" : "off") << "\nRounds: " << rounds
            << "\nDelta:  " << delta << "\nThreshold: " << threshold;
  if (chunk_mb) std::cout << "\nGPU Rolling Input Chunk: " << chunk_mb << " MiB";
  std::cout << "\nThreads: " << threads_line(threads, tb) << "\n\n";
  if (debug) enable_debug();
  CliContext cc;
  if (chunk_mb && !cc.set("encode_chunk", (int64_t)(chunk_mb * 1024ull * 1024ull / 4))) return fail();
  const auto t0 = Clock::now();
  gfz_compressed *c = nullptr;
  if (gfz_compress_file(cc.ctx, in.c_str(), rounds, (uint64_t)threshold, delta, threads, stats ? 1 : 0, &c) != GFZ_OK)
    return fail();
  const gfz_status st = gfz_serialize(c, out.c_str());
  gfz_compressed_free(c);
  if (st != GFZ_OK) return fail();
  const double s = std::chrono::duration<double>(Clock::now() - t0).count();
  std::cout << "Compression complete!" << std::endl;
  if (stats) {
    const long a = file_size(in), b = file_size(out);
    std::printf("Stats:\n  Time: %.3f s\n  Input: %ld B\n  Output: %ld B\n  Ratio: %.2fx\n  Throughput: %.2f MB/s\n", s,
                a, b, b ? (double)a / b : 0.0, a / 1048576.0 / (s > 0 ? s : 1));
  }
  return 0;
}

// extract-path, extract-walk, add-haplotypes: -j/--threads and -h as in the
// reference; --gpu is accepted as well (these always run on the GPU).
int simple_opts(int argc, char **argv, int &threads, const char *shortopts) {
  static struct option lo[] = {{"threads", required_argument, 0, 'j'},
                               {"gpu", no_argument, 0, 'g'},
                               {"help", no_argument, 0, 'h'},
                               {0, 0, 0, 0}};
  int opt;
  optind = 1;
  while ((opt = getopt_long(argc, argv, shortopts, lo, nullptr)) != -1) {
    switch (opt) {
      case 'j': threads = std::atoi(optarg); break;
      case 'g': break;
      case 'h': usage(); return 0;
      default: usage(); return 1;
    }
  }
  return -1;
}

// decompress_command.cpp:23-274.  --gpu-rolling-output-chunk-mb N (alias
// --gpu-max-expanded-chunk-mb) writes the P and W text in traversal groups
// of at most N MiB of expanded int32 steps, one group on the device at a
// time; without it the whole graph decodes in one pass.  --legacy (the
// reference's in-memory CPU mode) and --gpu-legacy write the same bytes as
// the default; the reference's checks on combining them are kept.
int do_decompress(int argc, char **argv) {
  int threads = 0;
  bool use_gpu = false, legacy = false, gpu_legacy = false, stats = false, debug = false;
  unsigned long long chunk_mb = kDefaultOutputChunkMb;
  bool chunk_given = false;
  static struct option lo[] = {{"threads", required_argument, 0, 'j'},
                               {"legacy", no_argument, 0, 'l'},
                               {"gpu", no_argument, 0, 'g'},
                               {"gpu-rolling-output-chunk-mb", required_argument, 0, kOptOutputChunkMb},
                               {"gpu-max-expanded-chunk-mb", required_argument, 0, kOptOutputChunkMb},
                               {"gpu-legacy", no_argument, 0, kOptGpuLegacy},
                               {"stats", no_argument, 0, 's'},
                               {"debug", no_argument, 0, kOptDebug},
                               {"help", no_argument, 0, 'h'},
                               {0, 0, 0, 0}};
  int opt;
  optind = 1;
  while ((opt = getopt_long(argc, argv, "j:lgsh", lo, nullptr)) != -1) {
    switch (opt) {
      case 'j': threads = std::atoi(optarg); break;
      case 'l': legacy = true; break;
      case 'g': use_gpu = true; break;
      case kOptOutputChunkMb:
        if (!positive_ull("--gpu-rolling-output-chunk-mb", optarg, chunk_mb)) return 1;
        chunk_given = true;
        break;
      case kOptGpuLegacy: gpu_legacy = true; break;
      case 's': stats = true; break;
      case kOptDebug: debug = true; break;
      case 'h': usage(); return 0;
      default: usage(); return 1;
    }
  }
  if (optind >= argc) {
    std::cerr << "Error: No input file specified\n";
    return 1;
  }
  const std::string in = argv[optind];
  if (!use_gpu && (chunk_mb != kDefaultOutputChunkMb || gpu_legacy)) {
    std::cerr << "Error: --gpu-rolling-output-chunk-mb and --gpu-legacy require --gpu\n";
    return 1;
  }
  if (use_gpu && legacy) {
    std::cerr << "Error: --legacy is the CPU legacy mode. Use --gpu-legacy for the old whole-graph GPU "
                 "decompression path.\n";
    return 1;
  }
  std::string out;
  if (optind + 1 < argc) out = argv[optind + 1];
  else if (in.size() > 5 && in.substr(in.size() - 5) == ".gfaz") out = in.substr(0, in.size() - 5);
  else out = in + ".decompressed";
  if (gpu_legacy && chunk_given) {
    std::cerr << "Note: --gpu-rolling-output-chunk-mb is ignored with --gpu-legacy." << std::endl;
    chunk_given = false;
  }
  std::string tb;
  std::cout << "=== GFAZ Decompress ===\nInput:  " << in << "\nOutput: " << out << "\nBackend: GPU\nStats: "
            << (stats ? "on" : "off") << "\nDebug: " << (debug ? "on" : "off");
  if (chunk_given) std::cout << "\nGPU Rolling Output Chunk: " << chunk_mb << " MiB";
  std::cout << "\nThreads: " << threads_line(threads, tb) << "\n\n";
  if (debug) enable_debug();
  CliContext cc;
  if (chunk_given && !cc.set("decode_chunk", (int64_t)(chunk_mb * 1024ull * 1024ull / 4))) return fail();
  const auto t0 = Clock::now();
  gfz_compressed *c = nullptr;
  if (gfz_deserialize(in.c_str(), &c) != GFZ_OK) return fail();
  const gfz_status st = gfz_write_gfa(cc.ctx, c, out.c_str(), threads);
  gfz_compressed_free(c);
  if (st != GFZ_OK) return fail();
  const double s = std::chrono::duration<double>(Clock::now() - t0).count();
  std::cout << "\nDecompression complete!" << std::endl;
  if (stats) {
    const long a = file_size(in), b = file_size(out);
    std::printf("Stats:\n  Time: %.3f s\n  Input: %ld B\n  Output: %ld B\n  Throughput: %.2f MB/s\n", s, a, b,
                b / 1048576.0 / (s > 0 ? s : 1));
  }
  return 0;
}

int print_and_free(gfz_status st, char *text, size_t len) {
  if (st != GFZ_OK) return fail();
  std::fwrite(text, 1, len, stdout);
  gfz_free(text);
  return 0;
}

int do_extract_path(int argc, char **argv) {
  int threads = 0;
  if (int r = simple_opts(argc, argv, threads, "j:gh"); r >= 0) return r;
  if (optind + 1 >= argc) {
    std::cerr << "Error: Expected <input.gfaz> and at least one <path_name>\n";
    return 1;
  }
  gfz_compressed *c = nullptr;
  if (gfz_deserialize(argv[optind], &c) != GFZ_OK) return fail();
  std::vector<const char *> names(argv + optind + 1, argv + argc);
  char *text = nullptr;
  size_t len = 0;
  const gfz_status st = gfz_extract_path_lines(nullptr, c, names.data(), names.size(), threads, &text, &len);
  gfz_compressed_free(c);
  return print_and_free(st, text, len);
}

int do_extract_walk(int argc, char **argv) {
  int threads = 0;
  if (int r = simple_opts(argc, argv, threads, "j:gh"); r >= 0) return r;
  if (optind + 5 >= argc) {
    std::cerr << "Error: Expected <input.gfaz> and at least one walk identifier tuple\n";
    return 1;
  }
  if ((argc - (optind + 1)) % 5 != 0) {
    std::cerr << "Error: Walk identifiers must be provided in groups of 5: "
                 "<sample_id> <hap_index> <seq_id> <seq_start> <seq_end>\n";
    return 1;
  }
  std::vector<gfz_walk_key> keys;
  try {
    for (int i = optind + 1; i < argc; i += 5) {
      gfz_walk_key k;
      k.sample_id = argv[i];
      k.hap_index = (uint32_t)std::stoul(argv[i + 1]);
      k.seq_id = argv[i + 2];
      k.seq_start = std::string(argv[i + 3]) == "*" ? -1 : std::stoll(argv[i + 3]);
      k.seq_end = std::string(argv[i + 4]) == "*" ? -1 : std::stoll(argv[i + 4]);
      keys.push_back(k);
    }
  } catch (const std::exception &e) {
    return fail(e.what());
  }
  gfz_compressed *c = nullptr;
  if (gfz_deserialize(argv[optind], &c) != GFZ_OK) return fail();
  char *text = nullptr;
  size_t len = 0;
  const gfz_status st = gfz_extract_walk_lines(nullptr, c, keys.data(), keys.size(), threads, &text, &len);
  gfz_compressed_free(c);
  return print_and_free(st, text, len);
}

int do_add_haplotypes(int argc, char **argv) {
  int threads = 0;
  if (int r = simple_opts(argc, argv, threads, "j:gh"); r >= 0) return r;
  if (optind + 1 >= argc) {
    std::cerr << "Error: Expected <input.gfaz> and <paths_or_walks.gfa>\n";
    return 1;
  }
  const std::string in = argv[optind], haps = argv[optind + 1];
  std::string out;
  if (optind + 2 < argc) out = argv[optind + 2];
  else if (in.size() > 5 && in.substr(in.size() - 5) == ".gfaz") out = in.substr(0, in.size() - 5) + ".updated.gfaz";
  else out = in + ".updated.gfaz";
  gfz_compressed *c = nullptr;
  if (gfz_deserialize(in.c_str(), &c) != GFZ_OK) return fail();
  gfz_status st = gfz_add_haplotypes(nullptr, c, haps.c_str(), threads);
  if (st == GFZ_OK) st = gfz_serialize(c, out.c_str());
  gfz_compressed_free(c);
  if (st != GFZ_OK) return fail();
  return 0;
}

// src/cli/growth_command.cpp: the growth table on stdout.
int do_growth(int argc, char **argv) {
  int threads = 0, group = 0;
  const char *label = "path";
  static struct option lo[] = {{"threads", required_argument, 0, 'j'},
                               {"group-by", required_argument, 0, 'G'},
                               {"help", no_argument, 0, 'h'},
                               {0, 0, 0, 0}};
  int opt;
  optind = 1;
  while ((opt = getopt_long(argc, argv, "j:G:h", lo, nullptr)) != -1) {
    if (opt == 'j') {
      threads = std::atoi(optarg);
    } else if (opt == 'G') {
      const std::string v = optarg;
      if (v == "path" || v == "per-line") group = 0, label = "path";
      else if (v == "sample-hap-seq" || v == "panacus") group = 1, label = "sample-hap-seq";
      else if (v == "sample-hap" || v == "haplotype") group = 2, label = "sample-hap";
      else if (v == "sample") group = 3, label = "sample";
      else {
        std::cerr << "Error: unknown --group-by value '" << v
                  << "'. Expected 'path', 'sample-hap-seq', 'sample-hap', or 'sample'.\n";
        return 1;
      }
    } else if (opt == 'h') {
      std::cout << "gfaz growth [-j N] [-G path|sample-hap-seq|sample-hap|sample] <input.gfaz>\n";
      return 0;
    } else {
      return 1;
    }
  }
  if (optind >= argc) {
    std::cerr << "Error: Expected <input.gfaz>\n";
    return 1;
  }
  gfz_compressed *c = nullptr;
  if (gfz_deserialize(argv[optind], &c) != GFZ_OK) return fail();
  uint32_t nh = 0, nn = 0;
  uint64_t *hist = nullptr;
  double *growth = nullptr;
  const gfz_status st = gfz_growth(nullptr, c, threads, group, &nh, &nn, &hist, &growth);
  gfz_compressed_free(c);
  if (st != GFZ_OK) return fail();
  std::cout << "# gfaz growth (count=node, coverage>=1, quorum>=0)\n# group-by=" << label
            << "\n# num_haplotypes=" << nh << " num_nodes=" << nn << "\nk\tgrowth\n";
  std::fflush(stdout);
  for (uint32_t k = 1; k <= nh; ++k) std::printf("%u\t%.4f\n", k, growth[k]);
  gfz_free(hist);
  gfz_free(growth);
  return 0;
}

// src/cli/pav_command.cpp: PAV ratios over BED ranges on stdout, one line
// per (range, group) or a matrix (-M); -B T prints 1 / 0 for ratio >= T.
int do_pav(int argc, char **argv) {
  std::string in, bed;
  int threads = 0, group = 0;
  bool by_sample = false, by_hap = false, matrix = false, binary = false;
  double threshold = 0.0;
  static struct option lo[] = {{"idx", required_argument, 0, 'i'},
                               {"input", required_argument, 0, 'i'},
                               {"bed-file", required_argument, 0, 'b'},
                               {"group-by-sample", no_argument, 0, 'S'},
                               {"group-by-haplotype", no_argument, 0, 'H'},
                               {"matrix-output", no_argument, 0, 'M'},
                               {"binary-values", required_argument, 0, 'B'},
                               {"threads", required_argument, 0, 't'},
                               {"help", no_argument, 0, 'h'},
                               {0, 0, 0, 0}};
  int opt;
  optind = 1;
  while ((opt = getopt_long(argc, argv, "i:b:SHMB:t:j:h", lo, nullptr)) != -1) {
    switch (opt) {
      case 'i': in = optarg; break;
      case 'b': bed = optarg; break;
      case 'S': by_sample = true, group = 3; break;
      case 'H': by_hap = true, group = 2; break;
      case 'M': matrix = true; break;
      case 'B': binary = true, threshold = std::stod(optarg); break;
      case 't':
      case 'j': threads = std::atoi(optarg); break;
      case 'h':
        std::cout << "gfaz pav -i <input.gfaz> -b <ranges.bed> [-S|-H] [-M] [-B T] [-t N]\n";
        return 0;
      default: return 1;
    }
  }
  if (by_sample && by_hap) {
    std::cerr << "Error: select only one grouping option: -S or -H\n";
    return 1;
  }
  if (binary && (threshold < 0.0 || threshold > 1.0)) {
    std::cerr << "Error: --binary-values threshold must be in [0,1]\n";
    return 1;
  }
  if (in.empty() && optind < argc) in = argv[optind++];
  if (in.empty()) {
    std::cerr << "Error: Expected -i <input.gfaz>\n";
    return 1;
  }
  if (bed.empty()) {
    std::cerr << "Error: Expected -b <ranges.bed>\n";
    return 1;
  }
  gfz_compressed *c = nullptr;
  if (gfz_deserialize(in.c_str(), &c) != GFZ_OK) return fail();
  char *rs = nullptr, *gs = nullptr;
  size_t rl = 0, gl = 0;
  uint64_t nr = 0, ng = 0, *den = nullptr, *num = nullptr;
  const gfz_status st = gfz_pav(nullptr, c, bed.c_str(), threads, group, &rs, &rl, &gs, &gl, &nr, &ng, &den, &num);
  gfz_compressed_free(c);
  if (st != GFZ_OK) return fail();
  auto lines = [](const char *p, size_t n) {
    std::vector<std::string> v;
    size_t b = 0;
    for (size_t i = 0; i < n; ++i)
      if (p[i] == '\n') {
        v.emplace_back(p + b, i - b);
        b = i + 1;
      }
    return v;
  };
  const std::vector<std::string> ranges = lines(rs, rl), groups = lines(gs, gl);
  auto ratio = [&](uint64_t w, uint64_t g) {
    return den[w] == 0 ? 0.0 : (double)num[w * ng + g] / (double)den[w];
  };
  std::cout << "chrom\tstart\tend\tname";
  if (matrix) {
    for (const auto &g : groups) std::cout << '\t' << g;
    std::cout << '\n';
    for (uint64_t w = 0; w < nr; ++w) {
      std::cout << ranges[w];
      for (uint64_t g = 0; g < ng; ++g) {
        if (binary) std::cout << '\t' << (ratio(w, g) >= threshold ? 1 : 0);
        else std::cout << '\t' << std::setprecision(5) << ratio(w, g);
      }
      std::cout << '\n';
    }
  } else {
    std::cout << "\tgroup\tpav\n";
    for (uint64_t w = 0; w < nr; ++w)
      for (uint64_t g = 0; g < ng; ++g) {
        std::cout << ranges[w] << '\t' << groups[g] << '\t';
        if (binary) std::cout << (ratio(w, g) >= threshold ? 1 : 0);
        else std::cout << std::setprecision(5) << ratio(w, g);
        std::cout << '\n';
      }
  }
  gfz_free(rs);
  gfz_free(gs);
  gfz_free(den);
  gfz_free(num);
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 2) {
    usage();
    return 1;
  }
  const std::string cmd = argv[1];
  if (cmd == "compress") return do_compress(argc - 1, argv + 1);
  if (cmd == "decompress") return do_decompress(argc - 1, argv + 1);
  if (cmd == "extract-path") return do_extract_path(argc - 1, argv + 1);
  if (cmd == "extract-walk") return do_extract_walk(argc - 1, argv + 1);
  if (cmd == "add-haplotypes") return do_add_haplotypes(argc - 1, argv + 1);
  if (cmd == "growth") return do_growth(argc - 1, argv + 1);
  if (cmd == "pav") return do_pav(argc - 1, argv + 1);
  if (cmd == "-h" || cmd == "--help" || cmd == "help") {
    usage();
    return 0;
  }
  std::cerr << "Unknown command: " << cmd << std::endl;
  usage();
  return 1;
}
