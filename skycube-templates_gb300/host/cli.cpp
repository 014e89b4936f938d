// skycube -- command-line driver of the GB300 skycube engine, with the flags
// of the suite's TemplatedSkycube binary (src/main.cu:44-178) for its GPU
// algorithms:
//
//   skycube -f <csv> -s <mdmc|sdsc> [-m max_d] [-d depth] [-g device]
//           [-e batched|plain] [-c] [-o] [-p] [-t threads] [-a alpha] [-q pq]
//
// The CSV holds one point per line, attributes separated by commas (a
// trailing comma is allowed), as read by the suite's read_data
// (src/utilities/utilities.h:140-178). The dimensionality selects the
// template instance (2..16, src/main.cu:141-173). The time of Execute() is
// printed in milliseconds followed by a tab, as the suite prints it
// (src/main.h:344-346).
//
// -c checks the result: the suite compares cuboid sizes against its CPU STSC
// (src/main.h:72-110); this driver compares full id sets per cuboid against
// the engine's other, independent algorithm (the per-cuboid skyline for
// -s mdmc, the bitmap form for -s sdsc) and exits 1 on any difference.
// -q sets the prefilter's pruner count for mdmc (the suite's pq_size, capped
// at 1024). -t, -a and -p are accepted for compatibility (no CPU workers
// run).
#include <getopt.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>

#include "skycube_templates.h"

namespace {

void usage() {
  printf("\nskycube - skycube computation on one GB300 (templated suite interface)\n\n");
  printf("USAGE: skycube -f <filename> -s <algorithm>\n");
  printf(" -f: input filename (CSV, one point per line)\n");
  printf(" -s: skycube algorithm: mdmc | sdsc\n");
  printf(" -m: maximum number of attributes of a cuboid in the result\n");
  printf(" -d: grid depth (2^depth cells per attribute, 1..7; default automatic)\n");
  printf(" -g: GPU device number (first of a comma separated list)\n");
  printf(" -e: execution form: batched (one launch for all cuboids, default) | plain\n");
  printf(" -c: check the result against the engine's other algorithm (id sets)\n");
  printf(" -o: print the work distribution\n");
  printf(" -q: prefilter pruners for mdmc (default 128, at most 1024)\n");
  printf(" -p, -t, -a, -i: accepted for compatibility; no CPU workers run\n\n");
}

std::vector<float> split_line(const std::string& line, bool* ok) {
  std::vector<float> out;
  std::stringstream ss(line);
  std::string tok;
  *ok = true;
  while (std::getline(ss, tok, ',')) {
    size_t a = tok.find_first_not_of(" \t\r");
    if (a == std::string::npos) continue;  // empty field, e.g. a trailing comma
    char* end = nullptr;
    const float v = std::strtof(tok.c_str() + a, &end);
    if (end == tok.c_str() + a) *ok = false;
    out.push_back(v);
  }
  return out;
}

// Reads every non-empty line; returns false with a message on bad input.
bool read_csv(const std::string& fname, std::vector<std::vector<float> >* rows, std::string* err) {
  std::ifstream f(fname);
  if (!f.is_open()) {
    *err = "..No such file: " + fname;
    return false;
  }
  std::string line;
  size_t lineno = 0;
  while (std::getline(f, line)) {
    ++lineno;
    if (line.find_first_not_of(" \t\r") == std::string::npos) continue;
    bool ok = true;
    std::vector<float> v = split_line(line, &ok);
    if (!ok || v.empty()) {
      *err = "PARSE FAILED at line " + std::to_string(lineno);
      return false;
    }
    if (!rows->empty() && v.size() != rows->front().size()) {
      *err = "line " + std::to_string(lineno) + " has " + std::to_string(v.size()) +
             " attributes, expected " + std::to_string(rows->front().size());
      return false;
    }
    rows->push_back(std::move(v));
  }
  if (rows->empty()) {
    *err = "no points in " + fname;
    return false;
  }
  return true;
}

long now_ms() {
  using namespace std::chrono;
  return (long)duration_cast<milliseconds>(steady_clock::now().time_since_epoch()).count();
}

template <int D>
std::vector<std::vector<unsigned> > sets_from_mdmc(MDMC<D>& m, int max_d) {
  std::vector<std::vector<unsigned> > out(1u << D);
  for (unsigned c = 1; c < (1u << D); ++c) {
    if (__builtin_popcount(c) > max_d && c != (1u << D) - 1) continue;
    std::vector<int> v = getsubspace(c, m.getHashCubeStructure());
    out[c].assign(v.begin(), v.end());
    std::sort(out[c].begin(), out[c].end());
  }
  return out;
}

template <int D>
std::vector<std::vector<unsigned> > sets_from_sdsc(SDSC<D>& s, int max_d) {
  std::vector<std::vector<unsigned> > out(1u << D);
  for (unsigned c = 1; c < (1u << D); ++c) {
    if (__builtin_popcount(c) > max_d && c != (1u << D) - 1) continue;
    out[c] = s.getLattice()[c].skyline;
    std::sort(out[c].begin(), out[c].end());
  }
  return out;
}

template <int D>
int run_algorithm(Config* cfg, float** data, uint32_t n) {
  const int max_d = cfg->max_d;
  std::vector<std::vector<unsigned> > got, other;
  long t0 = 0, t1 = 0;
  if (cfg->algo == "mdmc") {
    MDMC<D> cube(cfg, (int)n);
    cube.Init(data);
    t0 = now_ms();
    cube.Execute();
    t1 = now_ms();
    if (cfg->check) {
      got = sets_from_mdmc<D>(cube, max_d);
      Config c2 = *cfg;
      c2.mode = "plain";
      SDSC<D> ref(&c2, (int)n);
      ref.Init(data);
      ref.Execute();
      other = sets_from_sdsc<D>(ref, max_d);
    }
  } else {
    SDSC<D> cube(cfg, (int)n);
    cube.Init(data);
    t0 = now_ms();
    cube.Execute();
    t1 = now_ms();
    if (cfg->check) {
      got = sets_from_sdsc<D>(cube, max_d);
      Config c2 = *cfg;
      c2.mode = "batched";
      MDMC<D> ref(&c2, (int)n);
      ref.Init(data);
      ref.Execute();
      other = sets_from_mdmc<D>(ref, max_d);
    }
  }
  int status = 0;
  if (cfg->check) {
    printf("checking\n");
    size_t bad = 0;
    for (unsigned c = 1; c < (1u << D); ++c) {
      if (got[c] != other[c]) {
        ++bad;
        printf("In cuboid %u, truth: %zu, in: %zu\n", c, other[c].size(), got[c].size());
      }
    }
    printf("done checking\n");
    if (bad) status = 1;
  }
  if (cfg->cross_distribution) printf("GPU%d\n1.000000\n", skc::device_of(cfg));
  std::cout << (t1 - t0) << "\t" << std::flush;
  return status;
}

}  // namespace

int main(int argc, char** argv) {
  Config cfg;
  cfg.max_d = -1;
  int c = 0;
  opterr = 0;
  while ((c = getopt(argc, argv, "f:t:s:a:d:q:g:m:i:e:pco")) != -1) {
    switch (c) {
      case 'f': cfg.input_fname = optarg; break;
      case 't': cfg.threads = (uint32_t)atoi(optarg); break;
      case 's': cfg.algo = optarg; break;
      case 'a': cfg.alpha_size = (uint32_t)atoi(optarg); break;
      case 'd': cfg.partitioning_depth = (uint32_t)atoi(optarg); break;
      case 'q': cfg.pq_size = (uint32_t)atoi(optarg); break;
      case 'g': {
        std::stringstream ss(optarg);
        std::string tok;
        while (std::getline(ss, tok, ',')) cfg.devices.push_back(std::stoi(tok));
        break;
      }
      case 'm': cfg.max_d = atoi(optarg); break;
      case 'i': cfg.papi = optarg; break;
      case 'e': cfg.mode = optarg; break;
      case 'p': cfg.cpu = false; break;
      case 'c': cfg.check = true; break;
      case 'o': cfg.cross_distribution = true; break;
      default:
        if (isprint(optopt)) fprintf(stderr, "Unknown option `-%c'.\n", optopt);
        usage();
        return 1;
    }
  }
  if (cfg.input_fname.empty() || cfg.algo.empty()) {
    usage();
    return 1;
  }
  if (cfg.algo != "mdmc" && cfg.algo != "sdsc") {
    fprintf(stderr, "algorithm '%s' is not provided by this engine (GPU algorithms: mdmc, sdsc)\n",
            cfg.algo.c_str());
    return 1;
  }
  if (cfg.mode != "batched" && cfg.mode != "plain") {
    fprintf(stderr, "unknown execution form '%s' (batched|plain)\n", cfg.mode.c_str());
    return 1;
  }
  if (!cfg.papi.empty()) fprintf(stderr, "note: PAPI counters (-i) are not collected\n");
  std::vector<std::vector<float> > rows;
  std::string err;
  if (!read_csv(cfg.input_fname, &rows, &err)) {
    fprintf(stderr, "%s\n", err.c_str());
    return 1;
  }
  const int d = (int)rows.front().size();
  const uint32_t n = (uint32_t)rows.size();
  if (cfg.max_d == -1) cfg.max_d = d;
  std::vector<float*> ptrs(n);
  for (uint32_t i = 0; i < n; ++i) ptrs[i] = rows[i].data();
  float** data = ptrs.data();
  try {
    switch (d) {
#define SKC_CLI_CASE(D) case D: return run_algorithm<D>(&cfg, data, n);
      SKC_CLI_CASE(2) SKC_CLI_CASE(3) SKC_CLI_CASE(4) SKC_CLI_CASE(5) SKC_CLI_CASE(6)
      SKC_CLI_CASE(7) SKC_CLI_CASE(8) SKC_CLI_CASE(9) SKC_CLI_CASE(10) SKC_CLI_CASE(11)
      SKC_CLI_CASE(12) SKC_CLI_CASE(13) SKC_CLI_CASE(14) SKC_CLI_CASE(15) SKC_CLI_CASE(16)
#undef SKC_CLI_CASE
      default:
        printf("not supported yet, add it in the main method and template instantiations!\n");
        return 1;
    }
  } catch (const skc::Error& e) {
    fprintf(stderr, "skycube error %d: %s\n", e.code, e.what());
    return 2;
  }
}
