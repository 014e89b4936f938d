// Exercises the suite-shaped host interface (MDMC<D>, SDSC<D>, HashCube,
// getsubspace, lattice_node) on a CSV file and prints, per algorithm and
// execution form, every computed cuboid's sorted skyline ids:
//   <algo>-<form> <cuboid> <id> <id> ...
// Built and compared against the CPU oracle by tests/test_gpu_host_api.py.
#include <cstdio>
#include <fstream>
#include <sstream>

#include "skycube_templates.h"

template <int D>
void run(float** data, int n, int max_d) {
  for (const char* form : {"batched", "plain"}) {
    Config cfg;
    cfg.max_d = max_d;
    cfg.mode = form;
    {
      MDMC<D> m(&cfg, n);
      m.Init(data);
      m.Execute();
      for (unsigned c = 1; c < (1u << D); ++c) {
        if (__builtin_popcount(c) > max_d && c != (1u << D) - 1) continue;
        std::vector<int> v = getsubspace(c, m.getHashCubeStructure());
        std::sort(v.begin(), v.end());
        std::vector<int> w = m.getHashCube().getSubspace(c);
        std::sort(w.begin(), w.end());
        if (v != w) printf("MISMATCH getSubspace %u\n", c);
        printf("mdmc-%s %u", form, c);
        for (int x : v) printf(" %d", x);
        printf("\n");
      }
    }
    {
      SDSC<D> s(&cfg, n);
      s.Init(data);
      s.Execute();
      lattice_node* lat = s.getLattice();
      for (unsigned c = 1; c < (1u << D); ++c) {
        if (__builtin_popcount(c) > max_d && c != (1u << D) - 1) continue;
        std::vector<unsigned> v = lat[c].skyline;
        std::sort(v.begin(), v.end());
        printf("sdsc-%s %u", form, c);
        for (unsigned x : v) printf(" %u", x);
        printf("\n");
        std::vector<unsigned> e = lat[c].extended_sky;
        std::sort(e.begin(), e.end());
        printf("sdscext-%s %u", form, c);
        for (unsigned x : e) printf(" %u", x);
        printf("\n");
      }
    }
  }
}

int main(int argc, char** argv) {
  if (argc < 3) return 1;
  std::ifstream f(argv[1]);
  const int max_d = atoi(argv[2]);
  std::vector<std::vector<float> > rows;
  std::string line;
  while (std::getline(f, line)) {
    std::stringstream ss(line);
    std::string tok;
    std::vector<float> r;
    while (std::getline(ss, tok, ','))
      if (!tok.empty()) r.push_back(std::stof(tok));
    if (!r.empty()) rows.push_back(r);
  }
  std::vector<float*> p;
  for (auto& r : rows) p.push_back(r.data());
  const int d = (int)rows[0].size();
  try {
    switch (d) {
      case 4: run<4>(p.data(), (int)p.size(), max_d); break;
      case 7: run<7>(p.data(), (int)p.size(), max_d); break;
      case 12: run<12>(p.data(), (int)p.size(), max_d); break;
      default: return 3;
    }
  } catch (const skc::Error& e) {
    fprintf(stderr, "error %d: %s\n", e.code, e.what());
    return 2;
  }
  return 0;
}
