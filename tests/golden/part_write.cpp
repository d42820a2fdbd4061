// part_write.cpp -- test infrastructure for tests/golden/make_golden.py.
//
// Writes a particle state that the reference harness dumped (its <tag>_idp,
// <tag>_pos, <tag>_velrho raw arrays and <tag>_meta.txt) as
// <dirout>/data/Part_<part>.bi4, with the run header Part_Head.ibi4, by
// gbsph_run's own writers (gbio::save_head, gbio::save_part), so that the
// reference can be restarted from files this library wrote.
//
//   part_write <casedir> <casename> <dumpdir> <tag> <part> <dirout>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "gbsph_io.h"

template <typename T>
static bool read_raw(const std::string& path, std::vector<T>& v) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  const long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  v.resize((size_t)n / sizeof(T));
  const size_t got = v.empty() ? 0 : std::fread(v.data(), sizeof(T), v.size(), f);
  std::fclose(f);
  return got == v.size();
}

int main(int argc, char** argv) {
  if (argc != 7) {
    std::fprintf(stderr, "usage: %s <casedir> <casename> <dumpdir> <tag> <part> <dirout>\n", argv[0]);
    return 1;
  }
  const std::string casedir = argv[1], casename = argv[2], dump = argv[3], tag = argv[4], dirout = argv[6];
  const unsigned part = (unsigned)std::atoi(argv[5]);
  gbio::Case cs;
  std::string err;
  if (!gbio::load_case(casedir, casename, cs, err)) { std::fprintf(stderr, "load_case: %s\n", err.c_str()); return 1; }
  std::vector<unsigned> idp;
  std::vector<double> pos;
  std::vector<float> velrho;
  const std::string b = dump + "/" + tag + "_";
  if (!read_raw(b + "idp.bin", idp) || !read_raw(b + "pos.bin", pos) || !read_raw(b + "velrho.bin", velrho) ||
      pos.size() != 3 * idp.size() || velrho.size() != 4 * idp.size()) {
    std::fprintf(stderr, "cannot read the dumped state %s*\n", b.c_str());
    return 1;
  }
  std::map<std::string, std::string> meta;
  std::ifstream mf(b + "meta.txt");
  for (std::string line; std::getline(mf, line);) {
    const size_t e = line.find('=');
    if (e != std::string::npos) meta[line.substr(0, e)] = line.substr(e + 1);
  }
  const double timestep = std::atof(meta["timestep"].c_str()), dtpre = std::atof(meta["symplecticdtpre"].c_str());
  const unsigned nstep = (unsigned)std::atol(meta["nstep"].c_str());
  if (!gbio::save_head(dirout, cs, part, err) ||
      !gbio::save_part(dirout, cs, part, timestep, nstep, dtpre, (unsigned)idp.size(), pos.data(), velrho.data(),
                       idp.data(), err)) {
    std::fprintf(stderr, "save_part: %s\n", err.c_str());
    return 1;
  }
  return 0;
}
