// gbsph_driver.cpp -- gbsph_run: the Run loop of JSphGpuSingle
// (JSphGpuSingle.cpp:950-1010) over the gbsph C ABI.
//
//   gbsph_run <casedir>/<casename> <dirout> [-nsteps:N] [-tmax:T] [-tout:T] [-sv:none|bi4]
//             [-partbegin:N[:first] dir] [-cellmode:full|half] [-nograph] [-device:D] [-info]
//
// Loads the run XML and Case.bi4 (LoadConfig + LoadCaseParticles), derives the
// constants, uploads the particles, then steps until TimeMax (or N steps)
// writing data/Part_%04u.bi4 every TimeOut, and prints the run summary the
// reference prints at the end of Run.out (JSph::ShowResume, JSph.cpp:3522-3545).
#include <sys/stat.h>

#include <cctype>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "gbsph.h"
#include "gbsph_io.h"

namespace {

int fail(const char* what, const std::string& msg) {
  std::fprintf(stderr, "*** Exception: %s: %s\n", what, msg.c_str());
  return 1;
}

// Part files are written off the stepping thread: the particle data is read
// back into one of two host buffer sets, and a writer thread sorts it by id,
// encodes it and writes the file while the GPU goes on stepping (the reference
// writes its Parts inline in the Run loop).  With both buffer sets in use the
// next save waits for the writer, so at most two Parts are held in memory.
class PartWriter {
 public:
  struct Job {
    std::vector<double> pos;
    std::vector<float> velrho;
    std::vector<unsigned> idp;
    std::vector<uint16_t> code;
    unsigned part = 0, step = 0, np = 0;
    double t = 0, dtn = 0;
  };

  // cap: the particles the device may hold (periodic copies included)
  PartWriter(const std::string& dirout, const gbio::Case& cs, unsigned cap)
      : dirout_(dirout), cs_(cs), th_([this] { loop(); }) {
    std::lock_guard<std::mutex> lk(mu_);
    for (auto& b : bufs_) {
      b.pos.resize(3 * (size_t)cap);
      b.velrho.resize(4 * (size_t)cap);
      b.idp.resize(cap);
      b.code.resize(cap);
      free_.push_back(&b);
    }
  }
  ~PartWriter() { finish(); }

  // A free buffer set (waits while both are being written).
  Job* acquire() {
    std::unique_lock<std::mutex> lk(mu_);
    cv_.wait(lk, [this] { return !free_.empty(); });
    Job* j = free_.back();
    free_.pop_back();
    return j;
  }
  // Returns a buffer set unwritten.
  void release(Job* j) {
    { std::lock_guard<std::mutex> lk(mu_); free_.push_back(j); }
    cv_.notify_all();
  }
  void submit(Job* j) {
    { std::lock_guard<std::mutex> lk(mu_); todo_.push_back(j); }
    cv_.notify_all();
  }
  // Waits for every submitted Part; returns false (with the message) if a write failed.
  bool finish() {
    std::unique_lock<std::mutex> lk(mu_);
    if (!stop_) {
      cv_.wait(lk, [this] { return todo_.empty() && free_.size() == 2; });
      stop_ = true;
      lk.unlock();
      cv_.notify_all();
      th_.join();
      lk.lock();
    }
    return err_.empty();
  }
  std::string error() {
    std::lock_guard<std::mutex> lk(mu_);
    return err_;
  }
  double write_seconds() const { return write_s_; }

 private:
  void loop() {
    for (;;) {
      Job* j = nullptr;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [this] { return stop_ || !todo_.empty(); });
        if (todo_.empty()) return;
        j = todo_.front();
        todo_.erase(todo_.begin());
      }
      const auto t0 = std::chrono::steady_clock::now();
      // only normal particles are saved, not periodic copies (GetParticlesData
      // with onlynormal, JSphCpu.cpp:366-424)
      unsigned n = 0;
      for (unsigned p = 0; p < j->np; p++) {
        if (j->code[p] & 0xe000u) continue;
        if (n != p) {
          for (int k = 0; k < 3; k++) j->pos[3 * (size_t)n + k] = j->pos[3 * (size_t)p + k];
          for (int k = 0; k < 4; k++) j->velrho[4 * (size_t)n + k] = j->velrho[4 * (size_t)p + k];
          j->idp[n] = j->idp[p];
        }
        n++;
      }
      j->np = n;
      std::string e;
      const bool ok = gbio::save_part(dirout_, cs_, j->part, j->t, j->step, j->dtn, j->np, j->pos.data(),
                                      j->velrho.data(), j->idp.data(), e);
      write_s_ += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      {
        std::lock_guard<std::mutex> lk(mu_);
        if (!ok && err_.empty()) err_ = e;
        free_.push_back(j);
      }
      cv_.notify_all();
    }
  }

  std::string dirout_;
  const gbio::Case& cs_;
  Job bufs_[2];
  std::vector<Job*> free_, todo_;
  std::mutex mu_;
  std::condition_variable cv_;
  bool stop_ = false;
  std::string err_;
  double write_s_ = 0;
  std::thread th_;
};


// Command-line options: the subset of JSphCfgRun::LoadOpts (JSphCfgRun.cpp:
// 300-530) that bears on this path, same spelling (case-insensitive words,
// values after ':'), plus -nograph, -device:D and -info of this driver.
struct RunOptions {
  long nsteps = 0;
  double tmax = -1, tout = -1;
  bool save = true, graph = true, info = false;
  int cellmode_div = 1;  // cells of 2h (full) or h (half)
  int device = 0;
  // overrides of the case parameters (-1 / 0: not given)
  int tstep = 0, verletsteps = -1, tboundary = -1, tvisco = 0, tdensity = -1;
  float visco = 0, viscoboundfactor = -1, ddtvalue = -1;
  double cfl = 0;
  bool rhopout = false;
  float rhopoutmin = 0, rhopoutmax = 0;
  unsigned pipsmode = 0, pipssteps = 100;
  // restart (-partbegin:begin[:first] dir, JSphCfgRun): the Part to begin
  // from, the number of the first Part written, the directory of the Part
  unsigned partbegin = 0, partbeginfirst = 0;
  std::string partbegindir;
};

std::string upper(std::string t) {
  for (char& ch : t) ch = (char)std::toupper((unsigned char)ch);
  return t;
}

// One option; returns an empty string or the error.
std::string parse_option(const std::string& arg, RunOptions& o) {
  if (arg.size() < 2 || arg[0] != '-') return "unknown option " + arg;
  const size_t colon = arg.find(':');
  const std::string word = upper(arg.substr(1, colon == std::string::npos ? std::string::npos : colon - 1));
  const std::string full = colon == std::string::npos ? "" : arg.substr(colon + 1);
  const size_t c2 = full.find(':');
  const std::string opt1 = full.substr(0, c2), opt2 = c2 == std::string::npos ? "" : full.substr(c2 + 1);
  const auto enabled = [&] { return full.empty() || std::atoi(full.c_str()) != 0; };
  const std::string bad = "invalid option " + arg;
  if (word == "GPU") { if (!full.empty()) o.device = std::atoi(full.c_str()); }
  else if (word == "CPU") return "the CPU solver is not part of this library (" + arg + ")";
  else if (word == "SYMPLECTIC") o.tstep = GBSPH_STEP_SYMPLECTIC;
  else if (word == "VERLET") { o.tstep = GBSPH_STEP_VERLET; if (!full.empty()) o.verletsteps = std::atoi(full.c_str()); }
  else if (word == "WENDLAND") {}
  else if (word == "CUBIC") return "the cubic spline kernel is not supported (" + arg + ")";
  else if (word == "DBC") o.tboundary = GBSPH_BC_DBC;
  else if (word == "MDBC") o.tboundary = GBSPH_BC_MDBC;
  else if (word == "MDBC_NOSLIP" || word == "MDBC_FREESLIP") return "mDBC slip modes other than vel=0 are not supported (" + arg + ")";
  else if (word == "VISCOART") { o.visco = (float)std::atof(full.c_str()); if (o.visco > 10) return bad; o.tvisco = GBSPH_VISCO_ARTIFICIAL; }
  else if (word == "VISCOLAM") { o.visco = (float)std::atof(full.c_str()); if (o.visco > 0.001f) return bad; o.tvisco = GBSPH_VISCO_LAMINAR; }
  else if (word == "VISCOLAMSPS") { o.visco = (float)std::atof(full.c_str()); if (o.visco > 0.001f) return bad; o.tvisco = GBSPH_VISCO_LAMINARSPS; }
  else if (word == "VISCOBOUNDFACTOR") { o.viscoboundfactor = (float)std::atof(full.c_str()); if (o.viscoboundfactor < 0) return bad; }
  else if (word == "DDT") { const int v = std::atoi(full.c_str()); if (v < 0 || v > 3) return bad; o.tdensity = v; }
  else if (word == "DDTVALUE") { o.ddtvalue = (float)std::atof(full.c_str()); if (o.ddtvalue < 0 || o.ddtvalue > 1) return bad; }
  else if (word == "RHOPOUT") { o.rhopoutmin = (float)std::atof(opt1.c_str()); o.rhopoutmax = (float)std::atof(opt2.c_str()); o.rhopout = true; }
  else if (word == "CFL") { o.cfl = std::atof(full.c_str()); if (o.cfl <= 0) return bad; }
  else if (word == "TMAX") { o.tmax = std::atof(full.c_str()); if (o.tmax < 0) return bad; }
  else if (word == "TOUT") { o.tout = std::atof(full.c_str()); if (o.tout < 0) return bad; }
  else if (word == "NSTEPS") o.nsteps = std::atol(full.c_str());
  else if (word == "SV") {
    std::string rest = upper(full);
    while (!rest.empty()) {
      const size_t k = rest.find(',');
      const std::string f = rest.substr(0, k);
      rest = k == std::string::npos ? "" : rest.substr(k + 1);
      if (f == "NONE") o.save = false;
      else if (f == "BINX" || f == "BIN" || f == "BI4") o.save = true;
      else return "output format " + f + " is not supported (" + arg + ")";
    }
  }
  else if (word == "SVPIPS") {
    o.pipsmode = (unsigned)std::atoi(opt1.c_str());
    if (o.pipsmode > 2) return bad;
    if (!opt2.empty()) o.pipssteps = (unsigned)std::atoi(opt2.c_str());
    if (o.pipssteps == 0) o.pipssteps = 1;
  }
  else if (word == "CELLMODE") {
    const std::string v = upper(full);
    if (v == "HALF" || v == "H") o.cellmode_div = 2;
    else if (v == "FULL" || v == "2H") o.cellmode_div = 1;
    else return bad;
  }
  // accepted without effect: stable summation is the only mode here, run times
  // and timers are printed in the summary
  else if (word == "STABLE" || word == "NORTIMES" || word == "SVTIMERS") { (void)enabled; }
  else if (word == "PARTBEGIN") {
    if (opt1.empty() || std::atol(opt1.c_str()) <= 0) return bad;
    o.partbegin = (unsigned)std::atol(opt1.c_str());
    o.partbeginfirst = opt2.empty() ? 0u : (unsigned)std::atol(opt2.c_str());
  }
  else if (word == "NOGRAPH") o.graph = false;
  else if (word == "DEVICE") o.device = std::atoi(full.c_str());
  else if (word == "INFO") o.info = true;
  else return "unknown option " + arg;
  return "";
}

// The command line's overrides of the case parameters (JSph::LoadConfigCommands,
// JSph.cpp:876-995).
std::string apply_options(const RunOptions& o, gbio::Case& cs) {
  gbsph_params& p = cs.params;
  p.cellmode_div = o.cellmode_div;
  if (o.tboundary >= 0) p.tboundary = o.tboundary;
  if (p.tboundary == GBSPH_BC_MDBC && cs.boundnor.empty()) return "mDBC needs the boundary normals in the case";
  if (o.tstep) p.tstep = o.tstep;
  if (o.verletsteps >= 0) p.verletsteps = o.verletsteps;
  if (o.tvisco) { p.tvisco = o.tvisco; p.visco = o.visco; }
  if (o.viscoboundfactor >= 0) p.viscoboundfactor = o.viscoboundfactor;
  if (o.tdensity >= 0) {
    p.tdensity = o.tdensity;
    if (o.ddtvalue >= 0) p.ddtvalue = o.ddtvalue;
    else if (p.ddtvalue == 0) p.ddtvalue = 0.1f;
  }
  if (p.tdensity == GBSPH_DDT_NONE) p.ddtvalue = 0;
  else if (o.ddtvalue >= 0) p.ddtvalue = o.ddtvalue;
  if (o.cfl > 0) p.cflnumber = o.cfl;
  if (o.rhopout) { p.rhopoutmin = o.rhopoutmin; p.rhopoutmax = o.rhopoutmax; }
  return "";
}

// PIPS sampling (JDsPips, JDsPips.cpp:72-181): interaction counts taken every
// `steps` steps and at the last one; the interactions between two samples are
// integrated by the trapezoid rule, times the interaction passes per step.
struct PipsSample {
  unsigned nstep;
  double tstep, tsim;
  unsigned long long picb, pirb, picf, pirf;
};

struct Pips {
  unsigned steps = 100, ntimes = 2, next = 0;
  std::vector<PipsSample> data;
  bool take(gbsph_ctx* ctx, unsigned nstep, double t, double tsim) {
    unsigned long long v[4];
    if (gbsph_pips(ctx, v) != GBSPH_OK) return false;
    data.push_back({nstep, t, tsim, v[0], v[1], v[2], v[3]});
    next += steps;
    return true;
  }
  // GigaPIs of interval c (fluid rows or boundary rows)
  double gpis(size_t c, bool fluid, bool real = true) const {
    const PipsSample &a = data[c - 1], &b = data[c];
    const double p0 = (double)(real ? (fluid ? a.pirf : a.pirb) : (fluid ? a.picf : a.picb));
    const double p1 = (double)(real ? (fluid ? b.pirf : b.pirb) : (fluid ? b.picf : b.picb));
    const double n = (double)(b.nstep - a.nstep + 1);
    return ((p0 / 2 + p1 / 2) * n - p1) / 1e9 * ntimes;
  }
  void totals(double& f, double& b) const {
    f = b = 0;
    for (size_t c = 1; c < data.size(); c++) { f += gpis(c, true); b += gpis(c, false); }
  }
  // PIPS.csv of JDsPips::SaveData (JDsPips.cpp:114-141)
  bool save_csv(const std::string& dirout) const {
    mkdir(dirout.c_str(), 0755);  // may exist already
    FILE* fp = std::fopen((dirout + "/PIPS.csv").c_str(), "w");
    if (!fp) return false;
    std::fprintf(fp, "Time [s];RunTime [s];Nstep;RealFluid [PIs];RealBound [PIs];ChkFluid [PIs];ChkBound [PIs];"
                     "GPIPS;SumRealFluid [GPIs];SumRealBound [GPIs];SumChkFluid [GPIs];SumChkBound [GPIs]\n");
    double rf = 0, rb = 0, cf = 0, cb = 0;
    for (size_t c = 0; c < data.size(); c++) {
      const PipsSample& v = data[c];
      if (c) { rf += gpis(c, true); rb += gpis(c, false); cf += gpis(c, true, false); cb += gpis(c, false, false); }
      const double g = v.tsim > 0 ? (rf + rb) / v.tsim : 0;
      std::fprintf(fp, "%.9g;%.9g;%u;%llu;%llu;%llu;%llu;%.9g;%.9g;%.9g;%.9g;%.9g\n", v.tstep, v.tsim, v.nstep,
                   v.pirf, v.pirb, v.picf, v.picb, g, rf, rb, cf, cb);
    }
    return std::fclose(fp) == 0;
  }
};

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s <casedir>/<casename> <dirout> [-gpu[:id]] [-symplectic|-verlet[:steps]] "
                         "[-dbc|-mdbc] [-viscoart:v|-viscolam:v|-viscolamsps:v] [-viscoboundfactor:v] [-ddt:0-3] "
                         "[-ddtvalue:v] [-rhopout:min:max] [-cfl:v] [-tmax:T] [-tout:T] [-nsteps:N] [-sv:none|binx] "
                         "[-svpips:0-2[:steps]] [-partbegin:N[:first] dir] [-cellmode:full|half] [-stable] [-nortimes] "
                         "[-svtimers] [-nograph] "
                         "[-device:D] [-info]\n", argv[0]);
    return 1;
  }
  std::string casepath = argv[1], dirout = argv[2];
  RunOptions o;
  for (int i = 3; i < argc; i++) {
    const std::string e = parse_option(argv[i], o);
    if (!e.empty()) return fail("options", e);
    if (o.partbegin && o.partbegindir.empty()) {  // -partbegin:begin[:first] takes the directory next
      if (i + 1 >= argc) return fail("options", "-partbegin needs the directory of the Part files");
      o.partbegindir = argv[++i];
    }
  }
  const long nsteps = o.nsteps;
  double tmax = o.tmax;
  const double toutarg = o.tout;
  const bool save = o.save, graph = o.graph, info = o.info;
  const int device = o.device;
  const size_t slash = casepath.find_last_of('/');
  const std::string casedir = slash == std::string::npos ? "." : casepath.substr(0, slash);
  const std::string casename = slash == std::string::npos ? casepath : casepath.substr(slash + 1);
  gbio::Case cs;
  std::string err;
  if (!gbio::load_case(casedir, casename, cs, err)) return fail("LoadCase", err);
  err = apply_options(o, cs);
  if (!err.empty()) return fail("LoadCase", err);
  gbsph_consts c;
  if (gbsph_config(&cs.params, &c) != GBSPH_OK) return fail("ConfigConstants", "invalid case constants");
  // restart from a Part file (JPartsLoad4::LoadParticles, JSph::InitRun):
  // with first = 0 the run's clock starts at 0, otherwise at the Part's time;
  // SymplecticDtPre is the Part's
  double t_ini = 0, dtpre_ini = 0, part_time = 0;
  if (o.partbegin) {
    if (!cs.mot_objs.empty()) return fail("LoadCase", "a restart with moving boundaries is not supported");
    if (!gbio::load_part(o.partbegindir, o.partbegin, cs, part_time, dtpre_ini, err)) return fail("LoadPart", err);
    t_ini = o.partbeginfirst ? part_time : 0.0;
  }
  if (info) {
    // case summary as JSON (host only: no device is touched)
    std::printf("{\"np\": %u, \"npb\": %u, \"h\": %.17g, \"b\": %.17g, \"dp\": %.17g, \"maprealposmin\": "
                "[%.17g, %.17g, %.17g], \"maprealposmax\": [%.17g, %.17g, %.17g], \"kernelsize2\": %.9g, "
                "\"cs0\": %.17g, \"domcellcode\": %u, \"mapcells\": [%u, %u, %u], \"cellmode_div\": %d, \"tboundary\": %d, "
                "\"tstep\": %d, \"tdensity\": %d, \"tvisco\": %d, \"idsum\": %.17g, \"possum\": %.17g, "
                "\"rhosum\": %.17g, \"norsum\": %.17g, \"codesum\": %.17g, \"nmoving\": %u, \"nmovements\": %u, "
                "\"nevents\": %u, \"verletsteps\": %d, \"visco\": %.9g, \"viscoboundfactor\": %.9g, "
                "\"ddtvalue\": %.9g, \"cflnumber\": %.17g, \"rhopoutmin\": %.9g, \"rhopoutmax\": %.9g, "
                "\"parttime\": %.17g, \"timeini\": %.17g, \"dtpre\": %.17g}\n",
                cs.np, cs.npb, cs.params.h, cs.params.b, cs.params.dp, cs.params.maprealposmin[0],
                cs.params.maprealposmin[1], cs.params.maprealposmin[2], cs.params.maprealposmax[0],
                cs.params.maprealposmax[1], cs.params.maprealposmax[2], c.kernelsize2, c.cs0, c.domcellcode,
                c.mapcells[0], c.mapcells[1], c.mapcells[2], c.cellmode_div, c.tboundary, c.tstep, c.tdensity, c.tvisco,
                [&] { double s = 0; for (unsigned v : cs.idp) s += v; return s; }(),
                [&] { double s = 0; for (double v : cs.pos) s += v; return s; }(),
                [&] { double s = 0; for (size_t k = 3; k < cs.velrho.size(); k += 4) s += cs.velrho[k]; return s; }(),
                [&] { double s = 0; for (float v : cs.boundnor) s += v; return s; }(),
                [&] { double s = 0; for (uint16_t v : cs.code) s += v; return s; }(), cs.nmoving,
                (unsigned)cs.movs.size(), (unsigned)cs.evts.size(), cs.params.verletsteps, cs.params.visco,
                cs.params.viscoboundfactor, cs.params.ddtvalue, cs.params.cflnumber, cs.params.rhopoutmin,
                cs.params.rhopoutmax, part_time, t_ini, dtpre_ini);
    return 0;
  }
  gbsph_ctx* ctx = nullptr;
  // room for the periodic copies: at most 2^k - 1 per particle over k periodic
  // axes, and the copies of the last divide are still held while the new ones
  // are made
  const unsigned nperi = (c.peri[0] ? 1u : 0u) + (c.peri[1] ? 1u : 0u) + (c.peri[2] ? 1u : 0u);
  const unsigned long long capl = (unsigned long long)cs.np * (1ull + 2ull * ((1ull << nperi) - 1ull));
  if (capl > 0x7fffffffull) return fail("gbsph_create", "the periodic copies would not fit 2^31 particles");
  const unsigned cap = (unsigned)capl;
  int rc = gbsph_create(&c, cap, device, &ctx);
  if (rc != GBSPH_OK) return fail("gbsph_create", "code " + std::to_string(rc));
  rc = gbsph_upload(ctx, cs.np, cs.npb, cs.pos.data(), cs.velrho.data(), cs.idp.data(), cs.code.data(),
                    cs.boundnor.empty() ? nullptr : cs.boundnor.data());
  if (rc != GBSPH_OK) return fail("gbsph_upload", gbsph_last_error(ctx));
  if (o.partbegin) {
    const bool symp = c.tstep == GBSPH_STEP_SYMPLECTIC;
    rc = gbsph_set_step_state(ctx, t_ini, symp ? dtpre_ini : 0.0);
    if (rc != GBSPH_OK) return fail("LoadPart", gbsph_last_error(ctx));
  }
  // moving boundaries: JDsMotion::Init from the case's motion (JSph.cpp:1064-1067)
  gbsph_motion* motion = nullptr;
  if (!cs.mot_objs.empty()) {
    rc = gbsph_motion_create((unsigned)cs.mot_objs.size(), cs.mot_objs.data(), (unsigned)cs.movs.size(),
                             cs.movs.data(), (unsigned)cs.evts.size(), cs.evts.data(), cs.params.simulate2d, &motion);
    if (rc != GBSPH_OK) return fail("motion", "invalid motion in the case XML");
    rc = gbsph_set_motion(ctx, motion);
    if (rc != GBSPH_OK) return fail("motion", gbsph_last_error(ctx));
  }
  if (tmax < 0) tmax = cs.time_max;
  const double tout = toutarg > 0 ? toutarg : (cs.time_out > 0 ? cs.time_out : tmax);
  std::printf("Case %s: %u particles (%u boundary, %u fluid), h=%g, dp=%g\n", casename.c_str(), cs.np, cs.npb,
              cs.np - cs.npb, cs.params.h, cs.params.dp);
  gbsph_divinfo di;
  PartWriter writer(dirout, cs, cap);
  auto save_part = [&](unsigned part, double t, unsigned step, double dtn) -> bool {
    if (!save) return true;
    const std::string werr = writer.error();
    if (!werr.empty()) { err = werr; return false; }
    if (gbsph_get_divinfo(ctx, &di, nullptr, 0, nullptr, nullptr) != GBSPH_OK) return false;
    PartWriter::Job* j = writer.acquire();
    if (gbsph_download(ctx, j->pos.data(), j->velrho.data(), j->idp.data(), j->code.data(), nullptr) != GBSPH_OK) {
      writer.release(j);
      return false;
    }
    j->part = part; j->t = t; j->step = step; j->dtn = dtn; j->np = di.np;
    writer.submit(j);
    return true;
  };
  const double dt_ini = (o.partbegin && dtpre_ini > 0) ? dtpre_ini : c.dtini;
  const unsigned part_ini = o.partbegin ? o.partbeginfirst : 0u;
  if (save && !gbio::save_head(dirout, cs, part_ini, err)) return fail("SaveData", err);
  if (!save_part(part_ini, t_ini, 0, dt_ini)) return fail("SaveData", err.empty() ? gbsph_last_error(ctx) : err);
  unsigned part = part_ini + 1, nstep = 0;
  double t = t_ini, tnext = t_ini + tout, dtl = 0, dtn = dt_ini;
  const bool sym = c.tstep == GBSPH_STEP_SYMPLECTIC;
  const auto t0 = std::chrono::steady_clock::now();
  const auto runtime = [&] { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); };
  Pips pips;
  pips.steps = o.pipssteps;
  pips.ntimes = sym ? 2 : 1;
  if (o.pipsmode && !pips.take(ctx, 0, 0.0, 0.0)) return fail("ComputePips", gbsph_last_error(ctx));
  while (t < tmax && (nsteps == 0 || (long)nstep < nsteps)) {
    rc = sym ? gbsph_run(ctx, 1, graph ? 1 : 0) : gbsph_step(ctx);
    if (rc != GBSPH_OK) return fail("ComputeStep", gbsph_last_error(ctx));
    rc = gbsph_step_dt(ctx, &dtl, &dtn, &t);
    if (rc != GBSPH_OK) return fail("ComputeStep", gbsph_last_error(ctx));
    nstep++;
    const bool last = !(t < tmax && (nsteps == 0 || (long)nstep < nsteps));
    if (o.pipsmode && (last || nstep >= pips.next) && !pips.take(ctx, nstep, t, runtime()))
      return fail("ComputePips", gbsph_last_error(ctx));
    if (t >= tnext) {
      if (!save_part(part, t, nstep, dtn)) return fail("SaveData", err.empty() ? gbsph_last_error(ctx) : err);
      part++;
      tnext += tout;
    }
  }
  const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (!writer.finish()) return fail("SaveData", writer.error());
  gbsph_get_divinfo(ctx, &di, nullptr, 0, nullptr, nullptr);
  std::printf("Simulated time: %.6f s in %u steps (last dt %.6e)\n", t, nstep, dtl);
  std::printf("Particles: %u (excluded %u)\n", di.np, di.nout_total);
  std::printf("Runtime: %.3f s\nSteps per second: %.3f\n", wall, nstep / (wall > 0 ? wall : 1));
  if (save) std::printf("Part writing (overlapped with the steps): %.3f s\n", writer.write_seconds());
  if (o.pipsmode) {  // JSph::ShowResume (JSph.cpp:3543-3546)
    double f, b;
    pips.totals(f, b);
    std::printf("Particle Interactions Per Second.: %.8f GPIPS\n", wall > 0 ? (f + b) / wall : 0.0);
    std::printf("Total particle interactions (f+b): %.6f GPIs (%.4e + %.4e)\n", f + b, f * 1e9, b * 1e9);
    if (o.pipsmode == 2 && !pips.save_csv(dirout)) return fail("SavePips", "cannot write " + dirout + "/PIPS.csv");
  }
  gbsph_destroy(ctx);
  gbsph_motion_destroy(motion);
  return 0;
}
