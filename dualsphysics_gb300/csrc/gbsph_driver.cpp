// gbsph_driver.cpp -- gbsph_run: the Run loop of JSphGpuSingle
// (JSphGpuSingle.cpp:950-1010) over the gbsph C ABI.
//
//   gbsph_run <casedir>/<casename> <dirout> [-nsteps:N] [-tmax:T] [-tout:T] [-sv:none|bi4]
//             [-cellmode:full|half] [-nograph] [-device:D] [-info]
//
// Loads the run XML and Case.bi4 (LoadConfig + LoadCaseParticles), derives the
// constants, uploads the particles, then steps until TimeMax (or N steps)
// writing data/Part_%04u.bi4 every TimeOut, and prints the run summary the
// reference prints at the end of Run.out (JSph::ShowResume, JSph.cpp:3522-3545).
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

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s <casedir>/<casename> <dirout> [-nsteps:N] [-tmax:T] [-tout:T] [-sv:none|bi4] "
                         "[-cellmode:full|half] [-nograph] [-device:D] [-info]\n", argv[0]);
    return 1;
  }
  std::string casepath = argv[1], dirout = argv[2];
  long nsteps = 0;
  double tmax = -1, toutarg = -1;
  bool save = true, graph = true, info = false;
  int cellmode_div = 1;  // -cellmode (JSphCfgRun.cpp:354-355): cells of 2h (full) or h (half)
  int device = 0;
  for (int i = 3; i < argc; i++) {
    const std::string a = argv[i];
    if (a.rfind("-nsteps:", 0) == 0) nsteps = std::atol(a.c_str() + 8);
    else if (a.rfind("-tmax:", 0) == 0) tmax = std::atof(a.c_str() + 6);
    else if (a.rfind("-tout:", 0) == 0) toutarg = std::atof(a.c_str() + 6);
    else if (a == "-sv:none") save = false;
    else if (a == "-sv:bi4") save = true;
    else if (a == "-nograph") graph = false;
    else if (a.rfind("-device:", 0) == 0) device = std::atoi(a.c_str() + 8);
    else if (a == "-info") info = true;
    else if (a == "-cellmode:half" || a == "-cellmode:h") cellmode_div = 2;
    else if (a == "-cellmode:full" || a == "-cellmode:2h") cellmode_div = 1;
    else if (a == "-gpu" || a == "-symplectic") continue;
    else return fail("options", "unknown option " + a);
  }
  const size_t slash = casepath.find_last_of('/');
  const std::string casedir = slash == std::string::npos ? "." : casepath.substr(0, slash);
  const std::string casename = slash == std::string::npos ? casepath : casepath.substr(slash + 1);
  gbio::Case cs;
  std::string err;
  if (!gbio::load_case(casedir, casename, cs, err)) return fail("LoadCase", err);
  cs.params.cellmode_div = cellmode_div;
  gbsph_consts c;
  if (gbsph_config(&cs.params, &c) != GBSPH_OK) return fail("ConfigConstants", "invalid case constants");
  if (info) {
    // case summary as JSON (host only: no device is touched)
    std::printf("{\"np\": %u, \"npb\": %u, \"h\": %.17g, \"b\": %.17g, \"dp\": %.17g, \"maprealposmin\": "
                "[%.17g, %.17g, %.17g], \"maprealposmax\": [%.17g, %.17g, %.17g], \"kernelsize2\": %.9g, "
                "\"cs0\": %.17g, \"domcellcode\": %u, \"mapcells\": [%u, %u, %u], \"cellmode_div\": %d, \"tboundary\": %d, "
                "\"tstep\": %d, \"tdensity\": %d, \"tvisco\": %d, \"idsum\": %.17g, \"possum\": %.17g, "
                "\"rhosum\": %.17g, \"norsum\": %.17g, \"codesum\": %.17g, \"nmoving\": %u, \"nmovements\": %u, "
                "\"nevents\": %u}\n",
                cs.np, cs.npb, cs.params.h, cs.params.b, cs.params.dp, cs.params.maprealposmin[0],
                cs.params.maprealposmin[1], cs.params.maprealposmin[2], cs.params.maprealposmax[0],
                cs.params.maprealposmax[1], cs.params.maprealposmax[2], c.kernelsize2, c.cs0, c.domcellcode,
                c.mapcells[0], c.mapcells[1], c.mapcells[2], c.cellmode_div, c.tboundary, c.tstep, c.tdensity, c.tvisco,
                [&] { double s = 0; for (unsigned v : cs.idp) s += v; return s; }(),
                [&] { double s = 0; for (double v : cs.pos) s += v; return s; }(),
                [&] { double s = 0; for (size_t k = 3; k < cs.velrho.size(); k += 4) s += cs.velrho[k]; return s; }(),
                [&] { double s = 0; for (float v : cs.boundnor) s += v; return s; }(),
                [&] { double s = 0; for (uint16_t v : cs.code) s += v; return s; }(), cs.nmoving,
                (unsigned)cs.movs.size(), (unsigned)cs.evts.size());
    return 0;
  }
  gbsph_ctx* ctx = nullptr;
  // room for the periodic copies: each periodic axis can copy every particle once
  const unsigned cap = cs.np * (1u + (c.peri[0] ? 1u : 0u) + (c.peri[1] ? 1u : 0u) + (c.peri[2] ? 1u : 0u));
  int rc = gbsph_create(&c, cap, device, &ctx);
  if (rc != GBSPH_OK) return fail("gbsph_create", "code " + std::to_string(rc));
  rc = gbsph_upload(ctx, cs.np, cs.npb, cs.pos.data(), cs.velrho.data(), cs.idp.data(), cs.code.data(),
                    cs.boundnor.empty() ? nullptr : cs.boundnor.data());
  if (rc != GBSPH_OK) return fail("gbsph_upload", gbsph_last_error(ctx));
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
  if (!save_part(0, 0.0, 0, c.dtini)) return fail("SaveData", err.empty() ? gbsph_last_error(ctx) : err);
  unsigned part = 1, nstep = 0;
  double t = 0, tnext = tout, dtl = 0, dtn = c.dtini;
  const bool sym = c.tstep == GBSPH_STEP_SYMPLECTIC;
  const auto t0 = std::chrono::steady_clock::now();
  while (t < tmax && (nsteps == 0 || (long)nstep < nsteps)) {
    rc = sym ? gbsph_run(ctx, 1, graph ? 1 : 0) : gbsph_step(ctx);
    if (rc != GBSPH_OK) return fail("ComputeStep", gbsph_last_error(ctx));
    rc = gbsph_step_dt(ctx, &dtl, &dtn, &t);
    if (rc != GBSPH_OK) return fail("ComputeStep", gbsph_last_error(ctx));
    nstep++;
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
  gbsph_destroy(ctx);
  gbsph_motion_destroy(motion);
  return 0;
}
