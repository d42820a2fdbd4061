// gbsph_motion.cpp -- predefined motion of moving boundaries (host side).
//
// Advances the movements of the moving objects once per step, as the
// reference's JDsMotion::ProcesTime(MOMT_Simple) does (JDsMotion.cpp:121-136)
// over JMotion::ProcesTimeSimple / ProcesTime (JMotion.cpp:473-600) and
// JMotionObj::ProcesTime (JMotionObj.cpp:446-690): events start movements,
// each object's active movements consume the interval and hand what is left
// of it to their chained movement, and the object's displacement is gathered
// as a vector or, once a rotation takes part, as a 4x4 matrix
// (JMotionPos.cpp, JMatrix4.h).  The arithmetic follows the reference's
// expressions operation by operation (double precision, no contraction), so
// the motion data equal the reference's.
//
// Objects are one level deep (the reference's <objreal> without child
// objects); movement types: wait, rectilinear (+acceleration), rotation
// (+acceleration), sinusoidal rectilinear and rotation, null.
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "gbsph.h"
#include "gbsph_motion_internal.h"

namespace {

constexpr double kTORAD = 0.017453292519943295769;  // PI/180 (TypesDef.h:29)
constexpr double kTODEG = 57.29577951308232087684;  // 180/PI (TypesDef.h:30)
constexpr double kPI = 3.14159265358979323846;
constexpr double kTWOPI = 6.28318530717958647692;

// JMatrix4<double> (JMatrix4.h:52-500): row-major a11..a44.
struct Mat4 {
  double a[16];
  Mat4() { identity(); }
  void identity() {
    for (int i = 0; i < 16; i++) a[i] = (i % 5 == 0) ? 1.0 : 0.0;
  }
  double& at(int r, int c) { return a[4 * r + c]; }
  double at(int r, int c) const { return a[4 * r + c]; }
  // this = this * m2 (JMatrix4::Mul, JMatrix4.h:153-172)
  void mul(const Mat4& m2) {
    const Mat4 m1 = *this;
    for (int r = 0; r < 4; r++)
      for (int c = 0; c < 4; c++)
        at(r, c) = m1.at(r, 0) * m2.at(0, c) + m1.at(r, 1) * m2.at(1, c) + m1.at(r, 2) * m2.at(2, c) +
                   m1.at(r, 3) * m2.at(3, c);
  }
  static Mat4 mov(const double* p) {  // MatrixMov (JMatrix4.h:316-320)
    Mat4 m;
    m.at(0, 3) = p[0];
    m.at(1, 3) = p[1];
    m.at(2, 3) = p[2];
    return m;
  }
  // MatrixRot (JMatrix4.h:465-500): rotation of ang degrees about the axis p1->p2
  static Mat4 rot(double ang, const double* p1, const double* p2) {
    const double rad = ang * kTORAD;
    const double vx = p2[0] - p1[0], vy = p2[1] - p1[1], vz = p2[2] - p1[2];
    const double L = std::sqrt(vx * vx + vy * vy + vz * vz);
    const double L1 = std::sqrt(vy * vy + vz * vz);
    Mat4 t, tm1, rx, rxm1, ry, rym1, rz;
    t.at(0, 3) = p1[0];
    t.at(1, 3) = p1[1];
    t.at(2, 3) = p1[2];
    tm1.at(0, 3) = -p1[0];
    tm1.at(1, 3) = -p1[1];
    tm1.at(2, 3) = -p1[2];
    if (L1 == 0) {
      rx.at(1, 1) = 0; rx.at(1, 2) = 1; rx.at(2, 1) = -1; rx.at(2, 2) = 0;
      rxm1.at(1, 1) = 0; rxm1.at(1, 2) = -1; rxm1.at(2, 1) = 1; rxm1.at(2, 2) = 0;
    } else {
      rx.at(1, 1) = vz / L1; rx.at(1, 2) = vy / L1; rx.at(2, 1) = -vy / L1; rx.at(2, 2) = vz / L1;
      rxm1.at(1, 1) = vz / L1; rxm1.at(1, 2) = -vy / L1; rxm1.at(2, 1) = vy / L1; rxm1.at(2, 2) = vz / L1;
    }
    ry.at(0, 0) = L1 / L; ry.at(0, 2) = vx / L; ry.at(2, 0) = -vx / L; ry.at(2, 2) = L1 / L;
    rym1.at(0, 0) = L1 / L; rym1.at(0, 2) = -vx / L; rym1.at(2, 0) = vx / L; rym1.at(2, 2) = L1 / L;
    const double cs = std::cos(rad), sn = std::sin(rad);
    rz.at(0, 0) = cs; rz.at(0, 1) = sn; rz.at(1, 0) = -sn; rz.at(1, 1) = cs;
    t.mul(rx);
    t.mul(ry);
    t.mul(rz);
    t.mul(rym1);
    t.mul(rxm1);
    t.mul(tm1);
    return t;
  }
};

// JMotionPos (JMotionPos.cpp): a displacement, or a matrix once rotated.
struct ModPos {
  bool simple = true;
  double ps[3] = {0, 0, 0};
  Mat4 m;
  void reset() {
    ps[0] = ps[1] = ps[2] = 0;
    m.identity();
    simple = true;
  }
  void move(const double* d) {
    if (simple) {
      ps[0] = ps[0] + d[0];
      ps[1] = ps[1] + d[1];
      ps[2] = ps[2] + d[2];
    } else {
      m.mul(Mat4::mov(d));
    }
  }
  void to_matrix() {
    if (simple) {
      m = Mat4::mov(ps);
      simple = false;
    }
  }
  void rotate(double ang, const double* p1, const double* p2) {
    if (simple) to_matrix();
    m.mul(Mat4::rot(ang, p1, p2));
  }
};

// A movement definition (JMotionMov*, with the unit conversions of
// JMotion::MovAdd*, JMotion.cpp:186-300).
struct Mov {
  int type = 0;
  unsigned id = 0, nextid = 0;
  double time = 0;
  bool prev = false;
  double vel[3] = {0, 0, 0}, ace[3] = {0, 0, 0};      // rect / rectace
  double freq[3] = {0, 0, 0}, ampl[3] = {0, 0, 0}, phase[3] = {0, 0, 0};  // rectsinu
  double axisp1[3] = {0, 0, 0}, axisp2[3] = {0, 0, 0};
  double velang = 0, aceang = 0;                       // rot / rotace (degrees)
  double freq1 = 0, ampl1 = 0, phase1 = 0;             // rotsinu (amplitude in degrees, phase in radians)
  const Mov* next = nullptr;
};

// An active movement (JMotionMovActive, JMotionObj.cpp:40-104, 260-280).
struct ActiveMov {
  double eventfinish, start, finish;
  bool flash, del = false;
  double vel[3] = {0, 0, 0}, velang = 0, phase[3] = {0, 0, 0}, phaseuni = 0;
  const Mov* mov;
  ActiveMov(double st, double efinish, const Mov* m) : eventfinish(efinish), start(st), mov(m) {
    flash = mov->time < 0;
    finish = flash ? start : start + mov->time;
    if (eventfinish >= 0 && eventfinish < finish) finish = eventfinish;
    config();
  }
  void config() {
    for (int k = 0; k < 3; k++) vel[k] = phase[k] = 0;
    velang = phaseuni = 0;
    switch (mov->type) {
      case GBSPH_MOV_RECT:
      case GBSPH_MOV_RECTACE:
        for (int k = 0; k < 3; k++) vel[k] = mov->vel[k];
        break;
      case GBSPH_MOV_ROT:
      case GBSPH_MOV_ROTACE: velang = mov->velang; break;
      case GBSPH_MOV_RECTSINU:
        for (int k = 0; k < 3; k++) phase[k] = mov->phase[k];
        break;
      case GBSPH_MOV_ROTSINU: phaseuni = mov->phase1; break;
      default: break;
    }
  }
  void next_mov() {
    if (!mov->next) return;
    if (!flash) start += mov->time;
    mov = mov->next;
    flash = mov->time < 0;
    finish = flash ? start : start + mov->time;
    if (eventfinish >= 0 && eventfinish < finish) finish = eventfinish;
    double velp[3] = {vel[0], vel[1], vel[2]}, phasep[3] = {phase[0], phase[1], phase[2]};
    const double velangp = velang, phaseunip = phaseuni;
    config();
    if (mov->type == GBSPH_MOV_RECTACE && mov->prev)
      for (int k = 0; k < 3; k++) vel[k] = velp[k];
    if (mov->type == GBSPH_MOV_ROTACE && mov->prev) velang = velangp;
    if (mov->type == GBSPH_MOV_RECTSINU && mov->prev)
      for (int k = 0; k < 3; k++) phase[k] = phasep[k];
    if (mov->type == GBSPH_MOV_ROTSINU && mov->prev) phaseuni = phaseunip;
  }
};

struct Obj {
  int ref = -1;
  std::vector<std::unique_ptr<Mov>> movs;
  std::vector<std::unique_ptr<ActiveMov>> active_movs;
  bool active = false, moving = false;
  ModPos modpos;

  const Mov* find(unsigned id) const {
    for (auto& m : movs)
      if (m->id == id) return m.get();
    return nullptr;
  }

  // One movement's share of the interval (the switch of JMotionObj::ProcesTime).
  void apply(ActiveMov& am, double dtmov) {
    const Mov* mv = am.mov;
    const double t = am.flash ? -mv->time : dtmov;
    switch (mv->type) {
      case GBSPH_MOV_RECT: {
        const double d[3] = {mv->vel[0] * t, mv->vel[1] * t, mv->vel[2] * t};
        modpos.move(d);
      } break;
      case GBSPH_MOV_RECTACE: {
        const double at[3] = {mv->ace[0] * t, mv->ace[1] * t, mv->ace[2] * t};
        const double d[3] = {am.vel[0] * t + 0.5 * at[0] * t, am.vel[1] * t + 0.5 * at[1] * t,
                             am.vel[2] * t + 0.5 * at[2] * t};
        modpos.move(d);
        for (int k = 0; k < 3; k++) am.vel[k] = am.vel[k] + at[k];
      } break;
      case GBSPH_MOV_ROT: modpos.rotate(mv->velang * t, mv->axisp1, mv->axisp2); break;
      case GBSPH_MOV_ROTACE: {
        const double at = mv->aceang * t;
        modpos.rotate(am.velang * t + 0.5 * at * t, mv->axisp1, mv->axisp2);
        am.velang += at;
      } break;
      case GBSPH_MOV_RECTSINU: {
        double ph[3] = {am.phase[0], am.phase[1], am.phase[2]};
        double p1[3] = {0, 0, 0}, p2[3] = {0, 0, 0};
        for (int k = 0; k < 3; k++) {
          if (mv->ampl[k] != 0) {
            p1[k] = mv->ampl[k] * std::sin(ph[k]);
            ph[k] += mv->freq[k] * kTWOPI * t;
            p2[k] = mv->ampl[k] * std::sin(ph[k]);
          }
        }
        const double d[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
        modpos.move(d);
        for (int k = 0; k < 3; k++) am.phase[k] = ph[k];
      } break;
      case GBSPH_MOV_ROTSINU: {
        double ph = am.phaseuni;
        double ang = mv->ampl1 * std::sin(ph);
        ph += mv->freq1 * (kPI + kPI) * t;
        ang = mv->ampl1 * std::sin(ph) - ang;
        modpos.rotate(ang, mv->axisp1, mv->axisp2);
        am.phaseuni = ph;
      } break;
      default: return;  // wait, null: no displacement
    }
    modif_ = true;
  }

  bool modif_ = false;

  // JMotionObj::ProcesTime for an object without parent or children.
  // Returns whether the object stays active; *moved: whether it moved.
  bool process(double timestep, double dt, bool* moved) {
    active = true;
    modif_ = false;
    int na = int(active_movs.size());
    if (na) {
      const double tstepfin = timestep + dt;
      modpos.reset();
      for (int ca = 0; ca < na; ca++) {
        ActiveMov& am = *active_movs[ca];
        if (am.del) {
          active_movs.erase(active_movs.begin() + ca);
          ca--;
          na--;
          continue;
        }
        double dt2 = dt, timestep2 = timestep;
        bool rep;
        do {
          rep = false;
          double dtmov = (tstepfin > am.finish ? am.finish - timestep2 : dt2);
          const double dtover = dt2 - dtmov;
          if (timestep2 < am.start) dtmov -= (am.start - timestep2);
          if (dtmov > 0 || am.flash) apply(am, dtmov);
          if ((dtover > 0 || dtmov == 0) && am.mov->next) {
            am.next_mov();
            dt2 = dtover;
            timestep2 = am.start;
            if (timestep2 <= am.finish || am.flash) rep = true;
          }
        } while (rep);
        if (tstepfin > am.finish) am.del = true;
      }
    }
    *moved = false;
    if (modif_) {
      *moved = true;
      moving = true;
    } else if (moving) {
      moving = false;
    } else if (!na) {
      active = false;
    }
    return active;
  }
};

struct Event {
  unsigned obj;
  const Mov* mov;
  double start, finish;
};

}  // namespace

struct gbsph_motion {
  std::vector<gbsph_motion_object> objinfo;
  std::vector<Obj> objs;       // by reference
  std::vector<Event> events;   // last-starting first (JMotion::Prepare)
  int eventnext = -1;
  bool objsactive = false;
  bool simulate2d = false;
  double list_timestep = 0;    // JMotionList::TimeStep
};

namespace gbmotion {
unsigned object_count(const gbsph_motion* m) { return m ? unsigned(m->objinfo.size()) : 0u; }
const gbsph_motion_object* objects(const gbsph_motion* m) { return m ? m->objinfo.data() : nullptr; }
}  // namespace gbmotion

extern "C" {

int gbsph_motion_create(unsigned nobj, const gbsph_motion_object* objs, unsigned nmov, const gbsph_movement* movs,
                        unsigned nevt, const gbsph_motion_event* evts, int simulate2d, gbsph_motion** out) {
  if (!out || (nobj && !objs) || (nmov && !movs) || (nevt && !evts) || nobj == 0) return GBSPH_EINVAL;
  *out = nullptr;
  std::unique_ptr<gbsph_motion> m(new gbsph_motion());
  m->simulate2d = simulate2d != 0;
  m->objinfo.assign(objs, objs + nobj);
  m->objs.resize(nobj);
  for (unsigned k = 0; k < nobj; k++) m->objs[k].ref = int(k);
  for (unsigned i = 0; i < nmov; i++) {
    const gbsph_movement& d = movs[i];
    if (d.obj >= nobj || d.type < GBSPH_MOV_WAIT || d.type > GBSPH_MOV_NULL) return GBSPH_EINVAL;
    if (d.type == GBSPH_MOV_WAIT && d.duration < 0) return GBSPH_EINVAL;  // JMotion::MovAddWait
    Obj& o = m->objs[d.obj];
    if (o.find(d.id)) return GBSPH_EINVAL;
    std::unique_ptr<Mov> mv(new Mov());
    mv->type = d.type;
    mv->id = d.id;
    mv->nextid = d.nextid;
    mv->time = d.type == GBSPH_MOV_NULL ? 0 : d.duration;
    mv->prev = d.prev != 0;
    const bool deg = d.angdegrees != 0;
    for (int k = 0; k < 3; k++) {
      mv->axisp1[k] = d.axisp1[k];
      mv->axisp2[k] = d.axisp2[k];
    }
    switch (d.type) {
      case GBSPH_MOV_RECT:
        for (int k = 0; k < 3; k++) mv->vel[k] = d.v[k];
        break;
      case GBSPH_MOV_RECTACE:
        for (int k = 0; k < 3; k++) {
          mv->ace[k] = d.a[k];
          mv->vel[k] = mv->prev ? 0 : d.v[k];
        }
        break;
      case GBSPH_MOV_ROT: mv->velang = deg ? d.s[0] : d.s[0] * kTODEG; break;
      case GBSPH_MOV_ROTACE:
        mv->velang = mv->prev ? 0 : d.s[0];
        mv->aceang = d.s[1];
        if (!deg) {
          mv->aceang = mv->aceang * kTODEG;
          mv->velang = mv->velang * kTODEG;
        }
        break;
      case GBSPH_MOV_RECTSINU:
        for (int k = 0; k < 3; k++) {
          mv->freq[k] = d.v[k];
          mv->ampl[k] = d.a[k];
          const double ph = mv->prev ? 0 : d.p[k];
          mv->phase[k] = deg ? ph * kTORAD : ph;
        }
        break;
      case GBSPH_MOV_ROTSINU: {
        mv->freq1 = d.s[0];
        mv->ampl1 = deg ? d.s[1] : d.s[1] * kTODEG;
        const double ph = mv->prev ? 0 : d.s[2];
        mv->phase1 = deg ? ph * kTORAD : ph;
      } break;
      default: break;
    }
    if ((d.type == GBSPH_MOV_ROT || d.type == GBSPH_MOV_ROTACE || d.type == GBSPH_MOV_ROTSINU) &&
        d.axisp1[0] == d.axisp2[0] && d.axisp1[1] == d.axisp2[1] && d.axisp1[2] == d.axisp2[2])
      return GBSPH_EINVAL;  // rotation axis with equal points
    o.movs.push_back(std::move(mv));
  }
  // JMotionObj::LinkMovs
  for (auto& o : m->objs)
    for (auto& mv : o.movs)
      if (mv->nextid) {
        mv->next = o.find(mv->nextid);
        if (!mv->next) return GBSPH_EINVAL;
      }
  for (unsigned i = 0; i < nevt; i++) {
    if (evts[i].obj >= nobj) return GBSPH_EINVAL;
    const Mov* mv = m->objs[evts[i].obj].find(evts[i].mov);
    if (!mv) return GBSPH_EINVAL;
    m->events.push_back(Event{evts[i].obj, mv, evts[i].start, evts[i].finish});
  }
  // JMotion::Prepare: events ordered from the last to start to the first
  auto& ev = m->events;
  if (ev.size())
    for (size_t c = 0; c + 1 < ev.size(); c++)
      for (size_t c2 = c + 1; c2 < ev.size(); c2++)
        if (ev[c].start < ev[c2].start) std::swap(ev[c], ev[c2]);
  m->eventnext = int(ev.size()) - 1;
  *out = m.release();
  return GBSPH_OK;
}

void gbsph_motion_destroy(gbsph_motion* m) { delete m; }

int gbsph_motion_process(gbsph_motion* m, double timestep, double dt, gbsph_motion_data* out) {
  if (!m || !out) return GBSPH_EINVAL;
  // JMotion::ProcesTimeSimple
  if (m->list_timestep > timestep) return GBSPH_EINVAL;  // times must not go back
  const size_t nobj = m->objs.size();
  std::vector<char> moved(nobj, 0);
  bool looking = true;
  if (m->eventnext >= 0)
    for (int c = m->eventnext; c >= 0 && looking; c--) {
      const Event& e = m->events[c];
      if (e.start < timestep + dt) {
        Obj& o = m->objs[e.obj];
        o.active_movs.emplace_back(new ActiveMov(e.start, e.finish, e.mov));
        o.active = true;
        m->eventnext--;
        m->objsactive = true;
      } else {
        looking = false;
      }
    }
  bool any = false;
  if (m->objsactive) {
    m->objsactive = false;
    for (size_t k = 0; k < nobj; k++) {
      Obj& o = m->objs[k];
      if (o.active) {
        bool mv = false;
        m->objsactive |= o.process(timestep, dt, &mv);
        moved[k] = mv;
      }
    }
    any = m->objsactive;
  }
  m->list_timestep = timestep + dt;
  // JMotionList::Sp_Movedt / GetData and JDsMotion::ProcesTime
  for (size_t k = 0; k < nobj; k++) {
    gbsph_motion_data& d = out[k];
    memset(&d, 0, sizeof(d));
    if (!any || !moved[k]) continue;
    const ModPos& mp = m->objs[k].modpos;
    if (mp.simple) {
      d.type = 1;
      for (int c = 0; c < 3; c++) {
        d.linmov[c] = mp.ps[c];
        d.linvel[c] = mp.ps[c] / dt;
      }
      if (m->simulate2d) d.linmov[1] = d.linvel[1] = 0;
    } else {
      d.type = 2;
      memcpy(d.mat, mp.m.a, sizeof(d.mat));
    }
  }
  return any ? 1 : 0;
}

}  // extern "C"
