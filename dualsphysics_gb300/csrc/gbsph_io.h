// gbsph_io.h -- case input and particle output for the gbsph_run driver.
//
// Reads the reference's run XML (case.execution.{constants,parameters,
// particles}: JCaseCtes.cpp:208-222, JSph.cpp:663-857, JCaseParts.cpp:540-577)
// and its particle files in the JBinaryData container (JBinaryData.cpp:736-1420,
// JPartDataBi4.cpp:169-470); writes data/Part_%04u.bi4.
#pragma once
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "gbsph.h"

namespace gbio {

// ---- minimal XML tree --------------------------------------------------------
struct XmlNode {
  std::string name;
  std::map<std::string, std::string> attr;
  std::vector<std::unique_ptr<XmlNode>> kids;
  const XmlNode* child(const std::string& n) const;
  std::vector<const XmlNode*> children(const std::string& n) const;
  bool has(const std::string& a) const { return attr.count(a) != 0; }
  std::string get(const std::string& a, const std::string& def = "") const;
  double getd(const std::string& a) const;
};
std::unique_ptr<XmlNode> xml_parse_file(const std::string& path, std::string& err);

// ---- JBinaryData container ---------------------------------------------------
enum DatType {
  DatText = 1, DatBool = 2, DatChar = 3, DatUchar = 4, DatShort = 5, DatUshort = 6, DatInt = 7, DatUint = 8,
  DatLlong = 9, DatUllong = 10, DatFloat = 11, DatDouble = 12, DatInt3 = 20, DatUint3 = 21, DatFloat3 = 22,
  DatDouble3 = 23
};

struct Bi4Value {
  int type = 0;
  std::string text;
  double num[3] = {0, 0, 0};  // numeric payload (3 components for triples)
  unsigned long long u = 0;   // integer payload for 64-bit counts
};

struct Bi4Array {
  int type = 0;
  size_t count = 0;
  std::vector<unsigned char> data;
};

struct Bi4Item {
  std::string name;
  std::vector<std::pair<std::string, Bi4Value>> values;
  std::vector<std::pair<std::string, Bi4Array>> arrays;
  std::vector<Bi4Item> items;
  const Bi4Value* value(const std::string& n) const;
  const Bi4Array* array(const std::string& n) const;
  const Bi4Item* item(const std::string& n) const;
  void set_text(const std::string& n, const std::string& v);
  void set_num(const std::string& n, int type, double v);
  void set_u64(const std::string& n, int type, unsigned long long v);
  void set_triple(const std::string& n, int type, const double v[3]);
  void set_array(const std::string& n, int type, size_t count, const void* data, size_t bytes);
};

bool bi4_read(const std::string& path, const std::string& filecode, Bi4Item& root, std::string& err);
bool bi4_write(const std::string& path, const Bi4Item& root, std::string& err);

// ---- a loaded case -------------------------------------------------------------
struct Case {
  std::string name;
  gbsph_params params{};
  std::vector<double> pos;       // 3 per particle (case order: by id)
  std::vector<float> velrho;     // 4 per particle
  std::vector<unsigned> idp;
  std::vector<uint16_t> code;
  std::vector<float> boundnor;   // 3 per particle (empty without normals)
  unsigned np = 0, npb = 0;
  double time_max = 0, time_out = 0;
  bool savepos_double = false;
  double caseposmin[3] = {0, 0, 0}, caseposmax[3] = {0, 0, 0};
  // particle blocks of case.execution.particles, in id order (JCaseParts):
  // type 0 fixed, 1 moving, 3 fluid (TpParticles); mk; mkbound / mkfluid
  struct Block { int type; unsigned mk, mktype, begin, count; };
  std::vector<Block> blocks;
  // moving boundaries (case.execution.motion; empty without moving blocks)
  unsigned nmoving = 0;
  std::vector<gbsph_motion_object> mot_objs;
  std::vector<gbsph_movement> movs;
  std::vector<gbsph_motion_event> evts;
};

bool load_case(const std::string& casedir, const std::string& casename, Case& c, std::string& err);

// Restart state from dir/Part_%04u.bi4 (JPartsLoad4::LoadParticles with
// PartBegin, JPartsLoad4.cpp:164-290): replaces the particle arrays of `c` (a
// case loaded with load_case) by the Part's, ordered by id, with the codes
// and boundary normals of the case's particles of the same ids; returns the
// Part's TimeStep and SymplecticDtPre.
bool load_part(const std::string& dir, unsigned part, Case& c, double& timestep, double& dtpre, std::string& err);

// Writes dirout/data/Part_Head.ibi4, the run's particle-block and constants
// header that a restart checks (JSph::ConfigSaveData, JSph.cpp:2732-2748;
// JPartDataHead::SaveFile, JPartDataHead.cpp:208-272).
bool save_head(const std::string& dirout, const Case& c, unsigned firstpart, std::string& err);

// Writes dirout/data/Part_%04u.bi4 (JSph::SaveData, JSph.cpp:3062-3110, 3209).
bool save_part(const std::string& dirout, const Case& c, unsigned part, double timestep, unsigned step,
               double dtnext, unsigned np, const double* pos, const float* velrho, const unsigned* idp,
               std::string& err);

}  // namespace gbio
