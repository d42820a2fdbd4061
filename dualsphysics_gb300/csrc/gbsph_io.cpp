// gbsph_io.cpp -- run-XML reader, JBinaryData (bi4) reader/writer and case
// loading for the gbsph_run driver.  See gbsph_io.h for the reference formats.
#include "gbsph_io.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <sys/stat.h>

namespace gbio {

// ---- XML -----------------------------------------------------------------------
const XmlNode* XmlNode::child(const std::string& n) const {
  for (auto& k : kids)
    if (k->name == n) return k.get();
  return nullptr;
}

std::vector<const XmlNode*> XmlNode::children(const std::string& n) const {
  std::vector<const XmlNode*> out;
  for (auto& k : kids)
    if (n.empty() || k->name == n) out.push_back(k.get());
  return out;
}

std::string XmlNode::get(const std::string& a, const std::string& def) const {
  auto it = attr.find(a);
  return it == attr.end() ? def : it->second;
}

double XmlNode::getd(const std::string& a) const { return std::strtod(get(a, "0").c_str(), nullptr); }

namespace {

std::string unescape(const std::string& s) {
  std::string o;
  for (size_t i = 0; i < s.size(); i++) {
    if (s[i] == '&') {
      const size_t e = s.find(';', i);
      if (e != std::string::npos) {
        const std::string ent = s.substr(i + 1, e - i - 1);
        if (ent == "lt") o += '<';
        else if (ent == "gt") o += '>';
        else if (ent == "amp") o += '&';
        else if (ent == "quot") o += '"';
        else if (ent == "apos") o += '\'';
        else o += s.substr(i, e - i + 1);
        i = e;
        continue;
      }
    }
    o += s[i];
  }
  return o;
}

struct XmlParser {
  const std::string& s;
  size_t i = 0;
  std::string err;
  explicit XmlParser(const std::string& src) : s(src) {}
  void ws() { while (i < s.size() && std::isspace((unsigned char)s[i])) i++; }
  bool starts(const char* t) const { return s.compare(i, std::strlen(t), t) == 0; }
  bool skip_misc() {
    for (;;) {
      ws();
      if (starts("<?")) { size_t e = s.find("?>", i); if (e == std::string::npos) return false; i = e + 2; }
      else if (starts("<!--")) { size_t e = s.find("-->", i); if (e == std::string::npos) return false; i = e + 3; }
      else if (starts("<!")) { size_t e = s.find('>', i); if (e == std::string::npos) return false; i = e + 1; }
      else return true;
    }
  }
  std::unique_ptr<XmlNode> element() {
    if (!skip_misc() || i >= s.size() || s[i] != '<') { err = "expected element"; return nullptr; }
    i++;
    auto n = std::make_unique<XmlNode>();
    while (i < s.size() && !std::isspace((unsigned char)s[i]) && s[i] != '>' && s[i] != '/') n->name += s[i++];
    for (;;) {
      ws();
      if (i >= s.size()) { err = "unterminated tag"; return nullptr; }
      if (s[i] == '/') { if (i + 1 < s.size() && s[i + 1] == '>') { i += 2; return n; } err = "bad tag end"; return nullptr; }
      if (s[i] == '>') { i++; break; }
      std::string k;
      while (i < s.size() && s[i] != '=' && !std::isspace((unsigned char)s[i])) k += s[i++];
      ws();
      if (i >= s.size() || s[i] != '=') { err = "attribute without value: " + k; return nullptr; }
      i++;
      ws();
      const char qch = s[i];
      if (qch != '"' && qch != '\'') { err = "unquoted attribute: " + k; return nullptr; }
      const size_t e = s.find(qch, i + 1);
      if (e == std::string::npos) { err = "unterminated attribute"; return nullptr; }
      n->attr[k] = unescape(s.substr(i + 1, e - i - 1));
      i = e + 1;
    }
    for (;;) {
      // text content is skipped (the run XML carries everything in attributes)
      while (i < s.size() && s[i] != '<') i++;
      if (i >= s.size()) { err = "unterminated element " + n->name; return nullptr; }
      if (starts("<!--")) { size_t e = s.find("-->", i); if (e == std::string::npos) { err = "comment"; return nullptr; } i = e + 3; continue; }
      if (starts("</")) {
        const size_t e = s.find('>', i);
        if (e == std::string::npos) { err = "bad end tag"; return nullptr; }
        i = e + 1;
        return n;
      }
      auto k = element();
      if (!k) return nullptr;
      n->kids.push_back(std::move(k));
    }
  }
};

}  // namespace

std::unique_ptr<XmlNode> xml_parse_file(const std::string& path, std::string& err) {
  std::ifstream f(path, std::ios::binary);
  if (!f) { err = "cannot open " + path; return nullptr; }
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string src = ss.str();
  XmlParser p(src);
  auto root = p.element();
  if (!root) err = "XML error in " + path + ": " + p.err;
  return root;
}

// ---- JBinaryData -----------------------------------------------------------------
const Bi4Value* Bi4Item::value(const std::string& n) const {
  for (auto& v : values) if (v.first == n) return &v.second;
  return nullptr;
}
const Bi4Array* Bi4Item::array(const std::string& n) const {
  for (auto& a : arrays) if (a.first == n) return &a.second;
  return nullptr;
}
const Bi4Item* Bi4Item::item(const std::string& n) const {
  for (auto& i : items) if (i.name == n) return &i;
  return nullptr;
}
void Bi4Item::set_text(const std::string& n, const std::string& v) {
  Bi4Value x; x.type = DatText; x.text = v; values.emplace_back(n, x);
}
void Bi4Item::set_num(const std::string& n, int type, double v) {
  Bi4Value x; x.type = type; x.num[0] = v; values.emplace_back(n, x);
}
void Bi4Item::set_u64(const std::string& n, int type, unsigned long long v) {
  Bi4Value x; x.type = type; x.u = v; x.num[0] = (double)v; values.emplace_back(n, x);
}
void Bi4Item::set_triple(const std::string& n, int type, const double v[3]) {
  Bi4Value x; x.type = type; x.num[0] = v[0]; x.num[1] = v[1]; x.num[2] = v[2]; values.emplace_back(n, x);
}
void Bi4Item::set_array(const std::string& n, int type, size_t count, const void* data, size_t bytes) {
  Bi4Array a; a.type = type; a.count = count;
  a.data.assign((const unsigned char*)data, (const unsigned char*)data + bytes);
  arrays.emplace_back(n, std::move(a));
}

namespace {

size_t type_size(int t) {
  switch (t) {
    case DatBool: case DatInt: case DatUint: case DatFloat: return 4;
    case DatChar: case DatUchar: return 1;
    case DatShort: case DatUshort: return 2;
    case DatLlong: case DatUllong: case DatDouble: return 8;
    case DatInt3: case DatUint3: case DatFloat3: return 12;
    case DatDouble3: return 24;
    default: return 0;
  }
}

struct Rd {
  const unsigned char* b;
  size_t n, o = 0;
  bool si64;
  bool fail = false;
  bool take(void* dst, size_t k) {
    if (o + k > n) { fail = true; return false; }
    if (dst) std::memcpy(dst, b + o, k);
    o += k;
    return true;
  }
  unsigned u32() { unsigned v = 0; take(&v, 4); return v; }
  int i32() { int v = 0; take(&v, 4); return v; }
  unsigned long long size() {
    if (si64) { unsigned long long v = 0; take(&v, 8); return v; }
    return u32();
  }
  std::string str() {
    const unsigned len = u32();
    if (fail || o + len > n) { fail = true; return ""; }
    std::string s((const char*)b + o, len);
    o += len;
    return s;
  }
};

bool read_value(Rd& r, Bi4Item& it) {
  const std::string name = r.str();
  Bi4Value v;
  v.type = r.i32();
  switch (v.type) {
    case DatText: v.text = r.str(); break;
    case DatBool: case DatInt: v.num[0] = r.i32(); break;
    case DatUint: v.u = r.u32(); v.num[0] = (double)v.u; break;
    case DatChar: { signed char c = 0; r.take(&c, 1); v.num[0] = c; break; }
    case DatUchar: { unsigned char c = 0; r.take(&c, 1); v.num[0] = c; break; }
    case DatShort: { short c = 0; r.take(&c, 2); v.num[0] = c; break; }
    case DatUshort: { unsigned short c = 0; r.take(&c, 2); v.num[0] = c; break; }
    case DatLlong: { long long c = 0; r.take(&c, 8); v.num[0] = (double)c; v.u = (unsigned long long)c; break; }
    case DatUllong: { r.take(&v.u, 8); v.num[0] = (double)v.u; break; }
    case DatFloat: { float f = 0; r.take(&f, 4); v.num[0] = f; break; }
    case DatDouble: r.take(&v.num[0], 8); break;
    case DatInt3: case DatUint3: { int k[3]; r.take(k, 12); for (int j = 0; j < 3; j++) v.num[j] = v.type == DatInt3 ? k[j] : (double)(unsigned)k[j]; break; }
    case DatFloat3: { float f[3]; r.take(f, 12); for (int j = 0; j < 3; j++) v.num[j] = f[j]; break; }
    case DatDouble3: r.take(v.num, 24); break;
    default: return false;
  }
  it.values.emplace_back(name, v);
  return !r.fail;
}

bool read_item(Rd& r, Bi4Item& it, std::string& err) {
  r.u32();  // size of the item definition
  if (r.str() != "\nITEM\n") { err = "validation code is invalid (ITEM)"; return false; }
  it.name = r.str();
  r.i32(); r.i32();  // hide, hidevalues
  r.str(); r.str();  // float/double formats
  const unsigned narrays = r.u32(), nitems = r.u32(), sizevalues = r.u32();
  if (sizevalues) {
    if (r.str() != "\nVALUES") { err = "validation code is invalid (VALUES)"; return false; }
    const unsigned nv = r.u32();
    for (unsigned k = 0; k < nv; k++)
      if (!read_value(r, it)) { err = "invalid value"; return false; }
  }
  for (unsigned k = 0; k < narrays; k++) {
    r.u32();
    if (r.str() != "\nARRAY") { err = "validation code is invalid (ARRAY)"; return false; }
    const std::string name = r.str();
    r.i32();
    Bi4Array a;
    a.type = r.i32();
    a.count = (size_t)r.size();
    const size_t bytes = (size_t)r.size();
    if (a.type == DatText) { err = "text arrays are not supported"; return false; }
    if (bytes != type_size(a.type) * a.count) { err = "size of data is invalid"; return false; }
    a.data.resize(bytes);
    if (!r.take(a.data.data(), bytes)) { err = "overflow in reading data"; return false; }
    it.arrays.emplace_back(name, std::move(a));
  }
  for (unsigned k = 0; k < nitems; k++) {
    Bi4Item sub;
    if (!read_item(r, sub, err)) return false;
    it.items.push_back(std::move(sub));
  }
  if (r.fail) { err = "overflow in reading data"; return false; }
  return true;
}

void put(std::vector<unsigned char>& o, const void* p, size_t k) {
  o.insert(o.end(), (const unsigned char*)p, (const unsigned char*)p + k);
}
void put_u32(std::vector<unsigned char>& o, unsigned v) { put(o, &v, 4); }
void put_i32(std::vector<unsigned char>& o, int v) { put(o, &v, 4); }
void put_str(std::vector<unsigned char>& o, const std::string& s) { put_u32(o, (unsigned)s.size()); put(o, s.data(), s.size()); }

void write_values(std::vector<unsigned char>& o, const Bi4Item& it) {
  put_str(o, "\nVALUES");
  put_u32(o, (unsigned)it.values.size());
  for (auto& kv : it.values) {
    const Bi4Value& v = kv.second;
    put_str(o, kv.first);
    put_i32(o, v.type);
    switch (v.type) {
      case DatText: put_str(o, v.text); break;
      case DatBool: case DatInt: put_i32(o, (int)v.num[0]); break;
      case DatUint: put_u32(o, (unsigned)v.u); break;
      case DatUllong: case DatLlong: put(o, &v.u, 8); break;
      case DatFloat: { float f = (float)v.num[0]; put(o, &f, 4); break; }
      case DatDouble: put(o, &v.num[0], 8); break;
      case DatDouble3: put(o, v.num, 24); break;
      case DatFloat3: { float f[3] = {(float)v.num[0], (float)v.num[1], (float)v.num[2]}; put(o, f, 12); break; }
      default: break;
    }
  }
}

void write_item(std::vector<unsigned char>& o, const Bi4Item& it) {
  std::vector<unsigned char> vals;
  write_values(vals, it);
  std::vector<unsigned char> base;
  put_str(base, "\nITEM\n");
  put_str(base, it.name);
  put_i32(base, 0);
  put_i32(base, 0);
  put_str(base, "%.7E");
  put_str(base, "%.15E");
  put_u32(base, (unsigned)it.arrays.size());
  put_u32(base, (unsigned)it.items.size());
  put_u32(base, (unsigned)vals.size());
  put_u32(o, (unsigned)base.size());
  put(o, base.data(), base.size());
  put(o, vals.data(), vals.size());
  for (auto& kv : it.arrays) {
    std::vector<unsigned char> ab;
    put_str(ab, "\nARRAY");
    put_str(ab, kv.first);
    put_i32(ab, 0);
    put_i32(ab, kv.second.type);
    put_u32(ab, (unsigned)kv.second.count);
    put_u32(ab, (unsigned)kv.second.data.size());
    put_u32(o, (unsigned)ab.size());
    put(o, ab.data(), ab.size());
    put(o, kv.second.data.data(), kv.second.data.size());
  }
  for (auto& sub : it.items) write_item(o, sub);
}

}  // namespace

bool bi4_read(const std::string& path, const std::string& filecode, Bi4Item& root, std::string& err) {
  std::ifstream f(path, std::ios::binary);
  if (!f) { err = "cannot open " + path; return false; }
  std::vector<unsigned char> buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  if (buf.size() < 64) { err = "file too small: " + path; return false; }
  const std::string titu((const char*)buf.data(), 60);
  if (titu.compare(0, 8, "#FileJBD") != 0) { err = "the format file JBinaryData is invalid: " + path; return false; }
  if (!filecode.empty() && titu.compare(9, filecode.size(), filecode) != 0) { err = "the file code is invalid"; return false; }
  const bool si64 = buf[61] != 0;
  if ((buf[60] - (si64 ? 10 : 0)) != 0) { err = "the byte-order in file is invalid"; return false; }
  Rd r{buf.data() + 64, buf.size() - 64, 0, si64};
  return read_item(r, root, err);
}

bool bi4_write(const std::string& path, const Bi4Item& root, std::string& err) {
  std::vector<unsigned char> body;
  write_item(body, root);
  if (body.size() >= 4228102018ull) { err = "file larger than the 32-bit container"; return false; }
  char head[64];
  std::memset(head, ' ', 58);
  const std::string t = "#FileJBD " + root.name;
  std::memcpy(head, t.data(), std::min<size_t>(58, t.size()));
  head[58] = '\n';
  head[59] = 0;
  head[60] = 0;
  head[61] = 0;
  head[62] = 0;
  head[63] = 0;
  std::ofstream f(path, std::ios::binary);
  if (!f) { err = "cannot create " + path; return false; }
  f.write(head, 64);
  f.write((const char*)body.data(), (std::streamsize)body.size());
  return (bool)f;
}

// ---- case loading (JSph::LoadCaseConfig / LoadCaseParticles / ResizeMapLimits) -------
namespace {

bool pos_value(const std::string& in, bool isposmin, int& mode, double& value) {
  // JCaseEParms::CheckPosValue (JCaseEParms.cpp:374-414): 0 default, 1 fixed, 2 default+value, 3 default+%
  std::string v;
  for (char ch : in) if (!std::isspace((unsigned char)ch)) v += (char)std::tolower((unsigned char)ch);
  mode = 0;
  value = 0;
  if (v == "default") return true;
  if (v.rfind("default+", 0) == 0 || v.rfind("default-", 0) == 0) {
    const char sign = v[7];
    if ((isposmin && sign == '+') || (!isposmin && sign == '-')) return false;
    const bool prc = !v.empty() && v.back() == '%';
    const std::string num = v.substr(8, v.size() - 8 - (prc ? 1 : 0));
    value = std::strtod(num.c_str(), nullptr);
    mode = prc ? 3 : 2;
    if (prc) value /= 100.0;
    return true;
  }
  mode = 1;
  value = std::strtod(v.c_str(), nullptr);
  return true;
}

}  // namespace

// case.execution.motion as JMotion::ReadXml reads it (JMotion.cpp:692-905):
// one <objreal ref> per moving block (ref k = the k-th moving block), its
// movements and <begin> events; durations and event times are floats there.
static bool read_motion(const XmlNode* node, Case& c, std::string& err) {
  if (!node) { err = "moving particles without <motion> in the case XML"; return false; }
  auto f32 = [](double v) { return (double)(float)v; };
  auto vec3 = [](const XmlNode* e, double* v) {
    if (e) { v[0] = e->getd("x"); v[1] = e->getd("y"); v[2] = e->getd("z"); }
  };
  std::vector<char> seen(c.mot_objs.size(), 0);
  for (auto* obj : node->children("")) {
    if (obj->name.empty() || obj->name[0] == '_') continue;
    if (obj->name != "objreal") { err = "<" + obj->name + "> in <motion> is not supported"; return false; }
    const long ref = std::lround(obj->getd("ref"));
    if (ref < 0 || ref >= (long)c.mot_objs.size() || seen[ref]) { err = "motion reference does not match the moving blocks"; return false; }
    seen[ref] = 1;
    for (auto* e : obj->children("")) {
      if (e->name.empty() || e->name[0] == '_') continue;
      if (e->name == "begin") {
        c.evts.push_back(gbsph_motion_event{(unsigned)ref, (unsigned)e->getd("mov"), f32(e->getd("start")),
                                           e->has("finish") ? f32(e->getd("finish")) : -1.0});
        continue;
      }
      static const char* names[] = {"wait", "mvrect", "mvrectace", "mvrot", "mvrotace", "mvrectsinu", "mvrotsinu", "mvnull"};
      int type = 0;
      for (int k = 0; k < 8; k++) if (e->name == names[k]) type = k + 1;
      if (!type) { err = "movement <" + e->name + "> is not supported"; return false; }
      gbsph_movement m;
      memset(&m, 0, sizeof(m));
      m.type = type;
      m.obj = (unsigned)ref;
      m.id = (unsigned)e->getd("id");
      m.nextid = e->has("next") ? (unsigned)e->getd("next") : 0u;
      m.duration = type == GBSPH_MOV_NULL ? 0.0 : f32(e->getd("duration"));
      const std::string units = e->get("anglesunits", "degrees");
      if (units != "degrees" && units != "radians") { err = "anglesunits must be degrees or radians"; return false; }
      m.angdegrees = units == "degrees";
      auto ang = [&](const char* n, const char* a) { const XmlNode* x = e->child(n); return x ? x->getd(a) : 0.0; };
      switch (type) {
        case GBSPH_MOV_RECT: vec3(e->child("vel"), m.v); break;
        case GBSPH_MOV_RECTACE:
          vec3(e->child("ace"), m.a);
          m.prev = e->child("velini") == nullptr;
          vec3(e->child("velini"), m.v);
          break;
        case GBSPH_MOV_RECTSINU:
          vec3(e->child("freq"), m.v);
          vec3(e->child("ampl"), m.a);
          m.prev = e->child("phase") == nullptr;
          vec3(e->child("phase"), m.p);
          break;
        case GBSPH_MOV_ROT: case GBSPH_MOV_ROTACE: case GBSPH_MOV_ROTSINU:
          vec3(e->child("axisp1"), m.axisp1);
          vec3(e->child("axisp2"), m.axisp2);
          if (type == GBSPH_MOV_ROT) m.s[0] = ang("vel", "ang");
          else if (type == GBSPH_MOV_ROTACE) {
            m.s[1] = ang("ace", "ang");
            m.prev = e->child("velini") == nullptr;
            m.s[0] = ang("velini", "ang");
          } else {
            m.s[0] = ang("freq", "v");
            m.s[1] = ang("ampl", "v");
            m.prev = e->child("phase") == nullptr;
            m.s[2] = ang("phase", "v");
          }
          break;
        default: break;
      }
      c.movs.push_back(m);
    }
  }
  for (char v : seen) if (!v) { err = "the number of moving objects does not match the predefined motions"; return false; }
  return true;
}

bool load_case(const std::string& casedir, const std::string& casename, Case& c, std::string& err) {
  c = Case();
  c.name = casename;
  auto root = xml_parse_file(casedir + "/" + casename + ".xml", err);
  if (!root) return false;
  const XmlNode* ex = root->child("execution");
  const XmlNode* cte = ex ? ex->child("constants") : nullptr;
  const XmlNode* par = ex ? ex->child("parameters") : nullptr;
  const XmlNode* parts = ex ? ex->child("particles") : nullptr;
  if (!cte || !par || !parts) { err = "missing constants/parameters/particles in the case XML"; return false; }
  std::map<std::string, std::string> kv;
  for (auto* p : par->children("parameter")) kv[p->get("key")] = p->get("value");
  auto gi = [&](const char* k, int d) { return kv.count(k) ? (int)std::strtod(kv[k].c_str(), nullptr) : d; };
  auto gf = [&](const char* k, double d) { return kv.count(k) ? std::strtod(kv[k].c_str(), nullptr) : d; };
  if (gi("Kernel", 2) != 2) { err = "only the Wendland kernel (Kernel=2) is implemented"; return false; }
  // standard shifting (JSph.cpp:744-759); advanced shifting (4) is not built
  const int tshift = gi("Shifting", 0);
  if (tshift < 0 || tshift > 3) { err = "Shifting mode " + std::to_string(tshift) + " is not supported (0-3)"; return false; }
  gbsph_params& p = c.params;
  std::memset(&p, 0, sizeof(p));
  // periodic conditions (JSph.cpp:815-826)
  {
    static const char* keys[6] = {"XPeriodicIncY", "XPeriodicIncZ", "YPeriodicIncX", "YPeriodicIncZ", "ZPeriodicIncX", "ZPeriodicIncY"};
    static const int axis[6] = {0, 0, 1, 1, 2, 2}, comp[6] = {1, 2, 0, 2, 0, 1};
    for (int k = 0; k < 6; k++)
      if (kv.count(keys[k])) { p.peri[axis[k]] = 1; p.periinc[3 * axis[k] + comp[k]] = gf(keys[k], 0); }
    static const char* pkeys[3] = {"XYPeriodic", "XZPeriodic", "YZPeriodic"};
    static const int pax[3][3] = {{1, 1, 0}, {1, 0, 1}, {0, 1, 1}};
    for (int k = 0; k < 3; k++)
      if (kv.count(pkeys[k])) {
        for (int j = 0; j < 3; j++) p.peri[j] = pax[k][j];
        for (int j = 0; j < 9; j++) p.periinc[j] = 0;
      }
  }
  p.tshift = tshift;
  if (tshift) {
    p.shiftcoef = (float)gf("ShiftCoef", -2);
    p.shifttfs = (float)gf("ShiftTFS", 0);
  }
  p.tstep = gi("StepAlgorithm", 1);
  p.verletsteps = gi("VerletSteps", 40);
  p.tvisco = gi("ViscoTreatment", 1);
  p.visco = (float)gf("Visco", 0);
  p.viscoboundfactor = (float)gf("ViscoBoundFactor", 1);
  p.tboundary = gi("Boundary", 1);
  if (p.tboundary == 2 && gi("SlipMode", 1) != 1) { err = "only mDBC SlipMode=1 is implemented"; return false; }
  p.tdensity = gi("DensityDT", 0);
  p.ddtvalue = (float)gf("DensityDTvalue", 0.1);
  p.coefdtmin = (float)gf("CoefDtMin", 0.05);
  p.dtini = std::max(0.0, gf("DtIni", 0));
  p.dtmin = std::max(0.0, gf("DtMin", 0));
  p.dtallparticles = gi("DtAllParticles", 0) == 1;
  p.rhopoutmin = (float)gf("RhopOutMin", 700);
  p.rhopoutmax = (float)gf("RhopOutMax", 1300);
  p.cellmode_div = 1;
  c.time_max = gf("TimeMax", 0);
  c.time_out = gf("TimeOut", 0);
  c.savepos_double = gi("SavePosDouble", 0) != 0;
  const XmlNode* g = cte->child("gravity");
  if (!g) { err = "missing gravity"; return false; }
  p.gravity[0] = g->getd("x"); p.gravity[1] = g->getd("y"); p.gravity[2] = g->getd("z");
  auto cv = [&](const char* n) -> double {
    const XmlNode* e = cte->child(n);
    return e ? e->getd("value") : NAN;
  };
  p.cflnumber = cv("cflnumber"); p.gamma = cv("gamma"); p.rhop0 = cv("rhop0"); p.dp = cv("dp"); p.h = cv("h");
  p.b = cv("b"); p.massbound = cv("massbound"); p.massfluid = cv("massfluid");
  if (std::isnan(p.h) || std::isnan(p.b) || std::isnan(p.dp)) { err = "missing constants"; return false; }
  // blocks and codes (JCaseParts.cpp:540-577, JSphMk.cpp:86-123)
  struct Blk { bool fluid; unsigned begin, count, code; };
  std::vector<Blk> blocks;
  unsigned ifix = 0, imov = 0, ifl = 0;
  int lastkind = 0;  // fixed 0, moving 1, fluid 2: the reference's block order
  for (auto* b : parts->children("")) {
    if (b->name.empty() || b->name[0] == '_' || b->name == "properties") continue;
    const int kind = b->name == "fixed" ? 0 : b->name == "moving" ? 1 : b->name == "fluid" ? 2 : -1;
    if (kind < 0) { err = "particle block <" + b->name + "> is outside the implemented hot path"; return false; }
    if (kind < lastkind) { err = "particle blocks must come as fixed, moving, fluid"; return false; }
    lastkind = kind;
    const unsigned begin = (unsigned)b->getd("begin"), count = (unsigned)b->getd("count");
    c.blocks.push_back({kind == 2 ? 3 : kind, (unsigned)b->getd("mk"),
                        (unsigned)b->getd(kind == 2 ? "mkfluid" : "mkbound"), begin, count});
    if (kind == 0) blocks.push_back({false, begin, count, 0x0000u | ifix++});
    else if (kind == 1) {
      blocks.push_back({false, begin, count, 0x0800u | imov++});
      c.mot_objs.push_back(gbsph_motion_object{begin, count});
      c.nmoving += count;
    } else blocks.push_back({true, begin, count, 0x1800u | ifl++});
  }
  if (imov && !read_motion(ex->child("motion"), c, err)) return false;
  c.npb = (unsigned)parts->getd("nb");
  // particles (JPartsLoad4.cpp:164-290)
  Bi4Item bd;
  if (!bi4_read(casedir + "/" + casename + ".bi4", "JPartDataBi4", bd, err)) return false;
  const Bi4Item* pt = bd.item("PART_0000");
  if (!pt) { err = "PART data is invalid"; return false; }
  const Bi4Value* npok = pt->value("Npok");
  const Bi4Array* aidp = pt->array("Idp");
  const Bi4Array* apos = pt->array("Posd");
  const Bi4Array* aposf = pt->array("Pos");
  const Bi4Array* avel = pt->array("Vel");
  const Bi4Array* arho = pt->array("Rhop");
  if (!npok || !aidp || (!apos && !aposf) || !avel || !arho) { err = "particle arrays missing"; return false; }
  const unsigned n = (unsigned)npok->u;
  c.np = n;
  std::vector<unsigned> order(n);
  const unsigned* idp = (const unsigned*)aidp->data.data();
  for (unsigned k = 0; k < n; k++) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](unsigned x, unsigned y) { return idp[x] < idp[y]; });
  c.pos.resize(3 * (size_t)n); c.velrho.resize(4 * (size_t)n); c.idp.resize(n); c.code.resize(n);
  const Bi4Array* anor = pt->array("BoundNor");
  if (anor) c.boundnor.assign(3 * (size_t)n, 0.f);
  for (unsigned k = 0; k < n; k++) {
    const unsigned s = order[k];
    c.idp[k] = idp[s];
    for (int j = 0; j < 3; j++) {
      c.pos[3 * (size_t)k + j] = apos ? ((const double*)apos->data.data())[3 * (size_t)s + j]
                                      : (double)((const float*)aposf->data.data())[3 * (size_t)s + j];
      c.velrho[4 * (size_t)k + j] = ((const float*)avel->data.data())[3 * (size_t)s + j];
    }
    c.velrho[4 * (size_t)k + 3] = ((const float*)arho->data.data())[s];
    c.code[k] = 0;
    for (auto& b : blocks)
      if (c.idp[k] >= b.begin && c.idp[k] < b.begin + b.count) c.code[k] = (uint16_t)b.code;
    if (anor && c.idp[k] < c.npb)
      for (int j = 0; j < 3; j++) c.boundnor[3 * (size_t)k + j] = ((const float*)anor->data.data())[3 * (size_t)c.idp[k] + j];
    if (c.idp[k] >= c.npb) {
      const float rho = c.velrho[4 * (size_t)k + 3];
      if (rho < p.rhopoutmin || rho > p.rhopoutmax) { err = "initial fluid density is out of limits"; return false; }
    }
  }
  // map limits: case limits +- KernelH*BORDER_MAP, then <simulationdomain>
  double cmin[3], cmax[3];
  const Bi4Value* vmin = bd.value("CasePosMin");
  const Bi4Value* vmax = bd.value("CasePosMax");
  for (int j = 0; j < 3; j++) { cmin[j] = vmin ? vmin->num[j] : 0; cmax[j] = vmax ? vmax->num[j] : 0; }
  if (cmin[0] == cmax[0] && cmin[1] == cmax[1] && cmin[2] == cmax[2]) {
    for (int j = 0; j < 3; j++) { cmin[j] = 1e300; cmax[j] = -1e300; }
    for (unsigned k = 0; k < n; k++)
      for (int j = 0; j < 3; j++) { cmin[j] = std::min(cmin[j], c.pos[3 * (size_t)k + j]); cmax[j] = std::max(cmax[j], c.pos[3 * (size_t)k + j]); }
  }
  for (int j = 0; j < 3; j++) { c.caseposmin[j] = cmin[j]; c.caseposmax[j] = cmax[j]; }
  // JPartsLoad4::CalculeLimitsPos: dp/2 on periodic axes (JPartsLoad4.cpp:389-399)
  double mmin[3], mmax[3];
  for (int j = 0; j < 3; j++) {
    const double border = p.peri[j] ? p.dp / 2. : (double)(float)p.h * 0.05;
    mmin[j] = cmin[j] - border;
    mmax[j] = cmax[j] + border;
  }
  double dmin[3] = {mmin[0], mmin[1], mmin[2]}, dmax[3] = {mmax[0], mmax[1], mmax[2]};
  if (const XmlNode* sd = par->child("simulationdomain")) {
    const char* ax = "xyz";
    const XmlNode* pmin = sd->child("posmin");
    const XmlNode* pmax = sd->child("posmax");
    for (int j = 0; j < 3; j++) {
      const double dif = mmax[j] - mmin[j];
      int mode; double v;
      if (pmin && pmin->has(std::string(1, ax[j]))) {
        if (!pos_value(pmin->get(std::string(1, ax[j])), true, mode, v)) { err = "invalid simulationdomain"; return false; }
        if (mode == 3) dmin[j] -= dif * v; else if (mode == 2) dmin[j] -= v; else if (mode == 1) dmin[j] = v;
      }
      if (pmax && pmax->has(std::string(1, ax[j]))) {
        if (!pos_value(pmax->get(std::string(1, ax[j])), false, mode, v)) { err = "invalid simulationdomain"; return false; }
        if (mode == 3) dmax[j] += dif * v; else if (mode == 2) dmax[j] += v; else if (mode == 1) dmax[j] = v;
      }
      if (dmin[j] > mmin[j] || dmax[j] < mmax[j]) { err = "domain limits are not valid"; return false; }
    }
  }
  // ResizeMapLimits applies the domain to non-periodic axes only (JSph.cpp:1473-1475)
  for (int j = 0; j < 3; j++) {
    p.maprealposmin[j] = p.peri[j] ? mmin[j] : dmin[j];
    p.maprealposmax[j] = p.peri[j] ? mmax[j] : dmax[j];
  }
  return true;
}

bool load_part(const std::string& dir, unsigned part, Case& c, double& timestep, double& dtpre, std::string& err) {
  char fn[64];
  std::snprintf(fn, sizeof(fn), "/Part_%04u.bi4", part);
  Bi4Item bd;
  if (!bi4_read(dir + fn, "JPartDataBi4", bd, err)) return false;
  char nm[32];
  std::snprintf(nm, sizeof(nm), "PART_%04u", part);
  const Bi4Item* pt = bd.item(nm);
  if (!pt) { err = std::string("no ") + nm + " in " + dir + fn; return false; }
  const Bi4Value* npok = pt->value("Npok");
  const Bi4Value* vts = pt->value("TimeStep");
  const Bi4Value* vdt = pt->value("SymplecticDtPre");
  const Bi4Array* aidp = pt->array("Idp");
  const Bi4Array* apos = pt->array("Posd");
  const Bi4Array* aposf = pt->array("Pos");
  const Bi4Array* avel = pt->array("Vel");
  const Bi4Array* arho = pt->array("Rhop");
  if (!npok || !vts || !aidp || (!apos && !aposf) || !avel || !arho) { err = "Part arrays missing"; return false; }
  const unsigned n = (unsigned)npok->u;
  if (aidp->count < n || avel->count < n || arho->count < n || (apos ? apos->count : aposf->count) < n) {
    err = "Part arrays shorter than Npok";
    return false;
  }
  timestep = vts->num[0];
  dtpre = vdt ? vdt->num[0] : 0.0;
  // the case's particles by id (load_case leaves them ordered by id)
  const std::vector<unsigned> cid = c.idp;
  const std::vector<uint16_t> ccode = c.code;
  const std::vector<float> cnor = c.boundnor;
  const unsigned* idp = (const unsigned*)aidp->data.data();
  std::vector<unsigned> order(n);
  for (unsigned k = 0; k < n; k++) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](unsigned x, unsigned y) { return idp[x] < idp[y]; });
  c.pos.assign(3 * (size_t)n, 0.0);
  c.velrho.assign(4 * (size_t)n, 0.f);
  c.idp.assign(n, 0u);
  c.code.assign(n, 0);
  if (!cnor.empty()) c.boundnor.assign(3 * (size_t)n, 0.f);
  unsigned npb = 0;
  for (unsigned k = 0; k < n; k++) {
    const unsigned s = order[k], id = idp[s];
    const auto it = std::lower_bound(cid.begin(), cid.end(), id);
    if (it == cid.end() || *it != id) { err = "Part holds an id the case does not have"; return false; }
    if (k && id == c.idp[k - 1]) { err = "Part holds an id twice"; return false; }
    const size_t ci = (size_t)(it - cid.begin());
    c.idp[k] = id;
    c.code[k] = ccode[ci];
    if (id < c.npb) npb++;
    for (int j = 0; j < 3; j++) {
      c.pos[3 * (size_t)k + j] = apos ? ((const double*)apos->data.data())[3 * (size_t)s + j]
                                      : (double)((const float*)aposf->data.data())[3 * (size_t)s + j];
      c.velrho[4 * (size_t)k + j] = ((const float*)avel->data.data())[3 * (size_t)s + j];
      if (!cnor.empty()) c.boundnor[3 * (size_t)k + j] = cnor[3 * ci + j];
    }
    c.velrho[4 * (size_t)k + 3] = ((const float*)arho->data.data())[s];
  }
  c.np = n;
  c.npb = npb;
  return true;
}

namespace {
// PeriMode (the periodic axes as bits x=1, y=2, z=4: TpPeriFromPeriActive,
// JPeriodicDef.h:79) and the increment of each axis
void set_peri(Bi4Item& it, const gbsph_params& p) {
  it.set_num("PeriMode", DatInt, (p.peri[0] ? 1 : 0) | (p.peri[1] ? 2 : 0) | (p.peri[2] ? 4 : 0));
  const double z3[3] = {0, 0, 0};
  it.set_triple("PeriXinc", DatDouble3, p.peri[0] ? p.periinc : z3);
  it.set_triple("PeriYinc", DatDouble3, p.peri[1] ? p.periinc + 3 : z3);
  it.set_triple("PeriZinc", DatDouble3, p.peri[2] ? p.periinc + 6 : z3);
}
}  // namespace

bool save_head(const std::string& dirout, const Case& c, unsigned firstpart, std::string& err) {
  const std::string dd = dirout + "/data";
  mkdir(dirout.c_str(), 0755);
  mkdir(dd.c_str(), 0755);
  const gbsph_params& p = c.params;
  Bi4Item root;
  root.name = "JPartDataHead";
  root.set_num("FmtVersion", DatUint, 180324); root.values.back().second.u = 180324;
  root.set_text("AppName", "gbsph_run");
  root.set_text("Date", "???");
  root.set_text("RunCode", "00000000");
  root.set_text("CaseName", c.name);
  root.set_num("Data2d", DatBool, p.simulate2d ? 1 : 0);
  root.set_num("Data2dPosY", DatDouble, 0);
  root.set_num("Npiece", DatUint, 1); root.values.back().second.u = 1;
  root.set_num("FirstPart", DatUint, firstpart); root.values.back().second.u = firstpart;
  root.set_triple("CasePosMin", DatDouble3, c.caseposmin);
  root.set_triple("CasePosMax", DatDouble3, c.caseposmax);
  root.set_num("NpDynamic", DatBool, 0);
  root.set_num("ReuseIds", DatBool, 0);
  root.set_triple("MapPosMin", DatDouble3, p.maprealposmin);
  root.set_triple("MapPosMax", DatDouble3, p.maprealposmax);
  set_peri(root, p);
  root.set_num("ViscoType", DatUint, p.tvisco); root.values.back().second.u = (unsigned)p.tvisco;
  root.set_num("ViscoValue", DatFloat, p.visco);
  root.set_num("ViscoBoundFactor", DatFloat, p.viscoboundfactor);
  root.set_num("Symmetry", DatBool, 0);
  root.set_num("Splitting", DatBool, 0);
  root.set_num("Dp", DatDouble, p.dp);
  root.set_num("H", DatDouble, (double)(float)p.h);  // KernelH, a float in the reference
  root.set_num("B", DatDouble, (double)(float)p.b);  // CteB
  root.set_num("Gamma", DatDouble, (double)(float)p.gamma);
  root.set_num("RhopZero", DatDouble, (double)(float)p.rhop0);
  root.set_num("MassBound", DatDouble, (double)(float)p.massbound);
  root.set_num("MassFluid", DatDouble, (double)(float)p.massfluid);
  root.set_triple("Gravity", DatFloat3, p.gravity);
  root.set_u64("CaseNp", DatUllong, c.np);
  root.set_u64("CaseNfixed", DatUllong, c.npb - c.nmoving);
  root.set_u64("CaseNmoving", DatUllong, c.nmoving);
  root.set_u64("CaseNfloat", DatUllong, 0);
  root.set_u64("CaseNfluid", DatUllong, c.np - c.npb);
  Bi4Item mk;
  mk.name = "MkBlocks";
  mk.set_num("Count", DatUint, (double)c.blocks.size()); mk.values.back().second.u = c.blocks.size();
  static const char* tnames[4] = {"Fixed", "Moving", "Floating", "Fluid"};
  for (size_t k = 0; k < c.blocks.size(); k++) {
    const Case::Block& b = c.blocks[k];
    Bi4Item it;
    char nm[32];
    std::snprintf(nm, sizeof(nm), "MkBlock_%03u", (unsigned)k);
    it.name = nm;
    it.set_text("Type", tnames[b.type & 3]);
    it.set_num("Mk", DatUint, b.mk); it.values.back().second.u = b.mk;
    it.set_num("MkType", DatUint, b.mktype); it.values.back().second.u = b.mktype;
    it.set_num("Count", DatUint, b.count); it.values.back().second.u = b.count;
    mk.items.push_back(std::move(it));
  }
  root.items.push_back(std::move(mk));
  return bi4_write(dd + "/Part_Head.ibi4", root, err);
}

bool save_part(const std::string& dirout, const Case& c, unsigned part, double timestep, unsigned step,
               double dtnext, unsigned np, const double* pos, const float* velrho, const unsigned* idp,
               std::string& err) {
  const std::string dd = dirout + "/data";
  mkdir(dirout.c_str(), 0755);
  mkdir(dd.c_str(), 0755);
  // particles in id order: ids are unique and below the case count, so each
  // particle is placed at its id and the occupied slots are read in order (O(n))
  std::vector<unsigned> order;
  order.reserve(np);
  {
    const unsigned ncase = c.np;
    std::vector<unsigned> slot(ncase, 0xffffffffu);
    bool placed = true;
    for (unsigned k = 0; k < np; k++) {
      if (idp[k] >= ncase || slot[idp[k]] != 0xffffffffu) { placed = false; break; }
      slot[idp[k]] = k;
    }
    if (placed) {
      for (unsigned i = 0; i < ncase; i++)
        if (slot[i] != 0xffffffffu) order.push_back(slot[i]);
    } else {  // ids outside the case range or repeated: sort instead
      order.resize(np);
      for (unsigned k = 0; k < np; k++) order[k] = k;
      std::stable_sort(order.begin(), order.end(), [&](unsigned x, unsigned y) { return idp[x] < idp[y]; });
    }
  }
  std::vector<unsigned> oidp(np);
  std::vector<double> opos(3 * (size_t)np);
  std::vector<float> ofpos(3 * (size_t)np), ovel(3 * (size_t)np), orho(np);
  double dmn[3] = {0, 0, 0}, dmx[3] = {0, 0, 0};
  for (unsigned k = 0; k < np; k++) {
    const unsigned s = order[k];
    oidp[k] = idp[s];
    for (int j = 0; j < 3; j++) {
      const double v = pos[3 * (size_t)s + j];
      opos[3 * (size_t)k + j] = v;
      ofpos[3 * (size_t)k + j] = (float)v;
      ovel[3 * (size_t)k + j] = velrho[4 * (size_t)s + j];
      if (k == 0 || v < dmn[j]) dmn[j] = v;
      if (k == 0 || v > dmx[j]) dmx[j] = v;
    }
    orho[k] = velrho[4 * (size_t)s + 3];
  }
  const gbsph_params& p = c.params;
  Bi4Item root;
  root.name = "JPartDataBi4";
  root.set_num("Piece", DatUint, 0); root.values.back().second.u = 0;
  root.set_num("Npiece", DatUint, 1); root.values.back().second.u = 1;
  root.set_text("RunCode", "00000000");
  root.set_text("Date", "???");
  root.set_text("AppName", "gbsph_run");
  root.set_text("CaseName", c.name);
  root.set_num("Data2d", DatBool, 0);
  root.set_num("Data2dPosY", DatDouble, 0);
  root.set_triple("MapPosMin", DatDouble3, p.maprealposmin);
  root.set_triple("MapPosMax", DatDouble3, p.maprealposmax);
  set_peri(root, p);
  root.set_num("AxisDiv", DatInt, 0);
  root.set_u64("CaseNp", DatUllong, c.np);
  root.set_u64("CaseNfixed", DatUllong, c.npb - c.nmoving);
  root.set_u64("CaseNmoving", DatUllong, c.nmoving);
  root.set_u64("CaseNfloat", DatUllong, 0);
  root.set_u64("CaseNfluid", DatUllong, c.np - c.npb);
  root.set_triple("CasePosMin", DatDouble3, c.caseposmin);
  root.set_triple("CasePosMax", DatDouble3, c.caseposmax);
  root.set_num("NpDynamic", DatBool, 0);
  root.set_num("ReuseIds", DatBool, 0);
  root.set_num("Dp", DatDouble, p.dp);
  root.set_num("H", DatDouble, p.h);
  root.set_num("B", DatDouble, p.b);
  root.set_num("Rhop0", DatDouble, p.rhop0);
  root.set_num("Gamma", DatDouble, p.gamma);
  root.set_num("MassBound", DatDouble, p.massbound);
  root.set_num("MassFluid", DatDouble, p.massfluid);
  root.set_num("Symmetry", DatBool, 0);
  root.set_num("Splitting", DatBool, 0);
  Bi4Item pi;
  char nm[32];
  std::snprintf(nm, sizeof(nm), "PART_%04u", part);
  pi.name = nm;
  pi.set_num("Cpart", DatUint, part); pi.values.back().second.u = part;
  pi.set_num("TimeStep", DatDouble, timestep);
  pi.set_num("Npok", DatUint, np); pi.values.back().second.u = np;
  pi.set_num("Nout", DatUint, c.np - np); pi.values.back().second.u = c.np - np;
  pi.set_num("Step", DatUint, step); pi.values.back().second.u = step;
  pi.set_num("RunTime", DatDouble, 0);
  pi.set_triple("DomainMin", DatDouble3, dmn);
  pi.set_triple("DomainMax", DatDouble3, dmx);
  pi.set_num("SymplecticDtPre", DatDouble, dtnext);
  pi.set_num("DemDtForce", DatDouble, 0);
  pi.set_array("Idp", DatUint, np, oidp.data(), 4 * (size_t)np);
  if (c.savepos_double) pi.set_array("Posd", DatDouble3, np, opos.data(), 24 * (size_t)np);
  else pi.set_array("Pos", DatFloat3, np, ofpos.data(), 12 * (size_t)np);
  pi.set_array("Vel", DatFloat3, np, ovel.data(), 12 * (size_t)np);
  pi.set_array("Rhop", DatFloat, np, orho.data(), 4 * (size_t)np);
  root.items.push_back(std::move(pi));
  char fn[64];
  std::snprintf(fn, sizeof(fn), "/Part_%04u.bi4", part);
  return bi4_write(dd + fn, root, err);
}

}  // namespace gbio
