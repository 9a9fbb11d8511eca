// .conf / .json configuration loading with the reference's semantics
// (src/configParser.cpp:33-451), a small JSON reader of our own (the
// reference uses nlohmann-json), CSV/WAV source tables and the per-step
// source values.
#include "config.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>

#include "mshio.h"

namespace dgcfg {

namespace {

[[noreturn]] void fail(const std::string& m) { throw std::runtime_error(m); }

std::string extension(const std::string& f) {
  auto p = f.find_last_of('.');
  return p == std::string::npos ? "" : f.substr(p + 1);
}

double to_d(const std::string& s, const std::string& key) {
  try {
    size_t pos = 0;
    double v = std::stod(s, &pos);
    return v;
  } catch (...) {
    fail("invalid or missing number for '" + key + "': '" + s + "'");
  }
}

std::vector<std::string> split(const std::string& s, char d) {
  std::vector<std::string> out;
  std::stringstream ss(s);
  std::string tok;
  while (std::getline(ss, tok, d)) out.push_back(tok);
  return out;
}

std::string unquote(std::string s) {
  if (!s.empty() && s.front() == '"') s.erase(0, 1);
  if (!s.empty() && s.back() == '"') s.pop_back();
  return s;
}

// ---- minimal JSON value and parser ----
struct Json {
  enum Type { Null, Bool, Num, Str, Arr, Obj } type = Null;
  bool b = false;
  double n = 0;
  std::string s;
  std::vector<Json> a;
  std::vector<std::pair<std::string, Json>> o;
  const Json* get(const std::string& k) const {
    for (auto& kv : o)
      if (kv.first == k) return &kv.second;
    return nullptr;
  }
};

struct JsonParser {
  const std::string& t;
  size_t i = 0;
  explicit JsonParser(const std::string& text) : t(text) {}
  void ws() {
    while (i < t.size() && std::isspace((unsigned char)t[i])) ++i;
  }
  [[noreturn]] void err(const char* m) { fail(std::string("JSON: ") + m + " at offset " + std::to_string(i)); }
  Json value() {
    ws();
    if (i >= t.size()) err("unexpected end");
    char c = t[i];
    Json v;
    if (c == '{') {
      v.type = Json::Obj;
      ++i;
      ws();
      if (i < t.size() && t[i] == '}') return ++i, v;
      for (;;) {
        ws();
        if (i >= t.size() || t[i] != '"') err("expected key");
        std::string k = str();
        ws();
        if (i >= t.size() || t[i] != ':') err("expected ':'");
        ++i;
        v.o.emplace_back(k, value());
        ws();
        if (i < t.size() && t[i] == ',') {
          ++i;
          continue;
        }
        if (i < t.size() && t[i] == '}') return ++i, v;
        err("expected ',' or '}'");
      }
    }
    if (c == '[') {
      v.type = Json::Arr;
      ++i;
      ws();
      if (i < t.size() && t[i] == ']') return ++i, v;
      for (;;) {
        v.a.push_back(value());
        ws();
        if (i < t.size() && t[i] == ',') {
          ++i;
          continue;
        }
        if (i < t.size() && t[i] == ']') return ++i, v;
        err("expected ',' or ']'");
      }
    }
    if (c == '"') {
      v.type = Json::Str;
      v.s = str();
      return v;
    }
    if (t.compare(i, 4, "true") == 0) return i += 4, v.type = Json::Bool, v.b = true, v;
    if (t.compare(i, 5, "false") == 0) return i += 5, v.type = Json::Bool, v;
    if (t.compare(i, 4, "null") == 0) return i += 4, v;
    const char* start = t.c_str() + i;
    char* end = nullptr;
    v.n = std::strtod(start, &end);
    if (end == start) err("invalid value");
    i += end - start;
    v.type = Json::Num;
    return v;
  }
  std::string str() {
    std::string out;
    ++i;  // opening quote
    while (i < t.size() && t[i] != '"') {
      char c = t[i++];
      if (c == '\\' && i < t.size()) {
        char e = t[i++];
        switch (e) {
          case 'n': out += '\n'; break;
          case 't': out += '\t'; break;
          case 'r': out += '\r'; break;
          case 'b': out += '\b'; break;
          case 'f': out += '\f'; break;
          case 'u': {
            unsigned cp = (unsigned)std::strtoul(t.substr(i, 4).c_str(), nullptr, 16);
            i += 4;
            if (cp < 0x80) out += (char)cp;
            else if (cp < 0x800) out += (char)(0xC0 | (cp >> 6)), out += (char)(0x80 | (cp & 0x3F));
            else out += (char)(0xE0 | (cp >> 12)), out += (char)(0x80 | ((cp >> 6) & 0x3F)), out += (char)(0x80 | (cp & 0x3F));
            break;
          }
          default: out += e;
        }
      } else {
        out += c;
      }
    }
    if (i >= t.size()) err("unterminated string");
    ++i;
    return out;
  }
};

const Json& at(const Json& j, const std::string& path) {
  const Json* cur = &j;
  for (auto& key : split(path, '.')) {
    const Json* nx = cur->type == Json::Obj ? cur->get(key) : nullptr;
    if (!nx) fail("JSON: missing key '" + path + "'");
    cur = nx;
  }
  return *cur;
}
double num(const Json& j, const std::string& path) {
  const Json& v = at(j, path);
  if (v.type != Json::Num) fail("JSON: '" + path + "' must be a number");
  return v.n;
}
std::string text(const Json& j, const std::string& path) {
  const Json& v = at(j, path);
  if (v.type != Json::Str) fail("JSON: '" + path + "' must be a string");
  return v.s;
}

// dipole / quadrupole expansion into monopoles (src/configParser.cpp:87-115)
void add_pole(Config& c, const std::string& type, double x, double y, double z, double size, double amp, double freq,
              double phase, double dur) {
  auto mono = [&](double sx, double sy, double sz, double ssize, double sph) {
    Source s;
    s.kind = kSine;
    double p[8] = {sx, sy, sz, ssize, amp, freq, sph, dur};
    std::copy(p, p + 8, s.params);
    c.sources.push_back(s);
  };
  if (type == "dipole") {
    mono(x - size, y, z, size / 2., phase);
    mono(x + size, y, z, size / 2., phase + M_PI);
  } else if (type == "quadrupole") {
    mono(x - size, y, z, size / 2., phase);
    mono(x + size, y, z, size / 2., phase);
    mono(x, y - size, z, size / 2., phase + M_PI);
    mono(x, y + size, z, size / 2., phase + M_PI);
  } else {
    mono(x, y, z, size, phase);
  }
}

void add_formula(Config& c, const std::string& expr, double x, double y, double z, double size, double dur) {
  Source s;
  s.kind = kFormula;
  s.formula = expr;
  double p[8] = {x, y, z, size, 0, 0, 0, dur};
  std::copy(p, p + 8, s.params);
  c.sources.push_back(s);
}

void add_file(Config& c, const std::string& file, double x, double y, double z, double size) {
  Source s;
  s.kind = kTable;
  double p[8] = {x, y, z, size, 0, 0, 0, 0};
  std::copy(p, p + 8, s.params);
  std::string ext = extension(file);
  if (ext == "csv")
    s.table = read_csv_table(file);
  else if (ext == "wav")
    s.table = read_wav_table(file);
  else
    fail("Not supported data: '" + file + "'");
  c.sources.push_back(s);
}

dgmsh::MshFile open_mesh(const std::string& f) {
  std::ifstream m(f);
  if (!m.is_open()) fail("Mesh file '" + f + "' not found or corrupted");
  return dgmsh::read_msh(f);
}

std::vector<dgmsh::PhysicalGroup> bc_groups(const dgmsh::MshFile& mf) {
  return dgmsh::to_volume_mesh(mf).bc_groups;  // dim-1 groups, ascending tag
}

Config parse_conf(const std::string& name) {
  std::ifstream in(name);
  if (!in.is_open()) fail("Project file '" + name + "' not found or corrupted");
  Config c;
  std::map<std::string, std::string> kv;
  std::string line;
  while (std::getline(in, line)) {
    line.erase(std::remove_if(line.begin(), line.end(), [](unsigned char ch) { return std::isspace(ch); }), line.end());
    if (line.empty() || line[0] == '#') continue;
    auto pos = line.find('=');
    kv[line.substr(0, pos)] = pos == std::string::npos ? line : line.substr(pos + 1);
  }
  auto req = [&](const char* k) {
    auto it = kv.find(k);
    return it == kv.end() ? std::string() : it->second;
  };
  c.mesh_file = req("meshFileName");
  c.t_start = to_d(req("timeStart"), "timeStart");
  c.t_end = to_d(req("timeEnd"), "timeEnd");
  c.dt = to_d(req("timeStep"), "timeStep");
  c.t_rate = to_d(req("timeRate"), "timeRate");
  c.element_type = req("elementType");
  c.time_method = req("timeIntMethod");
  c.num_threads = (int)to_d(req("numThreads"), "numThreads");
  c.num_threads = c.num_threads == 1 ? 0 : c.num_threads;
  c.v0[0] = to_d(req("v0_x"), "v0_x");
  c.v0[1] = to_d(req("v0_y"), "v0_y");
  c.v0[2] = to_d(req("v0_z"), "v0_z");
  c.rho0 = to_d(req("rho0"), "rho0");
  c.c0 = to_d(req("c0"), "c0");
  if (kv.count("gpuPrecision")) c.precision = kv["gpuPrecision"];
  // sources, observers and ICs in key order (std::map: lexicographic)
  for (auto& e : kv) {
    const std::string& key = e.first;
    auto sep = split(e.second, ',');
    auto f = [&](size_t i) { return i < sep.size() ? to_d(sep[i], key) : to_d("", key); };
    if (key.find("source") == 0) {
      if (sep.empty()) fail("empty source '" + key + "'");
      if (sep[0] != "formula" && sep[0] != "file") {
        add_pole(c, sep[0], f(1), f(2), f(3), f(4), f(5), f(6), f(7), f(8));
      } else if (sep[0] == "formula") {
        add_formula(c, unquote(sep.size() > 1 ? sep[1] : ""), f(2), f(3), f(4), f(5), f(6));
      } else {
        add_file(c, unquote(sep.size() > 1 ? sep[1] : ""), f(2), f(3), f(4), f(5));
      }
    } else if (key.find("observer") == 0) {
      c.observers.push_back({f(0), f(1), f(2), f(3)});
    } else if (key.find("initialCondtition") == 0) {
      c.ics.push_back({f(1), f(2), f(3), f(4), f(5)});
    }
  }
  // BCs: each physical group of dim-1 by name (src/configParser.cpp:205-223)
  auto mf = open_mesh(c.mesh_file);
  for (auto& g : bc_groups(mf)) {
    auto it = kv.find(g.name);
    std::string v = it == kv.end() ? "" : it->second;
    if (v.find("Absorbing") == 0) c.bcs.push_back({g.tag, 0});
    else if (v.find("Reflecting") == 0) c.bcs.push_back({g.tag, 1});
  }
  return c;
}

Config parse_json(const std::string& name) {
  std::ifstream in(name);
  if (!in.is_open()) fail("Project file '" + name + "' not found or corrupted");
  std::stringstream ss;
  ss << in.rdbuf();
  std::string txt = ss.str();
  JsonParser jp(txt);
  Json j = jp.value();
  Config c;
  c.mesh_file = text(j, "mesh.File");
  int nbc = (int)num(j, "mesh.BC.number");
  (void)nbc;
  auto mf = open_mesh(c.mesh_file);
  auto groups = bc_groups(mf);
  // BC k is matched to the k-th physical group positionally (src/configParser.cpp:268-289)
  for (size_t p = 0; p < groups.size(); ++p) {
    const Json* b = j.get("mesh") ? j.get("mesh")->get("BC") : nullptr;
    b = b ? b->get("boundary" + std::to_string(p + 1)) : nullptr;
    if (!b || !b->get("name") || b->get("name")->type != Json::Str) continue;
    if (b->get("name")->s != groups[p].name) continue;
    const Json* ty = b->get("type");
    std::string t = ty && ty->type == Json::Str ? ty->s : "";
    if (t == "Absorbing") c.bcs.push_back({groups[p].tag, 0});
    else if (t == "Reflecting") c.bcs.push_back({groups[p].tag, 1});
  }
  c.t_start = num(j, "solver.time.start");
  c.t_end = num(j, "solver.time.end");
  c.dt = num(j, "solver.time.step");
  c.t_rate = num(j, "solver.time.rate");
  c.element_type = text(j, "solver.elementType");
  c.time_method = text(j, "solver.timeIntMethod");
  c.num_threads = (int)num(j, "solver.numThreads");
  c.num_threads = c.num_threads == 1 ? 0 : c.num_threads;
  c.v0[0] = num(j, "initialization.meanFlow.vx");
  c.v0[1] = num(j, "initialization.meanFlow.vy");
  c.v0[2] = num(j, "initialization.meanFlow.vz");
  c.rho0 = num(j, "initialization.meanFlow.rho");
  c.c0 = num(j, "initialization.meanFlow.c");
  int nic = (int)num(j, "initialization.number");
  for (int i = 0; i < nic; ++i) {
    std::string b = "initialization.initialCondition" + std::to_string(i + 1) + ".";
    c.ics.push_back({num(j, b + "x"), num(j, b + "y"), num(j, b + "z"), num(j, b + "size"), num(j, b + "amplitude")});
  }
  int nobs = (int)num(j, "observers.number");
  for (int i = 0; i < nobs; ++i) {
    std::string b = "observers.observer" + std::to_string(i + 1) + ".";
    c.observers.push_back({num(j, b + "x"), num(j, b + "y"), num(j, b + "z"), num(j, b + "size")});
  }
  int nsrc = (int)num(j, "sources.number");
  for (int i = 0; i < nsrc; ++i) {
    std::string b = "sources.source" + std::to_string(i + 1) + ".";
    std::string type = text(j, b + "type"), fct = text(j, b + "fct");
    double x = num(j, b + "x"), y = num(j, b + "y"), z = num(j, b + "z"), size = num(j, b + "size");
    double amp = num(j, b + "amplitude"), freq = num(j, b + "frequency"), phase = num(j, b + "phase");
    double dur = num(j, b + "duration");
    if (type != "formula" && type != "file") {
      add_pole(c, type, x, y, z, size, amp, freq, phase, dur);
    } else if (type == "formula") {
      fct.erase(std::remove_if(fct.begin(), fct.end(), [](unsigned char ch) { return std::isspace(ch); }), fct.end());
      add_formula(c, unquote(fct), x, y, z, size, dur);
    } else {
      add_file(c, unquote(fct), x, y, z, size);
    }
  }
  if (const Json* g = j.get("gpu"))
    if (const Json* p = g->get("precision"))
      if (p->type == Json::Str) c.precision = p->s;
  return c;
}

}  // namespace

Config load(const std::string& path) {
  std::string ext = extension(path);
  if (ext == "conf") return parse_conf(path);
  if (ext == "json") return parse_json(path);
  fail("configuration file must end in .conf or .json: '" + path + "'");
}

// include/configParser.h:38-58 (bisection over the (t, value) table)
static double interpolate(const std::vector<double>& tab, double t) {
  size_t rows = tab.size() / 2;
  if (rows == 0) return 0.0;
  size_t lo = 0, hi = rows - 1, m = 0;
  double tmin = tab[0], tmax = tab[2 * hi];
  int guard = 0;
  while (lo <= hi && t >= tmin && t <= tmax) {
    m = (lo + hi) / 2;
    if (t < tab[2 * m]) hi = m;
    else lo = m;
    if (hi == lo + 1)
      return tab[2 * lo + 1] + ((tab[2 * hi + 1] - tab[2 * lo + 1]) / (tab[2 * hi] - tab[2 * lo])) * (t - tab[2 * lo]);
    if (++guard > 200) break;  // one-row table: the reference never leaves this loop
  }
  return 0.0;
}

double source_value(const Source& s, double t) {
  if (s.kind == kSine) {
    double amp = s.params[4], freq = s.params[5], phase = s.params[6], duration = s.params[7];
    if (t < duration) return amp * std::sin(2 * M_PI * freq * t + phase);
    return std::numeric_limits<double>::quiet_NaN();
  }
  if (s.kind == kFormula) {
    if (!(t < s.params[7])) return std::numeric_limits<double>::quiet_NaN();
    double v = 0;
    eval_formula(s.formula, t, &v);
    return v;
  }
  return interpolate(s.table, t);
}

// src/utils.cpp:138-177: ';'-separated, first line and '#' lines skipped,
// fields parsed with stof (float precision).
std::vector<double> read_csv_table(const std::string& path) {
  std::ifstream in(path);
  if (!in.is_open()) fail("Could not read file " + path);
  std::vector<double> tab;
  std::string s;
  int l = 0;
  while (std::getline(in, s)) {
    ++l;
    if (l == 1 || (!s.empty() && s[0] == '#')) continue;
    std::vector<double> rec;
    for (auto& f : split(s, ';')) {
      try {
        rec.push_back((double)std::stof(f));
      } catch (...) {
        fail("invalid number '" + f + "' in " + path);
      }
    }
    if (rec.size() < 2) fail("CSV row with fewer than two columns in " + path);
    tab.push_back(rec[0]);
    tab.push_back(rec[1]);
  }
  return tab;
}

// src/utils.cpp:240-258: samples at t = k / sample_rate (accumulated)
std::vector<double> read_wav_table(const std::string& path);

}  // namespace dgcfg
