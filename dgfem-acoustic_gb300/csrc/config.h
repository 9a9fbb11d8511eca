// Configuration of a run: the reference's struct Config
// (include/configParser.h:69-115) as produced by config::parseConfig /
// config::parseJSON (src/configParser.cpp:33-451).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace dgcfg {

enum SourceKind { kSine = 0, kFormula = 1, kTable = 2 };

struct Source {
  int kind = kSine;
  double params[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // x, y, z, size, amp, freq, phase, duration
  std::string formula;
  std::vector<double> table;  // rows of (t, value)
};

struct Config {
  std::string mesh_file;
  double t_start = 0, t_end = 1, dt = 0.1, t_rate = 0.1;
  std::string element_type = "Lagrange";
  std::string time_method = "Euler1";
  int num_threads = 1;
  double v0[3] = {0, 0, 0};
  double rho0 = 1, c0 = 1;
  std::vector<std::pair<int, int>> bcs;  // (physical tag, 0 Absorbing / 1 Reflecting), ascending tag
  std::vector<Source> sources;
  std::vector<std::vector<double>> observers;  // x, y, z, size
  std::vector<std::vector<double>> ics;        // x, y, z, size, amp
  // project extension (absent from the reference): working precision
  std::string precision = "fp64";
};

// Throws std::runtime_error on missing files, malformed values or missing keys.
Config load(const std::string& path);

// Value written by a source at time t, NaN when it writes nothing
// (src/solver.cpp:455-483).
double source_value(const Source& s, double t);

// Formula evaluator (src/eqEdit.cpp): returns false and *value = -1 on a
// malformed expression.
bool eval_formula(const std::string& expr, double t, double* value);

// Reference file readers (src/utils.cpp:138-177, :213-258).
std::vector<double> read_csv_table(const std::string& path);
std::vector<double> read_wav_table(const std::string& path);

}  // namespace dgcfg
