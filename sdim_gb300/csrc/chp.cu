// .chp text straight to the op table of sdim_encode_circuit / sdim_run_tables,
// with no Circuit objects in between: the serving path's reader of the
// reference's circuit files (sdim/circuit_io.py:6-83).  Host code only.
//
// Format (as read by the reference):
//   * everything up to the first line that is "#" after stripping is a comment;
//   * if the first line after it starts with the token "d" (any case), its
//     second token is the dimension (default 2) and the line is consumed;
//   * the qudit count is one more than the largest all-digit token of the
//     remaining lines;
//   * every non-blank line is "NAME idx [idx] [key=value ...]": the all-digit
//     tokens are qudit indices (one or two), the tokens with '=' are
//     parameters (exactly one '=' each), the rest is ignored;
//   * a one-qudit line keeps its parameters on top of the gate's defaults
//     (N1: channel 'd', prob 0.01); a two-qudit line drops them, as
//     Circuit.add_gate does (sdim/circuit.py:97-121).
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sdim_gb300.h"

namespace {

// Gate names and aliases (sdim/gatedata.py:55-102) -> ids.
struct GateName {
  const char* name;
  int id;
};
const GateName kGateNames[] = {
    {"I", 0},          {"X", 1},          {"X_INV", 2},         {"Z", 3},          {"Z_INV", 4},
    {"H", 5},          {"R", 5},          {"DFT", 5},           {"H_INV", 6},      {"R_INV", 6},
    {"DFT_INV", 6},    {"H_DAG", 6},      {"R_DAG", 6},         {"DFT_DAG", 6},    {"P", 7},
    {"PHASE", 7},      {"S", 7},          {"P_INV", 8},         {"PHASE_INV", 8},  {"S_INV", 8},
    {"CNOT", 9},       {"SUM", 9},        {"CX", 9},            {"C", 9},          {"CNOT_INV", 10},
    {"SUM_INV", 10},   {"CX_INV", 10},    {"C_INV", 10},        {"CZ", 11},        {"CZ_INV", 12},
    {"SWAP", 13},      {"M", 14},         {"MEASURE", 14},      {"COLLAPSE", 14},  {"MZ", 14},
    {"M_X", 15},       {"MEASURE_X", 15}, {"MX", 15},           {"RESET", 16},     {"MR", 16},
    {"MEASURE_RESET", 16}, {"MEASURE_R", 16}, {"N1", 17},       {"NOISE1", 17},
};

int gate_id_of(const std::string& upper) {
  for (const GateName& g : kGateNames)
    if (upper == g.name) return g.id;
  return -1;
}

bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == '\v' || c == '\f'; }

std::vector<std::string> tokens_of(const char* b, const char* e) {
  std::vector<std::string> out;
  while (b < e) {
    while (b < e && is_space(*b)) ++b;
    const char* s = b;
    while (b < e && !is_space(*b)) ++b;
    if (b > s) out.emplace_back(s, b);
  }
  return out;
}

bool all_digits(const std::string& t) {
  if (t.empty()) return false;
  for (char c : t)
    if (c < '0' || c > '9') return false;
  return true;
}

std::string upper(std::string s) {
  for (char& c : s) c = (char)std::toupper((unsigned char)c);
  return s;
}

int set_err(char* err, size_t errlen, const std::string& msg) {
  if (err && errlen) {
    std::strncpy(err, msg.c_str(), errlen - 1);
    err[errlen - 1] = '\0';
  }
  return SDIM_EINVAL;
}

}  // namespace

extern "C" int sdim_parse_chp(const char* text, int64_t len, int32_t* rows, double* probs, int64_t cap,
                              int64_t* nrows, int32_t* n_out, int32_t* d_out, char* err, size_t errlen) {
  if (!text || len < 0 || !nrows || !n_out || !d_out) return set_err(err, errlen, "null argument");
  // lines
  std::vector<std::vector<std::string>> lines;
  const char* p = text;
  const char* end = text + len;
  bool started = false;
  while (p < end) {
    const char* e = static_cast<const char*>(std::memchr(p, '\n', (size_t)(end - p)));
    if (!e) e = end;
    std::vector<std::string> t = tokens_of(p, e);
    if (started)
      lines.push_back(std::move(t));
    else if (t.size() == 1 && t[0] == "#")
      started = true;
    p = e < end ? e + 1 : end;
  }
  if (!started) return set_err(err, errlen, "no line with only '#' (the end of the comment block)");
  if (lines.empty() || lines[0].empty()) return set_err(err, errlen, "no gate line after '#'");
  size_t first = 0;
  long long d = 2;
  if (upper(lines[0][0]) == "D") {
    if (lines[0].size() < 2) return set_err(err, errlen, "dimension line without a value");
    char* stop = nullptr;
    errno = 0;
    d = std::strtoll(lines[0][1].c_str(), &stop, 10);
    if (errno || !stop || *stop) return set_err(err, errlen, "dimension is not an integer: " + lines[0][1]);
    first = 1;
  }
  if (d < 2) return set_err(err, errlen, "Dimension must be greater than 1");
  if (d > 0x7fffffffLL) return set_err(err, errlen, "dimension too large");
  long long max_int = -1;
  for (size_t i = first; i < lines.size(); ++i)
    for (const std::string& t : lines[i])
      if (all_digits(t)) {
        if (t.size() > 9) return set_err(err, errlen, "qudit index too large: " + t);
        max_int = std::max(max_int, std::atoll(t.c_str()));
      }
  if (max_int < 0) return set_err(err, errlen, "no qudit index in the gate lines");
  int64_t count = 0;
  for (size_t i = first; i < lines.size(); ++i) {
    const std::vector<std::string>& t = lines[i];
    if (t.empty()) continue;
    const std::string name = upper(t[0]);
    std::vector<int> idx;
    std::string channel = "d";
    double prob = 0.01;
    bool has_noise_channel = false;
    for (size_t k = 1; k < t.size(); ++k) {
      if (all_digits(t[k])) {
        idx.push_back(std::atoi(t[k].c_str()));
      } else if (t[k].find('=') != std::string::npos) {
        const size_t eq = t[k].find('=');
        if (t[k].find('=', eq + 1) != std::string::npos)
          return set_err(err, errlen, "Extra parameter doesn't have the correct format.");
        const std::string key = t[k].substr(0, eq), val = t[k].substr(eq + 1);
        if (key == "noise_channel") {
          channel = val;
          has_noise_channel = true;
        } else if (key == "channel" && !has_noise_channel) {
          channel = val;
        } else if (key == "prob") {
          char* stop = nullptr;
          prob = std::strtod(val.c_str(), &stop);
          if (!stop || *stop || val.empty()) return set_err(err, errlen, "could not convert prob to a number: " + val);
        }
      }
    }
    if (idx.size() != 1 && idx.size() != 2)
      return set_err(err, errlen, "Unexpected number of arguments for gate " + name);
    const int id = gate_id_of(name);
    if (id < 0) return set_err(err, errlen, "Gate " + name + " not found");
    int ch = 0;
    double pr = 0.0;
    if (id == 17) {
      if (idx.size() == 2) {  // a two-qudit add_gate drops the parameters: the defaults stand
        channel = "d";
        prob = 0.01;
      }
      ch = channel == "d" ? 1 : channel == "f" ? 2 : channel == "p" ? 3 : 0;
      if (!ch) return set_err(err, errlen, "Must specify a valid noise channel.");
      pr = prob;
    }
    if (rows && count < cap) {
      rows[4 * count] = id;
      rows[4 * count + 1] = idx[0];
      rows[4 * count + 2] = idx.size() == 2 ? idx[1] : -1;
      rows[4 * count + 3] = ch;
      if (probs) probs[count] = pr;
    }
    ++count;
  }
  *nrows = count;
  *n_out = (int32_t)(max_int + 1);
  *d_out = (int32_t)d;
  if (rows && count > cap) return set_err(err, errlen, "row buffer too small");
  return SDIM_OK;
}
