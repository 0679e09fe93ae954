// Ephemeris ingest: NASA JPL Horizons vector tables (parseHorizonsFilez,
// src/SolarSystem.c:411-700, called from ofApp::setup, src/ofApp.cpp:51-70). Host code: the
// records feed initial conditions, nothing on the per-step path.
//
// A table holds, between the lines carrying "$$SOE" and "$$EOE", records of three lines
//   2460744.500000000 = A.D. 2025-Mar-10 00:00:00.0000 TDB
//    X =-1.895648544994110E+08 Y = 1.601275316244471E+08 Z = 8.026785557073921E+06
//    VX=-1.479251714253032E+01 VY=-1.637822455016202E+01 VZ= 1.972554752345790E-02
// (optionally followed by an LT / RG / RR line). Record boundaries follow the reference's scan
// exactly: a line containing " = A.D." starts a record (its Julian date is the text before the
// '=' when that text is a number, else 0); the next line must name X, Y and Z, the line after
// that VX, VY and VZ, and only then is the record counted. A line that breaks the pattern is
// skipped and the scan looks for the next date line.
//
// Values. The reference reads a value only from a whitespace-separated token that starts with
// the label and contains the '=' ("X=-1.8E+08"); in Horizons' own layout the '=' is followed or
// preceded by a space ("X =-1.8E+08", "VZ= 1.9E-02"), so it reads X, Y, Z as 0 always and VX,
// VY, VZ as 0 whenever the value is not glued to the '='. BH_HORIZONS_LITERAL reproduces that
// token rule (for bit-identical ingest); the default reads the number after each label's '='
// wherever the spaces fall, which is what the record holds.
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "bhgpu.h"

namespace {

// Lines as the reference reads them: split at '\n' (the '\n' dropped, anything else kept); a
// final line without '\n' counts, an empty tail after the last '\n' does not.
bool read_lines(const char* path, std::vector<std::string>* lines) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  std::string text;
  char buf[65536];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, got);
  std::fclose(f);
  size_t start = 0;
  while (start < text.size()) {
    const size_t nl = text.find('\n', start);
    if (nl == std::string::npos) {
      lines->push_back(text.substr(start));
      break;
    }
    lines->push_back(text.substr(start, nl - start));
    start = nl + 1;
  }
  return true;
}

// The reference's numeric test for a value text (string_is_numeric_with_alphanumeric,
// src/StringUtilities.c:278-395): optional leading whitespace and sign, digits with at most one
// '.', an optional exponent (e/E, optional sign, at least one digit) after at least one digit,
// then only whitespace; an empty text is not a number.
bool is_number(const char* s) {
  while (std::isspace((unsigned char)*s)) ++s;
  if (*s == '\0') return false;
  if (*s == '+' || *s == '-') ++s;
  bool digits = false, exp_digits = false, point = false, exponent = false;
  while (*s != '\0') {
    const unsigned char ch = (unsigned char)*s;
    if (std::isdigit(ch)) {
      (exponent ? exp_digits : digits) = true;
      ++s;
    } else if (ch == '.') {
      if (point || exponent) return false;
      point = true;
      ++s;
    } else if (ch == 'e' || ch == 'E') {
      if (exponent || !digits) return false;
      exponent = true;
      ++s;
      if (*s == '+' || *s == '-') ++s;
      if (!std::isdigit((unsigned char)*s)) return false;
      while (std::isdigit((unsigned char)*s)) ++s;
      exp_digits = true;
    } else if (std::isspace(ch)) {
      break;
    } else {
      return false;
    }
  }
  while (std::isspace((unsigned char)*s)) ++s;
  if (*s != '\0') return false;
  return exponent ? (digits && exp_digits) : digits;
}

bool contains(const std::string& line, const char* what) { return line.find(what) != std::string::npos; }

// Whitespace-separated tokens (space and tab), as strtok with " \t".
std::vector<std::string> tokens(const std::string& line) {
  std::vector<std::string> out;
  size_t i = 0;
  while (i < line.size()) {
    while (i < line.size() && (line[i] == ' ' || line[i] == '\t')) ++i;
    if (i >= line.size()) break;
    size_t j = i;
    while (j < line.size() && line[j] != ' ' && line[j] != '\t') ++j;
    out.push_back(line.substr(i, j - i));
    i = j;
  }
  return out;
}

// Literal rule: a token whose label matches (first letter for X / Y / Z, the first three
// characters "VX=" etc. for velocities) and that contains '=' gives the number after the '='.
void literal_values(const std::string& line, bool velocity, double out[3]) {
  out[0] = out[1] = out[2] = 0.0;
  for (const std::string& t : tokens(line)) {
    int axis = -1;
    if (velocity) {
      if (t.compare(0, 3, "VX=") == 0) axis = 0;
      else if (t.compare(0, 3, "VY=") == 0) axis = 1;
      else if (t.compare(0, 3, "VZ=") == 0) axis = 2;
    } else if (!t.empty()) {
      axis = t[0] == 'X' ? 0 : t[0] == 'Y' ? 1 : t[0] == 'Z' ? 2 : -1;
    }
    if (axis < 0) continue;
    const size_t eq = t.find('=');
    if (eq == std::string::npos) continue;
    const char* v = t.c_str() + eq + 1;
    if (is_number(v)) out[axis] = std::strtod(v, nullptr);
  }
}

// Intended rule: each label (at the start of the line or after whitespace), optional spaces,
// '=', optional spaces, then the number.
void label_values(const std::string& line, bool velocity, double out[3]) {
  static const char* const kPos[3] = {"X", "Y", "Z"};
  static const char* const kVel[3] = {"VX", "VY", "VZ"};
  out[0] = out[1] = out[2] = 0.0;
  for (int a = 0; a < 3; ++a) {
    const std::string label = velocity ? kVel[a] : kPos[a];
    size_t at = 0;
    while ((at = line.find(label, at)) != std::string::npos) {
      const bool word = at == 0 || line[at - 1] == ' ' || line[at - 1] == '\t';
      size_t k = at + label.size();
      while (k < line.size() && line[k] == ' ') ++k;
      if (word && k < line.size() && line[k] == '=') {
        ++k;
        while (k < line.size() && line[k] == ' ') ++k;
        out[a] = std::strtod(line.c_str() + k, nullptr);
        break;
      }
      at += label.size();
    }
  }
}

}  // namespace

extern "C" {

bh_status bh_parse_horizons(const char* path, int flags, bh_ephemeris* out, size_t cap, size_t* count) {
  if (!path || !count || (flags & ~BH_HORIZONS_LITERAL)) return BH_ERR_INVALID_ARG;
  *count = 0;
  std::vector<std::string> lines;
  if (!read_lines(path, &lines)) return BH_ERR_INVALID_ARG;
  // data region: after the first line holding "$$SOE", up to the next line holding "$$EOE"
  int start = -1, end = -1;
  for (int i = 0; i < (int)lines.size(); ++i) {
    if (start < 0) {
      if (contains(lines[i], "$$SOE")) start = i + 1;
    } else if (contains(lines[i], "$$EOE")) {
      end = i;
      break;
    }
  }
  if (start < 0 || end <= start) return BH_ERR_NOT_FOUND;
  const bool literal = (flags & BH_HORIZONS_LITERAL) != 0;
  bh_ephemeris cur;
  std::memset(&cur, 0, sizeof(cur));
  size_t n = 0;
  for (int i = start; i < end;) {
    const std::string& jd_line = lines[i];
    if (!contains(jd_line, " = A.D.")) {
      ++i;
      continue;
    }
    const std::string jd_text = jd_line.substr(0, std::min<size_t>(jd_line.find('='), 63));
    cur.jd_tdb = is_number(jd_text.c_str()) ? std::strtod(jd_text.c_str(), nullptr) : 0.0;
    if (++i >= end) break;
    const std::string& xl = lines[i];
    const bool has_xyz = (contains(xl, "X =") || contains(xl, "X=")) && (contains(xl, "Y =") || contains(xl, "Y=")) &&
                         (contains(xl, "Z =") || contains(xl, "Z="));
    ++i;
    if (!has_xyz) continue;
    if (literal)
      literal_values(xl, false, cur.pos);
    else
      label_values(xl, false, cur.pos);
    if (i >= end) break;
    const std::string& vl = lines[i];
    const bool has_v = (contains(vl, "VX=") || contains(vl, "VX =")) && (contains(vl, "VY=") || contains(vl, "VY =")) &&
                       (contains(vl, "VZ=") || contains(vl, "VZ ="));
    ++i;
    if (!has_v) continue;
    if (literal)
      literal_values(vl, true, cur.vel);
    else
      label_values(vl, true, cur.vel);
    if (out && n < cap) out[n] = cur;
    ++n;
    std::memset(&cur, 0, sizeof(cur));
  }
  *count = n;
  return BH_OK;
}

}  // extern "C"
