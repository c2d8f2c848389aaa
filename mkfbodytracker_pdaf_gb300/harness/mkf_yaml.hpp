// mkf_yaml.hpp -- reader and writer for the OpenCV FileStorage YAML subset the
// tracker's files use: "%YAML:1.0" header, top-level scalars, and matrices
// written as "name: !!opencv-matrix" mappings of rows / cols / dt / data (or
// untagged rows / cols / data mappings, as in cal.yml).  It replaces
// cv::FileStorage for the model files read at pfPose.cpp:34-55 (OpenCV is not
// a dependency here).  Matrices are held as row-major doubles with their dt.
#pragma once

#include <cstdio>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace mkf {
namespace yaml {

struct Matrix {
  int rows = 0, cols = 0;
  char dt = 'd';
  std::vector<double> data;
  double at(int r, int c) const { return data[static_cast<size_t>(r) * cols + c]; }
};

struct Document {
  std::map<std::string, Matrix> matrices;
  std::map<std::string, std::string> scalars;
  std::vector<std::string> order;   // key order as read / to write
  const Matrix& matrix(const std::string& k) const {
    auto it = matrices.find(k);
    if (it == matrices.end()) throw std::runtime_error("yaml: no matrix '" + k + "'");
    return it->second;
  }
};

inline std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r");
  if (a == std::string::npos) return "";
  size_t b = s.find_last_not_of(" \t\r");
  return s.substr(a, b - a + 1);
}

inline Document parse(const std::string& text) {
  Document doc;
  std::vector<std::string> lines;
  {
    std::istringstream is(text);
    std::string l;
    while (std::getline(is, l)) lines.push_back(l);
  }
  size_t i = 0;
  const size_t n = lines.size();
  auto indented = [&](const std::string& l) { return !l.empty() && (l[0] == ' ' || l[0] == '\t'); };
  while (i < n) {
    const std::string line = lines[i];
    const std::string t = trim(line);
    if (t.empty() || t[0] == '%' || t[0] == '#' || t == "---") { ++i; continue; }
    if (indented(line)) throw std::runtime_error("yaml: unexpected indentation at line " + std::to_string(i + 1));
    const size_t colon = line.find(':');
    if (colon == std::string::npos) throw std::runtime_error("yaml: no key at line " + std::to_string(i + 1));
    const std::string key = trim(line.substr(0, colon));
    const std::string rest = trim(line.substr(colon + 1));
    ++i;
    if (!rest.empty() && rest.rfind("!!", 0) != 0) {
      std::string v = rest;
      if (v.size() >= 2 && v.front() == '"' && v.back() == '"') v = v.substr(1, v.size() - 2);
      doc.scalars[key] = v;
      doc.order.push_back(key);
      continue;
    }
    Matrix m;
    bool have_rows = false, have_cols = false, have_data = false;
    while (i < n && (indented(lines[i]) || trim(lines[i]).empty())) {
      const std::string sub = trim(lines[i]);
      ++i;
      if (sub.empty()) continue;
      const size_t c2 = sub.find(':');
      if (c2 == std::string::npos) continue;
      const std::string k2 = trim(sub.substr(0, c2));
      std::string v2 = trim(sub.substr(c2 + 1));
      if (k2 == "rows") { m.rows = std::stoi(v2); have_rows = true; }
      else if (k2 == "cols") { m.cols = std::stoi(v2); have_cols = true; }
      else if (k2 == "dt") { m.dt = v2.empty() ? 'd' : v2[0]; }
      else if (k2 == "data") {
        std::string buf = v2;
        while (buf.find(']') == std::string::npos && i < n) buf += " " + trim(lines[i++]);
        const size_t a = buf.find('['), b = buf.rfind(']');
        if (a == std::string::npos || b == std::string::npos || b < a)
          throw std::runtime_error("yaml: malformed data of '" + key + "'");
        std::string inner = buf.substr(a + 1, b - a - 1);
        for (char& ch : inner) if (ch == ',') ch = ' ';
        std::istringstream ds(inner);
        std::string tok;
        while (ds >> tok) m.data.push_back(std::stod(tok));
        have_data = true;
      }
    }
    if (!(have_rows && have_cols && have_data)) throw std::runtime_error("yaml: incomplete matrix '" + key + "'");
    if (m.data.size() != static_cast<size_t>(m.rows) * m.cols)
      throw std::runtime_error("yaml: matrix '" + key + "' has " + std::to_string(m.data.size()) + " values for " +
                               std::to_string(m.rows) + "x" + std::to_string(m.cols));
    if (m.dt == 'f')
      for (double& v : m.data) v = static_cast<double>(static_cast<float>(v));   // convertTo(CV_64F) of a float matrix
    doc.matrices[key] = m;
    doc.order.push_back(key);
  }
  return doc;
}

inline Document load(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("yaml: cannot open " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  return parse(ss.str());
}

// FileStorage-style output: 17 significant digits for dt d, 9 for dt f, two
// values per data line; reading it back gives the same doubles
inline std::string dump(const Document& doc) {
  std::string out = "%YAML:1.0\n";
  char buf[64];
  for (const std::string& k : doc.order) {
    auto s = doc.scalars.find(k);
    if (s != doc.scalars.end()) { out += k + ": " + s->second + "\n"; continue; }
    const Matrix& m = doc.matrix(k);
    out += k + ": !!opencv-matrix\n   rows: " + std::to_string(m.rows) + "\n   cols: " + std::to_string(m.cols) +
           "\n   dt: " + std::string(1, m.dt) + "\n   data: [ ";
    for (size_t q = 0; q < m.data.size(); ++q) {
      std::snprintf(buf, sizeof(buf), m.dt == 'f' ? "%.9g" : "%.17g", m.data[q]);
      out += buf;
      if (q + 1 < m.data.size()) out += (q % 2 == 1) ? ",\n       " : ", ";
    }
    out += " ]\n";
  }
  return out;
}

inline void save(const std::string& path, const Document& doc) {
  std::ofstream f(path);
  if (!f) throw std::runtime_error("yaml: cannot write " + path);
  f << dump(doc);
}

}  // namespace yaml
}  // namespace mkf
