// pf_run.cpp -- PixelFlow's `program main` as a C++ host program over the C ABI
// of include/pixelflow_gpu.h, for users who run a reference project directory
// without Python.
//
// The reference's main programs (src/omp_parallel/ibm_2d_uniform_omp_cpu.f90:
// 1-140, ibm_3d_uniform_omp_cpu.f90:1-140 and the backstep, drag and
// air-condition variants) read config/controlDict.txt (read_settings,
// lib/global.f90:28-92) and the porosity CSV it names (grid_conditions,
// lib/grid.f90:36-47, 281-294), set the initial and boundary conditions, write
// the legacy-VTK file of step 0, then run istep_max steps, writing the VTK file
// every istep_out steps (output_paraview_temp_2d/_3d, lib/output.f90:421-537,
// 968-1088), and end with the same file of the final state as
// output_paraview.vtk (output_paraview_2d/_3d, :307-419, :800-910).  This
// program does the same from a project directory:
//
//   pf_run [--project DIR] [--steps N] [--device D] [--force-log]
//          [--save-state FILE] [--restart STATE] [--no-vtk]
//   pf_run [--project DIR] --print-config [--dump-porosity FILE]
//   pf_run [--project DIR] --vtk-from STATE [--istep K | --final]
//
// The step runs on the GPU through libpixelflow_gb300.so; VTK output uses the
// asynchronous snapshots (pf_snapshot_begin/_wait), so a file is written while
// the GPU runs the next interval.  --force-log prints the drag program's force
// log after every step (output_force_log_2d/_3d, lib/output.f90:244-305,
// :1090-1165; ibm_2d_drag_omp_cpu.f90:121).  An optional trailing
// &gpu_control namelist group (which the reference never reads) selects the
// precision form, the program variant (inflow_porosity, walls, slip_y) and
// the sweep options.
//
// --print-config and --vtk-from make no CUDA call: the first prints the parsed
// settings as JSON (and writes the raw porosity values), the second writes the
// VTK file of a state saved by --save-state.  Both exist so that the
// reading and writing halves of the program can be checked without a GPU.
//
// State files (--save-state): the 8-byte magic "PFSTATE1", int32 dim, m, n, l,
// int64 istep (the steps taken), then u, v, [w,] p as float64, each
// (m+2)(n+2)[(l+2)] values in the reference's Fortran order (i fastest, ghost
// layers included).  The state with its ghosts is all a step reads from the
// previous one, so --restart STATE (pf_set_state in place of the initial
// conditions) continues from step istep bit for bit as the run that saved it
// would have; the loop then ends at istep_max, or after --steps N more steps.
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include <sys/stat.h>
#include <sys/types.h>

#include "pixelflow_gpu.h"

namespace {

// ---------------------------------------------------------------------------
// Settings: the namelist members of lib/global.f90:18-26 with the defaults of
// template/config/controlDict.txt, plus the &gpu_control members.
struct Settings {
  double xnue = 0.001, xlambda = 0.0, density = 1.0, width = 1.0, height = 1.0, depth = 1.0, time = 1.0;
  double inlet_velocity = 0.1, outlet_pressure = 0.0, aoa = 0.0;
  long long istep_out = 1001, istep_max = 100;
  double thickness = 1.5, threshold = 1.0e-6, radius = 0.1, center_x = 0.5, center_y = 0.5, center_z = 0.5;
  bool nonslip = true;
  std::string output_folder = "output", csv_file = "data/porosity.csv";
  long long iter_max = 100;
  double relux_factor = 1.7;
  // &gpu_control
  std::string precision = "fp64";
  long long outer_max = 4, inner_sweeps = 25;
  double dc_tol = 0.0;
  bool track_sor_error = true;
  std::string sweep_form = "auto";
  long long fused_rows = 0, fused_planes = 0;
  std::string sor_path = "auto";
  bool inflow_porosity = false;
  bool has_walls = false;
  int walls[6] = {0, 0, 0, 0, 0, 0};
  bool slip_y = false;
};

struct Value {
  enum Kind { STR, BOOL, INT, REAL } kind = STR;
  std::string s;
  bool b = false;
  long long i = 0;
  double r = 0.0;
};

[[noreturn]] void die(const std::string& msg) { throw std::runtime_error(msg); }

std::string lower(std::string s) {
  for (char& ch : s)
    if (ch >= 'A' && ch <= 'Z') ch = static_cast<char>(ch - 'A' + 'a');
  return s;
}

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace(static_cast<unsigned char>(s[a]))) a++;
  while (b > a && std::isspace(static_cast<unsigned char>(s[b - 1]))) b--;
  return s.substr(a, b - a);
}

bool is_int_text(const std::string& v) {
  size_t k = (!v.empty() && (v[0] == '+' || v[0] == '-')) ? 1 : 0;
  if (k == v.size()) return false;
  for (; k < v.size(); k++)
    if (v[k] < '0' || v[k] > '9') return false;
  return true;
}

// A namelist value: a quoted string, a logical (.true. t .t. true and the
// .false. forms), an integer, or a real with an e or d exponent.
Value convert(const std::string& text) {
  Value out;
  const std::string v = trim(text);
  if (!v.empty() && (v[0] == '"' || v[0] == '\'')) {
    out.kind = Value::STR;
    out.s = v.size() >= 2 ? v.substr(1, v.size() - 2) : std::string();
    return out;
  }
  const std::string low = lower(v);
  if (low == ".true." || low == "t" || low == ".t." || low == "true") {
    out.kind = Value::BOOL;
    out.b = true;
    return out;
  }
  if (low == ".false." || low == "f" || low == ".f." || low == "false") {
    out.kind = Value::BOOL;
    out.b = false;
    return out;
  }
  if (is_int_text(v)) {
    errno = 0;
    char* end = nullptr;
    out.i = std::strtoll(v.c_str(), &end, 10);
    if (errno == ERANGE) die("namelist: integer out of range: " + v);
    out.kind = Value::INT;
    return out;
  }
  std::string e = low;
  for (char& ch : e)
    if (ch == 'd') ch = 'e';
  if (e.find('x') != std::string::npos) die("namelist: cannot parse value '" + v + "'");
  char* end = nullptr;
  out.r = std::strtod(e.c_str(), &end);
  if (e.empty() || end != e.c_str() + e.size()) die("namelist: cannot parse value '" + v + "'");
  out.kind = Value::REAL;
  return out;
}

using Groups = std::map<std::string, std::map<std::string, Value>>;

bool ident_start(char ch) { return std::isalpha(static_cast<unsigned char>(ch)) || ch == '_'; }
bool ident_char(char ch) { return std::isalnum(static_cast<unsigned char>(ch)) || ch == '_'; }

// Position of the first `ch` outside a quoted string (npos if none).
size_t outside_quotes(const std::string& line, char ch) {
  char q = 0;
  for (size_t k = 0; k < line.size(); k++) {
    const char c = line[k];
    if (q) {
      if (c == q) q = 0;
    } else if (c == '"' || c == '\'') {
      q = c;
    } else if (c == ch) {
      return k;
    }
  }
  return std::string::npos;
}

// Fortran namelist groups (&name ... /): `!` starts a comment and `/` ends
// the group, both outside quoted strings.  Members are `name = value` pairs
// separated by blanks or commas.
Groups parse_namelists(const std::string& text) {
  Groups groups;
  std::string current;
  bool in_group = false;
  size_t pos = 0;
  while (pos <= text.size()) {
    size_t nl = text.find('\n', pos);
    if (nl == std::string::npos) nl = text.size();
    std::string line = text.substr(pos, nl - pos);
    pos = nl + 1;
    const size_t bang = outside_quotes(line, '!');
    if (bang != std::string::npos) line.resize(bang);
    if (trim(line).empty()) continue;
    if (!in_group) {
      const std::string st = trim(line);
      if (st[0] != '&') continue;
      size_t k = 1;
      while (k < st.size() && !std::isspace(static_cast<unsigned char>(st[k]))) k++;
      current = lower(st.substr(1, k - 1));
      groups[current];
      in_group = true;
      line = st.substr(k);
    }
    size_t k = 0;
    const size_t L = line.size();
    while (k < L) {
      const char ch = line[k];
      if (ch == '/') {  // end of the group
        in_group = false;
        break;
      }
      if (!ident_start(ch)) {
        k++;
        continue;
      }
      size_t a = k;
      while (k < L && ident_char(line[k])) k++;
      const std::string name = lower(line.substr(a, k - a));
      size_t q = k;
      while (q < L && std::isspace(static_cast<unsigned char>(line[q]))) q++;
      if (q >= L || line[q] != '=') continue;  // not an assignment: skip the word
      q++;
      while (q < L && std::isspace(static_cast<unsigned char>(line[q]))) q++;
      if (q >= L) {
        k = q;
        continue;
      }
      size_t b = q;
      if (line[q] == '"' || line[q] == '\'') {
        const size_t close = line.find(line[q], q + 1);
        if (close == std::string::npos) die("namelist: unterminated string in &" + current);
        b = close + 1;
      } else {
        while (b < L && line[b] != ',' && line[b] != '/' && !std::isspace(static_cast<unsigned char>(line[b]))) b++;
      }
      groups[current][name] = convert(line.substr(q, b - q));
      k = b;
    }
  }
  return groups;
}

const char* const kGroups[] = {"physical", "file_control", "grid_control", "porosity_control",
                               "calculation_method", "directory_control", "solver_control"};

double as_real(const Value& v, const std::string& name) {
  if (v.kind == Value::INT) return static_cast<double>(v.i);
  if (v.kind == Value::REAL) return v.r;
  die("namelist: " + name + " needs a number");
}
long long as_int(const Value& v, const std::string& name) {
  if (v.kind == Value::INT) return v.i;
  if (v.kind == Value::REAL && std::isfinite(v.r)) return static_cast<long long>(v.r);  // truncates as int() does
  die("namelist: " + name + " needs an integer");
}
bool as_bool(const Value& v, const std::string& name) {
  if (v.kind == Value::BOOL) return v.b;
  if (v.kind == Value::INT) return v.i != 0;
  if (v.kind == Value::REAL) return v.r != 0.0;
  die("namelist: " + name + " needs a logical");
}
std::string as_str(const Value& v, const std::string& name) {
  if (v.kind == Value::STR) return v.s;
  die("namelist: " + name + " needs a quoted string");
}

// "1,0,0,0,0,2" -> the wall table (top, bottom, east, west, north, south);
// "" -> no table.
void parse_walls(const std::string& text, Settings& s) {
  std::vector<int> vals;
  std::string tok;
  auto flush = [&]() {
    if (tok.empty()) return;
    if (!is_int_text(tok)) die("walls: six entries of 0, 1 or 2 expected, got '" + text + "'");
    vals.push_back(std::atoi(tok.c_str()));
    tok.clear();
  };
  for (char ch : text) {
    if (ch == ',' || std::isspace(static_cast<unsigned char>(ch)))
      flush();
    else
      tok += ch;
  }
  flush();
  if (vals.empty()) {
    s.has_walls = false;
    return;
  }
  if (vals.size() != 6) die("walls: six entries of 0, 1 or 2 expected, got '" + text + "'");
  for (int f = 0; f < 6; f++) {
    if (vals[f] < 0 || vals[f] > 2) die("walls: six entries of 0, 1 or 2 expected, got '" + text + "'");
    s.walls[f] = vals[f];
  }
  s.has_walls = true;
}

void assign(Settings& s, const std::string& group, const std::string& k, const Value& v) {
  const std::string where = "&" + group + " " + k;
#define PF_REAL(name)              \
  if (k == #name) {                \
    s.name = as_real(v, where);    \
    return;                        \
  }
#define PF_INT(name)               \
  if (k == #name) {                \
    s.name = as_int(v, where);     \
    return;                        \
  }
#define PF_BOOL(name)              \
  if (k == #name) {                \
    s.name = as_bool(v, where);    \
    return;                        \
  }
#define PF_STR(name)               \
  if (k == #name) {                \
    s.name = as_str(v, where);     \
    return;                        \
  }
  if (group == "physical") {
    PF_REAL(xnue) PF_REAL(xlambda) PF_REAL(density) PF_REAL(width) PF_REAL(height) PF_REAL(depth) PF_REAL(time)
    PF_REAL(inlet_velocity) PF_REAL(outlet_pressure) PF_REAL(aoa)
  } else if (group == "file_control") {
    PF_INT(istep_out)
  } else if (group == "grid_control") {
    PF_INT(istep_max)
  } else if (group == "porosity_control") {
    PF_REAL(thickness) PF_REAL(threshold) PF_REAL(radius) PF_REAL(center_x) PF_REAL(center_y) PF_REAL(center_z)
  } else if (group == "calculation_method") {
    PF_BOOL(nonslip)
  } else if (group == "directory_control") {
    PF_STR(output_folder) PF_STR(csv_file)
  } else if (group == "solver_control") {
    PF_INT(iter_max) PF_REAL(relux_factor)
  } else if (group == "gpu_control") {
    PF_STR(precision) PF_INT(outer_max) PF_INT(inner_sweeps) PF_REAL(dc_tol) PF_BOOL(track_sor_error)
    PF_BOOL(inflow_porosity) PF_STR(sweep_form) PF_INT(fused_rows) PF_INT(fused_planes) PF_STR(sor_path)
    PF_BOOL(slip_y)
    if (k == "walls") {
      parse_walls(as_str(v, where), s);
      return;
    }
  }
#undef PF_REAL
#undef PF_INT
#undef PF_BOOL
#undef PF_STR
  die("&" + group + " has no member '" + k + "'");
}

std::string read_file(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) die("cannot open " + path);
  std::string out;
  char buf[1 << 16];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, got);
  std::fclose(f);
  return out;
}

// read_settings (lib/global.f90:28-92): all seven groups must be present, as
// the reference's read(11,nml=...) sequence requires; unknown members are an
// error.  A trailing &gpu_control group is optional.
Settings read_settings(const std::string& path) {
  const Groups groups = parse_namelists(read_file(path));
  Settings s;
  for (const char* g : kGroups) {
    auto it = groups.find(g);
    if (it == groups.end()) die(path + ": namelist group &" + g + " missing");
    for (const auto& kv : it->second) assign(s, g, kv.first, kv.second);
  }
  auto gpu = groups.find("gpu_control");
  if (gpu != groups.end())
    for (const auto& kv : gpu->second) assign(s, "gpu_control", kv.first, kv.second);
  return s;
}

// Host threads for parsing and formatting text: PF_RUN_THREADS, or the
// hardware threads; at most 64.
int host_threads() {
  static const int n = [] {
    const char* env = std::getenv("PF_RUN_THREADS");
    long v = env ? std::strtol(env, nullptr, 10) : 0;
    if (v <= 0) v = static_cast<long>(std::thread::hardware_concurrency());
    return static_cast<int>(std::max(1L, std::min(v, 64L)));
  }();
  return n;
}

// ---------------------------------------------------------------------------
// The porosity CSV (grid.f90:36-47, 281-294): a header "m,n[,l]" and one
// "i, j, k, value" record per cell, stored at porosity(i, j[, k]) whatever the
// record order.  Returns the raw values with i fastest (n*m or l*n*m).
struct Grid {
  int dim = 0, m = 0, n = 0, l = 1;
  std::vector<double> values;
};

Grid read_porosity_csv(const std::string& path) {
  const std::string text = read_file(path);
  size_t nl = text.find('\n');
  if (nl == std::string::npos) die(path + ": no records");
  std::string header = text.substr(0, nl);
  for (char& ch : header)
    if (ch == ',') ch = ' ';
  std::vector<long long> dims;
  {
    size_t k = 0;
    while (k < header.size()) {
      while (k < header.size() && std::isspace(static_cast<unsigned char>(header[k]))) k++;
      if (k >= header.size()) break;
      const char* a = header.c_str() + k;
      char* end = nullptr;
      const double v = std::strtod(a, &end);
      if (end == a) die(path + ": bad header");
      // the library's own limit on each extent (pf_create rejects larger)
      if (!(v >= 1.0 && v <= double(1 << 20))) die(path + ": grid size in the header out of range");
      dims.push_back(static_cast<long long>(v));
      k += static_cast<size_t>(end - a);
    }
  }
  Grid g;
  if (dims.size() == 2 || (dims.size() == 3 && dims[2] == 1)) {
    g.dim = 2;
    g.l = 1;
  } else if (dims.size() >= 3) {
    g.dim = 3;
    g.l = static_cast<int>(dims[2]);
  } else {
    die(path + ": header must be m,n[,l]");
  }
  g.m = static_cast<int>(dims[0]);
  g.n = static_cast<int>(dims[1]);
  const size_t cells = static_cast<size_t>(g.m) * g.n * g.l;
  if (cells >= (size_t(1) << 31)) die(path + ": grid too large (the library's arrays hold < 2^31 cells)");
  g.values.assign(cells, 0.0);
  // The records are parsed on all host threads, each a run of whole lines,
  // into (cell, value) pairs that are then stored in file order, so a cell
  // listed twice keeps its last value as in a sequential read, and an error
  // names the first bad line of the file.
  const int nidx = g.dim;
  auto parse = [&](size_t from, size_t to, std::vector<std::pair<size_t, double>>& out, std::string& err) {
    std::vector<double> cols;
    size_t pos = from;
    while (pos < to) {
      size_t e = text.find('\n', pos);
      if (e == std::string::npos || e > to) e = to;
      std::string line = text.substr(pos, e - pos);
      pos = e + 1;
      const size_t hash = line.find('#');
      if (hash != std::string::npos) line.resize(hash);
      if (trim(line).empty()) continue;
      cols.clear();
      size_t a = 0;
      while (true) {
        size_t c = line.find(',', a);
        const std::string tok = trim(line.substr(a, c == std::string::npos ? std::string::npos : c - a));
        char* end = nullptr;
        const double v = std::strtod(tok.c_str(), &end);
        if (tok.empty() || end != tok.c_str() + tok.size()) {
          err = path + ": bad record '" + line + "'";
          return;
        }
        cols.push_back(v);
        if (c == std::string::npos) break;
        a = c + 1;
      }
      if ((int)cols.size() < nidx + 1) {
        err = path + ": record with too few columns '" + line + "'";
        return;
      }
      for (int q = 0; q < nidx; q++)
        if (!(cols[q] >= 1.0 && cols[q] < double(1 << 21))) {
          err = path + ": index out of range in '" + line + "'";
          return;
        }
      const long long i = static_cast<long long>(cols[0]), j = static_cast<long long>(cols[1]);
      const long long k = g.dim == 3 ? static_cast<long long>(cols[2]) : 1;
      if (i < 1 || i > g.m || j < 1 || j > g.n || k < 1 || k > g.l) {
        err = path + ": index out of range in '" + line + "'";
        return;
      }
      out.emplace_back((size_t)(i - 1) + (size_t)g.m * ((size_t)(j - 1) + (size_t)g.n * (size_t)(k - 1)),
                       cols.back());
    }
  };
  const size_t body = nl + 1;
  const int T = static_cast<int>(std::min<size_t>(host_threads(), std::max<size_t>(1, (text.size() - body) >> 20)));
  std::vector<size_t> cut(T + 1, text.size());
  cut[0] = body;
  for (int t = 1; t < T; t++) {  // each run starts after a newline
    size_t c = body + (text.size() - body) / T * t;
    c = std::max(c, cut[t - 1]);
    const size_t e = text.find('\n', c);
    cut[t] = e == std::string::npos ? text.size() : e + 1;
  }
  std::vector<std::vector<std::pair<size_t, double>>> recs(T);
  std::vector<std::string> errs(T);
  std::vector<std::thread> pool;
  for (int t = 1; t < T; t++) pool.emplace_back(parse, cut[t], cut[t + 1], std::ref(recs[t]), std::ref(errs[t]));
  parse(cut[0], cut[1], recs[0], errs[0]);
  for (auto& th : pool) th.join();
  for (int t = 0; t < T; t++) {
    if (!errs[t].empty()) die(errs[t]);
    for (const auto& r : recs[t]) g.values[r.first] = r.second;
  }
  return g;
}

// ---------------------------------------------------------------------------
pf_params make_params(const Settings& s, const Grid& g) {
  pf_params p;
  std::memset(&p, 0, sizeof p);
  p.dim = g.dim;
  p.m = g.m;
  p.n = g.n;
  p.l = g.l;
  p.xnue = s.xnue;
  p.xlambda = s.xlambda;
  p.density = s.density;
  p.width = s.width;
  p.height = s.height;
  p.depth = s.depth;
  p.time = s.time;
  p.inlet_velocity = s.inlet_velocity;
  p.outlet_pressure = s.outlet_pressure;
  p.aoa = s.aoa;
  p.istep_max = static_cast<int32_t>(s.istep_max);
  p.iter_max = static_cast<int32_t>(s.iter_max);
  p.thickness = s.thickness;
  p.threshold = s.threshold;
  p.relux_factor = s.relux_factor;
  p.nonslip = s.nonslip ? 1 : 0;
  p.inflow_porosity = s.inflow_porosity ? 1 : 0;
  p.wall_mode = s.has_walls ? 1 : 0;
  for (int f = 0; f < 6; f++) p.walls[f] = s.has_walls ? s.walls[f] : 0;
  p.slip_y = s.slip_y ? 1 : 0;
  return p;
}

pf_options make_options(const Settings& s) {
  pf_options o;
  pf_default_options(&o);
  const std::string prec = lower(s.precision);
  if (prec == "fp64" || prec == "plain")
    o.precision = PF_PREC_FP64;
  else if (prec == "mixed")
    o.precision = PF_PREC_MIXED;
  else
    die("unknown precision '" + s.precision + "'");
  o.outer_max = static_cast<int32_t>(s.outer_max);
  o.inner_sweeps = static_cast<int32_t>(s.inner_sweeps);
  o.dc_tol = s.dc_tol;
  o.track_sor_error = s.track_sor_error ? 1 : 0;
  o.use_graph = 1;
  const std::string form = lower(s.sweep_form);
  if (form == "auto")
    o.sweep_form = PF_SWEEP_AUTO;
  else if (form == "split")
    o.sweep_form = PF_SWEEP_SPLIT;
  else if (form == "fused")
    o.sweep_form = PF_SWEEP_FUSED;
  else
    die("unknown sweep_form '" + s.sweep_form + "'");
  o.fused_rows = static_cast<int32_t>(s.fused_rows);
  o.fused_planes = static_cast<int32_t>(s.fused_planes);
  const std::string path = lower(s.sor_path);
  if (path == "auto")
    o.sor_path = PF_SOR_AUTO;
  else if (path == "cells")
    o.sor_path = PF_SOR_CELLS;
  else
    die("unknown sor_path '" + s.sor_path + "'");
  return o;
}

// ---------------------------------------------------------------------------
// Fields with ghosts in the Fortran layout: (m+2)(n+2)[(l+2)] doubles.
struct State {
  int dim = 2, m = 0, n = 0, l = 1;
  long long istep = 0;
  std::vector<double> u, v, w, p;
  size_t size() const { return (size_t)(m + 2) * (n + 2) * (dim == 3 ? l + 2 : 1); }
  void alloc(int d, int mm, int nn, int ll) {
    dim = d;
    m = mm;
    n = nn;
    l = ll;
    u.assign(size(), 0.0);
    v.assign(size(), 0.0);
    w.assign(dim == 3 ? size() : 0, 0.0);
    p.assign(size(), 0.0);
  }
};

void write_state(const std::string& path, const State& st) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) die("cannot write " + path);
  const int32_t hdr[4] = {st.dim, st.m, st.n, st.l};
  const int64_t istep = st.istep;
  bool ok = std::fwrite("PFSTATE1", 1, 8, f) == 8 && std::fwrite(hdr, sizeof hdr, 1, f) == 1 &&
            std::fwrite(&istep, sizeof istep, 1, f) == 1;
  const std::vector<double>* fields[4] = {&st.u, &st.v, &st.w, &st.p};
  for (const auto* a : fields)
    if (!a->empty()) ok = ok && std::fwrite(a->data(), sizeof(double), a->size(), f) == a->size();
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) die("short write to " + path);
}

State read_state(const std::string& path) {
  const std::string b = read_file(path);
  constexpr size_t kHeader = 32;
  if (b.size() < kHeader || b.compare(0, 8, "PFSTATE1") != 0) die(path + ": not a state file");
  int32_t hdr[4];
  int64_t istep = 0;
  std::memcpy(hdr, b.data() + 8, sizeof hdr);
  std::memcpy(&istep, b.data() + 24, sizeof istep);
  if ((hdr[0] != 2 && hdr[0] != 3) || hdr[1] < 1 || hdr[2] < 1 || hdr[3] < 1 || istep < 0)
    die(path + ": bad header");
  State st;
  st.alloc(hdr[0], hdr[1], hdr[2], hdr[3]);
  st.istep = istep;
  const size_t nf = st.dim == 3 ? 4 : 3;
  if (b.size() != kHeader + nf * st.size() * sizeof(double)) die(path + ": size does not match its header");
  size_t off = kHeader;
  std::vector<double>* fields[4] = {&st.u, &st.v, &st.w, &st.p};
  for (auto* a : fields) {
    if (a->empty()) continue;
    std::memcpy(a->data(), b.data() + off, a->size() * sizeof(double));
    off += a->size() * sizeof(double);
  }
  return st;
}

// Porosity with ghosts as the case holds it, computed on the host: the
// threshold clamp of grid.f90:43 on the interior (the VTK file uses only the
// interior values).
std::vector<double> clamped_porosity(const Grid& g, double threshold) {
  const size_t X = g.m + 2, Y = g.n + 2;
  std::vector<double> out(X * Y * (g.dim == 3 ? g.l + 2 : 1), 0.0);
  const int k0 = g.dim == 3 ? 1 : 0, k1 = g.dim == 3 ? g.l : 0;
  size_t q = 0;
  for (int k = k0; k <= k1; k++)
    for (int j = 1; j <= g.n; j++)
      for (int i = 1; i <= g.m; i++) {
        const double v = g.values[q++];
        out[i + X * (j + Y * k)] = v > threshold ? v : threshold;
      }
  return out;
}

// ---------------------------------------------------------------------------
// The legacy-VTK file of output_paraview_temp_2d/_3d (lib/output.f90:421-537,
// :968-1088): an ASCII structured grid of the interior nodes at
// x_i = dx (i-1) - width*center_x (y, z likewise; grid.f90:81-89, 333-345),
// each value as Fortran f16.4 and up to three per record, records in the
// reference's order (i fastest).  Arrays: velocity, velocityInFluid,
// (2D: dimless_v), porosity, pressure, VelocityDivergent, (2D: abs_dimless_v).
//
// Formatting the text is what costs (about 13 values per point; a 256^3 file
// is 7 GB), so each array's records are formatted on all host threads, in
// blocks of consecutive points written in order: the bytes do not depend on
// the thread count (host_threads).

class VtkWriter {
 public:
  VtkWriter(const std::string& path, int m, int n, int k0, int k1)
      : f_(std::fopen(path.c_str(), "wb")), path_(path), m_(m), n_(n), k0_(k0), k1_(k1) {
    if (!f_) die("cannot write " + path);
  }
  ~VtkWriter() {
    if (f_) std::fclose(f_);
  }
  void text(const char* s) { put(s, std::strlen(s)); }
  // One record of `ncols` values per interior point (i fastest), fn(i, j, k,
  // vals) giving the values: "%16.4f " per value, then a newline.
  template <class Fn>
  void rows(int ncols, Fn fn) {
    const long long npts = (long long)m_ * n_ * (k1_ - k0_ + 1);
    const int T = host_threads();
    const long long block = 1 << 16;  // points per thread and round
    std::vector<std::string> parts(T);
    for (long long base = 0; base < npts; base += block * T) {
      auto work = [&](int t) {
        std::string& out = parts[t];
        out.clear();
        const long long a = base + t * block, e = std::min(npts, a + block);
        if (a >= e) return;
        out.reserve(static_cast<size_t>(e - a) * (17 * ncols + 1));
        char tmp[64];
        double v[3];
        for (long long q = a; q < e; q++) {
          const int i = static_cast<int>(q % m_) + 1;
          const int j = static_cast<int>((q / m_) % n_) + 1;
          const int k = static_cast<int>(q / ((long long)m_ * n_)) + k0_;
          fn(i, j, k, v);
          for (int c = 0; c < ncols; c++) out.append(tmp, static_cast<size_t>(std::snprintf(tmp, sizeof tmp, "%16.4f ", v[c])));
          out += '\n';
        }
      };
      const int used = static_cast<int>(std::min<long long>(T, (npts - base + block - 1) / block));
      std::vector<std::thread> pool;
      for (int t = 1; t < used; t++) pool.emplace_back(work, t);
      work(0);
      for (auto& th : pool) th.join();
      for (int t = 0; t < used; t++) put(parts[t].data(), parts[t].size());
    }
  }
  void close() {
    const int rc = std::fclose(f_);
    f_ = nullptr;
    if (rc != 0) die("cannot write " + path_);
  }

 private:
  void put(const char* p, size_t len) {
    if (len && std::fwrite(p, 1, len, f_) != len) die("cannot write " + path_);
  }
  FILE* f_;
  std::string path_;
  int m_, n_, k0_, k1_;
};

std::vector<double> node_coords(int count, double length, double centre) {
  const double d = length / (count - 1);
  std::vector<double> x(count + 2);
  for (int i = 0; i < count + 2; i++) x[i] = d * (static_cast<double>(i) - 1.0) - length * centre;
  return x;
}

// final: the file of the end of the run (output_paraview_2d/_3d,
// output.f90:307-419, :793-910), whose 3D form writes porosity after
// VelocityDivergent instead of before pressure; the 2D form is the same text.
void write_vtk(const std::string& path, const State& st, const std::vector<double>& poro, const Settings& s,
               bool final = false) {
  const int dim = st.dim, m = st.m, n = st.n, l = dim == 3 ? st.l : 1;
  const size_t X = m + 2, Y = n + 2;
  const std::vector<double> xs = node_coords(m, s.width, s.center_x);
  const std::vector<double> ys = node_coords(n, s.height, s.center_y);
  const std::vector<double> zs = dim == 3 ? node_coords(l, s.depth, s.center_z) : std::vector<double>();
  const int k0 = dim == 3 ? 1 : 0, k1 = dim == 3 ? l : 0;
  auto at = [&](int i, int j, int k) { return (size_t)i + X * ((size_t)j + Y * (size_t)k); };
  const long long npts = (long long)m * n * l;
  const double U = s.inlet_velocity;
  VtkWriter w(path, m, n, k0, k1);
  char line[128];
  w.text("# vtk DataFile Version 3.0\n");
  w.text(dim == 2 ? "2D flow\n" : "3D flow\n");
  w.text("ASCII \n");
  w.text("DATASET STRUCTURED_GRID\n");
  std::snprintf(line, sizeof line, "DIMENSIONS  %4d %4d %4d\n", m, n, l);
  w.text(line);
  std::snprintf(line, sizeof line, "POINTS %9lld float\n", npts);
  w.text(line);
  w.rows(3, [&](int i, int j, int k, double* r) {
    r[0] = xs[i];
    r[1] = ys[j];
    r[2] = dim == 3 ? zs[k] : 0.0;
  });
  std::snprintf(line, sizeof line, "POINT_DATA %9lld\n", npts);
  w.text(line);
  w.text("VECTORS velocity float\n");
  w.rows(3, [&](int i, int j, int k, double* r) {
    const size_t q = at(i, j, k);
    r[0] = st.u[q];
    r[1] = st.v[q];
    r[2] = dim == 3 ? st.w[q] : 0.0;
  });
  w.text("VECTORS velocityInFluid float\n");
  w.rows(3, [&](int i, int j, int k, double* r) {
    const size_t q = at(i, j, k);
    r[0] = st.u[q] * poro[q];
    r[1] = st.v[q] * poro[q];
    r[2] = dim == 3 ? st.w[q] * poro[q] : 0.0;
  });
  if (dim == 2) {
    w.text("VECTORS dimless_v float\n");
    w.rows(3, [&](int i, int j, int k, double* r) {
      const size_t q = at(i, j, k);
      r[0] = st.u[q] * poro[q] / U;
      r[1] = st.v[q] * poro[q] / U;
      r[2] = 0.0;
    });
  }
  auto porosity_section = [&]() {
    w.text("SCALARS porosity float\n");
    w.text("LOOKUP_TABLE default\n");
    w.rows(1, [&](int i, int j, int k, double* r) { r[0] = poro[at(i, j, k)]; });
  };
  const bool porosity_last = final && dim == 3;
  if (!porosity_last) porosity_section();
  w.text("SCALARS pressure float\n");
  w.text("LOOKUP_TABLE default\n");
  w.rows(1, [&](int i, int j, int k, double* r) { r[0] = st.p[at(i, j, k)]; });
  // plain central divergence over the node spacing (output.f90:501-510, :1058-1069)
  w.text("SCALARS VelocityDivergent float\n");
  w.text("LOOKUP_TABLE default\n");
  w.rows(1, [&](int i, int j, int k, double* r) {
    double d = (st.u[at(i + 1, j, k)] - st.u[at(i - 1, j, k)]) / (xs[i + 1] - xs[i - 1]) +
               (st.v[at(i, j + 1, k)] - st.v[at(i, j - 1, k)]) / (ys[j + 1] - ys[j - 1]);
    if (dim == 3) d = d + (st.w[at(i, j, k + 1)] - st.w[at(i, j, k - 1)]) / (zs[k + 1] - zs[k - 1]);
    r[0] = d;
  });
  if (porosity_last) porosity_section();
  if (dim == 2) {
    w.text("SCALARS abs_dimless_v float\n");
    w.text("LOOKUP_TABLE default\n");
    w.rows(1, [&](int i, int j, int k, double* r) {
      const size_t q = at(i, j, k);
      const double a = st.u[q] * poro[q] / U, b = st.v[q] * poro[q] / U;
      r[0] = std::sqrt(a * a + b * b);
    });
  }
  w.close();
}

std::string vtk_path(const std::string& folder, long long istep) {
  char name[64];
  std::snprintf(name, sizeof name, "output_%05lld.vtk", istep);
  return folder + "/" + name;
}

void mkdir_p(const std::string& path) {
  std::string cur;
  for (size_t k = 0; k <= path.size(); k++) {
    if (k == path.size() || path[k] == '/') {
      if (!cur.empty() && ::mkdir(cur.c_str(), 0777) != 0 && errno != EEXIST) die("cannot create " + cur);
    }
    if (k < path.size()) cur += path[k];
  }
}

// ---------------------------------------------------------------------------
std::string json_num(double v) {
  if (std::isnan(v)) return "NaN";
  if (std::isinf(v)) return v > 0 ? "Infinity" : "-Infinity";
  char b[40];
  std::snprintf(b, sizeof b, "%.17g", v);
  return b;
}

std::string json_str(const std::string& s) {
  std::string o = "\"";
  for (char ch : s) {
    if (ch == '"' || ch == '\\') {
      o += '\\';
      o += ch;
    } else if (static_cast<unsigned char>(ch) < 0x20) {
      char b[8];
      std::snprintf(b, sizeof b, "\\u%04x", ch);
      o += b;
    } else {
      o += ch;
    }
  }
  return o + "\"";
}

void print_config(const Settings& s, const Grid& g) {
  std::string o = "{";
  auto num = [&](const char* k, double v) { o += json_str(k) + ": " + json_num(v) + ", "; };
  auto integer = [&](const char* k, long long v) { o += json_str(k) + ": " + std::to_string(v) + ", "; };
  auto boolean = [&](const char* k, bool v) { o += json_str(k) + ": " + (v ? "true" : "false") + ", "; };
  auto str = [&](const char* k, const std::string& v) { o += json_str(k) + ": " + json_str(v) + ", "; };
  num("xnue", s.xnue);
  num("xlambda", s.xlambda);
  num("density", s.density);
  num("width", s.width);
  num("height", s.height);
  num("depth", s.depth);
  num("time", s.time);
  num("inlet_velocity", s.inlet_velocity);
  num("outlet_pressure", s.outlet_pressure);
  num("aoa", s.aoa);
  integer("istep_out", s.istep_out);
  integer("istep_max", s.istep_max);
  num("thickness", s.thickness);
  num("threshold", s.threshold);
  num("radius", s.radius);
  num("center_x", s.center_x);
  num("center_y", s.center_y);
  num("center_z", s.center_z);
  boolean("nonslip", s.nonslip);
  str("output_folder", s.output_folder);
  str("csv_file", s.csv_file);
  integer("iter_max", s.iter_max);
  num("relux_factor", s.relux_factor);
  str("precision", s.precision);
  integer("outer_max", s.outer_max);
  integer("inner_sweeps", s.inner_sweeps);
  num("dc_tol", s.dc_tol);
  boolean("track_sor_error", s.track_sor_error);
  str("sweep_form", s.sweep_form);
  integer("fused_rows", s.fused_rows);
  integer("fused_planes", s.fused_planes);
  str("sor_path", s.sor_path);
  boolean("inflow_porosity", s.inflow_porosity);
  if (s.has_walls) {
    o += "\"walls\": [";
    for (int f = 0; f < 6; f++) o += std::to_string(s.walls[f]) + (f < 5 ? ", " : "");
    o += "], ";
  } else {
    o += "\"walls\": null, ";
  }
  boolean("slip_y", s.slip_y);
  o += "\"shape\": [" + std::to_string(g.m) + ", " + std::to_string(g.n) +
       (g.dim == 3 ? ", " + std::to_string(g.l) : std::string()) + "]}";
  std::printf("%s\n", o.c_str());
}

void write_raw(const std::string& path, const std::vector<double>& a) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) die("cannot write " + path);
  const bool ok = std::fwrite(a.data(), sizeof(double), a.size(), f) == a.size();
  if ((std::fclose(f) != 0) || !ok) die("short write to " + path);
}

// ---------------------------------------------------------------------------
void check(int rc, const char* what) {
  if (rc != PF_OK) die(std::string(what) + ": " + pf_strerror(rc) + " (" + pf_last_error() + ")");
}

struct Args {
  std::string project = ".";
  long long steps = -1;
  int device = 0;
  bool print_config = false, force_log = false, no_vtk = false, final = false;
  std::string dump_porosity, save_state, vtk_from, restart;
  long long istep = -1;
};

void usage() {
  std::fprintf(stderr,
               "usage: pf_run [--project DIR] [--steps N] [--device D] [--force-log] [--save-state FILE] "
               "[--restart STATE] [--no-vtk]\n"
               "       pf_run [--project DIR] --print-config [--dump-porosity FILE]\n"
               "       pf_run [--project DIR] --vtk-from STATE [--istep K | --final]\n");
}

long long int_arg(const std::string& flag, const std::string& text) {
  if (!is_int_text(text)) die(flag + " needs an integer, got '" + text + "'");
  errno = 0;
  const long long v = std::strtoll(text.c_str(), nullptr, 10);
  if (errno == ERANGE || v < 0 || v > INT_MAX) die(flag + " out of range: " + text);
  return v;
}

Args parse_args(int argc, char** argv) {
  Args a;
  for (int k = 1; k < argc; k++) {
    const std::string s = argv[k];
    auto next = [&]() -> std::string {
      if (k + 1 >= argc) die("missing value after " + s);
      return argv[++k];
    };
    if (s == "--project" || s == "-C")
      a.project = next();
    else if (s == "--steps")
      a.steps = int_arg(s, next());
    else if (s == "--device")
      a.device = static_cast<int>(int_arg(s, next()));
    else if (s == "--print-config")
      a.print_config = true;
    else if (s == "--dump-porosity")
      a.dump_porosity = next();
    else if (s == "--force-log")
      a.force_log = true;
    else if (s == "--save-state")
      a.save_state = next();
    else if (s == "--no-vtk")
      a.no_vtk = true;
    else if (s == "--restart")
      a.restart = next();
    else if (s == "--vtk-from")
      a.vtk_from = next();
    else if (s == "--final")
      a.final = true;
    else if (s == "--istep")
      a.istep = int_arg(s, next());
    else if (s == "-h" || s == "--help") {
      usage();
      std::exit(0);
    } else {
      usage();
      die("unknown argument " + s);
    }
  }
  return a;
}

std::string join(const std::string& dir, const std::string& rel) {
  if (!rel.empty() && rel[0] == '/') return rel;
  return dir + "/" + rel;
}

// The force log of the drag program after step istep: pressure part, wall
// friction part, their sum and the coefficients F / (density U^2 radius).
void force_log(pf_case* c, const Settings& s, int dim, long long istep) {
  double fp[3], fv[3];
  check(pf_forces(c, fp, fv), "pf_forces");
  const double ref = s.density * (s.inlet_velocity * s.inlet_velocity) * s.radius;
  std::printf("force istep=%lld", istep);
  const char* ax = "xyz";
  for (int d = 0; d < dim; d++) std::printf(" Fp%c=%.17g", ax[d], fp[d]);
  for (int d = 0; d < dim; d++) std::printf(" Fv%c=%.17g", ax[d], fv[d]);
  for (int d = 0; d < dim; d++) std::printf(" F%c=%.17g", ax[d], fp[d] + fv[d]);
  for (int d = 0; d < dim; d++) std::printf(" C%c=%.17g", ax[d], (fp[d] + fv[d]) / ref);
  std::printf("\n");
}

int run(const Args& a) {
  const Settings s = read_settings(join(a.project, "config/controlDict.txt"));
  const Grid g = read_porosity_csv(join(a.project, s.csv_file));
  if (a.print_config) {
    print_config(s, g);
    if (!a.dump_porosity.empty()) write_raw(a.dump_porosity, g.values);
    return 0;
  }
  const std::string folder = join(a.project, s.output_folder);
  if (!a.vtk_from.empty()) {  // host only: the VTK file of a saved state
    const State st = read_state(a.vtk_from);
    if (st.dim != g.dim || st.m != g.m || st.n != g.n || (g.dim == 3 && st.l != g.l))
      die("--vtk-from: the state's grid does not match the project's porosity file");
    mkdir_p(folder);
    const std::string out = a.final ? folder + "/output_paraview.vtk" : vtk_path(folder, a.istep >= 0 ? a.istep : st.istep);
    write_vtk(out, st, clamped_porosity(g, s.threshold), s, a.final);
    return 0;
  }
  if (s.istep_max <= 0 || s.istep_out <= 0) die("istep_max and istep_out must be > 0");
  if (s.istep_out > INT_MAX) die("istep_out must be below 2^31");
  State restart;
  if (!a.restart.empty()) {
    restart = read_state(a.restart);
    if (restart.dim != g.dim || restart.m != g.m || restart.n != g.n || (g.dim == 3 && restart.l != g.l))
      die("--restart: the state's grid does not match the project's porosity file");
  }
  const long long first = restart.istep;  // steps already taken (0 without --restart)
  const long long last = a.steps >= 0 ? first + a.steps : s.istep_max;
  if (last < first) die("--restart: the state is past istep_max; give --steps N");
  const pf_params prm = make_params(s, g);
  const pf_options opt = make_options(s);
  check(pf_set_device(a.device), "pf_set_device");
  pf_case* c = nullptr;
  check(pf_create(&prm, &opt, g.values.data(), &c), "pf_create");
  std::printf("# istep_max= %lld   istep_out= %lld   grid %d x %d%s\n", s.istep_max, s.istep_out, g.m, g.n,
              g.dim == 3 ? (" x " + std::to_string(g.l)).c_str() : "");
  try {
    const int ld1 = g.m + 2, ld2 = g.n + 2;
    if (a.restart.empty()) {
      check(pf_initial_conditions(c), "pf_initial_conditions");
    } else {
      check(pf_set_state(c, restart.u.data(), restart.v.data(), g.dim == 3 ? restart.w.data() : nullptr,
                         restart.p.data(), ld1, ld2),
            "pf_set_state");
      restart = State();  // the fields now live on the device
    }
    State buf;
    buf.alloc(g.dim, g.m, g.n, g.l);
    std::vector<double> poro(buf.size());
    check(pf_get_porosity(c, poro.data(), ld1, ld2), "pf_get_porosity");
    const bool vtk = !a.no_vtk;
    if (vtk) mkdir_p(folder);
    auto wait_into = [&](State& st) {
      check(pf_snapshot_wait(c, st.u.data(), st.v.data(), g.dim == 3 ? st.w.data() : nullptr, st.p.data(), ld1,
                             ld2),
            "pf_snapshot_wait");
    };
    // The step loop with its output every istep_out steps, the step-0 file
    // included (not on a restart): a snapshot is taken on the device right
    // after its step, the next interval's steps are enqueued, and only then
    // is the previous snapshot written, so the copies and the file writing
    // overlap the GPU.  Steps are numbered from the start of the run.
    long long done = first, pending = -1, ready = -1;
    if (vtk && first == 0) {
      check(pf_snapshot_begin(c), "pf_snapshot_begin");
      pending = 0;
    }
    while (done < last) {
      const long long k = std::min(s.istep_out - done % s.istep_out, last - done);
      if (a.force_log) {
        for (long long q = 0; q < k; q++) {
          check(pf_step(c, 1), "pf_step");
          force_log(c, s, g.dim, done + q + 1);
        }
      } else {
        check(pf_step(c, static_cast<int>(k)), "pf_step");
      }
      done += k;
      if (ready >= 0) {
        write_vtk(vtk_path(folder, ready), buf, poro, s);
        ready = -1;
      }
      if (vtk && done % s.istep_out == 0) {
        if (pending >= 0) {
          wait_into(buf);
          ready = pending;
        }
        check(pf_snapshot_begin(c), "pf_snapshot_begin");
        pending = done;
      }
    }
    if (ready >= 0) write_vtk(vtk_path(folder, ready), buf, poro, s);
    if (pending >= 0) {
      wait_into(buf);
      write_vtk(vtk_path(folder, pending), buf, poro, s);
    }
    double max_div = 0.0, sor_err = 0.0;
    const int rc = pf_norms(c, &max_div, &sor_err);
    std::printf("# steps %lld  max|div u| %.17g  SOR error %.17g\n", done, max_div, sor_err);
    check(rc, "pf_norms");
    if (vtk || !a.save_state.empty()) {
      check(pf_get_state(c, buf.u.data(), buf.v.data(), g.dim == 3 ? buf.w.data() : nullptr, buf.p.data(), ld1, ld2),
            "pf_get_state");
      buf.istep = done;
      // the main programs end with output_paraview_2d/_3d: the same file for
      // the final state, named output_paraview.vtk (output.f90:323, :816)
      if (vtk) write_vtk(folder + "/output_paraview.vtk", buf, poro, s, true);
      if (!a.save_state.empty()) write_state(a.save_state, buf);
    }
  } catch (...) {
    pf_destroy(c);
    throw;
  }
  check(pf_destroy(c), "pf_destroy");
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    return run(parse_args(argc, argv));
  } catch (const std::exception& e) {
    std::fflush(stdout);
    std::fprintf(stderr, "pf_run: %s\n", e.what());
    return 1;
  }
}
