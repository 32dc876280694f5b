// host_model.cpp -- settings, file formats, gene -> layer AP construction, lead displacement.
#include "host_model.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <stdexcept>

#include "../../include/ekgsim.h"

namespace ekg {

namespace {
std::string trim(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && (s[a] == ' ' || s[a] == '\t' || s[a] == '\r' || s[a] == '\n')) ++a;
    while (b > a && (s[b - 1] == ' ' || s[b - 1] == '\t' || s[b - 1] == '\r' || s[b - 1] == '\n')) --b;
    return s.substr(a, b - a);
}
std::string extension(const std::string &f) {
    size_t p = f.rfind('.');
    return p == std::string::npos ? std::string() : f.substr(p);
}
std::string dir_of(const std::string &path) {
    size_t p = path.find_last_of('/');
    return p == std::string::npos ? std::string() : path.substr(0, p + 1);
}
std::string resolve(const std::string &base_dir, const std::string &f) {
    if (f.empty() || f[0] == '/' || base_dir.empty()) return f;
    return base_dir + f;
}
}  // namespace

// ------------------------------------------------------------------ INI
bool Ini::load(const std::string &path) {
    std::ifstream in(path.c_str());
    if (!in.is_open()) return ok = false;
    std::string line, cur = "";
    sec[cur];
    while (std::getline(in, line)) {
        std::string t = trim(line);
        if (t.empty()) continue;
        if (t[0] == '[' && t[t.size() - 1] == ']') {
            cur = trim(t.substr(1, t.size() - 2));
            sec[cur];
            continue;
        }
        if (t[0] == ';') continue;
        size_t eq = t.find('=');
        if (eq == std::string::npos) continue;
        sec[cur][trim(t.substr(0, eq))] = trim(t.substr(eq + 1));
    }
    return ok = true;
}
bool Ini::has(const std::string &s, const std::string &k) const {
    auto i = sec.find(s);
    return i != sec.end() && i->second.count(k);
}
std::string Ini::str(const std::string &s, const std::string &k, const std::string &def) const {
    auto i = sec.find(s);
    if (i == sec.end()) return def;
    auto j = i->second.find(k);
    return j == i->second.end() ? def : j->second;
}
double Ini::num(const std::string &s, const std::string &k, double def) const {
    if (!has(s, k)) return def;
    std::istringstream is(str(s, k));
    double v;
    if (is >> v) return v;
    return def;
}
std::vector<double> Ini::vec(const std::string &s, const std::string &k) const {
    std::vector<double> out;
    if (!has(s, k)) return out;
    std::string v = str(s, k);
    for (char &c : v)
        if (c == ',') c = ' ';
    std::istringstream is(v);
    double x;
    while (is >> x) out.push_back(x);
    return out;
}

int nhood_code(const std::string &n) {
    if (n == "3D4") return EKG_NHOOD_3D4;
    if (n == "3D8" || n == "cube") return EKG_NHOOD_CUBE;
    if (n == "2D4") return EKG_NHOOD_2D4;
    if (n == "2D8") return EKG_NHOOD_2D8;
    return -1;
}

SimConfig load_config(const std::string &path) {
    Ini ini;
    SimConfig c;
    if (!ini.load(path)) throw std::runtime_error("could not open settings file " + path);
    c.shape = ini.str("model", "shape");
    c.excitation_in = ini.str("model", "excitation sequence");
    c.points = ini.str("model", "points");
    c.transfer = ini.str("model", "transfer");
    c.excitation_out = ini.str("output files", "excitation sequence");
    c.results = ini.str("output files", "results filename", "result.column");
    c.length = (double)(int)ini.num("simulation", "length", 800);
    c.start = (double)(int)ini.num("simulation", "start", 0);
    c.nhood = ini.str("simulation", "neighbourhood type");
    c.dt = ini.num("simulation", "time step", 1.0 / 3.0);
    c.ap_time_step = ini.num("action potentials", "resample time step", 1);
    for (int i = 1;; ++i) {
        std::vector<double> k = ini.vec("wohlfart ap", "base ap " + std::to_string(i));
        if (k.size() > 9) k.resize(9);
        if (k.size() != 9) break;
        c.base_aps.push_back(k);
    }
    if (c.base_aps.size() < 2) throw std::runtime_error("need at least 2 base APs");
    c.k_min = ini.vec("wohlfart ap", "k min");
    if (c.k_min.size() > 9) c.k_min.resize(9);
    if (c.k_min.size() != 9) throw std::runtime_error("could not read kMin");
    c.k_max = ini.vec("wohlfart ap", "k max");
    if (c.k_max.size() > 9) c.k_max.resize(9);
    if (c.k_max.size() != 9) throw std::runtime_error("could not read kMax");
    c.interpolation = ini.str("wohlfart ap", "interpolation");
    c.mid_position = ini.num("wohlfart ap", "mid AP position", 0.5);
    if (c.mid_position > 1.0 || c.mid_position < 0.0) c.mid_position = 0.5;
    for (double v : ini.vec("wohlfart ap", "free k")) c.free_k.push_back((int)v);
    if (!ini.has("measuring points", "displacement min")) throw std::runtime_error("could not read displacement min");
    if (!ini.has("measuring points", "displacement max")) throw std::runtime_error("could not read displacement max");
    for (double v : ini.vec("measuring points", "displacement min")) c.disp_min.push_back((int)v);
    for (double v : ini.vec("measuring points", "displacement max")) c.disp_max.push_back((int)v);
    c.targets_file = ini.str("optimization", "targets filename");
    int crit = (int)ini.num("optimization", "mode", 1);
    if (crit != 1 && crit != 9) throw std::runtime_error("invalid optimization mode");
    c.criteria_mode = crit;
    c.endo_epi_delay = ini.num("optimization", "endo-epi minimization criterion epi delay", -1);
    c.peak = (int)ini.num("optimization", "peak position is criterion", 0) > 0;
    c.optimize_points = ini.num("optimization", "optimize measuring points", 0) != 0;
    c.fast_is_crit = (int)ini.num("optimization", "fast approximation is criterion", 0) > 0;
    c.fast_delay = ini.num("optimization", "fast approximation epi delay", 0);
    c.fast_limit = ini.num("optimization", "fast approximation limit", 2);
    int cm = (int)ini.num("optimization", "comparison mode", 2);
    if (cm < 1 || cm > 4) throw std::runtime_error("invalid comparison mode");
    c.comparison_mode = cm;
    c.generations = (size_t)ini.num("optimization", "number of generations", 100);
    c.population = (size_t)ini.num("optimization", "population size", 0);
    c.queue_size = (int)ini.num("optimization", "queue size", 1);
    // file names are relative to the working directory, as in the reference; resolve them
    // against the ini's directory when that is not the working directory
    const std::string d = dir_of(path);
    c.shape = resolve(d, c.shape);
    c.points = resolve(d, c.points);
    c.transfer = resolve(d, c.transfer);
    c.targets_file = resolve(d, c.targets_file);
    if (!c.excitation_in.empty()) c.excitation_in = resolve(d, c.excitation_in);
    if (!c.excitation_out.empty()) c.excitation_out = resolve(d, c.excitation_out);
    return c;
}

// ------------------------------------------------------------------ excitation sequence files
static bool has_matrix_ext(const std::string &path) {
    const size_t dot = path.find_last_of('.');
    return dot != std::string::npos && path.substr(dot) == ".matrix";
}

void read_excitation(const std::string &path, int nz, int ny, int nx, std::vector<double> &at) {
    if (!has_matrix_ext(path)) throw std::runtime_error("can only import from .matrix for the time being");
    std::ifstream in(path);
    if (!in.is_open()) throw std::runtime_error("could not open file " + path + " to load excitation sequence");
    in.ignore(100000000, '\n');  // comment line
    std::string dim;
    in >> dim;
    if (!(dim.size() >= 2 && (dim[1] == 'D' || dim[1] == 'd') && dim[0] > '0' && dim[0] <= '3'))
        throw std::runtime_error("error while loading matrix, could not read dimensionality");
    long size[3] = {1, 1, 1};  // [0] z, [1] y, [2] x; the header lists x first
    int w = 2;
    in >> size[w];
    for (int k = dim[0] - '0' - 1; k > 0; --k) {
        in.ignore(100, 'x');
        --w;
        in >> size[w];
    }
    std::string rest, sep_name;
    std::getline(in, rest, '\n');
    std::istringstream(rest) >> sep_name;
    const char sep = sep_name == "tab" ? '\t' : (sep_name == "comma" || sep_name == "," ? ',' : (sep_name == "space" ? ' ' : 0));
    if (in.fail()) throw std::runtime_error("reading file " + path + " failed (while reading size)");
    if (size[0] != nz || size[1] != ny || size[2] != nx)
        throw std::runtime_error("failed to read excitation sequence due to its incompatible size");
    // one time per cell, z slowest; a failed extraction leaves 0 (the cells start at 0)
    at.assign((size_t)nz * ny * nx, 0.0);
    for (size_t i = 0; i < at.size() && in; ++i) {
        double v = 0.0;
        if (!(in >> v)) break;
        at[i] = v;
        if (sep == ',') in.ignore(1);
    }
}

void write_excitation(const std::string &path, int nz, int ny, int nx, const double *at) {
    if (!has_matrix_ext(path)) throw std::runtime_error("can only export to .matrix for the time being");
    std::FILE *f = std::fopen(path.c_str(), "w");
    if (!f) throw std::runtime_error("could not open file " + path + " to export the excitation sequence");
    std::fputs("Excitation file (next line specifies matrix type (2D) size (X x Y x Z) and elemet separator type "
               "(tab) after that comes data (x are rows, y are lines, z are blocks - separated with empty line)\n",
               f);
    if (nz > 1) std::fprintf(f, "3D %d x %d x %d tab\n", nx, ny, nz);
    else std::fprintf(f, "2D %d x %d tab\n", nx, ny);
    for (int z = 0; z < nz; ++z) {
        for (int y = 0; y < ny; ++y) {
            const double *row = at + ((size_t)z * ny + y) * nx;
            for (int x = 0; x < nx; ++x) std::fprintf(f, x ? "\t%.3f" : "%.3f", row[x]);
            std::fputc('\n', f);
        }
        std::fputc('\n', f);
    }
    if (std::fclose(f) != 0) throw std::runtime_error("could not write " + path);
}

// ------------------------------------------------------------------ .matrix
namespace {
struct MatrixHeader {
    int dim = 0;
    long size[3] = {1, 1, 1};  // [0] slowest (z), [2] fastest (x)
    char sep = 0;
};
void read_header(std::istream &in, const std::string &path, MatrixHeader &h, int max_dim) {
    in.ignore(100000000, '\n');
    std::string dimStr;
    in >> dimStr;
    if (dimStr.size() >= 2 && (dimStr[1] == 'D' || dimStr[1] == 'd') && dimStr[0] > '0' && dimStr[0] <= '0' + max_dim) {
        h.dim = dimStr[0] - '0';
    } else {
        throw std::runtime_error("error while loading matrix, could not read dimensionality");
    }
    int writeDim = max_dim - 1;
    long sz[3] = {1, 1, 1};
    in >> sz[writeDim];
    for (int d = h.dim - 1; d > 0; --d) {
        in.ignore(100, 'x');
        --writeDim;
        in >> sz[writeDim];
    }
    std::string sepLine;
    std::getline(in, sepLine, '\n');
    std::istringstream ss(sepLine);
    std::string st;
    ss >> st;
    h.sep = st == "tab" ? '\t' : ((st == "comma" || st == ",") ? ',' : (st == "space" ? ' ' : 0));
    if (in.fail()) throw std::runtime_error("reading file " + path + " failed (while reading size)");
    for (int i = 0; i < 3; ++i) h.size[i] = 1;
    for (int i = 0; i < max_dim; ++i) h.size[3 - max_dim + i] = sz[i];
}
}  // namespace

void read_shape(const std::string &path, int &nz, int &ny, int &nx, std::vector<int32_t> &layers) {
    if (extension(path) != ".matrix") throw std::runtime_error("can only import from .matrix files for the time being");
    std::ifstream in(path.c_str());
    if (!in.is_open()) throw std::runtime_error("could not open file " + path);
    MatrixHeader h;
    read_header(in, path, h, 3);
    nz = (int)h.size[0];
    ny = (int)h.size[1];
    nx = (int)h.size[2];
    const size_t n = (size_t)nz * ny * nx;
    layers.assign(n, 0);
    for (size_t i = 0; i < n; ++i) {
        if (h.sep == ',' || h.sep == '\t' || h.sep == ' ') {
            int v;
            in >> v;
            layers[i] = v;  // negative = stimulus voxel of layer |v| (simlib/matrix.h:125-129)
            if (h.sep == ',') {
                const bool last_of_row = ((i + 1) % (size_t)nx) == 0;
                if (!last_of_row) in.ignore(100, ',');
            }
        } else {
            char ch;
            in >> ch;
            if (ch == 'x' || ch == 'X') layers[i] = -1;
            else if (ch >= 'a') layers[i] = ch - 'a' + 10;
            else if (ch >= 'A') layers[i] = ch - 'A' + 10;
            else layers[i] = ch - '0';
        }
    }
    if (in.fail()) throw std::runtime_error("reading file " + path + " failed (while reading data)");
}

void read_transfer(const std::string &path, int &n, std::vector<double> &t) {
    if (extension(path) != ".matrix") throw std::runtime_error("can only import from .matrix files for the time being");
    std::ifstream in(path.c_str());
    if (!in.is_open()) throw std::runtime_error("could not open file " + path);
    MatrixHeader h;
    read_header(in, path, h, 2);
    const long rows = h.size[1], cols = h.size[2];
    t.assign((size_t)rows * cols, 0.0);
    for (long i = 0; i < rows * cols; ++i) {
        in >> t[i];
        if (h.sep == ',' && ((i + 1) % cols) != 0) in.ignore(100, ',');
    }
    if (in.fail()) throw std::runtime_error("reading file " + path + " failed (while reading data)");
    if (rows != cols) throw std::runtime_error("conduction matrix must be square");
    n = (int)rows;
}

void read_points(const std::string &path, std::vector<double> &zyx) {
    std::ifstream in(path.c_str());
    zyx.clear();
    while (in.is_open() && !in.eof()) {
        double p[3];
        in >> p[2];
        in.ignore(1000, ',');
        in >> p[1];
        in.ignore(1000, ',');
        in >> p[0];
        in.ignore(1000, '\n');
        if (in.fail()) break;
        zyx.insert(zyx.end(), p, p + 3);
    }
    if (zyx.empty()) throw std::runtime_error("failed to open file containing measuring points: " + path);
}

void read_columns(const std::string &path, std::vector<std::vector<double>> &cols) {
    if (extension(path) != ".column") throw std::runtime_error("ColumnFile::load only works on .column files");
    std::ifstream in(path.c_str());
    if (!in.is_open()) throw std::runtime_error("could not open " + path);
    while (in.peek() == '#' || in.peek() == '%') in.ignore(10000, '\n');
    std::string line;
    std::getline(in, line);
    std::istringstream ls(line);
    std::vector<double> tmp;
    double d;
    while (ls >> d) tmp.push_back(d);
    ls.clear();
    if (tmp.empty()) throw std::runtime_error("File has 0 columns");
    cols.assign(tmp.size(), std::vector<double>());
    while (in && ls) {
        for (size_t i = 0; i < cols.size(); ++i) cols[i].push_back(tmp[i]);
        std::getline(in, line);
        ls.clear();
        ls.str(line);
        for (size_t i = 0; i < tmp.size(); ++i) ls >> tmp[i];
    }
}

void resample(const std::vector<double> &src, std::vector<double> &dest, double factor, int start_offset) {
    if (factor == 1) {
        dest = src;
        return;
    }
    dest.resize(1u + (size_t)std::ceil((double)(src.size() - 1 - start_offset) * factor));
    for (size_t i = 0; i < dest.size(); ++i) {
        double oldPos = i / factor + start_offset;
        size_t fPos = (size_t)std::floor(oldPos);
        size_t cPos = (size_t)(1.0 + fPos);
        if (cPos < src.size()) dest[i] = src[cPos] * (oldPos - fPos) + src[fPos] * (cPos - oldPos);
        else dest[i] = src.back();
    }
}

void write_columns(const std::string &path, const std::vector<std::string> &names,
                   const std::vector<std::string> &comments, const std::vector<const std::vector<double> *> &data,
                   double start, double dt, const std::string &comment) {
    if (extension(path) != ".column") throw std::runtime_error("saving vectors to .column files only for the time being");
    std::ofstream out(path.c_str());
    out << "#Comment: " << comment << '\n';
    for (size_t i = 0; i < names.size(); ++i)
        if (i < comments.size() && !comments[i].empty()) out << "# " << names[i] << " : " << comments[i] << '\n';
    out << "# \n";
    if (dt > 0) out << "#Time[ms]\t";
    else out << "# ";
    for (size_t i = 0; i < names.size(); ++i) {
        if (i > 0) out << '\t';
        out << names[i];
    }
    out << '\n';
    double time = start;
    const size_t n = data.empty() ? 0 : data[0]->size();
    for (size_t i = 0; i < n; ++i) {
        if (i > 0) out << "\n";
        if (dt > 0) {
            out << std::fixed << std::setprecision(5) << std::setw(10) << time << '\t';
            time += dt;
        }
        for (size_t j = 0; j < data.size(); ++j) {
            if (j > 0) out << '\t';
            out << std::scientific << std::setw(10) << (*data[j])[i];
        }
    }
}

void load_targets(const SimConfig &c, const std::string &path, const std::string &out_dir,
                  std::vector<std::vector<double>> &targets, std::vector<double> &offsets) {
    std::vector<std::vector<double>> cols;
    read_columns(path, cols);
    const size_t ncol = cols.size();
    targets.assign(std::max<size_t>(1, ncol - 1), std::vector<double>());
    offsets.assign(targets.size(), 0.0);
    double target_dt = c.ap_time_step;
    const size_t ecg_cols = std::min<size_t>(1, ncol - 1);
    if (ecg_cols > 0) target_dt = cols[0][1] - cols[0][0];
    const int rstart = (int)(c.start / target_dt);
    for (size_t i = ecg_cols; i < ncol; ++i) {
        std::vector<double> &col = cols[i];
        double tmin = col[0], tmax = col[0];
        for (size_t j = 1; j < col.size(); ++j) {
            if (col[j] < tmin) tmin = col[j];
            else if (col[j] > tmax) tmax = col[j];
        }
        const double m = 1.0 / (tmax - tmin);
        for (double &v : col) v *= m;
        resample(col, targets[i - ecg_cols], target_dt / c.dt, rstart);
        offsets[i - ecg_cols] = 1.0 - (tmin / (tmax - tmin));
    }
    if (!out_dir.empty()) {
        std::vector<std::string> names;
        std::vector<const std::vector<double> *> data;
        for (size_t i = 0; i < targets.size(); ++i) {
            names.push_back("target " + std::to_string(i + 1));
            data.push_back(&targets[i]);
        }
        write_columns(out_dir + "/target_chk.column", names, {}, data, c.start, c.dt, "");
    }
}

// ------------------------------------------------------------------ Wohlfart AP and genes
// The formula as three factors, evaluated in the reference's operation order:
//   value = A * B * C + k0,  A = 1 / (1 + e^{-k1 t}),  B = k2 ((1 - k3) e^{-k4 t} + k3),
//   C = e^{-k5 t} R,  R = 1 - (1 + e^{-k7 (t - k8) + lc})^{ex},  lc = log(2^{k7/k6} - 1),  ex = -(k6/k7).
// lc and ex depend on the coefficients only, so callers that evaluate one AP at many times compute
// them once; a change of one coefficient re-evaluates only the factors it enters (same results).
namespace {
struct RepolConst {
    double lc, ex;
};
inline RepolConst repol_const(const double *k) { return {std::log(std::pow(2, (k[7] / k[6])) - 1), -(k[6] / k[7])}; }
inline double fac_a(const double *k, double t) { return 1.0 / (1.0 + std::exp(-k[1] * t)); }
inline double fac_b(const double *k, double e4) { return k[2] * ((1.0 - k[3]) * e4 + k[3]); }
inline double fac_r(const double *k, const RepolConst &rc, double t) {
    return 1 - std::pow((1 + std::exp(-k[7] * (t - k[8]) + rc.lc)), rc.ex);
}
inline double wohlfart_rc(const double *k, const RepolConst &rc, double t) {
    return fac_a(k, t) * fac_b(k, std::exp(-k[4] * t)) * (std::exp(-k[5] * t) * fac_r(k, rc, t)) + k[0];
}
}  // namespace

double wohlfart(const double *k, double t) { return wohlfart_rc(k, repol_const(k), t); }

WohlfartAP::WohlfartAP(const double *k) : k_(k) {
    const RepolConst rc = repol_const(k);
    lc_ = rc.lc;
    ex_ = rc.ex;
}
double WohlfartAP::operator()(double t) const { return wohlfart_rc(k_, RepolConst{lc_, ex_}, t); }

int GeneModel::n_free() const { return __builtin_popcount(free_mask & 0x1ffu); }

namespace {
struct AP {
    double k[9];
    double at = 0;
    double operator()(double t) const { return wohlfart(k, t - at); }
};
// The samples of a border AP at t = 0 .. 699 ms (the interpolation evaluator's curve) and its
// apd90, computed once per distinct border AP (the mid AP borders both segments).
struct Curve {
    double k[9];
    double y[701];
    double apd = -1.0;
};
// WohlfartPlus::apd90 (simlib/Wohlfart.h:206-223): the last downward crossing of k0 + k2/10 among
// the samples at 0 .. 999 ms, found by scanning from the end (the samples after it are the only
// ones that decide that it is the last).  The samples below 700 ms are the curve's (the same
// wohlfart_rc arguments, so the same doubles); the others are evaluated here.
double apd90(const double *k, const RepolConst &rc, const double *y) {
    const double target = k[0] + k[2] * 0.1;
    auto sample = [&](int i) { return i < 700 ? y[i] : wohlfart_rc(k, rc, (double)i); };
    double next = sample(999);
    for (int i = 999; i >= 1; --i) {
        const double prev = sample(i - 1);
        if (prev > target && next <= target) {
            const double a = i - 1, wa = prev - target, b = i, wb = target - next;
            return (a * wa + b * wb) / (wa + wb);
        }
        next = prev;
    }
    return -1.0;
}
// the curve of a border AP (activation time 0)
void make_curve(const double *k, Curve &c) {
    std::copy(k, k + 9, c.k);
    const RepolConst rc = repol_const(k);
    for (size_t i = 0; i < 700; ++i) c.y[i] = wohlfart_rc(k, rc, (double)i);
    c.y[700] = c.y[699];  // the reference reads one past its 700-sample buffer here; hold the last value
    c.apd = apd90(k, rc, c.y);
}
// WohlfartInterpolationEvaluator (sim.cpp:91-313): connectors between two border APs, points
// on them at a ratio, and the sum of squared distances of an AP from those points.
struct Evaluator {
    struct Conn {
        double k, n, x1, x2;
    };
    std::vector<Conn> conns;
    std::vector<double> pts;
    void set_border(const Curve &c1, const Curve &c2) {
        conns.clear();
        const size_t numPoints = 15, startX = 10;
        const double apd1 = c1.apd, apd2 = c2.apd;
        const double *y1 = c1.y, *y2 = c2.y;
        const double xs = 0.1;
        const size_t e1 = apd1 < 0 ? 0 : std::min<size_t>(700, (size_t)std::ceil(apd1));
        const size_t e2 = apd2 < 0 ? 0 : std::min<size_t>(700, (size_t)std::ceil(apd2));
        double len1 = 0.0, len2 = 0.0;
        for (size_t i = startX + 1; i < e1; ++i) len1 += std::sqrt((y1[i] - y1[i - 1]) * (y1[i] - y1[i - 1]) + xs);
        for (size_t i = startX; i < e2; ++i) len2 += std::sqrt((y2[i] - y2[i - 1]) * (y2[i] - y2[i - 1]) + xs);
        double cur1 = 0.0, cur2 = 0.0;
        size_t i1 = startX, i2 = startX;
        Conn lc{100, 0, 0, 0};
        for (size_t i = 0; i < numPoints; ++i) {
            double target = (double)i * len1 / (double)(numPoints - 2);
            for (double l1 = cur1; (l1 < target) && (i1 < 700); ++i1)
                l1 += std::sqrt((y1[i1 + 1] - y1[i1]) * (y1[i1 + 1] - y1[i1]) + xs);
            cur1 = target;
            target = (double)i * len2 / (double)(numPoints - 2);
            for (double l2 = cur2; (l2 < target) && (i2 < 700); ++i2)
                l2 += std::sqrt((y2[i2 + 1] - y2[i2]) * (y2[i2 + 1] - y2[i2]) + xs);
            cur2 = target;
            lc.x1 = (double)i1;
            lc.x2 = (double)i2;
            if (i1 == i2) lc.x2 += 0.001;
            lc.k = (y1[std::min<size_t>(i1, 700)] - y2[std::min<size_t>(i2, 700)]) / (lc.x1 - lc.x2);
            lc.n = y2[std::min<size_t>(i2, 700)] - lc.k * (double)i2;
            conns.push_back(lc);
        }
        static_assert(numPoints <= kMaxPts, "the fit's factor cache holds every point");
    }
    void set_ratio(double r) {
        pts.clear();
        for (const Conn &c : conns) {
            const double x = c.x1 + (c.x2 - c.x1) * r;
            pts.push_back(x);
            pts.push_back(c.k * x + c.n);
        }
    }
    double operator()(const AP &ap) const {
        double sum = 0;
        for (size_t i = 0; i < pts.size(); i += 2) {
            const double q = ap(pts[i]) - pts[i + 1];
            sum += q * q;
        }
        return sum;
    }
    // The same sum with the factors of every point kept (A, e^{-k4 t}, e^{-k5 t}, R): `full` computes
    // them all, `from` re-evaluates only the factors whose coefficients differ from those of the AP
    // `ref` the kept factors `c` belong to (and keeps the new ones in `out` when given).  Both give
    // the doubles operator() gives.
    static constexpr size_t kMaxPts = 16;  // set_border makes 15 points
    struct Factors {
        double a[kMaxPts], e4[kMaxPts], e5[kMaxPts], r[kMaxPts];
    };
    double full(const AP &ap, Factors &c) const {
        const RepolConst rc = repol_const(ap.k);
        double sum = 0;
        for (size_t i = 0, p = 0; i < pts.size(); i += 2, ++p) {
            const double t = pts[i] - ap.at;
            c.a[p] = fac_a(ap.k, t);
            c.e4[p] = std::exp(-ap.k[4] * t);
            c.e5[p] = std::exp(-ap.k[5] * t);
            c.r[p] = fac_r(ap.k, rc, t);
            const double q = (c.a[p] * fac_b(ap.k, c.e4[p]) * (c.e5[p] * c.r[p]) + ap.k[0]) - pts[i + 1];
            sum += q * q;
        }
        return sum;
    }
    double from(const AP &ap, const AP &ref, const Factors &c, Factors *out) const {
        const bool ka = ap.k[1] != ref.k[1] || ap.at != ref.at, k4 = ap.k[4] != ref.k[4] || ap.at != ref.at;
        const bool k5 = ap.k[5] != ref.k[5] || ap.at != ref.at;
        const bool kr = ap.k[6] != ref.k[6] || ap.k[7] != ref.k[7] || ap.k[8] != ref.k[8] || ap.at != ref.at;
        const RepolConst rc = kr ? repol_const(ap.k) : RepolConst{0, 0};
        double sum = 0;
        for (size_t i = 0, p = 0; i < pts.size(); i += 2, ++p) {
            const double t = pts[i] - ap.at;
            const double a = ka ? fac_a(ap.k, t) : c.a[p];
            const double e4 = k4 ? std::exp(-ap.k[4] * t) : c.e4[p];
            const double e5 = k5 ? std::exp(-ap.k[5] * t) : c.e5[p];
            const double r = kr ? fac_r(ap.k, rc, t) : c.r[p];
            if (out) {
                out->a[p] = a;
                out->e4[p] = e4;
                out->e5[p] = e5;
                out->r[p] = r;
            }
            const double q = (a * fac_b(ap.k, e4) * (e5 * r) + ap.k[0]) - pts[i + 1];
            sum += q * q;
        }
        return sum;
    }
};
// steepestDescend (nonlinearFit.h:92-168) over the 9 k values
// (the gradient probes and the step change some coefficients only, so they re-evaluate only the
// factors those enter)
void steepest(const Evaluator &f, AP &x0, const AP &d, double stepSize, double epsilon, int iterations) {
    AP grad = x0, oldGrad = x0, move = d;
    for (int i = 0; i < 9; ++i) oldGrad.k[i] = 0;
    Evaluator::Factors c0, c1;
    double y0 = f.full(x0, c0);
    for (; iterations > 0 && y0 > epsilon; --iterations) {
        bool stepChange = false;
        for (int i = 0; i < 9; ++i) {
            AP x1 = x0;
            if (d.k[i] != 0) {
                x1.k[i] += d.k[i] * .001;
                grad.k[i] = (f.from(x1, x0, c0, nullptr) - y0) / (d.k[i] * .001);
                if (grad.k[i] * oldGrad.k[i] < 0) {
                    move.k[i] *= 0.5;
                    stepChange = true;
                } else if (std::fabs(grad.k[i]) > 0.75 * std::fabs(oldGrad.k[i])) {
                    move.k[i] *= 1.5;
                }
            } else {
                grad.k[i] = 0;
            }
        }
        oldGrad = grad;
        AP x1 = x0;
        for (int i = 0; i < 9; ++i) x1.k[i] -= stepSize * ((grad.k[i] > 0) ? move.k[i] : -move.k[i]);
        const double y1 = f.from(x1, x0, c0, &c1);
        if (y1 < y0) {
            y0 = y1;
            x0 = x1;
            c0 = c1;
        } else if (!stepChange) {
            stepSize *= 0.5;
        }
    }
}
void combine(AP &dst, const AP &s1, const AP &s2, double ratio) {
    for (int i = 0; i < 9; ++i) dst.k[i] = s1.k[i] * (1 - ratio) + s2.k[i] * ratio;
}
}  // namespace

void layer_aps_setup(const GeneModel &m, int nl, const double *genes, double *out_k, double *violation,
                     std::vector<LayerFit> &fits) {
    std::fill(out_k, out_k + 9 * (size_t)nl, 0.0);
    int gi = 0;
    double viol = 0.0;
    auto fill = [&](const std::vector<double> &base, int row) {
        double *k = out_k + 9 * (size_t)row;
        std::copy(base.begin(), base.begin() + 9, k);
        for (int i = 0; i < 9; ++i)
            if (m.free_mask & (1u << i)) {
                k[i] = genes[gi++];
                if (k[i] < m.k_min[i]) viol += m.k_min[i] - k[i];
                else if (k[i] > m.k_max[i]) viol += k[i] - m.k_max[i];
            }
    };
    if (m.interpolation == 1) {
        fill(m.base.front(), 0);
        fill(m.base.back(), nl - 1);
        for (int i = 1; i < nl - 1; ++i) fits.push_back(LayerFit{i, 0, nl - 1, i / double(nl - 1)});
    } else {
        const int mid = (int)std::floor(m.mid_position * (nl - 1) + 0.5);
        fill(m.base.front(), 0);
        fill(m.base.back(), mid);  // the mid AP starts from the last base AP (sim.cpp:855-864)
        fill(m.base.back(), nl - 1);
        for (int i = 1; i + 1 < nl; ++i) {
            if (i < mid) fits.push_back(LayerFit{i, 0, mid, i / double(mid)});
            else if (i > mid) fits.push_back(LayerFit{i, mid, nl - 1, (i - mid) / double(nl - mid - 1)});
        }
    }
    *violation = viol;
}

void layer_aps_run_fits(const LayerFitJob *jobs, size_t n) {
    static const double kd[9] = {0, 0, 0, 0.001, 0, 0.00005, 0.0005, 0.01, 0.2};
    AP d;
    std::copy(kd, kd + 9, d.k);
    // the interpolation evaluator (connectors between the two border APs) is rebuilt only when the
    // border APs change from one fit to the next; the border APs' curves come from a small cache
    // (a simulation's mid AP borders both of its segments)
    Evaluator ev;
    double key[18];
    bool have = false;
    Curve cache[4];
    int ncache = 0, next_slot = 0;
    auto curve = [&](const double *kk) -> const Curve & {
        for (int i = 0; i < ncache; ++i)
            if (std::memcmp(cache[i].k, kk, 72) == 0) return cache[i];
        Curve &c = cache[next_slot];
        next_slot = (next_slot + 1) % 4;
        ncache = std::min(ncache + 1, 4);
        make_curve(kk, c);
        return c;
    };
    for (size_t j = 0; j < n; ++j) {
        const LayerFit &f = jobs[j].fit;
        double *k = jobs[j].out_k;
        AP a, b;
        std::copy(k + 9 * (size_t)f.a, k + 9 * (size_t)f.a + 9, a.k);
        std::copy(k + 9 * (size_t)f.b, k + 9 * (size_t)f.b + 9, b.k);
        if (!have || std::memcmp(key, a.k, 72) != 0 || std::memcmp(key + 9, b.k, 72) != 0) {
            const Curve &ca = curve(a.k);
            const Curve &cb = curve(b.k);  // the cache holds four curves: this never evicts ca
            ev.set_border(ca, cb);
            std::copy(a.k, a.k + 9, key);
            std::copy(b.k, b.k + 9, key + 9);
            have = true;
        }
        ev.set_ratio(f.ratio);
        AP x;
        combine(x, a, b, f.ratio);
        steepest(ev, x, d, 0.5, 1e-3, 100);
        std::copy(x.k, x.k + 9, k + 9 * (size_t)f.layer);
    }
}

void layer_aps_from_genes(const GeneModel &m, int nl, const double *genes, double *out_k, double *violation) {
    std::vector<LayerFit> fits;
    layer_aps_setup(m, nl, genes, out_k, violation, fits);
    std::vector<LayerFitJob> jobs;
    for (const LayerFit &f : fits) jobs.push_back(LayerFitJob{f, out_k});
    layer_aps_run_fits(jobs.data(), jobs.size());
}

void lead_frames(int n, const double *orig, double *uv) {
    for (int i = 0; i < n; ++i) {
        const double *p = orig + 3 * i;
        const double x[3] = {0, 0, 1};
        double u[3] = {x[1] * p[2] - x[2] * p[1], x[2] * p[0] - x[0] * p[2], x[0] * p[1] - x[1] * p[0]};
        double v[3] = {u[1] * p[2] - u[2] * p[1], u[2] * p[0] - u[0] * p[2], u[0] * p[1] - u[1] * p[0]};
        for (double &c : u) c *= -1;
        for (double *w : {u, v}) {
            double s = w[0] * w[0];
            s += w[1] * w[1];
            s += w[2] * w[2];
            const double l = std::sqrt(s);
            if (l != 0) {
                const double f = 1.0 / l;
                w[0] *= f;
                w[1] *= f;
                w[2] *= f;
            } else {
                w[0] *= 0.0;
                w[1] *= 0.0;
                w[2] *= 0.0;
            }
        }
        std::copy(u, u + 3, uv + 6 * i);
        std::copy(v, v + 3, uv + 6 * i + 3);
    }
}

void move_leads_framed(int n, const double *orig, const double *uv, const double *disp, double *out) {
    for (int i = 0; i < n; ++i) {
        const double *p = orig + 3 * i, *u = uv + 6 * i, *v = uv + 6 * i + 3;
        const double du = disp ? disp[2 * i] : 0.0, dv = disp ? disp[2 * i + 1] : 0.0;
        for (int c = 0; c < 3; ++c) out[3 * i + c] = (p[c] + du * u[c]) + dv * v[c];
    }
}

void move_leads(int n, const double *orig, const double *disp, double *out) {
    std::vector<double> uv(6 * (size_t)std::max(0, n));
    lead_frames(n, orig, uv.data());
    move_leads_framed(n, orig, uv.data(), disp, out);
}

}  // namespace ekg
