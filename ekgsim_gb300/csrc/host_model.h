// host_model.h -- host-side parts of one evaluation: simulator.ini settings, the reference's file
// formats, gene -> layer AP construction, lead displacement.  FP64 throughout; this is per-
// evaluation bookkeeping (microseconds for three layers), not the simulation itself, which runs
// on the device.
#pragma once

#include <stdint.h>

#include <map>
#include <string>
#include <vector>

namespace ekg {

// ------------------------------------------------------------------ INI (copyOfLibs/Ini.h semantics)
// Sections "[name]"; "name = value" lines (name and value trimmed of blanks/tabs); lines whose
// name starts with ';' are comments; a repeated name keeps its last value (copyOfLibs/Ini.cpp:171-200).
struct Ini {
    std::map<std::string, std::map<std::string, std::string>> sec;
    bool ok = false;
    bool load(const std::string &path);
    bool has(const std::string &s, const std::string &k) const;
    std::string str(const std::string &s, const std::string &k, const std::string &def = "") const;
    double num(const std::string &s, const std::string &k, double def) const;
    std::vector<double> vec(const std::string &s, const std::string &k) const;
};

// ------------------------------------------------------------------ settings
struct SimConfig {
    // [model] / [output files] / [simulation]  (simlib/simulator.h:107-145)
    std::string shape, transfer, points, excitation_in, excitation_out, results = "result.column";
    double start = 0, length = 800, dt = 1.0 / 3.0;
    std::string nhood;
    // [wohlfart ap] / [measuring points] / [optimization]  (SimSettings.h:158-356)
    std::vector<std::vector<double>> base_aps;
    std::vector<double> k_min, k_max;
    std::string interpolation;
    double mid_position = 0.5;
    std::vector<int> free_k;
    std::vector<int> disp_min, disp_max;
    std::string targets_file;
    int criteria_mode = 1, comparison_mode = 2;
    double endo_epi_delay = -1;
    bool peak = false, optimize_points = false, fast_is_crit = false;
    double fast_delay = 0, fast_limit = 2;
    size_t generations = 100, population = 0;
    int queue_size = 1;
    double ap_time_step = 1;  // [action potentials] resample time step (sim.cpp:1008)
};
// Parses the keys both SimLib::Settings and SimSettings read; throws std::runtime_error with the
// reference's messages on the errors the reference throws on.
SimConfig load_config(const std::string &ini_path);
int nhood_code(const std::string &name);  // EKG_NHOOD_* or -1

// ------------------------------------------------------------------ files
// importMatrix with shapeLoad (simlib/matrix.h:125-248): signed layer grid [z][y][x].
void read_shape(const std::string &path, int &nz, int &ny, int &nx, std::vector<int32_t> &layers);
// importMatrix with the default loader for the conduction matrix: n x n row-major.
void read_transfer(const std::string &path, int &n, std::vector<double> &t);
// Simulation::loadMeasuringPoints (simlib/simulator.cpp:369-397): returns (z,y,x) triples.
void read_points(const std::string &path, std::vector<double> &zyx);
// Simulation::loadExcitationSequence for .matrix files (simlib/simulator.cpp:288-367): one time per
// cell [z][y][x] after a comment line and the "<d>D X x Y x Z <sep>" header; the size must be the
// shape's.
void read_excitation(const std::string &path, int nz, int ny, int nx, std::vector<double> &at);
// exportShape with excit = true (simlib/simulator.cpp:71-106): times printed with 3 decimals.
void write_excitation(const std::string &path, int nz, int ny, int nx, const double *at);
// ColumnFile::load (simlib/columnFile.h:115-165).
void read_columns(const std::string &path, std::vector<std::vector<double>> &cols);
// SimImplementation::loadTargets (sim.cpp:999-1042); writes target_chk.column into out_dir
// unless out_dir is empty.
void load_targets(const SimConfig &c, const std::string &path, const std::string &out_dir,
                  std::vector<std::vector<double>> &targets, std::vector<double> &offsets);
// vectorMath.h:210-227
void resample(const std::vector<double> &src, std::vector<double> &dest, double factor, int start_offset);
// exportVectors for .column files (simlib/simulator.h:196-240).
void write_columns(const std::string &path, const std::vector<std::string> &names,
                   const std::vector<std::string> &comments, const std::vector<const std::vector<double> *> &data,
                   double start, double dt, const std::string &comment);

// ------------------------------------------------------------------ APs and genes
double wohlfart(const double *k, double t);  // WohlfartPlus::operator[] (simlib/Wohlfart.h:195-203)
// One AP evaluated at many times: the coefficient-only repolarisation constants are computed once;
// every value equals wohlfart(k, t) bit for bit.
class WohlfartAP {
  public:
    explicit WohlfartAP(const double *k);
    double operator()(double t) const;

  private:
    const double *k_;
    double lc_, ex_;
};

struct GeneModel {
    int interpolation = 2;  // 1 endo-epi, 2 endo-mid-epi
    double mid_position = 0.5;
    std::vector<std::vector<double>> base;  // base APs (9 each)
    std::vector<double> k_min, k_max;
    uint32_t free_mask = 0;
    int n_free() const;
};
// simUsingBorderAps / simUsingBorderAndMidAps (sim.cpp:751-916): layer APs [nl][9] and the
// violation of the gene-set APs (sim.cpp:582-596).
void layer_aps_from_genes(const GeneModel &m, int n_layers, const double *genes, double *out_k, double *violation);
// The same in two phases, so that the fits of many layers and simulations can run in parallel:
// layer_aps_setup writes the gene-set APs (rows of out_k) and the violation and lists the fits of the
// interpolated layers; each fit (steepest descent from the interpolated start, nonlinearFit.h:92-168)
// reads its two border rows and writes its own row, independently of the other fits (the start
// of layer i is fully overwritten by the interpolation, sim.cpp:800-830), so any order or split gives
// the same doubles.
struct LayerFit {
    int layer, a, b;  // fitted row, border rows
    double ratio;
};
struct LayerFitJob {
    LayerFit fit;
    double *out_k;    // the simulation's [nl][9]
};
void layer_aps_setup(const GeneModel &m, int n_layers, const double *genes, double *out_k, double *violation,
                     std::vector<LayerFit> &fits);
void layer_aps_run_fits(const LayerFitJob *jobs, size_t n);
// EkgSim::loadMeasuringPoints basis + moveMeasuringPoints (simlib/sim_lib.h:167-208).
void move_leads(int n, const double *orig_zyx, const double *disp_uv, double *out_zyx);
// the same in two parts: the per-lead displacement frames (u, v unit vectors, [n][6]), which depend
// only on the loaded positions, and the move itself (same arithmetic, same results)
void lead_frames(int n, const double *orig_zyx, double *uv);
void move_leads_framed(int n, const double *orig_zyx, const double *uv, const double *disp_uv, double *out_zyx);

}  // namespace ekg
