// ekgSim -- command-line drop-in for the reference's single-simulation mode, on the GPU engine.
//
//   ekgSim [free args] -sim p1,p2,...[,;] [-out result] [-out layer_aps] [-out "cell_aps i j ..."] [-?]
//
// Same arguments, stdout lines, output files and error behaviour as the reference's main.cpp:
// dash arguments take the next non-dash word as their value (a word starting with '-' and a digit
// is a value, so negative genes work), -out may repeat; the working directory must hold
// simulator.ini and the files it names; result.column / layer_aps.column / cell_aps.column are
// written in the reference's .column format; " criteria = <...>, violation = v" and "All done" go
// to stdout; errors are printed to stdout and the exit status stays 0 (main.cpp:387-414).
// The optimisation mode (no -sim) belongs to the AMS-DEMO optimiser and is not part of this
// program; it prints a message and exits like the reference does on missing arguments.
#include <cctype>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "ekgsim.h"

namespace {

struct Args {
    std::multimap<std::string, std::string> dash;
    std::vector<std::string> free;
    Args(int argc, char **argv) {
        std::multimap<std::string, std::string>::iterator last = dash.end();
        for (int i = 0; i < argc; ++i) {
            std::string a = argv[i];
            if (a.size() > 1 && a[0] == '-' && !std::isdigit((unsigned char)a[1])) {
                last = dash.insert(std::make_pair(a, std::string()));
            } else if (!dash.empty() && last != dash.end() && last->second.empty()) {
                last->second = a;
            } else {
                free.push_back(a);
            }
        }
    }
    bool has(const std::string &k) const { return dash.count(k) > 0; }
    std::vector<std::string> all(const std::string &k) const {
        std::vector<std::string> v;
        auto r = dash.equal_range(k);
        for (auto it = r.first; it != r.second; ++it) v.push_back(it->second);
        return v;
    }
};

template <class T>
std::string vec_str(const std::vector<T> &v) {  // "<a,b,c>" with default stream precision
    std::ostringstream s;
    s << "<";
    for (size_t i = 0; i < v.size(); ++i) s << (i ? "," : "") << v[i];
    s << ">";
    return s.str();
}

void check(int rc) {
    if (rc != EKG_OK) throw std::runtime_error(ekg_last_error());
}

// exportVectors (simlib/simulator.h:196-240): "#Comment: ...", "# name : comment" lines, "# ",
// the "#Time[ms]" header with tab-separated names, rows "%10.5f\t%10.5e..." (precision 5 sticks)
void write_column(const std::string &path, const std::vector<std::string> &names,
                  const std::vector<std::string> &comments, const std::vector<std::vector<double>> &data, double start,
                  double dt, const std::string &comment) {
    std::ofstream out(path.c_str());
    out << "#Comment: " << comment << '\n';
    for (size_t i = 0; i < names.size(); ++i)
        if (i < comments.size() && !comments[i].empty()) out << "# " << names[i] << " : " << comments[i] << '\n';
    out << "# \n";
    out << (dt > 0 ? "#Time[ms]\t" : "# ");
    for (size_t i = 0; i < names.size(); ++i) out << (i ? "\t" : "") << names[i];
    out << '\n';
    double time = start;
    const size_t n = data.empty() ? 0 : data[0].size();
    for (size_t i = 0; i < n; ++i) {
        if (i > 0) out << "\n";
        if (dt > 0) {
            out << std::fixed << std::setprecision(5) << std::setw(10) << time << '\t';
            time += dt;
        }
        for (size_t j = 0; j < data.size(); ++j) out << (j ? "\t" : "") << std::scientific << std::setw(10) << data[j][i];
    }
}

// OutputAps (sim.cpp:919-975): 700 samples at t = 0..699 per AP, "ap_<name>" columns with a
// "k = [k0, ..., k8]" comment (k8 already shifted by the activation time)
void write_aps(const std::string &path, const std::vector<std::string> &names, const std::vector<std::vector<double>> &ks,
               const std::vector<double> &ats) {
    std::vector<std::string> comments;
    std::vector<std::vector<double>> data;
    for (size_t i = 0; i < ks.size(); ++i) {
        double k[9];
        for (int j = 0; j < 9; ++j) k[j] = ks[i][j];
        k[8] -= ats[i];
        std::ostringstream c;
        c << "k = [" << k[0];
        for (int j = 1; j < 9; ++j) c << ", " << k[j];
        c << "]";
        comments.push_back(c.str());
        std::vector<double> v(700);
        for (int t = 0; t < 700; ++t) v[t] = ekg_ap_value(ks[i].data(), ats[i], (double)t);
        data.push_back(v);
    }
    if (!names.empty()) write_column(path, names, comments, data, 0, 1, "");
}

int run(int argc, char **argv) {
    Args args(argc, argv);
    std::cerr << "***** parsing program arguments ****************************\n";
    bool want_result = false, want_layer_aps = false;
    std::vector<size_t> cell_aps;
    bool help = args.has("-?");
    if (args.has("-out")) {
        for (const std::string &o : args.all("-out")) {
            std::istringstream st(o);
            std::string name;
            st >> name;
            if (name == "cell_aps") {
                while (st) {
                    st.ignore(1);
                    size_t num;
                    st >> num;
                    if (st) cell_aps.push_back(num);
                }
            } else if (name == "layer_aps") {
                want_layer_aps = true;
            } else if (name == "result") {
                want_result = true;
            } else {
                std::cerr << "skipping an unrecognized output opition: " << name << "\n";
            }
        }
        std::cout << "\n";
    }
    if (help || argc <= 1) {
        std::cout << "Argument list:\n"
                  << "   -? \tshow this help screen\n"
                  << "   -out \tspecify outputs of the program; possible values include result, layer_aps, "
                     "cell_aps <num> [<num>]*\n"
                  << "   -sim \tjust run single a simulation with parameters provided after -sim\n"
                  << "   -test \trun test function (changable function used for debugging)\n";
    }
    if (args.has("-test")) return 0;
    if (!args.has("-sim")) {
        if (!help) std::cout << "missing program arguments, stopping execution (the optimisation mode runs in the "
                                "AMS-DEMO optimiser; use -sim for a single simulation)\n";
        std::cout << "All done\n";
        return 0;
    }
    std::vector<double> genes;
    {
        std::string v;
        auto r = args.dash.equal_range("-sim");
        if (r.first != r.second) v = r.first->second;
        std::istringstream s(v);
        for (double t; s >> t;) {
            genes.push_back(t);
            const int c = s.peek();
            if (c == ',' || c == ';') s.ignore(1);
        }
        std::cout << " parameters for single simulator run: " << vec_str(genes) << "\n";
        if (genes.empty()) throw std::runtime_error(" Error: not enough parameters to run simulation: " + v);
    }
    std::cerr << "##### Running a single simulation experiment ####################\n";
    ekg_engine *eng = nullptr;
    check(ekg_engine_create(0, &eng));
    ekg_heart *heart = nullptr;
    check(ekg_heart_from_ini(eng, "simulator.ini", ".", &heart));
    ekg_heart_info info;
    check(ekg_heart_get_info(heart, &info));
    int32_t ng = 0, nc = 0;
    check(ekg_eval_shape(heart, &ng, &nc));
    std::vector<double> crit(nc), ecg((size_t)info.n_leads * info.steps), lk((size_t)info.n_layers * 9),
        leads((size_t)info.n_leads * 3);
    double viol = 0;
    const auto t0 = std::chrono::steady_clock::now();
    std::cout << "\reval 1  ";
    check(ekg_eval(heart, genes.data(), (int32_t)genes.size(), crit.data(), &viol, ecg.data(), lk.data(),
                   leads.data()));
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    int32_t simulated = 1;
    check(ekg_eval_simulated(heart, &simulated));
    // writeOutputs (sim.cpp:977-991)
    {
        std::vector<std::string> names;
        std::vector<std::vector<double>> ks;
        std::vector<double> ats;
        for (size_t idx : cell_aps) {
            int32_t L = 0;
            double at = 0;
            if (ekg_heart_cell_ap(heart, (int64_t)idx, &L, &at) != EKG_OK) continue;
            names.push_back("ap_" + std::to_string(idx));
            ks.emplace_back(lk.begin() + (L - 1) * 9, lk.begin() + L * 9);
            ats.push_back(at);
        }
        write_aps("cell_aps.column", names, ks, ats);
    }
    if (want_layer_aps) {
        std::vector<std::string> names;
        std::vector<std::vector<double>> ks;
        std::vector<double> ats;
        for (int L = 0; L < info.n_layers; ++L) {
            names.push_back("ap_" + std::to_string(L));
            ks.emplace_back(lk.begin() + L * 9, lk.begin() + (L + 1) * 9);
            ats.push_back(0.0);
        }
        write_aps("layer_aps.column", names, ks, ats);
    }
    if (want_result) {
        std::vector<std::string> names;
        std::vector<std::vector<double>> data;
        for (int l = 0; l < info.n_leads; ++l) {
            std::ostringstream nm;  // x,y,z of the (moved) lead, default precision
            nm << leads[3 * l + 2] << "," << leads[3 * l + 1] << "," << leads[3 * l + 0];
            names.push_back(nm.str());
            // a simulation the fast-approximation gate skipped has no measurement rows
            if (simulated) data.emplace_back(ecg.begin() + (size_t)l * info.steps, ecg.begin() + (size_t)(l + 1) * info.steps);
            else data.emplace_back();
        }
        double start = 0, length = 0, dt = 1;
        check(ekg_heart_time_axis(heart, &start, &length, &dt));
        write_column("result.column", names, {}, data, start, dt, "input=" + vec_str(genes) + "; ");
    }
    std::cout << " simulation done in " << secs << " seconds\n";
    std::cout << " criteria = " << vec_str(crit) << ", violation = " << viol << "\n";
    ekg_heart_destroy(heart);
    ekg_engine_destroy(eng);
    std::cout << "All done\n";
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    try {
        return run(argc, argv);
    } catch (const std::runtime_error &e) {
        std::cout << "runtime error caught: " << e.what() << "\n";
    } catch (const std::exception &e) {
        std::cout << "std exception caught: " << e.what() << "\n";
    } catch (...) {
        std::cout << "unknown exception caught, execution halted\n";
    }
    return 0;
}
