// frontend.cpp — host side of the drop-in boundary: the reference's input,
// xyz, parameter and cube readers, the System preparation of
// Simulation::initialize, pair-parameter resolution, and the scan-file writer.
//
// Behaviour (defaults, keywords, error texts, warnings, output formats) follows
// the reference so that `mechafm-gpu` is a drop-in for `mechafm-omp`:
//   readInputFile        parse.cpp:83-474
//   readXYZFile          parse.cpp:477-585
//   readParameterFile    parse.cpp:588-697 (+ readFlexibleParameters :699-782)
//   CubeReader           cube_io.cpp:10-139
//   Simulation::initialize / build*Interactions   simulation.cpp:31-65, 201-515
//   writeOutput / openUniverse / finalize          simulation.cpp:145-199,
//                                                  mechafm.cpp:37-80, 103-154
// Everything here is compiled with -ffp-contract=off: the reference is built
// for x86-64 without FMA, and the host arithmetic (centring, mixing, matrix
// inverse) must give the same bits on an aarch64 host.
#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <functional>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "mafm_internal.h"

namespace mafm {

static thread_local std::string g_last_error;

void set_last_error(const std::string& msg) { g_last_error = msg; }

void fail(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    throw Failure{code, buf};
}

namespace {

constexpr int kLine = 512;    // LINE_LENGTH (globals.hpp:6)
constexpr double kPi = 3.14159265358979323846;       // globals.hpp:10
constexpr double kSixthRoot2 = 1.12246204830937298142;  // globals.hpp:11
constexpr double kTolerance = 1e-10;                 // globals.hpp:8
constexpr double kBohr = 0.52917721092;              // cube_io.hpp:17
constexpr double kHartreeEV = 27.211386;             // globals.hpp:20-22
constexpr double kHartreeKJ = 2625.5002;
constexpr double kHartreeKcal = 627.50961;

enum Normal { NORMAL_X, NORMAL_Y, NORMAL_Z };

struct AtomParams {
    double eps = 0, sig = 0, q = 0, mass = 0;
};

struct Overwrite {
    std::string a, b;
    bool morse = false;
    double eps = 0, sig = 0, de = 0, alpha = 0, re = 0;
};

bool is_comment(const char* line) {
    return line[0] == '#' || line[0] == '%' || line[0] == '\n';
}

void lower(char* s) {
    for (; *s; ++s) *s = (char)tolower((unsigned char)*s);
}

bool is_int(const char* s) {
    for (; *s; ++s)
        if (!(isdigit((unsigned char)*s) || *s == '-' || *s == '+')) return false;
    return true;
}

int count_columns(const char* line) {
    char buf[kLine];
    snprintf(buf, sizeof buf, "%s", line);
    int n = 0;
    for (char* t = strtok(buf, " \t\n\r\f"); t; t = strtok(nullptr, " \t\n\r\f")) ++n;
    return n;
}

bool multiset_eq(const std::string& a, const std::string& b, const std::string& c,
                 const std::string& d) {
    return (a == c && b == d) || (a == d && b == c);
}

// 3x3 helpers with the reference's operation order (matrices.hpp:89-160).
struct M3 {
    double v[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double det() const {
        double d = 0;
        d = v[0][0] * (v[1][1] * v[2][2] - v[1][2] * v[2][1]);
        d += v[0][1] * (v[1][2] * v[2][0] - v[1][0] * v[2][2]);
        d += v[0][2] * (v[1][0] * v[2][1] - v[1][1] * v[2][0]);
        return d;
    }
    M3 inverse() const {
        M3 r;
        double inv_det = 1 / det();
        double a = v[0][0], b = v[0][1], c = v[0][2];
        double d = v[1][0], e = v[1][1], f = v[1][2];
        double g = v[2][0], h = v[2][1], i = v[2][2];
        r.v[0][0] = inv_det * (e * i - f * h);
        r.v[0][1] = -inv_det * (b * i - c * h);
        r.v[0][2] = inv_det * (b * f - c * e);
        r.v[1][0] = -inv_det * (d * i - f * g);
        r.v[1][1] = inv_det * (a * i - c * g);
        r.v[1][2] = -inv_det * (a * f - c * d);
        r.v[2][0] = inv_det * (d * h - e * g);
        r.v[2][1] = -inv_det * (a * h - b * g);
        r.v[2][2] = inv_det * (a * e - b * d);
        return r;
    }
    M3 mul(const M3& o) const {
        M3 r;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                for (int k = 0; k < 3; k++) r.v[i][j] += v[i][k] * o.v[k][j];
        return r;
    }
    M3 transpose() const {
        M3 r;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) r.v[i][j] = v[j][i];
        return r;
    }
};

}  // namespace
}  // namespace mafm

// The opaque input handle of the C ABI.
struct mafm_input {
    // --- options (InputOptions, simulation.hpp:30-60) ---
    std::string inputfolder, inputfile, xyzfile, paramfile, e_potential_file;
    std::string tipatom, dummyatom;
    double area[2] = {10, 10}, center[2] = {-1, -1};
    double dx = 0.1, dy = 0.1, dz = 0.1, zlow = 6.0, zhigh = 10.0;
    bool vdw_pbc = false;
    double cell_a[3] = {0, 0, 0}, cell_b[3] = {0, 0, 0}, cell_c[3] = {0, 0, 0};
    int normal = mafm::NORMAL_Z;
    int units = MAFM_UNITS_KCAL;
    bool coulomb = false, tip_dummy_coulomb = false, use_external_potential = false;
    int maxsteps = 5000;
    int minterm = -1;
    double etol = 0.01, ftol = 0.01, dt = 0.001;
    int bufsize = 1000;
    bool gzip = true, statistics = false, flexible = false, rigidgrid = false;
    bool xyz_charges = false;
    int minimiser = MAFM_MIN_FIRE, integrator = MAFM_INT_MIDPOINT;
    // --- interaction parameters (InteractionParameters, interactions.hpp:47-55) ---
    // qbase is only assigned by a `units` line in the reference (parse.cpp:278-298);
    // without one it is left uninitialised there.  Here it starts at the kcal/mol value.
    double qbase = 332.06371;
    double harm_k = 0, harm_r0 = 0;
    double bond_k = 0, angle_k = 0, dihedral_k = 0;
    double sub_eps = 0, sub_sig = 0, sub_lambda = 0, sub_rc = 0, sub_k = 0;
    struct TopoBond {
        std::string a, b;
        double r0;
    };
    std::vector<TopoBond> topobonds;   // possible_bonds_ (parse.cpp:748-765)
    std::map<std::string, mafm::AtomParams> ap;
    std::vector<mafm::Overwrite> ow;
    // --- System (system.hpp:13-77); index 0 dummy, 1 tip, 2.. surface ---
    int n_atoms = 0;   // including tip and dummy
    std::vector<std::string> types;
    std::vector<double> pos;      // 3 per atom
    std::vector<double> charges;
    std::vector<int> fixed;
    double offset[3] = {0, 0, 0};
    double tip_dummy_d = 0;
    mafm::M3 cell;
    bool tip_pbc = false;
    int np[3] = {0, 0, 0};
    // --- descriptor storage ---
    std::vector<double> d_pos, d_charge;
    std::vector<int32_t> d_type;
    // flexible topology (surface-atom indices), mafm_flex_desc storage
    std::vector<int32_t> f_fixed, f_bond_atoms, f_angle_atoms, f_dihedral_atoms, f_pair_atoms;
    std::vector<double> f_bond_param, f_angle_param, f_dihedral_param, f_pair_qq;
    std::vector<mafm_pair> f_pair_vdw;
    std::vector<mafm_pair> d_pairs;
    std::vector<std::string> type_names;
    mafm_pair dummy_pair{};
    double tip_q_eff = 0, dummy_q_eff = 0;
    std::vector<double> epot;
    int epot_n[3] = {0, 0, 0};
    mafm::M3 epot_basis;
    double epot_origin[3] = {0, 0, 0};
    bool verbose = false;
};

namespace mafm {
namespace {

void pretty(const mafm_input& in, const char* fmt, ...) {
    if (!in.verbose) return;
    char buf[2048];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    fprintf(stdout, "+- %s\n", buf);
}

void warn(const mafm_input& in, const char* fmt, ...) {
    if (!in.verbose) return;
    char buf[2048];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    fprintf(stderr, "+- WARNING: %s\n", buf);
}

bool on_off(const char* keyword, const char* value) {
    if (strcmp(value, "on") == 0) return true;
    if (strcmp(value, "off") == 0) return false;
    fail(MAFM_E_PARSE, "Option %s must be either on or off!", keyword);
}

// readInputFile, parse.cpp:83-474.
void read_input(mafm_input& in) {
    FILE* fp = fopen(in.inputfile.c_str(), "r");
    if (!fp) fail(MAFM_E_IO, "The file %s does not exist!", in.inputfile.c_str());
    struct Closer { FILE* f; ~Closer() { fclose(f); } } closer{fp};
    char line[kLine], keyword[128] = "", value[128] = "", dump[kLine];
    char tmp_units[128] = "kcal/mol", tmp_normal[128] = "z", tmp_minterm[128] = "";
    while (fgets(line, kLine, fp)) {
        if (is_comment(line)) continue;
        sscanf(line, "%127s %127s", keyword, value);
        lower(keyword);
        if (!strcmp(keyword, "xyzfile")) in.xyzfile = in.inputfolder + value;
        else if (!strcmp(keyword, "paramfile")) in.paramfile = in.inputfolder + value;
        else if (!strcmp(keyword, "e_potential_file")) in.e_potential_file = in.inputfolder + value;
        else if (!strcmp(keyword, "tipatom")) in.tipatom = value;
        else if (!strcmp(keyword, "dummyatom")) in.dummyatom = value;
        else if (!strcmp(keyword, "area")) sscanf(line, "%s %lf %lf", dump, &in.area[0], &in.area[1]);
        else if (!strcmp(keyword, "center")) sscanf(line, "%s %lf %lf", dump, &in.center[0], &in.center[1]);
        else if (!strcmp(keyword, "zhigh")) in.zhigh = atof(value);
        else if (!strcmp(keyword, "zlow")) in.zlow = atof(value);
        else if (!strcmp(keyword, "dx")) in.dx = atof(value);
        else if (!strcmp(keyword, "dy")) in.dy = atof(value);
        else if (!strcmp(keyword, "dz")) in.dz = atof(value);
        else if (!strcmp(keyword, "cell_a")) sscanf(line, "%s %lf %lf %lf", dump, &in.cell_a[0], &in.cell_a[1], &in.cell_a[2]);
        else if (!strcmp(keyword, "cell_b")) sscanf(line, "%s %lf %lf %lf", dump, &in.cell_b[0], &in.cell_b[1], &in.cell_b[2]);
        else if (!strcmp(keyword, "cell_c")) sscanf(line, "%s %lf %lf %lf", dump, &in.cell_c[0], &in.cell_c[1], &in.cell_c[2]);
        else if (!strcmp(keyword, "etol")) in.etol = atof(value);
        else if (!strcmp(keyword, "ftol")) in.ftol = atof(value);
        else if (!strcmp(keyword, "dt")) in.dt = atof(value);
        else if (!strcmp(keyword, "maxsteps")) in.maxsteps = atoi(value);
        else if (!strcmp(keyword, "bufsize")) in.bufsize = atoi(value);
        else if (!strcmp(keyword, "gzip")) in.gzip = on_off(keyword, value);
        else if (!strcmp(keyword, "statistics")) in.statistics = on_off(keyword, value);
        else if (!strcmp(keyword, "flexible")) in.flexible = on_off(keyword, value);
        else if (!strcmp(keyword, "rigidgrid")) in.rigidgrid = on_off(keyword, value);
        else if (!strcmp(keyword, "coulomb")) in.coulomb = on_off(keyword, value);
        else if (!strcmp(keyword, "tip_dummy_coulomb")) in.tip_dummy_coulomb = on_off(keyword, value);
        else if (!strcmp(keyword, "use_external_potential")) in.use_external_potential = on_off(keyword, value);
        else if (!strcmp(keyword, "vdw_pbc")) in.vdw_pbc = on_off(keyword, value);
        else if (!strcmp(keyword, "surface_normal")) {
            lower(value);
            if (!strcmp(value, "z")) in.normal = NORMAL_Z;
            else if (!strcmp(value, "y")) in.normal = NORMAL_Y;
            else if (!strcmp(value, "x")) in.normal = NORMAL_X;
            else fail(MAFM_E_PARSE, "Option %s must be either X, Y or Z!", keyword);
            snprintf(tmp_normal, sizeof tmp_normal, "%s", value);
        } else if (!strcmp(keyword, "minterm")) {
            if (!strcmp(value, "e")) in.minterm = MAFM_TERM_E;
            else if (!strcmp(value, "f")) in.minterm = MAFM_TERM_F;
            else if (!strcmp(value, "ef")) in.minterm = MAFM_TERM_EF;
            else fail(MAFM_E_PARSE, "Option %s must be either e, f or ef!", keyword);
            snprintf(tmp_minterm, sizeof tmp_minterm, "%s", value);
        } else if (!strcmp(keyword, "units")) {
            const double epermv = 1.0;
            if (!strcmp(value, "kcal/mol") || !strcmp(value, "kcal")) {
                in.units = MAFM_UNITS_KCAL;
                in.qbase = 332.06371 / epermv;
            } else if (!strcmp(value, "kJ/mol") || !strcmp(value, "kJ")) {
                in.units = MAFM_UNITS_KJ;
                in.qbase = 1389.354563 / epermv;
            } else if (!strcmp(value, "eV")) {
                in.units = MAFM_UNITS_EV;
                in.qbase = 14.39964901 / epermv;
            } else {
                fail(MAFM_E_PARSE, "Option %s must be either kcal/mol (default), kJ/mol or eV!", keyword);
            }
            snprintf(tmp_units, sizeof tmp_units, "%s", value);
        } else if (!strcmp(keyword, "minimiser")) {
            if (!strcmp(value, "SD")) in.minimiser = MAFM_MIN_SD;
            else if (!strcmp(value, "FIRE")) in.minimiser = MAFM_MIN_FIRE;
            else fail(MAFM_E_PARSE, "Unrecognised minimiser type!");
        } else if (!strcmp(keyword, "integrator")) {
            if (!strcmp(value, "euler")) in.integrator = MAFM_INT_EULER;
            else if (!strcmp(value, "midpoint")) in.integrator = MAFM_INT_MIDPOINT;
            else if (!strcmp(value, "rk4")) in.integrator = MAFM_INT_RK4;
            else fail(MAFM_E_PARSE, "Unrecognised integrator type!");
        } else {
            fail(MAFM_E_PARSE, "Unknown option %s!", keyword);
        }
    }
    if (in.xyzfile.empty()) fail(MAFM_E_PARSE, "Specify at least an xyzfile!");
    if (in.paramfile.empty()) fail(MAFM_E_PARSE, "Specify at least a parameter file!");
    if (in.tipatom.empty()) fail(MAFM_E_PARSE, "Specify at least a tip atom!");
    if (in.dummyatom.empty()) fail(MAFM_E_PARSE, "Specify at least a dummy atom!");
    if (in.minterm < 0)
        fail(MAFM_E_PARSE, "Specify at least a minimization termination criterion (e, f, or ef)!");
    if (in.center[0] == -1 && in.center[1] == -1) {
        in.center[0] = in.area[0] / 2;
        in.center[1] = in.area[1] / 2;
    }
    // Sanity checks, parse.cpp:386-405.
    if (in.rigidgrid && in.flexible)
        fail(MAFM_E_PARSE, "Cannot use a flexible molecule with a static force grid!");
    if (in.coulomb && in.use_external_potential)
        fail(MAFM_E_PARSE, "Cannot use Coulomb interaction and external electrostatic potential at the same time!");
    if (in.use_external_potential && in.flexible)
        fail(MAFM_E_PARSE, "External potential can be used only for non-flexible systems!");
    if (in.use_external_potential && in.e_potential_file.empty())
        fail(MAFM_E_PARSE, "If you want to use external electrostatic potential, you must specify a file that contains it!");
    if (in.vdw_pbc && in.coulomb)
        fail(MAFM_E_PARSE, "Implementation of Coulomb interaction does not support any periodic boundary conditions! Use periodic external electrostatic potential instead.");
    auto zero3 = [](const double* v) { return v[0] == 0 && v[1] == 0 && v[2] == 0; };
    if (in.vdw_pbc && !in.use_external_potential &&
        (zero3(in.cell_a) || zero3(in.cell_b) || zero3(in.cell_c)))
        fail(MAFM_E_PARSE, "The unit cell vectors must be given if periodic vdW is used.");

    // Option echo, parse.cpp:408-472.
    auto oo = [](bool b) { return b ? "on" : "off"; };
    pretty(in, "");
    pretty(in, "Input settings for        %s:", in.inputfile.c_str());
    pretty(in, "");
    pretty(in, "xyzfile:                  %-s", in.xyzfile.c_str());
    pretty(in, "paramfile:                %-s", in.paramfile.c_str());
    pretty(in, "tipatom:                  %-s", in.tipatom.c_str());
    pretty(in, "dummyatom:                %-s", in.dummyatom.c_str());
    pretty(in, "");
    pretty(in, "units:                    %-s", tmp_units);
    pretty(in, "");
    pretty(in, "minterm:                  %-s", tmp_minterm);
    pretty(in, "etol:                     %-8.4f", in.etol);
    pretty(in, "ftol:                     %-8.4f", in.ftol);
    pretty(in, "dt:                       %-8.4f", in.dt);
    pretty(in, "maxsteps:                 %-8d", in.maxsteps);
    pretty(in, "");
    pretty(in, "area:                     %-8.4f %-8.4f", in.area[0], in.area[1]);
    pretty(in, "center:                   %-8.4f %-8.4f", in.center[0], in.center[1]);
    pretty(in, "zhigh:                    %-8.4f", in.zhigh);
    pretty(in, "zlow:                     %-8.4f", in.zlow);
    pretty(in, "dx:                       %-8.4f", in.dx);
    pretty(in, "dy:                       %-8.4f", in.dy);
    pretty(in, "dz:                       %-8.4f", in.dz);
    pretty(in, "");
    pretty(in, "surface_normal:           %-s", tmp_normal);
    pretty(in, "vdw_pbc:                  %-s", oo(in.vdw_pbc));
    if (in.vdw_pbc && !in.use_external_potential) {
        pretty(in, "cell_a:                   %-8.4f %-8.4f %-8.4f", in.cell_a[0], in.cell_a[1], in.cell_a[2]);
        pretty(in, "cell_b:                   %-8.4f %-8.4f %-8.4f", in.cell_b[0], in.cell_b[1], in.cell_b[2]);
        pretty(in, "cell_c:                   %-8.4f %-8.4f %-8.4f", in.cell_c[0], in.cell_c[1], in.cell_c[2]);
    }
    pretty(in, "");
    pretty(in, "coulomb:                  %-s", oo(in.coulomb));
    pretty(in, "tip_dummy_coulomb:        %-s", oo(in.tip_dummy_coulomb));
    pretty(in, "use_external_potential:   %-s", oo(in.use_external_potential));
    if (in.use_external_potential)
        pretty(in, "e_potential_file:         %-s", in.e_potential_file.c_str());
    pretty(in, "");
    pretty(in, "flexible:                 %-s", oo(in.flexible));
    pretty(in, "rigidgrid:                %-s", oo(in.rigidgrid));
    pretty(in, "");
    pretty(in, "minimiser:         %-s", in.minimiser == MAFM_MIN_SD ? "SD" : "FIRE");
    static const char* integ[] = {"euler", "midpoint", "rk4"};
    pretty(in, "integrator:        %-s", integ[in.integrator]);
    pretty(in, "");
    pretty(in, "bufsize:           %-8d", in.bufsize);
    pretty(in, "gzip:              %-s", oo(in.gzip));
    pretty(in, "statistics:        %-s", oo(in.statistics));
    pretty(in, "");
}

// readXYZFile, parse.cpp:477-585.
void read_xyz(mafm_input& in) {
    FILE* fp = fopen(in.xyzfile.c_str(), "r");
    if (!fp) fail(MAFM_E_IO, "No such file: %s!", in.xyzfile.c_str());
    struct Closer { FILE* f; ~Closer() { fclose(f); } } closer{fp};
    char line[kLine], value[128] = "";
    int n = 0;
    bool firstline = true, realxyz = false;
    while (fgets(line, kLine, fp)) {
        if (is_comment(line)) continue;
        if (firstline) {
            sscanf(line, "%127s", value);
            if (is_int(value)) {
                n = atoi(value);
                realxyz = true;
                break;
            }
            firstline = false;
        }
        if (!firstline) n++;
    }
    rewind(fp);
    if (n < 0) fail(MAFM_E_PARSE, "Invalid number of atoms in the xyz file.");
    in.n_atoms = n + 2;
    in.types.assign(in.n_atoms, "");
    in.pos.assign(3 * (size_t)in.n_atoms, 0.0);
    in.charges.assign(in.n_atoms, 0.0);
    in.fixed.assign(in.n_atoms, 0);
    in.fixed[0] = 1;
    in.fixed[1] = 0;
    in.types[0] = in.dummyatom;
    in.types[1] = in.tipatom;
    int atom_i = 2, skipped = 0, ncols = 0;
    firstline = true;
    while (fgets(line, kLine, fp)) {
        if (realxyz && skipped < 2) {
            skipped++;
            continue;
        }
        if (is_comment(line)) continue;
        if (firstline) {
            ncols = count_columns(line);
            firstline = false;
        }
        char type[64] = "";
        double x = 0, y = 0, z = 0, q = 0;
        int fx = 0;
        if (ncols == 4) sscanf(line, "%63s %lf %lf %lf", type, &x, &y, &z);
        else if (ncols == 5) sscanf(line, "%63s %lf %lf %lf %lf", type, &x, &y, &z, &q);
        else if (ncols == 6) sscanf(line, "%63s %lf %lf %lf %lf %d", type, &x, &y, &z, &q, &fx);
        else fail(MAFM_E_PARSE, "Invalid number of columns in the xyz file.");
        if (atom_i >= in.n_atoms)
            fail(MAFM_E_PARSE, "More atoms in the xyz file than given on its first line.");
        in.types[atom_i] = type;
        in.pos[3 * atom_i] = x;
        in.pos[3 * atom_i + 1] = y;
        in.pos[3 * atom_i + 2] = z;
        in.charges[atom_i] = q;
        in.fixed[atom_i] = in.flexible ? fx : 1;
        atom_i++;
    }
    double check = 0;
    for (int i = 0; i < in.n_atoms; ++i) check += in.charges[i] * in.charges[i];
    if (fabs(check) < kTolerance) {
        in.xyz_charges = false;
        warn(in, "The RMSQ-error for the charges read from the XYZ-file is zero.\n"
                 "+-     Charges will be read from the parameter file.\n"
                 "+-     If you want zero charge, set the charge in the parameter file to zero.\n"
                 "+-");
    } else {
        in.xyz_charges = true;
    }
}

// readFlexibleParameters, parse.cpp:699-782.
void read_flexible(mafm_input& in, FILE* fp) {
    char line[kLine], keyword[128] = "", dump[128];
    bool b = false, a = false, d = false, s = false;
    while (fgets(line, kLine, fp)) {
        if (is_comment(line)) continue;
        sscanf(line, "%127s", keyword);
        if (!strcmp(keyword, "bond")) {
            if (b) warn(in, "Parameters for harmonic bond defined multiple times!");
            sscanf(line, "%127s %lf", dump, &in.bond_k);
            b = true;
        }
        if (!strcmp(keyword, "angle")) {
            if (a) warn(in, "Parameters for harmonic angle defined multiple times!");
            sscanf(line, "%127s %lf", dump, &in.angle_k);
            a = true;
        }
        if (!strcmp(keyword, "dihedral")) {
            if (d) warn(in, "Parameters for harmonic dihedral defined multiple times!");
            sscanf(line, "%127s %lf", dump, &in.dihedral_k);
            d = true;
        }
        if (!strcmp(keyword, "substrate")) {
            if (s) warn(in, "Parameters for substrate support defined multiple times!");
            sscanf(line, "%127s %lf %lf %lf %lf %lf", dump, &in.sub_eps, &in.sub_sig,
                   &in.sub_lambda, &in.sub_rc, &in.sub_k);
            s = true;
        }
        if (!strcmp(keyword, "topobond")) {
            char a1[128] = "", a2[128] = "";
            double r0 = 0;
            sscanf(line, "%127s %127s %127s %lf", dump, a1, a2, &r0);
            bool twice = false;
            for (const auto& tb : in.topobonds)
                if (multiset_eq(tb.a, tb.b, a1, a2)) twice = true;
            if (twice) warn(in, "The topobond for %s and %s is defined at least twice!", a1, a2);
            in.topobonds.push_back({a1, a2, r0});
        }
    }
    if (!b) fail(MAFM_E_PARSE, "No harmonic bond parameters found in parameter file!");
    if (!a) fail(MAFM_E_PARSE, "No harmonic angle parameters found in parameter file!");
    if (!d) fail(MAFM_E_PARSE, "No harmonic dihedral parameters found in parameter file!");
    if (!s) fail(MAFM_E_PARSE, "No harmonic substrate support parameters found in parameter file!");
}

// readParameterFile, parse.cpp:588-697.
void read_params(mafm_input& in) {
    FILE* fp = fopen(in.paramfile.c_str(), "r");
    if (!fp) fail(MAFM_E_IO, "No parameter file %s found!", in.paramfile.c_str());
    struct Closer { FILE* f; ~Closer() { fclose(f); } } closer{fp};
    char line[kLine], keyword[128] = "", dump[kLine], atom[64] = "", a1[64] = "", a2[64] = "",
         style[128] = "";
    double eps = 0, sig = 0, mass = 0, q = 0, de = 0, alpha = 0, re = 0;
    bool hcheck = false;
    while (fgets(line, kLine, fp)) {
        if (is_comment(line)) continue;
        sscanf(line, "%127s", keyword);
        if (!strcmp(keyword, "atom")) {
            sscanf(line, "%127s %63s %lf %lf %lf %lf", dump, atom, &eps, &sig, &mass, &q);
            if (in.ap.count(atom)) warn(in, "Parameters for atom type %s defined multiple times.", atom);
            AtomParams& p = in.ap[atom];
            p.eps = eps;
            p.sig = sig;
            p.q = q;
            p.mass = mass;
            if (in.dummyatom == atom) in.charges[0] = q;
            if (in.tipatom == atom) in.charges[1] = q;
        } else if (!strcmp(keyword, "harm")) {
            if (hcheck) fail(MAFM_E_PARSE, "Parameters for harmonic spring can only be specified once!");
            sscanf(line, "%127s %lf %lf", dump, &in.harm_k, &in.harm_r0);
            hcheck = true;
        } else if (!strcmp(keyword, "pair_ovwrt")) {
            sscanf(line, "%127s %63s %63s %127s", dump, a1, a2, style);
            int ncols = count_columns(line);
            if (!strcmp(style, "lj")) {
                if (ncols != 4 + 2) fail(MAFM_E_PARSE, "Only two parameters (eps, sig) allowed for LJ");
                sscanf(line, "%127s %127s %127s %127s %lf %lf", dump, dump, dump, dump, &eps, &sig);
                Overwrite o;
                o.a = a1; o.b = a2; o.eps = eps; o.sig = sig; o.morse = false;
                in.ow.push_back(o);
            } else if (!strcmp(style, "morse")) {
                if (ncols != 4 + 3) fail(MAFM_E_PARSE, "Only three parameters (De, a, re) allowed for Morse");
                sscanf(line, "%127s %127s %127s %127s %lf %lf %lf", dump, dump, dump, dump, &de, &alpha, &re);
                Overwrite o;
                o.a = a1; o.b = a2; o.de = de; o.alpha = alpha; o.re = re; o.morse = true;
                in.ow.push_back(o);
            } else {
                fail(MAFM_E_PARSE, "Unknown pair style overwrite '%s'", style);
            }
        }
    }
    if (!hcheck) fail(MAFM_E_PARSE, "No harmonic spring parameters found in parameter file!");
    if (in.flexible) {
        rewind(fp);
        read_flexible(in, fp);
    }
}

// Gaussian cube, CubeReader::readMetadata + readVolumetricData (cube_io.cpp:10-139).
struct Cube {
    int n[3] = {0, 0, 0};
    double voxel[3][3] = {{0}};   // voxel[i] = vector i (Angstrom)
    double origin[3] = {0, 0, 0};
    std::vector<double> values;
};

Cube read_cube(const std::string& path, bool with_values) {
    FILE* fp = fopen(path.c_str(), "r");
    if (!fp) fail(MAFM_E_IO, "Could not read metadata from the cube file. Check the format of the file.");
    std::string text;
    {
        char buf[1 << 16];
        size_t k;
        while ((k = fread(buf, 1, sizeof buf, fp)) > 0) text.append(buf, k);
        fclose(fp);
    }
    const char* p = text.c_str();
    for (int l = 0; l < 2; ++l) {
        const char* nl = strchr(p, '\n');
        if (!nl) fail(MAFM_E_PARSE, "Could not read metadata from the cube file. Check the format of the file.");
        p = nl + 1;
    }
    auto next_d = [&](double& v) {
        char* e;
        v = strtod(p, &e);
        if (e == p) fail(MAFM_E_PARSE, "Could not read metadata from the cube file. Check the format of the file.");
        p = e;
    };
    auto next_i = [&](int& v) {
        char* e;
        long x = strtol(p, &e, 10);
        if (e == p) fail(MAFM_E_PARSE, "Could not read metadata from the cube file. Check the format of the file.");
        v = (int)x;
        p = e;
    };
    Cube c;
    int natoms;
    next_i(natoms);
    for (int d = 0; d < 3; ++d) next_d(c.origin[d]);
    for (int v = 0; v < 3; ++v) {
        next_i(c.n[v]);
        for (int d = 0; d < 3; ++d) next_d(c.voxel[v][d]);
    }
    if (c.n[0] < 0) {
        for (int v = 0; v < 3; ++v) c.n[v] = -c.n[v];
    } else {
        for (int v = 0; v < 3; ++v)
            for (int d = 0; d < 3; ++d) c.voxel[v][d] *= kBohr;
        for (int d = 0; d < 3; ++d) c.origin[d] *= kBohr;
    }
    if (natoms < 0 || c.n[0] <= 0 || c.n[1] <= 0 || c.n[2] <= 0)
        fail(MAFM_E_PARSE, "Could not read metadata from the cube file. Check the format of the file.");
    for (int a = 0; a < natoms; ++a) {
        int z;
        double t;
        next_i(z);
        for (int k = 0; k < 4; ++k) next_d(t);
    }
    if (with_values) {
        const size_t total = (size_t)c.n[0] * c.n[1] * c.n[2];
        c.values.resize(total);
        for (size_t i = 0; i < total; ++i) {
            char* e;
            double v = strtod(p, &e);
            if (e == p)
                fail(MAFM_E_PARSE, "Could not read the volumetric data from the cube file. Check the format of the file.");
            c.values[i] = v;
            p = e;
        }
    }
    return c;
}

// System::rotateCoordAxes, system.cpp:68-90 (positions only).
void rotate_positions(mafm_input& in, const char* seq) {
    for (int a = 0; a < in.n_atoms; ++a) {
        double x = in.pos[3 * a], y = in.pos[3 * a + 1], z = in.pos[3 * a + 2];
        if (!strcmp(seq, "ZXY")) {
            in.pos[3 * a] = z; in.pos[3 * a + 1] = x; in.pos[3 * a + 2] = y;
        } else {
            in.pos[3 * a] = y; in.pos[3 * a + 1] = z; in.pos[3 * a + 2] = x;
        }
    }
}

// LJ or Morse parameters of a pair, Simulation::addVDWInteraction (simulation.cpp:238-267).
mafm_pair resolve_vdw(const mafm_input& in, const std::string& t1, const std::string& t2) {
    mafm_pair p{};
    for (const Overwrite& o : in.ow) {
        if (multiset_eq(o.a, o.b, t1, t2)) {
            if (o.morse) {
                p.kind = MAFM_PAIR_MORSE;
                p.p[0] = o.de; p.p[1] = o.alpha; p.p[2] = o.re;
            } else {
                p.kind = MAFM_PAIR_LJ;
                p.p[0] = 4 * o.eps * pow(o.sig, 6);
                p.p[1] = 4 * o.eps * pow(o.sig, 12);
            }
            return p;
        }
    }
    auto i1 = in.ap.find(t1), i2 = in.ap.find(t2);
    if (i1 == in.ap.end()) fail(MAFM_E_PARSE, "Parameters for atom type %s not found in parameter file!", t1.c_str());
    if (i2 == in.ap.end()) fail(MAFM_E_PARSE, "Parameters for atom type %s not found in parameter file!", t2.c_str());
    double m_eps = sqrt(i1->second.eps * i2->second.eps);
    double m_sig = (i1->second.sig + i2->second.sig) / 2;
    p.kind = MAFM_PAIR_LJ;
    p.p[0] = 4 * m_eps * pow(m_sig, 6);
    p.p[1] = 4 * m_eps * pow(m_sig, 12);
    return p;
}

// Charge of atom i for a Coulomb term, Simulation::addCoulombInteraction (simulation.cpp:269-289).
double coulomb_charge(const mafm_input& in, int i) {
    if (in.xyz_charges) return in.charges[i];
    auto it = in.ap.find(in.types[i]);
    if (it == in.ap.end())
        fail(MAFM_E_PARSE, "Parameters for atom type %s not found in parameter file!", in.types[i].c_str());
    return it->second.q;
}

// Simulation::buildSurfaceSurfaceInteractions (simulation.cpp:557-693) for a
// flexible molecule, with the reference's vector arithmetic (vectors.hpp:99-125):
// bonds between atoms closer than 1.1 r0 of a topobond (r0 of the spring = the
// distance), angles between bonds sharing an atom, dihedrals between angles
// (the reference's five patterns, each improper centre once), and van der
// Waals (+ Coulomb) pairs between atoms of different bonded fragments.
// "Connected" is the reference's breadth-first search to a depth of the atom
// count, i.e. the same bonded fragment.  Indices stored are surface indices.
void build_topology(mafm_input& in) {
    const int n = in.n_atoms;
    auto sub = [&](int a, int b, double r[3]) {
        for (int d = 0; d < 3; ++d) r[d] = in.pos[3 * (size_t)a + d] - in.pos[3 * (size_t)b + d];
    };
    auto len = [](const double r[3]) { return sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]); };
    auto dot = [](const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
    auto cross = [](const double a[3], const double b[3], double r[3]) {
        r[0] = a[1] * b[2] - a[2] * b[1];
        r[1] = a[2] * b[0] - a[0] * b[2];
        r[2] = a[0] * b[1] - a[1] * b[0];
    };
    auto normalized = [&](const double a[3], double r[3]) {
        const double l = len(a);
        for (int d = 0; d < 3; ++d) r[d] = l > 1e-10 ? a[d] / l : 0.0;
    };
    in.f_fixed.assign(in.fixed.begin() + 2, in.fixed.end());
    in.f_bond_atoms.clear(); in.f_bond_param.clear();
    in.f_angle_atoms.clear(); in.f_angle_param.clear();
    in.f_dihedral_atoms.clear(); in.f_dihedral_param.clear();
    in.f_pair_atoms.clear(); in.f_pair_vdw.clear(); in.f_pair_qq.clear();
    // bonds, and the bonded fragments (union-find)
    std::vector<int> root(n);
    for (int i = 0; i < n; ++i) root[i] = i;
    std::function<int(int)> find = [&](int x) { return root[x] == x ? x : (root[x] = find(root[x])); };
    std::vector<std::pair<int, int>> bonds;
    for (int i = 2; i < n; ++i)
        for (int j = i + 1; j < n; ++j) {
            double r0 = 0;
            for (const auto& tb : in.topobonds)
                if (multiset_eq(tb.a, tb.b, in.types[i], in.types[j])) r0 = tb.r0;
            double r[3];
            sub(i, j, r);
            const double atom_d = len(r);
            if (atom_d < 1.1 * r0) {
                bonds.emplace_back(i, j);
                root[find(i)] = find(j);
                in.f_bond_atoms.insert(in.f_bond_atoms.end(), {i - 2, j - 2});
                in.f_bond_param.insert(in.f_bond_param.end(), {in.bond_k, atom_d});
            }
        }
    // angles
    std::vector<std::array<int, 3>> angles;
    for (size_t bi = 0; bi < bonds.size(); ++bi)
        for (size_t bj = bi + 1; bj < bonds.size(); ++bj) {
            const auto b1 = bonds[bi], b2 = bonds[bj];
            int shared = -1, a1 = 0, a2 = 0;
            if (b1.first == b2.first) { shared = b1.first; a1 = b1.second; a2 = b2.second; }
            else if (b1.first == b2.second) { shared = b1.first; a1 = b1.second; a2 = b2.first; }
            else if (b1.second == b2.first) { shared = b1.second; a1 = b1.first; a2 = b2.second; }
            else if (b1.second == b2.second) { shared = b1.second; a1 = b1.first; a2 = b2.first; }
            if (shared == -1) continue;
            angles.push_back({shared, a1, a2});
            double d1[3], d2[3], n1[3], n2[3];
            sub(a1, shared, d1);
            sub(a2, shared, d2);
            normalized(d1, n1);
            normalized(d2, n2);
            const double theta0 = acos(dot(n1, n2));
            in.f_angle_atoms.insert(in.f_angle_atoms.end(), {shared - 2, a1 - 2, a2 - 2});
            in.f_angle_param.insert(in.f_angle_param.end(), {in.angle_k, theta0});
        }
    // dihedrals
    std::vector<int> improper;
    for (size_t ai = 0; ai < angles.size(); ++ai)
        for (size_t aj = ai + 1; aj < angles.size(); ++aj) {
            const auto& g1 = angles[ai];
            const auto& g2 = angles[aj];
            int t1 = -1, t2 = -1, t3 = -1, t4 = -1;
            if (g1[0] == g2[0] && std::find(improper.begin(), improper.end(), g1[0]) == improper.end()) {
                improper.push_back(g1[0]);
                t1 = g1[0]; t2 = g1[1]; t3 = g1[2];
                t4 = (g2[1] == g1[1] || g2[1] == g1[2]) ? g2[2] : g2[1];
            } else if (g1[1] == g2[0] && g2[1] == g1[0]) {
                t1 = g1[2]; t2 = g1[0]; t3 = g2[0]; t4 = g2[2];
            } else if (g1[2] == g2[0] && g2[1] == g1[0]) {
                t1 = g1[1]; t2 = g1[0]; t3 = g2[0]; t4 = g2[2];
            } else if (g1[1] == g2[0] && g2[2] == g1[0]) {
                t1 = g1[2]; t2 = g1[0]; t3 = g2[0]; t4 = g2[1];
            } else if (g1[2] == g2[0] && g2[2] == g1[0]) {
                t1 = g1[1]; t2 = g1[0]; t3 = g2[0]; t4 = g2[1];
            }
            if (t1 == -1) continue;
            double d12[3], d23[3], d43[3], m[3], nn[3];
            sub(t1, t2, d12);
            sub(t2, t3, d23);
            sub(t4, t3, d43);
            cross(d12, d23, m);
            cross(d43, d23, nn);
            const double tan_s = dot(nn, d12) * len(d23) / (dot(m, nn));
            const double sigma0 = atan(tan_s);
            in.f_dihedral_atoms.insert(in.f_dihedral_atoms.end(), {t1 - 2, t2 - 2, t3 - 2, t4 - 2});
            in.f_dihedral_param.insert(in.f_dihedral_param.end(), {in.dihedral_k, sigma0});
        }
    // non-bonded pairs between fragments: addVDWInteraction, addCoulombInteraction
    for (int i = 2; i < n; ++i)
        for (int j = i + 1; j < n; ++j) {
            if (find(i) == find(j)) continue;
            in.f_pair_atoms.insert(in.f_pair_atoms.end(), {i - 2, j - 2});
            in.f_pair_vdw.push_back(resolve_vdw(in, in.types[i], in.types[j]));
            double qq = 0;
            if (in.coulomb) {
                const double q1 = coulomb_charge(in, i), q2 = coulomb_charge(in, j);
                if (q1 != 0 && q2 != 0) qq = in.qbase * q1 * q2;
            }
            in.f_pair_qq.push_back(qq);
        }
}

// Simulation::initialize and the parameter part of buildInteractions.
void prepare(mafm_input& in) {
    in.np[0] = (int)(floor(in.area[0] / in.dx) + 1);
    in.np[1] = (int)(floor(in.area[1] / in.dy) + 1);
    in.np[2] = (int)(floor((in.zhigh - in.zlow) / in.dz) + 1);
    if (in.normal == NORMAL_X) rotate_positions(in, "YZX");
    else if (in.normal == NORMAL_Y) rotate_positions(in, "ZXY");
    if (in.vdw_pbc) {
        double cv[3][3];
        if (in.use_external_potential) {
            Cube c = read_cube(in.e_potential_file, false);
            for (int v = 0; v < 3; ++v)
                for (int d = 0; d < 3; ++d) cv[v][d] = c.n[v] * c.voxel[v][d];
        } else {
            for (int d = 0; d < 3; ++d) {
                cv[0][d] = in.cell_a[d]; cv[1][d] = in.cell_b[d]; cv[2][d] = in.cell_c[d];
            }
        }
        for (int v = 0; v < 3; ++v)
            for (int d = 0; d < 3; ++d) in.cell.v[d][v] = cv[v][d];
        in.tip_pbc = true;
    }
    // System::centerMolecule (system.cpp:119-136)
    double avgx = 0.0, avgy = 0.0;
    for (int i = 2; i < in.n_atoms; ++i) {
        avgx += in.pos[3 * i];
        avgy += in.pos[3 * i + 1];
    }
    avgx /= in.n_atoms - 2;
    avgy /= in.n_atoms - 2;
    double ddx = in.center[0] - avgx, ddy = in.center[1] - avgy;
    for (int i = 2; i < in.n_atoms; ++i) {
        in.pos[3 * i] += ddx;
        in.pos[3 * i + 1] += ddy;
    }
    in.offset[0] = ddx;
    in.offset[1] = ddy;
    // System::setMoleculeZ (system.cpp:103-116)
    double min_z = 10e10;
    for (int i = 2; i < in.n_atoms; ++i)
        if (in.pos[3 * i + 2] < min_z && in.types[i] != "H") min_z = in.pos[3 * i + 2];
    for (int i = 2; i < in.n_atoms; ++i) in.pos[3 * i + 2] -= min_z;
    in.offset[2] = -min_z;
    // Simulation::calculateTipDummyDistance (simulation.cpp:218-225)
    auto dm = in.ap.find(in.types[0]), tp = in.ap.find(in.types[1]);
    if (dm == in.ap.end()) fail(MAFM_E_PARSE, "Parameters for atom type %s not found in parameter file!", in.types[0].c_str());
    if (tp == in.ap.end()) fail(MAFM_E_PARSE, "Parameters for atom type %s not found in parameter file!", in.types[1].c_str());
    in.tip_dummy_d = (dm->second.sig + tp->second.sig) / 2 * kSixthRoot2;

    // Surface atoms: type table in order of first appearance, tip pair per type.
    std::map<std::string, int> index;
    const int ns = in.n_atoms - 2;
    in.d_pos.assign(3 * (size_t)ns, 0.0);
    in.d_charge.assign(ns, 0.0);
    in.d_type.assign(ns, 0);
    in.type_names.clear();
    in.d_pairs.clear();
    for (int i = 2; i < in.n_atoms; ++i) {
        auto it = index.find(in.types[i]);
        int t;
        if (it == index.end()) {
            t = (int)in.type_names.size();
            index[in.types[i]] = t;
            in.type_names.push_back(in.types[i]);
            in.d_pairs.push_back(resolve_vdw(in, in.types[1], in.types[i]));
        } else {
            t = it->second;
        }
        in.d_type[i - 2] = t;
        for (int d = 0; d < 3; ++d) in.d_pos[3 * (i - 2) + d] = in.pos[3 * i + d];
    }
    // Charges.  Whether read from the xyz file or looked up by type, the tip's
    // and the dummy's charges are System::charges_[1] and [0]: the parameter
    // file's line for their type sets both (parse.cpp:626-631).  The lookups
    // still run where the reference runs them, for its error messages.
    in.tip_q_eff = in.charges[1];
    in.dummy_q_eff = in.charges[0];
    if (in.coulomb && !in.vdw_pbc) {
        (void)coulomb_charge(in, 1);
        for (int i = 2; i < in.n_atoms; ++i) in.d_charge[i - 2] = coulomb_charge(in, i);
    }
    in.dummy_pair = resolve_vdw(in, in.types[0], in.types[1]);
    if (in.tip_dummy_coulomb) {
        (void)coulomb_charge(in, 0);
        (void)coulomb_charge(in, 1);
    }
    if (in.use_external_potential) {
        // The field's tip charge is System::charges_[1] as well (simulation.cpp:415).
        Cube c = read_cube(in.e_potential_file, true);
        double scale = in.units == MAFM_UNITS_EV ? -kHartreeEV
                     : in.units == MAFM_UNITS_KJ ? -kHartreeKJ : -kHartreeKcal;
        for (double& v : c.values) v *= scale;
        M3 basis;
        for (int v = 0; v < 3; ++v)
            for (int d = 0; d < 3; ++d) basis.v[d][v] = c.voxel[v][d];
        double origin[3] = {c.origin[0], c.origin[1], c.origin[2]};
        int n[3] = {c.n[0], c.n[1], c.n[2]};
        if (in.normal == NORMAL_X) {
            // The reference asks DataGrid::rotateCoordAxes for "ZYX", which it
            // rejects (simulation.cpp:358-359, data_grid.cpp:92-94).
            fail(MAFM_E_PARSE, "The coordinate sequence for rotateCoordAxes must be either ZXY or YZX.");
        } else if (in.normal == NORMAL_Y) {
            // DataGrid::rotateCoordAxes("ZXY"), data_grid.cpp:40-69
            int nn[3] = {n[2], n[0], n[1]};
            M3 S;
            S.v[2][0] = 1; S.v[0][1] = 1; S.v[1][2] = 1;
            basis = S.transpose().mul(basis.mul(S));
            double no[3] = {origin[2], origin[0], origin[1]};
            std::vector<double> nv(c.values.size());
            for (int ix = 0; ix < nn[0]; ix++)
                for (int iy = 0; iy < nn[1]; iy++)
                    for (int iz = 0; iz < nn[2]; iz++)
                        nv[((size_t)ix * nn[1] + iy) * nn[2] + iz] =
                            c.values[((size_t)iy * n[1] + iz) * n[2] + ix];
            c.values.swap(nv);
            for (int d = 0; d < 3; ++d) { n[d] = nn[d]; origin[d] = no[d]; }
        }
        for (int d = 0; d < 3; ++d) in.epot_origin[d] = origin[d] + in.offset[d];
        for (int d = 0; d < 3; ++d) in.epot_n[d] = n[d];
        in.epot_basis = basis;
        in.epot.swap(c.values);
    }
    if (in.flexible) build_topology(in);
}

}  // namespace

// ----- output (writeOutput, simulation.cpp:145-199) -------------------------

namespace {

// Longest "%W.Pf" of a double (309 integer digits, sign, point, decimals).
constexpr int kFieldMax = 340;

// printf("%W.Pf", x) for the writer's fields, without printf: glibc prints
// the exact binary value rounded to P decimals (to nearest, ties to even),
// so the value is taken apart (x = m 2^e, m < 2^53) and m 10^P 2^e is rounded
// in 128-bit integer arithmetic.  A negative value that rounds to zero keeps
// its sign ("-0.000"), as printf does.  Values that are not finite or not
// below 1e12 in magnitude go to snprintf.
char* put_fixed(char* o, double x, int width, int prec) {
    static const uint64_t kPow10[] = {1, 10, 100, 1000, 10000, 100000, 1000000};
    if (!(std::fabs(x) < 1e12) || prec > 6) return o + snprintf(o, kFieldMax, "%*.*f", width, prec, x);
    uint64_t bits;
    std::memcpy(&bits, &x, sizeof bits);
    const bool neg = (bits >> 63) != 0;
    const int bexp = (int)((bits >> 52) & 0x7ff);
    uint64_t m = bits & ((1ull << 52) - 1);
    int e;
    if (bexp == 0) {
        e = -1074;
    } else {
        m |= 1ull << 52;
        e = bexp - 1075;
    }
    const unsigned __int128 N = (unsigned __int128)m * kPow10[prec];   // < 2^73
    uint64_t q;
    if (e >= 0) {
        q = (uint64_t)(N << e);
    } else if (-e >= 100) {
        q = 0;   // m 10^P 2^e < 2^73 / 2^100: below one half
    } else {
        const int sh = -e;
        unsigned __int128 qq = N >> sh;
        const unsigned __int128 rem = N - (qq << sh);
        const unsigned __int128 half = (unsigned __int128)1 << (sh - 1);
        if (rem > half || (rem == half && (qq & 1))) ++qq;
        q = (uint64_t)qq;
    }
    char dig[32];
    int n = 0;
    do {
        dig[n++] = (char)('0' + q % 10);
        q /= 10;
    } while (q);
    while (n <= prec) dig[n++] = '0';   // one integer digit at least
    const int len = n + (prec > 0 ? 1 : 0) + (neg ? 1 : 0);
    for (int s = len; s < width; ++s) *o++ = ' ';
    if (neg) *o++ = '-';
    for (int d = n - 1; d >= prec; --d) *o++ = dig[d];
    if (prec > 0) {
        *o++ = '.';
        for (int d = prec - 1; d >= 0; --d) *o++ = dig[d];
    }
    return o;
}

// printf("%d", v)
char* put_int(char* o, long long v) {
    char dig[24];
    int n = 0;
    unsigned long long u = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
    do {
        dig[n++] = (char)('0' + u % 10);
        u /= 10;
    } while (u);
    if (v < 0) *o++ = '-';
    while (n) *o++ = dig[--n];
    return o;
}

// Rows of height k for pixel columns [cb, ce) (c = i ny + j), in column
// order; pts holds column c's points at (c - cb) nz + k.
void write_rows(const mafm_input& in, const mafm_point* pts, int k, long long cb, long long ce,
                FILE* f) {
    const int ny = in.np[1], nz = in.np[2];
    // Dummy z after k calls of lowerTip (system.hpp:51-54).
    double dz_acc = in.zhigh;
    for (int s = 0; s < k; ++s) dz_acc -= in.dz;
    const bool wrap = in.tip_pbc && !in.rigidgrid;
    const M3 inv = in.cell.inverse();
    std::string buf;
    buf.reserve((size_t)ny * 120);
    char row[16 * kFieldMax];
    for (long long c0 = cb; c0 < ce;) {
        // one x row (or the part of it inside the range) per buffer
        const long long c1 = std::min(ce, (c0 / ny + 1) * ny);
        buf.clear();
        for (long long c = c0; c < c1; ++c) {
            const int i = (int)(c / ny), j = (int)(c % ny);
            const mafm_point& p = pts[(size_t)(c - cb) * nz + k];
            const double x = i * in.dx, y = j * in.dy;
            double dxy[2] = {x, y};
            if (wrap) {
                // System::setDummyXY with periodic boundaries (system.cpp:139-162)
                double t[3] = {x - in.offset[0], y - in.offset[1], 0 - in.offset[2]};
                double cn[3];
                for (int r = 0; r < 3; ++r)
                    cn[r] = inv.v[r][0] * t[0] + inv.v[r][1] * t[1] + inv.v[r][2] * t[2];
                cn[0] -= floor(cn[0]);
                cn[1] -= floor(cn[1]);
                for (int r = 0; r < 2; ++r)
                    dxy[r] = in.cell.v[r][0] * cn[0] + in.cell.v[r][1] * cn[1] +
                             in.cell.v[r][2] * cn[2] + in.offset[r];
            }
            const double rx = p.tip[0] - dxy[0], ry = p.tip[1] - dxy[1], rz = p.tip[2] - dz_acc;
            const double r = sqrt(rx * rx + ry * ry + rz * rz);
            const double angle = atan2(sqrt(rx * rx + ry * ry), rz) * (180.0 / kPi);
            // "%d %d %d %6.3f %6.3f %6.3f %8.4f %8.4f %8.4f %6.3f %6.3f %6.3f %6.3f %8.4f %8.4f %d\n"
            char* o = row;
            o = put_int(o, k); *o++ = ' ';
            o = put_int(o, i); *o++ = ' ';
            o = put_int(o, j); *o++ = ' ';
            const double f3[3] = {x, y, dz_acc};
            for (double v : f3) { o = put_fixed(o, v, 6, 3); *o++ = ' '; }
            for (int c = 0; c < 3; ++c) { o = put_fixed(o, p.force[c], 8, 4); *o++ = ' '; }
            const double g4[4] = {rx, ry, rz, r};
            for (double v : g4) { o = put_fixed(o, v, 6, 3); *o++ = ' '; }
            o = put_fixed(o, angle, 8, 4); *o++ = ' ';
            o = put_fixed(o, p.energy, 8, 4); *o++ = ' ';
            o = put_int(o, p.steps);
            *o++ = '\n';
            buf.append(row, (size_t)(o - row));
        }
        fwrite(buf.data(), 1, buf.size(), f);
        c0 = c1;
    }
}

}  // namespace
}  // namespace mafm

// ----- C ABI ------------------------------------------------------------------

extern "C" {

const char* mafm_last_error(void) { return mafm::g_last_error.c_str(); }

int mafm_abi_version(void) { return MAFM_ABI_VERSION; }

int mafm_input_load(const char* input_file, int verbose, mafm_input** out) {
    return mafm::guarded([&] {
        if (!input_file || !out) mafm::fail(MAFM_E_INVALID, "null argument");
        *out = nullptr;
        auto* in = new mafm_input();
        try {
            in->verbose = verbose != 0;
            in->inputfile = input_file;
            size_t split = in->inputfile.rfind('/');
            if (split != std::string::npos) in->inputfolder = in->inputfile.substr(0, split + 1);
            mafm::read_input(*in);
            mafm::read_xyz(*in);
            mafm::read_params(*in);
            mafm::prepare(*in);
        } catch (...) {
            delete in;
            throw;
        }
        *out = in;
    });
}

int mafm_input_desc(const mafm_input* in, mafm_scan_desc* d) {
    return mafm::guarded([&] {
        if (!in || !d) mafm::fail(MAFM_E_INVALID, "null argument");
        *d = mafm_scan_desc{};
        d->flexible = in->flexible;
        d->n_atoms = in->n_atoms - 2;
        d->n_types = (int32_t)in->type_names.size();
        d->pos = in->d_pos.data();
        d->charge = in->d_charge.data();
        d->type = in->d_type.data();
        d->tip_pair = in->d_pairs.data();
        d->dummy_pair = in->dummy_pair;
        d->tip_charge = in->tip_q_eff;
        d->dummy_charge = in->dummy_q_eff;
        d->qbase = in->qbase;
        d->coulomb = in->coulomb && !in->vdw_pbc;
        d->tip_dummy_coulomb = in->tip_dummy_coulomb;
        d->harm_k = in->harm_k;
        d->harm_r0 = in->harm_r0;
        d->tip_dummy_d = in->tip_dummy_d;
        d->vdw_pbc = in->vdw_pbc;
        d->tip_pbc = in->tip_pbc;
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) d->cell[3 * r + c] = in->cell.v[r][c];
        for (int k = 0; k < 3; ++k) d->offset[k] = in->offset[k];
        d->nx = in->np[0];
        d->ny = in->np[1];
        d->nz = in->np[2];
        d->dx = in->dx;
        d->dy = in->dy;
        d->dz = in->dz;
        d->zhigh = in->zhigh;
        d->zlow = in->zlow;
        d->area[0] = in->area[0];
        d->area[1] = in->area[1];
        d->minimiser = in->minimiser;
        d->integrator = in->integrator;
        d->minterm = in->minterm;
        d->maxsteps = in->maxsteps;
        d->etol = in->etol;
        d->ftol = in->ftol;
        d->dt = in->dt;
        d->rigidgrid = in->rigidgrid;
        d->use_external_potential = in->use_external_potential;
        if (in->use_external_potential) {
            d->epot = in->epot.data();
            for (int k = 0; k < 3; ++k) d->epot_n[k] = in->epot_n[k];
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) d->epot_basis[3 * r + c] = in->epot_basis.v[r][c];
            for (int k = 0; k < 3; ++k) d->epot_origin[k] = in->epot_origin[k];
        }
    });
}

int mafm_input_flex_desc(const mafm_input* in, mafm_flex_desc* f) {
    return mafm::guarded([&] {
        if (!in || !f) mafm::fail(MAFM_E_INVALID, "null argument");
        if (!in->flexible) mafm::fail(MAFM_E_INVALID, "the input is not a flexible molecule");
        *f = mafm_flex_desc{};
        f->fixed = in->f_fixed.data();
        f->n_bonds = (int32_t)in->f_bond_param.size() / 2;
        f->bond_atoms = in->f_bond_atoms.data();
        f->bond_param = in->f_bond_param.data();
        f->n_angles = (int32_t)in->f_angle_param.size() / 2;
        f->angle_atoms = in->f_angle_atoms.data();
        f->angle_param = in->f_angle_param.data();
        f->n_dihedrals = (int32_t)in->f_dihedral_param.size() / 2;
        f->dihedral_atoms = in->f_dihedral_atoms.data();
        f->dihedral_param = in->f_dihedral_param.data();
        f->n_pairs = (int32_t)in->f_pair_qq.size();
        f->pair_atoms = in->f_pair_atoms.data();
        f->pair_vdw = in->f_pair_vdw.data();
        f->pair_qq = in->f_pair_qq.data();
        f->substrate[0] = in->sub_eps;
        f->substrate[1] = in->sub_sig;
        f->substrate[2] = in->sub_lambda;
        f->substrate[3] = in->sub_rc;
        f->substrate[4] = in->sub_k;
    });
}

int mafm_input_output_opts(const mafm_input* in, int32_t* gzip, int32_t* statistics,
                           int32_t* bufsize) {
    return mafm::guarded([&] {
        if (!in) mafm::fail(MAFM_E_INVALID, "null argument");
        if (gzip) *gzip = in->gzip;
        if (statistics) *statistics = in->statistics;
        if (bufsize) *bufsize = in->bufsize;
    });
}

int mafm_input_free(mafm_input* in) {
    delete in;
    return MAFM_OK;
}

// A scan's output files opened for appending rows in column order: each
// scan-%06.3f.dat[.gz] file holds the rows of one height in pixel order
// (simulation.cpp:145-199), so appending the columns of consecutive chunks
// writes the same bytes as one call with every point.
struct mafm_writer {
    const mafm_input* in = nullptr;
    bool gzip = false;
    long long next_col = 0;
    std::vector<FILE*> files;
    void close_files() {
        for (FILE*& f : files) {
            if (!f) continue;
            if (gzip) pclose(f);
            else fclose(f);
            f = nullptr;
        }
    }
};

int mafm_writer_open(const mafm_input* in, const char* folder, int32_t gzip, mafm_writer** out) {
    return mafm::guarded([&] {
        if (!in || !folder || !out) mafm::fail(MAFM_E_INVALID, "null argument");
        *out = nullptr;
        auto* w = new mafm_writer();
        w->in = in;
        w->gzip = gzip != 0;
        const int nz = in->np[2];
        w->files.assign(nz, nullptr);
        char name[1024];
        for (int k = 0; k < nz; ++k) {
            const double z = in->zhigh - k * in->dz;
            if (gzip) {
                snprintf(name, sizeof name, "gzip -6 > %sscan-%06.3f.dat.gz", folder, z);
                w->files[k] = popen(name, "w");
            } else {
                snprintf(name, sizeof name, "%sscan-%06.3f.dat", folder, z);
                w->files[k] = fopen(name, "w");
            }
            if (!w->files[k]) {
                w->close_files();
                delete w;
                mafm::fail(MAFM_E_IO, "cannot open %s", name);
            }
        }
        *out = w;
    });
}

int mafm_writer_append(mafm_writer* w, const mafm_point* pts, int32_t col_begin, int32_t col_end) {
    return mafm::guarded([&] {
        if (!w || (!pts && col_end > col_begin)) mafm::fail(MAFM_E_INVALID, "null argument");
        const long long n_cols = (long long)w->in->np[0] * w->in->np[1];
        if (col_begin != w->next_col || col_end < col_begin || col_end > n_cols)
            mafm::fail(MAFM_E_INVALID, "columns [%d, %d) do not continue the %lld written",
                       col_begin, col_end, w->next_col);
        const int nz = w->in->np[2];
        // the height files are independent: formatted and written in parallel
#pragma omp parallel for schedule(dynamic, 1)
        for (int k = 0; k < nz; ++k)
            mafm::write_rows(*w->in, pts, k, col_begin, col_end, w->files[k]);
        w->next_col = col_end;
    });
}

int mafm_writer_close(mafm_writer* w) {
    if (!w) return MAFM_OK;
    w->close_files();
    delete w;
    return MAFM_OK;
}

int mafm_write_output(const mafm_input* in, const mafm_point* pts, const char* folder,
                      int32_t gzip) {
    mafm_writer* w = nullptr;
    int st = mafm_writer_open(in, folder, gzip, &w);
    if (st != MAFM_OK) return st;
    st = mafm_writer_append(w, pts, 0, in->np[0] * in->np[1]);
    mafm_writer_close(w);
    return st;
}

int mafm_write_states(const mafm_input* in, const double* states, int32_t column,
                      const char* folder) {
    return mafm::guarded([&] {
        if (!in || !states || !folder) mafm::fail(MAFM_E_INVALID, "null argument");
        const int nx = in->np[0], ny = in->np[1], nz = in->np[2], na = in->n_atoms;
        if (column < 0 || column >= nx * ny) mafm::fail(MAFM_E_INVALID, "column %d outside the scan", column);
        const double x = (column / ny) * in->dx, y = (column % ny) * in->dy;
        double z = in->zhigh;
        for (int k = 0; k < nz; ++k) {
            char name[1024];
            snprintf(name, sizeof name, "%sstate_%.1f-%.1f-%.1f.xyz", folder, x, y, z);
            FILE* fp = fopen(name, "w");
            if (!fp) mafm::fail(MAFM_E_IO, "cannot open %s", name);
            fprintf(fp, "%d\n\n", na);
            for (int a = 0; a < na; ++a) {
                const double* p = states + ((size_t)k * na + a) * 3;
                fprintf(fp, "%s %8.4f %8.4f %8.4f\n", in->types[a].c_str(), p[0], p[1], p[2]);
            }
            fclose(fp);
            printf("+- Wrote %s\n", name);
            z -= in->dz;
        }
    });
}

int mafm_write_statistics(const mafm_input* in, const char* folder, uint64_t total_steps,
                          double wall_s, double total_s) {
    return mafm::guarded([&] {
        if (!in || !folder) mafm::fail(MAFM_E_INVALID, "null argument");
        std::string path = std::string(folder) + "statistics.txt";
        FILE* fp = fopen(path.c_str(), "w");
        if (!fp) mafm::fail(MAFM_E_IO, "cannot open %s", path.c_str());
        const int n_points = in->np[0] * in->np[1] * in->np[2];
        fprintf(fp, "Simulation run finished\n");
        fprintf(fp, "Statistics:\n");
        fprintf(fp, "    Computed %d tip positions\n", n_points);
        fprintf(fp, "    Needed %ld minimization steps in total\n", (long)total_steps);
        fprintf(fp, "    Which means approximately %.2f minimization steps per tip position\n",
                ((double)total_steps / n_points));
        fprintf(fp, "    The simulation wall time is %.2f seconds\n", wall_s);
        fprintf(fp, "    The entire simulation took %.2f seconds\n", total_s);
        fclose(fp);
    });
}

}  // extern "C"
