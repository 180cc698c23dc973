// ref_dump.cpp — test-infrastructure driver that links the reference's own,
// unmodified MechAFM sources (compiled out of tree by oracle/Makefile) and
// dumps full-precision results for golden fixtures.
//
// This file is part of the ORACLE, not of the product: only the fixture
// generator under tests/golden/ runs it.  It replaces the reference's
// src/mechafm.cpp main() (mechafm.cpp:209-233) with a driver that
//   * sizes the scan exactly like openUniverse (mechafm.cpp:47-49),
//   * runs the per-pixel loop body of Simulation::run (simulation.cpp:93-122)
//     over an optional pixel sub-range, and
//   * writes every output record with all 17 significant digits (the CLI
//     rounds to 3-4 decimals, simulation.cpp:180-195).
//
// Modes
//   ref_dump scan   INPUT OUT.bin [i0 i1 j0 j1]   per-point records (25 doubles)
//   ref_dump states INPUT OUT.bin i j              every atom after each height of column (i, j)
//   ref_dump system INPUT OUT.txt                 prepared System after initialize()
//   ref_dump sample_ts INPUT POINTS.bin OUT.bin   tip-surface F,E at given tip positions
//   ref_dump sample_es INPUT POINTS.bin OUT.bin   external-field F,E at given tip positions
//   ref_dump time   INPUT                          full scan timed, OpenMP over columns
//   ref_dump time_cols INPUT COLS.bin              the listed columns (int32 i*ny + j) timed
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "globals.hpp"
#include "interactions.hpp"
#include "minimiser.hpp"
#include "parse.hpp"
#include "simulation.hpp"
#include "system.hpp"

namespace {

void setup(Simulation& sim, const char* input) {
    // Single-process universe, as openParallelUniverse does without MPI
    // (mechafm.cpp:165-178).
    sim.root_process_ = 0;
    sim.current_process_ = 0;
    sim.n_processes_ = 1;
    sim.points_per_process_.assign(1, 0);
    char prog[] = "ref_dump";
    std::string in(input);
    std::vector<char> inbuf(in.begin(), in.end());
    inbuf.push_back('\0');
    char* argv[] = {prog, inbuf.data(), nullptr};
    parseCommandLine(2, argv, sim);
    readInputFile(sim);
    readXYZFile(sim);
    readParameterFile(sim);
    // Scan sizing of openUniverse (mechafm.cpp:47-49).
    InputOptions& o = sim.options_;
    sim.n_total_ = 0;
    sim.n_points_.x = floor(o.area.x / o.dx) + 1;
    sim.n_points_.y = floor(o.area.y / o.dy) + 1;
    sim.n_points_.z = floor((o.zhigh - o.zlow) / o.dz) + 1;
    sim.initialize();
}

// One pixel column: the loop body of Simulation::run (simulation.cpp:93-122).
void column(const Simulation& sim, int i, int j, double* rec) {
    const InputOptions& o = sim.options_;
    System s = sim.system;
    if (o.rigidgrid) s.setTipPbc(false);
    s.setDummyXY(i * o.dx, j * o.dy);
    s.setDummyZ(o.zhigh);
    for (int k = 0; k < sim.n_points_.z; ++k) {
        int n = 0;
        if (o.minimiser_type == STEEPEST_DESCENT) n = SDMinimisation(s, o);
        else n = FIREMinimisation(s, o);
        OutputData d = s.getOutput();
        double* r = rec + (size_t)k * 25;
        r[0] = i; r[1] = j; r[2] = k; r[3] = n;
        r[4] = s.positions_[1].x; r[5] = s.positions_[1].y; r[6] = s.positions_[1].z;
        r[7] = s.positions_[0].x; r[8] = s.positions_[0].y; r[9] = s.positions_[0].z;
        r[10] = d.position.x; r[11] = d.position.y; r[12] = d.position.z;
        r[13] = d.tip_force.x; r[14] = d.tip_force.y; r[15] = d.tip_force.z;
        r[16] = d.tip_energy;
        r[17] = d.r_vec.x; r[18] = d.r_vec.y; r[19] = d.r_vec.z;
        r[20] = d.r; r[21] = d.angle;
        r[22] = s.velocities_[1].x; r[23] = s.velocities_[1].y; r[24] = s.velocities_[1].z;
        s.lowerTip(o.dz);
    }
}

std::vector<double> read_points(const char* path) {
    FILE* f = fopen(path, "rb");
    if (!f) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
    std::vector<double> v;
    double buf[3];
    while (fread(buf, sizeof(double), 3, f) == 3) v.insert(v.end(), buf, buf + 3);
    fclose(f);
    return v;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: ref_dump MODE INPUT [...]\n");
        return 2;
    }
    std::string mode = argv[1];
    Simulation sim;
    setup(sim, argv[2]);
    const Vec3i np = sim.n_points_;

    if (mode == "scan") {
        if (argc < 4) return 2;
        int i0 = 0, i1 = np.x, j0 = 0, j1 = np.y;
        if (argc >= 8) {
            i0 = atoi(argv[4]); i1 = atoi(argv[5]); j0 = atoi(argv[6]); j1 = atoi(argv[7]);
        }
        const int ni = i1 - i0, nj = j1 - j0;
        std::vector<double> out((size_t)ni * nj * np.z * 25);
#pragma omp parallel for schedule(dynamic, 1) collapse(2)
        for (int i = i0; i < i1; ++i)
            for (int j = j0; j < j1; ++j)
                column(sim, i, j, out.data() + ((size_t)(i - i0) * nj + (j - j0)) * np.z * 25);
        FILE* f = fopen(argv[3], "wb");
        fwrite(out.data(), sizeof(double), out.size(), f);
        fclose(f);
        return 0;
    }
    if (mode == "states") {
        // every atom's position after each height of column (i, j)
        if (argc < 6) return 2;
        const int i = atoi(argv[4]), j = atoi(argv[5]);
        const InputOptions& o = sim.options_;
        System s = sim.system;
        if (o.rigidgrid) s.setTipPbc(false);
        s.setDummyXY(i * o.dx, j * o.dy);
        s.setDummyZ(o.zhigh);
        std::vector<double> out;
        for (int k = 0; k < np.z; ++k) {
            if (o.minimiser_type == STEEPEST_DESCENT) SDMinimisation(s, o);
            else FIREMinimisation(s, o);
            for (int a = 0; a < s.n_atoms_; ++a) {
                out.push_back(s.positions_[a].x);
                out.push_back(s.positions_[a].y);
                out.push_back(s.positions_[a].z);
            }
            s.lowerTip(o.dz);
        }
        FILE* f = fopen(argv[3], "wb");
        fwrite(out.data(), sizeof(double), out.size(), f);
        fclose(f);
        return 0;
    }
    if (mode == "system") {
        FILE* f = fopen(argv[3], "w");
        const System& s = sim.system;
        fprintf(f, "n_points %d %d %d\n", np.x, np.y, np.z);
        fprintf(f, "tip_dummy_d %.17g\n", sim.system.getTipDummyDistance());
        Vec3d off = sim.system.getOffset();
        fprintf(f, "offset %.17g %.17g %.17g\n", off.x, off.y, off.z);
        fprintf(f, "xyz_charges %d\n", (int)sim.options_.xyz_charges);
        fprintf(f, "qbase %.17g\n", sim.interaction_parameters_.qbase);
        fprintf(f, "n_interactions %zu\n", sim.interactions_.size());
        fprintf(f, "n_atoms %d\n", s.n_atoms_);
        for (int a = 0; a < s.n_atoms_; ++a)
            fprintf(f, "atom %s %.17g %.17g %.17g %.17g %d\n", s.types_[a].c_str(),
                    s.positions_[a].x, s.positions_[a].y, s.positions_[a].z,
                    s.charges_[a], s.fixed_[a]);
        fclose(f);
        return 0;
    }
    if (mode == "sample_ts" || mode == "sample_es") {
        if (argc < 5) return 2;
        std::vector<double> pts = read_points(argv[3]);
        const size_t n = pts.size() / 3;
        std::vector<double> out(n * 4);
        const bool es_only = mode == "sample_es";
        for (size_t p = 0; p < n; ++p) {
            std::vector<Vec3d> pos = sim.system.positions_;
            pos[1] = Vec3d(pts[3 * p], pts[3 * p + 1], pts[3 * p + 2]);
            std::vector<Vec3d> forces(pos.size(), Vec3d(0));
            std::vector<double> energies(pos.size(), 0);
            for (const auto& it : sim.interactions_) {
                if (!it->isTipSurface()) continue;
                if (es_only && dynamic_cast<ElectrostaticPotentialInteraction*>(it.get()) == nullptr)
                    continue;
                it->eval(pos, forces, energies);
            }
            out[4 * p] = forces[1].x; out[4 * p + 1] = forces[1].y;
            out[4 * p + 2] = forces[1].z; out[4 * p + 3] = energies[1];
        }
        FILE* f = fopen(argv[4], "wb");
        fwrite(out.data(), sizeof(double), out.size(), f);
        fclose(f);
        return 0;
    }
    if (mode == "time") {
        std::vector<double> rec((size_t)np.z * 25);
        unsigned long steps = 0;
        auto t0 = std::chrono::steady_clock::now();
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : steps)
        for (int i = 0; i < np.x; ++i) {
            std::vector<double> r((size_t)np.z * 25);
            for (int j = 0; j < np.y; ++j) {
                column(sim, i, j, r.data());
                for (int k = 0; k < np.z; ++k) steps += (unsigned long)r[(size_t)k * 25 + 3];
            }
        }
        double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        printf("points %d wall_s %.4f steps %lu\n", np.x * np.y * np.z, dt, steps);
        return 0;
    }
    if (mode == "time_cols") {
        if (argc < 4) return 2;
        std::vector<int> cols;
        FILE* f = fopen(argv[3], "rb");
        if (!f) return 2;
        int c;
        while (fread(&c, sizeof c, 1, f) == 1) cols.push_back(c);
        fclose(f);
        for (int col : cols)
            if (col < 0 || col >= np.x * np.y) return 2;
        unsigned long steps = 0;
        auto t0 = std::chrono::steady_clock::now();
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : steps)
        for (size_t m = 0; m < cols.size(); ++m) {
            std::vector<double> r((size_t)np.z * 25);
            column(sim, cols[m] / np.y, cols[m] % np.y, r.data());
            for (int k = 0; k < np.z; ++k) steps += (unsigned long)r[(size_t)k * 25 + 3];
        }
        double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        printf("points %zu wall_s %.4f steps %lu\n", cols.size() * (size_t)np.z, dt, steps);
        return 0;
    }
    fprintf(stderr, "unknown mode %s\n", mode.c_str());
    return 2;
}
