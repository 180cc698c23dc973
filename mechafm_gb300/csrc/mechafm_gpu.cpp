// mechafm_gpu.cpp — `mechafm-gpu INPUT-FILE [OUTPUT-FOLDER]`, a drop-in for the
// reference's `mechafm-omp` (src/mechafm.cpp:209-233) on one GPU.
//
// Same arguments, input/xyz/parameter/cube files, stdout banners and option
// echo, error messages and exit status, scan-%06.3f.dat[.gz] files and
// statistics.txt.  The relaxation runs through libmafm's C ABI.  By default
// it runs the double-float kernel, whose points take the reference's FP64
// steps and agree with its positions and forces to about 1e-10 (a rigid grid
// is built in double-float too); MAFM_PRECISION=fp64 / df / fp32c selects the
// plain FP64 kernel (the reference's bits), the double-float kernel or the
// faster FP32-compensated kernel.  A flexible molecule runs the FP64 flexible kernel and writes the
// middle pixel's state_*.xyz files like the reference.  MAFM_DEVICE picks the
// GPU (default 0).
//
// The scan runs in ten chunks of pixel rows (the reference's ten progress
// lines).  While the GPU relaxes a chunk, this thread formats and writes the
// previous one (mafm_writer_append; gzip runs in its own processes), so the
// text output, which takes longer than the relaxation at GPU speed, overlaps
// it; the files are byte-identical to writing every point at the end.
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <future>
#include <string>
#include <vector>

#include "mafm.h"

namespace {

void pretty(const char* fmt, ...) {
    char buf[2048];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    fprintf(stdout, "+- %s\n", buf);
}

[[noreturn]] void error(const char* msg) {
    // messages.cpp:12-27 of the reference
    fprintf(stderr, "+- ERROR (on process %d): %s\n", 0, msg);
    exit(1);
}

void check(int code) {
    if (code != MAFM_OK) error(mafm_last_error());
}

}  // namespace

int main(int argc, char* argv[]) {
    // parseCommandLine (parse.cpp:30-80)
    fprintf(stdout, "+ - - - - - - - - - - - - - - - - - - - - - - - - - - - - - - +\n");
    fprintf(stdout, "|                   Mechanical AFM Model                      |\n");
    fprintf(stdout, "|  Based on: P. Hapala et al, Phys. Rev. B, 90:085421 (2014)  |\n");
    fprintf(stdout, "|                  This implementation by                     |\n");
    fprintf(stdout, "|             Peter Spijker and Olli Keisanen                 |\n");
    fprintf(stdout, "|          2014-2015 (c) Aalto University, Finland            |\n");
    fprintf(stdout, "+ - - - - - - - - - - - - - - - - - - - - - - - - - - - - - - +\n");
    if (argc < 2) error("Specify an input file to be read!");
    if (argc > 3) error("Too many command line arguments!");
    std::string outdir;
    if (argc == 3) {
        outdir = argv[2];
        if (outdir.empty() || outdir.back() != '/') outdir += '/';
        std::string cmd = "mkdir -p " + outdir;
        if (system(cmd.c_str()) != 0) error(("cannot create " + outdir).c_str());
    }
    const char* prec_env = getenv("MAFM_PRECISION");
    const char* dev_env = getenv("MAFM_DEVICE");
    const int device = dev_env ? atoi(dev_env) : 0;

    mafm_input* in = nullptr;
    check(mafm_input_load(argv[1], 1, &in));
    mafm_scan_desc d;
    check(mafm_input_desc(in, &d));
    int32_t gzip = 0, statistics = 0, bufsize = 0;
    check(mafm_input_output_opts(in, &gzip, &statistics, &bufsize));
    int precision = MAFM_DF;
    if (prec_env && !strcmp(prec_env, "fp64")) precision = MAFM_FP64;
    if (prec_env && !strcmp(prec_env, "fp32c")) precision = MAFM_FP32C;

    // openUniverse (mechafm.cpp:37-80)
    const int n_total = d.nx * d.ny * d.nz;
    pretty("3D data grid is: %d x %d x %d (%d in total)", d.nx, d.ny, d.nz, n_total);
    const auto t_start = std::chrono::system_clock::now();

    // Simulation::initialize / buildInteractions messages (simulation.cpp:324,416,443,500)
    if (d.use_external_potential)
        pretty("Calculating energy and force on grid from external electrostatic potential.");
    mafm_scan* scan = nullptr;
    mafm_flex* flex = nullptr;
    if (d.flexible) {
        // flexible molecule: every atom relaxes (FP64 flexible kernel)
        mafm_flex_desc fd;
        check(mafm_input_flex_desc(in, &fd));
        check(mafm_flex_create(device, &d, &fd, &flex));
    } else {
        check(mafm_scan_create(device, &d, &scan));
    }
    if (d.use_external_potential) pretty("Done!");
    if (d.rigidgrid) {
        int32_t n[3];
        double basis[9], origin[3];
        check(mafm_scan_grid_info(scan, 0, n, basis, origin));
        pretty("Computing 3D force grid: %d, %d, %d (%d grid points)", n[0], n[1], n[2],
               n[0] * n[1] * n[2]);
        pretty("Done!");
    }

    // Simulation::run (simulation.cpp:67-143): the x rows in ten chunks; after
    // each, the reference's progress test (simulation.cpp:132-137: the float
    // fraction of pixels done against thresholds stepped by 0.1 in double),
    // so the same ten lines are printed whatever the number of rows.
    pretty("Starting simulation");
    const double report_interval = 0.1;
    double next_report = report_interval;
    auto report = [&](int pixels_done) {
        const double progress = 1.0f * pixels_done / (d.nx * d.ny);
        while (progress >= next_report) {
            pretty("Finished %4.1f %% of the simulation", 100 * next_report);
            next_report += report_interval;
        }
    };
    uint64_t total_steps = 0;
    const int chunks = 10;
    // flexible molecules: the middle pixel's states (simulation.cpp:114-116)
    const int state_col = (d.nx * d.ny) / 2;
    struct Chunk {
        int cb = 0, ce = 0;
        std::vector<mafm_point> pts;
        std::vector<double> states;
        bool with_states = false;
        uint64_t steps = 0;
    };
    // relax chunk c into ch (on a worker thread; only the GPU and ch are touched)
    auto relax = [&](int c, Chunk* ch) {
        const int i0 = (int)((long long)d.nx * c / chunks), i1 = (int)((long long)d.nx * (c + 1) / chunks);
        ch->cb = i0 * d.ny;
        ch->ce = i1 * d.ny;
        ch->pts.resize((size_t)(ch->ce - ch->cb) * d.nz);
        mafm_run_stats st{};
        if (ch->ce > ch->cb) {
            if (flex) {
                ch->with_states = state_col >= ch->cb && state_col < ch->ce;
                if (ch->with_states) ch->states.resize((size_t)d.nz * (d.n_atoms + 2) * 3);
                check(mafm_flex_run(flex, ch->cb, ch->ce, ch->pts.data(), &st, state_col,
                                    ch->with_states ? ch->states.data() : nullptr, nullptr));
            } else {
                mafm_run_opts o{};
                o.precision = precision;
                o.col_begin = ch->cb;
                o.col_end = ch->ce;
                check(mafm_run(scan, &o, ch->pts.data(), &st, nullptr));
            }
        }
        ch->steps = st.total_steps;
    };
    mafm_writer* writer = nullptr;
    check(mafm_writer_open(in, outdir.c_str(), gzip, &writer));
    Chunk buf[2];
    std::future<void> pending = std::async(std::launch::async, relax, 0, &buf[0]);
    for (int c = 0; c < chunks; ++c) {
        pending.get();
        Chunk& ch = buf[c % 2];
        if (c + 1 < chunks) pending = std::async(std::launch::async, relax, c + 1, &buf[(c + 1) % 2]);
        if (ch.ce <= ch.cb) continue;
        if (ch.with_states) check(mafm_write_states(in, ch.states.data(), state_col, outdir.c_str()));
        total_steps += ch.steps;
        report(ch.ce);
        check(mafm_writer_append(writer, ch.pts.data(), ch.cb, ch.ce));
    }
    check(mafm_writer_close(writer));
    if (scan) check(mafm_scan_destroy(scan));
    if (flex) check(mafm_flex_destroy(flex));

    // finalize (mechafm.cpp:103-154)
    const auto t_end = std::chrono::system_clock::now();
    const double secs = std::chrono::duration<double>(t_end - t_start).count();
    pretty("Simulation run finished");
    pretty("Statistics:");
    pretty("    Computed %d tip positions", n_total);
    pretty("    Needed %ld minimization steps in total", (long)total_steps);
    pretty("    Which means approximately %.2f minimization steps per tip position",
           (double)total_steps / n_total);
    pretty("    The simulation wall time is %.2f seconds", secs);
    pretty("    The entire simulation took %.2f seconds", secs);
    pretty("");
    if (statistics) check(mafm_write_statistics(in, outdir.c_str(), total_steps, secs, secs));
    // closeParallelUniverse (mechafm.cpp:183-207)
    pretty("How many x,y points did each process handle:");
    pretty("    Process %2d: %6d x,y points", 0, d.nx * d.ny);
    mafm_input_free(in);
    return 0;
}
