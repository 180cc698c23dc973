/*
 * mafm.h — C ABI of libmafm, the GB300 (sm_103a) implementation of the
 * MechAFM scan hot path.
 *
 * The reference (SINGROUP/MechAFM) has no library interface: its scan runs
 * inside one process (`mechafm-omp INPUT [OUTPUT]`, src/mechafm.cpp:209-233).
 * Its in-process seams are
 *   int FIREMinimisation(System&, const InputOptions&)        src/minimiser.hpp:23
 *   int SDMinimisation(System&, const InputOptions&)          src/minimiser.hpp:20
 *   void Interaction::eval(positions, forces, energies)       src/interactions.hpp:72
 * called per pixel from Simulation::run (src/simulation.cpp:67-143).  They
 * are too fine-grained for a GPU, so this ABI cuts one level higher: "relax
 * every pixel column of a scan".  Each entry point below names the reference
 * code it replaces.
 *
 * Conventions
 *   - Every function returns int status, 0 (MAFM_OK) on success.  No C++
 *     exception crosses this boundary.  mafm_last_error() gives the message
 *     of the last failure on the calling thread; for input-file errors it is
 *     the reference's own error() text (src/messages.cpp:12-27).
 *   - Plain pointers and sizes only.  Buffers passed in are owned by the
 *     caller; the library copies what it keeps.
 *   - Units are the reference's: Angstrom, energy unit chosen by `units`,
 *     charges in e.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 */
#ifndef MAFM_H
#define MAFM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MAFM_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------- */
enum {
    MAFM_OK = 0,
    MAFM_E_INVALID = 1,     /* bad argument or descriptor */
    MAFM_E_IO = 2,          /* file missing or unreadable */
    MAFM_E_PARSE = 3,       /* input/xyz/parameter/cube file error (reference error()) */
    MAFM_E_CUDA = 4,        /* CUDA runtime or launch failure */
    MAFM_E_NOMEM = 5,       /* device or host allocation failed */
    MAFM_E_RANGE = 6,       /* a size beyond a documented limit */
    MAFM_E_DEVICE = 7,      /* device-side error word set (bounded wait expired) */
    MAFM_E_UNSUPPORTED = 8  /* option combination not implemented on the GPU */
};

/* ---- enumerations mirroring the reference ------------------------------- */
enum { MAFM_MIN_SD = 0, MAFM_MIN_FIRE = 1 };                 /* minimiser.hpp:10-13 */
enum { MAFM_INT_EULER = 0, MAFM_INT_MIDPOINT = 1, MAFM_INT_RK4 = 2 }; /* integrators.hpp:4-8 */
enum { MAFM_TERM_E = 0, MAFM_TERM_F = 1, MAFM_TERM_EF = 2 };  /* simulation.hpp:21 */
enum { MAFM_PAIR_LJ = 0, MAFM_PAIR_MORSE = 1 };               /* interactions.hpp:79-119 */
enum { MAFM_UNITS_KCAL = 0, MAFM_UNITS_KJ = 1, MAFM_UNITS_EV = 2 }; /* simulation.hpp:27 */

/* Arithmetic of a run. */
enum {
    MAFM_FP64 = 0,   /* plain FP64, the reference's operation order */
    MAFM_FP32C = 1,  /* FP32 pair math, compensated sums, double-float tip
                        positions and energies: the fastest path; FIRE's
                        discrete decisions can differ from FP64's on near-ties
                        (about 0.07 % of the points of a 60-atom cluster scan
                        end more than 1e-3 A from the FP64 result) */
    MAFM_DF = 2      /* double-float: every pair term, sum, position, velocity
                        and FIRE quantity as an unevaluated sum of two FP32
                        numbers (48-bit significand) on the FP32 pipes, so FIRE
                        takes FP64's decisions; a column in which a decision
                        still came within the double-float error margin of its
                        threshold is re-relaxed in FP64 (MAFM_PT_FP64).  A
                        rigid grid is built in double-float too; the FP64
                        re-relaxation reads its FP64 copy (the grid's nodes
                        then agree with an FP64 build to about 1e-14, not bit
                        for bit) */
};

/* Per-point status bits (mafm_point.status). */
enum {
    MAFM_PT_MAXSTEPS = 1,   /* minimiser returned maxsteps without converging */
    MAFM_PT_NONFINITE = 2,  /* a force or energy was NaN/Inf */
    MAFM_PT_OUTSIDE = 4,    /* rigid grid lookup clamped at the border
                               (reference warns, force_grid.cpp:181-217) */
    MAFM_PT_NEAR_TIE = 8,   /* MAFM_DF: at this or an earlier height of the
                               column a FIRE decision (convergence test, sign of
                               P; minimiser.cpp:15-37, 107-124) lay within the
                               double-float error margin of its threshold */
    MAFM_PT_FP64 = 16       /* MAFM_DF: the column was then re-relaxed in FP64
                               from its first height: the point holds the plain
                               FP64 kernel's bits */
};

/* One tip–atom van der Waals pair.  LJ: p = {es6, es12, 0} with
 * es6 = 4 eps sig^6 and es12 = 4 eps sig^12 (simulation.cpp:245-246,263-264).
 * Morse: p = {De, a, re} (interactions.cpp:29-40). */
typedef struct mafm_pair {
    int32_t kind;
    int32_t reserved;
    double p[3];
} mafm_pair;

/*
 * Everything one scan needs, after the reference's host-side preparation
 * (Simulation::initialize, simulation.cpp:31-65): parsed options, surface
 * atoms centred and shifted (system.cpp:103-136), tip–dummy distance
 * (simulation.cpp:218-225), pair parameters mixed and overwritten
 * (simulation.cpp:227-267).  mafm_input_desc() fills one from input files.
 */
typedef struct mafm_scan_desc {
    /* surface atoms (System index 2.. in the reference) */
    int32_t n_atoms;
    int32_t n_types;
    const double* pos;          /* [n_atoms*3] x,y,z */
    const double* charge;       /* [n_atoms] Coulomb charge (xyz or parameter file,
                                   parse.cpp:571-584 and simulation.cpp:273-289) */
    const int32_t* type;        /* [n_atoms] index into tip_pair */
    const mafm_pair* tip_pair;  /* [n_types] tip–type pair */
    mafm_pair dummy_pair;       /* dummy–tip pair (buildTipDummyInteractions) */
    double tip_charge;
    double dummy_charge;
    double qbase;               /* Coulomb prefactor of the unit system (parse.cpp:278-298) */
    int32_t coulomb;            /* tip–surface Coulomb (off under vdw_pbc) */
    int32_t tip_dummy_coulomb;
    double harm_k;              /* TipHarmonicInteraction k, r0 (interactions.cpp:252-266) */
    double harm_r0;
    double tip_dummy_d;         /* initial dummy–tip z distance */
    /* periodicity (simulation.cpp:39-59, 297-312; system.cpp:139-162) */
    int32_t vdw_pbc;            /* sum 3x3 in-plane images of every atom */
    int32_t tip_pbc;            /* wrap pixel xy into the cell (setDummyXY) */
    double cell[9];             /* row-major; columns are the cell vectors */
    double offset[3];           /* System offset of the centring / z shift */
    /* scan geometry (mechafm.cpp:47-49, simulation.cpp:78-122) */
    int32_t nx, ny, nz;
    int32_t flexible;           /* 1: the surface atoms move (flexible on); such a
                                   scan runs through mafm_flex_* with its topology */
    double dx, dy, dz;
    double zhigh, zlow;
    double area[2];
    /* minimiser (simulation.hpp:50-59) */
    int32_t minimiser;
    int32_t integrator;
    int32_t minterm;
    int32_t maxsteps;
    double etol, ftol, dt;
    /* rigid force grid (simulation.cpp:420-501) */
    int32_t rigidgrid;
    /* external Hartree field (simulation.cpp:322-417), values already scaled to
       the energy unit and the origin already shifted by the System offset */
    int32_t use_external_potential;
    const double* epot;         /* [n0*n1*n2], index (i*n1 + j)*n2 + k */
    int32_t epot_n[3];
    int32_t reserved1;
    double epot_basis[9];       /* row-major; columns are the voxel vectors */
    double epot_origin[3];
} mafm_scan_desc;

/* One relaxed pixel·z point.  Point index p = (i*ny + j)*nz + k for pixel
 * (i, j) and height k, as OutputData.indices (simulation.cpp:117-119). */
typedef struct mafm_point {
    double tip[3];      /* relaxed tip position, System::positions_[1] */
    double force[3];    /* tip–surface force at the relaxed position (system.cpp:41-51) */
    double energy;      /* tip–surface energy */
    int32_t steps;      /* value returned by the minimiser (minimiser.cpp:79-80,128) */
    int32_t status;     /* MAFM_PT_* bits */
} mafm_point;

typedef struct mafm_run_opts {
    int32_t precision;          /* MAFM_FP64, MAFM_FP32C or MAFM_DF */
    int32_t lanes_per_column;   /* FP32C: 1,2,4,8,16,32 lanes share a column; 0 = default
                                   (from the column count; mafm_autotune measures).
                                   MAFM_DF: 1,2,4,8 lanes share a column's terms; 0 =
                                   default */
    int32_t block_threads;      /* 0 = default (256) */
    int32_t columns_per_tile;   /* FP32C: columns a warp takes from the shared queue at a
                                   time; 0 = default (1 for a large single scan, else one
                                   or four per group) */
    int32_t col_begin;          /* relax only columns [col_begin, col_end) of */
    int32_t col_end;            /*   i*ny + j; 0,0 = all */
} mafm_run_opts;

typedef struct mafm_run_stats {
    uint64_t total_steps;       /* sum of mafm_point.steps (statistics.txt, mechafm.cpp:140-152) */
    uint64_t force_evals;       /* tip force evaluations, output evaluations included */
    uint64_t pair_evals;        /* tip–atom pair terms evaluated (vdW + Coulomb) */
    uint32_t error_word;        /* OR of MAFM_PT_* over all points, plus device error bits */
    uint32_t fp64_columns;      /* MAFM_DF: columns re-relaxed in FP64 */
    double kernel_ms;           /* device time of the relax kernel(s) */
} mafm_run_stats;

typedef struct mafm_input mafm_input;   /* parsed input files + prepared System */
typedef struct mafm_scan mafm_scan;     /* device-resident scan */
typedef struct mafm_plan mafm_plan;     /* prepared batched launch */

/* ---- errors / version ---------------------------------------------------- */
const char* mafm_last_error(void);
int mafm_abi_version(void);

/* ---- input front-end (host) ---------------------------------------------
 * Replaces readInputFile / readXYZFile / readParameterFile (parse.cpp:83-782,
 * src/parse.hpp:5-10), CubeReader (cube_io.cpp:10-139) and the host part of
 * Simulation::initialize (simulation.cpp:31-65).  verbose != 0 prints the
 * reference's banner, option echo and warnings (parse.cpp:32-38,407-472). */
int mafm_input_load(const char* input_file, int verbose, mafm_input** out);
/* Fill a descriptor whose pointers refer to storage owned by `in`. */
int mafm_input_desc(const mafm_input* in, mafm_scan_desc* out);

/* ---- flexible molecules ------------------------------------------------------
 * With `flexible on` every surface atom whose xyz "fixed" column is not 1
 * moves (parse.cpp:559-563), held by the topology Simulation::
 * buildSurfaceSurfaceInteractions and buildSubstrateInteractions build
 * (simulation.cpp:516-693): harmonic bonds between atoms closer than 1.1 r0
 * of a `topobond`, angles between bonds sharing an atom, dihedrals between
 * angles, van der Waals (+ Coulomb) pairs between atoms not connected by
 * bonds, a substrate wall on every atom and an XY tether on atoms with
 * fixed = 2.  Atom indices below are surface-atom indices (0-based, the
 * reference's System index - 2); every list is in the reference's
 * interaction order, which is the order forces are summed per atom. */
typedef struct mafm_flex_desc {
    const int32_t* fixed;           /* [n_atoms] 0 free, 1 fixed, 2 XY-tethered */
    int32_t n_bonds;                /* HarmonicInteraction (interactions.cpp:298-309) */
    const int32_t* bond_atoms;      /* [n_bonds*2] i, j */
    const double* bond_param;       /* [n_bonds*2] k, r0 */
    int32_t n_angles;               /* HarmonicAngleInteraction (:311-338) */
    const int32_t* angle_atoms;     /* [n_angles*3] shared, atom1, atom2 */
    const double* angle_param;      /* [n_angles*2] k, theta0 */
    int32_t n_dihedrals;            /* HarmonicDihedralInteraction (:340-370) */
    const int32_t* dihedral_atoms;  /* [n_dihedrals*4] atom1..atom4 */
    const double* dihedral_param;   /* [n_dihedrals*2] k, sigma0 */
    int32_t n_pairs;                /* non-bonded surface pairs (simulation.cpp:678-690) */
    const int32_t* pair_atoms;      /* [n_pairs*2] i < j */
    const mafm_pair* pair_vdw;      /* [n_pairs] LJ / Morse */
    const double* pair_qq;          /* [n_pairs] qbase q_i q_j, 0 = no Coulomb term */
    double substrate[5];            /* eps, sig, lambda, rc, k (parse.cpp:741-747) */
} mafm_flex_desc;

/* The flexible topology of a `flexible on` input (storage owned by `in`). */
int mafm_input_flex_desc(const mafm_input* in, mafm_flex_desc* out);

/* A device-resident flexible scan: one warp relaxes every atom of a pixel
 * column in FP64, each atom's force summed in the reference's interaction
 * order.  Pair and Coulomb terms only (no rigid grid, no external field:
 * the reference refuses both with flexible molecules, parse.cpp:387-395). */
typedef struct mafm_flex mafm_flex;
int mafm_flex_create(int device, const mafm_scan_desc* desc, const mafm_flex_desc* flex,
                     mafm_flex** out);
int mafm_flex_destroy(mafm_flex* flex);
/* Relax columns [col_begin, col_end) (0, 0 = all); out as for mafm_run.
 * states != NULL receives, for column state_column, every atom's position
 * after each height: [nz][n_atoms + 2][3] (dummy, tip, surface atoms), what
 * System::makeXYZFile writes for the middle pixel (simulation.cpp:114-116). */
int mafm_flex_run(mafm_flex* flex, int32_t col_begin, int32_t col_end, mafm_point* out,
                  mafm_run_stats* stats, int32_t state_column, double* states, void* stream);
/* Output options of the input file: gzip, statistics, bufsize. */
int mafm_input_output_opts(const mafm_input* in, int32_t* gzip, int32_t* statistics,
                           int32_t* bufsize);
int mafm_input_free(mafm_input* in);

/* ---- device scan ----------------------------------------------------------
 * Uploads atoms and parameters, then builds what the reference builds in
 * buildInteractions (simulation.cpp:201-216): the external field by FFT
 * (ElectrostaticPotentialInteraction ctor, interactions.cpp:53-234) and the
 * rigid force grid (buildTipGridInteractions, simulation.cpp:420-501), in
 * FP64 for MAFM_FP64 runs and in FP32 for MAFM_FP32C runs.
 * device < 0 uses the current device. */
int mafm_scan_create(int device, const mafm_scan_desc* desc, mafm_scan** out);
int mafm_scan_destroy(mafm_scan* scan);
/* Number of points nx*ny*nz and columns nx*ny of the scan. */
int mafm_scan_size(const mafm_scan* scan, int64_t* n_points, int64_t* n_columns);

/* Relax every point of the scan: the pixel/z loops of Simulation::run
 * (simulation.cpp:78-122) with FIREMinimisation / SDMinimisation
 * (minimiser.cpp:39-129), the integrators (integrators.cpp:8-111) and
 * System::getOutput (system.cpp:28-51).  `out` holds n_points records and
 * may be host or device memory; for host memory the call returns when the
 * points are there.  Pinned (page-locked) host memory is written by the
 * kernel directly; pageable memory goes through a device staging buffer and
 * one copy.  `stats` may be NULL; when given, the call synchronises the
 * stream. */
int mafm_run(mafm_scan* scan, const mafm_run_opts* opts, mafm_point* out,
             mafm_run_stats* stats, void* stream);

/* Relax chosen pixel columns of a scan in plain FP64: for pixels (i, j)
 * given as columns[m] = i*ny + j, in any order and from anywhere in the scan,
 * out[m*nz + k] receives height k (n*nz records, host or device memory, as
 * for mafm_run).  One warp relaxes one column and adds every sum in the
 * reference's order, so the points are bit-identical to mafm_run's MAFM_FP64
 * points.  The pixel loop of Simulation::run (simulation.cpp:78-122) over a
 * sample of pixels: used to check a fast run against FP64 on pixels spread
 * over the whole scan.  Synchronises the stream. */
int mafm_run_columns(mafm_scan* scan, const int32_t* columns, int64_t n, mafm_point* out,
                     mafm_run_stats* stats, void* stream);

/* Relax several scans in one persistent launch (MAFM_FP32C or MAFM_DF).
 * outs[s] receives scan s's points; all outs must be device memory, or all
 * host (pinned host outputs are written directly, as for mafm_run). */
int mafm_run_batch(mafm_scan* const* scans, int32_t n_scans, const mafm_run_opts* opts,
                   mafm_point* const* outs, mafm_run_stats* stats, void* stream);

/* mafm_run_batch without any memory allocation.  No counterpart in the
 * reference: it exists for callers that cannot let a library call cudaMalloc
 * or cudaFree (their own capped memory pool, no implicit device-wide
 * synchronisation from cudaFree in a steady state, exact accounting of device
 * memory on a shared GPU).  The relax kernel's scratch — work-queue counters
 * and per-scan descriptors — lives in a fixed device array of the library
 * (256 B + MAFM_NOALLOC_MAX_SCANS descriptors of under 1 KB each), held by
 * every GPU that loads the library until the process exits.
 *   - At most MAFM_NOALLOC_MAX_SCANS scans per call, else MAFM_E_RANGE.
 *   - MAFM_FP32C, whole scans; every outs[s] must be device memory.
 *   - A scan with a rigid grid must have its FP32 grid built already (one
 *     mafm_run with MAFM_FP32C does that), else MAFM_E_INVALID.
 *   - The first call on a device looks up the array's device address; make
 *     that first call before any stream capture.
 *   - All calls share the array and it keeps the last call's contents; each
 *     call clears its counters first.  Calls that overlap on the GPU race:
 *     order them on one stream or with events.
 *   - The call synchronises the stream and reports device-side failures
 *     (watchdog, rigid-grid exit, staging timeout) like mafm_run_batch,
 *     whether or not stats is given; stats may be NULL (kernel_ms is left 0).
 *   - Outputs must be device memory of the scans' GPU, else MAFM_E_INVALID. */
#define MAFM_NOALLOC_MAX_SCANS 32
int mafm_run_batch_noalloc(mafm_scan* const* scans, int32_t n_scans, const mafm_run_opts* opts,
                           mafm_point* const* outs, mafm_run_stats* stats, void* stream);

/* A prepared batched relaxation (MAFM_FP32C or MAFM_DF; the same persistent
 * launch as mafm_run_batch) whose per-scan descriptors are uploaded once, so
 * that the launch itself allocates nothing, never synchronises and can be
 * replayed or captured in a CUDA graph.  Replaces the pixel loop of
 * Simulation::run (simulation.cpp:78-122) for many scans at once.  Creating a
 * plan also orders each scan's columns by measured cost (one FP32C
 * relaxation of the scan, once per scan; the launch then ends with fewer
 * idle lanes).  outs must be device memory and stay valid for the plan's
 * lifetime. */
int mafm_plan_create(mafm_scan* const* scans, int32_t n_scans, const mafm_run_opts* opts,
                     mafm_point* const* outs, mafm_plan** out);
/* Enqueue one relaxation of every scan of the plan on stream. */
int mafm_plan_launch(mafm_plan* plan, void* stream);
/* Counters of the last launch; synchronises the stream. */
int mafm_plan_stats(mafm_plan* plan, mafm_run_stats* stats, void* stream);
/* The launch shape the plan uses (lanes per column, block, tile). */
int mafm_plan_config(const mafm_plan* plan, mafm_run_opts* opts);
int mafm_plan_destroy(mafm_plan* plan);

/* Autotuner: times launch shapes of the FP32C kernel (lanes per column, block
 * size, columns per warp tile) on the given scans and returns the fastest in
 * best (pass it to mafm_run / mafm_run_batch / mafm_plan_create).  For a batch
 * of more than 32 scans the sweep runs on the first 32 and its winner is timed
 * against the default shape on the whole batch.  No
 * counterpart in the reference, whose OpenMP schedule is fixed (dynamic, 1,
 * simulation.cpp:78). */
int mafm_autotune(mafm_scan* const* scans, int32_t n_scans, mafm_run_opts* best, double* best_ms,
                  void* stream);

/* Gradients of a scalar loss L of the Fz image (no counterpart in the
 * reference, which has no derivatives).  Given the relaxed points of a run
 * (the checkpoint of every z-slice) and w_p = dL/dFz_p per point, the
 * gradient is taken by implicit differentiation at each relaxed tip position:
 * J = dF_total/dx (3x3) and dx/dtheta = -J^-1 dF_ts/dtheta, without
 * unrolling FIRE.  theta: surface atom positions as in the descriptor, the
 * per-type tip pair parameters tip_pair[t].p (LJ es6, es12; Morse De, a, re)
 * and the atom charges.  pts and dl_dfz (n_points each) may be host or device
 * memory; out arrays are host memory (any may be NULL).  Pair and external
 * field scans only (MAFM_E_UNSUPPORTED for rigid grids). */
typedef struct mafm_grad {
    double* dpos;      /* [n_atoms*3] */
    double* dcharge;   /* [n_atoms] */
    double* dpair;     /* [n_types*3] */
} mafm_grad;
int mafm_adjoint(mafm_scan* scan, const mafm_point* pts, const double* dl_dfz, mafm_grad* out,
                 void* stream);
/* mafm_adjoint with a precision: MAFM_FP64 (the same as mafm_adjoint) or
 * MAFM_FP32C (per-term Jacobians and parameter derivatives in FP32 with
 * compensated sums, the per-point 3x3 solve in FP64; gradients agree with
 * the FP64 ones to about 1e-5 relative).  No counterpart in the reference. */
int mafm_adjoint_ex(mafm_scan* scan, int32_t precision, const mafm_point* pts,
                    const double* dl_dfz, mafm_grad* out, void* stream);

/* ---- frequency-shift images ------------------------------------------------
 * The reference's post-processing (simple-vafm-image.py:77-89, 204) turns Fz
 * stacks into frequency-shift images with Giessibl's weights; these run that
 * operator on the GPU.  Parameters default (params = NULL) to the script's
 * A = 0.5 A, k = 1800 N/m = 1800*1.438978 kcal/mol/A^2, f0 = 25 kHz. */
typedef struct mafm_df_params {
    double amplitude;       /* oscillation amplitude A (Angstrom) */
    double k_cantilever;    /* cantilever stiffness (energy unit / A^2) */
    double f0;              /* resonance frequency (Hz) */
} mafm_df_params;
/* The window weights W (n_w values) and fshiftfac for height step dz. */
int mafm_df_weights(const mafm_df_params* params, double dz, double* w, int32_t cap, int32_t* n_w,
                    double* fshiftfac);
/* df[s][x][y] for every window s of n_w heights (nz - n_w windows, ascending
 * z): fz[((x*ny + y)*nz + k) * stride] is Fz at scan level k (k = 0 at zhigh);
 * stride 8 reads mafm_point.force[2] (pass &pts[0].force[2]).  Host or device
 * memory. */
int mafm_df(const double* fz, int64_t stride, int32_t nx, int32_t ny, int32_t nz, double dz,
            const mafm_df_params* params, double* df, void* stream);
/* Transpose of mafm_df: dL/dFz (nx*ny*nz, level order) from dL/ddf. */
int mafm_df_adjoint(const double* g_df, int32_t nx, int32_t ny, int32_t nz, double dz,
                    const mafm_df_params* params, double* g_fz, void* stream);

/* Evaluate the tip–surface force and energy at n given tip positions
 * (System::evalTipSurfaceForces, system.cpp:41-51): pairs, external field or
 * rigid grid, whatever the scan uses.  what: 0 = all tip–surface terms,
 * 1 = external field only.  pts[n*3] and out[n*4] = {Fx,Fy,Fz,E} are host
 * memory.  precision selects the FP64 or FP32 tables. */
int mafm_scan_sample(mafm_scan* scan, int32_t precision, int32_t what,
                     const double* pts, int64_t n, double* out);

/* Geometry of the rigid force grid (or of the external field when what = 1):
 * node counts, basis (row-major, columns = steps) and origin. */
int mafm_scan_grid_info(const mafm_scan* scan, int32_t what, int32_t n[3],
                        double basis[9], double origin[3]);
/* Copy the FP64 grid nodes {Fx,Fy,Fz,E} (n0*n1*n2*4 doubles, z fastest). */
int mafm_scan_grid_copy(const mafm_scan* scan, int32_t what, double* out);
/* (Re)build the rigid force grid of a rigidgrid scan for one precision on the
 * stream: Simulation::buildTipGridInteractions (simulation.cpp:420-501), which
 * the reference runs once per scan before the pixel loop.  mafm_run builds the
 * grid on first use; this call rebuilds it on demand.  The first call for a
 * precision allocates the grid; later calls only launch the build kernel(s)
 * (MAFM_DF: the double-float build and its FP64 copy), so they may be
 * captured in a CUDA graph together with mafm_plan_launch.
 * No-op (MAFM_OK) for a scan without a rigid grid. */
int mafm_scan_build_grid(mafm_scan* scan, int32_t precision, void* stream);

/* ---- output (host) ---------------------------------------------------------
 * Writes scan-%06.3f.dat[.gz] files and statistics.txt exactly as the
 * reference (openUniverse mechafm.cpp:60-75, writeOutput simulation.cpp:145-199,
 * finalize mechafm.cpp:140-152).  folder may be "" (current directory) and
 * must end in '/' otherwise.  Rows are written in point order. */
int mafm_write_output(const mafm_input* in, const mafm_point* pts, const char* folder,
                      int32_t gzip);
/* The same files written chunk by chunk, so that a caller can format and
 * write the points of one chunk of pixel columns while the GPU relaxes the
 * next (the reference writes each height file as its buffer fills,
 * simulation.cpp:123-138).  mafm_writer_open opens every height file;
 * mafm_writer_append writes columns [col_begin, col_end) (c = i*ny + j),
 * whose points pts holds at (c - col_begin)*nz + k (host memory); the ranges
 * must follow one another from column 0, so the files receive their rows in
 * pixel order and end up byte-identical to mafm_write_output's.
 * mafm_writer_close closes them (and waits for gzip). */
typedef struct mafm_writer mafm_writer;
int mafm_writer_open(const mafm_input* in, const char* folder, int32_t gzip, mafm_writer** out);
int mafm_writer_append(mafm_writer* w, const mafm_point* pts, int32_t col_begin, int32_t col_end);
int mafm_writer_close(mafm_writer* w);
/* System::makeXYZFile (system.cpp:54-66) for every height of one column of
 * a flexible scan: writes <folder>state_<x>-<y>-<z>.xyz (%.1f each: the pixel
 * position and the dummy height) with every atom's type and position, and
 * prints the reference's "+- Wrote <file>" line.  states as filled by
 * mafm_flex_run: [nz][n_atoms + 2][3]. */
int mafm_write_states(const mafm_input* in, const double* states, int32_t column,
                      const char* folder);
/* statistics.txt of finalize (mechafm.cpp:140-152). */
int mafm_write_statistics(const mafm_input* in, const char* folder, uint64_t total_steps,
                          double wall_s, double total_s);

#ifdef __cplusplus
}
#endif

#endif /* MAFM_H */
