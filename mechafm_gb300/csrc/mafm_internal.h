// mafm_internal.h — structures shared by the host library and the kernels.
//
// Device data layout (HBM):
//   atoms64  AtomRec64[n]   64 B per tip–atom term, in the reference's
//                           interaction order (simulation.cpp:297-320): for
//                           vdw_pbc the 3x3 images are the outer loop and the
//                           atoms the inner loop; positions already carry the
//                           image shift (interactions.cpp:16,30).
//   atoms32  AtomRec32[n]   32 B per term: float4 {x,y,z,qq} + float4 {p0,p1,p2,kind}
//   units32  TermPair32[u]  the FP32 terms two by two for packed (f32x2)
//                           arithmetic: the LJ terms, then the Morse terms,
//                           each run padded to an even count with a zero term
//   grid64   Node64[n]     rigid force grid {Fx,Fy,Fz,E}, index (i*ny+j)*nz+k
//   grid32   float4[n]      same in FP32
//   es64/es32               external-field grid, same layout
#pragma once

#include <cstdint>
#include <cstdlib>
#include <new>
#include <stdexcept>
#include <string>
#include <cuda_runtime.h>

#include "mafm.h"

namespace mafm {

// Host-side failure carried to the C ABI boundary, where it becomes a status
// code plus mafm_last_error() text.  Never crosses extern "C".
struct Failure {
    int code;
    std::string msg;
};
[[noreturn]] void fail(int code, const char* fmt, ...);
void set_last_error(const std::string& msg);

template <class F>
int guarded(F&& f) {
    try {
        f();
        return MAFM_OK;
    } catch (const Failure& e) {
        set_last_error(e.msg);
        return e.code;
    } catch (const std::bad_alloc&) {
        set_last_error("host allocation failed");
        return MAFM_E_NOMEM;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return MAFM_E_INVALID;
    }
}

inline void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) fail(MAFM_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// Time limit of the persistent relax kernels in nanoseconds: MAFM_WATCHDOG_S
// seconds (fractions allowed), else 120 s.  Unset, non-numeric, zero,
// negative or absurdly large values all give the 120 s default.
inline unsigned long long watchdog_ns_from_env() {
    const char* w = std::getenv("MAFM_WATCHDOG_S");
    double s = w ? std::atof(w) : 0.0;
    if (!(s > 0.0) || s > 1.0e6) s = 120.0;
    return (unsigned long long)(s * 1.0e9);
}

// Device error bits (mafm_run_stats.error_word, upper half; lower bits are MAFM_PT_*).
enum : uint32_t {
    ERR_GRID_INDEX = 1u << 16,   // corner outside a non-periodic grid (force_grid.cpp:236-240)
    ERR_STAGE_TIMEOUT = 1u << 17, // bounded wait on the atom staging barrier expired
    ERR_WATCHDOG = 1u << 18,      // a persistent warp ran past its time limit
    ERR_REPAIR_WAIT = 1u << 19    // a bounded wait for a near-tie column's list entry expired
};

struct __align__(16) AtomRec64 {
    double x, y, z, qq;    // image position, Coulomb prefactor qbase*q_tip*q_atom
    double p0, p1, p2;     // LJ: es6, es12, - ; Morse: De, a, re
    int32_t kind;          // MAFM_PAIR_*
    int32_t coul;          // 1 if a Coulomb term follows the vdW term
};

// One FP64 grid node {Fx, Fy, Fz, E}.
struct __align__(32) Node64 {
    double x, y, z, w;
};

struct __align__(16) AtomRec32 {
    float4 a;              // x, y, z, qq
    float4 b;              // p0, p1, p2, kind (int bits)
};

// Two FP32 terms side by side (component 0: term 2u, component 1: term 2u+1)
// for the relax kernel's packed arithmetic.  Signs are stored so that the
// loop needs packed adds, multiplies and FMAs only: positions, qq and LJ's
// es6 negated, Morse's a and re negated and its force prefactor stored as
// -2 De a.  A padding
// term has zero parameters and sits far away, so every part of it is 0.
struct __align__(16) TermPair32 {
    float4 xy;             // -x0, -x1, -y0, -y1
    float4 zq;             // -z0, -z1, -qq0, -qq1
    float4 pa;             // LJ -es6_0, -es6_1, es12_0, es12_1 | Morse De_0, De_1, -a_0, -a_1
    float4 pb;             // LJ -12 es12_0, -12 es12_1, 6 es6_0, 6 es6_1 | Morse -re_0, -re_1, -2 De a_0, -2 De a_1
};

// A trilinear force grid (ForceGrid, force_grid.hpp:15-51).
struct GridView {
    const Node64* g64;
    const float4* g32;
    int n[3];
    int periodic;
    int orthogonal;
    int pad;
    double basis[9];       // row-major, columns are the node steps
    double inv[9];         // inverse of basis (Matrix3::inverse)
    double origin[3];
};

// Everything a relax / build / sample kernel needs for one scan.
struct ScanParams {
    // tip–atom terms
    int n_terms;
    int n_terms_direct;    // terms evaluated per force call (0 in rigid-grid mode)
    const AtomRec64* atoms64;
    const AtomRec32* atoms32;
    const TermPair32* units32;
    int n_units;           // TermPair32 records
    int n_units_lj;        // of which the first n_units_lj hold LJ terms
    // tip–surface source of the relax: 0 pairs, 1 pairs + external field, 2 rigid grid
    int ts_mode;
    int has_coulomb;       // any term carries a Coulomb part
    GridView grid;         // rigid grid (ts_mode 2)
    GridView es;           // external field (ts_mode 1, and grid build)
    // tip–dummy coupling (buildTipDummyInteractions, simulation.cpp:503-515)
    int td_kind;
    int td_coul;
    double td_p[3];
    double td_qq;
    double harm_k, harm_r0;
    double tip_dummy_d;
    // pixel grid and z descent
    int nx, ny, nz;
    int tip_pbc;
    double dx, dy, dz, zhigh;
    double cell[9], cell_inv[9], offset[3];
    // minimiser
    int minimiser, integrator, minterm, maxsteps;
    double etol, ftol, dt;
};

// Counters the relax kernels update (device memory owned by the scan).
struct RunCounters {
    unsigned long long next_work;     // persistent work queue head
    unsigned long long total_steps;
    unsigned long long force_evals;
    unsigned long long pair_evals;
    unsigned int error_word;
    unsigned int n_tie;               // MAFM_DF: columns listed for FP64 re-relaxation
                                      // (may exceed the list's capacity)
    unsigned long long repair_next;   // queue head of the FP64 re-relaxation (taken in the
                                      // double-float kernel, then by repair64_kernel)
};

// Launchers implemented in relax64.cu / relax32.cu.  ctr points to zeroed
// device counters owned by the caller.
cudaError_t launch_relax64(const ScanParams& p, mafm_point* out, RunCounters* ctr,
                           int col_begin, int col_end, cudaStream_t s);
cudaError_t launch_sample64(const ScanParams& p, int what, const double* pts, int64_t n,
                            double* out, RunCounters* ctr, cudaStream_t s);
cudaError_t launch_grid_build64(const ScanParams& p, const GridView& g, Node64* out,
                                RunCounters* ctr, cudaStream_t s);

// One entry of a multi-scan work list for the FP32 persistent kernel.
struct BatchScan {
    ScanParams p;
    mafm_point* out;          // points of columns [col_begin, col_end), (col-col_begin)*nz+k
    long long tile_begin;     // first global tile index of this scan
    int col_begin, col_end;
    int n_pairs_per_eval;     // vdW + Coulomb terms per force evaluation
    int has_coulomb;
    const int* order;         // processing order of the columns (most expensive
                              // first), nullptr = index order; whole scans only
};

struct Relax32Config {
    int lanes;                // lanes per column (1,2,4,8,16,32)
    int block;                // threads per block
    int cols_per_tile;        // columns per warp work tile
    int smem_terms;           // terms staged per warp (larger scans read global memory)
    int blocks;               // 0 = fill the GPU
    unsigned long long watchdog_ns;   // persistent-kernel time limit
};

cudaError_t launch_relax32(const BatchScan* scans_dev, int n_scans, long long n_tiles,
                           const Relax32Config& cfg, RunCounters* ctr, cudaStream_t s);
// FP64 re-relaxation of listed columns (relax64.cu): list[i] = scan index << 32
// | column for i < min(count, cap), where count = ctr->n_tie when n_fixed < 0
// (the columns the double-float kernel flagged) and n_fixed otherwise.
// replace = true marks the points MAFM_PT_FP64 and corrects the step total
// for the records it overwrites.  The points of column c go to
// out + (c - col_begin) nz, or with list_out to out + i nz for list entry i.
cudaError_t launch_repair64(const BatchScan* scans, const unsigned long long* list, unsigned cap,
                            long long n_fixed, bool replace, bool list_out, RunCounters* ctr,
                            cudaStream_t s);
cudaError_t launch_sample32(const ScanParams& p, int what, const double* pts, int64_t n,
                            double* out, RunCounters* ctr, cudaStream_t s);
cudaError_t launch_grid_build32(const ScanParams& p, const GridView& g, float4* out,
                                RunCounters* ctr, cudaStream_t s);
int sm_count();
cudaError_t launch_adjoint(const ScanParams& p, int precision, const int* index32,
                           const mafm_point* pts, const double* w, long long n_points,
                           double qbase_qtip, double* gterm, RunCounters* ctr, cudaStream_t s);

}  // namespace mafm

// Read-only views of a scan for entry points defined outside scan.cu.
namespace mafm {
int scan_device(const mafm_scan* s);
long long scan_columns(const mafm_scan* s);
int scan_direct_terms(const mafm_scan* s);
bool scan_fp32_ready(const mafm_scan* s);   // FP32 tables on the device (rigid grid built if used)
BatchScan scan_batch_entry(const mafm_scan* s, mafm_point* out);
Relax32Config relax32_config(long long n_cols, int max_terms, const mafm_run_opts* o, int n_scans);
void check_run_errors(const RunCounters& c);
}  // namespace mafm
