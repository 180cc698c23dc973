// mafm_df.h — device data of the double-float path (MAFM_DF); CUDA only.
//
//   TermPairDF  two tip–atom terms of the same kind side by side, every FP64
//               quantity of AtomRec64 split into high and low FP32 parts,
//               128 B: the relax kernel evaluates both with packed f32x2
//               instructions
//   NodeDF      one external-field node {Fx, Fy, Fz, E} in double-float, 32 B
//   ScanParamsDF the scalars of ScanParams in double-float, with the same
//               member names, so the templated minimiser (relax_tpl.cuh)
//               reads either
//   BatchDF     one scan of a double-float launch
#pragma once

#include <vector>

#include "dfloat.cuh"
#include "mafm_internal.h"

namespace mafm {

// Element .x is the first term, .y the second; h / l the high and low parts.
// A scan's pairs hold its LJ terms, then its Morse terms, each run padded to
// an even count with a term of zero parameters and charge.
struct __align__(16) TermPairDF {
    float2 xh, xl, yh, yl, zh, zl;   // image positions
    float2 qqh, qql;                 // Coulomb prefactor qbase q_tip q_atom (0: no Coulomb term)
    float2 p0h, p0l, p1h, p1l;       // LJ es6, es12; Morse De, a
    float2 p2h, p2l;                 // Morse re
    int32_t coul;                    // 1 if either term has a Coulomb term
    int32_t pad[3];
};
static_assert(sizeof(TermPairDF) == 128, "128-byte term-pair records");

struct __align__(32) NodeDF {
    dfloat x, y, z, w;
};

struct GridViewDF {
    const NodeDF* g;
    int n[3];
    int periodic;
    int orthogonal;
    int pad;
    dfloat basis[9];       // row-major, columns are the node steps
    dfloat inv[9];
    dfloat origin[3];
};

// Near-tie margins (absolute): a convergence test within conv_e / conv_f of
// its tolerance, or a sign test of P = v.F with |P| < |v| (p_f + p_v |F|),
// marks the column for the FP64 re-relaxation.
struct TieMargins {
    dfloat conv_e, conv_f, p_f, p_v;
};

struct ScanParamsDF {
    int n_lj_pairs, n_morse_pairs;   // pairs[0, n_lj_pairs) LJ, then Morse
    int ts_mode;           // 0 pair terms, 1 pair terms + external field, 2 rigid grid
    const TermPairDF* pairs;
    GridViewDF es;
    GridViewDF grid;       // the double-float rigid grid (ts_mode 2)
    int td_kind, td_coul;
    dfloat td_p[3];
    dfloat td_qq;
    dfloat harm_k, harm_r0, tip_dummy_d;
    int nx, ny, nz, tip_pbc;
    dfloat dx, dy, dz, zhigh;
    dfloat cell[9], cell_inv[9], offset[3];
    int minimiser, integrator, minterm, maxsteps;
    dfloat etol, ftol, dt;
    TieMargins tie;
};

struct BatchDF {
    ScanParamsDF p;
    mafm_point* out;       // points of columns [col_begin, col_end), (col - col_begin) nz + k
    long long col_first;   // first queue index of this scan in the launch
    int col_begin, col_end;
    const int* order;      // processing order of a whole scan's columns, or null
    int n_pairs_per_eval;
    int pad;
};

// Host: the double-float parameter block of a scan whose term pairs
// (term_pairs_df) are at pairs, its external field at es_nodes and its
// double-float rigid grid at grid_nodes (p.grid's geometry).
ScanParamsDF params_df(const ScanParams& p, const TermPairDF* pairs, int n_lj_pairs,
                       int n_morse_pairs, const NodeDF* es_nodes, const NodeDF* grid_nodes);
// Host: a scan's FP64 terms as double-float pairs, LJ first, then Morse.
std::vector<TermPairDF> term_pairs_df(const std::vector<AtomRec64>& terms, int& n_lj_pairs,
                                      int& n_morse_pairs);

// Relax every column of the listed scans; columns with a near-tie decision
// go to repair_list (scan << 32 | column, capacity repair_cap; filled with
// all-ones first; null: none) and are re-relaxed in FP64 from scans64 (the
// same scans' FP64 descriptors) by warps that run out of columns; the
// entries left are for repair64_kernel.  lanes_per_column: 1, 2, 4 or 8
// lanes share a column's terms (0: default).
cudaError_t launch_relaxdf(const BatchDF* scans, const BatchScan* scans64, int n_scans, long long n_cols,
                           RunCounters* ctr, unsigned long long* repair_list, unsigned repair_cap,
                           unsigned long long watchdog_ns, int lanes_per_column, cudaStream_t s);
// The lanes per column a launch of n_cols columns uses for a request (0: default).
int df_lanes_per_column(long long n_cols, int requested);
// The external field's FP64 nodes as double-float.
cudaError_t launch_nodes_to_df(const Node64* in, NodeDF* out, long long n, cudaStream_t s);
// Simulation::buildTipGridInteractions (simulation.cpp:420-501) in
// double-float: the rigid grid of geometry p.grid (p.ts_mode 0 or 1: the
// terms, and the external field) into out, then its FP64 copy (each node's
// h + l, exact in FP64) into out64 for the FP64 re-relaxation; device error
// bits (a lookup of the external field) are ORed into *err_word.
cudaError_t launch_grid_builddf(const ScanParamsDF& p, NodeDF* out, Node64* out64, unsigned* err_word,
                                cudaStream_t s);

}  // namespace mafm
