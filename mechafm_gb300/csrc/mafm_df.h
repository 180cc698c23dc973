// mafm_df.h — device data of the double-float path (MAFM_DF); CUDA only.
//
//   AtomRecDF   one tip–atom term in double-float, 64 B: the FP64 term of
//               AtomRec64 split into high and low FP32 parts
//   NodeDF      one external-field node {Fx, Fy, Fz, E} in double-float, 32 B
//   ScanParamsDF the scalars of ScanParams in double-float, with the same
//               member names, so the templated minimiser (relax_tpl.cuh)
//               reads either
//   BatchDF     one scan of a double-float launch
#pragma once

#include "dfloat.cuh"
#include "mafm_internal.h"

namespace mafm {

struct __align__(16) AtomRecDF {
    dfloat x, y, z, qq;    // image position, Coulomb prefactor qbase q_tip q_atom
    dfloat p0, p1, p2;     // LJ es6, es12, -; Morse De, a, re
    int32_t kind;          // MAFM_PAIR_*
    int32_t coul;          // 1 if a Coulomb term follows the vdW term
};
static_assert(sizeof(AtomRecDF) == 64, "64-byte term records");

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
    int n_terms;
    int ts_mode;           // 0 pair terms, 1 pair terms + external field
    const AtomRecDF* atoms;
    GridViewDF es;
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

// Host: the double-float parameter block of a scan.
ScanParamsDF params_df(const ScanParams& p, const AtomRecDF* atoms, const NodeDF* es_nodes);
// Host: AtomRec64 -> AtomRecDF.
AtomRecDF term_df(const AtomRec64& r);

// Relax every column of the listed scans; columns with a near-tie decision
// go to repair_list (scan << 32 | column, capacity repair_cap; null: none).
cudaError_t launch_relaxdf(const BatchDF* scans, int n_scans, long long n_cols, RunCounters* ctr,
                           unsigned long long* repair_list, unsigned repair_cap,
                           unsigned long long watchdog_ns, cudaStream_t s);
// The external field's FP64 nodes as double-float.
cudaError_t launch_nodes_to_df(const Node64* in, NodeDF* out, long long n, cudaStream_t s);

}  // namespace mafm
