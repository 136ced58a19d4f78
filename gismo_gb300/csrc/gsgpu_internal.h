// Internal declarations shared by the host runtime and the sm_103a kernels of libgsgpu.
//
// Data model (all per patch; a "batch" is any list of tensor-product B-spline patches):
//   * per direction k: n[k] dofs, E[k] elements (non-empty knot spans), q[k] Gauss points per
//     element, Q[k] = E[k]*q[k] global quadrature abscissae, W[k] = 2 p[k] + 1 band offsets;
//   * quadrature-point fields are stored [component][g_{d-1}]...[g_0] (g_0 fastest);
//   * the element stiffness is never formed: the patch operator is produced in "band" layout
//     K[(i_{d-1},o_{d-1})]...[(i_0,o_0)] with o_k = j_k - i_k + p_k in [0, W_k) by three
//     (two in 2D) sum-factorised 1-D contractions over the global quadrature grid;
//   * the band is reduced into the global CSR matrix under the gsDofMapper numbering by a
//     gather over a symbolically precomputed slot -> band-entry map (no atomics).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace gsgpu {

constexpr int kMaxDim = 3;

struct DevPatch {
    int dim;
    int field_id;  // index of the patch's closed-form field constants (batches of independent problems)
    int p[3], n[3], E[3], q[3], Q[3], W[3];
    // per axis: element e's first active function is e, function i's support is elements
    // max(0, i-p)..min(E-1, i) (simple interior knots) and q = p + 1: the rows p..n-1-p then have
    // a fixed support shape (the unrolled interior contraction)
    int simple[3];
    int gp[3], gn[3];
    long long ngeo;   // geometry control points
    long long nq;     // quadrature points (Q0*Q1*Q2)
    long long ndof;   // n0*n1*n2
    // offsets into the packed per-direction arrays of the context
    long long qoff[3];     // quadrature abscissae / weights (Q[k] each)
    long long toff[3];     // discretisation basis tables: V/D [(g*(p+1)+s)]
    long long gtoff[3];    // geometry basis tables
    long long eoff[3];     // first active function per element (int)
    long long doff[3];     // support element range per dof: elo / ehi (int)
    long long gqoff[3];    // geometry first active function per quadrature abscissa (int)
    long long pfoff[3];    // pair factors [4][E][q][p+1][p+1]
    // offsets into the big buffers
    long long coef_off;    // geometry control points, [m][ngeo] (structure of arrays)
    long long field_off;   // coefficient field C, ncomp blocks of nq
    long long lfield_off;  // load field L (nq)
    long long y1_off, y2_off;   // geometry sum-factorisation intermediates
    long long s_off, u_off;     // stiffness contraction intermediates
    long long band_off;         // band matrix
    long long lv1_off, lv2_off; // load contraction intermediates
    long long lvec_off;         // patch load vector (ndof)
    long long bandsize;         // prod_k n[k]*W[k]
};

// one entry of a block -> (patch, first work item) table used by every batched kernel
struct BlkEnt {
    int patch;
    int pad;
    long long base;
};

// one 1-D basis evaluation: knots at koff, degree p, span, abscissa u, 2(p+1) outputs at out
struct TabJob {
    long long koff;
    long long out;
    double u;
    int p;
    int span;
};

// pair-factor table of one (patch, direction): 4*E*q*(p+1)^2 entries from the basis table
struct PfJob {
    long long tab;
    long long pf;
    long long count;
    int p, q, E, pad;
};

// one Neumann side: the patch, the fixed direction and end, the side directions t[0], t[1] (t[1] = -1
// in 2D), the first function and the values at the boundary parameter of the geometry (gfirst,
// gval) and discretisation (bfirst, bval) bases of the fixed direction, and the side's block of
// face quadrature values (qbase, nq = Q[t0] Q[t1] points, t0 fastest)
constexpr int kMaxNeuDeg = 15;
struct NeuSide {
    int patch, dir, upper, t[2];
    int gfirst, gp, bfirst, bp;
    int pad;
    double gval[kMaxNeuDeg + 1];
    double bval[kMaxNeuDeg + 1];
    long long qbase, nq;
};

// one patch-local dof on Neumann sides: its coordinates, its load-vector slot and the sides
struct NeuDof {
    int patch, nside;
    int side[6];
    int i[3];
    int pad;
    long long lvec;
};

// closed-form coefficient / source / exact-solution parameters (device constant-style struct)
constexpr int kMaxModes = 64;
struct FieldParams {
    int dim;
    int fourier;
    int nmodes;
    int ufreq;
    int kmax;  // largest wave number component over the modes
    int pad;
    double kconst, alpha, scale;
    double amp[kMaxModes];
    double phase[kMaxModes];
    double cph[kMaxModes], sph[kMaxModes];  // cos / sin of the phases
    int kk[kMaxModes][3];
};

// precision modes of assemble()
enum Precision : int {
    kFP64 = 0,   // plain FP64 everywhere
    kMixed = 1,  // FP32 inner operator + FP64-accurate outer operator (iterative refinement)
};

}  // namespace gsgpu

#define GSGPU_CUDA_TRY(expr)                                                   \
    do {                                                                       \
        cudaError_t _e = (expr);                                               \
        if (_e != cudaSuccess) throw gsgpu::CudaError(_e, #expr, __FILE__, __LINE__); \
    } while (0)
