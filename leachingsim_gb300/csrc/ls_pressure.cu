// ls_pressure.cu - Darcy pressure system of Simulation::setupPressureEqns +
// solvePressure (src/Simulation.cpp:658-855), matrix-free.
//
// Rows (one per voxel, src/Simulation.cpp:674-792):
//   Air/Rock/Sulphide/Precipitate: identity, value = ramped top pressure on Air voxels
//     that touch a non-Air voxel, else 0                                   (kind 1)
//   Pore: sum_n c_n P_n + diag P = b, c_n = harmonic(K)/mu, diag = -sum c_n
//     (floored to +1e-16 when |diag| < 1e-16: kind 3, else kind 2)
//   any other label: no entries at all (kind 0); Krylov methods leave such an unknown
//     at its initial value, so it keeps its current value here.
//
// Solver: FP64 iterative refinement on the assembled operator A. Each sweep computes
// r = b - A x in FP64 and the correction from a block-triangular splitting: floored
// rows (kind 3) are solved from their diagonal, the normal Pore rows (kind 2) from the
// symmetric positive definite system M d = A_SQ d_Q - r_S with M = -A_SS, solved by an
// inner PCG in FP32 (LS_PRESS_MIXED) or FP64, preconditioned by multigrid (or Jacobi for
// LS_PRESS_JACOBI64). M is scaled by sigma = 1/max(diagonal) and held as
// e_i x_i + sum_links c_ij (x_i - x_j) with e_i = links to rows that are not unknowns,
// which stays positive definite under FP32 rounding.
// Convergence is judged on the FP64 Jacobi-scaled residual ||D^-1 r|| / ||D^-1 b||, the
// norm PETSc's left-Jacobi GMRES tests in the reference.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <type_traits>

#include "ls_internal.cuh"

namespace ls {

template <typename T>
ls_status mg_setup(ls_ctx* c);
template <typename T>
ls_status mg_clear(ls_ctx* c);
template <typename T>
ls_status mg_apply(ls_ctx* c, const T* r, T* z, const T* dotv2, int* nblocks_out);
template <typename T>
ls_status mg_precondition(ls_ctx* c, const T* r, T* z, const T* dotv2, int slot);
int lpnet_tc_timeouts();
template <typename T>
ls_status inner_invd(ls_ctx* c);

// scalar slots
enum {
    SP_NUM = 16,   // sum (r/diag)^2 over rows
    SP_NAN = 17,
    SP_DEN = 18,   // sum (b/diag)^2
    SP_XMAX = 19,
    SP_XNMAX = 20, // max of -x
    SP_RZ = 24,    // inner: (r, z)
    SP_PQ = 25,    // inner: (p, q)
    SP_RZN = 26,   // inner: new (r, z)
    SP_ZQ = 27     // inner: (z_new, q), the flexible-CG direction term
};

// ---------------------------------------------------------------------------
// setup

struct PressConst {
    double eff_top, evap_dx;
    int bc_mode;             // ls_bc_mode
    double p_inlet, p_outlet;
};

template <typename L>
__device__ __forceinline__ double link_coeff(const L* __restrict__ label,
                                             const double* __restrict__ perm,
                                             const double* __restrict__ visc, long long self,
                                             long long nb) {
    // set_neighbor_link of src/Simulation.cpp:730-771 for the Pore voxel `self`
    double K_neighbor = ((int)label[nb] == kAir) ? 1.0e-9 : perm[nb];
    double K_self = smax(perm[self], 1e-25);
    double K_neigh = smax(K_neighbor, 1e-25);
    double K_avg = (2.0 * K_self * K_neigh) / (K_self + K_neigh);
    return K_avg / visc[self];
}

// Change test of the face inputs (pass 1 of the faces): the dirty bit of voxel r is set when
// its label, permeability or viscosity differ bitwise from the values at the last face
// evaluation.
template <typename L>
__global__ void __launch_bounds__(kBlock) k_faces_dirty(Grid g, const L* __restrict__ label,
                                                        const double* __restrict__ perm,
                                                        const double* __restrict__ visc,
                                                        L* __restrict__ sl, double* __restrict__ sp,
                                                        double* __restrict__ sv,
                                                        unsigned int* __restrict__ bits, int force) {
    for (long long r0 = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); r0 < g.N;
         r0 += (long long)gridDim.x * blockDim.x) {
        const long long r = r0 + (threadIdx.x & 31u);
        bool d = false;
        if (r < g.N) {
            const L lab = label[r];
            const long long pb = __double_as_longlong(perm[r]);
            const long long vb = __double_as_longlong(visc[r]);
            d = force || lab != sl[r] || pb != __double_as_longlong(sp[r]) || vb != __double_as_longlong(sv[r]);
            if (d) {
                sl[r] = lab;
                sp[r] = __longlong_as_double(pb);
                sv[r] = __longlong_as_double(vb);
            }
        }
        const unsigned int w = __ballot_sync(0xffffffffu, d);
        if ((threadIdx.x & 31u) == 0u) bits[r0 >> 5] = w;
    }
}

// Pass 2: voxels holding a face (their +i, +j, +k faces) with a dirty voxel on either side.
__global__ void __launch_bounds__(kBlock) k_faces_scan(Grid g, const unsigned int* __restrict__ bits,
                                                       long long nw, int* __restrict__ list,
                                                       unsigned int* __restrict__ count) {
    const int lane = (int)(threadIdx.x & 31u);
    // block-uniform trip count (block_append is called by every thread of the block)
    for (long long b0 = (long long)blockIdx.x * blockDim.x; b0 < g.N; b0 += (long long)gridDim.x * blockDim.x) {
        const long long r0 = b0 + (threadIdx.x & ~31u);
        const long long r = r0 + lane;
        const unsigned int own = dwin(bits, nw, r0), kp = dwin(bits, nw, r0 + 1),
                           jp = dwin(bits, nw, r0 + g.K), ip = dwin(bits, nw, r0 + g.JK);
        bool need = false;
        if (r < g.N) {
            int i, j, k;
            decode(g, r, i, j, k);
            need = dbit(own, lane) || (i + 1 < g.I && dbit(ip, lane)) || (j + 1 < g.J && dbit(jp, lane)) ||
                   (k + 1 < g.K && dbit(kp, lane));
        }
        block_append(need, (int)r, list, count);
    }
}

// Pass 3: face coefficients of the +i, +j, +k faces of the listed voxels. A face is used
// only by the Pore rows on its two sides and gives the same value from either side (the
// harmonic mean is symmetric bit for bit: (2a)b == (2b)a, a+b == b+a), so it is computed
// once; it is a pure function of the labels, permeabilities and viscosities of its two
// voxels, so faces between clean voxels keep their stored values.
template <typename L>
__global__ void __launch_bounds__(kBlock) k_press_faces(Grid g, const L* __restrict__ label,
                                                        const double* __restrict__ perm,
                                                        const double* __restrict__ visc,
                                                        double* __restrict__ f0,
                                                        double* __restrict__ f1,
                                                        double* __restrict__ f2,
                                                        const int* __restrict__ list,
                                                        const unsigned int* __restrict__ count) {
    const int n = (int)*count;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int r = list[q];
        int i, j, k;
        decode(g, r, i, j, k);
        const int t = (int)label[r];
        double* faces[3] = {f0, f1, f2};
        const long long offs[3] = {g.JK, g.K, 1};
        const bool hasp[3] = {i + 1 < g.I, j + 1 < g.J, k + 1 < g.K};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            double cf = 0.0;
            if (hasp[d]) {
                const long long nb = r + offs[d];
                const int tn = (int)label[nb];
                if (t == kPore) cf = link_coeff(label, perm, visc, r, nb);
                else if (tn == kPore) cf = link_coeff(label, perm, visc, nb, r);
            }
            faces[d][r] = cf;
        }
    }
}

// One row of src/Simulation.cpp:674-792: kind, diagonal and right-hand side. The diagonal
// subtracts the six link coefficients in the reference's order (+i, -i, +j, -j, +k, -k),
// read from the stored faces. With the flow-through model (LS_BC_FLOW_I, no counterpart in
// the reference) the Pore voxels of planes i = 0 and i = I-1 are identity rows.
template <typename L>
__device__ __forceinline__ void press_row_eval(const Grid& g, const PressConst& pcst, const L* __restrict__ label,
                                               const double* __restrict__ f0, const double* __restrict__ f1,
                                               const double* __restrict__ f2, long long r, int i, int j, int k,
                                               int8_t& kd, double& dg, double& bv) {
    const int t = (int)label[r];
    kd = 0;
    dg = 0.0;
    bv = 0.0;
    if (t == kAir || t == kRock || t == kSulphide || t == kPrecipitate) {
        kd = 1;
        dg = 1.0;
        if (t == kAir) {
            bool is_surface = (i + 1 < g.I && (int)label[r + g.JK] != kAir) ||
                              (i > 0 && (int)label[r - g.JK] != kAir) ||
                              (j + 1 < g.J && (int)label[r + g.K] != kAir) ||
                              (j > 0 && (int)label[r - g.K] != kAir) ||
                              (k + 1 < g.K && (int)label[r + 1] != kAir) ||
                              (k > 0 && (int)label[r - 1] != kAir);
            bv = 0.0 + (is_surface ? pcst.eff_top : 0.0);
        }
    } else if (t == kPore && pcst.bc_mode == LS_BC_FLOW_I && (i == 0 || i == g.I - 1)) {
        // flow-through model: the Pore voxels of the end planes hold the inlet / outlet pressure
        kd = 1;
        dg = 1.0;
        bv = 0.0 + (i == 0 ? pcst.p_inlet : pcst.p_outlet);
    } else if (t == kPore) {
        double diagonal_term = 0.0, source_term = 0.0;
        const long long nbs[6] = {r + g.JK, r - g.JK, r + g.K, r - g.K, r + 1, r - 1};
        const bool val[6] = {i + 1 < g.I, i > 0, j + 1 < g.J, j > 0, k + 1 < g.K, k > 0};
        const double cf[6] = {val[0] ? f0[r] : 0.0, val[1] ? f0[r - g.JK] : 0.0,
                              val[2] ? f1[r] : 0.0, val[3] ? f1[r - g.K] : 0.0,
                              val[4] ? f2[r] : 0.0, val[5] ? f2[r - 1] : 0.0};
#pragma unroll
        for (int d = 0; d < 6; ++d) {
            if (!val[d]) continue;
            if ((int)label[nbs[d]] == kAir) source_term -= pcst.evap_dx;
            diagonal_term -= cf[d];
        }
        kd = 2;
        if (fabs(diagonal_term) < 1e-16) {
            diagonal_term = 1e-16;
            kd = 3;
        }
        dg = diagonal_term;
        bv = 0.0 + source_term;
    }
}

// Rows pass 1: a row is a pure function of the labels of its voxel and six neighbours, of
// its six faces and of the evaporation constant, plus the ramped boundary pressure on Air
// rows; rows with a dirty voxel in that stencil (face change bits) and all Air rows are listed.
__global__ void __launch_bounds__(kBlock) k_rows_scan(Grid g, const unsigned int* __restrict__ bits, long long nw,
                                                      const uint8_t* __restrict__ label8,
                                                      const uint16_t* __restrict__ label16, int force,
                                                      int* __restrict__ list, unsigned int* __restrict__ count) {
    const int lane = (int)(threadIdx.x & 31u);
    // block-uniform trip count (block_append is called by every thread of the block)
    for (long long b0 = (long long)blockIdx.x * blockDim.x; b0 < g.N; b0 += (long long)gridDim.x * blockDim.x) {
        const long long r0 = b0 + (threadIdx.x & ~31u);
        const long long r = r0 + lane;
        const unsigned int own = dwin(bits, nw, r0);
        const unsigned int km = dwin(bits, nw, r0 - 1), kp = dwin(bits, nw, r0 + 1);
        const unsigned int jm = dwin(bits, nw, r0 - g.K), jp = dwin(bits, nw, r0 + g.K);
        const unsigned int im = dwin(bits, nw, r0 - g.JK), ip = dwin(bits, nw, r0 + g.JK);
        bool d = false;
        if (r < g.N) {
            int i, j, k;
            decode(g, r, i, j, k);
            const int t = label8 ? (int)label8[r] : (int)label16[r];
            d = force || t == kAir || dbit(own, lane) || (i > 0 && dbit(im, lane)) ||
                (i + 1 < g.I && dbit(ip, lane)) || (j > 0 && dbit(jm, lane)) || (j + 1 < g.J && dbit(jp, lane)) ||
                (k > 0 && dbit(km, lane)) || (k + 1 < g.K && dbit(kp, lane));
        }
        block_append(d, (int)r, list, count);
    }
}

// Rows pass 2: the listed rows, their (b/diag)^2 for the norm of the relative residual test
// and 1/|diag| of normal Pore rows (the weights of the scaled residual norm).
template <typename L>
__global__ void __launch_bounds__(kBlock) k_press_setup(Grid g, PressConst pcst, const L* __restrict__ label,
                                                        int8_t* __restrict__ kind, double* __restrict__ diag,
                                                        double* __restrict__ b, double* __restrict__ sb2,
                                                        double* __restrict__ isd,
                                                        const double* __restrict__ f0,
                                                        const double* __restrict__ f1,
                                                        const double* __restrict__ f2,
                                                        const int* __restrict__ list,
                                                        const unsigned int* __restrict__ count) {
    const int n = (int)*count;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int r = list[q];
        int i, j, k;
        decode(g, r, i, j, k);
        int8_t kd;
        double dg, bv;
        press_row_eval(g, pcst, label, f0, f1, f2, r, i, j, k, kd, dg, bv);
        kind[r] = kd;
        diag[r] = dg;
        b[r] = bv;
        double sb = (dg != 0.0) ? bv / dg : bv;
        sb2[r] = sb * sb;
        isd[r] = (kd == 2) ? drcp_nr(-dg) : 0.0;
    }
}

// Rows pass 3: partial sums of (b/diag)^2 over all rows, in a fixed order.
__global__ void __launch_bounds__(kBlock) k_press_den(Grid g, const double* __restrict__ sb2,
                                                      double* __restrict__ partials) {
    double acc[1] = {0.0};
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x)
        acc[0] += sb2[r];
    block_sum_store<1>(acc, partials);
}

// largest diagonal magnitude of the normal Pore rows (for the inner scaling sigma)
__global__ void __launch_bounds__(kBlock) k_press_maxd(Grid g, const int8_t* __restrict__ kind,
                                                       const double* __restrict__ diag,
                                                       double* __restrict__ partials) {
    double m[1] = {0.0};
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x)
        if (kind[r] == 2) m[0] = smax(m[0], -diag[r]);
    block_max_store<1>(m, partials);
}

// Inner operator sigma*M in excess + Laplacian form: e_i = sigma * (links of row i to rows
// that are not normal Pore rows), face c = sigma * link between two normal Pore rows.
// Rows that are not unknowns get e = 1 and no links.
template <typename T>
__global__ void k_inner_setup(Grid g, double sigma, const int8_t* __restrict__ kind,
                              const double* __restrict__ f0, const double* __restrict__ f1,
                              const double* __restrict__ f2, T* __restrict__ e, T* __restrict__ o0,
                              T* __restrict__ o1, T* __restrict__ o2) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, r, i, j, k);
        const bool u = kind[r] == 2;
        double ex = 0.0;
        if (u) {
            if (i > 0 && kind[r - g.JK] != 2) ex += f0[r - g.JK];
            if (j > 0 && kind[r - g.K] != 2) ex += f1[r - g.K];
            if (k > 0 && kind[r - 1] != 2) ex += f2[r - 1];
            if (k + 1 < g.K && kind[r + 1] != 2) ex += f2[r];
            if (j + 1 < g.J && kind[r + g.K] != 2) ex += f1[r];
            if (i + 1 < g.I && kind[r + g.JK] != 2) ex += f0[r];
        }
        e[r] = u ? (T)(sigma * ex) : (T)1;
        o0[r] = (u && i + 1 < g.I && kind[r + g.JK] == 2) ? (T)(sigma * f0[r]) : (T)0;
        o1[r] = (u && j + 1 < g.J && kind[r + g.K] == 2) ? (T)(sigma * f1[r]) : (T)0;
        o2[r] = (u && k + 1 < g.K && kind[r + 1] == 2) ? (T)(sigma * f2[r]) : (T)0;
    }
}

// Pore rows of the initial guess scaled by the ratio of the ramped boundary pressures of
// this solve and the previous one: without evaporative sources the solution is
// proportional to the boundary pressure, so the previous solution scaled is the best
// available starting point (the converged result does not depend on the starting point
// beyond the tolerance).
__global__ void k_press_scale_x(Grid g, const int8_t* __restrict__ kind, double ratio,
                                double* __restrict__ x) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x)
        if (kind[r] >= 2) x[r] *= ratio;
}

// Minimal-residual scaling of the warm start: with u = b - A x_fixed and y = A x_free on the
// Pore rows (x_fixed: identity and empty rows, x_free: Pore rows), the partials of the
// weighted dots (u,u), (u,y), (y,y) in the norm of the outer residual test; s = (u,y)/(y,y)
// minimises ||D^-1 (b - A (x_fixed + s x_free))||.
__global__ void __launch_bounds__(kBlock) k_press_guess_dots(Grid g, const int8_t* __restrict__ kind,
                                                             const double* __restrict__ diag,
                                                             const double* __restrict__ isd,
                                                             const double* __restrict__ b,
                                                             const double* __restrict__ f0,
                                                             const double* __restrict__ f1,
                                                             const double* __restrict__ f2,
                                                             const double* __restrict__ x,
                                                             double* __restrict__ partials) {
    double acc[3] = {0.0, 0.0, 0.0};
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        const int kd = kind[r];
        if (kd < 2) continue;
        int i, j, k;
        decode(g, r, i, j, k);
        double fixed = 0.0, free = diag[r] * x[r];
        const long long nb[6] = {r - g.JK, r - g.K, r - 1, r + 1, r + g.K, r + g.JK};
        const bool val[6] = {i > 0, j > 0, k > 0, k + 1 < g.K, j + 1 < g.J, i + 1 < g.I};
        const double cf[6] = {val[0] ? f0[nb[0]] : 0.0, val[1] ? f1[nb[1]] : 0.0, val[2] ? f2[nb[2]] : 0.0,
                              val[3] ? f2[r] : 0.0, val[4] ? f1[r] : 0.0, val[5] ? f0[r] : 0.0};
#pragma unroll
        for (int d = 0; d < 6; ++d) {
            if (!val[d]) continue;
            const double t = cf[d] * x[nb[d]];
            if (kind[nb[d]] >= 2) free += t;
            else fixed += t;
        }
        const double u = b[r] - fixed;
        const double id2 = (kd == 2) ? isd[r] : 1e16;
        const double w = id2 * id2;
        acc[0] += u * u * w;
        acc[1] += u * free * w;
        acc[2] += free * free * w;
    }
    block_sum_store<3>(acc, partials);
}

// identity rows take their value; other rows keep the warm start.
__global__ void k_press_init_x(Grid g, const int8_t* __restrict__ kind, const double* __restrict__ b,
                               double* __restrict__ x) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x)
        if (kind[r] == 1) x[r] = b[r];
}

// a supplied start on the Pore rows: x = scale * start
__global__ void k_press_start_x(Grid g, const int8_t* __restrict__ kind, const float* __restrict__ start,
                                double scale, double* __restrict__ x) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x)
        if (kind[r] >= 2) x[r] = scale * (double)start[r];
}

// A supplied start is kept only on the strong components (the multigrid's labelling) that
// are anchored to fixed values: a component none of whose cells has a significant excess
// (coupling to identity rows, e > 1e-3 of the row's diagonal) floats on links of ~1e-22 at
// most. Its rows get 0, the value a zero start gives them and the solve leaves there when
// their right-hand side is 0; a start that is not constant on such a component would have
// to be smoothed out through its near-null modes.
template <typename T>
__global__ void k_start_anchor(Grid g, const int* __restrict__ comp, const T* __restrict__ e,
                               const T* __restrict__ w0, const T* __restrict__ w1, const T* __restrict__ w2,
                               uint8_t* __restrict__ anchored) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        const int id = comp[r];
        if (id < 0) continue;
        // the finest-level link arrays carry zero padding, so r - JK etc. are readable
        const double links = (double)w0[r] + (double)w0[r - g.JK] + (double)w1[r] + (double)w1[r - g.K] +
                             (double)w2[r] + (double)w2[r - 1];
        const double ev = (double)e[r];
        if (ev > 1e-3 * (ev + links)) anchored[id] = 1;
    }
}

__global__ void k_start_unanchored(Grid g, const int8_t* __restrict__ kind, const int* __restrict__ comp,
                                   const uint8_t* __restrict__ anchored, double* __restrict__ x) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        if (kind[r] < 2) continue;
        const int id = comp[r];
        if (id < 0 || !anchored[id]) x[r] = 0.0;
    }
}

// Input fields of the learned start for the assembled system: the Pore-row mask, the
// log-permeability (log10 K + 15) / 3, and the fixed values of the identity rows relative
// to the effective top pressure (1 on the Air voxels that carry it, 0 elsewhere)
__global__ void k_press_learned_inputs(Grid g, const int8_t* __restrict__ kind, const double* __restrict__ perm,
                                       const double* __restrict__ b, double inv_top, float* __restrict__ mask,
                                       float* __restrict__ logk, float* __restrict__ bc) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        const int kd = kind[r];
        mask[r] = kd >= 2 ? 1.f : 0.f;
        // FP32 logarithm: the input feeds a BF16 network (an FP64 log10 per voxel made this
        // pass FP64-bound, 2.7 ms at 32 M voxels)
        const double kp = perm[r];
        const float k = kp > 1e-30 ? (float)kp : 1e-30f;
        logk[r] = (log10f(k) + 15.f) * (1.f / 3.f);
        bc[r] = kd == 1 ? (float)(b[r] * inv_top) : 0.f;
    }
}

// (A x)_r for a Pore row: diag x_r + sum_d c_d x_nb, summed in ascending column order.
__device__ __forceinline__ double press_row_apply(const Grid& g, long long r, int i, int j, int k,
                                                  double dg, const double* __restrict__ x,
                                                  const double* __restrict__ f0,
                                                  const double* __restrict__ f1,
                                                  const double* __restrict__ f2) {
    double acc = 0.0;
    if (i > 0) acc += f0[r - g.JK] * x[r - g.JK];
    if (j > 0) acc += f1[r - g.K] * x[r - g.K];
    if (k > 0) acc += f2[r - 1] * x[r - 1];
    acc += dg * x[r];
    if (k + 1 < g.K) acc += f2[r] * x[r + 1];
    if (j + 1 < g.J) acc += f1[r] * x[r + g.K];
    if (i + 1 < g.I) acc += f0[r] * x[r + g.JK];
    return acc;
}

// The same row product with fused multiply-adds, for the residual of the iterative solve
// (one FP64 operation per term instead of two; the residual is not a reference value).
__device__ __forceinline__ double press_row_apply_fma(const Grid& g, long long r, int i, int j, int k,
                                                      double dg, const double* __restrict__ x,
                                                      const double* __restrict__ f0,
                                                      const double* __restrict__ f1,
                                                      const double* __restrict__ f2) {
    double acc = dg * x[r];
    if (i > 0) acc = __fma_rn(f0[r - g.JK], x[r - g.JK], acc);
    if (j > 0) acc = __fma_rn(f1[r - g.K], x[r - g.K], acc);
    if (k > 0) acc = __fma_rn(f2[r - 1], x[r - 1], acc);
    if (k + 1 < g.K) acc = __fma_rn(f2[r], x[r + 1], acc);
    if (j + 1 < g.J) acc = __fma_rn(f1[r], x[r + g.K], acc);
    if (i + 1 < g.I) acc = __fma_rn(f0[r], x[r + g.JK], acc);
    return acc;
}

// Full operator y = A x (test hook; identity rows y = x, empty rows y = 0).
__global__ void k_press_apply_full(Grid g, const int8_t* __restrict__ kind,
                                   const double* __restrict__ diag, const double* __restrict__ f0,
                                   const double* __restrict__ f1, const double* __restrict__ f2,
                                   const double* __restrict__ x, double* __restrict__ y) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        int kd = kind[r];
        if (kd == 0) { y[r] = 0.0; continue; }
        if (kd == 1) { y[r] = x[r]; continue; }
        int i, j, k;
        decode(g, r, i, j, k);
        y[r] = press_row_apply(g, r, i, j, k, diag[r], x, f0, f1, f2);
    }
}

// The residual pass in two parts. k_press_xstat, over all rows: the block maxima of x and -x
// (the log line's min / max), the NaN count of x, and res = 0 on the rows that are not
// unknowns. k_press_resid_list, over the ascending list of the unknowns (kind >= 2, about a
// quarter of the rows): res, (r / diag)^2 and its NaN count. The FP64 row work thus runs in
// warps of unknowns only (a grid-stride pass over all rows issues it for every warp holding
// one unknown). Both write per-block partials (norm, NaN count) into their own halves of one
// array, summed in a fixed order.
__global__ void __launch_bounds__(kBlock) k_press_xstat(Grid g, const int8_t* __restrict__ kind,
                                                        const double* __restrict__ x, double* __restrict__ res,
                                                        double* __restrict__ partials,
                                                        double* __restrict__ partials_max) {
    double acc[2] = {0.0, 0.0};
    long long k0 = kKeyNegInf, k1 = kKeyNegInf;  // maxima of x and -x, as integer keys
    int nans = 0;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        const double xv = x[r];
        if (disnan(xv)) {
            ++nans;
        } else {
            k0 = max(k0, dkey(xv));
            k1 = max(k1, dkey_neg(xv));
        }
        if (kind[r] < 2) res[r] = 0.0;
    }
    acc[1] = (double)nans;
    double mx[2] = {dunkey(k0), dunkey(k1)};
    block_sum_store<2>(acc, partials);
    __syncthreads();
    block_max_store<2>(mx, partials_max);
}

__global__ void __launch_bounds__(kBlock) k_press_resid_list(Grid g, const int8_t* __restrict__ kind,
                                                             const double* __restrict__ diag,
                                                             const double* __restrict__ isd,
                                                             const double* __restrict__ b,
                                                             const double* __restrict__ f0,
                                                             const double* __restrict__ f1,
                                                             const double* __restrict__ f2,
                                                             const double* __restrict__ x,
                                                             const int* __restrict__ list,
                                                             const unsigned int* __restrict__ count,
                                                             double* __restrict__ res,
                                                             double* __restrict__ partials) {
    double acc[2] = {0.0, 0.0};
    const long long n = (long long)*count;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const long long r = list[q];
        const int kd = kind[r];
        int i, j, k;
        decode(g, r, i, j, k);
        const double rv = b[r] - press_row_apply_fma(g, r, i, j, k, diag[r], x, f0, f1, f2);
        // (r / diag)^2 without an FP64 division: 1/|diag| = isd for normal rows
        const double id2 = (kd == 2) ? isd[r] : 1e16;  // floored rows: diag = 1e-16
        const double wr = rv * id2;
        acc[0] = __fma_rn(wr, wr, acc[0]);
        if (disnan(rv)) acc[1] += 1.0;
        res[r] = rv;
    }
    block_sum_store<2>(acc, partials);
}

// Correction for floored rows and the inner right-hand side
//   d_Q = r_Q / diag_Q,  g = sigma (A_SQ d_Q - r_S).
template <typename T>
__global__ void k_press_inner_rhs(Grid g, double sigma, const int8_t* __restrict__ kind,
                                  const double* __restrict__ diag,
                                  const double* __restrict__ res, const double* __restrict__ f0,
                                  const double* __restrict__ f1, const double* __restrict__ f2,
                                  double* __restrict__ delta, T* __restrict__ rhs) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        int kd = kind[r];
        double dq = (kd == 3) ? res[r] / diag[r] : 0.0;
        delta[r] = dq;
        T gv = (T)0;
        if (kd == 2) {
            int i, j, k;
            decode(g, r, i, j, k);
            double acc = 0.0;
            // couplings to floored rows: their correction is d_Q = r_Q / diag_Q
            if (i > 0 && kind[r - g.JK] == 3) acc += f0[r - g.JK] * (res[r - g.JK] / diag[r - g.JK]);
            if (j > 0 && kind[r - g.K] == 3) acc += f1[r - g.K] * (res[r - g.K] / diag[r - g.K]);
            if (k > 0 && kind[r - 1] == 3) acc += f2[r - 1] * (res[r - 1] / diag[r - 1]);
            if (k + 1 < g.K && kind[r + 1] == 3) acc += f2[r] * (res[r + 1] / diag[r + 1]);
            if (j + 1 < g.J && kind[r + g.K] == 3) acc += f1[r] * (res[r + g.K] / diag[r + g.K]);
            if (i + 1 < g.I && kind[r + g.JK] == 3) acc += f0[r] * (res[r + g.JK] / diag[r + g.JK]);
            gv = (T)(sigma * (acc - res[r]));
        }
        rhs[r] = gv;
    }
}

// x += delta (floored rows) and x += inner solution (normal Pore rows), FP64.
template <typename T>
__global__ void k_press_accumulate(Grid g, const int8_t* __restrict__ kind,
                                   const double* __restrict__ delta, const T* __restrict__ xin,
                                   double* __restrict__ x) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        int kd = kind[r];
        if (kd == 3) x[r] += delta[r];
        else if (kd == 2) x[r] += (double)xin[r];
    }
}

// ---------------------------------------------------------------------------
// inner PCG on sigma*M (excess + Laplacian form)

template <typename T>
__device__ __forceinline__ T inner_apply_row(const Grid& g, long long r, int i, int j, int k,
                                             const T* __restrict__ v, const T* __restrict__ e,
                                             const T* __restrict__ w0, const T* __restrict__ w1,
                                             const T* __restrict__ w2) {
    const T vr = v[r];
    T acc = e[r] * vr;
    if (i > 0) acc += w0[r - g.JK] * (vr - v[r - g.JK]);
    if (j > 0) acc += w1[r - g.K] * (vr - v[r - g.K]);
    if (k > 0) acc += w2[r - 1] * (vr - v[r - 1]);
    if (k + 1 < g.K) acc += w2[r] * (vr - v[r + 1]);
    if (j + 1 < g.J) acc += w1[r] * (vr - v[r + g.K]);
    if (i + 1 < g.I) acc += w0[r] * (vr - v[r + g.JK]);
    return acc;
}

// The inner vectors are zero on voxels that are not inner unknowns (kind != 2) and no
// kernel writes them there (the buffers are cleared when allocated), so the inner PCG
// kernels skip those voxels: ~3/4 of the box in a porosity-0.25 medium.

// q = M p, partial (p, q)
template <typename T>
__global__ void __launch_bounds__(kBlock) k_cg_apply(Grid g, const int8_t* __restrict__ kind,
                                                     const T* __restrict__ p,
                                                     const T* __restrict__ e,
                                                     const T* __restrict__ w0,
                                                     const T* __restrict__ w1,
                                                     const T* __restrict__ w2, T* __restrict__ q,
                                                     double* __restrict__ partials) {
    pdl_enter();
    T a = (T)0;  // per-thread partial in the inner precision
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        if (kind[r] != 2) continue;
        int i, j, k;
        decode(g, r, i, j, k);
        T qv = inner_apply_row(g, r, i, j, k, p, e, w0, w1, w2);
        q[r] = qv;
        a += p[r] * qv;
    }
    double acc[1] = {(double)a};
    block_sum_store<1>(acc, partials);
}

// k_cg_apply on pairs of cells (FP32, K even, padded finest-level arrays)
__global__ void __launch_bounds__(kBlock) k_cg_apply0_pair(int N2, int JK2, int K2, const int8_t* __restrict__ kind,
                                                           const float* __restrict__ p, const float* __restrict__ e,
                                                           const float* __restrict__ w0, const float* __restrict__ w1,
                                                           const float* __restrict__ w2, float* __restrict__ q,
                                                           double* __restrict__ partials) {
    pdl_enter();
    float a = 0.f;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < N2; t += gridDim.x * blockDim.x) {
        const char2 kd = reinterpret_cast<const char2*>(kind)[t];
        const bool l0 = kd.x == 2, l1 = kd.y == 2;
        if (!l0 && !l1) continue;
        const float2 qv = m0_apply_pair(t, JK2, K2, e, w0, w1, w2, p);
        const float2 pv = reinterpret_cast<const float2*>(p)[t];
        if (l0) { q[2 * t] = qv.x; a += pv.x * qv.x; }
        if (l1) { q[2 * t + 1] = qv.y; a += pv.y * qv.y; }
    }
    double acc[1] = {(double)a};
    block_sum_store<1>(acc, partials);
}

// x += a p, r -= a q with a = (r,z)/(p,q) (0 when (p,q) <= 0)
template <typename T>
__global__ void k_cg_update(Grid g, const int8_t* __restrict__ kind, const double* __restrict__ scal,
                            const T* __restrict__ p, const T* __restrict__ q, T* __restrict__ x,
                            T* __restrict__ r_) {
    pdl_enter();
    const double pq = scal[SP_PQ];
    const T a = (T)((pq > 0.0) ? scal[SP_RZ] / pq : 0.0);
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        if (kind[r] != 2) continue;
        x[r] += a * p[r];
        r_[r] -= a * q[r];
    }
}

// Jacobi preconditioner: z = r / diag, partial (r, z)
template <typename T>
__global__ void __launch_bounds__(kBlock) k_cg_jacobi(Grid g, const T* __restrict__ invd,
                                                      const T* __restrict__ r_, T* __restrict__ z,
                                                      double* __restrict__ partials) {
    pdl_enter();
    T a = (T)0;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        T rv = r_[r];
        T zv = invd[r] * rv;
        z[r] = zv;
        a += rv * zv;
    }
    double acc[1] = {(double)a};
    block_sum_store<1>(acc, partials);
}

// p = z + b p with b = (r,z)_new / (r,z)_old (fixed preconditioner) or, for the flexible CG
// that the K-cycle needs, b = -(z_new, q) / (p, q) (Notay's FCG(1))
template <typename T>
__global__ void k_cg_dir(Grid g, const int8_t* __restrict__ kind, const double* __restrict__ scal,
                         const T* __restrict__ z, T* __restrict__ p, int flexible) {
    pdl_enter();
    const T beta = (T)(flexible ? ((scal[SP_PQ] > 0.0) ? -scal[SP_ZQ] / scal[SP_PQ] : 0.0)
                                : scal[SP_RZN] / scal[SP_RZ]);
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x)
        if (kind[r] == 2) p[r] = z[r] + beta * p[r];
}

// p = z, x = 0
template <typename T>
__global__ void k_copy_zero(Grid g, const T* __restrict__ a, T* __restrict__ b, T* __restrict__ z) {
    pdl_enter();
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        b[r] = a[r];
        z[r] = (T)0;
    }
}

__global__ void k_set_scalar(double* scal, int dst, int src) {
    pdl_enter();
    scal[dst] = scal[src];
}

template <typename T>
static ls_status inner_alloc(ls_ctx* c) {
    const int is64 = sizeof(T) == 8;
    if (c->inner_is64 == is64) return LS_OK;
    void** arrs[] = {&c->ie, &c->iface[0], &c->iface[1], &c->iface[2], &c->iinvd, &c->inner[0],
                     &c->inner[1], &c->inner[2], &c->inner[3], &c->inner[4]};
    for (int q = 0; q < 10; ++q) l0_free(c, q, arrs[q]);
    c->inner_is64 = -1;
    for (int q = 0; q < 10; ++q) LS_TRY(l0_alloc(c, q, sizeof(T), arrs[q]));
    c->inner_is64 = is64;
    return LS_OK;
}

// Inner PCG: solve sigma*M x = rhs (rhs in inner[1] on entry) until the preconditioned
// residual (r, z) has dropped by tol^2, preconditioned by one multigrid K-cycle (use_mg; the
// cycle is not a fixed linear operator, so the directions follow the flexible CG) or by
// Jacobi. Returns the iterations used in *its.
template <typename T>
static ls_status inner_pcg(ls_ctx* c, bool use_mg, double tol, int max_it, int* its,
                           double* rel_out) {
    T* x = (T*)c->inner[0];
    T* r = (T*)c->inner[1];
    T* z = (T*)c->inner[2];
    T* p = (T*)c->inner[3];
    T* q = (T*)c->inner[4];
    const T* e = (const T*)c->ie;
    const T* w0 = (const T*)c->iface[0];
    const T* w1 = (const T*)c->iface[1];
    const T* w2 = (const T*)c->iface[2];
    const Grid g = c->g;
    const int grid = grid_for(c, g.N);
    const int pgrid = grid_for(c, g.N / 2);
    // z = B r and (r, z) into slot; with the multigrid, also (qv, z) into slot + 1
    auto precondition = [&](int slot, const T* qv) -> ls_status {
        if (use_mg) return mg_precondition<T>(c, (const T*)r, z, qv, slot);
        LS_LAUNCH_PDL(c, k_cg_jacobi<T>, grid, kBlock, 0, g, (const T*)c->iinvd, (const T*)r, z, c->partials);
        return finalize_sum(c, grid, 1, slot);
    };
    // With the learned coarse solver (c->lpc_active) the cycle is checked as it goes: a
    // non-finite, negative or growing (r, z), a direction with (p, q) <= 0, two iterations in
    // a row that reduce (r, z) by less than kLpcSlow, or four that reduce it by less than
    // kLpcSlow^4 end the learned inner solve without a correction and hand the rest of the
    // solve to the plain cycle.
    const double kLpcSlow = 0.64;
    bool learned = use_mg && c->lpc_active;
    int slow = 0;
    double rz_hist[4] = {0.0, 0.0, 0.0, 0.0};  // (r, z) of the last four iterations
    *its = 0;
    *rel_out = 0.0;
    LS_TRY(precondition(SP_RZ, nullptr));
    double rz0 = 0.0;
    LS_TRY(read_scalars(c, SP_RZ, 1, &rz0));
    if (learned && !(rz0 >= 0.0 && rz0 < INFINITY)) {
        learned = false;
        c->lpc_active = 0;
        c->press_fallbacks++;
        LS_TRY(precondition(SP_RZ, nullptr));
        LS_TRY(read_scalars(c, SP_RZ, 1, &rz0));
    }
    if (rz0 != rz0) return set_error(c, LS_NONFINITE, "pressure: NaN in the inner right-hand side");
    if (!(rz0 > 0.0)) {
        LS_CUDA(c, cudaMemsetAsync(x, 0, sizeof(T) * (size_t)g.N, c->stream));
        return LS_OK;
    }
    LS_LAUNCH_PDL(c, k_copy_zero<T>, grid, kBlock, 0, g, (const T*)z, p, x);
    const double target = tol * tol * rz0;
    double rz = rz0;
    for (int it = 0; it < max_it; ++it) {
        {
            Timed tm(c, LS_T_CG_APPLY);
            if (std::is_same<T, float>::value && g.K % 2 == 0)
                LS_LAUNCH_PDL(c, k_cg_apply0_pair, pgrid, kBlock, 0, (int)(g.N / 2), (int)(g.JK / 2), g.K / 2,
                          (const int8_t*)c->pkind, (const float*)p, (const float*)e, (const float*)w0,
                          (const float*)w1, (const float*)w2, (float*)q, c->partials);
            else
                LS_LAUNCH_PDL(c, k_cg_apply<T>, grid, kBlock, 0, g, (const int8_t*)c->pkind, (const T*)p, e, w0, w1,
                          w2, q, c->partials);
            // p in, excess and three own face links, q out
            if (c->timing) c->timer_bytes[LS_T_CG_APPLY] += (double)g.N * 6.0 * sizeof(T);
        }
        LS_TRY(finalize_sum(c, (std::is_same<T, float>::value && g.K % 2 == 0) ? pgrid : grid, 1, SP_PQ));
        LS_LAUNCH_PDL(c, k_cg_update<T>, grid, kBlock, 0, g, (const int8_t*)c->pkind, (const double*)c->scal,
                  (const T*)p, (const T*)q, x, r);
        LS_TRY(precondition(SP_RZN, (const T*)q));
        *its = it + 1;
        double sc[3];
        LS_TRY(read_scalars(c, SP_PQ, 2, sc));  // (p, q) and the new (r, z)
        double pq = sc[0];
        const double rz_prev = rz;
        rz = sc[1];
        if (learned) {
            const bool bad = !(rz >= 0.0 && rz < INFINITY) || !(pq > 0.0) || rz > rz_prev;
            slow = (rz > kLpcSlow * rz_prev) ? slow + 1 : 0;
            const double rz4 = rz_hist[it & 3];  // (r, z) four iterations back (rz0 at it = 3)
            const bool slow4 = it >= 3 && rz > kLpcSlow * kLpcSlow * kLpcSlow * kLpcSlow * (it == 3 ? rz0 : rz4);
            rz_hist[it & 3] = rz;
            if (bad || slow >= 2 || slow4) {
                // Drop the learned iterations' correction and return: the FP64 refinement
                // then runs the plain cycle from the iterate this inner solve started from.
                // (Continuing from the learned iterate is no good: its error carries modes
                // the plain cycle reduces slowly -- measured, 560-610 plain iterations from
                // it against 28 from zero at 338x338x283.)
                c->lpc_active = 0;
                c->press_fallbacks++;
                LS_CUDA(c, cudaMemsetAsync(x, 0, sizeof(T) * (size_t)g.N, c->stream));
                rz = rz0;
                break;
            }
        }
        if (rz != rz) return set_error(c, LS_NONFINITE, "pressure: NaN in inner PCG");
        if (rz <= target || !(pq > 0.0) || rz < 0.0) break;
        LS_LAUNCH_PDL(c, k_cg_dir<T>, grid, kBlock, 0, g, (const int8_t*)c->pkind, (const double*)c->scal,
                  (const T*)z, p, use_mg ? 1 : 0);
        LS_LAUNCH_PDL(c, k_set_scalar, 1, 1, 0, c->scal, SP_RZ, SP_RZN);
    }
    *rel_out = sqrt(std::max(rz, 0.0) / rz0);
    return LS_OK;
}

// ---------------------------------------------------------------------------

ls_status pressure_setup_run(ls_ctx* c, double t) {
    PressConst pcst;
    const double ramp_duration = 3600.0;
    double effective_top_pressure = c->p.top_pressure;
    if (t < ramp_duration)
        effective_top_pressure = c->p.top_pressure * (t / ramp_duration) + 1e-6;
    pcst.eff_top = effective_top_pressure;
    pcst.bc_mode = c->p.bc_mode;
    pcst.p_inlet = c->p.p_inlet;
    pcst.p_outlet = c->p.p_outlet;
    // the pressure scale of the system: the ramped Air pressure, or in the flow-through model
    // the larger end pressure (fixed over time, so warm starts are not rescaled)
    c->p_eff = (c->p.bc_mode == LS_BC_FLOW_I) ? std::max(std::fabs(c->p.p_inlet), std::fabs(c->p.p_outlet))
                                              : effective_top_pressure;
    pcst.evap_dx = c->p.evaporative_flux * c->p.dx;
    const Grid g = c->g;
    const int grid = grid_for(c, g.N);
    const size_t n = (size_t)g.N;
    if (c->lean) {
        // every face and row afresh, in arrays that share memory with the transport's
        LS_TRY(lean_phase(c, kPhasePressure));
        double** rows[] = {&c->pdiag, &c->pb, &c->pface[0], &c->pface[1], &c->pface[2], &c->pisd, &c->pr,
                           &c->pdelta, &c->psb2};
        for (double** q : rows)
            if (!*q) LS_TRY(walloc_t(c, q, n));
        LS_TRY(wlist_all(c));
        if (c->label_bytes == 1)
            LS_LAUNCH(c, k_press_faces<uint8_t>, grid, kBlock, 0, g, (const uint8_t*)c->label, c->perm,
                      c->visc, c->pface[0], c->pface[1], c->pface[2], (const int*)c->wlist,
                      (const unsigned int*)c->wcount);
        else
            LS_LAUNCH(c, k_press_faces<uint16_t>, grid, kBlock, 0, g, (const uint16_t*)c->label, c->perm,
                      c->visc, c->pface[0], c->pface[1], c->pface[2], (const int*)c->wlist,
                      (const unsigned int*)c->wcount);
    } else if (!c->shf_perm) {
        LS_TRY(dalloc(c, &c->shf_label, n * c->label_bytes));
        LS_TRY(dalloc_t(c, &c->shf_perm, n));
        LS_TRY(dalloc_t(c, &c->shf_visc, n));
        LS_TRY(dalloc_t(c, &c->psb2, n));
        c->faces_force = 1;
    }
    const int faces_force = c->faces_force;
    c->faces_force = 0;
    const double rows_bc[3] = {(double)pcst.bc_mode, pcst.p_inlet, pcst.p_outlet};
    const int rows_force = (faces_force || c->rows_evap_dx != pcst.evap_dx ||
                            memcmp(rows_bc, c->rows_bc, sizeof(rows_bc)) != 0) ? 1 : 0;
    if (!c->lean) {
        LS_TRY(wlist_reset(c));
        if (c->label_bytes == 1)
            LS_LAUNCH(c, k_faces_dirty<uint8_t>, grid, kBlock, 0, g, (const uint8_t*)c->label, c->perm, c->visc,
                      (uint8_t*)c->shf_label, c->shf_perm, c->shf_visc, c->dbits, faces_force);
        else
            LS_LAUNCH(c, k_faces_dirty<uint16_t>, grid, kBlock, 0, g, (const uint16_t*)c->label, c->perm, c->visc,
                      (uint16_t*)c->shf_label, c->shf_perm, c->shf_visc, c->dbits, faces_force);
        LS_LAUNCH(c, k_faces_scan, grid, kBlock, 0, g, (const unsigned int*)c->dbits, c->dwords, c->wlist,
                  c->wcount);
        if (c->label_bytes == 1)
            LS_LAUNCH(c, k_press_faces<uint8_t>, grid, kBlock, 0, g, (const uint8_t*)c->label, c->perm,
                      c->visc, c->pface[0], c->pface[1], c->pface[2], (const int*)c->wlist,
                      (const unsigned int*)c->wcount);
        else
            LS_LAUNCH(c, k_press_faces<uint16_t>, grid, kBlock, 0, g, (const uint16_t*)c->label, c->perm,
                      c->visc, c->pface[0], c->pface[1], c->pface[2], (const int*)c->wlist,
                      (const unsigned int*)c->wcount);
        // rows: the same change bits (labels, faces), plus every Air row (boundary pressure)
        LS_CUDA(c, cudaMemsetAsync(c->wcount, 0, sizeof(unsigned int), c->stream));
        LS_LAUNCH(c, k_rows_scan, grid, kBlock, 0, g, (const unsigned int*)c->dbits, c->dwords,
                  c->label_bytes == 1 ? (const uint8_t*)c->label : (const uint8_t*)nullptr,
                  c->label_bytes == 2 ? (const uint16_t*)c->label : (const uint16_t*)nullptr, rows_force, c->wlist,
                  c->wcount);
    }  // lean: the work list still holds every voxel
    if (c->label_bytes == 1)
        LS_LAUNCH(c, k_press_setup<uint8_t>, grid, kBlock, 0, g, pcst, (const uint8_t*)c->label, c->pkind,
                  c->pdiag, c->pb, c->psb2, c->pisd, (const double*)c->pface[0], (const double*)c->pface[1],
                  (const double*)c->pface[2], (const int*)c->wlist, (const unsigned int*)c->wcount);
    else
        LS_LAUNCH(c, k_press_setup<uint16_t>, grid, kBlock, 0, g, pcst, (const uint16_t*)c->label, c->pkind,
                  c->pdiag, c->pb, c->psb2, c->pisd, (const double*)c->pface[0], (const double*)c->pface[1],
                  (const double*)c->pface[2], (const int*)c->wlist, (const unsigned int*)c->wcount);
    c->rows_evap_dx = pcst.evap_dx;
    memcpy(c->rows_bc, rows_bc, sizeof(rows_bc));
    LS_LAUNCH(c, k_press_den, grid, kBlock, 0, g, (const double*)c->psb2, c->partials);
    LS_TRY(finalize_sum(c, grid, 1, SP_DEN));
    // the unknowns, for the residual passes of the solve
    LS_TRY(ordered_list(c, (const int8_t*)c->pkind, 2));
    c->plist_valid = 1;
    c->p_t = t;
    c->p_ready = 1;
    return LS_OK;
}

ls_status pressure_apply_run(ls_ctx* c, const double* xh, double* yh) {
    const size_t bytes = sizeof(double) * (size_t)c->g.N;
    LS_CUDA(c, cudaMemcpyAsync(c->pdelta, xh, bytes, cudaMemcpyHostToDevice, c->stream));
    const int grid = grid_for(c, c->g.N);
    LS_LAUNCH(c, k_press_apply_full, grid, kBlock, 0, c->g, (const int8_t*)c->pkind,
              (const double*)c->pdiag, (const double*)c->pface[0], (const double*)c->pface[1],
              (const double*)c->pface[2], (const double*)c->pdelta, c->pr);
    LS_CUDA(c, cudaMemcpyAsync(yh, c->pr, bytes, cudaMemcpyDeviceToHost, c->stream));
    LS_CUDA(c, cudaStreamSynchronize(c->stream));
    c->p_ready = 1;
    return LS_OK;
}

template <typename T>
static ls_status pressure_solve_t(ls_ctx* c, ls_solve_info* info, const float* start, double start_scale) {
    const Grid g = c->g;
    const int grid = grid_for(c, g.N);
    double* x = c->P + (c->p.compat_shift ? g.JK : 0);
    LS_TRY(inner_alloc<T>(c));
    const bool use_mg = c->p.press_solver != LS_PRESS_JACOBI64;
    double sigma = 1.0;
    bool inner_ready = false;
    {
        Timed tm(c, LS_T_PRESS_SETUP);
        if (start)
            LS_LAUNCH(c, k_press_start_x, grid, kBlock, 0, g, (const int8_t*)c->pkind, start, start_scale, x);
        else if (c->p.evaporative_flux == 0.0 && c->p_eff_prev > 0.0 && c->p_eff != c->p_eff_prev)
            LS_LAUNCH(c, k_press_scale_x, grid, kBlock, 0, g, (const int8_t*)c->pkind,
                      c->p_eff / c->p_eff_prev, x);
        LS_LAUNCH(c, k_press_init_x, grid, kBlock, 0, g, (const int8_t*)c->pkind,
                  (const double*)c->pb, x);
    }
    // the inner operator and the multigrid hierarchy, built on the first sweep that needs
    // them
    auto build_inner = [&]() -> ls_status {
        Timed tm(c, LS_T_PRESS_SETUP);
        LS_LAUNCH(c, k_press_maxd, grid, kBlock, 0, g, (const int8_t*)c->pkind, (const double*)c->pdiag,
                  c->partials);
        LS_TRY(finalize_max(c, grid, 1, S_RED0));
        double maxd = 0.0;
        LS_TRY(read_scalars(c, S_RED0, 1, &maxd));
        sigma = (maxd > 0.0) ? 1.0 / maxd : 1.0;
        LS_LAUNCH(c, k_inner_setup<T>, grid, kBlock, 0, g, sigma, (const int8_t*)c->pkind,
                  (const double*)c->pface[0], (const double*)c->pface[1], (const double*)c->pface[2],
                  (T*)c->ie, (T*)c->iface[0], (T*)c->iface[1], (T*)c->iface[2]);
        LS_TRY(inner_invd<T>(c));
        if (use_mg) LS_TRY(mg_setup<T>(c));
        // the PCG and multigrid kernels skip voxels that are not inner unknowns, which must
        // hold 0 there: clear what earlier solves (with other unknowns) left behind
        for (int v = 0; v < 5; ++v)
            LS_CUDA(c, cudaMemsetAsync(c->inner[v], 0, sizeof(T) * (size_t)g.N, c->stream));
        if (use_mg) LS_TRY(mg_clear<T>(c));
        return LS_OK;
    };
    if (start && use_mg) {
        // build the inner operator and the components now, and keep the start only on the
        // anchored components
        LS_TRY(build_inner());
        inner_ready = true;
        if (!c->start_anchor) LS_TRY(walloc_t(c, &c->start_anchor, (size_t)g.N));
        LS_CUDA(c, cudaMemsetAsync(c->start_anchor, 0, (size_t)g.N, c->stream));
        LS_LAUNCH(c, k_start_anchor<T>, grid, kBlock, 0, g, (const int*)c->comp, (const T*)c->ie,
                  (const T*)c->iface[0], (const T*)c->iface[1], (const T*)c->iface[2], c->start_anchor);
        LS_LAUNCH(c, k_start_unanchored, grid, kBlock, 0, g, (const int8_t*)c->pkind, (const int*)c->comp,
                  (const uint8_t*)c->start_anchor, x);
    }
    double den = 0.0;
    LS_TRY(read_scalars(c, SP_DEN, 1, &den));
    const double rtol = c->p.press_rtol;
    // inner relative tolerance: enough to reach rtol from the current residual, but not
    // below what the inner precision resolves
    const double inner_floor = (sizeof(T) == 4) ? 1e-5 : 1e-13;
    int total_inner = 0, sweeps = 0;
    double rel = 0.0;
    ls_status result = LS_NOT_CONVERGED;
    double* pmax = c->partials + (size_t)kMaxPartials * 4;
    double prev_rel = INFINITY;
    int stagnant = 0;
    const int max_sweeps = 64;
    // A warm start that misses the tolerance is first rescaled by the minimal-residual
    // factor (it recovers the exact solution when only the boundary pressure changed, and
    // drops a start that no longer fits after the labels changed).
    bool rescaled = false;
    for (;;) {
        double sc[2] = {0.0, 0.0};
        {
            Timed tm(c, LS_T_PRESS_OUTER);
            if (!c->plist_valid) {
                LS_TRY(ordered_list(c, (const int8_t*)c->pkind, 2));
                c->plist_valid = 1;
            }
            LS_LAUNCH(c, k_press_xstat, grid, kBlock, 0, g, (const int8_t*)c->pkind, (const double*)x, c->pr,
                      c->partials, pmax);
            LS_LAUNCH(c, k_press_resid_list, grid, kBlock, 0, g, (const int8_t*)c->pkind, (const double*)c->pdiag,
                      (const double*)c->pisd, (const double*)c->pb, (const double*)c->pface[0],
                      (const double*)c->pface[1], (const double*)c->pface[2], (const double*)x,
                      (const int*)c->wlist, (const unsigned int*)c->wcount, c->pr, c->partials + 2 * grid);
            LS_TRY(finalize_sum(c, 2 * grid, 2, SP_NUM));
        }
        LS_TRY(read_scalars(c, SP_NUM, 2, sc));
        if (sc[1] > 0.0 || sc[0] != sc[0]) {
            result = set_error(c, LS_NONFINITE, "pressure: NaN in the FP64 residual");
            rel = NAN;
            break;
        }
        rel = (den > 0.0) ? sqrt(sc[0] / den) : sqrt(sc[0]);
        if (rel <= rtol || (den == 0.0 && sc[0] == 0.0)) { result = LS_OK; break; }
        if (!rescaled && sweeps == 0) {
            rescaled = true;
            double dots[3] = {0.0, 0.0, 0.0};
            {
                Timed tm(c, LS_T_PRESS_OUTER);
                LS_LAUNCH(c, k_press_guess_dots, grid, kBlock, 0, g, (const int8_t*)c->pkind,
                          (const double*)c->pdiag, (const double*)c->pisd, (const double*)c->pb,
                          (const double*)c->pface[0], (const double*)c->pface[1], (const double*)c->pface[2],
                          (const double*)x, c->partials);
                LS_TRY(finalize_sum(c, grid, 3, S_RED0));
            }
            LS_TRY(read_scalars(c, S_RED0, 3, dots));
            if (dots[2] > 0.0 && std::isfinite(dots[1] / dots[2])) {
                const double scale = dots[1] / dots[2];
                // keep the start unless the rescaled one has a smaller residual:
                // ||u - s y||^2 = (u,u) - (u,y)^2/(y,y)
                const double rr_scaled = std::max(dots[0] - dots[1] * scale, 0.0);
                if (rr_scaled < sc[0] && scale != 1.0) {
                    LS_LAUNCH(c, k_press_scale_x, grid, kBlock, 0, g, (const int8_t*)c->pkind, scale, x);
                    continue;
                }
            }
        }
        if (total_inner >= c->p.press_max_it || sweeps >= max_sweeps) break;
        if (rel > 0.5 * prev_rel) {
            if (++stagnant >= 8) break;
        } else {
            stagnant = 0;
        }
        prev_rel = rel;
        sweeps++;
        int its = 0;
        double irel = 0.0;
        if (!inner_ready) {
            ls_status st = build_inner();
            if (st != LS_OK) { result = st; break; }
            inner_ready = true;
        }
        {
            Timed tm(c, LS_T_PRESS_INNER);
            LS_LAUNCH(c, k_press_inner_rhs<T>, grid, kBlock, 0, g, sigma, (const int8_t*)c->pkind,
                      (const double*)c->pdiag, (const double*)c->pr,
                      (const double*)c->pface[0], (const double*)c->pface[1],
                      (const double*)c->pface[2], c->pdelta, (T*)c->inner[1]);
            double tol = std::max(inner_floor, 0.2 * rtol / std::max(rel, 1e-300));
            tol = std::min(tol, 0.5);
            ls_status st = inner_pcg<T>(c, use_mg, tol, c->p.press_max_it - total_inner, &its, &irel);
            if (st != LS_OK) { result = st; break; }
            LS_LAUNCH(c, k_press_accumulate<T>, grid, kBlock, 0, g, (const int8_t*)c->pkind,
                      (const double*)c->pdelta, (const T*)c->inner[0], x);
        }
        total_inner += its;
    }
    // min / max of the solution vector for the log line
    double mm[2] = {0.0, 0.0};
    // k_press_xstat left the block maxima of x and -x in pmax
    LS_LAUNCH(c, k_finalize<true>, 2, kFinalizeThreads, 0, pmax, grid, 2, c->scal + SP_XMAX);
    LS_TRY(read_scalars(c, SP_XMAX, 2, mm));
    if (result == LS_OK) c->p_eff_prev = c->p_eff;
    if (info) {
        info->iterations = total_inner;
        info->outer_iterations = sweeps;
        info->converged = (result == LS_OK) ? 1 : 0;
        info->reason = (result == LS_OK) ? 2 : (result == LS_NONFINITE ? -4 : -3);
        info->rel_residual = rel;
        info->max_value = mm[0];
        info->min_value = -mm[1];
    }
    if (result == LS_NOT_CONVERGED) {
        char buf[160];
        snprintf(buf, sizeof(buf), "pressure: not converged (rel %.3e after %d inner its, %d sweeps)",
                 rel, total_inner, sweeps);
        set_error(c, LS_NOT_CONVERGED, buf);
    }
    return result;
}

ls_status pressure_solve_run(ls_ctx* c, ls_solve_info* info, const float* start, double start_scale) {
    if (!c->p_ready) return set_error(c, LS_BAD_ARG, "pressure system not assembled");
    snap_fence(c, kSnapP);
    // a supplied start is relative to the effective (ramped) top pressure
    const double sc = start ? start_scale * (c->p_eff > 0.0 ? c->p_eff : 1.0) : 0.0;
    if (c->p.press_solver == LS_PRESS_MIXED || c->p.press_solver == LS_PRESS_LEARNED) {
        // the learned coarse solver is on for this solve until the flexible CG stagnates
        c->lpc_active = (c->p.press_solver == LS_PRESS_LEARNED) ? 1 : 0;
        ls_status st = pressure_solve_t<float>(c, info, start, sc);
        c->lpc_active = 0;
        // the solve has read its scalars back, so the network's convolutions have finished
        if (c->p.press_solver == LS_PRESS_LEARNED && lpnet_tc_timeouts() && st == LS_OK)
            st = set_error(c, LS_TIMEOUT, "learned coarse solve: a tensor-core wait gave up");
        return st;
    }
    return pressure_solve_t<double>(c, info, start, sc);
}

ls_status pressure_learned_inputs_run(ls_ctx* c, float* mask, float* logk, float* bc) {
    if (!c->p_ready) return set_error(c, LS_BAD_ARG, "pressure system not assembled");
    const double top = c->p_eff > 0.0 ? c->p_eff : 1.0;
    LS_LAUNCH(c, k_press_learned_inputs, grid_for(c, c->g.N), kBlock, 0, c->g, (const int8_t*)c->pkind,
              (const double*)c->perm, (const double*)c->pb, 1.0 / top, mask, logk, bc);
    LS_CUDA(c, cudaStreamSynchronize(c->stream));
    return LS_OK;
}

}  // namespace ls
