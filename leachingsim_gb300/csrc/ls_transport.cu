// ls_transport.cu - advection-diffusion-reaction transport of
// Simulation::setupConcentrationEqns + solveConc / solveAcid (src/Simulation.cpp:966-1295,
// 2167-2224) and the implicit saturation system of setupSaturationEqns + solveSaturation
// (src/Simulation.cpp:1858-2053), matrix-free.
//
// Transport rows (active code, src/Simulation.cpp:1129-1232):
//   Precipitate: c = c_old (identity); its flux is zeroed
//   Rock: (1/dt + alpha*n_pore) c - alpha * sum_{Pore nb} c_nb = c_old/dt; flux zeroed
//   others (Air, Pore, Sulphide, any other label): 1/dt diagonal plus, per neighbour:
//     Rock nb -> alpha exchange only; else theta-weighted diffusion (D*Dpore_fac to a Pore
//     nb, D otherwise) and upwind advection of q_face = +q_self on + faces, -q_nb on -
//     faces (zero next to Precipitate/Sulphide); explicit (1-theta) part on the RHS.
//   Links to neighbours outside the domain are skipped.
// conc and acid share the matrix (labels and flux are the same for both solves) and are
// solved together by one two-right-hand-side BiCGStab on the Jacobi-scaled system; the
// convergence test ||D^-1 r|| / ||D^-1 b|| is the one PETSc applies to left-Jacobi GMRES.
#include <algorithm>
#include <cmath>
#include <cstdio>

#include "ls_internal.cuh"

namespace ls {

enum {
    ST_BASE = 32,  // per right-hand side q: ST_BASE + 8*q + ...
    ST_RHO = 0,    // (rhat, r)
    ST_RHO_OLD = 1,
    ST_ALPHA = 2,
    ST_OMEGA = 3,
    ST_RV = 4,     // (rhat, v)
    ST_TS = 5,     // (t, s)
    ST_TT = 6,     // (t, t)
    ST_RR = 7      // (r, r)
};
// slot of value v for right-hand side q
__host__ __device__ __forceinline__ int sslot(int q, int v) { return ST_BASE + 8 * q + v; }
// 0/1 activity flags of the right-hand sides live in scal[S_RED0 + 8 + q]
__host__ __device__ __forceinline__ int aslot(int q) { return S_RED0 + 8 + q; }

struct TransConst {
    double inv_dt, theta, alpha, D, Dpore, dx2, dx;
};

// Coefficients of one transport row: diag, off[6] (+i,-i,+j,-j,+k,-k) and the explicit
// right-hand-side part for field f (f may be null). kind: 1 identity, 2 coupled.
template <typename L>
__device__ __forceinline__ int trans_row(const Grid& g, const TransConst& tc,
                                         const L* __restrict__ label,
                                         const double* __restrict__ fx,
                                         const double* __restrict__ fy,
                                         const double* __restrict__ fz, long long r, int i, int j,
                                         int k, double& diag, double off[6],
                                         const double* f0, const double* f1, double rhs[2]) {
    const int t = (int)label[r];
#pragma unroll
    for (int d = 0; d < 6; ++d) off[d] = 0.0;
    if (t == kPrecipitate) {
        diag = 1.0;
        if (f0) rhs[0] = 0.0 + f0[r];
        if (f1) rhs[1] = 0.0 + f1[r];
        return 1;
    }
    const long long nbs[6] = {r + g.JK, r - g.JK, r + g.K, r - g.K, r + 1, r - 1};
    const bool val[6] = {i + 1 < g.I, i > 0, j + 1 < g.J, j > 0, k + 1 < g.K, k > 0};
    if (t == kRock) {
        double dg = tc.inv_dt;
        if (f0) rhs[0] = 0.0 + f0[r] * tc.inv_dt;
        if (f1) rhs[1] = 0.0 + f1[r] * tc.inv_dt;
#pragma unroll
        for (int d = 0; d < 6; ++d) {
            if (val[d] && (int)label[nbs[d]] == kPore) {
                dg += tc.alpha;
                off[d] = -tc.alpha;
            }
        }
        diag = dg;
        return 2;
    }
    double dg = tc.inv_dt;
    double fr0 = 0.0, fr1 = 0.0;
    if (f0) { fr0 = f0[r]; rhs[0] = 0.0 + fr0 * tc.inv_dt; }
    if (f1) { fr1 = f1[r]; rhs[1] = 0.0 + fr1 * tc.inv_dt; }
#pragma unroll
    for (int d = 0; d < 6; ++d) {
        if (!val[d]) continue;
        const long long nb = nbs[d];
        const int nt = (int)label[nb];
        if (nt == kRock) {
            dg += tc.alpha;
            off[d] = -tc.alpha;
            continue;
        }
        double q_face;
        switch (d) {
        case 0: q_face = fx[r]; break;
        case 1: q_face = -fx[nb]; break;
        case 2: q_face = fy[r]; break;
        case 3: q_face = -fy[nb]; break;
        case 4: q_face = fz[r]; break;
        default: q_face = -fz[nb]; break;
        }
        double actual_q_face = (nt == kPrecipitate || nt == kSulphide) ? 0.0 : q_face;
        double D_eff = (nt == kPore) ? tc.Dpore : tc.D;
        double diffusion_coeff = -D_eff / tc.dx2;
        double coeff_neighbor = diffusion_coeff;
        double coeff_self = -diffusion_coeff;
        double adv_coeff = actual_q_face / tc.dx;
        if (adv_coeff > 0) coeff_self += adv_coeff;
        else coeff_neighbor -= adv_coeff;
        off[d] = tc.theta * coeff_neighbor;
        dg += tc.theta * coeff_self;
        if (f0) rhs[0] += (1.0 - tc.theta) * (-(coeff_self * fr0 + coeff_neighbor * f0[nb]));
        if (f1) rhs[1] += (1.0 - tc.theta) * (-(coeff_self * fr1 + coeff_neighbor * f1[nb]));
    }
    diag = dg;
    return 2;
}

struct SatConst {
    double phi_dt, dx, evap;
};

// Coefficients of one implicit-saturation row (src/Simulation.cpp:1877-1958), from the
// saturation before the solve (s).
template <typename L>
__device__ __forceinline__ int sat_row(const Grid& g, const SatConst& sc,
                                       const L* __restrict__ label,
                                       const double* __restrict__ fx,
                                       const double* __restrict__ fy,
                                       const double* __restrict__ fz,
                                       const double* __restrict__ s, long long r, int i, int j,
                                       int k, double& diag, double off[6], double* rhs) {
    const int t = (int)label[r];
#pragma unroll
    for (int d = 0; d < 6; ++d) off[d] = 0.0;
    if (t == kAir || t == kRock || t == kSulphide || t == kPrecipitate) {
        diag = 1.0;
        if (rhs) *rhs = 0.0 + s[r];
        return 1;
    }
    const long long nbs[6] = {r + g.JK, r - g.JK, r + g.K, r - g.K, r + 1, r - 1};
    const bool val[6] = {i + 1 < g.I, i > 0, j + 1 < g.J, j > 0, k + 1 < g.K, k > 0};
    int air_faces = 0;
#pragma unroll
    for (int d = 0; d < 6; ++d)
        if (val[d] && (int)label[nbs[d]] == kAir) air_faces++;
    double evap_sink = (air_faces * sc.evap) / sc.dx;
    const double sr = s[r];
    double coeff_self = sc.phi_dt;
    if (rhs) *rhs = 0.0 + ((sc.phi_dt * sr) - evap_sink);
    const double* fl[3] = {fx, fy, fz};
#pragma unroll
    for (int d = 0; d < 6; ++d) {
        if (!val[d]) continue;
        const double* f = fl[d >> 1];
        double q = (f[r] + f[nbs[d]]) / 2.0;
        double q_face_outward = (d & 1) ? -q : q;
        if (q_face_outward > 0) {
            double v_eff = q_face_outward / smax(sr, 1e-6);
            coeff_self += v_eff / sc.dx;
        } else {
            double v_eff = q_face_outward / smax(s[nbs[d]], 1e-6);
            off[d] = v_eff / sc.dx;
        }
    }
    diag = coeff_self;
    return 2;
}

// Operator descriptor handed to the Krylov kernels.
template <typename L>
struct Op {
    int mode;  // 0 transport, 1 implicit saturation
    Grid g;
    TransConst tc;
    SatConst sc;
    const L* label;
    const double *fx, *fy, *fz, *s;

    __device__ __forceinline__ int row(long long r, int i, int j, int k, double& diag,
                                       double off[6]) const {
        if (mode == 0)
            return trans_row(g, tc, label, fx, fy, fz, r, i, j, k, diag, off, nullptr, nullptr,
                             nullptr);
        return sat_row(g, sc, label, fx, fy, fz, s, r, i, j, k, diag, off, nullptr);
    }
};

// y_q = D^-1 A x_q (or A x_q when unscaled) for nrhs vectors; summed in ascending column
// order.
template <typename L>
__device__ __forceinline__ void op_apply_row(const Op<L>& op, long long r, int i, int j, int k,
                                             const double* const* x, double* yv, int nrhs,
                                             bool unscaled = false, int mask = 3) {
    double dg, off[6];
    op.row(r, i, j, k, dg, off);
    const Grid& g = op.g;
    for (int q = 0; q < nrhs; ++q) {
        if (!((mask >> q) & 1)) continue;
        const double* xv = x[q];
        double acc = 0.0;
        if (i > 0) acc += off[1] * xv[r - g.JK];
        if (j > 0) acc += off[3] * xv[r - g.K];
        if (k > 0) acc += off[5] * xv[r - 1];
        acc += dg * xv[r];
        if (k + 1 < g.K) acc += off[4] * xv[r + 1];
        if (j + 1 < g.J) acc += off[2] * xv[r + g.K];
        if (i + 1 < g.I) acc += off[0] * xv[r + g.JK];
        yv[q] = unscaled ? acc : acc / dg;
    }
}

struct KVec {
    double* b[2];
    double* x[2];
    double* r[2];
    double* rh[2];
    double* p[2];
    double* v[2];
    double* s[2];
    double* t[2];
};

// setup: scaled right-hand sides b~ = D^-1 b and their squared norms. Reads the fields
// only; x is written by k_kry_xid afterwards (with compat_shift x aliases field slots).
template <typename L>
__global__ void __launch_bounds__(kBlock) k_kry_setup(Op<L> op, KVec kv, int nrhs,
                                                      const double* f0, const double* f1,
                                                      double* __restrict__ partials) {
    double acc[2] = {0.0, 0.0};
    const Grid& g = op.g;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, r, i, j, k);
        double dg, off[6], rhs[2] = {0.0, 0.0};
        if (op.mode == 0)
            trans_row(g, op.tc, op.label, op.fx, op.fy, op.fz, r, i, j, k, dg, off, f0, f1, rhs);
        else
            sat_row(g, op.sc, op.label, op.fx, op.fy, op.fz, op.s, r, i, j, k, dg, off, rhs);
        for (int q = 0; q < nrhs; ++q) {
            double bt = rhs[q] / dg;
            kv.b[q][r] = bt;
            acc[q] += bt * bt;
        }
    }
    block_sum_store<2>(acc, partials);
}

// identity rows take their value: x = b~ (Precipitate for transport, inactive labels for
// the implicit saturation)
template <typename L>
__global__ void k_kry_xid(Op<L> op, KVec kv, int nrhs) {
    const Grid& g = op.g;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        int t = (int)op.label[r];
        bool ident = (op.mode == 0) ? (t == kPrecipitate)
                                    : (t == kAir || t == kRock || t == kSulphide || t == kPrecipitate);
        if (ident)
            for (int q = 0; q < nrhs; ++q) kv.x[q][r] = kv.b[q][r];
    }
}

// zero the flux of Rock and Precipitate voxels (src/Simulation.cpp:1134-1149), after the
// solve; no transport row uses the flux of such a voxel
template <typename L>
__global__ void k_zero_solid_flux(Grid g, const L* __restrict__ label, double* __restrict__ fx,
                                  double* __restrict__ fy, double* __restrict__ fz) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        int t = (int)label[r];
        if (t == kRock || t == kPrecipitate) { fx[r] = 0.0; fy[r] = 0.0; fz[r] = 0.0; }
    }
}

// r = b~ - A~ x, rhat = r, p = v = 0; partial (r, r)
template <typename L>
__global__ void __launch_bounds__(kBlock) k_kry_init(Op<L> op, KVec kv, int nrhs,
                                                     double* __restrict__ partials) {
    double acc[2] = {0.0, 0.0};
    const Grid& g = op.g;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, r, i, j, k);
        double y[2];
        const double* xs[2] = {kv.x[0], kv.x[1]};
        op_apply_row(op, r, i, j, k, xs, y, nrhs);
        for (int q = 0; q < nrhs; ++q) {
            double rv = kv.b[q][r] - y[q];
            kv.r[q][r] = rv;
            kv.rh[q][r] = rv;
            kv.p[q][r] = 0.0;
            kv.v[q][r] = 0.0;
            acc[q] += rv * rv;
        }
    }
    block_sum_store<2>(acc, partials);
}

// p = r + beta (p - omega v), beta = (rho/rho_old)(alpha/omega)
__global__ void k_kry_p(Grid g, KVec kv, int nrhs, int mask, const double* __restrict__ scal) {
    double beta[2], omega[2];
    bool act[2];
    for (int q = 0; q < nrhs; ++q) {
        act[q] = (mask >> q) & 1;
        omega[q] = scal[sslot(q, ST_OMEGA)];
        beta[q] = (scal[sslot(q, ST_RHO)] / scal[sslot(q, ST_RHO_OLD)]) *
                  (scal[sslot(q, ST_ALPHA)] / omega[q]);
    }
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x)
        for (int q = 0; q < nrhs; ++q)
            if (act[q]) kv.p[q][r] = kv.r[q][r] + beta[q] * (kv.p[q][r] - omega[q] * kv.v[q][r]);
}

// v = A~ p; partial (rhat, v)
template <typename L>
__global__ void __launch_bounds__(kBlock) k_kry_v(Op<L> op, KVec kv, int nrhs, int mask,
                                                  double* __restrict__ partials) {
    double acc[2] = {0.0, 0.0};
    const Grid& g = op.g;
    bool act[2] = {(mask & 1) != 0, (mask & 2) != 0};
    const double* ps[2] = {kv.p[0], kv.p[1]};
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, r, i, j, k);
        double y[2];
        op_apply_row(op, r, i, j, k, ps, y, nrhs, false, mask);
        for (int q = 0; q < nrhs; ++q) {
            if (!act[q]) continue;
            kv.v[q][r] = y[q];
            acc[q] += kv.rh[q][r] * y[q];
        }
    }
    block_sum_store<2>(acc, partials);
}

// s = r - alpha v (alpha = rho / (rhat, v)), written by this kernel for its own rows.
__global__ void k_kry_s(Grid g, KVec kv, int nrhs, int mask, const double* __restrict__ scal) {
    double alpha[2];
    bool act[2];
    for (int q = 0; q < nrhs; ++q) {
        act[q] = (mask >> q) & 1;
        alpha[q] = scal[sslot(q, ST_RHO)] / scal[sslot(q, ST_RV)];
    }
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x)
        for (int q = 0; q < nrhs; ++q)
            if (act[q]) kv.s[q][r] = kv.r[q][r] - alpha[q] * kv.v[q][r];
}

// t = A~ s; partials (t, s), (t, t)
template <typename L>
__global__ void __launch_bounds__(kBlock) k_kry_t(Op<L> op, KVec kv, int nrhs, int mask,
                                                  double* __restrict__ partials) {
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const Grid& g = op.g;
    bool act[2] = {(mask & 1) != 0, (mask & 2) != 0};
    const double* ss[2] = {kv.s[0], kv.s[1]};
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, r, i, j, k);
        double y[2];
        op_apply_row(op, r, i, j, k, ss, y, nrhs, false, mask);
        for (int q = 0; q < nrhs; ++q) {
            if (!act[q]) continue;
            kv.t[q][r] = y[q];
            acc[2 * q] += y[q] * kv.s[q][r];
            acc[2 * q + 1] += y[q] * y[q];
        }
    }
    block_sum_store<4>(acc, partials);
}

// x += alpha p + omega s; r = s - omega t; partials (rhat, r), (r, r)
__global__ void __launch_bounds__(kBlock) k_kry_x(Grid g, KVec kv, int nrhs, int mask,
                                                  const double* __restrict__ scal,
                                                  double* __restrict__ partials) {
    double alpha[2], omega[2];
    bool act[2] = {false, false};
    for (int q = 0; q < nrhs; ++q) {
        act[q] = (mask >> q) & 1;
        alpha[q] = scal[sslot(q, ST_RHO)] / scal[sslot(q, ST_RV)];
        double tt = scal[sslot(q, ST_TT)];
        omega[q] = (tt > 0.0) ? scal[sslot(q, ST_TS)] / tt : 0.0;
    }
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        for (int q = 0; q < nrhs; ++q) {
            if (!act[q]) continue;
            double sv = kv.s[q][r];
            kv.x[q][r] += alpha[q] * kv.p[q][r] + omega[q] * sv;
            double rv = sv - omega[q] * kv.t[q][r];
            kv.r[q][r] = rv;
            acc[2 * q] += kv.rh[q][r] * rv;
            acc[2 * q + 1] += rv * rv;
        }
    }
    block_sum_store<4>(acc, partials);
}

// Scalar bookkeeping between kernels (one thread).
// phase 0: after init: rho = (r,r) (rhat = r), rho_old = alpha = omega = 1
// phase 1: after v: (rhat, v) from generic slots 10+q
// phase 3: after t: (t, s), (t, t) from generic slots 12+2q, 13+2q
// phase 2: after x: alpha, omega kept for the next p update; rho_old = rho;
//          rho, (r, r) from generic slots 2q, 2q+1
__global__ void k_kry_scalars(double* scal, int nrhs, int phase) {
    for (int q = 0; q < nrhs; ++q) {
        if (phase == 0) {
            scal[sslot(q, ST_RHO)] = scal[sslot(q, ST_RR)];
            scal[sslot(q, ST_RHO_OLD)] = 1.0;
            scal[sslot(q, ST_ALPHA)] = 1.0;
            scal[sslot(q, ST_OMEGA)] = 1.0;
        } else if (phase == 1) {
            scal[sslot(q, ST_RV)] = scal[S_RED0 + 10 + q];
        } else if (phase == 3) {
            scal[sslot(q, ST_TS)] = scal[S_RED0 + 12 + 2 * q];
            scal[sslot(q, ST_TT)] = scal[S_RED0 + 13 + 2 * q];
        } else if (phase == 2) {
            if (scal[aslot(q)] == 0.0) continue;
            double alpha = scal[sslot(q, ST_RHO)] / scal[sslot(q, ST_RV)];
            double tt = scal[sslot(q, ST_TT)];
            double omega = (tt > 0.0) ? scal[sslot(q, ST_TS)] / tt : 0.0;
            scal[sslot(q, ST_ALPHA)] = alpha;
            scal[sslot(q, ST_OMEGA)] = omega;
            scal[sslot(q, ST_RHO_OLD)] = scal[sslot(q, ST_RHO)];
            scal[sslot(q, ST_RHO)] = scal[S_RED0 + 2 * q];
            scal[sslot(q, ST_RR)] = scal[S_RED0 + 2 * q + 1];
        }
    }
}

// min / max of x over the rows
__global__ void __launch_bounds__(kBlock) k_minmax(Grid g, const double* __restrict__ x,
                                                   double* __restrict__ partials) {
    double m[2] = {-INFINITY, -INFINITY};
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        double v = x[r];
        m[0] = smax(m[0], v);
        m[1] = smax(m[1], -v);
    }
    block_max_store<2>(m, partials);
}

// Scaled residual of x: sum (b~ - A~ x)^2 (diagnostic, once per solve)
template <typename L>
__global__ void __launch_bounds__(kBlock) k_kry_resid(Op<L> op, KVec kv, int nrhs,
                                                      double* __restrict__ partials) {
    double acc[2] = {0.0, 0.0};
    const Grid& g = op.g;
    const double* xs[2] = {kv.x[0], kv.x[1]};
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, r, i, j, k);
        double y[2];
        op_apply_row(op, r, i, j, k, xs, y, nrhs);
        for (int q = 0; q < nrhs; ++q) {
            double rv = kv.b[q][r] - y[q];
            acc[q] += rv * rv;
        }
    }
    block_sum_store<2>(acc, partials);
}

static ls_status kry_alloc(ls_ctx* c) {
    for (int q = 0; q < 14; ++q)
        if (!c->tv[q]) LS_TRY(dalloc_t(c, &c->tv[q], (size_t)c->g.N));
    return LS_OK;
}

static ls_status set_scalars(ls_ctx* c, int first, const double* v, int n) {
    for (int q = 0; q < n; ++q) c->h_scal[first + q] = v[q];
    LS_CUDA(c, cudaMemcpyAsync(c->scal + first, c->h_scal + first, sizeof(double) * n,
                               cudaMemcpyHostToDevice, c->stream));
    return LS_OK;
}

// BiCGStab on D^-1 A x = D^-1 b for nrhs right-hand sides (x warm-started in place).
template <typename L>
static ls_status bicgstab(ls_ctx* c, const Op<L>& op, KVec& kv, int nrhs, const double* f0,
                          const double* f1, double rtol, int max_it, ls_solve_info* info[2]) {
    const Grid g = c->g;
    const int grid = grid_for(c, g.N);
    LS_LAUNCH(c, k_kry_setup<L>, grid, kBlock, 0, op, kv, nrhs, f0, f1, c->partials);
    LS_TRY(finalize_sum(c, grid, 2, S_RED0 + 4));
    LS_LAUNCH(c, k_kry_xid<L>, grid, kBlock, 0, op, kv, nrhs);
    LS_LAUNCH(c, k_kry_init<L>, grid, kBlock, 0, op, kv, nrhs, c->partials);
    LS_TRY(finalize_sum(c, grid, 2, S_RED0));
    double h[8];
    LS_TRY(read_scalars(c, S_RED0, 6, h));
    double bn2[2] = {h[4], h[5]}, rr[2] = {h[0], h[1]};
    double act[2] = {0.0, 0.0};
    int its[2] = {0, 0};
    int reason[2] = {0, 0};
    int restarts[2] = {0, 0};
    for (int q = 0; q < nrhs; ++q) {
        if (rr[q] != rr[q] || bn2[q] != bn2[q]) { reason[q] = -4; continue; }
        double tgt = rtol * rtol * bn2[q];
        if (rr[q] <= tgt || rr[q] == 0.0) reason[q] = 2;
        else act[q] = 1.0;
    }
    LS_TRY(set_scalars(c, aslot(0), act, 2));
    double init_rr[2];
    for (int q = 0; q < nrhs; ++q) {
        init_rr[q] = rr[q];
        c->h_scal[sslot(q, ST_RR)] = rr[q];
        LS_CUDA(c, cudaMemcpyAsync(c->scal + sslot(q, ST_RR), c->h_scal + sslot(q, ST_RR),
                                   sizeof(double), cudaMemcpyHostToDevice, c->stream));
    }
    LS_LAUNCH(c, k_kry_scalars, 1, 1, 0, c->scal, nrhs, 0);
    int it = 0;
    while ((act[0] != 0.0 || act[1] != 0.0) && it < max_it) {
        const int mask = (act[0] != 0.0 ? 1 : 0) | (act[1] != 0.0 ? 2 : 0);
        const int nact = (mask & 1) + ((mask >> 1) & 1);
        // label 1 + own flux 3x8 + per live vector: input 8, output 8, rhat (or s) 8
        const double apply_bytes = (double)g.N * (1.0 + 24.0 + 24.0 * nact);
        LS_LAUNCH(c, k_kry_p, grid, kBlock, 0, g, kv, nrhs, mask, (const double*)c->scal);
        {
            Timed tm(c, LS_T_KRY_APPLY);
            LS_LAUNCH(c, k_kry_v<L>, grid, kBlock, 0, op, kv, nrhs, mask, c->partials);
            c->timer_bytes[LS_T_KRY_APPLY] += c->timing ? apply_bytes : 0.0;
        }
        LS_TRY(finalize_sum(c, grid, 2, S_RED0 + 10));
        LS_LAUNCH(c, k_kry_scalars, 1, 1, 0, c->scal, nrhs, 1);
        LS_LAUNCH(c, k_kry_s, grid, kBlock, 0, g, kv, nrhs, mask, (const double*)c->scal);
        {
            Timed tm(c, LS_T_KRY_APPLY);
            LS_LAUNCH(c, k_kry_t<L>, grid, kBlock, 0, op, kv, nrhs, mask, c->partials);
            c->timer_bytes[LS_T_KRY_APPLY] += c->timing ? apply_bytes : 0.0;
        }
        LS_TRY(finalize_sum(c, grid, 4, S_RED0 + 12));
        LS_LAUNCH(c, k_kry_scalars, 1, 1, 0, c->scal, nrhs, 3);
        LS_LAUNCH(c, k_kry_x, grid, kBlock, 0, g, kv, nrhs, mask, (const double*)c->scal, c->partials);
        LS_TRY(finalize_sum(c, grid, 4, S_RED0));
        LS_LAUNCH(c, k_kry_scalars, 1, 1, 0, c->scal, nrhs, 2);
        it++;
        double sc[32];
        LS_TRY(read_scalars(c, ST_BASE, 16, sc));
        bool changed = false;
        for (int q = 0; q < nrhs; ++q) {
            if (act[q] == 0.0) continue;
            its[q] = it;
            double rho = sc[8 * q + ST_RHO], r2 = sc[8 * q + ST_RR], om = sc[8 * q + ST_OMEGA];
            if (r2 != r2 || rho != rho) { reason[q] = -4; act[q] = 0.0; changed = true; continue; }
            if (r2 <= rtol * rtol * bn2[q]) { reason[q] = 2; act[q] = 0.0; changed = true; continue; }
            // breakdown: restart with rhat = r
            if (rho == 0.0 || om == 0.0 || fabs(rho) < 1e-30 * r2) {
                if (++restarts[q] > 20) { reason[q] = -5; act[q] = 0.0; changed = true; continue; }
                reason[q] = 1;  // marker: restart requested
            }
        }
        bool need_restart = false;
        for (int q = 0; q < nrhs; ++q)
            if (reason[q] == 1) { need_restart = true; reason[q] = 0; }
        if (changed) LS_TRY(set_scalars(c, aslot(0), act, 2));
        if (need_restart) {
            LS_LAUNCH(c, k_kry_init<L>, grid, kBlock, 0, op, kv, nrhs, c->partials);
            LS_TRY(finalize_sum(c, grid, 2, S_RED0));
            for (int q = 0; q < nrhs; ++q)
                LS_CUDA(c, cudaMemcpyAsync(c->scal + sslot(q, ST_RR), c->scal + S_RED0 + q,
                                           sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
            LS_LAUNCH(c, k_kry_scalars, 1, 1, 0, c->scal, nrhs, 0);
        }
    }
    for (int q = 0; q < nrhs; ++q)
        if (act[q] != 0.0) reason[q] = -3;
    // final scaled residual and min/max per right-hand side
    LS_LAUNCH(c, k_kry_resid<L>, grid, kBlock, 0, op, kv, nrhs, c->partials);
    LS_TRY(finalize_sum(c, grid, 2, S_RED0));
    double fr[2];
    LS_TRY(read_scalars(c, S_RED0, 2, fr));
    ls_status st = LS_OK;
    for (int q = 0; q < nrhs; ++q) {
        LS_LAUNCH(c, k_minmax, grid, kBlock, 0, g, (const double*)kv.x[q], c->partials);
        LS_TRY(finalize_max(c, grid, 2, S_RED0 + 2));
        double mm[2];
        LS_TRY(read_scalars(c, S_RED0 + 2, 2, mm));
        if (info[q]) {
            info[q]->iterations = its[q];
            info[q]->outer_iterations = restarts[q] + 1;
            info[q]->converged = reason[q] > 0;
            info[q]->reason = reason[q];
            info[q]->rel_residual = bn2[q] > 0.0 ? sqrt(fr[q] / bn2[q]) : sqrt(fr[q]);
            info[q]->max_value = mm[0];
            info[q]->min_value = -mm[1];
        }
        (void)init_rr;
        if (reason[q] == -4) st = set_error(c, LS_NONFINITE, "Krylov solve met NaN/Inf");
        else if (reason[q] <= 0 && st == LS_OK) {
            char buf[128];
            snprintf(buf, sizeof(buf), "Krylov solve not converged in %d iterations", its[q]);
            st = set_error(c, LS_NOT_CONVERGED, buf);
        }
    }
    return st;
}

static KVec make_kvec(ls_ctx* c, double* x0, double* x1) {
    KVec kv;
    for (int q = 0; q < 2; ++q) {
        kv.b[q] = c->tv[7 * q + 0];
        kv.r[q] = c->tv[7 * q + 1];
        kv.rh[q] = c->tv[7 * q + 2];
        kv.p[q] = c->tv[7 * q + 3];
        kv.v[q] = c->tv[7 * q + 4];
        kv.s[q] = c->tv[7 * q + 5];
        kv.t[q] = c->tv[7 * q + 6];
    }
    kv.x[0] = x0;
    kv.x[1] = x1;
    return kv;
}

static TransConst trans_const(const ls_ctx* c, double dt) {
    TransConst tc;
    tc.inv_dt = 1.0 / dt;
    tc.theta = c->p.theta;
    tc.alpha = c->p.alpha_transfer;
    tc.D = c->p.D;
    tc.Dpore = c->p.D * c->p.Dpore_fac;
    tc.dx = c->p.dx;
    tc.dx2 = c->p.dx * c->p.dx;
    return tc;
}

template <typename L>
static ls_status transport_t(ls_ctx* c, double dt, int which, ls_solve_info* ci, ls_solve_info* ai) {
    LS_TRY(kry_alloc(c));
    Op<L> op;
    op.mode = 0;
    op.g = c->g;
    op.tc = trans_const(c, dt);
    op.label = (const L*)c->label;
    op.fx = c->fx; op.fy = c->fy; op.fz = c->fz; op.s = nullptr;
    const long long sh = c->p.compat_shift ? c->g.JK : 0;
    double* fields[2] = {c->conc, c->acid};
    double* f[2];
    ls_solve_info* inf[2];
    int n = 0;
    if (which & 1) { f[n] = fields[0]; inf[n] = ci; n++; }
    if (which & 2) { f[n] = fields[1]; inf[n] = ai; n++; }
    KVec kv = make_kvec(c, f[0] + sh, n > 1 ? f[1] + sh : nullptr);
    ls_status st = bicgstab<L>(c, op, kv, n, f[0], n > 1 ? f[1] : nullptr, c->p.conc_rtol,
                               c->p.conc_max_it, inf);
    if (st != LS_OK && st != LS_NOT_CONVERGED && st != LS_NONFINITE) return st;
    LS_LAUNCH(c, k_zero_solid_flux<L>, grid_for(c, c->g.N), kBlock, 0, c->g, (const L*)c->label,
              c->fx, c->fy, c->fz);
    return st;
}

ls_status transport_run(ls_ctx* c, double dt, int which, ls_solve_info* ci, ls_solve_info* ai) {
    if (c->label_bytes == 1) return transport_t<uint8_t>(c, dt, which, ci, ai);
    return transport_t<uint16_t>(c, dt, which, ci, ai);
}

// test hook: y = A x (unscaled) for the transport operator at dt
template <typename L>
__global__ void k_trans_apply_full(Op<L> op, const double* __restrict__ x, double* __restrict__ y) {
    const Grid& g = op.g;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, r, i, j, k);
        double yv[1];
        const double* xs[1] = {x};
        op_apply_row(op, r, i, j, k, xs, yv, 1, true);
        y[r] = yv[0];
    }
}

template <typename L>
static ls_status transport_apply_t(ls_ctx* c, double dt, const double* xh, double* yh) {
    LS_TRY(kry_alloc(c));
    Op<L> op;
    op.mode = 0;
    op.g = c->g;
    op.tc = trans_const(c, dt);
    op.label = (const L*)c->label;
    op.fx = c->fx; op.fy = c->fy; op.fz = c->fz; op.s = nullptr;
    const size_t bytes = sizeof(double) * (size_t)c->g.N;
    LS_CUDA(c, cudaMemcpyAsync(c->tv[0], xh, bytes, cudaMemcpyHostToDevice, c->stream));
    LS_LAUNCH(c, k_trans_apply_full<L>, grid_for(c, c->g.N), kBlock, 0, op, (const double*)c->tv[0], c->tv[1]);
    LS_CUDA(c, cudaMemcpyAsync(yh, c->tv[1], bytes, cudaMemcpyDeviceToHost, c->stream));
    LS_CUDA(c, cudaStreamSynchronize(c->stream));
    return LS_OK;
}

ls_status transport_apply_run(ls_ctx* c, double dt, const double* x, double* y) {
    if (c->label_bytes == 1) return transport_apply_t<uint8_t>(c, dt, x, y);
    return transport_apply_t<uint16_t>(c, dt, x, y);
}

// ---------------------------------------------------------------------------
// implicit saturation

__global__ void k_clamp_sat(Grid g, double* __restrict__ s) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x)
        s[r] = smax(0.0, smin(1.0, s[r]));
}

template <typename L>
static ls_status sat_implicit_t(ls_ctx* c, double dt, ls_solve_info* info) {
    LS_TRY(kry_alloc(c));
    if (!c->s_old) LS_TRY(dalloc_t(c, &c->s_old, (size_t)c->g.NP));
    LS_CUDA(c, cudaMemcpyAsync(c->s_old, c->sat, sizeof(double) * (size_t)c->g.NP,
                               cudaMemcpyDeviceToDevice, c->stream));
    Op<L> op;
    op.mode = 1;
    op.g = c->g;
    op.sc.phi_dt = c->p.porosity * (1.0 / dt);
    op.sc.dx = c->p.dx;
    op.sc.evap = c->p.evaporative_flux;
    op.label = (const L*)c->label;
    op.fx = c->fx; op.fy = c->fy; op.fz = c->fz; op.s = c->s_old;
    const long long sh = c->p.compat_shift ? c->g.JK : 0;
    KVec kv = make_kvec(c, c->sat + sh, nullptr);
    ls_solve_info loc;
    ls_solve_info* inf[2] = {&loc, nullptr};
    ls_status st = bicgstab<L>(c, op, kv, 1, nullptr, nullptr, c->p.sat_rtol, c->p.sat_max_it, inf);
    if (info) *info = loc;
    if (st != LS_OK && st != LS_NOT_CONVERGED) return st;
    // physics check and clamp over the voxel slots (src/Simulation.cpp:2007-2047)
    bool valid = !(loc.max_value > 1.05 || loc.min_value < -0.05);
    if (valid) LS_LAUNCH(c, k_clamp_sat, grid_for(c, c->g.N), kBlock, 0, c->g, c->sat);
    if (st == LS_NOT_CONVERGED) return st;
    if (!valid) return set_error(c, LS_UNPHYSICAL, "implicit saturation outside [-0.05, 1.05]");
    return LS_OK;
}

ls_status saturation_implicit_run(ls_ctx* c, double dt, ls_solve_info* info) {
    if (c->label_bytes == 1) return sat_implicit_t<uint8_t>(c, dt, info);
    return sat_implicit_t<uint16_t>(c, dt, info);
}

}  // namespace ls
