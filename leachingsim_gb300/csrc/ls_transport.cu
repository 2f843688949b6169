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
// solved together, two right-hand sides per pass.
//
// Solver (GB300 has little FP64 throughput, so FP64 divisions and FP64 Krylov sweeps are
// kept out of the iteration): the FP64 row coefficients and right-hand sides are computed
// once per solve, exactly as the reference assembles them; an FP64 refinement loop forms
// the true residual r = b - A x and its Jacobi-scaled norm ||D^-1 r|| / ||D^-1 b|| (the
// test PETSc applies to left-Jacobi GMRES); each correction comes from an FP32 BiCGStab on
// the unit-diagonal system (D^-1 A) d = D^-1 r with FP32 scaled off-diagonals.
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
    double dc_pore, dc_other;  // -D_eff / dx^2 for a Pore neighbour / any other neighbour
    DxDiv dd;
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
        // -D_eff / dx^2 takes one of two values, evaluated once on the host
        double diffusion_coeff = (nt == kPore) ? tc.dc_pore : tc.dc_other;
        double coeff_neighbor = diffusion_coeff;
        double coeff_self = -diffusion_coeff;
        double adv_coeff = tc.dd.div(actual_q_face);
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
    DxDiv dd;
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
    double evap_sink = sc.dd.div(air_faces * sc.evap);
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
            coeff_self += sc.dd.div(v_eff);
        } else {
            double v_eff = q_face_outward / smax(s[nbs[d]], 1e-6);
            off[d] = sc.dd.div(v_eff);
        }
    }
    diag = coeff_self;
    return 2;
}


// ---------------------------------------------------------------------------
// setup: FP64 coefficients, right-hand sides, FP32 scaled off-diagonals

template <typename L>
struct Rows {
    int mode;  // 0 transport, 1 implicit saturation
    Grid g;
    TransConst tc;
    SatConst sc;
    const L* label;
    const double *fx, *fy, *fz, *s;
};

struct TBuf {
    double* c[7];
    double* b[2];
    float* o[6];
    double* inv;
    int8_t* kind;
};

template <typename L>
__global__ void __launch_bounds__(kBlock) k_t_setup(Rows<L> op, TBuf tb, int nrhs, const double* f0,
                                                    const double* f1, double* __restrict__ partials) {
    double acc[2] = {0.0, 0.0};
    const Grid& g = op.g;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, r, i, j, k);
        double dg, off[6], rhs[2] = {0.0, 0.0};
        int kind;
        if (op.mode == 0)
            kind = trans_row(g, op.tc, op.label, op.fx, op.fy, op.fz, r, i, j, k, dg, off, f0, f1, rhs);
        else
            kind = sat_row(g, op.sc, op.label, op.fx, op.fy, op.fz, op.s, r, i, j, k, dg, off, rhs);
        const double inv = 1.0 / dg;  // the one FP64 division of the row
        tb.c[0][r] = dg;
        tb.inv[r] = inv;
#pragma unroll
        for (int d = 0; d < 6; ++d) {
            tb.c[1 + d][r] = off[d];
            tb.o[d][r] = (float)(off[d] * inv);
        }
        tb.kind[r] = (int8_t)kind;
        for (int q = 0; q < nrhs; ++q) {
            tb.b[q][r] = rhs[q];
            double bt = rhs[q] * inv;
            acc[q] += bt * bt;
        }
    }
    block_sum_store<2>(acc, partials);
}

// identity rows take their value
__global__ void k_t_xid(Grid g, TBuf tb, double* x0, double* x1, int nrhs) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        if (tb.kind[r] != 1) continue;
        x0[r] = tb.b[0][r];
        if (nrhs > 1) x1[r] = tb.b[1][r];
    }
}

// FP64 A x with the stored coefficients, ascending column order
__device__ __forceinline__ double t_row_apply(const Grid& g, const TBuf& tb, long long r, int i, int j,
                                              int k, const double* __restrict__ x) {
    double acc = 0.0;
    if (i > 0) acc = __fma_rn(tb.c[2][r], x[r - g.JK], acc);
    if (j > 0) acc = __fma_rn(tb.c[4][r], x[r - g.K], acc);
    if (k > 0) acc = __fma_rn(tb.c[6][r], x[r - 1], acc);
    acc = __fma_rn(tb.c[0][r], x[r], acc);
    if (k + 1 < g.K) acc = __fma_rn(tb.c[5][r], x[r + 1], acc);
    if (j + 1 < g.J) acc = __fma_rn(tb.c[3][r], x[r + g.K], acc);
    if (i + 1 < g.I) acc = __fma_rn(tb.c[1][r], x[r + g.JK], acc);
    return acc;
}

// outer residual: rhs32 = D^-1 (b - A x) in FP32; partials sum (D^-1 r)^2 and NaN count
__global__ void __launch_bounds__(kBlock) k_t_resid(Grid g, TBuf tb, double* x0, double* x1,
                                                    float* r0, float* r1, int mask,
                                                    double* __restrict__ partials) {
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, r, i, j, k);
        const double inv = tb.inv[r];
        if (mask & 1) {
            double rv = (tb.b[0][r] - t_row_apply(g, tb, r, i, j, k, x0)) * inv;
            r0[r] = (float)rv;
            acc[0] += rv * rv;
            if (rv != rv) acc[2] += 1.0;
        }
        if (mask & 2) {
            double rv = (tb.b[1][r] - t_row_apply(g, tb, r, i, j, k, x1)) * inv;
            r1[r] = (float)rv;
            acc[1] += rv * rv;
            if (rv != rv) acc[3] += 1.0;
        }
    }
    block_sum_store<4>(acc, partials);
}

// ---------------------------------------------------------------------------
// inner FP32 BiCGStab on A^ = I + O (O: scaled off-diagonals), per right-hand side q:
// vectors tf[q] = {rhs, r, rh, p, v, s, t, d}

struct IVec {
    float* v[2][8];
};
enum { IV_RHS = 0, IV_R, IV_RH, IV_P, IV_V, IV_S, IV_T, IV_D };

__device__ __forceinline__ float i_apply(const Grid& g, const TBuf& tb, long long r, int i, int j,
                                         int k, const float* __restrict__ v) {
    float acc = v[r];
    if (i > 0) acc = __fmaf_rn(tb.o[1][r], v[r - g.JK], acc);
    if (j > 0) acc = __fmaf_rn(tb.o[3][r], v[r - g.K], acc);
    if (k > 0) acc = __fmaf_rn(tb.o[5][r], v[r - 1], acc);
    if (k + 1 < g.K) acc = __fmaf_rn(tb.o[4][r], v[r + 1], acc);
    if (j + 1 < g.J) acc = __fmaf_rn(tb.o[2][r], v[r + g.K], acc);
    if (i + 1 < g.I) acc = __fmaf_rn(tb.o[0][r], v[r + g.JK], acc);
    return acc;
}

// start: r = rh = rhs, p = v = d = 0; partial (r, r)
__global__ void __launch_bounds__(kBlock) k_i_init(Grid g, IVec iv, int mask, double* __restrict__ partials) {
    float acc[2] = {0.f, 0.f};
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        for (int q = 0; q < 2; ++q) {
            if (!((mask >> q) & 1)) continue;
            float rv = iv.v[q][IV_RHS][r];
            iv.v[q][IV_R][r] = rv;
            iv.v[q][IV_RH][r] = rv;
            iv.v[q][IV_P][r] = 0.f;
            iv.v[q][IV_V][r] = 0.f;
            iv.v[q][IV_D][r] = 0.f;
            acc[q] = __fmaf_rn(rv, rv, acc[q]);
        }
    }
    double a[2] = {acc[0], acc[1]};
    block_sum_store<2>(a, partials);
}

// p = r + beta (p - omega v)
__global__ void k_i_p(Grid g, IVec iv, int mask, const double* __restrict__ scal) {
    float beta[2] = {0.f, 0.f}, omega[2] = {0.f, 0.f};
    for (int q = 0; q < 2; ++q) {
        if (!((mask >> q) & 1)) continue;
        double om = scal[sslot(q, ST_OMEGA)];
        omega[q] = (float)om;
        beta[q] = (float)((scal[sslot(q, ST_RHO)] / scal[sslot(q, ST_RHO_OLD)]) * (scal[sslot(q, ST_ALPHA)] / om));
    }
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x)
        for (int q = 0; q < 2; ++q)
            if ((mask >> q) & 1)
                iv.v[q][IV_P][r] = __fmaf_rn(beta[q], __fmaf_rn(-omega[q], iv.v[q][IV_V][r], iv.v[q][IV_P][r]),
                                             iv.v[q][IV_R][r]);
}

// v = A^ p; partial (rh, v)
__global__ void __launch_bounds__(kBlock) k_i_v(Grid g, TBuf tb, IVec iv, int mask,
                                                double* __restrict__ partials) {
    float acc[2] = {0.f, 0.f};
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, r, i, j, k);
        for (int q = 0; q < 2; ++q) {
            if (!((mask >> q) & 1)) continue;
            float y = i_apply(g, tb, r, i, j, k, iv.v[q][IV_P]);
            iv.v[q][IV_V][r] = y;
            acc[q] = __fmaf_rn(iv.v[q][IV_RH][r], y, acc[q]);
        }
    }
    double a[2] = {acc[0], acc[1]};
    block_sum_store<2>(a, partials);
}

// s = r - alpha v
__global__ void k_i_s(Grid g, IVec iv, int mask, const double* __restrict__ scal) {
    float alpha[2] = {0.f, 0.f};
    for (int q = 0; q < 2; ++q)
        if ((mask >> q) & 1) alpha[q] = (float)(scal[sslot(q, ST_RHO)] / scal[sslot(q, ST_RV)]);
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x)
        for (int q = 0; q < 2; ++q)
            if ((mask >> q) & 1)
                iv.v[q][IV_S][r] = __fmaf_rn(-alpha[q], iv.v[q][IV_V][r], iv.v[q][IV_R][r]);
}

// t = A^ s; partials (t, s), (t, t)
__global__ void __launch_bounds__(kBlock) k_i_t(Grid g, TBuf tb, IVec iv, int mask,
                                                double* __restrict__ partials) {
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, r, i, j, k);
        for (int q = 0; q < 2; ++q) {
            if (!((mask >> q) & 1)) continue;
            float y = i_apply(g, tb, r, i, j, k, iv.v[q][IV_S]);
            iv.v[q][IV_T][r] = y;
            acc[2 * q] = __fmaf_rn(y, iv.v[q][IV_S][r], acc[2 * q]);
            acc[2 * q + 1] = __fmaf_rn(y, y, acc[2 * q + 1]);
        }
    }
    double a[4] = {acc[0], acc[1], acc[2], acc[3]};
    block_sum_store<4>(a, partials);
}

// d += alpha p + omega s; r = s - omega t; partials (rh, r), (r, r)
__global__ void __launch_bounds__(kBlock) k_i_x(Grid g, IVec iv, int mask, const double* __restrict__ scal,
                                                double* __restrict__ partials) {
    float alpha[2] = {0.f, 0.f}, omega[2] = {0.f, 0.f};
    for (int q = 0; q < 2; ++q) {
        if (!((mask >> q) & 1)) continue;
        alpha[q] = (float)(scal[sslot(q, ST_RHO)] / scal[sslot(q, ST_RV)]);
        double tt = scal[sslot(q, ST_TT)];
        omega[q] = (float)((tt > 0.0) ? scal[sslot(q, ST_TS)] / tt : 0.0);
    }
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        for (int q = 0; q < 2; ++q) {
            if (!((mask >> q) & 1)) continue;
            float sv = iv.v[q][IV_S][r];
            iv.v[q][IV_D][r] = __fmaf_rn(alpha[q], iv.v[q][IV_P][r], __fmaf_rn(omega[q], sv, iv.v[q][IV_D][r]));
            float rv = __fmaf_rn(-omega[q], iv.v[q][IV_T][r], sv);
            iv.v[q][IV_R][r] = rv;
            acc[2 * q] = __fmaf_rn(iv.v[q][IV_RH][r], rv, acc[2 * q]);
            acc[2 * q + 1] = __fmaf_rn(rv, rv, acc[2 * q + 1]);
        }
    }
    double a[4] = {acc[0], acc[1], acc[2], acc[3]};
    block_sum_store<4>(a, partials);
}

// Scalar bookkeeping between kernels (one thread).
// phase 0: after init: rho = (r,r) (rhat = r), rho_old = alpha = omega = 1
// phase 1: after v: (rhat, v) from generic slots 10+q
// phase 3: after t: (t, s), (t, t) from generic slots 12+2q, 13+2q
// phase 2: after x: alpha, omega kept for the next p update; rho_old = rho;
//          rho, (r, r) from generic slots 2q, 2q+1
__global__ void k_kry_scalars(double* scal, int mask, int phase) {
    for (int q = 0; q < 2; ++q) {
        if (!((mask >> q) & 1)) continue;
        if (phase == 0) {
            scal[sslot(q, ST_RHO)] = scal[S_RED0 + q];
            scal[sslot(q, ST_RR)] = scal[S_RED0 + q];
            scal[sslot(q, ST_RHO_OLD)] = 1.0;
            scal[sslot(q, ST_ALPHA)] = 1.0;
            scal[sslot(q, ST_OMEGA)] = 1.0;
        } else if (phase == 1) {
            scal[sslot(q, ST_RV)] = scal[S_RED0 + 10 + q];
        } else if (phase == 3) {
            scal[sslot(q, ST_TS)] = scal[S_RED0 + 12 + 2 * q];
            scal[sslot(q, ST_TT)] = scal[S_RED0 + 13 + 2 * q];
        } else if (phase == 2) {
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

// x += d (FP64 accumulation of the FP32 correction)
__global__ void k_t_accum(Grid g, const float* __restrict__ d0, const float* __restrict__ d1,
                          double* __restrict__ x0, double* __restrict__ x1, int mask) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        if (mask & 1) x0[r] += (double)d0[r];
        if (mask & 2) x1[r] += (double)d1[r];
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

static ls_status t_alloc(ls_ctx* c) {
    const size_t n = (size_t)c->g.N;
    for (int q = 0; q < 7; ++q)
        if (!c->tc[q]) LS_TRY(dalloc_t(c, &c->tc[q], n));
    for (int q = 0; q < 2; ++q)
        if (!c->tb[q]) LS_TRY(dalloc_t(c, &c->tb[q], n));
    for (int q = 0; q < 6; ++q)
        if (!c->to[q]) LS_TRY(dalloc_t(c, &c->to[q], n));
    for (int q = 0; q < 2; ++q)
        for (int v = 0; v < 8; ++v)
            if (!c->tf[q][v]) LS_TRY(dalloc_t(c, &c->tf[q][v], n));
    if (!c->tkind) LS_TRY(dalloc_t(c, &c->tkind, n));
    if (!c->tinv) LS_TRY(dalloc_t(c, &c->tinv, n));
    return LS_OK;
}

static TBuf make_tbuf(ls_ctx* c) {
    TBuf tb;
    for (int q = 0; q < 7; ++q) tb.c[q] = c->tc[q];
    for (int q = 0; q < 2; ++q) tb.b[q] = c->tb[q];
    for (int q = 0; q < 6; ++q) tb.o[q] = c->to[q];
    tb.inv = c->tinv;
    tb.kind = c->tkind;
    return tb;
}

static IVec make_ivec(ls_ctx* c) {
    IVec iv;
    for (int q = 0; q < 2; ++q)
        for (int v = 0; v < 8; ++v) iv.v[q][v] = c->tf[q][v];
    return iv;
}

// Inner FP32 BiCGStab for the right-hand sides in mask; each stops at its own relative
// tolerance tol[q] or on breakdown. Returns the iterations of each.
static ls_status inner_bicgstab(ls_ctx* c, const TBuf& tb, const IVec& iv, int mask, const double tol[2],
                                int max_it, int its[2]) {
    const Grid g = c->g;
    const int grid = grid_for(c, g.N);
    its[0] = its[1] = 0;
    LS_LAUNCH(c, k_i_init, grid, kBlock, 0, g, iv, mask, c->partials);
    LS_TRY(finalize_sum(c, grid, 2, S_RED0));
    LS_LAUNCH(c, k_kry_scalars, 1, 1, 0, c->scal, mask, 0);
    double rr0[2];
    LS_TRY(read_scalars(c, S_RED0, 2, rr0));
    int act = 0;
    for (int q = 0; q < 2; ++q)
        if (((mask >> q) & 1) && rr0[q] > 0.0 && rr0[q] == rr0[q]) act |= 1 << q;
    const double apply_bytes_per_rhs = (double)g.N * 4.0 * (1 + 1 + 1);  // in, out, rh or s
    int it = 0;
    while (act && it < max_it) {
        const int nact = (act & 1) + ((act >> 1) & 1);
        // scaled off-diagonals 6x4 per row + per live vector: input, output, rhat/s
        const double apply_bytes = (double)g.N * 24.0 + apply_bytes_per_rhs * nact;
        LS_LAUNCH(c, k_i_p, grid, kBlock, 0, g, iv, act, (const double*)c->scal);
        {
            Timed tm(c, LS_T_KRY_APPLY);
            LS_LAUNCH(c, k_i_v, grid, kBlock, 0, g, tb, iv, act, c->partials);
            if (c->timing) c->timer_bytes[LS_T_KRY_APPLY] += apply_bytes;
        }
        LS_TRY(finalize_sum(c, grid, 2, S_RED0 + 10));
        LS_LAUNCH(c, k_kry_scalars, 1, 1, 0, c->scal, act, 1);
        LS_LAUNCH(c, k_i_s, grid, kBlock, 0, g, iv, act, (const double*)c->scal);
        {
            Timed tm(c, LS_T_KRY_APPLY);
            LS_LAUNCH(c, k_i_t, grid, kBlock, 0, g, tb, iv, act, c->partials);
            if (c->timing) c->timer_bytes[LS_T_KRY_APPLY] += apply_bytes;
        }
        LS_TRY(finalize_sum(c, grid, 4, S_RED0 + 12));
        LS_LAUNCH(c, k_kry_scalars, 1, 1, 0, c->scal, act, 3);
        LS_LAUNCH(c, k_i_x, grid, kBlock, 0, g, iv, act, (const double*)c->scal, c->partials);
        LS_TRY(finalize_sum(c, grid, 4, S_RED0));
        LS_LAUNCH(c, k_kry_scalars, 1, 1, 0, c->scal, act, 2);
        it++;
        double sc[16];
        LS_TRY(read_scalars(c, ST_BASE, 16, sc));
        for (int q = 0; q < 2; ++q) {
            if (!((act >> q) & 1)) continue;
            its[q] = it;
            double rho = sc[8 * q + ST_RHO], r2 = sc[8 * q + ST_RR], om = sc[8 * q + ST_OMEGA];
            bool done = (r2 <= tol[q] * tol[q] * rr0[q]) || r2 != r2 || rho != rho || rho == 0.0 ||
                        om == 0.0;
            if (done) act &= ~(1 << q);
        }
    }
    return LS_OK;
}

// Mixed-precision solve of the rows in `rows` for nrhs right-hand sides (x warm-started in
// place), fields f0/f1 supplying the right-hand sides.
template <typename L>
static ls_status mixed_solve(ls_ctx* c, const Rows<L>& rows, int nrhs, const double* f0, const double* f1,
                             double* x0, double* x1, double rtol, int max_it, ls_solve_info* info[2]) {
    LS_TRY(t_alloc(c));
    const Grid g = c->g;
    const int grid = grid_for(c, g.N);
    TBuf tb = make_tbuf(c);
    IVec iv = make_ivec(c);
    LS_LAUNCH(c, k_t_setup<L>, grid, kBlock, 0, rows, tb, nrhs, f0, f1, c->partials);
    LS_TRY(finalize_sum(c, grid, 2, S_RED0 + 4));
    LS_LAUNCH(c, k_t_xid, grid, kBlock, 0, g, tb, x0, x1, nrhs);
    double den[2];
    LS_TRY(read_scalars(c, S_RED0 + 4, 2, den));
    int mask = nrhs > 1 ? 3 : 1;
    int its[2] = {0, 0}, sweeps[2] = {0, 0}, reason[2] = {0, 0};
    double rel[2] = {0.0, 0.0}, prev[2] = {INFINITY, INFINITY};
    int stagnant[2] = {0, 0};
    const int max_sweeps = 40;
    while (mask) {
        LS_LAUNCH(c, k_t_resid, grid, kBlock, 0, g, tb, x0, x1, iv.v[0][IV_RHS], iv.v[1][IV_RHS], mask,
                  c->partials);
        LS_TRY(finalize_sum(c, grid, 4, S_RED0));
        double h[4];
        LS_TRY(read_scalars(c, S_RED0, 4, h));
        int solve_mask = 0;
        double tol[2] = {0.5, 0.5};
        for (int q = 0; q < nrhs; ++q) {
            if (!((mask >> q) & 1)) continue;
            if (h[2 + q] > 0.0 || h[q] != h[q]) { reason[q] = -4; rel[q] = NAN; mask &= ~(1 << q); continue; }
            rel[q] = den[q] > 0.0 ? sqrt(h[q] / den[q]) : sqrt(h[q]);
            if (rel[q] <= rtol || h[q] == 0.0) { reason[q] = 2; mask &= ~(1 << q); continue; }
            if (its[q] >= max_it || sweeps[q] >= max_sweeps) { reason[q] = -3; mask &= ~(1 << q); continue; }
            if (rel[q] > 0.5 * prev[q]) {
                if (++stagnant[q] >= 6) { reason[q] = -3; mask &= ~(1 << q); continue; }
            } else {
                stagnant[q] = 0;
            }
            prev[q] = rel[q];
            tol[q] = std::min(0.5, std::max(1e-5, 0.2 * rtol / std::max(rel[q], 1e-300)));
            solve_mask |= 1 << q;
        }
        if (!solve_mask) break;
        int iits[2] = {0, 0};
        int budget = max_it - std::max(its[0], its[1]);
        LS_TRY(inner_bicgstab(c, tb, iv, solve_mask, tol, std::max(budget, 1), iits));
        for (int q = 0; q < 2; ++q)
            if ((solve_mask >> q) & 1) { its[q] += iits[q]; sweeps[q]++; }
        LS_LAUNCH(c, k_t_accum, grid, kBlock, 0, g, iv.v[0][IV_D], iv.v[1][IV_D], x0, x1, solve_mask);
    }
    ls_status st = LS_OK;
    double* xs[2] = {x0, x1};
    for (int q = 0; q < nrhs; ++q) {
        double mm[2] = {0.0, 0.0};
        LS_LAUNCH(c, k_minmax, grid, kBlock, 0, g, (const double*)xs[q], c->partials);
        LS_TRY(finalize_max(c, grid, 2, S_RED0 + 2));
        LS_TRY(read_scalars(c, S_RED0 + 2, 2, mm));
        if (info[q]) {
            info[q]->iterations = its[q];
            info[q]->outer_iterations = sweeps[q];
            info[q]->converged = reason[q] > 0;
            info[q]->reason = reason[q];
            info[q]->rel_residual = rel[q];
            info[q]->max_value = mm[0];
            info[q]->min_value = -mm[1];
        }
        if (reason[q] == -4) st = set_error(c, LS_NONFINITE, "Krylov solve met NaN/Inf");
        else if (reason[q] <= 0 && st == LS_OK) {
            char buf[160];
            snprintf(buf, sizeof(buf), "Krylov solve not converged (rel %.3e after %d its, %d sweeps)",
                     rel[q], its[q], sweeps[q]);
            st = set_error(c, LS_NOT_CONVERGED, buf);
        }
    }
    return st;
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
    tc.dc_pore = -tc.Dpore / tc.dx2;
    tc.dc_other = -tc.D / tc.dx2;
    tc.dd = make_dxdiv(c->p.dx);
    return tc;
}

template <typename L>
static Rows<L> trans_rows(ls_ctx* c, double dt) {
    Rows<L> rows;
    rows.mode = 0;
    rows.g = c->g;
    rows.tc = trans_const(c, dt);
    rows.sc = SatConst{0.0, 1.0, 0.0, make_dxdiv(1.0)};
    rows.label = (const L*)c->label;
    rows.fx = c->fx; rows.fy = c->fy; rows.fz = c->fz; rows.s = nullptr;
    return rows;
}

template <typename L>
static ls_status transport_t(ls_ctx* c, double dt, int which, ls_solve_info* ci, ls_solve_info* ai) {
    Rows<L> rows = trans_rows<L>(c, dt);
    const long long sh = c->p.compat_shift ? c->g.JK : 0;
    double* fields[2] = {c->conc, c->acid};
    double* f[2] = {nullptr, nullptr};
    ls_solve_info* inf[2] = {nullptr, nullptr};
    int n = 0;
    if (which & 1) { f[n] = fields[0]; inf[n] = ci; n++; }
    if (which & 2) { f[n] = fields[1]; inf[n] = ai; n++; }
    ls_status st = mixed_solve<L>(c, rows, n, f[0], f[1], f[0] + sh, n > 1 ? f[1] + sh : nullptr,
                                  c->p.conc_rtol, c->p.conc_max_it, inf);
    if (st != LS_OK && st != LS_NOT_CONVERGED && st != LS_NONFINITE) return st;
    LS_LAUNCH(c, k_zero_solid_flux<L>, grid_for(c, c->g.N), kBlock, 0, c->g, (const L*)c->label,
              c->fx, c->fy, c->fz);
    return st;
}

ls_status transport_run(ls_ctx* c, double dt, int which, ls_solve_info* ci, ls_solve_info* ai) {
    if (c->label_bytes == 1) return transport_t<uint8_t>(c, dt, which, ci, ai);
    return transport_t<uint16_t>(c, dt, which, ci, ai);
}

// test hook: y = A x (unscaled, separate multiply and add like an assembled matrix)
template <typename L>
__global__ void k_trans_apply_full(Rows<L> op, const double* __restrict__ x, double* __restrict__ y) {
    const Grid& g = op.g;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, r, i, j, k);
        double dg, off[6];
        trans_row(g, op.tc, op.label, op.fx, op.fy, op.fz, r, i, j, k, dg, off, nullptr, nullptr, nullptr);
        double acc = 0.0;
        if (i > 0) acc += off[1] * x[r - g.JK];
        if (j > 0) acc += off[3] * x[r - g.K];
        if (k > 0) acc += off[5] * x[r - 1];
        acc += dg * x[r];
        if (k + 1 < g.K) acc += off[4] * x[r + 1];
        if (j + 1 < g.J) acc += off[2] * x[r + g.K];
        if (i + 1 < g.I) acc += off[0] * x[r + g.JK];
        y[r] = acc;
    }
}

template <typename L>
static ls_status transport_apply_t(ls_ctx* c, double dt, const double* xh, double* yh) {
    LS_TRY(t_alloc(c));
    Rows<L> rows = trans_rows<L>(c, dt);
    const size_t bytes = sizeof(double) * (size_t)c->g.N;
    LS_CUDA(c, cudaMemcpyAsync(c->tc[0], xh, bytes, cudaMemcpyHostToDevice, c->stream));
    LS_LAUNCH(c, k_trans_apply_full<L>, grid_for(c, c->g.N), kBlock, 0, rows, (const double*)c->tc[0],
              c->tc[1]);
    LS_CUDA(c, cudaMemcpyAsync(yh, c->tc[1], bytes, cudaMemcpyDeviceToHost, c->stream));
    LS_CUDA(c, cudaStreamSynchronize(c->stream));
    return LS_OK;
}

ls_status transport_apply_run(ls_ctx* c, double dt, const double* x, double* y) {
    if (c->label_bytes == 1) return transport_apply_t<uint8_t>(c, dt, x, y);
    return transport_apply_t<uint16_t>(c, dt, x, y);
}

// ---------------------------------------------------------------------------
// implicit saturation: the coefficients are taken from the saturation before the solve
// (the setup kernel reads every slot before any solution slot is written)

__global__ void k_clamp_sat(Grid g, double* __restrict__ s) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x)
        s[r] = smax(0.0, smin(1.0, s[r]));
}

template <typename L>
static ls_status sat_implicit_t(ls_ctx* c, double dt, ls_solve_info* info) {
    Rows<L> rows;
    rows.mode = 1;
    rows.g = c->g;
    rows.tc = trans_const(c, 1.0);
    rows.sc.phi_dt = c->p.porosity * (1.0 / dt);
    rows.sc.dx = c->p.dx;
    rows.sc.evap = c->p.evaporative_flux;
    rows.sc.dd = make_dxdiv(c->p.dx);
    rows.label = (const L*)c->label;
    rows.fx = c->fx; rows.fy = c->fy; rows.fz = c->fz; rows.s = c->sat;
    const long long sh = c->p.compat_shift ? c->g.JK : 0;
    ls_solve_info loc;
    ls_solve_info* inf[2] = {&loc, nullptr};
    ls_status st = mixed_solve<L>(c, rows, 1, nullptr, nullptr, c->sat + sh, nullptr, c->p.sat_rtol,
                                  c->p.sat_max_it, inf);
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
