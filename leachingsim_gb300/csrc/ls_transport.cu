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
#include <cstring>

#include "ls_internal.cuh"

namespace ls {

struct TransConst {
    double inv_dt, theta, alpha, D, Dpore, dx2, dx;
    double dc_pore, dc_other;  // -D_eff / dx^2 for a Pore neighbour / any other neighbour
    DxDiv dd;
    int inlet;                 // flow-through model: plane i = 0 holds the inflow values
    double in_val[2];          // inflow value of right-hand side 0 / 1
};

// Inflow row of the flow-through model (LS_BC_FLOW_I, no counterpart in the reference): the
// Pore and Air voxels of plane i = 0 hold the inflow value, like the inlet_bc rows of the
// reference's disabled block (src/Simulation.cpp:997-1004).
__device__ __forceinline__ bool inflow_row(const TransConst& tc, int t, int i) {
    return tc.inlet && i == 0 && (t == kPore || t == kAir);
}

// Coefficients of one transport row: diag, off[6] (+i,-i,+j,-j,+k,-k) and the explicit
// right-hand-side part for field f (f may be null). kind: 1 identity holding its old value,
// 2 coupled, 3 identity holding the inflow value.
// EXPL = false is the fully implicit case theta = 1: the theta factors are 1 and the
// explicit part (1 - theta) * (...) adds zero to the right-hand side (for finite fields), so
// both are left out, which takes most of the FP64 work out of the row.
template <typename L, bool EXPL = true>
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
    if (inflow_row(tc, t, i)) {
        diag = 1.0;
        if (f0) rhs[0] = 0.0 + tc.in_val[0];
        if (f1) rhs[1] = 0.0 + tc.in_val[1];
        return 3;
    }
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
        if (dpos(adv_coeff)) coeff_self += adv_coeff;
        else coeff_neighbor -= adv_coeff;
        if (EXPL) {
            off[d] = tc.theta * coeff_neighbor;
            dg += tc.theta * coeff_self;
            if (f0) rhs[0] += (1.0 - tc.theta) * (-(coeff_self * fr0 + coeff_neighbor * f0[nb]));
            if (f1) rhs[1] += (1.0 - tc.theta) * (-(coeff_self * fr1 + coeff_neighbor * f1[nb]));
        } else {
            off[d] = coeff_neighbor;
            dg += coeff_self;
        }
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

template <typename L, bool EXPL>
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
            kind = trans_row<L, EXPL>(g, op.tc, op.label, op.fx, op.fy, op.fz, r, i, j, k, dg, off, f0, f1, rhs);
        else
            kind = sat_row(g, op.sc, op.label, op.fx, op.fy, op.fz, op.s, r, i, j, k, dg, off, rhs);
        // the row scaling (not a reference value): reciprocal without an FP64 division
        const double inv = drcp_nr(dg);
        const float inv32 = d2f_rz(inv);
        tb.c[0][r] = dg;
        tb.inv[r] = inv;
#pragma unroll
        for (int d = 0; d < 6; ++d) {
            tb.c[1 + d][r] = off[d];
            tb.o[d][r] = d2f_rz(off[d]) * inv32;
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

// Change test of the transport-row inputs (pass 1 of the fully implicit setup): the dirty
// bit of voxel r is set when its label or own face fluxes differ bitwise from their values at
// the last setup.
template <typename L>
__global__ void __launch_bounds__(kBlock) k_t_dirty(Grid g, const L* __restrict__ label,
                                                    const double* __restrict__ fx,
                                                    const double* __restrict__ fy,
                                                    const double* __restrict__ fz,
                                                    L* __restrict__ sl, double* __restrict__ sx,
                                                    double* __restrict__ sy, double* __restrict__ sz,
                                                    unsigned int* __restrict__ bits, int force) {
    for (long long r0 = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); r0 < g.N;
         r0 += (long long)gridDim.x * blockDim.x) {
        const long long r = r0 + (threadIdx.x & 31u);
        bool d = false;
        if (r < g.N) {
            const L lab = label[r];
            const long long xb = __double_as_longlong(fx[r]), yb = __double_as_longlong(fy[r]),
                            zb = __double_as_longlong(fz[r]);
            d = force || lab != sl[r] || xb != __double_as_longlong(sx[r]) || yb != __double_as_longlong(sy[r]) ||
                zb != __double_as_longlong(sz[r]);
            if (d) {
                sl[r] = lab;
                sx[r] = __longlong_as_double(xb);
                sy[r] = __longlong_as_double(yb);
                sz[r] = __longlong_as_double(zb);
            }
        }
        const unsigned int w = __ballot_sync(0xffffffffu, d);
        if ((threadIdx.x & 31u) == 0u) bits[r0 >> 5] = w;
    }
}

// Fully implicit (theta = 1) transport setup. A row is a pure function of its own and its
// six neighbours' labels and of its own and its lower neighbours' face fluxes; pass 2 lists
// the rows with a dirty voxel among those, pass 3 recomputes their coefficients, pass 4
// forms the right-hand sides of every row (old value over dt, or the old value on identity
// rows) and the partial norms in a fixed order.
__global__ void __launch_bounds__(kBlock) k_t_scan(Grid g, const unsigned int* __restrict__ bits, long long nw,
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
            d = dbit(own, lane) || (i > 0 && dbit(im, lane)) || (i + 1 < g.I && dbit(ip, lane)) ||
                (j > 0 && dbit(jm, lane)) || (j + 1 < g.J && dbit(jp, lane)) || (k > 0 && dbit(km, lane)) ||
                (k + 1 < g.K && dbit(kp, lane));
        }
        block_append(d, (int)r, list, count);
    }
}

template <typename L>
__global__ void __launch_bounds__(kBlock) k_t_rows(Rows<L> op, TBuf tb, const int* __restrict__ list,
                                                   const unsigned int* __restrict__ count) {
    const Grid& g = op.g;
    const int n = (int)*count;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int r = list[q];
        int i, j, k;
        decode(g, r, i, j, k);
        double dg, off[6], unused[2];
        const int kind = trans_row<L, false>(g, op.tc, op.label, op.fx, op.fy, op.fz, r, i, j, k, dg, off,
                                             nullptr, nullptr, unused);
        const double inv = drcp_nr(dg);
        const float inv32 = d2f_rz(inv);
        tb.c[0][r] = dg;
        tb.inv[r] = inv;
#pragma unroll
        for (int d = 0; d < 6; ++d) {
            tb.c[1 + d][r] = off[d];
            tb.o[d][r] = d2f_rz(off[d]) * inv32;
        }
        tb.kind[r] = (int8_t)kind;
    }
}

// Also counts, per right-hand side, the rows where b or the solution after k_t_xid (b on
// identity rows) is nonzero: a system with none has the exact solution x = 0 already.
__global__ void __launch_bounds__(kBlock) k_t_rhs(Grid g, double inv_dt, double in0, double in1, TBuf tb,
                                                  int nrhs, const double* f0, const double* f1,
                                                  const double* __restrict__ x0, const double* __restrict__ x1,
                                                  double* __restrict__ partials) {
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    unsigned int nz[2] = {0u, 0u};
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < (int)g.N; r += gridDim.x * blockDim.x) {
        const int kind = tb.kind[r];
        const double inv = tb.inv[r];
        for (int q = 0; q < nrhs; ++q) {
            const double fv = (q ? f1 : f0)[r];
            // trans_row's right-hand side at theta = 1: 0.0 + c_old on Precipitate rows,
            // the inflow value on inflow rows, 0.0 + c_old * (1/dt) on every other row
            const double rhs = (kind == 1) ? 0.0 + fv : (kind == 3) ? 0.0 + (q ? in1 : in0) : 0.0 + fv * inv_dt;
            tb.b[q][r] = rhs;
            double bt = rhs * inv;
            acc[q] += bt * bt;
            const double xv = (kind == 1 || kind == 3) ? rhs : (q ? x1 : x0)[r];
            const long long m = 0x7fffffffffffffffll;
            if ((__double_as_longlong(rhs) & m) != 0 || (__double_as_longlong(xv) & m) != 0) nz[q]++;
        }
    }
    acc[2] = (double)nz[0];
    acc[3] = (double)nz[1];
    block_sum_store<4>(acc, partials);
}

__global__ void k_set_ones(double* v) { v[threadIdx.x] = 1.0; }

// identity rows take their value
__global__ void k_t_xid(Grid g, TBuf tb, double* x0, double* x1, int nrhs) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        if (tb.kind[r] != 1 && tb.kind[r] != 3) continue;
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
        // the inner right-hand side in FP32 rounded toward zero on the integer pipe (its
        // rounding is the inner solve's business; the FP64 pipe bounds this pass)
        if (mask & 1) {
            double rv = (tb.b[0][r] - t_row_apply(g, tb, r, i, j, k, x0)) * inv;
            r0[r] = d2f_rz(rv);
            acc[0] = __fma_rn(rv, rv, acc[0]);
            if (disnan(rv)) acc[2] += 1.0;
        }
        if (mask & 2) {
            double rv = (tb.b[1][r] - t_row_apply(g, tb, r, i, j, k, x1)) * inv;
            r1[r] = d2f_rz(rv);
            acc[1] = __fma_rn(rv, rv, acc[1]);
            if (disnan(rv)) acc[3] += 1.0;
        }
    }
    block_sum_store<4>(acc, partials);
}

// ---------------------------------------------------------------------------
// Inner FP32 BiCGStab on A^ = I + O (O: FP32 off-diagonals scaled by the row diagonal), for
// NQ right-hand sides at once. With NQ = 2 both share the off-diagonal loads: each vector
// element is a float2 with one lane per right-hand side. Every vector has `pad` zero
// elements before and after its N rows, so the stencil needs no bounds tests (a link that
// leaves the domain has a zero coefficient, and 0 * 0 adds nothing).
//
// Iteration n, with the per-lane scalars a (alpha), w (omega), b (beta) on the device:
//   XP (n > 0): r = s - w t;  d += a p + w s;  p = r + b (p - w v)
//   V         : v = A^ p (n = 0: p = r);              dots (rh, v)
//   ST        : s = r - a v;  t = A^ s;               dots (t,s) (t,t) (rh,s) (rh,t) (s,s)
// ST recomputes s at the six neighbours from r and v instead of reading a stored s. The
// next rho = (rh, r) = (rh,s) - w (rh,t) and ||r||^2 = (s,s) - 2w (t,s) + w^2 (t,t) come from
// the ST dots, so one iteration takes two reductions. Each reduction's last block updates
// the scalars on the device; kernels return at once when no lane is active, so the host
// launches iterations in batches and reads the state once per batch. The update a p + w s
// still pending after the last iteration goes into the FP64 solution with d.

enum {
    TI_BASE = 64,    // lane l: TI_BASE + TI_STRIDE * l + TI_*
    TI_STRIDE = 16,
    TI_RHO = 0,
    TI_ALPHA,
    TI_OMEGA,
    TI_BETA,
    TI_R2,           // ||r||^2 after the last iteration
    TI_RR0,          // ||r0||^2
    TI_TOL2,         // (relative tolerance)^2
    TI_ACT,          // 1 while the lane iterates
    TI_ITS,
    TI_REASON,       // 1 converged, -1 breakdown, -4 NaN/Inf
    TI_ANY = 100,    // 1 while some lane iterates
    TI_RED = 104     // reduced dots of the last reduction (up to 10)
};
__host__ __device__ __forceinline__ int tslot(int l, int v) { return TI_BASE + TI_STRIDE * l + v; }
static_assert(TI_RED + 10 <= S_COUNT, "transport scalars exceed the scalar block");

enum { PH_INIT = 0, PH_V = 1, PH_ST = 2 };

template <int NQ>
struct Lanes;
template <>
struct Lanes<1> {
    using V = float;
    static __device__ __forceinline__ V zero() { return 0.f; }
    static __device__ __forceinline__ V fma_s(float a, V x, V y) { return __fmaf_rn(a, x, y); }
    static __device__ __forceinline__ V fma_l(V a, V x, V y) { return __fmaf_rn(a, x, y); }
    static __device__ __forceinline__ float lane(V v, int) { return v; }
    static __device__ __forceinline__ V scal(const double* s, int v, float sign) {
        return sign * (float)s[tslot(0, v)];
    }
    static __device__ __forceinline__ V gather(const float* const* f, int r) { return f[0][r]; }
};
template <>
struct Lanes<2> {
    using V = float2;
    static __device__ __forceinline__ V zero() { return make_float2(0.f, 0.f); }
    static __device__ __forceinline__ V fma_s(float a, V x, V y) {
        return make_float2(__fmaf_rn(a, x.x, y.x), __fmaf_rn(a, x.y, y.y));
    }
    static __device__ __forceinline__ V fma_l(V a, V x, V y) {
        return make_float2(__fmaf_rn(a.x, x.x, y.x), __fmaf_rn(a.y, x.y, y.y));
    }
    static __device__ __forceinline__ float lane(V v, int q) { return q ? v.y : v.x; }
    static __device__ __forceinline__ V scal(const double* s, int v, float sign) {
        return make_float2(sign * (float)s[tslot(0, v)], sign * (float)s[tslot(1, v)]);
    }
    static __device__ __forceinline__ V gather(const float* const* f, int r) {
        return make_float2(f[0][r], f[1][r]);
    }
};

// inner vectors: element pointers of row 0 in the active layout (float or float2)
struct TIVec {
    float *r, *rh, *p, *v, *s, *t, *d;
    const float* rhs[2];  // FP32 D^-1 (b - A x) per lane, unpadded
};

struct TOff {
    const float* o[6];  // +i,-i,+j,-j,+k,-k
};

// y = x + sum_d o_d x_nb, neighbours in the order -i, -j, -k, +k, +j, +i
template <int NQ>
__device__ __forceinline__ typename Lanes<NQ>::V ti_apply(const TOff& op, int r, int JK, int K,
                                                          const typename Lanes<NQ>::V* __restrict__ x) {
    using L = Lanes<NQ>;
    typename L::V acc = x[r];
    acc = L::fma_s(__ldg(op.o[1] + r), x[r - JK], acc);
    acc = L::fma_s(__ldg(op.o[3] + r), x[r - K], acc);
    acc = L::fma_s(__ldg(op.o[5] + r), x[r - 1], acc);
    acc = L::fma_s(__ldg(op.o[4] + r), x[r + 1], acc);
    acc = L::fma_s(__ldg(op.o[2] + r), x[r + K], acc);
    acc = L::fma_s(__ldg(op.o[0] + r), x[r + JK], acc);
    return acc;
}

// r = rh = rhs, d = 0, zero halos of r, p, v; dots (r, r)
template <int NQ>
__global__ void __launch_bounds__(kBlock) k_ti_init(int N, int pad, TIVec iv, double* __restrict__ partials) {
    using L = Lanes<NQ>;
    using V = typename L::V;
    V* __restrict__ R = reinterpret_cast<V*>(iv.r);
    V* __restrict__ RH = reinterpret_cast<V*>(iv.rh);
    V* __restrict__ D = reinterpret_cast<V*>(iv.d);
    V* __restrict__ P = reinterpret_cast<V*>(iv.p);
    V* __restrict__ VV = reinterpret_cast<V*>(iv.v);
    float acc[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[q] = 0.f;
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    for (int r = t0; r < N; r += stride) {
        V x = L::gather(iv.rhs, r);
        R[r] = x;
        RH[r] = x;
        D[r] = L::zero();
#pragma unroll
        for (int q = 0; q < NQ; ++q) acc[q] = __fmaf_rn(L::lane(x, q), L::lane(x, q), acc[q]);
    }
    for (int h = t0; h < pad; h += stride) {
        R[-1 - h] = L::zero(); R[N + h] = L::zero();
        P[-1 - h] = L::zero(); P[N + h] = L::zero();
        VV[-1 - h] = L::zero(); VV[N + h] = L::zero();
    }
    double a[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) a[q] = acc[q];
    block_sum_store<NQ>(a, partials);
}

// v = A^ p (FIRST: p = r, stored); dots (rh, v)
template <int NQ, bool FIRST>
__global__ void __launch_bounds__(kBlock) k_ti_v(int N, int JK, int K, TOff op, TIVec iv,
                                                 const double* __restrict__ scal,
                                                 double* __restrict__ partials) {
    pdl_enter();
    if (scal[TI_ANY] == 0.0) return;
    using L = Lanes<NQ>;
    using V = typename L::V;
    const V* __restrict__ X = reinterpret_cast<const V*>(FIRST ? iv.r : iv.p);
    const V* __restrict__ RH = reinterpret_cast<const V*>(iv.rh);
    V* __restrict__ VV = reinterpret_cast<V*>(iv.v);
    V* __restrict__ P = reinterpret_cast<V*>(iv.p);
    float acc[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[q] = 0.f;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < N; r += gridDim.x * blockDim.x) {
        const V y = ti_apply<NQ>(op, r, JK, K, X);
        VV[r] = y;
        if (FIRST) P[r] = X[r];
        const V h = RH[r];
#pragma unroll
        for (int q = 0; q < NQ; ++q) acc[q] = __fmaf_rn(L::lane(h, q), L::lane(y, q), acc[q]);
    }
    double a[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) a[q] = acc[q];
    block_sum_store<NQ>(a, partials);
}

// s = r - a v (at the row and, recomputed, at its neighbours); t = A^ s;
// dots (t,s) (t,t) (rh,s) (rh,t) (s,s) per lane
template <int NQ>
__global__ void __launch_bounds__(kBlock) k_ti_st(int N, int JK, int K, TOff op, TIVec iv,
                                                  const double* __restrict__ scal,
                                                  double* __restrict__ partials) {
    pdl_enter();
    if (scal[TI_ANY] == 0.0) return;
    using L = Lanes<NQ>;
    using V = typename L::V;
    const V* __restrict__ R = reinterpret_cast<const V*>(iv.r);
    const V* __restrict__ VV = reinterpret_cast<const V*>(iv.v);
    const V* __restrict__ RH = reinterpret_cast<const V*>(iv.rh);
    V* __restrict__ S = reinterpret_cast<V*>(iv.s);
    V* __restrict__ T = reinterpret_cast<V*>(iv.t);
    const V na = L::scal(scal, TI_ALPHA, -1.f);
    float acc[5 * NQ];
#pragma unroll
    for (int q = 0; q < 5 * NQ; ++q) acc[q] = 0.f;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < N; r += gridDim.x * blockDim.x) {
        const V s = L::fma_l(na, VV[r], R[r]);
        V t = s;
        t = L::fma_s(__ldg(op.o[1] + r), L::fma_l(na, VV[r - JK], R[r - JK]), t);
        t = L::fma_s(__ldg(op.o[3] + r), L::fma_l(na, VV[r - K], R[r - K]), t);
        t = L::fma_s(__ldg(op.o[5] + r), L::fma_l(na, VV[r - 1], R[r - 1]), t);
        t = L::fma_s(__ldg(op.o[4] + r), L::fma_l(na, VV[r + 1], R[r + 1]), t);
        t = L::fma_s(__ldg(op.o[2] + r), L::fma_l(na, VV[r + K], R[r + K]), t);
        t = L::fma_s(__ldg(op.o[0] + r), L::fma_l(na, VV[r + JK], R[r + JK]), t);
        S[r] = s;
        T[r] = t;
        const V h = RH[r];
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            const float sq = L::lane(s, q), tq = L::lane(t, q), hq = L::lane(h, q);
            acc[5 * q + 0] = __fmaf_rn(tq, sq, acc[5 * q + 0]);
            acc[5 * q + 1] = __fmaf_rn(tq, tq, acc[5 * q + 1]);
            acc[5 * q + 2] = __fmaf_rn(hq, sq, acc[5 * q + 2]);
            acc[5 * q + 3] = __fmaf_rn(hq, tq, acc[5 * q + 3]);
            acc[5 * q + 4] = __fmaf_rn(sq, sq, acc[5 * q + 4]);
        }
    }
    double a[5 * NQ];
#pragma unroll
    for (int q = 0; q < 5 * NQ; ++q) a[q] = acc[q];
    block_sum_store<5 * NQ>(a, partials);
}

// r = s - w t; d += a p + w s; p = r + b (p - w v)
template <int NQ>
__global__ void __launch_bounds__(kBlock) k_ti_xp(int N, TIVec iv, const double* __restrict__ scal) {
    pdl_enter();
    if (scal[TI_ANY] == 0.0) return;
    using L = Lanes<NQ>;
    using V = typename L::V;
    const V* __restrict__ S = reinterpret_cast<const V*>(iv.s);
    const V* __restrict__ T = reinterpret_cast<const V*>(iv.t);
    const V* __restrict__ VV = reinterpret_cast<const V*>(iv.v);
    V* __restrict__ R = reinterpret_cast<V*>(iv.r);
    V* __restrict__ P = reinterpret_cast<V*>(iv.p);
    V* __restrict__ D = reinterpret_cast<V*>(iv.d);
    const V a = L::scal(scal, TI_ALPHA, 1.f);
    const V w = L::scal(scal, TI_OMEGA, 1.f);
    const V nw = L::scal(scal, TI_OMEGA, -1.f);
    const V b = L::scal(scal, TI_BETA, 1.f);
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < N; r += gridDim.x * blockDim.x) {
        const V s = S[r], t = T[r], p = P[r], v = VV[r];
        const V rn = L::fma_l(nw, t, s);
        D[r] = L::fma_l(a, p, L::fma_l(w, s, D[r]));
        R[r] = rn;
        P[r] = L::fma_l(b, L::fma_l(nw, v, p), rn);
    }
}

// Single right-hand side with an even row length K: each thread takes a pair of rows
// (r, r+1), r even, with 8-byte loads (the +-j and +-i neighbours of an even row are even as
// K and J*K are even; the -k neighbour of r and the +k neighbour of r+1 are single loads).
// Same arithmetic per row as k_ti_v / k_ti_st / k_ti_xp, half the load instructions.

__device__ __forceinline__ float2 ti_apply_pair(const TOff& op, int t, int JK2, int K2,
                                                const float* __restrict__ x) {
    const float2* __restrict__ x2 = reinterpret_cast<const float2*>(x);
    const int r = 2 * t;
    const float2 xc = x2[t], xim = x2[t - JK2], xjm = x2[t - K2], xjp = x2[t + K2], xip = x2[t + JK2];
    const float xkm = x[r - 1], xkp = x[r + 2];
    const float2 o0 = __ldg(reinterpret_cast<const float2*>(op.o[0]) + t);
    const float2 o1 = __ldg(reinterpret_cast<const float2*>(op.o[1]) + t);
    const float2 o2 = __ldg(reinterpret_cast<const float2*>(op.o[2]) + t);
    const float2 o3 = __ldg(reinterpret_cast<const float2*>(op.o[3]) + t);
    const float2 o4 = __ldg(reinterpret_cast<const float2*>(op.o[4]) + t);
    const float2 o5 = __ldg(reinterpret_cast<const float2*>(op.o[5]) + t);
    float y0 = xc.x, y1 = xc.y;
    y0 = __fmaf_rn(o1.x, xim.x, y0); y1 = __fmaf_rn(o1.y, xim.y, y1);
    y0 = __fmaf_rn(o3.x, xjm.x, y0); y1 = __fmaf_rn(o3.y, xjm.y, y1);
    y0 = __fmaf_rn(o5.x, xkm, y0);   y1 = __fmaf_rn(o5.y, xc.x, y1);
    y0 = __fmaf_rn(o4.x, xc.y, y0);  y1 = __fmaf_rn(o4.y, xkp, y1);
    y0 = __fmaf_rn(o2.x, xjp.x, y0); y1 = __fmaf_rn(o2.y, xjp.y, y1);
    y0 = __fmaf_rn(o0.x, xip.x, y0); y1 = __fmaf_rn(o0.y, xip.y, y1);
    return make_float2(y0, y1);
}

template <bool FIRST>
__global__ void __launch_bounds__(kBlock) k_ti_v_pair(int N2, int JK2, int K2, TOff op, TIVec iv,
                                                      const double* __restrict__ scal,
                                                      double* __restrict__ partials) {
    pdl_enter();
    if (scal[TI_ANY] == 0.0) return;
    const float* __restrict__ X = FIRST ? iv.r : iv.p;
    const float2* __restrict__ RH = reinterpret_cast<const float2*>(iv.rh);
    float2* __restrict__ VV = reinterpret_cast<float2*>(iv.v);
    float2* __restrict__ P = reinterpret_cast<float2*>(iv.p);
    float acc = 0.f;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < N2; t += gridDim.x * blockDim.x) {
        const float2 y = ti_apply_pair(op, t, JK2, K2, X);
        VV[t] = y;
        if (FIRST) P[t] = reinterpret_cast<const float2*>(X)[t];
        const float2 h = RH[t];
        acc = __fmaf_rn(h.x, y.x, acc);
        acc = __fmaf_rn(h.y, y.y, acc);
    }
    double a[1] = {acc};
    block_sum_store<1>(a, partials);
}

__global__ void __launch_bounds__(kBlock) k_ti_st_pair(int N2, int JK2, int K2, TOff op, TIVec iv,
                                                       const double* __restrict__ scal,
                                                       double* __restrict__ partials) {
    pdl_enter();
    if (scal[TI_ANY] == 0.0) return;
    const float* __restrict__ R = iv.r;
    const float* __restrict__ VV = iv.v;
    const float2* __restrict__ R2 = reinterpret_cast<const float2*>(iv.r);
    const float2* __restrict__ V2 = reinterpret_cast<const float2*>(iv.v);
    const float2* __restrict__ RH = reinterpret_cast<const float2*>(iv.rh);
    float2* __restrict__ S = reinterpret_cast<float2*>(iv.s);
    float2* __restrict__ T = reinterpret_cast<float2*>(iv.t);
    const float na = -(float)scal[tslot(0, TI_ALPHA)];
    float acc[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < N2; t += gridDim.x * blockDim.x) {
        const int r = 2 * t;
        auto s2 = [&](int u) {
            const float2 rv = R2[u], vv = V2[u];
            return make_float2(__fmaf_rn(na, vv.x, rv.x), __fmaf_rn(na, vv.y, rv.y));
        };
        const float2 sc = s2(t), sim = s2(t - JK2), sjm = s2(t - K2), sjp = s2(t + K2), sip = s2(t + JK2);
        const float skm = __fmaf_rn(na, VV[r - 1], R[r - 1]);
        const float skp = __fmaf_rn(na, VV[r + 2], R[r + 2]);
        const float2 o0 = __ldg(reinterpret_cast<const float2*>(op.o[0]) + t);
        const float2 o1 = __ldg(reinterpret_cast<const float2*>(op.o[1]) + t);
        const float2 o2 = __ldg(reinterpret_cast<const float2*>(op.o[2]) + t);
        const float2 o3 = __ldg(reinterpret_cast<const float2*>(op.o[3]) + t);
        const float2 o4 = __ldg(reinterpret_cast<const float2*>(op.o[4]) + t);
        const float2 o5 = __ldg(reinterpret_cast<const float2*>(op.o[5]) + t);
        float t0 = sc.x, t1 = sc.y;
        t0 = __fmaf_rn(o1.x, sim.x, t0); t1 = __fmaf_rn(o1.y, sim.y, t1);
        t0 = __fmaf_rn(o3.x, sjm.x, t0); t1 = __fmaf_rn(o3.y, sjm.y, t1);
        t0 = __fmaf_rn(o5.x, skm, t0);   t1 = __fmaf_rn(o5.y, sc.x, t1);
        t0 = __fmaf_rn(o4.x, sc.y, t0);  t1 = __fmaf_rn(o4.y, skp, t1);
        t0 = __fmaf_rn(o2.x, sjp.x, t0); t1 = __fmaf_rn(o2.y, sjp.y, t1);
        t0 = __fmaf_rn(o0.x, sip.x, t0); t1 = __fmaf_rn(o0.y, sip.y, t1);
        S[t] = sc;
        T[t] = make_float2(t0, t1);
        const float2 h = RH[t];
        acc[0] = __fmaf_rn(t0, sc.x, acc[0]); acc[0] = __fmaf_rn(t1, sc.y, acc[0]);
        acc[1] = __fmaf_rn(t0, t0, acc[1]);   acc[1] = __fmaf_rn(t1, t1, acc[1]);
        acc[2] = __fmaf_rn(h.x, sc.x, acc[2]); acc[2] = __fmaf_rn(h.y, sc.y, acc[2]);
        acc[3] = __fmaf_rn(h.x, t0, acc[3]);  acc[3] = __fmaf_rn(h.y, t1, acc[3]);
        acc[4] = __fmaf_rn(sc.x, sc.x, acc[4]); acc[4] = __fmaf_rn(sc.y, sc.y, acc[4]);
    }
    double a[5] = {acc[0], acc[1], acc[2], acc[3], acc[4]};
    block_sum_store<5>(a, partials);
}

// k_ti_xp on pairs of rows (8-byte loads and stores)
__global__ void __launch_bounds__(kBlock) k_ti_xp_pair(int N2, TIVec iv, const double* __restrict__ scal) {
    pdl_enter();
    if (scal[TI_ANY] == 0.0) return;
    const float2* __restrict__ S = reinterpret_cast<const float2*>(iv.s);
    const float2* __restrict__ T = reinterpret_cast<const float2*>(iv.t);
    const float2* __restrict__ VV = reinterpret_cast<const float2*>(iv.v);
    float2* __restrict__ R = reinterpret_cast<float2*>(iv.r);
    float2* __restrict__ P = reinterpret_cast<float2*>(iv.p);
    float2* __restrict__ D = reinterpret_cast<float2*>(iv.d);
    const float a = (float)scal[tslot(0, TI_ALPHA)];
    const float w = (float)scal[tslot(0, TI_OMEGA)];
    const float b = (float)scal[tslot(0, TI_BETA)];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < N2; t += gridDim.x * blockDim.x) {
        const float2 s = S[t], tt = T[t], p = P[t], v = VV[t], d = D[t];
        const float2 rn = make_float2(__fmaf_rn(-w, tt.x, s.x), __fmaf_rn(-w, tt.y, s.y));
        D[t] = make_float2(__fmaf_rn(a, p.x, __fmaf_rn(w, s.x, d.x)), __fmaf_rn(a, p.y, __fmaf_rn(w, s.y, d.y)));
        R[t] = rn;
        P[t] = make_float2(__fmaf_rn(b, __fmaf_rn(-w, v.x, p.x), rn.x), __fmaf_rn(b, __fmaf_rn(-w, v.y, p.y), rn.y));
    }
}

// x_lane += d + a p + w s (the pending update of the last iteration)
template <int NQ>
__global__ void k_ti_accum(int N, TIVec iv, const double* __restrict__ scal, double* __restrict__ x0,
                           double* __restrict__ x1) {
    using L = Lanes<NQ>;
    using V = typename L::V;
    const V* __restrict__ S = reinterpret_cast<const V*>(iv.s);
    const V* __restrict__ P = reinterpret_cast<const V*>(iv.p);
    const V* __restrict__ D = reinterpret_cast<const V*>(iv.d);
    float a[NQ], w[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        a[q] = (float)scal[tslot(q, TI_ALPHA)];
        w[q] = (float)scal[tslot(q, TI_OMEGA)];
    }
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < N; r += gridDim.x * blockDim.x) {
        const V d = D[r];
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            float inc = L::lane(d, q);
            if (w[q] != 0.f) inc = __fmaf_rn(w[q], L::lane(S[r], q), inc);
            if (a[q] != 0.f) inc = __fmaf_rn(a[q], L::lane(P[r], q), inc);
            double* x = q ? x1 : x0;
            x[r] += (double)inc;
        }
    }
}

__device__ __forceinline__ bool finite_d(double v) { return v == v && fabs(v) < INFINITY; }

// scalar update after a reduction (one thread)
template <int PH, int NQ>
__device__ void ti_phase(double* scal, const double* red, double tol2_0, double tol2_1) {
    int any = 0;
#pragma unroll
    for (int l = 0; l < NQ; ++l) {
        double* s = scal + tslot(l, 0);
        if (PH == PH_INIT) {
            const double rr = red[l];
            s[TI_RR0] = rr;
            s[TI_RHO] = rr;
            s[TI_R2] = rr;
            s[TI_TOL2] = l ? tol2_1 : tol2_0;
            s[TI_ALPHA] = s[TI_OMEGA] = s[TI_BETA] = 0.0;
            s[TI_ITS] = 0.0;
            const bool ok = finite_d(rr) && rr > 0.0;
            s[TI_ACT] = ok ? 1.0 : 0.0;
            s[TI_REASON] = ok ? 0.0 : (finite_d(rr) ? 1.0 : -4.0);
        } else if (PH == PH_V) {
            if (s[TI_ACT] != 0.0) {
                const double rv = red[l];
                if (rv != 0.0 && finite_d(rv)) {
                    s[TI_ALPHA] = s[TI_RHO] / rv;
                } else {
                    s[TI_ACT] = 0.0;
                    s[TI_REASON] = finite_d(rv) ? -1.0 : -4.0;
                    s[TI_ALPHA] = s[TI_OMEGA] = s[TI_BETA] = 0.0;
                }
            } else {
                s[TI_ALPHA] = s[TI_OMEGA] = s[TI_BETA] = 0.0;
            }
        } else {  // PH_ST
            if (s[TI_ACT] != 0.0) {
                const double ts = red[5 * l + 0], tt = red[5 * l + 1], hs = red[5 * l + 2],
                             ht = red[5 * l + 3], ss = red[5 * l + 4];
                const double w = (tt > 0.0) ? ts / tt : 0.0;
                const double rho = hs - w * ht;
                const double r2 = fmax(ss - 2.0 * w * ts + w * w * tt, 0.0);
                s[TI_ITS] += 1.0;
                s[TI_OMEGA] = w;
                s[TI_R2] = r2;
                if (!(finite_d(w) && finite_d(rho) && finite_d(r2) && finite_d(s[TI_ALPHA]))) {
                    s[TI_ACT] = 0.0;
                    s[TI_REASON] = -4.0;
                    s[TI_ALPHA] = s[TI_OMEGA] = s[TI_BETA] = 0.0;
                } else if (r2 <= s[TI_TOL2] * s[TI_RR0]) {
                    s[TI_ACT] = 0.0;
                    s[TI_REASON] = 1.0;
                    s[TI_BETA] = 0.0;
                } else if (w == 0.0 || rho == 0.0) {
                    s[TI_ACT] = 0.0;
                    s[TI_REASON] = -1.0;
                    s[TI_BETA] = 0.0;
                } else {
                    s[TI_BETA] = (rho / s[TI_RHO]) * (s[TI_ALPHA] / w);
                    s[TI_RHO] = rho;
                }
            } else {
                s[TI_ALPHA] = s[TI_OMEGA] = s[TI_BETA] = 0.0;
            }
        }
        if (s[TI_ACT] != 0.0) any = 1;
    }
    scal[TI_ANY] = any ? 1.0 : 0.0;
}

// Fixed-order reduction of the per-block partials, one block per value (as k_finalize);
// the last block to finish applies the scalar update of phase PH.
template <int PH, int NQ>
__global__ void __launch_bounds__(kFinalizeThreads) k_ti_fin(const double* __restrict__ partials, int nblocks,
                                                             double* scal, unsigned int* counter,
                                                             double tol2_0, double tol2_1) {
    pdl_enter();
    if (PH != PH_INIT && scal[TI_ANY] == 0.0) return;
    constexpr int NV = (PH == PH_ST) ? 5 * NQ : NQ;
    __shared__ double sh[kFinalizeThreads];
    __shared__ bool last;
    const int v = blockIdx.x;
    double acc = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) acc += partials[(size_t)b * NV + v];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kFinalizeThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        scal[TI_RED + v] = sh[0];
        __threadfence();
        last = (atomicAdd(counter, 1u) == (unsigned int)(NV - 1));
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        double red[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) red[q] = __ldcg(scal + TI_RED + q);
        ti_phase<PH, NQ>(scal, red, tol2_0, tol2_1);
        *counter = 0u;
    }
}

// min / max of x over the rows
__global__ void __launch_bounds__(kBlock) k_minmax(Grid g, const double* __restrict__ x,
                                                   double* __restrict__ partials) {
    long long k0 = kKeyNegInf, k1 = kKeyNegInf;  // maxima of x and -x (NaN skipped), as integer keys
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        const double v = x[r];
        if (disnan(v)) continue;
        k0 = max(k0, dkey(v));
        k1 = max(k1, dkey_neg(v));
    }
    double m[2] = {dunkey(k0), dunkey(k1)};
    block_max_store<2>(m, partials);
}

// The Rock and Precipitate voxels at the end of a transport solve, one bit each: the voxels
// whose flux the reference zeroes then (src/Simulation.cpp:1134-1149; no transport row uses
// the flux of such a voxel). Labels change after the solve (precipitation makes Pore voxels
// Precipitate), so the deferred zeroing works from these bits, not from the labels it finds.
template <typename L>
__global__ void k_solid_bits(Grid g, const L* __restrict__ label, unsigned int* __restrict__ bits) {
    for (long long r0 = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); r0 < g.N;
         r0 += (long long)gridDim.x * blockDim.x) {
        const long long r = r0 + (threadIdx.x & 31u);
        bool s = false;
        if (r < g.N) {
            const int t = (int)label[r];
            s = t == kRock || t == kPrecipitate;
        }
        const unsigned int w = __ballot_sync(0xffffffffu, s);
        if ((threadIdx.x & 31u) == 0u) bits[r0 >> 5] = w;
    }
}

__global__ void k_zero_solid_flux(Grid g, const unsigned int* __restrict__ bits, double* __restrict__ fx,
                                  double* __restrict__ fy, double* __restrict__ fz) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        if ((bits[r >> 5] >> (r & 31)) & 1u) { fx[r] = 0.0; fy[r] = 0.0; fz[r] = 0.0; }
    }
}

static ls_status t_alloc(ls_ctx* c) {
    const size_t n = (size_t)c->g.N;
    LS_TRY(lean_phase(c, kPhaseTransport));  // lean: the transport arrays take the pressure solve's memory
    // largest first (lean: an arena sized for the other phase then wastes the least)
    if (!c->ti) {
        // 7 inner vectors of up to N float2 each, with `pad` elements on both sides
        c->ti_pad = ((c->g.JK + 31) / 32) * 32;
        c->ti_stride = ((2 * (c->g.N + 2 * c->ti_pad) + 63) / 64) * 64;
        LS_TRY(walloc_t(c, &c->ti, (size_t)c->ti_stride * 7));
        LS_CUDA(c, cudaMemsetAsync(c->ti, 0, sizeof(float) * (size_t)c->ti_stride * 7, c->stream));
    }
    for (int q = 0; q < 7; ++q)
        if (!c->tc[q]) LS_TRY(walloc_t(c, &c->tc[q], n));
    for (int q = 0; q < 2; ++q)
        if (!c->tb[q]) LS_TRY(walloc_t(c, &c->tb[q], n));
    if (!c->tinv) LS_TRY(walloc_t(c, &c->tinv, n));
    for (int q = 0; q < 6; ++q)
        if (!c->to[q]) LS_TRY(walloc_t(c, &c->to[q], n));
    for (int q = 0; q < 2; ++q)
        if (!c->trhs[q]) LS_TRY(walloc_t(c, &c->trhs[q], n));
    if (!c->tkind) LS_TRY(walloc_t(c, &c->tkind, n));
    if (!c->tcount) {
        LS_TRY(dalloc_t(c, &c->tcount, 1));
        LS_CUDA(c, cudaMemsetAsync(c->tcount, 0, sizeof(unsigned int), c->stream));
    }
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

// Inner solve of the right-hand sides lane_q[0..NQ-1] (indices into trhs / x), each to its
// relative tolerance tol[l]; the correction is added to x[lane_q[l]]. Returns the
// iterations of each lane.
template <int NQ>
static ls_status inner_solve(ls_ctx* c, const TBuf& tb, const int lane_q[NQ], const double tol[NQ],
                             int max_it, double* x[2], int its[NQ]) {
    const Grid g = c->g;
    const int N = (int)g.N, JK = (int)g.JK, K = g.K;
    const int grid = grid_for(c, g.N);
    TIVec iv;
    float** vecs[7] = {&iv.r, &iv.rh, &iv.p, &iv.v, &iv.s, &iv.t, &iv.d};
    for (int v = 0; v < 7; ++v) *vecs[v] = c->ti + (size_t)v * c->ti_stride + 2 * c->ti_pad;
    iv.rhs[0] = c->trhs[lane_q[0]];
    iv.rhs[1] = c->trhs[NQ > 1 ? lane_q[1] : lane_q[0]];
    TOff op;
    for (int d = 0; d < 6; ++d) op.o[d] = tb.o[d];
    const double t0 = tol[0] * tol[0], t1 = NQ > 1 ? tol[1] * tol[1] : 0.0;
    LS_LAUNCH(c, k_ti_init<NQ>, grid, kBlock, 0, N, (int)c->ti_pad, iv, c->partials);
    LS_LAUNCH(c, (k_ti_fin<PH_INIT, NQ>), NQ, kFinalizeThreads, 0, (const double*)c->partials, grid, c->scal,
              c->tcount, t0, t1);
    // algorithmic bytes of the two operator applications: FP32 off-diagonals (24 per row)
    // plus per lane 4 bytes for each vector read or written once
    const double v_bytes = (double)g.N * (24.0 + 12.0 * NQ);
    const double st_bytes = (double)g.N * (24.0 + 20.0 * NQ);
    int it = 0, batch = 4;
    double sc[TI_STRIDE * 2 + 8];
    // one right-hand side and an even row length: paired-row kernels
    const bool pair = (NQ == 1) && (K % 2 == 0);
    const int N2 = N / 2, JK2 = JK / 2, K2 = K / 2;
    const int kgrid = pair ? grid_for(c, N2) : grid;
    while (it < max_it) {
        const int nb = std::min(batch, max_it - it);
        for (int b = 0; b < nb; ++b, ++it) {
            if (it > 0) {
                if (pair) LS_LAUNCH_PDL(c, k_ti_xp_pair, kgrid, kBlock, 0, N2, iv, (const double*)c->scal);
                else LS_LAUNCH_PDL(c, k_ti_xp<NQ>, grid, kBlock, 0, N, iv, (const double*)c->scal);
            }
            {
                Timed tm(c, LS_T_KRY_APPLY);
                if (pair) {
                    if (it == 0)
                        LS_LAUNCH_PDL(c, k_ti_v_pair<true>, kgrid, kBlock, 0, N2, JK2, K2, op, iv,
                                  (const double*)c->scal, c->partials);
                    else
                        LS_LAUNCH_PDL(c, k_ti_v_pair<false>, kgrid, kBlock, 0, N2, JK2, K2, op, iv,
                                  (const double*)c->scal, c->partials);
                } else if (it == 0) {
                    LS_LAUNCH_PDL(c, (k_ti_v<NQ, true>), grid, kBlock, 0, N, JK, K, op, iv, (const double*)c->scal,
                              c->partials);
                } else {
                    LS_LAUNCH_PDL(c, (k_ti_v<NQ, false>), grid, kBlock, 0, N, JK, K, op, iv, (const double*)c->scal,
                              c->partials);
                }
                if (c->timing) c->timer_bytes[LS_T_KRY_APPLY] += v_bytes + (it == 0 ? 4.0 * NQ * g.N : 0.0);
            }
            LS_LAUNCH_PDL(c, (k_ti_fin<PH_V, NQ>), NQ, kFinalizeThreads, 0, (const double*)c->partials, kgrid,
                      c->scal, c->tcount, 0.0, 0.0);
            {
                Timed tm(c, LS_T_KRY_APPLY);
                if (pair)
                    LS_LAUNCH_PDL(c, k_ti_st_pair, kgrid, kBlock, 0, N2, JK2, K2, op, iv, (const double*)c->scal,
                              c->partials);
                else
                    LS_LAUNCH_PDL(c, k_ti_st<NQ>, grid, kBlock, 0, N, JK, K, op, iv, (const double*)c->scal,
                              c->partials);
                if (c->timing) c->timer_bytes[LS_T_KRY_APPLY] += st_bytes;
            }
            LS_LAUNCH_PDL(c, (k_ti_fin<PH_ST, NQ>), 5 * NQ, kFinalizeThreads, 0, (const double*)c->partials, kgrid,
                      c->scal, c->tcount, 0.0, 0.0);
        }
        LS_TRY(read_scalars(c, TI_BASE, TI_ANY - TI_BASE + 1, sc));
        if (sc[TI_ANY - TI_BASE] == 0.0) break;
        // next batch: the iterations the observed convergence rate still needs (at least 1)
        batch = 1;
        for (int l = 0; l < NQ; ++l) {
            const double* s = sc + TI_STRIDE * l;
            if (s[TI_ACT] == 0.0 || !(s[TI_R2] > 0.0) || !(s[TI_RR0] > 0.0) || s[TI_ITS] < 1.0) continue;
            const double red = s[TI_R2] / s[TI_RR0];
            const double per_it = log(red) / s[TI_ITS];
            if (per_it < 0.0) {
                const double need = log(s[TI_TOL2]) / per_it - s[TI_ITS];
                batch = std::max(batch, (int)std::min(16.0, std::max(1.0, ceil(need))));
            }
        }
    }
    LS_LAUNCH(c, k_ti_accum<NQ>, grid, kBlock, 0, N, iv, (const double*)c->scal, x[lane_q[0]],
              NQ > 1 ? x[lane_q[1]] : (double*)nullptr);
    for (int l = 0; l < NQ; ++l) its[l] = (int)sc[TI_STRIDE * l + TI_ITS];
    return LS_OK;
}

// Mixed-precision solve of the rows in `rows` for nrhs right-hand sides (x warm-started in
// place), fields f0/f1 supplying the right-hand sides.
template <typename L>
static ls_status mixed_solve(ls_ctx* c, const Rows<L>& rows, int nrhs, const double* f0, const double* f1,
                             double* x0, double* x1, double rtol, int max_it, ls_solve_info* info[2],
                             int* zero_lanes = nullptr) {
    LS_TRY(t_alloc(c));
    const Grid g = c->g;
    const int grid = grid_for(c, g.N);
    TBuf tb = make_tbuf(c);
    if (rows.mode == 0 && rows.tc.theta == 1.0 && !c->lean) {
        // fully implicit transport rows: recompute only the rows whose inputs changed
        const TransConst& tc = rows.tc;
        // the inflow values enter the right-hand sides only (k_t_rhs), not the rows
        const double consts[9] = {tc.inv_dt, tc.alpha, tc.D, tc.Dpore, tc.dx, tc.dc_pore, tc.dc_other,
                                  (double)tc.dd.pow2, (double)tc.inlet};
        if (!c->sht_fx) {
            const size_t n = (size_t)g.N;
            LS_TRY(dalloc(c, &c->sht_label, n * c->label_bytes));
            LS_TRY(dalloc_t(c, &c->sht_fx, n));
            LS_TRY(dalloc_t(c, &c->sht_fy, n));
            LS_TRY(dalloc_t(c, &c->sht_fz, n));
            c->t_valid = 0;
        }
        const int force = (!c->t_valid || memcmp(consts, c->t_consts, sizeof(consts)) != 0) ? 1 : 0;
        LS_TRY(wlist_reset(c));
        LS_LAUNCH(c, k_t_dirty<L>, grid, kBlock, 0, g, rows.label, rows.fx, rows.fy, rows.fz,
                  (L*)c->sht_label, c->sht_fx, c->sht_fy, c->sht_fz, c->dbits, force);
        LS_LAUNCH(c, k_t_scan, grid, kBlock, 0, g, (const unsigned int*)c->dbits, c->dwords, c->wlist, c->wcount);
        LS_LAUNCH(c, k_t_rows<L>, grid, kBlock, 0, rows, tb, (const int*)c->wlist, (const unsigned int*)c->wcount);
        LS_LAUNCH(c, k_t_rhs, grid, kBlock, 0, g, rows.tc.inv_dt, rows.tc.in_val[0], rows.tc.in_val[1], tb, nrhs,
                  f0, f1, (const double*)x0, (const double*)x1, c->partials);
        LS_TRY(finalize_sum(c, grid, 4, S_RED0 + 4));
        memcpy(c->t_consts, consts, sizeof(consts));
        c->t_valid = 1;
    } else {
        if (rows.mode == 0)
            LS_LAUNCH(c, (k_t_setup<L, true>), grid, kBlock, 0, rows, tb, nrhs, f0, f1, c->partials);
        else
            LS_LAUNCH(c, (k_t_setup<L, false>), grid, kBlock, 0, rows, tb, nrhs, f0, f1, c->partials);
        LS_TRY(finalize_sum(c, grid, 2, S_RED0 + 4));
        LS_LAUNCH(c, k_set_ones, 1, 2, 0, c->scal + S_RED0 + 6);
        c->t_valid = 0;  // the row buffers now hold other rows
    }
    LS_LAUNCH(c, k_t_xid, grid, kBlock, 0, g, tb, x0, x1, nrhs);
    double den[4];
    LS_TRY(read_scalars(c, S_RED0 + 4, 4, den));
    int mask = nrhs > 1 ? 3 : 1;
    int its[2] = {0, 0}, sweeps[2] = {0, 0}, reason[2] = {0, 0};
    // a system with b = 0 and x = 0 on every row is solved exactly: no residual pass
    for (int q = 0; q < nrhs; ++q)
        if (den[2 + q] == 0.0) { reason[q] = 2; mask &= ~(1 << q); }
    if (zero_lanes) {
        *zero_lanes = 0;
        for (int q = 0; q < nrhs; ++q)
            if (den[2 + q] == 0.0) *zero_lanes |= 1 << q;
    }
    double rel[2] = {0.0, 0.0}, prev[2] = {INFINITY, INFINITY};
    int stagnant[2] = {0, 0};
    const int max_sweeps = 40;
    while (mask) {
        LS_LAUNCH(c, k_t_resid, grid, kBlock, 0, g, tb, x0, x1, c->trhs[0], c->trhs[1], mask,
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
            // inner tolerance: what reaches rtol from here (with a margin), floored at what
            // the FP32 inner system still resolves (a relative 1e-6 is ~17 FP32 ulps)
            tol[q] = std::min(0.5, std::max(1e-6, 0.2 * rtol / std::max(rel[q], 1e-300)));
            solve_mask |= 1 << q;
        }
        if (!solve_mask) break;
        int lane_q[2] = {0, 0}, nq = 0;
        for (int q = 0; q < 2; ++q)
            if ((solve_mask >> q) & 1) lane_q[nq++] = q;
        const double ltol[2] = {tol[lane_q[0]], tol[lane_q[nq - 1]]};
        int lits[2] = {0, 0};
        const int budget = std::max(1, max_it - std::max(its[0], its[1]));
        double* xs[2] = {x0, x1};
        if (nq == 2) LS_TRY(inner_solve<2>(c, tb, lane_q, ltol, budget, xs, lits));
        else LS_TRY(inner_solve<1>(c, tb, lane_q, ltol, budget, xs, lits));
        for (int l = 0; l < nq; ++l) { its[lane_q[l]] += lits[l]; sweeps[lane_q[l]]++; }
    }
    ls_status st = LS_OK;
    double* xs[2] = {x0, x1};
    for (int q = 0; q < nrhs; ++q) {
        double mm[2] = {0.0, -0.0};  // max x, max -x
        if (den[2 + q] != 0.0) {  // otherwise x = 0 on every row
            LS_LAUNCH(c, k_minmax, grid, kBlock, 0, g, (const double*)xs[q], c->partials);
            LS_TRY(finalize_max(c, grid, 2, S_RED0 + 2));
            LS_TRY(read_scalars(c, S_RED0 + 2, 2, mm));
        }
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
    tc.inlet = (c->p.bc_mode == LS_BC_FLOW_I) ? 1 : 0;
    tc.in_val[0] = tc.in_val[1] = 0.0;
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
    // An acid field that is identically 0 (the last solve found b = 0 and x = 0 on every row,
    // and nothing has written the field since) gives b = 0 and x = 0 again: the solve would
    // leave it as it is, so it is skipped with the info such a solve reports. (A nonzero
    // inflow of acid gives b != 0 on the inflow rows, so no skip then.)
    const bool acid_inflow = rows.tc.inlet && c->p.acid_inlet != 0.0;
    if ((which & 2) && c->acid_zero && !acid_inflow) {
        which &= ~2;
        if (ai) {
            memset(ai, 0, sizeof(*ai));
            ai->converged = 1;
            ai->reason = 2;
        }
    }
    int n = 0, acid_lane = -1;
    if (which & 1) { f[n] = fields[0]; inf[n] = ci; rows.tc.in_val[n] = c->p.conc_inlet; n++; }
    if (which & 2) { f[n] = fields[1]; inf[n] = ai; rows.tc.in_val[n] = c->p.acid_inlet; acid_lane = n; n++; }
    ls_status st = LS_OK;
    if (n > 0) {
        int zero_lanes = 0;
        st = mixed_solve<L>(c, rows, n, f[0], f[1], f[0] + sh, n > 1 ? f[1] + sh : nullptr, c->p.conc_rtol,
                            c->p.conc_max_it, inf, &zero_lanes);
        if (acid_lane >= 0) c->acid_zero = (st == LS_OK && ((zero_lanes >> acid_lane) & 1)) ? 1 : 0;
    }
    if (st != LS_OK && st != LS_NOT_CONVERGED && st != LS_NONFINITE) return st;
    // the Rock / Precipitate fluxes are zeroed when next looked at: record which they are
    if (!c->solid_bits) {
        const size_t words = (size_t)((c->g.N + 31) / 32);
        LS_TRY(dalloc_t(c, &c->solid_bits, words));
        LS_TRY(dalloc_t(c, &c->solid_bits_b, words));
    }
    LS_LAUNCH(c, k_solid_bits<L>, grid_for(c, c->g.N), kBlock, 0, c->g, (const L*)c->label, c->solid_bits);
    c->flux_zero_pending = 1;
    return st;
}

// The reference zeroes the flux of Rock and Precipitate voxels after the transport solve
// (src/Simulation.cpp:1134-1149). Nothing in a time step reads those fluxes again before the
// next step's flux evaluation overwrites them, so the zeroing waits until something looks:
// the field transfers, counts and asynchronous downloads and the saturation updates call
// this first. It zeroes the voxels recorded at the solve (k_solid_bits), whatever their
// labels have become since; a snapshot keeps the pending state and those bits with the
// fields it copies. Until then the fluxes keep equal to the change-tracking shadows, and the
// next flux evaluation need not restore them.
ls_status flux_zero_now(ls_ctx* c) {
    if (!c->flux_zero_pending) return LS_OK;
    snap_fence(c, kSnapFlux);
    LS_LAUNCH(c, k_zero_solid_flux, grid_for(c, c->g.N), kBlock, 0, c->g, (const unsigned int*)c->solid_bits, c->fx,
              c->fy, c->fz);
    c->flux_zero_pending = 0;
    c->fx_is_shadow = 0;
    return LS_OK;
}

ls_status transport_run(ls_ctx* c, double dt, int which, ls_solve_info* ci, ls_solve_info* ai) {
    snap_fence(c, kSnapRest);  // conc, acid
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
    c->t_valid = 0;  // tc[0] and tc[1] serve as scratch below
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
    LS_TRY(flux_zero_now(c));  // after a transport without a flux evaluation since
    snap_fence(c, kSnapSat);
    if (c->label_bytes == 1) return sat_implicit_t<uint8_t>(c, dt, info);
    return sat_implicit_t<uint16_t>(c, dt, info);
}

}  // namespace ls
