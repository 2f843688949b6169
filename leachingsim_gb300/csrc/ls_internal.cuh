// ls_internal.cuh - shared definitions of the GB300 LeachingSim hot path.
//
// Device layout: every field has NP = (I+1)*J*K slots, voxel (i,j,k) in slot
// k + K*(j + J*i) (the reference's padded single-rank array, src/MPIDomain.h:75-97).
// Linear systems have N = I*J*K rows numbered the same way; with compat_shift the
// solution of row r is stored in slot r + J*K of its field, as on the reference's
// rank 0 (src/Simulation.cpp:808,1247,1975,2173).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/leachingsim.h"

namespace ls {

constexpr int kAir = 1, kPore = 2, kRock = 3, kSulphide = 4, kPrecipitate = 5;

// std::min / std::max semantics (NaN handling included): min(a,b) = (b<a)?b:a.
__host__ __device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }
__host__ __device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }

constexpr int kBlock = 256;        // threads per block of the streaming kernels
constexpr int kMaxPartials = 4096; // per-block partial results of one reduction

// Division of a 32-bit index by a fixed divisor through a multiply-high and a shift
// (Granlund-Montgomery): q = umulhi(n, m) >> s, exact for every n < 2^31.
struct FastDiv {
    unsigned int d, m, s;
};

inline FastDiv make_fastdiv(unsigned int d) {
    FastDiv f;
    f.d = d;
    unsigned int s = 0;
    while ((1ull << s) < d) ++s;  // s = ceil(log2 d)
    // m = ceil(2^(32+s) / d) - 2^32, valid for n < 2^31 with the add-back form below
    unsigned long long m = ((1ull << (32 + s)) + d - 1) / d;
    f.m = (unsigned int)(m - (1ull << 32));
    f.s = s;
    return f;
}

__host__ __device__ __forceinline__ unsigned int fdiv(const FastDiv& f, unsigned int n) {
#ifdef __CUDA_ARCH__
    unsigned int t = __umulhi(n, f.m);
#else
    unsigned int t = (unsigned int)(((unsigned long long)n * f.m) >> 32);
#endif
    return (unsigned int)(((unsigned long long)t + n) >> f.s);
}

struct Grid {
    int I, J, K;
    long long JK, N, NP;
    FastDiv div_jk, div_k;
};

inline void grid_init_div(Grid& g) {
    g.div_jk = make_fastdiv((unsigned int)g.JK);
    g.div_k = make_fastdiv((unsigned int)g.K);
}

__host__ __device__ __forceinline__ void decode(const Grid& g, long long r, int& i, int& j, int& k) {
    const unsigned int rr = (unsigned int)r;
    const unsigned int ii = fdiv(g.div_jk, rr);
    const unsigned int rem = rr - ii * (unsigned int)g.JK;
    const unsigned int jj = fdiv(g.div_k, rem);
    i = (int)ii;
    j = (int)jj;
    k = (int)(rem - jj * (unsigned int)g.K);
}

// Division by dx: when dx is a power of two, multiplying by its reciprocal gives the same
// double as dividing (both are exact scalings), without an FP64 division.
struct DxDiv {
    double dx, inv_dx;
    int pow2;
    __host__ __device__ __forceinline__ double div(double a) const { return pow2 ? a * inv_dx : a / dx; }
};

inline DxDiv make_dxdiv(double dx) {
    DxDiv d;
    d.dx = dx;
    d.inv_dx = 1.0 / dx;
    int e = 0;
    double m = frexp(dx, &e);
    d.pow2 = (m == 0.5) ? 1 : 0;
    return d;
}

// FP64 tests and narrowing on the integer pipe. GB300 issues FP64 compares and FP64 <->
// FP32 conversions on its FP64 pipe (2 operations per clock per SM, the cost of an FMA),
// which bounds the per-voxel FP64 kernels; these give the same results as the FP64
// instructions (NaN included) from the bit patterns.
__device__ __forceinline__ bool disnan(double x) {
    return (__double_as_longlong(x) & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
}
__device__ __forceinline__ bool dpos(double x) {  // x > 0
    const long long b = __double_as_longlong(x);
    return b > 0 && b <= 0x7ff0000000000000ll;
}

// Maxima of doubles on the integer pipe: an order-preserving map of the bit pattern to a
// signed 64-bit key (x < y iff key(x) < key(y); -0.0 and +0.0 both map to the key of +0.0;
// NaN is the caller's to skip). kKeyNegInf is the key of -Inf, the start of a maximum.
constexpr long long kKeyNegInf = -1ll - 0x7ff0000000000000ll;
__device__ __forceinline__ long long dkey_bits(long long b) {
    if (b == (long long)0x8000000000000000ull) b = 0;
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffll);
}
__device__ __forceinline__ long long dkey(double x) { return dkey_bits(__double_as_longlong(x)); }
__device__ __forceinline__ long long dkey_neg(double x) {  // key(-x)
    return dkey_bits(__double_as_longlong(x) ^ (long long)0x8000000000000000ull);
}
__device__ __forceinline__ double dunkey(long long k) {
    return __longlong_as_double(k >= 0 ? k : (k ^ 0x7fffffffffffffffll));
}

// float -> double, exact, on the integer pipe for normal, zero, infinite and NaN values
// (subnormal floats take the FP64 conversion)
__device__ __forceinline__ double f2d_exact(float f) {
    const unsigned int u = __float_as_uint(f);
    const unsigned int e = (u >> 23) & 0xffu;
    const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
    const unsigned long long man = (unsigned long long)(u & 0x7fffffu) << 29;
    if (e == 0) {
        if ((u & 0x7fffffu) == 0) return __longlong_as_double((long long)sign);
        return (double)f;
    }
    if (e == 0xffu) return __longlong_as_double((long long)(sign | 0x7ff0000000000000ull | man));
    return __longlong_as_double((long long)(sign | ((unsigned long long)(e + 896u) << 52) | man));
}

// double -> float rounded toward zero (|x| < 2^-126 -> +-0, |x| >= 2^128 -> +-Inf, NaN ->
// NaN); for FP32 copies whose rounding does not matter.
__device__ __forceinline__ float d2f_rz(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7ff) - 1023;
    const unsigned int mant = (unsigned int)((b >> 29) & 0x7fffffu);
    unsigned int out = sign | ((unsigned int)(e + 127) << 23) | mant;
    if (e < -126) out = sign;
    if (e > 127) out = sign | 0x7f800000u;
    if (e == 1024) out = sign | 0x7f800000u | ((b & 0xfffffffffffffull) ? 0x400000u : 0u);
    return __uint_as_float(out);
}

// 1/d for positive d in [2^-125, 2^126) (others: the FP64 division), within about an ulp:
// the FP32 reciprocal of the truncated significand, moved to FP64 on the integer pipe,
// then two Newton-Raphson steps y <- y + y (1 - d y). For scalings, not reference values.
__device__ __forceinline__ double drcp_nr(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const int e = (int)((b >> 52) & 0x7ff) - 1023;
    if ((b >> 63) || e < -125 || e > 125) return 1.0 / d;
    const float f = __uint_as_float(((unsigned int)(e + 127) << 23) | (unsigned int)((b >> 29) & 0x7fffffu));
    float yf;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(yf) : "f"(f));
    const unsigned int yb = __float_as_uint(yf);
    double y = __longlong_as_double((long long)(((unsigned long long)(((yb >> 23) & 0xffu) - 127 + 1023) << 52) |
                                                ((unsigned long long)(yb & 0x7fffffu) << 29)));
    y = __fma_rn(y, __fma_rn(-d, y, 1.0), y);
    return __fma_rn(y, __fma_rn(-d, y, 1.0), y);
}

// Dirty bits of the change-tracked kernels: one bit per voxel, word w holds voxels 32w ..
// 32w+31. The change tests run warp-aligned (a warp covers voxels r0 .. r0+31, r0 a multiple
// of 32) and store one ballot word per warp; the scans read windows of 32 neighbours' bits.
__device__ __forceinline__ unsigned int dwin(const unsigned int* __restrict__ bits, long long nwords,
                                             long long s) {
    // bits of voxels s .. s+31, 0 outside [0, N)
    const long long w = s >> 5;
    const int sh = (int)(s & 31);
    const unsigned int lo = (w >= 0 && w < nwords) ? __ldg(bits + w) : 0u;
    const unsigned int hi = (w + 1 >= 0 && w + 1 < nwords) ? __ldg(bits + w + 1) : 0u;
    return __funnelshift_r(lo, hi, sh);
}
__device__ __forceinline__ bool dbit(unsigned int window, int lane) { return (window >> lane) & 1u; }

// Append `value` to list[] for every thread of the block with pred set: one atomic per block
// (a single global counter takes ~one atomic per clock, so per-warp atomics over ~10^6 warps
// would serialise); every thread of the block must call it, the same number of times. The
// order of the entries is unspecified, so list consumers must not depend on it.
__device__ __forceinline__ void block_append(bool pred, int value, int* list, unsigned int* count) {
    __shared__ unsigned int warp_off[kBlock / 32];
    __shared__ unsigned int base;
    const int lane = (int)(threadIdx.x & 31u), warp = (int)(threadIdx.x >> 5);
    const unsigned int ballot = __ballot_sync(0xffffffffu, pred);
    if (lane == 0) warp_off[warp] = (unsigned int)__popc(ballot);
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int tot = 0u;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            const unsigned int c = warp_off[w];
            warp_off[w] = tot;
            tot += c;
        }
        base = tot ? atomicAdd(count, tot) : 0u;
    }
    __syncthreads();
    if (pred) list[base + warp_off[warp] + (unsigned int)__popc(ballot & ((1u << lane) - 1u))] = value;
    __syncthreads();
}

// Finest level of the inner pressure system, FP32, even row length K: (M x) for the pair of
// cells (r, r+1), r = 2t even, in the excess + Laplacian form
//   (M x)_r = e_r x_r + sum over the six faces c (x_r - x_nb),
// with the terms in the order -i, -j, -k, +k, +j, +i and separate multiply and add, as the
// per-cell kernels evaluate it. The arrays are padded (l0pad zero elements on both sides) and
// faces leaving the domain are zero, so no bounds tests are needed: such terms add 0 * (...).
__device__ __forceinline__ float2 m0_apply_pair(int t, int JK2, int K2, const float* __restrict__ e,
                                                const float* __restrict__ f0, const float* __restrict__ f1,
                                                const float* __restrict__ f2, const float* __restrict__ x) {
    const int r = 2 * t;
    const float2 ec = reinterpret_cast<const float2*>(e)[t];
    const float2 f0c = reinterpret_cast<const float2*>(f0)[t], f0m = reinterpret_cast<const float2*>(f0)[t - JK2];
    const float2 f1c = reinterpret_cast<const float2*>(f1)[t], f1m = reinterpret_cast<const float2*>(f1)[t - K2];
    const float2 f2c = reinterpret_cast<const float2*>(f2)[t];
    const float f2m = f2[r - 1];
    const float2* x2 = reinterpret_cast<const float2*>(x);
    const float2 xc = x2[t], xim = x2[t - JK2], xip = x2[t + JK2], xjm = x2[t - K2], xjp = x2[t + K2];
    const float xkm = x[r - 1], xkp = x[r + 2];
    float a0 = ec.x * xc.x;
    a0 += f0m.x * (xc.x - xim.x);
    a0 += f1m.x * (xc.x - xjm.x);
    a0 += f2m * (xc.x - xkm);
    a0 += f2c.x * (xc.x - xc.y);
    a0 += f1c.x * (xc.x - xjp.x);
    a0 += f0c.x * (xc.x - xip.x);
    float a1 = ec.y * xc.y;
    a1 += f0m.y * (xc.y - xim.y);
    a1 += f1m.y * (xc.y - xjm.y);
    a1 += f2c.x * (xc.y - xc.x);
    a1 += f2c.y * (xc.y - xkp);
    a1 += f1c.y * (xc.y - xjp.y);
    a1 += f0c.y * (xc.y - xip.y);
    return make_float2(a0, a1);
}

// Timed region record.
struct TimedRegion {
    int timer;
    cudaEvent_t start, stop;
};

// One captured multigrid preconditioner application (mg_precondition): the launches of a
// K-cycle depend only on these pointers, the output slot and the learned branch, and on the
// hierarchy's buffers, which stay in place until mg_free.
struct MGGraph {
    const void* r;
    void* z;
    const void* dv2;
    int slot, learned, is64;
    cudaGraphExec_t exec;
    long long launches;
};

// Device-side scalar slots (doubles) used by the solvers.
enum Scalar {
    S_RED0 = 0,       // generic reduction outputs S_RED0..S_RED0+15
    S_COUNT = 128
};

}  // namespace ls

struct ls_ctx {
    ls::Grid g;
    int label_bytes;
    ls_params p;
    int device;
    int num_sms;
    cudaStream_t stream;
    std::string err;

    // fields, NP slots each
    void* label;
    float* frac;
    float* kmult;         // intrinsic-permeability multiplier, allocated on first upload (else 1)
    double *perm, *visc, *P, *conc, *acid, *fx, *fy, *fz, *sat, *pc, *kr, *precip;
    // snapshot (src/Simulation.cpp:2312-2328)
    void* b_label;
    float* b_frac;
    double *b_precip, *b_sat, *b_P, *b_conc, *b_acid, *b_fx, *b_fy, *b_fz;

    // pressure system (N rows)
    int8_t* pkind;      // 0 empty row, 1 identity row, 2 Pore row, 3 Pore row with floored diagonal
    double* pdiag;      // diagonal of the assembled row
    double* pb;         // right-hand side (identity rows: the fixed value)
    double* pface[3];   // link coefficient of the +i, +j, +k face (used by Pore rows)
    double* pisd;       // 1/sqrt(d) of inner unknowns (normal Pore rows), else 0
    double* pr;         // FP64 outer residual
    double* pdelta;     // FP64 correction
    // inner pressure system on the normal Pore rows, sigma-scaled, in "excess + graph
    // Laplacian" form: (M x)_i = e_i x_i + sum_links c_ij (x_i - x_j). T = float or double.
    void* ie;           // excess e (links to rows that are not inner unknowns), T
    void* iface[3];     // link coefficients of the +i, +j, +k faces between two unknowns, T
    void* iinvd;        // 1 / (e + sum of the six links), T
    void* inner[5];     // inner PCG vectors x r z p q, T
    // the finest-level arrays (ie, iface, iinvd, inner, mg0_x, mg0_t) carry l0pad zero
    // elements on both sides, so stencil loads need no bounds tests; l0base holds the
    // allocations (slots: 0 ie, 1-3 iface, 4 iinvd, 5-9 inner, 10 mg0_x, 11 mg0_t)
    void* l0base[12];
    size_t l0bytes[12];
    long long l0pad;
    int inner_is64;     // -1 = not allocated
    double pscale_den;  // ||D^-1 b|| of the current pressure system
    double p_t;         // time the pressure system was assembled for
    double p_eff;       // ramped top pressure of the assembled system
    double p_eff_prev;  // ... of the previous solve (0 = none)
    int p_ready;

    // change tracking: the per-voxel property and face kernels keep shadow copies of their
    // inputs and recompute only voxels whose inputs changed bitwise since their last
    // evaluation (their results are pure functions of those inputs, so reuse is exact)
    void* sh_label;       // props inputs at the last evaluation of each voxel
    double* sh_sat;
    double* sh_precip;
    float* sh_frac;
    void* shf_label;      // pressure-face inputs at the last evaluation
    double* shf_perm;
    double* shf_visc;
    double* psb2;         // (b/diag)^2 of each pressure row, for the norm of the residual test
    double rows_evap_dx;  // evaporation constant the stored pressure rows were built with
    double rows_bc[3];    // bc_mode, p_inlet, p_outlet the stored pressure rows were built with
    double* sat_q;        // div q + evaporative sink of each active voxel (saturation update)
    unsigned int* dbits;  // dirty bits of the change tests: two planes of dwords words
    long long dwords;     // ceil(N / 32)
    int* wlist;           // voxel work list of the change-tracked kernels (N entries)
    int* olist_counts;    // per-chunk counts / offsets of ordered_list (olist_nb + 1 ints)
    long long olist_nb;
    int plist_valid;      // wlist holds the ascending list of the pressure unknowns (kind >= 2)
    unsigned int* wcount; // its length
    int props_force, faces_force;  // recompute every voxel on the next call
    void* sht_label;      // transport-row inputs at the last evaluation (fully implicit rows)
    double *sht_fx, *sht_fy, *sht_fz;
    int t_valid;          // the stored transport rows are fully implicit rows for t_consts
    int acid_zero;        // the acid field is identically 0: the last transport solve found
                          // b = 0 and x = 0; cleared by every write from outside
    double t_consts[10];
    double *shq_P, *shq_C, *shq_K, *shq_V;  // flux inputs at the last evaluation
    double *shq_fx, *shq_fy, *shq_fz;       // the fluxes last computed
    int flux_valid;
    int flux_zero_pending;    // the Rock / Precipitate fluxes are still to be zeroed (flux_zero_now)
    int flux_zero_pending_b;  // the same at the last snapshot
    unsigned int* solid_bits;    // the voxels that were Rock or Precipitate at the last transport
    unsigned int* solid_bits_b;  // the same at the last snapshot
    int fx_is_shadow;         // fx / fy / fz equal the change-tracking shadows at every voxel
    double flux_consts[2];

    // multigrid: the finest level is the inner system above (vectors mg0_x, mg0_t);
    // mg[l] are the coarse levels, each owning its arrays
    struct MGLevel {
        ls::Grid g;
        int* comp;          // owning component of the cell (-1 = no unknown)
        void* e;            // excess, T
        void* face[3];      // + face links, T
        void* invd;         // 1 / diagonal, T
        void* x;            // T
        void* b;            // T
        void* t;            // T
        void* kv[7];        // K-cycle vectors on this level (rr, za, zb, pd, q0, q1, e), T, or null
        int esize;          // sizeof(T)
    };
    std::vector<MGLevel> mg;
    void* mg0_x;
    void* mg0_t;
    int mg_is64;          // -1 = not allocated
    std::vector<ls::MGGraph> mg_graphs;  // captured preconditioner applications
    int mg_graphs_off;    // 1: launch the cycle kernel by kernel (LS_MG_GRAPHS=0)
    long long mg_tail_cells;  // coarse levels up to this many cells run as one block (LS_MG_TAIL_CELLS; 0: off)
    int pdl;                  // programmatic dependent launch in the multigrid cycle (LS_PDL; 0: off)
    int* comp;            // fine-level strong-component ids (-1 = not an inner unknown)
    uint8_t* start_anchor; // per component root: anchored to fixed values (supplied starts)
    int* cc_flag;         // device flag for the labelling loop
    // learned coarse solver of the multigrid (LS_PRESS_LEARNED): a network that stands in
    // for the V-cycle below the K-cycle levels
    ls_lpnet* lpc;                  // sized for the learned level's grid, or null
    std::vector<float> lpc_params;  // weights from ls_pressure_set_precond_weights
    int lpc_dims[3];                // the network's grid (the level's extents rounded up to 8)
    int lpc_ready;                  // the network's fixed inputs match the current hierarchy
    int lpc_active;                 // the learned cycle is in use in the current solve
    float *lpc_c0, *lpc_c1, *lpc_c2, *lpc_out;  // network grid: inputs, output channel 0
    float* lpc_isd;                 // learned level: 1/sqrt(diagonal) of served cells, else 0
    long long lpc_isd_n;            // its length
    uint8_t* lpc_anchor;            // per component id: anchored on the learned level
    long long press_fallbacks;      // learned solves that fell back to the plain cycle

    // transport / implicit saturation (2 right-hand sides)
    double* tc[7];        // FP64 row coefficients: diagonal, then +i,-i,+j,-j,+k,-k
    double* tb[2];        // FP64 right-hand sides
    float* to[6];         // FP32 off-diagonals scaled by the row diagonal
    double* tinv;         // FP64 1 / row diagonal
    float* trhs[2];       // FP32 D^-1 (b - A x) per right-hand side
    float* ti;            // FP32 inner vectors r rh p v s t d, padded, float or float2 rows
    long long ti_pad, ti_stride;  // zero elements around each vector; floats per vector
    unsigned int* tcount; // blocks done in the current transport reduction
    int8_t* tkind;        // 1 identity row, 2 coupled row

    // dissolution
    int* dz_list;         // active mineral voxels sorted by wavefront (or by dependency level)
    int* dz_count;
    int* dz_level_start;
    int* dz_tab;                    // per-level running totals of the skewed schedule's slices
    long long dz_tab_cap;
    std::vector<int> dz_tab_host;
    int dz_cap;
    // sparse schedule of the dissolution sweep: the voxels that can change (in any order),
    // the voxels fully leached during a call, and the pre-sweep state of the scheduled voxels
    int* dz_sel;
    int* dz_flips;
    float* dz_save_frac;
    double* dz_save_precip;
    double* dz_save_conc;
    void* dz_save_label;
    int dz_sel_cap;
    long long dz_fallbacks;  // calls that fell back to the full wavefront sweep
    int dz_no_threshold;     // no active voxel has 0 < frac <= 1e-4 (known after a dissolution call;
                             // cleared by every write of labels or frac from outside)

    // reductions
    double* partials;     // kMaxPartials * 8 doubles
    double* scal;         // device scalars
    double* h_scal;       // pinned host mirror
    int* d_int;           // device ints (counters, flags)
    int* h_int;           // pinned host mirror
    void* h_small;        // mapped pinned host memory for small readbacks (read_device)
    void* hd_small;       // its device address
    size_t h_small_bytes;

    // accounting
    long long launches;
    int timing;
    std::vector<ls::TimedRegion> regions;
    std::vector<cudaEvent_t> event_pool;
    double timer_ms[LS_T_COUNT];
    long long timer_count[LS_T_COUNT];
    double timer_bytes[LS_T_COUNT];
    unsigned long long initial_sulphide_count;
    size_t device_bytes;
    size_t device_peak;   // most device_bytes held at once
    size_t host_bytes;    // pinned (or pageable) host memory of the lean snapshot
    int lean;             // LS_MEM_LEAN
    // lean: the work arrays of the current phase (pressure or transport) are cut from one
    // arena, reset at every phase switch and sized to the larger phase's need
    void* arena;
    size_t arena_size, arena_used, arena_overflow, arena_need;
    int arena_phase;      // kPhase*
    int b_host_pinned;    // lean: the snapshot arrays came from cudaHostAlloc (else malloc)
    // Copies of fields to host memory (the lean snapshot, ls_download_fields_async) run on a
    // stream of their own, from the state the context's stream had reached; a kernel family
    // that writes a field waits for the pending copies of its group (snap_fence)
    cudaStream_t snap_stream;
    cudaEvent_t snap_ev[6];  // [0..4] copies of the groups kSnap*, [5] the start of a batch
    int snap_pending;        // groups whose copies the main stream has not waited for
    // resident layout: ls_download_fields_async copies the fields into this device staging
    // buffer first (a fast device copy), so that the steps that follow never wait for the
    // copies to the host; stage_free is recorded after the last copy out of it
    void* stage;
    size_t stage_bytes;
    cudaEvent_t stage_free;
};

namespace ls {

// error helpers ------------------------------------------------------------
ls_status set_error(ls_ctx* c, ls_status st, const std::string& msg);
ls_status check_cuda(ls_ctx* c, cudaError_t e, const char* what);
#define LS_CUDA(ctx, call)                                                          \
    do {                                                                            \
        cudaError_t e__ = (call);                                                   \
        if (e__ != cudaSuccess) return ls::check_cuda((ctx), e__, #call);           \
    } while (0)
#define LS_TRY(expr)                                                                \
    do {                                                                            \
        ls_status s__ = (expr);                                                     \
        if (s__ != LS_OK) return s__;                                               \
    } while (0)
// kernel launch + accounting + launch-error check
#define LS_LAUNCH(ctx, kernel, grid, block, smem, ...)                              \
    do {                                                                            \
        kernel<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);            \
        (ctx)->launches++;                                                          \
        cudaError_t e__ = cudaGetLastError();                                       \
        if (e__ != cudaSuccess) return ls::check_cuda((ctx), e__, #kernel);         \
    } while (0)

// Programmatic dependent launch, for the chains of small kernels of the multigrid cycle: the
// kernel may be scheduled while its predecessor in the stream still runs (once every block of
// the predecessor has passed its pdl_enter), so its launch overlaps the predecessor's work.
// Only kernels that begin with pdl_enter() are launched this way (ctx->pdl = 0: LS_PDL=0,
// ordinary launches).
#define LS_LAUNCH_PDL(ctx, kernel, grid, block, smem, ...)                          \
    do {                                                                            \
        cudaLaunchConfig_t cfg__ = {};                                              \
        cfg__.gridDim = dim3(grid);                                                 \
        cfg__.blockDim = dim3(block);                                               \
        cfg__.dynamicSmemBytes = (smem);                                            \
        cfg__.stream = (ctx)->stream;                                               \
        cudaLaunchAttribute at__[1];                                                \
        at__[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;            \
        at__[0].val.programmaticStreamSerializationAllowed = (ctx)->pdl ? 1 : 0;    \
        cfg__.attrs = at__;                                                         \
        cfg__.numAttrs = 1;                                                         \
        cudaError_t e__ = cudaLaunchKernelEx(&cfg__, kernel, __VA_ARGS__);          \
        (ctx)->launches++;                                                          \
        if (e__ == cudaSuccess) e__ = cudaGetLastError();                           \
        if (e__ != cudaSuccess) return ls::check_cuda((ctx), e__, #kernel);         \
    } while (0)

inline int grid_for(const ls_ctx* c, long long n) {
    long long want = (n + kBlock - 1) / kBlock;
    long long cap = (long long)c->num_sms * 8;
    if (want > cap) want = cap;
    if (want < 1) want = 1;
    return (int)want;
}

// timing
void region_begin(ls_ctx* c, int timer, cudaEvent_t* start);
void region_end(ls_ctx* c, int timer, cudaEvent_t start);
struct Timed {
    ls_ctx* c;
    int t;
    cudaEvent_t s;
    Timed(ls_ctx* ctx, int timer) : c(ctx), t(timer), s(nullptr) { region_begin(c, t, &s); }
    ~Timed() { region_end(c, t, s); }
};

// reductions: per-block partials -> device scalar (deterministic order)
ls_status finalize_sum(ls_ctx* c, int nblocks, int nvals, int out_slot);
ls_status finalize_max(ls_ctx* c, int nblocks, int nvals, int out_slot);
ls_status read_scalars(ls_ctx* c, int first, int count, double* out);
ls_status read_device(ls_ctx* c, const void* dev, void* out, size_t bytes);

// device block reduction of nvals doubles per thread into partials[blockIdx.x*nvals + v]
template <int NV>
__device__ __forceinline__ void block_sum_store(double (&v)[NV], double* partials) {
    __shared__ double sh[NV][kBlock / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double x = v[q];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sh[q][warp] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double s = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[q][w];
            partials[(size_t)blockIdx.x * NV + q] = s;
        }
    }
}

template <int NV>
__device__ __forceinline__ void block_max_store(double (&v)[NV], double* partials) {
    __shared__ double sh[NV][kBlock / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double x = v[q];
        for (int o = 16; o > 0; o >>= 1) x = smax(x, __shfl_down_sync(0xffffffffu, x, o));
        if (lane == 0) sh[q][warp] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double s = sh[q][0];
            for (int w = 1; w < (int)(blockDim.x >> 5); ++w) s = smax(s, sh[q][w]);
            partials[(size_t)blockIdx.x * NV + q] = s;
        }
    }
}

// The first statement of a kernel launched with LS_LAUNCH_PDL: wait until the grid before it
// in the stream has completed and its memory operations are visible, then let the next
// kernel be scheduled. In a kernel launched the ordinary way the wait returns at once.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// One block per value: a fixed-order tree reduction of the per-block partials (the
// result does not depend on timing).
constexpr int kFinalizeThreads = 256;
template <bool MAX>
__global__ void __launch_bounds__(kFinalizeThreads) k_finalize(const double* __restrict__ partials,
                                                               int nblocks, int nvals,
                                                               double* __restrict__ out) {
    pdl_enter();
    __shared__ double sh[kFinalizeThreads];
    const int v = blockIdx.x;
    double acc = MAX ? -INFINITY : 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
        double x = partials[(size_t)b * nvals + v];
        acc = MAX ? smax(acc, x) : acc + x;
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kFinalizeThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            double o = sh[threadIdx.x + w];
            sh[threadIdx.x] = MAX ? smax(sh[threadIdx.x], o) : sh[threadIdx.x] + o;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) out[v] = sh[0];
}

// label access
template <typename L>
__device__ __forceinline__ int lab(const L* a, long long r) { return (int)a[r]; }

// component-wise entry points implemented in the .cu files
ls_status props_run(ls_ctx* c);
ls_status flux_run(ls_ctx* c);
ls_status saturation_run(ls_ctx* c, double dt, ls_substep_info* info);
ls_status saturation_implicit_run(ls_ctx* c, double dt, ls_solve_info* info);
ls_status surface_run(ls_ctx* c);
ls_status precip_run(ls_ctx* c);
ls_status pressure_setup_run(ls_ctx* c, double t);
ls_status pressure_solve_run(ls_ctx* c, ls_solve_info* info, const float* start = nullptr,
                             double start_scale = 0.0);
ls_status pressure_learned_inputs_run(ls_ctx* c, float* mask, float* logk, float* bc);
ls_status pressure_apply_run(ls_ctx* c, const double* x, double* y);
ls_status transport_run(ls_ctx* c, double dt, int which, ls_solve_info* ci, ls_solve_info* ai);
ls_status flux_zero_now(ls_ctx* c);
ls_status transport_apply_run(ls_ctx* c, double dt, const double* x, double* y);
// acid_pre (optional, N doubles): receives the acid the sweeps start from; *swept tells
// whether they ran (otherwise nothing changed)
ls_status dissolve_run(ls_ctx* c, double dt, int* leached, ls_substep_info* info, double* acid_pre,
                       bool* swept);
// FP64 budget of the fields after a step (acid_pre: the acid before the dissolution sweep, or
// null when the sweep did not run)
ls_status budget_run(ls_ctx* c, const double* acid_pre, ls_budget* b);
ls_status init_frac_run(ls_ctx* c, unsigned long long* count);
ls_status init_saturation_run(ls_ctx* c);

// allocation helper tracking device bytes
ls_status dalloc(ls_ctx* c, void** p, size_t bytes);
// releases an array of `bytes` bytes from dalloc (null: nothing); *p becomes null
void dfree(ls_ctx* c, void** p, size_t bytes);
template <typename T>
void dfree_t(ls_ctx* c, T** p, size_t n) {
    dfree(c, reinterpret_cast<void**>(p), n * sizeof(T));
}
// The ascending list of the rows r < N with kind[r] >= min_kind into wlist / wcount (a
// deterministic order, so that reductions over it are reproducible).
ls_status ordered_list(ls_ctx* c, const int8_t* kind, int min_kind);
// the work list holding every voxel 0 .. N-1 (the change-tracked kernels without change
// tracking, LS_MEM_LEAN)
ls_status wlist_all(ls_ctx* c);
// Groups of fields copied to the host, in the order a step first writes them: the pressure,
// the fluxes, the saturation, then labels, frac, conc, acid and precipitate; the properties
// (K, viscosity, Pc, kr) are written by the props pass at the start of a step.
constexpr int kSnapP = 1, kSnapFlux = 2, kSnapSat = 4, kSnapRest = 8, kSnapProps = 16, kSnapAll = 31;
// make the context's stream wait until the snapshot copies of `groups` are done (no-op when
// none are pending)
void snap_fence(ls_ctx* c, int groups);
// Work arrays of one phase of the step (the pressure solve's or the transport solves'): in
// LS_MEM_LEAN cut from the context's arena, which lean_phase resets; otherwise dalloc.
ls_status walloc(ls_ctx* c, void** p, size_t bytes);
template <typename T>
ls_status walloc_t(ls_ctx* c, T** p, size_t n) {
    return walloc(c, reinterpret_cast<void**>(p), n * sizeof(T));
}
// LS_MEM_LEAN: enter a phase; on a switch every work array of either phase is released and
// the arena is reset (and grown to the largest need seen). No-op otherwise.
constexpr int kPhaseNone = 0, kPhasePressure = 1, kPhaseTransport = 2;
ls_status lean_phase(ls_ctx* c, int phase);
void mg_free(ls_ctx* c);
// the work list, its counter and the dirty flags, allocated on first use; resets the counter
ls_status wlist_reset(ls_ctx* c);
// finest-level array in slot `slot`: N elements of `esize` bytes with l0pad zero elements on
// both sides (cleared); *out points at element 0
ls_status l0_alloc(ls_ctx* c, int slot, size_t esize, void** out);
void l0_free(ls_ctx* c, int slot, void** p);
template <typename T>
ls_status dalloc_t(ls_ctx* c, T** p, size_t n) {
    return dalloc(c, reinterpret_cast<void**>(p), n * sizeof(T));
}

}  // namespace ls
