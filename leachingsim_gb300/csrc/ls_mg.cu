// ls_mg.cu - geometric multigrid preconditioner of the inner pressure PCG.
//
// Every level holds its operator in "excess + graph Laplacian" form,
//     (M x)_i = e_i x_i + sum_{links ij} c_ij (x_i - x_j),   e_i >= 0, c_ij >= 0,
// so M is symmetric positive (semi)definite for any rounding of e and c: the FP32 copy of
// the finest operator cannot turn indefinite, and the Galerkin coarse operators are sums of
// positive terms (no cancellation). The finest level is the inner system itself (excess =
// links of a Pore row to rows that are not inner unknowns).
//
// The Pore network is masked by Dirichlet voxels everywhere and its links span ~13 orders
// of magnitude, so plain 2x2x2 aggregation would hand coarse corrections to Pore clusters
// that merely share a block with the main network while being joined to it by no strong
// link; such a cluster's near-null mode then keeps the correction (its residual is ~1e-13
// of the error). The hierarchy therefore works per strong component:
//   * components: connected pieces of the unknowns over links with
//     c_ij / sqrt(d_i d_j) > kStrong (union-find on the device);
//   * aggregation: each 2x2x2 block becomes one coarse cell owned by the component with
//     most members in the block; only its members are restricted to / prolongated from it
//     (piecewise-constant interpolation); links from members to non-members become excess;
//   * V-cycle: two damped-Jacobi sweeps before and after the coarse correction, a fixed
//     number of Jacobi sweeps by one CTA on the coarsest level, so the cycle is a symmetric
//     operator usable inside CG.
#include <algorithm>
#include <functional>
#include <type_traits>
#include <cstdio>

#include "ls_internal.cuh"

namespace ls {

constexpr double kStrong = 1e-3;   // scaled link weight below which a link joins no components
constexpr double kOmega = 2.0 / 3.0;
constexpr int kCoarsestCells = 512;
constexpr int kCoarseSweeps = 48;
constexpr double kProlongScale = 1.8;
constexpr int kKLevels = 3;   // levels 1..kKLevels take a K-cycle coarse correction
constexpr int kKSlot0 = 32;   // device scalar slots of the K-cycle FCG (5 per level)
constexpr int kUnionSpin = 1 << 20;  // bound on the union-find retry loop
// learned coarse solver (LS_PRESS_LEARNED): the network solves level kLearnedLevel in place of
// the V-cycle below the K-cycle levels
constexpr int kLearnedLevel = kKLevels + 1;  // the level below the K-cycle levels
constexpr float kLpcOutScale = 64.f;  // network output x this x max|D^-1/2 b| = D^1/2 x
constexpr int kLpcSlot = 60;          // device scalar: max |D^-1/2 b| over the level's members

__device__ __forceinline__ long long lidx(const Grid& g, int i, int j, int k) {
    return (long long)k + (long long)g.K * ((long long)j + (long long)g.J * i);
}

// (M x)_r in difference form (links on the six faces; f0/f1/f2 hold the + faces)
template <typename T>
__device__ __forceinline__ T m_apply(const Grid& g, long long r, int i, int j, int k, const T* __restrict__ e,
                                     const T* __restrict__ f0, const T* __restrict__ f1,
                                     const T* __restrict__ f2, const T* __restrict__ x) {
    const T xr = x[r];
    T acc = e[r] * xr;
    if (i > 0) acc += f0[r - g.JK] * (xr - x[r - g.JK]);
    if (j > 0) acc += f1[r - g.K] * (xr - x[r - g.K]);
    if (k > 0) acc += f2[r - 1] * (xr - x[r - 1]);
    if (k + 1 < g.K) acc += f2[r] * (xr - x[r + 1]);
    if (j + 1 < g.J) acc += f1[r] * (xr - x[r + g.K]);
    if (i + 1 < g.I) acc += f0[r] * (xr - x[r + g.JK]);
    return acc;
}

// 1 / (e + sum of the six links) of live cells, 1 elsewhere
template <typename T>
__global__ void k_level_invd(Grid g, const int* __restrict__ comp, const int8_t* __restrict__ kind,
                             const T* __restrict__ e, const T* __restrict__ f0, const T* __restrict__ f1,
                             const T* __restrict__ f2, T* __restrict__ invd) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        T out = (T)1;
        bool live = comp ? comp[r] >= 0 : kind[r] == 2;
        if (live) {
            int i, j, k;
            decode(g, r, i, j, k);
            T d = e[r];
            if (i > 0) d += f0[r - g.JK];
            if (j > 0) d += f1[r - g.K];
            if (k > 0) d += f2[r - 1];
            if (k + 1 < g.K) d += f2[r];
            if (j + 1 < g.J) d += f1[r];
            if (i + 1 < g.I) d += f0[r];
            out = (d > (T)0) ? (T)1 / d : (T)1;
        }
        invd[r] = out;
    }
}

// ---------------------------------------------------------------------------
// strong components (union-find with path halving; ids are voxel indices, the root is the
// smallest voxel of the component)

// find with path halving (hooking). Each store points a non-root at one of its ancestors,
// and a parent value read from a stale L1 line (L1 is not coherent across SMs) is a former
// ancestor, so still an ancestor. A stale line can however show a root that another SM has
// hooked since; the CAS then fails, and the retry reads with FRESH loads that bypass L1.
template <bool FRESH>
__device__ __forceinline__ int cc_find(int* parent, int x) {
    int p = FRESH ? __ldcg(parent + x) : parent[x];
    int guard = 0;
    while (p != x && guard++ < kUnionSpin) {
        int gp = FRESH ? __ldcg(parent + p) : parent[p];
        parent[x] = gp;
        x = p;
        p = gp;
    }
    return x;
}

// read-only find (compression): a path-halving store from a stale parent value could
// otherwise overwrite a cell's final root with an intermediate ancestor
__device__ __forceinline__ int cc_find_ro(const int* parent, int x) {
    int p = parent[x];
    int guard = 0;
    while (p != x && guard++ < kUnionSpin) {
        x = p;
        p = parent[x];
    }
    return x;
}

__global__ void k_cc_init(Grid g, const int8_t* __restrict__ kind, int* __restrict__ parent) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x)
        parent[r] = (kind[r] == 2) ? (int)r : -1;
}

template <typename T>
__global__ void k_cc_hook(Grid g, const T* __restrict__ f0, const T* __restrict__ f1,
                          const T* __restrict__ f2, const T* __restrict__ invd, int* parent,
                          int* __restrict__ err) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        if (parent[r] < 0) continue;
        const T* fs[3] = {f0, f1, f2};
        const long long offs[3] = {g.JK, g.K, 1};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            T c = fs[d][r];
            if (!(c > (T)0)) continue;  // c > 0 only between two unknowns
            long long nb = r + offs[d];
            // c / sqrt(d_r d_nb) > kStrong, squared: no square root on the FP64 pipe
            const T w2 = c * c * invd[r] * invd[nb];
            if (!(w2 > (T)(kStrong * kStrong))) continue;
            int a = (int)r, b = (int)nb;
            int spins = 0;
            while (true) {
                int ra = spins ? cc_find<true>(parent, a) : cc_find<false>(parent, a);
                int rb = spins ? cc_find<true>(parent, b) : cc_find<false>(parent, b);
                if (ra == rb) break;
                int lo = ra < rb ? ra : rb, hi = ra < rb ? rb : ra;
                if (atomicCAS(&parent[hi], hi, lo) == hi) break;
                if (++spins > kUnionSpin) { atomicExch(err, 1); break; }
            }
        }
    }
}

__global__ void k_cc_compress(Grid g, int* parent) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        if (parent[r] < 0) continue;
        parent[r] = cc_find_ro(parent, (int)r);
    }
}

// ---------------------------------------------------------------------------
// hierarchy construction

// dominant component of each 2x2x2 block (most members; ties: smallest id)
__global__ void k_mg_dom(Grid f, Grid cg, const int* __restrict__ fcomp, int* __restrict__ ccomp) {
    for (long long R = blockIdx.x * (long long)blockDim.x + threadIdx.x; R < cg.N;
         R += (long long)gridDim.x * blockDim.x) {
        int I, J, K;
        decode(cg, R, I, J, K);
        int ids[8];
        int n = 0;
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                for (int c = 0; c < 2; ++c) {
                    int i = 2 * I + a, j = 2 * J + b, k = 2 * K + c;
                    if (i >= f.I || j >= f.J || k >= f.K) continue;
                    int id = fcomp[lidx(f, i, j, k)];
                    if (id >= 0) ids[n++] = id;
                }
        int best = -1, bestc = 0;
        for (int q = 0; q < n; ++q) {
            int cnt = 0;
            for (int s = 0; s < n; ++s) cnt += (ids[s] == ids[q]);
            if (cnt > bestc || (cnt == bestc && ids[q] < best)) { best = ids[q]; bestc = cnt; }
        }
        ccomp[R] = best;
    }
}

// is fine cell (i,j,k) a member of its own block's owner?
__device__ __forceinline__ bool is_member(const Grid& f, const Grid& cg, const int* fcomp, const int* ccomp,
                                          int i, int j, int k) {
    int id = fcomp[lidx(f, i, j, k)];
    return id >= 0 && ccomp[lidx(cg, i >> 1, j >> 1, k >> 1)] == id;
}

// Galerkin coarse operator P^T M P for piecewise-constant P restricted to the members of
// each block's owner: coarse excess = member excess + member links to non-members;
// coarse + face link = member-to-member links crossing the block's + face.
template <typename T>
__global__ void k_mg_coarse_op(Grid f, Grid cg, const int* __restrict__ fcomp, const int* __restrict__ ccomp,
                               const T* __restrict__ fe, const T* __restrict__ f0, const T* __restrict__ f1,
                               const T* __restrict__ f2, T* __restrict__ ce, T* __restrict__ c0,
                               T* __restrict__ c1, T* __restrict__ c2) {
    for (long long R = blockIdx.x * (long long)blockDim.x + threadIdx.x; R < cg.N;
         R += (long long)gridDim.x * blockDim.x) {
        int I, J, K;
        decode(cg, R, I, J, K);
        const int own = ccomp[R];
        double ex = 0.0, e0 = 0.0, e1 = 0.0, e2 = 0.0;
        if (own >= 0) {
            for (int a = 0; a < 2; ++a)
                for (int b = 0; b < 2; ++b)
                    for (int c = 0; c < 2; ++c) {
                        int i = 2 * I + a, j = 2 * J + b, k = 2 * K + c;
                        if (i >= f.I || j >= f.J || k >= f.K) continue;
                        long long fr = lidx(f, i, j, k);
                        if (fcomp[fr] != own) continue;
                        ex += (double)fe[fr];
                        // the six links of this member
                        const int di[6] = {1, -1, 0, 0, 0, 0}, dj[6] = {0, 0, 1, -1, 0, 0},
                                  dk[6] = {0, 0, 0, 0, 1, -1};
                        for (int d = 0; d < 6; ++d) {
                            int ni = i + di[d], nj = j + dj[d], nk = k + dk[d];
                            if (ni < 0 || nj < 0 || nk < 0 || ni >= f.I || nj >= f.J || nk >= f.K) continue;
                            long long nr = lidx(f, ni, nj, nk);
                            double cl;
                            switch (d) {
                            case 0: cl = (double)f0[fr]; break;
                            case 1: cl = (double)f0[nr]; break;
                            case 2: cl = (double)f1[fr]; break;
                            case 3: cl = (double)f1[nr]; break;
                            case 4: cl = (double)f2[fr]; break;
                            default: cl = (double)f2[nr]; break;
                            }
                            if (cl == 0.0) continue;
                            bool nmem = is_member(f, cg, fcomp, ccomp, ni, nj, nk);
                            bool same_block = (ni >> 1) == I && (nj >> 1) == J && (nk >> 1) == K;
                            if (!nmem) { ex += cl; continue; }  // P = 0 on the other end
                            if (same_block) continue;           // internal link
                            // member of another block: a coarse link (stored on + faces)
                            if (d == 0) e0 += cl;
                            else if (d == 2) e1 += cl;
                            else if (d == 4) e2 += cl;
                        }
                    }
        }
        ce[R] = (T)(own >= 0 ? ex : 1.0);
        c0[R] = (T)e0;
        c1[R] = (T)e1;
        c2[R] = (T)e2;
    }
}

// ---------------------------------------------------------------------------
// V-cycle kernels

// One damped-Jacobi update of cell r (shared by the level kernels and the one-block tail)
template <typename T>
__device__ __forceinline__ T smooth_cell(const Grid& g, long long r, const T* __restrict__ e,
                                         const T* __restrict__ f0, const T* __restrict__ f1,
                                         const T* __restrict__ f2, const T* __restrict__ invd,
                                         const T* __restrict__ b, const T* __restrict__ x) {
    const T bv = b[r];
    if (x) {
        int i, j, k;
        decode(g, r, i, j, k);
        const T res = bv - m_apply(g, r, i, j, k, e, f0, f1, f2, x);
        return x[r] + (T)kOmega * invd[r] * res;
    }
    return (T)kOmega * invd[r] * bv;
}

// x_out = x + omega invd (b - M x); x == nullptr means x = 0. With dotv, the per-block
// partial of (dotv, x_out) is stored (the (r, z) of the PCG).
// Cells that are not members keep 0 in every level vector: the buffers are cleared when
// allocated and nothing writes them there, so the smoother skips them (membership from the
// 1-byte kind on the finest level, the component id on coarse levels).
template <typename T>
__global__ void __launch_bounds__(kBlock) k_mg_smooth(Grid g, const int* __restrict__ comp,
                                                      const int8_t* __restrict__ kind0, const T* __restrict__ e,
                                                      const T* __restrict__ f0, const T* __restrict__ f1,
                                                      const T* __restrict__ f2, const T* __restrict__ invd,
                                                      const T* __restrict__ b, const T* __restrict__ x,
                                                      T* __restrict__ xo, const T* __restrict__ dotv,
                                                      const T* __restrict__ dotv2, double* __restrict__ partials) {
    pdl_enter();
    T acc = (T)0, acc2 = (T)0;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        const bool live = kind0 ? kind0[r] == 2 : comp[r] >= 0;
        if (!live) continue;
        const T out = smooth_cell(g, r, e, f0, f1, f2, invd, b, x);
        xo[r] = out;
        if (dotv) acc += dotv[r] * out;
        if (dotv2) acc2 += dotv2[r] * out;
    }
    if (dotv) {
        double a[2] = {(double)acc, (double)acc2};
        block_sum_store<2>(a, partials);
    }
}

// The finest-level smoother on pairs of cells (FP32, K even, padded arrays; see
// m0_apply_pair): the same sweep as k_mg_smooth for kind-2 cells.
__global__ void __launch_bounds__(kBlock) k_mg_smooth0_pair(int N2, int JK2, int K2,
                                                            const int8_t* __restrict__ kind,
                                                            const float* __restrict__ e, const float* __restrict__ f0,
                                                            const float* __restrict__ f1, const float* __restrict__ f2,
                                                            const float* __restrict__ invd, const float* __restrict__ b,
                                                            const float* __restrict__ x, float* __restrict__ xo,
                                                            const float* __restrict__ dotv,
                                                            const float* __restrict__ dotv2,
                                                            double* __restrict__ partials) {
    pdl_enter();
    float acc = 0.f, acc2 = 0.f;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < N2; t += gridDim.x * blockDim.x) {
        const char2 kd = reinterpret_cast<const char2*>(kind)[t];
        const bool l0 = kd.x == 2, l1 = kd.y == 2;
        if (!l0 && !l1) continue;
        const float2 bv = reinterpret_cast<const float2*>(b)[t];
        const float2 iv = reinterpret_cast<const float2*>(invd)[t];
        float o0, o1;
        if (x) {
            const float2 m = m0_apply_pair(t, JK2, K2, e, f0, f1, f2, x);
            const float2 xv = reinterpret_cast<const float2*>(x)[t];
            o0 = xv.x + (float)kOmega * iv.x * (bv.x - m.x);
            o1 = xv.y + (float)kOmega * iv.y * (bv.y - m.y);
        } else {
            o0 = (float)kOmega * iv.x * bv.x;
            o1 = (float)kOmega * iv.y * bv.y;
        }
        if (l0) xo[2 * t] = o0;
        if (l1) xo[2 * t + 1] = o1;
        if (dotv) {
            if (l0) acc += dotv[2 * t] * o0;
            if (l1) acc += dotv[2 * t + 1] * o1;
        }
        if (dotv2) {
            if (l0) acc2 += dotv2[2 * t] * o0;
            if (l1) acc2 += dotv2[2 * t + 1] * o1;
        }
    }
    if (dotv) {
        double a[2] = {(double)acc, (double)acc2};
        block_sum_store<2>(a, partials);
    }
}

// Finest-level residual b - M x of kind-2 cells on pairs (FP32, K even, padded arrays), for
// the restriction: each fine residual is formed once, by a coalesced fine-cell pass.
__global__ void __launch_bounds__(kBlock) k_mg_resid0_pair(int N2, int JK2, int K2, const int8_t* __restrict__ kind,
                                                           const float* __restrict__ e, const float* __restrict__ f0,
                                                           const float* __restrict__ f1, const float* __restrict__ f2,
                                                           const float* __restrict__ b, const float* __restrict__ x,
                                                           float* __restrict__ res) {
    pdl_enter();
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < N2; t += gridDim.x * blockDim.x) {
        const char2 kd = reinterpret_cast<const char2*>(kind)[t];
        const bool l0 = kd.x == 2, l1 = kd.y == 2;
        if (!l0 && !l1) continue;
        const float2 m = m0_apply_pair(t, JK2, K2, e, f0, f1, f2, x);
        const float2 bv = reinterpret_cast<const float2*>(b)[t];
        if (l0) res[2 * t] = bv.x - m.x;
        if (l1) res[2 * t + 1] = bv.y - m.y;
    }
}

// coarse right-hand side from stored fine residuals: b_c(R) = sum over owned members, in
// the child order of k_mg_restrict
template <typename T>
__global__ void k_mg_restrict_gather(Grid f, Grid cg, const int* __restrict__ fcomp, const int* __restrict__ ccomp,
                                     const T* __restrict__ res, T* __restrict__ cb) {
    pdl_enter();
    for (long long R = blockIdx.x * (long long)blockDim.x + threadIdx.x; R < cg.N;
         R += (long long)gridDim.x * blockDim.x) {
        int I, J, K;
        decode(cg, R, I, J, K);
        const int own = ccomp[R];
        T acc = (T)0;
        if (own >= 0) {
            for (int a = 0; a < 2; ++a)
                for (int b = 0; b < 2; ++b)
                    for (int c = 0; c < 2; ++c) {
                        int i = 2 * I + a, j = 2 * J + b, k = 2 * K + c;
                        if (i >= f.I || j >= f.J || k >= f.K) continue;
                        long long fr = lidx(f, i, j, k);
                        if (fcomp[fr] != own) continue;
                        acc += res[fr];
                    }
        }
        cb[R] = acc;
    }
}

// b_c(R) = sum over the owned members of (b - M x)
template <typename T>
__device__ __forceinline__ T restrict_cell(const Grid& f, const Grid& cg, long long R, const int* __restrict__ fcomp,
                                           const int* __restrict__ ccomp, const T* __restrict__ e,
                                           const T* __restrict__ f0, const T* __restrict__ f1,
                                           const T* __restrict__ f2, const T* __restrict__ fb,
                                           const T* __restrict__ fx) {
    int I, J, K;
    decode(cg, R, I, J, K);
    const int own = ccomp[R];
    T acc = (T)0;
    if (own >= 0) {
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                for (int c = 0; c < 2; ++c) {
                    int i = 2 * I + a, j = 2 * J + b, k = 2 * K + c;
                    if (i >= f.I || j >= f.J || k >= f.K) continue;
                    long long fr = lidx(f, i, j, k);
                    if (fcomp[fr] != own) continue;
                    acc += fb[fr] - m_apply(f, fr, i, j, k, e, f0, f1, f2, fx);
                }
    }
    return acc;
}

// coarse right-hand side: b_c(R) = sum over owned members of (b - M x)
template <typename T>
__global__ void k_mg_restrict(Grid f, Grid cg, const int* __restrict__ fcomp, const int* __restrict__ ccomp,
                              const T* __restrict__ e, const T* __restrict__ f0, const T* __restrict__ f1,
                              const T* __restrict__ f2, const T* __restrict__ fb, const T* __restrict__ fx,
                              T* __restrict__ cb) {
    pdl_enter();
    for (long long R = blockIdx.x * (long long)blockDim.x + threadIdx.x; R < cg.N;
         R += (long long)gridDim.x * blockDim.x)
        cb[R] = restrict_cell(f, cg, R, fcomp, ccomp, e, f0, f1, f2, fb, fx);
}

template <typename T>
__device__ __forceinline__ void prolong_cell(const Grid& f, const Grid& cg, long long r, const int* __restrict__ fcomp,
                                             const int* __restrict__ ccomp, const T* __restrict__ cx,
                                             T* __restrict__ fx, T scale) {
    const int id = fcomp[r];
    if (id < 0) return;
    int i, j, k;
    decode(f, r, i, j, k);
    const long long R = lidx(cg, i >> 1, j >> 1, k >> 1);
    if (ccomp[R] == id) fx[r] += scale * cx[R];
}

// x_f += kProlongScale * x_c(block) for owned members. Piecewise-constant prolongation
// undershoots smooth error; scaling the coarse correction (over-correction) roughly halves the
// PCG iterations on these pore-space operators (33 instead of 71 on a 96^3 porosity-0.25 field).
template <typename T>
__global__ void k_mg_prolong(Grid f, Grid cg, const int* __restrict__ fcomp, const int* __restrict__ ccomp,
                             const T* __restrict__ cx, T* __restrict__ fx, T scale) {
    pdl_enter();
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < f.N;
         r += (long long)gridDim.x * blockDim.x)
        prolong_cell(f, cg, r, fcomp, ccomp, cx, fx, scale);
}

// ---------------------------------------------------------------------------
// K-cycle (Notay-Vassilevski): on the levels 1..kKLevels the coarse correction is two
// flexible-CG iterations on that level, preconditioned by the cycle from that level down,
// instead of one cycle. The scalars of each level's FCG live on the device (slots kKSlot0 +
// 5 (level - 1) + {pq0, prr0, zq0, pq1, prr1}), so no host synchronisation is needed.

// q = M pd and the partial dots (pd, q), (pd, rr) over member cells
template <typename T>
__global__ void __launch_bounds__(kBlock) k_kc_apply(Grid g, const int* __restrict__ comp, const T* __restrict__ e,
                                                     const T* __restrict__ f0, const T* __restrict__ f1,
                                                     const T* __restrict__ f2, const T* __restrict__ pd,
                                                     const T* __restrict__ rr, T* __restrict__ q,
                                                     double* __restrict__ partials) {
    pdl_enter();
    T a0 = (T)0, a1 = (T)0;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        if (comp[r] < 0) continue;
        int i, j, k;
        decode(g, r, i, j, k);
        const T qv = m_apply(g, r, i, j, k, e, f0, f1, f2, pd);
        q[r] = qv;
        a0 += pd[r] * qv;
        a1 += pd[r] * rr[r];
    }
    double a[2] = {(double)a0, (double)a1};
    block_sum_store<2>(a, partials);
}

// first iteration: e = alpha pd, rr -= alpha q with alpha = (pd, rr) / (pd, q)
template <typename T>
__global__ void k_kc_first(Grid g, const int* __restrict__ comp, const double* __restrict__ s,
                           const T* __restrict__ pd, const T* __restrict__ q, T* __restrict__ e,
                           T* __restrict__ rr) {
    pdl_enter();
    const T a = (T)((s[0] > 0.0) ? s[1] / s[0] : 0.0);
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        if (comp[r] < 0) continue;
        e[r] = a * pd[r];
        rr[r] -= a * q[r];
    }
}

// second direction: pd1 = z - ((z, q0) / (pd0, q0)) pd0
template <typename T>
__global__ void k_kc_dir(Grid g, const int* __restrict__ comp, const double* __restrict__ s,
                         const T* __restrict__ z, const T* __restrict__ pd0, T* __restrict__ pd1) {
    pdl_enter();
    const T b = (T)((s[0] > 0.0) ? -s[2] / s[0] : 0.0);
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x)
        if (comp[r] >= 0) pd1[r] = z[r] + b * pd0[r];
}

// second iteration: e += alpha1 pd1, alpha1 = (pd1, rr) / (pd1, q1)
template <typename T>
__global__ void k_kc_second(Grid g, const int* __restrict__ comp, const double* __restrict__ s,
                            const T* __restrict__ pd1, T* __restrict__ e) {
    pdl_enter();
    const T a = (T)((s[3] > 0.0) ? s[4] / s[3] : 0.0);
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x)
        if (comp[r] >= 0) e[r] += a * pd1[r];
}

// coarsest level: a fixed number of damped Jacobi sweeps from zero by one CTA
template <typename T>
__device__ __forceinline__ void coarsest_block(const Grid& g, const int* __restrict__ comp, const T* __restrict__ e,
                                               const T* __restrict__ f0, const T* __restrict__ f1,
                                               const T* __restrict__ f2, const T* __restrict__ invd,
                                               const T* __restrict__ b, T* x, T* t, int sweeps) {
    for (long long r = threadIdx.x; r < g.N; r += blockDim.x)
        x[r] = (comp[r] >= 0) ? (T)kOmega * invd[r] * b[r] : (T)0;
    __syncthreads();
    for (int s = 1; s < sweeps; ++s) {
        for (long long r = threadIdx.x; r < g.N; r += blockDim.x) {
            T out = (T)0;
            if (comp[r] >= 0) {
                int i, j, k;
                decode(g, r, i, j, k);
                T res = b[r] - m_apply(g, r, i, j, k, e, f0, f1, f2, x);
                out = x[r] + (T)kOmega * invd[r] * res;
            }
            t[r] = out;
        }
        __syncthreads();
        for (long long r = threadIdx.x; r < g.N; r += blockDim.x) x[r] = t[r];
        __syncthreads();
    }
}

template <typename T>
__global__ void k_mg_coarsest(Grid g, const int* __restrict__ comp, const T* __restrict__ e,
                              const T* __restrict__ f0, const T* __restrict__ f1, const T* __restrict__ f2,
                              const T* __restrict__ invd, const T* __restrict__ b, T* x, T* t, int sweeps) {
    pdl_enter();
    coarsest_block(g, comp, e, f0, f1, f2, invd, b, x, t, sweeps);
}

// The V-cycle over the small coarse levels in one block. The levels from `first` down hold
// a few thousand cells at most, where a kernel per sweep costs more in launch than in work
// (the cycle over levels 5-6 of the 338x338x283 workload: 7 launches of ~7 us); one block
// of 1024 threads runs the same cycle -- the same per-cell updates in the same order, so
// the same results bit for bit -- with a barrier between sweeps. Level q of the tail reads
// its right-hand side from b[q] and leaves its correction in x[q] (t[q]: scratch), as the
// kernels of cycle() do.
constexpr int kMaxTail = 8;
template <typename T>
struct TailLevels {
    Grid g[kMaxTail];
    const int* comp[kMaxTail];
    const T *e[kMaxTail], *f0[kMaxTail], *f1[kMaxTail], *f2[kMaxTail], *invd[kMaxTail];
    T *x[kMaxTail], *b[kMaxTail], *t[kMaxTail];
    int n;  // levels in the tail; the last is the coarsest
};

template <typename T>
__global__ void __launch_bounds__(1024) k_mg_tail(TailLevels<T> L, T scale, int sweeps) {
    pdl_enter();
    const int n = L.n;
    // down: two smoothing sweeps from zero, then the restricted residual
    for (int q = 0; q + 1 < n; ++q) {
        const Grid& g = L.g[q];
        for (long long r = threadIdx.x; r < g.N; r += blockDim.x)
            if (L.comp[q][r] >= 0) L.t[q][r] = smooth_cell(g, r, L.e[q], L.f0[q], L.f1[q], L.f2[q], L.invd[q],
                                                          (const T*)L.b[q], (const T*)nullptr);
        __syncthreads();
        for (long long r = threadIdx.x; r < g.N; r += blockDim.x)
            if (L.comp[q][r] >= 0) L.x[q][r] = smooth_cell(g, r, L.e[q], L.f0[q], L.f1[q], L.f2[q], L.invd[q],
                                                          (const T*)L.b[q], (const T*)L.t[q]);
        __syncthreads();
        const Grid& cg = L.g[q + 1];
        for (long long R = threadIdx.x; R < cg.N; R += blockDim.x)
            L.b[q + 1][R] = restrict_cell(g, cg, R, L.comp[q], L.comp[q + 1], L.e[q], L.f0[q], L.f1[q], L.f2[q],
                                          (const T*)L.b[q], (const T*)L.x[q]);
        __syncthreads();
    }
    const int c = n - 1;
    coarsest_block(L.g[c], L.comp[c], L.e[c], L.f0[c], L.f1[c], L.f2[c], L.invd[c], (const T*)L.b[c], L.x[c],
                   L.t[c], sweeps);
    // up: the scaled coarse correction, then two smoothing sweeps
    for (int q = n - 2; q >= 0; --q) {
        const Grid& g = L.g[q];
        for (long long r = threadIdx.x; r < g.N; r += blockDim.x)
            prolong_cell(g, L.g[q + 1], r, L.comp[q], L.comp[q + 1], (const T*)L.x[q + 1], L.x[q], scale);
        __syncthreads();
        for (long long r = threadIdx.x; r < g.N; r += blockDim.x)
            if (L.comp[q][r] >= 0) L.t[q][r] = smooth_cell(g, r, L.e[q], L.f0[q], L.f1[q], L.f2[q], L.invd[q],
                                                          (const T*)L.b[q], (const T*)L.x[q]);
        __syncthreads();
        for (long long r = threadIdx.x; r < g.N; r += blockDim.x)
            if (L.comp[q][r] >= 0) L.x[q][r] = smooth_cell(g, r, L.e[q], L.f0[q], L.f1[q], L.f2[q], L.invd[q],
                                                          (const T*)L.b[q], (const T*)L.t[q]);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// learned coarse solver: the network maps (member mask, anchoring fraction e/d, D^-1/2 b / s)
// on a D x H x W grid holding the level at its origin to D^1/2 x / (s kLpcOutScale), the
// Jacobi-scaled correction, s = max |D^-1/2 b| over the members. The unit-diagonal scaling
// makes the inputs and outputs independent of the level's coefficient magnitudes.

__device__ __forceinline__ bool lpc_cell(const Grid& g, int W, int H, long long v, long long& r) {
    const long long hw = (long long)W * H;
    const int z = (int)(v / hw);
    const long long rem = v - (long long)z * hw;
    const int y = (int)(rem / W), x = (int)(rem - (long long)y * W);
    if (z >= g.I || y >= g.J || x >= g.K) return false;
    r = lidx(g, z, y, x);
    return true;
}

// Components the network serves: those with a cell on the level whose excess is above
// kLpcAnchor of its diagonal (coupled to fixed values). Elsewhere the level is singular or
// nearly so; a correction there would excite near-null modes that only smoothing removes,
// so those cells keep the zero correction. anchored is indexed by component id (N bytes).
constexpr float kLpcAnchor = 1e-3f;

template <typename T>
__global__ void k_lpc_anchor(Grid g, const int* __restrict__ comp, const T* __restrict__ e,
                             const T* __restrict__ invd, uint8_t* __restrict__ anchored) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N; r += (long long)gridDim.x * blockDim.x) {
        const int id = comp[r];
        if (id >= 0 && (float)e[r] * (float)invd[r] > kLpcAnchor) anchored[id] = 1;
    }
}

// the fixed inputs of a hierarchy: mask, anchoring fraction e/d (the share of the diagonal
// that couples to fixed values) and 1/sqrt(d) of the cells of anchored components (0 marks
// the cells the network does not serve)
template <typename T>
__global__ void k_lpc_setup(Grid g, int D, int H, int W, const int* __restrict__ comp, const T* __restrict__ e,
                            const T* __restrict__ invd, const uint8_t* __restrict__ anchored,
                            float* __restrict__ c0, float* __restrict__ c1, float* __restrict__ isd) {
    const long long n = (long long)D * H * W;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        long long r = 0;
        float m = 0.f, a = 0.f;
        if (lpc_cell(g, W, H, v, r)) {
            float q = 0.f;
            if (comp[r] >= 0 && anchored[comp[r]]) {
                m = 1.f;
                a = (float)e[r] * (float)invd[r];
                q = sqrtf((float)invd[r]);
            }
            isd[r] = q;
        }
        c0[v] = m;
        c1[v] = a;
    }
}

// s = max |b| / sqrt(d) over the served cells (one block; NaN entries are passed over here and
// reach the network through k_lpc_pack, whose output then carries them to the caller)
__global__ void __launch_bounds__(1024) k_lpc_scale(Grid g, const int* __restrict__ comp, const float* __restrict__ b,
                                                    const float* __restrict__ isd, double* __restrict__ out) {
    float m = 0.f;
    for (long long r = threadIdx.x; r < g.N; r += blockDim.x)
        if (comp[r] >= 0) m = fmaxf(m, fabsf(b[r] * isd[r]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float sh[32];
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) *out = (double)m;
    }
}

__global__ void k_lpc_pack(Grid g, int D, int H, int W, const int* __restrict__ comp, const float* __restrict__ b,
                           const float* __restrict__ isd, const double* __restrict__ s, float* __restrict__ c2) {
    const float inv = (*s > 0.0) ? (float)(1.0 / *s) : 0.f;
    const long long n = (long long)D * H * W;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        long long r = 0;
        float val = 0.f;
        if (lpc_cell(g, W, H, v, r) && comp[r] >= 0) val = b[r] * isd[r] * inv;  // isd 0: not served
        c2[v] = val;
    }
}

// x = s kLpcOutScale D^-1/2 y on the served cells, 0 on the other members (non-members keep
// their 0)
__global__ void k_lpc_unpack(Grid g, int H, int W, const int* __restrict__ comp, const float* __restrict__ y,
                             const float* __restrict__ isd, const double* __restrict__ s, float* __restrict__ x) {
    const float sc = (float)(*s) * kLpcOutScale;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N; r += (long long)gridDim.x * blockDim.x) {
        if (comp[r] < 0) continue;
        if (isd[r] == 0.f) {
            x[r] = 0.f;
            continue;
        }
        const int i = (int)(r / g.JK);
        const long long rem = r - (long long)i * g.JK;
        const int j = (int)(rem / g.K), k = (int)(rem - (long long)j * g.K);
        x[r] = sc * isd[r] * y[((long long)i * H + j) * W + k];
    }
}

ls_status lpnet_forward_on(ls_lpnet* n, cudaStream_t s, const float* c0, const float* c1, const float* c2,
                           float* out, std::string* err);

static int round8(int v) { return ((v + 7) / 8) * 8; }

void mg_graphs_clear(ls_ctx* c);

// Build (or reuse) the network for the learned level of the current hierarchy and its fixed
// inputs. Without weights the learned solver is an argument error; a hierarchy too shallow
// to have the level leaves the plain cycle in use.
static ls_status lpc_prepare(ls_ctx* c) {
    c->lpc_ready = 0;
    if (c->p.press_solver != LS_PRESS_LEARNED) return LS_OK;
    if (c->lpc_params.empty())
        return set_error(c, LS_BAD_ARG, "learned pressure solver: no weights (ls_pressure_set_precond_weights)");
    if (c->mg.size() < (size_t)kLearnedLevel) return LS_OK;
    const auto& lv = c->mg[kLearnedLevel - 1];
    const Grid lg = lv.g;
    const int dims[3] = {round8(lg.I), round8(lg.J), round8(lg.K)};
    if (!c->lpc || dims[0] != c->lpc_dims[0] || dims[1] != c->lpc_dims[1] || dims[2] != c->lpc_dims[2]) {
        mg_graphs_clear(c);  // captured cycles name the old network's buffers
        if (c->lpc) {
            ls_lpnet_destroy(c->lpc);
            c->lpc = nullptr;
        }
        const size_t old_nn = (size_t)c->lpc_dims[0] * c->lpc_dims[1] * c->lpc_dims[2];
        dfree_t(c, &c->lpc_c0, old_nn);
        dfree_t(c, &c->lpc_c1, old_nn);
        dfree_t(c, &c->lpc_c2, old_nn);
        dfree_t(c, &c->lpc_out, old_nn);
        dfree_t(c, &c->lpc_isd, (size_t)c->lpc_isd_n);
        ls_lpnet* n = nullptr;
        ls_status st = ls_lpnet_create(dims[0], dims[1], dims[2], 0, &n);
        if (st != LS_OK) return set_error(c, st, "learned pressure solver: network creation failed");
        c->lpc = n;
        if (ls_lpnet_param_count(n) != (long long)c->lpc_params.size())
            return set_error(c, LS_BAD_ARG, "learned pressure solver: weight count does not match the network");
        st = ls_lpnet_set_params(n, c->lpc_params.data(), (long long)c->lpc_params.size());
        if (st != LS_OK) return set_error(c, st, "learned pressure solver: loading the weights failed");
        const size_t nn = (size_t)dims[0] * dims[1] * dims[2];
        LS_TRY(dalloc_t(c, &c->lpc_c0, nn));
        LS_TRY(dalloc_t(c, &c->lpc_c1, nn));
        LS_TRY(dalloc_t(c, &c->lpc_c2, nn));
        LS_TRY(dalloc_t(c, &c->lpc_out, nn));
        LS_TRY(dalloc_t(c, &c->lpc_isd, (size_t)lg.N));
        c->lpc_isd_n = lg.N;
        for (int q = 0; q < 3; ++q) c->lpc_dims[q] = dims[q];
    }
    if (!c->lpc_anchor) LS_TRY(dalloc_t(c, &c->lpc_anchor, (size_t)c->g.N));
    LS_CUDA(c, cudaMemsetAsync(c->lpc_anchor, 0, (size_t)c->g.N, c->stream));
    LS_LAUNCH(c, k_lpc_anchor<float>, grid_for(c, lg.N), kBlock, 0, lg, (const int*)lv.comp, (const float*)lv.e,
              (const float*)lv.invd, c->lpc_anchor);
    const long long nn = (long long)dims[0] * dims[1] * dims[2];
    LS_LAUNCH(c, k_lpc_setup<float>, grid_for(c, nn), kBlock, 0, lg, dims[0], dims[1], dims[2],
              (const int*)lv.comp, (const float*)lv.e, (const float*)lv.invd, (const uint8_t*)c->lpc_anchor,
              c->lpc_c0, c->lpc_c1, c->lpc_isd);
    c->lpc_ready = 1;
    return LS_OK;
}

// x = the network's approximation of M_l^-1 b on the learned level
static ls_status lpc_solve(ls_ctx* c, const Grid& lg, const int* comp, const float* b, float* x) {
    const int* d = c->lpc_dims;
    const long long nn = (long long)d[0] * d[1] * d[2];
    LS_LAUNCH(c, k_lpc_scale, 1, 1024, 0, lg, comp, b, (const float*)c->lpc_isd, c->scal + kLpcSlot);
    LS_LAUNCH(c, k_lpc_pack, grid_for(c, nn), kBlock, 0, lg, d[0], d[1], d[2], comp, b, (const float*)c->lpc_isd,
              (const double*)(c->scal + kLpcSlot), c->lpc_c2);
    std::string err;
    const ls_status st = lpnet_forward_on(c->lpc, c->stream, c->lpc_c0, c->lpc_c1, c->lpc_c2, c->lpc_out, &err);
    if (st != LS_OK) return set_error(c, st, "learned coarse solve: " + err);
    c->launches += 16;  // the network's own launches: input pack, 8 convolutions, 3 poolings, 3 upsamplings, output
    LS_LAUNCH(c, k_lpc_unpack, grid_for(c, lg.N), kBlock, 0, lg, d[1], d[2], comp, (const float*)c->lpc_out,
              (const float*)c->lpc_isd, (const double*)(c->scal + kLpcSlot), x);
    return LS_OK;
}

// ---------------------------------------------------------------------------

static Grid coarse_of(const Grid& f) {
    Grid c;
    c.I = (f.I + 1) / 2;
    c.J = (f.J + 1) / 2;
    c.K = (f.K + 1) / 2;
    c.JK = (long long)c.J * c.K;
    c.N = (long long)c.I * c.JK;
    c.NP = c.N;
    grid_init_div(c);
    return c;
}

void mg_graphs_clear(ls_ctx* c) {
    for (auto& gr : c->mg_graphs)
        if (gr.exec) cudaGraphExecDestroy(gr.exec);
    c->mg_graphs.clear();
}

void mg_free(ls_ctx* c) {
    mg_graphs_clear(c);
    for (size_t m = 0; m < c->mg.size(); ++m) {
        auto& lv = c->mg[m];
        const size_t n = (size_t)lv.g.N, es = (size_t)lv.esize;
        dfree_t(c, &lv.comp, n);
        void** lp[] = {&lv.e, &lv.face[0], &lv.face[1], &lv.face[2], &lv.invd, &lv.x, &lv.b, &lv.t};
        for (void** q : lp) dfree(c, q, es * n);
        for (void*& q : lv.kv) dfree(c, &q, es * n);
    }
    c->mg.clear();
    l0_free(c, 10, &c->mg0_x);
    l0_free(c, 11, &c->mg0_t);
    c->mg_is64 = -1;
}

template <typename T>
static ls_status mg_alloc(ls_ctx* c) {
    const int is64 = sizeof(T) == 8;
    if (c->mg_is64 == is64) return LS_OK;
    mg_free(c);
    if (!c->comp) LS_TRY(walloc_t(c, &c->comp, (size_t)c->g.N));
    if (!c->cc_flag) LS_TRY(dalloc_t(c, &c->cc_flag, (size_t)4));
    LS_TRY(l0_alloc(c, 10, sizeof(T), &c->mg0_x));
    LS_TRY(l0_alloc(c, 11, sizeof(T), &c->mg0_t));
    Grid g = c->g;
    g.NP = g.N;
    while ((c->mg.empty() || g.N > kCoarsestCells) && (g.I > 1 || g.J > 1 || g.K > 1)) {
        Grid cg = coarse_of(g);
        ls_ctx::MGLevel lv = {};
        lv.g = cg;
        lv.esize = (int)sizeof(T);
        LS_TRY(walloc_t(c, &lv.comp, (size_t)cg.N));
        void** arrs[] = {&lv.e, &lv.face[0], &lv.face[1], &lv.face[2], &lv.invd, &lv.x, &lv.b, &lv.t};
        for (void** q : arrs) {
            LS_TRY(walloc(c, q, sizeof(T) * (size_t)cg.N));
            LS_CUDA(c, cudaMemsetAsync(*q, 0, sizeof(T) * (size_t)cg.N, c->stream));
        }
        c->mg.push_back(lv);
        g = cg;
    }
    // K-cycle vectors on the levels 1..kKLevels that have a coarser level below them
    for (size_t m = 1; m <= (size_t)kKLevels && m < c->mg.size(); ++m) {
        auto& lv = c->mg[m - 1];
        for (void*& q : lv.kv) {
            LS_TRY(walloc(c, &q, sizeof(T) * (size_t)lv.g.N));
            LS_CUDA(c, cudaMemsetAsync(q, 0, sizeof(T) * (size_t)lv.g.N, c->stream));
        }
    }
    c->mg_is64 = is64;
    return LS_OK;
}

// 1/diagonal of the finest inner operator (rows of kind 2 live)
template <typename T>
ls_status inner_invd(ls_ctx* c) {
    LS_LAUNCH(c, k_level_invd<T>, grid_for(c, c->g.N), kBlock, 0, c->g, (const int*)nullptr,
              (const int8_t*)c->pkind, (const T*)c->ie, (const T*)c->iface[0], (const T*)c->iface[1],
              (const T*)c->iface[2], (T*)c->iinvd);
    return LS_OK;
}

// Components and coarse operators for the current fine inner operator (c->ie, c->iface,
// c->iinvd, precision T).
template <typename T>
ls_status mg_setup(ls_ctx* c) {
    LS_TRY(mg_alloc<T>(c));
    const Grid g = c->g;
    const int grid = grid_for(c, g.N);
    LS_CUDA(c, cudaMemsetAsync(c->cc_flag, 0, sizeof(int), c->stream));
    LS_LAUNCH(c, k_cc_init, grid, kBlock, 0, g, (const int8_t*)c->pkind, c->comp);
    LS_LAUNCH(c, k_cc_hook<T>, grid, kBlock, 0, g, (const T*)c->iface[0], (const T*)c->iface[1],
              (const T*)c->iface[2], (const T*)c->iinvd, c->comp, c->cc_flag);
    LS_LAUNCH(c, k_cc_compress, grid, kBlock, 0, g, c->comp);
    Grid fg = g;
    const int* fcomp = c->comp;
    const T* fe = (const T*)c->ie;
    const T* ff[3] = {(const T*)c->iface[0], (const T*)c->iface[1], (const T*)c->iface[2]};
    for (size_t l = 0; l < c->mg.size(); ++l) {
        auto& cl = c->mg[l];
        const int cgd = grid_for(c, cl.g.N);
        LS_LAUNCH(c, k_mg_dom, cgd, kBlock, 0, fg, cl.g, fcomp, cl.comp);
        LS_LAUNCH(c, k_mg_coarse_op<T>, cgd, kBlock, 0, fg, cl.g, fcomp, (const int*)cl.comp, fe, ff[0], ff[1],
                  ff[2], (T*)cl.e, (T*)cl.face[0], (T*)cl.face[1], (T*)cl.face[2]);
        LS_LAUNCH(c, k_level_invd<T>, cgd, kBlock, 0, cl.g, (const int*)cl.comp, (const int8_t*)nullptr,
                  (const T*)cl.e, (const T*)cl.face[0], (const T*)cl.face[1], (const T*)cl.face[2],
                  (T*)cl.invd);
        fg = cl.g;
        fcomp = cl.comp;
        fe = (const T*)cl.e;
        ff[0] = (const T*)cl.face[0];
        ff[1] = (const T*)cl.face[1];
        ff[2] = (const T*)cl.face[2];
    }
    int flag = 0;
    LS_CUDA(c, cudaMemcpyAsync(&flag, c->cc_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    LS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (flag) return set_error(c, LS_TIMEOUT, "multigrid: component labelling gave up");
    if (std::is_same<T, float>::value) return lpc_prepare(c);
    c->lpc_ready = 0;
    return LS_OK;
}

// Zero every level vector (the smoother and the PCG skip non-member cells, which must hold 0).
template <typename T>
ls_status mg_clear(ls_ctx* c) {
    LS_CUDA(c, cudaMemsetAsync(c->mg0_x, 0, sizeof(T) * (size_t)c->g.N, c->stream));
    LS_CUDA(c, cudaMemsetAsync(c->mg0_t, 0, sizeof(T) * (size_t)c->g.N, c->stream));
    for (auto& lv : c->mg) {
        const size_t b = sizeof(T) * (size_t)lv.g.N;
        LS_CUDA(c, cudaMemsetAsync(lv.x, 0, b, c->stream));
        LS_CUDA(c, cudaMemsetAsync(lv.b, 0, b, c->stream));
        LS_CUDA(c, cudaMemsetAsync(lv.t, 0, b, c->stream));
        for (void* q : lv.kv)
            if (q) LS_CUDA(c, cudaMemsetAsync(q, 0, b, c->stream));
    }
    return LS_OK;
}

// z = B r: one K-cycle (levels 1..kKLevels take the two-iteration FCG coarse correction,
// deeper levels a plain V-cycle). The per-block partials of (r, z) and (dotv2, z) are left in
// c->partials (two values per block, dotv2 may be null) and their count in *nblocks_out.
template <typename T>
ls_status mg_apply(ls_ctx* c, const T* r, T* z, const T* dotv2, int* nblocks_out) {
    const size_t L = c->mg.size();  // coarse levels
    if (L == 0) return set_error(c, LS_BAD_ARG, "multigrid hierarchy missing");
    struct Lv {
        Grid g;
        const int* comp;
        const T *e, *f0, *f1, *f2, *invd;
        T *x, *b, *t;
        T* kv[7];
    };
    std::vector<Lv> lv(L + 1);
    lv[0] = {c->g, c->comp, (const T*)c->ie, (const T*)c->iface[0], (const T*)c->iface[1], (const T*)c->iface[2],
             (const T*)c->iinvd, (T*)c->mg0_x, nullptr, (T*)c->mg0_t, {}};
    for (size_t l = 0; l < L; ++l) {
        auto& m = c->mg[l];
        lv[l + 1] = {m.g, m.comp, (const T*)m.e, (const T*)m.face[0], (const T*)m.face[1], (const T*)m.face[2],
                     (const T*)m.invd, (T*)m.x, (T*)m.b, (T*)m.t, {}};
        for (int q = 0; q < 7; ++q) lv[l + 1].kv[q] = (T*)m.kv[q];
    }
    // one damped-Jacobi sweep on level l (paired finest-level kernel for FP32 and even K)
    const bool pair0 = std::is_same<T, float>::value && (c->g.K % 2 == 0);
    const bool learned = std::is_same<T, float>::value && c->lpc_active && c->lpc_ready && L >= (size_t)kLearnedLevel;
    auto smooth = [&](size_t l, const T* b, const T* x, T* xo, const T* dv, const T* dv2, int* nb) -> ls_status {
        Lv& a = lv[l];
        double* partials = dv ? c->partials : (double*)nullptr;
        if (l == 0 && pair0) {
            const int N2 = (int)(a.g.N / 2);
            const int gd = grid_for(c, N2);
            LS_LAUNCH_PDL(c, k_mg_smooth0_pair, gd, kBlock, 0, N2, (int)(a.g.JK / 2), a.g.K / 2,
                      (const int8_t*)c->pkind, (const float*)a.e, (const float*)a.f0, (const float*)a.f1,
                      (const float*)a.f2, (const float*)a.invd, (const float*)b, (const float*)x, (float*)xo,
                      (const float*)dv, (const float*)dv2, partials);
            if (nb) *nb = gd;
            return LS_OK;
        }
        const int gd = grid_for(c, a.g.N);
        LS_LAUNCH_PDL(c, k_mg_smooth<T>, gd, kBlock, 0, a.g, a.comp,
                  l == 0 ? (const int8_t*)c->pkind : (const int8_t*)nullptr, a.e, a.f0, a.f1, a.f2, a.invd, b, x,
                  xo, dv, dv2, partials);
        if (nb) *nb = gd;
        return LS_OK;
    };
    // cycle(l, b, out): out = B_l b; with dv non-null the final sweep leaves the partial dots
    // (dv, out), (dv2, out) and their block count in *nb. Level l's x and t are its scratch.
    std::function<ls_status(size_t, const T*, T*, const T*, const T*, int*)> cycle;
    // kfcg(m): two FCG iterations on level m for M_m e = b_m (m's b), result in kv[6]
    auto kfcg = [&](size_t m) -> ls_status {
        Lv& a = lv[m];
        T *rr = a.kv[0], *za = a.kv[1], *zb = a.kv[2], *pd = a.kv[3], *q0 = a.kv[4], *q1 = a.kv[5], *e = a.kv[6];
        const int slot = kKSlot0 + 5 * ((int)m - 1);
        const double* s = c->scal + slot;
        const int gd = grid_for(c, a.g.N);
        LS_CUDA(c, cudaMemcpyAsync(rr, a.b, sizeof(T) * (size_t)a.g.N, cudaMemcpyDeviceToDevice, c->stream));
        LS_TRY(cycle(m, (const T*)rr, za, nullptr, nullptr, nullptr));
        LS_LAUNCH_PDL(c, k_kc_apply<T>, gd, kBlock, 0, a.g, a.comp, a.e, a.f0, a.f1, a.f2, (const T*)za,
                  (const T*)rr, q0, c->partials);
        LS_TRY(finalize_sum(c, gd, 2, slot));  // (za, q0), (za, rr)
        LS_LAUNCH_PDL(c, k_kc_first<T>, gd, kBlock, 0, a.g, a.comp, s, (const T*)za, (const T*)q0, e, rr);
        int nb = 0;
        LS_TRY(cycle(m, (const T*)rr, zb, (const T*)q0, nullptr, &nb));
        LS_TRY(finalize_sum(c, nb, 2, slot + 2));  // (zb, q0)
        LS_LAUNCH_PDL(c, k_kc_dir<T>, gd, kBlock, 0, a.g, a.comp, s, (const T*)zb, (const T*)za, pd);
        LS_LAUNCH_PDL(c, k_kc_apply<T>, gd, kBlock, 0, a.g, a.comp, a.e, a.f0, a.f1, a.f2, (const T*)pd,
                  (const T*)rr, q1, c->partials);
        LS_TRY(finalize_sum(c, gd, 2, slot + 3));  // (pd, q1), (pd, rr)
        LS_LAUNCH_PDL(c, k_kc_second<T>, gd, kBlock, 0, a.g, a.comp, s, (const T*)pd, e);
        return LS_OK;
    };
    // the small coarse levels below the K-cycle run as one block (k_mg_tail)
    size_t tail_start = L + 1;
    if (c->mg_tail_cells > 0)
        for (size_t l = L; l > (size_t)kKLevels && l >= 1 && lv[l].g.N <= c->mg_tail_cells; --l) tail_start = l;
    if (tail_start <= L && L - tail_start + 1 > (size_t)kMaxTail) tail_start = L + 1 - kMaxTail;
    cycle = [&](size_t l, const T* b, T* out, const T* dv, const T* dv2, int* nb) -> ls_status {
        Lv& a = lv[l];
        if (l >= tail_start && !dv && b == a.b && out == a.x) {
            TailLevels<T> tl = {};
            tl.n = (int)(L - l + 1);
            for (int q = 0; q < tl.n; ++q) {
                const Lv& m = lv[l + q];
                tl.g[q] = m.g;
                tl.comp[q] = m.comp;
                tl.e[q] = m.e;
                tl.f0[q] = m.f0;
                tl.f1[q] = m.f1;
                tl.f2[q] = m.f2;
                tl.invd[q] = m.invd;
                tl.x[q] = m.x;
                tl.b[q] = m.b;
                tl.t[q] = m.t;
            }
            LS_LAUNCH_PDL(c, k_mg_tail<T>, 1, 1024, 0, tl, (T)kProlongScale, kCoarseSweeps);
            return LS_OK;
        }
        if (l == L) {
            LS_LAUNCH_PDL(c, k_mg_coarsest<T>, 1, 1024, 0, a.g, a.comp, a.e, a.f0, a.f1, a.f2, a.invd, b, out, a.t,
                      kCoarseSweeps);
            return LS_OK;
        }
        Lv& cl = lv[l + 1];
        LS_TRY(smooth(l, b, (const T*)nullptr, a.t, nullptr, nullptr, nullptr));
        LS_TRY(smooth(l, b, (const T*)a.t, a.x, nullptr, nullptr, nullptr));
        if (l == 0 && pair0) {
            // residual into the free ping-pong buffer, then the per-block sums
            const int N2 = (int)(a.g.N / 2);
            LS_LAUNCH_PDL(c, k_mg_resid0_pair, grid_for(c, N2), kBlock, 0, N2, (int)(a.g.JK / 2), a.g.K / 2,
                      (const int8_t*)c->pkind, (const float*)a.e, (const float*)a.f0, (const float*)a.f1,
                      (const float*)a.f2, (const float*)b, (const float*)a.x, (float*)a.t);
            LS_LAUNCH_PDL(c, k_mg_restrict_gather<T>, grid_for(c, cl.g.N), kBlock, 0, a.g, cl.g, a.comp, cl.comp,
                      (const T*)a.t, cl.b);
        } else {
            LS_LAUNCH_PDL(c, k_mg_restrict<T>, grid_for(c, cl.g.N), kBlock, 0, a.g, cl.g, a.comp, cl.comp, a.e, a.f0,
                      a.f1, a.f2, b, (const T*)a.x, cl.b);
        }
        const T* corr;
        T scale;
        if (l + 1 <= (size_t)kKLevels && l + 1 < L) {
            LS_TRY(kfcg(l + 1));
            corr = cl.kv[6];
            scale = (T)1;  // the FCG steps carry the optimal scaling
        } else if (learned && l + 1 == (size_t)kLearnedLevel) {
            LS_TRY(lpc_solve(c, cl.g, cl.comp, (const float*)cl.b, (float*)cl.x));
            corr = cl.x;
            scale = (T)1;
        } else {
            LS_TRY(cycle(l + 1, (const T*)cl.b, cl.x, nullptr, nullptr, nullptr));
            corr = cl.x;
            scale = (T)kProlongScale;
        }
        LS_LAUNCH_PDL(c, k_mg_prolong<T>, grid_for(c, a.g.N), kBlock, 0, a.g, cl.g, a.comp, cl.comp, corr, a.x,
                  scale);
        LS_TRY(smooth(l, b, (const T*)a.x, a.t, nullptr, nullptr, nullptr));
        return smooth(l, b, (const T*)a.t, out, dv, dv2, nb);
    };
    return cycle(0, r, z, r, dotv2, nblocks_out);
}

// z = B r and the partials of (r, z), (dotv2, z) finalized into slot, slot + 1. The cycle's
// ~150 launches (most on coarse levels, a few microseconds each) are captured into a CUDA graph
// on first use and replayed from then on: one launch per application.
template <typename T>
ls_status mg_precondition(ls_ctx* c, const T* r, T* z, const T* dotv2, int slot) {
    const int learned = (std::is_same<T, float>::value && c->lpc_active && c->lpc_ready) ? 1 : 0;
    const int is64 = sizeof(T) == 8;
    if (c->mg_graphs_off) {
        int nb = 0;
        LS_TRY(mg_apply<T>(c, r, z, dotv2, &nb));
        return finalize_sum(c, nb, 2, slot);
    }
    for (const auto& gr : c->mg_graphs)
        if (gr.r == r && gr.z == z && gr.dv2 == dotv2 && gr.slot == slot && gr.learned == learned &&
            gr.is64 == is64) {
            LS_CUDA(c, cudaGraphLaunch(gr.exec, c->stream));
            c->launches += gr.launches;
            return LS_OK;
        }
    const long long l0 = c->launches;
    LS_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int nb = 0;
    ls_status st = mg_apply<T>(c, r, z, dotv2, &nb);
    if (st == LS_OK) st = finalize_sum(c, nb, 2, slot);
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(c->stream, &graph);
    const long long n = c->launches - l0;
    c->launches = l0;
    if (st != LS_OK || ec != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return st != LS_OK ? st : set_error(c, LS_CUDA_ERROR, std::string("multigrid graph capture: ") +
                                                                  cudaGetErrorString(ec));
    }
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess)
        return set_error(c, LS_CUDA_ERROR, std::string("multigrid graph instantiation: ") + cudaGetErrorString(ei));
    c->mg_graphs.push_back(MGGraph{r, z, dotv2, slot, learned, is64, exec, n});
    LS_CUDA(c, cudaGraphLaunch(exec, c->stream));
    c->launches += n;
    return LS_OK;
}

template ls_status mg_precondition<float>(ls_ctx*, const float*, float*, const float*, int);
template ls_status mg_precondition<double>(ls_ctx*, const double*, double*, const double*, int);
template ls_status inner_invd<float>(ls_ctx*);
template ls_status inner_invd<double>(ls_ctx*);
template ls_status mg_setup<float>(ls_ctx*);
template ls_status mg_setup<double>(ls_ctx*);
template ls_status mg_clear<float>(ls_ctx*);
template ls_status mg_clear<double>(ls_ctx*);
template ls_status mg_apply<float>(ls_ctx*, const float*, float*, const float*, int*);
template ls_status mg_apply<double>(ls_ctx*, const double*, double*, const double*, int*);

}  // namespace ls
