// ls_mg.cu - geometric multigrid preconditioner of the inner pressure PCG.
//
// The inner system is W = I - L on the Pore unknowns (Jacobi-scaled, unit diagonal; L
// holds the positive scaled link weights of the +i, +j, +k faces). The Pore network is
// masked by Dirichlet voxels everywhere and its links span ~13 orders of magnitude, so
// plain 2x2x2 aggregation would hand coarse corrections to Pore clusters that merely share
// a block with the main network while being joined to it by no strong link. Such a
// cluster's own near-null mode then absorbs the correction and keeps it (the residual
// there is ~1e-13 of the error). The hierarchy therefore works per strong component:
//   * components: connected pieces of the unknowns over links with w > kStrong
//     (union-find on the device);
//   * aggregation: each 2x2x2 block becomes one coarse cell owned by the component with
//     most members in the block; only those members are restricted to / prolongated from
//     it (piecewise-constant interpolation), the rest are left to the smoother;
//   * coarse operators: Galerkin P^T W P, again a 7-point stencil (diag + 3 face weights);
//   * V-cycle: nu damped-Jacobi sweeps before and after (symmetric), a fixed number of
//     Jacobi sweeps by one CTA on the coarsest level, so the cycle is a symmetric operator
//     usable inside CG.
#include <algorithm>
#include <cstdio>

#include "ls_internal.cuh"

namespace ls {

constexpr double kStrong = 1e-3;   // scaled link weight below which a link does not join components
// two damped-Jacobi sweeps before and two after the coarse correction (mg_apply)
constexpr double kOmega = 2.0 / 3.0;
constexpr int kCoarsestCells = 4096;
constexpr int kCoarseSweeps = 48;
constexpr int kUnionSpin = 1 << 20;  // bound on the union-find retry loop

// ---------------------------------------------------------------------------
// strong components (union-find with path halving; ids are voxel indices, the root is the
// smallest voxel of the component)

__device__ __forceinline__ int cc_find(int* parent, int x) {
    int p = parent[x];
    int guard = 0;
    while (p != x && guard++ < kUnionSpin) {
        int gp = parent[p];
        parent[x] = gp;  // path halving; benign race
        x = p;
        p = gp;
    }
    return x;
}

__global__ void k_cc_init(Grid g, const double* __restrict__ isd, int* __restrict__ parent) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x)
        parent[r] = (isd[r] != 0.0) ? (int)r : -1;
}

template <typename T>
__global__ void k_cc_hook(Grid g, const T* __restrict__ w0, const T* __restrict__ w1,
                          const T* __restrict__ w2, int* parent, int* __restrict__ err) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        if (parent[r] < 0) continue;
        const T* ws[3] = {w0, w1, w2};
        const long long offs[3] = {g.JK, g.K, 1};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            if (!((double)ws[d][r] > kStrong)) continue;  // w > 0 only between two unknowns
            int a = (int)r, b = (int)(r + offs[d]);
            int spins = 0;
            while (true) {
                int ra = cc_find(parent, a), rb = cc_find(parent, b);
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
        parent[r] = cc_find(parent, (int)r);
    }
}

// ---------------------------------------------------------------------------
// hierarchy construction

__device__ __forceinline__ long long lidx(const Grid& g, int i, int j, int k) {
    return (long long)k + (long long)g.K * ((long long)j + (long long)g.J * i);
}

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

// Galerkin coarse operator P^T W P for piecewise-constant P restricted to the members of
// the owning component. fdiag == nullptr means unit diagonal (the finest level).
template <typename T>
__global__ void k_mg_coarse_op(Grid f, Grid cg, const int* __restrict__ fcomp,
                               const int* __restrict__ ccomp, const T* __restrict__ fdiag,
                               const T* __restrict__ fw0, const T* __restrict__ fw1,
                               const T* __restrict__ fw2, T* __restrict__ cdiag,
                               T* __restrict__ cw0, T* __restrict__ cw1, T* __restrict__ cw2) {
    for (long long R = blockIdx.x * (long long)blockDim.x + threadIdx.x; R < cg.N;
         R += (long long)gridDim.x * blockDim.x) {
        int I, J, K;
        decode(cg, R, I, J, K);
        const int own = ccomp[R];
        double dg = 0.0, e0 = 0.0, e1 = 0.0, e2 = 0.0;
        if (own >= 0) {
            for (int a = 0; a < 2; ++a)
                for (int b = 0; b < 2; ++b)
                    for (int c = 0; c < 2; ++c) {
                        int i = 2 * I + a, j = 2 * J + b, k = 2 * K + c;
                        if (i >= f.I || j >= f.J || k >= f.K) continue;
                        long long fr = lidx(f, i, j, k);
                        if (fcomp[fr] != own) continue;
                        dg += fdiag ? (double)fdiag[fr] : 1.0;
                        // + face links of this fine cell
                        if (i + 1 < f.I) {
                            long long nb = fr + f.JK;
                            if (a == 0) { if (fcomp[nb] == own) dg -= 2.0 * (double)fw0[fr]; }
                            else if (I + 1 < cg.I && fcomp[nb] == ccomp[R + cg.JK]) e0 += (double)fw0[fr];
                        }
                        if (j + 1 < f.J) {
                            long long nb = fr + f.K;
                            if (b == 0) { if (fcomp[nb] == own) dg -= 2.0 * (double)fw1[fr]; }
                            else if (J + 1 < cg.J && fcomp[nb] == ccomp[R + cg.K]) e1 += (double)fw1[fr];
                        }
                        if (k + 1 < f.K) {
                            long long nb = fr + 1;
                            if (c == 0) { if (fcomp[nb] == own) dg -= 2.0 * (double)fw2[fr]; }
                            else if (K + 1 < cg.K && fcomp[nb] == ccomp[R + 1]) e2 += (double)fw2[fr];
                        }
                    }
        }
        // the coarse neighbour must also be a live cell
        if (own < 0) { e0 = e1 = e2 = 0.0; dg = 1.0; }
        cdiag[R] = (T)dg;
        cw0[R] = (T)e0;
        cw1[R] = (T)e1;
        cw2[R] = (T)e2;
    }
}

// ---------------------------------------------------------------------------
// V-cycle kernels

template <typename T>
__device__ __forceinline__ T offsum(const Grid& g, long long r, int i, int j, int k,
                                    const T* __restrict__ v, const T* __restrict__ w0,
                                    const T* __restrict__ w1, const T* __restrict__ w2) {
    T acc = (T)0;
    if (i > 0) acc += w0[r - g.JK] * v[r - g.JK];
    if (j > 0) acc += w1[r - g.K] * v[r - g.K];
    if (k > 0) acc += w2[r - 1] * v[r - 1];
    if (k + 1 < g.K) acc += w2[r] * v[r + 1];
    if (j + 1 < g.J) acc += w1[r] * v[r + g.K];
    if (i + 1 < g.I) acc += w0[r] * v[r + g.JK];
    return acc;
}

// x_out = x + omega D^-1 (b - (D x - L x)); x == nullptr means x = 0.
// When dot != nullptr the per-block partial of (dotv, x_out) is stored (for (r, z)).
template <typename T>
__global__ void __launch_bounds__(kBlock) k_mg_smooth(Grid g, const int* __restrict__ comp,
                                                      const T* __restrict__ diag,
                                                      const T* __restrict__ w0,
                                                      const T* __restrict__ w1,
                                                      const T* __restrict__ w2,
                                                      const T* __restrict__ b,
                                                      const T* __restrict__ x,
                                                      T* __restrict__ xo,
                                                      const T* __restrict__ dotv,
                                                      double* __restrict__ partials) {
    double acc[1] = {0.0};
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        T out = (T)0;
        if (comp[r] >= 0) {
            T bv = b[r];
            if (x) {
                int i, j, k;
                decode(g, r, i, j, k);
                T xv = x[r];
                if (diag) {
                    T dg = diag[r];
                    T res = bv - (dg * xv - offsum(g, r, i, j, k, x, w0, w1, w2));
                    out = xv + (T)kOmega * res / dg;
                } else {  // unit diagonal (finest level)
                    T res = bv - (xv - offsum(g, r, i, j, k, x, w0, w1, w2));
                    out = xv + (T)kOmega * res;
                }
            } else {
                out = diag ? (T)kOmega * bv / diag[r] : (T)kOmega * bv;
            }
        }
        xo[r] = out;
        if (dotv) acc[0] += (double)dotv[r] * (double)out;
    }
    if (dotv) block_sum_store<1>(acc, partials);
}

// coarse right-hand side: b_c(R) = sum over owned members of (b - W x)
template <typename T>
__global__ void k_mg_restrict(Grid f, Grid cg, const int* __restrict__ fcomp,
                              const int* __restrict__ ccomp, const T* __restrict__ fdiag,
                              const T* __restrict__ w0, const T* __restrict__ w1,
                              const T* __restrict__ w2, const T* __restrict__ fb,
                              const T* __restrict__ fx, T* __restrict__ cb) {
    for (long long R = blockIdx.x * (long long)blockDim.x + threadIdx.x; R < cg.N;
         R += (long long)gridDim.x * blockDim.x) {
        int I, J, K;
        decode(cg, R, I, J, K);
        const int own = ccomp[R];
        double acc = 0.0;
        if (own >= 0) {
            for (int a = 0; a < 2; ++a)
                for (int b = 0; b < 2; ++b)
                    for (int c = 0; c < 2; ++c) {
                        int i = 2 * I + a, j = 2 * J + b, k = 2 * K + c;
                        if (i >= f.I || j >= f.J || k >= f.K) continue;
                        long long fr = lidx(f, i, j, k);
                        if (fcomp[fr] != own) continue;
                        T dg = fdiag ? fdiag[fr] : (T)1;
                        T res = fb[fr] - (dg * fx[fr] - offsum(f, fr, i, j, k, fx, w0, w1, w2));
                        acc += (double)res;
                    }
        }
        cb[R] = (T)acc;
    }
}

// x_f += x_c(block) for owned members
template <typename T>
__global__ void k_mg_prolong(Grid f, Grid cg, const int* __restrict__ fcomp,
                             const int* __restrict__ ccomp, const T* __restrict__ cx,
                             T* __restrict__ fx) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < f.N;
         r += (long long)gridDim.x * blockDim.x) {
        int id = fcomp[r];
        if (id < 0) continue;
        int i, j, k;
        decode(f, r, i, j, k);
        long long R = lidx(cg, i >> 1, j >> 1, k >> 1);
        if (ccomp[R] == id) fx[r] += cx[R];
    }
}

// coarsest level: fixed number of damped Jacobi sweeps from zero by one CTA
template <typename T>
__global__ void k_mg_coarsest(Grid g, const int* __restrict__ comp, const T* __restrict__ diag,
                              const T* __restrict__ w0, const T* __restrict__ w1,
                              const T* __restrict__ w2, const T* __restrict__ b, T* x, T* t,
                              int sweeps) {
    for (long long r = threadIdx.x; r < g.N; r += blockDim.x)
        x[r] = (comp[r] >= 0) ? (T)kOmega * b[r] / diag[r] : (T)0;
    __syncthreads();
    for (int s = 1; s < sweeps; ++s) {
        for (long long r = threadIdx.x; r < g.N; r += blockDim.x) {
            T out = (T)0;
            if (comp[r] >= 0) {
                int i, j, k;
                decode(g, r, i, j, k);
                T dg = diag[r];
                T res = b[r] - (dg * x[r] - offsum(g, r, i, j, k, x, w0, w1, w2));
                out = x[r] + (T)kOmega * res / dg;
            }
            t[r] = out;
        }
        __syncthreads();
        for (long long r = threadIdx.x; r < g.N; r += blockDim.x) x[r] = t[r];
        __syncthreads();
    }
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
    return c;
}

template <typename T>
static ls_status mg_alloc(ls_ctx* c) {
    const int is64 = sizeof(T) == 8;
    if (!c->mg.empty() && c->mg_is64 == is64) return LS_OK;
    for (auto& lv : c->mg) {
        void* lp[] = {lv.comp, lv.diag, lv.face[0], lv.face[1], lv.face[2], lv.x, lv.b, lv.t};
        for (void* q : lp)
            if (q) cudaFree(q);
    }
    c->mg.clear();
    if (!c->comp) LS_TRY(dalloc_t(c, &c->comp, (size_t)c->g.N));
    if (!c->cc_flag) LS_TRY(dalloc_t(c, &c->cc_flag, (size_t)4));
    // level 0 is the fine grid itself: comp = c->comp, unit diagonal, weights w32/w64; its
    // x/b/t vectors are allocated here
    ls_ctx::MGLevel l0 = {};
    l0.g = c->g;
    l0.g.NP = l0.g.N;
    l0.comp = c->comp;
    LS_TRY(dalloc(c, &l0.x, sizeof(T) * (size_t)l0.g.N));
    LS_TRY(dalloc(c, &l0.t, sizeof(T) * (size_t)l0.g.N));
    c->mg.push_back(l0);
    Grid g = c->g;
    while ((c->mg.size() < 2 || g.N > kCoarsestCells) && (g.I > 1 || g.J > 1 || g.K > 1)) {
        Grid cg = coarse_of(g);
        ls_ctx::MGLevel lv = {};
        lv.g = cg;
        LS_TRY(dalloc_t(c, &lv.comp, (size_t)cg.N));
        LS_TRY(dalloc(c, &lv.diag, sizeof(T) * (size_t)cg.N));
        for (int d = 0; d < 3; ++d) LS_TRY(dalloc(c, &lv.face[d], sizeof(T) * (size_t)cg.N));
        LS_TRY(dalloc(c, &lv.x, sizeof(T) * (size_t)cg.N));
        LS_TRY(dalloc(c, &lv.b, sizeof(T) * (size_t)cg.N));
        LS_TRY(dalloc(c, &lv.t, sizeof(T) * (size_t)cg.N));
        c->mg.push_back(lv);
        g = cg;
    }
    c->mg_is64 = is64;
    return LS_OK;
}

// Build components and coarse operators for the current fine weights.
template <typename T>
ls_status mg_setup(ls_ctx* c, T* const* w) {
    LS_TRY(mg_alloc<T>(c));
    const Grid g = c->g;
    const int grid = grid_for(c, g.N);
    LS_CUDA(c, cudaMemsetAsync(c->cc_flag, 0, sizeof(int), c->stream));
    LS_LAUNCH(c, k_cc_init, grid, kBlock, 0, g, (const double*)c->pisd, c->comp);
    LS_LAUNCH(c, k_cc_hook<T>, grid, kBlock, 0, g, (const T*)w[0], (const T*)w[1], (const T*)w[2],
              c->comp, c->cc_flag);
    LS_LAUNCH(c, k_cc_compress, grid, kBlock, 0, g, c->comp);
    c->mg[0].face[0] = w[0];
    c->mg[0].face[1] = w[1];
    c->mg[0].face[2] = w[2];
    for (size_t l = 1; l < c->mg.size(); ++l) {
        auto& f = c->mg[l - 1];
        auto& cl = c->mg[l];
        const int cgd = grid_for(c, cl.g.N);
        LS_LAUNCH(c, k_mg_dom, cgd, kBlock, 0, f.g, cl.g, (const int*)f.comp, cl.comp);
        LS_LAUNCH(c, k_mg_coarse_op<T>, cgd, kBlock, 0, f.g, cl.g, (const int*)f.comp,
                  (const int*)cl.comp, (const T*)f.diag, (const T*)f.face[0], (const T*)f.face[1],
                  (const T*)f.face[2], (T*)cl.diag, (T*)cl.face[0], (T*)cl.face[1], (T*)cl.face[2]);
    }
    int flag = 0;
    LS_CUDA(c, cudaMemcpyAsync(&flag, c->cc_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    LS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (flag) return set_error(c, LS_TIMEOUT, "multigrid: component labelling gave up");
    return LS_OK;
}

// z = B r (one V-cycle); the partial sums of (r, z) are left in c->partials for the caller.
template <typename T>
ls_status mg_apply(ls_ctx* c, const T* r, T* z, int* nblocks_out) {
    const size_t L = c->mg.size();
    // descending leg: level l solves W_l e = b_l; b_0 = r
    for (size_t l = 0; l + 1 < L; ++l) {
        auto& lv = c->mg[l];
        const T* b = (l == 0) ? r : (const T*)lv.b;
        T* x = (T*)lv.x;
        T* t = (T*)lv.t;
        const int gd = grid_for(c, lv.g.N);
        // nu sweeps from zero, ending in x
        LS_LAUNCH(c, k_mg_smooth<T>, gd, kBlock, 0, lv.g, (const int*)lv.comp, (const T*)lv.diag,
                  (const T*)lv.face[0], (const T*)lv.face[1], (const T*)lv.face[2], b, (const T*)nullptr,
                  t, (const T*)nullptr, (double*)nullptr);
        LS_LAUNCH(c, k_mg_smooth<T>, gd, kBlock, 0, lv.g, (const int*)lv.comp, (const T*)lv.diag,
                  (const T*)lv.face[0], (const T*)lv.face[1], (const T*)lv.face[2], b, (const T*)t,
                  x, (const T*)nullptr, (double*)nullptr);
        auto& cl = c->mg[l + 1];
        LS_LAUNCH(c, k_mg_restrict<T>, grid_for(c, cl.g.N), kBlock, 0, lv.g, cl.g,
                  (const int*)lv.comp, (const int*)cl.comp, (const T*)lv.diag, (const T*)lv.face[0],
                  (const T*)lv.face[1], (const T*)lv.face[2], b, (const T*)x, (T*)cl.b);
    }
    {
        auto& lv = c->mg[L - 1];
        if (L == 1) return set_error(c, LS_BAD_ARG, "multigrid needs at least two levels");
        LS_LAUNCH(c, k_mg_coarsest<T>, 1, 1024, 0, lv.g, (const int*)lv.comp, (const T*)lv.diag,
                  (const T*)lv.face[0], (const T*)lv.face[1], (const T*)lv.face[2],
                  (const T*)lv.b, (T*)lv.x, (T*)lv.t, kCoarseSweeps);
    }
    // ascending leg
    for (size_t l = L - 1; l-- > 0;) {
        auto& lv = c->mg[l];
        auto& cl = c->mg[l + 1];
        const T* b = (l == 0) ? r : (const T*)lv.b;
        T* x = (T*)lv.x;
        T* t = (T*)lv.t;
        const int gd = grid_for(c, lv.g.N);
        LS_LAUNCH(c, k_mg_prolong<T>, gd, kBlock, 0, lv.g, cl.g, (const int*)lv.comp,
                  (const int*)cl.comp, (const T*)cl.x, x);
        LS_LAUNCH(c, k_mg_smooth<T>, gd, kBlock, 0, lv.g, (const int*)lv.comp, (const T*)lv.diag,
                  (const T*)lv.face[0], (const T*)lv.face[1], (const T*)lv.face[2], b, (const T*)x,
                  t, (const T*)nullptr, (double*)nullptr);
        T* out = (l == 0) ? z : x;
        LS_LAUNCH(c, k_mg_smooth<T>, gd, kBlock, 0, lv.g, (const int*)lv.comp, (const T*)lv.diag,
                  (const T*)lv.face[0], (const T*)lv.face[1], (const T*)lv.face[2], b, (const T*)t,
                  out, (l == 0) ? r : (const T*)nullptr, (l == 0) ? c->partials : (double*)nullptr);
        if (l == 0 && nblocks_out) *nblocks_out = gd;
    }
    return LS_OK;
}

template ls_status mg_setup<float>(ls_ctx*, float* const*);
template ls_status mg_setup<double>(ls_ctx*, double* const*);
template ls_status mg_apply<float>(ls_ctx*, const float*, float*, int*);
template ls_status mg_apply<double>(ls_ctx*, const double*, double*, int*);

}  // namespace ls
