// ls_dissolve.cu - sulphide dissolution of Simulation::updateFrac (src/Simulation.cpp:315-617).
//
// The reference sweeps the grid sequentially (k outer, j, i inner) num_steps times; each
// active mineral voxel (label >= Sulphide, frac > 0) reads the acid and label of its six
// neighbours, consumes acid from them in place and may turn into Pore. Two active voxels
// interact only when their Manhattan distance is at most 2. Ordering the voxels by the
// wavefront index w = i + 2j + 3k respects every such dependence of the sequential sweep
// (w strictly increases along each of them), and two voxels with equal w are never within
// distance 2, so processing the levels w = 0, 1, 2, ... in order, each level in parallel,
// reproduces the sequential result exactly.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "ls_internal.cuh"

namespace ls {

struct DzConst {
    double D, dx, kreac, time_scalar, c_sat, dt_sub;
    double k_eff;      // 1/((1/(D/dx)) + (1/kreac)), the same expression as per neighbour
    DxDiv vol;         // division by the voxel volume dx*dx*dx (exact reciprocal when a power of two)
};

template <typename L>
__device__ __forceinline__ double dz_surface_flux(const Grid& g, const DzConst& dc,
                                                  const L* __restrict__ label,
                                                  const double* __restrict__ acid, bool valid,
                                                  long long nb) {
    // calc_surface_flux, src/Simulation.cpp:520-542
    if (valid) {
        int n_type = (int)label[nb];
        if (n_type == kPore || n_type == kRock) return dc.k_eff * acid[nb];
    }
    return 0.0;
}

// Rate pass (src/Simulation.cpp:320-420) plus counters deciding whether the sweeps can
// change anything: d_int[0] active voxels, [1] active voxels with non-zero flux sum,
// [2] active voxels already at or below the leaching threshold.
template <typename L>
__global__ void __launch_bounds__(kBlock) k_dz_rate(Grid g, DzConst dc, const L* __restrict__ label,
                                                    const double* __restrict__ acid,
                                                    const float* __restrict__ frac,
                                                    int* __restrict__ counters,
                                                    double* __restrict__ partials) {
    double mx[1] = {0.0};
    int n_active = 0, n_flux = 0, n_flip = 0;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        const int t = (int)label[r];
        if (t < kSulphide) continue;
        int i, j, k;
        decode(g, r, i, j, k);
        const long long nbs[6] = {r + g.JK, r - g.JK, r + g.K, r - g.K, r + 1, r - 1};
        const bool val[6] = {i + 1 < g.I, i > 0, j + 1 < g.J, j > 0, k + 1 < g.K, k > 0};
        double flux_sum = 0.0;
#pragma unroll
        for (int d = 0; d < 6; ++d) flux_sum += dz_surface_flux(g, dc, label, acid, val[d], nbs[d]);
        if (t == kSulphide) {
            double area_per_face = dc.dx * dc.dx;
            double voxel_volume = dc.dx * dc.dx * dc.dx;
            double vol_rate = flux_sum * area_per_face;
            double fractional_rate = dc.vol.div(vol_rate);
            (void)voxel_volume;
            if (fractional_rate > mx[0]) mx[0] = fractional_rate;
        }
        if (frac[r] > 0.0f) {
            n_active++;
            if (flux_sum != 0.0) n_flux++;
            if ((double)frac[r] <= 1e-4) n_flip++;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        n_active += __shfl_down_sync(0xffffffffu, n_active, o);
        n_flux += __shfl_down_sync(0xffffffffu, n_flux, o);
        n_flip += __shfl_down_sync(0xffffffffu, n_flip, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (n_active) atomicAdd(&counters[0], n_active);
        if (n_flux) atomicAdd(&counters[1], n_flux);
        if (n_flip) atomicAdd(&counters[2], n_flip);
    }
    block_max_store<1>(mx, partials);
}

__device__ __forceinline__ int dz_level(int i, int j, int k) { return i + 2 * j + 3 * k; }

template <typename L>
__global__ void k_dz_hist(Grid g, const L* __restrict__ label, const float* __restrict__ frac,
                          int* __restrict__ hist) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        if ((int)label[r] >= kSulphide && frac[r] > 0.0f) {
            int i, j, k;
            decode(g, r, i, j, k);
            atomicAdd(&hist[dz_level(i, j, k)], 1);
        }
    }
}

template <typename L>
__global__ void k_dz_scatter(Grid g, const L* __restrict__ label, const float* __restrict__ frac,
                             const int* __restrict__ start, int* __restrict__ cursor,
                             int* __restrict__ list) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        if ((int)label[r] >= kSulphide && frac[r] > 0.0f) {
            int i, j, k;
            decode(g, r, i, j, k);
            int w = dz_level(i, j, k);
            int pos = atomicAdd(&cursor[w], 1);
            list[start[w] + pos] = (int)r;
        }
    }
}

// One voxel of one sub-step (the body of src/Simulation.cpp:475-603).
template <typename L>
__device__ __forceinline__ void dz_voxel(const Grid& g, const DzConst& dc, long long r, L* __restrict__ label,
                                         float* __restrict__ frac, double* __restrict__ acid,
                                         double* __restrict__ precip, double* __restrict__ conc,
                                         int* __restrict__ leached, int* __restrict__ flips) {
    if (!((int)label[r] >= kSulphide && frac[r] > 0.0f)) return;
    int i, j, k;
    decode(g, r, i, j, k);
    const long long nbs[6] = {r + g.JK, r - g.JK, r + g.K, r - g.K, r + 1, r - 1};
    const bool val[6] = {i + 1 < g.I, i > 0, j + 1 < g.J, j > 0, k + 1 < g.K, k > 0};
    double f[6];
#pragma unroll
    for (int d = 0; d < 6; ++d) f[d] = dz_surface_flux(g, dc, label, acid, val[d], nbs[d]);
    double flux_sum = f[0] + f[1] + f[2] + f[3] + f[4] + f[5];
    double area_per_face = dc.dx * dc.dx;
    double mass_loss = flux_sum * area_per_face * dc.dt_sub;
    double fractional_loss = dc.vol.div(mass_loss);
    float fr = (float)((double)frac[r] - (fractional_loss * dc.time_scalar));
    frac[r] = fr;
    if (flux_sum > 0.0) {
#pragma unroll
        for (int d = 0; d < 6; ++d)
            if (val[d]) acid[nbs[d]] -= fractional_loss * (f[d] / flux_sum);
    }
    if ((double)fr <= 1e-4) {
        frac[r] = 0.0f;
        if ((int)label[r] == kSulphide) {
            label[r] = (L)kPore;
            precip[r] = 0.0;
            conc[r] = dc.c_sat;
            const int pos = atomicAdd(leached, 1);
            if (flips) flips[pos] = (int)r;  // a voxel leaches at most once per call
        }
    }
}

// Skewed wavefront over the sub-steps. A voxel's update reads and writes only itself and its
// six face neighbours, so two updates can interact only within Manhattan distance 2, where
// the wavefront index w = i + 2j + 3k differs by at most 6. Level l = w + kDzSkew * s (s the
// sub-step) orders every interacting pair of updates as the sequential sweeps do: in one
// sub-step by w; across sub-steps, (v, s) before (u, s + 1) for every u within distance 2,
// and (u, s) before (v, s + 1) even when u comes after v. Updates of one level never
// interact, so a level runs in parallel, and a call takes nlev + kDzSkew (num_steps - 1)
// levels instead of nlev x num_steps.
constexpr int kDzSkew = 7;

// The (sub-step, voxel) updates of one level are spread over all threads: the level holds
// the slices w = level - kDzSkew s of the sub-steps s it covers; one thread per update.
template <typename L>
__global__ void __launch_bounds__(kBlock) k_dz_skew(Grid g, DzConst dc, int level, int num_steps, int nlev,
                                                    const int* __restrict__ list, const int* __restrict__ tab,
                                                    int nsk, const int* __restrict__ start, L* __restrict__ label,
                                                    float* __restrict__ frac, double* __restrict__ acid,
                                                    double* __restrict__ precip, double* __restrict__ conc,
                                                    int* __restrict__ leached, int* __restrict__ flips) {
    const int s_lo = level >= nlev ? (level - nlev) / kDzSkew + 1 : 0;
    const int s_hi = min(num_steps - 1, level / kDzSkew);
    const int ns = s_hi - s_lo + 1;  // slices of this level, <= ceil(nlev / kDzSkew)
    // running totals of the slices' sizes from the level table the host built (tab: nsk + 1
    // offsets, then per level ns + 1 running totals), into shared memory <= kDzSliceCap slices
    // per pass
    const int* __restrict__ cumg = tab + (nsk + 1) + __ldg(tab + level);
    constexpr int kDzSliceCap = 512;
    __shared__ int cum[kDzSliceCap + 1];
    for (int s0 = 0; s0 < ns; s0 += kDzSliceCap) {
        const int m = min(kDzSliceCap, ns - s0);
        const int base = __ldg(cumg + s0);
        for (int t = threadIdx.x; t <= m; t += blockDim.x) cum[t] = __ldg(cumg + s0 + t) - base;
        __syncthreads();
        const int total = cum[m];
        for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
            int t = 0;
            while (cum[t + 1] <= idx) ++t;
            const int w = level - kDzSkew * (s_lo + s0 + t);
            const long long r = __ldg(list + __ldg(start + w) + (idx - cum[t]));
            dz_voxel<L>(g, dc, r, label, frac, acid, precip, conc, leached, flips);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Sparse schedule. A voxel changes something in a sub-step only when a Pore or Rock neighbour
// holds nonzero acid (flux_sum != 0) or its frac is at the threshold. During a call acid
// changes only by consumption and a label only by a leach (Sulphide -> Pore), which can make
// the leached voxel's own acid visible to its neighbours. The sweeps therefore visit S: the
// voxels live at the start and the active voxels within two face steps of them, in the
// wavefront order (a voxel outside S changes nothing, so dropping it leaves every other
// voxel's inputs as in the full sweep). If a voxel leached during the call has an active
// neighbour outside S, that
// neighbour could have become live: the call is undone (acid from its copy; frac, label,
// precip and conc of S from theirs) and redone with the full wavefront schedule, so the
// result is always the sequential sweep's.
//
// Dense map M over the N voxels: -2 not active, -1 active outside S, 0 in S; during the
// selection -3 / -4 mark the voxels one / two face steps from a live one.

template <typename L>
__global__ void __launch_bounds__(kBlock) k_dz_seed(Grid g, DzConst dc, const L* __restrict__ label,
                                                    const double* __restrict__ acid,
                                                    const float* __restrict__ frac, int* __restrict__ M) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        const int t = (int)label[r];
        const float f = frac[r];
        if (!(t >= kSulphide && f > 0.0f)) {
            M[r] = -2;
            continue;
        }
        int i, j, k;
        decode(g, r, i, j, k);
        const long long nbs[6] = {r + g.JK, r - g.JK, r + g.K, r - g.K, r + 1, r - 1};
        const bool val[6] = {i + 1 < g.I, i > 0, j + 1 < g.J, j > 0, k + 1 < g.K, k > 0};
        double flux_sum = 0.0;
#pragma unroll
        for (int d = 0; d < 6; ++d) flux_sum += dz_surface_flux(g, dc, label, acid, val[d], nbs[d]);
        M[r] = (flux_sum != 0.0 || (double)f <= 1e-4) ? 0 : -1;
    }
}

// active voxels outside S with a face neighbour marked `from` get `to`
__global__ void __launch_bounds__(kBlock) k_dz_grow(Grid g, int* __restrict__ M, int from, int to) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        if (M[r] != -1) continue;
        int i, j, k;
        decode(g, r, i, j, k);
        const bool hit = (i + 1 < g.I && M[r + g.JK] == from) || (i > 0 && M[r - g.JK] == from) ||
                         (j + 1 < g.J && M[r + g.K] == from) || (j > 0 && M[r - g.K] == from) ||
                         (k + 1 < g.K && M[r + 1] == from) || (k > 0 && M[r - 1] == from);
        if (hit) M[r] = to;
    }
}

// S as a list (any order), its members marked 0
__global__ void __launch_bounds__(kBlock) k_dz_collect(Grid g, int* __restrict__ M, int* __restrict__ list,
                                                       unsigned int* __restrict__ count) {
    // block-uniform trip count (block_append is called by every thread of the block)
    for (long long b0 = (long long)blockIdx.x * blockDim.x; b0 < g.N; b0 += (long long)gridDim.x * blockDim.x) {
        const long long r = b0 + threadIdx.x;
        bool in = false;
        if (r < g.N) {
            const int m = M[r];
            in = (m == 0 || m == -3 || m == -4);
            if (in) M[r] = 0;
        }
        block_append(in, (int)r, list, count);
    }
}

// wavefront levels of the listed voxels: histogram, then the list sorted by level
__global__ void k_dz_whist(Grid g, const int* __restrict__ list, int n, int* __restrict__ hist) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        int i, j, k;
        decode(g, list[q], i, j, k);
        atomicAdd(&hist[dz_level(i, j, k)], 1);
    }
}

__global__ void k_dz_wscatter(Grid g, const int* __restrict__ list, int n, const int* __restrict__ start,
                              int* __restrict__ cursor, int* __restrict__ out) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int v = list[q];
        int i, j, k;
        decode(g, v, i, j, k);
        const int w = dz_level(i, j, k);
        out[start[w] + atomicAdd(&cursor[w], 1)] = v;
    }
}

template <typename L>
__global__ void k_dz_save(const int* __restrict__ list, int n, const L* __restrict__ label,
                          const float* __restrict__ frac, const double* __restrict__ precip,
                          const double* __restrict__ conc, L* __restrict__ sl, float* __restrict__ sf,
                          double* __restrict__ sp, double* __restrict__ sc) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int v = list[q];
        sl[q] = label[v];
        sf[q] = frac[v];
        sp[q] = precip[v];
        sc[q] = conc[v];
    }
}

template <typename L>
__global__ void k_dz_restore(const int* __restrict__ list, int n, L* __restrict__ label, float* __restrict__ frac,
                             double* __restrict__ precip, double* __restrict__ conc, const L* __restrict__ sl,
                             const float* __restrict__ sf, const double* __restrict__ sp,
                             const double* __restrict__ sc) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int v = list[q];
        label[v] = sl[q];
        frac[v] = sf[q];
        precip[v] = sp[q];
        conc[v] = sc[q];
    }
}

// a voxel leached during the call with an active neighbour outside S
__global__ void k_dz_check(Grid g, const int* __restrict__ flips, const int* __restrict__ nflips,
                           const int* __restrict__ M, int* __restrict__ bad) {
    const int n = *nflips;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const long long r = flips[q];
        int i, j, k;
        decode(g, r, i, j, k);
        if ((i + 1 < g.I && M[r + g.JK] == -1) || (i > 0 && M[r - g.JK] == -1) || (j + 1 < g.J && M[r + g.K] == -1) ||
            (j > 0 && M[r - g.K] == -1) || (k + 1 < g.K && M[r + 1] == -1) || (k > 0 && M[r - 1] == -1))
            *bad = 1;
    }
}

template <typename L>
static ls_status dissolve_t(ls_ctx* c, double dt, int* leached_out, ls_substep_info* info, double* acid_pre,
                            bool* swept) {
    if (swept) *swept = false;
    const Grid g = c->g;
    const int grid = grid_for(c, g.N);
    DzConst dc;
    dc.D = c->p.D;
    dc.dx = c->p.dx;
    dc.kreac = c->p.kreac;
    dc.time_scalar = c->p.time_scalar;
    dc.c_sat = c->p.c_sat;
    dc.dt_sub = dt;
    {
        double k_trans = dc.D / dc.dx;
        dc.k_eff = 1.0 / ((1.0 / k_trans) + (1.0 / dc.kreac));
        dc.vol = make_dxdiv(dc.dx * dc.dx * dc.dx);
    }
    const L* label = (const L*)c->label;
    // With the acid field identically 0 (known from the transport solve that produced it) every
    // flux sum is k_eff * 0 = 0, the largest rate 0 and the sub-step count 1; with no active
    // voxel at the threshold either, the sweeps would change nothing: the rate pass is skipped.
    if (c->acid_zero && c->dz_no_threshold) {
        if (info) {
            info->max_rate = 0.0;
            info->num_steps = 1;
            info->dt_sub = dt;
        }
        if (leached_out) *leached_out = 0;
        return LS_OK;
    }
    LS_CUDA(c, cudaMemsetAsync(c->d_int, 0, sizeof(int) * 4, c->stream));
    LS_LAUNCH(c, k_dz_rate<L>, grid, kBlock, 0, g, dc, label, (const double*)c->acid,
              (const float*)c->frac, c->d_int, c->partials);
    LS_TRY(finalize_max(c, grid, 1, S_RED0));
    double global_max_rate = 0.0;
    LS_TRY(read_scalars(c, S_RED0, 1, &global_max_rate));
    LS_TRY(read_device(c, c->d_int, c->h_int, sizeof(int) * 4));
    const int n_active = c->h_int[0], n_flux = c->h_int[1], n_flip = c->h_int[2];
    // sub-step count, src/Simulation.cpp:423-452
    double effective_fractional_rate = global_max_rate * c->p.time_scalar;
    double dt_safe = dt;
    if (effective_fractional_rate > 1e-20) dt_safe = 0.1 / effective_fractional_rate;
    double calculated_steps = std::ceil(dt / dt_safe);
    int num_steps = 1;
    if (calculated_steps > 1000) num_steps = 1000;
    else if (calculated_steps > 1.0) num_steps = (int)calculated_steps;
    double dt_sub = dt / num_steps;
    dc.dt_sub = dt_sub;
    if (info) {
        info->max_rate = global_max_rate;
        info->num_steps = num_steps;
        info->dt_sub = dt_sub;
    }
    if (leached_out) *leached_out = 0;
    // With no acid reaching any active voxel and none at the threshold, every sweep leaves
    // every field unchanged (frac -= 0, nothing consumed, nothing flips).
    if (n_active == 0 || (n_flux == 0 && n_flip == 0)) {
        c->dz_no_threshold = 1;
        return LS_OK;
    }
    // after the sweeps every active voxel is above the threshold or has been cleared to 0
    c->dz_no_threshold = 1;

    const int nlev = (g.I - 1) + 2 * (g.J - 1) + 3 * (g.K - 1) + 1;
    auto grow_cap = [&](int need) -> ls_status {
        if (c->dz_cap < need || !c->dz_list) {
            dfree_t(c, &c->dz_list, (size_t)c->dz_cap);
            LS_TRY(dalloc_t(c, &c->dz_list, (size_t)need));
            c->dz_cap = need;
        }
        return LS_OK;
    };
    LS_TRY(grow_cap(n_active));
    if (!c->dz_level_start) {
        LS_TRY(dalloc_t(c, &c->dz_level_start, (size_t)nlev + 1));
        LS_TRY(dalloc_t(c, &c->dz_count, (size_t)nlev + 1));
    }
    int* d_leached = c->d_int + 8;
    int* d_flag = c->d_int + 12;
    // the acid the sweeps start from: for the budget, and for undoing a sparse call
    double* acid0 = acid_pre ? acid_pre : c->pr;
    LS_CUDA(c, cudaMemcpyAsync(acid0, c->acid, sizeof(double) * (size_t)g.N, cudaMemcpyDeviceToDevice, c->stream));
    if (swept) *swept = true;
    std::vector<int> hist(nlev + 1), start(nlev + 1);

    // every sub-step over the wavefront-sorted list (hist[w] voxels of level w from start[w];
    // on the device: dz_count and dz_level_start) by the skewed levels
    // threads per block of the level launches (LS_DZ_THREADS: 32 .. 256)
    static const int dz_threads = [] {
        const char* e = getenv("LS_DZ_THREADS");
        int v = e ? atoi(e) : 64;
        if (v < 32) v = 32;
        if (v > kBlock) v = kBlock;
        return (v / 32) * 32;
    }();
    auto run_sweeps = [&](int* flips) -> ls_status {
        LS_CUDA(c, cudaMemsetAsync(d_leached, 0, sizeof(int), c->stream));
        const int nsk = nlev + kDzSkew * (num_steps - 1);
        // the level table: per level the running totals of its slices' sizes (slice t of level
        // l: w = l - kDzSkew (s_lo + t)), so that no block sums them serially
        std::vector<int>& tab = c->dz_tab_host;
        tab.assign((size_t)nsk + 1, 0);
        std::vector<long long> totals((size_t)nsk, 0);
        for (int l = 0; l < nsk; ++l) {
            tab[l] = (int)(tab.size() - (size_t)(nsk + 1));
            const int s_lo = l >= nlev ? (l - nlev) / kDzSkew + 1 : 0;
            const int s_hi = std::min(num_steps - 1, l / kDzSkew);
            long long acc = 0;
            tab.push_back(0);
            for (int s = s_lo; s <= s_hi; ++s) {
                const int w = l - kDzSkew * s;
                acc += (w >= 0 && w < nlev) ? hist[w] : 0;
                tab.push_back((int)acc);
            }
            totals[l] = acc;
        }
        tab[nsk] = (int)(tab.size() - (size_t)(nsk + 1));
        if ((long long)tab.size() > c->dz_tab_cap) {
            dfree_t(c, &c->dz_tab, (size_t)c->dz_tab_cap);
            c->dz_tab_cap = 0;
            LS_TRY(dalloc_t(c, &c->dz_tab, tab.size()));
            c->dz_tab_cap = (long long)tab.size();
        }
        LS_CUDA(c, cudaMemcpyAsync(c->dz_tab, tab.data(), sizeof(int) * tab.size(), cudaMemcpyHostToDevice, c->stream));
        // small blocks: a level holds tens to thousands of updates of ~100 FP64 operations
        // each (six correctly rounded divisions among them), so its time is the FP64 issue of
        // the busiest SM; blocks of one or two warps put every warp on its own SM
        for (int l = 0; l < nsk; ++l) {
            const long long total = totals[l];
            if (total == 0) continue;
            const int bt = dz_threads;
            const int blocks = (int)std::min<long long>((total + bt - 1) / bt, (long long)c->num_sms * (kBlock / bt) * 8);
            LS_LAUNCH(c, k_dz_skew<L>, blocks, bt, 0, g, dc, l, num_steps, nlev, (const int*)c->dz_list,
                      (const int*)c->dz_tab, nsk, (const int*)c->dz_level_start, (L*)c->label, c->frac, c->acid,
                      c->precip, c->conc, d_leached, flips);
        }
        // the host table must outlive the asynchronous copy: the call ends with a synchronisation
        LS_CUDA(c, cudaStreamSynchronize(c->stream));
        return LS_OK;
    };
    auto prefix = [&](int total) -> ls_status {
        int acc = 0;
        for (int w = 0; w <= nlev; ++w) {
            start[w] = acc;
            acc += hist[w];
        }
        if (acc != total) return set_error(c, LS_CUDA_ERROR, "dissolution: schedule count mismatch");
        return LS_OK;
    };

    // ---- sparse schedule (see above); LS_DZ_SPARSE=0 keeps the full wavefront schedule
    static const bool sparse_on = [] {
        const char* e = getenv("LS_DZ_SPARSE");
        return !(e && e[0] == '0');
    }();
    bool done = false;
    if (sparse_on) {
        LS_TRY(wlist_reset(c));
        int* M = c->wlist;
        LS_LAUNCH(c, k_dz_seed<L>, grid, kBlock, 0, g, dc, label, (const double*)c->acid, (const float*)c->frac, M);
        LS_LAUNCH(c, k_dz_grow, grid, kBlock, 0, g, M, 0, -3);
        LS_LAUNCH(c, k_dz_grow, grid, kBlock, 0, g, M, -3, -4);
        if (c->dz_sel_cap < n_active) {
            const size_t cap = (size_t)c->dz_sel_cap;
            dfree_t(c, &c->dz_sel, cap);
            dfree_t(c, &c->dz_flips, cap);
            dfree_t(c, &c->dz_save_frac, cap);
            dfree_t(c, &c->dz_save_precip, cap);
            dfree_t(c, &c->dz_save_conc, cap);
            dfree(c, &c->dz_save_label, cap * c->label_bytes);
            c->dz_sel_cap = 0;
            LS_TRY(dalloc_t(c, &c->dz_sel, (size_t)n_active));
            LS_TRY(dalloc_t(c, &c->dz_flips, (size_t)n_active));
            LS_TRY(dalloc_t(c, &c->dz_save_frac, (size_t)n_active));
            LS_TRY(dalloc_t(c, &c->dz_save_precip, (size_t)n_active));
            LS_TRY(dalloc_t(c, &c->dz_save_conc, (size_t)n_active));
            LS_TRY(dalloc(c, &c->dz_save_label, (size_t)n_active * c->label_bytes));
            c->dz_sel_cap = n_active;
        }
        LS_LAUNCH(c, k_dz_collect, grid, kBlock, 0, g, M, c->dz_sel, c->wcount);
        unsigned int nsel_u = 0;
        LS_TRY(read_device(c, c->wcount, &nsel_u, sizeof(unsigned int)));
        const int nsel = (int)nsel_u;
        if (nsel < 1 || nsel > n_active) return set_error(c, LS_CUDA_ERROR, "dissolution: bad sparse selection");
        const int sgrid = std::min(grid, (nsel + kBlock - 1) / kBlock);
        // S sorted by wavefront level
        LS_CUDA(c, cudaMemsetAsync(c->dz_count, 0, sizeof(int) * (nlev + 1), c->stream));
        LS_LAUNCH(c, k_dz_whist, sgrid, kBlock, 0, g, (const int*)c->dz_sel, nsel, c->dz_count);
        LS_TRY(read_device(c, c->dz_count, hist.data(), sizeof(int) * (nlev + 1)));
        LS_TRY(prefix(nsel));
        LS_CUDA(c, cudaMemcpyAsync(c->dz_level_start, start.data(), sizeof(int) * (nlev + 1), cudaMemcpyHostToDevice,
                                   c->stream));
        LS_CUDA(c, cudaMemsetAsync(c->dz_count, 0, sizeof(int) * (nlev + 1), c->stream));
        LS_LAUNCH(c, k_dz_wscatter, sgrid, kBlock, 0, g, (const int*)c->dz_sel, nsel, (const int*)c->dz_level_start,
                  c->dz_count, c->dz_list);
        LS_LAUNCH(c, k_dz_save<L>, sgrid, kBlock, 0, (const int*)c->dz_sel, nsel, label, (const float*)c->frac,
                  (const double*)c->precip, (const double*)c->conc, (L*)c->dz_save_label, c->dz_save_frac,
                  c->dz_save_precip, c->dz_save_conc);
        LS_TRY(run_sweeps(c->dz_flips));
        LS_CUDA(c, cudaMemsetAsync(d_flag, 0, sizeof(int), c->stream));
        LS_LAUNCH(c, k_dz_check, sgrid, kBlock, 0, g, (const int*)c->dz_flips, (const int*)d_leached, (const int*)M,
                  d_flag);
        int bad = 0;
        LS_TRY(read_device(c, d_flag, &bad, sizeof(int)));
        if (!bad) {
            done = true;
        } else {
            // undo the call, then the full schedule below
            LS_LAUNCH(c, k_dz_restore<L>, sgrid, kBlock, 0, (const int*)c->dz_sel, nsel, (L*)c->label, c->frac,
                      c->precip, c->conc, (const L*)c->dz_save_label, (const float*)c->dz_save_frac,
                      (const double*)c->dz_save_precip, (const double*)c->dz_save_conc);
            LS_CUDA(c, cudaMemcpyAsync(c->acid, acid0, sizeof(double) * (size_t)g.N, cudaMemcpyDeviceToDevice,
                                       c->stream));
            c->dz_fallbacks++;
        }
    }
    if (!done) {
        // full schedule: every active voxel, sorted by wavefront level
        LS_CUDA(c, cudaMemsetAsync(c->dz_count, 0, sizeof(int) * (nlev + 1), c->stream));
        LS_LAUNCH(c, k_dz_hist<L>, grid, kBlock, 0, g, label, (const float*)c->frac, c->dz_count);
        LS_TRY(read_device(c, c->dz_count, hist.data(), sizeof(int) * (nlev + 1)));
        LS_TRY(prefix(n_active));
        LS_CUDA(c, cudaMemcpyAsync(c->dz_level_start, start.data(), sizeof(int) * (nlev + 1), cudaMemcpyHostToDevice,
                                   c->stream));
        LS_CUDA(c, cudaMemsetAsync(c->dz_count, 0, sizeof(int) * (nlev + 1), c->stream));
        LS_LAUNCH(c, k_dz_scatter<L>, grid, kBlock, 0, g, label, (const float*)c->frac,
                  (const int*)c->dz_level_start, c->dz_count, c->dz_list);
        LS_TRY(run_sweeps(nullptr));
    }
    int h = 0;
    LS_TRY(read_device(c, d_leached, &h, sizeof(int)));
    if (leached_out) *leached_out = h;
    c->p_ready = 0;
    return LS_OK;
}

ls_status dissolve_run(ls_ctx* c, double dt, int* leached, ls_substep_info* info, double* acid_pre,
                       bool* swept) {
    snap_fence(c, kSnapRest);
    if (c->label_bytes == 1) return dissolve_t<uint8_t>(c, dt, leached, info, acid_pre, swept);
    return dissolve_t<uint16_t>(c, dt, leached, info, acid_pre, swept);
}

}  // namespace ls
