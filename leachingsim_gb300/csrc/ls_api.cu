// ls_api.cu - C-ABI entry points, context life cycle, transfers, snapshot, timing and
// the time-step orchestration of src/main.cpp:303-432.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

#include "ls_internal.cuh"

using namespace ls;

namespace ls {

ls_status set_error(ls_ctx* c, ls_status st, const std::string& msg) {
    if (c) c->err = msg;
    return st;
}

ls_status check_cuda(ls_ctx* c, cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return set_error(c, LS_CUDA_ERROR, m);
}

ls_status dalloc(ls_ctx* c, void** p, size_t bytes) {
    if (bytes == 0) bytes = 256;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        char buf[160];
        snprintf(buf, sizeof(buf), "cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
        return set_error(c, LS_CUDA_ERROR, buf);
    }
    c->device_bytes += bytes;
    c->device_peak = std::max(c->device_peak, c->device_bytes);
    static const bool trace = [] {
        const char* e = getenv("LS_ALLOC_TRACE");
        return e && e[0] == '1';
    }();
    if (trace)
        fprintf(stderr, "[ls alloc] %zu bytes, held %zu, peak %zu, phase %d\n", bytes, c->device_bytes,
                c->device_peak, c->arena_phase);
    return LS_OK;
}

static bool in_arena(const ls_ctx* c, const void* p) {
    return c->arena && (const char*)p >= (const char*)c->arena && (const char*)p < (const char*)c->arena + c->arena_size;
}

ls_status walloc(ls_ctx* c, void** p, size_t bytes) {
    if (!c->lean || c->arena_phase == kPhaseNone) return dalloc(c, p, bytes);
    bytes = (std::max(bytes, (size_t)1) + 255) & ~(size_t)255;
    if (c->arena && c->arena_used + bytes <= c->arena_size) {
        *p = (char*)c->arena + c->arena_used;
        c->arena_used += bytes;
        return LS_OK;
    }
    // beyond the arena (the first steps): an array of its own, counted into the arena's next size
    c->arena_overflow += bytes;
    return dalloc(c, p, bytes);
}

void dfree(ls_ctx* c, void** p, size_t bytes) {
    if (!*p) return;
    if (in_arena(c, *p)) {  // the arena is reset as a whole
        *p = nullptr;
        return;
    }
    if (bytes == 0) bytes = 256;
    cudaFree(*p);
    c->device_bytes -= bytes;
    *p = nullptr;
}

// ---------------------------------------------------------------------------
// timing

static cudaEvent_t take_event(ls_ctx* c) {
    if (!c->event_pool.empty()) {
        cudaEvent_t e = c->event_pool.back();
        c->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void region_begin(ls_ctx* c, int timer, cudaEvent_t* start) {
    (void)timer;
    *start = nullptr;
    if (!c->timing) return;
    *start = take_event(c);
    cudaEventRecord(*start, c->stream);
}

void region_end(ls_ctx* c, int timer, cudaEvent_t start) {
    if (!c->timing || !start) return;
    cudaEvent_t stop = take_event(c);
    cudaEventRecord(stop, c->stream);
    c->regions.push_back(TimedRegion{timer, start, stop});
}

static void resolve_regions(ls_ctx* c) {
    if (c->regions.empty()) return;
    cudaStreamSynchronize(c->stream);
    for (auto& r : c->regions) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, r.start, r.stop);
        c->timer_ms[r.timer] += ms;
        c->timer_count[r.timer] += 1;
        c->event_pool.push_back(r.start);
        c->event_pool.push_back(r.stop);
    }
    c->regions.clear();
}

// ---------------------------------------------------------------------------
// reductions

ls_status l0_alloc(ls_ctx* c, int slot, size_t esize, void** out) {
    if (c->l0pad == 0) c->l0pad = ((c->g.JK + 31) / 32) * 32;
    const size_t bytes = esize * ((size_t)c->g.N + 2 * (size_t)c->l0pad);
    LS_TRY(walloc(c, &c->l0base[slot], bytes));
    c->l0bytes[slot] = bytes;
    LS_CUDA(c, cudaMemsetAsync(c->l0base[slot], 0, bytes, c->stream));
    *out = (char*)c->l0base[slot] + esize * (size_t)c->l0pad;
    return LS_OK;
}

void l0_free(ls_ctx* c, int slot, void** p) {
    dfree(c, &c->l0base[slot], c->l0bytes[slot]);
    c->l0bytes[slot] = 0;
    *p = nullptr;
}

__global__ void k_iota(long long n, int* __restrict__ list, unsigned int* __restrict__ count) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x)
        list[r] = (int)r;
    if (blockIdx.x == 0 && threadIdx.x == 0) *count = (unsigned int)n;
}

// Ordered compaction: block b takes the rows of chunk b (kOlistChunk consecutive rows), so the
// list is the chunks' rows in ascending order: count per chunk, one-block exclusive scan,
// then each block writes its chunk's rows tile by tile at its offset.
constexpr int kOlistChunk = 8192;

__device__ __forceinline__ int block_excl_scan(int v, int* total) {
    __shared__ int ws[kBlock / 32];
    const int lane = (int)(threadIdx.x & 31u), warp = (int)(threadIdx.x >> 5);
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < kBlock / 32 ? ws[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kBlock / 32) ws[lane] = w;
    }
    __syncthreads();
    const int before = (warp > 0 ? ws[warp - 1] : 0) + x - v;
    *total = ws[kBlock / 32 - 1];
    __syncthreads();
    return before;
}

__global__ void __launch_bounds__(kBlock) k_olist_count(long long n, const int8_t* __restrict__ kind, int min_kind,
                                                        int* __restrict__ counts) {
    const long long lo = (long long)blockIdx.x * kOlistChunk;
    const long long hi = lo + kOlistChunk < n ? lo + kOlistChunk : n;
    int cnt = 0;
    for (long long r = lo + threadIdx.x; r < hi; r += kBlock) cnt += (int)kind[r] >= min_kind ? 1 : 0;
    int total = 0;
    block_excl_scan(cnt, &total);
    if (threadIdx.x == 0) counts[blockIdx.x] = total;
}

// counts[0 .. nb) -> exclusive offsets in place, counts[nb] = the total; one block
__global__ void __launch_bounds__(kBlock) k_olist_scan(long long nb, int* __restrict__ counts,
                                                       unsigned int* __restrict__ total_out) {
    const long long per = (nb + kBlock - 1) / kBlock;
    const long long lo = threadIdx.x * per, hi = lo + per < nb ? lo + per : nb;
    int sum = 0;
    for (long long q = lo; q < hi; ++q) sum += counts[q];
    int total = 0;
    int run = block_excl_scan(sum, &total);
    for (long long q = lo; q < hi; ++q) {
        const int v = counts[q];
        counts[q] = run;
        run += v;
    }
    if (threadIdx.x == 0) {
        counts[nb] = total;
        *total_out = (unsigned int)total;
    }
}

__global__ void __launch_bounds__(kBlock) k_olist_fill(long long n, const int8_t* __restrict__ kind, int min_kind,
                                                       const int* __restrict__ offsets, int* __restrict__ list) {
    const long long lo = (long long)blockIdx.x * kOlistChunk;
    const long long hi = lo + kOlistChunk < n ? lo + kOlistChunk : n;
    int run = offsets[blockIdx.x];
    for (long long base = lo; base < hi; base += kBlock) {  // block-uniform trip count
        const long long r = base + threadIdx.x;
        const int pred = (r < hi && (int)kind[r] >= min_kind) ? 1 : 0;
        int total = 0;
        const int at = block_excl_scan(pred, &total);
        if (pred) list[run + at] = (int)r;
        run += total;
    }
}

ls_status ordered_list(ls_ctx* c, const int8_t* kind, int min_kind) {
    LS_TRY(wlist_reset(c));
    const long long nb = (c->g.N + kOlistChunk - 1) / kOlistChunk;
    if (!c->olist_counts) {
        LS_TRY(dalloc_t(c, &c->olist_counts, (size_t)nb + 1));
        c->olist_nb = nb;
    }
    LS_LAUNCH(c, k_olist_count, (int)nb, kBlock, 0, c->g.N, kind, min_kind, c->olist_counts);
    LS_LAUNCH(c, k_olist_scan, 1, kBlock, 0, nb, c->olist_counts, c->wcount);
    LS_LAUNCH(c, k_olist_fill, (int)nb, kBlock, 0, c->g.N, kind, min_kind, (const int*)c->olist_counts, c->wlist);
    return LS_OK;
}

ls_status wlist_all(ls_ctx* c) {
    LS_TRY(wlist_reset(c));
    LS_LAUNCH(c, k_iota, grid_for(c, c->g.N), kBlock, 0, c->g.N, c->wlist, c->wcount);
    return LS_OK;
}

void snap_fence(ls_ctx* c, int groups) {
    const int g = groups & c->snap_pending;
    if (!g) return;
    for (int q = 0; q < 5; ++q)
        if (g & (1 << q)) cudaStreamWaitEvent(c->stream, c->snap_ev[q], 0);
    c->snap_pending &= ~g;
}

static void lean_release_pressure(ls_ctx* c) {
    const size_t n = (size_t)c->g.N;
    double** rows[] = {&c->pdiag, &c->pb, &c->pface[0], &c->pface[1], &c->pface[2], &c->pisd, &c->pr,
                       &c->pdelta, &c->psb2, &c->sat_q};
    for (double** q : rows) dfree_t(c, q, n);
    void** inner[] = {&c->ie, &c->iface[0], &c->iface[1], &c->iface[2], &c->iinvd, &c->inner[0],
                      &c->inner[1], &c->inner[2], &c->inner[3], &c->inner[4]};
    for (int q = 0; q < 10; ++q) l0_free(c, q, inner[q]);
    c->inner_is64 = -1;
    mg_free(c);
    dfree_t(c, &c->comp, n);
    dfree_t(c, &c->start_anchor, n);
    c->p_ready = 0;
}

static void lean_release_transport(ls_ctx* c) {
    const size_t n = (size_t)c->g.N;
    for (double*& q : c->tc) dfree_t(c, &q, n);
    for (double*& q : c->tb) dfree_t(c, &q, n);
    for (float*& q : c->to) dfree_t(c, &q, n);
    for (float*& q : c->trhs) dfree_t(c, &q, n);
    dfree_t(c, &c->tinv, n);
    dfree_t(c, &c->tkind, n);
    dfree_t(c, &c->ti, (size_t)c->ti_stride * 7);
    c->t_valid = 0;
}

ls_status lean_phase(ls_ctx* c, int phase) {
    if (!c->lean || c->arena_phase == phase) return LS_OK;
    lean_release_pressure(c);
    lean_release_transport(c);
    c->arena_need = std::max(c->arena_need, c->arena_used + c->arena_overflow);
    c->arena_used = 0;
    c->arena_overflow = 0;
    if (c->arena_need > c->arena_size) {
        // grow (the first switches): the released arrays and the old arena are back with the
        // driver (cudaFree) before the new arena is mapped
        if (c->arena) {
            cudaFree(c->arena);
            c->device_bytes -= c->arena_size;
        }
        c->arena = nullptr;
        c->arena_size = 0;
        c->arena_phase = kPhaseNone;  // the arena itself is not cut from the arena
        LS_TRY(dalloc(c, &c->arena, c->arena_need));
        c->arena_size = c->arena_need;
    }
    c->arena_phase = phase;
    return LS_OK;
}

ls_status wlist_reset(ls_ctx* c) {
    const size_t n = (size_t)c->g.N;
    c->plist_valid = 0;
    if (!c->wlist) LS_TRY(dalloc_t(c, &c->wlist, n));
    if (!c->wcount) LS_TRY(dalloc_t(c, &c->wcount, 4));
    if (!c->dbits) {
        c->dwords = (long long)((n + 31) / 32);
        LS_TRY(dalloc_t(c, &c->dbits, 2 * (size_t)c->dwords));
    }
    LS_CUDA(c, cudaMemsetAsync(c->wcount, 0, sizeof(unsigned int), c->stream));
    return LS_OK;
}

ls_status finalize_sum(ls_ctx* c, int nblocks, int nvals, int out_slot) {
    LS_LAUNCH_PDL(c, k_finalize<false>, nvals, kFinalizeThreads, 0, c->partials, nblocks, nvals,
              c->scal + out_slot);
    return LS_OK;
}

ls_status finalize_max(ls_ctx* c, int nblocks, int nvals, int out_slot) {
    LS_LAUNCH(c, k_finalize<true>, nvals, kFinalizeThreads, 0, c->partials, nblocks, nvals,
              c->scal + out_slot);
    return LS_OK;
}

// Small device-to-host reads (scalars, counters, histograms) go through a kernel that
// writes mapped host memory, not through cudaMemcpyAsync: the copy engines may be carrying
// an output download to the host, and a step's readback queued behind it would wait for it.
__global__ void k_to_host(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, size_t bytes) {
    if (((((uintptr_t)src) | ((uintptr_t)dst) | bytes) & 7u) == 0) {
        for (size_t q = threadIdx.x; q < bytes / 8; q += blockDim.x)
            reinterpret_cast<unsigned long long*>(dst)[q] = reinterpret_cast<const unsigned long long*>(src)[q];
    } else {
        for (size_t b = threadIdx.x; b < bytes; b += blockDim.x) dst[b] = src[b];
    }
}

static ls_status small_host_buffer(ls_ctx* c, size_t bytes) {
    if (bytes <= c->h_small_bytes) return LS_OK;
    LS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (c->h_small) cudaFreeHost(c->h_small);
    c->h_small = nullptr;
    c->hd_small = nullptr;
    c->h_small_bytes = 0;
    const size_t want = std::max(bytes, (size_t)65536);
    LS_CUDA(c, cudaHostAlloc(&c->h_small, want, cudaHostAllocMapped));
    LS_CUDA(c, cudaHostGetDevicePointer(&c->hd_small, c->h_small, 0));
    c->h_small_bytes = want;
    return LS_OK;
}

ls_status read_device(ls_ctx* c, const void* dev, void* out, size_t bytes) {
    if (bytes == 0) return LS_OK;
    LS_TRY(small_host_buffer(c, bytes));
    LS_LAUNCH(c, k_to_host, 1, 256, 0, (const uint8_t*)dev, (uint8_t*)c->hd_small, bytes);
    LS_CUDA(c, cudaStreamSynchronize(c->stream));
    std::memcpy(out, c->h_small, bytes);
    return LS_OK;
}

ls_status read_scalars(ls_ctx* c, int first, int count, double* out) {
    return read_device(c, c->scal + first, out, sizeof(double) * (size_t)count);
}

// ---------------------------------------------------------------------------
// initialisation kernels

// Simulation::initFrac, src/Simulation.cpp:254-278 (the count uses an integer atomic,
// which is order-independent).
template <typename L>
__global__ void k_init_frac(Grid g, const L* __restrict__ label, float* __restrict__ frac,
                            unsigned long long* __restrict__ count) {
    unsigned long long local = 0;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        if ((int)label[r] == kSulphide) {
            frac[r] = 1.0f;
            local++;
        } else {
            frac[r] = 0.0f;
        }
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(count, local);
}

ls_status init_frac_run(ls_ctx* c, unsigned long long* count) {
    unsigned long long* d = reinterpret_cast<unsigned long long*>(c->d_int);
    LS_CUDA(c, cudaMemsetAsync(d, 0, sizeof(unsigned long long), c->stream));
    int grid = grid_for(c, c->g.N);
    if (c->label_bytes == 1)
        LS_LAUNCH(c, k_init_frac<uint8_t>, grid, kBlock, 0, c->g, (const uint8_t*)c->label, c->frac, d);
    else
        LS_LAUNCH(c, k_init_frac<uint16_t>, grid, kBlock, 0, c->g, (const uint16_t*)c->label, c->frac, d);
    unsigned long long h = 0;
    LS_CUDA(c, cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    LS_CUDA(c, cudaStreamSynchronize(c->stream));
    c->initial_sulphide_count = h;
    if (count) *count = h;
    return LS_OK;
}

// Simulation::initSaturation, src/Simulation.cpp:1573-1590.
template <typename L>
__global__ void k_init_sat(Grid g, const L* __restrict__ label, double* __restrict__ sat) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        int t = (int)label[r];
        sat[r] = (t == kPore || t == kSulphide) ? 0.1 : 0.0;
    }
}

ls_status init_saturation_run(ls_ctx* c) {
    int grid = grid_for(c, c->g.N);
    if (c->label_bytes == 1)
        LS_LAUNCH(c, k_init_sat<uint8_t>, grid, kBlock, 0, c->g, (const uint8_t*)c->label, c->sat);
    else
        LS_LAUNCH(c, k_init_sat<uint16_t>, grid, kBlock, 0, c->g, (const uint16_t*)c->label, c->sat);
    return LS_OK;
}

}  // namespace ls

// ===========================================================================
// C-ABI


static void* field_ptr(ls_ctx* c, ls_field f, size_t* esz) {
    switch (f) {
    case LS_F_LABEL: *esz = (size_t)c->label_bytes; return c->label;
    case LS_F_FRAC: *esz = 4; return c->frac;
    case LS_F_PERMEABILITY: *esz = 8; return c->perm;
    case LS_F_VISCOSITY: *esz = 8; return c->visc;
    case LS_F_PRESSURE: *esz = 8; return c->P;
    case LS_F_CONC: *esz = 8; return c->conc;
    case LS_F_ACID: *esz = 8; return c->acid;
    case LS_F_FLUX_X: *esz = 8; return c->fx;
    case LS_F_FLUX_Y: *esz = 8; return c->fy;
    case LS_F_FLUX_Z: *esz = 8; return c->fz;
    case LS_F_SATURATION: *esz = 8; return c->sat;
    case LS_F_CAP_PRESSURE: *esz = 8; return c->pc;
    case LS_F_REL_PERM: *esz = 8; return c->kr;
    case LS_F_PRECIPITATE: *esz = 8; return c->precip;
    case LS_F_KMULT: *esz = 4; return c->kmult;
    default: return nullptr;
    }
}

__global__ void k_fill_f32(float* a, long long n, float v) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x)
        a[r] = v;
}

extern "C" {

void ls_params_default(ls_params* p) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    // src/main.cpp:39 defaults
    p->D = 1.0;
    p->dx = 1.0;
    p->Dpore_fac = 1.0;
    p->kext = 1.0;
    p->kreac = 1.0;
    p->theta = 1.0;
    p->c_sat = 0.95;
    p->evaporative_flux = 0.0;
    p->top_pressure = 10000.0;
    p->max_cap_grad = 50000.0;
    p->porosity = 0.1;
    p->time_scalar = 1.0;
    p->rock_D_fac = 1e-4;
    p->alpha_transfer = 1e-5;
    // src/main.cpp:89-91
    p->vg_n = 2.0;
    p->vg_alpha = 1.0;
    p->s_res = 0.05;
    // never set by the reference (src/Simulation.h:135)
    p->solid_density = 1.0;
    p->compat_shift = 1;
    p->press_rtol = 1e-8;
    p->press_max_it = 10000;
    p->press_solver = LS_PRESS_MIXED;
    p->conc_rtol = 1e-10;
    p->conc_max_it = 10000;
    p->sat_rtol = 1e-10;
    p->sat_max_it = 10000;
    p->bc_mode = LS_BC_REFERENCE;
    p->p_inlet = 1.0;
    p->p_outlet = 0.0;
    p->conc_inlet = 0.0;
    p->acid_inlet = 0.0;
    // src/Simulation.cpp:190-191
    p->pore_permeability = 1.0e-12;
    p->rock_permeability = 1.0e-18;
}

int ls_abi_version(void) { return LS_ABI_VERSION; }

static ls_status validate_params(ls_ctx* c, const ls_params* p) {
    if (!(p->dx > 0.0)) return set_error(c, LS_BAD_ARG, "dx (voxel_size) must be > 0");
    if (!(p->porosity > 0.0)) return set_error(c, LS_BAD_ARG, "porosity must be > 0");
    if (!(p->vg_n > 1.0)) return set_error(c, LS_BAD_ARG, "vg_n must be > 1");
    if (p->press_max_it < 1 || p->conc_max_it < 1 || p->sat_max_it < 1)
        return set_error(c, LS_BAD_ARG, "max_it must be >= 1");
    if (p->press_solver < LS_PRESS_MIXED || p->press_solver > LS_PRESS_LEARNED)
        return set_error(c, LS_BAD_ARG, "unknown press_solver");
    if (p->bc_mode != LS_BC_REFERENCE && p->bc_mode != LS_BC_FLOW_I)
        return set_error(c, LS_BAD_ARG, "unknown bc_mode");
    if (p->memory_mode != LS_MEM_RESIDENT && p->memory_mode != LS_MEM_LEAN)
        return set_error(c, LS_BAD_ARG, "unknown memory_mode");
    if (!(p->pore_permeability > 0.0) || !(p->rock_permeability > 0.0))
        return set_error(c, LS_BAD_ARG, "pore_permeability and rock_permeability must be > 0");
    if (!std::isfinite(p->p_inlet) || !std::isfinite(p->p_outlet) || !std::isfinite(p->conc_inlet) ||
        !std::isfinite(p->acid_inlet))
        return set_error(c, LS_BAD_ARG, "inlet / outlet values must be finite");
    return LS_OK;
}

ls_status ls_create(ls_ctx** out, int I, int J, int K, int label_bytes, const ls_params* params) {
    if (!out) return LS_BAD_ARG;
    *out = nullptr;
    if (I < 2 || J < 2 || K < 2) return LS_BAD_ARG;
    if (label_bytes != 1 && label_bytes != 2) return LS_BAD_ARG;
    long long JK = (long long)J * K;
    long long NP = (long long)(I + 1) * JK;
    // 32-bit voxel ids (dissolution lists) and 32-bit row indices with a plane of padding on
    // each side and a grid stride of headroom (transport inner vectors)
    if (NP + J * (long long)K + (1LL << 22) >= (1LL << 31)) return LS_BAD_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return LS_NO_DEVICE;

    cudaGetLastError();  // a context starts without an error left pending by other code
    ls_ctx* c = new (std::nothrow) ls_ctx();
    if (!c) return LS_BAD_ARG;
    c->inner_is64 = -1;
    c->mg_is64 = -1;
    {
        const char* gv = getenv("LS_MG_GRAPHS");
        c->mg_graphs_off = (gv && gv[0] == '0') ? 1 : 0;
        const char* tv = getenv("LS_MG_TAIL_CELLS");
        c->mg_tail_cells = tv ? atoll(tv) : 4096;
        if (c->mg_tail_cells < 0) c->mg_tail_cells = 0;
        const char* pv = getenv("LS_PDL");
        c->pdl = (pv && pv[0] == '0') ? 0 : 1;
    }
    c->g.I = I; c->g.J = J; c->g.K = K;
    c->g.JK = JK;
    c->g.N = (long long)I * JK;
    c->g.NP = NP;
    grid_init_div(c->g);
    c->label_bytes = label_bytes;
    if (params) c->p = *params; else ls_params_default(&c->p);
    ls_status st = validate_params(c, &c->p);
    if (st != LS_OK) { delete c; return st; }
    cudaGetDevice(&c->device);
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
    if (c->num_sms < 1) c->num_sms = 1;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return LS_CUDA_ERROR;
    }
    if (c->p.memory_mode == LS_MEM_LEAN) {
        c->lean = 1;
        c->mg_graphs_off = 1;  // the hierarchy's arrays move between steps
    }
    if (cudaStreamCreateWithFlags(&c->snap_stream, cudaStreamNonBlocking) != cudaSuccess) {
        c->snap_stream = nullptr;
        ls_destroy(c);
        return LS_CUDA_ERROR;
    }
    for (cudaEvent_t& e : c->snap_ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
            e = nullptr;
            ls_destroy(c);
            return LS_CUDA_ERROR;
        }
    const size_t np = (size_t)NP, n = (size_t)c->g.N;
#define ALLOC(ptr, count)                                                     \
    do {                                                                      \
        st = dalloc_t(c, &(ptr), (count));                                    \
        if (st != LS_OK) { ls_destroy(c); return st; }                         \
        if (cudaMemsetAsync((ptr), 0, sizeof(*(ptr)) * (count), c->stream) != cudaSuccess) { \
            ls_destroy(c);                                                     \
            return LS_CUDA_ERROR;                                              \
        }                                                                      \
    } while (0)
    {
        uint8_t* lb = nullptr;
        ALLOC(lb, np * label_bytes);
        c->label = lb;
    }
    ALLOC(c->frac, np);
    double** f64[] = {&c->perm, &c->visc, &c->P, &c->conc, &c->acid, &c->fx, &c->fy, &c->fz,
                      &c->sat, &c->pc, &c->kr, &c->precip};
    for (double** q : f64) ALLOC(*q, np);
    // the snapshot of src/Simulation.cpp:2312-2328: device arrays, or (lean) host arrays
    void** snap[] = {&c->b_label, (void**)&c->b_frac, (void**)&c->b_precip, (void**)&c->b_sat, (void**)&c->b_P,
                     (void**)&c->b_conc, (void**)&c->b_acid, (void**)&c->b_fx, (void**)&c->b_fy, (void**)&c->b_fz};
    const size_t snap_bytes[] = {np * label_bytes, np * 4, np * 8, np * 8, np * 8, np * 8, np * 8, np * 8,
                                 np * 8, np * 8};
    // (the mineral fractions stay on the device in both layouts: the step's budget reads them)
    const int kSnapFrac = 1;
    if (c->lean) {
        c->b_host_pinned = 1;
        for (int q = 0; q < 10 && c->b_host_pinned; ++q)
            if (q != kSnapFrac && cudaHostAlloc(snap[q], snap_bytes[q], cudaHostAllocDefault) != cudaSuccess)
                c->b_host_pinned = 0;
        if (!c->b_host_pinned) {
            // not enough page-locked memory: pageable arrays (slower copies)
            cudaGetLastError();
            for (int q = 0; q < 10; ++q)
                if (q != kSnapFrac && *snap[q]) cudaFreeHost(*snap[q]), *snap[q] = nullptr;
            for (int q = 0; q < 10; ++q)
                if (q != kSnapFrac && !(*snap[q] = std::calloc(1, snap_bytes[q]))) {
                    ls_destroy(c);
                    return LS_CUDA_ERROR;
                }
        }
        for (int q = 0; q < 10; ++q)
            if (q != kSnapFrac) c->host_bytes += snap_bytes[q];
    }
    for (int q = 0; q < 10; ++q) {
        if (c->lean && q != kSnapFrac) continue;
        st = dalloc(c, snap[q], snap_bytes[q]);
        if (st != LS_OK) { ls_destroy(c); return st; }
        if (cudaMemsetAsync(*snap[q], 0, snap_bytes[q], c->stream) != cudaSuccess) {
            ls_destroy(c);
            return LS_CUDA_ERROR;
        }
    }
    ALLOC(c->pkind, n);
    if (!c->lean) {
        // the pressure rows (lean: allocated by each assembly, released before the transport)
        ALLOC(c->pdiag, n);
        ALLOC(c->pb, n);
        for (int d = 0; d < 3; ++d) ALLOC(c->pface[d], n);
        ALLOC(c->pisd, n);
        ALLOC(c->pr, n);
        ALLOC(c->pdelta, n);
    }
    ALLOC(c->partials, (size_t)kMaxPartials * 8);
    ALLOC(c->scal, (size_t)S_COUNT);
    ALLOC(c->d_int, (size_t)64);
#undef ALLOC
    if (cudaMallocHost(&c->h_scal, sizeof(double) * S_COUNT) != cudaSuccess ||
        cudaMallocHost(&c->h_int, sizeof(int) * 64) != cudaSuccess || small_host_buffer(c, 65536) != LS_OK) {
        ls_destroy(c);
        return LS_CUDA_ERROR;
    }
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
        ls_destroy(c);
        return LS_CUDA_ERROR;
    }
    *out = c;
    return LS_OK;
}

ls_status ls_destroy(ls_ctx* c) {
    if (!c) return LS_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->snap_stream) cudaStreamSynchronize(c->snap_stream);
    // device arrays of dalloc
    auto rel = [c](void* q) {
        if (!q || in_arena(c, q)) return;  // arrays cut from the arena go with it
        cudaFree(q);
    };
    void* snap[] = {c->b_label, c->b_frac, c->b_precip, c->b_sat, c->b_P, c->b_conc, c->b_acid, c->b_fx,
                    c->b_fy, c->b_fz};
    for (int q = 0; q < 10; ++q) {
        if (!snap[q]) continue;
        if (!c->lean || q == 1) rel(snap[q]);  // the mineral fractions: device memory in both layouts
        else if (c->b_host_pinned) cudaFreeHost(snap[q]);
        else std::free(snap[q]);
    }
    void* ptrs[] = {c->label, c->frac, c->perm, c->visc, c->P, c->conc,
                    c->acid, c->fx, c->fy, c->fz, c->sat, c->pc, c->kr, c->precip, c->pkind, c->pdiag, c->pb, c->pface[0], c->pface[1], c->pface[2],
                    c->pisd, c->pr, c->pdelta, c->comp, c->cc_flag, c->tkind, c->tinv, c->dz_list,
                    c->dz_count, c->dz_level_start, c->partials, c->scal, c->d_int,
                    c->sh_label, c->sh_sat, c->sh_precip, c->sh_frac, c->shf_label, c->shf_perm,
                    c->shf_visc, c->psb2, c->sat_q, c->dbits, c->sht_label, c->sht_fx, c->sht_fy, c->sht_fz,
                    c->shq_P, c->shq_C, c->shq_K, c->shq_V, c->shq_fx, c->shq_fy, c->shq_fz,
                    c->solid_bits, c->solid_bits_b,
                    c->wlist, c->wcount, c->olist_counts, c->dz_tab, c->kmult, c->dz_sel, c->dz_flips, c->dz_save_frac,
                    c->dz_save_precip, c->dz_save_conc, c->dz_save_label};
    for (void* q : ptrs) rel(q);
    for (void* q : c->l0base) rel(q);
    for (double* q : c->tc) rel(q);
    for (double* q : c->tb) rel(q);
    for (float* q : c->to) rel(q);
    for (float* q : c->trhs) rel(q);
    rel(c->ti);
    rel(c->start_anchor);
    rel(c->tcount);
    {
        void* lp[] = {c->lpc_c0, c->lpc_c1, c->lpc_c2, c->lpc_out, c->lpc_isd, c->lpc_anchor};
        for (void* q : lp) rel(q);
        if (c->lpc) ls_lpnet_destroy(c->lpc);
    }
    for (auto& gr : c->mg_graphs)
        if (gr.exec) cudaGraphExecDestroy(gr.exec);
    for (auto& lv : c->mg) {
        void* lp[] = {lv.comp, lv.e, lv.face[0], lv.face[1], lv.face[2], lv.invd, lv.x, lv.b, lv.t};
        for (void* q : lp) rel(q);
        for (void* q : lv.kv) rel(q);
    }
    if (c->h_scal) cudaFreeHost(c->h_scal);
    if (c->h_int) cudaFreeHost(c->h_int);
    if (c->h_small) cudaFreeHost(c->h_small);
    for (auto& r : c->regions) {
        cudaEventDestroy(r.start);
        cudaEventDestroy(r.stop);
    }
    for (auto e : c->event_pool) cudaEventDestroy(e);
    if (c->arena) cudaFree(c->arena);
    if (c->stage) cudaFree(c->stage);
    if (c->stage_free) cudaEventDestroy(c->stage_free);
    if (c->snap_stream) {
        cudaStreamSynchronize(c->snap_stream);
        cudaStreamDestroy(c->snap_stream);
    }
    for (cudaEvent_t e : c->snap_ev)
        if (e) cudaEventDestroy(e);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    cudaGetLastError();  // leave no error of the teardown pending for the next context
    return LS_OK;
}

const char* ls_last_error(const ls_ctx* c) { return c ? c->err.c_str() : "null context"; }

ls_status ls_set_params(ls_ctx* c, const ls_params* p) {
    if (!c || !p) return LS_BAD_ARG;
    LS_TRY(validate_params(c, p));
    if (p->memory_mode != c->p.memory_mode)
        return set_error(c, LS_BAD_ARG, "memory_mode is fixed when the context is created");
    // a new boundary model changes the pressure scale: no ratio rescaling of the warm start
    if (p->bc_mode != c->p.bc_mode || p->p_inlet != c->p.p_inlet || p->p_outlet != c->p.p_outlet)
        c->p_eff_prev = 0.0;
    if (p->bc_mode != c->p.bc_mode || p->acid_inlet != c->p.acid_inlet) c->acid_zero = 0;
    c->p = *p;
    c->p_ready = 0;
    c->props_force = 1;  // the property constants may have changed
    return LS_OK;
}

ls_status ls_get_params(const ls_ctx* c, ls_params* p) {
    if (!c || !p) return LS_BAD_ARG;
    *p = c->p;
    return LS_OK;
}

void* ls_stream(ls_ctx* c) { return c ? (void*)c->stream : nullptr; }

ls_status ls_synchronize(ls_ctx* c) {
    if (!c) return LS_BAD_ARG;
    LS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (c->snap_stream) LS_CUDA(c, cudaStreamSynchronize(c->snap_stream));
    return LS_OK;
}

size_t ls_device_bytes(const ls_ctx* c) { return c ? c->device_bytes : 0; }

size_t ls_device_peak_bytes(const ls_ctx* c) { return c ? c->device_peak : 0; }

size_t ls_host_bytes(const ls_ctx* c) { return c ? c->host_bytes : 0; }

static ls_status transfer(ls_ctx* c, ls_field f, void* host, size_t n, int padded, int up,
                          cudaMemcpyKind kind) {
    if (!c || !host) return LS_BAD_ARG;
    if (f == LS_F_KMULT && !c->kmult) {
        // held only once set: allocate with every voxel at 1 (the reference's permeabilities)
        if (!up) return set_error(c, LS_BAD_ARG, "no permeability multiplier has been uploaded");
        LS_TRY(dalloc_t(c, &c->kmult, (size_t)c->g.NP));
        LS_LAUNCH(c, k_fill_f32, grid_for(c, c->g.NP), kBlock, 0, c->kmult, c->g.NP, 1.0f);
    }
    size_t esz = 0;
    void* dev = field_ptr(c, f, &esz);
    if (!dev) return set_error(c, LS_BAD_ARG, "unknown field id");
    const bool flux = f == LS_F_FLUX_X || f == LS_F_FLUX_Y || f == LS_F_FLUX_Z;
    if (flux) LS_TRY(flux_zero_now(c));
    size_t want = padded ? (size_t)c->g.NP : (size_t)c->g.N;
    if (n != want) {
        char buf[128];
        snprintf(buf, sizeof(buf), "field transfer: %zu elements given, %zu expected", n, want);
        return set_error(c, LS_BAD_ARG, buf);
    }
    if (up) {
        snap_fence(c, kSnapAll);
        LS_CUDA(c, cudaMemcpyAsync(dev, host, n * esz, kind, c->stream));
        if (f == LS_F_LABEL || f == LS_F_PERMEABILITY || f == LS_F_VISCOSITY) c->p_ready = 0;
        // outputs of the property kernel written from outside: re-evaluate every voxel
        if (f == LS_F_PERMEABILITY || f == LS_F_VISCOSITY || f == LS_F_CAP_PRESSURE || f == LS_F_REL_PERM ||
            f == LS_F_KMULT)
            c->props_force = 1;
        if (f == LS_F_PRESSURE) c->p_eff_prev = 0.0;
        if (flux) c->fx_is_shadow = 0;
        if (f == LS_F_ACID) c->acid_zero = 0;
        if (f == LS_F_LABEL || f == LS_F_FRAC) c->dz_no_threshold = 0;
    } else {
        LS_CUDA(c, cudaMemcpyAsync(host, dev, n * esz, kind, c->stream));
    }
    LS_CUDA(c, cudaStreamSynchronize(c->stream));
    return LS_OK;
}

static int field_group(int f) {
    switch (f) {
    case LS_F_PRESSURE: return kSnapP;
    case LS_F_FLUX_X: case LS_F_FLUX_Y: case LS_F_FLUX_Z: return kSnapFlux;
    case LS_F_SATURATION: return kSnapSat;
    case LS_F_PERMEABILITY: case LS_F_VISCOSITY: case LS_F_CAP_PRESSURE: case LS_F_REL_PERM: return kSnapProps;
    default: return kSnapRest;
    }
}

// Device-to-device copy of `bytes` bytes on the SMs: 16-byte words, then the bytes after the
// last whole word (the snapshot's and the staging buffers are 256-byte aligned).
__global__ void k_dcopy(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, size_t bytes) {
    const size_t n16 = bytes / 16;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n16; q += stride)
        reinterpret_cast<uint4*>(dst)[q] = __ldg(reinterpret_cast<const uint4*>(src) + q);
    for (size_t b = n16 * 16 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; b < bytes; b += stride) dst[b] = src[b];
}

// The snapshot, the rollback and the output staging copy on the SMs rather than with
// cudaMemcpyAsync: the copy engines carry the output downloads to the host, and a step's
// snapshot queued behind one of those would wait for it.
static ls_status dcopy(ls_ctx* c, void* dst, const void* src, size_t bytes) {
    if (bytes == 0) return LS_OK;
    if ((((uintptr_t)dst) | ((uintptr_t)src)) & 15u) {
        LS_CUDA(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, c->stream));
        return LS_OK;
    }
    LS_LAUNCH(c, k_dcopy, grid_for(c, (long long)(bytes / 16 + 1)), kBlock, 0, (const uint8_t*)src, (uint8_t*)dst,
              bytes);
    return LS_OK;
}

ls_status ls_download_fields_async(ls_ctx* c, int count, const int* fields, void* const* hosts, int padded,
                                   void** done) {
    if (!c || count < 1 || !fields || !hosts || !done) return c ? set_error(c, LS_BAD_ARG, "bad arguments") : LS_BAD_ARG;
    *done = nullptr;
    const size_t n = padded ? (size_t)c->g.NP : (size_t)c->g.N;
    struct Item { void* dev; void* host; size_t bytes; int group; };
    std::vector<Item> items;
    for (int q = 0; q < count; ++q) {
        size_t esz = 0;
        void* dev = field_ptr(c, (ls_field)fields[q], &esz);
        if (!dev || !hosts[q]) return set_error(c, LS_BAD_ARG, "ls_download_fields_async: unknown field or null buffer");
        if (fields[q] == LS_F_FLUX_X || fields[q] == LS_F_FLUX_Y || fields[q] == LS_F_FLUX_Z)
            LS_TRY(flux_zero_now(c));
        items.push_back({dev, hosts[q], n * esz, field_group(fields[q])});
    }
    cudaEvent_t ev = nullptr;
    LS_CUDA(c, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaStream_t ss = c->snap_stream;
    size_t total = 0;
    for (const Item& it : items) total += (it.bytes + 255) & ~(size_t)255;
    if (!c->lean) {
        // resident layout: device copies into the staging buffer on the context's stream (the
        // fields are free to change right after), then the copies to the host from there
        if (c->stage_bytes < total) {
            if (c->stage) {
                LS_CUDA(c, cudaStreamSynchronize(ss));
                dfree(c, &c->stage, c->stage_bytes);
                c->stage_bytes = 0;
            }
            LS_TRY(dalloc(c, &c->stage, total));
            c->stage_bytes = total;
        } else if (c->stage_free) {
            LS_CUDA(c, cudaStreamWaitEvent(c->stream, c->stage_free, 0));  // the last batch is out of it
        }
        if (!c->stage_free) LS_CUDA(c, cudaEventCreateWithFlags(&c->stage_free, cudaEventDisableTiming));
        size_t off = 0;
        for (Item& it : items) {
            void* dst = (char*)c->stage + off;
            LS_TRY(dcopy(c, dst, it.dev, it.bytes));
            it.dev = dst;
            off += (it.bytes + 255) & ~(size_t)255;
        }
        LS_CUDA(c, cudaEventRecord(c->snap_ev[5], c->stream));
        LS_CUDA(c, cudaStreamWaitEvent(ss, c->snap_ev[5], 0));
        for (const Item& it : items) LS_CUDA(c, cudaMemcpyAsync(it.host, it.dev, it.bytes, cudaMemcpyDefault, ss));
        LS_CUDA(c, cudaEventRecord(c->stage_free, ss));
        LS_CUDA(c, cudaEventRecord(ev, ss));
        *done = ev;
        return LS_OK;
    }
    // lean layout (no room for a staging buffer): straight from the fields, and the kernels
    // that overwrite one wait for its copy
    LS_CUDA(c, cudaEventRecord(c->snap_ev[5], c->stream));
    LS_CUDA(c, cudaStreamWaitEvent(ss, c->snap_ev[5], 0));
    // in the order the next step overwrites the groups
    for (int q : {4, 0, 1, 2, 3}) {
        const int g = 1 << q;
        bool any = false;
        for (const Item& it : items)
            if (it.group == g) {
                LS_CUDA(c, cudaMemcpyAsync(it.host, it.dev, it.bytes, cudaMemcpyDefault, ss));
                any = true;
            }
        if (any) {
            LS_CUDA(c, cudaEventRecord(c->snap_ev[q], ss));
            c->snap_pending |= g;
        }
    }
    LS_CUDA(c, cudaEventRecord(ev, ss));
    *done = ev;
    return LS_OK;
}

ls_status ls_event_wait(void* done) {
    if (!done) return LS_BAD_ARG;
    return cudaEventSynchronize((cudaEvent_t)done) == cudaSuccess ? LS_OK : LS_CUDA_ERROR;
}

void ls_event_release(void* done) {
    if (done) cudaEventDestroy((cudaEvent_t)done);
}

void* ls_host_alloc(size_t bytes) {
    void* p = nullptr;
    if (cudaHostAlloc(&p, bytes ? bytes : 1, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

void ls_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

__global__ void k_count_nonfinite(long long n, const double* __restrict__ v, double* __restrict__ partials) {
    double acc[1] = {0.0};
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x)
        if ((__double_as_longlong(v[r]) & 0x7ff0000000000000ll) == 0x7ff0000000000000ll) acc[0] += 1.0;
    block_sum_store<1>(acc, partials);
}

ls_status ls_count_nonfinite(ls_ctx* c, ls_field f, long long* count) {
    if (!c || !count) return c ? set_error(c, LS_BAD_ARG, "null count") : LS_BAD_ARG;
    size_t esz = 0;
    void* dev = field_ptr(c, f, &esz);
    if (!dev || esz != 8) return set_error(c, LS_BAD_ARG, "ls_count_nonfinite: an FP64 field is needed");
    if (f == LS_F_FLUX_X || f == LS_F_FLUX_Y || f == LS_F_FLUX_Z) LS_TRY(flux_zero_now(c));
    const int grid = grid_for(c, c->g.N);
    LS_LAUNCH(c, k_count_nonfinite, grid, kBlock, 0, c->g.N, (const double*)dev, c->partials);
    LS_TRY(finalize_sum(c, grid, 1, S_RED0));
    double v = 0.0;
    LS_TRY(read_scalars(c, S_RED0, 1, &v));
    *count = (long long)v;
    return LS_OK;
}

ls_status ls_upload_field(ls_ctx* c, ls_field f, const void* host, size_t n, int padded) {
    return transfer(c, f, const_cast<void*>(host), n, padded, 1, cudaMemcpyHostToDevice);
}
ls_status ls_download_field(ls_ctx* c, ls_field f, void* host, size_t n, int padded) {
    return transfer(c, f, host, n, padded, 0, cudaMemcpyDeviceToHost);
}
ls_status ls_upload_field_device(ls_ctx* c, ls_field f, const void* dev, size_t n, int padded) {
    return transfer(c, f, const_cast<void*>(dev), n, padded, 1, cudaMemcpyDeviceToDevice);
}
ls_status ls_download_field_device(ls_ctx* c, ls_field f, void* dev, size_t n, int padded) {
    return transfer(c, f, dev, n, padded, 0, cudaMemcpyDeviceToDevice);
}

// Simulation::initFields, src/Simulation.cpp:165-180.
ls_status ls_init_fields(ls_ctx* c) {
    if (!c) return LS_BAD_ARG;
    snap_fence(c, kSnapAll);
    size_t bytes = sizeof(double) * (size_t)c->g.NP;
    double* f[] = {c->P, c->conc, c->fx, c->fy, c->fz, c->sat, c->pc, c->kr, c->precip};
    for (double* q : f) LS_CUDA(c, cudaMemsetAsync(q, 0, bytes, c->stream));
    c->flux_zero_pending = 0;
    c->fx_is_shadow = 0;
    c->p_ready = 0;
    c->p_eff_prev = 0.0;
    c->props_force = 1;  // kr and Pc were cleared
    c->acid_zero = 0;
    return LS_OK;
}

ls_status ls_init_frac(ls_ctx* c, unsigned long long* count) {
    if (!c) return LS_BAD_ARG;
    snap_fence(c, kSnapAll);
    c->dz_no_threshold = 0;
    return init_frac_run(c, count);
}

ls_status ls_init_saturation(ls_ctx* c) {
    if (!c) return LS_BAD_ARG;
    snap_fence(c, kSnapAll);
    return init_saturation_run(c);
}

// Simulation::initAcid, src/Simulation.cpp:285-310.
ls_status ls_init_acid(ls_ctx* c) {
    if (!c) return LS_BAD_ARG;
    snap_fence(c, kSnapAll);
    LS_CUDA(c, cudaMemsetAsync(c->acid, 0, sizeof(double) * (size_t)c->g.N, c->stream));
    c->acid_zero = 0;  // the plane beyond N keeps what it held
    return LS_OK;
}

ls_status ls_props(ls_ctx* c) {
    if (!c) return LS_BAD_ARG;
    Timed tm(c, LS_T_PROPS);
    return props_run(c);
}

ls_status ls_pressure_setup(ls_ctx* c, double t) {
    if (!c) return LS_BAD_ARG;
    Timed tm(c, LS_T_PRESS_SETUP);
    return pressure_setup_run(c, t);
}

ls_status ls_pressure_step(ls_ctx* c, double t, ls_solve_info* info) {
    if (!c) return LS_BAD_ARG;
    {
        Timed tm(c, LS_T_PRESS_SETUP);
        LS_TRY(pressure_setup_run(c, t));
    }
    return pressure_solve_run(c, info);
}

ls_status ls_pressure_learned_inputs(ls_ctx* c, float* mask, float* logk, float* bc) {
    if (!c || !mask || !logk || !bc) return LS_BAD_ARG;
    return pressure_learned_inputs_run(c, mask, logk, bc);
}

ls_status ls_pressure_solve_start(ls_ctx* c, const float* start, double scale, ls_solve_info* info) {
    if (!c || !start || !(scale == scale)) return LS_BAD_ARG;
    return pressure_solve_run(c, info, start, scale);
}

ls_status ls_pressure_set_precond_weights(ls_ctx* c, const float* params, long long count) {
    if (!c || count < 0 || (count > 0 && !params)) return LS_BAD_ARG;
    if (c->lpc && count > 0) {
        // the network exists already: check and load before keeping the copy, so that a
        // rejected call leaves the weights in use unchanged
        if (ls_lpnet_param_count(c->lpc) != count)
            return set_error(c, LS_BAD_ARG, "learned pressure solver: weight count does not match the network");
        const ls_status st = ls_lpnet_set_params(c->lpc, params, count);
        if (st != LS_OK) return set_error(c, st, "learned pressure solver: loading the weights failed");
    }
    c->lpc_params.assign(params, params + count);
    return LS_OK;
}

long long ls_pressure_fallbacks(const ls_ctx* c) { return c ? c->press_fallbacks : 0; }

long long ls_dissolve_fallbacks(const ls_ctx* c) { return c ? c->dz_fallbacks : 0; }

ls_status ls_pressure_mg_level(ls_ctx* c, int level, int* dims, int* comp, float* e, float* f0, float* f1,
                               float* f2) {
    if (!c || !dims || level < 1) return LS_BAD_ARG;
    if (c->mg_is64 != 0 || (size_t)level > c->mg.size())
        return set_error(c, LS_BAD_ARG, "no FP32 multigrid level of that number (run a mixed-precision solve first)");
    const auto& lv = c->mg[level - 1];
    dims[0] = lv.g.I;
    dims[1] = lv.g.J;
    dims[2] = lv.g.K;
    const size_t n = (size_t)lv.g.N;
    const void* src[5] = {lv.comp, lv.e, lv.face[0], lv.face[1], lv.face[2]};
    void* dst[5] = {comp, e, f0, f1, f2};
    for (int q = 0; q < 5; ++q)
        if (dst[q]) LS_CUDA(c, cudaMemcpyAsync(dst[q], src[q], 4 * n, cudaMemcpyDeviceToHost, c->stream));
    LS_CUDA(c, cudaStreamSynchronize(c->stream));
    return LS_OK;
}

ls_status ls_pressure_apply(ls_ctx* c, const double* x, double* y) {
    if (!c || !x || !y) return LS_BAD_ARG;
    if (!c->p_ready) return set_error(c, LS_BAD_ARG, "ls_pressure_setup must run first");
    return pressure_apply_run(c, x, y);
}

ls_status ls_pressure_rhs(ls_ctx* c, double* b) {
    if (!c || !b) return LS_BAD_ARG;
    if (!c->p_ready) return set_error(c, LS_BAD_ARG, "ls_pressure_setup must run first");
    LS_CUDA(c, cudaMemcpyAsync(b, c->pb, sizeof(double) * (size_t)c->g.N, cudaMemcpyDeviceToHost,
                               c->stream));
    LS_CUDA(c, cudaStreamSynchronize(c->stream));
    return LS_OK;
}

ls_status ls_flux(ls_ctx* c) {
    if (!c) return LS_BAD_ARG;
    Timed tm(c, LS_T_FLUX);
    return flux_run(c);
}

ls_status ls_saturation(ls_ctx* c, double dt, ls_substep_info* info) {
    if (!c || !(dt > 0.0)) return c ? set_error(c, LS_BAD_ARG, "dt must be > 0") : LS_BAD_ARG;
    Timed tm(c, LS_T_SATURATION);
    return saturation_run(c, dt, info);
}

ls_status ls_saturation_implicit(ls_ctx* c, double dt, ls_solve_info* info) {
    if (!c || !(dt > 0.0)) return c ? set_error(c, LS_BAD_ARG, "dt must be > 0") : LS_BAD_ARG;
    Timed tm(c, LS_T_SATURATION);
    return saturation_implicit_run(c, dt, info);
}

ls_status ls_surface(ls_ctx* c) {
    if (!c) return LS_BAD_ARG;
    Timed tm(c, LS_T_PRECIP);
    return surface_run(c);
}

ls_status ls_transport(ls_ctx* c, double dt, int which, ls_solve_info* ci, ls_solve_info* ai) {
    if (!c || !(dt > 0.0)) return c ? set_error(c, LS_BAD_ARG, "dt must be > 0") : LS_BAD_ARG;
    if (which < 1 || which > 3) return set_error(c, LS_BAD_ARG, "which must be 1, 2 or 3");
    Timed tm(c, LS_T_TRANSPORT);
    return transport_run(c, dt, which, ci, ai);
}

ls_status ls_transport_apply(ls_ctx* c, double dt, const double* x, double* y) {
    if (!c || !x || !y || !(dt > 0.0)) return LS_BAD_ARG;
    return transport_apply_run(c, dt, x, y);
}

ls_status ls_precip(ls_ctx* c) {
    if (!c) return LS_BAD_ARG;
    Timed tm(c, LS_T_PRECIP);
    return precip_run(c);
}

ls_status ls_dissolve(ls_ctx* c, double dt, int* leached, ls_substep_info* info) {
    if (!c || !(dt > 0.0)) return c ? set_error(c, LS_BAD_ARG, "dt must be > 0") : LS_BAD_ARG;
    Timed tm(c, LS_T_DISSOLVE);
    return dissolve_run(c, dt, leached, info, nullptr, nullptr);
}

// Simulation::saveState, src/Simulation.cpp:2312-2328.
ls_status ls_snapshot(ls_ctx* c) {
    if (!c) return LS_BAD_ARG;
    Timed tm(c, LS_T_SNAPSHOT);
    // the fluxes are copied as they are, with the zeroing still owed and the voxels it covers
    c->flux_zero_pending_b = c->flux_zero_pending;
    if (c->flux_zero_pending)
        LS_TRY(dcopy(c, c->solid_bits_b, c->solid_bits, sizeof(unsigned int) * (size_t)((c->g.N + 31) / 32)));
    size_t np = (size_t)c->g.NP, d8 = np * sizeof(double);
    cudaStream_t s = c->stream;
    LS_TRY(dcopy(c, c->b_frac, c->frac, np * sizeof(float)));
    if (c->lean) {
        // to host memory on the snapshot stream, from the state the context's stream has
        // reached here, in the order the step overwrites the fields (snap_fence)
        snap_fence(c, kSnapAll);  // a previous snapshot's copies are done before these start
        cudaStream_t ss = c->snap_stream;
        LS_CUDA(c, cudaEventRecord(c->snap_ev[5], s));
        LS_CUDA(c, cudaStreamWaitEvent(ss, c->snap_ev[5], 0));
        LS_CUDA(c, cudaMemcpyAsync(c->b_P, c->P, d8, cudaMemcpyDefault, ss));
        LS_CUDA(c, cudaEventRecord(c->snap_ev[0], ss));
        for (auto pr : {std::make_pair(c->b_fx, c->fx), std::make_pair(c->b_fy, c->fy), std::make_pair(c->b_fz, c->fz)})
            LS_CUDA(c, cudaMemcpyAsync(pr.first, pr.second, d8, cudaMemcpyDefault, ss));
        LS_CUDA(c, cudaEventRecord(c->snap_ev[1], ss));
        LS_CUDA(c, cudaMemcpyAsync(c->b_sat, c->sat, d8, cudaMemcpyDefault, ss));
        LS_CUDA(c, cudaEventRecord(c->snap_ev[2], ss));
        LS_CUDA(c, cudaMemcpyAsync(c->b_label, c->label, np * c->label_bytes, cudaMemcpyDefault, ss));
        for (auto pr : {std::make_pair(c->b_conc, c->conc), std::make_pair(c->b_acid, c->acid),
                        std::make_pair(c->b_precip, c->precip)})
            LS_CUDA(c, cudaMemcpyAsync(pr.first, pr.second, d8, cudaMemcpyDefault, ss));
        LS_CUDA(c, cudaEventRecord(c->snap_ev[3], ss));
        c->snap_pending = kSnapP | kSnapFlux | kSnapSat | kSnapRest;
        return LS_OK;
    }
    LS_TRY(dcopy(c, c->b_label, c->label, np * c->label_bytes));
    const std::pair<double*, double*> pairs[] = {
        {c->b_precip, c->precip}, {c->b_sat, c->sat}, {c->b_P, c->P}, {c->b_conc, c->conc},
        {c->b_acid, c->acid}, {c->b_fx, c->fx}, {c->b_fy, c->fy}, {c->b_fz, c->fz}};
    for (auto& pr : pairs) LS_TRY(dcopy(c, pr.first, pr.second, d8));
    return LS_OK;
}

// Simulation::restoreState, src/Simulation.cpp:2330-2353 (copy back, rebuild properties).
ls_status ls_rollback(ls_ctx* c) {
    if (!c) return LS_BAD_ARG;
    {
        Timed tm(c, LS_T_SNAPSHOT);
        size_t np = (size_t)c->g.NP, d8 = np * sizeof(double);
        cudaStream_t s = c->stream;
        snap_fence(c, kSnapAll);  // lean: the snapshot's copies to the host are done
        const cudaMemcpyKind kind = c->lean ? cudaMemcpyDefault : cudaMemcpyDeviceToDevice;  // lean: from host
        LS_CUDA(c, cudaMemcpyAsync(c->label, c->b_label, np * c->label_bytes, kind, s));
        LS_CUDA(c, cudaMemcpyAsync(c->frac, c->b_frac, np * sizeof(float), kind, s));
        const std::pair<double*, double*> pairs[] = {
            {c->precip, c->b_precip}, {c->sat, c->b_sat}, {c->P, c->b_P}, {c->conc, c->b_conc},
            {c->acid, c->b_acid}, {c->fx, c->b_fx}, {c->fy, c->b_fy}, {c->fz, c->b_fz}};
        for (auto& pr : pairs) LS_CUDA(c, cudaMemcpyAsync(pr.first, pr.second, d8, kind, s));
    }
    c->flux_zero_pending = c->flux_zero_pending_b;
    if (c->flux_zero_pending)
        LS_TRY(dcopy(c, c->solid_bits, c->solid_bits_b, sizeof(unsigned int) * (size_t)((c->g.N + 31) / 32)));
    c->fx_is_shadow = 0;
    c->p_ready = 0;
    c->p_eff_prev = 0.0;
    c->acid_zero = 0;
    c->dz_no_threshold = 0;
    return ls_props(c);
}

static bool solve_failed(ls_status st) { return st == LS_NOT_CONVERGED || st == LS_NONFINITE; }

// One attempt of src/main.cpp:303-432.
ls_status ls_step(ls_ctx* c, double t, double dt, ls_step_info* info) {
    if (!c || !(dt > 0.0)) return c ? set_error(c, LS_BAD_ARG, "dt must be > 0") : LS_BAD_ARG;
    ls_step_info loc;
    memset(&loc, 0, sizeof(loc));
    LS_TRY(ls_snapshot(c));
    bool ok = true;
    ls_status st = LS_OK;
    const int max_picard = c->p.use_implicit_saturation ? 3 : 1;
    bool physics_valid = true;
    for (int picard = 0; picard < max_picard; ++picard) {
        loc.picard_iterations = picard + 1;
        LS_TRY(ls_props(c));
        st = ls_pressure_step(c, t, &loc.pressure);
        if (solve_failed(st)) { ok = false; break; }
        if (st != LS_OK && st != LS_STAGNATED_FALLBACK_USED) return st;
        LS_TRY(ls_flux(c));
        if (c->p.use_implicit_saturation) {
            st = ls_saturation_implicit(c, dt, &loc.saturation_solve);
            if (solve_failed(st)) { ok = false; break; }
            if (st == LS_UNPHYSICAL) physics_valid = false;
            else { physics_valid = true; if (st != LS_OK) return st; }
        } else {
            LS_TRY(ls_saturation(c, dt, &loc.saturation));
        }
    }
    if (ok && c->p.use_implicit_saturation && !physics_valid) ok = false;
    if (ok) {
        LS_TRY(ls_surface(c));
        st = ls_transport(c, dt, 3, &loc.conc, &loc.acid);
        if (solve_failed(st)) ok = false;
        else if (st != LS_OK) return st;
    }
    if (ok) {
        LS_TRY(ls_precip(c));
        {
            // the sweep keeps the acid it starts from in the pressure residual buffer (free
            // between pressure solves) for the budget's consumed acid; lean: the pressure
            // arrays are released by now, and the first transport right-hand side is free
            Timed tm(c, LS_T_DISSOLVE);
            double* acid_pre = c->pr;
            if (c->lean) {
                LS_TRY(lean_phase(c, kPhaseTransport));
                if (!c->tb[0]) LS_TRY(walloc_t(c, &c->tb[0], (size_t)c->g.N));
                acid_pre = c->tb[0];
            }
            bool swept = false;
            LS_TRY(dissolve_run(c, dt, &loc.leached, &loc.leaching, acid_pre, &swept));
            LS_TRY(budget_run(c, swept ? acid_pre : nullptr, &loc.budget));
        }
    }
    loc.success = ok ? 1 : 0;
    if (info) *info = loc;
    return LS_OK;
}

ls_status ls_timing_enable(ls_ctx* c, int enable) {
    if (!c) return LS_BAD_ARG;
    if (!enable) resolve_regions(c);
    c->timing = enable ? 1 : 0;
    return LS_OK;
}

ls_status ls_timing_reset(ls_ctx* c) {
    if (!c) return LS_BAD_ARG;
    resolve_regions(c);
    for (int q = 0; q < LS_T_COUNT; ++q) {
        c->timer_ms[q] = 0.0;
        c->timer_count[q] = 0;
        c->timer_bytes[q] = 0.0;
    }
    c->launches = 0;
    return LS_OK;
}

ls_status ls_timing_get(ls_ctx* c, ls_timer t, double* total_ms, long long* count) {
    if (!c || t < 0 || t >= LS_T_COUNT) return LS_BAD_ARG;
    resolve_regions(c);
    if (total_ms) *total_ms = c->timer_ms[t];
    if (count) *count = c->timer_count[t];
    return LS_OK;
}

ls_status ls_timing_bytes(ls_ctx* c, ls_timer t, double* bytes) {
    if (!c || t < 0 || t >= LS_T_COUNT || !bytes) return LS_BAD_ARG;
    *bytes = c->timer_bytes[t];
    return LS_OK;
}

long long ls_kernel_launches(const ls_ctx* c) { return c ? c->launches : 0; }

}  // extern "C"
