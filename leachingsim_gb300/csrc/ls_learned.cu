// ls_learned.cu - the learned pressure network: a U-shaped 3D convolutional network (4
// levels, 16-64 channels, BF16 weights and activations, FP32 accumulation) that maps a
// pore mask, the log-permeability and a boundary / previous-pressure channel to a pressure
// field. It is the warm start of the pressure solve; the plain multigrid solver judges
// every start through the FP64 residual and finishes the solve.
//
// Kernels, all hand-written:
//  * k_lp_conv_tma: 3x3x3 convolution as an implicit GEMM on the 5th-generation tensor cores
//    (tcgen05.mma kind::f16, BF16 x BF16 -> FP32 accumulators in tensor memory), its input
//    halo brought into shared memory by TMA (cp.async.bulk.tensor), streamed through z with
//    the three dz taps stacked along N, warp-specialised (TMA / MMA / epilogue warps) on
//    persistent CTAs. Every layer (64 output channels from 64 inputs as two launches); with
//    flipped, transposed weights also the input-gradient pass. The default (LS_LPNET_TC=3).
//  * k_lp_conv_tc: the first tcgen05 form, a CTA per 16 x 8 x ZT output tile with its halo
//    staged three times by cp.async (LS_LPNET_TC=2: layers with up to 32 input channels;
//    1: the 32 -> 64 layer alone, mma.sync elsewhere).
//  * k_lp_conv / k_lp_conv_tiled: the same convolution with mma.sync m16n8k16 (BF16 x BF16
//    -> FP32 in registers): a warp computes 16 output voxels x all output channels; the K
//    dimension runs over 27 taps x input channels in chunks of 16. k_lp_conv serves the
//    64-channel layers outside LS_LPNET_TC=3; k_lp_conv_tiled is the LS_LPNET_TC=0 path of
//    the others.
//  * k_lp_conv_dw_mma: the weight / bias gradient, staged transposed through shared memory,
//    mma.sync m16n8k16 (k_lp_conv_dw: the same with FP32 FMA, LS_LPNET_DW=0).
//  * pooling, upsampling + skip addition and their backward passes, ReLU masking, the
//    masked mean-square loss and Adam.
//
// Layout: activations (D, H, W, C) with the channels innermost (BF16; the output layer FP32),
// gradients the same in FP32; weights [tap][cout][cin], tap = 9 (dz+1) + 3 (dy+1) + (dx+1). D, H and W are
// multiples of 8 (three 2x poolings).
#include <cuda.h>
#include <cuda_bf16.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "ls_internal.cuh"

namespace ls {

typedef __nv_bfloat16 bf16;

struct LpDims {
    int D, H, W;
    long long N;
};

namespace {

__host__ __device__ inline LpDims lp_dims(int D, int H, int W) {
    return LpDims{D, H, W, (long long)D * H * W};
}

__device__ __forceinline__ void lp_decode(const LpDims& d, long long r, int& z, int& y, int& x) {
    const long long hw = (long long)d.H * d.W;
    z = (int)(r / hw);
    const long long rem = r - (long long)z * hw;
    y = (int)(rem / d.W);
    x = (int)(rem - (long long)y * d.W);
}

// D = A (16x16, row) x B (16x8, col) + D, BF16 inputs, FP32 accumulators
__device__ __forceinline__ void mma_16816(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <typename T>
__device__ __forceinline__ void store_pair(T* p, float a, float b);
template <>
__device__ __forceinline__ void store_pair<bf16>(bf16* p, float a, float b) {
    *reinterpret_cast<__nv_bfloat162*>(p) = __floats2bfloat162_rn(a, b);
}
template <>
__device__ __forceinline__ void store_pair<float>(float* p, float a, float b) {
    *reinterpret_cast<float2*>(p) = make_float2(a, b);
}

// out[v, co] = act(bias[co] + sum_tap sum_ci w[tap][co][ci] in[v + tap, ci]), zero padding.
// Fragment layout of m16n8k16 (lane = 4 g + t): A rows g and g + 8, columns 2t, 2t + 1 and
// 2t + 8, 2t + 9; B column g, rows 2t, 2t + 1 and 2t + 8, 2t + 9; C rows g, g + 8, columns
// 2t, 2t + 1. Rows are voxels, A columns input channels, B columns output channels.
template <int CIN, int COUT, bool RELU, typename OutT>
__global__ void __launch_bounds__(128) k_lp_conv(LpDims d, const bf16* __restrict__ in, const bf16* __restrict__ w,
                                                 const float* __restrict__ bias, OutT* __restrict__ out) {
    static_assert(CIN % 16 == 0 && COUT % 8 == 0, "channel counts");
    constexpr int NT = COUT / 8, KC = CIN / 16;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, tg = lane & 3;
    const long long ntiles = (d.N + 15) / 16;
    const uint32_t* __restrict__ in32 = reinterpret_cast<const uint32_t*>(in);
    const uint32_t* __restrict__ w32 = reinterpret_cast<const uint32_t*>(w);
    for (long long tile = blockIdx.x * 4LL + warp; tile < ntiles; tile += gridDim.x * 4LL) {
        const long long r0 = tile * 16 + g, r1 = r0 + 8;
        const bool ok0 = r0 < d.N, ok1 = r1 < d.N;
        int z0 = 0, y0 = 0, x0 = 0, z1 = 0, y1 = 0, x1 = 0;
        if (ok0) lp_decode(d, r0, z0, y0, x0);
        if (ok1) lp_decode(d, r1, z1, y1, x1);
        float acc[NT][4];
#pragma unroll
        for (int n = 0; n < NT; ++n) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;
        for (int t = 0; t < 27; ++t) {
            const int dz = t / 9 - 1, dy = (t / 3) % 3 - 1, dx = t % 3 - 1;
            const int za = z0 + dz, ya = y0 + dy, xa = x0 + dx, zb = z1 + dz, yb = y1 + dy, xb = x1 + dx;
            const bool v0 = ok0 && za >= 0 && za < d.D && ya >= 0 && ya < d.H && xa >= 0 && xa < d.W;
            const bool v1 = ok1 && zb >= 0 && zb < d.D && yb >= 0 && yb < d.H && xb >= 0 && xb < d.W;
            const long long n0 = v0 ? ((long long)za * d.H + ya) * d.W + xa : 0;
            const long long n1 = v1 ? ((long long)zb * d.H + yb) * d.W + xb : 0;
            const uint32_t* p0 = in32 + n0 * (CIN / 2);
            const uint32_t* p1 = in32 + n1 * (CIN / 2);
#pragma unroll
            for (int kc = 0; kc < KC; ++kc) {
                uint32_t a[4];
                a[0] = v0 ? p0[kc * 8 + tg] : 0u;
                a[1] = v1 ? p1[kc * 8 + tg] : 0u;
                a[2] = v0 ? p0[kc * 8 + 4 + tg] : 0u;
                a[3] = v1 ? p1[kc * 8 + 4 + tg] : 0u;
#pragma unroll
                for (int n = 0; n < NT; ++n) {
                    const uint32_t* wp = w32 + ((size_t)t * COUT + n * 8 + g) * (CIN / 2);
                    const uint32_t b[2] = {__ldg(wp + kc * 8 + tg), __ldg(wp + kc * 8 + 4 + tg)};
                    mma_16816(acc[n], a, b);
                }
            }
        }
#pragma unroll
        for (int n = 0; n < NT; ++n) {
            const int co = n * 8 + tg * 2;
            const float b0 = bias ? bias[co] : 0.f, b1 = bias ? bias[co + 1] : 0.f;
            float c0 = acc[n][0] + b0, c1 = acc[n][1] + b1, c2 = acc[n][2] + b0, c3 = acc[n][3] + b1;
            if (RELU) {
                c0 = fmaxf(c0, 0.f); c1 = fmaxf(c1, 0.f); c2 = fmaxf(c2, 0.f); c3 = fmaxf(c3, 0.f);
            }
            if (ok0) store_pair<OutT>(out + r0 * COUT + co, c0, c1);
            if (ok1) store_pair<OutT>(out + r1 * COUT + co, c2, c3);
        }
    }
}

// The same convolution with the input tile staged in shared memory: a block computes a
// 16 (x) x 4 (y) x 2 (z) tile of output voxels (8 rows of 16 along x, two per warp) from
// an 18 x 6 x 4 halo tile loaded once with 16-byte loads (zeros outside the grid), and
// every tap's A fragment is an ldmatrix.x4 of 16 rows gathered from the tile (lane l gives
// the address of row l & 15, channel half l >> 4). A voxel occupies CIN + 8 BF16 in the
// tile, so the eight 16-byte rows of one 8x8 matrix fall in distinct bank groups. The B
// fragments (weights) come through L1 as before and serve both of a warp's rows.
constexpr int kTX = 16, kTY = 4, kTZ = 2, kHX = kTX + 2, kHY = kTY + 2, kHZ = kTZ + 2;
constexpr int kHalo = kHX * kHY * kHZ;

__device__ __forceinline__ void ldmatrix_x4(uint32_t (&r)[4], uint32_t addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr));
}

template <int CIN, int COUT, bool RELU, typename OutT>
__global__ void __launch_bounds__(128) k_lp_conv_tiled(LpDims d, const bf16* __restrict__ in,
                                                       const bf16* __restrict__ w, const float* __restrict__ bias,
                                                       OutT* __restrict__ out) {
    static_assert(CIN % 16 == 0 && CIN <= 32 && COUT % 8 == 0, "channel counts");
    constexpr int NT = COUT / 8, KC = CIN / 16, SC = CIN + 8, CH = CIN / 8;
    __shared__ __align__(16) bf16 tile[kHalo * SC];
    const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY, z0 = blockIdx.z * kTZ;
    // halo tile: kHalo voxels x CH chunks of 8 channels (16 bytes)
    for (int e = threadIdx.x; e < kHalo * CH; e += blockDim.x) {
        const int hv = e / CH, q = e - hv * CH;
        const int hx = hv % kHX, hy = (hv / kHX) % kHY, hz = hv / (kHX * kHY);
        const int gx = x0 + hx - 1, gy = y0 + hy - 1, gz = z0 + hz - 1;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (gx >= 0 && gx < d.W && gy >= 0 && gy < d.H && gz >= 0 && gz < d.D)
            v = __ldg(reinterpret_cast<const uint4*>(in + (((long long)gz * d.H + gy) * d.W + gx) * CIN) + q);
        *reinterpret_cast<uint4*>(tile + hv * SC + q * 8) = v;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, tg = lane & 3;
    const int row = lane & 15, kofs = (lane >> 4) * 8;
    const uint32_t tile_s = (uint32_t)__cvta_generic_to_shared(tile);
    const uint32_t* __restrict__ w32 = reinterpret_cast<const uint32_t*>(w);
    int yy[2], zz[2];
#pragma unroll
    for (int m = 0; m < 2; ++m) {
        const int mt = warp * 2 + m;  // 0..7
        yy[m] = mt % kTY;
        zz[m] = mt / kTY;
    }
    float acc[2][NT][4];
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int n = 0; n < NT; ++n) acc[m][n][0] = acc[m][n][1] = acc[m][n][2] = acc[m][n][3] = 0.f;
    for (int t = 0; t < 27; ++t) {
        const int dz = t / 9 - 1, dy = (t / 3) % 3 - 1, dx = t % 3 - 1;
        uint32_t base[2];
#pragma unroll
        for (int m = 0; m < 2; ++m) {
            const int hv = ((zz[m] + 1 + dz) * kHY + (yy[m] + 1 + dy)) * kHX + (row + 1 + dx);
            base[m] = tile_s + (uint32_t)((hv * SC + kofs) * 2);
        }
#pragma unroll
        for (int kc = 0; kc < KC; ++kc) {
            uint32_t a[2][4];
            ldmatrix_x4(a[0], base[0] + kc * 32);
            ldmatrix_x4(a[1], base[1] + kc * 32);
#pragma unroll
            for (int n = 0; n < NT; ++n) {
                const uint32_t* wp = w32 + ((size_t)t * COUT + n * 8 + g) * (CIN / 2);
                const uint32_t b[2] = {__ldg(wp + kc * 8 + tg), __ldg(wp + kc * 8 + 4 + tg)};
                mma_16816(acc[0][n], a[0], b);
                mma_16816(acc[1][n], a[1], b);
            }
        }
    }
#pragma unroll
    for (int m = 0; m < 2; ++m) {
        const int y = y0 + yy[m], z = z0 + zz[m];
        if (y >= d.H || z >= d.D) continue;
        const int xa = x0 + g, xb = x0 + g + 8;
        const long long ra = ((long long)z * d.H + y) * d.W + xa, rb = ra + 8;
#pragma unroll
        for (int n = 0; n < NT; ++n) {
            const int co = n * 8 + tg * 2;
            const float b0 = bias ? bias[co] : 0.f, b1 = bias ? bias[co + 1] : 0.f;
            float c0 = acc[m][n][0] + b0, c1 = acc[m][n][1] + b1, c2 = acc[m][n][2] + b0, c3 = acc[m][n][3] + b1;
            if (RELU) {
                c0 = fmaxf(c0, 0.f); c1 = fmaxf(c1, 0.f); c2 = fmaxf(c2, 0.f); c3 = fmaxf(c3, 0.f);
            }
            if (xa < d.W) store_pair<OutT>(out + ra * COUT + co, c0, c1);
            if (xb < d.W) store_pair<OutT>(out + rb * COUT + co, c2, c3);
        }
    }
}

// ---------------------------------------------------------------------------
// The same convolution on the 5th-generation tensor cores (tcgen05): a CTA computes a
// 16 (x) x 8 (y) x ZT (z) block of output voxels as ZT implicit GEMMs of M = 128 (one per
// plane), D_p[m][co] = sum over the 27 taps and CIN/16 K-steps of A_tap,p[m][k] B_tap[co][k],
// accumulated in tensor memory (TMEM, FP32, COUT columns per plane) by 27 ZT CIN/16
// tcgen05.mma instructions that one thread issues back to back; a tcgen05.commit on an
// mbarrier signals completion and the eight warps read the TMEM lanes (rows) of their lane
// quarter back for the bias / ReLU epilogue, two planes at a time. ZT planes share one
// staging of the weights and of the input halo, which cp.async copies bring in (zero-filled
// outside the grid) all in flight at once.
//
// Operands live in shared memory in the SWIZZLE_NONE K-major layout: 8 x 16-byte "core
// matrices" (8 rows of 8 BF16), the descriptor's leading byte offset (LBO) stepping along K
// and its stride byte offset (SBO) along M / N. The input halo is staged three times, once
// per x-shift dx = -1, 0, +1, each as [8-channel chunk][ZT + 2 planes][10 rows][16 voxels] x
// 16 B, so every tap's A operand is a plain descriptor: start = the (dx, plane + dz, dy) row,
// SBO = 128 B (8 voxels), LBO = one chunk (all planes). The weights sit as [tap][K-step][k8]
// [n8] core matrices (SBO = 128 B, LBO = COUT/8 x 128 B). Instruction descriptor: FP32
// accumulator, BF16 A and B, both K-major, N = COUT, M = 128.
constexpr int kTcX = 16, kTcY = 8, kTcRows = kTcY + 2;

__device__ int g_lp_tc_timeouts;  // CTAs whose wait for the tensor cores gave up

template <int CIN, int COUT, int ZT>
struct TcShape {
    static constexpr int KC = CIN / 16;
    static constexpr int planes = ZT + 2;
    static constexpr int chunk_bytes = planes * kTcRows * kTcX * 16;  // one 8-channel chunk of one copy
    static constexpr int copy_bytes = (CIN / 8) * chunk_bytes;
    static constexpr int a_bytes = 3 * copy_bytes;
    static constexpr int w_bytes = 27 * CIN * COUT * 2;
    static constexpr int smem = a_bytes + w_bytes;
    static constexpr int cols = ZT * COUT;
    static constexpr int tmem_cols = cols <= 32 ? 32 : cols <= 64 ? 64 : cols <= 128 ? 128 : cols <= 256 ? 256 : 512;
};

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);  // version 1, SWIZZLE_NONE
}

constexpr int kTcThreads = 256;

// 16-byte asynchronous global -> shared copy through L1 (the three x-shifted copies and the
// two halves of a 32-byte voxel hit the same lines); valid == false fills the 16 bytes with
// zeros (source size 0: nothing is read)
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, bool valid) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}

// A CTA runs tiles blockIdx.x, blockIdx.x + gridDim.x, ... (one tile when the grid covers
// them all; persistent CTAs otherwise). It stages the weights into shared memory once for all
// its tiles and, with NBUF = 2 halo buffers, stages tile i + 1 (cp.async) while the tensor
// cores run tile i, the epilogue of tile i overlapping the copies still in flight. One TMEM
// accumulator set serves all tiles (the epilogue of tile i ends before the MMAs of tile i + 1
// are issued); the mbarrier's phase flips once per tile.
template <int CIN, int COUT, int ZT, int NBUF, bool RELU, typename OutT>
__global__ void __launch_bounds__(kTcThreads) k_lp_conv_tc(LpDims d, const bf16* __restrict__ in,
                                                           const bf16* __restrict__ w, const float* __restrict__ bias,
                                                           OutT* __restrict__ out) {
    using S = TcShape<CIN, COUT, ZT>;
    static_assert(CIN % 16 == 0 && COUT % 16 == 0 && COUT <= 64 && S::cols <= 256, "channel counts");
    static_assert(NBUF == 1 || NBUF == 2, "halo buffers");
    extern __shared__ __align__(1024) uint8_t tc_smem[];
    __shared__ uint32_t tmem_slot;
    __shared__ __align__(8) uint64_t mbar;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    constexpr int CH = CIN / 8;
    uint8_t* sW = tc_smem;
    const uint32_t sW_s = (uint32_t)__cvta_generic_to_shared(sW);
    const uint32_t sA_s = sW_s + S::w_bytes;  // buffer k at sA_s + k * a_bytes
    const int tiles_x = (d.W + kTcX - 1) / kTcX, tiles_y = (d.H + kTcY - 1) / kTcY;
    const int ntiles = tiles_x * tiles_y * ((d.D + ZT - 1) / ZT);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         (uint32_t)__cvta_generic_to_shared(&tmem_slot)),
                     "r"(S::tmem_cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (tid == 0)
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"((uint32_t)__cvta_generic_to_shared(&mbar)),
                     "r"(1));
    // input halo of tile t into buffer k: three x-shifted copies, zeros outside the grid
    auto stage = [&](int t, int k) {
        const int tx = t % tiles_x, ty = (t / tiles_x) % tiles_y, tz = t / (tiles_x * tiles_y);
        const int x0 = tx * kTcX, y0 = ty * kTcY, z0 = tz * ZT;
        const uint32_t base = sA_s + k * S::a_bytes;
        for (int e = tid; e < 3 * CH * S::planes * kTcRows * kTcX; e += kTcThreads) {
            const int x = e % kTcX;
            int r = e / kTcX;
            const int ry = r % kTcRows;
            r /= kTcRows;
            const int pz = r % S::planes;
            r /= S::planes;
            const int q = r % CH, cp = r / CH;
            const int gx = x0 + x + cp - 1, gy = y0 + ry - 1, gz = z0 + pz - 1;
            const bool ok = gx >= 0 && gx < d.W && gy >= 0 && gy < d.H && gz >= 0 && gz < d.D;
            const bf16* src = ok ? in + (((long long)gz * d.H + gy) * d.W + gx) * CIN + q * 8 : in;
            cp_async16(base + cp * S::copy_bytes + q * S::chunk_bytes + ((pz * kTcRows + ry) * kTcX + x) * 16, src, ok);
        }
    };
    // weights [tap][co][ci] -> [tap][K-step][k8][n8] core matrices, once per CTA
    for (int e = tid; e < 27 * COUT * CH; e += kTcThreads) {
        const int q = e % CH;
        const int co = (e / CH) % COUT, t = e / (CH * COUT);
        const int kc = q >> 1, k8 = q & 1;
        cp_async16(sW_s + ((((t * S::KC + kc) * 2 + k8) * (COUT / 8) + (co >> 3)) * 128) + (co & 7) * 16,
                   w + ((size_t)t * COUT + co) * CIN + q * 8, true);
    }
    if ((int)blockIdx.x < ntiles) stage(blockIdx.x, 0);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = tmem_slot;
    const uint32_t mbar_s = (uint32_t)__cvta_generic_to_shared(&mbar);
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(COUT >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    int it = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
        const int buf = (NBUF == 2) ? (it & 1) : 0;
        if (tid == 0) {
            // the start address sits in the descriptor's low 14 bits (address >> 4, < 256 KB):
            // each operand's descriptor is a base descriptor plus a compile-time offset
            const uint64_t da0 = tc_desc(sA_s + buf * S::a_bytes, S::chunk_bytes, 128);
            const uint64_t db0 = tc_desc(sW_s, (COUT / 8) * 128, 128);
            for (int p = 0; p < ZT; ++p) {
                const uint64_t dap = da0 + (uint64_t)((p * kTcRows * kTcX * 16) >> 4);
                const uint32_t dtm = tmem + (uint32_t)(p * COUT);
#pragma unroll
                for (int t = 0; t < 27; ++t) {
                    const int dz = t / 9 - 1, dy = (t / 3) % 3 - 1, dx = t % 3 - 1;
#pragma unroll
                    for (int kc = 0; kc < S::KC; ++kc) {
                        const uint64_t da = dap + (uint64_t)(((dx + 1) * S::copy_bytes + 2 * kc * S::chunk_bytes +
                                                              (((1 + dz) * kTcRows + (1 + dy)) * kTcX) * 16) >> 4);
                        const uint64_t db = db0 + (uint64_t)(((t * S::KC + kc) * 2 * (COUT / 8) * 128) >> 4);
                        const uint32_t acc = (t | kc) ? 1u : 0u;
                        asm volatile(
                            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtm),
                            "l"(da), "l"(db), "r"(idesc), "r"(acc));
                    }
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar_s));
        }
        // the next tile's halo into the other buffer while the tensor cores run this one
        const int next = tile + gridDim.x;
        if (NBUF == 2 && next < ntiles) stage(next, buf ^ 1);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        // bounded wait for this tile's MMAs (phase it & 1); warps other than the issuing one
        // back off so that their polling does not take issue slots from it
        uint32_t done = 0;
        for (int k = 0; k < (1 << 22) && !done; ++k) {
            asm volatile(
                "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
                : "=r"(done)
                : "r"(mbar_s), "r"((uint32_t)(it & 1)));
            if (!done && warp != 0) __nanosleep(64);
        }
        if (__syncthreads_or(!done)) {
            // a wait gave up: stop here (no further MMAs or copies into buffers they may read)
            if (tid == 0) atomicAdd(&g_lp_tc_timeouts, 1);
            break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        {
            const int tx = tile % tiles_x, ty = (tile / tiles_x) % tiles_y, tz = tile / (tiles_x * tiles_y);
            const int x0 = tx * kTcX, y0 = ty * kTcY, z0 = tz * ZT;
            // warp w reads TMEM lanes 32 (w % 4) .. + 31 (rows m), of the planes p = w / 4 (mod 2)
            const int m = (warp & 3) * 32 + lane;
            const int x = x0 + (m % kTcX), y = y0 + m / kTcX;
            const bool okxy = x < d.W && y < d.H;
            for (int p = warp >> 2; p < ZT; p += kTcThreads / 128) {
                const bool ok = okxy && z0 + p < d.D;
                const long long v = ((long long)(z0 + p) * d.H + y) * d.W + x;
#pragma unroll
                for (int c0 = 0; c0 < COUT; c0 += 16) {
                    uint32_t r[16];
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                        : "r"(tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(p * COUT + c0)));
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                    if (ok) {
#pragma unroll
                        for (int q = 0; q < 16; q += 2) {
                            const int co = c0 + q;
                            float a = __uint_as_float(r[q]) + (bias ? bias[co] : 0.f);
                            float b = __uint_as_float(r[q + 1]) + (bias ? bias[co + 1] : 0.f);
                            if (RELU) {
                                a = fmaxf(a, 0.f);
                                b = fmaxf(b, 0.f);
                            }
                            store_pair<OutT>(out + v * COUT + co, a, b);
                        }
                    }
                }
            }
        }
        // with one buffer the next tile is staged only now, after this tile's MMAs
        if (NBUF == 1 && next < ntiles) {
            stage(next, 0);
            asm volatile("cp.async.commit_group;\n" ::: "memory");
        }
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(S::tmem_cols));
}

// ---------------------------------------------------------------------------
// The convolution streamed through z on the tensor cores, its input brought in by the tensor
// memory accelerator (TMA). A persistent CTA (one per SM) runs tiles of 8 (x) x 16 (y) output
// voxels x zt planes (TmShape::ZT, fewer on coarse grids, so that the tiles cover the SMs).
// For each input plane p of a tile (z0 - 1 .. z0 + zt) one TMA load per
// 8-channel chunk brings the plane's 10 x 18 halo into a stage of a ring of shared-memory
// buffers (zeros outside the grid: the tensor map's out-of-bounds fill), and nine (dy, dx) x
// CIN/16 tcgen05.mma instructions apply the plane to the three output planes it feeds at once:
// B stacks the dz = +1, 0, -1 weights along N (N = 3 COUT), so D is the consecutive
// COUT-column blocks of output planes p - 1, p, p + 1 in a tensor-memory region of ZT planes
// (at a tile's first and last planes the MMA takes only the part of N that lands inside it).
// Every (dy, dx) tap is a plain descriptor on the one halo copy: an output row of 8 voxels is
// one 8 x 16-byte core matrix, rows y are 160 bytes (10 voxels) apart (SBO), the two
// 8-channel halves of a K-step a chunk apart (LBO).
//
// Roles, synchronised by mbarriers: warp 0 issues the TMA loads (stage full / empty), warp 1
// the MMAs (a tcgen05.commit frees a stage once its MMAs have read it, another marks a region
// full after a tile's last plane), warps 2-5 read a full region back (tcgen05.ld; warp w owns
// the TMEM lanes of quarter w % 4), add the bias, apply ReLU, store the outputs and write
// zeros back, so that every MMA accumulates. Two regions alternate: a tile's epilogue
// overlaps the next tile's loads and MMAs. Every wait is bounded (kTmWaitCycles): one that gives
// up raises the CTA's abort flag, the CTA drains the copies and MMAs it issued (bounded
// waits too), frees its tensor memory, counts a timeout and returns.
constexpr int kTmX = 8, kTmY = 16, kTmHX = kTmX + 2, kTmHY = kTmY + 2;
constexpr int kTmBox = kTmHX * kTmHY * 16;                // bytes of one box: 8 channels x 10 x 18
constexpr int kTmChunk = (kTmBox + 127) / 128 * 128;      // its slot in a stage (128-byte aligned)
constexpr int kTmThreads = 192;

// COUT = the output channels of one launch (a 64-channel output runs as two launches of 32)
template <int CIN, int COUT>
struct TmShape {
    static constexpr int CH = CIN / 8, KC = CIN / 16;
    static constexpr int ZT = 256 / COUT;                 // two regions of ZT x COUT = 256 columns
    static constexpr int region = ZT * COUT;
    static constexpr int stage_bytes = CH * kTmChunk;
    static constexpr int NB = 3 * COUT / 8;               // n8 groups of the stacked B
    static constexpr int w_bytes = 27 * CIN * COUT * 2;
    // as many halo stages as fit beside the weights in 200 KB (4 to 32)
    static constexpr int fit = (200 * 1024 - w_bytes) / stage_bytes;
    static constexpr int stages = fit < 4 ? 4 : fit > 32 ? 32 : fit;
    static constexpr int smem = w_bytes + stages * stage_bytes + 1024;  // + alignment of the base
};

// bounded wait for the completion of the mbarrier phase of the given parity; false when it
// gave up (raising the abort flag) or another role raised it (abort null: drain waits). The
// bound is counted in SM clock cycles (kTmWaitCycles, about 2 s), read only once a first poll
// has failed.
constexpr long long kTmWaitCycles = 4000000000ll;

__device__ __forceinline__ bool tm_poll(uint32_t bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}

__device__ __forceinline__ bool tm_wait(uint32_t bar, uint32_t parity, volatile int* abort, bool backoff) {
    if (tm_poll(bar, parity)) return true;
    const long long t0 = clock64();
    while (true) {
        if (tm_poll(bar, parity)) return true;
        if (abort && *abort) return false;
        if (clock64() - t0 > kTmWaitCycles) {
            if (abort) *abort = 1;
            return false;
        }
        if (backoff) __nanosleep(32);
    }
}

__device__ __forceinline__ void tm_bar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void tm_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tm_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}

// 4-D tiled TMA load (coordinates innermost first) into shared memory, completing on bar
__device__ __forceinline__ void tm_load4(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                         uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];\n" ::"r"(dst),
        "l"((unsigned long long)map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tm_mma(uint32_t dtm, uint64_t da, uint64_t db, uint32_t idesc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtm),
        "l"(da), "l"(db), "r"(idesc), "r"(1u));
}

__device__ __forceinline__ void tm_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tm_ld16(uint32_t (&r)[16], uint32_t ta) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(ta));
}

__device__ __forceinline__ void tm_st16_zero(uint32_t ta) {
    const uint32_t z = 0u;
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};\n" ::"r"(ta),
        "r"(z), "r"(z), "r"(z), "r"(z), "r"(z), "r"(z), "r"(z), "r"(z), "r"(z), "r"(z), "r"(z), "r"(z), "r"(z), "r"(z),
        "r"(z), "r"(z)
        : "memory");
}

template <typename T>
__device__ __forceinline__ void store16(T* p, const float (&f)[16]);
template <>
__device__ __forceinline__ void store16<bf16>(bf16* p, const float (&f)[16]) {
    uint32_t u[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(f[2 * q], f[2 * q + 1]);
        u[q] = *reinterpret_cast<const uint32_t*>(&h);
    }
    reinterpret_cast<uint4*>(p)[0] = make_uint4(u[0], u[1], u[2], u[3]);
    reinterpret_cast<uint4*>(p)[1] = make_uint4(u[4], u[5], u[6], u[7]);
}
template <>
__device__ __forceinline__ void store16<float>(float* p, const float (&f)[16]) {
#pragma unroll
    for (int q = 0; q < 4; ++q)
        reinterpret_cast<float4*>(p)[q] = make_float4(f[4 * q], f[4 * q + 1], f[4 * q + 2], f[4 * q + 3]);
}

// Output channels co0 .. co0 + COUT - 1 of a layer with cout_total (the weights' and the
// bias's row count); out holds ostride values per voxel (only0: channel co0 alone, the
// network's output channel); zt <= TmShape::ZT output planes per tile
template <int CIN, int COUT, bool RELU, typename OutT>
__global__ void __launch_bounds__(kTmThreads, 1) k_lp_conv_tma(const __grid_constant__ CUtensorMap tmap, LpDims d,
                                                               const bf16* __restrict__ w,
                                                               const float* __restrict__ bias,
                                                               OutT* __restrict__ out, int cout_total, int co0,
                                                               int ostride, int only0, int zt) {
    using S = TmShape<CIN, COUT>;
    constexpr int kTmStages = S::stages;
    static_assert(CIN % 16 == 0 && CIN <= 64 && COUT % 16 == 0 && COUT <= 64, "channel counts");
    extern __shared__ uint8_t tm_smem_raw[];
    __shared__ __align__(8) uint64_t bar_full[kTmStages], bar_empty[kTmStages], bar_tfull[2], bar_tempty[2], bar_drain;
    __shared__ uint32_t tmem_slot;
    __shared__ int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t sW = ((uint32_t)__cvta_generic_to_shared(tm_smem_raw) + 1023u) & ~1023u;  // weights, then stages
    const uint32_t sA = sW + S::w_bytes;
    const int tiles_x = (d.W + kTmX - 1) / kTmX, tiles_y = (d.H + kTmY - 1) / kTmY;
    const int ntiles = tiles_x * tiles_y * ((d.D + zt - 1) / zt);
    auto sbar = [](uint64_t* b) { return (uint32_t)__cvta_generic_to_shared(b); };
    volatile int* abort = &s_abort;

    // the stacked weights: B[tap9][K-step][k8][n8 group] core matrices, row n = j COUT + co
    // holding the weights of dz = 1 - j (output plane p - 1 + j from input plane p)
    for (int e = tid; e < 27 * COUT * S::CH; e += kTmThreads) {
        const int q = e % S::CH;
        const int nn = (e / S::CH) % (3 * COUT), t9 = e / (S::CH * 3 * COUT);
        const int j = nn / COUT, co = nn % COUT;
        const uint4 v =
            __ldg(reinterpret_cast<const uint4*>(w + ((size_t)(9 * (2 - j) + t9) * cout_total + co0 + co) * CIN + q * 8));
        const uint32_t dst = sW + (uint32_t)((((t9 * S::KC + (q >> 1)) * 2 + (q & 1)) * S::NB + (nn >> 3)) * 128 +
                                             (nn & 7) * 16);
        asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};\n" ::"r"(dst), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w)
                     : "memory");
    }
    if (tid == 0) {
        s_abort = 0;
        for (int s = 0; s < kTmStages; ++s) {
            tm_bar_init(sbar(&bar_full[s]), 1);
            tm_bar_init(sbar(&bar_empty[s]), 1);
        }
        for (int r = 0; r < 2; ++r) {
            tm_bar_init(sbar(&bar_tfull[r]), 1);
            tm_bar_init(sbar(&bar_tempty[r]), 4);
        }
        tm_bar_init(sbar(&bar_drain), 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;\n" ::"r"(
                         (uint32_t)__cvta_generic_to_shared(&tmem_slot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = tmem_slot;
    if (warp >= 2) {  // every MMA accumulates: tensor memory starts at zero
        const uint32_t lanes = (uint32_t)((warp & 3) * 32) << 16;
        for (int c = 0; c < 512; c += 16) tm_st16_zero(tmem + lanes + (uint32_t)c);
        asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // the weights, for the MMAs
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");

    uint32_t loaded = 0;   // warp 0: planes whose loads were issued
    bool issued = false;   // warp 1: any MMA issued
    if (warp == 0) {
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
            const int tx = tile % tiles_x, ty = (tile / tiles_x) % tiles_y, tz = tile / (tiles_x * tiles_y);
            const int x0 = tx * kTmX, y0 = ty * kTmY, z0 = tz * zt;
            bool ok = true;
            for (int li = 0; li < zt + 2 && ok; ++li) {
                const int p = z0 - 1 + li;
                if (p < 0 || p >= d.D) continue;
                const int s = (int)(loaded % kTmStages);
                const uint32_t ph = (loaded / kTmStages) & 1u;
                if (lane == 0) {
                    ok = tm_wait(sbar(&bar_empty[s]), ph ^ 1u, abort, false);
                    if (ok) {
                        tm_expect_tx(sbar(&bar_full[s]), (uint32_t)(S::CH * kTmBox));
                        for (int q = 0; q < S::CH; ++q)
                            tm_load4(sA + (uint32_t)(s * S::stage_bytes + q * kTmChunk), &tmap, q * 8, x0 - 1, y0 - 1, p,
                                     sbar(&bar_full[s]));
                    }
                }
                ok = __shfl_sync(0xffffffffu, ok, 0);
                if (ok) ++loaded;
            }
            if (!ok) break;
        }
    } else if (warp == 1) {
        const uint32_t idesc0 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(128 >> 4) << 24);
        const uint64_t db0 = tc_desc(sW, S::NB * 128, 128);
        uint32_t used = 0;
        int it = 0;
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
            const int tz = tile / (tiles_x * tiles_y), z0 = tz * zt;
            const int r = it & 1;
            bool ok = true;
            if (lane == 0) ok = tm_wait(sbar(&bar_tempty[r]), (((uint32_t)it >> 1) & 1u) ^ 1u, abort, false);
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) break;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            for (int li = 0; li < zt + 2 && ok; ++li) {
                const int p = z0 - 1 + li;
                if (p < 0 || p >= d.D) continue;
                const int s = (int)(used % kTmStages);
                const uint32_t ph = (used / kTmStages) & 1u;
                if (lane == 0) {
                    ok = tm_wait(sbar(&bar_full[s]), ph, abort, false);
                    if (ok) {
                        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                        const int j0 = li < 2 ? 2 - li : 0;
                        const int j1 = zt + 2 - li < 3 ? zt + 2 - li : 3;
                        const uint32_t idesc = idesc0 | ((uint32_t)(((j1 - j0) * COUT) >> 3) << 17);
                        const uint32_t dtm = tmem + (uint32_t)(r * S::region + (li + j0 - 2) * COUT);
                        const uint64_t da0 = tc_desc(sA + (uint32_t)(s * S::stage_bytes), kTmChunk, kTmHX * 16);
                        const uint64_t dbj = db0 + (uint64_t)((j0 * (COUT / 8) * 128) >> 4);
#pragma unroll
                        for (int t9 = 0; t9 < 9; ++t9) {
                            const int dy = t9 / 3 - 1, dx = t9 % 3 - 1;
#pragma unroll
                            for (int kc = 0; kc < S::KC; ++kc) {
                                const uint64_t da =
                                    da0 + (uint64_t)((2 * kc * kTmChunk + ((dy + 1) * kTmHX + (dx + 1)) * 16) >> 4);
                                const uint64_t db = dbj + (uint64_t)(((t9 * S::KC + kc) * 2 * S::NB * 128) >> 4);
                                tm_mma(dtm, da, db, idesc);
                            }
                        }
                        tm_commit(sbar(&bar_empty[s]));  // the stage is free once these MMAs have read it
                        issued = true;
                    }
                }
                ok = __shfl_sync(0xffffffffu, ok, 0);
                if (ok) ++used;
            }
            if (!ok) break;
            if (lane == 0) tm_commit(sbar(&bar_tfull[r]));
        }
    } else {
        const int quarter = warp & 3;
        const uint32_t lanes = (uint32_t)(quarter * 32) << 16;
        const int m = quarter * 32 + lane;
        int it = 0;
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
            const int tx = tile % tiles_x, ty = (tile / tiles_x) % tiles_y, tz = tile / (tiles_x * tiles_y);
            const int x = tx * kTmX + (m & 7), y = ty * kTmY + (m >> 3), z0 = tz * zt;
            const int r = it & 1;
            if (!__all_sync(0xffffffffu, tm_wait(sbar(&bar_tfull[r]), ((uint32_t)it >> 1) & 1u, abort, true))) break;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const bool okxy = x < d.W && y < d.H;
            for (int s = 0; s < zt; ++s) {
                const int z = z0 + s;
                const bool ok = okxy && z < d.D;
                OutT* dst =
                    out + (((long long)(ok ? z : 0) * d.H + (ok ? y : 0)) * d.W + (ok ? x : 0)) * ostride + co0;
#pragma unroll
                for (int c0 = 0; c0 < COUT; c0 += 16) {
                    uint32_t v[16];
                    const uint32_t ta = tmem + lanes + (uint32_t)(r * S::region + s * COUT + c0);
                    tm_ld16(v, ta);
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                    tm_st16_zero(ta);
                    if (ok && !only0) {
                        float f[16];
#pragma unroll
                        for (int q = 0; q < 16; ++q) {
                            float a = __uint_as_float(v[q]) + (bias ? __ldg(bias + co0 + c0 + q) : 0.f);
                            f[q] = RELU ? fmaxf(a, 0.f) : a;
                        }
                        store16<OutT>(dst + c0, f);
                    } else if (ok && c0 == 0) {
                        const float a = __uint_as_float(v[0]) + (bias ? __ldg(bias + co0) : 0.f);
                        dst[0] = (OutT)(RELU ? fmaxf(a, 0.f) : a);
                    }
                }
            }
            asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) tm_arrive(sbar(&bar_tempty[r]));
        }
    }
    // drain: no copy or MMA of this CTA may be in flight when it frees its memory
    if (warp == 0 && lane == 0)
        for (uint32_t k = loaded > (uint32_t)kTmStages ? loaded - kTmStages : 0u; k < loaded; ++k)
            tm_wait(sbar(&bar_full[k % kTmStages]), (k / kTmStages) & 1u, nullptr, false);
    if (warp == 1 && lane == 0 && issued) {
        tm_commit(sbar(&bar_drain));
        tm_wait(sbar(&bar_drain), 0u, nullptr, false);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (tid == 0 && s_abort) atomicAdd(&g_lp_tc_timeouts, 1);
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;\n" ::"r"(tmem));
}

// dw[tap][co][ci] += sum_v dy[v, co] in[v + tap, ci]; db[co] += sum_v dy[v, co] (tap 13).
// Block (chunk of voxels, tap): 64-voxel slices of dy and of the shifted input staged in
// shared memory, each thread accumulating its (co, ci) pairs, one atomic add per pair.
template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_lp_conv_dw(LpDims d, const bf16* __restrict__ in, const bf16* __restrict__ dy,
                                                    float* __restrict__ dw, float* __restrict__ db, int chunk) {
    constexpr int PAIRS = CIN * COUT, PER = (PAIRS + 255) / 256;
    __shared__ float sD[64][COUT];
    __shared__ float sX[64][CIN + 1];
    __shared__ long long sN[64];
    const int t = blockIdx.y;
    const int dz = t / 9 - 1, dyy = (t / 3) % 3 - 1, dx = t % 3 - 1;
    const long long v0 = (long long)blockIdx.x * chunk;
    const long long vend = (v0 + chunk < d.N) ? v0 + chunk : d.N;
    float acc[PER];
#pragma unroll
    for (int q = 0; q < PER; ++q) acc[q] = 0.f;
    float bacc = 0.f;
    for (long long vb = v0; vb < vend; vb += 64) {
        if (threadIdx.x < 64) {
            const long long v = vb + threadIdx.x;
            long long nb = -1;
            if (v < vend) {
                int z, y, x;
                lp_decode(d, v, z, y, x);
                z += dz; y += dyy; x += dx;
                if (z >= 0 && z < d.D && y >= 0 && y < d.H && x >= 0 && x < d.W)
                    nb = ((long long)z * d.H + y) * d.W + x;
            }
            sN[threadIdx.x] = nb;
        }
        for (int e = threadIdx.x; e < 64 * COUT; e += 256) {
            const int vv = e / COUT, co = e - vv * COUT;
            const long long v = vb + vv;
            sD[vv][co] = (v < vend) ? __bfloat162float(dy[v * COUT + co]) : 0.f;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < 64 * CIN; e += 256) {
            const int vv = e / CIN, ci = e - vv * CIN;
            const long long nb = sN[vv];
            sX[vv][ci] = (nb >= 0) ? __bfloat162float(in[nb * CIN + ci]) : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int p = threadIdx.x + q * 256;
            if (p < PAIRS) {
                const int co = p / CIN, ci = p - co * CIN;
                float a = acc[q];
                for (int vv = 0; vv < 64; ++vv) a = fmaf(sD[vv][co], sX[vv][ci], a);
                acc[q] = a;
            }
        }
        if (t == 13 && threadIdx.x < COUT)
            for (int vv = 0; vv < 64; ++vv) bacc += sD[vv][threadIdx.x];
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int p = threadIdx.x + q * 256;
        if (p < PAIRS) {
            const int co = p / CIN, ci = p - co * CIN;
            atomicAdd(&dw[((size_t)t * COUT + co) * CIN + ci], acc[q]);
        }
    }
    if (t == 13 && threadIdx.x < COUT) atomicAdd(&db[threadIdx.x], bacc);
}

// The weight gradient on the tensor cores: for tap t, dW_t (COUT x CIN) = dY^T X_t, a GEMM
// whose K runs over the voxels (X_t: the input at the voxel shifted by the tap, 0 outside).
// A block takes one tap and a chunk of voxels and stages 64 voxels at a time in shared
// memory in their natural layout (a voxel's channels contiguous: 16-byte copies, rows padded
// by 16 bytes so that the eight rows of an 8x8 matrix fall in distinct bank groups); the
// fragments come from ldmatrix.trans (A = dY^T: rows = output channels; B = X_t: columns =
// input channels) and feed mma.sync m16n8k16 (BF16 x BF16 -> FP32). The (COUT/16) x (CIN/8)
// output tiles are spread over the 8 warps; with fewer tiles than warps the warps also split
// the 4 K-steps of a stage. Partial results go to dw with FP32 atomics; the bias gradient
// (the centre tap's blocks) is summed in FP32.
__device__ __forceinline__ void ldmatrix_x4_trans(uint32_t (&r)[4], uint32_t addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr));
}
__device__ __forceinline__ void ldmatrix_x2_trans(uint32_t (&r)[2], uint32_t addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n"
                 : "=r"(r[0]), "=r"(r[1])
                 : "r"(addr));
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_lp_conv_dw_mma(LpDims d, const bf16* __restrict__ in,
                                                        const bf16* __restrict__ dy, float* __restrict__ dw,
                                                        float* __restrict__ db, int chunk) {
    constexpr int SD = COUT + 8, SX = CIN + 8;   // row strides in bf16 (16-byte multiples)
    constexpr int TILES = (COUT / 16) * (CIN / 8);
    constexpr int KGROUPS = TILES >= 8 ? 1 : 8 / TILES;  // warps sharing the tiles split K
    constexpr int TW = 8 / KGROUPS;              // warps per K-group
    constexpr int PERW = (TILES + TW - 1) / TW;  // tiles per warp
    static_assert(COUT % 16 == 0 && CIN % 8 == 0 && 8 % KGROUPS == 0, "channel counts");
    __shared__ __align__(16) bf16 sD[64 * SD];   // sD[v][co]
    __shared__ __align__(16) bf16 sX[64 * SX];   // sX[v][ci]
    __shared__ long long sN[64];
    const int t = blockIdx.y;
    const int dz = t / 9 - 1, dyy = (t / 3) % 3 - 1, dx = t % 3 - 1;
    const long long v0 = (long long)blockIdx.x * chunk;
    const long long vend = (v0 + chunk < d.N) ? v0 + chunk : d.N;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, gid = lane >> 2, tig = lane & 3;
    const int kgroup = warp / TW, wt = warp - kgroup * TW;
    const uint32_t sD_s = (uint32_t)__cvta_generic_to_shared(sD);
    const uint32_t sX_s = (uint32_t)__cvta_generic_to_shared(sX);
    // ldmatrix row of this lane: matrix q = lane / 8, row lane % 8
    const int lq = lane >> 3, lr = lane & 7;
    float acc[PERW][4];
#pragma unroll
    for (int q = 0; q < PERW; ++q)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[q][e] = 0.f;
    float bacc = 0.f;
    for (long long vb = v0; vb < vend; vb += 64) {
        if (threadIdx.x < 64) {
            const long long v = vb + threadIdx.x;
            long long nb = -1;
            if (v < vend) {
                int z, y, x;
                lp_decode(d, v, z, y, x);
                z += dz; y += dyy; x += dx;
                if (z >= 0 && z < d.D && y >= 0 && y < d.H && x >= 0 && x < d.W)
                    nb = ((long long)z * d.H + y) * d.W + x;
            }
            sN[threadIdx.x] = nb;
        }
        // dY rows: 64 voxels x COUT / 8 chunks of 16 bytes
        for (int e = threadIdx.x; e < 64 * (COUT / 8); e += 256) {
            const int vv = e / (COUT / 8), c8 = e - vv * (COUT / 8);
            const long long v = vb + vv;
            uint4 val = make_uint4(0u, 0u, 0u, 0u);
            if (v < vend) val = *reinterpret_cast<const uint4*>(dy + v * COUT + c8 * 8);
            *reinterpret_cast<uint4*>(sD + vv * SD + c8 * 8) = val;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < 64 * (CIN / 8); e += 256) {
            const int vv = e / (CIN / 8), c8 = e - vv * (CIN / 8);
            const long long nb = sN[vv];
            uint4 val = make_uint4(0u, 0u, 0u, 0u);
            if (nb >= 0) val = *reinterpret_cast<const uint4*>(in + nb * CIN + c8 * 8);
            *reinterpret_cast<uint4*>(sX + vv * SX + c8 * 8) = val;
        }
        __syncthreads();
#pragma unroll
        for (int ks = kgroup; ks < 4; ks += KGROUPS) {
            const int k0 = ks * 16;
#pragma unroll
            for (int q = 0; q < PERW; ++q) {
                const int tile = wt + q * TW;
                if (tile < TILES) {
                    const int m0 = (tile / (CIN / 8)) * 16, n0 = (tile % (CIN / 8)) * 8;
                    uint32_t a[4], b[2];
                    // A (16 x 16, m = co, k = v) from sD[v][co]: matrix q = (m half q & 1, k half q >> 1)
                    ldmatrix_x4_trans(a, sD_s + 2u * (uint32_t)((k0 + (lq >> 1) * 8 + lr) * SD + m0 + (lq & 1) * 8));
                    // B (16 x 8, k = v, n = ci) from sX[v][ci]: matrix q = k half (lanes 0-15)
                    ldmatrix_x2_trans(b, sX_s + 2u * (uint32_t)((k0 + (lq & 1) * 8 + lr) * SX + n0));
                    mma_16816(acc[q], a, b);
                }
            }
        }
        if (t == 13 && threadIdx.x < COUT)
            for (int vv = 0; vv < 64; ++vv) bacc += __bfloat162float(sD[vv * SD + threadIdx.x]);
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < PERW; ++q) {
        const int tile = wt + q * TW;
        if (tile < TILES) {
            const int m0 = (tile / (CIN / 8)) * 16, n0 = (tile % (CIN / 8)) * 8;
            float* base = dw + (size_t)t * COUT * CIN;
            atomicAdd(&base[(size_t)(m0 + gid) * CIN + n0 + tig * 2], acc[q][0]);
            atomicAdd(&base[(size_t)(m0 + gid) * CIN + n0 + tig * 2 + 1], acc[q][1]);
            atomicAdd(&base[(size_t)(m0 + gid + 8) * CIN + n0 + tig * 2], acc[q][2]);
            atomicAdd(&base[(size_t)(m0 + gid + 8) * CIN + n0 + tig * 2 + 1], acc[q][3]);
        }
    }
    if (t == 13 && threadIdx.x < COUT) atomicAdd(&db[threadIdx.x], bacc);
}

// The weight / bias gradient of the layers with 16 or 32 input and output channels (16 -> 16,
// 16 -> 32, 32 -> 16), tiled like k_lp_conv_tiled: a persistent
// block walks tiles of 16 (x) x 4 (y) x 2 (z) voxels; per tile it stages the input halo
// (18 x 6 x 4 voxels, zeros outside the grid) and the tile's output gradient (zeros outside)
// once, and each of its 8 warps runs the GEMMs dW_t += dY^T X_t of its taps (t = warp,
// warp + 8, ...) over the tile's 128 voxels on mma.sync m16n8k16: per row of 16 voxels one
// A fragment (dY^T, ldmatrix.trans from [voxel][co]) serves all the warp's taps, each tap's B
// fragment (X shifted by the tap, ldmatrix.trans from the halo) is a plain row offset. The
// sums stay in registers across all the block's tiles; one atomic add per weight and block.
template <int CIN, int COUT>
__global__ void __launch_bounds__(256, (CIN * COUT > 256) ? 1 : 2)
    k_lp_conv_dw_tiled(LpDims d, const bf16* __restrict__ in, const bf16* __restrict__ dy, float* __restrict__ dw,
                       float* __restrict__ db) {
    static_assert((CIN == 16 || CIN == 32) && (COUT == 16 || COUT == 32) && CIN * COUT <= 512, "channel counts");
    constexpr int SX = CIN + 8, SD = COUT + 8, CH = CIN / 8, NT = CIN / 8, MT = COUT / 16, TPW = 4;
    constexpr int kTile = kTX * kTY * kTZ;
    __shared__ __align__(16) bf16 sX[kHalo * SX];
    __shared__ __align__(16) bf16 sD[kTile * SD];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, gid = lane >> 2, tig = lane & 3;
    const int lq = lane >> 3, lr = lane & 7;
    const uint32_t sX_s = (uint32_t)__cvta_generic_to_shared(sX);
    const uint32_t sD_s = (uint32_t)__cvta_generic_to_shared(sD);
    const int tiles_x = (d.W + kTX - 1) / kTX, tiles_y = (d.H + kTY - 1) / kTY;
    const long long ntiles = (long long)tiles_x * tiles_y * ((d.D + kTZ - 1) / kTZ);
    float acc[TPW][MT][NT][4];
#pragma unroll
    for (int q = 0; q < TPW; ++q)
#pragma unroll
        for (int mt = 0; mt < MT; ++mt)
#pragma unroll
            for (int nt = 0; nt < NT; ++nt)
                acc[q][mt][nt][0] = acc[q][mt][nt][1] = acc[q][mt][nt][2] = acc[q][mt][nt][3] = 0.f;
    float bacc = 0.f;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int tx = (int)(tile % tiles_x), ty = (int)((tile / tiles_x) % tiles_y), tz = (int)(tile / ((long long)tiles_x * tiles_y));
        const int x0 = tx * kTX, y0 = ty * kTY, z0 = tz * kTZ;
        for (int e = threadIdx.x; e < kHalo * CH; e += blockDim.x) {
            const int hv = e / CH, q = e - hv * CH;
            const int hx = hv % kHX, hy = (hv / kHX) % kHY, hz = hv / (kHX * kHY);
            const int gx = x0 + hx - 1, gy = y0 + hy - 1, gz = z0 + hz - 1;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (gx >= 0 && gx < d.W && gy >= 0 && gy < d.H && gz >= 0 && gz < d.D)
                v = __ldg(reinterpret_cast<const uint4*>(in + (((long long)gz * d.H + gy) * d.W + gx) * CIN) + q);
            *reinterpret_cast<uint4*>(sX + hv * SX + q * 8) = v;
        }
        for (int e = threadIdx.x; e < kTile * (COUT / 8); e += blockDim.x) {
            const int vv = e / (COUT / 8), c8 = e - vv * (COUT / 8);
            const int gx = x0 + vv % kTX, gy = y0 + (vv / kTX) % kTY, gz = z0 + vv / (kTX * kTY);
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (gx < d.W && gy < d.H && gz < d.D)
                v = __ldg(reinterpret_cast<const uint4*>(dy + (((long long)gz * d.H + gy) * d.W + gx) * COUT) + c8);
            *reinterpret_cast<uint4*>(sD + vv * SD + c8 * 8) = v;
        }
        __syncthreads();
        if (threadIdx.x < COUT)
            for (int vv = 0; vv < kTile; ++vv) bacc += __bfloat162float(sD[vv * SD + threadIdx.x]);
#pragma unroll 1
        for (int r = 0; r < kTY * kTZ; ++r) {  // rows of 16 voxels: the K steps
            const int ry = r % kTY, rz = r / kTY;
            uint32_t a[MT][4];
#pragma unroll
            for (int mt = 0; mt < MT; ++mt)
                ldmatrix_x4_trans(a[mt], sD_s + 2u * (uint32_t)((r * kTX + (lq >> 1) * 8 + lr) * SD + mt * 16 + (lq & 1) * 8));
#pragma unroll
            for (int q = 0; q < TPW; ++q) {
                const int t = warp + 8 * q;
                if (t < 27) {
                    const int tdz = t / 9 - 1, tdy = (t / 3) % 3 - 1, tdx = t % 3 - 1;
                    const int hrow = ((rz + 1 + tdz) * kHY + (ry + 1 + tdy)) * kHX + 1 + tdx;
#pragma unroll
                    for (int nt = 0; nt < NT; ++nt) {
                        uint32_t b[2];
                        ldmatrix_x2_trans(b, sX_s + 2u * (uint32_t)((hrow + (lq & 1) * 8 + lr) * SX + nt * 8));
#pragma unroll
                        for (int mt = 0; mt < MT; ++mt) mma_16816(acc[q][mt][nt], a[mt], b);
                    }
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < TPW; ++q) {
        const int t = warp + 8 * q;
        if (t < 27) {
            float* base = dw + (size_t)t * COUT * CIN;
#pragma unroll
            for (int mt = 0; mt < MT; ++mt)
#pragma unroll
                for (int nt = 0; nt < NT; ++nt) {
                    const size_t r0 = (size_t)(mt * 16 + gid) * CIN + nt * 8 + tig * 2, r1 = r0 + 8 * CIN;
                    atomicAdd(&base[r0], acc[q][mt][nt][0]);
                    atomicAdd(&base[r0 + 1], acc[q][mt][nt][1]);
                    atomicAdd(&base[r1], acc[q][mt][nt][2]);
                    atomicAdd(&base[r1 + 1], acc[q][mt][nt][3]);
                }
        }
    }
    if (threadIdx.x < COUT) atomicAdd(&db[threadIdx.x], bacc);
}

// wt[26 - tap][ci][co] = w[tap][co][ci] (the input-gradient convolution)
__global__ void k_lp_wt(const bf16* __restrict__ w, bf16* __restrict__ wt, int cin, int cout) {
    const int n = 27 * cin * cout;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const int t = e / (cin * cout), rem = e - t * cin * cout;
        const int co = rem / cin, ci = rem - co * cin;
        wt[((size_t)(26 - t) * cin + ci) * cout + co] = w[e];
    }
}

// the 16-channel input: channels 0..2 from three FP32 fields, the rest 0
// Elementwise kernels: one thread per voxel and 16-byte group of channels (8 BF16 or 4 FP32),
// so that each decodes its voxel once and moves whole 16-byte words; the arithmetic (order of
// the sums included) is per channel as written.
__device__ __forceinline__ void bf8_to_f(const uint4& u, float (&f)[8]) {
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        f[2 * q] = __uint_as_float(w[q] << 16);
        f[2 * q + 1] = __uint_as_float(w[q] & 0xffff0000u);
    }
}

__device__ __forceinline__ uint32_t bf2_bits(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

__device__ __forceinline__ uint4 f_to_bf8(const float (&f)[8]) {
    return make_uint4(bf2_bits(f[0], f[1]), bf2_bits(f[2], f[3]), bf2_bits(f[4], f[5]), bf2_bits(f[6], f[7]));
}

// the 16 input channels: the three fields, then zeros
__global__ void k_lp_pack(LpDims d, const float* __restrict__ c0, const float* __restrict__ c1,
                          const float* __restrict__ c2, bf16* __restrict__ x) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < d.N; v += (long long)gridDim.x * blockDim.x) {
        uint4* o = reinterpret_cast<uint4*>(x + v * 16);
        o[0] = make_uint4(bf2_bits(c0[v], c1[v]), bf2_bits(c2[v], 0.f), 0u, 0u);
        o[1] = make_uint4(0u, 0u, 0u, 0u);
    }
}

// coarse = mean of the 2x2x2 children (fine dims 2 dc), C a multiple of 8
__global__ void k_lp_pool(LpDims dc, int C, const bf16* __restrict__ fine, bf16* __restrict__ coarse) {
    const int Wf = dc.W * 2, Hf = dc.H * 2, CH = C / 8, sh = __ffs(CH) - 1;
    const long long n = dc.N * CH;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const long long v = e >> sh;
        const int q = (int)(e - (v << sh));
        int z, y, x;
        lp_decode(dc, v, z, y, x);
        float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                for (int c = 0; c < 2; ++c) {
                    float f[8];
                    bf8_to_f(__ldg(reinterpret_cast<const uint4*>(
                                 fine + ((((long long)(2 * z + a) * Hf) + 2 * y + b) * Wf + 2 * x + c) * C) + q),
                             f);
#pragma unroll
                    for (int k = 0; k < 8; ++k) s[k] += f[k];
                }
#pragma unroll
        for (int k = 0; k < 8; ++k) s[k] *= 0.125f;
        reinterpret_cast<uint4*>(coarse + v * C)[q] = f_to_bf8(s);
    }
}

// out(fine) = coarse(parent) + skip, C a multiple of 8
__global__ void k_lp_up_add(LpDims df, int C, const bf16* __restrict__ coarse, const bf16* __restrict__ skip,
                            bf16* __restrict__ out) {
    const int Wc = df.W / 2, Hc = df.H / 2, CH = C / 8, sh = __ffs(CH) - 1;
    const long long n = df.N * CH;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const long long v = e >> sh;
        const int q = (int)(e - (v << sh));
        int z, y, x;
        lp_decode(df, v, z, y, x);
        const long long p = (((long long)(z / 2) * Hc) + y / 2) * Wc + x / 2;
        float a[8], b[8];
        bf8_to_f(__ldg(reinterpret_cast<const uint4*>(coarse + p * C) + q), a);
        bf8_to_f(__ldg(reinterpret_cast<const uint4*>(skip + v * C) + q), b);
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] += b[k];
        reinterpret_cast<uint4*>(out + v * C)[q] = f_to_bf8(a);
    }
}

// coarse gradient = sum of the 8 children's gradients (backward of the upsampling), C a
// multiple of 4
__global__ void k_lp_up_bwd(LpDims dc, int C, const float* __restrict__ fine, float* __restrict__ coarse) {
    const int Wf = dc.W * 2, Hf = dc.H * 2, CH = C / 4, sh = __ffs(CH) - 1;
    const long long n = dc.N * CH;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const long long v = e >> sh;
        const int q = (int)(e - (v << sh));
        int z, y, x;
        lp_decode(dc, v, z, y, x);
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                for (int c = 0; c < 2; ++c) {
                    const float4 f = __ldg(reinterpret_cast<const float4*>(
                                               fine + ((((long long)(2 * z + a) * Hf) + 2 * y + b) * Wf + 2 * x + c) * C) +
                                           q);
                    s.x += f.x; s.y += f.y; s.z += f.z; s.w += f.w;
                }
        reinterpret_cast<float4*>(coarse + v * C)[q] = s;
    }
}

// fine gradient += coarse gradient (parent) / 8 (backward of the pooling), C a multiple of 4
__global__ void k_lp_pool_bwd_add(LpDims df, int C, const float* __restrict__ coarse, float* __restrict__ fine) {
    const int Wc = df.W / 2, Hc = df.H / 2, CH = C / 4, sh = __ffs(CH) - 1;
    const long long n = df.N * CH;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const long long v = e >> sh;
        const int q = (int)(e - (v << sh));
        int z, y, x;
        lp_decode(df, v, z, y, x);
        const long long p = (((long long)(z / 2) * Hc) + y / 2) * Wc + x / 2;
        const float4 c = __ldg(reinterpret_cast<const float4*>(coarse + p * C) + q);
        float4* f = reinterpret_cast<float4*>(fine + v * C) + q;
        float4 o = *f;
        o.x += c.x * 0.125f; o.y += c.y * 0.125f; o.z += c.z * 0.125f; o.w += c.w * 0.125f;
        *f = o;
    }
}

// BF16 gradient at a layer output: d masked by the ReLU (out > 0) when relu is set; n a
// multiple of 8
__global__ void k_lp_mask(long long n, const float* __restrict__ d, const bf16* __restrict__ out, int relu,
                          bf16* __restrict__ q) {
    const long long n8 = n / 8;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n8; e += (long long)gridDim.x * blockDim.x) {
        const float4 d0 = __ldg(reinterpret_cast<const float4*>(d) + 2 * e);
        const float4 d1 = __ldg(reinterpret_cast<const float4*>(d) + 2 * e + 1);
        float v[8] = {d0.x, d0.y, d0.z, d0.w, d1.x, d1.y, d1.z, d1.w};
        if (relu) {
            float o[8];
            bf8_to_f(__ldg(reinterpret_cast<const uint4*>(out) + e), o);
#pragma unroll
            for (int k = 0; k < 8; ++k) v[k] = o[k] > 0.f ? v[k] : 0.f;
        }
        reinterpret_cast<uint4*>(q)[e] = f_to_bf8(v);
    }
}

// masked mean-square loss on output channel 0 and its gradient (16 channels, the others 0);
// partial sums of the squared error per block
__global__ void __launch_bounds__(kBlock) k_lp_loss(long long N, const float* __restrict__ y, int ys,
                                                    const float* __restrict__ target, const float* __restrict__ mask,
                                                    float inv_n, float* __restrict__ dy, double* __restrict__ partials) {
    double acc = 0.0;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < N; v += (long long)gridDim.x * blockDim.x) {
        const float m = mask[v];
        const float diff = (y[v * ys] - target[v]) * m;
        acc += (double)diff * diff;
        float4* o = reinterpret_cast<float4*>(dy + v * 16);
        o[0] = make_float4(2.f * diff * inv_n, 0.f, 0.f, 0.f);
        for (int q = 1; q < 4; ++q) o[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    double a[1] = {acc};
    block_sum_store<1>(a, partials);
}

// output channel 0 to FP32
__global__ void k_lp_out(long long N, const float* __restrict__ y, int ys, float* __restrict__ out) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < N; v += (long long)gridDim.x * blockDim.x)
        out[v] = y[v * ys];
}

// Adam on the FP32 master parameters; the BF16 copy of every weight follows
__global__ void k_lp_adam(long long n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                          float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2,
                          const int* __restrict__ bf_index, bf16* __restrict__ pw) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float ge = g[e];
        const float me = b1 * m[e] + (1.f - b1) * ge;
        const float ve = b2 * v[e] + (1.f - b2) * ge * ge;
        m[e] = me;
        v[e] = ve;
        const float pe = p[e] - lr * (me / c1) / (sqrtf(ve / c2) + eps);
        p[e] = pe;
        const int bi = bf_index[e];
        if (bi >= 0) pw[bi] = __float2bfloat16_rn(pe);
    }
}

// FP32 -> BF16 copy of the weights (after a parameter upload)
__global__ void k_lp_cast(long long n, const float* __restrict__ p, const int* __restrict__ bf_index,
                          bf16* __restrict__ pw) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int bi = bf_index[e];
        if (bi >= 0) pw[bi] = __float2bfloat16_rn(p[e]);
    }
}

// coarse = sum(fine * wt) / sum(wt) over each 2x2x2 block (wt null: the mean; a block with
// no weight: 0); coarse dims dc, fine dims 2 dc
__global__ void k_lp_field_pool(LpDims dc, const float* __restrict__ fine, const float* __restrict__ wt,
                                float* __restrict__ coarse) {
    const int Wf = dc.W * 2, Hf = dc.H * 2;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < dc.N; v += (long long)gridDim.x * blockDim.x) {
        int z, y, x;
        lp_decode(dc, v, z, y, x);
        float s = 0.f, sw = 0.f;
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                for (int q = 0; q < 2; ++q) {
                    const long long f = (((long long)(2 * z + a) * Hf) + 2 * y + b) * Wf + 2 * x + q;
                    const float w = wt ? wt[f] : 1.f;
                    s += w * fine[f];
                    sw += w;
                }
        coarse[v] = sw > 0.f ? s / sw : 0.f;
    }
}

// fine = coarse(parent), fine dims df (even)
__global__ void k_lp_field_up(LpDims df, const float* __restrict__ coarse, float* __restrict__ fine) {
    const int Wc = df.W / 2, Hc = df.H / 2;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < df.N; v += (long long)gridDim.x * blockDim.x) {
        int z, y, x;
        lp_decode(df, v, z, y, x);
        fine[v] = coarse[(((long long)(z / 2) * Hc) + y / 2) * Wc + x / 2];
    }
}

}  // namespace
}  // namespace ls

// ---------------------------------------------------------------------------
// host side

namespace ls {

struct LpLayer {
    int cin, cout, relu;
    size_t w_off, b_off;    // FP32 parameter offsets (weights 27*cout*cin, bias cout)
    size_t wb_off;          // BF16 weight offset
};

constexpr int kLpLayers = 8;
// (cin, cout, relu): W0a, W0b, W1, W2, W3, U2, U1, U0
constexpr int kLpSpec[kLpLayers][3] = {{16, 16, 1}, {16, 16, 1}, {16, 32, 1}, {32, 64, 1},
                                       {64, 64, 1}, {64, 32, 1}, {32, 16, 1}, {16, 16, 0}};

}  // namespace ls

using ls::bf16;
using ls::kLpLayers;
using ls::kLpSpec;
using ls::LpDims;
using ls::LpLayer;

struct ls_lpnet {
    int D, H, W;
    int device, num_sms;
    int use_tc;             // convolutions: 3 the TMA-fed tcgen05 kernel (default), 0 mma.sync only, 1 the
                            // first tcgen05 kernel where it beat mma.sync
                            // (32 -> 64), 2 every layer with CIN <= 32 (LS_LPNET_TC)
    cudaStream_t stream;
    LpLayer layer[kLpLayers];
    size_t nparam, nweight_bf;
    float *p, *g, *m, *v;   // FP32 parameters, gradients, Adam moments
    int* bf_index;          // parameter -> BF16 weight index (-1 for biases)
    bf16* wb;               // BF16 weights
    bf16* wt;               // BF16 transposed, flipped weights (input gradients)
    int adam_t;
    // activations (BF16) per level
    bf16 *x, *a0, *s0, *p1, *s1, *p2, *s2, *p3, *a3, *u2, *b2, *u1, *b1, *u0;
    float* y;               // FP32 output layer (channel 0 used): y_stride values per voxel
    int y_stride;           // 16, or 1 where the layer stores channel 0 alone
    // gradients (FP32)
    float *gy, *g0, *g0b, *g1, *g1b, *g2, *g2b, *g3, *g3b;
    bf16* q;                // BF16 masked gradient scratch
    float* out;             // FP32 output (channel 0)
    double* partials;
    double* h_loss;
    std::vector<void*> allocs;
    std::string err;
};

namespace {

constexpr int kLpMaxDevices = 64;

ls_status lp_fail(ls_lpnet* n, const char* what, cudaError_t e) {
    if (n) {
        char buf[256];
        snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
        n->err = buf;
    }
    return LS_CUDA_ERROR;
}

#define LP_CUDA(n, expr)                                     \
    do {                                                     \
        cudaError_t e__ = (expr);                            \
        if (e__ != cudaSuccess) return lp_fail((n), #expr, e__); \
    } while (0)
#define LP_LAUNCH(n, kernel, grid, block, ...)                             \
    do {                                                                   \
        kernel<<<(grid), (block), 0, (n)->stream>>>(__VA_ARGS__);          \
        cudaError_t e__ = cudaGetLastError();                              \
        if (e__ != cudaSuccess) return lp_fail((n), #kernel, e__);         \
    } while (0)

template <typename T>
ls_status lp_alloc(ls_lpnet* n, T** p, size_t count) {
    void* v = nullptr;
    LP_CUDA(n, cudaMalloc(&v, count * sizeof(T) + 16));
    n->allocs.push_back(v);
    *p = (T*)v;
    return LS_OK;
}

int lp_grid(const ls_lpnet* n, long long work, int block) {
    long long b = (work + block - 1) / block;
    const long long cap = (long long)n->num_sms * 16;
    if (b > cap) b = cap;
    return (int)(b < 1 ? 1 : b);
}

// conv forward / input-gradient dispatch over the channel pairs of the network
// The first tcgen05 kernel (k_lp_conv_tc): planes per tile, halo buffers and persistence,
// measured per layer at 144x176x176 (the
// weights plus NBUF halo buffers fit one CTA's shared memory, <= 227 KB). The layers with
// 16 input or 16 output channels run one tile per CTA, two or three CTAs per SM overlapping
// one another's staging and MMAs (16 -> 16: 420 us so, 479 as persistent CTAs three per SM
// with the weights kept, 542 as one persistent CTA per SM with two halo buffers). 32 -> 64,
// whose weights take 110 KB, runs persistent CTAs that stage them once: 47 us against 54
// with one tile per CTA.
template <int CI, int CO>
struct TcPlanes {
    static constexpr int value = (CI == 16) ? 2 : (CO == 16 ? 4 : 1);
    static constexpr int nbuf = 1;
    static constexpr bool persist = (CI == 32 && CO == 64);
};

template <int CI, int CO, bool RELU, typename OutT>
ls_status lp_conv_tc(ls_lpnet* n, LpDims d, const bf16* in, const bf16* w, const float* bias, OutT* out) {
    constexpr int ZT = TcPlanes<CI, CO>::value, NB = TcPlanes<CI, CO>::nbuf;
    using S = ls::TcShape<CI, CO, ZT>;
    constexpr int smem = S::w_bytes + NB * S::a_bytes;
    static_assert(smem + 1024 <= 227 * 1024, "shared memory per CTA");
    // the dynamic shared-memory opt-in and the occupancy, once per instantiation and device
    // (a function attribute belongs to the device's context, so each device sets its own)
    static std::mutex mu;
    static int per_sm_dev[kLpMaxDevices] = {0};
    int dev = 0;
    LP_CUDA(n, cudaGetDevice(&dev));
    if (dev < 0 || dev >= kLpMaxDevices) return lp_fail(n, "k_lp_conv_tc: device index", cudaErrorInvalidDevice);
    int per_sm = 0;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (!per_sm_dev[dev]) {
            LP_CUDA(n, cudaFuncSetAttribute(ls::k_lp_conv_tc<CI, CO, ZT, NB, RELU, OutT>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
            int occ = 0;
            LP_CUDA(n, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ls::k_lp_conv_tc<CI, CO, ZT, NB, RELU, OutT>,
                                                                     ls::kTcThreads, smem));
            per_sm_dev[dev] = occ < 1 ? 1 : occ;
        }
        per_sm = per_sm_dev[dev];
    }
    const long long ntiles = (long long)((d.W + ls::kTcX - 1) / ls::kTcX) * ((d.H + ls::kTcY - 1) / ls::kTcY) *
                             ((d.D + ZT - 1) / ZT);
    // persistent CTAs: as many as fit the SMs at once; otherwise one tile per CTA
    const long long slots = TcPlanes<CI, CO>::persist ? (long long)per_sm * n->num_sms : ntiles;
    const int grid = (int)(ntiles < slots ? ntiles : slots);
    ls::k_lp_conv_tc<CI, CO, ZT, NB, RELU, OutT><<<grid, ls::kTcThreads, smem, n->stream>>>(d, in, w, bias, out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return lp_fail(n, "k_lp_conv_tc", e);
    return LS_OK;
}

// cuTensorMapEncodeTiled, from the driver through the runtime's entry-point query (no link
// against the driver library); resolved when a network is created, never during a capture
typedef CUresult (*LpEncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

LpEncodeTiled lp_encode_tiled() {
    static const LpEncodeTiled fn = []() -> LpEncodeTiled {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return (LpEncodeTiled)p;
    }();
    return fn;
}

// The TMA-fed convolution (k_lp_conv_tma): a tensor map over the input (channels, x, y, z),
// 8-channel x 10 x 18 x 1 boxes, zeros outside; one persistent CTA per SM (it takes all 512
// TMEM columns: the shared memory asked for keeps a second CTA off the SM).
template <int CI, int CO, bool RELU, typename OutT>
ls_status lp_conv_tma(ls_lpnet* n, LpDims d, const bf16* in, const bf16* w, const float* bias, OutT* out,
                      int cout_total = CO, int co0 = 0, int ostride = CO, int only0 = 0) {
    using S = ls::TmShape<CI, CO>;
    constexpr int smem = S::smem < 116 * 1024 ? 116 * 1024 : S::smem;
    static_assert(smem <= 227 * 1024, "shared memory per CTA");
    const LpEncodeTiled enc = lp_encode_tiled();
    if (!enc) return lp_fail(n, "cuTensorMapEncodeTiled: not available", cudaErrorNotSupported);
    if (((uintptr_t)in & 15u) != 0) return lp_fail(n, "k_lp_conv_tma: input not 16-byte aligned", cudaErrorInvalidValue);
    alignas(64) CUtensorMap map;
    const cuuint64_t dims[4] = {(cuuint64_t)CI, (cuuint64_t)d.W, (cuuint64_t)d.H, (cuuint64_t)d.D};
    const cuuint64_t strides[3] = {(cuuint64_t)CI * 2, (cuuint64_t)d.W * CI * 2, (cuuint64_t)d.H * d.W * CI * 2};
    const cuuint32_t box[4] = {8, (cuuint32_t)ls::kTmHX, (cuuint32_t)ls::kTmHY, 1};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    const CUresult cr = enc(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void*)in, dims, strides, box, es,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) return lp_fail(n, "cuTensorMapEncodeTiled", cudaErrorInvalidValue);
    static std::mutex mu;
    static bool set_dev[kLpMaxDevices] = {false};
    int dev = 0;
    LP_CUDA(n, cudaGetDevice(&dev));
    if (dev < 0 || dev >= kLpMaxDevices) return lp_fail(n, "k_lp_conv_tma: device index", cudaErrorInvalidDevice);
    {
        std::lock_guard<std::mutex> lock(mu);
        if (!set_dev[dev]) {
            LP_CUDA(n, cudaFuncSetAttribute(ls::k_lp_conv_tma<CI, CO, RELU, OutT>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
            set_dev[dev] = true;
        }
    }
    // planes per tile: the most the tensor memory holds, fewer where the tiles would not
    // cover the SMs (the coarse levels)
    const long long txy = (long long)((d.W + ls::kTmX - 1) / ls::kTmX) * ((d.H + ls::kTmY - 1) / ls::kTmY);
    int zt = S::ZT;
    while (zt > 1 && txy * ((d.D + zt - 1) / zt) < n->num_sms) zt /= 2;
    const long long ntiles = txy * ((d.D + zt - 1) / zt);
    const int grid = (int)(ntiles < n->num_sms ? ntiles : n->num_sms);
    ls::k_lp_conv_tma<CI, CO, RELU, OutT><<<grid, ls::kTmThreads, smem, n->stream>>>(map, d, w, bias, out, cout_total,
                                                                                      co0, ostride, only0, zt);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return lp_fail(n, "k_lp_conv_tma", e);
    return LS_OK;
}

template <bool RELU, typename OutT>
ls_status lp_conv(ls_lpnet* n, LpDims d, int cin, int cout, const bf16* in, const bf16* w, const float* bias,
                  OutT* out) {
    // Measured per layer of the 144x176x176 network (ncu launch list): the TMA-fed kernel
    // 16 -> 16 in 160 us (mma.sync 308, the first tcgen05 kernel 420), 16 -> 32 in 37 (80 / 86),
    // 32 -> 64 in 28 (67 / 47), 32 -> 16 in 49 (107 / 126), 64 -> 32 in 29 (mma.sync 175).
    // LS_LPNET_TC=1: the first tcgen05 kernel on the 32 -> 64 layer alone, where it beat
    // mma.sync; 2: on every layer with up to 32 input channels; 0: mma.sync only.
    if (n->use_tc == 3) {
#define LP_TMA(CI, CO) \
        if (cin == CI && cout == CO) return lp_conv_tma<CI, CO, RELU, OutT>(n, d, in, w, bias, out);
        LP_TMA(16, 16) LP_TMA(16, 32) LP_TMA(32, 64) LP_TMA(32, 16) LP_TMA(64, 32)
#undef LP_TMA
        if (cin == 64 && cout == 64) {  // 221 KB of weights: two launches of 32 output channels
            LS_TRY((lp_conv_tma<64, 32, RELU, OutT>(n, d, in, w, bias, out, 64, 0, 64)));
            return lp_conv_tma<64, 32, RELU, OutT>(n, d, in, w, bias, out, 64, 32, 64);
        }
    }
    if (n->use_tc == 2) {
#define LP_TC(CI, CO) \
        if (cin == CI && cout == CO) return lp_conv_tc<CI, CO, RELU, OutT>(n, d, in, w, bias, out);
        LP_TC(16, 16) LP_TC(16, 32) LP_TC(32, 64) LP_TC(32, 16)
#undef LP_TC
    } else if (n->use_tc == 1 && cin == 32 && cout == 64) {
        return lp_conv_tc<32, 64, RELU, OutT>(n, d, in, w, bias, out);
    }
    if (cin <= 32) {
        const dim3 tg((unsigned)((d.W + ls::kTX - 1) / ls::kTX), (unsigned)((d.H + ls::kTY - 1) / ls::kTY),
                      (unsigned)((d.D + ls::kTZ - 1) / ls::kTZ));
#define LP_TCASE(CI, CO)                                                                         \
        if (cin == CI && cout == CO) {                                                           \
            LP_LAUNCH(n, (ls::k_lp_conv_tiled<CI, CO, RELU, OutT>), tg, 128, d, in, w, bias, out); \
            return LS_OK;                                                                        \
        }
        LP_TCASE(16, 16) LP_TCASE(16, 32) LP_TCASE(32, 64) LP_TCASE(32, 16)
#undef LP_TCASE
    }
    const int grid = lp_grid(n, (d.N + 15) / 16, 4);
#define LP_CASE(CI, CO)                                                                        \
    if (cin == CI && cout == CO) {                                                             \
        LP_LAUNCH(n, (ls::k_lp_conv<CI, CO, RELU, OutT>), grid, 128, d, in, w, bias, out);     \
        return LS_OK;                                                                          \
    }
    LP_CASE(16, 16) LP_CASE(16, 32) LP_CASE(32, 64) LP_CASE(64, 64) LP_CASE(64, 32) LP_CASE(32, 16)
#undef LP_CASE
    n->err = "unsupported channel pair";
    return LS_BAD_ARG;
}

ls_status lp_conv_dw(ls_lpnet* n, LpDims d, int cin, int cout, const bf16* in, const bf16* dy, float* dw, float* db) {
    // voxels per block: up to 2048, fewer on the coarse levels so that the 27 taps' blocks
    // still cover the SMs a few times over (multiples of the 64-voxel stage)
    long long ch = d.N / ((long long)n->num_sms * 2);
    ch = std::max(256ll, std::min(2048ll, (ch + 63) / 64 * 64));
    const int chunk = (int)ch;
    const dim3 grid((unsigned)((d.N + chunk - 1) / chunk), 27);
    // tensor cores (mma.sync); LS_LPNET_DW=0 keeps the FP32 FMA kernel (for comparison)
    static const bool fma_only = [] {
        const char* e = getenv("LS_LPNET_DW");
        return e && e[0] == '0';
    }();
    if (!fma_only && cin <= 32 && cout <= 32 && cin * cout <= 512) {
        // the halo staged once per tile for all 27 taps; persistent blocks, two per SM (one
        // where the accumulators of 16 x 32 weights per tap take the registers)
        const long long ntiles = (long long)((d.W + ls::kTX - 1) / ls::kTX) * ((d.H + ls::kTY - 1) / ls::kTY) *
                                 ((d.D + ls::kTZ - 1) / ls::kTZ);
        const long long cap = (cin * cout > 256 ? 1LL : 2LL) * n->num_sms;
        const int grid = (int)(ntiles < cap ? ntiles : cap);
        if (cin == 16 && cout == 16) LP_LAUNCH(n, (ls::k_lp_conv_dw_tiled<16, 16>), grid, 256, d, in, dy, dw, db);
        else if (cin == 16) LP_LAUNCH(n, (ls::k_lp_conv_dw_tiled<16, 32>), grid, 256, d, in, dy, dw, db);
        else LP_LAUNCH(n, (ls::k_lp_conv_dw_tiled<32, 16>), grid, 256, d, in, dy, dw, db);
        return LS_OK;
    }
#define LP_CASE(CI, CO)                                                                          \
    if (cin == CI && cout == CO) {                                                               \
        if (fma_only)                                                                            \
            LP_LAUNCH(n, (ls::k_lp_conv_dw<CI, CO>), grid, 256, d, in, dy, dw, db, chunk);       \
        else                                                                                     \
            LP_LAUNCH(n, (ls::k_lp_conv_dw_mma<CI, CO>), grid, 256, d, in, dy, dw, db, chunk);   \
        return LS_OK;                                                                            \
    }
    LP_CASE(16, 16) LP_CASE(16, 32) LP_CASE(32, 64) LP_CASE(64, 64) LP_CASE(64, 32) LP_CASE(32, 16)
#undef LP_CASE
    n->err = "unsupported channel pair";
    return LS_BAD_ARG;
}

ls_status lp_refresh_wt(ls_lpnet* n) {
    for (int l = 0; l < kLpLayers; ++l) {
        const LpLayer& L = n->layer[l];
        const int cnt = 27 * L.cin * L.cout;
        LP_LAUNCH(n, ls::k_lp_wt, lp_grid(n, cnt, 256), 256, n->wb + L.wb_off, n->wt + L.wb_off, L.cin, L.cout);
    }
    return LS_OK;
}

ls_status lp_forward(ls_lpnet* n, const float* c0, const float* c1, const float* c2) {
    const LpDims d0 = ls::lp_dims(n->D, n->H, n->W), d1 = ls::lp_dims(n->D / 2, n->H / 2, n->W / 2),
                 d2 = ls::lp_dims(n->D / 4, n->H / 4, n->W / 4), d3 = ls::lp_dims(n->D / 8, n->H / 8, n->W / 8);
    const LpLayer* L = n->layer;
    auto wb = [&](int l) { return (const bf16*)(n->wb + L[l].wb_off); };
    auto bias = [&](int l) { return (const float*)(n->p + L[l].b_off); };
    LP_LAUNCH(n, ls::k_lp_pack, lp_grid(n, d0.N, 256), 256, d0, c0, c1, c2, n->x);
    LS_TRY((lp_conv<true, bf16>(n, d0, 16, 16, n->x, wb(0), bias(0), n->a0)));
    LS_TRY((lp_conv<true, bf16>(n, d0, 16, 16, n->a0, wb(1), bias(1), n->s0)));
    LP_LAUNCH(n, ls::k_lp_pool, lp_grid(n, d1.N * 2, 256), 256, d1, 16, (const bf16*)n->s0, n->p1);
    LS_TRY((lp_conv<true, bf16>(n, d1, 16, 32, n->p1, wb(2), bias(2), n->s1)));
    LP_LAUNCH(n, ls::k_lp_pool, lp_grid(n, d2.N * 4, 256), 256, d2, 32, (const bf16*)n->s1, n->p2);
    LS_TRY((lp_conv<true, bf16>(n, d2, 32, 64, n->p2, wb(3), bias(3), n->s2)));
    LP_LAUNCH(n, ls::k_lp_pool, lp_grid(n, d3.N * 8, 256), 256, d3, 64, (const bf16*)n->s2, n->p3);
    LS_TRY((lp_conv<true, bf16>(n, d3, 64, 64, n->p3, wb(4), bias(4), n->a3)));
    LP_LAUNCH(n, ls::k_lp_up_add, lp_grid(n, d2.N * 8, 256), 256, d2, 64, (const bf16*)n->a3, (const bf16*)n->s2, n->u2);
    LS_TRY((lp_conv<true, bf16>(n, d2, 64, 32, n->u2, wb(5), bias(5), n->b2)));
    LP_LAUNCH(n, ls::k_lp_up_add, lp_grid(n, d1.N * 4, 256), 256, d1, 32, (const bf16*)n->b2, (const bf16*)n->s1, n->u1);
    LS_TRY((lp_conv<true, bf16>(n, d1, 32, 16, n->u1, wb(6), bias(6), n->b1)));
    LP_LAUNCH(n, ls::k_lp_up_add, lp_grid(n, d0.N * 2, 256), 256, d0, 16, (const bf16*)n->b1, (const bf16*)n->s0, n->u0);
    if (n->use_tc == 3) {
        // only output channel 0 is read (inference and loss): the layer stores it alone
        LS_TRY((lp_conv_tma<16, 16, false, float>(n, d0, n->u0, wb(7), bias(7), n->y, 16, 0, 1, 1)));
        n->y_stride = 1;
    } else {
        LS_TRY((lp_conv<false, float>(n, d0, 16, 16, n->u0, wb(7), bias(7), n->y)));
        n->y_stride = 16;
    }
    return LS_OK;
}

// backward of one layer: q = mask(d), dW += in^T q, dIn = conv(q, W^T) (dIn null: skipped)
ls_status lp_layer_bwd(ls_lpnet* n, int l, LpDims d, const bf16* in, const bf16* out, const float* dout, float* din) {
    const LpLayer& L = n->layer[l];
    LP_LAUNCH(n, ls::k_lp_mask, lp_grid(n, d.N * L.cout / 8, 256), 256, d.N * L.cout, dout, out, L.relu, n->q);
    LS_TRY(lp_conv_dw(n, d, L.cin, L.cout, in, (const bf16*)n->q, n->g + L.w_off, n->g + L.b_off));
    if (din) LS_TRY((lp_conv<false, float>(n, d, L.cout, L.cin, (const bf16*)n->q, n->wt + L.wb_off, nullptr, din)));
    return LS_OK;
}

// the gradient buffers, allocated by the first training step (inference needs none)
ls_status lp_alloc_grads(ls_lpnet* n) {
    if (n->gy) return LS_OK;
    const long long v0 = (long long)n->D * n->H * n->W, v1 = v0 / 8, v2 = v0 / 64, v3 = v0 / 512;
    LS_TRY(lp_alloc(n, &n->gy, v0 * 16));
    LS_TRY(lp_alloc(n, &n->g0, v0 * 16));
    LS_TRY(lp_alloc(n, &n->g0b, v0 * 16));
    LS_TRY(lp_alloc(n, &n->g1, v1 * 32));
    LS_TRY(lp_alloc(n, &n->g1b, v1 * 16));
    LS_TRY(lp_alloc(n, &n->g2, v2 * 64));
    LS_TRY(lp_alloc(n, &n->g2b, v2 * 32));
    LS_TRY(lp_alloc(n, &n->g3, v3 * 64));
    LS_TRY(lp_alloc(n, &n->g3b, v3 * 64));
    LS_TRY(lp_alloc(n, &n->q, v0 * 16));
    return LS_OK;
}

ls_status lp_backward(ls_lpnet* n) {
    const LpDims d0 = ls::lp_dims(n->D, n->H, n->W), d1 = ls::lp_dims(n->D / 2, n->H / 2, n->W / 2),
                 d2 = ls::lp_dims(n->D / 4, n->H / 4, n->W / 4), d3 = ls::lp_dims(n->D / 8, n->H / 8, n->W / 8);
    LP_CUDA(n, cudaMemsetAsync(n->g, 0, sizeof(float) * n->nparam, n->stream));
    LS_TRY(lp_layer_bwd(n, 7, d0, n->u0, nullptr, n->gy, n->g0));                  // d_u0 = d_s0 (partial)
    LP_LAUNCH(n, ls::k_lp_up_bwd, lp_grid(n, d1.N * 4, 256), 256, d1, 16, (const float*)n->g0, n->g1b);  // d_b1
    LS_TRY(lp_layer_bwd(n, 6, d1, n->u1, n->b1, n->g1b, n->g1));                    // d_u1
    LP_LAUNCH(n, ls::k_lp_up_bwd, lp_grid(n, d2.N * 8, 256), 256, d2, 32, (const float*)n->g1, n->g2b);  // d_b2
    LS_TRY(lp_layer_bwd(n, 5, d2, n->u2, n->b2, n->g2b, n->g2));                    // d_u2
    LP_LAUNCH(n, ls::k_lp_up_bwd, lp_grid(n, d3.N * 16, 256), 256, d3, 64, (const float*)n->g2, n->g3);   // d_a3
    LS_TRY(lp_layer_bwd(n, 4, d3, n->p3, n->a3, n->g3, n->g3b));                    // d_p3
    LP_LAUNCH(n, ls::k_lp_pool_bwd_add, lp_grid(n, d2.N * 16, 256), 256, d2, 64, (const float*)n->g3b, n->g2);  // d_s2
    LS_TRY(lp_layer_bwd(n, 3, d2, n->p2, n->s2, n->g2, n->g2b));                    // d_p2
    LP_LAUNCH(n, ls::k_lp_pool_bwd_add, lp_grid(n, d1.N * 8, 256), 256, d1, 32, (const float*)n->g2b, n->g1);  // d_s1
    LS_TRY(lp_layer_bwd(n, 2, d1, n->p1, n->s1, n->g1, n->g1b));                    // d_p1
    LP_LAUNCH(n, ls::k_lp_pool_bwd_add, lp_grid(n, d0.N * 4, 256), 256, d0, 16, (const float*)n->g1b, n->g0);  // d_s0
    LS_TRY(lp_layer_bwd(n, 1, d0, n->a0, n->s0, n->g0, n->g0b));                    // d_a0
    LS_TRY(lp_layer_bwd(n, 0, d0, n->x, n->a0, n->g0b, nullptr));
    return LS_OK;
}

}  // namespace

namespace ls {

// CTAs of k_lp_conv_tc whose bounded wait for their MMAs gave up since the last call (the
// counter is cleared); synchronous
// (LS_LPNET_SIMULATE_TIMEOUT=1 makes it report one, for tests of the host's response; no
// device wait is shortened or skipped)
int lpnet_tc_timeouts() {
    int v = 0, zero = 0;
    if (cudaMemcpyFromSymbol(&v, g_lp_tc_timeouts, sizeof(int)) != cudaSuccess) return 0;
    if (v) cudaMemcpyToSymbol(g_lp_tc_timeouts, &zero, sizeof(int));
    const char* sim = getenv("LS_LPNET_SIMULATE_TIMEOUT");
    if (sim && sim[0] == '1') v += 1;
    return v;
}

// Forward pass on another stream (the pressure context's: the learned coarse solver of its
// multigrid), channel 0 of the output into out (D*H*W floats); the network's own stream is
// restored afterwards. Asynchronous: no synchronisation, no allocation.
ls_status lpnet_forward_on(ls_lpnet* n, cudaStream_t s, const float* c0, const float* c1, const float* c2,
                           float* out, std::string* err) {
    cudaStream_t own = n->stream;
    n->stream = s;
    ls_status st = lp_forward(n, c0, c1, c2);
    if (st == LS_OK) {
        const long long N = (long long)n->D * n->H * n->W;
        k_lp_out<<<lp_grid(n, N, 256), 256, 0, s>>>(N, (const float*)n->y, n->y_stride, out);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) st = lp_fail(n, "k_lp_out", e);
    }
    n->stream = own;
    if (st != LS_OK && err) *err = n->err;
    return st;
}

}  // namespace ls

extern "C" {

ls_status ls_lpnet_create(int D, int H, int W, int seed, ls_lpnet** out) {
    if (!out) return LS_BAD_ARG;
    *out = nullptr;
    if (D < 8 || H < 8 || W < 8 || D % 8 || H % 8 || W % 8) return LS_BAD_ARG;
    if ((long long)D * H * W * 64 >= (1LL << 40)) return LS_BAD_ARG;
    ls_lpnet* n = new (std::nothrow) ls_lpnet();
    if (!n) return LS_CUDA_ERROR;
    n->D = D; n->H = H; n->W = W;
    n->y_stride = 16;
    ls_status st = LS_OK;
    auto fail = [&](ls_status s) { ls_lpnet_destroy(n); return s; };
    if (cudaGetDevice(&n->device) != cudaSuccess) return fail(LS_CUDA_ERROR);
    {
        const char* tc = getenv("LS_LPNET_TC");
        n->use_tc = (tc && tc[0] >= '0' && tc[0] <= '3') ? tc[0] - '0' : 3;
        if (n->use_tc == 3 && !lp_encode_tiled()) n->use_tc = 1;  // no tensor maps from this driver
    }
    cudaDeviceGetAttribute(&n->num_sms, cudaDevAttrMultiProcessorCount, n->device);
    if (cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(LS_CUDA_ERROR);
    size_t off = 0, boff = 0;
    for (int l = 0; l < kLpLayers; ++l) {
        LpLayer& L = n->layer[l];
        L.cin = kLpSpec[l][0]; L.cout = kLpSpec[l][1]; L.relu = kLpSpec[l][2];
        L.w_off = off; off += (size_t)27 * L.cin * L.cout;
        L.b_off = off; off += (size_t)L.cout;
        L.wb_off = boff; boff += (size_t)27 * L.cin * L.cout;
    }
    n->nparam = off;
    n->nweight_bf = boff;
    const long long v0 = (long long)D * H * W, v1 = v0 / 8, v2 = v0 / 64, v3 = v0 / 512;
    st = [&]() -> ls_status {
        LS_TRY(lp_alloc(n, &n->p, n->nparam));
        LS_TRY(lp_alloc(n, &n->g, n->nparam));
        LS_TRY(lp_alloc(n, &n->m, n->nparam));
        LS_TRY(lp_alloc(n, &n->v, n->nparam));
        LS_TRY(lp_alloc(n, &n->bf_index, n->nparam));
        LS_TRY(lp_alloc(n, &n->wb, n->nweight_bf));
        LS_TRY(lp_alloc(n, &n->wt, n->nweight_bf));
        LS_TRY(lp_alloc(n, &n->x, v0 * 16));
        LS_TRY(lp_alloc(n, &n->a0, v0 * 16));
        LS_TRY(lp_alloc(n, &n->s0, v0 * 16));
        LS_TRY(lp_alloc(n, &n->p1, v1 * 16));
        LS_TRY(lp_alloc(n, &n->s1, v1 * 32));
        LS_TRY(lp_alloc(n, &n->p2, v2 * 32));
        LS_TRY(lp_alloc(n, &n->s2, v2 * 64));
        LS_TRY(lp_alloc(n, &n->p3, v3 * 64));
        LS_TRY(lp_alloc(n, &n->a3, v3 * 64));
        LS_TRY(lp_alloc(n, &n->u2, v2 * 64));
        LS_TRY(lp_alloc(n, &n->b2, v2 * 32));
        LS_TRY(lp_alloc(n, &n->u1, v1 * 32));
        LS_TRY(lp_alloc(n, &n->b1, v1 * 16));
        LS_TRY(lp_alloc(n, &n->u0, v0 * 16));
        LS_TRY(lp_alloc(n, &n->y, v0 * 16));
        LS_TRY(lp_alloc(n, &n->out, v0));
        LS_TRY(lp_alloc(n, &n->partials, (size_t)n->num_sms * 16));
        if (cudaMallocHost(&n->h_loss, sizeof(double)) != cudaSuccess) return LS_CUDA_ERROR;
        // parameter -> BF16 weight index, He-normal weights from the seed, zero biases
        std::vector<int> idx(n->nparam, -1);
        std::vector<float> p(n->nparam, 0.f);
        unsigned long long s = 0x9E3779B97F4A7C15ull ^ (unsigned long long)(unsigned)seed;
        auto next = [&]() {  // splitmix64
            s += 0x9E3779B97F4A7C15ull;
            unsigned long long z = s;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            return z ^ (z >> 31);
        };
        for (int l = 0; l < kLpLayers; ++l) {
            const LpLayer& L = n->layer[l];
            const size_t cnt = (size_t)27 * L.cin * L.cout;
            const double sd = sqrt(2.0 / (27.0 * L.cin));
            for (size_t e = 0; e < cnt; ++e) {
                idx[L.w_off + e] = (int)(L.wb_off + e);
                // Box-Muller from two uniforms
                const double u1 = ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0);
                const double u2 = ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0);
                p[L.w_off + e] = (float)(sd * sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2));
            }
        }
        LP_CUDA(n, cudaMemcpy(n->bf_index, idx.data(), sizeof(int) * n->nparam, cudaMemcpyHostToDevice));
        LP_CUDA(n, cudaMemcpy(n->p, p.data(), sizeof(float) * n->nparam, cudaMemcpyHostToDevice));
        LP_CUDA(n, cudaMemset(n->m, 0, sizeof(float) * n->nparam));
        LP_CUDA(n, cudaMemset(n->v, 0, sizeof(float) * n->nparam));
        LP_LAUNCH(n, ls::k_lp_cast, lp_grid(n, (long long)n->nparam, 256), 256, (long long)n->nparam,
                  (const float*)n->p, (const int*)n->bf_index, n->wb);
        LS_TRY(lp_refresh_wt(n));
        LP_CUDA(n, cudaStreamSynchronize(n->stream));
        return LS_OK;
    }();
    if (st != LS_OK) return fail(st);
    *out = n;
    return LS_OK;
}

ls_status ls_lpnet_destroy(ls_lpnet* n) {
    if (!n) return LS_OK;
    if (n->stream) cudaStreamSynchronize(n->stream);
    for (void* q : n->allocs) cudaFree(q);
    if (n->h_loss) cudaFreeHost(n->h_loss);
    if (n->stream) cudaStreamDestroy(n->stream);
    delete n;
    return LS_OK;
}

const char* ls_lpnet_last_error(const ls_lpnet* n) { return n ? n->err.c_str() : "null network"; }

long long ls_lpnet_param_count(const ls_lpnet* n) { return n ? (long long)n->nparam : 0; }

ls_status ls_lpnet_get_params(ls_lpnet* n, float* host, long long count) {
    if (!n || !host || count != (long long)n->nparam) return LS_BAD_ARG;
    LP_CUDA(n, cudaMemcpyAsync(host, n->p, sizeof(float) * n->nparam, cudaMemcpyDeviceToHost, n->stream));
    LP_CUDA(n, cudaStreamSynchronize(n->stream));
    return LS_OK;
}

ls_status ls_lpnet_set_params(ls_lpnet* n, const float* host, long long count) {
    if (!n || !host || count != (long long)n->nparam) return LS_BAD_ARG;
    LP_CUDA(n, cudaMemcpyAsync(n->p, host, sizeof(float) * n->nparam, cudaMemcpyHostToDevice, n->stream));
    LP_LAUNCH(n, ls::k_lp_cast, lp_grid(n, (long long)n->nparam, 256), 256, (long long)n->nparam,
              (const float*)n->p, (const int*)n->bf_index, n->wb);
    LS_TRY(lp_refresh_wt(n));
    LP_CUDA(n, cudaMemsetAsync(n->m, 0, sizeof(float) * n->nparam, n->stream));
    LP_CUDA(n, cudaMemsetAsync(n->v, 0, sizeof(float) * n->nparam, n->stream));
    n->adam_t = 0;
    LP_CUDA(n, cudaStreamSynchronize(n->stream));
    return LS_OK;
}

ls_status ls_lpnet_get_grads(ls_lpnet* n, float* host, long long count) {
    if (!n || !host || count != (long long)n->nparam) return LS_BAD_ARG;
    LP_CUDA(n, cudaMemcpyAsync(host, n->g, sizeof(float) * n->nparam, cudaMemcpyDeviceToHost, n->stream));
    LP_CUDA(n, cudaStreamSynchronize(n->stream));
    return LS_OK;
}

ls_status ls_lpnet_forward(ls_lpnet* n, const float* c0, const float* c1, const float* c2, float* out) {
    if (!n || !c0 || !c1 || !c2 || !out) return LS_BAD_ARG;
    LS_TRY(lp_forward(n, c0, c1, c2));
    const long long N = (long long)n->D * n->H * n->W;
    LP_LAUNCH(n, ls::k_lp_out, lp_grid(n, N, 256), 256, N, (const float*)n->y, n->y_stride, out);
    LP_CUDA(n, cudaStreamSynchronize(n->stream));
    if (ls::lpnet_tc_timeouts()) {
        // A tcgen05 wait gave up: the output is not valid, and the state a timed-out CTA left
        // (tensor memory, shared memory, MMAs still in flight) is not trusted again. This network
        // runs the mma.sync kernels from now on; the pass is recomputed with them.
        n->use_tc = 0;
        n->err = "tensor-core convolution: a wait for the MMAs gave up; recomputed with mma.sync";
        LS_TRY(lp_forward(n, c0, c1, c2));
        LP_LAUNCH(n, ls::k_lp_out, lp_grid(n, N, 256), 256, N, (const float*)n->y, n->y_stride, out);
        LP_CUDA(n, cudaStreamSynchronize(n->stream));
        return LS_STAGNATED_FALLBACK_USED;
    }
    return LS_OK;
}

ls_status ls_lpnet_train_step(ls_lpnet* n, const float* c0, const float* c1, const float* c2, const float* target,
                              const float* mask, long long mask_count, float lr, int update, double* loss) {
    if (!n || !c0 || !c1 || !c2 || !target || !mask || mask_count < 1 || !(lr >= 0.f)) return LS_BAD_ARG;
    LS_TRY(lp_alloc_grads(n));
    LS_TRY(lp_forward(n, c0, c1, c2));
    const long long N = (long long)n->D * n->H * n->W;
    const int nb = lp_grid(n, N, ls::kBlock);
    LP_LAUNCH(n, ls::k_lp_loss, nb, ls::kBlock, N, (const float*)n->y, n->y_stride, target, mask, (float)(1.0 / (double)mask_count),
              n->gy, n->partials);
    LS_TRY(lp_backward(n));
    if (update) {
        n->adam_t += 1;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = (float)(1.0 - pow((double)b1, n->adam_t)), c2 = (float)(1.0 - pow((double)b2, n->adam_t));
        LP_LAUNCH(n, ls::k_lp_adam, lp_grid(n, (long long)n->nparam, 256), 256, (long long)n->nparam, n->p,
                  (const float*)n->g, n->m, n->v, lr, b1, b2, 1e-8f, c1, c2, (const int*)n->bf_index, n->wb);
        LS_TRY(lp_refresh_wt(n));
    }
    std::vector<double> part(nb);
    LP_CUDA(n, cudaMemcpyAsync(part.data(), n->partials, sizeof(double) * nb, cudaMemcpyDeviceToHost, n->stream));
    LP_CUDA(n, cudaStreamSynchronize(n->stream));
    if (ls::lpnet_tc_timeouts()) {
        n->use_tc = 0;  // as in ls_lpnet_forward: no further tcgen05 launches on this network
        n->err = "tensor-core convolution: a wait for the MMAs gave up";
        return LS_TIMEOUT;
    }
    double sum = 0.0;
    for (double v : part) sum += v;
    if (loss) *loss = sum / (double)mask_count;
    return LS_OK;
}

ls_status ls_field_pool2(int D, int H, int W, const float* fine, const float* weight, float* coarse) {
    if (!fine || !coarse || D < 2 || H < 2 || W < 2 || D % 2 || H % 2 || W % 2) return LS_BAD_ARG;
    const LpDims dc = ls::lp_dims(D / 2, H / 2, W / 2);
    long long b = (dc.N + 255) / 256;
    if (b > 4096) b = 4096;
    ls::k_lp_field_pool<<<(int)b, 256>>>(dc, fine, weight, coarse);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return LS_CUDA_ERROR;
    return LS_OK;
}

ls_status ls_field_up2(int D, int H, int W, const float* coarse, float* fine) {
    if (!fine || !coarse || D < 2 || H < 2 || W < 2 || D % 2 || H % 2 || W % 2) return LS_BAD_ARG;
    const LpDims df = ls::lp_dims(D, H, W);
    long long b = (df.N + 255) / 256;
    if (b > 4096) b = 4096;
    ls::k_lp_field_up<<<(int)b, 256>>>(df, coarse, fine);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return LS_CUDA_ERROR;
    return LS_OK;
}

}  // extern "C"
