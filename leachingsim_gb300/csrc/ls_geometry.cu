// ls_geometry.cu - geometry pre-processing of label images on the GPU: the reference's
// coarsen_grid.py (2x2x2 ranked priority voting), clean_micro_ct.py (opening of the pore
// space, connected components, removal of pore islands not reached from the ambient Air or
// from the x = 0 face), micro_fracture.py (centre lines from encapsulated Sulphide to the
// nearest Pore through an exact Euclidean feature transform, widened by a 3x3x3 dilation)
// and a threshold classification of uint16 grey-level images.
//
// Stand-alone entry points on host buffers (no context): each allocates its device scratch,
// runs on the current device's default stream and returns when the result is in the host
// buffer.
#include <cstdio>
#include <cstring>

#include "ls_internal.cuh"

namespace ls {
namespace {

constexpr int kGeoSpin = 1 << 20;  // bound on the union-find retry loop

struct Dims {
    int I, J, K;
    long long JK, N;
};

__device__ __forceinline__ void gdecode(const Dims& d, long long r, int& i, int& j, int& k) {
    i = (int)(r / d.JK);
    const long long rem = r - (long long)i * d.JK;
    j = (int)(rem / d.K);
    k = (int)(rem - (long long)j * d.K);
}

// coarsen_grid.py:20-62: ranked priority voting over each 2x2x2 block; planes beyond the
// input's slowest extent are Air (the script's padding plane)
template <typename L>
__global__ void k_coarsen(Dims in, Dims out, const L* __restrict__ src, L* __restrict__ dst) {
    for (long long R = blockIdx.x * (long long)blockDim.x + threadIdx.x; R < out.N;
         R += (long long)gridDim.x * blockDim.x) {
        int I, J, K;
        gdecode(out, R, I, J, K);
        bool pore = false, air = false, sul = false;
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                for (int c = 0; c < 2; ++c) {
                    const int i = 2 * I + a, j = 2 * J + b, k = 2 * K + c;
                    const int v = (i < in.I) ? (int)src[(long long)i * in.JK + (long long)j * in.K + k] : kAir;
                    pore |= v == kPore;
                    air |= v == kAir;
                    sul |= v == kSulphide;
                }
        dst[R] = (L)(sul ? kSulphide : air ? kAir : pore ? kPore : kRock);
    }
}

// mask of label == v
template <typename L>
__global__ void k_mask_eq(Dims d, const L* __restrict__ lab, int v, uint8_t* __restrict__ m) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < d.N;
         r += (long long)gridDim.x * blockDim.x)
        m[r] = (int)lab[r] == v ? 1 : 0;
}

// mask of label != v
template <typename L>
__global__ void k_mask_ne(Dims d, const L* __restrict__ lab, int v, uint8_t* __restrict__ m) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < d.N;
         r += (long long)gridDim.x * blockDim.x)
        m[r] = (int)lab[r] != v ? 1 : 0;
}

// 6-neighbour erosion (ERODE) or dilation with the centre included; voxels outside the image
// count as background
template <bool ERODE>
__global__ void k_morph6(Dims d, const uint8_t* __restrict__ in, uint8_t* __restrict__ out) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < d.N;
         r += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        gdecode(d, r, i, j, k);
        const bool nb[6] = {i > 0 && in[r - d.JK], i + 1 < d.I && in[r + d.JK], j > 0 && in[r - d.K],
                            j + 1 < d.J && in[r + d.K], k > 0 && in[r - 1], k + 1 < d.K && in[r + 1]};
        bool v = in[r] != 0;
        for (int q = 0; q < 6; ++q) v = ERODE ? (v && nb[q]) : (v || nb[q]);
        out[r] = v ? 1 : 0;
    }
}

// union-find over 6-connected mask voxels; the root of a component is its smallest voxel.
// Hooking phase: find with path halving. Every store points a non-root at one of its
// ancestors, and a value read from a stale L1 line (L1 is not coherent across SMs) is a
// former ancestor, so the races between threads are benign. A stale line can show a root
// that another SM has hooked since: the CAS then fails, and the retry uses FRESH loads that
// bypass L1.
template <bool FRESH>
__device__ __forceinline__ int gfind(int* parent, int x) {
    int p = FRESH ? __ldcg(parent + x) : parent[x];
    int guard = 0;
    while (p != x && guard++ < kGeoSpin) {
        const int gp = FRESH ? __ldcg(parent + p) : parent[p];
        parent[x] = gp;
        x = p;
        p = gp;
    }
    return x;
}

// Compression phase: a read-only find. With path halving here, a thread holding an old
// parent value could overwrite a voxel's final root with an intermediate ancestor after the
// voxel's own thread had stored the root.
__device__ __forceinline__ int gfind_ro(const int* parent, int x) {
    int p = parent[x];
    int guard = 0;
    while (p != x && guard++ < kGeoSpin) {
        x = p;
        p = parent[x];
    }
    return x;
}

__global__ void k_uf_init(Dims d, const uint8_t* __restrict__ m, int* __restrict__ parent) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < d.N;
         r += (long long)gridDim.x * blockDim.x)
        parent[r] = m[r] ? (int)r : -1;
}

__global__ void k_uf_hook(Dims d, const uint8_t* __restrict__ m, int* parent, int* __restrict__ err) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < d.N;
         r += (long long)gridDim.x * blockDim.x) {
        if (!m[r]) continue;
        int i, j, k;
        gdecode(d, r, i, j, k);
        const bool has[3] = {i + 1 < d.I, j + 1 < d.J, k + 1 < d.K};
        const long long off[3] = {d.JK, d.K, 1};
        for (int q = 0; q < 3; ++q) {
            if (!has[q] || !m[r + off[q]]) continue;
            int a = (int)r, b = (int)(r + off[q]);
            int spins = 0;
            while (true) {
                const int ra = spins ? gfind<true>(parent, a) : gfind<false>(parent, a);
                const int rb = spins ? gfind<true>(parent, b) : gfind<false>(parent, b);
                if (ra == rb) break;
                const int lo = ra < rb ? ra : rb, hi = ra < rb ? rb : ra;
                if (atomicCAS(&parent[hi], hi, lo) == hi) break;
                if (++spins > kGeoSpin) { atomicExch(err, 1); break; }
            }
        }
    }
}

__global__ void k_uf_compress(Dims d, int* parent) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < d.N;
         r += (long long)gridDim.x * blockDim.x)
        if (parent[r] >= 0) parent[r] = gfind_ro(parent, (int)r);
}

// voxel count of every component at its root
__global__ void k_uf_count(Dims d, const int* __restrict__ parent, unsigned int* __restrict__ count) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < d.N;
         r += (long long)gridDim.x * blockDim.x)
        if (parent[r] >= 0) atomicAdd(&count[parent[r]], 1u);
}

// largest component (ties: smallest root, i.e. met first in raster order) as a 64-bit key
// count << 32 | (0xffffffff - root), maximised
__global__ void k_uf_largest(Dims d, const int* __restrict__ parent, const unsigned int* __restrict__ count,
                             unsigned long long* __restrict__ best) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < d.N;
         r += (long long)gridDim.x * blockDim.x)
        if (parent[r] == (int)r) {
            const unsigned long long key = ((unsigned long long)count[r] << 32) |
                                           (unsigned long long)(0xffffffffu - (unsigned int)r);
            atomicMax(best, key);
        }
}

// mask of the voxels of component `root` (root < 0: every voxel outside the Air mask)
__global__ void k_comp_mask(Dims d, const int* __restrict__ parent, int root, uint8_t* __restrict__ m) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < d.N;
         r += (long long)gridDim.x * blockDim.x)
        m[r] = (root >= 0) ? (parent[r] == root ? 1 : 0) : (parent[r] < 0 ? 1 : 0);
}

// flag the components (roots) of opened-pore voxels that lie in `sel` (sel == nullptr: on
// the x = 0 face)
__global__ void k_mark_valid(Dims d, const int* __restrict__ parent, const uint8_t* __restrict__ sel,
                             uint8_t* __restrict__ valid) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < d.N;
         r += (long long)gridDim.x * blockDim.x) {
        const int p = parent[r];
        if (p < 0) continue;
        const bool s = sel ? sel[r] != 0 : (r % d.K) == 0;
        if (s) valid[p] = 1;
    }
}

// Pore voxels outside the kept opened components become Rock
template <typename L>
__global__ void k_clean_apply(Dims d, const int* __restrict__ parent, const uint8_t* __restrict__ valid,
                              L* __restrict__ lab, unsigned long long* __restrict__ changed) {
    unsigned long long n = 0;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < d.N;
         r += (long long)gridDim.x * blockDim.x) {
        if ((int)lab[r] != kPore) continue;
        const int p = parent[r];
        if (p >= 0 && valid[p]) continue;
        lab[r] = (L)kRock;
        ++n;
    }
    if (n) atomicAdd(changed, n);
}

template <typename L>
__global__ void k_classify(Dims d, const uint16_t* __restrict__ grey, int nt, const uint16_t* __restrict__ thr,
                           const int* __restrict__ labels, L* __restrict__ out) {
    __shared__ uint16_t st[16];
    __shared__ int sl[17];
    if (threadIdx.x < nt) st[threadIdx.x] = thr[threadIdx.x];
    if (threadIdx.x <= nt) sl[threadIdx.x] = labels[threadIdx.x];
    __syncthreads();
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < d.N;
         r += (long long)gridDim.x * blockDim.x) {
        const uint16_t gv = grey[r];
        int idx = 0;
        for (int q = 0; q < nt; ++q) idx += (st[q] <= gv) ? 1 : 0;
        out[r] = (L)sl[idx];
    }
}

// ---------------------------------------------------------------------------
// micro_fracture.py:21-93

// Sulphide voxels with no Pore among their six face neighbours (the script's
// sulphide & ~binary_dilation(pore)); also counts the Pore voxels
template <typename L>
__global__ void k_encapsulated(Dims d, const L* __restrict__ lab, uint8_t* __restrict__ enc,
                               unsigned long long* __restrict__ counts) {
    unsigned long long ne = 0, np = 0;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < d.N;
         r += (long long)gridDim.x * blockDim.x) {
        const int v = (int)lab[r];
        np += v == kPore;
        bool e = false;
        if (v == kSulphide) {
            int i, j, k;
            gdecode(d, r, i, j, k);
            const bool exposed = (i > 0 && (int)lab[r - d.JK] == kPore) || (i + 1 < d.I && (int)lab[r + d.JK] == kPore) ||
                                 (j > 0 && (int)lab[r - d.K] == kPore) || (j + 1 < d.J && (int)lab[r + d.K] == kPore) ||
                                 (k > 0 && (int)lab[r - 1] == kPore) || (k + 1 < d.K && (int)lab[r + 1] == kPore);
            e = !exposed;
        }
        enc[r] = e ? 1 : 0;
        ne += e;
    }
    if (ne) atomicAdd(&counts[0], ne);
    if (np) atomicAdd(&counts[1], np);
}

// feature of every Pore voxel is itself; others have none yet
template <typename L>
__global__ void k_ft_init(Dims d, const L* __restrict__ lab, int* __restrict__ feat) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < d.N;
         r += (long long)gridDim.x * blockDim.x)
        feat[r] = (int)lab[r] == kPore ? (int)r : -1;
}

// One pass of the separable exact Euclidean feature transform of Maurer, Qi and Raghavan
// ("A linear time algorithm for computing exact Euclidean distance transforms of binary
// images in arbitrary dimensions", IEEE PAMI 25(2), 2003), along axis AX, one thread per
// line. The passes run over the slowest axis first; after them every voxel holds its
// nearest Pore voxel. The feature found for position q of the line lies in the plane
// x_AX = q, so its coordinate along the line is q and its squared distance off the line
// only involves the axes already processed. A site whose Voronoi cell on the line is empty
// is dropped (the paper's RemoveEDT), and each position takes the first site of the
// remaining sequence that no later site beats strictly: the ties go to the earlier site,
// which is the choice scipy.ndimage.distance_transform_edt makes. The line's stack of sites
// lives in scratch at the line's own addresses.
//
// TR: the pass along the fastest axis (AX = 2) on the transposed array featT[k][i J + j]
// (ft_transpose), whose lines run with stride I J, so that neighbouring threads (lines)
// touch neighbouring addresses; on the original layout each thread would walk its own
// contiguous line and a warp's loads would fall in 32 different sectors.
template <int AX, bool TR = false>
__global__ void k_ft_pass(Dims d, int* __restrict__ feat, int* __restrict__ st_site, int* __restrict__ st_pos,
                          long long* __restrict__ st_perp) {
    static_assert(!TR || AX == 2, "only the fastest-axis pass runs transposed");
    const long long nlines = AX == 0 ? d.JK : AX == 1 ? (long long)d.I * d.K : (long long)d.I * d.J;
    const int n = AX == 0 ? d.I : AX == 1 ? d.J : d.K;
    const long long stride = AX == 0 ? d.JK : AX == 1 ? (long long)d.K : (TR ? (long long)d.I * d.J : 1LL);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nlines;
         t += (long long)gridDim.x * blockDim.x) {
        long long base;
        int li = 0, lj = 0;  // the line's fixed coordinates on the axes before AX
        if (AX == 0) {
            base = t;
        } else if (AX == 1) {
            li = (int)(t / d.K);
            base = (long long)li * d.JK + (t - (long long)li * d.K);
        } else {
            li = (int)(t / d.J);
            lj = (int)(t - (long long)li * d.J);
            base = TR ? t : t * d.K;
        }
        // sweep 1: the sites whose cells on the line are not empty
        int ns = 0;
        for (int q = 0; q < n; ++q) {
            const int f = feat[base + q * stride];
            if (f < 0) continue;
            long long perp = 0;
            if (AX >= 1) {
                const long long di = (long long)(f / d.JK) - li;
                perp += di * di;
            }
            if (AX == 2) {
                const long long dj = (long long)((f / d.K) % d.J) - lj;
                perp += dj * dj;
            }
            while (ns >= 2) {
                const long long su = base + (ns - 2) * stride, sv = base + (ns - 1) * stride;
                const long long a = st_pos[sv] - st_pos[su], b = q - st_pos[sv], c = a + b;
                const long long v = c * st_perp[sv] - b * st_perp[su] - a * perp - a * b * c;
                if (v > 0) --ns;
                else break;
            }
            const long long sw = base + ns * stride;
            st_site[sw] = f;
            st_pos[sw] = q;
            st_perp[sw] = perp;
            ++ns;
        }
        if (ns == 0) continue;  // no site on the line: features stay -1
        // sweep 2: nearest site per position
        int l = 0;
        for (int q = 0; q < n; ++q) {
            while (l + 1 < ns) {
                const long long s0 = base + l * stride, s1 = s0 + stride;
                const long long d0 = st_perp[s0] + (long long)(st_pos[s0] - q) * (st_pos[s0] - q);
                const long long d1 = st_perp[s1] + (long long)(st_pos[s1] - q) * (st_pos[s1] - q);
                if (d0 > d1) ++l;
                else break;
            }
            feat[base + q * stride] = st_site[base + l * stride];
        }
    }
}

// out[c R + r] = in[r C + c]: the transpose of an R x C int matrix through 32 x 33 shared
// tiles (coalesced reads and writes)
__global__ void k_ft_transpose(const int* __restrict__ in, int* __restrict__ out, long long R, int C) {
    __shared__ int tile[32][33];
    const long long nbr = (R + 31) / 32;
    for (long long br = blockIdx.y; br < nbr; br += gridDim.y) {
        const long long r0 = br * 32;
        const int c0 = blockIdx.x * 32;
        for (int q = threadIdx.y; q < 32; q += blockDim.y) {
            const long long r = r0 + q;
            const int c = c0 + threadIdx.x;
            if (r < R && c < C) tile[q][threadIdx.x] = in[r * C + c];
        }
        __syncthreads();
        for (int q = threadIdx.y; q < 32; q += blockDim.y) {
            const int c = c0 + q;
            const long long r = r0 + threadIdx.x;
            if (r < R && c < C) out[(long long)c * R + r] = tile[threadIdx.x][q];
        }
        __syncthreads();
    }
}

int geo_grid(long long n);

// the three passes of the feature transform; the fastest-axis pass on the transposed
// features (featT: N ints of scratch)
static void ft_passes(const Dims& d, int* feat, int* featT, int* st_site, int* st_pos, long long* st_perp) {
    k_ft_pass<0><<<geo_grid(d.JK), 256>>>(d, feat, st_site, st_pos, st_perp);
    k_ft_pass<1><<<geo_grid((long long)d.I * d.K), 256>>>(d, feat, st_site, st_pos, st_perp);
    const long long R = (long long)d.I * d.J;
    const long long nbr = (R + 31) / 32;
    const dim3 blk(32, 8);
    const dim3 g1((unsigned)((d.K + 31) / 32), (unsigned)(nbr < 65535 ? nbr : 65535));
    k_ft_transpose<<<g1, blk>>>(feat, featT, R, d.K);  // [i J + j][k] -> [k][i J + j]
    k_ft_pass<2, true><<<geo_grid(R), 256>>>(d, featT, st_site, st_pos, st_perp);
    const long long nbr2 = ((long long)d.K + 31) / 32;
    const dim3 g2((unsigned)((R + 31) / 32), (unsigned)(nbr2 < 65535 ? nbr2 : 65535));
    k_ft_transpose<<<g2, blk>>>(featT, feat, d.K, (int)R);  // back
}

// sites of a float mask (> 0.5) for the distance transform
__global__ void k_ft_init_mask(Dims d, const float* __restrict__ sites, int* __restrict__ feat) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < d.N;
         r += (long long)gridDim.x * blockDim.x)
        feat[r] = sites[r] > 0.5f ? (int)r : -1;
}

// Euclidean distance to the nearest site (-1 when there is none)
__global__ void k_ft_distance(Dims d, const int* __restrict__ feat, float* __restrict__ dist) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < d.N;
         r += (long long)gridDim.x * blockDim.x) {
        const int f = feat[r];
        if (f < 0) {
            dist[r] = -1.f;
            continue;
        }
        int i, j, k, a, b, c;
        gdecode(d, r, i, j, k);
        gdecode(d, f, a, b, c);
        const double di = a - i, dj = b - j, dk = c - k;
        dist[r] = (float)sqrt(di * di + dj * dj + dk * dk);
    }
}

// one coordinate of numpy.linspace(s, p, num)[t] rounded half to even: the step is
// (p - s) / (num - 1), the point t * step + s (no fused multiply-add), the last point p
__device__ __forceinline__ int lin_point(int s, int p, long long t, long long num) {
    if (s == p) return s;
    if (t == num - 1) return p;
    const double step = __ddiv_rn((double)(p - s), (double)(num - 1));
    return (int)rint(__dadd_rn(__dmul_rn((double)t, step), (double)s));
}

// centre lines from each encapsulated Sulphide voxel to its nearest Pore voxel: ceil(dist) + 1
// points, the Rock voxels on them marked in frac
template <typename L>
__global__ void k_drill(Dims d, const L* __restrict__ lab, const uint8_t* __restrict__ enc,
                        const int* __restrict__ feat, uint8_t* __restrict__ frac) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < d.N;
         r += (long long)gridDim.x * blockDim.x) {
        if (!enc[r]) continue;
        const int f = feat[r];
        if (f < 0) continue;
        int si, sj, sk, pi, pj, pk;
        gdecode(d, r, si, sj, sk);
        gdecode(d, f, pi, pj, pk);
        const long long di = pi - si, dj = pj - sj, dk = pk - sk;
        const double dist = sqrt((double)(di * di + dj * dj + dk * dk));
        const long long num = (long long)ceil(dist) + 1;
        if (num <= 1) continue;
        for (long long t = 0; t < num; ++t) {
            const int i = lin_point(si, pi, t, num), j = lin_point(sj, pj, t, num), k = lin_point(sk, pk, t, num);
            const long long v = (long long)i * d.JK + (long long)j * d.K + k;
            if ((int)lab[v] == kRock) frac[v] = 1;
        }
    }
}

// Rock voxels within the 3x3x3 dilation of the fracture mask become Pore
template <typename L>
__global__ void k_widen(Dims d, const uint8_t* __restrict__ frac, L* __restrict__ lab,
                        unsigned long long* __restrict__ count) {
    unsigned long long n = 0;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < d.N;
         r += (long long)gridDim.x * blockDim.x) {
        if ((int)lab[r] != kRock) continue;
        int i, j, k;
        gdecode(d, r, i, j, k);
        bool hit = false;
        for (int a = -1; a <= 1 && !hit; ++a) {
            if (i + a < 0 || i + a >= d.I) continue;
            for (int b = -1; b <= 1 && !hit; ++b) {
                if (j + b < 0 || j + b >= d.J) continue;
                for (int c = -1; c <= 1; ++c) {
                    if (k + c < 0 || k + c >= d.K) continue;
                    if (frac[r + a * d.JK + b * d.K + c]) { hit = true; break; }
                }
            }
        }
        if (hit) {
            lab[r] = (L)kPore;
            ++n;
        }
    }
    if (n) atomicAdd(count, n);
}

// device buffers released on every return path
struct Scratch {
    void* p[16];
    int n = 0;
    ~Scratch() {
        for (int q = 0; q < n; ++q) cudaFree(p[q]);
    }
    template <typename T>
    bool get(T** out, size_t count) {
        void* v = nullptr;
        if (n >= 16 || cudaMalloc(&v, count * sizeof(T) + 16) != cudaSuccess) return false;
        p[n++] = v;
        *out = (T*)v;
        return true;
    }
};

int geo_grid(long long n) {
    long long b = (n + 255) / 256;
    if (b > 152LL * 16) b = 152LL * 16;
    if (b < 1) b = 1;
    return (int)b;
}

#define GEO_CHECK(expr)                                      \
    do {                                                     \
        if ((expr) != cudaSuccess) return LS_CUDA_ERROR;     \
    } while (0)
#define GEO_LAUNCH()                                         \
    do {                                                     \
        if (cudaGetLastError() != cudaSuccess) return LS_CUDA_ERROR; \
    } while (0)

bool dims_ok(int I, int J, int K) {
    if (I < 1 || J < 1 || K < 1) return false;
    const long long N = (long long)I * J * K;
    return N < (1LL << 31) - 1;
}

// the 6-connected components of mask m into parent (-1 outside the mask)
ls_status components(const Dims& d, const uint8_t* m, int* parent, int* err, int grid) {
    GEO_CHECK(cudaMemset(err, 0, sizeof(int)));
    k_uf_init<<<grid, 256>>>(d, m, parent);
    GEO_LAUNCH();
    k_uf_hook<<<grid, 256>>>(d, m, parent, err);
    GEO_LAUNCH();
    k_uf_compress<<<grid, 256>>>(d, parent);
    GEO_LAUNCH();
    int h_err = 0;
    GEO_CHECK(cudaMemcpy(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost));
    return h_err ? LS_TIMEOUT : LS_OK;
}

template <typename L>
ls_status clean_t(int I, int J, int K, void* labels_host, int mode, long long* changed) {
    Dims d{I, J, K, (long long)J * K, (long long)I * J * K};
    const int grid = geo_grid(d.N);
    Scratch s;
    L* lab;
    uint8_t *pore, *er, *opened, *air, *amb, *env, *valid;
    int *pp, *pa, *err;
    unsigned int* count;
    unsigned long long *best, *nchg;
    if (!s.get(&lab, d.N) || !s.get(&pore, d.N) || !s.get(&er, d.N) || !s.get(&opened, d.N) ||
        !s.get(&air, d.N) || !s.get(&amb, d.N) || !s.get(&env, d.N) || !s.get(&valid, d.N) ||
        !s.get(&pp, d.N) || !s.get(&pa, d.N) || !s.get(&err, 1) || !s.get(&count, d.N) || !s.get(&best, 1) ||
        !s.get(&nchg, 1))
        return LS_CUDA_ERROR;
    GEO_CHECK(cudaMemcpy(lab, labels_host, sizeof(L) * d.N, cudaMemcpyHostToDevice));
    // opening of the pore mask, then its components
    k_mask_eq<L><<<grid, 256>>>(d, lab, kPore, pore);
    GEO_LAUNCH();
    k_morph6<true><<<grid, 256>>>(d, pore, er);
    GEO_LAUNCH();
    k_morph6<false><<<grid, 256>>>(d, er, opened);
    GEO_LAUNCH();
    LS_TRY(components(d, opened, pp, err, grid));
    GEO_CHECK(cudaMemset(valid, 0, d.N));
    if (mode == 0) {
        // the ambient Air: the largest Air component (none: every non-Air voxel)
        k_mask_eq<L><<<grid, 256>>>(d, lab, kAir, air);
        GEO_LAUNCH();
        LS_TRY(components(d, air, pa, err, grid));
        GEO_CHECK(cudaMemset(count, 0, sizeof(unsigned int) * d.N));
        GEO_CHECK(cudaMemset(best, 0, sizeof(unsigned long long)));
        k_uf_count<<<grid, 256>>>(d, pa, count);
        GEO_LAUNCH();
        k_uf_largest<<<grid, 256>>>(d, pa, count, best);
        GEO_LAUNCH();
        unsigned long long h_best = 0;
        GEO_CHECK(cudaMemcpy(&h_best, best, sizeof(h_best), cudaMemcpyDeviceToHost));
        const int root = (h_best >> 32) ? (int)(0xffffffffu - (unsigned int)(h_best & 0xffffffffu)) : -1;
        k_comp_mask<<<grid, 256>>>(d, pa, root, amb);
        GEO_LAUNCH();
        k_morph6<false><<<grid, 256>>>(d, amb, env);
        GEO_LAUNCH();
        k_mark_valid<<<grid, 256>>>(d, pp, env, valid);
    } else {
        k_mark_valid<<<grid, 256>>>(d, pp, nullptr, valid);
    }
    GEO_LAUNCH();
    GEO_CHECK(cudaMemset(nchg, 0, sizeof(unsigned long long)));
    k_clean_apply<L><<<grid, 256>>>(d, pp, valid, lab, nchg);
    GEO_LAUNCH();
    GEO_CHECK(cudaMemcpy(labels_host, lab, sizeof(L) * d.N, cudaMemcpyDeviceToHost));
    unsigned long long h_n = 0;
    GEO_CHECK(cudaMemcpy(&h_n, nchg, sizeof(h_n), cudaMemcpyDeviceToHost));
    if (changed) *changed = (long long)h_n;
    return LS_OK;
}

template <typename L>
ls_status fracture_t(int I, int J, int K, void* labels_host, long long* drilled, long long* encapsulated) {
    Dims d{I, J, K, (long long)J * K, (long long)I * J * K};
    const int grid = geo_grid(d.N);
    Scratch s;
    L* lab;
    uint8_t *enc, *frac;
    int *feat, *featT, *st_site, *st_pos;
    long long* st_perp;
    unsigned long long* counts;
    if (!s.get(&lab, d.N) || !s.get(&enc, d.N) || !s.get(&frac, d.N) || !s.get(&feat, d.N) ||
        !s.get(&featT, d.N) || !s.get(&st_site, d.N) || !s.get(&st_pos, d.N) || !s.get(&st_perp, d.N) ||
        !s.get(&counts, 3))
        return LS_CUDA_ERROR;
    GEO_CHECK(cudaMemcpy(lab, labels_host, sizeof(L) * d.N, cudaMemcpyHostToDevice));
    GEO_CHECK(cudaMemset(counts, 0, 3 * sizeof(unsigned long long)));
    k_encapsulated<L><<<grid, 256>>>(d, lab, enc, counts);
    GEO_LAUNCH();
    unsigned long long h[2] = {0, 0};
    GEO_CHECK(cudaMemcpy(h, counts, sizeof(h), cudaMemcpyDeviceToHost));
    if (encapsulated) *encapsulated = (long long)h[0];
    if (drilled) *drilled = 0;
    if (h[1] == 0) return LS_BAD_ARG;  // no Pore voxel: nothing to drill towards
    if (h[0] == 0) return LS_OK;       // every Sulphide voxel is exposed already
    k_ft_init<L><<<grid, 256>>>(d, lab, feat);
    GEO_LAUNCH();
    ft_passes(d, feat, featT, st_site, st_pos, st_perp);
    GEO_LAUNCH();
    GEO_CHECK(cudaMemset(frac, 0, d.N));
    k_drill<L><<<grid, 256>>>(d, lab, enc, feat, frac);
    GEO_LAUNCH();
    k_widen<L><<<grid, 256>>>(d, frac, lab, counts + 2);
    GEO_LAUNCH();
    GEO_CHECK(cudaMemcpy(labels_host, lab, sizeof(L) * d.N, cudaMemcpyDeviceToHost));
    unsigned long long h_n = 0;
    GEO_CHECK(cudaMemcpy(&h_n, counts + 2, sizeof(h_n), cudaMemcpyDeviceToHost));
    if (drilled) *drilled = (long long)h_n;
    return LS_OK;
}

template <typename L>
ls_status coarsen_t(int I, int J, int K, const void* in_host, void* out_host) {
    Dims din{I, J, K, (long long)J * K, (long long)I * J * K};
    const int oI = (I + 1) / 2, oJ = J / 2, oK = K / 2;
    Dims dout{oI, oJ, oK, (long long)oJ * oK, (long long)oI * oJ * oK};
    Scratch s;
    L *src, *dst;
    if (!s.get(&src, din.N) || !s.get(&dst, dout.N)) return LS_CUDA_ERROR;
    GEO_CHECK(cudaMemcpy(src, in_host, sizeof(L) * din.N, cudaMemcpyHostToDevice));
    k_coarsen<L><<<geo_grid(dout.N), 256>>>(din, dout, src, dst);
    GEO_LAUNCH();
    GEO_CHECK(cudaMemcpy(out_host, dst, sizeof(L) * dout.N, cudaMemcpyDeviceToHost));
    return LS_OK;
}

template <typename L>
ls_status classify_t(int I, int J, int K, const uint16_t* grey_host, int nt, const uint16_t* thr_host,
                     const int* labels_host, void* out_host) {
    Dims d{I, J, K, (long long)J * K, (long long)I * J * K};
    Scratch s;
    uint16_t *grey, *thr;
    int* labs;
    L* out;
    if (!s.get(&grey, d.N) || !s.get(&thr, 16) || !s.get(&labs, 17) || !s.get(&out, d.N)) return LS_CUDA_ERROR;
    GEO_CHECK(cudaMemcpy(grey, grey_host, sizeof(uint16_t) * d.N, cudaMemcpyHostToDevice));
    if (nt) GEO_CHECK(cudaMemcpy(thr, thr_host, sizeof(uint16_t) * nt, cudaMemcpyHostToDevice));
    GEO_CHECK(cudaMemcpy(labs, labels_host, sizeof(int) * (nt + 1), cudaMemcpyHostToDevice));
    k_classify<L><<<geo_grid(d.N), 256>>>(d, grey, nt, thr, labs, out);
    GEO_LAUNCH();
    GEO_CHECK(cudaMemcpy(out_host, out, sizeof(L) * d.N, cudaMemcpyDeviceToHost));
    return LS_OK;
}

}  // namespace
}  // namespace ls

extern "C" ls_status ls_geom_coarsen(int I, int J, int K, int label_bytes, const void* in_host, void* out_host) {
    if (!in_host || !out_host || !ls::dims_ok(I, J, K) || J % 2 || K % 2) return LS_BAD_ARG;
    if (label_bytes == 1) return ls::coarsen_t<uint8_t>(I, J, K, in_host, out_host);
    if (label_bytes == 2) return ls::coarsen_t<uint16_t>(I, J, K, in_host, out_host);
    return LS_BAD_ARG;
}

extern "C" ls_status ls_geom_clean(int I, int J, int K, int label_bytes, void* labels_host, int mode,
                                   long long* changed) {
    if (!labels_host || !ls::dims_ok(I, J, K) || (mode != 0 && mode != 1)) return LS_BAD_ARG;
    if (label_bytes == 1) return ls::clean_t<uint8_t>(I, J, K, labels_host, mode, changed);
    if (label_bytes == 2) return ls::clean_t<uint16_t>(I, J, K, labels_host, mode, changed);
    return LS_BAD_ARG;
}

extern "C" ls_status ls_geom_fracture(int I, int J, int K, int label_bytes, void* labels_host, long long* drilled,
                                      long long* encapsulated) {
    if (!labels_host || !ls::dims_ok(I, J, K)) return LS_BAD_ARG;
    if (label_bytes == 1) return ls::fracture_t<uint8_t>(I, J, K, labels_host, drilled, encapsulated);
    if (label_bytes == 2) return ls::fracture_t<uint16_t>(I, J, K, labels_host, drilled, encapsulated);
    return LS_BAD_ARG;
}

extern "C" ls_status ls_geom_distance(int I, int J, int K, const float* sites, float* dist) {
    if (!sites || !dist || !ls::dims_ok(I, J, K)) return LS_BAD_ARG;
    ls::Dims d{I, J, K, (long long)J * K, (long long)I * J * K};
    ls::Scratch s;
    int *feat, *featT, *st_site, *st_pos;
    long long* st_perp;
    if (!s.get(&feat, d.N) || !s.get(&featT, d.N) || !s.get(&st_site, d.N) || !s.get(&st_pos, d.N) ||
        !s.get(&st_perp, d.N))
        return LS_CUDA_ERROR;
    const int grid = ls::geo_grid(d.N);
    ls::k_ft_init_mask<<<grid, 256>>>(d, sites, feat);
    GEO_LAUNCH();
    ls::ft_passes(d, feat, featT, st_site, st_pos, st_perp);
    GEO_LAUNCH();
    ls::k_ft_distance<<<grid, 256>>>(d, feat, dist);
    GEO_LAUNCH();
    GEO_CHECK(cudaDeviceSynchronize());
    return LS_OK;
}

extern "C" ls_status ls_geom_classify(int I, int J, int K, const uint16_t* grey_host, int n_thresholds,
                                      const uint16_t* thresholds, const int* labels, int label_bytes,
                                      void* out_host) {
    if (!grey_host || !labels || !out_host || !ls::dims_ok(I, J, K) || n_thresholds < 0 || n_thresholds > 16 ||
        (n_thresholds > 0 && !thresholds))
        return LS_BAD_ARG;
    for (int q = 1; q < n_thresholds; ++q)
        if (thresholds[q] < thresholds[q - 1]) return LS_BAD_ARG;
    if (label_bytes == 1) return ls::classify_t<uint8_t>(I, J, K, grey_host, n_thresholds, thresholds, labels, out_host);
    if (label_bytes == 2) return ls::classify_t<uint16_t>(I, J, K, grey_host, n_thresholds, thresholds, labels, out_host);
    return LS_BAD_ARG;
}
