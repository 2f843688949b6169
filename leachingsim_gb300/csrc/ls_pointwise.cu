// ls_pointwise.cu - per-voxel and nearest-neighbour kernels of the time step:
//   props  = updateRelativePermeability + updateCapillaryPressure + initProperties,
//            fused (src/Simulation.cpp:1634-1664, 1596-1628, 187-248)
//   flux   = calculateFlux (src/Simulation.cpp:866-953)
//   saturation = updateSaturation (src/Simulation.cpp:1672-1856)
//   surface = handleSurfaceEffects (src/Simulation.cpp:2063-2103)
//   precip  = handlePrecipitation (src/Simulation.cpp:2114-2165)
// Arithmetic follows the reference expression by expression; the library is built
// without FMA contraction so each product rounds on its own, as on the reference's host.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>

#include "ls_internal.cuh"

namespace ls {

struct PropsConst {
    double m, s_res, vg_n, vg_alpha, inv_alpha;
    double pore_permeability, rock_permeability;  // src/Simulation.cpp:190-191 (parameters here)
    double log_k_rock, log_k_pore;
    double k_clean_pore;     // pow(10, 0*log_k_rock + 1*log_k_pore), precipitate fraction 0
    double k_clogged_pore;   // pow(10, 1*log_k_rock + 0*log_k_pore), precipitate fraction 1
    int vg_n_is_2;           // m = 1/2: Se^(1/m) = Se*Se, (.)^m = sqrt, Se^(-1/m) = 1/(Se*Se)
};

// updateRelativePermeability / updateCapillaryPressure / initProperties for one voxel from
// its label t, saturation s, precipitate fraction, mineral fraction and intrinsic-permeability
// multiplier km (1 where none is set: K * 1 is K exactly).
__device__ __forceinline__ void props_eval(const PropsConst& pc, int t, double s, double precip_v,
                                           float ff, float km, double& krv, double& pcv, double& permv,
                                           double& viscv) {
    const double pore_permeability = pc.pore_permeability;
    const double rock_permeability = pc.rock_permeability;
    krv = 0.0;
    pcv = 0.0;
    if (t == kPore || t == kSulphide) {
        // relative permeability, src/Simulation.cpp:1643-1657
        double Se = (s - pc.s_res) / (1.0 - pc.s_res);
        double Sk = smax(0.0, smin(1.0, Se));
        if (Sk <= 0.0) {
            krv = 0.0;
        } else {
            double term1 = pc.vg_n_is_2 ? 1.0 - sqrt(1.0 - Sk * Sk)
                                        : 1.0 - pow(1.0 - pow(Sk, 1.0 / pc.m), pc.m);
            krv = sqrt(Sk) * term1 * term1;
        }
        // capillary pressure, src/Simulation.cpp:1605-1621
        double Sc = smax(1e-6, smin(1.0, Se));
        if (Sc >= 1.0) {
            pcv = 0.0;
        } else if (pc.vg_n_is_2) {
            pcv = pc.inv_alpha * sqrt(1.0 / (Sc * Sc) - 1.0);
        } else {
            double Se_inv_m = pow(Sc, -1.0 / pc.m);
            pcv = pc.inv_alpha * pow(Se_inv_m - 1.0, 1.0 / pc.vg_n);
        }
    }
    // intrinsic permeability and viscosity, src/Simulation.cpp:199-244
    double K_intrinsic = rock_permeability;
    if (t == kAir) {
        K_intrinsic = pore_permeability;
    } else if (t == kPore) {
        double p_frac = smax(0.0, smin(1.0, precip_v));
        if (p_frac == 0.0) K_intrinsic = pc.k_clean_pore;
        else if (p_frac == 1.0) K_intrinsic = pc.k_clogged_pore;
        else K_intrinsic = pow(10.0, (p_frac * pc.log_k_rock) + ((1.0 - p_frac) * pc.log_k_pore));
    } else if (t == kSulphide) {
        if (ff == 1.0f) K_intrinsic = pc.k_clogged_pore;
        else if (ff == 0.0f) K_intrinsic = pc.k_clean_pore;
        else {
            const double f = (double)ff;
            K_intrinsic = pow(10.0, (f * pc.log_k_rock) + ((1.0 - f) * pc.log_k_pore));
        }
    }
    if (km != 1.0f) K_intrinsic = K_intrinsic * (double)km;
    viscv = (t == kAir) ? 1.8e-5 : 1.0e-3;
    permv = K_intrinsic * smax(krv, 1e-15);
}

// Pass 1: voxels whose label, s, precip or frac differ bitwise from their values at the last
// evaluation (all voxels when forced) go to the work list, with their new inputs recorded;
// the others keep their properties, which are a pure function of those inputs.
template <typename L>
__global__ void __launch_bounds__(kBlock) k_props_scan(Grid g, const L* __restrict__ label,
                                                       const double* __restrict__ sat,
                                                       const double* __restrict__ precip,
                                                       const float* __restrict__ frac, L* __restrict__ sl,
                                                       double* __restrict__ ss, double* __restrict__ sp,
                                                       float* __restrict__ sf, int force,
                                                       int* __restrict__ list, unsigned int* __restrict__ count) {
    // block-uniform trip count (block_append is called by every thread of the block)
    for (int b0 = blockIdx.x * blockDim.x; b0 < (int)g.N; b0 += gridDim.x * blockDim.x) {
        const int r = b0 + (int)threadIdx.x;
        bool d = false;
        if (r < (int)g.N) {
            const L lab = label[r];
            const long long sb = __double_as_longlong(sat[r]);
            const long long pb = __double_as_longlong(precip[r]);
            const unsigned int fb = __float_as_uint(frac[r]);
            d = force || lab != sl[r] || sb != __double_as_longlong(ss[r]) || pb != __double_as_longlong(sp[r]) ||
                fb != __float_as_uint(sf[r]);
            if (d) {
                sl[r] = lab;
                ss[r] = __longlong_as_double(sb);
                sp[r] = __longlong_as_double(pb);
                sf[r] = __uint_as_float(fb);
            }
        }
        block_append(d, r, list, count);
    }
}

// Pass 2: the properties of the listed voxels (dense: every lane has work).
template <typename L>
__global__ void __launch_bounds__(kBlock) k_props(PropsConst pc, const L* __restrict__ label,
                                                  const double* __restrict__ sat,
                                                  const double* __restrict__ precip,
                                                  const float* __restrict__ frac,
                                                  const float* __restrict__ kmult,
                                                  double* __restrict__ kr, double* __restrict__ cap,
                                                  double* __restrict__ perm, double* __restrict__ visc,
                                                  const int* __restrict__ list,
                                                  const unsigned int* __restrict__ count) {
    const int n = (int)*count;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int r = list[q];
        double krv, pcv, pv, vv;
        props_eval(pc, (int)label[r], sat[r], precip[r], frac[r], kmult ? kmult[r] : 1.0f, krv, pcv, pv, vv);
        kr[r] = krv;
        cap[r] = pcv;
        perm[r] = pv;
        visc[r] = vv;
    }
}

ls_status props_run(ls_ctx* c) {
    snap_fence(c, kSnapProps);
    PropsConst pc;
    pc.m = 1.0 - (1.0 / c->p.vg_n);
    pc.s_res = c->p.s_res;
    pc.vg_n = c->p.vg_n;
    pc.vg_alpha = c->p.vg_alpha;
    pc.inv_alpha = 1.0 / c->p.vg_alpha;
    pc.pore_permeability = c->p.pore_permeability;
    pc.rock_permeability = c->p.rock_permeability;
    pc.log_k_rock = std::log10(pc.rock_permeability);
    pc.log_k_pore = std::log10(pc.pore_permeability);
    pc.k_clean_pore = std::pow(10.0, (0.0 * pc.log_k_rock) + ((1.0 - 0.0) * pc.log_k_pore));
    pc.k_clogged_pore = std::pow(10.0, (1.0 * pc.log_k_rock) + ((1.0 - 1.0) * pc.log_k_pore));
    pc.vg_n_is_2 = (c->p.vg_n == 2.0) ? 1 : 0;
    const size_t n = (size_t)c->g.N;
    int grid = grid_for(c, c->g.N);
    if (c->lean) {
        // no change tracking: every voxel
        c->props_force = 0;
        LS_TRY(wlist_all(c));
        if (c->label_bytes == 1)
            LS_LAUNCH(c, k_props<uint8_t>, grid, kBlock, 0, pc, (const uint8_t*)c->label, c->sat, c->precip,
                      c->frac, (const float*)c->kmult, c->kr, c->pc, c->perm, c->visc, (const int*)c->wlist,
                      (const unsigned int*)c->wcount);
        else
            LS_LAUNCH(c, k_props<uint16_t>, grid, kBlock, 0, pc, (const uint16_t*)c->label, c->sat, c->precip,
                      c->frac, (const float*)c->kmult, c->kr, c->pc, c->perm, c->visc, (const int*)c->wlist,
                      (const unsigned int*)c->wcount);
        c->p_ready = 0;
        return LS_OK;
    }
    if (!c->sh_sat) {
        LS_TRY(dalloc(c, &c->sh_label, n * c->label_bytes));
        LS_TRY(dalloc_t(c, &c->sh_sat, n));
        LS_TRY(dalloc_t(c, &c->sh_precip, n));
        LS_TRY(dalloc_t(c, &c->sh_frac, n));
        c->props_force = 1;
    }
    const int force = c->props_force;
    c->props_force = 0;
    LS_TRY(wlist_reset(c));
    if (c->label_bytes == 1) {
        LS_LAUNCH(c, k_props_scan<uint8_t>, grid, kBlock, 0, c->g, (const uint8_t*)c->label, c->sat, c->precip,
                  c->frac, (uint8_t*)c->sh_label, c->sh_sat, c->sh_precip, c->sh_frac, force, c->wlist, c->wcount);
        LS_LAUNCH(c, k_props<uint8_t>, grid, kBlock, 0, pc, (const uint8_t*)c->label, c->sat, c->precip,
                  c->frac, (const float*)c->kmult, c->kr, c->pc, c->perm, c->visc, (const int*)c->wlist,
                  (const unsigned int*)c->wcount);
    } else {
        LS_LAUNCH(c, k_props_scan<uint16_t>, grid, kBlock, 0, c->g, (const uint16_t*)c->label, c->sat, c->precip,
                  c->frac, (uint16_t*)c->sh_label, c->sh_sat, c->sh_precip, c->sh_frac, force, c->wlist,
                  c->wcount);
        LS_LAUNCH(c, k_props<uint16_t>, grid, kBlock, 0, pc, (const uint16_t*)c->label, c->sat, c->precip,
                  c->frac, (const float*)c->kmult, c->kr, c->pc, c->perm, c->visc, (const int*)c->wlist,
                  (const unsigned int*)c->wcount);
    }
    c->p_ready = 0;
    return LS_OK;
}

// ---------------------------------------------------------------------------
// calculateFlux: central differences inside, one-sided on the domain faces (np=1).

__device__ __forceinline__ double grad1(const double* __restrict__ f, long long r, long long off,
                                        int pos, int ext, const DxDiv& dd) {
    if (pos == 0) return dd.div(f[r + off] - f[r]);
    if (pos == ext - 1) return dd.div(f[r] - f[r - off]);
    // (a - b) / (2 dx): with dx a power of two this is (a - b) * (0.5 / dx) exactly
    double d = f[r + off] - f[r - off];
    return dd.pow2 ? d * (0.5 * dd.inv_dx) : d / (2.0 * dd.dx);
}

// Change test of the flux inputs (pass 1), against the values at the last flux evaluation:
// plane 0 bit = P or Pc of the voxel changed (they enter its neighbours' gradients too),
// plane 1 bit = its permeability or viscosity changed.
__global__ void __launch_bounds__(kBlock) k_flux_dirty(Grid g, const double* __restrict__ P,
                                                       const double* __restrict__ C,
                                                       const double* __restrict__ perm,
                                                       const double* __restrict__ visc,
                                                       double* __restrict__ sP, double* __restrict__ sC,
                                                       double* __restrict__ sK, double* __restrict__ sV,
                                                       unsigned int* __restrict__ bits, long long nw, int force) {
    for (long long r0 = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); r0 < g.N;
         r0 += (long long)gridDim.x * blockDim.x) {
        const long long r = r0 + (threadIdx.x & 31u);
        bool d0 = false, d1 = false;
        if (r < g.N) {
            const long long pb = __double_as_longlong(P[r]), cb = __double_as_longlong(C[r]);
            const long long kb = __double_as_longlong(perm[r]), vb = __double_as_longlong(visc[r]);
            d0 = force || pb != __double_as_longlong(sP[r]) || cb != __double_as_longlong(sC[r]);
            d1 = force || kb != __double_as_longlong(sK[r]) || vb != __double_as_longlong(sV[r]);
            if (d0) {
                sP[r] = __longlong_as_double(pb);
                sC[r] = __longlong_as_double(cb);
            }
            if (d1) {
                sK[r] = __longlong_as_double(kb);
                sV[r] = __longlong_as_double(vb);
            }
        }
        const unsigned int w0 = __ballot_sync(0xffffffffu, d0);
        const unsigned int w1 = __ballot_sync(0xffffffffu, d1);
        if ((threadIdx.x & 31u) == 0u) {
            bits[r0 >> 5] = w0;
            bits[nw + (r0 >> 5)] = w1;
        }
    }
}

// Pass 2: the flux of a voxel is a pure function of P and Pc at the voxel and its six
// neighbours and of its own permeability and viscosity. Voxels where one of those changed go
// to the work list; the others get their last computed flux back (the transport solve zeroes
// the flux of Rock and Precipitate voxels after use).
__global__ void __launch_bounds__(kBlock) k_flux_scan(Grid g, const unsigned int* __restrict__ bits, long long nw,
                                                      double* __restrict__ fx, double* __restrict__ fy,
                                                      double* __restrict__ fz, const double* __restrict__ sfx,
                                                      const double* __restrict__ sfy,
                                                      const double* __restrict__ sfz, int* __restrict__ list,
                                                      unsigned int* __restrict__ count) {
    const int lane = (int)(threadIdx.x & 31u);
    // block-uniform trip count (block_append is called by every thread of the block)
    for (long long b0 = (long long)blockIdx.x * blockDim.x; b0 < g.N; b0 += (long long)gridDim.x * blockDim.x) {
        const long long r0 = b0 + (threadIdx.x & ~31u);
        const long long r = r0 + lane;
        const unsigned int own = dwin(bits, nw, r0) | dwin(bits + nw, nw, r0);
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
            if (!d && sfx) {  // null: the fluxes already equal the shadows
                fx[r] = sfx[r];
                fy[r] = sfy[r];
                fz[r] = sfz[r];
            }
        }
        block_append(d, (int)r, list, count);
    }
}

// Pass 3: calculateFlux at the listed voxels.
__global__ void __launch_bounds__(kBlock) k_flux(Grid g, DxDiv dd, double mcg, const double* __restrict__ P,
                                                 const double* __restrict__ C, const double* __restrict__ perm,
                                                 const double* __restrict__ visc, double* __restrict__ fx,
                                                 double* __restrict__ fy, double* __restrict__ fz,
                                                 double* __restrict__ sfx, double* __restrict__ sfy,
                                                 double* __restrict__ sfz, const int* __restrict__ list,
                                                 const unsigned int* __restrict__ count) {
    const int n = (int)*count;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int r = list[q];
        int i, j, k;
        decode(g, r, i, j, k);
        double gPx = grad1(P, r, g.JK, i, g.I, dd);
        double gPy = grad1(P, r, g.K, j, g.J, dd);
        double gPz = grad1(P, r, 1, k, g.K, dd);
        double gCx = grad1(C, r, g.JK, i, g.I, dd);
        double gCy = grad1(C, r, g.K, j, g.J, dd);
        double gCz = grad1(C, r, 1, k, g.K, dd);
        gCx = smax(-mcg, smin(mcg, gCx));
        gCy = smax(-mcg, smin(mcg, gCy));
        gCz = smax(-mcg, smin(mcg, gCz));
        double transmissivity = perm[r] / visc[r];
        const double rho_g = 1000.0 * 9.81;
        const double qx = -transmissivity * ((gPx - gCx) - rho_g);
        const double qy = -transmissivity * (gPy - gCy);
        const double qz = -transmissivity * (gPz - gCz);
        fx[r] = qx; fy[r] = qy; fz[r] = qz;
        if (sfx) {  // null: no change tracking
            sfx[r] = qx; sfy[r] = qy; sfz[r] = qz;
        }
    }
}

ls_status flux_run(ls_ctx* c) {
    snap_fence(c, kSnapFlux);
    int grid = grid_for(c, c->g.N);
    const size_t n = (size_t)c->g.N;
    if (c->lean) {
        // no change tracking: every voxel, no shadow copies
        LS_TRY(wlist_all(c));
        LS_LAUNCH(c, k_flux, grid, kBlock, 0, c->g, make_dxdiv(c->p.dx), c->p.max_cap_grad, c->P, c->pc,
                  c->perm, c->visc, c->fx, c->fy, c->fz, (double*)nullptr, (double*)nullptr, (double*)nullptr,
                  (const int*)c->wlist, (const unsigned int*)c->wcount);
        c->flux_zero_pending = 0;  // every voxel written
        return LS_OK;
    }
    if (!c->shq_P) {
        double** arrs[] = {&c->shq_P, &c->shq_C, &c->shq_K, &c->shq_V, &c->shq_fx, &c->shq_fy, &c->shq_fz};
        for (double** q : arrs) LS_TRY(dalloc_t(c, q, n));
        c->flux_valid = 0;
    }
    const int force = (!c->flux_valid || c->flux_consts[0] != c->p.dx ||
                       c->flux_consts[1] != c->p.max_cap_grad) ? 1 : 0;
    LS_TRY(wlist_reset(c));
    LS_LAUNCH(c, k_flux_dirty, grid, kBlock, 0, c->g, c->P, c->pc, c->perm, c->visc, c->shq_P, c->shq_C,
              c->shq_K, c->shq_V, c->dbits, c->dwords, force);
    // unchanged voxels get their last computed flux back, unless the fluxes still hold it
    const bool restore = !c->fx_is_shadow || force;
    LS_LAUNCH(c, k_flux_scan, grid, kBlock, 0, c->g, (const unsigned int*)c->dbits, c->dwords, c->fx, c->fy, c->fz,
              restore ? (const double*)c->shq_fx : (const double*)nullptr,
              restore ? (const double*)c->shq_fy : (const double*)nullptr,
              restore ? (const double*)c->shq_fz : (const double*)nullptr, c->wlist, c->wcount);
    LS_LAUNCH(c, k_flux, grid, kBlock, 0, c->g, make_dxdiv(c->p.dx), c->p.max_cap_grad, c->P, c->pc,
              c->perm, c->visc, c->fx, c->fy, c->fz, c->shq_fx, c->shq_fy, c->shq_fz, (const int*)c->wlist,
              (const unsigned int*)c->wcount);
    c->flux_consts[0] = c->p.dx;
    c->flux_consts[1] = c->p.max_cap_grad;
    c->flux_valid = 1;
    c->flux_zero_pending = 0;  // every voxel holds its fresh flux, equal to its shadow
    c->fx_is_shadow = 1;
    return LS_OK;
}

// ---------------------------------------------------------------------------
// updateSaturation. div q and the evaporative sink of a voxel read only flux and labels,
// which do not change between sub-steps, so the reference's num_steps full sweeps equal
// num_steps repetitions of s <- clamp(s - dt_sub/phi*(div q + evap)) per voxel; the
// repetition stops early once s reaches a fixed point of that map (every later sweep
// would reproduce it bit for bit).

__device__ __forceinline__ bool sat_inactive(int t) {
    return t == kAir || t == kRock || t == kSulphide || t == kPrecipitate;
}

template <typename L>
__device__ __forceinline__ void sat_rates(const Grid& g, const L* __restrict__ label,
                                          const double* __restrict__ fx,
                                          const double* __restrict__ fy,
                                          const double* __restrict__ fz, long long r, int i,
                                          int j, int k, int t, const DxDiv& dd, double evap,
                                          double& div_q, double& evap_sink) {
    // (a + b) / 2.0 == (a + b) * 0.5 exactly
    const double fxr = fx[r], fyr = fy[r], fzr = fz[r];
    double q_xp = (i + 1 < g.I) ? (fxr + fx[r + g.JK]) * 0.5 : 0.0;
    double q_xm = (i > 0) ? (fxr + fx[r - g.JK]) * 0.5 : 0.0;
    double q_yp = (j + 1 < g.J) ? (fyr + fy[r + g.K]) * 0.5 : 0.0;
    double q_ym = (j > 0) ? (fyr + fy[r - g.K]) * 0.5 : 0.0;
    double q_zp = (k + 1 < g.K) ? (fzr + fz[r + 1]) * 0.5 : 0.0;
    double q_zm = (k > 0) ? (fzr + fz[r - 1]) * 0.5 : 0.0;
    div_q = dd.div((q_xp - q_xm) + (q_yp - q_ym) + (q_zp - q_zm));
    evap_sink = 0.0;
    if (t == kPore) {
        int air_faces = 0;
        if (i + 1 < g.I && (int)label[r + g.JK] == kAir) air_faces++;
        if (i > 0 && (int)label[r - g.JK] == kAir) air_faces++;
        if (j + 1 < g.J && (int)label[r + g.K] == kAir) air_faces++;
        if (j > 0 && (int)label[r - g.K] == kAir) air_faces++;
        if (k + 1 < g.K && (int)label[r + 1] == kAir) air_faces++;
        if (k > 0 && (int)label[r - 1] == kAir) air_faces++;
        // with evap = +0 the sink is air_faces * +0 = +0
        evap_sink = (__double_as_longlong(evap) == 0) ? 0.0 : dd.div(air_faces * evap);
    }
}

template <typename L>
__global__ void __launch_bounds__(kBlock) k_sat_update(Grid g, DxDiv dd, double evap,
                                                       double dt_sub_over_phi, int num_steps,
                                                       const L* __restrict__ label,
                                                       const double* __restrict__ fx,
                                                       const double* __restrict__ fy,
                                                       const double* __restrict__ fz,
                                                       double* __restrict__ sat) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.NP;
         r += (long long)gridDim.x * blockDim.x) {
        if (r >= g.N) {  // extra top plane of the freshly allocated array
            sat[r] = 0.0;
            continue;
        }
        int t = (int)label[r];
        if (sat_inactive(t)) {
            sat[r] = 0.0;  // never written by the reference's update (indeterminate there)
            continue;
        }
        int i, j, k;
        decode(g, r, i, j, k);
        double div_q, evap_sink;
        sat_rates(g, label, fx, fy, fz, r, i, j, k, t, dd, evap, div_q, evap_sink);
        double sv = sat[r];
        for (int step = 0; step < num_steps; ++step) {
            double new_sat = sv - dt_sub_over_phi * (div_q + evap_sink);
            double nv = smax(0.0, smin(1.0, new_sat));
            bool fixed = (nv == sv) || (nv != nv && sv != sv);
            sv = nv;
            if (fixed) break;
        }
        sat[r] = sv;
    }
}

// The context path of the update: the rate pass stores div q + evaporative sink of every
// active voxel (the update applies that same sum in every sub-step), so the update pass does
// no flux arithmetic. The rate pass runs over the list of the active (Pore) voxels: warps
// of active voxels only. div q in fewer FP64 operations, with the same value: the six face
// means are (f + f_nb) * 0.5 and every sum and difference of them is exact up to rounding
// that commutes with the exact halving (no result is subnormal: fluxes are far above
// 2^-1022), so ((A+ - A-) + (B+ - B-)) + (C+ - C-), halved once, equals the sum of the halved
// differences bit for bit; with dx a power of two the halving and 1/dx are one exact scaling.
template <typename L>
__global__ void __launch_bounds__(kBlock) k_sat_rate_list(Grid g, DxDiv dd, double evap,
                                                          const L* __restrict__ label,
                                                          const double* __restrict__ fx,
                                                          const double* __restrict__ fy,
                                                          const double* __restrict__ fz,
                                                          const int* __restrict__ list,
                                                          const unsigned int* __restrict__ count,
                                                          double* __restrict__ qsum,
                                                          double* __restrict__ partials) {
    double v[1] = {0.0};
    const long long n = (long long)*count;
    const double half_scale = dd.pow2 ? 0.5 * dd.inv_dx : 0.5;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const long long r = list[q];
        const int t = (int)label[r];
        int i, j, k;
        decode(g, r, i, j, k);
        const double fxr = fx[r], fyr = fy[r], fzr = fz[r];
        const double ap = (i + 1 < g.I) ? fxr + fx[r + g.JK] : 0.0;
        const double am = (i > 0) ? fxr + fx[r - g.JK] : 0.0;
        const double bp = (j + 1 < g.J) ? fyr + fy[r + g.K] : 0.0;
        const double bm = (j > 0) ? fyr + fy[r - g.K] : 0.0;
        const double cp = (k + 1 < g.K) ? fzr + fz[r + 1] : 0.0;
        const double cm = (k > 0) ? fzr + fz[r - 1] : 0.0;
        const double sum = ((ap - am) + (bp - bm)) + (cp - cm);
        const double div_q = dd.pow2 ? sum * half_scale : (sum * 0.5) / dd.dx;
        double evap_sink = 0.0;
        if (t == kPore && __double_as_longlong(evap) != 0) {
            int air_faces = 0;
            if (i + 1 < g.I && (int)label[r + g.JK] == kAir) air_faces++;
            if (i > 0 && (int)label[r - g.JK] == kAir) air_faces++;
            if (j + 1 < g.J && (int)label[r + g.K] == kAir) air_faces++;
            if (j > 0 && (int)label[r - g.K] == kAir) air_faces++;
            if (k + 1 < g.K && (int)label[r + 1] == kAir) air_faces++;
            if (k > 0 && (int)label[r - 1] == kAir) air_faces++;
            evap_sink = dd.div(air_faces * evap);
        }
        qsum[r] = div_q + evap_sink;
        const double total_rate = fabs(div_q) + evap_sink;
        if (total_rate > v[0]) v[0] = total_rate;
    }
    block_max_store<1>(v, partials);
}

__global__ void __launch_bounds__(kBlock) k_active_list_sat(Grid g, const uint8_t* __restrict__ l8,
                                                            const uint16_t* __restrict__ l16,
                                                            int* __restrict__ list, unsigned int* __restrict__ count) {
    // block-uniform trip count (block_append is called by every thread of the block)
    for (long long b0 = (long long)blockIdx.x * blockDim.x; b0 < g.N; b0 += (long long)gridDim.x * blockDim.x) {
        const long long r = b0 + threadIdx.x;
        bool act = false;
        if (r < g.N) act = !sat_inactive(l8 ? (int)l8[r] : (int)l16[r]);
        block_append(act, (int)r, list, count);
    }
}

template <typename L>
__global__ void __launch_bounds__(kBlock) k_sat_update_st(Grid g, double dt_sub_over_phi, int num_steps,
                                                          const L* __restrict__ label,
                                                          const double* __restrict__ qsum,
                                                          double* __restrict__ sat) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.NP;
         r += (long long)gridDim.x * blockDim.x) {
        if (r >= g.N) {  // extra top plane of the freshly allocated array
            sat[r] = 0.0;
            continue;
        }
        if (sat_inactive((int)label[r])) {
            sat[r] = 0.0;  // never written by the reference's update (indeterminate there)
            continue;
        }
        const double q = qsum[r];
        double sv = sat[r];
        for (int step = 0; step < num_steps; ++step) {
            double new_sat = sv - dt_sub_over_phi * q;
            double nv = smax(0.0, smin(1.0, new_sat));
            bool fixed = (nv == sv) || (nv != nv && sv != sv);
            sv = nv;
            if (fixed) break;
        }
        sat[r] = sv;
    }
}

ls_status saturation_run(ls_ctx* c, double dt, ls_substep_info* info) {
    LS_TRY(flux_zero_now(c));  // after a transport without a flux evaluation since
    snap_fence(c, kSnapSat);
    const DxDiv dx = make_dxdiv(c->p.dx);
    const double evap = c->p.evaporative_flux;
    int grid = grid_for(c, c->g.N);
    if (!c->sat_q) LS_TRY(walloc_t(c, &c->sat_q, (size_t)c->g.N));
    // the active voxels (any order: the pass writes per voxel and takes a maximum)
    LS_TRY(wlist_reset(c));
    LS_LAUNCH(c, k_active_list_sat, grid, kBlock, 0, c->g,
              c->label_bytes == 1 ? (const uint8_t*)c->label : (const uint8_t*)nullptr,
              c->label_bytes == 2 ? (const uint16_t*)c->label : (const uint16_t*)nullptr, c->wlist, c->wcount);
    if (c->label_bytes == 1)
        LS_LAUNCH(c, k_sat_rate_list<uint8_t>, grid, kBlock, 0, c->g, dx, evap, (const uint8_t*)c->label,
                  c->fx, c->fy, c->fz, (const int*)c->wlist, (const unsigned int*)c->wcount, c->sat_q, c->partials);
    else
        LS_LAUNCH(c, k_sat_rate_list<uint16_t>, grid, kBlock, 0, c->g, dx, evap, (const uint16_t*)c->label,
                  c->fx, c->fy, c->fz, (const int*)c->wlist, (const unsigned int*)c->wcount, c->sat_q, c->partials);
    LS_TRY(finalize_max(c, grid, 1, S_RED0));
    double max_div_q = 0.0;
    LS_TRY(read_scalars(c, S_RED0, 1, &max_div_q));
    // sub-step count, src/Simulation.cpp:1740-1767
    const double max_dsat = 0.1;
    double dt_safe = dt;
    if (max_div_q > 1e-20) dt_safe = (max_dsat * c->p.porosity) / max_div_q;
    double calculated_steps = std::ceil(dt / dt_safe);
    int num_steps = 1;
    if (std::isinf(calculated_steps) || std::isnan(calculated_steps)) num_steps = 1000;
    else if (calculated_steps > 1000) num_steps = 1000;
    else if (calculated_steps > 1.0) num_steps = (int)calculated_steps;
    double dt_sub = dt / num_steps;
    double dt_sub_over_phi = dt_sub / c->p.porosity;
    if (info) {
        info->max_rate = max_div_q;
        info->num_steps = num_steps;
        info->dt_sub = dt_sub;
    }
    int grid2 = grid_for(c, c->g.NP);
    if (c->label_bytes == 1)
        LS_LAUNCH(c, k_sat_update_st<uint8_t>, grid2, kBlock, 0, c->g, dt_sub_over_phi, num_steps,
                  (const uint8_t*)c->label, (const double*)c->sat_q, c->sat);
    else
        LS_LAUNCH(c, k_sat_update_st<uint16_t>, grid2, kBlock, 0, c->g, dt_sub_over_phi, num_steps,
                  (const uint16_t*)c->label, (const double*)c->sat_q, c->sat);
    return LS_OK;
}

// ---------------------------------------------------------------------------
// handleSurfaceEffects: a Pore voxel holding fluid next to Air clogs. Turning Pore into
// Precipitate never changes whether a neighbour is Air, so the voxels are independent.

template <typename L>
__global__ void __launch_bounds__(kBlock) k_surface(Grid g, L* __restrict__ label,
                                                    const double* __restrict__ sat,
                                                    double* __restrict__ conc) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        if ((int)label[r] != kPore || !(sat[r] > 0.0)) continue;
        int i, j, k;
        decode(g, r, i, j, k);
        bool s = (i + 1 < g.I && (int)label[r + g.JK] == kAir) ||
                 (i > 0 && (int)label[r - g.JK] == kAir) ||
                 (j + 1 < g.J && (int)label[r + g.K] == kAir) ||
                 (j > 0 && (int)label[r - g.K] == kAir) ||
                 (k + 1 < g.K && (int)label[r + 1] == kAir) ||
                 (k > 0 && (int)label[r - 1] == kAir);
        if (s) {
            conc[r] = 1.0;
            label[r] = (L)kPrecipitate;
        }
    }
}

ls_status surface_run(ls_ctx* c) {
    snap_fence(c, kSnapRest);
    int grid = grid_for(c, c->g.N);
    if (c->label_bytes == 1)
        LS_LAUNCH(c, k_surface<uint8_t>, grid, kBlock, 0, c->g, (uint8_t*)c->label, c->sat, c->conc);
    else
        LS_LAUNCH(c, k_surface<uint16_t>, grid, kBlock, 0, c->g, (uint16_t*)c->label, c->sat, c->conc);
    c->p_ready = 0;
    return LS_OK;
}

// ---------------------------------------------------------------------------
// handlePrecipitation (pointwise).

template <typename L>
__global__ void __launch_bounds__(kBlock) k_precip(Grid g, double c_sat, int instant,
                                                   double porosity, double solid_density,
                                                   double time_scalar, L* __restrict__ label,
                                                   double* __restrict__ conc,
                                                   const double* __restrict__ sat,
                                                   double* __restrict__ precip) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        double cv = conc[r];
        if ((int)label[r] == kPore && cv > c_sat) {
            double excess_conc = cv - c_sat;
            if (instant) {
                label[r] = (L)kPrecipitate;
            } else {
                double fluid_vol_fraction = porosity * sat[r];
                double precipitated_vol_fraction = (excess_conc * fluid_vol_fraction) / solid_density;
                double pv = precip[r] + (precipitated_vol_fraction * time_scalar);
                precip[r] = pv;
                if (pv > 0.90) label[r] = (L)kPrecipitate;
            }
            conc[r] = c_sat;
        }
    }
}

ls_status precip_run(ls_ctx* c) {
    snap_fence(c, kSnapRest);
    int grid = grid_for(c, c->g.N);
    const ls_params& p = c->p;
    if (c->label_bytes == 1)
        LS_LAUNCH(c, k_precip<uint8_t>, grid, kBlock, 0, c->g, p.c_sat, p.use_instant_precipitation,
                  p.porosity, p.solid_density, p.time_scalar, (uint8_t*)c->label, c->conc, c->sat,
                  c->precip);
    else
        LS_LAUNCH(c, k_precip<uint16_t>, grid, kBlock, 0, c->g, p.c_sat, p.use_instant_precipitation,
                  p.porosity, p.solid_density, p.time_scalar, (uint16_t*)c->label, c->conc, c->sat,
                  c->precip);
    c->p_ready = 0;
    return LS_OK;
}

// ---------------------------------------------------------------------------
// FP64 budget of a step: the field sums, the acid the dissolution sweep took (per voxel the
// acid before the sweep minus after, summed) and the mineral lost since the snapshot at the
// start of the step (frac changes only in the sweep), in a fixed reduction order.
template <typename L>
__global__ void __launch_bounds__(kBlock) k_budget(Grid g, const L* __restrict__ label,
                                                   const double* __restrict__ conc,
                                                   const double* __restrict__ acid,
                                                   const float* __restrict__ frac,
                                                   const float* __restrict__ frac0,
                                                   const double* __restrict__ precip,
                                                   const double* __restrict__ acid_pre,
                                                   double* __restrict__ partials) {
    // FP64 issue is what bounds this pass, so terms that add nothing are skipped on the integer
    // side: a sum that starts at +0.0 never becomes -0.0, so adding +-0.0 leaves it as it is,
    // and x - x = +0.0 (an unchanged voxel's consumed acid or lost mineral). The counts are
    // integers and the FP32 fractions widen exactly on the integer pipe.
    double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    long long n_sul = 0, n_pre = 0;
    const long long kMag = 0x7fffffffffffffffll;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < g.N;
         r += (long long)gridDim.x * blockDim.x) {
        const double a = acid[r];
        const double cv = conc[r], pv = precip[r];
        const float f = frac[r], f0 = frac0[r];
        const double fd = f2d_exact(f);
        if (__double_as_longlong(cv) & kMag) acc[0] += cv;
        if (__double_as_longlong(a) & kMag) acc[1] += a;
        if (__float_as_uint(f) & 0x7fffffffu) acc[2] += fd;
        if (__double_as_longlong(pv) & kMag) acc[3] += pv;
        if (acid_pre) {
            const double ap = acid_pre[r];
            if (__double_as_longlong(ap) != __double_as_longlong(a)) acc[4] += ap - a;
        }
        if (__float_as_uint(f0) != __float_as_uint(f)) acc[5] += f2d_exact(f0) - fd;
        const int t = (int)label[r];
        n_sul += (t == kSulphide) ? 1 : 0;
        n_pre += (t == kPrecipitate) ? 1 : 0;
    }
    acc[6] = (double)n_sul;
    acc[7] = (double)n_pre;
    block_sum_store<8>(acc, partials);
}

ls_status budget_run(ls_ctx* c, const double* acid_pre, ls_budget* b) {
    const int grid = grid_for(c, c->g.N);
    if (c->label_bytes == 1)
        LS_LAUNCH(c, k_budget<uint8_t>, grid, kBlock, 0, c->g, (const uint8_t*)c->label, (const double*)c->conc,
                  (const double*)c->acid, (const float*)c->frac, (const float*)c->b_frac,
                  (const double*)c->precip, acid_pre, c->partials);
    else
        LS_LAUNCH(c, k_budget<uint16_t>, grid, kBlock, 0, c->g, (const uint16_t*)c->label,
                  (const double*)c->conc, (const double*)c->acid, (const float*)c->frac,
                  (const float*)c->b_frac, (const double*)c->precip, acid_pre, c->partials);
    LS_TRY(finalize_sum(c, grid, 8, S_RED0));
    double v[8];
    LS_TRY(read_scalars(c, S_RED0, 8, v));
    b->conc = v[0];
    b->acid = v[1];
    b->mineral = v[2];
    b->precipitate = v[3];
    b->acid_consumed = v[4];
    b->mineral_dissolved = v[5];
    b->sulphide_voxels = (long long)v[6];
    b->precipitate_voxels = (long long)v[7];
    return LS_OK;
}

}  // namespace ls

// ===========================================================================
// Explicit saturation update on caller-owned device buffers, allocating nothing.
//
// Some callers cannot let this library call cudaMalloc: hosts that own all device memory
// through their own pool (a solver framework handing out preallocated work arrays, or a
// process run under a fixed device-memory budget), and time-stepping loops that must not
// pay for the device-wide synchronisation cudaMalloc/cudaFree may imply. For them the
// reduction scratch of this update lives in a file-scope device array of fixed size,
// loaded with the library and held on every GPU that loads it until the process exits.
// The first call on a device looks up the array's device address (cudaGetSymbolAddress,
// with that device current) and caches it, so that first call should come before any
// stream capture; later calls check that the cached address is still device memory of that
// device (it is not after a reset of the device's context) and look it up again if not.
// Each call waits for its own result on the host (it reads the largest rate back to choose
// the sub-step count). Every call uses the same array: two calls that overlap on the GPU (on
// different streams or host threads) race on it. Each call writes every slot it later
// reads (no accumulation), so nothing has to be cleared; the previous call's contents stay
// until overwritten.

namespace ls {

constexpr int kNoAllocVoxelsPerThread = 32;
constexpr int kNoAllocSlots = 16384;  // one block maximum per 256*32 voxels, + result slot
static __device__ __align__(256) double g_noalloc_sat_scratch[kNoAllocSlots + 32];

// block maxima of |div q| + evaporative sink over the active voxels of one chunk
template <typename L>
__global__ void __launch_bounds__(kBlock) k_noalloc_sat_rate(Grid g, DxDiv dd, double evap,
                                                             const L* __restrict__ label,
                                                             const double* __restrict__ fx,
                                                             const double* __restrict__ fy,
                                                             const double* __restrict__ fz,
                                                             double* __restrict__ scratch) {
    double v[1] = {0.0};
    const long long base = (long long)blockIdx.x * kBlock * kNoAllocVoxelsPerThread;
    for (int q = 0; q < kNoAllocVoxelsPerThread; ++q) {
        long long r = base + (long long)q * kBlock + threadIdx.x;
        if (r >= g.N) break;
        int t = (int)label[r];
        if (sat_inactive(t)) continue;
        int i, j, k;
        decode(g, r, i, j, k);
        double div_q, evap_sink;
        sat_rates(g, label, fx, fy, fz, r, i, j, k, t, dd, evap, div_q, evap_sink);
        double total_rate = fabs(div_q) + evap_sink;
        if (total_rate > v[0]) v[0] = total_rate;
    }
    block_max_store<1>(v, scratch);
}

// max of the block maxima into the result slot
__global__ void __launch_bounds__(kFinalizeThreads) k_noalloc_sat_final(int nblocks, double* __restrict__ scratch) {
    __shared__ double sh[kFinalizeThreads];
    double acc = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) acc = smax(acc, scratch[b]);
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kFinalizeThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] = smax(sh[threadIdx.x], sh[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) scratch[kNoAllocSlots] = sh[0];
}

static double* noalloc_scratch_address(int device, cudaError_t* err) {
    static std::mutex mu;
    static double* addr[128] = {nullptr};
    *err = cudaSuccess;
    if (device < 0 || device >= 128) {
        *err = cudaErrorInvalidDevice;
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(mu);
    if (addr[device]) {
        // the address is cached per device; a reset of the device's context reloads the module,
        // so check that the cached address is still device memory of this device, and look it
        // up again otherwise
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, addr[device]) != cudaSuccess || at.type != cudaMemoryTypeDevice ||
            at.device != device) {
            cudaGetLastError();  // the failed query leaves its own error pending
            addr[device] = nullptr;
        }
    }
    if (!addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_sat_scratch);
        if (e != cudaSuccess) {
            *err = e;
            return nullptr;
        }
        addr[device] = (double*)p;
    }
    return addr[device];
}

}  // namespace ls

static ls_status noalloc_fail(ls_status st, char* err, size_t len, const char* msg) {
    if (err && len) snprintf(err, len, "%s", msg);
    return st;
}

extern "C" ls_status ls_saturation_noalloc(int I, int J, int K, int label_bytes, const void* label,
                                           const double* flux_x, const double* flux_y,
                                           const double* flux_z, double* saturation, double dt,
                                           double dx, double porosity, double evaporative_flux,
                                           void* stream, ls_substep_info* info, char* err,
                                           size_t err_len) {
    using namespace ls;
    if (err && err_len) err[0] = '\0';
    if (I < 2 || J < 2 || K < 2 || (label_bytes != 1 && label_bytes != 2))
        return noalloc_fail(LS_BAD_ARG, err, err_len, "ls_saturation_noalloc: bad extents or label_bytes");
    if (!label || !flux_x || !flux_y || !flux_z || !saturation)
        return noalloc_fail(LS_BAD_ARG, err, err_len, "ls_saturation_noalloc: null device pointer");
    if (!(dt > 0.0) || !(dx > 0.0) || !(porosity > 0.0))
        return noalloc_fail(LS_BAD_ARG, err, err_len, "ls_saturation_noalloc: dt, dx and porosity must be > 0");
    const long long N = (long long)I * J * K;
    if (N > LS_NOALLOC_SAT_MAX_VOXELS) {
        char buf[200];
        snprintf(buf, sizeof(buf),
                 "ls_saturation_noalloc: %lld voxels exceed the fixed scratch limit of %lld voxels "
                 "(use ls_saturation on a context instead)", N, (long long)LS_NOALLOC_SAT_MAX_VOXELS);
        return noalloc_fail(LS_BAD_ARG, err, err_len, buf);
    }
    Grid g;
    g.I = I; g.J = J; g.K = K;
    g.JK = (long long)J * K;
    g.N = N;
    g.NP = N + g.JK;
    grid_init_div(g);
    int device = 0;
    cudaError_t ce = cudaGetDevice(&device);
    if (ce != cudaSuccess) return noalloc_fail(LS_CUDA_ERROR, err, err_len, cudaGetErrorString(ce));
    double* scratch = noalloc_scratch_address(device, &ce);
    if (!scratch) return noalloc_fail(LS_CUDA_ERROR, err, err_len, cudaGetErrorString(ce));
    cudaStream_t s = (cudaStream_t)stream;
    const DxDiv dd = make_dxdiv(dx);
    const int nblocks = (int)((N + (long long)kBlock * kNoAllocVoxelsPerThread - 1) /
                              ((long long)kBlock * kNoAllocVoxelsPerThread));
    if (label_bytes == 1)
        k_noalloc_sat_rate<uint8_t><<<nblocks, kBlock, 0, s>>>(g, dd, evaporative_flux, (const uint8_t*)label,
                                                              flux_x, flux_y, flux_z, scratch);
    else
        k_noalloc_sat_rate<uint16_t><<<nblocks, kBlock, 0, s>>>(g, dd, evaporative_flux, (const uint16_t*)label,
                                                               flux_x, flux_y, flux_z, scratch);
    k_noalloc_sat_final<<<1, kFinalizeThreads, 0, s>>>(nblocks, scratch);
    // launch errors of these two launches, read without clearing anything else pending
    ce = cudaPeekAtLastError();
    if (ce != cudaSuccess) return noalloc_fail(LS_CUDA_ERROR, err, err_len, cudaGetErrorString(ce));
    double max_div_q = 0.0;
    ce = cudaMemcpyAsync(&max_div_q, scratch + kNoAllocSlots, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) return noalloc_fail(LS_CUDA_ERROR, err, err_len, cudaGetErrorString(ce));
    // sub-step count, src/Simulation.cpp:1740-1767
    const double max_dsat = 0.1;
    double dt_safe = dt;
    if (max_div_q > 1e-20) dt_safe = (max_dsat * porosity) / max_div_q;
    double calculated_steps = std::ceil(dt / dt_safe);
    int num_steps = 1;
    if (std::isinf(calculated_steps) || std::isnan(calculated_steps)) num_steps = 1000;
    else if (calculated_steps > 1000) num_steps = 1000;
    else if (calculated_steps > 1.0) num_steps = (int)calculated_steps;
    double dt_sub = dt / num_steps;
    double dt_sub_over_phi = dt_sub / porosity;
    if (info) {
        info->max_rate = max_div_q;
        info->num_steps = num_steps;
        info->dt_sub = dt_sub;
    }
    const int grid2 = (int)std::min<long long>((g.NP + kBlock - 1) / kBlock, 152LL * 8);
    if (label_bytes == 1)
        k_sat_update<uint8_t><<<grid2, kBlock, 0, s>>>(g, dd, evaporative_flux, dt_sub_over_phi, num_steps,
                                                       (const uint8_t*)label, flux_x, flux_y, flux_z, saturation);
    else
        k_sat_update<uint16_t><<<grid2, kBlock, 0, s>>>(g, dd, evaporative_flux, dt_sub_over_phi, num_steps,
                                                        (const uint16_t*)label, flux_x, flux_y, flux_z, saturation);
    ce = cudaPeekAtLastError();
    if (ce != cudaSuccess) return noalloc_fail(LS_CUDA_ERROR, err, err_len, cudaGetErrorString(ce));
    return LS_OK;
}
