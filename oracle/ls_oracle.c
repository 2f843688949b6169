/*
 * ls_oracle.c - CPU restatement of the LeachingSim per-time-step algorithm.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline); the
 * product library never links or calls it. Parity is pinned to the reference's
 * own code compiled against single-rank MPI / PETSc / VTK stand-ins (oracle/_ref,
 * tests/test_ref_pin.py); see ls_oracle.h.
 *
 * Citations "S.cpp:N" are to src/Simulation.cpp of the reference project,
 * "main.cpp:N" to src/main.cpp, "M.h:N" to src/MPIDomain.h.
 *
 * Restated for one MPI rank. Every field has (I+1)*J*K slots (M.h:75-97:
 * rank 0 clips only its lower halo); voxel (i,j,k) lives in slot
 * k + K*(j + J*i). PETSc row (i,j,k) has the same linear number and, with
 * compat_shift, its solution is written to slot row + J*K (the solution
 * vector is placed at data + pad_size, S.cpp:808,1247,1975,2173).
 *
 * Floating point: compile with -ffp-contract=off. The reference is built with
 * plain -O3 for x86-64 (Makefile:46), which has no FMA, so every a*b+c in it
 * rounds twice; so must this file on every host.
 */
#include "ls_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { AIR = 1, PORE = 2, ROCK = 3, SULPHIDE = 4, PRECIPITATE = 5 };

/* std::min / std::max exactly: min(a,b) = (b < a) ? b : a; max(a,b) = (a < b) ? b : a. */
static inline double smin(double a, double b) { return (b < a) ? b : a; }
static inline double smax(double a, double b) { return (a < b) ? b : a; }

typedef struct ell_sys {
    double* A[6];   /* neighbour coefficients, directions +i,-i,+j,-j,+k,-k */
    double* diag;
    double* b;
    int8_t* kind;   /* 0 empty row, 1 identity-like row, 2 coupled row */
} ell_sys;

struct lso_state {
    int I, J, K, label_bytes;
    size_t JK, N, NP;
    ls_params p;
    lso_solver_cfg cfg;
    uint16_t* label;
    float* frac;
    float* kmult;       /* intrinsic-permeability multiplier (NULL: 1 everywhere) */
    double *perm, *visc, *P, *conc, *acid, *fx, *fy, *fz, *sat, *pc, *kr, *precip;
    uint16_t* b_label;
    float* b_frac;
    double *b_precip, *b_sat, *b_P, *b_conc, *b_acid, *b_fx, *b_fy, *b_fz;
    ell_sys press, trans, satsys;
    double* gm_work;    /* GMRES Krylov basis + scratch */
    int gm_restart;
    unsigned long long initial_sulphide_count, total_leached;
    int physics_valid;
};

/* ------------------------------------------------------------------------ */
/* indexing                                                                  */

static inline size_t IDX(const lso_state* s, int i, int j, int k) {
    return (size_t)k + (size_t)s->K * ((size_t)j + (size_t)s->J * (size_t)i);
}

/* neighbour in direction d (0:+i 1:-i 2:+j 3:-j 4:+k 5:-k); returns 0 when outside
   the global domain (SubIndex::valid(global), Domain.h:71-74). */
static inline int NB(const lso_state* s, int i, int j, int k, int d, size_t* nb) {
    switch (d) {
    case 0: if (i + 1 >= s->I) return 0; *nb = IDX(s, i + 1, j, k); return 1;
    case 1: if (i - 1 < 0) return 0; *nb = IDX(s, i - 1, j, k); return 1;
    case 2: if (j + 1 >= s->J) return 0; *nb = IDX(s, i, j + 1, k); return 1;
    case 3: if (j - 1 < 0) return 0; *nb = IDX(s, i, j - 1, k); return 1;
    case 4: if (k + 1 >= s->K) return 0; *nb = IDX(s, i, j, k + 1); return 1;
    default: if (k - 1 < 0) return 0; *nb = IDX(s, i, j, k - 1); return 1;
    }
}

/* ------------------------------------------------------------------------ */
/* life cycle                                                                */

static void* xcalloc(size_t n, size_t sz) {
    void* p = calloc(n ? n : 1, sz);
    if (!p) {
        fprintf(stderr, "ls_oracle: out of memory (%zu x %zu)\n", n, sz);
        abort();
    }
    return p;
}

static void ell_alloc(ell_sys* e, size_t n) {
    for (int d = 0; d < 6; ++d) e->A[d] = (double*)xcalloc(n, sizeof(double));
    e->diag = (double*)xcalloc(n, sizeof(double));
    e->b = (double*)xcalloc(n, sizeof(double));
    e->kind = (int8_t*)xcalloc(n, 1);
}

static void ell_free(ell_sys* e) {
    for (int d = 0; d < 6; ++d) free(e->A[d]);
    free(e->diag);
    free(e->b);
    free(e->kind);
}

lso_state* lso_create(int I, int J, int K, int label_bytes, const ls_params* p) {
    if (I < 2 || J < 2 || K < 2 || (label_bytes != 1 && label_bytes != 2)) return NULL;
    lso_state* s = (lso_state*)xcalloc(1, sizeof(lso_state));
    s->I = I; s->J = J; s->K = K; s->label_bytes = label_bytes;
    s->JK = (size_t)J * K;
    s->N = (size_t)I * s->JK;
    s->NP = s->N + s->JK;
    if (p) s->p = *p; else lso_params_default(&s->p);
    s->cfg.mode = LSO_SOLVE_REFERENCE;
    s->cfg.restart = 30;
    s->cfg.rtol = -1.0;
    s->cfg.max_it = -1;
    size_t NP = s->NP;
    s->label = (uint16_t*)xcalloc(NP, sizeof(uint16_t));
    s->frac = (float*)xcalloc(NP, sizeof(float));
    double** f[] = {&s->perm, &s->visc, &s->P, &s->conc, &s->acid, &s->fx, &s->fy,
                    &s->fz, &s->sat, &s->pc, &s->kr, &s->precip};
    for (size_t q = 0; q < sizeof(f) / sizeof(f[0]); ++q) *f[q] = (double*)xcalloc(NP, sizeof(double));
    s->b_label = (uint16_t*)xcalloc(NP, sizeof(uint16_t));
    s->b_frac = (float*)xcalloc(NP, sizeof(float));
    double** b[] = {&s->b_precip, &s->b_sat, &s->b_P, &s->b_conc, &s->b_acid,
                    &s->b_fx, &s->b_fy, &s->b_fz};
    for (size_t q = 0; q < sizeof(b) / sizeof(b[0]); ++q) *b[q] = (double*)xcalloc(NP, sizeof(double));
    ell_alloc(&s->press, s->N);
    ell_alloc(&s->trans, s->N);
    ell_alloc(&s->satsys, s->N);
    s->physics_valid = 1;
    return s;
}

void lso_destroy(lso_state* s) {
    if (!s) return;
    free(s->label); free(s->frac); free(s->kmult);
    double* f[] = {s->perm, s->visc, s->P, s->conc, s->acid, s->fx, s->fy, s->fz,
                   s->sat, s->pc, s->kr, s->precip, s->b_precip, s->b_sat, s->b_P,
                   s->b_conc, s->b_acid, s->b_fx, s->b_fy, s->b_fz};
    for (size_t q = 0; q < sizeof(f) / sizeof(f[0]); ++q) free(f[q]);
    free(s->b_label); free(s->b_frac);
    ell_free(&s->press); ell_free(&s->trans); ell_free(&s->satsys);
    free(s->gm_work);
    free(s);
}

void lso_set_params(lso_state* s, const ls_params* p) { s->p = *p; }

/* CLI defaults of src/main.cpp:39 and the constants of src/main.cpp:89-91. */
void lso_params_default(ls_params* p) {
    memset(p, 0, sizeof(*p));
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
    p->vg_alpha = 1.0;
    p->vg_n = 2.0;
    p->s_res = 0.05;
    p->porosity = 0.1;
    p->time_scalar = 1.0;
    p->rock_D_fac = 1e-4;
    p->alpha_transfer = 1e-5;
    p->solid_density = 1.0;
    p->compat_shift = 1;
    p->press_rtol = 1e-6;
    p->press_max_it = 10000;
    p->conc_rtol = 1e-6;
    p->conc_max_it = 10000;
    p->sat_rtol = 1e-6;
    p->sat_max_it = 10000;
    p->bc_mode = LS_BC_REFERENCE;
    p->p_inlet = 1.0;
    p->p_outlet = 0.0;
    p->conc_inlet = 0.0;
    p->acid_inlet = 0.0;
    p->pore_permeability = 1.0e-12;
    p->rock_permeability = 1.0e-18;
}
void lso_set_solver(lso_state* s, const lso_solver_cfg* cfg) { s->cfg = *cfg; }
unsigned long long lso_initial_sulphide_count(const lso_state* s) { return s->initial_sulphide_count; }

int lso_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void lso_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

static void* field_ptr(lso_state* s, int f, size_t* esz) {
    switch (f) {
    case LS_F_LABEL: *esz = 2; return s->label;
    case LS_F_FRAC: *esz = 4; return s->frac;
    case LS_F_PERMEABILITY: *esz = 8; return s->perm;
    case LS_F_VISCOSITY: *esz = 8; return s->visc;
    case LS_F_PRESSURE: *esz = 8; return s->P;
    case LS_F_CONC: *esz = 8; return s->conc;
    case LS_F_ACID: *esz = 8; return s->acid;
    case LS_F_FLUX_X: *esz = 8; return s->fx;
    case LS_F_FLUX_Y: *esz = 8; return s->fy;
    case LS_F_FLUX_Z: *esz = 8; return s->fz;
    case LS_F_SATURATION: *esz = 8; return s->sat;
    case LS_F_CAP_PRESSURE: *esz = 8; return s->pc;
    case LS_F_REL_PERM: *esz = 8; return s->kr;
    case LS_F_PRECIPITATE: *esz = 8; return s->precip;
    case LS_F_KMULT:
        *esz = 4;
        if (!s->kmult) {
            s->kmult = (float*)xcalloc(s->NP, sizeof(float));
            for (size_t r = 0; r < s->NP; ++r) s->kmult[r] = 1.0f;
        }
        return s->kmult;
    default: return NULL;
    }
}

int lso_set_field(lso_state* s, int f, const void* src, size_t n, int padded) {
    size_t esz = 0;
    void* dst = field_ptr(s, f, &esz);
    if (!dst || n != (padded ? s->NP : s->N)) return -1;
    memcpy(dst, src, n * esz);
    return 0;
}

int lso_get_field(lso_state* s, int f, void* dst, size_t n, int padded) {
    size_t esz = 0;
    void* src = field_ptr(s, f, &esz);
    if (!src || n != (padded ? s->NP : s->N)) return -1;
    memcpy(dst, src, n * esz);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* initialisation                                                            */

/* Simulation::initFields, S.cpp:165-180: zero nine arrays over the padded extent. */
void lso_init_fields(lso_state* s) {
    size_t NP = s->NP;
    double* f[] = {s->P, s->conc, s->fx, s->fy, s->fz, s->sat, s->pc, s->kr, s->precip};
    for (size_t q = 0; q < sizeof(f) / sizeof(f[0]); ++q) memset(f[q], 0, NP * sizeof(double));
}

/* Simulation::initFrac, S.cpp:254-278. */
unsigned long long lso_init_frac(lso_state* s) {
    unsigned long long count = 0;
    for (size_t r = 0; r < s->N; ++r) {
        if (s->label[r] == SULPHIDE) {
            s->frac[r] = 1.0f;
            count++;
        } else {
            s->frac[r] = 0.0f;
        }
    }
    s->initial_sulphide_count = count;
    s->total_leached = 0;
    return count;
}

/* Simulation::initSaturation, S.cpp:1573-1590. */
void lso_init_saturation(lso_state* s) {
    for (size_t r = 0; r < s->N; ++r) {
        uint16_t t = s->label[r];
        s->sat[r] = (t == PORE || t == SULPHIDE) ? 0.1 : 0.0;
    }
}

/* Simulation::initAcid, S.cpp:285-310. */
void lso_init_acid(lso_state* s) {
    for (size_t r = 0; r < s->N; ++r) s->acid[r] = 0.0;
}

/* ------------------------------------------------------------------------ */
/* material properties                                                       */

/* Simulation::updateRelativePermeability, S.cpp:1634-1664 (Mualem-van Genuchten). */
void lso_update_relperm(lso_state* s) {
    const double m = 1.0 - (1.0 / s->p.vg_n);
    const double s_res = s->p.s_res;
    const long N = (long)s->N;
#pragma omp parallel for schedule(static)
    for (long r = 0; r < N; ++r) {
        uint16_t t = s->label[r];
        if (t == PORE || t == SULPHIDE) {
            double Se = (s->sat[r] - s_res) / (1.0 - s_res);
            Se = smax(0.0, smin(1.0, Se));
            if (Se <= 0.0) {
                s->kr[r] = 0.0;
            } else {
                double term1 = 1.0 - pow(1.0 - pow(Se, 1.0 / m), m);
                s->kr[r] = sqrt(Se) * term1 * term1;
            }
        } else {
            s->kr[r] = 0.0;
        }
    }
}

/* Simulation::updateCapillaryPressure, S.cpp:1596-1628 (van Genuchten). */
void lso_update_cap(lso_state* s) {
    const double m = 1.0 - (1.0 / s->p.vg_n);
    const double s_res = s->p.s_res;
    const long N = (long)s->N;
#pragma omp parallel for schedule(static)
    for (long r = 0; r < N; ++r) {
        uint16_t t = s->label[r];
        if (t == PORE || t == SULPHIDE) {
            double Se = (s->sat[r] - s_res) / (1.0 - s_res);
            Se = smax(1e-6, smin(1.0, Se));
            if (Se >= 1.0) {
                s->pc[r] = 0.0;
            } else {
                double Se_inv_m = pow(Se, -1.0 / m);
                s->pc[r] = (1.0 / s->p.vg_alpha) * pow(Se_inv_m - 1.0, 1.0 / s->p.vg_n);
            }
        } else {
            s->pc[r] = 0.0;
        }
    }
}

/* Simulation::initProperties, S.cpp:187-248. The two permeability constants of
 * S.cpp:190-191 come from the parameters (the reference's values by default), and the
 * intrinsic permeability is multiplied by the per-voxel factor when one was set (an
 * extension: the reference has neither). */
void lso_init_properties(lso_state* s) {
    const double pore_permeability = s->p.pore_permeability;
    const double rock_permeability = s->p.rock_permeability;
    const float* kmult = s->kmult;
    const long N = (long)s->N;
#pragma omp parallel for schedule(static)
    for (long r = 0; r < N; ++r) {
        uint16_t type = s->label[r];
        double K_intrinsic = rock_permeability;
        double log_k_rock = log10(rock_permeability);
        double log_k_pore = log10(pore_permeability);
        if (type == AIR) {
            K_intrinsic = pore_permeability;
        } else if (type == PORE) {
            double p_frac = s->precip[r];
            p_frac = smax(0.0, smin(1.0, p_frac));
            double log_k_eff = (p_frac * log_k_rock) + ((1.0 - p_frac) * log_k_pore);
            K_intrinsic = pow(10.0, log_k_eff);
        } else if (type == SULPHIDE) {
            double f = s->frac[r];
            double log_k_eff = (f * log_k_rock) + ((1.0 - f) * log_k_pore);
            K_intrinsic = pow(10.0, log_k_eff);
        }
        if (kmult) K_intrinsic = K_intrinsic * (double)kmult[r];
        s->visc[r] = (type == AIR) ? 1.8e-5 : 1.0e-3;
        double K_rel = smax(s->kr[r], 1e-15);
        s->perm[r] = K_intrinsic * K_rel;
    }
}

/* ------------------------------------------------------------------------ */
/* ELL operator + Jacobi-left-preconditioned GMRES (PETSc KSPGMRES + PCJACOBI) */

/* y = A x. Entries are summed in ascending column order like an AIJ row. */
static void ell_apply(const lso_state* s, const ell_sys* e, const double* x, double* y) {
    const int I = s->I, J = s->J, K = s->K;
    const long JK = (long)s->JK;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < I; ++i) {
        for (int j = 0; j < J; ++j) {
            for (int k = 0; k < K; ++k) {
                long r = (long)k + (long)K * ((long)j + (long)J * i);
                double acc = 0.0;
                if (i > 0) acc += e->A[1][r] * x[r - JK];
                if (j > 0) acc += e->A[3][r] * x[r - K];
                if (k > 0) acc += e->A[5][r] * x[r - 1];
                acc += e->diag[r] * x[r];
                if (k + 1 < K) acc += e->A[4][r] * x[r + 1];
                if (j + 1 < J) acc += e->A[2][r] * x[r + K];
                if (i + 1 < I) acc += e->A[0][r] * x[r + JK];
                y[r] = acc;
            }
        }
    }
}

static double dot(const double* a, const double* b, long n) {
    double acc = 0.0;
#pragma omp parallel for reduction(+ : acc) schedule(static)
    for (long r = 0; r < n; ++r) acc += a[r] * b[r];
    return acc;
}

static double scaled_residual(lso_state* s, const ell_sys* e, const double* b, const double* x);

/* Left-preconditioned restarted GMRES with classical Gram-Schmidt (PETSc's defaults for
   KSPGMRES) and the default convergence test: ||B r_k|| <= max(rtol*||B b||, abstol),
   B = Jacobi (zero diagonal entries replaced by 1). Returns a PETSc-style reason. */
static int gmres(lso_state* s, const ell_sys* e, const double* b, double* x, int restart,
                 double rtol, int max_it, int* its_out, double* rel_out) {
    const long n = (long)s->N;
    const double abstol = 1e-50;
    if (restart < 1) restart = 1;
    if (s->gm_restart < restart || !s->gm_work) {
        free(s->gm_work);
        s->gm_work = (double*)xcalloc((size_t)(restart + 3) * (size_t)n, sizeof(double));
        s->gm_restart = restart;
    }
    double* V = s->gm_work;                          /* restart+1 basis vectors */
    double* w = s->gm_work + (size_t)(restart + 1) * n;
    double* dinv = w + n;
    double* H = (double*)xcalloc((size_t)(restart + 1) * restart, sizeof(double));
    double* cs = (double*)xcalloc(restart, sizeof(double));
    double* sn = (double*)xcalloc(restart, sizeof(double));
    double* g = (double*)xcalloc(restart + 1, sizeof(double));
    double* yv = (double*)xcalloc(restart, sizeof(double));

#pragma omp parallel for schedule(static)
    for (long r = 0; r < n; ++r) dinv[r] = (e->diag[r] != 0.0) ? 1.0 / e->diag[r] : 1.0;

    /* snorm = ||B b|| */
    double snorm = 0.0;
#pragma omp parallel for reduction(+ : snorm) schedule(static)
    for (long r = 0; r < n; ++r) {
        double t = dinv[r] * b[r];
        snorm += t * t;
    }
    snorm = sqrt(snorm);
    const double ttol = smax(rtol * snorm, abstol);
    int its = 0;
    int reason = 0;
    double rnorm = 0.0;

    for (;;) {
        /* r = B (b - A x) */
        ell_apply(s, e, x, w);
        double beta2 = 0.0;
#pragma omp parallel for reduction(+ : beta2) schedule(static)
        for (long r = 0; r < n; ++r) {
            double t = dinv[r] * (b[r] - w[r]);
            V[r] = t;
            beta2 += t * t;
        }
        double beta = sqrt(beta2);
        rnorm = beta;
        if (isnan(beta) || isinf(beta)) { reason = -4; break; }
        if (beta <= ttol) { reason = (beta < abstol) ? 3 : 2; break; }
        if (its >= max_it) { reason = -3; break; }
#pragma omp parallel for schedule(static)
        for (long r = 0; r < n; ++r) V[r] /= beta;
        memset(g, 0, sizeof(double) * (restart + 1));
        g[0] = beta;
        int jdone = 0;
        for (int j = 0; j < restart; ++j) {
            double* vj = V + (size_t)j * n;
            double* vn = V + (size_t)(j + 1) * n;
            ell_apply(s, e, vj, w);
#pragma omp parallel for schedule(static)
            for (long r = 0; r < n; ++r) vn[r] = dinv[r] * w[r];
            /* classical Gram-Schmidt: all projections from the unmodified vector */
            for (int q = 0; q <= j; ++q) H[q * restart + j] = dot(vn, V + (size_t)q * n, n);
#pragma omp parallel for schedule(static)
            for (long r = 0; r < n; ++r) {
                double t = vn[r];
                for (int q = 0; q <= j; ++q) t -= H[q * restart + j] * V[(size_t)q * n + r];
                vn[r] = t;
            }
            double hn = sqrt(dot(vn, vn, n));
            H[(j + 1) * restart + j] = hn;
            if (hn > 0.0) {
#pragma omp parallel for schedule(static)
                for (long r = 0; r < n; ++r) vn[r] /= hn;
            }
            /* apply previous rotations */
            for (int q = 0; q < j; ++q) {
                double a = H[q * restart + j], c = H[(q + 1) * restart + j];
                H[q * restart + j] = cs[q] * a + sn[q] * c;
                H[(q + 1) * restart + j] = -sn[q] * a + cs[q] * c;
            }
            double a = H[j * restart + j], c = H[(j + 1) * restart + j];
            double den = sqrt(a * a + c * c);
            if (den == 0.0) { cs[j] = 1.0; sn[j] = 0.0; }
            else { cs[j] = a / den; sn[j] = c / den; }
            H[j * restart + j] = cs[j] * a + sn[j] * c;
            H[(j + 1) * restart + j] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            its++;
            jdone = j + 1;
            rnorm = fabs(g[j + 1]);
            if (isnan(rnorm)) { reason = -4; break; }
            if (rnorm <= ttol) { reason = (rnorm < abstol) ? 3 : 2; break; }
            if (hn == 0.0) { reason = 2; break; } /* happy breakdown */
            if (its >= max_it) { reason = -3; break; }
        }
        /* x += V y, H y = g */
        for (int q = jdone - 1; q >= 0; --q) {
            double t = g[q];
            for (int c2 = q + 1; c2 < jdone; ++c2) t -= H[q * restart + c2] * yv[c2];
            yv[q] = (H[q * restart + q] != 0.0) ? t / H[q * restart + q] : 0.0;
        }
#pragma omp parallel for schedule(static)
        for (long r = 0; r < n; ++r) {
            double t = x[r];
            for (int q = 0; q < jdone; ++q) t += yv[q] * V[(size_t)q * n + r];
            x[r] = t;
        }
        if (reason != 0) break;
    }
    free(H); free(cs); free(sn); free(g); free(yv);
    *its_out = its;
    *rel_out = (snorm > 0.0) ? rnorm / snorm : rnorm;
    return reason;
}

/* ------------------------------------------------------------------------ */
/* Multigrid-preconditioned CG on the Pore block of the pressure system (test and baseline
   infrastructure: the stand-in for the algebraic-multigrid preconditioner the reference's
   production job scripts select for this system, -press_pc_type hypre -press_pc_hypre_type
   boomeramg, hpc_cx3_test.pbs:44-51; hypre is not part of the reference and is not
   restated). The unknowns S are the normal Pore rows (diagonal -sum of links < 0). With
   them the operator is M = -A_SS in "excess + Laplacian" form, (M x)_r = e_r x_r +
   sum over S neighbours of c (x_r - x_nb), c the row's link coefficient (the same seen from
   both ends) and e_r the links of r to rows outside S. Levels coarsen 2x2x2 by aggregation
   with Galerkin operators of the same form (sums of the children's excess and of the links
   crossing a coarse face); a symmetric V-cycle (two damped Jacobi sweeps before and after,
   a fixed number of sweeps on the coarsest level) preconditions CG. */

typedef struct mg_level {
    int I, J, K;
    long n;
    int8_t* mem;     /* member cell */
    int8_t* owned;   /* member restricted into its coarse cell (of the block's majority component) */
    int* comp;       /* strong component of a member (-1 otherwise) */
    double* e;       /* excess */
    double* c[3];    /* +i, +j, +k links */
    double* invd;    /* 1 / (e + sum of links) */
    double *x, *b, *t;
} mg_level;

typedef struct mg_hier {
    int nlev;
    mg_level L[24];
} mg_hier;

static void mg_level_alloc(mg_level* l, int I, int J, int K) {
    l->I = I; l->J = J; l->K = K;
    l->n = (long)I * J * K;
    l->mem = (int8_t*)xcalloc(l->n, 1);
    l->owned = (int8_t*)xcalloc(l->n, 1);
    l->comp = (int*)xcalloc(l->n, sizeof(int));
    l->e = (double*)xcalloc(l->n, sizeof(double));
    for (int d = 0; d < 3; ++d) l->c[d] = (double*)xcalloc(l->n, sizeof(double));
    l->invd = (double*)xcalloc(l->n, sizeof(double));
    l->x = (double*)xcalloc(l->n, sizeof(double));
    l->b = (double*)xcalloc(l->n, sizeof(double));
    l->t = (double*)xcalloc(l->n, sizeof(double));
}

static void mg_free(mg_hier* h) {
    for (int q = 0; q < h->nlev; ++q) {
        mg_level* l = &h->L[q];
        free(l->mem); free(l->owned); free(l->comp); free(l->e); free(l->invd); free(l->x); free(l->b); free(l->t);
        for (int d = 0; d < 3; ++d) free(l->c[d]);
    }
    h->nlev = 0;
}

static void mg_invd(mg_level* l) {
    const int I = l->I, J = l->J, K = l->K;
    const long JK = (long)J * K;
#pragma omp parallel for schedule(static)
    for (long r = 0; r < l->n; ++r) {
        if (!l->mem[r]) { l->invd[r] = 0.0; continue; }
        int i = (int)(r / JK), j = (int)((r / K) % J), k = (int)(r % K);
        double d = l->e[r] + l->c[0][r] + l->c[1][r] + l->c[2][r];
        if (i > 0) d += l->c[0][r - JK];
        if (j > 0) d += l->c[1][r - K];
        if (k > 0) d += l->c[2][r - 1];
        (void)I;
        l->invd[r] = d > 0.0 ? 1.0 / d : 0.0;
    }
}

/* y = M x on a level (members only; x is 0 off the members) */
static void mg_apply(const mg_level* l, const double* x, double* y) {
    const int J = l->J, K = l->K;
    const long JK = (long)J * K;
#pragma omp parallel for schedule(static)
    for (long r = 0; r < l->n; ++r) {
        if (!l->mem[r]) { y[r] = 0.0; continue; }
        int i = (int)(r / JK), j = (int)((r / K) % J), k = (int)(r % K);
        const double xr = x[r];
        double a = l->e[r] * xr;
        a += l->c[0][r] * (xr - x[r + (i + 1 < l->I ? JK : 0)]);
        a += l->c[1][r] * (xr - x[r + (j + 1 < J ? K : 0)]);
        a += l->c[2][r] * (xr - x[r + (k + 1 < K ? 1 : 0)]);
        if (i > 0) a += l->c[0][r - JK] * (xr - x[r - JK]);
        if (j > 0) a += l->c[1][r - K] * (xr - x[r - K]);
        if (k > 0) a += l->c[2][r - 1] * (xr - x[r - 1]);
        y[r] = a;
    }
}

/* Strong components of a level's members: a link is strong when c > 1e-3 sqrt(d_i d_j), d the
   cell's diagonal (e + its links). Union-find with path halving, roots = smallest index. */
static int uf_find(int* p, int x) {
    while (p[x] != x) {
        p[x] = p[p[x]];
        x = p[x];
    }
    return x;
}

static void mg_components(mg_level* l) {
    const long JK = (long)l->J * l->K;
    int* p = l->comp;
    for (long r = 0; r < l->n; ++r) p[r] = l->mem[r] ? (int)r : -1;
    for (long r = 0; r < l->n; ++r) {
        if (!l->mem[r]) continue;
        int i = (int)(r / JK), j = (int)((r / l->K) % l->J), k = (int)(r % l->K);
        const long off[3] = {JK, l->K, 1};
        const int ok[3] = {i + 1 < l->I, j + 1 < l->J, k + 1 < l->K};
        for (int d = 0; d < 3; ++d) {
            if (!ok[d]) continue;
            long nb = r + off[d];
            if (!l->mem[nb] || !(l->invd[r] > 0.0) || !(l->invd[nb] > 0.0)) continue;
            /* c^2 > 1e-6 d_r d_nb  <=>  c^2 invd_r invd_nb > 1e-6 */
            const double c = l->c[d][r];
            if (c * c * l->invd[r] * l->invd[nb] > 1e-6) {
                int a = uf_find(p, (int)r), b = uf_find(p, (int)nb);
                if (a != b) {
                    if (a < b) p[b] = a;
                    else p[a] = b;
                }
            }
        }
    }
    for (long r = 0; r < l->n; ++r)
        if (l->mem[r]) p[r] = uf_find(p, (int)r);
}

/* Coarsening 2x2x2: each block is owned by the strong component holding most of its member
   cells (ties: the smallest id); only those cells are restricted into the coarse cell and
   corrected from it. Galerkin operator of that piecewise-constant prolongation in the same
   form: coarse excess = the owned cells' excess plus their links to cells outside every
   aggregate or in their own block but not owned; coarse links = the links between owned
   cells of adjacent blocks. */
static long mg_cell(const mg_level* l, int i, int j, int k) { return (long)k + (long)l->K * ((long)j + (long)l->J * i); }

static void mg_coarsen(mg_level* f, mg_level* c) {
    mg_level_alloc(c, (f->I + 1) / 2, (f->J + 1) / 2, (f->K + 1) / 2);
    const long cJK = (long)c->J * c->K;
    /* pass 1: owner component per block, owned flags on the fine level */
#pragma omp parallel for schedule(static)
    for (long C = 0; C < c->n; ++C) {
        const int ci = (int)(C / cJK), cj = (int)((C / c->K) % c->J), ck = (int)(C % c->K);
        int ids[8], cnt[8], nid = 0;
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                for (int g = 0; g < 2; ++g) {
                    const int i = 2 * ci + a, j = 2 * cj + b, k = 2 * ck + g;
                    if (i >= f->I || j >= f->J || k >= f->K) continue;
                    const long r = mg_cell(f, i, j, k);
                    if (!f->mem[r]) continue;
                    int q = 0;
                    while (q < nid && ids[q] != f->comp[r]) q++;
                    if (q == nid) { ids[nid] = f->comp[r]; cnt[nid] = 0; nid++; }
                    cnt[q]++;
                }
        int owner = -1, best = 0;
        for (int q = 0; q < nid; ++q)
            if (cnt[q] > best || (cnt[q] == best && ids[q] < owner)) { best = cnt[q]; owner = ids[q]; }
        c->mem[C] = (int8_t)(nid > 0);
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                for (int g = 0; g < 2; ++g) {
                    const int i = 2 * ci + a, j = 2 * cj + b, k = 2 * ck + g;
                    if (i >= f->I || j >= f->J || k >= f->K) continue;
                    const long r = mg_cell(f, i, j, k);
                    f->owned[r] = (int8_t)(f->mem[r] && f->comp[r] == owner);
                }
    }
    /* pass 2: coarse excess and links */
    const long fJK = (long)f->J * f->K;
#pragma omp parallel for schedule(static)
    for (long C = 0; C < c->n; ++C) {
        if (!c->mem[C]) continue;
        const int ci = (int)(C / cJK), cj = (int)((C / c->K) % c->J), ck = (int)(C % c->K);
        double ex = 0.0, cf[3] = {0.0, 0.0, 0.0};
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                for (int g = 0; g < 2; ++g) {
                    const int i = 2 * ci + a, j = 2 * cj + b, k = 2 * ck + g;
                    if (i >= f->I || j >= f->J || k >= f->K) continue;
                    const long r = mg_cell(f, i, j, k);
                    if (!f->owned[r]) continue;
                    ex += f->e[r];
                    const int pos[3] = {i, j, k}, lim[3] = {f->I, f->J, f->K}, side[3] = {a, b, g};
                    const long off[3] = {fJK, f->K, 1};
                    for (int d = 0; d < 3; ++d) {
                        /* + neighbour */
                        if (pos[d] + 1 < lim[d] && f->mem[r + off[d]] && f->c[d][r] != 0.0) {
                            const long nb = r + off[d];
                            if (side[d] == 1 && f->owned[nb]) cf[d] += f->c[d][r];  /* into the + block */
                            else if (side[d] == 1 || !f->owned[nb]) ex += f->c[d][r]; /* out of every aggregate */
                        }
                        /* - neighbour */
                        if (pos[d] > 0 && f->mem[r - off[d]] && f->c[d][r - off[d]] != 0.0) {
                            const long nb = r - off[d];
                            if (side[d] == 0 && f->owned[nb]) { /* the - block's link, counted there */ }
                            else if (side[d] == 0 || !f->owned[nb]) ex += f->c[d][nb];
                        }
                    }
                }
        c->e[C] = ex;
        for (int d = 0; d < 3; ++d) c->c[d][C] = cf[d];
    }
    mg_invd(c);
}

static void mg_build(mg_hier* h, const lso_state* s, const ell_sys* e, const int8_t* cls) {
    mg_free(h);
    mg_level* l0 = &h->L[0];
    mg_level_alloc(l0, s->I, s->J, s->K);
    const int I = s->I, J = s->J, K = s->K;
    const long JK = (long)s->JK;
#pragma omp parallel for schedule(static)
    for (long r = 0; r < (long)s->N; ++r) {
        if (cls[r] != 1) continue;
        int i = (int)(r / JK), j = (int)((r / K) % J), k = (int)(r % K);
        l0->mem[r] = 1;
        double ex = -e->diag[r];
        long nb[6] = {r + JK, r - JK, r + K, r - K, r + 1, r - 1};
        int val[6] = {i + 1 < I, i > 0, j + 1 < J, j > 0, k + 1 < K, k > 0};
        for (int d = 0; d < 6; ++d)
            if (val[d] && cls[nb[d]] == 1) ex -= e->A[d][r];
        l0->e[r] = ex > 0.0 ? ex : 0.0;
        l0->c[0][r] = (val[0] && cls[nb[0]] == 1) ? e->A[0][r] : 0.0;
        l0->c[1][r] = (val[2] && cls[nb[2]] == 1) ? e->A[2][r] : 0.0;
        l0->c[2][r] = (val[4] && cls[nb[4]] == 1) ? e->A[4][r] : 0.0;
    }
    mg_invd(l0);
    h->nlev = 1;
    while (h->nlev < 24) {
        mg_level* f = &h->L[h->nlev - 1];
        if (f->n <= 512 || (f->I <= 2 && f->J <= 2 && f->K <= 2)) break;
        mg_components(f);
        mg_coarsen(f, &h->L[h->nlev]);
        h->nlev++;
    }
}

static void mg_jacobi(mg_level* l, const double* b, double* x, double* t, int sweeps, double w) {
    for (int q = 0; q < sweeps; ++q) {
        mg_apply(l, x, t);
#pragma omp parallel for schedule(static)
        for (long r = 0; r < l->n; ++r)
            if (l->mem[r]) x[r] += w * l->invd[r] * (b[r] - t[r]);
    }
}

/* z = V(r): one V-cycle from z = 0 (a fixed symmetric linear operator) */
static void mg_vcycle(mg_hier* h, int q, const double* b, double* x) {
    mg_level* l = &h->L[q];
    memset(x, 0, sizeof(double) * l->n);
    const double w = 0.6;
    if (q == h->nlev - 1) {
        mg_jacobi(l, b, x, l->t, 40, w);
        return;
    }
    mg_jacobi(l, b, x, l->t, 2, w);
    mg_apply(l, x, l->t);
    mg_level* c = &h->L[q + 1];
    const long fJK = (long)l->J * l->K, cJK = (long)c->J * c->K;
#pragma omp parallel for schedule(static)
    for (long C = 0; C < c->n; ++C) {
        const int ci = (int)(C / cJK), cj = (int)((C / c->K) % c->J), ck = (int)(C % c->K);
        double acc = 0.0;
        for (int a = 0; a < 2; ++a)
            for (int bb = 0; bb < 2; ++bb)
                for (int g = 0; g < 2; ++g) {
                    const int i = 2 * ci + a, j = 2 * cj + bb, k = 2 * ck + g;
                    if (i >= l->I || j >= l->J || k >= l->K) continue;
                    const long r = (long)k + (long)l->K * ((long)j + (long)l->J * i);
                    if (l->owned[r]) acc += b[r] - l->t[r];
                }
        c->b[C] = acc;
    }
    mg_vcycle(h, q + 1, c->b, c->x);
#pragma omp parallel for schedule(static)
    for (long r = 0; r < l->n; ++r) {
        if (!l->owned[r]) continue;
        int i = (int)(r / fJK), j = (int)((r / l->K) % l->J), k = (int)(r % l->K);
        long C = (long)(k / 2) + (long)c->K * ((long)(j / 2) + (long)c->J * (i / 2));
        x[r] += 1.8 * c->x[C];
    }
    /* post-smoothing from the corrected iterate (symmetric with the pre-smoothing) */
    mg_jacobi(l, b, x, l->t, 2, w);
}

/* Pressure solve on the Pore block (modes LSO_SOLVE_PCG and LSO_SOLVE_PRODUCTION). Identity
   rows take their value; S solves M x_S = A_SQ x_Q - b_S by multigrid-preconditioned CG until
   the Jacobi-scaled residual of the S rows is below rtol times the Jacobi-scaled norm of b
   (the test the GPU solver and PETSc's Jacobi-preconditioned GMRES apply); the floored Pore
   rows F (src/Simulation.cpp:783-786: diagonal +1e-16) are then evaluated from their own
   row, and the pair is repeated until the floored values settle (their links are ~1e-22 or
   smaller). */
static int pressure_pcg(lso_state* s, const ell_sys* e, double* x, double rtol, int max_it, int* its_out,
                        double* rel_out) {
    const long n = (long)s->N;
    const int I = s->I, J = s->J, K = s->K;
    const long JK = (long)s->JK;
    double* rhs = (double*)xcalloc(n, sizeof(double));
    double* rr = (double*)xcalloc(n, sizeof(double));
    double* z = (double*)xcalloc(n, sizeof(double));
    double* pp = (double*)xcalloc(n, sizeof(double));
    double* q = (double*)xcalloc(n, sizeof(double));
    int8_t* cls = (int8_t*)xcalloc(n, 1); /* 0 fixed/empty, 1 normal Pore (S), 2 floored (F) */
    double bden = 0.0;
    for (long r = 0; r < n; ++r) {
        if (e->kind[r] == 1) { x[r] = e->b[r]; cls[r] = 0; }
        else if (e->kind[r] == 2) cls[r] = (e->diag[r] < 0.0) ? 1 : 2;
        if (e->diag[r] != 0.0) {
            double t = e->b[r] / e->diag[r];
            bden += t * t;
        }
    }
    mg_hier h;
    memset(&h, 0, sizeof(h));
    mg_build(&h, s, e, cls);
    mg_level* l0 = &h.L[0];
    int its = 0, reason = 2;
    const double stop = rtol * rtol * (bden > 0.0 ? bden : 1.0);
    for (int outer = 0; outer < 8; ++outer) {
        /* rhs_S = -(b_S - sum over non-S neighbours of A x) */
#pragma omp parallel for schedule(static)
        for (long r = 0; r < n; ++r) {
            if (cls[r] != 1) { rhs[r] = 0.0; x[r] = (cls[r] == 1) ? x[r] : x[r]; continue; }
            int i = (int)(r / JK), j = (int)((r / K) % J), k = (int)(r % K);
            double a = e->b[r];
            long nb[6] = {r + JK, r - JK, r + K, r - K, r + 1, r - 1};
            int val[6] = {i + 1 < I, i > 0, j + 1 < J, j > 0, k + 1 < K, k > 0};
            for (int d = 0; d < 6; ++d)
                if (val[d] && cls[nb[d]] != 1) a -= e->A[d][r] * x[nb[d]];
            rhs[r] = -a;
        }
        /* the S part of x as a level-0 vector (zero elsewhere) */
#pragma omp parallel for schedule(static)
        for (long r = 0; r < n; ++r) q[r] = (cls[r] == 1) ? x[r] : 0.0;
        mg_apply(l0, q, z);
        double rz = 0.0, rn = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : rn)
        for (long r = 0; r < n; ++r) {
            rr[r] = (cls[r] == 1) ? rhs[r] - z[r] : 0.0;
            const double t = rr[r] / e->diag[r];
            if (cls[r] == 1) rn += t * t;
        }
        if (rn > stop) {
            mg_vcycle(&h, 0, rr, z);
#pragma omp parallel for schedule(static) reduction(+ : rz)
            for (long r = 0; r < n; ++r) {
                pp[r] = z[r];
                rz += rr[r] * z[r];
            }
        }
        while (rn > stop && its < max_it) {
            mg_apply(l0, pp, q);
            double pq = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : pq)
            for (long r = 0; r < n; ++r) pq += pp[r] * q[r];
            if (!(pq > 0.0)) { reason = (pq == pq) ? -3 : -4; break; }
            const double alpha = rz / pq;
            rn = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : rn)
            for (long r = 0; r < n; ++r) {
                if (cls[r] != 1) continue;
                x[r] += alpha * pp[r];
                rr[r] -= alpha * q[r];
                const double t = rr[r] / e->diag[r];
                rn += t * t;
            }
            its++;
            if (!(rn == rn)) { reason = -4; break; }
            if (rn <= stop) break;
            mg_vcycle(&h, 0, rr, z);
            double rzn = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : rzn)
            for (long r = 0; r < n; ++r) rzn += rr[r] * z[r];
            const double beta = rzn / rz;
            rz = rzn;
#pragma omp parallel for schedule(static)
            for (long r = 0; r < n; ++r) pp[r] = z[r] + beta * pp[r];
        }
        if (reason < 0) break;
        if (rn > stop) { reason = -3; break; }
        /* floored rows from their own row */
        double change = 0.0, mag = 0.0;
        for (long r = 0; r < n; ++r) {
            if (cls[r] != 2) continue;
            int i = (int)(r / JK), j = (int)((r / K) % J), k = (int)(r % K);
            double a = e->b[r];
            long nb[6] = {r + JK, r - JK, r + K, r - K, r + 1, r - 1};
            int val[6] = {i + 1 < I, i > 0, j + 1 < J, j > 0, k + 1 < K, k > 0};
            for (int d = 0; d < 6; ++d)
                if (val[d]) a -= e->A[d][r] * x[nb[d]];
            double v = a / e->diag[r];
            change = smax(change, fabs(v - x[r]));
            mag = smax(mag, fabs(v));
            x[r] = v;
        }
        if (change <= 1e-15 * smax(mag, 1e-300)) break;
    }
    mg_free(&h);
    free(rhs); free(rr); free(z); free(pp); free(q); free(cls);
    *its_out = its;
    *rel_out = scaled_residual(s, e, e->b, x);
    return reason;
}

/* Jacobi-scaled relative residual of the current x: ||B (b - A x)|| / ||B b||. */
static double scaled_residual(lso_state* s, const ell_sys* e, const double* b, const double* x) {
    const long n = (long)s->N;
    double* w = (double*)xcalloc(n, sizeof(double));
    ell_apply(s, e, x, w);
    double num = 0.0, den = 0.0;
#pragma omp parallel for reduction(+ : num, den) schedule(static)
    for (long r = 0; r < n; ++r) {
        double di = (e->diag[r] != 0.0) ? 1.0 / e->diag[r] : 1.0;
        double t = di * (b[r] - w[r]);
        double u = di * b[r];
        num += t * t;
        den += u * u;
    }
    free(w);
    return den > 0.0 ? sqrt(num / den) : sqrt(num);
}

/* Solve per the configured mode; fills info like the reference's log (S.cpp:823-849). */
/* REFERENCE mode uses the tolerances the reference hard-codes (KSPSetTolerances(ksp,
   1e-6, default, default, 10000), S.cpp:156) unless the solver config overrides them;
   TIGHT mode uses the config (default rtol 1e-13). The ls_params tolerances are used
   when the config gives none. */
static int run_solve(lso_state* s, const ell_sys* e, double* x, double rtol_param,
                     int maxit_param, int solves, ls_solve_info* info, int spd) {
    double rtol, max_it_d;
    if (s->cfg.mode == LSO_SOLVE_REFERENCE) {
        rtol = (s->cfg.rtol > 0.0) ? s->cfg.rtol : 1e-6;
        max_it_d = (s->cfg.max_it > 0) ? s->cfg.max_it : 10000;
    } else if (s->cfg.mode == LSO_SOLVE_PRODUCTION) {
        rtol = (s->cfg.rtol > 0.0) ? s->cfg.rtol : (rtol_param > 0.0 ? rtol_param : 1e-6);
        max_it_d = (s->cfg.max_it > 0) ? s->cfg.max_it : (maxit_param > 0 ? maxit_param : 10000);
    } else {
        rtol = (s->cfg.rtol > 0.0) ? s->cfg.rtol : (rtol_param > 0.0 ? rtol_param : 1e-13);
        max_it_d = (s->cfg.max_it > 0) ? s->cfg.max_it : (maxit_param > 0 ? maxit_param : 100000);
    }
    int max_it = (int)max_it_d;
    int restart = (s->cfg.mode == LSO_SOLVE_REFERENCE || s->cfg.mode == LSO_SOLVE_PRODUCTION)
                      ? 30 : (s->cfg.restart > 0 ? s->cfg.restart : 30);
    int its = 0, reason = 0;
    double rel = 0.0;
    int total = 0;
    for (int q = 0; q < solves; ++q) {
        if (spd && (s->cfg.mode == LSO_SOLVE_PCG || s->cfg.mode == LSO_SOLVE_PRODUCTION))
            reason = pressure_pcg(s, e, x, rtol, max_it, &its, &rel);
        else reason = gmres(s, e, e->b, x, restart, rtol, max_it, &its, &rel);
        total += its;
    }
    if (info) {
        double mn = x[0], mx = x[0];
        for (size_t r = 1; r < s->N; ++r) {
            if (x[r] < mn) mn = x[r];
            if (x[r] > mx) mx = x[r];
        }
        info->iterations = total;
        info->outer_iterations = solves;
        info->converged = reason > 0;
        info->reason = reason;
        info->rel_residual = scaled_residual(s, e, e->b, x);
        info->min_value = mn;
        info->max_value = mx;
    }
    return reason > 0;
}

static int solves_per_call(const lso_state* s) {
    /* KSPSolve runs twice per pressure/conc/acid solve (S.cpp:823-825, 1262-1264, 2188-2190). */
    return (s->cfg.mode == LSO_SOLVE_REFERENCE || s->cfg.mode == LSO_SOLVE_PRODUCTION) ? 2 : 1;
}

static double* solution_slots(lso_state* s, double* field) {
    return field + (s->p.compat_shift ? s->JK : 0);
}

/* ------------------------------------------------------------------------ */
/* pressure                                                                  */

/* Simulation::setupPressureEqns, S.cpp:658-798. With bc_mode LS_BC_FLOW_I (an extension)
 * the Pore voxels of the planes i = 0 and i = I-1 are identity rows holding p_inlet and
 * p_outlet; every other row is the reference's. */
void lso_setup_pressure(lso_state* s, double current_time) {
    const double ramp_duration = 3600.0;
    double effective_top_pressure = s->p.top_pressure;
    if (current_time < ramp_duration)
        effective_top_pressure = s->p.top_pressure * (current_time / ramp_duration) + 1e-6;
    const double evap = s->p.evaporative_flux, dx = s->p.dx;
    ell_sys* e = &s->press;
    const int I = s->I, J = s->J, K = s->K;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < I; ++i)
        for (int j = 0; j < J; ++j)
            for (int k = 0; k < K; ++k) {
                size_t r = IDX(s, i, j, k);
                for (int d = 0; d < 6; ++d) e->A[d][r] = 0.0;
                e->diag[r] = 0.0;
                e->b[r] = 0.0;
                e->kind[r] = 0;
                uint16_t t = s->label[r];
                if (t == AIR || t == ROCK || t == SULPHIDE || t == PRECIPITATE) {
                    e->diag[r] = 1.0;
                    e->kind[r] = 1;
                    if (t == AIR) {
                        int is_surface = 0;
                        for (int d = 0; d < 6; ++d) {
                            size_t nb;
                            if (NB(s, i, j, k, d, &nb) && s->label[nb] != AIR) is_surface = 1;
                        }
                        e->b[r] = 0.0 + (is_surface ? effective_top_pressure : 0.0);
                    }
                } else if (t == PORE && s->p.bc_mode == LS_BC_FLOW_I && (i == 0 || i == I - 1)) {
                    e->diag[r] = 1.0;
                    e->b[r] = 0.0 + (i == 0 ? s->p.p_inlet : s->p.p_outlet);
                    e->kind[r] = 1;
                } else if (t == PORE) {
                    double diagonal_term = 0.0, source_term = 0.0;
                    for (int d = 0; d < 6; ++d) {
                        size_t nb;
                        if (!NB(s, i, j, k, d, &nb)) continue;
                        double K_neighbor;
                        if (s->label[nb] == AIR) {
                            source_term -= evap * dx;
                            K_neighbor = 1.0e-9;
                        } else {
                            K_neighbor = s->perm[nb];
                        }
                        double K_self = smax(s->perm[r], 1e-25);
                        double K_neigh = smax(K_neighbor, 1e-25);
                        double K_avg = (2.0 * K_self * K_neigh) / (K_self + K_neigh);
                        double coeff = K_avg / s->visc[r];
                        e->A[d][r] = coeff;
                        diagonal_term -= coeff;
                    }
                    if (fabs(diagonal_term) < 1e-16) diagonal_term = 1e-16;
                    e->diag[r] = diagonal_term;
                    e->b[r] = 0.0 + source_term;
                    e->kind[r] = 2;
                }
                /* any other label: the reference inserts nothing -> an empty row */
            }
}

/* Simulation::solvePressure, S.cpp:804-855. */
int lso_solve_pressure(lso_state* s, ls_solve_info* info) {
    double* x = solution_slots(s, s->P);
    return run_solve(s, &s->press, x, s->p.press_rtol, s->p.press_max_it, solves_per_call(s), info, 1);
}

void lso_pressure_apply(const lso_state* s, const double* x, double* y) { ell_apply(s, &s->press, x, y); }
void lso_pressure_rhs(const lso_state* s, double* b) { memcpy(b, s->press.b, s->N * sizeof(double)); }
void lso_pressure_rowkind(const lso_state* s, int8_t* kind) { memcpy(kind, s->press.kind, s->N); }
void lso_pressure_diag(const lso_state* s, double* d) { memcpy(d, s->press.diag, s->N * sizeof(double)); }

/* ------------------------------------------------------------------------ */
/* flux and saturation                                                       */

/* Simulation::calculateFlux, S.cpp:866-953 (np=1: one-sided at the global faces). */
void lso_calculate_flux(lso_state* s) {
    const double dx = s->p.dx, mcg = s->p.max_cap_grad;
    const int I = s->I, J = s->J, K = s->K;
    const double* P = s->P;
    const double* C = s->pc;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < I; ++i)
        for (int j = 0; j < J; ++j)
            for (int k = 0; k < K; ++k) {
                size_t r = IDX(s, i, j, k);
                size_t xp = r + s->JK, xm = r - s->JK, yp = r + K, ym = r - K, zp = r + 1, zm = r - 1;
                double gPx, gPy, gPz, gCx, gCy, gCz;
                if (i == 0) gPx = (P[xp] - P[r]) / dx;
                else if (i == I - 1) gPx = (P[r] - P[xm]) / dx;
                else gPx = (P[xp] - P[xm]) / (2.0 * dx);
                if (j == 0) gPy = (P[yp] - P[r]) / dx;
                else if (j == J - 1) gPy = (P[r] - P[ym]) / dx;
                else gPy = (P[yp] - P[ym]) / (2.0 * dx);
                if (k == 0) gPz = (P[zp] - P[r]) / dx;
                else if (k == K - 1) gPz = (P[r] - P[zm]) / dx;
                else gPz = (P[zp] - P[zm]) / (2.0 * dx);
                if (i == 0) gCx = (C[xp] - C[r]) / dx;
                else if (i == I - 1) gCx = (C[r] - C[xm]) / dx;
                else gCx = (C[xp] - C[xm]) / (2.0 * dx);
                if (j == 0) gCy = (C[yp] - C[r]) / dx;
                else if (j == J - 1) gCy = (C[r] - C[ym]) / dx;
                else gCy = (C[yp] - C[ym]) / (2.0 * dx);
                if (k == 0) gCz = (C[zp] - C[r]) / dx;
                else if (k == K - 1) gCz = (C[r] - C[zm]) / dx;
                else gCz = (C[zp] - C[zm]) / (2.0 * dx);
                gCx = smax(-mcg, smin(mcg, gCx));
                gCy = smax(-mcg, smin(mcg, gCy));
                gCz = smax(-mcg, smin(mcg, gCz));
                double transmissivity = s->perm[r] / s->visc[r];
                const double rho_g = 1000.0 * 9.81;
                double lx = gPx - gCx, ly = gPy - gCy, lz = gPz - gCz;
                s->fx[r] = -transmissivity * (lx - rho_g);
                s->fy[r] = -transmissivity * ly;
                s->fz[r] = -transmissivity * lz;
            }
}

static inline int sat_inactive(uint16_t t) {
    return t == AIR || t == ROCK || t == SULPHIDE || t == PRECIPITATE;
}

/* Face-averaged flux divergence of S.cpp:1691-1706 plus the evaporative sink of
   S.cpp:1709-1727 (Pore only). */
static void sat_rates(const lso_state* s, int i, int j, int k, double* div_out, double* evap_out) {
    size_t r = IDX(s, i, j, k), nb;
    const double* fx = s->fx;
    const double* fy = s->fy;
    const double* fz = s->fz;
    double q_xp = NB(s, i, j, k, 0, &nb) ? (fx[r] + fx[nb]) / 2.0 : 0.0;
    double q_xm = NB(s, i, j, k, 1, &nb) ? (fx[r] + fx[nb]) / 2.0 : 0.0;
    double q_yp = NB(s, i, j, k, 2, &nb) ? (fy[r] + fy[nb]) / 2.0 : 0.0;
    double q_ym = NB(s, i, j, k, 3, &nb) ? (fy[r] + fy[nb]) / 2.0 : 0.0;
    double q_zp = NB(s, i, j, k, 4, &nb) ? (fz[r] + fz[nb]) / 2.0 : 0.0;
    double q_zm = NB(s, i, j, k, 5, &nb) ? (fz[r] + fz[nb]) / 2.0 : 0.0;
    double div_q = ((q_xp - q_xm) + (q_yp - q_ym) + (q_zp - q_zm)) / s->p.dx;
    double evap_sink = 0.0;
    if (s->label[r] == PORE) {
        int air_faces = 0;
        for (int d = 0; d < 6; ++d)
            if (NB(s, i, j, k, d, &nb) && s->label[nb] == AIR) air_faces++;
        evap_sink = (air_faces * s->p.evaporative_flux) / s->p.dx;
    }
    *div_out = div_q;
    *evap_out = evap_sink;
}

/* Simulation::updateSaturation, S.cpp:1672-1856.
 * div q and the evaporative sink of a voxel do not change between sub-steps (they read
 * only flux and labels), so the reference's num_steps sweeps equal num_steps repetitions
 * of s <- clamp(s - dt_sub/phi * (div_q + evap)) per voxel, done here voxel by voxel.
 * Inactive voxels (Air/Rock/Sulphide/Precipitate) end as 0.0: the reference writes only
 * active voxels into a freshly allocated array (S.cpp:1781-1848), leaving the rest
 * indeterminate; 0.0 is what a fresh page holds. */
void lso_update_saturation(lso_state* s, double dt, ls_substep_info* info) {
    const int I = s->I, J = s->J, K = s->K;
    double max_div_q = 0.0;
    for (int k = 0; k < K; ++k)
        for (int j = 0; j < J; ++j)
            for (int i = 0; i < I; ++i) {
                size_t r = IDX(s, i, j, k);
                if (sat_inactive(s->label[r])) continue;
                double div_q, evap_sink;
                sat_rates(s, i, j, k, &div_q, &evap_sink);
                double total_rate = fabs(div_q) + evap_sink;
                if (total_rate > max_div_q) max_div_q = total_rate;
            }
    const double max_dsat = 0.1;
    double dt_safe = dt;
    if (max_div_q > 1e-20) dt_safe = (max_dsat * s->p.porosity) / max_div_q;
    double calculated_steps = ceil(dt / dt_safe);
    int num_steps = 1;
    if (isinf(calculated_steps) || isnan(calculated_steps)) num_steps = 1000;
    else if (calculated_steps > 1000) num_steps = 1000;
    else if (calculated_steps > 1.0) num_steps = (int)calculated_steps;
    double dt_sub = dt / num_steps;
    double dt_sub_over_phi = dt_sub / s->p.porosity;
    if (info) {
        info->max_rate = max_div_q;
        info->num_steps = num_steps;
        info->dt_sub = dt_sub;
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < I; ++i)
        for (int j = 0; j < J; ++j)
            for (int k = 0; k < K; ++k) {
                size_t r = IDX(s, i, j, k);
                if (sat_inactive(s->label[r])) {
                    s->sat[r] = 0.0;
                    continue;
                }
                double div_q, evap_sink;
                sat_rates(s, i, j, k, &div_q, &evap_sink);
                double sv = s->sat[r];
                for (int step = 0; step < num_steps; ++step) {
                    double new_sat = sv - dt_sub_over_phi * (div_q + evap_sink);
                    sv = smax(0.0, smin(1.0, new_sat));
                }
                s->sat[r] = sv;
            }
    /* the extra top plane of the fresh array is indeterminate as well */
    memset(s->sat + s->N, 0, s->JK * sizeof(double));
}

/* Simulation::setupSaturationEqns, S.cpp:1858-1967. */
void lso_setup_saturation(lso_state* s, double dt) {
    const double inv_dt = 1.0 / dt;
    const double phi = s->p.porosity, dx = s->p.dx;
    ell_sys* e = &s->satsys;
    const int I = s->I, J = s->J, K = s->K;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < I; ++i)
        for (int j = 0; j < J; ++j)
            for (int k = 0; k < K; ++k) {
                size_t r = IDX(s, i, j, k), nb;
                for (int d = 0; d < 6; ++d) e->A[d][r] = 0.0;
                uint16_t t = s->label[r];
                if (sat_inactive(t)) {
                    e->diag[r] = 1.0;
                    e->b[r] = 0.0 + s->sat[r];
                    e->kind[r] = 1;
                    continue;
                }
                int air_faces = 0;
                for (int d = 0; d < 6; ++d)
                    if (NB(s, i, j, k, d, &nb) && s->label[nb] == AIR) air_faces++;
                double evap_sink = (air_faces * s->p.evaporative_flux) / dx;
                double coeff_self = phi * inv_dt;
                double explicit_rhs = (phi * inv_dt * s->sat[r]) - evap_sink;
                const double* fl[3] = {s->fx, s->fy, s->fz};
                for (int d = 0; d < 6; ++d) {
                    if (!NB(s, i, j, k, d, &nb)) continue;
                    const double* f = fl[d / 2];
                    double q = (f[r] + f[nb]) / 2.0;
                    double q_face_outward = (d % 2 == 0) ? q : -q;
                    if (q_face_outward > 0) {
                        double v_eff = q_face_outward / smax(s->sat[r], 1e-6);
                        coeff_self += v_eff / dx;
                    } else {
                        double v_eff = q_face_outward / smax(s->sat[nb], 1e-6);
                        e->A[d][r] = v_eff / dx;
                    }
                }
                e->diag[r] = coeff_self;
                e->b[r] = 0.0 + explicit_rhs;
                e->kind[r] = 2;
            }
}

/* Simulation::solveSaturation, S.cpp:1969-2053 (one KSPSolve). */
int lso_solve_saturation(lso_state* s, ls_solve_info* info, int* physics_valid) {
    double* x = solution_slots(s, s->sat);
    ls_solve_info loc;
    int ok = run_solve(s, &s->satsys, x, s->p.sat_rtol, s->p.sat_max_it, 1, &loc, 0);
    int valid = 1;
    if (loc.max_value > 1.05 || loc.min_value < -0.05) valid = 0;
    if (valid) {
        /* the clamp runs over voxel slots, not over the solution slots (S.cpp:2034-2046) */
        for (size_t r = 0; r < s->N; ++r) s->sat[r] = smax(0.0, smin(1.0, s->sat[r]));
    }
    s->physics_valid = valid;
    if (physics_valid) *physics_valid = valid;
    if (info) *info = loc;
    return ok;
}

/* Simulation::handleSurfaceEffects, S.cpp:2063-2103. */
void lso_handle_surface(lso_state* s) {
    const int I = s->I, J = s->J, K = s->K;
    /* order-independent: a voxel's test reads only whether its neighbours are Air, and the
       flips it makes (Pore -> Precipitate) never create Air */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < I; ++i)
        for (int j = 0; j < J; ++j)
            for (int k = 0; k < K; ++k) {
                size_t r = IDX(s, i, j, k), nb;
                if (s->label[r] == PORE && s->sat[r] > 0.0) {
                    int is_surface_voxel = 0;
                    for (int d = 0; d < 6; ++d)
                        if (NB(s, i, j, k, d, &nb) && s->label[nb] == AIR) { is_surface_voxel = 1; break; }
                    if (is_surface_voxel) {
                        s->conc[r] = 1.0;
                        s->label[r] = PRECIPITATE;
                    }
                }
            }
}

/* ------------------------------------------------------------------------ */
/* transport                                                                 */

/* Simulation::setupConcentrationEqns, active part S.cpp:1129-1232 (the block at
 * S.cpp:997-1128 is commented out). With bc_mode LS_BC_FLOW_I (an extension, after the
 * inlet_bc rows of that disabled block, S.cpp:997-1004) the Pore and Air voxels of plane
 * i = 0 are identity rows holding conc_inlet / acid_inlet. Links to neighbours outside the domain are
 * skipped: the reference evaluates flux_x[Index(i-1,j,k)] before set_pore_link's own
 * validity test (S.cpp:1227,1229,1231), which throws at the low faces; the link it
 * would build is skipped either way. */
void lso_setup_conc(lso_state* s, double dt, int which) {
    const double* field = which ? s->acid : s->conc;
    const double inv_dt = 1.0 / dt;
    const double theta = s->p.theta, alpha = s->p.alpha_transfer, dx = s->p.dx;
    ell_sys* e = &s->trans;
    const int I = s->I, J = s->J, K = s->K;
    /* Each row depends only on labels, fluxes and field values of its voxel and neighbours.
       The reference zeroes the fluxes of Rock and Precipitate voxels inside the same loop
       (S.cpp:1133-1148); no row uses the flux of such a neighbour (a Rock neighbour takes the
       exchange branch, a Precipitate neighbour's advection is zeroed), so the rows are built
       first, in parallel, and the fluxes zeroed after. */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < I; ++i)
        for (int j = 0; j < J; ++j)
            for (int k = 0; k < K; ++k) {
                size_t r = IDX(s, i, j, k), nb;
                uint16_t t = s->label[r];
                for (int d = 0; d < 6; ++d) e->A[d][r] = 0.0;
                if (s->p.bc_mode == LS_BC_FLOW_I && i == 0 && (t == PORE || t == AIR)) {
                    /* inlet plane (extension): the fluid voxels hold the inflow value */
                    e->diag[r] = 1.0;
                    e->b[r] = 0.0 + (which ? s->p.acid_inlet : s->p.conc_inlet);
                    e->kind[r] = 1;
                    continue;
                }
                if (t == PRECIPITATE) {
                    e->diag[r] = 1.0;
                    e->b[r] = 0.0 + field[r];
                    e->kind[r] = 1;
                    continue;
                }
                if (t == ROCK) {
                    double diag = inv_dt;
                    e->b[r] = 0.0 + field[r] * inv_dt;
                    for (int d = 0; d < 6; ++d) {
                        if (NB(s, i, j, k, d, &nb) && s->label[nb] == PORE) {
                            diag += alpha;
                            e->A[d][r] = -alpha;
                        }
                    }
                    e->diag[r] = diag;
                    e->kind[r] = 2;
                    continue;
                }
                double diag = inv_dt;
                double rhs = 0.0 + field[r] * inv_dt;
                for (int d = 0; d < 6; ++d) {
                    if (!NB(s, i, j, k, d, &nb)) continue;
                    uint16_t nt = s->label[nb];
                    if (nt == ROCK) {
                        diag += alpha;
                        e->A[d][r] = -alpha;
                        continue;
                    }
                    double q_face;
                    switch (d) {
                    case 0: q_face = s->fx[r]; break;
                    case 1: q_face = -s->fx[nb]; break;
                    case 2: q_face = s->fy[r]; break;
                    case 3: q_face = -s->fy[nb]; break;
                    case 4: q_face = s->fz[r]; break;
                    default: q_face = -s->fz[nb]; break;
                    }
                    double actual_q_face = q_face;
                    if (nt == PRECIPITATE || nt == SULPHIDE) actual_q_face = 0.0;
                    double D_eff = (nt == PORE) ? (s->p.D * s->p.Dpore_fac) : s->p.D;
                    double diffusion_coeff = -D_eff / (dx * dx);
                    double coeff_neighbor = diffusion_coeff;
                    double coeff_self = -diffusion_coeff;
                    double adv_coeff = actual_q_face / dx;
                    if (adv_coeff > 0) coeff_self += adv_coeff;
                    else coeff_neighbor -= adv_coeff;
                    e->A[d][r] = theta * coeff_neighbor;
                    diag += theta * coeff_self;
                    double explicit_rhs = -(coeff_self * field[r] + coeff_neighbor * field[nb]);
                    rhs += (1.0 - theta) * explicit_rhs;
                }
                e->diag[r] = diag;
                e->b[r] = rhs;
                e->kind[r] = 2;
            }
    const long N = (long)s->N;
#pragma omp parallel for schedule(static)
    for (long r = 0; r < N; ++r) {
        uint16_t t = s->label[r];
        if (t == PRECIPITATE || t == ROCK) { s->fx[r] = 0.0; s->fy[r] = 0.0; s->fz[r] = 0.0; }
    }
}

/* Simulation::solveConc (S.cpp:1243-1295) / solveAcid (S.cpp:2167-2224). */
int lso_solve_conc(lso_state* s, int which, ls_solve_info* info) {
    double* x = solution_slots(s, which ? s->acid : s->conc);
    return run_solve(s, &s->trans, x, s->p.conc_rtol, s->p.conc_max_it, solves_per_call(s), info, 0);
}

void lso_transport_apply(const lso_state* s, const double* x, double* y) { ell_apply(s, &s->trans, x, y); }
void lso_transport_rhs(const lso_state* s, double* b) { memcpy(b, s->trans.b, s->N * sizeof(double)); }

/* Simulation::handlePrecipitation, S.cpp:2114-2165. */
void lso_handle_precip(lso_state* s) {
    const double c_sat = s->p.c_sat;
    const long N = (long)s->N;
#pragma omp parallel for schedule(static)
    for (long r = 0; r < N; ++r) {
        if (s->label[r] == PORE && s->conc[r] > c_sat) {
            double excess_conc = s->conc[r] - c_sat;
            if (s->p.use_instant_precipitation) {
                s->label[r] = PRECIPITATE;
            } else {
                double fluid_vol_fraction = s->p.porosity * s->sat[r];
                double precipitated_vol_fraction = (excess_conc * fluid_vol_fraction) / s->p.solid_density;
                s->precip[r] += (precipitated_vol_fraction * s->p.time_scalar);
                const double critical_limit = 0.90;
                if (s->precip[r] > critical_limit) s->label[r] = PRECIPITATE;
            }
            s->conc[r] = c_sat;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* dissolution                                                               */

/* calc_surface_flux lambda, S.cpp:520-542 (same as S.cpp:371-393). */
static inline double surface_flux(const lso_state* s, int i, int j, int k, int d) {
    size_t nb;
    if (NB(s, i, j, k, d, &nb)) {
        uint16_t n_type = s->label[nb];
        if (n_type == PORE || n_type == ROCK) {
            double k_trans = s->p.D / s->p.dx;
            double k_eff = 1.0 / ((1.0 / k_trans) + (1.0 / s->p.kreac));
            double driving_force = s->acid[nb];
            return k_eff * driving_force;
        }
    }
    return 0.0;
}

/* Simulation::updateFrac, S.cpp:315-617: a rate pass, then num_steps sequential sweeps
 * in the reference's loop order (k outer, i inner) that consume neighbour acid in place
 * and turn fully leached Sulphide into Pore. */
int lso_update_frac(lso_state* s, double dt, ls_substep_info* info) {
    const int I = s->I, J = s->J, K = s->K;
    const double dx = s->p.dx;
    int leached_locally = 0;
    double max_rate = 0.0;
    /* the rate pass in parallel (a maximum does not depend on the order) */
#pragma omp parallel for schedule(static) reduction(max : max_rate)
    for (int i = 0; i < I; ++i)
        for (int j = 0; j < J; ++j)
            for (int k = 0; k < K; ++k) {
                size_t r = IDX(s, i, j, k);
                if (s->label[r] == SULPHIDE) {
                    double flux_sum = 0.0;
                    for (int d = 0; d < 6; ++d) flux_sum += surface_flux(s, i, j, k, d);
                    double area_per_face = dx * dx;
                    double voxel_volume = dx * dx * dx;
                    double vol_rate = flux_sum * area_per_face;
                    double fractional_rate = vol_rate / voxel_volume;
                    if (fractional_rate > max_rate) max_rate = fractional_rate;
                }
            }
    double effective_fractional_rate = max_rate * s->p.time_scalar;
    double dt_safe = dt;
    if (effective_fractional_rate > 1e-20) dt_safe = 0.1 / effective_fractional_rate;
    double calculated_steps = ceil(dt / dt_safe);
    int num_steps = 1;
    if (calculated_steps > 1000) num_steps = 1000;
    else if (calculated_steps > 1.0) num_steps = (int)calculated_steps;
    double dt_sub = dt / num_steps;
    if (info) {
        info->max_rate = max_rate;
        info->num_steps = num_steps;
        info->dt_sub = dt_sub;
    }
    static const int di[6] = {1, -1, 0, 0, 0, 0};
    static const int dj[6] = {0, 0, 1, -1, 0, 0};
    static const int dk[6] = {0, 0, 0, 0, 1, -1};
    /* The sweeps visit, in the reference's loop order (k outer, i inner), only the voxels that
       are active (label >= Sulphide, frac > 0) at the start: a sweep only ever lowers frac and
       turns Sulphide into Pore, so no other voxel becomes active during the call. */
    size_t nact = 0;
    for (size_t r = 0; r < s->N; ++r)
        if (s->label[r] >= SULPHIDE && s->frac[r] > 0.0) nact++;
    size_t* act = (size_t*)xcalloc(nact ? nact : 1, sizeof(size_t));
    {
        size_t q = 0;
        for (int k = 0; k < K; ++k)
            for (int j = 0; j < J; ++j)
                for (int i = 0; i < I; ++i) {
                    size_t r = IDX(s, i, j, k);
                    if (s->label[r] >= SULPHIDE && s->frac[r] > 0.0) act[q++] = r;
                }
    }
    for (int step = 0; step < num_steps; ++step) {
        for (size_t q = 0; q < nact; ++q) {
                    const size_t r = act[q];
                    const int i = (int)(r / s->JK), j = (int)((r / (size_t)K) % (size_t)J), k = (int)(r % (size_t)K);
                    if (s->label[r] >= SULPHIDE && s->frac[r] > 0.0) {
                        double f[6];
                        for (int d = 0; d < 6; ++d) f[d] = surface_flux(s, i, j, k, d);
                        double flux_sum = f[0] + f[1] + f[2] + f[3] + f[4] + f[5];
                        double area_per_face = dx * dx;
                        double voxel_volume = dx * dx * dx;
                        double mass_loss = flux_sum * area_per_face * dt_sub;
                        double fractional_loss = mass_loss / voxel_volume;
                        s->frac[r] -= (fractional_loss * s->p.time_scalar);
                        if (flux_sum > 0.0) {
                            for (int d = 0; d < 6; ++d) {
                                int ni = i + di[d], nj = j + dj[d], nk = k + dk[d];
                                if (ni < 0 || ni >= I || nj < 0 || nj >= J || nk < 0 || nk >= K) continue;
                                s->acid[IDX(s, ni, nj, nk)] -= fractional_loss * (f[d] / flux_sum);
                            }
                        }
                        if (s->frac[r] <= 1e-4) {
                            s->frac[r] = 0.0f;
                            if (s->label[r] == SULPHIDE) {
                                s->label[r] = PORE;
                                s->precip[r] = 0.0;
                                s->conc[r] = s->p.c_sat;
                                leached_locally++;
                            }
                        }
                    }
        }
    }
    free(act);
    return leached_locally;
}

/* ------------------------------------------------------------------------ */
/* snapshot / rollback, S.cpp:2312-2353                                      */

/* memcpy split over the threads */
static void pcopy(void* dst, const void* src, size_t bytes) {
    const long chunks = 64;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < chunks; ++c) {
        size_t a = bytes * (size_t)c / (size_t)chunks, b = bytes * (size_t)(c + 1) / (size_t)chunks;
        memcpy((char*)dst + a, (const char*)src + a, b - a);
    }
}

void lso_save_state(lso_state* s) {
    size_t n = s->NP;
    pcopy(s->b_label, s->label, n * sizeof(uint16_t));
    pcopy(s->b_frac, s->frac, n * sizeof(float));
    pcopy(s->b_precip, s->precip, n * sizeof(double));
    pcopy(s->b_sat, s->sat, n * sizeof(double));
    pcopy(s->b_P, s->P, n * sizeof(double));
    pcopy(s->b_conc, s->conc, n * sizeof(double));
    pcopy(s->b_acid, s->acid, n * sizeof(double));
    pcopy(s->b_fx, s->fx, n * sizeof(double));
    pcopy(s->b_fy, s->fy, n * sizeof(double));
    pcopy(s->b_fz, s->fz, n * sizeof(double));
}

void lso_restore_state(lso_state* s) {
    size_t n = s->NP;
    pcopy(s->label, s->b_label, n * sizeof(uint16_t));
    pcopy(s->frac, s->b_frac, n * sizeof(float));
    pcopy(s->precip, s->b_precip, n * sizeof(double));
    pcopy(s->sat, s->b_sat, n * sizeof(double));
    pcopy(s->P, s->b_P, n * sizeof(double));
    pcopy(s->conc, s->b_conc, n * sizeof(double));
    pcopy(s->acid, s->b_acid, n * sizeof(double));
    pcopy(s->fx, s->b_fx, n * sizeof(double));
    pcopy(s->fy, s->b_fy, n * sizeof(double));
    pcopy(s->fz, s->b_fz, n * sizeof(double));
    lso_update_relperm(s);
    lso_update_cap(s);
    lso_init_properties(s);
}

/* ------------------------------------------------------------------------ */
/* FP64 budget of a step (an extension; the reference keeps only the leached count,
 * main.cpp:414-431): sums over the N voxels in index order. acid_pre holds the acid
 * before the dissolution sweep (NULL: the sweep did not run), b_frac the frac at the
 * start of the step. */
static void lso_budget(const lso_state* s, const double* acid_pre, ls_budget* b) {
    memset(b, 0, sizeof(*b));
    for (size_t r = 0; r < s->N; ++r) {
        b->conc += s->conc[r];
        b->acid += s->acid[r];
        b->mineral += (double)s->frac[r];
        b->precipitate += s->precip[r];
        if (acid_pre) b->acid_consumed += acid_pre[r] - s->acid[r];
        b->mineral_dissolved += (double)s->b_frac[r] - (double)s->frac[r];
        if (s->label[r] == SULPHIDE) b->sulphide_voxels++;
        if (s->label[r] == PRECIPITATE) b->precipitate_voxels++;
    }
}

/* ------------------------------------------------------------------------ */
/* one attempt of the time step, main.cpp:303-432                           */

int lso_step(lso_state* s, double t, double dt, ls_step_info* info) {
    ls_step_info loc;
    memset(&loc, 0, sizeof(loc));
    lso_save_state(s);
    int ok = 1;
    int max_picard = s->p.use_implicit_saturation ? 3 : 1;
    for (int picard = 0; picard < max_picard; ++picard) {
        loc.picard_iterations = picard + 1;
        lso_update_relperm(s);
        lso_update_cap(s);
        lso_init_properties(s);
        lso_setup_pressure(s, t);
        if (!lso_solve_pressure(s, &loc.pressure)) { ok = 0; break; }
        lso_calculate_flux(s);
        if (s->p.use_implicit_saturation) {
            lso_setup_saturation(s, dt);
            int valid = 1;
            if (!lso_solve_saturation(s, &loc.saturation_solve, &valid)) { ok = 0; break; }
        } else {
            lso_update_saturation(s, dt, &loc.saturation);
        }
    }
    if (ok && s->p.use_implicit_saturation && !s->physics_valid) ok = 0;
    if (ok) {
        lso_handle_surface(s);
        lso_setup_conc(s, dt, 0);
        if (!lso_solve_conc(s, 0, &loc.conc)) ok = 0;
    }
    if (ok) {
        lso_setup_conc(s, dt, 1);
        if (!lso_solve_conc(s, 1, &loc.acid)) ok = 0;
    }
    if (ok) {
        lso_handle_precip(s);
        double* acid_pre = (double*)xcalloc(s->N, sizeof(double));
        memcpy(acid_pre, s->acid, s->N * sizeof(double));
        loc.leached = lso_update_frac(s, dt, &loc.leaching);
        s->total_leached += (unsigned long long)loc.leached;
        lso_budget(s, acid_pre, &loc.budget);
        free(acid_pre);
    }
    loc.success = ok;
    if (info) *info = loc;
    return ok;
}

/* ------------------------------------------------------------------------ */
/* checkpoint, S.cpp:2235-2307 (np=1: (I+1)*J*K elements per array)         */

int lso_write_checkpoint(lso_state* s, const char* path) {
    FILE* f = fopen(path, "wb");
    if (!f) return -1;
    size_t n = s->NP;
    int rc = 0;
    if (s->label_bytes == 1) {
        uint8_t* tmp = (uint8_t*)xcalloc(n, 1);
        for (size_t r = 0; r < n; ++r) tmp[r] = (uint8_t)s->label[r];
        rc |= fwrite(tmp, 1, n, f) != n;
        free(tmp);
    } else {
        rc |= fwrite(s->label, 2, n, f) != n;
    }
    rc |= fwrite(s->frac, 4, n, f) != n;
    const double* a[] = {s->precip, s->sat, s->P, s->conc, s->acid};
    for (int q = 0; q < 5; ++q) rc |= fwrite(a[q], 8, n, f) != n;
    fclose(f);
    return rc ? -1 : 0;
}

int lso_load_checkpoint(lso_state* s, const char* path) {
    FILE* f = fopen(path, "rb");
    if (!f) return -1;
    size_t n = s->NP;
    int rc = 0;
    if (s->label_bytes == 1) {
        uint8_t* tmp = (uint8_t*)xcalloc(n, 1);
        rc |= fread(tmp, 1, n, f) != n;
        for (size_t r = 0; r < n; ++r) s->label[r] = tmp[r];
        free(tmp);
    } else {
        rc |= fread(s->label, 2, n, f) != n;
    }
    rc |= fread(s->frac, 4, n, f) != n;
    double* a[] = {s->precip, s->sat, s->P, s->conc, s->acid};
    for (int q = 0; q < 5; ++q) rc |= fread(a[q], 8, n, f) != n;
    fclose(f);
    return rc ? -1 : 0;
}
