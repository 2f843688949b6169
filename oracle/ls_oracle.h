/*
 * ls_oracle.h - CPU restatement of the LeachingSim per-time-step algorithm.
 *
 * TEST INFRASTRUCTURE ONLY. This is the oracle the CUDA path is checked
 * against (tests/, __graft_entry__.smoke()) and the CPU baseline bench.py
 * times (--impl reference, cpu_baseline). The product library never links,
 * loads or calls it.
 *
 * PARITY PINNED to the reference's own code: the reference (javalosp/LeachingSim)
 * has no tests or golden outputs and needs MPI + PETSc + VTK + Boost, none of which
 * exist here; its per-time-step sources are compiled unchanged against single-rank
 * stand-ins for those libraries into oracle/_ref (oracle/build_ref.py), and
 * tests/test_ref_pin.py checks this restatement against them function by function
 * (bit for bit where no linear solve is involved) and over whole steps; two golden
 * fixtures under tests/golden/ come from that library. The restatement follows the
 * source line by line (citations are to files of the reference project) and is also
 * cross-checked against an independent numpy restatement in tests/twin.py.
 *
 * Semantics restated are those of a single MPI rank (np=1), including the
 * one-plane write-back offset of every linear solve (compat_shift), the
 * indeterminate saturation of inactive voxels after an explicit update
 * (defined here as 0.0) and the sequential in-place dissolution sweep.
 */
#ifndef LS_ORACLE_H_
#define LS_ORACLE_H_

#include <stddef.h>
#include <stdint.h>
#include "../include/leachingsim.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Linear solver modes. */
enum {
    LSO_SOLVE_REFERENCE = 0, /* GMRES(30)+Jacobi, rtol/max_it from params, KSPSolve called twice */
    LSO_SOLVE_TIGHT = 1,     /* GMRES(restart)+Jacobi to a tight rtol, once */
    LSO_SOLVE_PCG = 2,       /* as TIGHT, but the pressure system by multigrid-preconditioned CG
                                on its symmetric Pore block (faster at 64^3 and above) */
    LSO_SOLVE_PRODUCTION = 3 /* the reference's production configuration (its job scripts'
                                -press_pc_type hypre, an algebraic-multigrid preconditioner): the
                                pressure by multigrid-preconditioned CG, the transport systems by
                                GMRES(30)+Jacobi, tolerances from the parameters (the reference's
                                1e-6 unless set), KSPSolve twice per solve; the timed CPU baseline */
};

typedef struct lso_solver_cfg {
    int mode;
    int restart;       /* GMRES restart length */
    double rtol;       /* overrides params when > 0 */
    int max_it;        /* overrides params when > 0 */
} lso_solver_cfg;

typedef struct lso_state lso_state;

void lso_params_default(ls_params* p);
lso_state* lso_create(int I, int J, int K, int label_bytes, const ls_params* p);
void lso_destroy(lso_state* s);
void lso_set_params(lso_state* s, const ls_params* p);
void lso_set_solver(lso_state* s, const lso_solver_cfg* cfg);
int lso_num_threads(void);
void lso_set_num_threads(int n);

/* Field access. n must be I*J*K (padded=0) or (I+1)*J*K (padded=1). Labels are passed
   as uint16 regardless of label_bytes. Returns 0 on success. */
int lso_set_field(lso_state* s, int field, const void* src, size_t n, int padded);
int lso_get_field(lso_state* s, int field, void* dst, size_t n, int padded);

void lso_init_fields(lso_state* s);
unsigned long long lso_init_frac(lso_state* s);
void lso_init_saturation(lso_state* s);
void lso_init_acid(lso_state* s);

void lso_update_relperm(lso_state* s);
void lso_update_cap(lso_state* s);
void lso_init_properties(lso_state* s);

void lso_setup_pressure(lso_state* s, double t);
int lso_solve_pressure(lso_state* s, ls_solve_info* info);
/* y = A x and b of the assembled pressure system (I*J*K doubles). */
void lso_pressure_apply(const lso_state* s, const double* x, double* y);
void lso_pressure_rhs(const lso_state* s, double* b);
/* Row kind of the pressure system: 0 empty, 1 identity, 2 Pore. */
void lso_pressure_rowkind(const lso_state* s, int8_t* kind);
void lso_pressure_diag(const lso_state* s, double* d);

void lso_calculate_flux(lso_state* s);
void lso_update_saturation(lso_state* s, double dt, ls_substep_info* info);
void lso_setup_saturation(lso_state* s, double dt);
int lso_solve_saturation(lso_state* s, ls_solve_info* info, int* physics_valid);
void lso_handle_surface(lso_state* s);
/* which: 0 conc, 1 acid */
void lso_setup_conc(lso_state* s, double dt, int which);
int lso_solve_conc(lso_state* s, int which, ls_solve_info* info);
void lso_transport_apply(const lso_state* s, const double* x, double* y);
void lso_transport_rhs(const lso_state* s, double* b);
void lso_handle_precip(lso_state* s);
int lso_update_frac(lso_state* s, double dt, ls_substep_info* info);
void lso_save_state(lso_state* s);
void lso_restore_state(lso_state* s);

/* One attempt of src/main.cpp:303-432. Returns 1 on success. */
int lso_step(lso_state* s, double t, double dt, ls_step_info* info);

unsigned long long lso_initial_sulphide_count(const lso_state* s);

/* Checkpoint files in the reference's np=1 byte layout (src/Simulation.cpp:2235-2307). */
int lso_write_checkpoint(lso_state* s, const char* path);
int lso_load_checkpoint(lso_state* s, const char* path);

#ifdef __cplusplus
}
#endif

#endif /* LS_ORACLE_H_ */
