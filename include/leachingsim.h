/*
 * leachingsim.h - C-ABI of the GB300 LeachingSim per-time-step hot path.
 *
 * One opaque context (ls_ctx) owns every device buffer of one simulation
 * domain and one CUDA stream. All entry points are plain C: pointers, sizes
 * and POD structs only, no C++ or torch types. Host pointers passed in are
 * borrowed for the duration of the call. Every call returns an ls_status and
 * never throws or aborts; ls_last_error() gives the message of the last
 * failure on a context.
 *
 * Grid and layout (the reference's ZFastest scheme, src/Domain.cpp:107-117,
 * src/main.cpp:94): extents (I, J, K) = (zext, yext, xext); voxel (i, j, k)
 * has linear index  k + K*(j + J*i), k fastest, which is also the byte order
 * of the .raw input (src/MPIRawLoader.h:70).
 *
 * Every field lives on the device with (I+1)*J*K "slots": the reference's
 * padded single-rank array (src/MPIDomain.h:75-97 clips only the lower halo on
 * rank 0, so one extra top plane remains). Unpadded host transfers cover slots
 * [0, I*J*K); padded transfers cover all (I+1)*J*K slots, byte-compatible with
 * the reference's checkpoint arrays (src/Simulation.cpp:2235-2267).
 *
 * Label values follow src/compiler_opts.h:70-82: Air=1, Pore=2, Rock=3,
 * Sulphide=4, Precipitate=5; any other value is carried through with the
 * reference's semantics for "none of the above".
 */
#ifndef LEACHINGSIM_H_
#define LEACHINGSIM_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LS_ABI_VERSION 3

enum {
    LS_AIR = 1,
    LS_PORE = 2,
    LS_ROCK = 3,
    LS_SULPHIDE = 4,
    LS_PRECIPITATE = 5
};

typedef enum ls_status {
    LS_OK = 0,
    LS_NOT_CONVERGED = 1,            /* a linear solve hit its iteration cap */
    LS_STAGNATED_FALLBACK_USED = 2,  /* accepted, but only after a fallback solver ran */
    LS_NONFINITE = 3,                /* NaN/Inf met in a residual or a field */
    LS_BAD_ARG = 4,
    LS_CUDA_ERROR = 5,
    LS_TIMEOUT = 6,                  /* a bounded device wait gave up */
    LS_NO_DEVICE = 7,
    LS_UNPHYSICAL = 8                /* implicit saturation left [-0.05, 1.05] (src/Simulation.cpp:2008) */
} ls_status;

/* Field identifiers for upload/download. */
typedef enum ls_field {
    LS_F_LABEL = 0,        /* img_data, uint8 or uint16 per label_bytes */
    LS_F_FRAC = 1,         /* frac, float32 */
    LS_F_PERMEABILITY = 2, /* float64 from here on */
    LS_F_VISCOSITY = 3,
    LS_F_PRESSURE = 4,
    LS_F_CONC = 5,
    LS_F_ACID = 6,
    LS_F_FLUX_X = 7,       /* flux along i (Z, vertical) */
    LS_F_FLUX_Y = 8,
    LS_F_FLUX_Z = 9,       /* flux along k (X, fastest) */
    LS_F_SATURATION = 10,
    LS_F_CAP_PRESSURE = 11,
    LS_F_REL_PERM = 12,
    LS_F_PRECIPITATE = 13,
    LS_F_KMULT = 14,       /* float32 multiplier of the intrinsic permeability (1 = the reference's
                              value); no counterpart in the reference, whose permeabilities are
                              fixed per label (src/Simulation.cpp:190-191). Held only once
                              uploaded; downloading it before then is LS_BAD_ARG. Not part of
                              the snapshot (it does not change during a run). */
    LS_F_COUNT = 15
} ls_field;

/* Boundary-condition models (ls_params.bc_mode). */
typedef enum ls_bc_mode {
    LS_BC_REFERENCE = 0,   /* the reference's: Air voxels touching non-Air hold the ramped
                              top_pressure (src/Simulation.cpp:662-720), every other boundary is
                              closed and no species flows in */
    LS_BC_FLOW_I = 1       /* flow-through along i (Z), no counterpart in the reference: the Pore
                              voxels of plane i = 0 hold p_inlet and those of plane i = I-1 hold
                              p_outlet (identity rows of the pressure system), the sides stay
                              closed; in the transport systems the Pore and Air voxels of plane
                              i = 0 hold conc_inlet / acid_inlet (identity rows, like the inlet_bc
                              rows of the reference's disabled block, src/Simulation.cpp:997-1004).
                              Everything else follows the reference. */
} ls_bc_mode;

/* Device memory layout of a context, fixed when it is created (ls_params.memory_mode). */
typedef enum ls_memory_mode {
    LS_MEM_RESIDENT = 0,   /* every work array stays allocated, the FP64 per-voxel kernels
                              recompute only the voxels whose inputs changed (shadow copies of
                              their inputs), the state snapshot is in device memory: ~620 bytes
                              per voxel (uint16 labels, mixed precision) */
    LS_MEM_LEAN = 1        /* for domains that do not fit that way: the pressure solve's and the
                              transport solves' work arrays are cut from one device arena (the
                              set of a phase is released when the other phase starts), every
                              voxel is recomputed each step, the snapshot (but for the mineral
                              fractions) is in pinned host memory and copied on a stream of its
                              own while the step runs: ~285 bytes per voxel (mixed precision),
                              ~310 (FP64). Results are bit-identical to LS_MEM_RESIDENT. The
                              pressure system stays readable (ls_pressure_apply, ...) until the
                              next transport solve. */
} ls_memory_mode;

/* Pressure solver variants. */
typedef enum ls_press_solver {
    LS_PRESS_MIXED = 0,    /* FP32 MG-PCG inner solves, FP64 iterative refinement outside */
    LS_PRESS_FP64 = 1,     /* FP64 MG-PCG inner solves (the plain path) */
    LS_PRESS_JACOBI64 = 2, /* FP64 Jacobi-PCG inner solves (no multigrid; test path) */
    LS_PRESS_LEARNED = 3   /* LS_PRESS_MIXED with the learned coarse solver in the multigrid cycle
                              (ls_pressure_set_precond_weights); the plain cycle takes over when
                              the flexible CG stagnates */
} ls_press_solver;

/*
 * Physical and numerical parameters. Field names follow Simulation's public
 * members (src/Simulation.h:75-114) and the CLI (src/main.cpp:39, 69-91).
 * ls_params_default() fills the CLI defaults.
 */
typedef struct ls_params {
    double D;                 /* --D */
    double dx;                /* --voxel_size */
    double Dpore_fac;         /* --Dpore_fac */
    double kext;              /* --kext (kept for interface parity; unused by the physics) */
    double kreac;             /* --kreac */
    double theta;             /* --theta */
    double c_sat;             /* --csat */
    double evaporative_flux;  /* --evap_flux */
    double top_pressure;      /* --top_pressure */
    double max_cap_grad;      /* --max_cap_grad */
    double vg_alpha;          /* 1.0, src/main.cpp:90 */
    double vg_n;              /* 2.0, src/main.cpp:89 */
    double s_res;             /* 0.05, src/main.cpp:91 */
    double porosity;          /* --porosity */
    double time_scalar;       /* --time_scalar */
    double rock_D_fac;        /* --rock_D_fac (unused by the active transport code) */
    double alpha_transfer;    /* --alpha_transfer */
    double solid_density;     /* never initialised by the reference (src/Simulation.h:135); default 1.0 */
    int use_instant_precipitation; /* --instant_precip */
    int use_implicit_saturation;   /* --implicit_sat */
    int enable_microporosity;      /* --enable_microporosity (unused by the active code) */
    int debug_mode;                /* --debug: enables device NaN audits */
    int compat_shift;   /* 1 (default): linear-solve results land one i-plane up, as on the
                           reference's rank 0 (src/Simulation.cpp:808,1247,1975,2173);
                           0: corrected, results land in their own slots */
    /* Linear solver controls (the reference: GMRES(30)+Jacobi, rtol 1e-6, max_it 1e4,
       src/Simulation.cpp:146-157). rtol is on the Jacobi-scaled residual
       ||D^-1 (b - A x)||_2 / ||D^-1 b||_2, the norm PETSc's left-preconditioned
       GMRES tests. */
    double press_rtol;
    int press_max_it;         /* cap on inner Krylov iterations summed over refinement sweeps */
    int press_solver;         /* ls_press_solver */
    double conc_rtol;         /* conc and acid transport solves */
    int conc_max_it;
    double sat_rtol;          /* implicit saturation solve */
    int sat_max_it;
    /* Boundary model and permeability constants (ABI 2). */
    int bc_mode;              /* ls_bc_mode; 0 = the reference's model */
    double p_inlet;           /* LS_BC_FLOW_I: pressure of the Pore voxels of plane i = 0 (1.0) */
    double p_outlet;          /* LS_BC_FLOW_I: pressure of the Pore voxels of plane i = I-1 (0.0) */
    double conc_inlet;        /* LS_BC_FLOW_I: conc held on the fluid voxels of plane i = 0 (0.0) */
    double acid_inlet;        /* LS_BC_FLOW_I: acid held on the fluid voxels of plane i = 0 (0.0) */
    double pore_permeability; /* 1e-12: Air and clean Pore (src/Simulation.cpp:190) */
    double rock_permeability; /* 1e-18: Rock, and the clogged / unleached end of the log blend
                                 (src/Simulation.cpp:191) */
    /* ABI 3 */
    int memory_mode;          /* ls_memory_mode; fixed at ls_create (ls_set_params rejects a change) */
} ls_params;

/* Result of one linear solve (the reference's log line, src/Simulation.cpp:834-849). */
typedef struct ls_solve_info {
    int iterations;           /* inner Krylov iterations */
    int outer_iterations;     /* refinement sweeps (pressure) */
    int converged;            /* 1 = the reference's reason > 0 */
    int reason;               /* >0 converged, <0 diverged (PETSc-style codes: 2 rtol, -3 its, -4 nan) */
    double rel_residual;      /* final Jacobi-scaled relative residual, FP64 */
    double min_value;         /* min / max over the solution vector (I*J*K rows) */
    double max_value;
} ls_solve_info;

/* Sub-stepping summary (src/Simulation.cpp:455-464, 1770-1779). */
typedef struct ls_substep_info {
    double max_rate;          /* max |div q| + evap (saturation) or max fractional rate (leaching) */
    int num_steps;
    double dt_sub;
} ls_substep_info;

/* FP64 species and mineral budget of one step (ABI 2). The reference keeps only the count of
   leached voxels (src/main.cpp:414-431); these are sums over the I*J*K voxels of the values per
   voxel (an amount in voxel volumes for a concentration), reduced in FP64 in a fixed order. */
typedef struct ls_budget {
    double conc;              /* sum of conc after the step */
    double acid;              /* sum of acid after the step */
    double mineral;           /* sum of frac after the step (unleached mineral) */
    double precipitate;       /* sum of precipitate_inventory after the step */
    double acid_consumed;     /* acid taken from the neighbours of the mineral by the dissolution
                                 sweep during the step (src/Simulation.cpp:560-580) */
    double mineral_dissolved; /* frac the mineral voxels lost during the step; equals
                                 acid_consumed * time_scalar up to the FP32 rounding of frac, plus
                                 the remainders (<= 1e-4 each) cleared at the leach threshold */
    long long sulphide_voxels;     /* label == Sulphide after the step */
    long long precipitate_voxels;  /* label == Precipitate after the step */
} ls_budget;

/* One full time step (src/main.cpp:303-432). */
typedef struct ls_step_info {
    ls_solve_info pressure;
    ls_substep_info saturation;
    ls_solve_info saturation_solve;  /* implicit saturation only, last Picard iteration */
    ls_solve_info conc;
    ls_solve_info acid;
    ls_substep_info leaching;
    int leached;              /* voxels fully leached this step */
    int picard_iterations;
    int success;              /* 0 = the retry manager must roll back and halve dt */
    ls_budget budget;         /* filled when success = 1 */
} ls_step_info;

typedef struct ls_ctx ls_ctx;

void ls_params_default(ls_params* p);
int ls_abi_version(void);

/* Context life cycle. label_bytes is 1 (uint8 images) or 2 (uint16).
   Replaces Simulation::setupDomain + setupPETSc (src/Simulation.cpp:81-103, 131-159). */
ls_status ls_create(ls_ctx** out, int I, int J, int K, int label_bytes, const ls_params* params);
ls_status ls_destroy(ls_ctx* ctx);
const char* ls_last_error(const ls_ctx* ctx);
ls_status ls_set_params(ls_ctx* ctx, const ls_params* params);
ls_status ls_get_params(const ls_ctx* ctx, ls_params* params);
/* The context's CUDA stream (a cudaStream_t) for event timing by callers. */
void* ls_stream(ls_ctx* ctx);
ls_status ls_synchronize(ls_ctx* ctx);
/* Device bytes held by the context. */
size_t ls_device_bytes(const ls_ctx* ctx);
/* The most device bytes the context has held at once, and the host bytes it holds (the
   snapshot of LS_MEM_LEAN). */
size_t ls_device_peak_bytes(const ls_ctx* ctx);
size_t ls_host_bytes(const ls_ctx* ctx);

/* Host <-> device transfers. n_elems must be I*J*K (padded=0) or (I+1)*J*K (padded=1).
   The label upload replaces Simulation::readRAW's array (src/Simulation.cpp:68-74). */
ls_status ls_upload_field(ls_ctx* ctx, ls_field f, const void* host, size_t n_elems, int padded);
ls_status ls_download_field(ls_ctx* ctx, ls_field f, void* host, size_t n_elems, int padded);
/* Device-to-device variants (pointers in this process's CUDA context). */
ls_status ls_upload_field_device(ls_ctx* ctx, ls_field f, const void* dev, size_t n_elems, int padded);
ls_status ls_download_field_device(ls_ctx* ctx, ls_field f, void* dev, size_t n_elems, int padded);

/* Output without stalling the time loop (the reference's writeVTKFile downloads, src/
   Simulation.cpp:1306-1566, made asynchronous; ABI 3). Copies `count` fields (ls_field ids,
   I*J*K or (I+1)*J*K elements each) as they are now into host buffers, on a stream of the
   context's own, and returns at once; *done receives an event handle that ls_event_wait
   blocks on until every copy has landed (from any thread) and ls_event_release frees. The
   steps that follow run while the copies drain: in the resident layout the fields are first
   copied into a device staging buffer the context keeps (the size of the fields copied), so
   nothing waits for the host; in the lean layout the copies read the fields themselves and a
   later call that overwrites one waits on the device for its copy. The buffers should be
   page-locked (ls_host_alloc) for the copies to run asynchronously. */
ls_status ls_download_fields_async(ls_ctx* ctx, int count, const int* fields, void* const* host_buffers,
                                   int padded, void** done);
ls_status ls_event_wait(void* done);
void ls_event_release(void* done);
/* Page-locked host memory (null on failure) and its release. */
void* ls_host_alloc(size_t bytes);
void ls_host_free(void* p);
/* The number of NaN or infinite values of an FP64 field over the I*J*K voxels (the output
   writer's NaN scrub of src/Simulation.cpp:1487-1517 is needed only when it is nonzero). */
ls_status ls_count_nonfinite(ls_ctx* ctx, ls_field f, long long* count);

/* Initialisation (src/Simulation.cpp:165-180, 254-278, 285-310, 1573-1590, 109-125). */
ls_status ls_init_fields(ls_ctx* ctx);
ls_status ls_init_frac(ls_ctx* ctx, unsigned long long* initial_sulphide_count);
ls_status ls_init_saturation(ls_ctx* ctx);
ls_status ls_init_acid(ls_ctx* ctx);

/* Simulation::updateRelativePermeability + updateCapillaryPressure + initProperties,
   fused (src/Simulation.cpp:1634-1664, 1596-1628, 187-248). */
ls_status ls_props(ls_ctx* ctx);
/* Simulation::setupPressureEqns(t) + solvePressure (src/Simulation.cpp:658-855). */
ls_status ls_pressure_step(ls_ctx* ctx, double t, ls_solve_info* info);
/* The learned start of the pressure solve (no counterpart in the reference), on the system
   assembled by ls_pressure_setup(t): ls_pressure_learned_inputs writes the network's input
   fields to DEVICE float32 arrays of I*J*K values: the Pore-row mask (0/1), the
   log-permeability (log10 K + 15) / 3, and the identity-row values over the effective top
   pressure. ls_pressure_solve_start solves the assembled system from x = scale * p_top *
   start (start: DEVICE float32, I*J*K; p_top: the effective top pressure) on the Pore rows
   instead of the stored pressure; the FP64 refinement judges and finishes the solve
   exactly as in ls_pressure_step. */
ls_status ls_pressure_learned_inputs(ls_ctx* ctx, float* mask, float* logk, float* bc);
ls_status ls_pressure_solve_start(ls_ctx* ctx, const float* start, double scale, ls_solve_info* info);
/* Learned preconditioner of the pressure solve (no counterpart in the reference). With
   press_solver = LS_PRESS_LEARNED the inner flexible CG (FP32, inside the FP64 refinement) is
   preconditioned by the K-cycle whose coarse correction on multigrid level 4 (1/16 of the grid
   along each axis, the level below the three K-cycle levels) is the network of ls_lpnet_*
   applied to that level's residual, instead of a V-cycle over the levels below. Network input channels on a grid holding the level at
   its origin (extents rounded up to multiples of 8): the member mask, the anchoring fraction
   e/d (the share of a cell's diagonal coupling to fixed values) and D^-1/2 b / s, s the
   largest |D^-1/2 b| over the members; output D^1/2 x / (64 s). When the flexible CG
   stagnates (a non-finite, negative or growing (r, z), (p, q) <= 0, two iterations in a row
   that reduce (r, z) by less than 0.64, or four that reduce it by less than 0.64^4) the
   learned iterations' correction is dropped, the solve goes on with the plain K-cycle from
   the iterate the learned one started from, and ls_pressure_fallbacks counts it; the FP64
   residual judges every accepted solve either way. Grids too small to have level 4 use the
   plain cycle.
   params: count = ls_lpnet_param_count floats (host), copied. */
ls_status ls_pressure_set_precond_weights(ls_ctx* ctx, const float* params, long long count);
long long ls_pressure_fallbacks(const ls_ctx* ctx);
/* Training hook: multigrid level `level` (1 = the first coarse level) of the hierarchy of the
   last FP32-inner pressure solve: dims = its (I, J, K); for each non-null pointer, a host copy
   of I*J*K values: owning strong component (-1: no unknown), excess e and the +i, +j, +k face
   links (FP32, the sigma-scaled inner operator's Galerkin coarsening). */
ls_status ls_pressure_mg_level(ls_ctx* ctx, int level, int* dims, int* comp, float* e, float* f0, float* f1,
                               float* f2);
/* Simulation::calculateFlux (src/Simulation.cpp:866-953). */
ls_status ls_flux(ls_ctx* ctx);
/* Simulation::updateSaturation(dt), explicit sub-stepping (src/Simulation.cpp:1672-1856). */
ls_status ls_saturation(ls_ctx* ctx, double dt, ls_substep_info* info);
/* Simulation::setupSaturationEqns(dt) + solveSaturation (src/Simulation.cpp:1858-2053).
   Returns LS_UNPHYSICAL when the solution leaves [-0.05, 1.05]. */
ls_status ls_saturation_implicit(ls_ctx* ctx, double dt, ls_solve_info* info);
/* Explicit saturation update of ls_saturation on caller-owned device buffers that allocates
   no device memory. No counterpart in the reference: it is for callers that cannot let this
   library call cudaMalloc, such as hosts that own all device memory through their own pool
   (preallocated work arrays, a fixed device-memory budget) or stepping loops that cannot
   take the device-wide synchronisation an allocation may imply. Its reduction scratch is a
   fixed device array (LS_NOALLOC_SAT_SCRATCH_BYTES) held by every GPU that loads the
   library until the process exits; the first call on a device looks up that array's
   address. The call reads the largest rate back to the host and waits for it on the given
   stream before it picks the sub-step count, so it returns with its work done. All calls
   share the array: calls that overlap on the GPU race. Domains above
   LS_NOALLOC_SAT_MAX_VOXELS (512^3) are
   rejected with LS_BAD_ARG and a message in err (if given).
   Device pointers: label (I*J*K, uint8 or uint16 per label_bytes), flux_x/y/z (I*J*K
   float64), saturation ((I+1)*J*K float64, updated in place like the context's field).
   stream: a cudaStream_t, or NULL for the default stream. */
#define LS_NOALLOC_SAT_MAX_VOXELS 134217728LL
#define LS_NOALLOC_SAT_SCRATCH_BYTES ((16384 + 32) * 8)
ls_status ls_saturation_noalloc(int I, int J, int K, int label_bytes, const void* label,
                                const double* flux_x, const double* flux_y, const double* flux_z,
                                double* saturation, double dt, double dx, double porosity,
                                double evaporative_flux, void* stream, ls_substep_info* info,
                                char* err, size_t err_len);
/* Simulation::handleSurfaceEffects (src/Simulation.cpp:2063-2103). */
ls_status ls_surface(ls_ctx* ctx);
/* Simulation::setupConcentrationEqns + solveConc / solveAcid (src/Simulation.cpp:966-1295,
   2167-2224). which: bit 0 = conc, bit 1 = acid; both share one matrix and are solved as
   one two-right-hand-side solve. */
ls_status ls_transport(ls_ctx* ctx, double dt, int which, ls_solve_info* conc_info,
                       ls_solve_info* acid_info);
/* Simulation::handlePrecipitation (src/Simulation.cpp:2114-2165). */
ls_status ls_precip(ls_ctx* ctx);
/* Simulation::updateFrac(dt) (src/Simulation.cpp:315-617); *leached = voxels flipped. */
ls_status ls_dissolve(ls_ctx* ctx, double dt, int* leached, ls_substep_info* info);
/* Calls of ls_dissolve / ls_step whose sparse dissolution schedule (only the voxels that can
   change, ordered by their dependencies) met a leach that could reach beyond it and were redone
   with the full wavefront schedule (diagnostic; no counterpart in the reference). */
long long ls_dissolve_fallbacks(const ls_ctx* ctx);
/* Simulation::saveState / restoreState (src/Simulation.cpp:2312-2353); rollback also
   rebuilds the derived properties like the reference. */
ls_status ls_snapshot(ls_ctx* ctx);
ls_status ls_rollback(ls_ctx* ctx);
/* One attempt of the time step of src/main.cpp:303-432 (no output, no retry):
   snapshot, Picard loop (props, pressure, flux, saturation), surface effects,
   conc and acid transport, precipitation, dissolution. info->success==0 means
   the caller's retry manager must ls_rollback and halve dt. */
ls_status ls_step(ls_ctx* ctx, double t, double dt, ls_step_info* info);

/* Test hooks. y = A x for the assembled pressure operator of src/Simulation.cpp:674-792
   (rows of Air/Rock/Sulphide/Precipitate are identity, rows of other non-Pore labels are
   empty), after ls_pressure_setup(t). x, y are host float64 arrays of I*J*K. */
ls_status ls_pressure_setup(ls_ctx* ctx, double t);
ls_status ls_pressure_apply(ls_ctx* ctx, const double* x_host, double* y_host);
/* Right-hand side b of that system (host float64, I*J*K). */
ls_status ls_pressure_rhs(ls_ctx* ctx, double* b_host);
/* y = A x for the transport operator of src/Simulation.cpp:1129-1232 at time step dt. */
ls_status ls_transport_apply(ls_ctx* ctx, double dt, const double* x_host, double* y_host);

/* Geometry pre-processing of label images (host buffers, (z, y, x) order, no context; each
   call allocates its device scratch on the current device and returns when done).
   ls_geom_coarsen replaces coarsen_grid.py:20-62: 2x2x2 ranked priority voting (Sulphide >
   Air > Pore > Rock) into ((I+1)/2, J/2, K/2), an odd I padded with one Air plane; J and K
   must be even. ls_geom_clean replaces clean_micro_ct.py:33-114 in place: opening of the
   Pore mask (6-neighbour erosion then dilation), 6-connected pore components, and every Pore
   voxel outside the components reached from the ambient Air (mode 0, 'agglomerate': the
   one-voxel dilation of the largest Air component) or from the x = 0 face (mode 1,
   'core_sample') becomes Rock; *changed receives the number of such voxels.
   ls_geom_fracture replaces micro_fracture.py:21-93 in place: from every Sulphide voxel with
   no Pore face neighbour a centre line runs to its nearest Pore voxel (exact Euclidean
   feature transform, ties as scipy.ndimage.distance_transform_edt), sampled at
   ceil(distance) + 1 points as numpy.linspace + round; the Rock voxels on the lines, dilated
   by the full 3x3x3 element, become Pore. *drilled receives their number, *encapsulated the
   number of encapsulated Sulphide voxels; an image without Pore voxels is LS_BAD_ARG.
   ls_geom_classify labels a uint16 grey-level image: out = labels[i], i the number of the
   (ascending, at most 16) thresholds <= the grey value; labels has n_thresholds + 1 entries. */
ls_status ls_geom_coarsen(int I, int J, int K, int label_bytes, const void* in_host, void* out_host);
ls_status ls_geom_clean(int I, int J, int K, int label_bytes, void* labels_host, int mode,
                        long long* changed);
ls_status ls_geom_fracture(int I, int J, int K, int label_bytes, void* labels_host, long long* drilled,
                           long long* encapsulated);
/* Euclidean distance of every voxel to the nearest site (sites[v] > 0.5; -1 where there is
   no site), exact, through the same feature transform as ls_geom_fracture; DEVICE float32
   arrays of I*J*K values, synchronous. */
ls_status ls_geom_distance(int I, int J, int K, const float* sites, float* dist);
ls_status ls_geom_classify(int I, int J, int K, const uint16_t* grey_host, int n_thresholds,
                           const uint16_t* thresholds, const int* labels, int label_bytes,
                           void* out_host);

/* Learned pressure network (no counterpart in the reference): a U-shaped 3D convolutional
   network (4 levels, 16-64 channels, 3x3x3 convolutions, BF16 weights and activations,
   FP32 accumulation on the tensor cores) mapping three input fields (pore mask, normalised
   log-permeability, boundary / previous pressure) on a D x H x W grid (multiples of 8) to
   one output field. Field pointers are DEVICE pointers to D*H*W float32 values, (z, y, x)
   order. Parameters are float32, per layer (W0a, W0b, W1, W2, W3, U2, U1, U0) the weights
   [27][cout][cin] (tap = 9 (dz+1) + 3 (dy+1) + (dx+1)) then the biases [cout].
   ls_lpnet_train_step runs forward, the masked mean-square loss of output vs target over
   the mask_count voxels with mask 1, backward and (update != 0) one Adam step with rate lr;
   the gradients stay readable through ls_lpnet_get_grads. If a bounded wait of a tcgen05
   convolution gives up, the network switches to its mma.sync kernels for good: ls_lpnet_forward
   recomputes the pass with them and returns LS_STAGNATED_FALLBACK_USED (a valid output);
   ls_lpnet_train_step returns LS_TIMEOUT (discard that step). */
typedef struct ls_lpnet ls_lpnet;
ls_status ls_lpnet_create(int D, int H, int W, int seed, ls_lpnet** net);
ls_status ls_lpnet_destroy(ls_lpnet* net);
const char* ls_lpnet_last_error(const ls_lpnet* net);
long long ls_lpnet_param_count(const ls_lpnet* net);
ls_status ls_lpnet_get_params(ls_lpnet* net, float* host, long long count);
ls_status ls_lpnet_set_params(ls_lpnet* net, const float* host, long long count);
ls_status ls_lpnet_get_grads(ls_lpnet* net, float* host, long long count);
ls_status ls_lpnet_forward(ls_lpnet* net, const float* c0, const float* c1, const float* c2, float* out);
ls_status ls_lpnet_train_step(ls_lpnet* net, const float* c0, const float* c1, const float* c2,
                              const float* target, const float* mask, long long mask_count, float lr,
                              int update, double* loss);

/* Half-resolution transfers of a D x H x W float32 field (D, H, W even; DEVICE pointers,
   synchronous): ls_field_pool2 writes the (weighted) mean of every 2x2x2 block, weight may
   be null (plain mean; a block of zero weight gets 0); ls_field_up2 repeats each coarse
   value over its block. The learned start runs the network at half resolution. */
ls_status ls_field_pool2(int D, int H, int W, const float* fine, const float* weight, float* coarse);
ls_status ls_field_up2(int D, int H, int W, const float* coarse, float* fine);

/* Per-kernel-class device timing (CUDA events on the context stream). */
typedef enum ls_timer {
    LS_T_PROPS = 0,
    LS_T_PRESS_SETUP = 1,
    LS_T_PRESS_INNER = 2,   /* inner PCG iterations incl. the multigrid preconditioner */
    LS_T_PRESS_OUTER = 3,   /* FP64 residual + refinement update */
    LS_T_FLUX = 4,
    LS_T_SATURATION = 5,
    LS_T_TRANSPORT = 6,
    LS_T_PRECIP = 7,
    LS_T_DISSOLVE = 8,
    LS_T_SNAPSHOT = 9,
    LS_T_KRY_APPLY = 10,    /* each transport / implicit-saturation operator-apply launch */
    LS_T_CG_APPLY = 11,     /* each inner pressure operator-apply launch */
    LS_T_COUNT = 12
} ls_timer;
ls_status ls_timing_enable(ls_ctx* ctx, int enable);
ls_status ls_timing_reset(ls_ctx* ctx);
/* Total milliseconds and number of timed regions recorded for a class since the last reset. */
ls_status ls_timing_get(ls_ctx* ctx, ls_timer t, double* total_ms, long long* count);
/* Algorithmic bytes (compulsory reads + writes) moved by the timed launches of a class
   since the last reset; defined for LS_T_KRY_APPLY and LS_T_CG_APPLY. */
ls_status ls_timing_bytes(ls_ctx* ctx, ls_timer t, double* bytes);
/* Count of kernel launches issued by the library since the last reset. */
long long ls_kernel_launches(const ls_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif /* LEACHINGSIM_H_ */
