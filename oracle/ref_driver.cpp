// ref_driver.cpp - C entry points over the reference's own Simulation class (src/Simulation.h),
// compiled unchanged from the reference's sources with the single-rank shims of ref_shim/.
//
// TEST INFRASTRUCTURE ONLY: this is the parity library oracle/_ref/liblsref_u{8,16}.so that
// tests/test_ref_pin.py loads (through oracle/refsim.py) to check oracle/ls_oracle.c against
// the reference's code. It is built only where the reference's sources are present
// (oracle/build_ref.py) and is never part of the product.
//
// Every call returns 0 on success and -1 when the reference threw (lsref_last_error has the
// message): its bounds-checked indexing throws on some inputs (src/Domain.cpp:107-117).
#include <cstdlib>
#include <cstring>
#include <exception>
#include <new>
#include <stdexcept>
#include <string>

#include "Simulation.h"
#include "leachingsim.h"

// Array allocations of this library start zeroed. The reference leaves some arrays it
// allocates with new T[] uninitialised and reads them back (the saturation of voxels the
// explicit update skips, src/Simulation.cpp:1781-1848, a quirk the oracle defines as 0.0,
// the value of fresh pages); zeroing every new[] gives the reference that same value here.
// The library is linked with -Bsymbolic, so these definitions serve its own code only.
void* operator new[](std::size_t n) {
    void* p = std::calloc(1, n ? n : 1);
    if (!p) throw std::bad_alloc();
    return p;
}
void operator delete[](void* p) noexcept { std::free(p); }
void operator delete[](void* p, std::size_t) noexcept { std::free(p); }

namespace {
std::string g_err;

template <typename F>
int guard(F&& f) {
    try {
        f();
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
    } catch (...) {
        g_err = "unknown exception";
    }
    return -1;
}
}  // namespace

extern "C" {

const char* lsref_last_error(void) { return g_err.c_str(); }
int lsref_label_bytes(void) { return (int)sizeof(RAWType); }

// A Simulation of extents (I, J, K) = (zext, yext, xext) with the physical parameters of p
// (the fields of the reference's public members; the solver tolerances go through
// lsref_option, like the reference's PETSc command-line options).
void* lsref_create(int I, int J, int K, const ls_params* p) {
    Simulation* s = nullptr;
    int rc = guard([&] {
        Domain::BuildMPIDataType();
        s = new Simulation(42);
        s->D = p->D;
        s->dx = p->dx;
        s->Dpore_fac = p->Dpore_fac;
        s->kext = p->kext;
        s->kreac = p->kreac;
        s->theta = p->theta;
        s->use_gamma = false;
        s->c_sat = p->c_sat;
        s->evaporative_flux = p->evaporative_flux;
        s->top_pressure = p->top_pressure;
        s->max_cap_grad = p->max_cap_grad;
        s->vg_alpha = p->vg_alpha;
        s->vg_n = p->vg_n;
        s->s_res = p->s_res;
        s->use_instant_precipitation = p->use_instant_precipitation != 0;
        s->use_implicit_saturation = p->use_implicit_saturation != 0;
        s->solid_density = p->solid_density;
        s->porosity = p->porosity;
        s->alpha_transfer = p->alpha_transfer;
        s->time_scalar = p->time_scalar;
        s->enable_microporosity = p->enable_microporosity != 0;
        s->rock_D_fac = p->rock_D_fac;
        s->debug_mode = p->debug_mode != 0;
        s->physics_valid = true;
        s->setupDomain(int3(I, J, K));
        s->setupPETSc(true);
    });
    if (rc != 0) {
        delete s;
        return nullptr;
    }
    return s;
}

void lsref_destroy(void* h) { delete static_cast<Simulation*>(h); }

void lsref_option(const char* name, const char* value) { lsref_options_set(name, value); }

// The padded array of a field ((I+1)*J*K elements; ls_field numbering) and its element size.
void* lsref_field(void* h, int field, int* elem_bytes) {
    Simulation* s = static_cast<Simulation*>(h);
    switch (field) {
    case LS_F_LABEL: *elem_bytes = (int)sizeof(RAWType); return s->img_data.getData().get();
    case LS_F_FRAC: *elem_bytes = 4; return s->frac.getData().get();
    case LS_F_PERMEABILITY: *elem_bytes = 8; return s->permeability.getData().get();
    case LS_F_VISCOSITY: *elem_bytes = 8; return s->viscosity.getData().get();
    case LS_F_PRESSURE: *elem_bytes = 8; return s->pressure.getData().get();
    case LS_F_CONC: *elem_bytes = 8; return s->conc.getData().get();
    case LS_F_ACID: *elem_bytes = 8; return s->conc_acid.getData().get();
    case LS_F_FLUX_X: *elem_bytes = 8; return s->flux_x.getData().get();
    case LS_F_FLUX_Y: *elem_bytes = 8; return s->flux_y.getData().get();
    case LS_F_FLUX_Z: *elem_bytes = 8; return s->flux_z.getData().get();
    case LS_F_SATURATION: *elem_bytes = 8; return s->saturation.getData().get();
    case LS_F_CAP_PRESSURE: *elem_bytes = 8; return s->cap_pressure.getData().get();
    case LS_F_REL_PERM: *elem_bytes = 8; return s->rel_permeability.getData().get();
    case LS_F_PRECIPITATE: *elem_bytes = 8; return s->precipitate_inventory.getData().get();
    default: *elem_bytes = 0; return nullptr;
    }
}

// src/main.cpp:189-206 (a fresh start; the labels are set through lsref_field first)
int lsref_init(void* h) {
    Simulation* s = static_cast<Simulation*>(h);
    return guard([&] {
        s->initFields();
        s->initFrac();
        s->initSaturation();
        s->initAcid();
        s->setupReactionRates();
        s->doExchange();
        s->updateRelativePermeability();
        s->updateCapillaryPressure();
        s->initProperties();
    });
}

unsigned long long lsref_initial_sulphide_count(void* h) {
    return static_cast<Simulation*>(h)->initial_sulphide_count;
}

// One method of the time step at a time (names as in src/Simulation.h:42-72).
int lsref_call(void* h, const char* method, double arg, int* result) {
    Simulation* s = static_cast<Simulation*>(h);
    const std::string m = method;
    int r = 0;
    int rc = guard([&] {
        if (m == "updateRelativePermeability") s->updateRelativePermeability();
        else if (m == "updateCapillaryPressure") s->updateCapillaryPressure();
        else if (m == "initProperties") s->initProperties();
        else if (m == "setupPressureEqns") s->setupPressureEqns(arg);
        else if (m == "solvePressure") r = s->solvePressure() ? 1 : 0;
        else if (m == "calculateFlux") s->calculateFlux();
        else if (m == "updateSaturation") s->updateSaturation(arg);
        else if (m == "setupSaturationEqns") s->setupSaturationEqns(arg);
        else if (m == "solveSaturation") r = s->solveSaturation() ? 1 : 0;
        else if (m == "handleSurfaceEffects") s->handleSurfaceEffects();
        else if (m == "setupConcentrationEqns_conc") s->setupConcentrationEqns(arg, s->conc, 0.0, 1.0);
        else if (m == "solveConc") r = s->solveConc() ? 1 : 0;
        else if (m == "setupConcentrationEqns_acid") s->setupConcentrationEqns(arg, s->conc_acid, 1.0, 0.0);
        else if (m == "solveAcid") r = s->solveAcid() ? 1 : 0;
        else if (m == "handlePrecipitation") s->handlePrecipitation();
        else if (m == "updateFrac") r = s->updateFrac(arg);
        else if (m == "saveState") s->saveState();
        else if (m == "restoreState") s->restoreState();
        else if (m == "physics_valid") r = s->physics_valid ? 1 : 0;
        else throw std::runtime_error("unknown method " + m);
    });
    if (result) *result = r;
    return rc;
}

// Simulation::writeCheckpoint / loadCheckpoint (src/Simulation.cpp:2235-2307) into / from
// <dir>/checkpoint_rank0_<step>.bin
int lsref_checkpoint(void* h, const char* dir, int step, int write) {
    Simulation* s = static_cast<Simulation*>(h);
    return guard([&] {
        if (write) s->writeCheckpoint(dir, step);
        else s->loadCheckpoint(dir, step);
    });
}

}  // extern "C"
