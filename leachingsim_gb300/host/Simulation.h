// Simulation.h - host-side drop-in for the reference's Simulation class
// (src/Simulation.h:29-186): the same public method names, arguments and bool
// success returns, with every field held on the GPU behind the C-ABI of
// include/leachingsim.h. Host copies exist only while writing VTK output or
// checkpoints.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <thread>
#include <vector>

#include "leachingsim.h"

namespace lsh {

struct int3 {
    int i, j, k;
    int3() : i(0), j(0), k(0) {}
    int3(int a, int b, int c) : i(a), j(b), k(c) {}
    size_t size() const { return (size_t)i * (size_t)j * (size_t)k; }
};

// VTK output selection bits (src/Simulation.h:9-21)
enum VTKOutput {
    Conc = 0x001,
    Frac = 0x004,
    Type = 0x008,
    Pressure = 0x010,
    Permeability = 0x020,
    Saturation = 0x040,
    Flux_Vec = 0x080,
    CapPressure = 0x100,
    RelPermeability = 0x200,
    AcidConc = 0x400
};

class Simulation {
public:
    explicit Simulation(size_t seed, int label_bytes = 1);
    ~Simulation();
    Simulation(const Simulation&) = delete;
    Simulation& operator=(const Simulation&) = delete;

    // setup and I/O (src/Simulation.cpp:68-159)
    void setupDomain(int3 global_extent);
    void setupPETSc(bool zero_conc);
    void readRAW(const std::string& fname, size_t header);
    // Per-voxel multiplier of the intrinsic permeability from a float32 RAW file (k fastest,
    // no header); an extension with no counterpart in the reference.
    void readPermeabilityMultiplier(const std::string& fname);
    void writeVTKFile(const std::string& fname_root, size_t tstep, size_t data_flags);
    // Waits for the piece file of the last writeVTKFile (written on a background thread while
    // the time loop goes on); rethrows its error. Called by the next writeVTKFile, by
    // writeCheckpoint and by the destructor.
    void finishOutput();

    // initialisation and time stepping
    void initProperties();
    void initFields();
    void initFrac();
    void initAcid();
    void initSaturation();
    void setupReactionRates();
    int updateFrac(double dt);
    void doExchange();  // single domain: nothing to exchange

    void updateSaturation(double dt);
    void updateCapillaryPressure();
    void updateRelativePermeability();
    void handleSurfaceEffects();
    void handlePrecipitation();

    void setupPressureEqns(double current_time);
    // field: 0 = conc, 1 = conc_acid (the reference passes the MPIDomain itself)
    void setupConcentrationEqns(double dt, int field, double inlet_bc, double sulphide_bc);
    void setupSaturationEqns(double dt);
    void calculateFlux();

    bool solveAcid();
    bool solvePressure();
    bool solveSaturation();
    bool solveConc();

    void saveState();
    void restoreState();

    void writeCheckpoint(const std::string& out_dir, int step);
    void loadCheckpoint(const std::string& out_dir, int step);

    // one attempt of src/main.cpp:303-432 with conc and acid solved together
    bool step(double t, double dt, ls_step_info* info);

    // public parameters (src/Simulation.h:75-114)
    double D = 1.0, dx = 1.0, Dpore_fac = 1.0, kext = 1.0, kreac = 1.0, theta = 1.0;
    bool use_gamma = false;
    double gamma_alpha = 0.0, gamma_beta = 0.0;
    double c_sat = 0.95, evaporative_flux = 0.0, top_pressure = 10000.0, max_cap_grad = 50000.0;
    double vg_alpha = 1.0, vg_n = 2.0, s_res = 0.05;
    bool use_instant_precipitation = false, use_implicit_saturation = false;
    double solid_density = 1.0, porosity = 0.1;
    double alpha_transfer = 1e-5;
    double time_scalar = 1.0;
    bool enable_microporosity = false;
    double rock_D_fac = 1e-4;
    bool debug_mode = false;
    bool physics_valid = true;
    unsigned long long initial_sulphide_count = 0;
    unsigned long long total_leached_count = 0;
    // solver controls (mapped from -press_/-conc_/-acid_/-sat_ PETSc options)
    ls_params solver;
    // weights of the learned coarse solver (press_solver = LS_PRESS_LEARNED), handed to the
    // context when it is created
    std::vector<float> precond_weights;
    // Read a little-endian float32 .npy vector (the trained weights as saved by numpy).
    static std::vector<float> loadNpyFloat32(const std::string& path);

    int rank() const { return 0; }
    int3 global_extent() const { return global_; }
    ls_ctx* context() { return ctx_; }
    // Download one field into a host vector (unpadded, I*J*K elements).
    template <typename T>
    std::vector<T> download(ls_field f);

private:
    void sync_params();
    void check(ls_status st, const char* what);
    void props_if_needed();

    size_t seed_;
    int label_bytes_;
    int3 global_;
    ls_ctx* ctx_ = nullptr;
    std::vector<uint8_t> pending_labels_;
    bool props_valid_ = false;
    double press_time_ = 0.0;
    double conc_dt_ = 1.0;
    double sat_dt_ = 1.0;
    int conc_pending_ = 0;  // bit 0 conc, bit 1 acid set up and not yet solved
    size_t num_grains_ = 0;
    std::vector<double> ks_;
    // asynchronous output: page-locked copies of the fields (ls_download_fields_async) and the
    // thread that writes the .vti piece from them once they have landed
    std::vector<void*> out_bufs_;
    std::thread writer_;
    std::string writer_error_;
};

}  // namespace lsh
