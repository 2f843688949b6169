// main.cpp - command-line driver with the reference's flags and time loop
// (src/main.cpp:29-594) over the GPU Simulation of Simulation.h.
//
//   leachingsim --raw-file F --xext X --yext Y --zext Z [--dt ..] [--tmax ..] [--nout ..] ...
//
// Options follow src/main.cpp:39 (same names and defaults). Unknown options are passed
// over like Boost's allow_unregistered (src/main.cpp:55); of the PETSc solver options,
// -press_ksp_rtol/-press_ksp_max_it, -conc_ksp_rtol/-conc_ksp_max_it (also -acid_...) and
// -sat_ksp_rtol/-sat_ksp_max_it map onto this library's solvers; the rest are reported
// and ignored. Added options: --label_bits 8|16 (the reference builds one binary per
// width), --solid_density (never set by the reference), --compat_shift, --press_solver
// mixed|fp64|jacobi64, --dry-run (parse, print the resolved configuration, exit).
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "Simulation.h"
#include "vtk_writer.h"

using namespace std;

namespace {

struct Opt {
    string value;
    string help;
    bool required;
    bool set;
};

struct Options {
    map<string, Opt> o;
    vector<string> order;
    vector<string> unregistered;

    void add(const string& name, const string& def, const string& help, bool required = false) {
        o[name] = Opt{def, help, required, false};
        order.push_back(name);
    }
    bool has(const string& n) const { auto it = o.find(n); return it != o.end() && it->second.set; }
    string str(const string& n) const { return o.at(n).value; }
    double num(const string& n) const { return stod(o.at(n).value); }
    long long integer(const string& n) const { return stoll(o.at(n).value); }
    bool flag(const string& n) const {
        string v = o.at(n).value;
        transform(v.begin(), v.end(), v.begin(), ::tolower);
        if (v == "true" || v == "1" || v == "yes" || v == "on") return true;
        if (v == "false" || v == "0" || v == "no" || v == "off") return false;
        throw runtime_error("option --" + n + ": not a boolean: " + o.at(n).value);
    }
};

void usage(const Options& op) {
    cout << "Dynamic Advection-Diffusion Leaching Simulator (GB300)" << endl;
    cout << "Command line arguments:" << endl;
    for (const auto& n : op.order) {
        const Opt& x = op.o.at(n);
        cout << "  --" << left << setw(22) << n << x.help;
        if (!x.required && !x.value.empty()) cout << " (=" << x.value << ")";
        cout << endl;
    }
}

}  // namespace

int main(int argc, char* argv[]) {
    try {
        Options op;
        // src/main.cpp:39
        op.add("help", "", "Print this message and exit.");
        op.add("raw-file", "", "Input RAW file specifying the domain.", true);
        op.add("xext", "", "The x extent of the domain", true);
        op.add("yext", "", "The y extent of the domain", true);
        op.add("zext", "", "The z extent of the domain", true);
        op.add("out_dir", "./output", "The output directory");
        op.add("header_size", "0", "RAW file header size in bytes.");
        op.add("voxel_size", "1", "Size of voxels (m).");
        op.add("D", "1", "Diffusion constant (m^2/s).");
        op.add("kext", "1", "Mass transfer to exterior.");
        op.add("kreac", "1", "Reaction transfer from sulphide grains.");
        op.add("Dpore_fac", "1", "Pore diffusivity enhancement factor");
        op.add("dt", "1", "Simulation time step (s).");
        op.add("tmax", "10", "Maximum simulation time (s).");
        op.add("nout", "1", "Output every N-th time step.");
        op.add("seed", "42", "Pseudo-RNG seed value.");
        op.add("csat", "0.95", "Saturation concentration limit.");
        op.add("evap_flux", "0", "Evaporative flux (m/s)");
        op.add("theta", "1", "Time scheme (0=Explicit, 0.5=Crank-Nicolson, 1.0=Implicit)");
        op.add("instant_precip", "false", "Enable instant pore blinding upon supersaturation");
        op.add("porosity", "0.1", "Material porosity");
        op.add("top_pressure", "10000", "Applied pressure head at the top boundary (Pa)");
        op.add("max_cap_grad", "50000", "Maximum capillary pressure gradient (Pa/m)");
        op.add("implicit_sat", "false", "Toggle: True = Implicit solver, False = Explicit Sub-stepping");
        op.add("restart_step", "0", "Step to restart from (0 = fresh start)");
        op.add("chk_freq", "1000", "Number of steps between saving binary checkpoints");
        op.add("debug", "false", "Enable detailed runtime debugging and NaN checks");
        op.add("use_out_time", "false", "Toggle: output based on physical time instead of nout");
        op.add("out_time", "3600", "Physical time interval between VTK outputs (seconds)");
        op.add("time_scalar", "1", "Physical time accelerator for solid mass transfer");
        op.add("enable_microporosity", "false", "Toggle: acid diffusion and leaching through rock");
        op.add("rock_D_fac", "1e-4", "Multiplier for the diffusion coefficient inside the rock matrix");
        op.add("alpha_transfer", "1e-5", "Mass transfer coefficient for acid entering the rock matrix");
        // added by this implementation
        op.add("label_bits", "8", "Bits per voxel label of the RAW file (8 or 16)");
        op.add("solid_density", "1", "Density of the precipitate (unset in the original code)");
        op.add("compat_shift", "true", "Solve results land one i-plane up, as on the original's rank 0");
        op.add("press_solver", "mixed", "Pressure solver: mixed, fp64, jacobi64 or learned");
        op.add("precond_weights", "", "Weights (.npy) of the learned coarse solver (default: the shipped ones)");
        op.add("bc_mode", "reference",
               "Boundary model: reference (Air surface at the ramped top pressure) or flow (Pore voxels of "
               "z = 0 / z = max held at p_inlet / p_outlet, species inflow at z = 0)");
        op.add("p_inlet", "1", "flow model: pressure of the Pore voxels of the z = 0 plane (Pa)");
        op.add("p_outlet", "0", "flow model: pressure of the Pore voxels of the z = max plane (Pa)");
        op.add("conc_inlet", "0", "flow model: dissolved-mineral concentration flowing in at z = 0");
        op.add("acid_inlet", "0", "flow model: acid concentration flowing in at z = 0");
        op.add("pore_perm", "1e-12", "Intrinsic permeability of Air and clean Pore voxels (m^2)");
        op.add("rock_perm", "1e-18", "Intrinsic permeability of Rock voxels (m^2)");
        op.add("kmult_file", "", "float32 RAW file (k fastest) multiplying each voxel's intrinsic permeability");
        op.add("lean", "false",
               "Lean device layout for domains that do not fit otherwise: the pressure and transport solves "
               "share work memory, no change tracking, the retry snapshot in host memory");
        op.add("dry-run", "false", "Parse the options, print the configuration and exit");

        for (int a = 1; a < argc; ++a) {
            string s = argv[a];
            if (s == "-h" || s == "--help") { usage(op); return 0; }
            if (s.rfind("--", 0) == 0) {
                string name = s.substr(2), val;
                size_t eq = name.find('=');
                bool inl = eq != string::npos;
                if (inl) { val = name.substr(eq + 1); name = name.substr(0, eq); }
                auto it = op.o.find(name);
                if (it == op.o.end()) {
                    op.unregistered.push_back(s);
                    if (!inl && a + 1 < argc && argv[a + 1][0] != '-') op.unregistered.push_back(argv[++a]);
                    continue;
                }
                if (!inl) {
                    if (name == "dry-run") val = "true";
                    else if (a + 1 < argc) val = argv[++a];
                    else throw runtime_error("option --" + name + " needs a value");
                }
                it->second.value = val;
                it->second.set = true;
            } else if (s.size() > 1 && s[0] == '-') {
                // PETSc-style option passed through (src/main.cpp:55)
                op.unregistered.push_back(s);
                if (a + 1 < argc && (argv[a + 1][0] != '-' || isdigit((unsigned char)argv[a + 1][1])))
                    op.unregistered.push_back(argv[++a]);
            } else {
                throw runtime_error("unexpected argument: " + s);
            }
        }
        for (const auto& n : op.order)
            if (op.o[n].required && !op.o[n].set)
                throw runtime_error("the option '--" + n + "' is required but missing");

        const int label_bits = (int)op.integer("label_bits");
        if (label_bits != 8 && label_bits != 16) throw runtime_error("--label_bits must be 8 or 16");
        lsh::Simulation sim((size_t)op.integer("seed"), label_bits / 8);
        sim.D = op.num("D");
        sim.dx = op.num("voxel_size");
        sim.kext = op.num("kext");
        sim.kreac = op.num("kreac");
        sim.Dpore_fac = op.num("Dpore_fac");
        sim.c_sat = op.num("csat");
        sim.evaporative_flux = op.num("evap_flux");
        sim.top_pressure = op.num("top_pressure");
        sim.max_cap_grad = op.num("max_cap_grad");
        sim.theta = op.num("theta");
        sim.use_instant_precipitation = op.flag("instant_precip");
        sim.porosity = op.num("porosity");
        sim.use_implicit_saturation = op.flag("implicit_sat");
        sim.debug_mode = op.flag("debug");
        sim.time_scalar = op.num("time_scalar");
        sim.enable_microporosity = op.flag("enable_microporosity");
        sim.rock_D_fac = op.num("rock_D_fac");
        sim.alpha_transfer = op.num("alpha_transfer");
        sim.solid_density = op.num("solid_density");
        // src/main.cpp:89-91
        sim.vg_n = 2.0;
        sim.vg_alpha = 1.0;
        sim.s_res = 0.05;
        sim.solver.compat_shift = op.flag("compat_shift") ? 1 : 0;
        {
            string bm = op.str("bc_mode");
            if (bm == "reference") sim.solver.bc_mode = LS_BC_REFERENCE;
            else if (bm == "flow") sim.solver.bc_mode = LS_BC_FLOW_I;
            else throw runtime_error("--bc_mode must be reference or flow");
            sim.solver.p_inlet = op.num("p_inlet");
            sim.solver.p_outlet = op.num("p_outlet");
            sim.solver.conc_inlet = op.num("conc_inlet");
            sim.solver.acid_inlet = op.num("acid_inlet");
            sim.solver.pore_permeability = op.num("pore_perm");
            sim.solver.rock_permeability = op.num("rock_perm");
            sim.solver.memory_mode = op.flag("lean") ? LS_MEM_LEAN : LS_MEM_RESIDENT;
        }
        {
            string ps = op.str("press_solver");
            if (ps == "mixed") sim.solver.press_solver = LS_PRESS_MIXED;
            else if (ps == "fp64") sim.solver.press_solver = LS_PRESS_FP64;
            else if (ps == "jacobi64") sim.solver.press_solver = LS_PRESS_JACOBI64;
            else if (ps == "learned") sim.solver.press_solver = LS_PRESS_LEARNED;
            else throw runtime_error("--press_solver must be mixed, fp64, jacobi64 or learned");
            if (ps == "learned") {
                string wp = op.str("precond_weights");
                if (wp.empty()) {
                    // beside the executable, where the package ships them
                    char buf[4096];
                    const ssize_t len = readlink("/proc/self/exe", buf, sizeof(buf) - 1);
                    string exe = len > 0 ? string(buf, (size_t)len) : string(argv[0]);
                    const size_t slash = exe.rfind('/');
                    wp = (slash == string::npos ? string(".") : exe.substr(0, slash)) + "/lpnet_precond_weights.npy";
                }
                sim.precond_weights = lsh::Simulation::loadNpyFloat32(wp);
            }
        }
        // PETSc option passthrough onto this library's solvers
        for (size_t q = 0; q < op.unregistered.size(); ++q) {
            string k = op.unregistered[q];
            string v = (q + 1 < op.unregistered.size()) ? op.unregistered[q + 1] : "";
            auto take = [&](double& dst) { dst = stod(v); ++q; };
            auto takei = [&](int& dst) { dst = stoi(v); ++q; };
            if (k == "-press_ksp_rtol") take(sim.solver.press_rtol);
            else if (k == "-press_ksp_max_it") takei(sim.solver.press_max_it);
            else if (k == "-conc_ksp_rtol" || k == "-acid_ksp_rtol") take(sim.solver.conc_rtol);
            else if (k == "-conc_ksp_max_it" || k == "-acid_ksp_max_it") takei(sim.solver.conc_max_it);
            else if (k == "-sat_ksp_rtol") take(sim.solver.sat_rtol);
            else if (k == "-sat_ksp_max_it") takei(sim.solver.sat_max_it);
            else if (!k.empty() && k[0] == '-') cout << "[Note] option " << k << " is not used by the GPU solvers" << endl;
        }

        // (i, j, k) = (Z, Y, X), src/main.cpp:94
        lsh::int3 global_extent((int)op.integer("zext"), (int)op.integer("yext"), (int)op.integer("xext"));
        string out_dir = op.str("out_dir");

        // diffusive stability clamp, src/main.cpp:104-148
        double dx = sim.dx, D_coeff = sim.D, dt_user = op.num("dt");
        double dt_stable_max = (dx * dx) / (2.0 * D_coeff + 1e-30);
        double dt_actual;
        if (sim.theta >= 0.5) {
            dt_actual = dt_user;
            cout << "Using Theta=" << sim.theta << " (Unconditionally Stable). Using user dt = " << dt_actual
                 << "s." << endl;
        } else {
            double stability_factor = 0.9;
            if (dt_user > dt_stable_max) {
                dt_actual = stability_factor * dt_stable_max;
                cout << "[Warning] Explicit scheme requested. User dt (" << dt_user
                     << "s) exceeds stability limit (" << dt_stable_max << "s). Using adjusted dt = "
                     << dt_actual << "s." << endl;
            } else {
                dt_actual = dt_user;
                cout << "Using user-specified dt = " << dt_actual << "s (stable)." << endl;
            }
        }

        if (op.flag("dry-run")) {
            cout << "configuration:";
            for (const auto& n : op.order) cout << " " << n << "=" << op.o[n].value;
            cout << " press_rtol=" << sim.solver.press_rtol << " press_max_it=" << sim.solver.press_max_it
                 << " conc_rtol=" << sim.solver.conc_rtol << " conc_max_it=" << sim.solver.conc_max_it
                 << " sat_rtol=" << sim.solver.sat_rtol << " sat_max_it=" << sim.solver.sat_max_it
                 << " dt_actual=" << dt_actual << endl;
            return 0;
        }

        sim.setupDomain(global_extent);
        sim.setupPETSc(true);
        sim.readRAW(op.str("raw-file"), (size_t)op.integer("header_size"));
        if (!op.str("kmult_file").empty()) sim.readPermeabilityMultiplier(op.str("kmult_file"));

        double t = 0.0;
        size_t n = 0;
        int start_step = (int)op.integer("restart_step");
        if (start_step > 0) {
            cout << "Restarting simulation from step " << start_step << "..." << endl;
            sim.loadCheckpoint(out_dir, start_step);
            sim.setupReactionRates();
            sim.doExchange();
            sim.updateRelativePermeability();
            sim.updateCapillaryPressure();
            sim.initProperties();
            n = (size_t)start_step;
            t = start_step * dt_actual;
        } else {
            cout << "Initialising new simulation..." << endl;
            sim.initFields();
            sim.initFrac();
            sim.initSaturation();
            sim.initAcid();
            sim.setupReactionRates();
            sim.doExchange();
            sim.updateRelativePermeability();
            sim.updateCapillaryPressure();
            sim.initProperties();
        }

        double tmax = op.num("tmax");
        int nout = (int)op.integer("nout");
        bool use_out_time = op.flag("use_out_time");
        double out_time_interval = op.num("out_time");
        const char* output_mode = use_out_time ? "Physical time based (seconds)" : "Time steps based (timesteps)";
        double output_dump_frequency = use_out_time ? out_time_interval : 1.0 * nout;
        double next_out_time = std::floor(t / out_time_interval) * out_time_interval;
        if (t > 0.0 && t >= next_out_time) next_out_time += out_time_interval;

        // parameter banner, src/main.cpp:240-267
        cout << "\n======================================" << endl;
        cout << "  SIMULATION PARAMETERS" << endl;
        cout << "========================================" << endl;
        cout << "  Input file                       : " << op.str("raw-file") << endl;
        cout << "  Output folder                    : " << out_dir << endl;
        cout << "  Voxel size (dx)                  : " << sim.dx << " m" << endl;
        cout << "  File size in voxels (x, y, z)    : " << "(" << op.str("xext") << ")" << "(" << op.str("yext")
             << ")" << "(" << op.str("zext") << ")" << endl;
        cout << "  Porosity                         : " << sim.porosity << endl;
        cout << "  Diffusion (D)                    : " << sim.D << endl;
        cout << "  Reaction rate (kreac)            : " << sim.kreac << endl;
        cout << "  Saturation limit (csat)          : " << sim.c_sat << endl;
        cout << "  Top Pressure (Irrigation)        : " << sim.top_pressure << " Pa" << endl;
        cout << "  Evaporative flux                 : " << sim.evaporative_flux << endl;
        cout << "  Max Capillary Grad               : " << sim.max_cap_grad << " Pa/m" << endl;
        cout << "  Time step (dt)                   : " << dt_user << " s" << endl;
        cout << "  Time discretisation (Theta)      : " << sim.theta << endl;
        cout << "  Precipitation mode               : "
             << (sim.use_instant_precipitation ? "True (Instant)" : "False (Gradual)") << endl;
        cout << "  Saturation Solver                : "
             << (sim.use_implicit_saturation ? "Implicit (GPU)" : "Explicit (Sub-stepping)") << endl;
        cout << "  Debug Mode                       : " << (sim.debug_mode ? "True (Active)" : "False (Inactive)") << endl;
        cout << "  Output Mode                      : " << output_mode << endl;
        cout << "  Output Frequency                 : " << output_dump_frequency << endl;
        cout << "  Rock Microporosity               : "
             << (sim.enable_microporosity ? "True (Active)" : "False (Inactive)") << endl;
        cout << "  Pore - Rock Transfer factor      : " << sim.alpha_transfer << endl;
        cout << "==================================================\n" << endl;

        mkdir(out_dir.c_str(), 0755);
        cout << "\n*** Starting Simulation ***" << endl;

        // temporal ramping, src/main.cpp:276-287
        double dt_target = dt_actual;
        double current_dt = dt_target;
        bool use_ramping = true;
        if (use_ramping && start_step == 0) {
            current_dt = std::min(60.0, dt_target);
            cout << "Temporal Ramping Enabled: Starting at dt = " << current_dt << "s" << endl;
        }
        vector<double> history_t;
        vector<size_t> history_n;
        const int chk_freq = (int)op.integer("chk_freq");

        do {
            bool step_successful = false;
            while (!step_successful) {
                cout << "\nIteration: " << n << " | Time: " << t << "s | dt: " << current_dt << "s" << endl;
                ls_step_info info;
                step_successful = sim.step(t, current_dt, &info);
                // log lines of the solves, in the order the reference prints them
                const ls_solve_info& P = info.pressure;
                if (P.converged) {
                    cout << "    [Pressure] Converged in " << P.iterations << " iterations. (Reason Code: "
                         << P.reason << ")" << endl;
                    cout << "    [Pressure] Min Value: " << P.min_value << " Pa | Max Value: " << P.max_value
                         << " Pa" << endl;
                } else {
                    cout << "    [Pressure] DIVERGED/FAILED in " << P.iterations << " iterations! (Error Code: "
                         << P.reason << ")" << endl;
                }
                if (P.converged && !sim.use_implicit_saturation) {
                    cout << "    [Saturation] Max div(q): " << info.saturation.max_rate
                         << " | Sub-steps: " << info.saturation.num_steps << " (" << info.saturation.dt_sub
                         << "s)" << endl;
                    if (info.saturation.num_steps > 1)
                        cout << "    [Saturation] Sub-stepping required: " << info.saturation.num_steps
                             << " steps of " << info.saturation.dt_sub << "s." << endl;
                }
                if (step_successful) {
                    cout << "    [Concentration] Converged in " << info.conc.iterations
                         << " iterations. (Reason Code: " << info.conc.reason << ")" << endl;
                    cout << "    [Concentration] Min Value: " << info.conc.min_value
                         << " Pa | Max Value: " << info.conc.max_value << " Pa" << endl;
                    cout << "    [Acid Transport] Converged in " << info.acid.iterations
                         << " iterations. (Reason Code: " << info.acid.reason << ")" << endl;
                    cout << "    [Acid Transport] Min Value: " << info.acid.min_value
                         << " | Max Value: " << info.acid.max_value << endl;
                    cout << "    [Leaching] Max rate: " << info.leaching.max_rate
                         << " | Sub-steps: " << info.leaching.num_steps << " (" << info.leaching.dt_sub
                         << "s)" << endl;
                    sim.total_leached_count += (unsigned long long)info.leached;
                    double percentage = 0.0;
                    if (sim.initial_sulphide_count > 0)
                        percentage = (double)sim.total_leached_count / sim.initial_sulphide_count * 100.0;
                    cout << "Done iteration. [" << info.leached << " voxels fully leached this step.]" << endl;
                    const ls_budget& B = info.budget;
                    cout << "    [Budget] conc: " << std::setprecision(15) << B.conc << " | acid: " << B.acid
                         << " | mineral: " << B.mineral << " | precipitate: " << B.precipitate
                         << " | acid consumed: " << B.acid_consumed << " | mineral dissolved: " << B.mineral_dissolved
                         << " | sulphide voxels: " << B.sulphide_voxels << std::setprecision(6) << endl;
                    cout << "    [Leaching Progress] Total Leached: " << sim.total_leached_count << " / "
                         << sim.initial_sulphide_count << " (" << std::fixed << std::setprecision(4)
                         << percentage << "%)" << std::endl;
                    cout.unsetf(std::ios::fixed);
                    cout << std::setprecision(6);
                }
                if (!step_successful) {
                    cout << "    [Retry Manager] Physics diverged! Rolling back memory and halving dt..." << endl;
                    sim.restoreState();
                    current_dt *= 0.5;
                    if (current_dt < 1e-3) {
                        cout << "    [FATAL ERROR] Time step shrank below 1ms. Simulation is irreversibly "
                                "unstable. Aborting." << endl;
                        return 1;
                    }
                }
            }

            bool trigger_output = false;
            if (use_out_time) {
                if (t >= next_out_time - 1e-6) {
                    trigger_output = true;
                    while (next_out_time <= t) next_out_time += out_time_interval;
                }
            } else if (n % (size_t)nout == 0) {
                trigger_output = true;
            }
            if (trigger_output) {
                cout << "Syncing physical properties for VTK output at t = " << t << "s..." << endl;
                sim.updateRelativePermeability();
                sim.updateCapillaryPressure();
                sim.initProperties();
                cout << "Writing output for time step " << n << "..." << endl;
                size_t flags = lsh::Conc | lsh::Pressure | lsh::Frac | lsh::Type | lsh::Flux_Vec |
                               lsh::Saturation | lsh::CapPressure | lsh::RelPermeability |
                               lsh::Permeability | lsh::AcidConc;
                sim.writeVTKFile(out_dir + "/output", n, flags);
                history_t.push_back(t);
                history_n.push_back(n);
                lsh::write_pvd(out_dir + "/time_mapping.pvd", history_t, history_n);
            }
            if (n > 0 && n % (size_t)chk_freq == 0) sim.writeCheckpoint(out_dir, (int)n);

            t += current_dt;
            n++;
            if (use_ramping && current_dt < dt_target) {
                current_dt *= 1.5;
                if (current_dt > dt_target) {
                    current_dt = dt_target;
                    cout << "    [Time Manager] Ramping complete. Reached target dt = " << dt_target << "s." << endl;
                } else {
                    cout << "    [Time Manager] Accelerating next dt to " << current_dt << "s." << endl;
                }
            }
        } while (t < tmax);
        sim.finishOutput();

        cout << "\n*** Simulation Finished ***" << endl;
    } catch (const std::exception& e) {
        cerr << "An unhandled std::exception occurred on rank 0:" << endl;
        cerr << "\t" << e.what() << endl;
        return 1;
    }
    return 0;
}
