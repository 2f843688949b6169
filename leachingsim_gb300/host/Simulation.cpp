// Simulation.cpp - host-side drop-in Simulation over the C-ABI (see Simulation.h).
// Log lines keep the reference's wording so its log parsers (plot_benchmarks.py
// regexes "Sub-steps:\s+(\d+)", "[Implicit Saturation] Converged in\s+(\d+)") work.
#include "Simulation.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <stdexcept>

#include "vtk_writer.h"

using namespace std;

namespace lsh {

Simulation::Simulation(size_t seed, int label_bytes) : seed_(seed), label_bytes_(label_bytes) {
    ls_params_default(&solver);
}

Simulation::~Simulation() {
    try {
        finishOutput();
    } catch (const std::exception& e) {
        std::cerr << "VTK output: " << e.what() << std::endl;
    }
    for (void* p : out_bufs_) ls_host_free(p);
    if (ctx_) ls_destroy(ctx_);
}

void Simulation::finishOutput() {
    if (writer_.joinable()) writer_.join();
    if (!writer_error_.empty()) {
        std::string e = writer_error_;
        writer_error_.clear();
        throw std::runtime_error(e);
    }
}

void Simulation::check(ls_status st, const char* what) {
    if (st == LS_OK) return;
    std::string msg = std::string(what) + " failed (status " + std::to_string((int)st) + ")";
    if (ctx_) msg += std::string(": ") + ls_last_error(ctx_);
    throw std::runtime_error(msg);
}

void Simulation::sync_params() {
    ls_params p = solver;
    p.D = D;
    p.dx = dx;
    p.Dpore_fac = Dpore_fac;
    p.kext = kext;
    p.kreac = kreac;
    p.theta = theta;
    p.c_sat = c_sat;
    p.evaporative_flux = evaporative_flux;
    p.top_pressure = top_pressure;
    p.max_cap_grad = max_cap_grad;
    p.vg_alpha = vg_alpha;
    p.vg_n = vg_n;
    p.s_res = s_res;
    p.porosity = porosity;
    p.time_scalar = time_scalar;
    p.rock_D_fac = rock_D_fac;
    p.alpha_transfer = alpha_transfer;
    p.solid_density = solid_density;
    p.use_instant_precipitation = use_instant_precipitation;
    p.use_implicit_saturation = use_implicit_saturation;
    p.enable_microporosity = enable_microporosity;
    p.debug_mode = debug_mode;
    if (ctx_) check(ls_set_params(ctx_, &p), "ls_set_params");
}

// Simulation::setupDomain (src/Simulation.cpp:81-103): one domain, no decomposition.
void Simulation::setupDomain(int3 gextent) { global_ = gextent; }

// Simulation::setupPETSc (src/Simulation.cpp:131-159): here the device context.
void Simulation::setupPETSc(bool) {
    if (ctx_) return;
    ls_params p = solver;
    check(ls_create(&ctx_, global_.i, global_.j, global_.k, label_bytes_, &p), "ls_create");
    sync_params();
    if (!precond_weights.empty())
        check(ls_pressure_set_precond_weights(ctx_, precond_weights.data(), (long long)precond_weights.size()),
              "ls_pressure_set_precond_weights");
}

std::vector<float> Simulation::loadNpyFloat32(const std::string& path) {
    std::ifstream fin(path, std::ios::binary);
    if (!fin.is_open()) throw std::runtime_error("Cannot open file: " + path);
    char magic[8];
    fin.read(magic, 8);
    if (!fin || std::string(magic + 1, 5) != "NUMPY") throw std::runtime_error(path + ": not a .npy file");
    size_t hlen = 0;
    unsigned char b[4] = {0, 0, 0, 0};
    const int lenbytes = (unsigned char)magic[6] == 1 ? 2 : 4;  // format version 1: 2-byte length
    fin.read(reinterpret_cast<char*>(b), lenbytes);
    for (int q = lenbytes - 1; q >= 0; --q) hlen = (hlen << 8) | b[q];
    std::string header(hlen, ' ');
    fin.read(&header[0], (std::streamsize)hlen);
    if (!fin || header.find("'<f4'") == std::string::npos || header.find("'fortran_order': False") == std::string::npos)
        throw std::runtime_error(path + ": expected a C-order little-endian float32 array");
    const std::streampos data = fin.tellg();
    fin.seekg(0, std::ios::end);
    const size_t n = (size_t)(fin.tellg() - data) / sizeof(float);
    fin.seekg(data);
    std::vector<float> out(n);
    fin.read(reinterpret_cast<char*>(out.data()), (std::streamsize)(n * sizeof(float)));
    if (!fin) throw std::runtime_error(path + ": short read");
    return out;
}

// Simulation::readRAW (src/Simulation.cpp:68-74, src/MPIRawLoader.h:49-107): the file holds
// k-scanlines in (i, j) order, i.e. one contiguous block after the header.
void Simulation::readRAW(const std::string& fname, size_t header) {
    std::ifstream fin(fname, std::ios::binary);
    if (!fin.is_open()) throw std::runtime_error("Cannot open file: " + fname);
    size_t n = global_.size();
    std::vector<uint8_t> buf(n * label_bytes_);
    fin.seekg((std::streamoff)header);
    fin.read(reinterpret_cast<char*>(buf.data()), (std::streamsize)buf.size());
    if ((size_t)fin.gcount() != buf.size())
        throw std::runtime_error("RAW file " + fname + " is shorter than the domain");
    check(ls_upload_field(ctx_, LS_F_LABEL, buf.data(), n, 0), "label upload");
    props_valid_ = false;
}

void Simulation::readPermeabilityMultiplier(const std::string& fname) {
    std::ifstream fin(fname, std::ios::binary);
    if (!fin.is_open()) throw std::runtime_error("Cannot open file: " + fname);
    size_t n = global_.size();
    std::vector<float> buf(n);
    fin.read(reinterpret_cast<char*>(buf.data()), (std::streamsize)(n * sizeof(float)));
    if ((size_t)fin.gcount() != n * sizeof(float))
        throw std::runtime_error("multiplier file " + fname + " is shorter than the domain");
    check(ls_upload_field(ctx_, LS_F_KMULT, buf.data(), n, 0), "permeability multiplier upload");
    props_valid_ = false;
}

void Simulation::initFields() { check(ls_init_fields(ctx_), "initFields"); props_valid_ = false; }

void Simulation::initFrac() {
    unsigned long long cnt = 0;
    check(ls_init_frac(ctx_, &cnt), "initFrac");
    initial_sulphide_count = cnt;
    total_leached_count = 0;
    props_valid_ = false;
}

void Simulation::initAcid() { check(ls_init_acid(ctx_), "initAcid"); }

void Simulation::initSaturation() { check(ls_init_saturation(ctx_), "initSaturation"); props_valid_ = false; }

// Simulation::setupReactionRates (src/Simulation.cpp:109-125): a rate per grain id, read by
// no physics; kept for interface parity.
void Simulation::setupReactionRates() {
    num_grains_ = 1;
    ks_.assign(num_grains_, kreac);
}

void Simulation::doExchange() {}

void Simulation::props_if_needed() {
    if (props_valid_) return;
    sync_params();
    check(ls_props(ctx_), "properties");
    props_valid_ = true;
}

// The three property updates run as one fused kernel; each call makes sure it has run
// for the current state.
void Simulation::updateRelativePermeability() { props_valid_ = false; props_if_needed(); }
void Simulation::updateCapillaryPressure() { props_if_needed(); }
void Simulation::initProperties() { props_if_needed(); }

void Simulation::setupPressureEqns(double current_time) { press_time_ = current_time; }

bool Simulation::solvePressure() {
    sync_params();
    ls_solve_info info;
    ls_status st = ls_pressure_step(ctx_, press_time_, &info);
    if (st != LS_OK && st != LS_NOT_CONVERGED && st != LS_NONFINITE && st != LS_STAGNATED_FALLBACK_USED)
        check(st, "solvePressure");
    bool ok = info.converged != 0;
    if (ok) {
        cout << "    [Pressure] Converged in " << info.iterations << " iterations. (Reason Code: "
             << info.reason << ")" << endl;
        cout << "    [Pressure] Min Value: " << info.min_value << " Pa | Max Value: " << info.max_value
             << " Pa" << endl;
    } else {
        cout << "    [Pressure] DIVERGED/FAILED in " << info.iterations
             << " iterations! (Error Code: " << info.reason << ")" << endl;
    }
    return ok;
}

void Simulation::calculateFlux() { check(ls_flux(ctx_), "calculateFlux"); }

void Simulation::updateSaturation(double dt) {
    ls_substep_info info;
    check(ls_saturation(ctx_, dt, &info), "updateSaturation");
    cout << "    [Saturation] Max div(q): " << info.max_rate << " | Sub-steps: " << info.num_steps
         << " (" << info.dt_sub << "s)" << endl;
    if (info.num_steps > 1)
        cout << "    [Saturation] Sub-stepping required: " << info.num_steps << " steps of "
             << info.dt_sub << "s." << endl;
    props_valid_ = false;
}

void Simulation::setupSaturationEqns(double dt) { sat_dt_ = dt; }

bool Simulation::solveSaturation() {
    ls_solve_info info;
    ls_status st = ls_saturation_implicit(ctx_, sat_dt_, &info);
    if (st != LS_OK && st != LS_NOT_CONVERGED && st != LS_UNPHYSICAL && st != LS_NONFINITE)
        check(st, "solveSaturation");
    physics_valid = (st != LS_UNPHYSICAL);
    bool conv = info.converged != 0;
    if (conv && physics_valid) {
        cout << "    [Implicit Saturation] Converged in " << info.iterations
             << " iterations. (Reason Code: " << info.reason << ")" << endl;
        cout << "    [Implicit Saturation] Raw Min: " << info.min_value << " | Raw Max: " << info.max_value
             << endl;
    } else {
        int fail_code = conv ? -99 : info.reason;
        cout << "    [Implicit Saturation] DIVERGED/FAILED in " << info.iterations
             << " iterations. (Error/Physics Code: " << fail_code << ")" << endl;
        cout << "    [Implicit Saturation] Unphysical Raw Min: " << info.min_value
             << " | Raw Max: " << info.max_value << endl;
    }
    props_valid_ = false;
    return conv;
}

void Simulation::handleSurfaceEffects() { check(ls_surface(ctx_), "handleSurfaceEffects"); props_valid_ = false; }

void Simulation::setupConcentrationEqns(double dt, int field, double, double) {
    conc_dt_ = dt;
    conc_pending_ |= (field == 0) ? 1 : 2;
}

static void log_transport(const char* tag, const ls_solve_info& info, bool pa) {
    if (info.converged) {
        cout << "    [" << tag << "] Converged in " << info.iterations << " iterations. (Reason Code: "
             << info.reason << ")" << endl;
        cout << "    [" << tag << "] Min Value: " << info.min_value << (pa ? " Pa" : "")
             << " | Max Value: " << info.max_value << (pa ? " Pa" : "") << endl;
    } else {
        cout << "    [" << tag << "] DIVERGED/FAILED in " << info.iterations << " iterations"
             << (pa ? "! (Error Code: " : ". (Error Code: ") << info.reason << ")" << endl;
    }
}

bool Simulation::solveConc() {
    ls_solve_info ci;
    ls_status st = ls_transport(ctx_, conc_dt_, 1, &ci, nullptr);
    if (st != LS_OK && st != LS_NOT_CONVERGED && st != LS_NONFINITE) check(st, "solveConc");
    conc_pending_ &= ~1;
    log_transport("Concentration", ci, true);
    return ci.converged != 0;
}

bool Simulation::solveAcid() {
    ls_solve_info ai;
    ls_status st = ls_transport(ctx_, conc_dt_, 2, nullptr, &ai);
    if (st != LS_OK && st != LS_NOT_CONVERGED && st != LS_NONFINITE) check(st, "solveAcid");
    conc_pending_ &= ~2;
    log_transport("Acid Transport", ai, false);
    return ai.converged != 0;
}

void Simulation::handlePrecipitation() { check(ls_precip(ctx_), "handlePrecipitation"); props_valid_ = false; }

int Simulation::updateFrac(double dt) {
    int leached = 0;
    ls_substep_info info;
    check(ls_dissolve(ctx_, dt, &leached, &info), "updateFrac");
    cout << "    [Leaching] Max rate: " << info.max_rate << " | Sub-steps: " << info.num_steps << " ("
         << info.dt_sub << "s)" << endl;
    if (info.num_steps > 1)
        cout << "    [Leaching] Sub-stepping required: " << info.num_steps << " steps of " << info.dt_sub
             << "s." << endl;
    props_valid_ = false;
    return leached;
}

void Simulation::saveState() { check(ls_snapshot(ctx_), "saveState"); }

void Simulation::restoreState() {
    check(ls_rollback(ctx_), "restoreState");
    props_valid_ = true;  // ls_rollback rebuilds the properties
}

bool Simulation::step(double t, double dt, ls_step_info* info) {
    sync_params();
    ls_step_info loc;
    check(ls_step(ctx_, t, dt, &loc), "step");
    if (info) *info = loc;
    props_valid_ = false;
    return loc.success != 0;
}

template <typename T>
std::vector<T> Simulation::download(ls_field f) {
    std::vector<T> v(global_.size());
    check(ls_download_field(ctx_, f, v.data(), v.size(), 0), "download");
    return v;
}

template std::vector<double> Simulation::download<double>(ls_field);
template std::vector<float> Simulation::download<float>(ls_field);
template std::vector<uint8_t> Simulation::download<uint8_t>(ls_field);
template std::vector<uint16_t> Simulation::download<uint16_t>(ls_field);

// Simulation::writeVTKFile (src/Simulation.cpp:1306-1566), one piece (np=1). The fields are
// copied to page-locked buffers on the context's copy stream and the piece is written from
// them on a background thread, so the time loop goes on while the copies drain and the file
// is encoded (the next steps' kernels wait on the device only for the copies of the fields
// they overwrite). The reference scrubs NaNs of Pressure and CapillaryPressure in place
// (src/Simulation.cpp:1487-1517): when the device counts any, this output takes the
// synchronous path that does the same.
void Simulation::writeVTKFile(const std::string& fname_root, size_t tstep, size_t data_flags) {
    finishOutput();  // the previous piece is written and its buffers are free
    const size_t n = global_.size();
    struct Want { size_t flag; ls_field f; size_t esz; };
    const Want wants[] = {{Type, LS_F_LABEL, (size_t)label_bytes_}, {Conc, LS_F_CONC, 8}, {Pressure, LS_F_PRESSURE, 8},
                          {Frac, LS_F_FRAC, 4}, {Flux_Vec, LS_F_FLUX_X, 8}, {Flux_Vec, LS_F_FLUX_Y, 8},
                          {Flux_Vec, LS_F_FLUX_Z, 8}, {Saturation, LS_F_SATURATION, 8},
                          {CapPressure, LS_F_CAP_PRESSURE, 8}, {RelPermeability, LS_F_REL_PERM, 8},
                          {Permeability, LS_F_PERMEABILITY, 8}, {AcidConc, LS_F_ACID, 8}};
    const int nw = (int)(sizeof(wants) / sizeof(wants[0]));
    long long nan_p = 0, nan_c = 0;
    if (data_flags & Pressure) check(ls_count_nonfinite(ctx_, LS_F_PRESSURE, &nan_p), "count NaN");
    if (data_flags & CapPressure) check(ls_count_nonfinite(ctx_, LS_F_CAP_PRESSURE, &nan_c), "count NaN");
    if (out_bufs_.empty() && nan_p == 0 && nan_c == 0) {
        out_bufs_.assign(nw, nullptr);
        for (int q = 0; q < nw; ++q) {
            out_bufs_[q] = ls_host_alloc(n * wants[q].esz);
            if (!out_bufs_[q]) {  // no page-locked memory: synchronous output from now on
                for (void*& p : out_bufs_) ls_host_free(p), p = nullptr;
                out_bufs_.assign(1, nullptr);
                break;
            }
        }
    }
    const bool async = nan_p == 0 && nan_c == 0 && out_bufs_.size() == (size_t)nw;
    std::vector<std::vector<char>> sync_bufs;
    void* ptr[12] = {};
    if (async) {
        int ids[12];
        void* hosts[12];
        int cnt = 0;
        for (int q = 0; q < nw; ++q)
            if (data_flags & wants[q].flag) {
                ids[cnt] = (int)wants[q].f;
                hosts[cnt++] = out_bufs_[q];
                ptr[q] = out_bufs_[q];
            }
        void* done = nullptr;
        check(ls_download_fields_async(ctx_, cnt, ids, hosts, 0, &done), "download fields");
        write_pvti(fname_root, tstep, global_.i, global_.j, global_.k, data_flags, label_bytes_);
        VtkFields fields;
        fields.label_bytes = label_bytes_;
        fields.label = ptr[0];
        fields.conc = (const double*)ptr[1];
        fields.pressure = (const double*)ptr[2];
        fields.frac = (const float*)ptr[3];
        fields.fx = (const double*)ptr[4];
        fields.fy = (const double*)ptr[5];
        fields.fz = (const double*)ptr[6];
        fields.sat = (const double*)ptr[7];
        fields.pc = (const double*)ptr[8];
        fields.kr = (const double*)ptr[9];
        fields.perm = (const double*)ptr[10];
        fields.acid = (const double*)ptr[11];
        std::stringstream piece;
        piece << fname_root << "_0_" << setw(6) << setfill('0') << tstep << ".vti";
        const int3 g = global_;
        std::string path = piece.str();
        writer_ = std::thread([this, done, path, g, data_flags, fields]() {
            try {
                if (ls_event_wait(done) != LS_OK) throw std::runtime_error("field copies failed");
                write_vti(path, g.i, g.j, g.k, data_flags, fields);
            } catch (const std::exception& e) {
                writer_error_ = std::string("writing ") + path + ": " + e.what();
            }
            ls_event_release(done);
        });
        return;
    }
    // synchronous path (NaN scrub, or no page-locked memory)
    sync_bufs.resize(nw);
    for (int q = 0; q < nw; ++q)
        if (data_flags & wants[q].flag) {
            sync_bufs[q].resize(n * wants[q].esz);
            check(ls_download_field(ctx_, wants[q].f, sync_bufs[q].data(), n, 0), "download");
            ptr[q] = sync_bufs[q].data();
        }
    int scrub_p = 0, scrub_c = 0;
    auto scrub = [&](int q, int& cnt) {
        if (!ptr[q]) return;
        double* v = (double*)ptr[q];
        for (size_t r = 0; r < n; ++r)
            if (std::isnan(v[r]) || std::isinf(v[r])) { v[r] = 0.0; cnt++; }
    };
    scrub(2, scrub_p);
    scrub(8, scrub_c);
    if (scrub_p > 0) check(ls_upload_field(ctx_, LS_F_PRESSURE, ptr[2], n, 0), "upload P");
    if (scrub_c > 0) check(ls_upload_field(ctx_, LS_F_CAP_PRESSURE, ptr[8], n, 0), "upload Pc");
    if (scrub_p > 0 || scrub_c > 0)
        cout << "    [VTK Writer Rank 0] checked " << scrub_p << " Pressure NaNs and " << scrub_c
             << " CapPressure NaNs from boundary padding." << endl;
    write_pvti(fname_root, tstep, global_.i, global_.j, global_.k, data_flags, label_bytes_);
    VtkFields fields;
    fields.label_bytes = label_bytes_;
    fields.label = ptr[0];
    fields.conc = (const double*)ptr[1];
    fields.pressure = (const double*)ptr[2];
    fields.frac = (const float*)ptr[3];
    fields.fx = (const double*)ptr[4];
    fields.fy = (const double*)ptr[5];
    fields.fz = (const double*)ptr[6];
    fields.sat = (const double*)ptr[7];
    fields.pc = (const double*)ptr[8];
    fields.kr = (const double*)ptr[9];
    fields.perm = (const double*)ptr[10];
    fields.acid = (const double*)ptr[11];
    std::stringstream piece;
    piece << fname_root << "_0_" << setw(6) << setfill('0') << tstep << ".vti";
    write_vti(piece.str(), global_.i, global_.j, global_.k, data_flags, fields);
}

// Simulation::writeCheckpoint / loadCheckpoint (src/Simulation.cpp:2235-2307): the padded
// (I+1)*J*K arrays in the order img, frac, precipitate, saturation, pressure, conc, acid.
void Simulation::writeCheckpoint(const std::string& out_dir, int step) {
    finishOutput();  // the output written before a checkpoint is complete on disk with it
    std::stringstream fname;
    fname << out_dir << "/checkpoint_rank0_" << setw(6) << setfill('0') << step << ".bin";
    std::ofstream fout(fname.str(), std::ios::out | std::ios::binary);
    if (!fout.is_open()) {
        cerr << "    [Error] Rank 0 failed to open checkpoint file for writing!" << endl;
        return;
    }
    const size_t np = (size_t)(global_.i + 1) * global_.j * global_.k;
    std::vector<uint8_t> buf(np * 8);
    check(ls_download_field(ctx_, LS_F_LABEL, buf.data(), np, 1), "checkpoint label");
    fout.write(reinterpret_cast<char*>(buf.data()), (std::streamsize)(np * label_bytes_));
    check(ls_download_field(ctx_, LS_F_FRAC, buf.data(), np, 1), "checkpoint frac");
    fout.write(reinterpret_cast<char*>(buf.data()), (std::streamsize)(np * 4));
    const ls_field f64[] = {LS_F_PRECIPITATE, LS_F_SATURATION, LS_F_PRESSURE, LS_F_CONC, LS_F_ACID};
    for (ls_field f : f64) {
        check(ls_download_field(ctx_, f, buf.data(), np, 1), "checkpoint field");
        fout.write(reinterpret_cast<char*>(buf.data()), (std::streamsize)(np * 8));
    }
    cout << "    [Checkpoint] Successfully saved binary state for step " << step << " to " << out_dir
         << endl;
}

void Simulation::loadCheckpoint(const std::string& out_dir, int step) {
    std::stringstream fname;
    fname << out_dir << "/checkpoint_rank0_" << setw(6) << setfill('0') << step << ".bin";
    std::ifstream fin(fname.str(), std::ios::in | std::ios::binary);
    if (!fin.is_open())
        throw std::runtime_error("    [Fatal Error] Rank 0 failed to locate checkpoint file: " + fname.str());
    const size_t np = (size_t)(global_.i + 1) * global_.j * global_.k;
    std::vector<uint8_t> buf(np * 8);
    auto rd = [&](size_t bytes) {
        fin.read(reinterpret_cast<char*>(buf.data()), (std::streamsize)bytes);
        if ((size_t)fin.gcount() != bytes) throw std::runtime_error("checkpoint file truncated: " + fname.str());
    };
    rd(np * label_bytes_);
    check(ls_upload_field(ctx_, LS_F_LABEL, buf.data(), np, 1), "checkpoint label");
    rd(np * 4);
    check(ls_upload_field(ctx_, LS_F_FRAC, buf.data(), np, 1), "checkpoint frac");
    const ls_field f64[] = {LS_F_PRECIPITATE, LS_F_SATURATION, LS_F_PRESSURE, LS_F_CONC, LS_F_ACID};
    for (ls_field f : f64) {
        rd(np * 8);
        check(ls_upload_field(ctx_, f, buf.data(), np, 1), "checkpoint field");
    }
    props_valid_ = false;
    cout << "    [Checkpoint] Successfully loaded binary state from step " << step << endl;
}

}  // namespace lsh
