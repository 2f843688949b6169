// vtk_writer.h - VTK XML image output of one domain: the .pvti master, the .vti piece
// and the .pvd time collection of the reference (src/Simulation.cpp:1306-1566,
// src/main.cpp:512-525). The piece is written with appended raw binary data.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace lsh {

// The arrays of one output (null: not written), each I*J*K values in the solver's order;
// the memory belongs to the caller.
struct VtkFields {
    const void* label = nullptr;  // label_bytes per voxel
    int label_bytes = 1;
    const double *conc = nullptr, *pressure = nullptr, *fx = nullptr, *fy = nullptr, *fz = nullptr,
                 *sat = nullptr, *pc = nullptr, *kr = nullptr, *perm = nullptr, *acid = nullptr;
    const float* frac = nullptr;
};

// Voxel (i,j,k) of an I x J x K domain is stored at k + K*(j + J*i); VTK's x axis is i.
void write_pvti(const std::string& fname_root, size_t tstep, int I, int J, int K, size_t flags,
                int label_bytes);
void write_vti(const std::string& path, int I, int J, int K, size_t flags, const VtkFields& f);
void write_pvd(const std::string& path, const std::vector<double>& times,
               const std::vector<size_t>& steps);

}  // namespace lsh
