// vtk_writer.h - VTK XML image output of one domain: the .pvti master, the .vti piece
// and the .pvd time collection of the reference (src/Simulation.cpp:1306-1566,
// src/main.cpp:512-525). The piece is written with appended raw binary data.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace lsh {

struct VtkFields {
    std::vector<uint8_t> label;  // label_bytes per voxel
    int label_bytes = 1;
    std::vector<double> conc, pressure, fx, fy, fz, sat, pc, kr, perm, acid;
    std::vector<float> frac;
};

// Voxel (i,j,k) of an I x J x K domain is stored at k + K*(j + J*i); VTK's x axis is i.
void write_pvti(const std::string& fname_root, size_t tstep, int I, int J, int K, size_t flags,
                int label_bytes);
void write_vti(const std::string& path, int I, int J, int K, size_t flags, const VtkFields& f);
void write_pvd(const std::string& path, const std::vector<double>& times,
               const std::vector<size_t>& steps);

}  // namespace lsh
