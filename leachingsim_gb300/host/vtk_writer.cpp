// vtk_writer.cpp - see vtk_writer.h.
#include "vtk_writer.h"

#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <stdexcept>

#include "Simulation.h"

using namespace std;

namespace lsh {

// Array list in the order the reference adds them (src/Simulation.cpp:1401-1485).
struct ArraySpec {
    size_t flag;
    const char* type;
    const char* name;
    int ncomp;
};

static std::vector<ArraySpec> specs(size_t flags, int label_bytes) {
    std::vector<ArraySpec> v;
    if (flags & Type) v.push_back({Type, label_bytes == 2 ? "UInt16" : "UInt8", "MaterialType", 1});
    if (flags & Conc) v.push_back({Conc, "Float64", "Concentration", 1});
    if (flags & Pressure) v.push_back({Pressure, "Float64", "Pressure", 1});
    if (flags & Frac) v.push_back({Frac, "Float32", "SulphideFrac", 1});
    if (flags & Flux_Vec) v.push_back({Flux_Vec, "Float64", "Flux", 3});
    if (flags & Saturation) v.push_back({Saturation, "Float64", "Saturation", 1});
    if (flags & CapPressure) v.push_back({CapPressure, "Float64", "CapillaryPressure", 1});
    if (flags & RelPermeability) v.push_back({RelPermeability, "Float64", "RelativePermeability", 1});
    if (flags & Permeability) v.push_back({Permeability, "Float64", "EffectivePermeability", 1});
    if (flags & AcidConc) v.push_back({AcidConc, "Float64", "AcidConcentration", 1});
    return v;
}

// master file, src/Simulation.cpp:1309-1375 (np=1: one piece, no overlap)
void write_pvti(const std::string& fname_root, size_t tstep, int I, int J, int K, size_t flags,
                int label_bytes) {
    stringstream fname;
    fname << fname_root << "_" << setw(6) << setfill('0') << tstep << ".pvti";
    ofstream fout(fname.str().c_str());
    if (!fout.is_open()) throw std::runtime_error("cannot write " + fname.str());
    fout << "<?xml version=\"1.0\"?>" << endl;
    fout << "<VTKFile type=\"PImageData\" version=\"0.1\">" << endl;
    fout << "\t<PImageData WholeExtent=\"0 " << I - 1 << " 0 " << J - 1 << " 0 " << K - 1 << "\" ";
    fout << "GhostLevel=\"0\" Origin=\"0 0 0\" Spacing=\"1 1 1\">" << endl;
    fout << "\t\t<PPointData>" << endl;
    for (const auto& s : specs(flags, label_bytes)) {
        fout << "\t\t\t<PDataArray type=\"" << s.type << "\" Name=\"" << s.name << "\"";
        if (s.ncomp > 1) fout << " NumberOfComponents=\"" << s.ncomp << "\"";
        fout << "/>" << endl;
    }
    fout << "\t\t</PPointData>" << endl;
    string root_basename = fname_root.substr(fname_root.find_last_of("/\\") + 1);
    stringstream piece;
    piece << root_basename << "_0_" << setw(6) << setfill('0') << tstep << ".vti";
    fout << "\t\t<Piece Extent=\"0 " << I - 1 << " 0 " << J - 1 << " 0 " << K - 1 << "\" ";
    fout << "Source=\"" << piece.str() << "\"/>" << endl;
    fout << "\t</PImageData>" << endl;
    fout << "</VTKFile>" << endl;
    cout << "Wrote master VTK file: " << fname.str() << endl;
}

// gather a field into VTK point order (i fastest)
template <typename T>
static std::vector<T> to_vtk(const T* a, int I, int J, int K, int ncomp = 1, const T* b = nullptr,
                             const T* c = nullptr) {
    std::vector<T> out((size_t)I * J * K * ncomp);
    size_t cnt = 0;
    for (int k = 0; k < K; ++k)
        for (int j = 0; j < J; ++j)
            for (int i = 0; i < I; ++i) {
                size_t r = (size_t)k + (size_t)K * ((size_t)j + (size_t)J * i);
                out[cnt * ncomp] = a[r];
                if (ncomp == 3) {
                    out[cnt * 3 + 1] = b[r];
                    out[cnt * 3 + 2] = c[r];
                }
                cnt++;
            }
    return out;
}

void write_vti(const std::string& path, int I, int J, int K, size_t flags, const VtkFields& f) {
    std::vector<std::pair<ArraySpec, std::vector<char>>> blobs;
    auto add = [&](const ArraySpec& s, const void* p, size_t bytes) {
        std::vector<char> v(bytes);
        if (bytes) std::memcpy(v.data(), p, bytes);
        blobs.push_back({s, std::move(v)});
    };
    for (const auto& s : specs(flags, f.label_bytes)) {
        switch (s.flag) {
        case Type:
            if (f.label_bytes == 2) {
                auto o = to_vtk((const uint16_t*)f.label, I, J, K);
                add(s, o.data(), o.size() * 2);
            } else {
                auto o = to_vtk((const uint8_t*)f.label, I, J, K);
                add(s, o.data(), o.size());
            }
            break;
        case Conc: { auto o = to_vtk(f.conc, I, J, K); add(s, o.data(), o.size() * 8); } break;
        case Pressure: { auto o = to_vtk(f.pressure, I, J, K); add(s, o.data(), o.size() * 8); } break;
        case Frac: { auto o = to_vtk(f.frac, I, J, K); add(s, o.data(), o.size() * 4); } break;
        case Flux_Vec: { auto o = to_vtk(f.fx, I, J, K, 3, f.fy, f.fz); add(s, o.data(), o.size() * 8); } break;
        case Saturation: { auto o = to_vtk(f.sat, I, J, K); add(s, o.data(), o.size() * 8); } break;
        case CapPressure: { auto o = to_vtk(f.pc, I, J, K); add(s, o.data(), o.size() * 8); } break;
        case RelPermeability: { auto o = to_vtk(f.kr, I, J, K); add(s, o.data(), o.size() * 8); } break;
        case Permeability: { auto o = to_vtk(f.perm, I, J, K); add(s, o.data(), o.size() * 8); } break;
        case AcidConc: { auto o = to_vtk(f.acid, I, J, K); add(s, o.data(), o.size() * 8); } break;
        default: break;
        }
    }
    ofstream fout(path, ios::binary);
    if (!fout.is_open()) throw std::runtime_error("cannot write " + path);
    fout << "<?xml version=\"1.0\"?>\n";
    fout << "<VTKFile type=\"ImageData\" version=\"1.0\" byte_order=\"LittleEndian\" "
            "header_type=\"UInt64\">\n";
    fout << "  <ImageData WholeExtent=\"0 " << I - 1 << " 0 " << J - 1 << " 0 " << K - 1
         << "\" Origin=\"0 0 0\" Spacing=\"1 1 1\">\n";
    fout << "    <Piece Extent=\"0 " << I - 1 << " 0 " << J - 1 << " 0 " << K - 1 << "\">\n";
    fout << "      <PointData" << ((flags & Flux_Vec) ? " Vectors=\"Flux\"" : "") << ">\n";
    uint64_t offset = 0;
    for (const auto& b : blobs) {
        fout << "        <DataArray type=\"" << b.first.type << "\" Name=\"" << b.first.name << "\"";
        if (b.first.ncomp > 1) fout << " NumberOfComponents=\"" << b.first.ncomp << "\"";
        fout << " format=\"appended\" offset=\"" << offset << "\"/>\n";
        offset += 8 + b.second.size();
    }
    fout << "      </PointData>\n      <CellData>\n      </CellData>\n    </Piece>\n  </ImageData>\n";
    fout << "  <AppendedData encoding=\"raw\">\n   _";
    for (const auto& b : blobs) {
        uint64_t nbytes = b.second.size();
        fout.write(reinterpret_cast<const char*>(&nbytes), 8);
        fout.write(b.second.data(), (std::streamsize)b.second.size());
    }
    fout << "\n  </AppendedData>\n</VTKFile>\n";
}

// time_mapping.pvd, src/main.cpp:512-525
void write_pvd(const std::string& path, const std::vector<double>& times,
               const std::vector<size_t>& steps) {
    std::ofstream pvd(path);
    pvd << "<?xml version=\"1.0\"?>\n";
    pvd << "<VTKFile type=\"Collection\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
    pvd << "  <Collection>\n";
    for (size_t i = 0; i < times.size(); ++i)
        pvd << "    <DataSet timestep=\"" << times[i] << "\" file=\"output_" << std::setw(6)
            << std::setfill('0') << steps[i] << ".pvti\"/>\n";
    pvd << "  </Collection>\n";
    pvd << "</VTKFile>\n";
}

}  // namespace lsh
