/*
 * vtk_stub.h - stand-in for the few VTK classes Simulation::writeVTKFile uses
 * (src/Simulation.cpp:1306-1566), so that the reference's sources compile into the parity
 * library under oracle/_ref. TEST INFRASTRUCTURE ONLY: arrays keep their values in memory and
 * the writer writes nothing (the parity tests do not call writeVTKFile; the product has its
 * own .vti writer). Included by each vtk*.h shim header.
 */
#ifndef LSREF_SHIM_VTK_STUB_H_
#define LSREF_SHIM_VTK_STUB_H_

#include <map>
#include <memory>
#include <string>
#include <vector>

class vtkDataArray {
public:
    virtual ~vtkDataArray() {}
    void SetName(const char* n) { name = n; }
    void SetNumberOfComponents(int c) { comps = c; }
    void SetNumberOfValues(long long n) { values.assign((size_t)n, 0.0); }
    void SetNumberOfTuples(long long n) { values.assign((size_t)n * (size_t)comps, 0.0); }
    void SetTuple1(long long t, double v) { values[(size_t)t] = v; }
    void SetTuple3(long long t, double a, double b, double c) {
        values[(size_t)t * 3] = a;
        values[(size_t)t * 3 + 1] = b;
        values[(size_t)t * 3 + 2] = c;
    }
    std::string name;
    int comps = 1;
    std::vector<double> values;
};
class vtkDoubleArray : public vtkDataArray {};
class vtkFloatArray : public vtkDataArray {};
class vtkUnsignedShortArray : public vtkDataArray {};
class vtkUnsignedCharArray : public vtkDataArray {};

template <typename T>
class vtkSmartPointer {
public:
    vtkSmartPointer() {}
    static vtkSmartPointer New() {
        vtkSmartPointer p;
        p.ptr = std::make_shared<T>();
        return p;
    }
    T* operator->() const { return ptr.get(); }
    T* Get() const { return ptr.get(); }
    template <typename U>
    operator vtkSmartPointer<U>() const {
        vtkSmartPointer<U> q;
        q.ptr = std::static_pointer_cast<U>(ptr);
        return q;
    }
    std::shared_ptr<T> ptr;
};

class vtkPointData {
public:
    void AddArray(const vtkSmartPointer<vtkDataArray>& a) { arrays[a->name] = a; }
    void SetVectors(const vtkSmartPointer<vtkDataArray>& a) { arrays[a->name] = a; }
    vtkDataArray* GetArray(const char* n) { return arrays[n].Get(); }
    vtkDataArray* GetVectors(const char* n) { return arrays[n].Get(); }
    std::map<std::string, vtkSmartPointer<vtkDataArray>> arrays;
};

class vtkImageData {
public:
    void SetExtent(int, int, int, int, int, int) {}
    vtkPointData* GetPointData() { return &pd; }
    vtkPointData pd;
};

class vtkXMLImageDataWriter {
public:
    void SetFileName(const char*) {}
    void SetInputData(const vtkSmartPointer<vtkImageData>&) {}
    int Write() { return 1; }
};

#endif /* LSREF_SHIM_VTK_STUB_H_ */
