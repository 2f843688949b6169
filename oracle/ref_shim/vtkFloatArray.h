/* vtkFloatArray.h - see vtk_stub.h (test infrastructure for the parity library under oracle/_ref). */
#include "vtk_stub.h"
