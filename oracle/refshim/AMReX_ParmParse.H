// Test infrastructure only: stand-in for the AMReX header of this name (see AMReX_shim.H).
#include "AMReX_shim.H"
