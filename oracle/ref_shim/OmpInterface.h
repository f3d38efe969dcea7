// Stand-in for the reference's src/common/OmpInterface.h when its
// src/reorder/Hilbert.cpp is compiled alone for the oracle: declares only the
// two thread queries Hilbert.cpp calls (definitions in ref_driver.cpp), so the
// cmake-generated gmshfemDefines.h is not needed.
#pragma once
namespace gmshfem::omp {
unsigned int getNumThreads();
unsigned int getThreadNum();
}  // namespace gmshfem::omp
