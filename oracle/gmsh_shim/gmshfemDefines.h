// Hand-written configuration header of the reference build used by the oracle
// — TEST INFRASTRUCTURE ONLY. The reference generates this file with cmake
// from src/common/gmshfemDefines.h.in; here it states the configuration
// directly: gmsh (the project's stand-in), OpenMP and the vendored robin-hood
// map on; Bessel, Boost, PETSc, SLEPc and profiling off; the reference's
// default constants.
#ifndef H_GMSHFEM_GMSHFEMDEFINES
#define H_GMSHFEM_GMSHFEMDEFINES

#define HAVE_GMSH
#define HAVE_OPENMP
#define HAVE_ROBINHOOD

#define GMSHFEM_MAJOR_VERSION 1
#define GMSHFEM_MINOR_VERSION 0
#define GMSHFEM_PATCH_VERSION 0
#define GMSHFEM_DATE "oracle"
#define GMSHFEM_HOST "oracle"
#define GMSHFEM_PACKAGER "oracle"
#define GMSHFEM_OS "Linux"
#define GMSHFEM_CONFIG_OPTIONS "Gmsh(stand-in) OpenMP RobinHood"
#define GMSHFEM_CXX_FLAGS "-O2 -fopenmp"
#define GMSHFEM_CMAKE_BUILD_TYPE "Release"

#define GMSHFEM_DOF_FIELD_OFFSET 1024
#define GMSHFEM_DOF_MEMORY_POOL_SIZE 16384
#define GMSHFEM_FUNCTION_MEMORY_ALIGNMENT 512
#define GMSHFEM_FUNCTION_MEMORY_OVERSIZE_TOLERENCE 1.5
#define GMSHFEM_FUNCTION_MEMORY_RESIDUAL 1073741824
#define GMSHFEM_FUNCTION_MEMORY_SMALLBUFFER_SIZE 16
#define GMSHFEM_NUMA_ALLOCATOR 0

#endif
