// Installs the model the gmsh stand-in answers for — TEST INFRASTRUCTURE ONLY.
#pragma once
#include "../../fem-g_gb300/host/mesh.h"

// The current (and only) model of the stand-in: a mesh of this project's
// synthetic meshes, with its entities and physical names.
void oracleShimSetMesh(femg::Mesh &&m);
const femg::Mesh &oracleShimMesh();
