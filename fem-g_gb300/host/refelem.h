// Reference-element data: quadrature rules, geometric (Lagrange) basis, the
// hierarchical H1 basis with orientations and the hierarchical HCurl basis of orders 0 and 1.
//
// In the reference these come from gmsh:
//  - quadrature: gmsh::model::mesh::getIntegrationPoints(type, "GaussN") via
//    FunctionSpaceInterface::GetGaussInfo (src/field/FunctionSpaceInterface.cpp:470-481);
//  - Lagrange basis: getBasisFunctions("Lagrange"/"GradLagrange")
//    (src/field/FunctionSpaceLagrange.cpp:105-137);
//  - hierarchical H1: getBasisFunctions("H1Legendre<p>"/"GradH1Legendre<p>")
//    with per-element orientations (src/field/FunctionSpaceHierarchicalH1.cpp:83-109).
// gmsh is absent, so the rules and bases below are written from the published
// mathematics:
//  - "GaussN" on a simplex is the Grundmann-Moller rule of odd degree
//    2*ceil((N-1)/2)+1 >= N (A. Grundmann, H.M. Moller, SIAM J. Numer. Anal. 15,
//    1978), except "Gauss6" on the tetrahedron: the 24-point degree-6 rule of
//    Keast (1986), the point count of the published tetrahedral tables; on a
//    line it is the Gauss-Legendre rule with ceil((N+1)/2) points;
//  - the hierarchical basis is a Legendre-kernel family: vertex functions
//    lambda_v, edge functions lambda_a lambda_b P_k(lambda_b - lambda_a), face
//    and interior bubbles built the same way; edges and faces are oriented by
//    the global node order so the basis is conforming across elements.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace femg {

struct QuadRule {
  int nq = 0;
  std::vector<double> points;   // [nq][3] reference coordinates (u, v, w)
  std::vector<double> weights;  // [nq]
};

// integrationType "GaussN" on an element type (gmsh codes)
QuadRule gaussRule(const std::string &integrationType, int elementType);

// Geometric Lagrange basis of an element type at a point: values [nn], reference
// gradients [nn][3]
void lagrangeBasis(int elementType, const double *uvw, double *val, double *grad);

// Hierarchical H1 of order p on a simplex of dimension dim (2 or 3).
int hierarchicalCount(int dim, int p);
// Orientation code of an element from the global tags of its vertices: edge
// reversal bits followed by base-6 face permutation digits (3D only).
int hierarchicalOrientation(int dim, const int64_t *vertexTags);
// Basis values [n] and reference gradients [n][3] for an orientation code.
void hierarchicalBasis(int dim, int p, int orientationCode, const double *uvw, double *val, double *grad);

// Lowest-order HCurl (Whitney / Nedelec first kind edge functions) on a
// simplex: one function per edge (a, b) of simplexEdges, directed from the
// lower global vertex tag to the higher one,
//   w_ab = lambda_a grad(lambda_b) - lambda_b grad(lambda_a),  curl w_ab = 2 grad(lambda_a) x grad(lambda_b),
// in reference coordinates (the Form1 / Form2 maps apply J^-T and J / det).
// The orientation code is the edge reversal bits of hierarchicalOrientation.
int whitneyCount(int dim);
int whitneyOrientation(int dim, const int64_t *vertexTags);
// values [n][3] and curls [n][3] for an orientation code
void whitneyBasis(int dim, int orientationCode, const double *uvw, double *val, double *curl);

// Hierarchical HCurl of order p = 0 or 1 (the reference's
// FunctionSpaceHierarchicalHCurl, gmsh "HcurlLegendre<p>"): order 0 is
// whitneyBasis; order 1 spans the first-kind Nedelec space of degree 2 with,
// per edge (a, b) directed from the lower global tag to the higher,
//   w_ab and grad(lambda_a lambda_b)  (curl 0),
// and per face with vertices s0 < s1 < s2 in global tag order (3D; the
// triangle's own vertex order in 2D, where they are interior bubbles)
//   lambda_s2 w_s0s1 and lambda_s0 w_s1s2,
//   curl(lambda_c w_ab) = grad(lambda_c) x w_ab + 2 lambda_c grad(lambda_a) x grad(lambda_b).
// The face functions vanish tangentially on every edge, so the basis is
// conforming (tangential continuity) across elements. Orientation codes:
// whitneyOrientation for p = 0, hierarchicalOrientation for p = 1.
int hcurlCount(int dim, int p);
int hcurlOrientation(int dim, int p, const int64_t *vertexTags);
// values [n][3] and curls [n][3]; functions ordered edge by edge (w, grad),
// then face by face (two each)
void hcurlBasis(int dim, int p, int orientationCode, const double *uvw, double *val, double *curl);

// Legendre polynomial P_k and derivative
void legendre(int k, double x, double &p, double &dp);

}  // namespace femg
