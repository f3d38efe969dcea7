// Reference-element data: quadrature rules, geometric (Lagrange) basis, the
// hierarchical H1 basis with orientations and the hierarchical HCurl basis of any order.
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

// Hierarchical HCurl of order p (the reference's FunctionSpaceHierarchicalHCurl,
// gmsh "HcurlLegendre<p>"): order 0 is whitneyBasis; order p spans the
// first-kind Nedelec space of degree p + 1 (all vector polynomials of degree
// p plus the degree-(p+1) fields q with x . q = 0), of dimension (p+1)(p+3)
// on a triangle and (p+1)(p+3)(p+4)/2 on a tetrahedron, with
//  - per edge (a, b) directed from the lower global tag to the higher
//    (p + 1 functions): w_ab, then grad(lambda_a lambda_b P_k(lambda_b - lambda_a))
//    for k = 0 .. p-1 (curl 0; the gradients of the H1 edge functions of
//    degree up to p + 1);
//  - per face with vertices s0 < s1 < s2 in global tag order (3D; the
//    triangle's own vertex order in 2D, where they are interior bubbles),
//    for the face polynomials q = P_i(l_s1 - l_s0) P_j(l_s2 - l_s1), i + j = d,
//    d = 0 .. p-1 (i from d down to 0), the pair
//      lambda_s2 w_s0s1 q and lambda_s0 w_s1s2 q      (p(p+1) functions);
//  - per tetrahedron (p >= 2), for q = P_i(l1 - l0) P_j(l2 - l1) P_k(l3 - l2),
//    i + j + k = d, d = 0 .. p-2, the triple
//      lambda_2 lambda_3 w_01 q, lambda_0 lambda_3 w_12 q, lambda_0 lambda_1 w_23 q
//    ((p-1)p(p+1)/2 functions),
// with curl(s w_ab) = grad(s) x w_ab + 2 s grad(lambda_a) x grad(lambda_b).
// A face function vanishes tangentially on the face's edges and on the other
// faces, an interior function on every face, and a face's functions depend
// on its global vertex order only, so the basis is conforming (tangential
// continuity) across elements; each order's functions come first within
// their edge, face or element, so order p - 1 is a part of order p.
// Orientation codes: whitneyOrientation for p = 0, hierarchicalOrientation
// for p >= 1.
int hcurlCount(int dim, int p);
int hcurlOrientation(int dim, int p, const int64_t *vertexTags);
// Functions per edge, per face and per element interior (3D) of order p
void hcurlEntityCounts(int dim, int p, int &perEdge, int &perFace, int &perCell);
// values [n][3] and curls [n][3]; functions ordered edge by edge, then face
// by face, then the interior ones
void hcurlBasis(int dim, int p, int orientationCode, const double *uvw, double *val, double *curl);

// Legendre polynomial P_k and derivative
void legendre(int k, double x, double &p, double &dp);

}  // namespace femg
