#include "refelem.h"

#include <algorithm>
#include <cmath>
#include <stdexcept>

#include "mesh.h"

namespace femg {

namespace {

double factorial(int n) {
  double f = 1.0;
  for (int i = 2; i <= n; ++i) f *= i;
  return f;
}

// Grundmann-Moller rule with index s on the n-simplex (n = 2, 3): degree 2s+1,
// weights sum to the simplex volume 1/n!.
QuadRule grundmannMoller(int n, int s) {
  QuadRule r;
  const int d = 2 * s + 1;
  for (int i = 0; i <= s; ++i) {
    const int rr = s - i;
    const double D = d + n - 2 * i;
    const double w = ((i % 2) ? -1.0 : 1.0) * std::ldexp(1.0, -2 * s) * std::pow(D, d) / (factorial(i) * factorial(d + n - i));
    if (n == 2) {
      for (int b1 = 0; b1 <= rr; ++b1)
        for (int b2 = 0; b2 <= rr - b1; ++b2) {
          r.points.push_back((2 * b1 + 1) / D);
          r.points.push_back((2 * b2 + 1) / D);
          r.points.push_back(0.0);
          r.weights.push_back(w);
        }
    } else {
      for (int b1 = 0; b1 <= rr; ++b1)
        for (int b2 = 0; b2 <= rr - b1; ++b2)
          for (int b3 = 0; b3 <= rr - b1 - b2; ++b3) {
            r.points.push_back((2 * b1 + 1) / D);
            r.points.push_back((2 * b2 + 1) / D);
            r.points.push_back((2 * b3 + 1) / D);
            r.weights.push_back(w);
          }
    }
  }
  r.nq = (int)r.weights.size();
  return r;
}

QuadRule gaussLegendreLine(int npts) {
  QuadRule r;
  for (int i = 0; i < npts; ++i) {
    double x = std::cos(M_PI * (i + 0.75) / (npts + 0.5));
    for (int it = 0; it < 100; ++it) {
      double p, dp;
      legendre(npts, x, p, dp);
      double dx = p / dp;
      x -= dx;
      if (std::fabs(dx) < 1e-16) break;
    }
    double p, dp;
    legendre(npts, x, p, dp);
    r.points.push_back(x);
    r.points.push_back(0.0);
    r.points.push_back(0.0);
    r.weights.push_back(2.0 / ((1.0 - x * x) * dp * dp));
  }
  r.nq = npts;
  return r;
}

struct VG {
  double v;
  double g[3];
};

inline VG mul(const VG &a, const VG &b) {
  VG r;
  r.v = a.v * b.v;
  for (int c = 0; c < 3; ++c) r.g[c] = a.v * b.g[c] + b.v * a.g[c];
  return r;
}

inline VG leg(int k, const VG &lo, const VG &hi) {
  double p, dp;
  legendre(k, hi.v - lo.v, p, dp);
  VG r;
  r.v = p;
  for (int c = 0; c < 3; ++c) r.g[c] = dp * (hi.g[c] - lo.g[c]);
  return r;
}

void barycentric(int dim, const double *uvw, VG *lam) {
  for (int i = 0; i <= dim; ++i)
    for (int c = 0; c < 3; ++c) lam[i].g[c] = 0.0;
  if (dim == 1) {
    lam[0].v = 0.5 * (1.0 - uvw[0]);
    lam[1].v = 0.5 * (1.0 + uvw[0]);
    lam[0].g[0] = -0.5;
    lam[1].g[0] = 0.5;
    return;
  }
  double s = 0.0;
  for (int c = 0; c < dim; ++c) {
    lam[c + 1].v = uvw[c];
    lam[c + 1].g[c] = 1.0;
    s += uvw[c];
    lam[0].g[c] = -1.0;
  }
  lam[0].v = 1.0 - s;
}

const int kPerm3[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};

}  // namespace

void legendre(int k, double x, double &p, double &dp) {
  double p0 = 1.0, p1 = x;
  if (k == 0) {
    p = 1.0;
    dp = 0.0;
    return;
  }
  for (int n = 1; n < k; ++n) {
    double p2 = ((2 * n + 1) * x * p1 - n * p0) / (n + 1);
    p0 = p1;
    p1 = p2;
  }
  p = p1;
  // derivative from (x^2-1) P_k' = k (x P_k - P_{k-1}); at |x| = 1 use k(k+1)/2 * x^(k+1)
  if (std::fabs(std::fabs(x) - 1.0) < 1e-14)
    dp = 0.5 * k * (k + 1) * ((x > 0 || (k % 2 == 1)) ? 1.0 : -1.0);
  else
    dp = k * (x * p1 - p0) / (x * x - 1.0);
}

// The 24-point rule of degree 6 on the tetrahedron with three orbits of
// (a, a, a, 1 - 3a) and one of (a, a, b, 1 - 2a - b) in barycentric
// coordinates, all weights positive and all points inside (P. Keast, Comput.
// Methods Appl. Mech. Eng. 55, 1986, rule 6). The parameters below solve its
// moment equations (exact for every monomial of degree <= 6) to 25 digits;
// fem-g_gb300/host/tet_rule6.py recomputes them. Weights are for the
// reference tetrahedron of volume 1/6.
static QuadRule keastTet6() {
  static const double s31[3][2] = {{0.04067395853461135311557945, 0.001679535175886773824668873},
                                   {0.2146028712591520292888392, 0.006653791709694582016615105},
                                   {0.3223378901422755103439945, 0.009226196923942453682525546}};
  const double a = 0.06366100187501752529923553, b = 0.6030056647916491413674311, w211 = 0.008035714285714285714285714;
  QuadRule r;
  auto add = [&](const double lam[4], double w) {  // reference coordinates (lambda_1, lambda_2, lambda_3)
    r.points.insert(r.points.end(), {lam[1], lam[2], lam[3]});
    r.weights.push_back(w);
  };
  for (auto &o : s31)
    for (int k = 0; k < 4; ++k) {
      double lam[4] = {o[0], o[0], o[0], o[0]};
      lam[k] = 1.0 - 3.0 * o[0];
      add(lam, o[1]);
    }
  const double c = 1.0 - 2.0 * a - b;
  for (int i = 0; i < 4; ++i)      // position of b
    for (int j = 0; j < 4; ++j) {  // position of c
      if (j == i) continue;
      double lam[4] = {a, a, a, a};
      lam[i] = b;
      lam[j] = c;
      add(lam, w211);
    }
  r.nq = (int)r.weights.size();
  return r;
}

QuadRule gaussRule(const std::string &integrationType, int elementType) {
  if (integrationType.rfind("Gauss", 0) != 0) throw std::invalid_argument("unsupported integration type " + integrationType);
  const int N = std::stoi(integrationType.substr(5));
  const int dim = elementDim(elementType);
  if (dim == 0) {
    QuadRule r;
    r.nq = 1;
    r.points = {0, 0, 0};
    r.weights = {1.0};
    return r;
  }
  if (dim == 1) return gaussLegendreLine(std::max(1, (N + 2) / 2));
  if (dim == 3 && N == 6) return keastTet6();
  const int s = N <= 1 ? 0 : (N - 1 + 1) / 2;  // smallest s with 2s+1 >= N
  return grundmannMoller(dim, s);
}

void lagrangeBasis(int type, const double *uvw, double *val, double *grad) {
  const int dim = elementDim(type);
  const int order = elementOrder(type);
  const int nn = elementNodes(type);
  for (int i = 0; i < nn * 3; ++i) grad[i] = 0.0;
  if (dim == 0) {
    val[0] = 1.0;
    return;
  }
  VG lam[4];
  barycentric(dim, uvw, lam);
  const int nv = dim + 1;
  if (order == 1) {
    for (int i = 0; i < nv; ++i) {
      val[i] = lam[i].v;
      for (int c = 0; c < 3; ++c) grad[3 * i + c] = lam[i].g[c];
    }
    return;
  }
  for (int i = 0; i < nv; ++i) {
    val[i] = lam[i].v * (2.0 * lam[i].v - 1.0);
    for (int c = 0; c < 3; ++c) grad[3 * i + c] = (4.0 * lam[i].v - 1.0) * lam[i].g[c];
  }
  const auto &edges = simplexEdges(dim);
  for (size_t e = 0; e < edges.size(); ++e) {
    const VG &a = lam[edges[e][0]], &b = lam[edges[e][1]];
    val[nv + e] = 4.0 * a.v * b.v;
    for (int c = 0; c < 3; ++c) grad[3 * (nv + e) + c] = 4.0 * (a.v * b.g[c] + b.v * a.g[c]);
  }
}

int hierarchicalCount(int dim, int p) {
  if (dim == 2) return 3 + 3 * (p - 1) + (p - 1) * (p - 2) / 2;
  if (dim == 3) return 4 + 6 * (p - 1) + 4 * ((p - 1) * (p - 2) / 2) + (p - 1) * (p - 2) * (p - 3) / 6;
  throw std::invalid_argument("hierarchicalCount");
}

int hierarchicalOrientation(int dim, const int64_t *tags) {
  const auto &edges = simplexEdges(dim);
  int code = 0;
  for (size_t e = 0; e < edges.size(); ++e)
    if (tags[edges[e][0]] > tags[edges[e][1]]) code |= 1 << e;
  if (dim == 3) {
    int mult = 1 << edges.size();
    for (auto &f : simplexFaces(3)) {
      int digit = 0;
      for (int q = 0; q < 6; ++q) {
        const int *s = kPerm3[q];
        if (tags[f[s[0]]] < tags[f[s[1]]] && tags[f[s[1]]] < tags[f[s[2]]]) {
          digit = q;
          break;
        }
      }
      code += digit * mult;
      mult *= 6;
    }
  }
  return code;
}

int whitneyCount(int dim) { return (int)simplexEdges(dim).size(); }

int whitneyOrientation(int dim, const int64_t *tags) {
  const auto &edges = simplexEdges(dim);
  int code = 0;
  for (size_t e = 0; e < edges.size(); ++e)
    if (tags[edges[e][0]] > tags[edges[e][1]]) code |= 1 << e;
  return code;
}

void whitneyBasis(int dim, int code, const double *uvw, double *val, double *curl) {
  VG lam[4];
  barycentric(dim, uvw, lam);
  const auto &edges = simplexEdges(dim);
  for (size_t e = 0; e < edges.size(); ++e) {
    int a = edges[e][0], b = edges[e][1];
    if ((code >> e) & 1) std::swap(a, b);  // from the lower global tag to the higher
    const double *ga = lam[a].g, *gb = lam[b].g;
    for (int c = 0; c < 3; ++c) val[3 * e + c] = lam[a].v * gb[c] - lam[b].v * ga[c];
    curl[3 * e + 0] = 2.0 * (ga[1] * gb[2] - ga[2] * gb[1]);
    curl[3 * e + 1] = 2.0 * (ga[2] * gb[0] - ga[0] * gb[2]);
    curl[3 * e + 2] = 2.0 * (ga[0] * gb[1] - ga[1] * gb[0]);
  }
}

void hcurlEntityCounts(int dim, int p, int &perEdge, int &perFace, int &perCell) {
  if (p < 0 || (dim != 2 && dim != 3)) throw std::invalid_argument("hierarchical HCurl: order >= 0 on triangles and tetrahedra");
  perEdge = p + 1;
  perFace = p * (p + 1);
  perCell = dim == 3 ? (p - 1) * p * (p + 1) / 2 : 0;
}

int hcurlCount(int dim, int p) {
  if (p == 0) return whitneyCount(dim);
  int pe, pf, pc;
  hcurlEntityCounts(dim, p, pe, pf, pc);
  return (int)simplexEdges(dim).size() * pe + (dim == 3 ? 4 : 1) * pf + pc;
}

int hcurlOrientation(int dim, int p, const int64_t *tags) {
  return p == 0 ? whitneyOrientation(dim, tags) : hierarchicalOrientation(dim, tags);
}

void hcurlBasis(int dim, int p, int code, const double *uvw, double *val, double *curl) {
  if (p == 0) {
    whitneyBasis(dim, code, uvw, val, curl);
    return;
  }
  VG lam[4];
  barycentric(dim, uvw, lam);
  auto cross = [](const double *x, const double *y, double *z) {
    z[0] = x[1] * y[2] - x[2] * y[1];
    z[1] = x[2] * y[0] - x[0] * y[2];
    z[2] = x[0] * y[1] - x[1] * y[0];
  };
  int idx = 0;
  // w_ab and its curl 2 grad(lambda_a) x grad(lambda_b)
  auto whitney = [&](int a, int b, double *w, double *cw) {
    for (int c = 0; c < 3; ++c) w[c] = lam[a].v * lam[b].g[c] - lam[b].v * lam[a].g[c];
    cross(lam[a].g, lam[b].g, cw);
    for (int c = 0; c < 3; ++c) cw[c] *= 2.0;
  };
  // s w_ab for a scalar s (value and gradient)
  auto scaled = [&](const VG &sc, int a, int b) {
    double w[3], cw[3], gx[3];
    whitney(a, b, w, cw);
    cross(sc.g, w, gx);
    for (int k = 0; k < 3; ++k) {
      val[3 * idx + k] = sc.v * w[k];
      curl[3 * idx + k] = gx[k] + sc.v * cw[k];
    }
    ++idx;
  };
  const auto &edges = simplexEdges(dim);
  for (size_t e = 0; e < edges.size(); ++e) {
    int a = edges[e][0], b = edges[e][1];
    if ((code >> e) & 1) std::swap(a, b);
    whitney(a, b, &val[3 * idx], &curl[3 * idx]);
    ++idx;
    for (int c = 0; c < 3; ++c) {  // grad(lambda_a lambda_b)
      val[3 * idx + c] = lam[a].v * lam[b].g[c] + lam[b].v * lam[a].g[c];
      curl[3 * idx + c] = 0.0;
    }
    ++idx;
    const VG ab = mul(lam[a], lam[b]);
    for (int k = 1; k <= p - 1; ++k) {
      const VG f = mul(ab, leg(k, lam[a], lam[b]));
      for (int c = 0; c < 3; ++c) {
        val[3 * idx + c] = f.g[c];
        curl[3 * idx + c] = 0.0;
      }
      ++idx;
    }
  }
  auto faceFns = [&](int s0, int s1, int s2) {
    for (int d = 0; d <= p - 1; ++d)
      for (int i = d; i >= 0; --i) {
        const int j = d - i;
        if (d == 0) {  // q = 1
          scaled(lam[s2], s0, s1);
          scaled(lam[s0], s1, s2);
          continue;
        }
        const VG q = mul(leg(i, lam[s0], lam[s1]), leg(j, lam[s1], lam[s2]));
        scaled(mul(lam[s2], q), s0, s1);
        scaled(mul(lam[s0], q), s1, s2);
      }
  };
  if (dim == 2) {
    faceFns(0, 1, 2);
    return;
  }
  int digits = code >> edges.size();
  const auto &faces = simplexFaces(3);
  for (size_t f = 0; f < faces.size(); ++f) {
    const int *s = kPerm3[digits % 6];
    digits /= 6;
    faceFns(faces[f][s[0]], faces[f][s[1]], faces[f][s[2]]);
  }
  const VG l23 = mul(lam[2], lam[3]), l03 = mul(lam[0], lam[3]), l01 = mul(lam[0], lam[1]);
  for (int d = 0; d <= p - 2; ++d)
    for (int i = d; i >= 0; --i)
      for (int j = d - i; j >= 0; --j) {
        const int k = d - i - j;
        const VG q = mul(leg(i, lam[0], lam[1]), mul(leg(j, lam[1], lam[2]), leg(k, lam[2], lam[3])));
        scaled(mul(l23, q), 0, 1);
        scaled(mul(l03, q), 1, 2);
        scaled(mul(l01, q), 2, 3);
      }
}

void hierarchicalBasis(int dim, int p, int code, const double *uvw, double *val, double *grad) {
  VG lam[4];
  barycentric(dim, uvw, lam);
  int idx = 0;
  auto put = [&](const VG &f) {
    val[idx] = f.v;
    for (int c = 0; c < 3; ++c) grad[3 * idx + c] = f.g[c];
    ++idx;
  };
  const int nv = dim + 1;
  for (int i = 0; i < nv; ++i) put(lam[i]);
  const auto &edges = simplexEdges(dim);
  for (size_t e = 0; e < edges.size(); ++e) {
    int a = edges[e][0], b = edges[e][1];
    if ((code >> e) & 1) std::swap(a, b);
    const VG ab = mul(lam[a], lam[b]);
    for (int k = 0; k <= p - 2; ++k) put(mul(ab, leg(k, lam[a], lam[b])));
  }
  auto faceFns = [&](int s0, int s1, int s2) {
    const VG abc = mul(mul(lam[s0], lam[s1]), lam[s2]);
    for (int d = 0; d <= p - 3; ++d)
      for (int i = d; i >= 0; --i) {
        const int j = d - i;
        put(mul(abc, mul(leg(i, lam[s0], lam[s1]), leg(j, lam[s1], lam[s2]))));
      }
  };
  if (dim == 2) {
    faceFns(0, 1, 2);
    return;
  }
  int digits = code >> edges.size();
  const auto &faces = simplexFaces(3);
  for (size_t f = 0; f < faces.size(); ++f) {
    const int *s = kPerm3[digits % 6];
    digits /= 6;
    faceFns(faces[f][s[0]], faces[f][s[1]], faces[f][s[2]]);
  }
  const VG abcd = mul(mul(lam[0], lam[1]), mul(lam[2], lam[3]));
  for (int d = 0; d <= p - 4; ++d)
    for (int i = d; i >= 0; --i)
      for (int j = d - i; j >= 0; --j) {
        const int k = d - i - j;
        put(mul(abcd, mul(leg(i, lam[0], lam[1]), mul(leg(j, lam[1], lam[2]), leg(k, lam[2], lam[3])))));
      }
}

}  // namespace femg
