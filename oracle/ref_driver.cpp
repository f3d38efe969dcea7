// Driver around the reference's own numbering code — TEST INFRASTRUCTURE ONLY.
//
// Compiled (by oracle/build.py, recipe ref) together with the reference's
// fem-master/src/reorder/Hilbert.cpp and its vendored
// fem-master/contrib/robin-hood-hashing/robin_hood.h, read where they lie;
// the result goes to oracle/_ref/libref.so and is used only to pin the
// oracle's restatements (robin-hood iteration order, Hilbert order).
#include <complex>
#include <cstdint>
#include <vector>

#include "Hilbert.h"
#include "robin_hood.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace gmshfem::omp {
unsigned int getNumThreads() {
#ifdef _OPENMP
  return omp_get_num_threads();
#else
  return 1;
#endif
}
unsigned int getThreadNum() {
#ifdef _OPENMP
  return omp_get_thread_num();
#else
  return 0;
#endif
}
}  // namespace gmshfem::omp

namespace {
// a DOF key with the reference's Dof::hash (src/dofs/Dof.h:87-92)
struct Key {
  uint64_t numType, entity;
  uint32_t id;
};
struct KeyHash {
  size_t operator()(const Key *k) const noexcept {
    size_t seed = std::hash<unsigned long long>{}(k->entity) + 0x9e3779b9;
    seed ^= std::hash<unsigned long long>{}(k->numType) + 0x9e3779b9 + (seed << 6) + (seed >> 2);
    return seed;
  }
};
struct KeyEq {
  bool operator()(const Key *a, const Key *b) const noexcept { return a->entity == b->entity && a->numType == b->numType; }
};
}  // namespace

extern "C" {

// Replay reserve/insert events on robin_hood::unordered_map<Dof*, complex<double>>
// (the type of FieldInterface::_values for complex<double> formulations) and
// return the ids in iteration order.
int64_t ref_robin_order(int64_t n_ops, const int32_t *op_kind, const uint64_t *op_arg, const uint64_t *num_type,
                        const uint64_t *entity, uint32_t *order_out) {
  uint64_t maxId = 0;
  for (int64_t k = 0; k < n_ops; ++k)
    if (op_kind[k] == 1 && op_arg[k] + 1 > maxId) maxId = op_arg[k] + 1;
  std::vector<Key> keys(maxId);
  for (uint64_t i = 0; i < maxId; ++i) keys[i] = {num_type[i], entity[i], (uint32_t)i};
  robin_hood::unordered_map<Key *, std::complex<double>, KeyHash, KeyEq> map;
  for (int64_t k = 0; k < n_ops; ++k) {
    if (op_kind[k] == 0) map.reserve(op_arg[k]);
    else map.insert(robin_hood::pair<Key *, std::complex<double>>(&keys[op_arg[k]], 0.0));
  }
  int64_t c = 0;
  for (auto it = map.begin(); it != map.end(); ++it) order_out[c++] = it->first->id;
  return c;
}

// Hilbert<dim,N>::apply on n float points; perm_out[r] = input index of rank r
int ref_hilbert_order(int dim, int64_t n, const float *pts, const float *mn, const float *mx, uint32_t *perm_out) {
  if (dim == 2) {
    std::vector<gmshfem::reorder::SortedEntity<2>> v(n);
    for (int64_t i = 0; i < n; ++i) {
      v[i].f[0] = pts[2 * i];
      v[i].f[1] = pts[2 * i + 1];
      v[i].ptrA = reinterpret_cast<void *>(static_cast<uintptr_t>(i));
    }
    // the union keeps ptrA/ptrB at the same address; f is read before h is written
    for (int64_t i = 0; i < n; ++i) v[i].ptrB = v[i].ptrA;
    gmshfem::reorder::Hilbert<2, 4> h;
    h.apply(v, mn, mx);
    for (int64_t i = 0; i < n; ++i) perm_out[i] = (uint32_t) reinterpret_cast<uintptr_t>(v[i].ptrB);
  } else {
    std::vector<gmshfem::reorder::SortedEntity<3>> v(n);
    for (int64_t i = 0; i < n; ++i) {
      v[i].f[0] = pts[3 * i];
      v[i].f[1] = pts[3 * i + 1];
      v[i].f[2] = pts[3 * i + 2];
      v[i].ptrA = reinterpret_cast<void *>(static_cast<uintptr_t>(i));
    }
    gmshfem::reorder::Hilbert<3, 8> h;
    h.apply(v, mn, mx);
    for (int64_t i = 0; i < n; ++i) perm_out[i] = (uint32_t) reinterpret_cast<uintptr_t>(v[i].ptrB);
  }
  return 0;
}

}  // extern "C"
