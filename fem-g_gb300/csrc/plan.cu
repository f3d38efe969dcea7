// Plan creation: validation of the reference-side descriptors, upload of the
// element bucket and construction of the element -> nonzero map used by the
// deterministic CSR reduction.
//
// The map replaces the per-entry std::lower_bound of MatrixFactory::addValues
// (src/system/MatrixFactory.cpp:267) and the index bucket of
// FieldInterface::fillIndices (src/field/FieldInterface.cpp:1012-1076): for
// every element e, local test DOF i and local unknown DOF j it stores the
// position of column J inside the CSR row I, so the device never searches.
// Each row also gets the list of (element, local index) pairs that touch it,
// in element order; summing along that list is the fixed reduction order.
#include <omp.h>

#include <algorithm>
#include <atomic>
#include <complex>
#include <cstring>
#include <mutex>

#include "common.cuh"

namespace femg {

static std::atomic<int64_t> g_launches{0};

void countLaunch(int n) { g_launches += n; }

namespace {
struct ProfRecord {
  std::string name;
  cudaEvent_t a, b;
};
std::mutex g_profMutex;
std::vector<ProfRecord> g_prof;
std::vector<cudaEvent_t> g_eventPool;  // events reused across launches
std::atomic<bool> g_profOn{false};

cudaEvent_t takeEvent() {
  {
    std::lock_guard<std::mutex> lk(g_profMutex);
    if (!g_eventPool.empty()) {
      cudaEvent_t e = g_eventPool.back();
      g_eventPool.pop_back();
      return e;
    }
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return e;
}
}  // namespace

static thread_local bool t_profSuspended = false;
void profSuspend(bool on) { t_profSuspended = on; }
bool profEnabled() { return g_profOn.load(); }

ProfScope::ProfScope(const char *name, cudaStream_t s) : name_(name), s_(s) {
  if (!g_profOn.load() || t_profSuspended) return;
  a_ = takeEvent();
  b_ = takeEvent();
  if (!a_ || !b_) {
    a_ = b_ = nullptr;
    return;
  }
  cudaEventRecord(a_, s_);
}

ProfScope::~ProfScope() {
  if (!a_) return;
  cudaEventRecord(b_, s_);
  std::lock_guard<std::mutex> lk(g_profMutex);
  g_prof.push_back({name_, a_, b_});
}

int ensureDevice(void **ptr, size_t *cap, size_t bytes) {
  if (bytes <= *cap && *ptr) return FG_OK;
  if (*ptr) cudaFree(*ptr);
  *ptr = nullptr;
  *cap = 0;
  if (bytes == 0) return FG_OK;
  cudaError_t e = cudaMalloc(ptr, bytes);
  if (e != cudaSuccess) {
    *ptr = nullptr;
    setLastError(std::string("device allocation of ") + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(e));
    return FG_ERR_OOM;
  }
  *cap = bytes;
  return FG_OK;
}

bool isDevicePointer(const void *p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

template <typename T>
static int upload(fg_plan *plan, const T *host, size_t count, const T **dev) {
  *dev = nullptr;
  if (count == 0) return FG_OK;
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, count * sizeof(T));
  if (e != cudaSuccess) {
    setLastError(std::string("plan upload: ") + cudaGetErrorString(e));
    return FG_ERR_OOM;
  }
  plan->allocs.push_back(p);
  e = cudaMemcpy(p, host, count * sizeof(T), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    setLastError(std::string("plan upload copy: ") + cudaGetErrorString(e));
    return FG_ERR_CUDA;
  }
  *dev = (const T *)p;
  return FG_OK;
}

static bool isRow(int t) { return t == FG_AT_UNKNOWN || t == FG_AT_UNKNOWN_BUBBLE || t == FG_AT_UNKNOWN_GLOBAL; }

// uspace, uidx, utype: the unknown field of a two-field plan (columns), or
// null for a plan of one field
static int createPlan(const fg_mesh_desc *mesh, const fg_rule_desc *rule, const fg_space_desc *space, const fg_system_desc *sys,
                      fg_plan *plan, const fg_space_desc *uspace = nullptr, const uint64_t *uidx = nullptr,
                      const int32_t *utype = nullptr) {
  PlanDev &d = plan->d;
  std::memset(&d, 0, sizeof(d));  // every table absent until uploaded
  if (mesh->dim != 2 && mesh->dim != 3) {
    setLastError("fg_plan_create: element dimension must be 2 or 3");
    return FG_ERR_ARG;
  }
  if (mesh->nodes_per_element < mesh->dim + 1 || mesh->nodes_per_element > kMaxNodes) {
    setLastError("fg_plan_create: unsupported nodes_per_element");
    return FG_ERR_ARG;
  }
  const int n = space->n_basis * space->multiplicity;
  if (space->n_basis <= 0 || space->multiplicity <= 0 || n > kMaxDofs) {
    setLastError("fg_plan_create: element DOFs must be in [1, 64]");
    return FG_ERR_UNSUPPORTED;
  }
  if (mesh->n_elements < 0 || mesh->n_elements >= (int64_t(1) << 26) || mesh->n_nodes >= (int64_t(1) << 31)) {
    setLastError("fg_plan_create: element or node count out of range");
    return FG_ERR_ARG;
  }
  if (rule->nq <= 0 || space->n_orientations <= 0) {
    setLastError("fg_plan_create: empty rule or orientation table");
    return FG_ERR_ARG;
  }
  const int64_t E = mesh->n_elements;
  const int nn = mesh->nodes_per_element;
  d.dim = mesh->dim;
  d.nn = nn;
  d.nq = rule->nq;
  d.nb = space->n_basis;
  d.mult = space->multiplicity;
  d.form = space->form;
  if (d.form != FG_FORM_0 && d.form != FG_FORM_1) {
    setLastError("fg_plan_create: unknown space form");
    return FG_ERR_ARG;
  }
  if (d.form == FG_FORM_1 && d.mult != 1) {
    setLastError("fg_plan_create: HCurl fields have one component");
    return FG_ERR_UNSUPPORTED;
  }
  d.n = n;
  d.nOrient = space->n_orientations;
  const bool coupled = uspace != nullptr;
  int nc = n;
  if (coupled) {
    nc = uspace->n_basis * uspace->multiplicity;
    if (space->form != FG_FORM_0 || uspace->form != FG_FORM_0 || space->multiplicity != 1 || uspace->multiplicity != 1) {
      setLastError("fg_plan_create_coupled: scalar H1 fields (FG_FORM_0, one component) on both sides");
      return FG_ERR_UNSUPPORTED;
    }
    if (uspace->n_basis <= 0 || nc > kMaxDofs || uspace->n_orientations <= 0 || !uspace->basis_val || !uspace->basis_grad) {
      setLastError("fg_plan_create_coupled: unknown space: element DOFs must be in [1, 64], with basis tables");
      return FG_ERR_ARG;
    }
    if (sys->n_linked) {
      setLastError("fg_plan_create_coupled: linked DOFs are not supported in two-field plans");
      return FG_ERR_UNSUPPORTED;
    }
  }
  d.coupled = coupled ? 1 : 0;
  d.nc = nc;
  d.nbU = coupled ? uspace->n_basis : space->n_basis;
  d.nOrientU = coupled ? uspace->n_orientations : space->n_orientations;
  d.affine = (nn == mesh->dim + 1) ? 1 : 0;
  // first-order simplex with the standard basis: dN_0 = -1, dN_k = e_(k-1)
  d.p1geom = d.affine;
  for (int k = 0; k < nn && d.p1geom; ++k)
    for (int c = 0; c < mesh->dim; ++c) {
      const double want = k == 0 ? -1.0 : (c == k - 1 ? 1.0 : 0.0);
      if (rule->geo_grad[(size_t)k * 3 + c] != want) d.p1geom = 0;
    }
  d.E = E;
  d.nNodes = mesh->n_nodes;
  d.nRows = sys->n_rows;
  d.nnz = sys->ai[sys->n_rows];
  d.nFixed = sys->n_fixed;
  plan->E = E;
  plan->hAi.assign(sys->ai, sys->ai + sys->n_rows + 1);

  // element nodes as int32, orientations checked
  std::vector<int32_t> en((size_t)E * nn);
  int bad = 0;
#pragma omp parallel for reduction(+ : bad)
  for (int64_t i = 0; i < E * nn; ++i) {
    const int64_t v = mesh->elem_nodes[i];
    if (v < 0 || v >= mesh->n_nodes) ++bad;
    en[(size_t)i] = (int32_t)v;
  }
  if (bad) {
    setLastError("fg_plan_create: element node index out of range");
    return FG_ERR_INDEX;
  }
  // Geometrically affine elements (straight-sided second-order elements too):
  // the Jacobian at every quadrature point equals the one at the first point.
  if (!d.affine) {
    int curved = 0;
#pragma omp parallel for reduction(+ : curved)
    for (int64_t e = 0; e < E; ++e) {
      double J0[9] = {0}, scale = 0.0;
      for (int q = 0; q < rule->nq && !curved; ++q) {
        double J[9] = {0};
        for (int k = 0; k < nn; ++k) {
          const double *X = mesh->node_xyz + 3 * en[(size_t)(e * nn + k)];
          for (int c = 0; c < mesh->dim; ++c) {
            const double g = rule->geo_grad[((size_t)q * nn + k) * 3 + c];
            for (int r = 0; r < 3; ++r) J[3 * c + r] += X[r] * g;
          }
        }
        if (q == 0) {
          for (int k = 0; k < 9; ++k) {
            J0[k] = J[k];
            scale = std::max(scale, std::fabs(J[k]));
          }
        } else {
          for (int k = 0; k < 9; ++k)
            if (std::fabs(J[k] - J0[k]) > 1e-13 * scale) curved = 1;
        }
      }
    }
    d.affine = curved ? 0 : 1;
  }
  for (const fg_space_desc *sp : {space, uspace}) {
    if (!sp || sp->n_orientations <= 1) continue;
    if (!sp->elem_orientation) {
      setLastError("fg_plan_create: elem_orientation required with several orientations");
      return FG_ERR_ARG;
    }
    for (int64_t e = 0; e < E; ++e)
      if (sp->elem_orientation[e] < 0 || sp->elem_orientation[e] >= sp->n_orientations) {
        setLastError("fg_plan_create: orientation index out of range");
        return FG_ERR_INDEX;
      }
  }

  // element DOF map: row/column index (or fixed index) and type. A linked
  // DOF, bubble or not, takes its master's row and column
  // (MatrixFactory.cpp:241-246, :254-259), so it is stored as an Unknown DOF
  // of that row; its coefficient goes to the scale table the reduction
  // applies. The reference adds a linked bubble exactly as a linked DOF
  // (:306-309, :373-380, :409-442; VectorFactory.cpp:134, :195); the bubble
  // kind only changes the pattern, which the caller passes in.
  std::vector<uint32_t> edof((size_t)E * n);
  std::vector<uint8_t> etype((size_t)E * n);
  int linked = 0;
#pragma omp parallel for reduction(+ : bad, linked)
  for (int64_t i = 0; i < E * n; ++i) {
    const int t = sys->elem_dof_type[i];
    uint64_t v = sys->elem_dof_idx[i];
    etype[(size_t)i] = (uint8_t)t;
    if (t < 0 || t > FG_AT_LINKED_BUBBLE) ++bad;
    else if (t == FG_AT_LINKED || t == FG_AT_LINKED_BUBBLE) {
      if (!sys->linked_row || !sys->linked_value || v >= sys->n_linked || sys->linked_row[v] >= sys->n_rows) {
        ++bad;
      } else {
        v = sys->linked_row[v];
        etype[(size_t)i] = FG_AT_UNKNOWN;
        ++linked;
      }
    } else if (isRow(t) && v >= sys->n_rows) ++bad;
    else if (t == FG_AT_FIXED && v >= sys->n_fixed) ++bad;
    edof[(size_t)i] = (uint32_t)v;
  }
  if (bad) {
    setLastError("fg_plan_create: element DOF index/type out of range");
    return FG_ERR_INDEX;
  }
  // the columns: the unknown field's DOFs (a two-field plan), else the rows'
  std::vector<uint32_t> edofU;
  std::vector<uint8_t> etypeU;
  if (coupled) {
    edofU.resize((size_t)E * nc);
    etypeU.resize((size_t)E * nc);
#pragma omp parallel for reduction(+ : bad)
    for (int64_t i = 0; i < E * nc; ++i) {
      const int t = utype[i];
      const uint64_t v = uidx[i];
      if (t < 0 || t > FG_AT_LINKED_BUBBLE || t == FG_AT_LINKED || t == FG_AT_LINKED_BUBBLE) ++bad;
      else if (isRow(t) && v >= sys->n_rows) ++bad;
      else if (t == FG_AT_FIXED && v >= sys->n_fixed) ++bad;
      edofU[(size_t)i] = (uint32_t)v;
      etypeU[(size_t)i] = (uint8_t)t;
    }
    if (bad) {
      setLastError("fg_plan_create_coupled: unknown DOF index/type out of range (linked DOFs are not supported)");
      return FG_ERR_INDEX;
    }
    plan->fixedColumns = std::find(etypeU.begin(), etypeU.end(), (uint8_t)FG_AT_FIXED) != etypeU.end();
  }
  const std::vector<uint32_t> &cdof = coupled ? edofU : edof;
  const std::vector<uint8_t> &ctype = coupled ? etypeU : etype;

  // row -> (element, local test index) lists, element order
  std::vector<uint64_t> rowPtr(sys->n_rows + 1, 0);
  for (int64_t i = 0; i < E * n; ++i)
    if (isRow(etype[(size_t)i])) rowPtr[edof[(size_t)i] + 1]++;
  for (uint64_t r = 0; r < sys->n_rows; ++r) rowPtr[r + 1] += rowPtr[r];
  std::vector<uint32_t> rowElem(rowPtr[sys->n_rows]);
  {
    std::vector<uint64_t> fill(rowPtr.begin(), rowPtr.end() - 1);
    for (int64_t e = 0; e < E; ++e)
      for (int i = 0; i < n; ++i) {
        const size_t k = (size_t)e * n + i;
        if (isRow(etype[k])) rowElem[fill[edof[k]]++] = (uint32_t)((e << 6) | i);
      }
  }

  // gather visiting orders, rows grouped by contribution count (stable):
  // over all rows (rowOrder, for device outputs), and within kOutChunks
  // consecutive row ranges (rowOrderRanged, for host outputs: the visit
  // indices of a range are its rows' indices, so the CSR slice of a range is
  // complete once its part of the order has run, and can be copied out while
  // the next range reduces)
  std::vector<uint32_t> rowOrder(sys->n_rows), rowOrderRanged;
  const int nChunks = sys->n_rows >= (uint64_t)kOutChunks * 4096 ? kOutChunks : 1;
  {
    plan->outChunkRow.assign((size_t)nChunks + 1, 0);
    for (int c = 0; c <= nChunks; ++c) plan->outChunkRow[(size_t)c] = sys->n_rows * (uint64_t)c / (uint64_t)nChunks;
    uint64_t maxCnt = 0;
    for (uint64_t r = 0; r < sys->n_rows; ++r) maxCnt = std::max(maxCnt, rowPtr[r + 1] - rowPtr[r]);
    std::vector<uint64_t> bucket(maxCnt + 2);
    auto countSort = [&](uint64_t ra, uint64_t rb, std::vector<uint32_t> &order) {
      std::fill(bucket.begin(), bucket.end(), 0);
      bucket[0] = ra;
      for (uint64_t r = ra; r < rb; ++r) bucket[rowPtr[r + 1] - rowPtr[r] + 1]++;
      for (uint64_t k = 0; k <= maxCnt; ++k) bucket[k + 1] += bucket[k];
      for (uint64_t r = ra; r < rb; ++r) order[bucket[rowPtr[r + 1] - rowPtr[r]]++] = (uint32_t)r;
    };
    countSort(0, sys->n_rows, rowOrder);
    if (nChunks > 1) {
      rowOrderRanged.resize(sys->n_rows);
      for (int c = 0; c < nChunks; ++c) countSort(plan->outChunkRow[(size_t)c], plan->outChunkRow[(size_t)c + 1], rowOrderRanged);
    }
  }
  if (sys->n_rows >= (uint64_t(1) << 32) || d.nnz >= (uint64_t(1) << 32) || rowElem.size() >= (uint64_t(1) << 32)) {
    setLastError("fg_plan_create: more than 2^32 rows, nonzeros or element rows in one plan");
    return FG_ERR_UNSUPPORTED;
  }
  // visit table: one 16-byte record per row in visiting order (row, CSR
  // start, start of its element list, length | count << 16), the element
  // lists stored contiguously in that order
  std::vector<uint4> visit(sys->n_rows), visitRanged;
  std::vector<uint32_t> visitElem(rowElem.size()), visitElemRanged;
  auto buildVisit = [&](const std::vector<uint32_t> &order, std::vector<uint4> &vis, std::vector<uint32_t> &visElem) -> int {
    uint64_t pos = 0;
    for (uint64_t v = 0; v < sys->n_rows; ++v) {
      const uint32_t r = order[v];
      const uint64_t cnt = rowPtr[r + 1] - rowPtr[r];
      const uint64_t len = sys->ai[r + 1] - sys->ai[r];
      if (cnt > 0xFFFF || len > 0xFFFF) {
        setLastError("fg_plan_create: row with more than 65535 entries or contributions");
        return FG_ERR_UNSUPPORTED;
      }
      std::copy(rowElem.begin() + (int64_t)rowPtr[r], rowElem.begin() + (int64_t)rowPtr[r + 1], visElem.begin() + (int64_t)pos);
      vis[v] = make_uint4(r, (uint32_t)sys->ai[r], (uint32_t)pos, (uint32_t)(len | (cnt << 16)));
      pos += cnt;
    }
    return FG_OK;
  };
  if (int st0 = buildVisit(rowOrder, visit, visitElem)) return st0;
  if (nChunks > 1) {
    visitRanged.resize(sys->n_rows);
    visitElemRanged.resize(rowElem.size());
    if (int st0 = buildVisit(rowOrderRanged, visitRanged, visitElemRanged)) return st0;
  }

  // slots: position of each column inside its row
  uint64_t maxLen = 0;
  for (uint64_t r = 0; r < sys->n_rows; ++r) maxLen = std::max(maxLen, sys->ai[r + 1] - sys->ai[r]);
  if (maxLen >= 0xFFFE) {
    setLastError("fg_plan_create: CSR row longer than 65533 entries");
    return FG_ERR_UNSUPPORTED;
  }
  d.maxRowLen = (int32_t)maxLen;
  const bool narrow = maxLen < 0xFE;
  d.slotBytes = narrow ? 1 : 2;
  // one-byte slot rows of 17 to 32 entries take a whole 32-byte sector each:
  // an element row's slots then come in one sector instead of straddling two
  // (the padding reads as "ignore")
  const int nS = (narrow && nc > 16 && nc <= 32) ? 32 : nc;
  d.slotLd = nS;
  const size_t nSlots = (size_t)E * n * nS;
  std::vector<uint8_t> slot8;
  std::vector<uint16_t> slot16;
  if (narrow) slot8.assign(nSlots, 0xFF); else slot16.assign(nSlots, kSlotIgnore);
  int dup = 0;  // elements with two row columns on one DOF, or slots taken from the upper-storage lower_bound
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : bad, dup)
  for (int64_t e = 0; e < E; ++e) {
    {
      uint32_t cols[64];
      int m = 0;
      for (int j = 0; j < nc; ++j)
        if (isRow(ctype[(size_t)e * nc + j])) cols[m++] = cdof[(size_t)e * nc + j];
      std::sort(cols, cols + m);
      if (std::adjacent_find(cols, cols + m) != cols + m) ++dup;
    }
    for (int i = 0; i < n; ++i) {
      const size_t ki = (size_t)e * n + i;
      if (!isRow(etype[ki])) continue;
      const uint64_t I = edof[ki];
      const uint64_t *b = sys->aj + sys->ai[I];
      const uint64_t *en2 = sys->aj + sys->ai[I + 1];
      for (int j = 0; j < nc; ++j) {
        const size_t kj = (size_t)e * nc + j;
        const int t = ctype[kj];
        uint16_t s;
        if (t == FG_AT_FIXED) s = kSlotFixed;
        else if (!isRow(t)) s = kSlotIgnore;
        else if (sys->upper && cdof[kj] < I) s = kSlotIgnore;  // below the diagonal: not stored
        else {
          const uint64_t J = cdof[kj];
          const uint64_t *p = std::lower_bound(b, en2, J);
          if (p != en2 && (*p == J || sys->upper)) {
            // Upper storage: an aliased bubble row whose first bubble has a
            // larger index lacks the columns between the two; the reference
            // adds those entries at the lower_bound position without checking
            // it (MatrixFactory.cpp:267-268), and so does this map.
            if (*p != J) ++dup;
            s = (uint16_t)(p - b);
          } else {
            ++bad;
            s = kSlotIgnore;
          }
        }
        const size_t ks = ki * nS + j;
        if (narrow) slot8[ks] = s == kSlotFixed ? 0xFF : (s == kSlotIgnore ? 0xFE : (uint8_t)s);
        else slot16[ks] = s;
      }
    }
  }
  if (bad) {
    setLastError("fg_plan_create: an element DOF pair is missing from the CSR pattern");
    return FG_ERR_INDEX;
  }
  d.plainSlots = dup == 0;
  if (nS > nc)
    for (size_t r = 0; r < (size_t)E * n; ++r)
      std::fill(slot8.begin() + (int64_t)(r * nS + nc), slot8.begin() + (int64_t)((r + 1) * nS), (uint8_t)0xFE);

  int st;
  if ((st = upload(plan, mesh->node_xyz, (size_t)mesh->n_nodes * 3, &d.xyz))) return st;
  if ((st = upload(plan, en.data(), en.size(), &d.enodes))) return st;
  if ((st = upload(plan, rule->weights, (size_t)rule->nq, &d.w))) return st;
  if ((st = upload(plan, rule->geo_val, (size_t)rule->nq * nn, &d.geoVal))) return st;
  if ((st = upload(plan, rule->geo_grad, (size_t)rule->nq * nn * 3, &d.geoGrad))) return st;
  if ((st = upload(plan, space->basis_val, (size_t)space->n_orientations * rule->nq * space->n_basis * (d.form == FG_FORM_1 ? 3 : 1),
                    &d.bval)))
    return st;
  if ((st = upload(plan, space->basis_grad, (size_t)space->n_orientations * rule->nq * space->n_basis * 3, &d.bgrad))) return st;
  d.orient = nullptr;
  if (space->n_orientations > 1)
    if ((st = upload(plan, space->elem_orientation, (size_t)E, &d.orient))) return st;
  if ((st = upload(plan, edof.data(), edof.size(), &d.edof))) return st;
  if ((st = upload(plan, etype.data(), etype.size(), &d.etype))) return st;
  if (coupled) {
    if ((st = upload(plan, edofU.data(), edofU.size(), &d.edofU))) return st;
    if ((st = upload(plan, etypeU.data(), etypeU.size(), &d.etypeU))) return st;
    if ((st = upload(plan, uspace->basis_val, (size_t)uspace->n_orientations * rule->nq * uspace->n_basis, &d.bvalU))) return st;
    if ((st = upload(plan, uspace->basis_grad, (size_t)uspace->n_orientations * rule->nq * uspace->n_basis * 3, &d.bgradU)))
      return st;
    d.orientU = nullptr;
    if (uspace->n_orientations > 1)
      if ((st = upload(plan, uspace->elem_orientation, (size_t)E, &d.orientU))) return st;
  } else {
    d.edofU = d.edof;
    d.etypeU = d.etype;
    d.bvalU = d.bval;
    d.bgradU = d.bgrad;
    d.orientU = d.orient;
  }
  if ((st = upload(plan, sys->ai, (size_t)sys->n_rows + 1, &d.ai))) return st;
  if ((st = upload(plan, rowPtr.data(), rowPtr.size(), &d.rowPtr))) return st;
  if ((st = upload(plan, rowElem.data(), rowElem.size(), &d.rowElem))) return st;
  if ((st = upload(plan, visit.data(), visit.size(), &d.visit))) return st;
  if ((st = upload(plan, visitElem.data(), visitElem.size(), &d.visitElem))) return st;
  plan->visitRanged = d.visit;
  plan->visitElemRanged = d.visitElem;
  if (nChunks > 1) {
    if ((st = upload(plan, visitRanged.data(), visitRanged.size(), &plan->visitRanged))) return st;
    if ((st = upload(plan, visitElemRanged.data(), visitElemRanged.size(), &plan->visitElemRanged))) return st;
  }
  if (narrow) {
    const uint8_t *p;
    if ((st = upload(plan, slot8.data(), slot8.size(), &p))) return st;
    d.slot = p;
  } else {
    const uint16_t *p;
    if ((st = upload(plan, slot16.data(), slot16.size(), &p))) return st;
    d.slot = p;
  }
  if (linked) {
    std::vector<double2> ls((size_t)E * n, make_double2(1.0, 0.0));
    for (int64_t i = 0; i < E * n; ++i)
      if (sys->elem_dof_type[i] == FG_AT_LINKED || sys->elem_dof_type[i] == FG_AT_LINKED_BUBBLE) {
        const uint64_t v = sys->elem_dof_idx[i];
        ls[(size_t)i] = make_double2(sys->linked_value[2 * v], sys->linked_value[2 * v + 1]);
      }
    if ((st = upload(plan, ls.data(), ls.size(), &d.lscale))) return st;
  }
  // error word of the Jacobian modificators, and its pinned host copy
  const int zero = 0;
  const int *err = nullptr;
  if ((st = upload(plan, &zero, 1, &err))) return st;
  d.jmErr = const_cast<int *>(err);
  FG_CUDA(cudaMallocHost(&plan->jmErrHost, sizeof(int)));
  return FG_OK;
}

int coupledLiftCheck(const fg_plan *plan, const double *rhs) {
  if (!plan->d.coupled || !plan->fixedColumns || !rhs || plan->d.n == plan->d.nc) return FG_OK;
  setLastError("two-field plan: fixed unknown DOFs lift through VectorFactory::addValuesDC, which reads values[j * n_unknown + i]; "
               "with " + std::to_string(plan->d.n) + " test and " + std::to_string(plan->d.nc) +
               " unknown DOFs per element that entry lies outside the element matrix (pass rhs = NULL for the values alone)");
  return FG_ERR_UNSUPPORTED;
}

int uploadDirichlet(fg_plan *plan, const double *dirichlet, const double **out, cudaStream_t s) {
  *out = nullptr;
  if (plan->d.nFixed == 0) return FG_OK;
  if (!dirichlet) {
    setLastError("Dirichlet values required: the system has fixed DOFs");
    return FG_ERR_ARG;
  }
  if (isDevicePointer(dirichlet)) {
    *out = dirichlet;
    return FG_OK;
  }
  int st = ensureDevice((void **)&plan->dirichlet, &plan->dirichletBytes, plan->d.nFixed * 16);
  if (st) return st;
  FG_CUDA(cudaMemcpyAsync(plan->dirichlet, dirichlet, plan->d.nFixed * 16, cudaMemcpyHostToDevice, s));
  *out = plan->dirichlet;
  return FG_OK;
}

static int classify(const fg_expr &ex) {
  int cls = kExprConst;
  for (int k = 0; k < ex.n_code; ++k) {
    if (ex.code[k].op == FG_OP_X || ex.code[k].op == FG_OP_Y || ex.code[k].op == FG_OP_Z || ex.code[k].op == FG_OP_FIELD ||
        ex.code[k].op == FG_OP_POINT)
      return kExprPoint;
    if (ex.code[k].op == FG_OP_ELEM) cls = kExprElem;
  }
  return cls;
}

static bool isUnaryOp(int op) { return op == FG_OP_NEG || op == FG_OP_HEAVISIDE || (op >= FG_OP_SQRT && op <= FG_OP_CBRT); }
static bool isBinaryOp(int op) { return (op >= FG_OP_ADD && op <= FG_OP_DIV) || op == FG_OP_ATAN2; }

// A constant expression, evaluated once on the host with std::complex (the
// reference's own arithmetic for the same operators).
static std::complex<double> evalConst(const fg_expr &ex) {
  using C = std::complex<double>;
  std::vector<C> st;
  for (int k = 0; k < ex.n_code; ++k) {
    const fg_instr &in = ex.code[k];
    if (in.op == FG_OP_CONST) {
      st.push_back({in.re, in.im});
      continue;
    }
    if (isBinaryOp(in.op)) {
      auto b = st.back();
      st.pop_back();
      auto &a = st.back();
      if (in.op == FG_OP_ADD) a += b;
      else if (in.op == FG_OP_SUB) a -= b;
      else if (in.op == FG_OP_MUL) a *= b;
      else if (in.op == FG_OP_DIV) a /= b;
      else a = std::atan2(a.real(), b.real());
      continue;
    }
    C &a = st.back();
    switch (in.op) {
      case FG_OP_NEG: a = -a; break;
      case FG_OP_HEAVISIDE: a = a.real() > 0 ? 1.0 : (a.real() < 0 ? 0.0 : 0.5); break;
      case FG_OP_SQRT: a = std::sqrt(a); break;
      case FG_OP_EXP: a = std::exp(a); break;
      case FG_OP_LN: a = std::log(a); break;
      case FG_OP_LOG10: a = std::log10(a); break;
      case FG_OP_POW: a = in.arg == 1 ? a : in.arg == 2 ? a * a : in.arg == 3 ? a * a * a : in.arg == 4 ? (a * a) * (a * a)
                                                                                         : std::pow(a, (double)in.arg); break;
      case FG_OP_CBRT: a = std::pow(a, 1.0 / 3.0); break;
      case FG_OP_SIN: a = std::sin(a); break;
      case FG_OP_COS: a = std::cos(a); break;
      case FG_OP_TAN: a = std::tan(a); break;
      case FG_OP_SINH: a = std::sinh(a); break;
      case FG_OP_COSH: a = std::cosh(a); break;
      case FG_OP_TANH: a = std::tanh(a); break;
      case FG_OP_ASIN: a = std::asin(a); break;
      case FG_OP_ACOS: a = std::acos(a); break;
      case FG_OP_ATAN: a = std::atan(a); break;
      case FG_OP_ASINH: a = std::asinh(a); break;
      case FG_OP_ACOSH: a = std::acosh(a); break;
      case FG_OP_ATANH: a = std::atanh(a); break;
      case FG_OP_ABS: a = std::abs(a); break;
      case FG_OP_CONJ: a = std::conj(a); break;
      case FG_OP_REAL: a = a.real(); break;
      case FG_OP_IMAG: a = a.imag(); break;
    }
  }
  return st.empty() ? 0.0 : st.back();
}

// operators that can give a complex value from real operands
static bool mayTurnComplex(int op) {
  return op == FG_OP_SQRT || op == FG_OP_LN || op == FG_OP_LOG10 || op == FG_OP_CBRT || op == FG_OP_ASIN ||
         op == FG_OP_ACOS || op == FG_OP_ACOSH || op == FG_OP_ATANH;
}

static int validateExpr(const fg_expr &ex) {
  if (ex.n_code <= 0 || ex.n_code > FG_EXPR_MAX_CODE || ex.n_arrays < 0 || ex.n_arrays > FG_EXPR_MAX_ARRAYS) return 1;
  int depth = 0;
  for (int k = 0; k < ex.n_code; ++k) {
    const int op = ex.code[k].op;
    if (op <= FG_OP_ELEM || op == FG_OP_FIELD || op == FG_OP_POINT) {
      if ((op == FG_OP_ELEM || op == FG_OP_FIELD || op == FG_OP_POINT) &&
          (ex.code[k].arg < 0 || ex.code[k].arg >= ex.n_arrays || !ex.elem_values[ex.code[k].arg]))
        return 1;
      if (++depth > 16) return 1;
    } else if (isUnaryOp(op)) {
      if (depth < 1) return 1;
      if (op == FG_OP_POW && ex.code[k].arg < 0) return 1;
    } else if (isBinaryOp(op)) {
      if (depth < 2) return 1;
      --depth;
    } else {
      return 1;
    }
  }
  return depth == 1 ? 0 : 1;
}

// arrays: the device copies of per-element coefficient arrays ([E] complex
// each, [E][nb] for the field values of FG_OP_FIELD, [E][nq] for the point
// tables of FG_OP_POINT); the first `used` are
// this upload's, later ones are reused from the previous upload instead of
// freed and allocated again (a buffer too small for its new array is replaced).
static int devExpr(fg_plan *plan, const fg_expr &ex, DevExpr *out, bool *complexOut, std::vector<void *> &arrays, size_t &used) {
  if (validateExpr(ex)) {
    setLastError("invalid coefficient expression");
    return FG_ERR_ARG;
  }
  std::memset(out, 0, sizeof(*out));
  out->n_code = ex.n_code;
  for (int k = 0; k < ex.n_code; ++k) {
    out->code[k] = ex.code[k];
    if (ex.code[k].op == FG_OP_CONST && ex.code[k].im != 0.0) *complexOut = true;
  }
  out->cls = classify(ex);
  // a value known only per element or point: an operator that can leave the
  // reals makes the element matrices complex (a constant is evaluated below)
  if (out->cls != kExprConst)
    for (int k = 0; k < ex.n_code; ++k)
      if (mayTurnComplex(ex.code[k].op)) *complexOut = true;
  if (out->cls == kExprConst) {
    auto v = evalConst(ex);
    out->cval = make_double2(v.real(), v.imag());
    if (v.imag() != 0.0) *complexOut = true;
  }
  for (int a = 0; a < ex.n_arrays; ++a) {
    bool elem = false, field = false, point = false;
    for (int k = 0; k < ex.n_code; ++k) {
      elem = elem || (ex.code[k].op == FG_OP_ELEM && ex.code[k].arg == a);
      field = field || (ex.code[k].op == FG_OP_FIELD && ex.code[k].arg == a);
      point = point || (ex.code[k].op == FG_OP_POINT && ex.code[k].arg == a);
    }
    if ((int)elem + (int)field + (int)point > 1) {
      setLastError("a coefficient array is used in two ways (per element, per point, field values)");
      return FG_ERR_ARG;
    }
    if (field && plan->d.form != FG_FORM_0) {
      setLastError("field values (FG_OP_FIELD) need an H1 bucket");
      return FG_ERR_UNSUPPORTED;
    }
    if (field && plan->d.coupled) {
      setLastError("field values (FG_OP_FIELD) are not supported in two-field plans");
      return FG_ERR_UNSUPPORTED;
    }
    const size_t bytes = (size_t)plan->E * 16 * (field ? (size_t)plan->d.nb : point ? (size_t)plan->d.nq : 1);
    if (isDevicePointer(ex.elem_values[a])) {
      out->arr[a] = (const double2 *)ex.elem_values[a];
      *complexOut = true;  // cannot scan device data cheaply: assume complex
      continue;
    }
    for (size_t k = 0; k < bytes / 16; ++k)
      if (ex.elem_values[a][2 * k + 1] != 0.0) {
        *complexOut = true;
        break;
      }
    void *p = nullptr;
    if (used < arrays.size() && plan->arrayBytes[arrays[used]] >= bytes) {
      p = arrays[used];
    } else {
      if (cudaMalloc(&p, bytes) != cudaSuccess) {
        setLastError("coefficient upload: out of device memory");
        return FG_ERR_OOM;
      }
      plan->arrayBytes[p] = bytes;
      if (used < arrays.size()) {
        cudaFree(arrays[used]);
        arrays[used] = p;
      } else {
        arrays.push_back(p);
      }
    }
    ++used;
    if (cudaMemcpy(p, ex.elem_values[a], bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
      setLastError("coefficient upload failed");
      return FG_ERR_CUDA;
    }
    out->arr[a] = (const double2 *)p;
  }
  return FG_OK;
}

int uploadTerms(fg_plan *plan, const fg_term_desc *terms, int32_t nTerms, double frequency, DevTerms *out,
                std::vector<void *> &arrays) {
  // kernels of an earlier call may still read the arrays about to be
  // overwritten (the device-wide wait that freeing them used to imply)
  if (!arrays.empty() && cudaDeviceSynchronize() != cudaSuccess) {
    setLastError(std::string("coefficient upload: ") + cudaGetErrorString(cudaGetLastError()));
    return FG_ERR_CUDA;
  }
  size_t used = 0;
  struct Trim {  // on every return: free the arrays this upload did not use
    std::vector<void *> &a;
    size_t &u;
    ~Trim() {
      for (size_t k = u; k < a.size(); ++k) cudaFree(a[k]);
      a.resize(std::min(u, a.size()));
    }
  } trim{arrays, used};
  std::memset(out, 0, sizeof(*out));
  if (nTerms <= 0 || nTerms > kMaxTerms || !terms) {
    setLastError("term count must be in [1, 6]");
    return FG_ERR_ARG;
  }
  bool anyDt = false;
  for (int t = 0; t < nTerms; ++t) anyDt = anyDt || terms[t].dt != FG_DT_NONE;
  bool cplx = false;
  out->n = nTerms;
  out->nMod = 0;
  out->tensorTerm = -1;
  out->tensorMassTerm = -1;
  out->tensorFullTerm = -1;
  out->advectTerm = -1;
  out->vecGradTerm = -1;
  out->srcGradTerm = -1;
  for (int t = 0; t < nTerms; ++t) {
    const fg_term_desc &src = terms[t];
    DevTerm &dt = out->t[t];
    dt.kind = src.kind;
    dt.dt = src.dt;
    if (src.kind < FG_TERM_GRAD_GRAD || src.kind > FG_TERM_SOURCE_GRAD) {
      setLastError("unknown term kind");
      return FG_ERR_ARG;
    }
    const bool vectorKind = src.kind == FG_TERM_ADVECTION || src.kind == FG_TERM_VECTOR_GRAD_TEST || src.kind == FG_TERM_SOURCE_GRAD;
    if ((src.kind == FG_TERM_GRAD_GRAD_TENSOR_FULL || vectorKind) && (plan->d.mult != 1 || plan->d.form != FG_FORM_0)) {
      setLastError("the full-tensor, advection and vector terms need a scalar H1 field");
      return FG_ERR_UNSUPPORTED;
    }
    if (plan->d.coupled && src.kind != FG_TERM_GRAD_GRAD && src.kind != FG_TERM_MASS &&
        src.kind != FG_TERM_GRAD_GRAD_TENSOR_FULL && src.kind != FG_TERM_ADVECTION && src.kind != FG_TERM_VECTOR_GRAD_TEST) {
      setLastError(src.kind == FG_TERM_SOURCE || src.kind == FG_TERM_SOURCE_GRAD
                       ? "two-field plan: linear terms go to the test field's own plan"
                       : "two-field plan: grad-grad, mass, full-tensor, advection and vector terms only");
      return FG_ERR_UNSUPPORTED;
    }
    if (src.kind == FG_TERM_ELASTIC && plan->d.mult != 3) {
      setLastError("the elastic (Tensor4) term needs a 3-component compound field");
      return FG_ERR_UNSUPPORTED;
    }
    if (plan->d.form == FG_FORM_1 && (src.kind == FG_TERM_ELASTIC || src.kind == FG_TERM_SOURCE)) {
      setLastError("HCurl fields take the curl-curl and mass terms");
      return FG_ERR_UNSUPPORTED;
    }
    if (src.kind == FG_TERM_GRAD_GRAD_TENSOR && plan->d.mult != 1) {
      setLastError("the tensor grad-grad term needs a scalar H1 or an HCurl field");
      return FG_ERR_UNSUPPORTED;
    }
    if (src.kind == FG_TERM_MASS_TENSOR && plan->d.form != FG_FORM_1) {
      setLastError("the tensor mass term needs an HCurl field");
      return FG_ERR_UNSUPPORTED;
    }
    if (src.kind != FG_TERM_ELASTIC && plan->d.mult != 1 && src.kind != FG_TERM_MASS) {
      setLastError("compound fields support the elastic and mass terms only");
      return FG_ERR_UNSUPPORTED;
    }
    // AFrequency module factor (src/term/Assembler.cpp:283-295)
    if (src.dt == FG_DT_2) dt.factor = make_double2(-frequency * frequency, 0.0);
    else if (src.dt == FG_DT_1) {
      dt.factor = make_double2(0.0, -frequency);
      cplx = true;
    } else dt.factor = make_double2(1.0, 0.0);
    if (src.dt != FG_DT_NONE && (src.kind == FG_TERM_SOURCE || src.kind == FG_TERM_SOURCE_GRAD)) {
      setLastError("a linear term cannot carry a time derivative");
      return FG_ERR_ARG;
    }
    bool sourceComplex = false;  // the right-hand side is always complex
    const bool linear = src.kind == FG_TERM_SOURCE || src.kind == FG_TERM_SOURCE_GRAD;
    int st = devExpr(plan, src.coef, &dt.coef, linear ? &sourceComplex : &cplx, arrays, used);
    if (st) return st;
    if (src.kind == FG_TERM_ELASTIC) {
      st = devExpr(plan, src.coef2, &dt.coef2, &cplx, arrays, used);
      if (st) return st;
      out->hasElastic = 1;
    }
    if (linear) out->hasSource = 1;
    if (src.kind == FG_TERM_GRAD_GRAD_TENSOR || src.kind == FG_TERM_MASS_TENSOR) {
      const bool gg = src.kind == FG_TERM_GRAD_GRAD_TENSOR;
      int32_t &slot = gg ? out->tensorTerm : out->tensorMassTerm;
      if (slot >= 0 || !src.tensor) {
        setLastError(src.tensor ? "at most one tensor term of each kind per assembly" : "tensor term without tensor");
        return FG_ERR_ARG;
      }
      slot = t;
      DevExpr *D = gg ? out->tensor : out->tensorMass;
      for (int k = 0; k < 6; ++k) {
        st = devExpr(plan, src.tensor[k], &D[k], &cplx, arrays, used);
        if (st) return st;
        if (D[k].cls == kExprPoint) out->tensorPoint = 1;
      }
    }
    if (src.kind == FG_TERM_GRAD_GRAD_TENSOR_FULL || src.kind == FG_TERM_ADVECTION) {
      const bool full = src.kind == FG_TERM_GRAD_GRAD_TENSOR_FULL;
      int32_t &slot = full ? out->tensorFullTerm : out->advectTerm;
      if (slot >= 0 || !src.tensor) {
        setLastError(src.tensor ? "at most one full-tensor and one advection term per assembly"
                                : "full-tensor or advection term without its tensor / vector");
        return FG_ERR_ARG;
      }
      slot = t;
      DevExpr *D = full ? out->tensorFull : out->advect;
      for (int k = 0; k < (full ? 9 : 3); ++k) {
        st = devExpr(plan, src.tensor[k], &D[k], &cplx, arrays, used);
        if (st) return st;
      }
      out->nonSym = 1;
    }
    if (src.kind == FG_TERM_VECTOR_GRAD_TEST || src.kind == FG_TERM_SOURCE_GRAD) {
      const bool lin = src.kind == FG_TERM_SOURCE_GRAD;
      int32_t &slot = lin ? out->srcGradTerm : out->vecGradTerm;
      if (slot >= 0 || !src.tensor) {
        setLastError(src.tensor ? "at most one vector term of each kind per assembly" : "vector term without its vector");
        return FG_ERR_ARG;
      }
      slot = t;
      DevExpr *V = lin ? out->srcGrad : out->vecGrad;
      for (int k = 0; k < 3; ++k) {
        st = devExpr(plan, src.tensor[k], &V[k], lin ? &sourceComplex : &cplx, arrays, used);
        if (st) return st;
      }
      out->nonSym = 1;
    }
    // two-field plans: the full element-matrix kernel (FP64 path only)
    if (plan->d.coupled) out->nonSym = 1;
    // the term's Jacobian modificator: terms with equal ones share a group
    const fg_jacmod &jm = src.jacmod;
    if (jm.kind < FG_JACMOD_NONE || jm.kind > FG_JACMOD_SPHERICAL_SHELL) {
      setLastError("unknown Jacobian modificator");
      return FG_ERR_ARG;
    }
    DevJacMod m;
    std::memset(&m, 0, sizeof(m));
    m.kind = jm.kind;
    if (jm.kind >= FG_JACMOD_AXISYMMETRY_SHELL) {
      if (!(jm.r_min > 0.0) || !(jm.r_max > jm.r_min) || jm.exponent < 0 ||
          (jm.kind == FG_JACMOD_CYLINDRICAL_SHELL && (jm.axis < 0 || jm.axis > 2))) {
        setLastError("Jacobian modificator: needs 0 < r_min < r_max, exponent >= 0 and a cylinder axis in 0..2");
        return FG_ERR_ARG;
      }
      m.axis = jm.kind == FG_JACMOD_CYLINDRICAL_SHELL ? jm.axis : 0;
      m.exponent = jm.exponent;
      m.rmin = jm.r_min;
      m.rmax = jm.r_max;
      for (int c = 0; c < 3; ++c) m.center[c] = jm.center[c];
    }
    int g = 0;
    while (g < out->nMod && std::memcmp(&out->mods[g], &m, sizeof(m)) != 0) ++g;
    if (g == out->nMod) out->mods[out->nMod++] = m;
    dt.mod = g;
    if (m.kind != FG_JACMOD_NONE) out->hasJacMod = 1;
  }
  (void)anyDt;
  // linked DOFs scale element entries by complex coefficients: the reduction
  // then runs on complex element matrices
  if (plan->d.lscale) cplx = true;
  out->complexKe = cplx ? 1 : 0;
  return FG_OK;
}

int resolveTerms(fg_plan *plan, const fg_term_desc *terms, int32_t nTerms, double frequency, DevTerms *out,
                 const DevTerms **dev, cudaStream_t s) {
  if (!terms) {
    if (!plan->hasBound) {
      setLastError("no terms given and none bound to the plan");
      return FG_ERR_ARG;
    }
    *out = plan->bound;
    *dev = plan->boundDev;
    return FG_OK;
  }
  int st = uploadTerms(plan, terms, nTerms, frequency, out, plan->termArrays);
  if (st) return st;
  if (!plan->termsDev) FG_CUDA(cudaMalloc(&plan->termsDev, sizeof(DevTerms)));
  FG_CUDA(cudaMemcpyAsync(plan->termsDev, out, sizeof(DevTerms), cudaMemcpyHostToDevice, s));
  *dev = plan->termsDev;
  return FG_OK;
}

int smCount() {
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (!cached[dev]) cudaDeviceGetAttribute(&cached[dev], cudaDevAttrMultiProcessorCount, dev);
  return cached[dev] > 0 ? cached[dev] : 1;
}

}  // namespace femg

using namespace femg;

extern "C" {

int fg_plan_create(const fg_mesh_desc *mesh, const fg_rule_desc *rule, const fg_space_desc *space, const fg_system_desc *sys,
                   fg_plan **out) {
  if (!out) return FG_ERR_ARG;
  *out = nullptr;
  if (!mesh || !rule || !space || !sys || !mesh->node_xyz || !mesh->elem_nodes || !rule->weights || !rule->geo_val ||
      !rule->geo_grad || !space->basis_val || !space->basis_grad || !sys->ai || !sys->elem_dof_idx || !sys->elem_dof_type ||
      (!sys->aj && sys->ai[sys->n_rows] != 0)) {
    setLastError("fg_plan_create: null descriptor field");
    return FG_ERR_ARG;
  }
  int dev = 0;
  if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) {
    cudaGetLastError();
    setLastError("fg_plan_create: no CUDA device");
    return FG_ERR_NO_DEVICE;
  }
  fg_plan *plan = new (std::nothrow) fg_plan;
  if (!plan) return FG_ERR_OOM;
  int st;
  try {
    st = createPlan(mesh, rule, space, sys, plan);
  } catch (const std::bad_alloc &) {
    setLastError("fg_plan_create: host out of memory");
    st = FG_ERR_OOM;
  }
  if (st != FG_OK) {
    fg_plan_destroy(plan);
    return st;
  }
  *out = plan;
  return FG_OK;
}

int fg_plan_create_coupled(const fg_mesh_desc *mesh, const fg_rule_desc *rule, const fg_space_desc *space,
                           const fg_system_desc *sys, const fg_space_desc *unknown_space, const uint64_t *unknown_dof_idx,
                           const int32_t *unknown_dof_type, fg_plan **out) {
  if (!out) return FG_ERR_ARG;
  *out = nullptr;
  if (!mesh || !rule || !space || !sys || !unknown_space || !unknown_dof_idx || !unknown_dof_type || !mesh->node_xyz ||
      !mesh->elem_nodes || !rule->weights || !rule->geo_val || !rule->geo_grad || !space->basis_val || !space->basis_grad ||
      !sys->ai || !sys->elem_dof_idx || !sys->elem_dof_type || (!sys->aj && sys->ai[sys->n_rows] != 0)) {
    setLastError("fg_plan_create_coupled: null descriptor field");
    return FG_ERR_ARG;
  }
  int dev = 0;
  if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) {
    cudaGetLastError();
    setLastError("fg_plan_create_coupled: no CUDA device");
    return FG_ERR_NO_DEVICE;
  }
  fg_plan *plan = new (std::nothrow) fg_plan;
  if (!plan) return FG_ERR_OOM;
  int st;
  try {
    st = createPlan(mesh, rule, space, sys, plan, unknown_space, unknown_dof_idx, unknown_dof_type);
  } catch (const std::bad_alloc &) {
    setLastError("fg_plan_create_coupled: host out of memory");
    st = FG_ERR_OOM;
  }
  if (st != FG_OK) {
    fg_plan_destroy(plan);
    return st;
  }
  *out = plan;
  return FG_OK;
}

void mixedDestroy(fg_plan *plan);
void multiDestroy(fg_plan *plan);
void fp64fDestroy(fg_plan *plan);
void fusedDestroy(fg_plan *plan);

void fg_plan_destroy(fg_plan *plan) {
  if (!plan) return;
  for (void *p : plan->allocs) cudaFree(p);
  for (void *p : plan->termArrays) cudaFree(p);
  for (void *p : plan->boundArrays) cudaFree(p);
  if (plan->boundDev) cudaFree(plan->boundDev);
  if (plan->termsDev) cudaFree(plan->termsDev);
  if (plan->ke) cudaFree(plan->ke);
  if (plan->be) cudaFree(plan->be);
  if (plan->dirichlet) cudaFree(plan->dirichlet);
  if (plan->values) cudaFree(plan->values);
  if (plan->rhs) cudaFree(plan->rhs);
  mixedDestroy(plan);
  multiDestroy(plan);
  fp64fDestroy(plan);
  fusedDestroy(plan);
  if (plan->jmErrHost) cudaFreeHost(plan->jmErrHost);
  for (cudaEvent_t ev : plan->copyEvents)
    if (ev) cudaEventDestroy(ev);
  if (plan->copyStream) cudaStreamDestroy(plan->copyStream);
  delete plan;
}

int fg_plan_info(const fg_plan *plan, int64_t *nnz, int64_t *n_elements, int32_t *n_dofs, int32_t *nq, int32_t *n_orient) {
  if (!plan) return FG_ERR_ARG;
  if (nnz) *nnz = (int64_t)plan->d.nnz;
  if (n_elements) *n_elements = plan->d.E;
  if (n_dofs) *n_dofs = plan->d.n;
  if (nq) *nq = plan->d.nq;
  if (n_orient) *n_orient = plan->d.nOrient;
  return FG_OK;
}

int fg_plan_bind_terms(fg_plan *plan, const fg_term_desc *terms, int32_t n_terms, double frequency) {
  if (!plan) return FG_ERR_ARG;
  plan->hasBound = false;
  int st = uploadTerms(plan, terms, n_terms, frequency, &plan->bound, plan->boundArrays);
  if (st != FG_OK) return st;
  if (!plan->boundDev) FG_CUDA(cudaMalloc(&plan->boundDev, sizeof(DevTerms)));
  FG_CUDA(cudaMemcpy(plan->boundDev, &plan->bound, sizeof(DevTerms), cudaMemcpyHostToDevice));
  plan->hasBound = true;
  return FG_OK;
}

int fg_profile_enable(int on) {
  g_profOn = on != 0;
  return FG_OK;
}

int fg_profile_read(char *names, int32_t name_bytes, int64_t *launches, double *total_ms, int32_t cap) {
  std::vector<ProfRecord> recs;
  {
    std::lock_guard<std::mutex> lk(g_profMutex);
    recs.swap(g_prof);
  }
  std::vector<std::string> order;
  std::vector<int64_t> cnt;
  std::vector<double> ms;
  for (auto &r : recs) {
    float t = 0.0f;
    cudaEventSynchronize(r.b);
    cudaEventElapsedTime(&t, r.a, r.b);
    {
      std::lock_guard<std::mutex> lk(g_profMutex);
      g_eventPool.push_back(r.a);
      g_eventPool.push_back(r.b);
    }
    size_t k = 0;
    while (k < order.size() && order[k] != r.name) ++k;
    if (k == order.size()) {
      order.push_back(r.name);
      cnt.push_back(0);
      ms.push_back(0.0);
    }
    cnt[k]++;
    ms[k] += t;
  }
  cudaGetLastError();
  std::string joined;
  for (size_t k = 0; k < order.size() && (int32_t)k < cap; ++k) {
    if (launches) launches[k] = cnt[k];
    if (total_ms) total_ms[k] = ms[k];
    joined += order[k] + "\n";
  }
  if (names && name_bytes > 0) {
    std::strncpy(names, joined.c_str(), (size_t)name_bytes - 1);
    names[name_bytes - 1] = 0;
  }
  return (int)order.size();
}


int64_t fg_launch_count(void) { return g_launches.load(); }

int fg_host_alloc(void **ptr, size_t bytes) {
  if (!ptr) return FG_ERR_ARG;
  cudaError_t e = cudaMallocHost(ptr, bytes);
  if (e != cudaSuccess) {
    *ptr = nullptr;
    setLastError(std::string("fg_host_alloc: ") + cudaGetErrorString(e));
    return FG_ERR_OOM;
  }
  return FG_OK;
}

void fg_host_free(void *ptr) {
  if (ptr) cudaFreeHost(ptr);
}

}  // extern "C"
