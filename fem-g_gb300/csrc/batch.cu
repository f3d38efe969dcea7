// Batched assembly: many independent problems (element buckets of different
// meshes, orders, rules and coefficients) assembled by one fixed sequence of
// batched launches, captured once in a CUDA graph.
//
// The reference assembles problems one after another, each Formulation's
// assemble() looping over its own elements (src/problem/Formulation.cpp:1152-1215).
// Here the work of every problem goes into shared launches so that small
// problems do not leave the GPU idle between them:
//   mixed path: one factor-row launch over the elements of all problems, one
//     persistent tensor-core contraction over the tiles of all problems
//     (contiguous tile ranges per CTA balanced by cost), one row-owner
//     reduction per problem class;
//   FP64 path:  the FP64 element kernel per problem, one reduction per class.
// A class is (element type, order, quadrature rule, slot width, complex
// element matrices): its reduction shape (lanes per CSR row, warps per block)
// and, on the mixed path, the MMA width of its contraction tiles are picked by
// timing the candidates on the batch's own data in the first fg_batch_run.
// That run then executes the tuned launches directly and records them into a
// graph; later runs update the output pointers in the device-side job tables
// and launch the graph.
#include <algorithm>
#include <numeric>
#include <cstring>
#include <functional>
#include <map>
#include <tuple>
#include <vector>

#include "common.cuh"

using namespace femg;

// a failing CUDA call inside fg_batch_create: record it and undo the batch
#define FG_CUDA_RET(call, fail)                                                   \
  do {                                                                            \
    cudaError_t _e = (call);                                                      \
    if (_e != cudaSuccess) {                                                      \
      setLastError(std::string(#call) + ": " + cudaGetErrorString(_e));           \
      return fail(FG_ERR_CUDA);                                                   \
    }                                                                             \
  } while (0)

namespace {

constexpr int kTileChunk = 8;  // tiles per take of the dynamic contraction schedule

struct GatherClass {
  int dim = 0, nn = 0, n = 0, nq = 0, slotBytes = 1, kcplx = 0;
  int maxRowLen = 0;
  GatherShape shape;
  std::vector<int> probs;
  GatherJob *jobsDev = nullptr;
  GatherJob *jobsHost = nullptr;  // pinned
  int64_t blocks = 0;
};

struct GemmClass {
  int Npad = 0, K3 = 0, mmaN = 256;
  std::vector<int> probs;
};

float timeLaunches(cudaStream_t s, int reps, const std::function<int()> &f, int *st) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f;
  for (int r = 0; r < reps && *st == FG_OK; ++r) {
    cudaEventRecord(a, s);
    *st = f();
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    best = std::min(best, ms);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return best;
}

}  // namespace

struct fg_batch {
  std::vector<fg_plan *> plans;
  int mixed = 0;
  int n = 0;
  std::vector<DevTerms> terms;
  std::vector<const DevTerms *> termsDev;
  std::vector<DevTerms *> ownTermsDev;
  std::vector<std::vector<void *>> termArrays;
  std::vector<int> source;  // problem has source terms (element right-hand sides)
  std::vector<GatherClass> classes;
  // mixed path
  FactorJob *factorJobs = nullptr;
  int64_t totalElems = 0;
  std::vector<GemmProblem> gemmHost;
  GemmProblem *gemmDev = nullptr;
  std::vector<int4> tilesHost;
  int4 *tiles = nullptr;
  int32_t *ctaStart = nullptr;
  int nCta = 0, maxK3 = 0;
  size_t smem = 0;
  std::vector<GemmClass> gemmClasses;
  // contraction cost of one tile of problem q (CTA-milliseconds), measured
  // per class by the tuner; empty: the analytic estimate
  std::vector<double> tileCost;
  int *tileNext = nullptr;  // tile counter of the dynamic contraction schedule
  int *err = nullptr;
  int *errHost = nullptr;
  cudaEvent_t errEvent = nullptr;
  bool errPending = false;
  // outputs staged on the device for host pointers
  std::vector<double *> stageValues, stageRhs;
  cudaEvent_t jobsCopied = nullptr;
  // graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool tuned = false;
  std::string tuning;  // chosen shapes, as JSON
};

namespace {

int checkBatchError(fg_batch *b, bool wait) {
  if (!b->errPending) return FG_OK;
  if (wait) {
    if (cudaEventSynchronize(b->errEvent) != cudaSuccess) return FG_ERR_CUDA;
  } else if (cudaEventQuery(b->errEvent) != cudaSuccess) {
    return FG_OK;
  }
  b->errPending = false;
  if (*b->errHost) {
    *b->errHost = 0;
    cudaMemset(b->err, 0, sizeof(int));
    setLastError("batch: a tensor-core wait timed out; the outputs of that run are incomplete");
    return FG_ERR_TIMEOUT;
  }
  return FG_OK;
}

// block ranges of the class's jobs for its current shape
void layoutClass(fg_batch *b, GatherClass &c) {
  int64_t rows = 0;
  for (int q : c.probs) rows += (int64_t)b->plans[q]->d.nRows;
  const int64_t cap = (int64_t)smCount() * 16;
  int64_t start = 0;
  for (size_t k = 0; k < c.probs.size(); ++k) {
    const int64_t r = (int64_t)b->plans[c.probs[k]]->d.nRows;
    const int64_t need = (r + c.shape.rowsPerBlock - 1) / c.shape.rowsPerBlock;
    const int64_t share = rows > 0 ? (cap * r + rows - 1) / rows : 1;
    const int64_t nb = std::max<int64_t>(1, std::min(need, share));
    c.jobsHost[k].blockStart = start;
    c.jobsHost[k].nBlocks = nb;
    start += nb;
  }
  c.blocks = start;
}

int uploadJobs(GatherClass &c, cudaStream_t s) {
  FG_CUDA(cudaMemcpyAsync(c.jobsDev, c.jobsHost, c.probs.size() * sizeof(GatherJob), cudaMemcpyHostToDevice, s));
  return FG_OK;
}

int runGatherClass(fg_batch *b, GatherClass &c, cudaStream_t s) {
  return launchGatherBatch(c.jobsDev, (int)c.probs.size(), c.blocks, c.slotBytes, c.kcplx, b->mixed ? 1 : 0, c.shape, s);
}

int runElements(fg_batch *b, cudaStream_t s) {
  int st = FG_OK;
  if (b->mixed) {
    for (int q = 0; q < b->n; ++q)
      if (b->source[q])
        if ((st = launchRhsFp64(b->plans[q], b->termsDev[q], b->plans[q]->be, s))) return st;
    if ((st = launchFactorsBatch(b->factorJobs, b->n, b->totalElems, s))) return st;
    if (!b->tilesHost.empty())
      if ((st = launchContract(b->gemmDev, b->tiles, b->ctaStart, b->nCta, b->err, b->maxK3, b->smem, s, 512, nullptr,
                               b->tileNext, (int)b->tilesHost.size(), kTileChunk)))
        return st;
    return FG_OK;
  }
  for (int q = 0; q < b->n; ++q) {
    fg_plan *pl = b->plans[q];
    if (pl->d.E == 0) continue;
    if ((st = launchElementFp64(pl, b->terms[q], b->termsDev[q], pl->ke, b->source[q] ? pl->be : nullptr, s))) return st;
  }
  return FG_OK;
}

int runAll(fg_batch *b, cudaStream_t s) {
  int st = runElements(b, s);
  if (st) return st;
  for (auto &c : b->classes)
    if ((st = runGatherClass(b, c, s))) return st;
  return FG_OK;
}

// contraction schedule over the tiles of all problems (current mmaN per
// problem): contiguous tile ranges per CTA of equal total cost. The cost of a
// tile is its class's measured time per tile once the tuner has timed every
// class on its own (a tile of 16 columns costs about a sixteenth of one of
// 1232, not the 47th that its MMA work suggests: the A load and the fixed
// per-tile steps weigh more in narrow tiles), else the analytic estimate.
int buildGemmSchedule(fg_batch *b, const std::vector<int> *only, int4 **tiles, int32_t **ctaStart, int *nCta,
                      std::vector<int4> *hostTiles) {
  hostTiles->clear();
  std::vector<double> cost;
  const bool measured = !only && (int)b->tileCost.size() == b->n;
  // the final schedule takes its tiles dynamically: the costliest first, so
  // that the cheap ones even out the end
  std::vector<int> order(b->n);
  std::iota(order.begin(), order.end(), 0);
  if (measured)
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b->tileCost[x] > b->tileCost[y]; });
  for (int q : order) {
    if (only && std::find(only->begin(), only->end(), q) == only->end()) continue;
    std::vector<int4> t = mixedTiles(b->plans[q], q, b->gemmHost[q].rowsPerElem);
    const double full = measured ? b->tileCost[q] : (double)b->gemmHost[q].Npad * b->gemmHost[q].K3 + 256.0;
    for (const int4 &x : t) {
      hostTiles->push_back(x);
      // a partial tile drains fewer rows; its MMAs and loads cost the same
      cost.push_back(measured ? full * (0.5 + 0.5 * x.w / 128.0) : full);  // 128-row tiles
    }
  }
  *nCta = std::max(1, std::min(smCount(), (int)hostTiles->size()));
  std::vector<int32_t> start = partitionTiles(cost, *nCta);
  if (*tiles) cudaFree(*tiles);
  if (*ctaStart) cudaFree(*ctaStart);
  *tiles = nullptr;
  *ctaStart = nullptr;
  FG_CUDA(cudaMalloc(tiles, std::max<size_t>(hostTiles->size(), 1) * sizeof(int4)));
  if (!hostTiles->empty())
    FG_CUDA(cudaMemcpy(*tiles, hostTiles->data(), hostTiles->size() * sizeof(int4), cudaMemcpyHostToDevice));
  FG_CUDA(cudaMalloc(ctaStart, start.size() * sizeof(int32_t)));
  FG_CUDA(cudaMemcpy(*ctaStart, start.data(), start.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  return FG_OK;
}

int uploadGemmProblems(fg_batch *b) {
  FG_CUDA(cudaMemcpy(b->gemmDev, b->gemmHost.data(), b->gemmHost.size() * sizeof(GemmProblem), cudaMemcpyHostToDevice));
  return FG_OK;
}

// First run: time the candidate shapes of every class on this batch's data,
// keep the fastest, run once with them (the outputs of the call) and record
// the same launches into the graph.
int tune(fg_batch *b, cudaStream_t s) {
  int st = FG_OK;
  std::string js = "{\"gather\": [";
  if (b->mixed) {
    // contraction: MMA width per (Npad, K3) class, timed on that class's tiles
    std::string gj;
    for (size_t ci = 0; ci < b->gemmClasses.size(); ++ci) {
      GemmClass &gc = b->gemmClasses[ci];
      std::vector<int> cands;
      for (int w : {64, 128, 256})
        if (w < gc.Npad) cands.push_back(w);
      if (gc.Npad <= 256) cands.push_back(gc.Npad);  // one MMA per tile
      int4 *t = nullptr;
      int32_t *cs = nullptr;
      int nc = 0;
      std::vector<int4> ht;
      float best = 1e30f;
      int bestW = cands.back();
      // the factor rows must exist before any contraction is timed
      if (ci == 0)
        if ((st = launchFactorsBatch(b->factorJobs, b->n, b->totalElems, s))) return st;
      for (int w : cands) {
        for (int q : gc.probs) b->gemmHost[q].mmaN = w;
        if ((st = uploadGemmProblems(b))) return st;
        if ((st = buildGemmSchedule(b, &gc.probs, &t, &cs, &nc, &ht))) return st;
        const float ms = timeLaunches(s, 3, [&]() { return launchContract(b->gemmDev, t, cs, nc, b->err, b->maxK3, b->smem, s); }, &st);
        if (st) break;
        if (ms < best) {
          best = ms;
          bestW = w;
        }
      }
      cudaFree(t);
      cudaFree(cs);
      if (st) return st;
      gc.mmaN = bestW;
      for (int q : gc.probs) b->gemmHost[q].mmaN = bestW;
      if (b->tileCost.size() != (size_t)b->n) b->tileCost.assign(b->n, 0.0);
      for (int q : gc.probs) b->tileCost[q] = ht.empty() ? 0.0 : (double)best * nc / (double)ht.size();
      gj += std::string(ci ? ", " : "") + "{\"npad\": " + std::to_string(gc.Npad) + ", \"k3\": " + std::to_string(gc.K3) +
            ", \"mma_n\": " + std::to_string(bestW) + ", \"ms\": " + std::to_string(best) + "}";
    }
    if ((st = uploadGemmProblems(b))) return st;
    if ((st = buildGemmSchedule(b, nullptr, &b->tiles, &b->ctaStart, &b->nCta, &b->tilesHost))) return st;
    js = "{\"contract\": [" + gj + "], \"contract_schedule\": \"measured per-class tile costs\", \"gather\": [";
  }
  if ((st = runElements(b, s))) return st;
  for (size_t ci = 0; ci < b->classes.size(); ++ci) {
    GatherClass &c = b->classes[ci];
    const GatherShape base = gatherShape(c.n, c.maxRowLen, c.kcplx, b->mixed, 0, 0);
    std::vector<GatherShape> cands;
    for (int L : {base.L, base.L * 2})
      for (int w : {4, 8}) {
        if (L > 32) continue;
        GatherShape g = gatherShape(c.n, c.maxRowLen, c.kcplx, b->mixed, L, w);
        if (g.ok) cands.push_back(g);
      }
    // the vector-load kernel for real FP32 element matrices with n = 4k
    if (b->mixed && !c.kcplx && c.slotBytes == 1 && c.n % 4 == 0 && c.n <= 32)
      for (int w : {4, 8}) {
        GatherShape g = gatherShapeV4(c.n, c.maxRowLen, w);
        if (g.ok) cands.push_back(g);
      }
    if (cands.empty()) cands.push_back(base);
    float best = 1e30f;
    GatherShape bestShape = cands[0];
    for (const GatherShape &g : cands) {
      c.shape = g;
      layoutClass(b, c);
      if ((st = uploadJobs(c, s))) return st;
      const float ms = timeLaunches(s, 3, [&]() { return runGatherClass(b, c, s); }, &st);
      if (st) return st;
      if (ms < best) {
        best = ms;
        bestShape = g;
      }
    }
    c.shape = bestShape;
    layoutClass(b, c);
    if ((st = uploadJobs(c, s))) return st;
    js += std::string(ci ? ", " : "") + "{\"dim\": " + std::to_string(c.dim) + ", \"n\": " + std::to_string(c.n) +
          ", \"nq\": " + std::to_string(c.nq) + ", \"problems\": " + std::to_string(c.probs.size()) +
          ", \"lanes\": " + std::to_string(c.shape.L) + ", \"columns\": " + std::to_string(c.shape.J) +
          ", \"vector_loads\": " + std::string(c.shape.v4 ? "true" : "false") +
          ", \"warps\": " + std::to_string(c.shape.wpb) +
          ", \"ms\": " + std::to_string(best) + "}";
  }
  b->tuning = js + "]}";
  // the call's own results, with the chosen shapes
  if ((st = runAll(b, s))) return st;
  // the same launches into the graph
  cudaStream_t cs;
  FG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  FG_CUDA(cudaStreamSynchronize(s));
  profSuspend(true);
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    st = runAll(b, cs);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(cs, &g);
    if (st == FG_OK && e == cudaSuccess) {
      e = cudaGraphInstantiate(&b->exec, g, 0);
      b->graph = g;
    } else if (g) {
      cudaGraphDestroy(g);
    }
  }
  profSuspend(false);
  cudaStreamDestroy(cs);
  if (st) return st;
  if (e != cudaSuccess) {
    setLastError(std::string("batch: graph capture failed: ") + cudaGetErrorString(e));
    return FG_ERR_CUDA;
  }
  b->tuned = true;
  return FG_OK;
}

}  // namespace

extern "C" void fg_batch_destroy(fg_batch *b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (auto &c : b->classes) {
    cudaFree(c.jobsDev);
    if (c.jobsHost) cudaFreeHost(c.jobsHost);
  }
  for (auto *d : b->ownTermsDev) cudaFree(d);
  for (auto &v : b->termArrays)
    for (void *p : v) cudaFree(p);
  for (double *p : b->stageValues) cudaFree(p);
  for (double *p : b->stageRhs) cudaFree(p);
  cudaFree(b->factorJobs);
  cudaFree(b->gemmDev);
  cudaFree(b->tiles);
  cudaFree(b->ctaStart);
  cudaFree(b->tileNext);
  cudaFree(b->err);
  if (b->errHost) cudaFreeHost(b->errHost);
  if (b->errEvent) cudaEventDestroy(b->errEvent);
  if (b->jobsCopied) cudaEventDestroy(b->jobsCopied);
  delete b;
}

extern "C" int fg_batch_create(fg_plan *const *plans, const fg_term_desc *const *terms, const int32_t *n_terms, int32_t n_problems,
                               int32_t mixed, fg_batch **out) {
  if (!out) return FG_ERR_ARG;
  *out = nullptr;
  if (!plans || n_problems <= 0 || n_problems > 4096) {
    setLastError("fg_batch_create: 1..4096 plans required");
    return FG_ERR_ARG;
  }
  for (int32_t q = 0; q < n_problems; ++q)
    if (plans[q] && plans[q]->d.coupled) {
      setLastError("fg_batch_create: two-field plans are assembled with fg_assemble_fp64");
      return FG_ERR_UNSUPPORTED;
    }
  for (int32_t q = 0; q < n_problems; ++q)
    if (plans[q] && plans[q]->accumulate) {
      setLastError("fg_batch_create: a plan accumulates into shared outputs; batches overwrite theirs");
      return FG_ERR_UNSUPPORTED;
    }
  fg_batch *b = new (std::nothrow) fg_batch;
  if (!b) return FG_ERR_OOM;
  auto fail = [&](int st) {
    fg_batch_destroy(b);
    return st;
  };
  b->mixed = mixed ? 1 : 0;
  b->n = n_problems;
  b->plans.assign(plans, plans + n_problems);
  b->terms.resize(n_problems);
  b->termsDev.assign(n_problems, nullptr);
  b->termArrays.resize(n_problems);
  b->source.assign(n_problems, 0);
  int st = FG_OK;
  for (int q = 0; q < n_problems; ++q) {
    fg_plan *pl = plans[q];
    if (!pl) {
      setLastError("fg_batch_create: null plan");
      return fail(FG_ERR_ARG);
    }
    if (pl->d.nFixed > 0 || pl->d.lscale) {
      setLastError("fg_batch_create: problems with fixed (Dirichlet) or linked DOFs are assembled with fg_assemble_*");
      return fail(FG_ERR_UNSUPPORTED);
    }
    if (terms && terms[q]) {
      if ((st = uploadTerms(pl, terms[q], n_terms ? n_terms[q] : 0, 0.0, &b->terms[q], b->termArrays[q]))) return fail(st);
      DevTerms *d = nullptr;
      if (cudaMalloc(&d, sizeof(DevTerms)) != cudaSuccess) return fail(FG_ERR_OOM);
      b->ownTermsDev.push_back(d);
      FG_CUDA_RET(cudaMemcpy(d, &b->terms[q], sizeof(DevTerms), cudaMemcpyHostToDevice), fail);
      b->termsDev[q] = d;
    } else {
      if (!pl->hasBound) {
        setLastError("fg_batch_create: no terms given and none bound to the plan");
        return fail(FG_ERR_ARG);
      }
      b->terms[q] = pl->bound;
      b->termsDev[q] = pl->boundDev;
    }
    const DevTerms &dt = b->terms[q];
    if (dt.hasJacMod) {
      setLastError("fg_batch_create: terms with Jacobian modificators are assembled with fg_assemble_fp64");
      return fail(FG_ERR_UNSUPPORTED);
    }
    b->source[q] = dt.hasSource ? 1 : 0;
    if (b->source[q] && (st = ensureDevice((void **)&pl->be, &pl->beBytes, (size_t)pl->d.E * pl->d.n * 16))) return fail(st);
    if (b->mixed) {
      for (int t = 0; t < dt.n; ++t)
        if ((dt.t[t].kind != FG_TERM_SOURCE && dt.t[t].coef.cls == kExprPoint) || dt.tensorPoint || dt.nonSym) {
          setLastError("mixed path: bilinear coefficients must be constant per element, in symmetric terms");
          return fail(FG_ERR_UNSUPPORTED);
        }
      if ((st = prepareMixed(pl, dt.complexKe ? 2 : 1, 1))) return fail(st);
    } else {
      const int ncomp = dt.complexKe ? 2 : 1;
      if ((st = ensureDevice((void **)&pl->ke, &pl->keBytes, (size_t)pl->d.E * ncomp * pl->d.n * pl->d.n * sizeof(double)))) return fail(st);
    }
  }
  // reduction classes: (element type, order, rule, slot width, complex, field components)
  std::map<std::tuple<int, int, int, int, int, int, int>, int> classOf;
  for (int q = 0; q < n_problems; ++q) {
    const PlanDev &p = plans[q]->d;
    const int kc = b->terms[q].complexKe ? 1 : 0;
    auto key = std::make_tuple(p.dim, p.nn, p.n, p.nq, p.slotBytes, kc, p.mult);
    auto it = classOf.find(key);
    if (it == classOf.end()) {
      GatherClass c;
      c.dim = p.dim;
      c.nn = p.nn;
      c.n = p.n;
      c.nq = p.nq;
      c.slotBytes = p.slotBytes;
      c.kcplx = kc;
      it = classOf.emplace(key, (int)b->classes.size()).first;
      b->classes.push_back(c);
    }
    GatherClass &c = b->classes[it->second];
    c.probs.push_back(q);
    c.maxRowLen = std::max(c.maxRowLen, p.maxRowLen);
  }
  for (auto &c : b->classes) {
    c.shape = gatherShape(c.n, c.maxRowLen, c.kcplx, b->mixed, 0, 0);
    if (!c.shape.ok) {
      setLastError("fg_batch_create: CSR row too long for the shared-memory accumulator");
      return fail(FG_ERR_UNSUPPORTED);
    }
    if (cudaMalloc(&c.jobsDev, c.probs.size() * sizeof(GatherJob)) != cudaSuccess) return fail(FG_ERR_OOM);
    if (cudaMallocHost(&c.jobsHost, c.probs.size() * sizeof(GatherJob)) != cudaSuccess) return fail(FG_ERR_OOM);
    std::memset(c.jobsHost, 0, c.probs.size() * sizeof(GatherJob));
    for (size_t k = 0; k < c.probs.size(); ++k) {
      const int q = c.probs[k];
      fg_plan *pl = plans[q];
      GatherJob &J = c.jobsHost[k];
      J.p = pl->d;
      J.lay = keFull(pl->d.n);
      J.ke = b->mixed ? (const void *)mixedKe(pl, &J.lay) : (const void *)pl->ke;
      J.be = b->source[q] ? (const double2 *)pl->be : nullptr;
      J.uD = nullptr;
    }
    layoutClass(b, c);
  }
  if (b->mixed) {
    std::vector<FactorJob> fj;
    b->gemmHost.resize(n_problems);
    std::map<std::pair<int, int>, int> gcOf;
    for (int q = 0; q < n_problems; ++q) {
      fj.push_back(mixedFactorJob(plans[q], b->termsDev[q], b->terms[q].tensorTerm >= 0, b->totalElems));
      b->totalElems += plans[q]->d.E;
      b->gemmHost[q] = mixedGemmProblem(plans[q]);
      const GemmProblem &g = b->gemmHost[q];
      b->maxK3 = std::max(b->maxK3, g.K3);
      b->smem = std::max(b->smem, gemmSmem(g.Npad, g.K3));
      auto key = std::make_pair(g.Npad, g.K3);
      auto it = gcOf.find(key);
      if (it == gcOf.end()) {
        GemmClass gc;
        gc.Npad = g.Npad;
        gc.K3 = g.K3;
        it = gcOf.emplace(key, (int)b->gemmClasses.size()).first;
        b->gemmClasses.push_back(gc);
      }
      b->gemmClasses[it->second].probs.push_back(q);
    }
    // the A region is sized by the largest K3 of the launch
    size_t smemMax = 0;
    for (int q = 0; q < n_problems; ++q)
      smemMax = std::max(smemMax, gemmSmem(b->gemmHost[q].Npad, b->maxK3));
    b->smem = std::max(b->smem, smemMax);
    if (b->smem > 220 * 1024) {
      setLastError("fg_batch_create: contraction tiles too large for shared memory");
      return fail(FG_ERR_UNSUPPORTED);
    }
    if (cudaMalloc(&b->factorJobs, fj.size() * sizeof(FactorJob)) != cudaSuccess) return fail(FG_ERR_OOM);
    FG_CUDA_RET(cudaMemcpy(b->factorJobs, fj.data(), fj.size() * sizeof(FactorJob), cudaMemcpyHostToDevice), fail);
    if (cudaMalloc(&b->gemmDev, n_problems * sizeof(GemmProblem)) != cudaSuccess) return fail(FG_ERR_OOM);
    if ((st = uploadGemmProblems(b))) return fail(st);
    if ((st = buildGemmSchedule(b, nullptr, &b->tiles, &b->ctaStart, &b->nCta, &b->tilesHost))) return fail(st);
    if (cudaMalloc(&b->err, sizeof(int)) != cudaSuccess) return fail(FG_ERR_OOM);
    if (cudaMalloc(&b->tileNext, sizeof(int)) != cudaSuccess) return fail(FG_ERR_OOM);
    FG_CUDA_RET(cudaMemset(b->err, 0, sizeof(int)), fail);
    if (cudaMallocHost(&b->errHost, sizeof(int)) != cudaSuccess) return fail(FG_ERR_OOM);
    *b->errHost = 0;
    FG_CUDA_RET(cudaEventCreateWithFlags(&b->errEvent, cudaEventDisableTiming), fail);
  }
  FG_CUDA_RET(cudaEventCreateWithFlags(&b->jobsCopied, cudaEventDisableTiming), fail);
  b->stageValues.assign(n_problems, nullptr);
  b->stageRhs.assign(n_problems, nullptr);
  *out = b;
  return FG_OK;
}

extern "C" int fg_batch_run(fg_batch *b, double *const *csr_values, double *const *rhs, void *stream) {
  if (!b || !csr_values) return FG_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  int st = checkBatchError(b, false);
  if (st) return st;
  // output pointers of this run (host outputs through device staging)
  std::vector<char> hostV(b->n, 0), hostR(b->n, 0);
  std::vector<double *> dv(b->n), dr(b->n, nullptr);
  for (int q = 0; q < b->n; ++q) {
    const PlanDev &p = b->plans[q]->d;
    if (!csr_values[q]) {
      setLastError("fg_batch_run: csr_values[p] must not be NULL");
      return FG_ERR_ARG;
    }
    dv[q] = csr_values[q];
    if (!isDevicePointer(csr_values[q])) {
      hostV[q] = 1;
      size_t cap = b->stageValues[q] ? (size_t)p.nnz * 16 : 0;
      if ((st = ensureDevice((void **)&b->stageValues[q], &cap, (size_t)p.nnz * 16))) return st;
      dv[q] = b->stageValues[q];
    }
    if (rhs && rhs[q]) {
      dr[q] = rhs[q];
      if (!isDevicePointer(rhs[q])) {
        hostR[q] = 1;
        size_t cap = b->stageRhs[q] ? (size_t)p.nRows * 16 : 0;
        if ((st = ensureDevice((void **)&b->stageRhs[q], &cap, (size_t)p.nRows * 16))) return st;
        dr[q] = b->stageRhs[q];
      }
    }
  }
  FG_CUDA(cudaEventSynchronize(b->jobsCopied));  // the pinned job tables are free again
  for (auto &c : b->classes) {
    for (size_t k = 0; k < c.probs.size(); ++k) {
      c.jobsHost[k].values = (double2 *)dv[c.probs[k]];
      c.jobsHost[k].rhs = (double2 *)dr[c.probs[k]];
    }
    if ((st = uploadJobs(c, s))) return st;
  }
  FG_CUDA(cudaEventRecord(b->jobsCopied, s));
  if (!b->tuned) {
    if ((st = tune(b, s))) return st;
  } else if (profEnabled()) {
    // with the kernel timer on, the launches run one by one (the graph's
    // kernels cannot be timed apart), the same launches the graph holds
    if ((st = runAll(b, s))) return st;
  } else {
    ProfScope prof("fg_batch_graph", s);
    int nSource = 0;
    for (int q = 0; q < b->n; ++q) nSource += b->source[q];
    countLaunch((int)b->classes.size() + (b->mixed ? 2 + nSource : b->n));
    FG_CUDA(cudaGraphLaunch(b->exec, s));
  }
  if (b->mixed) {
    FG_CUDA(cudaMemcpyAsync(b->errHost, b->err, sizeof(int), cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaEventRecord(b->errEvent, s));
    b->errPending = true;
  }
  bool anyHost = false;
  for (int q = 0; q < b->n; ++q) {
    const PlanDev &p = b->plans[q]->d;
    if (hostV[q]) FG_CUDA(cudaMemcpyAsync(csr_values[q], dv[q], (size_t)p.nnz * 16, cudaMemcpyDeviceToHost, s));
    if (hostR[q]) FG_CUDA(cudaMemcpyAsync(rhs[q], dr[q], (size_t)p.nRows * 16, cudaMemcpyDeviceToHost, s));
    anyHost = anyHost || hostV[q] || hostR[q];
  }
  if (anyHost) {
    FG_CUDA(cudaStreamSynchronize(s));
    return checkBatchError(b, true);
  }
  return FG_OK;
}

extern "C" const char *fg_batch_tuning(const fg_batch *b) { return b ? b->tuning.c_str() : ""; }
