// Host runtime of libhpgpu.so: contexts, jobs, the batched outer-iteration
// driver and the C ABI declared in include/hpgpu.h.
//
// The outer loop mirrors AbstractISAWPart.do_partitioning
// (core/iterstock.py:159-193) for MBIS/GISA/aLISA and the gLISA solver loops
// (glisa.py:617-848); each call of hp_step advances every live job of a batch
// by one outer iteration with batched kernel launches on the context stream
// and a single host wait at the end (plus one per inner-solver chunk).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "hp_internal.cuh"
#include "hpgpu.h"

using namespace hp;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define HP_CK(call)                                                                   \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess)                                                            \
      return fail(HP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));   \
  } while (0)

constexpr int kMaxSlots = 4096;
constexpr size_t kAlign = 256;

size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

}  // namespace

namespace hp {
void set_error_text(const char* msg) { g_err = msg ? msg : ""; }
}  // namespace hp

struct hp_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  size_t budget = 0, used = 0;
  Mailbox* mail_dev = nullptr;
  Mailbox* mail_host = nullptr;
  std::vector<hp_job*> slots;
  JobDev* batch_dev = nullptr;     // JobDev array of the current batch
  JobDev* batch_host = nullptr;    // pinned staging
  int* prefix_dev = nullptr;       // [K_NKIND][kMaxSlots + 1]
  int* prefix_host = nullptr;      // pinned staging
  // kernel timing (hp_ctx_profile)
  bool prof = false;
  struct Pending {
    int fam;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> event_pool;
  double prof_ms[HP_KERNEL_COUNT] = {};
  int64_t prof_n[HP_KERNEL_COUNT] = {};
  long long launch_base = 0;
  int slots_hi = 0;  // one past the highest slot a job has used (mailboxes to read back)
  // Job memory (the carved job allocation and the packed G of fused gLISA
  // jobs) comes from this stream-ordered pool on the context's stream; freed
  // blocks stay in the pool (release threshold: never), so that a stream of
  // job creations and destructions does not map and unmap device memory
  // each time. Destroying the context returns it to the device.
  cudaMemPool_t pool = nullptr;
  // A second stream for the end-of-iteration bookkeeping of fused gLISA
  // jobs (k_glisa_point_ff, k_outer_finish), which then overlaps the next
  // iteration's reductions and Newton step (step_glisa); fork and join by
  // events.
  cudaStream_t side = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
};

namespace {

cudaError_t job_alloc(hp_ctx* c, void** p, size_t bytes) {
  return cudaMallocFromPoolAsync(p, bytes, c->pool, c->stream);
}

void job_free(hp_ctx* c, void* p) {
  if (p) cudaFreeAsync(p, c->stream);
}

}  // namespace

struct hp_job {
  hp_ctx* ctx = nullptr;
  int slot = -1;
  hp_job_desc desc{};
  JobDev dev{};
  void* mem = nullptr;
  size_t bytes = 0;
  // host-side state
  bool initialized = false;
  bool done = false;
  int status = HP_OK;
  int niter = 0;
  double change = 0.0;
  uint32_t warnings = 0;
  int last_inner = 4;
  double evals = 0.0;
  double inner_total = 0.0;
  bool converged = false;
  double prev_change = 1e300;
  int polish_iters = 0;  // outer iterations of a mixed job after its FP32 phase (FF or FP64)
  int f64_factors = 0;   // tensor-core gLISA: Newton steps factored in FP64
  int64_t g_active = -1; // fused gLISA: G values in the tiles' active rows (-1: not read yet)
  double skipped = 0.0;  // point-atom evaluations skipped by the per-atom cutoff
  bool host_driven = false;  // finished by hp_glisa_finish (histories kept by the host)
  void* pack_mem = nullptr;  // fused gLISA: packed G (dev.gpack, dev.gtile_off)
  size_t pack_bytes = 0;
  std::vector<double> changes;  // outer changes of this run
};

namespace {

// State of a mixed-precision job after an outer iteration:
//   MIXED_FLOOR: the outer change has stopped decreasing (the best change of
//     the last kFloorWindow iterations is not below the best of the window
//     before): the FP32 noise floor. A slowly but steadily converging job
//     (linear rate up to 0.999 per iteration) never reaches this state.
//   MIXED_NEAR: the change is within kNearFactor x the threshold.
enum MixedState { MIXED_GO = 0, MIXED_NEAR = 1, MIXED_FLOOR = 2 };
constexpr size_t kFloorWindow = 8;
constexpr double kNearFactor = 100.0;

int mixed_state(const hp_job* j) {
  const size_t n = j->changes.size();
  if (n >= 2 * kFloorWindow) {
    double a = 1e300, b = 1e300;
    for (size_t i = n - 2 * kFloorWindow; i < n - kFloorWindow; ++i) a = std::min(a, j->changes[i]);
    for (size_t i = n - kFloorWindow; i < n; ++i) b = std::min(b, j->changes[i]);
    if (b >= 0.999 * a) return MIXED_FLOOR;
  }
  if (j->change < kNearFactor * j->desc.threshold) return MIXED_NEAR;
  return MIXED_GO;
}

}  // namespace

namespace {

cudaEvent_t take_event(hp_ctx* ctx) {
  if (!ctx->event_pool.empty()) {
    cudaEvent_t e = ctx->event_pool.back();
    ctx->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Records CUDA events around the launches of one kernel family.
struct ProfScope {
  hp_ctx* ctx;
  int fam;
  cudaEvent_t a = nullptr;
  ProfScope(hp_ctx* c, int f) : ctx(c), fam(f) {
    if (ctx->prof) {
      a = take_event(ctx);
      cudaEventRecord(a, ctx->stream);
    }
  }
  ~ProfScope() {
    if (a) {
      cudaEvent_t b = take_event(ctx);
      cudaEventRecord(b, ctx->stream);
      ctx->pending.push_back({fam, a, b});
    }
  }
};

// After a stream synchronisation: fold finished event pairs into the totals.
void prof_collect(hp_ctx* ctx) {
  for (auto& p : ctx->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      ctx->prof_ms[p.fam] += ms;
      ctx->prof_n[p.fam] += 1;
    }
    ctx->event_pool.push_back(p.a);
    ctx->event_pool.push_back(p.b);
  }
  ctx->pending.clear();
}

int blocks_for(const JobDev& J, int kind) {
  switch (kind) {
    case K_POINT: return J.ntile;
    case K_POINT1: return (J.npoint + kThreads - 1) / kThreads;
    case K_ATOM_TILE: return J.natom * J.ntile;
    case K_ATOM: return J.natom;
    case K_JOB: return 1;
    case K_FUSE: return J.fuse ? std::min(J.ntile, kFuseCtas) : 0;
    case K_HESS:
      if (J.scheme != SCHEME_GLISA || J.fuse) return 0;  // fused jobs: in the fused pass
      return J.tc ? tc_hess_blocks(J) : J.nsplit * J.htiles * (J.htiles + 1) / 2;
    case K_SQUARE: return J.scheme == SCHEME_GLISA ? (J.nshell * J.nshell + kThreads - 1) / kThreads : 0;
  }
  return 0;
}

// Upload the batch description (JobDev copies and per-kind block prefixes).
int build_batch(hp_ctx* ctx, const std::vector<hp_job*>& jobs, HostBatch& hb) {
  const int n = (int)jobs.size();
  hb.nact_max = 0;
  for (int j = 0; j < n; ++j) {
    ctx->batch_host[j] = jobs[j]->dev;
    hb.nact_max = std::max(hb.nact_max, jobs[j]->dev.nact_max);
  }
  HP_CK(cudaMemcpyAsync(ctx->batch_dev, ctx->batch_host, sizeof(JobDev) * n,
                        cudaMemcpyHostToDevice, ctx->stream));
  for (int k = 0; k < K_NKIND; ++k) {
    int* pre = ctx->prefix_host + (size_t)k * (kMaxSlots + 1);
    pre[0] = 0;
    for (int j = 0; j < n; ++j) pre[j + 1] = pre[j] + blocks_for(jobs[j]->dev, k);
    hb.blocks[k] = pre[n];
    hb.b[k].jobs = ctx->batch_dev;
    hb.b[k].prefix = ctx->prefix_dev + (size_t)k * (kMaxSlots + 1);
    hb.b[k].njobs = n;
  }
  HP_CK(cudaMemcpyAsync(ctx->prefix_dev, ctx->prefix_host,
                        sizeof(int) * K_NKIND * (kMaxSlots + 1), cudaMemcpyHostToDevice,
                        ctx->stream));
  return HP_OK;
}

int read_mail(hp_ctx* ctx) {
  const int n = std::max(1, ctx->slots_hi);
  HP_CK(cudaMemcpyAsync(ctx->mail_host, ctx->mail_dev, sizeof(Mailbox) * n,
                        cudaMemcpyDeviceToHost, ctx->stream));
  HP_CK(cudaStreamSynchronize(ctx->stream));
  prof_collect(ctx);
  return HP_OK;
}

int check_launch() {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(HP_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return HP_OK;
}

int model_of(const hp_job* j) {
  return j->desc.scheme == HP_SCHEME_MBIS ? MODEL_MBIS
         : j->desc.scheme == HP_SCHEME_NLIS ? MODEL_NLIS
                                            : MODEL_BASIS;
}

// Map device error bits to a status.
int status_of(int err) {
  if (err == 0) return HP_OK;
  if (err & E_TIMEOUT) return HP_ERR_TIMEOUT;
  if (err & E_INNER_NOT_CONV) return HP_ERR_NOT_CONVERGED;
  return HP_ERR_NUMERIC;
}

const char* err_text(int err) {
  if (err & E_TIMEOUT) return "tensor-core Hessian: a bounded device wait ran out; MMAs issued before it may not have retired, so treat this context as suspect and recreate it";
  if (err & E_NEG_DENSITY) return "Negative pro-atom density found!";
  if (err & E_SINGULAR) return "Hessian is not positive definite (singular Newton system)";
  if (err & E_LINESEARCH) return "Line search failed!";
  if (err & E_INNER_NOT_CONV) return "Inner loop: Newton does not converge!";
  if (err & E_QP) return "GISA quadratic program did not converge";
  return "numerical failure";
}

// Inner-solver loop for a batch: launch chunks of inner iterations until no
// atom of any job is active.
template <typename F>
int run_inner(hp_ctx* ctx, const std::vector<hp_job*>& jobs, const HostBatch& hb, F launch_one,
              int max_launch) {
  launch_inner_init(hb, ctx->stream);
  int chunk = 1;
  for (hp_job* j : jobs) chunk = std::max(chunk, j->last_inner);
  int launched = 0;
  while (true) {
    for (int c = 0; c < chunk && launched < max_launch; ++c, ++launched) launch_one();
    launch_count_active(hb, ctx->stream);
    int rc = check_launch();
    if (rc) return rc;
    rc = read_mail(ctx);
    if (rc) return rc;
    int nact = 0;
    for (hp_job* j : jobs) nact += ctx->mail_host[j->slot].i[MI_NACTIVE];
    if (nact == 0) break;
    if (launched >= max_launch) break;
    chunk = 2;
  }
  for (hp_job* j : jobs) j->last_inner = std::max(1, std::min(launched, 64));
  return HP_OK;
}

// Work of a point tile in a fused pass, in row-equivalents per sub-tile: its
// active rows plus the per-sub-tile cost that does not depend on them (the
// per-point step, barriers and staging waits; about a hundred rows' worth
// measured on the 150-shell benchmark molecule, 64 taken).
constexpr int64_t kTileFixedRows = 64;

// Tile schedule of the fused passes (longest processing time first): the
// tiles by decreasing work (ties by index) each go to the least loaded of
// the nb persistent blocks (ties by block index); each block then takes its
// tiles in ascending order. A block's Hessian partial accumulates its tiles
// in that order, so the schedule, a function of the job's own active-row
// counts, keeps a job's results the same alone and in a batch. The trial
// pass (one block per tile) visits the tiles heaviest first, which the block
// scheduler turns into the same kind of balance.
std::vector<int> tile_schedule(const std::vector<int64_t>& work, int nb) {
  const int nt = (int)work.size();
  std::vector<int> order(nt);
  for (int t = 0; t < nt; ++t) order[t] = t;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return work[a] > work[b]; });
  std::vector<int64_t> load(nb, 0);
  std::vector<int> owner(nt, 0);
  // min-heap of (load, block): the comparator orders larger loads (then larger blocks) first
  std::vector<std::pair<int64_t, int>> heap;
  for (int b = 0; b < nb; ++b) heap.push_back({0, b});
  auto cmp = [](const std::pair<int64_t, int>& x, const std::pair<int64_t, int>& y) {
    return x.first != y.first ? x.first > y.first : x.second > y.second;
  };
  std::make_heap(heap.begin(), heap.end(), cmp);
  for (int t : order) {
    std::pop_heap(heap.begin(), heap.end(), cmp);
    auto& top = heap.back();
    owner[t] = top.second;
    top.first += work[t];
    std::push_heap(heap.begin(), heap.end(), cmp);
  }
  std::vector<int> out((size_t)nb + 1 + 2 * (size_t)nt, 0);
  for (int t = 0; t < nt; ++t) out[owner[t] + 1] += 1;
  for (int b = 0; b < nb; ++b) out[b + 1] += out[b];
  std::vector<int> fill(out.begin(), out.begin() + nb);
  for (int t = 0; t < nt; ++t) out[nb + 1 + fill[owner[t]]++] = t;  // ascending within a block
  for (int k = 0; k < nt; ++k) out[(size_t)nb + 1 + nt + k] = order[k];
  return out;
}

// Fused gLISA jobs: the packed layout of G's active rows (k_glisa_pack)
// from the per-tile active-row counts of k_glisa_active: tile t's sub-tiles
// start at gtile_off[t] in each plane and hold nact_t rows of 32 floats each;
// and the tile schedule of the passes (tile_schedule). The arrays are
// allocated at the first initialisation of a job (the counts depend only on
// G) and charged to the context.
int pack_layout(hp_ctx* ctx, const std::vector<hp_job*>& jobs) {
  bool any = false;
  for (hp_job* j : jobs) any |= j->dev.fuse && !j->dev.gpack;
  if (!any) return HP_OK;
  HP_CK(cudaStreamSynchronize(ctx->stream));
  for (hp_job* j : jobs) {
    JobDev& J = j->dev;
    if (!J.fuse || J.gpack) continue;
    const int S = J.nshell;
    std::vector<int> g((size_t)(S + 1) * J.ntile);
    HP_CK(cudaMemcpy(g.data(), J.gact, sizeof(int) * g.size(), cudaMemcpyDeviceToHost));
    std::vector<int64_t> off(J.ntile), work(J.ntile);
    int64_t total = 0;
    int nmax = 0;
    for (int t = 0; t < J.ntile; ++t) {
      const int nact = g[(size_t)t * (S + 1) + S];
      const int64_t pts = std::min<int64_t>(J.tile_points, (int64_t)J.npoint - (int64_t)t * J.tile_points);
      const int64_t nsub = (pts + 31) / 32;
      off[t] = total;
      total += nsub * 32 * (int64_t)nact;
      nmax = std::max(nmax, nact);
      work[t] = nsub * (nact + kTileFixedRows);
    }
    const int nb = std::min(J.ntile, kFuseCtas);
    const std::vector<int> sched = tile_schedule(work, nb);
    const size_t gbytes = 2 * 4 * (size_t)std::max<int64_t>(total, 1);
    const size_t bytes = gbytes + 8 * (size_t)J.ntile + 4 * sched.size();
    if (ctx->used + bytes > ctx->budget) return fail(HP_ERR_NO_MEMORY, "HBM budget exceeded (packed G)");
    void* mem = nullptr;
    if (job_alloc(ctx, &mem, bytes) != cudaSuccess) {
      cudaGetLastError();
      return fail(HP_ERR_NO_MEMORY, "device allocation failed");
    }
    J.gpack = reinterpret_cast<float*>(mem);
    J.gpack_plane = total;
    J.gtile_off = reinterpret_cast<int64_t*>(reinterpret_cast<char*>(mem) + gbytes);
    J.fsched = reinterpret_cast<int*>(reinterpret_cast<char*>(mem) + gbytes + 8 * (size_t)J.ntile);
    J.nact_max = nmax;
    j->pack_mem = mem;
    j->pack_bytes = bytes;
    j->bytes += bytes;
    ctx->used += bytes;
    // on the context stream, where the allocation is ordered (pageable
    // sources: each call returns once its source has been read)
    HP_CK(cudaMemcpyAsync(J.gtile_off, off.data(), 8 * (size_t)J.ntile, cudaMemcpyHostToDevice, ctx->stream));
    HP_CK(cudaMemcpyAsync(J.fsched, sched.data(), 4 * sched.size(), cudaMemcpyHostToDevice, ctx->stream));
  }
  return HP_OK;
}

int job_init(hp_ctx* ctx, const std::vector<hp_job*>& jobs, const HostBatch& hb) {
  launch_nelec(hb, ctx->stream);
  bool any_basis = false, any_basis_ff = false, any_rdist = false;
  for (hp_job* j : jobs) {
    any_basis |= j->dev.gmat != nullptr;
    any_basis_ff |= j->dev.gmat_lo != nullptr;
    any_rdist |= j->dev.rdist != nullptr;
  }
  if (any_rdist) launch_rdist_ff(hb, ctx->stream);
  if (any_basis) launch_glisa_basis(hb, ctx->stream);
  if (any_basis_ff) launch_glisa_basis_ff(hb, ctx->stream);
  int fuse_shells = 0;
  for (hp_job* j : jobs)
    if (j->dev.fuse) fuse_shells = std::max(fuse_shells, j->dev.nshell);
  // fused gLISA jobs: active shells per tile, then the first iteration's
  // promolecule and gradient
  if (fuse_shells > 0) {
    launch_glisa_active(hb, ctx->stream);
    int rc = pack_layout(ctx, jobs);
    if (rc) return rc;
    HostBatch hp;  // the jobs' descriptors now carry the packed arrays
    rc = build_batch(ctx, jobs, hp);
    if (rc) return rc;
    // the Gram blocks (tensor cores, from the dense planes) on the side
    // stream while the main stream packs G; joined before the first fused
    // pass, which overwrites hpart
    cudaEventRecord(ctx->fork_ev, ctx->stream);
    cudaStreamWaitEvent(ctx->side, ctx->fork_ev, 0);
    launch_glisa_wgram(hp, ctx->side);
    cudaEventRecord(ctx->join_ev, ctx->side);
    launch_glisa_pack(hp, ctx->stream);
    cudaStreamWaitEvent(ctx->stream, ctx->join_ev, 0);
    launch_glisa_fused_ff(hp, ctx->stream, 1, fuse_shells);
  }
  for (hp_job* j : jobs) j->initialized = true;
  return check_launch();
}

// One outer iteration of MBIS / GISA / aLISA for a homogeneous batch.
int step_iterstock(hp_ctx* ctx, const std::vector<hp_job*>& jobs, const HostBatch& hb) {
  const hp_job* j0 = jobs[0];
  const int mixed = j0->dev.mixed;  // current phase (a mixed job may finish in FP64)
  const int model = model_of(j0);
  cudaStream_t st = ctx->stream;
  launch_copy_old(hb, st);
  {
    ProfScope ps(ctx, HP_KERNEL_PROMOL);
    launch_promol(hb, st, mixed, model);
  }
  int rc = HP_OK;
  const bool local = j0->dev.local != 0;
  switch (j0->desc.scheme) {
    case HP_SCHEME_MBIS:
      if (local) {  // atom grids: every inner iteration of every atom in one launch
        ProfScope ps(ctx, HP_KERNEL_INNER);
        launch_inner_init(hb, st);
        launch_mbis_local(hb, st);
      } else {
        rc = run_inner(ctx, jobs, hb, [&] {
          ProfScope ps(ctx, HP_KERNEL_INNER);
          launch_mbis_inner(hb, st, mixed);
        }, j0->dev.inner_maxiter + 1);
      }
      break;
    case HP_SCHEME_NLIS:  // NLIS / GMBIS (FP64)
      if (local) {
        ProfScope ps(ctx, HP_KERNEL_INNER);
        launch_inner_init(hb, st);
        launch_nlis_local(hb, st);
      } else {
        rc = run_inner(ctx, jobs, hb, [&] {
          ProfScope ps(ctx, HP_KERNEL_INNER);
          launch_nlis_inner(hb, st);
        }, j0->dev.inner_maxiter + 1);
      }
      break;
    case HP_SCHEME_GISA: {
      ProfScope ps(ctx, HP_KERNEL_INNER);
      if (local) {  // moments on the radial grids, the same quadratic program
        launch_gisa_local(hb, st);
        launch_gisa_qp(hb, st);
      } else {
        launch_gisa(hb, st, mixed);
      }
      break;
    }
    case HP_SCHEME_LISA:
      if (local) {  // atom grids: every inner iteration of every atom in one launch
        ProfScope ps(ctx, HP_KERNEL_INNER);
        launch_inner_init(hb, st);
        launch_lisa_sc_local(hb, st);
      } else if (j0->dev.solver == SOLVER_SC)
        rc = run_inner(ctx, jobs, hb, [&] {
          ProfScope ps(ctx, HP_KERNEL_INNER);
          launch_lisa_sc_inner(hb, st, mixed);
        }, j0->dev.inner_maxiter + 1);
      else
        rc = run_inner(ctx, jobs, hb, [&] {
          ProfScope ps(ctx, HP_KERNEL_INNER);
          launch_lisa_newton_inner(hb, st, mixed,
                                   j0->dev.solver == SOLVER_M_NEWTON || j0->dev.solver == SOLVER_BFGS);
        }, j0->dev.inner_maxiter + 1);
      break;
  }
  if (rc) return rc;
  {
    ProfScope ps(ctx, HP_KERNEL_CHANGE);
    if (local) launch_change_radial(hb, st);
    else launch_change(hb, st, mixed, model);
  }
  launch_outer_finish(hb, st, 1);
  rc = check_launch();
  if (rc) return rc;
  rc = read_mail(ctx);
  if (rc) return rc;
  for (hp_job* j : jobs) {
    const Mailbox& m = ctx->mail_host[j->slot];
    j->niter = m.i[MI_ITER];
    j->change = m.d[MD_CHANGE];
    j->changes.push_back(j->change);
    j->warnings |= (uint32_t)m.i[MI_WARN];
    const double inner = m.d[MD_INNER_TOTAL];
    j->inner_total += inner;
    j->skipped = m.d[MD_SKIPPED];
    // point-atom evaluations in the reference's convention: weights pass,
    // one per inner iteration, two in compute_change (GISA: one q-vector pass)
    const double n = (double)j->dev.npoint;
    const double a = (double)j->dev.natom;
    const double inner_evals = j->desc.scheme == HP_SCHEME_GISA ? a : inner;
    if (j->dev.local)  // promolecule on the molecular grid; inner and change on the radial grids
      j->evals += n * a + (inner_evals + 2.0 * a) * (double)j->dev.nrad / a;
    else
      j->evals += n * (3.0 * a + inner_evals);
    if (j->dev.mixed != PH_FP32 && j->desc.precision == HP_PRECISION_MIXED) j->polish_iters += 1;
    if (m.i[MI_ERR]) {
      j->status = status_of(m.i[MI_ERR]);
      g_err = err_text(m.i[MI_ERR]);
      j->done = true;
    } else if (j->change < j->desc.threshold || j->niter >= j->desc.maxiter) {
      j->converged = j->change < j->desc.threshold;
      j->done = true;
    } else if (j->dev.mixed == PH_FP32) {
      // polish: finish in FP64 once the FP32-evaluated change is near the
      // threshold or at its noise floor (every buffer is rewritten by the
      // next FP64 pass); without polish, stay in FP32 until the threshold and
      // stop with a warning only at the noise floor
      const int st = mixed_state(j);
      if (j->desc.polish && st != MIXED_GO) {
        // MBIS finishes in float-float (FP64-class results on the FP32
        // pipes), the basis schemes in FP64
        j->dev.mixed = j->desc.scheme == HP_SCHEME_MBIS ? PH_FF : PH_FP64;
      } else if (!j->desc.polish && st == MIXED_FLOOR) {
        j->warnings |= HP_WARN_NOISE_FLOOR;
        j->converged = true;
        j->done = true;
      }
    }
    j->prev_change = j->change;
  }
  return HP_OK;
}

// Refinement steps per Newton iteration of the finish when the Hessian comes
// from the tensor cores (each: one exact H delta product, one fused pass over
// G); the kernels skip the jobs not in their finish (glisa_refine_now). The
// factor of the tensor-core Hessian leaves a relative direction error of
// ~1e-6; one step brings it to ~1e-12.
constexpr int kRefineSteps = 1;

// Up to `iters` gLISA solver iterations (glisa.py:748-798 for Newton,
// 805-848 for SC) queued back to back, then one host round trip. The device
// marks a job finished at the end of the iteration that converges, fails or
// reaches maxiter (MI_DONE, k_outer_finish), and the kernels of the queued
// iterations after it return at once for that job, so the results are those
// of one iteration per round trip. The m-newton line search needs the host
// between iterations (its retry pass), so it takes one iteration per call.
int step_glisa(hp_ctx* ctx, const std::vector<hp_job*>& jobs, const HostBatch& hb, int iters) {
  cudaStream_t st = ctx->stream;
  const int solver = jobs[0]->dev.solver;
  if (solver == SOLVER_M_NEWTON) iters = 1;
  const bool tc = jobs[0]->dev.tc != 0;
  const int gff = jobs[0]->dev.gff;
  // Jobs with at most kFuseMaxShells shells (batches are homogeneous in
  // this) take the fused passes: the promolecule + gradient (+ Hessian) pass
  // of an iteration runs at the end of the previous step (or at job start)
  // and also forms that step's change; the others take separate passes.
  const bool fused = jobs[0]->dev.fuse != 0;
  int fuse_shells = 0;
  for (hp_job* j : jobs) fuse_shells = std::max(fuse_shells, j->dev.nshell);
  if (!fused) fuse_shells = 0;
  const int unfused = fused ? 0 : 1;
  // fused projected-Newton jobs on the molecular grid: the point pass and
  // k_outer_finish of an iteration run on the side stream while the next
  // iteration's reduction and Newton step run here; the join comes before
  // the refinement, which reads the change that k_outer_finish writes
  // (glisa_refine_now), and before the trials, whose kernels must see the
  // job's done flag. The reduction and the Newton step read none of the
  // side kernels' outputs (a job that finished in the last iteration only
  // costs them a wasted pass; its parameters are not touched before the
  // join).
  bool any_local = false;
  for (hp_job* j : jobs) any_local |= j->dev.local != 0;
  const bool overlap = fused && !any_local && solver == SOLVER_PNEWTON && ctx->side != nullptr;
  bool pending = false;  // side work of the previous iteration not yet joined
  auto join = [&]() {
    if (pending) {
      cudaStreamWaitEvent(st, ctx->join_ev, 0);
      pending = false;
    }
  };
  for (int iter = 0; iter < iters; ++iter) {
  // projected Newton keeps the step's start in k_glisa_trial_pick
  if (solver != SOLVER_PNEWTON) launch_copy_old(hb, st);
  if (!fused) {
    ProfScope ps(ctx, HP_KERNEL_GLISA_PRO);
    if (gff) launch_glisa_pro_ff(hb, st);
    else launch_glisa_pro(hb, st);
  }
  if (!fused) {
    ProfScope ps(ctx, HP_KERNEL_GLISA_GRAD);
    if (gff) launch_glisa_grad_ff(hb, st);
    else launch_glisa_grad(hb, st);
  }
  if (solver != SOLVER_SC && !fused) {  // fused jobs: the Hessian comes with the fused pass
    ProfScope ps(ctx, HP_KERNEL_GLISA_HESS);
    if (tc) {
      int smax = 0, smin = 1 << 30;
      for (hp_job* j : jobs) {
        smax = std::max(smax, j->dev.nshell);
        smin = std::min(smin, j->dev.nshell);
      }
      launch_glisa_hess_tc(hb, st, smax, smin);
    }
    else launch_glisa_hess(hb, st);
  }
  {
    ProfScope ps(ctx, HP_KERNEL_GLISA_SOLVE);
    launch_glisa_reduce(hb, st);
    if (solver != SOLVER_SC) {
      // Newton system with the FP64 Hessian, or with the tensor-core one plus
      // iterative refinement against the exact FP64 product H delta.
      int smax = 0;
      for (hp_job* j : jobs) smax = std::max(smax, j->dev.nshell);
      launch_glisa_solve(hb, st, solver == SOLVER_PNEWTON ? 1 : 0, smax, tc ? 1 : 0);
      join();
      if (tc)
        for (int k = 0; k < kRefineSteps; ++k) launch_glisa_refine(hb, st, gff, fuse_shells, unfused);
    }
  }
  {
    ProfScope ps(ctx, HP_KERNEL_GLISA_TRIALS);
    if (solver == SOLVER_SC) {
      launch_glisa_apply(hb, st, 1);
    } else if (solver == SOLVER_PNEWTON) {
      launch_glisa_pnewton(hb, st, gff, fuse_shells);
    } else if (solver != SOLVER_SC) {
      if (solver == SOLVER_NEWTON) launch_glisa_apply(hb, st, 0);
      else {
        launch_glisa_keep(hb, st);
        launch_glisa_ls(hb, st, 0, 1);
      }
    }
  }
  if (solver == SOLVER_M_NEWTON) {
    {
      int rc = check_launch();
      if (rc) return rc;
      rc = read_mail(ctx);
      if (rc) return rc;
      bool retry = false;
      for (hp_job* j : jobs) retry |= ctx->mail_host[j->slot].d[MD_LS_X] < 0.0;
      if (retry) {
        // all remaining trials in one pass; jobs that already accepted x = tau
        // see no change because their propars were updated (first trial valid
        // again is not possible: only failed jobs are re-run below)
        std::vector<hp_job*> failed;
        for (hp_job* j : jobs)
          if (ctx->mail_host[j->slot].d[MD_LS_X] < 0.0) failed.push_back(j);
        HostBatch hb2;
        rc = build_batch(ctx, failed, hb2);
        if (rc) return rc;
        const int L = failed[0]->dev.linspace_size;
        launch_glisa_ls(hb2, st, 1, std::min(L - 1, 64));
        rc = check_launch();
        if (rc) return rc;
        rc = read_mail(ctx);
        if (rc) return rc;
        for (hp_job* j : failed)
          if (ctx->mail_host[j->slot].d[MD_LS_X] < 0.0) {
            j->status = HP_ERR_NUMERIC;
            g_err = "Line search failed!";
            j->done = true;
          }
        rc = build_batch(ctx, jobs, hb2);
        if (rc) return rc;
      }
    }
  }
  // the change: atom grids radial; fused jobs on the molecular grid from the
  // per-atom Gram blocks (in k_outer_finish); the others one pass over G
  const bool local = jobs[0]->dev.local != 0;
  join();  // (a solver without the Newton step above)
  if (fused) {  // next iteration's promolecule, gradient and Hessian
    ProfScope ps(ctx, HP_KERNEL_GLISA_PRO);
    launch_glisa_fused_ff(hb, st, 1, fuse_shells, !overlap);
  }
  if (overlap) {
    cudaEventRecord(ctx->fork_ev, st);
    cudaStreamWaitEvent(ctx->side, ctx->fork_ev, 0);
    launch_glisa_point_ff(hb, ctx->side);
    launch_outer_finish(hb, ctx->side, 0);
    cudaEventRecord(ctx->join_ev, ctx->side);
    pending = true;
    continue;  // the change is formed in k_outer_finish (Gram blocks)
  }
  if (local) {
    ProfScope ps(ctx, HP_KERNEL_CHANGE);
    launch_change_radial(hb, st);
  } else if (!fused) {
    ProfScope ps(ctx, HP_KERNEL_CHANGE);
    if (gff) launch_glisa_change_ff(hb, st);
    else launch_glisa_change(hb, st);
  }
  launch_outer_finish(hb, st, 0);
  }  // queued iterations
  join();
  int rc = check_launch();
  if (rc) return rc;
  rc = read_mail(ctx);
  if (rc) return rc;
  std::vector<hp_job*> conv;
  for (hp_job* j : jobs) {
    if (j->done) continue;
    const Mailbox& m = ctx->mail_host[j->slot];
    const int before = j->niter;
    j->niter = m.i[MI_ITER];
    j->change = m.d[MD_CHANGE];
    j->f64_factors = m.i[MI_F64_FACTORS];
    j->evals += 3.0 * (double)j->dev.npoint * (double)j->dev.natom * (double)(j->niter - before);
    if (m.i[MI_ERR]) {
      j->status = status_of(m.i[MI_ERR]);
      g_err = err_text(m.i[MI_ERR]);
      j->done = true;
    } else if (j->change < j->desc.threshold) {
      conv.push_back(j);
    } else if (j->niter >= j->desc.maxiter) {
      j->status = HP_ERR_NOT_CONVERGED;
      g_err = "Not converged!";
      j->done = true;
    }
  }
  if (!conv.empty()) {
    // converged: checks, then at_weights and charges with the final parameters
    // (glisa.py:268-278)
    HostBatch hc;
    rc = build_batch(ctx, conv, hc);
    if (rc) return rc;
    if (solver != SOLVER_SC) launch_glisa_check(hc, st);
    if (gff) {  // G as float-float planes: the promolecule from compensated sums
      launch_glisa_final_ff(hc, st);
    } else {
      launch_promol(hc, st, 0, MODEL_BASIS);
    }
    launch_charges(hc, st);
    rc = check_launch();
    if (rc) return rc;
    rc = read_mail(ctx);
    if (rc) return rc;
    for (hp_job* j : conv) {
      const Mailbox& m = ctx->mail_host[j->slot];
      j->warnings |= (uint32_t)m.i[MI_WARN];
      j->evals += (double)j->dev.npoint * (double)j->dev.natom;
      if (m.i[MI_ERR]) {
        j->status = status_of(m.i[MI_ERR]);
        g_err = err_text(m.i[MI_ERR]);
      }
      j->converged = true;
      j->done = true;
    }
  }
  return HP_OK;
}

int step_group(hp_ctx* ctx, const std::vector<hp_job*>& jobs, int iters) {
  // The pinned staging buffers are reused by every build_batch; each upload
  // is followed by a stream synchronisation before the next one.
  int rc;
  std::vector<hp_job*> fresh;
  for (hp_job* j : jobs)
    if (!j->initialized) fresh.push_back(j);
  if (!fresh.empty()) {
    HostBatch hf;
    rc = build_batch(ctx, fresh, hf);
    if (rc) return rc;
    rc = job_init(ctx, fresh, hf);
    if (rc) return rc;
    HP_CK(cudaStreamSynchronize(ctx->stream));
  }
  HostBatch hb;
  rc = build_batch(ctx, jobs, hb);
  if (rc) return rc;
  if (jobs[0]->desc.scheme == HP_SCHEME_GLISA) return step_glisa(ctx, jobs, hb, iters);
  return step_iterstock(ctx, jobs, hb);
}

// ---------------------------------------------------------------------------
// job creation
// ---------------------------------------------------------------------------

int validate(const hp_job_desc* d) {
  if (!d) return fail(HP_ERR_INVALID, "null descriptor");
  if (d->scheme < 0 || d->scheme > 4) return fail(HP_ERR_INVALID, "unknown scheme");
  if (d->scheme == HP_SCHEME_NLIS && d->precision != HP_PRECISION_FP64)
    return fail(HP_ERR_UNSUPPORTED, "NLIS / GMBIS run in FP64");
  if (d->natom <= 0 || d->npoint <= 0) return fail(HP_ERR_INVALID, "natom and npoint must be positive");
  if (d->npoint > (int64_t)2000000000) return fail(HP_ERR_INVALID, "npoint too large");
  if (!d->coordinates || !d->pseudo_numbers || !d->points || !d->weights || !d->density ||
      !d->shell_offsets || !d->initial_propars)
    return fail(HP_ERR_INVALID, "missing input array");
  if (d->grid_type != 1 && d->grid_type != 2 && d->grid_type != 3)
    return fail(HP_ERR_INVALID, "grid_type must be 1, 2 or 3");
  if (d->grid_type == 1) {
    if (d->scheme == HP_SCHEME_LISA && d->solver != HP_SOLVER_DEFAULT && d->solver != HP_SOLVER_SC)
      return fail(HP_ERR_UNSUPPORTED,
                  "grid_type 1 (atom grids) for aLISA is available with the sc solver");
    if (!d->radial_offsets || !d->shell_point_offsets || !d->point_sphere_weights ||
        !d->radial_points || !d->radial_weights || d->nrad <= 0)
      return fail(HP_ERR_INVALID, "grid_type 1 needs the atom-grid arrays");
    if (d->radial_offsets[0] != 0 || d->radial_offsets[d->natom] != d->nrad)
      return fail(HP_ERR_INVALID, "radial_offsets must run from 0 to nrad");
    for (int64_t a = 0; a < d->natom; ++a) {
      const int n = d->radial_offsets[a + 1] - d->radial_offsets[a];
      if (n <= 0 || n > 1024) return fail(HP_ERR_INVALID, "every atom needs 1 to 1024 radial nodes");
    }
    if (d->shell_point_offsets[0] != 0 || d->shell_point_offsets[d->nrad] != d->npoint)
      return fail(HP_ERR_INVALID, "shell_point_offsets must run from 0 to npoint");
    for (int64_t k = 0; k < d->nrad; ++k)
      if (d->shell_point_offsets[k + 1] < d->shell_point_offsets[k])
        return fail(HP_ERR_INVALID, "shell_point_offsets must not decrease");
  }
  const bool slater_like = d->scheme == HP_SCHEME_MBIS || d->scheme == HP_SCHEME_NLIS;
  if (!slater_like && (!d->shell_orders || !d->shell_exponents))
    return fail(HP_ERR_INVALID, "basis schemes need shell orders and exponents");
  if (d->shell_offsets[0] != 0) return fail(HP_ERR_INVALID, "shell_offsets[0] must be 0");
  for (int64_t a = 0; a < d->natom; ++a) {
    const int n = d->shell_offsets[a + 1] - d->shell_offsets[a];
    if (n <= 0) return fail(HP_ERR_INVALID, "every atom needs at least one shell");
    if (slater_like && n > 7) return fail(HP_ERR_INVALID, "MBIS / NLIS allow at most 7 shells");
    if (n > kMaxShells) return fail(HP_ERR_UNSUPPORTED, "at most 16 shells per atom");
  }
  if (d->maxiter <= 0) return fail(HP_ERR_INVALID, "maxiter must be positive");
  if (d->scheme == HP_SCHEME_LISA &&
      (d->solver != HP_SOLVER_SC && d->solver != HP_SOLVER_NEWTON && d->solver != HP_SOLVER_M_NEWTON &&
       d->solver != HP_SOLVER_QUASI_NEWTON && d->solver != HP_SOLVER_DEFAULT))
    return fail(HP_ERR_UNSUPPORTED, "aLISA solvers on this path: sc, newton, m-newton, quasi-newton");
  if (d->scheme != HP_SCHEME_LISA && d->solver == HP_SOLVER_QUASI_NEWTON)
    return fail(HP_ERR_UNSUPPORTED, "the device quasi-Newton solver is for aLISA");
  if (d->scheme == HP_SCHEME_GLISA &&
      (d->solver != HP_SOLVER_SC && d->solver != HP_SOLVER_NEWTON && d->solver != HP_SOLVER_M_NEWTON &&
       d->solver != HP_SOLVER_PNEWTON && d->solver != HP_SOLVER_DEFAULT))
    return fail(HP_ERR_UNSUPPORTED, "gLISA solvers on this path: newton, m-newton, sc, pnewton");
  if (d->scheme != HP_SCHEME_GLISA && d->solver == HP_SOLVER_PNEWTON)
    return fail(HP_ERR_UNSUPPORTED, "the projected Newton solver is for gLISA");
  if (d->linspace_size > 64 || (d->scheme == HP_SCHEME_LISA && d->linspace_size > 32))
    return fail(HP_ERR_UNSUPPORTED, "linspace_size too large");
  if (d->precision == HP_PRECISION_FF && d->scheme != HP_SCHEME_MBIS)
    return fail(HP_ERR_UNSUPPORTED, "float-float evaluation is available for MBIS");
  if (d->precision != HP_PRECISION_FP64 && d->precision != HP_PRECISION_MIXED &&
      d->precision != HP_PRECISION_FF)
    return fail(HP_ERR_INVALID, "unknown precision");
  if (d->precision == HP_PRECISION_MIXED && d->scheme == HP_SCHEME_LISA &&
      d->solver != HP_SOLVER_SC && d->solver != HP_SOLVER_DEFAULT)
    return fail(HP_ERR_UNSUPPORTED, "mixed precision is available for MBIS, GISA, aLISA sc and gLISA");
  if (d->precision == HP_PRECISION_MIXED && d->scheme == HP_SCHEME_GLISA &&
      d->solver == HP_SOLVER_SC)
    return fail(HP_ERR_UNSUPPORTED,
                "mixed precision for gLISA is the tensor-core Hessian of the Newton solvers");
  for (int64_t s = 0; !slater_like && s < d->shell_offsets[d->natom]; ++s) {
    if (!(d->shell_orders[s] > 0.0)) return fail(HP_ERR_INVALID, "n must be positive");
    if (d->shell_exponents[s] < 0.0) return fail(HP_ERR_INVALID, "alpha must be non-negative");
  }
  return HP_OK;
}

// Solver iterations queued per host round trip when running a job to the
// end: gLISA Newton converges quadratically, so near the threshold two
// iterations are queued, further away four (the iterations queued after the
// last one cost a few empty launches each).
int run_chunk(const hp_job* j) {
  if (j->desc.scheme != HP_SCHEME_GLISA) return 1;
  if (j->niter > 0 && j->change < 1e3 * j->desc.threshold) return 2;
  return 4;
}

}  // namespace

extern "C" {

int32_t hp_abi_version(void) { return HPGPU_ABI_VERSION; }

const char* hp_last_error(void) { return g_err.c_str(); }

int32_t hp_ctx_create(int32_t device, size_t hbm_budget, void* stream, hp_ctx** out) {
  if (!out) return fail(HP_ERR_INVALID, "null output pointer");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return fail(HP_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
  if (device < 0 || device >= ndev) return fail(HP_ERR_INVALID, "device index out of range");
  HP_CK(cudaSetDevice(device));
  cudaDeviceProp prop;
  HP_CK(cudaGetDeviceProperties(&prop, device));
  if (prop.major * 10 + prop.minor != 103)
    return fail(HP_ERR_CUDA, "libhpgpu is built for sm_103 (GB300) only");
  hp_ctx* c = new hp_ctx();
  c->device = device;
  if (stream) {
    c->stream = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete c;
      return fail(HP_ERR_CUDA, "cudaStreamCreate failed");
    }
    c->own_stream = true;
  }
  {
    cudaMemPoolProps pp{};
    pp.allocType = cudaMemAllocationTypePinned;
    pp.location.type = cudaMemLocationTypeDevice;
    pp.location.id = device;
    uint64_t keep = UINT64_MAX;
    if (cudaMemPoolCreate(&c->pool, &pp) != cudaSuccess ||
        cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) {
      cudaGetLastError();
      hp_ctx_destroy(c);
      return fail(HP_ERR_CUDA, "device memory pool creation failed");
    }
  }
  if (cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->join_ev, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    hp_ctx_destroy(c);
    return fail(HP_ERR_CUDA, "side stream creation failed");
  }
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  c->budget = hbm_budget ? hbm_budget : (size_t)(0.9 * (double)fr);
  c->slots.assign(kMaxSlots, nullptr);
  if (cudaMalloc(&c->mail_dev, sizeof(Mailbox) * kMaxSlots) != cudaSuccess ||
      cudaMallocHost(&c->mail_host, sizeof(Mailbox) * kMaxSlots) != cudaSuccess ||
      cudaMalloc(&c->batch_dev, sizeof(JobDev) * kMaxSlots) != cudaSuccess ||
      cudaMallocHost(&c->batch_host, sizeof(JobDev) * kMaxSlots) != cudaSuccess ||
      cudaMalloc(&c->prefix_dev, sizeof(int) * K_NKIND * (kMaxSlots + 1)) != cudaSuccess ||
      cudaMallocHost(&c->prefix_host, sizeof(int) * K_NKIND * (kMaxSlots + 1)) != cudaSuccess) {
    hp_ctx_destroy(c);
    return fail(HP_ERR_NO_MEMORY, "context allocation failed");
  }
  cudaMemsetAsync(c->mail_dev, 0, sizeof(Mailbox) * kMaxSlots, c->stream);
  memset(c->mail_host, 0, sizeof(Mailbox) * kMaxSlots);
  *out = c;
  return HP_OK;
}

int32_t hp_ctx_destroy(hp_ctx* c) {
  if (!c) return HP_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (hp_job* j : c->slots)
    if (j) hp_job_destroy(j);
  if (c->mail_dev) cudaFree(c->mail_dev);
  if (c->mail_host) cudaFreeHost(c->mail_host);
  if (c->batch_dev) cudaFree(c->batch_dev);
  if (c->batch_host) cudaFreeHost(c->batch_host);
  if (c->prefix_dev) cudaFree(c->prefix_dev);
  if (c->prefix_host) cudaFreeHost(c->prefix_host);
  prof_collect(c);
  for (cudaEvent_t e : c->event_pool) cudaEventDestroy(e);
  if (c->pool) {
    if (c->stream) cudaStreamSynchronize(c->stream);  // the jobs' frees have run
    cudaMemPoolDestroy(c->pool);
  }
  if (c->side) {
    cudaStreamSynchronize(c->side);
    cudaStreamDestroy(c->side);
  }
  if (c->fork_ev) cudaEventDestroy(c->fork_ev);
  if (c->join_ev) cudaEventDestroy(c->join_ev);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return HP_OK;
}

int32_t hp_ctx_synchronize(hp_ctx* c) {
  if (!c) return fail(HP_ERR_INVALID, "null context");
  HP_CK(cudaStreamSynchronize(c->stream));
  return HP_OK;
}

int32_t hp_ctx_memory(hp_ctx* c, size_t* used, size_t* budget) {
  if (!c) return fail(HP_ERR_INVALID, "null context");
  if (used) *used = c->used;
  if (budget) *budget = c->budget;
  return HP_OK;
}

int32_t hp_job_create(hp_ctx* ctx, const hp_job_desc* d, hp_job** out) {
  if (!ctx || !out) return fail(HP_ERR_INVALID, "null context or output pointer");
  *out = nullptr;
  int rc = validate(d);
  if (rc) return rc;
  HP_CK(cudaSetDevice(ctx->device));
  int slot = -1;
  for (int s = 0; s < kMaxSlots; ++s)
    if (!ctx->slots[s]) {
      slot = s;
      break;
    }
  if (slot < 0) return fail(HP_ERR_NO_MEMORY, "too many live jobs in this context");

  const int A = (int)d->natom;
  const int N = (int)d->npoint;
  const int S = d->shell_offsets[A];
  const bool mbis = d->scheme == HP_SCHEME_MBIS;
  const bool nlis = d->scheme == HP_SCHEME_NLIS;  // (N, S, n) per shell
  const bool glisa = d->scheme == HP_SCHEME_GLISA;
  const int P = mbis ? 2 * S : nlis ? 3 * S : S;
  int kmax = 1;
  for (int a = 0; a < A; ++a) kmax = std::max(kmax, d->shell_offsets[a + 1] - d->shell_offsets[a]);
  int solver = d->solver;
  if (solver == HP_SOLVER_DEFAULT) {
    if (d->scheme == HP_SCHEME_LISA) solver = HP_SOLVER_SC;
    else if (glisa) solver = HP_SOLVER_NEWTON;
    else if (d->scheme == HP_SCHEME_GISA) solver = HP_SOLVER_QP;
  }
  // tiles: aim for >= 2 * 152 point tiles when the grid is large enough
  // (mixed precision: at least 4 points per thread so the per-block
  // compensated reductions are amortised)
  const int ppt_min = d->precision != HP_PRECISION_FP64 && !glisa ? 4 : 2;
  // gLISA's passes over G keep one point tile per block: aim for 4 blocks per SM
  const int64_t tiles_target = glisa ? 4 * 152 : 2 * 152;
  int ppt = (int)std::min<int64_t>(
      64, std::max<int64_t>(ppt_min, (N + kThreads * tiles_target - 1) / (kThreads * tiles_target)));
  const int tile_points = kThreads * ppt;
  const int ntile = (N + tile_points - 1) / tile_points;
  int qa = 2 + std::max(2 * 7 + 1, kMaxShells + 1);
  if (d->scheme == HP_SCHEME_LISA && solver != HP_SOLVER_SC) qa = 2 + kNewtonQ(kmax);
  const int maxiter = d->maxiter;
  // gLISA keeps FP64 evaluation; its mixed mode is the tensor-core Hessian
  // FP32 / float-float buffers (mixed precision and ff)
  const bool mixed = d->precision != HP_PRECISION_FP64 && !glisa;
  const bool tc = d->precision == HP_PRECISION_MIXED && glisa;
  // gLISA with the tensor-core Hessian (Newton or projected Newton): G as
  // float-float planes, no FP64 copy
  const bool gff = tc && solver != HP_SOLVER_M_NEWTON && S <= kGffMaxShells;
  // float hi/lo coordinates: FP32 / float-float evaluation and the FF basis
  const bool hilo = mixed || gff;
  const int htiles = glisa ? (S + kHessTile - 1) / kHessTile : 0;
  const int npair = htiles * (htiles + 1) / 2;
  int nsplit = glisa ? std::max(1, std::min(1024, (4 * 152 + npair - 1) / std::max(1, npair))) : 0;
  if (glisa) nsplit = std::max(1, std::min(nsplit, (N + 255) / 256));
  if (tc) {
    // one 256-thread CTA per SM (two 97 KB shared-memory stages)
    JobDev probe{};
    probe.nshell = S;
    probe.nsplit = 1;
    const int tiles = tc_hess_blocks(probe);
    nsplit = std::max(1, std::min((152 + tiles - 1) / tiles, (N + 255) / 256));
  }
  // fused jobs form the Hessian inside the fused pass: one partial per block
  const bool fuse_job = tc && solver != HP_SOLVER_M_NEWTON && S <= kGffMaxShells && S <= kFuseMaxShells;
  if (fuse_job) nsplit = std::min(ntile, kFuseCtas);

  // carve one allocation
  struct Part { void** dst; size_t bytes; };
  std::vector<Part> parts;
  JobDev J{};
  auto add = [&](void* dst, size_t bytes) { parts.push_back({(void**)dst, bytes}); };
  add(&J.px, 8 * (size_t)N); add(&J.py, 8 * (size_t)N); add(&J.pz, 8 * (size_t)N);
  add(&J.w, 8 * (size_t)N); add(&J.rho, 8 * (size_t)N);
  if (hilo) {
    add(&J.pxh, 4 * (size_t)N); add(&J.pxl, 4 * (size_t)N);
    add(&J.pyh, 4 * (size_t)N); add(&J.pyl, 4 * (size_t)N);
    add(&J.pzh, 4 * (size_t)N); add(&J.pzl, 4 * (size_t)N);
    add(&J.atf, 4 * 6 * (size_t)A);
    add(&J.fpar, 4 * 4 * (size_t)S);
  }
  if (mixed) {
    add(&J.wf, 4 * (size_t)N); add(&J.rhof, 4 * (size_t)N); add(&J.promolf, 4 * (size_t)N);
    add(&J.wl, 4 * (size_t)N); add(&J.rhol, 4 * (size_t)N);
    add(&J.shf, 4 * 3 * (size_t)S);
    add(&J.fco, 4 * 8 * (size_t)S);
    add(&J.rdist, 8 * (size_t)A * N);
  }
  // GISA: per-atom QP matrices, precomputed once (they depend only on exponents)
  int qp_total = 0;
  std::vector<int> qp_off_h((size_t)A + 1, 0);
  for (int a = 0; a < A; ++a) {
    const int n = d->shell_offsets[a + 1] - d->shell_offsets[a];
    qp_off_h[a + 1] = qp_off_h[a] + n * n;
  }
  qp_total = qp_off_h[A];
  if (d->scheme == HP_SCHEME_GISA) {
    add(&J.qp_p, 8 * (size_t)qp_total);
    add(&J.qp_off, 4 * (size_t)(A + 1));
  }
  add(&J.ax, 8 * (size_t)A); add(&J.ay, 8 * (size_t)A); add(&J.az, 8 * (size_t)A);
  add(&J.zpseudo, 8 * (size_t)A);
  add(&J.shell_off, 4 * (size_t)(A + 1)); add(&J.par_off, 4 * (size_t)(A + 1));
  add(&J.sh_order, 8 * (size_t)S); add(&J.sh_alpha, 8 * (size_t)S); add(&J.sh_pref, 8 * (size_t)S);
  add(&J.propars, 8 * (size_t)P); add(&J.propars_init, 8 * (size_t)P);
  add(&J.propars_old, 8 * (size_t)P); add(&J.cur, 8 * (size_t)P);
  add(&J.prev, 8 * (size_t)P); add(&J.delta, 8 * (size_t)P); add(&J.keep, 8 * (size_t)P);
  if (d->solver == HP_SOLVER_QUASI_NEWTON) {
    add(&J.hinv, 8 * (size_t)A * kMaxShells * kMaxShells);
    add(&J.olddf, 8 * (size_t)P);
    add(&J.step, 8 * (size_t)P);
  }
  add(&J.promol, 8 * (size_t)N);
  add(&J.invpro, 8 * (size_t)N);
  add(&J.rhoa, 8 * (size_t)A * N);
  add(&J.apart, 8 * (size_t)A * qa * ntile);
  add(&J.jpart, 8 * (size_t)QJ_COUNT * ntile);
  add(&J.atom_out, 8 * (size_t)A * AO_COUNT);
  add(&J.active, 4 * (size_t)A); add(&J.inner_it, 4 * (size_t)A);
  add(&J.ls_fail, 8 * (size_t)A * ntile);
  // GISA / aLISA in FP64 keep the (fixed) unit-population shells on the device
  // when the matrix takes at most half of the remaining budget: every pass
  // then reads G instead of recomputing exponentials (gLISA always does).
  const size_t gbytes = 8 * (size_t)S * N;
  const size_t room = ctx->budget > ctx->used ? ctx->budget - ctx->used : 0;
  if (!glisa && !mbis && !nlis && !mixed && gbytes <= room / 2) add(&J.gmat, gbytes);
  if (glisa) {
    if (!gff) add(&J.gmat, 8 * (size_t)S * N);
    add(&J.gpart, 8 * (size_t)S * ntile);
    add(&J.hpart, 8 * (size_t)nsplit * S * S);
    add(&J.hess, 8 * (size_t)S * S);
    add(&J.chol, 8 * (size_t)S * S);
    add(&J.grad, 8 * (size_t)S);
    add(&J.dvec1, 8 * (size_t)N); add(&J.dvec2, 8 * (size_t)N);
    add(&J.ctrial, 8 * (size_t)kTrials * S);
    add(&J.tpart, 8 * 2 * (size_t)kTrials * ntile);  // per trial: difference, then the magnitude of its FP32 terms
    add(&J.freeidx, 4 * (size_t)(S + 2));
    add(&J.clip, 4 * (size_t)(2 * S + 1));
    add(&J.rho0, 8 * (size_t)N);
    if (tc) {
      add(&J.hsum, 8 * (size_t)S);
      add(&J.gmat32, 4 * (size_t)S * N);
      add(&J.hess_s, 4 * (size_t)N);
      if (gff) {
        add(&J.gmat_lo, 4 * (size_t)S * N);
        add(&J.clipf, 4 * 4 * (size_t)S);
        if (S <= kFuseMaxShells) {
          add(&J.gact, 4 * (size_t)(S + 1) * ntile);
          add(&J.wrf, 16 * (size_t)N);
          add(&J.r0f, 8 * (size_t)N);
          add(&J.d2f, 8 * (size_t)N);
          add(&J.r0t, 8 * (size_t)kTrials * N);
        }
        add(&J.d1f, 8 * (size_t)N);
        add(&J.hvf, 8 * (size_t)N);
      } else {
        add(&J.hvec, 8 * (size_t)N);
      }
    }
  }
  const bool local = d->grid_type == 1;
  const int nrad = local ? d->nrad : 0;
  // fused jobs on the molecular grid: per-atom Gram blocks for the change
  std::vector<int> wgoff_h;
  if (fuse_job && !local) {
    wgoff_h.assign((size_t)A + 1, 0);
    for (int a = 0; a < A; ++a) {
      const int k = d->shell_offsets[a + 1] - d->shell_offsets[a];
      wgoff_h[a + 1] = wgoff_h[a] + k * (k + 1) / 2;
    }
    add(&J.wgoff, 4 * (size_t)(A + 1));
    add(&J.wgram, 8 * (size_t)std::max(1, wgoff_h[A]));
    J.wgn = wgoff_h[A];
  }
  if (local) {
    add(&J.rad_off, 4 * (size_t)(A + 1));
    add(&J.shell_pt, 8 * (size_t)(nrad + 1));
    add(&J.wsph, 8 * (size_t)N);
    add(&J.rad_r, 8 * (size_t)nrad);
    add(&J.rad_w, 8 * (size_t)nrad);
    add(&J.radrho, 8 * (size_t)nrad);
  }
  // per-atom cutoff of the MBIS / aLISA sc inner solve and outer change
  // (molecular grid)
  const bool cutoff = (mbis || (d->scheme == HP_SCHEME_LISA && solver == HP_SOLVER_SC)) &&
                      d->grid_type != 1;
  if (cutoff) {
    add(&J.tgeo, 8 * 5 * (size_t)ntile);
    add(&J.amax, 4 * (size_t)A * ntile);
  }
  add(&J.hist_propars, 8 * (size_t)maxiter * P);
  add(&J.hist_charges, 8 * (size_t)maxiter * A);
  add(&J.hist_ent, 8 * (size_t)maxiter); add(&J.hist_chg, 8 * (size_t)maxiter);
  add(&J.charges, 8 * (size_t)A);
  size_t total = 0;
  for (auto& p : parts) total += align_up(p.bytes);
  if (ctx->used + total > ctx->budget)
    return fail(HP_ERR_NO_MEMORY, "job needs " + std::to_string(total) + " bytes; HBM budget exceeded");
  void* mem = nullptr;
  if (job_alloc(ctx, &mem, total) != cudaSuccess) {
    cudaGetLastError();
    return fail(HP_ERR_NO_MEMORY, "device allocation of " + std::to_string(total) + " bytes failed");
  }
  char* cur = (char*)mem;
  for (auto& p : parts) {
    *p.dst = cur;
    cur += align_up(p.bytes);
  }
  J.mail = ctx->mail_dev + slot;
  J.natom = A; J.npoint = N; J.ntile = ntile; J.nparam = P; J.nshell = S; J.qa = qa;
  J.scheme = d->scheme; J.solver = solver; J.maxiter = maxiter;
  J.mixed = !mixed ? PH_FP64 : d->precision == HP_PRECISION_FF ? PH_FF : PH_FP32;
  J.inner_maxiter = d->inner_maxiter > 0 ? d->inner_maxiter : 2000;
  J.linspace_size = d->linspace_size > 0 ? d->linspace_size : (glisa ? 40 : 20);
  J.nsplit = nsplit; J.ppt = ppt; J.tile_points = tile_points; J.htiles = htiles;
  J.tc = tc ? 1 : 0;
  J.gff = gff ? 1 : 0;
  J.fuse = gff && S <= kFuseMaxShells ? 1 : 0;
  J.refine = tc && d->polish ? 1 : 0;
  J.local = local ? 1 : 0;
  J.nrad = nrad;
  J.threshold = d->threshold;
  J.inner_threshold = d->inner_threshold < d->threshold ? d->inner_threshold : d->threshold;
  J.density_cutoff = d->density_cutoff; J.negative_cutoff = d->negative_cutoff;
  J.population_cutoff = d->population_cutoff; J.tau = d->tau;

  hp_job* job = new hp_job();
  job->ctx = ctx;
  job->slot = slot;
  job->desc = *d;
  job->desc.solver = solver;
  job->mem = mem;
  job->bytes = total;
  job->dev = J;

  // host staging: SoA grid, float hi/lo, atoms, shells
  cudaStream_t st = ctx->stream;
  auto up = [&](const void* dst, const void* src, size_t bytes) {
    return cudaMemcpyAsync((void*)dst, src, bytes, cudaMemcpyHostToDevice, st);
  };
  // every work array starts at zero, as in a fresh allocation: a job's results
  // never depend on what an earlier job left in recycled device memory. The
  // float-float planes of G are left out: k_glisa_basis_ff writes every
  // element of them before anything reads them (they are most of a gLISA
  // job's memory)
  bool ok = true;
  {
    std::vector<std::pair<char*, char*>> skip;
    auto plane = [&](const float* q) {
      if (q) skip.push_back({(char*)q, (char*)q + align_up(4 * (size_t)S * N)});
    };
    if (J.gmat_lo) {  // the float-float planes exist only together
      plane(J.gmat32);
      plane(J.gmat_lo);
    }
    std::sort(skip.begin(), skip.end());
    char* at = (char*)mem;
    for (const auto& r : skip) {
      if (r.first > at) ok &= cudaMemsetAsync(at, 0, (size_t)(r.first - at), st) == cudaSuccess;
      at = std::max(at, r.second);
    }
    char* end = (char*)mem + total;
    if (end > at) ok &= cudaMemsetAsync(at, 0, (size_t)(end - at), st) == cudaSuccess;
  }
  // the points as the caller holds them, (N, 3), split on the device
  // (k_stage_points, after w and rho are in place)
  void* ptmp = nullptr;
  ok &= job_alloc(ctx, &ptmp, 24 * (size_t)std::max(N, 1)) == cudaSuccess;
  if (ok) ok &= up(ptmp, d->points, 24 * (size_t)N) == cudaSuccess;
  ok &= up(J.w, d->weights, 8 * (size_t)N) == cudaSuccess;
  std::vector<double> tgeo;
  if (cutoff) {
    // per tile: bounding-box centre, the largest distance of its points from
    // it, and the sum of its weights
    tgeo.assign(5 * (size_t)ntile, 0.0);
    for (int t = 0; t < ntile; ++t) {
      const int64_t p0 = (int64_t)t * tile_points, p1 = std::min<int64_t>(p0 + tile_points, N);
      double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300}, wsum = 0.0;
      for (int64_t p = p0; p < p1; ++p) {
        for (int c = 0; c < 3; ++c) {
          lo[c] = std::min(lo[c], d->points[3 * p + c]);
          hi[c] = std::max(hi[c], d->points[3 * p + c]);
        }
        wsum += std::fabs(d->weights[p]);
      }
      double* g = tgeo.data() + 5 * (size_t)t;
      for (int c = 0; c < 3; ++c) g[c] = 0.5 * (lo[c] + hi[c]);
      double r2 = 0.0;
      for (int64_t p = p0; p < p1; ++p) {
        double e = 0.0;
        for (int c = 0; c < 3; ++c) e += (d->points[3 * p + c] - g[c]) * (d->points[3 * p + c] - g[c]);
        r2 = std::max(r2, e);
      }
      g[3] = std::sqrt(r2) * (1.0 + 1e-12) + 1e-12;  // rounding margin
      g[4] = wsum;
    }
    ok &= up(J.tgeo, tgeo.data(), 8 * 5 * (size_t)ntile) == cudaSuccess;
    ok &= cudaMemsetAsync(J.amax, 0x7f, 4 * (size_t)A * ntile, st) == cudaSuccess;  // large: no skip before the first at_weights pass
  }
  ok &= up(J.rho, d->density, 8 * (size_t)N) == cudaSuccess;
  if (local) {
    ok &= up(J.rad_off, d->radial_offsets, 4 * (size_t)(A + 1)) == cudaSuccess;
    ok &= up(J.shell_pt, d->shell_point_offsets, 8 * (size_t)(nrad + 1)) == cudaSuccess;
    ok &= up(J.wsph, d->point_sphere_weights, 8 * (size_t)N) == cudaSuccess;
    ok &= up(J.rad_r, d->radial_points, 8 * (size_t)nrad) == cudaSuccess;
    ok &= up(J.rad_w, d->radial_weights, 8 * (size_t)nrad) == cudaSuccess;
  }
  if (ok) {
    StageArgs sa{};
    sa.pts = static_cast<const double*>(ptmp);
    sa.n = N;
    // the job's arrays are read-only to the kernels that use them; this is
    // where they are written
    auto wd = [](const double* q) { return const_cast<double*>(q); };
    auto wfl = [](const float* q) { return const_cast<float*>(q); };
    sa.xyz[0] = wd(J.px); sa.xyz[1] = wd(J.py); sa.xyz[2] = wd(J.pz);
    if (hilo) {
      sa.hi[0] = wfl(J.pxh); sa.hi[1] = wfl(J.pyh); sa.hi[2] = wfl(J.pzh);
      sa.lo[0] = wfl(J.pxl); sa.lo[1] = wfl(J.pyl); sa.lo[2] = wfl(J.pzl);
    }
    sa.w = J.w;
    sa.rho = J.rho;
    if (mixed) {
      sa.wf = wfl(J.wf); sa.wl = wfl(J.wl);
      sa.rf = wfl(J.rhof); sa.rl = wfl(J.rhol);
    }
    launch_stage_points(sa, st);
    ok &= cudaGetLastError() == cudaSuccess;
  }
  job_free(ctx, ptmp);
  std::vector<double> ac((size_t)A);
  for (int c = 0; c < 3 && ok; ++c) {
    for (int a = 0; a < A; ++a) ac[a] = d->coordinates[(size_t)3 * a + c];
    ok &= up(c == 0 ? J.ax : c == 1 ? J.ay : J.az, ac.data(), 8 * (size_t)A) == cudaSuccess;
  }
  ok &= up(J.zpseudo, d->pseudo_numbers, 8 * (size_t)A) == cudaSuccess;
  std::vector<float> atf32;
  if (hilo) {
    atf32.resize(6 * (size_t)A);
    for (int a = 0; a < A; ++a)
      for (int c = 0; c < 3; ++c) {
        const double x = d->coordinates[(size_t)3 * a + c];
        const float h = (float)x;
        atf32[6 * a + 2 * c] = h;
        atf32[6 * a + 2 * c + 1] = (float)(x - (double)h);
      }
    ok &= up(J.atf, atf32.data(), 4 * 6 * (size_t)A) == cudaSuccess;
  }
  std::vector<double> qp_h;
  if (d->scheme == HP_SCHEME_GISA) {
    // P_kl = 2 / pi^1.5 (a_k a_l)^1.5 / (a_k + a_l)^1.5, symmetrised (gisa.py:387-393)
    qp_h.resize((size_t)qp_total);
    for (int a = 0; a < A; ++a) {
      const int s0 = d->shell_offsets[a], n = d->shell_offsets[a + 1] - s0;
      double* P = qp_h.data() + qp_off_h[a];
      for (int k = 0; k < n; ++k)
        for (int l = 0; l < n; ++l) {
          const double ak = d->shell_exponents[s0 + k], al = d->shell_exponents[s0 + l];
          P[k * n + l] = 2.0 / std::pow(M_PI, 1.5) * std::pow(ak * al, 1.5) / std::pow(ak + al, 1.5);
        }
      for (int k = 0; k < n; ++k)
        for (int l = 0; l < k; ++l) {
          const double v = 0.5 * (P[k * n + l] + P[l * n + k]);
          P[k * n + l] = v;
          P[l * n + k] = v;
        }
    }
    ok &= up(J.qp_p, qp_h.data(), 8 * (size_t)qp_total) == cudaSuccess;
    ok &= up(J.qp_off, qp_off_h.data(), 4 * (size_t)(A + 1)) == cudaSuccess;
  }
  ok &= up(J.shell_off, d->shell_offsets, 4 * (size_t)(A + 1)) == cudaSuccess;
  std::vector<int> poff((size_t)A + 1);
  for (int a = 0; a <= A; ++a)
    poff[a] = mbis ? 2 * d->shell_offsets[a] : nlis ? 3 * d->shell_offsets[a] : d->shell_offsets[a];
  ok &= up(J.par_off, poff.data(), 4 * (size_t)(A + 1)) == cudaSuccess;
  std::vector<double> ord((size_t)S, 1.0), alp((size_t)S, 0.0), pref((size_t)S, 0.0);
  if (!mbis && !nlis) {
    for (int s = 0; s < S; ++s) {
      ord[s] = d->shell_orders[s];
      alp[s] = d->shell_exponents[s];
      pref[s] = ord[s] * std::pow(alp[s], 3.0 / ord[s]) / (4.0 * M_PI * std::tgamma(3.0 / ord[s]));
    }
  }
  ok &= up(J.sh_order, ord.data(), 8 * (size_t)S) == cudaSuccess;
  ok &= up(J.sh_alpha, alp.data(), 8 * (size_t)S) == cudaSuccess;
  ok &= up(J.sh_pref, pref.data(), 8 * (size_t)S) == cudaSuccess;
  std::vector<float> shf32;
  if (mixed) {
    shf32.resize(3 * (size_t)S);
    for (int s = 0; s < S; ++s) {
      shf32[3 * s] = (float)ord[s];
      shf32[3 * s + 1] = (float)alp[s];
      shf32[3 * s + 2] = (float)pref[s];
    }
    ok &= up(J.shf, shf32.data(), 4 * 3 * (size_t)S) == cudaSuccess;
  }
  std::vector<float> fpar32;
  if (gff) {  // (pref hi, pref lo, alpha hi, alpha lo) per shell for the FF basis
    fpar32.resize(4 * (size_t)S);
    for (int s = 0; s < S; ++s) {
      fpar32[4 * s] = (float)pref[s];
      fpar32[4 * s + 1] = (float)(pref[s] - (double)fpar32[4 * s]);
      fpar32[4 * s + 2] = (float)alp[s];
      fpar32[4 * s + 3] = (float)(alp[s] - (double)fpar32[4 * s + 2]);
    }
    ok &= up(J.fpar, fpar32.data(), 4 * 4 * (size_t)S) == cudaSuccess;
  }
  if (J.wgoff) ok &= up(J.wgoff, wgoff_h.data(), 4 * wgoff_h.size()) == cudaSuccess;
  ok &= up(J.propars, d->initial_propars, 8 * (size_t)P) == cudaSuccess;
  ok &= up(J.propars_init, d->initial_propars, 8 * (size_t)P) == cudaSuccess;
  ok &= cudaMemsetAsync(J.apart, 0, 8 * (size_t)A * qa * ntile, st) == cudaSuccess;
  ok &= cudaMemsetAsync(J.atom_out, 0, 8 * (size_t)A * AO_COUNT, st) == cudaSuccess;
  ok &= cudaMemsetAsync(J.charges, 0, 8 * (size_t)A, st) == cudaSuccess;

  ok &= cudaMemsetAsync(ctx->mail_dev + slot, 0, sizeof(Mailbox), st) == cudaSuccess;
  ok &= cudaStreamSynchronize(st) == cudaSuccess;
  if (!ok) {
    job_free(ctx, mem);
    delete job;
    return fail(HP_ERR_CUDA, "upload of job inputs failed");
  }
  memset(&ctx->mail_host[slot], 0, sizeof(Mailbox));
  ctx->slots[slot] = job;
  ctx->slots_hi = std::max(ctx->slots_hi, slot + 1);
  ctx->used += total;
  *out = job;
  return HP_OK;
}

int32_t hp_job_destroy(hp_job* job) {
  if (!job) return HP_OK;
  hp_ctx* ctx = job->ctx;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  job_free(ctx, job->mem);  // back to the context's pool, in stream order
  job_free(ctx, job->pack_mem);
  ctx->used -= job->bytes;
  ctx->slots[job->slot] = nullptr;
  delete job;
  return HP_OK;
}

namespace {
int step_jobs(hp_ctx* ctx, hp_job* const* jobs, int32_t njobs, int iters, int32_t* n_live) {
  if (!ctx || (njobs > 0 && !jobs)) return fail(HP_ERR_INVALID, "null argument");
  if (njobs > kMaxSlots) return fail(HP_ERR_INVALID, "too many jobs in one step");
  HP_CK(cudaSetDevice(ctx->device));
  // group live jobs by (scheme, solver, precision)
  std::vector<std::vector<hp_job*>> groups;
  for (int i = 0; i < njobs; ++i) {
    hp_job* j = jobs[i];
    if (!j || j->ctx != ctx) return fail(HP_ERR_INVALID, "job does not belong to this context");
    if (j->done) continue;
    bool placed = false;
    for (auto& g : groups) {
      const hp_job* h = g[0];
      if (h->desc.scheme == j->desc.scheme && h->dev.solver == j->dev.solver &&
          h->dev.mixed == j->dev.mixed && h->dev.tc == j->dev.tc &&
          h->dev.local == j->dev.local && h->dev.fuse == j->dev.fuse) {
        g.push_back(j);
        placed = true;
        break;
      }
    }
    if (!placed) groups.push_back({j});
  }
  for (auto& g : groups) {
    int rc = step_group(ctx, g, iters);
    if (rc) return rc;
  }
  int live = 0;
  for (int i = 0; i < njobs; ++i)
    if (!jobs[i]->done) ++live;
  if (n_live) *n_live = live;
  return HP_OK;
}
}  // namespace

int32_t hp_step(hp_ctx* ctx, hp_job* const* jobs, int32_t njobs, int32_t* n_live) {
  return step_jobs(ctx, jobs, njobs, 1, n_live);
}

int32_t hp_step_n(hp_ctx* ctx, hp_job* const* jobs, int32_t njobs, int32_t max_iterations,
                  int32_t* n_live) {
  if (max_iterations < 1 || max_iterations > 64)
    return fail(HP_ERR_INVALID, "max_iterations must be 1..64");
  return step_jobs(ctx, jobs, njobs, max_iterations, n_live);
}

int32_t hp_job_run(hp_ctx* ctx, hp_job* job) {
  if (!ctx || !job) return fail(HP_ERR_INVALID, "null argument");
  int32_t live = 1;
  while (!job->done) {
    int rc = step_jobs(ctx, &job, 1, run_chunk(job), &live);
    if (rc) return rc;
  }
  if (job->status != HP_OK) return fail(job->status, g_err.empty() ? "job failed" : g_err);
  return HP_OK;
}

int32_t hp_job_reset(hp_job* job) {
  if (!job) return fail(HP_ERR_INVALID, "null job");
  hp_ctx* ctx = job->ctx;
  HP_CK(cudaSetDevice(ctx->device));
  const JobDev& J = job->dev;
  HP_CK(cudaMemcpyAsync(J.propars, J.propars_init, 8 * (size_t)J.nparam, cudaMemcpyDeviceToDevice,
                        ctx->stream));
  HP_CK(cudaMemsetAsync(ctx->mail_dev + job->slot, 0, sizeof(Mailbox), ctx->stream));
  HP_CK(cudaStreamSynchronize(ctx->stream));
  memset(&ctx->mail_host[job->slot], 0, sizeof(Mailbox));
  job->initialized = false;
  job->done = false;
  job->status = HP_OK;
  job->niter = 0;
  job->change = 0.0;
  job->warnings = 0;
  job->last_inner = 4;
  job->evals = 0.0;
  job->inner_total = 0.0;
  job->converged = false;
  job->prev_change = 1e300;
  job->polish_iters = 0;
  job->f64_factors = 0;
  job->skipped = 0.0;
  job->host_driven = false;
  job->changes.clear();
  if (job->desc.scheme == HP_SCHEME_GLISA || job->desc.precision == HP_PRECISION_FP64)
    job->dev.mixed = PH_FP64;
  else
    job->dev.mixed = job->desc.precision == HP_PRECISION_FF ? PH_FF : PH_FP32;
  return HP_OK;
}

// ---------------------------------------------------------------------------
// evaluation service of the host-driven gLISA solvers
// ---------------------------------------------------------------------------

namespace {

// An FP64 gLISA job on the molecular grid, initialised (basis matrix on the
// device), with its one-job batch in hb.
int eval_ready(hp_job* job, HostBatch& hb) {
  if (!job) return fail(HP_ERR_INVALID, "null job");
  if (job->desc.scheme != HP_SCHEME_GLISA || !job->dev.gmat || job->dev.tc || job->dev.local)
    return fail(HP_ERR_UNSUPPORTED,
                "the host-driven gLISA solvers run on FP64 gLISA jobs on the molecular grid");
  hp_ctx* ctx = job->ctx;
  HP_CK(cudaSetDevice(ctx->device));
  std::vector<hp_job*> one{job};
  int rc = build_batch(ctx, one, hb);
  if (rc) return rc;
  if (!job->initialized) {
    rc = job_init(ctx, one, hb);
    if (rc) return rc;
    HP_CK(cudaStreamSynchronize(ctx->stream));
  }
  return HP_OK;
}

int upload(hp_job* job, double* dst, const double* src) {
  HP_CK(cudaMemcpyAsync(dst, src, 8 * (size_t)job->dev.nparam, cudaMemcpyHostToDevice,
                        job->ctx->stream));
  return HP_OK;
}

}  // namespace

int32_t hp_glisa_evaluate(hp_job* job, const double* x, int32_t nderiv, double* f, double* grad,
                          double* hess, double* pro_pop) {
  if (!x || nderiv < 0 || nderiv > 2) return fail(HP_ERR_INVALID, "bad argument");
  HostBatch hb;
  int rc = eval_ready(job, hb);
  if (rc) return rc;
  hp_ctx* ctx = job->ctx;
  const JobDev& J = job->dev;
  cudaStream_t st = ctx->stream;
  rc = upload(job, J.propars, x);
  if (rc) return rc;
  launch_glisa_pro(hb, st);
  if (nderiv >= 1) launch_glisa_grad(hb, st);
  if (nderiv == 2) launch_glisa_hess(hb, st);
  if (nderiv >= 1) launch_glisa_reduce(hb, st);
  launch_glisa_eval(hb, st, 0);
  rc = check_launch();
  if (rc) return rc;
  rc = read_mail(ctx);
  if (rc) return rc;
  const Mailbox& m = ctx->mail_host[job->slot];
  if (f) *f = m.d[MD_EVAL_A];
  if (pro_pop) *pro_pop = m.d[MD_EVAL_B];
  const size_t S = (size_t)J.nshell;
  if (grad && nderiv >= 1) HP_CK(cudaMemcpy(grad, J.grad, 8 * S, cudaMemcpyDeviceToHost));
  if (hess && nderiv == 2) HP_CK(cudaMemcpy(hess, J.hess, 8 * S * S, cudaMemcpyDeviceToHost));
  job->evals += (double)J.npoint * (double)J.natom;
  return HP_OK;
}

int32_t hp_glisa_change(hp_job* job, const double* x, const double* y, int32_t kind,
                        double* change) {
  if (!x || !y || !change || kind < 0 || kind > 1) return fail(HP_ERR_INVALID, "bad argument");
  HostBatch hb;
  int rc = eval_ready(job, hb);
  if (rc) return rc;
  hp_ctx* ctx = job->ctx;
  const JobDev& J = job->dev;
  cudaStream_t st = ctx->stream;
  if (kind == 0) {  // promolecule difference
    std::vector<double> d((size_t)J.nparam);
    for (int i = 0; i < J.nparam; ++i) d[i] = x[i] - y[i];
    rc = upload(job, J.delta, d.data());
    if (rc) return rc;
    HP_CK(cudaStreamSynchronize(st));  // d leaves scope
    launch_glisa_eval(hb, st, 1);
  } else {  // compute_change: per-atom pro-atom differences
    rc = upload(job, J.propars, x);
    if (!rc) rc = upload(job, J.propars_old, y);
    if (rc) return rc;
    launch_glisa_change(hb, st);
    launch_glisa_eval(hb, st, 2);
  }
  rc = check_launch();
  if (rc) return rc;
  rc = read_mail(ctx);
  if (rc) return rc;
  *change = ctx->mail_host[job->slot].d[MD_EVAL_A];
  job->evals += 2.0 * (double)J.npoint * (double)J.natom;
  return HP_OK;
}

int32_t hp_glisa_line_search(hp_job* job, const double* x, const double* delta, const double* keep,
                             double* step, double* x_out) {
  if (!x || !delta || !keep || !step || !x_out) return fail(HP_ERR_INVALID, "bad argument");
  HostBatch hb;
  int rc = eval_ready(job, hb);
  if (rc) return rc;
  hp_ctx* ctx = job->ctx;
  const JobDev& J = job->dev;
  cudaStream_t st = ctx->stream;
  rc = upload(job, J.propars, x);
  if (!rc) rc = upload(job, J.delta, delta);
  if (!rc) rc = upload(job, J.keep, keep);
  if (rc) return rc;
  launch_glisa_ls(hb, st, 0, std::min(J.linspace_size, 64));
  rc = check_launch();
  if (rc) return rc;
  rc = read_mail(ctx);
  if (rc) return rc;
  *step = ctx->mail_host[job->slot].d[MD_LS_X];
  HP_CK(cudaMemcpy(x_out, J.propars, 8 * (size_t)J.nparam, cudaMemcpyDeviceToHost));
  job->evals += (double)J.npoint * (double)J.natom;
  return HP_OK;
}

int32_t hp_glisa_finish(hp_job* job, const double* x, int32_t niter) {
  if (!x || niter < 0) return fail(HP_ERR_INVALID, "bad argument");
  HostBatch hb;
  int rc = eval_ready(job, hb);
  if (rc) return rc;
  hp_ctx* ctx = job->ctx;
  cudaStream_t st = ctx->stream;
  rc = upload(job, job->dev.propars, x);
  if (rc) return rc;
  launch_glisa_pro(hb, st);  // negativity of the final promolecule
  launch_glisa_check(hb, st);
  launch_promol(hb, st, 0, MODEL_BASIS);  // at_weights and populations (glisa.py:268-278)
  launch_charges(hb, st);
  rc = check_launch();
  if (rc) return rc;
  rc = read_mail(ctx);
  if (rc) return rc;
  const Mailbox& m = ctx->mail_host[job->slot];
  job->warnings |= (uint32_t)m.i[MI_WARN];
  if (m.i[MI_ERR]) {
    job->status = status_of(m.i[MI_ERR]);
    g_err = err_text(m.i[MI_ERR]);
  }
  job->niter = niter;
  job->converged = m.i[MI_ERR] == 0;
  job->done = true;
  job->host_driven = true;
  job->evals += 2.0 * (double)job->dev.npoint * (double)job->dev.natom;
  return job->status == HP_OK ? HP_OK : fail(job->status, g_err);
}

int32_t hp_ctx_profile(hp_ctx* c, int32_t enable) {
  if (!c) return fail(HP_ERR_INVALID, "null context");
  HP_CK(cudaStreamSynchronize(c->stream));
  prof_collect(c);
  c->prof = enable != 0;
  c->launch_base = g_launch_count;
  for (int k = 0; k < HP_KERNEL_COUNT; ++k) {
    c->prof_ms[k] = 0.0;
    c->prof_n[k] = 0;
  }
  return HP_OK;
}

int32_t hp_ctx_profile_get(hp_ctx* c, int32_t family, double* ms, int64_t* launches) {
  if (!c || family < 0 || family > HP_KERNEL_COUNT) return fail(HP_ERR_INVALID, "bad argument");
  HP_CK(cudaStreamSynchronize(c->stream));
  prof_collect(c);
  if (family == HP_KERNEL_COUNT) {  // all kernel launches since profiling was enabled
    if (ms) *ms = 0.0;
    if (launches) *launches = g_launch_count - c->launch_base;
    return HP_OK;
  }
  if (ms) *ms = c->prof_ms[family];
  if (launches) *launches = c->prof_n[family];
  return HP_OK;
}

int32_t hp_job_info_get(hp_job* job, hp_job_info* out) {
  if (!job || !out) return fail(HP_ERR_INVALID, "null argument");
  out->natom = job->dev.natom;
  out->npoint = job->dev.npoint;
  out->nparam = job->dev.nparam;
  out->niter = job->niter;
  out->inner_iterations = (int64_t)job->inner_total;
  out->change = job->change;
  out->done = job->done ? 1 : 0;
  out->status = job->status;
  out->warnings = job->warnings;
  out->converged = job->converged ? 1 : 0;
  out->device_bytes = (int64_t)job->bytes;
  out->point_atom_evals = job->evals;
  out->polish_iterations = job->polish_iters;
  out->f64_factors = job->f64_factors;
  if (job->g_active < 0 && job->initialized && job->dev.fuse && job->dev.gact) {
    // per tile: active-row count at gact[tile][S]; times the tile's points
    const JobDev& J = job->dev;
    std::vector<int> g((size_t)(J.nshell + 1) * J.ntile);
    HP_CK(cudaSetDevice(job->ctx->device));
    HP_CK(cudaStreamSynchronize(job->ctx->stream));
    HP_CK(cudaMemcpy(g.data(), J.gact, sizeof(int) * g.size(), cudaMemcpyDeviceToHost));
    int64_t total = 0;
    for (int t = 0; t < J.ntile; ++t) {
      const int64_t pts = std::min<int64_t>(J.tile_points, (int64_t)J.npoint - (int64_t)t * J.tile_points);
      total += (int64_t)g[(size_t)t * (J.nshell + 1) + J.nshell] * pts;
    }
    job->g_active = total;
  }
  out->g_active_values = job->g_active > 0 ? job->g_active : 0;
  out->point_atom_evals_skipped = job->skipped;
  return HP_OK;
}

int32_t hp_job_results_get(hp_job* job, const hp_job_results* r) {
  if (!job || !r) return fail(HP_ERR_INVALID, "null argument");
  hp_ctx* ctx = job->ctx;
  HP_CK(cudaSetDevice(ctx->device));
  const JobDev& J = job->dev;
  const size_t A = J.natom, N = J.npoint, P = J.nparam;
  const size_t nit = job->host_driven ? 0 : std::min(job->niter, J.maxiter);
  cudaStream_t st = ctx->stream;
  if (r->at_weights) {
    if (!job->done) return fail(HP_ERR_STATE, "at_weights are available once the job is done");
    std::vector<hp_job*> one{job};
    HostBatch hb;
    int rc = build_batch(ctx, one, hb);
    if (rc) return rc;
    const int glisa = job->desc.scheme == HP_SCHEME_GLISA;
    launch_final_atweights(hb, st, glisa ? 0 : J.mixed, model_of(job), glisa ? 0 : 1);
    rc = check_launch();
    if (rc) return rc;
  }
  HP_CK(cudaStreamSynchronize(st));
  if (r->charges) HP_CK(cudaMemcpy(r->charges, J.charges, 8 * A, cudaMemcpyDeviceToHost));
  if (r->propars) HP_CK(cudaMemcpy(r->propars, J.propars, 8 * P, cudaMemcpyDeviceToHost));
  if (r->history_propars && nit)
    HP_CK(cudaMemcpy(r->history_propars, J.hist_propars, 8 * P * nit, cudaMemcpyDeviceToHost));
  if (r->history_charges && nit)
    HP_CK(cudaMemcpy(r->history_charges, J.hist_charges, 8 * A * nit, cudaMemcpyDeviceToHost));
  if (r->history_entropies && nit)
    HP_CK(cudaMemcpy(r->history_entropies, J.hist_ent, 8 * nit, cudaMemcpyDeviceToHost));
  if (r->history_changes && nit)
    HP_CK(cudaMemcpy(r->history_changes, J.hist_chg, 8 * nit, cudaMemcpyDeviceToHost));
  if (r->promoldens) {
    HP_CK(cudaMemcpy(r->promoldens, J.promol, 8 * N, cudaMemcpyDeviceToHost));
    if (J.mixed) {  // float pairs (hi, lo) -> double, plus 1e-100 per atom as the reference
      for (size_t p = 0; p < N; ++p) {
        float pair[2];
        memcpy(pair, &r->promoldens[p], sizeof(pair));
        r->promoldens[p] = (double)pair[0] + (double)pair[1] + 1e-100 * (double)A;
      }
    }
  }
  if (r->at_weights) HP_CK(cudaMemcpy(r->at_weights, J.rhoa, 8 * A * N, cudaMemcpyDeviceToHost));
  return HP_OK;
}

// ---------------------------------------------------------------------------
// Density generator (hp_density.cu)
// ---------------------------------------------------------------------------

struct hp_density_plan {
  hp_ctx* ctx = nullptr;
  DensityArgs args{};
  double* dev = nullptr;                 // centers, amin, exps, coefs, mats
  int* info = nullptr;
  unsigned long long* stats = nullptr;   // [3]
  size_t bytes = 0;
  double* scratch = nullptr;             // host-pointer evaluations: points and out
  size_t scratch_points = 0;
};

int32_t hp_density_plan_create(hp_ctx* ctx, const hp_density_desc* d, hp_density_plan** out) {
  if (!out) return fail(HP_ERR_INVALID, "null output pointer");
  *out = nullptr;
  if (!ctx || !d) return fail(HP_ERR_INVALID, "null argument");
  if (d->nshell < 0 || d->nprim < 0 || d->nbasis < 0 || d->nmat < 1 || !d->mats ||
      (d->nshell > 0 && (!d->centers || !d->shell_info || !d->exponents || !d->coeffs)))
    return fail(HP_ERR_INVALID, "incomplete density description");
  const int ns = d->nshell, nb = d->nbasis;
  std::vector<double> amin(ns, 0.0);
  int nf = 0;
  bool pure2 = false, pure3 = false;
  for (int s = 0; s < ns; ++s) {
    const int* in = d->shell_info + 5 * s;
    const int l = in[0], pure = in[1], np = in[2], k0 = in[3], f0 = in[4];
    if (l < 0 || l > 3) return fail(HP_ERR_UNSUPPORTED, "shells up to f (l <= 3) only");
    if (np < 1 || k0 < 0 || k0 + np > d->nprim) return fail(HP_ERR_INVALID, "shell primitives out of range");
    const int nfs = (pure && l >= 2) ? 2 * l + 1 : (l + 1) * (l + 2) / 2;
    if (f0 != nf) return fail(HP_ERR_INVALID, "shell functions must be consecutive");
    nf += nfs;
    if (pure && l == 2) pure2 = true;
    if (pure && l == 3) pure3 = true;
    double a = INFINITY;
    for (int k = k0; k < k0 + np; ++k) {
      if (!(d->exponents[k] > 0.0)) return fail(HP_ERR_INVALID, "exponents must be positive");
      if (d->coeffs[k] != 0.0) a = std::min(a, d->exponents[k]);
    }
    amin[s] = std::isfinite(a) ? a : 1e300;  // a shell with no nonzero coefficient is never significant
  }
  if (nf != nb) return fail(HP_ERR_INVALID, "shell functions do not add up to nbasis");
  if ((pure2 && !d->pure2) || (pure3 && !d->pure3))
    return fail(HP_ERR_INVALID, "pure shells need their Cartesian-to-pure matrix");
  const int tile = density_tile(nb, ns);
  if (tile == 0) return fail(HP_ERR_UNSUPPORTED, "basis too large for one point tile");
  HP_CK(cudaSetDevice(ctx->device));
  const size_t ndbl = 3 * (size_t)ns + ns + 2 * (size_t)d->nprim + (size_t)d->nmat * nb * nb;
  const size_t bytes = 8 * ndbl + 4 * 5 * (size_t)ns + 8 * 3;
  if (ctx->used + bytes > ctx->budget) return fail(HP_ERR_NO_MEMORY, "HBM budget exceeded");
  hp_density_plan* p = new hp_density_plan();
  p->ctx = ctx;
  if (cudaMalloc(&p->dev, 8 * std::max<size_t>(ndbl, 1)) != cudaSuccess ||
      cudaMalloc(&p->info, 4 * std::max<size_t>(5 * (size_t)ns, 1)) != cudaSuccess ||
      cudaMalloc(&p->stats, 8 * 3) != cudaSuccess) {
    hp_density_plan_destroy(p);
    return fail(HP_ERR_NO_MEMORY, "device allocation failed");
  }
  double* cen = p->dev;
  double* am = cen + 3 * (size_t)ns;
  double* ex = am + ns;
  double* co = ex + d->nprim;
  double* mats = co + d->nprim;
  cudaStream_t st = ctx->stream;
  int rc = 0;
  rc |= cudaMemcpyAsync(cen, d->centers, 8 * 3 * (size_t)ns, cudaMemcpyHostToDevice, st) != cudaSuccess;
  rc |= cudaMemcpyAsync(am, amin.data(), 8 * (size_t)ns, cudaMemcpyHostToDevice, st) != cudaSuccess;
  rc |= cudaMemcpyAsync(ex, d->exponents, 8 * (size_t)d->nprim, cudaMemcpyHostToDevice, st) != cudaSuccess;
  rc |= cudaMemcpyAsync(co, d->coeffs, 8 * (size_t)d->nprim, cudaMemcpyHostToDevice, st) != cudaSuccess;
  rc |= cudaMemcpyAsync(mats, d->mats, 8 * (size_t)d->nmat * nb * nb, cudaMemcpyHostToDevice, st) != cudaSuccess;
  rc |= cudaMemcpyAsync(p->info, d->shell_info, 4 * 5 * (size_t)ns, cudaMemcpyHostToDevice, st) != cudaSuccess;
  rc |= cudaMemsetAsync(p->stats, 0, 8 * 3, st) != cudaSuccess;
  if (pure2 || pure3) {
    double t2[30] = {0.0}, t3[70] = {0.0};
    if (d->pure2) memcpy(t2, d->pure2, sizeof(t2));
    if (d->pure3) memcpy(t3, d->pure3, sizeof(t3));
    rc |= set_pure_tables(t2, t3);
  }
  rc |= cudaStreamSynchronize(st) != cudaSuccess;
  if (rc) {
    hp_density_plan_destroy(p);
    return fail(HP_ERR_CUDA, "density plan upload failed");
  }
  p->bytes = bytes;
  ctx->used += bytes;
  DensityArgs& a = p->args;
  a.nshell = ns;
  a.nbasis = nb;
  a.nmat = d->nmat;
  a.tile = tile;
  a.centers = cen;
  a.info = p->info;
  a.amin = am;
  a.exps = ex;
  a.coefs = co;
  a.mats = mats;
  a.stats = p->stats;
  *out = p;
  return HP_OK;
}

int32_t hp_density_plan_eval(hp_density_plan* p, int64_t npoint, const double* points, double* out,
                             int32_t device_ptrs) {
  if (!p || (npoint > 0 && (!points || !out)) || npoint < 0) return fail(HP_ERR_INVALID, "bad argument");
  if (npoint == 0) return HP_OK;
  hp_ctx* ctx = p->ctx;
  HP_CK(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  DensityArgs a = p->args;
  a.npoint = npoint;
  const size_t nout = (size_t)a.nmat * (size_t)npoint;
  if (device_ptrs) {
    a.points = points;
    a.out = out;
    launch_density(a, st);
    return check_launch();
  }
  const size_t need = 3 * (size_t)npoint + nout;
  if (p->scratch_points < need) {
    if (p->scratch) {
      cudaFree(p->scratch);
      ctx->used -= 8 * p->scratch_points;
      p->scratch = nullptr;
      p->scratch_points = 0;
    }
    if (ctx->used + 8 * need > ctx->budget) return fail(HP_ERR_NO_MEMORY, "HBM budget exceeded");
    if (cudaMalloc(&p->scratch, 8 * need) != cudaSuccess) return fail(HP_ERR_NO_MEMORY, "device allocation failed");
    p->scratch_points = need;
    ctx->used += 8 * need;
  }
  double* dpts = p->scratch;
  double* dout = dpts + 3 * (size_t)npoint;
  HP_CK(cudaMemcpyAsync(dpts, points, 8 * 3 * (size_t)npoint, cudaMemcpyHostToDevice, st));
  a.points = dpts;
  a.out = dout;
  launch_density(a, st);
  int rc = check_launch();
  if (rc) return rc;
  HP_CK(cudaMemcpyAsync(out, dout, 8 * nout, cudaMemcpyDeviceToHost, st));
  HP_CK(cudaStreamSynchronize(st));
  return HP_OK;
}

int32_t hp_density_plan_stats(hp_density_plan* p, uint64_t* stats) {
  if (!p || !stats) return fail(HP_ERR_INVALID, "null argument");
  HP_CK(cudaSetDevice(p->ctx->device));
  HP_CK(cudaStreamSynchronize(p->ctx->stream));
  unsigned long long h[3];
  HP_CK(cudaMemcpy(h, p->stats, sizeof(h), cudaMemcpyDeviceToHost));
  for (int k = 0; k < 3; ++k) stats[k] = (uint64_t)h[k];
  return HP_OK;
}

int32_t hp_density_plan_destroy(hp_density_plan* p) {
  if (!p) return HP_OK;
  if (p->ctx) {
    cudaSetDevice(p->ctx->device);
    cudaStreamSynchronize(p->ctx->stream);
    p->ctx->used -= p->bytes + 8 * p->scratch_points;
  }
  if (p->dev) cudaFree(p->dev);
  if (p->info) cudaFree(p->info);
  if (p->stats) cudaFree(p->stats);
  if (p->scratch) cudaFree(p->scratch);
  delete p;
  return HP_OK;
}

}  // extern "C"
