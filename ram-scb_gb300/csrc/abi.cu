// abi.cu -- the extern "C" entry points declared in include/ramgpu.h.
//
// The context owns every device buffer.  ramgpu_ram_run enqueues, per call,
//   member tables (VT, E x B, U terms) and DRIFTR ghost planes   2 kernels
//   "last inflow line" scan of the stale DRIFTR ghosts           1
// and then, for each item group (a slice of the active (member, species)
// list, on its own stream; 1 to 8 groups, autotuned):
//   R, P, E, MU (+ fused CEX/ATMOL)      4   (forward half, CFL tracked)
//   MU, E, P, R                          4   (reverse half)
//   periodic copy + magnetopause mask    1
//   ANISCH moments                       2
// mirroring the species loop of src/ModRamRun.f90:64-222; optionally the
// status pass (1).  The whole call is one CUDA graph when graphs are on.
//
// Sections, in order:
//   context        struct ramgpu_ctx, error and allocation helpers,
//                  work-list rebuild and the per-DTs tables (prepare)
//   step           the sweep sequence, item groups on concurrent streams,
//                  the status pass, the graph of ram_run
//   adjoint calls  recorded and replayed calls, checkpoint copies
//   host pipeline  ramgpu_ram_run_host's uploads / sweeps / read-backs
//   ABI            the entry points: lifecycle, inputs, state transfer,
//                  runs, outputs, tuning, outputs for satellites and SCB,
//                  the adjoint window, diagnostics
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/ramgpu.h"
#include "kernels.cuh"
#include "diag.cuh"

using namespace ramgpu;

namespace {
thread_local std::string g_create_error;
constexpr int kSumrcBlocks = 64;
constexpr int kSumrcStages = 9;  // 0-5 ram_run, 6-7 pitch-angle diffusion, 8 reset
}  // namespace

struct ramgpu_ctx {
  ramgpu_config cfg;
  Dev d;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  std::vector<void*> allocs;
  // host mirrors
  std::vector<int> qs, cex;
  std::vector<int> member_active;
  std::vector<std::vector<int>> member_species;
  std::vector<int2> items_h;
  int2* items_d = nullptr;
  bool items_dirty = true;
  bool have_grid = false, have_fields = false;
  bool field_dirty = true, static_dirty = true;
  double tables_dts = -1.0;
  // sweeps (bit w: R, P, E, MU) whose face coefficients the forward half
  // stores for the reverse half; measured on GB300, only DRIFTE (two FP64
  // operations for C) gains, the others lose more to the stores than they
  // save in FP64 work
  unsigned coef_mask = 4u;
  // implicit pitch-angle diffusion: species with a coefficient, tables state
  std::vector<int> pd_on_h;
  bool pd_alloc = false, pd_dirty = false;
  double pd_dts = -1.0;
  int pd_any() const { for (int v : pd_on_h) if (v) return 1; return 0; }
  int any_outside = 0;
  double last_dts = 0.0;
  // loss bookkeeping on the device: per slot {SETRC, LSDR, LSCHA, LSATM, valid}
  double* losses = nullptr;
  double* sumrc_part = nullptr;
  double* upa_h_dummy = nullptr;
  long long launches = 0;
  long long graph_launch_count = 0;
  // CUDA graph of the ram_run sequence, replayed while (dts, items, flags)
  // are unchanged; inputs (Kp, VT, FGEOS, F2) are read at execution time
  bool graph_on = false;
  cudaGraphExec_t graph_exec = nullptr;
  double graph_dts = -1.0;
  long long graph_items = -1;
  unsigned graph_flags = 0;
  int graph_shape = -1;
  long long items_version = 0;
  int shape_version = 0;
  // frozen-limiter adjoint window
  struct Adj {
    bool ready = false;
    int ncalls = 0, k = 0, nseg = 0, nobs = 0;
    double dts = 0.0;
    long long items_version = -1;
    std::vector<double> kp;          // ncalls * nm
    std::vector<int> obs_calls;      // observations per call
    double* kp_d = nullptr;          // the same on the device (copied per call device-to-device)
    ObsDev* obs = nullptr;
    double *fm = nullptr, *fm2 = nullptr, *J = nullptr, *J2 = nullptr, *ckpt = nullptr;
    unsigned char* rec = nullptr;
    unsigned long long* digest = nullptr;
    size_t rec_call = 0;             // bytes of one call's record (8 sweeps, 4 bits per face)
    bool rec_stale = false;          // the record ring no longer holds the kept segments
    int nkeep = 1;                   // trailing segments whose records the ring keeps
  } adj;
  unsigned long long* sep_dev = nullptr;  // separability measure of FFACTOR (bits of a double)
  // device bytes the adjoint's branch-record ring may use (-1: half of the
  // free device memory when the window starts)
  long long adj_record_budget = -1;
  // ramgpu_adj_backward's overlapped recomputation: the segment before the
  // one being transposed is recomputed on a second stream meanwhile, with
  // its own copies of the per-member tables and ghost planes (adj_q points
  // into adj_shadow); per ring slot the events "recomputed" and
  // "transposed", then one for the start and the end
  bool adj_overlap = true;
  cudaStream_t adj_stream = nullptr;
  void* adj_shadow = nullptr;
  double* adj_shadow_coef = nullptr;  // the second stream's DRIFTE coefficient store
  void* adj_ring = nullptr;           // the transposes' per-call table sets
  std::vector<cudaEvent_t> adj_ring_events;
  size_t adj_shadow_coef_bytes = 0;
  std::vector<cudaEvent_t> adj_events;
  // ramgpu_ram_run_host: item groups, their streams and events, and the
  // graph of the whole pipeline for one set of host buffers
  int pipe_groups = 4;  // ramgpu_ram_run_host's copy groups
  // the host calls' plane-chunk pipeline: chunks of L planes (0: off) and
  // its events (per chunk: input landed, forward R/P/E done, chunk done;
  // then start, tables, pitch-angle sweeps done)
  int pipe_chunks = -1;  // -1: per call (item groups for per-species arrays, 4 chunks for the reference layout)
  std::vector<cudaEvent_t> chunk_events;
  int step_groups = 4;  // ram_run's concurrent item groups (autotuned)
  cudaGraphExec_t pipe_exec = nullptr;
  std::vector<const void*> pipe_key;
  double pipe_dts = -1.0;
  long long pipe_items = -1, pipe_launches = 0;
  unsigned pipe_flags = 0;
  int pipe_shape = -1, pipe_g = 0;
  std::vector<cudaStream_t> pipe_streams;
  std::vector<cudaEvent_t> pipe_events;  // per group: uploads done, group done; then one for the tables
  // per group: a companion stream for the F2 read-back, the event after the
  // closing mask it starts from, and its completion
  std::vector<cudaStream_t> pipe_copy_streams;
  std::vector<cudaEvent_t> pipe_fin_events, pipe_copy_done;
  cudaEvent_t finish_hook = nullptr;  // recorded after the closing mask when set
  // host pointer classification of the last ramgpu_ram_run_host pointer set:
  // per pointer, pageable memory the SMs copy; any pageable pointer the copy
  // engines must move (no graph then)
  std::vector<const void*> cls_key;
  std::vector<char> cls_pageable;
  bool cls_engine_pageable = false;
  // ramgpu_ram_run_ref: graph of the whole call for one set of host arrays
  // (their addresses and how the device reaches them), and a device staging
  // buffer of one member's F2 for arrays only the copy engines reach
  cudaGraphExec_t ref_exec = nullptr;
  std::vector<const void*> ref_key;
  double ref_dts = -1.0;
  long long ref_items = -1, ref_launches = 0;
  unsigned ref_flags = 0;
  int ref_shape = -1, ref_g = 0;
  double* ref_stage = nullptr;
  // best whole-step trial times of the last autotune per sweep, plain grid
  // and persistent grid [ms] (0: not tried)
  double tune_plain_ms[4] = {0, 0, 0, 0}, tune_pers_ms[4] = {0, 0, 0, 0};
  bool ref_force_stage = false;  // move reachable arrays by the copy engines too
  // ramgpu_ram_run_ref: page-locked F2 arrays through the copy engines chunk
  // by chunk (a device staging area per member) instead of SM reads over the
  // host link
  bool ref_ce = false;
  double* ref_ce_stage = nullptr;
  size_t ref_ce_bytes = 0;
  int nsm = 0;
  // status word: device words and their page-locked copy; the pass is
  // appended to every call while check_on
  unsigned long long* status_d = nullptr;
  // ramgpu_f2_stats: the partial content sums and the min/max keys
  double* stat_part = nullptr;
  unsigned long long* stat_mm = nullptr;
  unsigned long long* status_h = nullptr;
  bool check_on = false;
  bool status_valid = false;
  // optional timeline of ramgpu_ram_run_host (diagnostics): start, then per
  // group uploads landed, sweeps done, read-back done
  bool pipe_trace = false;
  std::vector<cudaEvent_t> trace_ev;
  std::vector<float> trace_ms;
  // optional per-kernel-class timing
  bool timing = false;
  std::vector<cudaEvent_t> ev_free;
  struct Span { int kind; cudaEvent_t a, b; };
  std::vector<Span> spans;
};

namespace ramgpu {
void set_thread_error(const std::string& msg) { g_create_error = msg; }
}  // namespace ramgpu

// ------------------------------------------------------------------ helpers
static cudaEvent_t take_event(ramgpu_ctx* c) {
  cudaEvent_t e = nullptr;
  if (!c->ev_free.empty()) {
    e = c->ev_free.back();
    c->ev_free.pop_back();
  } else {
    cudaEventCreate(&e);
  }
  return e;
}
// NVTX range names of the kernel classes (the classes of ramgpu_kernel_times).
static const char* const kClassName[] = {"member tables", "DRIFTR ghost planes", "DRIFTR", "DRIFTP", "DRIFTE",
                                         "DRIFTMU", "periodic copy and mask", "ANISCH", "DTs tables",
                                         "SUMRC", "WPADIF"};
// An NVTX range over a scope (a no-op unless a profiler injects NVTX).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};
// Brackets a launch group with an NVTX range of its kernel class and, when
// timing is enabled, with events.
struct Timed {
  ramgpu_ctx* c;
  int kind;
  cudaEvent_t a = nullptr;
  Timed(ramgpu_ctx* c_, int k) : c(c_), kind(k) {
    nvtxRangePushA(kClassName[k]);
    if (c->timing) {
      a = take_event(c);
      cudaEventRecord(a, c->stream);
    }
  }
  ~Timed() {
    if (c->timing && a) {
      cudaEvent_t b = take_event(c);
      cudaEventRecord(b, c->stream);
      c->spans.push_back({kind, a, b});
    }
    nvtxRangePop();
  }
};
static int fail(ramgpu_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  else g_create_error = msg;
  return code;
}
static int cuda_fail(ramgpu_ctx* c, cudaError_t e, const char* where) {
  return fail(c, RAMGPU_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
#define CK(call)                                                  \
  do {                                                            \
    cudaError_t e_ = (call);                                      \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call);      \
  } while (0)
#define CKL(where)                                                \
  do {                                                            \
    cudaError_t e_ = cudaGetLastError();                          \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, where);      \
  } while (0)

template <class T>
static T* dalloc(ramgpu_ctx* c, size_t n, bool* ok) {
  void* p = nullptr;
  if (n == 0) n = 1;
  if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) {
    *ok = false;
    return nullptr;
  }
  cudaMemset(p, 0, n * sizeof(T));
  c->allocs.push_back(p);
  return (T*)p;
}

static int check_ctx(ramgpu_ctx* ctx) { return ctx ? RAMGPU_OK : RAMGPU_ERR_ARG; }

static int check_ms(ramgpu_ctx* ctx, int member, int s) {
  if (member < 0 || member >= ctx->cfg.n_members) return fail(ctx, RAMGPU_ERR_ARG, "member out of range");
  if (s < 0 || s >= ctx->cfg.ns) return fail(ctx, RAMGPU_ERR_ARG, "species out of range");
  return RAMGPU_OK;
}

static int rebuild_items(ramgpu_ctx* ctx) {
  ctx->items_h.clear();
  for (int m = 0; m < ctx->cfg.n_members; ++m) {
    if (!ctx->member_active[m]) continue;
    for (int s : ctx->member_species[m]) ctx->items_h.push_back(make_int2(m, s));
  }
  if (!ctx->items_h.empty())
    CK(cudaMemcpyAsync(ctx->items_d, ctx->items_h.data(), sizeof(int2) * ctx->items_h.size(),
                       cudaMemcpyHostToDevice, ctx->stream));
  ctx->d.items = ctx->items_d;
  ctx->d.nitems = (int)ctx->items_h.size();
  ctx->items_dirty = false;
  ctx->items_version += 1;
  return RAMGPU_OK;
}

static unsigned dev_flags(const ramgpu_ctx* ctx) {
  return (ctx->cfg.flags & 7u) | (ctx->any_outside ? 0x80000000u : 0u);
}

// Bring every derived table up to date for step length dts.
static int prepare(ramgpu_ctx* ctx, double dts) {
  if (!ctx->have_grid || !ctx->have_fields)
    return fail(ctx, RAMGPU_ERR_STATE, "ramgpu_set_grid and ramgpu_set_fields must be called first");
  if (!(dts > 0.0) || !isfinite(dts)) return fail(ctx, RAMGPU_ERR_ARG, "dts must be positive and finite");
  ctx->d.flags = dev_flags(ctx);
  Timed tm_(ctx, 8);
  if (ctx->field_dirty) {
    launch_field_tables(ctx->d, ctx->stream);
    ctx->launches += 1;
    CKL("field tables");
    ctx->field_dirty = false;
    ctx->static_dirty = true;
    ctx->tables_dts = -1.0;
    ctx->pd_dirty = true;
  }
  if (ctx->static_dirty) {
    // the moment sums take the two-fma form when FFACTOR is separable to
    // rounding (the ARRAYS formula); deciding that reads one value back
    const int sep_before = ctx->d.mom_sep;
    ctx->d.mom_sep = 0;
    launch_species_static(ctx->d, ctx->sep_dev, ctx->stream);
    ctx->launches += 3;
    CKL("species tables");
    unsigned long long dev_bits = ~0ULL;
    CK(cudaMemcpyAsync(&dev_bits, ctx->sep_dev, sizeof(dev_bits), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    double dev = 1.0;
    memcpy(&dev, &dev_bits, sizeof(dev));
    ctx->d.mom_sep = (dev <= 1e-13) ? 1 : 0;
    if (ctx->d.mom_sep != sep_before) ctx->shape_version += 1;  // another moment kernel: recapture
    ctx->static_dirty = false;
    ctx->tables_dts = -1.0;
  }
  if (ctx->tables_dts != dts) {
    launch_dts_tables(ctx->d, dts, ctx->stream);
    ctx->launches += 4;
    CKL("dts tables");
    ctx->tables_dts = dts;
  }
  if (ctx->pd_any() && (ctx->pd_dirty || ctx->pd_dts != dts)) {
    launch_padif_tables(ctx->d, dts, ctx->stream);
    ctx->launches += 2;
    CKL("pitch-angle diffusion tables");
    ctx->pd_dirty = false;
    ctx->pd_dts = dts;
  }
  if (ctx->items_dirty) {
    int rc = rebuild_items(ctx);
    if (rc) return rc;
  }
  // face-coefficient store for the reverse half: 64 bytes per cell and item,
  // kept only while it takes at most a quarter of the free device memory
  if (ctx->coef_mask && ctx->d.coef_items < ctx->d.nitems) {
    cudaFree(ctx->d.coef);
    ctx->d.coef = nullptr;
    ctx->d.coef_items = 0;
    int nw = 0;
    for (int w = 0; w < 4; ++w) ctx->d.coef_slot[w] = ((ctx->coef_mask >> w) & 1u) ? nw++ : -1;
    const size_t need = (size_t)2 * nw * ctx->d.nitems * ctx->d.ncell * sizeof(double);
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) == cudaSuccess && need <= fr / 4 &&
        cudaMalloc(&ctx->d.coef, need) == cudaSuccess) {
      ctx->d.coef_items = ctx->d.nitems;
    } else {
      ctx->d.coef = nullptr;
      cudaGetLastError();
    }
    ctx->shape_version += 1;  // launch sequence changed: recapture the graph
  }
  return RAMGPU_OK;
}

// SUMRC of every item into stage buffer `stage`, then fold into the device
// accumulators: which = -1 (set SETRC only), 1 LSDR, 2 LSCHA, 3 LSATM,
// 5 LSWAE (index 4 marks a valid SETRC).
__global__ void k_losses_fold(Dev d, const double* part, int nblk, double* losses, int which) {
  const int it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= d.nitems) return;
  const int2 item = d.items[it];
  const int slot = item.x * d.ns + item.y;
  double s = 0.0;
  for (int b = 0; b < nblk; ++b) s += part[(long long)it * nblk + b];
  double* L = losses + (long long)slot * 6;
  if (which >= 1 && L[4] != 0.0) L[which] += L[0] - s;  // ELORC = ENOLD - SETRC
  L[0] = s;
  L[4] = 1.0;
}

static int sumrc_stage(ramgpu_ctx* ctx, int stage, int which) {
  double* part = ctx->sumrc_part + (size_t)stage * ctx->d.nm * ctx->d.ns * kSumrcBlocks;
  Timed tm_(ctx, 9);
  launch_sumrc(ctx->d, part, kSumrcBlocks, ctx->stream);
  k_losses_fold<<<(ctx->d.nitems + 127) / 128, 128, 0, ctx->stream>>>(ctx->d, part, kSumrcBlocks,
                                                                     ctx->losses, which);
  ctx->launches += 2;
  CKL("sumrc");
  return RAMGPU_OK;
}

// Forward sweeps with the CFL reduction; when the coefficient store exists
// they also keep each face's C and CORR factor for the reverse half.
static int enqueue_forward(ramgpu_ctx* ctx, double dts, bool loss_fused, const double* loss_table,
                           bool clear_cfl = true) {
  if (clear_cfl)
    CK(cudaMemsetAsync(ctx->d.cflq, 0, sizeof(unsigned long long) * 5 * ctx->d.nm * ctx->d.ns, ctx->stream));
  const Dev& d = ctx->d;
  auto co = [&](int w) { return (d.coef && d.coef_slot[w] >= 0) ? 1 : 0; };
  { Timed t(ctx, 2); launch_sweep_r(d, dts, true, ctx->stream, nullptr, false, co(0)); }
  { Timed t(ctx, 3); launch_sweep_p(d, dts, true, ctx->stream, nullptr, false, co(1)); }
  { Timed t(ctx, 4); launch_sweep_e(d, dts, true, ctx->stream, nullptr, false, co(2)); }
  { Timed t(ctx, 5); launch_sweep_mu(d, dts, true, loss_fused ? 1 : 0, loss_table, ctx->stream, nullptr, false, co(3)); }
  ctx->launches += 4;
  CKL("forward sweeps");
  return RAMGPU_OK;
}

// Reverse sweeps; after_forward: the forward half of the same call ran just
// before, so its stored face coefficients are read back.
static int enqueue_reverse(ramgpu_ctx* ctx, double dts, bool loss_fused, const double* loss_table,
                           bool after_forward) {
  const Dev& d = ctx->d;
  auto co = [&](int w) { return (after_forward && d.coef && d.coef_slot[w] >= 0) ? 2 : 0; };
  { Timed t(ctx, 5); launch_sweep_mu(d, dts, false, loss_fused ? 2 : 0, loss_table, ctx->stream, nullptr, false, co(3)); }
  { Timed t(ctx, 4); launch_sweep_e(d, dts, false, ctx->stream, nullptr, false, co(2)); }
  { Timed t(ctx, 3); launch_sweep_p(d, dts, false, ctx->stream, nullptr, false, co(1)); }
  { Timed t(ctx, 2); launch_sweep_r(d, dts, false, ctx->stream, nullptr, false, co(0)); }
  ctx->launches += 4;
  CKL("reverse sweeps");
  return RAMGPU_OK;
}

// The sweeps, losses and tail of one ram_run call for the work items of
// ctx->d (the per-member tables and ghost planes are enqueued before);
// clear_cfl: reset the CFL accumulators first.
static int enqueue_sweeps(ramgpu_ctx* ctx, double dts, bool clear_cfl) {
  int rc = RAMGPU_OK;
  const bool losses = ctx->cfg.flags & RAMGPU_FLAG_LOSSES;
  const bool pd = ctx->pd_any();
  if (!losses && !pd) {
    // R,P,E,MU then CEX,ATMOL,ATMOL,CEX folded into the MU store
    if ((rc = enqueue_forward(ctx, dts, true, ctx->d.loss2, clear_cfl))) return rc;
    if ((rc = enqueue_reverse(ctx, dts, false, nullptr, true))) return rc;
  } else if (!losses) {
    // R,P,E,MU, WPADIF, CEX,ATMOL,ATMOL,CEX (folded into WPADIF's store), WPADIF, MU,E,P,R
    if ((rc = enqueue_forward(ctx, dts, false, nullptr, clear_cfl))) return rc;
    { Timed t(ctx, 10); launch_padif(ctx->d, ctx->d.loss2, ctx->stream); }
    { Timed t(ctx, 10); launch_padif(ctx->d, nullptr, ctx->stream); }
    ctx->launches += 2;
    CKL("pitch-angle diffusion");
    if ((rc = enqueue_reverse(ctx, dts, false, nullptr, true))) return rc;
  } else {
    if ((rc = enqueue_forward(ctx, dts, false, nullptr, clear_cfl))) return rc;
    if ((rc = sumrc_stage(ctx, 0, 1))) return rc;
    if (pd) {
      { Timed t(ctx, 10); launch_padif(ctx->d, nullptr, ctx->stream); }
      ctx->launches += 1;
      if ((rc = sumrc_stage(ctx, 6, 5))) return rc;
    }
    { Timed t(ctx, 9); launch_loss_apply(ctx->d, ctx->d.charge, ctx->stream); }
    if ((rc = sumrc_stage(ctx, 1, 2))) return rc;
    { Timed t(ctx, 9); launch_loss_apply(ctx->d, ctx->d.atm, ctx->stream); }
    if ((rc = sumrc_stage(ctx, 2, 3))) return rc;
    { Timed t(ctx, 9); launch_loss_apply(ctx->d, ctx->d.atm, ctx->stream); }
    if ((rc = sumrc_stage(ctx, 3, 3))) return rc;
    { Timed t(ctx, 9); launch_loss_apply(ctx->d, ctx->d.charge, ctx->stream); }
    if ((rc = sumrc_stage(ctx, 4, 2))) return rc;
    ctx->launches += 4;
    if (pd) {
      { Timed t(ctx, 10); launch_padif(ctx->d, nullptr, ctx->stream); }
      ctx->launches += 1;
      if ((rc = sumrc_stage(ctx, 7, 5))) return rc;
    }
    if ((rc = enqueue_reverse(ctx, dts, false, nullptr, true))) return rc;
    if ((rc = sumrc_stage(ctx, 5, 1))) return rc;
  }
  { Timed t(ctx, 6); launch_finish(ctx->d, ctx->stream); }
  if (ctx->finish_hook) CK(cudaEventRecord(ctx->finish_hook, ctx->stream));
  { Timed t(ctx, 7); launch_moments(ctx->d, ctx->stream); }
  ctx->launches += 3;
  CKL("finish/moments");
  return RAMGPU_OK;
}

static int enqueue_tables(ramgpu_ctx* ctx, double dts) {
  { Timed t(ctx, 0); launch_member_coef(ctx->d, dts, ctx->stream); }
  { Timed t(ctx, 1); launch_ghost(ctx->d, ctx->stream); }
  ctx->launches += 3;
  CKL("member tables");
  return RAMGPU_OK;
}

static int enqueue_pipeline(ramgpu_ctx* ctx, double dts, double* const* f2, double* const* ppert,
                            double* const* ppart, int G, const std::vector<char>& pageable);
static int ensure_group_streams(ramgpu_ctx* ctx, int G);

// Runs fn() once per item group, each on its own stream with ctx->d
// narrowed to the group's items (ctx->stream is the group's stream
// meanwhile); the groups start after the work enqueued so far on the
// context's stream, which then waits for all of them.  G == 1: fn() on the
// context's stream, no events.  Every buffer a group's kernels write is
// indexed by slot or by the item's place in the list (Dev::item0 and the
// per-group offsets fn applies), so the groups never write the same bytes.
template <class F>
static int over_groups(ramgpu_ctx* ctx, int G, F&& fn) {
  if (G <= 1) return fn(0);
  const cudaStream_t main = ctx->stream;
  const Dev full = ctx->d;
  const int nit = full.nitems;
  cudaEvent_t ev0 = ctx->pipe_events[2 * G + 1];
  CK(cudaEventRecord(ev0, main));
  for (int g = 0; g < G; ++g) {
    const int i0 = (int)((long long)nit * g / G), i1 = (int)((long long)nit * (g + 1) / G);
    cudaStream_t st = ctx->pipe_streams[g];
    CK(cudaStreamWaitEvent(st, ev0, 0));
    ctx->stream = st;
    ctx->d.items = full.items + i0;
    ctx->d.nitems = i1 - i0;
    ctx->d.item0 = full.item0 + i0;
    const int rc = fn(i0);
    ctx->d = full;
    ctx->stream = main;
    if (rc) return rc;
    CK(cudaEventRecord(ctx->pipe_events[2 * g + 1], st));
    CK(cudaStreamWaitEvent(main, ctx->pipe_events[2 * g + 1], 0));
  }
  return RAMGPU_OK;
}

// Item groups of a step: 1 with the loss bookkeeping (its partial sums are
// indexed by list position) and in per-kernel timing passes (the events sit
// on one stream), else the given count, at most one group per item.
static int clamp_groups(const ramgpu_ctx* ctx, int groups) {
  if ((ctx->cfg.flags & RAMGPU_FLAG_LOSSES) || ctx->timing) return 1;
  return std::max(1, std::min(groups, ctx->d.nitems));
}

// One ram_run step on the device-resident F2.  With more than one item
// group the groups' sweeps run on concurrent streams: one group's launch
// tails and the gaps between its dependent launches are filled by the
// others' CTAs (the same groups as ramgpu_ram_run_host, without copies).
// The status pass (status.cu) and the copy of its word to the host, on the
// context's stream.
static int enqueue_status(ramgpu_ctx* ctx) {
  launch_status(ctx->d, ctx->status_d, ctx->stream);
  ctx->launches += ctx->d.nitems ? 1 : 0;
  CK(cudaMemcpyAsync(ctx->status_h, ctx->status_d, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CKL("status pass");
  return RAMGPU_OK;
}

static int enqueue_body(ramgpu_ctx* ctx, double dts) {
  const int G = clamp_groups(ctx, ctx->step_groups);
  int rc = RAMGPU_OK;
  if (G > 1) {
    if ((rc = ensure_group_streams(ctx, G))) return rc;
    rc = enqueue_pipeline(ctx, dts, nullptr, nullptr, nullptr, G, {});
  } else {
    if ((rc = enqueue_tables(ctx, dts))) return rc;
    rc = enqueue_sweeps(ctx, dts, true);
  }
  if (!rc && ctx->check_on) rc = enqueue_status(ctx);
  return rc;
}

static void adj_free(ramgpu_ctx* ctx) {
  auto& a = ctx->adj;
  cudaFree(a.obs); cudaFree(a.fm); cudaFree(a.fm2); cudaFree(a.J); cudaFree(a.J2); cudaFree(a.ckpt);
  cudaFree(a.rec); cudaFree(a.digest); cudaFree(a.kp_d);
  a.obs = nullptr; a.fm = a.fm2 = a.J = a.J2 = a.ckpt = a.kp_d = nullptr; a.rec = nullptr; a.digest = nullptr;
  a.ready = false;
}

// One ram_run call with every sweep recording its branches into rec
// (8 instances of nitems*ncell bytes: R,P,E,MU forward, MU,E,P,R reverse),
// the sweeps over the step's item groups (the record of item i sits at
// i*ncell in each instance).
static int enqueue_call_rec(ramgpu_ctx* ctx, double dts, unsigned char* rec, bool moments) {
  const size_t isz = (size_t)ctx->d.nitems * ctx->d.ncell;
  // positions no sweep writes (e.g. cell 1 of a DRIFTR line) are the same
  // in every call and stay zero from the ring's allocation
  launch_member_coef(ctx->d, dts, ctx->stream);
  launch_ghost(ctx->d, ctx->stream);
  ctx->launches += 3;
  const int G = clamp_groups(ctx, ctx->step_groups);
  if (int rc = ensure_group_streams(ctx, G)) return rc;
  // DRIFTE keeps its face coefficients for the reverse half as in the plain
  // step (same DTs and VT within a call)
  const int co_e = (ctx->d.coef && ctx->d.coef_slot[2] >= 0) ? 1 : 0;
  return over_groups(ctx, G, [&](int i0) {
    const Dev& d = ctx->d;
    const cudaStream_t st = ctx->stream;
    unsigned char* r = rec + (size_t)i0 * d.ncell;
    launch_sweep_r(d, dts, false, st, r + 0 * isz, false, 0, 4);
    launch_sweep_p(d, dts, false, st, r + 1 * isz, false, 0, 4);
    launch_sweep_e(d, dts, false, st, r + 2 * isz, false, co_e, 4);
    launch_sweep_mu(d, dts, false, 1, d.loss2, st, r + 3 * isz, false, 0, 4);
    launch_sweep_mu(d, dts, false, 0, nullptr, st, r + 3 * isz, false, 0, 0);
    launch_sweep_e(d, dts, false, st, r + 2 * isz, false, 2 * co_e, 0);
    launch_sweep_p(d, dts, false, st, r + 1 * isz, false, 0, 0);
    launch_sweep_r(d, dts, false, st, r + 0 * isz, false, 0, 0);
    launch_finish(d, st);
    if (moments) launch_moments(d, st);
    else launch_anisch_state(d, st);
    ctx->launches += moments ? 11 : 10;
    CKL("recorded ram_run");
    return RAMGPU_OK;
  });
}

// One ram_run call with every sweep taking its branches and clips from rec
// (the frozen-limiter scheme of a recorded call, applied to the current F2).
static int enqueue_call_replay(ramgpu_ctx* ctx, double dts, unsigned char* rec) {
  const size_t isz = (size_t)ctx->d.nitems * ctx->d.ncell;
  launch_member_coef(ctx->d, dts, ctx->stream);
  launch_ghost(ctx->d, ctx->stream);
  ctx->launches += 3;
  const int G = clamp_groups(ctx, ctx->step_groups);
  if (int rc = ensure_group_streams(ctx, G)) return rc;
  return over_groups(ctx, G, [&](int i0) {
    const Dev& d = ctx->d;
    const cudaStream_t st = ctx->stream;
    unsigned char* r = rec + (size_t)i0 * d.ncell;
    launch_sweep_r(d, dts, false, st, r + 0 * isz, true, 0, 4);
    launch_sweep_p(d, dts, false, st, r + 1 * isz, true, 0, 4);
    launch_sweep_e(d, dts, false, st, r + 2 * isz, true, 0, 4);
    launch_sweep_mu(d, dts, false, 1, d.loss2, st, r + 3 * isz, true, 0, 4);
    launch_sweep_mu(d, dts, false, 0, nullptr, st, r + 3 * isz, true, 0, 0);
    launch_sweep_e(d, dts, false, st, r + 2 * isz, true, 0, 0);
    launch_sweep_p(d, dts, false, st, r + 1 * isz, true, 0, 0);
    launch_sweep_r(d, dts, false, st, r + 0 * isz, true, 0, 0);
    launch_finish(d, st);
    launch_anisch_state(d, st);
    ctx->launches += 10;
    CKL("replayed ram_run");
    return RAMGPU_OK;
  });
}

static int adj_copy_items(ramgpu_ctx* ctx, double* dst, bool to_ckpt) {
  const size_t n = ctx->d.ncell;
  for (size_t i = 0; i < ctx->items_h.size(); ++i) {
    const int slot = ctx->items_h[i].x * ctx->d.ns + ctx->items_h[i].y;
    double* f = ctx->d.f2 + (size_t)slot * n;
    CK(cudaMemcpyAsync(to_ckpt ? dst + i * n : f, to_ckpt ? f : dst + i * n, sizeof(double) * n,
                       cudaMemcpyDeviceToDevice, ctx->stream));
  }
  return RAMGPU_OK;
}

// Kp of every member for one call of the window, device to device (the host
// does not wait for the stream).
static int adj_set_kp(ramgpu_ctx* ctx, int call) {
  const int nm = ctx->cfg.n_members;
  CK(cudaMemcpyAsync(ctx->d.kp, ctx->adj.kp_d + (size_t)call * nm, sizeof(double) * nm,
                     cudaMemcpyDeviceToDevice, ctx->stream));
  return RAMGPU_OK;
}

static void drop_graph(ramgpu_ctx* ctx) {
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  ctx->graph_exec = nullptr;
}

static int enqueue_ram_run(ramgpu_ctx* ctx, double dts) {
  int rc = prepare(ctx, dts);
  if (rc) return rc;
  ctx->last_dts = dts;
  if (ctx->d.nitems == 0) return RAMGPU_OK;
  if (!ctx->graph_on || ctx->timing) return enqueue_body(ctx, dts);
  // CUDA graph: capture once per (dts, work list, flags, launch shapes), replay
  if (!ctx->graph_exec || ctx->graph_dts != dts || ctx->graph_items != ctx->items_version ||
      ctx->graph_flags != ctx->d.flags || ctx->graph_shape != ctx->shape_version) {
    drop_graph(ctx);
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const long long l0 = ctx->launches;
    rc = enqueue_body(ctx, dts);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "graph capture");
    e = cudaGraphInstantiate(&ctx->graph_exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      ctx->graph_exec = nullptr;
      return cuda_fail(ctx, e, "graph instantiate");
    }
    ctx->graph_launch_count = ctx->launches - l0;
    ctx->launches = l0;
    ctx->graph_dts = dts;
    ctx->graph_items = ctx->items_version;
    ctx->graph_flags = ctx->d.flags;
    ctx->graph_shape = ctx->shape_version;
  }
  CK(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
  ctx->launches += ctx->graph_launch_count;
  return RAMGPU_OK;
}

// FP64 fma throughput probe: 8 independent chains per thread.
__global__ void k_probe_dfma(double* out, double a, double b, int iters) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

// L2 read-bandwidth probe: every thread streams 16-byte loads that bypass
// L1 over a buffer resident in L2, many passes; the XOR of what it read is
// stored so the loads stay.
__global__ void k_probe_l2(const uint4* __restrict__ buf, long long n16, int passes, unsigned* out) {
  unsigned acc = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  for (int p = 0; p < passes; ++p)
    for (long long i = t0; i < n16; i += stride) {
      const uint4 v = __ldcg(buf + i);
      acc ^= v.x ^ v.y ^ v.z ^ v.w;
    }
  out[t0] = acc;
}

// =================================================================== ABI
// Copy of n doubles by the SMs, for host memory the device reaches without
// registration (pageable memory on a coherent host link, such as a Fortran
// allocatable): asynchronous and graph-capturable where a copy-engine
// transfer from pageable memory blocks the host.  16-byte vectors when both
// ends allow them.
__global__ void k_copy_f64(const double* __restrict__ src, double* __restrict__ dst, long long n) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if ((((uintptr_t)src | (uintptr_t)dst) & 15u) == 0) {
    const double2* s2 = reinterpret_cast<const double2*>(src);
    double2* d2 = reinterpret_cast<double2*>(dst);
    for (long long i = t0; i < n / 2; i += stride) d2[i] = s2[i];
    if (t0 == 0 && (n & 1)) dst[n - 1] = src[n - 1];
  } else {
    for (long long i = t0; i < n; i += stride) dst[i] = src[i];
  }
}

// One transfer of the pipeline: a copy-engine copy, or the SM copy when the
// host side is pageable memory the device can reach (ctx->pageable_sm).
static int pipe_copy(ramgpu_ctx* ctx, double* dst, const double* src, size_t n, bool host_is_pageable,
                     cudaStream_t st) {
  if (host_is_pageable) {
    k_copy_f64<<<64, 256, 0, st>>>(src, dst, (long long)n);
    ctx->launches += 1;
    CKL("pageable copy");
  } else {
    CK(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDefault, st));
  }
  return RAMGPU_OK;
}

// Streams and events for G item groups.  Group g's stream gets the g-th
// highest priority, so the block scheduler favours the groups in upload
// order.
static int ensure_group_streams(ramgpu_ctx* ctx, int G) {
  if ((int)ctx->pipe_streams.size() < G) {
    int least = 0, greatest = 0;
    CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    while ((int)ctx->pipe_streams.size() < G) {
      const int prio = std::min(least, greatest + (int)ctx->pipe_streams.size());
      cudaStream_t st = nullptr;
      CK(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, prio));
      ctx->pipe_streams.push_back(st);
    }
  }
  while ((int)ctx->pipe_events.size() < 2 * G + 2) {
    cudaEvent_t e = nullptr;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    ctx->pipe_events.push_back(e);
  }
  while ((int)ctx->pipe_copy_streams.size() < G) {
    const size_t g = ctx->pipe_copy_streams.size();
    int prio = 0;
    CK(cudaStreamGetPriority(ctx->pipe_streams[g], &prio));
    cudaStream_t st = nullptr;
    CK(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, prio));
    ctx->pipe_copy_streams.push_back(st);
    cudaEvent_t a = nullptr, b = nullptr;
    CK(cudaEventCreateWithFlags(&a, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&b, cudaEventDisableTiming));
    ctx->pipe_fin_events.push_back(a);
    ctx->pipe_copy_done.push_back(b);
  }
  return RAMGPU_OK;
}

// ram_run with F2 crossing the host boundary, pipelined over chunks of L
// planes.  L is the slowest index of F2, in the library's per-species
// blocks and in the reference's F2(NS,NR,NT,NE,NPA) alike, so a chunk of
// planes is one contiguous range of every array; and every line of the R,
// P and E sweeps and of the closing copy/mask lies in one plane.  So the
// forward R, P, E of chunk c run as soon as its planes have landed (while
// the next chunk's arrive over the host link), the pitch-angle sweeps
// (whose lines span every plane) run once all chunks are in, and the
// reverse E, P, R and the copy/mask of chunk c are followed at once by its
// read-back (while the next chunk computes).  ANISCH, which rewrites the
// L = 1 plane, runs last; that plane and the moments go back after it.
// Streams: chunk c on its own stream; inputs chained in chunk order (they
// share the link); the per-member tables, ghost planes and pitch-angle
// sweeps on the context's stream, joined by events.  in(c, stream, l0, l1)
// and out(c, stream, l0, l1) enqueue the copies of planes [l0, l1);
// tail(stream) the L = 1 plane and the moments.  The sweeps over disjoint
// planes write disjoint cells, and CFL maxima and clip counts combine by
// atomic max/add, so results equal the resident step's bit for bit.
static int ensure_chunk_events(ramgpu_ctx* ctx, int C) {
  while ((int)ctx->chunk_events.size() < 3 * C + 3) {
    cudaEvent_t e = nullptr;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    ctx->chunk_events.push_back(e);
  }
  return RAMGPU_OK;
}

template <class In, class Out, class Tail>
static int enqueue_chunked(ramgpu_ctx* ctx, double dts, int C, In&& in, Out&& out, Tail&& tail) {
  if (int rc = ensure_group_streams(ctx, C)) return rc;
  if (int rc = ensure_chunk_events(ctx, C)) return rc;
  const Dev full = ctx->d;
  const cudaStream_t main = ctx->stream;
  const int npa = full.npa;
  auto lo = [&](int c) { return (int)((long long)npa * c / C); };
  cudaEvent_t* ev = ctx->chunk_events.data();
  cudaEvent_t ev_start = ev[3 * C], ev_tab = ev[3 * C + 1], ev_mu = ev[3 * C + 2];
  auto co = [&](int w, int k) { return (full.coef && full.coef_slot[w] >= 0) ? k : 0; };
  int rc = RAMGPU_OK;
  CK(cudaEventRecord(ev_start, main));
  if ((rc = enqueue_tables(ctx, dts))) return rc;
  CK(cudaMemsetAsync(full.cflq, 0, sizeof(unsigned long long) * 5 * full.nm * full.ns, main));
  CK(cudaEventRecord(ev_tab, main));
  for (int c = 0; c < C; ++c) {
    cudaStream_t st = ctx->pipe_streams[c];
    CK(cudaStreamWaitEvent(st, c == 0 ? ev_start : ev[3 * (c - 1)], 0));
    if ((rc = in(c, st, lo(c), lo(c + 1)))) return rc;
    CK(cudaEventRecord(ev[3 * c], st));
    CK(cudaStreamWaitEvent(st, ev_tab, 0));
    Dev dc = full;
    dc.lw0 = lo(c);
    dc.lw1 = lo(c + 1);
    { NvtxRange r("DRIFTR"); launch_sweep_r(dc, dts, true, st, nullptr, false, co(0, 1)); }
    { NvtxRange r("DRIFTP"); launch_sweep_p(dc, dts, true, st, nullptr, false, co(1, 1)); }
    { NvtxRange r("DRIFTE"); launch_sweep_e(dc, dts, true, st, nullptr, false, co(2, 1)); }
    ctx->launches += 3;
    CKL("chunk forward sweeps");
    CK(cudaEventRecord(ev[3 * c + 1], st));
    CK(cudaStreamWaitEvent(main, ev[3 * c + 1], 0));
  }
  {
    NvtxRange r("DRIFTMU");
    launch_sweep_mu(full, dts, true, 1, full.loss2, main, nullptr, false, co(3, 1));
    launch_sweep_mu(full, dts, false, 0, nullptr, main, nullptr, false, co(3, 2));
    ctx->launches += 2;
    CKL("pitch-angle sweeps");
  }
  CK(cudaEventRecord(ev_mu, main));
  for (int c = 0; c < C; ++c) {
    cudaStream_t st = ctx->pipe_streams[c];
    CK(cudaStreamWaitEvent(st, ev_mu, 0));
    Dev dc = full;
    dc.lw0 = lo(c);
    dc.lw1 = lo(c + 1);
    { NvtxRange r("DRIFTE"); launch_sweep_e(dc, dts, false, st, nullptr, false, co(2, 2)); }
    { NvtxRange r("DRIFTP"); launch_sweep_p(dc, dts, false, st, nullptr, false, co(1, 2)); }
    { NvtxRange r("DRIFTR"); launch_sweep_r(dc, dts, false, st, nullptr, false, co(0, 2)); }
    launch_finish(dc, st);
    ctx->launches += 4;
    CKL("chunk reverse sweeps");
    if ((rc = out(c, st, lo(c), lo(c + 1)))) return rc;
    CK(cudaEventRecord(ev[3 * c + 2], st));
    CK(cudaStreamWaitEvent(main, ev[3 * c + 2], 0));
  }
  { NvtxRange r("ANISCH"); launch_moments(full, main); }
  ctx->launches += 2;
  CKL("moments");
  if ((rc = tail(main))) return rc;
  if (ctx->check_on) rc = enqueue_status(ctx);
  return rc;
}

// Whether the host calls take the plane-chunk pipeline: not with the loss
// bookkeeping, the pitch-angle diffusion or the per-group trace (those keep
// the item-group pipeline), and only with at least two planes per chunk.
// auto_chunks: the count used while the setting is automatic (-1).  Measured
// on the four-species step: per-species page-locked arrays go faster over
// the item-group pipeline (0.69 ms per call against 0.93-1.07 ms chunked),
// the reference layout over 4 chunks (0.88 ms against 0.91 ms unchunked).
static int chunk_count(const ramgpu_ctx* ctx, int auto_chunks) {
  const int want = ctx->pipe_chunks < 0 ? auto_chunks : ctx->pipe_chunks;
  if (want <= 0 || (ctx->cfg.flags & RAMGPU_FLAG_LOSSES) || ctx->pd_any() || ctx->pipe_trace) return 0;
  return std::max(1, std::min(want, ctx->d.npa / 2));
}

// Uploads, sweeps and read-back of ram_run pipelined over item groups.
// Stream order: the context's stream (previous work) -> event -> group
// uploads chained in group order (so the first group starts computing
// first) ; the per-member tables, ghost planes and CFL reset on the
// context's stream -> event ; group g: its uploads, the tables event, its
// sweeps and tail on a view of the work list, its read-back -> event the
// context's stream waits for.  The coefficient store is indexed by the
// item's place in the full list (Dev::item0), so groups never share it.
// f2 == NULL: no copies at all (the resident step over groups).
// Enqueue only (direct launches or inside a graph capture of the context's
// stream, which the group streams join through the events).
static int enqueue_pipeline(ramgpu_ctx* ctx, double dts, double* const* f2, double* const* ppert,
                            double* const* ppart, int G, const std::vector<char>& pageable) {
  const int nit = ctx->d.nitems;
  cudaEvent_t ev_prev = ctx->pipe_events[2 * G], ev_tab = ctx->pipe_events[2 * G + 1];
  const size_t n = ctx->d.ncell, nm2 = (size_t)ctx->d.nr * ctx->d.nt;
  const cudaStream_t main = ctx->stream;
  const Dev full = ctx->d;
  auto slot_of = [&](int it) { return ctx->items_h[it].x * full.ns + ctx->items_h[it].y; };
  const bool trace = ctx->pipe_trace && f2;
  if (trace) CK(cudaEventRecord(ctx->trace_ev[0], main));
  CK(cudaEventRecord(ev_prev, main));
  // uploads, in group order
  for (int g = 0; g < G && f2; ++g) {
    const int i0 = (int)((long long)nit * g / G), i1 = (int)((long long)nit * (g + 1) / G);
    cudaStream_t st = ctx->pipe_streams[g];
    CK(cudaStreamWaitEvent(st, g == 0 ? ev_prev : ctx->pipe_events[2 * (g - 1)], 0));
    for (int it = i0; it < i1; ++it) {
      const int slot = slot_of(it);
      if (f2[slot])
        if (int rc = pipe_copy(ctx, full.f2 + (size_t)slot * n, f2[slot], n, pageable[slot], st)) return rc;
    }
    CK(cudaEventRecord(ctx->pipe_events[2 * g], st));
    if (trace) CK(cudaEventRecord(ctx->trace_ev[1 + 3 * g], st));
  }
  // per-member tables and ghost planes of every item, CFL accumulators
  if (int rc = enqueue_tables(ctx, dts)) return rc;
  CK(cudaMemsetAsync(full.cflq, 0, sizeof(unsigned long long) * 5 * full.nm * full.ns, main));
  CK(cudaEventRecord(ev_tab, main));
  for (int g = 0; g < G; ++g) {
    const int i0 = (int)((long long)nit * g / G), i1 = (int)((long long)nit * (g + 1) / G);
    cudaStream_t st = ctx->pipe_streams[g];
    CK(cudaStreamWaitEvent(st, ev_tab, 0));
    ctx->stream = st;
    ctx->d.items = full.items + i0;
    ctx->d.nitems = i1 - i0;
    ctx->d.item0 = i0;
    ctx->finish_hook = f2 ? ctx->pipe_fin_events[g] : nullptr;
    const int rc = enqueue_sweeps(ctx, dts, false);
    ctx->finish_hook = nullptr;
    ctx->d = full;
    ctx->stream = main;
    if (rc) return rc;
    if (trace) CK(cudaEventRecord(ctx->trace_ev[2 + 3 * g], st));
    if (f2) {
      // F2 is final after the closing mask except its L = 1 plane, which
      // ANISCH then overwrites (F2(:,:,:,1) = F2(:,:,:,2)): the L >= 2 part
      // (contiguous after the first NR*NT*NE values) goes back on the
      // companion stream while the moments run, the L = 1 plane after them
      const size_t n1 = (size_t)full.nr * full.nt * full.ne;
      cudaStream_t cs = ctx->pipe_copy_streams[g];
      CK(cudaStreamWaitEvent(cs, ctx->pipe_fin_events[g], 0));
      const size_t ns2 = (size_t)full.nm * full.ns;
      for (int it = i0; it < i1; ++it) {
        const int slot = slot_of(it);
        int rc2 = RAMGPU_OK;
        if (f2[slot]) {
          rc2 = pipe_copy(ctx, f2[slot] + n1, full.f2 + (size_t)slot * n + n1, n - n1, pageable[slot], cs);
          if (!rc2) rc2 = pipe_copy(ctx, f2[slot], full.f2 + (size_t)slot * n, n1, pageable[slot], st);
        }
        if (!rc2 && ppert && ppert[slot])
          rc2 = pipe_copy(ctx, ppert[slot], full.ppert + (size_t)slot * nm2, nm2, pageable[ns2 + slot], st);
        if (!rc2 && ppart && ppart[slot])
          rc2 = pipe_copy(ctx, ppart[slot], full.ppart + (size_t)slot * nm2, nm2, pageable[2 * ns2 + slot], st);
        if (rc2) return rc2;
      }
      CK(cudaEventRecord(ctx->pipe_copy_done[g], cs));
      CK(cudaStreamWaitEvent(st, ctx->pipe_copy_done[g], 0));
    }
    if (trace) CK(cudaEventRecord(ctx->trace_ev[3 + 3 * g], st));
    CK(cudaEventRecord(ctx->pipe_events[2 * g + 1], st));
    CK(cudaStreamWaitEvent(main, ctx->pipe_events[2 * g + 1], 0));
  }
  return RAMGPU_OK;
}

extern "C" {

int ramgpu_create(const ramgpu_config* cfg, ramgpu_ctx** out) {
  if (!cfg || !out) return fail(nullptr, RAMGPU_ERR_ARG, "null argument");
  *out = nullptr;
  if (cfg->nr < 4 || cfg->nt < 5 || cfg->ne < 31 || cfg->npa < 5 || cfg->ns < 1 || cfg->n_members < 1)
    return fail(nullptr, RAMGPU_ERR_ARG,
                "grid too small: need NR>=4, NT>=5, NE>=31 (ANISCH bands), NPA>=5, NS>=1, members>=1");
  const long long ncell = (long long)cfg->nr * cfg->nt * cfg->ne * cfg->npa;
  if (ncell > (1LL << 40)) return fail(nullptr, RAMGPU_ERR_ARG, "grid too large");
  // non-persistent launches put the work item in gridDim.y (at most 65535)
  if ((long long)cfg->n_members * cfg->ns > 65535)
    return fail(nullptr, RAMGPU_ERR_ARG, "members x species above 65535 (the launch grid's item dimension)");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)
    return fail(nullptr, RAMGPU_ERR_CUDA, "no CUDA device");
  ramgpu_ctx* ctx = new ramgpu_ctx();
  ctx->cfg = *cfg;
  ctx->cfg.betalim = cfg->betalim > 2.0 ? 2.0 : (cfg->betalim < 1.0 ? 1.0 : cfg->betalim);
  Dev& d = ctx->d;
  memset(&d, 0, sizeof(d));
  d.nr = cfg->nr; d.nt = cfg->nt; d.ne = cfg->ne; d.npa = cfg->npa;
  d.ns = cfg->ns; d.nm = cfg->n_members; d.ncell = ncell; d.nf = cfg->nr + 1;
  d.betalim = ctx->cfg.betalim;
  const int blk0[4] = {128, 128, 64, 64};
  for (int w = 0; w < 4; ++w) { d.blk[w] = blk0[w]; d.pers[w] = 0; }
  d.mu_lanes = d.npa >= 12 ? 2 : 1;
  d.lw0 = 0;
  d.lw1 = d.npa;
  const size_t nr = d.nr, nt = d.nt, ne = d.ne, npa = d.npa, ns = d.ns, nm = d.nm, nf = d.nf;
  const size_t nijl = nr * nt * npa, nfield = nf * nt * npa, nslot = nm * ns;
  bool ok = true;
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) ok = false;
  ctx->own_stream = ok;
  d.lz = dalloc<double>(ctx, nf, &ok); d.rlz = dalloc<double>(ctx, nf, &ok);
  d.phi = dalloc<double>(ctx, nt, &ok);
  d.lr2 = dalloc<double>(ctx, nf, &ok); d.sinphi = dalloc<double>(ctx, nt, &ok);
  d.ekev = dalloc<double>(ctx, ne, &ok); d.ebnd = dalloc<double>(ctx, ne, &ok);
  d.we = dalloc<double>(ctx, ne, &ok); d.de = dalloc<double>(ctx, ne, &ok);
  d.mu = dalloc<double>(ctx, npa, &ok); d.dmu = dalloc<double>(ctx, npa, &ok);
  d.wmu = dalloc<double>(ctx, npa, &ok);
  d.upa_atm = dalloc<int>(ctx, nr, &ok); d.upa_mom = dalloc<int>(ctx, nr, &ok);
  d.mhde = dalloc<double>(ctx, ne, &ok); d.iwe = dalloc<double>(ctx, ne, &ok);
  d.ide = dalloc<double>(ctx, ne, &ok);
  d.mhdmu = dalloc<double>(ctx, npa, &ok); d.iwmu = dalloc<double>(ctx, npa, &ok);
  d.idmu = dalloc<double>(ctx, npa, &ok);
  d.bmhde = dalloc<double>(ctx, ne, &ok); d.bmhdmu = dalloc<double>(ctx, npa, &ok);
  d.grel = dalloc<double>(ctx, ns * ne, &ok); d.grbnd = dalloc<double>(ctx, ns * ne, &ok);
  d.vel = dalloc<double>(ctx, ns * ne, &ok); d.epp = dalloc<double>(ctx, ns * ne, &ok);
  d.rmas = dalloc<double>(ctx, ns, &ok);
  d.qs = dalloc<int>(ctx, ns, &ok); d.cex_kind = dalloc<int>(ctx, ns, &ok);
  d.ffactor = dalloc<double>(ctx, ns * nr * ne * npa, &ok);
  d.fnhs = dalloc<double>(ctx, nfield, &ok); d.fnis = dalloc<double>(ctx, nfield, &ok);
  d.bounhs = dalloc<double>(ctx, nfield, &ok); d.bounis = dalloc<double>(ctx, nfield, &ok);
  d.hdns = dalloc<double>(ctx, nfield, &ok); d.didt = dalloc<double>(ctx, nfield, &ok);
  d.dibndt = dalloc<double>(ctx, nfield, &ok);
  d.bnes = dalloc<double>(ctx, nf * nt, &ok); d.dbdt = dalloc<double>(ctx, nf * nt, &ok);
  d.eir = dalloc<double>(ctx, nf * nt, &ok); d.eip = dalloc<double>(ctx, nf * nt, &ok);
  d.outside = dalloc<int>(ctx, nr * nt, &ok);
  d.grt = dalloc<double>(ctx, nijl, &ok); d.gpt = dalloc<double>(ctx, nijl, &ok);
  d.gre = dalloc<double>(ctx, nijl, &ok); d.gpe = dalloc<double>(ctx, nijl, &ok);
  d.ze = dalloc<double>(ctx, nijl, &ok); d.wet = dalloc<double>(ctx, nijl, &ok);
  d.gmr = dalloc<double>(ctx, nijl, &ok); d.gmp = dalloc<double>(ctx, nijl, &ok);
  d.zm = dalloc<double>(ctx, nijl, &ok); d.hm = dalloc<double>(ctx, nijl, &ok);
  d.cmu0 = dalloc<double>(ctx, nijl, &ok); d.wm = dalloc<double>(ctx, nijl, &ok);
  d.cmudot = dalloc<double>(ctx, nijl, &ok);
  d.rho = dalloc<double>(ctx, nr * nt, &ok);
  d.mw_a = dalloc<double>(ctx, ns * npa * ne * nr, &ok);
  d.mw_be = dalloc<double>(ctx, npa * nt * nr, &ok); d.mw_ba = dalloc<double>(ctx, npa * nt * nr, &ok);
  d.mws_a = dalloc<double>(ctx, ns * ne * nr, &ok);
  d.mws_be = dalloc<double>(ctx, npa * nt * nr, &ok); d.mws_ba = dalloc<double>(ctx, npa * nt * nr, &ok);
  ctx->sep_dev = dalloc<unsigned long long>(ctx, 1, &ok);
  d.p4 = dalloc<double>(ctx, ns * ne, &ok);
  d.p2 = dalloc<double>(ctx, ns * ne * nr, &ok); d.edot = dalloc<double>(ctx, ns * ne * nr, &ok);
  d.eb = dalloc<double>(ctx, ns * ne, &ok); d.ek = dalloc<double>(ctx, ns * ne, &ok);
  d.kap = dalloc<double>(ctx, ns * 2, &ok);
  d.loss1 = dalloc<double>(ctx, ns * ncell, &ok); d.loss2 = dalloc<double>(ctx, ns * ncell, &ok);
  d.charge = dalloc<double>(ctx, ns * ncell, &ok); d.atm = dalloc<double>(ctx, ns * ncell, &ok);
  d.kp = dalloc<double>(ctx, nm, &ok); d.vt_mode = dalloc<int>(ctx, nm, &ok);
#ifdef RAMGPU_BOUNDS_CHECK
  d.bounds = dalloc<unsigned long long>(ctx, 3, &ok);  // the bounds log (zeroed)
#else
  d.bounds = nullptr;
#endif
  d.vt = dalloc<double>(ctx, nm * nf * nt, &ok);
  d.cr = dalloc<double>(ctx, nm * nr * nt, &ok); d.ca = dalloc<double>(ctx, nm * nr * nt, &ok);
  d.ue = dalloc<double>(ctx, nm * nijl, &ok); d.um = dalloc<double>(ctx, nm * nijl, &ok);
  d.drd1 = dalloc<double>(ctx, nm * nr * nt, &ok); d.dpd1 = dalloc<double>(ctx, nm * nr * nt, &ok);
  d.mij = dalloc<double>(ctx, 8 * nr * nt, &ok);
  d.f2 = dalloc<double>(ctx, nslot * ncell, &ok);
  d.fgeos = dalloc<double>(ctx, nslot * nt * ne * npa, &ok);
  d.plane_last = dalloc<double>(ctx, nslot * ne * npa, &ok);
  d.plane_has = dalloc<int>(ctx, nslot * ne * npa, &ok);
  d.plane_carry = dalloc<double>(ctx, nslot * ne * npa, &ok);
  d.plane_last_src = dalloc<int>(ctx, nslot * ne * npa, &ok);
  d.lam = dalloc<double>(ctx, nslot * ncell, &ok);
  d.gfg = dalloc<double>(ctx, nslot * nt * ne * npa, &ok);
  d.plane_carry_src = dalloc<int>(ctx, nslot * ne * npa, &ok);
  // CFL accumulators (4 per slot) followed by the clip counters (1 per
  // slot): one reset clears both
  d.cflq = dalloc<unsigned long long>(ctx, nslot * 5, &ok);
  d.clipq = d.cflq ? d.cflq + 4 * nslot : nullptr;
  d.count_clips = 0;
  d.mom_part = dalloc<double>(ctx, nslot * 4 * nr * nt * ne * 2, &ok);
  d.ppert = dalloc<double>(ctx, nslot * nr * nt, &ok);
  d.ppart = dalloc<double>(ctx, nslot * nr * nt, &ok);
  ctx->items_d = dalloc<int2>(ctx, nslot, &ok);
  ctx->losses = dalloc<double>(ctx, nslot * 6, &ok);
  ctx->sumrc_part = dalloc<double>(ctx, (size_t)kSumrcStages * nslot * kSumrcBlocks, &ok);
  ctx->status_d = dalloc<unsigned long long>(ctx, 5, &ok);
  ctx->stat_part = dalloc<double>(ctx, kF2StatBlocks, &ok);
  ctx->stat_mm = dalloc<unsigned long long>(ctx, 2, &ok);
  if (ok && cudaHostAlloc(&ctx->status_h, 5 * sizeof(unsigned long long), cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    ctx->status_h = nullptr;
    ok = false;
  }
  if (!ok) {
    ramgpu_destroy(ctx);
    return fail(nullptr, RAMGPU_ERR_NOMEM, "device allocation failed");
  }
  if (cudaDeviceSynchronize() != cudaSuccess) {
    ramgpu_destroy(ctx);
    return fail(nullptr, RAMGPU_ERR_CUDA, "device initialisation failed");
  }
  ctx->qs.assign(ns, 1);
  ctx->cex.assign(ns, 0);
  ctx->member_active.assign(nm, 1);
  ctx->member_species.assign(nm, std::vector<int>());
  for (size_t m = 0; m < nm; ++m)
    for (size_t s = 0; s < ns; ++s) ctx->member_species[m].push_back((int)s);
  std::vector<int> one(ns, 1);
  cudaMemcpy((void*)d.qs, one.data(), sizeof(int) * ns, cudaMemcpyHostToDevice);
  *out = ctx;
  return RAMGPU_OK;
}

int ramgpu_destroy(ramgpu_ctx* ctx) {
  if (!ctx) return RAMGPU_ERR_ARG;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  drop_graph(ctx);
  adj_free(ctx);
  cudaFree(ctx->d.coef);
  for (void* p : ctx->allocs) cudaFree(p);
  for (auto& sp : ctx->spans) { cudaEventDestroy(sp.a); cudaEventDestroy(sp.b); }
  for (cudaEvent_t e : ctx->ev_free) cudaEventDestroy(e);
  if (ctx->pipe_exec) cudaGraphExecDestroy(ctx->pipe_exec);
  if (ctx->ref_exec) cudaGraphExecDestroy(ctx->ref_exec);
  cudaFree(ctx->ref_stage);
  cudaFree(ctx->ref_ce_stage);
  for (cudaStream_t st : ctx->pipe_streams) cudaStreamDestroy(st);
  for (cudaEvent_t e : ctx->pipe_events) cudaEventDestroy(e);
  for (cudaEvent_t e : ctx->trace_ev) cudaEventDestroy(e);
  for (cudaStream_t st : ctx->pipe_copy_streams) cudaStreamDestroy(st);
  for (cudaEvent_t e : ctx->pipe_fin_events) cudaEventDestroy(e);
  for (cudaEvent_t e : ctx->pipe_copy_done) cudaEventDestroy(e);
  for (cudaEvent_t e : ctx->chunk_events) cudaEventDestroy(e);
  for (cudaEvent_t e : ctx->adj_events) cudaEventDestroy(e);
  if (ctx->adj_stream) cudaStreamDestroy(ctx->adj_stream);
  cudaFree(ctx->adj_shadow);
  cudaFree(ctx->adj_shadow_coef);
  cudaFree(ctx->adj_ring);
  for (cudaEvent_t e : ctx->adj_ring_events) cudaEventDestroy(e);
  if (ctx->status_h) cudaFreeHost(ctx->status_h);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return RAMGPU_OK;
}

int ramgpu_last_error(const ramgpu_ctx* ctx, char* buf, size_t len) {
  if (!buf || len == 0) return RAMGPU_ERR_ARG;
  const std::string& e = ctx ? ctx->err : g_create_error;
  snprintf(buf, len, "%s", e.c_str());
  return RAMGPU_OK;
}

int ramgpu_set_stream(ramgpu_ctx* ctx, void* stream) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  if (stream) {
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    ctx->own_stream = false;
    ctx->stream = (cudaStream_t)stream;
  }
  return RAMGPU_OK;
}

int ramgpu_set_species(ramgpu_ctx* ctx, int s, int charge, int cex_kind) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  if (s < 0 || s >= ctx->cfg.ns) return fail(ctx, RAMGPU_ERR_ARG, "species out of range");
  if (charge == 0) return fail(ctx, RAMGPU_ERR_ARG, "species charge must be nonzero");
  if (cex_kind < 0 || cex_kind > 3) return fail(ctx, RAMGPU_ERR_ARG, "unknown cex_kind");
  ctx->qs[s] = charge;
  ctx->cex[s] = cex_kind;
  CK(cudaMemcpy((void*)ctx->d.qs, ctx->qs.data(), sizeof(int) * ctx->cfg.ns, cudaMemcpyHostToDevice));
  CK(cudaMemcpy((void*)ctx->d.cex_kind, ctx->cex.data(), sizeof(int) * ctx->cfg.ns, cudaMemcpyHostToDevice));
  ctx->static_dirty = true;
  ctx->tables_dts = -1.0;
  return RAMGPU_OK;
}

int ramgpu_set_grid(ramgpu_ctx* ctx, const ramgpu_grid* g) {
  if (check_ctx(ctx) || !g) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  const ramgpu_grid& G = *g;
  if (!G.lz || !G.rlz || !G.phi || !G.ekev || !G.ebnd || !G.we || !G.de || !G.mu || !G.dmu ||
      !G.wmu || !G.upa || !G.rmas || !G.grel || !G.grbnd || !G.v || !G.epp || !G.ffactor)
    return fail(ctx, RAMGPU_ERR_ARG, "ramgpu_grid has a null array");
  Dev& d = ctx->d;
  const int nr = d.nr, nt = d.nt, ne = d.ne, npa = d.npa, ns = d.ns;
  d.dl1 = G.dl1; d.mdr = G.mdr; d.dphi = G.dphi; d.conf1 = G.conf1; d.conf2 = G.conf2;
  auto up = [&](const double* dst, const double* src, size_t n) {
    return cudaMemcpy((void*)dst, src, n * sizeof(double), cudaMemcpyHostToDevice);
  };
  CK(up(d.lz, G.lz, nr + 1)); CK(up(d.rlz, G.rlz, nr + 1)); CK(up(d.phi, G.phi, nt));
  {  // VOLS factors (src/ModRamRun.f90:51): (LZ(I)*RE)**2 and SIN(PHI(J)-PHIOFS), PHIOFS = 0
    std::vector<double> lr2(nr + 1), sp(nt);
    for (int i = 0; i <= nr; ++i) { const double lr = G.lz[i] * kRE; lr2[i] = lr * lr; }
    for (int j = 0; j < nt; ++j) sp[j] = sin(G.phi[j] - 0.0);
    CK(up(d.lr2, lr2.data(), nr + 1));
    CK(up(d.sinphi, sp.data(), nt));
  }
  CK(up(d.ekev, G.ekev, ne)); CK(up(d.ebnd, G.ebnd, ne)); CK(up(d.we, G.we, ne)); CK(up(d.de, G.de, ne));
  CK(up(d.mu, G.mu, npa)); CK(up(d.dmu, G.dmu, npa)); CK(up(d.wmu, G.wmu, npa));
  CK(up(d.rmas, G.rmas, ns));
  std::vector<int> ua(nr), um(nr);
  for (int i = 0; i < nr; ++i) {
    ua[i] = (int)G.upa[i];          // int(UPA(I)) in ATMOL
    um[i] = (int)(G.upa[i] - 1);    // int(UPA(I)-1) in ANISCH
    if (ua[i] < 2 || ua[i] > npa + 1) return fail(ctx, RAMGPU_ERR_ARG, "UPA out of range");
  }
  CK(cudaMemcpy((void*)d.upa_atm, ua.data(), sizeof(int) * nr, cudaMemcpyHostToDevice));
  CK(cudaMemcpy((void*)d.upa_mom, um.data(), sizeof(int) * nr, cudaMemcpyHostToDevice));
  std::vector<double> r1(ne), r2(ne), r3(ne), q1(npa), q2(npa), q3(npa);
  for (int k = 0; k < ne; ++k) { r1[k] = -0.5 / G.de[k]; r2[k] = 1.0 / G.we[k]; r3[k] = 1.0 / G.de[k]; }
  for (int l = 0; l < npa; ++l) { q1[l] = -0.5 / G.dmu[l]; q2[l] = 1.0 / G.wmu[l]; q3[l] = 1.0 / G.dmu[l]; }
  CK(up(d.mhde, r1.data(), ne)); CK(up(d.iwe, r2.data(), ne)); CK(up(d.ide, r3.data(), ne));
  CK(up(d.mhdmu, q1.data(), npa)); CK(up(d.iwmu, q2.data(), npa)); CK(up(d.idmu, q3.data(), npa));
  for (int k = 0; k < ne; ++k) r1[k] *= d.betalim;
  for (int l = 0; l < npa; ++l) q1[l] *= d.betalim;
  CK(up(d.bmhde, r1.data(), ne)); CK(up(d.bmhdmu, q1.data(), npa));
  // (NS,NE) Fortran -> [s][k]
  std::vector<double> t(ns * ne);
  auto tr2 = [&](const double* dst, const double* src) {
    for (int s = 0; s < ns; ++s)
      for (int k = 0; k < ne; ++k) t[s * ne + k] = src[(size_t)k * ns + s];
    return up(dst, t.data(), (size_t)ns * ne);
  };
  CK(tr2(d.grel, G.grel)); CK(tr2(d.grbnd, G.grbnd)); CK(tr2(d.vel, G.v)); CK(tr2(d.epp, G.epp));
  // FFACTOR(NS,NR,NE,NPA) -> [s][(L*NE+K)*NR+I]
  const size_t per = (size_t)nr * ne * npa;
  std::vector<double> ff(ns * per);
  for (size_t c = 0; c < per; ++c)
    for (int s = 0; s < ns; ++s) ff[(size_t)s * per + c] = G.ffactor[c * ns + s];
  CK(up(d.ffactor, ff.data(), ns * per));
  ctx->have_grid = true;
  ctx->field_dirty = true;
  return RAMGPU_OK;
}

int ramgpu_set_fields(ramgpu_ctx* ctx, const double* fnhs, const double* fnis, const double* bounhs,
                      const double* bounis, const double* hdns, const double* didt,
                      const double* dibndt, const double* bnes, const double* dbdt,
                      const double* eir, const double* eip, const int* outside_mgnp) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  if (!fnhs || !fnis || !bounhs || !bounis || !hdns || !didt || !dibndt || !bnes || !dbdt || !eir ||
      !eip || !outside_mgnp)
    return fail(ctx, RAMGPU_ERR_ARG, "null field array");
  Dev& d = ctx->d;
  const size_t nfield = (size_t)d.nf * d.nt * d.npa, n2 = (size_t)d.nf * d.nt;
  auto up = [&](const double* dst, const double* src, size_t n) {
    return cudaMemcpy((void*)dst, src, n * sizeof(double), cudaMemcpyHostToDevice);
  };
  CK(up(d.fnhs, fnhs, nfield)); CK(up(d.fnis, fnis, nfield)); CK(up(d.bounhs, bounhs, nfield));
  CK(up(d.bounis, bounis, nfield)); CK(up(d.hdns, hdns, nfield)); CK(up(d.didt, didt, nfield));
  CK(up(d.dibndt, dibndt, nfield));
  CK(up(d.bnes, bnes, n2)); CK(up(d.dbdt, dbdt, n2)); CK(up(d.eir, eir, n2)); CK(up(d.eip, eip, n2));
  CK(cudaMemcpy((void*)d.outside, outside_mgnp, sizeof(int) * d.nr * d.nt, cudaMemcpyHostToDevice));
  ctx->any_outside = 0;
  for (int i = 0; i < d.nr * d.nt; ++i)
    if (outside_mgnp[i] == 1) ctx->any_outside = 1;
  ctx->have_fields = true;
  ctx->field_dirty = true;
  return RAMGPU_OK;
}

int ramgpu_get_fields(ramgpu_ctx* ctx, double* fnhs, double* fnis, double* bounhs, double* bounis,
                      double* hdns, double* didt, double* dibndt, double* bnes, double* dbdt, double* eir,
                      double* eip) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  if (!ctx->have_fields) return fail(ctx, RAMGPU_ERR_STATE, "fields not set");
  Dev& d = ctx->d;
  const size_t nfield = (size_t)d.nf * d.nt * d.npa, n2 = (size_t)d.nf * d.nt;
  CK(cudaStreamSynchronize(ctx->stream));
  auto dn = [&](double* dst, const double* src, size_t n) {
    return dst ? cudaMemcpy(dst, src, n * sizeof(double), cudaMemcpyDefault) : cudaSuccess;
  };
  CK(dn(fnhs, d.fnhs, nfield)); CK(dn(fnis, d.fnis, nfield)); CK(dn(bounhs, d.bounhs, nfield));
  CK(dn(bounis, d.bounis, nfield)); CK(dn(hdns, d.hdns, nfield)); CK(dn(didt, d.didt, nfield));
  CK(dn(dibndt, d.dibndt, nfield));
  CK(dn(bnes, d.bnes, n2)); CK(dn(dbdt, d.dbdt, n2)); CK(dn(eir, d.eir, n2)); CK(dn(eip, d.eip, n2));
  return RAMGPU_OK;
}

int ramgpu_set_boundary(ramgpu_ctx* ctx, int member, int s, const double* fgeos_s) {
  if (check_ctx(ctx) || !fgeos_s) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  const size_t n = (size_t)ctx->d.nt * ctx->d.ne * ctx->d.npa;
  int m0 = member, m1 = member + 1;
  if (member < 0) { m0 = 0; m1 = ctx->cfg.n_members; }
  for (int m = m0; m < m1; ++m) {
    if (int rc = check_ms(ctx, m, s)) return rc;
    CK(cudaMemcpy(ctx->d.fgeos + (size_t)(m * ctx->d.ns + s) * n, fgeos_s, n * sizeof(double),
                  cudaMemcpyDefault));
  }
  return RAMGPU_OK;
}

int ramgpu_set_pa_diffusion(ramgpu_ctx* ctx, int s, const double* daa) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  if (s < 0 || s >= ctx->cfg.ns) return fail(ctx, RAMGPU_ERR_ARG, "species out of range");
  Dev& d = ctx->d;
  if (ctx->pd_on_h.empty()) ctx->pd_on_h.assign(d.ns, 0);
  if (daa && !ctx->pd_alloc) {
    bool ok = true;
    d.pd_on = dalloc<int>(ctx, d.ns, &ok);
    d.pd_d = dalloc<double>(ctx, (size_t)d.ns * d.ncell, &ok);
    d.pd_gn = dalloc<double>(ctx, (size_t)d.ns * d.ncell, &ok);
    d.pd_inv = dalloc<double>(ctx, (size_t)d.ns * d.ncell, &ok);
    d.pd_rl = dalloc<double>(ctx, (size_t)d.ns * d.ncell, &ok);
    d.pd_fac = dalloc<double>(ctx, (size_t)d.nr * d.nt * d.npa, &ok);
    d.pd_ifac = dalloc<double>(ctx, (size_t)d.nr * d.nt * d.npa, &ok);
    if (!ok) return fail(ctx, RAMGPU_ERR_NOMEM, "pitch-angle diffusion tables: device allocation failed");
    ctx->pd_alloc = true;
  }
  if (daa)
    CK(cudaMemcpy((void*)(d.pd_d + (size_t)s * d.ncell), daa, sizeof(double) * d.ncell, cudaMemcpyDefault));
  ctx->pd_on_h[s] = daa ? 1 : 0;
  if (ctx->pd_alloc)
    CK(cudaMemcpy((void*)d.pd_on, ctx->pd_on_h.data(), sizeof(int) * d.ns, cudaMemcpyHostToDevice));
  ctx->pd_dirty = true;
  ctx->shape_version += 1;  // the ram_run launch sequence changes: recapture the graph
  return RAMGPU_OK;
}

int ramgpu_set_potential(ramgpu_ctx* ctx, int member, const double* vt) {
  if (check_ctx(ctx) || !vt) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (int rc = check_ms(ctx, member, 0)) return rc;
  const size_t n = (size_t)ctx->d.nf * ctx->d.nt;
  CK(cudaMemcpy(ctx->d.vt + (size_t)member * n, vt, n * sizeof(double), cudaMemcpyHostToDevice));
  int zero = 0;
  CK(cudaMemcpy(ctx->d.vt_mode + member, &zero, sizeof(int), cudaMemcpyHostToDevice));
  return RAMGPU_OK;
}

// Kp (VOLS mode) of members m0..m1-1, written in stream order by a tiny
// kernel so that the host neither waits nor keeps a staging buffer alive.
__global__ void k_set_kp(double* kp, int* vt_mode, int m0, int m1, double v) {
  const int m = m0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (m < m1) { kp[m] = v; vt_mode[m] = 1; }
}

int ramgpu_set_kp(ramgpu_ctx* ctx, int member, double kp) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  if (!isfinite(kp)) return fail(ctx, RAMGPU_ERR_ARG, "kp must be finite");
  int m0 = member, m1 = member + 1;
  if (member < 0) { m0 = 0; m1 = ctx->cfg.n_members; }
  if (int rc = check_ms(ctx, m0, 0)) return rc;
  if (int rc = check_ms(ctx, m1 - 1, 0)) return rc;
  k_set_kp<<<(m1 - m0 + 127) / 128, 128, 0, ctx->stream>>>(ctx->d.kp, ctx->d.vt_mode, m0, m1, kp);
  ctx->launches += 1;
  CKL("set_kp");
  return RAMGPU_OK;
}

int ramgpu_set_kp_all(ramgpu_ctx* ctx, const double* kp) {
  if (check_ctx(ctx) || !kp) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  const int nm = ctx->cfg.n_members;
  for (int m = 0; m < nm; ++m)
    if (!isfinite(kp[m])) return fail(ctx, RAMGPU_ERR_ARG, "kp must be finite");
  std::vector<int> one(nm, 1);
  CK(cudaMemcpyAsync(ctx->d.kp, kp, sizeof(double) * nm, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d.vt_mode, one.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return RAMGPU_OK;
}

int ramgpu_set_member_species(ramgpu_ctx* ctx, int member, int n, const int* list) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  if (int rc = check_ms(ctx, member, 0)) return rc;
  if (n < 0 || n > ctx->cfg.ns || (n > 0 && !list)) return fail(ctx, RAMGPU_ERR_ARG, "bad species list");
  std::vector<int> v;
  for (int i = 0; i < n; ++i) {
    if (list[i] < 0 || list[i] >= ctx->cfg.ns) return fail(ctx, RAMGPU_ERR_ARG, "species out of range");
    for (int x : v)
      if (x == list[i]) return fail(ctx, RAMGPU_ERR_ARG, "duplicate species in list");
    v.push_back(list[i]);
  }
  ctx->member_species[member] = v;
  ctx->items_dirty = true;
  return RAMGPU_OK;
}

int ramgpu_set_member_active(ramgpu_ctx* ctx, int member, int active) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  if (int rc = check_ms(ctx, member, 0)) return rc;
  ctx->member_active[member] = active ? 1 : 0;
  ctx->items_dirty = true;
  return RAMGPU_OK;
}

int ramgpu_upload_f2(ramgpu_ctx* ctx, int member, int s, const double* f2_s) {
  if (check_ctx(ctx) || !f2_s) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (int rc = check_ms(ctx, member, s)) return rc;
  const size_t n = ctx->d.ncell;
  CK(cudaMemcpyAsync(ctx->d.f2 + (size_t)(member * ctx->d.ns + s) * n, f2_s, n * sizeof(double),
                     cudaMemcpyDefault, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return RAMGPU_OK;
}

int ramgpu_download_f2(ramgpu_ctx* ctx, int member, int s, double* f2_s) {
  if (check_ctx(ctx) || !f2_s) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (int rc = check_ms(ctx, member, s)) return rc;
  const size_t n = ctx->d.ncell;
  CK(cudaMemcpyAsync(f2_s, ctx->d.f2 + (size_t)(member * ctx->d.ns + s) * n, n * sizeof(double),
                     cudaMemcpyDefault, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return RAMGPU_OK;
}

int ramgpu_upload_f2_async(ramgpu_ctx* ctx, int member, int s, const double* f2_s) {
  if (check_ctx(ctx) || !f2_s) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (int rc = check_ms(ctx, member, s)) return rc;
  const size_t n = ctx->d.ncell;
  CK(cudaMemcpyAsync(ctx->d.f2 + (size_t)(member * ctx->d.ns + s) * n, f2_s, n * sizeof(double),
                     cudaMemcpyDefault, ctx->stream));
  return RAMGPU_OK;
}

int ramgpu_download_f2_async(ramgpu_ctx* ctx, int member, int s, double* f2_s) {
  if (check_ctx(ctx) || !f2_s) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (int rc = check_ms(ctx, member, s)) return rc;
  const size_t n = ctx->d.ncell;
  CK(cudaMemcpyAsync(f2_s, ctx->d.f2 + (size_t)(member * ctx->d.ns + s) * n, n * sizeof(double),
                     cudaMemcpyDefault, ctx->stream));
  return RAMGPU_OK;
}

int ramgpu_moments_async(ramgpu_ctx* ctx, int member, int s, double* ppert, double* ppart) {
  if (check_ctx(ctx) || !ppert || !ppart) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (int rc = check_ms(ctx, member, s)) return rc;
  const size_t n = (size_t)ctx->d.nr * ctx->d.nt, o = (size_t)(member * ctx->d.ns + s) * n;
  CK(cudaMemcpyAsync(ppert, ctx->d.ppert + o, n * sizeof(double), cudaMemcpyDefault, ctx->stream));
  CK(cudaMemcpyAsync(ppart, ctx->d.ppart + o, n * sizeof(double), cudaMemcpyDefault, ctx->stream));
  return RAMGPU_OK;
}

int ramgpu_synchronize(ramgpu_ctx* ctx) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  return RAMGPU_OK;
}

// ---------------------------------------------- F2 in the reference layout
// How the device reaches a caller's array: the device address kernels may
// read or write it through, or null when only the copy engines can move it
// (pageable memory without a coherent host link).  Looked up on every call,
// so memory freed and reallocated at the same address is classified anew.
static double* reach(const void* p, bool pma) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    at.type = cudaMemoryTypeUnregistered;
  }
  if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) return (double*)p;
  if (at.type == cudaMemoryTypeHost) return (double*)at.devicePointer;
  return pma ? (double*)p : nullptr;
}

static int ensure_nsm(ramgpu_ctx* ctx, int* pma) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (!ctx->nsm) CK(cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, dev));
  *pma = 0;
  CK(cudaDeviceGetAttribute(pma, cudaDevAttrPageableMemoryAccess, dev));
  return RAMGPU_OK;
}

static int ensure_stage(ramgpu_ctx* ctx) {
  if (!ctx->ref_stage) CK(cudaMalloc(&ctx->ref_stage, sizeof(double) * ctx->d.ns * ctx->d.ncell));
  return RAMGPU_OK;
}

// A member's interleaved array (NS values per cell, ncell cells; r its
// device address or null) into its NS slot blocks (stride apart).
static int ref_in(ramgpu_ctx* ctx, const double* host, const double* r, double* slots, long long stride,
                  long long ncell, cudaStream_t st) {
  const int ns = ctx->d.ns;
  if (!r) {
    if (int rc = ensure_stage(ctx)) return rc;
    CK(cudaMemcpyAsync(ctx->ref_stage, host, sizeof(double) * ns * ncell, cudaMemcpyHostToDevice, st));
    r = ctx->ref_stage;
  }
  launch_ref_gather(r, slots, ns, stride, 0, ncell, ctx->nsm, st);
  ctx->launches += 1;
  CKL("reference-layout gather");
  return RAMGPU_OK;
}

// Cells [c0, c1) of a member's NS slot blocks into its interleaved array
// (w its device address, or null: through the staging buffer).
static int ref_out(ramgpu_ctx* ctx, double* host, double* w, const double* slots, long long stride, long long c0,
                   long long c1, cudaStream_t st) {
  const int ns = ctx->d.ns;
  if (!w) {
    if (int rc = ensure_stage(ctx)) return rc;
    launch_ref_scatter(slots, ctx->ref_stage, ns, stride, c0, c1, ctx->nsm, st);
    ctx->launches += 1;
    CKL("reference-layout scatter");
    CK(cudaMemcpyAsync(host + c0 * ns, ctx->ref_stage + c0 * ns, sizeof(double) * ns * (c1 - c0),
                       cudaMemcpyDeviceToHost, st));
    return RAMGPU_OK;
  }
  launch_ref_scatter(slots, w, ns, stride, c0, c1, ctx->nsm, st);
  ctx->launches += 1;
  CKL("reference-layout scatter");
  return RAMGPU_OK;
}

int ramgpu_upload_f2_all(ramgpu_ctx* ctx, int member, const double* f2) {
  if (check_ctx(ctx) || !f2) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (int rc = check_ms(ctx, member, 0)) return rc;
  int pma = 0;
  if (int rc = ensure_nsm(ctx, &pma)) return rc;
  const long long n = ctx->d.ncell;
  const double* r = ctx->ref_force_stage ? nullptr : reach(f2, pma);
  if (int rc = ref_in(ctx, f2, r, ctx->d.f2 + (size_t)member * ctx->d.ns * n, n, n, ctx->stream))
    return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  return RAMGPU_OK;
}

int ramgpu_download_f2_all(ramgpu_ctx* ctx, int member, double* f2) {
  if (check_ctx(ctx) || !f2) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (int rc = check_ms(ctx, member, 0)) return rc;
  int pma = 0;
  if (int rc = ensure_nsm(ctx, &pma)) return rc;
  const long long n = ctx->d.ncell;
  double* w = ctx->ref_force_stage ? nullptr : reach(f2, pma);
  if (int rc = ref_out(ctx, f2, w, ctx->d.f2 + (size_t)member * ctx->d.ns * n, n, 0, n, ctx->stream))
    return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  return RAMGPU_OK;
}

int ramgpu_f2_device_ptr(ramgpu_ctx* ctx, int member, int s, double** dptr) {
  if (check_ctx(ctx) || !dptr) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (int rc = check_ms(ctx, member, s)) return rc;
  *dptr = ctx->d.f2 + (size_t)(member * ctx->d.ns + s) * ctx->d.ncell;
  return RAMGPU_OK;
}

int ramgpu_ram_run_async(ramgpu_ctx* ctx, double dts) {
  NvtxRange range_("ramgpu_ram_run_async");
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  return enqueue_ram_run(ctx, dts);
}

int ramgpu_set_pipeline_groups(ramgpu_ctx* ctx, int groups) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  if (groups < 1 || groups > 8) return fail(ctx, RAMGPU_ERR_ARG, "groups must be 1..8");
  ctx->pipe_groups = groups;
  return RAMGPU_OK;
}

int ramgpu_pipeline_groups(const ramgpu_ctx* ctx) {
  return ctx ? ctx->pipe_groups : 0;
}

int ramgpu_set_step_groups(ramgpu_ctx* ctx, int groups) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  if (groups < 1 || groups > 8) return fail(ctx, RAMGPU_ERR_ARG, "groups must be 1..8");
  if (groups != ctx->step_groups) ctx->shape_version += 1;  // ram_run's graph holds the groups
  ctx->step_groups = groups;
  return RAMGPU_OK;
}

int ramgpu_step_groups(const ramgpu_ctx* ctx) {
  return ctx ? ctx->step_groups : 0;
}


// Status word in the page-locked copy -> struct; RAMGPU_ERR_NUMERIC when
// a value was not finite.
static int status_out(ramgpu_ctx* ctx, ramgpu_status* st) {
  const unsigned long long* w = ctx->status_h;
  int fm = -1, fs = -1;
  if (w[3] != ~0ULL && w[3] < ctx->items_h.size()) {
    fm = ctx->items_h[w[3]].x;
    fs = ctx->items_h[w[3]].y;
  }
  if (st) {
    st->f2_nonfinite = (long long)w[0];
    st->moments_nonfinite = (long long)w[1];
    st->cfl_over = (long long)w[2];
    st->clips = (long long)w[4];
    st->first_member = fm;
    st->first_species = fs;
  }
  if (w[0] | w[1]) {
    char msg[160];
    snprintf(msg, sizeof msg, "non-finite values: %llu F2 cells, %llu moments (first in member %d, species %d)",
             w[0], w[1], fm, fs);
    return fail(ctx, RAMGPU_ERR_NUMERIC, msg);
  }
  return RAMGPU_OK;
}

int ramgpu_ram_run_host(ramgpu_ctx* ctx, double dts, double* const* f2, double* const* ppert,
                        double* const* ppart) {
  NvtxRange range_("ramgpu_ram_run_host");
  if (check_ctx(ctx) || !f2) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  int rc = prepare(ctx, dts);
  if (rc) return rc;
  ctx->last_dts = dts;
  const int nit = ctx->d.nitems;
  if (nit == 0) return RAMGPU_OK;
  // the loss bookkeeping indexes its partial sums by list position: one group
  const bool timing = ctx->timing;
  ctx->timing = false;
  const int G = clamp_groups(ctx, ctx->pipe_groups);
  if ((rc = ensure_group_streams(ctx, G))) {
    ctx->timing = timing;
    return rc;
  }
  // Pageable host buffers are moved by the SMs where the device reaches
  // pageable memory (a coherent host link), else by blocking copies.  A
  // graph holds the buffers' addresses, so it is kept per buffer set, and
  // not built when a copy would come from pageable memory through the copy
  // engines (not capturable).
  const int nslot = ctx->d.nm * ctx->d.ns;
  std::vector<const void*> key;
  bool capturable = ctx->graph_on && !ctx->pipe_trace;  // a traced call runs direct
  if (ctx->pipe_trace) {
    while ((int)ctx->trace_ev.size() < 1 + 3 * G) {
      cudaEvent_t e = nullptr;
      CK(cudaEventCreate(&e));
      ctx->trace_ev.push_back(e);
    }
    ctx->trace_ms.clear();
  }
  for (double* const* tab : {f2, ppert, ppart})
    for (int k = 0; k < nslot; ++k) key.push_back(tab ? (const void*)tab[k] : nullptr);
  // Every pointer is classified on every call (cudaPointerGetAttributes is
  // cheap next to the call): a buffer freed and reallocated at the same
  // address may have changed from page-locked to pageable.  A changed
  // classification drops the graph built on the old one.
  {
    int dev = 0, pma = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, dev);
    std::vector<char> cls;
    bool engine = false;
    cls.reserve(key.size());
    for (const void* p : key) {
      bool pg = false;
      if (p) {
        cudaPointerAttributes at{};
        if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
          cudaGetLastError();
          at.type = cudaMemoryTypeUnregistered;
        }
        pg = at.type == cudaMemoryTypeUnregistered;
        if (pg && !pma) engine = true;
      }
      cls.push_back(pg && pma ? 1 : 0);
    }
    if (key != ctx->cls_key || cls != ctx->cls_pageable || engine != ctx->cls_engine_pageable) {
      if (ctx->pipe_exec) cudaGraphExecDestroy(ctx->pipe_exec);
      ctx->pipe_exec = nullptr;
      ctx->cls_pageable = cls;
      ctx->cls_engine_pageable = engine;
      ctx->cls_key = key;
    }
  }
  const std::vector<char>& pageable = ctx->cls_pageable;
  if (ctx->cls_engine_pageable) capturable = false;
  const int C = ctx->cls_engine_pageable ? 0 : chunk_count(ctx, 0);
  // the copies of planes [l0, l1) of every item with a host array
  const long long plane = (long long)ctx->d.nr * ctx->d.nt * ctx->d.ne;
  const size_t nm2 = (size_t)ctx->d.nr * ctx->d.nt, ns2 = (size_t)nslot;
  auto h_in = [&](int, cudaStream_t st, int l0, int l1) {
    for (size_t i = 0; i < ctx->items_h.size(); ++i) {
      const int slot = ctx->items_h[i].x * ctx->d.ns + ctx->items_h[i].y;
      if (f2[slot])
        if (int r = pipe_copy(ctx, ctx->d.f2 + (size_t)slot * ctx->d.ncell + l0 * plane, f2[slot] + l0 * plane,
                              (size_t)(l1 - l0) * plane, pageable[slot], st))
          return r;
    }
    return RAMGPU_OK;
  };
  auto h_out = [&](int, cudaStream_t st, int l0, int l1) {
    const int a = std::max(l0, 1);  // the L = 1 plane goes back after ANISCH
    for (size_t i = 0; i < ctx->items_h.size() && a < l1; ++i) {
      const int slot = ctx->items_h[i].x * ctx->d.ns + ctx->items_h[i].y;
      if (f2[slot])
        if (int r = pipe_copy(ctx, f2[slot] + a * plane, ctx->d.f2 + (size_t)slot * ctx->d.ncell + a * plane,
                              (size_t)(l1 - a) * plane, pageable[slot], st))
          return r;
    }
    return RAMGPU_OK;
  };
  auto h_tail = [&](cudaStream_t st) {
    for (size_t i = 0; i < ctx->items_h.size(); ++i) {
      const int slot = ctx->items_h[i].x * ctx->d.ns + ctx->items_h[i].y;
      int r = RAMGPU_OK;
      if (f2[slot])
        r = pipe_copy(ctx, f2[slot], ctx->d.f2 + (size_t)slot * ctx->d.ncell, (size_t)plane, pageable[slot], st);
      if (!r && ppert && ppert[slot])
        r = pipe_copy(ctx, ppert[slot], ctx->d.ppert + (size_t)slot * nm2, nm2, pageable[ns2 + slot], st);
      if (!r && ppart && ppart[slot])
        r = pipe_copy(ctx, ppart[slot], ctx->d.ppart + (size_t)slot * nm2, nm2, pageable[2 * ns2 + slot], st);
      if (r) return r;
    }
    return RAMGPU_OK;
  };
  auto enqueue = [&]() {
    if (C > 0) return enqueue_chunked(ctx, dts, C, h_in, h_out, h_tail);
    int r = enqueue_pipeline(ctx, dts, f2, ppert, ppart, G, pageable);
    if (!r && ctx->check_on) r = enqueue_status(ctx);
    return r;
  };
  if (!capturable) {
    rc = enqueue();
  } else {
    if (!ctx->pipe_exec || ctx->pipe_key != key || ctx->pipe_dts != dts || ctx->pipe_items != ctx->items_version ||
        ctx->pipe_flags != ctx->d.flags || ctx->pipe_shape != ctx->shape_version || ctx->pipe_g != G + 16 * C) {
      if (ctx->pipe_exec) cudaGraphExecDestroy(ctx->pipe_exec);
      ctx->pipe_exec = nullptr;
      cudaGraph_t g = nullptr;
      const long long l0 = ctx->launches;
      CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
      rc = enqueue();
      cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
      ctx->pipe_launches = ctx->launches - l0;  // kernels per replay
      ctx->launches = l0;
      if (rc) {
        if (g) cudaGraphDestroy(g);
        ctx->timing = timing;
        return rc;
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&ctx->pipe_exec, g, 0);
      if (g) cudaGraphDestroy(g);
      if (e != cudaSuccess) {
        ctx->pipe_exec = nullptr;
        ctx->timing = timing;
        return cuda_fail(ctx, e, "pipeline graph");
      }
      ctx->pipe_key = key;
      ctx->pipe_dts = dts;
      ctx->pipe_items = ctx->items_version;
      ctx->pipe_flags = ctx->d.flags;
      ctx->pipe_shape = ctx->shape_version;
      ctx->pipe_g = G + 16 * C;
    }
    CK(cudaGraphLaunch(ctx->pipe_exec, ctx->stream));
    ctx->launches += ctx->pipe_launches;
  }
  ctx->timing = timing;
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->pipe_trace) {
    for (int k = 1; k < 1 + 3 * G; ++k) {
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, ctx->trace_ev[0], ctx->trace_ev[k]));
      ctx->trace_ms.push_back(ms);
    }
  }
  if (ctx->check_on) {
    ctx->status_valid = true;
    return status_out(ctx, nullptr);
  }
  return RAMGPU_OK;
}

int ramgpu_set_pipeline_trace(ramgpu_ctx* ctx, int enable) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  ctx->pipe_trace = enable != 0;
  ctx->trace_ms.clear();
  return RAMGPU_OK;
}

int ramgpu_pipeline_trace(ramgpu_ctx* ctx, int* groups, float* ms) {
  if (check_ctx(ctx) || !groups || !ms) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (ctx->trace_ms.empty()) return fail(ctx, RAMGPU_ERR_STATE, "no traced ramgpu_ram_run_host call");
  *groups = (int)ctx->trace_ms.size() / 3;
  for (size_t k = 0; k < ctx->trace_ms.size(); ++k) ms[k] = ctx->trace_ms[k];
  return RAMGPU_OK;
}

// One member's arrays in the reference layout and their device addresses
// (null: staged through the copy engines).
struct RefMem {
  double *f2 = nullptr, *pe = nullptr, *pa = nullptr;
  double *f2r = nullptr, *per = nullptr, *par = nullptr;
  double* f2ce = nullptr;  // device staging of a page-locked F2 moved by the copy engines
};

// ramgpu_ram_run_ref's work: F2 of every member gathered from the
// reference layout, the step over the item groups, then F2 scattered back:
// its L >= 2 planes on a companion stream as soon as every group's closing
// mask is done (they are final then), while the moments run; the L = 1
// plane, which ANISCH's side effect rewrites, and the moments after them.
// staged: some array is reachable only by the copy engines; everything
// then runs in stream order on the context's stream.
static int enqueue_ref(ramgpu_ctx* ctx, double dts, const std::vector<RefMem>& mem, bool staged, int G) {
  const Dev full = ctx->d;
  const int ns = full.ns, nm = full.nm, nit = full.nitems;
  const long long n = full.ncell, nm2 = (long long)full.nr * full.nt, n1 = (long long)full.nr * full.nt * full.ne;
  const cudaStream_t main = ctx->stream;
  int rc = RAMGPU_OK;
  for (int m = 0; m < nm; ++m)
    if (mem[m].f2 && (rc = ref_in(ctx, mem[m].f2, mem[m].f2r, full.f2 + (size_t)m * ns * n, n, n, main))) return rc;
  if ((rc = enqueue_tables(ctx, dts))) return rc;
  CK(cudaMemsetAsync(full.cflq, 0, sizeof(unsigned long long) * 5 * full.nm * full.ns, main));
  cudaEvent_t ev_tab = ctx->pipe_events[2 * G + 1];
  CK(cudaEventRecord(ev_tab, main));
  for (int g = 0; g < G; ++g) {
    const int i0 = (int)((long long)nit * g / G), i1 = (int)((long long)nit * (g + 1) / G);
    cudaStream_t st = G > 1 ? ctx->pipe_streams[g] : main;
    if (G > 1) CK(cudaStreamWaitEvent(st, ev_tab, 0));
    ctx->stream = st;
    ctx->d.items = full.items + i0;
    ctx->d.nitems = i1 - i0;
    ctx->d.item0 = i0;
    ctx->finish_hook = staged ? nullptr : ctx->pipe_fin_events[g];
    rc = enqueue_sweeps(ctx, dts, false);
    ctx->finish_hook = nullptr;
    ctx->d = full;
    ctx->stream = main;
    if (rc) return rc;
    if (G > 1) {
      CK(cudaEventRecord(ctx->pipe_events[2 * g + 1], st));
      CK(cudaStreamWaitEvent(main, ctx->pipe_events[2 * g + 1], 0));
    }
  }
  const long long f2_from = staged ? 0 : n1;
  if (!staged) {
    cudaStream_t cs = ctx->pipe_copy_streams[0];
    for (int g = 0; g < G; ++g) CK(cudaStreamWaitEvent(cs, ctx->pipe_fin_events[g], 0));
    for (int m = 0; m < nm; ++m)
      if (mem[m].f2 && (rc = ref_out(ctx, mem[m].f2, mem[m].f2r, full.f2 + (size_t)m * ns * n, n, n1, n, cs)))
        return rc;
    CK(cudaEventRecord(ctx->pipe_copy_done[0], cs));
  }
  for (int m = 0; m < nm; ++m) {
    if (mem[m].f2 && (rc = ref_out(ctx, mem[m].f2, mem[m].f2r, full.f2 + (size_t)m * ns * n, n, 0,
                                   staged ? n : f2_from, main)))
      return rc;
    if (mem[m].pe && (rc = ref_out(ctx, mem[m].pe, mem[m].per, full.ppert + (size_t)m * ns * nm2, nm2, 0, nm2, main)))
      return rc;
    if (mem[m].pa && (rc = ref_out(ctx, mem[m].pa, mem[m].par, full.ppart + (size_t)m * ns * nm2, nm2, 0, nm2, main)))
      return rc;
  }
  if (!staged) CK(cudaStreamWaitEvent(main, ctx->pipe_copy_done[0], 0));
  if (ctx->check_on) rc = enqueue_status(ctx);
  return rc;
}

int ramgpu_ram_run_ref(ramgpu_ctx* ctx, double dts, double* const* f2, double* const* ppert, double* const* ppart) {
  NvtxRange range_("ramgpu_ram_run_ref");
  if (check_ctx(ctx) || !f2) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  int rc = prepare(ctx, dts);
  if (rc) return rc;
  ctx->last_dts = dts;
  if (ctx->d.nitems == 0) return RAMGPU_OK;
  int pma = 0;
  if ((rc = ensure_nsm(ctx, &pma))) return rc;
  const int nm = ctx->d.nm;
  std::vector<RefMem> mem(nm);
  std::vector<const void*> key;
  bool staged = false;
  for (int m = 0; m < nm; ++m) {
    RefMem& r = mem[m];
    r.f2 = f2[m];
    r.pe = ppert ? ppert[m] : nullptr;
    r.pa = ppart ? ppart[m] : nullptr;
    const bool fs = ctx->ref_force_stage;
    if (r.f2) staged |= !(r.f2r = fs ? nullptr : reach(r.f2, pma));
    if (r.f2 && r.f2r && ctx->ref_ce) {
      cudaPointerAttributes at{};
      if (cudaPointerGetAttributes(&at, r.f2) != cudaSuccess) cudaGetLastError();
      if (at.type == cudaMemoryTypeHost) {
        const size_t need = sizeof(double) * (size_t)nm * ctx->d.ns * ctx->d.ncell;
        if (ctx->ref_ce_bytes < need) {
          cudaFree(ctx->ref_ce_stage);
          ctx->ref_ce_stage = nullptr;
          ctx->ref_ce_bytes = 0;
          CK(cudaMalloc(&ctx->ref_ce_stage, need));
          ctx->ref_ce_bytes = need;
        }
        r.f2ce = ctx->ref_ce_stage + (size_t)m * ctx->d.ns * ctx->d.ncell;
      }
    }
    if (r.pe) staged |= !(r.per = fs ? nullptr : reach(r.pe, pma));
    if (r.pa) staged |= !(r.par = fs ? nullptr : reach(r.pa, pma));
    for (const void* p : {(const void*)r.f2, (const void*)r.pe, (const void*)r.pa, (const void*)r.f2r,
                          (const void*)r.per, (const void*)r.par, (const void*)r.f2ce})
      key.push_back(p);
  }
  const bool timing = ctx->timing;
  ctx->timing = false;  // one call, one set of streams: no per-kernel events
  const int G = clamp_groups(ctx, ctx->step_groups);
  if ((rc = ensure_group_streams(ctx, G))) {
    ctx->timing = timing;
    return rc;
  }
  const int C = staged ? 0 : chunk_count(ctx, 4);
  const long long plane = (long long)ctx->d.nr * ctx->d.nt * ctx->d.ne;
  const int ns = ctx->d.ns;
  const long long n = ctx->d.ncell, nm2 = (long long)ctx->d.nr * ctx->d.nt;
  auto r_in = [&](int, cudaStream_t st, int l0, int l1) {
    for (int m = 0; m < nm; ++m)
      if (mem[m].f2) {
        const double* src = mem[m].f2r;
        if (mem[m].f2ce) {  // the chunk by the copy engines, then gathered on the device
          const size_t o = (size_t)l0 * plane * ns, b = sizeof(double) * (size_t)(l1 - l0) * plane * ns;
          CK(cudaMemcpyAsync(mem[m].f2ce + o, mem[m].f2 + o, b, cudaMemcpyHostToDevice, st));
          src = mem[m].f2ce;
        }
        launch_ref_gather(src, ctx->d.f2 + (size_t)m * ns * n, ns, n, l0 * plane, l1 * plane, ctx->nsm, st);
        ctx->launches += 1;
      }
    CKL("reference-layout gather");
    return RAMGPU_OK;
  };
  auto r_out = [&](int, cudaStream_t st, int l0, int l1) {
    const int a = std::max(l0, 1);  // the L = 1 plane goes back after ANISCH
    for (int m = 0; m < nm && a < l1; ++m)
      if (mem[m].f2) {
        double* dst = mem[m].f2ce ? mem[m].f2ce : mem[m].f2r;
        launch_ref_scatter(ctx->d.f2 + (size_t)m * ns * n, dst, ns, n, a * plane, l1 * plane, ctx->nsm, st);
        ctx->launches += 1;
        if (mem[m].f2ce) {
          const size_t o = (size_t)a * plane * ns, b = sizeof(double) * (size_t)(l1 - a) * plane * ns;
          CK(cudaMemcpyAsync(mem[m].f2 + o, mem[m].f2ce + o, b, cudaMemcpyDeviceToHost, st));
        }
      }
    CKL("reference-layout scatter");
    return RAMGPU_OK;
  };
  auto r_tail = [&](cudaStream_t st) {
    for (int m = 0; m < nm; ++m) {
      int r = RAMGPU_OK;
      if (mem[m].f2) r = ref_out(ctx, mem[m].f2, mem[m].f2r, ctx->d.f2 + (size_t)m * ns * n, n, 0, plane, st);
      if (!r && mem[m].pe) r = ref_out(ctx, mem[m].pe, mem[m].per, ctx->d.ppert + (size_t)m * ns * nm2, nm2, 0, nm2, st);
      if (!r && mem[m].pa) r = ref_out(ctx, mem[m].pa, mem[m].par, ctx->d.ppart + (size_t)m * ns * nm2, nm2, 0, nm2, st);
      if (r) return r;
    }
    return RAMGPU_OK;
  };
  auto enqueue = [&]() {
    return C > 0 ? enqueue_chunked(ctx, dts, C, r_in, r_out, r_tail) : enqueue_ref(ctx, dts, mem, staged, G);
  };
  if (!ctx->graph_on || staged) {
    rc = enqueue();
  } else {
    if (!ctx->ref_exec || ctx->ref_key != key || ctx->ref_dts != dts || ctx->ref_items != ctx->items_version ||
        ctx->ref_flags != ctx->d.flags || ctx->ref_shape != ctx->shape_version || ctx->ref_g != G + 16 * C) {
      if (ctx->ref_exec) cudaGraphExecDestroy(ctx->ref_exec);
      ctx->ref_exec = nullptr;
      cudaGraph_t g = nullptr;
      const long long l0 = ctx->launches;
      CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
      rc = enqueue();
      cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
      ctx->ref_launches = ctx->launches - l0;
      ctx->launches = l0;
      if (!rc && e == cudaSuccess) e = cudaGraphInstantiate(&ctx->ref_exec, g, 0);
      if (g) cudaGraphDestroy(g);
      if (!rc && e != cudaSuccess) {
        ctx->ref_exec = nullptr;
        rc = cuda_fail(ctx, e, "reference-layout graph");
      }
      if (!rc) {
        ctx->ref_key = key;
        ctx->ref_dts = dts;
        ctx->ref_items = ctx->items_version;
        ctx->ref_flags = ctx->d.flags;
        ctx->ref_shape = ctx->shape_version;
        ctx->ref_g = G + 16 * C;
      }
    }
    if (!rc) {
      CK(cudaGraphLaunch(ctx->ref_exec, ctx->stream));
      ctx->launches += ctx->ref_launches;
    }
  }
  ctx->timing = timing;
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->check_on) {
    ctx->status_valid = true;
    return status_out(ctx, nullptr);
  }
  return RAMGPU_OK;
}

int ramgpu_set_pipeline_chunks(ramgpu_ctx* ctx, int chunks) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  if (chunks < -1 || chunks > 8) return fail(ctx, RAMGPU_ERR_ARG, "chunks must be -1..8");
  ctx->pipe_chunks = chunks;
  return RAMGPU_OK;
}

int ramgpu_set_ref_staging(ramgpu_ctx* ctx, int force) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  if (force < 0 || force > 2) return fail(ctx, RAMGPU_ERR_ARG, "force: 0, 1 or 2");
  ctx->ref_force_stage = force == 1;
  ctx->ref_ce = force == 2;
  return RAMGPU_OK;
}

int ramgpu_ram_run(ramgpu_ctx* ctx, double dts) {
  NvtxRange range_("ramgpu_ram_run");
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  int rc = enqueue_ram_run(ctx, dts);
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->check_on && ctx->d.nitems) {
    ctx->status_valid = true;
    return status_out(ctx, nullptr);
  }
  return RAMGPU_OK;
}

int ramgpu_check(ramgpu_ctx* ctx, ramgpu_status* st) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  // the pass reads the grid's DMU (the DRIFTMU CFL floor)
  if (!ctx->have_grid) return fail(ctx, RAMGPU_ERR_STATE, "ramgpu_set_grid must be called first");
  if (ctx->items_dirty)
    if (int rc = rebuild_items(ctx)) return rc;
  if (int rc = enqueue_status(ctx)) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->status_valid = true;
  return status_out(ctx, st);
}

int ramgpu_set_check(ramgpu_ctx* ctx, int enable) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  if ((enable != 0) != ctx->check_on) ctx->shape_version += 1;  // the graphs hold the pass
  ctx->check_on = enable != 0;
  ctx->d.count_clips = ctx->check_on ? 1 : 0;  // the sweeps count clip events meanwhile
  return RAMGPU_OK;
}

int ramgpu_last_status(ramgpu_ctx* ctx, ramgpu_status* st) {
  if (check_ctx(ctx) || !st) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (!ctx->status_valid && !ctx->check_on) return fail(ctx, RAMGPU_ERR_STATE, "no status pass has run");
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->status_valid = true;
  return status_out(ctx, st);
}

int ramgpu_half_step(ramgpu_ctx* ctx, double dts, int order) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  if (order != 0 && order != 1) return fail(ctx, RAMGPU_ERR_ARG, "order must be 0 or 1");
  int rc = prepare(ctx, dts);
  if (rc) return rc;
  ctx->last_dts = dts;
  if (ctx->d.nitems == 0) return RAMGPU_OK;
  launch_member_coef(ctx->d, dts, ctx->stream);
  launch_ghost(ctx->d, ctx->stream);
  ctx->launches += 3;
  CKL("member tables");
  if (order == 0) rc = enqueue_forward(ctx, dts, true, ctx->d.loss1);
  else rc = enqueue_reverse(ctx, dts, true, ctx->d.loss1, false);
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  return RAMGPU_OK;
}

int ramgpu_apply_op(ramgpu_ctx* ctx, double dts, int op, int cfl) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  if (op < 0 || op > 7) return fail(ctx, RAMGPU_ERR_ARG, "unknown op");
  int rc = prepare(ctx, dts);
  if (rc) return rc;
  ctx->last_dts = dts;
  if (ctx->d.nitems == 0) return RAMGPU_OK;
  launch_member_coef(ctx->d, dts, ctx->stream);
  launch_ghost(ctx->d, ctx->stream);
  ctx->launches += 3;
  if (cfl) CK(cudaMemsetAsync(ctx->d.cflq, 0, sizeof(unsigned long long) * 5 * ctx->d.nm * ctx->d.ns, ctx->stream));
  switch (op) {
    case 0: launch_sweep_r(ctx->d, dts, cfl != 0, ctx->stream); break;
    case 1: launch_sweep_p(ctx->d, dts, cfl != 0, ctx->stream); break;
    case 2: launch_sweep_e(ctx->d, dts, cfl != 0, ctx->stream); break;
    case 3: launch_sweep_mu(ctx->d, dts, cfl != 0, 0, nullptr, ctx->stream); break;
    case 4: launch_loss_apply(ctx->d, ctx->d.charge, ctx->stream); break;
    case 5: launch_loss_apply(ctx->d, ctx->d.atm, ctx->stream); break;
    case 6: launch_moments(ctx->d, ctx->stream); ctx->launches += 1; break;
    case 7: launch_padif(ctx->d, nullptr, ctx->stream); break;
    default: break;
  }
  ctx->launches += 1;
  CKL("apply_op");
  CK(cudaStreamSynchronize(ctx->stream));
  return RAMGPU_OK;
}

int ramgpu_moments(ramgpu_ctx* ctx, int member, int s, double* ppert, double* ppart) {
  if (check_ctx(ctx) || !ppert || !ppart) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (int rc = check_ms(ctx, member, s)) return rc;
  const size_t n = (size_t)ctx->d.nr * ctx->d.nt, o = (size_t)(member * ctx->d.ns + s) * n;
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpy(ppert, ctx->d.ppert + o, n * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(ppart, ctx->d.ppart + o, n * sizeof(double), cudaMemcpyDeviceToHost));
  return RAMGPU_OK;
}

int ramgpu_f2_stats(ramgpu_ctx* ctx, int member, int s, double* f2_min, double* f2_max, double* content) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  if (int rc = check_ms(ctx, member, s)) return rc;
  if (!ctx->have_grid) return fail(ctx, RAMGPU_ERR_STATE, "grid not set");
  launch_f2_stats(ctx->d, (long long)member * ctx->d.ns + s, ctx->stat_part, ctx->stat_mm, ctx->stream);
  ctx->launches += 1;
  CKL("f2 statistics");
  double part[kF2StatBlocks];
  unsigned long long mm[2];
  CK(cudaMemcpyAsync(part, ctx->stat_part, sizeof part, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(mm, ctx->stat_mm, sizeof mm, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  double sum = 0.0;
  for (int b = 0; b < kF2StatBlocks; ++b) sum += part[b];  // fixed order
  if (f2_min) *f2_min = f2_stats_key_value(mm[0]);
  if (f2_max) *f2_max = f2_stats_key_value(mm[1]);
  if (content) *content = sum;
  return RAMGPU_OK;
}

int ramgpu_flux(ramgpu_ctx* ctx, int member, int s, double* flux_s) {
  if (check_ctx(ctx) || !flux_s) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (int rc = check_ms(ctx, member, s)) return rc;
  if (!ctx->have_grid || !ctx->have_fields) return fail(ctx, RAMGPU_ERR_STATE, "grid/fields not set");
  const size_t n = ctx->d.ncell;
  double* tmp = nullptr;
  CK(cudaMalloc(&tmp, n * sizeof(double)));
  launch_flux(ctx->d, member * ctx->d.ns + s, s, tmp, ctx->stream);
  ctx->launches += 1;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(flux_s, tmp, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(tmp);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "flux");
  return RAMGPU_OK;
}

int ramgpu_cfl(ramgpu_ctx* ctx, int member, int s, double* out5) {
  if (check_ctx(ctx) || !out5) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (int rc = check_ms(ctx, member, s)) return rc;
  const int ns = ctx->d.ns;
  std::vector<unsigned long long> q(4 * ns);
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpy(q.data(), ctx->d.cflq + (size_t)member * ns * 4, sizeof(unsigned long long) * 4 * ns,
                cudaMemcpyDeviceToHost));
  const double fr = ctx->cfg.fraccfl * ctx->last_dts;
  const double init[4] = {100000.0, 100000.0, 10000.0, 10000.0};
  // smallest 1/DMU(NPA) floor term of DRIFTMU's L = NPA face (CDriftMu = 0 there)
  double dmu_n = 0.0;
  CK(cudaMemcpy(&dmu_n, ctx->d.dmu + ctx->d.npa - 1, sizeof(double), cudaMemcpyDeviceToHost));
  double dtsnext = 1e300;
  for (int sp : ctx->member_species[member]) {
    for (int w = 0; w < 4; ++w) {
      double qq;
      unsigned long long b = q[sp * 4 + w];
      memcpy(&qq, &b, sizeof(double));
      if (w == 3 && b != 0ULL) qq = fmax(qq, 1E-32 / dmu_n);
      double dt = b ? fmin(init[w], fr / qq) : init[w];
      if (sp == s) out5[w] = dt;
      dtsnext = fmin(dtsnext, dt);
    }
  }
  if (ctx->member_species[member].empty()) dtsnext = ctx->cfg.dtsmin;
  out5[4] = fmax(dtsnext, ctx->cfg.dtsmin);
  return RAMGPU_OK;
}

int ramgpu_losses(ramgpu_ctx* ctx, int member, int s, double* out4) {
  if (check_ctx(ctx) || !out4) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (int rc = check_ms(ctx, member, s)) return rc;
  double v[6];
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpy(v, ctx->losses + (size_t)(member * ctx->d.ns + s) * 6, sizeof(v), cudaMemcpyDeviceToHost));
  for (int i = 0; i < 4; ++i) out4[i] = v[i];
  return RAMGPU_OK;
}

int ramgpu_loss_wae(ramgpu_ctx* ctx, int member, int s, double* lswae) {
  if (check_ctx(ctx) || !lswae) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (int rc = check_ms(ctx, member, s)) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpy(lswae, ctx->losses + (size_t)(member * ctx->d.ns + s) * 6 + 5, sizeof(double),
                cudaMemcpyDeviceToHost));
  return RAMGPU_OK;
}

int ramgpu_reset_losses(ramgpu_ctx* ctx) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  CK(cudaMemsetAsync(ctx->losses, 0, sizeof(double) * 6 * ctx->d.nm * ctx->d.ns, ctx->stream));
  // baseline SETRC of the current state (the ENOLD of the next SUMRC)
  if (ctx->have_grid && ctx->have_fields) {
    if (ctx->items_dirty) {
      int rc = rebuild_items(ctx);
      if (rc) return rc;
    }
    if (ctx->d.nitems > 0) {
      int rc = sumrc_stage(ctx, kSumrcStages - 1, -1);
      if (rc) return rc;
    }
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return RAMGPU_OK;
}

int ramgpu_bounds_report(ramgpu_ctx* ctx, int* checked, long long* failures, int* check, long long* value) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  unsigned long long log[3] = {0ULL, 0ULL, 0ULL};
  if (ctx->d.bounds) {
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(log, ctx->d.bounds, sizeof(log), cudaMemcpyDeviceToHost));
  }
  if (checked) *checked = ctx->d.bounds ? 1 : 0;
  if (failures) *failures = (long long)log[0];
  if (check) *check = log[0] ? (int)log[1] - 1 : 0;
  if (value) *value = (long long)log[2];
  return RAMGPU_OK;
}

long long ramgpu_launch_count(const ramgpu_ctx* ctx) { return ctx ? ctx->launches : -1; }

int ramgpu_selftest_arith(long long n, unsigned long long seed, long long* mismatches) {
  if (!mismatches || n < 0) return RAMGPU_ERR_ARG;
  unsigned long long* bad = nullptr;
  if (cudaMalloc(&bad, sizeof(unsigned long long)) != cudaSuccess) return RAMGPU_ERR_CUDA;
  cudaError_t e = cudaMemset(bad, 0, sizeof(unsigned long long));
  if (e == cudaSuccess) {
    launch_selftest_mul(n, seed, bad, 0);
    e = cudaGetLastError();
  }
  unsigned long long h = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&h, bad, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(bad);
  if (e != cudaSuccess) return RAMGPU_ERR_CUDA;
  *mismatches = (long long)h;
  return RAMGPU_OK;
}

int ramgpu_probe_fp64(double* lane_ops_per_s) {
  if (!lane_ops_per_s) return RAMGPU_ERR_ARG;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return fail(nullptr, RAMGPU_ERR_CUDA, "no CUDA device");
  const int block = 256, grid = nsm * 8, iters = 4096;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * block * grid) != cudaSuccess)
    return fail(nullptr, RAMGPU_ERR_NOMEM, "probe allocation failed");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int r = 0; r < 4; ++r) {
    cudaEventRecord(e0, 0);
    k_probe_dfma<<<grid, block>>>(out, 0.999999, 1e-7, iters);
    cudaEventRecord(e1, 0);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (r > 0 && ms < best) best = ms;
  }
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return fail(nullptr, RAMGPU_ERR_CUDA, cudaGetErrorString(e));
  *lane_ops_per_s = 8.0 * iters * (double)block * grid / (best * 1e-3);
  return RAMGPU_OK;
}

int ramgpu_probe_l2(double* bytes_per_s) {
  if (!bytes_per_s) return RAMGPU_ERR_ARG;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return fail(nullptr, RAMGPU_ERR_CUDA, "no CUDA device");
  const size_t bytes = 32u << 20;  // within either die's half of L2
  const int block = 256, grid = nsm * 4, passes = 200;
  void* buf = nullptr;
  unsigned* out = nullptr;
  if (cudaMalloc(&buf, bytes) != cudaSuccess || cudaMalloc(&out, sizeof(unsigned) * block * grid) != cudaSuccess) {
    cudaFree(buf);
    cudaGetLastError();
    return fail(nullptr, RAMGPU_ERR_NOMEM, "probe allocation failed");
  }
  cudaMemset(buf, 1, bytes);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int r = 0; r < 4; ++r) {  // the first run brings the buffer into L2
    cudaEventRecord(e0, 0);
    k_probe_l2<<<grid, block>>>((const uint4*)buf, (long long)(bytes / 16), passes, out);
    cudaEventRecord(e1, 0);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (r > 0 && ms < best) best = ms;
  }
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  cudaFree(out);
  if (e != cudaSuccess) return fail(nullptr, RAMGPU_ERR_CUDA, cudaGetErrorString(e));
  *bytes_per_s = (double)passes * (double)bytes / (best * 1e-3);
  return RAMGPU_OK;
}

int ramgpu_set_coef_store(ramgpu_ctx* ctx, int mask) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  if (mask < 0 || mask > 15) return fail(ctx, RAMGPU_ERR_ARG, "mask: bits 0-3 (R, P, E, MU)");
  if ((unsigned)mask == ctx->coef_mask) return RAMGPU_OK;
  ctx->coef_mask = (unsigned)mask;
  CK(cudaStreamSynchronize(ctx->stream));
  cudaFree(ctx->d.coef);  // reallocated for the new set by the next step
  ctx->d.coef = nullptr;
  ctx->d.coef_items = 0;
  ctx->shape_version += 1;
  return RAMGPU_OK;
}

int ramgpu_set_graph(ramgpu_ctx* ctx, int enable) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  ctx->graph_on = enable != 0;
  if (!ctx->graph_on) drop_graph(ctx);
  // the host pipeline's graph and pointer classification are rebuilt on
  // the next ramgpu_ram_run_host
  if (ctx->pipe_exec) cudaGraphExecDestroy(ctx->pipe_exec);
  ctx->pipe_exec = nullptr;
  ctx->cls_key.clear();
  if (ctx->ref_exec) cudaGraphExecDestroy(ctx->ref_exec);
  ctx->ref_exec = nullptr;
  return RAMGPU_OK;
}

int ramgpu_set_launch_shape(ramgpu_ctx* ctx, int sweep, int threads, int persistent_ctas) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  if (sweep < 0 || sweep > 3) return fail(ctx, RAMGPU_ERR_ARG, "sweep must be 0..3");
  if (threads < 32 || threads > 256 || (threads % 32)) return fail(ctx, RAMGPU_ERR_ARG, "threads must be 32..256, multiple of 32");
  if (persistent_ctas < 0) return fail(ctx, RAMGPU_ERR_ARG, "persistent_ctas must be >= 0");
  ctx->d.blk[sweep] = threads;
  ctx->d.pers[sweep] = persistent_ctas;
  ctx->shape_version += 1;
  return RAMGPU_OK;
}

int ramgpu_set_mu_lanes(ramgpu_ctx* ctx, int lanes) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  if (lanes != 1 && lanes != 2 && lanes != 4) return fail(ctx, RAMGPU_ERR_ARG, "lanes must be 1, 2 or 4");
  if (lanes == 2 && ctx->d.npa < 12) return fail(ctx, RAMGPU_ERR_ARG, "two lanes per line need NPA >= 12");
  if (lanes == 4 && ctx->d.npa < 24) return fail(ctx, RAMGPU_ERR_ARG, "four lanes per line need NPA >= 24");
  ctx->d.mu_lanes = lanes;
  ctx->shape_version += 1;
  return RAMGPU_OK;
}

int ramgpu_get_launch_shape(ramgpu_ctx* ctx, int* threads4, int* persistent4) {
  if (check_ctx(ctx) || !threads4 || !persistent4) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  for (int w = 0; w < 4; ++w) { threads4[w] = ctx->d.blk[w]; persistent4[w] = ctx->d.pers[w]; }
  return RAMGPU_OK;
}

int ramgpu_autotune(ramgpu_ctx* ctx, double dts, int reps, double* best_ms4) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  if (reps < 1) reps = 3;
  int rc = prepare(ctx, dts);
  if (rc) return rc;
  if (ctx->d.nitems == 0) return RAMGPU_OK;
  launch_member_coef(ctx->d, dts, ctx->stream);
  launch_ghost(ctx->d, ctx->stream);
  ctx->launches += 3;
  // the trials advance F2: keep a copy of every active slot and restore it
  const size_t ncell = ctx->d.ncell;
  double* snap = nullptr;
  CK(cudaMalloc(&snap, sizeof(double) * ncell * ctx->items_h.size()));
  for (size_t i = 0; i < ctx->items_h.size(); ++i) {
    const int slot = ctx->items_h[i].x * ctx->d.ns + ctx->items_h[i].y;
    CK(cudaMemcpyAsync(snap + i * ncell, ctx->d.f2 + (size_t)slot * ncell, sizeof(double) * ncell,
                       cudaMemcpyDeviceToDevice, ctx->stream));
  }
  int nsm = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int cand_blk[4] = {32, 64, 128, 256};
  for (int w = 0; w < 4; ++w) {
    ctx->tune_plain_ms[w] = ctx->tune_pers_ms[w] = 0.0;
    float best = 1e30f;
    int bb = ctx->d.blk[w], bp = ctx->d.pers[w], bl = ctx->d.mu_lanes;
    // DRIFTMU: 4, 2 and 1 lanes per line, as NPA allows
    const int nlanes = w != 3 ? 1 : (ctx->d.npa >= 24 ? 4 : (ctx->d.npa >= 12 ? 2 : 1));
    for (int lanes = nlanes; lanes >= 1; lanes /= 2)
    for (int ib = 0; ib < 4; ++ib) {
      for (int persist = 0; persist < 2; ++persist) {
        const int blk = cand_blk[ib];
        if (w == 3) ctx->d.mu_lanes = lanes;
        int pc = 0;
        if (persist) {
          const int per_sm = sweep_max_blocks_per_sm(w, blk);
          if (per_sm <= 0) continue;
          pc = per_sm * nsm;
        }
        ctx->d.blk[w] = blk;
        ctx->d.pers[w] = pc;
        // one trial = a whole ram_run step (direct launches) with this
        // sweep's shape and the others' current ones: the sweeps interact
        // through L2 and the SM schedule, so isolated sweeps mislead; best
        // of reps after one warm-up step
        float tbest = 1e30f;
        for (int r = 0; r <= reps; ++r) {
          cudaEventRecord(e0, ctx->stream);
          if (int rc2 = enqueue_body(ctx, dts)) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            cudaFree(snap);
            return rc2;
          }
          cudaEventRecord(e1, ctx->stream);
          cudaEventSynchronize(e1);
          float ms = 0.f;
          cudaEventElapsedTime(&ms, e0, e1);
          if (r > 0 && ms < tbest) tbest = ms;
        }
        if (tbest < best) { best = tbest; bb = blk; bp = pc; bl = ctx->d.mu_lanes; }
        double& rec = persist ? ctx->tune_pers_ms[w] : ctx->tune_plain_ms[w];
        if (rec == 0.0 || tbest < rec) rec = tbest;
      }
    }
    ctx->d.blk[w] = bb;
    ctx->d.pers[w] = bp;
    if (w == 3) ctx->d.mu_lanes = bl;
    if (best_ms4) best_ms4[w] = best;
  }
  // then the number of concurrent item groups, 1, 2, 4 or 8 (at most one
  // per item), on the chosen shapes
  if (!(ctx->cfg.flags & RAMGPU_FLAG_LOSSES)) {
    float best = 1e30f;
    int bg = ctx->step_groups;
    for (int G = 1; G <= 8 && G <= ctx->d.nitems; G *= 2) {
      ctx->step_groups = G;
      float tbest = 1e30f;
      for (int r = 0; r <= reps; ++r) {
        cudaEventRecord(e0, ctx->stream);
        if (int rc2 = enqueue_body(ctx, dts)) {
          cudaEventDestroy(e0);
          cudaEventDestroy(e1);
          cudaFree(snap);
          return rc2;
        }
        cudaEventRecord(e1, ctx->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r > 0 && ms < tbest) tbest = ms;
      }
      if (tbest < best) { best = tbest; bg = G; }
    }
    ctx->step_groups = bg;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (size_t i = 0; i < ctx->items_h.size(); ++i) {
    const int slot = ctx->items_h[i].x * ctx->d.ns + ctx->items_h[i].y;
    cudaMemcpyAsync(ctx->d.f2 + (size_t)slot * ncell, snap + i * ncell, sizeof(double) * ncell,
                    cudaMemcpyDeviceToDevice, ctx->stream);
  }
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  cudaFree(snap);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "autotune");
  ctx->shape_version += 1;
  return RAMGPU_OK;
}

int ramgpu_autotune_trials(ramgpu_ctx* ctx, double* plain_ms4, double* persistent_ms4) {
  if (check_ctx(ctx) || !plain_ms4 || !persistent_ms4) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  for (int w = 0; w < 4; ++w) {
    plain_ms4[w] = ctx->tune_plain_ms[w];
    persistent_ms4[w] = ctx->tune_pers_ms[w];
  }
  return RAMGPU_OK;
}


// ------------------------------------------------------------- snapshots
// The evolving state of a context in one file (the counterpart of RAM's
// write_restart/read_restart, src/ModRamRestart.f90:12,386, for the state
// this library owns; grid and field tables are inputs and are not saved).
// Layout, little-endian:
//   header (128 bytes): "RAMGPUS1", version 1, header bytes 128, NR, NT,
//     NE, NPA, NS, members, flags, 0, the caller's time [s], payload bytes,
//     checksum, zero padding;
//   payload: per member {species mask, active, VT mode (int32), 0 (int32),
//     Kp, VT(NR+1,NT)} then per (member, species) slot {F2(NR,NT,NE,NPA),
//     FGEOS(NT,NE,NPA), PPERT(NR,NT), PPART(NR,NT)} (doubles).
// The checksum is FNV-1a over the payload's 64-bit words.
namespace {
constexpr char kSnapMagic[8] = {'R', 'A', 'M', 'G', 'P', 'U', 'S', '1'};
constexpr uint64_t kFnvOffset = 1469598103934665603ULL, kFnvPrime = 1099511628211ULL;
struct SnapHeader {
  char magic[8];
  uint32_t version, header_bytes;
  int32_t nr, nt, ne, npa, ns, nm;
  uint32_t flags, pad0;
  double time;
  uint64_t payload_bytes, checksum;
  unsigned char pad[128 - 8 - 8 - 24 - 8 - 8 - 16];
};
static_assert(sizeof(SnapHeader) == 128, "snapshot header is 128 bytes");
uint64_t fnv_words(uint64_t h, const void* p, size_t nbytes) {
  const unsigned char* b = (const unsigned char*)p;
  for (size_t i = 0; i + 8 <= nbytes; i += 8) {
    uint64_t w;
    memcpy(&w, b + i, 8);
    h = (h ^ w) * kFnvPrime;
  }
  return h;
}
uint64_t snap_payload_bytes(long long nr, long long nt, long long ne, long long npa, long long ns, long long nm) {
  const long long member = 16 + 8 + 8 * (nr + 1) * nt;
  const long long slot = 8 * (nr * nt * ne * npa + nt * ne * npa + 2 * nr * nt);
  return (uint64_t)(nm * member + nm * ns * slot);
}
// Reads the header and checks the payload against its checksum.
int snap_verify(FILE* f, SnapHeader* h, std::string* why) {
  if (fread(h, sizeof(*h), 1, f) != 1) { *why = "short header"; return RAMGPU_ERR_IO; }
  if (memcmp(h->magic, kSnapMagic, 8) != 0 || h->version != 1 || h->header_bytes != 128) {
    *why = "not a ramgpu snapshot (magic, version or header size)";
    return RAMGPU_ERR_IO;
  }
  if (h->nr < 1 || h->nt < 1 || h->ne < 1 || h->npa < 1 || h->ns < 1 || h->nm < 1 ||
      h->payload_bytes != snap_payload_bytes(h->nr, h->nt, h->ne, h->npa, h->ns, h->nm)) {
    *why = "snapshot sizes inconsistent";
    return RAMGPU_ERR_IO;
  }
  std::vector<unsigned char> buf(1 << 24);
  uint64_t left = h->payload_bytes, hs = kFnvOffset;
  while (left > 0) {
    const size_t n = (size_t)std::min<uint64_t>(left, buf.size());
    if (fread(buf.data(), 1, n, f) != n) { *why = "snapshot payload truncated"; return RAMGPU_ERR_IO; }
    hs = fnv_words(hs, buf.data(), n);
    left -= n;
  }
  if (hs != h->checksum) { *why = "snapshot checksum mismatch"; return RAMGPU_ERR_IO; }
  return RAMGPU_OK;
}
}  // namespace

int ramgpu_snapshot_info(const char* path, ramgpu_snapshot_info_t* info) {
  if (!path) return fail(nullptr, RAMGPU_ERR_ARG, "null path");
  FILE* f = fopen(path, "rb");
  if (!f) return fail(nullptr, RAMGPU_ERR_IO, std::string("cannot open ") + path);
  SnapHeader h{};
  std::string why;
  const int rc = snap_verify(f, &h, &why);
  fclose(f);
  if (rc) return fail(nullptr, rc, why);
  if (info) {
    info->nr = h.nr; info->nt = h.nt; info->ne = h.ne; info->npa = h.npa; info->ns = h.ns; info->n_members = h.nm;
    info->flags = h.flags;
    info->time = h.time;
  }
  return RAMGPU_OK;
}

int ramgpu_save_state(ramgpu_ctx* ctx, const char* path, double time) {
  if (check_ctx(ctx) || !path) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  NvtxRange range_("ramgpu_save_state");
  const Dev& d = ctx->d;
  const int nm = d.nm, ns = d.ns;
  const size_t ncell = d.ncell, nfg = (size_t)d.nt * d.ne * d.npa, nm2 = (size_t)d.nr * d.nt;
  const size_t nvt = (size_t)d.nf * d.nt;
  CK(cudaStreamSynchronize(ctx->stream));
  SnapHeader h{};
  memcpy(h.magic, kSnapMagic, 8);
  h.version = 1; h.header_bytes = 128;
  h.nr = d.nr; h.nt = d.nt; h.ne = d.ne; h.npa = d.npa; h.ns = ns; h.nm = nm;
  h.flags = ctx->cfg.flags;
  h.time = time;
  h.payload_bytes = snap_payload_bytes(d.nr, d.nt, d.ne, d.npa, ns, nm);
  FILE* f = fopen(path, "wb");
  if (!f) return fail(ctx, RAMGPU_ERR_IO, std::string("cannot create ") + path);
  bool ok = fwrite(&h, sizeof(h), 1, f) == 1;
  uint64_t hs = kFnvOffset;
  auto put = [&](const void* p, size_t n) {
    if (ok) ok = fwrite(p, 1, n, f) == n;
    hs = fnv_words(hs, p, n);
  };
  std::vector<double> kp(nm), vt(nvt), buf(ncell);
  std::vector<int> mode(nm);
  cudaError_t e = cudaMemcpy(kp.data(), d.kp, sizeof(double) * nm, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(mode.data(), d.vt_mode, sizeof(int) * nm, cudaMemcpyDeviceToHost);
  for (int m = 0; m < nm && e == cudaSuccess; ++m) {
    int32_t rec[4] = {0, ctx->member_active[m], mode[m], 0};
    for (int sp : ctx->member_species[m]) rec[0] |= 1 << sp;
    put(rec, sizeof(rec));
    put(&kp[m], sizeof(double));
    e = cudaMemcpy(vt.data(), d.vt + (size_t)m * nvt, sizeof(double) * nvt, cudaMemcpyDeviceToHost);
    put(vt.data(), sizeof(double) * nvt);
  }
  for (int slot = 0; slot < nm * ns && e == cudaSuccess; ++slot) {
    const struct { const double* src; size_t n; } parts[4] = {
        {d.f2 + (size_t)slot * ncell, ncell}, {d.fgeos + (size_t)slot * nfg, nfg},
        {d.ppert + (size_t)slot * nm2, nm2}, {d.ppart + (size_t)slot * nm2, nm2}};
    for (const auto& q : parts) {
      if (e == cudaSuccess) e = cudaMemcpy(buf.data(), q.src, sizeof(double) * q.n, cudaMemcpyDeviceToHost);
      put(buf.data(), sizeof(double) * q.n);
    }
  }
  h.checksum = hs;
  if (ok) ok = fseek(f, 0, SEEK_SET) == 0 && fwrite(&h, sizeof(h), 1, f) == 1;
  ok = (fclose(f) == 0) && ok;
  if (e != cudaSuccess) return cuda_fail(ctx, e, "ramgpu_save_state");
  if (!ok) return fail(ctx, RAMGPU_ERR_IO, std::string("write failed: ") + path);
  return RAMGPU_OK;
}

int ramgpu_load_state(ramgpu_ctx* ctx, const char* path, double* time) {
  if (check_ctx(ctx) || !path) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  NvtxRange range_("ramgpu_load_state");
  Dev& d = ctx->d;
  const int nm = d.nm, ns = d.ns;
  const size_t ncell = d.ncell, nfg = (size_t)d.nt * d.ne * d.npa, nm2 = (size_t)d.nr * d.nt;
  const size_t nvt = (size_t)d.nf * d.nt;
  FILE* f = fopen(path, "rb");
  if (!f) return fail(ctx, RAMGPU_ERR_IO, std::string("cannot open ") + path);
  // the whole file is checked before anything on the device changes
  SnapHeader h{};
  std::string why;
  if (int rc = snap_verify(f, &h, &why)) {
    fclose(f);
    return fail(ctx, rc, why);
  }
  if (h.nr != d.nr || h.nt != d.nt || h.ne != d.ne || h.npa != d.npa || h.ns != ns || h.nm != nm) {
    fclose(f);
    return fail(ctx, RAMGPU_ERR_ARG, "snapshot dimensions differ from the context's");
  }
  fseek(f, sizeof(SnapHeader), SEEK_SET);
  bool ok = true;
  auto get = [&](void* p, size_t n) { if (ok) ok = fread(p, 1, n, f) == n; };
  std::vector<double> vt(nvt), buf(ncell);
  int rc = RAMGPU_OK;
  for (int m = 0; m < nm && ok && !rc; ++m) {
    int32_t rec[4];
    double kp = 0.0;
    get(rec, sizeof(rec));
    get(&kp, sizeof(kp));
    get(vt.data(), sizeof(double) * nvt);
    if (!ok) break;
    std::vector<int> list;
    for (int sp = 0; sp < ns; ++sp)
      if (rec[0] & (1 << sp)) list.push_back(sp);
    rc = ramgpu_set_member_species(ctx, m, (int)list.size(), list.data());
    if (!rc) rc = ramgpu_set_member_active(ctx, m, rec[1]);
    if (!rc) rc = rec[2] ? ramgpu_set_kp(ctx, m, kp) : ramgpu_set_potential(ctx, m, vt.data());
    if (!rc && rec[2]) {
      // the potential of the last call, as saved (VOLS recomputes it from Kp anyway)
      CK(cudaMemcpyAsync(d.vt + (size_t)m * nvt, vt.data(), sizeof(double) * nvt, cudaMemcpyHostToDevice,
                         ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
    }
  }
  for (int slot = 0; slot < nm * ns && ok && !rc; ++slot) {
    double* const dst[4] = {d.f2 + (size_t)slot * ncell, d.fgeos + (size_t)slot * nfg, d.ppert + (size_t)slot * nm2,
                            d.ppart + (size_t)slot * nm2};
    const size_t cnt[4] = {ncell, nfg, nm2, nm2};
    for (int q = 0; q < 4 && ok; ++q) {
      get(buf.data(), sizeof(double) * cnt[q]);
      if (ok) CK(cudaMemcpy(dst[q], buf.data(), sizeof(double) * cnt[q], cudaMemcpyHostToDevice));
    }
  }
  fclose(f);
  if (rc) return rc;
  if (!ok) return fail(ctx, RAMGPU_ERR_IO, std::string("read failed: ") + path);
  if (time) *time = h.time;
  return RAMGPU_OK;
}

// Bit s set when species s belongs to the member (retired members keep
// their last state and are still sampled).
static unsigned species_mask(const ramgpu_ctx* ctx, int member) {
  unsigned m = 0u;
  for (int s : ctx->member_species[member]) m |= 1u << s;
  return m;
}

// Bilinear stencil of an equatorial point (L-shell [RE], MLT [h]) on the
// FLUX grid: corners I = i0, i0+1 (0-based, I >= 2 where FLUX is defined)
// and J = j0, j1 with J = NT folded onto J = 1; weights of the upper
// corners clamped to [0,1] (points beyond the grid take the edge value).
static void equatorial_stencil(const Dev& d, const std::vector<double>& lz, const std::vector<double>& phi,
                               double lshell, double mlt, int* i0o, double* wi, int* j0o, int* j1o,
                               double* wj) {
  int i0 = 1;
  while (i0 + 1 < d.nr - 1 && lz[i0 + 1] <= lshell) ++i0;
  *i0o = i0;
  *wi = fmin(1.0, fmax(0.0, (lshell - lz[i0]) / (lz[i0 + 1] - lz[i0])));
  const double twopi = 2.0 * kPI;
  double ph = fmod(mlt * kPI / 12.0, twopi);
  if (ph < 0) ph += twopi;
  int j0 = (int)(ph / d.dphi);
  if (j0 > d.nt - 2) j0 = d.nt - 2;
  *j0o = j0;
  *j1o = (j0 + 1 == d.nt - 1) ? 0 : j0 + 1;
  *wj = fmin(1.0, fmax(0.0, (ph - phi[j0]) / d.dphi));
}

int ramgpu_fly_sats(ramgpu_ctx* ctx, const ramgpu_sat* sats, int nsat, double* sat_flux, double* omni_flux) {
  if (check_ctx(ctx) || (nsat > 0 && !sats) || (!sat_flux && !omni_flux))
    return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (nsat < 0) return fail(ctx, RAMGPU_ERR_ARG, "nsat >= 0");
  if (!ctx->have_grid || !ctx->have_fields) return fail(ctx, RAMGPU_ERR_STATE, "grid/fields not set");
  if (nsat == 0) return RAMGPU_OK;
  Dev& d = ctx->d;
  if (d.ns > 32) return fail(ctx, RAMGPU_ERR_ARG, "fly_sats supports ns <= 32");
  std::vector<double> lz(d.nf), phi(d.nt);
  CK(cudaMemcpy(lz.data(), d.lz, sizeof(double) * d.nf, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(phi.data(), d.phi, sizeof(double) * d.nt, cudaMemcpyDeviceToHost));
  std::vector<SatDev> sh(nsat);
  for (int t = 0; t < nsat; ++t) {
    const ramgpu_sat& o = sats[t];
    if (o.member < 0 || o.member >= ctx->cfg.n_members || !isfinite(o.lshell) || !isfinite(o.mlt))
      return fail(ctx, RAMGPU_ERR_ARG, "satellite member or position out of range");
    SatDev& q = sh[t];
    q.member = o.member;
    q.active_mask = 0u;
    q.active_mask = species_mask(ctx, o.member);
    equatorial_stencil(d, lz, phi, o.lshell, o.mlt, &q.i0, &q.wi, &q.j0, &q.j1, &q.wj);
  }
  const size_t nfl = (size_t)nsat * d.ns * d.ne * d.npa, nom = (size_t)nsat * d.ns * d.ne;
  void* buf = nullptr;
  const size_t bytes = sizeof(SatDev) * nsat + sizeof(double) * (nfl + nom);
  CK(cudaMalloc(&buf, bytes));
  SatDev* qd = (SatDev*)buf;
  double* fl = (double*)((char*)buf + sizeof(SatDev) * nsat);
  double* om = fl + nfl;
  cudaError_t e = cudaMemcpyAsync(qd, sh.data(), sizeof(SatDev) * nsat, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) {
    launch_fly_sats(d, qd, nsat, fl, om, ctx->stream);
    ctx->launches += 1;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && sat_flux)
    e = cudaMemcpyAsync(sat_flux, fl, sizeof(double) * nfl, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess && omni_flux)
    e = cudaMemcpyAsync(omni_flux, om, sizeof(double) * nom, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(buf);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "fly_sats");
  return RAMGPU_OK;
}

int ramgpu_bounce_integrals(ramgpu_ctx* ctx, int nthe, const double* chi, const double* x, const double* y,
                            const double* z, const double* b, const double* dens, int ieq, double* h,
                            double* fi, double* hdens, double* bmirror) {
  if (check_ctx(ctx) || !chi || !x || !y || !z || !b || !h || !fi || (hdens && !dens))
    return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (!ctx->have_grid || !ctx->have_fields) return fail(ctx, RAMGPU_ERR_STATE, "grid/fields not set");
  if (nthe < 3 || ieq < 1 || ieq > nthe) return fail(ctx, RAMGPU_ERR_ARG, "nthe >= 3 and 1 <= ieq <= nthe");
  Dev& d = ctx->d;
  const size_t nl = (size_t)d.nr * d.nt, nln = nl * nthe, na = nl * d.npa;
  // one device block: lines (x,y,z,b,dens), chi, per-line and per-angle scratch, outputs
  const size_t nd = 5 * nln + nthe + 2 * nl + 5 * na + 4 * na;
  double* buf = nullptr;
  unsigned char* sbuf = nullptr;
  int* okb = nullptr;
  CK(cudaMalloc(&buf, nd * sizeof(double)));
  cudaError_t e = cudaMalloc(&sbuf, 2 * na);
  if (e == cudaSuccess) e = cudaMalloc(&okb, nl * sizeof(int));
  BounceDev q{};
  q.nr = d.nr; q.nt = d.nt; q.npa = d.npa; q.nthe = nthe; q.ieq = ieq;
  double* p = buf;
  double *dx = p; p += nln;
  double *dy = p; p += nln;
  double *dz = p; p += nln;
  double *db = p; p += nln;
  double *dd = p; p += nln;
  double *dchi = p; p += nthe;
  q.length = p; p += nl;
  q.r0 = p; p += nl;
  q.mirror = p; p += na;
  q.mirror2 = p; p += na;
  q.yi = p; p += na;
  q.yh = p; p += na;
  q.yd = p; p += na;
  q.h_out = p; p += na;
  q.i_out = p; p += na;
  q.d_out = p; p += na;
  q.m_out = p; p += na;
  q.x = dx; q.y = dy; q.z = dz; q.b = db; q.chi = dchi; q.mu = d.mu; q.outside = d.outside;
  q.dens = dens ? dd : nullptr;
  if (!dens) q.yd = nullptr;
  q.st = sbuf; q.sd = sbuf + na; q.line_ok = okb;
  const size_t bytes = nln * sizeof(double);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, bytes, cudaMemcpyDefault, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dy, y, bytes, cudaMemcpyDefault, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dz, z, bytes, cudaMemcpyDefault, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(db, b, bytes, cudaMemcpyDefault, ctx->stream);
  if (e == cudaSuccess && dens) e = cudaMemcpyAsync(dd, dens, bytes, cudaMemcpyDefault, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dchi, chi, nthe * sizeof(double), cudaMemcpyDefault, ctx->stream);
  if (e == cudaSuccess) {
    launch_bounce(q, ctx->stream);
    ctx->launches += 3;
    e = cudaGetLastError();
  }
  const size_t ob = na * sizeof(double);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, q.h_out, ob, cudaMemcpyDefault, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(fi, q.i_out, ob, cudaMemcpyDefault, ctx->stream);
  if (e == cudaSuccess && hdens) e = cudaMemcpyAsync(hdens, q.d_out, ob, cudaMemcpyDefault, ctx->stream);
  if (e == cudaSuccess && bmirror) e = cudaMemcpyAsync(bmirror, q.m_out, ob, cudaMemcpyDefault, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(buf);
  cudaFree(sbuf);
  cudaFree(okb);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "bounce_integrals");
  return RAMGPU_OK;
}

int ramgpu_compute_hI(ramgpu_ctx* ctx, int nthe, const double* chi, const double* x, const double* y,
                      const double* z, const double* b, const double* dens, int ieq, const double* pa,
                      const double* pabn, double bnormal, double dthi) {
  if (check_ctx(ctx) || !chi || !x || !y || !z || !b || !dens || !pa || !pabn)
    return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (!ctx->have_grid || !ctx->have_fields) return fail(ctx, RAMGPU_ERR_STATE, "grid/fields not set");
  if (nthe < 3 || ieq < 1 || ieq > nthe) return fail(ctx, RAMGPU_ERR_ARG, "nthe >= 3 and 1 <= ieq <= nthe");
  Dev& d = ctx->d;
  const size_t nl = (size_t)d.nr * d.nt, nln = nl * nthe, na = nl * d.npa;
  const size_t nd = 5 * nln + nthe + 2 * nl + 9 * na + 2 * na + 6 * nl * d.npa + d.npa + d.npa;
  double* buf = nullptr;
  unsigned char* sbuf = nullptr;
  int* okb = nullptr;
  CK(cudaMalloc(&buf, nd * sizeof(double)));
  cudaError_t e = cudaMalloc(&sbuf, 2 * na);
  if (e == cudaSuccess) e = cudaMalloc(&okb, nl * sizeof(int));
  BounceDev q{};
  q.nr = d.nr; q.nt = d.nt; q.npa = d.npa; q.nthe = nthe; q.ieq = ieq;
  double* p = buf;
  double *dx = p; p += nln;
  double *dy = p; p += nln;
  double *dz = p; p += nln;
  double *db = p; p += nln;
  double *dd = p; p += nln;
  double *dchi = p; p += nthe;
  q.length = p; p += nl;
  q.r0 = p; p += nl;
  q.mirror = p; p += na;
  q.mirror2 = p; p += na;
  q.yi = p; p += na;
  q.yh = p; p += na;
  q.yd = p; p += na;
  q.h_out = p; p += na;
  q.i_out = p; p += na;
  q.d_out = p; p += na;
  q.m_out = p; p += na;
  q.x = dx; q.y = dy; q.z = dz; q.b = db; q.chi = dchi; q.mu = d.mu; q.outside = d.outside;
  q.dens = dd;
  q.st = sbuf; q.sd = sbuf + na; q.line_ok = okb;
  HiDev hq{};
  hq.nr = d.nr; hq.nt = d.nt; hq.npa = d.npa; hq.dthi = dthi; hq.bnormal = bnormal;
  hq.outside = d.outside;
  hq.h = q.h_out; hq.fi = q.i_out; hq.hd = q.d_out; hq.beq = q.m_out;  // L = 1 mirror = equatorial B
  hq.hb = p; p += na;
  hq.ib = p; p += na;
  hq.scratch = p; p += 6 * nl * d.npa;
  double* dpa = p; p += d.npa;
  double* dpr = p; p += d.npa;
  hq.pa = dpa; hq.pabn_rev = dpr;
  hq.fnhs = (double*)d.fnhs; hq.fnis = (double*)d.fnis; hq.hdns = (double*)d.hdns;
  hq.bounhs = (double*)d.bounhs; hq.bounis = (double*)d.bounis; hq.didt = (double*)d.didt;
  hq.dibndt = (double*)d.dibndt; hq.bnes = (double*)d.bnes; hq.dbdt = (double*)d.dbdt;
  hq.eir = (double*)d.eir; hq.eip = (double*)d.eip;
  std::vector<double> lz0(1), pr(d.npa, 0.0);
  if (e == cudaSuccess) e = cudaMemcpy(lz0.data(), d.lz, sizeof(double), cudaMemcpyDeviceToHost);
  hq.lz0 = lz0[0];
  for (int qq = 0; qq < d.npa - 2; ++qq) pr[qq] = pabn[d.npa - 2 - qq];
  const size_t bytes = nln * sizeof(double);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, bytes, cudaMemcpyDefault, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dy, y, bytes, cudaMemcpyDefault, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dz, z, bytes, cudaMemcpyDefault, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(db, b, bytes, cudaMemcpyDefault, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dd, dens, bytes, cudaMemcpyDefault, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dchi, chi, nthe * sizeof(double), cudaMemcpyDefault, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dpa, pa, d.npa * sizeof(double), cudaMemcpyDefault, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dpr, pr.data(), d.npa * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) {
    launch_bounce(q, ctx->stream);
    launch_hi_fill(hq, ctx->stream);
    ctx->launches += 7;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(buf);
  cudaFree(sbuf);
  cudaFree(okb);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "compute_hI");
  ctx->field_dirty = true;  // derived tables follow on the next step
  return RAMGPU_OK;
}

int ramgpu_sum_pressure(ramgpu_ctx* ctx, int member, double* pallsum, double* pparsum) {
  if (check_ctx(ctx) || !pallsum || !pparsum) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (member < 0 || member >= ctx->cfg.n_members) return fail(ctx, RAMGPU_ERR_ARG, "member out of range");
  Dev& d = ctx->d;
  if (d.ns > 32) return fail(ctx, RAMGPU_ERR_ARG, "sum_pressure supports ns <= 32");
  const unsigned mask = species_mask(ctx, member);
  const size_t n = (size_t)d.nr * d.nt;
  double* buf = nullptr;
  CK(cudaMalloc(&buf, 2 * n * sizeof(double)));
  launch_sum_pressure(d, member, mask, buf, buf + n, ctx->stream);
  ctx->launches += 1;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(pallsum, buf, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(pparsum, buf + n, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(buf);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "sum_pressure");
  return RAMGPU_OK;
}

// Ring position of call c's branch record: segment c/k sits in slot
// (c/k) mod nkeep, so the last nkeep segments survive the forward pass.
static size_t adj_rec_slot(const ramgpu_ctx::Adj& a, int c) {
  return (size_t)((c / a.k) % a.nkeep) * a.k + (size_t)(c % a.k);
}

int ramgpu_set_adj_record_budget(ramgpu_ctx* ctx, long long bytes) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  ctx->adj_record_budget = bytes < 0 ? -1 : bytes;
  return RAMGPU_OK;
}

int ramgpu_adj_segments(ramgpu_ctx* ctx, int* nseg, int* nkeep) {
  if (check_ctx(ctx) || !nseg || !nkeep) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (!ctx->adj.ready) return fail(ctx, RAMGPU_ERR_STATE, "ramgpu_adj_forward must run first");
  *nseg = ctx->adj.nseg;
  *nkeep = ctx->adj.nkeep;
  return RAMGPU_OK;
}

int ramgpu_adj_forward(ramgpu_ctx* ctx, int ncalls, double dts, const double* kp, int k_ckpt,
                       const ramgpu_obs* obs, int nobs, double* J) {
  NvtxRange range_("ramgpu_adj_forward");
  if (check_ctx(ctx) || !kp || (nobs > 0 && !obs)) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (ncalls < 1 || k_ckpt < 1 || nobs < 0) return fail(ctx, RAMGPU_ERR_ARG, "ncalls, k_ckpt >= 1, nobs >= 0");
  if (ctx->cfg.flags & RAMGPU_FLAG_LOSSES)
    return fail(ctx, RAMGPU_ERR_ARG, "the adjoint window runs without RAMGPU_FLAG_LOSSES");
  if (ctx->pd_any())
    return fail(ctx, RAMGPU_ERR_ARG, "the adjoint does not cover the pitch-angle diffusion");
  Dev& d = ctx->d;
  if (d.nr < 4 || d.nt < 7 || d.ne < 6 || d.npa < 9)
    return fail(ctx, RAMGPU_ERR_ARG, "the adjoint needs NR >= 4, NT >= 7, NE >= 6, NPA >= 9");
  int rc = prepare(ctx, dts);
  if (rc) return rc;
  if (d.nitems == 0) return fail(ctx, RAMGPU_ERR_STATE, "no active (member, species)");
  const int nm = ctx->cfg.n_members;
  for (long long i = 0; i < (long long)ncalls * nm; ++i)
    if (!isfinite(kp[i])) return fail(ctx, RAMGPU_ERR_ARG, "kp must be finite");
  // observations -> device form (corners and weights of the bilinear stencil)
  std::vector<ObsDev> oh(nobs);
  std::vector<double> lz(d.nf), phi(d.nt);
  CK(cudaMemcpy(lz.data(), d.lz, sizeof(double) * d.nf, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(phi.data(), d.phi, sizeof(double) * d.nt, cudaMemcpyDeviceToHost));
  for (int t = 0; t < nobs; ++t) {
    const ramgpu_obs& o = obs[t];
    if (int r2 = check_ms(ctx, o.member, o.s)) return r2;
    if (o.call < 0 || o.call >= ncalls || o.k < 1 || o.k >= d.ne || o.l < 1 || o.l >= d.npa ||
        !isfinite(o.lshell) || !isfinite(o.mlt) || !isfinite(o.log_obs))
      return fail(ctx, RAMGPU_ERR_ARG, "observation out of range");
    bool found = false;
    for (auto& it : ctx->items_h) found |= (it.x == o.member && it.y == o.s);
    if (!found) return fail(ctx, RAMGPU_ERR_ARG, "observation of an inactive (member, species)");
    ObsDev& q = oh[t];
    q.member = o.member; q.slot = o.member * d.ns + o.s; q.call = o.call; q.k = o.k; q.l = o.l;
    q.item = 0;
    for (size_t it = 0; it < ctx->items_h.size(); ++it)
      if (ctx->items_h[it].x == o.member && ctx->items_h[it].y == o.s) q.item = (int)it;
    q.log_obs = o.log_obs;
    equatorial_stencil(d, lz, phi, o.lshell, o.mlt, &q.i0, &q.wi, &q.j0, &q.j1, &q.wj);
  }
  auto& a = ctx->adj;
  a.ready = false;
  const int nseg = (ncalls + k_ckpt - 1) / k_ckpt;
  const size_t rec_call = (size_t)4 * d.nitems * d.ncell;
  const int kseg = k_ckpt < ncalls ? k_ckpt : ncalls;
  // The ring keeps the records of the last nkeep segments, as many as the
  // budget allows (at least one, two with the overlapped recomputation:
  // the segment being recomputed and the one being transposed); only the
  // segments before them are recomputed from their checkpoints in the
  // backward pass.
  const long long least = (ctx->adj_overlap && nseg > 1) ? 2 : 1;
  int nkeep = 1;
  {
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    // the ring this window would reuse counts as free
    if (a.rec && a.rec_call == rec_call && a.k == kseg) free_b += a.rec_call * kseg * a.nkeep;
    const long long budget = ctx->adj_record_budget >= 0 ? ctx->adj_record_budget : (long long)(free_b / 2);
    const long long seg_bytes = (long long)(rec_call * kseg);
    long long nk = budget / seg_bytes;
    nkeep = (int)(nk < least ? least : (nk > nseg ? nseg : nk));
  }
  // buffers of the previous window are reused when the new one has the
  // same shape (a window run again, as finite differences do)
  const bool reuse = a.rec && a.ckpt && a.rec_call == rec_call && a.k == kseg && a.nkeep == nkeep &&
                     a.nseg == nseg && a.nobs == nobs && a.ncalls == ncalls;
  if (!reuse) adj_free(ctx);
  a.ncalls = ncalls; a.k = k_ckpt; a.nseg = nseg; a.nobs = nobs; a.dts = dts;
  a.kp.assign(kp, kp + (size_t)ncalls * nm);
  a.obs_calls.assign(ncalls, 0);
  for (int t = 0; t < nobs; ++t) a.obs_calls[obs[t].call] += 1;
  a.items_version = ctx->items_version;
  a.rec_call = rec_call;
  a.nkeep = nkeep;
  bool ok = true;
  if (!reuse) {
    ok = cudaMalloc(&a.ckpt, sizeof(double) * a.nseg * d.nitems * d.ncell) == cudaSuccess;
    if (ok && cudaMalloc(&a.rec, a.rec_call * kseg * a.nkeep) != cudaSuccess) {
      cudaGetLastError();
      a.nkeep = 1;
      ok = cudaMalloc(&a.rec, a.rec_call * kseg) == cudaSuccess;
    }
    // record positions no sweep writes stay zero in every call
    if (ok) ok = cudaMemsetAsync(a.rec, 0, a.rec_call * kseg * a.nkeep, ctx->stream) == cudaSuccess;
  }
  if (reuse) {
    // the same shape: obs, fm, J and the rest are reused too
  } else {
  ok = ok && cudaMalloc(&a.obs, sizeof(ObsDev) * (nobs > 0 ? nobs : 1)) == cudaSuccess;
  ok = ok && cudaMalloc(&a.fm, sizeof(double) * (nobs > 0 ? nobs : 1)) == cudaSuccess;
  ok = ok && cudaMalloc(&a.fm2, sizeof(double) * (nobs > 0 ? nobs : 1)) == cudaSuccess;
  ok = ok && cudaMalloc(&a.J, sizeof(double) * nm) == cudaSuccess;
  ok = ok && cudaMalloc(&a.J2, sizeof(double) * nm) == cudaSuccess;
  ok = ok && cudaMalloc(&a.digest, sizeof(unsigned long long)) == cudaSuccess;
  ok = ok && cudaMalloc(&a.kp_d, sizeof(double) * (size_t)ncalls * nm) == cudaSuccess;
  }
  if (!ok) {
    adj_free(ctx);
    return fail(ctx, RAMGPU_ERR_NOMEM, "adjoint buffers: device allocation failed");
  }
  if (nobs > 0) CK(cudaMemcpy(a.obs, oh.data(), sizeof(ObsDev) * nobs, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(a.kp_d, a.kp.data(), sizeof(double) * (size_t)ncalls * nm, cudaMemcpyHostToDevice));
  std::vector<int> one(nm, 1);
  CK(cudaMemcpyAsync(d.vt_mode, one.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemsetAsync(a.J, 0, sizeof(double) * nm, ctx->stream));
  CK(cudaMemsetAsync(a.digest, 0, sizeof(unsigned long long), ctx->stream));
  // Segments whose records the ring keeps run the recording step; the
  // earlier ones, which the backward pass recomputes from their checkpoints
  // anyway, run the plain step (the same F2 bits, no record traffic; from
  // its CUDA graph when graphs are on).  The digest covers the recorded calls.
  const int first_kept = a.nseg - a.nkeep;
  for (int c = 0; c < ncalls; ++c) {
    if (c % k_ckpt == 0)
      if ((rc = adj_copy_items(ctx, a.ckpt + (size_t)(c / k_ckpt) * d.nitems * d.ncell, true))) return rc;
    if ((rc = adj_set_kp(ctx, c))) return rc;
    if (c / k_ckpt < first_kept) {
      if ((rc = enqueue_ram_run(ctx, dts))) return rc;
    } else {
      unsigned char* r = a.rec + adj_rec_slot(a, c) * a.rec_call;
      if ((rc = enqueue_call_rec(ctx, dts, r, c == ncalls - 1))) return rc;
      launch_digest(r, (long long)a.rec_call, a.digest, ctx->stream);
      ctx->launches += 1;
    }
    if (a.obs_calls[c]) {  // calls with observations only
      launch_obs_fwd(d, a.obs, nobs, c, a.fm, a.J, ctx->stream);
      ctx->launches += 1;
    }
    CKL("adjoint forward");
  }
  CK(cudaStreamSynchronize(ctx->stream));
  if (J) CK(cudaMemcpy(J, a.J, sizeof(double) * nm, cudaMemcpyDeviceToHost));
  ctx->last_dts = dts;
  a.ready = true;
  a.rec_stale = false;
  return RAMGPU_OK;
}

int ramgpu_set_adj_overlap(ramgpu_ctx* ctx, int on) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  ctx->adj_overlap = on != 0;
  return RAMGPU_OK;
}

// The second stream, its events (2 per ring slot + 2) and the shadow copies
// of everything a recorded call writes besides F2 and its record: the
// per-member tables CR, CA, DRD1, DPD1, UE, UM and the DRIFTR ghost planes,
// and a coefficient store of its own when the context has one (without it
// the DRIFTE reverse recomputes its coefficients: the same bits, two FP64
// operations per cell more).  Returns in q the context's Dev with those
// pointers replaced and without clip counting.
// One set of the tables a call writes besides F2: per member CR, CA, DRD1,
// DPD1, UE, UM, per slot the DRIFTR ghost planes (256-byte pieces).
static size_t table_set_bytes(const Dev& d) {
  const size_t nm = (size_t)d.nm, nij = nm * d.nr * d.nt, nijl = nij * d.npa;
  const size_t npl = nm * d.ns * d.ne * d.npa;
  auto up = [](size_t n) { return (n + 31) / 32 * 32; };
  return 8 * (4 * up(nij) + 2 * up(nijl) + 2 * up(npl)) + 4 * 3 * up(npl);
}
// q's table pointers into the set at base.
static void table_set_assign(void* base, Dev& q) {
  const size_t nm = (size_t)q.nm, nij = nm * q.nr * q.nt, nijl = nij * q.npa;
  const size_t npl = nm * q.ns * q.ne * q.npa;
  auto up = [](size_t n) { return (n + 31) / 32 * 32; };
  double* p = (double*)base;
  auto take = [&](size_t n) { double* r = p; p += up(n); return r; };
  q.cr = take(nij); q.ca = take(nij); q.drd1 = take(nij); q.dpd1 = take(nij);
  q.ue = take(nijl); q.um = take(nijl);
  q.plane_last = take(npl); q.plane_carry = take(npl);
  int* ip = (int*)p;
  q.plane_has = ip; ip += up(npl);
  q.plane_last_src = ip; ip += up(npl);
  q.plane_carry_src = ip;
}

static int adj_shadow_prepare(ramgpu_ctx* ctx, Dev& q) {
  const Dev& d = ctx->d;
  if (!ctx->adj_shadow && cudaMalloc(&ctx->adj_shadow, table_set_bytes(d)) != cudaSuccess) {
    cudaGetLastError();
    ctx->adj_shadow = nullptr;
    return fail(ctx, RAMGPU_ERR_NOMEM, "adjoint recomputation tables: device allocation failed");
  }
  if (!ctx->adj_stream) {
    int prio = 0;
    if (!ctx->pipe_streams.empty()) CK(cudaStreamGetPriority(ctx->pipe_streams[0], &prio));
    CK(cudaStreamCreateWithPriority(&ctx->adj_stream, cudaStreamNonBlocking, prio));
  }
  const size_t nev = 2 * (size_t)ctx->adj.nkeep + 2;
  while (ctx->adj_events.size() < nev) {
    cudaEvent_t e = nullptr;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    ctx->adj_events.push_back(e);
  }
  q = d;
  table_set_assign(ctx->adj_shadow, q);
  q.coef = nullptr;
  if (d.coef) {
    int nw = 0;
    for (int w = 0; w < 4; ++w) nw += d.coef_slot[w] >= 0 ? 1 : 0;
    const size_t need = (size_t)2 * nw * d.coef_items * d.ncell * sizeof(double);
    if (ctx->adj_shadow_coef_bytes != need) {
      cudaFree(ctx->adj_shadow_coef);
      ctx->adj_shadow_coef = nullptr;
      ctx->adj_shadow_coef_bytes = 0;
      if (cudaMalloc(&ctx->adj_shadow_coef, need) == cudaSuccess) ctx->adj_shadow_coef_bytes = need;
      else { ctx->adj_shadow_coef = nullptr; cudaGetLastError(); }
    }
    q.coef = ctx->adj_shadow_coef;
  }
  q.count_clips = 0;
  return RAMGPU_OK;
}

// The transposes' ring of kAdjTableRing table sets (per call: the tables of
// call c sit in set c mod kAdjTableRing) and its events: per set "tables
// written" and, per item group, "group done with them", then the fork.
constexpr int kAdjTableRing = 3;
static int adj_ring_prepare(ramgpu_ctx* ctx, int G) {
  const size_t per = table_set_bytes(ctx->d);
  if (!ctx->adj_ring) {
    if (cudaMalloc(&ctx->adj_ring, per * kAdjTableRing) != cudaSuccess) {
      cudaGetLastError();
      ctx->adj_ring = nullptr;
      return fail(ctx, RAMGPU_ERR_NOMEM, "adjoint table ring: device allocation failed");
    }
  }
  const size_t nev = (size_t)kAdjTableRing * (1 + G) + 1;
  while (ctx->adj_ring_events.size() < nev) {
    cudaEvent_t e = nullptr;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    ctx->adj_ring_events.push_back(e);
  }
  return RAMGPU_OK;
}

// Call `call` of the window recomputed on stream st with the shadow tables
// q, every sweep recording into rec: the sequence of enqueue_call_rec over
// the whole work list as one group (the same records: a group's record
// sits at its items' place in the list).
static int adj_recompute_call(ramgpu_ctx* ctx, const Dev& q, cudaStream_t st, int call, double dts,
                              unsigned char* rec) {
  Dev qc = q;  // Kp of the call read from the window's array
  qc.kp = ctx->adj.kp_d + (size_t)call * ctx->cfg.n_members;
  const size_t isz = (size_t)q.nitems * q.ncell;
  const int co_e = (q.coef && q.coef_slot[2] >= 0) ? 1 : 0;
  launch_member_coef(qc, dts, st);
  launch_ghost(q, st);
  launch_sweep_r(q, dts, false, st, rec + 0 * isz, false, 0, 4);
  launch_sweep_p(q, dts, false, st, rec + 1 * isz, false, 0, 4);
  launch_sweep_e(q, dts, false, st, rec + 2 * isz, false, co_e, 4);
  launch_sweep_mu(q, dts, false, 1, q.loss2, st, rec + 3 * isz, false, 0, 4);
  launch_sweep_mu(q, dts, false, 0, nullptr, st, rec + 3 * isz, false, 0, 0);
  launch_sweep_e(q, dts, false, st, rec + 2 * isz, false, 2 * co_e, 0);
  launch_sweep_p(q, dts, false, st, rec + 1 * isz, false, 0, 0);
  launch_sweep_r(q, dts, false, st, rec + 0 * isz, false, 0, 0);
  launch_finish(q, st);
  launch_anisch_state(q, st);
  ctx->launches += 13;
  CKL("adjoint recomputation");
  return RAMGPU_OK;
}

int ramgpu_adj_backward(ramgpu_ctx* ctx, double* grad_f2, double* grad_fgeos) {
  NvtxRange range_("ramgpu_adj_backward");
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  auto& a = ctx->adj;
  if (!a.ready) return fail(ctx, RAMGPU_ERR_STATE, "ramgpu_adj_forward must run first");
  if (ctx->items_dirty || a.items_version != ctx->items_version)
    return fail(ctx, RAMGPU_ERR_STATE, "active members/species changed since ramgpu_adj_forward");
  Dev& d = ctx->d;
  int rc = prepare(ctx, a.dts);
  if (rc) return rc;
  const size_t nslot = (size_t)d.nm * d.ns, nfg = (size_t)d.nt * d.ne * d.npa;
  const size_t isz = (size_t)d.nitems * d.ncell;
  const int G = clamp_groups(ctx, ctx->step_groups);
  if ((rc = ensure_group_streams(ctx, G))) return rc;
  // the first DRIFTE transpose of each call keeps its face coefficients in
  // the DRIFTE coefficient store for the second
  const int co_e = (d.coef && d.coef_slot[2] >= 0) ? 1 : 0;
  CK(cudaMemsetAsync(d.lam, 0, sizeof(double) * nslot * d.ncell, ctx->stream));
  CK(cudaMemsetAsync(d.gfg, 0, sizeof(double) * nslot * nfg, ctx->stream));
  // The records of the last nkeep segments are still the forward pass's
  // own (the observation values fm are kept from it for every call);
  // earlier segments are recomputed from their checkpoint, recording
  // branches into their ring slot (whose previous segment is done).
  auto needs = [&](int seg) { return seg < a.nseg - a.nkeep || a.rec_stale; };
  auto calls_of = [&](int seg, int& c0, int& c1) {
    c0 = seg * a.k;
    c1 = (c0 + a.k < a.ncalls) ? c0 + a.k : a.ncalls;
  };
  // The transposes of a segment: call c's per-member tables go into table
  // set c mod kAdjTableRing on the context's stream, and each item group
  // streams through the segment's calls on its own stream, waiting only for
  // its call's tables; the table set is rewritten once every group is done
  // with it.  No join between calls: one group's launch tails and the gaps
  // between its dependent launches are filled by the others.
  if ((rc = adj_ring_prepare(ctx, G))) return rc;
  const size_t tset = table_set_bytes(d);
  auto transpose = [&](int seg) -> int {
    int c0, c1;
    calls_of(seg, c0, c1);
    const cudaStream_t main = ctx->stream;
    const Dev full = ctx->d;
    const int T = kAdjTableRing;
    cudaEvent_t* evTab = ctx->adj_ring_events.data();
    cudaEvent_t* evUse = evTab + T;  // [g * T + set]
    cudaEvent_t evFork = evTab[T * (1 + G)];
    auto gstream = [&](int g) { return G > 1 ? ctx->pipe_streams[g] : main; };
    if (G > 1) {
      CK(cudaEventRecord(evFork, main));
      for (int g = 0; g < G; ++g) CK(cudaStreamWaitEvent(gstream(g), evFork, 0));
    }
    for (int c = c1 - 1; c >= c0; --c) {  // transpose call c
      const int sl = c % T;
      if (G > 1)
        for (int g = 0; g < G; ++g) CK(cudaStreamWaitEvent(main, evUse[g * T + sl], 0));
      Dev dk = full;
      table_set_assign((char*)ctx->adj_ring + tset * sl, dk);
      dk.kp = a.kp_d + (size_t)c * ctx->cfg.n_members;  // Kp read from the window's array
      launch_member_coef(dk, a.dts, main);
      launch_ghost(dk, main);
      ctx->launches += 3;
      if (G > 1) CK(cudaEventRecord(evTab[sl], main));
      const unsigned char* rcall = a.rec + adj_rec_slot(a, c) * a.rec_call;
      for (int g = 0; g < G; ++g) {
        const int i0 = (int)((long long)full.nitems * g / G), i1 = (int)((long long)full.nitems * (g + 1) / G);
        if (i1 <= i0) continue;
        const cudaStream_t st = gstream(g);
        if (G > 1) CK(cudaStreamWaitEvent(st, evTab[sl], 0));
        Dev dg = dk;
        dg.items = full.items + i0;
        dg.nitems = i1 - i0;
        dg.item0 = full.item0 + i0;
        if (a.obs_calls[c]) {  // the group's observations of call c
          launch_obs_adj(dg, a.obs, a.nobs, c, a.fm, st);
          ctx->launches += 1;
        }
        const unsigned char* r = rcall + (size_t)i0 * dg.ncell;
        launch_adj_tail(dg, st);
        launch_adj_sweep(dg, 0, r + 0 * isz, 0, st);
        launch_adj_sweep(dg, 1, r + 1 * isz, 0, st);
        launch_adj_sweep(dg, 2, r + 2 * isz, 0, st, co_e);
        launch_adj_sweep(dg, 3, r + 3 * isz, 0, st);
        launch_adj_sweep(dg, 3, r + 3 * isz, 4, st, 0, dg.loss2);  // CEX/ATMOL^T fused
        launch_adj_sweep(dg, 2, r + 2 * isz, 4, st, 2 * co_e);
        launch_adj_sweep(dg, 1, r + 1 * isz, 4, st);
        launch_adj_sweep(dg, 0, r + 0 * isz, 4, st);
        ctx->launches += 10;
        CKL("adjoint backward");
        if (G > 1) CK(cudaEventRecord(evUse[g * T + sl], st));
      }
    }
    if (G > 1)  // join: the segment's last call in every group
      for (int g = 0; g < G; ++g) CK(cudaStreamWaitEvent(main, evUse[g * T + c0 % T], 0));
    return RAMGPU_OK;
  };
  const bool any_recompute = a.rec_stale || a.nseg > a.nkeep;
  if (ctx->adj_overlap && any_recompute && a.nkeep >= 2) {
    // Segment seg - 1 is recomputed on the second stream while segment seg
    // is transposed: their ring slots differ (nkeep >= 2), the second
    // stream has its own per-member tables and ghost planes, and the
    // transposes read neither F2 nor those tables.  Recomputing segment s
    // waits until the segment that last held its slot (s + nkeep) has been
    // transposed; transposing s waits until s is recomputed.  An event per
    // slot suffices: when either wait is enqueued, the slot's latest record
    // is the one waited for.
    Dev q;
    if ((rc = adj_shadow_prepare(ctx, q))) return rc;
    const cudaStream_t qs = ctx->adj_stream;
    const int nk = a.nkeep;
    cudaEvent_t* evR = ctx->adj_events.data();
    cudaEvent_t* evT = evR + nk;
    cudaEvent_t evStart = evT[nk], evEnd = evT[nk + 1];
    CK(cudaEventRecord(evStart, ctx->stream));
    CK(cudaStreamWaitEvent(qs, evStart, 0));
    auto recompute = [&](int seg) -> int {
      if (seg + nk < a.nseg) CK(cudaStreamWaitEvent(qs, evT[seg % nk], 0));
      const size_t n = d.ncell;
      for (size_t i = 0; i < ctx->items_h.size(); ++i) {
        const int slot = ctx->items_h[i].x * d.ns + ctx->items_h[i].y;
        CK(cudaMemcpyAsync(d.f2 + (size_t)slot * n, a.ckpt + (size_t)seg * isz + i * n, sizeof(double) * n,
                           cudaMemcpyDeviceToDevice, qs));
      }
      int c0, c1;
      calls_of(seg, c0, c1);
      for (int c = c0; c < c1; ++c)
        if (int r2 = adj_recompute_call(ctx, q, qs, c, a.dts, a.rec + adj_rec_slot(a, c) * a.rec_call)) return r2;
      CK(cudaEventRecord(evR[seg % nk], qs));
      return RAMGPU_OK;
    };
    const int top = a.nseg - 1;
    if (needs(top) && (rc = recompute(top))) return rc;
    for (int seg = top; seg >= 0; --seg) {
      if (seg >= 1 && needs(seg - 1) && (rc = recompute(seg - 1))) return rc;
      if (needs(seg)) CK(cudaStreamWaitEvent(ctx->stream, evR[seg % nk], 0));
      if ((rc = transpose(seg))) return rc;
      CK(cudaEventRecord(evT[seg % nk], ctx->stream));
    }
    CK(cudaEventRecord(evEnd, qs));
    CK(cudaStreamWaitEvent(ctx->stream, evEnd, 0));
  } else {
    for (int seg = a.nseg - 1; seg >= 0; --seg) {
      if (needs(seg)) {
        if ((rc = adj_copy_items(ctx, a.ckpt + (size_t)seg * isz, false))) return rc;
        int c0, c1;
        calls_of(seg, c0, c1);
        for (int c = c0; c < c1; ++c) {
          if ((rc = adj_set_kp(ctx, c))) return rc;
          if ((rc = enqueue_call_rec(ctx, a.dts, a.rec + adj_rec_slot(a, c) * a.rec_call, false))) return rc;
        }
      }
      if ((rc = transpose(seg))) return rc;
    }
  }
  if ((rc = adj_copy_items(ctx, a.ckpt, false))) return rc;  // F2 back to the initial state
  if ((rc = adj_set_kp(ctx, 0))) return rc;                  // and Kp that of its first call
  a.rec_stale = a.nseg > a.nkeep;  // recomputed segments replaced kept ones
  CK(cudaStreamSynchronize(ctx->stream));
  if (grad_f2) CK(cudaMemcpy(grad_f2, d.lam, sizeof(double) * nslot * d.ncell, cudaMemcpyDefault));
  if (grad_fgeos) CK(cudaMemcpy(grad_fgeos, d.gfg, sizeof(double) * nslot * nfg, cudaMemcpyDefault));
  return RAMGPU_OK;
}

int ramgpu_adj_replay(ramgpu_ctx* ctx, double* J) {
  if (check_ctx(ctx) || !J) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  auto& a = ctx->adj;
  if (!a.ready) return fail(ctx, RAMGPU_ERR_STATE, "ramgpu_adj_forward must run first");
  if (a.nseg > a.nkeep || a.rec_stale)
    return fail(ctx, RAMGPU_ERR_STATE,
                "replay needs every call's record: ramgpu_adj_forward with k_ckpt >= ncalls or a record budget "
                "that keeps every segment");
  if (ctx->items_dirty || a.items_version != ctx->items_version)
    return fail(ctx, RAMGPU_ERR_STATE, "active members/species changed since ramgpu_adj_forward");
  int rc = prepare(ctx, a.dts);
  if (rc) return rc;
  Dev& d = ctx->d;
  const int nm = ctx->cfg.n_members;
  CK(cudaMemsetAsync(a.J2, 0, sizeof(double) * nm, ctx->stream));
  for (int c = 0; c < a.ncalls; ++c) {
    if ((rc = adj_set_kp(ctx, c))) return rc;
    if ((rc = enqueue_call_replay(ctx, a.dts, a.rec + adj_rec_slot(a, c) * a.rec_call))) return rc;
    if (a.obs_calls[c]) {
      launch_obs_fwd(d, a.obs, a.nobs, c, a.fm2, a.J2, ctx->stream);
      ctx->launches += 1;
    }
  }
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpy(J, a.J2, sizeof(double) * nm, cudaMemcpyDeviceToHost));
  return RAMGPU_OK;
}

int ramgpu_adj_record(ramgpu_ctx* ctx, int call, unsigned char* out) {
  if (check_ctx(ctx) || !out) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  auto& a = ctx->adj;
  if (!a.ready) return fail(ctx, RAMGPU_ERR_STATE, "ramgpu_adj_forward must run first");
  if (call < 0 || call >= a.ncalls || call / a.k < a.nseg - a.nkeep)
    return fail(ctx, RAMGPU_ERR_ARG, "only calls of the kept checkpoint segments have a record");
  if (a.rec_stale)
    return fail(ctx, RAMGPU_ERR_STATE, "the record was replaced by ramgpu_adj_backward's recomputation");
  CK(cudaStreamSynchronize(ctx->stream));
  // the device keeps sweeps w and 7-w in the high and low nibbles of one
  // byte (instance w < 4); unpack into one byte per face and sweep
  std::vector<unsigned char> packed(a.rec_call);
  CK(cudaMemcpy(packed.data(), a.rec + adj_rec_slot(a, call) * a.rec_call, a.rec_call, cudaMemcpyDeviceToHost));
  const size_t isz = a.rec_call / 4;
  for (int w = 0; w < 8; ++w) {
    const unsigned char* src = packed.data() + (size_t)(w < 4 ? w : 7 - w) * isz;
    const int sh = w < 4 ? 4 : 0;
    unsigned char* dst = out + (size_t)w * isz;
    for (size_t i = 0; i < isz; ++i) dst[i] = (unsigned char)((src[i] >> sh) & 0x0F);
  }
  return RAMGPU_OK;
}

int ramgpu_adj_digest(ramgpu_ctx* ctx, unsigned long long* digest) {
  if (check_ctx(ctx) || !digest) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  if (!ctx->adj.ready) return fail(ctx, RAMGPU_ERR_STATE, "ramgpu_adj_forward must run first");
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpy(digest, ctx->adj.digest, sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  return RAMGPU_OK;
}

int ramgpu_set_timing(ramgpu_ctx* ctx, int enable) {
  if (check_ctx(ctx)) return RAMGPU_ERR_ARG;
  ctx->timing = enable != 0;
  return RAMGPU_OK;
}

int ramgpu_kernel_times(ramgpu_ctx* ctx, double* ms, long long* counts) {
  if (check_ctx(ctx) || !ms || !counts) return fail(ctx, RAMGPU_ERR_ARG, "null argument");
  CK(cudaStreamSynchronize(ctx->stream));
  for (auto& sp : ctx->spans) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, sp.a, sp.b) == cudaSuccess && sp.kind >= 0 && sp.kind < RAMGPU_NKCLASS) {
      ms[sp.kind] += t;
      counts[sp.kind] += 1;
    }
    ctx->ev_free.push_back(sp.a);
    ctx->ev_free.push_back(sp.b);
  }
  ctx->spans.clear();
  return RAMGPU_OK;
}

}  // extern "C"
