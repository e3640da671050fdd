// Host runtime and C ABI (include/mattohf.h).
//
// Owns the device-resident state of one run (orbitals, tables, potentials,
// Krylov blocks, Fock partial-sum scratch) and sequences the kernels of
// k_hpsi.cu / k_gs.cu / k_table.cu on one CUDA stream.  The RK4 step is
// captured once into a CUDA graph and replayed; the step index lives on the
// device so one graph serves every step.
#include "internal.h"
#include "../../include/mattohf.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <string>
#include <vector>
#include <mutex>
#include <tuple>
#include <map>
#include <algorithm>
#include <functional>

using namespace mattohf;

namespace {

constexpr double kPi = 3.14159265358979323846264338327950288;

__global__ void k_twiddles(double2* tw, int n) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m < n) {
    double s, c;
    sincospi(-2.0 * (double)m / (double)n, &s, &c);
    tw[m] = make_double2(c, s);
  }
}

// FP64 FMA throughput probe: 8 independent dependency chains per thread.
__global__ void k_dfma_probe(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  const double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == -12345.0) out[0] = s;
}

// FP64 tensor-core (DMMA, mma.sync m8n8k4 f64) throughput probe: 8
// independent accumulator pairs per lane; 512 FLOP per warp instruction.
__global__ void k_dmma_probe(double* out, int iters) {
  const double a = 1.0 + threadIdx.x * 1e-9, b = 1.0 - threadIdx.x * 1e-9;
  double c[8][2];
#pragma unroll
  for (int j = 0; j < 8; ++j) c[j][0] = c[j][1] = 0.0;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                   : "+d"(c[j][0]), "+d"(c[j][1])
                   : "d"(a), "d"(b));
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += c[j][0] + c[j][1];
  if (s == -12345.0) out[0] = s;
}

}  // namespace

struct mattohf_ctx {
  int NG = 0, NK = 0, NB = 0, NBocc = 0, hf = 1, device = 0;
  double acell = 0, vcell = 0, dvcell = 0, bx = 0, occ = 0;
  std::vector<double> rx, Gx, kx, vion;
  std::vector<double> Zeff, alpha, Rion;
  std::vector<int> Kion;
  cudaStream_t st = nullptr;
  // side stream: the density of an RK4 stage runs beside that stage's exchange
  cudaStream_t st_side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // tables
  double2* tw = nullptr;
  double *d_Gx = nullptr, *d_kx = nullptr, *d_vCG = nullptr, *d_vcq = nullptr, *d_kern = nullptr;
  double *d_vion = nullptr, *d_vloc = nullptr, *d_rho = nullptr, *d_scal = nullptr, *d_out = nullptr;
  double* d_dpart = nullptr;  // [kDensChunks][NG] density partials
  // state
  double2 *d_u = nullptr, *d_us = nullptr, *d_k[4] = {nullptr, nullptr, nullptr, nullptr};
  double2* d_hpre = nullptr;  // T_A w + vloc w of an RK4 stage, made beside the exchange
  // staging for host-array entry points
  double2 *d_a = nullptr, *d_b = nullptr, *d_c = nullptr;
  size_t stage_cap = 0;
  // Fock partial sums
  double2* d_scratch = nullptr;
  size_t scratch_cap = 0;
  double* d_colbuf = nullptr;
  size_t colbuf_cap = 0;
  double2* d_sym = nullptr;   // symmetric-exchange tile partials
  size_t sym_cap = 0;
  double2* d_symF = nullptr;  // reduced symmetric exchange [NK*NBocc][NG]
  float4* d_udf = nullptr;    // double-float copy of the occupied orbitals
  float2* d_kern_df = nullptr;
  float4* d_tw_df = nullptr;
  int opt_df = 0;             // exchange transforms in double-float arithmetic
  int opt_tile = 0;           // symmetric-exchange tile size (0 = automatic)
  int opt_small = 2;          // fused small-problem RK4 stages: 0 off, 1 on, 2 automatic
  int opt_small_ctas = 0;     // CTAs per column of the fused stages (0 = automatic)
  bool step_small = false;    // the captured step graph uses the fused stages
  unsigned* d_ticket = nullptr;  // completion counters of the fused stages [1 + NK*NB]
  double2* d_small_part = nullptr;  // exchange partials of the fused stages
  size_t small_part_cap = 0;
  int small_P = 1;                // CTAs per column of the fused stages
  int small_P_adj = 1;            // CTAs per column of the fused reverse stages
  double* d_small_obs = nullptr;  // [2][NG] density and vH of a fused step's input (observables)
  int nsm = 0;                    // multiprocessors of the device
  int* d_int = nullptr;  // [0] = step counter, [1] = non-finite flag, [2] = solver flag,
                         // [3] = the fused stages' shadow of the step counter
  // RT series
  double *d_A = nullptr, *d_Aave = nullptr, *d_sE = nullptr, *d_sJ = nullptr, *d_sN = nullptr;
  int series_cap = 0;
  // GS work
  double2 *d_work = nullptr, *d_hwork = nullptr, *d_M = nullptr, *d_V = nullptr;
  double* d_evals = nullptr;
  size_t gs_cap = 0;
  double *d_eps = nullptr, *d_err = nullptr;
  // options
  int opt_graph = 1, opt_chunks = 0, opt_timing = 0, opt_sym = 1;
  long long opt_flush = 0;            // bytes written between timed RK4 steps (0 = no flush)
  void* d_flush = nullptr;
  size_t flush_cap = 0;
  std::vector<cudaEvent_t> step_events;
  // adjoint work
  double2 *d_ckpt = nullptr, *d_store = nullptr, *d_lam = nullptr, *d_lamu = nullptr, *d_vbuf = nullptr,
          *d_Fa = nullptr, *d_uN = nullptr, *d_u0 = nullptr;
  double2* d_lamk[4] = {nullptr, nullptr, nullptr, nullptr};
  double *d_psi = nullptr, *d_sig = nullptr, *d_gcol = nullptr, *d_gstage = nullptr, *d_gvion = nullptr,
         *d_vloc_adj = nullptr, *d_dpart2 = nullptr;
  int* d_adj_int = nullptr;  // [0] step n, [1] segment start
  double last_adj_ms = 0, last_adj_fwd_ms = 0;
  // graph of one RK4 step
  cudaGraphExec_t step_exec = nullptr;
  cudaGraphExec_t multi_exec = nullptr;  // kGraphSteps steps in one graph
  double step_dt = 0;
  // timing
  double last_run_ms = 0, last_fock_ms = 0;
  int last_fock_launches = 0;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> fock_events;
  size_t fock_event_used = 0;
  bool capturing = false;
  std::string err;
};

namespace {

void destroy_graph(mattohf_ctx* c);

int fail(mattohf_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

#define CK(call)                                                                        \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return fail(ctx, MATTOHF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define CKR(expr)              \
  do {                         \
    int r_ = (expr);           \
    if (r_ != MATTOHF_OK) return r_; \
  } while (0)

template <typename T>
int dalloc(mattohf_ctx* ctx, T** p, size_t n) {
  if (*p) {
    cudaFree(*p);
    *p = nullptr;
  }
  if (n == 0) return MATTOHF_OK;
  cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    return fail(ctx, MATTOHF_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  return MATTOHF_OK;
}

size_t orb_elems(const mattohf_ctx* c, int nb) { return (size_t)c->NK * nb * c->NG; }

int ensure_stage(mattohf_ctx* ctx, size_t elems) {
  if (elems <= ctx->stage_cap) return MATTOHF_OK;
  CKR(dalloc(ctx, &ctx->d_a, elems));
  CKR(dalloc(ctx, &ctx->d_b, elems));
  CKR(dalloc(ctx, &ctx->d_c, elems));
  ctx->stage_cap = elems;
  return MATTOHF_OK;
}

// Pair chunking of the Fock kernel: enough items to fill the device's SMs
// eight times over, each chunk a whole number of team rounds.
void fock_split(const mattohf_ctx* c, int ncols, int* nchunks, int* chunk) {
  const int npairs = c->NK * c->NBocc;
  int nch = c->opt_chunks;
  if (nch <= 0) {
    const int target = std::max(1, c->nsm) * 8;
    nch = (target + ncols - 1) / ncols;
  }
  nch = std::max(1, std::min(nch, npairs));
  int ch = (npairs + nch - 1) / nch;
  nch = (npairs + ch - 1) / ch;
  *nchunks = nch;
  *chunk = ch;
}

int ensure_scratch(mattohf_ctx* ctx, int ncols) {
  int nch, ch;
  fock_split(ctx, ncols, &nch, &ch);
  const size_t need = (size_t)ncols * nch * ctx->NG;
  if (need > ctx->scratch_cap) {
    if (ctx->capturing) return fail(ctx, MATTOHF_ERR_STATE, "scratch growth during capture");
    destroy_graph(ctx);  // the captured step holds the old pointer
    CKR(dalloc(ctx, &ctx->d_scratch, need));
    ctx->scratch_cap = need;
  }
  const size_t cb = (size_t)ncols * 4;
  if (cb > ctx->colbuf_cap) {
    if (ctx->capturing) return fail(ctx, MATTOHF_ERR_STATE, "colbuf growth during capture");
    destroy_graph(ctx);
    CKR(dalloc(ctx, &ctx->d_colbuf, cb));
    ctx->colbuf_cap = cb;
  }
  return MATTOHF_OK;
}

AField aval(double A) {
  AField f;
  f.mode = AVAL;
  f.val = A;
  f.A = nullptr;
  f.Aave = nullptr;
  f.it = nullptr;
  return f;
}

int enq_density(mattohf_ctx* ctx, Block u, cudaStream_t st = nullptr) {
  DensArgs a;
  a.u = u;
  a.nbocc = ctx->NBocc;
  a.occ = ctx->occ;
  a.vCG = ctx->d_vCG;
  a.vion = ctx->d_vion;
  a.tw = ctx->tw;
  a.dvcell = ctx->dvcell;
  a.rho = ctx->d_rho;
  a.vloc = ctx->d_vloc;
  a.scal = ctx->d_scal;
  a.nk = ctx->NK;
  a.part = ctx->d_dpart;
  a.mu = nullptr;
  a.gvion = nullptr;
  CK(launch_density(ctx->NG, a, st ? st : ctx->st));
  return MATTOHF_OK;
}

// Which exchange partials a combine launch reads.
struct FockPlan {
  int nchunks = 1;            // chunked partials per column (bands >= b0)
  int b0 = 0;                 // first band served by the chunked partials
  const double2* sym = nullptr;
  int S = 0, T = 0;
  bool any = false;           // exchange present at all
};

int ensure_sym(mattohf_ctx* ctx, size_t need) {
  if (need <= ctx->sym_cap) return MATTOHF_OK;
  if (ctx->capturing) return fail(ctx, MATTOHF_ERR_STATE, "sym scratch growth during capture");
  destroy_graph(ctx);
  CKR(dalloc(ctx, &ctx->d_sym, need));
  ctx->sym_cap = need;
  return MATTOHF_OK;
}

// A CUDA event destroyed on every exit path of the function that made it.
struct ScopedEvent {
  cudaEvent_t e = nullptr;
  cudaError_t create() { return cudaEventCreate(&e); }
  ~ScopedEvent() {
    if (e) cudaEventDestroy(e);
  }
  operator cudaEvent_t() const { return e; }
};

int timed_begin(mattohf_ctx* ctx) {
  if (!(ctx->opt_timing && !ctx->capturing)) return MATTOHF_OK;
  if (ctx->fock_event_used == ctx->fock_events.size()) {
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    ctx->fock_events.push_back({e0, e1});
  }
  CK(cudaEventRecord(ctx->fock_events[ctx->fock_event_used].first, ctx->st));
  return MATTOHF_OK;
}

int timed_end(mattohf_ctx* ctx) {
  if (!(ctx->opt_timing && !ctx->capturing)) return MATTOHF_OK;
  CK(cudaEventRecord(ctx->fock_events[ctx->fock_event_used].second, ctx->st));
  ctx->fock_event_used++;
  return MATTOHF_OK;
}

// RK4 steps captured in one graph for mattohf_rk4_run (divides 256)
constexpr int kGraphSteps = 8;

int sym_tile(const mattohf_ctx* ctx) {
  return ctx->opt_tile > 0 ? ctx->opt_tile : choose_sym_tile(ctx->NG, ctx->NK * ctx->NBocc, ctx->nsm);
}

// Every buffer the RK4 step's exchange applies need, allocated up front so a
// graph capture never has to grow one.
int ensure_fock_buffers(mattohf_ctx* ctx) {
  CKR(ensure_scratch(ctx, ctx->NK * ctx->NB));
  const int M = ctx->NK * ctx->NBocc;
  const int S = sym_tile(ctx);
  const int T = (M + S - 1) / S;
  CKR(ensure_sym(ctx, (size_t)T * (T + 1) / 2 * 2 * S * ctx->NG));
  if (!ctx->d_symF) CKR(dalloc(ctx, &ctx->d_symF, (size_t)M * ctx->NG));
  if (!ctx->d_udf) CKR(dalloc(ctx, &ctx->d_udf, (size_t)M * ctx->NG));
  return MATTOHF_OK;
}

// Exchange partials of h[u] w.  When w is u itself (all RK4 stages, Ex,
// Subspace_diag, eps) the occupied rows use the symmetric pair kernel and only
// the unoccupied rows (if any) take the chunked kernel.
int enq_fock(mattohf_ctx* ctx, Block u, Block w, FockPlan* plan) {
  *plan = FockPlan();
  plan->any = true;
  const bool same = (w.p == u.p) && (w.kstride == u.kstride) && (w.nb == u.nb);
  const int NG = ctx->NG;
  if (same && ctx->opt_sym) {
    const int M = ctx->NK * ctx->NBocc;
    const int S = sym_tile(ctx);
    const int T = (M + S - 1) / S;
    CKR(ensure_sym(ctx, (size_t)T * (T + 1) / 2 * 2 * S * NG));
    if (!ctx->d_symF) CKR(dalloc(ctx, &ctx->d_symF, (size_t)M * NG));
    FockSymArgs a;
    a.u = u;
    a.nk = ctx->NK;
    a.nbocc = ctx->NBocc;
    a.S = S;
    a.T = T;
    a.kern = ctx->d_kern;
    a.tw = ctx->tw;
    a.scratch = ctx->d_sym;
    a.F = ctx->d_symF;
    CKR(timed_begin(ctx));
    if (ctx->opt_df) {
      if (!ctx->d_udf) CKR(dalloc(ctx, &ctx->d_udf, (size_t)M * NG));
      FockSymDfArgs d;
      d.u = ctx->d_udf;
      d.nk = ctx->NK;
      d.nbocc = ctx->NBocc;
      d.S = S;
      d.T = T;
      d.kern = ctx->d_kern_df;
      d.tw = ctx->d_tw_df;
      d.scratch = reinterpret_cast<float4*>(ctx->d_sym);  // same 16-byte elements
      d.F = ctx->d_symF;
      CK(launch_fock_sym_df(NG, d, u.p, u.kstride, ctx->d_udf, ctx->st));
    } else {
      CK(launch_fock_sym(NG, a, ctx->st));
    }
    CKR(timed_end(ctx));
    plan->sym = ctx->d_symF;
    plan->S = S;
    plan->T = T;
    plan->b0 = ctx->NBocc;
    if (w.nb == ctx->NBocc) return MATTOHF_OK;
  }
  Block wr = w;
  wr.p = w.p + (size_t)plan->b0 * NG;
  wr.nb = w.nb - plan->b0;
  const int ncols = ctx->NK * wr.nb;
  CKR(ensure_scratch(ctx, ncols));
  FockArgs a;
  a.u = u;
  a.w = wr;
  a.nk = ctx->NK;
  a.nbocc = ctx->NBocc;
  a.kern = ctx->d_kern;
  a.tw = ctx->tw;
  a.scratch = ctx->d_scratch;
  fock_split(ctx, ncols, &a.nchunks, &a.chunk);
  plan->nchunks = a.nchunks;
  CKR(timed_begin(ctx));
  CK(launch_fock(ctx->NG, a, ncols, ctx->st));
  CKR(timed_end(ctx));
  return MATTOHF_OK;
}

CombineArgs combine_base(mattohf_ctx* ctx, Block w, AField af, int mode, const FockPlan& fp) {
  CombineArgs a;
  std::memset(&a, 0, sizeof(a));
  a.w = w;
  const bool ex = ctx->hf && mode != CM_T && fp.any;
  a.scratch = ex ? ctx->d_scratch : nullptr;
  a.sym = ex ? fp.sym : nullptr;
  a.sym_S = fp.S;
  a.sym_T = fp.T;
  a.chunk_b0 = fp.b0;
  a.nchunks = fp.nchunks;
  a.vloc = ctx->d_vloc;
  a.Gx = ctx->d_Gx;
  a.kx = ctx->d_kx;
  a.tw = ctx->tw;
  a.af = af;
  a.mode = mode;
  a.nk = ctx->NK;
  a.nbocc = ctx->NBocc;
  a.occ = ctx->occ;
  a.colbuf = ctx->d_colbuf;
  a.nonfinite = ctx->d_int + 1;
  a.u0 = ctx->d_u;
  for (int s = 0; s < 4; ++s) a.kbuf[s] = ctx->d_k[s];
  return a;
}

// h[u] w -> out  (mode CM_H), or the exchange / kinetic term alone.
int enq_hpsi(mattohf_ctx* ctx, Block u, Block w, BlockOut out, AField af, int mode) {
  FockPlan fp;
  if (mode == CM_H) CKR(enq_density(ctx, u));
  if (ctx->hf && mode != CM_T) CKR(enq_fock(ctx, u, w, &fp));
  else if (mode == CM_F) {
    CK(cudaMemsetAsync(out.p, 0, sizeof(double2) * (size_t)ctx->NK * out.kstride, ctx->st));
    return MATTOHF_OK;
  }
  CKR(ensure_scratch(ctx, ctx->NK * w.nb));
  CombineArgs a = combine_base(ctx, w, af, mode, fp);
  a.out = out;
  CK(launch_combine(ctx->NG, a, ctx->NK * w.nb, ctx->st));
  return MATTOHF_OK;
}

Block blk(const double2* p, int ld, int NG, int nb) {
  Block b;
  b.p = p;
  b.kstride = ld * NG;
  b.nb = nb;
  return b;
}
BlockOut blko(double2* p, int ld, int NG, int nb) {
  BlockOut b;
  b.p = p;
  b.kstride = ld * NG;
  b.nb = nb;
  return b;
}

// Observables of `u` at field af (RT:43-47): density scalars, Fock partials,
// per-column Ekin/Je/<u|F u>, then the ordered reduction.
// With `defer_ex` the exchange energy is left out of Etot (and no Fock apply
// is made); the next RK4 step's first stage, which applies the exchange
// operator of the same orbitals, adds it (k_ex_finalize).
int enq_observables(mattohf_ctx* ctx, const double2* u, AField af, bool advance, bool defer_ex,
                    FockPlan* plan_out = nullptr) {
  const int NG = ctx->NG, NB = ctx->NB;
  Block ub = blk(u, NB, NG, NB);
  CKR(enq_density(ctx, ub));
  FockPlan fp;
  fp.any = false;
  if (ctx->hf && !defer_ex) CKR(enq_fock(ctx, ub, ub, &fp));
  CKR(ensure_scratch(ctx, ctx->NK * NB));
  if (plan_out) *plan_out = fp;
  CombineArgs a = combine_base(ctx, ub, af, CM_OBS, fp);
  CK(launch_combine(NG, a, ctx->NK * NB, ctx->st));
  ObsReduceArgs r;
  r.colbuf = ctx->d_colbuf;
  r.scal = ctx->d_scal;
  r.nk = ctx->NK;
  r.nb = NB;
  r.nbocc = ctx->NBocc;
  r.occ = ctx->occ;
  r.dvcell = ctx->dvcell;
  r.vcell = ctx->vcell;
  r.NGd = (double)NG;
  r.hf = ctx->hf;
  r.defer_ex = defer_ex ? 1 : 0;
  r.out = ctx->d_out;
  r.series_E = advance ? ctx->d_sE : nullptr;
  r.series_J = advance ? ctx->d_sJ : nullptr;
  r.series_N = advance ? ctx->d_sN : nullptr;
  r.it = ctx->d_int;
  r.advance = advance ? 1 : 0;
  r.nonfinite = ctx->d_int + 1;
  CK(launch_obs_reduce(r, ctx->st));
  return MATTOHF_OK;
}

// One RK4 step (RT:165-170); fields either from host values or from the
// device series indexed by the device step counter.
ExArgs ex_args(mattohf_ctx* ctx, double* series, int idx, double* out) {
  ExArgs e;
  e.colbuf = ctx->d_colbuf;
  e.nk = ctx->NK;
  e.nb = ctx->NB;
  e.nbocc = ctx->NBocc;
  e.occ = ctx->occ;
  e.dvcell = ctx->dvcell;
  e.series_E = series;
  e.it = ctx->d_int;
  e.idx = idx;
  e.out = out;
  return e;
}

// One RK4 step (RT:165-170); fields either from host values or from the
// device series indexed by the device step counter.  With `ex_series` the
// first stage also completes Etot(it-1) with the exchange energy of the
// step's input orbitals (the same exchange operator the stage applies).
int launch_store_stage(mattohf_ctx* ctx, const double2* src, int slot);

// One RK4 step.  With `store`, the four stage inputs also go to the adjoint's
// stage store at slot (it - seg0) * 4 + s.
int enq_rk4(mattohf_ctx* ctx, AField f_m, AField f_ave, AField f_cur, double dt,
            double* ex_series = nullptr, bool store = false) {
  const int NG = ctx->NG, NB = ctx->NB;
  const int modes[4] = {CM_RK0, CM_RK1, CM_RK2, CM_RK3};
  const AField fs[4] = {f_m, f_ave, f_ave, f_cur};
  CKR(ensure_scratch(ctx, ctx->NK * NB));
  if (store) CKR(launch_store_stage(ctx, ctx->d_u, 0));
  for (int s = 0; s < 4; ++s) {
    const double2* in = (s == 0) ? ctx->d_u : ctx->d_us;
    Block ub = blk(in, NB, NG, NB);
    FockPlan fp;
    const bool side = ctx->hf != 0;
    if (side) {
      // The density and the kinetic + local-potential part of h w need only
      // the stage input: they run on the side stream beside the exchange.
      CK(cudaEventRecord(ctx->ev_fork, ctx->st));
      CK(cudaStreamWaitEvent(ctx->st_side, ctx->ev_fork, 0));
      CKR(enq_density(ctx, ub, ctx->st_side));
      CombineArgs pre = combine_base(ctx, ub, fs[s], modes[s], FockPlan());
      pre.split = 1;
      pre.hpre = ctx->d_hpre;
      CK(launch_combine(NG, pre, ctx->NK * NB, ctx->st_side));
      CK(cudaEventRecord(ctx->ev_join, ctx->st_side));
      CKR(enq_fock(ctx, ub, ub, &fp));
      CK(cudaStreamWaitEvent(ctx->st, ctx->ev_join, 0));
    } else {
      CKR(enq_density(ctx, ub));
    }
    CombineArgs a = combine_base(ctx, ub, fs[s], modes[s], fp);
    a.out = blko(ctx->d_us, NB, NG, NB);
    a.dt = dt;
    a.ex_cols = (s == 0 && ex_series != nullptr && ctx->hf) ? 1 : 0;
    if (side) {
      a.split = 2;
      a.hpre = ctx->d_hpre;
    }
    CK(launch_combine(NG, a, ctx->NK * NB, ctx->st));
    if (a.ex_cols) CK(launch_ex_finalize(ex_args(ctx, ex_series, -1, nullptr), ctx->st));
    if (store && s < 3) CKR(launch_store_stage(ctx, ctx->d_us, s + 1));
  }
  return MATTOHF_OK;
}

// Fused small-problem stages: is this context's RK loop better served by
// one launch per stage (one CTA per column) than by the tiled exchange?
bool use_small(const mattohf_ctx* ctx) {
  if (ctx->opt_small == 0 || ctx->opt_df || ctx->opt_timing || !small_stage_supported(ctx->NG)) return false;
  if (ctx->opt_small == 1) return true;
  // measured on GB300 with mattohf_autotune (us per step, fused vs tiled):
  // NG=64 NK=8 Nocc=2 29 vs 129; NG=128 NK=16 Nocc=2 and NK=8 Nocc=4 96 vs 235
  // (M^2 NG = 2^17); NG=64 NK=16 Nocc=4 171 vs 156, NG=64 NK=32 Nocc=2 173 vs
  // 158 (2^18); NG=256 NK=8 Nocc=4 178 vs 253 (2^18, M = 32); NG=128 NK=32
  // Nocc=2 320 vs 285 (2^19)
  const size_t M = (size_t)ctx->NK * ctx->NBocc;
  if (ctx->NK * ctx->NB > 64) return false;
  return M * M * ctx->NG <= ((size_t)1 << 17) || (ctx->NG == 256 && M <= 32);
}

// CTAs per column.  A warp issues at most one FP64 instruction per ~64
// cycles and an SM about one per 19 cycles in all (measured on GB300 with
// independent FMA chains: 2 warps run at the single-warp rate, 4 at 76 cycles
// each, 8 at 152), so a pair chain is fastest with about 4 FP64-busy warps per
// SM.  With more than one CTA per column the first CTA takes no pairs (it
// carries the density, the kinetic and Hartree transforms), so with Q = the
// teams of 4 warps each of the other P - 1 CTAs takes up to Q pairs,
// P = 1 + ceil(M / Q), unless that needs more CTAs than there are
// multiprocessors.
int small_ctas_per_column(const mattohf_ctx* ctx) {
  const int ncols = ctx->NK * ctx->NB, M = ctx->NK * ctx->NBocc;
  const int pair_teams = small_pair_teams(ctx->NG);   // 6 warps' teams
  if (ctx->opt_small_ctas > 0)  // set (or tuned): at most M and a cluster's CTAs
    return std::max(1, std::min(std::min(ctx->opt_small_ctas, std::max(1, M)), kSmallMaxCtas));
  const int Q = std::max(1, 4 * (pair_teams / 6));
  const int full = std::max(1, 8 * (pair_teams / 6));  // teams of a CTA's eight warps
  int P = 1 + (M + Q - 1) / Q;
  if (ncols * P > ctx->nsm) P = std::max(1, ctx->nsm / ncols);
  // one round of the pair teams at most
  if ((P == 1 && M > pair_teams) || (P > 1 && (P - 1) * full < M)) P = 1 + (M + full - 1) / full;
  return std::max(1, std::min(std::min(P, std::max(1, M)), kSmallMaxCtas));  // one cluster per column
}

// CTAs per column of the fused reverse stages: one round of the pass teams
// (each orbital b takes a pass-A and a pass-B team), unless that needs more
// CTAs than there are multiprocessors.
// CTAs per column of the fused reverse stage.  The stage is bound by each
// SM's FP64 rate, and two of its CTAs fit on an SM (128 registers x 256
// threads), so the columns' CTAs are spread until they fill every SM twice:
// at NK = 16, Nocc = 2 (32 columns) that is 9 CTAs per column on all 152 SMs
// rather than 4 on 128 (reverse sweep 1625 -> 1469 ms over 4000 steps).
int small_adj_ctas_per_column(const mattohf_ctx* ctx) {
  const int ncols = ctx->NK * ctx->NB, M = ncols;
  const int per_round = std::max(1, small_adj_pair_warps_teams(ctx->NG));
  const int slots = 2 * std::max(1, ctx->nsm);
  int P = std::max((M + per_round - 1) / per_round, slots / ncols);
  if (ncols * P > slots) P = std::max(1, slots / ncols);
  return std::max(1, std::min(P, M));
}

// Buffers of the fused stages, sized before any capture.
int ensure_small_buffers(mattohf_ctx* ctx) {
  ctx->small_P = small_ctas_per_column(ctx);
  ctx->small_P_adj = small_adj_ctas_per_column(ctx);
  // partials [ncols][P][NG], then (rho, vH) and the kinetic term, [ncols][NG] each
  const size_t need = (size_t)ctx->NK * ctx->NB * (std::max(ctx->small_P, ctx->small_P_adj) + 2) * ctx->NG;
  if (need > ctx->small_part_cap) {
    if (ctx->capturing) return fail(ctx, MATTOHF_ERR_STATE, "fused-stage scratch growth during capture");
    destroy_graph(ctx);  // a captured step holds the old pointer
    CKR(dalloc(ctx, &ctx->d_small_part, need));
    ctx->small_part_cap = need;
  }
  if (!ctx->d_small_obs) {
    if (ctx->capturing) return fail(ctx, MATTOHF_ERR_STATE, "fused-stage scratch growth during capture");
    CKR(dalloc(ctx, &ctx->d_small_obs, 2 * (size_t)ctx->NG));
  }
  return MATTOHF_OK;
}

SmallStageArgs small_base(mattohf_ctx* ctx, double dt) {
  SmallStageArgs a;
  std::memset(&a, 0, sizeof(a));
  a.u0 = ctx->d_u;
  for (int s = 0; s < 3; ++s) a.kbuf[s] = ctx->d_k[s];
  a.dt = dt;
  a.nk = ctx->NK;
  a.nb = ctx->NB;
  a.nbocc = ctx->NBocc;
  a.hf = ctx->hf;
  a.occ = ctx->occ;
  a.dvcell = ctx->dvcell;
  a.vcell = ctx->vcell;
  a.kern = ctx->d_kern;
  a.vCG = ctx->d_vCG;
  a.vion = ctx->d_vion;
  a.Gx = ctx->d_Gx;
  a.kx = ctx->d_kx;
  a.tw = ctx->tw;
  a.P = ctx->small_P;
  a.part = ctx->d_small_part;
  a.Aobs = ctx->d_A;
  a.colbuf = ctx->d_colbuf;
  a.series_E = ctx->d_sE;
  a.series_J = ctx->d_sJ;
  a.series_N = ctx->d_sN;
  a.it = ctx->d_int;
  a.nonfinite = ctx->d_int + 1;
  a.ticket = ctx->d_ticket;
  a.obs_dens = ctx->d_small_obs;
  return a;
}

// One RK4 step as four fused stage launches.  Stage inputs and outputs
// alternate between d_us and d_hpre so that no launch writes its own input.
// Stage 0 also writes the observables of the previous step (its input).
// With `store`, each stage input also goes to the adjoint's stage store (the
// stage kernel copies it).
// The step counter d_int[0] holds the step index between steps (the host,
// the checkpoint and store copies read and set it there).  Stage 0 copies it
// to the shadow d_int[3]; stage 3 reads its field at the shadow's index and
// writes index + 1 to d_int[0], which none of its CTAs reads.
// With `ckpt_every` > 0, stage 0 also writes its input to checkpoint
// (it + ckpt_phase) / ckpt_every when it is a segment start (as k_checkpoint).
int enq_small_step(mattohf_ctx* ctx, AField f_m, AField f_ave, AField f_cur, double dt, bool store = false,
                   int ckpt_every = 0, int ckpt_phase = 0) {
  SmallStageArgs a = small_base(ctx, dt);
  const double2* in[4] = {ctx->d_u, ctx->d_us, ctx->d_hpre, ctx->d_us};
  double2* out[4] = {ctx->d_us, ctx->d_hpre, ctx->d_us, nullptr};
  AField fs[4] = {f_m, f_ave, f_ave, f_cur};
  int* const shadow = ctx->d_int + 3;
  fs[3].it = shadow;
  for (int s = 0; s < 4; ++s) {
    // with `store`, each stage copies its input into the adjoint's stage
    // store itself (no separate copy launch between the stages)
    a.store = store ? ctx->d_store : nullptr;
    a.seg0 = ctx->d_adj_int + 1;
    a.store_slot = s;
    a.ckpt = (ckpt_every > 0 && s == 0) ? ctx->d_ckpt : nullptr;
    a.ckpt_every = ckpt_every;
    a.ckpt_phase = ckpt_phase;
    a.u = in[s];
    a.out = out[s];
    a.mode = s;
    a.af = fs[s];
    a.it = s == 3 ? shadow : ctx->d_int;
    a.it_out = s == 0 ? shadow : s == 3 ? ctx->d_int : nullptr;
    a.it_inc = s == 3 ? 1 : 0;
    CK(launch_small_stage(ctx->NG, a, ctx->st));
  }
  return MATTOHF_OK;
}

// Observables of the last step's orbitals (the stage-0 launch that would
// supply them does not happen).
int enq_small_close(mattohf_ctx* ctx) {
  SmallStageArgs a = small_base(ctx, 0.0);
  a.u = ctx->d_u;
  a.mode = 4;
  a.af = aval(0.0);
  a.out_obs = ctx->d_out;
  CK(launch_small_stage(ctx->NG, a, ctx->st));
  return MATTOHF_OK;
}

int check_ctx(mattohf_ctx* ctx) {
  if (!ctx) return MATTOHF_ERR_ARG;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return fail(ctx, MATTOHF_ERR_CUDA, cudaGetErrorString(e));
  return MATTOHF_OK;
}

int sync_and_flag(mattohf_ctx* ctx) {
  CK(cudaStreamSynchronize(ctx->st));
  return MATTOHF_OK;
}

void destroy_graph(mattohf_ctx* c) {
  if (c->step_exec) {
    cudaGraphExecDestroy(c->step_exec);
    c->step_exec = nullptr;
  }
  if (c->multi_exec) {
    cudaGraphExecDestroy(c->multi_exec);
    c->multi_exec = nullptr;
  }
}

// Coulomb tables already built in this process, by (acell, NG, NK): runs that
// share a cell (pulse variants, repeated contexts) reuse the k_vCk sums, which
// at NG = 512, NK = 128 take 1.7e11 terms.  Values are the kernel's own output,
// bit for bit.  At most kTableCacheMax entries (1 MiB each at that size).
constexpr size_t kTableCacheMax = 64;
std::mutex g_table_mu;
std::map<std::tuple<uint64_t, int, int>, std::vector<double>> g_tables;

int compute_tables(mattohf_ctx* ctx) {
  const int NG = ctx->NG, NK = ctx->NK;
  const int nd = 2 * NK - 1;
  uint64_t abits = 0;
  std::memcpy(&abits, &ctx->acell, sizeof abits);
  const auto key = std::make_tuple(abits, NG, NK);
  std::vector<double> cached;
  {
    std::lock_guard<std::mutex> lk(g_table_mu);
    auto it = g_tables.find(key);
    if (it != g_tables.end()) cached = it->second;
  }
  std::vector<double> q((size_t)nd * NG + NG);
  for (int d = 0; d < nd; ++d) {
    const int diff = d - (NK - 1);              // kr - kc
    const int kr = std::max(0, diff);
    const int kc = kr - diff;
    for (int g = 0; g < NG; ++g) q[(size_t)d * NG + g] = (ctx->Gx[g] + ctx->kx[kr]) - ctx->kx[kc];
  }
  for (int g = 0; g < NG; ++g) q[(size_t)nd * NG + g] = ctx->Gx[g];
  double* d_q = nullptr;
  double* d_all = nullptr;
  double* d_g = nullptr;
  CKR(dalloc(ctx, &d_all, q.size()));
  if (cached.size() == q.size()) {
    CK(cudaMemcpyAsync(d_all, cached.data(), q.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
  } else {
    CKR(dalloc(ctx, &d_q, q.size()));
    CKR(dalloc(ctx, &d_g, (size_t)vck_points(ctx->acell, NG, NK)));
    CK(cudaMemcpyAsync(d_q, q.data(), q.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
    CK(launch_vck_table(NG, NK, ctx->acell, d_q, (int)q.size(), d_g, d_all, ctx->st));
    std::vector<double> h(q.size());
    CK(cudaMemcpyAsync(h.data(), d_all, q.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    std::lock_guard<std::mutex> lk(g_table_mu);
    if (g_tables.size() >= kTableCacheMax) g_tables.clear();
    g_tables[key] = std::move(h);
  }
  CKR(dalloc(ctx, &ctx->d_vcq, (size_t)nd * NG));
  CKR(dalloc(ctx, &ctx->d_vCG, NG));
  CKR(dalloc(ctx, &ctx->d_kern, (size_t)nd * NG));
  CK(cudaMemcpyAsync(ctx->d_vcq, d_all, sizeof(double) * nd * NG, cudaMemcpyDeviceToDevice, ctx->st));
  CK(cudaMemcpyAsync(ctx->d_vCG, d_all + (size_t)nd * NG, sizeof(double) * NG,
                     cudaMemcpyDeviceToDevice, ctx->st));
  CK(cudaMemsetAsync(ctx->d_vCG, 0, sizeof(double), ctx->st));  // vCG(1) = 0 (I:146)
  CK(launch_make_kern(NG, NK, ctx->d_vcq, ctx->d_kern, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  cudaFree(d_q);
  cudaFree(d_all);
  cudaFree(d_g);
  return MATTOHF_OK;
}

void compute_vion(mattohf_ctx* c) {
  const int NG = c->NG;
  c->vion.assign(NG, 0.0);
  const double ax = c->acell;
  for (size_t ii = 0; ii < c->Rion.size(); ++ii) {
    const int sp = c->Kion[ii] - 1;
    const double Za = c->Zeff[sp], al = c->alpha[sp];
    for (int icell = -4 * c->NK; icell <= 4 * c->NK; ++icell) {
      for (int g = 0; g < NG; ++g) {
        const double dist = std::fabs(c->rx[g] - ax * c->Rion[ii] - ax * (double)icell);
        c->vion[g] = c->vion[g] - Za / std::sqrt(dist * dist + al * al);
      }
    }
  }
  double top = c->vion.empty() ? 0.0 : c->vion[0];
  for (double v : c->vion) top = std::max(top, v);
  for (double& v : c->vion) v = v - top;
}

// Chain rule from dL/dvion(x) to the parameters of the ion potential
// (src/Prep_periodic_ion_potential.f90:10-20):
//   vraw(x) = -sum_ii sum_icell Z_s / sqrt(d^2 + alpha_s^2),  d = x - a R_ii - a icell,
//   vion(x) = vraw(x) - max_x' vraw(x'),
// so dL/dp = sum_x g(x) dvraw(x)/dp - (sum_x g(x)) dvraw(x*)/dp, x* the grid
// point of the maximum.  The shift is differentiable wherever the maximum is
// attained at one grid point; at a tie the first such point in grid order is
// taken (one of the one-sided gradients).  Per ion and cell image, with
// r = (d^2 + alpha^2)^(-1/2):
//   dvraw/dZ_s = -r,  dvraw/dalpha_s = Z alpha r^3,  dvraw/dR_ii = -a Z d r^3.
void ion_param_grad(const mattohf_ctx* c, const double* g, double* dZ, double* dal, double* dR) {
  const int NG = c->NG;
  const double ax = c->acell;
  std::vector<double> vraw(NG, 0.0);
  for (size_t ii = 0; ii < c->Rion.size(); ++ii) {
    const int sp = c->Kion[ii] - 1;
    const double Za = c->Zeff[sp], al = c->alpha[sp];
    for (int icell = -4 * c->NK; icell <= 4 * c->NK; ++icell)
      for (int x = 0; x < NG; ++x) {
        const double dist = std::fabs(c->rx[x] - ax * c->Rion[ii] - ax * (double)icell);
        vraw[x] = vraw[x] - Za / std::sqrt(dist * dist + al * al);
      }
  }
  int xs = 0;
  for (int x = 1; x < NG; ++x)
    if (vraw[x] > vraw[xs]) xs = x;
  double gsum = 0.0;
  for (int x = 0; x < NG; ++x) gsum += g[x];
  const size_t ns = c->Zeff.size(), ni = c->Rion.size();
  std::fill(dZ, dZ + ns, 0.0);
  std::fill(dal, dal + ns, 0.0);
  std::fill(dR, dR + ni, 0.0);
  for (size_t ii = 0; ii < ni; ++ii) {
    const int sp = c->Kion[ii] - 1;
    const double Za = c->Zeff[sp], al = c->alpha[sp];
    double sZ = 0.0, sa = 0.0, sR = 0.0;
    for (int icell = -4 * c->NK; icell <= 4 * c->NK; ++icell)
      for (int x = 0; x < NG; ++x) {
        const double w = x == xs ? g[x] - gsum : g[x];
        const double d = c->rx[x] - ax * c->Rion[ii] - ax * (double)icell;
        const double r = 1.0 / std::sqrt(d * d + al * al), r3 = r * r * r;
        sZ += w * -r;
        sa += w * Za * al * r3;
        sR += w * -ax * Za * d * r3;
      }
    dZ[sp] += sZ;
    dal[sp] += sa;
    dR[ii] += sR;
  }
}

// The adjoint's segment storage (checkpoints and stage inputs), the only
// buffers of the adjoint that scale with the window.
void release_adjoint_storage(mattohf_ctx* ctx) {
  dalloc(ctx, &ctx->d_ckpt, 0);
  dalloc(ctx, &ctx->d_store, 0);
}

int ensure_series(mattohf_ctx* ctx, int nt) {
  if (nt <= ctx->series_cap) return MATTOHF_OK;
  destroy_graph(ctx);  // graph holds the old pointers
  CKR(dalloc(ctx, &ctx->d_A, nt));
  CKR(dalloc(ctx, &ctx->d_Aave, nt));
  CKR(dalloc(ctx, &ctx->d_sE, nt));
  CKR(dalloc(ctx, &ctx->d_sJ, nt));
  CKR(dalloc(ctx, &ctx->d_sN, nt));
  ctx->series_cap = nt;
  return MATTOHF_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* mattohf_status_string(int s) {
  switch (s) {
    case MATTOHF_OK: return "ok";
    case MATTOHF_ERR_ARG: return "invalid argument";
    case MATTOHF_ERR_CUDA: return "CUDA error";
    case MATTOHF_ERR_NONFINITE: return "non-finite state";
    case MATTOHF_ERR_TIMEOUT: return "device wait timed out";
    case MATTOHF_ERR_NOTCONV: return "not converged";
    case MATTOHF_ERR_ALLOC: return "device allocation failed";
    case MATTOHF_ERR_STATE: return "invalid state";
    case MATTOHF_ERR_TOO_LARGE: return "problem exceeds the fixed scratch size";
    default: return "unknown status";
  }
}

const char* mattohf_last_error(const mattohf_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int mattohf_create(const mattohf_config* cfg, mattohf_ctx** out) {
  if (!cfg || !out) return MATTOHF_ERR_ARG;
  *out = nullptr;
  const int NG = cfg->NG;
  if (!(NG == 16 || NG == 32 || NG == 64 || NG == 128 || NG == 256 || NG == 512)) return MATTOHF_ERR_ARG;
  if (cfg->NK < 1 || cfg->NB < 1 || cfg->NBocc < 1 || cfg->NBocc > cfg->NB) return MATTOHF_ERR_ARG;
  if (!(cfg->acell > 0.0) || !std::isfinite(cfg->acell)) return MATTOHF_ERR_ARG;
  if (cfg->nion < 0 || cfg->nspecies < 0) return MATTOHF_ERR_ARG;
  if (cfg->nspecies > 0 && (!cfg->Zeff || !cfg->alpha)) return MATTOHF_ERR_ARG;
  if (cfg->nion > 0 && (!cfg->Rion || !cfg->Kion || !cfg->Zeff || !cfg->alpha)) return MATTOHF_ERR_ARG;
  for (int i = 0; i < cfg->nion; ++i)
    if (cfg->Kion[i] < 1 || cfg->Kion[i] > cfg->nspecies) return MATTOHF_ERR_ARG;
  if ((long long)cfg->NK * cfg->NB * NG > (1LL << 28)) return MATTOHF_ERR_ARG;

  mattohf_ctx* ctx = new mattohf_ctx();
  ctx->NG = NG;
  ctx->NK = cfg->NK;
  ctx->NB = cfg->NB;
  ctx->NBocc = cfg->NBocc;
  ctx->hf = cfg->functional_hf ? 1 : 0;
  ctx->device = cfg->device;
  ctx->acell = cfg->acell;
  ctx->Zeff.assign(cfg->Zeff, cfg->Zeff + cfg->nspecies);
  ctx->alpha.assign(cfg->alpha, cfg->alpha + cfg->nspecies);
  ctx->Rion.assign(cfg->Rion, cfg->Rion + cfg->nion);
  ctx->Kion.assign(cfg->Kion, cfg->Kion + cfg->nion);
  // cell and grids (I:46-49, I:62, I:93-112)
  ctx->vcell = std::fabs(cfg->acell);
  ctx->bx = 2.0 * kPi / cfg->acell;
  ctx->dvcell = ctx->vcell / (double)NG;
  ctx->occ = 2.0 / (double)cfg->NK;
  ctx->rx.resize(NG);
  ctx->Gx.resize(NG);
  for (int i = 0; i < NG; ++i) {
    ctx->rx[i] = (double)i / (double)NG * cfg->acell;
    ctx->Gx[i] = (i < NG / 2 ? (double)i : (double)(i - NG)) * ctx->bx;
  }
  ctx->kx.resize(cfg->NK);
  for (int i = 1; i <= cfg->NK; ++i)
    ctx->kx[i - 1] = (-0.5 + (2.0 * i - 1.0) / (double)(2 * cfg->NK)) * ctx->bx;
  compute_vion(ctx);

  int rc = MATTOHF_OK;
  auto bail = [&](int r) {
    mattohf_destroy(ctx);
    return r;
  };
  {
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return bail(MATTOHF_ERR_CUDA);
    e = cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->st_side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming);
    if (e != cudaSuccess) return bail(MATTOHF_ERR_CUDA);
    e = configure_kernels();
    if (e == cudaSuccess) e = configure_adjoint_kernels();
    if (e == cudaSuccess) e = configure_df_kernels();
    if (e == cudaSuccess) e = configure_small_kernels();
    if (e == cudaSuccess) e = configure_small_adj_kernels();
    if (e != cudaSuccess) return bail(MATTOHF_ERR_CUDA);
  }
  const size_t nu = orb_elems(ctx, ctx->NB);
  if ((rc = dalloc(ctx, &ctx->tw, NG)) || (rc = dalloc(ctx, &ctx->d_Gx, NG)) ||
      (rc = dalloc(ctx, &ctx->d_kx, ctx->NK)) || (rc = dalloc(ctx, &ctx->d_vion, NG)) ||
      (rc = dalloc(ctx, &ctx->d_vloc, NG)) || (rc = dalloc(ctx, &ctx->d_rho, NG)) ||
      (rc = dalloc(ctx, &ctx->d_scal, 8)) || (rc = dalloc(ctx, &ctx->d_out, 8)) ||
      (rc = dalloc(ctx, &ctx->d_u, nu)) || (rc = dalloc(ctx, &ctx->d_us, nu)) ||
      (rc = dalloc(ctx, &ctx->d_int, 8)) || (rc = dalloc(ctx, &ctx->d_dpart, (size_t)kDensChunks * NG)))
    return bail(rc);
  for (int s = 0; s < 4; ++s)
    if ((rc = dalloc(ctx, &ctx->d_k[s], nu))) return bail(rc);
  if ((rc = dalloc(ctx, &ctx->d_hpre, nu))) return bail(rc);
  const size_t ntick = 1 + (size_t)ctx->NK * ctx->NB;
  if (cudaMalloc(&ctx->d_ticket, sizeof(unsigned) * ntick) != cudaSuccess ||
      cudaMemset(ctx->d_ticket, 0, sizeof(unsigned) * ntick) != cudaSuccess ||
      cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess)
    return bail(MATTOHF_ERR_ALLOC);
  if (cudaMemsetAsync(ctx->d_u, 0, nu * sizeof(double2), ctx->st) != cudaSuccess ||
      cudaMemsetAsync(ctx->d_int, 0, 8 * sizeof(int), ctx->st) != cudaSuccess ||
      cudaMemcpyAsync(ctx->d_Gx, ctx->Gx.data(), NG * sizeof(double), cudaMemcpyHostToDevice, ctx->st) != cudaSuccess ||
      cudaMemcpyAsync(ctx->d_kx, ctx->kx.data(), ctx->NK * sizeof(double), cudaMemcpyHostToDevice, ctx->st) != cudaSuccess ||
      cudaMemcpyAsync(ctx->d_vion, ctx->vion.data(), NG * sizeof(double), cudaMemcpyHostToDevice, ctx->st) != cudaSuccess)
    return bail(MATTOHF_ERR_CUDA);
  k_twiddles<<<(NG + 127) / 128, 128, 0, ctx->st>>>(ctx->tw, NG);
  if (cudaGetLastError() != cudaSuccess) return bail(MATTOHF_ERR_CUDA);
  if ((rc = compute_tables(ctx))) return bail(rc);
  if ((rc = dalloc(ctx, &ctx->d_kern_df, (size_t)(2 * ctx->NK - 1) * NG)) || (rc = dalloc(ctx, &ctx->d_tw_df, NG)))
    return bail(rc);
  if (launch_to_df_tables(ctx->d_kern, (2 * ctx->NK - 1) * NG, ctx->d_kern_df, ctx->tw, NG, ctx->d_tw_df, ctx->st) !=
          cudaSuccess ||
      cudaStreamSynchronize(ctx->st) != cudaSuccess)
    return bail(MATTOHF_ERR_CUDA);
  *out = ctx;
  return MATTOHF_OK;
}

int mattohf_destroy(mattohf_ctx* ctx) {
  if (!ctx) return MATTOHF_OK;
  cudaSetDevice(ctx->device);
  if (ctx->st) cudaStreamSynchronize(ctx->st);
  destroy_graph(ctx);
  {
    void* adj[] = {ctx->d_ckpt, ctx->d_store, ctx->d_lam, ctx->d_lamu, ctx->d_vbuf, ctx->d_Fa, ctx->d_uN,
                   ctx->d_u0, ctx->d_lamk[0], ctx->d_lamk[1], ctx->d_lamk[2], ctx->d_lamk[3], ctx->d_psi,
                   ctx->d_sig, ctx->d_gcol, ctx->d_gstage, ctx->d_gvion, ctx->d_vloc_adj, ctx->d_dpart2,
                   ctx->d_adj_int};
    for (void* p : adj)
      if (p) cudaFree(p);
  }
  for (auto ev : ctx->step_events) cudaEventDestroy(ev);
  if (ctx->d_flush) cudaFree(ctx->d_flush);
  for (auto& ev : ctx->fock_events) {
    cudaEventDestroy(ev.first);
    cudaEventDestroy(ev.second);
  }
  void* ptrs[] = {ctx->tw, ctx->d_Gx, ctx->d_kx, ctx->d_vCG, ctx->d_vcq, ctx->d_kern, ctx->d_vion,
                  ctx->d_vloc, ctx->d_rho, ctx->d_scal, ctx->d_out, ctx->d_u, ctx->d_us, ctx->d_k[0],
                  ctx->d_k[1], ctx->d_k[2], ctx->d_k[3], ctx->d_a, ctx->d_b, ctx->d_c,
                  ctx->d_scratch, ctx->d_colbuf, ctx->d_int, ctx->d_A, ctx->d_Aave, ctx->d_sE,
                  ctx->d_sJ, ctx->d_sN, ctx->d_work, ctx->d_hwork, ctx->d_M, ctx->d_V, ctx->d_evals,
                  ctx->d_eps, ctx->d_err, ctx->d_sym, ctx->d_symF, ctx->d_dpart,
                  ctx->d_udf, ctx->d_kern_df, ctx->d_tw_df, ctx->d_hpre, ctx->d_ticket,
                  ctx->d_small_part, ctx->d_small_obs};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  if (ctx->st_side) cudaStreamDestroy(ctx->st_side);
  if (ctx->st) cudaStreamDestroy(ctx->st);
  delete ctx;
  return MATTOHF_OK;
}

int mattohf_set_option(mattohf_ctx* ctx, int option, long long value) {
  if (!ctx) return MATTOHF_ERR_ARG;
  switch (option) {
    case MATTOHF_OPT_GRAPH: ctx->opt_graph = value ? 1 : 0; break;
    case MATTOHF_OPT_FOCK_CHUNKS:
      if (value < 0) return fail(ctx, MATTOHF_ERR_ARG, "chunks must be >= 0");
      ctx->opt_chunks = (int)value;
      break;
    case MATTOHF_OPT_KERNEL_TIMING: ctx->opt_timing = value ? 1 : 0; break;
    case MATTOHF_OPT_SYMMETRIC: ctx->opt_sym = value ? 1 : 0; break;
    case MATTOHF_OPT_FOCK_DF64: ctx->opt_df = value ? 1 : 0; break;
    case MATTOHF_OPT_SYM_TILE:
      if (value < 0 || value > fock_sym_teams(ctx->NG) || (value & (value - 1)))
        return fail(ctx, MATTOHF_ERR_ARG, "tile size must be 0 or a power of two up to the CTA's teams");
      ctx->opt_tile = (int)value;
      break;
    case MATTOHF_OPT_SMALL_STAGES:
      if (value < 0 || value > 2) return fail(ctx, MATTOHF_ERR_ARG, "small-stage option must be 0, 1 or 2");
      if (value == 1 && !small_stage_supported(ctx->NG))
        return fail(ctx, MATTOHF_ERR_ARG, "fused small stages need NG <= 256");
      ctx->opt_small = (int)value;
      break;
    case MATTOHF_OPT_L2_FLUSH:
      if (value < 0 || value > (4LL << 30)) return fail(ctx, MATTOHF_ERR_ARG, "flush bytes out of range");
      ctx->opt_flush = value;
      break;
    case MATTOHF_OPT_SMALL_CTAS:
      if (value < 0 || value > 4096) return fail(ctx, MATTOHF_ERR_ARG, "CTAs per column must be 0..4096");
      ctx->opt_small_ctas = (int)value;
      break;
    default: return fail(ctx, MATTOHF_ERR_ARG, "unknown option");
  }
  destroy_graph(ctx);
  return MATTOHF_OK;
}

int mattohf_get_grids(mattohf_ctx* ctx, double* rx, double* Gx, double* kx, double* cell) {
  if (!ctx) return MATTOHF_ERR_ARG;
  if (rx) std::memcpy(rx, ctx->rx.data(), sizeof(double) * ctx->NG);
  if (Gx) std::memcpy(Gx, ctx->Gx.data(), sizeof(double) * ctx->NG);
  if (kx) std::memcpy(kx, ctx->kx.data(), sizeof(double) * ctx->NK);
  if (cell) {
    cell[0] = ctx->vcell;
    cell[1] = ctx->dvcell;
    cell[2] = ctx->bx;
  }
  return MATTOHF_OK;
}

int mattohf_get_coulomb(mattohf_ctx* ctx, double* vCG, double* vCq) {
  CKR(check_ctx(ctx));
  if (vCG) CK(cudaMemcpyAsync(vCG, ctx->d_vCG, sizeof(double) * ctx->NG, cudaMemcpyDeviceToHost, ctx->st));
  if (vCq)
    CK(cudaMemcpyAsync(vCq, ctx->d_vcq, sizeof(double) * ctx->NG * (2 * ctx->NK - 1),
                       cudaMemcpyDeviceToHost, ctx->st));
  return sync_and_flag(ctx);
}

int mattohf_vck(mattohf_ctx* ctx, const double* q, int n, double* out) {
  CKR(check_ctx(ctx));
  if (n < 0 || (n > 0 && (!q || !out))) return fail(ctx, MATTOHF_ERR_ARG, "bad vck arguments");
  if (n == 0) return MATTOHF_OK;
  double* d = nullptr;
  const size_t ng = (size_t)vck_points(ctx->acell, ctx->NG, ctx->NK);
  CKR(dalloc(ctx, &d, 2 * (size_t)n + ng));
  int rc = MATTOHF_OK;
  if (cudaMemcpyAsync(d, q, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->st) != cudaSuccess ||
      launch_vck_table(ctx->NG, ctx->NK, ctx->acell, d, n, d + 2 * (size_t)n, d + n, ctx->st) != cudaSuccess ||
      cudaMemcpyAsync(out, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->st) != cudaSuccess ||
      cudaStreamSynchronize(ctx->st) != cudaSuccess)
    rc = fail(ctx, MATTOHF_ERR_CUDA, "k_vCk evaluation failed");
  cudaFree(d);
  return rc;
}

int mattohf_get_vion(mattohf_ctx* ctx, double* vion) {
  if (!ctx || !vion) return MATTOHF_ERR_ARG;
  std::memcpy(vion, ctx->vion.data(), sizeof(double) * ctx->NG);
  return MATTOHF_OK;
}

int mattohf_set_vion(mattohf_ctx* ctx, const double* vion) {
  CKR(check_ctx(ctx));
  if (!vion) return fail(ctx, MATTOHF_ERR_ARG, "null vion");
  ctx->vion.assign(vion, vion + ctx->NG);
  CK(cudaMemcpyAsync(ctx->d_vion, ctx->vion.data(), sizeof(double) * ctx->NG, cudaMemcpyHostToDevice, ctx->st));
  return sync_and_flag(ctx);
}

int mattohf_ion_param_grad(mattohf_ctx* ctx, const double* dLdvion, double* dLdZeff, double* dLdalpha,
                           double* dLdRion) {
  CKR(check_ctx(ctx));
  if (!dLdvion || !dLdZeff || !dLdalpha || !dLdRion) return fail(ctx, MATTOHF_ERR_ARG, "null argument");
  ion_param_grad(ctx, dLdvion, dLdZeff, dLdalpha, dLdRion);
  return MATTOHF_OK;
}

int mattohf_set_orbitals(mattohf_ctx* ctx, const double* ubk) {
  CKR(check_ctx(ctx));
  if (!ubk) return fail(ctx, MATTOHF_ERR_ARG, "null ubk");
  CK(cudaMemcpyAsync(ctx->d_u, ubk, sizeof(double2) * orb_elems(ctx, ctx->NB), cudaMemcpyHostToDevice, ctx->st));
  return sync_and_flag(ctx);
}

int mattohf_get_orbitals(mattohf_ctx* ctx, double* ubk) {
  CKR(check_ctx(ctx));
  if (!ubk) return fail(ctx, MATTOHF_ERR_ARG, "null ubk");
  CK(cudaMemcpyAsync(ubk, ctx->d_u, sizeof(double2) * orb_elems(ctx, ctx->NB), cudaMemcpyDeviceToHost, ctx->st));
  return sync_and_flag(ctx);
}

int mattohf_init_wf(mattohf_ctx* ctx) {
  CKR(check_ctx(ctx));
  // Init_wf (M:159-184) with quickrnd (M:186-196)
  std::vector<double> u(2 * orb_elems(ctx, ctx->NB));
  int iseed = 123;
  for (int ik = 0; ik < ctx->NK; ++ik)
    for (int ib = 0; ib < ctx->NB; ++ib) {
      iseed = (iseed * 106 + 1283) % 6075;
      const double rnd = (double)iseed / 6075.0;
      const double rxc = rnd * ctx->acell;
      for (int g = 0; g < ctx->NG; ++g) {
        const double d = ctx->rx[g] - rxc;
        const size_t o = 2 * (((size_t)ik * ctx->NB + ib) * ctx->NG + g);
        u[o] = std::exp(-0.5 * (d * d));
        u[o + 1] = 0.0;
      }
    }
  return mattohf_set_orbitals(ctx, u.data());
}

int mattohf_gram_schmidt(mattohf_ctx* ctx) {
  CKR(check_ctx(ctx));
  GsArgs a;
  a.u = ctx->d_u;
  a.kstride = ctx->NB * ctx->NG;
  a.nb = ctx->NB;
  a.weight = ctx->vcell / (double)ctx->NG;
  a.flag = ctx->d_int + 2;
  CK(launch_gram_schmidt(ctx->NG, a, ctx->NK, ctx->st));
  return sync_and_flag(ctx);
}

static int hpsi_host(mattohf_ctx* ctx, const double* ubk, const double* wbk, int nbw, double A,
                     double* out, int mode) {
  CKR(check_ctx(ctx));
  if (!wbk || !out || nbw < 1 || (mode != CM_T && !ubk))
    return fail(ctx, MATTOHF_ERR_ARG, "bad hpsi arguments");
  const int NG = ctx->NG, NB = ctx->NB;
  const size_t nw = orb_elems(ctx, nbw), nu = orb_elems(ctx, NB);
  CKR(ensure_stage(ctx, std::max(nw, nu)));
  // h[u] u (the same host array passed twice) keeps u and w in one device
  // buffer, which selects the symmetric exchange kernel.
  const bool same = (ubk == wbk) && nbw == NB;
  if (mode != CM_T)
    CK(cudaMemcpyAsync(ctx->d_a, ubk, sizeof(double2) * nu, cudaMemcpyHostToDevice, ctx->st));
  if (!same)
    CK(cudaMemcpyAsync(ctx->d_b, wbk, sizeof(double2) * nw, cudaMemcpyHostToDevice, ctx->st));
  const double2* wd = same ? ctx->d_a : ctx->d_b;
  CKR(enq_hpsi(ctx, blk(ctx->d_a, NB, NG, NB), blk(wd, nbw, NG, nbw),
               blko(ctx->d_c, nbw, NG, nbw), aval(A), mode));
  CK(cudaMemcpyAsync(out, ctx->d_c, sizeof(double2) * nw, cudaMemcpyDeviceToHost, ctx->st));
  return sync_and_flag(ctx);
}

int mattohf_hpsi(mattohf_ctx* ctx, const double* ubk, const double* wbk, int nbw, double A, double* hwbk) {
  return hpsi_host(ctx, ubk, wbk, nbw, A, hwbk, CM_H);
}

int mattohf_fock(mattohf_ctx* ctx, const double* ubk, const double* wbk, int nbw, double* vF) {
  return hpsi_host(ctx, ubk, wbk, nbw, 0.0, vF, CM_F);
}

int mattohf_kinetic(mattohf_ctx* ctx, const double* wbk, int nbw, double A, double* tbk) {
  return hpsi_host(ctx, nullptr, wbk, nbw, A, tbk, CM_T);
}

int mattohf_hpsi_device(mattohf_ctx* ctx, const double* d_ubk, const double* d_wbk, int nbw, double A,
                        double* d_hwbk) {
  CKR(check_ctx(ctx));
  if (!d_ubk || !d_wbk || !d_hwbk || nbw < 1) return fail(ctx, MATTOHF_ERR_ARG, "bad hpsi arguments");
  const int NG = ctx->NG, NB = ctx->NB;
  return enq_hpsi(ctx, blk((const double2*)d_ubk, NB, NG, NB), blk((const double2*)d_wbk, nbw, NG, nbw),
                  blko((double2*)d_hwbk, nbw, NG, nbw), aval(A), CM_H);
}

// Rows of the output k-points k0 .. k0+nkl-1 only.  The pair kernel and the
// combine index the kernel table by d = kr - kc + NK - 1 and kx by kr, so a
// slice is the same launch with kern and kx advanced by k0 rows.
static int kslice_args(mattohf_ctx* ctx, const double* d_uocc, int k0, int nkl, const double* d_w, int nbw) {
  CKR(check_ctx(ctx));
  if (!d_uocc || !d_w || nbw < 1 || nkl < 1 || k0 < 0 || k0 + nkl > ctx->NK)
    return fail(ctx, MATTOHF_ERR_ARG, "bad k-slice arguments");
  return MATTOHF_OK;
}

static int enq_kslice(mattohf_ctx* ctx, const double* d_uocc, int k0, int nkl, const double* d_w, int nbw,
                      AField af, int mode, BlockOut out) {
  const int NG = ctx->NG;
  Block u = blk((const double2*)d_uocc, ctx->NBocc, NG, ctx->NBocc);
  Block w = blk((const double2*)d_w, nbw, NG, nbw);
  const int ncols = nkl * nbw;
  if (mode == CM_H || mode == CM_OBS) CKR(enq_density(ctx, u));
  CKR(ensure_scratch(ctx, ncols));
  FockPlan fp;
  if (ctx->hf && mode != CM_T) {
    FockArgs a;
    a.u = u;
    a.w = w;
    a.nk = ctx->NK;
    a.nbocc = ctx->NBocc;
    a.kern = ctx->d_kern + (size_t)k0 * NG;
    a.tw = ctx->tw;
    a.scratch = ctx->d_scratch;
    fock_split(ctx, ncols, &a.nchunks, &a.chunk);
    fp.nchunks = a.nchunks;
    fp.any = true;
    CK(launch_fock(NG, a, ncols, ctx->st));
  } else if (mode == CM_F) {
    CK(cudaMemsetAsync(out.p, 0, sizeof(double2) * (size_t)nkl * out.kstride, ctx->st));
    return MATTOHF_OK;
  }
  CombineArgs c = combine_base(ctx, w, af, mode, fp);
  c.kx = ctx->d_kx + k0;
  c.nk = nkl;
  c.out = out;
  CK(launch_combine(NG, c, ncols, ctx->st));
  return MATTOHF_OK;
}

int mattohf_hpsi_kslice_device(mattohf_ctx* ctx, const double* d_uocc, int k0, int nkl, const double* d_wbk,
                               int nbw, double A, int term, double* d_hwbk) {
  CKR(kslice_args(ctx, d_uocc, k0, nkl, d_wbk, nbw));
  if (!d_hwbk || term < 0 || term > 2) return fail(ctx, MATTOHF_ERR_ARG, "bad k-slice output or term");
  const int mode = term == 0 ? CM_H : (term == 1 ? CM_F : CM_T);
  return enq_kslice(ctx, d_uocc, k0, nkl, d_wbk, nbw, aval(A), mode,
                    blko((double2*)d_hwbk, nbw, ctx->NG, nbw));
}

int mattohf_observables_kslice_device(mattohf_ctx* ctx, const double* d_uocc, int k0, int nkl,
                                      const double* d_ubk, double A, double* partial, double* scal) {
  CKR(kslice_args(ctx, d_uocc, k0, nkl, d_ubk, ctx->NB));
  if (!partial || !scal) return fail(ctx, MATTOHF_ERR_ARG, "null observable outputs");
  const int NB = ctx->NB;
  CKR(enq_kslice(ctx, d_uocc, k0, nkl, d_ubk, NB, aval(A), CM_OBS, BlockOut()));
  std::vector<double> cb((size_t)nkl * NB * 4);
  double s[3];
  CK(cudaMemcpyAsync(cb.data(), ctx->d_colbuf, sizeof(double) * cb.size(), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(s, ctx->d_scal, sizeof(double) * 3, cudaMemcpyDeviceToHost, ctx->st));
  CKR(sync_and_flag(ctx));
  // the single-context reduction's column order (k, then band)
  double ekin = 0.0, jre = 0.0, exr = 0.0;
  for (int c = 0; c < nkl * NB; ++c) {
    const int ib = c % NB;
    const double occ = ib < ctx->NBocc ? ctx->occ : 0.0;
    ekin += occ * cb[(size_t)c * 4] * ctx->dvcell;
    jre += occ * cb[(size_t)c * 4 + 1];
    if (ib < ctx->NBocc) exr += occ * cb[(size_t)c * 4 + 2] * ctx->dvcell;
  }
  partial[0] = ekin;
  partial[1] = -(jre * ctx->dvcell / ctx->vcell);
  partial[2] = ctx->hf ? 0.5 * exr : 0.0;
  scal[0] = s[0];
  scal[1] = s[1];
  scal[2] = s[2];
  return MATTOHF_OK;
}

int mattohf_density(mattohf_ctx* ctx, const double* ubk, double* dns, double* vH) {
  CKR(check_ctx(ctx));
  if (!ubk) return fail(ctx, MATTOHF_ERR_ARG, "null ubk");
  const size_t nu = orb_elems(ctx, ctx->NB);
  CKR(ensure_stage(ctx, nu));
  CK(cudaMemcpyAsync(ctx->d_a, ubk, sizeof(double2) * nu, cudaMemcpyHostToDevice, ctx->st));
  CKR(enq_density(ctx, blk(ctx->d_a, ctx->NB, ctx->NG, ctx->NB)));
  std::vector<double> vloc(ctx->NG);
  if (dns) CK(cudaMemcpyAsync(dns, ctx->d_rho, sizeof(double) * ctx->NG, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(vloc.data(), ctx->d_vloc, sizeof(double) * ctx->NG, cudaMemcpyDeviceToHost, ctx->st));
  CKR(sync_and_flag(ctx));
  // vloc = vH + vion on the device; the Hartree part alone is recovered exactly
  // only up to rounding, so vH is recomputed from a zero-vion pass instead.
  if (vH) {
    CK(cudaMemsetAsync(ctx->d_vion, 0, sizeof(double) * ctx->NG, ctx->st));
    CKR(enq_density(ctx, blk(ctx->d_a, ctx->NB, ctx->NG, ctx->NB)));
    CK(cudaMemcpyAsync(vH, ctx->d_vloc, sizeof(double) * ctx->NG, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(ctx->d_vion, ctx->vion.data(), sizeof(double) * ctx->NG, cudaMemcpyHostToDevice, ctx->st));
    CKR(sync_and_flag(ctx));
  }
  return MATTOHF_OK;
}

int mattohf_observables(mattohf_ctx* ctx, double A, double* Ecomps, double* Etot, double* Je, double* Nele) {
  CKR(check_ctx(ctx));
  CKR(enq_observables(ctx, ctx->d_u, aval(A), false, false));
  double o[8];
  CK(cudaMemcpyAsync(o, ctx->d_out, sizeof(double) * 7, cudaMemcpyDeviceToHost, ctx->st));
  CKR(sync_and_flag(ctx));
  if (Ecomps) {
    Ecomps[0] = o[1];
    Ecomps[1] = o[2];
    Ecomps[2] = o[3];
    Ecomps[3] = o[4];
  }
  if (Etot) *Etot = o[0];
  if (Je) *Je = o[5];
  if (Nele) *Nele = o[6];
  return MATTOHF_OK;
}

int mattohf_rk4_step(mattohf_ctx* ctx, double Aave, double A, double dt) {
  CKR(check_ctx(ctx));
  CK(cudaMemsetAsync(ctx->d_int + 1, 0, sizeof(int), ctx->st));
  CKR(enq_rk4(ctx, aval(2.0 * Aave - A), aval(Aave), aval(A), dt));
  int flag = 0;
  CK(cudaMemcpyAsync(&flag, ctx->d_int + 1, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  CKR(sync_and_flag(ctx));
  if (flag) return fail(ctx, MATTOHF_ERR_NONFINITE, "non-finite orbitals after RK4 step");
  return MATTOHF_OK;
}

int mattohf_rk4_run(mattohf_ctx* ctx, int nt, double dt, const double* A, const double* Aave,
                    double* Etot, double* Je, double* Nele) {
  CKR(check_ctx(ctx));
  if (nt < 0 || (nt > 0 && (!A || !Aave))) return fail(ctx, MATTOHF_ERR_ARG, "bad rk4_run arguments");
  if (nt == 0) return MATTOHF_OK;
  CKR(ensure_series(ctx, nt));
  CKR(ensure_fock_buffers(ctx));
  CK(cudaMemcpyAsync(ctx->d_A, A, sizeof(double) * nt, cudaMemcpyHostToDevice, ctx->st));
  CK(cudaMemcpyAsync(ctx->d_Aave, Aave, sizeof(double) * nt, cudaMemcpyHostToDevice, ctx->st));
  CK(cudaMemsetAsync(ctx->d_int, 0, 2 * sizeof(int), ctx->st));
  AField fm, fave, fcur;
  fm.A = fave.A = fcur.A = ctx->d_A;
  fm.Aave = fave.Aave = fcur.Aave = ctx->d_Aave;
  fm.it = fave.it = fcur.it = ctx->d_int;
  fm.val = fave.val = fcur.val = 0.0;
  fm.mode = AM;
  fave.mode = AAVE;
  fcur.mode = ACUR;
  const bool use_graph = ctx->opt_graph && !ctx->opt_timing;
  const bool small = use_small(ctx);
  if (small) CKR(ensure_small_buffers(ctx));
  CK(cudaMemsetAsync(ctx->d_ticket, 0, sizeof(unsigned) * (1 + (size_t)ctx->NK * ctx->NB), ctx->st));
  if (use_graph && (!ctx->step_exec || ctx->step_dt != dt || ctx->step_small != small)) {
    destroy_graph(ctx);
    // one step, and kGraphSteps steps in one graph: the launch of a graph is a
    // full dependency, while within it consecutive stages overlap
    // (programmatic dependent launches)
    for (int steps : {1, kGraphSteps}) {
      cudaGraph_t g;
      ctx->capturing = true;
      CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
      int rc = MATTOHF_OK;
      for (int s = 0; s < steps && rc == MATTOHF_OK; ++s) {
        if (small) {
          rc = enq_small_step(ctx, fm, fave, fcur, dt);
        } else {
          rc = enq_rk4(ctx, fm, fave, fcur, dt, ctx->d_sE);
          if (rc == MATTOHF_OK) rc = enq_observables(ctx, ctx->d_u, fcur, true, true);
        }
      }
      cudaError_t ec = cudaStreamEndCapture(ctx->st, &g);
      ctx->capturing = false;
      if (rc != MATTOHF_OK) return rc;
      CK(ec);
      cudaError_t ei = cudaGraphInstantiate(steps == 1 ? &ctx->step_exec : &ctx->multi_exec, g, 0);
      cudaGraphDestroy(g);
      CK(ei);
    }
    ctx->step_dt = dt;
    ctx->step_small = small;
  }
  ctx->fock_event_used = 0;
  // Optional per-step timing with an L2 flush between steps: each step (and
  // the closing exchange apply) is bracketed by its own events and the flush
  // runs outside them.
  const bool stepwise = ctx->opt_flush > 0;
  if (stepwise) {
    if ((size_t)ctx->opt_flush > ctx->flush_cap) {
      if (ctx->d_flush) cudaFree(ctx->d_flush);
      ctx->d_flush = nullptr;
      CK(cudaMalloc(&ctx->d_flush, (size_t)ctx->opt_flush));
      ctx->flush_cap = (size_t)ctx->opt_flush;
    }
    while (ctx->step_events.size() < 2 * (size_t)(nt + 1)) {
      cudaEvent_t ev;
      CK(cudaEventCreate(&ev));
      ctx->step_events.push_back(ev);
    }
  }
  ScopedEvent e0, e1;
  CK(e0.create());
  CK(e1.create());
  CK(cudaEventRecord(e0, ctx->st));
  int flag = 0;
  int bad_at = -1;
  for (int it = 0; it < nt; ++it) {
    if (stepwise) {
      CK(cudaMemsetAsync(ctx->d_flush, it & 0xff, (size_t)ctx->opt_flush, ctx->st));
      CK(cudaEventRecord(ctx->step_events[2 * it], ctx->st));
    }
    if (use_graph && !stepwise && it % kGraphSteps == 0 && nt - it >= kGraphSteps) {
      CK(cudaGraphLaunch(ctx->multi_exec, ctx->st));  // steps it .. it + kGraphSteps - 1
      it += kGraphSteps - 1;
    } else if (use_graph) {
      CK(cudaGraphLaunch(ctx->step_exec, ctx->st));
    } else if (small) {
      CKR(enq_small_step(ctx, fm, fave, fcur, dt));
    } else {
      CKR(enq_rk4(ctx, fm, fave, fcur, dt, ctx->d_sE));
      CKR(enq_observables(ctx, ctx->d_u, fcur, true, true));
    }
    if (stepwise) CK(cudaEventRecord(ctx->step_events[2 * it + 1], ctx->st));
    // bounded detection of a blow-up: poll the flag every 256 steps
    // (kGraphSteps divides 256, so a multi-step launch ends on each check)
    if ((it & 255) == 255 && it + 1 < nt) {
      CK(cudaMemcpyAsync(&flag, ctx->d_int + 1, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
      CK(cudaStreamSynchronize(ctx->st));
      if (flag) {
        bad_at = it;
        break;
      }
    }
  }
  {
    // exchange energy of the last step's orbitals (the next stage-1 apply that
    // would supply it does not happen)
    const int last = bad_at >= 0 ? bad_at : nt - 1;
    if (stepwise) {
      CK(cudaMemsetAsync(ctx->d_flush, 0x5a, (size_t)ctx->opt_flush, ctx->st));
      CK(cudaEventRecord(ctx->step_events[2 * nt], ctx->st));
    }
    if (small) {
      CKR(enq_small_close(ctx));
    } else if (ctx->hf) {
      FockPlan fp;
      CKR(enq_observables(ctx, ctx->d_u, aval(0.0), false, false, &fp));
      (void)fp;
      CK(launch_ex_finalize(ex_args(ctx, ctx->d_sE, last, nullptr), ctx->st));
    }
  }
  CK(cudaEventRecord(e1, ctx->st));
  CK(cudaEventSynchronize(e1));
  cudaEvent_t e1_copy = e1;
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, e0, e1));
  if (stepwise) {
    const int ndone_steps = bad_at >= 0 ? bad_at + 1 : nt;
    double sum = 0.0;
    for (int it = 0; it < ndone_steps; ++it) {
      float f = 0;
      CK(cudaEventElapsedTime(&f, ctx->step_events[2 * it], ctx->step_events[2 * it + 1]));
      sum += f;
    }
    float f = 0;
    CK(cudaEventElapsedTime(&f, ctx->step_events[2 * nt], e1_copy));
    sum += f;
    ms = (float)sum;
  }
  ctx->last_run_ms = ms;
  ctx->last_fock_ms = 0;
  ctx->last_fock_launches = (int)ctx->fock_event_used;
  for (size_t i = 0; i < ctx->fock_event_used; ++i) {
    float f = 0;
    CK(cudaEventElapsedTime(&f, ctx->fock_events[i].first, ctx->fock_events[i].second));
    ctx->last_fock_ms += f;
  }
  const int ndone = bad_at >= 0 ? bad_at + 1 : nt;
  std::vector<double> sE(ndone), sJ(ndone), sN(ndone);
  CK(cudaMemcpyAsync(sE.data(), ctx->d_sE, sizeof(double) * ndone, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(sJ.data(), ctx->d_sJ, sizeof(double) * ndone, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(sN.data(), ctx->d_sN, sizeof(double) * ndone, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(&flag, ctx->d_int + 1, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  CKR(sync_and_flag(ctx));
  if (Etot) std::copy(sE.begin(), sE.end(), Etot);
  if (Je) std::copy(sJ.begin(), sJ.end(), Je);
  if (Nele) std::copy(sN.begin(), sN.end(), Nele);
  if (flag) {
    int first = ndone - 1;
    for (int i = 0; i < ndone; ++i)
      if (!(std::isfinite(sE[i]) && std::isfinite(sJ[i]) && std::isfinite(sN[i]))) {
        first = i;
        break;
      }
    char buf[160];
    std::snprintf(buf, sizeof(buf), "non-finite state at RK4 step %d (1-based it=%d); %d steps run",
                  first, first + 1, ndone);
    return fail(ctx, MATTOHF_ERR_NONFINITE, buf);
  }
  return MATTOHF_OK;
}

// Autotuner: times the context's tunable launch shapes on its own orbitals
// and keeps the fastest.  The orbitals (and the step counter) are restored.
//   * symmetric-exchange tile S: one exchange apply h[u]u (k_fock_sym +
//     k_sym_reduce, or the double-float kernels) for S = 1, 2, 4, ... up to the
//     teams of a CTA;
//   * fused-stage CTAs per column P, for the grids the fused stages support:
//     graph-replayed mattohf_rk4_run steps for every P from one round of all
//     pair teams up to twice the multiprocessors over the columns (at most 8);
//   * fused stages vs the tiled step: the faster of the best of each.
// out: [0] S, [1] P (0 when the fused stages do not apply), [2] 1 when the
// fused stages won; us: [0] exchange apply at S, [1] step of the tiled path,
// [2] step of the fused path (0 when not timed), in microseconds.
extern "C" int mattohf_autotune(mattohf_ctx* ctx, int steps, int* out, double* us) {
  CKR(check_ctx(ctx));
  if (steps < 1 || steps > 100000) return fail(ctx, MATTOHF_ERR_ARG, "autotune steps must be 1..100000");
  if (ctx->capturing) return fail(ctx, MATTOHF_ERR_STATE, "autotune during capture");
  const int NG = ctx->NG, NB = ctx->NB, NK = ctx->NK;
  const size_t elems = orb_elems(ctx, NB);
  struct DevBuf {
    double2* p = nullptr;
    ~DevBuf() {
      if (p) cudaFree(p);
    }
  } saved;
  CK(cudaMalloc((void**)&saved.p, sizeof(double2) * elems));
  CK(cudaMemcpyAsync(saved.p, ctx->d_u, sizeof(double2) * elems, cudaMemcpyDeviceToDevice, ctx->st));
  ScopedEvent e0, e1;
  CK(e0.create());
  CK(e1.create());
  auto restore = [&]() -> int {
    CK(cudaMemcpyAsync(ctx->d_u, saved.p, sizeof(double2) * elems, cudaMemcpyDeviceToDevice, ctx->st));
    CK(cudaMemsetAsync(ctx->d_int, 0, 2 * sizeof(int), ctx->st));
    return MATTOHF_OK;
  };
  // ---- exchange tile
  int bestS = sym_tile(ctx);
  double tS = 0.0;
  if (ctx->hf && ctx->opt_sym && ctx->NBocc > 0) {
    const int reps = std::max(2, std::min(steps, 20));
    double best = 1e300;
    const int M = NK * ctx->NBocc, Smax = fock_sym_teams(NG);
    for (int S = 1; S <= Smax; S <<= 1) {
      // tiles far beyond a few waves only add partial-sum traffic (and scratch)
      const long long T = (M + S - 1) / S;
      if (S < Smax && T * (T + 1) / 2 > 32LL * ctx->nsm) continue;
      ctx->opt_tile = S;
      CKR(ensure_fock_buffers(ctx));
      const Block ub = blk(ctx->d_u, NB, NG, NB);
      FockPlan fp;
      CKR(enq_fock(ctx, ub, ub, &fp));  // warm-up
      CK(cudaEventRecord(e0, ctx->st));
      for (int r = 0; r < reps; ++r) CKR(enq_fock(ctx, ub, ub, &fp));
      CK(cudaEventRecord(e1, ctx->st));
      CK(cudaEventSynchronize(e1));
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      const double t = 1e3 * ms / reps;
      if (t < best) {
        best = t;
        bestS = S;
      }
    }
    ctx->opt_tile = bestS;
    tS = best;
  }
  // ---- stepping: tiled, then the fused stages for each P
  std::vector<double> A(steps, 0.0), h1(steps), h2(steps), h3(steps);
  auto time_steps = [&](double* t_us) -> int {
    destroy_graph(ctx);
    CKR(restore());
    int rc = mattohf_rk4_run(ctx, steps, 1e-4, A.data(), A.data(), h1.data(), h2.data(), h3.data());
    if (rc != MATTOHF_OK) return rc;  // first call captures the graph
    CKR(restore());
    rc = mattohf_rk4_run(ctx, steps, 1e-4, A.data(), A.data(), h1.data(), h2.data(), h3.data());
    if (rc != MATTOHF_OK) return rc;
    *t_us = 1e3 * ctx->last_run_ms / steps;
    return MATTOHF_OK;
  };
  const int opt_small0 = ctx->opt_small, opt_ctas0 = ctx->opt_small_ctas;
  double t_tiled = 0.0, t_fused = 0.0;
  int bestP = 0;
  ctx->opt_small = 0;
  int rc = time_steps(&t_tiled);
  const bool fused_ok = small_stage_supported(NG) && !ctx->opt_df && !ctx->opt_timing && ctx->NBocc > 0;
  if (rc == MATTOHF_OK && fused_ok) {
    const int ncols = NK * NB, M = NK * ctx->NBocc;
    const int lo = std::min(kSmallMaxCtas, std::max(1, (M + small_pair_teams(NG) - 1) / small_pair_teams(NG)));
    const int hi = std::min(kSmallMaxCtas, std::max(lo, std::min(M, std::max(1, 2 * ctx->nsm / ncols))));
    ctx->opt_small = 1;
    ctx->opt_small_ctas = 0;
    std::vector<int> cand{small_ctas_per_column(ctx)};
    for (int P = lo; P <= hi; ++P)
      if (P != cand[0]) cand.push_back(P);
    double best = 1e300;
    for (int P : cand) {
      ctx->opt_small_ctas = P;
      double t = 0.0;
      if ((rc = time_steps(&t)) != MATTOHF_OK) break;
      if (t < best) {
        best = t;
        bestP = P;
      }
    }
    t_fused = best;
  }
  // restore the state whatever happened, then keep the winners
  const int rr = restore();
  destroy_graph(ctx);
  if (rc != MATTOHF_OK) {
    ctx->opt_small = opt_small0;
    ctx->opt_small_ctas = opt_ctas0;
    return rc;
  }
  if (rr != MATTOHF_OK) return rr;
  const bool fused_wins = bestP > 0 && t_fused < t_tiled;
  ctx->opt_small = fused_wins ? 1 : 0;
  ctx->opt_small_ctas = bestP;
  CK(cudaStreamSynchronize(ctx->st));
  if (out) {
    out[0] = bestS;
    out[1] = bestP;
    out[2] = fused_wins ? 1 : 0;
  }
  if (us) {
    us[0] = tS;
    us[1] = t_tiled;
    us[2] = bestP > 0 ? t_fused : 0.0;
  }
  return MATTOHF_OK;
}

int mattohf_last_run_timing(mattohf_ctx* ctx, double* run_ms, double* fock_ms, int* fock_launches) {
  if (!ctx) return MATTOHF_ERR_ARG;
  if (run_ms) *run_ms = ctx->last_run_ms;
  if (fock_ms) *fock_ms = ctx->last_fock_ms;
  if (fock_launches) *fock_launches = ctx->last_fock_launches;
  return MATTOHF_OK;
}

static int ensure_gs(mattohf_ctx* ctx, int m) {
  const size_t need = orb_elems(ctx, m);
  if (need <= ctx->gs_cap) return MATTOHF_OK;
  CKR(dalloc(ctx, &ctx->d_work, need));
  CKR(dalloc(ctx, &ctx->d_hwork, need));
  CKR(dalloc(ctx, &ctx->d_M, (size_t)ctx->NK * m * m));
  CKR(dalloc(ctx, &ctx->d_V, (size_t)ctx->NK * m * m));
  CKR(dalloc(ctx, &ctx->d_evals, (size_t)ctx->NK * m));
  CKR(dalloc(ctx, &ctx->d_eps, (size_t)ctx->NK * ctx->NB));
  CKR(dalloc(ctx, &ctx->d_err, (size_t)ctx->NK * ctx->NB));
  ctx->gs_cap = need;
  return MATTOHF_OK;
}

// Rayleigh-Ritz of the m columns in x (their h-images in hx) keeping the
// lowest nout Ritz vectors into out.
static int enq_rayleigh_ritz(mattohf_ctx* ctx, const double2* x, const double2* hx, int m, int nout,
                             double2* out) {
  const int NG = ctx->NG;
  CK(launch_project(NG, x, hx, m * NG, m, ctx->dvcell, ctx->d_M, ctx->NK, ctx->st));
  CK(launch_jacobi(ctx->d_M, m, ctx->d_evals, ctx->d_V, ctx->NK, ctx->d_int + 2, ctx->st));
  CK(launch_rotate(NG, x, m * NG, m, ctx->d_V, nout, out, ctx->NB * NG, ctx->NK, ctx->st));
  return MATTOHF_OK;
}

int mattohf_eps(mattohf_ctx* ctx, double* epsbk, double* epserrorbk) {
  CKR(check_ctx(ctx));
  const int NG = ctx->NG, NB = ctx->NB;
  CKR(ensure_gs(ctx, NB));
  Block ub = blk(ctx->d_u, NB, NG, NB);
  CKR(enq_hpsi(ctx, ub, ub, blko(ctx->d_hwork, NB, NG, NB), aval(0.0), CM_H));
  CK(launch_eps(NG, ctx->d_u, ctx->d_hwork, NB * NG, NB, ctx->dvcell, ctx->d_eps, ctx->d_err, ctx->NK, ctx->st));
  if (epsbk) CK(cudaMemcpyAsync(epsbk, ctx->d_eps, sizeof(double) * ctx->NK * NB, cudaMemcpyDeviceToHost, ctx->st));
  if (epserrorbk)
    CK(cudaMemcpyAsync(epserrorbk, ctx->d_err, sizeof(double) * ctx->NK * NB, cudaMemcpyDeviceToHost, ctx->st));
  return sync_and_flag(ctx);
}

int mattohf_gs_run(mattohf_ctx* ctx, int nscf, int ncg, double* Etot_iter, double* Je_iter,
                   double* dnsdiff, double* epsbk, double* epserrorbk) {
  CKR(check_ctx(ctx));
  const int NG = ctx->NG, NB = ctx->NB, NK = ctx->NK;
  if (nscf < 0 || ncg < 1) return fail(ctx, MATTOHF_ERR_ARG, "nscf >= 0 and ncg >= 1 required");
  const int m = NB * ncg;
  if (m > 64 || m > NG) return fail(ctx, MATTOHF_ERR_ARG, "NB*NCG must be <= 64 and <= NG");
  CKR(ensure_gs(ctx, m));
  CK(cudaMemsetAsync(ctx->d_int + 2, 0, sizeof(int), ctx->st));
  const double dnsmix = 0.5;
  std::vector<double> dprev(NG), dnew(NG);
  double o[8];
  // Etotscf(0) and dnsscf(:,1) (GS:26-27)
  CKR(enq_observables(ctx, ctx->d_u, aval(0.0), false, false));
  CK(cudaMemcpyAsync(o, ctx->d_out, sizeof(double) * 7, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(dprev.data(), ctx->d_rho, sizeof(double) * NG, cudaMemcpyDeviceToHost, ctx->st));
  CKR(sync_and_flag(ctx));
  if (Etot_iter) Etot_iter[0] = o[0];
  GsArgs gsa;
  gsa.u = ctx->d_u;
  gsa.kstride = NB * NG;
  gsa.nb = NB;
  gsa.weight = ctx->vcell / (double)NG;
  gsa.flag = ctx->d_int + 2;
  Block ub = blk(ctx->d_u, NB, NG, NB);
  for (int iter = 0; iter < nscf; ++iter) {
    CK(launch_gram_schmidt(NG, gsa, NK, ctx->st));
    // KS_ubk2_SVD (GS:124-194): Krylov block [u, h u, h^2 u, ...]
    CK(cudaMemcpy2DAsync(ctx->d_work, sizeof(double2) * m * NG, ctx->d_u, sizeof(double2) * NB * NG,
                         sizeof(double2) * NB * NG, NK, cudaMemcpyDeviceToDevice, ctx->st));
    for (int icg = 1; icg < ncg; ++icg) {
      Block wb = blk(ctx->d_work + (size_t)(icg - 1) * NB * NG, m, NG, NB);
      BlockOut ob = blko(ctx->d_work + (size_t)icg * NB * NG, m, NG, NB);
      CKR(enq_hpsi(ctx, ub, wb, ob, aval(0.0), CM_H));
    }
    CK(launch_block_orth(NG, ctx->d_work, m * NG, m, ctx->dvcell, NK, ctx->d_int + 2, ctx->st));
    CKR(enq_hpsi(ctx, ub, blk(ctx->d_work, m, NG, m), blko(ctx->d_hwork, m, NG, m), aval(0.0), CM_H));
    CKR(enq_rayleigh_ritz(ctx, ctx->d_work, ctx->d_hwork, m, NB, ctx->d_u));
    CK(launch_gram_schmidt(NG, gsa, NK, ctx->st));
    // Subspace_diag (GS:197-237)
    CKR(enq_hpsi(ctx, ub, ub, blko(ctx->d_hwork, NB, NG, NB), aval(0.0), CM_H));
    CK(cudaMemcpyAsync(ctx->d_work, ctx->d_u, sizeof(double2) * orb_elems(ctx, NB), cudaMemcpyDeviceToDevice, ctx->st));
    CKR(enq_rayleigh_ritz(ctx, ctx->d_work, ctx->d_hwork, NB, NB, ctx->d_u));
    // Etot, Je (GS:36-38); the Fock partials of h[u]u are then reused for the
    // Ritz values and residuals (GS:42-43), which apply the same operator.
    FockPlan fp;
    CKR(enq_observables(ctx, ctx->d_u, aval(0.0), false, false, &fp));
    {
      CombineArgs a = combine_base(ctx, ub, aval(0.0), CM_H, fp);
      a.out = blko(ctx->d_hwork, NB, NG, NB);
      CK(launch_combine(NG, a, NK * NB, ctx->st));
    }
    CK(launch_eps(NG, ctx->d_u, ctx->d_hwork, NB * NG, NB, ctx->dvcell, ctx->d_eps, ctx->d_err, NK, ctx->st));
    CK(cudaMemcpyAsync(o, ctx->d_out, sizeof(double) * 7, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(dnew.data(), ctx->d_rho, sizeof(double) * NG, cudaMemcpyDeviceToHost, ctx->st));
    CKR(sync_and_flag(ctx));
    if (Etot_iter) Etot_iter[iter + 1] = o[0];
    if (Je_iter) Je_iter[iter] = o[5];
    double dd = 0.0;
    for (int g = 0; g < NG; ++g) {
      const double mixed = dnsmix * dnew[g] + (1.0 - dnsmix) * dprev[g];  // GS:44
      dd += std::fabs(mixed - dprev[g]);
      dprev[g] = mixed;
    }
    if (dnsdiff) dnsdiff[iter] = dd / (double)NG;
  }
  if (epsbk) CK(cudaMemcpyAsync(epsbk, ctx->d_eps, sizeof(double) * NK * NB, cudaMemcpyDeviceToHost, ctx->st));
  if (epserrorbk) CK(cudaMemcpyAsync(epserrorbk, ctx->d_err, sizeof(double) * NK * NB, cudaMemcpyDeviceToHost, ctx->st));
  int flag = 0;
  CK(cudaMemcpyAsync(&flag, ctx->d_int + 2, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  CKR(sync_and_flag(ctx));
  if (flag) return fail(ctx, MATTOHF_ERR_NOTCONV, flag == 2 ? "Jacobi eigensolver did not converge"
                                                             : "orthonormalisation met a zero column");
  return MATTOHF_OK;
}

int mattohf_diag_fp64_peak(int device, double* tflops) {
  if (!tflops) return MATTOHF_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MATTOHF_ERR_CUDA;
  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return MATTOHF_ERR_CUDA;
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double)) != cudaSuccess) return MATTOHF_ERR_ALLOC;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = nsm * 8, threads = 256, iters = 200;
  k_dfma_probe<<<blocks, threads>>>(d, iters, 1.0000001, 1e-9);
  cudaEventRecord(e0);
  k_dfma_probe<<<blocks, threads>>>(d, iters, 1.0000001, 1e-9);
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  if (e != cudaSuccess || ms <= 0) return MATTOHF_ERR_CUDA;
  const double fmas = (double)blocks * threads * iters * 16 * 8;
  *tflops = 2.0 * fmas / (ms * 1e-3) / 1e12;
  return MATTOHF_OK;
}

int mattohf_diag_dmma_peak(int device, double* tflops) {
  if (!tflops) return MATTOHF_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MATTOHF_ERR_CUDA;
  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return MATTOHF_ERR_CUDA;
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double)) != cudaSuccess) return MATTOHF_ERR_ALLOC;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = nsm * 8, threads = 256, iters = 400;
  k_dmma_probe<<<blocks, threads>>>(d, iters);
  cudaEventRecord(e0);
  k_dmma_probe<<<blocks, threads>>>(d, iters);
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  if (e != cudaSuccess || ms <= 0) return MATTOHF_ERR_CUDA;
  const double warp_mmas = (double)blocks * (threads / 32) * iters * 8;
  *tflops = warp_mmas * 512.0 / (ms * 1e-3) / 1e12;
  return MATTOHF_OK;
}

int mattohf_synchronize(mattohf_ctx* ctx) {
  CKR(check_ctx(ctx));
  return sync_and_flag(ctx);
}

}  // extern "C"


// ===========================================================================
// Adjoint of the RK4 real-time loop (no counterpart in the reference).
// ===========================================================================
namespace {

// Recompute one forward step from d_u, storing its four stage inputs in the
// segment store at slot (it - seg0)*4 + s.
int enq_recompute_step(mattohf_ctx* ctx, AField fm, AField fave, AField fcur, double dt) {
  if (use_small(ctx)) return enq_small_step(ctx, fm, fave, fcur, dt, true);  // advances the counter itself
  CKR(enq_rk4(ctx, fm, fave, fcur, dt, nullptr, true));
  CK(launch_counter_add(ctx->d_int, 1, ctx->st));
  return MATTOHF_OK;
}

// One backward RK4 step at n = d_adj_int[0] (RT:165-170 reversed).
int enq_adjoint_step(mattohf_ctx* ctx, double dt, size_t elems) {
  const int NG = ctx->NG, NB = ctx->NB, NK = ctx->NK;
  int* n = ctx->d_adj_int;
  int* seg0 = ctx->d_adj_int + 1;
  CK(launch_adj_init(ctx->d_lam, ctx->d_lamu, ctx->d_lamk, dt, elems, ctx->st));
  const double cst[3] = {0.5 * dt, 0.5 * dt, dt};
  const int amodes[4] = {AM, AAVE, AAVE, ACUR};
  if (use_small(ctx)) {
    // one fused launch per reverse stage; stage 0 also copies lam = lam_u and
    // steps the counter back
    SmallAdjArgs a;
    std::memset(&a, 0, sizeof(a));
    a.store = ctx->d_store;
    a.n = n;
    a.seg0 = seg0;
    a.lam_u = ctx->d_lamu;
    a.lam = ctx->d_lam;
    a.af.A = ctx->d_A;
    a.af.Aave = ctx->d_Aave;
    a.af.it = n;
    a.nk = NK;
    a.nb = NB;
    a.P = ctx->small_P_adj;
    a.occ = ctx->occ;
    a.kern = ctx->d_kern;
    a.vCG = ctx->d_vCG;
    a.vion = ctx->d_vion;
    a.Gx = ctx->d_Gx;
    a.kx = ctx->d_kx;
    a.tw = ctx->tw;
    a.part = ctx->d_small_part;
    a.gcol = ctx->d_gcol;
    a.gstage = ctx->d_gstage;
    a.gvion = ctx->d_gvion;
    a.ticket = ctx->d_ticket;
    for (int s = 3; s >= 0; --s) {
      a.slot = s;
      a.mu = ctx->d_lamk[s];
      a.lam_prev = s > 0 ? ctx->d_lamk[s - 1] : nullptr;
      a.cprev = s > 0 ? cst[s - 1] : 0.0;
      a.af.mode = amodes[s];
      CK(launch_small_adj(NG, a, ctx->st));
    }
    return MATTOHF_OK;
  }
  const int M = NK * ctx->NBocc;
  const int S = sym_tile(ctx);
  const int T = (M + S - 1) / S;
  const bool side = ctx->hf != 0;
  cudaStream_t ss = side ? ctx->st_side : ctx->st;
  for (int s = 3; s >= 0; --s) {
    CK(launch_stage_copy(ctx->d_vbuf, nullptr, ctx->d_store, n, seg0, s, elems, 0, ctx->st));
    Block vb = blk(ctx->d_vbuf, NB, NG, NB);
    // the densities and the exchange-free part of the combine run on the side
    // stream, beside the adjoint exchange
    if (side) {
      CK(cudaEventRecord(ctx->ev_fork, ctx->st));
      CK(cudaStreamWaitEvent(ctx->st_side, ctx->ev_fork, 0));
    }
    CKR(enq_density(ctx, vb, ss));  // vloc = vH[rho(v)] + vion
    // sigma = sum Im(conj(mu) v) -> psi = vH[sigma]; accumulate the vion gradient
    DensArgs d;
    d.u = vb;
    d.nbocc = ctx->NBocc;
    d.occ = ctx->occ;
    d.vCG = ctx->d_vCG;
    d.vion = ctx->d_vion;
    d.tw = ctx->tw;
    d.dvcell = ctx->dvcell;
    d.rho = ctx->d_sig;
    d.vloc = ctx->d_psi;
    d.scal = ctx->d_scal + 4;
    d.nk = NK;
    d.part = ctx->d_dpart2;
    d.mu = ctx->d_lamk[s];
    d.gvion = ctx->d_gvion;
    CK(launch_density(NG, d, ss));
    AdjCombineArgs c;
    c.mu = ctx->d_lamk[s];
    c.v = ctx->d_vbuf;
    c.Fa = ctx->d_Fa;
    c.psi = ctx->d_psi;
    c.vloc = ctx->d_vloc;
    c.Gx = ctx->d_Gx;
    c.kx = ctx->d_kx;
    c.tw = ctx->tw;
    c.af.mode = amodes[s];
    c.af.val = 0.0;
    c.af.A = ctx->d_A;
    c.af.Aave = ctx->d_Aave;
    c.af.it = n;
    c.nb = NB;
    c.occ = ctx->occ;
    c.lam_u = ctx->d_lamu;
    c.lam_prev = s > 0 ? ctx->d_lamk[s - 1] : nullptr;
    c.cprev = s > 0 ? cst[s - 1] : 0.0;
    c.gcol = ctx->d_gcol;
    c.gstage = ctx->d_gstage;
    c.n = n;
    c.slot = s;
    c.split = 0;
    c.lpre = ctx->d_hpre;
    if (side) {
      AdjCombineArgs pre = c;
      pre.split = 1;
      CK(launch_adj_combine(NG, pre, NK * NB, ctx->st_side));
      CK(cudaEventRecord(ctx->ev_join, ctx->st_side));
      c.split = 2;
    }
    if (ctx->hf) {
      AdjFockArgs f;
      f.v = ctx->d_vbuf;
      f.mu = ctx->d_lamk[s];
      f.kstride = NB * NG;
      f.nk = NK;
      f.nbocc = ctx->NBocc;
      f.S = S;
      f.T = T;
      f.kern = ctx->d_kern;
      f.tw = ctx->tw;
      f.scratch = ctx->d_sym;
      CKR(timed_begin(ctx));
      CK(launch_fock_adj(NG, f, ctx->st));
      CK(launch_sym_reduce(ctx->d_sym, S, T, M, NG, ctx->d_Fa, ctx->st));
      CKR(timed_end(ctx));
    }
    if (side) CK(cudaStreamWaitEvent(ctx->st, ctx->ev_join, 0));
    CK(launch_adj_combine(NG, c, NK * NB, ctx->st));
  }
  CK(cudaMemcpyAsync(ctx->d_lam, ctx->d_lamu, sizeof(double2) * elems, cudaMemcpyDeviceToDevice, ctx->st));
  CK(launch_counter_add(n, -1, ctx->st));
  return MATTOHF_OK;
}

int launch_store_stage(mattohf_ctx* ctx, const double2* src, int slot) {
  CK(launch_stage_copy(nullptr, src, ctx->d_store, ctx->d_int, ctx->d_adj_int + 1, slot, orb_elems(ctx, ctx->NB), 1,
                       ctx->st));
  return MATTOHF_OK;
}

int capture(mattohf_ctx* ctx, cudaGraphExec_t* exec, const std::function<int()>& body) {
  cudaGraph_t g;
  ctx->capturing = true;
  CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
  const int rc = body();
  const cudaError_t ec = cudaStreamEndCapture(ctx->st, &g);
  ctx->capturing = false;
  if (rc != MATTOHF_OK) return rc;
  CK(ec);
  const cudaError_t ei = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  CK(ei);
  return MATTOHF_OK;
}

}  // namespace

extern "C" int mattohf_adjoint(mattohf_ctx* ctx, int objective, int nt, double dt, const double* A,
                               int ckpt_every, double* L, double* dLdA, double* dLdvion) {
  CKR(check_ctx(ctx));
  if (objective != 0 && objective != 1) return fail(ctx, MATTOHF_ERR_ARG, "objective must be 0 (energy) or 1 (current)");
  if (nt < 1 || !A || !(dt > 0.0)) return fail(ctx, MATTOHF_ERR_ARG, "bad adjoint arguments");
  if (ctx->NB != ctx->NBocc) return fail(ctx, MATTOHF_ERR_ARG, "the adjoint needs all bands occupied (NB == NBocc)");
  const int NG = ctx->NG, NB = ctx->NB, NK = ctx->NK;
  const size_t elems = orb_elems(ctx, NB);
  // Segments of at most C steps, aligned to the END of the window: the last
  // segment is [nt - C, nt) and the first one takes the remainder.  The
  // forward pass keeps a checkpoint at the start of every segment but the
  // last, and stores the stage inputs of the last segment itself, so the
  // backward pass recomputes only the nt - C steps before it (none when
  // C >= nt).  Automatic (ckpt_every <= 0): the largest C whose stage inputs
  // (4 per step), checkpoints and work buffers fit in three quarters of the
  // free device memory.
  release_adjoint_storage(ctx);   // a previous call's segments do not count against this one
  size_t freeb = 0, totalb = 0;
  CK(cudaMemGetInfo(&freeb, &totalb));
  int C = ckpt_every;
  if (C <= 0) {
    const long long slots = (long long)(freeb / 4 * 3 / (sizeof(double2) * elems));   // stage-input sized
    long long c = std::min<long long>(nt, (slots - 12) / 4);
    while (c > 1 && 4 * c + (nt + c - 1) / c + 12 > slots) --c;
    C = (int)std::max<long long>(1, c);
  }
  C = std::min(C, nt);
  const int phase = (C - nt % C) % C;        // segment starts: 0 and t with (t + phase) % C == 0
  const int nseg = (nt + phase) / C;
  const int s_last = nt - C;                 // start of the last segment (0 when C == nt)
  const size_t need = sizeof(double2) * elems * ((size_t)nseg + 4 * (size_t)C + 10);
  if (need > freeb) return fail(ctx, MATTOHF_ERR_ALLOC, "checkpoint storage exceeds free device memory; lower ckpt_every");
  CKR(ensure_series(ctx, nt));
  CKR(ensure_scratch(ctx, NK * NB));
  const int M = NK * ctx->NBocc;
  const int S = sym_tile(ctx);
  const int T = (M + S - 1) / S;
  CKR(ensure_sym(ctx, (size_t)T * (T + 1) / 2 * 2 * S * NG));
  if (!ctx->d_symF) CKR(dalloc(ctx, &ctx->d_symF, (size_t)M * NG));
  destroy_graph(ctx);
  CKR(dalloc(ctx, &ctx->d_ckpt, elems * nseg));
  CKR(dalloc(ctx, &ctx->d_store, elems * 4 * C));
  double2** bufs[] = {&ctx->d_lam, &ctx->d_lamu, &ctx->d_vbuf, &ctx->d_Fa, &ctx->d_uN, &ctx->d_u0,
                      &ctx->d_lamk[0], &ctx->d_lamk[1], &ctx->d_lamk[2], &ctx->d_lamk[3]};
  for (double2** b : bufs) CKR(dalloc(ctx, b, elems));
  CKR(dalloc(ctx, &ctx->d_psi, NG));
  CKR(dalloc(ctx, &ctx->d_sig, NG));
  CKR(dalloc(ctx, &ctx->d_vloc_adj, NG));
  CKR(dalloc(ctx, &ctx->d_gvion, NG));
  CKR(dalloc(ctx, &ctx->d_dpart2, (size_t)kDensChunks * NG));
  CKR(dalloc(ctx, &ctx->d_gcol, (size_t)NK * NB));
  CKR(dalloc(ctx, &ctx->d_gstage, (size_t)nt * 4));
  CKR(dalloc(ctx, &ctx->d_adj_int, 4));
  // fields (RT:227-230)
  std::vector<double> Ah(A, A + nt), Aave(nt);
  Aave[0] = 0.5 * (Ah[0] + 0.0);
  for (int i = 1; i < nt; ++i) Aave[i] = 0.5 * (Ah[i] + Ah[i - 1]);
  CK(cudaMemcpyAsync(ctx->d_A, Ah.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, ctx->st));
  CK(cudaMemcpyAsync(ctx->d_Aave, Aave.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, ctx->st));
  AField fm, fave, fcur;
  fm.A = fave.A = fcur.A = ctx->d_A;
  fm.Aave = fave.Aave = fcur.Aave = ctx->d_Aave;
  fm.it = fave.it = fcur.it = ctx->d_int;
  fm.val = fave.val = fcur.val = 0.0;
  fm.mode = AM;
  fave.mode = AAVE;
  fcur.mode = ACUR;

  ScopedEvent e0, e1, e2;
  CK(e0.create());
  CK(e1.create());
  CK(e2.create());
  CK(cudaEventRecord(e0, ctx->st));
  // ---- objective at t = 0 and the forward pass with checkpoints
  double o0[8];
  std::vector<double> rho0(NG), rhoN(NG);
  CKR(enq_observables(ctx, ctx->d_u, aval(0.0), false, false));
  CK(cudaMemcpyAsync(o0, ctx->d_out, sizeof(double) * 7, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(rho0.data(), ctx->d_rho, sizeof(double) * NG, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(ctx->d_u0, ctx->d_u, sizeof(double2) * elems, cudaMemcpyDeviceToDevice, ctx->st));
  CK(cudaMemsetAsync(ctx->d_int, 0, 2 * sizeof(int), ctx->st));
  // the three step graphs, destroyed on every exit path
  // each loop also as kGraphSteps steps in one graph (a graph launch is a
  // full dependency; inside a graph the stages overlap)
  struct Execs {
    cudaGraphExec_t g[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    ~Execs() {
      for (auto x : g)
        if (x) cudaGraphExecDestroy(x);
    }
  } ex;
  cudaGraphExec_t &gfwd = ex.g[0], &grec = ex.g[1], &gadj = ex.g[2];
  cudaGraphExec_t &gfwd8 = ex.g[3], &grec8 = ex.g[4], &gadj8 = ex.g[5];
  auto capture_steps = [&](cudaGraphExec_t* one, cudaGraphExec_t* many, const std::function<int()>& body) {
    int rc = capture(ctx, one, body);
    if (rc == MATTOHF_OK)
      rc = capture(ctx, many, [&]() {
        for (int k = 0; k < kGraphSteps; ++k) CKR(body());
        return MATTOHF_OK;
      });
    return rc;
  };
  auto replay = [&](cudaGraphExec_t one, cudaGraphExec_t many, int n) -> int {
    int j = 0;
    for (; j + kGraphSteps <= n; j += kGraphSteps) CK(cudaGraphLaunch(many, ctx->st));
    for (; j < n; ++j) CK(cudaGraphLaunch(one, ctx->st));
    return MATTOHF_OK;
  };
  // stage-store base step: the store slot of step it is (it - seg0)
  CK(cudaMemsetAsync(ctx->d_adj_int, 0, 4 * sizeof(int), ctx->st));
  // small problems run their forward steps through the fused stages
  if (use_small(ctx)) CKR(ensure_small_buffers(ctx));
  CK(cudaMemsetAsync(ctx->d_ticket, 0, sizeof(unsigned) * (1 + (size_t)NK * NB), ctx->st));
  // gfwd: a step that keeps the segment checkpoint; grec: a step that stores
  // its stage inputs (the last segment in the forward pass, and every
  // recomputed segment)
  int rc = MATTOHF_OK;
  if (nseg > 1)
    rc = capture_steps(&gfwd, &gfwd8, [&]() {
      // the fused stage 0 writes the checkpoint itself
      if (use_small(ctx)) return enq_small_step(ctx, fm, fave, fcur, dt, false, C, phase);
      CK(launch_checkpoint(ctx->d_ckpt, ctx->d_u, ctx->d_int, C, phase, elems, ctx->st));
      CKR(enq_rk4(ctx, fm, fave, fcur, dt, nullptr));
      CK(launch_counter_add(ctx->d_int, 1, ctx->st));
      return MATTOHF_OK;
    });
  if (rc == MATTOHF_OK)
    rc = capture_steps(&grec, &grec8, [&]() { return enq_recompute_step(ctx, fm, fave, fcur, dt); });
  if (rc == MATTOHF_OK) rc = capture_steps(&gadj, &gadj8, [&]() { return enq_adjoint_step(ctx, dt, elems); });
  if (rc != MATTOHF_OK) return rc;
  if (nseg > 1) CKR(replay(gfwd, gfwd8, s_last));
  // the last segment's stage inputs go to store slots it - s_last
  CK(cudaMemcpyAsync(ctx->d_adj_int + 1, &s_last, sizeof(int), cudaMemcpyHostToDevice, ctx->st));
  CKR(replay(grec, grec8, nt - s_last));
  CK(cudaEventRecord(e1, ctx->st));
  // ---- objective at t = T and its gradient
  const double Afin = Ah[nt - 1];
  double oN[8];
  CKR(enq_observables(ctx, ctx->d_u, aval(Afin), false, false));
  CK(cudaMemcpyAsync(oN, ctx->d_out, sizeof(double) * 7, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(rhoN.data(), ctx->d_rho, sizeof(double) * NG, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(ctx->d_uN, ctx->d_u, sizeof(double2) * elems, cudaMemcpyDeviceToDevice, ctx->st));
  Block ub = blk(ctx->d_u, NB, NG, NB);
  if (objective == 0) {
    // dE = <2 occ dvcell h[u] u + (exchange Nyquist term), du>
    CKR(enq_hpsi(ctx, ub, ub, blko(ctx->d_lam, NB, NG, NB), aval(Afin), CM_H));
    CK(launch_scale2(ctx->d_lam, 2.0 * ctx->occ * ctx->dvcell, elems, ctx->st));
    if (ctx->hf)
      CK(launch_energy_grad_nyquist(ctx->d_u, ctx->d_lam, ctx->d_kern, NG, NK, NB, ctx->occ * ctx->dvcell,
                                    ctx->st));
  } else {
    // dJ = <-2 occ (dvcell/vcell) P_A u, du>
    CK(launch_velocity(NG, ctx->d_u, ctx->d_lam, ctx->tw, ctx->d_Gx, ctx->d_kx, NB, Afin,
                       -2.0 * ctx->occ * ctx->dvcell / ctx->vcell, NK * NB, ctx->st));
  }
  CK(cudaMemsetAsync(ctx->d_gvion, 0, sizeof(double) * NG, ctx->st));
  CK(cudaMemsetAsync(ctx->d_gstage, 0, sizeof(double) * 4 * nt, ctx->st));
  // ---- backward over segments: recompute stage inputs, then reverse them
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int s0 = std::max(0, seg * C - phase), len = std::min(nt, (seg + 1) * C - phase) - s0;
    const int hv[2] = {s0 + len - 1, s0};
    if (seg < nseg - 1) {
      CK(cudaMemcpyAsync(ctx->d_u, ctx->d_ckpt + (size_t)seg * elems, sizeof(double2) * elems,
                         cudaMemcpyDeviceToDevice, ctx->st));
      CK(cudaMemcpyAsync(ctx->d_int, &s0, sizeof(int), cudaMemcpyHostToDevice, ctx->st));
      CK(cudaMemcpyAsync(ctx->d_adj_int + 1, &s0, sizeof(int), cudaMemcpyHostToDevice, ctx->st));
      CKR(replay(grec, grec8, len));
    }
    CK(cudaMemcpyAsync(ctx->d_adj_int, hv, 2 * sizeof(int), cudaMemcpyHostToDevice, ctx->st));
    CKR(replay(gadj, gadj8, len));
    CK(cudaStreamSynchronize(ctx->st));  // host values above are stack-resident
  }
  CK(cudaEventRecord(e2, ctx->st));
  std::vector<double> gst((size_t)nt * 4), gv(NG);
  CK(cudaMemcpyAsync(gst.data(), ctx->d_gstage, sizeof(double) * 4 * nt, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(gv.data(), ctx->d_gvion, sizeof(double) * NG, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(ctx->d_u, ctx->d_uN, sizeof(double2) * elems, cudaMemcpyDeviceToDevice, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  float fwd_ms = 0, tot_ms = 0;
  cudaEventElapsedTime(&fwd_ms, e0, e1);
  cudaEventElapsedTime(&tot_ms, e0, e2);
  ctx->last_adj_fwd_ms = fwd_ms;
  ctx->last_adj_ms = tot_ms;
  // ---- chain rule: stage fields (2 Aave - A, Aave, Aave, A) -> samples A[n]
  std::vector<double> gA(nt, 0.0), gAave(nt, 0.0);
  for (int i = 0; i < nt; ++i) {
    const double* g = &gst[(size_t)i * 4];
    gAave[i] += g[1] + g[2] + 2.0 * g[0];
    gA[i] += g[3] - g[0];
  }
  gA[nt - 1] += objective == 0 ? -oN[5] * ctx->vcell : -oN[6] / ctx->vcell;
  for (int i = 0; i < nt; ++i) {
    gA[i] += 0.5 * gAave[i];
    if (i + 1 < nt) gA[i] += 0.5 * gAave[i + 1];
  }
  if (L) *L = objective == 0 ? oN[0] - o0[0] : oN[5];
  if (dLdA) std::copy(gA.begin(), gA.end(), dLdA);
  if (dLdvion) {
    for (int g = 0; g < NG; ++g)
      dLdvion[g] = gv[g] + (objective == 0 ? (rhoN[g] - rho0[g]) * ctx->dvcell : 0.0);
  }
  return MATTOHF_OK;
}

// Taylor expansion of exp(-i dt h[base]) applied to `target` in place
// (RT_TE_ubk, RT:83-89); uses d_k[2] (workbk) and d_k[3] (h workbk).
static int enq_taylor(mattohf_ctx* ctx, double2* target, const double2* base, double Aave, double dt) {
  const int NG = ctx->NG, NB = ctx->NB;
  const size_t n = orb_elems(ctx, NB);
  double2* w = ctx->d_k[2];
  double2* hw = ctx->d_k[3];
  CK(cudaMemcpyAsync(w, target, sizeof(double2) * n, cudaMemcpyDeviceToDevice, ctx->st));
  for (int iorder = 1; iorder <= 4; ++iorder) {
    CKR(enq_hpsi(ctx, blk(base, NB, NG, NB), blk(w, NB, NG, NB), blko(hw, NB, NG, NB), aval(Aave), CM_H));
    CK(launch_te_update(w, hw, nullptr, dt, (double)iorder, target, n, ctx->st));
  }
  return MATTOHF_OK;
}

extern "C" int mattohf_te_step(mattohf_ctx* ctx, int variant, double Aave, double dt) {
  CKR(check_ctx(ctx));
  if (variant < 0 || variant > 2) return fail(ctx, MATTOHF_ERR_ARG, "variant must be 0 (TE), 1 (TEPC) or 2 (TEPC2)");
  const int NG = ctx->NG, NB = ctx->NB;
  const size_t n = orb_elems(ctx, NB);
  double2* u0 = ctx->d_k[0];
  double2* u1 = ctx->d_k[1];
  CK(cudaMemcpyAsync(u0, ctx->d_u, sizeof(double2) * n, cudaMemcpyDeviceToDevice, ctx->st));
  if (variant == 0) {
    CKR(enq_taylor(ctx, ctx->d_u, u0, Aave, dt));
  } else {
    CK(cudaMemcpyAsync(u1, ctx->d_u, sizeof(double2) * n, cudaMemcpyDeviceToDevice, ctx->st));
    CKR(enq_taylor(ctx, u1, u0, Aave, dt));  // predictor (RT:107-112, RT:135-141)
    if (variant == 1) {
      // corrector with the average of h[u0] and h[u1] (RT:114-118)
      double2* w = ctx->d_k[2];
      double2* h0 = ctx->d_k[3];
      double2* h1 = ctx->d_us;
      CK(cudaMemcpyAsync(w, ctx->d_u, sizeof(double2) * n, cudaMemcpyDeviceToDevice, ctx->st));
      for (int iorder = 1; iorder <= 4; ++iorder) {
        CKR(enq_hpsi(ctx, blk(u0, NB, NG, NB), blk(w, NB, NG, NB), blko(h0, NB, NG, NB), aval(Aave), CM_H));
        CKR(enq_hpsi(ctx, blk(u1, NB, NG, NB), blk(w, NB, NG, NB), blko(h1, NB, NG, NB), aval(Aave), CM_H));
        CK(launch_te_update(w, h0, h1, 0.5 * dt, (double)iorder, ctx->d_u, n, ctx->st));
      }
    } else {
      CK(launch_half_sum(u0, u0, u1, n, ctx->st));  // ubk0 = (ubk0 + ubk1)/2 (RT:144)
      CKR(enq_taylor(ctx, ctx->d_u, u0, Aave, dt));
    }
  }
  return sync_and_flag(ctx);
}

extern "C" int mattohf_adjoint_timing(mattohf_ctx* ctx, double* forward_ms, double* total_ms) {
  if (!ctx) return MATTOHF_ERR_ARG;
  if (forward_ms) *forward_ms = ctx->last_adj_fwd_ms;
  if (total_ms) *total_ms = ctx->last_adj_ms;
  return MATTOHF_OK;
}

// ===========================================================================
// Batched ensemble: many independent runs (uneven NK, NB, acell, fields)
// advanced together.  Each run keeps its own mattohf_ctx (tables, orbitals,
// stage buffers, series); per step the batch launches each phase once for
// all runs — density, symmetric exchange over the union of all runs' tile
// pairs, combine over the union of all columns — from argument arrays in
// device memory, and the step is captured once in a CUDA graph.
// ===========================================================================
struct mattohf_batch {
  int R = 0, NG = 0, device = 0;
  std::vector<mattohf_ctx*> runs;
  cudaStream_t st = nullptr;
  int* d_int = nullptr;  // [0] step counter, [1] non-finite flag
  static constexpr int kVariants = 6;  // stages 0..3, observables, observables with exchange
  DensArgs* d_dens[kVariants] = {};
  FockSymArgs* d_fsym[kVariants] = {};
  FockSymDfArgs* d_fsym_df[kVariants] = {};
  CombineArgs* d_comb[kVariants] = {};
  CombineArgs* d_comb_pre[4] = {};  // stages' kinetic + local-potential pass (beside the exchange)
  cudaStream_t st_side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int opt_df = 0;  // exchange transforms in double-float arithmetic
  int opt_tile = 0;  // symmetric-exchange tile of every run (0 = the CTA's teams)
  ObsReduceArgs* d_obs = nullptr;
  ExArgs* d_ex = nullptr;
  ExArgs* d_exf = nullptr;
  int *d_tile_pre = nullptr, *d_elem_pre = nullptr, *d_cta_pre = nullptr;
  int total_tiles = 0, total_elems = 0, total_ctas = 0;
  cudaGraphExec_t exec = nullptr;
  int built_nt = -1;
  std::vector<double> dts;
  double last_ms = 0;
  std::string err;
};

namespace {

int bfail(mattohf_batch* b, int code, const std::string& m) {
  if (b) b->err = m;
  return code;
}

#define BCK(call)                                                                          \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return bfail(b, MATTOHF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
int bupload(mattohf_batch* b, T** d, const std::vector<T>& h) {
  if (*d) cudaFree(*d);
  *d = nullptr;
  if (cudaMalloc((void**)d, sizeof(T) * std::max<size_t>(1, h.size())) != cudaSuccess)
    return bfail(b, MATTOHF_ERR_ALLOC, "batch argument allocation failed");
  BCK(cudaMemcpyAsync(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, b->st));
  return MATTOHF_OK;
}

// Exchange partials of every run for argument variant v (FP64 or double-float).
cudaError_t batch_exchange(mattohf_batch* b, int v) {
  if (b->opt_df)
    return launch_fock_sym_df_batch(b->NG, b->d_fsym[v], b->d_fsym_df[v], b->d_tile_pre, b->R, b->total_tiles,
                                    b->d_elem_pre, b->total_elems, b->st);
  return launch_fock_sym_batch(b->NG, b->d_fsym[v], b->d_tile_pre, b->R, b->total_tiles, b->d_elem_pre,
                               b->total_elems, b->st);
}

// (Re)build every per-run argument array for runs of `nt` steps.
int batch_prepare(mattohf_batch* b, int nt) {
  if (b->built_nt >= nt && b->exec) return MATTOHF_OK;
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  const int R = b->R, NG = b->NG;
  std::vector<DensArgs> dens[mattohf_batch::kVariants];
  std::vector<FockSymArgs> fsym[mattohf_batch::kVariants];
  std::vector<FockSymDfArgs> fsdf[mattohf_batch::kVariants];
  std::vector<CombineArgs> comb[mattohf_batch::kVariants];
  std::vector<CombineArgs> comb_pre[4];
  std::vector<ObsReduceArgs> obs(R);
  std::vector<ExArgs> ex(R), exf(R);
  std::vector<int> tile_pre(R + 1, 0), elem_pre(R + 1, 0), cta_pre(R + 1, 0);
  const int cpc = combine_cols_per_cta(NG);
  // one launch shape (a CTA's teams) for every run; a smaller tile leaves
  // teams idle but gives small runs more CTAs
  const int S = b->opt_tile > 0 ? b->opt_tile : fock_sym_teams(NG);
  for (int r = 0; r < R; ++r) {
    mattohf_ctx* ctx = b->runs[r];
    int rc;
    if ((rc = ensure_series(ctx, nt)) || (rc = ensure_scratch(ctx, ctx->NK * ctx->NB)))
      return bfail(b, rc, ctx->err);
    const int M = ctx->NK * ctx->NBocc;
    const int T = (M + S - 1) / S;
    if ((rc = ensure_sym(ctx, (size_t)T * (T + 1) / 2 * 2 * S * NG))) return bfail(b, rc, ctx->err);
    if (!ctx->d_symF && (rc = dalloc(ctx, &ctx->d_symF, (size_t)M * NG))) return bfail(b, rc, ctx->err);
    if (!ctx->d_udf && (rc = dalloc(ctx, &ctx->d_udf, (size_t)M * NG))) return bfail(b, rc, ctx->err);
    tile_pre[r + 1] = tile_pre[r] + T * (T + 1) / 2;
    elem_pre[r + 1] = elem_pre[r] + M * NG;
    cta_pre[r + 1] = cta_pre[r] + (ctx->NK * ctx->NB + cpc - 1) / cpc;
    AField fld[4];
    for (int i = 0; i < 4; ++i) {
      fld[i].A = ctx->d_A;
      fld[i].Aave = ctx->d_Aave;
      fld[i].it = b->d_int;
      fld[i].val = 0.0;
    }
    fld[0].mode = AM;
    fld[1].mode = AAVE;
    fld[2].mode = AAVE;
    fld[3].mode = ACUR;
    const int modes[4] = {CM_RK0, CM_RK1, CM_RK2, CM_RK3};
    for (int v = 0; v < mattohf_batch::kVariants; ++v) {
      const double2* uin = (v >= 1 && v <= 3) ? ctx->d_us : ctx->d_u;
      Block ub = blk(uin, ctx->NB, NG, ctx->NB);
      DensArgs d;
      d.u = ub;
      d.nbocc = ctx->NBocc;
      d.occ = ctx->occ;
      d.vCG = ctx->d_vCG;
      d.vion = ctx->d_vion;
      d.tw = ctx->tw;
      d.dvcell = ctx->dvcell;
      d.rho = ctx->d_rho;
      d.vloc = ctx->d_vloc;
      d.scal = ctx->d_scal;
      d.nk = ctx->NK;
      d.part = ctx->d_dpart;
      d.mu = nullptr;
      d.gvion = nullptr;
      dens[v].push_back(d);
      FockSymArgs f;
      f.u = ub;
      f.nk = ctx->NK;
      f.nbocc = ctx->NBocc;
      f.S = S;
      f.T = T;
      f.kern = ctx->d_kern;
      f.tw = ctx->tw;
      f.scratch = ctx->d_sym;
      f.F = ctx->d_symF;
      fsym[v].push_back(f);
      FockSymDfArgs fd;
      fd.u = ctx->d_udf;
      fd.nk = ctx->NK;
      fd.nbocc = ctx->NBocc;
      fd.S = S;
      fd.T = T;
      fd.kern = ctx->d_kern_df;
      fd.tw = ctx->d_tw_df;
      fd.scratch = reinterpret_cast<float4*>(ctx->d_sym);
      fd.F = ctx->d_symF;
      fsdf[v].push_back(fd);
      FockPlan fp;
      fp.any = (v != 4);
      fp.sym = ctx->d_symF;
      fp.S = S;
      fp.T = T;
      fp.b0 = ctx->NBocc;
      const AField af = v < 4 ? fld[v] : fld[3];
      CombineArgs c = combine_base(ctx, ub, af, v < 4 ? modes[v] : CM_OBS, fp);
      if (v == 4) {
        c.sym = nullptr;
        c.scratch = nullptr;
      }
      if (v == 5) c.af = aval(0.0);
      c.out = blko(ctx->d_us, ctx->NB, NG, ctx->NB);
      c.dt = b->dts[r];
      c.ex_cols = (v == 0 && ctx->hf) ? 1 : 0;
      c.nonfinite = b->d_int + 1;
      if (v < 4) {
        CombineArgs cp = c;
        cp.split = 1;
        cp.hpre = ctx->d_hpre;
        comb_pre[v].push_back(cp);
        c.split = 2;
        c.hpre = ctx->d_hpre;
      }
      comb[v].push_back(c);
    }
    ObsReduceArgs o;
    o.colbuf = ctx->d_colbuf;
    o.scal = ctx->d_scal;
    o.nk = ctx->NK;
    o.nb = ctx->NB;
    o.nbocc = ctx->NBocc;
    o.occ = ctx->occ;
    o.dvcell = ctx->dvcell;
    o.vcell = ctx->vcell;
    o.NGd = (double)NG;
    o.hf = ctx->hf;
    o.defer_ex = 1;
    o.out = ctx->d_out;
    o.series_E = ctx->d_sE;
    o.series_J = ctx->d_sJ;
    o.series_N = ctx->d_sN;
    o.it = b->d_int;
    o.advance = 2;
    o.nonfinite = b->d_int + 1;
    obs[r] = o;
    ex[r] = ex_args(ctx, ctx->d_sE, -1, nullptr);
    ex[r].it = b->d_int;
    exf[r] = ex_args(ctx, ctx->d_sE, nt - 1, nullptr);
    exf[r].it = b->d_int;
  }
  int rc;
  for (int v = 0; v < mattohf_batch::kVariants; ++v) {
    if ((rc = bupload(b, &b->d_dens[v], dens[v])) || (rc = bupload(b, &b->d_fsym[v], fsym[v])) ||
        (rc = bupload(b, &b->d_fsym_df[v], fsdf[v])) || (rc = bupload(b, &b->d_comb[v], comb[v])))
      return rc;
    if (v < 4 && (rc = bupload(b, &b->d_comb_pre[v], comb_pre[v]))) return rc;
  }
  if ((rc = bupload(b, &b->d_obs, obs)) || (rc = bupload(b, &b->d_ex, ex)) || (rc = bupload(b, &b->d_exf, exf)) ||
      (rc = bupload(b, &b->d_tile_pre, tile_pre)) || (rc = bupload(b, &b->d_elem_pre, elem_pre)) ||
      (rc = bupload(b, &b->d_cta_pre, cta_pre)))
    return rc;
  b->total_tiles = tile_pre[R];
  b->total_elems = elem_pre[R];
  b->total_ctas = cta_pre[R];
  BCK(cudaStreamSynchronize(b->st));
  // capture one step for all runs
  cudaGraph_t g;
  BCK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  for (int s = 0; s < 4 && e == cudaSuccess; ++s) {
    // density and the kinetic + local-potential pass beside the exchange
    e = cudaEventRecord(b->ev_fork, b->st);
    if (e != cudaSuccess) break;
    cudaError_t es = cudaStreamWaitEvent(b->st_side, b->ev_fork, 0);
    if (es == cudaSuccess) es = launch_density_batch(NG, b->d_dens[s], R, b->st_side);
    if (es == cudaSuccess)
      es = launch_combine_batch(NG, b->d_comb_pre[s], b->d_cta_pre, R, b->total_ctas, b->st_side);
    const cudaError_t ej = cudaEventRecord(b->ev_join, b->st_side);
    e = batch_exchange(b, s);
    const cudaError_t ew = cudaStreamWaitEvent(b->st, b->ev_join, 0);
    if (e == cudaSuccess) e = es != cudaSuccess ? es : (ej != cudaSuccess ? ej : ew);
    if (e == cudaSuccess) e = launch_combine_batch(NG, b->d_comb[s], b->d_cta_pre, R, b->total_ctas, b->st);
    if (e == cudaSuccess && s == 0) e = launch_ex_finalize_batch(b->d_ex, R, b->st);
  }
  if (e == cudaSuccess) e = launch_density_batch(NG, b->d_dens[4], R, b->st);
  if (e == cudaSuccess) e = launch_combine_batch(NG, b->d_comb[4], b->d_cta_pre, R, b->total_ctas, b->st);
  if (e == cudaSuccess) e = launch_obs_reduce_batch(b->d_obs, R, b->st);
  if (e == cudaSuccess) e = launch_step_advance(b->d_int, b->st);
  cudaError_t ec = cudaStreamEndCapture(b->st, &g);
  BCK(e);
  BCK(ec);
  cudaError_t ei = cudaGraphInstantiate(&b->exec, g, 0);
  cudaGraphDestroy(g);
  BCK(ei);
  b->built_nt = nt;
  return MATTOHF_OK;
}

}  // namespace

extern "C" {

int mattohf_batch_create(int nruns, const mattohf_config* cfgs, mattohf_batch** out) {
  if (!out || !cfgs || nruns < 1) return MATTOHF_ERR_ARG;
  *out = nullptr;
  for (int r = 0; r < nruns; ++r) {
    if (cfgs[r].NG != cfgs[0].NG || cfgs[r].device != cfgs[0].device) return MATTOHF_ERR_ARG;
    if (cfgs[r].NB != cfgs[r].NBocc) return MATTOHF_ERR_ARG;  // all bands occupied (symmetric exchange)
  }
  mattohf_batch* b = new mattohf_batch();
  b->R = nruns;
  b->NG = cfgs[0].NG;
  b->device = cfgs[0].device;
  b->dts.assign(nruns, 0.0);
  for (int r = 0; r < nruns; ++r) {
    mattohf_ctx* c = nullptr;
    const int rc = mattohf_create(&cfgs[r], &c);
    if (rc != MATTOHF_OK) {
      mattohf_batch_destroy(b);
      return rc;
    }
    b->runs.push_back(c);
  }
  if (cudaSetDevice(b->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->st_side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming) != cudaSuccess ||
      cudaMalloc(&b->d_int, 4 * sizeof(int)) != cudaSuccess ||
      cudaMemset(b->d_int, 0, 4 * sizeof(int)) != cudaSuccess) {
    mattohf_batch_destroy(b);
    return MATTOHF_ERR_CUDA;
  }
  *out = b;
  return MATTOHF_OK;
}

int mattohf_batch_destroy(mattohf_batch* b) {
  if (!b) return MATTOHF_OK;
  cudaSetDevice(b->device);
  if (b->st) cudaStreamSynchronize(b->st);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  for (int v = 0; v < mattohf_batch::kVariants; ++v) {
    cudaFree(b->d_dens[v]);
    cudaFree(b->d_fsym[v]);
    cudaFree(b->d_fsym_df[v]);
    cudaFree(b->d_comb[v]);
  }
  void* ptrs[] = {b->d_obs, b->d_ex, b->d_exf, b->d_tile_pre, b->d_elem_pre, b->d_cta_pre, b->d_int};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (auto* c : b->runs) mattohf_destroy(c);
  for (int v = 0; v < 4; ++v) cudaFree(b->d_comb_pre[v]);
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  if (b->ev_join) cudaEventDestroy(b->ev_join);
  if (b->st_side) cudaStreamDestroy(b->st_side);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
  return MATTOHF_OK;
}

const char* mattohf_batch_last_error(const mattohf_batch* b) { return b ? b->err.c_str() : "null batch"; }

mattohf_ctx* mattohf_batch_run(mattohf_batch* b, int run) {
  if (!b || run < 0 || run >= b->R) return nullptr;
  return b->runs[run];
}

int mattohf_batch_rk4_run(mattohf_batch* b, int nt, const double* dt, const double* A, const double* Aave,
                          double* Etot, double* Je, double* Nele) {
  if (!b || nt < 0 || (nt > 0 && (!dt || !A || !Aave))) return MATTOHF_ERR_ARG;
  if (nt == 0) return MATTOHF_OK;
  BCK(cudaSetDevice(b->device));
  bool dt_changed = false;
  for (int r = 0; r < b->R; ++r) {
    if (!(dt[r] > 0.0) || !std::isfinite(dt[r])) return bfail(b, MATTOHF_ERR_ARG, "dt must be positive");
    if (b->dts[r] != dt[r]) dt_changed = true;
    b->dts[r] = dt[r];
  }
  if (dt_changed || b->built_nt < nt) {
    b->built_nt = -1;
    int rc = batch_prepare(b, nt);
    if (rc != MATTOHF_OK) return rc;
  } else {
    // the final-exchange arguments depend on nt
    std::vector<ExArgs> exf(b->R);
    for (int r = 0; r < b->R; ++r) {
      exf[r] = ex_args(b->runs[r], b->runs[r]->d_sE, nt - 1, nullptr);
      exf[r].it = b->d_int;
    }
    BCK(cudaMemcpyAsync(b->d_exf, exf.data(), sizeof(ExArgs) * b->R, cudaMemcpyHostToDevice, b->st));
  }
  // every run's orbitals were set on its own stream
  for (auto* c : b->runs) BCK(cudaStreamSynchronize(c->st));
  for (int r = 0; r < b->R; ++r) {
    mattohf_ctx* c = b->runs[r];
    BCK(cudaMemcpyAsync(c->d_A, A + (size_t)r * nt, sizeof(double) * nt, cudaMemcpyHostToDevice, b->st));
    BCK(cudaMemcpyAsync(c->d_Aave, Aave + (size_t)r * nt, sizeof(double) * nt, cudaMemcpyHostToDevice, b->st));
  }
  BCK(cudaMemsetAsync(b->d_int, 0, 2 * sizeof(int), b->st));
  ScopedEvent e0, e1;
  BCK(e0.create());
  BCK(e1.create());
  BCK(cudaEventRecord(e0, b->st));
  int flag = 0, bad_at = -1;
  for (int it = 0; it < nt; ++it) {
    BCK(cudaGraphLaunch(b->exec, b->st));
    if ((it & 255) == 255 && it + 1 < nt) {
      BCK(cudaMemcpyAsync(&flag, b->d_int + 1, sizeof(int), cudaMemcpyDeviceToHost, b->st));
      BCK(cudaStreamSynchronize(b->st));
      if (flag) {
        bad_at = it;
        break;
      }
    }
  }
  // exchange energy of the last step's orbitals
  const int NG = b->NG;
  BCK(launch_density_batch(NG, b->d_dens[5], b->R, b->st));
  BCK(batch_exchange(b, 5));
  BCK(launch_combine_batch(NG, b->d_comb[5], b->d_cta_pre, b->R, b->total_ctas, b->st));
  BCK(launch_ex_finalize_batch(b->d_exf, b->R, b->st));
  BCK(cudaEventRecord(e1, b->st));
  BCK(cudaEventSynchronize(e1));
  float ms = 0;
  BCK(cudaEventElapsedTime(&ms, e0, e1));
  b->last_ms = ms;
  const int ndone = bad_at >= 0 ? bad_at + 1 : nt;
  for (int r = 0; r < b->R; ++r) {
    mattohf_ctx* c = b->runs[r];
    if (Etot) BCK(cudaMemcpyAsync(Etot + (size_t)r * nt, c->d_sE, sizeof(double) * ndone, cudaMemcpyDeviceToHost, b->st));
    if (Je) BCK(cudaMemcpyAsync(Je + (size_t)r * nt, c->d_sJ, sizeof(double) * ndone, cudaMemcpyDeviceToHost, b->st));
    if (Nele) BCK(cudaMemcpyAsync(Nele + (size_t)r * nt, c->d_sN, sizeof(double) * ndone, cudaMemcpyDeviceToHost, b->st));
  }
  BCK(cudaMemcpyAsync(&flag, b->d_int + 1, sizeof(int), cudaMemcpyDeviceToHost, b->st));
  BCK(cudaStreamSynchronize(b->st));
  if (flag) return bfail(b, MATTOHF_ERR_NONFINITE, "non-finite state in the ensemble");
  return MATTOHF_OK;
}

int mattohf_batch_set_option(mattohf_batch* b, int option, long long value) {
  if (!b) return MATTOHF_ERR_ARG;
  if (option == MATTOHF_OPT_FOCK_DF64) {
    b->opt_df = value ? 1 : 0;
  } else if (option == MATTOHF_OPT_SYM_TILE) {
    if (value < 0 || value > fock_sym_teams(b->NG) || (value & (value - 1)))
      return bfail(b, MATTOHF_ERR_ARG, "tile size must be 0 or a power of two up to the CTA's teams");
    b->opt_tile = (int)value;
  } else {
    return bfail(b, MATTOHF_ERR_ARG, "unsupported batch option");
  }
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  b->built_nt = -1;
  return MATTOHF_OK;
}

// Batch autotuner: the exchange tile shared by every run's tile pairs, timed
// over `steps` graph-replayed ensemble steps (dt = 1e-4, A = 0) per
// candidate on the runs' current orbitals, which are restored.  out: the tile
// kept; us: microseconds of an ensemble step at that tile.
int mattohf_batch_autotune(mattohf_batch* b, int steps, int* tile, double* us) {
  if (!b || steps < 1 || steps > 100000) return MATTOHF_ERR_ARG;
  BCK(cudaSetDevice(b->device));
  for (auto* c : b->runs) BCK(cudaStreamSynchronize(c->st));
  std::vector<double2*> saved(b->R, nullptr);
  struct Free {
    std::vector<double2*>& v;
    ~Free() {
      for (auto* p : v)
        if (p) cudaFree(p);
    }
  } guard{saved};
  for (int r = 0; r < b->R; ++r) {
    mattohf_ctx* c = b->runs[r];
    const size_t n = orb_elems(c, c->NB);
    BCK(cudaMalloc((void**)&saved[r], sizeof(double2) * n));
    BCK(cudaMemcpyAsync(saved[r], c->d_u, sizeof(double2) * n, cudaMemcpyDeviceToDevice, b->st));
  }
  auto restore = [&]() -> int {
    for (int r = 0; r < b->R; ++r) {
      mattohf_ctx* c = b->runs[r];
      BCK(cudaMemcpyAsync(c->d_u, saved[r], sizeof(double2) * orb_elems(c, c->NB), cudaMemcpyDeviceToDevice,
                          b->st));
    }
    BCK(cudaStreamSynchronize(b->st));
    return MATTOHF_OK;
  };
  const std::vector<double> dts0 = b->dts;
  const int tile0 = b->opt_tile;
  std::vector<double> A((size_t)b->R * steps, 0.0), dt(b->R, 1e-4);
  double best = 1e300;
  int bestS = 0, rc = MATTOHF_OK;
  for (int S = fock_sym_teams(b->NG); S >= 1 && rc == MATTOHF_OK; S >>= 1) {
    b->opt_tile = S;
    b->built_nt = -1;
    double t = 0.0;
    for (int pass = 0; pass < 2 && rc == MATTOHF_OK; ++pass) {  // the first pass builds the graph
      if ((rc = restore()) != MATTOHF_OK) break;
      rc = mattohf_batch_rk4_run(b, steps, dt.data(), A.data(), A.data(), nullptr, nullptr, nullptr);
      t = 1e3 * b->last_ms / steps;
    }
    if (rc == MATTOHF_OK && t < best) {
      best = t;
      bestS = S;
    }
  }
  const int rr = restore();
  b->dts = dts0;
  b->built_nt = -1;
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  if (rc != MATTOHF_OK) {
    b->opt_tile = tile0;
    return rc;
  }
  if (rr != MATTOHF_OK) return rr;
  b->opt_tile = bestS;
  if (tile) *tile = bestS;
  if (us) *us = best;
  return MATTOHF_OK;
}

int mattohf_batch_last_run_ms(mattohf_batch* b, double* ms) {
  if (!b || !ms) return MATTOHF_ERR_ARG;
  *ms = b->last_ms;
  return MATTOHF_OK;
}

// The adjoint of every member, one member at a time.  A member of the largest
// shapes (NG = 512, NK = 128, Nocc = 8: half a million exchange pairs per
// apply) fills the FP64 pipe by itself, so members side by side would gain no
// throughput and would split the device memory that the checkpoint segments
// use; in turn, each member gets all of it (its segment is fitted to the free
// memory when ckpt_every <= 0) and releases it before the next one starts.
int mattohf_batch_adjoint(mattohf_batch* b, int objective, int nt, const double* dt, const double* A,
                          int ckpt_every, double* L, double* dLdA, double* dLdvion) {
  if (!b) return MATTOHF_ERR_ARG;
  if (nt < 1 || !dt || !A) return bfail(b, MATTOHF_ERR_ARG, "bad batch adjoint arguments");
  double ms = 0.0;
  for (int r = 0; r < b->R; ++r) {
    mattohf_ctx* c = b->runs[r];
    const int rc = mattohf_adjoint(c, objective, nt, dt[r], A + (size_t)r * nt, ckpt_every,
                                   L ? L + r : nullptr, dLdA ? dLdA + (size_t)r * nt : nullptr,
                                   dLdvion ? dLdvion + (size_t)r * b->NG : nullptr);
    release_adjoint_storage(c);
    if (rc != MATTOHF_OK) return bfail(b, rc, "run " + std::to_string(r) + ": " + c->err);
    ms += c->last_adj_ms;
  }
  b->last_ms = ms;
  return MATTOHF_OK;
}

}  // extern "C"
