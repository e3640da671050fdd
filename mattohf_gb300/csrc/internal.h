// Internal declarations shared by the host runtime and the kernel translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace mattohf {

constexpr int kThreads = 128;  // threads per CTA for the column/pair kernels (4 warps)
constexpr int kDensChunks = 32; // column chunks of the two-stage density reduction
constexpr int kCombineWarps = 1; // warps per CTA of the per-column combine kernels (spread over SMs)

// How a kernel obtains the vector potential of the current launch.
//   AVAL : use `A_val` directly
//   AM   : A(it-1) recovered as 2*Aave(it) - A(it)        (src/RT_calculation.f90:165)
//   AAVE : Aave(it)
//   ACUR : A(it)
enum AMode : int { AVAL = 0, AM = 1, AAVE = 2, ACUR = 3 };

struct AField {
  int mode;
  double val;
  const double* A;      // device, per time step
  const double* Aave;   // device, per time step
  const int* it;        // device step counter (0-based)
};

__device__ __forceinline__ double afield_value(const AField& f) {
  if (f.mode == AVAL) return f.val;
  const int it = *f.it;
  if (f.mode == AM) return 2.0 * f.Aave[it] - f.A[it];
  if (f.mode == AAVE) return f.Aave[it];
  return f.A[it];
}

// Orbital-like arrays are [NK][ld][NG] complex128; a "block" view selects `nb`
// consecutive bands starting at band offset `b0` of every k.
struct Block {
  const double2* p;  // points at band b0 of k = 0
  int kstride;       // complex elements between consecutive k (ld * NG)
  int nb;            // bands per k in this view
};
struct BlockOut {
  double2* p;
  int kstride;
  int nb;
};

struct DensArgs {
  Block u;            // all NB bands
  int nbocc;
  double occ;         // 2/NK for occupied bands, 0 otherwise (src/Initialization.f90:179-186)
  const double* vCG;  // NG
  const double* vion; // NG
  const double2* tw;  // NG forward twiddles
  double dvcell;
  double* rho;        // NG out
  double* vloc;       // NG out: vH + vion
  double* scal;       // out: [0]=Nele, [1]=Eion, [2]=EH
  int nk;
  double* part;       // scratch [kDensChunks][NG] partial densities
  // adjoint mode (mu != null): accumulate sigma = sum_cols Im(conj(mu) u)
  // instead of the density, write vH[sigma] to vloc (no vion), and add
  // sigma to gvion (if non-null)
  const double2* mu;
  double* gvion;
};

struct FockArgs {
  Block u;              // occupied orbitals (bands 0..nbocc-1 used)
  Block w;              // rows the exchange operator acts on
  int nk, nbocc;
  const double* kern;   // (2NK-1) x NG : -v(G + kx(kr) - kx(kc)) / (NG*NK), index d = kr-kc+NK-1
  const double2* tw;
  double2* scratch;     // [ncols*nchunks][NG] partial sums
  int nchunks;
  int chunk;            // pairs per chunk
};

// Occupied-pair symmetric exchange (w == u): tiles of S occupied orbitals,
// one CTA per tile pair (i <= j); partials [tp][2][S][NG] (rows, columns).
struct FockSymArgs {
  Block u;
  int nk, nbocc;
  int S;                // tile size = teams per CTA
  int T;                // number of tiles = ceil(NK*nbocc / S)
  const double* kern;
  const double2* tw;
  double2* scratch;
  double2* F;           // reduced exchange term of the occupied orbitals [NK*nbocc][NG]
};

// Symmetric exchange with double-float pair transforms (k_fock_df.cu).
struct FockSymDfArgs {
  const float4* u;      // occupied orbitals as df [NK*nbocc][NG]
  int nk, nbocc;
  int S, T;
  const float2* kern;   // df copy of the kernel table
  const float4* tw;     // df twiddles
  float4* scratch;      // tile partials (double-float), layout as FockSymArgs
  double2* F;           // reduced exchange [NK*nbocc][NG]
};
cudaError_t launch_fock_sym_df(int NG, const FockSymDfArgs& a, const double2* u, int kstride, float4* udf,
                               cudaStream_t s);
cudaError_t configure_df_kernels();
cudaError_t launch_fock_sym_df_batch(int NG, const FockSymArgs* d_src, const FockSymDfArgs* d_args,
                                     const int* d_tile_pre, int nruns, int total_tiles, const int* d_elem_pre,
                                     int total_elems, cudaStream_t s);
cudaError_t launch_to_df_tables(const double* kern, int nkern, float2* kern_df, const double2* tw, int ntw,
                                float4* tw_df, cudaStream_t s);

__host__ __device__ __forceinline__ int sym_tp(int i, int j, int T) {
  return i * T - (i * (i - 1)) / 2 + (j - i);
}

// The reduction of the symmetric-exchange partials sums, for output orbital
// (tile i, slot l) at grid point q, the T + 1 terms t = 0 .. T in a fixed
// order: the column partials of tile pairs (t, i), t < i; the row and then the
// column partial of (i, i); the row partials of (i, t - 1), t > i + 1.
// Each output element is split into kRedQ contiguous runs of terms summed by
// separate threads, then added in run order: deterministic, and kRedQ times
// more loads in flight than one thread per element.
constexpr int kRedQ = 4;    // term runs per output element
constexpr int kRedE = 64;   // output elements per CTA (CTA = kRedQ * kRedE threads)
__device__ __forceinline__ size_t sym_term(int t, int i, int l, int q, int S, int T, int N) {
  const size_t SN = (size_t)S * N;
  size_t tp;
  bool col;
  if (t < i) {
    tp = sym_tp(t, i, T);
    col = true;
  } else if (t == i) {
    tp = sym_tp(i, i, T);
    col = false;
  } else if (t == i + 1) {
    tp = sym_tp(i, i, T);
    col = true;
  } else {
    tp = sym_tp(i, t - 1, T);
    col = false;
  }
  return tp * 2 * SN + (col ? SN : 0) + (size_t)l * N + q;
}
__device__ __forceinline__ void sym_run_bounds(int T, int c, int* t0, int* t1) {
  const int nt = T + 1, L = (nt + kRedQ - 1) / kRedQ;
  *t0 = c * L;
  *t1 = min(nt, *t0 + L);
}

enum CombineMode : int {
  CM_H = 0,     // out = T_A w + vloc w + F
  CM_RK0 = 1,   // k0 = -i h ; next = u0 + (0.5 dt) k0
  CM_RK1 = 2,   // k1 = -i h ; next = u0 + (0.5 dt) k1
  CM_RK2 = 3,   // k2 = -i h ; next = u0 + dt k2
  CM_RK3 = 4,   // u0 += (k0 + 2 k1 + 2 k2 + k3) dt / 6
  CM_OBS = 5,   // per-column Ekin, Je, <w|F> partials (no array output)
  CM_F = 6,     // out = F only (exchange term alone)
  CM_T = 7,     // out = T_A w only (kinetic term alone)
};

struct CombineArgs {
  Block w;                  // columns being processed (the h-apply's wbk)
  const double2* sym;       // reduced symmetric exchange [NK*nbocc][NG] for occupied columns (or null)
  int sym_S, sym_T;
  int chunk_b0;             // first band whose exchange comes from the chunked partials
  int ex_cols;              // CM_RK0: also store <w|F> per occupied column (deferred Ex)
  BlockOut out;             // h output (CM_H / CM_F / CM_T) or stage input (CM_RK0..2)
  double2* u0;              // RK4 base state [NK][NB][NG] (CM_RK*)
  double2* kbuf[4];         // RK4 stage derivatives [NK][NB][NG]
  const double2* scratch;   // Fock partials (may be null when the Fock term is off)
  int nchunks;
  const double* vloc;       // NG
  const double* Gx;         // NG
  const double* kx;         // NK
  const double2* tw;
  AField af;
  double dt;
  int mode;
  int nk;
  int nbocc;
  double occ;
  double* colbuf;           // CM_OBS: [ncols][4] = Ekin part, J part, Re<w|F>, Im<w|F>
  int* nonfinite;           // set to 1 if any output is not finite
  // 0: whole combine.  1: only T_A w + vloc w -> hpre (runs beside the
  // exchange).  2: hpre + exchange, then the mode's epilogue (no transforms).
  int split;
  double2* hpre;            // [NK][NB][NG]
};

// Fused RK4 stage for small problems (k_small.cu).  Each output column (k, b)
// is served by P CTAs that share its exchange pairs; the last of them to
// finish (a per-column ticket) sums the P partials in a fixed order and does
// the density-dependent kinetic/local terms and the stage's RK4 update, and
// the last column to finish (a global ticket) writes the observables.  A step
// is 4 launches instead of about 29, spread over ncols * P CTAs.
struct SmallStageArgs {
  const double2* u;         // stage input [NK][NB][NG]
  double2* u0;              // base state (updated in place by stage 3)
  double2* out;             // stage output (stages 0..2), never the input
  double2* kbuf[3];         // RK4 stage derivatives
  int mode;                 // 0..3: RK4 stage; 4: observables of u0 only (closing pass)
  double dt;
  AField af;
  const double* Aobs;       // A(t) samples: observables of stage 0 / mode 4 use A[it - 1]
  int nk, nb, nbocc, hf;
  int P;                    // CTAs per column
  double occ, dvcell, vcell;
  const double* kern;       // (2NK-1) x NG exchange kernel table
  const double* vCG;
  const double* vion;
  const double* Gx;
  const double* kx;
  const double2* tw;
  double2* part;            // [ncols][P][NG] exchange partials, then [ncols][NG] (rho, vH),
                            // then [ncols][NG] kinetic term T_A w
  double* colbuf;           // [ncols][4]: Ekin part, J part, Re<u|F>, Im<u|F>
  double* series_E;         // per-step observables, indexed by the step counter
  double* series_J;
  double* series_N;
  int* it;                  // step counter read by this stage
  int* it_out;              // if set, block 0 writes *it + it_inc here (a counter no CTA of
  int it_inc;               // this stage reads): stage 0 copies the counter to its shadow,
                            // stage 3 reads the shadow and writes the next step's index
  int* nonfinite;
  unsigned* ticket;         // [1 + ncols]: global, then per-column completion counters
  double* out_obs;          // mode 4: [7] Etot, Ekin, Eion, EH, Ex, Je, Nele
  double* obs_dens;         // [2][NG]: density and vH of stage 0's input (column 0), read by stage 1
  double2* store;           // if set: the adjoint's stage store; the stage input goes to slot
  const int* seg0;          // ((*it - *seg0) * 4 + store_slot) (each CTA copies its points)
  int store_slot;
  double2* ckpt;            // stage 0, if set: the input goes to checkpoint (it + ckpt_phase) /
  int ckpt_every;           // ckpt_every when it == 0 or (it + ckpt_phase) % ckpt_every == 0
  int ckpt_phase;
};
// CTAs per column of the fused stages: one thread-block cluster per column
// (the portable cluster size)
constexpr int kSmallMaxCtas = 8;
cudaError_t launch_small_stage(int NG, const SmallStageArgs& a, cudaStream_t s);
bool small_stage_supported(int NG);
int small_pair_teams(int NG);
cudaError_t configure_small_kernels();

// Fused reverse RK4 stage for small problems (all bands occupied): the
// adjoint of one stage as enq_adjoint_step forms it, in one launch over
// ncols * P CTAs.  Column a's CTAs split the ordered pairs (a, b) of the
// adjoint exchange; the column's first CTA also forms vloc = vH[rho(v)] + vion,
// psi = vH[sigma] and the kinetic term and field-gradient partial of column a;
// the column's last CTA does the stage bookkeeping, the last column the
// ordered field-gradient sum.
struct SmallAdjArgs {
  const double2* store;     // stage-input store; v = store[(n - seg0) * 4 + slot]
  int* n;                   // backward step (device); stage 0 decrements it
  const int* seg0;          // first step of the stored segment (device)
  int slot;                 // RK4 stage 0..3
  const double2* mu;        // this stage's adjoint lam_k[slot]
  double2* lam_u;           // += J^T mu
  double2* lam_prev;        // += cprev * J^T mu (lam_k[slot - 1]), or null
  double cprev;
  double2* lam;             // stage 0: lam = lam_u after the update
  AField af;                // stage field (it = n)
  int nk, nb, P;
  double occ;
  const double* kern;
  const double* vCG;
  const double* vion;
  const double* Gx;
  const double* kx;
  const double2* tw;
  double2* part;            // [ncols][P][NG] partials, then [ncols][NG] (vloc, psi), then [ncols][NG] T_A mu
  double* gcol;             // [ncols] field-gradient partials
  double* gstage;           // [nt][4]
  double* gvion;            // += sigma
  unsigned* ticket;         // [1 + ncols], as for the forward stages
};
cudaError_t launch_small_adj(int NG, const SmallAdjArgs& a, cudaStream_t s);
int small_adj_pair_warps_teams(int NG);
cudaError_t configure_small_adj_kernels();

struct ObsReduceArgs {
  const double* colbuf;     // [nk*nb][4]
  const double* scal;       // dens scalars: Nele, Eion, EH
  int nk, nb, nbocc;
  double occ, dvcell, vcell, NGd;
  int hf;
  int defer_ex;             // 1: Etot excludes Ex (added later by k_ex_finalize)
  double* out;              // [0]=Etot [1]=Ekin [2]=Eion [3]=EH [4]=Ex [5]=Je [6]=Nele
  double* series_E;         // per step (may be null)
  double* series_J;
  double* series_N;
  int* it;                  // step counter
  int advance;              // 0: no series; 1: write series[it] and increment it; 2: write only
  int* nonfinite;
};

// Launchers (defined in k_hpsi.cu); all return cudaGetLastError() of the launch.
cudaError_t launch_density(int NG, const DensArgs& a, cudaStream_t s);
cudaError_t launch_fock(int NG, const FockArgs& a, int ncols, cudaStream_t s);
cudaError_t launch_fock_sym(int NG, const FockSymArgs& a, cudaStream_t s);
int fock_sym_teams(int NG);  // teams of a full symmetric-exchange CTA (largest tile size)
int choose_sym_tile(int NG, int M, int nsm);  // tile size for a single run of M occupied orbitals on nsm SMs
cudaError_t sym_launch_params(int NG, int S, int* threads, size_t* smem);
cudaError_t configure_kernels();
struct ExArgs {
  const double* colbuf;
  int nk, nb, nbocc;
  double occ, dvcell;
  double* series_E;   // Etot series; Ex added to entry it-1 (or `idx` when >= 0)
  const int* it;
  int idx;
  double* out;        // optional: [0] += Ex, [4] = Ex
};
cudaError_t launch_ex_finalize(const ExArgs& a, cudaStream_t s);
cudaError_t launch_combine(int NG, const CombineArgs& a, int ncols, cudaStream_t s);
cudaError_t launch_obs_reduce(const ObsReduceArgs& a, cudaStream_t s);

// Batched launchers: per-run argument structs live in device memory; work
// items map to runs through exclusive prefix arrays (pre[0] = 0, pre[nruns] = total).
cudaError_t launch_density_batch(int NG, const DensArgs* d_args, int nruns, cudaStream_t s);
cudaError_t launch_fock_sym_batch(int NG, const FockSymArgs* d_args, const int* d_tile_pre, int nruns,
                                  int total_tiles, const int* d_elem_pre, int total_elems,
                                  cudaStream_t s);
int combine_cols_per_cta(int NG);
cudaError_t launch_combine_batch(int NG, const CombineArgs* d_args, const int* d_cta_pre, int nruns,
                                 int total_ctas, cudaStream_t s);
cudaError_t launch_obs_reduce_batch(const ObsReduceArgs* d_args, int nruns, cudaStream_t s);
cudaError_t launch_ex_finalize_batch(const ExArgs* d_args, int nruns, cudaStream_t s);
cudaError_t launch_step_advance(int* it, cudaStream_t s);

// ---- adjoint (k_adjoint.cu) ----
struct AdjFockArgs {
  const double2* v;     // stage input [NK][NB][NG]
  const double2* mu;    // adjoint of the stage derivative, same layout
  int kstride;          // NB * NG
  int nk, nbocc, S, T;
  const double* kern;
  const double2* tw;
  double2* scratch;     // tile partials, as FockSymArgs
};
struct AdjCombineArgs {
  const double2* mu;
  const double2* v;
  const double2* Fa;    // reduced exchange part of J^T mu (includes the factor i)
  const double* psi;    // vH[sigma]
  const double* vloc;   // vH[rho(v)] + vion
  const double* Gx;
  const double* kx;
  const double2* tw;
  AField af;
  int nb;
  double occ;
  double2* lam_u;       // += J^T mu
  double2* lam_prev;    // += cprev * J^T mu (previous stage's adjoint), or null
  double cprev;
  double* gcol;         // per-column field-gradient partials
  double* gstage;       // [nt][4] stage-field gradients
  const int* n;         // current step
  int slot;             // stage index 0..3
  // 0: whole pass.  1: the part without the exchange, i (T_a + vloc) mu -> lpre,
  // and the field-gradient partials (runs beside the exchange).  2: lpre + Fa
  // + Hartree response, then the stage bookkeeping (no transforms).
  int split;
  double2* lpre;        // [NK][NB][NG]
};
cudaError_t launch_fock_adj(int NG, const AdjFockArgs& a, cudaStream_t s);
cudaError_t configure_adjoint_kernels();
cudaError_t launch_sym_reduce(const double2* part, int S, int T, int M, int N, double2* F, cudaStream_t s);
cudaError_t launch_adj_combine(int NG, const AdjCombineArgs& a, int ncols, cudaStream_t s);
cudaError_t launch_adj_init(const double2* lam, double2* lam_u, double2* const* lamk, double dt, size_t n,
                            cudaStream_t s);
cudaError_t launch_stage_copy(double2* dst, const double2* src, double2* store, const int* n, const int* seg0,
                              int slot, size_t elems, int to_store, cudaStream_t s);
cudaError_t launch_checkpoint(double2* ckpt, const double2* u, const int* it, int every, int phase, size_t elems,
                              cudaStream_t s);
cudaError_t launch_counter_add(int* p, int d, cudaStream_t s);
cudaError_t launch_velocity(int NG, const double2* u, double2* out, const double2* tw, const double* Gx,
                            const double* kx, int nb, double A, double scale, int ncols, cudaStream_t s);
cudaError_t launch_scale2(double2* x, double sc, size_t n, cudaStream_t s);
// g += the Nyquist term of the exchange-energy gradient (all nk*nb columns of u
// occupied); sc = occ * dvcell
cudaError_t launch_energy_grad_nyquist(const double2* u, double2* g, const double* kern, int NG, int nk, int nb,
                                       double sc, cudaStream_t s);

cudaError_t launch_te_update(double2* w, const double2* h0, const double2* h1, double c, double iorder,
                             double2* acc, size_t n, cudaStream_t s);
cudaError_t launch_half_sum(double2* out, const double2* a, const double2* b, size_t n, cudaStream_t s);

// Tables (k_table.cu)
// k_vCk (F:33-52) at nq arguments; d_g: scratch of vck_points(acell, NG, NK) doubles
long long vck_points(double acell, int NG, int NK);
cudaError_t launch_vck_table(int NG, int NK, double acell, const double* d_q, int nq, double* d_g,
                             double* d_out, cudaStream_t s);
cudaError_t launch_make_kern(int NG, int NK, const double* vcq, double* kern, cudaStream_t s);

// Ground-state kernels (k_gs.cu)
struct GsArgs {
  double2* u;      // [NK][ld][NG]
  int kstride;     // ld*NG
  int nb;          // columns per k to process
  double weight;   // inner-product weight (vcell/NG or dvcell)
  int* flag;       // error flag
};
cudaError_t launch_gram_schmidt(int NG, const GsArgs& a, int nk, cudaStream_t s);
// Projected matrix M[k][i][j] = <x_i|y_j>*weight for i,j < m
cudaError_t launch_project(int NG, const double2* x, const double2* y, int kstride, int m,
                           double weight, double2* M, int nk, cudaStream_t s);
// Jacobi eigen-decomposition of nk Hermitian m x m matrices (hermitised from the
// lower triangle, real diagonal); eigenvalues ascending, vectors in columns.
cudaError_t launch_jacobi(const double2* M, int m, double* evals, double2* evecs, int nk,
                          int* flag, cudaStream_t s);
// out[k][b] = sum_c x[k][c] * C[k][c][b] for b < nout
cudaError_t launch_rotate(int NG, const double2* x, int xkstride, int m, const double2* C,
                          int nout, double2* out, int okstride, int nk, cudaStream_t s);
// Orthonormalise m columns per k (two passes of MGS) under weight.
cudaError_t launch_block_orth(int NG, double2* x, int kstride, int m, double weight,
                              int nk, int* flag, cudaStream_t s);
// eps[k][b] = Re<u|h u> w ; err[k][b] = sqrt(sum|h u - eps u| * w)
cudaError_t launch_eps(int NG, const double2* u, const double2* hu, int kstride, int nb,
                       double w, double* eps, double* err, int nk, cudaStream_t s);

}  // namespace mattohf
