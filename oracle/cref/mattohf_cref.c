/* C restatement of mATTOHF's real-time hot path — TEST INFRASTRUCTURE ONLY.
 *
 * The timed CPU baseline (bench.py `cpu_baseline` and `--impl reference`) and
 * a cross-check of the numpy oracle.  Nothing in the product links it.
 *
 * parity unpinned: the reference (Fortran + MPI + FFTW3 + LAPACK) cannot be
 * built on either machine (no Fortran compiler, FFTW or LAPACK), so this is a
 * restatement of its loops, cross-checked against the numpy oracle.
 *
 * Follows, routine by routine:
 *   k_vCk                src/Functions.f90:33-52
 *   ubk_dns              src/Functions.f90:55-71     (ig -> ik -> ib order)
 *   dns_vH               src/Functions.f90:147-162
 *   ubk_tubk             src/Functions.f90:212-234
 *   ubkwbk_vFwbk         src/Functions.f90:237-261   (kk -> ibr -> ibc order per output)
 *   ubkwbk_hwbk          src/Functions.f90:187-209
 *   ubk_Ekin/Eion/EH/Ex  src/Functions.f90:94-183
 *   ubk_Je               src/Functions.f90:289-318
 *   RT_RK4_ubk           src/RT_calculation.f90:154-173
 *   RT loop body         src/RT_calculation.f90:38-60
 * The reference's MPI split of the k-pair loop (F:247, reduced by
 * MPI_ALLREDUCE at F:258) becomes an OpenMP loop over output columns.
 * FFTW is replaced by a radix-2 Stockham FFT with the same sign and
 * normalisation conventions (forward e^{-i}, backward e^{+i}, unnormalised).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  int NG, NK, NB, NBocc, hf;
  double acell, vcell, dvcell, bx, occ;
  double *Gx, *kx, *rx, *vion, *vCG, *vCq; /* vCq[(2NK-1)*NG], index kr-kc+NK-1 */
  double *tw;                              /* 2*NG: exp(-2 pi i m / NG) */
  double *k[4], *us, *hw, *rho, *vloc;
} cref;

static const double PI_ = 3.14159265358979323846264338327950288;

/* ---------------------------------------------------------------- FFT ---- */
/* Stockham radix-2 (decimation in frequency, autosort), x and y 2*n doubles;
 * result in x.  sign -1 forward, +1 backward. */
static void fft(int n, double* x, double* y, const double* tw, int sign) {
  double* a = x;
  double* b = y;
  int s = 1;
  for (int len = n; len > 1; len >>= 1, s <<= 1) {
    const int m = len >> 1;
    for (int p = 0; p < m; ++p) {
      const double wr = tw[2 * (p * s)], wi = sign < 0 ? tw[2 * (p * s) + 1] : -tw[2 * (p * s) + 1];
      for (int q = 0; q < s; ++q) {
        const double* pa = a + 2 * (q + s * p);
        const double* pb = a + 2 * (q + s * (p + m));
        const double ar = pa[0], ai = pa[1], br = pb[0], bi = pb[1];
        double* o0 = b + 2 * (q + s * (2 * p));
        double* o1 = b + 2 * (q + s * (2 * p + 1));
        o0[0] = ar + br;
        o0[1] = ai + bi;
        const double dr = ar - br, di = ai - bi;
        o1[0] = dr * wr - di * wi;
        o1[1] = dr * wi + di * wr;
      }
    }
    double* t = a;
    a = b;
    b = t;
  }
  if (a != x) memcpy(x, a, sizeof(double) * 2 * n);
}

/* ------------------------------------------------------------ tables ---- */
static double k_vCk(double k, double acell, int NG, int NK) {
  const double dx = acell / (double)NG / 20.0;
  const double lim = (double)NK * acell;
  double v = 0.0;
  long long ix = 0;
  while ((double)ix * dx < lim) {
    const double x0 = (double)ix * dx, x1 = (double)(ix + 1) * dx;
    v = v + 0.5 * (cos(k * x0) / sqrt(x0 * x0 + 1.0) + cos(k * x1) / sqrt(x1 * x1 + 1.0));
    ++ix;
  }
  return 2.0 * v * dx;
}

cref* cref_create(int NG, int NK, int NB, int NBocc, double acell, int hf, const double* vion,
                  const double* vCG, const double* vCq) {
  cref* c = (cref*)calloc(1, sizeof(cref));
  c->NG = NG; c->NK = NK; c->NB = NB; c->NBocc = NBocc; c->hf = hf;
  c->acell = acell;
  c->vcell = fabs(acell);
  c->bx = 2.0 * PI_ / acell;
  c->dvcell = c->vcell / (double)NG;
  c->occ = 2.0 / (double)NK;
  c->Gx = malloc(sizeof(double) * NG);
  c->rx = malloc(sizeof(double) * NG);
  c->kx = malloc(sizeof(double) * NK);
  c->vion = malloc(sizeof(double) * NG);
  c->vCG = malloc(sizeof(double) * NG);
  c->vCq = malloc(sizeof(double) * (size_t)(2 * NK - 1) * NG);
  c->tw = malloc(sizeof(double) * 2 * NG);
  for (int i = 0; i < NG; ++i) {
    c->rx[i] = (double)i / (double)NG * acell;
    c->Gx[i] = (i < NG / 2 ? (double)i : (double)(i - NG)) * c->bx;
    c->tw[2 * i] = cos(2.0 * PI_ * i / NG);
    c->tw[2 * i + 1] = -sin(2.0 * PI_ * i / NG);
  }
  for (int i = 1; i <= NK; ++i) c->kx[i - 1] = (-0.5 + (2.0 * i - 1.0) / (double)(2 * NK)) * c->bx;
  memcpy(c->vion, vion, sizeof(double) * NG);
  if (vCG && vCq) {
    memcpy(c->vCG, vCG, sizeof(double) * NG);
    memcpy(c->vCq, vCq, sizeof(double) * (size_t)(2 * NK - 1) * NG);
  } else {
    /* vCGkk columns for each distinct kr-kc (I:130-137) and vCG (I:143-146) */
    const int nd = 2 * NK - 1;
#pragma omp parallel for schedule(dynamic, 4)
    for (int t = 0; t < (nd + 1) * NG; ++t) {
      const int d = t / NG, g = t % NG;
      if (d < nd) {
        const int diff = d - (NK - 1);
        const int kr = diff > 0 ? diff : 0, kc = kr - diff;
        c->vCq[t] = k_vCk((c->Gx[g] + c->kx[kr]) - c->kx[kc], acell, NG, NK);
      } else {
        c->vCG[g] = k_vCk(c->Gx[g], acell, NG, NK);
      }
    }
    c->vCG[0] = 0.0;
  }
  const size_t nu = (size_t)2 * NK * NB * NG;
  for (int s = 0; s < 4; ++s) c->k[s] = malloc(sizeof(double) * nu);
  c->us = malloc(sizeof(double) * nu);
  c->hw = malloc(sizeof(double) * nu);
  c->rho = malloc(sizeof(double) * NG);
  c->vloc = malloc(sizeof(double) * NG);
  return c;
}

void cref_get_tables(const cref* c, double* vCG, double* vCq) {
  if (vCG) memcpy(vCG, c->vCG, sizeof(double) * c->NG);
  if (vCq) memcpy(vCq, c->vCq, sizeof(double) * (size_t)(2 * c->NK - 1) * c->NG);
}

void cref_destroy(cref* c) {
  if (!c) return;
  free(c->Gx); free(c->rx); free(c->kx); free(c->vion); free(c->vCG); free(c->vCq); free(c->tw);
  for (int s = 0; s < 4; ++s) free(c->k[s]);
  free(c->us); free(c->hw); free(c->rho); free(c->vloc);
  free(c);
}

int cref_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Threads for the following calls (n >= 1); returns the count now in effect. */
int cref_set_threads(int n) {
#ifdef _OPENMP
  if (n >= 1) omp_set_num_threads(n);
#else
  (void)n;
#endif
  return cref_threads();
}

/* ------------------------------------------------------------ kernels ---- */
static void density(const cref* c, const double* u, double* rho) {
  const int NG = c->NG, NB = c->NB;
  for (int ig = 0; ig < NG; ++ig) {
    double s = 0.0;
    for (int ik = 0; ik < c->NK; ++ik)
      for (int ib = 0; ib < NB; ++ib) {
        const double occ = ib < c->NBocc ? c->occ : 0.0;
        const double* z = u + 2 * (((size_t)ik * NB + ib) * NG + ig);
        s += (occ * z[0]) * z[0] + (occ * z[1]) * z[1];
      }
    rho[ig] = s;
  }
}

static void hartree(const cref* c, const double* rho, double* vH) {
  const int NG = c->NG;
  double* x = malloc(sizeof(double) * 4 * NG);
  double* y = x + 2 * NG;
  for (int g = 0; g < NG; ++g) { x[2 * g] = rho[g]; x[2 * g + 1] = 0.0; }
  fft(NG, x, y, c->tw, -1);
  for (int g = 0; g < NG; ++g) { x[2 * g] *= c->vCG[g]; x[2 * g + 1] *= c->vCG[g]; }
  fft(NG, x, y, c->tw, +1);
  for (int g = 0; g < NG; ++g) vH[g] = x[2 * g] / (double)NG;
  free(x);
}

/* h[u] w for nbw bands of w; `fock_only` skips kinetic/local. */
static void hpsi(cref* c, const double* u, const double* w, int nbw, double A, double* hw,
                 int fock_only) {
  const int NG = c->NG, NK = c->NK, NB = c->NB, NBocc = c->NBocc;
  density(c, u, c->rho);
  hartree(c, c->rho, c->vloc);
  for (int g = 0; g < NG; ++g) c->vloc[g] += c->vion[g];
#pragma omp parallel
  {
    double* x = malloc(sizeof(double) * 6 * NG);
    double* y = x + 2 * NG;
    double* acc = y + 2 * NG;
#pragma omp for schedule(dynamic, 1)
    for (int col = 0; col < NK * nbw; ++col) {
      const int kr = col / nbw, ibr = col % nbw;
      const double* wc = w + 2 * (size_t)col * NG;
      double* out = hw + 2 * (size_t)col * NG;
      /* kinetic (F:224-232) + local (F:199-203) */
      const double kAx = c->kx[kr] + A, kA2 = kAx * kAx;
      if (fock_only) {
        memset(out, 0, sizeof(double) * 2 * NG);
      } else {
      memcpy(x, wc, sizeof(double) * 2 * NG);
      fft(NG, x, y, c->tw, -1);
      for (int g = 0; g < NG; ++g) {
        const double G = c->Gx[g];
        const double m = 0.5 * (G * G + 2.0 * G * kAx + kA2);
        x[2 * g] = m * x[2 * g] / (double)NG;
        x[2 * g + 1] = m * x[2 * g + 1] / (double)NG;
      }
      fft(NG, x, y, c->tw, +1);
      for (int g = 0; g < NG; ++g) {
        out[2 * g] = x[2 * g] + c->vloc[g] * wc[2 * g];
        out[2 * g + 1] = x[2 * g + 1] + c->vloc[g] * wc[2 * g + 1];
      }
      }
      if (!c->hf) continue;
      /* Fock (F:247-257) for this output column */
      memset(acc, 0, sizeof(double) * 2 * NG);
      for (int kc = 0; kc < NK; ++kc) {
        const double* v = c->vCq + (size_t)(kr - kc + NK - 1) * NG;
        for (int ibc = 0; ibc < NBocc; ++ibc) {
          const double* uc = u + 2 * (((size_t)kc * NB + ibc) * NG);
          for (int g = 0; g < NG; ++g) {
            const double wr = wc[2 * g], wi = wc[2 * g + 1], ur = uc[2 * g], ui = uc[2 * g + 1];
            x[2 * g] = (wr * ur + wi * ui) / (double)NK;
            x[2 * g + 1] = (wi * ur - wr * ui) / (double)NK;
          }
          fft(NG, x, y, c->tw, -1);
          for (int g = 0; g < NG; ++g) {
            x[2 * g] = -v[g] * x[2 * g] / (double)NG;
            x[2 * g + 1] = -v[g] * x[2 * g + 1] / (double)NG;
          }
          fft(NG, x, y, c->tw, +1);
          for (int g = 0; g < NG; ++g) {
            const double fr = x[2 * g], fi = x[2 * g + 1], ur = uc[2 * g], ui = uc[2 * g + 1];
            acc[2 * g] += fr * ur - fi * ui;
            acc[2 * g + 1] += fr * ui + fi * ur;
          }
        }
      }
      for (int g = 0; g < 2 * NG; ++g) out[g] = out[g] + acc[g];
    }
    free(x);
  }
}

void cref_hpsi(cref* c, const double* u, const double* w, int nbw, double A, double* hw) {
  hpsi(c, u, w, nbw, A, hw, 0);
}

/* Etot, Je, Nele of u at field A (F:74-183, F:289-318, RT:43-45). */
static void observables(cref* c, const double* u, double A, double* Etot, double* Je, double* Nele) {
  const int NG = c->NG, NK = c->NK, NB = c->NB, NBocc = c->NBocc;
  density(c, u, c->rho);
  double* vH = malloc(sizeof(double) * NG);
  hartree(c, c->rho, vH);
  double sn = 0, si = 0, sh = 0;
  for (int g = 0; g < NG; ++g) {
    sn += c->rho[g];
    si += c->vion[g] * c->rho[g];
    sh += vH[g] * c->rho[g];
  }
  free(vH);
  double ekin = 0.0, jre = 0.0;
  double* x = malloc(sizeof(double) * 4 * NG);
  double* y = x + 2 * NG;
  for (int ik = 0; ik < NK; ++ik)
    for (int ib = 0; ib < NB; ++ib) {
      const double occ = ib < NBocc ? c->occ : 0.0;
      const double* uc = u + 2 * (((size_t)ik * NB + ib) * NG);
      memcpy(x, uc, sizeof(double) * 2 * NG);
      fft(NG, x, y, c->tw, -1);
      const double kAx = c->kx[ik] + A, kA2 = kAx * kAx;
      double ek = 0.0, je = 0.0;
      for (int g = 0; g < NG; ++g) {
        const double G = c->Gx[g];
        const double m2 = x[2 * g] * x[2 * g] + x[2 * g + 1] * x[2 * g + 1];
        ek += 0.5 * (G * G + 2.0 * G * kAx + kA2) * m2;
        je += (G + c->kx[ik] + A) * m2;
      }
      ekin += occ * (ek / (double)NG) * c->dvcell;
      jre += occ * (je / (double)NG);
    }
  free(x);
  double ex = 0.0;
  if (c->hf) {
    /* Ex = 0.5 sum_occ occ <u|VF u> dvcell: one Fock apply with w = u (F:165-183) */
    double* vF = malloc(sizeof(double) * 2 * (size_t)NK * NB * NG);
    hpsi(c, u, u, NB, A, vF, 1);
    for (int ik = 0; ik < NK; ++ik)
      for (int ib = 0; ib < NBocc; ++ib) {
        const size_t o = 2 * (((size_t)ik * NB + ib) * NG);
        double s = 0.0;
        for (int g = 0; g < NG; ++g) s += u[o + 2 * g] * vF[o + 2 * g] + u[o + 2 * g + 1] * vF[o + 2 * g + 1];
        ex += c->occ * s * c->dvcell;
      }
    free(vF);
  }
  *Etot = ekin + si * c->dvcell + 0.5 * sh * c->dvcell + 0.5 * ex;
  *Je = -(jre * c->dvcell / c->vcell);
  *Nele = sn * c->dvcell;
}

void cref_observables(cref* c, const double* u, double A, double* Etot, double* Je, double* Nele) {
  observables(c, u, A, Etot, Je, Nele);
}

/* RT_RK4_ubk (RT:154-173) then the observables of RT:43-47, nt times. */
void cref_rk4_run(cref* c, double* u, int nt, double dt, const double* Aarr, const double* Aave,
                  double* Et, double* Jt, double* Nt) {
  const size_t n = (size_t)2 * c->NK * c->NB * c->NG;
  const int NB = c->NB;
  for (int it = 0; it < nt; ++it) {
    const double A = Aarr[it], Aa = Aave[it], Am = 2.0 * Aa - A;
    const double fld[4] = {Am, Aa, Aa, A};
    const double cdt[3] = {0.5 * dt, 0.5 * dt, dt};
    for (int s = 0; s < 4; ++s) {
      const double* in = s == 0 ? u : c->us;
      hpsi(c, in, in, NB, fld[s], c->hw, 0);
      double* k = c->k[s];
      for (size_t i = 0; i < n; i += 2) {  /* k = -i h */
        k[i] = c->hw[i + 1];
        k[i + 1] = -c->hw[i];
      }
      if (s < 3)
        for (size_t i = 0; i < n; ++i) c->us[i] = u[i] + cdt[s] * k[i];
    }
    for (size_t i = 0; i < n; ++i) {
      double sx = c->k[0][i] + 2.0 * c->k[1][i];
      sx = sx + 2.0 * c->k[2][i];
      sx = sx + c->k[3][i];
      u[i] = u[i] + sx * dt / 6.0;
    }
    double E, J, N;
    observables(c, u, A, &E, &J, &N);
    if (Et) Et[it] = E;
    if (Jt) Jt[it] = J;
    if (Nt) Nt[it] = N;
  }
}
