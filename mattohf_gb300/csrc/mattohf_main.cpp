// mattohf: drop-in driver for the reference program over the C ABI.
//
// The reference's `Program Main` (src/mATTOHF.f90:1-131) reads the name of an
// input file from standard input (src/mATTOHF.f90:45), reads the keyword
// input (Read_input, src/mATTOHF.f90:198-272), then runs Initialization, the
// initial guess and Gram_Schmidt, GS_calculation and RT_calculation and
// writes its output files.  This program does the same with every hot-path
// step on the GPU through libmattohf.so, and writes the same files:
//
//   potential.out            rx, vion                  (src/Prep_periodic_ion_potential.f90:23-27)
//   vk.out                   Gx+kx, k_vCk(Gx+kx)       (src/Initialization.f90:149-155)
//   <sys>_GSinfo.out         SCF history + energy components (src/GS_calculation.f90:21-24, 49-52, 63-90)
//   <sys>_DoS.out, _band.out band energies and broadened DoS (src/GS_calculation.f90:93-118, 239-265)
//   <sys>_EtotNJEAt.out      time, Etot, dEtot, Nele, dNele, J, E, A (src/RT_calculation.f90:22-24, 52-53)
//   <sys>_JEAF.out, _sigmaeps.out (LR) or _JEAF_window.out (LP)   (src/RT_calculation.f90:246-351)
//   <sys>_dipole.out         time, P = -int J dt (extension; trapezoid from J(0))
//
// Usage: `echo '"input.dat"' | mattohf [output directory]`.  An empty name
// keeps every default of src/Global_variables.f90:7-26.  Exit status 0 on
// success, 1 on any library or input error (the message names the call).
#include <algorithm>
#include <charconv>
#include <chrono>
#include <cmath>
#include <limits>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "mattohf.h"

namespace {

// src/Constants.f90:5-18
const double kPi = 4.0 * std::atan(1.0);
const double kHartree = 27.2116;
const double kAtomtime = 0.02419;
const double kAtomfield = 514.2;
const double kAtomfluence = 3.509e16 * kAtomtime * 1.0e-15;

// The reference's global inputs with their defaults (src/Global_variables.f90:7-26).
struct Config {
  double acell = 10.0;
  int NG = 64, NK = 8, NB = 2, NBocc = 2;
  std::vector<double> Zeff{2.0}, alpha{1.0}, Rion{0.5};
  std::vector<int> Kion{1};
  std::string functional = "HF";
  std::string sys_name;
  int Nscf = 100, NCG = 5, NT = 2000;
  double dt = 0.5;
  int Nomega = 4000;
  double omegaM = 4.0;
  std::string field_option = "LP";
  double dAc = (double)0.0001f;  // single-precision default literal (GV:19)
  double omegac = 1.55;          // eV
  double Tpulse = 16.0;          // fs
  double phiCEP = 0.5;           // units of 2 pi
  int nenvelope = 4;
  double E0 = 1.0;               // V/nm
};

struct Failure : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// ---------------------------------------------------------------------------
// Read_input (src/mATTOHF.f90:198-272): a keyword on its own record, its value
// on the following record(s), list-directed (only the first value counts;
// unknown records are skipped; `functional` has no case and keeps its default).
// ---------------------------------------------------------------------------
std::string trim(const std::string& s) {
  const size_t a = s.find_first_not_of(" \t\r\n");
  if (a == std::string::npos) return "";
  const size_t b = s.find_last_not_of(" \t\r\n");
  return s.substr(a, b - a + 1);
}

// First list-directed item of a record; empty for a blank record.
std::string first_token(const std::string& line, bool* blank) {
  const std::string s = trim(line);
  *blank = s.empty();
  if (s.empty()) return "";
  if (s[0] == '\'' || s[0] == '"') {
    const size_t end = s.find(s[0], 1);
    return end == std::string::npos ? s.substr(1) : s.substr(1, end - 1);
  }
  const size_t end = s.find_first_of(" \t,/");
  return end == std::string::npos ? s : s.substr(0, end);
}

struct Records {
  std::vector<std::string> lines;
  size_t pos = 0;

  // n items from the next records (a list-directed READ of n values).
  std::vector<std::string> items(int n) {
    std::vector<std::string> out;
    while ((int)out.size() < n) {
      if (pos >= lines.size()) throw Failure("input ended inside a read");
      std::string rec = trim(lines[pos++]);
      if (rec.empty()) continue;
      std::replace(rec.begin(), rec.end(), ',', ' ');
      std::istringstream ss(rec);
      std::string t;
      while (ss >> t) {
        if (t == "/") break;
        t.erase(std::remove(t.begin(), t.end(), '\''), t.end());
        t.erase(std::remove(t.begin(), t.end(), '"'), t.end());
        out.push_back(t);
        if ((int)out.size() == n) break;
      }
    }
    return out;
  }
};

double freal(std::string t) {
  for (char& c : t)
    if (c == 'd' || c == 'D') c = 'e';
  size_t used = 0;
  const double v = std::stod(t, &used);
  if (used != t.size()) throw Failure("bad real value '" + t + "'");
  return v;
}

int fint(const std::string& t) {
  size_t used = 0;
  const int v = std::stoi(t, &used);
  if (used != t.size()) throw Failure("bad integer value '" + t + "'");
  return v;
}

Config read_input(const std::string& path) {
  std::ifstream in(path);
  if (!in) throw Failure("cannot open input file '" + path + "'");
  Records r;
  for (std::string l; std::getline(in, l);) r.lines.push_back(l);
  Config c;
  while (r.pos < r.lines.size()) {
    bool blank = false;
    const std::string key = first_token(r.lines[r.pos++], &blank);
    if (blank) continue;
    if (key == "NB") c.NB = fint(r.items(1)[0]);
    else if (key == "NBocc") c.NBocc = fint(r.items(1)[0]);
    else if (key == "NG") c.NG = fint(r.items(1)[0]);
    else if (key == "NK") c.NK = fint(r.items(1)[0]);
    else if (key == "Nscf") c.Nscf = fint(r.items(1)[0]);
    else if (key == "NCG") c.NCG = fint(r.items(1)[0]);
    else if (key == "NT") c.NT = fint(r.items(1)[0]);
    else if (key == "Nomega") c.Nomega = fint(r.items(1)[0]);
    else if (key == "nenvelope") c.nenvelope = fint(r.items(1)[0]);
    else if (key == "acell") c.acell = freal(r.items(1)[0]);
    else if (key == "dt") c.dt = freal(r.items(1)[0]);
    else if (key == "omegaM") c.omegaM = freal(r.items(1)[0]);
    else if (key == "dAc") c.dAc = freal(r.items(1)[0]);
    else if (key == "omegac") c.omegac = freal(r.items(1)[0]);
    else if (key == "Tpulse") c.Tpulse = freal(r.items(1)[0]);
    else if (key == "phiCEP") c.phiCEP = freal(r.items(1)[0]);
    else if (key == "E0") c.E0 = freal(r.items(1)[0]);
    else if (key == "sys_name" || key == "field_option") {
      bool b = true;
      std::string v;
      while (r.pos < r.lines.size() && b) v = first_token(r.lines[r.pos++], &b);
      if (key == "field_option") c.field_option = v.substr(0, 2);
      else c.sys_name = v;
    } else if (key == "dir_name" || key == "DFT_option" || key == "TD_option" || key == "Band_option") {
      r.items(1);
    } else if (key == "atoms") {
      const int ns = fint(r.items(1)[0]);
      const std::vector<std::string> z = r.items(ns), a = r.items(ns);
      const int ni = fint(r.items(1)[0]);
      c.Zeff.clear();
      c.alpha.clear();
      c.Rion.clear();
      c.Kion.clear();
      for (const auto& t : z) c.Zeff.push_back(freal(t));
      for (const auto& t : a) c.alpha.push_back(freal(t));
      for (int i = 0; i < ni; ++i) {
        const std::vector<std::string> rk = r.items(2);
        c.Rion.push_back(freal(rk[0]));
        c.Kion.push_back(fint(rk[1]));
      }
    }
  }
  return c;
}

// x**m for integer m by square-and-multiply (how x**n is evaluated in Fortran).
double powi(double x, int m) {
  int n = std::abs(m);
  double y = (n % 2) ? x : 1.0;
  n >>= 1;
  while (n) {
    x = x * x;
    if (n % 2) y = y * x;
    n >>= 1;
  }
  return m < 0 ? 1.0 / y : y;
}

// Define_Afield (src/RT_calculation.f90:175-244).
void define_afield(const Config& c, std::vector<double>& time, std::vector<double>& A, std::vector<double>& Aave,
                   std::vector<double>& E) {
  const int NT = c.NT;
  time.assign(NT, 0.0);
  A.assign(NT, 0.0);
  Aave.assign(NT, 0.0);
  E.assign(NT, 0.0);
  for (int it = 0; it < NT; ++it) time[it] = c.dt * (double)it;
  if (c.field_option == "LR") {
    std::fill(A.begin(), A.end(), c.dAc);
  } else if (c.field_option == "LP") {
    const double omegac = c.omegac / kHartree, Tpulse = c.Tpulse / kAtomtime, E0 = c.E0 / kAtomfield;
    const double Aamp = E0 / omegac;
    const int NTpulse = (int)std::min(Tpulse / c.dt, (double)NT);
    for (int it = 0; it < NTpulse; ++it) {
      const double t = time[it];
      A[it] = Aamp * std::sin(omegac * (t - 0.5 * Tpulse) + 2.0 * kPi * c.phiCEP) *
              powi(std::sin(kPi * t / Tpulse), c.nenvelope);
    }
  } else {
    throw Failure("field_option must be 'LR' or 'LP'");
  }
  for (int it = 0; it < NT; ++it) {
    const double prev = it ? A[it - 1] : 0.0;
    Aave[it] = 0.5 * (A[it] + prev);
    E[it] = -(A[it] - prev) / c.dt;
  }
}

// ---------------------------------------------------------------------------
// Output formats
// ---------------------------------------------------------------------------
// Fortran Ew.d (Ee) edit descriptor: 0.ddddE+xx right-justified in w columns.
std::string fortran_e(double x, int w = 20, int d = 12, int e = 2) {
  std::string s;
  if (!std::isfinite(x)) {
    s = std::isnan(x) ? "NaN" : (x > 0 ? "Infinity" : "-Infinity");
  } else {
    std::string mant;
    int ex = 0;
    bool neg;
    if (x == 0.0) {
      mant.assign(d, '0');
      neg = std::signbit(x);
    } else {
      neg = x < 0;
      char buf[64];
      std::snprintf(buf, sizeof buf, "%.*e", d - 1, std::fabs(x));
      const char* ep = std::strchr(buf, 'e');
      for (const char* p = buf; p < ep; ++p)
        if (*p != '.') mant.push_back(*p);
      ex = std::atoi(ep + 1) + 1;
    }
    int lim = 1;
    for (int i = 0; i < e; ++i) lim *= 10;
    char eb[16];
    if (std::abs(ex) < lim) std::snprintf(eb, sizeof eb, "E%c%0*d", ex >= 0 ? '+' : '-', e, std::abs(ex));
    else std::snprintf(eb, sizeof eb, "%c%0*d", ex >= 0 ? '+' : '-', e + 1, std::abs(ex));
    s = std::string(neg ? "-" : "") + "0." + mant + eb;
    if ((int)s.size() > w) return std::string(w, '*');
  }
  return std::string(std::max(0, w - (int)s.size()), ' ') + s;
}

std::string row(const std::vector<double>& v, int w = 20, int d = 12, int e = 2) {
  std::string s;
  for (double x : v) s += fortran_e(x, w, d, e);
  return s;
}

// Shortest round-trip decimal, laid out like Python's repr of a float.
std::string repr(double x) {
  if (!std::isfinite(x)) return std::isnan(x) ? "nan" : (x > 0 ? "inf" : "-inf");
  char buf[64];
  auto res = std::to_chars(buf, buf + sizeof buf, x, std::chars_format::scientific);
  std::string sci(buf, res.ptr);
  const size_t ep = sci.find('e');
  std::string digits = sci.substr(0, ep);
  const int ex = std::atoi(sci.c_str() + ep + 1);
  const bool neg = digits[0] == '-';
  if (neg) digits.erase(0, 1);
  digits.erase(std::remove(digits.begin(), digits.end(), '.'), digits.end());
  std::string out;
  if (ex < -4 || ex >= 16) {
    out = digits.substr(0, 1);
    if (digits.size() > 1) out += "." + digits.substr(1);
    char eb[16];
    std::snprintf(eb, sizeof eb, "e%c%02d", ex >= 0 ? '+' : '-', std::abs(ex));
    out += eb;
  } else if (ex < 0) {
    out = "0." + std::string(-ex - 1, '0') + digits;
  } else if ((int)digits.size() <= ex + 1) {
    out = digits + std::string(ex + 1 - digits.size(), '0') + ".0";
  } else {
    out = digits.substr(0, ex + 1) + "." + digits.substr(ex + 1);
  }
  return (neg ? "-" : "") + out;
}

std::string rjust(const std::string& s, int w) { return std::string(std::max(0, w - (int)s.size()), ' ') + s; }

// Fortran Fw.d: w asterisks when the value does not fit, Infinity for +-inf.
std::string fixed(double x, int w, int d) {
  if (std::isinf(x)) return rjust(x > 0 ? "Infinity" : "-Infinity", w);
  char b[400];
  std::snprintf(b, sizeof b, "%.*f", d, x);
  std::string s = b;
  if ((int)s.size() > w && (s.rfind("0.", 0) == 0 || s.rfind("-0.", 0) == 0)) s.erase(s.find('0'), 1);
  return (int)s.size() <= w ? rjust(s, w) : std::string(w, '*');
}

const double kHuge = std::numeric_limits<double>::max();  // Fortran huge(1.d0): minval of an empty section

// '(i5,3e20.12,4x,1e20.12,4x,1000e20.12)' (src/GS_calculation.f90:102, 114): the
// first group takes kx, the mean residual and epsbk(1); each 4x and the group
// after it appear only while bands remain.
std::string band_record(int ik, double kx, double errsum, const std::vector<double>& ek) {
  std::vector<double> items{kx, errsum};
  items.insert(items.end(), ek.begin(), ek.end());
  char b[16];
  std::snprintf(b, sizeof b, "%5d", ik);
  std::string s = b + row(std::vector<double>(items.begin(), items.begin() + std::min<size_t>(3, items.size())));
  if (items.size() > 3) s += "    " + row({items[3]});
  if (items.size() > 4) s += "    " + row(std::vector<double>(items.begin() + 4, items.end()));
  return s;
}

// The last two GSinfo columns (src/GS_calculation.f90:51-52).  With every band
// occupied, minval over the empty conduction section is huge(1.d0), and the
// second column reads epsbk(NB+1,ik), i.e. epsbk(1,ik+1) in column-major
// storage; the k-point ik = NK, whose read lies past the array, is left out.
std::vector<double> gap_columns(const std::vector<double>& eps, int NK, int NB, int NBocc) {
  double vmax = -kHuge, cmin = kHuge, opt = kHuge;
  for (int ik = 0; ik < NK; ++ik)
    for (int ib = 0; ib < NB; ++ib) {
      const double x = eps[(size_t)ik * NB + ib];
      if (ib < NBocc) vmax = std::max(vmax, x);
      else cmin = std::min(cmin, x);
    }
  if (NBocc < NB) {
    for (int ik = 0; ik < NK; ++ik)
      opt = std::min(opt, eps[(size_t)ik * NB + NBocc] - eps[(size_t)ik * NB + NBocc - 1]);
    return {cmin - vmax, opt};
  }
  for (int ik = 0; ik + 1 < NK; ++ik) opt = std::min(opt, eps[(size_t)(ik + 1) * NB] - eps[(size_t)ik * NB + NB - 1]);
  return {kHuge - vmax, opt};
}

// ---------------------------------------------------------------------------
// Library calls
// ---------------------------------------------------------------------------
void check(mattohf_ctx* ctx, int st, const char* what) {
  if (st == MATTOHF_OK) return;
  std::string m = std::string(what) + ": " + mattohf_status_string(st);
  if (ctx) m += ": " + std::string(mattohf_last_error(ctx));
  throw Failure(m);
}

struct Context {
  mattohf_ctx* h = nullptr;
  explicit Context(const Config& c) {
    mattohf_config m{};
    m.NG = c.NG;
    m.NK = c.NK;
    m.NB = c.NB;
    m.NBocc = c.NBocc;
    m.acell = c.acell;
    m.functional_hf = trim(c.functional) == "HF" ? 1 : 0;
    m.device = 0;
    m.nspecies = (int)c.Zeff.size();
    m.Zeff = c.Zeff.data();
    m.alpha = c.alpha.data();
    m.nion = (int)c.Rion.size();
    m.Rion = c.Rion.data();
    m.Kion = c.Kion.data();
    check(nullptr, mattohf_create(&m, &h), "mattohf_create");
  }
  ~Context() { mattohf_destroy(h); }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
};

struct Obs {
  double Ecomps[4], Etot, Je, Nele;
};

Obs observables(mattohf_ctx* h, double A) {
  Obs o;
  check(h, mattohf_observables(h, A, o.Ecomps, &o.Etot, &o.Je, &o.Nele), "mattohf_observables");
  return o;
}

std::vector<double> density_of_state(mattohf_ctx* h, const Config& c) {
  std::vector<double> u((size_t)c.NK * c.NB * c.NG * 2), d(c.NG);
  check(h, mattohf_get_orbitals(h, u.data()), "mattohf_get_orbitals");
  check(h, mattohf_density(h, u.data(), d.data(), nullptr), "mattohf_density");
  return d;
}

// FourierTr (RT:246-303, polynomial filter) or WindowFourierTr (RT:305-351).
std::vector<double> fourier(const Config& c, const std::vector<double>& t, const std::vector<double>& J, double J0,
                            const std::vector<double>& E, const std::vector<double>& A, bool window) {
  const int nt = (int)t.size();
  std::vector<double> filt(nt, 0.0);
  if (window) {
    const double Tp = c.Tpulse / kAtomtime;
    const int ntp = (int)std::min(Tp / c.dt, (double)nt);
    for (int it = 0; it < ntp; ++it) filt[it] = powi(std::sin(kPi * t[it] / Tp), c.nenvelope);
  } else {
    for (int it = 0; it < nt; ++it) {
      const double tn = t[nt - 1] != 0.0 ? t[it] / t[nt - 1] : 0.0;
      filt[it] = 1.0 - 3.0 * (tn * tn) + 2.0 * std::pow(tn, 3.0);
    }
  }
  std::vector<double> out((size_t)c.Nomega * 7);
  check(nullptr,
        mattohf_fourier(0, nt, t.data(), J.data(), J0, E.data(), A.data(), filt.data(), c.Nomega, c.omegaM, c.dt,
                        out.data()),
        "mattohf_fourier");
  return out;
}

std::ofstream open_out(const std::string& dir, const std::string& name) {
  std::ofstream f(dir + "/" + name);
  if (!f) throw Failure("cannot write " + dir + "/" + name);
  return f;
}

double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

int run(const Config& c, const std::string& dir) {
  const int NG = c.NG, NK = c.NK, NB = c.NB, NBocc = c.NBocc;
  const std::string sysn = trim(c.sys_name);
  Context ctx(c);
  mattohf_ctx* h = ctx.h;
  std::vector<double> rx(NG), Gx(NG), kx(NK), cell(3), vion(NG);
  check(h, mattohf_get_grids(h, rx.data(), Gx.data(), kx.data(), cell.data()), "mattohf_get_grids");
  check(h, mattohf_get_vion(h, vion.data()), "mattohf_get_vion");
  {
    std::ofstream f = open_out(dir, "potential.out");
    for (int ig = 0; ig < NG; ++ig) f << " " << rjust(repr(rx[ig]), 24) << " " << rjust(repr(vion[ig]), 24) << "\n";
  }
  {
    std::vector<double> q((size_t)NG * NK), vk((size_t)NG * NK);
    for (int ig = 0; ig < NG; ++ig)
      for (int ik = 0; ik < NK; ++ik) q[(size_t)ig * NK + ik] = Gx[ig] + kx[ik];  // I:149-155
    check(h, mattohf_vck(h, q.data(), NG * NK, vk.data()), "mattohf_vck");
    std::ofstream f = open_out(dir, "vk.out");
    for (size_t i = 0; i < q.size(); ++i) f << " " << rjust(repr(q[i]), 24) << " " << rjust(repr(vk[i]), 24) << "\n";
  }
  check(h, mattohf_init_wf(h), "mattohf_init_wf");
  check(h, mattohf_gram_schmidt(h), "mattohf_gram_schmidt");
  const Obs e0 = observables(h, 0.0);
  std::cout << " Number of particle per cell " << repr(e0.Nele) << "\n";
  std::cout << " Total energy at initial = " << repr(e0.Etot) << "\n";

  // ---- ground state (GS:26-121)
  const auto t_gs0 = std::chrono::steady_clock::now();
  std::vector<double> dprev = density_of_state(h, c);
  double Et_prev = e0.Etot;
  // the format literal continues on the next source line with its leading blanks (GS:23-24)
  std::vector<std::string> lines{
      "#iter, Etotscf(iter), Etoscf(iter)-Etotscf(iter-1), ,sum(abs(dnsscf(:,iter+1)-dnsscf(:,iter)))/dble(NG) "
      "         sum(epserrorbk)/dble(NB*NK),maxval(epserrorbk),Fundamental gap, Optical Gap"};
  std::vector<double> eps((size_t)NK * NB), err((size_t)NK * NB);
  bool have_eps = false;
  for (int it = 1; it <= c.Nscf; ++it) {
    double Eit[2], Je;
    check(h, mattohf_gs_run(h, 1, c.NCG, Eit, &Je, nullptr, eps.data(), err.data()), "mattohf_gs_run");
    have_eps = true;
    const double Et = Eit[1];
    std::vector<double> dcur = density_of_state(h, c);
    double dd = 0.0;
    for (int ig = 0; ig < NG; ++ig) {
      const double dnew = 0.5 * dcur[ig] + 0.5 * dprev[ig];
      dd += std::fabs(dnew - dprev[ig]);
      dprev[ig] = dnew;
    }
    dd /= NG;
    double esum = 0.0, emax = -INFINITY;
    for (double x : err) {
      esum += x;
      emax = std::max(emax, x);
    }
    std::vector<double> vals{Et, Et - Et_prev, dd, esum / (NB * NK), emax};
    for (double g : gap_columns(eps, NK, NB, NBocc)) vals.push_back(g);
    char ib[16];
    std::snprintf(ib, sizeof ib, "%5d", it);
    lines.push_back(std::string("  ") + ib + row(vals));
    char lg[160];
    std::snprintf(lg, sizeof lg, "iter, Etotscf(iter), JeGS =%4d%14.8f%12.4E  %12.4E", it, Et, Et - Et_prev, Je);
    std::cout << lg << "\n";
    Et_prev = Et;
  }
  const Obs ec = observables(h, 0.0);
  const char* labs[4] = {"Ekin ", "Eion ", "EH   ", "Exc  "};
  for (int i = 0; i < 4; ++i) lines.push_back(std::string("#") + labs[i] + " at SCF:" + fixed(ec.Ecomps[i], 12, 8));
  if (have_eps) {
    // GS:75-90; the conduction-bottom line prints maxval of the conduction
    // bands, as the reference does
    const double mn = *std::min_element(eps.begin(), eps.end()), mx = *std::max_element(eps.begin(), eps.end());
    double vtop = -kHuge, cmax = -kHuge;
    for (int ik = 0; ik < NK; ++ik)
      for (int ib = 0; ib < NB; ++ib) {
        const double x = eps[(size_t)ik * NB + ib];
        if (ib < NBocc) vtop = std::max(vtop, x);
        else cmax = std::max(cmax, x);
      }
    const std::vector<double> gp = gap_columns(eps, NK, NB, NBocc);
    const std::pair<const char*, double> rows[] = {
        {"#Min. value of the spectra: minval(epsbk)    =", mn},
        {"#Max. value of the spectra: maxval(epsbk)    =", mx},
        {"#Valence top: maxval(epsbk(:NBocc,:))        =", vtop},
        {"#Conduction bottom: minval(epsbk(NBocc+1:,:))=", cmax},
        {"#Fundamental gap: ", gp[0]},
        {"#Min. gap among same k-point: ", gp[1]}};
    for (const auto& r : rows)
      lines.push_back(std::string(r.first) + fixed(r.second, 12, 8) + " =" + fixed(r.second * kHartree, 12, 8) +
                      " [eV]");
  }
  {
    std::ofstream f = open_out(dir, sysn + "_GSinfo.out");
    for (const auto& l : lines) f << l << "\n";
  }
  if (have_eps) {
    // Make_DoS (GS:239-265) on the reference's energy mesh (GS:93-97)
    const int n = 10000;
    const double lo = *std::min_element(eps.begin(), eps.end()), hi = *std::max_element(eps.begin(), eps.end());
    const double emin = lo - 0.1 * (hi - lo), emax = hi + 0.1 * (hi - lo);
    std::vector<double> e(n), dos(n, 0.0), docc(n, 0.0);
    for (int i = 0; i < n; ++i) e[i] = emin + (emax - emin) * (double)i / (double)n;
    const double width = 5.0 * (e[1] - e[0]);
    for (int ik = 0; ik < NK; ++ik) {
      const double occmax = 2.0 / NK;  // occbk(1,ik): band 1 is always occupied
      for (int ib = 0; ib < NB; ++ib) {
        const double occ = ib < NBocc ? 2.0 / NK : 0.0;
        const double ev = eps[(size_t)ik * NB + ib];
        for (int i = 0; i < n; ++i) {
          const double df = ev - e[i];
          const double val = std::exp(-(df * df) / (width * width));
          dos[i] += occmax * val;
          docc[i] += occ * val;
        }
      }
    }
    const double norm = width * std::sqrt(kPi);
    std::string head = " # ik,kx(ik),  sum(epserrorbk(:,ik))/dble(NB),  epsbk(:,ik)\n";
    std::ofstream fd = open_out(dir, sysn + "_DoS.out"), fb = open_out(dir, sysn + "_band.out");
    fd << head;
    fb << head;
    for (int ik = 0; ik < NK; ++ik) {
      double es = 0.0;
      for (int ib = 0; ib < NB; ++ib) es += err[(size_t)ik * NB + ib];
      std::vector<double> ek(eps.begin() + (size_t)ik * NB, eps.begin() + (size_t)(ik + 1) * NB);
      const std::string rec = band_record(ik + 1, kx[ik], es / NB, ek);
      fd << "# " << rec << "\n";
      fb << rec << "\n";
    }
    for (int i = 0; i < n; ++i) fd << row({e[i], dos[i] / norm, docc[i] / norm}, 20, 12, 3) << "\n";
  }
  const double t_gs = seconds_since(t_gs0);

  // ---- real time (RT:2-69)
  const auto t_rt0 = std::chrono::steady_clock::now();
  std::vector<double> time, A, Aave, E;
  define_afield(c, time, A, Aave, E);
  const Obs ini = observables(h, 0.0);
  const int NT = c.NT;
  std::vector<double> Et(NT), Je(NT), Ne(NT);
  const int chunk = 1000;
  for (int s0 = 0; s0 < NT; s0 += chunk) {
    const int s1 = std::min(NT, s0 + chunk);
    check(h, mattohf_rk4_run(h, s1 - s0, c.dt, A.data() + s0, Aave.data() + s0, Et.data() + s0, Je.data() + s0,
                             Ne.data() + s0),
          "mattohf_rk4_run");
    char lg[128];
    std::snprintf(lg, sizeof lg, "%6d %14.6E%14.6E%14.6E", s1, time[s1 - 1], Et[s1 - 1], Et[s1 - 1] - ini.Etot);
    std::cout << lg << "\n";
  }
  {
    std::ofstream f = open_out(dir, sysn + "_EtotNJEAt.out");
    f << "#time(it), Etot(it)-Etot0, N(it)-N0, J(it), E(it), A(it)\n";
    for (int it = 0; it < NT; ++it)
      f << row({time[it], Et[it], Et[it] - ini.Etot, Ne[it], Ne[it] - ini.Nele, Je[it], E[it], A[it]}) << "\n";
  }
  {
    // extension (no reference counterpart): dipole P = -int J dt, trapezoid from J(0)
    std::ofstream f = open_out(dir, sysn + "_dipole.out");
    f << "#time(it), P(it)\n";
    double acc = 0.0, prev = ini.Je;
    for (int it = 0; it < NT; ++it) {
      acc -= 0.5 * c.dt * (prev + Je[it]);
      prev = Je[it];
      f << row({time[it], acc}) << "\n";
    }
  }
  const double t_rt = seconds_since(t_rt0);

  // ---- spectra (RT:64-65)
  if (NT > 0) {
    const std::vector<double> ft = fourier(c, time, Je, ini.Je, E, A, false);
    {
      std::ofstream f = open_out(dir, sysn + "_JEAF.out");
      f << "#omega(iomega), JF(iomega), EF(iomega), AF(iomega)\n";
      for (int i = 0; i < c.Nomega; ++i) f << row(std::vector<double>(ft.begin() + i * 7, ft.begin() + i * 7 + 7)) << "\n";
    }
    if (c.field_option == "LR") {
      std::ofstream f = open_out(dir, sysn + "_sigmaeps.out");
      f << "#omega(iomega), sigma(iomega), eps(iomega)\n";
      for (int i = 0; i < c.Nomega; ++i) {
        const double w = ft[i * 7], sr = -ft[i * 7 + 1] / c.dAc, si = -ft[i * 7 + 2] / c.dAc;
        const double ar = 0.0, ai = 4.0 * kPi;  // 4 pi i sigma / omega
        const double er = (ar * sr - ai * si) / w, ei = (ar * si + ai * sr) / w;
        f << row({w, sr, si, er, ei}) << "\n";
      }
    } else {
      const std::vector<double> fw = fourier(c, time, Je, ini.Je, E, A, true);
      std::ofstream f = open_out(dir, sysn + "_JEAF_window.out");
      f << "#omega(iomega), JF(iomega), EF(iomega), AF(iomega)\n";
      for (int i = 0; i < c.Nomega; ++i) f << row(std::vector<double>(fw.begin() + i * 7, fw.begin() + i * 7 + 7)) << "\n";
    }
  }
  char lg[128];
  std::snprintf(lg, sizeof lg, "Time for GS calculatoin =%12.4E [sec]", t_gs);
  std::cout << lg << "\n";
  std::snprintf(lg, sizeof lg, "Time for RT calculatoin =%12.4E [sec]", t_rt);
  std::cout << lg << "\n";
  std::snprintf(lg, sizeof lg, "Time for an interaction in RT =%12.4E [sec]", t_rt / std::max(NT, 1));
  std::cout << lg << "\n";
  double e2 = 0.0;
  for (double x : E) e2 += x * x;
  std::cout << "Fluence of the field: " << repr(e2 * c.dt * kAtomfluence) << " J/cm^2\n";
  return 0;
}

// The input-file name: the first list-directed item of standard input (M:45).
std::string read_name() {
  std::string line;
  if (!std::getline(std::cin, line)) return "";
  bool blank = false;
  return first_token(line, &blank);
}

}  // namespace

int main(int argc, char** argv) {
  const std::string dir = argc > 1 ? argv[1] : ".";
  try {
    const std::string name = read_name();
    const Config c = name.empty() ? Config() : read_input(name);
    return run(c, dir);
  } catch (const std::exception& e) {
    std::cerr << "mattohf: " << e.what() << "\n";
    return 1;
  }
}
