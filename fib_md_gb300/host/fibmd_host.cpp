// fibmd_host.cpp — host-side set-up of a FIB_MD run (not on the GPU path).
//
// C++ restatement of the reference's Fortran initialisation so a driver
// without a Fortran compiler can prepare the same state the reference
// prepares: siga.in (src/prms.f90:221-275), pureepi (src/prms.f90:484-557),
// initranions / initIons / assignmass / randvel (src/data.f90:169-285),
// knock (src/knock.f90:21-55) and ran1 (src/ran1.f, Park & Miller's minimal
// standard generator with Schrage's factorisation and a Bays-Durham shuffle
// table of 32). Compiled with -ffp-contract=off; expressions keep Fortran's
// left-to-right evaluation.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/fibmd_host.h"

namespace {

double through_text(double x, int sig) {
  // an Ew.d field written by Fortran and read back list-directed
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.*E", sig - 1, x);
  return std::strtod(buf, nullptr);
}

// Tokens of list-directed input: separated by blanks or commas; everything
// after a backslash on a line is commentary.
struct ListReader {
  std::ifstream in;
  std::vector<std::string> tok;
  size_t pos = 0;
  int line = 0;
  bool next_record() {
    std::string s;
    if (!std::getline(in, s)) return false;
    line++;
    size_t bs = s.find('\\');
    if (bs != std::string::npos) s = s.substr(0, bs);
    for (char& c : s)
      if (c == ',') c = ' ';
    std::istringstream is(s);
    tok.clear();
    pos = 0;
    std::string t;
    while (is >> t) tok.push_back(t);
    return true;
  }
  // One READ statement: take n values, continuing onto later records when a
  // record runs out; the rest of the last record is skipped.
  bool read(std::vector<std::string>& out, int n) {
    out.clear();
    if (!next_record()) return false;
    while ((int)out.size() < n) {
      if (pos < tok.size()) {
        out.push_back(tok[pos++]);
      } else if (!next_record()) {
        return false;
      }
    }
    return true;
  }
};

bool to_int(const std::string& s, int* v) {
  char* e = nullptr;
  long x = std::strtol(s.c_str(), &e, 10);
  if (!e || *e) return false;
  *v = (int)x;
  return true;
}

bool to_real(const std::string& s, double* v) {
  std::string t = s;
  for (char& c : t)
    if (c == 'd' || c == 'D') c = 'E';
  char* e = nullptr;
  *v = std::strtod(t.c_str(), &e);
  return e && !*e;
}

}  // namespace

extern "C" {

void fibmd_host_rng_seed(fibmd_rng* r, int seed) {
  std::memset(r, 0, sizeof(*r));
  r->idum = seed;
}

double fibmd_host_ran1(fibmd_rng* r) {
  const int IA = 16807, IM = 2147483647, IQ = 127773, IR = 2836, NTAB = 32;
  const int NDIV = 1 + (IM - 1) / NTAB;
  const double AM = 1. / IM, EPS = 1.2e-7, RNMX = 1. - EPS;
  if (r->idum <= 0 || r->iy == 0) {
    r->idum = (-r->idum > 1) ? -r->idum : 1;
    for (int j = NTAB + 8; j >= 1; j--) {
      const int k = r->idum / IQ;
      r->idum = IA * (r->idum - k * IQ) - IR * k;
      if (r->idum < 0) r->idum += IM;
      if (j <= NTAB) r->iv[j - 1] = r->idum;
    }
    r->iy = r->iv[0];
  }
  const int k = r->idum / IQ;
  r->idum = IA * (r->idum - k * IQ) - IR * k;
  if (r->idum < 0) r->idum += IM;
  const int j = 1 + r->iy / NDIV;
  r->iy = r->iv[j - 1];
  r->iv[j - 1] = r->idum;
  const double v = AM * r->iy;
  return v < RNMX ? v : RNMX;
}

int fibmd_host_read_siga(const char* path, fibmd_params* p, fibmd_siga* s, char* msg,
                         int msglen) {
  ListReader R;
  R.in.open(path);
  auto err = [&](const char* what) {
    if (msg && msglen > 0)
      std::snprintf(msg, (size_t)msglen, "%s: cannot read %s (line %d)", path, what, R.line);
    return FIBMD_EINVAL;
  };
  if (!R.in) return err("file");
  std::vector<std::string> v;
  std::memset(s, 0, sizeof(*s));
#define RI(dst, name) \
  if (!R.read(v, 1) || !to_int(v[0], &(dst))) return err(name)
#define RR(dst, name) \
  if (!R.read(v, 1) || !to_real(v[0], &(dst))) return err(name)
  RI(s->amorcrys, "amorcrys");
  RI(s->whichic, "whichic");
  RI(s->startimpact, "startimpact");
  RR(s->eV, "eV");
  if (!R.read(v, 3) || !to_int(v[0], &s->Nc[0]) || !to_int(v[1], &s->Nc[1]) ||
      !to_int(v[2], &s->Nc[2]))
    return err("Nc1,Nc2,Nc3");
  if (!R.read(v, 3) || !to_int(v[0], &s->Npc[0]) || !to_int(v[1], &s->Npc[1]) ||
      !to_int(v[2], &s->Npc[2]))
    return err("Npc");
  RI(p->Nlj, "Nlj");
  RI(s->Nt, "Nt");
  RR(p->Ts_i, "Ts_i");
  RR(p->Ts_r, "Ts_r");
  RR(p->Ttar1, "Ttar1");
  RR(p->ke_limit_1, "ke_limit_1");
  RR(s->ke_limit_2, "ke_limit_2");
  RR(p->Tau_i, "Tau_i");
  RR(p->Tau_r, "Tau_r");
  RR(p->Teps, "Teps");
  RR(s->Uo, "Uo");
  RI(p->ntlist_i, "ntlist_i");
  RI(p->ntlist_r, "ntlist_r");
  RI(p->atlist_i, "atlist_i");
  RI(p->atlist_r, "atlist_r");
  RI(p->dslist_i, "dslist_i");
  RI(p->dslist_r, "dslist_r");
  RI(p->atm_out_i, "atm_out_i");
  RI(p->atm_out_r, "atm_out_r");
  RI(p->res_out, "res_out");
  RI(s->eng_out, "eng_out");
  RI(s->tmp_out, "tmp_out");
  RI(s->Nrand, "Nrand");
  for (int k = 0; k < 4; k++) RR(p->outz[k], "outz");
  RR(p->atomz[0], "atomz(1)");
  RR(p->atomz[1], "atomz(2)");
  RR(p->ionz, "ionz");
  RR(p->knockz, "knockz");
  RR(p->sidewidth, "sidewidth");
  RR(p->dti, "dti");
  RR(s->fwhm, "fwhm");
  RR(s->phiz, "phiz");
  RR(s->phixy, "phixy");
#undef RI
#undef RR
  if (s->amorcrys == 0) {
    // pureepi's box and counts (prms.f90:494, 536-541)
    const double L = 5.431073E-10;
    p->Lb[0] = L * s->Nc[0];
    p->Lb[1] = L * s->Nc[1];
    p->Lb[2] = L * s->Nc[2] * 10;
    p->Nsg = 8 * s->Nc[0] * s->Nc[1] * s->Nc[2];
    p->Natm = p->Nsg + p->Nlj;
  }
  return FIBMD_OK;
}

int fibmd_host_pureepi(int Nc1, int Nc2, int Nc3, double* XX, int* xsides, double Lb[3]) {
  const double L[3] = {5.431073E-10, 5.431073E-10, 5.431073E-10};
  const double uc[8][3] = {{0.00, 0.00, 0.00},
                           {0.00, 0.50 * L[1], 0.50 * L[2]},
                           {0.250 * L[0], 0.250 * L[1], 0.750 * L[2]},
                           {0.250 * L[0], 0.750 * L[1], 0.250 * L[2]},
                           {0.50 * L[0], 0.0 * L[1], 0.50 * L[2]},
                           {0.50 * L[0], 0.50 * L[1], 0.0 * L[2]},
                           {0.750 * L[0], 0.250 * L[1], 0.250 * L[2]},
                           {0.750 * L[0], 0.750 * L[1], 0.750 * L[2]}};
  const int n = 8 * Nc1 * Nc2 * Nc3;
  std::vector<double> raw(3 * (size_t)n);
  int m = 0;
  for (int i = 1; i <= Nc1; i++)
    for (int j = 1; j <= Nc2; j++)
      for (int k = 1; k <= Nc3; k++)
        for (int l = 0; l < 8; l++) {
          raw[m] = uc[l][0] + L[0] * (double)(i - 1);
          raw[(size_t)n + m] = uc[l][1] + L[1] * (double)(j - 1);
          raw[2 * (size_t)n + m] = uc[l][2] + L[2] * (double)(k - 1);
          m++;
        }
  double maxx = -1e300, maxy = -1e300;
  for (int i = 0; i < n; i++) {
    if (raw[i] > maxx) maxx = raw[i];
    if (raw[(size_t)n + i] > maxy) maxy = raw[(size_t)n + i];
  }
  for (int i = 0; i < n; i++) {
    const double x = raw[i], y = raw[(size_t)n + i];
    if (xsides)
      xsides[i] = (x < 1.0e-10 || y < 1.0e-10 || x > maxx - 1.0e-10 || y > maxy - 1.0e-10)
                      ? i + 1
                      : 0;
    for (int d = 0; d < 3; d++)
      XX[(size_t)d * n + i] = through_text(raw[(size_t)d * n + i], 10);
  }
  if (Lb) {
    Lb[0] = L[0] * Nc1;
    Lb[1] = L[1] * Nc2;
    Lb[2] = L[2] * Nc3 * 10;
  }
  return n;
}

void fibmd_host_initranions(fibmd_rng* r, int Nrand, double fwhm, double* Xrand) {
  const double Pi = 4. * std::atan(1.0);
  for (int i = 0; i < Nrand; i++) {
    const double r1 = fibmd_host_ran1(r);
    const double r2 = fibmd_host_ran1(r);
    const double a = std::sqrt(-2 * std::log(r1)) * std::cos(2 * Pi * r2) * fwhm / 2.35 * 1.E-9;
    const double b = std::sqrt(-2 * std::log(r2)) * std::sin(2 * Pi * r1) * fwhm / 2.35 * 1.E-9;
    Xrand[i] = through_text(a, 6);
    Xrand[(size_t)Nrand + i] = through_text(b, 6);
  }
}

int fibmd_host_init_state(const fibmd_params* p, fibmd_rng* r, double Uo, double* X,
                          double* Xi, double* V, double* mass, int* atype) {
  const int N = p->Natm, Nsg = p->Nsg;
  if (N <= 0 || Nsg < 0 || Nsg > N) return FIBMD_EINVAL;
  auto x = [&](int i, int d) -> double& { return X[(size_t)d * N + i - 1]; };
  auto v = [&](int i, int d) -> double& { return V[(size_t)d * N + i - 1]; };
  for (int i = 1; i <= Nsg; i++) atype[i - 1] = 1;
  // initIons, data.f90:223-260
  for (int i = Nsg + 1; i <= N; i++) {
    x(i, 0) = p->Lb[0] * fibmd_host_ran1(r);
    x(i, 1) = p->Lb[1] * fibmd_host_ran1(r);
    x(i, 2) = p->ionz * p->Lb[2] / 10.0;
    atype[i - 1] = 3;
  }
  for (int i = Nsg + 1; i <= N; i++)
    for (int j = Nsg + 1; j <= N; j++)
      if (i > j) {
        for (;;) {
          const double a = x(i, 0) - x(j, 0), b = x(i, 1) - x(j, 1);
          if (std::sqrt(a * a + b * b) < p->sigmaSi) {
            x(i, 0) = p->Lb[0] * fibmd_host_ran1(r);
            x(i, 1) = p->Lb[1] * fibmd_host_ran1(r);
            continue;
          }
          break;
        }
      }
  std::memcpy(Xi, X, sizeof(double) * 3 * (size_t)N);
  // assignmass, data.f90:207-220
  for (int i = 0; i < N; i++)
    mass[i] = atype[i] == 1 ? p->massSi : atype[i] == 2 ? p->massGe : p->massGa;
  // randvel, data.f90:169-204
  double mm[3] = {0.0, 0.0, 0.0};
  for (int i = 1; i <= Nsg; i++) {
    v(i, 0) = Uo * (fibmd_host_ran1(r) - 0.5);
    v(i, 1) = Uo * (fibmd_host_ran1(r) - 0.5);
    v(i, 2) = Uo * (fibmd_host_ran1(r) - 0.5);
    for (int d = 0; d < 3; d++) mm[d] = mm[d] + mass[i - 1] * v(i, d);
  }
  for (int d = 0; d < 3; d++) mm[d] = mm[d] / Nsg;
  for (int i = 1; i <= Nsg; i++)
    for (int d = 0; d < 3; d++) v(i, d) = v(i, d) - mm[d] / mass[i - 1];
  for (int i = Nsg + 1; i <= N; i++)
    for (int d = 0; d < 3; d++) v(i, d) = 0.0;
  return FIBMD_OK;
}

void fibmd_host_maxwell(fibmd_rng* r, int n, int N, const double* mass, double T, double kB,
                        double* V) {
  // Box-Muller (Box and Muller, 1958) on consecutive ran1 pairs, the method
  // initranions uses for its impact table (data.f90:263-285)
  const double Pi = 4. * std::atan(1.0);
  const long long nv = 3 * (long long)n;
  for (long long m = 0; m < nv; m += 2) {
    const double u1 = fibmd_host_ran1(r);
    const double u2 = fibmd_host_ran1(r);
    const double rad = std::sqrt(-2. * std::log(u1));
    const double z[2] = {rad * std::cos(2. * Pi * u2), rad * std::sin(2. * Pi * u2)};
    for (int q = 0; q < 2 && m + q < nv; q++) {
      const long long e = m + q;
      const int i = (int)(e / 3), d = (int)(e % 3);
      V[(size_t)d * (size_t)N + (size_t)i] = z[q] * std::sqrt(kB * T / mass[i]);
    }
  }
  double P[3] = {0.0, 0.0, 0.0}, M = 0.0;
  for (int i = 0; i < n; i++) {
    M = M + mass[i];
    for (int d = 0; d < 3; d++) P[d] = P[d] + mass[i] * V[(size_t)d * (size_t)N + (size_t)i];
  }
  for (int i = 0; i < n; i++)
    for (int d = 0; d < 3; d++)
      V[(size_t)d * (size_t)N + (size_t)i] = V[(size_t)d * (size_t)N + (size_t)i] - P[d] / M;
}

int fibmd_host_knock(const fibmd_params* p, fibmd_rng* r, int knc, double eV, double phiz,
                     double phixy, const double* Xrand, int Nrand, double x[3], double v[3]) {
  const double Pi = 4. * std::atan(1.0);
  const double L3 = p->Lb[2];
  const double kv = 1663.6334 * std::sqrt(eV);
  const double dr = std::tan(phiz * Pi / 180) * (p->knockz * L3 / 10 - L3 / 10);
  const double dx = dr * std::cos(phixy * Pi / 180) * std::sin(phiz * Pi / 180);
  const double dy = dr * std::sin(phixy * Pi / 180) * std::sin(phiz * Pi / 180);
  int ri = (int)std::lround(fibmd_host_ran1(r) * Nrand);
  if (ri < 1) ri = 1;
  v[0] = kv * std::cos(phixy * Pi / 180) * std::sin(phiz * Pi / 180);
  v[1] = kv * std::sin(phixy * Pi / 180) * std::sin(phiz * Pi / 180);
  v[2] = -1.0 * kv * std::cos(phiz * Pi / 180);
  x[0] = Xrand[ri - 1] + p->Lb[0] / 2.0 - dx;
  x[1] = Xrand[(size_t)Nrand + ri - 1] + p->Lb[1] / 2.0 - dy;
  x[2] = p->knockz * L3 / 10.0;
  return p->Nsg + knc;
}

}  // extern "C"
