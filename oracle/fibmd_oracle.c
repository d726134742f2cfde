/*
 * fibmd_oracle.c — binary64 CPU restatement of the FIB_MD hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see fibmd_oracle.h): the checker for the GPU
 * library and the timed CPU baseline. Parity with the reference's own outputs
 * is unpinned (no Fortran compiler, no reference fixtures); the restatement
 * is pinned by known answers of the reference's formulas in tests/.
 *
 * Each function cites the reference routine it restates (paths relative to
 * the reference project). Expressions keep Fortran's left-to-right order; the
 * file must be compiled with -ffp-contract=off.
 */
#include "fibmd_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define CM(a, N, i, d) (a)[(size_t)(d) * (size_t)(N) + (size_t)(i) - 1]
#define NSS1(s, i) (s)->nss[(i) - 1]
#define NSS2(s, i) (s)->nss[(size_t)(s)->Natm + (i) - 1]
#define NSSLJ1(s, i) (s)->nsslj[(i) - 1]
#define NSSLJ2(s, i) (s)->nsslj[(size_t)(s)->Natm + (i) - 1]

/* Fortran NINT: nearest integer, halves away from zero. */
static inline double f_nint(double x) { return (double)lround(x); }
/* Fortran INT of a real: truncation toward zero. */
static inline int f_int(double x) { return (int)x; }

/* prms.f90:172-216 constants and the reference's shipped siga.in. */
void orc_params_default(fibmd_params* p) {
  memset(p, 0, sizeof(*p));
  p->abi_version = FIBMD_ABI_VERSION;
  p->mode = FIBMD_MODE_REF;
  p->precision = FIBMD_PREC_FP64;
  p->A = 7.049556277;
  p->B = 0.6022245584;
  p->psi = 4.0;
  p->qsi = 0.0;
  p->al = 1.8;
  p->gamma = 1.2;
  p->lambdaSi = 21.0;
  p->lambdaGe = 31.0;
  p->epsSi = 3.473928E-19;
  p->epsGe = 3.085E-19;
  p->sigmaSi = 2.0951E-10;
  p->sigmaGe = 2.0951E-10;
  p->massSi = 46.637063E-27;
  p->massGe = 120.6049350E-27;
  p->massGa = 1.157777417E-25;
  p->ZSi = 14.0;
  p->ZGe = 32.0;
  p->ZGa = 31.0;
  p->Amol = 0.35;
  p->Bmol = 0.55;
  p->Cmol = 0.10;
  p->alpha_mol = 0.3;
  p->beta_mol = 1.2;
  p->gamma_mol = 6.0;
  p->kB = 1.381E-23;
  p->eps0 = 8.854187E-12;
  p->ec = 1.60217646E-19;
  p->ao = 0.053E-09;
  p->listfac = 1.1;
  p->Ntable = 12000;
  /* siga.in as shipped */
  p->Ts_i = 2.0E-17;
  p->Ts_r = 2.0E-16;
  p->Ttar1 = 300.0;
  p->ke_limit_1 = 600.0;
  p->Tau_i = 1.E-13;
  p->Tau_r = 1.E-13;
  p->Teps = 30.0;
  p->ntlist_i = 50;
  p->ntlist_r = 20;
  p->atlist_i = 50;
  p->atlist_r = 20;
  p->dslist_i = 500;
  p->dslist_r = 500;
  p->atm_out_i = 50;
  p->atm_out_r = 500;
  p->res_out = -5000;
  p->outz[0] = 1.3;
  p->outz[1] = 3.5;
  p->outz[2] = 7.5;
  p->outz[3] = 9.8;
  p->atomz[0] = 4.5;
  p->atomz[1] = 6.5;
  p->ionz = 5.5;
  p->knockz = 1.25;
  p->sidewidth = 1.5;
  p->dti = 1e-12;
  p->dt_max = 1.0e-15;
  p->dx_max = 0.05e-10;
  p->tau_spec = 1.0e-13;
  p->remove_z = -1.0;
  p->mixed_mol_fp64_r = 1.0e-10;
  p->list_skin = 0.0;
}

/* ---- set-up: setupSiGe / setupMol (prms.f90:433-480), init_nlist
        (si.f90:48-80), mktables (si.f90:575-597) ------------------------- */
static void mktables(orc_sys* s) {
  const fibmd_params* p = &s->p;
  int Nt = p->Ntable;
  s->table2bd = (double*)calloc((size_t)Nt + 2, sizeof(double));
  s->u = (double*)calloc((size_t)Nt + 2, sizeof(double));
  s->umax = 2.5 * p->listfac * p->al;
  double du = s->umax / (double)(Nt - 1);
  for (int i = 2; i <= Nt; i++) {
    double ui = s->umax * (double)(i - 1) / (double)(Nt - 1);
    s->u[i - 1] = ui;
    if (ui < .999 * p->al) {
      double ex = exp(1. / (ui - p->al));
      double y = (p->B * pow(ui, -p->psi) - pow(ui, -p->qsi)) /
                     ((ui - p->al) * (ui - p->al)) +
                 (p->psi * p->B * pow(ui, -p->psi - 1) -
                  p->qsi * pow(ui, -p->qsi - 1));
      s->table2bd[i - 1] = -(p->A * ex * y / (du * du));
    } else {
      s->table2bd[i - 1] = 0.;
    }
  }
  /* u(1)/table2bd(1) are left unset by the reference; they are only read
     for ue < umax/(Ntable-1), which a listed pair never reaches. */
}

int orc_init(orc_sys* s, const fibmd_params* p) {
  memset(s, 0, sizeof(*s));
  s->p = *p;
  s->Natm = p->Natm;
  s->Nsg = p->Nsg;
  s->Nlj = p->Nlj;
  for (int d = 0; d < 3; d++) {
    s->Lb[d] = p->Lb[d];
    s->iLb[d] = 1. / p->Lb[d];
  }
  s->Pi = 4. * atan(1.0);
  s->thrd = 1. / 3.;
  /* setupSiGe, prms.f90:452-480 (index 0 = Si, 1 = Ge) */
  s->eps[0][0] = p->epsSi;
  s->eps[0][1] = 0.5 * (p->epsSi + p->epsGe);
  s->eps[1][1] = p->epsGe;
  s->eps[1][0] = 0.5 * (p->epsSi + p->epsGe);
  s->isigma[0][0] = 1. / p->sigmaSi;
  s->isigma[0][1] = 2. / (p->sigmaSi + p->sigmaGe);
  s->isigma[1][1] = 1. / p->sigmaGe;
  s->isigma[1][0] = 2. / (p->sigmaSi + p->sigmaGe);
  double lS = p->lambdaSi * p->epsSi, lG = p->lambdaGe * p->epsGe;
  s->leps[0][0][0] = lS;
  s->leps[0][0][1] = 2. * p->lambdaSi * p->epsSi / 3. + p->lambdaGe * p->epsGe / 3.;
  s->leps[0][1][0] = s->leps[0][0][1];
  s->leps[1][0][0] = s->leps[0][0][1];
  s->leps[0][1][1] = p->lambdaSi * p->epsSi / 3. + 2. * p->lambdaGe * p->epsGe / 3.;
  s->leps[1][1][0] = s->leps[0][1][1];
  s->leps[1][0][1] = s->leps[0][1][1];
  s->leps[1][1][1] = lG;
  (void)lS;
  s->epssig[0][0] = p->epsSi / p->sigmaSi;
  s->epssig[0][1] = (p->epsSi + p->epsGe) / (p->sigmaSi + p->sigmaGe);
  s->epssig[1][0] = s->epssig[0][1];
  s->epssig[1][1] = p->epsGe / p->sigmaGe;
  /* setupMol, prms.f90:433-449 */
  s->Zmol[0] = p->ZSi;
  s->Zmol[1] = p->ZGe;
  s->Zmol[2] = p->ZGa;
  memset(s->aamol, 0, sizeof(s->aamol));
  s->aamol[0][2] = 0.885 * p->ao * pow(sqrt(p->ZSi) + sqrt(p->ZGa), -(2. / 3.));
  s->aamol[1][2] = 0.885 * p->ao * pow(sqrt(p->ZGe) + sqrt(p->ZGa), -(2. / 3.));
  s->aamol[2][0] = s->aamol[0][2];
  s->aamol[2][1] = s->aamol[1][2];
  s->aamol[2][2] = 0.885 * p->ao * pow(sqrt(p->ZGa) + sqrt(p->ZGa), -(2. / 3.));
  s->ie0 = 1 / (4 * s->Pi * p->eps0);

  /* init_nlist, si.f90:48-61 (Nl = Natm on one domain) */
  int Nl = s->Natm;
  s->ML3 = Nl * 200;
  s->MLlj = s->Nlj * 1500;
  s->ML2 = Nl * 40;
  double sigmax = p->sigmaGe > p->sigmaSi ? p->sigmaGe : p->sigmaSi;
  s->rc = p->listfac * p->al * sigmax;
  double rlj2 = 2.5 * sigmax;
  s->rclj = p->listfac * rlj2;
  s->rlj2 = rlj2 * rlj2;
  s->spec = p->mode == FIBMD_MODE_SPEC;
  if (s->spec && p->list_skin > 0.0) {
    /* spec mode: interaction cutoff + skin */
    s->rc = 0.999 * p->al * sigmax + p->list_skin;
    s->rclj = rlj2 + p->list_skin;
  }
  for (int d = 0; d < 3; d++) {
    int n = f_int(s->Lb[d] / s->rc);
    s->Nc[d] = n > 1 ? n : 1;
  }

  s->cap2 = s->ML2 > 64 ? s->ML2 : 64;
  s->cap3 = s->ML3 > 64 ? s->ML3 : 64;
  s->caplj = s->MLlj > 64 ? s->MLlj : 64;
  s->nss = (int*)calloc((size_t)Nl * 2, sizeof(int));
  s->nsslj = (int*)calloc((size_t)Nl * 2, sizeof(int));
  s->nlist2 = (int*)calloc((size_t)s->cap2 + 1, sizeof(int));
  s->nlistlj = (int*)calloc((size_t)s->caplj + 1, sizeof(int));
  s->nlist3 = (int*)calloc((size_t)s->cap3 * 3, sizeof(int));

  mktables(s);

  size_t N = (size_t)s->Natm;
  s->X = (double*)calloc(N * 3, sizeof(double));
  s->Xi = (double*)calloc(N * 3, sizeof(double));
  s->V = (double*)calloc(N * 3, sizeof(double));
  s->F = (double*)calloc(N * 3, sizeof(double));
  s->mass = (double*)calloc(N, sizeof(double));
  s->atype = (int*)calloc(N, sizeof(int));
  s->xsides = (int*)calloc(N, sizeof(int));
  if (s->spec) {
    s->tags = (unsigned*)calloc(N, sizeof(unsigned));
    s->Xb = (double*)calloc(N * 3, sizeof(double));
    /* the half skin, the smaller of the two lists' skins (1 % margin) */
    double skin = s->rc - 0.999 * p->al * sigmax;
    if (s->rclj - rlj2 < skin) skin = s->rclj - rlj2;
    double half = 0.5 * skin * 0.99;
    s->sp_trig2 = half * half;
    s->sp_rule = 1;
    s->sp_zopen = p->remove_z > 0.0 && p->remove_z + s->rc < s->Lb[2];
    s->sp_remove_zlo = s->sp_zopen ? -10.0e-10 : -1.0e300;
    s->sp_thermo_s = 1.0;
  }
  orc_ionrun(s, 1);
  s->impact = 0;
  s->atom_is_fast = 1;
  s->atom_is_slow = 0;
  return 0;
}

void orc_free(orc_sys* s) {
  free(s->nss);
  free(s->nsslj);
  free(s->nlist2);
  free(s->nlistlj);
  free(s->nlist3);
  free(s->table2bd);
  free(s->u);
  free(s->X);
  free(s->Xi);
  free(s->V);
  free(s->F);
  free(s->mass);
  free(s->atype);
  free(s->xsides);
  free(s->tags);
  free(s->Xb);
  memset(s, 0, sizeof(*s));
}

/* ---- chainlist / atomcell, nlist.f90:20-66 ------------------------------ */
static void chainlist(orc_sys* s, int* LL, int* HOC, const double* X) {
  int N = s->Natm;
  int n1 = s->Nc[0], n2 = s->Nc[1], n3 = s->Nc[2];
  int s1 = n1 + 2, s2 = n2 + 2, s3 = n3 + 2;
  double HMf[3];
  for (int d = 0; d < 3; d++) HMf[d] = s->Lb[d] / (double)s->Nc[d];
  memset(HOC, 0, sizeof(int) * (size_t)s1 * s2 * s3);
  for (int i = 1; i <= N; i++) {
    /* spec mode bins the lattice atoms still in the run; pairs with an ion
       are found by the ion scan of spec_moliere_pairs */
    if (s->spec && (s->atype[i - 1] >= 3 || (s->tags[i - 1] & FIBMD_TAG_REMOVED))) {
      LL[i - 1] = 0;
      continue;
    }
    int ic[3];
    for (int d = 0; d < 3; d++) {
      double x = CM(X, N, i, d);
      double fl = floor(x * s->iLb[d]);
      ic[d] = f_int((x - fl * s->Lb[d]) / HMf[d]) + 1;
    }
    if (ic[0] < 0 || ic[0] > n1 + 1 || ic[1] < 0 || ic[1] > n2 + 1 ||
        ic[2] < 0 || ic[2] > n3 + 1) {
      /* the reference would write outside HOC here */
      s->cell_oob++;
      LL[i - 1] = 0;
      continue;
    }
    if (ic[0] == 0 || ic[0] == n1 + 1 || ic[1] == 0 || ic[1] == n2 + 1 ||
        ic[2] == 0 || ic[2] == n3 + 1)
      s->cell_oob++; /* lands in a ghost layer, as the reference allows */
    size_t h = (size_t)ic[0] + (size_t)s1 * ((size_t)ic[1] + (size_t)s2 * ic[2]);
    LL[i - 1] = HOC[h];
    HOC[h] = i;
  }
#define HOCI(a, b, c) HOC[(size_t)(a) + (size_t)s1 * ((size_t)(b) + (size_t)s2 * (size_t)(c))]
  if (n1 > 2)
    for (int c = 0; c < s3; c++)
      for (int b = 0; b < s2; b++) {
        HOCI(0, b, c) = HOCI(n1, b, c);
        HOCI(n1 + 1, b, c) = HOCI(1, b, c);
      }
  if (n2 > 2)
    for (int c = 0; c < s3; c++)
      for (int a = 0; a < s1; a++) {
        HOCI(a, 0, c) = HOCI(a, n2, c);
        HOCI(a, n2 + 1, c) = HOCI(a, 1, c);
      }
  if (n3 > 2)
    for (int b = 0; b < s2; b++)
      for (int a = 0; a < s1; a++) {
        HOCI(a, b, 0) = HOCI(a, b, n3);
        HOCI(a, b, n3 + 1) = HOCI(a, b, 1);
      }
#undef HOCI
}

static void grow_int(int** a, int* cap, int need, int width) {
  if (need < *cap) return;
  int nc = *cap;
  while (nc <= need) nc = nc * 2 + 16;
  int* b = (int*)calloc((size_t)nc * width + 1, sizeof(int));
  if (width == 1) {
    memcpy(b, *a, sizeof(int) * ((size_t)*cap + 1));
  } else {
    for (int w = 0; w < width; w++)
      memcpy(b + (size_t)w * nc, *a + (size_t)w * (*cap), sizeof(int) * (size_t)*cap);
  }
  free(*a);
  *a = b;
  *cap = nc;
}

/* minimum-image separation of atoms i and j (1-based), the reference's
   `X(i,:) - X(j,:) - NINT((X(i,:) - X(j,:))*iLb)*Lb` */
static inline void min_image(const orc_sys* s, const double* X, int i, int j,
                             double xx[3]) {
  int N = s->Natm;
  for (int d = 0; d < 3; d++) {
    double dd = CM(X, N, i, d) - CM(X, N, j, d);
    xx[d] = dd - f_nint(dd * s->iLb[d]) * s->Lb[d];
  }
}

/* Spec mode: every pair with an ion closer than the Moliere list radius (no
   stencil limit), each once as (i, j), i < j, in i's half list, by a direct
   scan over the atoms for each ion; removed atoms take no part. */
static int cmp_pair(const void* a, const void* b);
static void spec_moliere_pairs(orc_sys* s, const double* X) {
  int N = s->Natm;
  double rv2lj = s->rclj * s->rclj;
  int cap = 64, n = 0;
  int* pr = (int*)malloc(sizeof(int) * 2 * (size_t)cap);
  for (int a = 1; a <= N; a++) {
    if (s->atype[a - 1] != 3 || (s->tags[a - 1] & FIBMD_TAG_REMOVED)) continue;
    for (int b = 1; b <= N; b++) {
      if (b == a || (s->tags[b - 1] & FIBMD_TAG_REMOVED)) continue;
      if (s->atype[b - 1] == 3 && b < a) continue; /* an ion pair once */
      double xx[3];
      min_image(s, X, a, b, xx);
      double rij2 = xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2];
      if (!(rij2 < rv2lj)) continue;
      if (n == cap) {
        cap *= 2;
        pr = (int*)realloc(pr, sizeof(int) * 2 * (size_t)cap);
      }
      pr[2 * n] = a < b ? a : b;
      pr[2 * n + 1] = a < b ? b : a;
      n++;
    }
  }
  qsort(pr, (size_t)n, 2 * sizeof(int), cmp_pair);
  grow_int(&s->nlistlj, &s->caplj, n + 1, 1);
  int l = 0;
  for (int i = 1; i <= N; i++) {
    NSSLJ1(s, i) = l + 1;
    while (l < n && pr[2 * l] == i) {
      s->nlistlj[l] = pr[2 * l + 1];
      l++;
    }
    NSSLJ2(s, i) = l;
  }
  s->nbr_cntlj_full = 2 * (long long)n;
  free(pr);
}

/* ---- si_nlistG, si.f90:102-276 (one domain: P_big(i) == myid for all) --- */
void orc_si_nlist(orc_sys* s, const double* X) {
  int N = s->Natm;
  int n1 = s->Nc[0], n2 = s->Nc[1], n3 = s->Nc[2];
  int s1 = n1 + 2, s2 = n2 + 2, s3 = n3 + 2;
  int* LL = (int*)calloc((size_t)N, sizeof(int));
  int* HOC = (int*)calloc((size_t)s1 * s2 * s3, sizeof(int));
  double rv2 = s->rc * s->rc;
  double rv2lj = s->rclj * s->rclj;
  s->cell_oob = 0;
  chainlist(s, LL, HOC, X);

  int nbr_cnt = 1, nbr_cntlj = 1;
  for (int i = 1; i <= N; i++) {
    NSS2(s, i) = -1;
    NSS1(s, i) = 0;
    NSSLJ2(s, i) = -1;
    NSSLJ1(s, i) = 0;
  }
#define HOCI(a, b, c) HOC[(size_t)(a) + (size_t)s1 * ((size_t)(b) + (size_t)s2 * (size_t)(c))]
  for (int ic3 = 1; ic3 <= n3; ic3++)
    for (int ic2 = 1; ic2 <= n2; ic2++)
      for (int ic1 = 1; ic1 <= n1; ic1++) {
        int i = HOCI(ic1, ic2, ic3);
        while (i != 0) {
          NSS1(s, i) = nbr_cnt;
          NSSLJ1(s, i) = nbr_cntlj;
          for (int a = -1; a <= 1; a++)
            for (int b = -1; b <= 1; b++)
              for (int c = -1; c <= 1; c++) {
                int j = HOCI(ic1 + a, ic2 + b, ic3 + c);
                while (j != 0) {
                  if (i != j) {
                    double xx[3];
                    min_image(s, X, i, j, xx);
                    double rij2 = xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2];
                    int ti = s->atype[i - 1], tj = s->atype[j - 1];
                    if ((ti > tj ? ti : tj) < 3) {
                      if (rij2 < rv2) {
                        grow_int(&s->nlist2, &s->cap2, nbr_cnt, 1);
                        s->nlist2[nbr_cnt - 1] = j;
                        nbr_cnt++;
                      }
                    } else {
                      if (rij2 < rv2lj) {
                        grow_int(&s->nlistlj, &s->caplj, nbr_cntlj, 1);
                        s->nlistlj[nbr_cntlj - 1] = j;
                        nbr_cntlj++;
                      }
                    }
                  }
                  j = LL[j - 1];
                }
              }
          NSS2(s, i) = nbr_cnt - 1;
          NSSLJ2(s, i) = nbr_cntlj - 1;
          i = LL[i - 1];
        }
      }
#undef HOCI
  s->nbr_cnt_full = nbr_cnt - 1;
  s->nbr_cntlj_full = nbr_cntlj - 1;

  /* connected triplets, si.f90:191-232 */
  int Nbrs = 0;
  for (int i = 1; i <= N; i++) {
    for (int l = NSS1(s, i); l <= NSS2(s, i); l++) {
      int j = s->nlist2[l - 1];
      if (j > i) {
        for (int m = l + 1; m <= NSS2(s, i); m++) {
          int k = s->nlist2[m - 1];
          if (k > i) {
            grow_int(&s->nlist3, &s->cap3, Nbrs + 1, 3);
            Nbrs++;
            int mn = i < j ? (i < k ? i : k) : (j < k ? j : k);
            int mx = i > j ? (i > k ? i : k) : (j > k ? j : k);
            s->nlist3[Nbrs - 1] = mn;
            s->nlist3[(size_t)s->cap3 + Nbrs - 1] = j + k + i - mn - mx;
            s->nlist3[2 * (size_t)s->cap3 + Nbrs - 1] = mx;
          }
        }
        for (int m = NSS1(s, j); m <= NSS2(s, j); m++) {
          int k = s->nlist2[m - 1];
          if (k > i) {
            int found = 0;
            for (int n = NSS1(s, i); n <= NSS2(s, i); n++)
              if (k == s->nlist2[n - 1]) {
                found = 1;
                break;
              }
            if (found) continue;
            grow_int(&s->nlist3, &s->cap3, Nbrs + 1, 3);
            Nbrs++;
            int mn = i < j ? (i < k ? i : k) : (j < k ? j : k);
            int mx = i > j ? (i > k ? i : k) : (j > k ? j : k);
            s->nlist3[Nbrs - 1] = mn;
            s->nlist3[(size_t)s->cap3 + Nbrs - 1] = j + k + i - mn - mx;
            s->nlist3[2 * (size_t)s->cap3 + Nbrs - 1] = mx;
          }
        }
      }
    }
  }
  s->Nbrs = Nbrs;

  /* drop j < i entries, si.f90:234-260 (Fortran DO bounds are fixed at
     loop entry, so l runs over the original range) */
  for (int i = 1; i <= N; i++) {
    int lo = NSS1(s, i), hi = NSS2(s, i);
    for (int l = lo; l <= hi; l++) {
      int j = s->nlist2[l - 1];
      while (j < i && NSS2(s, i) > l) {
        s->nlist2[l - 1] = s->nlist2[NSS2(s, i) - 1];
        j = s->nlist2[l - 1];
        NSS2(s, i) = NSS2(s, i) - 1;
      }
      if (NSS2(s, i) == l && j < i) NSS2(s, i) = NSS2(s, i) - 1;
    }
  }
  for (int i = 1; i <= N; i++) {
    int lo = NSSLJ1(s, i), hi = NSSLJ2(s, i);
    for (int l = lo; l <= hi; l++) {
      int j = s->nlistlj[l - 1];
      while (j < i && NSSLJ2(s, i) > l) {
        s->nlistlj[l - 1] = s->nlistlj[NSSLJ2(s, i) - 1];
        j = s->nlistlj[l - 1];
        NSSLJ2(s, i) = NSSLJ2(s, i) - 1;
      }
      if (NSSLJ2(s, i) == l && j < i) NSSLJ2(s, i) = NSSLJ2(s, i) - 1;
    }
  }

  s->overflow = 0;
  if (Nbrs >= s->ML3) s->overflow |= 2;
  if (nbr_cnt >= s->ML2) s->overflow |= 1;
  if (nbr_cntlj >= s->MLlj) s->overflow |= 4;
  free(LL);
  free(HOC);
  if (s->spec) {
    spec_moliere_pairs(s, X);
    memcpy(s->Xb, X, sizeof(double) * 3 * (size_t)N);
  }
}

/* ---- itable2bd, si.f90:554-573 ------------------------------------------- */
double orc_itable2bd(orc_sys* s, double ue) {
  int Nt = s->p.Ntable;
  int i = f_int(ue / s->umax * (double)(Nt - 1)) + 1;
  if (i > Nt) {
    s->table_err++;
    return 0.0;
  }
  double d1 = ue - s->u[i - 1];
  double d2 = ue - s->u[i];
  double d3 = ue - s->u[i + 1];
  return 0.5 * d2 * d3 * s->table2bd[i - 1] - d1 * d3 * s->table2bd[i] +
         0.5 * d1 * d2 * s->table2bd[i + 1];
}

/* per-pair/per-triplet kernels shared by the serial and OpenMP force */
static inline void pair_sw_force(orc_sys* s, const double* Xp, int i, int j,
                                 double fi[3]) {
  double xx[3];
  min_image(s, Xp, i, j, xx);
  double rij = sqrt(xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2]);
  int ti = s->atype[i - 1] - 1, tj = s->atype[j - 1] - 1;
  double rijs = rij * s->isigma[ti][tj];
  double df = orc_itable2bd(s, rijs);
  for (int d = 0; d < 3; d++) fi[d] = -(df * xx[d] / rij * s->epssig[ti][tj]);
}

static inline int pair_mol_force(const orc_sys* s, const double* Xp, int i,
                                 int j, double fi[3]) {
  double xx[3];
  min_image(s, Xp, i, j, xx);
  double rij2 = 0.0;
  rij2 += xx[0] * xx[0];
  rij2 += xx[1] * xx[1];
  rij2 += xx[2] * xx[2];
  if (!(rij2 < s->rlj2)) return 0;
  double rij = sqrt(rij2);
  int ti = s->atype[i - 1] - 1, tj = s->atype[j - 1] - 1;
  double aa = s->aamol[ti][tj];
  const fibmd_params* p = &s->p;
  double e1 = exp(-(p->alpha_mol * rij / aa));
  double e2 = exp(-(p->beta_mol * rij / aa));
  double e3 = exp(-(p->gamma_mol * rij / aa));
  double fc = s->ie0 * s->Zmol[ti] * s->Zmol[tj] * p->ec * p->ec / rij *
              ((p->Amol * e1 + p->Bmol * e2 + p->Cmol * e3) / rij +
               (p->Amol * p->alpha_mol / aa * e1 + p->Bmol * p->beta_mol / aa * e2 +
                p->Cmol * p->gamma_mol / aa * e3));
  for (int d = 0; d < 3; d++) fi[d] = fc * xx[d] / rij;
  return 1;
}

/* one nlist3 entry of si_force, si.f90:451-546 */
static inline void triplet_force(const orc_sys* s, const double* Xp, int i,
                                 int j, int k, double fi[3], double fj[3],
                                 double fk[3]) {
  const double al = s->p.al, gamma = s->p.gamma, thrd = s->thrd;
  int ti = s->atype[i - 1] - 1, tj = s->atype[j - 1] - 1, tk = s->atype[k - 1] - 1;
  double isigij = s->isigma[ti][tj];
  double isigik = s->isigma[ti][tk];
  double isigjk = s->isigma[tj][tk];
  double lepsijk = s->leps[ti][tj][tk];
  double xxij[3], xxik[3], xxjk[3], dxxij[3], dxxik[3], dxxjk[3];
  min_image(s, Xp, i, j, xxij);
  double rij = 1. / sqrt(xxij[0] * xxij[0] + xxij[1] * xxij[1] + xxij[2] * xxij[2]);
  for (int d = 0; d < 3; d++) dxxij[d] = xxij[d] * rij;
  double rijs = isigij / rij;
  min_image(s, Xp, i, k, xxik);
  double rik = 1. / sqrt(xxik[0] * xxik[0] + xxik[1] * xxik[1] + xxik[2] * xxik[2]);
  for (int d = 0; d < 3; d++) dxxik[d] = xxik[d] * rik;
  double riks = isigik / rik;
  min_image(s, Xp, j, k, xxjk);
  double rjk = 1. / sqrt(xxjk[0] * xxjk[0] + xxjk[1] * xxjk[1] + xxjk[2] * xxjk[2]);
  for (int d = 0; d < 3; d++) dxxjk[d] = xxjk[d] * rjk;
  double rjks = isigjk / rjk;

  double ctjik = (dxxij[0] * dxxik[0] + dxxij[1] * dxxik[1] + dxxij[2] * dxxik[2]);
  double ctijk = -(dxxij[0] * dxxjk[0] + dxxij[1] * dxxjk[1] + dxxij[2] * dxxjk[2]);
  double ctikj = (dxxik[0] * dxxjk[0] + dxxik[1] * dxxjk[1] + dxxik[2] * dxxjk[2]);
  double dctjik[3], dctijk[3], dctikj[3];
  for (int d = 0; d < 3; d++) {
    dctjik[d] = dxxij[d] * rik + dxxik[d] * rij - ctjik * (dxxij[d] * rij + dxxik[d] * rik);
    dctijk[d] = -dxxjk[d] * rij - ctijk * dxxij[d] * rij;
    dctikj[d] = +dxxjk[d] * rik - ctikj * dxxik[d] * rik;
  }
  double Erijs = 0., Eriks = 0., Erjks = 0.;
  double irijsal = 1. / (rijs - al);
  double iriksal = 1. / (riks - al);
  double irjksal = 1. / (rjks - al);
  double cut = 0.999 * al;
  if (rijs < cut) Erijs = exp(gamma * irijsal);
  if (riks < cut) Eriks = exp(gamma * iriksal);
  if (rjks < cut) Erjks = exp(gamma * irjksal);
  double fijk = (rijs < cut && rjks < cut) ? 1. : 0.;
  double fikj = (riks < cut && rjks < cut) ? 1. : 0.;
  double fjik = (rijs < cut && riks < cut) ? 1. : 0.;
  double dErijs = -gamma * irijsal * irijsal;
  double dEriks = -gamma * iriksal * iriksal;
  double dErjks = -gamma * irjksal * irjksal;
  double Wjik = (ctjik + thrd) * (ctjik + thrd);
  double Wijk = (ctijk + thrd) * (ctijk + thrd);
  double Wikj = (ctikj + thrd) * (ctikj + thrd);
  for (int d = 0; d < 3; d++) {
    fi[d] = -(lepsijk *
              (Erijs * (fjik * Eriks *
                            (Wjik * (dErijs * dxxij[d] * isigij + dEriks * dxxik[d] * isigik) +
                             (ctjik + thrd) * dctjik[d] * 2.) +
                        fijk * Erjks *
                            (dErijs * Wijk * dxxij[d] * isigij + (ctijk + thrd) * dctijk[d] * 2.)) +
               fikj * Eriks * Erjks *
                   (dEriks * Wikj * dxxik[d] * isigik + (ctikj + thrd) * dctikj[d] * 2.)));
  }
  for (int d = 0; d < 3; d++) {
    dctjik[d] = -dxxik[d] * rij + ctjik * dxxij[d] * rij;
    dctijk[d] = -dxxij[d] * rjk + dxxjk[d] * rij + ctijk * (dxxij[d] * rij - dxxjk[d] * rjk);
    dctikj[d] = +dxxik[d] * rjk - ctikj * dxxjk[d] * rjk;
  }
  for (int d = 0; d < 3; d++) {
    fj[d] = -(lepsijk *
              (+Erijs * (fjik * Eriks * (-dErijs * Wjik * dxxij[d] * isigij +
                                         (ctjik + thrd) * dctjik[d] * 2.) +
                         fijk * Erjks *
                             (Wijk * (-dErijs * dxxij[d] * isigij + dErjks * dxxjk[d] * isigjk) +
                              (ctijk + thrd) * dctijk[d] * 2.)) +
               fikj * Eriks * Erjks *
                   (dErjks * Wikj * dxxjk[d] * isigjk + (ctikj + thrd) * dctikj[d] * 2.)));
  }
  for (int d = 0; d < 3; d++) fk[d] = -fi[d] - fj[d];
}

/* Spec mode: an atom removed since the last list build acts on nothing
   (its pairs and triplets are skipped until the lists drop it). */
static inline int gone(const orc_sys* s, int i) {
  return s->spec && (s->tags[i - 1] & FIBMD_TAG_REMOVED);
}

/* ---- si_force, si.f90:384-552 -------------------------------------------- */
void orc_si_force(orc_sys* s, const double* Xp, double* F) {
  int N = s->Natm;
  int lim = s->Nsg + s->impact;
  memset(F, 0, sizeof(double) * 3 * (size_t)N);
  for (int i = 1; i <= N; i++) {
    if (gone(s, i)) continue;
    for (int l = NSS1(s, i); l <= NSS2(s, i); l++) {
      int j = s->nlist2[l - 1];
      if (i > lim || j > lim || gone(s, j)) continue;
      double fi[3];
      pair_sw_force(s, Xp, i, j, fi);
      for (int d = 0; d < 3; d++) {
        CM(F, N, i, d) = CM(F, N, i, d) + fi[d];
        CM(F, N, j, d) = CM(F, N, j, d) - fi[d];
      }
    }
    for (int l = NSSLJ1(s, i); l <= NSSLJ2(s, i); l++) {
      int j = s->nlistlj[l - 1];
      if (i > lim || j > lim || gone(s, j)) continue;
      double fi[3];
      if (pair_mol_force(s, Xp, i, j, fi)) {
        for (int d = 0; d < 3; d++) {
          CM(F, N, i, d) = CM(F, N, i, d) + fi[d];
          CM(F, N, j, d) = CM(F, N, j, d) - fi[d];
        }
      }
    }
  }
  for (int l = 1; l <= s->Nbrs; l++) {
    int i = s->nlist3[l - 1];
    int j = s->nlist3[(size_t)s->cap3 + l - 1];
    int k = s->nlist3[2 * (size_t)s->cap3 + l - 1];
    if (i > lim || j > lim || k > lim) continue;
    if (gone(s, i) || gone(s, j) || gone(s, k)) continue;
    double fi[3], fj[3], fk[3];
    triplet_force(s, Xp, i, j, k, fi, fj, fk);
    for (int d = 0; d < 3; d++) {
      CM(F, N, i, d) = CM(F, N, i, d) + fi[d];
      CM(F, N, j, d) = CM(F, N, j, d) + fj[d];
      CM(F, N, k, d) = CM(F, N, k, d) + fk[d];
    }
  }
}

/* Same algorithm over all host threads (the CPU baseline): each thread
   accumulates into a private copy of F, summed at the end. */
void orc_si_force_omp(orc_sys* s, const double* Xp, double* F, int nthreads) {
#ifdef _OPENMP
  int N = s->Natm;
  int lim = s->Nsg + s->impact;
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  size_t n3 = 3 * (size_t)N;
  double* priv = (double*)calloc(n3 * (size_t)nthreads, sizeof(double));
  int terr = 0;
#pragma omp parallel num_threads(nthreads) reduction(+ : terr)
  {
    int t = omp_get_thread_num();
    double* Fl = priv + n3 * (size_t)t;
    orc_sys local = *s;
    local.table_err = 0;
#pragma omp for schedule(dynamic, 256)
    for (int i = 1; i <= N; i++) {
      if (gone(s, i)) continue;
      for (int l = NSS1(s, i); l <= NSS2(s, i); l++) {
        int j = s->nlist2[l - 1];
        if (i > lim || j > lim || gone(s, j)) continue;
        double fi[3];
        pair_sw_force(&local, Xp, i, j, fi);
        for (int d = 0; d < 3; d++) {
          CM(Fl, N, i, d) += fi[d];
          CM(Fl, N, j, d) -= fi[d];
        }
      }
      for (int l = NSSLJ1(s, i); l <= NSSLJ2(s, i); l++) {
        int j = s->nlistlj[l - 1];
        if (i > lim || j > lim || gone(s, j)) continue;
        double fi[3];
        if (pair_mol_force(s, Xp, i, j, fi))
          for (int d = 0; d < 3; d++) {
            CM(Fl, N, i, d) += fi[d];
            CM(Fl, N, j, d) -= fi[d];
          }
      }
    }
#pragma omp for schedule(static, 4096)
    for (int l = 1; l <= s->Nbrs; l++) {
      int i = s->nlist3[l - 1];
      int j = s->nlist3[(size_t)s->cap3 + l - 1];
      int k = s->nlist3[2 * (size_t)s->cap3 + l - 1];
      if (i > lim || j > lim || k > lim) continue;
      if (gone(s, i) || gone(s, j) || gone(s, k)) continue;
      double fi[3], fj[3], fk[3];
      triplet_force(s, Xp, i, j, k, fi, fj, fk);
      for (int d = 0; d < 3; d++) {
        CM(Fl, N, i, d) += fi[d];
        CM(Fl, N, j, d) += fj[d];
        CM(Fl, N, k, d) += fk[d];
      }
    }
    terr += local.table_err;
#pragma omp for schedule(static)
    for (size_t e = 0; e < n3; e++) {
      double acc = 0.0;
      for (int q = 0; q < nthreads; q++) acc += priv[n3 * (size_t)q + e];
      F[e] = acc;
    }
  }
  s->table_err += terr;
  free(priv);
#else
  (void)nthreads;
  orc_si_force(s, Xp, F);
#endif
}

/* ---- si_potential + h, si.f90:278-380 ------------------------------------ */
static inline double h3(const orc_sys* s, double u, double v, double w) {
  double al = s->p.al, gamma = s->p.gamma;
  if (u < 0.999 * al && v < 0.999 * al)
    return exp(gamma / (u - al) + gamma / (v - al)) * ((w + 1. / 3.) * (w + 1. / 3.));
  return 0.;
}

void orc_si_potential(orc_sys* s, const double* X, double* Utot_out, double* u) {
  int N = s->Natm;
  const fibmd_params* p = &s->p;
  double Utot = 0.;
  memset(u, 0, sizeof(double) * (size_t)N);
  for (int i = 1; i <= N; i++) {
    if (gone(s, i)) continue;
    for (int l = NSS1(s, i); l <= NSS2(s, i); l++) {
      int j = s->nlist2[l - 1];
      if (gone(s, j)) continue;
      double xx[3];
      min_image(s, X, i, j, xx);
      double rij = sqrt(xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2]);
      int ti = s->atype[i - 1] - 1, tj = s->atype[j - 1] - 1;
      double r = rij * s->isigma[ti][tj];
      if (r < 0.999 * p->al) {
        double ul = 0.5 * s->eps[ti][tj] * p->A * (p->B * pow(r, -p->psi) - pow(r, -p->qsi)) *
                    exp(1. / (r - p->al));
        u[i - 1] = u[i - 1] + ul;
        u[j - 1] = u[j - 1] + ul;
        Utot = Utot + 2. * ul;
      }
    }
    for (int l = NSSLJ1(s, i); l <= NSSLJ2(s, i); l++) {
      int j = s->nlistlj[l - 1];
      if (gone(s, j)) continue;
      double xx[3];
      min_image(s, X, i, j, xx);
      double rij2 = 0.0;
      rij2 += xx[0] * xx[0];
      rij2 += xx[1] * xx[1];
      rij2 += xx[2] * xx[2];
      if (rij2 < s->rlj2) {
        double rij = sqrt(rij2);
        int ti = s->atype[i - 1] - 1, tj = s->atype[j - 1] - 1;
        double aa = s->aamol[ti][tj];
        double ul = s->ie0 * s->Zmol[ti] * s->Zmol[tj] * p->ec * p->ec / rij *
                    (p->Amol * exp(-(p->alpha_mol * rij / aa)) +
                     p->Bmol * exp(-(p->beta_mol * rij / aa)) +
                     p->Cmol * exp(-(p->gamma_mol * rij / aa)));
        u[i - 1] = u[i - 1] + ul / 2.;
        u[j - 1] = u[j - 1] + ul / 2.;
        Utot = Utot + ul;
      }
    }
  }
  for (int l = 1; l <= s->Nbrs; l++) {
    int i = s->nlist3[l - 1];
    int j = s->nlist3[(size_t)s->cap3 + l - 1];
    int k = s->nlist3[2 * (size_t)s->cap3 + l - 1];
    if (gone(s, i) || gone(s, j) || gone(s, k)) continue;
    int ti = s->atype[i - 1] - 1, tj = s->atype[j - 1] - 1, tk = s->atype[k - 1] - 1;
    double xxij[3], xxik[3], xxjk[3];
    min_image(s, X, i, j, xxij);
    double rij = sqrt(xxij[0] * xxij[0] + xxij[1] * xxij[1] + xxij[2] * xxij[2]);
    double rijs = rij * s->isigma[ti][tj];
    min_image(s, X, i, k, xxik);
    double rik = sqrt(xxik[0] * xxik[0] + xxik[1] * xxik[1] + xxik[2] * xxik[2]);
    double riks = rik * s->isigma[ti][tk];
    min_image(s, X, j, k, xxjk);
    double rjk = sqrt(xxjk[0] * xxjk[0] + xxjk[1] * xxjk[1] + xxjk[2] * xxjk[2]);
    double rjks = rjk * s->isigma[tj][tk];
    double ctjik = (xxij[0] * xxik[0] + xxij[1] * xxik[1] + xxij[2] * xxik[2]) / rij / rik;
    double ctijk = -(xxij[0] * xxjk[0] + xxij[1] * xxjk[1] + xxij[2] * xxjk[2]) / rij / rjk;
    double ctikj = (xxik[0] * xxjk[0] + xxik[1] * xxjk[1] + xxik[2] * xxjk[2]) / rik / rjk;
    double ul = 1. / 3. * s->leps[ti][tj][tk] *
                (h3(s, rijs, riks, ctjik) + h3(s, rijs, rjks, ctijk) + h3(s, riks, rjks, ctikj));
    u[i - 1] = u[i - 1] + ul;
    u[j - 1] = u[j - 1] + ul;
    u[k - 1] = u[k - 1] + ul;
    Utot = Utot + 3. * ul;
  }
  *Utot_out = Utot;
}

/* ---- temperature, temp.f90:183-205 --------------------------------------- */
double orc_temperature(orc_sys* s, const double* V) {
  int N = s->Natm;
  double T = 0.;
  for (int i = 1; i <= N; i++) {
    if (s->atype[i - 1] < 3) {
      double v1 = CM(V, N, i, 0), v2 = CM(V, N, i, 1), v3 = CM(V, N, i, 2);
      T = T + s->mass[i - 1] * (v1 * v1 + v2 * v2 + v3 * v3);
    }
  }
  return T / 3. / (double)s->Nsg / s->p.kB;
}

/* ---- adjusttemp, temp.f90:160-179 ---------------------------------------- */
void orc_adjusttemp(orc_sys* s, double Temp, double Ttar) {
  int N = s->Natm;
  double sc = sqrt(1. + s->Ts / s->Tau * (Ttar / Temp - 1.));
  for (int i = 1; i <= N; i++)
    if (s->atype[i - 1] < 3)
      for (int d = 0; d < 3; d++) CM(s->V, N, i, d) = sc * CM(s->V, N, i, d);
}

/* ---- controlsidetemp, temp.f90:32-67 (Fortran .and. binds tighter than
        .or.: x-edge .or. (y-edge .and. z-band)) ---------------------------- */
void orc_controlsidetemp(orc_sys* s, double Ttar) {
  int N = s->Natm;
  const fibmd_params* p = &s->p;
  double nm = 1.0e-9;
  double sw = p->sidewidth * nm;
  double zlo = p->outz[0] * s->Lb[2] / 10.0, zhi = p->outz[3] * s->Lb[2] / 10.0;
  double ts = 0.0;
  int kk = 0;
  int* list = (int*)malloc(sizeof(int) * (size_t)N);
  for (int i = 1; i <= N; i++) {
    double x = CM(s->X, N, i, 0), y = CM(s->X, N, i, 1), z = CM(s->X, N, i, 2);
    int xe = (x < sw) || (x > (s->Lb[0] - sw));
    int ye = (y < sw) || (y > (s->Lb[1] - sw));
    int zb = (z < zlo) || (z > zhi);
    if (xe || (ye && zb)) {
      if (s->atype[i - 1] < 3) {
        double v1 = CM(s->V, N, i, 0), v2 = CM(s->V, N, i, 1), v3 = CM(s->V, N, i, 2);
        ts = ts + s->mass[i - 1] * (v1 * v1 + v2 * v2 + v3 * v3);
        list[kk++] = i;
      }
    }
  }
  if (kk > 0) {
    ts = ts / 3. / (double)kk / p->kB;
    double sc = sqrt(1. + s->Ts / s->Tau * (Ttar / ts - 1.));
    for (int q = 0; q < kk; q++)
      for (int d = 0; d < 3; d++) CM(s->V, N, list[q], d) = sc * CM(s->V, N, list[q], d);
  }
  free(list);
}

/* ---- frzsptrdatms, temp.f90:99-127 --------------------------------------- */
void orc_frzsptrdatms(orc_sys* s) {
  int N = s->Natm;
  const fibmd_params* p = &s->p;
  double buffer = 0.3;
  double L3 = s->Lb[2];
  for (int i = 1; i <= N; i++) {
    double z = CM(s->X, N, i, 2);
    int hit = 0;
    if ((z > p->outz[0] * L3 / 10.0) && (z < p->outz[1] * L3 / 10.0)) {
      CM(s->X, N, i, 2) = p->atomz[0] * L3 / 10.0;
      hit = 1;
    } else if ((z > p->outz[2] * L3 / 10.0) && (z < p->outz[3] * L3 / 10.0)) {
      CM(s->X, N, i, 2) = p->atomz[1] * L3 / 10.0;
      hit = 1;
    } else if ((z > (p->atomz[0] - buffer) * L3 / 10.0) && (z < (p->atomz[0] + buffer) * L3 / 10.0)) {
      hit = 1;
    } else if ((z > (p->atomz[1] - buffer) * L3 / 10.0) && (z < (p->atomz[1] + buffer) * L3 / 10.0)) {
      hit = 1;
    } else if ((z > (p->ionz - buffer) * L3 / 10.0) && (z < (p->ionz + buffer) * L3 / 10.0)) {
      hit = 1;
    }
    if (hit)
      for (int d = 0; d < 3; d++) {
        CM(s->V, N, i, d) = 0.0;
        CM(s->F, N, i, d) = 0.0;
      }
  }
}

/* ---- rebox / freezsidesN, tools.f90:26-51 -------------------------------- */
void orc_rebox(orc_sys* s) {
  int N = s->Natm;
  for (int d = 0; d < 3; d++)
    for (int i = 1; i <= N; i++)
      CM(s->X, N, i, d) = fmod(CM(s->X, N, i, d) + 2. * s->Lb[d], s->Lb[d]);
}

void orc_freezsidesN(orc_sys* s) {
  int N = s->Natm;
  for (int i = 1; i <= N; i++)
    if (s->xsides[i - 1] > 0)
      for (int d = 0; d < 3; d++) {
        CM(s->X, N, i, d) = CM(s->Xi, N, i, d);
        CM(s->V, N, i, d) = 0.;
      }
}

/* ---- ionrun, prms.f90:563-584 -------------------------------------------- */
void orc_ionrun(orc_sys* s, int tic) {
  const fibmd_params* p = &s->p;
  if (tic == 1) {
    s->Ts = p->Ts_i;
    s->atm_out = p->atm_out_i;
    s->ntlist = p->ntlist_i;
    s->atlist = p->atlist_i;
    s->Tau = p->Tau_i;
    s->dslist = p->dslist_i;
  } else if (tic == 2) {
    s->Ts = p->Ts_r;
    s->atm_out = p->atm_out_r;
    s->ntlist = p->ntlist_r;
    s->atlist = p->atlist_r;
    s->Tau = p->Tau_r;
    s->dslist = p->dslist_r;
  }
}

/* ---- calc_atm, timeint.f90:277-298 --------------------------------------- */
void orc_calc_atm(orc_sys* s) {
  int N = s->Natm;
  double kmax = -1.0;
  for (int i = 1; i <= N; i++) {
    double ss = 0.0;
    for (int d = 0; d < 3; d++) ss += CM(s->V, N, i, d) * CM(s->V, N, i, d);
    double ke = 0.5 * s->mass[i - 1] * ss / s->p.ec;
    if (i == 1 || ke > kmax) kmax = ke;
  }
  if (kmax < s->p.ke_limit_1 && s->atom_is_fast) {
    orc_ionrun(s, 2);
    s->atom_is_fast = 0;
  }
}

/* ---- onestep, timeint.f90:158-242 (one domain: sendposN, initparaops_l
        and combfN move no data) --------------------------------------------- */
void orc_onestep(orc_sys* s, int whichctrl, double Ttar, long long lt,
                 double* time, double* temp, int nthreads) {
  int N = s->Natm;
  *time = *time + s->Ts;
  if (whichctrl == 0) {
    orc_adjusttemp(s, *temp, Ttar);
    *temp = orc_temperature(s, s->V);
  }
  if (whichctrl > 0) orc_controlsidetemp(s, Ttar);
  for (int i = 1; i <= N; i++) {
    double m = s->mass[i - 1];
    for (int d = 0; d < 3; d++)
      CM(s->X, N, i, d) = CM(s->X, N, i, d) + CM(s->V, N, i, d) * s->Ts +
                          0.5 * CM(s->F, N, i, d) * s->Ts * s->Ts / m;
  }
  orc_freezsidesN(s);
  orc_rebox(s);
  if (lt % s->atlist == 0) orc_frzsptrdatms(s);
  if (lt % s->ntlist == 0) orc_si_nlist(s, s->X);
  if (lt % s->dslist == 0 && whichctrl == 1) orc_calc_atm(s);
  double* Fp = (double*)malloc(sizeof(double) * 3 * (size_t)N);
  if (nthreads > 1)
    orc_si_force_omp(s, s->X, Fp, nthreads);
  else
    orc_si_force(s, s->X, Fp);
  for (int i = 1; i <= N; i++) {
    double m = s->mass[i - 1];
    for (int d = 0; d < 3; d++)
      CM(s->V, N, i, d) = CM(s->V, N, i, d) +
                          0.5 * (CM(s->F, N, i, d) + CM(Fp, N, i, d)) * s->Ts / m;
  }
  memcpy(s->F, Fp, sizeof(double) * 3 * (size_t)N);
  free(Fp);
  if (whichctrl > 0) {
    /* iostuff recomputes temp on atm_out/res_out steps (out.f90:131-150) */
    int dump = (s->p.res_out > 0 && lt % s->p.res_out == 0) ||
               (s->atm_out > 0 && lt % s->atm_out == 0);
    if (dump) *temp = orc_temperature(s, s->V);
  }
}

/* ---- TI, timeint.f90:123-155 --------------------------------------------- */
long long orc_TI(orc_sys* s, int whichctrl, double Ttar, long long Nt,
                 double* time, long long* lt, double* temp, long long max_steps,
                 int nthreads) {
  long long n = 0;
  if (whichctrl == 0) {
    *temp = orc_temperature(s, s->V);
    while (fabs(*temp - Ttar) > s->p.Teps) {
      if (max_steps > 0 && n >= max_steps) break;
      *lt = *lt + 1;
      orc_onestep(s, whichctrl, Ttar, *lt, time, temp, nthreads);
      n++;
    }
  } else if (whichctrl == 1) {
    while (!s->atom_is_slow) {
      if (max_steps > 0 && n >= max_steps) break;
      *lt = *lt + 1;
      if (*time > (double)s->impact * s->p.dti) {
        s->atom_is_slow = 1;
        break;
      }
      orc_onestep(s, whichctrl, Ttar, *lt, time, temp, nthreads);
      n++;
    }
  } else {
    for (long long q = 0; q < Nt; q++) {
      if (max_steps > 0 && n >= max_steps) break;
      *lt = *lt + 1;
      orc_onestep(s, whichctrl, Ttar, *lt, time, temp, nthreads);
      n++;
    }
  }
  return n;
}

/* ---- ran1, src/ran1.f: Park & Miller (1988) minimal standard generator,
        Schrage factorisation, Bays-Durham shuffle of 32 ------------------- */
void orc_rng_seed(orc_rng* r, int seed) {
  memset(r, 0, sizeof(*r));
  r->idum = seed;
}

double orc_ran1(orc_rng* r) {
  const int IA = 16807, IM = 2147483647, IQ = 127773, IR = 2836, NTAB = 32;
  const int NDIV = 1 + (IM - 1) / NTAB;
  const double AM = 1. / IM, EPS = 1.2e-7, RNMX = 1. - EPS;
  if (r->idum <= 0 || r->iy == 0) {
    r->idum = (-r->idum > 1) ? -r->idum : 1;
    for (int j = NTAB + 8; j >= 1; j--) {
      int k = r->idum / IQ;
      r->idum = IA * (r->idum - k * IQ) - IR * k;
      if (r->idum < 0) r->idum += IM;
      if (j <= NTAB) r->iv[j - 1] = r->idum;
    }
    r->iy = r->iv[0];
  }
  int k = r->idum / IQ;
  r->idum = IA * (r->idum - k * IQ) - IR * k;
  if (r->idum < 0) r->idum += IM;
  int j = 1 + r->iy / NDIV;
  r->iy = r->iv[j - 1];
  r->iv[j - 1] = r->idum;
  double v = AM * r->iy;
  return v < RNMX ? v : RNMX;
}

/* round through a text field of `sig` significant digits as Fortran's Ew.d
   output read back by a list-directed READ */
static double through_text(double x, int sig) {
  char buf[64];
  snprintf(buf, sizeof buf, "%.*E", sig - 1, x);
  return strtod(buf, NULL);
}

/* ---- pureepi, prms.f90:484-557 ------------------------------------------- */
int orc_pureepi(int Nc1, int Nc2, int Nc3, double* XX, int* xsides, double Lb[3]) {
  double L[3] = {5.431073E-10, 5.431073E-10, 5.431073E-10};
  double uc[8][3] = {{0.00, 0.00, 0.00},
                     {0.00, 0.50 * L[1], 0.50 * L[2]},
                     {0.250 * L[0], 0.250 * L[1], 0.750 * L[2]},
                     {0.250 * L[0], 0.750 * L[1], 0.250 * L[2]},
                     {0.50 * L[0], 0.0 * L[1], 0.50 * L[2]},
                     {0.50 * L[0], 0.50 * L[1], 0.0 * L[2]},
                     {0.750 * L[0], 0.250 * L[1], 0.250 * L[2]},
                     {0.750 * L[0], 0.750 * L[1], 0.750 * L[2]}};
  int n = 8 * Nc1 * Nc2 * Nc3;
  double* raw = (double*)malloc(sizeof(double) * 3 * (size_t)n);
  int m = 1;
  for (int i = 1; i <= Nc1; i++)
    for (int j = 1; j <= Nc2; j++)
      for (int k = 1; k <= Nc3; k++)
        for (int l = 0; l < 8; l++) {
          CM(raw, n, m, 0) = uc[l][0] + L[0] * (double)(i - 1);
          CM(raw, n, m, 1) = uc[l][1] + L[1] * (double)(j - 1);
          CM(raw, n, m, 2) = uc[l][2] + L[2] * (double)(k - 1);
          m++;
        }
  double maxx = -1e300, maxy = -1e300;
  for (int i = 1; i <= n; i++) {
    if (CM(raw, n, i, 0) > maxx) maxx = CM(raw, n, i, 0);
    if (CM(raw, n, i, 1) > maxy) maxy = CM(raw, n, i, 1);
  }
  for (int i = 1; i <= n; i++) {
    double x = CM(raw, n, i, 0), y = CM(raw, n, i, 1);
    xsides[i - 1] = (x < 1.0e-10 || y < 1.0e-10 || x > maxx - 1.0e-10 || y > maxy - 1.0e-10) ? i : 0;
    for (int d = 0; d < 3; d++) CM(XX, n, i, d) = through_text(CM(raw, n, i, d), 10);
  }
  Lb[0] = L[0] * Nc1;
  Lb[1] = L[1] * Nc2;
  Lb[2] = L[2] * Nc3 * 10;
  free(raw);
  return n;
}

/* ---- initranions, data.f90:263-285 --------------------------------------- */
void orc_initranions(orc_rng* r, int Nrand, double fwhm, double Pi, double* Xrand) {
  for (int i = 1; i <= Nrand; i++) {
    double r1 = orc_ran1(r);
    double r2 = orc_ran1(r);
    double r3 = sqrt(-2 * log(r1)) * cos(2 * Pi * r2) * fwhm / 2.35 * 1.E-9;
    double r4 = sqrt(-2 * log(r2)) * sin(2 * Pi * r1) * fwhm / 2.35 * 1.E-9;
    CM(Xrand, Nrand, i, 0) = through_text(r3, 6);
    CM(Xrand, Nrand, i, 1) = through_text(r4, 6);
  }
}

/* ---- initIons, data.f90:223-260 (the re-draw rechecks the same j only,
        as the reference's `goto 79` does) ---------------------------------- */
void orc_initIons(orc_sys* s, orc_rng* r) {
  int N = s->Natm;
  for (int i = s->Nsg + 1; i <= N; i++) {
    CM(s->X, N, i, 0) = s->Lb[0] * orc_ran1(r);
    CM(s->X, N, i, 1) = s->Lb[1] * orc_ran1(r);
    CM(s->X, N, i, 2) = s->p.ionz * s->Lb[2] / 10.0;
    s->atype[i - 1] = 3;
  }
  for (int i = s->Nsg + 1; i <= N; i++)
    for (int j = s->Nsg + 1; j <= N; j++)
      if (i > j) {
        for (;;) {
          double x0 = CM(s->X, N, i, 0) - CM(s->X, N, j, 0);
          double x1 = CM(s->X, N, i, 1) - CM(s->X, N, j, 1);
          double rij = sqrt(x0 * x0 + x1 * x1);
          if (rij < s->p.sigmaSi) {
            CM(s->X, N, i, 0) = s->Lb[0] * orc_ran1(r);
            CM(s->X, N, i, 1) = s->Lb[1] * orc_ran1(r);
            continue;
          }
          break;
        }
      }
}

/* ---- assignmass, data.f90:207-220 ---------------------------------------- */
void orc_assignmass(orc_sys* s) {
  for (int i = 0; i < s->Natm; i++) {
    if (s->atype[i] == 1) s->mass[i] = s->p.massSi;
    else if (s->atype[i] == 2) s->mass[i] = s->p.massGe;
    else if (s->atype[i] == 3) s->mass[i] = s->p.massGa;
  }
}

/* ---- randvel, data.f90:169-204 (crystalline target) ---------------------- */
void orc_randvel(orc_sys* s, orc_rng* r, double Uo) {
  int N = s->Natm;
  double mm[3] = {0.0, 0.0, 0.0};
  for (int i = 1; i <= s->Nsg; i++) {
    CM(s->V, N, i, 0) = Uo * (orc_ran1(r) - 0.5);
    CM(s->V, N, i, 1) = Uo * (orc_ran1(r) - 0.5);
    CM(s->V, N, i, 2) = Uo * (orc_ran1(r) - 0.5);
    for (int d = 0; d < 3; d++) mm[d] = mm[d] + s->mass[i - 1] * CM(s->V, N, i, d);
  }
  for (int d = 0; d < 3; d++) mm[d] = mm[d] / s->Nsg;
  for (int i = 1; i <= s->Nsg; i++)
    for (int d = 0; d < 3; d++) CM(s->V, N, i, d) = CM(s->V, N, i, d) - mm[d] / s->mass[i - 1];
  for (int i = s->Nsg + 1; i <= N; i++)
    for (int d = 0; d < 3; d++) CM(s->V, N, i, d) = 0.0;
}

/* ---- knock, knock.f90:21-55. NINT(ran1*Nrand) can be 0, which the
        reference reads out of bounds; here index 0 is taken as 1. -------- */
void orc_knock(orc_sys* s, orc_rng* r, int knc, double eV, double phiz,
               double phixy, const double* Xrand, int Nrand) {
  int N = s->Natm;
  double Pi = s->Pi;
  double L3 = s->Lb[2];
  double kv = 1663.6334 * sqrt(eV);
  double dr = tan(phiz * Pi / 180) * (s->p.knockz * L3 / 10 - L3 / 10);
  double dx = dr * cos(phixy * Pi / 180) * sin(phiz * Pi / 180);
  double dy = dr * sin(phixy * Pi / 180) * sin(phiz * Pi / 180);
  int ri = (int)lround(orc_ran1(r) * Nrand);
  if (ri < 1) ri = 1;
  int ion = s->Nsg + knc;
  CM(s->V, N, ion, 0) = kv * cos(phixy * Pi / 180) * sin(phiz * Pi / 180);
  CM(s->V, N, ion, 1) = kv * sin(phixy * Pi / 180) * sin(phiz * Pi / 180);
  CM(s->V, N, ion, 2) = -1.0 * kv * cos(phiz * Pi / 180);
  CM(s->X, N, ion, 0) = CM(Xrand, Nrand, ri, 0) + s->Lb[0] / 2.0 - dx;
  CM(s->X, N, ion, 1) = CM(Xrand, Nrand, ri, 1) + s->Lb[1] / 2.0 - dy;
  CM(s->X, N, ion, 2) = s->p.knockz * L3 / 10.0;
}

/* ---- spec mode ------------------------------------------------------------
   The specified set-up of the benchmark slabs (the reference has none of
   it): each function restates the step of the GPU library's spec mode in
   plain binary64 with the order of operations written out. */

/* the next step and the thermostat factor from the current velocities
   (after a kick): dt = min(dt_max, dx_max / max|v|) over the atoms in the
   run; the Berendsen factor sqrt(1 + dt/tau (Ttar/T - 1)) of the tagged
   layer's lattice atoms, T from their sum of m v^2 */
static void spec_reduce(orc_sys* s) {
  int N = s->Natm;
  const fibmd_params* p = &s->p;
  double vmax2 = 0.0, tsum = 0.0;
  int tcnt = 0;
  for (int i = 1; i <= N; i++) {
    if (s->tags[i - 1] & FIBMD_TAG_REMOVED) continue;
    double v1 = CM(s->V, N, i, 0), v2 = CM(s->V, N, i, 1), v3 = CM(s->V, N, i, 2);
    double vv = v1 * v1 + v2 * v2 + v3 * v3;
    if (vv > vmax2) vmax2 = vv;
    if ((s->tags[i - 1] & FIBMD_TAG_THERMO) && s->atype[i - 1] < 3) {
      tsum = tsum + s->mass[i - 1] * vv;
      tcnt++;
    }
  }
  s->sp_vmax2 = vmax2;
  double vm = sqrt(vmax2);
  double nd = p->dt_max;
  if (vm > 0.0 && p->dx_max / vm < nd) nd = p->dx_max / vm;
  s->sp_dt = nd;
  double sf = 1.0;
  if (tcnt > 0) {
    double T = tsum / 3. / (double)tcnt / p->kB;
    if (T > 0.0) sf = sqrt(1. + nd / p->tau_spec * (p->Ttar1 / T - 1.));
  }
  s->sp_thermo_s = sf;
}

void orc_spec_init(orc_sys* s, const unsigned* tags, double time0) {
  if (!s->spec) return;
  for (int i = 0; i < s->Natm; i++) s->tags[i] = tags ? tags[i] & 0xffu : 0u;
  s->sp_time = time0;
  s->sp_removed = s->sp_ions_removed = 0;
  s->sp_rebuilds = 0;
  spec_reduce(s);
}

/* round(x * qscale) to the nearest integer (ties to even) in one rounding,
   the fixed-point coordinate of x (qscale = 2^32 / Lb) */
static inline double fixed_coord(double x, double qscale) {
  return fma(x, qscale, 6755399441055744.0) - 6755399441055744.0;
}

int orc_spec_step(orc_sys* s, int nthreads) {
  int N = s->Natm;
  const fibmd_params* p = &s->p;
  double dt = s->sp_dt, h2 = 0.5 * dt * dt, hdt = 0.5 * dt, ts = s->sp_thermo_s;
  double qs[3];
  for (int d = 0; d < 3; d++) qs[d] = 4294967296.0 / s->Lb[d];
  int trig = 0;
  /* the pair rule's two largest squared displacements at or above the
     reporting bound (a quarter of the skin) */
  const double low2 = 0.25 * s->sp_trig2;
  double top1 = 0.0, top2 = 0.0;
  /* drift: thermostat scaling, X += V dt + F dt^2/(2m), pinning, removal
     (on the unwrapped height), wrap of atoms that left the box, and the
     rebuild test against the positions of the last build */
  for (int i = 1; i <= N; i++) {
    unsigned tg = s->tags[i - 1];
    if (tg & FIBMD_TAG_REMOVED) continue;
    double x[3], v[3];
    for (int d = 0; d < 3; d++) {
      x[d] = CM(s->X, N, i, d);
      v[d] = CM(s->V, N, i, d);
    }
    if (tg & FIBMD_TAG_THERMO)
      for (int d = 0; d < 3; d++) v[d] = v[d] * ts;
    double c = h2 * (1.0 / s->mass[i - 1]);
    for (int d = 0; d < 3; d++) x[d] = x[d] + v[d] * dt + c * CM(s->F, N, i, d);
    if (tg & FIBMD_TAG_FROZEN)
      for (int d = 0; d < 3; d++) {
        x[d] = CM(s->Xi, N, i, d);
        v[d] = 0.0;
      }
    int removed = (p->remove_z > 0.0 && x[2] > p->remove_z) || x[2] < s->sp_remove_zlo;
    /* an atom outside [0, Lb) by its fixed-point coordinate moves one box
       back; z stays unwrapped on an open axis */
    for (int d = 0; d < 3; d++) {
      if (d == 2 && s->sp_zopen) continue;
      double k = fixed_coord(x[d], qs[d]);
      if (k < 0.0 || k >= 4294967296.0) x[d] = x[d] + (k < 0.0 ? s->Lb[d] : -s->Lb[d]);
    }
    if (removed) {
      s->tags[i - 1] = tg | FIBMD_TAG_REMOVED;
      for (int d = 0; d < 3; d++) v[d] = 0.0;
      if (s->atype[i - 1] < 3) s->sp_removed++;
      else s->sp_ions_removed++;
    }
    for (int d = 0; d < 3; d++) {
      CM(s->X, N, i, d) = x[d];
      CM(s->V, N, i, d) = v[d];
    }
    if (!removed) {
      double dd = 0.0;
      for (int d = 0; d < 3; d++) {
        double e = x[d] - CM(s->Xb, N, i, d);
        e = e - f_nint(e * s->iLb[d]) * s->Lb[d];
        dd = dd + e * e;
      }
      if (!s->sp_rule) {
        if (dd >= s->sp_trig2) trig = 1;
      } else if (dd >= low2) {
        if (dd > top1) {
          top2 = top1;
          top1 = dd;
        } else if (dd > top2) {
          top2 = dd;
        }
      }
    }
  }
  /* a pair outside the list radius at the build comes within the cutoff
     only once the two atoms' displacements add up to the skin */
  if (s->sp_rule && top1 > 0.0 &&
      sqrt(top1) + sqrt(top2 > low2 ? top2 : low2) >= 2.0 * sqrt(s->sp_trig2))
    trig = 1;
  if (trig || s->sp_force_rebuild) {
    orc_si_nlist(s, s->X);
    s->sp_rebuilds++;
    s->sp_force_rebuild = 0;
    trig = 1;
  }
  double* Fp = (double*)malloc(sizeof(double) * 3 * (size_t)N);
  if (nthreads > 1)
    orc_si_force_omp(s, s->X, Fp, nthreads);
  else
    orc_si_force(s, s->X, Fp);
  /* kick: V += (F + Fp) dt/(2m) for the atoms in the run (pinned ones
     included: the next drift pins them again) */
  for (int i = 1; i <= N; i++) {
    if (s->tags[i - 1] & FIBMD_TAG_REMOVED) continue;
    double c = hdt * (1.0 / s->mass[i - 1]);
    for (int d = 0; d < 3; d++)
      CM(s->V, N, i, d) = CM(s->V, N, i, d) + c * (CM(s->F, N, i, d) + CM(Fp, N, i, d));
  }
  memcpy(s->F, Fp, sizeof(double) * 3 * (size_t)N);
  free(Fp);
  s->sp_time = s->sp_time + dt;
  spec_reduce(s);
  return trig;
}

void orc_spec_set_rule(orc_sys* s, int rule) { s->sp_rule = rule ? 1 : 0; }

void orc_spec_scalars(orc_sys* s, double* out7) {
  out7[0] = s->sp_time;
  out7[1] = s->sp_dt;
  out7[2] = s->sp_thermo_s;
  out7[3] = s->sp_vmax2;
  out7[4] = (double)s->sp_removed;
  out7[5] = (double)s->sp_ions_removed;
  out7[6] = (double)s->sp_rebuilds;
}

const unsigned* orc_spec_tags(orc_sys* s) { return s->tags; }

void orc_spec_inject(orc_sys* s, int i, const double x[3], const double v[3]) {
  int N = s->Natm;
  s->tags[i - 1] &= ~(unsigned)FIBMD_TAG_REMOVED;
  for (int d = 0; d < 3; d++) {
    CM(s->X, N, i, d) = x[d];
    CM(s->V, N, i, d) = v[d];
    CM(s->F, N, i, d) = 0.0;
  }
  s->sp_force_rebuild = 1;
  spec_reduce(s);
}

void orc_maxwell(orc_rng* r, int n, int N, const double* mass, double T, double kB, double* V) {
  const double Pi = 4. * atan(1.0);
  long long nv = 3 * (long long)n;
  for (long long m = 0; m < nv; m += 2) {
    double u1 = orc_ran1(r);
    double u2 = orc_ran1(r);
    double rad = sqrt(-2. * log(u1));
    double z[2] = {rad * cos(2. * Pi * u2), rad * sin(2. * Pi * u2)};
    for (int q = 0; q < 2 && m + q < nv; q++) {
      long long e = m + q;
      int i = (int)(e / 3), d = (int)(e % 3);
      V[(size_t)d * (size_t)N + (size_t)i] = z[q] * sqrt(kB * T / mass[i]);
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

/* ---- test helpers --------------------------------------------------------- */
static int cmp_pair(const void* a, const void* b) {
  const int* x = (const int*)a;
  const int* y = (const int*)b;
  if (x[0] != y[0]) return x[0] < y[0] ? -1 : 1;
  if (x[1] != y[1]) return x[1] < y[1] ? -1 : 1;
  return 0;
}
static int cmp_trip(const void* a, const void* b) {
  const int* x = (const int*)a;
  const int* y = (const int*)b;
  for (int d = 0; d < 3; d++)
    if (x[d] != y[d]) return x[d] < y[d] ? -1 : 1;
  return 0;
}

long long orc_get_pairs(orc_sys* s, int kind, int* ij, long long cap) {
  long long n = 0;
  for (int i = 1; i <= s->Natm; i++) {
    int lo = kind ? NSSLJ1(s, i) : NSS1(s, i);
    int hi = kind ? NSSLJ2(s, i) : NSS2(s, i);
    for (int l = lo; l <= hi; l++) {
      if (n < cap) {
        ij[2 * n] = i;
        ij[2 * n + 1] = kind ? s->nlistlj[l - 1] : s->nlist2[l - 1];
      }
      n++;
    }
  }
  if (n <= cap) qsort(ij, (size_t)n, 2 * sizeof(int), cmp_pair);
  return n;
}

long long orc_get_triplets(orc_sys* s, int* ijk, long long cap) {
  long long n = s->Nbrs;
  if (n > cap) return n;
  for (long long l = 0; l < n; l++) {
    ijk[3 * l] = s->nlist3[l];
    ijk[3 * l + 1] = s->nlist3[(size_t)s->cap3 + l];
    ijk[3 * l + 2] = s->nlist3[2 * (size_t)s->cap3 + l];
  }
  qsort(ijk, (size_t)n, 3 * sizeof(int), cmp_trip);
  return n;
}

/* ---- accessors for the Python test harness -------------------------------- */
orc_sys* orc_create(const fibmd_params* p) {
  orc_sys* s = (orc_sys*)calloc(1, sizeof(orc_sys));
  if (orc_init(s, p) != 0) {
    free(s);
    return NULL;
  }
  return s;
}

void orc_destroy(orc_sys* s) {
  if (!s) return;
  orc_free(s);
  free(s);
}

void orc_arrays(orc_sys* s, double** X, double** Xi, double** V, double** F, double** mass,
                int** atype, int** xsides) {
  *X = s->X;
  *Xi = s->Xi;
  *V = s->V;
  *F = s->F;
  *mass = s->mass;
  *atype = s->atype;
  *xsides = s->xsides;
}

void orc_set_impact(orc_sys* s, int impact) { s->impact = impact; }
void orc_set_tau(orc_sys* s, double tau) { s->Tau = tau; }
void orc_set_fast(orc_sys* s, int fast, int slow) {
  s->atom_is_fast = fast;
  s->atom_is_slow = slow;
}

void orc_regime(orc_sys* s, double* Ts, double* Tau, int* ints5) {
  *Ts = s->Ts;
  *Tau = s->Tau;
  ints5[0] = s->ntlist;
  ints5[1] = s->atlist;
  ints5[2] = s->dslist;
  ints5[3] = s->atm_out;
  ints5[4] = s->atom_is_fast;
}

void orc_list_info(orc_sys* s, long long* out6) {
  out6[0] = s->nbr_cnt_full;
  out6[1] = s->nbr_cntlj_full;
  out6[2] = s->Nbrs;
  out6[3] = s->overflow;
  out6[4] = s->cell_oob;
  out6[5] = s->table_err;
}

void orc_geometry(orc_sys* s, double* rc_rclj_rlj2_umax, int* Nc) {
  rc_rclj_rlj2_umax[0] = s->rc;
  rc_rclj_rlj2_umax[1] = s->rclj;
  rc_rclj_rlj2_umax[2] = s->rlj2;
  rc_rclj_rlj2_umax[3] = s->umax;
  Nc[0] = s->Nc[0];
  Nc[1] = s->Nc[1];
  Nc[2] = s->Nc[2];
}

const double* orc_table(orc_sys* s, int which) { return which ? s->u : s->table2bd; }
