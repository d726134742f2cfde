/*
 * fibmd_oracle.h — CPU oracle for the FIB_MD hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C, binary64 restatement of the
 * reference's Fortran routines on the per-step path (nanoMFG/FIB_MD,
 * src/si.f90, src/nlist.f90, src/timeint.f90, src/temp.f90, src/tools.f90,
 * src/prms.f90, src/data.f90, src/knock.f90, src/ran1.f). Only the tests,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it, and
 * only as the checker or the timed CPU baseline; the GPU library never links
 * or calls it.
 *
 * Parity status: the reference is Fortran and no Fortran compiler exists
 * where this is built, and the reference ships no tests, fixtures or golden
 * vectors. Parity with the reference's own outputs is therefore UNPINNED;
 * the restatement is pinned instead by known answers that follow from the
 * reference's formulas (perfect-diamond energy -2*eps per atom, Newton's
 * third law, F = -dU/dX of si_potential for the 3-body and Moliere terms,
 * the published Park-Miller/Bays-Durham sequence of ran1).
 *
 * Semantics: Fortran 1-based indexing is kept (atom ids in the lists are
 * 1-based), arrays are column-major (Natm,3), and each expression keeps the
 * reference's left-to-right evaluation order. Build with -ffp-contract=off
 * and without fast-math so no FMA contraction changes the rounding.
 */
#ifndef FIBMD_ORACLE_H
#define FIBMD_ORACLE_H

#include "../include/fibmd_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sys {
  fibmd_params p;
  int Natm, Nsg, Nlj;
  double Lb[3], iLb[3];

  /* derived constants (prms.f90 readprms/setupSiGe/setupMol) */
  double Pi, thrd;
  double eps[2][2], isigma[2][2], leps[2][2][2], epssig[2][2];
  double Zmol[3], aamol[3][3], ie0;

  /* neighbour lists (si.f90 module variables) */
  double rc, rclj, rlj2;
  int Nc[3];
  int ML2, ML3, MLlj;          /* reference capacities (warning thresholds) */
  int cap2, cap3, caplj;       /* allocated sizes (grown on demand)          */
  int* nss;                    /* (Natm,2) col-major                          */
  int* nsslj;                  /* (Natm,2)                                    */
  int* nlist2;                 /* full list, then halved in place             */
  int* nlistlj;
  int* nlist3;                 /* (cap3,3) col-major                          */
  int Nbrs;                    /* triplet count                               */
  long long nbr_cnt_full;      /* full SW entries before halving              */
  long long nbr_cntlj_full;    /* full Moliere entries before halving         */
  int overflow;                /* bit0 ML2, bit1 ML3, bit2 MLlj exceeded      */
  int cell_oob;                /* atoms whose cell index fell outside 0..N+1  */

  /* 2-body table (mktables) */
  double umax;
  double* table2bd;            /* 1-based: table2bd[i-1]                      */
  double* u;
  int table_err;               /* itable2bd index > Ntable events             */

  /* state */
  double *X, *Xi, *V, *F, *mass;
  int *atype, *xsides;

  /* regime (prms.f90 ionrun) and impact counter */
  double Ts, Tau;
  int ntlist, atlist, dslist, atm_out;
  int impact;
  int atom_is_fast, atom_is_slow;

  /* spec mode: the specified set-up, which the reference does not have
     (variable dt, skin-triggered rebuild, layer tags, removal); see
     orc_spec_* */
  int spec;                    /* lists and steps follow spec mode           */
  unsigned* tags;              /* FIBMD_TAG_* bits per atom                  */
  double* Xb;                  /* positions at the last list build (Natm,3)  */
  double sp_dt, sp_thermo_s;   /* current step, thermostat-layer factor      */
  double sp_time, sp_vmax2;    /* simulated time, max |v|^2 of the last kick */
  double sp_remove_zlo;        /* atoms below are removed (open z axis)      */
  double sp_trig2;             /* squared half skin: the rebuild trigger     */
  int sp_rule;                 /* 1: pair rule (default), 0: half skin        */
  int sp_zopen;                /* z is an open axis (not wrapped)            */
  int sp_force_rebuild;        /* the next step rebuilds the lists           */
  int sp_removed, sp_ions_removed;
  long long sp_rebuilds;
} orc_sys;

/* Park-Miller minimal standard with Bays-Durham shuffle (ran1, src/ran1.f). */
typedef struct orc_rng {
  int iv[32];
  int iy;
  int idum;
} orc_rng;

/* prms.f90:172-216 constants and the reference's shipped siga.in */
void orc_params_default(fibmd_params* p);
int orc_init(orc_sys* s, const fibmd_params* p);
void orc_free(orc_sys* s);

/* si.f90 */
void orc_si_nlist(orc_sys* s, const double* X);
double orc_itable2bd(orc_sys* s, double ue);
void orc_si_force(orc_sys* s, const double* Xp, double* F);
void orc_si_force_omp(orc_sys* s, const double* Xp, double* F, int nthreads);
void orc_si_potential(orc_sys* s, const double* X, double* Utot, double* u);

/* temp.f90 / tools.f90 / timeint.f90 */
double orc_temperature(orc_sys* s, const double* V);
void orc_adjusttemp(orc_sys* s, double Temp, double Ttar);
void orc_controlsidetemp(orc_sys* s, double Ttar);
void orc_frzsptrdatms(orc_sys* s);
void orc_rebox(orc_sys* s);
void orc_freezsidesN(orc_sys* s);
void orc_calc_atm(orc_sys* s);
void orc_ionrun(orc_sys* s, int tic);
void orc_onestep(orc_sys* s, int whichctrl, double Ttar, long long lt,
                 double* time, double* temp, int nthreads);
/* TI loop; returns the number of onestep calls made (bounded by max_steps
   when max_steps > 0). */
long long orc_TI(orc_sys* s, int whichctrl, double Ttar, long long Nt,
                 double* time, long long* lt, double* temp,
                 long long max_steps, int nthreads);

/* set-up restatements (prms.f90 pureepi, data.f90, knock.f90, ran1.f) */
void orc_rng_seed(orc_rng* r, int seed);
double orc_ran1(orc_rng* r);
/* pureepi: fills XX (8*Nc1*Nc2*Nc3,3) already rounded through the si.dat
   text format (3E20.10) as readlat reads it back, xsides from the unrounded
   lattice, and Lb. Returns Nsg. */
int orc_pureepi(int Nc1, int Nc2, int Nc3, double* XX, int* xsides,
                double Lb[3]);
/* initranions: Xrand (Nrand,2) rounded through fwhm.dat's E12.6 format. */
void orc_initranions(orc_rng* r, int Nrand, double fwhm, double Pi,
                     double* Xrand);
void orc_initIons(orc_sys* s, orc_rng* r);
void orc_assignmass(orc_sys* s);
void orc_randvel(orc_sys* s, orc_rng* r, double Uo);
void orc_knock(orc_sys* s, orc_rng* r, int knc, double eV, double phiz,
               double phixy, const double* Xrand, int Nrand);

/* ---- spec mode ------------------------------------------------------------
   The specified physical set-up of the benchmark slabs, which the
   reference lacks (restated from the GPU library's spec mode as
   fibmd_gpu.h documents it; it is on when the parameters' mode is
   FIBMD_MODE_SPEC):
   variable dt = min(dt_max, dx_max / max|v|); lists of radius cutoff + skin
   (0.999 a sigma + list_skin for Si/Ge pairs, 2.5 sigma + list_skin for
   pairs with an ion, every such pair found) rebuilt when the two largest
   displacements since the last build add up to the skin (orc_spec_set_rule
   1, the default) or one reaches half of it (0); frozen and thermostatted
   layers as
   per-atom tags; atoms above remove_z removed (and, with z an open axis,
   atoms 10 A below z = 0). A step: thermostat scaling of the tagged layer,
   drift, pinning, removal, wrap, the rebuild test, [rebuild], force, kick,
   then the reductions that set the next dt and thermostat factor. */

/* Spec mode on: tags (Natm entries, may be NULL for none), the state's V
   gives the first dt and thermostat factor, time0 the start time. Call
   after the state is loaded and before orc_si_nlist; afterwards
   orc_si_nlist builds spec-mode lists and orc_si_force skips removed
   atoms. */
void orc_spec_init(orc_sys* s, const unsigned* tags, double time0);
/* One spec-mode step (nthreads > 1: the OpenMP force). Returns 1 when the
   lists were rebuilt in it. */
int orc_spec_step(orc_sys* s, int nthreads);
/* The rebuild rule: 1 (the default), rebuild when the two largest
   displacements since the last build add up to the skin (those under a
   quarter of the skin counted at that bound); 0, when any atom's reaches half
   the skin. Both with the 1 % margin of the skin. */
void orc_spec_set_rule(orc_sys* s, int rule);
/* time, dt, thermostat factor, vmax2, removed lattice atoms, removed ions,
   rebuilds since orc_spec_init */
void orc_spec_scalars(orc_sys* s, double* out7);
/* One impact of a dose (the device side of knock repeated): atom i
   (1-based, a pre-allocated ion kept removed until now) joins the run at
   position x with velocity v and zero force, the lists are rebuilt at the
   next step, and the step and thermostat factor are recomputed for the new
   velocities. */
void orc_spec_inject(orc_sys* s, int i, const double x[3], const double v[3]);
const unsigned* orc_spec_tags(orc_sys* s);

/* Maxwell-Boltzmann velocities at temperature T for rows 0..n-1 of V
   ((N,3) column-major): normal deviates by the Box-Muller method (Box and
   Muller, 1958) from consecutive ran1 pairs, filled atom by atom (x, y, z),
   scaled by sqrt(kB T / m); then the mass-weighted mean velocity is
   removed. */
void orc_maxwell(orc_rng* r, int n, int N, const double* mass, double T, double kB, double* V);

/* accessors for the Python test harness */
orc_sys* orc_create(const fibmd_params* p);
void orc_destroy(orc_sys* s);
void orc_arrays(orc_sys* s, double** X, double** Xi, double** V, double** F, double** mass,
                int** atype, int** xsides);
void orc_set_impact(orc_sys* s, int impact);
void orc_set_tau(orc_sys* s, double tau);
void orc_set_fast(orc_sys* s, int fast, int slow);
void orc_regime(orc_sys* s, double* Ts, double* Tau, int* ints5);
void orc_list_info(orc_sys* s, long long* out6);
void orc_geometry(orc_sys* s, double* rc_rclj_rlj2_umax, int* Nc);
const double* orc_table(orc_sys* s, int which);

/* helpers for tests: half lists as sorted 1-based pairs, triplets sorted */
long long orc_get_pairs(orc_sys* s, int kind, int* ij, long long cap);
long long orc_get_triplets(orc_sys* s, int* ijk, long long cap);

#ifdef __cplusplus
}
#endif
#endif
