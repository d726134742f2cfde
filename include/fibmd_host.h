/*
 * fibmd_host.h — host-side set-up of a FIB_MD run, exported by
 * libfibmd_gpu.so next to the GPU entry points.
 *
 * In a Fortran build these routines stay the reference's own (prms.f90,
 * data.f90, knock.f90, ran1.f); this C++ restatement lets the C++ driver
 * (mdrun2_gpu) and the Python package run the same set-up without a Fortran
 * compiler. None of it is on the per-step path.
 */
#ifndef FIBMD_HOST_H
#define FIBMD_HOST_H

#include "fibmd_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* siga.in values that the GPU step does not need (src/prms.f90:223-275). */
typedef struct fibmd_siga {
  int amorcrys, whichic, startimpact;
  double eV;
  int Nc[3];
  int Npc[3];
  int Nt;
  double ke_limit_2;
  double Uo;
  int eng_out, tmp_out;
  int Nrand;
  double fwhm;
  double phiz, phixy;
} fibmd_siga;

/* ran1 state: Park & Miller's minimal standard generator with the
   Bays-Durham shuffle (src/ran1.f). A seed <= 0 (re)initialises. */
typedef struct fibmd_rng {
  int iv[32];
  int iy;
  int idum;
} fibmd_rng;

void fibmd_host_rng_seed(fibmd_rng* r, int seed);
double fibmd_host_ran1(fibmd_rng* r);

/* Read siga.in's 45 list-directed values in order (src/prms.f90:221-275);
   text after a backslash on a line is a comment. p keeps its potential
   constants; its siga.in fields are overwritten. Returns FIBMD_OK or
   FIBMD_EINVAL (missing/unreadable value; msg gets the reason). */
int fibmd_host_read_siga(const char* path, fibmd_params* p, fibmd_siga* s,
                         char* msg, int msglen);

/* pureepi (src/prms.f90:484-557): diamond-cubic slab of Nc1 x Nc2 x Nc3
   unit cells; XX (8*Nc1*Nc2*Nc3, 3) column-major, rounded through si.dat's
   3E20.10 text format as readlat reads it back; xsides from the unrounded
   lattice; Lb with z = 10 x slab. Returns the atom count. */
int fibmd_host_pureepi(int Nc1, int Nc2, int Nc3, double* XX, int* xsides, double Lb[3]);

/* initranions (src/data.f90:263-285): Xrand (Nrand,2), rounded through
   fwhm.dat's E12.6 format. */
void fibmd_host_initranions(fibmd_rng* r, int Nrand, double fwhm, double* Xrand);

/* ic case 4 after pureepi (src/data.f90:56-67,115-123,207-260,169-204):
   ions at ionz with lateral re-draws, Xi = X, masses, uniform random
   velocities of amplitude Uo with zero net momentum. X, Xi, V: (Natm,3);
   mass, atype: (Natm). The first Nsg rows of X must hold the lattice. */
int fibmd_host_init_state(const fibmd_params* p, fibmd_rng* r, double Uo, double* X,
                          double* Xi, double* V, double* mass, int* atype);

/* knock (src/knock.f90:21-55): start point and velocity of ion knc.
   NINT(ran1*Nrand) may be 0 in the reference (an out-of-bounds read); here
   index 0 is taken as 1. Returns the 1-based atom index (Nsg + knc). */
int fibmd_host_knock(const fibmd_params* p, fibmd_rng* r, int knc, double eV, double phiz,
                     double phixy, const double* Xrand, int Nrand, double x[3], double v[3]);

#ifdef __cplusplus
}
#endif
#endif
