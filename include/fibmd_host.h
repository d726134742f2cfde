/*
 * fibmd_host.h — host-side set-up of a FIB_MD run, exported by
 * libfibmd_gpu.so next to the GPU entry points.
 *
 * In a Fortran build these routines stay the reference's own (prms.f90,
 * data.f90, knock.f90, ran1.f, out.f90); this C++ restatement lets C/C++
 * hosts and the Python package run the same set-up and write the same dump
 * files without a Fortran compiler. None of it is on the per-step path.
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

/* Maxwell-Boltzmann velocities at temperature T (K) for rows 0..n-1 of V
   ((N,3) column-major; mass in kg, kB in J/K): normal deviates by the
   Box-Muller method from consecutive ran1 pairs, filled atom by atom
   (x, y, z), scaled by sqrt(kB T / m), then the mass-weighted mean velocity
   removed. The reference starts from uniform velocities (randvel,
   src/data.f90:169-204) and a warm-up; this is the spec-mode set-up's
   thermal start, which has no counterpart there. */
void fibmd_host_maxwell(fibmd_rng* r, int n, int N, const double* mass, double T, double kB,
                        double* V);

/* knock (src/knock.f90:21-55): start point and velocity of ion knc.
   NINT(ran1*Nrand) may be 0 in the reference (an out-of-bounds read); here
   index 0 is taken as 1. Returns the 1-based atom index (Nsg + knc). */
int fibmd_host_knock(const fibmd_params* p, fibmd_rng* r, int knc, double eV, double phiz,
                     double phixy, const double* Xrand, int Nrand, double x[3], double v[3]);

/* ---- dump files (src/out.f90) ---------------------------------------------
   writeatoms (src/out.f90:62-100): frames appended to an extended-xyz file
   (data/mdrun2.xyz in the reference) in its fixed-width layout — the atom
   count (I9); "Time (ps) = " and the time with the column titles; per atom
   x y z in Angstrom (3F12.4), the species (A8), the owning process (I8, 0
   here) and the kinetic energy in eV (ES14.3) — and, if snap_path is given,
   the snapshot file (data/3dmol2.xyz) rewritten with each frame. A
   background thread formats and writes queued frames, so a host can queue
   a frame (fibmd_gpu_xyz_frame fills its arrays) and step on. Type 2 is
   written "Ge" (the reference leaves that name unset). */
typedef struct fibmd_xyz_writer fibmd_xyz_writer;
int fibmd_host_xyz_open(const char* path, const char* snap_path, fibmd_xyz_writer** out);
/* Queue one frame; the arrays are copied (xyz_A: (natm,3) column-major;
   proc may be NULL). */
int fibmd_host_xyz_write(fibmd_xyz_writer* w, int natm, double time_s, const double* xyz_A,
                         const int* atype, const double* ke_eV, const int* proc);
/* Wait until every queued frame is written. */
int fibmd_host_xyz_flush(fibmd_xyz_writer* w);
/* Flush, stop the writer thread and close the file. */
int fibmd_host_xyz_close(fibmd_xyz_writer* w);

/* writerestart (src/out.f90:34-58) and its reader: Fortran unformatted
   sequential records with gfortran's 4-byte length markers — (lt,
   restart_time), (X, V, mass, atype), (impact); X, V: (natm,3) column-major
   binary64, atype 4-byte integers. The reader checks every marker against
   natm and fails on a mismatch. */
int fibmd_host_write_restart(const char* path, int natm, int lt, double restart_time,
                             const double* X, const double* V, const double* mass,
                             const int* atype, int impact);
int fibmd_host_read_restart(const char* path, int natm, int* lt, double* restart_time, double* X,
                            double* V, double* mass, int* atype, int* impact);

#ifdef __cplusplus
}
#endif
#endif
