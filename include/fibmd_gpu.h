/*
 * fibmd_gpu.h — C-ABI of the GB300 (sm_103a) backend for the FIB_MD per-step
 * hot path: cell binning, Verlet-list build, the fused Stillinger-Weber 2/3-body
 * + Moliere force, and the velocity-Verlet step with the Berendsen edge
 * thermostat, side freezing, reboxing and sputter parking.
 *
 * The reference (nanoMFG/FIB_MD, Fortran 90 + MPI) has no plugin API: the hot
 * path is a set of module subroutines called from `onestep`
 * (src/timeint.f90:158-242). Each entry point below names the routine(s) it
 * replaces. A Fortran host binds them with ISO_C_BINDING (the interface
 * module fib_md_gb300/fortran/fibmd_gpu_mod.f90 declares every one); the C++
 * host driver and the Python package `fib_md_gb300` bind the same symbols.
 *
 * Conventions (mirroring the reference's):
 *   - Every real is IEEE binary64 (the reference builds with -fdefault-real-8,
 *     src/Makefile:4). SI units: metres, seconds, kilograms, joules.
 *   - Per-atom vectors are passed column-major as the Fortran arrays
 *     X(Natm,3): all x, then all y, then all z (src/data.f90:19-24).
 *   - Atom indices that cross the ABI are 1-based, as in Fortran.
 *   - Every entry point returns an int status (FIBMD_OK == 0). No exception or
 *     abort crosses the ABI; fibmd_gpu_last_error() gives the message.
 *   - Ownership: the caller keeps its host arrays; the context owns all device
 *     memory and copies on upload/download.
 *   - Threading: one context per host thread; calls on one context are not
 *     re-entrant. All work of a context is ordered on one CUDA stream.
 */
#ifndef FIBMD_GPU_H
#define FIBMD_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FIBMD_ABI_VERSION 1

/* ---- status codes --------------------------------------------------------- */
enum {
  FIBMD_OK = 0,
  FIBMD_EINVAL = 1,    /* bad argument / inconsistent parameters            */
  FIBMD_ECUDA = 2,     /* a CUDA runtime call failed                          */
  FIBMD_EOVERFLOW = 3, /* a neighbour-list capacity was exceeded (list kept
                          truncated; the reference prints and continues,
                          src/si.f90:264-272)                                 */
  FIBMD_ENAN = 4,      /* non-finite position/velocity/force detected         */
  FIBMD_ETIMEOUT = 5,  /* a bounded device wait gave up                       */
  FIBMD_ESTATE = 6,    /* call order violated (e.g. steps before upload)      */
  FIBMD_ENOMEM = 7,    /* device allocation failed                            */
  FIBMD_ETABLE = 8     /* 2-body table index beyond Ntable (the reference
                          prints "ERRRRRRROR" and uses 0, src/si.f90:562-564) */
};

/* ---- modes ------------------------------------------------------------------ */
enum {
  /* Exact reference semantics: two-level fixed time step switched by
     calc_atm/ionrun, lists rebuilt every ntlist steps (stale lists kept),
     lateral edge thermostat with the reference's predicate, sputter parking. */
  FIBMD_MODE_REF = 0,
  /* Specified physical set-up: variable dt = min(dt_max, dx_max/max|v|),
     rebuild when the max displacement since the last build exceeds half the
     skin, thermostat/fixed layers given as per-atom tags, removal of
     sputtered atoms above a height. */
  FIBMD_MODE_SPEC = 1
};
enum {
  FIBMD_PREC_FP64 = 0,  /* all force arithmetic in binary64                   */
  FIBMD_PREC_MIXED = 1  /* SW/Moliere arithmetic in binary32 (reduced units),
                           binary64 accumulation, positions, velocities, VV,
                           dt, and Moliere below mixed_mol_fp64_r           */
};

/* per-atom tag bits (fibmd_gpu_set_tags) */
enum {
  FIBMD_TAG_FROZEN = 1u,   /* pinned to Xi with V = 0 each step (spec mode's
                              fixed bottom layers; ref mode uses xsides)      */
  FIBMD_TAG_THERMO = 2u,   /* member of the Berendsen layer (spec mode)       */
  FIBMD_TAG_REMOVED = 4u   /* sputtered and removed (spec mode); set by the
                              device, excluded from lists, forces, dynamics   */
};

/* reasons a fibmd_gpu_steps() call returned (bit set) */
enum {
  FIBMD_STOP_MAXSTEPS = 1, /* ran the requested number of steps              */
  FIBMD_STOP_DUMP = 2,     /* lt is an atm_out/res_out step: download + write */
  FIBMD_STOP_DONE = 4,     /* the TI loop ended: warm-up converged
                              (whichctrl 0) or time > impact*dti (1)          */
  FIBMD_STOP_REGIME = 8    /* calc_atm switched to the slow regime (ionrun 2) */
};

/*
 * Run parameters. fibmd_gpu_params_default() fills the potential constants
 * hard-coded in src/prms.f90:172-216 and the siga.in defaults shipped with
 * the reference (siga.in:1-53); the host overwrites what siga.in sets.
 */
typedef struct fibmd_params {
  int abi_version;           /* must be FIBMD_ABI_VERSION                      */
  int mode;                  /* FIBMD_MODE_*                                   */
  int precision;             /* FIBMD_PREC_*                                   */
  int Natm, Nsg, Nlj;        /* atoms; Si/Ge atoms (1..Nsg); ions (Nsg+1..)    */
  double Lb[3];              /* periodic box (m); z is 10x the slab            */

  /* Stillinger-Weber and Moliere constants (src/prms.f90:172-216, 433-480) */
  double A, B, psi, qsi, al, gamma;
  double lambdaSi, lambdaGe, epsSi, epsGe, sigmaSi, sigmaGe;
  double massSi, massGe, massGa;
  double ZSi, ZGe, ZGa;
  double Amol, Bmol, Cmol, alpha_mol, beta_mol, gamma_mol;
  double kB, eps0, ec, ao;
  double listfac;            /* list radius factor (1.1)                      */
  int Ntable;                /* 2-body table size (12000)                     */

  /* run control read from siga.in (src/prms.f90:223-275) */
  double Ts_i, Ts_r;         /* fast / slow regime time steps (s)             */
  double Ttar1;              /* thermostat target (K)                         */
  double ke_limit_1;         /* slow-regime switch threshold (eV)             */
  double Tau_i, Tau_r;       /* Berendsen time constants (s)                  */
  double Teps;               /* warm-up tolerance (K)                         */
  int ntlist_i, ntlist_r, atlist_i, atlist_r, dslist_i, dslist_r;
  int atm_out_i, atm_out_r, res_out;
  double outz[4], atomz[2], ionz, knockz;  /* in units of Lb(3)/10            */
  double sidewidth;          /* edge thermostat width (nm)                    */
  double dti;                /* time between impacts (s)                      */

  /* spec mode */
  double dt_max;             /* variable-dt cap (s), default 1 fs             */
  double dx_max;             /* max displacement per step (m), default 0.05 A */
  double tau_spec;           /* Berendsen constant of the thermo layer (s)    */
  double remove_z;           /* atoms above this z (m) are removed; <=0 off   */

  /* mixed precision */
  double mixed_mol_fp64_r;   /* Moliere pairs closer than this (m) stay fp64  */

  /* spec mode: list radius = interaction cutoff + list_skin (m) for the SW
     list (cutoff 0.999*a*sigma) and the Moliere list (2.5*sigma); 0 keeps
     the reference's radii (listfac 1.1); < 0 starts from 0.6 A. With a
     skin, the context also derives 0.75 and 1.35 times it and, in long
     step calls, re-times the three on the current state and keeps the
     fastest (options "skin_tune", "skin"). Spec mode always finds every
     Moliere pair (the reference's 27-cell stencil misses those beyond one
     cell). With remove_z > 0 (and remove_z + list radius < Lb(3)) spec mode
     treats z as an open axis: positions are not wrapped in z, the cell
     grid covers [0, remove_z + list radius) only, and an atom more than
     10 A below z = 0 (a transmitted ion) is removed like one above
     remove_z. */
  double list_skin;

  /* capacities; 0 = defaults */
  int max_sw_nbrs;           /* SW list slots per atom, default 48            */
  int max_mol_pairs;         /* full Moliere list entries, default
                                max(1500*Nlj, 65536) (the reference's MLlj is
                                1500*Nlj, src/si.f90:51)                      */
  int reserved[8];
} fibmd_params;

typedef struct fibmd_ctx fibmd_ctx;

/* Fill prms.f90's constants and siga.in's shipped defaults. */
int fibmd_gpu_params_default(fibmd_params* p);

/* Library / device information. Returns the ABI version. */
int fibmd_gpu_abi_version(void);
/* sizeof(fibmd_params) as compiled into the library, for FFI layout checks. */
int fibmd_gpu_params_size(void);

/* Create a context on the current CUDA device: sizes the cell grid and the
   list capacities (replaces init_nlist, src/si.f90:48-80) and builds the
   2-body table bit-identically to mktables (src/si.f90:575-597). */
int fibmd_gpu_create(const fibmd_params* p, fibmd_ctx** out);
void fibmd_gpu_destroy(fibmd_ctx* ctx);

/* Last error message of this context (or of the last failed create when ctx
   is NULL). Copies at most len-1 bytes plus NUL. */
int fibmd_gpu_last_error(const fibmd_ctx* ctx, char* buf, int len);

/* Upload the full atom state (replaces the host arrays of src/data.f90:19-24
   and src/prms.f90:43). X, V, F, Xi: (Natm,3) column-major; mass: (Natm);
   atype: (Natm) 1=Si 2=Ge 3=Ga; xsides: (Natm), >0 marks an atom pinned by
   freezsidesN (src/tools.f90:38-51). F may be NULL (zeros). */
int fibmd_gpu_upload(fibmd_ctx* ctx, const double* X, const double* V,
                     const double* F, const double* Xi, const double* mass,
                     const int* atype, const int* xsides);

/* Download the atom state (what updateroot gathers, src/par.f90:94-121).
   Any pointer may be NULL. */
int fibmd_gpu_download(fibmd_ctx* ctx, double* X, double* V, double* F);

/* Spec-mode per-atom tags (FIBMD_TAG_* bits), (Natm) entries. */
int fibmd_gpu_set_tags(fibmd_ctx* ctx, const uint32_t* tags);
/* The current tags, (Natm) entries: spec mode sets FIBMD_TAG_REMOVED on the
   device when an atom is removed (the reference's counterpart is the
   parking of sputtered atoms in frzsptrdatms, src/temp.f90:99-127, which
   leaves no mark); ref mode reports FIBMD_TAG_FROZEN for atoms pinned by
   xsides. */
int fibmd_gpu_get_tags(fibmd_ctx* ctx, uint32_t* tags);

/* The device side of writeatoms (src/out.f90:62-100): the columns of an
   extended-xyz frame computed on the GPU — x y z in Angstrom ((Natm,3)
   column-major) and the kinetic energy 0.5 m |v|^2 in eV (the reference's
   J->eV factor 6.252e18) — copied into host arrays (either may be NULL).
   fibmd_host_xyz_write (fibmd_host.h) then writes the frame on a background
   thread. */
int fibmd_gpu_xyz_frame(fibmd_ctx* ctx, double* xyz_A, double* ke_eV);

/* Overwrite one atom's position and velocity (1-based index). This is the
   device side of knock (src/knock.f90:21-55): the host draws the ion's start
   point and velocity and sends them here. */
int fibmd_gpu_set_atom(fibmd_ctx* ctx, int i, const double x[3],
                       const double v[3]);

/* Set the impact counter (module variable `impact`, src/prms.f90:24): atoms
   with index > Nsg+impact are unfired ions and are skipped by the force
   (src/si.f90:415,428,457). */
int fibmd_gpu_set_impact(fibmd_ctx* ctx, int impact);

/* Switch regime (ionrun, src/prms.f90:563-584): tic 1 = fast (Ts_i,
   ntlist_i, atlist_i, Tau_i, dslist_i, atm_out_i), tic 2 = slow. Also sets
   the calc_atm latch atom_is_fast = (tic == 1). */
int fibmd_gpu_ionrun(fibmd_ctx* ctx, int tic);

/* Override the Berendsen constant Tau (tint sets Tau = 1e-14 s for the
   warm-up, src/timeint.f90:85-88). */
int fibmd_gpu_set_tau(fibmd_ctx* ctx, double tau);

/* Build the neighbour lists at the current device positions (replaces
   si_nlist -> si_nlistG + chainlist, src/si.f90:87-276, src/nlist.f90:20-66). */
int fibmd_gpu_nlist(fibmd_ctx* ctx);

/* Number of list entries: full SW pairs, full Moliere pairs, and the
   connected SW triplets the reference would store in nlist3. Any pointer
   may be NULL. */
int fibmd_gpu_list_counts(fibmd_ctx* ctx, long long* n_sw_full,
                          long long* n_mol_full, long long* n_triplets);

/* Export the half lists the reference keeps after dropping j<i entries
   (src/si.f90:234-260) as sorted 1-based (i,j) pairs, i<j. kind 0 = SW list
   (nlist2), 1 = Moliere list (nlistlj). ij has room for 2*cap ints; *n
   receives the pair count (which may exceed cap: nothing past cap is
   written). */
int fibmd_gpu_get_pairs(fibmd_ctx* ctx, int kind, int* n, int* ij, int cap);

/* Export the connected-triplet set of the SW list graph, each triple sorted
   (min,mid,max) and 1-based, in lexicographic order: the set si_nlistG
   stores in nlist3 (src/si.f90:191-232). ijk has room for 3*cap ints. */
int fibmd_gpu_get_triplets(fibmd_ctx* ctx, long long* n, int* ijk,
                           long long cap);

/* Force at the current device positions with the current lists; the result
   becomes the state's F (tint's `call si_force(X,F,lt)`,
   src/timeint.f90:69). F_out (Natm,3) may be NULL. If u_out or Utot is
   non-NULL the per-atom and total potential energy of si_potential
   (src/si.f90:278-380) are computed too. */
int fibmd_gpu_force(fibmd_ctx* ctx, double* F_out, double* u_out,
                    double* Utot);

/* Run the TI loop (src/timeint.f90:123-155) over onestep
   (src/timeint.f90:158-242) on the device for at most max_steps steps.
   whichctrl: 0 warm-up (global Berendsen until |T-Ttar| <= Teps),
   1 impact (until time > impact*dti), 2 free run (max_steps steps).
   lt, time, temp are the caller's loop variables (in/out). Returns early at
   an atm_out/res_out dump step (whichctrl > 0). *reason receives
   FIBMD_STOP_* bits. */
int fibmd_gpu_steps(fibmd_ctx* ctx, int whichctrl, long long max_steps,
                    long long* lt, double* time, double* temp, int* reason);

/* temperature (src/temp.f90:183-205) of the device velocities. */
int fibmd_gpu_temperature(fibmd_ctx* ctx, double* T);

/* Current time step Ts (s) and regime (1 fast, 2 slow). */
int fibmd_gpu_regime(fibmd_ctx* ctx, double* Ts, int* tic);

/* Phase timers since the last reset, in seconds, and call counts, as the
   reference's calc_time report (src/timeint.f90:302-331): at = parking and
   redistribution, nt = neighbour lists, ds = calc_atm, f = force. */
int fibmd_gpu_timers(fibmd_ctx* ctx, double* at, double* nt, double* ds,
                     double* f, long long* counts4, int reset);

/* Device time (s) and call counts per phase since the last reset, from
   CUDA events on the context's stream: [0] parking (at), [1] neighbour
   lists (nt), [2] calc_atm (ds), [3] force phase (f), [4] main force kernel
   (with "kernel_timing"), [5] thermostat + drift, [6] kick. */
int fibmd_gpu_phase_times(fibmd_ctx* ctx, double* seconds7, long long* counts7,
                          int reset);

/* Options: "timers" (phase timers of fibmd_gpu_timers, default 1),
   "kernel_timing" (CUDA events around every launch of the main force
   kernel, default 0), "graph" (spec mode runs step pairs as one CUDA
   graph launch with device-side rebuild decisions, default 1; phase and
   kernel timers see only the steps run outside the graph), "autotune"
   (mixed precision: before a dose, and in the spec-mode steps of a graph
   run 1000 steps after an upload or a change of path and then after
   doubling intervals up to 8000 steps, time the binary32 force paths (each
   stage with 128 or 64 centres per block, and eight lanes per centre) on
   the current state and keep the fastest, default 1) and "stage" (the
   binary32 force path: 6 or 10 staged leg candidates per centre with one thread per centre, or 1 for
   eight lanes per centre, the faster on small systems; setting it turns
   "autotune" off) and "pdl" (default 0; 1: the step loop's kernels are
   launched as programmatic dependents of the kernel before them, so each
   is dispatched during its predecessor's tail and waits in hardware for its
   completion; a graph that cannot be captured so is captured with plain
   launches and the option reads 0 afterwards), "fuse" (default 1: where
   every chunk of 256 atoms gets a block in one resident wave, the graph
   runs each step's kick and the next step's drift as one persistent
   kernel whose blocks meet at a grid barrier with a bounded wait; reads 1
   where that is in use; a wait
   that gives up ends the call with FIBMD_ETIMEOUT and leaves the state
   invalid until the next upload) and "kd_grid" (that kernel's grid; 0, the
   default, is the number of its blocks the device holds at once, which
   every wait relies on; a larger value makes the waits give up, a hook for
   testing the time-out), "rebuild_rule" (spec mode, per replica in a
   batch: default 1, the lists are rebuilt once the two largest
   displacements since the last build add up to the skin, those under a
   quarter of it counted at that bound, and in a batch with them those of
   the replicas whose sum has reached half the skin; 0, once any atom's
   displacement reaches half the skin, in a batch with those that moved a
   quarter of it), "skin_tune" (default 1: in spec-mode calls of at
   least 2000 steps, before every 5000 steps, each candidate list skin runs
   one step pair and then 20 timed pairs of the graph step loop, and the
   fastest per step is kept; the trial steps are steps of the run, and the
   trajectory does not depend on the skin since the lists stay complete),
   "skin" (reads the skin in use in Angstrom; set to one of the candidates
   it fixes the skin: the lists are rebuilt at the next step) and
   "skin_candidates" (read only: how many), "force_block" (centres per
   block of the one-thread-per-centre binary32 force kernel, 128 or 64;
   "autotune" times both with each stage; setting it turns "autotune" off)
   and "build_block" (atoms per block of the pair-list build, 64, 128 or
   256, re-timed with the skin; setting it fixes it), "reactions" (mixed
   precision with max_sw_nbrs <= 64 only; default 0: each centre of the
   one-thread-per-centre kernel adds its force and the 3-body reactions on
   its legs by binary64 atomics; 1: it stores them and a second pass
   gathers them per atom, summing in binary64 on the SM, which on this part
   is slower than the atomics; FIBMD_EINVAL where the context holds no
   buffers for it) and "heavy_if" (default 0; 1: the step graph runs the
   many-leg kernel in an IF node that the force kernel opens when it finds
   a centre with more legs than its stage, which skips the launch in steps
   without such centres but costs more per step than the launch it saves). */
int fibmd_gpu_set_option(fibmd_ctx* ctx, const char* key, double value);
/* The current value of an option ("stage" reads the force path in use,
   which "autotune" changes as the run goes). */
int fibmd_gpu_get_option(fibmd_ctx* ctx, const char* key, double* value);

/* Total device time (s) and number of launches of the main force kernel
   since the last reset, from the events of the "kernel_timing" option. */
int fibmd_gpu_kernel_time(fibmd_ctx* ctx, double* force_kernel_s,
                          long long* launches, int reset);

/* Measured FMA throughput of the current device in TFLOP/s (an FMA is 2
   flops): independent binary64 and binary32 FMA chains over every SM. A
   diagnostic for reporting the force kernel against its arithmetic pipe. */
int fibmd_gpu_pipe_peaks(double* fp64_tflops, double* fp32_tflops);

/* Work counters: [0] active SW pairs (i<j with a non-zero table entry),
   [1] non-zero 3-body angle terms, [2] Moliere pairs evaluated and [3]
   stale-list angle terms added by the correction pass, all of the last
   fibmd_gpu_force call; [4] neighbour-list builds since creation; [5]
   centres of the last force evaluation with more active legs than the
   per-thread stage holds (evaluated by the warp-per-centre path). */
int fibmd_gpu_work_counters(fibmd_ctx* ctx, long long counts[6]);

/* Virial of the current positions, sum over interactions of r (x) f in J
   (W[0..5] = xx, yy, zz, xy, xz, yz): for each pair the separation from
   partner to atom times the force on the atom, for each 3-body term minus
   each leg's separation from the centre times the force on that leg; the
   Moliere pairs of fired ions included. Evaluated in binary64 from the
   current lists in either precision (reference mode's stale-list terms
   excluded). w_atom (Natm x 6, column-major, may be NULL): per atom, the
   terms of which it is the centre and half of each of its pairs. The
   reference computes no virial (src/stats.f90:34-81 reports PE, KE and
   momentum); this is the per-atom virial the hot path's specification
   adds to forces and energies. */
int fibmd_gpu_virial(fibmd_ctx* ctx, double W[6], double* w_atom);

/* CUDA stream the context orders its work on (cudaStream_t as void*). */
void* fibmd_gpu_stream(fibmd_ctx* ctx);

/* Force of one configuration with no device allocation. This entry point
   has no counterpart in the reference. It is for hosts that cannot ask the
   driver for device memory when they need a force: hosts whose device
   memory is handed out by a pool manager or an embedding runtime that
   forbids driver allocations after start-up, and drivers that must keep a
   fixed device footprint on a shared GPU. It computes si_force in binary64
   with the reference's semantics (lists built from X, table SW 2-body,
   Moliere for fired ions, SW 3-body) and writes F.
   X_dev, F_dev: device (Natm,3) column-major; atype_dev: device (Natm) with
   values 1..3; impact: atoms with index > Nsg+impact are unfired ions;
   stream: a cudaStream_t (NULL for the default stream); returns after
   synchronising it.
   All scratch memory (4.2 MB: cells, lists, shadows, scalars, the 2-body
   table) is one fixed device array inside the library, held by every device
   that loads it until the process exits. Limits: Natm <= 8192, at most
   65536 cells in the reference's cell grid, Ntable <= 12000,
   max_sw_nbrs <= 48, max_mol_pairs <= 65536, precision FP64; beyond them
   the call returns FIBMD_EINVAL and fibmd_gpu_last_error(NULL, ...) says
   which limit. The first call on a device looks up the array's device
   address and uploads the 2-body table: make that first call before any
   stream capture. Every call shares the array; calls that overlap on the
   GPU (other streams or host threads) race, so serialise them. */
int fibmd_gpu_force_noalloc(const fibmd_params* p, const double* X_dev,
                            const int* atype_dev, int impact, double* F_dev,
                            void* stream);

/* A dose of successive impacts on one spec-mode system without host round
   trips (the device side of knock, src/knock.f90:21-55, repeated): impact k
   brings atom ion_atoms[k] (1-based; a pre-allocated ion kept removed, for
   example tagged FIBMD_TAG_REMOVED, until its turn) to position x (nimp,3
   column-major, m) with velocity v (m/s), then runs `steps` steps (rounded
   up to even) and a relaxation of relax_s seconds of simulated time (<= 0:
   none). All impacts are enqueued before the first finishes. Outputs, nimp
   entries each (any may be NULL): lattice atoms removed (sputtered) and ions
   removed (backscattered) so far, the simulated time, and the MD steps this
   call has run, after each impact.
   Needs lists built and the graph step loop (fibmd_gpu_set_option "graph"). */
int fibmd_gpu_dose(fibmd_ctx* ctx, int nimp, const int* ion_atoms, const double* x,
                   const double* v, long long steps, double relax_s, int* removed_after,
                   int* ions_removed_after, double* time_after, long long* steps_after);

/* ---- batched ensemble (spec mode) -----------------------------------------
   Independent impacts advanced together: each replica has its own box,
   atoms, cell grid, variable dt, thermostat factor and removal count; the
   kernels of one step handle every replica's atoms at once. There is no
   counterpart in the reference, which runs one impact per process. */
typedef struct fibmd_replica {
  int natm;          /* atoms of the replica: lattice atoms first, then ions */
  int nsg;           /* lattice atoms (atype 1 or 2)                         */
  double Lb[3];      /* its periodic box (m); z is open when remove_z > 0    */
  double remove_z;   /* removal height (m), <= 0: none                       */
  int reserved[4];
} fibmd_replica;

/* Create a batch context from shared physics p (mode must be
   FIBMD_MODE_SPEC; p's Natm, Nsg, Nlj, Lb and remove_z are ignored) and
   nrep replicas. The replicas' atoms are concatenated, each starting at a
   multiple of 256; the slots between replicas are padding. Every per-atom
   array of upload/download/set_tags then has the padded length
   offsets[nrep] (fibmd_gpu_batch_layout); padding slots take any position,
   mass > 0 and atype 1, and are kept as removed atoms. Lists, forces and
   steps run as for a single system; fibmd_gpu_steps' time argument is the
   start time of every replica and returns replica 0's. */
int fibmd_gpu_batch_create(const fibmd_params* p, int nrep, const fibmd_replica* reps,
                           fibmd_ctx** out);
/* The outcome of each impact (a batch's replicas, or a single system as one
   replica), computed on the device, after the statistics of temp.f90:70-127
   that the reference writes per impact: lattice atoms removed (sputtered),
   lattice atoms farther than displaced_m from their initial site (minimum
   image in x and y; removed atoms left out), and the depth of the replica's
   first ion below surface_z[r] (m; NaN when the ion is above it or
   removed). surface_z and the outputs have one entry per replica; any
   output may be NULL. */
int fibmd_gpu_impact_stats(fibmd_ctx* ctx, const double* surface_z, double displaced_m,
                           int* sputtered, int* displaced, double* ion_depth);
/* Replica count and, if offsets is not NULL, the first atom of each replica
   in offsets[0..nrep-1] and the padded atom count in offsets[nrep]. */
int fibmd_gpu_batch_layout(fibmd_ctx* ctx, int* nrep, int* offsets);
/* Per-replica simulated time (s), current step (s) and count of removed
   (sputtered) atoms; any pointer may be NULL, else nrep entries. */
int fibmd_gpu_batch_scalars(fibmd_ctx* ctx, double* time, double* dt, int* removed);

#ifdef __cplusplus
}
#endif
#endif /* FIBMD_GPU_H */
