// fibmd_internal.cuh — device-side data layout and helpers shared by the
// kernels of the FIB_MD GB300 backend.
//
// HBM layout (one context, N atoms, 0-based index = Fortran index - 1):
//   pos, vel, frc, frc_new, xi : double4_32a[N]  (x, y, z, unused)
//   posq      : int4[N]   fixed-point positions, x = round(x/Lb * 2^32) mod
//               2^32, w = atype | (flags & 0xff) << 8 | replica << 16
//               (flags bits 16..31 hold the atom's replica, 0 for a single
//               system). Differences of two fixed-point
//               coordinates wrap modulo 2^32, which is the minimum image, and
//               convert to binary32 with the precision of the separation
//               itself (not of the absolute coordinate).
//   mass      : double[N];  atype : int8[N];  flags : uint32[N]
//   cells     : cell_start[ncell+1], cell_atoms[N] and posq_cell[N] (counting
//               sort by cell; posq_cell streams a cell's candidates)
//   nbr_sw    : int[max_sw * N], slot-major (nbr_sw[k*N + i]) so a warp of
//               consecutive centres reads one coalesced row per slot
//   mol_pairs : int2[cap] full Moliere pair list (both orders)
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fibmd_gpu.h"

namespace fibmd {

constexpr int kMaxLegs = 12;       // active 3-body legs held per centre
constexpr int kRedThreads = 256;   // threads of reduction kernels
constexpr int kMaxRedBlocks = 16384;  // row stride of the reduction partials
constexpr int kKickThreads = 256;  // spec kick block; replicas start at multiples
// Binary32 SW legs with exp(gamma/(u-a)) below this are dropped: an angle
// term is at most lambda*eps*E_a*E_b (~45 eV E_a E_b), so such a leg moves a
// force by less than 1e-8 eV/A, far below the binary32 arithmetic's own
// error, and second neighbours squeezed inside the cutoff by thermal motion
// stop counting as legs.
constexpr float kLegEmin = 1e-12f;

enum : uint32_t {
  FL_FROZEN = 1u,   // xsides > 0 (ref) / FIBMD_TAG_FROZEN (spec)
  FL_THERMO = 2u,   // spec-mode thermostat layer
  FL_REMOVED = 4u,  // spec-mode sputtered and removed
};

// Box and cell geometry of one replica. A context holds one system
// (replica 0) or a batch of independent replicas, each with its own box,
// cell grid (a slice of the context's cells) and atom range; kernels that
// handle atoms of any replica read their geometry here.
struct Geo {
  double Lb[3], iLb[3], hcell[3];
  double qscale[3];   // 2^32 / Lb
  double inv_hz;      // 1 / cell height in z (open z axis)
  double remove_z;    // spec mode: atoms above are removed (<= 0: never)
  double remove_zlo;  // spec mode, open z axis: atoms below are removed too
  float qinvA[3];     // Lb / 2^32 in Angstrom
  int nc[3];
  int wrap[3];        // periodic cell stencil per axis (the reference: Nc > 2)
  int zcompact;       // spec mode: open z axis, cell grid over [0, zext)
  int mol_reach;      // cells scanned for Moliere pairs (spec mode)
  int cell_off, ncell;      // this replica's cells in the context's grid
  int atom_begin, atom_end;  // its atoms
  int blk_begin, blk_end;    // its kick blocks (kKickThreads atoms each)
};

__device__ __forceinline__ int rep_of_w(int w) { return (int)((unsigned)w >> 16); }
__device__ __forceinline__ int rep_of_flags(uint32_t fl) { return (int)(fl >> 16); }
__device__ __forceinline__ int posq_w(int8_t type, uint32_t fl) {
  return (int)(uint8_t)type | (int)((fl & 0xffu) << 8) | (int)(fl & 0xffff0000u);
}

// Derived constants handed to every kernel by value.
struct DevParams {
  int N, Nsg, nfired;  // atoms with index >= nfired are unfired ions
  int uniform;         // every lattice atom is Si (type 1): set at upload
  int nrep;            // replicas (1: a single system)
  int nion;            // ions (entries of DevState::ion_list)
  int mode, precision;
  int max_sw;
  int mol_cap;
  int Ntable, tab_last;  // tab_last: last 0-based index with a non-zero entry
  int nc[3];
  int ncell;
  int wrap[3];      // periodic cell stencil per axis (the reference: Nc > 2)
  int zcompact;     // spec mode: cell grid in z covers [0, zext) only
  double inv_hz;    //            1 / cell height in z
  int mol_reach;    // cells scanned for Moliere pairs (1: the reference's
                    // 27-cell stencil; spec mode: enough for the radius)
  double Lb[3], iLb[3], hcell[3];
  double qscale[3];      // 2^32 / Lb
  float qinvA[3];        // Lb / 2^32 in Angstrom
  double rv2, rv2lj, rlj2;
  float pre_sw2A, pre_mol2A;   // binary32 prefilter radii^2 (A^2), widened
  float acc_sw2A, acc_mol2A;   // binary32 accept radii^2 (A^2), narrowed
  float pre3A2;                // prefilter for active SW legs (A^2)
  float pre3mA2;               // binary32 path: u < a - gamma/110, beyond which
                               // every SW exponential underflows (A^2)
  float pre3lA2;               // binary32 legs: exp(gamma/(u-a)) > kLegEmin (A^2)
  // Stillinger-Weber (types 1, 2 -> index 0, 1)
  double al, gam, cut3, thrd, A, B, psi, qsi;
  double eps[2][2], isig[2][2], leps[2][2][2], epssig[2][2];
  // Moliere (types 1..3 -> index 0..2)
  double Zmol[3], aamol[3][3], ie0, ec;
  double Amol, Bmol, Cmol, amol, bmol, gmol;
  // 2-body table
  double umax;
  // stale-list bookkeeping
  double disp_fast2;  // squared displacement (m^2) that marks an atom fast
  float disp_fastA2;  // the same in A^2
  // spec-mode rebuild rule (per replica): 0, any atom displaced half the
  // skin; 1 (pair_rule), the two largest displacements together reaching the
  // skin, atoms below disp_lowA2 counted at that bound
  int pair_rule;
  float disp_skinA;   // the skin (A, with the 1 % margin of disp_fast2)
  float disp_lowA2;   // squared reporting bound of the pair rule (A^2)
  // mixed precision, reduced units (A, eV)
  float epsA[2][2], sigA[2][2], lepsA[2][2][2];
  float isigA[2][2], epssigA[2][2];  // 1/sigma (1/A), eps/sigma (eV/A)
  float molKA[3][3];       // ie0*Zi*Zj*ec*ec in eV*A
  float amolA[3][3];       // screening length in A
  double f_evA_to_N;       // eV/A -> N
  double e_eV_to_J;        // eV -> J
  float mol_fp64_rA;       // Moliere pairs below this stay binary64 (A)
  // integrator geometry (siga.in values resolved once per context)
  double kB;
  double side_sw, side_zlo, side_zhi;        // controlsidetemp band (m)
  double park_o[4], park_a[2];               // outz(k)*Lb3/10, atomz(k)*Lb3/10
  double park_al[2], park_ah[2];             // (atomz(k) -/+ 0.3)*Lb3/10
  double park_il, park_ih;                   // (ionz -/+ 0.3)*Lb3/10
  // spec mode
  double remove_z, dt_max, dx_max, tau_spec;
};

// Device scalars written by reductions and read by later kernels or the
// host (through a pinned mirror).
struct DevScalars {
  double side_sum;     // controlsidetemp: sum m v^2 over edge atoms
  double side_cnt;     //                  number of edge atoms
  double side_s;       //                  its Berendsen factor (1 if none)
  double thermo_s;     // spec: Berendsen factor of the thermostat layer
  double temp;         // temperature() of the current velocities
  double ke_max;       // calc_atm: max 0.5 m v^2 / ec
  double vmax2;        // spec: max |v|^2
  double dt;           // spec: current step
  double half_dt;      //       dt / 2 (kick)
  double half_dt2;     //       dt^2 / 2 (drift)
  double dt_next;      // spec: step chosen from this step's velocities
  double thermo_sum, thermo_cnt;  // spec thermostat layer
  double ekin, epot;   // energies (J)
  double time;         // spec: simulated time
  double disp_max2;    // spec: max squared displacement since build
  int fast_count;
  int mol_count;
  int heavy_count;
  int overflow_sw;
  int sw_needed;       // SW slots the most crowded atom needed (overflow)
  int overflow_mol;
  int table_err;
  int cell_oob;
  int nan_flag;
  int need_rebuild;
  int rep_rebuild;     // spec batch: this replica is due a rebuild (the rule)
  int rep_soon;        //             ... halfway there
  int rebuild_all;     // spec batch: the next rebuild covers every replica
                       // (a skin switch, an injection)
  int removed_count;   // spec: lattice atoms removed (sputtered)
  int ions_removed;    //       ions removed (backscattered)
  unsigned kd_gen;     // fused kick-drift: barrier generation
  unsigned kd_reps;    //                   replicas finalized this step
  int kd_cont;         //                   the step loop goes on (drift)
  int kd_timeout;      //                   a barrier wait gave up
  unsigned long long rebuilds;  // list builds since creation
  unsigned long long acc_vmax2;  // spec kick: running max |v|^2 (bits), sum m v^2
  double acc_tsum;               //            and count of the thermostat layer,
  int acc_tcnt;                  //            cleared by the replica's last chunk
  unsigned disp_max;     // pair rule: the step's largest reported |d|^2 (float
                         // bits), cleared by the kick's last chunk
  unsigned int ticket[8];
  unsigned long long counters[4];
};

// Step-loop control of the spec-mode graph: step pairs left, and a time at
// which the loop stops early (a relaxation of given length).
struct LoopCtl {
  long long pairs;
  double t_stop;
  long long pairs_run;  // step pairs run since the context was created
};

// One impact of a dose: the pre-allocated ion atom and its start state.
struct Impact {
  int atom;
  double x[3], v[3];
};

struct DevState {
  int N;
  double4_32a* pos;
  double4_32a* vel;
  double4_32a* frc;      // F (previous step)
  double4_32a* frc_new;  // Fp (this step)
  double4_32a* xi;
  int4* posq;
  int4* posq_build;  // fixed-point positions at the last list build
  double* mass;
  double* inv_mass;
  int8_t* atype;
  uint32_t* flags;
  // cells
  int* cell_count;
  int* cell_start;
  int* cell_atoms;
  int4* posq_cell;   // posq in cell order (filled with cell_atoms)
  int* atom_cell;
  int* scan_blocks;
  // lists
  int* nbr_sw;
  int* n_sw;
  int* sw_extra;     // per atom: SW partners beyond the max_sw slots (overflow)
  int2* mol_pairs;
  // binary32 path with stored reactions (allocated for mixed precision with
  // at most kReactMaxList list slots): rev_sw holds, per list entry (i, k),
  // the slot of i in the partner's list; legpos[i] the list positions of the
  // centre's staged legs (6 bits each, leg count in bits 60-63, kLegsHeavy
  // for a centre of the many-leg kernel); react[a * N + i] the 3-body
  // reaction the centre exerts on its leg a (eV/A); fown[i] the centre's own
  // force from its terms (eV/A)
  int* rev_sw;
  unsigned long long* legpos;
  float4* react;
  float4* fown;
  // stale-list and heavy-centre work lists
  uint8_t* fast_flag;
  int* fast_list;
  int* heavy_list;
  // 2-body table
  const double* tab;
  const double* tabu;
  // energy
  double* epot;
  // reductions
  double* partials;
  DevScalars* sc;    // one per replica; context-wide fields live in sc[0]
  // replicas
  const Geo* geo;    // nrep entries
  const int* ion_list;  // the ions (atype 3), ascending
};

// ---- programmatic dependent launch -----------------------------------------
// A kernel launched with the programmatic stream-serialization attribute
// (launch_k with pdl = true) may be dispatched while its predecessor in the
// stream still runs. pdl_wait() returns once the predecessor has completed
// and its writes are visible (a hardware wait, no spin; a no-op for a kernel
// launched without the attribute), so every kernel of the step loop calls it
// before its first load: a predecessor completes only after its own
// predecessor has, so completion is transitive along the chain.
// pdl_trigger() lets the successor's blocks be dispatched onto SMs as this
// grid's blocks retire, which hides the successor's launch and ramp-up
// behind this grid's tail.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// ---- small device helpers ------------------------------------------------

__device__ __forceinline__ int type_index(int8_t t) { return t - 1; }

// The reference's minimum image, X(i)-X(j) - NINT((X(i)-X(j))*iLb)*Lb,
// with each operation rounded separately (no FMA), so neighbour decisions
// reproduce binary64 host arithmetic bit for bit.
__device__ __forceinline__ double min_image_exact(double xi, double xj,
                                                  double iLb, double Lb) {
  double d = __dsub_rn(xi, xj);
  double n = round(__dmul_rn(d, iLb));
  return __dsub_rn(d, __dmul_rn(n, Lb));
}

// Same separation for force arithmetic (contraction allowed).
__device__ __forceinline__ double min_image(double xi, double xj, double iLb,
                                            double Lb) {
  double d = xi - xj;
  return d - round(d * iLb) * Lb;
}

// The reference's rebox, MOD(x + 2 Lb, Lb). Fortran's MOD of reals is
// exact (fmod); for a = x + 2Lb in [Lb, 3Lb) the subtraction of Lb or 2Lb
// is exact too (Sterbenz), so this returns fmod's bits at a fraction of its
// binary64 instructions and falls back to fmod outside that range.
__device__ __forceinline__ double rebox1(double x, double L) {
  const double a = x + 2.0 * L;
  const double L2 = 2.0 * L;
  if (a >= L2) {
    const double r = a - L2;
    if (r < L) return r;
  } else if (a >= L) {
    return a - L;
  }
  return fmod(a, L);
}

// round(x * qscale) mod 2^32 with one binary64 FMA: adding 1.5 * 2^52 puts
// the nearest integer (ties to even) into the low mantissa bits, valid for
// |x * qscale| < 2^51.
__device__ __forceinline__ unsigned int fixq(double x, double qscale) {
  return (unsigned int)__double_as_longlong(fma(x, qscale, 6755399441055744.0));
}

// The same integer without the wrap: round(x * qscale) as a signed 64-bit
// value, whose high bits say how many boxes x lies away from [0, Lb).
__device__ __forceinline__ long long fixq64(double x, double qscale) {
  return __double_as_longlong(fma(x, qscale, 6755399441055744.0)) - 0x4338000000000000ll;
}

// binary32 separation (Angstrom) of two fixed-point positions.
__device__ __forceinline__ float3 qsep(const int4& a, const int4& b,
                                       const float qinvA[3]) {
  float3 d;
  d.x = (float)(int)((unsigned)a.x - (unsigned)b.x) * qinvA[0];
  d.y = (float)(int)((unsigned)a.y - (unsigned)b.y) * qinvA[1];
  d.z = (float)(int)((unsigned)a.z - (unsigned)b.z) * qinvA[2];
  return d;
}

__device__ __forceinline__ void atomic_add3(double4_32a* f, int i, double x,
                                            double y, double z) {
  atomicAdd(&f[i].x, x);
  atomicAdd(&f[i].y, y);
  atomicAdd(&f[i].z, z);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block-wide sum of n doubles per thread (kRedThreads threads). Result valid
// in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV]) {
  __shared__ double sh[NV][kRedThreads / 32];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; q++) v[q] = warp_sum(v[q]);
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NV; q++) sh[q][w] = v[q];
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int q = 0; q < NV; q++) {
      double t = lane < (kRedThreads / 32) ? sh[q][lane] : 0.0;
      v[q] = warp_sum(t);
    }
  }
  __syncthreads();
}

__device__ __forceinline__ double block_max(double v) {
  __shared__ double sh[kRedThreads / 32];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_max(v);
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    double t = lane < (kRedThreads / 32) ? sh[lane] : -1.0e300;
    v = warp_max(t);
  }
  __syncthreads();
  return v;
}

// Deterministic grid reduction: every block stores its partial(s); the last
// block to finish (ticket) sums them in block order. Returns true in thread 0
// of the last block, with the totals in out[].
template <int NV, bool MAXOP>
__device__ __forceinline__ bool grid_finish(double (&v)[NV], double* partials,
                                            unsigned int* ticket) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NV; q++) partials[q * kMaxRedBlocks + blockIdx.x] = v[q];
    __threadfence();
    unsigned int t = atomicAdd(ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double acc[NV];
#pragma unroll
  for (int q = 0; q < NV; q++) acc[q] = MAXOP ? -1.0e300 : 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
#pragma unroll
    for (int q = 0; q < NV; q++) {
      double x = ((volatile double*)partials)[q * kMaxRedBlocks + b];
      acc[q] = MAXOP ? fmax(acc[q], x) : acc[q] + x;
    }
  if (MAXOP) {
#pragma unroll
    for (int q = 0; q < NV; q++) acc[q] = block_max(acc[q]);
  } else {
    block_sum<NV>(acc);
  }
#pragma unroll
  for (int q = 0; q < NV; q++) v[q] = acc[q];
  if (threadIdx.x == 0) *ticket = 0u;
  return threadIdx.x == 0;
}

// ---- host-side parameter derivation (fibmd_capi.cu) ------------------------
// Records the message fibmd_gpu_last_error(NULL, ...) returns (no heap use).
void set_noctx_error(const char* msg);
// mktables into caller buffers of Ntable + 2 entries.
void build_ref_table(const fibmd_params& p, double* tab, double* tabu, double* umax,
                     int* last_nz);
// Box and cell geometry of one replica with box Lb and removal height
// remove_z (the list radii and mode come from p); allocates nothing.
int derive_geo(const fibmd_params& p, const double Lb[3], double remove_z, Geo& G, char* err,
               int errlen);
// init_nlist/setupSiGe/setupMol constants for the kernels, and the
// geometry G of the single system p describes; allocates nothing.
int derive_dev_params(const fibmd_params& p, int impact, double umax, int tab_last,
                      DevParams& P, Geo& G, char* err, int errlen);

// ---- launchers (defined in the .cu files) --------------------------------
// The binary32 force path, chosen per context at run time by timing each
// on the current state: one thread per centre with kStageSmall or
// kStageLarge staged candidates (a crystal at 300 K has 4 legs, rarely more
// than 6, and the small stage leaves more resident warps; damaged slabs, a
// batch of small cascades, have many centres beyond it, which the many-leg
// kernel then takes), or eight lanes per centre for every centre
// (kStageGroup, the "stage" value 1: one kernel, faster on systems too
// small to fill the GPU one thread per centre).
constexpr int kStageSmall = 6;
constexpr int kStageLarge = 10;
constexpr int kStageGroup = 1;
constexpr int kReactMaxList = 64;  // list slots addressable by legpos's 6-bit fields
constexpr unsigned long long kLegsHeavy = 15;  // legpos count code of a many-leg centre

struct Launch {
  cudaStream_t stream;
  int sms;
  bool pdl = false;               // launch the step loop's kernels with
                                  // programmatic dependent launch
  cudaEvent_t force_a = nullptr;  // recorded around the main force kernel
  cudaEvent_t force_b = nullptr;  // when kernel timing is on
  int stage = kStageSmall;        // binary32 force kernel: staged candidates
                                  // per centre (kStageSmall or kStageLarge)
  int force_block = 128;          // its centres per block (64 or 128)
  int build_block = 128;          // atoms per block of the pair-list build
                                  // (64, 128 or 256)
  bool react = false;             // binary32 path: reactions stored per leg
                                  // and gathered per atom (no force atomics
                                  // from the centres of the main kernel)
  bool heavy_if = false;          // launch_force leaves out the many-leg
                                  // kernel (the caller adds it in an IF node
                                  // whose condition heavy_handle the main
                                  // kernel sets when it finds such a centre)
  cudaGraphConditionalHandle heavy_handle = 0;
};

// A kernel launch, with the programmatic stream-serialization attribute when
// pdl is set (the kernel must call pdl_wait() before its first load).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                            cudaStream_t s, bool pdl, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = pdl ? at : nullptr;
  cfg.numAttrs = pdl ? 1u : 0u;
  return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

// fibmd_nlist.cu
cudaError_t launch_update_posq(const Launch& L, const DevParams& P, const DevState& S);
// rebuild_from_flag: 0 builds every list; 1 only if need_rebuild is set;
// 2 as 1, and in a spec-mode batch only the replicas whose atoms moved half
// the skin (rep_rebuild) unless rebuild_all is set: the others keep their
// SW lists (the Moliere list and the cells are rebuilt for all)
cudaError_t launch_build_lists(const Launch& L, const DevParams& P, const DevState& S,
                               int rebuild_from_flag);
cudaError_t launch_count_triplets(const Launch& L, const DevParams& P, const DevState& S,
                                  unsigned long long* d_count, int3* out, long long cap);
// fibmd_force.cu
// spec_step: inside the spec-mode step, where the drift has reset the force
// counters and the kick has zeroed the accumulation buffer
cudaError_t launch_force(const Launch& L, const DevParams& P, const DevState& S,
                         bool energy, bool count, bool spec_step = false);
// the many-leg kernel alone (forces, no energy), for the step graph's IF node
cudaError_t launch_force_heavy(const Launch& L, const DevParams& P, const DevState& S);
// the virial in binary64: d_tot (6 doubles) and, if given, d_atom (6 x N,
// component-major)
cudaError_t launch_virial(const Launch& L, const DevParams& P, const DevState& S,
                          double* d_atom, double* d_tot);
// fibmd_integrate.cu
cudaError_t launch_side_reduce(const Launch& L, const DevParams& P, const DevState& S,
                               double Ts, double Tau, double Ttar);
cudaError_t launch_adjust_and_temp(const Launch& L, const DevParams& P, const DevState& S,
                                   double Ts, double Tau, double Ttar);
cudaError_t launch_drift(const Launch& L, const DevParams& P, const DevState& S, double Ts,
                         double Tau, double Ttar, int side_thermo);
cudaError_t launch_park(const Launch& L, const DevParams& P, const DevState& S);
cudaError_t launch_kick(const Launch& L, const DevParams& P, const DevState& S, double Ts);
cudaError_t launch_temperature(const Launch& L, const DevParams& P, const DevState& S);
cudaError_t launch_ke_max(const Launch& L, const DevParams& P, const DevState& S);
cudaError_t launch_pack(const Launch& L, int N, double4_32a* dst, const double* src_cm);
cudaError_t launch_unpack(const Launch& L, int N, const double4_32a* src, double* dst_cm);
cudaError_t launch_track_all(const Launch& L, const DevParams& P, const DevState& S);
cudaError_t launch_energy_sum(const Launch& L, const DevParams& P, const DevState& S);
// cond (in a captured graph): the IF handle the rebuild hangs on
// pdl_first: the drift may itself be launched as a programmatic dependent of
// the kernel before it (a kick); the condition kernel always is (L.pdl)
// heavy (with cond): the IF handle of the step's many-leg kernel, closed here
cudaError_t launch_pair_clear(const Launch& L, const DevParams& P, const DevState& S);
cudaError_t launch_spec_drift(const Launch& L, const DevParams& P, const DevState& S,
                              double Ttar, const cudaGraphConditionalHandle* cond = nullptr,
                              bool pdl_first = false,
                              const cudaGraphConditionalHandle* heavy = nullptr);
cudaError_t launch_spec_kick(const Launch& L, const DevParams& P, const DevState& S,
                             double Ttar, int apply);
// the kick of a step fused with the drift of the next (a grid of at most
// max_blocks resident blocks); in a graph, hif is the following rebuild IF
// node's handle and, when last_of_pair, hwhile the step loop's WHILE node;
// heavy: the IF handle of the next step's many-leg kernel, closed here
cudaError_t launch_spec_kd(const Launch& L, const DevParams& P, const DevState& S, double Ttar,
                           LoopCtl* loop, cudaGraphConditionalHandle hif,
                           cudaGraphConditionalHandle hwhile, int last_of_pair, int max_blocks,
                           const cudaGraphConditionalHandle* heavy = nullptr);
int spec_kd_resident_blocks(int nrep, int sms);
// fibmd_graph.cu: device-side conditions of the CUDA-graph step loop
cudaError_t launch_loop_ctl(cudaStream_t s, LoopCtl* loop, const DevScalars* sc,
                            cudaGraphConditionalHandle h, bool pdl = false);
// sets the loop to `pairs` step pairs, stopping early once the time of
// replica 0 passes its value at this point plus `relax` (relax <= 0: no stop)
cudaError_t launch_loop_set(cudaStream_t s, LoopCtl* loop, const DevScalars* sc, long long pairs,
                            double relax);
// dose: bring impact k's ion into the run; record the counts after it
cudaError_t launch_inject(const Launch& L, const DevParams& P, const DevState& S,
                          const Impact* table, int k);
// per replica: displaced lattice atoms and the first ion's depth
cudaError_t launch_impact_stats(const Launch& L, const DevParams& P, const DevState& S,
                                const double* surface_z, double thr, int* displaced,
                                double* ion_depth);
// writeatoms' columns: x y z (Angstrom, (N,3) column-major) and KE (eV)
cudaError_t launch_xyz_frame(const Launch& L, const DevState& S, int N, double* xyz, double* ke);
cudaError_t launch_dose_record(const Launch& L, const DevState& S, const LoopCtl* loop, int k,
                               int* removed, int* ions_removed, double* time, long long* steps);

}  // namespace fibmd
