// fibmd_capi.cu — the C-ABI of libfibmd_gpu.so: context lifetime, transfers,
// and the TI/onestep driver (src/timeint.f90:123-242) issuing the kernels.
//
// Host arithmetic in this file that feeds decisions the reference makes
// (radii, cell counts, the 2-body table, regime switches, loop exits) keeps
// the reference's binary64 operation order; the library is compiled with
// -ffp-contract=off on the host side.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "fibmd_internal.cuh"

using namespace fibmd;

namespace fibmd {
// Message of the last failure that had no context (create, the
// allocation-free entry point); a fixed buffer so reporting allocates nothing.
char g_noctx_error[512] = "";

void set_noctx_error(const char* msg) {
  std::snprintf(g_noctx_error, sizeof g_noctx_error, "%s", msg);
}
}  // namespace fibmd

namespace {



// Timed phases: the reference's calc_time report (at, nt, ds, f), the main
// force kernel alone, and the velocity-Verlet halves with their reductions.
enum Phase { PH_AT = 0, PH_NT = 1, PH_DS = 2, PH_F = 3, PH_FK = 4, PH_DRIFT = 5, PH_KICK = 6,
             PH_COUNT = 7 };

struct TimedRange {
  int phase;
  cudaEvent_t a, b;
};

}  // namespace

struct fibmd_ctx {
  fibmd_params p;
  int dev = 0;
  int sms = 152;
  cudaStream_t stream = nullptr;
  DevParams P;
  DevState S;
  DevScalars* h_sc = nullptr;  // pinned mirror
  double* d_stage = nullptr;   // 3N doubles
  double* d_ke = nullptr;      // N doubles (xyz frames)
  unsigned long long* d_u64 = nullptr;
  double* d_vir = nullptr;       // 6 doubles (virial), allocated on first use
  double* d_vir_atom = nullptr;  // 6 N doubles (per-atom virial), on first use
  std::vector<void*> allocs;
  std::vector<double> tab, tabu;
  // regime (prms.f90 module variables)
  double Ts = 0, Tau = 0;
  int ntlist = 1, atlist = 1, dslist = 1, atm_out = 0;
  int tic = 1;
  int impact = 0;
  bool atom_is_fast = true;
  bool uploaded = false, lists_built = false, spec_ready = false;
  // timers
  bool timers_on = true;
  bool kernel_timing = false;
  double t[PH_COUNT] = {};
  long long c[PH_COUNT] = {};
  std::vector<TimedRange> pending;
  std::vector<cudaEvent_t> pool;
  long long spec_lt = 0;
  // CUDA-graph step loop (spec mode)
  bool use_graph = true;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  cudaStream_t cap2 = nullptr;
  double4_32a* graph_frc = nullptr;  // S.frc when the graph was captured
  int graph_nfired = -1;
  int graph_stage = 0;               // the force stage size it was captured with
  // binary32 force kernel: stage size, re-chosen by timing (autotune) before
  // each chunk of spec-mode steps (kTuneSteps, doubling up to 8 times that
  // while the choice stands)
  int stage = kStageSmall;
  bool autotune = true;
  long long tune_pairs = 0;   // step pairs between tunings (0: kTuneSteps / 2)
  long long tune_left = 0;    // step pairs left before the next tuning
  int tune_count = 0;         // tunings so far
  float tune_ms[5] = {};      // each candidate's last timing
  bool tune_switched = false; // the last tuning changed the path
  // atoms per block of the binary32 force kernel (128 or 64, tuned with the
  // force path) and of the pair-list build (64, 128 or 256, tuned with the
  // skin); the graph is captured again when one changes
  int force_block = 128;
  int build_block = 128;
  int graph_force_block = -1, graph_build_block = -1, graph_uniform = -1, graph_pair = -1;
  int uniform = 0;  // the uploaded lattice holds no Ge
  bool react = false;  // binary32 path: stored reactions instead of atomics
  int graph_react = -1;
  // step graph: the many-leg kernel in an IF node that the force kernel
  // opens (off: the node's evaluation costs more than the empty launch)
  bool heavy_if = false;
  int graph_heavy_if = -1;
  // programmatic dependent launch of the step loop's kernels (option "pdl";
  // off by default: measured no faster on the graph step loop)
  bool pdl = false;
  int graph_pdl = -1;                // the pdl setting the graph was captured with
  // the graph's kick of each step fused with the next step's drift (option
  // "fuse"), in a grid of at most kd_blocks resident blocks
  bool fuse = true;
  // spec-mode rebuild rule (option "rebuild_rule"), per replica in a batch:
  // 1, the two largest displacements since the build reach the skin; 0, any
  // atom's displacement reaches half the skin
  int rebuild_rule = 1;
  int kd_blocks = 0;       // resident blocks of the fused kernel (0: unavailable)
  int kd_grid = 0;         // option "kd_grid": its grid size instead (tests)
  int graph_fuse = -1;
  LoopCtl* d_loop = nullptr;
  // spec mode: the candidate list skins, each with its parameters and
  // per-replica geometry (cell grids differ with the list radius); the one
  // in use is skin_cur, re-chosen by timing ("skin_tune")
  struct SkinSet {
    double skin = 0.0;
    DevParams P;
    std::vector<Geo> geo;
    Geo* d_geo = nullptr;
  };
  std::vector<SkinSet> skins;
  int skin_cur = 0;
  bool skin_tune = true;
  bool build_tune = true;   // the build's block size, tuned with the skin
  int graph_skin = -1;
  long long graph_chunks = 0;  // tuning chunks run (the skin's re-tuning cadence)
  double umax = 0.0;           // the 2-body table's extent
  int tab_last = 0;
  std::vector<fibmd_replica> reps;       // a batch's replicas
  std::vector<long long> rep_begin;      // and their first atoms
  // replicas: one for a single system, several for a batched ensemble
  Geo geo0;                 // the single system's geometry
  std::vector<Geo> geo;     // per replica (uploaded to S.geo)
  std::vector<int> rep_of;  // replica of each atom, -1 for padding slots
  std::string err;
};

// ---- helpers -------------------------------------------------------------------
static int fail(fibmd_ctx* ctx, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (ctx) ctx->err = buf;
  else set_noctx_error(buf);
  return code;
}

#define CK(call)                                                                  \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess)                                                        \
      return fail(ctx, FIBMD_ECUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
static int dalloc(fibmd_ctx* ctx, T** ptr, size_t count) {
  void* p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc(&p, sizeof(T) * count);
  if (e != cudaSuccess)
    return fail(ctx, FIBMD_ENOMEM, "cudaMalloc(%zu bytes): %s", sizeof(T) * count,
                cudaGetErrorString(e));
  ctx->allocs.push_back(p);
  *ptr = static_cast<T*>(p);
  return FIBMD_OK;
}

static Launch launch_of(const fibmd_ctx* ctx) {
  Launch L;
  L.stream = ctx->stream;
  L.sms = ctx->sms;
  L.stage = ctx->stage;
  L.pdl = ctx->pdl;
  L.force_block = ctx->force_block;
  L.build_block = ctx->build_block;
  L.react = ctx->react;
  return L;
}

// The fused kick-drift runs when allowed ("fuse") and, unless the kd_grid
// test hook sets its grid, only where every chunk gets a block of its own
// in one resident wave (measured: no faster where blocks take two chunks)
static bool fuse_in_use(const fibmd_ctx* ctx) {
  if (!ctx->fuse || ctx->kd_blocks <= 0) return false;
  const int nchunk = (ctx->P.N + kKickThreads - 1) / kKickThreads;
  return ctx->kd_grid > 0 || nchunk <= ctx->kd_blocks;
}

// Switches to candidate skin k: its parameters and geometry; the next step
// rebuilds the lists for the new radius (and the step graph is captured
// again, the parameters being kernel arguments).
static int set_skin(fibmd_ctx* ctx, int k) {
  if (k == ctx->skin_cur) return FIBMD_OK;
  const fibmd_ctx::SkinSet& set = ctx->skins[(size_t)k];
  const int nfired = ctx->P.nfired;
  ctx->P = set.P;
  ctx->P.nfired = nfired;
  ctx->geo = set.geo;
  ctx->S.geo = set.d_geo;
  ctx->skin_cur = k;
  // every replica's lists, for the new radius and grid
  const int one = 1;
  cudaError_t e = cudaMemcpyAsync(&ctx->S.sc->need_rebuild, &one, sizeof(int),
                                  cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&ctx->S.sc->rebuild_all, &one, sizeof(int), cudaMemcpyHostToDevice,
                        ctx->stream);
  if (e == cudaSuccess) cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    ctx->err = std::string("set_skin: ") + cudaGetErrorString(e);
    return FIBMD_ECUDA;
  }
  return FIBMD_OK;
}

static cudaEvent_t get_event(fibmd_ctx* ctx) {
  if (!ctx->pool.empty()) {
    cudaEvent_t e = ctx->pool.back();
    ctx->pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

static void flush_timers(fibmd_ctx* ctx) {
  for (auto& r : ctx->pending) {
    float ms = 0.f;
    cudaEventSynchronize(r.b);
    if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) ctx->t[r.phase] += 1e-3 * ms;
    ctx->pool.push_back(r.a);
    ctx->pool.push_back(r.b);
  }
  ctx->pending.clear();
}

struct PhaseTimer {
  fibmd_ctx* ctx;
  int phase;
  cudaEvent_t a = nullptr;
  PhaseTimer(fibmd_ctx* c, int ph) : ctx(c), phase(ph) {
    ctx->c[phase]++;
    if (ctx->timers_on) {
      a = get_event(ctx);
      cudaEventRecord(a, ctx->stream);
    }
  }
  ~PhaseTimer() {
    if (!a) return;
    cudaEvent_t b = get_event(ctx);
    cudaEventRecord(b, ctx->stream);
    ctx->pending.push_back({phase, a, b});
    if (ctx->pending.size() > 4096) flush_timers(ctx);
  }
};

// ---- parameter derivation --------------------------------------------------------
namespace fibmd {

// mktables, src/si.f90:575-597, in the reference's operation order, into
// caller buffers of Ntable + 2 entries.
void build_ref_table(const fibmd_params& p, double* tab, double* tabu, double* umax_out,
                     int* last_nz) {
  const int Nt = p.Ntable;
  for (int i = 0; i < Nt + 2; i++) tab[i] = tabu[i] = 0.0;
  const double umax = 2.5 * p.listfac * p.al;
  const double du = umax / (double)(Nt - 1);
  int last = 0;
  for (int i = 2; i <= Nt; i++) {
    const double ui = umax * (double)(i - 1) / (double)(Nt - 1);
    tabu[i - 1] = ui;
    if (ui < .999 * p.al) {
      const double ex = std::exp(1. / (ui - p.al));
      const double y = (p.B * std::pow(ui, -p.psi) - std::pow(ui, -p.qsi)) /
                           ((ui - p.al) * (ui - p.al)) +
                       (p.psi * p.B * std::pow(ui, -p.psi - 1) - p.qsi * std::pow(ui, -p.qsi - 1));
      tab[i - 1] = -(p.A * ex * y / (du * du));
      if (tab[i - 1] != 0.0) last = i - 1;
    }
  }
  // u(1) is never set by the reference; a listed pair never reads it
  *umax_out = umax;
  *last_nz = last;
}

// List radii (m): the reference's listfac * a * sigma and listfac * 2.5 sigma
// (init_nlist, si.f90:56-61), or in spec mode with a list skin, cutoff + skin.
static void list_radii(const fibmd_params& p, double* rc, double* rclj) {
  const double sigmax = p.sigmaGe > p.sigmaSi ? p.sigmaGe : p.sigmaSi;
  *rc = p.listfac * p.al * sigmax;
  *rclj = p.listfac * 2.5 * sigmax;
  if (p.mode == FIBMD_MODE_SPEC && p.list_skin > 0.0) {
    *rc = 0.999 * p.al * sigmax + p.list_skin;
    *rclj = 2.5 * sigmax + p.list_skin;
  }
}

constexpr double kRemoveBelow = 10.0e-10;  // m below the lowest plane
// spec mode's list skin when the parameters ask for it to be chosen
// (list_skin < 0): the start of the run-time tuning
constexpr double kDefaultSkin = 0.6e-10;

int derive_geo(const fibmd_params& p, const double Lb[3], double remove_z, Geo& G, char* err,
               int errlen) {
  std::memset(&G, 0, sizeof G);
  double rc, rclj;
  list_radii(p, &rc, &rclj);
  const bool spec = p.mode == FIBMD_MODE_SPEC;
  for (int d = 0; d < 3; d++) {
    if (!(Lb[d] > 0.0)) {
      std::snprintf(err, (size_t)errlen, "box length %d is %g", d + 1, Lb[d]);
      return FIBMD_EINVAL;
    }
    G.Lb[d] = Lb[d];
    G.iLb[d] = 1. / Lb[d];
    const int n = (int)(Lb[d] / rc);
    G.nc[d] = n > 1 ? n : 1;
    G.hcell[d] = Lb[d] / (double)G.nc[d];  // chainlist's HMf = Lb/REAL(N)
    G.wrap[d] = G.nc[d] > 2;                // ghost layers only when Nc > 2
    G.qscale[d] = 4294967296.0 / Lb[d];
    G.qinvA[d] = (float)(Lb[d] * 1.0e10 / 4294967296.0);
  }
  G.remove_z = remove_z;
  G.remove_zlo = -1.0e300;
  G.mol_reach = 1;
  if (spec) {
    // atoms above remove_z are removed, so the grid need not cover the
    // vacuum above it; pairs never straddle z = 0 (no wrap in z)
    if (remove_z > 0.0 && remove_z + rc < Lb[2]) {
      const double zext = remove_z + rc;
      const int n = (int)(zext / (rc * (1.0 + 1e-6)));
      G.nc[2] = n > 1 ? n : 1;
      G.hcell[2] = zext / (double)G.nc[2];
      G.inv_hz = 1.0 / G.hcell[2];
      G.zcompact = 1;
      G.wrap[2] = 0;
      // an atom that leaves through the bottom (a transmitted ion) is
      // removed once it is beyond every interaction range of the lowest
      // plane (z = 0), as the reference's periodic z sends it into the
      // vacuum bands where frzsptrdatms parks it
      G.remove_zlo = -kRemoveBelow;
    }
    const double hmin = std::min(G.hcell[0], std::min(G.hcell[1], G.hcell[2]));
    G.mol_reach = (int)std::ceil(rclj / hmin);
  }
  const long long ncell = (long long)G.nc[0] * G.nc[1] * G.nc[2];
  if (ncell > (1ll << 30)) {
    std::snprintf(err, (size_t)errlen, "cell grid too large (%lld)", ncell);
    return FIBMD_EINVAL;
  }
  G.ncell = (int)ncell;
  return FIBMD_OK;
}

int derive_dev_params(const fibmd_params& p, int impact, double umax, int tab_last, DevParams& P,
                      Geo& G, char* err, int errlen) {
  std::memset(&P, 0, sizeof P);
  P.N = p.Natm;
  P.Nsg = p.Nsg;
  P.nfired = p.Nsg + impact;
  P.nrep = 1;
  P.nion = p.Natm - p.Nsg;
  P.mode = p.mode;
  P.precision = p.precision;
  P.max_sw = p.max_sw_nbrs > 0 ? p.max_sw_nbrs : 48;
  const double sigmax = p.sigmaGe > p.sigmaSi ? p.sigmaGe : p.sigmaSi;
  double rc, rclj;
  list_radii(p, &rc, &rclj);
  const double rlj = 2.5 * sigmax;
  int rcg = derive_geo(p, p.Lb, p.remove_z, G, err, errlen);
  if (rcg) return rcg;
  G.atom_begin = 0;
  G.atom_end = p.Natm;
  G.blk_begin = 0;
  G.blk_end = (p.Natm + kKickThreads - 1) / kKickThreads;
  for (int d = 0; d < 3; d++) {
    P.Lb[d] = G.Lb[d];
    P.iLb[d] = G.iLb[d];
    P.nc[d] = G.nc[d];
    P.hcell[d] = G.hcell[d];
    P.wrap[d] = G.wrap[d];
    P.qscale[d] = G.qscale[d];
    P.qinvA[d] = G.qinvA[d];
  }
  P.zcompact = G.zcompact;
  P.inv_hz = G.inv_hz;
  P.mol_reach = G.mol_reach;
  P.ncell = G.ncell;
  P.rv2 = rc * rc;
  P.rv2lj = rclj * rclj;
  P.rlj2 = rlj * rlj;
  const double rcA = rc * 1e10, rcljA = rclj * 1e10;
  P.pre_sw2A = (float)((rcA * (1 + 1e-4)) * (rcA * (1 + 1e-4)));
  P.acc_sw2A = (float)((rcA * (1 - 1e-4)) * (rcA * (1 - 1e-4)));
  P.pre_mol2A = (float)((rcljA * (1 + 1e-4)) * (rcljA * (1 + 1e-4)));
  P.acc_mol2A = (float)((rcljA * (1 - 1e-4)) * (rcljA * (1 - 1e-4)));
  // Stillinger-Weber constants, setupSiGe (prms.f90:452-480)
  P.al = p.al;
  P.gam = p.gamma;
  P.cut3 = 0.999 * p.al;
  P.thrd = 1. / 3.;
  P.A = p.A;
  P.B = p.B;
  P.psi = p.psi;
  P.qsi = p.qsi;
  P.eps[0][0] = p.epsSi;
  P.eps[0][1] = 0.5 * (p.epsSi + p.epsGe);
  P.eps[1][1] = p.epsGe;
  P.eps[1][0] = 0.5 * (p.epsSi + p.epsGe);
  P.isig[0][0] = 1. / p.sigmaSi;
  P.isig[0][1] = 2. / (p.sigmaSi + p.sigmaGe);
  P.isig[1][1] = 1. / p.sigmaGe;
  P.isig[1][0] = 2. / (p.sigmaSi + p.sigmaGe);
  const double l112 = 2. * p.lambdaSi * p.epsSi / 3. + p.lambdaGe * p.epsGe / 3.;
  const double l122 = p.lambdaSi * p.epsSi / 3. + 2. * p.lambdaGe * p.epsGe / 3.;
  P.leps[0][0][0] = p.lambdaSi * p.epsSi;
  P.leps[0][0][1] = P.leps[0][1][0] = P.leps[1][0][0] = l112;
  P.leps[0][1][1] = P.leps[1][1][0] = P.leps[1][0][1] = l122;
  P.leps[1][1][1] = p.lambdaGe * p.epsGe;
  P.epssig[0][0] = p.epsSi / p.sigmaSi;
  P.epssig[0][1] = P.epssig[1][0] = (p.epsSi + p.epsGe) / (p.sigmaSi + p.sigmaGe);
  P.epssig[1][1] = p.epsGe / p.sigmaGe;
  // Moliere constants, setupMol (prms.f90:433-449)
  const double Pi = 4. * std::atan(1.0);
  P.Zmol[0] = p.ZSi;
  P.Zmol[1] = p.ZGe;
  P.Zmol[2] = p.ZGa;
  std::memset(P.aamol, 0, sizeof P.aamol);
  P.aamol[0][2] = 0.885 * p.ao * std::pow(std::sqrt(p.ZSi) + std::sqrt(p.ZGa), -(2. / 3.));
  P.aamol[1][2] = 0.885 * p.ao * std::pow(std::sqrt(p.ZGe) + std::sqrt(p.ZGa), -(2. / 3.));
  P.aamol[2][0] = P.aamol[0][2];
  P.aamol[2][1] = P.aamol[1][2];
  P.aamol[2][2] = 0.885 * p.ao * std::pow(std::sqrt(p.ZGa) + std::sqrt(p.ZGa), -(2. / 3.));
  P.ie0 = 1 / (4 * Pi * p.eps0);
  P.ec = p.ec;
  P.Amol = p.Amol;
  P.Bmol = p.Bmol;
  P.Cmol = p.Cmol;
  P.amol = p.alpha_mol;
  P.bmol = p.beta_mol;
  P.gmol = p.gamma_mol;
  // 2-body table (built separately by build_ref_table)
  P.umax = umax;
  P.tab_last = tab_last;
  P.Ntable = p.Ntable;
  // a listed pair's table coordinate INT(u/umax*(Ntable-1)) + 1 must stay
  // within Ntable (itable2bd reports an error past it, src/si.f90:562-564):
  // a list radius beyond the table is refused here
  {
    const double sigmin = p.sigmaGe < p.sigmaSi ? p.sigmaGe : p.sigmaSi;
    const double ulist = rc / sigmin;
    if (ulist / umax * (double)(p.Ntable - 1) >= (double)p.Ntable) {
      std::snprintf(err, (size_t)errlen,
                    "list radius %.4g A (u = %.4g) reaches beyond the 2-body table (umax %.4g, "
                    "Ntable %d)", rc * 1e10, ulist, umax, p.Ntable);
      return FIBMD_ETABLE;
    }
  }
  // abscissa after the last non-zero entry: u(k+1) = umax*k/(Ntable-1)
  const double u_next = umax * (double)(tab_last + 1) / (double)(p.Ntable - 1);
  const double usup = std::max(P.cut3, u_next);
  const double rsupA = usup * sigmax * 1e10 * (1 + 1e-4);
  P.pre3A2 = (float)(rsupA * rsupA);
  // binary32: a pair at u > a - gamma/110 has exp(gamma/(u-a)) < e^-110 (zero
  // in binary32) and exp(1/(u-a)) < e^-91 (a 2-body force below 1e-35 eV/A)
  const double um = std::min(P.cut3, p.al - p.gamma / 110.0);
  const double rmA = um * sigmax * 1e10 * (1 + 1e-4);
  P.pre3mA2 = (float)(rmA * rmA);
  const double ul = std::min(um, p.al + p.gamma / std::log((double)kLegEmin));
  const double rlA = ul * sigmax * 1e10 * (1 + 1e-4);
  P.pre3lA2 = (float)(rlA * rlA);
  // fast atoms: displaced by at least half the smaller list skin
  const double skin = std::min(rc - P.cut3 * sigmax, rclj - rlj);
  const double half = 0.5 * skin * 0.99;
  P.disp_fast2 = half * half;
  P.disp_fastA2 = (float)(half * half * 1e20);
  // the pair rule: a pair outside the list radius at the build comes within
  // the cutoff only once the two atoms' displacements add up to the skin;
  // displacements under a quarter of it are counted at that bound (so that
  // the thermal atoms of a slab report nothing for most of a list's life)
  P.pair_rule = 0;
  P.disp_skinA = (float)(2.0 * half * 1e10);
  P.disp_lowA2 = (float)((0.5 * half * 1e10) * (0.5 * half * 1e10));
  // binary32 reduced units
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++) {
      P.epsA[a][b] = (float)(P.eps[a][b] / p.ec);
      P.sigA[a][b] = (float)(1e10 / P.isig[a][b]);
      P.isigA[a][b] = (float)(P.isig[a][b] * 1e-10);
      P.epssigA[a][b] = (float)(P.eps[a][b] / p.ec * P.isig[a][b] * 1e-10);
      for (int c = 0; c < 2; c++) P.lepsA[a][b][c] = (float)(P.leps[a][b][c] / p.ec);
    }
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++) {
      P.molKA[a][b] = (float)(P.ie0 * P.Zmol[a] * P.Zmol[b] * p.ec * 1e10);
      P.amolA[a][b] = (float)(P.aamol[a][b] * 1e10);
    }
  P.f_evA_to_N = p.ec * 1e10;
  P.e_eV_to_J = p.ec;
  P.mol_fp64_rA = (float)(p.mixed_mol_fp64_r * 1e10);
  // integrator geometry
  P.kB = p.kB;
  const double nm = 1.0e-9;
  const double L3 = p.Lb[2];
  P.side_sw = p.sidewidth * nm;
  P.side_zlo = p.outz[0] * L3 / 10.0;
  P.side_zhi = p.outz[3] * L3 / 10.0;
  for (int k = 0; k < 4; k++) P.park_o[k] = p.outz[k] * L3 / 10.0;
  const double buffer = 0.3;
  for (int k = 0; k < 2; k++) {
    P.park_a[k] = p.atomz[k] * L3 / 10.0;
    P.park_al[k] = (p.atomz[k] - buffer) * L3 / 10.0;
    P.park_ah[k] = (p.atomz[k] + buffer) * L3 / 10.0;
  }
  P.park_il = (p.ionz - buffer) * L3 / 10.0;
  P.park_ih = (p.ionz + buffer) * L3 / 10.0;
  P.remove_z = p.remove_z;
  P.dt_max = p.dt_max;
  P.dx_max = p.dx_max;
  P.tau_spec = p.tau_spec;
  // Moliere full-list capacity: at least the reference's MLlj = 1500*Nlj
  long long mlj = 1500ll * (p.Nlj > 0 ? p.Nlj : 1);
  P.mol_cap = p.max_mol_pairs > 0 ? p.max_mol_pairs : (int)std::max<long long>(mlj, 1 << 16);
  return FIBMD_OK;
}

}  // namespace fibmd

static int derive_params(fibmd_ctx* ctx) {
  const fibmd_params& p = ctx->p;
  ctx->tab.assign((size_t)p.Ntable + 2, 0.0);
  ctx->tabu.assign((size_t)p.Ntable + 2, 0.0);
  double umax = 0.0;
  int last = 0;
  build_ref_table(p, ctx->tab.data(), ctx->tabu.data(), &umax, &last);
  ctx->umax = umax;
  ctx->tab_last = last;
  char err[256] = "";
  const int rc = derive_dev_params(p, ctx->impact, umax, last, ctx->P, ctx->geo0, err, sizeof err);
  if (rc) return fail(ctx, rc, "%s", err);
  ctx->P.uniform = ctx->uniform;
  return FIBMD_OK;
}

// Parameters and per-replica geometry of the context with list skin `skin`
// (a single system, or the batch whose replicas ctx->reps holds).
static int derive_skin(const fibmd_ctx* ctx, double skin, fibmd_ctx::SkinSet& out, char* err,
                       int errlen) {
  fibmd_params q = ctx->p;
  q.list_skin = skin;
  Geo g0;
  int rc = derive_dev_params(q, ctx->impact, ctx->umax, ctx->tab_last, out.P, g0, err, errlen);
  if (rc) return rc;
  out.P.uniform = ctx->uniform;
  out.P.pair_rule = (ctx->rebuild_rule == 1 && q.mode == FIBMD_MODE_SPEC) ? 1 : 0;
  out.skin = skin;
  if (ctx->reps.empty()) {
    out.geo.assign(1, g0);
    return FIBMD_OK;
  }
  const int nrep = (int)ctx->reps.size();
  out.geo.resize((size_t)nrep);
  long long cells = 0, nion = 0;
  int reach = 1;
  for (int r = 0; r < nrep; r++) {
    const fibmd_replica& R = ctx->reps[(size_t)r];
    Geo& G = out.geo[(size_t)r];
    rc = derive_geo(q, R.Lb, R.remove_z, G, err, errlen);
    if (rc) return rc;
    G.cell_off = (int)cells;
    cells += G.ncell;
    G.atom_begin = (int)ctx->rep_begin[(size_t)r];
    G.atom_end = (int)(ctx->rep_begin[(size_t)r] + R.natm);
    G.blk_begin = G.atom_begin / kKickThreads;
    G.blk_end = (G.atom_end + kKickThreads - 1) / kKickThreads;
    reach = std::max(reach, G.mol_reach);
    nion += R.natm - R.nsg;
  }
  if (cells > (1ll << 30)) {
    std::snprintf(err, (size_t)errlen, "batch: %lld cells", cells);
    return FIBMD_EINVAL;
  }
  out.P.nrep = nrep;
  out.P.nion = (int)nion;
  out.P.nfired = q.Natm;
  out.P.ncell = (int)cells;
  out.P.mol_reach = reach;
  return FIBMD_OK;
}

// The candidate skins: spec mode with a list skin takes 0.75, 1 and 1.35
// times the start value (a candidate whose radius leaves the 2-body table is
// dropped); otherwise the one set of the parameters as given.
static int derive_skins(fibmd_ctx* ctx) {
  const double s0 = ctx->p.list_skin;
  std::vector<double> cand;
  if (ctx->p.mode == FIBMD_MODE_SPEC && s0 > 0.0) cand = {0.75 * s0, s0, 1.35 * s0};
  else cand = {s0};
  ctx->skins.clear();
  char err[256] = "";
  for (double sk : cand) {
    fibmd_ctx::SkinSet set;
    const int rc = derive_skin(ctx, sk, set, err, sizeof err);
    if (rc) {
      if (sk == s0) return fail(ctx, rc, "%s", err);
      continue;
    }
    if (sk == s0) ctx->skin_cur = (int)ctx->skins.size();
    ctx->skins.push_back(set);
  }
  const fibmd_ctx::SkinSet& cur = ctx->skins[(size_t)ctx->skin_cur];
  ctx->P = cur.P;
  ctx->geo = cur.geo;
  return FIBMD_OK;
}

// ionrun, src/prms.f90:563-584
static void set_regime(fibmd_ctx* ctx, int tic) {
  const fibmd_params& p = ctx->p;
  if (tic == 1) {
    ctx->Ts = p.Ts_i;
    ctx->atm_out = p.atm_out_i;
    ctx->ntlist = p.ntlist_i;
    ctx->atlist = p.atlist_i;
    ctx->Tau = p.Tau_i;
    ctx->dslist = p.dslist_i;
  } else if (tic == 2) {
    ctx->Ts = p.Ts_r;
    ctx->atm_out = p.atm_out_r;
    ctx->ntlist = p.ntlist_r;
    ctx->atlist = p.atlist_r;
    ctx->Tau = p.Tau_r;
    ctx->dslist = p.dslist_r;
  }
  ctx->tic = tic;
}

static int sync_scalars(fibmd_ctx* ctx) {
  CK(cudaMemcpyAsync(ctx->h_sc, ctx->S.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return FIBMD_OK;
}

// Force launch, with events around the main kernel when kernel timing is on.
static int force_launch(fibmd_ctx* ctx, bool energy, bool count, bool spec_step = false) {
  Launch L = launch_of(ctx);
  if (ctx->kernel_timing) {
    L.force_a = get_event(ctx);
    L.force_b = get_event(ctx);
  }
  cudaError_t e = launch_force(L, ctx->P, ctx->S, energy, count, spec_step);
  if (L.force_a) {
    ctx->pending.push_back({PH_FK, L.force_a, L.force_b});
    ctx->c[PH_FK]++;
  }
  if (e != cudaSuccess) return fail(ctx, FIBMD_ECUDA, "force launch: %s", cudaGetErrorString(e));
  return FIBMD_OK;
}

// ---- C-ABI -----------------------------------------------------------------------
extern "C" {

int fibmd_gpu_abi_version(void) { return FIBMD_ABI_VERSION; }

int fibmd_gpu_params_size(void) { return (int)sizeof(fibmd_params); }

int fibmd_gpu_params_default(fibmd_params* p) {
  if (!p) return FIBMD_EINVAL;
  std::memset(p, 0, sizeof(*p));
  p->abi_version = FIBMD_ABI_VERSION;
  p->mode = FIBMD_MODE_REF;
  p->precision = FIBMD_PREC_FP64;
  // prms.f90:172-216
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
  // siga.in as shipped with the reference
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
  // spec-mode defaults: 1 fs cap, 0.05 A per step, 0.1 ps thermostat
  p->dt_max = 1.0e-15;
  p->dx_max = 0.05e-10;
  p->tau_spec = 1.0e-13;
  p->remove_z = -1.0;
  p->mixed_mol_fp64_r = 1.0e-10;
  p->list_skin = 0.0;
  return FIBMD_OK;
}

int fibmd_gpu_last_error(const fibmd_ctx* ctx, char* buf, int len) {
  if (!buf || len <= 0) return FIBMD_EINVAL;
  std::snprintf(buf, (size_t)len, "%s", ctx ? ctx->err.c_str() : g_noctx_error);
  return FIBMD_OK;
}

static int finish_create(fibmd_ctx* ctx, const std::vector<int>& ions, fibmd_ctx** out);

int fibmd_gpu_create(const fibmd_params* p, fibmd_ctx** out) {
  fibmd_ctx* ctx = nullptr;
  if (!p || !out) return fail(nullptr, FIBMD_EINVAL, "null argument");
  *out = nullptr;
  if (p->abi_version != FIBMD_ABI_VERSION)
    return fail(nullptr, FIBMD_EINVAL, "abi_version %d, library has %d", p->abi_version,
                FIBMD_ABI_VERSION);
  if (p->Natm <= 0 || p->Nsg < 0 || p->Nsg > p->Natm || p->Lb[0] <= 0 || p->Lb[1] <= 0 ||
      p->Lb[2] <= 0 || p->Ntable < 8)
    return fail(nullptr, FIBMD_EINVAL, "bad sizes (Natm %d Nsg %d Ntable %d)", p->Natm, p->Nsg,
                p->Ntable);
  if (p->max_sw_nbrs > 64)
    return fail(nullptr, FIBMD_EINVAL, "max_sw_nbrs %d exceeds 64", p->max_sw_nbrs);
  if (p->precision == FIBMD_PREC_MIXED && (p->psi != 4.0 || p->qsi != 0.0))
    return fail(nullptr, FIBMD_EINVAL, "mixed precision implements psi = 4, qsi = 0 only");

  // the parameters are checked (host arithmetic only) before the device is
  ctx = new fibmd_ctx();
  ctx->p = *p;
  if (ctx->p.mode == FIBMD_MODE_SPEC && ctx->p.list_skin < 0.0) ctx->p.list_skin = kDefaultSkin;
  int rc = derive_params(ctx);
  if (rc == FIBMD_OK) rc = derive_skins(ctx);
  if (rc) {
    set_noctx_error(ctx->err.c_str());
    delete ctx;
    return rc;
  }
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    delete ctx;
    return fail(nullptr, FIBMD_ECUDA, "no CUDA device: %s", cudaGetErrorString(e));
  }
  ctx->rep_of.assign((size_t)p->Natm, 0);
  std::vector<int> ions;
  for (int i = p->Nsg; i < p->Natm; i++) ions.push_back(i);
  return finish_create(ctx, ions, out);
}

// Allocates and initialises the device state of a context whose P, geo and
// rep_of are set; deletes the context on failure.
static int finish_create(fibmd_ctx* ctx, const std::vector<int>& ions, fibmd_ctx** out) {
  cudaGetDevice(&ctx->dev);
  cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, ctx->dev);
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    set_noctx_error("cudaStreamCreate failed");
    delete ctx;
    return FIBMD_ECUDA;
  }
  const size_t N = (size_t)ctx->P.N;
  const size_t R = ctx->geo.size();
  DevState& S = ctx->S;
  std::memset(&S, 0, sizeof S);
  S.N = (int)N;
  // the cell arrays hold the largest grid of the candidate skins
  int max_cells = 0;
  for (const auto& k : ctx->skins) max_cells = std::max(max_cells, k.P.ncell);
  int nscan = (max_cells + 1 + 1023) / 1024;
#define AL(ptr, n)                       \
  do {                                   \
    int r_ = dalloc(ctx, &(ptr), (n));   \
    if (r_) {                            \
      set_noctx_error(ctx->err.c_str());         \
      fibmd_gpu_destroy(ctx);            \
      return r_;                         \
    }                                    \
  } while (0)
  AL(S.pos, N);
  AL(S.vel, N);
  AL(S.frc, N);
  AL(S.frc_new, N);
  AL(S.xi, N);
  AL(S.posq, N);
  AL(S.posq_build, N);
  AL(S.mass, N);
  AL(S.inv_mass, N);
  AL(S.atype, N);
  AL(S.flags, N);
  AL(S.cell_count, (size_t)max_cells + 1);
  AL(S.cell_start, (size_t)max_cells + 1);
  AL(S.cell_atoms, N);
  AL(S.posq_cell, N);
  AL(S.atom_cell, N);
  AL(S.scan_blocks, (size_t)nscan + 1);
  AL(S.nbr_sw, (size_t)ctx->P.max_sw * N);
  AL(S.n_sw, N);
  AL(S.sw_extra, N);
  AL(S.mol_pairs, (size_t)ctx->P.mol_cap);
  AL(S.fast_flag, N);
  AL(S.fast_list, N);
  AL(S.heavy_list, N);
  double* tab = nullptr;
  double* tabu = nullptr;
  AL(tab, ctx->tab.size());
  AL(tabu, ctx->tabu.size());
  S.tab = tab;
  S.tabu = tabu;
  AL(S.epot, N);
  AL(S.partials, 3 * (size_t)kMaxRedBlocks);
  AL(S.sc, R);
  for (auto& k : ctx->skins) AL(k.d_geo, R);
  int* ion_list = nullptr;
  AL(ion_list, ions.size());
  S.geo = ctx->skins[(size_t)ctx->skin_cur].d_geo;
  S.ion_list = ion_list;
  AL(ctx->d_stage, 3 * N);
  AL(ctx->d_ke, N);
  AL(ctx->d_u64, 4);
  AL(ctx->d_loop, 1);
  cudaMemsetAsync(ctx->d_loop, 0, sizeof(LoopCtl), ctx->stream);
#undef AL
  if (cudaMallocHost((void**)&ctx->h_sc, sizeof(DevScalars)) != cudaSuccess) {
    set_noctx_error("cudaMallocHost failed");
    fibmd_gpu_destroy(ctx);
    return FIBMD_ENOMEM;
  }
  cudaMemcpyAsync(tab, ctx->tab.data(), sizeof(double) * ctx->tab.size(),
                  cudaMemcpyHostToDevice, ctx->stream);
  cudaMemcpyAsync(tabu, ctx->tabu.data(), sizeof(double) * ctx->tabu.size(),
                  cudaMemcpyHostToDevice, ctx->stream);
  for (auto& k : ctx->skins)
    cudaMemcpyAsync(k.d_geo, k.geo.data(), sizeof(Geo) * R, cudaMemcpyHostToDevice, ctx->stream);
  if (!ions.empty())
    cudaMemcpyAsync(ion_list, ions.data(), sizeof(int) * ions.size(), cudaMemcpyHostToDevice,
                    ctx->stream);
  cudaMemsetAsync(S.sc, 0, sizeof(DevScalars) * R, ctx->stream);
  cudaMemsetAsync(S.fast_flag, 0, N, ctx->stream);
  cudaMemsetAsync(S.n_sw, 0, sizeof(int) * N, ctx->stream);
  cudaMemsetAsync(S.frc, 0, sizeof(double4_32a) * N, ctx->stream);
  cudaMemsetAsync(S.flags, 0, sizeof(uint32_t) * N, ctx->stream);
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
    set_noctx_error("initialisation copies failed");
    fibmd_gpu_destroy(ctx);
    return FIBMD_ECUDA;
  }
  set_regime(ctx, 1);
  ctx->kd_blocks = spec_kd_resident_blocks(ctx->P.nrep, ctx->sms);
  cudaGetLastError();
  *out = ctx;
  return FIBMD_OK;
}

int fibmd_gpu_batch_create(const fibmd_params* p, int nrep, const fibmd_replica* reps,
                           fibmd_ctx** out) {
  if (!p || !reps || !out || nrep < 1) return fail(nullptr, FIBMD_EINVAL, "batch: bad arguments");
  *out = nullptr;
  if (p->abi_version != FIBMD_ABI_VERSION)
    return fail(nullptr, FIBMD_EINVAL, "abi_version %d, library has %d", p->abi_version,
                FIBMD_ABI_VERSION);
  if (p->mode != FIBMD_MODE_SPEC) return fail(nullptr, FIBMD_EINVAL, "batch needs spec mode");
  if (nrep > 65535) return fail(nullptr, FIBMD_EINVAL, "batch: %d replicas (max 65535)", nrep);
  if (p->max_sw_nbrs > 64)
    return fail(nullptr, FIBMD_EINVAL, "max_sw_nbrs %d exceeds 64", p->max_sw_nbrs);
  if (p->precision == FIBMD_PREC_MIXED && (p->psi != 4.0 || p->qsi != 0.0))
    return fail(nullptr, FIBMD_EINVAL, "mixed precision implements psi = 4, qsi = 0 only");
  long long off = 0, nion = 0;
  std::vector<long long> begin((size_t)nrep);
  for (int r = 0; r < nrep; r++) {
    const fibmd_replica& q = reps[r];
    if (q.natm < 1 || q.nsg < 0 || q.nsg > q.natm)
      return fail(nullptr, FIBMD_EINVAL, "replica %d: natm %d nsg %d", r, q.natm, q.nsg);
    begin[r] = off;
    off += q.natm;
    off = (off + kKickThreads - 1) / kKickThreads * kKickThreads;
    nion += q.natm - q.nsg;
  }
  if (off > (1ll << 30)) return fail(nullptr, FIBMD_EINVAL, "batch: %lld atoms", off);
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return fail(nullptr, FIBMD_ECUDA, "no CUDA device: %s", cudaGetErrorString(e));

  if (off / kKickThreads > kMaxRedBlocks) return fail(nullptr, FIBMD_EINVAL, "batch: too many atoms");

  fibmd_ctx* ctx = new fibmd_ctx();
  fibmd_params q = *p;
  q.Natm = (int)off;
  q.Nsg = (int)off;  // every ion is fired; ions are found through the ion list
  q.Nlj = (int)nion;
  for (int d = 0; d < 3; d++) q.Lb[d] = reps[0].Lb[d];
  q.remove_z = reps[0].remove_z;
  if (q.list_skin < 0.0) q.list_skin = kDefaultSkin;
  ctx->p = q;
  ctx->reps.assign(reps, reps + nrep);
  ctx->rep_begin = begin;
  int rc = derive_params(ctx);
  if (rc == FIBMD_OK) rc = derive_skins(ctx);
  if (rc) {
    set_noctx_error(ctx->err.c_str());
    delete ctx;
    return rc;
  }
  ctx->rep_of.assign((size_t)off, -1);
  std::vector<int> ions;
  for (int r = 0; r < nrep; r++) {
    const Geo& G = ctx->geo[(size_t)r];
    for (int i = G.atom_begin; i < G.atom_end; i++) ctx->rep_of[(size_t)i] = r;
    for (int i = G.atom_begin + reps[r].nsg; i < G.atom_end; i++) ions.push_back(i);
  }
  return finish_create(ctx, ions, out);
}

int fibmd_gpu_impact_stats(fibmd_ctx* ctx, const double* surface_z, double displaced_m,
                           int* sputtered, int* displaced, double* ion_depth) {
  if (!ctx || !surface_z || !(displaced_m > 0.0)) return FIBMD_EINVAL;
  if (!ctx->uploaded) return fail(ctx, FIBMD_ESTATE, "impact stats before upload");
  const int R = ctx->P.nrep;
  double* d_sz = nullptr;
  int* d_cnt = nullptr;
  double* d_depth = nullptr;
  if (cudaMalloc((void**)&d_sz, sizeof(double) * R) != cudaSuccess ||
      cudaMalloc((void**)&d_cnt, sizeof(int) * R) != cudaSuccess ||
      cudaMalloc((void**)&d_depth, sizeof(double) * R) != cudaSuccess) {
    cudaFree(d_sz);
    cudaFree(d_cnt);
    cudaFree(d_depth);
    return fail(ctx, FIBMD_ENOMEM, "impact stats: %d replicas", R);
  }
  std::vector<int> cnt((size_t)R);
  std::vector<double> depth((size_t)R);
  std::vector<DevScalars> h((size_t)R);
  cudaError_t e = cudaMemcpyAsync(d_sz, surface_z, sizeof(double) * R, cudaMemcpyHostToDevice,
                                  ctx->stream);
  if (e == cudaSuccess)
    e = launch_impact_stats(launch_of(ctx), ctx->P, ctx->S, d_sz, displaced_m, d_cnt, d_depth);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(cnt.data(), d_cnt, sizeof(int) * R, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(depth.data(), d_depth, sizeof(double) * R, cudaMemcpyDeviceToHost,
                        ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h.data(), ctx->S.sc, sizeof(DevScalars) * R, cudaMemcpyDeviceToHost,
                        ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d_sz);
  cudaFree(d_cnt);
  cudaFree(d_depth);
  if (e != cudaSuccess) return fail(ctx, FIBMD_ECUDA, "impact stats: %s", cudaGetErrorString(e));
  for (int r = 0; r < R; r++) {
    if (sputtered) sputtered[r] = h[(size_t)r].removed_count;
    if (displaced) displaced[r] = cnt[(size_t)r];
    if (ion_depth) ion_depth[r] = depth[(size_t)r];
  }
  return FIBMD_OK;
}

int fibmd_gpu_batch_layout(fibmd_ctx* ctx, int* nrep, int* offsets) {
  if (!ctx) return FIBMD_EINVAL;
  const int R = (int)ctx->geo.size();
  if (nrep) *nrep = R;
  if (offsets) {
    for (int r = 0; r < R; r++) offsets[r] = ctx->geo[(size_t)r].atom_begin;
    offsets[R] = ctx->P.N;
  }
  return FIBMD_OK;
}

int fibmd_gpu_batch_scalars(fibmd_ctx* ctx, double* time, double* dt, int* removed) {
  if (!ctx) return FIBMD_EINVAL;
  const size_t R = ctx->geo.size();
  std::vector<DevScalars> h(R);
  CK(cudaMemcpyAsync(h.data(), ctx->S.sc, sizeof(DevScalars) * R, cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (size_t r = 0; r < R; r++) {
    if (time) time[r] = h[r].time;
    if (dt) dt[r] = h[r].dt;
    if (removed) removed[r] = h[r].removed_count;
  }
  return FIBMD_OK;
}

static void drop_graph(fibmd_ctx* ctx) {
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  if (ctx->graph) cudaGraphDestroy(ctx->graph);
  ctx->graph_exec = nullptr;
  ctx->graph = nullptr;
  ctx->graph_frc = nullptr;
}

void fibmd_gpu_destroy(fibmd_ctx* ctx) {
  if (!ctx) return;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  drop_graph(ctx);
  if (ctx->cap2) cudaStreamDestroy(ctx->cap2);
  flush_timers(ctx);
  for (auto e : ctx->pool) cudaEventDestroy(e);
  for (void* p : ctx->allocs) cudaFree(p);
  if (ctx->h_sc) cudaFreeHost(ctx->h_sc);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

void* fibmd_gpu_stream(fibmd_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

// Per-atom flags word: the tag bits and the atom's replica in bits 16..31;
// padding slots of a batch are removed atoms of the replica before them.
static uint32_t replica_flags(const fibmd_ctx* ctx, int i, uint32_t tag) {
  int r = ctx->rep_of[(size_t)i];
  if (r < 0) {
    r = 0;
    for (int k = i; k >= 0; k--)
      if (ctx->rep_of[(size_t)k] >= 0) {
        r = ctx->rep_of[(size_t)k];
        break;
      }
    tag = FL_REMOVED;
  }
  return (tag & 0xffu) | ((uint32_t)r << 16);
}

int fibmd_gpu_upload(fibmd_ctx* ctx, const double* X, const double* V, const double* F,
                     const double* Xi, const double* mass, const int* atype,
                     const int* xsides) {
  if (!ctx || !X || !V || !Xi || !mass || !atype || !xsides)
    return fail(ctx, FIBMD_EINVAL, "upload: null array");
  const int N = ctx->P.N;
  const size_t b3 = sizeof(double) * 3 * (size_t)N;
  Launch L = launch_of(ctx);
  std::vector<int8_t> t8((size_t)N);
  std::vector<uint32_t> fl((size_t)N);
  int uniform = 1;
  for (int i = 0; i < N; i++) {
    if (atype[i] < 1 || atype[i] > 3)
      return fail(ctx, FIBMD_EINVAL, "atype(%d) = %d is not 1, 2 or 3", i + 1, atype[i]);
    if (atype[i] == 2) uniform = 0;
    t8[i] = (int8_t)atype[i];
    fl[i] = replica_flags(ctx, i, xsides[i] > 0 ? FL_FROZEN : 0u);
  }
  const double* src[4] = {X, V, F, Xi};
  double4_32a* dst[4] = {ctx->S.pos, ctx->S.vel, ctx->S.frc, ctx->S.xi};
  for (int k = 0; k < 4; k++) {
    if (!src[k]) {
      CK(cudaMemsetAsync(dst[k], 0, sizeof(double4_32a) * (size_t)N, ctx->stream));
      continue;
    }
    CK(cudaMemcpyAsync(ctx->d_stage, src[k], b3, cudaMemcpyHostToDevice, ctx->stream));
    CK(launch_pack(L, N, dst[k], ctx->d_stage));
  }
  std::vector<double> inv((size_t)N);
  for (int i = 0; i < N; i++) {
    if (!(mass[i] > 0.0)) return fail(ctx, FIBMD_EINVAL, "mass(%d) = %g", i + 1, mass[i]);
    inv[i] = 1.0 / mass[i];
  }
  CK(cudaMemcpyAsync(ctx->S.mass, mass, sizeof(double) * (size_t)N, cudaMemcpyHostToDevice,
                     ctx->stream));
  CK(cudaMemcpyAsync(ctx->S.inv_mass, inv.data(), sizeof(double) * (size_t)N,
                     cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->S.atype, t8.data(), (size_t)N, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->S.flags, fl.data(), sizeof(uint32_t) * (size_t)N,
                     cudaMemcpyHostToDevice, ctx->stream));
  CK(launch_update_posq(L, ctx->P, ctx->S));
  if (ctx->lists_built) CK(launch_track_all(L, ctx->P, ctx->S));
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemsetAsync(&ctx->S.sc->nan_flag, 0, sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(&ctx->S.sc->kd_timeout, 0, sizeof(int), ctx->stream));
  CK(launch_pair_clear(L, ctx->P, ctx->S));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->uploaded = true;
  ctx->spec_ready = false;
  // a new state: the force path is timed again before its first steps
  ctx->tune_pairs = 0;
  ctx->tune_left = 0;
  // a slab without Ge takes the binary32 force kernel's single-species path
  ctx->uniform = uniform;
  ctx->P.uniform = uniform;
  for (auto& k : ctx->skins) k.P.uniform = uniform;
  return FIBMD_OK;
}

int fibmd_gpu_set_tags(fibmd_ctx* ctx, const uint32_t* tags) {
  if (!ctx || !tags) return FIBMD_EINVAL;
  const int N = ctx->P.N;
  std::vector<uint32_t> fl((size_t)N);
  for (int i = 0; i < N; i++) fl[i] = replica_flags(ctx, i, tags[i] & 0xffu);
  CK(cudaMemcpyAsync(ctx->S.flags, fl.data(), sizeof(uint32_t) * (size_t)N,
                     cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  CK(launch_update_posq(launch_of(ctx), ctx->P, ctx->S));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->spec_ready = false;
  return FIBMD_OK;
}

int fibmd_gpu_get_tags(fibmd_ctx* ctx, uint32_t* tags) {
  if (!ctx || !tags) return FIBMD_EINVAL;
  if (!ctx->uploaded) return fail(ctx, FIBMD_ESTATE, "get_tags before upload");
  const int N = ctx->P.N;
  std::vector<uint32_t> fl((size_t)N);
  CK(cudaMemcpyAsync(fl.data(), ctx->S.flags, sizeof(uint32_t) * (size_t)N,
                     cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (int i = 0; i < N; i++) tags[i] = fl[(size_t)i] & 0xffu;
  return FIBMD_OK;
}

int fibmd_gpu_download(fibmd_ctx* ctx, double* X, double* V, double* F) {
  if (!ctx) return FIBMD_EINVAL;
  if (!ctx->uploaded) return fail(ctx, FIBMD_ESTATE, "download before upload");
  const int N = ctx->P.N;
  const size_t b3 = sizeof(double) * 3 * (size_t)N;
  Launch L = launch_of(ctx);
  double* dstv[3] = {X, V, F};
  const double4_32a* srcv[3] = {ctx->S.pos, ctx->S.vel, ctx->S.frc};
  for (int k = 0; k < 3; k++) {
    if (!dstv[k]) continue;
    CK(launch_unpack(L, N, srcv[k], ctx->d_stage));
    CK(cudaMemcpyAsync(dstv[k], ctx->d_stage, b3, cudaMemcpyDeviceToHost, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return FIBMD_OK;
}

int fibmd_gpu_xyz_frame(fibmd_ctx* ctx, double* xyz_A, double* ke_eV) {
  if (!ctx) return FIBMD_EINVAL;
  if (!ctx->uploaded) return fail(ctx, FIBMD_ESTATE, "xyz frame before upload");
  const int N = ctx->P.N;
  CK(launch_xyz_frame(launch_of(ctx), ctx->S, N, ctx->d_stage, ctx->d_ke));
  if (xyz_A)
    CK(cudaMemcpyAsync(xyz_A, ctx->d_stage, sizeof(double) * 3 * (size_t)N,
                       cudaMemcpyDeviceToHost, ctx->stream));
  if (ke_eV)
    CK(cudaMemcpyAsync(ke_eV, ctx->d_ke, sizeof(double) * (size_t)N, cudaMemcpyDeviceToHost,
                       ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return FIBMD_OK;
}

int fibmd_gpu_set_atom(fibmd_ctx* ctx, int i, const double x[3], const double v[3]) {
  if (!ctx || i < 1 || i > ctx->P.N || !x || !v) return fail(ctx, FIBMD_EINVAL, "set_atom: bad args");
  double4_32a px = make_double4_32a(x[0], x[1], x[2], 0.0);
  double4_32a pv = make_double4_32a(v[0], v[1], v[2], 0.0);
  CK(cudaMemcpyAsync(ctx->S.pos + (i - 1), &px, sizeof px, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->S.vel + (i - 1), &pv, sizeof pv, cudaMemcpyHostToDevice, ctx->stream));
  CK(launch_update_posq(launch_of(ctx), ctx->P, ctx->S));
  if (ctx->lists_built) CK(launch_track_all(launch_of(ctx), ctx->P, ctx->S));
  CK(cudaStreamSynchronize(ctx->stream));
  return FIBMD_OK;
}

int fibmd_gpu_set_impact(fibmd_ctx* ctx, int impact) {
  if (!ctx || impact < 0) return FIBMD_EINVAL;
  ctx->impact = impact;
  ctx->P.nfired = ctx->p.Nsg + impact;
  for (auto& k : ctx->skins) k.P.nfired = ctx->P.nfired;
  return FIBMD_OK;
}

int fibmd_gpu_ionrun(fibmd_ctx* ctx, int tic) {
  if (!ctx || (tic != 1 && tic != 2)) return FIBMD_EINVAL;
  set_regime(ctx, tic);
  ctx->atom_is_fast = (tic == 1);
  return FIBMD_OK;
}

int fibmd_gpu_set_tau(fibmd_ctx* ctx, double tau) {
  if (!ctx || !(tau > 0)) return FIBMD_EINVAL;
  ctx->Tau = tau;
  return FIBMD_OK;
}

int fibmd_gpu_regime(fibmd_ctx* ctx, double* Ts, int* tic) {
  if (!ctx) return FIBMD_EINVAL;
  if (Ts) *Ts = ctx->Ts;
  if (tic) *tic = ctx->tic;
  return FIBMD_OK;
}

static int check_list_status(fibmd_ctx* ctx) {
  const DevScalars& h = *ctx->h_sc;
  if (h.nan_flag)
    return fail(ctx, FIBMD_ENAN, "non-finite velocity after a kick (upload a valid state)");
  if (h.kd_timeout)
    return fail(ctx, FIBMD_ETIMEOUT,
                "the fused kick-drift's grid barrier gave up (blocks not resident together); "
                "the state is not valid: upload a state, or set the option \"fuse\" to 0");
  if (h.overflow_sw)
    return fail(ctx, FIBMD_EOVERFLOW,
                "SW list slots exceeded (%d entries dropped): capacity %d, needed %d "
                "(max_sw_nbrs)", h.overflow_sw, ctx->P.max_sw, h.sw_needed);
  if (h.overflow_mol)
    return fail(ctx, FIBMD_EOVERFLOW, "Moliere list needs %d entries, capacity %d",
                h.overflow_mol, ctx->P.mol_cap);
  if (h.table_err)
    return fail(ctx, FIBMD_ETABLE, "2-body table index beyond Ntable (%d pairs)", h.table_err);
  return FIBMD_OK;
}

int fibmd_gpu_nlist(fibmd_ctx* ctx) {
  if (!ctx) return FIBMD_EINVAL;
  if (!ctx->uploaded) return fail(ctx, FIBMD_ESTATE, "nlist before upload");
  {
    PhaseTimer t(ctx, PH_NT);
    CK(launch_build_lists(launch_of(ctx), ctx->P, ctx->S, 0));
  }
  int rc = sync_scalars(ctx);
  if (rc) return rc;
  ctx->lists_built = true;
  return check_list_status(ctx);
}

int fibmd_gpu_list_counts(fibmd_ctx* ctx, long long* n_sw_full, long long* n_mol_full,
                          long long* n_triplets) {
  if (!ctx || !ctx->lists_built) return fail(ctx, FIBMD_ESTATE, "lists not built");
  const int N = ctx->P.N;
  if (n_sw_full) {
    std::vector<int> n((size_t)N);
    CK(cudaMemcpy(n.data(), ctx->S.n_sw, sizeof(int) * (size_t)N, cudaMemcpyDeviceToHost));
    long long s = 0;
    for (int v : n) s += v;
    *n_sw_full = s;
  }
  int rc = sync_scalars(ctx);
  if (rc) return rc;
  if (n_mol_full) *n_mol_full = ctx->h_sc->mol_count;
  if (n_triplets) {
    CK(cudaMemsetAsync(ctx->d_u64, 0, sizeof(unsigned long long), ctx->stream));
    CK(launch_count_triplets(launch_of(ctx), ctx->P, ctx->S, ctx->d_u64, nullptr, 0));
    unsigned long long c = 0;
    CK(cudaMemcpyAsync(&c, ctx->d_u64, sizeof c, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    *n_triplets = (long long)c;
  }
  return FIBMD_OK;
}

int fibmd_gpu_get_pairs(fibmd_ctx* ctx, int kind, int* n, int* ij, int cap) {
  if (!ctx || !n || (kind != 0 && kind != 1)) return FIBMD_EINVAL;
  if (!ctx->lists_built) return fail(ctx, FIBMD_ESTATE, "lists not built");
  const int N = ctx->P.N;
  std::vector<std::pair<int, int>> pr;
  if (kind == 0) {
    std::vector<int> cnt((size_t)N), nb((size_t)ctx->P.max_sw * N);
    CK(cudaMemcpy(cnt.data(), ctx->S.n_sw, sizeof(int) * (size_t)N, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(nb.data(), ctx->S.nbr_sw, sizeof(int) * nb.size(), cudaMemcpyDeviceToHost));
    for (int i = 0; i < N; i++)
      for (int k = 0; k < cnt[i]; k++) {
        int j = nb[(size_t)k * N + i];
        if (j > i) pr.emplace_back(i + 1, j + 1);
      }
  } else {
    int rc = sync_scalars(ctx);
    if (rc) return rc;
    int m = std::min(ctx->h_sc->mol_count, ctx->P.mol_cap);
    std::vector<int2> mp((size_t)m);
    if (m) CK(cudaMemcpy(mp.data(), ctx->S.mol_pairs, sizeof(int2) * (size_t)m, cudaMemcpyDeviceToHost));
    for (auto& q : mp)
      if (q.y > q.x) pr.emplace_back(q.x + 1, q.y + 1);
  }
  std::sort(pr.begin(), pr.end());
  *n = (int)pr.size();
  if (ij)
    for (int k = 0; k < (int)pr.size() && k < cap; k++) {
      ij[2 * k] = pr[k].first;
      ij[2 * k + 1] = pr[k].second;
    }
  return FIBMD_OK;
}

int fibmd_gpu_get_triplets(fibmd_ctx* ctx, long long* n, int* ijk, long long cap) {
  if (!ctx || !n) return FIBMD_EINVAL;
  long long total = 0;
  int rc = fibmd_gpu_list_counts(ctx, nullptr, nullptr, &total);
  if (rc) return rc;
  *n = total;
  if (!ijk || total == 0) return FIBMD_OK;
  int3* d = nullptr;
  CK(cudaMalloc(&d, sizeof(int3) * (size_t)total));
  CK(cudaMemsetAsync(ctx->d_u64, 0, sizeof(unsigned long long), ctx->stream));
  CK(launch_count_triplets(launch_of(ctx), ctx->P, ctx->S, ctx->d_u64, d, total));
  std::vector<int3> h((size_t)total);
  CK(cudaMemcpyAsync(h.data(), d, sizeof(int3) * (size_t)total, cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  cudaFree(d);
  std::sort(h.begin(), h.end(), [](const int3& a, const int3& b) {
    if (a.x != b.x) return a.x < b.x;
    if (a.y != b.y) return a.y < b.y;
    return a.z < b.z;
  });
  for (long long k = 0; k < total && k < cap; k++) {
    ijk[3 * k] = h[k].x + 1;
    ijk[3 * k + 1] = h[k].y + 1;
    ijk[3 * k + 2] = h[k].z + 1;
  }
  return FIBMD_OK;
}

int fibmd_gpu_force(fibmd_ctx* ctx, double* F_out, double* u_out, double* Utot) {
  if (!ctx) return FIBMD_EINVAL;
  if (!ctx->lists_built) return fail(ctx, FIBMD_ESTATE, "force before nlist");
  const bool energy = u_out || Utot;
  {
    PhaseTimer t(ctx, PH_F);
    int rcf = force_launch(ctx, energy, true);
    if (rcf) return rcf;
  }
  std::swap(ctx->S.frc, ctx->S.frc_new);
  if (F_out) {
    int rc = fibmd_gpu_download(ctx, nullptr, nullptr, F_out);
    if (rc) return rc;
  }
  if (energy) {
    const int N = ctx->P.N;
    std::vector<double> u((size_t)N);
    CK(cudaMemcpyAsync(u.data(), ctx->S.epot, sizeof(double) * (size_t)N,
                       cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (u_out) std::memcpy(u_out, u.data(), sizeof(double) * (size_t)N);
    if (Utot) {
      double s = 0.0;
      for (double v : u) s += v;
      *Utot = s;
    }
  }
  int rc = sync_scalars(ctx);
  if (rc) return rc;
  return check_list_status(ctx);
}

int fibmd_gpu_virial(fibmd_ctx* ctx, double W[6], double* w_atom) {
  if (!ctx || !W) return FIBMD_EINVAL;
  if (!ctx->lists_built) return fail(ctx, FIBMD_ESTATE, "virial before nlist");
  const size_t N = (size_t)ctx->P.N;
  if (!ctx->d_vir) {
    int rc = dalloc(ctx, &ctx->d_vir, 6);
    if (rc) return rc;
  }
  if (w_atom && !ctx->d_vir_atom) {
    int rc = dalloc(ctx, &ctx->d_vir_atom, 6 * N);
    if (rc) return rc;
  }
  double* d_atom = w_atom ? ctx->d_vir_atom : nullptr;
  CK(launch_virial(launch_of(ctx), ctx->P, ctx->S, d_atom, ctx->d_vir));
  CK(cudaMemcpyAsync(W, ctx->d_vir, 6 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (w_atom)
    CK(cudaMemcpyAsync(w_atom, d_atom, 6 * sizeof(double) * N, cudaMemcpyDeviceToHost,
                       ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return FIBMD_OK;
}

int fibmd_gpu_work_counters(fibmd_ctx* ctx, long long counts[6]) {
  if (!ctx || !counts) return FIBMD_EINVAL;
  int rc = sync_scalars(ctx);
  if (rc) return rc;
  counts[0] = (long long)(ctx->h_sc->counters[0] / 2);
  counts[1] = (long long)ctx->h_sc->counters[1];
  counts[2] = (long long)(ctx->h_sc->counters[2] / 2);
  counts[3] = (long long)ctx->h_sc->counters[3];
  counts[4] = (long long)ctx->h_sc->rebuilds;
  counts[5] = (long long)ctx->h_sc->heavy_count;
  return FIBMD_OK;
}

int fibmd_gpu_temperature(fibmd_ctx* ctx, double* T) {
  if (!ctx || !T) return FIBMD_EINVAL;
  CK(launch_temperature(launch_of(ctx), ctx->P, ctx->S));
  int rc = sync_scalars(ctx);
  if (rc) return rc;
  *T = ctx->h_sc->temp;
  return FIBMD_OK;
}

int fibmd_gpu_timers(fibmd_ctx* ctx, double* at, double* nt, double* ds, double* f,
                     long long* counts4, int reset) {
  if (!ctx) return FIBMD_EINVAL;
  cudaStreamSynchronize(ctx->stream);
  flush_timers(ctx);
  if (at) *at = ctx->t[PH_AT];
  if (nt) *nt = ctx->t[PH_NT];
  if (ds) *ds = ctx->t[PH_DS];
  if (f) *f = ctx->t[PH_F];
  if (counts4)
    for (int k = 0; k < 4; k++) counts4[k] = ctx->c[k];
  if (reset)
    for (int k = 0; k < 4; k++) {
      ctx->t[k] = 0;
      ctx->c[k] = 0;
    }
  return FIBMD_OK;
}

int fibmd_gpu_phase_times(fibmd_ctx* ctx, double* seconds7, long long* counts7, int reset) {
  if (!ctx) return FIBMD_EINVAL;
  cudaStreamSynchronize(ctx->stream);
  flush_timers(ctx);
  for (int k = 0; k < PH_COUNT; k++) {
    if (seconds7) seconds7[k] = ctx->t[k];
    if (counts7) counts7[k] = ctx->c[k];
    if (reset) {
      ctx->t[k] = 0;
      ctx->c[k] = 0;
    }
  }
  return FIBMD_OK;
}

int fibmd_gpu_set_option(fibmd_ctx* ctx, const char* key, double value) {
  if (!ctx || !key) return FIBMD_EINVAL;
  if (!std::strcmp(key, "timers")) {
    ctx->timers_on = value != 0.0;
  } else if (!std::strcmp(key, "kernel_timing")) {
    ctx->kernel_timing = value != 0.0;
  } else if (!std::strcmp(key, "graph")) {
    ctx->use_graph = value != 0.0;
  } else if (!std::strcmp(key, "autotune")) {
    ctx->autotune = value != 0.0;
  } else if (!std::strcmp(key, "pdl")) {
    ctx->pdl = value != 0.0;
  } else if (!std::strcmp(key, "fuse")) {
    ctx->fuse = value != 0.0;
  } else if (!std::strcmp(key, "rebuild_rule")) {
    if (value != 0.0 && value != 1.0) return fail(ctx, FIBMD_EINVAL, "rebuild_rule must be 0 or 1");
    ctx->rebuild_rule = (int)value;
    const int pr = (ctx->rebuild_rule == 1 && ctx->p.mode == FIBMD_MODE_SPEC) ? 1 : 0;
    ctx->P.pair_rule = pr;
    for (auto& k : ctx->skins) k.P.pair_rule = pr;
  } else if (!std::strcmp(key, "skin_tune")) {
    ctx->skin_tune = value != 0.0;
  } else if (!std::strcmp(key, "heavy_if")) {
    ctx->heavy_if = value != 0.0;
  } else if (!std::strcmp(key, "reactions")) {
    if (value != 0.0 && !ctx->S.react) {
      if (ctx->P.precision != FIBMD_PREC_MIXED || ctx->P.max_sw > kReactMaxList)
        return fail(ctx, FIBMD_EINVAL, "stored reactions need mixed precision and "
                    "max_sw_nbrs <= %d", kReactMaxList);
      // the buffers on first use, and the lists rebuilt with each entry's
      // slot in the partner's list
      const size_t N = (size_t)ctx->P.N;
      DevState& S = ctx->S;
      int rc = dalloc(ctx, &S.rev_sw, (size_t)ctx->P.max_sw * N);
      if (!rc) rc = dalloc(ctx, &S.legpos, N);
      if (!rc) rc = dalloc(ctx, &S.react, (size_t)kStageLarge * N);
      if (!rc) rc = dalloc(ctx, &S.fown, N);
      if (rc) {
        S.rev_sw = nullptr;
        S.legpos = nullptr;
        S.react = nullptr;
        S.fown = nullptr;
        return rc;
      }
      if (ctx->lists_built) {
        CK(launch_build_lists(launch_of(ctx), ctx->P, S, 0));
        CK(cudaStreamSynchronize(ctx->stream));
      }
      drop_graph(ctx);
    }
    ctx->react = value != 0.0;
  } else if (!std::strcmp(key, "force_block")) {
    if (value != 64.0 && value != 128.0)
      return fail(ctx, FIBMD_EINVAL, "force_block must be 64 or 128");
    ctx->force_block = (int)value;
    ctx->autotune = false;
  } else if (!std::strcmp(key, "build_block")) {
    if (value != 64.0 && value != 128.0 && value != 256.0)
      return fail(ctx, FIBMD_EINVAL, "build_block must be 64, 128 or 256");
    ctx->build_block = (int)value;
    ctx->build_tune = false;
  } else if (!std::strcmp(key, "skin")) {
    // one of the candidate skins (Angstrom); fixes it (no more tuning)
    int k = -1;
    for (size_t q = 0; q < ctx->skins.size(); q++)
      if (std::fabs(ctx->skins[q].skin * 1e10 - value) < 1e-6) k = (int)q;
    if (k < 0) return fail(ctx, FIBMD_EINVAL, "skin %g A is not one of the candidates", value);
    ctx->skin_tune = false;
    int rc = set_skin(ctx, k);
    if (rc) return rc;
  } else if (!std::strcmp(key, "kd_grid")) {
    if (value < 0.0 || value > (double)kMaxRedBlocks)
      return fail(ctx, FIBMD_EINVAL, "kd_grid %g out of range", value);
    ctx->kd_grid = (int)value;
    ctx->graph_fuse = -1;  // recapture
  } else if (!std::strcmp(key, "stage")) {
    if (value != kStageSmall && value != kStageLarge && value != kStageGroup)
      return fail(ctx, FIBMD_EINVAL, "stage must be %d, %d or %d", kStageSmall, kStageLarge,
                  kStageGroup);
    ctx->stage = (int)value;
    ctx->autotune = false;
  } else {
    return fail(ctx, FIBMD_EINVAL, "unknown option '%s'", key);
  }
  return FIBMD_OK;
}

int fibmd_gpu_get_option(fibmd_ctx* ctx, const char* key, double* value) {
  if (!ctx || !key || !value) return FIBMD_EINVAL;
  if (!std::strcmp(key, "timers")) {
    *value = ctx->timers_on ? 1.0 : 0.0;
  } else if (!std::strcmp(key, "kernel_timing")) {
    *value = ctx->kernel_timing ? 1.0 : 0.0;
  } else if (!std::strcmp(key, "graph")) {
    *value = ctx->use_graph ? 1.0 : 0.0;
  } else if (!std::strcmp(key, "autotune")) {
    *value = ctx->autotune ? 1.0 : 0.0;
  } else if (!std::strcmp(key, "pdl")) {
    *value = ctx->pdl ? 1.0 : 0.0;
  } else if (!std::strcmp(key, "fuse")) {
    *value = fuse_in_use(ctx) ? 1.0 : 0.0;
  } else if (!std::strcmp(key, "rebuild_rule")) {
    *value = (double)ctx->P.pair_rule;
  } else if (!std::strcmp(key, "skin_tune")) {
    *value = ctx->skin_tune ? 1.0 : 0.0;
  } else if (!std::strcmp(key, "heavy_if")) {
    *value = ctx->heavy_if ? 1.0 : 0.0;
  } else if (!std::strcmp(key, "reactions")) {
    *value = ctx->react ? 1.0 : 0.0;
  } else if (!std::strcmp(key, "force_block")) {
    *value = (double)ctx->force_block;
  } else if (!std::strcmp(key, "build_block")) {
    *value = (double)ctx->build_block;
  } else if (!std::strcmp(key, "skin")) {
    *value = ctx->skins[(size_t)ctx->skin_cur].skin * 1e10;
  } else if (!std::strcmp(key, "skin_candidates")) {
    *value = (double)ctx->skins.size();
  } else if (!std::strcmp(key, "kd_grid")) {
    *value = (double)(ctx->kd_grid > 0 ? ctx->kd_grid : ctx->kd_blocks);
  } else if (!std::strcmp(key, "stage")) {
    *value = (double)ctx->stage;
  } else {
    return fail(ctx, FIBMD_EINVAL, "unknown option '%s'", key);
  }
  return FIBMD_OK;
}

int fibmd_gpu_kernel_time(fibmd_ctx* ctx, double* force_kernel_s, long long* launches,
                          int reset) {
  if (!ctx) return FIBMD_EINVAL;
  cudaStreamSynchronize(ctx->stream);
  flush_timers(ctx);
  if (force_kernel_s) *force_kernel_s = ctx->t[PH_FK];
  if (launches) *launches = ctx->c[PH_FK];
  if (reset) {
    ctx->t[PH_FK] = 0;
    ctx->c[PH_FK] = 0;
  }
  return FIBMD_OK;
}

// ---- one reference step (onestep, timeint.f90:158-242) ---------------------------
static int onestep(fibmd_ctx* ctx, int whichctrl, long long lt, double* time, int* why) {
  const Launch L = launch_of(ctx);
  const DevParams& P = ctx->P;
  const double Ttar = ctx->p.Ttar1;
  *time = *time + ctx->Ts;
  {
    PhaseTimer t(ctx, PH_DRIFT);
    if (whichctrl == 0) CK(launch_adjust_and_temp(L, P, ctx->S, ctx->Ts, ctx->Tau, Ttar));
    if (whichctrl > 0) CK(launch_side_reduce(L, P, ctx->S, ctx->Ts, ctx->Tau, Ttar));
    CK(launch_drift(L, P, ctx->S, ctx->Ts, ctx->Tau, Ttar, whichctrl > 0));
  }
  if (ctx->atlist > 0 && lt % ctx->atlist == 0) {
    PhaseTimer t(ctx, PH_AT);
    CK(launch_park(L, P, ctx->S));
  }
  if (ctx->ntlist > 0 && lt % ctx->ntlist == 0) {
    PhaseTimer t(ctx, PH_NT);
    CK(launch_build_lists(L, P, ctx->S, 0));
  }
  if (ctx->dslist > 0 && lt % ctx->dslist == 0 && whichctrl == 1) {
    {
      PhaseTimer t(ctx, PH_DS);
      CK(launch_ke_max(L, P, ctx->S));
    }
    int rc = sync_scalars(ctx);
    if (rc) return rc;
    if (ctx->h_sc->ke_max < ctx->p.ke_limit_1 && ctx->atom_is_fast) {
      set_regime(ctx, 2);
      ctx->atom_is_fast = false;
      *why |= FIBMD_STOP_REGIME;
    }
  }
  {
    PhaseTimer t(ctx, PH_F);
    int rcf = force_launch(ctx, false, false);
    if (rcf) return rcf;
  }
  {
    PhaseTimer t(ctx, PH_KICK);
    CK(launch_kick(L, P, ctx->S, ctx->Ts));
  }
  std::swap(ctx->S.frc, ctx->S.frc_new);
  return FIBMD_OK;
}

// The spec-mode step loop as one CUDA graph: a WHILE node runs step pairs
// (the force buffers swap back after two steps) until the device-side loop
// counter or the relaxation's end time stops it; after each drift an IF node
// runs the list rebuild only when the drift found it due (the rebuild rule).
//   unfused: WHILE { [drift, cond, IF{rebuild}, force, kick] x 2, loop control }
//   fused ("fuse", the default): drift, cond, IF{rebuild},
//            WHILE { [force, kick + next drift, IF{rebuild}] x 2 }
// In the fused form each kick runs in one persistent kernel with the next
// step's drift (k_spec_kd), which also sets the IF condition and, at the end
// of a pair, the WHILE condition; when the loop stops it does not drift, so
// the state on exit is that of a completed step in both forms.
static int build_spec_graph(fibmd_ctx* ctx) {
  drop_graph(ctx);
  if (!ctx->cap2) CK(cudaStreamCreateWithFlags(&ctx->cap2, cudaStreamNonBlocking));
  const DevParams& P = ctx->P;
  const double Ttar = ctx->p.Ttar1;
  const bool fused = fuse_in_use(ctx);
  cudaGraph_t g = nullptr;
  CK(cudaGraphCreate(&g, 0));
  ctx->graph = g;
  cudaGraphConditionalHandle hw;
  CK(cudaGraphConditionalHandleCreate(&hw, g, 1, cudaGraphCondAssignDefault));

  cudaStream_t cs = ctx->stream;
  Launch L = launch_of(ctx);
  Launch L2 = L;
  L2.stream = ctx->cap2;
  DevState Sx = ctx->S;
  auto abort_capture = [&](cudaError_t e, const char* what) {
    cudaGraph_t tmp = nullptr;
    cudaStreamEndCapture(cs, &tmp);
    drop_graph(ctx);
    return fail(ctx, FIBMD_ECUDA, "graph capture (%s): %s", what, cudaGetErrorString(e));
  };
#define CKC(call, what)                                     \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return abort_capture(e_, what);  \
  } while (0)
  // an IF node on the capture's current dependencies, its body what body()
  // launches on the second stream (L2), made the new dependency
  auto add_if = [&](cudaGraphConditionalHandle hi, auto body) -> cudaError_t {
    cudaStreamCaptureStatus st;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(cs, &st, nullptr, &cg, &deps, nullptr, &nd);
    if (e != cudaSuccess) return e;
    cudaGraphNodeParams ip = {};
    ip.type = cudaGraphNodeTypeConditional;
    ip.conditional.handle = hi;
    ip.conditional.type = cudaGraphCondTypeIf;
    ip.conditional.size = 1;
    cudaGraphNode_t inode;
    e = cudaGraphAddNode(&inode, cg, deps, nullptr, nd, &ip);
    if (e != cudaSuccess) return e;
    e = cudaStreamUpdateCaptureDependencies(cs, &inode, nullptr, 1,
                                            cudaStreamSetCaptureDependencies);
    if (e != cudaSuccess) return e;
    cudaGraph_t ib = ip.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(ctx->cap2, ib, nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    const cudaError_t eb = body();
    cudaGraph_t tmp = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(ctx->cap2, &tmp);
    return eb != cudaSuccess ? eb : ee;
  };
  auto add_rebuild_if = [&](cudaGraphConditionalHandle hi) -> cudaError_t {
    return add_if(hi, [&] { return launch_build_lists(L2, P, Sx, 2); });
  };
  // With the option "heavy_if", the many-leg kernel of each step sits in an
  // IF node: the force kernel opens it when a centre has more legs than its
  // stage (a cascade core), the kernel before the force closes it, so steps
  // without such centres skip the launch. The eight-lanes-per-centre path
  // has no such centres. Off by default: on the 256k cascade the step took
  // 101.3 us with the nodes against 91.8 us with a plain launch every step.
  const bool heavy_if =
      ctx->heavy_if && !(P.precision == FIBMD_PREC_MIXED && ctx->stage == kStageGroup);
  Launch L2h = L2;
  L2h.pdl = false;
  cudaGraphNodeParams wp = {};
  wp.type = cudaGraphNodeTypeConditional;
  wp.conditional.handle = hw;
  wp.conditional.type = cudaGraphCondTypeWhile;
  wp.conditional.size = 1;
  if (fused) {
    // the prologue: the first step's drift and rebuild, then the WHILE node
    CK(cudaStreamBeginCaptureToGraph(cs, g, nullptr, nullptr, 0,
                                     cudaStreamCaptureModeThreadLocal));
    cudaGraphConditionalHandle h0;
    CKC(cudaGraphConditionalHandleCreate(&h0, g, 0, cudaGraphCondAssignDefault), "handle");
    CKC(launch_spec_drift(L, P, Sx, Ttar, &h0), "drift");
    CKC(add_rebuild_if(h0), "rebuild");
    cudaStreamCaptureStatus st;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    CKC(cudaStreamGetCaptureInfo(cs, &st, nullptr, nullptr, &deps, nullptr, &nd), "deps");
    cudaGraphNode_t wnode;
    CKC(cudaGraphAddNode(&wnode, g, deps, nullptr, nd, &wp), "while node");
    CKC(cudaStreamUpdateCaptureDependencies(cs, &wnode, nullptr, 1,
                                            cudaStreamSetCaptureDependencies), "update");
    cudaGraph_t tmp = nullptr;
    CK(cudaStreamEndCapture(cs, &tmp));
  } else {
    cudaGraphNode_t wnode;
    CK(cudaGraphAddNode(&wnode, g, nullptr, nullptr, 0, &wp));
  }
  cudaGraph_t body = wp.conditional.phGraph_out[0];
  // (a handle that no IF node uses fails the instantiation)
  cudaGraphConditionalHandle hh[2] = {0, 0};
  if (heavy_if)
    for (int half = 0; half < 2; half++)
      CK(cudaGraphConditionalHandleCreate(&hh[half], body, 0, cudaGraphCondAssignDefault));
  CK(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0,
                                   cudaStreamCaptureModeThreadLocal));
  for (int half = 0; half < 2; half++) {
    cudaStreamCaptureStatus st;
    cudaGraph_t cg = nullptr;
    CKC(cudaStreamGetCaptureInfo(cs, &st, nullptr, &cg, nullptr, nullptr, nullptr), "info");
    cudaGraphConditionalHandle hi;
    CKC(cudaGraphConditionalHandleCreate(&hi, cg, 0, cudaGraphCondAssignDefault), "handle");
    Launch Lf = L;
    Lf.heavy_if = heavy_if;
    Lf.heavy_handle = hh[half];
    auto force = [&]() -> cudaError_t {
      cudaError_t e = launch_force(Lf, P, Sx, false, false, true);
      if (e == cudaSuccess && heavy_if)
        e = add_if(hh[half], [&] { return launch_force_heavy(L2h, P, Sx); });
      return e;
    };
    if (fused) {
      CKC(force(), "force");
      CKC(launch_spec_kd(L, P, Sx, Ttar, ctx->d_loop, hi, hw, half == 1,
                         ctx->kd_grid > 0 ? ctx->kd_grid : ctx->kd_blocks,
                         heavy_if ? &hh[1 - half] : nullptr),
          "kick-drift");
      CKC(add_rebuild_if(hi), "rebuild");
    } else {
      // the drift's last block sets the rebuild condition; the second
      // step's drift follows the first step's kick as its programmatic
      // dependent
      CKC(launch_spec_drift(L, P, Sx, Ttar, &hi, half == 1, heavy_if ? &hh[half] : nullptr),
          "drift");
      CKC(add_rebuild_if(hi), "rebuild");
      CKC(force(), "force");
      CKC(launch_spec_kick(L, P, Sx, Ttar, 1), "kick");
    }
    std::swap(Sx.frc, Sx.frc_new);
  }
  if (!fused) CKC(launch_loop_ctl(cs, ctx->d_loop, Sx.sc, hw, L.pdl), "loop");
#undef CKC
  cudaGraph_t out = nullptr;
  CK(cudaStreamEndCapture(cs, &out));
  cudaError_t ei = cudaGraphInstantiate(&ctx->graph_exec, g, 0);
  if (ei != cudaSuccess) {
    drop_graph(ctx);
    return fail(ctx, FIBMD_ECUDA, "graph instantiate: %s", cudaGetErrorString(ei));
  }
  ctx->graph_frc = ctx->S.frc;
  ctx->graph_stage = ctx->stage;
  ctx->graph_nfired = P.nfired;
  ctx->graph_pdl = ctx->pdl ? 1 : 0;
  ctx->graph_fuse = ctx->fuse ? 1 : 0;
  ctx->graph_skin = ctx->skin_cur;
  ctx->graph_force_block = ctx->force_block;
  ctx->graph_build_block = ctx->build_block;
  ctx->graph_uniform = ctx->P.uniform;
  ctx->graph_pair = ctx->P.pair_rule;
  ctx->graph_react = ctx->react ? 1 : 0;
  ctx->graph_heavy_if = ctx->heavy_if ? 1 : 0;
  return FIBMD_OK;
}

// Runs `pairs` x 2 spec-mode steps with one graph launch.
// Enqueues `pairs` step pairs (stopping early after `relax` seconds of
// simulated time when relax > 0); returns without waiting.
constexpr long long kTuneSteps = 1000;  // spec-mode steps between stage re-tunings

// Times the binary32 force kernel with each stage size on the current state
// (one untimed and two timed evaluations each) and keeps the faster one. It
// reads the lists, so it runs only once they are built; the evaluations
// accumulate into the next-force buffer, which the caller clears.
// Device time (ms) of three force evaluations with the given stage, each a
// launch of a captured graph as the step loop runs it, so that a path of
// fewer kernels is credited with the launch gaps it saves.
static int time_force_graph(fibmd_ctx* ctx, int stage, int block, bool react, cudaEvent_t a,
                            cudaEvent_t b, float* ms) {
  Launch L = launch_of(ctx);
  L.stage = stage;
  L.force_block = block;
  L.react = react;
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  const cudaError_t e = launch_force(L, ctx->P, ctx->S, false, false, false);
  const cudaError_t ee = cudaStreamEndCapture(ctx->stream, &g);
  if (e != cudaSuccess || ee != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return fail(ctx, FIBMD_ECUDA, "force-stage timing capture: %s",
                cudaGetErrorString(e != cudaSuccess ? e : ee));
  }
  cudaGraphExec_t x = nullptr;
  cudaError_t r = cudaGraphInstantiate(&x, g, 0);
  cudaGraphDestroy(g);
  if (r == cudaSuccess) r = cudaGraphLaunch(x, ctx->stream);
  if (r == cudaSuccess) r = cudaEventRecord(a, ctx->stream);
  for (int k = 0; k < 3 && r == cudaSuccess; k++) r = cudaGraphLaunch(x, ctx->stream);
  if (r == cudaSuccess) r = cudaEventRecord(b, ctx->stream);
  if (r == cudaSuccess) r = cudaEventSynchronize(b);
  if (r == cudaSuccess) r = cudaEventElapsedTime(ms, a, b);
  if (x) cudaGraphExecDestroy(x);
  if (r != cudaSuccess)
    return fail(ctx, FIBMD_ECUDA, "force-stage timing: %s", cudaGetErrorString(r));
  return FIBMD_OK;
}

static int tune_stage(fibmd_ctx* ctx) {
  if (ctx->P.precision != FIBMD_PREC_MIXED || !ctx->autotune || !ctx->lists_built)
    return FIBMD_OK;
  cudaEvent_t a = get_event(ctx), b = get_event(ctx);
  // (force path, centres per block): one thread per centre with the small
  // or large stage in blocks of 128 or 64, or eight lanes per centre
  // (the stored-reaction form is not a candidate: its gather pass runs its
  // binary64 sums on the SM's FP64 pipe, where the atomics have the L2 do
  // them, and costs several times the atomics it saves)
  constexpr int kCand = 5;
  const int stages[kCand] = {kStageSmall, kStageSmall, kStageLarge, kStageLarge, kStageGroup};
  const int blocks[kCand] = {128, 64, 128, 64, 128};
  int cur = 0;
  for (int q = 0; q < kCand; q++)
    if (stages[q] == ctx->stage && (stages[q] == kStageGroup || blocks[q] == ctx->force_block))
      cur = q;
  // every fourth tuning times all candidates; the others skip those that
  // were over 1.5 times the best last time (the tuning runs are steps'
  // worth of force evaluations)
  float* ms = ctx->tune_ms;
  float last_best = 0.f;
  const bool full = ctx->tune_count % 4 == 0;
  if (!full) {
    last_best = ms[0];
    for (int q = 1; q < kCand; q++) last_best = std::min(last_best, ms[q]);
  }
  int rc = FIBMD_OK;
  for (int q = 0; q < kCand && rc == FIBMD_OK; q++) {
    if (!full && q != cur && ms[q] > 1.5f * last_best) continue;
    rc = time_force_graph(ctx, stages[q], blocks[q], ctx->react, a, b, &ms[q]);
  }
  ctx->pool.push_back(a);
  ctx->pool.push_back(b);
  if (rc) return rc;
  ctx->tune_count++;
  // switch only for a clear gain: a switch recaptures the step graph
  int best = 0;
  for (int q = 0; q < kCand; q++)
    if (ms[q] < ms[best]) best = q;
  ctx->tune_switched = ms[best] < 0.97f * ms[cur];
  if (ctx->tune_switched) {
    ctx->stage = stages[best];
    ctx->force_block = blocks[best];
  }
  return FIBMD_OK;
}

static int run_spec_graph(fibmd_ctx* ctx, long long pairs, double relax = 0.0) {
  if (!ctx->graph_exec || ctx->graph_frc != ctx->S.frc || ctx->graph_nfired != ctx->P.nfired ||
      ctx->graph_stage != ctx->stage || ctx->graph_pdl != (ctx->pdl ? 1 : 0) ||
      ctx->graph_fuse != (ctx->fuse ? 1 : 0) || ctx->graph_skin != ctx->skin_cur ||
      ctx->graph_force_block != ctx->force_block || ctx->graph_build_block != ctx->build_block ||
      ctx->graph_uniform != ctx->P.uniform || ctx->graph_pair != ctx->P.pair_rule ||
      ctx->graph_react != (ctx->react ? 1 : 0) ||
      ctx->graph_heavy_if != (ctx->heavy_if ? 1 : 0)) {
    int rc = build_spec_graph(ctx);
    if (rc && ctx->pdl) {
      // a device or driver without programmatic edges in conditional
      // bodies: capture the graph with plain launches instead
      cudaGetLastError();
      ctx->pdl = false;
      rc = build_spec_graph(ctx);
    }
    if (rc) return rc;
  }
  if (pairs <= 0) return FIBMD_OK;
  CK(launch_loop_set(ctx->stream, ctx->d_loop, ctx->S.sc, pairs, relax));
  CK(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
  return FIBMD_OK;
}

constexpr long long kSkinTrialPairs = 20;      // step pairs timed per candidate skin
constexpr long long kSkinTuneEvery = 5;        // tuning chunks between skin tunings
constexpr long long kSkinTuneMinSteps = 2000;  // shorter calls keep the skin in use

// The list skin, re-chosen on the current state: each candidate runs one
// step pair (its forced list rebuild and graph capture) and then
// kSkinTrialPairs pairs timed with CUDA events, the one in use last; the
// fastest per step is kept if it beats the one in use by 3 %. The trial
// steps are steps of the run: with any of the skins the lists hold every
// pair inside the cutoffs, so the trajectory does not depend on the choice.
// *pairs_run receives the step pairs taken.
static int tune_skin(fibmd_ctx* ctx, long long* pairs_run) {
  *pairs_run = 0;
  const int n = (int)ctx->skins.size();
  const int start = ctx->skin_cur;
  cudaEvent_t a = get_event(ctx), b = get_event(ctx);
  std::vector<float> ms((size_t)n, 0.f);
  int rc = FIBMD_OK;
  for (int q = 0; q < n && rc == FIBMD_OK; q++) {
    const int k = (start + 1 + q) % n;
    rc = set_skin(ctx, k);
    if (rc == FIBMD_OK) rc = run_spec_graph(ctx, 1);
    if (rc) break;
    cudaEventRecord(a, ctx->stream);
    rc = run_spec_graph(ctx, kSkinTrialPairs);
    if (rc) break;
    cudaEventRecord(b, ctx->stream);
    const cudaError_t e = cudaEventSynchronize(b);
    if (e != cudaSuccess) {
      rc = fail(ctx, FIBMD_ECUDA, "skin tuning: %s", cudaGetErrorString(e));
      break;
    }
    cudaEventElapsedTime(&ms[(size_t)k], a, b);
    *pairs_run += 1 + kSkinTrialPairs;
  }
  ctx->pool.push_back(a);
  ctx->pool.push_back(b);
  if (rc) return rc;
  int best = start;
  for (int k = 0; k < n; k++)
    if (ms[(size_t)k] < ms[(size_t)best]) best = k;
  if (ms[(size_t)best] < 0.97f * ms[(size_t)start]) rc = set_skin(ctx, best);
  return rc;
}

// The pair-list build's atoms per block, re-chosen on the current state:
// two list builds timed with CUDA events for each of 64, 128 and 256 (the
// lists are those of the current positions whichever builds them); kept
// if 3 % faster than the one in use.
static int tune_build(fibmd_ctx* ctx) {
  const int cand[3] = {64, 128, 256};
  float ms[3] = {};
  cudaEvent_t a = get_event(ctx), b = get_event(ctx);
  cudaError_t e = cudaSuccess;
  for (int q = 0; q < 3 && e == cudaSuccess; q++) {
    Launch L = launch_of(ctx);
    L.build_block = cand[q];
    e = launch_build_lists(L, ctx->P, ctx->S, 0);
    if (e == cudaSuccess) e = cudaEventRecord(a, ctx->stream);
    for (int r = 0; r < 2 && e == cudaSuccess; r++) e = launch_build_lists(L, ctx->P, ctx->S, 0);
    if (e == cudaSuccess) e = cudaEventRecord(b, ctx->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[q], a, b);
  }
  ctx->pool.push_back(a);
  ctx->pool.push_back(b);
  if (e != cudaSuccess) return fail(ctx, FIBMD_ECUDA, "build tuning: %s", cudaGetErrorString(e));
  int cur = 1, best = 0;
  for (int q = 0; q < 3; q++) {
    if (cand[q] == ctx->build_block) cur = q;
    if (ms[q] < ms[best]) best = q;
  }
  if (ms[best] < 0.97f * ms[cur]) ctx->build_block = cand[best];
  return FIBMD_OK;
}

static int spec_steps(fibmd_ctx* ctx, long long max_steps, long long* lt, double* time,
                      double* temp, int* reason) {
  const Launch L = launch_of(ctx);
  const DevParams& P = ctx->P;
  const double Ttar = ctx->p.Ttar1;
  if (!ctx->spec_ready) {
    const double t0 = *time;
    for (int r = 0; r < P.nrep; r++)
      CK(cudaMemcpyAsync(&ctx->S.sc[r].time, &t0, sizeof(double), cudaMemcpyHostToDevice,
                         ctx->stream));
    CK(launch_spec_kick(L, P, ctx->S, Ttar, 0));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->spec_ready = true;
  }
  // the step's force accumulates into a buffer the previous kick zeroed;
  // the first step of a call starts from whatever the buffer holds
  CK(cudaMemsetAsync(ctx->S.frc_new, 0, sizeof(double4_32a) * (size_t)P.N, ctx->stream));
  long long todo = max_steps;
  if (ctx->use_graph && todo >= 2) {
    // in chunks, before each of which the binary32 force kernel's stage size
    // is re-chosen on the current state when it is due: kTuneSteps steps
    // after an upload or a change of path, then twice as many as last time,
    // up to 8 * kTuneSteps, counted across calls
    const bool tune = ctx->autotune && P.precision == FIBMD_PREC_MIXED && ctx->lists_built;
    // and in long calls, before every kSkinTuneEvery-th chunk, the list skin
    const bool stune = ctx->skin_tune && ctx->skins.size() > 1 && ctx->lists_built &&
                       todo >= kSkinTuneMinSteps;
    for (long long pairs = todo / 2; pairs > 0;) {
      if (stune && ctx->graph_chunks % kSkinTuneEvery == 0 &&
          pairs > (long long)ctx->skins.size() * (kSkinTrialPairs + 1)) {
        CK(cudaStreamSynchronize(ctx->stream));
        long long pr = 0;
        int rs = tune_skin(ctx, &pr);
        if (rs == FIBMD_OK && ctx->build_tune) {
          CK(cudaStreamSynchronize(ctx->stream));
          rs = tune_build(ctx);
        }
        if (rs) return rs;
        pairs -= pr;
      }
      ctx->graph_chunks++;
      if (tune && ctx->tune_left <= 0) {
        CK(cudaStreamSynchronize(ctx->stream));
        int rt = tune_stage(ctx);
        if (rt) return rt;
        CK(cudaMemsetAsync(ctx->S.frc_new, 0, sizeof(double4_32a) * (size_t)P.N, ctx->stream));
        // the next tuning comes later while the choice stands
        const long long base = kTuneSteps / 2;
        ctx->tune_pairs = (ctx->tune_switched || ctx->tune_pairs <= 0)
                              ? base
                              : std::min(2 * ctx->tune_pairs, 8 * base);
        ctx->tune_left = ctx->tune_pairs;
      }
      const long long chunk =
          tune ? std::min(pairs, ctx->tune_left) : stune ? std::min(pairs, kTuneSteps / 2) : pairs;
      int rc = run_spec_graph(ctx, chunk);
      if (rc) return rc;
      pairs -= chunk;
      if (tune) ctx->tune_left -= chunk;
    }
    *lt += 2 * (todo / 2);
    todo -= 2 * (todo / 2);
  }
  for (long long n = 0; n < todo; n++) {
    {
      PhaseTimer t(ctx, PH_DRIFT);
      CK(launch_spec_drift(L, P, ctx->S, Ttar));
    }
    {
      PhaseTimer t(ctx, PH_NT);
      CK(launch_build_lists(L, P, ctx->S, 2));
    }
    {
      PhaseTimer t(ctx, PH_F);
      int rcf = force_launch(ctx, false, false, true);
      if (rcf) return rcf;
    }
    {
      PhaseTimer t(ctx, PH_KICK);
      CK(launch_spec_kick(L, P, ctx->S, Ttar, 1));
    }
    std::swap(ctx->S.frc, ctx->S.frc_new);
    *lt = *lt + 1;
  }
  int rc = sync_scalars(ctx);
  if (rc) return rc;
  *time = ctx->h_sc->time;
  if (temp) {
    rc = fibmd_gpu_temperature(ctx, temp);
    if (rc) return rc;
  }
  *reason = FIBMD_STOP_MAXSTEPS;
  return check_list_status(ctx);
}

int fibmd_gpu_dose(fibmd_ctx* ctx, int nimp, const int* ion_atoms, const double* x,
                   const double* v, long long steps, double relax_s, int* removed_after,
                   int* ions_removed_after, double* time_after, long long* steps_after) {
  if (!ctx || nimp < 0 || (nimp > 0 && (!ion_atoms || !x || !v)) || steps < 1)
    return fail(ctx, FIBMD_EINVAL, "dose: bad arguments");
  if (ctx->P.mode != FIBMD_MODE_SPEC || ctx->P.nrep != 1)
    return fail(ctx, FIBMD_ESTATE, "dose: needs a single spec-mode system");
  if (!ctx->use_graph) return fail(ctx, FIBMD_ESTATE, "dose: needs the graph step loop");
  if (!ctx->lists_built) return fail(ctx, FIBMD_ESTATE, "dose: lists not built");
  if (nimp == 0) return FIBMD_OK;
  const int N = ctx->P.N;
  std::vector<Impact> tab((size_t)nimp);
  for (int k = 0; k < nimp; k++) {
    const int a = ion_atoms[k];
    if (a < 1 || a > N) return fail(ctx, FIBMD_EINVAL, "dose: ion atom %d out of range", a);
    tab[k].atom = a - 1;
    for (int d = 0; d < 3; d++) {
      tab[k].x[d] = x[(size_t)d * nimp + k];
      tab[k].v[d] = v[(size_t)d * nimp + k];
    }
  }
  Impact* d_tab = nullptr;
  int* d_rec = nullptr;
  double* d_time = nullptr;
  long long* d_steps = nullptr;
  if (cudaMalloc((void**)&d_tab, sizeof(Impact) * (size_t)nimp) != cudaSuccess ||
      cudaMalloc((void**)&d_rec, sizeof(int) * 2 * (size_t)nimp) != cudaSuccess ||
      cudaMalloc((void**)&d_time, sizeof(double) * (size_t)nimp) != cudaSuccess ||
      cudaMalloc((void**)&d_steps, sizeof(long long) * (size_t)(nimp + 1)) != cudaSuccess) {
    cudaFree(d_tab);
    cudaFree(d_rec);
    cudaFree(d_time);
    cudaFree(d_steps);
    return fail(ctx, FIBMD_ENOMEM, "dose: %d impacts", nimp);
  }
  auto done = [&](int rc) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(d_tab);
    cudaFree(d_rec);
    cudaFree(d_time);
    cudaFree(d_steps);
    return rc;
  };
  const Launch L = launch_of(ctx);
  const DevParams& P = ctx->P;
  const double Ttar = ctx->p.Ttar1;
  // the force stage size for the whole dose, chosen on the slab as it is
  {
    int rt = tune_stage(ctx);
    if (rt) return done(rt);
  }
  cudaError_t e = cudaMemcpyAsync(d_tab, tab.data(), sizeof(Impact) * (size_t)nimp,
                                  cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(ctx->S.frc_new, 0, sizeof(double4_32a) * (size_t)N, ctx->stream);
  if (e != cudaSuccess) return done(fail(ctx, FIBMD_ECUDA, "dose: %s", cudaGetErrorString(e)));
  ctx->spec_ready = true;
  // the step count before the first impact
  if (e == cudaSuccess) e = launch_dose_record(L, ctx->S, ctx->d_loop, 0, d_rec, d_rec + nimp,
                                               d_time, d_steps);
  if (e != cudaSuccess) return done(fail(ctx, FIBMD_ECUDA, "dose: %s", cudaGetErrorString(e)));
  // every impact is enqueued at once: inject, a fresh step size for the new
  // ion's speed, the cascade steps, the relaxation, the counts
  for (int k = 0; k < nimp; k++) {
    e = launch_inject(L, P, ctx->S, d_tab, k);
    if (e == cudaSuccess) e = launch_spec_kick(L, P, ctx->S, Ttar, 0);
    if (e != cudaSuccess) return done(fail(ctx, FIBMD_ECUDA, "dose: %s", cudaGetErrorString(e)));
    int rc = run_spec_graph(ctx, (steps + 1) / 2);
    if (rc == FIBMD_OK && relax_s > 0.0) rc = run_spec_graph(ctx, 1ll << 50, relax_s);
    if (rc) return done(rc);
    e = launch_dose_record(L, ctx->S, ctx->d_loop, k, d_rec, d_rec + nimp, d_time, d_steps + 1);
    if (e != cudaSuccess) return done(fail(ctx, FIBMD_ECUDA, "dose: %s", cudaGetErrorString(e)));
  }
  std::vector<int> rec(2 * (size_t)nimp);
  std::vector<double> tm((size_t)nimp);
  std::vector<long long> st((size_t)nimp + 1);
  e = cudaMemcpyAsync(st.data(), d_steps, sizeof(long long) * st.size(), cudaMemcpyDeviceToHost,
                      ctx->stream);
  if (e != cudaSuccess) return done(fail(ctx, FIBMD_ECUDA, "dose: %s", cudaGetErrorString(e)));
  e = cudaMemcpyAsync(rec.data(), d_rec, sizeof(int) * rec.size(), cudaMemcpyDeviceToHost,
                      ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(tm.data(), d_time, sizeof(double) * tm.size(), cudaMemcpyDeviceToHost,
                        ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return done(fail(ctx, FIBMD_ECUDA, "dose: %s", cudaGetErrorString(e)));
  for (int k = 0; k < nimp; k++) {
    if (removed_after) removed_after[k] = rec[k];
    if (ions_removed_after) ions_removed_after[k] = rec[nimp + k];
    if (time_after) time_after[k] = tm[k];
    if (steps_after) steps_after[k] = st[k + 1] - st[0];
  }
  int rc = sync_scalars(ctx);
  if (rc == FIBMD_OK) rc = check_list_status(ctx);
  return done(rc);
}

int fibmd_gpu_steps(fibmd_ctx* ctx, int whichctrl, long long max_steps, long long* lt,
                    double* time, double* temp, int* reason) {
  if (!ctx || !lt || !time || !temp || !reason) return FIBMD_EINVAL;
  if (!ctx->uploaded || !ctx->lists_built)
    return fail(ctx, FIBMD_ESTATE, "steps before upload and nlist");
  if (whichctrl < 0 || whichctrl > 2) return fail(ctx, FIBMD_EINVAL, "whichctrl %d", whichctrl);
  *reason = 0;
  if (ctx->p.mode == FIBMD_MODE_SPEC) return spec_steps(ctx, max_steps, lt, time, temp, reason);
  const double Ttar = ctx->p.Ttar1;
  int why = 0;
  if (whichctrl == 0) {
    // adjusttemp uses the temperature the caller's loop holds
    CK(cudaMemcpyAsync(&ctx->S.sc->temp, temp, sizeof(double), cudaMemcpyHostToDevice,
                       ctx->stream));
  }
  long long n = 0;
  for (;;) {
    if (whichctrl == 0 && !(std::fabs(*temp - Ttar) > ctx->p.Teps)) {
      why |= FIBMD_STOP_DONE;
      break;
    }
    if (n >= max_steps) {
      why |= FIBMD_STOP_MAXSTEPS;
      break;
    }
    const long long l = *lt + 1;
    *lt = l;
    if (whichctrl == 1 && *time > (double)ctx->impact * ctx->p.dti) {
      why |= FIBMD_STOP_DONE;
      break;
    }
    int rc = onestep(ctx, whichctrl, l, time, &why);
    if (rc) return rc;
    n++;
    if (whichctrl == 0) {
      rc = sync_scalars(ctx);
      if (rc) return rc;
      *temp = ctx->h_sc->temp;
    } else {
      // iostuff: atm_out/res_out steps hand the state to the host writer
      const bool dump = (ctx->p.res_out > 0 && l % ctx->p.res_out == 0) ||
                        (ctx->atm_out > 0 && l % ctx->atm_out == 0);
      if (dump) {
        rc = fibmd_gpu_temperature(ctx, temp);
        if (rc) return rc;
        why |= FIBMD_STOP_DUMP;
        break;
      }
    }
  }
  *reason = why;
  int rc = sync_scalars(ctx);
  if (rc) return rc;
  return check_list_status(ctx);
}

}  // extern "C"
