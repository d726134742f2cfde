// fibmd_force.cu — fused Stillinger-Weber 2/3-body + Moliere force.
//
// Replaces si_force (src/si.f90:384-552), itable2bd (src/si.f90:554-573) and
// si_potential (src/si.f90:278-380).
//
// The reference loops over a half pair list (table-interpolated SW 2-body),
// a half Moliere list, and every connected triplet of the build-time list
// graph (all three angle terms, each gated by both legs < 0.999*a*sigma).
// Here one thread owns one centre atom and its full list:
//   - 2-body: the reference's table interpolation for every listed pair, the
//     centre's own share only (the partner's thread computes the mirror
//     term, bit-identical with opposite sign), so no atomics.
//   - 3-body: the centre's active legs (u < 0.999a) are staged in shared
//     memory; every leg pair (a,b) is one angle term centred here. Its
//     reactions on the legs are summed per leg and scattered with one
//     binary64 atomic per leg component.
//   - Moliere: a pair-parallel kernel over the full Moliere list.
//   - Stale lists: the reference also evaluates angle terms whose centre-leg
//     is missing from the build-time list when the other two edges of the
//     triple are listed. Such a term is non-zero only if that pair moved
//     more than the list skin (rc - 0.999a*sigma) since the build, so only
//     atoms displaced by at least half the skin ("fast" atoms, flagged by
//     the integrator) can carry one; a correction kernel enumerates them.
//     With it the set of non-zero terms equals the reference's exactly.
// Centres with more than kMaxLegs active legs are deferred to a direct
// binary64 kernel.
#include <algorithm>
#include <atomic>
#include <type_traits>

#include "fibmd_internal.cuh"

namespace fibmd {

// 3-point Lagrange interpolation of the derivative table (itable2bd).
// it = INT(ue/umax*(Ntable-1)) is the 0-based first stencil point.
__device__ __forceinline__ double table_df(const DevParams& P, const double* __restrict__ tab,
                                           const double* __restrict__ tabu, double ue,
                                           int* err) {
  const double t = ue / P.umax * (double)(P.Ntable - 1);
  // a non-finite ue (a corrupted state, reported by the kick) must not
  // become an index
  if (!(t >= 0.0)) return 0.0;
  // the reference's check: i = INT(t) + 1 > Ntable is an error, and 0 is used
  if (t >= (double)P.Ntable) {
    *err = 1;
    return 0.0;
  }
  // all three stencil entries are zero beyond tab_last
  if (!(t < (double)(P.tab_last + 1))) return 0.0;
  const int it = (int)t;
  const double d1 = ue - __ldg(&tabu[it]);
  const double d2 = ue - __ldg(&tabu[it + 1]);
  const double d3 = ue - __ldg(&tabu[it + 2]);
  return 0.5 * d2 * d3 * __ldg(&tab[it]) - d1 * d3 * __ldg(&tab[it + 1]) +
         0.5 * d1 * d2 * __ldg(&tab[it + 2]);
}

// ---- binary64 per-centre kernel --------------------------------------------
// Each thread stages up to kMaxLegs active legs (unit vector, 1/r, E, g and
// a reaction accumulator: 9 doubles) in shared memory and evaluates every
// unordered leg pair once: binary64 instructions are the scarce resource on
// this GPU, so no term is computed twice.
constexpr int kLegF64 = 9;   // ux uy uz rinv E g fx fy fz
constexpr int kBlock64 = 64;
constexpr int kLegF32 = 6;   // ux uy uz rinv E g
constexpr int kBlock32 = 128;
constexpr int kCandF64 = 16;  // prefiltered neighbours staged per centre (binary64 kernel)
// (the binary32 paths, kStageSmall, kStageLarge and kStageGroup, are in
// fibmd_internal.cuh: the context chooses among them)

constexpr int kBatch = 8;    // neighbour gathers in flight per thread

template <typename R, int BLOCK, int F>
struct LegSmem {
  R* v;
  int* j;
  __device__ __forceinline__ R& at(int l, int f) { return v[(l * F + f) * BLOCK + threadIdx.x]; }
  __device__ __forceinline__ int& idx(int l) { return j[l * BLOCK + threadIdx.x]; }
};

// set_hh: the step graph runs the many-leg kernel in an IF node whose
// condition hh a centre that goes to it sets (the node stays closed in the
// many steps without such centres).
template <bool ENERGY, bool COUNT>
__global__ void __launch_bounds__(kBlock64) k_force_fp64(DevParams P, DevState S,
                                                         cudaGraphConditionalHandle hh,
                                                         int set_hh) {
  pdl_wait();
  pdl_trigger();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  LegSmem<double, kBlock64, kLegF64> leg;
  leg.v = reinterpret_cast<double*>(smem_raw);
  leg.j = reinterpret_cast<int*>(smem_raw + sizeof(double) * kMaxLegs * kLegF64 * kBlock64);
  int* cand = leg.j + kMaxLegs * kBlock64;  // [kCandF64][kBlock64]

  const int i = blockIdx.x * kBlock64 + threadIdx.x;
  if (i >= P.N) return;
  const int4 qi = S.posq[i];
  const int ti = qi.w & 0xff;
  if (ti >= 3 || ((qi.w >> 8) & FL_REMOVED)) return;
  const int n = S.n_sw[i];
  if (n == 0) return;
  const double4_32a pi = S.pos[i];
  const int ta = ti - 1;
  const Geo& G = S.geo[rep_of_w(qi.w)];
  const float qinvA[3] = {G.qinvA[0], G.qinvA[1], G.qinvA[2]};
  const double Lb[3] = {G.Lb[0], G.Lb[1], G.Lb[2]}, iLb[3] = {G.iLb[0], G.iLb[1], G.iLb[2]};

  double fx = 0.0, fy = 0.0, fz = 0.0, ui = 0.0;
  int nl = 0, terr = 0;
  unsigned int cnt_pairs = 0, cnt_ang = 0;

  // One listed neighbour inside the prefilter: the table 2-body force on the
  // centre and, inside 0.999*a*sigma, its staged leg.
  auto neighbour = [&](int j, int tb) {
    const double4_32a pj = S.pos[j];
    const double dx = min_image(pi.x, pj.x, iLb[0], Lb[0]);
    const double dy = min_image(pi.y, pj.y, iLb[1], Lb[1]);
    const double dz = min_image(pi.z, pj.z, iLb[2], Lb[2]);
    const double r2 = dx * dx + dy * dy + dz * dz;
    const double r = sqrt(r2);
    const double rinv = 1.0 / r;
    const double isig = P.isig[ta][tb];
    const double ue = r * isig;
    const double df = table_df(P, S.tab, S.tabu, ue, &terr);
    if (df != 0.0) {
      const double c = -(df * rinv * P.epssig[ta][tb]);
      fx += c * dx;
      fy += c * dy;
      fz += c * dz;
      if (COUNT) cnt_pairs++;
    }
    if (ue < P.cut3) {
      const double inv = 1.0 / (ue - P.al);
      if (ENERGY)
        ui += 0.5 * P.eps[ta][tb] * P.A * (P.B * pow(ue, -P.psi) - pow(ue, -P.qsi)) * exp(inv);
      if (nl < kMaxLegs) {
        leg.at(nl, 0) = dx * rinv;
        leg.at(nl, 1) = dy * rinv;
        leg.at(nl, 2) = dz * rinv;
        leg.at(nl, 3) = rinv;
        leg.at(nl, 4) = exp(P.gam * inv);
        leg.at(nl, 5) = -P.gam * inv * inv * isig;
        leg.at(nl, 6) = 0.0;
        leg.at(nl, 7) = 0.0;
        leg.at(nl, 8) = 0.0;
        leg.idx(nl) = j | (tb << 30);
      }
      nl++;
    }
  };

  // Phase 1: gather the listed neighbours and keep (in list order) the few
  // inside the prefilter; phase 2 runs the binary64 work on that compacted
  // set, so the lanes of a warp issue it together (binary64 instructions are
  // the scarce resource, and a warp instruction costs the pipe the same
  // whether 8 or 32 lanes take part). Candidates beyond the slots are
  // evaluated at once.
  int nc = 0;
  for (int k0 = 0; k0 < n; k0 += kBatch) {
    int jj[kBatch];
    int4 qq[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; u++) jj[u] = (k0 + u < n) ? S.nbr_sw[(size_t)(k0 + u) * P.N + i] : i;
#pragma unroll
    for (int u = 0; u < kBatch; u++) qq[u] = S.posq[jj[u]];
#pragma unroll
    for (int u = 0; u < kBatch; u++) {
      if (k0 + u >= n) break;
      const float3 dq = qsep(qi, qq[u], qinvA);
      const float r2f = dq.x * dq.x + dq.y * dq.y + dq.z * dq.z;
      // beyond the table support and 3-body cutoff, or removed (spec mode:
      // a removed atom acts on nothing from the step it leaves)
      if (r2f > P.pre3A2 || ((qq[u].w >> 8) & FL_REMOVED)) continue;
      const int tb = (qq[u].w & 0xff) - 1;
      if (nc < kCandF64) cand[nc++ * kBlock64 + threadIdx.x] = jj[u] | (tb << 30);
      else neighbour(jj[u], tb);
    }
  }
  // Phase 2
  for (int c = 0; c < nc; c++) {
    const int e = cand[c * kBlock64 + threadIdx.x];
    neighbour(e & 0x3fffffff, (unsigned)e >> 30);
  }

  if (nl > kMaxLegs) {
    // the warp-per-centre kernel evaluates this centre's angle terms
    const int slot = atomicAdd(&S.sc->heavy_count, 1);
    S.heavy_list[slot] = i;
    if (set_hh) cudaGraphSetConditional(hh, 1u);
  } else {
    const double thrd = P.thrd;
    double cfx = 0, cfy = 0, cfz = 0, cu = 0;
    for (int a = 0; a < nl; a++) {
      const double ax = leg.at(a, 0), ay = leg.at(a, 1), az = leg.at(a, 2);
      const double ar = leg.at(a, 3), aE = leg.at(a, 4), ag = leg.at(a, 5);
      const int tbA = (unsigned)leg.idx(a) >> 30;
      // F_a = pref [W g_a p_a + 2(c+1/3)(p_b - c p_a)/r_a], p = unit(X_c - X_a),
      // summed over b as p_a sum_b q (c3 g_a - 2 c / r_a) + (2 / r_a) sum_b q p_b
      // with q = pref c3, c3 = c + 1/3 (leg a in registers), and leg b's
      // term q (c3 g_b - 2 c / r_b) p_b + (2 q / r_b) p_a into its slots
      const double m2ar = -2.0 * ar;
      double swa = 0, sbx = 0, sby = 0, sbz = 0, ae = 0;
      for (int b = a + 1; b < nl; b++) {
        const double bx = leg.at(b, 0), by = leg.at(b, 1), bz = leg.at(b, 2);
        const double br = leg.at(b, 3), bE = leg.at(b, 4), bg = leg.at(b, 5);
        const int tbB = (unsigned)leg.idx(b) >> 30;
        const double cs = ax * bx + ay * by + az * bz;
        const double c3 = cs + thrd;
        const double pref = P.leps[ta][tbA][tbB] * aE * bE;
        const double q = pref * c3;
        swa += q * (c3 * ag + m2ar * cs);
        sbx += q * bx;
        sby += q * by;
        sbz += q * bz;
        const double tb = q * (c3 * bg - 2.0 * br * cs), ub = 2.0 * br * q;
        leg.at(b, 6) += tb * bx + ub * ax;
        leg.at(b, 7) += tb * by + ub * ay;
        leg.at(b, 8) += tb * bz + ub * az;
        if (ENERGY) {
          const double e = q * c3;
          cu += e;
          ae += e;
          atomicAdd(&S.epot[leg.idx(b) & 0x3fffffff], e / 3.0);
        }
        if (COUNT && pref != 0.0) cnt_ang++;
      }
      // leg a's terms with the legs before it are already in its slots
      const double tar = -m2ar;
      const double Fax = leg.at(a, 6) + (swa * ax + tar * sbx);
      const double Fay = leg.at(a, 7) + (swa * ay + tar * sby);
      const double Faz = leg.at(a, 8) + (swa * az + tar * sbz);
      leg.at(a, 6) = Fax;
      leg.at(a, 7) = Fay;
      leg.at(a, 8) = Faz;
      cfx -= Fax;
      cfy -= Fay;
      cfz -= Faz;
      if (ENERGY && ae != 0.0) atomicAdd(&S.epot[leg.idx(a) & 0x3fffffff], ae / 3.0);
    }
    // each angle term gives a third of its energy to each of its atoms
    if (ENERGY) ui += cu / 3.0;
    for (int a = 0; a < nl; a++)
      atomic_add3(S.frc_new, leg.idx(a) & 0x3fffffff, leg.at(a, 6), leg.at(a, 7), leg.at(a, 8));
    fx += cfx;
    fy += cfy;
    fz += cfz;
  }
  atomic_add3(S.frc_new, i, fx, fy, fz);
  if (ENERGY && ui != 0.0) atomicAdd(&S.epot[i], ui);
  if (terr) atomicAdd(&S.sc->table_err, 1);
  if (COUNT) {
    // one atomic per converged group of lanes
    const unsigned m = __activemask();
    const unsigned sp = __reduce_add_sync(m, cnt_pairs), sa = __reduce_add_sync(m, cnt_ang);
    if ((threadIdx.x & 31) == __ffs(m) - 1) {
      if (sp) atomicAdd(&S.sc->counters[0], (unsigned long long)sp);
      if (sa) atomicAdd(&S.sc->counters[1], (unsigned long long)sa);
    }
  }
}

// ---- binary32 (mixed) per-centre kernel ------------------------------------
// Separations come from the fixed-point shadow (binary32 with the precision
// of the separation), arithmetic is binary32 in Angstrom/eV; per-thread
// partial sums are binary32 over at most a few dozen terms, and every
// cross-thread accumulation of the per-atom force is a binary64 atomic.
// The leg pairs are evaluated as ordered pairs: each leg's reaction is summed
// in registers over its row and scattered once, so the shared-memory stage
// holds only 6 floats per leg (more resident warps for the gathers).
template <bool MIXED, bool ENERGY>
__device__ __forceinline__ void moliere_entries(const DevParams& P, const DevState& S, int first,
                                                int stride);
// blocks of the mixed force kernel that do the Moliere pairs: one per two
// ions (an ion has a few dozen listed pairs, both orders), at least two
inline int mol_blocks(const DevParams& P) { return std::max(2, std::min(1024, (P.nion + 1) / 2)); }

// BLK centres per block (128, or 64 chosen by the context's tuning); the
// resident threads per SM are the same for both (896). UNI: every lattice
// atom is Si (P.uniform), so the per-species constants are the [0] entries,
// read directly rather than through a computed index. REACT: the reactions
// on the legs and the centre's own force are stored (S.react, S.fown,
// S.legpos) for k_force_gather instead of added by binary64 atomics.
template <bool ENERGY, bool COUNT, int LEGS, int BLK, bool UNI = false, bool REACT = false>
__global__ void __launch_bounds__(BLK, 896 / BLK) k_force_mixed(DevParams P, DevState S,
                                                                cudaGraphConditionalHandle hh,
                                                                int set_hh) {
  pdl_wait();
  pdl_trigger();
  // the last mol_blocks blocks evaluate the Moliere list (a few dozen pairs
  // per ion), which saves a launch per step
  const int nbm = (P.N + BLK - 1) / BLK;
  if ((int)blockIdx.x >= nbm) {
    moliere_entries<true, ENERGY>(P, S, ((int)blockIdx.x - nbm) * BLK + threadIdx.x,
                                  ((int)gridDim.x - nbm) * BLK);
    return;
  }
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // per slot and thread: A = (dq, r^2) of a candidate, then (unit vector, E)
  // of a leg; B = (1/r, g) of a leg; I = neighbour index | type << 30. Vector
  // accesses keep the shared-memory instruction count low.
  float4* sA = reinterpret_cast<float4*>(smem_raw);
  float2* sB = reinterpret_cast<float2*>(smem_raw + sizeof(float4) * LEGS * BLK);
  int* sI = reinterpret_cast<int*>(smem_raw + (sizeof(float4) + sizeof(float2)) * LEGS *
                                                  BLK);
  const int t = threadIdx.x;

  const int i = blockIdx.x * BLK + threadIdx.x;
  if (i >= P.N) return;
  const int4 qi = S.posq[i];
  const int ti = qi.w & 0xff;
  const int n = S.n_sw[i];
  if (ti >= 3 || ((qi.w >> 8) & FL_REMOVED) || n == 0) {
    if (REACT) {
      S.legpos[i] = 0ull;
      S.fown[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    return;
  }
  const int ta = UNI ? 0 : ti - 1;
  const Geo& G = S.geo[rep_of_w(qi.w)];
  const float qinvA[3] = {G.qinvA[0], G.qinvA[1], G.qinvA[2]};
  const float al = (float)P.al, cut = (float)P.cut3, gm = (float)P.gam;
  const float Bc = (float)P.B, Ac = (float)P.A;

  float fx = 0.f, fy = 0.f, fz = 0.f, ui = 0.f;
  int nl = 0;
  unsigned int cnt_pairs = 0, cnt_ang = 0;

  // One listed pair inside the SW cutoff: its 2-body force on the centre and
  // its leg parameters. Returns false outside the cutoff.
  // The exponentials and the reciprocal use the hardware approximations
  // (a few binary32 ulps, inside the binary32 path's stated error).
  auto pair_leg = [&](const float3& dq, float r2f, int tb_in, float* rinv_o, float* E_o,
                      float* g_o) -> bool {
    const int tb = UNI ? 0 : tb_in;
    const float rinv = rsqrtf(r2f);
    const float r = r2f * rinv;
    const float is = P.isigA[ta][tb];
    const float ue = r * is;
    if (!(ue < cut)) return false;
    const float inv = __fdividef(1.0f, ue - al);
    const float ex = __expf(inv);
    const float iu = P.sigA[ta][tb] * rinv;  // 1/u
    const float u2 = iu * iu;
    const float u4 = u2 * u2;
    // psi = 4, qsi = 0: dphi/du = A e^{1/(u-a)} [ -4 B u^-5 - (B u^-4 - 1)/(u-a)^2 ]
    const float dphi = Ac * ex * (-4.0f * Bc * u4 * iu - (Bc * u4 - 1.0f) * inv * inv);
    const float c = -(dphi * rinv * P.epssigA[ta][tb]);
    fx += c * dq.x;
    fy += c * dq.y;
    fz += c * dq.z;
    if (COUNT) cnt_pairs++;
    if (ENERGY) ui += 0.5f * P.epsA[ta][tb] * Ac * (Bc * u4 - 1.0f) * ex;
    *rinv_o = rinv;
    *E_o = __expf(gm * inv);
    *g_o = -gm * inv * inv * is;
    return true;
  };

  // Phase 1: gather the listed neighbours and stage the few that can be legs
  // (about 4 of 16 in a crystal) in the leg slots, so the costly pair/leg
  // arithmetic of phase 2 runs on compacted candidates with the lanes of a
  // warp busy together. Pairs between the leg radius and the cutoff (2-body
  // only) are evaluated in place; a centre with more legs than slots
  // evaluates the rest in place and goes to the many-leg kernel.
  int nc = 0, extra = 0;
  for (int k0 = 0; k0 < n; k0 += kBatch) {
    int jj[kBatch];
    int4 qq[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; u++) jj[u] = (k0 + u < n) ? S.nbr_sw[(size_t)(k0 + u) * P.N + i] : i;
#pragma unroll
    for (int u = 0; u < kBatch; u++) qq[u] = S.posq[jj[u]];
#pragma unroll
    for (int u = 0; u < kBatch; u++) {
      if (k0 + u >= n) break;
      const float3 dq = qsep(qi, qq[u], qinvA);
      const float r2f = dq.x * dq.x + dq.y * dq.y + dq.z * dq.z;
      if (r2f > P.pre3mA2 || ((qq[u].w >> 8) & FL_REMOVED)) continue;
      const int tb = (qq[u].w & 0xff) - 1;
      if (r2f <= P.pre3lA2 && nc < LEGS) {
        sA[nc * BLK + t] = make_float4(dq.x, dq.y, dq.z, r2f);
        // the partner, or with stored reactions its list position
        sI[nc * BLK + t] = (REACT ? k0 + u : jj[u]) | (tb << 30);
        nc++;
      } else {
        float rinv, E, g;
        if (pair_leg(dq, r2f, tb, &rinv, &E, &g) && E > kLegEmin) extra++;
      }
    }
  }
  // Phase 2: pair forces and legs of the staged candidates; active legs are
  // compacted in place (slot nl <= c is written after slot c is read).
#pragma unroll 2
  for (int c = 0; c < nc; c++) {
    const float4 cd = sA[c * BLK + t];
    const float3 dq = make_float3(cd.x, cd.y, cd.z);
    const float r2f = cd.w;
    const int idx = sI[c * BLK + t];
    float rinv, E, g;
    if (!pair_leg(dq, r2f, (unsigned)idx >> 30, &rinv, &E, &g)) continue;
    if (E > kLegEmin) {
      sA[nl * BLK + t] = make_float4(dq.x * rinv, dq.y * rinv, dq.z * rinv, E);
      sB[nl * BLK + t] = make_float2(rinv, g);
      sI[nl * BLK + t] = idx;
      nl++;
    }
  }
  // legs beyond the slots were not staged: the many-leg kernel takes the centre
  if (extra) nl = kMaxLegs + 1;

  // eV/A -> N in binary32 (a normal number: 1.6e-9 times the force), so each
  // binary64 atomic costs one conversion
  const float convf = (float)P.f_evA_to_N;
  double ue_J = 0.0;
  unsigned long long lpos = 0ull;  // legpos of the centre (REACT)
  if (nl > kMaxLegs) {
    const int slot = atomicAdd(&S.sc->heavy_count, 1);
    S.heavy_list[slot] = i;
    if (set_hh) cudaGraphSetConditional(hh, 1u);
    lpos = kLegsHeavy << 60;
  } else {
    const float thrd = (float)P.thrd;
    float cu = 0.f;
    for (int a = 0; a < nl; a++) {
      const float4 la = sA[a * BLK + t];
      const float2 lb = sB[a * BLK + t];
      const float ax = la.x, ay = la.y, az = la.z, aE = la.w;
      const float ar = lb.x, ag = lb.y;
      const int ia = sI[a * BLK + t];
      const int tbA = (unsigned)ia >> 30;
      // The force on leg a from its terms with the other legs b, with
      // q = pref (cos + 1/3), pref = lambda E_a E_b:
      //   sum_b pref [W g_a a + 2 (cos + 1/3) r_a^-1 (b - cos a)]
      //     = a sum_b q ((cos + 1/3) g_a - 2 r_a^-1 cos) + 2 r_a^-1 sum_b q b,
      // so the loop sums one scalar and one vector per pair.
      const float m2ar = -2.0f * ar;
      float sw = 0.f, sbx = 0.f, sby = 0.f, sbz = 0.f, ae = 0.f;
      // not unrolled: 79.1 against 79.4 us per step with two (four: 79.4)
#pragma unroll 1
      for (int b = 0; b < nl; b++) {
        if (b == a) continue;
        const float4 lbb = sA[b * BLK + t];
        const int tbB = (unsigned)sI[b * BLK + t] >> 30;
        const float cs = ax * lbb.x + ay * lbb.y + az * lbb.z;
        const float c3 = cs + thrd;
        const float pref = P.lepsA[ta][UNI ? 0 : tbA][UNI ? 0 : tbB] * aE * lbb.w;
        const float q = pref * c3;
        sw += q * (c3 * ag + m2ar * cs);
        sbx += q * lbb.x;
        sby += q * lbb.y;
        sbz += q * lbb.z;
        if (ENERGY) ae += q * c3;
        if (COUNT && b > a && pref != 0.f) cnt_ang++;
      }
      const float tar = -m2ar;
      const float afx = sw * ax + tar * sbx;
      const float afy = sw * ay + tar * sby;
      const float afz = sw * az + tar * sbz;
      if (REACT) {
        S.react[(size_t)a * P.N + i] = make_float4(afx, afy, afz, 0.f);
        lpos |= (unsigned long long)(ia & 63) << (6 * a);
      } else {
        atomic_add3(S.frc_new, ia & 0x3fffffff, (double)(convf * afx), (double)(convf * afy),
                    (double)(convf * afz));
      }
      fx -= afx;
      fy -= afy;
      fz -= afz;
      if (ENERGY) {
        // leg a's share of its terms; the centre gets a third of each term
        if (ae != 0.f) atomicAdd(&S.epot[ia & 0x3fffffff], P.e_eV_to_J * (double)ae / 3.0);
        cu += ae;
      }
    }
    if (ENERGY) ue_J = P.e_eV_to_J * (double)cu / 6.0;
    lpos |= (unsigned long long)nl << 60;
  }
  if (REACT) {
    S.legpos[i] = lpos;
    S.fown[i] = make_float4(fx, fy, fz, 0.f);
  } else {
    atomic_add3(S.frc_new, i, (double)(convf * fx), (double)(convf * fy), (double)(convf * fz));
  }
  if (ENERGY) {
    const double e = P.e_eV_to_J * (double)ui + ue_J;
    if (e != 0.0) atomicAdd(&S.epot[i], e);
  }
  if (COUNT) {
    const unsigned m = __activemask();
    const unsigned sp = __reduce_add_sync(m, cnt_pairs), sa = __reduce_add_sync(m, cnt_ang);
    if ((threadIdx.x & 31) == __ffs(m) - 1) {
      if (sp) atomicAdd(&S.sc->counters[0], (unsigned long long)sp);
      if (sa) atomicAdd(&S.sc->counters[1], (unsigned long long)sa);
    }
  }
}

// ---- one angle term in binary64, used by the direct and correction paths ---
// Centre c with legs a, b (separations p = X_c - X_leg, lengths r). Adds the
// forces to fc/fa/fb and returns the term energy; zero unless both legs are
// inside 0.999*a*sigma.
struct Leg64 {
  double dx, dy, dz, r, u, isig;
  int t;
};

__device__ __forceinline__ Leg64 make_leg(const DevParams& P, const Geo& G,
                                          const double4_32a& pc, const double4_32a& pl,
                                          int tc, int tl) {
  Leg64 L;
  L.dx = min_image(pc.x, pl.x, G.iLb[0], G.Lb[0]);
  L.dy = min_image(pc.y, pl.y, G.iLb[1], G.Lb[1]);
  L.dz = min_image(pc.z, pl.z, G.iLb[2], G.Lb[2]);
  L.r = sqrt(L.dx * L.dx + L.dy * L.dy + L.dz * L.dz);
  L.isig = P.isig[tc - 1][tl - 1];
  L.u = L.r * L.isig;
  L.t = tl - 1;
  return L;
}

__device__ __forceinline__ bool angle_term(const DevParams& P, int tc, const Leg64& A,
                                           const Leg64& B, double fc[3], double fa[3],
                                           double fb[3], double* e) {
  *e = 0.0;
  if (!(A.u < P.cut3 && B.u < P.cut3)) return false;
  const double ia = 1.0 / (A.u - P.al), ib = 1.0 / (B.u - P.al);
  const double Ea = exp(P.gam * ia), Eb = exp(P.gam * ib);
  const double ga = -P.gam * ia * ia * A.isig, gb = -P.gam * ib * ib * B.isig;
  const double ra = 1.0 / A.r, rb = 1.0 / B.r;
  const double ax = A.dx * ra, ay = A.dy * ra, az = A.dz * ra;
  const double bx = B.dx * rb, by = B.dy * rb, bz = B.dz * rb;
  const double cs = ax * bx + ay * by + az * bz;
  const double c3 = cs + P.thrd, W = c3 * c3, s2 = 2.0 * c3;
  const double pref = P.leps[tc - 1][A.t][B.t] * Ea * Eb;
  const double wa = W * ga - s2 * cs * ra, sa = s2 * ra;
  const double wb = W * gb - s2 * cs * rb, sb = s2 * rb;
  fa[0] = pref * (wa * ax + sa * bx);
  fa[1] = pref * (wa * ay + sa * by);
  fa[2] = pref * (wa * az + sa * bz);
  fb[0] = pref * (wb * bx + sb * ax);
  fb[1] = pref * (wb * by + sb * ay);
  fb[2] = pref * (wb * bz + sb * az);
  fc[0] = -(fa[0] + fb[0]);
  fc[1] = -(fa[1] + fb[1]);
  fc[2] = -(fa[2] + fb[2]);
  *e = pref * W;
  return true;
}

// ---- virial (an observable, binary64 in both precisions) -------------------
// W = sum over interactions of r (x) f: for a pair, the separation from
// the partner to the centre times the force on the centre (each side of a
// full-list pair adds half); for an angle term, minus the separation from
// the centre to each leg times the force on that leg. Per atom, each
// centre's terms (and half of each of its pairs) are its own. One warp per
// centre: lanes take the listed neighbours (2-body table force, legs staged
// in shared memory), then the unordered leg pairs. Components xx, yy, zz,
// xy, xz, yz, in J. The Moliere pairs are added by k_virial_mol; the
// reference mode's stale-list angle terms are not included.
constexpr int kVirWarps = 4;
constexpr int kVirLegs = 64;  // >= max_sw (checked at context creation)
__device__ __forceinline__ void vir_add(double v[6], double dx, double dy, double dz, double fx,
                                        double fy, double fz, double s) {
  v[0] += s * dx * fx;
  v[1] += s * dy * fy;
  v[2] += s * dz * fz;
  v[3] += s * 0.5 * (dx * fy + dy * fx);
  v[4] += s * 0.5 * (dx * fz + dz * fx);
  v[5] += s * 0.5 * (dy * fz + dz * fy);
}

__global__ void __launch_bounds__(32 * kVirWarps) k_virial(DevParams P, DevState S,
                                                           double* w_atom, double* w_tot) {
  __shared__ Leg64 legs[kVirWarps][kVirLegs];
  __shared__ int nleg[kVirWarps];
  __shared__ double btot[kVirWarps][6];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t N = (size_t)P.N;
  double acc[6] = {0, 0, 0, 0, 0, 0};  // this warp's total (lane 0)
  int terr = 0;
  for (int c = blockIdx.x * kVirWarps + w; c < P.N; c += gridDim.x * kVirWarps) {
    if (lane == 0) nleg[w] = 0;
    __syncwarp();
    double v[6] = {0, 0, 0, 0, 0, 0};
    const int4 qc = S.posq[c];
    const int tc = qc.w & 0xff;
    const bool live = tc < 3 && !((qc.w >> 8) & FL_REMOVED);
    if (live) {
      const int n = min(S.n_sw[c], P.max_sw);
      const double4_32a pc = S.pos[c];
      const Geo& G = S.geo[rep_of_w(qc.w)];
      for (int k = lane; k < n; k += 32) {
        const int j = S.nbr_sw[(size_t)k * N + c];
        const int4 qj = S.posq[j];
        if ((qj.w >> 8) & FL_REMOVED) continue;
        const int tj = qj.w & 0xff;
        const Leg64 L = make_leg(P, G, pc, S.pos[j], tc, tj);
        const double df = table_df(P, S.tab, S.tabu, L.u, &terr);
        if (df != 0.0) {
          const double cf = -(df / L.r * P.epssig[tc - 1][tj - 1]);
          vir_add(v, L.dx, L.dy, L.dz, cf * L.dx, cf * L.dy, cf * L.dz, 0.5);
        }
        if (L.u < P.cut3) {
          const int q = atomicAdd(&nleg[w], 1);
          if (q < kVirLegs) legs[w][q] = L;
        }
      }
    }
    __syncwarp();
    const int nl = min(nleg[w], kVirLegs);
    for (int a = lane; a < nl; a += 32) {
      const Leg64 A = legs[w][a];
      for (int b = a + 1; b < nl; b++) {
        const Leg64 B = legs[w][b];
        double fc[3], fa[3], fb[3], e;
        if (!angle_term(P, tc, A, B, fc, fa, fb, &e)) continue;
        vir_add(v, A.dx, A.dy, A.dz, fa[0], fa[1], fa[2], -1.0);
        vir_add(v, B.dx, B.dy, B.dz, fb[0], fb[1], fb[2], -1.0);
      }
    }
#pragma unroll
    for (int k = 0; k < 6; k++) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    }
    if (lane == 0) {
      if (w_atom)
        for (int k = 0; k < 6; k++) w_atom[(size_t)k * N + c] = v[k];
      for (int k = 0; k < 6; k++) acc[k] += v[k];
    }
    __syncwarp();
  }
  if (lane == 0)
    for (int k = 0; k < 6; k++) btot[w][k] = acc[k];
  __syncthreads();
  if (threadIdx.x < 6) {
    double t = 0.0;
    for (int q = 0; q < kVirWarps; q++) t += btot[q][threadIdx.x];
    atomicAdd(&w_tot[threadIdx.x], t);
  }
}

// The Moliere pairs' share: each list entry (i, j) adds half of r (x) f for
// the force on i (both orders are listed); unfired ions are skipped, as in
// the force.
__global__ void k_virial_mol(DevParams P, DevState S, double* w_atom, double* w_tot) {
  int cnt = *((volatile int*)&S.sc->mol_count);
  if (cnt > P.mol_cap) cnt = P.mol_cap;
  double v[6] = {0, 0, 0, 0, 0, 0};
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += gridDim.x * blockDim.x) {
    const int2 pr = S.mol_pairs[e];
    const int i = pr.x, j = pr.y;
    if (!(i < P.nfired && j < P.nfired)) continue;
    if ((S.flags[i] | S.flags[j]) & FL_REMOVED) continue;
    const int ti = S.atype[i] - 1, tj = S.atype[j] - 1;
    const double4_32a pi = S.pos[i], pj = S.pos[j];
    const Geo& G = S.geo[rep_of_flags(S.flags[i])];
    const double dx = min_image(pi.x, pj.x, G.iLb[0], G.Lb[0]);
    const double dy = min_image(pi.y, pj.y, G.iLb[1], G.Lb[1]);
    const double dz = min_image(pi.z, pj.z, G.iLb[2], G.Lb[2]);
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (!(r2 < P.rlj2)) continue;
    const double rij = sqrt(r2);
    const double aa = P.aamol[ti][tj];
    const double e1 = exp(-(P.amol * rij / aa)), e2 = exp(-(P.bmol * rij / aa)),
                 e3 = exp(-(P.gmol * rij / aa));
    const double K = P.ie0 * P.Zmol[ti] * P.Zmol[tj] * P.ec * P.ec;
    const double fc = K / rij *
                      ((P.Amol * e1 + P.Bmol * e2 + P.Cmol * e3) / rij +
                       (P.Amol * P.amol / aa * e1 + P.Bmol * P.bmol / aa * e2 +
                        P.Cmol * P.gmol / aa * e3));
    const double fcr = fc / rij;
    double u[6] = {0, 0, 0, 0, 0, 0};
    vir_add(u, dx, dy, dz, fcr * dx, fcr * dy, fcr * dz, 0.5);
    for (int k = 0; k < 6; k++) {
      if (w_atom) atomicAdd(&w_atom[(size_t)k * (size_t)P.N + i], u[k]);
      v[k] += u[k];
    }
  }
  for (int k = 0; k < 6; k++) {
    double t = v[k];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0 && t != 0.0) atomicAdd(&w_tot[k], t);
  }
}

cudaError_t launch_virial(const Launch& L, const DevParams& P, const DevState& S,
                          double* d_atom, double* d_tot) {
  const int side = L.sms > 0 ? L.sms : 152;
  cudaError_t e = cudaMemsetAsync(d_tot, 0, 6 * sizeof(double), L.stream);
  if (e == cudaSuccess && d_atom)
    e = cudaMemsetAsync(d_atom, 0, 6 * sizeof(double) * (size_t)P.N, L.stream);
  if (e != cudaSuccess) return e;
  const int nb = std::max(1, std::min(8 * side, (P.N + kVirWarps - 1) / kVirWarps));
  k_virial<<<nb, 32 * kVirWarps, 0, L.stream>>>(P, S, d_atom, d_tot);
  k_virial_mol<<<side, 128, 0, L.stream>>>(P, S, d_atom, d_tot);
  return cudaGetLastError();
}

// Centres with more than kMaxLegs active legs (compressed cascade regions,
// damaged slabs): a group of lanes per centre, 8 or 32 in binary32 and the
// whole warp in binary64 (k_force_heavy chooses). The group first computes every listed leg and stages the active
// ones in shared memory, then takes legs as rows: a lane sums its leg's
// reaction over every other leg in registers and scatters it once. Each
// angle term is evaluated in both of its rows, which costs less than
// splitting the pairs over the lanes (shared-memory atomics on the leg sums,
// on which lanes sharing a leg serialise). A centre has ~10-30 legs, so 8
// lanes keep busy where a warp would leave most of its lanes idle; the
// centre's force is reduced over the group.
constexpr int kHeavyWarps = 4;
constexpr int kHeavyLegs = 64;  // >= max_sw (checked at context creation)

// One pass over the many-leg centres with GROUP lanes per centre (stages in
// sl/sj/snl: kHeavyWarps * 32 / GROUP of them).
template <bool MIXED, bool ENERGY, int GROUP, bool UNI, typename R>
__device__ __forceinline__ void heavy_centres(const DevParams& P, const DevState& S, int cnt,
                                              R (*sl)[6][kHeavyLegs], int (*sj)[kHeavyLegs],
                                              int* snl) {
  constexpr int GPW = 32 / GROUP;  // centres per warp
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gl = lane % GROUP;            // lane within the group
  const int sg = w * GPW + lane / GROUP;  // the group's stage
  const double conv = MIXED ? P.f_evA_to_N : 1.0;
  const double econv = MIXED ? P.e_eV_to_J : 1.0;
  // warp-uniform loop: every lane takes part in the group reductions
  for (int base = (blockIdx.x * kHeavyWarps + w) * GPW; base < cnt;
       base += gridDim.x * kHeavyWarps * GPW) {
    const int h = base + lane / GROUP;
    const int c = h < cnt ? S.heavy_list[h] : -1;
    if (gl == 0) snl[sg] = 0;
    __syncwarp();
    int tc = 1;
    if (c >= 0) {
      tc = S.atype[c];
      const int n = S.n_sw[c];
      const Geo& G = S.geo[rep_of_flags(S.flags[c])];
      const int4 qc = S.posq[c];
      // three neighbours per lane in flight
      constexpr int kG = 3;
      for (int k0 = gl; k0 < n; k0 += kG * GROUP) {
        int jj[kG];
        int4 qq[kG];
#pragma unroll
        for (int u = 0; u < kG; u++) {
          const int k = k0 + u * GROUP;
          jj[u] = k < n ? S.nbr_sw[(size_t)k * P.N + c] : c;
        }
#pragma unroll
        for (int u = 0; u < kG; u++) qq[u] = S.posq[jj[u]];
#pragma unroll
        for (int u = 0; u < kG; u++) {
          if (k0 + u * GROUP >= n) break;
          const int j = jj[u];
          const int tj = qq[u].w & 0xff;
          if ((qq[u].w >> 8) & FL_REMOVED) continue;
          if constexpr (MIXED) {
            const float3 dq = qsep(qc, qq[u], G.qinvA);
            const float r2 = dq.x * dq.x + dq.y * dq.y + dq.z * dq.z;
            const float rinv = rsqrtf(r2);
            const float is = UNI ? P.isigA[0][0] : P.isigA[tc - 1][tj - 1];
            const float ue = r2 * rinv * is;
            if (!(ue < (float)P.cut3)) continue;
            const float ia = __fdividef(1.0f, ue - (float)P.al);
            const float E = __expf((float)P.gam * ia);
            if (!(E > kLegEmin)) continue;
            const int q = atomicAdd(&snl[sg], 1);
            sl[sg][0][q] = dq.x * rinv;
            sl[sg][1][q] = dq.y * rinv;
            sl[sg][2][q] = dq.z * rinv;
            sl[sg][3][q] = rinv;
            sl[sg][4][q] = E;
            sl[sg][5][q] = -(float)P.gam * ia * ia * is;
            sj[sg][q] = j | ((tj - 1) << 30);
          } else {
            const Leg64 L = make_leg(P, G, S.pos[c], S.pos[j], tc, tj);
            if (!(L.u < P.cut3)) continue;
            const int q = atomicAdd(&snl[sg], 1);
            const double ra = 1.0 / L.r, ia = 1.0 / (L.u - P.al);
            sl[sg][0][q] = L.dx * ra;
            sl[sg][1][q] = L.dy * ra;
            sl[sg][2][q] = L.dz * ra;
            sl[sg][3][q] = ra;
            sl[sg][4][q] = exp(P.gam * ia);
            sl[sg][5][q] = -P.gam * ia * ia * L.isig;
            sj[sg][q] = j | (L.t << 30);
          }
        }
      }
    }
    __syncwarp();
    const int nl = snl[sg];
    // rows: lane sums leg a's reaction over every other leg b in registers
    R fcx = 0, fcy = 0, fcz = 0, uc = 0;
    const R thrd = (R)P.thrd;
    for (int a = gl; a < nl; a += GROUP) {
      const R ax = sl[sg][0][a], ay = sl[sg][1][a], az = sl[sg][2][a];
      const R ar = sl[sg][3][a], aE = sl[sg][4][a], ag = sl[sg][5][a];
      const int ja = sj[sg][a];
      // leg a's force as in the one-thread kernel: one scalar and one vector
      // summed per pair, a's direction applied once
      const R m2ar = (R)-2 * ar;
      R sw = 0, sbx = 0, sby = 0, sbz = 0, ae = 0;
      // unrolled for independent shared-memory loads; leg a itself enters
      // with a zero weight (its terms are finite)
#pragma unroll 4
      for (int b = 0; b < nl; b++) {
        const R bx = sl[sg][0][b], by = sl[sg][1][b], bz = sl[sg][2][b];
        const int jb = sj[sg][b];
        const R cs = ax * bx + ay * by + az * bz;
        const R c3 = cs + thrd;
        R lp;
        if constexpr (MIXED)
          lp = UNI ? P.lepsA[0][0][0] : P.lepsA[tc - 1][(unsigned)ja >> 30][(unsigned)jb >> 30];
        else lp = P.leps[tc - 1][(unsigned)ja >> 30][(unsigned)jb >> 30];
        const R pref = b == a ? (R)0 : lp * aE * sl[sg][4][b];
        const R q = pref * c3;
        sw += q * (c3 * ag + m2ar * cs);
        sbx += q * bx;
        sby += q * by;
        sbz += q * bz;
        if (ENERGY) ae += q * c3;
      }
      const R tar = -m2ar;
      const R afx = sw * ax + tar * sbx;
      const R afy = sw * ay + tar * sby;
      const R afz = sw * az + tar * sbz;
      const int j = ja & 0x3fffffff;
      if constexpr (MIXED) {
        // eV/A -> N in binary32 (as in the one-thread kernel): one conversion
        const float cf = (float)conv;
        atomic_add3(S.frc_new, j, (double)(cf * afx), (double)(cf * afy), (double)(cf * afz));
      } else {
        atomic_add3(S.frc_new, j, conv * (double)afx, conv * (double)afy, conv * (double)afz);
      }
      if (ENERGY && ae != (R)0) atomicAdd(&S.epot[j], econv * (double)ae / 3.0);
      fcx -= afx;
      fcy -= afy;
      fcz -= afz;
      if (ENERGY) uc += ae;
    }
    // the centre's third of each term, counted in both rows
    if (ENERGY) uc /= (R)6;
    __syncwarp();
    // the centre's force summed over the group in R (binary32 in mixed
    // mode, as the lanes' shares are), converted once
#pragma unroll
    for (int o = GROUP / 2; o > 0; o >>= 1) {
      fcx += __shfl_xor_sync(0xffffffffu, fcx, o);
      fcy += __shfl_xor_sync(0xffffffffu, fcy, o);
      fcz += __shfl_xor_sync(0xffffffffu, fcz, o);
    }
    double duc = ENERGY ? econv * (double)uc : 0.0;
    if (ENERGY) {
#pragma unroll
      for (int o = GROUP / 2; o > 0; o >>= 1) duc += __shfl_xor_sync(0xffffffffu, duc, o);
    }
    if (gl == 0 && c >= 0) {
      if constexpr (MIXED) {
        const float cf = (float)conv;
        atomic_add3(S.frc_new, c, (double)(cf * fcx), (double)(cf * fcy), (double)(cf * fcz));
      } else {
        atomic_add3(S.frc_new, c, conv * (double)fcx, conv * (double)fcy, conv * (double)fcz);
      }
      if (ENERGY && duc != 0.0) atomicAdd(&S.epot[c], duc);
    }
    __syncwarp();
  }
}

// Binary32: eight lanes per centre (four centres per warp) where the centres
// outnumber the grid's warps (damaged slabs, cascade cores of a batch), the
// whole warp per centre where they fit in one pass (a few cascade-core
// centres: the pass is then as long as one centre's chain, which the wider
// group shortens). Binary64: the whole warp (its leg stage is twice the size).
template <bool MIXED, bool ENERGY, bool UNI = false>
__global__ void __launch_bounds__(32 * kHeavyWarps) k_force_heavy(DevParams P, DevState S) {
  pdl_wait();
  pdl_trigger();
  // binary32 legs in mixed mode (Angstrom, eV), binary64 otherwise
  using R = typename std::conditional<MIXED, float, double>::type;
  constexpr int NG = kHeavyWarps * (MIXED ? 4 : 1);  // stages: centres per block at most
  __shared__ R sl[NG][6][kHeavyLegs];
  __shared__ int sj[NG][kHeavyLegs];
  __shared__ int snl[NG];
  const int cnt = *((volatile int*)&S.sc->heavy_count);
  if (cnt == 0) return;
  if constexpr (MIXED) {
    if (cnt > (int)gridDim.x * kHeavyWarps) {
      heavy_centres<MIXED, ENERGY, 8, UNI>(P, S, cnt, sl, sj, snl);
      return;
    }
  }
  heavy_centres<MIXED, ENERGY, 32, UNI>(P, S, cnt, sl, sj, snl);
}

// Binary32 force with eight lanes per centre for every centre (four centres
// per warp), for systems too small to fill the GPU one thread per centre:
// each lane takes every eighth listed neighbour (2-body force on the centre
// and the leg parameters, active legs staged in shared memory), then legs
// as rows as in the many-leg kernel, and the group reduces the centre's
// force. Twice the warps of a one-thread-per-centre pass per eight atoms and
// a fraction of its dependent chain; chosen by the force-stage autotune
// where it is faster (tens of thousands of atoms).
// UNI: every lattice atom is Si (P.uniform): the [Si][Si] constants directly.
template <bool ENERGY, bool COUNT, bool UNI = false>
__global__ void __launch_bounds__(32 * kHeavyWarps) k_force_group(DevParams P, DevState S) {
  pdl_wait();
  pdl_trigger();
  constexpr int GROUP = 8;
  constexpr int GPW = 32 / GROUP;
  constexpr int NG = kHeavyWarps * GPW;
  const int nbg = (P.N + NG - 1) / NG;
  // the last mol_blocks blocks evaluate the Moliere list
  if ((int)blockIdx.x >= nbg) {
    moliere_entries<true, ENERGY>(P, S, ((int)blockIdx.x - nbg) * (32 * kHeavyWarps) + threadIdx.x,
                                  ((int)gridDim.x - nbg) * (32 * kHeavyWarps));
    return;
  }
  __shared__ float sl[NG][6][kHeavyLegs];
  __shared__ int sj[NG][kHeavyLegs];
  __shared__ int snl[NG];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gl = lane % GROUP;            // lane within the group
  const int sg = w * GPW + lane / GROUP;  // the group's stage
  const int c = blockIdx.x * NG + sg;
  if (gl == 0) snl[sg] = 0;
  __syncwarp();
  int tc = 1, n = 0;
  int4 qc = make_int4(0, 0, 0, 0);
  if (c < P.N) {
    qc = S.posq[c];
    tc = qc.w & 0xff;
    if (tc < 3 && !((qc.w >> 8) & FL_REMOVED)) n = S.n_sw[c];
  }
  const int ta = UNI ? 0 : tc - 1;
  float fx = 0.f, fy = 0.f, fz = 0.f, ui = 0.f;
  unsigned cnt_pairs = 0, cnt_ang = 0;
  if (n > 0) {
    const Geo& G = S.geo[rep_of_w(qc.w)];
    const float al = (float)P.al, cut = (float)P.cut3, gm = (float)P.gam;
    const float Bc = (float)P.B, Ac = (float)P.A;
    // three neighbours per lane in flight (a crystal lists 16)
    constexpr int kG = 3;
    for (int k0 = gl; k0 < n; k0 += kG * GROUP) {
      int jj[kG];
      int4 qq[kG];
#pragma unroll
      for (int u = 0; u < kG; u++) {
        const int k = k0 + u * GROUP;
        jj[u] = k < n ? S.nbr_sw[(size_t)k * P.N + c] : c;
      }
#pragma unroll
      for (int u = 0; u < kG; u++) qq[u] = S.posq[jj[u]];
#pragma unroll
      for (int u = 0; u < kG; u++) {
        if (k0 + u * GROUP >= n) break;
        const int j = jj[u];
        const int4 qj = qq[u];
        const float3 dq = qsep(qc, qj, G.qinvA);
        const float r2f = dq.x * dq.x + dq.y * dq.y + dq.z * dq.z;
        if (r2f > P.pre3mA2 || ((qj.w >> 8) & FL_REMOVED)) continue;
        const int tb = UNI ? 0 : (qj.w & 0xff) - 1;
        const float rinv = rsqrtf(r2f);
        const float is = P.isigA[ta][tb];
        const float ue = r2f * rinv * is;
        if (!(ue < cut)) continue;
        const float inv = __fdividef(1.0f, ue - al);
        const float ex = __expf(inv);
        const float iu = P.sigA[ta][tb] * rinv;  // 1/u
        const float u2 = iu * iu;
        const float u4 = u2 * u2;
        // psi = 4, qsi = 0: dphi/du = A e^{1/(u-a)} [ -4 B u^-5 - (B u^-4 - 1)/(u-a)^2 ]
        const float dphi = Ac * ex * (-4.0f * Bc * u4 * iu - (Bc * u4 - 1.0f) * inv * inv);
        const float cf = -(dphi * rinv * P.epssigA[ta][tb]);
        fx += cf * dq.x;
        fy += cf * dq.y;
        fz += cf * dq.z;
        if (COUNT) cnt_pairs++;
        if (ENERGY) ui += 0.5f * P.epsA[ta][tb] * Ac * (Bc * u4 - 1.0f) * ex;
        const float E = __expf(gm * inv);
        if (!(E > kLegEmin)) continue;
        const int q = atomicAdd(&snl[sg], 1);
        sl[sg][0][q] = dq.x * rinv;
        sl[sg][1][q] = dq.y * rinv;
        sl[sg][2][q] = dq.z * rinv;
        sl[sg][3][q] = rinv;
        sl[sg][4][q] = E;
        sl[sg][5][q] = -gm * inv * inv * is;
        sj[sg][q] = j | (tb << 30);
      }
    }
  }
  __syncwarp();
  const int nl = snl[sg];
  const float thrd = (float)P.thrd;
  const float conv = (float)P.f_evA_to_N;
  float uc = 0.f;
  for (int a = gl; a < nl; a += GROUP) {
    const float ax = sl[sg][0][a], ay = sl[sg][1][a], az = sl[sg][2][a];
    const float ar = sl[sg][3][a], aE = sl[sg][4][a], ag = sl[sg][5][a];
    const int ja = sj[sg][a];
    // leg a's force as in the one-thread kernel: one scalar and one vector
    // summed per pair, a's direction applied once
    const float m2ar = -2.0f * ar;
    float sw = 0.f, sbx = 0.f, sby = 0.f, sbz = 0.f, ae = 0.f;
    // unrolled for independent shared-memory loads; leg a itself enters
    // with a zero weight (its terms are finite)
#pragma unroll 4
    for (int b = 0; b < nl; b++) {
      const float bx = sl[sg][0][b], by = sl[sg][1][b], bz = sl[sg][2][b];
      const float cs = ax * bx + ay * by + az * bz;
      const float c3 = cs + thrd;
      const float lp = UNI ? P.lepsA[0][0][0]
                           : P.lepsA[ta][(unsigned)ja >> 30][(unsigned)sj[sg][b] >> 30];
      const float pref = b == a ? 0.f : lp * aE * sl[sg][4][b];
      const float q = pref * c3;
      sw += q * (c3 * ag + m2ar * cs);
      sbx += q * bx;
      sby += q * by;
      sbz += q * bz;
      if (ENERGY) ae += q * c3;
      if (COUNT && b > a && pref != 0.f) cnt_ang++;
    }
    const float tar = -m2ar;
    const float afx = sw * ax + tar * sbx;
    const float afy = sw * ay + tar * sby;
    const float afz = sw * az + tar * sbz;
    const int j = ja & 0x3fffffff;
    atomic_add3(S.frc_new, j, (double)(conv * afx), (double)(conv * afy), (double)(conv * afz));
    if (ENERGY && ae != 0.f) atomicAdd(&S.epot[j], P.e_eV_to_J * (double)ae / 3.0);
    fx -= afx;
    fy -= afy;
    fz -= afz;
    if (ENERGY) uc += ae;
  }
  // the centre's force over the group: the lanes' binary32 shares summed in
  // binary32 (as the one-thread kernel sums a centre's terms), then one
  // binary64 atomic per component; binary64 lane sums would put ~100 FP64
  // instructions per centre on the SM's thin FP64 pipe
#pragma unroll
  for (int o = GROUP / 2; o > 0; o >>= 1) {
    fx += __shfl_xor_sync(0xffffffffu, fx, o);
    fy += __shfl_xor_sync(0xffffffffu, fy, o);
    fz += __shfl_xor_sync(0xffffffffu, fz, o);
  }
  // the centre's half of each pair, and a third of each angle term (counted
  // in both of its rows)
  double duc = ENERGY ? P.e_eV_to_J * ((double)ui + (double)uc / 6.0) : 0.0;
  if (ENERGY) {
#pragma unroll
    for (int o = GROUP / 2; o > 0; o >>= 1) duc += __shfl_xor_sync(0xffffffffu, duc, o);
  }
  if (gl == 0 && n > 0) {
    atomic_add3(S.frc_new, c, (double)(conv * fx), (double)(conv * fy), (double)(conv * fz));
    if (ENERGY && duc != 0.0) atomicAdd(&S.epot[c], duc);
  }
  if (COUNT) {
    const unsigned sp = __reduce_add_sync(0xffffffffu, cnt_pairs);
    const unsigned sa = __reduce_add_sync(0xffffffffu, cnt_ang);
    if (lane == 0) {
      if (sp) atomicAdd(&S.sc->counters[0], (unsigned long long)sp);
      if (sa) atomicAdd(&S.sc->counters[1], (unsigned long long)sa);
    }
  }
}

__device__ __forceinline__ bool in_list(const DevParams& P, const DevState& S, int c, int x) {
  const int n = S.n_sw[c];
  for (int q = 0; q < n; q++)
    if (S.nbr_sw[(size_t)q * P.N + c] == x) return true;
  return false;
}

// Stale-list correction: for each fast atom f, every path f - a - x of the
// build-time list graph whose closing edge f-x is not listed contributes the
// two angle terms the reference evaluates through the triple {f,a,x} but a
// per-centre sweep does not: centre f (legs a, x) and centre x (legs a, f).
template <bool ENERGY>
__global__ void k_force_stale(DevParams P, DevState S) {
  pdl_wait();
  pdl_trigger();
  const int cnt = *((volatile int*)&S.sc->fast_count);
  for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < cnt; h += gridDim.x * blockDim.x) {
    const int f = S.fast_list[h];
    const int tf = S.atype[f];
    if (tf >= 3) continue;
    const double4_32a pf = S.pos[f];
    const int4 qf = S.posq[f];
    const int nf = S.n_sw[f];
    const Geo& G = S.geo[rep_of_w(qf.w)];
    unsigned int terms = 0;
    for (int ia = 0; ia < nf; ia++) {
      const int a = S.nbr_sw[(size_t)ia * P.N + f];
      const int na = S.n_sw[a];
      for (int ix = 0; ix < na; ix++) {
        const int x = S.nbr_sw[(size_t)ix * P.N + a];
        if (x == f) continue;
        const int4 qx = S.posq[x];
        const float3 dq = qsep(qf, qx, G.qinvA);
        if (dq.x * dq.x + dq.y * dq.y + dq.z * dq.z > P.pre3A2) continue;
        if (S.fast_flag[x] && x < f) continue;  // the pair is handled from x
        if (in_list(P, S, f, x)) continue;
        const int ta = S.atype[a], tx = S.atype[x];
        const double4_32a pa = S.pos[a], px = S.pos[x];
        double f0[3], f1[3], f2[3], e;
        // centre f, legs a and x
        {
          const Leg64 A = make_leg(P, G, pf, pa, tf, ta);
          const Leg64 X = make_leg(P, G, pf, px, tf, tx);
          if (angle_term(P, tf, A, X, f0, f1, f2, &e)) {
            atomic_add3(S.frc_new, f, f0[0], f0[1], f0[2]);
            atomic_add3(S.frc_new, a, f1[0], f1[1], f1[2]);
            atomic_add3(S.frc_new, x, f2[0], f2[1], f2[2]);
            if (ENERGY) {
              atomicAdd(&S.epot[f], e / 3.0);
              atomicAdd(&S.epot[a], e / 3.0);
              atomicAdd(&S.epot[x], e / 3.0);
            }
            terms++;
          }
        }
        // centre x, legs a and f
        {
          const Leg64 A = make_leg(P, G, px, pa, tx, ta);
          const Leg64 Fl = make_leg(P, G, px, pf, tx, tf);
          if (angle_term(P, tx, A, Fl, f0, f1, f2, &e)) {
            atomic_add3(S.frc_new, x, f0[0], f0[1], f0[2]);
            atomic_add3(S.frc_new, a, f1[0], f1[1], f1[2]);
            atomic_add3(S.frc_new, f, f2[0], f2[1], f2[2]);
            if (ENERGY) {
              atomicAdd(&S.epot[x], e / 3.0);
              atomicAdd(&S.epot[a], e / 3.0);
              atomicAdd(&S.epot[f], e / 3.0);
            }
            terms++;
          }
        }
      }
    }
    if (terms) atomicAdd(&S.sc->counters[3], (unsigned long long)terms);
  }
}

// Moliere (si.f90:426-446): one thread per full-list entry (i, j) adds the
// force on i; the (j, i) entry adds the mirror. Unfired ions are skipped.
// Entries first, first + stride, ...
template <bool MIXED, bool ENERGY>
__device__ __forceinline__ void moliere_entries(const DevParams& P, const DevState& S, int first,
                                                int stride) {
  int cnt = *((volatile int*)&S.sc->mol_count);
  if (cnt > P.mol_cap) cnt = P.mol_cap;
  unsigned int npair = 0;
  for (int e = first; e < cnt; e += stride) {
    const int2 pr = S.mol_pairs[e];
    const int i = pr.x, j = pr.y;
    // si_force skips unfired ions (si.f90:428); si_potential does not
    const bool fired = i < P.nfired && j < P.nfired;
    if (!ENERGY && !fired) continue;
    if ((S.flags[i] | S.flags[j]) & FL_REMOVED) continue;
    const int ti = S.atype[i] - 1, tj = S.atype[j] - 1;
    const double4_32a pi = S.pos[i], pj = S.pos[j];
    const Geo& G = S.geo[rep_of_flags(S.flags[i])];
    const double dx = min_image(pi.x, pj.x, G.iLb[0], G.Lb[0]);
    const double dy = min_image(pi.y, pj.y, G.iLb[1], G.Lb[1]);
    const double dz = min_image(pi.z, pj.z, G.iLb[2], G.Lb[2]);
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (!(r2 < P.rlj2)) continue;
    if (fired) npair++;
    double fcr, ul = 0.0;  // fc / r
    const double rA = sqrt(r2) * 1.0e10;
    if (MIXED && rA >= (double)P.mol_fp64_rA) {
      const float r = (float)rA, aa = P.amolA[ti][tj];
      const float e1 = expf(-(float)P.amol * r / aa), e2 = expf(-(float)P.bmol * r / aa),
                  e3 = expf(-(float)P.gmol * r / aa);
      const float sum0 = (float)P.Amol * e1 + (float)P.Bmol * e2 + (float)P.Cmol * e3;
      const float sum1 = (float)P.Amol * (float)P.amol / aa * e1 +
                         (float)P.Bmol * (float)P.bmol / aa * e2 +
                         (float)P.Cmol * (float)P.gmol / aa * e3;
      const float fc = P.molKA[ti][tj] / r * (sum0 / r + sum1);  // eV/A
      fcr = P.f_evA_to_N * (double)(fc / r) * 1.0e10;             // N per m of separation
      if (ENERGY) ul = P.e_eV_to_J * (double)(P.molKA[ti][tj] / r * sum0);
    } else {
      const double rij = sqrt(r2);
      const double aa = P.aamol[ti][tj];
      const double e1 = exp(-(P.amol * rij / aa)), e2 = exp(-(P.bmol * rij / aa)),
                   e3 = exp(-(P.gmol * rij / aa));
      const double K = P.ie0 * P.Zmol[ti] * P.Zmol[tj] * P.ec * P.ec;
      const double fc = K / rij *
                        ((P.Amol * e1 + P.Bmol * e2 + P.Cmol * e3) / rij +
                         (P.Amol * P.amol / aa * e1 + P.Bmol * P.bmol / aa * e2 +
                          P.Cmol * P.gmol / aa * e3));
      fcr = fc / rij;
      if (ENERGY) ul = K / rij * (P.Amol * e1 + P.Bmol * e2 + P.Cmol * e3);
    }
    if (fired) atomic_add3(S.frc_new, i, fcr * dx, fcr * dy, fcr * dz);
    if (ENERGY) atomicAdd(&S.epot[i], ul / 2.0);
  }
  if (npair) atomicAdd(&S.sc->counters[2], (unsigned long long)npair);
}

template <bool MIXED, bool ENERGY>
__global__ void k_force_moliere(DevParams P, DevState S) {
  pdl_wait();
  pdl_trigger();
  moliere_entries<MIXED, ENERGY>(P, S, blockIdx.x * blockDim.x + threadIdx.x,
                                 gridDim.x * blockDim.x);
}

// The second pass of the stored-reaction form: atom m adds its own centre
// force and, for each SW partner j of which it is a leg, the reaction that
// j's centre stored for it, each converted to N and summed in binary64 into
// the force buffer (which holds the Moliere and many-leg atomics). A centre
// of the many-leg kernel looks through its whole list, since its legs are
// not recorded; a partner of the many-leg kernel added its reactions itself.
// Being a leg is symmetric (the same binary32 distance both ways), so every
// stored reaction is gathered exactly once.
__global__ void __launch_bounds__(256) k_force_gather(DevParams P, DevState S) {
  pdl_wait();
  pdl_trigger();
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= P.N) return;
  const unsigned long long lp = S.legpos[m];
  const int cnt = (int)(lp >> 60);
  const float4 fo = S.fown[m];
  if (cnt == 0 && fo.x == 0.f && fo.y == 0.f && fo.z == 0.f) return;
  const float convf = (float)P.f_evA_to_N;
  const size_t N = (size_t)P.N;
  double fx = (double)(convf * fo.x), fy = (double)(convf * fo.y), fz = (double)(convf * fo.z);
  auto gather = [&](int k) {
    const int j = S.nbr_sw[(size_t)k * N + m];
    const int r = S.rev_sw[(size_t)k * N + m];
    if (r < 0) return;
    const unsigned long long lj = S.legpos[j];
    const int cj = (int)(lj >> 60);
    if (cj > kStageLarge) return;
    for (int b = 0; b < cj; b++) {
      if ((int)((lj >> (6 * b)) & 63ull) == r) {
        const float4 R = S.react[(size_t)b * N + j];
        fx += (double)(convf * R.x);
        fy += (double)(convf * R.y);
        fz += (double)(convf * R.z);
        return;
      }
    }
  };
  if (cnt == (int)kLegsHeavy) {
    const int n = min(S.n_sw[m], P.max_sw);
    for (int k = 0; k < n; k++) gather(k);
  } else {
    for (int a = 0; a < cnt; a++) gather((int)((lp >> (6 * a)) & 63ull));
  }
  double4_32a& F = S.frc_new[m];
  F.x += fx;
  F.y += fy;
  F.z += fz;
}

__global__ void k_force_begin(DevState S) {
  if (threadIdx.x == 0) {
    S.sc->heavy_count = 0;
    S.sc->table_err = 0;
  }
  if (threadIdx.x < 4) S.sc->counters[threadIdx.x] = 0ull;
}

// A group of lanes per many-leg centre; the count is known only on the
// device, so the grid covers thousands of centres (cascade cores of a batch)
// in one round and idle warps return at once.
template <bool MIXED, bool ENERGY>
static cudaError_t heavy_impl(const Launch& L, const DevParams& P, const DevState& S, bool pdl) {
  const int side = L.sms > 0 ? L.sms : 152;
  const int heavy_blocks =
      std::max(side, std::min(8 * side, (P.N / 64 + kHeavyWarps - 1) / kHeavyWarps));
  if (MIXED && !ENERGY && P.uniform)
    return launch_k(k_force_heavy<MIXED, ENERGY, true>, heavy_blocks, 32 * kHeavyWarps, 0,
                    L.stream, pdl, P, S);
  return launch_k(k_force_heavy<MIXED, ENERGY>, heavy_blocks, 32 * kHeavyWarps, 0, L.stream, pdl,
                  P, S);
}

template <bool MIXED, bool ENERGY, bool COUNT, int LEGS, int BLK = kBlock32>
static cudaError_t force_impl(const Launch& L, const DevParams& P, const DevState& S) {
  constexpr int BLOCK = MIXED ? BLK : kBlock64;
  const size_t smem = MIXED ? (sizeof(float) * LEGS * kLegF32 + sizeof(int) * LEGS) * BLOCK
                            : (sizeof(double) * kMaxLegs * kLegF64 +
                               sizeof(int) * (kMaxLegs + kCandF64)) * BLOCK;
  void (*kern)(DevParams, DevState, cudaGraphConditionalHandle, int) = nullptr;
  const int uni = (MIXED && !ENERGY && P.uniform) ? 1 : 0;
  // stored reactions: only where the context allocated their buffers
  const int react = (MIXED && !ENERGY && L.react && S.react) ? 1 : 0;
  if constexpr (MIXED) {
    if constexpr (!ENERGY) {
      if (react) kern = uni ? k_force_mixed<ENERGY, COUNT, LEGS, BLK, true, true>
                            : k_force_mixed<ENERGY, COUNT, LEGS, BLK, false, true>;
      else kern = uni ? k_force_mixed<ENERGY, COUNT, LEGS, BLK, true>
                      : k_force_mixed<ENERGY, COUNT, LEGS, BLK, false>;
    } else {
      kern = k_force_mixed<ENERGY, COUNT, LEGS, BLK, false>;
    }
  } else {
    kern = k_force_fp64<ENERGY, COUNT>;
  }
  // the dynamic shared-memory limit is a per-device attribute of the kernel:
  // set it once on each device that launches it
  static std::atomic<unsigned long long> attr_devices[4] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  const unsigned long long bit = 1ull << (dev & 63);
  const int variant = uni + 2 * react;
  if (!(attr_devices[variant].load() & bit)) {
    const cudaError_t ea =
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (ea != cudaSuccess) return ea;
    attr_devices[variant].fetch_or(bit);
  }
  if (L.force_a) cudaEventRecord(L.force_a, L.stream);
  kern<<<(P.N + BLOCK - 1) / BLOCK + (MIXED ? mol_blocks(P) : 0), BLOCK, smem, L.stream>>>(
      P, S, L.heavy_handle, L.heavy_if ? 1 : 0);
  if (L.force_b) cudaEventRecord(L.force_b, L.stream);
  const int side = L.sms > 0 ? L.sms : 152;
  // the kernels after the main one are programmatic dependents (L.pdl)
  const bool pdl = L.pdl && !L.force_b;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && !MIXED)
    e = launch_k(k_force_moliere<MIXED, ENERGY>, side, 128, 0, L.stream, pdl, P, S);
  // the many-leg centres (the step graph adds this launch in an IF node)
  if (e == cudaSuccess && !L.heavy_if) e = heavy_impl<MIXED, ENERGY>(L, P, S, pdl);
  if (e == cudaSuccess && react)
    e = launch_k(k_force_gather, (P.N + 255) / 256, 256, 0, L.stream, pdl, P, S);
  if (e == cudaSuccess && P.mode == FIBMD_MODE_REF)
    e = launch_k(k_force_stale<ENERGY>, side, 64, 0, L.stream, pdl, P, S);
  return e;
}

// The eight-lanes-per-centre path: one kernel for the SW terms of every
// centre and the Moliere list.
template <bool ENERGY, bool COUNT>
static cudaError_t group_impl(const Launch& L, const DevParams& P, const DevState& S) {
  constexpr int NG = kHeavyWarps * 4;  // centres per block
  if (L.force_a) cudaEventRecord(L.force_a, L.stream);
  const int nb = (P.N + NG - 1) / NG + mol_blocks(P);
  if (!ENERGY && P.uniform)
    k_force_group<ENERGY, COUNT, true><<<nb, 32 * kHeavyWarps, 0, L.stream>>>(P, S);
  else
    k_force_group<ENERGY, COUNT><<<nb, 32 * kHeavyWarps, 0, L.stream>>>(P, S);
  if (L.force_b) cudaEventRecord(L.force_b, L.stream);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && P.mode == FIBMD_MODE_REF) {
    const int side = L.sms > 0 ? L.sms : 152;
    e = launch_k(k_force_stale<ENERGY>, side, 64, 0, L.stream, L.pdl && !L.force_b, P, S);
  }
  return e;
}

cudaError_t launch_force_heavy(const Launch& L, const DevParams& P, const DevState& S) {
  if (P.precision == FIBMD_PREC_MIXED) return heavy_impl<true, false>(L, P, S, L.pdl);
  return heavy_impl<false, false>(L, P, S, L.pdl);
}

cudaError_t launch_force(const Launch& L, const DevParams& P, const DevState& S, bool energy,
                         bool count, bool spec_step) {
  cudaError_t e = cudaSuccess;
  if (!spec_step) {
    e = cudaMemsetAsync(S.frc_new, 0, sizeof(double4_32a) * (size_t)P.N, L.stream);
    if (e != cudaSuccess) return e;
  }
  if (energy) {
    e = cudaMemsetAsync(S.epot, 0, sizeof(double) * (size_t)P.N, L.stream);
    if (e != cudaSuccess) return e;
  }
  if (!spec_step) k_force_begin<<<1, 32, 0, L.stream>>>(S);
  const bool mixed = P.precision == FIBMD_PREC_MIXED;
  if (mixed) {
    if (L.stage == kStageGroup) {
      if (energy) return count ? group_impl<true, true>(L, P, S) : group_impl<true, false>(L, P, S);
      return count ? group_impl<false, true>(L, P, S) : group_impl<false, false>(L, P, S);
    }
    if (L.stage == kStageLarge) {
      if (energy)
        return count ? force_impl<true, true, true, kStageLarge>(L, P, S)
                     : force_impl<true, true, false, kStageLarge>(L, P, S);
      if (L.force_block == 64)
        return count ? force_impl<true, false, true, kStageLarge, 64>(L, P, S)
                     : force_impl<true, false, false, kStageLarge, 64>(L, P, S);
      return count ? force_impl<true, false, true, kStageLarge>(L, P, S)
                   : force_impl<true, false, false, kStageLarge>(L, P, S);
    }
    if (energy)
      return count ? force_impl<true, true, true, kStageSmall>(L, P, S)
                   : force_impl<true, true, false, kStageSmall>(L, P, S);
    if (L.force_block == 64)
      return count ? force_impl<true, false, true, kStageSmall, 64>(L, P, S)
                   : force_impl<true, false, false, kStageSmall, 64>(L, P, S);
    return count ? force_impl<true, false, true, kStageSmall>(L, P, S)
                 : force_impl<true, false, false, kStageSmall>(L, P, S);
  }
  if (energy)
    return count ? force_impl<false, true, true, 0>(L, P, S) : force_impl<false, true, false, 0>(L, P, S);
  return count ? force_impl<false, false, true, 0>(L, P, S) : force_impl<false, false, false, 0>(L, P, S);
}

}  // namespace fibmd
