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
#include <type_traits>

#include "fibmd_internal.cuh"

namespace fibmd {

constexpr int kLegF = 9;  // ux uy uz rinv E g fx fy fz

// Threads per block of the main force kernel: binary64 stages 12 legs x 9
// doubles per thread (55 KB per 64 threads, 3 blocks per SM); binary32
// stages floats (55 KB per 128 threads).
template <bool MIXED>
struct ForceBlock {
  static constexpr int value = MIXED ? 128 : 64;
};

template <typename R, int BLOCK>
struct LegSmem {
  R* v;
  int* j;
  __device__ __forceinline__ R& at(int l, int f) {
    return v[(l * kLegF + f) * BLOCK + threadIdx.x];
  }
  __device__ __forceinline__ int& idx(int l) { return j[l * BLOCK + threadIdx.x]; }
};

// 3-point Lagrange interpolation of the derivative table (itable2bd).
// it = INT(ue/umax*(Ntable-1)) is the 0-based first stencil point.
__device__ __forceinline__ double table_df(const DevParams& P, const double* __restrict__ tab,
                                           const double* __restrict__ tabu, double ue,
                                           int* err) {
  int it = (int)(ue / P.umax * (double)(P.Ntable - 1));
  if (it > P.tab_last) return 0.0;  // all three stencil entries are zero
  if (it + 1 > P.Ntable) {
    *err = 1;
    return 0.0;
  }
  double d1 = ue - __ldg(&tabu[it]);
  double d2 = ue - __ldg(&tabu[it + 1]);
  double d3 = ue - __ldg(&tabu[it + 2]);
  return 0.5 * d2 * d3 * __ldg(&tab[it]) - d1 * d3 * __ldg(&tab[it + 1]) +
         0.5 * d1 * d2 * __ldg(&tab[it + 2]);
}

// ---- main per-centre kernel ------------------------------------------------
template <bool MIXED, bool ENERGY, bool COUNT>
__global__ void __launch_bounds__(ForceBlock<MIXED>::value) k_force(DevParams P, DevState S) {
  using R = typename std::conditional<MIXED, float, double>::type;
  constexpr int BLOCK = ForceBlock<MIXED>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  LegSmem<R, BLOCK> leg;
  leg.v = reinterpret_cast<R*>(smem_raw);
  leg.j = reinterpret_cast<int*>(smem_raw + sizeof(R) * kMaxLegs * kLegF * BLOCK);

  const int i = blockIdx.x * BLOCK + threadIdx.x;
  if (i >= P.N) return;
  const int4 qi = S.posq[i];
  const int ti = qi.w & 0xff;
  if (ti >= 3 || ((qi.w >> 8) & FL_REMOVED)) return;
  const int n = S.n_sw[i];
  if (n == 0) return;
  const double4_32a pi = S.pos[i];
  const int ta = ti - 1;

  double fx = 0.0, fy = 0.0, fz = 0.0, ui = 0.0;
  float mfx = 0.f, mfy = 0.f, mfz = 0.f, mui = 0.f;
  int nl = 0;
  int terr = 0;
  unsigned int cnt_pairs = 0, cnt_ang = 0;

  for (int k = 0; k < n; k++) {
    const int j = S.nbr_sw[(size_t)k * P.N + i];
    const int4 qj = S.posq[j];
    const float3 dq = qsep(qi, qj, P.qinvA);
    const float r2f = dq.x * dq.x + dq.y * dq.y + dq.z * dq.z;
    if (r2f > P.pre3A2) continue;  // beyond the table support and 3-body cutoff
    const int tb = (qj.w & 0xff) - 1;
    if constexpr (!MIXED) {
      const double4_32a pj = S.pos[j];
      const double dx = min_image(pi.x, pj.x, P.iLb[0], P.Lb[0]);
      const double dy = min_image(pi.y, pj.y, P.iLb[1], P.Lb[1]);
      const double dz = min_image(pi.z, pj.z, P.iLb[2], P.Lb[2]);
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
    } else {
      // binary32 in reduced units (Angstrom, eV); psi = 4, qsi = 0
      const float rinv = rsqrtf(r2f);
      const float r = r2f * rinv;
      const float sg = P.sigA[ta][tb];
      const float ue = r / sg;
      const float cut = (float)P.cut3;
      if (ue < cut) {
        const float al = (float)P.al;
        const float inv = 1.0f / (ue - al);
        const float ex = expf(inv);
        const float u2 = 1.0f / (ue * ue);
        const float u4 = u2 * u2;
        const float B = (float)P.B, A = (float)P.A;
        // dphi/du = A e^{1/(u-a)} [ -4 B u^-5 - (B u^-4 - 1)/(u-a)^2 ]
        const float dphi = A * ex * (-4.0f * B * u4 / ue - (B * u4 - 1.0f) * inv * inv);
        const float c = -(dphi * rinv * (P.epsA[ta][tb] / sg));
        mfx += c * dq.x;
        mfy += c * dq.y;
        mfz += c * dq.z;
        if (COUNT) cnt_pairs++;
        if (ENERGY) mui += 0.5f * P.epsA[ta][tb] * A * (B * u4 - 1.0f) * ex;
        if (nl < kMaxLegs) {
          const float gm = (float)P.gam;
          leg.at(nl, 0) = dq.x * rinv;
          leg.at(nl, 1) = dq.y * rinv;
          leg.at(nl, 2) = dq.z * rinv;
          leg.at(nl, 3) = rinv;
          leg.at(nl, 4) = expf(gm * inv);
          leg.at(nl, 5) = -gm * inv * inv / sg;
          leg.at(nl, 6) = 0.f;
          leg.at(nl, 7) = 0.f;
          leg.at(nl, 8) = 0.f;
          leg.idx(nl) = j | (tb << 30);
        }
        nl++;
      }
    }
  }

  if (nl > kMaxLegs) {
    // the direct kernel evaluates this centre's angle terms
    int slot = atomicAdd(&S.sc->heavy_count, 1);
    S.heavy_list[slot] = i;
  } else {
    const R thrd = (R)P.thrd;
    R cfx = 0, cfy = 0, cfz = 0, cu = 0;
    for (int a = 0; a < nl; a++) {
      const R ax = leg.at(a, 0), ay = leg.at(a, 1), az = leg.at(a, 2);
      const R ar = leg.at(a, 3), aE = leg.at(a, 4), ag = leg.at(a, 5);
      const int tbA = (unsigned)leg.idx(a) >> 30;
      R afx = 0, afy = 0, afz = 0;
      for (int b = a + 1; b < nl; b++) {
        const R bx = leg.at(b, 0), by = leg.at(b, 1), bz = leg.at(b, 2);
        const R br = leg.at(b, 3), bE = leg.at(b, 4), bg = leg.at(b, 5);
        const int tbB = (unsigned)leg.idx(b) >> 30;
        R lp;
        if constexpr (MIXED) lp = P.lepsA[ta][tbA][tbB];
        else lp = P.leps[ta][tbA][tbB];
        const R cs = ax * bx + ay * by + az * bz;
        const R c3 = cs + thrd;
        const R W = c3 * c3;
        const R pref = lp * aE * bE;
        const R s2 = (R)2 * c3;
        // F_a = pref [W g_a p_a + 2(c+1/3)(p_b - c p_a)/r_a], p = unit(X_c - X_a)
        const R wa = W * ag - s2 * cs * ar, sa = s2 * ar;
        const R Fax = pref * (wa * ax + sa * bx);
        const R Fay = pref * (wa * ay + sa * by);
        const R Faz = pref * (wa * az + sa * bz);
        const R wb = W * bg - s2 * cs * br, sb = s2 * br;
        const R Fbx = pref * (wb * bx + sb * ax);
        const R Fby = pref * (wb * by + sb * ay);
        const R Fbz = pref * (wb * bz + sb * az);
        afx += Fax;
        afy += Fay;
        afz += Faz;
        leg.at(b, 6) += Fbx;
        leg.at(b, 7) += Fby;
        leg.at(b, 8) += Fbz;
        cfx -= Fax + Fbx;
        cfy -= Fay + Fby;
        cfz -= Faz + Fbz;
        if (ENERGY) cu += pref * W;
        if (COUNT && pref != (R)0) cnt_ang++;
      }
      leg.at(a, 6) += afx;
      leg.at(a, 7) += afy;
      leg.at(a, 8) += afz;
    }
    // scatter leg reactions (binary64 accumulation)
    const double conv = MIXED ? P.f_evA_to_N : 1.0;
    for (int a = 0; a < nl; a++) {
      const int j = leg.idx(a) & 0x3fffffff;
      atomic_add3(S.frc_new, j, conv * (double)leg.at(a, 6), conv * (double)leg.at(a, 7),
                  conv * (double)leg.at(a, 8));
    }
    if constexpr (MIXED) {
      mfx += cfx;
      mfy += cfy;
      mfz += cfz;
    } else {
      fx += cfx;
      fy += cfy;
      fz += cfz;
    }
    if (ENERGY && nl > 1) {
      // each angle term gives a third of its energy to each of its atoms
      const double e3 = (MIXED ? P.e_eV_to_J : 1.0) * (double)cu / 3.0;
      if (e3 != 0.0) {
        ui += e3;
        for (int a = 0; a < nl; a++) {
          // a leg's share: sum over the terms it belongs to
          double sh = 0.0;
          for (int b = 0; b < nl; b++) {
            if (b == a) continue;
            const R cs = leg.at(a, 0) * leg.at(b, 0) + leg.at(a, 1) * leg.at(b, 1) +
                         leg.at(a, 2) * leg.at(b, 2);
            const R c3 = cs + thrd;
            const int tbA = (unsigned)leg.idx(a) >> 30, tbB = (unsigned)leg.idx(b) >> 30;
            R lp;
            if constexpr (MIXED) lp = P.lepsA[ta][tbA][tbB];
            else lp = P.leps[ta][tbA][tbB];
            sh += (double)(lp * leg.at(a, 4) * leg.at(b, 4) * c3 * c3);
          }
          atomicAdd(&S.epot[leg.idx(a) & 0x3fffffff],
                    (MIXED ? P.e_eV_to_J : 1.0) * sh / 3.0);
        }
      }
    }
  }
  if constexpr (MIXED) {
    fx += P.f_evA_to_N * (double)mfx;
    fy += P.f_evA_to_N * (double)mfy;
    fz += P.f_evA_to_N * (double)mfz;
    if (ENERGY) ui += P.e_eV_to_J * (double)mui;
  }
  atomic_add3(S.frc_new, i, fx, fy, fz);
  if (ENERGY && ui != 0.0) atomicAdd(&S.epot[i], ui);
  if (terr) atomicAdd(&S.sc->table_err, 1);
  if (COUNT) {
    if (cnt_pairs) atomicAdd(&S.sc->counters[0], (unsigned long long)cnt_pairs);
    if (cnt_ang) atomicAdd(&S.sc->counters[1], (unsigned long long)cnt_ang);
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

__device__ __forceinline__ Leg64 make_leg(const DevParams& P, const double4_32a& pc,
                                          const double4_32a& pl, int tc, int tl) {
  Leg64 L;
  L.dx = min_image(pc.x, pl.x, P.iLb[0], P.Lb[0]);
  L.dy = min_image(pc.y, pl.y, P.iLb[1], P.Lb[1]);
  L.dz = min_image(pc.z, pl.z, P.iLb[2], P.Lb[2]);
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

// Centres with more than kMaxLegs active legs: every leg pair, direct.
template <bool ENERGY>
__global__ void k_force_heavy(DevParams P, DevState S) {
  const int cnt = *((volatile int*)&S.sc->heavy_count);
  for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < cnt; h += gridDim.x * blockDim.x) {
    const int c = S.heavy_list[h];
    const int tc = S.atype[c];
    const double4_32a pc = S.pos[c];
    const int n = S.n_sw[c];
    double fcx = 0, fcy = 0, fcz = 0, uc = 0;
    for (int a = 0; a < n; a++) {
      const int ja = S.nbr_sw[(size_t)a * P.N + c];
      const Leg64 A = make_leg(P, pc, S.pos[ja], tc, S.atype[ja]);
      if (!(A.u < P.cut3)) continue;
      for (int b = a + 1; b < n; b++) {
        const int jb = S.nbr_sw[(size_t)b * P.N + c];
        const Leg64 B = make_leg(P, pc, S.pos[jb], tc, S.atype[jb]);
        double f0[3], f1[3], f2[3], e;
        if (!angle_term(P, tc, A, B, f0, f1, f2, &e)) continue;
        fcx += f0[0];
        fcy += f0[1];
        fcz += f0[2];
        atomic_add3(S.frc_new, ja, f1[0], f1[1], f1[2]);
        atomic_add3(S.frc_new, jb, f2[0], f2[1], f2[2]);
        if (ENERGY) {
          uc += e / 3.0;
          atomicAdd(&S.epot[ja], e / 3.0);
          atomicAdd(&S.epot[jb], e / 3.0);
        }
      }
    }
    atomic_add3(S.frc_new, c, fcx, fcy, fcz);
    if (ENERGY && uc != 0.0) atomicAdd(&S.epot[c], uc);
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
  const int cnt = *((volatile int*)&S.sc->fast_count);
  for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < cnt; h += gridDim.x * blockDim.x) {
    const int f = S.fast_list[h];
    const int tf = S.atype[f];
    if (tf >= 3) continue;
    const double4_32a pf = S.pos[f];
    const int4 qf = S.posq[f];
    const int nf = S.n_sw[f];
    unsigned int terms = 0;
    for (int ia = 0; ia < nf; ia++) {
      const int a = S.nbr_sw[(size_t)ia * P.N + f];
      const int na = S.n_sw[a];
      for (int ix = 0; ix < na; ix++) {
        const int x = S.nbr_sw[(size_t)ix * P.N + a];
        if (x == f) continue;
        const int4 qx = S.posq[x];
        const float3 dq = qsep(qf, qx, P.qinvA);
        if (dq.x * dq.x + dq.y * dq.y + dq.z * dq.z > P.pre3A2) continue;
        if (S.fast_flag[x] && x < f) continue;  // the pair is handled from x
        if (in_list(P, S, f, x)) continue;
        const int ta = S.atype[a], tx = S.atype[x];
        const double4_32a pa = S.pos[a], px = S.pos[x];
        double f0[3], f1[3], f2[3], e;
        // centre f, legs a and x
        {
          const Leg64 A = make_leg(P, pf, pa, tf, ta);
          const Leg64 X = make_leg(P, pf, px, tf, tx);
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
          const Leg64 A = make_leg(P, px, pa, tx, ta);
          const Leg64 Fl = make_leg(P, px, pf, tx, tf);
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
template <bool MIXED, bool ENERGY>
__global__ void k_force_moliere(DevParams P, DevState S) {
  int cnt = *((volatile int*)&S.sc->mol_count);
  if (cnt > P.mol_cap) cnt = P.mol_cap;
  unsigned int npair = 0;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += gridDim.x * blockDim.x) {
    const int2 pr = S.mol_pairs[e];
    const int i = pr.x, j = pr.y;
    // si_force skips unfired ions (si.f90:428); si_potential does not
    const bool fired = i < P.nfired && j < P.nfired;
    if (!ENERGY && !fired) continue;
    const int ti = S.atype[i] - 1, tj = S.atype[j] - 1;
    const double4_32a pi = S.pos[i], pj = S.pos[j];
    const double dx = min_image(pi.x, pj.x, P.iLb[0], P.Lb[0]);
    const double dy = min_image(pi.y, pj.y, P.iLb[1], P.Lb[1]);
    const double dz = min_image(pi.z, pj.z, P.iLb[2], P.Lb[2]);
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

__global__ void k_force_begin(DevState S) {
  if (threadIdx.x == 0) {
    S.sc->heavy_count = 0;
    S.sc->table_err = 0;
  }
  if (threadIdx.x < 4) S.sc->counters[threadIdx.x] = 0ull;
}

template <bool MIXED, bool ENERGY, bool COUNT>
static cudaError_t force_impl(const Launch& L, const DevParams& P, const DevState& S) {
  const size_t rsz = MIXED ? sizeof(float) : sizeof(double);
  constexpr int BLOCK = ForceBlock<MIXED>::value;
  const size_t smem = rsz * kMaxLegs * kLegF * BLOCK + sizeof(int) * kMaxLegs * BLOCK;
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_force<MIXED, ENERGY, COUNT>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr_set = true;
  }
  if (L.force_a) cudaEventRecord(L.force_a, L.stream);
  k_force<MIXED, ENERGY, COUNT><<<(P.N + BLOCK - 1) / BLOCK, BLOCK, smem, L.stream>>>(P, S);
  if (L.force_b) cudaEventRecord(L.force_b, L.stream);
  const int side = L.sms > 0 ? L.sms : 152;
  k_force_moliere<MIXED, ENERGY><<<side, 128, 0, L.stream>>>(P, S);
  k_force_heavy<ENERGY><<<side, 64, 0, L.stream>>>(P, S);
  if (P.mode == FIBMD_MODE_REF) k_force_stale<ENERGY><<<side, 64, 0, L.stream>>>(P, S);
  return cudaGetLastError();
}

cudaError_t launch_force(const Launch& L, const DevParams& P, const DevState& S, bool energy,
                         bool count) {
  cudaError_t e = cudaMemsetAsync(S.frc_new, 0, sizeof(double4_32a) * (size_t)P.N, L.stream);
  if (e != cudaSuccess) return e;
  if (energy) {
    e = cudaMemsetAsync(S.epot, 0, sizeof(double) * (size_t)P.N, L.stream);
    if (e != cudaSuccess) return e;
  }
  k_force_begin<<<1, 32, 0, L.stream>>>(S);
  const bool mixed = P.precision == FIBMD_PREC_MIXED;
  if (mixed) {
    if (energy) return count ? force_impl<true, true, true>(L, P, S) : force_impl<true, true, false>(L, P, S);
    return count ? force_impl<true, false, true>(L, P, S) : force_impl<true, false, false>(L, P, S);
  }
  if (energy) return count ? force_impl<false, true, true>(L, P, S) : force_impl<false, true, false>(L, P, S);
  return count ? force_impl<false, false, true>(L, P, S) : force_impl<false, false, false>(L, P, S);
}

}  // namespace fibmd
