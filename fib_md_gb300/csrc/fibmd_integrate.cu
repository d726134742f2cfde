// fibmd_integrate.cu — velocity-Verlet step and its reductions.
//
// Replaces onestep's position and velocity updates (src/timeint.f90:185-188,
// 231-236), controlsidetemp (src/temp.f90:32-67), adjusttemp/temperature
// (src/temp.f90:160-205), freezsidesN and rebox (src/tools.f90:26-51),
// frzsptrdatms (src/temp.f90:99-127) and calc_atm (src/timeint.f90:277-298).
// All updates are binary64 and keep the reference's operation order. The
// reference-mode sums use a deterministic two-level reduction (block
// partials summed in block order by the last block), so repeated runs give
// identical thermostat factors; the spec-mode kick adds its block partials
// with atomics (see spec_kick_chunk).
#include "fibmd_internal.cuh"

namespace fibmd {

// controlsidetemp's predicate, temp.f90:45-47. Fortran's .and. binds tighter
// than .or.: x-edge .or. (y-edge .and. z-band).
__device__ __forceinline__ bool ref_side_atom(const DevParams& P, double x, double y,
                                              double z) {
  const bool xe = (x < P.side_sw) || (x > (P.Lb[0] - P.side_sw));
  const bool ye = (y < P.side_sw) || (y > (P.Lb[1] - P.side_sw));
  const bool zb = (z < P.side_zlo) || (z > P.side_zhi);
  return xe || (ye && zb);
}

// Marks an atom displaced by at least half the list skin since the last
// build (its angle terms may include stale-list terms, ref mode) and returns
// the squared displacement in A^2 (spec-mode rebuild trigger). The
// displacement is taken between fixed-point positions, whose wrapping
// difference is the minimum image; its binary32 error (~1e-7 A) is far
// inside the 1% margin of the threshold.
__device__ __forceinline__ float track_displacement(const DevParams& P, const Geo& G,
                                                    const DevState& S, int i, const int4& q) {
  const float3 d = qsep(q, S.posq_build[i], G.qinvA);
  const float d2 = d.x * d.x + d.y * d.y + d.z * d.z;
  if (P.mode == FIBMD_MODE_REF && d2 >= P.disp_fastA2 && !S.fast_flag[i]) {
    S.fast_flag[i] = 1;
    const int slot = atomicAdd(&S.sc->fast_count, 1);
    S.fast_list[slot] = i;
  }
  return d2;
}

__device__ __forceinline__ int4 store_posq(const Geo& G, const DevState& S, int i, double x,
                                           double y, double z, uint32_t fl) {
  int4 q;
  q.x = (int)fixq(x, G.qscale[0]);
  q.y = (int)fixq(y, G.qscale[1]);
  q.z = (int)fixq(z, G.qscale[2]);
  q.w = posq_w(S.atype[i], fl);
  S.posq[i] = q;
  return q;
}

static int red_blocks(const DevParams& P) {
  int nb = (P.N + kRedThreads - 1) / kRedThreads;
  if (nb < 1) nb = 1;
  if (nb > kMaxRedBlocks) nb = kMaxRedBlocks;
  return nb;
}

// ---- controlsidetemp: sum m v^2 and count over edge atoms (atype < 3) -----
__global__ void __launch_bounds__(kRedThreads) k_side_reduce(DevParams P, DevState S, double Ts,
                                                             double Tau, double Ttar) {
  double v[2] = {0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.N; i += gridDim.x * blockDim.x) {
    if (S.atype[i] >= 3) continue;
    const double4_32a p = S.pos[i];
    if (!ref_side_atom(P, p.x, p.y, p.z)) continue;
    const double4_32a u = S.vel[i];
    v[0] += S.mass[i] * (u.x * u.x + u.y * u.y + u.z * u.z);
    v[1] += 1.0;
  }
  block_sum<2>(v);
  if (grid_finish<2, false>(v, S.partials, &S.sc->ticket[0])) {
    S.sc->side_sum = v[0];
    S.sc->side_cnt = v[1];
    double sf = 1.0;
    if (v[1] > 0.0) {
      // temp.f90:56-60, evaluated once for all edge atoms
      const double ts = v[0] / 3. / v[1] / P.kB;
      sf = sqrt(1. + Ts / Tau * (Ttar / ts - 1.));
    }
    S.sc->side_s = sf;
  }
}

cudaError_t launch_side_reduce(const Launch& L, const DevParams& P, const DevState& S,
                               double Ts, double Tau, double Ttar) {
  k_side_reduce<<<red_blocks(P), kRedThreads, 0, L.stream>>>(P, S, Ts, Tau, Ttar);
  return cudaGetLastError();
}

// ---- adjusttemp followed by temperature (warm-up, whichctrl 0) -------------
__global__ void __launch_bounds__(kRedThreads) k_adjust_temp(DevParams P, DevState S,
                                                             double Ts, double Tau,
                                                             double Ttar) {
  const double Temp = ((volatile DevScalars*)S.sc)->temp;
  const double s = sqrt(1. + Ts / Tau * (Ttar / Temp - 1.));
  double v[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.N; i += gridDim.x * blockDim.x) {
    if (S.atype[i] >= 3) continue;
    double4_32a u = S.vel[i];
    u.x = s * u.x;
    u.y = s * u.y;
    u.z = s * u.z;
    S.vel[i] = u;
    v[0] += S.mass[i] * (u.x * u.x + u.y * u.y + u.z * u.z);
  }
  block_sum<1>(v);
  // the last block writes the new temperature after every block has read
  // the old one
  if (grid_finish<1, false>(v, S.partials, &S.sc->ticket[1]))
    S.sc->temp = v[0] / 3. / (double)P.Nsg / P.kB;
}

cudaError_t launch_adjust_and_temp(const Launch& L, const DevParams& P, const DevState& S,
                                   double Ts, double Tau, double Ttar) {
  k_adjust_temp<<<red_blocks(P), kRedThreads, 0, L.stream>>>(P, S, Ts, Tau, Ttar);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(kRedThreads) k_temperature(DevParams P, DevState S) {
  double v[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.N; i += gridDim.x * blockDim.x) {
    if (S.atype[i] >= 3) continue;
    const double4_32a u = S.vel[i];
    v[0] += S.mass[i] * (u.x * u.x + u.y * u.y + u.z * u.z);
  }
  block_sum<1>(v);
  if (grid_finish<1, false>(v, S.partials, &S.sc->ticket[2]))
    S.sc->temp = v[0] / 3. / (double)P.Nsg / P.kB;
}

cudaError_t launch_temperature(const Launch& L, const DevParams& P, const DevState& S) {
  k_temperature<<<red_blocks(P), kRedThreads, 0, L.stream>>>(P, S);
  return cudaGetLastError();
}

// ---- drift: edge thermostat, X += V Ts + F Ts^2/(2m), freeze, rebox --------
__global__ void __launch_bounds__(256) k_drift(DevParams P, DevState S, double Ts, int side) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.N) return;
  double4_32a x = S.pos[i];
  double4_32a v = S.vel[i];
  if (side && S.atype[i] < 3 && ref_side_atom(P, x.x, x.y, x.z)) {
    const double s = S.sc->side_s;
    v.x = s * v.x;
    v.y = s * v.y;
    v.z = s * v.z;
  }
  const double4_32a f = S.frc[i];
  const double c = 0.5 * Ts * Ts * S.inv_mass[i];
  x.x = x.x + v.x * Ts + c * f.x;
  x.y = x.y + v.y * Ts + c * f.y;
  x.z = x.z + v.z * Ts + c * f.z;
  const uint32_t fl = S.flags[i];
  if (fl & FL_FROZEN) {
    const double4_32a xi = S.xi[i];
    x.x = xi.x;
    x.y = xi.y;
    x.z = xi.z;
    v.x = 0.;
    v.y = 0.;
    v.z = 0.;
  }
  x.x = rebox1(x.x, P.Lb[0]);
  x.y = rebox1(x.y, P.Lb[1]);
  x.z = rebox1(x.z, P.Lb[2]);
  S.pos[i] = x;
  S.vel[i] = v;
  const Geo& G = S.geo[0];
  const int4 q = store_posq(G, S, i, x.x, x.y, x.z, fl);
  track_displacement(P, G, S, i, q);
}

cudaError_t launch_drift(const Launch& L, const DevParams& P, const DevState& S, double Ts,
                         double Tau, double Ttar, int side_thermo) {
  (void)Tau;
  (void)Ttar;
  k_drift<<<(P.N + 255) / 256, 256, 0, L.stream>>>(P, S, Ts, side_thermo);
  return cudaGetLastError();
}

// ---- frzsptrdatms: park sputtered atoms in the vacuum bands ----------------
__global__ void __launch_bounds__(256) k_park(DevParams P, DevState S) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.N) return;
  double4_32a x = S.pos[i];
  const double z = x.z;
  bool hit = false, moved = false;
  if ((z > P.park_o[0]) && (z < P.park_o[1])) {
    x.z = P.park_a[0];
    hit = moved = true;
  } else if ((z > P.park_o[2]) && (z < P.park_o[3])) {
    x.z = P.park_a[1];
    hit = moved = true;
  } else if ((z > P.park_al[0]) && (z < P.park_ah[0])) {
    hit = true;
  } else if ((z > P.park_al[1]) && (z < P.park_ah[1])) {
    hit = true;
  } else if ((z > P.park_il) && (z < P.park_ih)) {
    hit = true;
  }
  if (!hit) return;
  S.vel[i] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
  S.frc[i] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
  if (moved) {
    S.pos[i] = x;
    const Geo& G = S.geo[0];
    const int4 q = store_posq(G, S, i, x.x, x.y, x.z, S.flags[i]);
    track_displacement(P, G, S, i, q);
  }
}

cudaError_t launch_park(const Launch& L, const DevParams& P, const DevState& S) {
  k_park<<<(P.N + 255) / 256, 256, 0, L.stream>>>(P, S);
  return cudaGetLastError();
}

// ---- kick: V += (F + Fp) Ts / (2m) -----------------------------------------
__global__ void __launch_bounds__(256) k_kick(DevParams P, DevState S, double Ts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.N) return;
  double4_32a v = S.vel[i];
  const double4_32a f = S.frc[i];
  const double4_32a g = S.frc_new[i];
  const double c = 0.5 * Ts * S.inv_mass[i];
  v.x = v.x + c * (f.x + g.x);
  v.y = v.y + c * (f.y + g.y);
  v.z = v.z + c * (f.z + g.z);
  S.vel[i] = v;
  if (!(v.x * v.x + v.y * v.y + v.z * v.z < INFINITY)) atomicOr(&S.sc->nan_flag, 1);
}

cudaError_t launch_kick(const Launch& L, const DevParams& P, const DevState& S, double Ts) {
  k_kick<<<(P.N + 255) / 256, 256, 0, L.stream>>>(P, S, Ts);
  return cudaGetLastError();
}

// ---- calc_atm: max over atoms of 0.5 m |v|^2 / ec --------------------------
__global__ void __launch_bounds__(kRedThreads) k_ke_max(DevParams P, DevState S) {
  double v[1] = {-1.0e300};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.N; i += gridDim.x * blockDim.x) {
    const double4_32a u = S.vel[i];
    double ss = 0.0;
    ss += u.x * u.x;
    ss += u.y * u.y;
    ss += u.z * u.z;
    v[0] = fmax(v[0], 0.5 * S.mass[i] * ss / P.ec);
  }
  v[0] = block_max(v[0]);
  if (grid_finish<1, true>(v, S.partials, &S.sc->ticket[3])) S.sc->ke_max = v[0];
}

cudaError_t launch_ke_max(const Launch& L, const DevParams& P, const DevState& S) {
  k_ke_max<<<red_blocks(P), kRedThreads, 0, L.stream>>>(P, S);
  return cudaGetLastError();
}

// Re-evaluates every atom's displacement since the last list build after the
// host replaced positions (upload, set_atom), so stale-list terms stay
// covered.
__global__ void k_track_all(DevParams P, DevState S) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.N) return;
  const int4 q = S.posq[i];
  track_displacement(P, S.geo[rep_of_w(q.w)], S, i, q);
}

cudaError_t launch_track_all(const Launch& L, const DevParams& P, const DevState& S) {
  k_track_all<<<(P.N + 255) / 256, 256, 0, L.stream>>>(P, S);
  return cudaGetLastError();
}

// ---- layout conversion: (N,3) column-major <-> double4_32a ---------------------
__global__ void k_pack(int N, double4_32a* dst, const double* src) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  dst[i] = make_double4_32a(src[i], src[(size_t)N + i], src[2 * (size_t)N + i], 0.0);
}

__global__ void k_unpack(int N, const double4_32a* src, double* dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const double4_32a v = src[i];
  dst[i] = v.x;
  dst[(size_t)N + i] = v.y;
  dst[2 * (size_t)N + i] = v.z;
}

cudaError_t launch_pack(const Launch& L, int N, double4_32a* dst, const double* src_cm) {
  k_pack<<<(N + 255) / 256, 256, 0, L.stream>>>(N, dst, src_cm);
  return cudaGetLastError();
}

cudaError_t launch_unpack(const Launch& L, int N, const double4_32a* src, double* dst_cm) {
  k_unpack<<<(N + 255) / 256, 256, 0, L.stream>>>(N, src, dst_cm);
  return cudaGetLastError();
}

// ---- total energies ---------------------------------------------------------
__global__ void __launch_bounds__(kRedThreads) k_energy_sum(DevParams P, DevState S) {
  double v[2] = {0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.N; i += gridDim.x * blockDim.x) {
    if (S.flags[i] & FL_REMOVED) continue;
    const double4_32a u = S.vel[i];
    v[0] += 0.5 * S.mass[i] * (u.x * u.x + u.y * u.y + u.z * u.z);
    v[1] += S.epot[i];
  }
  block_sum<2>(v);
  if (grid_finish<2, false>(v, S.partials, &S.sc->ticket[4])) {
    S.sc->ekin = v[0];
    S.sc->epot = v[1];
  }
}

cudaError_t launch_energy_sum(const Launch& L, const DevParams& P, const DevState& S) {
  k_energy_sum<<<red_blocks(P), kRedThreads, 0, L.stream>>>(P, S);
  return cudaGetLastError();
}

// ---- spec mode ----------------------------------------------------------------
// Both spec-mode kernels issue every load of an atom before its first use, so
// a thread waits for one memory round trip rather than a chain of them (the
// flags, then the replica's scalars, then the state); removal only masks the
// stores. BATCH = 0 (a single system) takes the replica's geometry and
// scalars without reading the flags first.

// ---- the pair rule, decided where the displacements are ----
// The chunk's two largest reported |d|^2 b1 >= b2 (non-negative binary32,
// ordered as their bit patterns) and one atomicMax on the replica's running
// largest of the step, which returns the largest reported before: the
// chunk's candidate pair is (max(b1, old), max(min(b1, old), b2)). The
// step's two largest t1 >= t2 are the candidate pair of the chunk holding
// both, or of the later of the two chunks holding them (the running largest
// it sees is the other one), and no chunk's pair exceeds them, so some chunk
// reaches each threshold exactly when (t1, t2) does: the rule needs no pass
// after the drift. Returns, in thread 0: 2, a rebuild (sqrt(p1) +
// sqrt(max(p2, the bound)) reaching the skin; the unreported displacements
// are below the bound); 1, half of it reached (a batch rebuilds such
// replicas with those that must, as the half-skin rule does those that
// moved a quarter of the skin); 0, neither. Called by every thread of the
// block; the kick's last chunk clears the running largest for the next step.
__device__ __forceinline__ int pair_report(const DevParams& P, DevScalars* R, float rep) {
  __shared__ unsigned top[2][kKickThreads / 32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned u = __float_as_uint(rep);
  const unsigned m1 = __reduce_max_sync(0xffffffffu, u);
  const unsigned first = __ffs(__ballot_sync(0xffffffffu, u == m1)) - 1;
  const unsigned m2 = __reduce_max_sync(0xffffffffu, lane == (int)first ? 0u : u);
  if (lane == 0) {
    top[0][w] = m1;
    top[1][w] = m2;
  }
  __syncthreads();
  if (threadIdx.x != 0) return 0;
  unsigned b1 = 0u, b2 = 0u;
  for (int k = 0; k < kKickThreads / 32; k++) {
    const unsigned a1 = top[0][k], a2 = top[1][k];
    if (a1 > b1) {
      b2 = max(b1, a2);
      b1 = a1;
    } else {
      b2 = max(b2, a1);
    }
  }
  const unsigned old = atomicMax(&R->disp_max, b1);
  const float p1 = __uint_as_float(max(b1, old));
  const float p2 = __uint_as_float(max(min(b1, old), b2));
  const float sum = sqrtf(p1) + sqrtf(fmaxf(p2, P.disp_lowA2));
  return sum >= P.disp_skinA ? 2 : (sum >= 0.5f * P.disp_skinA ? 1 : 0);
}

// Drift with the variable step held on the device, Berendsen scaling of the
// tagged thermostat layer, fixed-layer pinning, removal of atoms above
// remove_z (and, with an open z axis, of atoms 10 A below the lowest plane),
// and the rebuild trigger: the kKickThreads atoms of chunk c, one per
// thread. Returns, in every thread, bit 0 if an atom of the chunk moved half
// the skin since the last list build and (a batch) bit 1 if one moved a
// quarter of it. With the pair rule the chunk's two largest squared
// displacements at or above disp_lowA2 decide the same bits instead
// (pair_report: a rebuild of the replica, one halfway due), in thread 0
// only, which is where the callers read them.
template <int BATCH>
__device__ __forceinline__ int spec_drift_chunk(const DevParams& P, const DevState& S, int c) {
  const int i = c * kKickThreads + threadIdx.x;
  const bool pair = P.pair_rule;
  bool trig = false, soon = false;
  float rep = 0.f;                 // pair rule: this atom's reported |d|^2
  DevScalars* Rrep = S.sc;         // and its replica's scalars
  if (i < P.N) {
    uint32_t fl = S.flags[i];
    double4_32a x = S.pos[i];
    double4_32a v = S.vel[i];
    const double4_32a f = S.frc[i];
    const double im = S.inv_mass[i];
    const int8_t at = S.atype[i];
    const int4 qb = S.posq_build[i];
    const int r = BATCH ? rep_of_flags(fl) : 0;
    const Geo& G = S.geo[r];
    DevScalars* R = S.sc + r;
    Rrep = R;
    const double dt = R->dt;
    const double h2 = R->half_dt2;
    const double ts = R->thermo_s;
    if (!(fl & FL_REMOVED)) {
      if (fl & FL_THERMO) {
        v.x *= ts;
        v.y *= ts;
        v.z *= ts;
      }
      const double cc = h2 * im;
      x.x = x.x + v.x * dt + cc * f.x;
      x.y = x.y + v.y * dt + cc * f.y;
      x.z = x.z + v.z * dt + cc * f.z;
      if (fl & FL_FROZEN) {
        const double4_32a xi = S.xi[i];
        x.x = xi.x;
        x.y = xi.y;
        x.z = xi.z;
        v.x = v.y = v.z = 0.0;
      }
      // removal looks at the unwrapped height, so an atom leaving through
      // the bottom of a periodic box is not taken for a sputtered one
      const bool removed = (G.remove_z > 0.0 && x.z > G.remove_z) || x.z < G.remove_zlo;
      // spec mode has no bit-compatibility constraint with the reference's
      // MOD(X + 2Lb, Lb): only atoms that left the box are wrapped, found
      // from the integer part of the fixed-point shadow (one binary64 FMA
      // per axis gives both); with the cell grid cut at remove_z, z is an
      // open axis and is not wrapped
      long long k[3];
      double* xc[3] = {&x.x, &x.y, &x.z};
#pragma unroll
      for (int d = 0; d < 3; d++) {
        k[d] = fixq64(*xc[d], G.qscale[d]);
        if ((d < 2 || !G.zcompact) && (unsigned long long)k[d] >> 32) {
          *xc[d] += k[d] < 0 ? G.Lb[d] : -G.Lb[d];
          k[d] = fixq64(*xc[d], G.qscale[d]);
        }
      }
      if (removed) {
        // the force kernels skip removed neighbours, so the lists need no
        // rebuild for it
        fl |= FL_REMOVED;
        S.flags[i] = fl;
        v.x = v.y = v.z = 0.0;
        atomicAdd(at < 3 ? &R->removed_count : &R->ions_removed, 1);
      }
      S.pos[i] = x;
      // the velocity changes here only by the thermostat, pinning or removal
      if ((fl & (FL_THERMO | FL_FROZEN)) || removed) S.vel[i] = v;
      const int4 q = make_int4((int)(unsigned)k[0], (int)(unsigned)k[1], (int)(unsigned)k[2],
                               posq_w(at, fl));
      S.posq[i] = q;
      const float3 d = qsep(q, qb, G.qinvA);
      const float d2 = d.x * d.x + d.y * d.y + d.z * d.z;
      if (pair) {
        if (!removed && d2 >= P.disp_lowA2) rep = d2;
      } else if (!removed && d2 >= P.disp_fastA2) {
        trig = true;
      }
      // a batch also rebuilds, with a replica that must, those that have
      // moved a quarter of the skin: rebuilds stay few and in step
      if (BATCH && !removed && d2 >= 0.25f * P.disp_fastA2) soon = true;
    }
  }
  if (pair) {
    // thread 0 holds the chunk's first atom, of the chunk's replica
    if (!__syncthreads_or(rep > 0.f)) return 0;
    const int k = pair_report(P, Rrep, rep);
    return k == 2 ? 3 : (k == 1 ? 2 : 0);
  }
  const int any = __syncthreads_or(trig) ? 1 : 0;
  if (!BATCH) return any;
  return any | (__syncthreads_or(soon) ? 2 : 0);
}

// the force counters of the coming step (the previous step's force is done)
__device__ __forceinline__ void reset_force_counters(const DevState& S) {
  S.sc->heavy_count = 0;
  S.sc->table_err = 0;
  for (int k = 0; k < 4; k++) S.sc->counters[k] = 0ull;
}

template <int BATCH>
__global__ void __launch_bounds__(kKickThreads, 6) k_spec_drift(DevParams P, DevState S) {
  pdl_wait();
  pdl_trigger();
  const int moved = spec_drift_chunk<BATCH>(P, S, blockIdx.x);
  if (threadIdx.x != 0) return;
  if (moved & 1) S.sc->need_rebuild = 1;
  // a batch rebuilds the replicas that moved (chunks never straddle two)
  if (BATCH && moved) {
    DevScalars& R = S.sc[rep_of_flags(S.flags[blockIdx.x * kKickThreads])];
    if (moved & 1) R.rep_rebuild = 1;
    if (moved & 2) R.rep_soon = 1;
  }
  if (blockIdx.x == 0) reset_force_counters(S);
}

// Sets the graph's rebuild condition from the drift's flag. A kernel of its
// own rather than a last-block ticket in the drift: a same-address atomic
// from each of ~1000 blocks serialises in L2 for longer than a launch.
// With has_heavy, it also closes the step's many-leg IF node (heavy), which
// the force kernel opens when it finds such a centre.
__global__ void k_spec_cond(DevState S, cudaGraphConditionalHandle cond,
                            cudaGraphConditionalHandle heavy, int has_heavy) {
  pdl_wait();
  pdl_trigger();
  if (threadIdx.x == 0) {
    cudaGraphSetConditional(cond, ((volatile DevScalars*)S.sc)->need_rebuild ? 1u : 0u);
    if (has_heavy) cudaGraphSetConditional(heavy, 0u);
  }
}

// Clears every replica's running largest displacement of the pair rule (a
// new state).
__global__ void k_pair_clear(DevState S, int nrep) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nrep) S.sc[r].disp_max = 0u;
}

cudaError_t launch_pair_clear(const Launch& L, const DevParams& P, const DevState& S) {
  k_pair_clear<<<(P.nrep + 255) / 256, 256, 0, L.stream>>>(S, P.nrep);
  return cudaGetLastError();
}

cudaError_t launch_spec_drift(const Launch& L, const DevParams& P, const DevState& S,
                              double Ttar, const cudaGraphConditionalHandle* cond,
                              bool pdl_first, const cudaGraphConditionalHandle* heavy) {
  (void)Ttar;
  const int nb = (P.N + kKickThreads - 1) / kKickThreads;
  cudaError_t e = launch_k(P.nrep > 1 ? k_spec_drift<1> : k_spec_drift<0>, nb, kKickThreads, 0,
                           L.stream, L.pdl && pdl_first, P, S);
  // in a graph, the rebuild condition of the IF node that follows
  if (e == cudaSuccess && cond)
    e = launch_k(k_spec_cond, 1, 32, 0, L.stream, L.pdl, S, *cond,
                 heavy ? *heavy : cudaGraphConditionalHandle(0), heavy ? 1 : 0);
  return e;
}

// Kick (apply != 0) followed by the reductions the next step needs: the
// largest speed (variable dt = min(dt_max, dx_max / max|v|)) and the
// thermostat layer's sum m v^2 and count.
//
// The reductions stay off the critical path of the ~1000 co-resident
// blocks: the max of v^2 >= 0 is taken on its bit pattern (integer order),
// the layer count is an integer, only warps holding layer atoms sum m v^2
// (binary64 is scarce: a warp instruction holds the SM's FP64 unit for 16
// cycles), and after one barrier only warp 0 goes on. Each chunk adds its
// partial to the replica's running values with fire-and-forget atomics and
// counts itself on the replica's ticket; the last chunk reads the three
// values and derives dt and the Berendsen factor. (Completion counted in
// two levels, a ticket per group of 32 chunks whose last chunk combined the
// group's partials, took ~8 us of a 19.5 us kick at 256k on its critical
// path; this form 3 us less per step.) The thermostat sum's order is that
// in which the atomics arrive.

// Warp max of non-negative doubles held as bits: redux.sync on the high
// words, then on the low words of the lanes holding the high maximum.
__device__ __forceinline__ unsigned long long warp_max_bits(unsigned long long v) {
  const unsigned hi = __reduce_max_sync(0xffffffffu, (unsigned)(v >> 32));
  const unsigned lo = __reduce_max_sync(0xffffffffu, (unsigned)(v >> 32) == hi ? (unsigned)v : 0u);
  return ((unsigned long long)hi << 32) | lo;
}

__device__ __forceinline__ void kick_combine(unsigned long long& m, double& a, int& c) {
  m = warp_max_bits(m);
  c = (int)__reduce_add_sync(0xffffffffu, (unsigned)c);
  if (c) a = warp_sum(a);
}

// The kick of chunk c (kKickThreads atoms, one per thread; a chunk lies
// inside one replica, replicas starting at multiples of the chunk) and its
// share of the step's reductions. The block-partial stage is double-buffered
// by `buf`, so a block can take its next chunk while its warp 0 finishes the
// completion of this one. Returns the replica this call finalized (dt, the
// thermostat factor and the time written) in lane 0 of warp 0 of the block
// that finalized it, -1 everywhere else.
template <int BATCH>
__device__ __forceinline__ int spec_kick_chunk(const DevParams& P, const DevState& S, int c,
                                               int apply, double Ttar, int buf) {
  const int i = c * kKickThreads + threadIdx.x;
  uint32_t fl = FL_REMOVED;
  unsigned long long vb = 0ull;  // bits of v^2
  double ts = 0.0;
  int tc = 0;
  if (i < P.N) {
    fl = S.flags[i];
    double4_32a v = S.vel[i];
    double4_32a f = {}, g = {};
    double im = 0.0;
    if (apply) {
      f = S.frc[i];
      g = S.frc_new[i];
      im = S.inv_mass[i];
    }
    const double m = S.mass[i];
    const int8_t at = S.atype[i];
    const double hdt = S.sc[BATCH ? rep_of_flags(fl) : 0].half_dt;
    if (!(fl & FL_REMOVED)) {
      if (apply) {
        const double cc = hdt * im;
        v.x = v.x + cc * (f.x + g.x);
        v.y = v.y + cc * (f.y + g.y);
        v.z = v.z + cc * (f.z + g.z);
        S.vel[i] = v;
        // the old force's buffer accumulates the next force (after the swap)
        S.frc[i] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
      }
      const double v2 = v.x * v.x + v.y * v.y + v.z * v.z;
      vb = (unsigned long long)__double_as_longlong(v2);
      // a non-finite force or velocity shows here (exponent all ones, or a
      // negative NaN); the host reports it
      if (vb >= 0x7ff0000000000000ull) {
        atomicOr(&S.sc->nan_flag, 1);
        vb = 0ull;
      } else if ((fl & FL_THERMO) && at < 3) {
        ts = m * v2;
        tc = 1;
      }
    }
  }
  kick_combine(vb, ts, tc);
  __shared__ unsigned long long smax[2][kKickThreads / 32];
  __shared__ double ssum[2][kKickThreads / 32];
  __shared__ int scnt[2][kKickThreads / 32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    smax[buf][w] = vb;
    ssum[buf][w] = ts;
    scnt[buf][w] = tc;
  }
  __syncthreads();
  if (w != 0) return -1;
  // warp 0: the chunk's partial
  constexpr int kWarps = kKickThreads / 32;
  unsigned long long m = lane < kWarps ? smax[buf][lane] : 0ull;
  int cnt = lane < kWarps ? scnt[buf][lane] : 0;
  double a = cnt ? ssum[buf][lane] : 0.0;
  kick_combine(m, a, cnt);
  // the replica of this chunk: its first atom's, lane 0's (chunks never
  // straddle replicas, and a replica's padding only ends its last chunk)
  const int r = BATCH ? __shfl_sync(0xffffffffu, rep_of_flags(fl), 0) : 0;
  const Geo& G = S.geo[r];
  const int nblk = G.blk_end - G.blk_begin;
  DevScalars* R = S.sc + r;
  // The chunk adds its partial to the replica's running max (bit patterns
  // of non-negative binary64 values order as integers), thermostat-layer sum
  // and count, then counts itself; the replica's last chunk reads and
  // clears them. One level, three values read at the end: the completion
  // stays short on the critical path of every step.
  int st = 0;
  if (lane == 0) {
    if (m) atomicMax(&R->acc_vmax2, m);
    if (cnt) {
      atomicAdd(&R->acc_tsum, a);
      atomicAdd(&R->acc_tcnt, cnt);
    }
    __threadfence();
    st = atomicAdd(&R->ticket[5], 1u) == (unsigned)(nblk - 1);
  }
  if (!__shfl_sync(0xffffffffu, st, 0)) return -1;
  if (lane != 0) return -1;
  __threadfence();
  m = atomicExch(&R->acc_vmax2, 0ull);
  a = __longlong_as_double(
      (long long)atomicExch(reinterpret_cast<unsigned long long*>(&R->acc_tsum), 0ull));
  cnt = atomicExch(&R->acc_tcnt, 0);
  R->ticket[5] = 0u;
  const double mx = __longlong_as_double((long long)m);
  const double tsum = a, tcnt = (double)cnt;
  R->thermo_sum = tsum;
  R->thermo_cnt = tcnt;
  R->vmax2 = mx;
  // the pair rule's running largest displacement, for the next drift
  R->disp_max = 0u;
  if (apply) R->time += R->dt;
  const double vm = sqrt(mx);
  double nd = P.dt_max;
  if (vm > 0.0 && P.dx_max / vm < nd) nd = P.dx_max / vm;
  R->dt = nd;
  R->half_dt = 0.5 * nd;
  R->half_dt2 = 0.5 * nd * nd;
  // Berendsen factor of the thermostat layer for the next step
  double sf = 1.0;
  if (tcnt > 0.0) {
    const double T = tsum / 3. / tcnt / P.kB;
    if (T > 0.0) sf = sqrt(1. + nd / P.tau_spec * (Ttar / T - 1.));
  }
  R->thermo_s = sf;
  return r;
}

template <int BATCH>
__global__ void __launch_bounds__(kKickThreads) k_spec_kick(DevParams P, DevState S, int apply,
                                                             double Ttar) {
  pdl_wait();
  pdl_trigger();
  spec_kick_chunk<BATCH>(P, S, blockIdx.x, apply, Ttar, 0);
}

cudaError_t launch_spec_kick(const Launch& L, const DevParams& P, const DevState& S,
                             double Ttar, int apply) {
  const int nb = (P.N + kKickThreads - 1) / kKickThreads;
  if (nb > kMaxRedBlocks) return cudaErrorInvalidConfiguration;
  // a programmatic dependent of the force kernels before it
  return launch_k(P.nrep > 1 ? k_spec_kick<1> : k_spec_kick<0>, nb, kKickThreads, 0, L.stream,
                  L.pdl && apply, P, S, apply, Ttar);
}

// ---- the kick of a step fused with the drift of the next -----------------
// One persistent grid of at most as many blocks as the device holds at once
// takes the chunks of kKickThreads atoms in turn: it kicks every chunk (the
// kick above, completion tickets and all), waits at a grid barrier, then
// drifts every chunk with the dt and thermostat factor just derived (the
// drift above). The barrier is the kick's own completion: the warp that
// finalizes the step's reductions (for a batch, the last of the replicas'
// final warps) also decides whether the step loop goes on, sets the graph's
// conditions (the rebuild IF node's to 0, the loop's WHILE node's when the
// kernel ends a step pair), resets the force counters and releases the
// others by advancing a generation counter; they spin on it with a bounded
// wait (kKdSpinLimit polls, then a time-out flag that the host reports as
// FIBMD_ETIMEOUT, and no drift). When the loop stops, nothing drifts and the
// state is that of a completed step. A block whose chunk moved an atom half
// the skin sets the rebuild condition to 1.
constexpr long long kKdSpinLimit = 1ll << 22;  // ~0.5 s with the back-off below

__device__ __forceinline__ void kd_release(const DevState& S, LoopCtl* loop,
                                           cudaGraphConditionalHandle hif,
                                           cudaGraphConditionalHandle hwhile, int last_of_pair,
                                           cudaGraphConditionalHandle hheavy, int has_heavy) {
  DevScalars* sc = S.sc;
  reset_force_counters(S);
  // the next step's many-leg IF node: closed until its force opens it
  if (has_heavy) cudaGraphSetConditional(hheavy, 0u);
  int cont = 1;
  if (last_of_pair) {
    const long long r = loop->pairs - 1;
    loop->pairs = r;
    loop->pairs_run += 1;
    cont = (r > 0 && ((volatile DevScalars*)sc)->time < loop->t_stop) ? 1 : 0;
    cudaGraphSetConditional(hwhile, (unsigned)cont);
  }
  cudaGraphSetConditional(hif, 0u);
  sc->kd_cont = cont;
  __threadfence();
  atomicAdd(&sc->kd_gen, 1u);
}

template <int BATCH>
__global__ void __launch_bounds__(kKickThreads) k_spec_kd(DevParams P, DevState S, double Ttar,
                                                           LoopCtl* loop,
                                                           cudaGraphConditionalHandle hif,
                                                           cudaGraphConditionalHandle hwhile,
                                                           int last_of_pair,
                                                           cudaGraphConditionalHandle hheavy,
                                                           int has_heavy) {
  const int nchunk = (P.N + kKickThreads - 1) / kKickThreads;
  DevScalars* sc = S.sc;
  __shared__ unsigned gen0;
  __shared__ int go;
  // the generation before this block's chunks can complete the step
  if (threadIdx.x == 0) gen0 = ((volatile DevScalars*)sc)->kd_gen;
  __syncthreads();
  int it = 0;
  for (int c = blockIdx.x; c < nchunk; c += gridDim.x, it++) {
    const int r = spec_kick_chunk<BATCH>(P, S, c, 1, Ttar, it & 1);
    if (r >= 0) {
      bool release = true;
      if (BATCH) {
        __threadfence();
        release = atomicAdd(&sc->kd_reps, 1u) == (unsigned)(P.nrep - 1);
        if (release) sc->kd_reps = 0u;
      }
      if (release) {
        __threadfence();
        kd_release(S, loop, hif, hwhile, last_of_pair, hheavy, has_heavy);
      }
    }
  }
  if (threadIdx.x == 0) {
    long long n = 0;
    int ok = 1;
    while (((volatile DevScalars*)sc)->kd_gen == gen0) {
      if (++n > kKdSpinLimit) {
        ok = 0;
        atomicOr(&sc->kd_timeout, 1);
        break;
      }
      __nanosleep(100);
    }
    __threadfence();
    go = ok && ((volatile DevScalars*)sc)->kd_cont;
  }
  __syncthreads();
  if (!go) return;
  // the drift of the next step uses the force just computed (the host swaps
  // the two buffers after a kick; here the kick zeroed the older one)
  DevState Sn = S;
  Sn.frc = S.frc_new;
  Sn.frc_new = S.frc;
  for (int c = blockIdx.x; c < nchunk; c += gridDim.x) {
    const int moved = spec_drift_chunk<BATCH>(P, Sn, c);
    if (threadIdx.x == 0 && moved) {
      if (BATCH) {
        DevScalars& R = S.sc[rep_of_flags(S.flags[c * kKickThreads])];
        if (moved & 1) R.rep_rebuild = 1;
        if (moved & 2) R.rep_soon = 1;
      }
      if (moved & 1) {
        sc->need_rebuild = 1;
        cudaGraphSetConditional(hif, 1u);
      }
    }
  }
}

// Blocks of k_spec_kd the device holds at once (the grid of every launch is
// at most this, so that all of its blocks are resident together).
int spec_kd_resident_blocks(int nrep, int sms) {
  int per_sm = 0;
  const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, nrep > 1 ? k_spec_kd<1> : k_spec_kd<0>, kKickThreads, 0);
  if (e != cudaSuccess || per_sm < 1) return 0;
  return per_sm * sms;
}

cudaError_t launch_spec_kd(const Launch& L, const DevParams& P, const DevState& S, double Ttar,
                           LoopCtl* loop, cudaGraphConditionalHandle hif,
                           cudaGraphConditionalHandle hwhile, int last_of_pair, int max_blocks,
                           const cudaGraphConditionalHandle* heavy) {
  const int nchunk = (P.N + kKickThreads - 1) / kKickThreads;
  if (nchunk > kMaxRedBlocks || max_blocks < 1) return cudaErrorInvalidConfiguration;
  const int nb = min(nchunk, max_blocks);
  const cudaGraphConditionalHandle hh = heavy ? *heavy : cudaGraphConditionalHandle(0);
  const int has = heavy ? 1 : 0;
  if (P.nrep > 1)
    k_spec_kd<1><<<nb, kKickThreads, 0, L.stream>>>(P, S, Ttar, loop, hif, hwhile, last_of_pair,
                                                    hh, has);
  else
    k_spec_kd<0><<<nb, kKickThreads, 0, L.stream>>>(P, S, Ttar, loop, hif, hwhile, last_of_pair,
                                                    hh, has);
  return cudaGetLastError();
}

// ---- dose: successive impacts without host round trips ---------------------
// The device side of knock (src/knock.f90:21-55) for a dose: impact k's ion,
// a pre-allocated atom kept removed until now, gets its start position and
// velocity and joins the run; the lists are rebuilt before the next force.
__global__ void k_inject(DevParams P, DevState S, const Impact* table, int k) {
  const Impact m = table[k];
  const int i = m.atom;
  const uint32_t fl = S.flags[i] & ~(uint32_t)FL_REMOVED;
  S.flags[i] = fl;
  S.pos[i] = make_double4_32a(m.x[0], m.x[1], m.x[2], 0.0);
  S.vel[i] = make_double4_32a(m.v[0], m.v[1], m.v[2], 0.0);
  S.frc[i] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
  S.frc_new[i] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
  const int4 q = store_posq(S.geo[rep_of_flags(fl)], S, i, m.x[0], m.x[1], m.x[2], fl);
  S.posq_build[i] = q;
  S.sc->need_rebuild = 1;
  S.sc->rebuild_all = 1;
  (void)P;
}

cudaError_t launch_inject(const Launch& L, const DevParams& P, const DevState& S,
                          const Impact* table, int k) {
  k_inject<<<1, 1, 0, L.stream>>>(P, S, table, k);
  return cudaGetLastError();
}

__global__ void k_dose_record(DevState S, const LoopCtl* loop, int k, int* removed,
                              int* ions_removed, double* time, long long* steps) {
  const volatile DevScalars* sc = S.sc;
  removed[k] = sc->removed_count;
  ions_removed[k] = sc->ions_removed;
  time[k] = sc->time;
  steps[k] = 2 * ((const volatile LoopCtl*)loop)->pairs_run;
}

cudaError_t launch_dose_record(const Launch& L, const DevState& S, const LoopCtl* loop, int k,
                               int* removed, int* ions_removed, double* time, long long* steps) {
  k_dose_record<<<1, 1, 0, L.stream>>>(S, loop, k, removed, ions_removed, time, steps);
  return cudaGetLastError();
}

// ---- writeatoms' columns, packed on the device ----------------------------------
// x y z in Angstrom ((N,3) column-major) and 0.5 m |v|^2 in eV with the
// reference's factor and operation order (src/out.f90:82-90).
__global__ void k_xyz_frame(int N, const double4_32a* __restrict__ pos,
                            const double4_32a* __restrict__ vel, const double* __restrict__ mass,
                            double* xyz, double* ke) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const double4_32a x = pos[i], v = vel[i];
  xyz[i] = x.x * 1e10;
  xyz[(size_t)N + i] = x.y * 1e10;
  xyz[2 * (size_t)N + i] = x.z * 1e10;
  const double coef = 6.252e18;  // J -> eV as the reference writes it
  ke[i] = 0.5 * mass[i] * (v.x * v.x + v.y * v.y + v.z * v.z) * coef;
}

cudaError_t launch_xyz_frame(const Launch& L, const DevState& S, int N, double* xyz, double* ke) {
  k_xyz_frame<<<(N + 255) / 256, 256, 0, L.stream>>>(N, S.pos, S.vel, S.mass, xyz, ke);
  return cudaGetLastError();
}

// ---- outcome of each impact, one block per replica -----------------------------
// Lattice atoms farther than `thr` from their initial site (minimum image in
// x and y, removed atoms left out), and the depth of the replica's first ion
// below its surface height (NaN when the ion is above it or removed).
__global__ void __launch_bounds__(256) k_impact_stats(DevState S, const double* surface_z,
                                                      double thr2, int* displaced,
                                                      double* ion_depth) {
  const int r = blockIdx.x;
  const Geo& G = S.geo[r];
  int cnt = 0;
  int ion = 0x7fffffff;
  for (int i = G.atom_begin + threadIdx.x; i < G.atom_end; i += blockDim.x) {
    const uint32_t fl = S.flags[i];
    if (fl & FL_REMOVED) continue;
    if (S.atype[i] == 3) {
      ion = min(ion, i);
      continue;
    }
    const double4_32a x = S.pos[i], x0 = S.xi[i];
    double dx = x.x - x0.x, dy = x.y - x0.y;
    dx -= G.Lb[0] * rint(dx * G.iLb[0]);
    dy -= G.Lb[1] * rint(dy * G.iLb[1]);
    const double dz = x.z - x0.z;
    if (dx * dx + dy * dy + dz * dz > thr2) cnt++;
  }
  __shared__ int s_cnt, s_ion;
  if (threadIdx.x == 0) {
    s_cnt = 0;
    s_ion = 0x7fffffff;
  }
  __syncthreads();
  if (cnt) atomicAdd(&s_cnt, cnt);
  if (ion != 0x7fffffff) atomicMin(&s_ion, ion);
  __syncthreads();
  if (threadIdx.x != 0) return;
  displaced[r] = s_cnt;
  double depth = nan("");
  if (s_ion != 0x7fffffff) {
    const double z = S.pos[s_ion].z;
    if (z <= surface_z[r]) depth = surface_z[r] - z;
  }
  ion_depth[r] = depth;
}

cudaError_t launch_impact_stats(const Launch& L, const DevParams& P, const DevState& S,
                                const double* surface_z, double thr, int* displaced,
                                double* ion_depth) {
  k_impact_stats<<<P.nrep, 256, 0, L.stream>>>(S, surface_z, thr * thr, displaced, ion_depth);
  return cudaGetLastError();
}

}  // namespace fibmd
