// fibmd_nlist.cu — cell binning and Verlet-list build.
//
// Replaces chainlist/atomcell (src/nlist.f90:20-66) and the pair part of
// si_nlistG (src/si.f90:102-189). The reference threads a linked list
// (HOC/LL) through (Nc+2)^3 cells with periodic ghost layers copied only when
// Nc > 2; here the same cell geometry is a counting sort (count, scan,
// scatter, per-cell order), and each centre scans the same 27-cell stencil
// (wrapping only on axes with Nc > 2). Pairs are decided by the reference's
// binary64 test r^2 < rc^2 (rclj^2 for pairs with an ion) on its minimum
// image, evaluated without contraction; a binary32 fixed-point prefilter
// with a safety band skips the binary64 work for pairs far from the radius.
#include "fibmd_internal.cuh"

namespace fibmd {

// ---- fixed-point shadow --------------------------------------------------
__global__ void k_update_posq(DevParams P, DevState S) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.N) return;
  double4_32a p = S.pos[i];
  const uint32_t fl = S.flags[i];
  const Geo& G = S.geo[rep_of_flags(fl)];
  int4 q;
  q.x = (int)fixq(p.x, G.qscale[0]);
  q.y = (int)fixq(p.y, G.qscale[1]);
  q.z = (int)fixq(p.z, G.qscale[2]);
  q.w = posq_w(S.atype[i], fl);
  S.posq[i] = q;
}

cudaError_t launch_update_posq(const Launch& L, const DevParams& P, const DevState& S) {
  int nb = (P.N + 255) / 256;
  k_update_posq<<<nb, 256, 0, L.stream>>>(P, S);
  return cudaGetLastError();
}

// ---- counting sort into the reference's cell grid ------------------------
__device__ __forceinline__ bool rebuild_skipped(const DevState& S, int from_flag) {
  return from_flag && !((volatile DevScalars*)S.sc)->need_rebuild;
}

// Whether replica r's SW lists are rebuilt (from_flag 2: per replica, those
// due by the rebuild rule and, with them, those halfway there).
__device__ __forceinline__ bool rep_rebuilt(const DevParams& P, const DevState& S, int from_flag,
                                            int r) {
  if (from_flag != 2 || P.nrep <= 1 || ((volatile DevScalars*)S.sc)->rebuild_all) return true;
  const volatile DevScalars* R = S.sc + r;
  return R->rep_rebuild || R->rep_soon;
}

__global__ void k_build_begin(DevParams P, DevState S, int from_flag) {
  if (rebuild_skipped(S, from_flag)) return;
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < P.ncell + 1) S.cell_count[c] = 0;
  if (c == 0) {
    S.sc->mol_count = 0;
    S.sc->fast_count = 0;
    S.sc->overflow_sw = 0;
    S.sc->sw_needed = 0;
    S.sc->overflow_mol = 0;
    S.sc->cell_oob = 0;
    S.sc->disp_max2 = 0.0;
  }
}

// atomcell (nlist.f90:28-30): Icell = INT((X - FLOOR(X*iLb)*Lb)/h) + 1.
// The cell along an axis is floor(x nc / Lb), which the fixed-point shadow
// q = round(x 2^32 / Lb) gives as (q nc) >> 32 with integer arithmetic. The
// two agree except within ~nc 2^-33 of a cell boundary; there (fraction
// within 1e-6 of a boundary) the reference's binary64 formula decides, so
// the cell of every atom is the reference's.
__device__ __forceinline__ int ref_cell(const Geo& G, double x, int d) {
  const double fl = floor(__dmul_rn(x, G.iLb[d]));
  const double t = __ddiv_rn(__dsub_rn(x, __dmul_rn(fl, G.Lb[d])), G.hcell[d]);
  return (int)t;
}

__global__ void k_cell_assign(DevParams P, DevState S, int from_flag) {
  if (rebuild_skipped(S, from_flag)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.N) return;
  const int4 q = S.posq[i];
  // every atom is binned (the ion pairs and the rebuilt replicas' stencils
  // read the cells); only a rebuilt replica's lists restart
  const bool act = rep_rebuilt(P, S, from_flag, rep_of_w(q.w));
  if (act) {
    S.n_sw[i] = 0;  // the list build appends with atomics
    S.sw_extra[i] = 0;
  }
  if ((q.w >> 8) & FL_REMOVED) {
    S.atom_cell[i] = -1;
    if (act) {
      S.posq_build[i] = q;
      S.fast_flag[i] = 0;
    }
    return;
  }
  const Geo& G = S.geo[rep_of_w(q.w)];
  const unsigned qq[3] = {(unsigned)q.x, (unsigned)q.y, (unsigned)q.z};
  constexpr unsigned kGuard = 4295u;  // 1e-6 of a cell, in units of 2^-32
  int ic[3];
  bool oob = false;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const unsigned long long t = (unsigned long long)qq[d] * (unsigned long long)G.nc[d];
    int c = (int)(t >> 32);
    const unsigned frac = (unsigned)t;
    if (d == 2 && G.zcompact) {
      // spec mode with an open z axis: the grid covers [0, remove_z + rc);
      // an atom above it (an ion: other atoms there are removed) joins the
      // top layer and an atom below z = 0 the bottom one, which hold every
      // atom within rc of it
      const double zc = S.pos[i].z * G.inv_hz;
      c = zc < 0.0 ? 0 : (zc >= (double)G.nc[2] ? G.nc[2] - 1 : (int)zc);
    } else if (frac < kGuard || frac > 0xffffffffu - kGuard) {
      const double4_32a p = S.pos[i];
      c = ref_cell(G, d == 0 ? p.x : d == 1 ? p.y : p.z, d);
    }
    if (c < 0 || c >= G.nc[d]) {
      oob = true;
      c = c < 0 ? 0 : G.nc[d] - 1;
    }
    ic[d] = c;
  }
  if (oob) atomicAdd(&S.sc->cell_oob, 1);
  const int cell = G.cell_off + ic[0] + G.nc[0] * (ic[1] + G.nc[1] * ic[2]);
  S.atom_cell[i] = cell;
  atomicAdd(&S.cell_count[cell], 1);
}

// Exclusive scan of cell_count (ncell+1 entries) into cell_start.
constexpr int kScanBlock = 1024;

__global__ void k_scan_local(DevParams P, DevState S, int from_flag) {
  if (rebuild_skipped(S, from_flag)) return;
  __shared__ int warp_tot[32];
  int n = P.ncell + 1;
  int g = blockIdx.x * kScanBlock + threadIdx.x;
  int v = g < n ? S.cell_count[g] : 0;
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  if (w == 0) {
    int t = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    warp_tot[lane] = t;
  }
  __syncthreads();
  int base = w > 0 ? warp_tot[w - 1] : 0;
  if (g < n) S.cell_start[g] = base + x - v;
  if (threadIdx.x == kScanBlock - 1) S.scan_blocks[blockIdx.x] = base + x;
}

__global__ void k_scan_top(DevParams P, DevState S, int nblocks, int from_flag) {
  if (rebuild_skipped(S, from_flag)) return;
  __shared__ int warp_tot[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int base0 = 0; base0 < nblocks; base0 += kScanBlock) {
    int g = base0 + threadIdx.x;
    int v = g < nblocks ? S.scan_blocks[g] : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
      int t = warp_tot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      warp_tot[lane] = t;
    }
    __syncthreads();
    int wb = w > 0 ? warp_tot[w - 1] : 0;
    int c0 = carry;
    if (g < nblocks) S.scan_blocks[g] = c0 + wb + x - v;  // exclusive
    __syncthreads();
    if (threadIdx.x == kScanBlock - 1) carry = c0 + wb + x;
    __syncthreads();
  }
}

__global__ void k_scan_add(DevParams P, DevState S, int from_flag) {
  if (rebuild_skipped(S, from_flag)) return;
  int n = P.ncell + 1;
  int g = blockIdx.x * kScanBlock + threadIdx.x;
  if (g < n) {
    S.cell_start[g] += S.scan_blocks[blockIdx.x];
    if (g < P.ncell) S.cell_count[g] = 0;  // reused as the fill cursor
  }
}

__global__ void k_cell_fill(DevParams P, DevState S, int from_flag) {
  if (rebuild_skipped(S, from_flag)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.N) return;
  const int c = S.atom_cell[i];
  if (c < 0) return;
  const int slot = S.cell_start[c] + atomicAdd(&S.cell_count[c], 1);
  S.cell_atoms[slot] = i;
  int4 q = S.posq[i];
  // spec mode lists ion pairs in a scan of its own: half a box away in x,
  // an ion never passes the SW distance test of the per-atom scan
  if (P.mol_reach > 1 && (q.w & 0xff) == 3) q.x = (int)((unsigned)q.x + 0x80000000u);
  S.posq_cell[slot] = q;
}

// ---- pair lists (si_nlistG pair loop, si.f90:130-189) ---------------------
// Exact list membership of a candidate already inside the FP32 prefilter
// band: the reference's binary64 minimum-image distance decides.
__device__ __forceinline__ bool exact_in(const Geo& G, const DevState& S, int i, int j,
                                         double rv2) {
  const double4_32a pi = S.pos[i], pj = S.pos[j];
  const double xx = min_image_exact(pi.x, pj.x, G.iLb[0], G.Lb[0]);
  const double yy = min_image_exact(pi.y, pj.y, G.iLb[1], G.Lb[1]);
  const double zz = min_image_exact(pi.z, pj.z, G.iLb[2], G.Lb[2]);
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(xx, xx), __dmul_rn(yy, yy)), __dmul_rn(zz, zz));
  return r2 < rv2;
}

// One thread per binned atom, in cell order, over half the stencil: the
// forward cells (dz = +1; dz = 0, dy = +1; dz = dy = 0, dx = +1) and the
// atoms after it in its own cell, so each pair is tested once and entered in
// both atoms' lists. The lanes of a warp hold the atoms of a few x-adjacent
// cells and walk nearly the same rows; a row of x-adjacent cells is one run
// of the cell-sorted arrays (two where it wraps in x). Candidates are tested
// in binary32 on the fixed-point separations; those inside the prefilter
// are buffered in shared memory and resolved after the scan (within 1e-4
// of a radius the reference's binary64 test decides), and the accepted
// pairs entered: the centre's own entries with one atomic reservation, each
// partner's with one atomic slot. A pair with an ion goes
// to the Moliere pair list in both orders; with WIDE (spec mode) the ion
// scan below lists those and ions are skipped here.
constexpr int kBuildThreads = 128;  // the default block (atoms per block)
constexpr int kBuildBuf = 24;  // buffered candidates per atom

// Entries of atom x that found its list full: counted per atom, so that the
// capacity the most crowded atom needed is known (max_sw + its extras).
__device__ __forceinline__ void list_spill(const DevParams& P, const DevState& S, int x, int n) {
  const int extra = atomicAdd(&S.sw_extra[x], n) + n;
  atomicAdd(&S.sc->overflow_sw, 1);
  atomicMax(&S.sc->sw_needed, P.max_sw + extra);
}

// A slot in atom x's list, or -1 (counted) when the list is full; the count
// ends at min(entries, max_sw) whatever the order of the atomics.
__device__ __forceinline__ int list_slot(const DevParams& P, const DevState& S, int x) {
  const int slot = atomicAdd(&S.n_sw[x], 1);
  if (slot < P.max_sw) return slot;
  atomicSub(&S.n_sw[x], 1);
  list_spill(P, S, x, 1);
  return -1;
}

// Spec mode: every pair with an ion inside the Moliere list radius (the
// radius exceeds the cell width, which the reference's 27-cell stencil does
// not cover). kIonSplit blocks share out each ion's (2R+1)^3 stencil cells,
// R = mol_reach; q is this block's index among nq such blocks. The ion
// stores an ion-atom pair in both orders; an ion-ion pair is stored once by
// each of its two ions.
constexpr int kIonSplit = 8;
__device__ __forceinline__ void ion_pairs(const DevParams& P, const DevState& S, int q, int nq) {
  for (int u = q; u < P.nion * kIonSplit; u += nq) {
    const int k = u / kIonSplit, part = u % kIonSplit;
    const int i = S.ion_list[k];
    const int4 qi = S.posq[i];
    const int ci0 = S.atom_cell[i];
    if ((qi.w & 0xff) != 3 || ci0 < 0) continue;
    const Geo& G = S.geo[rep_of_w(qi.w)];
    const int nx = G.nc[0], ny = G.nc[1], nz = G.nc[2];
    const int R = G.mol_reach, W = 2 * R + 1;
    const int ci = ci0 - G.cell_off;
    const int cx = ci % nx, cy = (ci / nx) % ny, cz = ci / (nx * ny);
    for (int s = part * blockDim.x + threadIdx.x; s < W * W * W; s += kIonSplit * blockDim.x) {
      const int ox = s % W, oy = (s / W) % W, oz = s / (W * W);
      int x = cx + ox - R, y = cy + oy - R, z = cz + oz - R;
      // a stencil wider than a periodic axis would visit a cell twice
      if (G.wrap[0]) { if (ox >= nx) continue; x = ((x % nx) + nx) % nx; }
      else if (x < 0 || x >= nx) continue;
      if (G.wrap[1]) { if (oy >= ny) continue; y = ((y % ny) + ny) % ny; }
      else if (y < 0 || y >= ny) continue;
      if (G.wrap[2]) { if (oz >= nz) continue; z = ((z % nz) + nz) % nz; }
      else if (z < 0 || z >= nz) continue;
      const int c = G.cell_off + x + nx * (y + ny * z);
      const int b = S.cell_start[c], e = S.cell_start[c + 1];
      for (int p = b; p < e; p++) {
        const int j = S.cell_atoms[p];
        if (j == i) continue;
        const int4 qj = S.posq[j];  // posq_cell holds ions shifted
        const float3 d = qsep(qi, qj, G.qinvA);
        const float r2f = d.x * d.x + d.y * d.y + d.z * d.z;
        if (r2f > P.pre_mol2A) continue;
        if (r2f >= P.acc_mol2A && !exact_in(G, S, i, j, P.rv2lj)) continue;
        const bool ion_j = (qj.w & 0xff) == 3;
        const int nw = ion_j ? 1 : 2;
        const int slot = atomicAdd(&S.sc->mol_count, nw);
        if (slot < P.mol_cap) S.mol_pairs[slot] = make_int2(i, j);
        if (!ion_j && slot + 1 < P.mol_cap) S.mol_pairs[slot + 1] = make_int2(j, i);
      }
    }
  }
}

// BT atoms per block (64, 128 or 256, chosen by the context's tuning); the
// resident threads per SM are the same for each (896)
template <bool WIDE, int BT>
__global__ void __launch_bounds__(BT, 896 / BT) k_build_atoms(DevParams P, DevState S,
                                                                   int from_flag) {
  if (rebuild_skipped(S, from_flag)) return;
  // spec mode: the blocks after the atoms' build the ion-pair (Moliere)
  // list at the same time
  const int nb_atoms = (P.N + BT - 1) / BT;
  if (WIDE && (int)blockIdx.x >= nb_atoms) {
    ion_pairs(P, S, (int)blockIdx.x - nb_atoms, (int)gridDim.x - nb_atoms);
    return;
  }
  __shared__ int buf[kBuildBuf][BT];     // candidate slots, then partners
  __shared__ float bufr[kBuildBuf][BT];  // their binary32 r^2 (A^2)
  const int t = threadIdx.x;
  const int h = blockIdx.x * BT + t;
  if (h >= S.cell_start[P.ncell]) return;
  const int i = S.cell_atoms[h];
  const int4 qi = S.posq_cell[h];
  // a replica that keeps its lists keeps its build positions too
  if (!rep_rebuilt(P, S, from_flag, rep_of_w(qi.w))) return;
  const int ti = qi.w & 0xff;
  const size_t stride = (size_t)P.N;
  int n = 0;  // buffered candidates, then accepted SW partners
  if (!(WIDE && ti == 3)) {
    const Geo& G = S.geo[rep_of_w(qi.w)];
    const int c = S.atom_cell[i] - G.cell_off;
    const int nx = G.nc[0], ny = G.nc[1], nz = G.nc[2];
    const int cx = c % nx, cy = (c / nx) % ny, cz = c / (nx * ny);
    const float qinvA[3] = {G.qinvA[0], G.qinvA[1], G.qinvA[2]};
    // inclusive x ranges of a full stencil row (periodic only with > 2 cells)
    int xa0, xa1, xb0 = 0, xb1 = -1;
    if (G.wrap[0]) {
      if (cx == 0) {
        xa0 = 0; xa1 = 1; xb0 = xb1 = nx - 1;
      } else if (cx == nx - 1) {
        xa0 = nx - 2; xa1 = nx - 1; xb0 = xb1 = 0;
      } else {
        xa0 = cx - 1; xa1 = cx + 1;
      }
    } else {
      xa0 = max(cx - 1, 0);
      xa1 = min(cx + 1, nx - 1);
    }
    // binary32 bound of any listed pair of this atom
    const float thr = WIDE ? P.pre_sw2A : fmaxf(P.pre_sw2A, P.pre_mol2A);
    const int4* __restrict__ qc = S.posq_cell;
    // The buffered candidates: the exact test where the prefilter is not
    // conclusive, Moliere pairs (reference mode) to their list, accepted SW
    // partners compacted to the front of buf as atom indices (direct:
    // entered at once instead). Returns the number compacted.
    auto resolve = [&](int nc, bool direct) -> int {
      int na = 0;
      for (int k = 0; k < nc; k++) {
        const int p = buf[k][t];
        const float r2f = bufr[k][t];
        const int j = __ldg(&S.cell_atoms[p]);
        bool sw = true;
        if (!WIDE) {
          const int tj = __ldg(&qc[p].w) & 0xff;
          sw = (ti > tj ? ti : tj) < 3;
          if (sw && r2f > P.pre_sw2A) continue;
        }
        if (r2f >= (sw ? P.acc_sw2A : P.acc_mol2A) && !exact_in(G, S, i, j, sw ? P.rv2 : P.rv2lj))
          continue;
        if (!sw) {
          const int slot = atomicAdd(&S.sc->mol_count, 2);
          if (slot < P.mol_cap) S.mol_pairs[slot] = make_int2(i, j);
          if (slot + 1 < P.mol_cap) S.mol_pairs[slot + 1] = make_int2(j, i);
        } else if (direct) {
          const int si = list_slot(P, S, i);
          if (si >= 0) S.nbr_sw[(size_t)si * stride + i] = j;
          const int sj = list_slot(P, S, j);
          if (sj >= 0) S.nbr_sw[(size_t)sj * stride + j] = i;
          if (S.rev_sw) {
            if (si >= 0) S.rev_sw[(size_t)si * stride + i] = sj;
            if (sj >= 0) S.rev_sw[(size_t)sj * stride + j] = si;
          }
        } else {
          buf[na][t] = j;
          na++;
        }
      }
      return na;
    };
    // candidate runs: [b, e) of the cell-sorted arrays. Candidates inside
    // the prefilter are buffered by predicated stores, so the lanes of a
    // warp stay converged through the scan (about one candidate in eight
    // passes it); a nearly full buffer is resolved at once.
    auto scan = [&](int b, int e) {
      for (int p0 = b; p0 < e; p0 += 4) {
        int4 qq[4];
#pragma unroll
        for (int u = 0; u < 4; u++) qq[u] = __ldg(&qc[min(p0 + u, e - 1)]);
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const float3 d = qsep(qi, qq[u], qinvA);
          const float r2f = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
          const bool in = r2f <= thr && p0 + u < e;
          if (in) {
            buf[n][t] = p0 + u;
            bufr[n][t] = r2f;
          }
          n += in;
        }
        if (n > kBuildBuf - 4) {  // room for the next four
          resolve(n, true);
          n = 0;
        }
      }
    };
    const int rowc = G.cell_off + nx * (cy + ny * cz);
    // own row: the atoms after this one in its cell and the cell at x + 1
    if (G.wrap[0] && cx == nx - 1) {
      scan(h + 1, S.cell_start[rowc + nx]);
      scan(S.cell_start[rowc], S.cell_start[rowc + 1]);
    } else {
      const int xe = min(cx + 1, nx - 1);
      scan(h + 1, S.cell_start[rowc + xe + 1]);
    }
    // forward rows: (dy, dz) = (+1, 0) and (-1..+1, +1)
    for (int r = 0; r < 4; r++) {
      const int dy = r == 0 ? 1 : r - 2, dz = r == 0 ? 0 : 1;
      int z = cz + dz;
      if (G.wrap[2]) z = z >= nz ? z - nz : z;
      else if (z >= nz) continue;
      int y = cy + dy;
      if (G.wrap[1]) y = y < 0 ? y + ny : (y >= ny ? y - ny : y);
      else if (y < 0 || y >= ny) continue;
      const int row = G.cell_off + nx * (y + ny * z);
      scan(S.cell_start[row + xa0], S.cell_start[row + xa1 + 1]);
      if (xb1 >= xb0) scan(S.cell_start[row + xb0], S.cell_start[row + xb1 + 1]);
    }
    n = resolve(n, false);
  }
  // enter the accepted partners: the centre's entries in one reservation,
  // then the partners' (independent atomics, several in flight)
  const int nb = n;
  if (nb > 0) {
    int base = atomicAdd(&S.n_sw[i], nb);
    int keep = min(nb, max(0, P.max_sw - base));
    if (keep < nb) {
      atomicSub(&S.n_sw[i], nb - keep);
      list_spill(P, S, i, nb - keep);
    }
    for (int k = 0; k < nb; k++) {
      const int j = buf[k][t];
      if (k < keep) S.nbr_sw[(size_t)(base + k) * stride + i] = j;
      const int sj = list_slot(P, S, j);
      if (sj >= 0) S.nbr_sw[(size_t)sj * stride + j] = i;
      // each entry's slot in the partner's list (-1 where a list overflowed)
      if (S.rev_sw) {
        if (k < keep) S.rev_sw[(size_t)(base + k) * stride + i] = sj;
        if (sj >= 0) S.rev_sw[(size_t)sj * stride + j] = k < keep ? base + k : -1;
      }
    }
  }
  S.posq_build[i] = (WIDE && ti == 3) ? S.posq[i] : qi;
  S.fast_flag[i] = 0;
}

__global__ void k_build_end(DevParams P, DevState S, int from_flag) {
  if (rebuild_skipped(S, from_flag)) return;
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    if (S.sc->mol_count > P.mol_cap) S.sc->overflow_mol = S.sc->mol_count;
    // the replicas' flags (read by the kernels above), then the context's
    for (int r = 1; r < P.nrep; r++) {
      S.sc[r].rep_rebuild = 0;
      S.sc[r].rep_soon = 0;
    }
    S.sc->rep_rebuild = 0;
    S.sc->rep_soon = 0;
    S.sc->need_rebuild = 0;
    S.sc->rebuild_all = 0;
    S.sc->rebuilds++;
  }
}

cudaError_t launch_build_lists(const Launch& L, const DevParams& P, const DevState& S,
                               int from_flag) {
  int nb_atoms = (P.N + 255) / 256;
  int ncell1 = P.ncell + 1;
  int nb_cells = (ncell1 + 255) / 256;
  int nscan = (ncell1 + kScanBlock - 1) / kScanBlock;
  k_build_begin<<<nb_cells, 256, 0, L.stream>>>(P, S, from_flag);
  k_cell_assign<<<nb_atoms, 256, 0, L.stream>>>(P, S, from_flag);
  k_scan_local<<<nscan, kScanBlock, 0, L.stream>>>(P, S, from_flag);
  k_scan_top<<<1, kScanBlock, 0, L.stream>>>(P, S, nscan, from_flag);
  k_scan_add<<<nscan, kScanBlock, 0, L.stream>>>(P, S, from_flag);
  k_cell_fill<<<nb_atoms, 256, 0, L.stream>>>(P, S, from_flag);
  const int bt = (L.build_block == 64 || L.build_block == 256) ? L.build_block : kBuildThreads;
  const bool wide = P.mol_reach > 1;
  // with the spec-mode ion-pair blocks after the atoms'
  const int nb_build =
      (P.N + bt - 1) / bt + (wide && P.nion > 0 ? min(P.nion * kIonSplit, 4096) : 0);
  if (bt == 64) {
    if (wide) k_build_atoms<true, 64><<<nb_build, 64, 0, L.stream>>>(P, S, from_flag);
    else k_build_atoms<false, 64><<<nb_build, 64, 0, L.stream>>>(P, S, from_flag);
  } else if (bt == 256) {
    if (wide) k_build_atoms<true, 256><<<nb_build, 256, 0, L.stream>>>(P, S, from_flag);
    else k_build_atoms<false, 256><<<nb_build, 256, 0, L.stream>>>(P, S, from_flag);
  } else {
    if (wide) k_build_atoms<true, 128><<<nb_build, 128, 0, L.stream>>>(P, S, from_flag);
    else k_build_atoms<false, 128><<<nb_build, 128, 0, L.stream>>>(P, S, from_flag);
  }
  k_build_end<<<1, 32, 0, L.stream>>>(P, S, from_flag);
  return cudaGetLastError();
}

// ---- connected triplets (si_nlistG triplet rules, si.f90:191-232) ----------
// For centre i (the smallest index of the triple): every unordered pair
// {j,k} of listed neighbours above i, and every j above i with a neighbour
// k above i that is not itself a neighbour of i. Each connected triple of
// the symmetric list graph is produced once, as the reference stores it.
__global__ void k_triplets(DevParams P, DevState S, unsigned long long* count, int3* out,
                           long long cap) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.N) return;
  int ni = S.n_sw[i];
  unsigned long long local = 0;
  for (int a = 0; a < ni; a++) {
    int j = S.nbr_sw[(size_t)a * P.N + i];
    if (j <= i) continue;
    for (int b = a + 1; b < ni; b++) {
      int k = S.nbr_sw[(size_t)b * P.N + i];
      if (k <= i) continue;
      if (out) {
        unsigned long long s = atomicAdd(count, 1ull);
        if ((long long)s < cap) out[s] = make_int3(i, min(j, k), max(j, k));
      } else {
        local++;
      }
    }
    int nj = S.n_sw[j];
    for (int m = 0; m < nj; m++) {
      int k = S.nbr_sw[(size_t)m * P.N + j];
      if (k <= i) continue;
      bool found = false;
      for (int q = 0; q < ni; q++)
        if (S.nbr_sw[(size_t)q * P.N + i] == k) {
          found = true;
          break;
        }
      if (found) continue;
      if (out) {
        unsigned long long s = atomicAdd(count, 1ull);
        if ((long long)s < cap) out[s] = make_int3(i, min(j, k), max(j, k));
      } else {
        local++;
      }
    }
  }
  if (!out && local) atomicAdd(count, local);
}

cudaError_t launch_count_triplets(const Launch& L, const DevParams& P, const DevState& S,
                                  unsigned long long* d_count, int3* out, long long cap) {
  k_triplets<<<(P.N + 127) / 128, 128, 0, L.stream>>>(P, S, d_count, out, cap);
  return cudaGetLastError();
}

}  // namespace fibmd
