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
  int4 q;
  q.x = (int)fixq(p.x, P.qscale[0]);
  q.y = (int)fixq(p.y, P.qscale[1]);
  q.z = (int)fixq(p.z, P.qscale[2]);
  q.w = (int)(uint8_t)S.atype[i] | (int)(S.flags[i] << 8);
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

__global__ void k_build_begin(DevParams P, DevState S, int from_flag) {
  if (rebuild_skipped(S, from_flag)) return;
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < P.ncell + 1) S.cell_count[c] = 0;
  if (c == 0) {
    S.sc->mol_count = 0;
    S.sc->fast_count = 0;
    S.sc->overflow_sw = 0;
    S.sc->overflow_mol = 0;
    S.sc->cell_oob = 0;
    S.sc->disp_max2 = 0.0;
    S.sc->nonempty_count = 0;
  }
}

// atomcell (nlist.f90:28-30): Icell = INT((X - FLOOR(X*iLb)*Lb)/h) + 1.
// The cell along an axis is floor(x nc / Lb), which the fixed-point shadow
// q = round(x 2^32 / Lb) gives as (q nc) >> 32 with integer arithmetic. The
// two agree except within ~nc 2^-33 of a cell boundary; there (fraction
// within 1e-6 of a boundary) the reference's binary64 formula decides, so
// the cell of every atom is the reference's.
__device__ __forceinline__ int ref_cell(const DevParams& P, double x, int d) {
  const double fl = floor(__dmul_rn(x, P.iLb[d]));
  const double t = __ddiv_rn(__dsub_rn(x, __dmul_rn(fl, P.Lb[d])), P.hcell[d]);
  return (int)t;
}

__global__ void k_cell_assign(DevParams P, DevState S, int from_flag) {
  if (rebuild_skipped(S, from_flag)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.N) return;
  const int4 q = S.posq[i];
  if ((q.w >> 8) & FL_REMOVED) {
    S.atom_cell[i] = -1;
    S.n_sw[i] = 0;
    S.posq_build[i] = q;
    S.fast_flag[i] = 0;
    return;
  }
  const unsigned qq[3] = {(unsigned)q.x, (unsigned)q.y, (unsigned)q.z};
  constexpr unsigned kGuard = 4295u;  // 1e-6 of a cell, in units of 2^-32
  int ic[3];
  bool oob = false;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const unsigned long long t = (unsigned long long)qq[d] * (unsigned long long)P.nc[d];
    int c = (int)(t >> 32);
    const unsigned frac = (unsigned)t;
    if (d == 2 && P.zcompact) {
      // spec mode with an open z axis: the grid covers [0, remove_z + rc);
      // an atom above it (an ion: other atoms there are removed) joins the
      // top layer and an atom below z = 0 the bottom one, which hold every
      // atom within rc of it
      const double zc = S.pos[i].z * P.inv_hz;
      c = zc < 0.0 ? 0 : (zc >= (double)P.nc[2] ? P.nc[2] - 1 : (int)zc);
    } else if (frac < kGuard || frac > 0xffffffffu - kGuard) {
      const double4_32a p = S.pos[i];
      c = ref_cell(P, d == 0 ? p.x : d == 1 ? p.y : p.z, d);
    }
    if (c < 0 || c >= P.nc[d]) {
      oob = true;
      c = c < 0 ? 0 : P.nc[d] - 1;
    }
    ic[d] = c;
  }
  if (oob) atomicAdd(&S.sc->cell_oob, 1);
  const int cell = ic[0] + P.nc[0] * (ic[1] + P.nc[1] * ic[2]);
  S.atom_cell[i] = cell;
  if (atomicAdd(&S.cell_count[cell], 1) == 0) S.nonempty[atomicAdd(&S.sc->nonempty_count, 1)] = cell;
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
  S.posq_cell[slot] = S.posq[i];
}

// ---- pair lists (si_nlistG pair loop, si.f90:130-189) ---------------------
// One warp per non-empty cell. The warp stages the candidates of the
// 27-cell stencil (9 rows of three x-adjacent cells, each row one
// contiguous range of the cell-sorted arrays when it does not wrap) in
// shared memory with coalesced loads, then tests every home atom of the
// cell against them, 32 candidates at a time; accepted SW neighbours are
// compacted into the home atom's list slots with a ballot and prefix count.
constexpr int kBuildWarps = 4;
constexpr int kCand = 256;   // staged candidates per warp (flushed when full)
constexpr int kHome = 64;    // home atoms handled per pass over the stencil

struct BuildStage {
  int4 q[kBuildWarps][kCand];
  int j[kBuildWarps][kCand];
  int n[kBuildWarps][kHome];
};

__device__ __forceinline__ bool pair_in_list(const DevParams& P, const DevState& S, int i,
                                             const int4& qi, int j, const int4& qj, bool* sw) {
  const int ti = qi.w & 0xff, tj = qj.w & 0xff;
  *sw = (ti > tj ? ti : tj) < 3;
  if (j == i) return false;
  if (!*sw && P.mol_reach > 1) return false;  // k_build_ion_pairs lists these
  const float3 d = qsep(qi, qj, P.qinvA);
  const float r2f = d.x * d.x + d.y * d.y + d.z * d.z;
  if (r2f > (*sw ? P.pre_sw2A : P.pre_mol2A)) return false;
  if (r2f < (*sw ? P.acc_sw2A : P.acc_mol2A)) return true;
  // within 1e-4 of the radius: the reference's binary64 test decides
  const double4_32a pi = S.pos[i], pj = S.pos[j];
  const double xx = min_image_exact(pi.x, pj.x, P.iLb[0], P.Lb[0]);
  const double yy = min_image_exact(pi.y, pj.y, P.iLb[1], P.Lb[1]);
  const double zz = min_image_exact(pi.z, pj.z, P.iLb[2], P.Lb[2]);
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(xx, xx), __dmul_rn(yy, yy)), __dmul_rn(zz, zz));
  return r2 < (*sw ? P.rv2 : P.rv2lj);
}

// Tests home atoms [h0, h1) against the K staged candidates.
__device__ __forceinline__ void test_staged(const DevParams& P, const DevState& S,
                                            BuildStage& st, int w, int lane, int h0, int h1,
                                            int K) {
  for (int h = h0; h < h1; h++) {
    const int i = S.cell_atoms[h];
    const int4 qi = S.posq_cell[h];
    int n = st.n[w][h - h0];
    for (int k0 = 0; k0 < K; k0 += 32) {
      const int k = k0 + lane;
      bool sw = true, in = false;
      int j = -1;
      if (k < K) {
        j = st.j[w][k];
        in = pair_in_list(P, S, i, qi, j, st.q[w][k], &sw);
      }
      const unsigned m = __ballot_sync(0xffffffffu, in && sw);
      if (in && sw) {
        const int slot = n + __popc(m & ((1u << lane) - 1u));
        if (slot < P.max_sw) S.nbr_sw[(size_t)slot * P.N + i] = j;
      } else if (in) {
        const int slot = atomicAdd(&S.sc->mol_count, 1);
        if (slot < P.mol_cap) S.mol_pairs[slot] = make_int2(i, j);
      }
      n += __popc(m);
    }
    if (lane == 0) st.n[w][h - h0] = n;
  }
  __syncwarp();
}

__global__ void __launch_bounds__(32 * kBuildWarps) k_build_cells(DevParams P, DevState S,
                                                                  int from_flag) {
  if (rebuild_skipped(S, from_flag)) return;
  __shared__ BuildStage st;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ncells = ((volatile DevScalars*)S.sc)->nonempty_count;
  const int nx = P.nc[0], ny = P.nc[1], nz = P.nc[2];
  // lane s < 27 owns stencil cell (dx, dy, dz) = (s%3, s/3%3, s/9) - 1
  const int sdx = lane % 3 - 1, sdy = (lane / 3) % 3 - 1, sdz = lane / 9 - 1;
  for (int wc = blockIdx.x * kBuildWarps + w; wc < ncells; wc += gridDim.x * kBuildWarps) {
    const int c = S.nonempty[wc];
    const int hb = S.cell_start[c], he = S.cell_start[c + 1];
    const int cx = c % nx, cy = (c / nx) % ny, cz = c / (nx * ny);
    // this lane's stencil cell and its atom range (periodic wrap only on
    // axes with more than two cells, as the reference's ghost layers)
    int b = 0, e = 0;
    if (lane < 27) {
      int x = cx + sdx, y = cy + sdy, z = cz + sdz;
      bool ok = true;
      if (P.wrap[0]) x = (x + nx) % nx; else ok &= (x >= 0 && x < nx);
      if (P.wrap[1]) y = (y + ny) % ny; else ok &= (y >= 0 && y < ny);
      if (P.wrap[2]) z = (z + nz) % nz; else ok &= (z >= 0 && z < nz);
      if (ok) {
        const int cc = x + nx * (y + ny * z);
        b = S.cell_start[cc];
        e = S.cell_start[cc + 1];
      }
    }
    const int cnt = e - b;
    int off = cnt;  // inclusive warp scan of the counts
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, off, o);
      if (lane >= o) off += t;
    }
    const int total = __shfl_sync(0xffffffffu, off, 31);
    off -= cnt;  // exclusive
    for (int h0 = hb; h0 < he; h0 += kHome) {
      const int h1 = min(he, h0 + kHome);
      for (int h = h0 + lane; h < h1; h += 32) st.n[w][h - h0] = 0;
      // stage the candidates in chunks of kCand; each lane copies its cell
      for (int base = 0; base < total; base += kCand) {
        __syncwarp();
        const int lo = max(off, base), hi = min(off + cnt, base + kCand);
        for (int k = lo; k < hi; k++) {
          st.q[w][k - base] = S.posq_cell[b + (k - off)];
          st.j[w][k - base] = S.cell_atoms[b + (k - off)];
        }
        __syncwarp();
        test_staged(P, S, st, w, lane, h0, h1, min(kCand, total - base));
      }
      for (int h = h0 + lane; h < h1; h += 32) {
        const int i = S.cell_atoms[h];
        int n = st.n[w][h - h0];
        if (n > P.max_sw) {
          atomicAdd(&S.sc->overflow_sw, 1);
          n = P.max_sw;
        }
        S.n_sw[i] = n;
        S.posq_build[i] = S.posq_cell[h];
        S.fast_flag[i] = 0;
      }
      __syncwarp();
    }
  }
}

// Spec mode: every pair with an ion inside the Moliere list radius. One
// warp per ion scans the cells within mol_reach (the radius exceeds the
// cell width, which the reference's 27-cell stencil does not cover). The
// ion stores an ion-atom pair in both orders; an ion-ion pair is stored
// once by each of its two ions.
__global__ void __launch_bounds__(128) k_build_ion_pairs(DevParams P, DevState S,
                                                         int from_flag) {
  if (rebuild_skipped(S, from_flag)) return;
  const int lane = threadIdx.x & 31;
  const int nion = P.N - P.Nsg;
  const int nx = P.nc[0], ny = P.nc[1], nz = P.nc[2];
  const int R = P.mol_reach, W = 2 * R + 1;
  for (int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < nion;
       k += (gridDim.x * blockDim.x) >> 5) {
    const int i = P.Nsg + k;
    const int4 qi = S.posq[i];
    const int ci = S.atom_cell[i];
    if ((qi.w & 0xff) != 3 || ci < 0) continue;
    const int cx = ci % nx, cy = (ci / nx) % ny, cz = ci / (nx * ny);
    for (int s = lane; s < W * W * W; s += 32) {
      int x = cx + s % W - R, y = cy + (s / W) % W - R, z = cz + s / (W * W) - R;
      // a stencil wider than an axis would visit a cell twice: skip repeats
      if (P.wrap[0]) { if (W > nx && (s % W) >= nx) continue; x = ((x % nx) + nx) % nx; }
      else if (x < 0 || x >= nx) continue;
      if (P.wrap[1]) { if (W > ny && ((s / W) % W) >= ny) continue; y = ((y % ny) + ny) % ny; }
      else if (y < 0 || y >= ny) continue;
      if (P.wrap[2]) { if (W > nz && (s / (W * W)) >= nz) continue; z = ((z % nz) + nz) % nz; }
      else if (z < 0 || z >= nz) continue;
      const int c = x + nx * (y + ny * z);
      const int b = S.cell_start[c], e = S.cell_start[c + 1];
      for (int p = b; p < e; p++) {
        const int j = S.cell_atoms[p];
        if (j == i) continue;
        const int4 qj = S.posq_cell[p];
        const bool ion_j = (qj.w & 0xff) == 3;
        const float3 d = qsep(qi, qj, P.qinvA);
        const float r2f = d.x * d.x + d.y * d.y + d.z * d.z;
        if (r2f > P.pre_mol2A) continue;
        bool in = r2f < P.acc_mol2A;
        if (!in) {
          const double4_32a pi = S.pos[i], pj = S.pos[j];
          const double xx = min_image_exact(pi.x, pj.x, P.iLb[0], P.Lb[0]);
          const double yy = min_image_exact(pi.y, pj.y, P.iLb[1], P.Lb[1]);
          const double zz = min_image_exact(pi.z, pj.z, P.iLb[2], P.Lb[2]);
          const double r2 =
              __dadd_rn(__dadd_rn(__dmul_rn(xx, xx), __dmul_rn(yy, yy)), __dmul_rn(zz, zz));
          in = r2 < P.rv2lj;
        }
        if (!in) continue;
        const int nw = ion_j ? 1 : 2;
        const int slot = atomicAdd(&S.sc->mol_count, nw);
        if (slot < P.mol_cap) S.mol_pairs[slot] = make_int2(i, j);
        if (!ion_j && slot + 1 < P.mol_cap) S.mol_pairs[slot + 1] = make_int2(j, i);
      }
    }
  }
}

__global__ void k_build_end(DevParams P, DevState S, int from_flag) {
  if (rebuild_skipped(S, from_flag)) return;
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    if (S.sc->mol_count > P.mol_cap) S.sc->overflow_mol = S.sc->mol_count;
    S.sc->need_rebuild = 0;
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
  const int side = L.sms > 0 ? L.sms : 152;
  k_build_cells<<<side * 16, 32 * kBuildWarps, 0, L.stream>>>(P, S, from_flag);
  if (P.mol_reach > 1 && P.N > P.Nsg)
    k_build_ion_pairs<<<(P.N - P.Nsg + 3) / 4, 128, 0, L.stream>>>(P, S, from_flag);
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
