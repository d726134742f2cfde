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
  }
}

// atomcell (nlist.f90:28-30): Icell = INT((X - FLOOR(X*iLb)*Lb)/h) + 1.
__global__ void k_cell_assign(DevParams P, DevState S, int from_flag) {
  if (rebuild_skipped(S, from_flag)) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.N) return;
  if (S.flags[i] & FL_REMOVED) {
    S.atom_cell[i] = -1;
    return;
  }
  double4_32a p = S.pos[i];
  double x[3] = {p.x, p.y, p.z};
  int ic[3];
  bool oob = false;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    double fl = floor(__dmul_rn(x[d], P.iLb[d]));
    double t = __ddiv_rn(__dsub_rn(x[d], __dmul_rn(fl, P.Lb[d])), P.hcell[d]);
    int c = (int)t;  // 0-based (the reference adds 1)
    if (c < 0 || c >= P.nc[d]) {
      oob = true;
      c = c < 0 ? 0 : P.nc[d] - 1;
    }
    ic[d] = c;
  }
  if (oob) atomicAdd(&S.sc->cell_oob, 1);
  int cell = ic[0] + P.nc[0] * (ic[1] + P.nc[1] * ic[2]);
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
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.N) return;
  int c = S.atom_cell[i];
  if (c < 0) return;
  int slot = S.cell_start[c] + atomicAdd(&S.cell_count[c], 1);
  S.cell_atoms[slot] = i;
}

// Order each cell's members by atom index so list order (and so the force
// summation order) does not depend on atomic scheduling.
__global__ void k_cell_order(DevParams P, DevState S, int from_flag) {
  if (rebuild_skipped(S, from_flag)) return;
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= P.ncell) return;
  int b = S.cell_start[c], e = S.cell_start[c + 1];
  for (int a = b + 1; a < e; a++) {
    int v = S.cell_atoms[a];
    int q = a - 1;
    while (q >= b && S.cell_atoms[q] > v) {
      S.cell_atoms[q + 1] = S.cell_atoms[q];
      q--;
    }
    S.cell_atoms[q + 1] = v;
  }
}

// ---- pair lists (si_nlistG pair loop, si.f90:130-189) ---------------------
__global__ void __launch_bounds__(128) k_build_pairs(DevParams P, DevState S, int from_flag) {
  if (rebuild_skipped(S, from_flag)) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.N) return;
  int ci = S.atom_cell[i];
  S.pos_build[i] = S.pos[i];
  S.fast_flag[i] = 0;
  if (ci < 0) {
    S.n_sw[i] = 0;
    return;
  }
  const int4 qi = S.posq[i];
  const double4_32a pi = S.pos[i];
  const int ti = (int)S.atype[i];
  int cx = ci % P.nc[0];
  int cy = (ci / P.nc[0]) % P.nc[1];
  int cz = ci / (P.nc[0] * P.nc[1]);
  int n = 0;
  for (int dz = -1; dz <= 1; dz++) {
    int z = cz + dz;
    if (P.nc[2] > 2) z = (z + P.nc[2]) % P.nc[2];
    else if (z < 0 || z >= P.nc[2]) continue;
    for (int dy = -1; dy <= 1; dy++) {
      int y = cy + dy;
      if (P.nc[1] > 2) y = (y + P.nc[1]) % P.nc[1];
      else if (y < 0 || y >= P.nc[1]) continue;
      for (int dx = -1; dx <= 1; dx++) {
        int x = cx + dx;
        if (P.nc[0] > 2) x = (x + P.nc[0]) % P.nc[0];
        else if (x < 0 || x >= P.nc[0]) continue;
        int c2 = x + P.nc[0] * (y + P.nc[1] * z);
        int b = S.cell_start[c2], e = S.cell_start[c2 + 1];
        for (int p = b; p < e; p++) {
          int j = S.cell_atoms[p];
          if (j == i) continue;
          int4 qj = S.posq[j];
          int tj = qj.w & 0xff;
          float3 d = qsep(qi, qj, P.qinvA);
          float r2f = d.x * d.x + d.y * d.y + d.z * d.z;
          bool sw = (ti > tj ? ti : tj) < 3;
          float pre = sw ? P.pre_sw2A : P.pre_mol2A;
          if (r2f > pre) continue;
          bool in;
          if (r2f < (sw ? P.acc_sw2A : P.acc_mol2A)) {
            in = true;
          } else {
            double4_32a pj = S.pos[j];
            double xx = min_image_exact(pi.x, pj.x, P.iLb[0], P.Lb[0]);
            double yy = min_image_exact(pi.y, pj.y, P.iLb[1], P.Lb[1]);
            double zz = min_image_exact(pi.z, pj.z, P.iLb[2], P.Lb[2]);
            double r2 = __dadd_rn(__dadd_rn(__dmul_rn(xx, xx), __dmul_rn(yy, yy)),
                                  __dmul_rn(zz, zz));
            in = r2 < (sw ? P.rv2 : P.rv2lj);
          }
          if (!in) continue;
          if (sw) {
            if (n < P.max_sw) S.nbr_sw[(size_t)n * P.N + i] = j;
            n++;
          } else {
            int slot = atomicAdd(&S.sc->mol_count, 1);
            if (slot < P.mol_cap) S.mol_pairs[slot] = make_int2(i, j);
          }
        }
      }
    }
  }
  if (n > P.max_sw) {
    atomicAdd(&S.sc->overflow_sw, 1);
    n = P.max_sw;
  }
  S.n_sw[i] = n;
}

__global__ void k_build_end(DevParams P, DevState S, int from_flag) {
  if (rebuild_skipped(S, from_flag)) return;
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    if (S.sc->mol_count > P.mol_cap) S.sc->overflow_mol = S.sc->mol_count;
    S.sc->need_rebuild = 0;
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
  k_cell_order<<<(P.ncell + 255) / 256, 256, 0, L.stream>>>(P, S, from_flag);
  k_build_pairs<<<(P.N + 127) / 128, 128, 0, L.stream>>>(P, S, from_flag);
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
