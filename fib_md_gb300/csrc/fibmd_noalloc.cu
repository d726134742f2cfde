// fibmd_noalloc.cu — a force entry point that allocates nothing.
//
// Some hosts cannot ask the driver for device memory at the moment they need
// a force: a host whose device memory is handed out by a pool manager or an
// embedding runtime that forbids driver allocations after start-up, or a
// Fortran/C driver that must keep a fixed device footprint on a shared GPU.
// For them, fibmd_gpu_force_noalloc evaluates si_force (binary64, the
// reference's semantics: cell binning, Verlet lists, table SW 2-body, Moliere
// for fired ions, SW 3-body) for one configuration held in the caller's
// device buffers, with every piece of scratch memory (cells, lists, position
// shadows, reduction scalars, the 2-body table) carved out of one file-scope
// device array of fixed size.
//
// Limits: at most kNaAtoms atoms, kNaCells cells of the reference's cell
// grid, Ntable <= kNaTable, max_sw_nbrs <= kNaMaxSw, kNaMolPairs Moliere list
// entries. The array (4.2 MB) stays resident on every device that loads the
// library until the process exits. Every call shares it and finds the
// previous call's contents there; calls that overlap on the GPU race.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "fibmd_internal.cuh"

namespace fibmd {
namespace {

constexpr int kNaAtoms = 8192;
constexpr int kNaCells = 1 << 16;
constexpr int kNaTable = 12000;
constexpr int kNaMaxSw = 48;
constexpr int kNaMolPairs = 1 << 16;

constexpr size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// byte offsets of the sub-arrays inside the scratch array
struct Layout {
  size_t pos, frc_new, posq, posq_build, posq_cell, atype, flags, cell_count, cell_start,
      cell_atoms, atom_cell, scan_blocks, nbr_sw, n_sw, sw_extra, mol_pairs, fast_flag,
      fast_list, heavy_list, tab, tabu, partials, sc, geo, ion_list, total;
};

constexpr Layout make_layout() {
  Layout L{};
  size_t o = 0;
  const size_t N = kNaAtoms, C = kNaCells + 1;
  L.pos = o; o += align256(sizeof(double4_32a) * N);
  L.frc_new = o; o += align256(sizeof(double4_32a) * N);
  L.posq = o; o += align256(sizeof(int4) * N);
  L.posq_build = o; o += align256(sizeof(int4) * N);
  L.posq_cell = o; o += align256(sizeof(int4) * N);
  L.atype = o; o += align256(sizeof(int8_t) * N);
  L.flags = o; o += align256(sizeof(uint32_t) * N);
  L.cell_count = o; o += align256(sizeof(int) * C);
  L.cell_start = o; o += align256(sizeof(int) * C);
  L.cell_atoms = o; o += align256(sizeof(int) * N);
  L.atom_cell = o; o += align256(sizeof(int) * N);
  L.scan_blocks = o; o += align256(sizeof(int) * (C / 1024 + 2));
  L.nbr_sw = o; o += align256(sizeof(int) * (size_t)kNaMaxSw * N);
  L.n_sw = o; o += align256(sizeof(int) * N);
  L.sw_extra = o; o += align256(sizeof(int) * N);
  L.mol_pairs = o; o += align256(sizeof(int2) * kNaMolPairs);
  L.fast_flag = o; o += align256(sizeof(uint8_t) * N);
  L.fast_list = o; o += align256(sizeof(int) * N);
  L.heavy_list = o; o += align256(sizeof(int) * N);
  L.tab = o; o += align256(sizeof(double) * (kNaTable + 2));
  L.tabu = o; o += align256(sizeof(double) * (kNaTable + 2));
  L.partials = o; o += align256(sizeof(double) * 3 * kMaxRedBlocks);
  L.sc = o; o += align256(sizeof(DevScalars));
  L.geo = o; o += align256(sizeof(Geo));
  L.ion_list = o; o += align256(sizeof(int) * N);
  L.total = o;
  return L;
}

constexpr Layout kLayout = make_layout();

// The scratch memory of every call. In host code this name is only a handle
// for cudaGetSymbolAddress, never a device address.
__device__ __align__(256) unsigned char g_noalloc_scratch[kLayout.total];

// Per-device set-up: the array's device address, the parameters of the
// 2-body table currently loaded into it, and that table's extent (umax and
// the last non-zero entry). The key, the device table and the extent change
// together, inside one critical section, so they always describe the same
// table.
struct DeviceSlot {
  bool ready = false;
  unsigned char* base = nullptr;
  bool table_loaded = false;
  double tab_key[7] = {};
  double umax = 0.0;
  int tab_last = 0;
};
constexpr int kMaxDevices = 64;
DeviceSlot g_slots[kMaxDevices];
std::mutex g_slots_mutex;

// host staging of the table, reused by every call (no heap)
double g_tab_host[kNaTable + 2];
double g_tabu_host[kNaTable + 2];

__global__ void k_na_import(int N, int Nsg, const double* __restrict__ X,
                            const int* __restrict__ atype, DevState S, int* ion_list,
                            int* bad_type) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  if (i >= Nsg) ion_list[i - Nsg] = i;
  S.pos[i] = make_double4_32a(X[i], X[(size_t)N + i], X[2 * (size_t)N + i], 0.0);
  const int t = atype[i];
  if (t < 1 || t > 3) atomicExch(bad_type, 1);
  S.atype[i] = (int8_t)(t < 1 ? 1 : (t > 3 ? 3 : t));
  S.flags[i] = 0u;
}

int fail_na(int code, const char* msg) {
  set_noctx_error(msg);
  return code;
}

}  // namespace
}  // namespace fibmd

using namespace fibmd;

extern "C" int fibmd_gpu_force_noalloc(const fibmd_params* p, const double* X_dev,
                                       const int* atype_dev, int impact, double* F_dev,
                                       void* stream) {
  char msg[256];
  if (!p || !X_dev || !atype_dev || !F_dev || impact < 0)
    return fail_na(FIBMD_EINVAL, "force_noalloc: null argument or negative impact");
  if (p->abi_version != FIBMD_ABI_VERSION)
    return fail_na(FIBMD_EINVAL, "force_noalloc: abi_version mismatch");
  if (p->Natm <= 0 || p->Natm > kNaAtoms) {
    std::snprintf(msg, sizeof msg, "force_noalloc: %d atoms, the limit is %d", p->Natm, kNaAtoms);
    return fail_na(FIBMD_EINVAL, msg);
  }
  if (p->Ntable < 8 || p->Ntable > kNaTable) {
    std::snprintf(msg, sizeof msg, "force_noalloc: Ntable %d, the limit is %d", p->Ntable,
                  kNaTable);
    return fail_na(FIBMD_EINVAL, msg);
  }
  if (p->max_sw_nbrs > kNaMaxSw) {
    std::snprintf(msg, sizeof msg, "force_noalloc: max_sw_nbrs %d, the limit is %d",
                  p->max_sw_nbrs, kNaMaxSw);
    return fail_na(FIBMD_EINVAL, msg);
  }
  if (p->precision != FIBMD_PREC_FP64)
    return fail_na(FIBMD_EINVAL, "force_noalloc: binary64 only (precision must be FP64)");
  if (p->max_mol_pairs > kNaMolPairs) {
    std::snprintf(msg, sizeof msg, "force_noalloc: max_mol_pairs %d, the limit is %d",
                  p->max_mol_pairs, kNaMolPairs);
    return fail_na(FIBMD_EINVAL, msg);
  }
  fibmd_params q = *p;
  q.mode = FIBMD_MODE_REF;
  q.max_sw_nbrs = q.max_sw_nbrs > 0 ? q.max_sw_nbrs : kNaMaxSw;
  q.max_mol_pairs = kNaMolPairs;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail_na(FIBMD_ECUDA, "force_noalloc: no usable current device");
  cudaStream_t s = (cudaStream_t)stream;

  // per-device set-up on the first call (the device address of the array),
  // then the 2-body table: its key is compared, and on a change the table is
  // built, uploaded and recorded with its extent, all under one lock, so a
  // thread calling with other parameters cannot slip its table in between
  DeviceSlot& slot = g_slots[dev];
  double umax = 0.0;
  int last = 0;
  {
    std::lock_guard<std::mutex> lock(g_slots_mutex);
    if (!slot.ready) {
      void* base = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&base, g_noalloc_scratch);
      if (e != cudaSuccess || !base) {
        std::snprintf(msg, sizeof msg, "force_noalloc: cudaGetSymbolAddress: %s",
                      cudaGetErrorString(e));
        return fail_na(FIBMD_ECUDA, msg);
      }
      slot.base = static_cast<unsigned char*>(base);
      slot.ready = true;
    }
    const double key[7] = {q.A, q.B, q.psi, q.qsi, q.al, q.listfac, (double)q.Ntable};
    if (!slot.table_loaded || std::memcmp(key, slot.tab_key, sizeof key) != 0) {
      slot.table_loaded = false;
      double um = 0.0;
      int lz = 0;
      build_ref_table(q, g_tab_host, g_tabu_host, &um, &lz);
      const size_t tb = sizeof(double) * (size_t)(q.Ntable + 2);
      cudaError_t e1 = cudaMemcpyAsync(slot.base + kLayout.tab, g_tab_host, tb,
                                       cudaMemcpyHostToDevice, s);
      cudaError_t e2 = cudaMemcpyAsync(slot.base + kLayout.tabu, g_tabu_host, tb,
                                       cudaMemcpyHostToDevice, s);
      cudaError_t e3 = cudaStreamSynchronize(s);  // the host staging is shared
      if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess)
        return fail_na(FIBMD_ECUDA, "force_noalloc: table upload failed");
      std::memcpy(slot.tab_key, key, sizeof key);
      slot.umax = um;
      slot.tab_last = lz;
      slot.table_loaded = true;
    }
    umax = slot.umax;
    last = slot.tab_last;
  }
  DevParams P;
  Geo G;
  const int rc = derive_dev_params(q, impact, umax, last, P, G, msg, sizeof msg);
  if (rc) return fail_na(rc, msg);
  if (P.ncell > kNaCells) {
    std::snprintf(msg, sizeof msg, "force_noalloc: %d cells in the reference grid, the limit is %d",
                  P.ncell, kNaCells);
    return fail_na(FIBMD_EINVAL, msg);
  }
  unsigned char* b = slot.base;
  DevState S;
  std::memset(&S, 0, sizeof S);
  S.N = q.Natm;
  S.pos = reinterpret_cast<double4_32a*>(b + kLayout.pos);
  S.frc_new = reinterpret_cast<double4_32a*>(b + kLayout.frc_new);
  S.posq = reinterpret_cast<int4*>(b + kLayout.posq);
  S.posq_build = reinterpret_cast<int4*>(b + kLayout.posq_build);
  S.posq_cell = reinterpret_cast<int4*>(b + kLayout.posq_cell);
  S.atype = reinterpret_cast<int8_t*>(b + kLayout.atype);
  S.flags = reinterpret_cast<uint32_t*>(b + kLayout.flags);
  S.cell_count = reinterpret_cast<int*>(b + kLayout.cell_count);
  S.cell_start = reinterpret_cast<int*>(b + kLayout.cell_start);
  S.cell_atoms = reinterpret_cast<int*>(b + kLayout.cell_atoms);
  S.atom_cell = reinterpret_cast<int*>(b + kLayout.atom_cell);
  S.scan_blocks = reinterpret_cast<int*>(b + kLayout.scan_blocks);
  S.nbr_sw = reinterpret_cast<int*>(b + kLayout.nbr_sw);
  S.n_sw = reinterpret_cast<int*>(b + kLayout.n_sw);
  S.sw_extra = reinterpret_cast<int*>(b + kLayout.sw_extra);
  S.mol_pairs = reinterpret_cast<int2*>(b + kLayout.mol_pairs);
  S.fast_flag = reinterpret_cast<uint8_t*>(b + kLayout.fast_flag);
  S.fast_list = reinterpret_cast<int*>(b + kLayout.fast_list);
  S.heavy_list = reinterpret_cast<int*>(b + kLayout.heavy_list);
  S.tab = reinterpret_cast<const double*>(b + kLayout.tab);
  S.tabu = reinterpret_cast<const double*>(b + kLayout.tabu);
  S.partials = reinterpret_cast<double*>(b + kLayout.partials);
  S.sc = reinterpret_cast<DevScalars*>(b + kLayout.sc);
  Geo* geo_dev = reinterpret_cast<Geo*>(b + kLayout.geo);
  int* ion_dev = reinterpret_cast<int*>(b + kLayout.ion_list);
  S.geo = geo_dev;
  S.ion_list = ion_dev;

  int dev_sms = 152;
  cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, dev);
  Launch L;
  L.stream = s;
  L.sms = dev_sms;
  // the array keeps the previous call's contents: the scalars (counters,
  // reduction tickets, the bad-type flag) must start at zero
  cudaError_t e = cudaMemsetAsync(S.sc, 0, sizeof(DevScalars), s);
  // the geometry of this call (a pageable copy: staged before the call returns)
  if (e == cudaSuccess) e = cudaMemcpyAsync(geo_dev, &G, sizeof G, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    k_na_import<<<(q.Natm + 255) / 256, 256, 0, s>>>(
        q.Natm, q.Nsg, X_dev, atype_dev, S, ion_dev, &S.sc->nan_flag);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = launch_update_posq(L, P, S);
  if (e == cudaSuccess) e = launch_build_lists(L, P, S, 0);
  if (e == cudaSuccess) e = launch_force(L, P, S, false, false);
  if (e == cudaSuccess) e = launch_unpack(L, q.Natm, S.frc_new, F_dev);
  DevScalars h;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, S.sc, sizeof h, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    std::snprintf(msg, sizeof msg, "force_noalloc: %s", cudaGetErrorString(e));
    return fail_na(FIBMD_ECUDA, msg);
  }
  if (h.nan_flag) return fail_na(FIBMD_EINVAL, "force_noalloc: atype outside 1..3");
  if (h.overflow_sw) {
    std::snprintf(msg, sizeof msg, "force_noalloc: SW list slots exceeded: capacity %d, needed %d",
                  P.max_sw, h.sw_needed);
    return fail_na(FIBMD_EOVERFLOW, msg);
  }
  if (h.overflow_mol) return fail_na(FIBMD_EOVERFLOW, "force_noalloc: Moliere list exceeded");
  if (h.table_err) return fail_na(FIBMD_ETABLE, "force_noalloc: 2-body table index beyond Ntable");
  return FIBMD_OK;
}
