// fibmd_io.cpp — the reference's dump files, written on the host.
//
// writeatoms (src/out.f90:62-100): an extended-xyz frame per dump appended
// to data/mdrun2.xyz (count, a header with the time, then x y z in Angstrom,
// the species, the owning process and the kinetic energy in eV), and the
// snapshot data/3dmol2.xyz rewritten each time. The device packs positions
// and kinetic energies (fibmd_gpu_xyz_frame); here a background thread
// formats and writes the frames, so the step loop does not wait for the
// file system. writerestart (src/out.f90:34-58): three Fortran unformatted
// sequential records, each framed by 4-byte length markers as gfortran writes
// them.
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "fibmd_host.h"

namespace {

const char* species(int t) {
  // the reference names types 1 and 3; type 2 (Ge) is named here too
  return t == 3 ? "Ga" : (t == 2 ? "Ge" : "Si");
}

struct Frame {
  int natm;
  double time_s;
  std::vector<double> xyz;  // (natm,3) column-major, Angstrom
  std::vector<int> atype, proc;
  std::vector<double> ke;
};

}  // namespace

struct fibmd_xyz_writer {
  std::FILE* f = nullptr;
  std::string snap;
  std::mutex m;
  std::condition_variable cv;
  std::deque<Frame> q;
  bool closing = false;
  int err = 0;
  std::thread th;

  void write_frame(const Frame& fr) {
    const int n = fr.natm;
    const double tps = fr.time_s * 1e12;
    // (I9) and the header (1A12,F12.5,3A12,2A8,3A16,...) of writeatoms
    std::fprintf(f, "%9d\n", n);
    std::fprintf(f, "Time (ps) = %12.5f%12s%12s%12s%8s%8s%16s\n", tps, "x (A)", "y (A)", "z (A)",
                 "type", "proc#", "KE (eV)");
    for (int i = 0; i < n; i++)
      std::fprintf(f, "%12.4f%12.4f%12.4f%8s%8d%14.3E\n", fr.xyz[i], fr.xyz[(size_t)n + i],
                   fr.xyz[2 * (size_t)n + i], species(fr.atype[i]),
                   fr.proc.empty() ? 0 : fr.proc[i], fr.ke[i]);
    if (std::fflush(f) != 0) err = 1;
    if (!snap.empty()) {
      std::FILE* s = std::fopen(snap.c_str(), "w");
      if (!s) {
        err = 1;
        return;
      }
      // (I9), (5A12,F12.5), (A8,3F10.4)
      std::fprintf(s, "%9d\n", n);
      std::fprintf(s, "%12s%12s%12s%12sTime (ps) = %12.5f\n", "type", "x (A)", "y (A)", "z (A)",
                   tps);
      for (int i = 0; i < n; i++)
        std::fprintf(s, "%8s%10.4f%10.4f%10.4f\n", species(fr.atype[i]), fr.xyz[i],
                     fr.xyz[(size_t)n + i], fr.xyz[2 * (size_t)n + i]);
      if (std::fclose(s) != 0) err = 1;
    }
  }

  void run() {
    for (;;) {
      Frame fr;
      {
        std::unique_lock<std::mutex> lk(m);
        cv.wait(lk, [&] { return closing || !q.empty(); });
        if (q.empty()) return;
        fr = std::move(q.front());
      }
      write_frame(fr);
      {
        std::lock_guard<std::mutex> lk(m);
        q.pop_front();
      }
      cv.notify_all();
    }
  }
};

extern "C" {

int fibmd_host_xyz_open(const char* path, const char* snap_path, fibmd_xyz_writer** out) {
  if (!path || !out) return FIBMD_EINVAL;
  *out = nullptr;
  std::FILE* f = std::fopen(path, "a");
  if (!f) return FIBMD_EINVAL;
  fibmd_xyz_writer* w = new fibmd_xyz_writer();
  w->f = f;
  if (snap_path) w->snap = snap_path;
  w->th = std::thread([w] { w->run(); });
  *out = w;
  return FIBMD_OK;
}

int fibmd_host_xyz_write(fibmd_xyz_writer* w, int natm, double time_s, const double* xyz_A,
                         const int* atype, const double* ke_eV, const int* proc) {
  if (!w || natm < 0 || !xyz_A || !atype || !ke_eV) return FIBMD_EINVAL;
  Frame fr;
  fr.natm = natm;
  fr.time_s = time_s;
  fr.xyz.assign(xyz_A, xyz_A + 3 * (size_t)natm);
  fr.atype.assign(atype, atype + natm);
  fr.ke.assign(ke_eV, ke_eV + natm);
  if (proc) fr.proc.assign(proc, proc + natm);
  {
    std::lock_guard<std::mutex> lk(w->m);
    if (w->err) return FIBMD_EINVAL;
    w->q.push_back(std::move(fr));
  }
  w->cv.notify_all();
  return FIBMD_OK;
}

int fibmd_host_xyz_flush(fibmd_xyz_writer* w) {
  if (!w) return FIBMD_EINVAL;
  std::unique_lock<std::mutex> lk(w->m);
  w->cv.wait(lk, [&] { return w->q.empty(); });
  return w->err ? FIBMD_EINVAL : FIBMD_OK;
}

int fibmd_host_xyz_close(fibmd_xyz_writer* w) {
  if (!w) return FIBMD_EINVAL;
  {
    std::lock_guard<std::mutex> lk(w->m);
    w->closing = true;
  }
  w->cv.notify_all();
  w->th.join();
  int rc = w->err ? FIBMD_EINVAL : FIBMD_OK;
  if (std::fclose(w->f) != 0) rc = FIBMD_EINVAL;
  delete w;
  return rc;
}

// ---- writerestart / its reader -------------------------------------------------
namespace {
bool put_record(std::FILE* f, const std::vector<const void*>& parts,
                const std::vector<size_t>& bytes) {
  size_t total = 0;
  for (size_t b : bytes) total += b;
  if (total > 0x7fffffffu) return false;
  const int32_t len = (int32_t)total;
  if (std::fwrite(&len, 4, 1, f) != 1) return false;
  for (size_t k = 0; k < parts.size(); k++)
    if (bytes[k] && std::fwrite(parts[k], 1, bytes[k], f) != bytes[k]) return false;
  return std::fwrite(&len, 4, 1, f) == 1;
}

bool get_record(std::FILE* f, const std::vector<void*>& parts, const std::vector<size_t>& bytes) {
  size_t total = 0;
  for (size_t b : bytes) total += b;
  int32_t a = 0, b = 0;
  if (std::fread(&a, 4, 1, f) != 1 || a < 0 || (size_t)a != total) return false;
  for (size_t k = 0; k < parts.size(); k++)
    if (bytes[k] && std::fread(parts[k], 1, bytes[k], f) != bytes[k]) return false;
  return std::fread(&b, 4, 1, f) == 1 && b == a;
}
}  // namespace

int fibmd_host_write_restart(const char* path, int natm, int lt, double restart_time,
                             const double* X, const double* V, const double* mass,
                             const int* atype, int impact) {
  if (!path || natm <= 0 || !X || !V || !mass || !atype) return FIBMD_EINVAL;
  std::FILE* f = std::fopen(path, "wb");
  if (!f) return FIBMD_EINVAL;
  const size_t n = (size_t)natm;
  const int32_t lt4 = lt, imp4 = impact;
  std::vector<int32_t> t4(atype, atype + n);
  bool ok = put_record(f, {&lt4, &restart_time}, {4, 8}) &&
            put_record(f, {X, V, mass, t4.data()}, {24 * n, 24 * n, 8 * n, 4 * n}) &&
            put_record(f, {&imp4}, {4});
  ok = (std::fclose(f) == 0) && ok;
  return ok ? FIBMD_OK : FIBMD_EINVAL;
}

int fibmd_host_read_restart(const char* path, int natm, int* lt, double* restart_time, double* X,
                            double* V, double* mass, int* atype, int* impact) {
  if (!path || natm <= 0 || !lt || !restart_time || !X || !V || !mass || !atype || !impact)
    return FIBMD_EINVAL;
  std::FILE* f = std::fopen(path, "rb");
  if (!f) return FIBMD_EINVAL;
  const size_t n = (size_t)natm;
  int32_t lt4 = 0, imp4 = 0;
  std::vector<int32_t> t4(n);
  bool ok = get_record(f, {&lt4, restart_time}, {4, 8}) &&
            get_record(f, {X, V, mass, t4.data()}, {24 * n, 24 * n, 8 * n, 4 * n}) &&
            get_record(f, {&imp4}, {4});
  std::fclose(f);
  if (!ok) return FIBMD_EINVAL;
  *lt = lt4;
  *impact = imp4;
  for (size_t i = 0; i < n; i++) atype[i] = t4[i];
  return FIBMD_OK;
}

}  // extern "C"
