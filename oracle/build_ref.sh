#!/bin/bash
# Recipe for oracle/_ref: the reference's own mdrun2 (Fortran 90 + MPI),
# built from its sources where they lie, with the flags of its Makefile
# (mpif90 -fdefault-real-8 -O3 -fbacktrace -ffree-line-length-none,
# src/Makefile:1-5), as a second oracle and CPU baseline.
# It needs a Fortran compiler and MPI; it probes for them first and says
# which are missing (this is the probe whose output is summarised in
# profiles/). Output goes only to oracle/_ref/.
set -u
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_SRC="${FIBMD_REF_SRC:-/root/reference/src}"
echo "host: $(uname -m), $(nproc) cores"
found=""
for t in gfortran f95 flang flang-new nvfortran lfortran ifort ifx mpif90 mpifort mpirun mpiexec; do
  p=$(command -v "$t" 2>/dev/null)
  echo "$t: ${p:-absent}"
  [ -n "$p" ] && found="$found $t"
done
ls /usr/lib/gcc/*/*/f951 >/dev/null 2>&1 && echo "f951 (gcc Fortran front end): present" \
  || echo "f951 (gcc Fortran front end): absent"
if ! command -v mpif90 >/dev/null 2>&1 || ! command -v mpirun >/dev/null 2>&1; then
  echo "oracle/_ref: unbuildable here (no mpif90/mpirun; the reference is Fortran 90 + MPI)"
  exit 0
fi
if [ ! -d "$REF_SRC" ]; then
  echo "oracle/_ref: reference sources not found at $REF_SRC"
  exit 0
fi
mkdir -p "$HERE/_ref/obj"
cd "$HERE/_ref/obj" || exit 1
# modules in the dependency order of the reference's Makefile (src/Makefile:14-60)
FLAGS="-fdefault-real-8 -O3 -fbacktrace -ffree-line-length-none"
for f in ran1.f parallel.f90 prms.f90 data.f90 par.f90 tools.f90 nlist.f90 si.f90 stats.f90 \
         temp.f90 out.f90 knock.f90 timeint.f90 main.f90; do
  mpif90 $FLAGS -c "$REF_SRC/$f" || exit 1
done
mpif90 -o "$HERE/_ref/mdrun2" ./*.o && echo "built oracle/_ref/mdrun2"
