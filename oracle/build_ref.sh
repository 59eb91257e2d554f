#!/usr/bin/env bash
# Builds the reference's own single-rank implementation (src/pore_extraction.hpp, compiled
# unmodified from the read-only reference checkout) against the project's Kokkos shim.
# Output goes only to oracle/_ref/ (git-ignored). Test infrastructure: used to pin the C
# restatement (oracle/pnm_oracle.c) and to generate tests/golden/ fixtures.
#
#   PNM_REFERENCE=/path/to/reference oracle/build_ref.sh
#
# Exits 0 without building when the reference checkout is absent.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${PNM_REFERENCE:-/root/reference}"
if [ ! -f "$REF/src/pore_extraction.hpp" ]; then
  echo "build_ref: reference checkout not found at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$HERE/_ref"
CXX="${CXX:-g++}"
FLAGS=(-std=c++20 -O2 -fPIC -shared -ffp-contract=off -I"$HERE/kokkos_compat" -I"$REF/src")
# serial: deterministic pore emission and FP64 accumulation order
"$CXX" "${FLAGS[@]}" "$HERE/ref_capi.cpp" -o "$HERE/_ref/libpnm_ref.so" &
# OpenMP: the same source on all host threads (timing only)
"$CXX" "${FLAGS[@]}" -fopenmp -DPNM_SHIM_OPENMP "$HERE/ref_capi.cpp" -o "$HERE/_ref/libpnm_ref_omp.so" &
# the reference's VTI reader (src/sdf_reader.cpp), pins pnm_read_vti
"$CXX" -std=c++17 -O2 -fPIC -shared -I"$REF/src" "$HERE/ref_vti.cpp" "$REF/src/sdf_reader.cpp" \
  -o "$HERE/_ref/libpnm_ref_vti.so" &
wait
echo "build_ref: built $HERE/_ref/libpnm_ref.so, libpnm_ref_omp.so and libpnm_ref_vti.so"
