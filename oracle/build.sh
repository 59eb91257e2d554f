#!/usr/bin/env bash
# Builds the CPU restatement (oracle/pnm_oracle.cpp) into oracle/libpnm_oracle.so.
# Test and baseline infrastructure only. No FMA contraction (-ffp-contract=off), no
# machine-specific flags, so x86-64 and aarch64 builds round identically.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
CXX="${CXX:-g++}"
"$CXX" -std=c++20 -O3 -fopenmp -ffp-contract=off -fPIC -shared \
  "$HERE/pnm_oracle.cpp" -o "$HERE/libpnm_oracle.so"
