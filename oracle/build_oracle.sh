#!/bin/sh
# Builds the CPU oracle (the scalar restatement in this directory) as
# oracle/liboracle_port.so.  Portable C++17: no intrinsics, no -march, so the
# same sources build on x86-64 and aarch64.  -ffp-contract=off keeps the
# double-precision SSIM tie-break unfused.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/liboracle_port.so"
g++ -O3 -std=c++17 -fPIC -shared -ffp-contract=off -fno-strict-aliasing \
  "$HERE/port_tables.cpp" "$HERE/port_core.cpp" "$HERE/port_block.cpp" \
  "$HERE/port_modes.cpp" "$HERE/port_pca.cpp" "$HERE/port_api.cpp" -o "$OUT" -lpthread
echo "built $OUT"
# the same sources with the work counters of port_counters.h
g++ -O3 -std=c++17 -fPIC -shared -ffp-contract=off -fno-strict-aliasing -DNEBC7_PORT_COUNTERS \
  "$HERE/port_tables.cpp" "$HERE/port_core.cpp" "$HERE/port_block.cpp" \
  "$HERE/port_modes.cpp" "$HERE/port_pca.cpp" "$HERE/port_api.cpp" -o "$HERE/liboracle_port_counters.so" -lpthread
echo "built $HERE/liboracle_port_counters.so"
